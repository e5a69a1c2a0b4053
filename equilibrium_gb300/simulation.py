"""Host-side mirror of the reference's simulation API over the C ABI.

Same names, argument meanings and error behaviour as the reference's Rust
module ``src/simulation`` (vkabadzhova/equilibrium):

* ``SimulationConfigs`` / ``FluidConfigs``      -- configs.rs:5-60
* ``Rectangle`` (panics -> ``InvalidRectangle``) -- obstacle.rs:29-87
* ``ContainerWall``                              -- fluid.rs:10-17
* ``Fluid`` (new / default / step / fill_obstacle / add_noise / clone, pub
  fields density, velocities_x, velocities_y, cells_type) -- fluid.rs:51-620
* ``CurrentSimulation`` (simulate / mark_fluid_obstacles) -- renderer_helpers.rs:29-81

Every numeric operation runs in ``libeqfluid.so`` on the GPU; the pub fields
are host snapshots read back from the device on access, as a Rust wrapper
keeps its ``Vec<f32>`` fields coherent after each ``step()``.
"""
from __future__ import annotations

import ctypes
import enum
import math
import random
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Tuple

import numpy as np

from . import _lib
from ._lib import EqError, check

Point = Tuple[int, int]


class InvalidRectangle(ValueError):
    """Raised where the reference panics with "Invalid input for Rectangle"."""


class ContainerWall(enum.Enum):
    DefaultWall = 1
    NoWall = 0


@dataclass
class SimulationConfigs:
    delta_t: float = 0.02
    frames: int = 16
    size: int = 128

    @staticmethod
    def new(delta_t: float, frames: int, fluid_container_size: int) -> "SimulationConfigs":
        return SimulationConfigs(delta_t, frames, fluid_container_size)


@dataclass
class FluidConfigs:
    diffusion: float = 0.0
    viscousity: float = 0.001
    has_perlin_noise: bool = True
    fluid_color: Tuple[int, int, int, int] = (208, 88, 157, 220)
    world_color: Tuple[int, int, int, int] = (94, 146, 162, 128)


class Rectangle:
    """Axis-parallel rectangle obstacle (obstacle.rs:29-87)."""

    def __init__(self, down_left_point: Point, up_right_point: Point,
                 fluid_container_size: int):
        self.down_left_point = tuple(down_left_point)
        self.up_right_point = tuple(up_right_point)
        self.approximate_points = [self.down_left_point, self.up_right_point]
        if not self.are_all_points_valid(fluid_container_size):
            raise InvalidRectangle("Invalid input for Rectangle")

    @staticmethod
    def default() -> "Rectangle":
        return Rectangle((80, 80), (110, 110), SimulationConfigs().size)

    def are_all_points_valid(self, fluid_container_size: int) -> bool:
        dl, ur = self.down_left_point, self.up_right_point
        return _lib.load().eq_rectangle_check(dl[0], dl[1], ur[0], ur[1],
                                              int(fluid_container_size)) == _lib.EQ_OK

    def get_approximate_points(self) -> List[Point]:
        return self.approximate_points

    def clone(self) -> "Rectangle":
        r = Rectangle.__new__(Rectangle)
        r.down_left_point, r.up_right_point = self.down_left_point, self.up_right_point
        r.approximate_points = list(self.approximate_points)
        return r


ObstaclesType = Rectangle  # the reference's enum has the single variant Rectangle


def _as_f32(a, n: int) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1))
    if a.size != n:
        raise ValueError(f"expected {n} elements, got {a.size}")
    return a


class Fluid:
    """The stable-fluids state of one scene, resident on the GPU."""

    def __init__(self, init_fluid: Optional[FluidConfigs] = None,
                 init_simulation: Optional[SimulationConfigs] = None, device: int = -1,
                 _handle=None, lib=None):
        self.fluid_configs = init_fluid if init_fluid is not None else FluidConfigs()
        self.simulation_configs = (init_simulation if init_simulation is not None
                                   else SimulationConfigs())
        self._L = lib if lib is not None else _lib.load()
        if _handle is not None:
            self._h = _handle
            return
        h = ctypes.c_void_p()
        fc = _lib.FluidConfigsC(self.fluid_configs.diffusion, self.fluid_configs.viscousity,
                                int(bool(self.fluid_configs.has_perlin_noise)))
        sc = _lib.SimulationConfigsC(self.simulation_configs.delta_t,
                                     int(self.simulation_configs.frames),
                                     int(self.simulation_configs.size))
        check(self._L.eq_fluid_new(ctypes.byref(fc), ctypes.byref(sc), device, ctypes.byref(h)))
        self._h = h

    # -- construction -------------------------------------------------------
    @staticmethod
    def new(init_fluid: FluidConfigs, init_simulation: SimulationConfigs) -> "Fluid":
        return Fluid(init_fluid, init_simulation)

    @staticmethod
    def default(device: int = -1) -> "Fluid":
        L = _lib.load()
        h = ctypes.c_void_p()
        check(L.eq_fluid_default(device, ctypes.byref(h)))
        return Fluid(FluidConfigs(), SimulationConfigs(), _handle=h)

    def clone(self) -> "Fluid":
        self._push_configs()
        h = ctypes.c_void_p()
        check(self._L.eq_fluid_clone(self._h, ctypes.byref(h)))
        return Fluid(FluidConfigs(**vars(self.fluid_configs)),
                     SimulationConfigs(**vars(self.simulation_configs)), _handle=h)

    def close(self):
        if getattr(self, "_h", None):
            self._L.eq_fluid_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- the hot path ---------------------------------------------------------
    def _push_configs(self):
        fc = _lib.FluidConfigsC(self.fluid_configs.diffusion, self.fluid_configs.viscousity,
                                int(bool(self.fluid_configs.has_perlin_noise)))
        sc = _lib.SimulationConfigsC(self.simulation_configs.delta_t,
                                     int(self.simulation_configs.frames),
                                     int(self.simulation_configs.size))
        check(self._L.eq_fluid_set_configs(self._h, ctypes.byref(fc), ctypes.byref(sc)))

    def step(self):
        """fluid.rs:437-524 (asynchronous; field reads synchronise)."""
        self._push_configs()
        check(self._L.eq_fluid_step(self._h))

    def step_n(self, nframes: int):
        self._push_configs()
        check(self._L.eq_fluid_step_n(self._h, int(nframes)))

    def synchronize(self):
        check(self._L.eq_fluid_synchronize(self._h))

    # -- sources ----------------------------------------------------------------
    def add_density(self, x: int, y: int, amount: float):
        check(self._L.eq_fluid_add_density(self._h, x, y, amount))

    def add_velocity(self, x: int, y: int, amount_x: float, amount_y: float):
        check(self._L.eq_fluid_add_velocity(self._h, x, y, amount_x, amount_y))

    def add_sources(self, xs, ys, density=None, vx=None, vy=None):
        xs = np.ascontiguousarray(xs, dtype=np.uint32)
        ys = np.ascontiguousarray(ys, dtype=np.uint32)
        n = xs.size
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float32)
                for a in (density, vx, vy)]
        ptr = [None if a is None else a.ctypes.data for a in arrs]
        check(self._L.eq_fluid_add_sources(self._h, n, xs.ctypes.data, ys.ctypes.data, *ptr))

    def add_noise(self, seed: Optional[int] = None):
        """fluid.rs:575-599 on the device: a velocity impulse at the centre whose
        value is twice a uniformly drawn cell rotated about the centre by the
        gradient-noise angle at (dt, dt) (eq_noise_angle). The reference's angle
        comes from the `noise` crate's Perlin and its cell from `thread_rng`,
        so this matches it in distribution only. `seed` None draws one."""
        if seed is None:
            seed = random.getrandbits(64)
        check(self._L.eq_fluid_add_noise(self._h, int(seed) & (2**64 - 1)))

    def step_graph(self, nframes: int, with_noise: bool = False, seed: int = 0):
        """`nframes` frames (optional device noise, then step) replayed from one
        captured CUDA graph: the frame loop without a host sync per frame."""
        check(self._L.eq_fluid_step_graph(self._h, int(nframes), int(bool(with_noise)),
                                          int(seed) & (2**64 - 1)))

    def render_rgba(self, colors=None) -> np.ndarray:
        """render_image's pixels (renderer_helpers.rs:115-180) as (size, size, 4) RGBA8,
        row y, column x. `colors` = (fluid, world, obstacles) RGBA tuples or None."""
        n = int(self.simulation_configs.size)
        out = np.empty((n, n, 4), dtype=np.uint8)
        c = None
        if colors is not None:
            c = _lib.RenderColorsC((ctypes.c_uint8 * 4)(*colors[0]), (ctypes.c_uint8 * 4)(*colors[1]),
                                   (ctypes.c_uint8 * 4)(*colors[2]))
        check(self._L.eq_fluid_render_rgba(self._h, ctypes.byref(c) if c is not None else None,
                                           out.ctypes.data, out.nbytes))
        return out

    # -- obstacles ------------------------------------------------------------
    def fill_obstacle(self, obstacle: Rectangle):
        """fluid.rs:610-619, rasterised on the device (mask and boundary codes
        updated in place)."""
        p = obstacle.get_approximate_points()
        check(self._L.eq_fluid_fill_obstacle_device(self._h, p[0][0], p[0][1], p[1][0],
                                                    p[1][1]))

    # -- the pub fields -----------------------------------------------------------
    def _n(self) -> int:
        s = int(self.simulation_configs.size)
        return s * s

    def read_field(self, field_index: int) -> np.ndarray:
        out = np.empty(self._n(), dtype=np.float32)
        check(self._L.eq_fluid_read_field(self._h, field_index, out.ctypes.data, out.size))
        return out

    def read_fields(self, field_indices, outs=None) -> list:
        """Several fields at once (one device-side packing, one copy each, one
        synchronisation); `outs` may give the host arrays (pinned memory for
        the fastest copies)."""
        import ctypes
        k = len(field_indices)
        if outs is None:
            outs = [np.empty(self._n(), dtype=np.float32) for _ in range(k)]
        fi = (ctypes.c_int * k)(*field_indices)
        ptrs = (ctypes.c_void_p * k)(*[o.ctypes.data if isinstance(o, np.ndarray)
                                       else o.data_ptr() for o in outs])
        check(self._L.eq_fluid_read_fields(self._h, k, ctypes.cast(fi, ctypes.c_void_p),
                                           ctypes.cast(ptrs, ctypes.c_void_p), self._n()))
        return outs

    def read_fields_async(self, field_indices, outs) -> list:
        """read_fields without waiting: the copies run on a read-back stream of
        their own while later steps compute, and are complete at the next
        synchronize(). `outs` (pinned host arrays or tensors) must stay alive
        until then."""
        import ctypes
        k = len(field_indices)
        fi = (ctypes.c_int * k)(*field_indices)
        ptrs = (ctypes.c_void_p * k)(*[o.ctypes.data if isinstance(o, np.ndarray)
                                       else o.data_ptr() for o in outs])
        check(self._L.eq_fluid_read_fields_async(self._h, k, ctypes.cast(fi, ctypes.c_void_p),
                                                 ctypes.cast(ptrs, ctypes.c_void_p), self._n()))
        return outs

    def write_field(self, field_index: int, values):
        a = _as_f32(values, self._n())
        check(self._L.eq_fluid_write_field(self._h, field_index, a.ctypes.data, a.size))

    @property
    def density(self) -> np.ndarray:
        return self.read_field(_lib.FIELD_DENSITY)

    @density.setter
    def density(self, v):
        self.write_field(_lib.FIELD_DENSITY, v)

    @property
    def velocities_x(self) -> np.ndarray:
        return self.read_field(_lib.FIELD_VX)

    @velocities_x.setter
    def velocities_x(self, v):
        self.write_field(_lib.FIELD_VX, v)

    @property
    def velocities_y(self) -> np.ndarray:
        return self.read_field(_lib.FIELD_VY)

    @velocities_y.setter
    def velocities_y(self, v):
        self.write_field(_lib.FIELD_VY, v)

    @property
    def cells_type(self) -> np.ndarray:
        """uint8 per cell, 1 = ContainerWall.DefaultWall."""
        out = np.empty(self._n(), dtype=np.uint8)
        check(self._L.eq_fluid_read_cells(self._h, out.ctypes.data, out.size))
        return out

    @cells_type.setter
    def cells_type(self, v):
        a = np.ascontiguousarray(np.asarray(v, dtype=np.uint8).reshape(-1))
        check(self._L.eq_fluid_write_cells(self._h, a.ctypes.data, a.size))

    def all_fields(self) -> List[np.ndarray]:
        """The six arrays in declaration order (scratch, density, vx, vy, vx0, vy0)."""
        return [self.read_field(f) for f in range(6)]

    def set_all_fields(self, fields):
        for f, v in enumerate(fields):
            self.write_field(f, v)

    @property
    def handle(self):
        return self._h


def _fade(t):
    return t * t * t * (t * (t * 6 - 15) + 10)


def _gradient_noise_2d(x: float, y: float, seed: int = 0) -> float:
    """Improved-Perlin gradient noise in [-1, 1] with a fixed permutation."""
    perm = list(range(256))
    random.Random(seed).shuffle(perm)
    perm += perm
    xi, yi = int(math.floor(x)) & 255, int(math.floor(y)) & 255
    xf, yf = x - math.floor(x), y - math.floor(y)
    u, v = _fade(xf), _fade(yf)

    def grad(h, dx, dy):
        h &= 3
        return (dx if h & 1 == 0 else -dx) + (dy if h & 2 == 0 else -dy)

    aa, ab = perm[perm[xi] + yi], perm[perm[xi] + yi + 1]
    ba, bb = perm[perm[xi + 1] + yi], perm[perm[xi + 1] + yi + 1]
    x1 = grad(aa, xf, yf) + u * (grad(ba, xf - 1, yf) - grad(aa, xf, yf))
    x2 = grad(ab, xf, yf - 1) + u * (grad(bb, xf - 1, yf - 1) - grad(ab, xf, yf - 1))
    return max(-1.0, min(1.0, (x1 + v * (x2 - x1)) / 2.0 * 2.0))


@dataclass
class FluidStep:
    """renderer_helpers.rs:21-24: a frame's snapshot sent to the renderer."""
    fluid: Fluid
    frame_number: int


@dataclass
class CurrentSimulation:
    """renderer_helpers.rs:29-81: the frame loop around Fluid::step."""
    fluid: Fluid = None
    obstacles: List[Rectangle] = field(default_factory=list)

    @staticmethod
    def default() -> "CurrentSimulation":
        return CurrentSimulation(Fluid.default(), [Rectangle.default()])

    def mark_fluid_obstacles(self):
        for obstacle in self.obstacles:
            self.fluid.fill_obstacle(obstacle)

    def simulate(self, tx: Callable[[FluidStep], None]):
        """Marks obstacles, then per frame: optional noise, step(), send a clone."""
        self.mark_fluid_obstacles()
        for i in range(int(self.fluid.simulation_configs.frames)):
            if self.fluid.fluid_configs.has_perlin_noise:
                self.fluid.add_noise()
            self.fluid.step()
            tx(FluidStep(self.fluid.clone(), i))


def write_png(path: str, rgba: np.ndarray):
    """A frame image (H, W, 4) RGBA8 as a PNG file (stdlib zlib; the reference
    saves JPEGs through the `image` crate, renderer_helpers.rs:166-179)."""
    import struct
    import zlib
    h, w = rgba.shape[:2]
    raw = b"".join(b"\x00" + rgba[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return (struct.pack(">I", len(data)) + tag + data +
                struct.pack(">I", zlib.crc32(tag + data) & 0xffffffff))

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))
