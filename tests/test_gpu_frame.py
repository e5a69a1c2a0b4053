"""The code either side of the step: the frame image (render_image), device
add_noise, device obstacle rasterisation, the graph-captured frame loop and
the packed read-back of the pub fields."""
import math

import numpy as np
import pytest

import oracle
from equilibrium_gb300 import _lib
from equilibrium_gb300.simulation import (Fluid, FluidConfigs, Rectangle, SimulationConfigs,
                                          write_png)
from tests.util import assert_bitexact, random_rects

pytestmark = pytest.mark.gpu


def L():
    return _lib.load()


def fluid(size=66, frames=20, dt=0.1, diff=1e-4, visc=1e-4):
    return Fluid(FluidConfigs(diff, visc, False), SimulationConfigs(dt, frames, size))


@pytest.mark.parametrize("colors", [None, ((10, 200, 30, 40), (1, 2, 3, 4), (9, 8, 7, 6))])
def test_render_rgba_matches_reference_rule(eqlib, tmp_path, colors):
    g = fluid()
    assert L().eq_fluid_fill_obstacle(g.handle, 10, 12, 20, 25) == 0
    rng = np.random.default_rng(0)
    d = rng.uniform(-10, 400, 66 * 66).astype(np.float32)
    d[rng.integers(0, d.size, 200)] = 0.0
    d[5] = np.nan
    g.write_field(_lib.FIELD_DENSITY, d)
    img = g.render_rgba(colors)
    kw = {} if colors is None else dict(fluid=colors[0], world=colors[1], obstacles=colors[2])
    ref = oracle.render_rgba(d, g.cells_type, 66, **kw)
    np.testing.assert_array_equal(img, ref)
    write_png(str(tmp_path / "density0.png"), img)
    assert (tmp_path / "density0.png").stat().st_size > 100
    g.close()


def test_fill_obstacle_device_equals_host_path(eqlib):
    rng = np.random.default_rng(4)
    a, b = fluid(97), fluid(97)
    for r in random_rects(rng, 97, 5) + [(0, 40, 97, 41), (-5, -5, 3, 200)]:
        assert L().eq_fluid_fill_obstacle(a.handle, *r) == 0
        assert L().eq_fluid_fill_obstacle_device(b.handle, *r) == 0
    np.testing.assert_array_equal(a.cells_type, b.cells_type)
    for _ in range(3):
        a.step()
        b.step()
    for f in range(6):
        assert_bitexact(b.read_field(f), a.read_field(f), f"device obstacles field {f}", 97)
    a.close()
    b.close()


@pytest.mark.parametrize("size,noise", [(66, False), (66, True), (258, True)])
def test_step_graph_equals_eager_steps(eqlib, size, noise):
    a, b = fluid(size), fluid(size)
    for h in (a, b):
        assert L().eq_fluid_fill_obstacle(h.handle, size // 3, size // 4, size // 2, size // 3) == 0
    b.step_graph(3, noise, seed=99)
    b.step_graph(3, noise, seed=99)  # replayed
    for _ in range(6):
        if noise:
            a.add_noise(seed=99)
        a.step()
    a.synchronize()
    b.synchronize()
    for f in range(6):
        assert_bitexact(b.read_field(f), a.read_field(f), f"graph frames field {f}", size)
    a.close()
    b.close()


def test_add_noise_impulse_geometry(eqlib):
    size, dt = 130, 0.05
    g = fluid(size, dt=dt)
    c = size // 2
    q = c * size + c
    angle = math.radians(L().eq_noise_angle(np.float32(dt)))
    for k in range(8):
        vx0, vy0 = g.read_field(_lib.FIELD_VX)[q], g.read_field(_lib.FIELD_VY)[q]
        g.add_noise(seed=1234)
        ix = (g.read_field(_lib.FIELD_VX)[q] - vx0) / 2.0
        iy = (g.read_field(_lib.FIELD_VY)[q] - vy0) / 2.0
        # undo the rotation about the centre: the drawn cell is integral, in the grid
        ox, oy = ix - c, iy - c
        rx = c + ox * math.cos(-angle) - oy * math.sin(-angle)
        ry = c + ox * math.sin(-angle) + oy * math.cos(-angle)
        assert abs(rx - round(rx)) < 0.05 and abs(ry - round(ry)) < 0.05
        assert 0 <= round(rx) < size and 0 <= round(ry) < size
    g.close()


def test_read_fields_matches_read_field(eqlib):
    """eq_fluid_read_fields (device packing, one copy per field) gives each
    field bit for bit as eq_fluid_read_field does, into numpy and pinned
    torch buffers, for one to six fields; bad arguments are refused."""
    import torch
    size = 133
    f = Fluid(FluidConfigs(1e-4, 1e-4, False), SimulationConfigs(0.1, 5, size))
    rng = np.random.default_rng(3)
    for k in range(6):
        f.write_field(k, rng.uniform(-1, 1, size * size).astype(np.float32))
    f.step()
    want = [f.read_field(k) for k in range(6)]
    for sel in ((1,), (1, 2, 3), (5, 0, 4, 2), tuple(range(6))):
        got = f.read_fields(sel)
        for k, g in zip(sel, got):
            np.testing.assert_array_equal(g.view(np.uint32), want[k].view(np.uint32))
    pinned = [torch.empty(size * size, dtype=torch.float32).pin_memory() for _ in range(3)]
    f.read_fields((1, 2, 3), pinned)
    for k, t in zip((1, 2, 3), pinned):
        np.testing.assert_array_equal(t.numpy().view(np.uint32), want[k].view(np.uint32))
    with pytest.raises(_lib.EqError):
        f.read_fields((1, 7))
    f.close()


@pytest.mark.gpu
def test_read_fields_async_overlaps_later_steps(eqlib):
    """eq_fluid_read_fields_async after each of four steps, into two pinned
    buffer sets used in turn (the read-back of frame n in flight while frame
    n+1 computes), gives every frame's fields bit for bit as a synchronous
    read after the same frames; growing the field count reallocates the
    staging; bad arguments are refused."""
    import torch
    size = 133
    cfg = (FluidConfigs(1e-4, 1e-4, False), SimulationConfigs(0.1, 5, size))
    rng = np.random.default_rng(5)
    init = [rng.uniform(-1, 1, size * size).astype(np.float32) for _ in range(6)]
    ref, f = Fluid(*cfg), Fluid(*cfg)
    for g in (ref, f):
        for k in range(6):
            g.write_field(k, init[k])
    sel = (1, 2, 3)
    want = []
    for _ in range(4):
        ref.step()
        want.append(ref.read_fields(sel))
    bufs = [[torch.empty(size * size, dtype=torch.float32).pin_memory() for _ in sel]
            for _ in range(4)]
    for fr in range(4):
        f.step()
        f.read_fields_async(sel, bufs[fr])
    f.synchronize()
    for fr in range(4):
        for w, t in zip(want[fr], bufs[fr]):
            np.testing.assert_array_equal(t.numpy().view(np.uint32), w.view(np.uint32))
    six = [torch.empty(size * size, dtype=torch.float32).pin_memory() for _ in range(6)]
    f.read_fields_async(tuple(range(6)), six)
    f.synchronize()
    now = f.read_fields(tuple(range(6)))
    for w, t in zip(now, six):
        np.testing.assert_array_equal(t.numpy().view(np.uint32), w.view(np.uint32))
    with pytest.raises(_lib.EqError):
        f.read_fields_async((1, 7), six[:2])
    ref.close()
    f.close()
