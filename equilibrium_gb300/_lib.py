"""ctypes binding of the C ABI in ``include/eqfluid.h`` (``libeqfluid.so``).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "libeqfluid.so")
LIB_FMA_PATH = os.path.join(HERE, "libeqfluid_fma.so")
HEADER = os.path.join(ROOT, "include", "eqfluid.h")

EQ_OK, EQ_ERR_ARG, EQ_ERR_CUDA, EQ_ERR_TIMEOUT, EQ_ERR_OOM, EQ_ERR_STATE = range(6)
FIELD_SCRATCH, FIELD_DENSITY, FIELD_VX, FIELD_VY, FIELD_VX0, FIELD_VY0 = range(6)
MODE_ADJUST_ROW, MODE_ADJUST_COLUMN, MODE_PASSIVE = range(3)
STORE_F16, STORE_BF16, STORE_F16_SCALARS = 1, 2, 3


class EqError(RuntimeError):
    """A non-zero status from the C ABI (the reference panics in these places)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[eqfluid status {code}] {msg}")
        self.code = code


class SimulationConfigsC(ctypes.Structure):
    _fields_ = [("delta_t", ctypes.c_float), ("frames", ctypes.c_int64),
                ("size", ctypes.c_uint32)]


class SceneDescC(ctypes.Structure):
    _fields_ = [("size", ctypes.c_uint32), ("delta_t", ctypes.c_float),
                ("frames", ctypes.c_int64), ("diffusion", ctypes.c_float),
                ("viscousity", ctypes.c_float)]


class HStatsC(ctypes.Structure):
    _fields_ = [("ir_iterations", ctypes.c_int32 * 2), ("rel_residual", ctypes.c_double * 2),
                ("div_norm_before", ctypes.c_double * 2), ("div_norm", ctypes.c_double * 2)]


class RenderColorsC(ctypes.Structure):
    _fields_ = [("fluid", ctypes.c_uint8 * 4), ("world", ctypes.c_uint8 * 4),
                ("obstacles", ctypes.c_uint8 * 4)]


class FluidConfigsC(ctypes.Structure):
    _fields_ = [("diffusion", ctypes.c_float), ("viscousity", ctypes.c_float),
                ("has_perlin_noise", ctypes.c_int32)]


_lib = None
_others = {}  # libraries loaded from other paths (the FMA build)


def header_functions() -> list[str]:
    """Every function the public header declares."""
    with open(HEADER) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(eq_[a-z0-9_]+)\s*\(", text)))


def load(path: str = LIB_PATH):
    """Load the library and declare signatures. Raises if it is missing."""
    global _lib
    if path == LIB_PATH and _lib is not None:
        return _lib
    if path in _others:
        return _others[path]
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            " (the CUDA library is required; there is no CPU fallback)")
    L = ctypes.CDLL(path)
    P, H = ctypes.c_void_p, ctypes.c_void_p
    i32, i64, u32, u64, f32 = (ctypes.c_int, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint64,
                               ctypes.c_float)
    PP = ctypes.POINTER(ctypes.c_void_p)
    sigs = {
        "eq_abi_version": (i32, []),
        "eq_last_error": (ctypes.c_char_p, []),
        "eq_fluid_new": (i32, [ctypes.POINTER(FluidConfigsC), ctypes.POINTER(SimulationConfigsC),
                               i32, PP]),
        "eq_fluid_default": (i32, [i32, PP]),
        "eq_fluid_init": (i32, [H]),
        "eq_fluid_clone": (i32, [H, PP]),
        "eq_fluid_free": (i32, [H]),
        "eq_fluid_get_configs": (i32, [H, ctypes.POINTER(FluidConfigsC),
                                       ctypes.POINTER(SimulationConfigsC)]),
        "eq_fluid_set_configs": (i32, [H, ctypes.POINTER(FluidConfigsC),
                                       ctypes.POINTER(SimulationConfigsC)]),
        "eq_fluid_step": (i32, [H]),
        "eq_fluid_step_n": (i32, [H, i64]),
        "eq_fluid_synchronize": (i32, [H]),
        "eq_fluid_add_density": (i32, [H, u32, u32, f32]),
        "eq_fluid_add_velocity": (i32, [H, u32, u32, f32, f32]),
        "eq_fluid_add_sources": (i32, [H, i64, P, P, P, P, P]),
        "eq_fluid_run_device_sources": (i32, [H, i64, i64, P, P, P, P, P]),
        "eq_rectangle_check": (i32, [i64, i64, i64, i64, u32]),
        "eq_fluid_fill_obstacle": (i32, [H, i64, i64, i64, i64]),
        "eq_fluid_read_field": (i32, [H, i32, P, u64]),
        "eq_fluid_write_field": (i32, [H, i32, P, u64]),
        "eq_fluid_read_field_async": (i32, [H, i32, P, u64]),
        "eq_fluid_read_fields": (i32, [H, i32, P, P, u64]),
        "eq_fluid_read_fields_async": (i32, [H, i32, P, P, u64]),
        "eq_fluid_write_field_async": (i32, [H, i32, P, u64]),
        "eq_fluid_read_cells": (i32, [H, P, u64]),
        "eq_fluid_write_cells": (i32, [H, P, u64]),
        "eq_fluid_set_boundaries": (i32, [H, i32, i32]),
        "eq_fluid_lin_solve": (i32, [H, i32, i32, i32, f32, f32]),
        "eq_fluid_diffuse": (i32, [H, i32, i32, i32, f32]),
        "eq_fluid_project": (i32, [H, i32, i32, i32, i32]),
        "eq_fluid_advect": (i32, [H, i32, i32, i32, i32, i32]),
        "eq_fluid_device_field": (i32, [H, i32, PP, ctypes.POINTER(ctypes.c_uint32)]),
        "eq_fluid_launch_count": (i32, [H, ctypes.POINTER(ctypes.c_uint64)]),
        "eq_fluid_set_spin_limit": (i32, [H, i64]),
        "eq_fluid_set_solver": (i32, [H, i32]),
        "eq_fluid_set_concurrency": (i32, [H, i32]),
        "eq_fluid_get_solver": (i32, [H, ctypes.POINTER(ctypes.c_int)]),
        "eq_fluid_get_cluster_form": (i32, [H, ctypes.POINTER(ctypes.c_int)]),
        "eq_fluid_set_cluster_interval": (i32, [H, i32]),
        "eq_fluid_set_strip_groups": (i32, [H, i32]),
        "eq_fluid_set_strip_slack": (i32, [H, i32]),
        "eq_fluid_get_stream": (i32, [H, PP]),
        "eq_fluid_set_profiling": (i32, [H, i32]),
        "eq_fluid_kernel_stats": (i32, [H, i32, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_uint64)]),
        "eq_fluid_render_rgba": (i32, [H, ctypes.POINTER(RenderColorsC), P, u64]),
        "eq_fluid_render_rgba_device": (i32, [H, ctypes.POINTER(RenderColorsC), P]),
        "eq_fluid_add_noise": (i32, [H, u64]),
        "eq_noise_angle": (ctypes.c_double, [f32]),
        "eq_fluid_fill_obstacle_device": (i32, [H, i64, i64, i64, i64]),
        "eq_fluid_step_graph": (i32, [H, i64, i32, u64]),
        "eq_batch_new": (i32, [i64, ctypes.POINTER(SceneDescC), i32, PP]),
        "eq_batch_new_storage": (i32, [i64, ctypes.POINTER(SceneDescC), i32, i32, PP]),
        "eq_batch_free": (i32, [H]),
        "eq_batch_scene_count": (i32, [H, ctypes.POINTER(ctypes.c_int64)]),
        "eq_batch_cell_count": (i32, [H, ctypes.POINTER(ctypes.c_uint64)]),
        "eq_batch_fill_obstacle": (i32, [H, i64, i64, i64, i64, i64]),
        "eq_batch_read_cells": (i32, [H, i64, P, u64]),
        "eq_batch_set_sources": (i32, [H, i64, i64, P, P, P, P, P]),
        "eq_batch_read_field": (i32, [H, i64, i32, P, u64]),
        "eq_batch_read_fields": (i32, [H, i32, P, u64]),
        "eq_batch_write_field": (i32, [H, i64, i32, P, u64]),
        "eq_batch_step": (i32, [H, i64]),
        "eq_batch_step_eager": (i32, [H, i64]),
        "eq_batch_synchronize": (i32, [H]),
        "eq_batch_lin_solve": (i32, [H, i32, i32, i32, f32, f32]),
        "eq_batch_diffuse": (i32, [H, i32, i32, i32, f32]),
        "eq_batch_project": (i32, [H, i32, i32, i32, i32]),
        "eq_batch_advect": (i32, [H, i32, i32, i32, i32, i32]),
        "eq_batch_set_boundaries": (i32, [H, i32, i32]),
        "eq_batch_set_tuning": (i32, [H, i32, i32]),
        "eq_batch_get_tuning": (i32, [H, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_int)]),
        "eq_batch_autotune": (i32, [H, i32, ctypes.POINTER(ctypes.c_double), i32,
                                    ctypes.POINTER(ctypes.c_int)]),
        "eq_batch_get_stream": (i32, [H, PP]),
        "eq_hfluid_new": (i32, [ctypes.POINTER(FluidConfigsC), ctypes.POINTER(SimulationConfigsC),
                                i32, ctypes.c_double, i32, i32, PP]),
        "eq_hfluid_free": (i32, [H]),
        "eq_hfluid_fill_obstacle": (i32, [H, i64, i64, i64, i64]),
        "eq_hfluid_add_sources": (i32, [H, i64, P, P, P, P, P]),
        "eq_hfluid_step": (i32, [H]),
        "eq_hfluid_synchronize": (i32, [H]),
        "eq_hfluid_read_field": (i32, [H, i32, P, u64]),
        "eq_hfluid_write_field": (i32, [H, i32, P, u64]),
        "eq_hfluid_stats": (i32, [H, ctypes.POINTER(HStatsC)]),
        "eq_hfluid_get_stream": (i32, [H, PP]),
        "eq_hfluid_launch_count": (i32, [H, ctypes.POINTER(ctypes.c_uint64)]),
        "eq_hfluid_set_concurrency": (i32, [H, i32]),
        "eq_hfluid_set_solver": (i32, [H, i32]),
        "eq_batch_launch_count": (i32, [H, ctypes.POINTER(ctypes.c_uint64)]),
        "eq_grad_new": (i32, [H, i64, i64, PP]),
        "eq_grad_free": (i32, [H]),
        "eq_grad_forward": (i32, [H, i64, P, u64]),
        "eq_grad_forward_device": (i32, [H, i64, P]),
        "eq_grad_l2_loss": (i32, [H, P, u64, ctypes.POINTER(ctypes.c_double), P]),
        "eq_grad_backward": (i32, [H, P, u64, P, u64, P, u64]),
        "eq_grad_backward_device": (i32, [H, P, P, P]),
        "eq_grad_frames": (i32, [H, ctypes.POINTER(ctypes.c_int64)]),
        "eq_grad_set_wavefront_storage": (i32, [H, i32]),
        "eq_grad_set_cluster_interval": (i32, [H, i32]),
        "eq_grad_get_wavefront_storage": (i32, [H, ctypes.POINTER(ctypes.c_int),
                                                ctypes.POINTER(ctypes.c_int)]),
        "eq_grad_set_profiling": (i32, [H, i32]),
        "eq_grad_kernel_stats": (i32, [H, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_uint64)]),
        "eq_grad_launch_count": (i32, [H, ctypes.POINTER(ctypes.c_uint64)]),
        "eq_grad_set_boundaries_adj": (i32, [H, i32, P, u64]),
        "eq_grad_lin_solve_adj": (i32, [H, i32, P, P, f32, f32, u64]),
        "eq_grad_advect_adj": (i32, [H, i32, P, P, P, P, P, P, P, u64]),
        "eq_grad_project_adj": (i32, [H, P, P, P, P, u64]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path == LIB_PATH:
        _lib = L
    else:
        _others[path] = L
    return L


def load_fma():
    """The library built with FMA contraction (libeqfluid_fma.so): the plain
    form's arithmetic with a*b+c fused, within 1e-6 relative of the reference."""
    return load(LIB_FMA_PATH)


def check(rc: int, lib=None):
    if rc != EQ_OK:
        msg = (lib or load()).eq_last_error()
        raise EqError(rc, msg.decode() if msg else "")
