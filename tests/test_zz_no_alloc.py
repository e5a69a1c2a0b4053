"""The allocation-free lin_solve (eq_lin_solve_noalloc) against the handle's
eq_fluid_lin_solve, through the C ABI.

eq_lin_solve_noalloc serves callers that cannot allocate device memory: a
solver embedded in a host application whose own allocator or budget owns all
device memory, and frame loops that must not take the device-wide
synchronisation of a cudaMalloc / cudaFree. They pass their own grids and the
entry point keeps its scratch in a static device array of bounded size. This
test allocates its own input/output buffers (the test is allowed to), calls
the entry point several times in a row with different modes, sizes, pitches
and sweep counts, and checks every result bit for bit against the existing
entry point -- the same bar as every other parity test. It is collected last
so that a failure here cannot hide the other tests.
"""
import ctypes

import numpy as np
import pytest

from equilibrium_gb300 import _lib
from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
from tests.util import random_rects

pytestmark = pytest.mark.gpu


def _noalloc_fn(L):
    fn = L.eq_lin_solve_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int64, ctypes.c_float,
                   ctypes.c_float, ctypes.c_void_p]
    return fn


def _scene(seed, size):
    rng = np.random.default_rng(seed)
    cells = np.zeros((size, size), np.uint8)
    cells[0, :] = cells[-1, :] = cells[:, 0] = cells[:, -1] = 1
    for x0, y0, x1, y1 in random_rects(rng, size, 5):
        cells[y0:y1, x0:x1] = 1
    x = rng.uniform(-1, 1, (size, size)).astype(np.float32)
    x0 = rng.uniform(-1, 1, (size, size)).astype(np.float32)
    return cells, x, x0


def _reference(cells, x, x0, mode, a, c, iters):
    """The existing entry point on a handle."""
    size = cells.shape[0]
    L = _lib.load()
    f = Fluid(FluidConfigs(0.0, 0.0, False), SimulationConfigs(0.1, iters, size), device=0)
    f.cells_type = cells.reshape(-1)
    f.write_field(_lib.FIELD_VX0, x.reshape(-1))
    f.write_field(_lib.FIELD_VX, x0.reshape(-1))
    _lib.check(L.eq_fluid_lin_solve(f.handle, mode, _lib.FIELD_VX0, _lib.FIELD_VX, a, c))
    out = f.read_field(_lib.FIELD_VX0).reshape(size, size)
    f.close()
    return out


def _noalloc(cells, x, x0, mode, a, c, iters, pitch):
    """One call of the entry point on padded device copies; returns (rc, x)."""
    import torch
    size = cells.shape[0]
    fn = _noalloc_fn(_lib.load())
    dev = torch.device("cuda", 0)
    pad = ((0, 0), (0, pitch - size))
    tx = torch.from_numpy(np.pad(x, pad)).to(dev)
    tx0 = torch.from_numpy(np.pad(x0, pad)).to(dev)
    tc = torch.from_numpy(np.pad(cells, pad, constant_values=1)).to(dev)
    stream = torch.cuda.current_stream(dev)
    rc = fn(mode, tx.data_ptr(), tx0.data_ptr(), tc.data_ptr(), size, pitch, iters,
            ctypes.c_float(a), ctypes.c_float(c), ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    return rc, tx.cpu().numpy()[:, :size]


def _diffusion_coeffs(a):
    a = np.float32(a)
    return float(a), float(np.float32(1.0) + np.float32(4.0) * a)


# (mode, a, c, seed, size, pitch, sweeps): the pressure form and both velocity
# forms; a pitch unlike the handle's; more than 64 sweeps (three wavefront
# launches with the tags carried between them); the largest grid the scratch
# holds, at its largest pitch.
CALLS = [
    (_lib.MODE_PASSIVE, 1.0, 4.0, 11, 130, 136, 20),
    (_lib.MODE_ADJUST_COLUMN, *_diffusion_coeffs(0.37), 12, 130, 136, 20),
    (_lib.MODE_ADJUST_ROW, *_diffusion_coeffs(0.91), 13, 98, 100, 20),
    (_lib.MODE_ADJUST_COLUMN, *_diffusion_coeffs(0.05), 14, 66, 68, 150),
    (_lib.MODE_ADJUST_ROW, *_diffusion_coeffs(0.2), 15, 258, 288, 20),
]


def test_noalloc_lin_solve_matches_the_handle_path_call_after_call(eqlib):
    import torch
    torch.cuda.init()
    for mode, a, c, seed, size, pitch, iters in CALLS:
        cells, x, x0 = _scene(seed, size)
        want = _reference(cells, x, x0, mode, a, c, iters)
        rc, got = _noalloc(cells, x, x0, mode, a, c, iters, pitch)
        assert rc == _lib.EQ_OK, (mode, size, iters, rc)
        diff = int((got.view(np.uint32) != want.view(np.uint32)).sum())
        assert diff == 0, (mode, size, pitch, iters, diff)


def test_noalloc_rejects_a_frame_with_a_hole_before_touching_x(eqlib):
    import torch
    torch.cuda.init()
    cells, x, x0 = _scene(21, 66)
    cells[0, 17] = 0  # a fluid cell on the ghost frame
    rc, got = _noalloc(cells, x, x0, _lib.MODE_PASSIVE, 1.0, 4.0, 20, 68)
    assert rc == _lib.EQ_ERR_ARG
    assert np.array_equal(got.view(np.uint32), x.view(np.uint32))
    # the next call with a valid mask is unaffected by the rejected one
    cells[0, 17] = 1
    want = _reference(cells, x, x0, _lib.MODE_PASSIVE, 1.0, 4.0, 20)
    rc, got = _noalloc(cells, x, x0, _lib.MODE_PASSIVE, 1.0, 4.0, 20, 68)
    assert rc == _lib.EQ_OK
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_noalloc_rejects_grids_beyond_its_scratch(eqlib):
    fn = _noalloc_fn(_lib.load())
    # no device pointer is touched: the size check comes first
    assert fn(0, 16, 32, 48, 259, 288, 20, 1.0, 4.0, None) == _lib.EQ_ERR_ARG
    assert fn(0, 16, 32, 48, 258, 290, 20, 1.0, 4.0, None) == _lib.EQ_ERR_ARG
