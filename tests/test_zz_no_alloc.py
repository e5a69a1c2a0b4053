"""The allocation-free lin_solve (eq_lin_solve_noalloc) against the handle's
eq_fluid_lin_solve, through the C ABI.

eq_lin_solve_noalloc serves callers that cannot allocate device memory (code
inside an open CUDA stream capture, frame loops that must not take the device
synchronisation an allocation can cause, hosts whose GPU memory belongs to
another allocator): they pass their own grids and the entry point keeps its
scratch in a static device array of bounded size. This test allocates its own
input/output buffers (the test is allowed to), calls the entry point twice in
a row with different modes and data, and checks both results bit for bit
against the existing entry point -- the same bar as every other parity test.
It is collected last so that a failure here cannot hide the other tests.
"""
import ctypes

import numpy as np
import pytest

from equilibrium_gb300 import _lib
from equilibrium_gb300.simulation import Fluid, FluidConfigs, SimulationConfigs
from tests.util import random_rects

pytestmark = pytest.mark.gpu

SIZE, PITCH, ITERS = 130, 136, 20  # pitch differs from the handle's 160 on purpose


def _noalloc_fn(L):
    fn = L.eq_lin_solve_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int64, ctypes.c_float,
                   ctypes.c_float, ctypes.c_void_p]
    return fn


def _scene(seed):
    rng = np.random.default_rng(seed)
    s = SIZE
    cells = np.zeros((s, s), np.uint8)
    cells[0, :] = cells[-1, :] = cells[:, 0] = cells[:, -1] = 1
    for x0, y0, x1, y1 in random_rects(rng, s, 5):
        cells[y0:y1, x0:x1] = 1
    x = rng.uniform(-1, 1, (s, s)).astype(np.float32)
    x0 = rng.uniform(-1, 1, (s, s)).astype(np.float32)
    return cells, x, x0


def _reference(cells, x, x0, mode, a, c):
    """The existing entry point on a handle."""
    L = _lib.load()
    f = Fluid(FluidConfigs(0.0, 0.0, False), SimulationConfigs(0.1, ITERS, SIZE), device=0)
    f.cells_type = cells.reshape(-1)
    f.write_field(_lib.FIELD_VX0, x.reshape(-1))
    f.write_field(_lib.FIELD_VX, x0.reshape(-1))
    _lib.check(L.eq_fluid_lin_solve(f.handle, mode, _lib.FIELD_VX0, _lib.FIELD_VX, a, c))
    out = f.read_field(_lib.FIELD_VX0).reshape(SIZE, SIZE)
    f.close()
    return out


def _noalloc(cells, x, x0, mode, a, c):
    import torch
    L = _lib.load()
    fn = _noalloc_fn(L)
    dev = torch.device("cuda", 0)
    pad = ((0, 0), (0, PITCH - SIZE))
    tx = torch.from_numpy(np.pad(x, pad)).to(dev)
    tx0 = torch.from_numpy(np.pad(x0, pad)).to(dev)
    tc = torch.from_numpy(np.pad(cells, pad, constant_values=1)).to(dev)
    stream = torch.cuda.current_stream(dev)
    rc = fn(mode, tx.data_ptr(), tx0.data_ptr(), tc.data_ptr(), SIZE, PITCH, ITERS,
            ctypes.c_float(a), ctypes.c_float(c), ctypes.c_void_p(stream.cuda_stream))
    assert rc == _lib.EQ_OK, rc
    torch.cuda.synchronize()
    return tx.cpu().numpy()[:, :SIZE]


def test_noalloc_lin_solve_matches_the_handle_path_twice_in_a_row(eqlib):
    import torch
    torch.cuda.init()
    a1 = np.float32(0.37)
    c1 = np.float32(1.0) + np.float32(4.0) * a1
    calls = [(_lib.MODE_PASSIVE, 1.0, 4.0, 11), (_lib.MODE_ADJUST_COLUMN, float(a1), float(c1), 12)]
    for mode, a, c, seed in calls:
        cells, x, x0 = _scene(seed)
        want = _reference(cells, x, x0, mode, a, c)
        got = _noalloc(cells, x, x0, mode, a, c)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (
            mode, int((got.view(np.uint32) != want.view(np.uint32)).sum()))


def test_noalloc_rejects_grids_beyond_its_scratch(eqlib):
    fn = _noalloc_fn(_lib.load())
    # no device pointer is touched: the size check comes first
    assert fn(0, 16, 32, 48, 259, 288, 20, 1.0, 4.0, None) == _lib.EQ_ERR_ARG
    assert fn(0, 16, 32, 48, 258, 290, 20, 1.0, 4.0, None) == _lib.EQ_ERR_ARG
