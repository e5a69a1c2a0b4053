"""CPU tests of the drop-in boundary: the CUDA library builds for sm_103a,
loads, and exports every function include/eqfluid.h declares; argument
checks that need no device; the host-side API mirror's validation."""
import ctypes

import pytest

from equilibrium_gb300 import _lib


@pytest.fixture(scope="module")
def L():
    from equilibrium_gb300 import build
    build.build()
    return _lib.load()


def test_every_header_function_is_exported(L):
    names = _lib.header_functions()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_abi_version(L):
    assert L.eq_abi_version() == 1


def test_rectangle_check_mirrors_obstacle_rs(L):
    # obstacle.rs:97-115: both reference tests must panic
    assert L.eq_rectangle_check(50, 120, 127, 110, 128) == _lib.EQ_ERR_ARG
    assert L.eq_last_error() == b"Invalid input for Rectangle"
    assert L.eq_rectangle_check(12, 12, 10, 10, 128) == _lib.EQ_ERR_ARG
    assert L.eq_rectangle_check(80, 80, 110, 110, 128) == _lib.EQ_OK


def test_null_arguments_are_rejected_without_a_device(L):
    assert L.eq_fluid_step(None) == _lib.EQ_ERR_ARG
    assert L.eq_fluid_free(None) == _lib.EQ_OK
    out = ctypes.c_void_p()
    sim = _lib.SimulationConfigsC(0.1, 20, 10)  # size < 20 underflows fluid.rs:534
    fl = _lib.FluidConfigsC(0.0, 0.0, 0)
    assert L.eq_fluid_new(ctypes.byref(fl), ctypes.byref(sim), -1, ctypes.byref(out)) == \
        _lib.EQ_ERR_ARG
    sim = _lib.SimulationConfigsC(0.1, -1, 64)
    assert L.eq_fluid_new(ctypes.byref(fl), ctypes.byref(sim), -1, ctypes.byref(out)) == \
        _lib.EQ_ERR_ARG


def test_python_rectangle_raises_like_the_reference_panics(L):
    from equilibrium_gb300 import InvalidRectangle, Rectangle
    with pytest.raises(InvalidRectangle):
        Rectangle((50, 120), (127, 110), 128)
    with pytest.raises(InvalidRectangle):
        Rectangle((12, 12), (10, 10), 128)
    r = Rectangle.default()
    assert r.get_approximate_points() == [(80, 80), (110, 110)]
