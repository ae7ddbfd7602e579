"""gb_res_calculate_noalloc (residual norm with the library's static device scratch, no
allocation) against gb_res_calculate, called through the C-ABI. The file sorts last so that the
entry point is also exercised after every other GPU test has run in the same process.

Tolerance: 1e-13 relative per component. Both entry points sum the same per-cell terms in a fixed
order, but over different numbers of blocks, so they agree to rounding."""
import ctypes

import numpy as np
import pytest

from conftest import golden_dir

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _close(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("name,precision,dirs,level", [
    ("duct_9x9x17", "FP64", 1, 1),
    ("rotor_9x9x33_mg", "FP64", 2, 2),
    ("rotor_9x9x33_mg", "MIXED", 3, 1),
    # multi-block cases: the blocks of a case count their arrivals on its first slot, and the last
    # block to arrive folds the partials of every block of the case
    ("rotor_9x9x33_3block", "FP64", 1, 1),
    ("rotor_9x9x33_3block", "MIXED", 2, 1),
    ("rotor_9x9x33_3block_mg", "FP64", 2, 2),
])
def test_noalloc_norm_matches_res_calculate(gpu_lib, name, precision, dirs, level):
    with gpu_lib.Solver([golden_dir(name)] * dirs, getattr(gpu_lib, precision)) as s:
        s.init_uniform()
        s.iterate(8, history=False)     # past the 5 coarse-only start iterations of the multigrid case
        if level == 2:
            s.time_marching(2)
        ref = s.res_calculate(level)
        assert np.all(np.isfinite(ref)) and np.all(ref > 0)
        for _ in range(2):      # two calls in a row: the arrival counters must be back at zero
            got = s.res_calculate_noalloc(level)
            assert got.shape == ref.shape
            assert _close(got, ref) <= TOL


def test_noalloc_norm_feeds_the_driver(gpu_lib):
    """The norms it writes into the solve states are the ones the CFL ramp reads next."""
    d = golden_dir("duct_9x9x17")
    with gpu_lib.Solver(d, gpu_lib.FP64) as a, gpu_lib.Solver(d, gpu_lib.FP64) as b:
        for s in (a, b):
            s.init_uniform()
            s.iterate(3, history=False)
        a.res_calculate(1)
        b.res_calculate_noalloc(1)
        ha, hb = a.iterate(3), b.iterate(3)
        assert _close(hb[:, :, [1, 6, 7, 8]], ha[:, :, [1, 6, 7, 8]]) <= TOL


def test_noalloc_rejects_bad_arguments(gpu_lib):
    L = gpu_lib.load()
    out = np.zeros(5)
    assert L.gb_res_calculate_noalloc(None, 1, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == -1
    with gpu_lib.Solver(golden_dir("duct_9x9x17"), gpu_lib.FP64) as s:
        s.init_uniform()
        with pytest.raises(gpu_lib.GBError, match="level"):
            s.res_calculate_noalloc(2)


def test_noalloc_rejects_batches_beyond_its_scratch(gpu_lib):
    with gpu_lib.Solver([golden_dir("duct_9x9x17")] * 129, gpu_lib.FP64) as s:
        s.init_uniform()
        with pytest.raises(gpu_lib.GBError, match="GB_NOALLOC_MAX_SOLVES"):
            s.res_calculate_noalloc(1)
        assert s.res_calculate(1).shape == (129, 5)
