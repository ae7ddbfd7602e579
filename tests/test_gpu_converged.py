"""Long runs on the GPU against the reference's own 2000-iteration history of the 65x33x33 annular
duct (Roe + MUSCL3, Baldwin-Lomax, LU-SGS, CFL 3, single grid; fixture written by
tests/golden/make_golden.py from the reference build, case regenerated here by the same
generator call).

Bars: the FP64 GPU path reproduces the reference's integrals (mass flow in and out, total
pressure ratio, efficiency) after 2000 iterations to 1e-6 relative; the mixed-precision form
stays within 0.1% in mass flow and 1e-4 in total-pressure ratio of the FP64 GPU solve."""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

NAME = "duct_33x33x65_2000"
INTEGRALS = {"m_in": 6, "m_out": 7, "PR": 8, "eta": 9}


@pytest.fixture(scope="module")
def long_case(tmp_path_factory, meshgen):
    ref = np.load(f"{GOLDEN}/{NAME}.npz")["history"]
    d = str(tmp_path_factory.mktemp("long") / NAME)
    meshgen.write_case(meshgen.annular_duct(IM=33, JM=33, KM=65, options={}, name=NAME), d)
    return d, ref


@pytest.fixture(scope="module")
def fp64_history(long_case, gpu_lib):
    d, ref = long_case
    with gpu_lib.Solver(d, gpu_lib.FP64) as s:
        s.init_uniform()
        return s.iterate(ref.shape[0])[:, 0, :]


def test_fp64_integrals_after_2000_iterations(long_case, fp64_history):
    _, ref = long_case
    h = fp64_history
    assert h.shape == ref.shape
    for name, col in INTEGRALS.items():
        err = abs(h[-1, col] - ref[-1, col]) / abs(ref[-1, col])
        assert err < 1e-6, (name, h[-1, col], ref[-1, col], err)
    # the density residual follows the reference's convergence history
    rd = np.abs(h[:, 1] - ref[:, 1]) / np.abs(ref[:, 1])
    assert float(rd.max()) < 1e-4, float(rd.max())


def test_mixed_form_tracks_fp64_gpu(long_case, fp64_history, gpu_lib):
    d, ref = long_case
    with gpu_lib.Solver(d, gpu_lib.MIXED) as s:
        s.init_uniform()
        h = s.iterate(ref.shape[0])[:, 0, :]
    f = fp64_history
    for col in (INTEGRALS["m_in"], INTEGRALS["m_out"]):
        assert abs(h[-1, col] - f[-1, col]) / abs(f[-1, col]) < 1e-3
    assert abs(h[-1, INTEGRALS["PR"]] - f[-1, INTEGRALS["PR"]]) < 1e-4
