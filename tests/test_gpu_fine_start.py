"""Starting from a given fine field (gb_start_from_fine_state, the path of the learned warm start):
the field set by gb_set_cv, the coarse levels' time steps and spectral radii evaluated once at the
restricted field, then full cycles from the first iteration with the fine level's integrals
reported. A case started from the field another run reached follows that run's own continuation
(the integrals within 1e-3, the density residual at most three times the continuation's), with a two-level cycle, a
three-block case and the three-level extension. Before the coarse evaluation the first cycle
turned to NaN (zero coarse time steps); before the reporting fix the captured cycle graph replayed
the coarse level's integrals (pressure ratio 8% off)."""
import numpy as np
import pytest

from conftest import golden_dir

pytestmark = pytest.mark.gpu


def _rotor(meshgen, path, KM=65):
    meshgen.write_case(meshgen.rotor_passage(IM=17, JM=17, KM=KM, options={
        "Pout": "%.1f" % (1.10 * 101325.0), "multigrid": "Y", "coarse_iter": "3", "Ma0": "0.45"}), str(path))
    return str(path)


def _continued_and_restarted(gpu_lib, d, levels, n, prec):
    with gpu_lib.Solver(d, prec, levels=levels) as s:
        s.init_uniform()
        s.iterate(n, history=False)
        cvs = [s.get("cv", solve=q)[1:-1, 1:-1, 1:-1] for q in s.slots(0)]
        hc = s.iterate(6)[:, 0, :]
    with gpu_lib.Solver(d, prec, levels=levels) as s:
        s.init_uniform()
        for q, cv in zip(s.slots(0), cvs):
            s.set_cv(cv, solve=q)
        s.start_from_fine_state()
        dt2 = s.get("dt", solve=0, level=2)
        h2 = s.iterate(6)[:, 0, :]
    return hc, h2, dt2


@pytest.mark.parametrize("case,levels", [("rotor_17x17x65", 2), ("rotor_17x17x65", 3), ("rotor_9x9x33_3block_mg", 2)])
def test_restart_from_a_field_follows_the_continuation(gpu_lib, meshgen, tmp_path, case, levels):
    d = _rotor(meshgen, tmp_path / "c") if case == "rotor_17x17x65" else golden_dir(case)
    hc, h2, dt2 = _continued_and_restarted(gpu_lib, d, levels, 800, gpu_lib.FP64)
    assert np.all(np.isfinite(h2[:, [1, 6, 7, 8, 9]]))
    assert np.all(dt2 > 0.0)                                # the coarse level's time steps were evaluated
    for col in (6, 7, 8):                                   # m_in, m_out, pressure ratio of the fine level
        err = np.abs(h2[:, col] - hc[:, col]) / np.abs(hc[:, col])
        assert np.all(err < 1e-3), (col, err)
    assert np.all(h2[:, 1] < 3.0 * hc[:, 1] + 1e-7)
