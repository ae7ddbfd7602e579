"""Imposed mass flow through the back pressure (CSolver::MassFlowImposed with the driver's
conditions, source/Solver.cpp:142-145 and source/Structured_FV3D.cpp:186-193), against the
reference run of the same case (fixture rotor_9x9x33_massflow: 25 kg/s imposed, relaxation 0.2,
every 2 iterations, residual gate 1.0, 20 iterations). The back pressure the reference used in
every iteration is recorded in the fixture; the GPU's after each iteration must be the one the
reference used in the next. Tolerances as in the other history checks (1e-9)."""
import numpy as np
import pytest

from conftest import golden_dir, load_golden

pytestmark = pytest.mark.gpu

HIST_COLS = [0, 1, 6, 7, 8, 9, 11]


def _rel(a, b):
    return float(np.max(np.abs(a - b) / np.abs(b)))


def test_imposed_mass_flow_follows_the_reference(gpu_lib):
    g = load_golden("rotor_9x9x33_massflow")
    ref, pref = g["history"], g["pout"]
    n = ref.shape[0]
    with gpu_lib.Solver(golden_dir("rotor_9x9x33_massflow"), gpu_lib.FP64) as s:
        s.init_uniform()
        assert _rel(s.outlet_pressure(), pref[:1]) < 1e-15
        rows, pout = [], []
        for _ in range(n):
            rows.append(s.iterate(1)[0, 0])
            pout.append(s.outlet_pressure()[0])
    h = np.array(rows)
    assert _rel(h[:, HIST_COLS], ref[:, HIST_COLS]) < 1e-9
    assert _rel(np.array(pout[:-1]), pref[1:]) < 1e-9
    assert np.ptp(pref) > 0.05 * pref[0]            # the control did move the back pressure


def test_only_the_imposed_solve_moves_its_back_pressure(gpu_lib):
    dirs = [golden_dir("rotor_9x9x33_massflow"), golden_dir("rotor_9x9x33")]
    with gpu_lib.Solver(dirs, gpu_lib.FP64) as s:
        s.init_uniform()
        p0 = s.outlet_pressure()
        s.iterate(6, history=False)
        p1 = s.outlet_pressure()
    assert p1[0] != p0[0] and p1[1] == p0[1]
