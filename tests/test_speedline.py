"""Speedline driver: point directories written from a template case (CPU), and a batch of
operating points run to the reference's convergence rule on the GPU, each point's report equal
to the same point run alone (the batch computes every solve independently)."""
import os

import numpy as np
import pytest

from conftest import golden_dir


@pytest.fixture(scope="module")
def speedline():
    import speedline as sl
    return sl


def test_points_rewrite_only_the_back_pressure(speedline, tmp_path):
    t = golden_dir("duct_9x9x17")
    dirs = speedline.make_points(t, [0.90, 0.95], str(tmp_path), ratio_of="Ptin",
                                 overrides={speedline.LINE_CONVTOL: "1.0E-3"})
    base = open(os.path.join(t, "config.dat")).read().splitlines()
    for d, r in zip(dirs, (0.90, 0.95)):
        got = open(os.path.join(d, "config.dat")).read().splitlines()
        assert len(got) == len(base)
        diff = [i for i, (a, b) in enumerate(zip(got, base)) if a != b]
        assert diff == [speedline.LINE_POUT, speedline.LINE_CONVTOL]
        assert float(got[speedline.LINE_POUT].split()[0]) == pytest.approx(r * 101325.0)
        assert got[speedline.LINE_POUT].endswith("# static pressure at outlet [Pa]")
        for f in ("grid.dat", "BoundaryDefinition.dat"):
            assert os.path.exists(os.path.join(d, f))


@pytest.mark.gpu
def test_speedline_points_equal_single_solves(speedline, gpu_lib, tmp_path):
    dirs = speedline.make_points(golden_dir("duct_9x9x17"), [0.90, 0.92, 0.94], str(tmp_path), ratio_of="Ptin",
                                 overrides={speedline.LINE_CONVTOL: "1.0E-3"})
    table = speedline.run(dirs, precision=gpu_lib.FP64, max_iter=400, chunk=100)
    assert [t["case"] for t in table] == dirs
    for t in table:
        with gpu_lib.Solver(t["case"], gpu_lib.FP64) as s:
            s.init_uniform()
            h = s.iterate(t["iteration"])[-1, 0]
        assert h[6] == t["m_in"] and h[8] == t["pressure_ratio"]
        if t["converged"]:
            assert t["res_dens"] <= 1e-3 and t["mass_ratio"] <= 0.003
    m = [t["m_in"] for t in table]
    assert m[0] > m[1] > m[2]                 # higher back pressure, less mass flow
