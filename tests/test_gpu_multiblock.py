"""Multi-block cases (several blocks per solve, joined by interfaces: CMesh::BndCondInterior,
source/BndCondInteriorPeriodic.cpp:8-34, applied before the periodic pairs,
source/BoundaryCondition.cpp:46-58, or by a mixing plane: CMesh::BndCondMixingPlane,
source/BndCondMixingPlane.cpp:287-520, applied last) through the C-ABI, against the reference's
own runs of the same cases (made by tests/golden/make_golden.py): rotor_9x9x33_3block and
rotor_9x9x33_3block_mg, the 9x9x33 passage cut at its blade's leading- and trailing-edge planes
in the arrangement of the reference's rotor-67 example; stage_9x9x17 and stage_9x9x17_mg, a
22-blade rotor at 16000 rpm and a stationary 30-blade row joined by a mixing plane. Tolerances as the single-block
parity tests: 1e-11 on geometry, 1e-10 normwise on a residual evaluation and its intermediates,
1e-9 on the driver history; the solution files as the restart tests (six printed digits)."""
import numpy as np
import pytest

from conftest import golden_dir, load_golden, rel_err
from test_gpu_restart import _compare_text

pytestmark = pytest.mark.gpu

HIST_COLS = [0, 1, 6, 7, 8, 9, 11]
R1_KEYS = ["cv", "pv", "mut", "omega", "lamcK", "lamvK", "dt", "FcK", "FvK", "FcJ", "res", "dKS_pv", "dKP_pv"]
CASES = ["rotor_9x9x33_3block", "rotor_9x9x33_3block_mg", "stage_9x9x17", "stage_9x9x17_mg"]


def _hist_err(a, b):
    a, b = a[:, HIST_COLS], b[:, HIST_COLS]
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("name", CASES)
def test_blocks_match_the_reference(name, gpu_lib, tmp_path):
    g = load_golden(name)
    nb = sum(1 for k in g if k.endswith("_g1_cell"))
    with gpu_lib.Solver(golden_dir(name), gpu_lib.FP64) as s:
        assert s.n == 1 and s.n_slots == nb and list(s.slots(0)) == list(range(nb))
        for b, slot in enumerate(s.slots(0), 1):
            for key in ("faceK", "cell", "totalvol"):
                assert rel_err(s.get(key, solve=slot), g[f"b{b}_g1_{key}"]) < 1e-11, (b, key)
        s.init_uniform()
        n = g["history"].shape[0]
        h = s.iterate(n)[:, 0, :]
        assert _hist_err(h, g["history"]) < 1e-9
        s.write_restart(0, str(tmp_path / "RestartSolution.dat"))
        s.write_solution(0, str(tmp_path / "RelativeSolution.plt"))
        s.resflux(1)
        for b, slot in enumerate(s.slots(0), 1):
            for key in R1_KEYS:
                e = rel_err(s.get(key, solve=slot), g[f"b{b}_r1_{key}"])
                assert e < 1e-10, (b, key, e)
        assert int(s.status()[0]) & 1 == 0
    same_r = _compare_text((tmp_path / "RestartSolution.dat").read_bytes(), g["restart_file"].tobytes())
    same_s = _compare_text((tmp_path / "RelativeSolution.plt").read_bytes(), g["solution_file"].tobytes())
    assert same_r > 0.98 and same_s > 0.98, (same_r, same_s)


def test_multiblock_case_in_a_batch_equals_alone(gpu_lib):
    """slots of a three-block case between single-block cases: same results as each case alone"""
    dirs = [golden_dir("rotor_9x9x33"), golden_dir("rotor_9x9x33_3block"), golden_dir("duct_9x9x17")]
    with gpu_lib.Solver(dirs, gpu_lib.FP64) as b:
        assert b.n == 3 and b.n_slots == 5
        assert list(b.slots(1)) == [1, 2, 3] and list(b.slots(2)) == [4]
        b.init_uniform()
        hb = b.iterate(6)
        for q, d in enumerate(dirs):
            with gpu_lib.Solver(d, gpu_lib.FP64) as s:
                s.init_uniform()
                hs = s.iterate(6)[:, 0, :]
                assert np.array_equal(hb[:, q, HIST_COLS], hs[:, HIST_COLS]), d
                for sb, ss in zip(b.slots(q), s.slots(0)):
                    assert np.array_equal(b.get("cv", solve=sb), s.get("cv", solve=ss))


def test_multiblock_restart_round_trip(gpu_lib, tmp_path):
    """the three-block restart file written by the GPU reads back into the same state (to the six
    printed digits), block by block"""
    name = "rotor_9x9x33_3block"
    with gpu_lib.Solver(golden_dir(name), gpu_lib.FP64) as s:
        s.init_uniform()
        s.iterate(4, history=False)
        s.write_restart(0, str(tmp_path / "r.dat"))
        before = [s.get("cv", solve=q)[1:-1, 1:-1, 1:-1] for q in s.slots(0)]
        s.read_restart(0, str(tmp_path / "r.dat"))
        after = [s.get("cv", solve=q)[1:-1, 1:-1, 1:-1] for q in s.slots(0)]
    for a, b in zip(before, after):
        assert rel_err(b, a) < 1e-5


def test_mixed_form_of_a_multiblock_case_tracks_fp64(gpu_lib):
    name = "rotor_9x9x33_3block_mg"
    res = {}
    for prec in (gpu_lib.FP64, gpu_lib.MIXED):
        with gpu_lib.Solver(golden_dir(name), prec) as s:
            s.init_uniform()
            res[prec] = s.iterate(12)[:, 0, :]
    a, b = res[gpu_lib.MIXED], res[gpu_lib.FP64]
    for col in (6, 7, 8):
        assert float(np.max(np.abs(a[:, col] - b[:, col]) / np.abs(b[:, col]))) < 1e-4


def test_noalloc_norm_of_a_multiblock_case(gpu_lib):
    name = "rotor_9x9x33_3block"
    with gpu_lib.Solver([golden_dir(name), golden_dir("rotor_9x9x33")], gpu_lib.FP64) as s:
        s.init_uniform()
        s.iterate(3, history=False)
        a = s.res_calculate(1)
        b = s.res_calculate_noalloc(1)
    assert a.shape == (2, 5) and b.shape == (2, 5)
    assert float(np.max(np.abs(a - b) / np.abs(a))) < 1e-12
