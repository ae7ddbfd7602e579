"""GPU path through the C-ABI against the reference's own outputs (golden fixtures) and the CPU
oracle. FP64 tolerance: 1e-10 normwise relative on a residual evaluation and its intermediate
arrays, 1e-9 relative on the driver history (density residual norm, mass flows, pressure ratio,
efficiency) -- the GPU reassociates sums and contracts multiply-adds, so it is not bitwise."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, REFERENCE_ONLY_CASES, golden_dir, load_golden, rel_err

pytestmark = pytest.mark.gpu

R1_KEYS = ["cv", "pv", "mut", "ev", "res_ev", "omega", "lamcI", "lamcJ", "lamcK", "lamvI", "lamvJ", "lamvK", "dt", "FcI", "FcJ",
           "FcK", "FvI", "FvJ", "FvK", "res", "dIS_pv", "dIP_pv", "dJS_pv", "dJP_pv", "dKS_pv", "dKP_pv", "dIS_cv",
           "dKP_cv"]
HIST_COLS = [0, 1, 6, 7, 8, 9, 11]     # iter, Res.dens, m_in, m_out, PR, eta, CFL (others divide by zero momenta)
TOL_FIELD = 1e-10
TOL_HIST = 1e-9


def hist_err(a, b):
    a, b = a[:, HIST_COLS], b[:, HIST_COLS]
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("name", GOLDEN_CASES + REFERENCE_ONLY_CASES)
def test_fp64_matches_reference(name, gpu_lib):
    g = load_golden(name)
    with gpu_lib.Solver(golden_dir(name), gpu_lib.FP64) as s:
        for key in ("faceI", "faceJ", "faceK", "cell", "totalvol", "dwall"):
            if "g1_" + key in g:
                assert rel_err(s.get(key), g["g1_" + key]) < 1e-11, key
        s.init_uniform()
        n = g["history"].shape[0]
        h = s.iterate(n)[:, 0, :]
        assert hist_err(h, g["history"]) < TOL_HIST
        s.resflux(1)
        for key in R1_KEYS:
            if "r1_" + key in g:
                e = rel_err(s.get(key), g["r1_" + key])
                assert e < TOL_FIELD, (key, e)
        assert s.status()[0] & 1 == 0


def test_fp64_matches_oracle_larger_duct(gpu_lib, oracle_mod, meshgen, tmp_path):
    case = meshgen.annular_duct(IM=17, JM=17, KM=33)
    meshgen.write_case(case, str(tmp_path))
    o = oracle_mod.Oracle(str(tmp_path))
    ref = o.run(30)
    with gpu_lib.Solver(str(tmp_path), gpu_lib.FP64) as s:
        s.init_uniform()
        h = s.iterate(30)[:, 0, :]
        assert hist_err(h, ref) < TOL_HIST
        cv = s.get("cv")[1:-1, 1:-1, 1:-1]
        assert rel_err(cv, o.get("cv")[1:-1, 1:-1, 1:-1]) < TOL_FIELD


def test_fp64_matches_oracle_multigrid_rotor(gpu_lib, oracle_mod, meshgen, tmp_path):
    case = meshgen.rotor_passage(IM=17, JM=17, KM=65, options={"multigrid": "Y", "coarse_iter": "6"})
    meshgen.write_case(case, str(tmp_path))
    o = oracle_mod.Oracle(str(tmp_path))
    ref = o.run(16)
    with gpu_lib.Solver(str(tmp_path), gpu_lib.FP64) as s:
        assert s.ng == 2
        s.init_uniform()
        h = s.iterate(16)[:, 0, :]
        assert hist_err(h, ref) < TOL_HIST


def test_batch_equals_individual_solves(gpu_lib, meshgen, tmp_path):
    dirs = []
    for q, (dims, pb) in enumerate([((9, 9, 33), 1.20), ((13, 9, 41), 1.15)]):
        c = meshgen.rotor_passage(IM=dims[0], JM=dims[1], KM=dims[2], options={"Pout": "%.1f" % (pb * 101325.0)})
        d = str(tmp_path / f"c{q}")
        meshgen.write_case(c, d)
        dirs.append(d)
    with gpu_lib.Solver(dirs, gpu_lib.FP64) as b:
        b.init_uniform()
        hb = b.iterate(8)
        for q, d in enumerate(dirs):
            with gpu_lib.Solver(d, gpu_lib.FP64) as s:
                s.init_uniform()
                hs = s.iterate(8)[:, 0, :]
                assert np.array_equal(hb[:, q, HIST_COLS], hs[:, HIST_COLS])
                assert np.array_equal(b.get("cv", solve=q), s.get("cv"))


def test_graph_replay_equals_eager(gpu_lib):
    name = "rotor_9x9x33_mg"
    out = []
    for graphs in (True, False):
        with gpu_lib.Solver(golden_dir(name), gpu_lib.FP64) as s:
            s.set_graphs(graphs)
            s.init_uniform()
            out.append((s.iterate(10)[:, 0, HIST_COLS], s.get("cv")))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


def test_call_surface_step_by_step_equals_driver(gpu_lib):
    """gb_solver_step + gb_integrals (the reference's CSolver::Solver and OutputGeneralParameters
    called one by one) give the driver loop's history."""
    name = "duct_9x9x17"
    g = load_golden(name)
    with gpu_lib.Solver(golden_dir(name), gpu_lib.FP64) as s:
        s.init_uniform()
        rows = []
        for _ in range(5):
            s.solver_step()
            res = s.res_calculate(1)      # recomputed from Q_old, Q: same norm
            integ = s.integrals(1)[0]
            rows.append([res[0, 0], integ[0], integ[1], integ[2], integ[3]])
        rows = np.array(rows)
        ref = g["history"][:5][:, [1, 6, 7, 8, 9]]
        assert float(np.max(np.abs(rows - ref) / np.abs(ref))) < TOL_HIST


def test_mixed_precision_tracks_fp64(gpu_lib):
    name = "rotor_9x9x33"
    res = {}
    for prec in (gpu_lib.FP64, gpu_lib.MIXED):
        with gpu_lib.Solver(golden_dir(name), prec) as s:
            s.init_uniform()
            res[prec] = s.iterate(20)[:, 0, :]
    a, b = res[gpu_lib.MIXED], res[gpu_lib.FP64]
    # mass flows, pressure ratio within 1e-4 relative after 20 iterations
    for col in (6, 7, 8):
        assert float(np.max(np.abs(a[:, col] - b[:, col]) / np.abs(b[:, col]))) < 1e-4


def test_bad_case_is_reported(gpu_lib, meshgen, tmp_path):
    case = meshgen.annular_duct(IM=9, JM=9, KM=17, options={"scheme": "400"})
    meshgen.write_case(case, str(tmp_path))
    with pytest.raises(gpu_lib.GBError, match="not on this path"):
        gpu_lib.Solver(str(tmp_path))


def test_prolongation_of_a_synthetic_coarse_field(gpu_lib):
    """CSolver::Interpolate alone: the fine field interpolated from a coarse field with distinct
    values in every cell, ghosts included (set through the state of a coarse start-up phase)."""
    name = "rotor_9x9x33_mg"
    with gpu_lib.Solver(golden_dir(name), gpu_lib.FP64) as s:
        s.init_uniform()
        s.iterate(3)                        # coarse-level iterations fill the coarse ghosts
        I, J, K, _ = s.dims(0, 2)
        rng = np.random.default_rng(1)
        cvc = s.get("cv", level=2).copy()
        cvc[1:-1, 1:-1, 1:-1] *= 1.0 + 0.01 * rng.standard_normal(cvc[1:-1, 1:-1, 1:-1].shape)
        s.set_cv(cvc[1:-1, 1:-1, 1:-1], level=2)
        s.corner_treatment(2)
        s.interpolate(True)
        C = s.get("cv", level=2)
        F = s.get("cv", level=1)

        def nb(n):
            return (n // 2, n // 2 + 1) if n % 2 == 0 else (n // 2 + 1, n // 2)
        IF, JF, KF, _ = s.dims(0, 1)
        P = np.zeros_like(F)
        for i in range(1, IF):
            a1, a2 = nb(i)
            for j in range(1, JF):
                b1, b2 = nb(j)
                for k in range(1, KF):
                    c1, c2 = nb(k)
                    P[i, j, k] = (27 / 64 * C[a1, b1, c1] + 9 / 64 * (C[a1, b1, c2] + C[a1, b2, c1] + C[a2, b1, c1])
                                  + 3 / 64 * (C[a2, b2, c1] + C[a1, b2, c2] + C[a2, b1, c2]) + 1 / 64 * C[a2, b2, c2])
        sl = (slice(1, -1),) * 3
        assert rel_err(F[sl], P[sl]) < 1e-14


def test_sweep_autotuner_picks_a_candidate(gpu_lib):
    shapes = {(1, 1), (2, 1), (4, 1), (10, 1), (4, 4), (10, 4), (10, 8)}
    with gpu_lib.Solver(golden_dir("rotor_9x9x33_mg"), gpu_lib.MIXED) as s:
        assert s.sweep_tuning(1) == (10, 1) and s.sweep_tuning(2) == (10, 1)     # small batch: default shape
        with pytest.raises(gpu_lib.GBError):
            s.sweep_tuning(3)
    with gpu_lib.Solver([golden_dir("rotor_9x9x33_mg")] * 4, gpu_lib.MIXED) as s:  # timed candidates
        assert s.sweep_tuning(1) in shapes and s.sweep_tuning(2) in shapes


def test_mixed_precision_jst_tracks_fp64(gpu_lib):
    name = "rotor_9x9x33_jst_mg"
    res = {}
    for prec in (gpu_lib.FP64, gpu_lib.MIXED):
        with gpu_lib.Solver(golden_dir(name), prec) as s:
            s.init_uniform()
            res[prec] = s.iterate(12)[:, 0, :]
    a, b = res[gpu_lib.MIXED], res[gpu_lib.FP64]
    for col in (6, 7, 8):
        assert float(np.max(np.abs(a[:, col] - b[:, col]) / np.abs(b[:, col]))) < 1e-4


def test_spalart_allmaras_restart_round_trip(gpu_lib, tmp_path):
    """the restart file of a Spalart-Allmaras case carries the variable as a twelfth column and
    reads back into the same state (to the six printed digits)"""
    name = "rotor_9x9x33_sa"
    with gpu_lib.Solver(golden_dir(name), gpu_lib.FP64) as s:
        s.init_uniform()
        s.iterate(4, history=False)
        s.write_restart(0, str(tmp_path / "r.dat"))
        ev = s.get("ev")[1:-1, 1:-1, 1:-1]
        s.read_restart(0, str(tmp_path / "r.dat"))
        ev2 = s.get("ev")[1:-1, 1:-1, 1:-1]
        h = s.iterate(3)[:, 0, :]
    assert all(len(l.split()) == 12 for l in open(tmp_path / "r.dat").read().splitlines()[:50])
    assert rel_err(ev2, ev) < 1e-5
    assert np.all(np.isfinite(h[:, HIST_COLS]))


def test_mixed_precision_spalart_allmaras_tracks_fp64(gpu_lib):
    name = "rotor_9x9x33_sa"
    res = {}
    for prec in (gpu_lib.FP64, gpu_lib.MIXED):
        with gpu_lib.Solver(golden_dir(name), prec) as s:
            s.init_uniform()
            res[prec] = s.iterate(12)[:, 0, :]
    a, b = res[gpu_lib.MIXED], res[gpu_lib.FP64]
    for col in (6, 7, 8):
        assert float(np.max(np.abs(a[:, col] - b[:, col]) / np.abs(b[:, col]))) < 1e-4


def test_spalart_allmaras_with_multigrid_is_refused(gpu_lib, meshgen, tmp_path):
    case = meshgen.annular_duct(IM=9, JM=9, KM=17, options={"turb": "200", "multigrid": "Y", "coarse_iter": "2"})
    meshgen.write_case(case, str(tmp_path))
    with pytest.raises(gpu_lib.GBError, match="single grid"):
        gpu_lib.Solver(str(tmp_path))
