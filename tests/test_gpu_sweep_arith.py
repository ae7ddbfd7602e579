"""The FP64 form's optional double-float LU-SGS sweep (gb_set_sweep_arith: the dQ-dependent half of
every hyperplane, the flux difference in delta form, the combination and the division by the
diagonal, in pairs of FP32 numbers with about 47 significant bits). It is not the reference's
rounding, so it is held to what that precision gives: at the benchmark size, four iterations from
the uniform start against the oracle at the FP64 sweep's own bars (history 1e-9, state 1e-10;
measured 9e-12); the converged rotor against the reference's long run is in
test_gpu_converged.py. Also: graph replay gives the same bits as eager launches, switching back
gives the FP64 sweep's bits, and a mixed-precision handle refuses the option."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

HIST_COLS = [0, 1, 6, 7, 8, 9, 11]


def _passage(meshgen, path, IM, JM, KM, pb=1.20):
    case = meshgen.rotor_passage(IM=IM, JM=JM, KM=KM, options={
        "Pout": "%.1f" % (pb * 101325.0), "multigrid": "Y", "coarse_iter": "2", "Ma0": "0.45"})
    meshgen.write_case(case, str(path))
    return str(path)


def _hist_err(a, b):
    a, b = a[:, HIST_COLS], b[:, HIST_COLS]
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def test_double_float_sweep_matches_oracle_at_benchmark_size(gpu_lib, oracle_mod, meshgen, tmp_path):
    d = _passage(meshgen, tmp_path / "case", 49, 49, 129)
    o = oracle_mod.Oracle(d)
    ref = o.run(4)
    with gpu_lib.Solver(d, gpu_lib.FP64) as s:
        s.set_sweep_arith(True)
        s.init_uniform()
        h = s.iterate(4)[:, 0, :]
        assert _hist_err(h, ref) < 1e-9
        cv = s.get("cv")[1:-1, 1:-1, 1:-1]
    assert rel_err(cv, o.get("cv")[1:-1, 1:-1, 1:-1]) < 1e-10


def test_graphs_switching_and_refusal(gpu_lib, meshgen, tmp_path):
    d = _passage(meshgen, tmp_path / "case", 17, 17, 33, 1.10)
    runs = {}
    for key, df, graphs in (("df_graphs", True, True), ("df_eager", True, False), ("fp64", False, True),
                            ("df_then_fp64", None, True)):
        with gpu_lib.Solver(d, gpu_lib.FP64) as s:
            s.set_graphs(graphs)
            if df is None:
                s.set_sweep_arith(True)
                s.set_sweep_arith(False)
            else:
                s.set_sweep_arith(df)
            s.init_uniform()
            runs[key] = (s.iterate(8)[:, 0, :], s.get("cv"))
    assert np.array_equal(runs["df_graphs"][0], runs["df_eager"][0], equal_nan=True)
    assert np.array_equal(runs["df_graphs"][1], runs["df_eager"][1])
    assert np.array_equal(runs["df_then_fp64"][1], runs["fp64"][1])
    # the two sweeps differ in the last bits only
    assert not np.array_equal(runs["df_graphs"][1], runs["fp64"][1])
    assert rel_err(runs["df_graphs"][1][1:-1, 1:-1, 1:-1], runs["fp64"][1][1:-1, 1:-1, 1:-1]) < 1e-10
    with gpu_lib.Solver(d, gpu_lib.MIXED) as s:
        with pytest.raises(gpu_lib.GBError):
            s.set_sweep_arith(True)
        s.set_sweep_arith(False)
