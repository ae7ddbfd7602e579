"""Parity at the benchmark sizes: the FP64 GPU path against the CPU oracle on the 129x49x49 rotor
passage of the benchmark (two-level FAS, the start-up iterations and the first full cycles) and
on the largest mesh of the sampled batch (161x65x65), history at 1e-9 and the final state at
1e-10, as the small parity cases; and the batch and graph properties that do not depend on
size: a batch of the two passages gives the same bits as each alone, graph replay the same bits
as eager launches."""
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


@pytest.mark.parametrize("dims,n", [((49, 49, 129), 4), ((65, 65, 161), 3)])
def test_fp64_matches_oracle_at_benchmark_size(gpu_lib, oracle_mod, meshgen, tmp_path, dims, n):
    d = _passage(meshgen, tmp_path / "case", *dims)
    o = oracle_mod.Oracle(d)
    ref = o.run(n)
    with gpu_lib.Solver(d, gpu_lib.FP64) as s:
        s.init_uniform()
        h = s.iterate(n)[:, 0, :]
        assert _hist_err(h, ref) < 1e-9
        cv = s.get("cv")[1:-1, 1:-1, 1:-1]
    assert rel_err(cv, o.get("cv")[1:-1, 1:-1, 1:-1]) < 1e-10


def test_batch_and_graphs_are_bitwise_at_benchmark_size(gpu_lib, meshgen, tmp_path):
    a = _passage(meshgen, tmp_path / "a", 49, 49, 129, 1.10)
    b = _passage(meshgen, tmp_path / "b", 65, 65, 161, 1.25)
    with gpu_lib.Solver([a, b], gpu_lib.MIXED) as s:
        s.init_uniform()
        hb = s.iterate(6)
        cvb = [s.get("cv", solve=q) for q in range(2)]
    for q, d in enumerate((a, b)):
        for graphs in (True, False):
            with gpu_lib.Solver(d, gpu_lib.MIXED) as s:
                s.set_graphs(graphs)
                s.init_uniform()
                h = s.iterate(6)[:, 0, :]
                assert np.array_equal(h[:, HIST_COLS], hb[:, q, HIST_COLS]), (d, graphs)
                assert np.array_equal(s.get("cv"), cvb[q]), (d, graphs)
