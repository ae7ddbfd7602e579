"""The learned warm start on the GPU (gb_ws_*): the tcgen05 products of the network against the
CPU oracle (oracle/mlp_oracle.py, BF16 rounding at the kernels' storage points, float64
accumulation): outputs at 1e-2 (the fused inference kernel, which gb_ws_forward runs, and its
bitwise equality with the layer-by-layer forward that training uses) and every parameter gradient at 3e-2 relative (normwise per
tensor; the kernels accumulate in FP32 in another order, and one BF16 ulp of a stored
intermediate is 4e-3); the fallback rule; and what a trained network gains over the uniform start
on a family of small rotor passages."""
import numpy as np
import pytest

import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def _params(seed):
    rng = np.random.default_rng(seed)
    p = []
    for l, (n, k) in enumerate(mo.LAYERS):
        a = np.sqrt(6.0 / (n + k))
        w = rng.uniform(-a, a, size=(n, k))
        if l == len(mo.LAYERS) - 1:
            w[mo.N_USED:] = 0.0
        p.append(w.ravel())
        p.append(rng.uniform(-0.2, 0.2, size=n) * (np.arange(n) < (mo.N_USED if l == 5 else n)))
    return np.concatenate(p).astype(np.float32)


def _split(flat):
    out, o = [], 0
    for n, k in mo.LAYERS:
        out.append(flat[o:o + n * k])
        o += n * k
        out.append(flat[o:o + n])
        o += n
    return out


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("M", [128, 1000, 4133])
def test_forward_matches_oracle(gpu_lib, M):
    p = _params(1)
    x = np.random.default_rng(M).uniform(-1.0, 1.0, size=(M, mo.N_IN)).astype(np.float32)
    with gpu_lib.WarmStart(seed=5) as w:
        w.set_params(p)
        assert np.array_equal(w.get_params(), p)
        y = w.forward(x)
    yo, _ = mo.forward(p, x)
    assert _rel(y[:, :mo.N_USED], yo[:, :mo.N_USED]) < 1e-2
    assert np.all(y[:, mo.N_USED:] == 0.0)


@pytest.mark.parametrize("M", [4133, 65536])
def test_fused_inference_equals_the_layer_by_layer_forward(gpu_lib, M):
    """the fused inference kernel (every layer in one launch, activations in shared memory and TMEM)
    runs the layer-by-layer forward's arithmetic in the same order: the same bits on random rows,
    including a last tile with fewer than 128 rows"""
    with gpu_lib.WarmStart(seed=9) as w:
        ms_f, ms_s, ms_i, dmax = w.benchmark(M, iters=2)
    assert ms_f > 0.0 and ms_s > 0.0 and ms_i > 0.0
    assert dmax == 0.0, dmax


@pytest.mark.parametrize("M", [256, 1777])
def test_gradients_match_oracle(gpu_lib, M):
    p = _params(2)
    rng = np.random.default_rng(7 + M)
    x = rng.uniform(-1.0, 1.0, size=(M, mo.N_IN)).astype(np.float32)
    t = rng.normal(size=(M, mo.N_USED)).astype(np.float32)
    with gpu_lib.WarmStart(seed=5) as w:
        w.set_params(p)
        loss, g = w.forward_backward(x, t)
    loss_o, go = mo.loss_and_grad(p, x, t)
    assert abs(loss - loss_o) / loss_o < 1e-2
    for q, (a, b) in enumerate(zip(_split(g), _split(go))):
        if np.linalg.norm(b) == 0.0:
            assert np.all(a == 0.0), q
            continue
        assert _rel(a, b) < 3e-2, (q, _rel(a, b))


def test_untrained_network_falls_back_to_the_uniform_start(gpu_lib, meshgen, tmp_path):
    """random weights give a field with a larger residual than the uniform start: every case falls
    back, and the run is the plain start-up, bit for bit"""
    case = meshgen.rotor_passage(IM=9, JM=9, KM=33, options={"multigrid": "Y", "coarse_iter": "2"})
    meshgen.write_case(case, str(tmp_path))
    with gpu_lib.Solver(str(tmp_path), gpu_lib.MIXED) as s:
        s.init_uniform()
        h0 = s.iterate(8)
    with gpu_lib.WarmStart(seed=11) as w:
        w.set_norm([0.0, 0.1, -0.2, 0.2, 0.25, 0.2, 1.2, 1.0, 0.0, 0.1, 0.1, 1.0,
                    1.2, 0.5, 0.1, 0.1, 2.5, 0.0, 0.2, 0.2, 0.2, 0.2, 0.5, 1e-4])
        with gpu_lib.Solver(str(tmp_path), gpu_lib.MIXED) as s:
            used, rw, ru = w.apply(s, [[1.2, 1.0, 0.0]])
            assert used[0] == 0 and not rw[0] < ru[0]
            h1 = s.iterate(8)
    assert np.array_equal(h0, h1, equal_nan=True)       # (the reference's momentum norms are NaN where Q_old is 0)


def _cycles_to(h, ref, tol):
    """first cycle from which mass flow and pressure ratio both stay within tol of ref"""
    err = np.maximum(np.abs(h[:, 6] - ref[6]) / abs(ref[6]), np.abs(h[:, 8] - ref[8]) / abs(ref[8]))
    bad = np.nonzero(err >= tol)[0]
    return 0 if bad.size == 0 else int(bad[-1]) + 1


def test_trained_network_reaches_the_converged_integrals_sooner(gpu_lib, meshgen, tmp_path):
    """a family of 17 x 17 x 33 rotor passages (two-level multigrid, mixed form): the network
    trained on the fields of five back pressures (600 cycles each) starts a held-out one (1.20 x
    p_t), which reaches the converged mass flow and pressure ratio of the uniform start's 600-cycle
    solve (within 2e-3) in at most half the cycles of the uniform start, and ends on the same state"""
    def case(pb, name):
        d = str(tmp_path / name)
        meshgen.write_case(meshgen.rotor_passage(IM=17, JM=17, KM=33, options={
            "Pout": "%.1f" % (pb * 101325.0), "multigrid": "Y", "coarse_iter": "2", "Ma0": "0.45"}), d)
        return d
    pbs = [1.05, 1.10, 1.15, 1.25, 1.30]
    train = [case(pb, f"t{q}") for q, pb in enumerate(pbs)]
    held = case(1.20, "held")
    with gpu_lib.WarmStart(seed=1) as w:
        with gpu_lib.Solver(train, gpu_lib.MIXED) as s:
            s.init_uniform()
            s.iterate(600, history=False)
            w.add_solves(s, [[pb, 1.0, 0.0] for pb in pbs])
        assert w.samples == 5 * 16 * 16 * 32
        first = w.train(100, batch=16384, lr=1e-3)
        last = w.train(1900, batch=16384, lr=1e-3)
        assert last < 0.5 * first
        with gpu_lib.Solver(held, gpu_lib.MIXED) as s:
            s.init_uniform()
            ref = s.iterate(600)[-1, 0, :]
        n = 300
        with gpu_lib.Solver(held, gpu_lib.MIXED) as s:
            s.init_uniform()
            hu = s.iterate(n)[:, 0, :]
        with gpu_lib.Solver(held, gpu_lib.MIXED) as s:
            used, rw, ru = w.apply(s, [[1.20, 1.0, 0.0]])
            assert used[0] == 1 and rw[0] < ru[0]
            hw = s.iterate(n)[:, 0, :]
    cu, cw = _cycles_to(hu, ref, 2e-3), _cycles_to(hw, ref, 2e-3)
    assert cw <= n // 2 and cw <= cu // 2, (cw, cu)
    assert np.all(np.isfinite(hw[:, [6, 7, 8, 9]]))
    for col in (6, 8, 9):
        assert abs(hw[-1, col] - ref[col]) / abs(ref[col]) < 2e-3, col
