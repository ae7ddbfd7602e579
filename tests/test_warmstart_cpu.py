"""The warm-start network's CPU oracle (oracle/mlp_oracle.py) on its own, no GPU: its analytic
gradient against central finite differences (float64, no rounding), its BF16 rounding, its
features, and the parameter count against the library's (gb_ws_num_params, which needs no
device)."""
import numpy as np
import pytest

import mlp_oracle as mo


def _params(rng, scale=1.0):
    p = []
    for n, k in mo.LAYERS:
        a = scale * np.sqrt(6.0 / (n + k))
        p.append(rng.uniform(-a, a, size=n * k))
        p.append(rng.uniform(-0.1, 0.1, size=n))
    return np.concatenate(p)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = _params(rng)
    x = rng.normal(size=(8, mo.N_IN))
    t = rng.normal(size=(8, mo.N_USED))
    loss, g = mo.loss_and_grad(p, x, t, emulate=False)
    assert g.shape == (mo.n_params(),)
    offs, o = [], 0
    for n, k in mo.LAYERS:
        offs.append((o, n * k, o + n * k, n))
        o += n * k + n
    idx = []
    for w0, nw, b0, nb in offs:
        idx += list(w0 + rng.integers(0, nw, size=6)) + list(b0 + rng.integers(0, nb, size=2))
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (mo.loss_and_grad(p + e, x, t, emulate=False)[0] - mo.loss_and_grad(p - e, x, t, emulate=False)[0]) / (2 * h)
        if i >= offs[-1][0] + mo.N_USED * mo.HIDDEN and i < offs[-1][2]:
            assert g[i] == 0.0                     # padded outputs carry no loss
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-9, (i, fd, g[i])


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, -2.5, 3.0e38], dtype=np.float32)
    r = mo.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                             # tie to even (down)
    assert r[2] == np.float32(1.0 + 4 * 2.0 ** -8)  # tie to even (up)
    assert r[3] == 1.0
    assert r[4] == -2.5
    assert (r.view(np.uint32) & 0xFFFF == 0).all()


def test_features_in_range():
    norm = np.array([0, 0.1, -0.2, 0.3, 0.25, 0.2, 1.2, 0.9, 0.0, 0.07, 0.08, 1.0] + [0] * 6 + [1] * 6, dtype=np.float32)
    rng = np.random.default_rng(0)
    z, r, th = rng.uniform(0, 0.3, 50), rng.uniform(0.1, 0.25, 50), rng.uniform(-0.2, 0.2, 50)
    prm = np.stack([rng.uniform(1.05, 1.3, 50), rng.uniform(0.8, 1.0, 50), rng.normal(0, 1, 50)], axis=1)
    f = mo.features(z, r, th, prm, norm)
    assert f.shape == (50, mo.N_IN)
    assert np.all(np.abs(f[:, :48]) <= 1.0 + 1e-6)
    assert np.all(f[:, 54:] == 0.0)


def test_parameter_count_matches_library(gbturbo):
    import build as pkg_build
    pkg_build.build()
    assert int(gbturbo.load().gb_ws_num_params()) == mo.n_params()
