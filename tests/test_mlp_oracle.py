"""CPU checks of the MLP oracle (the checker of the GPU MLP kernels) and of
the host-side feature map.  No GPU needed."""
import numpy as np
import pytest

from oracle import oracle
from sph_fem_2d_cutting_gpu_gb300 import abi, learned, setups

P = oracle.MLP_NPARAMS


def random_net(seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    p = np.zeros(P)
    p[0:256] = rng.uniform(-0.5, 0.5, 256) * scale
    p[256:320] = rng.uniform(-0.5, 0.5, 64) * scale
    for off in (320, 4480):
        p[off:off + 4096] = rng.uniform(-0.125, 0.125, 4096) * scale
        p[off + 4096:off + 4160] = rng.uniform(-0.125, 0.125, 64) * scale
    p[8640:8704] = rng.uniform(-0.125, 0.125, 64) * scale
    p[8704] = 0.1
    norm = np.array([0.1, 0.2, -0.3, 0.4, 1.5, 0.7, 2.0, 0.3, -1.0, 2.0], np.float32)
    return p.astype(np.float32).astype(np.float64), norm


def data(n, seed=1):
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1, (n, 4)).astype(np.float32)
    t = (np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2] - 0.2 * x[:, 3] ** 2).astype(np.float32)
    return x, t


def test_oracle_gradient_matches_finite_differences(oracle_lib):
    p, norm = random_net()
    x, t = data(24)
    _, g, _ = oracle.mlp_eval(p, norm, x, t, bf16=False, grad=True)
    rng = np.random.default_rng(5)
    # every bias and W1/W4 entry plus a sample of the 64x64 weights
    idx = list(range(256, 320)) + list(range(0, 256, 7)) + list(range(8640, 8705))
    idx += list(rng.choice(np.arange(320, 4416), 40, replace=False)) + list(rng.choice(np.arange(4480, 8576), 40,
                                                                                      replace=False))
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp = oracle.mlp_eval(pp, norm, x, t, bf16=False)[2]
        lm = oracle.mlp_eval(pm, norm, x, t, bf16=False)[2]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8, (i, fd, g[i])


def test_oracle_bf16_mode_close_to_exact(oracle_lib):
    p, norm = random_net(3)
    x, t = data(300, 4)
    y0, g0, l0 = oracle.mlp_eval(p, norm, x, t, bf16=False, grad=True)
    y1, g1, l1 = oracle.mlp_eval(p, norm, x, t, bf16=True, grad=True)
    assert np.max(np.abs(y1 - y0)) / np.max(np.abs(y0)) < 3e-2
    assert np.max(np.abs(g1 - g0)) / np.max(np.abs(g0)) < 5e-2
    assert abs(l1 - l0) / l0 < 3e-2


def test_oracle_adam_matches_numpy(oracle_lib):
    rng = np.random.default_rng(2)
    p = rng.normal(0, 0.1, P).astype(np.float32)
    m1 = rng.normal(0, 0.01, P).astype(np.float32)
    m2 = np.abs(rng.normal(0, 0.01, P)).astype(np.float32)
    g = rng.normal(0, 0.1, P).astype(np.float32)
    lr, t = np.float32(1e-3), 3
    a = (np.float32(0.9) * m1 + (np.float32(1) - np.float32(0.9)) * g).astype(np.float32)
    v = (np.float32(0.999) * m2 + (np.float32(1) - np.float32(0.999)) * g * g).astype(np.float32)
    c1 = np.float32(1 / (1 - 0.9 ** t))
    c2 = np.float32(1 / (1 - 0.999 ** t))
    want = p - lr * (a * c1) / (np.sqrt(v * c2) + np.float32(1e-8))
    got, gm1, gm2 = oracle.mlp_adam(p.copy(), m1.copy(), m2.copy(), g, t, lr)
    assert np.allclose(got, want, rtol=1e-6, atol=1e-9)
    assert np.allclose(gm1, a, rtol=1e-6) and np.allclose(gm2, v, rtol=1e-6)


def test_features_of_logged_states():
    c = setups.make_constants(setups.AISI1045, 2.5e-4, 1.7)
    rec = np.array([[0.008, 0.1, 2e-6, 600.0, 0.0065, 3e-5, 3.0, 2.6e-4]], np.float32)
    x, t = learned.features(rec, c)
    jc = c.joco
    assert np.isclose(x[0, 0], np.log(0.008 / jc.A), rtol=1e-6)
    assert np.isclose(x[0, 1], 0.1)
    assert np.isclose(x[0, 2], np.log1p(2e-6 / jc.eps_dot_ref), rtol=1e-6)
    assert np.isclose(x[0, 3], (600.0 - jc.Tref) / (jc.Tmelt - jc.Tref), rtol=1e-6)
    assert np.isclose(t[0], np.log(2 * c.phys.G * 3e-5 / 0.0065), rtol=1e-5)


def test_valid_records_drop_undefined_targets():
    rec = np.array([[0.008, 0.1, 2e-6, 600.0, 0.0065, 3e-5, 3.0, 2.6e-4],
                    [0.0, 0.1, 0.0, 1733.0, 0.0, 0.0, 1.0, 2.6e-4],       # melted: zero deviator
                    [0.008, 0.1, 2e-6, 600.0, 0.0065, 0.0, 1.0, 2.6e-4],  # zero increment
                    [np.nan, 0.1, 2e-6, 600.0, 0.0065, 3e-5, 3.0, 2.6e-4]], np.float32)
    ok = learned.valid_records(rec)
    assert len(ok) == 1 and np.array_equal(ok[0], rec[0])
