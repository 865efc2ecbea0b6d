"""The learned warm start on the GPU: tensor-core forward and gradients
against the CPU oracle, the Adam update, training, and the warm-started
return mapping in a cutting run."""
import numpy as np
import pytest

from oracle import oracle
from sph_fem_2d_cutting_gpu_gb300 import abi, learned, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver
from test_mlp_oracle import data, random_net

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def net_with(p, norm):
    m = learned.Mlp(seed=1)
    n = abi.MlpNorm()
    n.x_mean[:] = list(norm[0:4])
    n.x_std[:] = list(norm[4:8])
    n.y_mean, n.y_std = float(norm[8]), float(norm[9])
    m.set_params(p.astype(np.float32), n)
    return m


@pytest.mark.parametrize("form", ["tensor", "warp"])
@pytest.mark.parametrize("n", [5, 128, 1000, 40_000])
def test_forward_matches_oracle(lib, n, form):
    """tensor: the tcgen05 tile kernel; warp: the warp-per-sample form the
    fused step runs in its epilogue (the packed W2 / W3 copy included)."""
    p, norm = random_net(7)
    x, _ = data(n, 8)
    m = net_with(p, norm)
    y = m.predict(x) if form == "tensor" else m.predict_warp(x)
    y_ref, _, _ = oracle.mlp_eval(p, norm, x, bf16=True)
    assert rel(y, y_ref) < 5e-3
    m.close()


def test_warp_form_tracks_training(lib):
    """The packed weight copy follows every Adam step: after training, both
    forms agree with each other and with the oracle on the trained weights."""
    p, norm = random_net(3)
    x, t = data(4096, 9)
    m = net_with(p, norm)
    m.train(x, t, epochs=2, batch=512, lr=1e-3, seed=4)
    p2, _ = m.params()
    y_ref, _, _ = oracle.mlp_eval(p2.astype(np.float64), norm, x, bf16=True)
    yt, yw = m.predict(x), m.predict_warp(x)
    m.close()
    assert rel(yt, y_ref) < 5e-3 and rel(yw, y_ref) < 5e-3
    assert rel(yw, yt) < 5e-3


@pytest.mark.parametrize("n", [100, 128 * 400 + 17])
def test_gradients_match_oracle(lib, n):
    # n = 51217: 401 tiles over 304 CTAs, so CTAs accumulate two tiles in TMEM
    p, norm = random_net(9)
    x, t = data(n, 10)
    m = net_with(p, norm)
    g, loss = m.gradients(x, t)
    _, g_ref, l_ref = oracle.mlp_eval(p, norm, x, t, bf16=True, grad=True)
    blocks = {"W1": (0, 256), "b1": (256, 320), "W2": (320, 4416), "b2": (4416, 4480), "W3": (4480, 8576),
              "b3": (8576, 8640), "W4": (8640, 8704), "b4": (8704, 8705)}
    for name, (a, b) in blocks.items():
        assert rel(g[a:b], g_ref[a:b]) < 2e-2, name
    assert abs(loss - l_ref) / l_ref < 1e-3
    _, g_exact, _ = oracle.mlp_eval(p, norm, x, t, bf16=False, grad=True)
    assert rel(g, g_exact) < 8e-2
    m.close()


def test_adam_step_matches_oracle(lib):
    p, norm = random_net(11)
    x, t = data(2048, 12)
    m = net_with(p, norm)
    g, _ = m.gradients(x, t)
    m.adam_step(x, t, 1e-3)
    p1, _ = m.params()
    want, _, _ = oracle.mlp_adam(p.astype(np.float32), np.zeros(abi.MLP_NPARAMS, np.float32),
                                 np.zeros(abi.MLP_NPARAMS, np.float32), g, 1, 1e-3)
    assert np.allclose(p1, want, rtol=1e-5, atol=1e-8)
    m.close()


def test_training_reduces_loss(lib):
    x, t = data(200_000, 13)
    m = learned.Mlp(seed=3)
    m.fit_norm(x, t)
    losses = m.train(x, t, epochs=6, batch=4096, lr=2e-3, seed=1)
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.1 * losses[0], losses
    y = m.predict(x[:5000])
    assert np.mean((y - t[:5000]) ** 2) < 0.05 * np.var(t)
    m.close()


def warm_case():
    c = setups.cutting("warm", setups.AISI1045, 60, 24, 5e-4, 1.7, 300.0, 0.004, 0.0, 5.0, 5e-4, 0.35,
                       s_min=2e-4, s_max=2.5e-3, tool_size=0.015)
    return setups.placed(c, preload_dx=0.5)


@pytest.mark.parametrize("inference", [abi.SPH_MLP_WARP, abi.SPH_MLP_TENSOR])
def test_warm_start_run(lib, inference):
    """Log the plain FP32K run, train on it, rerun with the warm start (in the
    neighbour-sum epilogue, or in the tensor-core kernel after it): fewer
    secant iterations per return mapping, same results within the secant
    tolerance's effect."""
    case = warm_case()
    steps = 300
    plain = Solver(case, abi.SPH_PREC_FP32K, place_tool=False)
    plain.jc_log_enable(2_000_000)
    plain.jc_stats(True, reset=True)
    plain.step(steps)
    rec, offered = plain.jc_log_read()
    calls0, iters0 = plain.jc_stats(True)
    F0 = plain.reduce_force()
    T0 = plain.max_T()
    P0 = plain.download(["pos", "S", "eps_pl", "T"])
    plain.close()
    assert offered == len(rec) and calls0 == len(rec) > 1000
    x, t = learned.features(learned.valid_records(rec), case.constants)
    m = learned.Mlp(seed=5)
    m.fit_norm(x, t)
    losses = m.train(x, t, epochs=30, batch=2048, lr=2e-3, seed=2)
    assert losses[-1] < 0.5 * losses[0]
    warm = Solver(case, abi.SPH_PREC_FP32K, place_tool=False)
    warm.attach_mlp(m, inference)
    warm.jc_stats(True, reset=True)
    warm.step(steps)
    assert warm.status() & abi.STATUS_BITS["secant_maxiter"] == 0
    calls1, iters1 = warm.jc_stats(True)
    F1 = warm.reduce_force()
    T1 = warm.max_T()
    P1 = warm.download(["pos", "S", "eps_pl", "T"])
    warm.close()
    m.close()
    print(f"return mappings {calls0} -> {calls1}, secant iterations per return mapping "
          f"{iters0 / calls0:.3f} -> {iters1 / calls1:.3f}; loss {losses[0]:.4f} -> {losses[-1]:.4f}; "
          f"force {F0} -> {F1}; max T {T0:.2f} -> {T1:.2f}")
    assert abs(calls1 - calls0) <= 0.02 * calls0
    assert iters1 / calls1 < iters0 / calls0, (iters0 / calls0, iters1 / calls1)
    assert np.linalg.norm(F1 - F0) <= 0.01 * np.linalg.norm(F0)
    assert abs(T1 - T0) <= 0.01 * (T0 - 300.0)
    # the two runs may order a pair of particles differently in the cell sort:
    # match particles by position before comparing fields
    from scipy.spatial import cKDTree
    d, j = cKDTree(P0["pos"]).query(P1["pos"])
    assert np.max(d) < 1e-2 * 5e-4
    for f in ("S", "eps_pl", "T"):
        assert rel(P1[f], P0[f][j]) < 1e-2, f
