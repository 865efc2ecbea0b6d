"""Failure paths on the GPU, driven without a fault.

- The staged neighbour copies: sph_set_test_faults(SPH_TEST_SKIP_BULK_COPY)
  makes the staged launch shape announce its bulk copies and issue none, so
  the bounded wait runs out (1 s): the step reports SPH_STATUS_COPY_TIMEOUT,
  falls back to global loads and gives the results of an undisturbed run.
- The learned warm start: SPH_TEST_SKIP_MMA issues no tensor-core MMA, so the
  wait runs out: SPH_STATUS_MMA_TIMEOUT, the kernel frees its TMEM (the next
  steps allocate it again and run), and the warm start works again once the
  knob is cleared.
- NaN and Inf in the uploaded state: do_invalidate blanks the particles whose
  rates turn non-finite (SPH_STATUS_NAN_BLANKED), in the same set as the CPU
  oracle's.  The set reaches past the kernel support: the reference runs the
  pair body for every active particle of the cell stencil, with zero weights
  outside the support, and 0 x NaN is NaN.
- A lowered secant cap (no iteration past the first): SPH_STATUS_SECANT_MAXITER
  in both precision forms.
"""
import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, learned, setups, tune
from sph_fem_2d_cutting_gpu_gb300.solver import Solver
from oracle.oracle import OracleSim

pytestmark = pytest.mark.gpu

SKIP_BULK_COPY, SKIP_MMA = 1, 2
STATE = ["pos", "vel", "rho", "S", "T", "eps_pl", "eps_pl_dot", "blanked", "hash", "idx"]


def set_faults(s, faults, cap=-1):
    s._ck(s.lib.sph_set_test_faults(s.ctx, faults, cap), "sph_set_test_faults")


def staged_variant():
    for v, (_, _, staged, _) in enumerate(tune.launch_variants()):
        if staged:
            return v
    pytest.skip("no staged launch shape compiled")


def test_copy_timeout_falls_back_to_global_loads(lib):
    c = setups.micro(n_side=64, seed=4, cell_factor=2, stencil=1)
    runs = {}
    for name, faults in (("plain", 0), ("skip", SKIP_BULK_COPY)):
        s = Solver(c, abi.SPH_PREC_FP32K)
        tune.set_variant(s, staged_variant())
        set_faults(s, faults)
        s.step()
        runs[name] = (s.status(), s.download(STATE))
        set_faults(s, 0)
        s.step()
        runs[name + "_after"] = s.status()
        s.close()
    assert runs["plain"][0] == 0
    assert runs["skip"][0] & abi.STATUS_BITS["copy_timeout"]
    assert runs["skip_after"] == 0 and runs["plain_after"] == 0
    for f in STATE:
        assert np.array_equal(runs["skip"][1][f], runs["plain"][1][f]), f


def warm_case():
    c = setups.cutting("warm", setups.AISI1045, 60, 24, 5e-4, 1.7, 300.0, 0.004, 0.0, 5.0, 5e-4, 0.35,
                       s_min=2e-4, s_max=2.5e-3, tool_size=0.015)
    return setups.placed(c, preload_dx=0.5)


def test_mma_timeout_frees_tmem_and_recovers(lib):
    case = warm_case()
    rng = np.random.default_rng(0)
    m = learned.Mlp(seed=3)
    m.fit_norm(rng.normal(size=(4096, 4)).astype(np.float32), rng.normal(size=4096).astype(np.float32))
    s = Solver(case, abi.SPH_PREC_FP32K, place_tool=False)
    s.step(40)                                   # plastic flow under the tool
    s.attach_mlp(m, abi.SPH_MLP_TENSOR)          # the tensor-core tile kernel and its bounded waits
    s.jc_stats(True, reset=True)
    s.step(2)
    calls, _ = s.jc_stats(True, reset=True)
    assert calls > 0, "no yielding particles: the warm start would not run"
    assert s.status() & abi.STATUS_BITS["mma_timeout"] == 0
    set_faults(s, SKIP_MMA)
    s.step()
    assert s.status() & abi.STATUS_BITS["mma_timeout"]
    set_faults(s, 0)
    s.step(5)                                    # TMEM was freed: the next steps allocate it and run
    assert s.status() & abi.STATUS_BITS["mma_timeout"] == 0
    s.jc_stats(True, reset=True)
    s.step(2)
    assert s.jc_stats(True, reset=True)[0] > 0
    s.close()
    m.close()


def test_nan_and_inf_inputs_are_blanked_like_the_oracle(lib):
    c = setups.micro(n_side=48, seed=6)
    P = c.particles
    P["vel"][100, 0] = np.nan
    P["S"][500, 1] = np.inf
    P["S_t"][900, 2] = -np.inf
    s = Solver(c)
    o = OracleSim(c.constants, c.grid, s.download(), c.dt)
    s.step()
    st_o = o.step()
    G = s.download()
    assert s.status() & abi.STATUS_BITS["nan_blanked"]
    assert st_o & abi.STATUS_BITS["nan_blanked"]
    assert np.array_equal(G["blanked"], o.P["blanked"])
    assert (G["blanked"] == 1.0).sum() >= 3


@pytest.mark.parametrize("precision", [abi.SPH_PREC_FP64, abi.SPH_PREC_FP32K], ids=["fp64", "fp32k"])
def test_lowered_secant_cap_reports_maxiter(lib, precision):
    case = warm_case()
    flags = {}
    for cap in (-1, 0):                          # the reference's cap, then none past the first iteration
        s = Solver(case, precision, place_tool=False)
        set_faults(s, 0, cap)
        s.step(60)
        flags[cap] = s.status()
        s.close()
    assert flags[-1] & abi.STATUS_BITS["secant_maxiter"] == 0
    assert flags[0] & abi.STATUS_BITS["secant_maxiter"]
