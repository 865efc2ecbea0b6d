"""The fused FP32K step as one persistent cooperative launch
(SPH_STEP_PERSISTENT) against the same step as its chain of graph-replayed
launches: the same per-element code in the same stage order, so the same
results bit for bit -- without a tool, with the FEM tool, for a batched context
of uneven cases, and with the learned warm start in the neighbour-sum
epilogue.  Its grid barriers are bounded: a block that never arrives (a test
knob) ends the launch with SPH_STATUS_GRID_TIMEOUT instead of a hang."""
import ctypes as C
import time

import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, learned, setups, tune
from sph_fem_2d_cutting_gpu_gb300.solver import Batch, Solver
from test_gpu_batch import small_cases
from conftest import rel_err

pytestmark = pytest.mark.gpu

STATE = ["pos", "vel", "rho", "S", "T", "eps_pl", "eps_pl_dot", "fc", "ft", "n", "pos_t", "vel_t", "rho_t", "S_t",
         "T_t", "on_seg", "blanked", "fixed", "tool_particle", "hash"]
STEPS = 40


def solver_run(case, form, steps=STEPS, mlp=None, place=True):
    s = Solver(case, abi.SPH_PREC_FP32K, place_tool=place)
    if mlp is not None:
        s.attach_mlp(mlp)
    tune.set_step_form(s, form)
    s.step(2)                              # the first step starts from the FP64 upload (launches)
    n0 = s.launch_count()
    s.step(steps - 2)
    per_step = (s.launch_count() - n0) / (steps - 2)
    P = s.download(STATE)
    T = s.fem()["T"] if case.tool_mesh is not None else None
    st = s.status()
    s.close()
    return P, T, st, per_step


def assert_same(a, b, what=""):
    for f in a:
        assert np.array_equal(a[f], b[f], equal_nan=True), \
            f"{what}{f}: {np.count_nonzero(a[f] != b[f])} entries differ"


@pytest.mark.parametrize("name", ["micro", "small_cut", "ti64_cut"])
def test_persistent_step_is_bit_identical(lib, name):
    case = setups.micro(n_side=96) if name == "micro" else getattr(setups, name)()
    P0, T0, st0, n_launch = solver_run(case, abi.SPH_STEP_LAUNCHES)
    P1, T1, st1, n_pers = solver_run(case, abi.SPH_STEP_PERSISTENT)
    assert_same(P1, P0)
    if T0 is not None:
        assert np.array_equal(T1, T0)
    assert st1 == st0
    assert st1 & abi.STATUS_BITS["grid_timeout"] == 0
    assert n_pers == 1 and n_launch > 1, (n_pers, n_launch)


def test_persistent_batched_cases(lib):
    cases = small_cases()
    out = {}
    for form in (abi.SPH_STEP_LAUNCHES, abi.SPH_STEP_PERSISTENT):
        b = Batch(cases, abi.SPH_PREC_FP32K)
        tune.set_step_form(b, form)
        b.step(STEPS)
        out[form] = (b.download_cases(STATE), b.reduce(), b.fem_T(), b.status())
        b.close()
    (P0, r0, T0, s0), (P1, r1, T1, s1) = out[abi.SPH_STEP_LAUNCHES], out[abi.SPH_STEP_PERSISTENT]
    for k in range(len(cases)):
        assert_same(P1[k], P0[k], f"case {k}: ")
        assert np.array_equal(T1[k], T0[k])
    assert np.array_equal(r1, r0) and s1 == s0


def test_persistent_with_learned_warm_start(lib):
    """The warp-level forward pass inside the persistent kernel's neighbour sums.
    In this instantiation nvcc contracts a few products of the corrector into FMAs
    differently from the separate kernel's, so the two runs part at FP32
    rounding from the first persistent step on and then drift apart as any two
    FP32 runs of a plastic flow do: 1e-5 norm-wise after 12 steps (8e-5 in the
    stress after 60).  Each form alone is deterministic run to run."""
    from test_gpu_mlp import warm_case
    case = warm_case()
    rng = np.random.default_rng(2)
    m = learned.Mlp(seed=4)
    m.fit_norm(rng.normal(size=(4096, 4)).astype(np.float32), rng.normal(size=4096).astype(np.float32))
    P0, T0, st0, _ = solver_run(case, abi.SPH_STEP_LAUNCHES, steps=12, mlp=m, place=False)
    P1, T1, st1, _ = solver_run(case, abi.SPH_STEP_PERSISTENT, steps=12, mlp=m, place=False)
    P2, _, _, _ = solver_run(case, abi.SPH_STEP_PERSISTENT, steps=12, mlp=m, place=False)
    m.close()
    assert_same(P2, P1)                       # deterministic
    for f in ("on_seg", "blanked", "fixed", "tool_particle", "hash"):
        assert np.array_equal(P1[f], P0[f]), f
    for f in ("pos", "vel", "rho", "S", "T", "eps_pl", "eps_pl_dot", "fc", "ft"):
        assert rel_err(P1[f], P0[f]) <= 1e-5, f
    assert rel_err(T1, T0) <= 1e-6 and st1 == st0


def test_persistent_form_is_fp32k_only(lib):
    s = Solver(setups.micro(n_side=32), abi.SPH_PREC_FP64)
    cfg = tune.get_config(s)
    cfg.step_form = abi.SPH_STEP_PERSISTENT
    assert s.lib.sph_set_launch_config(s.ctx, C.byref(cfg)) == abi.SPH_ERR_STATE
    cfg.step_form = 7
    assert s.lib.sph_set_launch_config(s.ctx, C.byref(cfg)) == abi.SPH_ERR_INVALID
    s.close()


def test_grid_barrier_timeout_ends_the_launch(lib):
    """Block 0 skips its first arrival: every wait runs out after about 1 s,
    the step reports SPH_STATUS_GRID_TIMEOUT, and the context keeps working."""
    case = setups.micro(n_side=64)
    s = Solver(case, abi.SPH_PREC_FP32K)
    tune.set_step_form(s, abi.SPH_STEP_PERSISTENT)
    s.step(2)
    s.sync()
    assert s.status() & abi.STATUS_BITS["grid_timeout"] == 0
    s._ck(s.lib.sph_set_test_faults(s.ctx, abi.SPH_TEST_SKIP_GRID_ARRIVAL, -1), "sph_set_test_faults")
    t0 = time.perf_counter()
    s.step()
    s.sync()
    el = time.perf_counter() - t0
    assert s.status() & abi.STATUS_BITS["grid_timeout"]
    assert el < 10.0, el
    s._ck(s.lib.sph_set_test_faults(s.ctx, 0, -1), "sph_set_test_faults")
    s.upload(case.particles)                 # a fresh state; the next steps run normally
    s.step(3)
    s.sync()
    assert s.status() & abi.STATUS_BITS["grid_timeout"] == 0
    s.close()
