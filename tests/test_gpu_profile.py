"""sph_profile_steps issues the fused step stage by stage, with CUDA events
between the stages and no graph: the state it leaves must be the one the
graph-replayed step leaves (the tool with the wear shift, the rigid tool with
PSE conduction, the micro workload in FP32K), and the stage times must be
there.  Tolerances: float fields 1e-10 relative norm-wise (the contact and
friction sums add with atomics, in launch order), flags and the cell list
bit-exact."""
import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import PROFILE_STAGES, Solver
from conftest import rel_err
from test_gpu_parity import EXACT, RATES, RTOL, STATE

pytestmark = pytest.mark.gpu

WC = abi.WearConstants(10.0, 300.0, 10.0, 300.0)


def same_state(s1, s2, what):
    A, B = s1.download(), s2.download()
    act = A["blanked"] != 1
    for f in STATE + RATES:
        a, b = (A[f][act], B[f][act]) if f in RATES else (A[f], B[f])
        assert rel_err(a, b) <= RTOL, f"{what} {f}"
    for f in EXACT:
        assert np.array_equal(A[f], B[f]), f"{what} {f}"
    assert s1.status() == 0 and s2.status() == 0


def check_stages(ms, steps):
    assert tuple(ms) == PROFILE_STAGES
    assert all(v >= 0 for v in ms.values())
    assert ms["neighbour sums+epilogue"] > 0 and sum(ms.values()) > 0


def wear_solver(precision):
    c = setups.small_cut()
    s = Solver(c, precision)
    s.move_tool(0.3 * c.info["dx"] / c.tool_speed)
    s.set_wear(abi.SPH_WEAR_SHIFT, WC)
    return s


@pytest.mark.parametrize("precision", [abi.SPH_PREC_FP64, abi.SPH_PREC_FP32K], ids=["fp64", "fp32k"])
def test_profile_follows_fused_with_wear(lib, precision):
    s1, s2 = wear_solver(precision), wear_solver(precision)
    s1.step(5)
    check_stages(s2.profile_steps(5), 5)
    same_state(s1, s2, "[wear]")
    w1, w2 = s1.wear_state(), s2.wear_state()
    assert np.max(w1["wear_nodes"]) > 0
    for k in ("M", "phys_para", "wear_nodes"):
        assert rel_err(w1[k], w2[k]) <= 1e-10, k
    f1, f2 = s1.fem(), s2.fem()
    for k in ("position", "T", "M_inv"):
        assert rel_err(f1[k], f2[k]) <= 1e-10, k
    assert s1.tool_state().flank_retreat == pytest.approx(s2.tool_state().flank_retreat, rel=1e-9, abs=1e-16)


@pytest.mark.parametrize("precision", [abi.SPH_PREC_FP64, abi.SPH_PREC_FP32K], ids=["fp64", "fp32k"])
def test_profile_follows_fused_rigid_pse(lib, precision):
    c = setups.ref_cut(ny=8, length=0.02, preload_dx=1.5)
    s1, s2 = Solver(c, precision), Solver(c, precision)
    for s in (s1, s2):
        s.set_thermal_model(abi.SPH_THERMAL_PSE)
    s1.step(4)
    check_stages(s2.profile_steps(4), 4)
    same_state(s1, s2, "[rigid pse]")
    t1, t2 = s1.rigid_tool(), s2.rigid_tool()
    assert [t1.left[i][0] for i in range(t1.n_seg)] == [t2.left[i][0] for i in range(t2.n_seg)]


def test_profile_then_graph_steps_continue(lib):
    """Profiled steps and graph steps interleave on one context."""
    c = setups.micro(n_side=64)
    s1, s2 = Solver(c, abi.SPH_PREC_FP32K), Solver(c, abi.SPH_PREC_FP32K)
    s1.step(6)
    s2.step(2)
    check_stages(s2.profile_steps(2), 2)
    s2.step(2)
    same_state(s1, s2, "[micro]")
