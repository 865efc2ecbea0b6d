"""GPU parity against the CPU oracle, through the C ABI.

Integer/index work (hashes, sort permutation, cell tables, contact segment
ids, blanking) is compared bit-exactly; FP64 fields within 1e-10 relative
(norm-wise: max|a-b| / max(max|b|, rms b)).  Rates of blanked particles are
excluded: in the reference they are garbage computed from stale slots.
"""
import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver
from oracle.oracle import OracleSim
from conftest import rel_err

pytestmark = pytest.mark.gpu

RTOL = 1e-10
STATE = ["pos", "vel", "rho", "S", "T", "eps_pl", "eps_pl_dot", "p", "R", "fc", "ft", "n", "h"]
RATES = ["pos_t", "vel_t", "rho_t", "S_t", "T_t"]
EXACT = ["hash", "idx", "on_seg", "blanked", "fixed", "tool_particle"]


def pair(case, precision=abi.SPH_PREC_FP64, preload_dx=0.0):
    s = Solver(case, precision)
    if s.has_tool and preload_dx:
        # push the tool into the workpiece so contact is active from the first step
        v = case.tool_speed
        dx = case.info["dx"]
        s.move_tool(preload_dx * dx / v)
    P = s.download()
    tool = None
    if s.has_tool:
        ts = s.tool_state()
        tool = dict(segments=s.segments(), fem=s.fem(), state=ts, n_cut_colors=ts.n_cut_colors)
    o = OracleSim(case.constants, case.grid, P, case.dt, tool=tool)
    return s, o


def compare(s, o, fields=STATE + RATES + EXACT, rtol=RTOL, what=""):
    G = s.download()
    act = o.P["blanked"] != 1.0
    errs = {}
    for f in fields:
        a, b = G[f], o.P[f]
        if f in RATES:
            a, b = a[act], b[act]
        if f in EXACT:
            assert np.array_equal(a, b), f"{what} {f}: {np.count_nonzero(a != b)} entries differ"
        else:
            e = rel_err(a, b)
            errs[f] = e
            assert e <= rtol, f"{what} {f}: relative error {e:.3e} > {rtol:.1e}"
    if s.has_tool and o.tool:
        seg = s.segments()
        for k in ("left", "right"):
            assert np.array_equal(seg[k], o.seg[k]), f"{what} segments {k}"
        assert rel_err(seg["heat_exchange"], o.seg["heat_exchange"]) <= rtol, f"{what} heat_exchange"
        fem = s.fem()
        assert rel_err(fem["T"], o.fem["T"]) <= rtol, f"{what} FEM T"
    return errs


# ---- cell list: bit-exact ----------------------------------------------------------------------
def shuffled_micro(n=96, seed=11):
    c = setups.micro(n_side=n, seed=seed)
    rng = np.random.default_rng(seed)
    perm = rng.permutation(c.N)
    c.particles = {k: np.ascontiguousarray(v[perm]) for k, v in c.particles.items()}
    return c


def test_cells_bit_exact(lib):
    c = shuffled_micro()
    s, o = pair(c)
    for rep in range(3):
        s.assign_hashes()
        s.sort()
        o.assign_hashes()
        o.sort()
        G = s.download()
        for f in ["hash", "idx"]:
            assert np.array_equal(G[f], o.P[f]), f
        cs, ce = s.cells()
        assert np.array_equal(cs, o.cell_start)
        ne = cs != -1
        assert np.array_equal(ce[ne], o.cell_end[ne])
        for f in STATE[:7] + ["fc", "ft", "n", "h", "fixed", "blanked", "on_seg"] + RATES:
            if f in ("p", "R"):
                continue
            assert np.array_equal(G[f], o.P[f]), f"sort moved {f} differently"
        # perturb positions between sorts so the permutation changes
        P = s.download(["pos"])
        P["pos"] += np.random.default_rng(rep).normal(0, 0.3 * c.info["dx"], P["pos"].shape)
        s.upload(P)
        o.P["pos"][:] = P["pos"]


def test_cells_blanked_and_out_of_grid(lib):
    c = shuffled_micro(n=48, seed=2)
    P = c.particles
    P["blanked"][::7] = 1.0          # blanked keep their (stale) hash
    P["hash"][::7] = 5
    P["pos"][3] = [-1.0, -1.0]       # outside the grid
    P["pos"][10] = [50.0, 0.0]
    s, o = pair(c)
    s.assign_hashes()
    s.sort()
    o.assign_hashes()
    o.sort()
    G = s.download()
    assert np.array_equal(G["hash"], o.P["hash"])
    assert np.array_equal(G["idx"], o.P["idx"])
    cs, ce = s.cells()
    assert np.array_equal(cs, o.cell_start)
    assert s.status() & abi.STATUS_BITS["out_of_grid"]


# ---- every stage of leap_frog::step in the reference order ----------------------------------------
def staged_sequence(s, o, has_tool, check):
    dt = o.dt
    s.update_geometry()
    s.assign_hashes(); o.assign_hashes()
    s.sort(); o.sort()
    check("sort", STATE[:7] + ["fc", "ft", "n"] + RATES + EXACT)
    s.init(); o.init()
    if has_tool:
        s.fem_reset_server(); o.fem_reset_server()
    s.predict(); o.predict()
    if has_tool:
        s.fem_calculate_temp(0.5 * dt); o.fem_calculate_temp(0.5 * dt)
    check("predict", ["pos", "vel", "S", "rho", "T"])
    s.material_eos(); o.material_eos()
    check("eos", ["p"])
    s.corrector_artificial_stress(); o.corrector_artificial_stress()
    check("artificial stress", ["R"])
    s.interactions_monaghan(); o.interactions_monaghan()
    check("interactions", ["S_der", "v_der", "pos_t", "vel_t", "T_t"])
    s.material_stress_rate_jaumann(); o.material_stress_rate_jaumann()
    check("jaumann", ["S_t"])
    s.contmech_continuity(); o.contmech_continuity()
    check("continuity", ["rho_t"])
    s.contmech_momentum(); o.contmech_momentum()
    check("momentum", ["vel_t"])
    s.contmech_advection(); o.contmech_advection()
    check("advection", ["pos_t"])
    s.correct(); o.correct()
    check("correct", ["pos", "vel", "S", "rho", "T"])
    if has_tool:
        s.material_fric_heat_gen_fem(); o.material_fric_heat_gen_fem()
        check("friction heat", ["T", "blanked"])
        s.fem_apply_robin(); o.fem_apply_robin()
        s.fem_calculate_temp_rate(); o.fem_calculate_temp_rate()
        s.fem_calculate_temp(dt); o.fem_calculate_temp(dt)
    s.plasticity_johnson_cook(); o.plasticity_johnson_cook()
    check("plasticity", ["S", "eps_pl", "eps_pl_dot", "T", "blanked"])
    if has_tool:
        s.move_tool(dt); o.move_tool(dt)
        s.compute_contact_forces_fem(); o.compute_contact_forces_fem()
        check("contact", ["fc", "ft", "n", "on_seg", "T", "blanked"])
    s.perform_boundary_conditions(); o.perform_boundary_conditions()
    s.perform_boundary_conditions_thermal(); o.perform_boundary_conditions_thermal()
    s.debug_invalidate(); o.debug_invalidate()
    check("bc+invalidate", STATE + RATES + EXACT)


@pytest.mark.parametrize("kind", ["micro", "cut"])
def test_stage_by_stage(lib, kind):
    if kind == "micro":
        c = shuffled_micro(n=64, seed=4)
        s, o = pair(c)
    else:
        c = setups.small_cut()
        s, o = pair(c, preload_dx=0.3)

    def check(stage, fields):
        compare(s, o, fields, what=f"[{kind}:{stage}]")

    for _ in range(2):
        staged_sequence(s, o, s.has_tool, check)
    if kind == "cut":
        G = s.download(["on_seg"])
        assert (G["on_seg"] >= 0).sum() > 0, "contact never became active"


# ---- fused, graph-captured step ------------------------------------------------------------------
FUSED = STATE + RATES + EXACT


@pytest.mark.parametrize("kind", ["micro", "micro_2h", "cut"])
def test_fused_step_matches_oracle(lib, kind):
    if kind == "micro":
        c = shuffled_micro(n=80, seed=9)
        s, o = pair(c)
    elif kind == "micro_2h":
        c = setups.micro(n_side=80, seed=9, cell_factor=2, stencil=1)
        s, o = pair(c)
    else:
        c = setups.small_cut()
        s, o = pair(c, preload_dx=0.3)
    for k in range(4):
        s.step()
        o.step()
        compare(s, o, FUSED, what=f"[{kind} step {k}]")
    assert s.status() == 0


def test_staged_step_matches_fused(lib):
    c = setups.small_cut()
    s1, o = pair(c, preload_dx=0.3)
    s2 = Solver(c)
    s2.move_tool(0.3 * c.info["dx"] / c.tool_speed)
    for _ in range(3):
        s1.step()
        s2.step_staged()
    A, B = s1.download(), s2.download()
    act = A["blanked"] != 1
    for f in STATE + RATES:
        a, b = (A[f][act], B[f][act]) if f in RATES else (A[f], B[f])
        assert rel_err(a, b) <= RTOL, f
    for f in EXACT:
        assert np.array_equal(A[f], B[f]), f


def test_fp32_compensated_full_size_2h(lib):
    """The headline workload itself (2048 x 2048 = 4,194,304 particles, cells of
    2h / 3x3 stencil), one fused step in FP32K against one in FP64 (the FP64 form
    is pinned to the oracle at 1e-10 per step): the same cell lists and sort
    permutation, rates and state within the FP32K bound of the small case."""
    c = setups.micro(n_side=2048, seed=9, cell_factor=2, stencil=1)
    out = {}
    for prec in (abi.SPH_PREC_FP64, abi.SPH_PREC_FP32K):
        s = Solver(c, precision=prec)
        s.step()
        out[prec] = s.download(["hash", "idx", "blanked", "vel_t", "pos_t", "S_t", "rho_t", "vel", "S", "rho",
                                "eps_pl"])
        st = s.status()
        s.close()
        assert st & abi.STATUS_BITS["nan_blanked"] == 0
    G, R = out[abi.SPH_PREC_FP32K], out[abi.SPH_PREC_FP64]
    for f in ("hash", "idx", "blanked"):
        assert np.array_equal(G[f], R[f]), f
    assert (R["eps_pl"] > 0).sum() > 1000, "plastic flow: the return mapping runs"
    for f in ("vel_t", "pos_t", "S_t", "rho_t", "vel", "S", "rho"):
        e = rel_err(G[f], R[f])
        assert e < 2e-5, f"FP32K {f}: {e:.2e}"


def test_fp32_compensated_error_bound(lib):
    c = shuffled_micro(n=80, seed=9)
    s64, o = pair(c)
    s32 = Solver(c, precision=abi.SPH_PREC_FP32K)
    s32.step()
    o.step()
    G = s32.download()
    act = o.P["blanked"] != 1
    # cell-list work stays bit-exact in the FP32 form
    for f in ["hash", "idx"]:
        assert np.array_equal(G[f], o.P[f]), f
    errs = {f: rel_err(G[f][act], o.P[f][act]) for f in ["vel_t", "pos_t", "S_t", "rho_t", "T_t", "vel", "S", "rho"]}
    for f, e in errs.items():
        assert e < 2e-5, f"FP32K {f}: {e:.2e}"
