"""GPU parity of the rigid (SPH-mode) tool step -- leap_frog::step(particles,
grid) (leap_frog.cu:99-160): tool_gpu.cu motion and penalty contact, the
friction heat of do_material_fric_heat_gen (actions_gpu.cu:316-343), tool
particles that take part in heat conduction only -- and of the PSE conduction
build (interactions_gpu.cu:84-140), against the CPU oracle through the C ABI.

FP64 fields within 1e-10 relative (norm-wise, as the other parity tests); the
tool outline, which both sides move with the same host arithmetic, bit-exact;
flags and the cell list bit-exact.
"""
import ctypes as C

import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver, SphError
from oracle.oracle import OracleSim
from conftest import rel_err
from test_gpu_parity import EXACT, RATES, RTOL, STATE, compare

pytestmark = pytest.mark.gpu

FUSED = STATE + RATES + EXACT


def rigid_case(**kw):
    args = dict(ny=8, length=0.02, preload_dx=1.5)
    args.update(kw)
    return setups.ref_cut(**args)


def rigid_pair(case, precision=abi.SPH_PREC_FP64, pse=False):
    s = Solver(case, precision)
    if pse:
        s.set_thermal_model(abi.SPH_THERMAL_PSE)
    o = OracleSim(case.constants, case.grid, s.download(), case.dt, rigid=case.rigid.to_struct(), pse=pse)
    return s, o


def tool_arrays(t: abi.RigidTool) -> dict:
    n = t.n_seg
    return dict(left=np.array([[t.left[i][0], t.left[i][1]] for i in range(n)]),
                right=np.array([[t.right[i][0], t.right[i][1]] for i in range(n)]),
                la=np.array(t.la[:n]), lb=np.array(t.lb[:n]), vertical=np.array(t.vertical[:n]),
                fillet_p=np.array(t.fillet_p[:]))


def compare_tool(s, o, what=""):
    a, b = tool_arrays(s.rigid_tool()), tool_arrays(o.rigid)
    for k in a:
        assert np.array_equal(a[k], b[k]), f"{what} tool {k}: {a[k]} vs {b[k]}"


@pytest.mark.parametrize("geom", [dict(), dict(chamfer=0.0), dict(rake=6.0), dict(rake=-6.0, chamfer=2e-3)],
                         ids=["fillet", "sharp", "rake6", "rake-6"])
def test_rigid_fused_step_matches_oracle(lib, geom):
    c = rigid_case(**geom)
    s, o = rigid_pair(c)
    for k in range(4):
        s.step()
        o.step()
        compare(s, o, FUSED, what=f"[rigid {geom} step {k}]")
        compare_tool(s, o, what=f"[step {k}]")
    G = s.download(["fc", "tool_particle"])
    wp = G["tool_particle"] == 0
    assert np.count_nonzero(np.abs(G["fc"][wp]).sum(1)) > 0, "contact never became active"
    assert s.status() == 0


def staged_rigid(s, o, pse, check):
    s.update_geometry()
    s.assign_hashes(); o.assign_hashes()
    s.sort(); o.sort()
    s.init(); o.init()
    s.predict(); o.predict()
    s.material_eos(); o.material_eos()
    s.corrector_artificial_stress(); o.corrector_artificial_stress()
    s.interactions_monaghan(); o.interactions_monaghan()
    check("interactions", ["S_der", "v_der", "pos_t", "vel_t", "T_t"])
    if pse:
        s.interactions_heat_pse(); o.interactions_heat_pse()
        check("heat pse", ["T_t"])
    s.material_stress_rate_jaumann(); o.material_stress_rate_jaumann()
    s.contmech_continuity(); o.contmech_continuity()
    s.contmech_momentum(); o.contmech_momentum()
    s.contmech_advection(); o.contmech_advection()
    s.correct(); o.correct()
    check("correct", ["pos", "vel", "S", "rho", "T"])
    s.material_fric_heat_gen(); o.material_fric_heat_gen()
    check("friction heat", ["T"])
    s.plasticity_johnson_cook(); o.plasticity_johnson_cook()
    check("plasticity", ["S", "eps_pl", "eps_pl_dot", "T", "blanked"])
    s.rigid_tool_update(); o.rigid_tool_update()
    check("tool update", ["pos"])
    s.compute_contact_forces(); o.compute_contact_forces()
    check("contact", ["fc", "ft", "n"])
    s.perform_boundary_conditions(); o.perform_boundary_conditions()
    s.perform_boundary_conditions_thermal(); o.perform_boundary_conditions_thermal()
    s.debug_invalidate(); o.debug_invalidate()
    check("bc+invalidate", FUSED)


@pytest.mark.parametrize("pse", [False, True], ids=["brookshaw", "pse"])
def test_rigid_stage_by_stage(lib, pse):
    c = rigid_case()
    s, o = rigid_pair(c, pse=pse)

    def check(stage, fields):
        compare(s, o, fields, what=f"[rigid pse={pse}:{stage}]")

    for _ in range(2):
        staged_rigid(s, o, pse, check)
        compare_tool(s, o)


def test_rigid_pse_fused_matches_oracle(lib):
    c = rigid_case()
    s, o = rigid_pair(c, pse=True)
    for k in range(4):
        s.step()
        o.step()
        compare(s, o, FUSED, what=f"[rigid pse step {k}]")
    # heat flows from the (friction-heated) workpiece: the tool particles' T changes
    G = s.download(["T_t", "tool_particle", "blanked"])
    tp = (G["tool_particle"] == 1) & (G["blanked"] != 1)
    assert np.isfinite(G["T_t"][tp]).all()


def test_rigid_staged_step_matches_fused(lib):
    c = rigid_case()
    s1, _ = rigid_pair(c)
    s2 = Solver(c)
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


def test_rigid_blanked_particle_heated_and_in_contact(lib):
    """A blanked workpiece particle skips the corrector and the return mapping,
    but the rigid tool's friction heat and contact still apply to it
    (actions_gpu.cu:316-343 and tool_gpu.cu:146-202 have no blanked test)."""
    c = rigid_case(preload_dx=2.5)
    s, o = rigid_pair(c)
    for _ in range(2):
        s.step()
        o.step()
    G = s.download()
    wp = (G["tool_particle"] == 0) & (G["blanked"] != 1) & (G["fixed"] == 0)
    cand = np.flatnonzero(wp & (np.abs(G["ft"]).sum(1) > 0))
    assert len(cand) > 0, "no free particle with friction force"
    G["blanked"][cand[0]] = 1.0
    s.upload({"blanked": G["blanked"]})
    o.P["blanked"][:] = G["blanked"]
    T0 = G["T"][cand[0]]
    for k in range(3):
        s.step()
        o.step()
        compare(s, o, FUSED, what=f"[blanked step {k}]")
    bi = np.flatnonzero(o.P["blanked"] == 1)
    assert len(bi) == 1
    assert o.P["T"][bi[0]] > T0, "friction heat did not reach the blanked particle"


def test_rigid_fp32k_error_bound(lib):
    c = rigid_case()
    s32 = Solver(c, precision=abi.SPH_PREC_FP32K)
    _, o = rigid_pair(c)
    for _ in range(2):
        s32.step()
        o.step()
    G = s32.download()
    for f in ["hash", "idx", "blanked"]:
        assert np.array_equal(G[f], o.P[f]), f
    act = o.P["blanked"] != 1
    for f in ["pos", "vel", "S", "rho", "T", "fc", "ft"]:
        e = rel_err(G[f][act], o.P[f][act])
        assert e < 2e-5, f"FP32K rigid {f}: {e:.2e}"


def test_rigid_pse_fp32k_error_bound(lib):
    """The FP32K form of the PSE build (FP32 records, expf, Kahan sum) against the
    FP64 oracle of the same build."""
    c = rigid_case()
    s32 = Solver(c, precision=abi.SPH_PREC_FP32K)
    s32.set_thermal_model(abi.SPH_THERMAL_PSE)
    _, o = rigid_pair(c, pse=True)
    for _ in range(3):
        s32.step()
        o.step()
    G = s32.download()
    for f in ["hash", "idx", "blanked"]:
        assert np.array_equal(G[f], o.P[f]), f
    act = o.P["blanked"] != 1
    for f in ["pos", "vel", "S", "rho", "T", "fc", "ft"]:
        e = rel_err(G[f][act], o.P[f][act])
        assert e < 2e-5, f"FP32K rigid PSE {f}: {e:.2e}"
    # the conduction rate itself, on the particles where heat flows: norm-wise
    # against the largest rate, 1.8e-3 measured (FP32 Gaussian weights and
    # temperature differences), inside the 1 % the FP32K form is held to
    e = rel_err(G["T_t"][act], o.P["T_t"][act])
    assert e < 3e-3, f"FP32K PSE T_t: {e:.2e}"
    assert np.max(np.abs(o.P["T_t"][act])) > 0


def test_rigid_api_errors(lib):
    c = rigid_case()
    s = Solver(c)
    t = c.rigid.to_struct()
    bad = abi.RigidTool()
    C.memmove(C.byref(bad), C.byref(t), C.sizeof(abi.RigidTool))
    bad.has_fillet = 0                  # 5 segments need the fillet
    with pytest.raises(SphError):
        s.set_rigid_tool(bad)
    bad.n_seg = 0
    with pytest.raises(SphError):
        s.set_rigid_tool(bad)
    s.set_rigid_tool(None)              # removed: the rigid calls refuse
    with pytest.raises(SphError):
        s.compute_contact_forces()
    s.set_rigid_tool(t)
    s.compute_contact_forces()
    # PSE needs cells of edge h (FP64 or FP32K)
    s32 = Solver(c, precision=abi.SPH_PREC_FP32K)
    s32.set_thermal_model(abi.SPH_THERMAL_PSE)
    c2 = rigid_case(cell_factor=2, stencil=1)
    s2 = Solver(c2)
    with pytest.raises(SphError):
        s2.set_thermal_model(abi.SPH_THERMAL_PSE)
    # a FEM-tool context takes no rigid tool
    cut = setups.small_cut()
    sf = Solver(cut)
    with pytest.raises(SphError):
        sf.set_rigid_tool(t)
