"""GPU parity of the wear path (WEAR_NODE_SHIFT) against the CPU oracle,
through the C ABI: the per-segment statistics gathered by the friction heat
(actions_gpu.cu:401-419) and wear_adjustment (actions_gpu.cu:1009-1020: layer
retreat / resume, Usui rake/flank nodal shift, segment update, flank
correction, lumped inverse mass), in the staged calls and in the fused step.

Tolerances: particle fields as the other parity tests (1e-10 relative,
norm-wise; flags and the cell list bit-exact).  The wear shift evaluates exp on
the device and on the host, so node positions, segments, the FEM matrices and
the statistics are compared within 1e-10 relative (the node displacements
themselves within 1e-9).
"""
import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver, SphError
from oracle.oracle import OracleSim
from conftest import rel_err
from test_gpu_parity import EXACT, RATES, RTOL, STATE

pytestmark = pytest.mark.gpu

FUSED = STATE + RATES + EXACT
WC = abi.WearConstants(10.0, 300.0, 10.0, 300.0)   # flank A, B; rake C, D


def wear_pair(mode, precision=abi.SPH_PREC_FP64, preload_dx=0.3):
    c = setups.small_cut()
    s = Solver(c, precision)
    s.move_tool(preload_dx * c.info["dx"] / c.tool_speed)
    s.set_wear(mode, WC)
    ts = s.tool_state()
    tool = dict(segments=s.segments(), fem=s.fem(), state=ts, n_cut_colors=ts.n_cut_colors)
    w = s.wear_state()
    o = OracleSim(c.constants, c.grid, s.download(), c.dt, tool=tool,
                  wear=dict(mode=mode, constants=WC, elements=w["elements"], layer=w["layer"], M=w["M"]))
    return c, s, o


def compare_particles(s, o, fields, what):
    G = s.download()
    act = o.P["blanked"] != 1.0
    for f in fields:
        a, b = G[f], o.P[f]
        if f in RATES:
            a, b = a[act], b[act]
        if f in EXACT:
            assert np.array_equal(a, b), f"{what} {f}: {np.count_nonzero(a != b)} entries differ"
        else:
            e = rel_err(a, b)
            assert e <= RTOL, f"{what} {f}: relative error {e:.3e}"


def compare_tool(s, o, what, pos0=None):
    seg = s.segments()
    for k in ("left", "right", "normal"):
        e = rel_err(seg[k], o.seg[k])
        assert e <= 1e-10, f"{what} segments {k}: {e:.3e}"
    fem = s.fem()
    for k in ("position", "T", "K", "M_inv"):
        e = rel_err(fem[k], o.fem[k])
        assert e <= 1e-10, f"{what} FEM {k}: {e:.3e}"
    if pos0 is not None:   # the displacement itself
        d_gpu, d_orc = fem["position"] - pos0, o.fem["position"] - pos0
        if np.max(np.abs(d_orc)) > 0:
            e = rel_err(d_gpu, d_orc)
            assert e <= 1e-9, f"{what} node displacement: {e:.3e}"
    w = s.wear_state()
    for k in ("M", "phys_para", "sliding_force", "wear_nodes"):
        e = rel_err(w[k], o.wear[k])
        assert e <= 1e-10, f"{what} wear {k}: {e:.3e}"
    ts = s.tool_state()
    assert ts.flank_contact == pytest.approx(o.ts.flank_contact, rel=1e-14, abs=1e-18), what
    assert ts.flank_retreat == pytest.approx(o.ts.flank_retreat, rel=1e-9, abs=1e-16), what


def test_wear_stage_by_stage(lib):
    c, s, o = wear_pair(abi.SPH_WEAR_SHIFT)
    dt = o.dt
    pos0 = s.fem()["position"]
    for rep in range(2):
        s.update_geometry()
        s.assign_hashes(); o.assign_hashes()
        s.sort(); o.sort()
        s.init(); o.init()
        s.fem_reset_server(); o.fem_reset_server()
        s.segments_wear_rate_reset(); o.segments_wear_rate_reset()
        s.predict(); o.predict()
        s.fem_calculate_temp(0.5 * dt); o.fem_calculate_temp(0.5 * dt)
        s.material_eos(); o.material_eos()
        s.corrector_artificial_stress(); o.corrector_artificial_stress()
        s.interactions_monaghan(); o.interactions_monaghan()
        s.material_stress_rate_jaumann(); o.material_stress_rate_jaumann()
        s.contmech_continuity(); o.contmech_continuity()
        s.contmech_momentum(); o.contmech_momentum()
        s.contmech_advection(); o.contmech_advection()
        s.correct(); o.correct()
        s.material_fric_heat_gen_fem(); o.material_fric_heat_gen_fem()
        compare_particles(s, o, ["T", "blanked"], f"[rep {rep} friction heat]")
        w = s.wear_state()
        assert w["phys_para"][:, 0].sum() > 0, "no segment gathered wear statistics"
        for k in ("phys_para", "sliding_force"):
            assert rel_err(w[k], o.wear[k]) <= 1e-10, k
        s.fem_apply_robin(); o.fem_apply_robin()
        s.fem_calculate_temp_rate(); o.fem_calculate_temp_rate()
        s.fem_calculate_temp(dt); o.fem_calculate_temp(dt)
        s.plasticity_johnson_cook(); o.plasticity_johnson_cook()
        s.wear_adjustment(); o.wear_adjustment()
        compare_tool(s, o, f"[rep {rep} wear adjustment]", pos0)
        if rep > 0:   # the first pass has no contact forces yet (zero pressure, no wear)
            assert np.max(np.abs(s.wear_state()["wear_nodes"])) > 0, "no wear"
        s.move_tool(dt); o.move_tool(dt)
        compare_tool(s, o, f"[rep {rep} tool move]")
        s.compute_contact_forces_fem(); o.compute_contact_forces_fem()
        s.perform_boundary_conditions(); o.perform_boundary_conditions()
        s.perform_boundary_conditions_thermal(); o.perform_boundary_conditions_thermal()
        s.debug_invalidate(); o.debug_invalidate()
        compare_particles(s, o, FUSED, f"[rep {rep} end]")


@pytest.mark.parametrize("mode", [abi.SPH_WEAR_ACCUMULATE, abi.SPH_WEAR_SHIFT], ids=["accumulate", "shift"])
def test_wear_fused_step_matches_oracle(lib, mode):
    c, s, o = wear_pair(mode)
    pos0 = s.fem()["position"]
    for k in range(6):
        s.step()
        o.step()
        compare_particles(s, o, FUSED, f"[wear mode {mode} step {k}]")
        compare_tool(s, o, f"[wear mode {mode} step {k}]", pos0)
    w = s.wear_state()
    assert w["phys_para"][:, 0].sum() > 0
    if mode == abi.SPH_WEAR_SHIFT:
        assert np.max(w["wear_nodes"]) > 0
        assert np.max(np.abs(w["M"] - o.wear["M"])) <= 1e-10 * np.max(np.abs(w["M"]))
    else:   # statistics only: the mesh does not change
        assert np.all(w["wear_nodes"] == 0)
    assert s.status() == 0


def test_wear_switched_on_mid_run(lib):
    """wear_pro turns on part-way through the reference's run (mfree_gpu.cpp:300):
    the context re-captures its step graph and follows the oracle."""
    c, s, o = wear_pair(abi.SPH_WEAR_ACCUMULATE)
    for k in range(6):
        if k == 3:
            s.set_wear(abi.SPH_WEAR_SHIFT, WC)
            o.wear_mode = abi.SPH_WEAR_SHIFT
        s.step()
        o.step()
    compare_particles(s, o, FUSED, "[mid-run switch]")
    compare_tool(s, o, "[mid-run switch]")
    assert np.max(s.wear_state()["wear_nodes"]) > 0


def test_wear_fp32k_runs_and_wears(lib):
    c, s, o = wear_pair(abi.SPH_WEAR_SHIFT, precision=abi.SPH_PREC_FP32K)
    s.step(6)
    o.step(); o.step(); o.step(); o.step(); o.step(); o.step()
    w = s.wear_state()
    assert np.max(w["wear_nodes"]) > 0 and s.status() == 0
    fem = s.fem()
    # nodes, FEM temperature and the rebuilt inverse mass stay close to the FP64 oracle
    assert rel_err(fem["position"], o.fem["position"]) < 1e-9
    assert rel_err(fem["T"], o.fem["T"]) < 1e-4
    assert rel_err(fem["M_inv"], o.fem["M_inv"]) < 1e-6


def test_wear_api_errors(lib):
    c = setups.micro(n_side=16)
    s = Solver(c)                                # no tool
    with pytest.raises(SphError):
        s.set_wear(abi.SPH_WEAR_ACCUMULATE, WC)
    c, s, o = wear_pair(abi.SPH_WEAR_OFF)
    with pytest.raises(SphError):
        s.set_wear(abi.SPH_WEAR_SHIFT, None)     # the shift needs constants
    with pytest.raises(SphError):
        s.set_wear(7, WC)
    with pytest.raises(SphError):
        s.wear_adjustment()                      # wear is off
    s.set_wear(abi.SPH_WEAR_ACCUMULATE, None)    # statistics need no constants
    with pytest.raises(SphError):
        s.wear_adjustment()                      # only in the shift mode


def test_segment_vtk_carries_wear_fields(lib, tmp_path):
    """vtk_writer_write_FEM_segments (vtk_writer.cu:368-516): each segment as a
    triangle left, right, right + |segment| n; the wear fields on its third point."""
    c, s, o = wear_pair(abi.SPH_WEAR_SHIFT)
    s.step(5)
    path = tmp_path / "seg.vtk"
    s.write_vtk_segments(path)
    seg, w = s.segments(), s.wear_state()
    ns = len(seg["left"])
    lines = path.read_text().splitlines()
    i = lines.index(f"POINTS {3 * ns} float")
    pts = np.array([[float(v) for v in lines[i + 1 + k].split()] for k in range(3 * ns)])
    np.testing.assert_allclose(pts[0::3, :2], seg["left"], atol=1e-6)
    np.testing.assert_allclose(pts[1::3, :2], seg["right"], atol=1e-6)
    length = np.linalg.norm(seg["left"] - seg["right"], axis=1)
    np.testing.assert_allclose(pts[2::3, :2], seg["right"] + length[:, None] * seg["normal"], atol=1e-6)

    def field(name):
        j = lines.index(f"SCALARS {name} float 1")
        return np.array([float(v) for v in lines[j + 2:j + 2 + 3 * ns]])

    pp = w["phys_para"]
    hit = pp[:, 0] != 0
    assert hit.any()
    p = field("PressureGPa")
    assert np.all(p[0::3] == 0) and np.all(p[1::3] == 0)
    np.testing.assert_allclose(p[2::3][hit], pp[hit, 1] / pp[hit, 0] * 100.0, rtol=1e-5, atol=1e-6)
    assert np.all(p[2::3][~hit] == 0)
    np.testing.assert_allclose(field("Temperature")[2::3][hit], pp[hit, 3] / pp[hit, 0], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(field("Wear_rate")[2::3][hit], w["wear_nodes"][hit] * 1e10, rtol=1e-5, atol=1e-6)
