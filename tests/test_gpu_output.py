"""Output in the reference's formats: legacy-ASCII VTK of particles and of the
FEM tool (vtk_writer.cu) and the force log (mfree_gpu.cpp), parsed back and
checked against the downloaded state."""
import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def parse_vtk(path):
    """{'POINTS': array, 'CELLS': lines, 'CELL_TYPES': ints, name: array} of a legacy VTK file."""
    lines = [l.strip() for l in open(path)]
    out, i = {}, 0
    assert lines[0] == "# vtk DataFile Version 2.0" and lines[2] == "ASCII"
    while i < len(lines):
        t = lines[i].split()
        if not t:
            i += 1
            continue
        if t[0] == "POINTS":
            n = int(t[1])
            out["POINTS"] = np.array([[float(v) for v in lines[i + 1 + k].split()] for k in range(n)])
            i += 1 + n
        elif t[0] == "CELLS":
            n = int(t[1])
            out["CELLS"] = [[int(v) for v in lines[i + 1 + k].split()] for k in range(n)]
            i += 1 + n
        elif t[0] == "CELL_TYPES":
            n = int(t[1])
            out["CELL_TYPES"] = [int(lines[i + 1 + k]) for k in range(n)]
            i += 1 + n
        elif t[0] == "POINT_DATA":
            out["n_point_data"] = int(t[1])
            i += 1
        elif t[0] == "SCALARS":
            n = out["n_point_data"]
            out[t[1]] = np.array([float(lines[i + 2 + k]) for k in range(n)])
            i += 2 + n
        elif t[0] == "VECTORS":
            n = out["n_point_data"]
            out[t[1]] = np.array([[float(v) for v in lines[i + 1 + k].split()] for k in range(n)])
            i += 1 + n
        else:
            i += 1
    return out


def test_vtk_particles_tool_and_force_log(lib, tmp_path):
    case = setups.placed(setups.small_cut(), preload_dx=0.3)
    s = Solver(case, abi.SPH_PREC_FP64, place_tool=False)
    tl0 = np.array([s.tool_state().tl_point_ref[0], s.tool_state().tl_point_ref[1]])
    s.step(20)
    P = s.download(["pos", "vel", "T", "eps_pl", "blanked", "on_seg", "fc", "ft", "n", "S", "p"])
    s.write_vtk(tmp_path / "p.vtk")
    v = parse_vtk(tmp_path / "p.vtk")
    live = P["blanked"] != 1.0
    m = int(live.sum())
    assert v["POINTS"].shape == (m, 3)
    assert np.allclose(v["POINTS"][:, :2], P["pos"][live], atol=1e-6)
    assert v["CELLS"] == [[1, k] for k in range(m)] and v["CELL_TYPES"] == [1] * m
    assert np.allclose(v["Temperature"], P["T"][live], atol=1e-6)
    assert np.array_equal(v["on_seg"], P["on_seg"][live])
    assert np.allclose(v["EquivAccumPlasticStrain"], P["eps_pl"][live], atol=1e-6)
    assert np.allclose(v["Velocity"][:, :2], P["vel"][live], atol=1e-6)
    assert np.allclose(v["fc"][:, :2], 1e5 * P["fc"][live], atol=1e-6)
    assert np.allclose(v["ft"][:, :2], 1e5 * P["ft"][live], atol=1e-6)
    S, p = P["S"][live], P["p"][live]
    cxx, cyy, czz, cxy = S[:, 0] - p, S[:, 2] - p, S[:, 3] - p, S[:, 1]
    svm = np.sqrt(np.maximum(cxx**2 + cyy**2 + czz**2 - cxx * cyy - cxx * czz - cyy * czz + 3 * cxy**2, 0))
    assert np.allclose(v["SvM"], svm, atol=1e-6)
    # tool: nodes, triangles, nodal temperature; and the same tool moved back to tl0
    fem = s.fem()
    s.write_vtk_tool(tmp_path / "t.vtk")
    t = parse_vtk(tmp_path / "t.vtk")
    assert np.allclose(t["POINTS"][:, :2], fem["position"], atol=1e-6)
    assert all(c[0] == 3 for c in t["CELLS"]) and set(t["CELL_TYPES"]) == {5}
    assert len(t["CELLS"]) == len(case.tool_mesh["elements"])
    assert np.allclose(t["temperature"], fem["T"], atol=1e-6)
    s.write_vtk_tool(tmp_path / "t0.vtk", tl_ref=tl0)
    t0 = parse_vtk(tmp_path / "t0.vtk")
    moved = np.array(s.tool_state().tl_point_ref) - tl0
    assert np.abs(moved[0]) > 0
    assert np.allclose(t0["POINTS"][:, :2], fem["position"] - moved, atol=1e-6)
    # force log
    for _ in range(3):
        s.append_force_log(tmp_path / "force")
        s.step(5)
    rows = [list(map(float, l.split())) for l in open(tmp_path / "force")]
    assert len(rows) == 3 and all(len(r) == 2 for r in rows)
    s.close()


def test_usui_wear_log_matches_oracle(lib):
    from oracle.oracle import eval_usui
    case = setups.placed(setups.small_cut(), preload_dx=0.3)
    s = Solver(case, abi.SPH_PREC_FP64, place_tool=False)
    s.step(15)
    K_usui, alpha = 1e-8, -2500.0
    got = s.eval_usui(K_usui, alpha, dt=case.dt)
    P = s.download(["fc", "ft", "vel", "n", "h", "T"])
    want = eval_usui(P, K_usui, alpha, (case.tool_speed, 0.0))
    assert want[1] > 0, "no particle in contact"
    assert np.allclose(got, want, rtol=1e-12, atol=0)
    assert np.isclose(s.accum_wear, case.dt * want[2], rtol=1e-12)
    s.close()
