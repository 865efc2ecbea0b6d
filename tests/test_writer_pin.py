"""The product's VTK writers and force report against the reference's own
output code (vtk_writer.cu, output.cu) built for the host from the reference
tree (oracle/_ref/ref_writer_pin; skipped where it was not built).  No GPU:
the state is a small cut advanced by the CPU oracle, written by the product's
host writers (the device-context writers download the state and call them)
and by the reference's writers from the same arrays.  The files must agree
byte for byte; report_force (a thrust reduction on the GPU, left to right in
the host build) agrees with the sum of fc + ft to rounding.

The reference's particle writer reads an uninitialised blanked array
(vtk_writer.cu:67-82) and numbers vertex cells by particle index; with no
particle blanked (asserted) its output is defined and the two agree."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from oracle.oracle import OracleSim

ROOT = Path(__file__).resolve().parents[1]
PIN = ROOT / "oracle" / "_ref" / "ref_writer_pin"


@pytest.fixture(scope="module")
def state():
    if not PIN.exists():
        pytest.skip("reference writer pin not built (no reference tree)")
    case = setups.placed(setups.small_cut(), preload_dx=0.3)
    tool = abi.tool_model_host(case)
    o = OracleSim(case.constants, case.grid, case.particles, case.dt,
                  tool=dict(segments=tool["segments"], fem=tool["fem"], state=tool["state"],
                            n_cut_colors=tool["n_cut_colors"]))
    for _ in range(25):
        o.step()
    P = o.P
    assert np.all(P["blanked"] != 1.0)
    assert np.abs(P["fc"]).max() > 0, "no contact: the force fields would all be zero"
    rng = np.random.default_rng(4)
    ns = len(o.seg["fric_heat"])
    phys = np.abs(rng.normal(size=(ns, 4))) * np.array([3.0, 1e-3, 1e-4, 400.0])
    phys[::3, 0] = 0.0                                   # segments no particle touched
    wear = dict(phys_para=phys, sliding_force=np.abs(rng.normal(size=ns)) * 1e-3,
                wear_rate=np.abs(rng.normal(size=ns)) * 1e-12)
    elements = np.zeros((len(case.tool_mesh["elements"]), 4), np.int32)
    elements[:, :3] = case.tool_mesh["elements"]
    tl_now = np.array([o.ts.tl_point_ref[0], o.ts.tl_point_ref[1]])
    tl_ref = tl_now - np.array([3e-4, -1e-4])
    return dict(P=P, fem=o.fem, seg=o.seg, wear=wear, elements=elements, tl_now=tl_now, tl_ref=tl_ref)


def run_reference(st, tmp):
    P, fem, seg, w = st["P"], st["fem"], st["seg"], st["wear"]
    N, nn, ne, ns = len(P["rho"]), len(fem["T"]), len(st["elements"]), len(seg["fric_heat"])
    parts = [np.array([N, nn, ne, ns], np.int32)]
    for k in ("pos", "vel", "fc", "ft", "n", "S", "p", "T", "eps_pl", "rho", "h", "fixed"):
        parts.append(np.ascontiguousarray(P[k], np.float64))
    parts += [np.ascontiguousarray(P["idx"], np.int32), np.ascontiguousarray(P["on_seg"], np.int32),
              np.ascontiguousarray(fem["position"], np.float64), np.ascontiguousarray(fem["T"], np.float64),
              st["elements"]]
    for k in ("left", "right", "normal"):
        parts.append(np.ascontiguousarray(seg[k], np.float64))
    parts += [w["phys_para"], w["sliding_force"], w["wear_rate"], np.concatenate([st["tl_now"], st["tl_ref"]])]
    (tmp / "results").mkdir()
    with open(tmp / "in.bin", "wb") as f:
        for a in parts:
            f.write(np.ascontiguousarray(a).tobytes())
    out = subprocess.run([str(PIN), str(tmp / "in.bin")], cwd=tmp, capture_output=True, text=True, check=True)
    fx, fy = out.stdout.split()[1:3]
    return {k: (tmp / "results" / f"{k}_000000.vtk").read_bytes()
            for k in ("vtk_out", "vtk_tool", "vtk_seg", "vtk_tool_org")}, np.array([float(fx), float(fy)])


def test_writers_match_the_reference_byte_for_byte(lib, state, tmp_path):
    ref, _ = run_reference(state, tmp_path)
    P, fem, seg, w = state["P"], state["fem"], state["seg"], state["wear"]
    mine = tmp_path / "mine"
    mine.mkdir()
    h = abi.particles_struct(P, len(P["rho"]))
    assert lib.sph_vtk_write_particles_host(C.byref(h), str(mine / "p.vtk").encode()) == abi.SPH_OK
    el = np.ascontiguousarray(state["elements"])
    pos, T = np.ascontiguousarray(fem["position"]), np.ascontiguousarray(fem["T"])
    assert lib.sph_vtk_write_tool_host(len(T), abi.ptr(pos), abi.ptr(T), len(el), abi.ptr(el), None,
                                       str(mine / "t.vtk").encode()) == abi.SPH_OK
    shift = np.ascontiguousarray(state["tl_now"] - state["tl_ref"])
    assert lib.sph_vtk_write_tool_host(len(T), abi.ptr(pos), abi.ptr(T), len(el), abi.ptr(el), abi.ptr(shift),
                                       str(mine / "to.vtk").encode()) == abi.SPH_OK
    ns = len(seg["fric_heat"])
    args = [np.ascontiguousarray(seg[k]) for k in ("left", "right", "normal")]
    args += [np.ascontiguousarray(w[k]) for k in ("phys_para", "sliding_force", "wear_rate")]
    assert lib.sph_vtk_write_segments_host(ns, *[abi.ptr(a) for a in args], str(mine / "s.vtk").encode()) == abi.SPH_OK
    for name, ours in (("vtk_out", "p.vtk"), ("vtk_tool", "t.vtk"), ("vtk_tool_org", "to.vtk"), ("vtk_seg", "s.vtk")):
        a, b = (mine / ours).read_bytes(), ref[name]
        assert a == b, f"{name}: first difference at byte {next(i for i in range(min(len(a), len(b))) if a[i] != b[i]) if a[:len(b)] != b[:len(a)] else min(len(a), len(b))}"


def test_report_force_is_the_sum_of_contact_forces(state, tmp_path):
    _, f_ref = run_reference(state, tmp_path)
    P = state["P"]
    f = P["fc"].sum(0) + P["ft"].sum(0)
    assert np.allclose(f_ref, f, rtol=1e-12, atol=1e-300)
