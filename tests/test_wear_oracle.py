"""CPU tests of the wear-by-nodal-shift restatements (WEAR_NODE_SHIFT, no GPU):
the cutting-edge layers (mesh_structure_GPU.cu:1063-1148) of the product's host
set-up against the oracle, and known answers of the oracle's wear_adjustment
(actions_gpu.cu:1009-1020): the Usui rake/flank shift of the cutting-edge
nodes, the retreat / resume of the layers' lumped mass and the flank
correction."""
import ctypes as C
import math

import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups


def host_model(case, lib):
    tool, keep = case.tool_struct()
    h = C.c_void_p()
    assert lib.sph_tool_build(C.byref(tool), C.byref(case.constants.tool), C.byref(h)) == abi.SPH_OK
    return h, keep


@pytest.mark.parametrize("name", ["small_cut", "ti64_cut"])
def test_layers_match_oracle(lib, oracle_lib, name):
    case = getattr(setups, name)()
    m = case.tool_mesh
    h, keep = host_model(case, lib)
    ne, nn = len(m["elements"]), len(m["nodes"])
    mine = np.zeros((ne, 2), np.int32)
    assert lib.sph_tool_host_layers(h, abi.ptr(mine)) == abi.SPH_OK
    lib.sph_tool_host_destroy(h)
    ref = np.zeros((ne, 2), np.int32)
    oracle_lib.orc_wear_layers(ne, abi.ptr(np.ascontiguousarray(m["elements"], np.int32)),
                               abi.ptr(np.ascontiguousarray(m["cutting_flags"], np.int32)), nn, abi.ptr(ref))
    assert np.array_equal(mine, ref)
    cut = (np.asarray(m["cutting_flags"]).reshape(ne, 3) != 0).any(1)
    assert np.array_equal(ref[:, 0] == 1, cut)
    assert ref[:, 1].sum() > 0 and not np.any(ref[:, 0] & ref[:, 1])


def one_segment_state(rake_face=True):
    """Two triangles sharing the edge (0, 1); element 0 holds the cutting
    segment 0 -> 1 whose normal is (1, 0) (rake face) or (0, -1) (flank)."""
    if rake_face:
        pos = np.array([[0.0, 0.0], [0.0, 1.0], [-1.0, 0.5], [1.0, 0.5]])
        normal = [1.0, 0.0]
    else:
        pos = np.array([[1.0, 0.0], [0.0, 0.0], [0.5, 1.0], [0.5, -1.0]])
        normal = [0.0, -1.0]
    elements = np.array([[0, 1, 2, 1], [0, 3, 1, 2]], np.int32)
    rows = [[0, 1, 2, 3], [0, 1, 2, 3], [0, 1, 2], [0, 1, 3]]
    row_ptr = np.zeros(5, np.int32)
    row_ptr[1:] = np.cumsum([len(r) for r in rows])
    col_ind = np.array([c for r in rows for c in r], np.int32)
    return pos, normal, elements, row_ptr, col_ind


def run_adjustment(oracle_lib, rake_face, stats, T=600.0, wc=(2.0, 1200.0, 3.0, 2500.0), dt=0.1):
    pos, normal, elements, row_ptr, col_ind = one_segment_state(rake_face)
    nn = len(pos)
    K = np.zeros(len(col_ind))
    M = np.full(nn, 5.0)
    F = abi.Fem()
    arrays = dict(position=pos.copy(), row_ptr=row_ptr, col_ind=col_ind, K=K, M_inv=1.0 / M,
                  f=np.zeros(nn), T=np.full(nn, T), k=np.zeros(nn))
    F.n_nodes, F.nnz = nn, len(col_ind)
    for k, v in arrays.items():
        setattr(F, k, abi.ptr(v))
    seg = dict(left=np.array([pos[0]]), right=np.array([pos[1]]), normal=np.array([normal]),
               marks=np.array([[0, 1, 0, 1]], np.int32), heat_exchange=np.zeros((1, 2)), fric_heat=np.zeros(1))
    S = abi.Segments()
    S.n = 1
    for k, v in seg.items():
        setattr(S, k, abi.ptr(v))
    ts = abi.ToolState()
    ts.flank_contact = -0.25
    W = dict(elements=elements, layer=np.array([[1, 0], [0, 1]], np.int32), M=M.copy(),
             phys_para=np.array([stats], np.float64), sliding_force=np.zeros(1), wear_nodes=np.zeros(1))
    w = abi.WearState()
    w.n_elements, w.n_seg = 2, 1
    for k, v in W.items():
        setattr(w, k, abi.ptr(v))
    c = abi.Constants()
    c.tool.cp, c.tool.rho, c.tool.k = 2.0, 3.0, 0.5
    wcs = abi.WearConstants(*wc)
    oracle_lib.orc_wear_adjustment(C.byref(F), C.byref(S), C.byref(ts), C.byref(w), C.byref(c), C.byref(wcs), dt)
    return pos, arrays, seg, ts, W, c


def p1_mass(pos, el, cp, rho):
    p0, p1, p2 = pos[el[0]], pos[el[1]], pos[el[2]]
    det = abs((p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1]))
    return 1.0 / 3.0 * 0.5 * cp * rho * det


@pytest.mark.parametrize("rake_face", [True, False], ids=["rake", "flank"])
def test_nodal_shift_known_answer(oracle_lib, rake_face):
    count, psum, vsum = 4.0, 4 * 0.02, 4 * 0.001
    dt, T = 0.1, 600.0
    A, B, Cc, D = 2.0, 1200.0, 3.0, 2500.0
    pos0, arrays, seg, ts, W, c = run_adjustment(oracle_lib, rake_face, [count, psum, vsum, 0.0], T=T,
                                                 wc=(A, B, Cc, D), dt=dt)
    p, v = 0.02, 0.001
    w = dt * (Cc * p * v * math.exp(-D / T) if rake_face else A * p * v * math.exp(-B / T))
    n = np.array([1.0, 0.0]) if rake_face else np.array([0.0, -1.0])
    moved = arrays["position"]
    np.testing.assert_allclose(moved[0] - pos0[0], n * w, rtol=1e-12, atol=0)
    np.testing.assert_allclose(moved[1] - pos0[1], n * w, rtol=1e-12, atol=0)
    assert np.all(moved[2:] == pos0[2:])
    np.testing.assert_allclose(W["wear_nodes"][0], 2 * w / dt, rtol=1e-12)
    # the segment follows its nodes; its normal is recomputed from them
    np.testing.assert_array_equal(seg["left"][0], moved[0])
    np.testing.assert_array_equal(seg["right"][0], moved[1])
    # lumped mass: 5 - m(old) + m(new) per node of a layer element; M_inv = 1 / M
    elements = [[0, 1, 2], [0, 3, 1]]
    expect = np.full(4, 5.0)
    for el in elements:
        dm = p1_mass(moved, el, 2.0, 3.0) - p1_mass(pos0, el, 2.0, 3.0)
        for a in el:
            expect[a] += dm
    np.testing.assert_allclose(W["M"], expect, rtol=1e-13)
    np.testing.assert_allclose(arrays["M_inv"], 1.0 / W["M"], rtol=1e-15)
    # flank correction: flank_contact - lowest left end
    assert ts.flank_retreat == pytest.approx(-0.25 - moved[0][1], abs=1e-15)


def test_no_statistics_no_shift(oracle_lib):
    pos0, arrays, seg, ts, W, c = run_adjustment(oracle_lib, True, [0.0, 0.0, 0.0, 0.0])
    assert np.array_equal(arrays["position"], pos0)
    np.testing.assert_allclose(W["M"], 5.0, rtol=1e-14)
    assert np.max(np.abs(arrays["K"])) < 1e-14        # retreat and resume cancel
    # too fast sliding (mean speed above 0.008) shifts nothing either
    pos0, arrays, seg, ts, W, c = run_adjustment(oracle_lib, True, [1.0, 0.02, 0.009, 0.0])
    assert np.array_equal(arrays["position"], pos0)
