"""remesh_low_level (tool_FEM.cu:1696-1705), the remesh of the worn tool without
gmsh, against the reference's own kernels (do_mesh_shift and
do_nodal_value_interpolation_old from the cubin of the unmodified tool_FEM.cu)
and the host assembly of the moved mesh:

- node positions after the shift within 1e-15 norm-wise (the same formula and
  CUDA's pow; contraction of a product into the final sum may differ);
- nodal temperatures interpolated from the old mesh within 1e-12;
- the thermal system assembled again on the moved mesh: bit for bit the host
  assembly of a tool model built on the moved nodes.
"""
import copy
import ctypes as C

import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver
from conftest import rel_err

pytestmark = pytest.mark.gpu


def node_edges(mesh):
    """Per node: on a cutting-edge (1) / fixed-edge (2) element edge (mesh_structure_GPU.cu:430-471)."""
    el, cf, ff = (np.asarray(mesh[k]) for k in ("elements", "cutting_flags", "fixed_flags"))
    flag = np.zeros(len(mesh["nodes"]), np.int32)
    for a in range(3):
        b = (a + 1) % 3
        for fl, bit in ((cf, 1), (ff, 2)):
            on = fl[:, a] != 0
            flag[el[on, a]] |= bit
            flag[el[on, b]] |= bit
    return flag


@pytest.mark.parametrize("freq", [1, 400])
def test_remesh_low_level_matches_the_reference(lib, freq):
    torch = pytest.importorskip("torch")
    from oracle import ref_gpu
    try:
        tool_m = ref_gpu.RefModule("tool")
    except FileNotFoundError:
        pytest.skip("reference cubins not built")
    case = setups.small_cut()
    s = Solver(case, place_tool=False)
    rng = np.random.default_rng(freq)
    nn = len(case.tool_mesh["nodes"])
    s.upload_fem_state(T=300.0 + 400.0 * rng.random(nn))
    before = s.fem()
    ts = s.tool_state()
    elements = abi.tool_model_host(case)["elements"]
    assert s.lib.sph_remesh_low_level(s.ctx, freq) == abi.SPH_OK
    after = s.fem()
    s.close()
    moved = np.abs(after["position"] - before["position"]).max(1) > 0
    assert moved.any() and not moved.all()
    # the reference's kernels on the state before the remesh
    cuda = torch.device("cuda", 0)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    pos, pos_map, T_map = d(before["position"]), d(before["position"]), d(before["T"])
    flags = node_edges(case.tool_mesh)
    cut, fix = d((flags & 1).astype(np.int32)), d(((flags >> 1) & 1).astype(np.int32))
    T = torch.zeros(nn, dtype=torch.float64, device=cuda)
    el = d(elements)
    mesh = ref_gpu.MeshGPU()
    mesh.position, mesh.cutting_edge_flag, mesh.fixed_edge_flag = ref_gpu.ptr(pos), ref_gpu.ptr(cut), ref_gpu.ptr(fix)
    mesh.position_mapping, mesh.node_num_mapping = ref_gpu.ptr(pos_map), ref_gpu.ptr(el)
    tool_m.launch("ref_set_flank", 1, C.c_double(ts.flank_retreat), C.c_double(ts.flank_contact), block=1)
    tl = ref_gpu.Vec2(ts.tl_point_ref[0], ts.tl_point_ref[1])
    br = ref_gpu.Vec2(ts.br_point[0], ts.br_point[1])
    tool_m.launch("do_mesh_shift", nn, C.c_int32(nn), C.c_int32(freq), mesh, tl, br)
    tool_m.launch("do_nodal_value_interpolation_old", nn, C.c_int32(nn), C.c_int32(len(elements)), mesh,
                  ref_gpu.ptr(T_map), ref_gpu.ptr(T))
    torch.cuda.synchronize()
    assert rel_err(after["position"], pos.cpu().numpy()) <= 1e-15
    assert rel_err(after["T"] - 300.0, T.cpu().numpy() - 300.0) <= 1e-12
    # re-assembly: the host assembly of the moved mesh
    c2 = copy.copy(case)
    c2.tool_mesh = dict(case.tool_mesh, nodes=np.ascontiguousarray(after["position"]))
    host = abi.tool_model_host(c2)["fem"]
    for k in ("K", "M_inv", "f"):
        assert np.array_equal(after[k], host[k]), f"{k}: {np.count_nonzero(after[k] != host[k])} entries differ"
