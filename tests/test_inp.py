"""Abaqus .inp tool meshes (mesh_read, mesh_structure_GPU.cu:784-1257): the
reader's edge flags and full-element correction, and a round trip of a
generated tool mesh through write_inp / read_inp into the host tool set-up."""
import numpy as np

from sph_fem_2d_cutting_gpu_gb300 import abi, setups, tool_mesh


def test_inp_reader_flags_and_correction(tmp_path):
    # two triangles on the cutting edge; element 2 has all three nodes in the set,
    # and its node 4 is in no other boundary element: the edge opposite it is unflagged
    text = """*Heading
# a comment line, skipped
*Node
1, 0., 0.
2, 100., 0.
3, 100., 100.
4, 200., 100.
*Element, type=CPS3
1, 1, 2, 3
2, 2, 4, 3
*Nset, nset=CuttingEdge
1, 2, 3, 4
*Elset, elset=CuttingEdge
1, 2
*Nset, nset=FixedBoundary
1, 3
*Elset, elset=FixedBoundary
1
*End Part
"""
    p = tmp_path / "t.inp"
    p.write_text(text)
    m = tool_mesh.read_inp(str(p))
    assert np.allclose(m["nodes"], [[0, 0], [1, 0], [1, 1], [2, 1]])
    assert m["elements"].tolist() == [[0, 1, 2], [1, 3, 2]]
    # element 1 (nodes 1, 2, 3): its node 1 (local 0) is in no other boundary
    # element -> the opposite edge (b, c) is unflagged
    assert m["cutting_flags"][0].tolist() == [1, 0, 1]
    # element 2 (nodes 2, 4, 3): node 4 (local 1) is not shared -> edge (c, a) unflagged
    assert m["cutting_flags"][1].tolist() == [1, 1, 0]
    # fixed: element 1 edge (c, a) = nodes 3, 1
    assert m["fixed_flags"][0].tolist() == [0, 0, 1]
    assert m["fixed_flags"][1].tolist() == [0, 0, 0]


def test_inp_round_trip_of_generated_tool(lib, tmp_path):
    c = setups.small_cut()
    mesh = c.tool_mesh
    p = tmp_path / "tool.inp"
    tool_mesh.write_inp(mesh, str(p))
    back = tool_mesh.read_inp(str(p), tl=mesh["tl"])
    assert np.allclose(back["nodes"], mesh["nodes"], rtol=0, atol=1e-15)
    assert np.array_equal(back["elements"], mesh["elements"])
    # the same interface segments come out of the host tool set-up
    c2 = setups.Case(**{**c.__dict__, "tool_mesh": back})
    a = abi.tool_model_host(c)["segments"]
    b = abi.tool_model_host(c2)["segments"]
    assert a["left"].shape == b["left"].shape
    assert np.allclose(a["left"], b["left"], atol=1e-15) and np.allclose(a["right"], b["right"], atol=1e-15)
