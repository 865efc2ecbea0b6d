"""CPU tests of the C ABI: the library loads and exports every declared
symbol; host-only tool set-up (segments, CSR, FEM assembly) is consistent."""
import re
from pathlib import Path

import numpy as np

from sph_fem_2d_cutting_gpu_gb300 import abi, setups

HEADER = Path(__file__).resolve().parents[1] / "include" / "sphfem.h"


def declared_symbols():
    txt = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*\**\s*(sph_\w+)\s*\(", txt, re.M)))


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.sph_abi_version() == 1


def test_tool_setup_segments_form_oriented_chain(lib):
    c = setups.small_cut()
    tm = abi.tool_model_host(c)
    seg = tm["segments"]
    L, R, n = seg["left"], seg["right"], seg["normal"]
    # consecutive segments share end points (one open chain, tool_FEM.cu:877-966)
    assert np.array_equal(R[:-1], L[1:])
    assert np.allclose(np.hypot(n[:, 0], n[:, 1]), 1.0, atol=1e-12)
    # normals point into the tool: towards the tool's top-left corner
    tl = c.tool_mesh["tl"]
    assert np.all(((tl - L) * n).sum(1) >= 0)
    # the chain starts at the top of the rake face (y == y_max)
    assert L[0, 1] == max(L[:, 1].max(), R[:, 1].max())
    st = tm["state"]
    assert st.lowest_point == min(L[:, 1].min(), R[:, 1].min())
    assert st.right_point == max(L[:, 0].max(), R[:, 0].max())
    # marks hold the mesh nodes at the segment ends
    pos = tm["fem"]["position"]
    assert np.array_equal(pos[seg["marks"][:, 2]], L)
    assert np.array_equal(pos[seg["marks"][:, 3]], R)


def p1_assembly(nodes, elems, k, cp, rho):
    N = len(nodes)
    K = np.zeros((N, N))
    M = np.zeros(N)
    for a, b, c in elems:
        P = nodes[[a, b, c]]
        J = np.array([[P[1, 0] - P[0, 0], P[2, 0] - P[0, 0]], [P[1, 1] - P[0, 1], P[2, 1] - P[0, 1]]])
        det = abs(np.linalg.det(J))
        g = np.linalg.inv(J).T @ np.array([[-1.0, 1.0, 0.0], [-1.0, 0.0, 1.0]])
        K[np.ix_([a, b, c], [a, b, c])] += 0.5 * det * k * (g.T @ g)
        M[[a, b, c]] += cp * rho * det / 6.0
    return K, M


def test_fem_assembly_matches_independent_p1(lib):
    c = setups.small_cut()
    tm = abi.tool_model_host(c)
    fem = tm["fem"]
    mesh = c.tool_mesh
    t = c.constants.tool
    K, M = p1_assembly(mesh["nodes"], mesh["elements"], t.k, t.cp, t.rho)
    rp, ci, Kv = fem["row_ptr"], fem["col_ind"], fem["K"]
    Kd = np.zeros_like(K)
    for i in range(len(rp) - 1):
        Kd[i, ci[rp[i]:rp[i + 1]]] = Kv[rp[i]:rp[i + 1]]
    # Dirichlet nodes: row = identity, column zeroed; f holds -K_orig * T0 for neighbours
    fixed = np.zeros(len(K), bool)
    for e, fl in zip(mesh["elements"], mesh["fixed_flags"]):
        for k_, (a, b) in enumerate(((0, 1), (1, 2), (2, 0))):
            if fl[k_]:
                fixed[e[a]] = fixed[e[b]] = True
    free = ~fixed
    assert fixed.sum() > 3 and free.sum() > 3
    np.testing.assert_allclose(Kd[np.ix_(free, free)], K[np.ix_(free, free)], rtol=1e-12, atol=1e-12 * np.abs(K).max())
    assert np.all(Kd[fixed][:, fixed] == np.eye(fixed.sum()))
    assert np.all(Kd[np.ix_(free, fixed)] == 0)
    np.testing.assert_allclose(1.0 / fem["M_inv"][free], M[free], rtol=1e-12)
    f_exp = -(K[np.ix_(free, fixed)] @ np.full(fixed.sum(), t.T0))
    np.testing.assert_allclose(fem["f"][free], f_exp, rtol=1e-10, atol=1e-10 * np.abs(f_exp).max())
    assert np.all(fem["f"][fixed] == t.T0)
    # CSR rows sorted and containing the diagonal
    for i in range(len(rp) - 1):
        row = ci[rp[i]:rp[i + 1]]
        assert np.all(np.diff(row) > 0) and i in row


def test_ti64_tool_mesh_size(lib):
    c = setups.ti64_cut()
    assert 1500 <= c.info["nodes"] <= 2500
    tm = abi.tool_model_host(c)
    assert tm["state"].n_segments > 20
