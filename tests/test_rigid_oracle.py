"""CPU tests of the rigid-tool and PSE restatements in the oracle and of the
host-side tool geometry (no GPU): known answers of the penalty contact and
friction (tool_gpu.cu:146-202), the friction heat (actions_gpu.cu:316-343),
the PSE Laplacian (interactions_gpu.cu:84-140, kernels.cuh:67-84), the fillet
construction (tool.cpp:27-93) and the tool motion (tool.cpp:202-212)."""
import ctypes as C
import math

import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.rigid_tool import Line, RigidTool
from oracle.oracle import OracleSim


def square_tool(mu=0.0, vel=(0.0, 0.0)):
    t = RigidTool.from_points([(0.0, 1.0), (1.0, 1.0), (1.0, 0.0), (0.0, 0.0)], mu)
    t.vel = vel
    return t


def one_particle(pos, vel=(0.0, 0.0), ft=(0.0, 0.0), tool=0.0):
    P = abi.empty_particles(1)
    P["pos"][0] = pos
    P["vel"][0] = vel
    P["ft"][0] = ft
    P["tool_particle"][0] = tool
    P["rho"][0] = 1.0
    P["h"][0] = 0.1
    return P


def constants(mass=2.0, alpha=0.075, eta=0.9, cp=5e-6):
    c = abi.Constants()
    c.phys.mass = mass
    c.tool.contact_alpha = alpha
    c.trml_wp.eta = eta
    c.trml_wp.cp = cp
    return c


def contact(P, t, c, dt, oracle_lib):
    p = abi.particles_struct(P, len(P["rho"]))
    rt = t.to_struct()
    oracle_lib.orc_contact_rigid(C.byref(p), C.byref(rt), C.byref(c), dt)


def test_penalty_force_known_answer(oracle_lib):
    c, dt = constants(), 0.01
    P = one_particle((0.5, 0.9))
    contact(P, square_tool(), c, dt, oracle_lib)
    # nearest primitive: the top edge, outward normal (0, 1), gap -0.1
    np.testing.assert_allclose(P["n"][0], [0.0, 1.0], atol=0)
    np.testing.assert_allclose(P["fc"][0], [0.0, 2.0 * 0.1 / dt ** 2 * 0.075], rtol=1e-12)
    assert np.all(P["ft"][0] == 0.0)           # mu = 0: no friction
    # outside: everything zeroed, previous friction dropped
    P = one_particle((1.5, 0.5), ft=(3.0, 4.0))
    contact(P, square_tool(mu=0.3), c, dt, oracle_lib)
    assert np.all(P["fc"] == 0) and np.all(P["ft"] == 0) and np.all(P["n"] == 0)


def test_friction_ls_dyna_known_answer(oracle_lib):
    c, dt, mu = constants(), 0.01, 0.3
    tool = square_tool(mu=mu, vel=(0.5, 0.0))
    P = one_particle((0.5, 0.9), vel=(2.5, 3.0), ft=(1.0, 0.0))
    contact(P, tool, c, dt, oracle_lib)
    fN = np.array([0.0, 2.0 * 0.1 / dt ** 2 * 0.075])
    v = np.array([2.0, 3.0])                   # relative to the tool
    vr = v - v * np.array([0.0, 1.0])          # component-wise, as glm
    fstar = np.array([1.0, 0.0]) - 0.075 * 2.0 * vr / dt
    fy = mu * np.linalg.norm(fN)
    expect = fy * fstar / np.linalg.norm(fstar) if np.linalg.norm(fstar) > fy else fstar
    np.testing.assert_allclose(P["ft"][0], expect, rtol=1e-12)
    # tool particles never get contact forces
    P = one_particle((0.5, 0.9), tool=1.0)
    contact(P, tool, c, dt, oracle_lib)
    assert np.all(P["fc"] == 0)


def test_fillet_and_vertical_primitives(oracle_lib):
    """A particle near the fillet takes the fillet's normal; one near a vertical
    face takes the horizontal normal of the face."""
    t = RigidTool.from_angles((0.0, 1.0), 1.0, 1.0, 0.0, 7.0, 0.1, 0.0)
    assert len(t.segments) == 5 and t.fillet is not None
    f = t.fillet
    q = (f.p[0] + 0.09 * math.cos(-0.6), f.p[1] + 0.09 * math.sin(-0.6))   # inside the disc, below-right
    c, dt = constants(), 0.01
    P = one_particle(q)
    contact(P, t, c, dt, oracle_lib)
    n_expect = np.array(q) - np.array(f.p)
    n_expect /= np.linalg.norm(n_expect)
    np.testing.assert_allclose(P["n"][0], n_expect, rtol=1e-12)
    gN = (0.09 - 0.1)                          # depth below the arc
    np.testing.assert_allclose(P["fc"][0], -2.0 * gN * n_expect / dt ** 2 * 0.075, rtol=1e-9)
    # the rake face of a 0-degree tool is vertical: x = front
    seg = t.segments[1]
    assert seg.line.vertical
    P = one_particle((seg.left[0] - 0.02, 0.7))
    contact(P, t, c, dt, oracle_lib)
    np.testing.assert_allclose(P["n"][0], [1.0, 0.0], atol=0)
    np.testing.assert_allclose(P["fc"][0], [2.0 * 0.02 / dt ** 2 * 0.075, 0.0], rtol=1e-9)


def test_fillet_is_tangent_to_both_faces():
    for rake, clear, r in [(0.0, 7.0, 5e-4), (6.0, 7.0, 5e-4), (-6.0, 5.0, 2e-3), (10.0, 3.0, 1e-3)]:
        t = RigidTool.from_angles((-0.05, 0.1), 0.04, 0.04, rake, clear, r, 0.35)
        f = t.fillet
        # segments 1 and 3 end / start where the arc meets the faces; the centre
        # is r away from both face lines
        for k in (1, 3):
            s = t.segments[k]
            d = abs((s.right[0] - s.left[0]) * (s.left[1] - f.p[1]) - (s.left[0] - f.p[0]) * (s.right[1] - s.left[1]))
            d /= math.hypot(s.right[0] - s.left[0], s.right[1] - s.left[1])
            assert abs(d - r) < 1e-12 * max(1.0, 1 / r) * r + 1e-15, (rake, clear, k, d, r)
        assert 0 < f.t1 <= 2 * math.pi and 0 < f.t2 <= 2 * math.pi


def test_tool_motion_matches_host_restatement(oracle_lib):
    """orc_rigid_move (C++) and RigidTool.update (Python) are the same host
    arithmetic: bit-identical outlines over many steps."""
    t = RigidTool.from_angles((-0.05, 0.1), 0.04, 0.04, 6.0, 7.0, 5e-4, 0.35)
    t.vel = (8.3333328e-4, 1e-5)
    rt = t.to_struct()
    for _ in range(200):
        oracle_lib.orc_rigid_move(C.byref(rt), 0.37)
        t.update(0.37)
    ref = t.to_struct()
    for i in range(t.to_struct().n_seg):
        assert tuple(rt.left[i]) == tuple(ref.left[i])
        assert tuple(rt.right[i]) == tuple(ref.right[i])
        assert (rt.la[i], rt.lb[i], rt.vertical[i]) == (ref.la[i], ref.lb[i], ref.vertical[i])
    assert tuple(rt.fillet_p) == tuple(ref.fillet_p)


def test_friction_heat_known_answer(oracle_lib):
    c, dt = constants(mass=2.0, eta=0.9, cp=5e-6), 0.01
    P = one_particle((0.5, 0.5), vel=(2.0, 1.0), ft=(3.0, 4.0))
    P["n"][0] = (0.0, 1.0)
    P["T"][0] = 300.0
    p = abi.particles_struct(P, 1)
    vt = np.array([0.5, 0.0])
    oracle_lib.orc_fric_heat_rigid(C.byref(p), C.byref(c), abi.ptr(vt), dt)
    f = float(np.float32(25.0) ** 0.5)           # sqrtf of |ft|^2
    vrel = float(np.sqrt(np.float32(1.5 ** 2)))  # tangential part of v - v_tool
    np.testing.assert_allclose(P["T"][0], 300.0 + 0.9 * dt * f * vrel / (5e-6 * 2.0), rtol=1e-13)
    # eta == 0 switches it off
    P["T"][0] = 300.0
    c.trml_wp.eta = 0.0
    oracle_lib.orc_fric_heat_rigid(C.byref(p), C.byref(c), abi.ptr(vt), dt)
    assert P["T"][0] == 300.0


def pse_lattice(n=24, dx=1.0, hdx=1.5, field=lambda x, y: 0 * x):
    c = setups.micro(n_side=n, dx=dx, hdx=hdx, seed=1)
    P = c.particles
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    P["pos"][:] = np.stack([i.ravel() * dx, j.ravel() * dx], 1)
    P["rho"][:] = 1.0
    P["T"][:] = field(P["pos"][:, 0], P["pos"][:, 1])
    c.constants.phys.mass = dx * dx
    c.constants.trml_wp.alpha = 1.0
    c.constants.trml_tool_sph.alpha = 1.0
    return c


def run_pse(c):
    o = OracleSim(c.constants, c.grid, c.particles, c.dt, pse=True)
    o.assign_hashes()
    o.sort()
    o.interactions_heat_pse()
    return o


def test_pse_laplacian_known_answers(oracle_lib):
    h = 1.5
    # constant field: zero flux everywhere
    o = run_pse(pse_lattice(field=lambda x, y: 300.0 + 0 * x))
    assert np.all(o.P["T_t"] == 0.0)
    # T = x^2 + 3 y^2: Laplacian 8 in the interior (Gaussian truncated at the
    # 5x5 block of cells of edge h: a few per cent)
    o = run_pse(pse_lattice(field=lambda x, y: x * x + 3 * y * y))
    x, y = o.P["pos"][:, 0], o.P["pos"][:, 1]
    inner = (x > 4 * h) & (x < 23 - 4 * h) & (y > 4 * h) & (y < 23 - 4 * h)
    assert inner.sum() > 20
    np.testing.assert_allclose(o.P["T_t"][inner], 8.0, rtol=0.08)


def test_pse_matches_direct_block_sum(oracle_lib):
    """The oracle's cell-block PSE equals a direct numpy evaluation over the
    same 5x5 cell block (no support cut-off, blanked neighbours included).  The
    tool diffusivity applies to tool particles in the first half of the sorted
    order only: the reference binds its tool-flag texture over N ints of the
    N-double array (interactions_gpu.cu:448), so later ones read flag 0."""
    rng = np.random.default_rng(3)
    c = pse_lattice(n=16, field=lambda x, y: 300 + 10 * np.sin(x) * np.cos(0.7 * y))
    c.particles["pos"][:] += rng.uniform(-0.2, 0.2, c.particles["pos"].shape)
    c.particles["blanked"][::11] = 1.0
    c.particles["tool_particle"][::7] = 1.0
    c.constants.trml_tool_sph.alpha = 0.25
    o = run_pse(c)
    g = o.g
    P = o.P
    hashes = P["hash"]
    gi, gj = hashes // g.ny, hashes % g.ny
    for k in range(o.N):
        if P["blanked"][k] == 1.0:
            continue
        nb = (np.abs(gi - gi[k]) <= 2) & (np.abs(gj - gj[k]) <= 2)
        d = P["pos"][nb] - P["pos"][k]
        xx = np.sqrt((d * d).sum(1))
        hi = P["h"][k]
        w2 = 4.0 / (hi ** 4 * math.pi) * np.exp(-xx * xx / hi ** 2)
        s = np.sum((P["T"][nb] - P["T"][k]) * w2 * c.constants.phys.mass / P["rho"][nb])
        alpha = 0.25 if (P["tool_particle"][k] == 1.0 and k < o.N // 2) else 1.0
        assert abs(P["T_t"][k] - alpha * s) <= 1e-12 * max(1.0, abs(alpha * s)), k


def test_rigid_step_without_tool_is_the_plain_step(oracle_lib):
    """orc_step_rigid with no tool and the Brookshaw build is orc_step with no
    tool: the same call sequence, bit-identical states."""
    c = setups.micro(n_side=24, seed=5)
    a = OracleSim(c.constants, c.grid, c.particles, c.dt)
    b = OracleSim(c.constants, c.grid, c.particles, c.dt)
    for _ in range(2):
        a.step()
        p = b.pstruct()
        b.lib.orc_step_rigid(C.byref(p), abi.ptr(b.cell_start), abi.ptr(b.cell_end), C.byref(b.g), C.byref(b.C),
                             b.dt, None, 0)
    for k in a.P:
        assert np.array_equal(a.P[k], b.P[k], equal_nan=True), k


def test_ref_cut_setup_matches_reference_placement():
    """setup_ref_cut places the tool front at the workpiece front and its lowest
    point at the target feed below the top (benchmarks.cpp:388-412); tool
    particles lie inside the outline, fixed on its left and top rows."""
    for kw in [dict(), dict(chamfer=0.0), dict(rake=6.0)]:
        c = setups.ref_cut(ny=10, length=0.03, **kw)
        t = c.rigid
        assert abs((c.info["hi_y"] - t.low()) - c.feed) < 1e-12
        xmax = max(max(s.left[0], s.right[0]) for s in t.segments)
        if t.fillet:
            xmax = max(xmax, t.fillet.p[0] + t.fillet.r)
        P = c.particles
        tp = P["tool_particle"] == 1.0
        assert tp.sum() == c.info["n_tool"] > 0
        assert t.inside(P["pos"][tp]).all()
        assert np.all(P["rho"][tp] == 15.25)
        assert P["fixed"][tp].sum() > 0
        assert abs(t.vel[0] - 83.333328e-5) < 1e-18 and t.vel[1] == 0.0
        assert Line.through((0.0, 0.0), (0.0, 1.0)).vertical


# ---- pinned to the reference's own tool.cpp / geometric_primitives.cpp ------------------------------
GOLDEN_TOOL = __import__("pathlib").Path(__file__).resolve().parent / "golden" / "ref_tool_pin.npz"


def test_tool_geometry_matches_reference_golden():
    """RigidTool.from_angles + place + sample reproduce the reference's host
    geometry bit for bit (fixture from tests/golden/make_tool_golden.py)."""
    from sph_fem_2d_cutting_gpu_gb300.rigid_tool import place
    g = np.load(GOLDEN_TOOL)
    rows = g["inputs"]
    for k, r in enumerate(rows):
        tlx, tly, length, height, rake, clear, rad, mu, vel, lo_x, hi_y, feed, dx, pre = r
        t = RigidTool.from_angles((tlx, tly), length, height, rake, clear, rad, mu)
        place(t, lo_x, hi_y, feed, vel, pre)
        segs = np.array([[*s.left, *s.right, *s.n, s.line.a, s.line.b, 1.0 if s.line.vertical else 0.0]
                         for s in t.segments])
        ref = g[f"segs_{k}"]
        assert segs.shape == ref.shape, k
        # -0.0 and 0.0 print the same way; compare values
        assert np.array_equal(segs, ref), (k, np.argwhere(segs != ref))
        fr = g[f"fillet_{k}"]
        if t.fillet is None:
            assert np.isnan(fr).all(), k
        else:
            f = t.fillet
            assert np.array_equal([f.p[0], f.p[1], f.r, f.t1, f.t2], fr), k
        assert np.array_equal([t.low(), t.front], g[f"scalars_{k}"]), k
        assert np.array_equal(t.safe_bb(0.1 * dx), g[f"bb_{k}"]), k
        smp = t.sample(dx)
        assert np.array_equal(smp, g[f"samples_{k}"]), (k, len(smp), len(g[f"samples_{k}"]))
        # the packed struct the device moves carries the same outline
        st = t.to_struct()
        for i, s in enumerate(t.segments):
            assert (st.la[i], st.lb[i]) == (s.line.a, s.line.b)
