"""Scenario set-ups in the reference's unit system (cm, g, microsecond; stress
in Mbar = 100 GPa; temperature in K), following the template of
setup_ref_cut_FEM_tool_no_wear_thermal_paper (benchmarks_NZ.cpp:51-367).

Workloads:
  * ``ti64_cut``     -- Ti6Al4V orthogonal cut, 200 x 60 particles, dx = 5 um,
                        tool mesh of about 2,000 nodes (rake 0, clearance 7 deg,
                        edge radius 5 um), 70 m/min, uncut chip thickness 80 um.
  * ``micro``        -- 2048 x 2048 jittered lattice with dx = 2.5 um, random
                        velocity / stress / density, no tool.
  * ``aisi1045_cut`` -- AISI 1045 cut, 1600 x 400 particles, dx = 2.5 um, tool
                        mesh of about 20,000 nodes (rake -6, clearance 5 deg,
                        edge radius 20 um), 120 m/min, 100 um.
  * ``ref_cut``      -- the reference's SPH-tool cut (setup_ref_cut,
                        benchmarks.cpp:247-530): Ti6Al4V, workpiece 1.95 mm
                        long and 3 x feed high, rigid tool with optional
                        edge radius, sampled with thermal-only tool particles.
  * ``batched_sweep`` -- independent AISI 1045 cuts of uneven sizes (particle
                        counts log-uniform in [20k, 300k], height 0.5 mm,
                        speed U(30, 300) m/min, uncut chip thickness
                        U(20, 150) um, rake U(-10, 15) deg, tools of 2,000 to
                        8,000 nodes) for the batched context.
Unit conversions: 1 m/s = 1e-4 cm/us; 1 MPa = 1e-5 Mbar; 1 J/(kg K) = 1e-8
(g cm^2/us^2)/(g K); 1 W/(m K) = 1e-13 bomb units.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .rigid_tool import RigidTool
from .rigid_tool import place as place_rigid
from .tool_mesh import mesh_tool

MPMIN_TO_CMUS = 1.0 / 60.0 * 1e-4      # m/min -> cm/us


def wdeltap(hdx: float, dx: float) -> float:
    """Cubic-spline value at one particle spacing (benchmarks_NZ.cpp:131-136)."""
    h1 = 1.0 / (hdx * dx)
    q = dx * h1
    fac = 10 * (1.0 / math.pi) / 7.0 * h1 * h1
    return fac * (1 - 1.5 * q * q * (1 - 0.5 * q))


@dataclass
class Material:
    E: float
    nu: float
    rho0: float
    A: float
    B: float
    C: float
    n: float
    m: float
    Tmelt: float
    Tref: float = 300.0
    eps_dot_ref: float = 1e-6
    cp: float = 0.0
    k: float = 0.0
    tq: float = 0.9
    eta: float = 0.9


TI64 = Material(E=1.138, nu=0.342, rho0=4.43, A=0.00862, B=0.00331, C=0.012, n=0.34, m=0.8, Tmelt=1836.0,
                cp=526e-8, k=6.8e-13)
# AISI 1045: Johnson-Cook from the workload description; thermal data (not in
# the reference) cp = 486 J/(kg K), k = 49.8 W/(m K).
AISI1045 = Material(E=2.0, nu=0.3, rho0=7.85, A=0.005531, B=0.006008, C=0.0134, n=0.234, m=1.0, Tmelt=1733.0,
                    cp=486e-8, k=49.8e-13)


def make_constants(mat: Material, dx: float, hdx: float, mu: float = 0.35, plastic: bool = True,
                   thermal: bool = True) -> abi.Constants:
    c = abi.Constants()
    G = mat.E / (2.0 * (1.0 + mat.nu))
    c.phys.E, c.phys.nu, c.phys.rho0 = mat.E, mat.nu, mat.rho0
    c.phys.G = G
    c.phys.K = 2.0 * G * (1 + mat.nu) / (3 * (1 - 2 * mat.nu))
    c.phys.mass = dx * dx * mat.rho0
    rho_tool = 15.25
    c.phys.mass_tool = dx * dx * rho_tool
    c.joco.A, c.joco.B, c.joco.C, c.joco.n, c.joco.m = mat.A, mat.B, mat.C, mat.n, mat.m
    c.joco.Tmelt, c.joco.Tref, c.joco.eps_dot_ref = mat.Tmelt, mat.Tref, mat.eps_dot_ref
    if thermal:
        c.trml_wp.cp, c.trml_wp.tq, c.trml_wp.k = mat.cp, mat.tq, mat.k
        c.trml_wp.alpha = mat.k / (mat.rho0 * mat.cp)
        c.trml_wp.eta, c.trml_wp.T_init = mat.eta, mat.Tref
        # tool thermal constants of the reference set-up (benchmarks_NZ.cpp:118-122)
        c.trml_tool.cp, c.trml_tool.k = 15e-8, 59e-13
        c.trml_tool.alpha = c.trml_tool.k / (rho_tool * c.trml_tool.cp)
        c.trml_tool.T_init = mat.Tref
    c.corr.alpha, c.corr.beta, c.corr.eta = 1.0, 1.0, 0.1
    c.corr.xspheps, c.corr.stresseps = 0.5, 0.3
    c.corr.wdeltap = wdeltap(hdx, dx)
    # tool constants (benchmarks_NZ.cpp:194-205)
    t = c.tool
    t.cp, t.tq, t.k, t.eta, t.rho, t.T0 = 292e-8, 0.9, 88e-13, 1.0, 15.25, mat.Tref
    t.h, t.beta, t.mu, t.contact_alpha, t.slave_mass = 2e-10, 0.5, mu, 0.02, c.phys.mass
    c.plastic = 1 if plastic else 0
    return c


@dataclass
class Case:
    name: str
    constants: abi.Constants
    grid: abi.GridParams
    particles: dict            # numpy arrays by sph_particles field name
    N: int
    dt: float
    tool_mesh: dict | None = None
    tool_speed: float = 0.0
    feed: float = 0.0
    steps: int = 0
    info: dict = field(default_factory=dict)
    rigid: RigidTool | None = None     # rigid (SPH-mode) tool instead of a FEM tool

    def tool_struct(self):
        if self.tool_mesh is None:
            return None, []
        m = self.tool_mesh
        keep = [m["nodes"], m["elements"], m["cutting_flags"], m["fixed_flags"]]
        s = abi.ToolMesh()
        s.n_nodes = len(m["nodes"])
        s.n_elements = len(m["elements"])
        s.nodes = abi.ptr(m["nodes"])
        s.elements = abi.ptr(m["elements"])
        s.cutting_flags = abi.ptr(m["cutting_flags"])
        s.fixed_flags = abi.ptr(m["fixed_flags"])
        s.T_init = None
        s.tl[0], s.tl[1] = float(m["tl"][0]), float(m["tl"][1])
        return s, keep


def grid_params(bbmin, bbmax, h, cell_factor=1, stencil=2) -> abi.GridParams:
    g = abi.GridParams()
    g.bbmin[0], g.bbmin[1] = bbmin
    g.bbmax[0], g.bbmax[1] = bbmax
    g.h = h
    g.cell_factor = cell_factor
    g.stencil = stencil
    return g


def micro(n_side: int = 2048, dx: float = 2.5e-4, hdx: float = 1.7, seed: int = 0, cell_factor: int = 1,
          stencil: int = 2) -> Case:
    """Interaction micro-benchmark: jittered n_side x n_side lattice, no tool."""
    rng = np.random.default_rng(seed)
    N = n_side * n_side
    P = abi.empty_particles(N)
    i, j = np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="ij")
    pos = np.stack([i.ravel() * dx, j.ravel() * dx], 1)
    pos += rng.uniform(-0.05 * dx, 0.05 * dx, size=pos.shape)
    P["pos"][:] = pos
    P["vel"][:] = rng.normal(0.0, 1e-4, size=(N, 2))             # N(0, 1 m/s)
    sxx, sxy, syy, szz = (rng.normal(0.0, 0.002, size=N) for _ in range(4))   # N(0, 200 MPa)
    P["S"][:] = np.stack([sxx, sxy, syy, szz], 1)
    mat = AISI1045
    P["rho"][:] = mat.rho0 * (1.0 + rng.uniform(-1e-3, 1e-3, size=N))
    P["h"][:] = hdx * dx
    P["T"][:] = 300.0
    P["on_seg"][:] = -1
    c = make_constants(mat, dx, hdx)
    h = hdx * dx
    lo = pos.min(0) - 1e-8
    hi = pos.max(0) + 1e-8
    # margin of two smoothing lengths so the one step stays inside the grid
    g = grid_params((lo[0] - 2 * h, lo[1] - 2 * h), (hi[0] + 2 * h, hi[1] + 2 * h), h, cell_factor, stencil)
    dt = 0.3 * hdx * dx / (math.sqrt(c.phys.K / c.phys.rho0))
    return Case("micro", c, g, P, N, dt, info=dict(n_side=n_side, dx=dx, hdx=hdx, seed=seed))


def cutting(name: str, mat: Material, nx: int, ny: int, dx: float, hdx: float, speed_mpmin: float, feed: float,
            rake: float, clearance: float, r: float, mu: float, s_min: float, s_max: float, tool_size: float,
            cfl: float = 0.3, steps: int = 0, cell_factor: int = 1, stencil: int = 2) -> Case:
    """Orthogonal cut following benchmarks_NZ.cpp:51-367 (lattice, fixed
    boundaries, tool placement at the target feed, locked grid, CFL step)."""
    lo_x, lo_y = 0.005, 0.0
    hi_y = lo_y + (ny - 1) * dx
    N = nx * ny
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    pos = np.stack([i.ravel() * dx + lo_x, j.ravel() * dx + lo_y], 1)
    min_x, min_y = pos.min(0)
    max_x, max_y = pos.max(0)
    P = abi.empty_particles(N)
    P["pos"][:] = pos
    P["rho"][:] = mat.rho0
    P["h"][:] = hdx * dx
    P["T"][:] = mat.Tref
    fixed = (pos[:, 1] < min_y + 0.5 * dx)
    fixed |= (pos[:, 0] < min_x + dx / 2) & (pos[:, 1] < min_y + 0.5 * (hi_y - lo_y))
    fixed |= pos[:, 0] > max_x - dx
    P["fixed"][:] = fixed.astype(np.float64)
    P["on_seg"][:] = 0
    c = make_constants(mat, dx, hdx, mu=mu)
    vel_tool = speed_mpmin * MPMIN_TO_CMUS
    tl = (-tool_size, hi_y + 0.5 * tool_size)
    mesh = mesh_tool(tl, tool_size, tool_size, rake, clearance, r, s_min=s_min, s_max=s_max)
    bbmin = pos.min(0) - 1e-8
    bbmax = pos.max(0) + 1e-8 + np.array([300 * dx, 500 * dx])
    bbmax[1] = max(bbmax[1], hi_y + (max_x + dx) - lo_x)
    g = grid_params(tuple(bbmin), tuple(bbmax), hdx * dx, cell_factor, stencil)
    dt = cfl * hdx * dx / (math.sqrt(c.phys.K / c.phys.rho0) + math.sqrt(vel_tool))   # benchmarks_NZ.cpp:360
    case = Case(name, c, g, P, N, dt, tool_mesh=mesh, tool_speed=vel_tool, feed=feed, steps=steps,
                info=dict(nx=nx, ny=ny, dx=dx, hdx=hdx, lo_x=lo_x, hi_y=hi_y, rake=rake, clearance=clearance, r=r,
                          nodes=len(mesh["nodes"]), elements=len(mesh["elements"])))
    return case


def ti64_cut(steps: int = 2000, **kw) -> Case:
    return cutting("ti64_cut", TI64, 200, 60, 5e-4, 1.7, 70.0, 0.008, 0.0, 7.0, 5e-4, 0.35,
                   s_min=1.0e-4, s_max=3.0e-3, tool_size=0.06, steps=steps, **kw)


def aisi1045_cut(steps: int = 20000, **kw) -> Case:
    return cutting("aisi1045_cut", AISI1045, 1600, 400, 2.5e-4, 1.7, 120.0, 0.01, -6.0, 5.0, 2e-3, 0.35,
                   s_min=5.5e-5, s_max=2.5e-3, tool_size=0.2, steps=steps, **kw)


def small_cut(nx: int = 40, ny: int = 16, steps: int = 20, **kw) -> Case:
    """A few hundred particles and a coarse tool: sizes the CPU oracle finishes in seconds."""
    return cutting("small_cut", TI64, nx, ny, 5e-4, 1.7, 300.0, 0.002, 0.0, 7.0, 5e-4, 0.35,
                   s_min=2e-4, s_max=2.5e-3, tool_size=0.015, steps=steps, **kw)


def placed(case: Case, preload_dx: float = 0.0, mode: str = "reference") -> Case:
    """Copy of a cutting case whose tool mesh is already at its start position.

    mode "reference": the placement of benchmarks_NZ.cpp:247-267 -- the tool
    moves left until its right point (largest node x) is 0.01 dx left of the
    workpiece, then vertically to the target uncut chip thickness.  With a
    negative rake angle the right point is the top of the rake face, above
    the workpiece, and the cutting edge starts far from the workpiece.
    mode "edge": after the vertical move, the rightmost node at or below the
    workpiece top is put 0.01 dx left of the workpiece, so every rake angle
    starts in contact.
    The moves are applied to the mesh nodes (and the mesh's top-left
    reference point) on the host, as one translation, so the case needs no
    tool moves on the device (batched contexts take placed tools).
    ``preload_dx`` moves the tool that many dx further in the cutting
    direction (contact from the first step)."""
    import copy
    assert case.tool_mesh is not None
    st = abi.tool_model_host(case)["state"]
    dx = case.info["dx"]
    current_feed = case.info["hi_y"] - st.lowest_point
    sign = 1.0 if current_feed > case.feed else -1.0
    shift_y = sign * abs(current_feed - case.feed)
    nodes = case.tool_mesh["nodes"]
    if mode == "reference":
        shift_x = -(st.right_point - case.info["lo_x"] + dx * 0.01)
    elif mode == "edge":
        band = nodes[:, 1] + shift_y <= case.info["hi_y"] + 1e-12
        shift_x = case.info["lo_x"] - dx * 0.01 - float(nodes[band, 0].max())
    else:
        raise ValueError(mode)
    shift_x += preload_dx * dx
    out = copy.copy(case)
    m = dict(case.tool_mesh)
    m["nodes"] = np.ascontiguousarray(nodes + np.array([shift_x, shift_y]))
    m["tl"] = (case.tool_mesh["tl"][0] + shift_x, case.tool_mesh["tl"][1] + shift_y)
    out.tool_mesh = m
    out.info = dict(case.info, placed_shift=(shift_x, shift_y), placement=mode)
    return out


def _tool_size_for(nodes: float) -> float:
    """Tool edge length (cm) whose graded mesh (s_min 1 um, s_max 30 um, edge
    radius 20 um) has about `nodes` nodes; piecewise linear fit of measured
    counts."""
    return float(np.interp(nodes, [2600.0, 3700.0, 6400.0, 8000.0], [0.03, 0.06, 0.10, 0.115]))


def batched_sweep(n_cases: int = 64, seed: int = 0, n_min: int = 20_000, n_max: int = 300_000,
                  dx: float = 2.5e-4, height: float = 0.05, steps: int = 5000, cell_factor: int = 1,
                  stencil: int = 2) -> list[Case]:
    """Independent AISI 1045 cuts of uneven sizes (placed tools), drawn from `seed`."""
    rng = np.random.default_rng(seed)
    ny = int(round(height / dx))
    cases = []
    for k in range(n_cases):
        count = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
        nx = max(8, int(round(count / ny)))
        speed = rng.uniform(30.0, 300.0)
        feed = rng.uniform(20e-4, 150e-4)
        rake = rng.uniform(-10.0, 15.0)
        target_nodes = rng.uniform(2000.0, 8000.0)
        size = _tool_size_for(max(target_nodes, 2600.0))
        c = cutting(f"sweep{k}", AISI1045, nx, ny, dx, 1.7, speed, feed, rake, 5.0, 2e-3, 0.35,
                    s_min=1e-4, s_max=3e-3, tool_size=size, steps=steps, cell_factor=cell_factor, stencil=stencil)
        c.info.update(speed_mpmin=speed, target_nodes=target_nodes, case_index=k, seed=seed)
        cases.append(placed(c, mode="edge"))
    return cases


def moved(case: Case, shift_x: float, shift_y: float = 0.0) -> Case:
    """Copy of a placed case with its tool mesh translated by (shift_x,
    shift_y): the tool of a run restarted from a state in which the tool has
    advanced (the rigid motion of tool_FEM.cu:109-139 as one translation)."""
    import copy
    out = copy.copy(case)
    m = dict(case.tool_mesh)
    m["nodes"] = np.ascontiguousarray(case.tool_mesh["nodes"] + np.array([shift_x, shift_y]))
    m["tl"] = (case.tool_mesh["tl"][0] + shift_x, case.tool_mesh["tl"][1] + shift_y)
    out.tool_mesh = m
    return out


# tool of setup_ref_cut, from Ruettimann's FEM simulations (benchmarks.cpp:384-390)
REF_CUT_TOOL_TL = (-0.05 + 0.004, 0.0986074)
REF_CUT_TOOL_LENGTH = -0.0086824 - -0.05
REF_CUT_TOOL_HEIGHT = 0.0986074 - 0.0555074

# Ti6Al4V of setup_ref_cut (benchmarks.cpp:263-287, Johnson 85)
TI64_REF = Material(E=1.1, nu=0.35, rho0=4.429998, A=0.0085200, B=0.0033890, C=0.02754, n=0.148, m=0.5961,
                    Tmelt=1836.0, cp=580e-8, k=7.3e-13)


def ref_cut(ny: int = 10, rake: float = 0.0, clear: float = 7.0, chamfer: float = 5e-4, speed: float = 0.0,
            feed: float = 0.002, length: float = 0.195, sample_tool: bool = True, preload_dx: float = 0.0,
            steps: int = 0, cell_factor: int = 1, stencil: int = 2) -> Case:
    """setup_ref_cut (benchmarks.cpp:247-530): Ti6Al4V workpiece of ny rows and
    3 x feed height (length 1.95 mm in the reference; shorter here for small
    cases), a rigid tool of rake / clearance angle (degrees) and edge radius
    `chamfer` placed at the workpiece front and the target feed, and the tool
    sampled with particles that take part in heat conduction only.  speed in
    cm/us (0: the reference's 500 m/min).  preload_dx moves the tool that many
    particle spacings into the workpiece (0 in the reference)."""
    mat = TI64_REF
    hi_y, lo_x = 0.060, 0.005
    hi_x = lo_x + length
    lo_y = hi_y - 3 * feed
    dy = (hi_y - lo_y) / (ny - 1)
    dx = dy
    nx = int((hi_x - lo_x) / dx)
    hdx = 1.5
    c = make_constants(mat, dx, hdx, mu=0.35)
    rho_tool = 15.25
    c.phys.mass_tool = dx * dx * rho_tool
    c.joco.tanh_a, c.joco.tanh_b, c.joco.tanh_c, c.joco.tanh_d = 1.1, 0.4, 12.0, 1.0
    # tool thermal constants (benchmarks.cpp:303-309); the same for the SPH tool's
    # conduction and for the thermal boundary switch
    for t in (c.trml_tool, c.trml_tool_sph):
        t.cp, t.tq, t.k, t.eta = 292e-8, 0.0, 88e-13, 0.0
        t.alpha = t.k / (rho_tool * t.cp)
        t.T_init = mat.Tref
    c.tool.contact_alpha = 0.075           # benchmarks.cpp:414
    c.tool.slave_mass = c.phys.mass
    # workpiece lattice and its fixed boundaries (benchmarks.cpp:326-374)
    i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    pos = np.stack([i.ravel() * dx + lo_x, j.ravel() * dx + lo_y], 1)
    min_x, min_y = pos.min(0)
    max_x, max_y = pos.max(0)
    fixed = pos[:, 1] < min_y + 0.5 * dx
    fixed |= (pos[:, 0] < min_x + dx / 2) & (pos[:, 1] < min_y + 0.5 * (hi_y - lo_y))
    fixed |= pos[:, 0] > max_x - dx
    vel_tool = 83.333328 * 1e-5 if speed == 0.0 else speed
    # tool from Ruettimann's FEM simulations, moved to the workpiece front and the
    # target feed (benchmarks.cpp:378-412)
    tl = REF_CUT_TOOL_TL
    tool = RigidTool.from_angles(tl, REF_CUT_TOOL_LENGTH, REF_CUT_TOOL_HEIGHT, rake, clear, chamfer, 0.35)
    place_rigid(tool, lo_x, hi_y, feed, vel_tool, preload_dx * dx / vel_tool)
    n_wp = nx * ny
    # tool particles (benchmarks.cpp:418-450)
    tpos = tool.sample(dx) if sample_tool else np.zeros((0, 2))
    n_tool = len(tpos)
    N = n_wp + n_tool
    P = abi.empty_particles(N)
    P["pos"][:n_wp] = pos
    P["pos"][n_wp:] = tpos
    P["rho"][:n_wp] = mat.rho0
    P["rho"][n_wp:] = rho_tool
    P["h"][:] = hdx * dx
    P["T"][:] = mat.Tref
    P["fixed"][:n_wp] = fixed.astype(np.float64)
    if n_tool:
        tfix = (tpos[:, 0] < tpos[:, 0].min() + dx / 2) | (tpos[:, 1] > tpos[:, 1].max() - dx / 2)
        P["fixed"][n_wp:] = tfix.astype(np.float64)
    P["tool_particle"][n_wp:] = 1.0
    P["on_seg"][:] = -1
    # domain (benchmarks.cpp:456-487)
    allpos = P["pos"]
    bbmin = allpos.min(0) - 1e-8
    bbmax = allpos.max(0) + 1e-8
    tx0, tx1, ty0, ty1 = tool.safe_bb(1e-3)
    bbmin = np.minimum(bbmin, [tx0, ty0])
    bbmax = np.array([max(bbmax[0], tx1) + 10 * dx, max(bbmax[1], ty1)])
    bbmax[1] = max(bbmax[1], hi_y + hi_x - lo_x)
    g = grid_params(tuple(bbmin), tuple(bbmax), hdx * dx, cell_factor, stencil)
    dt = 0.32 * hdx * dx / (math.sqrt(c.phys.K / c.phys.rho0) + math.sqrt(vel_tool))   # benchmarks.cpp:518
    return Case("ref_cut", c, g, P, N, dt, tool_speed=vel_tool, feed=feed, steps=steps,
                info=dict(nx=nx, ny=ny, dx=dx, hdx=hdx, n_workpiece=n_wp, n_tool=n_tool, rake=rake, clear=clear,
                          chamfer=chamfer, lo_x=lo_x, hi_y=hi_y, usui_K=7.8 / 100, usui_alpha=2500.0),
                rigid=tool)
