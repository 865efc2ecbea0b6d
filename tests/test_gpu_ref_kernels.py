"""Parity pinned to the reference's own CUDA code.

The reference's actions_gpu.cu, leap_frog.cu, grid.cu and interactions_gpu.cu are compiled,
unmodified, into cubins (oracle/Makefile target ``ref_gpu``; built where the
reference tree is present and carried to the GPU host with the other built
files).  Each test uploads one seeded state to the product, runs one staged
call through the C ABI, runs the reference kernel that call replaces on a
copy of the same state (oracle/ref_gpu.py, CUDA driver API) and compares:
  - every field bit for bit (EOS, continuity, momentum, advection, the
    Johnson-Cook return mapping, boundary conditions, invalidation,
    predictor / corrector, cell hashes), except
  - the Jaumann rate within 1e-13 relative, norm-wise: the reference forms it
    with GLM 3x3 matrix products, the product with the expanded 2-D terms, and
    the compiler contracts them into FMAs differently;
  - the artificial stress R within 1e-6: the reference evaluates the stress
    angle's atan2f / cosf / sinf with CUDA's float functions, the product
    evaluates them in double and rounds once to float (so that the CPU oracle
    reproduces it), and the two agree to a few float ULPs (2^-23 relative).
The state is a small cut after 15 fused steps with the tool in contact, then
spread out so every branch of the kernels runs: random velocity and stress
gradients, stresses beyond yield, temperatures above melting, tool, fixed and
blanked particles, NaN / Inf rates for the invalidation.
"""
import ctypes as C

import numpy as np
import pytest

from sph_fem_2d_cutting_gpu_gb300 import abi, setups
from sph_fem_2d_cutting_gpu_gb300.solver import Solver
from conftest import rel_err

pytestmark = pytest.mark.gpu

RTOL = 0.0   # bit for bit
RTOL_JAUMANN = 1e-13
RTOL_FLOAT_TRIG = 1e-6   # R: CUDA's float atan2f / cosf / sinf against double-evaluated, once-rounded
torch = pytest.importorskip("torch")
ref_gpu = pytest.importorskip("oracle.ref_gpu")
if not all((ref_gpu.REF_DIR / f).exists() for f in ref_gpu.CUBINS.values()):
    pytest.skip("the reference cubins are not built here (oracle/Makefile target ref_gpu needs the "
                "reference tree at build time)", allow_module_level=True)


def module(which):
    try:
        return ref_gpu.RefModule(which)
    except FileNotFoundError as e:
        pytest.skip(f"reference cubin not built here: {e}")


@pytest.fixture(scope="module")
def base():
    c = setups.small_cut()
    s = Solver(c)
    s.move_tool(0.3 * c.info["dx"] / c.tool_speed)
    s.step(15)
    H = s.download()
    s.close()
    return c, spread(H)


def spread(H, seed=5):
    rng = np.random.default_rng(seed)
    H = {k: v.copy() for k, v in H.items()}
    N = len(H["rho"])

    def noise(a, scale):
        return a + rng.normal(0.0, 1.0, a.shape) * scale

    for f in ("v_der", "S_der"):
        H[f] = noise(H[f], 3.0 * np.abs(H[f]).std() + 1e-6)
    for f in ("fc", "ft", "n"):
        H[f] = noise(H[f], np.abs(H[f]).std() + 1e-9)
    sel = rng.random(N) < 0.3                          # beyond yield
    H["S"][sel] *= rng.uniform(1.5, 4.0, (sel.sum(), 1))
    H["S"] = noise(H["S"], 0.05 * np.abs(H["S"]).std())
    H["eps_pl"] = np.abs(noise(H["eps_pl"], 0.05))
    H["eps_pl_dot"] = np.abs(noise(H["eps_pl_dot"], 1e-3))
    hot = rng.random(N) < 0.1                          # some above melting
    H["T"][hot] += rng.uniform(0.0, 2000.0, hot.sum())
    H["rho"] = H["rho"] * rng.uniform(0.97, 1.03, N)
    for f, frac in (("tool_particle", 0.05), ("fixed", 0.05), ("blanked", 0.03)):
        H[f] = (rng.random(N) < frac).astype(np.float64)
    for f in ("pos_t", "vel_t", "S_t", "rho_t", "T_t"):
        H[f] = noise(H[f], np.abs(H[f]).std() + 1e-9)
    return H


def device(H):
    return {k: torch.tensor(np.ascontiguousarray(v), device="cuda") for k, v in H.items()}


def particle_struct(T, N):
    pg = ref_gpu.ParticleGPU()
    for f, _, _ in abi.PARTICLE_FIELDS:
        setattr(pg, f, ref_gpu.ptr(T[f]))
    pg.N = N
    return pg


@pytest.fixture(scope="module")
def actions(lib, base):
    m = module("actions")
    c = base[0].constants
    m.launch("ref_set_actions_constants", 1, c.phys, c.corr, c.joco, c.trml_wp, c.trml_tool, c.tool,
             abi.WearConstants(0.0, 0.0, 0.0, 0.0), block=1)
    return m


def product_after(case, H, calls):
    s = Solver(case)
    s.upload(H)
    for name, *args in calls:
        s.call(name, *args)
    G = s.download()
    s.close()
    return G


def check(G, R, fields, exact=(), rtol=RTOL):
    for f in fields:
        a, b = G[f], R[f]
        if f in exact:
            assert np.array_equal(a, b, equal_nan=True), f"{f}: {np.count_nonzero(a != b)} entries differ"
        else:
            fin = np.isfinite(b)
            assert np.array_equal(np.isfinite(a), fin), f"{f}: non-finite entries differ"
            if rtol == 0.0:
                assert np.array_equal(a, b, equal_nan=True), f"{f}: {np.count_nonzero(a != b)} entries differ"
            else:
                e = rel_err(a[fin], b[fin])
                assert e <= rtol, f"{f}: relative error {e:.3e}"


def ref_run(H, launch):
    T = device(H)
    N = len(H["rho"])
    launch(T, particle_struct(T, N), N)
    return {k: v.cpu().numpy() for k, v in T.items()}


P = ref_gpu.ptr if ref_gpu else None


def test_eos(actions, base):
    c, H = base
    G = product_after(c, H, [("sph_material_eos",)])
    R = ref_run(H, lambda T, pg, N: actions.launch("do_material_eos", N, P(T["rho"]), P(T["p"]),
                                                    P(T["tool_particle"]), C.c_int32(N)))
    check(G, R, ["p"])


def test_artificial_stress(actions, base):
    c, H = base
    G = product_after(c, H, [("sph_corrector_artificial_stress",)])
    R = ref_run(H, lambda T, pg, N: actions.launch("do_corrector_artificial_stress", N, P(T["rho"]), P(T["p"]),
                                                    P(T["S"]), P(T["tool_particle"]), P(T["R"]), C.c_int32(N)))
    check(G, R, ["R"], rtol=RTOL_FLOAT_TRIG)


def test_jaumann(actions, base):
    c, H = base
    G = product_after(c, H, [("sph_material_stress_rate_jaumann",)])
    R = ref_run(H, lambda T, pg, N: actions.launch("do_material_stress_rate_jaumann", N, P(T["v_der"]), P(T["S"]),
                                                    P(T["tool_particle"]), P(T["S_t"]), C.c_int32(N)))
    check(G, R, ["S_t"], rtol=RTOL_JAUMANN)


def test_continuity_momentum_advection(actions, base):
    c, H = base
    G = product_after(c, H, [("sph_contmech_continuity",), ("sph_contmech_momentum",), ("sph_contmech_advection",)])

    def launch(T, pg, N):
        actions.launch("do_contmech_continuity", N, P(T["rho"]), P(T["v_der"]), P(T["tool_particle"]),
                       P(T["rho_t"]), C.c_int32(N))
        actions.launch("do_contmech_momentum", N, P(T["S_der"]), P(T["fc"]), P(T["ft"]), P(T["tool_particle"]),
                       P(T["vel_t"]), C.c_int32(N))
        actions.launch("do_contmech_advection", N, P(T["vel"]), P(T["tool_particle"]), P(T["pos_t"]), C.c_int32(N))

    R = ref_run(H, launch)
    check(G, R, ["rho_t", "vel_t", "pos_t"])


def test_plasticity(actions, base):
    c, H = base
    assert c.constants.plastic
    G = product_after(c, H, [("sph_material_eos",), ("sph_plasticity_johnson_cook",)])

    def launch(T, pg, N):
        actions.launch("do_material_eos", N, P(T["rho"]), P(T["p"]), P(T["tool_particle"]), C.c_int32(N))
        actions.launch("do_plasticity_johnson_cook", N, pg, C.c_double(c.dt))

    R = ref_run(H, launch)
    check(G, R, ["S", "eps_pl", "eps_pl_dot", "T", "blanked"], exact=["blanked"])
    yielded = R["eps_pl_dot"] > 0
    assert yielded.sum() > 50, "the state exercises the return mapping"
    assert np.count_nonzero(R["blanked"] != H["blanked"]) > 0, "and the melting cap"


def test_boundary_conditions(actions, base):
    c, H = base
    calls = [("sph_perform_boundary_conditions",)]
    thermal = c.constants.trml_tool.alpha != 0.0
    if thermal:
        calls.append(("sph_perform_boundary_conditions_thermal",))
    G = product_after(c, H, calls)

    def launch(T, pg, N):
        actions.launch("do_boundary_conditions", N, pg)
        if thermal:
            actions.launch("do_boundary_conditions_thermal", N, pg)

    R = ref_run(H, launch)
    check(G, R, ["vel", "fc", "pos_t", "vel_t", "T"])


def test_invalidate(actions, base):
    c, H = base
    H = {k: v.copy() for k, v in H.items()}
    rng = np.random.default_rng(9)
    N = len(H["rho"])
    for f, bad in (("pos_t", np.nan), ("vel_t", np.inf), ("S_t", -np.inf), ("rho_t", np.nan), ("T_t", np.inf)):
        idx = rng.choice(N, 3, replace=False)
        H[f][idx] = bad
    G = product_after(c, H, [("sph_debug_invalidate",)])
    R = ref_run(H, lambda T, pg, N: actions.launch("do_invalidate", N, pg, C.c_int32(0)))
    check(G, R, ["blanked"], exact=["blanked"])
    assert np.count_nonzero(R["blanked"] != H["blanked"]) >= 10


@pytest.mark.parametrize("stage", ["predict", "correct"])
def test_leap_frog(lib, base, stage):
    m = module("leap_frog")
    c, H = base
    G = product_after(c, H, [("sph_init",), ("sph_" + stage,)])
    N = len(H["rho"])
    ini = {"pos_init": (N, 2), "vel_init": (N, 2), "S_init": (N, 4), "rho_init": (N,), "T_init": (N,),
           "T_init_tool": (1,)}
    I = {k: torch.zeros(v, dtype=torch.float64, device="cuda") for k, v in ini.items()}
    st = ref_gpu.IniState(**{k: ref_gpu.ptr(v) for k, v in I.items()})

    def launch(T, pg, N):
        m.launch("init", N, pg, st)
        m.launch(stage, N, pg, st, C.c_double(c.dt))

    R = ref_run(H, launch)
    check(G, R, ["pos", "vel", "S", "rho", "T"])


def test_compute_hashes(lib, base):
    """compute_hashes (grid.cu:25-42) against the product's FP32-first cell index:
    positions on, next to and between cell edges, blanked particles keep a stale hash."""
    m = module("grid")
    c, H = base
    s = Solver(c)
    g = s.geometry()
    s.close()
    rng = np.random.default_rng(17)
    N = len(H["rho"])
    ix = rng.integers(0, g.nx, N)
    iy = rng.integers(0, g.ny, N)
    frac = rng.choice([0.0, 1e-15, 0.5, 1 - 1e-15, 1 - 2.2e-16], (N, 2))
    H = {k: v.copy() for k, v in H.items()}
    H["pos"][:, 0] = g.bbmin_x + (ix + frac[:, 0]) * g.dx
    H["pos"][:, 1] = g.bbmin_y + (iy + frac[:, 1]) * g.dx
    H["hash"] = rng.integers(-5, 5, N).astype(np.int32)   # stale values the blanked particles keep
    G = product_after(c, H, [("sph_assign_hashes",)])
    R = ref_run(H, lambda T, pg, N: m.launch("compute_hashes", N, P(T["blanked"]), P(T["pos"]), P(T["hash"]),
                                              C.c_int32(N), C.c_double(g.dx), C.c_int32(g.ny),
                                              C.c_double(g.bbmin_x), C.c_double(g.bbmin_y)))
    check(G, R, ["hash"], exact=["hash"])


# ---- contact and friction heat with the FEM tool (live tool state) -------------------------------
@pytest.fixture(scope="module")
def cut(lib):
    """The 12,000-particle Ti6Al4V cut with the tool pushed 0.3 dx into the
    workpiece, after 40 fused steps (about 15 particles in contact; a deeper
    push blanks the penetrated particles instead); the solver stays open."""
    c = setups.ti64_cut()
    s = Solver(c)
    s.move_tool(0.3 * c.info["dx"] / c.tool_speed)
    s.step(40)
    yield c, s
    s.close()


def segment_struct(seg, n, wear=None):
    T = {k: torch.tensor(np.ascontiguousarray(v), device="cuda") for k, v in seg.items()}
    W = wear or dict(wear_rate=np.zeros((n, 2)), wear_nodes=np.zeros(n), physical_para=np.zeros((n, 4)),
                     sliding_force=np.zeros(n))
    T.update({k: torch.tensor(np.ascontiguousarray(v), device="cuda") for k, v in W.items()})
    sg = ref_gpu.SegmentFEMGPU()
    sg.segment_num = n
    for k, src in (("left", "left"), ("right", "right"), ("n", "normal"), ("marks", "marks"),
                   ("heat_exchange", "heat_exchange"), ("fric_heat", "fric_heat"), ("wear_rate", "wear_rate"),
                   ("wear_nodes", "wear_nodes"), ("physical_para", "physical_para"), ("sliding_force", "sliding_force")):
        setattr(sg, k, ref_gpu.ptr(T[src]))
    return T, sg


def test_contact_forces(actions, cut):
    """compute_contact_forces_FEM_tool_v3 (actions_gpu.cu:983-999 -> :423-617): penalty
    normal force, friction, segment ids, penetration blanking, the particle-segment
    heat exchange (FP64 atomics: sums within 1e-13).  Both reference kernels call
    __syncthreads() after their early returns, so they run here one thread per
    block: no thread of a block can have left before the barrier."""
    c, s = cut
    H, seg, ts, fem = s.download(), s.segments(), s.tool_state(), s.fem()
    n = ts.n_segments
    s.call("sph_compute_contact_forces_fem")
    G, Gseg = s.download(), s.segments()
    S, sg = segment_struct(seg, n)
    Tn = torch.tensor(fem["T"], device="cuda")

    def launch(T, pg, N):
        actions.launch("do_compute_contact_forces_FEM_tool_v3_s1", N, C.c_int32(N), pg, sg,
                       ref_gpu.Vec2(*ts.tl_point_ref), C.c_double(ts.ref_dist), ref_gpu.Vec2(*ts.vel),
                       C.c_double(c.dt), C.c_int32(n), block=1)
        actions.launch("do_compute_contact_forces_FEM_tool_v3_s2", N, C.c_int32(N), pg, sg, P(Tn),
                       C.c_double(c.dt), block=1)

    R = ref_run(H, launch)
    check(G, R, ["on_seg", "blanked", "fc", "ft", "n", "T"], exact=["on_seg", "blanked"])
    assert np.count_nonzero(R["on_seg"] >= 0) >= 8, "particles in contact"
    e = rel_err(Gseg["heat_exchange"], S["heat_exchange"].cpu().numpy())
    assert e <= 1e-13, f"heat_exchange: {e:.3e}"


@pytest.mark.parametrize("wear", [False, True], ids=["plain", "wear_statistics"])
def test_friction_heat(actions, cut, wear):
    """material_fric_heat_gen_FEM_v2 (actions_gpu.cu:967-981 -> :345-420): particle
    heating, the tool's share per segment and, with WEAR_NODE_SHIFT, the segment
    statistics (FP64 atomics: sums within 1e-13)."""
    c, s = cut
    if wear:
        s.set_wear(abi.SPH_WEAR_ACCUMULATE, abi.WearConstants(10.0, 300.0, 10.0, 300.0))
        s.call("sph_segments_wear_rate_reset")
    H, seg, ts, fem = s.download(), s.segments(), s.tool_state(), s.fem()
    n = ts.n_segments
    s.call("sph_material_fric_heat_gen_fem")
    G, Gseg = s.download(), s.segments()
    S, sg = segment_struct(seg, n)
    Tn = torch.tensor(fem["T"], device="cuda")
    R = ref_run(H, lambda T, pg, N: actions.launch("do_material_fric_heat_gen_FEM_v21", N, pg, sg,
                                                    ref_gpu.Vec2(*ts.vel), P(Tn), C.c_double(c.dt), C.c_int32(N)))
    check(G, R, ["T", "blanked"], exact=["blanked"])
    assert np.count_nonzero(G["T"] != H["T"]) >= 4, "particles heated by friction"
    e = rel_err(Gseg["fric_heat"], S["fric_heat"].cpu().numpy())
    assert e <= 1e-13, f"fric_heat: {e:.3e}"
    if wear:
        w = s.wear_state()
        for k, src in (("phys_para", "physical_para"), ("sliding_force", "sliding_force")):
            e = rel_err(w[k], S[src].cpu().numpy())
            assert e <= 1e-13, f"{k}: {e:.3e}"
        assert w["phys_para"][:, 0].sum() > 0
        s.set_wear(abi.SPH_WEAR_OFF)


# ---- neighbour sums: do_interactions_monaghan and do_interactions_heat_pse -----------------------
# interactions_gpu.cu with its texture references served by ref_shim/texture_ref.h.
# The product visits the same cells in the same order but skips out-of-support
# candidates (the reference adds exact zeros for them) and folds per-neighbour
# quotients into its records (reassociation at the 1e-16 level per term), so the
# sums are compared within 1e-12 relative, norm-wise.
RTOL_SUMS = 1e-12


def interactions_module(c, geom):
    m = module("interactions")
    k = c.constants
    ge = ref_gpu.GeomConstants(geom.nx, geom.ny, geom.bbmin_x, geom.bbmin_y, geom.dx)
    m.launch("ref_set_interactions_constants", 1, k.phys, k.corr, ge, k.trml_wp, k.trml_tool_sph, k.tool, block=1)
    return m


def sorted_product(c, H, pse=False):
    """The product on state H, sorted into cells, with pressure and artificial stress."""
    s = Solver(c)
    if pse:
        s.set_thermal_model(abi.SPH_THERMAL_PSE)
    s.upload(H)
    for name in ("sph_assign_hashes", "sph_sort", "sph_material_eos", "sph_corrector_artificial_stress"):
        s.call(name)
    return s


def test_interactions_monaghan(lib, base):
    c, H = base
    s = sorted_product(c, H)
    H2, (cs, ce), g = s.download(), s.cells(), s.geometry()
    assert c.grid.cell_factor == 1 and c.grid.stencil == 2      # the reference's cells of h, 5x5
    s.call("sph_interactions_monaghan")
    G = s.download()
    s.close()
    m = interactions_module(c, g)
    N = len(H2["rho"])
    T = device(H2)
    CS, CE = torch.tensor(cs, device="cuda"), torch.tensor(ce, device="cuda")
    m.launch("ref_bind_interactions", 1, P(T["pos"]), P(T["vel"]), P(T["S"]), P(T["R"]), P(T["h"]), P(T["rho"]),
             P(T["p"]), P(T["T"]), P(T["hash"]), P(T["tool_particle"]), P(T["fc"]), P(CS), P(CE), C.c_int32(N),
             C.c_int32(g.num_cell), block=1)
    m.launch("do_interactions_monaghan", N, P(T["blanked"]), P(T["v_der"]), P(T["S_der"]), P(T["pos_t"]),
             P(T["vel_t"]), P(T["T_t"]), C.c_uint32(N))
    R = {k: v.cpu().numpy() for k, v in T.items()}
    check(G, R, ["v_der", "S_der", "pos_t", "vel_t", "T_t"], rtol=RTOL_SUMS)
    assert np.abs(R["S_der"]).max() > 0 and np.abs(R["T_t"]).max() > 0


def test_interactions_heat_pse(lib, base):
    """do_interactions_heat_pse with the reference's bindings: its tool-flag
    texture covers N ints of the N-double array, so particles from index N/2 on
    take the workpiece diffusivity; the product keeps that."""
    c, H = base
    k = c.constants
    saved = k.trml_tool_sph.alpha
    k.trml_tool_sph.alpha = 2.5 * k.trml_wp.alpha          # tool particles of both halves matter
    try:
        s = sorted_product(c, H, pse=True)
        H2, (cs, ce), g = s.download(), s.cells(), s.geometry()
        s.call("sph_interactions_heat_pse")
        G = s.download()
        s.close()
        m = interactions_module(c, g)
    finally:
        k.trml_tool_sph.alpha = saved
    N = len(H2["rho"])
    T = device(H2)
    CS, CE = torch.tensor(cs, device="cuda"), torch.tensor(ce, device="cuda")
    m.launch("ref_bind_interactions_pse", 1, P(T["pos"]), P(T["h"]), P(T["rho"]), P(T["T"]), P(T["hash"]),
             P(T["tool_particle"]), P(CS), P(CE), C.c_int32(N), C.c_int32(g.num_cell), block=1)
    m.launch("do_interactions_heat_pse", N, P(T["blanked"]), P(T["T_t"]), C.c_int32(N),
             C.c_double(c.constants.trml_wp.alpha), C.c_double(2.5 * c.constants.trml_wp.alpha))
    R = {k: v.cpu().numpy() for k, v in T.items()}
    check(G, R, ["T_t"], rtol=RTOL_SUMS)
    tool = H2["tool_particle"] == 1.0
    idx = np.arange(N)
    assert tool[idx < N // 2].any() and tool[idx >= N // 2].any()


# ---- cell list: grid_gpu_green::sort ----------------------------------------------------------
def test_sort_and_cell_tables(lib, base):
    """grid_gpu_green::sort (grid_gpu_green.cu:185-209) on a shuffled state:
    compute_hashes, thrust::sort_by_key of the int hashes (a stable radix sort;
    numpy's stable argsort stands in for it here), then the reference's own
    reorder_data_and_find_cell_start; permutation, sorted hashes, every
    reordered field and the cell tables bit for bit (cell_end where the cell is
    occupied: the reference leaves it stale elsewhere)."""
    grid, green = module("grid"), module("green")
    c, H = base
    rng = np.random.default_rng(23)
    perm = rng.permutation(len(H["rho"]))
    H = {k: np.ascontiguousarray(v[perm]) for k, v in H.items()}
    s = Solver(c)
    g = s.geometry()
    s.upload(H)
    s.call("sph_assign_hashes")
    s.call("sph_sort")
    G, (cs, ce) = s.download(), s.cells()
    s.close()
    N = len(H["rho"])
    T = device(H)
    grid.launch("compute_hashes", N, P(T["blanked"]), P(T["pos"]), P(T["hash"]), C.c_int32(N), C.c_double(g.dx),
                C.c_int32(g.ny), C.c_double(g.bbmin_x), C.c_double(g.bbmin_y))
    hashes = T["hash"].cpu().numpy()
    assert hashes.min() >= 0 and hashes.max() < g.num_cell, "the reorder kernel indexes its cell tables by hash"
    order = np.argsort(hashes, kind="stable").astype(np.int32)
    T["hash"] = torch.tensor(hashes[order], device="cuda")
    T["idx"] = torch.tensor(order, device="cuda")
    Bf = {k: torch.empty_like(T[k]) for k, _, _ in abi.PARTICLE_FIELDS if k in [f for f, _ in ref_gpu.DeviceBuffer._fields_]}
    buf = ref_gpu.DeviceBuffer(**{k: ref_gpu.ptr(v) for k, v in Bf.items()})
    CS = torch.full((g.num_cell,), -1, dtype=torch.int32, device="cuda")
    CE = torch.full((g.num_cell,), -7, dtype=torch.int32, device="cuda")
    green.launch("reorder_data_and_find_cell_start", N, particle_struct(T, N), buf, P(CS), P(CE), C.c_int32(N),
                 block=512, shared=(512 + 1) * 4)
    assert np.array_equal(G["idx"], order) and np.array_equal(G["hash"], hashes[order])
    for k, v in Bf.items():
        assert np.array_equal(G[k], v.cpu().numpy(), equal_nan=True), k
    rcs, rce = CS.cpu().numpy(), CE.cpu().numpy()
    assert np.array_equal(cs, rcs)
    occ = rcs != -1
    assert np.array_equal(ce[occ], rce[occ]) and occ.sum() > 100


# ---- the tool's FEM heat step and the tool / segment moves -----------------------------------------
def test_fem_heat_step(actions, cut):
    """reset_FEM_server, apply_robin_bdc over the cutting-edge colours,
    calculate_temp_rate and calculate_temp (FEM_thermal_gpu.cu:443-468,865-921)
    after a contact and friction pass has filled the segments' heat exchange:
    temperature rate and temperature of every node within 1e-13 relative,
    norm-wise.  The product adds the Robin terms to each node in one fixed
    order; the reference adds them colour by colour with FP64 atomics, so the
    diagonal and right-hand side can round differently."""
    c, s = cut
    fem_m = module("fem")
    fem_m.launch("ref_set_fem_constants", 1, c.constants.tool, block=1)
    s.call("sph_compute_contact_forces_fem")
    s.call("sph_material_fric_heat_gen_fem")
    seg, fem, ts = s.segments(), s.fem(), s.tool_state()
    assert np.abs(seg["heat_exchange"][:, 1]).sum() > 0, "segments in contact"
    s.call("sph_fem_reset_server")
    s.call("sph_fem_apply_robin")
    s.call("sph_fem_calculate_temp_rate")
    k_prod = s.fem()["k"]
    s.call("sph_fem_calculate_temp", C.c_double(c.dt))
    T_prod = s.fem()["T"]
    D = {k: torch.tensor(np.ascontiguousarray(v), device="cuda") for k, v in fem.items()}
    Sg = {k: torch.tensor(np.ascontiguousarray(v), device="cuda") for k, v in seg.items()}
    nn, nz, ns = len(fem["T"]), len(fem["K"]), ts.n_segments
    K_temp, f_temp, T_old = torch.empty_like(D["K"]), torch.empty_like(D["f"]), torch.empty_like(D["T"])
    fem_m.launch("do_copy_vector", nn, C.c_int32(nn), P(D["T"]), P(T_old))
    fem_m.launch("do_copy_vector", nn, C.c_int32(nn), P(D["f"]), P(f_temp))
    fem_m.launch("do_copy_vector", nz, C.c_int32(nz), P(D["K"]), P(K_temp))
    for colour in range(1, ts.n_cut_colors + 1):
        fem_m.launch("do_apply_heat_boundary_condition", ns, C.c_int32(colour), C.c_int32(ns), P(Sg["marks"]),
                     P(Sg["heat_exchange"]), P(Sg["fric_heat"]), P(Sg["left"]), P(Sg["right"]), P(D["row_ptr"]),
                     P(D["col_ind"]), P(K_temp), P(f_temp), block=16)
    fem_m.launch("do_calculate_temp_rate", nn, C.c_int32(nn), P(D["M_inv"]), P(K_temp), P(D["row_ptr"]),
                 P(D["col_ind"]), P(f_temp), P(D["k"]), P(D["T"]))
    e = rel_err(k_prod, D["k"].cpu().numpy())
    assert e <= 1e-13, f"FEM temperature rate: {e:.3e}"
    fem_m.launch("do_calculate_temp", nn, C.c_int32(nn), P(D["k"]), P(D["T"]), P(T_old), C.c_double(c.dt))
    e = rel_err(T_prod, D["T"].cpu().numpy())
    assert e <= 1e-13, f"FEM temperature: {e:.3e}"
    assert np.abs(k_prod).max() > 0


def test_tool_and_segment_move(cut):
    """tool_update_FEM_gpu and segments_update (tool_FEM.cu:109-139,1552-1582):
    node positions, segment end points (with the flank retreat) and the reset
    of the segments' heat exchange and friction heat, bit for bit."""
    c, s = cut
    tool_m = module("tool")
    seg, fem, ts = s.segments(), s.fem(), s.tool_state()
    dt = 7.0 * c.dt
    s.call("sph_segments_update", C.c_double(dt))
    s.call("sph_tool_update_fem", C.c_double(dt))
    seg2, pos2 = s.segments(), s.fem()["position"]
    tool_m.launch("ref_set_flank", 1, C.c_double(ts.flank_retreat), C.c_double(ts.flank_contact), block=1)
    Sg = {k: torch.tensor(np.ascontiguousarray(v), device="cuda") for k, v in seg.items()}
    X = torch.tensor(fem["position"], device="cuda")
    vel = ref_gpu.Vec2(*ts.vel)
    n, nn = ts.n_segments, len(fem["T"])
    tool_m.launch("do_segments_update", n, C.c_int32(n), P(Sg["left"]), P(Sg["right"]), P(Sg["heat_exchange"]),
                  P(Sg["fric_heat"]), vel, C.c_double(dt))
    tool_m.launch("do_tool_update_FEM_gpu", nn, C.c_int32(nn), P(X), vel, C.c_double(dt))
    for k in ("left", "right", "heat_exchange", "fric_heat"):
        assert np.array_equal(seg2[k], Sg[k].cpu().numpy()), k
    assert np.array_equal(pos2, X.cpu().numpy())
    assert np.any(pos2 != fem["position"])


# ---- the whole step ------------------------------------------------------------------------------------
@pytest.mark.parametrize("art_stress", [True, False], ids=["art_stress", "no_art_stress"])
def test_fused_step_against_reference_step(lib, art_stress):
    """Three fused, graph-replayed steps of the product against three
    leap_frog::step(particles, grid, tool_FEM) (leap_frog.cu:162-248) composed
    from the reference's own kernels (oracle/ref_gpu.RefFemStep), on the
    Ti6Al4V cut with the tool in contact: cell list, permutation, segment ids
    and blanking bit for bit; particle state, rates, FEM temperatures and the
    segments norm-wise within
      - 1e-12 without artificial stress: only the neighbour sums' 1e-16
        reassociations, carried through three steps;
      - 1e-8 with it: the stress angle's float trigonometry (CUDA's atan2f /
        cosf / sinf in the reference, double-evaluated and rounded once here)
        differs by float ULPs in R, and R enters the momentum sums."""
    c = setups.ti64_cut()
    if not art_stress:
        c.constants.corr.stresseps = 0.0
    tol = 1e-8 if art_stress else 1e-12
    s = Solver(c)
    s.move_tool(0.3 * c.info["dx"] / c.tool_speed)
    s.step(20)
    ref = ref_gpu.RefFemStep(c.constants, s.geometry(), c.dt, s.download(), s.fem(), s.segments(), s.tool_state())
    for _ in range(3):
        s.step()
        ref.step()
    G, Gf, Gs = s.download(), s.fem(), s.segments()
    s.close()
    R, Rf, Rs = ref.host()
    for f in ("hash", "idx", "on_seg", "blanked", "fixed", "tool_particle"):
        assert np.array_equal(G[f], R[f]), f"{f}: {np.count_nonzero(G[f] != R[f])} entries differ"
    act = R["blanked"] != 1.0
    for f in ("pos", "vel", "rho", "S", "T", "eps_pl", "eps_pl_dot", "p", "R", "fc", "ft", "n", "h"):
        e = rel_err(G[f], R[f])
        assert e <= (RTOL_FLOAT_TRIG if f == "R" else tol), f"{f}: {e:.3e}"
    for f in ("pos_t", "vel_t", "rho_t", "S_t", "T_t"):
        e = rel_err(G[f][act], R[f][act])
        assert e <= tol, f"{f}: {e:.3e}"
    for f in ("T", "k", "position"):
        e = rel_err(Gf[f], Rf[f])
        assert e <= tol, f"FEM {f}: {e:.3e}"
    for f in ("left", "right", "heat_exchange", "fric_heat"):
        e = rel_err(Gs[f], Rs[f]) if np.abs(Rs[f]).max() > 0 else float(np.abs(Gs[f]).max())
        assert e <= tol, f"segments {f}: {e:.3e}"
    assert np.count_nonzero(R["on_seg"] >= 0) >= 8


# ---- the rigid (SPH-particle) tool: tool_gpu.cu ------------------------------------------------------------
@pytest.fixture(scope="module")
def rigid(lib):
    """setup_ref_cut (benchmarks.cpp:247-530) at 30 rows, the tool 0.8 dx into the
    workpiece, after 5 fused steps (about 10 particles in contact); the solver
    stays open."""
    c = setups.ref_cut(ny=30, length=0.04, preload_dx=0.8)
    s = Solver(c)
    s.step(5)
    m = module("toolgpu")
    yield c, s, m
    s.close()


def set_rigid(m, c, s):
    raw, args = ref_gpu.rigid_tool_args(s.rigid_tool(), c.constants.tool.contact_alpha, c.constants.phys.mass)
    m.launch("ref_set_rigid_tool", 1, *args, block=1)
    return raw


def test_rigid_contact_forces(rigid):
    """compute_contact_forces (tool_gpu.cu:146-203): penalty normal force and
    LS-DYNA friction against the rigid outline and its fillet, within 1e-13
    relative, norm-wise: the product keeps the host geometry's uncontracted
    roundings (it is pinned bit for bit to tool.cpp), the reference's device
    code lets the compiler contract them into FMAs (1e-16 seen on other states)."""
    c, s, m = rigid
    raw = set_rigid(m, c, s)
    H = s.download()
    s.call("sph_compute_contact_forces")
    G = s.download()
    R = ref_run(H, lambda T, pg, N: m.launch("do_compute_contact_forces", N, pg, C.c_double(c.dt)))
    check(G, R, ["fc", "ft", "n"], rtol=1e-13)
    assert np.count_nonzero(np.abs(R["fc"]).sum(1) > 0) >= 5, "particles in contact"
    del raw


def test_rigid_friction_heat(actions, rigid):
    """material_fric_heat_gen (actions_gpu.cu:316-343, :956-965), bit for bit."""
    c, s, m = rigid
    k = c.constants
    actions.launch("ref_set_actions_constants", 1, k.phys, k.corr, k.joco, k.trml_wp, k.trml_tool, k.tool,
                   abi.WearConstants(0.0, 0.0, 0.0, 0.0), block=1)
    assert k.trml_wp.eta != 0.0
    H = s.download()
    s.call("sph_material_fric_heat_gen")
    G = s.download()
    vt = s.rigid_tool().vel
    R = ref_run(H, lambda T, pg, N: actions.launch("do_material_fric_heat_gen", N, P(T["vel"]), P(T["ft"]), P(T["n"]),
                                                    P(T["tool_particle"]), P(T["T"]), ref_gpu.Vec2(*vt),
                                                    C.c_double(c.dt), C.c_int32(N)))
    check(G, R, ["T"])
    assert np.count_nonzero(G["T"] != H["T"]) >= 3, "particles heated by friction"


def test_rigid_tool_particle_move(rigid):
    """update_tool_particles (tool_gpu.cu:205-216) inside tool_gpu_update_tool:
    the tool particles move by vel * dt, bit for bit."""
    c, s, m = rigid
    H = s.download()
    vt = s.rigid_tool().vel
    s.call("sph_rigid_tool_update")
    G = s.download()
    R = ref_run(H, lambda T, pg, N: m.launch("update_tool_particles", N, pg, ref_gpu.Vec2(*vt), C.c_double(c.dt)))
    check(G, R, ["pos"])
    tool = H["tool_particle"] == 1.0
    assert tool.sum() > 100 and np.all(np.any(G["pos"][tool] != H["pos"][tool], axis=1))


@pytest.mark.parametrize("art_stress,pse", [(True, False), (False, False), (True, True), (False, True)],
                         ids=["brookshaw", "brookshaw_no_art_stress", "pse", "pse_no_art_stress"])
def test_fused_rigid_step_against_reference_step(lib, oracle_lib, art_stress, pse):
    """Three fused product steps with the rigid tool against three
    leap_frog::step(particles, grid) (leap_frog.cu:99-160) composed from the
    reference's own kernels (oracle/ref_gpu.RefRigidStep; the outline moved by
    the oracle's restatement of tool::update_tool, pinned bit for bit to
    tool.cpp), in the Brookshaw and in the Thermal_Conduction_PSE build.  Cell
    list, permutation and blanking bit for bit; the state within 1e-12 without
    artificial stress and 1e-8 with it (R itself 1e-6: the float trigonometry
    of the stress angle)."""
    c = setups.ref_cut(ny=30, length=0.04, preload_dx=0.8)
    if not art_stress:
        c.constants.corr.stresseps = 0.0
    tol = 1e-8 if art_stress else 1e-12
    s = Solver(c)
    if pse:
        s.set_thermal_model(abi.SPH_THERMAL_PSE)
    s.step(5)
    ref = ref_gpu.RefRigidStep(c.constants, s.geometry(), c.dt, s.download(), s.rigid_tool(),
                               lambda t, dt: oracle_lib.orc_rigid_move(C.byref(t), dt), pse=pse)
    for _ in range(3):
        s.step()
        ref.step()
    G, tool = s.download(), s.rigid_tool()
    s.close()
    R = ref.host_particles()
    for f in ("hash", "idx", "blanked", "fixed", "tool_particle"):
        assert np.array_equal(G[f], R[f]), f"{f}: {np.count_nonzero(G[f] != R[f])} entries differ"
    act = R["blanked"] != 1.0
    for f in ("pos", "vel", "rho", "S", "T", "eps_pl", "eps_pl_dot", "p", "R", "fc", "ft", "n", "h"):
        e = rel_err(G[f], R[f])
        assert e <= (RTOL_FLOAT_TRIG if f == "R" else tol), f"{f}: {e:.3e}"
    for f in ("pos_t", "vel_t", "rho_t", "S_t", "T_t"):
        e = rel_err(G[f][act], R[f][act])
        assert e <= tol, f"{f}: {e:.3e}"
    for i in range(tool.n_seg):
        assert list(tool.left[i]) == list(ref.tool.left[i]) and list(tool.right[i]) == list(ref.tool.right[i])
    assert np.count_nonzero(np.abs(R["fc"]).sum(1) > 0) >= 5


# ---- wear by nodal shift (WEAR_NODE_SHIFT) ---------------------------------------------------------
def test_wear_adjustment(actions, cut):
    """wear_adjustment (actions_gpu.cu:1009-1020) as the reference runs it:
    mesh_retreat_wear and mesh_resume_wear over the element colours
    (do_mesh_adjustment_wear, one thread per block: it calls __syncthreads()
    after its early returns), the Usui rake/flank nodal shift
    (do_nodal_shift_wear_smooth_temp), do_segment_wear_update,
    do_correct_flank_contact and the lumped inverse mass, after a contact and
    friction pass has gathered the segment statistics.  Node positions (FP64
    atomics in the reference), lumped mass, stiffness, segments and the flank
    retreat within 1e-13 relative, norm-wise; the per-segment wear rate bit for
    bit."""
    c, s = cut
    fem_m, tool_m = module("fem"), module("tool")
    wc = abi.WearConstants(10.0, 300.0, 10.0, 300.0)
    fem_m.launch("ref_set_fem_constants", 1, c.constants.tool, block=1)
    s.set_wear(abi.SPH_WEAR_SHIFT, wc)
    s.call("sph_segments_wear_rate_reset")
    s.call("sph_compute_contact_forces_fem")
    s.call("sph_material_fric_heat_gen_fem")
    fem, seg, ts, w = s.fem(), s.segments(), s.tool_state(), s.wear_state()
    assert w["phys_para"][:, 0].sum() > 0, "segments with wear statistics"
    s.call("sph_wear_adjustment")
    Gf, Gs, Gt, Gw = s.fem(), s.segments(), s.tool_state(), s.wear_state()
    s.set_wear(abi.SPH_WEAR_OFF)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    n, ne, nn = ts.n_segments, len(w["elements"]), len(fem["T"])
    assert n <= 512, "do_correct_flank_contact reduces in one block of 512"
    X, K, Mi, Tn = dev(fem["position"]), dev(fem["K"]), dev(fem["M_inv"]), dev(fem["T"])
    M, layer, elem = dev(w["M"]), dev(w["layer"]), dev(w["elements"])
    rp, ci = dev(fem["row_ptr"]), dev(fem["col_ind"])
    Sg, sg = segment_struct(seg, n, wear=dict(wear_rate=np.zeros((n, 2)), wear_nodes=np.zeros(n),
                                              physical_para=w["phys_para"], sliding_force=w["sliding_force"]))
    mesh = ref_gpu.MeshGPU()
    mesh.position = ref_gpu.ptr(X)
    colours = int(w["elements"][:, 3].max())
    tool_m.launch("ref_set_wear", 1, C.c_double(ts.flank_retreat), C.c_double(ts.flank_contact), wc, block=1)

    def adjust(sign):
        for colour in range(1, colours + 1):
            fem_m.launch("do_mesh_adjustment_wear", ne, C.c_int32(colour), C.c_int32(ne), P(layer), P(X), P(elem),
                         P(rp), P(ci), C.c_int32(colours), P(M), P(K), C.c_int32(sign), block=1)

    adjust(-1)
    tool_m.launch("do_nodal_shift_wear_smooth_temp", n, C.c_int32(n), C.c_double(c.dt), sg, mesh, P(Tn))
    adjust(+1)
    tool_m.launch("do_segment_wear_update", n, C.c_int32(n), sg, mesh, block=512)
    tool_m.launch("do_correct_flank_contact", 512, C.c_int32(n), P(Sg["left"]), block=512)
    fem_m.launch("do_inverse_mass_matrix_lumped", nn, C.c_int32(nn), P(Mi), P(M))
    flank = torch.zeros(2, dtype=torch.float64, device="cuda")
    tool_m.launch("ref_get_flank", 1, P(flank), block=1)
    for name, a, b in (("position", Gf["position"], X), ("K", Gf["K"], K), ("M_inv", Gf["M_inv"], Mi),
                       ("M", Gw["M"], M), ("left", Gs["left"], Sg["left"]), ("right", Gs["right"], Sg["right"]),
                       ("normal", Gs["normal"], Sg["normal"])):
        e = rel_err(a, b.cpu().numpy())
        assert e <= 1e-13, f"{name}: {e:.3e}"
    assert np.array_equal(Gw["wear_nodes"], Sg["wear_nodes"].cpu().numpy())
    assert np.max(Gw["wear_nodes"]) > 0 and np.any(Gf["position"] != fem["position"])
    fr = flank.cpu().numpy()
    assert Gt.flank_retreat == pytest.approx(fr[0], rel=1e-13, abs=1e-18)


# ---- full size: the neighbour sums on the 4.19 M-particle micro workload -----------------------------------
def test_interactions_full_size(lib, capsys):
    """do_interactions_monaghan on the 2048 x 2048 micro workload (4,194,304
    particles, cells of h, the reference's geometry): the product's FP64 sums
    against the reference's own kernel at full size, within 1e-12 relative,
    norm-wise.  The device times of both launches are printed (CUDA events,
    after a warm-up launch); the reference's texture fetches are served by the
    stand-in's bounds-checked loads, so its time is indicative only."""
    c = setups.micro(n_side=2048, cell_factor=1, stencil=2)
    s = Solver(c)
    for name in ("sph_assign_hashes", "sph_sort", "sph_material_eos", "sph_corrector_artificial_stress"):
        s.call(name)
    H, (cs, ce), g = s.download(), s.cells(), s.geometry()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    s.call("sph_interactions_monaghan")
    s.sync()
    ev[0].record()
    s.call("sph_interactions_monaghan")
    s.sync()
    ev[1].record()
    G = s.download()
    s.close()
    m = interactions_module(c, g)
    N = len(H["rho"])
    T = device(H)
    CS, CE = torch.tensor(cs, device="cuda"), torch.tensor(ce, device="cuda")
    m.launch("ref_bind_interactions", 1, P(T["pos"]), P(T["vel"]), P(T["S"]), P(T["R"]), P(T["h"]), P(T["rho"]),
             P(T["p"]), P(T["T"]), P(T["hash"]), P(T["tool_particle"]), P(T["fc"]), P(CS), P(CE), C.c_int32(N),
             C.c_int32(g.num_cell), block=1)
    args = (P(T["blanked"]), P(T["v_der"]), P(T["S_der"]), P(T["pos_t"]), P(T["vel_t"]), P(T["T_t"]), C.c_uint32(N))
    m.launch("do_interactions_monaghan", N, *args)
    torch.cuda.synchronize()
    ev[2].record()
    m.launch("do_interactions_monaghan", N, *args)
    ev[3].record()
    torch.cuda.synchronize()
    R = {k: v.cpu().numpy() for k, v in T.items()}
    check(G, R, ["v_der", "S_der", "pos_t", "vel_t", "T_t"], rtol=RTOL_SUMS)
    with capsys.disabled():
        print(f"\n[micro 2048x2048 FP64 neighbour sums] product {ev[0].elapsed_time(ev[1]):.2f} ms "
              f"(staged call, records + sums), reference kernel {ev[2].elapsed_time(ev[3]):.2f} ms")


def test_plain_step_full_size(lib, capsys):
    """leap_frog::step(particles, grid) without a tool, composed from the
    reference's own kernels (oracle/ref_gpu.RefPlainStep), against the
    product's fused FP64 step on the 2048 x 2048 micro workload (4,194,304
    particles, the reference's cells of h), with the artificial-stress
    coefficient set to zero: the workload's random stresses make the
    artificial stress large, and the stress angle's float trigonometry (CUDA's
    atan2f / cosf / sinf in the reference) would reach the velocities at 2e-8
    and, through the float-rounded plastic increment, eps_pl at 2e-7 after two
    steps (the kernels still run in full; R comes out zero).  Two steps: cell
    list and permutation bit for bit, state and rates within 1e-11.  The device
    time of the reference's kernels
    per step (its sort's thrust::sort_by_key left out) and of the product's
    fused step are printed."""
    c = setups.micro(n_side=2048, cell_factor=1, stencil=2)
    c.constants.corr.stresseps = 0.0
    s = Solver(c)
    ref = ref_gpu.RefPlainStep(c.constants, s.geometry(), c.dt, s.download(), timed=True)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    s.step()
    s.sync()
    e[0].record()
    s.step()
    s.sync()
    e[1].record()
    e[1].synchronize()
    for _ in range(2):
        ref.step()
    G = s.download()
    s.close()
    R = ref.host_particles()
    for f in ("hash", "idx", "blanked"):
        assert np.array_equal(G[f], R[f]), f
    act = R["blanked"] != 1.0
    for f in ("pos", "vel", "rho", "S", "T", "eps_pl", "eps_pl_dot", "p"):
        e_ = rel_err(G[f], R[f])
        assert e_ <= 1e-11, f"{f}: {e_:.3e}"
    for f in ("pos_t", "vel_t", "rho_t", "S_t"):
        e_ = rel_err(G[f][act], R[f][act])
        assert e_ <= 1e-11, f"{f}: {e_:.3e}"
    with capsys.disabled():
        print(f"\n[micro 2048x2048 FP64 step] product fused step {e[0].elapsed_time(e[1]):.2f} ms, "
              f"reference kernels {ref.kernel_ms / 2:.2f} ms per step (sort excluded)")
