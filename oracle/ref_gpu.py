"""Test infrastructure: the reference's own CUDA kernels, run on the GPU as a
parity pin.

``oracle/Makefile`` (target ``ref_gpu``) compiles the reference's
actions_gpu.cu, leap_frog.cu, grid.cu, grid_gpu_green.cu, interactions_gpu.cu,
FEM_thermal_gpu.cu, tool_FEM.cu and tool_gpu.cu, unmodified,
from the read-only reference tree into cubins for sm_103a under
``oracle/_ref/`` (with the stand-in GLM, gmsh and texture-reference headers of
``oracle/ref_shim``).  This module loads them
through the CUDA driver API (``libcuda``, via ctypes), finds each kernel by its
name and launches it on device buffers the caller owns (torch tensors).  It is
never part of the product; only the GPU tests import it.

Kernel arguments are ctypes values: ``ptr(tensor)`` for a device pointer,
``C.c_int32`` / ``C.c_double`` scalars, and the ctypes structures below,
which restate the reference's by-value parameter types (particle_gpu.h:22-79,
leap_frog.cu:13-23, segment_FEM_gpu.h:31-48, grid_gpu_green.h:33-63) field for
field.
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

REF_DIR = Path(__file__).resolve().parent / "_ref"
CUBINS = {"actions": "ref_gpu_actions.cubin", "leap_frog": "ref_gpu_leapfrog.cubin", "grid": "ref_gpu_grid.cubin",
          "interactions": "ref_gpu_interactions.cubin", "green": "ref_gpu_green.cubin", "fem": "ref_gpu_fem.cubin",
          "tool": "ref_gpu_tool.cubin", "toolgpu": "ref_gpu_toolgpu.cubin",
          "interactions_pse": "ref_gpu_interactions_pse.cubin"}
BLOCK_SIZE = 256   # the reference's BLOCK_SIZE (types.h)

P = C.c_uint64     # device pointer


class ParticleGPU(C.Structure):
    """particle_gpu (particle_gpu.h:22-79), USE_DOUBLE: the fields in declaration order."""
    _fields_ = [(n, P) for n in ("pos", "vel", "h", "rho", "p", "S", "R", "fc", "ft", "n", "fixed", "blanked",
                                 "tool_particle", "eps_pl", "eps_pl_dot", "T", "pos_t", "vel_t", "rho_t", "S_t",
                                 "T_t", "S_der", "v_der", "idx", "hash", "on_seg")] + [("N", C.c_uint32)]


class IniState(C.Structure):
    """inistate_struct (leap_frog.cu:13-23)."""
    _fields_ = [(n, P) for n in ("pos_init", "vel_init", "S_init", "rho_init", "T_init", "T_init_tool")]


class SegmentFEMGPU(C.Structure):
    """segment_FEM_gpu (segment_FEM_gpu.h:31-48) with WEAR_NODE_SHIFT: a vtable
    pointer first (the class has a virtual destructor), then the members."""
    _fields_ = [("vptr", P), ("segment_num", C.c_int32), ("pad", C.c_int32)] + \
        [(n, P) for n in ("left", "right", "n", "marks", "heat_exchange", "fric_heat", "wear_rate", "wear_nodes",
                          "physical_para", "sliding_force")]


class DeviceBuffer(C.Structure):
    """grid_gpu_green::device_buffer (grid_gpu_green.h:33-63) with USE_FEM_TOOL."""
    _fields_ = [(n, P) for n in ("pos", "vel", "fc", "ft", "h", "n", "rho", "S", "eps_pl", "eps_pl_dot", "T",
                                 "fixed", "blanked", "tool_particle", "pos_t", "vel_t", "rho_t", "S_t", "T_t",
                                 "on_seg")]


class MeshGPU(C.Structure):
    """mesh_GPU_m (mesh_structure_GPU.h:80-125) with WEAR_NODE_SHIFT, 160 bytes:
    the element arrays before offset 80 are left unset (the kernels that take
    it by value -- the wear updates, do_mesh_shift, the nodal interpolation --
    read the node arrays and the mapping copies only)."""
    _fields_ = [("head", C.c_uint8 * 80), ("position", P), ("cutting_edge_flag", P), ("fixed_edge_flag", P),
                ("T_nodes", P), ("f", P), ("k", P), ("position_mapping", P), ("node_num_mapping", P),
                ("csr_row_ptr", P), ("csr_col_ind", P)]


class GeomConstants(C.Structure):
    """geom_constants (constants_structs.h:70-76)."""
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("bbmin_x", C.c_double), ("bbmin_y", C.c_double),
                ("dx", C.c_double)]


class LineGPU(C.Structure):
    """line_gpu (tool_gpu.cuh:23-27)."""
    _fields_ = [("a", C.c_double), ("b", C.c_double), ("vertical", C.c_bool)]


class SegmentGPU(C.Structure):
    """segment_gpu (tool_gpu.cuh:29-34): double2 members are 16-byte aligned."""
    _fields_ = [("left", C.c_double * 2), ("right", C.c_double * 2), ("l", LineGPU), ("pad", C.c_double),
                ("n", C.c_double * 2)]


class CircleSegmentGPU(C.Structure):
    """circle_segment_gpu (tool_gpu.cuh:36-41)."""
    _fields_ = [("r", C.c_double), ("t1", C.c_double), ("t2", C.c_double), ("pad", C.c_double),
                ("p", C.c_double * 2)]


def rigid_tool_args(tool, contact_alpha: float, mass: float):
    """The setter arguments of ref_set_rigid_tool for a product sph_rigid_tool:
    (device buffer of segment_gpu, its torch tensor, count, fillet, has_fillet,
    mu, alpha, mass, velocity)."""
    import torch
    segs = (SegmentGPU * max(1, tool.n_seg))()
    for i in range(tool.n_seg):
        s = segs[i]
        s.left[:] = list(tool.left[i])
        s.right[:] = list(tool.right[i])
        s.n[:] = list(tool.n[i])
        s.l.a, s.l.b, s.l.vertical = tool.la[i], tool.lb[i], bool(tool.vertical[i])
    raw = torch.tensor(list(bytes(segs)), dtype=torch.uint8, device="cuda")
    fil = CircleSegmentGPU(tool.fillet_r, tool.fillet_t1, tool.fillet_t2, 0.0, (C.c_double * 2)(*tool.fillet_p))
    return raw, (ptr(raw), C.c_int32(tool.n_seg), fil, C.c_int32(tool.has_fillet), C.c_double(tool.mu),
                 C.c_double(contact_alpha), C.c_double(mass), Vec2(*tool.vel))


class Vec2(C.Structure):
    """glm::dvec2 / double2 passed by value."""
    _fields_ = [("x", C.c_double), ("y", C.c_double)]


def ptr(t) -> P:
    """Device pointer of a CUDA tensor (or 0 for None)."""
    return P(0 if t is None else t.data_ptr())


class _Driver:
    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        self.cu.cuFuncGetName.argtypes = [C.POINTER(C.c_char_p), C.c_void_p]

    def ck(self, r, what):
        if r != 0:
            name = C.c_char_p()
            self.cu.cuGetErrorName(r, C.byref(name))
            raise RuntimeError(f"{what}: {name.value.decode() if name.value else r}")


class RefModule:
    """One reference cubin in the current (primary) CUDA context."""

    def __init__(self, which: str):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")   # make the primary context current
        path = REF_DIR / CUBINS[which]
        if not path.exists():
            raise FileNotFoundError(path)
        self.d = _Driver()
        self.mod = C.c_void_p()
        self.d.ck(self.d.cu.cuModuleLoad(C.byref(self.mod), str(path).encode()), f"cuModuleLoad {path.name}")
        n = C.c_uint()
        self.d.ck(self.d.cu.cuModuleGetFunctionCount(C.byref(n), self.mod), "cuModuleGetFunctionCount")
        funcs = (C.c_void_p * n.value)()
        self.d.ck(self.d.cu.cuModuleEnumerateFunctions(funcs, n, self.mod), "cuModuleEnumerateFunctions")
        self.names = {}
        for f in funcs:
            s = C.c_char_p()
            self.d.ck(self.d.cu.cuFuncGetName(C.byref(s), C.c_void_p(f)), "cuFuncGetName")
            self.names[s.value.decode()] = C.c_void_p(f)

    def func(self, name: str):
        """The kernel named ``name``: an extern "C" name, or an Itanium-mangled
        one holding ``name`` with its length prefix."""
        pat = re.compile(r"(?<!\d)" + str(len(name)) + re.escape(name))
        hits = [k for k in self.names if k == name or pat.search(k)]
        if len(hits) != 1:
            raise KeyError(f"{name}: {hits or 'not found'} among {sorted(self.names)}")
        return self.names[hits[0]]

    def launch(self, name: str, n_threads: int, *args, block: int = BLOCK_SIZE, shared: int = 0):
        """Launches ``name`` over n_threads (the reference's 1-D grids, ``shared``
        bytes of dynamic shared memory) and waits."""
        f = self.func(name)
        grid = max(1, (n_threads + block - 1) // block)
        holders = list(args)
        argv = (C.c_void_p * max(1, len(holders)))(*[C.cast(C.pointer(a), C.c_void_p) for a in holders])
        self.d.ck(self.d.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, shared, None, argv, None), f"launch {name}")
        self.d.ck(self.d.cu.cuCtxSynchronize(), f"sync {name}")


# ---- the reference's steps, composed from its own kernels -------------------------------------------
SORTED = [n for n, _ in DeviceBuffer._fields_]          # the fields grid_gpu_green reorders


class _RefStep:
    """What leap_frog::step's two forms share: the sort, the predictor, EOS,
    artificial stress, the neighbour sums, the rates and the corrector, each a
    launch of the reference's own kernel in the reference's order.  Particle
    state lives in torch tensors ``P`` (particle_gpu fields)."""

    MODULES = ("actions", "leap_frog", "grid", "green", "interactions")

    def __init__(self, constants, geom, dt, particles: dict):
        import numpy as np
        import torch
        self.torch, self.np = torch, np
        self.c, self.g, self.dt = constants, geom, float(dt)
        self.m = {k: RefModule(k) for k in self.MODULES}
        k = constants
        self.m["actions"].launch("ref_set_actions_constants", 1, k.phys, k.corr, k.joco, k.trml_wp, k.trml_tool,
                                 k.tool, (C.c_double * 4)(), block=1)
        ge = GeomConstants(geom.nx, geom.ny, geom.bbmin_x, geom.bbmin_y, geom.dx)
        self.m["interactions"].launch("ref_set_interactions_constants", 1, k.phys, k.corr, ge, k.trml_wp,
                                      k.trml_tool_sph, k.tool, block=1)
        self.P = {f: torch.tensor(np.ascontiguousarray(v), device="cuda") for f, v in particles.items()}
        self.N = len(particles["rho"])
        self.cell_start = torch.full((geom.num_cell,), -1, dtype=torch.int32, device="cuda")
        self.cell_end = torch.zeros(geom.num_cell, dtype=torch.int32, device="cuda")
        ini = {"pos_init": (self.N, 2), "vel_init": (self.N, 2), "S_init": (self.N, 4), "rho_init": (self.N,),
               "T_init": (self.N,), "T_init_tool": (1,)}
        self.I = {f: torch.zeros(s, dtype=torch.float64, device="cuda") for f, s in ini.items()}

    def particles(self):
        st = ParticleGPU()
        for f, _ in ParticleGPU._fields_[:-1]:
            setattr(st, f, ptr(self.P[f]))
        st.N = self.N
        return st

    def inistate(self):
        return IniState(**{f: ptr(v) for f, v in self.I.items()})

    def sort(self):
        """grid_base::assign_hashes + grid_gpu_green::sort (grid.cu:25-42,80-86;
        grid_gpu_green.cu:185-209): compute_hashes, thrust::sort_by_key of the int
        hashes (a stable radix sort; a stable argsort here), the reorder kernel and
        the double-buffer swap."""
        torch, np, g, N = self.torch, self.np, self.g, self.N
        P = self.P
        self.m["grid"].launch("compute_hashes", N, ptr(P["blanked"]), ptr(P["pos"]), ptr(P["hash"]), C.c_int32(N),
                              C.c_double(g.dx), C.c_int32(g.ny), C.c_double(g.bbmin_x), C.c_double(g.bbmin_y))
        h = P["hash"].cpu().numpy()
        if h.min() < 0 or h.max() >= g.num_cell:
            raise ValueError("a particle hashed outside the grid: the reference's reorder kernel would index "
                             "its cell tables out of range")
        order = np.argsort(h, kind="stable").astype(np.int32)
        P["hash"] = torch.tensor(h[order], device="cuda")
        P["idx"] = torch.tensor(order, device="cuda")
        buf = {f: torch.empty_like(P[f]) for f in SORTED}
        self.cell_start.fill_(-1)
        self.m["green"].launch("reorder_data_and_find_cell_start", N, self.particles(),
                               DeviceBuffer(**{f: ptr(v) for f, v in buf.items()}), ptr(self.cell_start),
                               ptr(self.cell_end), C.c_int32(N), block=512, shared=(512 + 1) * 4)
        P.update(buf)

    def sums_and_rates(self):
        """material_eos .. contmech_advection (leap_frog.cu:119-134 / :191-206)."""
        a, it = self.m["actions"], self.m["interactions"]
        P, N = self.P, self.N
        a.launch("do_material_eos", N, ptr(P["rho"]), ptr(P["p"]), ptr(P["tool_particle"]), C.c_int32(N))
        a.launch("do_corrector_artificial_stress", N, ptr(P["rho"]), ptr(P["p"]), ptr(P["S"]),
                 ptr(P["tool_particle"]), ptr(P["R"]), C.c_int32(N))
        it.launch("ref_bind_interactions", 1, ptr(P["pos"]), ptr(P["vel"]), ptr(P["S"]), ptr(P["R"]), ptr(P["h"]),
                  ptr(P["rho"]), ptr(P["p"]), ptr(P["T"]), ptr(P["hash"]), ptr(P["tool_particle"]), ptr(P["fc"]),
                  ptr(self.cell_start), ptr(self.cell_end), C.c_int32(N), C.c_int32(self.g.num_cell), block=1)
        if not getattr(self, "pse", False):
            it.launch("do_interactions_monaghan", N, ptr(P["blanked"]), ptr(P["v_der"]), ptr(P["S_der"]),
                      ptr(P["pos_t"]), ptr(P["vel_t"]), ptr(P["T_t"]), C.c_uint32(N))
        else:   # PSE build: no Brookshaw term, then interactions_heat_pse (:434-463) when alpha_wp != 0
            it.launch("do_interactions_monaghan", N, ptr(P["blanked"]), ptr(P["v_der"]), ptr(P["S_der"]),
                      ptr(P["pos_t"]), ptr(P["vel_t"]), C.c_uint32(N))
            if self.c.trml_wp.alpha != 0.0:
                it.launch("ref_bind_interactions_pse", 1, ptr(P["pos"]), ptr(P["h"]), ptr(P["rho"]), ptr(P["T"]),
                          ptr(P["hash"]), ptr(P["tool_particle"]), ptr(self.cell_start), ptr(self.cell_end),
                          C.c_int32(N), C.c_int32(self.g.num_cell), block=1)
                it.launch("do_interactions_heat_pse", N, ptr(P["blanked"]), ptr(P["T_t"]), C.c_int32(N),
                          C.c_double(self.c.trml_wp.alpha), C.c_double(self.c.trml_tool_sph.alpha))
        a.launch("do_material_stress_rate_jaumann", N, ptr(P["v_der"]), ptr(P["S"]), ptr(P["tool_particle"]),
                 ptr(P["S_t"]), C.c_int32(N))
        a.launch("do_contmech_continuity", N, ptr(P["rho"]), ptr(P["v_der"]), ptr(P["tool_particle"]),
                 ptr(P["rho_t"]), C.c_int32(N))
        a.launch("do_contmech_momentum", N, ptr(P["S_der"]), ptr(P["fc"]), ptr(P["ft"]), ptr(P["tool_particle"]),
                 ptr(P["vel_t"]), C.c_int32(N))
        a.launch("do_contmech_advection", N, ptr(P["vel"]), ptr(P["tool_particle"]), ptr(P["pos_t"]), C.c_int32(N))

    def finish(self):
        """perform_boundary_conditions(_thermal) and debug_invalidate."""
        a, N = self.m["actions"], self.N
        a.launch("do_boundary_conditions", N, self.particles())
        if self.c.trml_tool.alpha != 0.0:
            a.launch("do_boundary_conditions_thermal", N, self.particles())
        a.launch("do_invalidate", N, self.particles(), C.c_int32(0))

    def host_particles(self):
        return {f: v.cpu().numpy() for f, v in self.P.items()}


class RefFemStep(_RefStep):
    """leap_frog::step(particles, grid, tool_FEM) (leap_frog.cu:162-248) run as
    the reference runs it: every kernel launch of the step, in its order, from
    the reference's own cubins, with the host side restated (the sort's
    argsort, the buffer swap, the tool's host reference points, the colour loop
    of apply_robin_bdc).  ``F`` holds the FEM system (position, row_ptr,
    col_ind, K, M_inv, f, T, k and the step's K_temp, f_temp, T_old), ``S`` the
    segments.  No wear (wear_pro off)."""

    MODULES = _RefStep.MODULES + ("fem", "tool")

    def __init__(self, constants, geom, dt, particles: dict, fem: dict, segments: dict, tool_state):
        super().__init__(constants, geom, dt, particles)
        torch, np = self.torch, self.np
        self.m["fem"].launch("ref_set_fem_constants", 1, constants.tool, block=1)
        dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
        self.F = {f: dev(v) for f, v in fem.items()}
        self.F["K_temp"], self.F["f_temp"], self.F["T_old"] = (torch.empty_like(self.F["K"]),
                                                               torch.empty_like(self.F["f"]),
                                                               torch.empty_like(self.F["T"]))
        n = len(segments["left"])
        self.S = {f: dev(v) for f, v in segments.items()}
        for f, shape in (("wear_rate", (n, 2)), ("wear_nodes", (n,)), ("physical_para", (n, 4)),
                         ("sliding_force", (n,))):
            self.S[f] = torch.zeros(shape, dtype=torch.float64, device="cuda")
        self.n_seg, self.n_colors = n, tool_state.n_cut_colors
        self.vel = (tool_state.vel[0], tool_state.vel[1])
        self.tl_ref = [tool_state.tl_point_ref[0], tool_state.tl_point_ref[1]]
        self.ref_dist = tool_state.ref_dist
        self.lowest = tool_state.lowest_point

    def segments(self):
        sg = SegmentFEMGPU()
        sg.segment_num = self.n_seg
        for f, src in (("left", "left"), ("right", "right"), ("n", "normal"), ("marks", "marks"),
                       ("heat_exchange", "heat_exchange"), ("fric_heat", "fric_heat"), ("wear_rate", "wear_rate"),
                       ("wear_nodes", "wear_nodes"), ("physical_para", "physical_para"),
                       ("sliding_force", "sliding_force")):
            setattr(sg, f, ptr(self.S[src]))
        return sg

    def step(self):
        a, lf, fm, tl = (self.m[k] for k in ("actions", "leap_frog", "fem", "tool"))
        P, F, S, N, dt, k = self.P, self.F, self.S, self.N, self.dt, self.c
        I = self.inistate()
        nn, nz = len(self.F["T"]), len(self.F["K"])
        self.sort()
        lf.launch("init", N, self.particles(), I)
        fm.launch("do_copy_vector", nn, C.c_int32(nn), ptr(F["T"]), ptr(F["T_old"]))           # reset_FEM_server
        fm.launch("do_copy_vector", nn, C.c_int32(nn), ptr(F["f"]), ptr(F["f_temp"]))
        fm.launch("do_copy_vector", nz, C.c_int32(nz), ptr(F["K"]), ptr(F["K_temp"]))
        lf.launch("predict", N, self.particles(), I, C.c_double(dt))
        fm.launch("do_calculate_temp", nn, C.c_int32(nn), ptr(F["k"]), ptr(F["T"]), ptr(F["T_old"]),
                  C.c_double(0.5 * dt))
        self.sums_and_rates()
        lf.launch("correct", N, self.particles(), I, C.c_double(dt))
        vel2 = Vec2(*self.vel)
        a.launch("do_material_fric_heat_gen_FEM_v21", N, self.particles(), self.segments(), vel2, ptr(F["T"]),
                 C.c_double(dt), C.c_int32(N))
        for colour in range(1, self.n_colors + 1):                                             # apply_robin_bdc
            fm.launch("do_apply_heat_boundary_condition", self.n_seg, C.c_int32(colour), C.c_int32(self.n_seg),
                      ptr(S["marks"]), ptr(S["heat_exchange"]), ptr(S["fric_heat"]), ptr(S["left"]),
                      ptr(S["right"]), ptr(F["row_ptr"]), ptr(F["col_ind"]), ptr(F["K_temp"]), ptr(F["f_temp"]),
                      block=16)
        fm.launch("do_calculate_temp_rate", nn, C.c_int32(nn), ptr(F["M_inv"]), ptr(F["K_temp"]), ptr(F["row_ptr"]),
                  ptr(F["col_ind"]), ptr(F["f_temp"]), ptr(F["k"]), ptr(F["T"]))
        fm.launch("do_calculate_temp", nn, C.c_int32(nn), ptr(F["k"]), ptr(F["T"]), ptr(F["T_old"]), C.c_double(dt))
        if k.plastic:
            a.launch("do_plasticity_johnson_cook", N, self.particles(), C.c_double(dt))
        tl.launch("ref_set_flank", 1, C.c_double(0.0), C.c_double(self.lowest), block=1)
        tl.launch("do_segments_update", self.n_seg, C.c_int32(self.n_seg), ptr(S["left"]), ptr(S["right"]),
                  ptr(S["heat_exchange"]), ptr(S["fric_heat"]), vel2, C.c_double(dt))
        tl.launch("do_tool_update_FEM_gpu", nn, C.c_int32(nn), ptr(F["position"]), vel2, C.c_double(dt))
        self.tl_ref = [self.tl_ref[0] + self.vel[0] * dt, self.tl_ref[1] + self.vel[1] * dt]   # tool_update_FEM_gpu
        self.lowest = self.lowest + self.vel[1] * dt
        # contact s1/s2 call __syncthreads() after early returns: one thread per block
        a.launch("do_compute_contact_forces_FEM_tool_v3_s1", N, C.c_int32(N), self.particles(), self.segments(),
                 Vec2(*self.tl_ref), C.c_double(self.ref_dist), vel2, C.c_double(dt), C.c_int32(self.n_seg), block=1)
        a.launch("do_compute_contact_forces_FEM_tool_v3_s2", N, C.c_int32(N), self.particles(), self.segments(),
                 ptr(F["T"]), C.c_double(dt), block=1)
        self.finish()

    def host(self):
        return (self.host_particles(), {f: v.cpu().numpy() for f, v in self.F.items()},
                {f: v.cpu().numpy() for f, v in self.S.items()})


class RefRigidStep(_RefStep):
    """leap_frog::step(particles, grid) with a rigid tool (leap_frog.cu:99-160),
    Brookshaw build, or with ``pse`` the Thermal_Conduction_PSE build: the
    reference's kernels in its order.  The tool outline
    moves on the host in the reference (tool::update_tool, tool.cpp:202-212);
    here ``move_tool(tool, dt)`` does it (the tests pass the CPU oracle's
    restatement, pinned bit for bit to tool.cpp), and the moved outline is
    installed as tool_gpu_update_tool does."""

    MODULES = _RefStep.MODULES + ("toolgpu",)

    def __init__(self, constants, geom, dt, particles: dict, tool, move_tool, pse: bool = False):
        self.pse = pse
        if pse:   # the Thermal_Conduction_PSE build of interactions_gpu.cu
            self.MODULES = self.MODULES + ("interactions_pse",)
        super().__init__(constants, geom, dt, particles)
        if pse:
            self.m["interactions"] = self.m.pop("interactions_pse")
            k = constants
            ge = GeomConstants(geom.nx, geom.ny, geom.bbmin_x, geom.bbmin_y, geom.dx)
            self.m["interactions"].launch("ref_set_interactions_constants", 1, k.phys, k.corr, ge, k.trml_wp,
                                          k.trml_tool_sph, k.tool, block=1)
        self.tool, self.move_tool = tool, move_tool
        self._install()

    def _install(self):
        self._raw, args = rigid_tool_args(self.tool, self.c.tool.contact_alpha, self.c.phys.mass)
        self.m["toolgpu"].launch("ref_set_rigid_tool", 1, *args, block=1)

    def step(self):
        a, lf, tg = self.m["actions"], self.m["leap_frog"], self.m["toolgpu"]
        P, N, dt, k = self.P, self.N, self.dt, self.c
        I = self.inistate()
        self.sort()
        lf.launch("init", N, self.particles(), I)
        lf.launch("predict", N, self.particles(), I, C.c_double(dt))
        self.sums_and_rates()
        lf.launch("correct", N, self.particles(), I, C.c_double(dt))
        vel = Vec2(*self.tool.vel)
        if k.trml_wp.eta != 0.0:                                                 # material_fric_heat_gen
            a.launch("do_material_fric_heat_gen", N, ptr(P["vel"]), ptr(P["ft"]), ptr(P["n"]),
                     ptr(P["tool_particle"]), ptr(P["T"]), vel, C.c_double(dt), C.c_int32(N))
        if k.plastic:
            a.launch("do_plasticity_johnson_cook", N, self.particles(), C.c_double(dt))
        self.move_tool(self.tool, dt)                                            # tool_gpu_update_tool
        self._install()
        tg.launch("update_tool_particles", N, self.particles(), vel, C.c_double(dt))
        tg.launch("do_compute_contact_forces", N, self.particles(), C.c_double(dt))
        self.finish()


class RefPlainStep(_RefStep):
    """leap_frog::step(particles, grid) without a tool (leap_frog.cu:99-160 with
    global_tool null): the reference's kernels in its order.  With ``timed``,
    ``kernel_ms`` accumulates the device time of the step's kernels (CUDA
    events on the default stream); the host-side argsort standing in for
    thrust::sort_by_key is left out of it."""

    def __init__(self, constants, geom, dt, particles: dict, timed: bool = False):
        super().__init__(constants, geom, dt, particles)
        self.timed, self.kernel_ms = timed, 0.0

    def _span(self):
        ev = self.torch.cuda.Event(enable_timing=True)
        ev.record()
        return ev

    def sort(self):
        if not self.timed:
            return super().sort()
        # time compute_hashes and the reorder kernel, not the host argsort between them
        torch, np, g, N, P = self.torch, self.np, self.g, self.N, self.P
        e0 = self._span()
        self.m["grid"].launch("compute_hashes", N, ptr(P["blanked"]), ptr(P["pos"]), ptr(P["hash"]), C.c_int32(N),
                              C.c_double(g.dx), C.c_int32(g.ny), C.c_double(g.bbmin_x), C.c_double(g.bbmin_y))
        e1 = self._span()
        e1.synchronize()
        self.kernel_ms += e0.elapsed_time(e1)
        h = P["hash"].cpu().numpy()
        if h.min() < 0 or h.max() >= g.num_cell:
            raise ValueError("a particle hashed outside the grid")
        order = np.argsort(h, kind="stable").astype(np.int32)
        P["hash"] = torch.tensor(h[order], device="cuda")
        P["idx"] = torch.tensor(order, device="cuda")
        buf = {f: torch.empty_like(P[f]) for f in SORTED}
        self.cell_start.fill_(-1)
        e0 = self._span()
        self.m["green"].launch("reorder_data_and_find_cell_start", N, self.particles(),
                               DeviceBuffer(**{f: ptr(v) for f, v in buf.items()}), ptr(self.cell_start),
                               ptr(self.cell_end), C.c_int32(N), block=512, shared=(512 + 1) * 4)
        e1 = self._span()
        e1.synchronize()
        self.kernel_ms += e0.elapsed_time(e1)
        P.update(buf)

    def step(self):
        a, lf = self.m["actions"], self.m["leap_frog"]
        N, dt = self.N, self.dt
        I = self.inistate()
        self.sort()
        e0 = self._span() if self.timed else None
        lf.launch("init", N, self.particles(), I)
        lf.launch("predict", N, self.particles(), I, C.c_double(dt))
        self.sums_and_rates()
        lf.launch("correct", N, self.particles(), I, C.c_double(dt))
        if self.c.plastic:
            a.launch("do_plasticity_johnson_cook", N, self.particles(), C.c_double(dt))
        self.finish()
        if self.timed:
            e1 = self._span()
            e1.synchronize()
            self.kernel_ms += e0.elapsed_time(e1)
