"""ctypes wrapper of the CPU ORACLE (test infrastructure only).

Loads oracle/liboracle.so (built by oracle/Makefile) -- the plain C++
restatement of the reference's per-step functions.  Only the tests,
``__graft_entry__.smoke()`` and the CPU arms of ``bench.py`` use it, as the
checker and the CPU baseline; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from sph_fem_2d_cutting_gpu_gb300 import abi

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"

_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        build()
    lib = C.CDLL(str(LIB))
    P = C.POINTER(abi.Particles)
    K = C.POINTER(abi.Constants)
    G = C.POINTER(abi.GeomConstants)
    S = C.POINTER(abi.Segments)
    F = C.POINTER(abi.Fem)
    T = C.POINTER(abi.ToolState)
    R = C.POINTER(abi.RigidTool)
    Wp = C.POINTER(abi.WearState)
    Wc = C.POINTER(abi.WearConstants)
    PD, PI, D, I = abi.PD, abi.PI, C.c_double, C.c_int
    sig = {
        "orc_num_threads": ([], I),
        "orc_set_num_threads": ([I], None),
        "orc_cubic_spline": ([I, PD, PD, PD, PD], None),
        "orc_sigma_yield": ([C.POINTER(abi.JocoConstants), I, PD, PD, PD, PD], None),
        "orc_solve_secant": ([C.POINTER(abi.JocoConstants), I, PD, D, PD, PD, PD, D, D, PD, PI], None),
        "orc_set_geometry": ([C.POINTER(abi.GridParams), G], None),
        "orc_compute_hashes": ([P, G], None),
        "orc_sort_green": ([P, PI, PI, I], I),
        "orc_init": ([P, PD, PD, PD, PD, PD], None),
        "orc_predict": ([P, PD, PD, PD, PD, PD, D], None),
        "orc_correct": ([P, PD, PD, PD, PD, PD, D], None),
        "orc_material_eos": ([P, K], None),
        "orc_corrector_artificial_stress": ([P, K], None),
        "orc_interactions_monaghan": ([P, PI, PI, G, K], None),
        "orc_material_stress_rate_jaumann": ([P, K], None),
        "orc_contmech_continuity": ([P], None),
        "orc_contmech_momentum": ([P, K], None),
        "orc_contmech_advection": ([P], None),
        "orc_plasticity_johnson_cook": ([P, K, D, C.POINTER(C.c_int64)], I),
        "orc_boundary_conditions": ([P], None),
        "orc_boundary_conditions_thermal": ([P, K], None),
        "orc_invalidate": ([P], I),
        "orc_fric_heat_gen_fem": ([P, S, K, PD, D], I),
        "orc_contact_s1": ([P, S, K, PD, D, PD, D], C.c_uint32),
        "orc_contact_s2": ([P, S, K, PD, D], None),
        "orc_segments_update": ([S, PD, D], None),
        "orc_tool_update": ([F, T, D], None),
        "orc_fem_reset_server": ([F, PD, PD, PD], None),
        "orc_fem_apply_robin": ([F, S, K, I, PD, PD], None),
        "orc_fem_calculate_temp_rate": ([F, PD, PD], None),
        "orc_fem_calculate_temp": ([F, PD, D], None),
        "orc_step": ([P, PI, PI, G, K, D, S, F, T, I], C.c_uint32),
        "orc_interactions_monaghan_pse_build": ([P, PI, PI, G, K], None),
        "orc_rigid_move": ([R, D], None),
        "orc_rigid_move_particles": ([P, PD, D], None),
        "orc_contact_rigid": ([P, R, K, D], None),
        "orc_fric_heat_rigid": ([P, K, PD, D], None),
        "orc_interactions_heat_pse": ([P, PI, PI, G, K], None),
        "orc_step_rigid": ([P, PI, PI, G, K, D, R, I], C.c_uint32),
        "orc_wear_layers": ([I, PI, PI, I, PI], None),
        "orc_wear_reset": ([Wp], None),
        "orc_wear_adjustment": ([F, S, T, Wp, K, Wc, D], None),
        "orc_fric_heat_gen_fem_wear": ([P, S, K, PD, D, PD, Wp], I),
        "orc_segments_update_flank": ([S, PD, D, D], None),
        "orc_step_wear": ([P, PI, PI, G, K, D, S, F, T, I, Wp, Wc, I], C.c_uint32),
        "orc_mlp_eval": ([PD, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int64, I, PD,
                          PD, PD], I),
        "orc_mlp_adam": ([C.POINTER(C.c_float)] * 4 + [C.c_int64, C.c_float], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def geometry(grid: abi.GridParams) -> abi.GeomConstants:
    g = abi.GeomConstants()
    load().orc_set_geometry(C.byref(grid), C.byref(g))
    return g


def _struct_from(d: dict, cls, n_field, n):
    s = cls()
    setattr(s, n_field, n)
    for k, v in d.items():
        if hasattr(s, k) and isinstance(v, np.ndarray):
            setattr(s, k, abi.ptr(v))
    return s


class OracleSim:
    """Oracle state of one simulation: particle arrays, cell tables and, with a
    tool, the interface segments, FEM system and tool kinematics."""

    def __init__(self, constants: abi.Constants, grid: abi.GridParams, particles: dict, dt: float,
                 tool: dict | None = None, rigid: abi.RigidTool | None = None, pse: bool = False,
                 wear: dict | None = None):
        self.lib = load()
        self.C = constants
        self.grid = grid
        self.g = geometry(grid)
        self.dt = float(dt)
        self.N = len(particles["rho"])
        self.P = {k: np.ascontiguousarray(v).copy() for k, v in particles.items()}
        self.cell_start = np.full(self.g.num_cell, -1, np.int32)
        self.cell_end = np.zeros(self.g.num_cell, np.int32)
        self.tool = None
        if tool is not None:
            self.seg = {k: np.ascontiguousarray(v).copy() for k, v in tool["segments"].items()}
            self.fem = {k: np.ascontiguousarray(v).copy() for k, v in tool["fem"].items()}
            st = tool["state"]
            self.ts = abi.ToolState()
            C.memmove(C.byref(self.ts), C.byref(st), C.sizeof(abi.ToolState))
            self.n_colors = int(tool.get("n_cut_colors", 6))
            self.tool = True
        # rigid (SPH-mode) tool and the thermal solver of leap_frog::step(particles, grid)
        self.rigid = None
        if rigid is not None:
            self.rigid = abi.RigidTool()
            C.memmove(C.byref(self.rigid), C.byref(rigid), C.sizeof(abi.RigidTool))
        self.pse = bool(pse)
        # wear by nodal shift: dict(mode, constants, elements, layer, M) (statistics start at zero)
        self.wear_mode = 0
        if wear is not None:
            ns = len(self.seg["fric_heat"])
            self.wear = dict(elements=np.ascontiguousarray(wear["elements"], np.int32).copy(),
                             layer=np.ascontiguousarray(wear["layer"], np.int32).copy(),
                             M=np.ascontiguousarray(wear["M"], np.float64).copy(),
                             phys_para=np.zeros((ns, 4)), sliding_force=np.zeros(ns), wear_nodes=np.zeros(ns))
            self.wear_mode = int(wear["mode"])
            self.wear_c = abi.WearConstants()
            c = wear.get("constants")
            if c is not None:
                C.memmove(C.byref(self.wear_c), C.byref(c), C.sizeof(abi.WearConstants))

    def pstruct(self):
        return abi.particles_struct(self.P, self.N)

    def sstruct(self):
        return _struct_from(self.seg, abi.Segments, "n", len(self.seg["fric_heat"]))

    def wstruct(self):
        w = self.wear
        s = abi.WearState()
        s.n_elements = len(w["elements"])
        s.n_seg = len(w["sliding_force"])
        for k in ("elements", "layer", "M", "phys_para", "sliding_force", "wear_nodes"):
            setattr(s, k, abi.ptr(w[k]))
        return s

    def fstruct(self):
        f = _struct_from(self.fem, abi.Fem, "n_nodes", len(self.fem["T"]))
        f.nnz = len(self.fem["K"])
        return f

    def step(self) -> int:
        p = self.pstruct()
        if self.rigid is not None or self.pse:
            return self.lib.orc_step_rigid(C.byref(p), abi.ptr(self.cell_start), abi.ptr(self.cell_end),
                                           C.byref(self.g), C.byref(self.C), self.dt,
                                           C.byref(self.rigid) if self.rigid is not None else None, int(self.pse))
        if self.tool:
            s, f = self.sstruct(), self.fstruct()
            if self.wear_mode:
                w = self.wstruct()
                return self.lib.orc_step_wear(C.byref(p), abi.ptr(self.cell_start), abi.ptr(self.cell_end),
                                              C.byref(self.g), C.byref(self.C), self.dt, C.byref(s), C.byref(f),
                                              C.byref(self.ts), self.n_colors, C.byref(w), C.byref(self.wear_c),
                                              self.wear_mode)
            return self.lib.orc_step(C.byref(p), abi.ptr(self.cell_start), abi.ptr(self.cell_end), C.byref(self.g),
                                     C.byref(self.C), self.dt, C.byref(s), C.byref(f), C.byref(self.ts),
                                     self.n_colors)
        return self.lib.orc_step(C.byref(p), abi.ptr(self.cell_start), abi.ptr(self.cell_end), C.byref(self.g),
                                 C.byref(self.C), self.dt, None, None, None, 0)

    # single stages (same names as the reference calls)
    def assign_hashes(self):
        p = self.pstruct()
        self.lib.orc_compute_hashes(C.byref(p), C.byref(self.g))

    def sort(self) -> int:
        p = self.pstruct()
        return self.lib.orc_sort_green(C.byref(p), abi.ptr(self.cell_start), abi.ptr(self.cell_end), self.g.num_cell)

    def material_eos(self):
        p = self.pstruct()
        self.lib.orc_material_eos(C.byref(p), C.byref(self.C))

    def corrector_artificial_stress(self):
        p = self.pstruct()
        self.lib.orc_corrector_artificial_stress(C.byref(p), C.byref(self.C))

    def interactions_monaghan(self):
        p = self.pstruct()
        fn = self.lib.orc_interactions_monaghan_pse_build if self.pse else self.lib.orc_interactions_monaghan
        fn(C.byref(p), abi.ptr(self.cell_start), abi.ptr(self.cell_end), C.byref(self.g), C.byref(self.C))

    def interactions_heat_pse(self):
        p = self.pstruct()
        self.lib.orc_interactions_heat_pse(C.byref(p), abi.ptr(self.cell_start), abi.ptr(self.cell_end),
                                           C.byref(self.g), C.byref(self.C))

    # rigid tool (tool_gpu.cu, actions_gpu.cu:316-343)
    def rigid_tool_update(self):
        p = self.pstruct()
        self.lib.orc_rigid_move(C.byref(self.rigid), self.dt)
        vel = np.array(self.rigid.vel[:], dtype=np.float64)
        self.lib.orc_rigid_move_particles(C.byref(p), abi.ptr(vel), self.dt)

    def compute_contact_forces(self):
        p = self.pstruct()
        self.lib.orc_contact_rigid(C.byref(p), C.byref(self.rigid), C.byref(self.C), self.dt)

    def material_fric_heat_gen(self):
        p = self.pstruct()
        vel = np.array(self.rigid.vel[:], dtype=np.float64)
        self.lib.orc_fric_heat_rigid(C.byref(p), C.byref(self.C), abi.ptr(vel), self.dt)

    def material_stress_rate_jaumann(self):
        p = self.pstruct()
        self.lib.orc_material_stress_rate_jaumann(C.byref(p), C.byref(self.C))

    def contmech_continuity(self):
        p = self.pstruct()
        self.lib.orc_contmech_continuity(C.byref(p))

    def contmech_momentum(self):
        p = self.pstruct()
        self.lib.orc_contmech_momentum(C.byref(p), C.byref(self.C))

    def contmech_advection(self):
        p = self.pstruct()
        self.lib.orc_contmech_advection(C.byref(p))

    def plasticity_johnson_cook(self) -> tuple[int, int]:
        p = self.pstruct()
        its = C.c_int64()
        capped = self.lib.orc_plasticity_johnson_cook(C.byref(p), C.byref(self.C), self.dt, C.byref(its))
        return capped, its.value

    def perform_boundary_conditions(self):
        p = self.pstruct()
        self.lib.orc_boundary_conditions(C.byref(p))

    def perform_boundary_conditions_thermal(self):
        p = self.pstruct()
        self.lib.orc_boundary_conditions_thermal(C.byref(p), C.byref(self.C))

    def debug_invalidate(self) -> int:
        p = self.pstruct()
        return self.lib.orc_invalidate(C.byref(p))

    def compute_contact_forces_fem(self) -> int:
        p, s = self.pstruct(), self.sstruct()
        ev = self.lib.orc_contact_s1(C.byref(p), C.byref(s), C.byref(self.C), self.ts.tl_point_ref, self.ts.ref_dist,
                                     self.ts.vel, self.dt)
        self.lib.orc_contact_s2(C.byref(p), C.byref(s), C.byref(self.C), abi.ptr(self.fem["T"]), self.dt)
        return ev

    def material_fric_heat_gen_fem(self) -> int:
        p, s = self.pstruct(), self.sstruct()
        if self.wear_mode:
            w = self.wstruct()
            return self.lib.orc_fric_heat_gen_fem_wear(C.byref(p), C.byref(s), C.byref(self.C), self.ts.vel, self.dt,
                                                       abi.ptr(self.fem["T"]), C.byref(w))
        return self.lib.orc_fric_heat_gen_fem(C.byref(p), C.byref(s), C.byref(self.C), self.ts.vel, self.dt)

    def move_tool(self, dt: float):
        s, f = self.sstruct(), self.fstruct()
        self.lib.orc_segments_update_flank(C.byref(s), self.ts.vel, dt, self.ts.flank_retreat)
        self.lib.orc_tool_update(C.byref(f), C.byref(self.ts), dt)

    # wear by nodal shift (leap_frog.cu:183-186,224-229)
    def segments_wear_rate_reset(self):
        w = self.wstruct()
        self.lib.orc_wear_reset(C.byref(w))

    def wear_adjustment(self):
        f, s, w = self.fstruct(), self.sstruct(), self.wstruct()
        self.lib.orc_wear_adjustment(C.byref(f), C.byref(s), C.byref(self.ts), C.byref(w), C.byref(self.C),
                                     C.byref(self.wear_c), self.dt)

    # leap-frog snapshots (leap_frog.cu:25-96)
    def init(self):
        N = self.N
        self.snap = dict(pos=np.zeros((N, 2)), vel=np.zeros((N, 2)), S=np.zeros((N, 4)), rho=np.zeros(N),
                         T=np.zeros(N))
        p = self.pstruct()
        s = self.snap
        self.lib.orc_init(C.byref(p), abi.ptr(s["pos"]), abi.ptr(s["vel"]), abi.ptr(s["S"]), abi.ptr(s["rho"]),
                          abi.ptr(s["T"]))

    def _pc(self, fn):
        p = self.pstruct()
        s = self.snap
        fn(C.byref(p), abi.ptr(s["pos"]), abi.ptr(s["vel"]), abi.ptr(s["S"]), abi.ptr(s["rho"]), abi.ptr(s["T"]),
           self.dt)

    def predict(self):
        self._pc(self.lib.orc_predict)

    def correct(self):
        self._pc(self.lib.orc_correct)

    # FEM thermal calls (FEM_thermal_gpu.cu:865-921)
    def fem_reset_server(self):
        f = self.fstruct()
        self.fem_tmp = dict(T_old=np.zeros_like(self.fem["T"]), f_temp=np.zeros_like(self.fem["f"]),
                            K_temp=np.zeros_like(self.fem["K"]))
        t = self.fem_tmp
        self.lib.orc_fem_reset_server(C.byref(f), abi.ptr(t["T_old"]), abi.ptr(t["f_temp"]), abi.ptr(t["K_temp"]))

    def fem_calculate_temp(self, dt: float):
        f = self.fstruct()
        self.lib.orc_fem_calculate_temp(C.byref(f), abi.ptr(self.fem_tmp["T_old"]), dt)

    def fem_apply_robin(self):
        f, s = self.fstruct(), self.sstruct()
        t = self.fem_tmp
        self.lib.orc_fem_apply_robin(C.byref(f), C.byref(s), C.byref(self.C), self.n_colors, abi.ptr(t["K_temp"]),
                                     abi.ptr(t["f_temp"]))

    def fem_calculate_temp_rate(self):
        f = self.fstruct()
        t = self.fem_tmp
        self.lib.orc_fem_calculate_temp_rate(C.byref(f), abi.ptr(t["K_temp"]), abi.ptr(t["f_temp"]))


def set_threads(n: int):
    load().orc_set_num_threads(int(n))


def num_threads() -> int:
    return int(load().orc_num_threads())


# ---- learned warm start (mlp_oracle.cpp) --------------------------------------------------------
MLP_NPARAMS = 8705


def _fptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def norm_array(norm) -> np.ndarray:
    """sph_mlp_norm (or a 10-vector) as float32 [x_mean(4), x_std(4), y_mean, y_std]."""
    if isinstance(norm, np.ndarray):
        return np.ascontiguousarray(norm, np.float32)
    return np.array(list(norm.x_mean) + list(norm.x_std) + [norm.y_mean, norm.y_std], np.float32)


def mlp_eval(params, norm, x, t=None, bf16=True, grad=False):
    """Returns (y, grad or None, loss or None) of the MLP oracle."""
    lib = load()
    p = np.ascontiguousarray(params, np.float64)
    nm = norm_array(norm)
    x = np.ascontiguousarray(x, np.float32)
    n = x.shape[0]
    tt = None if t is None else np.ascontiguousarray(t, np.float32)
    y = np.zeros(n)
    g = np.zeros(MLP_NPARAMS) if grad else None
    loss = np.zeros(1) if tt is not None else None
    r = lib.orc_mlp_eval(abi.ptr(p), _fptr(nm), _fptr(x), _fptr(tt), n, 1 if bf16 else 0, abi.ptr(y),
                         abi.ptr(g) if g is not None else None, abi.ptr(loss) if loss is not None else None)
    assert r == 0
    return y, g, (None if loss is None else float(loss[0]))


def mlp_adam(params, m1, m2, grad, t, lr):
    """One FP32 Adam step in place (oracle of the GPU update)."""
    arrs = [np.ascontiguousarray(a, np.float32) for a in (params, m1, m2, grad)]
    load().orc_mlp_adam(*[_fptr(a) for a in arrs], int(t), float(lr))
    return arrs[0], arrs[1], arrs[2]


# ---- tool_wear::eval_usui (tool_wear.cu:14-54) ---------------------------------------------------
def eval_usui(P: dict, K_usui: float, alpha: float, tool_vel):
    """(min, max, mean) Usui wear rate over the particles in contact, restated with
    the reference's in-contact test (fc.x, fc.y, ft.x, fc.y) and its component-wise
    v - v*n."""
    fc, ft, v, n, h, T = P["fc"], P["ft"], P["vel"], P["n"], P["h"], P["T"]
    inc = (np.abs(fc[:, 0]) > 0) | (np.abs(fc[:, 1]) > 0) | (np.abs(ft[:, 0]) > 0) | (np.abs(fc[:, 1]) > 0)
    if not inc.any():
        return 0.0, 0.0, 0.0
    vv = v[inc] - np.asarray(tool_vel)[None, :]
    vr = vv - vv * n[inc]
    vmag = np.sqrt((vr ** 2).sum(1))
    fmag = np.sqrt((fc[inc] ** 2).sum(1))
    p = fmag / (2 * h[inc] * np.pi)
    w = K_usui * np.exp(alpha / T[inc]) * p * vmag
    return float(w.min()), float(w.max()), float(w.mean())
