"""ctypes mirror of include/sphfem.h and the loader of the CUDA library.

The library is ``sph_fem_2d_cutting_gpu_gb300/lib/libsphfem.so`` built by
``build.py`` for sm_103a.  There is no fallback: if the library is missing or
does not load, ``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libsphfem.so"

SPH_OK, SPH_ERR_INVALID, SPH_ERR_CUDA, SPH_ERR_NO_DEVICE, SPH_ERR_ALLOC, SPH_ERR_STATE = range(6)
SPH_PREC_FP64, SPH_PREC_FP32K = 0, 1
SPH_THERMAL_BROOKSHAW, SPH_THERMAL_PSE = 0, 1
SPH_RIGID_MAX_SEG = 5
SPH_WEAR_OFF, SPH_WEAR_ACCUMULATE, SPH_WEAR_SHIFT = 0, 1, 2

STATUS_BITS = {
    "out_of_grid": 1 << 0,
    "secant_maxiter": 1 << 1,
    "nan_blanked": 1 << 2,
    "contact_noseg": 1 << 3,
    "contact_deep": 1 << 4,
    "melt_blanked": 1 << 5,
    "fric_nan": 1 << 6,
    "cell_overflow": 1 << 7,
    "mma_timeout": 1 << 8,
    "copy_timeout": 1 << 9,
    "grid_timeout": 1 << 10,
}

D = C.c_double
I32 = C.c_int32
PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int32)
PF = C.POINTER(C.c_float)


def _fields(names, t=D):
    return [(n, t) for n in names]


class PhysConstants(C.Structure):
    _fields_ = _fields(["E", "nu", "rho0", "K", "G", "mass", "mass_tool"])


class TrmlConstants(C.Structure):
    _fields_ = _fields(["cp", "tq", "k", "alpha", "T_init", "eta"])


class CorrConstants(C.Structure):
    _fields_ = _fields(["wdeltap", "stresseps", "xspheps", "alpha", "beta", "eta"])


class JocoConstants(C.Structure):
    _fields_ = _fields(["A", "B", "C", "n", "m", "Tmelt", "Tref", "eps_dot_ref", "tanh_a", "tanh_b", "tanh_c",
                        "tanh_d"])


class ToolConstants(C.Structure):
    _fields_ = _fields(["cp", "tq", "k", "eta", "rho", "T0", "h", "beta", "mu", "contact_alpha", "slave_mass", "hc"])


class Constants(C.Structure):
    _fields_ = [("phys", PhysConstants), ("corr", CorrConstants), ("joco", JocoConstants),
                ("trml_wp", TrmlConstants), ("trml_tool", TrmlConstants), ("trml_tool_sph", TrmlConstants),
                ("tool", ToolConstants), ("plastic", I32), ("pad0", I32)]


class GridParams(C.Structure):
    _fields_ = [("bbmin", D * 2), ("bbmax", D * 2), ("h", D), ("cell_factor", I32), ("stencil", I32)]


class GeomConstants(C.Structure):
    _fields_ = [("nx", I32), ("ny", I32), ("bbmin_x", D), ("bbmin_y", D), ("dx", D), ("num_cell", I32),
                ("stencil", I32)]


# (name, doubles-or-ints per particle, dtype) in sph_particles order
PARTICLE_FIELDS = [
    ("pos", 2, np.float64), ("vel", 2, np.float64), ("h", 1, np.float64), ("rho", 1, np.float64),
    ("p", 1, np.float64), ("S", 4, np.float64), ("R", 4, np.float64), ("fc", 2, np.float64),
    ("ft", 2, np.float64), ("n", 2, np.float64), ("fixed", 1, np.float64), ("blanked", 1, np.float64),
    ("tool_particle", 1, np.float64), ("eps_pl", 1, np.float64), ("eps_pl_dot", 1, np.float64),
    ("T", 1, np.float64), ("pos_t", 2, np.float64), ("vel_t", 2, np.float64), ("rho_t", 1, np.float64),
    ("S_t", 4, np.float64), ("T_t", 1, np.float64), ("S_der", 4, np.float64), ("v_der", 4, np.float64),
    ("idx", 1, np.int32), ("hash", 1, np.int32), ("on_seg", 1, np.int32),
]


class Particles(C.Structure):
    _fields_ = [("N", I32), ("pad0", I32)] + [(n, PI if dt == np.int32 else PD) for n, _, dt in PARTICLE_FIELDS]


class Segments(C.Structure):
    _fields_ = [("n", I32), ("pad0", I32), ("left", PD), ("right", PD), ("normal", PD), ("marks", PI),
                ("heat_exchange", PD), ("fric_heat", PD)]


class Fem(C.Structure):
    _fields_ = [("n_nodes", I32), ("nnz", I32), ("position", PD), ("row_ptr", PI), ("col_ind", PI), ("K", PD),
                ("M_inv", PD), ("f", PD), ("T", PD), ("k", PD)]


class ToolMesh(C.Structure):
    _fields_ = [("n_nodes", I32), ("n_elements", I32), ("nodes", PD), ("elements", PI), ("cutting_flags", PI),
                ("fixed_flags", PI), ("T_init", PD), ("tl", D * 2)]


class ToolState(C.Structure):
    _fields_ = [("vel", D * 2), ("tl_point_ref", D * 2), ("br_point", D * 2), ("ref_dist", D),
                ("lowest_point", D), ("right_point", D), ("n_segments", I32), ("n_cut_colors", I32),
                ("flank_retreat", D), ("flank_contact", D)]


class MlpNorm(C.Structure):
    _fields_ = [("x_mean", C.c_float * 4), ("x_std", C.c_float * 4), ("y_mean", C.c_float), ("y_std", C.c_float)]


MLP_NPARAMS = 8705
SPH_MLP_WARP, SPH_MLP_TENSOR = 0, 1   # sph_mlp_set_inference
JC_LOG_WIDTH = 8


class LaunchConfig(C.Structure):
    _fields_ = [("interact_variant", I32), ("step_form", I32)]


SPH_STEP_LAUNCHES, SPH_STEP_PERSISTENT = 0, 1
# sph_set_test_faults
SPH_TEST_SKIP_BULK_COPY, SPH_TEST_SKIP_MMA, SPH_TEST_SKIP_GRID_ARRIVAL = 1, 2, 4


class WearConstants(C.Structure):
    """sph_wear_constants (constants_structs.h:113-119): flank A, B; rake C, D."""
    _fields_ = _fields(["A", "B", "C", "D"])


class WearState(C.Structure):
    _fields_ = [("n_elements", I32), ("n_seg", I32), ("elements", PI), ("layer", PI), ("M", PD),
                ("phys_para", PD), ("sliding_force", PD), ("wear_nodes", PD)]


class RigidTool(C.Structure):
    """sph_rigid_tool: the segments of a rigid tool outline (tool_gpu.h) and its fillet."""
    _fields_ = [("n_seg", I32), ("has_fillet", I32),
                ("left", (D * 2) * SPH_RIGID_MAX_SEG), ("right", (D * 2) * SPH_RIGID_MAX_SEG),
                ("n", (D * 2) * SPH_RIGID_MAX_SEG), ("la", D * SPH_RIGID_MAX_SEG), ("lb", D * SPH_RIGID_MAX_SEG),
                ("vertical", I32 * SPH_RIGID_MAX_SEG), ("pad0", I32),
                ("fillet_p", D * 2), ("fillet_r", D), ("fillet_t1", D), ("fillet_t2", D),
                ("vel", D * 2), ("mu", D)]


class CaseDesc(C.Structure):
    _fields_ = [("host", C.POINTER(Particles)), ("tool", C.POINTER(ToolMesh)), ("dt", D), ("tool_vel", D * 2),
                ("bbmin", D * 2), ("bbmax", D * 2)]


def ptr(a: np.ndarray | None):
    """Pointer of a C-contiguous numpy array (or NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    t = {np.dtype(np.int32): PI, np.dtype(np.float32): PF, np.dtype(np.int64): C.POINTER(C.c_int64)}.get(a.dtype, PD)
    if t is PD:
        assert a.dtype == np.float64, f"unsupported dtype {a.dtype}"
    return a.ctypes.data_as(t)


def particles_struct(arrays: dict, N: int) -> Particles:
    """sph_particles pointing at numpy arrays (missing fields are NULL)."""
    s = Particles()
    s.N = N
    for name, w, dt in PARTICLE_FIELDS:
        a = arrays.get(name)
        if a is not None:
            assert a.dtype == dt and a.size == N * w, f"field {name}: dtype/size mismatch"
            setattr(s, name, ptr(a))
    return s


def empty_particles(N: int) -> dict:
    return {name: np.zeros(N * w if w > 1 else N, dtype=dt).reshape((N, w) if w > 1 else (N,))
            for name, w, dt in PARTICLE_FIELDS}


_lib = None


def load() -> C.CDLL:
    """Load the sm_103a library; raise if it is absent (there is no CPU path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"CUDA library not built: {LIB_PATH} (run sph_fem_2d_cutting_gpu_gb300.build.build())")
    lib = C.CDLL(str(LIB_PATH))
    P = C.c_void_p
    proto = {
        "sph_abi_version": ([], C.c_int),
        "sph_ctx_create": ([C.POINTER(Constants), C.POINTER(GridParams), C.POINTER(Particles), C.POINTER(ToolMesh),
                            D, I32, I32, C.POINTER(P)], C.c_int),
        "sph_ctx_destroy": ([P], C.c_int),
        "sph_last_error": ([P], C.c_char_p),
        "sph_set_dt": ([P, D], C.c_int),
        "sph_get_geometry": ([P, C.POINTER(GeomConstants)], C.c_int),
        "sph_set_constants": ([P, C.POINTER(Constants)], C.c_int),
        "sph_sync": ([P], C.c_int),
        "sph_status": ([P, C.POINTER(C.c_uint32), I32], C.c_int),
        "sph_get_stream": ([P, C.POINTER(P)], C.c_int),
        "sph_get_particles": ([P, C.POINTER(Particles)], C.c_int),
        "sph_upload_particles": ([P, C.POINTER(Particles)], C.c_int),
        "sph_download_particles": ([P, C.POINTER(Particles)], C.c_int),
        "sph_get_cells": ([P, C.POINTER(PI), C.POINTER(PI), C.POINTER(I32)], C.c_int),
        "sph_download_cells": ([P, PI, PI], C.c_int),
        "sph_set_tool_velocity": ([P, D, D], C.c_int),
        "sph_get_tool_state": ([P, C.POINTER(ToolState)], C.c_int),
        "sph_get_segments": ([P, C.POINTER(Segments)], C.c_int),
        "sph_download_segments": ([P, C.POINTER(Segments)], C.c_int),
        "sph_get_fem": ([P, C.POINTER(Fem)], C.c_int),
        "sph_download_fem": ([P, C.POINTER(Fem)], C.c_int),
        "sph_upload_fem_state": ([P, PD, PD], C.c_int),
        "sph_segments_update": ([P, D], C.c_int),
        "sph_tool_update_fem": ([P, D], C.c_int),
        "sph_fem_calculate_temp": ([P, D], C.c_int),
        "sph_run": ([P, I32], C.c_int),
        "sph_reduce_force": ([P, PD], C.c_int),
        "sph_reduce_max_T": ([P, PD], C.c_int),
        "sph_launch_count": ([P, C.POINTER(C.c_int64)], C.c_int),
        "sph_cells_build_noalloc": ([P, P, P, I32, C.POINTER(GeomConstants), P, P, P, P, P, C.c_char_p, I32],
                                    C.c_int),
        "sph_profile_steps":([P, I32, C.POINTER(C.c_float), C.POINTER(I32)], C.c_int),
        "sph_tool_build":([C.POINTER(ToolMesh), C.POINTER(ToolConstants), C.POINTER(P)], C.c_int),
        "sph_tool_host_info": ([P, C.POINTER(ToolState), C.POINTER(I32), C.POINTER(I32), C.POINTER(I32)], C.c_int),
        "sph_tool_host_export": ([P, C.POINTER(Segments), C.POINTER(Fem)], C.c_int),
        "sph_tool_host_destroy": ([P], C.c_int),
        "sph_batch_create": ([C.POINTER(Constants), C.POINTER(GridParams), I32, C.POINTER(CaseDesc), I32, I32,
                              C.POINTER(P)], C.c_int),
        "sph_batch_case_info": ([P, I32, PI, PI, PD, PI, PI, PI, PI], C.c_int),
        "sph_batch_n_cases": ([P, PI], C.c_int),
        "sph_batch_reduce": ([P, PD], C.c_int),
        "sph_batch_case_of_particles": ([P, PI], C.c_int),
        "sph_mlp_create": ([I32, C.c_uint64, C.POINTER(P)], C.c_int),
        "sph_mlp_destroy": ([P], C.c_int),
        "sph_mlp_last_error": ([P], C.c_char_p),
        "sph_mlp_get_params": ([P, PF, C.POINTER(MlpNorm)], C.c_int),
        "sph_mlp_set_params": ([P, PF, C.POINTER(MlpNorm)], C.c_int),
        "sph_mlp_fit_norm": ([P, PF, PF, C.c_int64], C.c_int),
        "sph_mlp_predict": ([P, PF, C.c_int64, PF], C.c_int),
        "sph_mlp_predict_warp": ([P, PF, C.c_int64, PF], C.c_int),
        "sph_mlp_gradients": ([P, PF, PF, C.c_int64, PF, PF], C.c_int),
        "sph_mlp_adam_step": ([P, PF, PF, C.c_int64, C.c_float, PF], C.c_int),
        "sph_mlp_train": ([P, PF, PF, C.c_int64, I32, I32, C.c_float, C.c_uint64, PF], C.c_int),
        "sph_jc_log_enable": ([P, C.c_int64], C.c_int),
        "sph_jc_log_read": ([P, PF, C.c_int64, C.POINTER(C.c_int64)], C.c_int),
        "sph_jc_stats": ([P, I32, C.POINTER(C.c_int64), I32], C.c_int),
        "sph_mlp_attach": ([P, P], C.c_int),
        "sph_mlp_set_inference": ([P, I32], C.c_int),
        "sph_launch_variants": ([PI, PI, PI, PI, PI], C.c_int),
        "sph_upload_particles_async": ([P, C.POINTER(Particles)], C.c_int),
        "sph_write_vtk_particles": ([P, C.c_char_p], C.c_int),
        "sph_write_vtk_tool": ([P, C.c_char_p, PD], C.c_int),
        "sph_write_vtk_segments": ([P, C.c_char_p], C.c_int),
        "sph_append_force_log": ([P, C.c_char_p], C.c_int),
        "sph_eval_usui": ([P, D, D, PD, D, PD, PD], C.c_int),
        "sph_download_particles_async": ([P, C.POINTER(Particles)], C.c_int),
        "sph_set_launch_config": ([P, C.POINTER(LaunchConfig)], C.c_int),
        "sph_set_test_faults": ([P, C.c_uint32, I32], C.c_int),
        "sph_vtk_write_particles_host": ([C.POINTER(Particles), C.c_char_p], C.c_int),
        "sph_vtk_write_tool_host": ([I32, PD, PD, I32, PI, PD, C.c_char_p], C.c_int),
        "sph_vtk_write_segments_host": ([I32, PD, PD, PD, PD, PD, PD, C.c_char_p], C.c_int),
        "sph_get_launch_config": ([P, C.POINTER(LaunchConfig)], C.c_int),
        "sph_set_rigid_tool": ([P, C.POINTER(RigidTool)], C.c_int),
        "sph_get_rigid_tool": ([P, C.POINTER(RigidTool)], C.c_int),
        "sph_set_thermal_model": ([P, I32], C.c_int),
        "sph_set_wear": ([P, I32, C.POINTER(WearConstants)], C.c_int),
        "sph_download_wear": ([P, C.POINTER(WearState)], C.c_int),
        "sph_upload_wear": ([P, C.POINTER(WearState)], C.c_int),
        "sph_tool_host_layers": ([P, PI], C.c_int),
        "sph_tool_host_elements": ([P, PI], C.c_int),
        "sph_remesh_low_level": ([P, I32], C.c_int),
    }
    for name in STAGE_FUNCTIONS:
        proto.setdefault(name, ([P], C.c_int))
    for name, (args, res) in proto.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def tool_model_host(case) -> dict:
    """Host-only tool set-up (no GPU): segments, FEM system and tool state, as
    sph_ctx_create would build them for this case."""
    lib = load()
    tool, keep = case.tool_struct()
    h = C.c_void_p()
    r = lib.sph_tool_build(C.byref(tool), C.byref(case.constants.tool), C.byref(h))
    try:
        if r != SPH_OK:
            raise RuntimeError(f"sph_tool_build failed ({r})")
        st = ToolState()
        nn, nz, ncol = I32(), I32(), I32()
        lib.sph_tool_host_info(h, C.byref(st), C.byref(nn), C.byref(nz), C.byref(ncol))
        n = st.n_segments
        seg = dict(left=np.zeros((n, 2)), right=np.zeros((n, 2)), normal=np.zeros((n, 2)),
                   marks=np.zeros((n, 4), np.int32), heat_exchange=np.zeros((n, 2)), fric_heat=np.zeros(n))
        fem = dict(position=np.zeros((nn.value, 2)), row_ptr=np.zeros(nn.value + 1, np.int32),
                   col_ind=np.zeros(nz.value, np.int32), K=np.zeros(nz.value), M_inv=np.zeros(nn.value),
                   f=np.zeros(nn.value), T=np.zeros(nn.value), k=np.zeros(nn.value))
        s = Segments()
        s.n = n
        for k, v in seg.items():
            setattr(s, k, ptr(v))
        f = Fem()
        f.n_nodes, f.nnz = nn.value, nz.value
        for k, v in fem.items():
            setattr(f, k, ptr(v))
        if lib.sph_tool_host_export(h, C.byref(s), C.byref(f)) != SPH_OK:
            raise RuntimeError("sph_tool_host_export failed")
        elements = np.zeros((len(case.tool_mesh["elements"]), 4), np.int32)
        if lib.sph_tool_host_elements(h, ptr(elements)) != SPH_OK:
            raise RuntimeError("sph_tool_host_elements failed")
        return dict(segments=seg, fem=fem, state=st, n_colors=ncol.value, n_cut_colors=st.n_cut_colors,
                    elements=elements)
    finally:
        if h.value:
            lib.sph_tool_host_destroy(h)
        del keep


# Entry points that take only the context (the stage calls of leap_frog::step).
STAGE_FUNCTIONS = [
    "sph_update_geometry", "sph_assign_hashes", "sph_sort", "sph_init", "sph_predict", "sph_correct",
    "sph_material_eos", "sph_corrector_artificial_stress", "sph_material_stress_rate_jaumann",
    "sph_contmech_continuity", "sph_contmech_momentum", "sph_contmech_advection", "sph_plasticity_johnson_cook",
    "sph_perform_boundary_conditions", "sph_perform_boundary_conditions_thermal", "sph_debug_invalidate",
    "sph_interactions_monaghan", "sph_material_fric_heat_gen_fem", "sph_compute_contact_forces_fem",
    "sph_fem_reset_server", "sph_fem_apply_robin", "sph_fem_calculate_temp_rate", "sph_step", "sph_step_staged",
    "sph_rigid_tool_update", "sph_compute_contact_forces", "sph_material_fric_heat_gen", "sph_interactions_heat_pse",
    "sph_segments_wear_rate_reset", "sph_wear_adjustment",
]
