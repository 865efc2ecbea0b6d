"""Test infrastructure: the reference's own CUDA kernels, run on the GPU as a
parity pin.

``oracle/Makefile`` (target ``ref_gpu``) compiles the reference's
actions_gpu.cu, leap_frog.cu, grid.cu, grid_gpu_green.cu, interactions_gpu.cu,
FEM_thermal_gpu.cu and tool_FEM.cu, unmodified,
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
          "tool": "ref_gpu_tool.cubin"}
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


class GeomConstants(C.Structure):
    """geom_constants (constants_structs.h:70-76)."""
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("bbmin_x", C.c_double), ("bbmin_y", C.c_double),
                ("dx", C.c_double)]


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
