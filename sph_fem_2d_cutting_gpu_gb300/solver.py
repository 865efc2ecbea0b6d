"""Python host mirror of the reference's step interface over the C ABI.

``Solver`` owns one ``sph_ctx``.  Its methods carry the names of the calls
that ``leap_frog::step`` makes (leap_frog.cu:162-248) and raise ``SphError``
on any non-zero status, so host code (and the parity tests) read like the
reference's call sequence.  All compute runs in the sm_103a library; there is
no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .setups import Case

# the seven stages of sph_profile_steps, in order
PROFILE_STAGES = ("hash+histogram", "scan+scatter+rank", "reorder+predict+eos+artstress+records",
                  "fem half step+pse", "neighbour sums+epilogue", "fem update+wear+tool move",
                  "contact/bc/invalidate tail")


class SphError(RuntimeError):
    pass


class Solver:
    def __init__(self, case: Case, precision: int = abi.SPH_PREC_FP64, device: int = 0, place_tool: bool = True):
        self.lib = abi.load()
        self.case = case
        self.N = case.N
        self._keep = []
        host = abi.particles_struct(case.particles, case.N)
        tool, keep = case.tool_struct()
        self._keep += keep
        ctx = C.c_void_p()
        r = self.lib.sph_ctx_create(C.byref(case.constants), C.byref(case.grid), C.byref(host),
                                    C.byref(tool) if tool is not None else None, case.dt, precision, device,
                                    C.byref(ctx))
        self.ctx = ctx
        if r != abi.SPH_OK:
            msg = self.lib.sph_last_error(ctx).decode() if ctx.value else ""
            if ctx.value:
                self.lib.sph_ctx_destroy(ctx)
                self.ctx = C.c_void_p()
            raise SphError(f"sph_ctx_create failed ({r}): {msg}")
        self.has_tool = tool is not None
        if self.has_tool:
            if place_tool:
                self.place_tool()
            else:   # tool already placed (setups.placed): cutting velocity only
                self.set_vel(case.tool_speed, 0.0)
        if case.rigid is not None:
            self.set_rigid_tool(case.rigid.to_struct())

    # ---- plumbing -------------------------------------------------------------------------
    def _ck(self, r: int, what: str):
        if r != abi.SPH_OK:
            raise SphError(f"{what} failed ({r}): {self.lib.sph_last_error(self.ctx).decode()}")

    def call(self, name: str, *args):
        self._ck(getattr(self.lib, name)(self.ctx, *args), name)

    def close(self):
        if getattr(self, "ctx", None) is not None and self.ctx.value:
            self.lib.sph_ctx_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        self.call("sph_sync")

    def status(self, clear: bool = True) -> int:
        s = C.c_uint32()
        self._ck(self.lib.sph_status(self.ctx, C.byref(s), 1 if clear else 0), "sph_status")
        return s.value

    def geometry(self) -> abi.GeomConstants:
        g = abi.GeomConstants()
        self._ck(self.lib.sph_get_geometry(self.ctx, C.byref(g)), "sph_get_geometry")
        return g

    def launch_count(self) -> int:
        n = C.c_int64()
        self._ck(self.lib.sph_launch_count(self.ctx, C.byref(n)), "sph_launch_count")
        return n.value

    # ---- data movement ----------------------------------------------------------------------
    def download(self, fields=None) -> dict:
        out = abi.empty_particles(self.N)
        if fields is not None:
            out = {k: v for k, v in out.items() if k in fields}
        s = abi.particles_struct(out, self.N)
        self._ck(self.lib.sph_download_particles(self.ctx, C.byref(s)), "sph_download_particles")
        return out

    def upload(self, arrays: dict):
        arrays = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
        s = abi.particles_struct(arrays, self.N)
        self._ck(self.lib.sph_upload_particles(self.ctx, C.byref(s)), "sph_upload_particles")

    def eval_usui(self, K_usui: float, alpha: float, dt: float = 0.0, tool_vel=None):
        """tool_wear::eval_usui: (min, max, mean) Usui wear rate of the particles in
        contact; the accumulated wear (dt * mean per call) is kept on the object."""
        vt = np.array([self.case.tool_speed, 0.0] if tool_vel is None else tool_vel, np.float64)
        out = np.zeros(3)
        acc = np.array([getattr(self, "accum_wear", 0.0)])
        self._ck(self.lib.sph_eval_usui(self.ctx, K_usui, alpha, abi.ptr(vt), dt, abi.ptr(out), abi.ptr(acc)),
                 "sph_eval_usui")
        self.accum_wear = float(acc[0])
        return tuple(out)

    # ---- output in the reference's formats (vtk_writer.cu, mfree_gpu.cpp) ------------------------
    def write_vtk(self, path: str):
        """Particles as legacy-ASCII VTK (vtk_writer_write(particle_gpu*, step))."""
        self._ck(self.lib.sph_write_vtk_particles(self.ctx, str(path).encode()), "sph_write_vtk_particles")

    def write_vtk_tool(self, path: str, tl_ref=None):
        """The FEM tool as legacy-ASCII VTK (vtk_writer_write_FEM_tool); with tl_ref,
        moved back to where its top-left point was tl_ref (vtk_writer_write_tool_org)."""
        ref = None if tl_ref is None else np.ascontiguousarray(tl_ref, np.float64)
        self._ck(self.lib.sph_write_vtk_tool(self.ctx, str(path).encode(), abi.ptr(ref)), "sph_write_vtk_tool")

    def write_vtk_segments(self, path: str):
        """The contact segments with their wear statistics (vtk_writer_write_FEM_segments)."""
        self._ck(self.lib.sph_write_vtk_segments(self.ctx, str(path).encode()), "sph_write_vtk_segments")

    def append_force_log(self, path: str):
        """One line 'fx fy' of the cutting force (the reference's force log)."""
        self._ck(self.lib.sph_append_force_log(self.ctx, str(path).encode()), "sph_append_force_log")

    # ---- pipelined host I/O (sph_upload_particles_async / sph_download_particles_async) --------
    def upload_async(self, struct: abi.Particles):
        """Queue the upload of a particles struct of page-locked arrays (the arrays
        must stay alive and unchanged until ``sync``)."""
        self._ck(self.lib.sph_upload_particles_async(self.ctx, C.byref(struct)), "sph_upload_particles_async")

    def download_async(self, struct: abi.Particles):
        self._ck(self.lib.sph_download_particles_async(self.ctx, C.byref(struct)), "sph_download_particles_async")

    def cells(self):
        g = self.geometry()
        cs = np.zeros(g.num_cell, np.int32)
        ce = np.zeros(g.num_cell, np.int32)
        self._ck(self.lib.sph_download_cells(self.ctx, abi.ptr(cs), abi.ptr(ce)), "sph_download_cells")
        return cs, ce

    def tool_state(self) -> abi.ToolState:
        t = abi.ToolState()
        self._ck(self.lib.sph_get_tool_state(self.ctx, C.byref(t)), "sph_get_tool_state")
        return t

    def segments(self) -> dict:
        n = self.tool_state().n_segments
        out = dict(left=np.zeros((n, 2)), right=np.zeros((n, 2)), normal=np.zeros((n, 2)),
                   marks=np.zeros((n, 4), np.int32), heat_exchange=np.zeros((n, 2)), fric_heat=np.zeros(n))
        s = abi.Segments()
        s.n = n
        for k, v in out.items():
            setattr(s, k, abi.ptr(v))
        self._ck(self.lib.sph_download_segments(self.ctx, C.byref(s)), "sph_download_segments")
        return out

    def fem(self) -> dict:
        f = abi.Fem()
        self._ck(self.lib.sph_get_fem(self.ctx, C.byref(f)), "sph_get_fem")
        nn, nz = f.n_nodes, f.nnz
        out = dict(position=np.zeros((nn, 2)), row_ptr=np.zeros(nn + 1, np.int32), col_ind=np.zeros(nz, np.int32),
                   K=np.zeros(nz), M_inv=np.zeros(nn), f=np.zeros(nn), T=np.zeros(nn), k=np.zeros(nn))
        h = abi.Fem()
        h.n_nodes, h.nnz = nn, nz
        for k, v in out.items():
            setattr(h, k, abi.ptr(v))
        self._ck(self.lib.sph_download_fem(self.ctx, C.byref(h)), "sph_download_fem")
        return out

    def upload_fem_state(self, T=None, k=None):
        self._ck(self.lib.sph_upload_fem_state(self.ctx, abi.ptr(None if T is None else np.ascontiguousarray(T)),
                                               abi.ptr(None if k is None else np.ascontiguousarray(k))),
                 "sph_upload_fem_state")

    # ---- tool ---------------------------------------------------------------------------
    def set_vel(self, vx: float, vy: float):
        self._ck(self.lib.sph_set_tool_velocity(self.ctx, vx, vy), "sph_set_tool_velocity")

    def move_tool(self, dt: float):
        """segments_update + tool_update_FEM_gpu with the current velocity."""
        self._ck(self.lib.sph_segments_update(self.ctx, dt), "sph_segments_update")
        self._ck(self.lib.sph_tool_update_fem(self.ctx, dt), "sph_tool_update_fem")

    def place_tool(self):
        """Tool placement of benchmarks_NZ.cpp:247-267."""
        case = self.case
        dx = case.info["dx"]
        v = case.tool_speed
        ts = self.tool_state()
        distance = ts.right_point - case.info["lo_x"] + dx * 0.01
        time = distance / v
        self.set_vel(v, 0.0)
        self.move_tool(-time)
        ts = self.tool_state()
        current_feed = case.info["hi_y"] - ts.lowest_point
        dist_to_target = abs(current_feed - case.feed)
        correction_time = dist_to_target / v
        sign = 1.0 if current_feed > case.feed else -1.0
        self.set_vel(0.0, v)
        self.move_tool(correction_time * sign)
        self.set_vel(v, 0.0)

    # ---- the step and its stages -------------------------------------------------------------
    # ---- rigid (SPH-mode) tool and thermal model (leap_frog.cu:99-160) -------------------------
    def set_rigid_tool(self, tool: abi.RigidTool | None):
        self._ck(self.lib.sph_set_rigid_tool(self.ctx, C.byref(tool) if tool is not None else None),
                 "sph_set_rigid_tool")

    def rigid_tool(self) -> abi.RigidTool:
        t = abi.RigidTool()
        self._ck(self.lib.sph_get_rigid_tool(self.ctx, C.byref(t)), "sph_get_rigid_tool")
        return t

    # ---- tool wear by nodal shift (WEAR_NODE_SHIFT) ------------------------------------------
    def set_wear(self, mode: int, constants: abi.WearConstants | None = None):
        self._ck(self.lib.sph_set_wear(self.ctx, int(mode), C.byref(constants) if constants is not None else None),
                 "sph_set_wear")

    def wear_state(self) -> dict:
        seg_n = self.tool_state().n_segments
        f = abi.Fem()
        self._ck(self.lib.sph_get_fem(self.ctx, C.byref(f)), "sph_get_fem")
        nn = f.n_nodes
        ne = self.case.tool_mesh["elements"].shape[0] if self.case.tool_mesh is not None else 0
        out = dict(elements=np.zeros((ne, 4), np.int32), layer=np.zeros((ne, 2), np.int32), M=np.zeros(nn),
                   phys_para=np.zeros((seg_n, 4)), sliding_force=np.zeros(seg_n), wear_nodes=np.zeros(seg_n))
        w = abi.WearState()
        for k, v in out.items():
            setattr(w, k, abi.ptr(v))
        self._ck(self.lib.sph_download_wear(self.ctx, C.byref(w)), "sph_download_wear")
        return out

    def set_thermal_model(self, model: int):
        self._ck(self.lib.sph_set_thermal_model(self.ctx, int(model)), "sph_set_thermal_model")

    def step(self, n: int = 1):
        """leap_frog::step (fused kernels, CUDA-graph replay)."""
        if n == 1:
            self.call("sph_step")
        else:
            self._ck(self.lib.sph_run(self.ctx, n), "sph_run")

    def profile_steps(self, n: int = 1) -> dict:
        """n fused steps issued stage by stage with CUDA events between the
        stages (no graph); returns the summed device ms per stage."""
        ms = (C.c_float * 7)()
        ns = abi.I32()
        self._ck(self.lib.sph_profile_steps(self.ctx, n, ms, C.byref(ns)), "sph_profile_steps")
        return dict(zip(PROFILE_STAGES, list(ms)[:ns.value]))

    def step_staged(self):
        """leap_frog::step issued as the reference's separate calls."""
        self.call("sph_step_staged")

    def reduce_force(self):
        out = np.zeros(2)
        self._ck(self.lib.sph_reduce_force(self.ctx, abi.ptr(out)), "sph_reduce_force")
        return out

    def max_T(self) -> float:
        out = np.zeros(1)
        self._ck(self.lib.sph_reduce_max_T(self.ctx, abi.ptr(out)), "sph_reduce_max_T")
        return float(out[0])

    # ---- return-mapping log / statistics / learned warm start -------------------------------
    def jc_log_enable(self, capacity: int):
        self._ck(self.lib.sph_jc_log_enable(self.ctx, capacity), "sph_jc_log_enable")

    def jc_log_read(self, max_records: int | None = None):
        """(records [n, 8] float32, number of return mappings offered to the log)."""
        n = C.c_int64()
        self._ck(self.lib.sph_jc_log_read(self.ctx, None, 0, C.byref(n)), "sph_jc_log_read")
        m = n.value if max_records is None else min(n.value, max_records)
        rec = np.zeros((m, abi.JC_LOG_WIDTH), np.float32)
        if m:
            self._ck(self.lib.sph_jc_log_read(self.ctx, abi.ptr(rec), m, C.byref(n)), "sph_jc_log_read")
            held = min(n.value, m)
            rec = rec[:held]
        return rec, n.value

    def jc_stats(self, enable: bool = True, reset: bool = False):
        """(return mappings, secant iterations) counted since the last reset."""
        out = np.zeros(2, np.int64)
        self._ck(self.lib.sph_jc_stats(self.ctx, 1 if enable else 0, abi.ptr(out), 1 if reset else 0),
                 "sph_jc_stats")
        return int(out[0]), int(out[1])

    def attach_mlp(self, mlp, inference: int = abi.SPH_MLP_WARP):
        """Start the FP32K return mappings from the network's prediction (None
        detaches); `inference`: SPH_MLP_WARP (in the neighbour-sum epilogue) or
        SPH_MLP_TENSOR (a tensor-core tile kernel after it)."""
        self._ck(self.lib.sph_mlp_set_inference(self.ctx, inference), "sph_mlp_set_inference")
        self._ck(self.lib.sph_mlp_attach(self.ctx, mlp.h if mlp is not None else None), "sph_mlp_attach")

    def __getattr__(self, name):
        # stage calls by their reference names: update_geometry, assign_hashes, sort,
        # material_eos, interactions_monaghan, ... -> sph_<name>(ctx)
        if name.startswith("_"):
            raise AttributeError(name)
        full = "sph_" + name
        if full in abi.STAGE_FUNCTIONS:
            return lambda: self.call(full)
        raise AttributeError(name)

    def fem_calculate_temp(self, dt: float):
        self._ck(self.lib.sph_fem_calculate_temp(self.ctx, dt), "sph_fem_calculate_temp")


class Batch:
    """Many independent cases in one batched context (sph_batch_create).

    Every case keeps its own particles, FEM tool, tool velocity and time step;
    one fused step advances all of them.  Tools must be placed already
    (``setups.placed``).  Results come back per case in the case's own frame."""

    def __init__(self, cases: list[Case], precision: int = abi.SPH_PREC_FP32K, device: int = 0):
        self.lib = abi.load()
        self.cases = cases
        self.n_cases = len(cases)
        self._keep = []
        descs = (abi.CaseDesc * self.n_cases)()
        hosts = []
        for k, case in enumerate(cases):
            host = abi.particles_struct(case.particles, case.N)
            hosts.append(host)
            tool, keep = case.tool_struct()
            self._keep += keep + [tool]
            d = descs[k]
            d.host = C.pointer(host)
            d.tool = C.pointer(tool) if tool is not None else None
            d.dt = case.dt
            d.tool_vel[0], d.tool_vel[1] = case.tool_speed, 0.0
            d.bbmin[0], d.bbmin[1] = case.grid.bbmin[0], case.grid.bbmin[1]
            d.bbmax[0], d.bbmax[1] = case.grid.bbmax[0], case.grid.bbmax[1]
        self._keep += hosts
        c0 = cases[0]
        ctx = C.c_void_p()
        r = self.lib.sph_batch_create(C.byref(c0.constants), C.byref(c0.grid), self.n_cases, descs, precision,
                                      device, C.byref(ctx))
        self.ctx = ctx
        if r != abi.SPH_OK:
            msg = self.lib.sph_last_error(ctx).decode() if ctx.value else ""
            if ctx.value:
                self.lib.sph_ctx_destroy(ctx)
                self.ctx = C.c_void_p()
            raise SphError(f"sph_batch_create failed ({r}): {msg}")
        self.N = sum(c.N for c in cases)
        self.info = [self.case_info(k) for k in range(self.n_cases)]

    def _ck(self, r: int, what: str):
        if r != abi.SPH_OK:
            raise SphError(f"{what} failed ({r}): {self.lib.sph_last_error(self.ctx).decode()}")

    def close(self):
        if getattr(self, "ctx", None) is not None and self.ctx.value:
            self.lib.sph_ctx_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def case_info(self, k: int) -> dict:
        first, count, sf, sc, nf, nc = (C.c_int32() for _ in range(6))
        off = np.zeros(2)
        self._ck(self.lib.sph_batch_case_info(self.ctx, k, C.byref(first), C.byref(count), abi.ptr(off),
                                              C.byref(sf), C.byref(sc), C.byref(nf), C.byref(nc)),
                 "sph_batch_case_info")
        return dict(first=first.value, count=count.value, offset=off, seg_first=sf.value, seg_count=sc.value,
                    node_first=nf.value, node_count=nc.value)

    def step(self, n: int = 1):
        self._ck(self.lib.sph_run(self.ctx, n), "sph_run")

    def launch_count(self) -> int:
        n = C.c_int64()
        self._ck(self.lib.sph_launch_count(self.ctx, C.byref(n)), "sph_launch_count")
        return n.value

    def sync(self):
        self._ck(self.lib.sph_sync(self.ctx), "sph_sync")

    def status(self, clear: bool = True) -> int:
        s = C.c_uint32()
        self._ck(self.lib.sph_status(self.ctx, C.byref(s), 1 if clear else 0), "sph_status")
        return s.value

    def attach_mlp(self, mlp, inference: int = abi.SPH_MLP_WARP):
        """Start the FP32K return mappings of every case from the network's prediction (None detaches)."""
        self._ck(self.lib.sph_mlp_set_inference(self.ctx, inference), "sph_mlp_set_inference")
        self._ck(self.lib.sph_mlp_attach(self.ctx, mlp.h if mlp is not None else None), "sph_mlp_attach")

    def reduce(self) -> np.ndarray:
        """[n_cases, 3]: force x, force y (sum of fc + ft), max T of non-blanked particles."""
        out = np.zeros((self.n_cases, 3))
        self._ck(self.lib.sph_batch_reduce(self.ctx, abi.ptr(out)), "sph_batch_reduce")
        return out

    def download_cases(self, fields=None) -> list[dict]:
        """Per-case particle arrays in the current order, positions in the case frame."""
        out = abi.empty_particles(self.N)
        if fields is not None:
            out = {k: v for k, v in out.items() if k in fields}
        s = abi.particles_struct(out, self.N)
        self._ck(self.lib.sph_download_particles(self.ctx, C.byref(s)), "sph_download_particles")
        case_of = np.zeros(self.N, np.int32)
        self._ck(self.lib.sph_batch_case_of_particles(self.ctx, abi.ptr(case_of)), "sph_batch_case_of_particles")
        res = []
        for k in range(self.n_cases):
            sel = case_of == k
            d = {name: a[sel] for name, a in out.items()}
            if "pos" in d:
                d["pos"] = d["pos"] - self.info[k]["offset"]
            if "on_seg" in d:
                o = d["on_seg"]
                d["on_seg"] = np.where(o >= 0, o - self.info[k]["seg_first"], o).astype(np.int32)
            res.append(d)
        return res

    def fem_T(self) -> list[np.ndarray]:
        f = abi.Fem()
        self._ck(self.lib.sph_get_fem(self.ctx, C.byref(f)), "sph_get_fem")
        T = np.zeros(f.n_nodes)
        h = abi.Fem()
        h.n_nodes, h.nnz = f.n_nodes, f.nnz
        h.T = abi.ptr(T)
        self._ck(self.lib.sph_download_fem(self.ctx, C.byref(h)), "sph_download_fem")
        return [T[i["node_first"]:i["node_first"] + i["node_count"]] for i in self.info]
