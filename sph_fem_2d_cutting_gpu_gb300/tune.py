"""Autotuner of the fused step's launch shape and cell geometry.

Candidates: every compiled launch shape of the FP32K neighbour-sum kernel
(``sph_launch_variants``: threads per block, minimum resident blocks per SM,
neighbour records staged in shared memory), and the persistent one-launch
step (``SPH_STEP_PERSISTENT``), times every cell geometry in ``CELL_GEOMETRIES`` (cell edge = h x factor,
stencil half-width in cells; both cover the 2h kernel support).  Each
candidate is timed on the workload itself with CUDA events over whole fused
steps after a warm-up; the fastest is returned with the full table.  The
state a trial advances is thrown away (each geometry gets a fresh context),
so tuning does not change the run that follows.
"""
from __future__ import annotations

import copy
import ctypes as C
import time

from . import abi

CELL_GEOMETRIES = [(1, 2), (2, 1)]


def launch_variants():
    """[(threads per block, min blocks per SM, staged records, lanes per particle)] of the compiled shapes."""
    lib = abi.load()
    n = C.c_int32(0)
    lib.sph_launch_variants(C.byref(n), None, None, None, None)
    blk = (C.c_int32 * n.value)()
    mb = (C.c_int32 * n.value)()
    st = (C.c_int32 * n.value)()
    ln = (C.c_int32 * n.value)()
    cap = C.c_int32(n.value)
    lib.sph_launch_variants(C.byref(cap), blk, mb, st, ln)
    return [(blk[i], mb[i], st[i], ln[i]) for i in range(n.value)]


def shape_name(shape) -> str:
    """'128x6', '128x3s640' (staged records), '128x6l4' (lanes per particle)."""
    b, m, c, l = shape
    return f"{b}x{m}" + (f"s{c}" if c else "") + (f"l{l}" if l > 1 else "")


def get_config(obj) -> abi.LaunchConfig:
    cfg = abi.LaunchConfig()
    obj._ck(obj.lib.sph_get_launch_config(obj.ctx, C.byref(cfg)), "sph_get_launch_config")
    return cfg


def set_variant(obj, v: int):
    """Launch shape of the neighbour sums (the step form is kept)."""
    cfg = get_config(obj)
    cfg.interact_variant = v
    obj._ck(obj.lib.sph_set_launch_config(obj.ctx, C.byref(cfg)), "sph_set_launch_config")


def set_step_form(obj, form: int):
    """abi.SPH_STEP_LAUNCHES or abi.SPH_STEP_PERSISTENT (the launch shape is kept)."""
    cfg = get_config(obj)
    cfg.step_form = form
    obj._ck(obj.lib.sph_set_launch_config(obj.ctx, C.byref(cfg)), "sph_set_launch_config")


def apply(obj, best: dict):
    """Set the launch shape and step form of an autotune result."""
    set_variant(obj, best["variant"])
    set_step_form(obj, best.get("step_form", abi.SPH_STEP_LAUNCHES))


def _time_steps(obj, warmup: int, steps: int) -> float:
    import torch
    stream_ptr = C.c_void_p()
    obj.lib.sph_get_stream(obj.ctx, C.byref(stream_ptr))
    dev = torch.cuda.current_device()
    ext = torch.cuda.ExternalStream(stream_ptr.value, device=torch.device("cuda", dev))
    obj.step(warmup)
    obj.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    obj.step(steps)
    e1.record(ext)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def with_geometry(case, factor: int, stencil: int):
    c = copy.copy(case)
    g = abi.GridParams()
    C.pointer(g)[0] = case.grid
    g.cell_factor, g.stencil = factor, stencil
    c.grid = g
    return c


def autotune(make, cases, warmup: int = 3, steps: int = 10, geometries=None, variants=None, persistent=True):
    """Times every (geometry, launch variant) on contexts built by
    ``make(cases_with_geometry)`` (a Solver or Batch factory), and with
    `persistent` the persistent one-launch step on each geometry, and returns
    (best dict, table).  ``cases`` is a case or a list of cases."""
    geometries = geometries or CELL_GEOMETRIES
    all_v = launch_variants()
    variants = list(range(len(all_v))) if variants is None else variants
    table = []
    t0 = time.perf_counter()
    for factor, stencil in geometries:
        cs = [with_geometry(c, factor, stencil) for c in cases] if isinstance(cases, list) else \
            with_geometry(cases, factor, stencil)
        obj = make(cs)
        for v in variants:
            set_variant(obj, v)
            ms = _time_steps(obj, warmup, steps)
            table.append(dict(cell_factor=factor, stencil=stencil, variant=v, block=all_v[v][0],
                              min_blocks=all_v[v][1], staged=all_v[v][2], lanes=all_v[v][3],
                              step_form=abi.SPH_STEP_LAUNCHES, ms_per_step=ms))
        if persistent:   # one cooperative launch per step (128-particle blocks of the neighbour sums)
            set_variant(obj, 0)
            set_step_form(obj, abi.SPH_STEP_PERSISTENT)
            ms = _time_steps(obj, warmup, steps)
            table.append(dict(cell_factor=factor, stencil=stencil, variant=0, block=128, min_blocks=6, staged=0,
                              lanes=1, step_form=abi.SPH_STEP_PERSISTENT, ms_per_step=ms))
            set_step_form(obj, abi.SPH_STEP_LAUNCHES)
        obj.close()
    best = min(table, key=lambda r: r["ms_per_step"])
    return dict(best, tune_s=time.perf_counter() - t0), table
