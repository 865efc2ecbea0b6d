#!/usr/bin/env python
"""Benchmark of the SPH workpiece hot path on GB300 (one JSON line on rank 0).

Workload: the interaction micro-benchmark -- 4,194,304 particles on a
2048 x 2048 lattice (dx = 2.5 um, positions jittered +-0.05 dx, velocity
N(0, 1 m/s), symmetric Cauchy stress N(0, 200 MPa), density 7850 kg/m^3 x
(1 + U(-1e-3, 1e-3)), h = 1.7 dx, AISI 1045 Johnson-Cook), seeded synthetic
data.  One step = one full leap-frog step of leap_frog::step without a tool:
cell-list build (hash, stable sort, cell tables, reorder), predictor, EOS,
artificial stress, neighbour sums, stress rate / continuity / momentum /
advection, corrector, Johnson-Cook return mapping, boundary conditions and
invalidation.  Metric: particle-steps/s (higher is better).

Arms:
  default            the CUDA library (fused kernels, CUDA-graph replay); the
                     headline is the FP32-compensated form, the plain FP64
                     form is reported beside it.
  --impl reference   the reference's CPU implementation of the path (the CPU
                     oracle restatement, all host threads) on a bounded
                     sample of the same workload.
Multi-GPU (--gpus N under torchrun): replicas -- every rank advances its own
copy of the workload; no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s on 1 GB300, plain FP64 vs chosen form at <=1% force/temp error"
UNIT = "particle-steps/s"

# Algorithmic bytes per particle of the fused neighbour-sum kernel (one launch
# processes N particles): its own record, hash, the start-of-step state it
# corrects and the rates / state it writes; neighbour records are counted as
# cache hits (each is read from HBM once per launch, by its owner).
ALGO_BYTES = {
    "fp64": dict(read=128 + 4 + (16 + 16 + 32 + 8 + 8) + 32 + 8 + 16 + 16 + 8 + 8 + 8,
                 write=(16 + 16 + 32 + 8 + 8) + (16 + 16 + 32 + 8 + 8) + 8 + 8 + 4),
    # compact FP32 state: record 64, hash 4, S + S_t 32, fc + ft 16, pos 16 (FP64),
    # vel 8, rho 8 (FP64), T + T_t 8, eps_pl + eps_pl_dot 8, p 4; writes S_t,
    # rho_t, pos_t, vel_t (36) and the corrected pos, vel, rho, S, T, eps_pl,
    # eps_pl_dot (60)
    "fp32k": dict(read=64 + 4 + 32 + 16 + (16 + 8 + 8 + 8) + 8 + 4,
                  write=(16 + 4 + 8 + 8) + (16 + 8 + 8 + 16 + 4 + 4 + 4)),
}
# DRAM bytes (read + write) per particle of one full-size launch of the fused
# neighbour sums, from ncu on the 2048x2048 micro workload with 2h cells
# (dram__bytes_read.sum 723,139,584 + dram__bytes_write.sum 398,211,584 for
# 4,194,304 particles, k_interact32<fused, 128x6>; one-pass capture).
NCU_TRAFFIC_PER_PARTICLE = {"fp32k": (723_139_584 + 398_211_584) / 4_194_304}
# Floating-point work per particle of the fused neighbour sums, from ncu's SASS
# instruction counters (dadd + dmul + 2 dfma; fadd + fmul + 2 ffma) on the
# 512x512 micro workload with 2h cells (262,144 particles): k_interact64 executes
# 1,401,475,197 FP64 flops, k_interact32 (compact state, 128x6) 1,402,179,265 FP32 flops.
NCU_FLOPS_PER_PARTICLE = {"fp64": 1_401_475_197 / 262_144, "fp32k": 1_402_179_265 / 262_144}
# Nominal GB300 rates (no measured figure exists for these pipes): FP64 1.25 TFLOP/s;
# FP32 152 SMs x 128 lanes x 2 flops x 2.07 GHz = 80.5 TFLOP/s.
NOMINAL_TFLOPS = {"fp64": 1.25, "fp32k": 80.5}
# the seven stages of sph_profile_steps (the solver's PROFILE_STAGES)
STAGES = ["hash+histogram", "scan+scatter+rank", "reorder+predict+eos+artstress+records", "fem half step+pse",
          "neighbour sums+epilogue", "fem update+wear+tool move", "contact/bc/invalidate tail"]
# fields a caller moves per step in the end-to-end arm (the persistent state)
E2E_FIELDS = ["pos", "vel", "h", "rho", "S", "fc", "ft", "n", "fixed", "blanked", "tool_particle", "eps_pl",
              "eps_pl_dot", "T", "pos_t", "vel_t", "rho_t", "S_t", "T_t", "on_seg", "hash"]


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def rank_collectives(dist, device):
    """The two collectives of the replica runs: a barrier around the timed
    region and the max over ranks of a time (the slowest replica sets the
    whole job's time).  dist = None for one process."""
    import torch

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    return barrier, max_over_ranks


def replica_value(world: int, particles_per_rank: int, ms_per_step: float) -> float:
    """Whole-job particle-steps/s of `world` replicas of `particles_per_rank`
    particles each, from the slowest rank's time per step."""
    return world * particles_per_rank / (ms_per_step * 1e-3)


def cpu_sample(case, max_seconds=15.0, min_steps=1):
    """Time whole oracle steps of the workload (all host threads)."""
    from oracle.oracle import OracleSim, num_threads
    o = OracleSim(case.constants, case.grid, case.particles, case.dt)
    o.step()   # warm-up (first touch, thread pool)
    t0 = time.perf_counter()
    n = 0
    while True:
        o.step()
        n += 1
        el = time.perf_counter() - t0
        if n >= min_steps and el >= max_seconds:
            break
        if el + el / n > 2.5 * max_seconds:
            break
    return case.N * n / el, num_threads(), n, el


def run_reference(args):
    """--impl reference: the reference's CPU implementation (oracle restatement)."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from sph_fem_2d_cutting_gpu_gb300 import setups
    from oracle.oracle import OracleSim, num_threads
    case = setups.micro(n_side=args.n_side, seed=args.seed, cell_factor=args.cell_factor, stencil=args.stencil)
    # the whole workload (one oracle step of the 2048 x 2048 lattice takes about 0.9 s on
    # 16 Grace cores); --ref-side bounds it to a square sub-lattice on slower hosts
    side = min(args.n_side, args.ref_side) if args.ref_side > 0 else args.n_side
    sub = setups.micro(n_side=side, seed=args.seed, cell_factor=args.cell_factor, stencil=args.stencil)
    o = OracleSim(sub.constants, sub.grid, sub.particles, sub.dt)
    for _ in range(args.warmup):
        o.step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step()
    el = time.perf_counter() - t0
    v = sub.N * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"micro {case.info['n_side']}x{case.info['n_side']} lattice ({case.N} particles), "
                               f"dx=2.5um, h=1.7dx, cells {args.cell_factor}h / "
                               f"{2 * args.stencil + 1}x{2 * args.stencil + 1} stencil, AISI 1045 JC; full "
                               "leap-frog step without tool", "particles": case.N,
                   "sample_particles": sub.N},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": num_threads(), "kind": "port",
                         "sample": (f"{args.steps} whole steps of the full workload" if side == args.n_side else
                                    f"{args.steps} whole steps of a {side}x{side} sub-lattice of the workload")
                                   + " (reference CPU restatement, OpenMP)"},
        "same_config": side == args.n_side,
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def tune_fresh(make, warmup: int, steps: int):
    """Launch shape of the FP32K neighbour sums for a small workload: every shape
    timed on a fresh context from make() over the same steps (a cut advances its
    tool with the steps, so a reused context would time a later phase).
    Returns (best variant, {shape name: ms per step})."""
    from sph_fem_2d_cutting_gpu_gb300 import tune
    shapes = tune.launch_variants()
    table = []
    for v in range(len(shapes)):
        t = make()
        tune.set_variant(t, v)
        table.append(tune._time_steps(t, warmup, steps))
        t.close()
    best = min(range(len(table)), key=lambda v: table[v])
    return best, {tune.shape_name(sh): ms for sh, ms in zip(shapes, table)}


def stream_of(obj, local):
    """The library stream of a context, as a torch stream (for CUDA events on it)."""
    import ctypes as C

    import torch
    stream_ptr = C.c_void_p()
    obj.lib.sph_get_stream(obj.ctx, C.byref(stream_ptr))
    return torch.cuda.ExternalStream(stream_ptr.value, device=torch.device("cuda", local))


def time_batch(b, local, warmup, steps):
    """Device ms per step of `steps` fused steps of a batch (CUDA events on its stream)."""
    import torch
    ext = stream_of(b, local)
    b.step(warmup)
    b.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    b.step(steps)
    e1.record(ext)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps, ext


def run_sweep_full(args, local, cases, tuned, mlp):
    """The batched sweep at its stated length: all cases for `sweep_steps` steps
    in FP32K (force and peak temperature of every case every `sweep_every`
    steps, status after the run), three of them (smallest, median, largest) run
    alone in plain FP64 as the reference of their error curves; then the same
    batch timed in plain FP64 and in FP32K with the learned warm start."""
    import numpy as np
    import torch

    from sph_fem_2d_cutting_gpu_gb300 import abi, tune
    from sph_fem_2d_cutting_gpu_gb300.solver import Batch, Solver

    steps, every = args.sweep_steps, args.sweep_every
    b = Batch(cases, abi.SPH_PREC_FP32K, device=local)
    if tuned is not None:
        tune.apply(b, tuned)
    ext = stream_of(b, local)
    hist, ms = [], 0.0
    for _ in range(steps // every):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        b.step(every)
        e1.record(ext)
        e1.synchronize()
        ms += e0.elapsed_time(e1)
        hist.append(b.reduce())
    status = b.status()
    b.close()
    torch.cuda.empty_cache()
    H = np.stack(hist)                    # [checkpoints, cases, 3]
    order = sorted(range(len(cases)), key=lambda k: cases[k].N)
    picks = {"smallest": order[0], "median": order[len(order) // 2], "largest": order[-1]}
    per_case = {}
    for label, k in picks.items():
        s = Solver(cases[k], abi.SPH_PREC_FP64, device=local, place_tool=False)
        h64 = []
        for _ in range(steps // every):
            s.step(every)
            h64.append((*s.reduce_force(), s.max_T()))
        st64 = s.status()
        s.close()
        errs = curve_errors(h64, [tuple(H[c, k]) for c in range(len(h64))])
        per_case[label] = dict(case=k, particles=cases[k].N, fem_nodes=cases[k].info["nodes"],
                               speed_mpmin=cases[k].info.get("speed_mpmin"), status_fp64=st64,
                               peak_force_fp64=float(max(np.hypot(h[0], h[1]) for h in h64)),
                               T_rise_fp64=float(max(h[2] for h in h64) - 300.0), **errs,
                               curve_fp64=[list(map(float, h)) for h in h64],
                               curve_batched=[list(map(float, H[c, k])) for c in range(len(h64))])
        torch.cuda.empty_cache()
    n_total = sum(c.N for c in cases)
    out = {"steps": steps, "every": every, "status": status, "ms_per_step": ms / steps,
           "value": n_total / (ms / steps * 1e-3), "unit": UNIT,
           "peak_T_max": float(H[:, :, 2].max()), "peak_T_rise_max": float(H[:, :, 2].max() - 300.0),
           "reference_runs": per_case,
           "max_errors_vs_fp64": {"force_err_of_peak": max(v["force_err_of_peak"] for v in per_case.values()),
                                  "peak_T_err_of_rise": max(v["peak_T_err_of_rise"] for v in per_case.values())}}
    # the same batch in plain FP64, and in FP32K with the learned warm start
    forms = {}
    b = Batch(cases, abi.SPH_PREC_FP64, device=local)
    ms64, _ = time_batch(b, local, args.warmup, max(3, args.steps // 2))
    forms["fp64"] = {"ms_per_step": ms64, "value": n_total / (ms64 * 1e-3), "status": b.status()}
    b.close()
    torch.cuda.empty_cache()
    if mlp is not None:
        b = Batch(cases, abi.SPH_PREC_FP32K, device=local)
        if tuned is not None:
            tune.apply(b, tuned)
        msp, _ = time_batch(b, local, args.warmup, args.steps)
        b.attach_mlp(mlp)
        msm, _ = time_batch(b, local, args.warmup, args.steps)
        forms["fp32k"] = {"ms_per_step": msp, "value": n_total / (msp * 1e-3)}
        forms["fp32k_mlp"] = {"ms_per_step": msm, "value": n_total / (msm * 1e-3), "status": b.status()}
        forms["speedup_fp32k_mlp_vs_fp64"] = ms64 / msm
        forms["speedup_fp32k_vs_fp64"] = ms64 / msp
        b.close()
        torch.cuda.empty_cache()
    out["forms"] = forms
    return out


def run_batched(args, local, max_over_ranks, barrier, mlp=None):
    """The batched sweep: independent AISI 1045 cuts of uneven sizes advanced
    by one fused, graph-replayed step over all cases (FP32-compensated)."""
    import ctypes as C

    import torch

    from sph_fem_2d_cutting_gpu_gb300 import abi, setups
    from sph_fem_2d_cutting_gpu_gb300.solver import Batch

    from sph_fem_2d_cutting_gpu_gb300 import tune

    t0 = time.perf_counter()
    cases = setups.batched_sweep(n_cases=args.batched_cases, seed=args.seed)
    setup_s = time.perf_counter() - t0
    tuned, table = None, None
    if not args.no_tune:
        tuned, table = tune.autotune(lambda cs: Batch(cs, abi.SPH_PREC_FP32K, device=local), cases,
                                     warmup=args.warmup, steps=max(3, args.steps // 2))
        cases = [tune.with_geometry(c, tuned["cell_factor"], tuned["stencil"]) for c in cases]
    b = Batch(cases, abi.SPH_PREC_FP32K, device=local)
    if tuned is not None:
        tune.apply(b, tuned)
    stream_ptr = C.c_void_p()
    b.lib.sph_get_stream(b.ctx, C.byref(stream_ptr))
    ext = torch.cuda.ExternalStream(stream_ptr.value, device=torch.device("cuda", local))
    b.step(args.warmup)
    b.sync()
    barrier()
    n0 = C.c_int64()
    b.lib.sph_launch_count(b.ctx, C.byref(n0))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    b.step(args.steps)
    e1.record(ext)
    e1.synchronize()
    n1 = C.c_int64()
    b.lib.sph_launch_count(b.ctx, C.byref(n1))
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
    stage_ms = (C.c_float * 7)()
    ns = C.c_int32()
    b._ck(b.lib.sph_profile_steps(b.ctx, args.steps, stage_ms, C.byref(ns)), "sph_profile_steps")
    st = b.status()
    nodes = sum(i["node_count"] for i in b.info)
    out = {"value": b.N / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "cases": b.n_cases, "particles": b.N,
           "particles_min": min(c.N for c in cases), "particles_max": max(c.N for c in cases),
           "fem_nodes": nodes, "launches_per_step": (n1.value - n0.value) / args.steps,
           "stage_ms": dict(zip(STAGES, [v / args.steps for v in stage_ms])), "status": st,
           "setup_s": setup_s, "dtype": "f32k",
           "autotune": None if tuned is None else {"best": tuned, "table": table},
           "workload": f"{b.n_cases} AISI 1045 cuts, counts log-uniform 20k-300k (height 0.5 mm, dx 2.5 um), "
                       "speed U(30,300) m/min, uncut chip U(20,150) um, rake U(-10,15) deg, own FEM tool each; "
                       "one fused step over all cases, CUDA-graph replay"}
    b.close()
    torch.cuda.empty_cache()
    if args.sweep_steps > 0:
        out["sweep_run"] = run_sweep_full(args, local, cases, tuned, mlp)
    return out


def run_small_cut(args, local):
    """The small plain-method case (Ti6Al4V cut, 200 x 60 = 12,000 particles, FEM
    tool of about 2,000 nodes, 70 m/min, 80 um): per-step time of the fused,
    graph-replayed step in FP64 and FP32K, and the CPU oracle's step beside it.
    At this size the step is latency- and launch-bound, not HBM-bound."""
    import ctypes as C

    import torch

    from sph_fem_2d_cutting_gpu_gb300 import abi, setups, tune
    from sph_fem_2d_cutting_gpu_gb300.solver import Solver
    from oracle.oracle import OracleSim, num_threads

    case = setups.ti64_cut()
    row = {"particles": case.N, "fem_nodes": case.info["nodes"]}
    for name, prec in (("fp64", abi.SPH_PREC_FP64), ("fp32k", abi.SPH_PREC_FP32K)):
        s = Solver(case, prec, device=local)
        sp = C.c_void_p()
        s.lib.sph_get_stream(s.ctx, C.byref(sp))
        ext = torch.cuda.ExternalStream(sp.value, device=torch.device("cuda", local))
        if prec == abi.SPH_PREC_FP32K and not args.no_tune:   # launch shape on this workload
            best_v, table = tune_fresh(lambda: Solver(case, prec, device=local), args.warmup, max(args.steps, 50))
            tune.set_variant(s, best_v)
            row["launch_tuning"] = {"chosen": list(table)[best_v], "ms_per_step": table}
        s.step(args.warmup)
        s.sync()
        n0 = s.launch_count()
        steps = max(args.steps, 50)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        s.step(steps)
        e1.record(ext)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        row[name] = {"ms_per_step": ms, "value": case.N / (ms * 1e-3),
                     "launches_per_step": (s.launch_count() - n0) / steps, "status": s.status()}
        # the same step with tool wear by nodal shift (WEAR_NODE_SHIFT, after wear_pro)
        s.set_wear(abi.SPH_WEAR_SHIFT, abi.WearConstants(10.0, 300.0, 10.0, 300.0))
        s.step(args.warmup)
        s.sync()
        n0 = s.launch_count()
        e0.record(ext)
        s.step(steps)
        e1.record(ext)
        e1.synchronize()
        msw = e0.elapsed_time(e1) / steps
        row[name + "_wear"] = {"ms_per_step": msw, "value": case.N / (msw * 1e-3),
                               "launches_per_step": (s.launch_count() - n0) / steps, "status": s.status()}
        s.set_wear(abi.SPH_WEAR_OFF, None)
        if prec == abi.SPH_PREC_FP32K:   # the same steps as one persistent launch each (fresh context)
            t = Solver(case, prec, device=local)
            tune.set_step_form(t, abi.SPH_STEP_PERSISTENT)
            t.step(args.warmup)
            t.sync()
            n0 = t.launch_count()
            text = stream_of(t, local)
            e0.record(text)
            t.step(steps)
            e1.record(text)
            e1.synchronize()
            msp = e0.elapsed_time(e1) / steps
            row["fp32k_persistent"] = {"ms_per_step": msp, "value": case.N / (msp * 1e-3),
                                       "launches_per_step": (t.launch_count() - n0) / steps, "status": t.status()}
            t.close()
        if prec == abi.SPH_PREC_FP64 and not args.no_cpu:
            P = s.download()
            ts = s.tool_state()
            tool = dict(segments=s.segments(), fem=s.fem(), state=ts, n_cut_colors=ts.n_cut_colors)
            o = OracleSim(case.constants, case.grid, P, case.dt, tool=tool)
            o.step()
            t0, n = time.perf_counter(), 0
            while n < 1 or (time.perf_counter() - t0 < 2.0 and n < 500):
                o.step()
                n += 1
            el = time.perf_counter() - t0
            row["cpu_oracle"] = {"value": case.N * n / el, "ms_per_step": 1e3 * el / n, "steps": n,
                                 "cores": num_threads()}
        s.close()
    if "cpu_oracle" in row:
        row["fp64_vs_cpu"] = row["cpu_oracle"]["ms_per_step"] / row["fp64"]["ms_per_step"]
    row["workload"] = ("Ti6Al4V orthogonal cut, 200 x 60 particles (dx 5 um, h 1.7 dx), FEM tool of about 2,000 "
                       "nodes (rake 0, clearance 7 deg, r 5 um), 70 m/min, uncut chip 80 um")
    return row



def run_tiny_sweep(args, local):
    """Many tiny cases in one batched context (16 AISI 1045 cuts of 3,000 to
    12,000 particles, each with its own FEM tool): the fused FP32K step as its
    chain of graph-replayed launches and as one persistent launch."""
    import torch

    from sph_fem_2d_cutting_gpu_gb300 import abi, setups, tune
    from sph_fem_2d_cutting_gpu_gb300.solver import Batch

    cases = setups.batched_sweep(n_cases=16, seed=args.seed + 1, n_min=3000, n_max=12000, height=0.025)
    steps = max(args.steps, 50)
    best_v, table = (0, None) if args.no_tune else \
        tune_fresh(lambda: Batch(cases, abi.SPH_PREC_FP32K, device=local), args.warmup, steps)
    out = None
    for name, form in (("launches", abi.SPH_STEP_LAUNCHES), ("persistent", abi.SPH_STEP_PERSISTENT)):
        b = Batch(cases, abi.SPH_PREC_FP32K, device=local)   # a fresh batch: both forms time the same steps
        tune.set_variant(b, best_v)
        tune.set_step_form(b, form)
        if out is None:
            out = {"workload": f"{b.n_cases} AISI 1045 cuts of {min(c.N for c in cases)}-{max(c.N for c in cases)} "
                               f"particles ({b.N} in all), own FEM tool each "
                               f"({sum(i['node_count'] for i in b.info)} nodes in all), FP32K",
                   "particles": b.N, "cases": b.n_cases}
            if table is not None:
                out["launch_tuning"] = {"chosen": list(table)[best_v], "ms_per_step": table}
        ext = stream_of(b, local)
        b.step(args.warmup)
        b.sync()
        n0 = b.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        b.step(steps)
        e1.record(ext)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[name] = {"ms_per_step": ms, "value": b.N / (ms * 1e-3),
                     "launches_per_step": (b.launch_count() - n0) / steps, "status": b.status()}
        b.close()
        torch.cuda.empty_cache()
    out["persistent_speedup"] = out["launches"]["ms_per_step"] / out["persistent"]["ms_per_step"]
    return out


def run_rigid(args, local):
    """The reference's SPH-tool cut (setup_ref_cut with mfree_gpu.cpp's default
    arguments: rake 0, clearance 4.5 deg, edge radius 3.5 um, uncut chip 100 um,
    300 in the reference's speed unit) at ny = 30 rows -- the reference's own
    size -- and at larger ny: leap_frog::step(particles, grid) with the rigid
    tool, the Brookshaw build and the PSE build, each in FP64 and FP32K; the
    CPU oracle's whole-step time beside each size."""
    import ctypes as C

    import torch

    from sph_fem_2d_cutting_gpu_gb300 import abi, setups, tune
    from sph_fem_2d_cutting_gpu_gb300.solver import Solver
    from oracle.oracle import OracleSim, num_threads

    speed = 83.333328e-5 / 200 * 300
    rows = []
    for ny in args.rigid_ny:
        case = setups.ref_cut(ny=ny, rake=0.0, clear=4.5, chamfer=0.00035, speed=speed, feed=0.01)
        row = {"ny": ny, "particles": case.N, "workpiece": case.info["n_workpiece"], "tool": case.info["n_tool"]}
        best_v = 0
        if not args.no_tune:   # launch shape of the FP32K neighbour sums (Brookshaw build)
            best_v, table = tune_fresh(lambda: Solver(case, abi.SPH_PREC_FP32K, device=local), args.warmup,
                                       args.steps)
            row["launch_tuning"] = {"chosen": list(table)[best_v], "ms_per_step": table}
        for name, prec, pse in (("fp64", abi.SPH_PREC_FP64, False), ("fp32k", abi.SPH_PREC_FP32K, False),
                                ("fp64_pse", abi.SPH_PREC_FP64, True), ("fp32k_pse", abi.SPH_PREC_FP32K, True)):
            s = Solver(case, prec, device=local)
            if pse:
                s.set_thermal_model(abi.SPH_THERMAL_PSE)
            if prec == abi.SPH_PREC_FP32K:
                tune.set_variant(s, best_v)
            sp = C.c_void_p()
            s.lib.sph_get_stream(s.ctx, C.byref(sp))
            ext = torch.cuda.ExternalStream(sp.value, device=torch.device("cuda", local))
            s.step(args.warmup)
            s.sync()
            n0 = s.launch_count()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            s.step(args.steps)
            e1.record(ext)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            row[name] = {"ms_per_step": ms, "value": case.N / (ms * 1e-3),
                         "launches_per_step": (s.launch_count() - n0) / args.steps, "status": s.status()}
            s.close()
        if not args.no_cpu:
            o = OracleSim(case.constants, case.grid, case.particles, case.dt, rigid=case.rigid.to_struct())
            o.step()
            t0, n = time.perf_counter(), 0
            while n < 1 or (time.perf_counter() - t0 < args.cpu_seconds / 4 and n < 200):
                o.step()
                n += 1
            el = time.perf_counter() - t0
            row["cpu_oracle"] = {"value": case.N * n / el, "ms_per_step": 1e3 * el / n, "steps": n,
                                 "cores": num_threads()}
            row["fp64_vs_cpu"] = row["cpu_oracle"]["ms_per_step"] / row["fp64"]["ms_per_step"]
        rows.append(row)
        torch.cuda.empty_cache()
    return {"unit": UNIT, "rows": rows,
            "workload": "setup_ref_cut (benchmarks.cpp:247-530) with mfree_gpu.cpp's default arguments: Ti6Al4V, "
                        "workpiece 1.95 mm x 0.3 mm, rigid tool (rake 0, clearance 4.5 deg, r 3.5 um) sampled "
                        "with thermal tool particles, 1.25e-3 cm/us; ny rows (30: the reference's size)"}


def curve_run(s, steps, every, ext, log_records=0):
    """Advance `s` by `steps` fused steps in chunks of `every`, recording the
    cutting force (sum of fc + ft) and the peak temperature after each chunk.
    Device time is taken with CUDA events around the chunks (the reductions
    between chunks are outside it).  With log_records, return mappings are
    logged until that many states are held; those chunks are timed apart."""
    import torch

    hist, chunk_ms, ms_run, ms_log, n_run, n_log = [], [], 0.0, 0.0, 0, 0
    logging = log_records > 0
    if logging:
        s.jc_log_enable(log_records)
    s.jc_stats(True, reset=True)
    rec = None
    for _ in range(steps // every):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        s.step(every)
        e1.record(ext)
        e1.synchronize()
        chunk_ms.append(e0.elapsed_time(e1))
        if logging:
            ms_log += e0.elapsed_time(e1)
            n_log += every
            if s.jc_log_read(0)[1] >= log_records:
                rec = s.jc_log_read()
                s.jc_log_enable(0)
                logging = False
        else:
            ms_run += e0.elapsed_time(e1)
            n_run += every
        F = s.reduce_force()
        hist.append((float(F[0]), float(F[1]), s.max_T()))
    if logging:
        rec = s.jc_log_read()
        s.jc_log_enable(0)
    calls, iters = s.jc_stats(True, reset=True)
    # a run that logged throughout has only its logging chunks to time
    return dict(hist=hist, chunk_ms=chunk_ms, ms_per_step=(ms_run / n_run) if n_run else ms_log / max(n_log, 1),
                ms_per_step_logging=(ms_log / n_log) if n_log else None, steps_logging=n_log,
                returns=calls, iters_per_return=iters / max(calls, 1), status=s.status()), rec


def curve_errors(ref, other):
    """Force error relative to the reference run's peak force, peak-temperature
    error relative to its rise above 300 K, over all checkpoints."""
    import numpy as np
    F0 = np.array([h[:2] for h in ref])
    T0 = np.array([h[2] for h in ref])
    F = np.array([h[:2] for h in other])
    T = np.array([h[2] for h in other])
    fmax = float(np.linalg.norm(F0, axis=1).max())
    rise = max(float(T0.max()) - 300.0, 1.0)
    return {"force_err_of_peak": float(np.linalg.norm(F - F0, axis=1).max() / max(fmax, 1e-300)),
            "peak_T_err_of_rise": float(np.abs(T - T0).max() / rise)}


def run_config3(args, local):
    """The AISI 1045 cut at its stated size and length (640,000 particles, tool
    of about 20,000 nodes, 20,000 steps): the plain FP64 form, the FP32K form
    (logging its return mappings until `learned_records` states), then the MLP
    trained on the logged states (90 %, scored on the held-out 10 %) and the
    FP32K + MLP form, each over the whole run from the same start.  Cutting
    force and peak temperature every `config3_every` steps; the FP64 form is the
    reference of the error curves (it matches the CPU restatement of the
    reference to 1e-10 per step)."""
    import ctypes as C

    import numpy as np
    import torch

    from sph_fem_2d_cutting_gpu_gb300 import abi, learned, setups
    from sph_fem_2d_cutting_gpu_gb300.solver import Solver

    def solver(prec):
        s = Solver(case, prec, device=local, place_tool=False)
        stream_ptr = C.c_void_p()
        s.lib.sph_get_stream(s.ctx, C.byref(stream_ptr))
        return s, torch.cuda.ExternalStream(stream_ptr.value, device=torch.device("cuda", local))

    steps, every = args.config3_steps, args.config3_every
    case = setups.placed(setups.aisi1045_cut(steps=steps), mode="edge")
    runs = {}
    s, ext = solver(abi.SPH_PREC_FP64)
    runs["fp64"], _ = curve_run(s, steps, every, ext)
    s.close()
    torch.cuda.empty_cache()
    s, ext = solver(abi.SPH_PREC_FP32K)
    t0 = time.perf_counter()
    runs["fp32k"], logged = curve_run(s, steps, every, ext, log_records=args.learned_records)
    s.close()
    rec, offered = logged
    n_logged = len(rec)
    rec = learned.valid_records(rec)
    x, t = learned.features(rec, case.constants)
    rng = np.random.default_rng(args.seed)
    perm = rng.permutation(len(t))
    n_ho = max(1, len(t) // 10)
    ho, tr = perm[:n_ho], perm[n_ho:]
    m = learned.Mlp(device=local, seed=args.seed)
    m.fit_norm(x[tr], t[tr])
    t0 = time.perf_counter()
    losses = m.train(x[tr], t[tr], epochs=args.learned_epochs, batch=8192, lr=2e-3, seed=args.seed)
    train_s = time.perf_counter() - t0
    dl_max = rec[ho, learned.NORM] / np.float32(2.0 * case.constants.phys.G)
    dl_true = rec[ho, learned.DL]
    dl_mlp = np.minimum(np.exp(m.predict(x[ho])) * dl_max, dl_max)
    dl_ref = np.maximum(rec[ho, learned.EPSD] * rec[ho, learned.DT] * np.float32(np.sqrt(2.0 / 3.0)),
                        np.float32(1e-8))
    err_mlp = np.abs(dl_mlp - dl_true) / dl_true
    err_ref = np.abs(dl_ref - dl_true) / dl_true
    for name, mode in (("fp32k_mlp", abi.SPH_MLP_WARP), ("fp32k_mlp_tensor", abi.SPH_MLP_TENSOR)):
        s, ext = solver(abi.SPH_PREC_FP32K)
        s.attach_mlp(m, mode)
        runs[name], _ = curve_run(s, steps, every, ext)
        s.close()
        torch.cuda.empty_cache()
    ms64 = runs["fp64"]["ms_per_step"]
    # every form timed over the same window: the steps after the FP32K run's logging
    w0 = runs["fp32k"]["steps_logging"] // every
    window = {n: sum(r["chunk_ms"][w0:]) / max((len(r["chunk_ms"]) - w0) * every, 1) for n, r in runs.items()}
    curve = [{"step": (k + 1) * every, **{f"{n}": {"force": list(r["hist"][k][:2]), "peak_T": r["hist"][k][2]}
                                         for n, r in runs.items()}} for k in range(steps // every)]
    T64 = [h[2] for h in runs["fp64"]["hist"]]
    config3 = {
        "workload": f"AISI 1045 cut 1600x400 ({case.N} particles), tool of {case.info['nodes']} nodes (rake -6 deg, "
                    f"clearance 5 deg, edge radius 20 um), 120 m/min, uncut chip 100 um, edge placement, "
                    f"{steps} steps of dt {case.dt:.4g} us",
        "steps": steps, "every": every, "particles": case.N, "tool_nodes": case.info["nodes"],
        "peak_T_fp64": float(max(T64)), "T_rise_fp64": float(max(T64) - 300.0),
        "peak_force_fp64": float(max(np.hypot(h[0], h[1]) for h in runs["fp64"]["hist"])),
        "errors_vs_fp64": {n: curve_errors(runs["fp64"]["hist"], runs[n]["hist"])
                           for n in ("fp32k", "fp32k_mlp", "fp32k_mlp_tensor")},
        "ms_per_step": {n: r["ms_per_step"] for n, r in runs.items()},
        "window_steps": [w0 * every, steps],
        "ms_per_step_same_window": window,
        "iters_per_return": {n: r["iters_per_return"] for n, r in runs.items()},
        "status": {n: r["status"] for n, r in runs.items()},
        "speedup_vs_fp64": {n: window["fp64"] / window[n] for n in ("fp32k", "fp32k_mlp", "fp32k_mlp_tensor")},
        "curve": curve,
    }
    learned_line = {
        "workload": config3["workload"],
        "records_logged": int(n_logged), "records_offered": int(offered), "records_usable": int(len(rec)),
        "steps_logged": runs["fp32k"]["steps_logging"],
        "ms_per_step_while_logging": runs["fp32k"]["ms_per_step_logging"],
        "train_samples": int(len(tr)), "train_epochs": args.learned_epochs,
        "train_s": train_s, "train_loss": [float(v) for v in losses],
        "heldout": {"samples": int(n_ho),
                    "median_rel_err_mlp": float(np.median(err_mlp)),
                    "p90_rel_err_mlp": float(np.quantile(err_mlp, 0.9)),
                    "median_rel_err_reference_start": float(np.median(err_ref)),
                    "p90_rel_err_reference_start": float(np.quantile(err_ref, 0.9)),
                    "logged_iters_per_return": float(rec[:, learned.ITERS].mean())},
        "fp32k_plain": {"value": case.N / (runs["fp32k"]["ms_per_step"] * 1e-3),
                        "ms_per_step": runs["fp32k"]["ms_per_step"], "returns": runs["fp32k"]["returns"],
                        "iters_per_return": runs["fp32k"]["iters_per_return"],
                        "timed_steps": steps - runs["fp32k"]["steps_logging"]},
        "fp32k_mlp": {"value": case.N / (runs["fp32k_mlp"]["ms_per_step"] * 1e-3),
                      "ms_per_step": runs["fp32k_mlp"]["ms_per_step"], "returns": runs["fp32k_mlp"]["returns"],
                      "iters_per_return": runs["fp32k_mlp"]["iters_per_return"], "timed_steps": steps,
                      "inference": "warp per yielding particle, in the neighbour-sum epilogue"},
        "fp32k_mlp_tensor": {"value": case.N / (runs["fp32k_mlp_tensor"]["ms_per_step"] * 1e-3),
                             "ms_per_step": runs["fp32k_mlp_tensor"]["ms_per_step"],
                             "returns": runs["fp32k_mlp_tensor"]["returns"],
                             "iters_per_return": runs["fp32k_mlp_tensor"]["iters_per_return"], "timed_steps": steps,
                             "inference": "tcgen05 tiles of 128 queued particles, a second kernel"},
        "fp64_plain": {"value": case.N / (ms64 * 1e-3), "ms_per_step": ms64, "returns": runs["fp64"]["returns"],
                       "iters_per_return": runs["fp64"]["iters_per_return"], "timed_steps": steps},
        "same_window": {"steps": [w0 * every, steps], "ms_per_step": window},
        "speedup_mlp_vs_fp64": window["fp64"] / window["fp32k_mlp"],
        "unit": UNIT,
    }
    return config3, learned_line, m


def run_product(args):
    import ctypes as C

    import numpy as np
    import torch

    from sph_fem_2d_cutting_gpu_gb300 import abi, setups
    from sph_fem_2d_cutting_gpu_gb300.solver import Solver

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    barrier, max_over_ranks = rank_collectives(dist, torch.device("cuda", local))

    # cells of 2h with a 3x3 stencil, as the micro-benchmark specifies
    case = setups.micro(n_side=args.n_side, seed=args.seed + rank, cell_factor=args.cell_factor,
                        stencil=args.stencil)
    hbm_peak, peak_kind = peaks()
    results = {}
    for prec_name, prec in (("fp32k", abi.SPH_PREC_FP32K), ("fp64", abi.SPH_PREC_FP64)):
        if args.precision != "both" and args.precision != prec_name:
            continue
        s = Solver(case, prec, device=local)
        stream_ptr = C.c_void_p()
        s.lib.sph_get_stream(s.ctx, C.byref(stream_ptr))
        ext = torch.cuda.ExternalStream(stream_ptr.value, device=torch.device("cuda", local))
        variant_table = None
        if prec == abi.SPH_PREC_FP32K and not args.no_tune:
            # launch shape of the neighbour sums: timed on this workload (the state it
            # advances is restored afterwards, so the timed run starts from step 0)
            from sph_fem_2d_cutting_gpu_gb300 import tune
            P0 = s.download()
            variant_table = []
            for v in range(len(tune.launch_variants())):   # 12 steps each: shapes within 2 % of each other
                tune.set_variant(s, v)
                variant_table.append(tune._time_steps(s, 3, 12))
            best_v = min(range(len(variant_table)), key=lambda v: variant_table[v])
            tune.set_variant(s, 0)
            tune.set_step_form(s, abi.SPH_STEP_PERSISTENT)   # the one-launch step (128-particle blocks)
            persistent_ms = tune._time_steps(s, 3, 12)
            use_persistent = persistent_ms < variant_table[best_v]
            if not use_persistent:
                tune.set_step_form(s, abi.SPH_STEP_LAUNCHES)
                tune.set_variant(s, best_v)
            s.upload(P0)
            del P0
        # clock samples (every 200 ms) span the loaded period around the timed steps:
        # warm-up, timed steps, stage profile and the end-to-end loop
        clocks = Clocks(local) if rank == 0 else None
        for _ in range(args.warmup):
            s.step()
        s.sync()
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        n0 = s.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        s.step(args.steps)
        e1.record(ext)
        e1.synchronize()
        launches = s.launch_count() - n0
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1) / args.steps
        ms = max_over_ranks(ms)
        st = s.status()
        # per-stage device times (same kernels, issued without the graph)
        stage_ms = (C.c_float * 7)()
        ns = C.c_int32()
        s._ck(s.lib.sph_profile_steps(s.ctx, args.steps, stage_ms, C.byref(ns)), "sph_profile_steps")
        stage = [v / args.steps for v in stage_ms]
        res = dict(ms=ms, launches=launches / args.steps * args.steps, status=st,
                   stage_ms=dict(zip(STAGES, stage)), launches_per_step=launches / args.steps)
        if variant_table is not None:
            from sph_fem_2d_cutting_gpu_gb300 import tune
            shapes = tune.launch_variants()
            res["launch_tuning"] = {"chosen": ({"step_form": "persistent", "block": 128, "min_blocks": 6,
                                                "staged_records": 0, "lanes_per_particle": 1} if use_persistent else
                                               {"step_form": "launches", "block": shapes[best_v][0],
                                                "min_blocks": shapes[best_v][1], "staged_records": shapes[best_v][2],
                                                "lanes_per_particle": shapes[best_v][3]}),
                                    "ms_per_step": {tune.shape_name(sh): t for sh, t in zip(shapes, variant_table)},
                                    "persistent_ms_per_step": persistent_ms}
        # end-to-end through the C ABI with pinned host buffers
        if not args.no_e2e:
            fields = {}
            full = s.download(E2E_FIELDS)
            for k, v in full.items():
                t = torch.empty(v.shape, dtype=torch.float64 if v.dtype == np.float64 else torch.int32,
                                pin_memory=True)
                a = t.numpy()
                a[...] = v
                fields[k] = (t, a)
            host_in = {k: a for k, (_, a) in fields.items()}
            outs = {}
            for k, v in full.items():
                t = torch.empty(v.shape, dtype=torch.float64 if v.dtype == np.float64 else torch.int32,
                                pin_memory=True)
                outs[k] = (t, t.numpy())
            host_out = {k: a for k, (_, a) in outs.items()}
            pin_in = abi.particles_struct(host_in, s.N)
            pin_out = abi.particles_struct(host_out, s.N)
            nbytes = sum(a.nbytes for a in host_in.values())
            for _ in range(max(1, args.warmup // 2)):
                s._ck(s.lib.sph_upload_particles(s.ctx, C.byref(pin_in)), "upload")
                s.step()
                s._ck(s.lib.sph_download_particles(s.ctx, C.byref(pin_out)), "download")
            barrier()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                s._ck(s.lib.sph_upload_particles(s.ctx, C.byref(pin_in)), "upload")
                s.step()
                s._ck(s.lib.sph_download_particles(s.ctx, C.byref(pin_out)), "download")
            el = time.perf_counter() - t0
            el = max_over_ranks(el)
            e2e_sync = dict(value=world * case.N * args.steps / el, unit=UNIT, h2d_bytes_per_step=nbytes,
                            d2h_bytes_per_step=nbytes, api="sph_upload_particles + sph_step + sph_download_particles")
            # pipelined: each step's state in and result out, the upload of the next state
            # overlapping the download of the last result (sph_*_particles_async)

            def pipelined(n):
                s.upload_async(pin_in)
                for k in range(n):
                    s.step()
                    s.download_async(pin_out)
                    if k + 1 < n:
                        s.upload_async(pin_in)
                s.sync()

            pipelined(max(2, args.warmup))
            barrier()
            n_e2e = max(args.steps, args.e2e_steps)   # a stream of requests: the first upload and
            t0 = time.perf_counter()                  # the last download are not overlapped
            pipelined(n_e2e)
            el = max_over_ranks(time.perf_counter() - t0)
            res["e2e"] = dict(value=world * case.N * n_e2e / el, unit=UNIT, h2d_bytes_per_step=nbytes,
                              d2h_bytes_per_step=nbytes, requests=n_e2e,
                              api="sph_upload_particles_async + sph_step + sph_download_particles_async")
            res["e2e_sync"] = e2e_sync
        res["clocks"] = clocks.stop() if clocks else None
        stage_interact = stage[4]
        ab = ALGO_BYTES[prec_name]
        algo = (ab["read"] + ab["write"]) * case.N
        ach = algo / (stage_interact * 1e-3) / 1e9
        fl = NCU_FLOPS_PER_PARTICLE[prec_name] * case.N / (stage_interact * 1e-3) / 1e12
        res["compute"] = {"pipe": "fp64" if prec_name == "fp64" else "fp32", "achieved": fl,
                          "peak": NOMINAL_TFLOPS[prec_name], "unit": "TFLOP/s",
                          "frac": fl / NOMINAL_TFLOPS[prec_name], "peak_kind": "nominal",
                          "flops_per_particle": NCU_FLOPS_PER_PARTICLE[prec_name]}
        res["roofline"] = {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                           "frac": ach / hbm_peak,
                           "traffic": (NCU_TRAFFIC_PER_PARTICLE[prec_name] * case.N
                                       if prec_name in NCU_TRAFFIC_PER_PARTICLE and args.cell_factor == 2 else None),
                           "kernel": f"k_interact{'32' if prec_name == 'fp32k' else '64'}<fused>",
                           "algo_bytes_per_particle": ab["read"] + ab["write"], "peak_kind": peak_kind}
        results[prec_name] = res
        s.close()
        del s
        torch.cuda.empty_cache()

    # the same micro workload on the reference's cell geometry (cells of h, 5x5)
    alt = None
    if args.cell_factor == 2 and not args.no_alt_geometry:
        alt = {}
        hc = setups.micro(n_side=args.n_side, seed=args.seed + rank, cell_factor=1, stencil=2)
        for prec_name, prec in (("fp32k", abi.SPH_PREC_FP32K), ("fp64", abi.SPH_PREC_FP64)):
            if args.precision != "both" and args.precision != prec_name:
                continue
            s = Solver(hc, prec, device=local)
            stream_ptr = C.c_void_p()
            s.lib.sph_get_stream(s.ctx, C.byref(stream_ptr))
            ext = torch.cuda.ExternalStream(stream_ptr.value, device=torch.device("cuda", local))
            s.step(args.warmup)
            s.sync()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            s.step(args.steps)
            e1.record(ext)
            e1.synchronize()
            ms = max_over_ranks(e0.elapsed_time(e1) / args.steps)
            alt[prec_name] = {"value": world * hc.N / (ms * 1e-3), "ms_per_step": ms}
            s.close()
            torch.cuda.empty_cache()
    learned_line, config3_line, mlp = None, None, None
    if args.config3_steps > 0 and args.learned_records > 0 and rank == 0:
        config3_line, learned_line, mlp = run_config3(args, local)
        torch.cuda.empty_cache()
    batched = None
    if args.batched_cases > 0:
        batched = run_batched(args, local, max_over_ranks, barrier, mlp)
        torch.cuda.empty_cache()
    if mlp is not None:
        mlp.close()
    small_line = tiny_line = None
    if not args.no_small and rank == 0:
        small_line = run_small_cut(args, local)
        torch.cuda.empty_cache()
        tiny_line = run_tiny_sweep(args, local)
        torch.cuda.empty_cache()
    rigid_line = None
    if args.rigid_ny and rank == 0:
        rigid_line = run_rigid(args, local)
        torch.cuda.empty_cache()

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0
    head_name = "fp32k" if "fp32k" in results else "fp64"
    head = results[head_name]
    value = replica_value(world, case.N, head["ms"])
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32k" if head_name == "fp32k" else "f64",
        "data": "synthetic (seeded): jittered lattice, random velocity/stress/density",
        "config": {"workload": f"micro {case.info['n_side']}x{case.info['n_side']} lattice ({case.N} particles), "
                               f"dx=2.5um, h=1.7dx, cells {args.cell_factor}h / "
                               f"{2 * args.stencil + 1}x{2 * args.stencil + 1} stencil, AISI 1045 JC; full "
                               "leap-frog step without tool",
                   "particles": case.N, "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (about 3 GB of particle state per GPU)",
                   "form": "FP32 neighbour sums with Kahan compensation, FP64 state/positions/residual"
                           if head_name == "fp32k" else "plain FP64"},
        "roofline": head["roofline"],
        "compute": head["compute"],
        "clocks": head["clocks"],
        "gpu_launches": int(round(head["launches"])),
        "stage_ms": head["stage_ms"],
        "status": head["status"],
    }
    if "launch_tuning" in head:
        line["launch_tuning"] = head["launch_tuning"]
    if "e2e" in head:
        line["e2e"] = head["e2e"]
        line["e2e_sync"] = head["e2e_sync"]
    if "fp64" in results and head_name != "fp64":
        f = results["fp64"]
        line["fp64"] = {"value": world * case.N / (f["ms"] * 1e-3), "ms_per_step": f["ms"],
                        "stage_ms": f["stage_ms"], "roofline": f["roofline"], "compute": f["compute"],
                        "clocks": f["clocks"],
                        "e2e": f.get("e2e")}
        line["speedup_vs_fp64"] = f["ms"] / head["ms"]
    if alt:
        line["micro_cells_h"] = dict(alt, workload="the same micro workload with cells of h / 5x5 stencil "
                                                   "(the reference's geometry), default launch shape")
    if batched is not None:
        batched["value"] *= world
        line["batched_sweep"] = batched
    if learned_line is not None:
        line["learned_warm_start"] = learned_line
    if config3_line is not None:
        line["config3_run"] = config3_line
    if rigid_line is not None:
        line["rigid_tool_cut"] = rigid_line
    if small_line is not None:
        line["ti64_cut_small"] = small_line
    if tiny_line is not None:
        line["tiny_sweep"] = tiny_line
    if not args.no_cpu:
        v, cores, n, el = cpu_sample(case, max_seconds=args.cpu_seconds)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"{n} whole steps of the full workload in {el:.1f}s "
                                          f"(CPU oracle restatement, OpenMP)"}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="product", choices=["product", "reference"])
    ap.add_argument("--precision", default="both", choices=["both", "fp32k", "fp64"])
    ap.add_argument("--n-side", type=int, default=2048)
    ap.add_argument("--ref-side", type=int, default=0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=40,
                    help="requests in the timed pipelined end-to-end stream (at least --steps)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--batched-cases", type=int, default=64, help="cases of the batched sweep (0: skip)")
    ap.add_argument("--learned-records", type=int, default=10_000_000,
                    help="return-mapping states logged for the learned warm start (0: skip)")
    ap.add_argument("--learned-max-steps", type=int, default=20_000)
    ap.add_argument("--learned-epochs", type=int, default=3)
    ap.add_argument("--config3-steps", type=int, default=20000,
                    help="AISI 1045 cut (640,000 particles): steps of the FP64 / FP32K / FP32K+MLP runs (0: skip)")
    ap.add_argument("--config3-every", type=int, default=500, help="checkpoint interval of the config-3 runs")
    ap.add_argument("--sweep-steps", type=int, default=5000,
                    help="batched sweep: steps of the full-length run with FP64 reference cases (0: skip)")
    ap.add_argument("--sweep-every", type=int, default=500, help="checkpoint interval of the sweep run")
    ap.add_argument("--no-tune", action="store_true", help="no launch-shape / cell-geometry autotuning")
    ap.add_argument("--cell-factor", type=int, default=2, help="micro workload: cell edge in h")
    ap.add_argument("--no-alt-geometry", action="store_true", help="skip the cells-of-h micro line")
    ap.add_argument("--stencil", type=int, default=1, help="micro workload: stencil half-width in cells")
    ap.add_argument("--no-small", action="store_true", help="skip the 12,000-particle Ti6Al4V cut line")
    ap.add_argument("--rigid-ny", type=int, nargs="*", default=[30, 240],
                    help="rows of the rigid-tool cut sizes to time (none: skip)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    return args


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_product(args)


if __name__ == "__main__":
    sys.exit(main())
