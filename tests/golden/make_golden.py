"""Generate tests/golden/ref_pin.npz from the reference's own arithmetic.

Builds oracle/_ref/ref_pin (oracle/Makefile target ``ref``: the reference's
kernels.cuh and plasticity.cuh compiled for the host from the read-only
reference tree) and records, for seeded inputs:
  * cubic_spline(posi, posj, h)                          (kernels.cuh:25-65)
  * sigma_yield(jc, eps_pl, eps_pl_dot, T)               (plasticity.cuh:21-39)
  * solve_secant(jc, init, tol, normS, eps_pl, T, dt, mu) (plasticity.cuh:128-162)
Run here (where the reference tree exists); the fixture travels, the
reference does not.  Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
OUT = Path(__file__).resolve().parent / "ref_pin.npz"
REF_BIN = ROOT / "oracle" / "_ref" / "ref_pin"

# Johnson-Cook sets (A, B, C, n, m, Tmelt, Tref, eps_dot_ref): Ti6Al4V, AISI 1045,
# and the reference's own Ti6Al4V set (benchmarks_NZ.cpp:90-97)
JC_SETS = np.array([
    [0.00862, 0.00331, 0.012, 0.34, 0.8, 1836.0, 300.0, 1e-6],
    [0.005531, 0.006008, 0.0134, 0.234, 1.0, 1733.0, 300.0, 1e-6],
    [0.0085200, 0.0033890, 0.02754, 0.148, 0.5961, 1836.0, 300.0, 1e-6],
])


def run(mode: str, rows: np.ndarray) -> np.ndarray:
    txt = "\n".join(" ".join(f"{v:.17g}" for v in r) for r in rows) + "\n"
    r = subprocess.run([str(REF_BIN), mode], input=txt, capture_output=True, text=True, check=True)
    return np.array([[float(x) for x in line.split()] for line in r.stdout.strip().splitlines()])


def main():
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref"], check=True)
    rng = np.random.default_rng(20241203)
    # ---- cubic spline: pairs around h, including both branches, the support
    # edge, the 1e-8 inner cutoff and q exactly 1 / 2
    n = 4000
    h = rng.uniform(2e-4, 1e-3, n)
    r = h * rng.uniform(0.0, 2.2, n)
    ang = rng.uniform(0, 2 * np.pi, n)
    pi = rng.uniform(-0.1, 0.1, (n, 2))
    pj = pi - np.stack([r * np.cos(ang), r * np.sin(ang)], 1)
    pj[:8] = pi[:8] - np.array([[1.0, 0.0]]) * (h[:8] * np.array([1.0, 2.0, 0.0, 1e-5, 1.9999999, 1.0000001, 0.5, 1.5]))[:, None]
    spl_in = np.concatenate([pi, pj, h[:, None]], 1)
    spl_out = run("spline", spl_in)
    # ---- sigma_yield over strain, rate (both branches of eps_dot > 1) and T
    m = 3000
    jc = JC_SETS[rng.integers(0, len(JC_SETS), m)]
    eps = np.where(rng.random(m) < 0.2, 0.0, rng.uniform(0, 3, m))
    epsdot = 10 ** rng.uniform(-9, -2, m)
    T = rng.uniform(300, 1800, m)
    y_in = np.concatenate([jc, eps[:, None], epsdot[:, None], T[:, None]], 1)
    y_out = run("yield", y_in)
    # ---- secant return mapping (plasticity.cuh:128-162) with the call site's
    # initial guess fmax(eps_pl_dot*dt*sqrt(2/3), 1e-8) (actions_gpu.cu:725)
    k = 3000
    jc = JC_SETS[rng.integers(0, len(JC_SETS), k)]
    mu = np.where(jc[:, 0] > 0.0085, 0.4237, 0.7692)
    dt = 10 ** rng.uniform(-5, -3.5, k)
    eps = np.where(rng.random(k) < 0.3, 0.0, rng.uniform(0, 2, k))
    epsdot = np.where(rng.random(k) < 0.3, 0.0, 10 ** rng.uniform(-6, -1, k))
    T = rng.uniform(300, 1500, k)
    normS = jc[:, 0] * rng.uniform(0.9, 3.0, k)
    init = np.maximum(epsdot * dt * np.sqrt(2.0 / 3.0), 1e-8)
    tol = np.full(k, 1e-6)
    s_in = np.concatenate([jc, init[:, None], tol[:, None], normS[:, None], eps[:, None], T[:, None], dt[:, None],
                           mu[:, None]], 1)
    s_out = run("secant", s_in)
    np.savez_compressed(OUT, spline_in=spl_in, spline_out=spl_out, yield_in=y_in, yield_out=y_out,
                        secant_in=s_in, secant_out=s_out)
    print(f"wrote {OUT}: {len(spl_in)} spline, {len(y_in)} yield, {len(s_in)} secant cases")


if __name__ == "__main__":
    sys.exit(main())
