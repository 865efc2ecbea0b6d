"""The fused step's contact kernel runs find_shortest_distance_v1's loops
(actions_gpu.cu:139-220) with the 32 lanes of a warp: lane k takes segments
k, k + 32, ..., keeps its own best with the reference's strict `<`, and the warp
takes the smallest (value, index).  This restates both forms in numpy and
checks they pick the same segment as the reference's single loop -- with ties,
with candidates rejected after the distance test (the intersection check), and
with nothing accepted."""
import numpy as np

FLT_MAX = float(np.finfo(np.float32).max)


def reference_loop(d, ok):
    """The first loop: `if (ok && d >= 0 && d < depth) { depth = d; seg = i; }`."""
    depth, seg = FLT_MAX, -1
    for i in range(len(d)):
        if d[i] >= 0.0 and d[i] < depth and ok[i]:
            depth, seg = d[i], i
    return seg, depth


def warp_loop(d, ok, lanes=32):
    best = []
    for lane in range(lanes):
        b, bi = FLT_MAX, 0x7FFFFFFF
        for i in range(lane, len(d), lanes):
            if d[i] >= 0.0 and d[i] < b and ok[i]:
                b, bi = d[i], i
        best.append((b, bi))
    b, bi = min(best)                 # (value, index) lexicographic
    return (-1, FLT_MAX) if bi == 0x7FFFFFFF else (bi, b)


def test_warp_argmin_matches_the_reference_loop():
    rng = np.random.default_rng(7)
    for trial in range(3000):
        n = int(rng.integers(0, 300))
        levels = rng.uniform(-1e-3, 1e-2, int(rng.integers(1, 8)))
        d = rng.choice(levels, n) if rng.random() < 0.5 else rng.uniform(-1e-3, 1e-2, n)   # many ties
        d[rng.random(n) < 0.05] = np.inf
        d[rng.random(n) < 0.02] = np.nan
        ok = rng.random(n) < rng.uniform(0.0, 1.0)
        assert reference_loop(d, ok) == warp_loop(d, ok), trial


def test_first_match_is_the_smallest_index():
    rng = np.random.default_rng(8)
    for trial in range(2000):
        n = int(rng.integers(0, 300))
        hit = rng.random(n) < rng.uniform(0, 0.1)
        ref = next((j for j in range(n) if hit[j]), None)
        firsts = [next((j for j in range(lane, n, 32) if hit[j]), 0x7FFFFFFF) for lane in range(32)]
        got = min(firsts)
        assert (ref is None and got == 0x7FFFFFFF) or got == ref, trial
