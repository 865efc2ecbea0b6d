"""The cell index of compute_hashes, (int)((x - bbmin)/dx) in FP64 (grid.cu:36-39),
is computed on the device from an FP32 quotient with an error margin, and the
FP64 division only near an integer.  This restates that rule in numpy (IEEE
FP32 multiply, truncation) and checks it never disagrees with the FP64
division -- on random offsets and on offsets placed at cell edges."""
import numpy as np


def fast_cell(a: np.ndarray, dx: float):
    """(index, used_fallback) of the device rule for offsets a >= 0."""
    inv = np.float32(1.0 / dx)
    qf = a.astype(np.float32) * inv
    t = np.trunc(qf)
    fr = qf - t
    m = np.float32(2.5e-7) * qf + np.float32(1e-30)
    ok = (fr > m) & (fr < np.float32(1) - m)
    exact = np.trunc(a / dx)
    return np.where(ok, t.astype(np.float64), exact), ok


def test_fast_cell_index_matches_fp64_division():
    rng = np.random.default_rng(0)
    for dx in (4.25e-4, 8.5e-4, 2.5e-4 * 1.7 * 2, 3.3333e-3):
        # random offsets over a grid of up to 40,000 cells: the FP32 path decides almost all
        r = rng.uniform(0, 40_000 * dx, 5_000_000)
        assert fast_cell(r, dx)[1].mean() > 0.98
        a = r
        # offsets at and next to cell edges (the cases the margin exists for)
        k = rng.integers(0, 40_000, 1_000_000).astype(np.float64)
        edge = k * dx
        near = np.concatenate([edge, np.nextafter(edge, 0), np.nextafter(edge, np.inf),
                               edge * (1 + 1e-9), edge * (1 - 1e-9)])
        a = np.concatenate([a, near[near >= 0]])
        got, ok = fast_cell(a, dx)
        want = np.trunc(a / dx)
        assert np.array_equal(got, want)
