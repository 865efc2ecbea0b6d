"""The FEM-tool contact search skips work on bounds that must never change a
result: a particle right of its y-bin's x bound counts no ray crossing
(on_segment_mesh, actions_gpu.cu:51-63, with its float-rounded y-range), and
every segment that can count a crossing at a height is listed in that height's
bin.  This restates the bin construction and the bound of k_seg_bins in numpy
(IEEE FP64, the float rounding of the y-range) and checks both properties on
random segment chains, including points placed at the bound and segments with
steep and flat slopes."""
import numpy as np

KBINS = 64


def f32(x):
    return np.float32(x).astype(np.float64)


def crossings(L, R, p):
    """on_segment_mesh of every segment for the point p (FP64 with float-rounded y-range)."""
    ymax = f32(np.maximum(f32(L[:, 1]), f32(R[:, 1])))
    ymin = f32(np.minimum(f32(L[:, 1]), f32(R[:, 1])))
    inr = (p[1] <= ymax) & (p[1] >= ymin)
    vert = (L[:, 0] == R[:, 0]) & (p[0] < L[:, 0])
    dy = L[:, 1] - R[:, 1]
    with np.errstate(divide="ignore", invalid="ignore"):
        x_on = R[:, 0] + (L[:, 0] - R[:, 0]) / dy * (p[1] - R[:, 1])
    sloped = (np.abs(dy) != 0) & (x_on > p[0]) & (x_on != L[:, 0])
    flat = (np.abs(dy) == 0) & (p[0] <= np.maximum(L[:, 0], R[:, 0]))
    return inr & (vert | sloped | flat)


def bins(L, R):
    """Bin lists and x bounds as k_seg_bins builds them."""
    ylo = np.minimum(L[:, 1], R[:, 1])
    yhi = np.maximum(L[:, 1], R[:, 1])
    seg_ymin, seg_ymax = ylo.min(), yhi.max()
    y0, y1 = f32(seg_ymin), f32(seg_ymax)
    scale = KBINS / (y1 - y0)

    def b_of(y):
        return np.clip(np.floor((y - y0) * scale), 0, KBINS - 1).astype(int)

    b0 = np.maximum(b_of(f32(np.minimum(f32(L[:, 1]), f32(R[:, 1])))) - 1, 0)
    b1 = np.minimum(b_of(f32(np.maximum(f32(L[:, 1]), f32(R[:, 1])))) + 1, KBINS - 1)
    dy = np.abs(L[:, 1] - R[:, 1])
    dxdy = np.max(np.where(dy > 0, np.abs(L[:, 0] - R[:, 0]) / np.where(dy > 0, dy, 1), 0))
    margin = dxdy * max(abs(seg_ymin), abs(seg_ymax)) * 2.384185791015625e-7 + 1e-12
    members = [[] for _ in range(KBINS)]
    xmax = np.full(KBINS, -np.inf)
    for i, (a, c) in enumerate(zip(b0, b1)):
        for b in range(a, c + 1):
            members[b].append(i)
            xmax[b] = max(xmax[b], max(L[i, 0], R[i, 0]))
    bound = np.where(np.isfinite(xmax), xmax + margin, -np.inf)
    return b_of, members, bound


def chain(rng, n, steep):
    """A tool-like chain of segments: random walk with flat and steep pieces."""
    pts = [np.array([0.02, 0.09])]
    for _ in range(n):
        ang = rng.uniform(-np.pi, np.pi)
        if steep and rng.random() < 0.3:
            ang = np.pi / 2 + rng.normal(0, 1e-4)      # nearly vertical
        if rng.random() < 0.3:
            ang = rng.normal(0, 1e-3)                    # nearly horizontal
        pts.append(pts[-1] + rng.uniform(1e-4, 2e-3) * np.array([np.cos(ang), np.sin(ang)]))
    P = np.array(pts)
    return P[1:], P[:-1]   # left, right (as the reference's segments join right to the next left)


def test_points_right_of_the_bin_bound_cross_nothing():
    rng = np.random.default_rng(3)
    for trial in range(12):
        L, R = chain(rng, 150, steep=trial % 2 == 0)
        b_of, members, bound = bins(L, R)
        y0, y1 = np.min(np.minimum(L[:, 1], R[:, 1])), np.max(np.maximum(L[:, 1], R[:, 1]))
        ys = rng.uniform(y0 - 1e-4, y1 + 1e-4, 3000)
        for y in ys:
            b = b_of(y)
            if not np.isfinite(bound[b]):
                continue
            # at the bound, just right of it, and farther right
            for x in (bound[b], np.nextafter(bound[b], np.inf), bound[b] + rng.uniform(0, 1e-2)):
                if x <= bound[b]:
                    continue
                assert not crossings(L, R, np.array([x, y])).any(), (trial, y, x)


def test_crossing_segments_are_in_the_bin():
    rng = np.random.default_rng(5)
    for trial in range(8):
        L, R = chain(rng, 200, steep=True)
        b_of, members, _ = bins(L, R)
        lo, hi = np.min(L[:, 0]) - 0.01, np.max(L[:, 0]) + 0.01
        y0, y1 = np.min(np.minimum(L[:, 1], R[:, 1])), np.max(np.maximum(L[:, 1], R[:, 1]))
        ys = np.concatenate([rng.uniform(y0, y1, 2000), f32(L[:, 1]), np.nextafter(f32(L[:, 1]), np.inf)])
        for y in ys:
            hit = np.flatnonzero(crossings(L, R, np.array([rng.uniform(lo, hi), y])))
            assert set(hit) <= set(members[b_of(y)]), (trial, y)
