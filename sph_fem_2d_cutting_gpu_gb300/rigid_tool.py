"""Host-side geometry of the rigid (SPH-mode) tool: the outline of
tool::tool(tl, length, height, rake, clearance, r, mu) (tool.cpp:335-369) with
its fillet (tool.cpp:27-93), the line / segment primitives
(geometric_primitives.cpp:11-113), placement by tool::update_tool
(tool.cpp:202-212), the inside test and the particle sampling of
tool::sample_tool (tool.cpp:95-135), and the packing into sph_rigid_tool.

All arithmetic is IEEE double without fused multiply-adds, as the reference's
host code; the device moves the tool every step from the packed state.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import abi

DBL_MAX = 1.7976931348623157e308


@dataclass
class Line:
    """y = a x + b, or x = b when vertical (geometric_primitives.h)."""
    a: float
    b: float
    vertical: bool

    @staticmethod
    def through(p1, p2) -> "Line":
        # geometric_primitives.cpp:58-75
        detM = p1[0] * 1.0 - 1.0 * p2[0]
        if abs(detM) < 1e-12:
            return Line(DBL_MAX, p1[0], True)
        a = (p1[1] * 1.0 - 1.0 * p2[1]) / detM
        b = (p2[1] * p1[0] - p2[0] * p1[1]) / detM
        return Line(a, b, False)

    def intersect(self, l: "Line"):
        # geometric_primitives.cpp:11-38
        if self.vertical and l.vertical:
            return (DBL_MAX, DBL_MAX)
        if abs(self.a - l.a) < 1e-12:
            return (DBL_MAX, DBL_MAX)
        if self.vertical:
            x = self.b
            return (x, l.a * x + l.b)
        if l.vertical:
            x = l.b
            return (x, self.a * x + self.b)
        x = (l.b - self.b) / (self.a - l.a)
        return (x, self.a * x + self.b)

    def closest_point(self, q):
        # geometric_primitives.cpp:40-54
        if self.vertical:
            return (self.b, q[1])
        bb, cc, aa = -1.0, self.b, self.a
        px = (bb * (bb * q[0] - aa * q[1]) - aa * cc) / (aa * aa + bb * bb)
        py = (aa * (-bb * q[0] + aa * q[1]) - bb * cc) / (aa * aa + bb * bb)
        return (px, py)


def _normalize(v):
    """glm::normalize: v * (1 / sqrt(dot(v, v)))."""
    inv = 1.0 / math.sqrt(v[0] * v[0] + v[1] * v[1])
    return (v[0] * inv, v[1] * inv)


def _myatan2(y, x):
    """tool.cpp:18-25: atan2 mapped to (0, 2 pi]."""
    t = math.atan2(y, x)
    return t if t > 0.0 else t + 2 * math.pi


@dataclass
class Segment:
    left: tuple
    right: tuple
    n: tuple = (0.0, 0.0)
    line: Line | None = None

    def __post_init__(self):
        # geometric_primitives.cpp:103-113: outward normal (dy, -dx), normalised
        d = (self.right[0] - self.left[0], self.right[1] - self.left[1])
        self.n = _normalize((d[1], -d[0]))
        self.line = Line.through(self.left, self.right)


@dataclass
class Fillet:
    r: float
    t1: float
    t2: float
    p: tuple


@dataclass
class RigidTool:
    """A rigid tool: closed outline of 4 segments, or 5 with a fillet on the
    third (tool.cpp:55-62,64-93), a velocity and a friction coefficient."""
    segments: list = field(default_factory=list)
    fillet: Fillet | None = None
    vel: tuple = (0.0, 0.0)
    mu: float = 0.0
    front: float = 0.0

    @staticmethod
    def from_points(points, mu: float) -> "RigidTool":
        n = len(points)
        segs = [Segment(tuple(points[i]), tuple(points[(i + 1) % n])) for i in range(n)]
        return RigidTool(segs, None, (0.0, 0.0), mu)

    @staticmethod
    def from_angles(tl, length: float, height: float, rake: float, clearance: float, r: float,
                    mu: float) -> "RigidTool":
        """tool.cpp:335-369: top-left corner, length, height, rake and clearance
        angles in degrees and the edge radius (0: sharp edge)."""
        tl = (float(tl[0]), float(tl[1]))
        tr = (tl[0] + length, tl[1])
        bl = (tl[0], tl[1] - height)
        a_rake = rake * math.pi / 180.0
        a_free = (180 - 90 - clearance) * math.pi / 180.0
        # down * rot (glm row vector times the column-major rotation) = (sin a, -cos a)
        trc = (tr[0] + math.sin(a_rake), tr[1] - math.cos(a_rake))
        blc = (bl[0] + math.sin(a_free), bl[1] - math.cos(a_free))
        br = Line.through(tr, trc).intersect(Line.through(bl, blc))
        if r == 0.0:
            t = RigidTool.from_points([tl, tr, br, bl], mu)
        else:
            pts, fil = _points_and_fillet(tl, tr, br, bl, r)
            t = RigidTool.from_points(pts, mu)
            t.fillet = fil
        t.front = br[0]
        return t

    # ---- tool.cpp:178-212 ----
    def low(self) -> float:
        if self.fillet:
            return self.fillet.p[1] - self.fillet.r
        return min(s.left[1] for s in self.segments)

    def update(self, dt: float):
        v = self.vel
        for s in self.segments:
            s.left = (s.left[0] + dt * v[0], s.left[1] + dt * v[1])
            s.right = (s.right[0] + dt * v[0], s.right[1] + dt * v[1])
            s.line = Line.through(s.left, s.right)
        if self.fillet:
            p = self.fillet.p
            self.fillet.p = (p[0] + dt * v[0], p[1] + dt * v[1])

    def safe_bb(self, safety: float):
        """tool.cpp:147-176: (xmin, xmax, ymin, ymax) of the outline plus a margin."""
        xs = [s.left[0] for s in self.segments]
        ys = [s.left[1] for s in self.segments]
        x_min, x_max, y_min, y_max = min(xs), max(xs), min(ys), max(ys)
        if self.fillet:
            y_min = self.low()
            x_max = self.fillet.p[0] + self.fillet.r
        return x_min - safety, x_max + safety, y_min - safety, y_max + safety

    def inside(self, pos: np.ndarray) -> np.ndarray:
        """tool.cpp:95-110 for an (n, 2) array of points."""
        q = np.asarray(pos, dtype=np.float64)
        inn = np.ones(len(q), dtype=bool)
        for s in self.segments:
            inn &= (s.left[0] - q[:, 0]) * s.n[0] + (s.left[1] - q[:, 1]) * s.n[1] < 0.0
        if self.fillet:
            d = np.sqrt((self.fillet.p[0] - q[:, 0]) ** 2 + (self.fillet.p[1] - q[:, 1]) ** 2)
            inn |= d < self.fillet.r
        return inn

    def sample(self, dx: float) -> np.ndarray:
        """tool.cpp:112-135 sample_tool: lattice points of spacing dx inside the
        outline, i outer, j inner."""
        x0, x1, y0, y1 = self.safe_bb(0.1 * dx)
        nx = int((x1 - x0) / dx + 1)
        ny = int((y1 - y0) / dx + 1)
        i, j = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
        pts = np.stack([i.ravel() * dx + x0, j.ravel() * dx + y0], 1)
        return pts[self.inside(pts)]

    def to_struct(self) -> abi.RigidTool:
        """Packed sph_rigid_tool (tool_gpu.cu:219-264 tool_gpu_set_up_tool)."""
        t = abi.RigidTool()
        t.n_seg = len(self.segments)
        t.has_fillet = 1 if self.fillet else 0
        for i, s in enumerate(self.segments):
            t.left[i][0], t.left[i][1] = s.left
            t.right[i][0], t.right[i][1] = s.right
            t.n[i][0], t.n[i][1] = s.n
            t.la[i], t.lb[i] = s.line.a, s.line.b
            t.vertical[i] = 1 if s.line.vertical else 0
        if self.fillet:
            t.fillet_p[0], t.fillet_p[1] = self.fillet.p
            t.fillet_r, t.fillet_t1, t.fillet_t2 = self.fillet.r, self.fillet.t1, self.fillet.t2
        t.vel[0], t.vel[1] = self.vel
        t.mu = self.mu
        return t


def _fit_fillet(r: float, lm: Line, l1: Line):
    """tool.cpp:27-53: centre of the fillet of radius r on the bisector lm."""
    if l1.vertical:
        return Line(DBL_MAX, l1.b - r, True).intersect(lm)
    A0, B0, a, b = lm.a, lm.b, l1.a, l1.b
    A, B = a - A0, b - B0
    Cc = r * math.sqrt(a * a + 1.0)
    qa, qb, qc = A * A, 2 * A * B, B * B - Cc * Cc
    x1 = (-qb + math.sqrt(qb * qb - 4 * qa * qc)) / (2 * qa)
    x2 = (-qb - math.sqrt(qb * qb - 4 * qa * qc)) / (2 * qa)
    xm = min(x1, x2)
    return (xm, lm.a * xm + lm.b)


def _points_and_fillet(tl, tr, br, bl, r: float):
    """tool.cpp:64-93 construct_points_and_fillet."""
    nt = _normalize((tr[0] - br[0], tr[1] - br[1]))
    nl = _normalize((bl[0] - br[0], bl[1] - br[1]))
    nm = _normalize((0.5 * (nt[0] + nl[0]), 0.5 * (nt[1] + nl[1])))
    lm = Line.through(br, (br[0] + nm[0], br[1] + nm[1]))
    l1 = Line.through(tr, br)
    l2 = Line.through(bl, br)
    p = _fit_fillet(r, lm, l1)
    trc = l1.closest_point(p)
    blc = l2.closest_point(p)
    t1 = _myatan2(p[1] - trc[1], p[0] - trc[0])
    t2 = _myatan2(p[1] - blc[1], p[0] - blc[0])
    return [tl, tr, trc, blc, bl], Fillet(r, t1, t2, p)


def place(tool: RigidTool, lo_x: float, hi_y: float, feed: float, vel_tool: float, preload_time: float = 0.0):
    """setup_ref_cut's placement (benchmarks.cpp:388-412): move the tool front
    to the workpiece front lo_x, then vertically until its lowest point is
    `feed` below the workpiece top hi_y; leave it moving at (vel_tool, 0).
    preload_time > 0 moves it further along x (0 in the reference)."""
    distance = tool.front - lo_x
    time = distance / vel_tool
    tool.vel = (vel_tool, 0.0)
    tool.update(-time)
    current_feed = hi_y - tool.low()
    correction_time = abs(current_feed - feed) / vel_tool
    sign = 1.0 if current_feed > feed else -1.0
    tool.vel = (0.0, vel_tool)
    tool.update(correction_time * sign)
    tool.vel = (vel_tool, 0.0)
    if preload_time != 0.0:
        tool.update(preload_time)
    return tool
