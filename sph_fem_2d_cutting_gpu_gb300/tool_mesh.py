"""Linear-triangle mesh of the FEM cutting tool.

The reference reads its tool meshes from Abaqus ``.inp`` files or gmsh
(mesh_structure_GPU.cu:213-1257); neither the meshes nor gmsh ship, so this
module generates them.  The tool outline follows tool_FEM's constructor and
fillet construction (tool_FEM.cu:623-660,705-769 with the line primitives of
geometric_primitives.cpp:86-151): corners tl, tr, bl, the rake face from tr,
the flank face from bl, and a fillet of radius r at the cutting edge.

Points are graded from ``s_min`` at the cutting edge to ``s_max`` far away;
boundary points follow the outline, interior points are layers of triangular
lattices, and scipy's Delaunay triangulation of the (convex) outline gives the
elements.  Boundary edges on the rake face, fillet and flank face are the
contact interface ("CuttingEdge" set); edges on the top and left faces are the
fixed-temperature boundary ("FixedBoundary" set).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

DBL_MAX = 1.7976931348623157e308


@dataclass
class Line:
    """geometric_primitives.h line: y = a x + b, or x = b when vertical."""
    a: float = 0.0
    b: float = 0.0
    vertical: bool = False

    @staticmethod
    def through(p1, p2) -> "Line":
        det = p1[0] * 1.0 - 1.0 * p2[0]
        if abs(det) < 1e-12:
            return Line(DBL_MAX, p1[0], True)
        a = (p1[1] * 1.0 - 1.0 * p2[1]) / det
        b = (p2[1] * p1[0] - p2[0] * p1[1]) / det
        return Line(a, b, False)

    def intersect(self, o: "Line"):
        if self.vertical and o.vertical:
            return (DBL_MAX, DBL_MAX)
        if abs(self.a - o.a) < 1e-12:
            return (DBL_MAX, DBL_MAX)
        if self.vertical:
            return (self.b, o.a * self.b + o.b)
        if o.vertical:
            return (o.b, self.a * o.b + self.b)
        x = (o.b - self.b) / (self.a - o.a)
        return (x, self.a * x + self.b)

    def closest_point(self, q):
        if self.vertical:
            return (self.b, q[1])
        bb, cc, aa = -1.0, self.b, self.a
        px = (bb * (bb * q[0] - aa * q[1]) - aa * cc) / (aa * aa + bb * bb)
        py = (aa * (-bb * q[0] + aa * q[1]) - bb * cc) / (aa * aa + bb * bb)
        return (px, py)


def _normalize(v):
    n = math.hypot(v[0], v[1])
    return (v[0] / n, v[1] / n)


def tool_outline(tl, length, height, rake_deg, clearance_deg, r):
    """Corner points and fillet of tool_FEM(tl, length, height, rake, clearance, r).

    Returns dict with tl, tr, trc, blc, bl, br (sharp corner), fillet centre p,
    radius r and the reference distance of the constructor."""
    tl = (float(tl[0]), float(tl[1]))
    tr = (tl[0] + length, tl[1])
    bl = (tl[0], tl[1] - height)
    a_rake = rake_deg * math.pi / 180.0
    a_free = (180.0 - 90.0 - clearance_deg) * math.pi / 180.0
    # down * rot (row vector times GLM column-major matrix)
    trc0 = (tr[0] + math.sin(a_rake), tr[1] - math.cos(a_rake))
    blc0 = (bl[0] + math.sin(a_free), bl[1] - math.cos(a_free))
    br = Line.through(tr, trc0).intersect(Line.through(bl, blc0))
    out = dict(tl=tl, tr=tr, bl=bl, br=br, r=r)
    if r == 0.0:
        out.update(trc=br, blc=br, p=br)
        return out
    nt = _normalize((tr[0] - br[0], tr[1] - br[1]))
    nl = _normalize((bl[0] - br[0], bl[1] - br[1]))
    nm = _normalize((0.5 * (nt[0] + nl[0]), 0.5 * (nt[1] + nl[1])))
    lm = Line.through(br, (br[0] + nm[0], br[1] + nm[1]))
    l1 = Line.through(tr, br)
    l2 = Line.through(bl, br)
    if l1.vertical:
        p = Line(DBL_MAX, l1.b - r, True).intersect(lm)
    else:
        A, B = l1.a - lm.a, l1.b - lm.b
        Cc = r * math.sqrt(l1.a * l1.a + 1.0)
        qa, qb, qc = A * A, 2 * A * B, B * B - Cc * Cc
        disc = math.sqrt(qb * qb - 4 * qa * qc)
        xm = min((-qb + disc) / (2 * qa), (-qb - disc) / (2 * qa))
        p = (xm, lm.a * xm + lm.b)
    out.update(trc=l1.closest_point(p), blc=l2.closest_point(p), p=p)
    return out


def _sample_segment(a, b, size_fn, side):
    """Points from a (included) to b (excluded), spacing from size_fn."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    L = float(np.hypot(*(b - a)))
    pts, sides = [], []
    t = 0.0
    while t < L - 1e-12 * max(L, 1.0):
        p = a + (b - a) * (t / L)
        pts.append(p)
        sides.append(side)
        h = size_fn(p)
        # keep the last interval no shorter than half a spacing
        if t + h > L - 0.5 * size_fn(b):
            if L - t > 1.5 * h:
                t += h
                continue
            break
        t += h
    return pts, sides


def _sample_arc(p, r, a0, a1, size_fn, side):
    """Arc from angle a0 to a1 (shorter way), start included, end excluded."""
    d = a1 - a0
    while d > math.pi:
        d -= 2 * math.pi
    while d < -math.pi:
        d += 2 * math.pi
    arclen = abs(d) * r
    h = size_fn(np.asarray(p))
    n = max(2, int(math.ceil(arclen / h)))
    pts = [np.array([p[0] + r * math.cos(a0 + d * k / n), p[1] + r * math.sin(a0 + d * k / n)]) for k in range(n)]
    return pts, [side] * n


SIDE_TOP, SIDE_RAKE, SIDE_ARC, SIDE_FLANK, SIDE_LEFT = range(5)
CUTTING_SIDES = (SIDE_RAKE, SIDE_ARC, SIDE_FLANK)
FIXED_SIDES = (SIDE_TOP, SIDE_LEFT)


def mesh_tool(tl, length, height, rake_deg, clearance_deg, r, s_min, s_max, grading=0.25, seed=7):
    """Triangulate the tool.  Returns dict(nodes, elements, cutting_flags,
    fixed_flags, tl, outline).  ``grading`` is d(size)/d(distance)."""
    from scipy.spatial import Delaunay

    o = tool_outline(tl, length, height, rake_deg, clearance_deg, r)
    edge = np.array(o["p"], float)

    def size_fn(q):
        d = float(np.hypot(*(np.asarray(q, float) - edge))) - r
        return float(min(s_max, s_min + grading * max(d, 0.0)))

    pts, sides = [], []
    # outline counter-clockwise: tl -> bl -> blc -> arc -> trc -> tr -> tl
    for a, b, sd in ((o["tl"], o["bl"], SIDE_LEFT), (o["bl"], o["blc"], SIDE_FLANK)):
        p_, s_ = _sample_segment(a, b, size_fn, sd)
        pts += p_
        sides += s_
    if r > 0.0:
        pc = o["p"]
        a0 = math.atan2(o["blc"][1] - pc[1], o["blc"][0] - pc[0])
        a1 = math.atan2(o["trc"][1] - pc[1], o["trc"][0] - pc[0])
        p_, s_ = _sample_arc(pc, r, a0, a1, size_fn, SIDE_ARC)
        pts += p_
        sides += s_
    for a, b, sd in ((o["trc"], o["tr"], SIDE_RAKE), (o["tr"], o["tl"], SIDE_TOP)):
        p_, s_ = _sample_segment(a, b, size_fn, sd)
        pts += p_
        sides += s_
    bnd = np.array(pts)
    nb = len(bnd)
    # side membership: every boundary point belongs to its segment and, at a
    # corner, also to the previous one
    member = [set([s]) for s in sides]
    for k in range(nb):
        if k == 0 or sides[k] != sides[k - 1]:
            member[k].add(sides[k - 1])
    # interior points: triangular lattices, one level per size octave
    poly = bnd
    xmin, ymin = poly.min(0)
    xmax, ymax = poly.max(0)
    rng = np.random.default_rng(seed)

    def inside(q, margin):
        # convex polygon (counter-clockwise): inside if left of every edge by margin
        e0 = poly
        e1 = np.roll(poly, -1, axis=0)
        cr = (e1[:, 0] - e0[:, 0]) * (q[:, None, 1] - e0[:, 1]) - (e1[:, 1] - e0[:, 1]) * (q[:, None, 0] - e0[:, 0])
        ln = np.hypot(e1[:, 0] - e0[:, 0], e1[:, 1] - e0[:, 1])
        return np.all(cr / np.maximum(ln, 1e-300) >= margin[:, None], axis=1)

    interior = []
    level = s_min
    while level <= s_max * 1.0001 + 1e-15:
        dy = level * math.sqrt(3) / 2
        ys = np.arange(ymin + 0.5 * dy, ymax, dy)
        cand = []
        for j, y in enumerate(ys):
            off = 0.5 * level if j % 2 else 0.0
            xs = np.arange(xmin + off, xmax, level)
            cand.append(np.stack([xs, np.full_like(xs, y)], 1))
        cand = np.concatenate(cand) if cand else np.zeros((0, 2))
        if len(cand):
            d = np.hypot(cand[:, 0] - edge[0], cand[:, 1] - edge[1]) - r
            s = np.minimum(s_max, s_min + grading * np.maximum(d, 0.0))
            last = level * 2 > s_max * 1.0001
            keep = (s >= level) & ((s < 2 * level) | last)
            cand = cand[keep]
            s = s[keep]
            if len(cand):
                ok = inside(cand, 0.6 * s)
                cand = cand[ok]
                interior.append(cand)
        level *= 2
    inter = np.concatenate(interior) if interior else np.zeros((0, 2))
    if len(inter):
        jit = (rng.random(inter.shape) - 0.5) * 1e-3
        inter = inter + jit * np.array([[s_min, s_min]])
    nodes = np.concatenate([bnd, inter])
    tri = Delaunay(nodes).simplices.astype(np.int64)
    # orient counter-clockwise, drop degenerate triangles
    P = nodes[tri]
    area2 = (P[:, 1, 0] - P[:, 0, 0]) * (P[:, 2, 1] - P[:, 0, 1]) - (P[:, 2, 0] - P[:, 0, 0]) * (P[:, 1, 1] - P[:, 0, 1])
    tri = np.where((area2 < 0)[:, None], tri[:, [0, 2, 1]], tri)
    tri = tri[np.abs(area2) > 1e-10 * s_min * s_min]
    # boundary edges (appear in one triangle only) and their side
    flags_cut = np.zeros((len(tri), 3), np.int32)
    flags_fix = np.zeros((len(tri), 3), np.int32)
    edges = {}
    for e, t in enumerate(tri):
        for k in range(3):
            a, b = int(t[k]), int(t[(k + 1) % 3])
            key = (min(a, b), max(a, b))
            edges.setdefault(key, []).append((e, k))
    for (a, b), occ in edges.items():
        if len(occ) != 1 or a >= nb or b >= nb:
            continue
        common = member[a] & member[b]
        if not common:
            continue
        e, k = occ[0]
        if common & set(CUTTING_SIDES):
            flags_cut[e, k] = 1
        if common & set(FIXED_SIDES):
            flags_fix[e, k] = 1
    return dict(nodes=np.ascontiguousarray(nodes, np.float64), elements=np.ascontiguousarray(tri, np.int32),
                cutting_flags=flags_cut, fixed_flags=flags_fix, tl=np.array(o["tl"], float), outline=o)


# ---- Abaqus .inp meshes (mesh_structure_GPU.cu:784-1257 mesh_read) ---------------------------------
def _ints(line: str):
    return [int(t) for t in line.replace(" ", "").split(",") if t.strip()]


def _edge_flags(tri, nodes_in_set):
    """Edge flags of boundary elements: edge (a,b) -> 0, (b,c) -> 1, (c,a) -> 2 is
    flagged when both of its nodes are in the node set."""
    a, b, c = (int(v) in nodes_in_set for v in tri)
    return [int(a and b), int(b and c), int(c and a)]


def _correct_full(flags, elements, boundary, full):
    """Elements with all three edges flagged (mesh_structure_GPU.cu:862-890): the
    edge opposite a node that no other boundary element shares is unflagged."""
    for e in full:
        others = [b for b in boundary if b != e]
        for k, opp in ((0, 1), (1, 2), (2, 0)):
            node = elements[e][k]
            if not any(node in elements[b][:3] for b in others):
                flags[e][opp] = 0


def read_inp(path: str, scale: float = 0.01, tl=(0.0, 0.0)) -> dict:
    """Tool mesh from an Abaqus-style .inp file, as mesh_read reads it: '*Node'
    lines 'id, x, y' (coordinates times `scale`, 1/100 in the reference), an
    'Element' header and lines 'id, n1, n2, n3' (1-based), node sets ('Nset')
    and element sets ('Elset') named 'CuttingEdge' and 'FixedBoundary', 'End'.
    Lines containing '#' are skipped.  Returns the dict ``mesh_tool`` returns
    (nodes, elements, cutting_flags, fixed_flags, tl); `tl` is the tool's
    top-left reference point (tool_FEM ctor), not part of the file."""
    nodes, elements = [], []
    cut_nodes, fix_nodes = set(), set()
    cut_elems, fix_elems = [], []
    mode = None
    with open(path) as f:
        for line in f:
            if "#" in line:
                continue
            if "*Node" in line:
                mode = "node"
                continue
            if "Element" in line:
                mode = "elem"
                continue
            if "CuttingEdge" in line and "Nset" in line:
                mode = "cut_nodes"
                continue
            if "CuttingEdge" in line and "Elset" in line:
                mode = "cut_elems"
                continue
            if "FixedBoundary" in line and "Nset" in line:
                mode = "fix_nodes"
                continue
            if "FixedBoundary" in line and "Elset" in line:
                mode = "fix_elems"
                continue
            if "End" in line:
                break
            if not line.strip():
                continue
            if mode == "node":
                t = [s for s in line.split(",")]
                nodes.append((float(t[1]) * scale, float(t[2]) * scale))
            elif mode == "elem":
                v = _ints(line)
                elements.append([v[1] - 1, v[2] - 1, v[3] - 1])
            elif mode == "cut_nodes":
                cut_nodes.update(v - 1 for v in _ints(line))
            elif mode == "cut_elems":
                cut_elems += [v - 1 for v in _ints(line)]
            elif mode == "fix_nodes":
                fix_nodes.update(v - 1 for v in _ints(line))
            elif mode == "fix_elems":
                fix_elems += [v - 1 for v in _ints(line)]
    n_el = len(elements)
    cut = [[0, 0, 0] for _ in range(n_el)]
    fix = [[0, 0, 0] for _ in range(n_el)]
    for flags, boundary, in_set in ((cut, cut_elems, cut_nodes), (fix, fix_elems, fix_nodes)):
        full = []
        for e in boundary:
            flags[e] = _edge_flags(elements[e], in_set)
            if all(flags[e]):
                full.append(e)
        _correct_full(flags, elements, boundary, full)
    return dict(nodes=np.ascontiguousarray(nodes, np.float64), elements=np.ascontiguousarray(elements, np.int32),
                cutting_flags=np.ascontiguousarray(cut, np.int32), fixed_flags=np.ascontiguousarray(fix, np.int32),
                tl=np.array(tl, float))


def write_inp(mesh: dict, path: str, scale: float = 0.01):
    """Writes a mesh in the layout ``read_inp`` reads (coordinates divided by
    `scale`); the boundary sets are the nodes and elements of flagged edges."""
    nodes, el = mesh["nodes"], mesh["elements"]
    with open(path, "w") as f:
        f.write("*Heading\n*Node\n")
        for i, (x, y) in enumerate(nodes):
            f.write(f"{i + 1}, {x / scale:.17g}, {y / scale:.17g}\n")
        f.write("*Element, type=CPS3\n")
        for i, (a, b, c) in enumerate(el):
            f.write(f"{i + 1}, {a + 1}, {b + 1}, {c + 1}\n")
        for name, key in (("CuttingEdge", "cutting_flags"), ("FixedBoundary", "fixed_flags")):
            fl = mesh[key]
            elems = [i for i in range(len(el)) if fl[i].any()]
            nds = set()
            for i in elems:
                a, b, c = el[i]
                for k, (p, q) in enumerate(((a, b), (b, c), (c, a))):
                    if fl[i][k]:
                        nds.update((int(p), int(q)))
            f.write(f"*Nset, nset={name}\n")
            ids = sorted(n + 1 for n in nds)
            for k in range(0, len(ids), 16):
                f.write(", ".join(str(v) for v in ids[k:k + 16]) + "\n")
            f.write(f"*Elset, elset={name}\n")
            ids = [i + 1 for i in elems]
            for k in range(0, len(ids), 16):
                f.write(", ".join(str(v) for v in ids[k:k + 16]) + "\n")
        f.write("*End Part\n")
