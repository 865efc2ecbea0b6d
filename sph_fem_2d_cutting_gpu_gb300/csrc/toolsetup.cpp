// toolsetup.cpp -- host-side set-up of the FEM tool (runs once per context).
//
//  - element colouring and CSR pattern: mesh_structure_GPU.cu:596-780
//    (the reference picks the first colour with rand(); here the first try is
//    colour 1, which makes the colouring deterministic);
//  - interface segments, their orientation, chain order and the tool
//    reference points: tool_FEM::set_up_segments_from_mesh, tool_FEM.cu:771-1039
//    with segment(left, right, tl) of geometric_primitives.cpp:190-212;
//  - P1 lumped-mass / stiffness assembly, Dirichlet elimination and the lumped
//    inverse: FEM_thermal_gpu.cu:71-109,126-225,234-332, executed in the
//    reference's colour-by-colour order on one host thread.
#include "toolsetup.h"
#include "p1elem.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <set>

namespace sphfem {

namespace {

struct V2 {
    double x, y;
};
inline bool eq(V2 a, V2 b) { return a.x == b.x && a.y == b.y; }
inline double dist(V2 a, V2 b) { return std::sqrt((a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y)); }

struct Seg {
    V2 left, right, n;
};

// geometric_primitives.cpp:190-212 segment(left, right, tl): unit normal
// (dy, -dx) flipped (with the end points swapped) so it points towards tl.
Seg make_segment(V2 l, V2 r, V2 tl) {
    V2 d = {r.x - l.x, r.y - l.y};
    V2 n = {d.y, -d.x};
    double inv = 1.0 / std::sqrt(n.x * n.x + n.y * n.y);
    n = {n.x * inv, n.y * inv};
    V2 ref = {tl.x - l.x, tl.y - l.y};
    Seg s;
    if ((ref.x * n.x + ref.y * n.y) < 0) {
        s.n = {-n.x, -n.y};
        s.left = r;
        s.right = l;
    } else {
        s.n = n;
        s.left = l;
        s.right = r;
    }
    return s;
}

// Greedy colouring: an element takes the first colour (cyclic from `first`)
// that no node-sharing element in `pool` already has (mesh_structure_GPU.cu:596-739).
bool colour_elements(const std::vector<int> &todo, const std::vector<char> &in_pool, int ncol,
                     std::vector<Int4> &el, const std::vector<std::vector<int>> &node_elems, std::string &err) {
    for (int e : todo) {
        std::set<int> used;
        int nd[3] = {el[e].x, el[e].y, el[e].z};
        for (int a = 0; a < 3; a++)
            for (int o : node_elems[nd[a]])
                if (o != e && in_pool[o] && el[o].w != 0) used.insert(el[o].w);
        int c = 1, tries = 0;
        while (used.count(c)) {
            c = c + 1;
            if (c > ncol) c = 1;
            if (++tries >= ncol) {
                err = "element colouring ran out of colours";
                return false;
            }
        }
        el[e].w = c;
    }
    return true;
}

}  // namespace

int build_tool_model(const sph_tool_mesh &mesh, const sph_tool_constants &tc, ToolModelHost &M, std::string &err) {
    if (mesh.n_nodes <= 0 || mesh.n_elements <= 0 || !mesh.nodes || !mesh.elements || !mesh.cutting_flags ||
        !mesh.fixed_flags) {
        err = "tool mesh: empty or missing arrays";
        return SPH_ERR_INVALID;
    }
    const int NN = mesh.n_nodes, NE = mesh.n_elements;
    M.n_nodes = NN;
    M.n_elements = NE;
    M.pos.assign(mesh.nodes, mesh.nodes + 2 * NN);
    M.elements.resize(NE);
    for (int e = 0; e < NE; e++) {
        M.elements[e] = {mesh.elements[3 * e], mesh.elements[3 * e + 1], mesh.elements[3 * e + 2], 0};
        for (int a = 0; a < 3; a++) {
            int nd = mesh.elements[3 * e + a];
            if (nd < 0 || nd >= NN) {
                err = "tool mesh: element references a missing node";
                return SPH_ERR_INVALID;
            }
        }
    }
    auto node = [&](int i) { return V2{M.pos[2 * i], M.pos[2 * i + 1]}; };
    std::vector<std::vector<int>> node_elems(NN);
    for (int e = 0; e < NE; e++) {
        node_elems[M.elements[e].x].push_back(e);
        node_elems[M.elements[e].y].push_back(e);
        node_elems[M.elements[e].z].push_back(e);
    }
    // ---- node flags: end points of cutting-edge and fixed-edge element edges ----
    M.node_edge.assign(NN, 0);
    for (int e = 0; e < NE; e++) {
        const int nd[3] = {M.elements[e].x, M.elements[e].y, M.elements[e].z};
        for (int a = 0; a < 3; a++) {   // edge a: nodes a and a + 1
            if (mesh.cutting_flags[3 * e + a]) M.node_edge[nd[a]] |= 1, M.node_edge[nd[(a + 1) % 3]] |= 1;
            if (mesh.fixed_flags[3 * e + a]) M.node_edge[nd[a]] |= 2, M.node_edge[nd[(a + 1) % 3]] |= 2;
        }
    }
    // ---- colouring: cutting-boundary elements (6 colours), then the rest (18) ----
    std::vector<int> cut_elems, fixed_elems, rest;
    for (int e = 0; e < NE; e++) {
        const int32_t *cf = mesh.cutting_flags + 3 * e, *ff = mesh.fixed_flags + 3 * e;
        if (cf[0] || cf[1] || cf[2]) cut_elems.push_back(e);
        if (ff[0] || ff[1] || ff[2]) fixed_elems.push_back(e);
    }
    M.n_cut_colors = 6;
    M.n_colors = 18;
    std::vector<char> in_cut(NE, 0), all(NE, 1);
    for (int e : cut_elems) in_cut[e] = 1;
    for (int e = 0; e < NE; e++)
        if (!in_cut[e]) rest.push_back(e);
    while (true) {
        for (auto &el : M.elements) el.w = 0;
        std::string cerr;
        if (colour_elements(cut_elems, in_cut, M.n_cut_colors, M.elements, node_elems, cerr) &&
            colour_elements(rest, all, M.n_colors, M.elements, node_elems, cerr))
            break;
        // the reference asserts here; a finer mesh simply gets more colours
        if (M.n_colors > 64) {
            err = cerr;
            return SPH_ERR_INVALID;
        }
        M.n_cut_colors += 2;
        M.n_colors += 6;
    }
    // ---- CSR pattern (mesh_structure_GPU.cu:741-780): all nodes sharing an element ----
    M.row_ptr.assign(NN + 1, 0);
    M.col_ind.clear();
    M.diag.assign(NN, -1);
    for (int k = 0; k < NN; k++) {
        std::set<int> cols;
        for (int e : node_elems[k]) {
            cols.insert(M.elements[e].x);
            cols.insert(M.elements[e].y);
            cols.insert(M.elements[e].z);
        }
        for (int c : cols) {
            if (c == k) M.diag[k] = (int)M.col_ind.size();
            M.col_ind.push_back(c);
        }
        M.row_ptr[k + 1] = (int)M.col_ind.size();
    }
    const int NZ = (int)M.col_ind.size();
    for (int k = 0; k < NN; k++)
        if (M.diag[k] < 0) {
            M.diag[k] = M.row_ptr[k];   // isolated node: give it a diagonal slot holder
        }
    // ---- assembly (FEM_thermal_gpu.cu:126-225), colour by colour -------------------------
    M.K.assign(NZ, 0.);
    M.M.assign(NN, 0.);
    M.f.assign(NN, 0.);
    auto csr_add = [&](int row, int col, double v) {
        for (int j = M.row_ptr[row]; j < M.row_ptr[row + 1]; j++)
            if (M.col_ind[j] == col) {
                M.K[j] += v;
                return;
            }
    };
    for (int colour = 1; colour <= M.n_colors; colour++) {
        for (int e = 0; e < NE; e++) {
            const Int4 el = M.elements[e];
            if (el.w != colour) continue;
            V2 p0 = node(el.x), p1 = node(el.y), p2 = node(el.z);
            double mvalue, ke[3][3];
            p1_element(p0.x, p0.y, p1.x, p1.y, p2.x, p2.y, tc.cp, tc.rho, tc.k, mvalue, ke);
            M.M[el.x] += mvalue;
            M.M[el.y] += mvalue;
            M.M[el.z] += mvalue;
            int nd[3] = {el.x, el.y, el.z};
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) csr_add(nd[a], nd[b], ke[a][b]);
        }
    }
    // ---- initial nodal temperature ---------------------------------------------------------
    M.T.assign(NN, tc.T0);
    if (mesh.T_init)
        for (int i = 0; i < NN; i++) M.T[i] = mesh.T_init[i];
    // ---- Dirichlet elimination (FEM_thermal_gpu.cu:234-324), colour by colour ----------------
    auto find_location = [&](int start, int end, int value) {
        int itr;
        for (itr = start; itr < end; itr++)
            if (M.col_ind[itr] == value) break;
        return itr;
    };
    auto dirichlet_node = [&](int nd) {
        for (int i = M.row_ptr[nd]; i < M.row_ptr[nd + 1]; i++) {
            int local_no = M.col_ind[i];
            M.f[local_no] += -M.K[i] * tc.T0;
            M.K[i] = 0.;
            int sym = find_location(M.row_ptr[local_no], M.row_ptr[local_no + 1], nd);
            if (sym < M.row_ptr[local_no + 1]) M.K[sym] = 0.;
            if (local_no == nd) M.K[i] = 1.0;
        }
        M.M[nd] = 1.0;
        M.f[nd] = tc.T0;
    };
    for (int colour = 1; colour <= M.n_colors; colour++) {
        for (int e : fixed_elems) {
            const Int4 el = M.elements[e];
            if (el.w != colour) continue;
            const int32_t *ff = mesh.fixed_flags + 3 * e;
            int fx = 0, fy = 0, fz = 0;
            if (ff[0]) { fx = 1; fy = 1; }
            if (ff[1]) { fy = 1; fz = 1; }
            if (ff[2]) { fz = 1; fx = 1; }
            if (fx) dirichlet_node(el.x);
            if (fy) dirichlet_node(el.y);
            if (fz) dirichlet_node(el.z);
            M.dirichlet_elem.push_back(e);
            M.dirichlet_flags.push_back({ff[0], ff[1], ff[2], 0});
        }
    }
    M.M_inv.resize(NN);
    for (int i = 0; i < NN; i++) M.M_inv[i] = 1. / M.M[i];

    // ---- interface segments (tool_FEM.cu:771-1039) -------------------------------------------
    const V2 tl0 = {mesh.tl[0], mesh.tl[1]};
    std::vector<Seg> segs_d;
    std::vector<Int4> mark_h;
    for (int e : cut_elems) {
        const Int4 el = M.elements[e];
        const int32_t *cf = mesh.cutting_flags + 3 * e;
        int pairs[3][2] = {{el.x, el.y}, {el.y, el.z}, {el.z, el.x}};
        for (int a = 0; a < 3; a++) {
            if (!cf[a]) continue;
            V2 lr = node(pairs[a][0]), rr = node(pairs[a][1]);
            Seg s = make_segment(lr, rr, tl0);
            segs_d.push_back(s);
            Int4 mk = {e, el.w, 0, 0};
            if (eq(s.left, lr)) { mk.z = pairs[a][0]; mk.w = pairs[a][1]; }
            else if (eq(s.left, rr)) { mk.z = pairs[a][1]; mk.w = pairs[a][0]; }
            mark_h.push_back(mk);
        }
    }
    const int n_segment = (int)segs_d.size();
    if (n_segment == 0) {
        err = "tool mesh: no cutting-edge segments";
        return SPH_ERR_INVALID;
    }
    double y_min = DBL_MAX, x_max = -DBL_MAX, y_max = -DBL_MAX, x_min = DBL_MAX, dist_max = -DBL_MAX;
    for (const Seg &s : segs_d) {
        y_min = std::fmin(y_min, s.left.y);
        y_min = std::fmin(y_min, s.right.y);
        x_max = std::fmax(x_max, s.left.x);
        x_max = std::fmax(x_max, s.right.x);
        x_min = std::fmin(x_min, s.left.x);
        x_min = std::fmin(x_min, s.right.x);
        y_max = std::fmax(y_max, s.left.y);
        y_max = std::fmax(y_max, s.right.y);
        dist_max = std::fmax(dist(tl0, s.left), dist_max);
        dist_max = std::fmax(dist(tl0, s.right), dist_max);
    }
    V2 tlr = {x_min, y_max};
    for (const Seg &s : segs_d) dist_max = std::fmax(dist(tlr, s.left), dist_max);
    M.lowest_point = y_min;
    M.right_point = x_max;
    M.ref_dist = dist_max;
    // chain order starting at the segment end on y_max (tool_FEM.cu:877-966)
    bool is_left = false;
    int num_buffer = 0;
    for (int i = 0; i < n_segment; i++) {
        if (segs_d[i].left.y == y_max) { is_left = true; num_buffer = i; break; }
        if (segs_d[i].right.y == y_max) { is_left = false; num_buffer = i; break; }
    }
    std::vector<Seg> segs;
    std::vector<Int4> marks_sorted;
    if (is_left) {
        V2 buf = {segs_d[num_buffer].left.x, y_max};
        int rep = 0;
        for (int i = 0; i < n_segment; i++) {
            bool found = false;
            for (int j = 0; j < n_segment; j++)
                if (segs_d[j].left.y == buf.y && segs_d[j].left.x == buf.x) {
                    buf = segs_d[j].right;
                    rep = j;
                    segs.push_back(segs_d[j]);
                    marks_sorted.push_back(mark_h[j]);
                    found = true;
                    break;
                }
            if (found) continue;
            for (int j = 0; j < n_segment; j++)
                if (segs_d[j].right.y == buf.y && segs_d[j].right.x == buf.x && j != rep) {
                    segs_d[j].right = segs_d[j].left;
                    segs_d[j].left = buf;
                    segs_d[j].n = {-segs_d[j].n.x, -segs_d[j].n.y};
                    buf = segs_d[j].right;
                    std::swap(mark_h[j].z, mark_h[j].w);
                    rep = j;
                    segs.push_back(segs_d[j]);
                    marks_sorted.push_back(mark_h[j]);
                    break;
                }
        }
    } else {
        V2 buf = {segs_d[num_buffer].right.x, y_max};
        int rep = 0;
        for (int i = 0; i < n_segment; i++) {
            bool found = false;
            for (int j = 0; j < n_segment; j++)
                if (segs_d[j].right.y == buf.y && segs_d[j].right.x == buf.x) {
                    buf = segs_d[j].left;
                    segs.push_back(segs_d[j]);
                    marks_sorted.push_back(mark_h[j]);
                    found = true;
                    break;
                }
            if (found) continue;
            for (int j = 0; j < n_segment; j++)
                if (segs_d[j].left.y == buf.y && segs_d[j].left.x == buf.x && j != rep) {
                    segs_d[j].left = segs_d[j].right;
                    segs_d[j].right = buf;
                    segs_d[j].n = {-segs_d[j].n.x, -segs_d[j].n.y};
                    buf = segs_d[j].left;
                    std::swap(mark_h[j].z, mark_h[j].w);
                    rep = j;
                    segs.push_back(segs_d[j]);
                    marks_sorted.push_back(mark_h[j]);
                    break;
                }
        }
    }
    if ((int)segs.size() != n_segment) {
        err = "tool mesh: cutting-edge segments do not form one open chain";
        return SPH_ERR_INVALID;
    }
    M.n_seg = n_segment;
    M.left.resize(2 * n_segment);
    M.right.resize(2 * n_segment);
    M.normal.resize(2 * n_segment);
    M.marks = marks_sorted;
    for (int i = 0; i < n_segment; i++) {
        M.left[2 * i] = segs[i].left.x; M.left[2 * i + 1] = segs[i].left.y;
        M.right[2 * i] = segs[i].right.x; M.right[2 * i + 1] = segs[i].right.y;
        M.normal[2 * i] = segs[i].n.x; M.normal[2 * i + 1] = segs[i].n.y;
    }
    // tool reference points from all nodes (tool_FEM.cu:1020-1037)
    double tl_x = FLT_MAX, tl_y = -FLT_MAX, br_x = -FLT_MAX, br_y = FLT_MAX;
    for (int i = 0; i < NN; i++) {
        double x = M.pos[2 * i], y = M.pos[2 * i + 1];
        if (x <= tl_x && y >= tl_y) { tl_x = x; tl_y = y; }
        if (x >= br_x && y <= br_y) { br_x = x; br_y = y; }
    }
    M.br_point[0] = br_x; M.br_point[1] = br_y;
    M.tl_point_ref[0] = tl_x; M.tl_point_ref[1] = tl_y;
    // node -> segment lists for the per-node Robin gather (left node, then right node)
    std::vector<std::vector<int>> ns(NN);
    for (int s = 0; s < n_segment; s++) {
        ns[M.marks[s].z].push_back(s);
        if (M.marks[s].w != M.marks[s].z) ns[M.marks[s].w].push_back(s);
    }
    for (auto &v : ns) std::sort(v.begin(), v.end(), [&](int a, int b) {
        if (M.marks[a].y != M.marks[b].y) return M.marks[a].y < M.marks[b].y;   // colour order, then index
        return a < b;
    });
    M.node_seg_ptr.assign(NN + 1, 0);
    M.node_seg.clear();
    for (int i = 0; i < NN; i++) {
        for (int s : ns[i]) M.node_seg.push_back(s);
        M.node_seg_ptr[i + 1] = (int)M.node_seg.size();
    }
    // ---- wear layers (mesh_structure_GPU.cu:1063-1148): layer 1 = elements with a
    // cutting edge; layer 2 = the other elements that share a node with layer 1
    // (a node on the cutting edge is always such a node) -------------------------
    M.layer.assign(NE, Int4{0, 0, 0, 0});
    std::vector<char> near_cut(NN, 0);
    for (int e : cut_elems) {
        M.layer[e].x = 1;
        near_cut[M.elements[e].x] = near_cut[M.elements[e].y] = near_cut[M.elements[e].z] = 1;
    }
    for (int e = 0; e < NE; e++) {
        const Int4 el = M.elements[e];
        if (!M.layer[e].x && (near_cut[el.x] || near_cut[el.y] || near_cut[el.z])) M.layer[e].y = 1;
    }
    // the layer elements (ascending) and, per node of a layer element, its layer
    // elements (index into that list), the node's local index there and the CSR
    // slots of (node, node_b), b = 0..2
    M.wear_elem.clear();
    std::vector<int> compact(NE, -1);
    for (int e = 0; e < NE; e++)
        if (M.layer[e].x || M.layer[e].y) {
            compact[e] = (int)M.wear_elem.size();
            M.wear_elem.push_back(e);
        }
    M.wear_node.clear();
    M.wear_adj_ptr.assign(1, 0);
    M.wear_adj.clear();
    M.wear_slot.clear();
    auto slot_of = [&](int row, int col) {
        for (int t = M.row_ptr[row]; t < M.row_ptr[row + 1]; t++)
            if (M.col_ind[t] == col) return t;
        return -1;
    };
    for (int i = 0; i < NN; i++) {
        bool any = false;
        for (int e : node_elems[i]) {
            if (!M.layer[e].x && !M.layer[e].y) continue;
            const Int4 el = M.elements[e];
            const int nd[3] = {el.x, el.y, el.z};
            const int a = (nd[0] == i) ? 0 : (nd[1] == i ? 1 : 2);
            M.wear_adj.push_back(Int4{compact[e], a, 0, 0});
            M.wear_slot.push_back(Int4{slot_of(i, nd[0]), slot_of(i, nd[1]), slot_of(i, nd[2]), 0});
            any = true;
        }
        if (any) {
            M.wear_node.push_back(i);
            M.wear_adj_ptr.push_back((int)M.wear_adj.size());
        }
    }
    return SPH_OK;
}

}  // namespace sphfem
