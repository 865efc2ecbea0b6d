// wear.cu -- tool wear by nodal shift (WEAR_NODE_SHIFT): wear_adjustment of the
// reference (actions_gpu.cu:1009-1020) on the device.
//
// The reference adds and removes the element matrices of the two cutting-edge
// layers colour by colour (do_mesh_adjustment_wear, FEM_thermal_gpu.cu:476-577)
// and shifts the nodes with atomics (tool_FEM.cu:423-430).  Here every node of
// a layer element gathers the contributions of its own layer elements into its
// own mass entry and CSR row, and every cutting-edge node adds the shifts of
// the segments ending on it in segment order: the same sums, without atomics
// or colour launches, in a fixed order.
#include "launch.cuh"
#include "p1elem.h"

namespace sphfem {

// Lumped mass and stiffness of every layer element at the current node
// positions (do_mass_ele_matrix_construction_p1q3 /
// do_stiffness_ele_matrix_construction_p1q3), one element per thread.
__global__ void __launch_bounds__(kBlock) k_wear_elements(KConsts K, FemDev F, WearDev W, double *__restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= W.n_elem) return;
    const int4 el = W.elements[W.elem[k]];
    const double2 p0 = F.position[el.x], p1 = F.position[el.y], p2 = F.position[el.z];
    double m, ke[3][3];
    p1_element(p0.x, p0.y, p1.x, p1.y, p2.x, p2.y, K.c.tool.cp, K.c.tool.rho, K.c.tool.k, m, ke);
    double *o = out + 10 * (size_t)k;
    o[0] = m;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) o[1 + 3 * a + b] = ke[a][b];
}

// mesh_retreat_wear then mesh_resume_wear (FEM_thermal_gpu.cu:923-950) for the
// layer nodes: each node takes its layer elements' contributions at the old
// positions out of its mass entry and CSR row, then puts them back at the new
// positions, and rebuilds its lumped inverse mass (do_inverse_mass_matrix_lumped,
// FEM_thermal_gpu.cu:326-331; the other nodes' entries do not change).
__global__ void __launch_bounds__(kBlock) k_wear_layers(FemDev F, WearDev W) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= W.n_nodes) return;
    const int i = W.node[idx];
    const int t0 = W.adj_ptr[idx], t1 = W.adj_ptr[idx + 1];
    double Mi = F.M[i];
    for (int pass = 0; pass < 2; pass++) {
        const double sign = pass ? 1. : -1.;
        const double *mat = pass ? W.mat_new : W.mat_old;
        for (int t = t0; t < t1; t++) {
            const int4 ad = W.adj[t];
            const double *o = mat + 10 * (size_t)ad.x;
            Mi += sign * o[0];
            const int4 sl = W.slot[t];
            const int a = ad.y;
            F.K[sl.x] += sign * o[1 + 3 * a + 0];
            F.K[sl.y] += sign * o[1 + 3 * a + 1];
            F.K[sl.z] += sign * o[1 + 3 * a + 2];
        }
    }
    F.M[i] = Mi;
    F.M_inv[i] = 1. / Mi;
}

// do_nodal_shift_wear_smooth_temp (tool_FEM.cu:299-432) with RESTRICT_WEAR_TEMP and
// USE_USUI_RAKE_FLANK, one segment per thread: the wear depth of its left and
// right node from the segment's mean pressure and sliding speed and the nodal
// temperatures, and the shift along the segment normal (nodal_shift,
// tool_FEM.cu:49-55).  The shift is applied by k_wear_node_shift.
__global__ void __launch_bounds__(kBlock) k_wear_segment_shift(FemDev F, SegDev seg, WearDev W, double dt) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= seg.n) return;
    W.seg_delta[s] = mk4(0., 0., 0., 0.);
    const dbl4 w = seg.wear.pp[s];
    if (w.x == 0.) return;
    const int4 mk = seg.marks[s];
    double pressure = w.y / w.x;
    double vel = w.z / w.x;
    double Tl = F.T[mk.z], Tr = F.T[mk.w];
    if (vel > 0.008) return;
    Tl = fmin(Tl, 1350.);
    Tr = fmin(Tr, 1350.);
    vel = fmin(vel, 0.008);
    pressure = fmin(pressure, 0.04);
    const double2 n = seg.normal[s];
    double wl, wr;
    if (fabs(n.x) > 0.85) {   // rake face
        wl = dt * W.C * pressure * vel * exp(-W.D / Tl);
        wr = dt * W.C * pressure * vel * exp(-W.D / Tr);
    } else {                  // flank face
        wl = dt * W.A * pressure * vel * exp(-W.B / Tl);
        wr = dt * W.A * pressure * vel * exp(-W.B / Tr);
    }
    seg.wear_rate[s] = (wl + wr) / dt;
    W.seg_delta[s] = mk4(n.x * wl, n.y * wl, n.x * wr, n.y * wr);
}

// Each node adds the shifts of the segments ending on it, in segment order.
__global__ void __launch_bounds__(kBlock) k_wear_node_shift(FemDev F, SegDev seg, WearDev W) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.n_nodes) return;
    const int t0 = F.node_seg_ptr[i], t1 = F.node_seg_ptr[i + 1];
    if (t0 == t1) return;
    double2 p = F.position[i];
    for (int t = t0; t < t1; t++) {
        const int s = F.node_seg[t];
        const int4 mk = seg.marks[s];
        const dbl4 d = W.seg_delta[s];
        if (mk.z == i) {
            p.x += d.x;
            p.y += d.y;
        }
        if (mk.w == i) {
            p.x += d.z;
            p.y += d.w;
        }
    }
    F.position[i] = p;
}

// do_segment_wear_update (tool_FEM.cu:520-545): segments follow their nodes;
// do_correct_flank_contact (tool_FEM.cu:559-587): flank_retreat = flank_contact
// - the lowest left end among the first 512 segments (the reference reduces
// over one block of 512 threads); and the segments' bounds that the contact
// search's exact prefilters use.  One block.
constexpr int kFlankSegments = 512;
constexpr int kFlankThreads = 256;
__global__ void __launch_bounds__(kFlankThreads) k_wear_segments_flank(FemDev F, SegDev seg, ToolDev *tool) {
    __shared__ double s_min[kFlankThreads], s_ymin[kFlankThreads], s_ymax[kFlankThreads], s_xmax[kFlankThreads],
        s_dxdy[kFlankThreads];
    double mn = 3.402823466385288598e38, ymin = INFINITY, ymax = -INFINITY, xmax = -INFINITY, dxdy = 0.;
    for (int s = threadIdx.x; s < seg.n; s += blockDim.x) {
        const int4 mk = seg.marks[s];
        const double2 l = F.position[mk.z], r = F.position[mk.w];
        seg.left[s] = l;
        seg.right[s] = r;
        const double dx = r.x - l.x, dy = r.y - l.y;
        const double inv = 1. / sqrt(dy * dy + dx * dx);   // glm::normalize(vec2(dy, -dx))
        seg.normal[s] = make_double2(dy * inv, -dx * inv);
        if (s < kFlankSegments) mn = fmin(mn, l.y);
        ymin = fmin(ymin, fmin(l.y, r.y));
        ymax = fmax(ymax, fmax(l.y, r.y));
        xmax = fmax(xmax, fmax(l.x, r.x));
        if (l.y != r.y) dxdy = fmax(dxdy, 1.01 * fabs(l.x - r.x) / fabs(l.y - r.y));
    }
    const int t = threadIdx.x;
    s_min[t] = mn; s_ymin[t] = ymin; s_ymax[t] = ymax; s_xmax[t] = xmax; s_dxdy[t] = dxdy;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (t < o) {
            s_min[t] = fmin(s_min[t], s_min[t + o]);
            s_ymin[t] = fmin(s_ymin[t], s_ymin[t + o]);
            s_ymax[t] = fmax(s_ymax[t], s_ymax[t + o]);
            s_xmax[t] = fmax(s_xmax[t], s_xmax[t + o]);
            s_dxdy[t] = fmax(s_dxdy[t], s_dxdy[t + o]);
        }
        __syncthreads();
    }
    if (t == 0) {
        tool->flank_retreat = tool->flank_contact - s_min[0];
        tool->seg_ymin = s_ymin[0];
        tool->seg_ymax = s_ymax[0];
        tool->seg_xmax = s_xmax[0];
        tool->seg_dxdy = s_dxdy[0];
    }
}

// ---- host launchers -------------------------------------------------------------------------------
void launch_wear_reset(cudaStream_t s, const SegDev &seg) {
    cudaMemsetAsync(seg.wear.pp, 0, sizeof(dbl4) * (size_t)seg.n, s);
    cudaMemsetAsync(seg.wear.sf, 0, sizeof(double) * (size_t)seg.n, s);
    cudaMemsetAsync(seg.wear_rate, 0, sizeof(double) * (size_t)seg.n, s);
}

// Few hundred threads of FP64 element work: blocks as small as needed to
// spread them over the SMs (fp64_block).
void launch_wear_adjustment(cudaStream_t s, const KConsts &K, const FemDev &F, const SegDev &seg, const WearDev &W,
                            ToolDev *tool, double dt) {
    const int ne = W.n_elem > 0 ? W.n_elem : 1, nl = W.n_nodes > 0 ? W.n_nodes : 1, ns = seg.n > 0 ? seg.n : 1;
    const int be = fp64_block(ne), bl = fp64_block(nl), bs = fp64_block(ns), bn = fp64_block(F.n_nodes);
    k_wear_elements<<<div_up(ne, be), be, 0, s>>>(K, F, W, W.mat_old);
    k_wear_segment_shift<<<div_up(ns, bs), bs, 0, s>>>(F, seg, W, dt);
    k_wear_node_shift<<<div_up(F.n_nodes, bn), bn, 0, s>>>(F, seg, W);
    k_wear_elements<<<div_up(ne, be), be, 0, s>>>(K, F, W, W.mat_new);
    k_wear_layers<<<div_up(nl, bl), bl, 0, s>>>(F, W);
    k_wear_segments_flank<<<1, kFlankThreads, 0, s>>>(F, seg, tool);
}

// ---- remesh_low_level (tool_FEM.cu:1696-1705) -----------------------------------------------
// do_mesh_shift (tool_FEM.cu:589-616): the nodes on neither the cutting nor the
// fixed edge follow the flank wear -- a shift of at least 6.5e-6 cm, weighted by
// the node's place between the tool's top-left and bottom-right points.
__global__ void __launch_bounds__(kBlock) k_mesh_shift(int N, int freq, double2 *__restrict__ pos,
                                                       const int32_t *__restrict__ node_edge,
                                                       const ToolDev *__restrict__ tool) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N || node_edge[i] != 0) return;
    const ToolDev &t = tool[0];
    double shift_value = t.flank_retreat * 1.0 * freq;
    shift_value = fmin(shift_value, -0.0000065);
    const double2 p = pos[i];
    const double tlx = t.tl_point_ref[0], tly = t.tl_point_ref[1], brx = t.br_point[0], bry = t.br_point[1];
    const double weight_y = (p.x - tlx) / (brx - tlx);
    const double weight_x = fmin(1.0, (p.y - tly) / (bry - tly));
    const double center_KT = 0.94;
    double x = p.x, y = p.y;
    if (weight_x <= center_KT)
        x += 1.45 * shift_value * (pow(center_KT, 0.7) - pow(fabs(weight_x - center_KT), 0.55)) * weight_y * weight_y *
             weight_y;
    else if (weight_x < 1.1 && weight_x > center_KT)
        x += 1.45 * shift_value * (pow(center_KT, 0.7) - pow(fabs(weight_x - center_KT), 0.55)) * weight_y * weight_y;
    if (weight_y < 1.01)
        y += -0.9 * shift_value * fmin(pow(weight_y, 6), 1.) * pow(weight_x, 6);
    else if (weight_y >= 0.99)
        y += -0.9 * shift_value * fmin(pow(weight_y, 6), 1.) * weight_x * weight_x * weight_x * weight_x;
    pos[i] = make_double2(x, y);
}

// do_nodal_value_interpolation_old + value_interpolation_in_layer_element
// (tool_FEM.cu:57-107,434-443): each node's new temperature from the first
// element of the old mesh (in element order) that holds its new position, by
// the barycentric weights of that element; its old value when none does.
__global__ void __launch_bounds__(kBlock) k_nodal_interpolation(int N, int n_elem, const int4 *__restrict__ elements,
                                                                const double2 *__restrict__ pos_old,
                                                                const double *__restrict__ T_old,
                                                                const double2 *__restrict__ pos,
                                                                double *__restrict__ T) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const double2 x_ = pos[i];
    auto cross = [](double ax, double ay, double bx, double by) { return ax * by - ay * bx; };
    for (int e = 0; e < n_elem; e++) {
        const int4 el = elements[e];
        const double2 xA = pos_old[el.x];
        const double xBx = pos_old[el.y].x - xA.x, xBy = pos_old[el.y].y - xA.y;
        const double xCx = pos_old[el.z].x - xA.x, xCy = pos_old[el.z].y - xA.y;
        const double xPx = x_.x - xA.x, xPy = x_.y - xA.y;
        const double xBCx = xBx - xCx, xBCy = xBy - xCy;
        const double d = cross(xBx, xBy, xCx, xCy);
        if (fabs(d) > 1e-13) {
            const double wA = cross(xBx, xBy, xCx, xCy) + cross(xPx, xPy, xBCx, xBCy);
            const double wB = cross(xPx, xPy, xCx, xCy);
            const double wC = -cross(xPx, xPy, xBx, xBy);
            if (wA >= 0 && wB >= 0 && wC >= 0 && wA <= 1 && wB <= 1 && wC <= 1) {
                T[i] = (T_old[el.x] * wA + T_old[el.y] * wB + T_old[el.z] * wC) / d;
                return;
            }
        }
    }
    T[i] = T_old[i];
}

void launch_remesh_low_level(cudaStream_t s, const FemDev &F, const int4 *elements, int n_elem, int n_colors,
                             const int32_t *node_edge, const ToolDev *tool, int freq, const int32_t *dir_elems,
                             const int4 *dir_flags, int n_dir, const sph_tool_constants &tc, double2 *pos_old,
                             double *T_old) {
    // mapping_data_copy (tool_FEM.cu:1611-1622)
    cudaMemcpyAsync(pos_old, F.position, sizeof(double2) * (size_t)F.n_nodes, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(T_old, F.T, sizeof(double) * (size_t)F.n_nodes, cudaMemcpyDeviceToDevice, s);
    k_mesh_shift<<<div_up(F.n_nodes, kBlock), kBlock, 0, s>>>(F.n_nodes, freq, F.position, node_edge, tool);
    // reset_FEM_matrix + stiffness_mass_matrix_construction + dirichlet_bdc + inverse_mass_matrix
    launch_fem_assemble(s, F, elements, n_elem, n_colors, dir_elems, dir_flags, n_dir, tc.cp, tc.rho, tc.k, tc.T0,
                        F.M);
    k_nodal_interpolation<<<div_up(F.n_nodes, kBlock), kBlock, 0, s>>>(F.n_nodes, n_elem, elements, pos_old, T_old,
                                                                       F.position, F.T);
}

}  // namespace sphfem
