// fem.cuh -- per-node and per-segment bodies of the FEM tool's explicit
// thermal update and of the tool motion, shared by their kernels (fem.cu) and
// the persistent step kernel (persistent.cu).
#pragma once

#include "launch.cuh"

namespace sphfem {

// Robin terms of node i (FEM_thermal_gpu.cu:342-386): rhs and diagonal additions.
__device__ __forceinline__ void robin_terms(const KConsts &K, const FemDev &F, const SegDev &seg, int i, double &df,
                                            double &dk) {
    df = 0.;
    dk = 0.;
    for (int t = F.node_seg_ptr[i]; t < F.node_seg_ptr[i + 1]; t++) {
        int s = F.node_seg[t];
        double2 hx = seg.heat_exchange[s];
        if (hx.y == 0) continue;
        double T_cont_particle = hx.x / hx.y;
        double fric_eng = seg.fric_heat[s];
        double2 l = seg.left[s], r = seg.right[s];
        double ddx = l.x - r.x, ddy = l.y - r.y;
        double dist = sqrtf_d(ddx * ddx + ddy * ddy);
        df += 0.5 * K.c.tool.h * dist * T_cont_particle + 0.5 * fric_eng;
        dk += K.c.tool.h * (0.5 * dist);
    }
}

// calculate_temp(0.5*dt) at the start of the step (FEM_thermal_gpu.cu:460-468,
// with T_old == T right after reset_FEM_server): T_half = 0.5 dt k + T.
// Time step of the case a node belongs to (one case unless batched).
__device__ __forceinline__ const ToolDev &node_case(const KConsts &K, const ToolDev *tool, int i) {
    return tool[K.case_of_node ? K.case_of_node[i] : 0];
}

__device__ __forceinline__ void fem_half_one(int i, const KConsts &K, const FemDev &F,
                                             const ToolDev *__restrict__ tool) {
    F.T_half[i] = node_case(K, tool, i).hdt * F.k[i] + F.T[i];
}

// apply_robin_bdc + calculate_temp_rate + calculate_temp(dt), one row per
// thread (FEM_thermal_gpu.cu:342-386,443-468).  Reads T_half, writes k and T.
__device__ __forceinline__ void fem_rate_update_one(int i, const KConsts &K, const FemDev &F, const SegDev &seg,
                                                    const ToolDev *__restrict__ tool) {
    const double dt = node_case(K, tool, i).dt;
    double df, dk;
    robin_terms(K, F, seg, i, df, dk);
    double buffer = 0.;
    for (int t = F.row_ptr[i]; t < F.row_ptr[i + 1]; t++) {
        int c = F.col_ind[t];
        double kij = F.K[t];
        if (c == i) kij += dk;
        buffer += kij * F.T_half[c];
    }
    double k = F.M_inv[i] * ((F.f[i] + df) - buffer);
    F.k[i] = k;
    F.T[i] = dt * k + F.T[i];
}

// tool_FEM.cu:119-139 do_segments_update: y + v.y dt + flank_retreat, evaluated
// left to right (flank_retreat is 0 without wear).
__device__ __forceinline__ double seg_y_move(double y, double vy, double dt, double fr) {
    return __dadd_rn(__dadd_rn(y, __dmul_rn(vy, dt)), fr);
}
__device__ __forceinline__ void segment_move(const SegDev &seg, int s, const double *vel, double dt, double fr) {
    double2 l = seg.left[s], r = seg.right[s];
    seg.left[s] = make_double2(add_mul_rn(l.x, vel[0], dt), seg_y_move(l.y, vel[1], dt, fr));
    seg.right[s] = make_double2(add_mul_rn(r.x, vel[0], dt), seg_y_move(r.y, vel[1], dt, fr));
    seg.heat_exchange[s] = make_double2(0., 0.);
    seg.fric_heat[s] = 0.;
}

// tool_FEM.cu:109-117 do_tool_update_FEM_gpu + the host bookkeeping of
// tool_update_FEM_gpu (tool_FEM.cu:1555-1559), kept on the device.
// position.y += v.y dt + flank_retreat (tool_FEM.cu:115)
__device__ __forceinline__ void node_move(const FemDev &F, int i, const double *vel, double dt, double fr) {
    double2 p = F.position[i];
    double dy = __dadd_rn(__dmul_rn(vel[1], dt), fr);
    F.position[i] = make_double2(add_mul_rn(p.x, vel[0], dt), __dadd_rn(p.y, dy));
}

__device__ __forceinline__ void tool_state_move(ToolDev *tool, double dt) {
    const double vx = tool->vel[0], vy = tool->vel[1];
    tool->tl_point_ref[0] = add_mul_rn(tool->tl_point_ref[0], vx, dt);
    tool->tl_point_ref[1] = add_mul_rn(tool->tl_point_ref[1], vy, dt);
    tool->br_point[0] = add_mul_rn(tool->br_point[0], vx, dt);
    tool->br_point[1] = add_mul_rn(tool->br_point[1], vy, dt);
    tool->lowest_point = add_mul_rn(tool->lowest_point, vy, dt);
    tool->right_point = add_mul_rn(tool->right_point, vx, dt);
    tool->flank_contact = tool->lowest_point;   // tool_FEM.cu:1567-1569
}

// The segments' y-range of a case, moved with segment_move's arithmetic.
__device__ __forceinline__ void tool_range_move(ToolDev &t, double dt) {
    t.seg_ymin = seg_y_move(t.seg_ymin, t.vel[1], dt, t.flank_retreat);
    t.seg_ymax = seg_y_move(t.seg_ymax, t.vel[1], dt, t.flank_retreat);
    t.seg_xmax = add_mul_rn(t.seg_xmax, t.vel[0], dt);
}

// A case's tool state and segment y-range (what = 3 of tool_move_one for that case).
__device__ __forceinline__ void tool_case_move(ToolDev &t, double dt) {
    tool_state_move(&t, dt);
    tool_range_move(t, dt);
}

// what = 1: segments only; 2: nodes + tool state only; 3: both.  With
// per_case the velocity and time step of each segment's / node's case are
// used (the fused step, batched or not); otherwise case 0 with `dt`.
__device__ __forceinline__ void tool_move_one(int i, const KConsts &K, const SegDev &seg, const FemDev &F,
                                              ToolDev *tool, double dt, int what, int per_case) {
    if ((what & 1) && i < seg.n) {
        const ToolDev &tc = tool[(per_case && K.case_of_seg) ? K.case_of_seg[i] : 0];
        segment_move(seg, i, tc.vel, per_case ? tc.dt : dt, tc.flank_retreat);
    }
    if ((what & 2) && i < F.n_nodes) {
        const ToolDev &tc = tool[(per_case && K.case_of_node) ? K.case_of_node[i] : 0];
        node_move(F, i, tc.vel, per_case ? tc.dt : dt, tc.flank_retreat);
    }
    if ((what & 2) && i < (per_case ? K.n_cases : 1)) tool_state_move(tool + i, per_case ? tool[i].dt : dt);
    if ((what & 1) && i < (per_case ? K.n_cases : 1)) tool_range_move(tool[i], per_case ? tool[i].dt : dt);
}

}  // namespace sphfem
