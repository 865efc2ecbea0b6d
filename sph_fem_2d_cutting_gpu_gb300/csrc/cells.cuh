// cells.cuh -- per-element bodies of the cell-list build and the FP32K
// reorder gather, shared by their kernels (cells.cu) and the persistent step
// kernel (persistent.cu).
#pragma once

#include "launch.cuh"

namespace sphfem {

__device__ __forceinline__ float2 f2(double2 v) { return make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ float2 f2(float2 v) { return v; }
__device__ __forceinline__ float4 f4(dbl4 v) { return make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w); }
__device__ __forceinline__ float4 f4(float4 v) { return v; }
__device__ __forceinline__ bool nonfinite4(dbl4 v) {
    return is_nan_or_inf(v.x) || is_nan_or_inf(v.y) || is_nan_or_inf(v.z) || is_nan_or_inf(v.w);
}
__device__ __forceinline__ bool nonfinite4(float4 v) {
    return is_nan_or_inf(v.x) || is_nan_or_inf(v.y) || is_nan_or_inf(v.z) || is_nan_or_inf(v.w);
}

// ---- exclusive scan of the per-cell counts -----------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int block_exclusive_scan(int v, int *smem_warp, int &total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int nw = blockDim.x >> 5;
        int s = (lane < nw) ? smem_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) smem_warp[lane] = s;
    }
    __syncthreads();
    int warp_prefix = (wid > 0) ? smem_warp[wid - 1] : 0;
    total = smem_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
    return warp_prefix + x - v;
}

// ---- scatter into the cell's slot range (arbitrary order inside the cell) -------------
__device__ __forceinline__ void scatter_one(int i, const int32_t *__restrict__ key, const int32_t *__restrict__ arrival,
                                            const int32_t *__restrict__ offsets, int32_t *__restrict__ slots) {
    slots[offsets[key[i]] + arrival[i]] = i;
}

// ---- stable order inside each cell: rank by original index -------------------------------
// perm[k] = original index of the particle that lands at sorted position k
// (the reference's particles->idx after sort_by_key).
__device__ __forceinline__ void rank_one(int s, const int32_t *__restrict__ key, const int32_t *__restrict__ offsets,
                                         const int32_t *__restrict__ slots, int32_t *__restrict__ perm,
                                         uint32_t *status) {
    int i = slots[s];
    int c = key[i];
    int cs = offsets[c], ce = offsets[c + 1];
    if (ce - cs > kCellRankCap && s == cs) set_status(status, SPH_STATUS_CELL_OVERFLOW);
    int rank = 0;
    for (int t = cs; t < ce; t++) rank += (__ldg(slots + t) < i) ? 1 : 0;
    perm[cs + rank] = i;
}

// FP32-compensated form of the fused reorder: the same gather into the compact
// FP32 state (SortedFields32), with the predictor, EOS and artificial stress of
// the predicted state evaluated in FP32 (positions and density stay FP64: rho -
// rho0 is a small difference, FP32 would lose its leading digits) and written
// into the FP32 record.  SF / FF: the state the step starts from -- the FP64
// arrays after an upload or a staged call, the compact arrays after a fused
// step.  p and R of tool particles are kept from FF at the sorted position, as
// the reference leaves them (they are not part of the Green sort's buffer).
template <class SF, class FF>
__device__ __forceinline__ void gather32_one(int k, const int32_t *__restrict__ perm, const KConsts &K, const SF &A,
                                             const FF &Fsrc, const SortedFields32 &B, const FixedFields32 &F,
                                             int32_t *__restrict__ idx, const int32_t *__restrict__ hash_src,
                                             float4 *__restrict__ rec, float2 *__restrict__ cand,
                                             const ToolDev *__restrict__ tools) {
    int i = perm[k];
    idx[k] = i;
    const double2 pos = A.pos[i];
    const float2 vel = f2(A.vel[i]), pos_t = f2(A.pos_t[i]), vel_t = f2(A.vel_t[i]);
    const float4 S = f4(A.S[i]), S_t = f4(A.S_t[i]);
    const double rho = A.rho[i];
    const float T = (float)A.T[i], h = (float)A.h[i], rho_t = (float)A.rho_t[i], T_t = (float)A.T_t[i];
    const float blanked = (float)A.blanked[i], tool = (float)A.tool_particle[i];
    const int hash = hash_src[i];
    B.pos[k] = pos;
    B.vel[k] = vel;
    B.fc[k] = f2(A.fc[i]);
    B.ft[k] = f2(A.ft[i]);
    B.h[k] = h;
    B.n[k] = f2(A.n[i]);
    B.rho[k] = rho;
    B.S[k] = S;
    B.eps_pl[k] = (float)A.eps_pl[i];
    B.eps_pl_dot[k] = (float)A.eps_pl_dot[i];
    B.T[k] = T;
    B.fixed[k] = (float)A.fixed[i];
    B.blanked[k] = blanked;
    B.tool_particle[k] = tool;
    B.pos_t[k] = pos_t;
    B.vel_t[k] = vel_t;
    B.rho_t[k] = rho_t;
    B.S_t[k] = S_t;
    B.T_t[k] = T_t;
    B.on_seg[k] = A.on_seg[i];
    B.hash[k] = hash;
    const bool is_blanked = flag_is_one(blanked), is_tool = flag_nonzero(tool);
    // predictor (leap_frog.cu:45-69)
    double2 pp = pos;
    double rp = rho;
    float vx = vel.x, vy = vel.y;
    float4 Sp = S;
    float Tp = T;
    if (!is_blanked) {
        const ToolDev &tc = tools[case_of_hash(K, hash)];   // time step of the particle's case
        const double hdt = tc.hdt;
        const float hdtf = tc.hdtf;
        pp.x = pos.x + hdt * (double)pos_t.x;
        pp.y = pos.y + hdt * (double)pos_t.y;
        rp = rho + hdt * (double)rho_t;
        vx = fmaf(hdtf, vel_t.x, vx);
        vy = fmaf(hdtf, vel_t.y, vy);
        Sp.x = fmaf(hdtf, S_t.x, Sp.x);
        Sp.y = fmaf(hdtf, S_t.y, Sp.y);
        Sp.z = fmaf(hdtf, S_t.z, Sp.z);
        Sp.w = fmaf(hdtf, S_t.w, Sp.w);
        Tp = fmaf(hdtf, T_t, Tp);
    }
    const float rhof = (float)rp;
    float p;
    float4 R;
    if (!is_tool) {
        p = (float)(K.c0sq * (rp - K.c.phys.rho0));                 // do_material_eos
        R = artificial_stress_f32(K.f.stresseps, rhof, p, Sp);
        R.w = 0.f;
    } else {
        p = (float)Fsrc.p[k];
        R = f4(Fsrc.R[k]);
    }
    F.p[k] = p;
    F.R[k] = R;
    const float Tn = Tp;   // every record carries T (k_build_records)
    // record: (xr, yr, flags|row, h) (vx, vy, rho, c) (sA, sB, sC, m/rho) (Rxx, Rxy, Ryy, T)
    const sph_geom_constants &g = K.g;
    int ci = 0, cj = 0;
    if (hash >= 0 && hash < g.num_cell) { ci = hash / g.ny; cj = hash - ci * g.ny; }
    const float xr = (float)(pp.x - (g.bbmin_x + (double)ci * g.dx));
    const float yr = (float)(pp.y - (g.bbmin_y + (double)cj * g.dx));
    int flags = (cj & kRowMask) | (is_blanked ? kFlagBlanked : 0) | (is_tool ? kFlagTool : 0);
    const float rho21 = 1.f / (rhof * rhof);
    float4 r0 = make_float4(xr, yr, 0.f, h);
    const float4 r1 = make_float4(vx, vy, rhof, sqrtf(K.f.K_bulk / rhof));
    const float4 r2 = make_float4((Sp.x - p) * rho21, Sp.y * rho21, (Sp.z - p) * rho21, K.f.mass / rhof);
    const float4 r3 = make_float4(R.x, R.y, R.z, Tn);
    if (!(flags & kFlagBlanked) && (nonfinite4(r0) || nonfinite4(r1) || nonfinite4(r2) || nonfinite4(r3)))
        flags |= kFlagNonFinite;   // blanked records are skipped as neighbours: no mark
    r0.z = __int_as_float(flags);
    rec[4 * k + 0] = r0;
    rec[4 * k + 1] = r1;
    rec[4 * k + 2] = r2;
    rec[4 * k + 3] = r3;
    cand[k] = cand_pack(r0.x, r0.y, flags);
}

}  // namespace sphfem
