// interact32.cuh -- the FP32 neighbour-sum kernel with Kahan-compensated
// sums (k_interact32), its fused epilogue and launch shapes; included by
// interactions.cu (the plain fused step and the staged call) and
// interactions_mlp.cu (the fused step with the learned warm start folded into
// its epilogue).  The kernel's comments are in interactions.cu's header.
#pragma once

#include <type_traits>

#include "async.cuh"
#include "launch.cuh"
#include "mlp_warp.cuh"
#include "rigid.cuh"

namespace sphfem {

// Kahan-compensated FP32 accumulator.
struct KahanF {
    float s, c;
    __device__ __forceinline__ void add(float v) {
        float y = v - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    // Adds the partner lane's (s, c) (lane ^ o within mask): the two sums by an
    // error-free two-sum, whose rounding error joins the compensations.
    __device__ __forceinline__ void merge(unsigned mask, int o) {
        const float so = __shfl_xor_sync(mask, s, o), co = __shfl_xor_sync(mask, c, o);
        const float t = s + so;
        const float bp = t - s;
        const float e = (s - (t - bp)) + (so - bp);
        c = (c + co) - e;
        s = t;
    }
};

// One 32-byte-aligned 256-bit load (two float4) through the non-coherent path:
// the neighbour records are read-only while the pair loops run.
__device__ __forceinline__ void ld_nc_256(const float4 *p, float4 &a, float4 &b) {
    asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
                 : "l"(p));
}

// The candidate flag bits (kCandBlanked, kCandNonFinite) of a record's flag word.
__device__ __forceinline__ int rec_cand_flags(int fj) {
    return ((fj & kFlagBlanked) ? kCandBlanked : 0) | ((fj & kFlagNonFinite) ? kCandNonFinite : 0);
}

// The row difference gj - row of a candidate entry (cand_pack): its y carries the
// row modulo 8 in the three lowest bits, and |gj - row| <= kMaxStencil = 3, so the
// low three bits of the difference, sign-extended, are the difference.
__device__ __forceinline__ int cand_row_diff(int gj, float cy) {
    return (int)(((unsigned)gj - (unsigned)__float_as_int(cy)) << 29) >> 29;
}

// In-support neighbours collected per pass of the pair loops.  With h = 1.7 dx
// a particle has about 36 (a disc of radius 2h): 40 covers nearly all of them
// in one pass.  A second, short pass costs more than its share: the lanes of a
// warp hold 0 to 10 pairs in it, and it re-enters the candidate scan (36 or 32
// entries: 13-15 % slower on the 4.19 M lattice).  Larger lists take shared
// memory from the L1 that serves the neighbour records: at 128 threads x 6
// blocks, 40 entries take 120 KB of shared memory per SM, 48 take 144 KB and
// were 1.3 % slower (44: the same as 48).
constexpr int kChunk32 = 40;
constexpr int kChunk64 = 48;   // FP64: 48 x 256 threads x 4 B = the 48 KB static limit

// Sums of the fused FP32 pair loop, each Kahan-compensated.  The epilogue needs
// the stress divergence and the artificial viscosity only through the
// acceleration (actions_gpu.cu:641-671: vel_t = visc + (S_der.x + S_der.y) +
// forces / m), so both go into one sum per component: nine sums instead of
// the staged form's thirteen.
struct Acc32Fused {
    KahanF vd0, vd1, vd2, vd3, ax, ay, xt0, xt1, tl;
};

// A particle blanked before the step skips the neighbour sums, the corrector and
// the return mapping, but the rigid tool's do_material_fric_heat_gen
// (actions_gpu.cu:316-343) has no blanked test and still heats it.
template <class SF>
__device__ __forceinline__ void rigid_heat_blanked(int k, const KConsts &K, const SF &B) {
    if (!K.rigid || K.c.trml_wp.eta == 0. || flag_nonzero(B.tool_particle[k])) return;
    const double T0 = B.T[k];
    double T = T0;
    rigid_fric_heat_one(K, K.dt, K.rigid->vel, d2(B.vel[k]), d2(B.ft[k]), d2(B.n[k]), T);
    if (T != T0) put(B.T[k], T);
}

// FP32-compensated epilogue on the compact FP32 state: the rates (Jaumann,
// continuity, momentum, advection) and the return mapping in FP32; the
// corrector keeps positions and density in FP64.  vd, sd, vt, xt as in the
// FP64 epilogue.
// kMlp: a yielding particle only sets `pending`; its return mapping runs after
// the warp's forward passes of the learned warm start (jc_warm_warp).
template <bool kMlp>
__device__ __forceinline__ void fused_epilogue32(int k, const KConsts &K, const SortedFields32 &B,
                                                 const FixedFields32 &F, const SegDev &seg,
                                                 const ToolDev *__restrict__ tool, int32_t *__restrict__ secant_iters,
                                                 uint32_t *status, bool is_tool, float2 vel_pred, float rho_pred,
                                                 float4 vd, float4 sd, float2 vt, float2 xt, bool thermal, float T_t_new,
                                                 bool &pending) {
    const ToolDev &tc = tool[case_of_hash(K, B.hash[k])];   // the particle's case (time step, tool)
    const double dt = tc.dt;
    const float dtf = tc.dtf, hdtf = tc.hdtf;
    const float inv_mass = K.f.inv_mass;
    const float4 S0 = B.S[k];
    float4 St;
    float2 pos_t, vel_t;
    float rho_t;
    if (!is_tool) {
        const float4 Sto = B.S_t[k];
        float4 Sp = make_float4(fmaf(hdtf, Sto.x, S0.x), fmaf(hdtf, Sto.y, S0.y), fmaf(hdtf, Sto.z, S0.z),
                                fmaf(hdtf, Sto.w, S0.w));
        St = jaumann_f32(K.f.G, vd, Sp);
        rho_t = -rho_pred * (vd.x + vd.w);
        const float2 fc = B.fc[k], ft = B.ft[k];
        vel_t.x = vt.x + ((sd.x + sd.y) + (fc.x + ft.x) * inv_mass);
        vel_t.y = vt.y + ((sd.z + sd.w) + (fc.y + ft.y) * inv_mass);
        pos_t.x = xt.x + vel_pred.x;
        pos_t.y = xt.y + vel_pred.y;
        B.S_t[k] = St;
        B.rho_t[k] = rho_t;
    } else {
        St = B.S_t[k];
        rho_t = B.rho_t[k];
        if (K.thermal_pse) {   // PSE build: tool particles leave the sums unwritten
            vel_t = B.vel_t[k];
            pos_t = B.pos_t[k];
        } else {
            vel_t = vt;
            pos_t = xt;
        }
    }
    const float T_t = thermal ? T_t_new : B.T_t[k];
    B.pos_t[k] = pos_t;
    B.vel_t[k] = vel_t;
    if (thermal) B.T_t[k] = T_t;
    // corrector (leap_frog.cu:71-96)
    double2 pos = B.pos[k];
    pos.x = pos.x + dt * (double)pos_t.x;
    pos.y = pos.y + dt * (double)pos_t.y;
    B.pos[k] = pos;
    const float2 v0 = B.vel[k];
    const float2 vel = make_float2(fmaf(dtf, vel_t.x, v0.x), fmaf(dtf, vel_t.y, v0.y));
    B.vel[k] = vel;
    float4 S = make_float4(fmaf(dtf, St.x, S0.x), fmaf(dtf, St.y, S0.y), fmaf(dtf, St.z, S0.z), fmaf(dtf, St.w, S0.w));
    const double rho = B.rho[k] + dt * (double)rho_t;
    B.rho[k] = rho;
    float T = fmaf(dtf, T_t, B.T[k]);
    uint32_t st = 0;
    bool blanked = false;
    if (K.has_tool) {   // friction heat (actions_gpu.cu:345-420) for particles in contact
        const int on = B.on_seg[k];
        if (on >= 0 && on < seg.n) {
            double Td = (double)T, bl = 0.;
            st |= fric_heat_one(K, dt, tc.vel, make_double2(vel.x, vel.y), d2(B.ft[k]), d2(B.n[k]), d2(B.fc[k]), rho,
                                (double)B.eps_pl[k], on, seg.n, Td, bl, seg.fric_heat, seg.wear);
            T = (float)Td;
            blanked = flag_is_one(bl);
        }
    } else if (K.rigid && !is_tool && K.c.trml_wp.eta != 0.) {   // actions_gpu.cu:316-343
        double Td = (double)T;
        rigid_fric_heat_one(K, dt, K.rigid->vel, make_double2(vel.x, vel.y), d2(B.ft[k]), d2(B.n[k]), Td);
        T = (float)Td;
    }
    if (K.c.plastic && !is_tool && !blanked) {   // return mapping (actions_gpu.cu:689-754)
        const JcF32 &j = K.f.jc;
        float eps_pl = B.eps_pl[k], eps_pl_dot = B.eps_pl_dot[k];
        int it = 0;
        if constexpr (kMlp) {
            JcTrial tr;
            if (jc_trial_f32(j, S, F.p[k], eps_pl, eps_pl_dot, T, tr)) pending = true;
            else B.eps_pl_dot[k] = 0.f;
        } else if (K.jc_list) {
            // learned warm start: the trial state is stored below and a yielding
            // particle finishes its return mapping in k_jc_warm
            JcTrial tr;
            if (jc_trial_f32(j, S, F.p[k], eps_pl, eps_pl_dot, T, tr)) {
                const unsigned mask = __activemask();
                const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(K.jc_list_count, __popc(mask));
                base = __shfl_sync(mask, base, leader);
                K.jc_list[base + __popc(mask & ((1u << lane) - 1u))] = k;
            } else {
                B.eps_pl_dot[k] = 0.f;
            }
        } else {
            st |= plasticity_f32(K, j, dtf, tc.inv_dtf, S, F.p[k], (float)rho, eps_pl, eps_pl_dot, T, blanked, &it);
            B.eps_pl[k] = eps_pl;
            B.eps_pl_dot[k] = eps_pl_dot;
        }
        if (secant_iters) secant_iters[k] = it;
    }
    B.S[k] = S;
    B.T[k] = T;
    if (blanked) B.blanked[k] = 1.f;
    if (st) set_status(status, st);
}

// ---- FP32 with Kahan-compensated sums --------------------------------------------------
// Staged blocks: the records of the block's cells and their stencil halo,
// one contiguous run per grid column (cells are column-major in the sorted
// order), copied into shared memory by the bulk-copy engine before the pair
// loops.  Staged only when all of the block's particles lie in one grid column
// and the region holds at most `cap` records; otherwise global loads.
struct StageHdr {
    int staged, ix, r_lo, r_hi, c_lo;
    int delta[2 * kMaxStencil + 1];   // shared slot minus global record index, per column
};

template <class SF>
__device__ __forceinline__ void stage_issue(int vb, int N, int kB, const KConsts &K, const int32_t *__restrict__ offsets,
                                            const float4 *__restrict__ rec, const SF &B, int cap,
                                            float4 *srec, StageHdr &h, uint32_t mbar) {
    const sph_geom_constants &g = K.g;
    const int R = g.stencil;
    const int b0 = vb * kB;
    const int hf = B.hash[b0], hl = B.hash[min(b0 + kB, N) - 1];
    h.staged = 0;
    if (hf < 0 || hl >= g.num_cell || hl < hf) return;
    const int ix = hf / g.ny;
    if (hl / g.ny != ix) return;
    const int r_lo = max(hf - ix * g.ny - R, 0), r_hi = min(hl - ix * g.ny + R, g.ny - 1);
    const int c_lo = max(ix - R, 0), c_hi = min(ix + R, g.nx - 1);
    int total = 0, start[2 * kMaxStencil + 1], len[2 * kMaxStencil + 1];
    for (int c = c_lo; c <= c_hi; c++) {
        start[c - c_lo] = __ldg(offsets + c * g.ny + r_lo);
        len[c - c_lo] = __ldg(offsets + c * g.ny + r_hi + 1) - start[c - c_lo];
        h.delta[c - c_lo] = total - start[c - c_lo];
        total += len[c - c_lo];
    }
    if (total <= 0 || total > cap) return;
    mbar_init(mbar);
    mbar_arrive_expect_tx(mbar, (uint32_t)total * 64u);
    const bool issue = !(K.test_faults & SPH_TEST_SKIP_BULK_COPY);   // a test lets the wait run out
    for (int c = c_lo; c <= c_hi; c++)
        if (issue && len[c - c_lo] > 0)
            bulk_g2s(smem_u32(srec + 4 * (start[c - c_lo] + h.delta[c - c_lo])), rec + 4 * (size_t)start[c - c_lo],
                     (uint32_t)len[c - c_lo] * 64u, mbar);
    h.staged = 1;
    h.ix = ix;
    h.r_lo = r_lo;
    h.r_hi = r_hi;
    h.c_lo = c_lo;
}

// L2 prefetch by one thread at block start, overlapped with the neighbour loops:
// the block's slice of the start-of-step state its epilogue reads, and, when
// the block lies in one grid column, the neighbour records of its stencil
// (one contiguous run of rows per column).  Hints only: every range lies
// inside its array.
template <class SF, class FF>
__device__ __forceinline__ void block_prefetch_l2(int vb, int N, int kB, const KConsts &K,
                                                  const int32_t *__restrict__ offsets, const float4 *__restrict__ rec,
                                                  const float2 *__restrict__ cand, const SF &B, const FF &F) {
    const int b0 = vb * kB;
    const uint32_t n = (uint32_t)min(kB, N - b0);
    prefetch_l2_bulk(B.S + b0, n * (uint32_t)sizeof(B.S[0]));
    prefetch_l2_bulk(B.S_t + b0, n * (uint32_t)sizeof(B.S_t[0]));
    prefetch_l2_bulk(B.pos + b0, n * 16u);
    prefetch_l2_bulk(B.vel + b0, n * (uint32_t)sizeof(B.vel[0]));
    prefetch_l2_bulk(B.fc + b0, n * (uint32_t)sizeof(B.fc[0]));
    prefetch_l2_bulk(B.ft + b0, n * (uint32_t)sizeof(B.ft[0]));
    prefetch_l2_bulk(B.rho + b0, n * 8u);
    prefetch_l2_bulk(B.T + b0, n * (uint32_t)sizeof(B.T[0]));
    prefetch_l2_bulk(B.eps_pl + b0, n * (uint32_t)sizeof(B.eps_pl[0]));
    prefetch_l2_bulk(B.eps_pl_dot + b0, n * (uint32_t)sizeof(B.eps_pl_dot[0]));
    prefetch_l2_bulk(F.p + b0, n * (uint32_t)sizeof(F.p[0]));
    const sph_geom_constants &g = K.g;
    const int R = g.stencil;
    const int hf = B.hash[b0], hl = B.hash[b0 + (int)n - 1];
    if (hf < 0 || hl >= g.num_cell || hl < hf) return;
    const int ix = hf / g.ny;
    if (hl / g.ny != ix) return;
    const int r_lo = max(hf - ix * g.ny - R, 0), r_hi = min(hl - ix * g.ny + R, g.ny - 1);
    for (int c = max(ix - R, 0); c <= min(ix + R, g.nx - 1); c++) {
        const int s0 = __ldg(offsets + c * g.ny + r_lo), s1 = __ldg(offsets + c * g.ny + r_hi + 1);
        if (s1 > s0) {
            prefetch_l2_bulk(rec + 4 * (size_t)s0, (uint32_t)(s1 - s0) * 64u);
            const int a0 = s0 & ~1;   // 16-byte aligned start; the size is rounded down
            prefetch_l2_bulk(cand + a0, (uint32_t)(s1 - a0) * 8u);
        }
    }
}

// kB threads per block, at least kMinB resident blocks per SM (a register
// budget for the compiler): the launch shapes the autotuner chooses from.
// kStaged: neighbour records from shared memory (dynamic: cap records + the
// pair lists).
// The fused form works on the compact FP32 state (SortedFields32 / FixedFields32);
// the staged form (sph_interactions_monaghan) on the FP64 arrays.
template <bool kFused>
using Sorted32Of = std::conditional_t<kFused, SortedFields32, SortedFields>;
template <bool kFused>
using Fixed32Of = std::conditional_t<kFused, FixedFields32, FixedFields>;

// kMlp (fused only): the learned warm start of the return mapping in the
// epilogue, one warp-wide forward pass per yielding particle; every lane of a
// warp reaches it, so the per-particle body returns from a lambda.
// One block of kB / kSplit particles, vb-th in sorted order (the kernel's
// blockIdx.x, or a persistent kernel's virtual block).  kSplit > 1 (small
// systems, fused form): kSplit consecutive lanes share a particle, each
// scanning every kSplit-th candidate of each stencil column; their sums are
// merged (compensated) before the epilogue, which the first lane runs.
template <bool kFused, int kB, bool kStaged, bool kMlp, int kSplit = 1>
__device__ __forceinline__ void interact32_block(int vb, int N, const KConsts &K, const int32_t *__restrict__ offsets,
                                                 const float4 *__restrict__ rec, const float2 *__restrict__ cand,
                                                 const Sorted32Of<kFused> &B,
                                                 const Fixed32Of<kFused> &F, const SegDev &seg,
                                                 const ToolDev *__restrict__ tool, int32_t *__restrict__ secant_iters,
                                                 uint32_t *status, int cap, const MlpDev &mlp) {
    static_assert(kFused || !kMlp, "the warm start is folded into the fused epilogue only");
    static_assert(kSplit == 1 || (kFused && !kStaged && 32 % kSplit == 0), "split lanes: fused, unstaged");
    constexpr int kPPB = kB / kSplit;   // particles per block
    const int k = vb * kPPB + (int)threadIdx.x / kSplit;
    const int sub = (int)threadIdx.x % kSplit;
    const unsigned gmask = ((1u << kSplit) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(kSplit - 1));
    if (kFused && threadIdx.x == 0) block_prefetch_l2(vb, N, kPPB, K, offsets, rec, cand, B, F);
    int (*s_list)[kB];
    const float4 *nrec = rec;   // where the neighbour records are read from
    __shared__ StageHdr s_hdr;
    __shared__ alignas(8) unsigned long long s_mbar;
    bool staged = false;
    if constexpr (kStaged) {
        extern __shared__ __align__(128) float4 s_dyn[];
        s_list = (int (*)[kB])(s_dyn + 4 * cap);
        if (threadIdx.x == 0) stage_issue(vb, N, kB, K, offsets, rec, B, cap, s_dyn, s_hdr, smem_u32(&s_mbar));
        __syncthreads();
        if (s_hdr.staged) {
            staged = mbar_wait(smem_u32(&s_mbar), 0);
            if (staged) {
                nrec = s_dyn;
            } else {   // copies late: report, wait once more (bounded) for them, use global loads
                if (threadIdx.x == 0) set_status(status, SPH_STATUS_COPY_TIMEOUT);
                mbar_wait(smem_u32(&s_mbar), 0);
            }
        }
    } else {
        __shared__ int s_list_st[kChunk32][kB];
        s_list = s_list_st;
    }
    bool pending = false;   // kMlp: this particle yields and waits for its warm start
    auto particle = [&]() {
    if (k >= N) return;
    const float4 i0 = rec[4 * k + 0];
    const int fi = __float_as_int(i0.z);
    if (fi & kFlagBlanked) {
        if (kFused && sub == 0) rigid_heat_blanked(k, K, B);   // one lane per particle
        return;
    }
    const bool tool_i = (fi & kFlagTool) != 0;
    const float4 i1 = rec[4 * k + 1], i2 = rec[4 * k + 2], i3 = rec[4 * k + 3];
    const float xri = i0.x, yri = i0.y, hi = i0.w;
    const float vix = i1.x, viy = i1.y, rhoi = i1.z, ci = i1.w;
    const float sAi = i2.x, sBi = i2.y, sCi = i2.z;
    const float Rxxi = i3.x, Rxyi = i3.y, Ryyi = i3.z, Ti = i3.w;
    const float thermal_alpha = (!tool_i) ? K.f.alpha_wp : K.f.alpha_tool_sph;
    const bool thermal = thermal_alpha != 0.f && !K.thermal_pse;   // Brookshaw build only
    const bool pse_tool = K.thermal_pse && tool_i;                  // PSE build: tool particles return at once
    const float h1 = 1.f / hi;
    const float fourh2 = 4.f * hi * hi;
    const float fac = (float)kPiFac * h1 * h1;
    const float alpha = K.f.alpha, beta = K.f.beta, eta2 = K.f.eta2;
    const float inv_wdp = K.f.inv_wdp;
    const float cell = K.f.cell;

    KahanF vd0 = {}, vd1 = {}, vd2 = {}, vd3 = {}, sd0 = {}, sd1 = {}, sd2 = {}, sd3 = {};
    KahanF vt0 = {}, vt1 = {}, xt0 = {}, xt1 = {}, tl = {};
    Acc32Fused af = {};
    // cubic spline (kernels.cuh:25-65) with the per-particle factors folded:
    // q > 1: W = fac/4 (2-q)^6, dW/(r dr) = -3/4 fac h1 (2-q)^2 / r;
    // q <= 1: W = fac (1 - 3/2 q^2 + 3/4 q^3), dW/(r dr) = fac h1^2 (-3 + 9/4 q)
    const float kwa = 0.25f * fac, kda = -0.75f * fac * h1;
    const float kwc = -1.5f * fac, kwd = 0.75f * fac;
    const float kde = -3.f * fac * h1 * h1, kdf = 2.25f * fac * h1 * h1;
    const int hash = B.hash[k];
    const sph_geom_constants &g = K.g;
    int gi = 0, gj = 0, ii = 0, hi_i = 0, lo_j = 0, hi_j = 0, j = 0, j1 = 0;
    const int R = g.stencil;
    bool done = true;
    if (hash >= 0 && hash < g.num_cell && !pse_tool) {
        gi = hash / g.ny;
        gj = hash - gi * g.ny;
        ii = max(gi - R, 0);
        hi_i = min(gi + R + 1, g.nx);
        lo_j = max(gj - R, 0);
        hi_j = min(gj + R + 1, g.ny);
        j = __ldg(offsets + ii * g.ny + lo_j) + sub;
        j1 = __ldg(offsets + ii * g.ny + hi_j);
        done = false;
    }
    // a particle whose stencil lies inside the staged region reads shared memory
    // (slot = global index + per-column delta); any other uses global loads
    bool use_s = false;
    if constexpr (kStaged) {
        use_s = staged && !done && gi == s_hdr.ix && lo_j >= s_hdr.r_lo && hi_j - 1 <= s_hdr.r_hi;
        if (use_s) {
            j += s_hdr.delta[ii - s_hdr.c_lo];
            j1 += s_hdr.delta[ii - s_hdr.c_lo];
        }
    }
    const float4 *__restrict__ nb = use_s ? nrec : rec;
    // Pass 0 sums over the in-support neighbours.  In the reference every active
    // particle of the stencil (this one included) runs the pair body, with zero
    // kernel weights outside the support: exact zeros for finite data, but NaN
    // when one of the factors is NaN or infinite.  So a particle whose stencil
    // holds a record marked non-finite repeats its sums over every active
    // candidate with the reference's zero weights (pass 1).
    // OR of the candidate flags over the stencil (bit kCandNonFinite is the one
    // read; blanked candidates carry no mark)
    int marks = 0;
    auto sweep = [&](auto all_tag) {
    constexpr bool all = decltype(all_tag)::value;
    // the candidate test on (xr, yr), the row difference and the flag bits
    auto take = [&](int &cnt, int jj, float cx, float cy, int drow, int cf, float dxc) {
        const float dx = dxc + (xri - cx);
        const float dy = (float)drow * cell + (yri - cy);
        const float rr2 = dx * dx + dy * dy;
        if (!all) marks |= cf;
        if ((all || (rr2 < fourh2 && rr2 >= 1e-8f)) && !(cf & kCandBlanked))
            s_list[cnt++][threadIdx.x] = (jj << 3) | (gi - ii + R);
    };
    while (!done) {
        // phase 1: collect the next in-support, active neighbours (column offset packed in 3 bits)
        // from the 8-byte candidate entries (cand_pack), or from the staged records' first 16
        // bytes; four candidates per round keep four loads in flight
        int cnt = 0;
        while (cnt < kChunk32) {
            const float dxc = (float)(gi - ii) * cell;
            if (j + 4 * kSplit - (kSplit - 1) <= j1 && cnt <= kChunk32 - 4) {
                if (!kStaged || !use_s) {
                    float2 c[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) c[u] = __ldg(cand + j + u * kSplit);
#pragma unroll
                    for (int u = 0; u < 4; u++)
                        take(cnt, j + u * kSplit, c[u].x, c[u].y, cand_row_diff(gj, c[u].y),
                             __float_as_int(c[u].x), dxc);
                } else {
                    float4 n[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) n[u] = nb[4 * (j + u * kSplit)];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int fj = __float_as_int(n[u].z);
                        take(cnt, j + u * kSplit, n[u].x, n[u].y, gj - (fj & kRowMask), rec_cand_flags(fj), dxc);
                    }
                }
                j += 4 * kSplit;
            } else if (j < j1) {
                if (!kStaged || !use_s) {
                    const float2 c = __ldg(cand + j);
                    take(cnt, j, c.x, c.y, cand_row_diff(gj, c.y), __float_as_int(c.x), dxc);
                } else {
                    const float4 n0 = nb[4 * j + 0];
                    const int fj = __float_as_int(n0.z);
                    take(cnt, j, n0.x, n0.y, gj - (fj & kRowMask), rec_cand_flags(fj), dxc);
                }
                j += kSplit;
            } else {
                if (++ii >= hi_i) {
                    done = true;
                    break;
                }
                j = __ldg(offsets + ii * g.ny + lo_j) + sub;
                j1 = __ldg(offsets + ii * g.ny + hi_j);
                if constexpr (kStaged) {
                    if (use_s) {
                        j += s_hdr.delta[ii - s_hdr.c_lo];
                        j1 += s_hdr.delta[ii - s_hdr.c_lo];
                    }
                }
            }
        }
        // phase 2: the pair body over the collected list, lanes in step.  No
        // software prefetch of the next record: the 32 registers it holds cost
        // more resident warps than it hides latency.
        for (int t = 0; t < cnt; t++) {
            const int e = s_list[t][threadIdx.x];
            const int jn = e >> 3;
            // the 64-byte record of an in-support neighbour: two 256-bit loads (the
            // kernel is bound by L1 wavefronts, and one request per 32 bytes halves them)
            float4 n0, n1, n2, n3;
            if (use_s) {
                n0 = nb[4 * jn + 0];
                n1 = nb[4 * jn + 1];
                n2 = nb[4 * jn + 2];
                n3 = nb[4 * jn + 3];
            } else {
                ld_nc_256(rec + 4 * jn, n0, n1);
                ld_nc_256(rec + 4 * jn + 2, n2, n3);
            }
            const int fj = __float_as_int(n0.z);
            const float dx = (float)((e & 7) - R) * cell + (xri - n0.x);
            const float dy = (float)(gj - (fj & kRowMask)) * cell + (yri - n0.y);
            const float rr2 = dx * dx + dy * dy;
            // FP32 form: hardware reciprocal square root instead of sqrt and division
            const float inv_r = rsqrtf(rr2);
            const float q = rr2 * inv_r * h1;
            // pass 1: cubic_spline's zero weights outside the support (kernels.cuh:37-39)
            const bool zero_w = all && (rr2 >= fourh2 || rr2 < 1e-8f);
            if constexpr (kFused) {
                float w, dwf;
                if (q > 1.f) {
                    const float tq = 2.f - q, t2 = tq * tq;
                    w = kwa * (t2 * t2 * t2);
                    dwf = kda * t2 * inv_r;
                } else {
                    w = fmaf(q * q, fmaf(kwd, q, kwc), fac);
                    dwf = fmaf(kdf, q, kde);
                }
                if (zero_w) w = dwf = 0.f;
                const float wx = dwf * dx, wy = dwf * dy;
                const float volj = n2.w;
                if (!tool_i && !(fj & kFlagTool)) {
                    const float dvx = n1.x - vix, dvy = n1.y - viy;
                    const float tx = wx * volj, ty = wy * volj;
                    af.vd0.add(dvx * tx);
                    af.vd1.add(dvx * ty);
                    af.vd2.add(dvy * tx);
                    af.vd3.add(dvy * ty);
                    float fab = w * inv_wdp;
                    fab *= fab;
                    fab *= fab;
                    const float sxx = (sAi + n2.x) + fab * (Rxxi + n3.x);
                    const float sxy = (sBi + n2.y) + fab * (Rxyi + n3.y);
                    const float syy = (sCi + n2.z) + fab * (Ryyi + n3.z);
                    const float vijposij = -(dvx * dx + dvy * dy);
                    const float irho = __fdividef(2.f, rhoi + n1.z);
                    float piij = 0.f;
                    if (vijposij < 0.f) {
                        const float cij = 0.5f * (ci + n1.w);
                        const float hij = 0.5f * (hi + n0.w);
                        const float muij = __fdividef(hij * vijposij, rr2 + eta2 * hij * hij);
                        piij = (-alpha * cij * muij + beta * muij * muij) * irho;
                    }
                    // acceleration / mass: (stress terms - viscosity) . grad W
                    af.ax.add(fmaf(sxx - piij, wx, sxy * wy));
                    af.ay.add(fmaf(sxy, wx, (syy - piij) * wy));
                    const float wr = w * irho;
                    af.xt0.add(wr * dvx);
                    af.xt1.add(wr * dvy);
                }
                if (thermal && (!zero_w || rr2 > 1e-16f)) af.tl.add(volj * (Ti - n3.w) * dwf);
            } else {
                float val, der;
                if (q > 1.f) {
                    const float t = 2.f - q, t2 = t * t;
                    val = 0.25f * t2 * t2 * t2;
                    der = -0.75f * t2 * h1 * inv_r;
                } else {
                    val = 1.f - 1.5f * q * q * (1.f - 0.5f * q);
                    der = -3.0f * q * (1.f - 0.75f * q) * h1 * inv_r;
                }
                const float w = zero_w ? 0.f : val * fac;
                const float dwf = zero_w ? 0.f : der * fac;
                const float wx = dwf * dx, wy = dwf * dy;
                const float volj = n2.w;
                if (!tool_i && !(fj & kFlagTool)) {
                    const float dvx = n1.x - vix, dvy = n1.y - viy;
                    const float tx = wx * volj, ty = wy * volj;
                    vd0.add(dvx * tx);
                    vd1.add(dvx * ty);
                    vd2.add(dvy * tx);
                    vd3.add(dvy * ty);
                    float fab = w * inv_wdp;
                    fab *= fab;
                    fab *= fab;
                    const float ax = (sAi + n2.x) + fab * (Rxxi + n3.x);
                    const float ay = (sBi + n2.y) + fab * (Rxyi + n3.y);
                    const float az = (sCi + n2.z) + fab * (Ryyi + n3.z);
                    sd0.add(ax * wx);
                    sd1.add(ay * wy);
                    sd2.add(ay * wx);
                    sd3.add(az * wy);
                    const float vijposij = -(dvx * dx + dvy * dy);
                    const float irho = __fdividef(2.f, rhoi + n1.z);
                    if (vijposij < 0.f) {
                        const float cij = 0.5f * (ci + n1.w);
                        const float hij = 0.5f * (hi + n0.w);
                        const float muij = __fdividef(hij * vijposij, rr2 + eta2 * hij * hij);
                        const float piij = (-alpha * cij * muij + beta * muij * muij) * irho;
                        vt0.add(piij * wx);
                        vt1.add(piij * wy);
                    }
                    const float wr = w * irho;
                    xt0.add(wr * dvx);
                    xt1.add(wr * dvy);
                }
                if (thermal && (!zero_w || rr2 > 1e-16f)) tl.add(volj * (Ti - n3.w) * dwf);
            }
        }
    }
    };
    sweep(std::false_type{});
    if constexpr (kSplit > 1) {   // the particle's stencil as a whole
#pragma unroll
        for (int o = 1; o < kSplit; o <<= 1) marks |= __shfl_xor_sync(gmask, marks, o);
    }
    if (marks & kCandNonFinite) {   // rare: the reference's full stencil with zero weights
        vd0 = vd1 = vd2 = vd3 = sd0 = sd1 = sd2 = sd3 = vt0 = vt1 = xt0 = xt1 = tl = KahanF{};
        af = Acc32Fused{};
        ii = max(gi - R, 0);
        j = __ldg(offsets + ii * g.ny + lo_j) + sub;
        j1 = __ldg(offsets + ii * g.ny + hi_j);
        if constexpr (kStaged) {
            if (use_s) {
                j += s_hdr.delta[ii - s_hdr.c_lo];
                j1 += s_hdr.delta[ii - s_hdr.c_lo];
            }
        }
        done = false;
        sweep(std::true_type{});
    }
    if constexpr (kFused) {
        if constexpr (kSplit > 1) {   // merge the lanes' compensated sums; the first lane goes on
#pragma unroll
            for (int o = 1; o < kSplit; o <<= 1) {
                af.vd0.merge(gmask, o);
                af.vd1.merge(gmask, o);
                af.vd2.merge(gmask, o);
                af.vd3.merge(gmask, o);
                af.ax.merge(gmask, o);
                af.ay.merge(gmask, o);
                af.xt0.merge(gmask, o);
                af.xt1.merge(gmask, o);
                af.tl.merge(gmask, o);
            }
            if (sub != 0) return;
        }
        const float mass = K.f.mass;
        const float xs = K.f.xs_mass;
        const float4 vd = make_float4(af.vd0.s, af.vd1.s, af.vd2.s, af.vd3.s);
        // the whole acceleration sum rides in sd.x / sd.z (vt zero): the epilogue adds sd.x + sd.y + vt.x
        const float4 sd = make_float4(mass * af.ax.s, 0.f, mass * af.ay.s, 0.f);
        const float2 xt = make_float2(xs * af.xt0.s, xs * af.xt1.s);
        const float T_t = thermal_alpha * (2.0f * af.tl.s);
        // predicted velocity and density from this particle's record
        fused_epilogue32<kMlp>(k, K, B, F, seg, tool, secant_iters, status, tool_i, make_float2(vix, viy), rhoi, vd,
                               sd, make_float2(0.f, 0.f), xt, thermal, T_t, pending);
    } else {
        const float mass = K.f.mass;
        const float xs = K.f.xs_mass;
        const float4 vd = make_float4(vd0.s, vd1.s, vd2.s, vd3.s);
        const float4 sd = make_float4(mass * sd0.s, mass * sd1.s, mass * sd2.s, mass * sd3.s);
        const float2 vt = make_float2(-mass * vt0.s, -mass * vt1.s);
        const float2 xt = make_float2(xs * xt0.s, xs * xt1.s);
        const float T_t = thermal_alpha * (2.0f * tl.s);
        if (pse_tool) return;
        F.S_der[k] = mk4(sd.x, sd.y, sd.z, sd.w);
        F.v_der[k] = mk4(vd.x, vd.y, vd.z, vd.w);
        B.pos_t[k] = make_double2(xt.x, xt.y);
        B.vel_t[k] = make_double2(vt.x, vt.y);
        if (thermal) B.T_t[k] = (double)T_t;
    }
    };
    particle();
    if constexpr (kMlp) jc_warm_warp(K, B, F, tool, mlp, k, pending, secant_iters, status);
}

template <bool kFused, int kB = kBlock, int kMinB = 1, bool kStaged = false, bool kMlp = false, int kSplit = 1>
__global__ void __launch_bounds__(kB, kMinB) k_interact32(int N, KConsts K, const int32_t *__restrict__ offsets,
                                                       const float4 *__restrict__ rec,
                                                       const float2 *__restrict__ cand, Sorted32Of<kFused> B,
                                                       Fixed32Of<kFused> F, SegDev seg,
                                                       const ToolDev *__restrict__ tool,
                                                       int32_t *__restrict__ secant_iters, uint32_t *status,
                                                       int cap, MlpDev mlp) {
    interact32_block<kFused, kB, kStaged, kMlp, kSplit>(blockIdx.x, N, K, offsets, rec, cand, B, F, seg, tool,
                                                        secant_iters, status, cap, mlp);
}

template <int kB, int kMinB, bool kStaged, bool kMlp = false, int kSplit = 1>
static void launch_i32(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets, const SortedFields32 &B,
                       const FixedFields32 &F, const StepScratch &W, const SegDev &seg, const ToolDev *tool, int cap,
                       const MlpDev &mlp = MlpDev{}) {
    size_t smem = 0;
    if (kStaged) {
        smem = (size_t)cap * 64 + sizeof(int) * kChunk32 * kB;
        static bool configured = false;   // opt in above 48 KB of dynamic shared memory, once
        if (!configured) {
            cudaFuncSetAttribute(k_interact32<true, kB, kMinB, kStaged, kMlp, kSplit>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            configured = true;
        }
    }
    k_interact32<true, kB, kMinB, kStaged, kMlp, kSplit><<<div_up(N, kB / kSplit), kB, smem, s>>>(
        N, K, offsets, W.rec32, W.cand32, B, F, seg, tool, W.secant_iters, W.status, cap, mlp);
}

// The launch shapes of kInteractVariants (interactions.cu), in its order.
template <bool kMlp>
void launch_i32_variant(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets, const SortedFields32 &B,
                        const FixedFields32 &F, const StepScratch &W, const SegDev &seg, const ToolDev *tool,
                        int variant, const MlpDev &mlp) {
    switch (variant) {
        case 1: launch_i32<64, 12, false, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 0, mlp); break;
        case 2: launch_i32<64, 8, false, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 0, mlp); break;
        case 3: launch_i32<128, 4, false, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 0, mlp); break;
        case 4: launch_i32<256, 3, false, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 0, mlp); break;
        case 5: launch_i32<256, 1, false, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 0, mlp); break;
        case 6: launch_i32<128, 3, true, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 640, mlp); break;
        case 7: launch_i32<128, 2, true, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 1024, mlp); break;
        case 8: launch_i32<64, 6, true, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 384, mlp); break;
        case 9: launch_i32<256, 2, true, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 1024, mlp); break;
        case 10: launch_i32<128, 6, false, kMlp, 2>(s, N, K, offsets, B, F, W, seg, tool, 0, mlp); break;
        case 11: launch_i32<128, 6, false, kMlp, 4>(s, N, K, offsets, B, F, W, seg, tool, 0, mlp); break;
        case 12: launch_i32<128, 5, false, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 0, mlp); break;
        case 13: launch_i32<64, 10, false, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 0, mlp); break;
        default: launch_i32<128, 6, false, kMlp>(s, N, K, offsets, B, F, W, seg, tool, 0, mlp); break;
    }
}

}  // namespace sphfem
