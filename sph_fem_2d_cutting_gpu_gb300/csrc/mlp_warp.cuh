// mlp_warp.cuh -- the learned warm start evaluated by one warp per sample, for
// the fused FP32K neighbour-sum kernel's epilogue, and the warm-started return
// mapping shared with the tensor-core tile kernel (mlp.cu).
//
// A yielding particle's 4 features are broadcast to its warp; lane l owns
// units 2l and 2l+1 of every 64-wide layer.  The hidden activations travel as
// BF16 pairs (one 32-bit shuffle per two inputs), as the tensor-core form
// rounds them into its BF16 A operand; weights are BF16, sums FP32.  W2 and W3
// are read from a copy packed for this access: for input group i4 (4 inputs)
// lane l loads one 16-byte word holding W[2l][4 i4 .. 4 i4 + 3] and
// W[2l + 1][...] interleaved, so a warp's load is 512 contiguous bytes.
#pragma once

#include <cuda_bf16.h>

#include "physics.cuh"
#include "state.cuh"

namespace sphfem {

__device__ __forceinline__ float sigmoidf_(float z) { return 1.f / (1.f + expf(-z)); }
__device__ __forceinline__ float siluf_(float z) { return z * sigmoidf_(z); }
__device__ __forceinline__ float bf16_bits_to_f(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }
__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
}

// Slot of W2 / W3 element (out o, in i) in the packed copy (layer 0 = W2).
__host__ __device__ __forceinline__ int mlp_packed_slot(int layer, int o, int i) {
    return kMlpWbPk + layer * kMlpH * kMlpH + 2 * ((((i >> 2) * 32 + (o >> 1)) << 2) + (i & 3)) + (o & 1);
}

__device__ __forceinline__ void normalise(const MlpDev &m, const float *x, float *xn) {
#pragma unroll
    for (int c = 0; c < kMlpIn; c++) xn[c] = (x[c] - m.x_mean[c]) * m.x_inv_std[c];
}

// Features of a yielding trial state: log(svm / A), eps_pl, log(1 + eps_pl_dot
// / eps_dot_ref), homologous temperature.  Target: log(2 mu dl / |dev S|).
__device__ __forceinline__ void jc_features(const JcF32 &j, float svm, float eps, float epsd, float T, float *x) {
    x[0] = logf(svm / j.A);
    x[1] = eps;
    x[2] = log1pf(epsd * j.inv_epsdot_ref);
    x[3] = (T - j.Tref) * j.inv_dT;
}

// Forward pass of one sample (standardised features xn, the same in every
// lane) by the whole warp; every lane returns the standardised output.  All
// 32 lanes must call it together.
__device__ __forceinline__ float mlp_forward_warp(const MlpDev &m, const float *xn) {
    constexpr unsigned kFull = 0xffffffffu;
    const int l = threadIdx.x & 31;
    const uint4 w1 = __ldg((const uint4 *)(m.wb + kMlpWbW1) + l);   // W1 rows 2l, 2l+1
    const float2 b1 = __ldg((const float2 *)(m.params + kMlpOffB1) + l);
    float z0 = b1.x, z1 = b1.y;
    z0 = fmaf(bf16_lo(w1.x), xn[0], z0);
    z0 = fmaf(bf16_hi(w1.x), xn[1], z0);
    z0 = fmaf(bf16_lo(w1.y), xn[2], z0);
    z0 = fmaf(bf16_hi(w1.y), xn[3], z0);
    z1 = fmaf(bf16_lo(w1.z), xn[0], z1);
    z1 = fmaf(bf16_hi(w1.z), xn[1], z1);
    z1 = fmaf(bf16_lo(w1.w), xn[2], z1);
    z1 = fmaf(bf16_hi(w1.w), xn[3], z1);
    uint32_t act = pack_bf16x2(siluf_(z0), siluf_(z1));
    const uint4 *wpk = (const uint4 *)(m.wb + kMlpWbPk);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll 1
    for (int layer = 0; layer < 2; layer++) {
        float a0 = 0.f, a1 = 0.f;
#pragma unroll 4
        for (int i4 = 0; i4 < kMlpH / 4; i4++) {
            const uint4 w = __ldg(wpk + (layer * (kMlpH / 4) + i4) * 32 + l);
            const uint32_t p0 = __shfl_sync(kFull, act, 2 * i4), p1 = __shfl_sync(kFull, act, 2 * i4 + 1);
            const float x0 = bf16_lo(p0), x1 = bf16_hi(p0), x2 = bf16_lo(p1), x3 = bf16_hi(p1);
            a0 = fmaf(bf16_lo(w.x), x0, a0);
            a1 = fmaf(bf16_hi(w.x), x0, a1);
            a0 = fmaf(bf16_lo(w.y), x1, a0);
            a1 = fmaf(bf16_hi(w.y), x1, a1);
            a0 = fmaf(bf16_lo(w.z), x2, a0);
            a1 = fmaf(bf16_hi(w.z), x2, a1);
            a0 = fmaf(bf16_lo(w.w), x3, a0);
            a1 = fmaf(bf16_hi(w.w), x3, a1);
        }
        const float2 b = __ldg((const float2 *)(m.params + (layer == 0 ? kMlpOffB2 : kMlpOffB3)) + l);
        s0 = siluf_(a0 + b.x);
        s1 = siluf_(a1 + b.y);
        act = pack_bf16x2(s0, s1);
    }
    const uint32_t w4 = __ldg((const uint32_t *)(m.wb + kMlpWbW4) + l);
    float y = fmaf(bf16_hi(w4), s1, bf16_lo(w4) * s0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(kFull, y, o);
    return y + __ldg(m.params + kMlpOffB4);
}

// State of a yielding particle for the warm-started return mapping, re-read
// from the compact arrays after the fused epilogue has written the corrected
// stress and temperature (the plastic strain is still the start-of-step one).
struct JcWarmState {
    float4 S;
    float p, rho, eps, epsd, T;
    JcTrial tr;
};

// Loads the state of particle k and its features (the trial is the one that
// queued the particle: the same values, so it yields).
__device__ __forceinline__ void jc_warm_load(const KConsts &K, const SortedFields32 &B, const FixedFields32 &F, int k,
                                             JcWarmState &s, float *x) {
    const JcF32 &j = K.f.jc;
    s.S = B.S[k];
    s.p = F.p[k];
    s.rho = (float)B.rho[k];
    s.eps = B.eps_pl[k];
    s.epsd = B.eps_pl_dot[k];
    s.T = B.T[k];
    jc_trial_f32(j, s.S, s.p, s.eps, s.epsd, s.T, s.tr);
    jc_features(j, s.tr.svm, s.eps, s.epsd, s.T, x);
}

// The return mapping from the network's prediction yh (standardised output):
// dl0 = exp(yh sigma + mean) |dev S| / 2 mu, kept inside (0, |dev S| / 2 mu]
// (a full return); a non-finite prediction falls back to the reference's
// start.  The secant runs to the reference's tolerance from there.
__device__ __forceinline__ void jc_warm_finish(const KConsts &K, const SortedFields32 &B,
                                               const ToolDev *__restrict__ tool, const MlpDev &m, int k, float yh,
                                               JcWarmState &s, int32_t *__restrict__ secant_iters, uint32_t *status) {
    const ToolDev &tc = tool[case_of_hash(K, B.hash[k])];
    const float dl_max = s.tr.norm / (2.f * K.f.G);
    float dl0 = expf(yh * m.y_std + m.y_mean) * dl_max;
    dl0 = (dl0 == dl0) ? fminf(fmaxf(dl0, 1e-8f), dl_max) : jc_default_start(s.epsd, tc.dtf);
    int it = 0;
    bool blanked = false;
    const uint32_t st =
        jc_return_f32(K, K.f.jc, tc.dtf, tc.inv_dtf, s.S, s.rho, s.eps, s.epsd, s.T, blanked, &it, s.tr, dl0);
    B.S[k] = s.S;
    B.T[k] = s.T;
    B.eps_pl[k] = s.eps;
    B.eps_pl_dot[k] = s.epsd;
    if (blanked) B.blanked[k] = 1.f;
    if (secant_iters) secant_iters[k] = it;
    if (st) set_status(status, st);
}

// The warm start of the lanes of this warp whose particles yield (pending):
// one warp-wide forward pass per such lane, then each finishes its own return
// mapping.  All 32 lanes must call it together.
__device__ __forceinline__ void jc_warm_warp(const KConsts &K, const SortedFields32 &B, const FixedFields32 &F,
                                             const ToolDev *__restrict__ tool, const MlpDev &m, int k, bool pending,
                                             int32_t *__restrict__ secant_iters, uint32_t *status) {
    constexpr unsigned kFull = 0xffffffffu;
    unsigned todo = __ballot_sync(kFull, pending);
    if (!todo) return;
    JcWarmState s;
    float xn[kMlpIn] = {0.f, 0.f, 0.f, 0.f};
    if (pending) {
        float x[kMlpIn];
        jc_warm_load(K, B, F, k, s, x);
        normalise(m, x, xn);
    }
    float mine = 0.f;
    while (todo) {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1;
        float xb[kMlpIn];
#pragma unroll
        for (int c = 0; c < kMlpIn; c++) xb[c] = __shfl_sync(kFull, xn[c], src);
        const float y = mlp_forward_warp(m, xb);
        if ((int)(threadIdx.x & 31) == src) mine = y;
    }
    if (pending) jc_warm_finish(K, B, tool, m, k, mine, s, secant_iters, status);
}

}  // namespace sphfem
