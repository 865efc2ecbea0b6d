// mlp_warp.cuh -- the learned warm start evaluated by one warp for up to 16
// samples at a time, for the fused FP32K neighbour-sum kernel's epilogue, and
// the warm-started return mapping shared with the tile kernel (mlp.cu).
//
// The yielding particles of a warp are the rows of a 16-row tile; the two
// 64x64 hidden layers are warp-level tensor-core MMAs (mma.sync m16n8k16, BF16
// operands, FP32 accumulation: 32 per layer), whose FP32 results stay in
// registers and become the next layer's A fragments after bias, SiLU and BF16
// rounding -- the C fragment of an m16n8 tile holds the same (row, column)
// pairs as the A fragment of a k16 slice.  B fragments are read straight from
// the row-major BF16 weights: the two K-adjacent values a lane needs are one
// 32-bit word.  The 4 -> 64 input layer and the 64 -> 1 output run on the CUDA
// cores.  Activations are rounded to BF16 between layers as in the tile
// kernel's A operands; SiLU uses the fast exponential and division.
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

__device__ __forceinline__ float silu_fast(float z) { return __fdividef(z, 1.f + __expf(-z)); }

// D += A B for one m16n8k16 tile: BF16 A (4 words) and B (2 words), FP32 D.
__device__ __forceinline__ void mma_bf16_16816(float *d, const uint32_t *a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One n-tile of a hidden layer: acc = rows x outputs 8j..8j+7 of A W^T over the
// four k16 slices of the input, W [64 out][64 in] BF16 row-major.
__device__ __forceinline__ void hidden_tile(const uint16_t *__restrict__ W, const uint32_t (&a)[4][4], int j,
                                            float (&acc)[4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    acc[0] = acc[1] = acc[2] = acc[3] = 0.f;
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
        const uint16_t *w = W + (8 * j + g) * kMlpH + 16 * kk + 2 * t;
        mma_bf16_16816(acc, a[kk], __ldg((const uint32_t *)w), __ldg((const uint32_t *)(w + 8)));
    }
}

// Forward pass of the samples of the lanes in `rows` (at most 16; row r = the
// r-th of them in lane order) by the whole warp; xn: this lane's standardised
// features (read when its bit is set).  Each lane of `rows` gets its sample's
// standardised output.  All 32 lanes must call it together.
__device__ __forceinline__ float mlp_forward_warp16(const float *__restrict__ params, const uint16_t *__restrict__ wb,
                                                  unsigned rows, const float *xn) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    // the lanes holding rows g and g + 8 (a row past the last reads lane 0; its output is unused)
    unsigned ra = rows;
    for (int q = 0; q < g && ra; q++) ra &= ra - 1;
    unsigned rb = ra;
    for (int q = 0; q < 8 && rb; q++) rb &= rb - 1;
    const int src_a = ra ? __ffs(ra) - 1 : 0, src_b = rb ? __ffs(rb) - 1 : 0;
    float xa[kMlpIn], xb[kMlpIn];
#pragma unroll
    for (int c = 0; c < kMlpIn; c++) {
        xa[c] = __shfl_sync(kFull, xn[c], src_a);
        xb[c] = __shfl_sync(kFull, xn[c], src_b);
    }
    // input layer into the A fragments: slice kk, units 16kk + 2t (+1) and 16kk + 2t + 8 (+1)
    uint32_t a[4][4];
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int u = 16 * kk + 2 * t + 8 * h;
            float za[2], zb[2];
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const uint2 w = __ldg((const uint2 *)(wb + kMlpWbW1 + 4 * (u + e)));   // W1[u + e][0..3]
                const float b = __ldg(params + kMlpOffB1 + u + e);
                const float w0 = bf16_lo(w.x), w1 = bf16_hi(w.x), w2 = bf16_lo(w.y), w3 = bf16_hi(w.y);
                za[e] = fmaf(w3, xa[3], fmaf(w2, xa[2], fmaf(w1, xa[1], fmaf(w0, xa[0], b))));
                zb[e] = fmaf(w3, xb[3], fmaf(w2, xb[2], fmaf(w1, xb[1], fmaf(w0, xb[0], b))));
            }
            a[kk][2 * h] = pack_bf16x2(silu_fast(za[0]), silu_fast(za[1]));
            a[kk][2 * h + 1] = pack_bf16x2(silu_fast(zb[0]), silu_fast(zb[1]));
        }
    }
    // hidden layer 2: bias, SiLU, BF16 -- the C fragments of n-tile j are A words of slice j / 2
    uint32_t a2[4][4];
#pragma unroll
    for (int j = 0; j < 8; j++) {
        float acc[4];
        hidden_tile(wb + kMlpWbW2, a, j, acc);
        const float2 b = __ldg((const float2 *)(params + kMlpOffB2 + 8 * j + 2 * t));
        a2[j >> 1][2 * (j & 1)] = pack_bf16x2(silu_fast(acc[0] + b.x), silu_fast(acc[1] + b.y));
        a2[j >> 1][2 * (j & 1) + 1] = pack_bf16x2(silu_fast(acc[2] + b.x), silu_fast(acc[3] + b.y));
    }
    // hidden layer 3 and the output layer (rows g and g + 8 of this lane's columns)
    float ya = 0.f, yb = 0.f;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        float acc[4];
        hidden_tile(wb + kMlpWbW3, a2, j, acc);
        const float2 b = __ldg((const float2 *)(params + kMlpOffB3 + 8 * j + 2 * t));
        const uint32_t w4 = __ldg((const uint32_t *)(wb + kMlpWbW4 + 8 * j + 2 * t));
        ya = fmaf(bf16_lo(w4), silu_fast(acc[0] + b.x), ya);
        ya = fmaf(bf16_hi(w4), silu_fast(acc[1] + b.y), ya);
        yb = fmaf(bf16_lo(w4), silu_fast(acc[2] + b.x), yb);
        yb = fmaf(bf16_hi(w4), silu_fast(acc[3] + b.y), yb);
    }
    ya += __shfl_xor_sync(kFull, ya, 1);
    ya += __shfl_xor_sync(kFull, ya, 2);
    yb += __shfl_xor_sync(kFull, yb, 1);
    yb += __shfl_xor_sync(kFull, yb, 2);
    // this lane's row r: rows g (< 8) come from group r, rows g + 8 from group r - 8
    const int r = __popc(rows & ((1u << lane) - 1u));
    const float va = __shfl_sync(kFull, ya, 4 * (r & 7)), vb = __shfl_sync(kFull, yb, 4 * (r & 7));
    return (r < 8 ? va : vb) + __ldg(params + kMlpOffB4);
}

__device__ __forceinline__ float mlp_forward_warp16(const MlpDev &m, unsigned rows, const float *xn) {
    return mlp_forward_warp16(m.params, m.wb, rows, xn);
}

// The same as a call (the neighbour-sum kernel keeps its registers for its own
// loop: only the few values live across the call are saved around it).
static __device__ __noinline__ float mlp_forward_warp16_call(const float *params, const uint16_t *wb, unsigned rows, float x0,
                                                      float x1, float x2, float x3) {
    const float xn[kMlpIn] = {x0, x1, x2, x3};
    return mlp_forward_warp16(params, wb, rows, xn);
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
// warp-wide forward passes of up to 16 of them at a time, then each finishes
// its own return mapping.  All 32 lanes must call it together.
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
    while (todo) {   // up to 16 yielding lanes per pass
        unsigned batch = 0, rest = todo;
        for (int q = 0; q < 16 && rest; q++) {
            batch |= rest & (0u - rest);
            rest &= rest - 1;
        }
        const float y = mlp_forward_warp16_call(m.params, m.wb, batch, xn[0], xn[1], xn[2], xn[3]);
        if ((batch >> (threadIdx.x & 31)) & 1u) mine = y;
        todo = rest;
    }
    if (pending) jc_warm_finish(K, B, tool, m, k, mine, s, secant_iters, status);
}

}  // namespace sphfem
