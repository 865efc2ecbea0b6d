// mlp.cu -- the learned warm start of the Johnson-Cook return mapping: a
// 4-64-64-64-1 SiLU MLP with BF16 weights and FP32 accumulation that predicts
// the plastic-multiplier increment, its training (forward, backward, Adam)
// and the warm-started return mapping of the fused FP32-compensated step.
//
// The 64x64 hidden layers run on the 5th-generation tensor cores: operands in
// shared memory in the no-swizzle K-major layout, tcgen05.mma issued by one
// thread, accumulators in TMEM, completion through tcgen05.commit on an
// mbarrier.  A tile is 128 samples = 128 threads = the 128 TMEM lanes of an
// M=128 accumulator, so thread r reads row r with tcgen05.ld 32x32b and keeps
// its sample's activations in registers between layers.  In training the two
// 64x64 weight gradients of a tile are one M=128, N=128, K=128 MMA
// ([dZ3^T; dZ2^T] x [A2 | A1]: the two diagonal blocks are dW3 and dW2) that
// accumulates in TMEM over all tiles of the CTA.
//
// Every wait on the tensor cores is bounded (1 s, then SPH_STATUS_MMA_TIMEOUT
// and an orderly exit that still frees TMEM).
#include <cuda_bf16.h>

#include "async.cuh"
#include "launch.cuh"
#include "mlp_warp.cuh"

namespace sphfem {
namespace {

constexpr int kTile = 128;                 // samples per tile = threads per CTA
constexpr uint32_t kTmemCols = 256;        // training: [0,64) layer, [64,192) stacked dW
constexpr uint32_t kTmemColsFwd = 64;      // inference

// Instruction descriptor of tcgen05.mma kind::f16: D F32 (bits 4-5 = 1), A and
// B BF16 (bits 7-9, 10-12 = 1), both K-major, N>>3 at bit 17, M>>4 at bit 24.
constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Byte offset of element (row r, column k) of a K-major BF16 operand with kt
// columns: 8x8 core matrices of 8 rows x 16 bytes (128 contiguous bytes);
// along K the core matrices are 128 bytes apart (leading byte offset), along
// the rows the 8-row groups are kt*16 bytes apart (stride byte offset).
__device__ __forceinline__ uint32_t cm_off(int r, int k, int kt) {
    return (uint32_t)((r >> 3) * (kt * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor (no swizzle, version 1 at bits 46-48).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

// D[128 x N] (+)= A[128 x kt] * B[N x kt]^T, both K-major in shared memory.
__device__ __forceinline__ void gemm_issue(uint32_t tmem_d, uint32_t a_saddr, uint32_t b_saddr, int kt, int N,
                                           bool accumulate) {
    const uint32_t sbo = (uint32_t)kt * 16;
    const uint32_t idesc = idesc_bf16(128, N);
    for (int s = 0; s < kt / 16; s++) {
        uint64_t a = sdesc(a_saddr + 256u * s, 128, sbo);
        uint64_t b = sdesc(b_saddr + 256u * s, 128, sbo);
        mma_bf16(tmem_d, a, b, idesc, (accumulate || s > 0) ? 1u : 0u);
    }
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Whole warp: allocate `ncols` TMEM columns, address written to smem slot.
__device__ __forceinline__ void tmem_alloc(uint32_t slot_saddr, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_saddr), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (load + wait in one
// statement, so no use of the registers can be scheduled before the wait).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// This thread's row of a 64-column accumulator starting at column `col`.
__device__ __forceinline__ void tmem_row64(uint32_t tmem, uint32_t col, float *v) {
    const uint32_t lane = (threadIdx.x >> 5) * 32u;
    const uint32_t a = tmem + (lane << 16) + col;
    tmem_ld16(a, v);
    tmem_ld16(a + 16, v + 16);
    tmem_ld16(a + 32, v + 32);
    tmem_ld16(a + 48, v + 48);
}

__device__ __forceinline__ float dsiluf_(float z) {
    float s = sigmoidf_(z);
    return s * (1.f + z * (1.f - s));
}
__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Row r of a K-major 64-column operand from 64 floats (rounded to BF16).
__device__ __forceinline__ void store_row64(unsigned char *base, int r, const float *v) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
        uint4 q = make_uint4(pack_bf16x2(v[8 * c + 0], v[8 * c + 1]), pack_bf16x2(v[8 * c + 2], v[8 * c + 3]),
                             pack_bf16x2(v[8 * c + 4], v[8 * c + 5]), pack_bf16x2(v[8 * c + 6], v[8 * c + 7]));
        *(uint4 *)(base + cm_off(r, 8 * c, 64)) = q;
    }
}

// Column k of a K-major 128-column operand, rows row0..row0+63, from 64 floats
// (the transposed copies that feed the weight-gradient MMA).
__device__ __forceinline__ void store_col(unsigned char *base, int row0, int k, const float *v) {
#pragma unroll
    for (int j = 0; j < 64; j++) *(__nv_bfloat16 *)(base + cm_off(row0 + j, k, 128)) = __float2bfloat16_rn(v[j]);
}

// Shared parameter block of a CTA (FP32 values of the BF16 weights of the
// CUDA-core layers, biases).
struct MlpSmall {
    float w1[kMlpH * kMlpIn], b1[kMlpH], b2[kMlpH], b3[kMlpH], w4[kMlpH], b4;
};

__device__ void load_small(MlpSmall &s, const MlpDev &m) {
    for (int i = threadIdx.x; i < kMlpH * kMlpIn; i += blockDim.x) s.w1[i] = bf16_bits_to_f(m.wb[kMlpWbW1 + i]);
    for (int i = threadIdx.x; i < kMlpH; i += blockDim.x) {
        s.b1[i] = m.params[kMlpOffB1 + i];
        s.b2[i] = m.params[kMlpOffB2 + i];
        s.b3[i] = m.params[kMlpOffB3 + i];
        s.w4[i] = bf16_bits_to_f(m.wb[kMlpWbW4 + i]);
    }
    if (threadIdx.x == 0) s.b4 = m.params[kMlpOffB4];
}

// W [64 out][64 in] as the B operand of X W^T (rows n = out, K = in), or
// transposed (rows n = in, K = out) as the B operand of dZ W.
__device__ void load_weight(unsigned char *dst, const uint16_t *w, bool transpose) {
    if (!transpose) {   // 8 consecutive inputs of one output = one 16-byte core-matrix row
        for (int i = threadIdx.x; i < kMlpH * kMlpH / 8; i += blockDim.x) {
            const int o = i >> 3, k8 = (i & 7) * 8;
            *(uint4 *)(dst + cm_off(o, k8, 64)) = *(const uint4 *)(w + o * kMlpH + k8);
        }
        return;
    }
    for (int i = threadIdx.x; i < kMlpH * kMlpH; i += blockDim.x) {
        int o = i >> 6, in = i & 63;
        int n = transpose ? in : o, k = transpose ? o : in;
        *(uint16_t *)(dst + cm_off(n, k, 64)) = w[i];
    }
}


__device__ __forceinline__ void layer1(const MlpSmall &s, const float *xn, float *a, float *z) {
#pragma unroll
    for (int j = 0; j < kMlpH; j++) {
        float acc = s.b1[j];
#pragma unroll
        for (int c = 0; c < kMlpIn; c++) acc = fmaf(s.w1[j * kMlpIn + c], xn[c], acc);
        if (z) z[j] = acc;
        a[j] = siluf_(acc);
    }
}

// Shared memory of the forward-only kernels.
struct FwdSmem {
    alignas(128) unsigned char w2[kMlpH * kMlpH * 2];
    alignas(128) unsigned char w3[kMlpH * kMlpH * 2];
    alignas(128) unsigned char act[kTile * kMlpH * 2];
    MlpSmall small;
    alignas(8) unsigned long long mbar;
    uint32_t tmem_slot;
    int fail;
};

// Forward pass of this CTA's tile; xn = standardised features of this
// thread's row.  Returns the standardised output, or sets *timeout.
// 16 columns [c0, c0+16) of row r of a K-major 64-column operand (BF16).
__device__ __forceinline__ void store_row16(unsigned char *base, int r, int c0, const float *v) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const float *w = v + 8 * h;
        *(uint4 *)(base + cm_off(r, c0 + 8 * h, 64)) =
            make_uint4(pack_bf16x2(w[0], w[1]), pack_bf16x2(w[2], w[3]), pack_bf16x2(w[4], w[5]),
                       pack_bf16x2(w[6], w[7]));
    }
}

// Forward pass of this CTA's tile; xn = standardised features of this
// thread's row.  Returns the standardised output, or sets *timeout.  The
// activations go 16 columns at a time (TMEM load, SiLU, store) in a rolled
// loop: the code stays small enough for the instruction cache of a short,
// latency-bound launch.
// skip_mma (failure-path tests): issue no MMA, so the bounded wait runs out.
__device__ float forward_tile(FwdSmem &sh, uint32_t tmem, uint32_t &phase, const float *xn, bool &timeout,
                              bool skip_mma = false) {
    const uint32_t mbar = smem_u32(&sh.mbar);
    const int r = threadIdx.x;
    const uint32_t trow = tmem + (((uint32_t)threadIdx.x >> 5) * 32u << 16);
    float v[16];
#pragma unroll 1
    for (int c0 = 0; c0 < kMlpH; c0 += 16) {   // layer 1 on the CUDA cores
#pragma unroll
        for (int q = 0; q < 16; q++) {
            float acc = sh.small.b1[c0 + q];
#pragma unroll
            for (int c = 0; c < kMlpIn; c++) acc = fmaf(sh.small.w1[(c0 + q) * kMlpIn + c], xn[c], acc);
            v[q] = siluf_(acc);
        }
        store_row16(sh.act, r, c0, v);
    }
    float y = sh.small.b4;
#pragma unroll 1
    for (int layer = 0; layer < 2; layer++) {
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (r == 0 && !skip_mma) {
            tc_fence_after();
            gemm_issue(tmem, smem_u32(sh.act), smem_u32(layer == 0 ? sh.w2 : sh.w3), 64, 64, false);
            mma_commit(mbar);
        }
        bool ok = mbar_wait(mbar, phase);
        phase ^= 1u;
        if (__syncthreads_or(!ok)) {
            timeout = true;
            return 0.f;
        }
        tc_fence_after();
        const float *b = layer == 0 ? sh.small.b2 : sh.small.b3;
#pragma unroll 1
        for (int c0 = 0; c0 < kMlpH; c0 += 16) {
            tmem_ld16(trow + c0, v);
            if (layer == 0) {   // the MMA has read act: overwrite it with A2 (next MMA after the barrier)
#pragma unroll
                for (int q = 0; q < 16; q++) v[q] = siluf_(v[q] + b[c0 + q]);
                store_row16(sh.act, r, c0, v);
            } else {
#pragma unroll
                for (int q = 0; q < 16; q++) y = fmaf(sh.small.w4[c0 + q], siluf_(v[q] + b[c0 + q]), y);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    return y;
}

__device__ bool fwd_setup(FwdSmem &sh, const MlpDev &m, uint32_t &tmem) {
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&sh.mbar));
        sh.fail = 0;
    }
    load_small(sh.small, m);
    load_weight(sh.w2, m.wb + kMlpWbW2, false);
    load_weight(sh.w3, m.wb + kMlpWbW3, false);
    if (threadIdx.x < 32) tmem_alloc(smem_u32(&sh.tmem_slot), kTmemColsFwd);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    tmem = sh.tmem_slot;
    return true;
}

__device__ void fwd_teardown(FwdSmem &sh, uint32_t tmem) {
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemColsFwd);
    }
}

// ---- batch inference (raw features in, raw target out) -------------------------------------------
__global__ void __launch_bounds__(kTile, 1) k_mlp_predict(MlpDev m, const float *__restrict__ x, int64_t n,
                                                         float *__restrict__ y, uint32_t *status) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    FwdSmem &sh = *(FwdSmem *)smem_raw;
    const int64_t ntiles = (n + kTile - 1) / kTile;
    if ((int64_t)blockIdx.x >= ntiles) return;
    uint32_t tmem;
    fwd_setup(sh, m, tmem);
    uint32_t phase = 0;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t i = t * kTile + threadIdx.x;
        float xr[kMlpIn] = {0.f, 0.f, 0.f, 0.f}, xn[kMlpIn];
        if (i < n) {
            float4 q = *(const float4 *)(x + 4 * i);
            xr[0] = q.x; xr[1] = q.y; xr[2] = q.z; xr[3] = q.w;
        }
        normalise(m, xr, xn);
        bool timeout = false;
        float yh = forward_tile(sh, tmem, phase, xn, timeout);
        if (timeout) {
            if (threadIdx.x == 0) set_status(status, SPH_STATUS_MMA_TIMEOUT);
            break;
        }
        if (i < n) y[i] = yh * m.y_std + m.y_mean;
    }
    fwd_teardown(sh, tmem);
}

// ---- batch inference, 16 samples per warp pass (the fused step's in-epilogue form) -----------------
__global__ void __launch_bounds__(256) k_mlp_predict_warp(MlpDev m, const float *__restrict__ x, int64_t n,
                                                         float *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w * 16 < n; w += warps) {
        const int64_t i = w * 16 + lane;   // lanes 0..15 hold the samples (warp-uniform loop)
        const bool valid = lane < 16 && i < n;
        float xr[kMlpIn] = {0.f, 0.f, 0.f, 0.f}, xn[kMlpIn];
        if (valid) {
            const float4 q = __ldg((const float4 *)x + i);
            xr[0] = q.x; xr[1] = q.y; xr[2] = q.z; xr[3] = q.w;
        }
        normalise(m, xr, xn);
        const unsigned rows = __ballot_sync(0xffffffffu, valid);
        const float yh = mlp_forward_warp16(m, rows, xn);
        if (valid) y[i] = yh * m.y_std + m.y_mean;
    }
}

// ---- warm-started return mapping of the fused FP32 step (tensor-core form) -----------------------
__global__ void __launch_bounds__(kTile, 1)
    k_jc_warm(KConsts K, SortedFields32 B, FixedFields32 F, const ToolDev *__restrict__ tool, MlpDev m,
              int32_t *__restrict__ secant_iters, uint32_t *status) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    FwdSmem &sh = *(FwdSmem *)smem_raw;
    const int count = *K.jc_list_count;
    const int ntiles = (count + kTile - 1) / kTile;
    if ((int)blockIdx.x >= ntiles) return;
    uint32_t tmem;
    fwd_setup(sh, m, tmem);
    uint32_t phase = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int e = t * kTile + threadIdx.x;
        const bool valid = e < count;
        const int k = valid ? K.jc_list[e] : 0;
        JcWarmState st{};
        float x[kMlpIn] = {0.f, 0.f, 0.f, 0.f}, xn[kMlpIn];
        if (valid) jc_warm_load(K, B, F, k, st, x);
        normalise(m, x, xn);
        bool timeout = false;
        const float yh = forward_tile(sh, tmem, phase, xn, timeout, (K.test_faults & SPH_TEST_SKIP_MMA) != 0);
        if (timeout) {
            if (threadIdx.x == 0) set_status(status, SPH_STATUS_MMA_TIMEOUT);
            break;
        }
        if (valid) jc_warm_finish(K, B, tool, m, k, yh, st, secant_iters, status);
    }
    fwd_teardown(sh, tmem);
}

// ---- training: gradients of one minibatch ---------------------------------------------------------
struct TrainSmem {
    alignas(128) unsigned char w2f[kMlpH * kMlpH * 2];   // W2 as B of A1 W2^T
    alignas(128) unsigned char w3f[kMlpH * kMlpH * 2];
    alignas(128) unsigned char w2b[kMlpH * kMlpH * 2];   // W2^T as B of dZ2 W2
    alignas(128) unsigned char w3b[kMlpH * kMlpH * 2];
    alignas(128) unsigned char act[kTile * kMlpH * 2];   // A operand of the 64-wide GEMMs
    alignas(128) unsigned char adw[kTile * kTile * 2];   // [dZ3^T; dZ2^T]  (rows: neurons, K: samples)
    alignas(128) unsigned char bdw[kTile * kTile * 2];   // [A2^T; A1^T]
    float zs[kTile][kMlpH + 1];                          // Z2 of each sample, then dZ1
    float xn[kTile][kMlpIn];
    float dw4[4][kMlpH];
    float db4[4], loss[4];
    MlpSmall small;
    alignas(8) unsigned long long mbar;
    uint32_t tmem_slot;
};

// Per-CTA partial sums over the samples of its tiles, written to
// part[blockIdx.x][0..kMlpParams) (gradient of the mean loss) and
// part[..][kMlpParams] (sum of 0.5 (y - t)^2 in standardised units).
__global__ void __launch_bounds__(kTile, 1)
    k_mlp_grad(MlpDev m, const float *__restrict__ x, const float *__restrict__ tgt, const int32_t *__restrict__ idx,
               int64_t nb, float inv_nb, float *__restrict__ part, uint32_t *status) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TrainSmem &sh = *(TrainSmem *)smem_raw;
    const int r = threadIdx.x, warp = r >> 5, lane = r & 31;
    float *out = part + (size_t)blockIdx.x * (kMlpParams + 1);
    const int64_t ntiles = (nb + kTile - 1) / kTile;
    if ((int64_t)blockIdx.x >= ntiles) {
        for (int i = r; i < kMlpParams + 1; i += kTile) out[i] = 0.f;
        return;
    }
    const uint32_t mbar = smem_u32(&sh.mbar);
    if (r == 0) mbar_init(mbar);
    load_small(sh.small, m);
    load_weight(sh.w2f, m.wb + kMlpWbW2, false);
    load_weight(sh.w3f, m.wb + kMlpWbW3, false);
    load_weight(sh.w2b, m.wb + kMlpWbW2, true);
    load_weight(sh.w3b, m.wb + kMlpWbW3, true);
    for (int i = r; i < 4 * kMlpH; i += kTile) (&sh.dw4[0][0])[i] = 0.f;
    if (r < 4) { sh.db4[r] = 0.f; sh.loss[r] = 0.f; }
    if (warp == 0) tmem_alloc(smem_u32(&sh.tmem_slot), kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh.tmem_slot;
    uint32_t phase = 0;
    bool timeout = false;
    // per-thread accumulators: thread j < 64 owns dW1[j][:], db1[j], db3[j]; thread 64 + j owns db2[j]
    float acc_w1[kMlpIn] = {0.f, 0.f, 0.f, 0.f}, acc_b1 = 0.f, acc_b23 = 0.f;
    int tiles_done = 0;
    float v[kMlpH];

    auto mma_wait = [&]() -> bool {
        bool ok = mbar_wait(mbar, phase);
        phase ^= 1u;
        return !__syncthreads_or(!ok);
    };
    auto sync_for_mma = [&]() {
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
    };

    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t e = t * kTile + r;
        const bool valid = e < nb;
        float xr[kMlpIn] = {0.f, 0.f, 0.f, 0.f}, xn[kMlpIn], tn = 0.f;
        if (valid) {
            const int64_t i = idx ? idx[e] : e;
            float4 q = *(const float4 *)(x + 4 * i);
            xr[0] = q.x; xr[1] = q.y; xr[2] = q.z; xr[3] = q.w;
            tn = (tgt[i] - m.y_mean) / m.y_std;
        }
        normalise(m, xr, xn);
#pragma unroll
        for (int c = 0; c < kMlpIn; c++) sh.xn[r][c] = xn[c];
        // layer 1 (CUDA cores): A1 -> act and bdw rows 64..127
        layer1(sh.small, xn, v, nullptr);
#pragma unroll
        for (int jj = 0; jj < kMlpH; jj++) v[jj] = bf16_round(v[jj]);
        store_row64(sh.act, r, v);
        store_col(sh.bdw, 64, r, v);
        // layer 2: Z2 = A1 W2^T + b2
        sync_for_mma();
        if (r == 0) {
            tc_fence_after();
            gemm_issue(tmem, smem_u32(sh.act), smem_u32(sh.w2f), 64, 64, false);
            mma_commit(mbar);
        }
        if (!mma_wait()) { timeout = true; break; }
        tc_fence_after();
        tmem_row64(tmem, 0, v);
#pragma unroll
        for (int jj = 0; jj < kMlpH; jj++) {
            v[jj] += sh.small.b2[jj];
            sh.zs[r][jj] = v[jj];
            v[jj] = bf16_round(siluf_(v[jj]));
        }
        tc_fence_before();
        __syncthreads();
        store_row64(sh.act, r, v);
        store_col(sh.bdw, 0, r, v);
        // layer 3: Z3 = A2 W3^T + b3, output, dZ3
        sync_for_mma();
        if (r == 0) {
            tc_fence_after();
            gemm_issue(tmem, smem_u32(sh.act), smem_u32(sh.w3f), 64, 64, false);
            mma_commit(mbar);
        }
        if (!mma_wait()) { timeout = true; break; }
        tc_fence_after();
        tmem_row64(tmem, 0, v);
        float y = sh.small.b4;
#pragma unroll
        for (int jj = 0; jj < kMlpH; jj++) {
            v[jj] += sh.small.b3[jj];
            y = fmaf(sh.small.w4[jj], siluf_(v[jj]), y);
        }
        const float err = valid ? (y - tn) : 0.f;
        const float g = err * inv_nb;
        // dW4 = sum g a3, db4 = sum g (warp sums, then per-warp slots)
#pragma unroll
        for (int jj = 0; jj < kMlpH; jj++) {
            float c = g * siluf_(v[jj]);
            for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
            if (lane == 0) sh.dw4[warp][jj] += c;
        }
        {
            float c = g, l = 0.5f * err * err;
            for (int o = 16; o > 0; o >>= 1) {
                c += __shfl_xor_sync(0xffffffffu, c, o);
                l += __shfl_xor_sync(0xffffffffu, l, o);
            }
            if (lane == 0) { sh.db4[warp] += c; sh.loss[warp] += l; }
        }
#pragma unroll
        for (int jj = 0; jj < kMlpH; jj++) v[jj] = bf16_round(g * sh.small.w4[jj] * dsiluf_(v[jj]));
        tc_fence_before();
        __syncthreads();
        store_row64(sh.act, r, v);   // dZ3 as A of dA2 = dZ3 W3
        store_col(sh.adw, 0, r, v);  // dZ3^T
        sync_for_mma();
        if (r == 0) {
            tc_fence_after();
            gemm_issue(tmem, smem_u32(sh.act), smem_u32(sh.w3b), 64, 64, false);
            mma_commit(mbar);
        }
        if (!mma_wait()) { timeout = true; break; }
        tc_fence_after();
        tmem_row64(tmem, 0, v);
#pragma unroll
        for (int jj = 0; jj < kMlpH; jj++) v[jj] = bf16_round(v[jj] * dsiluf_(sh.zs[r][jj]));
        tc_fence_before();
        __syncthreads();
        store_row64(sh.act, r, v);    // dZ2 as A of dA1 = dZ2 W2
        store_col(sh.adw, 64, r, v);  // dZ2^T
        // [dW3 | . ; . | dW2] += [dZ3^T; dZ2^T] [A2 | A1] over this tile's samples, and dA1
        sync_for_mma();
        if (r == 0) {
            tc_fence_after();
            gemm_issue(tmem + 64, smem_u32(sh.adw), smem_u32(sh.bdw), 128, 128, tiles_done > 0);
            gemm_issue(tmem, smem_u32(sh.act), smem_u32(sh.w2b), 64, 64, false);
            mma_commit(mbar);
        }
        if (!mma_wait()) { timeout = true; break; }
        tc_fence_after();
        tmem_row64(tmem, 0, v);
#pragma unroll
        for (int jj = 0; jj < kMlpH; jj++) {   // dZ1 = dA1 * silu'(Z1) (FP32), Z1 recomputed
            float z = sh.small.b1[jj];
#pragma unroll
            for (int c = 0; c < kMlpIn; c++) z = fmaf(sh.small.w1[jj * kMlpIn + c], xn[c], z);
            v[jj] *= dsiluf_(z);
        }
        tc_fence_before();
        __syncthreads();   // zs (Z2) no longer needed by any thread
#pragma unroll
        for (int jj = 0; jj < kMlpH; jj++) sh.zs[r][jj] = v[jj];
        __syncthreads();
        if (r < kMlpH) {
            // dW1 row r, db1[r]; db3[r] = sum over samples of dZ3[:, r] (row r of adw)
            for (int s2 = 0; s2 < kTile; s2++) {
                const float d = sh.zs[s2][r];
                acc_b1 += d;
#pragma unroll
                for (int c = 0; c < kMlpIn; c++) acc_w1[c] = fmaf(d, sh.xn[s2][c], acc_w1[c]);
            }
        }
        {
            // db3 (threads < 64) or db2 (threads >= 64): sum of row r of adw
            float sum = 0.f;
            for (int k8 = 0; k8 < kTile; k8 += 8) {
                uint4 q = *(const uint4 *)(sh.adw + cm_off(r, k8, 128));
                const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int h = 0; h < 4; h++)
                    sum += __uint_as_float(w[h] << 16) + __uint_as_float(w[h] & 0xffff0000u);
            }
            acc_b23 += sum;
        }
        tiles_done++;
        __syncthreads();
    }
    if (timeout) {
        if (r == 0) set_status(status, SPH_STATUS_MMA_TIMEOUT);
        for (int i = r; i < kMlpParams + 1; i += kTile) out[i] = 0.f;
    } else {
        // weight gradients from TMEM: rows < 64 hold dW3 (columns 64..127), rows >= 64 dW2 (columns 128..191)
        tc_fence_after();
        const bool upper = r < kMlpH;
        tmem_row64(tmem, upper ? 64u : 128u, v);
        float *dst = out + (upper ? kMlpOffW3 + r * kMlpH : kMlpOffW2 + (r - kMlpH) * kMlpH);
#pragma unroll
        for (int jj = 0; jj < kMlpH; jj++) dst[jj] = v[jj];
        if (upper) {
#pragma unroll
            for (int c = 0; c < kMlpIn; c++) out[kMlpOffW1 + r * kMlpIn + c] = acc_w1[c];
            out[kMlpOffB1 + r] = acc_b1;
            out[kMlpOffB3 + r] = acc_b23;
            out[kMlpOffW4 + r] = sh.dw4[0][r] + sh.dw4[1][r] + sh.dw4[2][r] + sh.dw4[3][r];
        } else {
            out[kMlpOffB2 + (r - kMlpH)] = acc_b23;
        }
        if (r == 0) {
            out[kMlpOffB4] = sh.db4[0] + sh.db4[1] + sh.db4[2] + sh.db4[3];
            out[kMlpParams] = sh.loss[0] + sh.loss[1] + sh.loss[2] + sh.loss[3];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

// BF16 copy of parameter p if it is a weight.
__device__ __forceinline__ void store_wb(uint16_t *__restrict__ wb, int p, float w) {
    int q = -1;
    if (p < kMlpOffB1) q = kMlpWbW1 + p;
    else if (p >= kMlpOffW2 && p < kMlpOffB2) q = kMlpWbW2 + (p - kMlpOffW2);
    else if (p >= kMlpOffW3 && p < kMlpOffB3) q = kMlpWbW3 + (p - kMlpOffW3);
    else if (p >= kMlpOffW4 && p < kMlpOffB4) q = kMlpWbW4 + (p - kMlpOffW4);
    if (q >= 0) wb[q] = __bfloat16_as_ushort(__float2bfloat16_rn(w));
}

// Sum of the per-CTA partials in CTA order (deterministic); with `adam`, one
// Adam step on the FP32 parameters and refreshed BF16 weight copies.
__global__ void k_mlp_reduce_adam(const float *__restrict__ part, int nparts, float *__restrict__ grad_out,
                                  float *__restrict__ loss_out, float *__restrict__ params, float *__restrict__ m1,
                                  float *__restrict__ m2, uint16_t *__restrict__ wb, float lr, float beta1, float beta2,
                                  float eps, float c1, float c2, int adam) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > kMlpParams) return;
    float g = 0.f;
    for (int c = 0; c < nparts; c++) g += part[(size_t)c * (kMlpParams + 1) + p];
    if (grad_out) grad_out[p] = g;
    if (p == kMlpParams) {
        if (loss_out) *loss_out = g;
        return;
    }
    if (!adam) return;
    const float a = beta1 * m1[p] + (1.f - beta1) * g;
    const float b = beta2 * m2[p] + (1.f - beta2) * g * g;
    m1[p] = a;
    m2[p] = b;
    const float w = params[p] - lr * (a * c1) / (sqrtf(b * c2) + eps);
    params[p] = w;
    store_wb(wb, p, w);
}

__global__ void k_mlp_refresh_wb(const float *__restrict__ params, uint16_t *__restrict__ wb) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kMlpParams) return;
    store_wb(wb, p, params[p]);
}

}  // namespace

// ---- host launchers ----------------------------------------------------------------------------
size_t mlp_fwd_smem() { return sizeof(FwdSmem); }
size_t mlp_train_smem() { return sizeof(TrainSmem); }

cudaError_t mlp_configure() {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FwdSmem));
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_jc_warm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(FwdSmem));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
}

void launch_mlp_predict(cudaStream_t s, const MlpDev &m, const float *x, int64_t n, float *y, uint32_t *status,
                        int grid) {
    k_mlp_predict<<<grid, kTile, sizeof(FwdSmem), s>>>(m, x, n, y, status);
}

void launch_mlp_predict_warp(cudaStream_t s, const MlpDev &m, const float *x, int64_t n, float *y, int grid) {
    k_mlp_predict_warp<<<grid, 256, 0, s>>>(m, x, n, y);
}

void launch_jc_warm(cudaStream_t s, int grid, const KConsts &K, const SortedFields32 &B, const FixedFields32 &F,
                    const ToolDev *tool, const MlpDev &m, int32_t *secant_iters, uint32_t *status) {
    k_jc_warm<<<grid, kTile, sizeof(FwdSmem), s>>>(K, B, F, tool, m, secant_iters, status);
}

void launch_mlp_grad(cudaStream_t s, int grid, const MlpDev &m, const float *x, const float *t, const int32_t *idx,
                     int64_t nb, float *part, uint32_t *status) {
    k_mlp_grad<<<grid, kTile, sizeof(TrainSmem), s>>>(m, x, t, idx, nb, 1.f / (float)nb, part, status);
}

void launch_mlp_reduce_adam(cudaStream_t s, const float *part, int nparts, float *grad_out, float *loss_out,
                            float *params, float *m1, float *m2, uint16_t *wb, float lr, float beta1, float beta2,
                            float eps, float c1, float c2, bool adam) {
    k_mlp_reduce_adam<<<div_up(kMlpParams + 1, 256), 256, 0, s>>>(part, nparts, grad_out, loss_out, params, m1, m2,
                                                                  wb, lr, beta1, beta2, eps, c1, c2, adam ? 1 : 0);
}

void launch_mlp_refresh_wb(cudaStream_t s, const float *params, uint16_t *wb) {
    k_mlp_refresh_wb<<<div_up(kMlpParams, 256), 256, 0, s>>>(params, wb);
}

}  // namespace sphfem
