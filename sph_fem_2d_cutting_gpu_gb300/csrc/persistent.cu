// persistent.cu -- the fused FP32K step as one persistent, cooperative launch.
//
// The graph form of the step is a chain of launches (scan, scatter, rank,
// reorder gather, FEM half step, neighbour sums, FEM update, tool move,
// segment bins, contact, tail); each boundary drains and refills the GPU.  Here
// one launch with every block resident runs the same stages in the same order,
// separated by grid-wide barriers: the per-element bodies are the ones the
// separate kernels run (cells.cuh, fem.cuh, interact32.cuh, tail.cuh), over
// grid-stride loops, and the neighbour sums over virtual blocks of 128
// particles.  Results are those of the graph form, bit for bit: every element
// is computed by the same code from the same inputs, and the only cross-thread
// sums (segment heat exchange, histogram arrivals) are the same atomics.  (With
// the learned warm start folded in, nvcc contracts a few products of the
// epilogue into FMAs differently in the two instantiations: the states then
// agree to FP32 rounding.)
//
// Every barrier wait is bounded (1 s): a block that gives up, or sees that
// another gave up, sets SPH_STATUS_GRID_TIMEOUT and leaves the kernel, so the
// launch always ends.  Supported: FP32K contexts stepping from the compact
// state, with or without the FEM tool (no wear, no rigid tool, no PSE
// conduction), with the learned warm start off or in its in-epilogue form.
#include <algorithm>

#include "cells.cuh"
#include "fem.cuh"
#include "interact32.cuh"
#include "tail.cuh"

namespace sphfem {

namespace {

constexpr int kPB = 128;                     // threads per block
constexpr int kPMinBlocks = 6;               // register budget: 6 resident blocks per SM
constexpr int kPItems = kScanTile / kPB;     // scan buckets per thread (the separate kernels' tiles)
constexpr int kScanOneBlockTiles = 2;        // bucket grids up to 2 tiles are scanned by one block

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid-wide barrier of the cooperative launch.  bar[0] arrivals, bar[1]
// generation, bar[2] abort flag (all zero at launch).  The last block to
// arrive resets the arrivals and opens the next generation; the others wait
// for it with a bounded spin.  The fences on both sides make every write of a
// block before the barrier visible to every block after it.
// skip_arrival (failure-path tests): this block does not arrive, so no wait ends.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, uint32_t *status, bool skip_arrival = false) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        bool ok = true;
        const unsigned gen = ld_acquire_gpu(bar + 1);
        __threadfence();
        const unsigned arrived = skip_arrival ? 0u : atomicAdd(bar, 1u) + 1u;
        if (arrived == gridDim.x) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const unsigned long long t0 = global_ns();
            ok = false;
            for (uint32_t it = 0; it < (1u << 28); it++) {   // one polling thread per block
                if (ld_acquire_gpu(bar + 1) != gen) {
                    ok = true;
                    break;
                }
                if ((it & 63u) == 63u) {
                    if (ld_acquire_gpu(bar + 2) != 0u) break;   // another block gave up
                    if (global_ns() - t0 > kWaitNs) break;
                }
            }
            if (!ok) {
                atomicExch(bar + 2, 1u);
                set_status(status, SPH_STATUS_GRID_TIMEOUT);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// ---- the exclusive scan of the bucket counts in kScanTile tiles (k_scan_*) ----------
__device__ __forceinline__ void scan_reduce_tile(int t, const int32_t *__restrict__ in, int n,
                                                 int32_t *__restrict__ block_sums) {
    __shared__ int sw[32];
    const int base = t * kScanTile + threadIdx.x * kPItems;
    int s = 0;
#pragma unroll
    for (int k = 0; k < kPItems; k++)
        if (base + k < n) s += in[base + k];
    int total;
    block_exclusive_scan(s, sw, total);
    if (threadIdx.x == 0) block_sums[t] = total;
}

// Exclusive scan of the nb tile sums by one block: each thread sums a run of
// consecutive tiles, the block scans the run sums, each thread writes its run.
__device__ __forceinline__ void scan_top_block(int32_t *__restrict__ block_sums, int nb) {
    __shared__ int sw[32];
    const int per = (nb + kPB - 1) / kPB;
    const int b0 = min((int)threadIdx.x * per, nb), b1 = min(b0 + per, nb);
    int s = 0;
    for (int i = b0; i < b1; i++) s += block_sums[i];
    int total;
    int ex = block_exclusive_scan(s, sw, total);
    for (int i = b0; i < b1; i++) {
        const int v = block_sums[i];
        block_sums[i] = ex;
        ex += v;
    }
}

__device__ __forceinline__ void scan_down_tile(int t, const SortScratch &X, int n, int num_cell) {
    __shared__ int sw[32];
    const int base = t * kScanTile + threadIdx.x * kPItems;
    int v[kPItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kPItems; k++) {
        v[k] = (base + k < n) ? X.counts[base + k] : 0;
        s += v[k];
    }
    int total;
    int ex = block_exclusive_scan(s, sw, total) + X.block_sums[t];
#pragma unroll
    for (int k = 0; k < kPItems; k++) {
        const int c = base + k;
        if (c < n) {
            X.offsets[c] = ex;
            if (c < num_cell) {
                if (v[k] > 0) {
                    X.cell_start[c] = ex;
                    X.cell_end[c] = ex + v[k];
                } else {
                    X.cell_start[c] = -1;
                }
            }
            if (c == n - 1) X.offsets[n] = ex + v[k];
        }
        ex += v[k];
    }
}

template <bool kTool, bool kMlp>
__global__ void __launch_bounds__(kPB, kPMinBlocks) k_step_persistent(PersistArgs P) {
    const KConsts &K = P.K;
    const int N = P.N;
    const int gtid = blockIdx.x * kPB + threadIdx.x, gstride = gridDim.x * kPB;
    const int n_buckets = K.g.num_cell + 1;
    const int n_tiles = (n_buckets + kScanTile - 1) / kScanTile;
    uint32_t *status = P.W.status;
    const bool skip_arrival = blockIdx.x == 0 && (K.test_faults & SPH_TEST_SKIP_GRID_ARRIVAL);
    // the FEM half step (independent of the sort)
    if (kTool)
        for (int i = gtid; i < P.fem.n_nodes; i += gstride) fem_half_one(i, K, P.fem, P.tool);
    if (n_tiles <= kScanOneBlockTiles) {   // a small grid: block 0 scans alone, one barrier
        if (blockIdx.x == 0) {
            for (int t = 0; t < n_tiles; t++) scan_reduce_tile(t, P.X.counts, n_buckets, P.X.block_sums);
            __syncthreads();   // the tile sums (written by thread 0) before their scan
            scan_top_block(P.X.block_sums, n_tiles);
            __syncthreads();
            for (int t = 0; t < n_tiles; t++) scan_down_tile(t, P.X, n_buckets, K.g.num_cell);
        }
        if (!grid_barrier(P.bar, status, skip_arrival)) return;
    } else {   // tile sums | their scan (one block) | down-sweep
        for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) scan_reduce_tile(t, P.X.counts, n_buckets, P.X.block_sums);
        if (!grid_barrier(P.bar, status, skip_arrival)) return;
        if (blockIdx.x == 0) scan_top_block(P.X.block_sums, n_tiles);
        if (!grid_barrier(P.bar, status)) return;
        for (int t = blockIdx.x; t < n_tiles; t += gridDim.x) scan_down_tile(t, P.X, n_buckets, K.g.num_cell);
        if (!grid_barrier(P.bar, status)) return;
    }
    // scatter; the histogram of the next step starts from zero (the scan has read it)
    for (int i = gtid; i < N; i += gstride) scatter_one(i, P.X.key, P.X.arrival, P.X.offsets, P.X.slots);
    for (int c = gtid; c < n_buckets; c += gstride) P.X.counts[c] = 0;
    if (!grid_barrier(P.bar, status)) return;
    for (int s = gtid; s < N; s += gstride) rank_one(s, P.X.key, P.X.offsets, P.X.slots, P.perm, status);
    if (!grid_barrier(P.bar, status)) return;
    // reorder + predictor + EOS + artificial stress + records
    for (int k = gtid; k < N; k += gstride)
        gather32_one(k, P.perm, K, P.A, P.F32, P.B, P.F32, P.perm, P.X.hash_next, P.W.rec32, P.W.cand32, P.tool);
    if (!grid_barrier(P.bar, status)) return;
    // neighbour sums + epilogue, 128 particles per virtual block
    const int n_vb = (N + kPB - 1) / kPB;
    for (int vb = blockIdx.x; vb < n_vb; vb += gridDim.x)
        interact32_block<true, kPB, false, kMlp>(vb, N, K, P.X.offsets, P.W.rec32, P.W.cand32, P.B, P.F32, P.seg,
                                                  P.tool, P.W.secant_iters, status, 0, P.mlp);
    if (!grid_barrier(P.bar, status)) return;
    if (kTool) {
        for (int i = gtid; i < P.fem.n_nodes; i += gstride) fem_rate_update_one(i, K, P.fem, P.seg, P.tool);
        if (!grid_barrier(P.bar, status)) return;
        // tool move: nodes over the grid; each case's segments, tool state and segment
        // y-bins by one block (the bins read the moved segments of their case only)
        for (int i = gtid; i < P.fem.n_nodes; i += gstride) {
            const ToolDev &tc = node_case(K, P.tool, i);
            node_move(P.fem, i, tc.vel, tc.dt, tc.flank_retreat);
        }
        for (int c = blockIdx.x; c < K.n_cases; c += gridDim.x) {
            ToolDev &tc = P.tool[c];
            for (int q = threadIdx.x; q < tc.seg_count; q += kPB)
                segment_move(P.seg, tc.seg_first + q, tc.vel, tc.dt, tc.flank_retreat);
            __syncthreads();
            if (threadIdx.x == 0) tool_case_move(tc, tc.dt);
            __syncthreads();
            if (P.seg.bin_count) seg_bins_block(c, P.seg, P.tool);
            __syncthreads();
        }
        if (!grid_barrier(P.bar, status)) return;
        for (int i = gtid; i < N; i += gstride) contact_fem_one(i, K, P.B, P.seg, P.tool, P.fem.T, status);
        if (!grid_barrier(P.bar, status)) return;
    }
    // boundary conditions, invalidation, the next step's hashes and histogram
    for (int i = gtid; i < N; i += gstride) step_tail_one<0, true>(i, K, P.B, P.X, status);
}

template <bool kTool, bool kMlp>
int resident_blocks(int num_sms) {
    static int per_sm[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    int &b = per_sm[dev & 63];
    if (!b) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_step_persistent<kTool, kMlp>, kPB, 0) != cudaSuccess ||
            b < 1)
            b = 1;
    }
    return b * num_sms;
}

template <bool kTool, bool kMlp>
cudaError_t launch_persistent(cudaStream_t s, const PersistArgs &P, int num_sms) {
    const int want = std::max(num_sms, (P.N + kPB - 1) / kPB);
    const int grid = std::min(want, resident_blocks<kTool, kMlp>(num_sms));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kPB);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_step_persistent<kTool, kMlp>, P);
}

}  // namespace

cudaError_t launch_step_persistent(cudaStream_t s, const PersistArgs &P, bool tool, bool mlp, int num_sms) {
    cudaError_t e = cudaMemsetAsync(P.bar, 0, 4 * sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    if (tool) return mlp ? launch_persistent<true, true>(s, P, num_sms) : launch_persistent<true, false>(s, P, num_sms);
    return mlp ? launch_persistent<false, true>(s, P, num_sms) : launch_persistent<false, false>(s, P, num_sms);
}

}  // namespace sphfem
