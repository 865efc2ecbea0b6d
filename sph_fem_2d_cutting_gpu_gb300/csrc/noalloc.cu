// noalloc.cu -- cell-list build that allocates nothing.
//
// Some callers of this library cannot call cudaMalloc at the point where
// they need a cell list.  Examples:
//  - a host application whose own memory manager owns all device memory
//    and forbids allocations from outside it;
//  - a latency-critical loop that cannot afford the device synchronisation
//    an allocation may cause;
//  - a recovery path that must keep working when device memory is
//    exhausted.
// sph_cells_build_noalloc serves them.  The caller passes the inputs and
// outputs as device arrays.  The counting sort's scratch (keys, arrival
// slots, cell counts and offsets, in-cell slots, scan partials) lives in
// one file-scope device array, g_cells_scratch.  Its size is fixed at
// kNoAllocMaxParticles particles and kNoAllocMaxCells cells.
//
// Contract:
//  - Each GPU that loads the library holds this array until the process
//    exits: about 5.2 MB per device.
//  - The first call in each CUDA context (a device's primary context, or a
//    context the application created with the driver API) looks up the
//    array's address in that context.  Make that first call before any
//    stream capture.  A context created later (after cudaDeviceReset, say)
//    gets its own lookup on its first call.
//  - Every call shares the same array.  Calls that overlap on the GPU (two
//    streams, or two host threads, in flight at once) race on it, so
//    serialise them.
//  - Each call clears the parts that must start at zero (the cell counts)
//    before using them.  Nothing else carries over from the previous call.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "launch.cuh"

namespace sphfem {
namespace {

constexpr int kNoAllocMaxParticles = 262144;
constexpr int kNoAllocMaxCells = 262143;              // buckets = cells + 1 (out-of-grid)
constexpr int kNoAllocBuckets = kNoAllocMaxCells + 1;
constexpr int kScanItemsNA = 256;                     // per thread, single block of 1024 threads
constexpr int kNoAllocWords = 3 * kNoAllocMaxParticles   // key, arrival, slots
                              + kNoAllocBuckets          // counts
                              + kNoAllocBuckets + 1;     // offsets
static_assert(kNoAllocBuckets <= 1024 * kScanItemsNA, "single-block scan must cover every bucket");

static __device__ __align__(256) int32_t g_cells_scratch[kNoAllocWords];

struct ScratchView {
    int32_t *key, *arrival, *slots, *counts, *offsets;
};

__host__ __device__ inline ScratchView carve(int32_t *base) {
    ScratchView v;
    v.key = base;
    v.arrival = v.key + kNoAllocMaxParticles;
    v.slots = v.arrival + kNoAllocMaxParticles;
    v.counts = v.slots + kNoAllocMaxParticles;
    v.offsets = v.counts + kNoAllocBuckets;
    return v;
}

// compute_hashes (grid.cu:25-42) + the counting-sort histogram
__global__ void __launch_bounds__(kBlock) k_na_hash_count(int n, const double2 *__restrict__ pos,
                                                          const double *__restrict__ blanked,
                                                          int32_t *__restrict__ hash, sph_geom_constants g,
                                                          float inv_dxf, ScratchView X) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int h;
    if (blanked[i] != 1.) {
        double2 p = pos[i];
        int ix = cell_coord(p.x, g.bbmin_x, g.dx, inv_dxf);
        int iy = cell_coord(p.y, g.bbmin_y, g.dx, inv_dxf);
        h = ix * g.ny + iy;
        hash[i] = h;
    } else {
        h = hash[i];
    }
    int k = (h < 0 || h >= g.num_cell) ? g.num_cell : h;
    X.key[i] = k;
    X.arrival[i] = histogram_slot(X.counts, k);
}

// exclusive scan of the buckets in one block; also writes cell_start /
// cell_end like grid_gpu_green (empty cells: start -1, end untouched)
__global__ void __launch_bounds__(1024) k_na_scan(int buckets, int num_cell, ScratchView X,
                                                  int32_t *__restrict__ cell_start, int32_t *__restrict__ cell_end) {
    __shared__ int warp_sums[32];
    const int base = threadIdx.x * kScanItemsNA;
    int s = 0;
    for (int k = 0; k < kScanItemsNA; k++)
        if (base + k < buckets) s += X.counts[base + k];
    // block exclusive scan of the per-thread sums
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = s;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    int ex = (wid > 0 ? warp_sums[wid - 1] : 0) + x - s;
    for (int k = 0; k < kScanItemsNA; k++) {
        int c = base + k;
        if (c >= buckets) break;
        int cnt = X.counts[c];
        X.offsets[c] = ex;
        if (c < num_cell) {
            if (cnt > 0) {
                cell_start[c] = ex;
                cell_end[c] = ex + cnt;
            } else {
                cell_start[c] = -1;
            }
        }
        if (c == buckets - 1) X.offsets[buckets] = ex + cnt;
        ex += cnt;
    }
}

__global__ void __launch_bounds__(kBlock) k_na_scatter(int n, ScratchView X) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    X.slots[X.offsets[X.key[i]] + X.arrival[i]] = i;
}

// stable order inside a cell: rank by original index (thrust::sort_by_key order)
__global__ void __launch_bounds__(kBlock) k_na_rank(int n, ScratchView X, const int32_t *__restrict__ hash,
                                                    int32_t *__restrict__ perm, int32_t *__restrict__ hash_sorted) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    int i = X.slots[s];
    int c = X.key[i];
    int cs = X.offsets[c], ce = X.offsets[c + 1];
    int rank = 0;
    for (int t = cs; t < ce; t++) rank += (X.slots[t] < i) ? 1 : 0;
    perm[cs + rank] = i;
    if (hash_sorted) hash_sorted[cs + rank] = hash[i];
}

// Address of g_cells_scratch in the CUDA context current at the call.  A
// module's __device__ array has one copy per context: the device's primary
// context (what the runtime API uses by default) and every context an
// application creates itself with the driver API (cuCtxCreate) each hold
// their own.  The cache is therefore keyed on the context's unique id
// (cuCtxGetId, never reused within a process), not on the device ordinal:
// after cudaDeviceReset the primary context is a new one with a new id, and
// the lookup runs again.
typedef int (*PFN_ctx_current)(void **ctx);
typedef int (*PFN_ctx_id)(void *ctx, unsigned long long *id);
constexpr int kCacheSlots = 64;
struct ScratchSlot {
    unsigned long long ctx_id;
    int32_t *addr;
};
ScratchSlot g_scratch_cache[kCacheSlots] = {};
int g_scratch_next = 0;
PFN_ctx_current g_ctx_current = nullptr;
PFN_ctx_id g_ctx_id = nullptr;
std::mutex g_scratch_mu;

int current_context_id(unsigned long long *id, char *err, int err_len) {
    if (!g_ctx_current || !g_ctx_id) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
        cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
            q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
            if (err && err_len > 0)
                snprintf(err, err_len, "driver entry points cuCtxGetCurrent / cuCtxGetId unavailable: %s",
                         cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
            return SPH_ERR_NO_DEVICE;
        }
        g_ctx_current = (PFN_ctx_current)f1;
        g_ctx_id = (PFN_ctx_id)f2;
    }
    void *ctx = nullptr;
    if (g_ctx_current(&ctx) == 0 && !ctx) {
        // no context current yet: make the device's primary context current (no
        // allocation); with a context of the caller's current this is not reached
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaSetDevice(dev) == cudaSuccess) g_ctx_current(&ctx);
    }
    if (!ctx || g_ctx_id(ctx, id) != 0) {
        if (err && err_len > 0) snprintf(err, err_len, "no current CUDA context");
        return SPH_ERR_NO_DEVICE;
    }
    return SPH_OK;
}

int scratch_for_current_context(int32_t **out, char *err, int err_len) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0) {
        if (err && err_len > 0) snprintf(err, err_len, "cudaGetDevice failed: %s", cudaGetErrorString(e));
        return SPH_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    unsigned long long id = 0;
    int r = current_context_id(&id, err, err_len);
    if (r != SPH_OK) return r;
    for (const ScratchSlot &s : g_scratch_cache)
        if (s.addr && s.ctx_id == id) {
            *out = s.addr;
            return SPH_OK;
        }
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_cells_scratch);
    if (e != cudaSuccess || !p) {
        if (err && err_len > 0)
            snprintf(err, err_len, "cudaGetSymbolAddress(g_cells_scratch) failed on device %d: %s", dev,
                     cudaGetErrorString(e));
        return SPH_ERR_CUDA;
    }
    g_scratch_cache[g_scratch_next] = {id, (int32_t *)p};   // oldest entry replaced when full
    g_scratch_next = (g_scratch_next + 1) % kCacheSlots;
    *out = (int32_t *)p;
    return SPH_OK;
}

}  // namespace
}  // namespace sphfem

using namespace sphfem;

extern "C" int sph_cells_build_noalloc(const double *pos, const double *blanked, int32_t *hash, int32_t n,
                                       const sph_geom_constants *g, int32_t *perm, int32_t *hash_sorted,
                                       int32_t *cell_start, int32_t *cell_end, void *stream, char *err,
                                       int32_t err_len) {
    if (err && err_len > 0) err[0] = '\0';
    if (!pos || !blanked || !hash || !g || !perm || !cell_start || !cell_end || n < 1) {
        if (err && err_len > 0) snprintf(err, err_len, "sph_cells_build_noalloc: missing array or n < 1");
        return SPH_ERR_INVALID;
    }
    if (n > kNoAllocMaxParticles || g->num_cell < 1 || g->num_cell > kNoAllocMaxCells) {
        if (err && err_len > 0)
            snprintf(err, err_len,
                     "sph_cells_build_noalloc: %d particles / %d cells exceed the fixed scratch "
                     "(at most %d particles and %d cells)",
                     n, g->num_cell, kNoAllocMaxParticles, kNoAllocMaxCells);
        return SPH_ERR_INVALID;
    }
    int32_t *base = nullptr;
    int r = scratch_for_current_context(&base, err, err_len);
    if (r != SPH_OK) return r;
    ScratchView X = carve(base);
    cudaStream_t s = (cudaStream_t)stream;
    const int buckets = g->num_cell + 1;
    cudaError_t e = cudaMemsetAsync(X.counts, 0, sizeof(int32_t) * (size_t)buckets, s);
    if (e == cudaSuccess) {
        const int grid = div_up(n, kBlock);
        k_na_hash_count<<<grid, kBlock, 0, s>>>(n, (const double2 *)pos, blanked, hash, *g, (float)(1.0 / g->dx), X);
        k_na_scan<<<1, 1024, 0, s>>>(buckets, g->num_cell, X, cell_start, cell_end);
        k_na_scatter<<<grid, kBlock, 0, s>>>(n, X);
        k_na_rank<<<grid, kBlock, 0, s>>>(n, X, hash, perm, hash_sorted);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        if (err && err_len > 0) snprintf(err, err_len, "sph_cells_build_noalloc: %s", cudaGetErrorString(e));
        return SPH_ERR_CUDA;
    }
    return SPH_OK;
}
