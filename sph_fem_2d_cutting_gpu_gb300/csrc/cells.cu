// cells.cu -- cell-list build on sm_103a: hashing (grid.cu:25-42), the stable
// key sort of grid_gpu_green (grid_gpu_green.cu:185-209) and the cell tables
// plus reorder gather (grid_gpu_green.cu:13-115).
//
// The sort is a counting sort over cells rather than a radix sort: keys are
// cell ids of a locked grid, so one histogram, one scan and one scatter give
// every particle its cell's slot range.  The order inside a cell is then made
// identical to thrust::sort_by_key's stable order by ranking each particle
// among its cell-mates by original index.  The scan also yields cell_start /
// cell_end directly.
#include "cells.cuh"

namespace sphfem {

// ---- hashing: grid.cu:25-42 compute_hashes --------------------------------------
// kHash: write hash for non-blanked particles (blanked keep their stale hash).
// kCount: derive the sort key and take an arrival slot in the key's bucket.
template <bool kHash, bool kCount, class Bl>
__global__ void __launch_bounds__(kBlock) k_hash_count(int N, const double2 *__restrict__ pos,
                                                       const Bl *__restrict__ blanked, int32_t *__restrict__ hash,
                                                       int32_t *__restrict__ key, int32_t *__restrict__ arrival,
                                                       int32_t *__restrict__ counts, int32_t *__restrict__ hash_next,
                                                       sph_geom_constants g, float inv_dxf, uint32_t *status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    int h;
    if (kHash && !flag_is_one(blanked[i])) {
        double2 p = pos[i];
        int ix = cell_coord(p.x, g.bbmin_x, g.dx, inv_dxf);
        int iy = cell_coord(p.y, g.bbmin_y, g.dx, inv_dxf);
        h = ix * g.ny + iy;
        hash[i] = h;
    } else {
        h = hash[i];
    }
    if (kCount) {
        int k = h;
        if (h < 0 || h >= g.num_cell) {
            k = g.num_cell;
            set_status(status, SPH_STATUS_OUT_OF_GRID);
        }
        key[i] = k;
        arrival[i] = histogram_slot(counts, k);
        hash_next[i] = h;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int32_t *__restrict__ in, int n,
                                                              int32_t *__restrict__ block_sums) {
    __shared__ int sw[32];
    int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) s += in[base + k];
    int total;
    block_exclusive_scan(s, sw, total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_top(int32_t *__restrict__ block_sums, int nb) {
    __shared__ int sw[32];
    int carry = 0;
    for (int base = 0; base < nb; base += blockDim.x) {
        int i = base + threadIdx.x;
        int v = (i < nb) ? block_sums[i] : 0;
        int total;
        int ex = block_exclusive_scan(v, sw, total);
        if (i < nb) block_sums[i] = carry + ex;
        carry += total;
    }
}

// Writes offsets[0..n] (n = num_cell + 1 buckets, offsets[n] = N) and the
// reference's cell tables: cell_start = first slot or -1 when empty; cell_end
// = one past the last slot, left untouched for empty cells (stale, as the
// reference leaves it).
__global__ void __launch_bounds__(kScanThreads) k_scan_down(const int32_t *__restrict__ counts, int n,
                                                            const int32_t *__restrict__ block_sums,
                                                            int32_t *__restrict__ offsets,
                                                            int32_t *__restrict__ cell_start,
                                                            int32_t *__restrict__ cell_end, int num_cell) {
    __shared__ int sw[32];
    int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = (base + k < n) ? counts[base + k] : 0;
        s += v[k];
    }
    int total;
    int ex = block_exclusive_scan(s, sw, total) + block_sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int c = base + k;
        if (c < n) {
            offsets[c] = ex;
            if (c < num_cell) {
                if (v[k] > 0) {
                    cell_start[c] = ex;
                    cell_end[c] = ex + v[k];
                } else {
                    cell_start[c] = -1;
                }
            }
            if (c == n - 1) offsets[n] = ex + v[k];
        }
        ex += v[k];
    }
}

// ---- scatter into the cell's slot range (arbitrary order inside the cell) -------------
__global__ void __launch_bounds__(kBlock) k_scatter(int N, const int32_t *__restrict__ key,
                                                    const int32_t *__restrict__ arrival,
                                                    const int32_t *__restrict__ offsets, int32_t *__restrict__ slots) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) scatter_one(i, key, arrival, offsets, slots);
}

__global__ void __launch_bounds__(kBlock) k_rank(int N, const int32_t *__restrict__ key,
                                                 const int32_t *__restrict__ offsets,
                                                 const int32_t *__restrict__ slots, int32_t *__restrict__ perm,
                                                 uint32_t *status) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < N) rank_one(s, key, offsets, slots, perm, status);
}

// ---- reorder gather (grid_gpu_green.cu:55-113) ----------------------------------------------
__global__ void __launch_bounds__(kBlock) k_gather_plain(int N, const int32_t *__restrict__ perm, SortedFields A,
                                                         SortedFields B) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    int i = perm[k];
    B.pos[k] = A.pos[i];
    B.vel[k] = A.vel[i];
    B.fc[k] = A.fc[i];
    B.ft[k] = A.ft[i];
    B.h[k] = A.h[i];
    B.n[k] = A.n[i];
    B.rho[k] = A.rho[i];
    B.S[k] = A.S[i];
    B.eps_pl[k] = A.eps_pl[i];
    B.eps_pl_dot[k] = A.eps_pl_dot[i];
    B.T[k] = A.T[i];
    B.fixed[k] = A.fixed[i];
    B.blanked[k] = A.blanked[i];
    B.tool_particle[k] = A.tool_particle[i];
    B.pos_t[k] = A.pos_t[i];
    B.vel_t[k] = A.vel_t[i];
    B.rho_t[k] = A.rho_t[i];
    B.S_t[k] = A.S_t[i];
    B.T_t[k] = A.T_t[i];
    B.on_seg[k] = A.on_seg[i];
    B.hash[k] = A.hash[i];
}

// ---- neighbour records ----------------------------------------------------------------

// FP64 record: (x, y, vx, vy) (sA, sB, sC, Rxx) (Rxy, Ryy, h, rho) (c, vol, T, flags)
// with sA = (Sxx-p)/rho^2, sB = Sxy/rho^2, sC = (Syy-p)/rho^2 (interactions_gpu.cu:278-281),
// c = sqrtf(K/rho) (:294-295), vol = mass/rho (:250).
__device__ __forceinline__ void write_record64(dbl4 *__restrict__ rec, int k, const KConsts &K, double2 pos,
                                               double2 vel, dbl4 S, dbl4 R, double p, double h, double rho,
                                               double T, double blanked, double tool, int row) {
    double rho21 = 1. / (rho * rho);
    dbl4 r0 = mk4(pos.x, pos.y, vel.x, vel.y);
    dbl4 r1 = mk4((S.x - p) * rho21, S.y * rho21, (S.z - p) * rho21, R.x);
    dbl4 r2 = mk4(R.y, R.z, h, rho);
    int flags = (row & kRowMask) | (blanked == 1. ? kFlagBlanked : 0) | (tool == 1. ? kFlagTool : 0);
    const double c = sqrtf_d(K.c.phys.K / rho), vol = K.c.phys.mass / rho;
    if (!(flags & kFlagBlanked) && (nonfinite4(r0) || nonfinite4(r1) || nonfinite4(r2) || is_nan_or_inf(c) ||
                                    is_nan_or_inf(vol) || is_nan_or_inf(T)))
        flags |= kFlagNonFinite;   // blanked records are skipped as neighbours: no mark
    dbl4 r3 = mk4(c, vol, T, __longlong_as_double((long long)flags));
    rec[4 * k + 0] = r0;
    rec[4 * k + 1] = r1;
    rec[4 * k + 2] = r2;
    rec[4 * k + 3] = r3;
}

// FP32 record: (xr, yr, flags|row, h) (vx, vy, rho, c) (sA, sB, sC, vol) (Rxx, Rxy, Ryy, T)
// xr, yr = offset of the particle from its cell's lower-left corner; the first
// 16 bytes are all the candidate test needs.
__device__ __forceinline__ void write_record32(float4 *__restrict__ rec, float2 *__restrict__ cand, int k,
                                               const KConsts &K, double2 pos,
                                               double2 vel, dbl4 S, dbl4 R, double p, double h, double rho,
                                               double T, double blanked, double tool, int hash) {
    const sph_geom_constants &g = K.g;
    int ci = 0, cj = 0;
    if (hash >= 0 && hash < g.num_cell) { ci = hash / g.ny; cj = hash - ci * g.ny; }
    double xr = pos.x - (g.bbmin_x + (double)ci * g.dx);
    double yr = pos.y - (g.bbmin_y + (double)cj * g.dx);
    double rho21 = 1. / (rho * rho);
    int flags = (cj & kRowMask) | (blanked == 1. ? kFlagBlanked : 0) | (tool == 1. ? kFlagTool : 0);
    float4 r0 = make_float4((float)xr, (float)yr, 0.f, (float)h);
    const float4 r1 = make_float4((float)vel.x, (float)vel.y, (float)rho, sqrtf((float)(K.c.phys.K / rho)));
    const float4 r2 = make_float4((float)((S.x - p) * rho21), (float)(S.y * rho21), (float)((S.z - p) * rho21),
                                  (float)(K.c.phys.mass / rho));
    const float4 r3 = make_float4((float)R.x, (float)R.y, (float)R.z, (float)T);
    if (!(flags & kFlagBlanked) && (nonfinite4(r0) || nonfinite4(r1) || nonfinite4(r2) || nonfinite4(r3)))
        flags |= kFlagNonFinite;   // blanked records are skipped as neighbours: no mark
    r0.z = __int_as_float(flags);
    rec[4 * k + 0] = r0;
    rec[4 * k + 1] = r1;
    rec[4 * k + 2] = r2;
    rec[4 * k + 3] = r3;
    cand[k] = cand_pack(r0.x, r0.y, flags);
}

// Staged path helper: records from the particle arrays as they are now
// (interactions_monaghan reads pos, vel, S, R, h, rho, p, T, tool, blanked).
__global__ void __launch_bounds__(kBlock) k_build_records(int N, KConsts K, SortedFields A, FixedFields F,
                                                          dbl4 *__restrict__ rec64, float4 *__restrict__ rec32,
                                                          float2 *__restrict__ cand32) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    double tool = A.tool_particle[k];
    // every record carries T: a particle whose own diffusivity is zero (a tool
    // particle of a non-conducting tool) still passes its temperature to the
    // conducting neighbours that sum over it (interactions_gpu.cu:242-247 gate
    // the fetch on the summing particle's alpha, not the neighbour's)
    double T = A.T[k];
    int hash = A.hash[k];
    if (rec64) {
        int row = 0;
        if (hash >= 0 && hash < K.g.num_cell) row = hash - (hash / K.g.ny) * K.g.ny;
        write_record64(rec64, k, K, A.pos[k], A.vel[k], A.S[k], F.R[k], F.p[k], A.h[k], A.rho[k], T, A.blanked[k],
                       tool, row);
    } else {
        write_record32(rec32, cand32, k, K, A.pos[k], A.vel[k], A.S[k], F.R[k], F.p[k], A.h[k], A.rho[k], T, A.blanked[k],
                       tool, hash);
    }
}

// Fused reorder: gather (grid_gpu_green.cu:55-113) + init snapshot (the sorted
// state itself, leap_frog.cu:25-37) + predict (leap_frog.cu:45-69) +
// do_material_eos (actions_gpu.cu:222-232) + do_corrector_artificial_stress
// (actions_gpu.cu:234-278) + the neighbour record of the predicted state.
// The sorted arrays B keep the start-of-step state (the reference's *_init
// snapshots); the predicted values live only in the records and in p / R.
// hash_src: the hashes the histogram pass took (compute_hashes of this step).
template <bool kF32>
__global__ void __launch_bounds__(kBlock) k_gather_fused(int N, const int32_t *__restrict__ perm, KConsts K,
                                                         SortedFields A, SortedFields B, FixedFields F,
                                                         const int32_t *__restrict__ hash_src,
                                                         dbl4 *__restrict__ rec64, float4 *__restrict__ rec32,
                                                         float2 *__restrict__ cand32, const ToolDev *__restrict__ tools) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    int i = perm[k];
    F.idx[k] = i;
    double2 pos = A.pos[i], vel = A.vel[i];
    dbl4 S = A.S[i];
    double rho = A.rho[i], T = A.T[i], h = A.h[i];
    double blanked = A.blanked[i], tool = A.tool_particle[i];
    double2 pos_t = A.pos_t[i], vel_t = A.vel_t[i];
    double rho_t = A.rho_t[i], T_t = A.T_t[i];
    dbl4 S_t = A.S_t[i];
    int hash = hash_src[i];
    B.pos[k] = pos;
    B.vel[k] = vel;
    B.fc[k] = A.fc[i];
    B.ft[k] = A.ft[i];
    B.h[k] = h;
    B.n[k] = A.n[i];
    B.rho[k] = rho;
    B.S[k] = S;
    B.eps_pl[k] = A.eps_pl[i];
    B.eps_pl_dot[k] = A.eps_pl_dot[i];
    B.T[k] = T;
    B.fixed[k] = A.fixed[i];
    B.blanked[k] = blanked;
    B.tool_particle[k] = tool;
    B.pos_t[k] = pos_t;
    B.vel_t[k] = vel_t;
    B.rho_t[k] = rho_t;
    B.S_t[k] = S_t;
    B.T_t[k] = T_t;
    B.on_seg[k] = A.on_seg[i];
    B.hash[k] = hash;
    // predict (half step) for active particles
    if (blanked != 1.) {
        const double hdt = tools[case_of_hash(K, hash)].hdt;   // half the time step of the particle's case
        pos.x = pos.x + hdt * pos_t.x;
        pos.y = pos.y + hdt * pos_t.y;
        vel.x = vel.x + hdt * vel_t.x;
        vel.y = vel.y + hdt * vel_t.y;
        S.x = S.x + hdt * S_t.x;
        S.y = S.y + hdt * S_t.y;
        S.z = S.z + hdt * S_t.z;
        S.w = S.w + hdt * S_t.w;
        rho = rho + hdt * rho_t;
        T = T + hdt * T_t;
    }
    double p = F.p[k];
    dbl4 R = F.R[k];
    if (tool == 0.) {
        p = eos_one(K, rho);
        R = artificial_stress_one(K, rho, p, S);
        F.p[k] = p;
        F.R[k] = R;
    }
    double Tn = T;   // every record carries T (k_build_records)
    if (!kF32) {
        int row = 0;
        if (hash >= 0 && hash < K.g.num_cell) row = hash - (hash / K.g.ny) * K.g.ny;
        write_record64(rec64, k, K, pos, vel, S, R, p, h, rho, Tn, blanked, tool, row);
    } else {
        write_record32(rec32, cand32, k, K, pos, vel, S, R, p, h, rho, Tn, blanked, tool, hash);
    }
}


template <class SF, class FF>
__global__ void __launch_bounds__(kBlock) k_gather_fused32(int N, const int32_t *__restrict__ perm, KConsts K, SF A,
                                                           FF Fsrc, SortedFields32 B, FixedFields32 F,
                                                           int32_t *__restrict__ idx,
                                                           const int32_t *__restrict__ hash_src,
                                                           float4 *__restrict__ rec, float2 *__restrict__ cand,
                                                           const ToolDev *__restrict__ tools) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < N) gather32_one(k, perm, K, A, Fsrc, B, F, idx, hash_src, rec, cand, tools);
}

// The compact FP32 state (state) and its p, R (pr) widened into the FP64
// arrays: exact.
__global__ void __launch_bounds__(kBlock) k_state_to64(int N, SortedFields32 A, FixedFields32 Fa, SortedFields B,
                                                       FixedFields F, bool state, bool pr) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    if (pr) {
        F.p[k] = Fa.p[k];
        const float4 R = Fa.R[k];
        F.R[k] = mk4(R.x, R.y, R.z, 0.);
    }
    if (!state) return;
    B.pos[k] = A.pos[k];
    B.vel[k] = d2(A.vel[k]);
    B.fc[k] = d2(A.fc[k]);
    B.ft[k] = d2(A.ft[k]);
    B.n[k] = d2(A.n[k]);
    B.h[k] = A.h[k];
    B.rho[k] = A.rho[k];
    B.eps_pl[k] = A.eps_pl[k];
    B.eps_pl_dot[k] = A.eps_pl_dot[k];
    B.T[k] = A.T[k];
    B.fixed[k] = A.fixed[k];
    B.blanked[k] = A.blanked[k];
    B.tool_particle[k] = A.tool_particle[k];
    B.S[k] = d4(A.S[k]);
    B.pos_t[k] = d2(A.pos_t[k]);
    B.vel_t[k] = d2(A.vel_t[k]);
    B.rho_t[k] = A.rho_t[k];
    B.T_t[k] = A.T_t[k];
    B.S_t[k] = d4(A.S_t[k]);
    B.on_seg[k] = A.on_seg[k];
    B.hash[k] = A.hash[k];
}

// ---- host launchers ---------------------------------------------------------------------
void launch_hash(cudaStream_t s, int N, const SortedFields &A, sph_geom_constants g) {
    k_hash_count<true, false><<<div_up(N, kBlock), kBlock, 0, s>>>(N, A.pos, A.blanked, A.hash, nullptr, nullptr,
                                                                     nullptr, nullptr, g, (float)(1.0 / g.dx),
                                                                     nullptr);
}

template <class SF>
static void count(cudaStream_t s, int N, const SF &A, const SortScratch &X, sph_geom_constants g, uint32_t *status,
                  bool with_hash) {
    cudaMemsetAsync(X.counts, 0, sizeof(int32_t) * (size_t)(g.num_cell + 1), s);
    if (with_hash)
        k_hash_count<true, true><<<div_up(N, kBlock), kBlock, 0, s>>>(N, A.pos, A.blanked, A.hash, X.key, X.arrival,
                                                                       X.counts, X.hash_next, g, (float)(1.0 / g.dx), status);
    else
        k_hash_count<false, true><<<div_up(N, kBlock), kBlock, 0, s>>>(N, A.pos, A.blanked, A.hash, X.key, X.arrival,
                                                                        X.counts, X.hash_next, g, (float)(1.0 / g.dx), status);
}
void launch_count(cudaStream_t s, int N, const SortedFields &A, const SortScratch &X, sph_geom_constants g,
                  uint32_t *status, bool with_hash) {
    count(s, N, A, X, g, status, with_hash);
}
void launch_count(cudaStream_t s, int N, const SortedFields32 &A, const SortScratch &X, sph_geom_constants g,
                  uint32_t *status, bool with_hash) {
    count(s, N, A, X, g, status, with_hash);
}

int scan_blocks(int num_cell) { return div_up(num_cell + 1, kScanTile); }

void launch_sort_rest(cudaStream_t s, int N, const SortScratch &X, sph_geom_constants g, int32_t *perm,
                      uint32_t *status) {
    const int n = g.num_cell + 1;
    const int nb = scan_blocks(g.num_cell);
    k_scan_reduce<<<nb, kScanThreads, 0, s>>>(X.counts, n, X.block_sums);
    k_scan_top<<<1, 1024, 0, s>>>(X.block_sums, nb);
    k_scan_down<<<nb, kScanThreads, 0, s>>>(X.counts, n, X.block_sums, X.offsets, X.cell_start, X.cell_end, g.num_cell);
    k_scatter<<<div_up(N, kBlock), kBlock, 0, s>>>(N, X.key, X.arrival, X.offsets, X.slots);
    k_rank<<<div_up(N, kBlock), kBlock, 0, s>>>(N, X.key, X.offsets, X.slots, perm, status);
}

void launch_gather_plain(cudaStream_t s, int N, const int32_t *perm, const SortedFields &A, const SortedFields &B) {
    k_gather_plain<<<div_up(N, kBlock), kBlock, 0, s>>>(N, perm, A, B);
}

void launch_gather_fused(cudaStream_t s, int N, const int32_t *perm, const KConsts &K, const SortedFields &A,
                         const SortedFields &B, const FixedFields &F, const StepScratch &W, const int32_t *hash_src,
                         const ToolDev *tool) {
    const int tb = fp64_block(N);   // EOS and artificial stress per particle: spread small systems
    k_gather_fused<false><<<div_up(N, tb), tb, 0, s>>>(N, perm, K, A, B, F, hash_src, W.rec64, W.rec32, W.cand32, tool);
}

void launch_gather_fused32(cudaStream_t s, int N, const int32_t *perm, const KConsts &K, const SortedFields *A64,
                           const SortedFields32 *A32, bool pr32, const FixedFields &F, const FixedFields32 &F32,
                           const SortedFields32 &B, int32_t *idx, const StepScratch &W, const int32_t *hash_src,
                           const ToolDev *tool) {
    const int tb = fp64_block(N), g = div_up(N, tb);
    if (A32 && pr32)
        k_gather_fused32<<<g, tb, 0, s>>>(N, perm, K, *A32, F32, B, F32, idx, hash_src, W.rec32, W.cand32, tool);
    else if (A32)
        k_gather_fused32<<<g, tb, 0, s>>>(N, perm, K, *A32, F, B, F32, idx, hash_src, W.rec32, W.cand32, tool);
    else if (pr32)
        k_gather_fused32<<<g, tb, 0, s>>>(N, perm, K, *A64, F32, B, F32, idx, hash_src, W.rec32, W.cand32, tool);
    else
        k_gather_fused32<<<g, tb, 0, s>>>(N, perm, K, *A64, F, B, F32, idx, hash_src, W.rec32, W.cand32, tool);
}

void launch_state_to64(cudaStream_t s, int N, const SortedFields32 &A, const FixedFields32 &Fa, const SortedFields &B,
                       const FixedFields &F, bool state, bool pr) {
    k_state_to64<<<div_up(N, kBlock), kBlock, 0, s>>>(N, A, Fa, B, F, state, pr);
}

void launch_build_records(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F,
                          const StepScratch &W) {
    k_build_records<<<div_up(N, kBlock), kBlock, 0, s>>>(N, K, A, F, K.precision == SPH_PREC_FP32K ? nullptr : W.rec64,
                                                         W.rec32, W.cand32);
}

}  // namespace sphfem
