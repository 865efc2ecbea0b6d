// common.cuh -- shared device-side definitions of the sm_103a SPH hot path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sphfem.h"

namespace sphfem {

// 32-byte aligned 4-vector of doubles (CUDA 13 deprecates the 16-byte-aligned
// double4); cudaMalloc'd arrays of it allow 256-bit accesses.
using dbl4 = double4_32a;
__host__ __device__ __forceinline__ dbl4 mk4(double x, double y, double z, double w) {
    return make_double4_32a(x, y, z, w);
}

constexpr int kBlock = 256;          // particle kernels
constexpr int kMaxStencil = 3;       // the pair list packs the column offset in 3 bits
constexpr int kCellRankCap = 4096;   // cells larger than this are ranked by the slow path
constexpr double kPiFac = 0.454728408833987;   // PI_FAC, kernels.cuh:19 (10/(7 pi))

struct JcF32 {   // Johnson-Cook constants in FP32 (plasticity.cuh:21-39)
    float A, B, C, n, m, Tref, inv_dT, inv_epsdot_ref, Tmelt;
};

// FP32 copies of the constants the FP32-compensated kernels use, computed
// once on the host: on GB300 a per-thread double->float conversion or double
// division runs on the narrow FP64 pipe in every warp.
struct KF32 {
    float mass, inv_mass, xs_mass, alpha, beta, eta2, inv_wdp, cell, G, K_bulk, c0sq, stresseps;
    float dt, hdt, inv_dt, tq_over_cp, alpha_wp, alpha_tool_sph, T_init;
    float inv_cell;   // (float)(1 / cell edge), for cell_coord
    JcF32 jc;
};

// Every constant a kernel needs, passed by value (lands in the kernel
// parameter bank; no __constant__ symbol, so CUDA graphs capture it as is).
struct KConsts {
    sph_constants c;
    sph_geom_constants g;
    double dt;
    // derived once on the host
    double c0sq;          // (sqrtf(K/rho0))^2 of do_material_eos (actions_gpu.cu:228-230)
    double inv_wdeltap;   // 1/wdeltap (interactions_gpu.cu:269)
    double eta2;          // eta*eta (interactions_gpu.cu:301)
    double inv_dx;        // 1/cell edge
    int32_t has_tool;
    int32_t precision;
    int32_t thermal_bc;   // m_thermal: thermals_tool.alpha != 0 (actions_gpu.cu:938-944)
    int32_t n_cases;      // 1, or the number of cases of a batched context
    KF32 f;
    // batched contexts: case of every grid column / FEM node / segment (NULL: one case)
    const uint16_t *case_of_col;
    const uint16_t *case_of_node;
    const uint16_t *case_of_seg;
    // return mapping: state log, statistics and the learned warm start (NULL: off)
    float *jc_log;                        // [jc_log_cap][kJcLogWidth]
    unsigned long long *jc_log_count;     // records offered (may exceed the capacity)
    long long jc_log_cap;
    unsigned long long *jc_stats;         // [0] return mappings, [1] secant iterations
    int32_t *jc_list;                     // yielding particles deferred to the warm-started return mapping
    int32_t *jc_list_count;
    // rigid tool (device copy, moved every step) and the PSE conduction switch
    sph_rigid_tool *rigid;
    int32_t thermal_pse;
    // secant iterations before SPH_STATUS_SECANT_MAXITER (the reference's 100;
    // sph_set_test_faults may lower it) and the failure-path test bits (SPH_TEST_*)
    int32_t secant_cap;
    uint32_t test_faults;
};

// One logged return mapping: trial von Mises stress, equivalent plastic
// strain and its rate before the step, temperature, |dev S_trial|, the
// converged plastic-multiplier increment, secant iterations, time step.
constexpr int kJcLogWidth = 8;

__device__ __forceinline__ void jc_log_record(const KConsts &K, float svm, float eps, float epsd, float T, float norm,
                                              float dl, int iters, float dt) {
    if (!K.jc_log) return;
    unsigned long long at = atomicAdd(K.jc_log_count, 1ull);
    if ((long long)at >= K.jc_log_cap) return;
    float4 *r = (float4 *)(K.jc_log + at * kJcLogWidth);
    r[0] = make_float4(svm, eps, epsd, T);
    r[1] = make_float4(norm, dl, (float)iters, dt);
}

// Return-mapping counters, aggregated over the active lanes of the warp.
__device__ __forceinline__ void jc_count(const KConsts &K, int iters) {
    if (!K.jc_stats) return;
    const unsigned mask = __activemask();
    const unsigned n = __popc(mask);
    const unsigned it = __reduce_add_sync(mask, (unsigned)iters);
    if ((threadIdx.x & 31) == __ffs(mask) - 1) {
        atomicAdd(K.jc_stats, (unsigned long long)n);
        atomicAdd(K.jc_stats + 1, (unsigned long long)it);
    }
}

// Case of a particle from its cell hash (its grid column).
__device__ __forceinline__ int case_of_hash(const KConsts &K, int hash) {
    if (!K.case_of_col) return 0;
    int ix = hash / K.g.ny;
    ix = ix < 0 ? 0 : (ix >= K.g.nx ? K.g.nx - 1 : ix);
    return K.case_of_col[ix];
}

// ---- flags stored as double 0/1 (particle_gpu.h:41-43), tested on the integer
// pipe: GB300's FP64 pipe is narrow and a double compare occupies it.
__device__ __forceinline__ bool flag_is_one(double v) {            // v == 1.
    return __double_as_longlong(v) == 0x3FF0000000000000LL;
}
__device__ __forceinline__ bool flag_nonzero(double v) {           // v != 0. (NaN counts as non-zero)
    return (__double_as_longlong(v) << 1) != 0;
}
__device__ __forceinline__ bool is_nan_or_inf(double v) {          // isnan(v) || isinf(v)
    return (__double_as_longlong(v) & 0x7FF0000000000000LL) == 0x7FF0000000000000LL;
}

// The same tests on the 0/1 flags of the compact FP32 state.
__device__ __forceinline__ bool flag_is_one(float v) { return __float_as_int(v) == 0x3F800000; }
__device__ __forceinline__ bool flag_nonzero(float v) { return (__float_as_int(v) << 1) != 0; }
__device__ __forceinline__ bool is_nan_or_inf(float v) { return (__float_as_int(v) & 0x7F800000) == 0x7F800000; }

// Values of either state form widened to FP64, and FP64 values stored into
// either form (rounded once to FP32 in the compact form).
__device__ __forceinline__ double2 d2(double2 v) { return v; }
__device__ __forceinline__ double2 d2(float2 v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ dbl4 d4(dbl4 v) { return v; }
__device__ __forceinline__ dbl4 d4(float4 v) { return mk4(v.x, v.y, v.z, v.w); }
__device__ __forceinline__ void put(double2 &dst, double2 v) { dst = v; }
__device__ __forceinline__ void put(float2 &dst, double2 v) { dst = make_float2((float)v.x, (float)v.y); }
__device__ __forceinline__ void put(dbl4 &dst, dbl4 v) { dst = v; }
__device__ __forceinline__ void put(float4 &dst, dbl4 v) {
    dst = make_float4((float)v.x, (float)v.y, (float)v.z, (float)v.w);
}
__device__ __forceinline__ void put(double &dst, double v) { dst = v; }
__device__ __forceinline__ void put(float &dst, double v) { dst = (float)v; }

// compute_hashes' cell index (int)((x - bbmin)/dx) (grid.cu:36-39), bit for bit.
// The quotient is first formed in FP32 with inv_dxf = (float)(1/dx): against the
// FP64 quotient its error is below 3*2^-24 relative (three FP32 roundings and the
// FP64 division's own), so when its fractional part is more than 2.5e-7*q away
// from an integer both truncate to the same cell and the FP64 division -- a long
// sequence on GB300's narrow FP64 pipe -- is skipped.  Negative, huge or
// non-finite offsets take the FP64 division.
__device__ __forceinline__ int cell_coord(double x, double bbmin, double dx, float inv_dxf) {
    const double a = x - bbmin;
    if (a >= 0.) {
        const float qf = (float)a * inv_dxf;
        const float t = truncf(qf);
        const float fr = qf - t;
        const float m = 2.5e-7f * qf + 1e-30f;
        if (fr > m && fr < 1.f - m) return (int)t;
    }
    return __double2int_rz(a / dx);
}

// A slot in bucket `key` of a histogram (the counting sort's arrival index):
// the lanes of a warp with the same key -- consecutive particles mostly share
// a cell -- take their slots with one atomic, in lane order.  Any order inside
// a bucket is valid: the rank pass orders each cell by original index.
// One-dimensional blocks (lane = threadIdx.x % 32).
__device__ __forceinline__ int histogram_slot(int32_t *counts, int key) {
    const unsigned active = __activemask();
    const unsigned peers = __match_any_sync(active, key);
    const int lane = (int)(threadIdx.x & 31u);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counts + key, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

// Device copy of the rigid tool kinematics that tool_FEM keeps on the host
// (tool_FEM.h:57-77); updated by the tool-move kernel so a captured CUDA graph
// needs no host round trip.
// In a batched context there is one per case, with the case's time step and
// its range of interface segments.
struct ToolDev {
    double vel[2];
    double tl_point_ref[2];
    double br_point[2];
    double ref_dist;
    double lowest_point, right_point;
    double dt, hdt;                 // time step of the case and half of it
    float dtf, hdtf, inv_dtf;       // the same in FP32
    int32_t seg_first, seg_count;   // the case's interface segments
    double seg_ymin, seg_ymax;      // y-range of those segments (moved with them)
    double seg_xmax;                // largest x of their end points (moved with them)
    double seg_dxdy;                // largest |dx/dy| of a non-horizontal segment
    double flank_retreat;           // wear: added to the y motion of nodes and segments (tool_FEM.cu:19)
    double flank_contact;           // wear: lowest_point after the last tool update (tool_FEM.cu:20)
    double bin_y0, bin_scale;       // segment y-bins: bin = floor((y - bin_y0) * bin_scale) (k_seg_bins)
    // the contact pre-filter's bounds as order keys (k_seg_bins): float-rounded
    // segment y-range and the x bound right of which no crossing can lie
    long long key_y0, key_y1, key_x1;
};

// Order key of a double: for non-NaN a, b, a <= b exactly when key(a) <= key(b)
// as signed integers (sign-magnitude bits made two's-complement ordered; -0
// taken as +0).  NaN keys sort outside every finite range, so a NaN fails a
// two-sided range test as the IEEE comparisons do.  Compares on the integer
// pipe: GB300's FP64 pipe is narrow.
__device__ __forceinline__ long long order_key(double x) {
    long long b = __double_as_longlong(x);
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
// The double of an order key (the inverse map; -0 comes back as +0).
__device__ __forceinline__ double order_key_value(long long k) {
    return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffll));
}

// Per-segment wear statistics gathered by the friction-heat kernel
// (WEAR_NODE_SHIFT, actions_gpu.cu:401-419); pp == NULL: not gathered.
struct WearAcc {
    dbl4 *pp;                 // count, sum contact pressure, sum sliding speed, sum segment T
    double *sf;               // sum sliding force / length
    const int4 *marks;        // segment nodes (z: left, w: right)
    const double *T_nodes;    // FEM nodal temperature when the friction heat runs
};

// ---- float narrowings of the reference (double argument -> float call) ------
__device__ __forceinline__ double sqrtf_d(double x) { return (double)sqrtf((float)x); }
__device__ __forceinline__ double fmaxf_d(double a, double b) { return (double)fmaxf((float)a, (float)b); }
__device__ __forceinline__ double fminf_d(double a, double b) { return (double)fminf((float)a, (float)b); }
// atan2f/cosf/sinf of the artificial stress: evaluated in double, rounded once
// to float, the same formulation as the CPU oracle so both sides agree.
__device__ __forceinline__ float sph_atan2f(float y, float x) { return (float)atan2((double)y, (double)x); }
__device__ __forceinline__ float sph_cosf(float x) { return (float)cos((double)x); }
__device__ __forceinline__ float sph_sinf(float x) { return (float)sin((double)x); }

__device__ __forceinline__ void set_status(uint32_t *status, uint32_t bits) {
    if (status) atomicOr(status, bits);
}

// Non-contracted a + b*c (keeps host and device bit-identical for the tool kinematics).
__device__ __forceinline__ double add_mul_rn(double a, double b, double c) { return __dadd_rn(a, __dmul_rn(b, c)); }

__host__ __device__ __forceinline__ int div_up(int64_t a, int b) { return (int)((a + b - 1) / b); }

}  // namespace sphfem
