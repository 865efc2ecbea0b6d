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
constexpr int kCellRankCap = 4096;   // cells larger than this are ranked by the slow path
constexpr double kPiFac = 0.454728408833987;   // PI_FAC, kernels.cuh:19 (10/(7 pi))

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
    int32_t has_tool;
    int32_t precision;
};

// Device copy of the rigid tool kinematics that tool_FEM keeps on the host
// (tool_FEM.h:57-77); updated by the tool-move kernel so a captured CUDA graph
// needs no host round trip.
struct ToolDev {
    double vel[2];
    double tl_point_ref[2];
    double br_point[2];
    double ref_dist;
    double lowest_point, right_point;
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
