// Test infrastructure: the reference pin on the GPU.  Compiles the reference's
// own tool_gpu.cu (the rigid tool's contact and tool-particle move, unmodified,
// from the read-only reference tree) into a cubin for sm_103a; oracle/ref_gpu.py
// loads it.  The standard and thrust headers come first (the reference's
// `#define float_t double` would otherwise reach libcu++'s `using ::float_t`),
// texture_ref.h maps the removed cudaThreadSynchronize, and the __constant__
// tool description becomes plain device globals that ref_set_rigid_tool fills
// as tool_gpu_set_up_tool does (tool_gpu.cu:212-262).
#include <cuda_runtime.h>
#include <cuda/std/cmath>
#include <thrust/device_vector.h>
#include <thrust/extrema.h>
#include "texture_ref.h"
#undef __constant__
#define __constant__ __device__
#include "tool_gpu.cu"

extern "C" __global__ void ref_set_rigid_tool(const segment_gpu *segs, int n, circle_segment_gpu fil, int has_fillet,
                                              double mu, double alpha, double mass, double2 vel) {
    for (int i = 0; i < n && i < TOOL_MAX_SEG; i++) segments[i] = segs[i];
    num_seg = n;
    if (has_fillet) fillet = fil;
    friction_mu = mu;
    contact_alpha = alpha;
    slave_mass = mass;
    tool_vel = vel;
}
