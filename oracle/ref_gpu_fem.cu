// Test infrastructure: the reference pin on the GPU.  Compiles the reference's
// own FEM_thermal_gpu.cu (the tool's FEM heat kernels, unmodified, from the
// read-only reference tree) into a cubin for sm_103a; oracle/ref_gpu.py loads
// it.  Its __constant__ tool constants become a plain device global that
// ref_set_fem_constants fills.
#include <cuda_runtime.h>
#undef __constant__
#define __constant__ __device__
#include "FEM_thermal_gpu.cu"

extern "C" __global__ void ref_set_fem_constants(tool_constants to) { tc = to; }
