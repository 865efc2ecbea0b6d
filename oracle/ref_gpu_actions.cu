// Test infrastructure: the reference pin on the GPU.  Compiles the reference's
// own actions_gpu.cu (from the read-only reference tree, unmodified) into a
// cubin for sm_103a; oracle/ref_gpu.py loads it through the CUDA driver API and
// the GPU parity tests run its kernels beside the product's staged calls.
// The reference keeps its physical constants in __constant__ blocks that its
// host code fills with cudaMemcpyToSymbol; here they become plain device
// globals so that the one setter kernel below can install the same bytes.
#include <cuda_runtime.h>
#undef __constant__
#define __constant__ __device__
#include "actions_gpu.cu"

extern "C" __global__ void ref_set_actions_constants(phys_constants ph, corr_constants co, joco_constants jc,
                                                     trml_constants tw, trml_constants tt, tool_constants tc,
                                                     wear_constants wc) {
    physics = ph;
    correctors = co;
    johnson_cook = jc;
    thermals_wp = tw;
    thermals_tool = tt;
    tool_consts = tc;
    wear_consts = wc;
}
