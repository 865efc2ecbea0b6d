// Test infrastructure: the reference pin on the GPU.  Compiles the reference's
// own tool_FEM.cu (tool and segment moves, wear kernels; unmodified, from the
// read-only reference tree) into a cubin for sm_103a; oracle/ref_gpu.py loads
// it.  ref_set_flank sets the file's flank_retreat / flank_contact device
// globals, which its host code fills with cudaMemcpyToSymbol.
#include <cuda_runtime.h>
#include "tool_FEM.cu"

extern "C" __global__ void ref_set_flank(double retreat, double contact) {
    flank_retreat = retreat;
    flank_contact = contact;
}
