// Test infrastructure: the reference pin on the GPU.  Compiles the reference's
// own tool_FEM.cu (tool and segment moves, wear kernels; unmodified, from the
// read-only reference tree) into a cubin for sm_103a; oracle/ref_gpu.py loads
// it.  ref_set_flank / ref_set_wear set the file's flank_retreat, flank_contact
// and wear_para device globals, which its host code fills with
// cudaMemcpyToSymbol; ref_get_flank reads the first two back.
#include <cuda_runtime.h>
#include "tool_FEM.cu"

extern "C" __global__ void ref_set_flank(double retreat, double contact) {
    flank_retreat = retreat;
    flank_contact = contact;
}

extern "C" __global__ void ref_set_wear(double retreat, double contact, wear_constants wc) {
    flank_retreat = retreat;
    flank_contact = contact;
    wear_para = wc;
}

extern "C" __global__ void ref_get_flank(double *out) {
    out[0] = flank_retreat;
    out[1] = flank_contact;
}
