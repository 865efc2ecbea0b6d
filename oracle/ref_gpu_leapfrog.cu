// Test infrastructure: the reference pin on the GPU.  Compiles the reference's
// own leap_frog.cu (init / predict / correct kernels, unmodified, from the
// read-only reference tree) into a cubin for sm_103a; oracle/ref_gpu.py loads it.
#include <cuda_runtime.h>
#include "leap_frog.cu"
