// Test infrastructure: the reference pin on the GPU.  Compiles the reference's
// own grid.cu (compute_hashes, unmodified, from the read-only reference tree)
// into a cubin for sm_103a; oracle/ref_gpu.py loads it.
#include <cuda_runtime.h>
#include "grid.cu"
