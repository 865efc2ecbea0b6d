// Test infrastructure: the reference pin on the GPU.  Compiles the reference's
// own grid_gpu_green.cu (the cell-table and reorder kernel, unmodified, from the
// read-only reference tree) into a cubin for sm_103a; oracle/ref_gpu.py loads
// it.  The file relies on <thrust/sort.h> arriving through other headers in
// the thrust version it was written for; it is included here first.
#include <cuda_runtime.h>
#include <thrust/sort.h>
#include "grid_gpu_green.cu"
