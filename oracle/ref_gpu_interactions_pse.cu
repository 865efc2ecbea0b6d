// Test infrastructure: the reference pin on the GPU, PSE build.  The
// reference selects its conduction model in types.h (Thermal_Conduction_Brookshaw
// or Thermal_Conduction_PSE, types.h:122-123).  types.h is read first here and
// its switch turned to the PSE build (its include guard keeps the header from
// being read again); the rest is ref_gpu_interactions.cu.  The standard and
// thrust headers come first: types.h's `#define float_t double` must not reach
// libcu++'s `using ::float_t`.
#include <cuda_runtime.h>
#include <cuda/std/cmath>
#include <thrust/device_vector.h>
#include <thrust/sequence.h>
#include "types.h"
#undef Thermal_Conduction_Brookshaw
#define Thermal_Conduction_PSE
#include "ref_gpu_interactions.cu"
