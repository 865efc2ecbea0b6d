// interactions_mlp.cu -- the fused FP32K neighbour sums with the learned warm
// start of the return mapping folded into the epilogue
// (k_interact32<..., kMlp = true>), in every launch shape of the plain kernel.
// A warp whose particles yield runs one warp-wide forward pass of the network
// per yielding particle (CUDA cores, BF16 weights, FP32 sums), then each
// yielding lane runs the secant from the prediction (mlp_warp.cuh).
#include "interact32.cuh"

namespace sphfem {

void launch_interactions32_fused_mlp(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets,
                                     const SortedFields32 &B, const FixedFields32 &F, const StepScratch &W,
                                     const SegDev &seg, const ToolDev *tool, int variant, const MlpDev &mlp) {
    launch_i32_variant<true>(s, N, K, offsets, B, F, W, seg, tool, variant, mlp);
}

}  // namespace sphfem
