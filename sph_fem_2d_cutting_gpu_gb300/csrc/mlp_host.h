// mlp_host.h -- the host-side MLP object (sph_mlp) shared by the MLP entry
// points and the context's warm-start attachment.
#pragma once

#include <string>
#include <vector>

#include "launch.cuh"

struct sph_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    float *params = nullptr, *m1 = nullptr, *m2 = nullptr;   // FP32 parameters and Adam moments
    uint16_t *wb = nullptr;                                  // BF16 weight copies
    float *part = nullptr;                                   // per-CTA gradient partials
    int part_rows = 0;
    float *grad = nullptr;                                   // [kMlpParams + 1]
    float *loss = nullptr;                                   // per-step losses of a training run
    int64_t loss_cap = 0;
    uint32_t *status = nullptr;
    sph_mlp_norm norm{};
    int64_t adam_t = 0;
    std::vector<void *> allocs;
    std::string err;
};

namespace sphfem {
MlpDev mlp_view(const sph_mlp *m, const float *params, const uint16_t *wb);
}
