// mlp_oracle.cpp -- CPU oracle of the learned warm start (TEST INFRASTRUCTURE:
// only the tests use it, as the checker of the GPU MLP kernels).
//
// The 4-64-64-64-1 SiLU network, its loss 0.5 (y - t)^2 in standardised units
// averaged over the samples, the gradient of that loss and one Adam step,
// restated in plain C++ with double accumulation.  Two modes:
//  - exact (bf16 = 0): double throughout, smooth in the parameters; the
//    finite-difference check of the gradient runs on this mode;
//  - bf16 (bf16 = 1): the GPU's numerics -- weights W1..W4 rounded to BF16,
//    hidden activations A1, A2 and the back-propagated dZ3, dZ2 rounded to
//    BF16 where the GPU feeds them to the tensor cores, the standardisation
//    and the output scaling in FP32.
// The network itself has no counterpart in the reference; the quantity it
// predicts is the plastic-multiplier increment of the secant return mapping
// (plasticity.cuh:128-162, actions_gpu.cu:689-754).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int kIn = 4, kH = 64;
constexpr int kW1 = 0, kB1 = 256, kW2 = 320, kB2 = 4416, kW3 = 4480, kB3 = 8576, kW4 = 8640, kB4 = 8704, kP = 8705;

// round-to-nearest-even FP32 -> BF16 -> FP32 (finite values)
float bf16(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

double sig(double z) { return 1.0 / (1.0 + std::exp(-z)); }
double silu(double z) { return z * sig(z); }
double dsilu(double z) {
    double s = sig(z);
    return s * (1.0 + z * (1.0 - s));
}

}  // namespace

extern "C" {

// norm = x_mean[4], x_std[4], y_mean, y_std.  y_out (raw target units), grad
// [8705] and loss are optional; t is needed for grad / loss.
int orc_mlp_eval(const double *params, const float *norm, const float *x, const float *t, int64_t n, int32_t bf16m,
                 double *y_out, double *grad, double *loss) {
    if (!params || !norm || !x || n < 1) return 1;
    const bool b = bf16m != 0;
    std::vector<double> W(params, params + kP);
    if (b) {
        auto r = [&](int off, int cnt) {
            for (int i = 0; i < cnt; i++) W[off + i] = bf16((float)W[off + i]);
        };
        r(kW1, 256); r(kW2, 4096); r(kW3, 4096); r(kW4, 64);
    }
    std::vector<double> g(kP, 0.0);
    double lsum = 0.0;
    const double inv_n = b ? (double)(1.f / (float)n) : 1.0 / (double)n;
    double z1[kH], a1[kH], z2[kH], a2[kH], z3[kH], a3[kH], d3[kH], d2[kH], d1[kH];
    for (int64_t s = 0; s < n; s++) {
        double xn[kIn];
        for (int c = 0; c < kIn; c++) {
            if (b) {
                float inv = 1.f / norm[4 + c];
                xn[c] = (double)((x[4 * s + c] - norm[c]) * inv);
            } else {
                xn[c] = ((double)x[4 * s + c] - norm[c]) / norm[4 + c];
            }
        }
        for (int j = 0; j < kH; j++) {
            double acc = W[kB1 + j];
            for (int c = 0; c < kIn; c++) acc += W[kW1 + j * kIn + c] * xn[c];
            z1[j] = acc;
            a1[j] = b ? bf16((float)silu(acc)) : silu(acc);
        }
        for (int j = 0; j < kH; j++) {
            double acc = 0.0;
            for (int i = 0; i < kH; i++) acc += W[kW2 + j * kH + i] * a1[i];
            z2[j] = acc + W[kB2 + j];
            a2[j] = b ? bf16((float)silu(z2[j])) : silu(z2[j]);
        }
        double y = W[kB4];
        for (int j = 0; j < kH; j++) {
            double acc = 0.0;
            for (int i = 0; i < kH; i++) acc += W[kW3 + j * kH + i] * a2[i];
            z3[j] = acc + W[kB3 + j];
            a3[j] = silu(z3[j]);
            y += W[kW4 + j] * a3[j];
        }
        if (y_out) y_out[s] = b ? (double)((float)y * norm[9] + norm[8]) : y * norm[9] + norm[8];
        if (!t) continue;
        const double tn = b ? (double)((t[s] - norm[8]) / norm[9]) : ((double)t[s] - norm[8]) / norm[9];
        const double e = y - tn;
        lsum += 0.5 * e * e;
        if (!grad) continue;
        const double gy = e * inv_n;
        g[kB4] += gy;
        for (int j = 0; j < kH; j++) {
            g[kW4 + j] += gy * a3[j];
            d3[j] = gy * W[kW4 + j] * dsilu(z3[j]);
            if (b) d3[j] = bf16((float)d3[j]);
            g[kB3 + j] += d3[j];
            for (int i = 0; i < kH; i++) g[kW3 + j * kH + i] += d3[j] * a2[i];
        }
        for (int i = 0; i < kH; i++) {
            double acc = 0.0;
            for (int j = 0; j < kH; j++) acc += d3[j] * W[kW3 + j * kH + i];
            d2[i] = acc * dsilu(z2[i]);
            if (b) d2[i] = bf16((float)d2[i]);
        }
        for (int j = 0; j < kH; j++) {
            g[kB2 + j] += d2[j];
            for (int i = 0; i < kH; i++) g[kW2 + j * kH + i] += d2[j] * a1[i];
        }
        for (int i = 0; i < kH; i++) {
            double acc = 0.0;
            for (int j = 0; j < kH; j++) acc += d2[j] * W[kW2 + j * kH + i];
            d1[i] = acc * dsilu(z1[i]);
            g[kB1 + i] += d1[i];
            for (int c = 0; c < kIn; c++) g[kW1 + i * kIn + c] += d1[i] * xn[c];
        }
    }
    if (grad) std::memcpy(grad, g.data(), sizeof(double) * kP);
    if (loss) *loss = lsum / (double)n;
    return 0;
}

// One Adam step in FP32 (beta1 0.9, beta2 0.999, eps 1e-8, bias corrections
// of step t), the update the GPU applies to its FP32 parameters.
int orc_mlp_adam(float *params, float *m1, float *m2, const float *grad, int64_t t, float lr) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)t)));
    const float c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)t)));
    for (int p = 0; p < kP; p++) {
        const float gp = grad[p];
        const float a = b1 * m1[p] + (1.f - b1) * gp;
        const float v = b2 * m2[p] + (1.f - b2) * gp * gp;
        m1[p] = a;
        m2[p] = v;
        params[p] = params[p] - lr * (a * c1) / (std::sqrt(v * c2) + eps);
    }
    return 0;
}

}  // extern "C"
