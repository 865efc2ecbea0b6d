// mlp_host.cu -- C ABI of the learned warm start (include/sphfem.h): the MLP
// object, its initialisation, batch inference, gradients and Adam training.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>

#include "mlp_host.h"

using namespace sphfem;

namespace sphfem {
MlpDev mlp_view(const sph_mlp *m, const float *params, const uint16_t *wb) {
    MlpDev d{};
    d.params = params;
    d.wb = wb;
    for (int c = 0; c < kMlpIn; c++) {
        d.x_mean[c] = m->norm.x_mean[c];
        d.x_inv_std[c] = 1.f / m->norm.x_std[c];
    }
    d.y_mean = m->norm.y_mean;
    d.y_std = m->norm.y_std;
    return d;
}
}  // namespace sphfem

namespace {

int mfail(sph_mlp *m, int code, const std::string &msg) {
    if (m) m->err = msg;
    return code;
}

#define MCK(call)                                                                                   \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess) return mfail(m, SPH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int malloc_dev(sph_mlp *m, T **p, size_t count) {
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) return mfail(m, SPH_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    m->allocs.push_back((void *)*p);
    return SPH_OK;
}

#define MALLOC(p, n)                              \
    do {                                          \
        int r_ = malloc_dev(m, &(p), (n));        \
        if (r_ != SPH_OK) return r_;              \
    } while (0)

// splitmix64: deterministic initialisation independent of the C library
uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double uniform01(uint64_t &s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

// Device scratch for n samples (features, targets, indices), grown on demand.
struct Batch {
    float *x = nullptr, *t = nullptr;
    int32_t *idx = nullptr;
};

int ensure_part(sph_mlp *m, int rows) {
    if (m->part_rows >= rows) return SPH_OK;
    if (m->part) {
        cudaFree(m->part);
        m->allocs.erase(std::find(m->allocs.begin(), m->allocs.end(), (void *)m->part));
        m->part = nullptr;
    }
    MALLOC(m->part, (size_t)rows * (kMlpParams + 1));
    m->part_rows = rows;
    return SPH_OK;
}

int grad_grid(const sph_mlp *m, int64_t nb) {
    int64_t tiles = (nb + 127) / 128;
    return (int)std::max<int64_t>(1, std::min<int64_t>(tiles, 2 * (int64_t)m->num_sms));
}

// Gradient (and loss) of the mean loss over samples idx[0..nb) (or 0..nb) into
// m->grad; with lr > 0 also one Adam step.
int grad_step(sph_mlp *m, const float *x, const float *t, const int32_t *idx, int64_t nb, float lr, bool adam,
              float *loss_dst) {
    const int grid = grad_grid(m, nb);
    int r = ensure_part(m, grid);
    if (r) return r;
    MlpDev d = mlp_view(m, m->params, m->wb);
    launch_mlp_grad(m->stream, grid, d, x, t, idx, nb, m->part, m->status);
    float c1 = 1.f, c2 = 1.f;
    if (adam) {
        m->adam_t++;
        c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)m->adam_t)));
        c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)m->adam_t)));
    }
    launch_mlp_reduce_adam(m->stream, m->part, grid, adam ? nullptr : m->grad, loss_dst, m->params, m->m1, m->m2,
                           m->wb, lr, 0.9f, 0.999f, 1e-8f, c1, c2, adam);
    MCK(cudaGetLastError());
    return SPH_OK;
}

int upload_batch(sph_mlp *m, const float *x, const float *t, int64_t n, Batch &b) {
    MCK(cudaMallocAsync((void **)&b.x, sizeof(float) * 4 * (size_t)n, m->stream));
    MCK(cudaMallocAsync((void **)&b.t, sizeof(float) * (size_t)n, m->stream));
    MCK(cudaMemcpyAsync(b.x, x, sizeof(float) * 4 * (size_t)n, cudaMemcpyHostToDevice, m->stream));
    if (t) MCK(cudaMemcpyAsync(b.t, t, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, m->stream));
    return SPH_OK;
}

void free_batch(sph_mlp *m, Batch &b) {
    if (b.x) cudaFreeAsync(b.x, m->stream);
    if (b.t) cudaFreeAsync(b.t, m->stream);
    if (b.idx) cudaFreeAsync(b.idx, m->stream);
    b = Batch{};
}

int check_status(sph_mlp *m) {
    uint32_t st = 0;
    MCK(cudaMemcpyAsync(&st, m->status, sizeof(st), cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    if (st & SPH_STATUS_MMA_TIMEOUT) return mfail(m, SPH_ERR_CUDA, "tensor-core wait timed out");
    return SPH_OK;
}

}  // namespace

extern "C" {

int sph_mlp_create(int32_t device, uint64_t seed, sph_mlp **out) {
    if (!out) return SPH_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device) return SPH_ERR_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaSetDevice(device) != cudaSuccess || cudaGetDeviceProperties(&prop, device) != cudaSuccess)
        return SPH_ERR_NO_DEVICE;
    if (!(prop.major == 10 && prop.minor == 3)) return SPH_ERR_NO_DEVICE;
    sph_mlp *m = new sph_mlp();
    *out = m;
    m->device = device;
    m->num_sms = prop.multiProcessorCount;
    MCK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    MCK(mlp_configure());
    MALLOC(m->params, kMlpParams);
    MALLOC(m->m1, kMlpParams);
    MALLOC(m->m2, kMlpParams);
    MALLOC(m->wb, kMlpWb);
    MALLOC(m->grad, kMlpParams + 1);
    MALLOC(m->status, 1);
    MCK(cudaMemset(m->status, 0, sizeof(uint32_t)));
    // nn.Linear-style initialisation: U(-1/sqrt(fan_in), 1/sqrt(fan_in)) for weights and biases
    std::vector<float> p(kMlpParams);
    uint64_t s = seed;
    auto fill = [&](int off, int count, int fan_in) {
        const double b = 1.0 / std::sqrt((double)fan_in);
        for (int i = 0; i < count; i++) p[off + i] = (float)((2.0 * uniform01(s) - 1.0) * b);
    };
    fill(kMlpOffW1, 256, 4); fill(kMlpOffB1, 64, 4);
    fill(kMlpOffW2, 4096, 64); fill(kMlpOffB2, 64, 64);
    fill(kMlpOffW3, 4096, 64); fill(kMlpOffB3, 64, 64);
    fill(kMlpOffW4, 64, 64); fill(kMlpOffB4, 1, 64);
    for (int c = 0; c < 4; c++) {
        m->norm.x_mean[c] = 0.f;
        m->norm.x_std[c] = 1.f;
    }
    m->norm.y_mean = 0.f;
    m->norm.y_std = 1.f;
    return sph_mlp_set_params(m, p.data(), nullptr);
}

int sph_mlp_destroy(sph_mlp *m) {
    if (!m) return SPH_ERR_INVALID;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    for (void *p : m->allocs) cudaFree(p);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return SPH_OK;
}

const char *sph_mlp_last_error(const sph_mlp *m) { return m ? m->err.c_str() : "no mlp"; }

int sph_mlp_get_params(sph_mlp *m, float *params, sph_mlp_norm *norm) {
    if (!m) return SPH_ERR_INVALID;
    MCK(cudaSetDevice(m->device));
    if (params) {
        MCK(cudaMemcpyAsync(params, m->params, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, m->stream));
        MCK(cudaStreamSynchronize(m->stream));
    }
    if (norm) *norm = m->norm;
    return SPH_OK;
}

int sph_mlp_set_params(sph_mlp *m, const float *params, const sph_mlp_norm *norm) {
    if (!m) return SPH_ERR_INVALID;
    MCK(cudaSetDevice(m->device));
    if (norm) {
        for (int c = 0; c < 4; c++)
            if (!(norm->x_std[c] > 0.f)) return mfail(m, SPH_ERR_INVALID, "x_std must be positive");
        if (!(norm->y_std > 0.f)) return mfail(m, SPH_ERR_INVALID, "y_std must be positive");
        m->norm = *norm;
    }
    if (params) {
        MCK(cudaMemcpyAsync(m->params, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, m->stream));
        MCK(cudaMemsetAsync(m->m1, 0, sizeof(float) * kMlpParams, m->stream));
        MCK(cudaMemsetAsync(m->m2, 0, sizeof(float) * kMlpParams, m->stream));
        m->adam_t = 0;
        launch_mlp_refresh_wb(m->stream, m->params, m->wb);
        MCK(cudaGetLastError());
        MCK(cudaStreamSynchronize(m->stream));
    }
    return SPH_OK;
}

int sph_mlp_fit_norm(sph_mlp *m, const float *x, const float *t, int64_t n) {
    if (!m || !x || !t || n < 2) return SPH_ERR_INVALID;
    double sx[4] = {0, 0, 0, 0}, sxx[4] = {0, 0, 0, 0}, st = 0, stt = 0;
    for (int64_t i = 0; i < n; i++) {
        for (int c = 0; c < 4; c++) {
            double v = x[4 * i + c];
            sx[c] += v;
            sxx[c] += v * v;
        }
        st += t[i];
        stt += (double)t[i] * t[i];
    }
    sph_mlp_norm nm;
    for (int c = 0; c < 4; c++) {
        double mu = sx[c] / n, var = std::max(sxx[c] / n - mu * mu, 0.0);
        nm.x_mean[c] = (float)mu;
        nm.x_std[c] = (float)std::max(std::sqrt(var), 1e-6);
    }
    double mu = st / n, var = std::max(stt / n - mu * mu, 0.0);
    nm.y_mean = (float)mu;
    nm.y_std = (float)std::max(std::sqrt(var), 1e-6);
    m->norm = nm;
    return SPH_OK;
}

int sph_mlp_predict(sph_mlp *m, const float *x, int64_t n, float *y) {
    if (!m || !x || !y || n < 0) return SPH_ERR_INVALID;
    if (n == 0) return SPH_OK;
    MCK(cudaSetDevice(m->device));
    Batch b;
    int r = upload_batch(m, x, nullptr, n, b);
    if (r) return r;
    MlpDev d = mlp_view(m, m->params, m->wb);
    const int grid = (int)std::min<int64_t>((n + 127) / 128, 4 * (int64_t)m->num_sms);
    launch_mlp_predict(m->stream, d, b.x, n, b.t, m->status, grid);
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(y, b.t, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, m->stream));
    free_batch(m, b);
    return check_status(m);
}

int sph_mlp_predict_warp(sph_mlp *m, const float *x, int64_t n, float *y) {
    if (!m || !x || !y || n < 0) return SPH_ERR_INVALID;
    if (n == 0) return SPH_OK;
    MCK(cudaSetDevice(m->device));
    Batch b;
    int r = upload_batch(m, x, nullptr, n, b);
    if (r) return r;
    MlpDev d = mlp_view(m, m->params, m->wb);
    launch_mlp_predict_warp(m->stream, d, b.x, n, b.t, 8 * m->num_sms);
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(y, b.t, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, m->stream));
    free_batch(m, b);
    return check_status(m);
}

int sph_mlp_gradients(sph_mlp *m, const float *x, const float *t, int64_t n, float *grad, float *loss) {
    if (!m || !x || !t || n < 1) return SPH_ERR_INVALID;
    MCK(cudaSetDevice(m->device));
    Batch b;
    int r = upload_batch(m, x, t, n, b);
    if (r) return r;
    r = grad_step(m, b.x, b.t, nullptr, n, 0.f, false, nullptr);
    if (r) return r;
    std::vector<float> g(kMlpParams + 1);
    MCK(cudaMemcpyAsync(g.data(), m->grad, sizeof(float) * (kMlpParams + 1), cudaMemcpyDeviceToHost, m->stream));
    free_batch(m, b);
    r = check_status(m);
    if (r) return r;
    if (grad) std::memcpy(grad, g.data(), sizeof(float) * kMlpParams);
    if (loss) *loss = g[kMlpParams] / (float)n;
    return SPH_OK;
}

int sph_mlp_adam_step(sph_mlp *m, const float *x, const float *t, int64_t n, float lr, float *loss) {
    if (!m || !x || !t || n < 1) return SPH_ERR_INVALID;
    MCK(cudaSetDevice(m->device));
    Batch b;
    int r = upload_batch(m, x, t, n, b);
    if (r) return r;
    if (!m->loss || m->loss_cap < 1) {
        MALLOC(m->loss, 1);
        m->loss_cap = 1;
    }
    r = grad_step(m, b.x, b.t, nullptr, n, lr, true, m->loss);
    if (r) return r;
    float l = 0.f;
    MCK(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    free_batch(m, b);
    r = check_status(m);
    if (r) return r;
    if (loss) *loss = l / (float)n;
    return SPH_OK;
}

int sph_mlp_train(sph_mlp *m, const float *x, const float *t, int64_t n, int32_t epochs, int32_t batch, float lr,
                  uint64_t seed, float *epoch_loss) {
    if (!m || !x || !t || n < 1 || epochs < 1 || batch < 1) return SPH_ERR_INVALID;
    if (n > INT32_MAX) return mfail(m, SPH_ERR_INVALID, "too many samples");
    MCK(cudaSetDevice(m->device));
    Batch b;
    int r = upload_batch(m, x, t, n, b);
    if (r) return r;
    MCK(cudaMallocAsync((void **)&b.idx, sizeof(int32_t) * (size_t)n, m->stream));
    const int64_t steps = (n + batch - 1) / batch;
    if (m->loss_cap < steps) {
        if (m->loss) {
            cudaFree(m->loss);
            m->allocs.erase(std::find(m->allocs.begin(), m->allocs.end(), (void *)m->loss));
            m->loss = nullptr;
        }
        MALLOC(m->loss, (size_t)steps);
        m->loss_cap = steps;
    }
    std::vector<int32_t> perm(n);
    std::vector<float> losses(steps);
    std::mt19937_64 rng(seed);
    for (int ep = 0; ep < epochs; ep++) {
        std::iota(perm.begin(), perm.end(), 0);
        std::shuffle(perm.begin(), perm.end(), rng);
        MCK(cudaMemcpyAsync(b.idx, perm.data(), sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, m->stream));
        for (int64_t s = 0; s < steps; s++) {
            const int64_t nb = std::min<int64_t>(batch, n - s * batch);
            r = grad_step(m, b.x, b.t, b.idx + s * batch, nb, lr, true, m->loss + s);
            if (r) {
                free_batch(m, b);
                return r;
            }
        }
        MCK(cudaMemcpyAsync(losses.data(), m->loss, sizeof(float) * (size_t)steps, cudaMemcpyDeviceToHost,
                            m->stream));
        MCK(cudaStreamSynchronize(m->stream));   // the permutation buffer is reused next epoch
        if (epoch_loss) {
            double sum = 0;
            for (float l : losses) sum += l;
            epoch_loss[ep] = (float)(sum / (double)n);
        }
    }
    free_batch(m, b);
    return check_status(m);
}

}  // extern "C"
