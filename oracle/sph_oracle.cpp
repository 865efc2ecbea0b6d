// sph_oracle.cpp -- CPU ORACLE (test infrastructure only).
//
// A plain C++17 restatement of the reference's per-timestep SPH workpiece
// path (nyzhang1227/SPH_FEM_2D_cutting_gpu), one function per reference
// kernel, each citing the reference file:line it follows.  It is the checker
// for the CUDA product and the timed CPU baseline; the product never links,
// loads or calls it.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline arm may use it.
//
// Parity pins: cubic_spline and the Johnson-Cook secant return mapping are
// checked against the reference's own kernels.cuh / plasticity.cuh compiled
// on the host (oracle/ref_pin.cpp, golden vectors in tests/golden/); the
// rigid tool's outline, fillet, placement and particle sampling (the host
// set-up the rigid-tool functions below consume) against the reference's own
// tool.cpp / geometric_primitives.cpp (oracle/ref_tool_pin.cpp).  The device
// kernels of tool_gpu.cu cannot be built for the host (kernel-launch syntax),
// so the rigid contact below, like the rest of the path, is pinned by analytic
// known-answer tests only; the reference has no tests, golden vectors or
// fixtures of its own.
//
// Semantics kept from the reference on purpose:
//  - float narrowings: sqrtf/fmaxf/fminf of double arguments round the
//    argument to float (kernels.cuh:45, interactions_gpu.cu:294-295,
//    actions_gpu.cu:53,182,208,228,354,372,385,387,507,604,703,716,728-729).
//  - atan2f/cosf/sinf of the artificial stress (actions_gpu.cu:48,257-258) are
//    evaluated in double and rounded once to float (sph_atan2f/sph_cosf/
//    sph_sinf below).  The CUDA product uses the same formulation so host and
//    device agree; it stays within the ULP bounds of CUDA's float functions.
//  - cubic spline value 0.25*(2-q)^6 for q > 1 (kernels.cuh:51-53).
//  - every candidate in the 5x5 cell block runs the full pair body
//    (interactions_gpu.cu:230-337).
//  - atomic accumulations are done in particle / segment index order.
//
// Build: oracle/Makefile (g++ -O3 -fopenmp -shared -fPIC).

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "../include/sphfem.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---- float narrowings ------------------------------------------------------
inline double sqrtf_d(double x) { return (double)sqrtf((float)x); }
inline double fmaxf_d(double a, double b) { return (double)fmaxf((float)a, (float)b); }
inline double fminf_d(double a, double b) { return (double)fminf((float)a, (float)b); }
inline float sph_atan2f(float y, float x) { return (float)atan2((double)y, (double)x); }
inline float sph_cosf(float x) { return (float)cos((double)x); }
inline float sph_sinf(float x) { return (float)sin((double)x); }

// ---- kernels.cuh:25-65 cubic_spline ---------------------------------------
inline void cubic_spline(double pix, double piy, double pjx, double pjy, double hi,
                         double &w, double &wx, double &wy) {
    const double PI_FAC = 0.454728408833987;  // kernels.cuh:19
    w = 0.; wx = 0.; wy = 0.;
    double xij = pix - pjx;
    double yij = piy - pjy;
    double rr2 = xij * xij + yij * yij;
    double h1 = 1 / hi;
    double fourh2 = 4 * hi * hi;
    if (rr2 >= fourh2 || rr2 < 1e-8) return;
    double der, val;
    double rad = sqrtf_d(rr2);
    double q = rad * h1;
    double fac = PI_FAC * h1 * h1;
    if (q > 1) {
        double _2mq = 2 - q;
        double _2mq2 = _2mq * _2mq;
        val = 0.25 * _2mq2 * _2mq2 * _2mq2;
        der = -0.75 * _2mq2 * h1 / rad;
    } else {
        val = 1 - 1.5 * q * q * (1 - 0.5 * q);
        der = -3.0 * q * (1 - 0.75 * q) * h1 / rad;
    }
    w = val * fac;
    wx = der * xij * fac;
    wy = der * yij * fac;
}

// ---- plasticity.cuh:21-39 sigma_yield ---------------------------------------
inline double sigma_yield(const sph_joco_constants &jc, double eps_pl, double eps_pl_dot, double t) {
    double theta = (t - jc.Tref) / (jc.Tmelt - jc.Tref);
    if (theta > 1.) theta = 1.;
    double Term_A = jc.A + jc.B * pow(eps_pl, jc.n);
    double Term_B = 1.0;
    double eps_dot = eps_pl_dot / jc.eps_dot_ref;
    if (eps_dot > 1.0) Term_B = 1.0 + jc.C * log(eps_dot);
    else Term_B = pow((1.0 + eps_dot), jc.C);
    double Term_C = 1.0 - pow(theta, jc.m);
    return Term_A * Term_B * Term_C;
}

// ---- plasticity.cuh:117-126 opt_fun -----------------------------------------
inline double opt_fun(const sph_joco_constants &jc, double delta_lambda, double norm_Strial,
                      double eps_pl_init, double t, double delta_t, double mu) {
    double eps_pl_equiv = eps_pl_init + sqrt(2.0 / 3.0) * fmax(delta_lambda, 0.);
    double eps_pl_equiv_dot = sqrt(2.0 / 3.0) * fmax(delta_lambda, 0.) / delta_t;
    double sigmaY = sigma_yield(jc, eps_pl_equiv, eps_pl_equiv_dot, t);
    return norm_Strial - 2 * mu * delta_lambda - sqrt(2.0 / 3.0) * sigmaY;
}

// ---- plasticity.cuh:128-162 solve_secant ------------------------------------
inline double solve_secant(const sph_joco_constants &jc, double init, double tol, double norm_Strial,
                           double eps_pl_init, double t, double delta_t, double mu, int *iters) {
    double delta_lambda = init;
    double delta_lambda_old = delta_lambda;
    int iter = 0;
    const int max_iter = 100;
    do {
        double g = opt_fun(jc, delta_lambda, norm_Strial, eps_pl_init, t, delta_t, mu);
        double delta_lambda_1 = delta_lambda * 1.01;
        double g_1 = opt_fun(jc, delta_lambda_1, norm_Strial, eps_pl_init, t, delta_t, mu);
        double slope = (g - g_1) / (delta_lambda - delta_lambda_1);
        delta_lambda_old = delta_lambda;
        delta_lambda = delta_lambda - g / slope;
        if (delta_lambda < 0.) delta_lambda = -0.1 * delta_lambda;
        if (fabs(delta_lambda - delta_lambda_old) < tol) { if (iters) *iters = iter + 1; return delta_lambda; }
        if (iter > max_iter) { if (iters) *iters = -(iter + 1); return delta_lambda; }
        iter++;
    } while (true);
}

// ---- actions_gpu.cu:45-49 stress_angle --------------------------------------
inline double stress_angle(double sxx, double sxy, double syy, double eps) {
    double numer = 2. * sxy;
    double denom = sxx - syy + eps;
    return 0.5 * (double)sph_atan2f((float)numer, (float)denom);
}

// ---- actions_gpu.cu:33-43 find_max / find_min ---------------------------------
inline double find_max(double a, double b) { return (a >= b) ? a : b; }
inline double find_min(double a, double b) { return (a >= b) ? b : a; }

// ---- actions_gpu.cu:51-63 on_segment_mesh ---------------------------------------
inline int on_segment_mesh(const double *left, const double *right, const double *point) {
    if (point[1] <= fmaxf_d(left[1], right[1]) && point[1] >= fminf_d(left[1], right[1])) {
        if (left[0] == right[0] && point[0] < left[0]) return 1;
        if (fabs(left[1] - right[1]) != 0) {
            double x_on_seg = right[0] + (left[0] - right[0]) / (left[1] - right[1]) * (point[1] - right[1]);
            if (x_on_seg > point[0] && x_on_seg != left[0]) return 1;
        } else {
            if (point[0] <= fmax(left[0], right[0])) return 1;
        }
    }
    return 0;
}

// ---- actions_gpu.cu:83-93 inside_judgement --------------------------------------
inline int inside_judgement(const double *qp, const double *left, const double *right, int num_seg) {
    int intersections = 0;
    for (int i = 0; i < num_seg; i++) intersections += on_segment_mesh(left + 2 * i, right + 2 * i, qp);
    if (intersections % 2 == 0) return 0;
    return 1;
}

// ---- actions_gpu.cu:139-220 find_shortest_distance_v1 ---------------------------
inline int find_shortest_distance_v1(const double *qp, double &dN, double n_re[2], const double *left,
                                     const double *right, const double *n, int num_seg) {
    int seg = -1;
    double depth = FLT_MAX;
    const double limit_value = 2.5e-4;
    for (int i = 0; i < num_seg; i++) {
        double d = 0.;
        double ymax = find_max(left[2 * i + 1], right[2 * i + 1]);
        double ymin = find_min(left[2 * i + 1], right[2 * i + 1]);
        double xmax = find_max(left[2 * i], right[2 * i]);
        double xmin = find_min(left[2 * i], right[2 * i]);
        if (qp[0] > xmin - 0.0008 && qp[0] < xmax + 0.0008 && qp[1] > ymin - 0.0008 && qp[1] < ymax + 0.0008) {
            d = (qp[0] - left[2 * i]) * n[2 * i] + (qp[1] - left[2 * i + 1]) * n[2 * i + 1];
            if (d >= 0. && d < depth) {
                double intersec_x = qp[0] - d * n[2 * i];
                double intersec_y = qp[1] - d * n[2 * i + 1];
                if (intersec_y <= ymax && intersec_y >= ymin && intersec_x <= xmax && intersec_x >= xmin) {
                    depth = d;
                    seg = i;
                }
            }
        }
    }
    if (seg != -1 && depth <= limit_value) {
        n_re[0] = -n[2 * seg];
        n_re[1] = -n[2 * seg + 1];
        dN = -depth;
    } else {
        depth = FLT_MAX;
        double d_trial = 0.;
        for (int i = 0; i < num_seg; i++) {
            d_trial = sqrtf_d((qp[0] - right[2 * i]) * (qp[0] - right[2 * i]) +
                              (qp[1] - right[2 * i + 1]) * (qp[1] - right[2 * i + 1]));
            if (d_trial < depth) { depth = d_trial; seg = i; }
        }
        if (seg == -1) return seg;
        double nsx = n[2 * seg], nsy = n[2 * seg + 1];
        for (int j = 0; j < num_seg; j++) {
            if (left[2 * j + 1] == right[2 * seg + 1] && left[2 * j] == right[2 * seg]) {
                nsx = (n[2 * j] + n[2 * seg]) / 2.;
                nsy = (n[2 * j + 1] + n[2 * seg + 1]) / 2.;
                break;
            }
        }
        double n_length = sqrtf_d(nsx * nsx + nsy * nsy);
        n_re[0] = -nsx / n_length;
        n_re[1] = -nsy / n_length;
        dN = -1.0 * depth;
    }
    return seg;
}

}  // namespace

extern "C" {

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

// kernels.cuh:25-65 (exported for the golden-vector pin)
void orc_cubic_spline(int n, const double *pi, const double *pj, const double *hi, double *out3) {
    for (int k = 0; k < n; k++)
        cubic_spline(pi[2 * k], pi[2 * k + 1], pj[2 * k], pj[2 * k + 1], hi[k], out3[3 * k], out3[3 * k + 1], out3[3 * k + 2]);
}

// plasticity.cuh:21-39 (exported for the golden-vector pin)
void orc_sigma_yield(const sph_joco_constants *jc, int n, const double *eps, const double *epsdot,
                     const double *T, double *out) {
    for (int k = 0; k < n; k++) out[k] = sigma_yield(*jc, eps[k], epsdot[k], T[k]);
}

// plasticity.cuh:128-162 (exported for the golden-vector pin); iters < 0 marks the cap
void orc_solve_secant(const sph_joco_constants *jc, int n, const double *init, double tol,
                      const double *normS, const double *eps, const double *T, double dt, double mu,
                      double *out, int32_t *iters) {
    for (int k = 0; k < n; k++) {
        int it = 0;
        out[k] = solve_secant(*jc, init[k], tol, normS[k], eps[k], T[k], dt, mu, &it);
        if (iters) iters[k] = it;
    }
}

// grid.cu:130-149 set_geometry (locked grid).  cell_factor/stencil generalise
// the reference's fixed kernel_width = 2 / 5x5 block.
void orc_set_geometry(const sph_grid_params *g, sph_geom_constants *out) {
    double bbmin_x = g->bbmin[0] - 1e-6;
    double bbmin_y = g->bbmin[1] - 1e-6;
    double bbmax_x = g->bbmax[0] + 1e-6;
    double bbmax_y = g->bbmax[1] + 1e-6;
    double kernel_width = 2.;
    double dx = g->h * kernel_width / 2. * (double)g->cell_factor;
    double lx = bbmax_x - bbmin_x;
    double ly = bbmax_y - bbmin_y;
    unsigned int nx = (unsigned int)ceil(lx / dx);
    unsigned int ny = (unsigned int)ceil(ly / dx);
    out->nx = (int)nx;
    out->ny = (int)ny;
    out->bbmin_x = bbmin_x;
    out->bbmin_y = bbmin_y;
    out->dx = dx;
    out->num_cell = (int)(nx * ny);
    out->stencil = g->stencil;
}

// grid.cu:25-42 compute_hashes
void orc_compute_hashes(sph_particles *P, const sph_geom_constants *g) {
    const int N = P->N;
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < N; idx++) {
        if (P->blanked[idx] == 1.) continue;
        double px = P->pos[2 * idx], py = P->pos[2 * idx + 1];
        int ix = (int)((px - g->bbmin_x) / g->dx);
        int iy = (int)((py - g->bbmin_y) / g->dx);
        P->hash[idx] = ix * g->ny + iy;
    }
}

// grid_gpu_green.cu:185-209 do_sort + :13-115 reorder_data_and_find_cell_start.
// thrust::sort_by_key on int keys is stable; out-of-range keys (the reference
// writes cell_start out of bounds for them) sort after every in-range key and
// touch no cell.  cell_end of empty cells is left as it was (stale).
// Returns the number of out-of-range particles.
int orc_sort_green(sph_particles *P, int32_t *cell_start, int32_t *cell_end, int num_cell) {
    const int N = P->N;
    std::vector<int> order(N);
    std::iota(order.begin(), order.end(), 0);
    std::vector<int> key(N);
    int oob = 0;
    for (int i = 0; i < N; i++) {
        int h = P->hash[i];
        bool in = (h >= 0 && h < num_cell);
        if (!in) oob++;
        key[i] = in ? h : num_cell;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
    std::vector<int> shash(N);
    for (int k = 0; k < N; k++) shash[k] = P->hash[order[k]];
    for (int c = 0; c < num_cell; c++) cell_start[c] = -1;
    for (int k = 0; k < N; k++) {
        int hk = key[order[k]];
        if (hk >= num_cell) continue;
        if (k == 0 || hk != key[order[k - 1]]) {
            cell_start[hk] = k;
            if (k > 0 && key[order[k - 1]] < num_cell) cell_end[key[order[k - 1]]] = k;
        }
        if (k == N - 1 || key[order[k + 1]] != hk) cell_end[hk] = k + 1;
    }
    // gather the 20 reordered fields (grid_gpu_green.cu:55-113)
    auto gather = [&](double *a, int w) {
        if (!a) return;
        std::vector<double> tmp((size_t)N * w);
        for (int k = 0; k < N; k++)
            for (int c = 0; c < w; c++) tmp[(size_t)k * w + c] = a[(size_t)order[k] * w + c];
        std::memcpy(a, tmp.data(), sizeof(double) * (size_t)N * w);
    };
    gather(P->pos, 2); gather(P->vel, 2); gather(P->fc, 2); gather(P->ft, 2);
    gather(P->h, 1); gather(P->n, 2); gather(P->rho, 1); gather(P->S, 4);
    gather(P->eps_pl, 1); gather(P->eps_pl_dot, 1); gather(P->T, 1); gather(P->fixed, 1);
    gather(P->blanked, 1); gather(P->tool_particle, 1); gather(P->pos_t, 2); gather(P->vel_t, 2);
    gather(P->rho_t, 1); gather(P->S_t, 4); gather(P->T_t, 1);
    if (P->on_seg) {
        std::vector<int> t(N);
        for (int k = 0; k < N; k++) t[k] = P->on_seg[order[k]];
        std::memcpy(P->on_seg, t.data(), sizeof(int) * N);
    }
    for (int k = 0; k < N; k++) { P->idx[k] = order[k]; P->hash[k] = shash[k]; }
    return oob;
}

// leap_frog.cu:25-37 init (snapshot arrays are caller-owned)
void orc_init(const sph_particles *P, double *pos_init, double *vel_init, double *S_init,
              double *rho_init, double *T_init) {
    const int N = P->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        if (P->blanked[i] == 1.) continue;
        pos_init[2 * i] = P->pos[2 * i]; pos_init[2 * i + 1] = P->pos[2 * i + 1];
        vel_init[2 * i] = P->vel[2 * i]; vel_init[2 * i + 1] = P->vel[2 * i + 1];
        for (int c = 0; c < 4; c++) S_init[4 * i + c] = P->S[4 * i + c];
        rho_init[i] = P->rho[i];
        T_init[i] = P->T[i];
    }
}

// leap_frog.cu:45-69 predict (fac = 0.5) and :71-96 correct (fac = 1)
static void predict_correct(sph_particles *P, const double *pos_init, const double *vel_init,
                            const double *S_init, const double *rho_init, const double *T_init,
                            double dt, bool half) {
    const int N = P->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        if (P->blanked[i] == 1.) continue;
        if (half) {
            for (int c = 0; c < 2; c++) P->pos[2 * i + c] = pos_init[2 * i + c] + 0.5 * dt * P->pos_t[2 * i + c];
            for (int c = 0; c < 2; c++) P->vel[2 * i + c] = vel_init[2 * i + c] + 0.5 * dt * P->vel_t[2 * i + c];
            for (int c = 0; c < 4; c++) P->S[4 * i + c] = S_init[4 * i + c] + 0.5 * dt * P->S_t[4 * i + c];
            P->rho[i] = rho_init[i] + 0.5 * dt * P->rho_t[i];
            P->T[i] = T_init[i] + 0.5 * dt * P->T_t[i];
        } else {
            for (int c = 0; c < 2; c++) P->pos[2 * i + c] = pos_init[2 * i + c] + dt * P->pos_t[2 * i + c];
            for (int c = 0; c < 2; c++) P->vel[2 * i + c] = vel_init[2 * i + c] + dt * P->vel_t[2 * i + c];
            for (int c = 0; c < 4; c++) P->S[4 * i + c] = S_init[4 * i + c] + dt * P->S_t[4 * i + c];
            P->rho[i] = rho_init[i] + dt * P->rho_t[i];
            P->T[i] = T_init[i] + dt * P->T_t[i];
        }
    }
}

void orc_predict(sph_particles *P, const double *pos_init, const double *vel_init, const double *S_init,
                 const double *rho_init, const double *T_init, double dt) {
    predict_correct(P, pos_init, vel_init, S_init, rho_init, T_init, dt, true);
}

void orc_correct(sph_particles *P, const double *pos_init, const double *vel_init, const double *S_init,
                 const double *rho_init, const double *T_init, double dt) {
    predict_correct(P, pos_init, vel_init, S_init, rho_init, T_init, dt, false);
}

// actions_gpu.cu:222-232 do_material_eos
void orc_material_eos(sph_particles *P, const sph_constants *C) {
    const int N = P->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        if (P->tool_particle[i] != 0.) continue;
        double rho0 = C->phys.rho0;
        double c0 = sqrtf_d(C->phys.K / rho0);
        P->p[i] = c0 * c0 * (P->rho[i] - rho0);
    }
}

// actions_gpu.cu:234-278 do_corrector_artificial_stress
void orc_corrector_artificial_stress(sph_particles *P, const sph_constants *C) {
    const int N = P->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        if (P->tool_particle[i] != 0.) continue;
        double eps = C->corr.stresseps;
        double rhoi = P->rho[i];
        double pi = P->p[i];
        double sxx = P->S[4 * i], sxy = P->S[4 * i + 1], syy = P->S[4 * i + 2];
        sxx -= pi;
        syy -= pi;
        double rhoi21 = 1. / (rhoi * rhoi);
        double theta = stress_angle(sxx, sxy, syy, 0.);
        double cos_theta = (double)sph_cosf((float)theta);
        double sin_theta = (double)sph_sinf((float)theta);
        double cos_theta2 = cos_theta * cos_theta;
        double sin_theta2 = sin_theta * sin_theta;
        double rot_sxx = cos_theta2 * sxx + 2.0 * cos_theta * sin_theta * sxy + sin_theta2 * syy;
        double rot_syy = sin_theta2 * sxx - 2.0 * cos_theta * sin_theta * sxy + cos_theta2 * syy;
        double rot_rxx = 0., rot_ryy = 0.;
        if (rot_sxx > 0) rot_rxx = -eps * rot_sxx * rhoi21;
        if (rot_syy > 0) rot_ryy = -eps * rot_syy * rhoi21;
        P->R[4 * i + 0] = cos_theta2 * rot_rxx + sin_theta2 * rot_ryy;
        P->R[4 * i + 1] = cos_theta * sin_theta * (rot_rxx - rot_ryy);
        P->R[4 * i + 2] = sin_theta2 * rot_rxx + cos_theta2 * rot_ryy;
        P->R[4 * i + 3] = 0.;
    }
}

// interactions_gpu.cu:143-379 do_interactions_monaghan (SURFACE off) with
// unhash/hash (:75-82); cell stencil generalised to g->stencil cells per side.
// pse == 0: the Brookshaw build (types.h:122).  pse != 0: the
// Thermal_Conduction_PSE build -- tool particles return before any write
// (:156-158) and the Brookshaw sum is compiled out (T_t comes from
// interactions_heat_pse).
static void monaghan_impl(sph_particles *P, const int32_t *cell_start, const int32_t *cell_end,
                          const sph_geom_constants *g, const sph_constants *C, int pse) {
    const int N = P->N;
    const int R = g->stencil;
#pragma omp parallel for schedule(dynamic, 256)
    for (int pidx = 0; pidx < N; pidx++) {
        if (P->blanked[pidx] == 1.) continue;
        double is_tool_particle_i = P->tool_particle[pidx];
        if (pse && is_tool_particle_i == 1.) continue;
        double mass = C->phys.mass;
        double K = C->phys.K;
        double thermal_alpha = pse ? 0. : ((is_tool_particle_i == 0.) ? C->trml_wp.alpha : C->trml_tool_sph.alpha);
        double wdeltap = C->corr.wdeltap, alpha = C->corr.alpha, beta = C->corr.beta,
               eta = C->corr.eta, eps = C->corr.xspheps;
        int nx = g->nx, ny = g->ny;
        double pix = P->pos[2 * pidx], piy = P->pos[2 * pidx + 1];
        double vix = P->vel[2 * pidx], viy = P->vel[2 * pidx + 1];
        const double *Si = P->S + 4 * pidx;
        const double *Ri = P->R + 4 * pidx;
        double hi = P->h[pidx], rhoi = P->rho[pidx], prsi = P->p[pidx];
        double Ti = 0.;
        if (thermal_alpha != 0.) Ti = P->T[pidx];
        double rhoi21 = 1. / (rhoi * rhoi);
        int hashi = P->hash[pidx];
        double vd[4] = {0, 0, 0, 0}, sd[4] = {0, 0, 0, 0}, vt[2] = {0, 0}, xt[2] = {0, 0};
        double T_lapl = 0.;
        if (hashi >= 0 && hashi < g->num_cell) {
            int gi = hashi / ny;
            int gj = hashi - gi * ny;
            int low_i = gi - R < 0 ? 0 : gi - R;
            int low_j = gj - R < 0 ? 0 : gj - R;
            int high_i = gi + R + 1 > nx ? nx : gi + R + 1;
            int high_j = gj + R + 1 > ny ? ny : gj + R + 1;
            for (int ii = low_i; ii < high_i; ii++) {
                for (int jj = low_j; jj < high_j; jj++) {
                    int idx = ii * ny + jj;
                    int c_start = cell_start[idx];
                    int c_end = cell_end[idx];
                    if (c_start == -1) continue;
                    for (int iter = c_start; iter < c_end; iter++) {
                        if (P->blanked[iter] == 1.) continue;
                        double pjx = P->pos[2 * iter], pjy = P->pos[2 * iter + 1];
                        double vjx = P->vel[2 * iter], vjy = P->vel[2 * iter + 1];
                        const double *Sj = P->S + 4 * iter;
                        const double *Rj = P->R + 4 * iter;
                        double hj = P->h[iter], rhoj = P->rho[iter], prsj = P->p[iter];
                        double Tj = 0.;
                        if (thermal_alpha != 0.) Tj = P->T[iter];
                        double is_tool_particle_j = P->tool_particle[iter];
                        double volj = mass / rhoj;
                        double rhoj21 = 1. / (rhoj * rhoj);
                        double w, w_x, w_y;
                        cubic_spline(pix, piy, pjx, pjy, hi, w, w_x, w_y);
                        if (!(is_tool_particle_i == 1.) && !(is_tool_particle_j == 1.)) {
                            vd[0] += (vjx - vix) * w_x * volj;
                            vd[1] += (vjx - vix) * w_y * volj;
                            vd[2] += (vjy - viy) * w_x * volj;
                            vd[3] += (vjy - viy) * w_y * volj;
                            double fab = w / wdeltap;
                            fab *= fab;
                            fab *= fab;
                            double Rx = fab * (Ri[0] + Rj[0]);
                            double Ry = fab * (Ri[1] + Rj[1]);
                            double Rz = fab * (Ri[2] + Rj[2]);
                            sd[0] += mass * ((Si[0] - prsi) * rhoi21 + (Sj[0] - prsj) * rhoj21 + Rx) * w_x;
                            sd[1] += mass * (Si[1] * rhoi21 + Sj[1] * rhoj21 + Ry) * w_y;
                            sd[2] += mass * (Si[1] * rhoi21 + Sj[1] * rhoj21 + Ry) * w_x;
                            sd[3] += mass * ((Si[2] - prsi) * rhoi21 + (Sj[2] - prsj) * rhoj21 + Rz) * w_y;
                            double xij = pix - pjx, yij = piy - pjy;
                            double vijx = vix - vjx, vijy = viy - vjy;
                            double vijposij = vijx * xij + vijy * yij;
                            double rhoij = 0.5 * (rhoi + rhoj);
                            if (vijposij < 0.) {
                                double ci = sqrtf_d(K / rhoi);
                                double cj = sqrtf_d(K / rhoj);
                                double cij = 0.5 * (ci + cj);
                                double hij = 0.5 * (hi + hj);
                                double r2ij = xij * xij + yij * yij;
                                double muij = (hij * vijposij) / (r2ij + eta * eta * hij * hij);
                                double piij = (-alpha * cij * muij + beta * muij * muij) / rhoij;
                                vt[0] += -mass * piij * w_x;
                                vt[1] += -mass * piij * w_y;
                            }
                            xt[0] += -eps * w * mass / rhoij * vijx;
                            xt[1] += -eps * w * mass / rhoij * vijy;
                        }
                        if (thermal_alpha != 0.) {
                            double xij = pix - pjx, yij = piy - pjy;
                            double rij = sqrt(xij * xij + yij * yij);
                            if (rij > 1e-8) {
                                double eijx = xij / rij, eijy = yij / rij;
                                double rij1 = 1. / rij;
                                T_lapl += 2.0 * (mass / rhoj) * (Ti - Tj) * rij1 * (eijx * w_x + eijy * w_y);
                            }
                        }
                    }
                }
            }
        }
        for (int c = 0; c < 4; c++) { P->S_der[4 * pidx + c] = sd[c]; P->v_der[4 * pidx + c] = vd[c]; }
        P->pos_t[2 * pidx] = xt[0]; P->pos_t[2 * pidx + 1] = xt[1];
        P->vel_t[2 * pidx] = vt[0]; P->vel_t[2 * pidx + 1] = vt[1];
        if (thermal_alpha != 0.) P->T_t[pidx] = thermal_alpha * T_lapl;
    }
}

void orc_interactions_monaghan(sph_particles *P, const int32_t *cell_start, const int32_t *cell_end,
                               const sph_geom_constants *g, const sph_constants *C) {
    monaghan_impl(P, cell_start, cell_end, g, C, 0);
}

void orc_interactions_monaghan_pse_build(sph_particles *P, const int32_t *cell_start, const int32_t *cell_end,
                                         const sph_geom_constants *g, const sph_constants *C) {
    monaghan_impl(P, cell_start, cell_end, g, C, 1);
}

// actions_gpu.cu:280-314 do_material_stress_rate_jaumann (GLM column-major 3x3
// products written out; see the element formulas in the comments)
void orc_material_stress_rate_jaumann(sph_particles *P, const sph_constants *C) {
    const int N = P->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        if (P->tool_particle[i] == 1.) continue;
        double G = C->phys.G;
        double vx_x = P->v_der[4 * i], vx_y = P->v_der[4 * i + 1], vy_x = P->v_der[4 * i + 2], vy_y = P->v_der[4 * i + 3];
        double Sxx = P->S[4 * i], Sxy = P->S[4 * i + 1], Syy = P->S[4 * i + 2], Szz = P->S[4 * i + 3];
        double e01 = 0.5 * (vx_y + vy_x);
        double om_c1r0 = 0.5 * (vx_y - vy_x);   // omega[1][0]
        double om_c0r1 = 0.5 * (vy_x - vx_y);   // omega[0][1]
        double tr = vx_x + vy_y + 0.;
        double s = (1. / 3.) * tr;
        double twoG = 2. * G;
        // 2G (epsdot - tr/3 I)
        double a00 = twoG * (vx_x - s), a01 = twoG * (e01 - 0.), a11 = twoG * (vy_y - s), a22 = twoG * (0. - s);
        // omega*S and S*transpose(omega): only the omega[1][0], omega[0][1] terms survive
        double oS00 = om_c1r0 * Sxy;            // omega[1][0]*S[0][1]
        double oS01 = om_c0r1 * Sxx;            // omega[0][1]*S[0][0]
        double oS11 = om_c0r1 * Sxy;            // omega[0][1]*S[1][0]
        double So00 = Sxy * om_c1r0;            // S[1][0]*omegaT[0][1]
        double So01 = Syy * om_c1r0;            // S[1][1]*omegaT[0][1]  (element [0][1])
        double So11 = Sxy * om_c0r1;            // S[0][1]*omegaT[1][0]
        P->S_t[4 * i + 0] = (a00 + oS00) + So00;
        P->S_t[4 * i + 1] = (a01 + oS01) + So01;
        P->S_t[4 * i + 2] = (a11 + oS11) + So11;
        P->S_t[4 * i + 3] = (a22 + 0.) + 0.;
    }
}

// actions_gpu.cu:626-639 do_contmech_continuity
void orc_contmech_continuity(sph_particles *P) {
    const int N = P->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        if (P->tool_particle[i] != 0.) continue;
        P->rho_t[i] = -P->rho[i] * (P->v_der[4 * i] + P->v_der[4 * i + 3]);
    }
}

// actions_gpu.cu:641-671 do_contmech_momentum
void orc_contmech_momentum(sph_particles *P, const sph_constants *C) {
    const int N = P->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        if (P->tool_particle[i] != 0.) continue;
        double mass = C->phys.mass;
        const double *sd = P->S_der + 4 * i;
        P->vel_t[2 * i] += sd[0] + sd[1] + P->fc[2 * i] / mass + P->ft[2 * i] / mass;
        P->vel_t[2 * i + 1] += sd[2] + sd[3] + P->fc[2 * i + 1] / mass + P->ft[2 * i + 1] / mass;
    }
}

// actions_gpu.cu:673-687 do_contmech_advection
void orc_contmech_advection(sph_particles *P) {
    const int N = P->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        if (P->tool_particle[i] != 0.) continue;
        P->pos_t[2 * i] = P->pos_t[2 * i] + P->vel[2 * i];
        P->pos_t[2 * i + 1] = P->pos_t[2 * i + 1] + P->vel[2 * i + 1];
    }
}

// actions_gpu.cu:689-754 do_plasticity_johnson_cook.  Returns the number of
// particles whose secant solve hit the iteration cap.
int orc_plasticity_johnson_cook(sph_particles *P, const sph_constants *C, double dt, int64_t *secant_iters) {
    const int N = P->N;
    int capped = 0;
    int64_t its = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : capped, its)
    for (int pidx = 0; pidx < N; pidx++) {
        if (P->tool_particle[pidx] != 0.) continue;
        if (P->blanked[pidx] == 1.) continue;
        double mu = C->phys.G;
        double Sxx = P->S[4 * pidx], Sxy = P->S[4 * pidx + 1], Syy = P->S[4 * pidx + 2], Szz = P->S[4 * pidx + 3];
        double norm_Strial = sqrtf_d(Sxx * Sxx + Syy * Syy + Szz * Szz + 2. * Sxy * Sxy);
        double p = P->p[pidx];
        double cxx = Sxx - p, cyy = Syy - p, czz = Szz - p, cxy = Sxy;
        double eps_pl = P->eps_pl[pidx];
        double eps_pl_dot = P->eps_pl_dot[pidx];
        double T = P->T[pidx];
        double svm = sqrtf_d((cxx * cxx + cyy * cyy + czz * czz) - cxx * cyy - cxx * czz - cyy * czz + 3.0 * cxy * cxy);
        double sigma_Y = sigma_yield(C->joco, eps_pl, eps_pl_dot, T);
        if (svm < sigma_Y) { P->eps_pl_dot[pidx] = 0.; continue; }
        int it = 0;
        double delta_lambda = solve_secant(C->joco, fmax(eps_pl_dot * dt * sqrt(2. / 3.), 1e-8), 1e-6,
                                           norm_Strial, eps_pl, T, dt, C->phys.G, &it);
        if (it < 0) { capped++; it = -it; }
        its += it;
        // sqrtf(2.0/3.0) * fmaxf(delta_lambda, 0.): both calls return float, so the
        // reference multiplies in float (actions_gpu.cu:728-729)
        const float inc = sqrtf((float)(2.0 / 3.0)) * fmaxf((float)delta_lambda, 0.f);
        double eps_pl_new = eps_pl + (double)inc;
        double eps_pl_dot_new = (double)inc / dt;
        P->eps_pl[pidx] = eps_pl_new;
        P->eps_pl_dot[pidx] = eps_pl_dot_new;
        P->S[4 * pidx + 0] = Sxx - Sxx / norm_Strial * delta_lambda * 2. * mu;
        P->S[4 * pidx + 2] = Syy - Syy / norm_Strial * delta_lambda * 2. * mu;
        P->S[4 * pidx + 3] = Szz - Szz / norm_Strial * delta_lambda * 2. * mu;
        P->S[4 * pidx + 1] = Sxy - Sxy / norm_Strial * delta_lambda * 2. * mu;
        if (C->trml_wp.tq != 0.) {
            double delta_eps_pl = eps_pl_new - eps_pl;
            double sY = sigma_yield(C->joco, eps_pl_new, eps_pl_dot_new, T);
            double rho = P->rho[pidx];
            P->T[pidx] += C->trml_wp.tq / (C->trml_wp.cp * rho) * delta_eps_pl * sY;
        }
        if (P->T[pidx] > C->joco.Tmelt) {
            P->T[pidx] = C->joco.Tmelt;
            P->blanked[pidx] = 1.;
        }
    }
    if (secant_iters) *secant_iters = its;
    return capped;
}

// actions_gpu.cu:765-781 do_boundary_conditions
void orc_boundary_conditions(sph_particles *P) {
    const int N = P->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++) {
        if (P->tool_particle[i] != 0.) continue;
        if (P->fixed[i] != 0.) {
            P->vel[2 * i] = 0.; P->vel[2 * i + 1] = 0.;
            P->fc[2 * i] = 0.; P->fc[2 * i + 1] = 0.;
            P->pos_t[2 * i] = 0.; P->pos_t[2 * i + 1] = 0.;
            P->vel_t[2 * i] = 0.; P->vel_t[2 * i + 1] = 0.;
        }
    }
}

// actions_gpu.cu:756-763 do_boundary_conditions_thermal (launched only when
// thermals_tool.alpha != 0, actions_gpu.cu:881-886,938-944)
void orc_boundary_conditions_thermal(sph_particles *P, const sph_constants *C) {
    if (C->trml_tool.alpha == 0.) return;
    const int N = P->N;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; i++)
        if (P->fixed[i] == 1.) P->T[i] = C->trml_wp.T_init;
}

// actions_gpu.cu:787-824 do_invalidate.  Returns the number blanked.
int orc_invalidate(sph_particles *P) {
    const int N = P->N;
    int cnt = 0;
#pragma omp parallel for schedule(static) reduction(+ : cnt)
    for (int i = 0; i < N; i++) {
        if (P->blanked[i] == 1.) continue;
        bool invalid = false;
        auto bad = [](double v) { return std::isnan(v) || std::isinf(v); };
        invalid = invalid || bad(P->pos_t[2 * i]) || bad(P->pos_t[2 * i + 1]);
        invalid = invalid || bad(P->vel_t[2 * i]) || bad(P->vel_t[2 * i + 1]);
        for (int c = 0; c < 4; c++) invalid = invalid || bad(P->S_t[4 * i + c]);
        invalid = invalid || bad(P->rho_t[i]) || bad(P->T_t[i]);
        if (invalid) { P->blanked[i] = 1.; cnt++; }
    }
    return cnt;
}

// actions_gpu.cu:345-420 do_material_fric_heat_gen_FEM_v21 (WEAR_NODE_SHIFT off).
// fric_heat is accumulated in particle index order.  Returns NaN-blanked count.
// WEAR_NODE_SHIFT statistics (actions_gpu.cu:401-419) when W != NULL:
// T_nodes = the FEM temperature at that point of the step.
static int fric_heat_impl(sph_particles *P, sph_segments *Sg, const sph_constants *C, const double vel_tool[2],
                          double dt, const double *T_nodes, sph_wear_state *W) {
    const int N = P->N;
    int nanb = 0;
    for (int pidx = 0; pidx < N; pidx++) {
        if (P->blanked[pidx] == 1.) continue;
        if (P->eps_pl[pidx] > 20.) continue;
        double ftx = P->ft[2 * pidx], fty = P->ft[2 * pidx + 1];
        double f_fric_mag = sqrtf_d(ftx * ftx + fty * fty);
        int seg = P->on_seg[pidx];
        if (seg < 0 || seg >= Sg->n) continue;   // the reference stores only -1 or a valid id
        double partition_wp = C->tool.beta;
        double nx = P->n[2 * pidx], ny = P->n[2 * pidx + 1];
        double vpx = P->vel[2 * pidx], vpy = P->vel[2 * pidx + 1];
        double vdx = vpx - vel_tool[0], vdy = vpy - vel_tool[1];
        double vdn = vdx * nx + vdy * ny;
        double vrx = vdx - vdn * nx, vry = vdy - vdn * ny;
        double v_rel_mag = sqrtf_d(vrx * vrx + vry * vry);
        double value = C->tool.eta * f_fric_mag * v_rel_mag;
        if (std::isnan(v_rel_mag)) { P->blanked[pidx] = 1.; nanb++; continue; }
        double fcx = P->fc[2 * pidx], fcy = P->fc[2 * pidx + 1];
        double f_normal = sqrtf_d(fcx * fcx + fcy * fcy);
        double rho_ = P->rho[pidx];
        double length = sqrtf_d(C->tool.slave_mass / rho_);
        if (v_rel_mag > 0.03) continue;
        double T_buffer = P->T[pidx] + value * (1 - partition_wp) * dt / C->trml_wp.cp / C->phys.mass;
        if (T_buffer > 1550.) {
            P->T[pidx] = 1550.;
            continue;
        } else {
            P->T[pidx] = T_buffer;
            Sg->fric_heat[seg] += value * partition_wp;
        }
        if (W) {
            int left_no = Sg->marks[4 * seg + 2], right_no = Sg->marks[4 * seg + 3];
            double T_seg = 0.5 * (T_nodes[left_no] + T_nodes[right_no]);
            double vel_tool_norm = sqrt(vel_tool[0] * vel_tool[0] + vel_tool[1] * vel_tool[1]);
            if (v_rel_mag > 0.008) continue;
            else if (v_rel_mag > vel_tool_norm * 8.0 && fabs(ny) > 0.5) continue;
            double pressure_trial = f_normal / length;
            W->phys_para[4 * seg + 0] += 1.;
            W->phys_para[4 * seg + 1] += pressure_trial;
            W->phys_para[4 * seg + 2] += v_rel_mag;
            W->phys_para[4 * seg + 3] += T_seg;
            W->sliding_force[seg] += f_fric_mag / length;
        }
    }
    return nanb;
}

int orc_fric_heat_gen_fem(sph_particles *P, sph_segments *Sg, const sph_constants *C, const double vel_tool[2],
                          double dt) {
    return fric_heat_impl(P, Sg, C, vel_tool, dt, nullptr, nullptr);
}

int orc_fric_heat_gen_fem_wear(sph_particles *P, sph_segments *Sg, const sph_constants *C, const double vel_tool[2],
                               double dt, const double *T_nodes, sph_wear_state *W) {
    return fric_heat_impl(P, Sg, C, vel_tool, dt, T_nodes, W);
}

// actions_gpu.cu:423-583 do_compute_contact_forces_FEM_tool_v3_s1.
// Returns a bitmask of SPH_STATUS_CONTACT_* events.
uint32_t orc_contact_s1(sph_particles *P, const sph_segments *Sg, const sph_constants *C, const double tl_ref[2],
                        double ref_dist, const double vel_t[2], double dt) {
    const int N = P->N;
    const int seg_num = Sg->n;
    uint32_t ev = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : ev)
    for (int idx = 0; idx < N; idx++) {
        if (P->blanked[idx] == 1.) continue;
        double pos[2] = {P->pos[2 * idx], P->pos[2 * idx + 1]};
        double vs[2] = {P->vel[2 * idx], P->vel[2 * idx + 1]};
        int inside = 0;
        double ddx = pos[0] - tl_ref[0], ddy = pos[1] - tl_ref[1];
        if (sqrt(ddx * ddx + ddy * ddy) < 1.05 * ref_dist)
            inside = inside_judgement(pos, Sg->left, Sg->right, seg_num);
        auto zero_out = [&]() {
            P->fc[2 * idx] = 0.; P->fc[2 * idx + 1] = 0.;
            P->ft[2 * idx] = 0.; P->ft[2 * idx + 1] = 0.;
            P->n[2 * idx] = 0.; P->n[2 * idx + 1] = 0.;
            P->on_seg[idx] = -1;
        };
        if (inside == 0) { zero_out(); continue; }
        double gN = 0., n_[2] = {0., 0.};
        int seg_no = find_shortest_distance_v1(pos, gN, n_, Sg->left, Sg->right, Sg->normal, seg_num);
        P->on_seg[idx] = seg_no;
        if (seg_no == -1) { zero_out(); ev |= SPH_STATUS_CONTACT_NOSEG; continue; }
        if (gN < -0.00025) {
            P->blanked[idx] = 1.;
            zero_out();
            ev |= SPH_STATUS_CONTACT_DEEP;
            continue;
        }
        double dt2 = dt * dt;
        double s1 = -C->tool.slave_mass * gN;
        double fN[2] = {s1 * n_[0] / dt2 * C->tool.contact_alpha, s1 * n_[1] / dt2 * C->tool.contact_alpha};
        double v[2] = {vs[0] - vel_t[0], vs[1] - vel_t[1]};
        double vel_dot_nor = v[0] * n_[0] + v[1] * n_[1];
        double vr[2] = {v[0] - n_[0] * vel_dot_nor, v[1] - n_[1] * vel_dot_nor};
        double fricold[2] = {P->ft[2 * idx], P->ft[2 * idx + 1]};
        double am = C->tool.contact_alpha * C->tool.slave_mass;
        double kdeltae[2] = {am * vr[0] / dt, am * vr[1] / dt};
        double cof = C->tool.mu;
        double fy = cof * sqrt(fN[0] * fN[0] + fN[1] * fN[1]);
        double fstar[2] = {fricold[0] - kdeltae[0], fricold[1] - kdeltae[1]};
        double lfs = sqrt(fstar[0] * fstar[0] + fstar[1] * fstar[1]);
        double fT[2];
        if (lfs > fy) {
            fT[0] = fy * fstar[0] / lfs;
            fT[1] = fy * fstar[1] / lfs;
        } else {
            fT[0] = fstar[0];
            fT[1] = fstar[1];
        }
        P->fc[2 * idx] = fN[0]; P->fc[2 * idx + 1] = fN[1];
        P->ft[2 * idx] = fT[0]; P->ft[2 * idx + 1] = fT[1];
        P->n[2 * idx] = n_[0]; P->n[2 * idx + 1] = n_[1];
    }
    return ev;
}

// actions_gpu.cu:585-617 do_compute_contact_forces_FEM_tool_v3_s2 (accumulation
// in particle index order)
void orc_contact_s2(sph_particles *P, sph_segments *Sg, const sph_constants *C, const double *T_nodes, double dt) {
    const int N = P->N;
    for (int idx = 0; idx < N; idx++) {
        if (P->blanked[idx] == 1.) continue;
        int seg_no = P->on_seg[idx];
        if (seg_no < 0 || seg_no >= Sg->n) continue;
        int left_no = Sg->marks[4 * seg_no + 2];
        int right_no = Sg->marks[4 * seg_no + 3];
        double T_ = P->T[idx];
        double rho_ = P->rho[idx];
        double T_seg = 0.5 * (T_nodes[left_no] + T_nodes[right_no]);
        double delta_T = T_seg - T_;
        double length = sqrtf_d(C->tool.slave_mass / rho_);
        Sg->heat_exchange[2 * seg_no] += T_ * length;
        Sg->heat_exchange[2 * seg_no + 1] += length;
        double delta_T_part = delta_T * C->tool.h * length / C->trml_wp.cp / C->tool.slave_mass * dt;
        if (delta_T_part < 0) P->T[idx] += fmax(delta_T_part, delta_T);
        else P->T[idx] += fmin(delta_T_part, delta_T);
    }
}

// tool_FEM.cu:119-139 do_segments_update (flank_retreat == 0 without wear)
// (y + vel.y dt + flank_retreat, left to right; flank_retreat is 0 without wear)
void orc_segments_update_flank(sph_segments *Sg, const double vel[2], double dt, double flank_retreat) {
    for (int i = 0; i < Sg->n; i++) {
        double lx = Sg->left[2 * i], ly = Sg->left[2 * i + 1], rx = Sg->right[2 * i], ry = Sg->right[2 * i + 1];
        Sg->left[2 * i] = lx + vel[0] * dt;
        Sg->left[2 * i + 1] = ly + vel[1] * dt + flank_retreat;
        Sg->right[2 * i] = rx + vel[0] * dt;
        Sg->right[2 * i + 1] = ry + vel[1] * dt + flank_retreat;
        Sg->heat_exchange[2 * i] = 0; Sg->heat_exchange[2 * i + 1] = 0;
        Sg->fric_heat[i] = 0.;
    }
}

void orc_segments_update(sph_segments *Sg, const double vel[2], double dt) { orc_segments_update_flank(Sg, vel, dt, 0.); }

// tool_FEM.cu:109-117 do_tool_update_FEM_gpu and the host bookkeeping of
// tool_FEM::tool_update_FEM_gpu (:1552-1559)
// (position.y += vel.y dt + flank_retreat, tool_FEM.cu:115; flank_contact =
// lowest_point afterwards, tool_FEM.cu:1567-1569)
void orc_tool_update(sph_fem *F, sph_tool_state *ts, double dt) {
    for (int i = 0; i < F->n_nodes; i++) {
        F->position[2 * i] += ts->vel[0] * dt;
        F->position[2 * i + 1] += ts->vel[1] * dt + ts->flank_retreat;
    }
    ts->tl_point_ref[0] += ts->vel[0] * dt; ts->tl_point_ref[1] += ts->vel[1] * dt;
    ts->br_point[0] += ts->vel[0] * dt; ts->br_point[1] += ts->vel[1] * dt;
    ts->lowest_point += ts->vel[1] * dt;
    ts->right_point += ts->vel[0] * dt;
    ts->flank_contact = ts->lowest_point;
}

// FEM_thermal_gpu.cu:902-921 reset_FEM_server: T_old = T, f_temp = f, K_temp = K
void orc_fem_reset_server(const sph_fem *F, double *T_old, double *f_temp, double *K_temp) {
    std::memcpy(T_old, F->T, sizeof(double) * F->n_nodes);
    std::memcpy(f_temp, F->f, sizeof(double) * F->n_nodes);
    std::memcpy(K_temp, F->K, sizeof(double) * F->nnz);
}

// FEM_thermal_gpu.cu:865-877 apply_robin_bdc -> :342-386 (colour launches
// 1..n_colors in order, segments in index order within a colour)
void orc_fem_apply_robin(const sph_fem *F, const sph_segments *Sg, const sph_constants *C, int n_colors,
                         double *K_temp, double *f_temp) {
    for (int col = 1; col < n_colors + 1; col++) {
        for (int idx = 0; idx < Sg->n; idx++) {
            if (Sg->marks[4 * idx + 1] != col) continue;
            if (Sg->heat_exchange[2 * idx + 1] == 0) continue;
            double T_cont_particle = Sg->heat_exchange[2 * idx] / Sg->heat_exchange[2 * idx + 1];
            double fric_eng = Sg->fric_heat[idx];
            int l = Sg->marks[4 * idx + 2], r = Sg->marks[4 * idx + 3];
            double dxs = Sg->left[2 * idx] - Sg->right[2 * idx], dys = Sg->left[2 * idx + 1] - Sg->right[2 * idx + 1];
            double dist = sqrtf_d(dxs * dxs + dys * dys);
            f_temp[l] += 0.5 * C->tool.h * dist * T_cont_particle + 0.5 * fric_eng;
            f_temp[r] += 0.5 * C->tool.h * dist * T_cont_particle + 0.5 * fric_eng;
            double em = 0.5 * dist;
            for (int k = F->row_ptr[l]; k < F->row_ptr[l + 1]; k++)
                if (F->col_ind[k] == l) { K_temp[k] += C->tool.h * em; break; }
            for (int k = F->row_ptr[r]; k < F->row_ptr[r + 1]; k++)
                if (F->col_ind[k] == r) { K_temp[k] += C->tool.h * em; break; }
        }
    }
}

// FEM_thermal_gpu.cu:443-458 do_calculate_temp_rate (uses K_temp, f_temp, T)
void orc_fem_calculate_temp_rate(sph_fem *F, const double *K_temp, const double *f_temp) {
    for (int idx = 0; idx < F->n_nodes; idx++) {
        double buffer = 0.;
        for (int i = F->row_ptr[idx]; i < F->row_ptr[idx + 1]; i++) buffer += K_temp[i] * F->T[F->col_ind[i]];
        F->k[idx] = F->M_inv[idx] * (f_temp[idx] - buffer);
    }
}

// FEM_thermal_gpu.cu:460-468 do_calculate_temp
void orc_fem_calculate_temp(sph_fem *F, const double *T_old, double dt) {
    for (int idx = 0; idx < F->n_nodes; idx++) F->T[idx] = dt * F->k[idx] + T_old[idx];
}

// ---- tool wear by nodal shift (WEAR_NODE_SHIFT) -----------------------------------------
// mesh_structure_GPU.cu:1063-1148: layer 1 = elements with a cutting edge
// (cutting_boundary_elements); layer 2 = every other element with a node on the
// cutting edge (CuttingEdgeNum) or a node of a layer-1 element.
void orc_wear_layers(int n_elements, const int32_t *elements, const int32_t *cutting_flags, int n_nodes,
                     int32_t *layer) {
    std::vector<char> edge_node(n_nodes, 0), l1_node(n_nodes, 0);
    for (int e = 0; e < n_elements; e++) {
        const int32_t *el = elements + 3 * e, *cf = cutting_flags + 3 * e;
        const int pairs[3][2] = {{el[0], el[1]}, {el[1], el[2]}, {el[2], el[0]}};
        layer[2 * e] = layer[2 * e + 1] = 0;
        for (int a = 0; a < 3; a++)
            if (cf[a]) {
                edge_node[pairs[a][0]] = edge_node[pairs[a][1]] = 1;
                layer[2 * e] = 1;
            }
    }
    for (int e = 0; e < n_elements; e++)
        if (layer[2 * e])
            for (int a = 0; a < 3; a++) l1_node[elements[3 * e + a]] = 1;
    for (int e = 0; e < n_elements; e++) {
        if (layer[2 * e]) continue;
        for (int a = 0; a < 3; a++) {
            const int nd = elements[3 * e + a];
            if (edge_node[nd] || l1_node[nd]) layer[2 * e + 1] = 1;
        }
    }
}

// tool_FEM.cu:1595-1609 segments_wear_rate_reset
void orc_wear_reset(sph_wear_state *W) {
    for (int s = 0; s < W->n_seg; s++) {
        for (int c = 0; c < 4; c++) W->phys_para[4 * s + c] = 0.;
        W->sliding_force[s] = 0.;
        W->wear_nodes[s] = 0.;
    }
}

// FEM_thermal_gpu.cu:71-109: lumped mass m and stiffness ke of a linear triangle,
// ke = w 3 k |det J| B^T B with B = J^-T grad_ref (the glm::inverse of the
// transposed Jacobian written out).
static void p1_element_ref(const double *pos, const int32_t *el, const sph_tool_constants &tc, double &m,
                           double ke[3][3]) {
    const double weights = 1. / 3. * 0.5;
    const double c0x = pos[2 * el[0]], c0y = pos[2 * el[0] + 1];
    const double J0x = pos[2 * el[1]] - c0x, J0y = pos[2 * el[1] + 1] - c0y;   // jacobian[0]
    const double J1x = pos[2 * el[2]] - c0x, J1y = pos[2 * el[2] + 1] - c0y;   // jacobian[1]
    const double determinant = fabs(J0x * J1y - J1x * J0y);
    m = weights * tc.cp * tc.rho * determinant;
    // transpose(J) has rows J0, J1; its inverse: (1 / det) [[J1y, -J0y], [-J1x, J0x]]
    const double d = J0x * J1y - J0y * J1x;
    const double iT[2][2] = {{J1y / d, -J0y / d}, {-J1x / d, J0x / d}};
    const double G[3][2] = {{-1., -1.}, {1., 0.}, {0., 1.}};
    double B[3][2];
    for (int a = 0; a < 3; a++) {
        B[a][0] = iT[0][0] * G[a][0] + iT[0][1] * G[a][1];
        B[a][1] = iT[1][0] * G[a][0] + iT[1][1] * G[a][1];
    }
    const double value = tc.k * determinant;
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) ke[a][b] = weights * 3. * value * (B[a][0] * B[b][0] + B[a][1] * B[b][1]);
}

// do_mesh_adjustment_wear (FEM_thermal_gpu.cu:476-577) over every layer element,
// sign -1 (mesh_retreat_wear) or +1 (mesh_resume_wear).
static void mesh_adjust(sph_fem *F, sph_wear_state *W, const sph_tool_constants &tc, double sign) {
    for (int e = 0; e < W->n_elements; e++) {
        if (W->layer[2 * e] == 0 && W->layer[2 * e + 1] == 0) continue;
        const int32_t *el = W->elements + 4 * e;
        double m, ke[3][3];
        p1_element_ref(F->position, el, tc, m, ke);
        for (int a = 0; a < 3; a++) {
            W->M[el[a]] += sign * m;
            for (int k = F->row_ptr[el[a]]; k < F->row_ptr[el[a] + 1]; k++)
                for (int b = 0; b < 3; b++)
                    if (F->col_ind[k] == el[b]) F->K[k] += sign * ke[b][a];
        }
    }
}

// actions_gpu.cu:1009-1020 wear_adjustment: retreat, nodal shift
// (do_nodal_shift_wear_smooth_temp, tool_FEM.cu:299-432, RESTRICT_WEAR_TEMP and
// USE_USUI_RAKE_FLANK), resume, do_segment_wear_update (tool_FEM.cu:520-545),
// do_correct_flank_contact over the first 512 segments (tool_FEM.cu:559-587) and
// the lumped inverse mass.  Segments in index order.
void orc_wear_adjustment(sph_fem *F, sph_segments *Sg, sph_tool_state *ts, sph_wear_state *W,
                         const sph_constants *C, const sph_wear_constants *wc, double dt) {
    const sph_tool_constants &tc = C->tool;
    mesh_adjust(F, W, tc, -1.);
    for (int s = 0; s < Sg->n; s++) {
        const double *w = W->phys_para + 4 * s;
        if (w[0] == 0.) continue;
        const int left = Sg->marks[4 * s + 2], right = Sg->marks[4 * s + 3];
        double pressure = w[1] / w[0];
        double vel = w[2] / w[0];
        double Tl = F->T[left], Tr = F->T[right];
        if (vel > 0.008) continue;
        Tl = fmin(Tl, 1350.);
        Tr = fmin(Tr, 1350.);
        vel = fmin(vel, 0.008);
        pressure = fmin(pressure, 0.04);
        const double nx = Sg->normal[2 * s], ny = Sg->normal[2 * s + 1];
        double wl, wr;
        if (fabs(nx) > 0.85) {
            wl = dt * wc->C * pressure * vel * exp(-wc->D / Tl);
            wr = dt * wc->C * pressure * vel * exp(-wc->D / Tr);
        } else {
            wl = dt * wc->A * pressure * vel * exp(-wc->B / Tl);
            wr = dt * wc->A * pressure * vel * exp(-wc->B / Tr);
        }
        W->wear_nodes[s] = (wl + wr) / dt;
        F->position[2 * left] += nx * wl;
        F->position[2 * left + 1] += ny * wl;
        F->position[2 * right] += nx * wr;
        F->position[2 * right + 1] += ny * wr;
    }
    mesh_adjust(F, W, tc, 1.);
    double mn = FLT_MAX;
    for (int s = 0; s < Sg->n; s++) {
        const int l = Sg->marks[4 * s + 2], r = Sg->marks[4 * s + 3];
        const double lx = F->position[2 * l], ly = F->position[2 * l + 1];
        const double rx = F->position[2 * r], ry = F->position[2 * r + 1];
        Sg->left[2 * s] = lx; Sg->left[2 * s + 1] = ly;
        Sg->right[2 * s] = rx; Sg->right[2 * s + 1] = ry;
        const double dx = rx - lx, dy = ry - ly;
        const double inv = 1. / sqrt(dy * dy + (-dx) * (-dx));
        Sg->normal[2 * s] = dy * inv;
        Sg->normal[2 * s + 1] = -dx * inv;
        if (s < 512) mn = fmin(mn, ly);
    }
    ts->flank_retreat = ts->flank_contact - mn;
    for (int i = 0; i < F->n_nodes; i++) F->M_inv[i] = 1. / W->M[i];
}

// leap_frog.cu:162-248 leap_frog::step(particle_gpu*, grid_base*, tool_FEM*) with
// WEAR_NODE_SHIFT off; without a tool (Sg == NULL) the tool calls are skipped
// (leap_frog.cu:99-160 with no SPH tool).  cell_start/cell_end persist between
// calls (cell_end of empty cells stays stale as in the reference).
// Returns SPH_STATUS_* bits observed during the step.
uint32_t orc_step_wear(sph_particles *P, int32_t *cell_start, int32_t *cell_end, const sph_geom_constants *g,
                       const sph_constants *C, double dt, sph_segments *Sg, sph_fem *F, sph_tool_state *ts,
                       int n_colors, sph_wear_state *W, const sph_wear_constants *wc, int wear_mode) {
    if (!W) wear_mode = 0;
    const int N = P->N;
    uint32_t st = 0;
    std::vector<double> pos_init(2 * (size_t)N), vel_init(2 * (size_t)N), S_init(4 * (size_t)N), rho_init(N), T_init(N);
    orc_compute_hashes(P, g);
    if (orc_sort_green(P, cell_start, cell_end, g->num_cell) > 0) st |= SPH_STATUS_OUT_OF_GRID;
    orc_init(P, pos_init.data(), vel_init.data(), S_init.data(), rho_init.data(), T_init.data());
    std::vector<double> T_old, f_temp, K_temp;
    if (Sg) {
        T_old.resize(F->n_nodes); f_temp.resize(F->n_nodes); K_temp.resize(F->nnz);
        orc_fem_reset_server(F, T_old.data(), f_temp.data(), K_temp.data());
        if (wear_mode) orc_wear_reset(W);
    }
    orc_predict(P, pos_init.data(), vel_init.data(), S_init.data(), rho_init.data(), T_init.data(), dt);
    if (Sg) orc_fem_calculate_temp(F, T_old.data(), 0.5 * dt);
    orc_material_eos(P, C);
    orc_corrector_artificial_stress(P, C);
    orc_interactions_monaghan(P, cell_start, cell_end, g, C);
    orc_material_stress_rate_jaumann(P, C);
    orc_contmech_continuity(P);
    orc_contmech_momentum(P, C);
    orc_contmech_advection(P);
    orc_correct(P, pos_init.data(), vel_init.data(), S_init.data(), rho_init.data(), T_init.data(), dt);
    if (Sg) {
        if (fric_heat_impl(P, Sg, C, ts->vel, dt, F->T, wear_mode ? W : nullptr) > 0) st |= SPH_STATUS_FRIC_NAN;
        orc_fem_apply_robin(F, Sg, C, n_colors, K_temp.data(), f_temp.data());
        orc_fem_calculate_temp_rate(F, K_temp.data(), f_temp.data());
        orc_fem_calculate_temp(F, T_old.data(), dt);
    }
    if (C->plastic) {
        int64_t its = 0;
        if (orc_plasticity_johnson_cook(P, C, dt, &its) > 0) st |= SPH_STATUS_SECANT_MAXITER;
    }
    if (Sg && wear_mode == 2) orc_wear_adjustment(F, Sg, ts, W, C, wc, dt);
    if (Sg) {
        orc_segments_update_flank(Sg, ts->vel, dt, ts->flank_retreat);
        orc_tool_update(F, ts, dt);
        st |= orc_contact_s1(P, Sg, C, ts->tl_point_ref, ts->ref_dist, ts->vel, dt);
        orc_contact_s2(P, Sg, C, F->T, dt);
    }
    orc_boundary_conditions(P);
    orc_boundary_conditions_thermal(P, C);
    if (orc_invalidate(P) > 0) st |= SPH_STATUS_NAN_BLANKED;
    return st;
}


// ---- rigid (SPH-mode) tool ---------------------------------------------------------------
// geometric_primitives.cpp:58-75 line(p1, p2)
static void rigid_line(const double *p1, const double *p2, double &a, double &b, int32_t &vertical) {
    double detM = p1[0] * 1. - 1. * p2[0];
    if (fabs(detM) < 1e-12) {
        vertical = 1;
        a = DBL_MAX;
        b = p1[0];
        return;
    }
    vertical = 0;
    a = (p1[1] * 1. - 1. * p2[1]) / detM;
    b = (p2[1] * p1[0] - p2[0] * p1[1]) / detM;
}

// tool.cpp:202-212 tool::update_tool: segment ends and fillet centre move by
// dt * velocity, the lines are rebuilt, the normals stay.
void orc_rigid_move(sph_rigid_tool *t, double dt) {
    for (int i = 0; i < t->n_seg; i++) {
        for (int a = 0; a < 2; a++) {
            t->left[i][a] += dt * t->vel[a];
            t->right[i][a] += dt * t->vel[a];
        }
        rigid_line(t->left[i], t->right[i], t->la[i], t->lb[i], t->vertical[i]);
    }
    if (t->has_fillet) {
        t->fillet_p[0] += dt * t->vel[0];
        t->fillet_p[1] += dt * t->vel[1];
    }
}

// tool_gpu.cu:205-216 update_tool_particles
void orc_rigid_move_particles(sph_particles *P, const double vel[2], double dt) {
    for (int i = 0; i < P->N; i++) {
        if (P->tool_particle[i] == 0.) continue;
        P->pos[2 * i] += dt * vel[0];
        P->pos[2 * i + 1] += dt * vel[1];
    }
}

// tool_gpu.cu:24-31 myatan2
static double rigid_myatan2(double y, double x) {
    double t = atan2(y, x);
    return (t > 0.) ? t : t + 2 * M_PI;
}

// tool_gpu.cu:33-58 circle_segment_distance
static double rigid_fillet_distance(const sph_rigid_tool *t, double qx, double qy) {
    double Ax = t->fillet_p[0], Ay = t->fillet_p[1], r = t->fillet_r;
    double Cx = Ax + r * (qx - Ax) / sqrt((qx - Ax) * (qx - Ax) + (qy - Ay) * (qy - Ay));
    double Cy = Ay + r * (qy - Ay) / sqrt((qx - Ax) * (qx - Ax) + (qy - Ay) * (qy - Ay));
    double th = rigid_myatan2(Ay - Cy, Ax - Cx);
    bool valid = th > fmin(t->fillet_t1, t->fillet_t2) && th < fmax(t->fillet_t1, t->fillet_t2);
    if (!valid) return FLT_MAX;
    return sqrt((Cx - qx) * (Cx - qx) + (Cy - qy) * (Cy - qy));
}

// tool_gpu.cu:60-76 segment_closest_point
static void rigid_closest(const sph_rigid_tool *t, int i, double qx, double qy, double &px, double &py) {
    if (t->vertical[i]) {
        px = t->lb[i];
        py = qy;
        return;
    }
    double bb = -1, cc = t->lb[i], aa = t->la[i];
    px = (bb * (bb * qx - aa * qy) - aa * cc) / (aa * aa + bb * bb);
    py = (aa * (-bb * qx + aa * qy) - bb * cc) / (aa * aa + bb * bb);
}

// glm::normalize: v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x)
static void rigid_normalize(double x, double y, double &nx, double &ny) {
    double inv = 1. / sqrt(x * x + y * y);
    nx = x * inv;
    ny = y * inv;
}

// tool_gpu.cu:82-134 establish_contact (a fillet exists iff there are 5 segments)
static bool rigid_establish_contact(const sph_rigid_tool *t, double qx, double qy, double cp[2], double n[2]) {
    bool has_fillet = t->n_seg == SPH_RIGID_MAX_SEG;
    bool in = true;
    for (int i = 0; i < t->n_seg; i++)
        in = in && ((t->left[i][0] - qx) * t->n[i][0] + (t->left[i][1] - qy) * t->n[i][1] < 0.);
    if (has_fillet) {
        double dx = t->fillet_p[0] - qx, dy = t->fillet_p[1] - qy;
        in = in || sqrt(dx * dx + dy * dy) < t->fillet_r;
    }
    if (!in) return false;
    double depth = FLT_MAX;
    for (int i = 0; i < t->n_seg; i++) {
        double d;
        if (t->vertical[i]) {
            d = fabs(t->left[i][0] - qx);
            if (d < depth) {
                depth = d;
                rigid_normalize(t->left[i][0] - qx, 0., n[0], n[1]);
                cp[0] = t->left[i][0];
                cp[1] = qy;
            }
        } else if (has_fillet && i == 2) {
            d = rigid_fillet_distance(t, qx, qy);
            if (d < depth) {
                depth = d;
                rigid_normalize(qx - t->fillet_p[0], qy - t->fillet_p[1], n[0], n[1]);
                cp[0] = t->fillet_p[0] + n[0] * t->fillet_r;
                cp[1] = t->fillet_p[1] + n[1] * t->fillet_r;
            }
        } else {
            double px, py;
            rigid_closest(t, i, qx, qy, px, py);
            d = sqrt((px - qx) * (px - qx) + (py - qy) * (py - qy));
            if (d < depth) {
                depth = d;
                n[0] = -t->n[i][0];
                n[1] = -t->n[i][1];
                cp[0] = px;
                cp[1] = py;
            }
        }
    }
    return true;
}

// tool_gpu.cu:146-202 do_compute_contact_forces (penalty with slave_mass =
// phys.mass, contact_alpha of the tool constants; LS-DYNA friction).  Blanked
// particles are not skipped, as in the reference.
void orc_contact_rigid(sph_particles *P, const sph_rigid_tool *t, const sph_constants *C, double dt) {
    const double ms = C->phys.mass, alpha = C->tool.contact_alpha;
    for (int i = 0; i < P->N; i++) {
        if (P->tool_particle[i] != 0.) continue;
        double xs[2] = {P->pos[2 * i], P->pos[2 * i + 1]}, vs[2] = {P->vel[2 * i], P->vel[2 * i + 1]};
        double xm[2] = {0., 0.}, n[2] = {0., 0.};
        if (!rigid_establish_contact(t, xs[0], xs[1], xm, n)) {
            for (int a = 0; a < 2; a++) P->fc[2 * i + a] = P->ft[2 * i + a] = P->n[2 * i + a] = 0.;
            continue;
        }
        double dt2 = dt * dt;
        double gN = (xs[0] - xm[0]) * n[0] + (xs[1] - xm[1]) * n[1];
        double fN[2], fT[2] = {0., 0.};
        for (int a = 0; a < 2; a++) fN[a] = -ms * gN * n[a] / dt2 * alpha;
        if (t->mu != 0.) {
            double v[2] = {vs[0] - t->vel[0], vs[1] - t->vel[1]};
            double vr[2] = {v[0] - v[0] * n[0], v[1] - v[1] * n[1]};
            double fricold[2] = {P->ft[2 * i], P->ft[2 * i + 1]};
            double kdeltae[2] = {alpha * ms * vr[0] / dt, alpha * ms * vr[1] / dt};
            double fy = t->mu * sqrt(fN[0] * fN[0] + fN[1] * fN[1]);
            double fstar[2] = {fricold[0] - kdeltae[0], fricold[1] - kdeltae[1]};
            double ls = sqrt(fstar[0] * fstar[0] + fstar[1] * fstar[1]);
            if (ls > fy) {
                fT[0] = fy * fstar[0] / ls;
                fT[1] = fy * fstar[1] / ls;
            } else {
                fT[0] = fstar[0];
                fT[1] = fstar[1];
            }
        }
        for (int a = 0; a < 2; a++) {
            P->fc[2 * i + a] = fN[a];
            P->ft[2 * i + a] = fT[a];
            P->n[2 * i + a] = n[a];
        }
    }
}

// actions_gpu.cu:316-343 do_material_fric_heat_gen (launched only when
// thermals_wp.eta != 0, actions_gpu.cu:955-965); blanked particles are not skipped.
void orc_fric_heat_rigid(sph_particles *P, const sph_constants *C, const double vel_tool[2], double dt) {
    if (C->trml_wp.eta == 0.) return;
    for (int i = 0; i < P->N; i++) {
        if (P->tool_particle[i] != 0.) continue;
        double fx = P->ft[2 * i], fy = P->ft[2 * i + 1];
        double f = sqrtf_d(fx * fx + fy * fy);
        if (f == 0.) continue;
        double nx = P->n[2 * i], ny = P->n[2 * i + 1];
        double vdx = P->vel[2 * i] - vel_tool[0], vdy = P->vel[2 * i + 1] - vel_tool[1];
        double vdn = vdx * nx + vdy * ny;
        double vrx = vdx - vdn * nx, vry = vdy - vdn * ny;
        double v = sqrtf_d(vrx * vrx + vry * vry);
        P->T[i] += C->trml_wp.eta * dt * f * v / (C->trml_wp.cp * C->phys.mass);
    }
}

// interactions_gpu.cu:84-140 do_interactions_heat_pse with kernels.cuh:67-84
// lapl_pse, over the 5x5 block of cells of edge h (launched only when
// thermals_workpiece.alpha != 0, :434-435).  alpha by the tool flag as the
// reference reads it: its tool-flag texture is bound over N ints of an N-double
// array (:448), so from index N/2 on the fetch reads flag 0 (workpiece alpha).
void orc_interactions_heat_pse(sph_particles *P, const int32_t *cell_start, const int32_t *cell_end,
                               const sph_geom_constants *g, const sph_constants *C) {
    if (C->trml_wp.alpha == 0.) return;
    const int N = P->N, nx = g->nx, ny = g->ny;
    const double mass = C->phys.mass;
#pragma omp parallel for schedule(dynamic, 256)
    for (int pidx = 0; pidx < N; pidx++) {
        if (P->blanked[pidx] == 1.) continue;
        double pix = P->pos[2 * pidx], piy = P->pos[2 * pidx + 1], hi = P->h[pidx], Ti = P->T[pidx];
        int hashi = P->hash[pidx];
        double alpha = (pidx < N / 2 && P->tool_particle[pidx] == 1.) ? C->trml_tool_sph.alpha : C->trml_wp.alpha;
        double T_ti = 0.;
        if (hashi >= 0 && hashi < g->num_cell) {
            int gi = hashi / ny, gj = hashi - gi * ny;
            int low_i = gi - 2 < 0 ? 0 : gi - 2, low_j = gj - 2 < 0 ? 0 : gj - 2;
            int high_i = gi + 3 > nx ? nx : gi + 3, high_j = gj + 3 > ny ? ny : gj + 3;
            for (int ii = low_i; ii < high_i; ii++)
                for (int jj = low_j; jj < high_j; jj++) {
                    int idx = ii * ny + jj;
                    int c_start = cell_start[idx], c_end = cell_end[idx];
                    if (c_start == -1) continue;
                    for (int iter = c_start; iter < c_end; iter++) {
                        double xij = pix - P->pos[2 * iter], yij = piy - P->pos[2 * iter + 1];
                        double xx = sqrt(xij * xij + yij * yij);
                        double h2 = hi * hi, h4 = h2 * h2;
                        double w2 = +4. / (h4 * M_PI) * exp(-xx * xx / (h2));
                        T_ti += (P->T[iter] - Ti) * w2 * mass / P->rho[iter];
                    }
                }
        }
        P->T_t[pidx] = alpha * T_ti;
    }
}

// leap_frog.cu:99-160 leap_frog::step(particle_gpu*, grid_base*) with an SPH
// (rigid) tool t (NULL: no tool); pse selects the Thermal_Conduction_PSE
// build.  Returns SPH_STATUS_* bits observed during the step.
uint32_t orc_step_rigid(sph_particles *P, int32_t *cell_start, int32_t *cell_end, const sph_geom_constants *g,
                        const sph_constants *C, double dt, sph_rigid_tool *t, int pse) {
    const int N = P->N;
    uint32_t st = 0;
    std::vector<double> pos_init(2 * (size_t)N), vel_init(2 * (size_t)N), S_init(4 * (size_t)N), rho_init(N), T_init(N);
    orc_compute_hashes(P, g);
    if (orc_sort_green(P, cell_start, cell_end, g->num_cell) > 0) st |= SPH_STATUS_OUT_OF_GRID;
    orc_init(P, pos_init.data(), vel_init.data(), S_init.data(), rho_init.data(), T_init.data());
    orc_predict(P, pos_init.data(), vel_init.data(), S_init.data(), rho_init.data(), T_init.data(), dt);
    orc_material_eos(P, C);
    orc_corrector_artificial_stress(P, C);
    monaghan_impl(P, cell_start, cell_end, g, C, pse);
    if (pse) orc_interactions_heat_pse(P, cell_start, cell_end, g, C);
    orc_material_stress_rate_jaumann(P, C);
    orc_contmech_continuity(P);
    orc_contmech_momentum(P, C);
    orc_contmech_advection(P);
    orc_correct(P, pos_init.data(), vel_init.data(), S_init.data(), rho_init.data(), T_init.data(), dt);
    if (t) orc_fric_heat_rigid(P, C, t->vel, dt);
    if (C->plastic) {
        int64_t its = 0;
        if (orc_plasticity_johnson_cook(P, C, dt, &its) > 0) st |= SPH_STATUS_SECANT_MAXITER;
    }
    if (t) {
        orc_rigid_move(t, dt);
        orc_rigid_move_particles(P, t->vel, dt);
        orc_contact_rigid(P, t, C, dt);
    }
    orc_boundary_conditions(P);
    orc_boundary_conditions_thermal(P, C);
    if (orc_invalidate(P) > 0) st |= SPH_STATUS_NAN_BLANKED;
    return st;
}


uint32_t orc_step(sph_particles *P, int32_t *cell_start, int32_t *cell_end, const sph_geom_constants *g,
                  const sph_constants *C, double dt, sph_segments *Sg, sph_fem *F, sph_tool_state *ts,
                  int n_colors) {
    return orc_step_wear(P, cell_start, cell_end, g, C, dt, Sg, F, ts, n_colors, nullptr, nullptr, 0);
}

}  // extern "C"
