// physics.cuh -- per-particle device functions of the SPH workpiece path.
// Each function cites the reference kernel it restates.  They are shared by
// the staged kernels (one launch per reference call) and the fused step.
#pragma once

#include <cfloat>

#include "common.cuh"

namespace sphfem {

// ---- kernels.cuh:25-65 cubic_spline (reference form, FP64) -------------------
__device__ __forceinline__ void cubic_spline(double xij, double yij, double hi, double &w, double &wx, double &wy) {
    w = 0.; wx = 0.; wy = 0.;
    double rr2 = xij * xij + yij * yij;
    double h1 = 1 / hi;
    double fourh2 = 4 * hi * hi;
    if (rr2 >= fourh2 || rr2 < 1e-8) return;
    double der, val;
    double rad = sqrtf_d(rr2);
    double q = rad * h1;
    double fac = kPiFac * h1 * h1;
    if (q > 1) {
        double t = 2 - q;
        double t2 = t * t;
        val = 0.25 * t2 * t2 * t2;
        der = -0.75 * t2 * h1 / rad;
    } else {
        val = 1 - 1.5 * q * q * (1 - 0.5 * q);
        der = -3.0 * q * (1 - 0.75 * q) * h1 / rad;
    }
    w = val * fac;
    wx = der * xij * fac;
    wy = der * yij * fac;
}

// ---- plasticity.cuh:21-39 sigma_yield ----------------------------------------
// Term_C depends only on the temperature, which is constant during one return
// mapping, so callers may pass it precomputed (identical arithmetic).
__device__ __forceinline__ double jc_term_c(const sph_joco_constants &jc, double t) {
    double theta = (t - jc.Tref) / (jc.Tmelt - jc.Tref);
    if (theta > 1.) theta = 1.;
    return 1.0 - pow(theta, jc.m);
}

__device__ __forceinline__ double sigma_yield_tc(const sph_joco_constants &jc, double eps_pl, double eps_pl_dot,
                                                 double term_c) {
    double Term_A = jc.A + jc.B * pow(eps_pl, jc.n);
    double Term_B;
    double eps_dot = eps_pl_dot / jc.eps_dot_ref;
    if (eps_dot > 1.0) Term_B = 1.0 + jc.C * log(eps_dot);
    else Term_B = pow((1.0 + eps_dot), jc.C);
    return Term_A * Term_B * term_c;
}

__device__ __forceinline__ double sigma_yield(const sph_joco_constants &jc, double eps_pl, double eps_pl_dot, double t) {
    return sigma_yield_tc(jc, eps_pl, eps_pl_dot, jc_term_c(jc, t));
}

// Same flow stress with the rate/strain terms in FP32 (powf/logf).  Used by the
// FP32-compensated mode, where only the secant residual stays in FP64.
__device__ __forceinline__ double sigma_yield_tc_f32(const sph_joco_constants &jc, double eps_pl, double eps_pl_dot,
                                                     double term_c) {
    float Term_A = (float)jc.A + (float)jc.B * powf((float)eps_pl, (float)jc.n);
    float Term_B;
    float eps_dot = (float)(eps_pl_dot / jc.eps_dot_ref);
    if (eps_dot > 1.0f) Term_B = 1.0f + (float)jc.C * logf(eps_dot);
    else Term_B = powf(1.0f + eps_dot, (float)jc.C);
    return (double)(Term_A * Term_B) * term_c;
}

// ---- plasticity.cuh:117-162 opt_fun + solve_secant ----------------------------
// Returns delta_lambda; *iters = iterations used, negative when the 100
// iteration cap was hit (plasticity.cuh:155-158).
template <bool kF32Yield>
__device__ __forceinline__ double solve_secant(const sph_joco_constants &jc, double init, double tol,
                                              double norm_Strial, double eps_pl_init, double term_c, double delta_t,
                                              double mu, int *iters, int max_iter = 100) {
    const double s23 = sqrt(2.0 / 3.0);
    auto opt_fun = [&](double dl) {
        double eq = eps_pl_init + s23 * fmax(dl, 0.);
        double eqd = s23 * fmax(dl, 0.) / delta_t;
        double sY = kF32Yield ? sigma_yield_tc_f32(jc, eq, eqd, term_c) : sigma_yield_tc(jc, eq, eqd, term_c);
        return norm_Strial - 2 * mu * dl - s23 * sY;
    };
    double delta_lambda = init;
    double delta_lambda_old = delta_lambda;
    int iter = 0;
    while (true) {
        double g = opt_fun(delta_lambda);
        double delta_lambda_1 = delta_lambda * 1.01;
        double g_1 = opt_fun(delta_lambda_1);
        double slope = (g - g_1) / (delta_lambda - delta_lambda_1);
        delta_lambda_old = delta_lambda;
        delta_lambda = delta_lambda - g / slope;
        if (delta_lambda < 0.) delta_lambda = -0.1 * delta_lambda;
        if (fabs(delta_lambda - delta_lambda_old) < tol) { *iters = iter + 1; return delta_lambda; }
        if (iter > max_iter) { *iters = -(iter + 1); return delta_lambda; }
        iter++;
    }
}

// ---- actions_gpu.cu:689-754 do_plasticity_johnson_cook (one particle) --------
// Reads/writes the particle's S, eps_pl, eps_pl_dot, T, blanked.  Returns
// status bits.  `iters_out` receives the secant iteration count (0 if elastic).
// dt: the time step of the particle's case.
template <bool kF32Yield>
__device__ __forceinline__ uint32_t plasticity_one(const KConsts &K, double dt, dbl4 &S, double p, double rho,
                                                   double &eps_pl, double &eps_pl_dot, double &T, double &blanked,
                                                   int *iters_out) {
    const sph_joco_constants &jc = K.c.joco;
    const double mu = K.c.phys.G;
    double Sxx = S.x, Syy = S.z, Szz = S.w, Sxy = S.y;
    double norm_Strial = sqrtf_d(Sxx * Sxx + Syy * Syy + Szz * Szz + 2. * Sxy * Sxy);
    double cxx = Sxx - p, cyy = Syy - p, czz = Szz - p, cxy = Sxy;
    double svm = sqrtf_d((cxx * cxx + cyy * cyy + czz * czz) - cxx * cyy - cxx * czz - cyy * czz + 3.0 * cxy * cxy);
    double term_c = jc_term_c(jc, T);
    double sigma_Y = kF32Yield ? sigma_yield_tc_f32(jc, eps_pl, eps_pl_dot, term_c)
                               : sigma_yield_tc(jc, eps_pl, eps_pl_dot, term_c);
    *iters_out = 0;
    if (svm < sigma_Y) {
        eps_pl_dot = 0.;
        return 0u;
    }
    int it = 0;
    double delta_lambda = solve_secant<kF32Yield>(jc, fmax(eps_pl_dot * dt * sqrt(2. / 3.), 1e-8), 1e-6, norm_Strial,
                                                  eps_pl, term_c, dt, mu, &it, K.secant_cap);
    uint32_t st = 0;
    if (it < 0) { st |= SPH_STATUS_SECANT_MAXITER; it = -it; }
    *iters_out = it;
    jc_log_record(K, (float)svm, (float)eps_pl, (float)eps_pl_dot, (float)T, (float)norm_Strial, (float)delta_lambda,
                  it, (float)dt);
    jc_count(K, it);
    // sqrtf(2.0/3.0) * fmaxf(delta_lambda, 0.): both calls return float, so the
    // reference multiplies in float (actions_gpu.cu:728-729)
    const float inc = sqrtf((float)(2.0 / 3.0)) * fmaxf((float)delta_lambda, 0.f);
    double eps_pl_new = eps_pl + (double)inc;
    double eps_pl_dot_new = (double)inc / dt;
    double eps_old = eps_pl;
    eps_pl = eps_pl_new;
    eps_pl_dot = eps_pl_dot_new;
    S.x = Sxx - Sxx / norm_Strial * delta_lambda * 2. * mu;
    S.z = Syy - Syy / norm_Strial * delta_lambda * 2. * mu;
    S.w = Szz - Szz / norm_Strial * delta_lambda * 2. * mu;
    S.y = Sxy - Sxy / norm_Strial * delta_lambda * 2. * mu;
    if (K.c.trml_wp.tq != 0.) {
        double delta_eps_pl = eps_pl_new - eps_old;
        double sY = kF32Yield ? sigma_yield_tc_f32(jc, eps_pl_new, eps_pl_dot_new, term_c)
                              : sigma_yield_tc(jc, eps_pl_new, eps_pl_dot_new, term_c);
        T += K.c.trml_wp.tq / (K.c.trml_wp.cp * rho) * delta_eps_pl * sY;
    }
    if (T > jc.Tmelt) {
        T = jc.Tmelt;
        blanked = 1.;
        st |= SPH_STATUS_MELT_BLANKED;
    }
    return st;
}

// ---- actions_gpu.cu:345-420 do_material_fric_heat_gen_FEM_v21 (one particle) --
// WEAR_NODE_SHIFT statistics are not part of the path.  Returns status bits.
// A segment id outside [0, n_seg) (the reference only ever stores -1 or a
// valid id) is treated like -1, so caller-uploaded data cannot index out of range.
__device__ __forceinline__ uint32_t fric_heat_one(const KConsts &K, double dt, const double *vel_tool, double2 vel,
                                                  double2 ft, double2 nrm, double2 fc, double rho, double eps_pl,
                                                  int seg, int n_seg, double &T, double &blanked,
                                                  double *__restrict__ fric_heat, const WearAcc &wear) {
    if (blanked == 1.) return 0u;
    if (eps_pl > 20.) return 0u;
    double f_fric_mag = sqrtf_d(ft.x * ft.x + ft.y * ft.y);
    if (seg < 0 || seg >= n_seg) return 0u;
    const double partition_wp = K.c.tool.beta;
    double vdx = vel.x - vel_tool[0], vdy = vel.y - vel_tool[1];
    double vdn = vdx * nrm.x + vdy * nrm.y;
    double vrx = vdx - vdn * nrm.x, vry = vdy - vdn * nrm.y;
    double v_rel_mag = sqrtf_d(vrx * vrx + vry * vry);
    double value = K.c.tool.eta * f_fric_mag * v_rel_mag;
    if (isnan(v_rel_mag)) {
        blanked = 1.;
        return SPH_STATUS_FRIC_NAN;
    }
    if (v_rel_mag > 0.03) return 0u;
    double T_buffer = T + value * (1 - partition_wp) * dt / K.c.trml_wp.cp / K.c.phys.mass;
    if (T_buffer > 1550.) {
        T = 1550.;
        return 0u;
    }
    T = T_buffer;
    atomicAdd(fric_heat + seg, value * partition_wp);
    if (wear.pp) {   // WEAR_NODE_SHIFT statistics (actions_gpu.cu:401-419)
        const int4 mk = wear.marks[seg];
        const double T_seg = 0.5 * (wear.T_nodes[mk.z] + wear.T_nodes[mk.w]);
        const double vel_tool_norm = sqrt(vel_tool[0] * vel_tool[0] + vel_tool[1] * vel_tool[1]);
        if (v_rel_mag > 0.008) return 0u;
        if (v_rel_mag > vel_tool_norm * 8.0 && fabs(nrm.y) > 0.5) return 0u;   // around the flank face
        const double f_normal = sqrtf_d(fc.x * fc.x + fc.y * fc.y);
        const double length = sqrtf_d(K.c.tool.slave_mass / rho);
        const double pressure_trial = f_normal / length;
        atomicAdd(&wear.pp[seg].x, 1.);
        atomicAdd(&wear.pp[seg].y, pressure_trial);
        atomicAdd(&wear.pp[seg].z, v_rel_mag);
        atomicAdd(&wear.pp[seg].w, T_seg);
        atomicAdd(wear.sf + seg, f_fric_mag / length);
    }
    return 0u;
}

// ---- actions_gpu.cu:222-232 do_material_eos ----------------------------------
__device__ __forceinline__ double eos_one(const KConsts &K, double rho) {
    double c0 = sqrtf_d(K.c.phys.K / K.c.phys.rho0);
    return c0 * c0 * (rho - K.c.phys.rho0);
}

// ---- actions_gpu.cu:234-278 do_corrector_artificial_stress (+ stress_angle :45-49)
__device__ __forceinline__ dbl4 artificial_stress_one(const KConsts &K, double rho, double p, dbl4 S) {
    double eps = K.c.corr.stresseps;
    double sxx = S.x - p, sxy = S.y, syy = S.z - p;
    double rhoi21 = 1. / (rho * rho);
    double numer = 2. * sxy;
    double denom = sxx - syy + 0.;
    double theta = 0.5 * (double)sph_atan2f((float)numer, (float)denom);
    double cos_theta = (double)sph_cosf((float)theta);
    double sin_theta = (double)sph_sinf((float)theta);
    double cos_theta2 = cos_theta * cos_theta;
    double sin_theta2 = sin_theta * sin_theta;
    double rot_sxx = cos_theta2 * sxx + 2.0 * cos_theta * sin_theta * sxy + sin_theta2 * syy;
    double rot_syy = sin_theta2 * sxx - 2.0 * cos_theta * sin_theta * sxy + cos_theta2 * syy;
    double rot_rxx = 0., rot_ryy = 0.;
    if (rot_sxx > 0) rot_rxx = -eps * rot_sxx * rhoi21;
    if (rot_syy > 0) rot_ryy = -eps * rot_syy * rhoi21;
    return mk4(cos_theta2 * rot_rxx + sin_theta2 * rot_ryy, cos_theta * sin_theta * (rot_rxx - rot_ryy),
                        sin_theta2 * rot_rxx + cos_theta2 * rot_ryy, 0.);
}

// ---- actions_gpu.cu:280-314 do_material_stress_rate_jaumann -------------------
// S_t = 2G (epsdot - tr/3 I) + Omega S + S Omega^T (Belytschko 3.7.9); the GLM
// column-major products reduce to these element formulas.
__device__ __forceinline__ dbl4 jaumann_one(const KConsts &K, dbl4 vd, dbl4 S) {
    double G = K.c.phys.G;
    double vx_x = vd.x, vx_y = vd.y, vy_x = vd.z, vy_y = vd.w;
    double e01 = 0.5 * (vx_y + vy_x);
    double om10 = 0.5 * (vx_y - vy_x);
    double om01 = 0.5 * (vy_x - vx_y);
    double tr = vx_x + vy_y + 0.;
    double s = (1. / 3.) * tr;
    double twoG = 2. * G;
    dbl4 r;
    r.x = (twoG * (vx_x - s) + om10 * S.y) + S.y * om10;
    r.y = (twoG * (e01 - 0.) + om01 * S.x) + S.z * om10;
    r.z = (twoG * (vy_y - s) + om01 * S.y) + S.y * om01;
    r.w = (twoG * (0. - s) + 0.) + 0.;
    return r;
}

// ============================================================================
// FP32 forms used by SPH_PREC_FP32K.  Same formulas as above in single
// precision; only the return-mapping residual is evaluated in FP64.
// ============================================================================

// actions_gpu.cu:234-278 in FP32
__device__ __forceinline__ float4 artificial_stress_f32(float stresseps, float rho, float p, float4 S) {
    float sxx = S.x - p, sxy = S.y, syy = S.z - p;
    float rhoi21 = 1.f / (rho * rho);
    float theta = 0.5f * atan2f(2.f * sxy, sxx - syy);
    float cs, sn;
    sincosf(theta, &sn, &cs);
    float cs2 = cs * cs, sn2 = sn * sn;
    float rot_sxx = cs2 * sxx + 2.f * cs * sn * sxy + sn2 * syy;
    float rot_syy = sn2 * sxx - 2.f * cs * sn * sxy + cs2 * syy;
    float rxx = rot_sxx > 0.f ? -stresseps * rot_sxx * rhoi21 : 0.f;
    float ryy = rot_syy > 0.f ? -stresseps * rot_syy * rhoi21 : 0.f;
    return make_float4(cs2 * rxx + sn2 * ryy, cs * sn * (rxx - ryy), sn2 * rxx + cs2 * ryy, 0.f);
}

// actions_gpu.cu:280-314 in FP32
__device__ __forceinline__ float4 jaumann_f32(float G, float4 vd, float4 S) {
    float om10 = 0.5f * (vd.y - vd.z);
    float om01 = -om10;
    float e01 = 0.5f * (vd.y + vd.z);
    float s = (1.f / 3.f) * (vd.x + vd.w);
    float twoG = 2.f * G;
    return make_float4(twoG * (vd.x - s) + 2.f * om10 * S.y, twoG * e01 + om01 * S.x + S.z * om10,
                       twoG * (vd.w - s) + 2.f * om01 * S.y, -twoG * s);
}

__device__ __forceinline__ float jc_term_c_f32(const JcF32 &j, float T) {
    float theta = fminf((T - j.Tref) * j.inv_dT, 1.f);
    return 1.f - powf(theta, j.m);
}

__device__ __forceinline__ float sigma_yield_f32(const JcF32 &j, float eps, float epsd, float term_c) {
    float eps_dot = epsd * j.inv_epsdot_ref;
    float term_b = (eps_dot > 1.f) ? 1.f + j.C * logf(eps_dot) : powf(1.f + eps_dot, j.C);
    return (j.A + j.B * powf(eps, j.n)) * term_b * term_c;
}

// Trial state of the FP32 return mapping (actions_gpu.cu:689-720): deviatoric
// norm, von Mises stress of the Cauchy stress S - p I, thermal softening term
// and yield stress at the state before the step.  Returns true if yielding.
struct JcTrial {
    float norm, svm, term_c;
};

__device__ __forceinline__ bool jc_trial_f32(const JcF32 &j, const float4 &S, float p, float eps_pl, float eps_pl_dot,
                                             float T, JcTrial &tr) {
    tr.norm = sqrtf(S.x * S.x + S.z * S.z + S.w * S.w + 2.f * S.y * S.y);
    float cxx = S.x - p, cyy = S.z - p, czz = S.w - p, cxy = S.y;
    tr.svm = sqrtf((cxx * cxx + cyy * cyy + czz * czz) - cxx * cyy - cxx * czz - cyy * czz + 3.f * cxy * cxy);
    tr.term_c = jc_term_c_f32(j, T);
    float sY = sigma_yield_f32(j, eps_pl, eps_pl_dot, tr.term_c);
    return !(tr.svm < sY);
}

// Radial return from a yielding trial state (actions_gpu.cu:720-754,
// plasticity.cuh:117-162) in FP32 with the secant residual
// g(dl) = |S_trial| - 2 mu dl - sqrt(2/3) sigma_Y in FP64, started from dl_init.
// The stopping rule (|dl - dl_old| < 1e-6, at most 101 iterations) is the
// reference's, so any start converges to the same tolerance.
__device__ __forceinline__ uint32_t jc_return_f32(const KConsts &K, const JcF32 &j, float dt, float inv_dt, float4 &S,
                                                  float rho, float &eps_pl, float &eps_pl_dot, float &T, bool &blanked,
                                                  int *iters_out, const JcTrial &tr, float dl_init) {
    const float mu = K.f.G;
    const float s23 = 0.816496580927726f;   // sqrt(2/3)
    const double norm_d = (double)tr.norm, two_mu = 2.0 * K.c.phys.G, s23d = 0.816496580927726;
    auto residual = [&](float dl) {   // FP64 residual
        float dlp = fmaxf(dl, 0.f);
        float sy = sigma_yield_f32(j, eps_pl + s23 * dlp, s23 * dlp * inv_dt, tr.term_c);
        return norm_d - two_mu * (double)dl - s23d * (double)sy;
    };
    float dl = dl_init, dl_old;
    int iter = 0;
    uint32_t st = 0;
    while (true) {
        double g = residual(dl);
        float dl1 = dl * 1.01f;
        double g1 = residual(dl1);
        float slope = (float)(g - g1) / (dl - dl1);
        dl_old = dl;
        dl = dl - (float)g / slope;
        if (dl < 0.f) dl = -0.1f * dl;
        if (fabsf(dl - dl_old) < 1e-6f) { iter++; break; }
        if (iter > K.secant_cap) { st |= SPH_STATUS_SECANT_MAXITER; iter++; break; }
        iter++;
    }
    *iters_out = iter;
    jc_log_record(K, tr.svm, eps_pl, eps_pl_dot, T, tr.norm, dl, iter, dt);
    jc_count(K, iter);
    float dlp = fmaxf(dl, 0.f);
    float eps_new = eps_pl + s23 * dlp;
    float epsd_new = s23 * dlp * inv_dt;
    float f = dl * 2.f * mu / tr.norm;
    S.x -= S.x * f;
    S.y -= S.y * f;
    S.z -= S.z * f;
    S.w -= S.w * f;
    if (K.c.trml_wp.tq != 0.) {
        float sy_new = sigma_yield_f32(j, eps_new, epsd_new, tr.term_c);
        T += K.f.tq_over_cp / rho * (eps_new - eps_pl) * sy_new;
    }
    eps_pl = eps_new;
    eps_pl_dot = epsd_new;
    if (T > j.Tmelt) {
        T = j.Tmelt;
        blanked = true;
        st |= SPH_STATUS_MELT_BLANKED;
    }
    return st;
}

// The reference's start dl0 = max(eps_pl_dot dt sqrt(2/3), 1e-8) (actions_gpu.cu:724).
__device__ __forceinline__ float jc_default_start(float eps_pl_dot, float dt) {
    return fmaxf(eps_pl_dot * dt * 0.816496580927726f, 1e-8f);
}

// actions_gpu.cu:689-754 + plasticity.cuh:117-162 in FP32 (trial + return).
__device__ __forceinline__ uint32_t plasticity_f32(const KConsts &K, const JcF32 &j, float dt, float inv_dt, float4 &S,
                                                   float p, float rho, float &eps_pl, float &eps_pl_dot, float &T,
                                                   bool &blanked, int *iters_out) {
    JcTrial tr;
    *iters_out = 0;
    if (!jc_trial_f32(j, S, p, eps_pl, eps_pl_dot, T, tr)) {
        eps_pl_dot = 0.f;
        return 0u;
    }
    return jc_return_f32(K, j, dt, inv_dt, S, rho, eps_pl, eps_pl_dot, T, blanked, iters_out, tr,
                         jc_default_start(eps_pl_dot, dt));
}

// ---- actions_gpu.cu:33-43 find_max / find_min -----------------------------------
__device__ __forceinline__ double find_max(double a, double b) { return (a >= b) ? a : b; }
__device__ __forceinline__ double find_min(double a, double b) { return (a >= b) ? b : a; }

// ---- actions_gpu.cu:51-63 on_segment_mesh -----------------------------------------
__device__ __forceinline__ int on_segment_mesh(double2 left, double2 right, double2 point) {
    if (point.y <= fmaxf_d(left.y, right.y) && point.y >= fminf_d(left.y, right.y)) {
        if (left.x == right.x && point.x < left.x) return 1;
        if (fabs(left.y - right.y) != 0) {
            double x_on_seg = right.x + (left.x - right.x) / (left.y - right.y) * (point.y - right.y);
            if (x_on_seg > point.x && x_on_seg != left.x) return 1;
        } else {
            if (point.x <= fmax(left.x, right.x)) return 1;
        }
    }
    return 0;
}

// ---- actions_gpu.cu:83-93 inside_judgement (ray casting towards +x) ------------
__device__ __forceinline__ int inside_judgement(double2 qp, const double2 *__restrict__ left,
                                                const double2 *__restrict__ right, int num_seg) {
    int intersections = 0;
    for (int i = 0; i < num_seg; i++) intersections += on_segment_mesh(__ldg(left + i), __ldg(right + i), qp);
    return (intersections % 2 == 0) ? 0 : 1;
}

// ---- actions_gpu.cu:139-220 find_shortest_distance_v1 ------------------------------
// The branch for no segment within limit_value (:182-219): the nearest right end
// point, its normal averaged with the next segment's.  seg: the first loop's
// result, kept when no end point is nearer than FLT_MAX (as the reference).
__device__ __forceinline__ int shortest_distance_fallback(double2 qp, double &dN, double2 &n_re,
                                                          const double2 *__restrict__ left,
                                                          const double2 *__restrict__ right,
                                                          const double2 *__restrict__ n, int num_seg, int seg) {
    double depth = FLT_MAX;
    for (int i = 0; i < num_seg; i++) {
        double2 Rr = __ldg(right + i);
        double d_trial = sqrtf_d((qp.x - Rr.x) * (qp.x - Rr.x) + (qp.y - Rr.y) * (qp.y - Rr.y));
        if (d_trial < depth) { depth = d_trial; seg = i; }
    }
    if (seg == -1) return seg;
    double2 ns = __ldg(n + seg);
    double2 rs = __ldg(right + seg);
    double nsx = ns.x, nsy = ns.y;
    for (int j = 0; j < num_seg; j++) {
        double2 Lj = __ldg(left + j);
        if (Lj.y == rs.y && Lj.x == rs.x) {
            double2 nj = __ldg(n + j);
            nsx = (nj.x + ns.x) / 2.;
            nsy = (nj.y + ns.y) / 2.;
            break;
        }
    }
    double n_length = sqrtf_d(nsx * nsx + nsy * nsy);
    n_re = make_double2(-nsx / n_length, -nsy / n_length);
    dN = -1.0 * depth;
    return seg;
}

__device__ __forceinline__ int find_shortest_distance_v1(double2 qp, double &dN, double2 &n_re,
                                                         const double2 *__restrict__ left,
                                                         const double2 *__restrict__ right,
                                                         const double2 *__restrict__ n, int num_seg) {
    int seg = -1;
    double depth = FLT_MAX;
    const double limit_value = 2.5e-4;
    for (int i = 0; i < num_seg; i++) {
        double2 L = __ldg(left + i), Rr = __ldg(right + i);
        double ymax = find_max(L.y, Rr.y), ymin = find_min(L.y, Rr.y);
        double xmax = find_max(L.x, Rr.x), xmin = find_min(L.x, Rr.x);
        if (qp.x > xmin - 0.0008 && qp.x < xmax + 0.0008 && qp.y > ymin - 0.0008 && qp.y < ymax + 0.0008) {
            double2 ni = __ldg(n + i);
            double d = (qp.x - L.x) * ni.x + (qp.y - L.y) * ni.y;
            if (d >= 0. && d < depth) {
                double intersec_x = qp.x - d * ni.x;
                double intersec_y = qp.y - d * ni.y;
                if (intersec_y <= ymax && intersec_y >= ymin && intersec_x <= xmax && intersec_x >= xmin) {
                    depth = d;
                    seg = i;
                }
            }
        }
    }
    if (seg != -1 && depth <= limit_value) {
        double2 ns = __ldg(n + seg);
        n_re = make_double2(-ns.x, -ns.y);
        dN = -depth;
        return seg;
    }
    return shortest_distance_fallback(qp, dN, n_re, left, right, n, num_seg, seg);
}

}  // namespace sphfem
