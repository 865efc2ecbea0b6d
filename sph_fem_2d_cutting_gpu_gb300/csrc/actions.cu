// actions.cu -- per-particle kernels of the step (actions_gpu.cu, leap_frog.cu):
// the staged form (one launch per reference call, same order and arrays) and
// the fused contact / boundary-condition / invalidate kernel of the step.
#include "tail.cuh"

namespace sphfem {

#define PARTICLE_LOOP_HEAD                                \
    const int i = blockIdx.x * blockDim.x + threadIdx.x; \
    if (i >= N) return;

// ---- leap_frog.cu:25-37 init --------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_init(int N, SortedFields A, StepScratch W) {
    PARTICLE_LOOP_HEAD
    if (A.blanked[i] == 1.) return;
    W.pos_init[i] = A.pos[i];
    W.vel_init[i] = A.vel[i];
    W.S_init[i] = A.S[i];
    W.rho_init[i] = A.rho[i];
    W.T_init[i] = A.T[i];
}

// ---- leap_frog.cu:45-96 predict (fac 0.5) / correct (fac 1) --------------------------------
__global__ void __launch_bounds__(kBlock) k_predict_correct(int N, SortedFields A, StepScratch W, double fdt) {
    PARTICLE_LOOP_HEAD
    if (A.blanked[i] == 1.) return;
    double2 p0 = W.pos_init[i], pt = A.pos_t[i], v0 = W.vel_init[i], vt = A.vel_t[i];
    A.pos[i] = make_double2(p0.x + fdt * pt.x, p0.y + fdt * pt.y);
    A.vel[i] = make_double2(v0.x + fdt * vt.x, v0.y + fdt * vt.y);
    dbl4 S0 = W.S_init[i], St = A.S_t[i];
    A.S[i] = mk4(S0.x + fdt * St.x, S0.y + fdt * St.y, S0.z + fdt * St.z, S0.w + fdt * St.w);
    A.rho[i] = W.rho_init[i] + fdt * A.rho_t[i];
    A.T[i] = W.T_init[i] + fdt * A.T_t[i];
}

// ---- actions_gpu.cu:222-232 do_material_eos ------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_eos(int N, KConsts K, SortedFields A, FixedFields F) {
    PARTICLE_LOOP_HEAD
    if (A.tool_particle[i] != 0.) return;
    F.p[i] = eos_one(K, A.rho[i]);
}

// ---- actions_gpu.cu:234-278 do_corrector_artificial_stress ---------------------------------
__global__ void __launch_bounds__(kBlock) k_artificial_stress(int N, KConsts K, SortedFields A, FixedFields F) {
    PARTICLE_LOOP_HEAD
    if (A.tool_particle[i] != 0.) return;
    F.R[i] = artificial_stress_one(K, A.rho[i], F.p[i], A.S[i]);
}

// ---- actions_gpu.cu:280-314 do_material_stress_rate_jaumann --------------------------------
__global__ void __launch_bounds__(kBlock) k_jaumann(int N, KConsts K, SortedFields A, FixedFields F) {
    PARTICLE_LOOP_HEAD
    if (A.tool_particle[i] == 1.) return;
    A.S_t[i] = jaumann_one(K, F.v_der[i], A.S[i]);
}

// ---- actions_gpu.cu:626-639 do_contmech_continuity ------------------------------------------
__global__ void __launch_bounds__(kBlock) k_continuity(int N, SortedFields A, FixedFields F) {
    PARTICLE_LOOP_HEAD
    if (A.tool_particle[i] != 0.) return;
    dbl4 vd = F.v_der[i];
    A.rho_t[i] = -A.rho[i] * (vd.x + vd.w);
}

// ---- actions_gpu.cu:641-671 do_contmech_momentum --------------------------------------------
__global__ void __launch_bounds__(kBlock) k_momentum(int N, KConsts K, SortedFields A, FixedFields F) {
    PARTICLE_LOOP_HEAD
    if (A.tool_particle[i] != 0.) return;
    const double mass = K.c.phys.mass;
    dbl4 sd = F.S_der[i];
    double2 fc = A.fc[i], ft = A.ft[i], vt = A.vel_t[i];
    vt.x += sd.x + sd.y + fc.x / mass + ft.x / mass;
    vt.y += sd.z + sd.w + fc.y / mass + ft.y / mass;
    A.vel_t[i] = vt;
}

// ---- actions_gpu.cu:673-687 do_contmech_advection -------------------------------------------
__global__ void __launch_bounds__(kBlock) k_advection(int N, SortedFields A) {
    PARTICLE_LOOP_HEAD
    if (A.tool_particle[i] != 0.) return;
    double2 v = A.vel[i], pt = A.pos_t[i];
    A.pos_t[i] = make_double2(pt.x + v.x, pt.y + v.y);
}

// ---- actions_gpu.cu:689-754 do_plasticity_johnson_cook ---------------------------------------
__global__ void __launch_bounds__(kBlock) k_plasticity(int N, KConsts K, SortedFields A, FixedFields F,
                                                       int32_t *__restrict__ secant_iters, uint32_t *status) {
    PARTICLE_LOOP_HEAD
    if (A.tool_particle[i] != 0.) return;
    if (A.blanked[i] == 1.) return;
    dbl4 S = A.S[i];
    double eps_pl = A.eps_pl[i], eps_pl_dot = A.eps_pl_dot[i], T = A.T[i], blanked = 0.;
    int it = 0;
    uint32_t st = (K.precision == SPH_PREC_FP32K)
                      ? plasticity_one<true>(K, K.dt, S, F.p[i], A.rho[i], eps_pl, eps_pl_dot, T, blanked, &it)
                      : plasticity_one<false>(K, K.dt, S, F.p[i], A.rho[i], eps_pl, eps_pl_dot, T, blanked, &it);
    if (secant_iters) secant_iters[i] = it;
    A.S[i] = S;
    A.eps_pl[i] = eps_pl;
    A.eps_pl_dot[i] = eps_pl_dot;
    A.T[i] = T;
    if (blanked == 1.) A.blanked[i] = 1.;
    if (st) set_status(status, st);
}

// ---- actions_gpu.cu:345-420 do_material_fric_heat_gen_FEM_v21 --------------------------------
__global__ void __launch_bounds__(kBlock) k_fric_heat(int N, KConsts K, SortedFields A, SegDev seg,
                                                      const ToolDev *__restrict__ tool, uint32_t *status) {
    PARTICLE_LOOP_HEAD
    double T = A.T[i], blanked = A.blanked[i];
    uint32_t st = fric_heat_one(K, K.dt, tool->vel, A.vel[i], A.ft[i], A.n[i], A.fc[i], A.rho[i], A.eps_pl[i], A.on_seg[i],
                                seg.n, T, blanked, seg.fric_heat, seg.wear);
    if (T != A.T[i]) A.T[i] = T;
    if (blanked != A.blanked[i]) A.blanked[i] = blanked;
    if (st) set_status(status, st);
}

// ---- y-bins of the interface segments (tail.cuh): one block per case -------------------------------
__global__ void __launch_bounds__(256) k_seg_bins(SegDev seg, ToolDev *tool) { seg_bins_block(blockIdx.x, seg, tool); }

__global__ void __launch_bounds__(kBlock) k_contact_s1(int N, KConsts K, SortedFields A, SegDev seg,
                                                       const ToolDev *__restrict__ tool, uint32_t *status) {
    PARTICLE_LOOP_HEAD
    if (A.blanked[i] == 1.) return;
    double2 fc = A.fc[i], ft = A.ft[i], nrm = A.n[i];
    int on = A.on_seg[i];
    double blanked = 0.;
    uint32_t st = contact_s1_one(K, K.dt, seg, *tool, A.pos[i], A.vel[i], fc, ft, nrm, on, blanked);
    A.fc[i] = fc; A.ft[i] = ft; A.n[i] = nrm; A.on_seg[i] = on;
    if (blanked == 1.) A.blanked[i] = 1.;
    if (st) set_status(status, st);
}

__global__ void __launch_bounds__(kBlock) k_contact_s2(int N, KConsts K, SortedFields A, SegDev seg,
                                                       const double *__restrict__ T_nodes) {
    PARTICLE_LOOP_HEAD
    if (A.blanked[i] == 1.) return;
    int on = A.on_seg[i];
    if (on < 0 || on >= seg.n) return;
    double T = A.T[i];
    contact_s2_one(K, K.dt, seg, T_nodes, on, A.rho[i], T);
    A.T[i] = T;
}

// ---- actions_gpu.cu:765-781 do_boundary_conditions ------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_bc(int N, SortedFields A) {
    PARTICLE_LOOP_HEAD
    if (A.tool_particle[i] != 0.) return;
    if (A.fixed[i] != 0.) {
        A.vel[i] = make_double2(0., 0.);
        A.fc[i] = make_double2(0., 0.);
        A.pos_t[i] = make_double2(0., 0.);
        A.vel_t[i] = make_double2(0., 0.);
    }
}

// ---- actions_gpu.cu:756-763 do_boundary_conditions_thermal ------------------------------------------
__global__ void __launch_bounds__(kBlock) k_bc_thermal(int N, KConsts K, SortedFields A) {
    PARTICLE_LOOP_HEAD
    if (A.fixed[i] == 1.) A.T[i] = K.c.trml_wp.T_init;
}

// ---- actions_gpu.cu:787-824 do_invalidate ----------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_invalidate(int N, SortedFields A, uint32_t *status) {
    PARTICLE_LOOP_HEAD
    if (A.blanked[i] == 1.) return;
    if (invalid_rates(A.pos_t[i], A.vel_t[i], A.S_t[i], A.rho_t[i], A.T_t[i])) {
        A.blanked[i] = 1.;
        set_status(status, SPH_STATUS_NAN_BLANKED);
    }
}

// ---- rigid (SPH-mode) tool: tool_gpu.cu, actions_gpu.cu:316-343 ----------------------------------
// tool::update_tool (tool.cpp:202-212) on the device copy of the tool.
__global__ void k_rigid_move(sph_rigid_tool *t, double dt) {
    if (threadIdx.x == 0 && blockIdx.x == 0) rigid_move(*t, dt);
}

// tool_gpu.cu:205-216 update_tool_particles
__global__ void __launch_bounds__(kBlock) k_rigid_move_particles(int N, SortedFields A,
                                                                 const sph_rigid_tool *__restrict__ t, double dt) {
    PARTICLE_LOOP_HEAD
    if (!flag_nonzero(A.tool_particle[i])) return;
    double2 pos = A.pos[i];
    pos.x += dt * t->vel[0];
    pos.y += dt * t->vel[1];
    A.pos[i] = pos;
}

// tool_gpu.cu:146-202 do_compute_contact_forces (no blanked test, as there)
__global__ void __launch_bounds__(kBlock) k_contact_rigid(int N, KConsts K, SortedFields A, double dt) {
    PARTICLE_LOOP_HEAD
    if (flag_nonzero(A.tool_particle[i])) return;
    double2 fc, ft = A.ft[i], nrm;
    rigid_contact_one(K, *K.rigid, dt, A.pos[i], A.vel[i], fc, ft, nrm);
    A.fc[i] = fc;
    A.ft[i] = ft;
    A.n[i] = nrm;
}

// actions_gpu.cu:316-343 do_material_fric_heat_gen (no blanked test, as there)
__global__ void __launch_bounds__(kBlock) k_fric_heat_rigid(int N, KConsts K, SortedFields A, double dt) {
    PARTICLE_LOOP_HEAD
    if (flag_nonzero(A.tool_particle[i])) return;
    double T = A.T[i];
    rigid_fric_heat_one(K, dt, K.rigid->vel, A.vel[i], A.ft[i], A.n[i], T);
    if (T != A.T[i]) A.T[i] = T;
}

// ---- the FEM tool's contact of the fused step and the fused tail (tail.cuh) ---------------------------
template <class SF>
__global__ void __launch_bounds__(kBlock) k_contact_fem(int N, KConsts K, SF A, SegDev seg,
                                                        const ToolDev *__restrict__ tool,
                                                        const double *__restrict__ T_nodes, uint32_t *status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg.geo && seg.bin_xkey && (blockDim.x & 31u) == 0) {   // every lane takes part in the warp searches
        contact_fem_warp(i, N, K, A, seg, tool, T_nodes, status);
        return;
    }
    if (i >= N) return;
    contact_fem_one(i, K, A, seg, tool, T_nodes, status);
}

template <int kMode, bool kNextHash, class SF>
__global__ void __launch_bounds__(kBlock) k_step_tail(int N, KConsts K, SF A, SegDev seg,
                                                      const ToolDev *__restrict__ tool,
                                                      const double *__restrict__ T_nodes, SortScratch X,
                                                      uint32_t *status) {
    PARTICLE_LOOP_HEAD
    step_tail_one<kMode, kNextHash>(i, K, A, X, status);
}

// ---- measurement hooks: output.cu:41-49 report_force (sum of fc + ft); peak T ----------------------
__global__ void __launch_bounds__(kBlock) k_reduce_force_T(int N, SortedFields A, double *__restrict__ out) {
    __shared__ double sx[kBlock], sy[kBlock], sm[kBlock];
    double fx = 0., fy = 0., tm = -1e300;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        double2 fc = A.fc[i], ft = A.ft[i];
        fx += fc.x + ft.x;
        fy += fc.y + ft.y;
        if (A.blanked[i] != 1.) tm = fmax(tm, A.T[i]);
    }
    sx[threadIdx.x] = fx; sy[threadIdx.x] = fy; sm[threadIdx.x] = tm;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sx[threadIdx.x] += sx[threadIdx.x + o];
            sy[threadIdx.x] += sy[threadIdx.x + o];
            sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[3 * blockIdx.x + 0] = sx[0];
        out[3 * blockIdx.x + 1] = sy[0];
        out[3 * blockIdx.x + 2] = sm[0];
    }
}

// Per-case sums of fc + ft and max T of non-blanked particles, one block per
// case over its contiguous particle range.  With `offsets` (the state is in
// cell order; cases own disjoint column ranges, so whole cases are contiguous)
// case k spans cells [cell_bound[k], cell_bound[k+1]); otherwise particles
// [part_bound[k], part_bound[k+1]) (the concatenation order of the upload).
__global__ void __launch_bounds__(kBlock) k_reduce_cases(SortedFields A, const int32_t *__restrict__ offsets,
                                                         const int32_t *__restrict__ cell_bound,
                                                         const int32_t *__restrict__ part_bound,
                                                         double *__restrict__ out) {
    __shared__ double sx[kBlock], sy[kBlock], sm[kBlock];
    const int k = blockIdx.x;
    const int b = offsets ? offsets[cell_bound[k]] : part_bound[k];
    const int e = offsets ? offsets[cell_bound[k + 1]] : part_bound[k + 1];
    double fx = 0., fy = 0., tm = -1e300;
    for (int i = b + threadIdx.x; i < e; i += blockDim.x) {
        double2 fc = A.fc[i], ft = A.ft[i];
        fx += fc.x + ft.x;
        fy += fc.y + ft.y;
        if (A.blanked[i] != 1.) tm = fmax(tm, A.T[i]);
    }
    sx[threadIdx.x] = fx; sy[threadIdx.x] = fy; sm[threadIdx.x] = tm;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sx[threadIdx.x] += sx[threadIdx.x + o];
            sy[threadIdx.x] += sy[threadIdx.x + o];
            sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[3 * k + 0] = sx[0];
        out[3 * k + 1] = sy[0];
        out[3 * k + 2] = sm[0];
    }
}

// tool_wear::eval_usui (tool_wear.cu:14-54) per particle, reduced per block:
// in-contact particles (|fc.x|, |fc.y|, |ft.x| or -- as the reference tests it --
// |fc.y| again nonzero) contribute K exp(alpha/T) p |v_r| with p = |fc| / (2 pi h)
// and v_r = v - v*n (component-wise product, as glm's vec2 * vec2).
// out[4 * block + 0..3] = min, max, sum, count.
__global__ void __launch_bounds__(kBlock) k_usui(int N, SortedFields A, double K_usui, double alpha, double vtx,
                                                 double vty, double *__restrict__ out) {
    __shared__ double smin[kBlock], smax[kBlock], ssum[kBlock], scnt[kBlock];
    double mn = 1.7976931348623157e308, mx = 0., sm = 0., cnt = 0.;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double2 fc = A.fc[i], ft = A.ft[i];
        if (!(fabs(fc.x) > 0. || fabs(fc.y) > 0. || fabs(ft.x) > 0. || fabs(fc.y) > 0.)) continue;
        const double2 v0 = A.vel[i], n = A.n[i];
        const double vx = v0.x - vtx, vy = v0.y - vty;
        const double rx = vx - vx * n.x, ry = vy - vy * n.y;
        const double vmag = sqrt(rx * rx + ry * ry);
        const double fmag = sqrt(fc.x * fc.x + fc.y * fc.y);
        const double p = fmag / (2. * A.h[i] * 3.14159265358979323846);
        const double w = K_usui * exp(alpha / A.T[i]) * p * vmag;
        mn = fmin(mn, w);
        mx = fmax(mx, w);
        sm += w;
        cnt += 1.;
    }
    smin[threadIdx.x] = mn; smax[threadIdx.x] = mx; ssum[threadIdx.x] = sm; scnt[threadIdx.x] = cnt;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
            ssum[threadIdx.x] += ssum[threadIdx.x + o];
            scnt[threadIdx.x] += scnt[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[4 * blockIdx.x + 0] = smin[0];
        out[4 * blockIdx.x + 1] = smax[0];
        out[4 * blockIdx.x + 2] = ssum[0];
        out[4 * blockIdx.x + 3] = scnt[0];
    }
}

// ---- host launchers --------------------------------------------------------------------------------
#define GRID div_up(N, kBlock), kBlock, 0, s

void launch_init(cudaStream_t s, int N, const SortedFields &A, const StepScratch &W) { k_init<<<GRID>>>(N, A, W); }
void launch_predict_correct(cudaStream_t s, int N, const SortedFields &A, const StepScratch &W, double fdt) {
    k_predict_correct<<<GRID>>>(N, A, W, fdt);
}
void launch_eos(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F) {
    k_eos<<<GRID>>>(N, K, A, F);
}
void launch_artificial_stress(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F) {
    k_artificial_stress<<<GRID>>>(N, K, A, F);
}
void launch_jaumann(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F) {
    k_jaumann<<<GRID>>>(N, K, A, F);
}
void launch_continuity(cudaStream_t s, int N, const SortedFields &A, const FixedFields &F) {
    k_continuity<<<GRID>>>(N, A, F);
}
void launch_momentum(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F) {
    k_momentum<<<GRID>>>(N, K, A, F);
}
void launch_advection(cudaStream_t s, int N, const SortedFields &A) { k_advection<<<GRID>>>(N, A); }
void launch_plasticity(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F,
                       const StepScratch &W) {
    k_plasticity<<<GRID>>>(N, K, A, F, W.secant_iters, W.status);
}
void launch_fric_heat(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const SegDev &seg,
                      const ToolDev *tool, uint32_t *status) {
    k_fric_heat<<<GRID>>>(N, K, A, seg, tool, status);
}
void launch_seg_bins(cudaStream_t s, int n_cases, const SegDev &seg, ToolDev *tool) {
    if (seg.bin_count) k_seg_bins<<<n_cases, 256, 0, s>>>(seg, tool);
}
void launch_contact(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const SegDev &seg,
                    ToolDev *tool, const double *T_nodes, uint32_t *status) {
    launch_seg_bins(s, 1, seg, tool);
    k_contact_s1<<<GRID>>>(N, K, A, seg, tool, status);
    k_contact_s2<<<GRID>>>(N, K, A, seg, T_nodes);
}
void launch_bc(cudaStream_t s, int N, const SortedFields &A) { k_bc<<<GRID>>>(N, A); }
void launch_bc_thermal(cudaStream_t s, int N, const KConsts &K, const SortedFields &A) {
    k_bc_thermal<<<GRID>>>(N, K, A);
}
void launch_invalidate(cudaStream_t s, int N, const SortedFields &A, uint32_t *status) {
    k_invalidate<<<GRID>>>(N, A, status);
}
template <class SF>
static void step_tail(cudaStream_t s, int N, const KConsts &K, const SF &A, const SegDev &seg, ToolDev *tool,
                      const double *T_nodes, const SortScratch &X, uint32_t *status, bool next_hash) {
    const int tb = fp64_block(N);   // the contact search is FP64 work: spread small systems over all SMs
    if (K.has_tool) launch_seg_bins(s, K.n_cases, seg, tool);
#undef GRID
#define GRID div_up(N, tb), tb, 0, s
    if (K.has_tool) {   // the contact pass, then the tail of a step without tool
        k_contact_fem<<<GRID>>>(N, K, A, seg, tool, T_nodes, status);
        if (next_hash) k_step_tail<0, true><<<GRID>>>(N, K, A, seg, tool, T_nodes, X, status);
        else k_step_tail<0, false><<<GRID>>>(N, K, A, seg, tool, T_nodes, X, status);
    } else if (K.rigid) {
        if (next_hash) k_step_tail<2, true><<<GRID>>>(N, K, A, seg, tool, T_nodes, X, status);
        else k_step_tail<2, false><<<GRID>>>(N, K, A, seg, tool, T_nodes, X, status);
    } else {
        if (next_hash) k_step_tail<0, true><<<GRID>>>(N, K, A, seg, tool, T_nodes, X, status);
        else k_step_tail<0, false><<<GRID>>>(N, K, A, seg, tool, T_nodes, X, status);
    }
}
void launch_step_tail(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const SegDev &seg,
                      ToolDev *tool, const double *T_nodes, const SortScratch &X, uint32_t *status,
                      bool next_hash) {
    step_tail(s, N, K, A, seg, tool, T_nodes, X, status, next_hash);
}
void launch_step_tail(cudaStream_t s, int N, const KConsts &K, const SortedFields32 &A, const SegDev &seg,
                      ToolDev *tool, const double *T_nodes, const SortScratch &X, uint32_t *status,
                      bool next_hash) {
    step_tail(s, N, K, A, seg, tool, T_nodes, X, status, next_hash);
}
#undef GRID
#define GRID div_up(N, kBlock), kBlock, 0, s
void launch_rigid_move(cudaStream_t s, sph_rigid_tool *t, double dt) { k_rigid_move<<<1, 32, 0, s>>>(t, dt); }
void launch_rigid_move_particles(cudaStream_t s, int N, const SortedFields &A, const sph_rigid_tool *t, double dt) {
    k_rigid_move_particles<<<GRID>>>(N, A, t, dt);
}
void launch_contact_rigid(cudaStream_t s, int N, const KConsts &K, const SortedFields &A) {
    k_contact_rigid<<<GRID>>>(N, K, A, K.dt);
}
void launch_fric_heat_rigid(cudaStream_t s, int N, const KConsts &K, const SortedFields &A) {
    k_fric_heat_rigid<<<GRID>>>(N, K, A, K.dt);
}
int reduce_blocks() { return 304; }
void launch_reduce_force_T(cudaStream_t s, int N, const SortedFields &A, double *out) {
    k_reduce_force_T<<<reduce_blocks(), kBlock, 0, s>>>(N, A, out);
}
void launch_usui(cudaStream_t s, int N, const SortedFields &A, double K_usui, double alpha, double vtx, double vty,
                 double *out) {
    k_usui<<<reduce_blocks(), kBlock, 0, s>>>(N, A, K_usui, alpha, vtx, vty, out);
}
void launch_reduce_cases(cudaStream_t s, int n_cases, const SortedFields &A, const int32_t *offsets,
                         const int32_t *cell_bound, const int32_t *part_bound, double *out) {
    k_reduce_cases<<<n_cases, kBlock, 0, s>>>(A, offsets, cell_bound, part_bound, out);
}

}  // namespace sphfem
