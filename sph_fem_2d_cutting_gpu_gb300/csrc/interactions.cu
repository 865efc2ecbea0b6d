// interactions.cu -- neighbour sums of do_interactions_monaghan
// (interactions_gpu.cu:143-379: velocity gradient, stress divergence with
// Gray-Monaghan artificial stress, Monaghan artificial viscosity, XSPH and
// Brookshaw heat conduction) on sm_103a.
//
// One thread per particle in sorted order.  Neighbours are visited column by
// column: the cells (ii, gj-R .. gj+R) of one grid column are consecutive
// keys, so their particles form one contiguous slot range [offsets[c0],
// offsets[c1+1]) -- the reference's visiting order (ii outer, jj inner,
// sorted order inside a cell) without per-cell bookkeeping.
//
// Out-of-support candidates are skipped: in the reference they run the full
// body with W = dW = 0 and add exact zeros (interactions_gpu.cu:230-337), so
// skipping them changes no sum.  Per-neighbour quotients that depend only on
// the neighbour ((S-p)/rho^2, mass/rho, sqrtf(K/rho)) come precomputed in the
// neighbour record; constant factors (mass, -eps*mass, 2*alpha) are applied
// once after the loop.  These reassociations change results by O(1e-16)
// relative.
//
// Fused mode adds, per particle, the rest of the particle chain up to the
// return mapping: do_material_stress_rate_jaumann, do_contmech_continuity /
// _momentum / _advection (actions_gpu.cu:280-314,626-687), correct
// (leap_frog.cu:71-96), do_material_fric_heat_gen_FEM_v21
// (actions_gpu.cu:345-420) and do_plasticity_johnson_cook
// (actions_gpu.cu:689-754).  Correct writes the start-of-step arrays in
// place (only this thread touches them); neighbours read the predicted state
// from the records, so there is no read/write race.
#include "interact32.cuh"

namespace sphfem {

struct Sums64 {
    double vd0, vd1, vd2, vd3;     // v_der
    double sd0, sd1, sd2, sd3;     // S_der / mass
    double vt0, vt1;               // vel_t / (-mass)
    double xt0, xt1;               // pos_t / (eps*mass)
    double tl;                     // T_lapl / 2
};

// ---- per-particle epilogue shared by both precisions (fused mode) ---------------------
// vd, sd (= S_der), vt (= vel_t from viscosity), xt (= pos_t from XSPH), T_t.
__device__ __forceinline__ void fused_epilogue(int k, const KConsts &K, const SortedFields &B, const FixedFields &F,
                                               const SegDev &seg, const ToolDev *__restrict__ tool,
                                               int32_t *__restrict__ secant_iters, uint32_t *status, bool is_tool,
                                               double2 vel_pred, double rho_pred, dbl4 vd, dbl4 sd,
                                               double2 vt, double2 xt, bool thermal, double T_t_new) {
    const ToolDev &tc = tool[case_of_hash(K, B.hash[k])];   // the particle's case (time step, tool)
    const double dt = tc.dt;
    const double mass = K.c.phys.mass;
    dbl4 S0 = B.S[k];
    dbl4 St = B.S_t[k];
    double2 pos_t, vel_t;
    double rho_t = B.rho_t[k];
    if (!is_tool) {
        const double hdt = 0.5 * dt;
        dbl4 Sp = mk4(S0.x + hdt * St.x, S0.y + hdt * St.y, S0.z + hdt * St.z, S0.w + hdt * St.w);
        St = jaumann_one(K, vd, Sp);                                  // actions_gpu.cu:280-314
        rho_t = -rho_pred * (vd.x + vd.w);                            // actions_gpu.cu:626-639
        double2 fc = B.fc[k], ft = B.ft[k];
        vel_t.x = vt.x + (((sd.x + sd.y) + fc.x / mass) + ft.x / mass);   // actions_gpu.cu:641-671
        vel_t.y = vt.y + (((sd.z + sd.w) + fc.y / mass) + ft.y / mass);
        pos_t.x = xt.x + vel_pred.x;                                  // actions_gpu.cu:673-687
        pos_t.y = xt.y + vel_pred.y;
    } else if (K.thermal_pse) {   // PSE build: tool particles leave the sums unwritten
        vel_t = B.vel_t[k];
        pos_t = B.pos_t[k];
    } else {
        vel_t = vt;
        pos_t = xt;
    }
    double T_t = thermal ? T_t_new : B.T_t[k];
    B.pos_t[k] = pos_t;
    B.vel_t[k] = vel_t;
    B.S_t[k] = St;
    B.rho_t[k] = rho_t;
    B.T_t[k] = T_t;
    // correct (leap_frog.cu:71-96)
    double2 pos = B.pos[k], vel = B.vel[k];
    pos.x = pos.x + dt * pos_t.x;
    pos.y = pos.y + dt * pos_t.y;
    vel.x = vel.x + dt * vel_t.x;
    vel.y = vel.y + dt * vel_t.y;
    dbl4 S = mk4(S0.x + dt * St.x, S0.y + dt * St.y, S0.z + dt * St.z, S0.w + dt * St.w);
    double rho = B.rho[k] + dt * rho_t;
    double T = B.T[k] + dt * T_t;
    B.pos[k] = pos;
    B.vel[k] = vel;
    B.rho[k] = rho;
    double blanked = 0.;
    uint32_t st = 0;
    // friction heat (actions_gpu.cu:345-420), tool runs only
    if (K.has_tool) st |= fric_heat_one(K, dt, tc.vel, vel, B.ft[k], B.n[k], B.fc[k], rho, B.eps_pl[k], B.on_seg[k],
                                        seg.n, T, blanked, seg.fric_heat, seg.wear);
    else if (K.rigid && !is_tool && K.c.trml_wp.eta != 0.)   // actions_gpu.cu:316-343
        rigid_fric_heat_one(K, dt, K.rigid->vel, vel, B.ft[k], B.n[k], T);
    // return mapping (actions_gpu.cu:689-754)
    if (K.c.plastic && !is_tool && blanked != 1.) {
        double eps_pl = B.eps_pl[k], eps_pl_dot = B.eps_pl_dot[k];
        int it = 0;
        if (K.precision == SPH_PREC_FP32K)
            st |= plasticity_one<true>(K, dt, S, F.p[k], rho, eps_pl, eps_pl_dot, T, blanked, &it);
        else
            st |= plasticity_one<false>(K, dt, S, F.p[k], rho, eps_pl, eps_pl_dot, T, blanked, &it);
        B.eps_pl[k] = eps_pl;
        B.eps_pl_dot[k] = eps_pl_dot;
        if (secant_iters) secant_iters[k] = it;
    }
    B.S[k] = S;
    B.T[k] = T;
    if (blanked == 1.) B.blanked[k] = 1.;
    if (st) set_status(status, st);
}

// ---- FP64 ---------------------------------------------------------------------------
template <bool kFused, int kB = kBlock>
__global__ void __launch_bounds__(kB) k_interact64(int N, KConsts K, const int32_t *__restrict__ offsets,
                                                       const dbl4 *__restrict__ rec, SortedFields B, FixedFields F,
                                                       SegDev seg, const ToolDev *__restrict__ tool,
                                                       int32_t *__restrict__ secant_iters, uint32_t *status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const dbl4 i3 = rec[4 * k + 3];
    const int fi = (int)__double_as_longlong(i3.w);
    if (fi & kFlagBlanked) {
        if (kFused) rigid_heat_blanked(k, K, B);
        return;
    }
    const bool tool_i = (fi & kFlagTool) != 0;
    const bool pse_tool = K.thermal_pse && tool_i;   // PSE build: tool particles return at once
    const dbl4 i0 = rec[4 * k + 0], i1 = rec[4 * k + 1], i2 = rec[4 * k + 2];
    const double xi = i0.x, yi = i0.y, vix = i0.z, viy = i0.w;
    const double sAi = i1.x, sBi = i1.y, sCi = i1.z, Rxxi = i1.w;
    const double Rxyi = i2.x, Ryyi = i2.y, hi = i2.z, rhoi = i2.w;
    const double ci = i3.x, Ti = i3.z;
    const double thermal_alpha = (!tool_i) ? K.c.trml_wp.alpha : K.c.trml_tool_sph.alpha;
    const bool thermal = thermal_alpha != 0. && !K.thermal_pse;   // Brookshaw build only
    const double h1 = 1 / hi;
    const double fourh2 = 4 * hi * hi;
    const double fac = kPiFac * h1 * h1;
    const double alpha = K.c.corr.alpha, beta = K.c.corr.beta, eta2 = K.eta2, inv_wdp = K.inv_wdeltap;

    Sums64 a = {};
    const int hash = B.hash[k];
    const sph_geom_constants &g = K.g;
    __shared__ int s_list[kChunk64][kB];
    int ii = 0, hi_i = 0, lo_j = 0, hi_j = 0, jc = 0, j1 = 0, ii0 = 0;
    bool done = true;
    if (hash >= 0 && hash < g.num_cell && !pse_tool) {
        const int gi = hash / g.ny, gj = hash - gi * g.ny, R = g.stencil;
        ii = ii0 = max(gi - R, 0);
        hi_i = min(gi + R + 1, g.nx);
        lo_j = max(gj - R, 0);
        hi_j = min(gj + R + 1, g.ny);
        jc = __ldg(offsets + ii * g.ny + lo_j);
        j1 = __ldg(offsets + ii * g.ny + hi_j);
        done = false;
    }
    // Pass 0 sums over the in-support neighbours; a stencil holding a record
    // marked non-finite repeats them over every active candidate with the
    // reference's zero weights outside the support (pass 1; see k_interact32).
    int marks = 0;   // OR of the flags of the stencil's candidates (blanked ones carry no mark)
    auto sweep = [&](auto all_tag) {
    constexpr bool all = decltype(all_tag)::value;
    while (!done) {
        // phase 1: collect the next in-support candidates (columns ii, cells lo_j..hi_j)
        int cnt = 0;
        while (cnt < kChunk64) {
            if (jc < j1) {
                const dbl4 n0 = rec[4 * jc + 0];
                const int fj = (int)__double_as_longlong(rec[4 * jc + 3].w);
                const double dx = xi - n0.x, dy = yi - n0.y;
                const double rr2 = dx * dx + dy * dy;
                if (!all) marks |= fj;
                if (all || (rr2 < fourh2 && rr2 >= 1e-8)) s_list[cnt++][threadIdx.x] = jc;
                jc++;
            } else {
                if (++ii >= hi_i) {
                    done = true;
                    break;
                }
                jc = __ldg(offsets + ii * g.ny + lo_j);
                j1 = __ldg(offsets + ii * g.ny + hi_j);
            }
        }
        // phase 2: pair body over the list, lanes in step
        for (int t = 0; t < cnt; t++) {
            const int j = s_list[t][threadIdx.x];
            {
                const dbl4 n0 = rec[4 * j + 0];
                const double dx = xi - n0.x, dy = yi - n0.y;
                const double rr2 = dx * dx + dy * dy;
                const dbl4 n3 = rec[4 * j + 3];
                const int fj = (int)__double_as_longlong(n3.w);
                if (fj & kFlagBlanked) continue;
                // cubic spline (kernels.cuh:25-65)
                const double rad = sqrtf_d(rr2);
                const double q = rad * h1;
                double val, der;
                if (q > 1) {
                    const double t = 2 - q, t2 = t * t;
                    val = 0.25 * t2 * t2 * t2;
                    der = -0.75 * t2 * h1 / rad;
                } else {
                    val = 1 - 1.5 * q * q * (1 - 0.5 * q);
                    der = -3.0 * q * (1 - 0.75 * q) * h1 / rad;
                }
                // pass 1: cubic_spline's zero weights outside the support (kernels.cuh:37-39)
                const bool zero_w = all && (rr2 >= fourh2 || rr2 < 1e-8);
                const double w = zero_w ? 0. : val * fac;
                const double dwf = zero_w ? 0. : der * fac;
                const double wx = dwf * dx, wy = dwf * dy;
                const double volj = n3.y;
                if (!tool_i && !(fj & kFlagTool)) {
                    const dbl4 n1 = rec[4 * j + 1];
                    const dbl4 n2 = rec[4 * j + 2];
                    const double dvx = n0.z - vix, dvy = n0.w - viy;
                    const double tx = wx * volj, ty = wy * volj;
                    a.vd0 += dvx * tx;
                    a.vd1 += dvx * ty;
                    a.vd2 += dvy * tx;
                    a.vd3 += dvy * ty;
                    double fab = w * inv_wdp;
                    fab *= fab;
                    fab *= fab;
                    const double ax = (sAi + n1.x) + fab * (Rxxi + n1.w);
                    const double ay = (sBi + n1.y) + fab * (Rxyi + n2.x);
                    const double az = (sCi + n1.z) + fab * (Ryyi + n2.y);
                    a.sd0 += ax * wx;
                    a.sd1 += ay * wy;
                    a.sd2 += ay * wx;
                    a.sd3 += az * wy;
                    const double vijposij = -(dvx * dx + dvy * dy);
                    const double irho = 1. / (0.5 * (rhoi + n2.w));
                    if (vijposij < 0.) {
                        const double cij = 0.5 * (ci + n3.x);
                        const double hij = 0.5 * (hi + n2.z);
                        const double muij = (hij * vijposij) / (rr2 + eta2 * hij * hij);
                        const double piij = (-alpha * cij * muij + beta * muij * muij) * irho;
                        a.vt0 += piij * wx;
                        a.vt1 += piij * wy;
                    }
                    const double wr = w * irho;
                    a.xt0 += wr * dvx;
                    a.xt1 += wr * dvy;
                }
                // Brookshaw, (e.dW)/r == dW/dr; the reference skips it at r <= 1e-8 (interactions_gpu.cu:328)
                if (thermal && (!zero_w || rr2 > 1e-16)) a.tl += volj * (Ti - n3.z) * dwf;
            }
        }
    }
    };
    sweep(std::false_type{});
    if (marks & kFlagNonFinite) {   // rare: the reference's full stencil with zero weights
        a = Sums64{};
        ii = ii0;
        jc = __ldg(offsets + ii * g.ny + lo_j);
        j1 = __ldg(offsets + ii * g.ny + hi_j);
        done = false;
        sweep(std::true_type{});
    }
    const double mass = K.c.phys.mass;
    const dbl4 vd = mk4(a.vd0, a.vd1, a.vd2, a.vd3);
    const dbl4 sd = mk4(mass * a.sd0, mass * a.sd1, mass * a.sd2, mass * a.sd3);
    const double2 vt = make_double2(-mass * a.vt0, -mass * a.vt1);
    const double xs = K.c.corr.xspheps * mass;
    const double2 xt = make_double2(xs * a.xt0, xs * a.xt1);
    const double T_t = thermal_alpha * (2.0 * a.tl);
    if (!kFused) {
        if (pse_tool) return;
        F.S_der[k] = sd;
        F.v_der[k] = vd;
        B.pos_t[k] = xt;
        B.vel_t[k] = vt;
        if (thermal) B.T_t[k] = T_t;
    } else {
        fused_epilogue(k, K, B, F, seg, tool, secant_iters, status, tool_i, make_double2(vix, viy), rhoi, vd, sd, vt,
                       xt, thermal, T_t);
    }
}

// Launch shapes of the fused FP32K neighbour-sum kernel: (threads per block,
// minimum resident blocks per SM, staged records: 0 = global loads, lanes per
// particle).  Variant 0 is the default: 6 blocks (24 warps) per SM at 76
// registers (80 with the learned warm start in the epilogue).  A minimum of 5
// blocks of 128 (or 10 of 64) lets the compiler keep 80 registers at the same
// 24 warps; a free choice (91 registers) drops to 20 warps.  On the 4.19 M
// lattice 64x10, 128x6 and 256x3 lie within 2 % of each other, 128x5 4 % behind;
// with the warm start 128x5 and 64x10 need 96 registers (20 warps).
const int kInteractVariants[][4] = {{128, 6, 0, 1},   {64, 12, 0, 1},   {64, 8, 0, 1},     {128, 4, 0, 1},
                                    {256, 3, 0, 1},   {256, 1, 0, 1},   {128, 3, 640, 1},  {128, 2, 1024, 1},
                                    {64, 6, 384, 1},  {256, 2, 1024, 1}, {128, 6, 0, 2},    {128, 6, 0, 4},
                                    {128, 5, 0, 1},   {64, 10, 0, 1}};

int interact_variant_count() { return (int)(sizeof(kInteractVariants) / sizeof(kInteractVariants[0])); }
void interact_variant_shape(int v, int *block, int *min_blocks, int *staged, int *lanes) {
    *block = kInteractVariants[v][0];
    *min_blocks = kInteractVariants[v][1];
    *staged = kInteractVariants[v][2];
    *lanes = kInteractVariants[v][3];
}

// Threads per block of the FP64 per-particle kernels: the largest of 256, 128,
// 64 that still gives every SM two blocks, else 32.  The FP64 pipe is narrow, so
// a small system (the reference's own cases are 7k-12k particles) must spread
// over all SMs rather than fill a few.  Results do not depend on it: each
// particle's sums run in one thread in the same order.
int fp64_block(int N) {
    static int sms[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    int &n = sms[dev & 63];
    if (!n) {
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 152;
    }
    for (int kb : {256, 128, 64})
        if (div_up(N, kb) >= 2 * n) return kb;
    return 32;
}

// ---- interactions_gpu.cu:84-140 do_interactions_heat_pse (FP64) --------------------------
// T_t = alpha * sum_j (T_j - T_i) W2(r_ij, h_i) m / rho_j over every particle of
// the 5x5 block of cells of edge h around the particle's cell (no support
// cut-off, blanked neighbours included), W2 = 4 / (h^4 pi) exp(-|r|^2 / h^2)
// (kernels.cuh:67-84).  Reads the predicted state from the FP64 records; the
// block's columns are contiguous slot ranges as in the neighbour sums.
template <int kB>
__global__ void __launch_bounds__(kB) k_heat_pse64(int N, KConsts K, const int32_t *__restrict__ offsets,
                                                       const dbl4 *__restrict__ rec,
                                                       const int32_t *__restrict__ hashes, double *__restrict__ T_t) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const dbl4 i3 = rec[4 * k + 3];
    const int fi = (int)__double_as_longlong(i3.w);
    if (fi & kFlagBlanked) return;
    const dbl4 i0 = rec[4 * k + 0], i2 = rec[4 * k + 2];
    const double xi = i0.x, yi = i0.y, hi = i2.z, Ti = i3.z;
    // the reference binds the tool flags (doubles) for N ints, half the array
    // (interactions_gpu.cu:448): from index N/2 on its fetch reads zero
    const double alpha = ((fi & kFlagTool) && k < N / 2) ? K.c.trml_tool_sph.alpha : K.c.trml_wp.alpha;
    const double h2 = hi * hi, h4 = h2 * h2;
    const double c = 4. / (h4 * kRigidPi);
    const double inv_h2 = 1. / h2;
    double sum = 0.;
    const int hash = hashes[k];
    const sph_geom_constants &g = K.g;
    if (hash >= 0 && hash < g.num_cell) {
        const int gi = hash / g.ny, gj = hash - gi * g.ny;
        const int lo_i = max(gi - 2, 0), hi_i = min(gi + 3, g.nx);
        const int lo_j = max(gj - 2, 0), hi_j = min(gj + 3, g.ny);
        for (int ii = lo_i; ii < hi_i; ii++) {
            const int j1 = __ldg(offsets + ii * g.ny + hi_j);
            for (int j = __ldg(offsets + ii * g.ny + lo_j); j < j1; j++) {
                const dbl4 n0 = rec[4 * j + 0], n3 = rec[4 * j + 3];
                const double xij = xi - n0.x, yij = yi - n0.y;
                // |r|^2 / h^2 as a product with 1/h^2; n3.y = m / rho_j.  Both differ
                // from the reference's sqrt-square, division and m / rho_j order by
                // rounding only (relative 1e-16 per term).
                const double w2 = c * exp(-(xij * xij + yij * yij) * inv_h2);
                sum += (n3.z - Ti) * w2 * n3.y;
            }
        }
    }
    T_t[k] = alpha * sum;
}

// FP32-compensated form of the PSE sum over the FP32 records: positions as
// offsets from the cell corners (cells of edge h), the Gaussian with expf, the
// sum Kahan-compensated; T_t written in FP64.
template <class TT>   // T_t: double (staged call, FP64 arrays) or float (the compact state)
__global__ void __launch_bounds__(kBlock) k_heat_pse32(int N, KConsts K, const int32_t *__restrict__ offsets,
                                                       const float4 *__restrict__ rec,
                                                       const int32_t *__restrict__ hashes, TT *__restrict__ T_t) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const float4 i0 = rec[4 * k + 0];
    const int fi = __float_as_int(i0.z);
    if (fi & kFlagBlanked) return;
    const float xri = i0.x, yri = i0.y, hi = i0.w, Ti = rec[4 * k + 3].w;
    const double alpha = ((fi & kFlagTool) && k < N / 2) ? K.c.trml_tool_sph.alpha : K.c.trml_wp.alpha;
    const float h2 = hi * hi;
    const float c = 4.f / (h2 * h2 * (float)kRigidPi);
    const float inv_h2 = 1.f / h2;
    const float cell = K.f.cell;
    KahanF sum = {};
    const int hash = hashes[k];
    const sph_geom_constants &g = K.g;
    if (hash >= 0 && hash < g.num_cell) {
        const int gi = hash / g.ny, gj = hash - gi * g.ny;
        const int lo_i = max(gi - 2, 0), hi_i = min(gi + 3, g.nx);
        const int lo_j = max(gj - 2, 0), hi_j = min(gj + 3, g.ny);
        for (int ii = lo_i; ii < hi_i; ii++) {
            const float dxc = (float)(gi - ii) * cell;
            const int j1 = __ldg(offsets + ii * g.ny + hi_j);
#pragma unroll 4   // several neighbours' loads in flight (the kernel waits on loads, not on math)
            for (int j = __ldg(offsets + ii * g.ny + lo_j); j < j1; j++) {
                const float4 n0 = rec[4 * j + 0];
                const float dx = dxc + (xri - n0.x);
                const float dy = (float)(gj - (__float_as_int(n0.z) & kRowMask)) * cell + (yri - n0.y);
                const float w2 = c * expf(-(dx * dx + dy * dy) * inv_h2);
                sum.add((rec[4 * j + 3].w - Ti) * w2 * rec[4 * j + 2].w);
            }
        }
    }
    T_t[k] = alpha * (double)sum.s;
}

void launch_heat_pse(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets, const StepScratch &W,
                     const SortedFields32 &B) {
    const int tb = fp64_block(N);
    k_heat_pse32<<<div_up(N, tb), tb, 0, s>>>(N, K, offsets, W.rec32, B.hash, B.T_t);
}

void launch_heat_pse(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets, const StepScratch &W,
                     const SortedFields &B) {
    if (K.precision == SPH_PREC_FP32K) {
        const int tb = fp64_block(N);
        k_heat_pse32<<<div_up(N, tb), tb, 0, s>>>(N, K, offsets, W.rec32, B.hash, B.T_t);
        return;
    }
    switch (fp64_block(N)) {
        case 32: k_heat_pse64<32><<<div_up(N, 32), 32, 0, s>>>(N, K, offsets, W.rec64, B.hash, B.T_t); break;
        case 64: k_heat_pse64<64><<<div_up(N, 64), 64, 0, s>>>(N, K, offsets, W.rec64, B.hash, B.T_t); break;
        case 128: k_heat_pse64<128><<<div_up(N, 128), 128, 0, s>>>(N, K, offsets, W.rec64, B.hash, B.T_t); break;
        default: k_heat_pse64<256><<<div_up(N, 256), 256, 0, s>>>(N, K, offsets, W.rec64, B.hash, B.T_t); break;
    }
}

void launch_interactions32_fused(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets,
                                 const SortedFields32 &B, const FixedFields32 &F, const StepScratch &W,
                                 const SegDev &seg, const ToolDev *tool, int variant) {
    launch_i32_variant<false>(s, N, K, offsets, B, F, W, seg, tool, variant, MlpDev{});
}

void launch_interactions(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets, const SortedFields &B,
                         const FixedFields &F, const StepScratch &W, const SegDev &seg, const ToolDev *tool,
                         bool fused, int variant) {
    const int grid = div_up(N, kBlock);
    if (K.precision == SPH_PREC_FP32K) {
        // the fused FP32K step runs on the compact state (launch_interactions32_fused)
        k_interact32<false><<<grid, kBlock, 0, s>>>(N, K, offsets, W.rec32, W.cand32, B, F, seg, tool, W.secant_iters,
                                                    W.status, 0, MlpDev{});
    } else {
        const int kb = fp64_block(N);
        const int g64 = div_up(N, kb);
#define I64(F, B) k_interact64<F, B><<<g64, B, 0, s>>>(N, K, offsets, W.rec64, B_, F_, seg, tool, W.secant_iters, W.status)
        const SortedFields &B_ = B;
        const FixedFields &F_ = F;
        if (fused) {
            switch (kb) {
                case 32: I64(true, 32); break;
                case 64: I64(true, 64); break;
                case 128: I64(true, 128); break;
                default: I64(true, 256); break;
            }
        } else {
            switch (kb) {
                case 32: I64(false, 32); break;
                case 64: I64(false, 64); break;
                case 128: I64(false, 128); break;
                default: I64(false, 256); break;
            }
        }
#undef I64
    }
}

}  // namespace sphfem
