// fem.cu -- explicit FEM thermal update of the tool and the rigid tool motion
// (FEM_thermal_gpu.cu:342-468,865-921; tool_FEM.cu:109-139,1552-1582).
//
// The reference copies K -> K_temp and f -> f_temp every step
// (reset_FEM_server), adds the Robin terms of every contact segment with
// atomics in six colour launches (apply_robin_bdc) and then runs a
// one-thread-per-row SpMV.  Here each node gathers the Robin terms of the
// (at most a few) segments that end on it, in a fixed order, and applies them
// inside its own SpMV row: the same arithmetic without the per-step matrix
// copy, without atomics and without the colour launches.
#include "fem.cuh"
#include "p1elem.h"

namespace sphfem {

__global__ void __launch_bounds__(kBlock) k_fem_half(KConsts K, FemDev F, const ToolDev *__restrict__ tool) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < F.n_nodes) fem_half_one(i, K, F, tool);
}

__global__ void __launch_bounds__(kBlock) k_fem_rate_update(KConsts K, FemDev F, SegDev seg,
                                                            const ToolDev *__restrict__ tool) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < F.n_nodes) fem_rate_update_one(i, K, F, seg, tool);
}

// Staged forms: the reference's separate calls.  K_temp / f_temp hold the
// per-step copies that reset_FEM_server makes.
__global__ void __launch_bounds__(kBlock) k_fem_reset(FemDev F, double *__restrict__ T_old,
                                                      double *__restrict__ f_temp, double *__restrict__ K_temp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < F.n_nodes) {
        T_old[i] = F.T[i];
        f_temp[i] = F.f[i];
    }
    if (i < F.nnz) K_temp[i] = F.K[i];
}

__global__ void __launch_bounds__(kBlock) k_fem_robin(KConsts K, FemDev F, SegDev seg, double *__restrict__ f_temp,
                                                      double *__restrict__ K_temp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.n_nodes) return;
    double df, dk;
    robin_terms(K, F, seg, i, df, dk);
    f_temp[i] += df;
    K_temp[F.diag[i]] += dk;
}

__global__ void __launch_bounds__(kBlock) k_fem_rate(FemDev F, const double *__restrict__ f_temp,
                                                     const double *__restrict__ K_temp) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.n_nodes) return;
    double buffer = 0.;
    for (int t = F.row_ptr[i]; t < F.row_ptr[i + 1]; t++) buffer += K_temp[t] * F.T[F.col_ind[t]];
    F.k[i] = F.M_inv[i] * (f_temp[i] - buffer);
}

__global__ void __launch_bounds__(kBlock) k_fem_temp(FemDev F, const double *__restrict__ T_old, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= F.n_nodes) return;
    F.T[i] = dt * F.k[i] + T_old[i];
}

__global__ void __launch_bounds__(kBlock) k_tool_move(KConsts K, SegDev seg, FemDev F, ToolDev *tool, double dt,
                                                      int what, int per_case) {
    tool_move_one(blockIdx.x * blockDim.x + threadIdx.x, K, seg, F, tool, dt, what, per_case);
}

// ---- host launchers ---------------------------------------------------------------------------
void launch_fem_half(cudaStream_t s, const KConsts &K, const FemDev &F, const ToolDev *tool) {
    k_fem_half<<<div_up(F.n_nodes, kBlock), kBlock, 0, s>>>(K, F, tool);
}
void launch_fem_rate_update(cudaStream_t s, const KConsts &K, const FemDev &F, const SegDev &seg,
                            const ToolDev *tool) {
    k_fem_rate_update<<<div_up(F.n_nodes, kBlock), kBlock, 0, s>>>(K, F, seg, tool);
}
void launch_fem_reset(cudaStream_t s, const FemDev &F, double *T_old, double *f_temp, double *K_temp) {
    k_fem_reset<<<div_up(F.nnz > F.n_nodes ? F.nnz : F.n_nodes, kBlock), kBlock, 0, s>>>(F, T_old, f_temp, K_temp);
}
void launch_fem_robin(cudaStream_t s, const KConsts &K, const FemDev &F, const SegDev &seg, double *f_temp,
                      double *K_temp) {
    k_fem_robin<<<div_up(F.n_nodes, kBlock), kBlock, 0, s>>>(K, F, seg, f_temp, K_temp);
}
void launch_fem_rate(cudaStream_t s, const FemDev &F, const double *f_temp, const double *K_temp) {
    k_fem_rate<<<div_up(F.n_nodes, kBlock), kBlock, 0, s>>>(F, f_temp, K_temp);
}
void launch_fem_temp(cudaStream_t s, const FemDev &F, const double *T_old, double dt) {
    k_fem_temp<<<div_up(F.n_nodes, kBlock), kBlock, 0, s>>>(F, T_old, dt);
}
void launch_tool_move(cudaStream_t s, const KConsts &K, const SegDev &seg, const FemDev &F, ToolDev *tool, double dt,
                      int what, bool per_case) {
    int n = per_case ? K.n_cases : 1;
    if ((what & 1) && seg.n > n) n = seg.n;
    if ((what & 2) && F.n_nodes > n) n = F.n_nodes;
    k_tool_move<<<div_up(n, kBlock), kBlock, 0, s>>>(K, seg, F, tool, dt, what, per_case ? 1 : 0);
}

// ---- set-up of the thermal system on the device (FEM_thermal_gpu.cu:126-332) ----------
// do_stiffness_mass_matrix_construction_p1q3 for the elements of one colour:
// elements of a colour share no node, so every K entry and mass slot receives
// at most one term per launch and the colours run in order -- the sums are
// formed in the same order as the host assembly's colour-by-colour loop.
__global__ void __launch_bounds__(kBlock) k_fem_assemble(int colour, int n_elem, const int4 *__restrict__ elements,
                                                         const double2 *__restrict__ pos,
                                                         const int32_t *__restrict__ row_ptr,
                                                         const int32_t *__restrict__ col_ind, double cp, double rho,
                                                         double k, double *__restrict__ K, double *__restrict__ M) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    const int4 el = elements[e];
    if (el.w != colour) return;
    const double2 p0 = pos[el.x], p1 = pos[el.y], p2 = pos[el.z];
    double m, ke[3][3];
    p1_element(p0.x, p0.y, p1.x, p1.y, p2.x, p2.y, cp, rho, k, m, ke);
    const int nd[3] = {el.x, el.y, el.z};
    for (int a = 0; a < 3; a++) {
        M[nd[a]] = __dadd_rn(M[nd[a]], m);
        for (int b = 0; b < 3; b++)
            for (int j = row_ptr[nd[a]]; j < row_ptr[nd[a] + 1]; j++)
                if (col_ind[j] == nd[b]) {
                    K[j] = __dadd_rn(K[j], ke[a][b]);
                    break;
                }
    }
}

// do_dirichlet_bdc_p1q3 (FEM_thermal_gpu.cu:234-324) in the reference's
// processing order -- colour by colour, then element order -- by one thread:
// the reference's threads of one colour read and zero each other's symmetric
// entries, so only a fixed order gives one answer.  The fixed boundary holds
// a few hundred elements; this runs once per context.
__global__ void k_fem_dirichlet(int n, const int32_t *__restrict__ elems, const int4 *__restrict__ flags,
                                const int4 *__restrict__ elements, const int32_t *__restrict__ row_ptr,
                                const int32_t *__restrict__ col_ind, double T0, double *__restrict__ K,
                                double *__restrict__ M, double *__restrict__ f) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    auto node = [&](int nd) {
        for (int i = row_ptr[nd]; i < row_ptr[nd + 1]; i++) {
            const int local_no = col_ind[i];
            f[local_no] = __dadd_rn(f[local_no], -__dmul_rn(K[i], T0));
            K[i] = 0.;
            for (int t = row_ptr[local_no]; t < row_ptr[local_no + 1]; t++)   // find_location
                if (col_ind[t] == nd) {
                    K[t] = 0.;
                    break;
                }
            if (local_no == nd) K[i] = 1.0;
        }
        M[nd] = 1.0;
        f[nd] = T0;
    };
    for (int q = 0; q < n; q++) {
        const int4 el = elements[elems[q]];
        const int4 ff = flags[q];
        bool fx = false, fy = false, fz = false;
        if (ff.x) fx = fy = true;
        if (ff.y) fy = fz = true;
        if (ff.z) fz = fx = true;
        if (fx) node(el.x);
        if (fy) node(el.y);
        if (fz) node(el.z);
    }
}

// do_inverse_mass_matrix_lumped (FEM_thermal_gpu.cu:326-332)
__global__ void __launch_bounds__(kBlock) k_fem_inverse_mass(int n, const double *__restrict__ M,
                                                             double *__restrict__ M_inv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) M_inv[i] = 1. / M[i];
}

void launch_fem_assemble(cudaStream_t s, const FemDev &F, const int4 *elements, int n_elem, int n_colors,
                         const int32_t *dir_elems, const int4 *dir_flags, int n_dir, double cp, double rho, double k,
                         double T0, double *M) {
    cudaMemsetAsync(F.K, 0, sizeof(double) * (size_t)F.nnz, s);
    cudaMemsetAsync(M, 0, sizeof(double) * (size_t)F.n_nodes, s);
    cudaMemsetAsync(F.f, 0, sizeof(double) * (size_t)F.n_nodes, s);
    for (int c = 1; c <= n_colors; c++)
        k_fem_assemble<<<div_up(n_elem, kBlock), kBlock, 0, s>>>(c, n_elem, elements, F.position, F.row_ptr,
                                                                 F.col_ind, cp, rho, k, F.K, M);
    if (n_dir > 0)
        k_fem_dirichlet<<<1, 1, 0, s>>>(n_dir, dir_elems, dir_flags, elements, F.row_ptr, F.col_ind, T0, F.K, M, F.f);
    k_fem_inverse_mass<<<div_up(F.n_nodes, kBlock), kBlock, 0, s>>>(F.n_nodes, M, F.M_inv);
}

}  // namespace sphfem
