// launch.cuh -- host-side launchers of the device kernels (one stream each).
#pragma once

#include "common.cuh"
#include "physics.cuh"
#include "state.cuh"

namespace sphfem {

// cells.cu
void launch_hash(cudaStream_t s, int N, const SortedFields &A, sph_geom_constants g);
void launch_count(cudaStream_t s, int N, const SortedFields &A, const SortScratch &X, sph_geom_constants g,
                  uint32_t *status, bool with_hash);
void launch_count(cudaStream_t s, int N, const SortedFields32 &A, const SortScratch &X, sph_geom_constants g,
                  uint32_t *status, bool with_hash);
int scan_blocks(int num_cell);
void launch_sort_rest(cudaStream_t s, int N, const SortScratch &X, sph_geom_constants g, int32_t *perm,
                      uint32_t *status);
void launch_gather_plain(cudaStream_t s, int N, const int32_t *perm, const SortedFields &A, const SortedFields &B);
void launch_gather_fused(cudaStream_t s, int N, const int32_t *perm, const KConsts &K, const SortedFields &A,
                         const SortedFields &B, const FixedFields &F, const StepScratch &W, const int32_t *hash_src,
                         const ToolDev *tool);
void launch_build_records(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F,
                          const StepScratch &W);
// FP32K fused reorder into the compact state B, from the FP64 state (A64) or the
// compact one (A32, exactly one of the two non-null); the p, R that tool
// particles keep come from F32 (pr32) or F
void launch_gather_fused32(cudaStream_t s, int N, const int32_t *perm, const KConsts &K, const SortedFields *A64,
                           const SortedFields32 *A32, bool pr32, const FixedFields &F, const FixedFields32 &F32,
                           const SortedFields32 &B, int32_t *idx, const StepScratch &W, const int32_t *hash_src,
                           const ToolDev *tool);
// the compact state (state) and F32's p, R (pr) widened into the FP64 arrays
void launch_state_to64(cudaStream_t s, int N, const SortedFields32 &A, const FixedFields32 &Fa, const SortedFields &B,
                       const FixedFields &F, bool state, bool pr);

// interactions.cu
void launch_interactions(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets, const SortedFields &B,
                         const FixedFields &F, const StepScratch &W, const SegDev &seg, const ToolDev *tool,
                         bool fused, int variant = 0);
// the fused FP32K neighbour sums and epilogue on the compact state
void launch_interactions32_fused(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets,
                                 const SortedFields32 &B, const FixedFields32 &F, const StepScratch &W,
                                 const SegDev &seg, const ToolDev *tool, int variant);
// the same with the learned warm start folded into the epilogue (interactions_mlp.cu)
void launch_interactions32_fused_mlp(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets,
                                     const SortedFields32 &B, const FixedFields32 &F, const StepScratch &W,
                                     const SegDev &seg, const ToolDev *tool, int variant, const MlpDev &mlp);
void launch_heat_pse(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets, const StepScratch &W,
                     const SortedFields &B);
void launch_heat_pse(cudaStream_t s, int N, const KConsts &K, const int32_t *offsets, const StepScratch &W,
                     const SortedFields32 &B);
int interact_variant_count();
int fp64_block(int N);   // threads per block of the FP64 per-particle kernels for N particles
void interact_variant_shape(int v, int *block, int *min_blocks, int *staged, int *lanes);

// actions.cu
void launch_init(cudaStream_t s, int N, const SortedFields &A, const StepScratch &W);
void launch_predict_correct(cudaStream_t s, int N, const SortedFields &A, const StepScratch &W, double fdt);
void launch_eos(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F);
void launch_artificial_stress(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F);
void launch_jaumann(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F);
void launch_continuity(cudaStream_t s, int N, const SortedFields &A, const FixedFields &F);
void launch_momentum(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F);
void launch_advection(cudaStream_t s, int N, const SortedFields &A);
void launch_plasticity(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const FixedFields &F,
                       const StepScratch &W);
void launch_fric_heat(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const SegDev &seg,
                      const ToolDev *tool, uint32_t *status);
// the contact's segment y-bins of every case (k_seg_bins); a no-op without bins
void launch_seg_bins(cudaStream_t s, int n_cases, const SegDev &seg, ToolDev *tool);
// builds the bins first (the tool state moves), then contact s1 / s2
void launch_contact(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const SegDev &seg,
                    ToolDev *tool, const double *T_nodes, uint32_t *status);
void launch_bc(cudaStream_t s, int N, const SortedFields &A);
void launch_bc_thermal(cudaStream_t s, int N, const KConsts &K, const SortedFields &A);
void launch_invalidate(cudaStream_t s, int N, const SortedFields &A, uint32_t *status);
// with the FEM tool: the segment y-bins and the contact pass (k_contact_fem) first (two more launches)
void launch_step_tail(cudaStream_t s, int N, const KConsts &K, const SortedFields &A, const SegDev &seg,
                      ToolDev *tool, const double *T_nodes, const SortScratch &X, uint32_t *status,
                      bool next_hash);
void launch_step_tail(cudaStream_t s, int N, const KConsts &K, const SortedFields32 &A, const SegDev &seg,
                      ToolDev *tool, const double *T_nodes, const SortScratch &X, uint32_t *status,
                      bool next_hash);
void launch_rigid_move(cudaStream_t s, sph_rigid_tool *t, double dt);
void launch_rigid_move_particles(cudaStream_t s, int N, const SortedFields &A, const sph_rigid_tool *t, double dt);
void launch_contact_rigid(cudaStream_t s, int N, const KConsts &K, const SortedFields &A);
void launch_fric_heat_rigid(cudaStream_t s, int N, const KConsts &K, const SortedFields &A);
int reduce_blocks();
void launch_usui(cudaStream_t s, int N, const SortedFields &A, double K_usui, double alpha, double vtx, double vty,
                 double *out);
void launch_reduce_force_T(cudaStream_t s, int N, const SortedFields &A, double *out);
void launch_reduce_cases(cudaStream_t s, int n_cases, const SortedFields &A, const int32_t *offsets,
                         const int32_t *cell_bound, const int32_t *part_bound, double *out);

// fem.cu
void launch_fem_half(cudaStream_t s, const KConsts &K, const FemDev &F, const ToolDev *tool);
void launch_fem_rate_update(cudaStream_t s, const KConsts &K, const FemDev &F, const SegDev &seg,
                            const ToolDev *tool);
void launch_fem_reset(cudaStream_t s, const FemDev &F, double *T_old, double *f_temp, double *K_temp);
void launch_fem_robin(cudaStream_t s, const KConsts &K, const FemDev &F, const SegDev &seg, double *f_temp,
                      double *K_temp);
void launch_fem_rate(cudaStream_t s, const FemDev &F, const double *f_temp, const double *K_temp);
void launch_fem_temp(cudaStream_t s, const FemDev &F, const double *T_old, double dt);
// the tool's thermal system assembled on the device: K, lumped M (into M), the
// Dirichlet elimination in the given order (f) and M_inv
void launch_fem_assemble(cudaStream_t s, const FemDev &F, const int4 *elements, int n_elem, int n_colors,
                         const int32_t *dir_elems, const int4 *dir_flags, int n_dir, double cp, double rho, double k,
                         double T0, double *M);
void launch_tool_move(cudaStream_t s, const KConsts &K, const SegDev &seg, const FemDev &F, ToolDev *tool, double dt,
                      int what, bool per_case);

// wear.cu
void launch_wear_reset(cudaStream_t s, const SegDev &seg);
void launch_wear_adjustment(cudaStream_t s, const KConsts &K, const FemDev &F, const SegDev &seg, const WearDev &W,
                            ToolDev *tool, double dt);
// remesh_low_level (tool_FEM.cu:1696-1705): interior nodes shifted, the
// thermal system re-assembled, nodal temperatures interpolated from the old
// mesh (pos_old, T_old: scratch of n_nodes)
void launch_remesh_low_level(cudaStream_t s, const FemDev &F, const int4 *elements, int n_elem, int n_colors,
                             const int32_t *node_edge, const ToolDev *tool, int freq, const int32_t *dir_elems,
                             const int4 *dir_flags, int n_dir, const sph_tool_constants &tc, double2 *pos_old,
                             double *T_old);

// mlp.cu
size_t mlp_fwd_smem();
size_t mlp_train_smem();
cudaError_t mlp_configure();
void launch_mlp_predict(cudaStream_t s, const MlpDev &m, const float *x, int64_t n, float *y, uint32_t *status,
                        int grid);
// one warp per sample, the fused step's in-epilogue form (grid: blocks of 256)
void launch_mlp_predict_warp(cudaStream_t s, const MlpDev &m, const float *x, int64_t n, float *y, int grid);
void launch_jc_warm(cudaStream_t s, int grid, const KConsts &K, const SortedFields32 &B, const FixedFields32 &F,
                    const ToolDev *tool, const MlpDev &m, int32_t *secant_iters, uint32_t *status);
void launch_mlp_grad(cudaStream_t s, int grid, const MlpDev &m, const float *x, const float *t, const int32_t *idx,
                     int64_t nb, float *part, uint32_t *status);
void launch_mlp_reduce_adam(cudaStream_t s, const float *part, int nparts, float *grad_out, float *loss_out,
                            float *params, float *m1, float *m2, uint16_t *wb, float lr, float beta1, float beta2,
                            float eps, float c1, float c2, bool adam);
void launch_mlp_refresh_wb(cudaStream_t s, const float *params, uint16_t *wb);

// persistent.cu: the fused FP32K step from the compact state as one cooperative
// launch (A -> B, perm = the sort's idx array; bar: 4 words of device memory)
struct PersistArgs {
    int N;
    KConsts K;
    SortScratch X;
    SortedFields32 A, B;
    FixedFields32 F32;
    int32_t *perm;
    StepScratch W;
    SegDev seg;
    FemDev fem;
    ToolDev *tool;
    MlpDev mlp;
    unsigned *bar;
};
cudaError_t launch_step_persistent(cudaStream_t s, const PersistArgs &P, bool tool, bool mlp, int num_sms);

}  // namespace sphfem
