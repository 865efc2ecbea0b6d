/*
 * sphfem.h -- C ABI of the GB300 (sm_103a) SPH workpiece hot path.
 *
 * Drop-in boundary for the per-timestep path of the hybrid SPH-FEM 2D
 * cutting solver (nyzhang1227/SPH_FEM_2D_cutting_gpu).  The reference has no
 * plugin layer; its boundary is the set of C++ functions and methods that
 * `leap_frog::step(particle_gpu*, grid_base*, tool_FEM*)` calls
 * (leap_frog.cu:162-248).  Every entry point below replaces one of those
 * calls; the replaced reference interface is cited beside each one.
 *
 * Conventions
 *  - Every function returns an int status (SPH_OK == 0).  No exceptions or
 *    process exits cross the ABI; CUDA errors map to SPH_ERR_CUDA and the
 *    message is available from sph_last_error().
 *  - All arithmetic state is FP64 in the caller-visible views ("double" for
 *    the reference's float_t with USE_DOUBLE, types.h:22,57-86).  Vector
 *    fields are interleaved exactly like the reference's double2/double4.
 *  - One context == one CUDA device + one CUDA stream.  Calls on one context
 *    are not thread-safe; separate contexts are independent.
 *  - Device memory is owned by the context.  Host arrays passed in or out are
 *    owned by the caller and copied synchronously.
 *  - Like the reference's Green grid (grid_gpu_green.cu:152-182,204-205) the
 *    sort swaps the particle arrays with a second buffer, so device pointers
 *    returned by sph_get_particles() are valid only until the next sort/step.
 */
#ifndef SPHFEM_H
#define SPHFEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHFEM_ABI_VERSION 1

/* ---- return codes ------------------------------------------------------ */
enum {
    SPH_OK = 0,
    SPH_ERR_INVALID = 1,   /* bad argument or size                         */
    SPH_ERR_CUDA = 2,      /* a CUDA runtime call failed                   */
    SPH_ERR_NO_DEVICE = 3, /* no CUDA device / wrong architecture          */
    SPH_ERR_ALLOC = 4,     /* device or host allocation failed             */
    SPH_ERR_STATE = 5      /* call not valid in this state (e.g. no tool)  */
};

/* ---- device status word bits (sph_status) ------------------------------- */
#define SPH_STATUS_OUT_OF_GRID    (1u << 0) /* a particle hashed outside the cell grid (reference: UB)   */
#define SPH_STATUS_SECANT_MAXITER (1u << 1) /* return mapping hit 100 iterations (plasticity.cuh:155)    */
#define SPH_STATUS_NAN_BLANKED    (1u << 2) /* NaN/Inf rate -> particle blanked (actions_gpu.cu:816)      */
#define SPH_STATUS_CONTACT_NOSEG  (1u << 3) /* inside tool, no segment found (actions_gpu.cu:188-191)     */
#define SPH_STATUS_CONTACT_DEEP   (1u << 4) /* blanked for penetration > 2.5e-4 (actions_gpu.cu:479-492)  */
#define SPH_STATUS_MELT_BLANKED   (1u << 5) /* T > Tmelt -> blanked (actions_gpu.cu:750-753)              */
#define SPH_STATUS_FRIC_NAN       (1u << 6) /* NaN sliding velocity -> blanked (actions_gpu.cu:375-380)   */
#define SPH_STATUS_CELL_OVERFLOW  (1u << 7) /* a cell held more particles than the in-cell ranker allows  */
#define SPH_STATUS_MMA_TIMEOUT    (1u << 8) /* a tensor-core wait of the learned warm start gave up (1 s)  */
#define SPH_STATUS_COPY_TIMEOUT   (1u << 9) /* a staged neighbour copy did not complete in 1 s (global loads used) */
#define SPH_STATUS_GRID_TIMEOUT   (1u << 10) /* a grid-wide barrier of the persistent step gave up (1 s)     */

/* ---- precision of the particle path ------------------------------------ */
enum {
    SPH_PREC_FP64 = 0,     /* plain FP64 (reference USE_DOUBLE semantics)                         */
    SPH_PREC_FP32K = 1     /* FP32 neighbour sums with Kahan compensation; FP64 positions, FP64
                              return-mapping residual and FP64 FEM thermal solve                   */
};

/* ---- constant collections (constants_structs.h:18-121) ----------------- */
typedef struct sph_phys_constants {      /* phys_constants, constants_structs.h:18-26 */
    double E, nu, rho0, K, G, mass, mass_tool;
} sph_phys_constants;

typedef struct sph_trml_constants {      /* trml_constants, constants_structs.h:30-37 */
    double cp, tq, k, alpha, T_init, eta;
} sph_trml_constants;

typedef struct sph_corr_constants {      /* corr_constants, constants_structs.h:41-48 */
    double wdeltap, stresseps, xspheps, alpha, beta, eta;
} sph_corr_constants;

typedef struct sph_joco_constants {      /* joco_constants, constants_structs.h:52-66 */
    double A, B, C, n, m, Tmelt, Tref, eps_dot_ref;
    double tanh_a, tanh_b, tanh_c, tanh_d;
} sph_joco_constants;

typedef struct sph_tool_constants {      /* tool_constants, constants_structs.h:80-109 (no *_FRI variants) */
    double cp, tq, k, eta, rho, T0, h, beta, mu, contact_alpha, slave_mass, hc;
} sph_tool_constants;

/* Everything the reference installs with actions_setup_* / interactions_setup_*
 * (actions_gpu.cu:913-954, interactions_gpu.cu:476-507). */
typedef struct sph_constants {
    sph_phys_constants phys;
    sph_corr_constants corr;
    sph_joco_constants joco;
    sph_trml_constants trml_wp;        /* workpiece: actions thermals_wp and interactions trml       */
    sph_trml_constants trml_tool;      /* actions thermals_tool; alpha != 0 enables thermal BCs      */
    sph_trml_constants trml_tool_sph;  /* interactions trml_tool (SPH tool particles); zero when the
                                          reference never calls interactions_setup_thermal_constants_tool */
    sph_tool_constants tool;
    int32_t plastic;                   /* actions_setup_johnson_cook_constants called (m_plastic)    */
    int32_t pad0;
} sph_constants;

/* Locked cell grid: grid_base(num_part, bbmin, bbmax, h) -> set_geometry
 * (grid.cu:130-149).  The reference uses cell edge == h and a 5x5 stencil
 * (cell_factor = 1, stencil = 2).  cell_factor = 2, stencil = 1 gives 2h
 * cells with a 3x3 stencil; results then differ only by summation order. */
typedef struct sph_grid_params {
    double bbmin[2];
    double bbmax[2];
    double h;
    int32_t cell_factor;
    int32_t stencil;
} sph_grid_params;

/* Derived grid geometry: geom_constants (constants_structs.h:70-76). */
typedef struct sph_geom_constants {
    int32_t nx, ny;
    double bbmin_x, bbmin_y, dx;
    int32_t num_cell;
    int32_t stencil;
} sph_geom_constants;

/* ---- particle SoA (particle_gpu, particle_gpu.h:23-83) ------------------ */
typedef struct sph_particles {
    int32_t N;
    int32_t pad0;
    double *pos, *vel;                      /* [N][2] */
    double *h, *rho, *p;                    /* [N]    */
    double *S, *R;                          /* [N][4] S = (Sxx, Sxy, Syy, Szz), R = (Rxx, Rxy, Ryy, 0) */
    double *fc, *ft, *n;                    /* [N][2] */
    double *fixed, *blanked, *tool_particle;/* [N] 0/1 flags stored as double, as the reference */
    double *eps_pl, *eps_pl_dot, *T;        /* [N]    */
    double *pos_t, *vel_t;                  /* [N][2] */
    double *rho_t;                          /* [N]    */
    double *S_t;                            /* [N][4] */
    double *T_t;                            /* [N]    */
    double *S_der, *v_der;                  /* [N][4] */
    int32_t *idx, *hash, *on_seg;           /* [N]    */
} sph_particles;

/* ---- FEM tool interface segments (segment_FEM_gpu, segment_FEM_gpu.h:31-56) */
typedef struct sph_segments {
    int32_t n;
    int32_t pad0;
    double *left, *right, *normal;          /* [n][2] */
    int32_t *marks;                         /* [n][4] element, colour, node left, node right */
    double *heat_exchange;                  /* [n][2] (sum T*length, sum length) */
    double *fric_heat;                      /* [n]    */
} sph_segments;

/* ---- FEM thermal system of the tool (FEM_thermal_2D_GPU, FEM_thermal_gpu.h:35-93) */
typedef struct sph_fem {
    int32_t n_nodes, nnz;
    double *position;                       /* [n_nodes][2] mesh_GPU_m::position */
    int32_t *row_ptr;                       /* [n_nodes+1] */
    int32_t *col_ind;                       /* [nnz] */
    double *K;                              /* [nnz] m_stiffness_matrix (after Dirichlet) */
    double *M_inv;                          /* [n_nodes] m_mass_matrix_inverse (lumped) */
    double *f;                              /* [n_nodes] m_f (after Dirichlet) */
    double *T;                              /* [n_nodes] m_T */
    double *k;                              /* [n_nodes] m_k (temperature rate) */
} sph_fem;

/* Host description of a linear-triangle tool mesh: what mesh_read produces
 * (mesh_structure_GPU.h:37-78) before colouring and CSR construction. */
typedef struct sph_tool_mesh {
    int32_t n_nodes, n_elements;
    const double *nodes;                    /* [n_nodes][2] (cm) */
    const int32_t *elements;                /* [n_elements][3] node ids */
    const int32_t *cutting_flags;           /* [n_elements][3] edge (a,b),(b,c),(c,a) on the contact interface */
    const int32_t *fixed_flags;             /* [n_elements][3] edge on the fixed-temperature boundary */
    const double *T_init;                   /* [n_nodes] initial nodal temperature, or NULL for tool.T0 */
    double tl[2];                           /* tool_FEM ctor top-left point (segment normal reference) */
} sph_tool_mesh;

/* Rigid tool kinematics kept on the host by tool_FEM (tool_FEM.h:57-77). */
typedef struct sph_tool_state {
    double vel[2];
    double tl_point_ref[2];
    double br_point[2];
    double ref_dist;
    double lowest_point, right_point;
    int32_t n_segments, n_cut_colors;
    /* wear (WEAR_NODE_SHIFT): flank_retreat (tool_FEM.cu:19) is added to the y
     * motion of nodes and segments every step; flank_contact (tool_FEM.cu:20) is
     * lowest_point after the last tool update.  Both 0 / lowest_point without wear. */
    double flank_retreat, flank_contact;
} sph_tool_state;

typedef struct sph_ctx sph_ctx;
typedef struct sph_tool_host sph_tool_host;

/* ---- host-only tool set-up (no GPU needed) -------------------------------
 * The set-up that sph_ctx_create performs for a tool mesh, on the host only:
 * mesh colouring and CSR pattern (mesh_structure_GPU.cu:596-780), interface
 * segments (tool_FEM::set_up_segments_from_mesh, tool_FEM.cu:771-1039) and
 * the assembled FEM system (FEM_thermal_gpu.cu:126-332). */
int sph_tool_build(const sph_tool_mesh *mesh, const sph_tool_constants *tc, sph_tool_host **out);
int sph_tool_host_info(const sph_tool_host *t, sph_tool_state *state, int32_t *n_nodes, int32_t *nnz,
                       int32_t *n_colors);
/* Copies into caller arrays (NULL fields skipped); sizes must match. */
int sph_tool_host_export(const sph_tool_host *t, sph_segments *seg, sph_fem *fem);
/* Wear layers of the host tool model (layer[e][0]: layer 1, layer[e][1]: layer 2;
 * mesh_structure_GPU.cu:1063-1148). */
int sph_tool_host_layers(const sph_tool_host *t, int32_t *layer);
/* Elements of the host tool model after colouring: elements[e] = (node a, b, c,
 * colour 1..n_colors) (mesh_GPU_m::node_num, mesh_structure_GPU.cu:596-739). */
int sph_tool_host_elements(const sph_tool_host *t, int32_t *elements);
int sph_tool_host_destroy(sph_tool_host *t);

/* ---- context ------------------------------------------------------------ */
/* Allocates particle_gpu (particle_gpu.cu:11-104), the Green grid buffers
 * (grid_gpu_green.cu:224-266), leap_frog snapshots (leap_frog.cu:261-271),
 * and, with a tool mesh, sets up the interface segments
 * (tool_FEM::set_up_segments_from_mesh, tool_FEM.cu:771-1039) and assembles
 * the FEM thermal system (FEM_thermal_gpu.cu:584-603).  `tool` may be NULL
 * for a tool-less run.  `host` arrays that are NULL start at zero, except
 * on_seg which starts at 0 like the reference. */
int sph_ctx_create(const sph_constants *c, const sph_grid_params *g,
                   const sph_particles *host, const sph_tool_mesh *tool,
                   double dt, int32_t precision, int32_t device, sph_ctx **out);
int sph_ctx_destroy(sph_ctx *ctx);
const char *sph_last_error(const sph_ctx *ctx);
int sph_abi_version(void);

int sph_set_dt(sph_ctx *ctx, double dt);                         /* global_dt */
int sph_get_geometry(const sph_ctx *ctx, sph_geom_constants *out);
int sph_set_constants(sph_ctx *ctx, const sph_constants *c);     /* *_setup_*_constants */
int sph_sync(sph_ctx *ctx);
int sph_status(sph_ctx *ctx, uint32_t *status, int32_t clear);
/* The CUDA stream the context launches on (cudaStream_t as void*). */
int sph_get_stream(const sph_ctx *ctx, void **stream);

/* ---- particle data in and out ------------------------------------------ */
int sph_get_particles(sph_ctx *ctx, sph_particles *dev_view);    /* device pointers (post-swap) */
int sph_upload_particles(sph_ctx *ctx, const sph_particles *host);   /* non-NULL fields only */
int sph_download_particles(sph_ctx *ctx, sph_particles *host);       /* non-NULL fields only */
int sph_get_cells(sph_ctx *ctx, int32_t **cell_start, int32_t **cell_end, int32_t *num_cell); /* device */
int sph_download_cells(sph_ctx *ctx, int32_t *cell_start, int32_t *cell_end);

/* ---- grid (grid.cu, grid_gpu_green.cu) ---------------------------------- */
int sph_update_geometry(sph_ctx *ctx);   /* grid_base::update_geometry: no-op on a locked grid (grid.cu:88-91) */
int sph_assign_hashes(sph_ctx *ctx);     /* grid_base::assign_hashes -> compute_hashes (grid.cu:25-42,80-86) */
int sph_sort(sph_ctx *ctx);              /* grid_gpu_green::sort -> do_sort (grid_gpu_green.cu:185-212)       */

/* ---- leap-frog (leap_frog.cu:25-96) ------------------------------------- */
int sph_init(sph_ctx *ctx);              /* init: snapshot pos, vel, S, rho, T (leap_frog.cu:25-37) */
int sph_predict(sph_ctx *ctx);           /* predict with 0.5*dt (leap_frog.cu:45-69)                */
int sph_correct(sph_ctx *ctx);           /* correct with dt (leap_frog.cu:71-96)                    */

/* ---- per-particle actions (actions_gpu.cu) ------------------------------ */
int sph_material_eos(sph_ctx *ctx);                    /* material_eos, :838-842 -> :222-232              */
int sph_corrector_artificial_stress(sph_ctx *ctx);     /* corrector_artificial_stress, :844-848 -> :234-278 */
int sph_material_stress_rate_jaumann(sph_ctx *ctx);    /* :850-854 -> :280-314                           */
int sph_contmech_continuity(sph_ctx *ctx);             /* :856-860 -> :626-639                           */
int sph_contmech_momentum(sph_ctx *ctx);               /* :862-866 -> :641-671                           */
int sph_contmech_advection(sph_ctx *ctx);              /* :868-872 -> :673-687                           */
int sph_plasticity_johnson_cook(sph_ctx *ctx);         /* :874-879 -> :689-754, plasticity.cuh:21-162    */
int sph_perform_boundary_conditions(sph_ctx *ctx);     /* :888-892 -> :765-781                           */
int sph_perform_boundary_conditions_thermal(sph_ctx *ctx); /* :881-886 -> :756-763                       */
int sph_debug_invalidate(sph_ctx *ctx);                /* :907-911 -> :787-824                           */

/* ---- neighbour sums (interactions_gpu.cu) ------------------------------- */
int sph_interactions_monaghan(sph_ctx *ctx);           /* interactions_monaghan, :381-432 -> :143-379    */

/* ---- FEM tool coupling -------------------------------------------------- */
int sph_material_fric_heat_gen_fem(sph_ctx *ctx);      /* material_fric_heat_gen_FEM_v2, actions_gpu.cu:967-981 -> :345-420 */
int sph_compute_contact_forces_fem(sph_ctx *ctx);      /* compute_contact_forces_FEM_tool_v3, actions_gpu.cu:983-999 -> :423-617 */
int sph_segments_update(sph_ctx *ctx, double dt);      /* tool_FEM::segments_update, tool_FEM.cu:1572-1582 -> :119-139 */
int sph_tool_update_fem(sph_ctx *ctx, double dt);      /* tool_FEM::tool_update_FEM_gpu, tool_FEM.cu:1552-1570 -> :109-117 */
int sph_fem_reset_server(sph_ctx *ctx);                /* FEM_thermal_2D_GPU::reset_FEM_server, FEM_thermal_gpu.cu:902-921 */
int sph_fem_apply_robin(sph_ctx *ctx);                 /* tool_FEM::apply_heat_boundary_condition -> apply_robin_bdc, :865-877 -> :342-386 */
int sph_fem_calculate_temp_rate(sph_ctx *ctx);         /* calculate_temp_rate, :879-889 -> :443-458     */
int sph_fem_calculate_temp(sph_ctx *ctx, double dt);   /* calculate_temp, :891-900 -> :460-468          */
int sph_set_tool_velocity(sph_ctx *ctx, double vx, double vy);   /* tool::set_vel */
int sph_get_tool_state(sph_ctx *ctx, sph_tool_state *out);
int sph_get_segments(sph_ctx *ctx, sph_segments *dev_view);
int sph_download_segments(sph_ctx *ctx, sph_segments *host);
int sph_get_fem(sph_ctx *ctx, sph_fem *dev_view);
int sph_download_fem(sph_ctx *ctx, sph_fem *host);
int sph_upload_fem_state(sph_ctx *ctx, const double *T, const double *k); /* nodal T and rate, NULL = keep */

/* ---- whole step ---------------------------------------------------------- */
/* leap_frog::step(particle_gpu*, grid_base*, tool_FEM*) (leap_frog.cu:162-248),
 * or the tool-less leap_frog::step(particle_gpu*, grid_base*) (:99-160 without
 * the SPH-particle tool) when the context has no tool.  Runs fused kernels;
 * the first call records a CUDA graph that later calls replay. */
int sph_step(sph_ctx *ctx);
int sph_run(sph_ctx *ctx, int32_t nsteps);
/* Same step, issued as the unfused per-stage kernels in reference order. */
int sph_step_staged(sph_ctx *ctx);

/* ---- rigid tool (the reference's SPH-tool mode) --------------------------------------
 * leap_frog::step(particle_gpu*, grid_base*) with a global `tool` (leap_frog.cu:
 * 99-160): a rigid polygon tool of up to five segments and an optional fillet
 * (tool.cpp, tool_gpu.cu), penalty contact with LS-DYNA friction
 * (do_compute_contact_forces, tool_gpu.cu:142-198), friction heat
 * (do_material_fric_heat_gen, actions_gpu.cu:316-343, when trml_wp.eta != 0),
 * tool particles moved with the tool (update_tool_particles, tool_gpu.cu:201-213)
 * and the segments moved on the host every step (tool::update_tool,
 * tool.cpp).  Segment i runs left -> right with outward normal n, the line
 * y = a x + b (x = b when vertical) through its end points; with a fillet the
 * tool has five segments and the fillet replaces segment 2 in the distance
 * search.  The penalty uses phys.mass and tool.contact_alpha.  A context has
 * either a FEM tool or a rigid tool. */
#define SPH_RIGID_MAX_SEG 5
typedef struct sph_rigid_tool {
    int32_t n_seg, has_fillet;
    double left[SPH_RIGID_MAX_SEG][2], right[SPH_RIGID_MAX_SEG][2], n[SPH_RIGID_MAX_SEG][2];
    double la[SPH_RIGID_MAX_SEG], lb[SPH_RIGID_MAX_SEG];
    int32_t vertical[SPH_RIGID_MAX_SEG], pad0;
    double fillet_p[2], fillet_r, fillet_t1, fillet_t2;   /* centre, radius, angle range */
    double vel[2];
    double mu;                                           /* Coulomb friction; 0: none */
} sph_rigid_tool;

int sph_set_rigid_tool(sph_ctx *ctx, const sph_rigid_tool *tool);   /* NULL removes it */
int sph_get_rigid_tool(sph_ctx *ctx, sph_rigid_tool *tool);
/* Staged calls of the rigid-tool step: tool_gpu_update_tool (segments and tool
 * particles by vel * dt), compute_contact_forces, material_fric_heat_gen. */
int sph_rigid_tool_update(sph_ctx *ctx);
int sph_compute_contact_forces(sph_ctx *ctx);
int sph_material_fric_heat_gen(sph_ctx *ctx);

/* Thermal conduction model of the neighbour sums: SPH_THERMAL_BROOKSHAW (the
 * reference's default, interactions_gpu.cu:143-379) or SPH_THERMAL_PSE
 * (do_interactions_heat_pse, interactions_gpu.cu:84-140; contexts on cells of edge h,
 * FP64 or FP32K). */
#define SPH_THERMAL_BROOKSHAW 0
#define SPH_THERMAL_PSE 1
int sph_set_thermal_model(sph_ctx *ctx, int32_t model);
int sph_interactions_heat_pse(sph_ctx *ctx);

/* ---- wear log: tool_wear::eval_usui (tool_wear.cu:14-54) ---------------------------
 * Usui wear rate K exp(alpha/T) p |v_r| over the particles in contact (p = |fc| /
 * (2 pi h), v_r = v - v*n with the component-wise product of the reference, and
 * its in-contact test on fc.x, fc.y, ft.x, fc.y): out = {min, max, mean}, 0 when
 * no particle is in contact; *accum_wear (if given) += dt * mean. */
int sph_eval_usui(sph_ctx *ctx, double K_usui, double alpha, const double tool_vel[2], double dt, double out[3],
                  double *accum_wear);

/* ---- output in the reference's formats ---------------------------------------------
 * Legacy-ASCII VTK as vtk_writer.cu writes it: particles (vtk_writer.cu:11-220:
 * non-blanked particles as vertex cells with Temperature, on_seg,
 * EquivAccumPlasticStrain, Velocity, fc and ft x 1e5, normal, SvM) and the FEM
 * tool (vtk_writer.cu:304-366: nodes, triangles, nodal temperature; with tl_ref
 * the tool moved back by its travel since its top-left point was at tl_ref,
 * vtk_writer.cu:518-587).  Vertex cells index the written points (the
 * reference indexes the full particle array, which points past the POINTS list
 * once particles are blanked).  sph_append_force_log appends the line
 * "%.9g %.9g\n" of sph_reduce_force (mfree_gpu.cpp:336-338). */
int sph_write_vtk_particles(sph_ctx *ctx, const char *path);
int sph_write_vtk_tool(sph_ctx *ctx, const char *path, const double *tl_ref);
/* vtk_writer.cu:368-516 (WEAR_NODE_SHIFT builds): the contact segments with
 * the wear statistics of the last step (see sph_set_wear). */
int sph_write_vtk_segments(sph_ctx *ctx, const char *path);
int sph_append_force_log(sph_ctx *ctx, const char *path);
/* The same three writers on host arrays (no context, no GPU): the calls above
 * download the state and use these.  Particles: pos, vel, fc, ft, n, S, p, T,
 * eps_pl, on_seg and blanked of *h.  Tool: nodes [n][2], nodal T, elements
 * [n][4] (a, b, c, colour), shift (NULL, or the top-left point's travel
 * since tl_ref).  Segments: left, right, normal [n][2]; phys_para [n][4],
 * sliding_force and wear_rate [n], all three NULL without wear statistics. */
int sph_vtk_write_particles_host(const sph_particles *h, const char *path);
int sph_vtk_write_tool_host(int32_t n_nodes, const double *position, const double *T, int32_t n_elements,
                            const int32_t *elements, const double *shift, const char *path);
int sph_vtk_write_segments_host(int32_t n_seg, const double *left, const double *right, const double *normal,
                                const double *phys_para, const double *sliding_force, const double *wear_rate,
                                const char *path);

/* ---- pipelined host I/O ------------------------------------------------------------
 * No counterpart in the reference.  For callers that feed a state in and read the
 * result out every step: the copies run on the context's own copy streams and return
 * at once, so the upload of the next state (into the particle buffer the last step
 * read, free once that step has finished) overlaps the download of the last result.
 * Every later call on the context -- the step included -- first waits for them;
 * sph_sync waits for everything.  Host arrays must stay untouched until then and be
 * page-locked for the copies to overlap.
 * sph_upload_particles_async takes the state fields only: p, R, S_der, v_der and idx
 * are recomputed by the step and must be NULL. */
int sph_upload_particles_async(sph_ctx *ctx, const sph_particles *host);
int sph_download_particles_async(sph_ctx *ctx, sph_particles *host);

/* ---- measurement hooks (output.cu:41-49 report_force; peak temperature) -- */
int sph_reduce_force(sph_ctx *ctx, double out[2]);     /* sum over particles of fc + ft */
int sph_reduce_max_T(sph_ctx *ctx, double *out);       /* max over non-blanked particles of T */

/* ---- batched multi-case runs ------------------------------------------------------
 * Many independent cutting cases advanced together: every case keeps its own
 * particles, FEM tool, tool velocity and time step; they share the material
 * and corrector constants, the smoothing length (cell geometry) and the
 * precision form (SPH_PREC_FP32K or SPH_PREC_FP64).  Each case is moved to its own
 * strip of one global cell grid (x offset, gaps wider than the stencil), so
 * every step stage runs as one launch over all cases and one CUDA graph per
 * step replays them all.  The tool of each case must already be placed
 * (positions in the case's own frame).  No counterpart call in the reference:
 * it runs one case per process (mfree_gpu.cpp:141-381). */
typedef struct sph_case_desc {
    const sph_particles *host;      /* particles of this case (case frame)            */
    const sph_tool_mesh *tool;      /* tool mesh of this case (case frame, placed)    */
    double dt;                      /* time step of this case                         */
    double tool_vel[2];             /* tool velocity (tool::set_vel)                  */
    double bbmin[2], bbmax[2];      /* this case's locked grid box (case frame)       */
} sph_case_desc;

/* `cell` gives the shared h, cell_factor and stencil; its bbmin/bbmax are
 * ignored (each case brings its own box).  Case k is moved by offset_k so
 * that its box starts at its own column range of the global grid and its
 * bottom lines up with the others; with cells of the same edge, a particle
 * sees the cells it sees in a single-case context on that box.  A particle
 * that leaves its case box stays in the global grid (a single-case grid sends
 * it to the overflow bucket); cases whose particles stay in their boxes do
 * not interact (the gap between cases is wider than the stencil). */
int sph_batch_create(const sph_constants *c, const sph_grid_params *cell, int32_t n_cases,
                     const sph_case_desc *cases, int32_t precision, int32_t device, sph_ctx **out);
/* Particle range [first, first+count) of case k in the concatenated arrays
 * before the first sort (cases are concatenated in order), the offset added
 * to the case's positions (x, y), and its first segment / FEM node and counts. */
int sph_batch_case_info(const sph_ctx *ctx, int32_t k, int32_t *first, int32_t *count, double offset[2],
                        int32_t *seg_first, int32_t *seg_count, int32_t *node_first, int32_t *node_count);
int sph_batch_n_cases(const sph_ctx *ctx, int32_t *n_cases);
/* Per case k: out[3k], out[3k+1] = sum of fc + ft over the case's particles
 * (report_force, output.cu:41-49), out[3k+2] = max T over its non-blanked
 * particles.  Works on single-case contexts too (n_cases = 1). */
int sph_batch_reduce(sph_ctx *ctx, double *out);
/* Case of every particle of the current (caller-visible) order, [N]. */
int sph_batch_case_of_particles(sph_ctx *ctx, int32_t *case_of);

/* ---- learned warm start of the return mapping -----------------------------------
 * No counterpart in the reference.  A 4-64-64-64-1 SiLU MLP (BF16 weights,
 * FP32 accumulation, tensor-core layers) predicts the plastic-multiplier
 * increment of a yielding trial state from x = (log(svm / A), eps_pl,
 * log(1 + eps_pl_dot / eps_dot_ref), (T - Tref) / (Tmelt - Tref)); its target
 * is t = log(2 G dl / |dev S_trial|).  Attached to an FP32K context, the
 * prediction replaces the reference's start dl0 = max(eps_pl_dot dt sqrt(2/3),
 * 1e-8) of the secant return mapping (actions_gpu.cu:724, plasticity.cuh:128-
 * 162), which still runs to the reference tolerance.
 * Parameter vector (SPH_MLP_NPARAMS floats): W1 [64][4], b1 [64], W2 [64][64],
 * b2 [64], W3 [64][64], b3 [64], W4 [64], b4 (W row-major [out][in]).  Inputs
 * and target are standardised with `norm` before the network.  Losses are
 * 0.5 (y - t)^2 in standardised units, averaged over the samples. */
#define SPH_MLP_NPARAMS 8705
typedef struct sph_mlp sph_mlp;
typedef struct sph_mlp_norm {
    float x_mean[4], x_std[4];
    float y_mean, y_std;
} sph_mlp_norm;

int sph_mlp_create(int32_t device, uint64_t seed, sph_mlp **out);       /* uniform(+-1/sqrt(fan_in)) init */
int sph_mlp_destroy(sph_mlp *m);
const char *sph_mlp_last_error(const sph_mlp *m);
int sph_mlp_get_params(sph_mlp *m, float *params, sph_mlp_norm *norm);  /* NULL outputs skipped */
int sph_mlp_set_params(sph_mlp *m, const float *params, const sph_mlp_norm *norm);
int sph_mlp_fit_norm(sph_mlp *m, const float *x, const float *t, int64_t n);   /* moments of the data */
int sph_mlp_predict(sph_mlp *m, const float *x, int64_t n, float *y);  /* host x [n][4] -> host y [n] */
/* The same through the warp-per-sample form the fused step runs in its epilogue (SPH_MLP_WARP). */
int sph_mlp_predict_warp(sph_mlp *m, const float *x, int64_t n, float *y);
/* Gradient of the mean loss over the n samples (host in/out; grad [SPH_MLP_NPARAMS]). */
int sph_mlp_gradients(sph_mlp *m, const float *x, const float *t, int64_t n, float *grad, float *loss);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the gradient of these n samples. */
int sph_mlp_adam_step(sph_mlp *m, const float *x, const float *t, int64_t n, float lr, float *loss);
/* Minibatch Adam over `epochs` shuffled passes (seeded); epoch_loss [epochs] = mean loss of each pass. */
int sph_mlp_train(sph_mlp *m, const float *x, const float *t, int64_t n, int32_t epochs, int32_t batch, float lr,
                  uint64_t seed, float *epoch_loss);

/* Return-mapping log: every yielding return mapping of the fused step appends
 * (svm, eps_pl, eps_pl_dot, T, |dev S_trial|, dl, secant iterations, dt) as 8
 * floats while fewer than `capacity` records are held; capacity 0 turns it off. */
int sph_jc_log_enable(sph_ctx *ctx, int64_t capacity);
int sph_jc_log_read(sph_ctx *ctx, float *records, int64_t max_records, int64_t *n_offered);
/* Counters of return mappings and secant iterations (enable 1/0; out[2] may
 * be NULL; reset zeroes them after the read). */
int sph_jc_stats(sph_ctx *ctx, int32_t enable, int64_t *out, int32_t reset);
/* Copies the network into the context and starts the return mappings of the
 * fused FP32K step from its prediction; NULL detaches. */
int sph_mlp_attach(sph_ctx *ctx, const sph_mlp *m);
/* Where the attached network runs in the fused step:
 * SPH_MLP_WARP (default) -- inside the neighbour-sum kernel's epilogue: a warp
 *   with yielding particles runs one warp-wide forward pass per such particle
 *   on the CUDA cores (BF16 weights, FP32 sums), no extra launch;
 * SPH_MLP_TENSOR -- yielding particles are queued and a second kernel runs the
 *   hidden layers on the tensor cores, 128 particles per tile.
 * Both then run the same secant to the reference tolerance. */
#define SPH_MLP_WARP 0
#define SPH_MLP_TENSOR 1
int sph_mlp_set_inference(sph_ctx *ctx, int32_t mode);

/* ---- launch shapes -------------------------------------------------------------
 * No counterpart in the reference (its launches are fixed at 256 threads).
 * The fused FP32K neighbour-sum kernel is compiled for several launch shapes
 * (threads per block, minimum resident blocks per SM, and the number of
 * neighbour records a block stages in shared memory -- 0 for global loads);
 * an autotuner times the step with each and sets the fastest.  Variant 0 is
 * the default.  Shapes with lanes_per_particle > 1 (for small systems, which
 * leave most of the GPU idle) let that many lanes share a particle's
 * candidates and merge their compensated sums.
 * step_form: SPH_STEP_LAUNCHES (default) -- the fused step as its chain of
 * launches (scan, scatter, rank, gather, FEM, neighbour sums, tool, contact,
 * tail), replayed from a CUDA graph; SPH_STEP_PERSISTENT -- the same stages in
 * one cooperative launch with every block resident, separated by bounded
 * grid-wide barriers (SPH_STATUS_GRID_TIMEOUT if one gives up), captured in the
 * graph the same way; the same results bit for bit.  FP32K contexts only; a
 * step it does not cover (the first one after an FP64 upload, wear, the rigid
 * tool, PSE conduction, SPH_MLP_TENSOR) runs as launches.  The neighbour sums
 * of the persistent form use 128-particle blocks (interact_variant is ignored). */
#define SPH_STEP_LAUNCHES 0
#define SPH_STEP_PERSISTENT 1
typedef struct sph_launch_config {
    int32_t interact_variant;
    int32_t step_form;
} sph_launch_config;
/* *n: in, capacity of the output arrays (each may be NULL); out, number of variants. */
int sph_launch_variants(int32_t *n, int32_t *block, int32_t *min_blocks, int32_t *staged_records,
                        int32_t *lanes_per_particle);
int sph_set_launch_config(sph_ctx *ctx, const sph_launch_config *cfg);
int sph_get_launch_config(const sph_ctx *ctx, sph_launch_config *cfg);

/* ---- failure paths under test -----------------------------------------------------
 * No counterpart in the reference.  Lets a test drive the bounded waits and the
 * secant cap into their failure paths without a fault: with
 * SPH_TEST_SKIP_BULK_COPY the staged neighbour sums announce their record
 * copies but issue none, so the wait runs out after 1 s, the step reports
 * SPH_STATUS_COPY_TIMEOUT and falls back to global loads (same results); with
 * SPH_TEST_SKIP_MMA the learned warm start issues no tensor-core MMA, so its
 * wait runs out, it reports SPH_STATUS_MMA_TIMEOUT, frees its TMEM and leaves
 * the return mappings of that step undone; with SPH_TEST_SKIP_GRID_ARRIVAL
 * block 0 of the persistent step does not arrive at its first grid barrier,
 * so every block's wait runs out, the step reports SPH_STATUS_GRID_TIMEOUT
 * and the launch ends (that step's results are not usable).  secant_cap >= 0 replaces the
 * reference's cap of the return mapping's secant iterations (it stops with
 * SPH_STATUS_SECANT_MAXITER once the iteration counter exceeds the cap: 100
 * in the reference, plasticity.cuh:155-158); < 0 restores it.  faults = 0 and
 * secant_cap = -1 is normal operation. */
#define SPH_TEST_SKIP_BULK_COPY (1u << 0)
#define SPH_TEST_SKIP_MMA       (1u << 1)
#define SPH_TEST_SKIP_GRID_ARRIVAL (1u << 2)
int sph_set_test_faults(sph_ctx *ctx, uint32_t faults, int32_t secant_cap);

/* ---- per-stage timing ---------------------------------------------------------
 * Runs `nsteps` fused steps without the CUDA graph, with CUDA events on the
 * context stream between the stages; stage_ms[k] receives the summed device
 * time of stage k over the steps: 0 histogram/hash (previous step's tail when
 * chained), 1 scan+scatter+rank, 2 reorder gather (+predict, EOS, artificial
 * stress, records), 3 FEM half step (+ PSE conduction), 4 neighbour sums +
 * fused epilogue (+ wear statistics reset, warm-started return mapping),
 * 5 FEM rate/update (+ wear adjustment) + tool move (+ rigid tool move),
 * 6 contact/BC/invalidate tail (+ next histogram).  The steps are the same
 * as those of sph_step_fused.  n_stages receives 7. */
int sph_profile_steps(sph_ctx *ctx, int32_t nsteps, float *stage_ms, int32_t *n_stages);

/* ---- tool wear by nodal shift (WEAR_NODE_SHIFT) --------------------------------
 * The reference's wear path of the FEM-tool step (types.h:25):
 *  - every step the segment statistics are reset (segments_wear_rate_reset,
 *    tool_FEM.cu:1595-1609) and the friction-heat kernel adds, per contact
 *    segment, the count, contact pressure, sliding speed, segment temperature
 *    and sliding force of its particles (actions_gpu.cu:401-419);
 *  - once wear is switched on (the reference's `wear_pro`, mfree_gpu.cpp:300),
 *    wear_adjustment (actions_gpu.cu:1009-1020) runs after the return mapping:
 *    the elements of the two cutting-edge layers leave the lumped mass and
 *    stiffness (mesh_retreat_wear, FEM_thermal_gpu.cu:923-936), the cutting-edge
 *    nodes move along the segment normals by the Usui rake/flank wear
 *    (do_nodal_shift_wear_smooth_temp with RESTRICT_WEAR_TEMP and
 *    USE_USUI_RAKE_FLANK, tool_FEM.cu:299-432), the layers return at the new
 *    node positions (mesh_resume_wear), the segments follow the nodes
 *    (do_segment_wear_update, tool_FEM.cu:520-545), the flank correction sets
 *    flank_retreat (do_correct_flank_contact, tool_FEM.cu:559-587) and the
 *    lumped inverse mass is rebuilt (FEM_thermal_gpu.cu:326-331,838-844).
 * The gmsh remesh of the reference's main loop is not part of this (no gmsh).
 * Single-case contexts with a FEM tool only. */
typedef struct sph_wear_constants {   /* constants_structs.h:113-119 */
    double A, B, C, D;                /* flank: A, B; rake (|n.x| > 0.85): C, D */
} sph_wear_constants;

#define SPH_WEAR_OFF 0          /* build without WEAR_NODE_SHIFT */
#define SPH_WEAR_ACCUMULATE 1   /* WEAR_NODE_SHIFT, wear_pro false: segment statistics only */
#define SPH_WEAR_SHIFT 2        /* WEAR_NODE_SHIFT, wear_pro true: statistics + wear_adjustment each step */

int sph_set_wear(sph_ctx *ctx, int32_t mode, const sph_wear_constants *wc);

/* Host view of the wear state (any pointer may be NULL to skip that field). */
typedef struct sph_wear_state {
    int32_t n_elements, n_seg;
    int32_t *elements;        /* [n_elements][4] node a, b, c, colour (mesh_GPU_m::node_num) */
    int32_t *layer;           /* [n_elements][2] cutting_boundary_layer: layer 1, layer 2 */
    double *M;                /* [n_nodes] lumped mass (m_mass_matrix, after Dirichlet) */
    double *phys_para;        /* [n_seg][4] count, sum pressure, sum sliding speed, sum segment T */
    double *sliding_force;    /* [n_seg] */
    double *wear_nodes;       /* [n_seg] wear rate of the segment (left + right) / dt */
} sph_wear_state;
int sph_download_wear(sph_ctx *ctx, sph_wear_state *host);
int sph_upload_wear(sph_ctx *ctx, const sph_wear_state *host);   /* M, phys_para, sliding_force, wear_nodes */

/* Stage entry points: m_tool->segments_wear_rate_reset() (leap_frog.cu:183-186)
 * and wear_adjustment(m_tool) (leap_frog.cu:224-229). */
int sph_segments_wear_rate_reset(sph_ctx *ctx);
/* remesh_low_level(tool_FEM*, freq) (tool_FEM.cu:1696-1705), the remesh of the
 * worn tool without gmsh (mfree_gpu.cpp:356): the mesh nodes on neither the
 * cutting nor the fixed edge are shifted with the flank wear (do_mesh_shift,
 * tool_FEM.cu:589-616, scaled by freq), the thermal system is assembled again
 * on the moved mesh (stiffness, lumped mass, Dirichlet, inverse mass), and every
 * node's temperature is interpolated from the old mesh
 * (do_nodal_value_interpolation_old, tool_FEM.cu:57-107,434-443).  Single-case
 * contexts with a FEM tool. */
int sph_remesh_low_level(sph_ctx *ctx, int32_t freq);
int sph_wear_adjustment(sph_ctx *ctx);

/* ---- cell-list build that allocates nothing ------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * when they need a cell list: a host application whose own memory manager
 * owns all device memory, a latency-critical loop that cannot afford an
 * allocation's synchronisation, a recovery path that must work when device
 * memory is exhausted.
 *
 * Computes the same results as sph_assign_hashes + sph_sort
 * (compute_hashes + stable sort_by_key + cell tables, grid.cu:25-42,
 * grid_gpu_green.cu:13-115,185-209) for device arrays the caller owns:
 *  - pos [n][2], blanked [n]: inputs;
 *  - hash [n]: in/out; recomputed for non-blanked particles, kept (stale)
 *    for blanked ones;
 *  - perm [n]: sorted position -> original index;
 *  - hash_sorted [n]: optional (NULL to skip);
 *  - cell_start / cell_end [g->num_cell]: cell_end is left untouched for
 *    empty cells.
 * Particles outside the grid (and blanked particles whose stale hash lies
 * outside [0, num_cell)) go to one trailing bucket after every cell, in
 * original-index order, exactly as in the allocating path; unlike that path,
 * this call raises no status bit for them (SPH_STATUS_OUT_OF_GRID) nor for
 * crowded cells (SPH_STATUS_CELL_OVERFLOW).  The in-cell ranking costs the
 * square of a bucket's size, so many out-of-grid particles make it slow.
 * Scratch is a fixed file-scope device array (about 5.2 MB held by every GPU
 * that loads the library).  Limits: n <= 262144 particles and
 * g->num_cell <= 262143 cells; larger sizes return SPH_ERR_INVALID with a
 * message in err (err_len bytes, may be NULL).  The first call in each CUDA
 * context (the device's primary context, or one the caller created with the
 * driver API and made current) looks up the array's address in that context;
 * make it before any stream capture.  The lookup is cached per context, so a
 * context created later (also after cudaDeviceReset) gets its own.
 * All calls share the scratch, so calls that overlap on the GPU race:
 * serialise them.  Work is queued on `stream` (cudaStream_t, NULL = default
 * stream); the call does not synchronise. */
int sph_cells_build_noalloc(const double *pos, const double *blanked, int32_t *hash, int32_t n,
                            const sph_geom_constants *g, int32_t *perm, int32_t *hash_sorted,
                            int32_t *cell_start, int32_t *cell_end, void *stream, char *err, int32_t err_len);

/* ---- kernel launch accounting ---------------------------------------------- */
int sph_launch_count(const sph_ctx *ctx, int64_t *count);   /* kernels launched by this context */

#ifdef __cplusplus
}
#endif

#endif /* SPHFEM_H */
