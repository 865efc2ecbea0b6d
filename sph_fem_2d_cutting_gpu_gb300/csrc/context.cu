// context.cu -- the C ABI (include/sphfem.h): context, data movement, the
// stage entry points that mirror the calls of leap_frog::step
// (leap_frog.cu:162-248) and the fused, graph-captured step.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "launch.cuh"
#include "mlp_host.h"
#include "toolsetup.h"

using namespace sphfem;

// Particle-state buffers: two for stepping; four once pipelined host I/O is
// used, so that the upload of the next request, the current step and the
// download of the last result each have a buffer of their own and the two copy
// directions run at the same time.
constexpr int kBufs = 4;

struct sph_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int N = 0;
    KConsts K{};
    sph_grid_params grid{};
    SortedFields buf[kBufs]{};           // the third and fourth only once pipelined I/O is used
    int nbuf = 2;
    int cur = 0;                         // buf[cur] holds the particle state
    int last_in = -1;                    // the buffer the last step read
    FixedFields F{};
    // FP32K contexts: the compact FP32 state the fused step reads and writes, one
    // per particle buffer, and which form of each buffer holds its state.  The
    // FP64 arrays (the caller-visible particle_gpu layout) are filled from the
    // compact ones on demand (sync64) before any call that reads or writes them.
    SortedFields32 c32[kBufs]{};
    FixedFields32 F32{};
    bool v64[kBufs] = {true, true, true, true};   // buf[b] holds buffer b's state
    bool v32[kBufs] = {};                          // c32[b] holds it
    bool pr64 = true, pr32 = false;                // F / F32 hold the newest p and R
    SortScratch X{};
    StepScratch W{};
    bool counts_valid = false;           // X.key/arrival/counts match the current state
    // tool
    bool has_tool = false;
    ToolModelHost tool_host;
    SegDev seg{};
    FemDev fem{};
    ToolDev *tool_dev = nullptr;
    int4 *fem_elements = nullptr;        // tool elements: nodes a, b, c and colour
    int32_t *fem_dir_elems = nullptr;    // the Dirichlet elimination's order (elements, fixed-edge flags)
    int4 *fem_dir_flags = nullptr;
    int fem_n_dir = 0;
    int32_t *fem_node_edge = nullptr;    // remesh: per node, on a cutting (1) / fixed (2) edge
    double2 *fem_pos_old = nullptr;      // remesh: the mesh and temperatures before the shift
    double *fem_T_map = nullptr;
    double *fem_T_old = nullptr, *fem_f_temp = nullptr, *fem_K_temp = nullptr;
    // graphs, one per buffer parity
    // [input buffer][output buffer][FP32K: input in the compact form][FP32K: p, R from F32]
    cudaGraphExec_t graph[kBufs][kBufs][2][2] = {};
    int64_t graph_launches[kBufs][kBufs][2][2] = {};
    bool use_graph = true;
    int64_t launches = 0;
    double *h_reduce = nullptr;          // pinned
    bool in_cell_order = false;          // the state is in the order of the last sort (X.offsets)
    // batched contexts (one case otherwise): per-case ranges and offsets
    std::vector<int32_t> case_first, case_count, case_seg_first, case_seg_count, case_node_first, case_node_count;
    std::vector<double> case_offset;                 // [n_cases][2]
    std::vector<uint16_t> case_of_col_h;             // [nx]
    int32_t *case_cell_bound = nullptr;              // [n_cases + 1] first cell of each case's columns
    int32_t *case_part_bound = nullptr;              // [n_cases + 1] prefix of case particle counts
    double *case_reduce = nullptr;                   // [n_cases][3]
    // return-mapping log / statistics / learned warm start
    int num_sms = 0;
    float *jc_log = nullptr;
    unsigned long long *jc_log_count = nullptr;
    int64_t jc_log_cap = 0;
    unsigned long long *jc_stats = nullptr;
    int32_t *jc_list = nullptr, *jc_list_count = nullptr;
    float *mlp_params = nullptr;
    uint16_t *mlp_wb = nullptr;
    MlpDev mlp{};
    bool mlp_on = false;
    int mlp_mode = SPH_MLP_WARP;   // sph_mlp_set_inference
    int interact_variant = 0;            // launch shape of the fused FP32K neighbour sums
    int step_form = SPH_STEP_LAUNCHES;   // the fused step as a chain of launches or one persistent launch
    unsigned *grid_bar = nullptr;        // [4] the persistent step's grid barrier
    double *usui_scratch = nullptr;      // per-block partials of sph_eval_usui
    sph_rigid_tool *rigid_dev = nullptr; // the rigid tool, moved on the device every step (NULL: none)
    // wear by nodal shift (WEAR_NODE_SHIFT): SPH_WEAR_* mode, device layer data
    int wear_mode = SPH_WEAR_OFF;
    bool wear_ready = false;
    WearDev wear{};
    dbl4 *wear_pp = nullptr;             // per-segment statistics (seg.wear points here while wear is on)
    double *wear_sf = nullptr;
    // pipelined host I/O: uploads into a free particle buffer and downloads run on
    // their own streams, ordered per buffer by events; a step waits only for the
    // copies into its input and out of its output buffer
    cudaStream_t io_up = nullptr, io_down = nullptr;
    cudaEvent_t ev_used[kBufs] = {}, ev_up[kBufs] = {}, ev_down[kBufs] = {}, ev_fixed = nullptr;
    bool up_pending[kBufs] = {}, down_pending[kBufs] = {}, fixed_pending = false;
    int64_t down_seq[kBufs] = {}, n_downloads = 0;   // issue order of each buffer's last download
    std::vector<void *> allocs;
    std::string err;
};

namespace {

const char *g_no_ctx = "no context";

int fail(sph_ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return fail(ctx, SPH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));         \
    } while (0)

#define CK_LAUNCH()                                                                                    \
    do {                                                                                               \
        cudaError_t e_ = cudaGetLastError();                                                           \
        if (e_ != cudaSuccess) return fail(ctx, SPH_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e_)); \
    } while (0)

template <class T>
int dalloc(sph_ctx *ctx, T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * count);
    if (e != cudaSuccess) return fail(ctx, SPH_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    ctx->allocs.push_back((void *)*p);
    return SPH_OK;
}

// Makes the compute stream wait for the pending copies into (upload) / out of
// (download) buffer b, or for every pending copy with b < 0.
int wait_io(sph_ctx *ctx, int b) {
    for (int i = 0; i < kBufs; i++) {
        if (b >= 0 && i != b) continue;
        if (ctx->up_pending[i]) {
            CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_up[i], 0));
            ctx->up_pending[i] = false;
        }
        if (ctx->down_pending[i]) {
            CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_down[i], 0));
            ctx->down_pending[i] = false;
        }
    }
    if (ctx->fixed_pending) {   // downloads of p, R, S_der, v_der, idx (written by every step)
        CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_fixed, 0));
        ctx->fixed_pending = false;
    }
    return SPH_OK;
}

int join_io(sph_ctx *ctx) { return wait_io(ctx, -1); }

// After compute that used buffers a and b: mark the point on the compute stream.
int mark_used(sph_ctx *ctx, int a, int b) {
    if (!ctx->io_up) return SPH_OK;
    CK(cudaEventRecord(ctx->ev_used[a], ctx->stream));
    if (b != a) CK(cudaEventRecord(ctx->ev_used[b], ctx->stream));
    return SPH_OK;
}

// The buffer a step (or sort) reading buf[cur] writes: one whose copies are not
// in flight if there is one, else the lowest other index (the step then waits).
int pick_out(const sph_ctx *ctx) {
    int fallback = -1;
    for (int b = 0; b < ctx->nbuf; b++) {
        if (b == ctx->cur) continue;
        if (fallback < 0) fallback = b;
        if (!ctx->up_pending[b] && !ctx->down_pending[b]) return b;
    }
    return fallback;
}

#define DALLOC(p, n)                          \
    do {                                      \
        int r_ = dalloc(ctx, &(p), (n));      \
        if (r_ != SPH_OK) return r_;          \
    } while (0)

void geometry_from(const sph_grid_params &g, sph_geom_constants &out) {
    // grid.cu:130-149 set_geometry (locked grid); cell edge = h * cell_factor
    double bbmin_x = g.bbmin[0] - 1e-6, bbmin_y = g.bbmin[1] - 1e-6;
    double bbmax_x = g.bbmax[0] + 1e-6, bbmax_y = g.bbmax[1] + 1e-6;
    double kernel_width = 2.;
    double dx = g.h * kernel_width / 2. * (double)g.cell_factor;
    unsigned int nx = (unsigned int)ceil((bbmax_x - bbmin_x) / dx);
    unsigned int ny = (unsigned int)ceil((bbmax_y - bbmin_y) / dx);
    out.nx = (int)nx;
    out.ny = (int)ny;
    out.bbmin_x = bbmin_x;
    out.bbmin_y = bbmin_y;
    out.dx = dx;
    out.num_cell = (int)(nx * ny);
    out.stencil = g.stencil;
}

void derive(KConsts &K) {
    double c0 = (double)sqrtf((float)(K.c.phys.K / K.c.phys.rho0));   // actions_gpu.cu:228 (float sqrt)
    K.c0sq = c0 * c0;
    K.inv_wdeltap = 1. / K.c.corr.wdeltap;
    K.eta2 = K.c.corr.eta * K.c.corr.eta;
    K.inv_dx = 1. / K.g.dx;
    K.thermal_bc = (K.c.trml_tool.alpha != 0.) ? 1 : 0;
    KF32 &f = K.f;
    f.mass = (float)K.c.phys.mass;
    f.inv_mass = (float)(1.0 / K.c.phys.mass);
    f.xs_mass = (float)K.c.corr.xspheps * f.mass;
    f.alpha = (float)K.c.corr.alpha;
    f.beta = (float)K.c.corr.beta;
    f.eta2 = (float)K.eta2;
    f.inv_wdp = (float)K.inv_wdeltap;
    f.cell = (float)K.g.dx;
    f.inv_cell = (float)(1.0 / K.g.dx);
    f.G = (float)K.c.phys.G;
    f.K_bulk = (float)K.c.phys.K;
    f.c0sq = (float)K.c0sq;
    f.stresseps = (float)K.c.corr.stresseps;
    f.dt = (float)K.dt;
    f.hdt = (float)(0.5 * K.dt);
    f.inv_dt = (float)(1.0 / K.dt);
    f.tq_over_cp = K.c.trml_wp.cp != 0. ? (float)(K.c.trml_wp.tq / K.c.trml_wp.cp) : 0.f;
    f.alpha_wp = (float)K.c.trml_wp.alpha;
    f.alpha_tool_sph = (float)K.c.trml_tool_sph.alpha;
    f.T_init = (float)K.c.trml_wp.T_init;
    const sph_joco_constants &jc = K.c.joco;
    f.jc.A = (float)jc.A; f.jc.B = (float)jc.B; f.jc.C = (float)jc.C; f.jc.n = (float)jc.n; f.jc.m = (float)jc.m;
    f.jc.Tref = (float)jc.Tref;
    f.jc.inv_dT = (float)(1.0 / (jc.Tmelt - jc.Tref));
    f.jc.inv_epsdot_ref = (float)(1.0 / jc.eps_dot_ref);
    f.jc.Tmelt = (float)jc.Tmelt;
}

void set_case_dt(ToolDev &td, double dt) {
    td.dt = dt;
    td.hdt = 0.5 * dt;
    td.dtf = (float)dt;
    td.hdtf = (float)(0.5 * dt);
    td.inv_dtf = (float)(1.0 / dt);
}

void invalidate_graphs(sph_ctx *ctx) {
    for (int a = 0; a < kBufs; a++)
        for (int b = 0; b < kBufs; b++)
            for (int c = 0; c < 2; c++)
                for (int d = 0; d < 2; d++)
                    if (ctx->graph[a][b][c][d]) {
                        cudaGraphExecDestroy(ctx->graph[a][b][c][d]);
                        ctx->graph[a][b][c][d] = nullptr;
                    }
}

// Field descriptors for upload/download of the caller-visible view.
struct FieldDesc {
    size_t off_view;      // offset of the double*/int* member in sph_particles
    int width;            // 8-byte (or 4-byte for ints) words per particle
    bool is_int;
};

sph_particles view_of_buf(const sph_ctx *ctx, int b) {
    const SortedFields &A = ctx->buf[b];
    sph_particles v;
    std::memset(&v, 0, sizeof(v));
    v.N = ctx->N;
    v.pos = (double *)A.pos; v.vel = (double *)A.vel; v.h = A.h; v.rho = A.rho; v.p = ctx->F.p;
    v.S = (double *)A.S; v.R = (double *)ctx->F.R; v.fc = (double *)A.fc; v.ft = (double *)A.ft; v.n = (double *)A.n;
    v.fixed = A.fixed; v.blanked = A.blanked; v.tool_particle = A.tool_particle;
    v.eps_pl = A.eps_pl; v.eps_pl_dot = A.eps_pl_dot; v.T = A.T;
    v.pos_t = (double *)A.pos_t; v.vel_t = (double *)A.vel_t; v.rho_t = A.rho_t; v.S_t = (double *)A.S_t; v.T_t = A.T_t;
    v.S_der = (double *)ctx->F.S_der; v.v_der = (double *)ctx->F.v_der;
    v.idx = ctx->F.idx; v.hash = A.hash; v.on_seg = A.on_seg;
    return v;
}

sph_particles view_of(const sph_ctx *ctx) { return view_of_buf(ctx, ctx->cur); }

const FieldDesc kFields[] = {
    {offsetof(sph_particles, pos), 2, false},   {offsetof(sph_particles, vel), 2, false},
    {offsetof(sph_particles, h), 1, false},     {offsetof(sph_particles, rho), 1, false},
    {offsetof(sph_particles, p), 1, false},     {offsetof(sph_particles, S), 4, false},
    {offsetof(sph_particles, R), 4, false},     {offsetof(sph_particles, fc), 2, false},
    {offsetof(sph_particles, ft), 2, false},    {offsetof(sph_particles, n), 2, false},
    {offsetof(sph_particles, fixed), 1, false}, {offsetof(sph_particles, blanked), 1, false},
    {offsetof(sph_particles, tool_particle), 1, false}, {offsetof(sph_particles, eps_pl), 1, false},
    {offsetof(sph_particles, eps_pl_dot), 1, false},    {offsetof(sph_particles, T), 1, false},
    {offsetof(sph_particles, pos_t), 2, false}, {offsetof(sph_particles, vel_t), 2, false},
    {offsetof(sph_particles, rho_t), 1, false}, {offsetof(sph_particles, S_t), 4, false},
    {offsetof(sph_particles, T_t), 1, false},   {offsetof(sph_particles, S_der), 4, false},
    {offsetof(sph_particles, v_der), 4, false}, {offsetof(sph_particles, idx), 1, true},
    {offsetof(sph_particles, hash), 1, true},   {offsetof(sph_particles, on_seg), 1, true},
};

template <class M>
M member(const sph_particles &v, size_t off) {
    return *(const M *)((const char *)&v + off);
}

int alloc_sorted(sph_ctx *ctx, SortedFields &S, int N) {
    DALLOC(S.pos, N); DALLOC(S.vel, N); DALLOC(S.fc, N); DALLOC(S.ft, N); DALLOC(S.n, N);
    DALLOC(S.h, N); DALLOC(S.rho, N); DALLOC(S.eps_pl, N); DALLOC(S.eps_pl_dot, N); DALLOC(S.T, N);
    DALLOC(S.fixed, N); DALLOC(S.blanked, N); DALLOC(S.tool_particle, N); DALLOC(S.S, N);
    DALLOC(S.pos_t, N); DALLOC(S.vel_t, N); DALLOC(S.rho_t, N); DALLOC(S.T_t, N); DALLOC(S.S_t, N);
    DALLOC(S.on_seg, N); DALLOC(S.hash, N);
    return SPH_OK;
}

int alloc_sorted32(sph_ctx *ctx, SortedFields32 &S, int N) {
    DALLOC(S.pos, N); DALLOC(S.vel, N); DALLOC(S.fc, N); DALLOC(S.ft, N); DALLOC(S.n, N);
    DALLOC(S.h, N); DALLOC(S.rho, N); DALLOC(S.eps_pl, N); DALLOC(S.eps_pl_dot, N); DALLOC(S.T, N);
    DALLOC(S.fixed, N); DALLOC(S.blanked, N); DALLOC(S.tool_particle, N); DALLOC(S.S, N);
    DALLOC(S.pos_t, N); DALLOC(S.vel_t, N); DALLOC(S.rho_t, N); DALLOC(S.T_t, N); DALLOC(S.S_t, N);
    DALLOC(S.on_seg, N); DALLOC(S.hash, N);
    return SPH_OK;
}

// FP32K contexts: makes the FP64 arrays of the current buffer (and F.p, F.R)
// hold the state, widening the compact form into them if a fused step left it
// there.  `modify`: the caller may change the FP64 state, so the compact form
// (and F32's p, R) no longer count and the next fused step starts from FP64.
int sync64(sph_ctx *ctx, bool modify) {
    if (ctx->K.precision != SPH_PREC_FP32K) return SPH_OK;
    const int b = ctx->cur;
    if (!ctx->v64[b] || !ctx->pr64) {
        int r = wait_io(ctx, b);   // copies into or out of buf[b] still in flight
        if (r) return r;
        launch_state_to64(ctx->stream, ctx->N, ctx->c32[b], ctx->F32, ctx->buf[b], ctx->F, !ctx->v64[b],
                          !ctx->pr64);
        ctx->launches++;
        CK_LAUNCH();
        ctx->v64[b] = true;
        ctx->pr64 = true;
    }
    if (modify) {
        ctx->v32[b] = false;
        ctx->pr32 = false;
    }
    return SPH_OK;
}

int zero_all(sph_ctx *ctx) {
    sph_particles v = view_of(ctx);
    for (const FieldDesc &fd : kFields) {
        void *dst = member<void *>(v, fd.off_view);
        size_t bytes = (size_t)ctx->N * fd.width * (fd.is_int ? 4 : 8);
        CK(cudaMemsetAsync(dst, 0, bytes, ctx->stream));
    }
    return SPH_OK;
}

// Copy streams, per-buffer events and the third and fourth particle buffers of
// pipelined I/O.
int ensure_io(sph_ctx *ctx) {
    if (ctx->io_up) return SPH_OK;
    for (int b = 2; b < kBufs; b++) {
        int r = alloc_sorted(ctx, ctx->buf[b], ctx->N);
        if (!r && ctx->K.precision == SPH_PREC_FP32K) r = alloc_sorted32(ctx, ctx->c32[b], ctx->N);
        if (r) return r;
    }
    ctx->nbuf = kBufs;
    CK(cudaStreamCreateWithFlags(&ctx->io_up, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&ctx->io_down, cudaStreamNonBlocking));
    for (int b = 0; b < kBufs; b++) {
        CK(cudaEventCreateWithFlags(&ctx->ev_used[b], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ctx->ev_up[b], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&ctx->ev_down[b], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&ctx->ev_fixed, cudaEventDisableTiming));
    // the buffers' last users are whatever the compute stream has queued so far
    for (int b = 0; b < kBufs; b++) CK(cudaEventRecord(ctx->ev_used[b], ctx->stream));
    return SPH_OK;
}

// ---- staged FEM helpers ----------------------------------------------------------------
int ensure_fem_temp(sph_ctx *ctx) {
    if (ctx->fem_T_old) return SPH_OK;
    DALLOC(ctx->fem_T_old, ctx->fem.n_nodes);
    DALLOC(ctx->fem_f_temp, ctx->fem.n_nodes);
    DALLOC(ctx->fem_K_temp, ctx->fem.nnz);
    return SPH_OK;
}

#define REQUIRE_CTX()                            \
    if (!ctx) return SPH_ERR_INVALID;            \
    {                                            \
        int jr_ = join_io(ctx);                  \
        if (jr_ != SPH_OK) return jr_;           \
    }
// Calls that read (modify false) or may write (modify true) the particle state
// through the FP64 arrays.
#define REQUIRE_STATE(modify)                    \
    {                                            \
        int sr_ = sync64(ctx, modify);           \
        if (sr_ != SPH_OK) return sr_;           \
    }
#define REQUIRE_TOOL() \
    if (!ctx->has_tool) return fail(ctx, SPH_ERR_STATE, "context has no tool");
// Calls that take one time step or one tool for the whole context.
#define REQUIRE_SINGLE_CASE() \
    if (ctx->K.n_cases > 1) return fail(ctx, SPH_ERR_STATE, "batched context: only the fused step runs per case");

SortedFields &CUR(sph_ctx *ctx) { return ctx->buf[ctx->cur]; }

// CTAs of the warm-started return mapping: persistent, about 4 per SM.
int jc_warm_grid(const sph_ctx *ctx) {
    int tiles = (ctx->N + 127) / 128;
    return std::max(1, std::min(tiles, 4 * std::max(ctx->num_sms, 1)));
}

// The PSE conduction sum runs in this step (interactions_heat_pse returns at
// once without workpiece conduction, interactions_gpu.cu:434-435).
bool pse_active(const sph_ctx *ctx) { return ctx->K.thermal_pse && ctx->K.c.trml_wp.alpha != 0.; }

// The fused step body (everything after the histogram of the current state),
// reading buf[cur] and writing buf[w] -- in FP32K contexts the compact form
// c32[w], from c32[cur] when it holds the state (v32) and buf[cur] otherwise.
// ev (profiling, may be null): events recorded after the sort, the reorder, the
// FEM half step + PSE, the neighbour sums, the tool updates and the tail
// (ev[0..5]).
// The persistent form covers this step: FP32K from the compact state, no wear,
// rigid tool or PSE conduction, the warm start (if any) in its in-epilogue form.
bool persistent_step(const sph_ctx *ctx) {
    return ctx->step_form == SPH_STEP_PERSISTENT && ctx->grid_bar && ctx->K.precision == SPH_PREC_FP32K &&
           ctx->v32[ctx->cur] && ctx->pr32 && !ctx->K.rigid && !pse_active(ctx) && ctx->wear_mode == SPH_WEAR_OFF &&
           !(ctx->mlp_on && ctx->mlp_mode == SPH_MLP_TENSOR);
}

int issue_fused_body(sph_ctx *ctx, int64_t &n, int w, cudaEvent_t *ev = nullptr) {
    const int N = ctx->N;
    cudaStream_t s = ctx->stream;
    const bool f32 = ctx->K.precision == SPH_PREC_FP32K;
    SortedFields &A = ctx->buf[ctx->cur];
    SortedFields &B = ctx->buf[w];
    SortedFields32 &B32 = ctx->c32[w];
    if (!ev && persistent_step(ctx)) {   // the per-stage profile keeps the separate launches
        PersistArgs P;
        P.N = N;
        P.K = ctx->K;
        P.X = ctx->X;
        P.A = ctx->c32[ctx->cur];
        P.B = B32;
        P.F32 = ctx->F32;
        P.perm = ctx->F.idx;
        P.W = ctx->W;
        P.seg = ctx->seg;
        P.fem = ctx->fem;
        P.tool = ctx->tool_dev;
        P.mlp = ctx->mlp;
        P.bar = ctx->grid_bar;
        CK(launch_step_persistent(s, P, ctx->has_tool, ctx->mlp_on, ctx->num_sms));
        n += 1;
        CK_LAUNCH();
        return SPH_OK;
    }
    launch_sort_rest(s, N, ctx->X, ctx->K.g, ctx->F.idx, ctx->W.status);
    n += 5;
    if (ev) CK(cudaEventRecord(ev[0], s));
    if (f32)
        launch_gather_fused32(s, N, ctx->F.idx, ctx->K, ctx->v32[ctx->cur] ? nullptr : &A,
                              ctx->v32[ctx->cur] ? &ctx->c32[ctx->cur] : nullptr, ctx->pr32, ctx->F, ctx->F32, B32,
                              ctx->F.idx, ctx->W, ctx->X.hash_next, ctx->tool_dev);
    else
        launch_gather_fused(s, N, ctx->F.idx, ctx->K, A, B, ctx->F, ctx->W, ctx->X.hash_next, ctx->tool_dev);
    n += 1;
    if (ev) CK(cudaEventRecord(ev[1], s));
    if (ctx->has_tool) {
        launch_fem_half(s, ctx->K, ctx->fem, ctx->tool_dev);
        n += 1;
    }
    if (pse_active(ctx)) {
        if (f32) launch_heat_pse(s, N, ctx->K, ctx->X.offsets, ctx->W, B32);
        else launch_heat_pse(s, N, ctx->K, ctx->X.offsets, ctx->W, B);
        n += 1;
    }
    if (ev) CK(cudaEventRecord(ev[2], s));
    SegDev sw = ctx->seg;
    if (ctx->wear_mode != SPH_WEAR_OFF) {   // segments_wear_rate_reset (leap_frog.cu:183-186)
        launch_wear_reset(s, ctx->seg);
        sw.wear.T_nodes = ctx->fem.T_half;  // the friction heat sees the half-step FEM temperature
    }
    const bool mlp_tensor = ctx->mlp_on && ctx->mlp_mode == SPH_MLP_TENSOR;
    if (mlp_tensor) CK(cudaMemsetAsync(ctx->jc_list_count, 0, sizeof(int32_t), s));
    if (f32 && ctx->mlp_on && !mlp_tensor)
        launch_interactions32_fused_mlp(s, N, ctx->K, ctx->X.offsets, B32, ctx->F32, ctx->W, sw, ctx->tool_dev,
                                        ctx->interact_variant, ctx->mlp);
    else if (f32)
        launch_interactions32_fused(s, N, ctx->K, ctx->X.offsets, B32, ctx->F32, ctx->W, sw, ctx->tool_dev,
                                    ctx->interact_variant);
    else
        launch_interactions(s, N, ctx->K, ctx->X.offsets, B, ctx->F, ctx->W, sw, ctx->tool_dev, true,
                            ctx->interact_variant);
    n += 1;
    if (mlp_tensor) {   // FP32K only (sph_mlp_attach)
        launch_jc_warm(s, jc_warm_grid(ctx), ctx->K, B32, ctx->F32, ctx->tool_dev, ctx->mlp, ctx->W.secant_iters,
                       ctx->W.status);
        n += 1;
    }
    if (ev) CK(cudaEventRecord(ev[3], s));
    if (ctx->has_tool) {
        launch_fem_rate_update(s, ctx->K, ctx->fem, ctx->seg, ctx->tool_dev);
        n += 1;
        if (ctx->wear_mode == SPH_WEAR_SHIFT) {   // wear_adjustment (leap_frog.cu:224-229)
            launch_wear_adjustment(s, ctx->K, ctx->fem, ctx->seg, ctx->wear, ctx->tool_dev, ctx->K.dt);
            n += 6;
        }
        launch_tool_move(s, ctx->K, ctx->seg, ctx->fem, ctx->tool_dev, ctx->K.dt, 3, true);
        n += 1;
    }
    if (ctx->K.rigid) {
        launch_rigid_move(s, ctx->K.rigid, ctx->K.dt);
        n += 1;
    }
    if (ev) CK(cudaEventRecord(ev[4], s));
    CK(cudaMemsetAsync(ctx->X.counts, 0, sizeof(int32_t) * (size_t)(ctx->K.g.num_cell + 1), s));
    if (f32) launch_step_tail(s, N, ctx->K, B32, ctx->seg, ctx->tool_dev, ctx->fem.T, ctx->X, ctx->W.status, true);
    else launch_step_tail(s, N, ctx->K, B, ctx->seg, ctx->tool_dev, ctx->fem.T, ctx->X, ctx->W.status, true);
    n += ctx->has_tool ? 3 : 1;   // with the FEM tool: the segment y-bins and the contact pass, then the tail
    if (ev) CK(cudaEventRecord(ev[5], s));
    CK_LAUNCH();
    return SPH_OK;
}

// The histogram of the current state, when the last call left it stale.
int count_current(sph_ctx *ctx) {
    if (ctx->counts_valid) return SPH_OK;
    if (ctx->K.precision == SPH_PREC_FP32K && ctx->v32[ctx->cur])
        launch_count(ctx->stream, ctx->N, ctx->c32[ctx->cur], ctx->X, ctx->K.g, ctx->W.status, true);
    else
        launch_count(ctx->stream, ctx->N, ctx->buf[ctx->cur], ctx->X, ctx->K.g, ctx->W.status, true);
    ctx->launches += 1;
    CK_LAUNCH();
    return SPH_OK;
}

// After a fused step from buffer p into w: the bookkeeping of both forms.
void finish_step(sph_ctx *ctx, int p, int w) {
    if (ctx->K.precision == SPH_PREC_FP32K) {
        ctx->v32[w] = true;
        ctx->v64[w] = false;
        ctx->pr32 = true;
        ctx->pr64 = false;
    }
    ctx->last_in = p;
    ctx->cur = w;
    ctx->counts_valid = true;
    ctx->in_cell_order = true;
}

}  // namespace

struct sph_tool_host {
    ToolModelHost m;
    std::string err;
};

extern "C" {

int sph_abi_version(void) { return SPHFEM_ABI_VERSION; }

// ---- host-only tool set-up ------------------------------------------------------------------
int sph_tool_build(const sph_tool_mesh *mesh, const sph_tool_constants *tc, sph_tool_host **out) {
    if (!mesh || !tc || !out) return SPH_ERR_INVALID;
    sph_tool_host *t = new sph_tool_host();
    *out = t;
    return build_tool_model(*mesh, *tc, t->m, t->err);
}

int sph_tool_host_info(const sph_tool_host *t, sph_tool_state *st, int32_t *n_nodes, int32_t *nnz,
                       int32_t *n_colors) {
    if (!t) return SPH_ERR_INVALID;
    const ToolModelHost &M = t->m;
    if (st) {
        std::memset(st, 0, sizeof(*st));
        for (int a = 0; a < 2; a++) {
            st->tl_point_ref[a] = M.tl_point_ref[a];
            st->br_point[a] = M.br_point[a];
        }
        st->ref_dist = M.ref_dist;
        st->lowest_point = M.lowest_point;
        st->right_point = M.right_point;
        st->n_segments = M.n_seg;
        st->n_cut_colors = M.n_cut_colors;
        st->flank_retreat = 0.;
        st->flank_contact = M.lowest_point;
    }
    if (n_nodes) *n_nodes = M.n_nodes;
    if (nnz) *nnz = (int32_t)M.col_ind.size();
    if (n_colors) *n_colors = M.n_colors;
    return SPH_OK;
}

int sph_tool_host_export(const sph_tool_host *t, sph_segments *seg, sph_fem *fem) {
    if (!t) return SPH_ERR_INVALID;
    const ToolModelHost &M = t->m;
    if (seg) {
        if (seg->n != M.n_seg) return SPH_ERR_INVALID;
        const size_t n = (size_t)M.n_seg;
        if (seg->left) std::memcpy(seg->left, M.left.data(), 16 * n);
        if (seg->right) std::memcpy(seg->right, M.right.data(), 16 * n);
        if (seg->normal) std::memcpy(seg->normal, M.normal.data(), 16 * n);
        if (seg->marks) std::memcpy(seg->marks, M.marks.data(), 16 * n);
        if (seg->heat_exchange) std::memset(seg->heat_exchange, 0, 16 * n);
        if (seg->fric_heat) std::memset(seg->fric_heat, 0, 8 * n);
    }
    if (fem) {
        if (fem->n_nodes != M.n_nodes || fem->nnz != (int32_t)M.col_ind.size()) return SPH_ERR_INVALID;
        const size_t nn = (size_t)M.n_nodes, nz = M.col_ind.size();
        if (fem->position) std::memcpy(fem->position, M.pos.data(), 16 * nn);
        if (fem->row_ptr) std::memcpy(fem->row_ptr, M.row_ptr.data(), 4 * (nn + 1));
        if (fem->col_ind) std::memcpy(fem->col_ind, M.col_ind.data(), 4 * nz);
        if (fem->K) std::memcpy(fem->K, M.K.data(), 8 * nz);
        if (fem->M_inv) std::memcpy(fem->M_inv, M.M_inv.data(), 8 * nn);
        if (fem->f) std::memcpy(fem->f, M.f.data(), 8 * nn);
        if (fem->T) std::memcpy(fem->T, M.T.data(), 8 * nn);
        if (fem->k) std::memset(fem->k, 0, 8 * nn);
    }
    return SPH_OK;
}

int sph_tool_host_layers(const sph_tool_host *t, int32_t *layer) {
    if (!t || !layer) return SPH_ERR_INVALID;
    for (int e = 0; e < t->m.n_elements; e++) {
        layer[2 * e] = t->m.layer[e].x;
        layer[2 * e + 1] = t->m.layer[e].y;
    }
    return SPH_OK;
}

int sph_tool_host_elements(const sph_tool_host *t, int32_t *elements) {
    if (!t || !elements) return SPH_ERR_INVALID;
    for (int e = 0; e < t->m.n_elements; e++) {
        const Int4 &el = t->m.elements[e];
        elements[4 * e] = el.x;
        elements[4 * e + 1] = el.y;
        elements[4 * e + 2] = el.z;
        elements[4 * e + 3] = el.w;
    }
    return SPH_OK;
}

int sph_tool_host_destroy(sph_tool_host *t) {
    if (!t) return SPH_ERR_INVALID;
    delete t;
    return SPH_OK;
}

const char *sph_last_error(const sph_ctx *ctx) { return ctx ? ctx->err.c_str() : g_no_ctx; }

int sph_ctx_destroy(sph_ctx *ctx) {
    if (!ctx) return SPH_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->io_up) {
        cudaStreamSynchronize(ctx->io_up);
        cudaStreamSynchronize(ctx->io_down);
        cudaStreamDestroy(ctx->io_up);
        cudaStreamDestroy(ctx->io_down);
        for (int b = 0; b < kBufs; b++) {
            cudaEventDestroy(ctx->ev_used[b]);
            cudaEventDestroy(ctx->ev_up[b]);
            cudaEventDestroy(ctx->ev_down[b]);
        }
        cudaEventDestroy(ctx->ev_fixed);
    }
    invalidate_graphs(ctx);
    for (void *p : ctx->allocs) cudaFree(p);
    if (ctx->tool_dev) cudaFree(ctx->tool_dev);
    if (ctx->h_reduce) cudaFreeHost(ctx->h_reduce);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SPH_OK;
}

}  // extern "C"

namespace {

int check_cell_params(const sph_grid_params *g) {
    if (g->cell_factor < 1 || g->stencil < 1 || !(g->h > 0)) return SPH_ERR_INVALID;
    if ((double)g->stencil * (double)g->cell_factor < 2.0) return SPH_ERR_INVALID;   // stencil must cover 2h
    if (g->stencil > kMaxStencil) return SPH_ERR_INVALID;
    return SPH_OK;
}

// Device checks, particle / sort / scratch allocation (particle_gpu ctor,
// particle_gpu.cu:11-104, and the Green grid buffers) for N particles on the
// cell geometry `geo`.  On SPH_OK or a context-reported error *out is set.
int ctx_begin(const sph_constants *c, const sph_grid_params *g, const sph_geom_constants &geo, int N, double dt,
              int32_t precision, int32_t device, sph_ctx **out) {
    sph_ctx *ctx = new sph_ctx();
    ctx->device = device;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device) {
        delete ctx;
        return SPH_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaSetDevice(device) != cudaSuccess || cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
        delete ctx;
        return SPH_ERR_NO_DEVICE;
    }
    if (!(prop.major == 10 && prop.minor == 3)) {   // built for sm_103a only
        delete ctx;
        return SPH_ERR_NO_DEVICE;
    }
    *out = ctx;   // from here on errors are reported through ctx (caller destroys)
    ctx->num_sms = prop.multiProcessorCount;
    CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    ctx->N = N;
    ctx->grid = *g;
    ctx->K.c = *c;
    ctx->K.g = geo;
    if (geo.nx <= 0 || geo.ny <= 0 || (int64_t)geo.nx * geo.ny > (int64_t)1 << 30)
        return fail(ctx, SPH_ERR_INVALID, "grid geometry out of range");
    ctx->K.dt = dt;
    ctx->K.precision = precision;
    ctx->K.n_cases = 1;
    ctx->K.secant_cap = 100;   // plasticity.cuh:155-158
    derive(ctx->K);
    // particle arrays (particle_gpu ctor, particle_gpu.cu:11-104) and the Green buffer
    for (int b = 0; b < 2; b++) {
        int r = alloc_sorted(ctx, ctx->buf[b], N);
        if (!r && precision == SPH_PREC_FP32K) r = alloc_sorted32(ctx, ctx->c32[b], N);
        if (r) return r;
    }
    if (precision == SPH_PREC_FP32K) {
        DALLOC(ctx->F32.p, N);
        DALLOC(ctx->F32.R, N);
    }
    DALLOC(ctx->F.p, N); DALLOC(ctx->F.R, N); DALLOC(ctx->F.S_der, N); DALLOC(ctx->F.v_der, N); DALLOC(ctx->F.idx, N);
    const int nc = ctx->K.g.num_cell;
    DALLOC(ctx->X.key, N); DALLOC(ctx->X.arrival, N); DALLOC(ctx->X.slots, N); DALLOC(ctx->X.hash_next, N);
    DALLOC(ctx->X.counts, (size_t)nc + 1); DALLOC(ctx->X.offsets, (size_t)nc + 2);
    DALLOC(ctx->X.block_sums, (size_t)scan_blocks(nc) + 1);
    DALLOC(ctx->X.cell_start, nc); DALLOC(ctx->X.cell_end, nc);
    if (precision == SPH_PREC_FP32K) {
        DALLOC(ctx->W.rec32, (size_t)4 * N);
        DALLOC(ctx->W.cand32, N);
    } else {
        DALLOC(ctx->W.rec64, (size_t)4 * N);
    }
    DALLOC(ctx->W.pos_init, N); DALLOC(ctx->W.vel_init, N); DALLOC(ctx->W.S_init, N);
    DALLOC(ctx->W.rho_init, N); DALLOC(ctx->W.T_init, N);
    DALLOC(ctx->W.secant_iters, N); DALLOC(ctx->W.status, 1);
    DALLOC(ctx->W.reduce, (size_t)3 * reduce_blocks());
    DALLOC(ctx->jc_stats, 2);
    CK(cudaMemset(ctx->jc_stats, 0, 2 * sizeof(unsigned long long)));
    CK(cudaMallocHost((void **)&ctx->h_reduce, sizeof(double) * 3 * reduce_blocks()));
    int r = zero_all(ctx);
    if (r) return r;
    for (int b = 0; b < 2; b++) CK(cudaMemsetAsync(ctx->buf[b].hash, 0, sizeof(int32_t) * N, ctx->stream));
    CK(cudaMemsetAsync(ctx->W.status, 0, sizeof(uint32_t), ctx->stream));
    CK(cudaMemsetAsync(ctx->W.secant_iters, 0, sizeof(int32_t) * N, ctx->stream));
    CK(cudaMemsetAsync(ctx->X.cell_end, 0, sizeof(int32_t) * nc, ctx->stream));
    CK(cudaMemsetAsync(ctx->X.cell_start, 0xff, sizeof(int32_t) * nc, ctx->stream));
    {   // idx = 0..N-1 (thrust::sequence, particle_gpu.cu:56-57)
        std::vector<int32_t> seq(N);
        for (int i = 0; i < N; i++) seq[i] = i;
        CK(cudaMemcpyAsync(ctx->F.idx, seq.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return SPH_OK;
}

// Uploads the tool model ctx->tool_host (segments, FEM system, node ->
// segment lists) and the per-case kinematic states `tds` (one per case).
int ctx_upload_tool(sph_ctx *ctx, bool with_model, const std::vector<ToolDev> &tds) {
    CK(cudaMalloc((void **)&ctx->tool_dev, sizeof(ToolDev) * tds.size()));
    if (with_model) {
        ToolModelHost &M = ctx->tool_host;
        ctx->has_tool = true;
        ctx->K.has_tool = 1;
        SegDev &S = ctx->seg;
        S.n = M.n_seg;
        DALLOC(S.left, M.n_seg); DALLOC(S.right, M.n_seg); DALLOC(S.normal, M.n_seg); DALLOC(S.marks, M.n_seg);
        DALLOC(S.heat_exchange, M.n_seg); DALLOC(S.fric_heat, M.n_seg);
        DALLOC(S.bin_count, (size_t)kSegBins * tds.size());
        DALLOC(S.bin_list, (size_t)kSegBins * kSegBinCap * tds.size());
        DALLOC(S.geo, M.n_seg);
        DALLOC(S.bin_xkey, (size_t)kSegBins * tds.size());
        CK(cudaMemcpy(S.left, M.left.data(), sizeof(double) * 2 * M.n_seg, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(S.right, M.right.data(), sizeof(double) * 2 * M.n_seg, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(S.normal, M.normal.data(), sizeof(double) * 2 * M.n_seg, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(S.marks, M.marks.data(), sizeof(int4) * M.n_seg, cudaMemcpyHostToDevice));
        CK(cudaMemset(S.heat_exchange, 0, sizeof(double2) * M.n_seg));
        CK(cudaMemset(S.fric_heat, 0, sizeof(double) * M.n_seg));
        FemDev &Fm = ctx->fem;
        Fm.n_nodes = M.n_nodes;
        Fm.nnz = (int)M.col_ind.size();
        DALLOC(Fm.position, M.n_nodes); DALLOC(Fm.row_ptr, M.n_nodes + 1); DALLOC(Fm.col_ind, Fm.nnz);
        DALLOC(Fm.diag, M.n_nodes); DALLOC(Fm.K, Fm.nnz); DALLOC(Fm.M_inv, M.n_nodes); DALLOC(Fm.f, M.n_nodes);
        DALLOC(Fm.M, M.n_nodes); DALLOC(ctx->fem_elements, M.n_elements);
        DALLOC(Fm.T, M.n_nodes); DALLOC(Fm.k, M.n_nodes); DALLOC(Fm.T_half, M.n_nodes);
        DALLOC(Fm.node_seg_ptr, M.n_nodes + 1); DALLOC(Fm.node_seg, M.node_seg.size());
        CK(cudaMemcpy(Fm.position, M.pos.data(), sizeof(double) * 2 * M.n_nodes, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(Fm.row_ptr, M.row_ptr.data(), sizeof(int) * (M.n_nodes + 1), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(Fm.col_ind, M.col_ind.data(), sizeof(int) * Fm.nnz, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(Fm.diag, M.diag.data(), sizeof(int) * M.n_nodes, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->fem_elements, M.elements.data(), sizeof(int4) * M.n_elements, cudaMemcpyHostToDevice));
        {   // K, lumped M, the Dirichlet elimination (f) and M_inv assembled on the device
            const int nd = (int)M.dirichlet_elem.size();
            int32_t *&dir_e = ctx->fem_dir_elems;
            int4 *&dir_f = ctx->fem_dir_flags;
            ctx->fem_n_dir = nd;
            DALLOC(dir_e, std::max(nd, 1));
            DALLOC(dir_f, std::max(nd, 1));
            if (nd) {
                CK(cudaMemcpy(dir_e, M.dirichlet_elem.data(), sizeof(int32_t) * nd, cudaMemcpyHostToDevice));
                CK(cudaMemcpy(dir_f, M.dirichlet_flags.data(), sizeof(int4) * nd, cudaMemcpyHostToDevice));
            }
            const sph_tool_constants &tc = ctx->K.c.tool;
            launch_fem_assemble(ctx->stream, Fm, ctx->fem_elements, M.n_elements, M.n_colors, dir_e, dir_f, nd,
                                tc.cp, tc.rho, tc.k, tc.T0, Fm.M);
            ctx->launches += M.n_colors + 2;
            CK_LAUNCH();
            CK(cudaStreamSynchronize(ctx->stream));
        }
        CK(cudaMemcpy(Fm.T, M.T.data(), sizeof(double) * M.n_nodes, cudaMemcpyHostToDevice));
        CK(cudaMemset(Fm.k, 0, sizeof(double) * M.n_nodes));
        CK(cudaMemcpy(Fm.T_half, M.T.data(), sizeof(double) * M.n_nodes, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(Fm.node_seg_ptr, M.node_seg_ptr.data(), sizeof(int) * (M.n_nodes + 1), cudaMemcpyHostToDevice));
        if (!M.node_seg.empty())
            CK(cudaMemcpy(Fm.node_seg, M.node_seg.data(), sizeof(int) * M.node_seg.size(), cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(ctx->tool_dev, tds.data(), sizeof(ToolDev) * tds.size(), cudaMemcpyHostToDevice));
    CK(cudaDeviceSynchronize());
    return SPH_OK;
}

// Kinematic state of a tool model (tool_FEM.h:57-77) on case slots
// [seg_first, seg_first + seg_count).
ToolDev tool_state_of(const ToolModelHost &M, double dt, int seg_first) {
    ToolDev td{};
    td.tl_point_ref[0] = M.tl_point_ref[0]; td.tl_point_ref[1] = M.tl_point_ref[1];
    td.br_point[0] = M.br_point[0]; td.br_point[1] = M.br_point[1];
    td.ref_dist = M.ref_dist; td.lowest_point = M.lowest_point; td.right_point = M.right_point;
    td.flank_retreat = 0.;
    td.flank_contact = M.lowest_point;   // as after a tool update (tool_FEM.cu:1567-1569)
    td.seg_first = seg_first;
    td.seg_count = M.n_seg;
    td.seg_ymin = INFINITY;
    td.seg_ymax = -INFINITY;
    td.seg_xmax = -INFINITY;
    td.seg_dxdy = 0.;
    for (int s = 0; s < M.n_seg; s++) {
        const double lx = M.left[2 * s], ly = M.left[2 * s + 1], rx = M.right[2 * s], ry = M.right[2 * s + 1];
        td.seg_ymin = std::min({td.seg_ymin, ly, ry});
        td.seg_ymax = std::max({td.seg_ymax, ly, ry});
        td.seg_xmax = std::max({td.seg_xmax, lx, rx});
        if (ly != ry) td.seg_dxdy = std::max(td.seg_dxdy, 1.01 * std::fabs(lx - rx) / std::fabs(ly - ry));
    }
    set_case_dt(td, dt);
    return td;
}

// Appends tool model `b` to `a` (block-diagonal FEM system, shifted node,
// element, nonzero and segment ids).
void append_tool_model(ToolModelHost &a, const ToolModelHost &b) {
    const int no = a.n_nodes, ne = a.n_elements, nz = (int)a.col_ind.size(), ns = a.n_seg;
    const int nsl = (int)a.node_seg.size();
    a.pos.insert(a.pos.end(), b.pos.begin(), b.pos.end());
    for (const Int4 &e : b.elements) a.elements.push_back({e.x + no, e.y + no, e.z + no, e.w});
    if (a.row_ptr.empty()) a.row_ptr.push_back(0);
    for (size_t i = 1; i < b.row_ptr.size(); i++) a.row_ptr.push_back(b.row_ptr[i] + nz);
    for (int c : b.col_ind) a.col_ind.push_back(c + no);
    for (int d : b.diag) a.diag.push_back(d + nz);
    a.K.insert(a.K.end(), b.K.begin(), b.K.end());
    a.M.insert(a.M.end(), b.M.begin(), b.M.end());
    a.M_inv.insert(a.M_inv.end(), b.M_inv.begin(), b.M_inv.end());
    a.f.insert(a.f.end(), b.f.begin(), b.f.end());
    a.T.insert(a.T.end(), b.T.begin(), b.T.end());
    a.left.insert(a.left.end(), b.left.begin(), b.left.end());
    a.right.insert(a.right.end(), b.right.begin(), b.right.end());
    a.normal.insert(a.normal.end(), b.normal.begin(), b.normal.end());
    for (const Int4 &m : b.marks) a.marks.push_back({m.x + ne, m.y, m.z + no, m.w + no});
    if (a.node_seg_ptr.empty()) a.node_seg_ptr.push_back(0);
    for (size_t i = 1; i < b.node_seg_ptr.size(); i++) a.node_seg_ptr.push_back(b.node_seg_ptr[i] + nsl);
    for (int s : b.node_seg) a.node_seg.push_back(s + ns);
    a.node_edge.insert(a.node_edge.end(), b.node_edge.begin(), b.node_edge.end());
    // one Dirichlet pass over the cases in turn: each case's rows are its own
    for (int e : b.dirichlet_elem) a.dirichlet_elem.push_back(e + ne);
    a.dirichlet_flags.insert(a.dirichlet_flags.end(), b.dirichlet_flags.begin(), b.dirichlet_flags.end());
    a.n_nodes += b.n_nodes;
    a.n_elements += b.n_elements;
    a.n_seg += b.n_seg;
    a.n_colors = std::max(a.n_colors, b.n_colors);
    a.n_cut_colors = std::max(a.n_cut_colors, b.n_cut_colors);
}

// Uploads the per-case reduction bounds (cells of each case's columns and the
// upload order's particle ranges) from the host case tables.
int finish_cases(sph_ctx *ctx, const std::vector<int32_t> &cell_bound) {
    const int n = (int)ctx->case_first.size();
    std::vector<int32_t> part_bound(n + 1, 0);
    for (int k = 0; k < n; k++) part_bound[k + 1] = part_bound[k] + ctx->case_count[k];
    DALLOC(ctx->case_cell_bound, (size_t)n + 1);
    DALLOC(ctx->case_part_bound, (size_t)n + 1);
    DALLOC(ctx->case_reduce, (size_t)3 * n);
    CK(cudaMemcpy(ctx->case_cell_bound, cell_bound.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->case_part_bound, part_bound.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice));
    return SPH_OK;
}

}  // namespace

extern "C" {

int sph_ctx_create(const sph_constants *c, const sph_grid_params *g, const sph_particles *host,
                   const sph_tool_mesh *tool, double dt, int32_t precision, int32_t device, sph_ctx **out) {
    if (!c || !g || !host || !out) return SPH_ERR_INVALID;
    *out = nullptr;
    if (host->N <= 0) return SPH_ERR_INVALID;
    if (precision != SPH_PREC_FP64 && precision != SPH_PREC_FP32K) return SPH_ERR_INVALID;
    if (check_cell_params(g)) return SPH_ERR_INVALID;
    sph_geom_constants geo;
    geometry_from(*g, geo);
    int r = ctx_begin(c, g, geo, host->N, dt, precision, device, out);
    sph_ctx *ctx = *out;
    if (r) return r;
    r = sph_upload_particles(ctx, host);
    if (r) return r;
    if (tool) {
        r = build_tool_model(*tool, c->tool, ctx->tool_host, ctx->err);
        if (r) return r;
    }
    std::vector<ToolDev> tds(1, tool ? tool_state_of(ctx->tool_host, dt, 0) : ToolDev{});
    if (!tool) set_case_dt(tds[0], dt);
    r = ctx_upload_tool(ctx, tool != nullptr, tds);
    if (r) return r;
    ctx->case_first = {0};
    ctx->case_count = {ctx->N};
    ctx->case_offset = {0., 0.};
    ctx->case_seg_first = {0};
    ctx->case_seg_count = {ctx->seg.n};
    ctx->case_node_first = {0};
    ctx->case_node_count = {ctx->fem.n_nodes};
    return finish_cases(ctx, {0, ctx->K.g.num_cell});
}

int sph_set_dt(sph_ctx *ctx, double dt) {
    REQUIRE_CTX();
    REQUIRE_SINGLE_CASE();
    ctx->K.dt = dt;
    derive(ctx->K);
    invalidate_graphs(ctx);
    ToolDev td;
    CK(cudaMemcpyAsync(&td, ctx->tool_dev, sizeof(ToolDev), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    set_case_dt(td, dt);
    CK(cudaMemcpyAsync(ctx->tool_dev, &td, sizeof(ToolDev), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_get_geometry(const sph_ctx *ctx, sph_geom_constants *out) {
    if (!ctx || !out) return SPH_ERR_INVALID;
    *out = ctx->K.g;
    return SPH_OK;
}

int sph_set_constants(sph_ctx *ctx, const sph_constants *c) {
    REQUIRE_CTX();
    if (!c) return SPH_ERR_INVALID;
    ctx->K.c = *c;
    derive(ctx->K);
    invalidate_graphs(ctx);
    return SPH_OK;
}

int sph_sync(sph_ctx *ctx) {
    REQUIRE_CTX();
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->io_up) {
        CK(cudaStreamSynchronize(ctx->io_up));
        CK(cudaStreamSynchronize(ctx->io_down));
    }
    CK(cudaGetLastError());
    return SPH_OK;
}

int sph_status(sph_ctx *ctx, uint32_t *status, int32_t clear) {
    REQUIRE_CTX();
    if (!status) return SPH_ERR_INVALID;
    CK(cudaMemcpyAsync(status, ctx->W.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    if (clear) CK(cudaMemsetAsync(ctx->W.status, 0, sizeof(uint32_t), ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_get_stream(const sph_ctx *ctx, void **stream) {
    if (!ctx || !stream) return SPH_ERR_INVALID;
    *stream = (void *)ctx->stream;
    return SPH_OK;
}

int sph_launch_count(const sph_ctx *ctx, int64_t *count) {
    if (!ctx || !count) return SPH_ERR_INVALID;
    *count = ctx->launches;
    return SPH_OK;
}

int sph_get_particles(sph_ctx *ctx, sph_particles *dev_view) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    if (!dev_view) return SPH_ERR_INVALID;
    *dev_view = view_of(ctx);
    return SPH_OK;
}

int sph_upload_particles(sph_ctx *ctx, const sph_particles *host) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    if (!host || host->N != ctx->N) return fail(ctx, SPH_ERR_INVALID, "upload: particle count mismatch");
    sph_particles v = view_of(ctx);
    for (const FieldDesc &fd : kFields) {
        const void *src = member<const void *>(*host, fd.off_view);
        if (!src) continue;
        void *dst = member<void *>(v, fd.off_view);
        CK(cudaMemcpyAsync(dst, src, (size_t)ctx->N * fd.width * (fd.is_int ? 4 : 8), cudaMemcpyHostToDevice,
                           ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->counts_valid = false;
    ctx->in_cell_order = false;
    return SPH_OK;
}

int sph_download_particles(sph_ctx *ctx, sph_particles *host) {
    REQUIRE_CTX();
    REQUIRE_STATE(false);
    if (!host || host->N != ctx->N) return fail(ctx, SPH_ERR_INVALID, "download: particle count mismatch");
    sph_particles v = view_of(ctx);
    for (const FieldDesc &fd : kFields) {
        void *dst = member<void *>(*host, fd.off_view);
        if (!dst) continue;
        const void *src = member<void *>(v, fd.off_view);
        CK(cudaMemcpyAsync(dst, src, (size_t)ctx->N * fd.width * (fd.is_int ? 4 : 8), cudaMemcpyDeviceToHost,
                           ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

// ---- pipelined host I/O ------------------------------------------------------------------------
int sph_upload_particles_async(sph_ctx *ctx, const sph_particles *host) {
    if (!ctx) return SPH_ERR_INVALID;
    if (!host || host->N != ctx->N) return fail(ctx, SPH_ERR_INVALID, "upload: particle count mismatch");
    if (host->p || host->R || host->S_der || host->v_der || host->idx)
        return fail(ctx, SPH_ERR_INVALID, "async upload: p, R, S_der, v_der, idx are recomputed by the step");
    int r = ensure_io(ctx);
    if (r) return r;
    // a buffer neither holding the current state nor read by the last queued step:
    // one no download reads, else the one whose download was issued first (the
    // upload then waits for the oldest download, not the one just queued)
    int t = -1;
    for (int b = 0; b < kBufs; b++) {
        if (b == ctx->cur || b == ctx->last_in) continue;
        if (t < 0) {
            t = b;
            continue;
        }
        const bool tb = ctx->down_pending[t], bb = ctx->down_pending[b];
        if ((tb && !bb) || (tb && bb && ctx->down_seq[b] < ctx->down_seq[t])) t = b;
    }
    CK(cudaStreamWaitEvent(ctx->io_up, ctx->ev_used[t], 0));                  // its last compute user
    if (ctx->down_pending[t]) CK(cudaStreamWaitEvent(ctx->io_up, ctx->ev_down[t], 0));   // a download out of it
    const sph_particles v = view_of_buf(ctx, t);
    for (const FieldDesc &fd : kFields) {
        const void *src = member<const void *>(*host, fd.off_view);
        if (!src) continue;
        void *dst = member<void *>(v, fd.off_view);
        CK(cudaMemcpyAsync(dst, src, (size_t)ctx->N * fd.width * (fd.is_int ? 4 : 8), cudaMemcpyHostToDevice,
                           ctx->io_up));
    }
    CK(cudaEventRecord(ctx->ev_up[t], ctx->io_up));
    ctx->up_pending[t] = true;
    ctx->cur = t;
    ctx->v64[t] = true;    // the next step reads the uploaded FP64 arrays
    ctx->v32[t] = false;
    ctx->counts_valid = false;
    ctx->in_cell_order = false;
    return SPH_OK;
}

int sph_download_particles_async(sph_ctx *ctx, sph_particles *host) {
    if (!ctx) return SPH_ERR_INVALID;
    if (!host || host->N != ctx->N) return fail(ctx, SPH_ERR_INVALID, "download: particle count mismatch");
    int r = ensure_io(ctx);
    if (r) return r;
    const int src_b = ctx->cur;
    const bool fixed = host->p || host->R || host->S_der || host->v_der || host->idx;
    if (ctx->K.precision == SPH_PREC_FP32K && (!ctx->v64[src_b] || (fixed && !ctx->pr64))) {
        // the step left the state in the compact form: widen it into buf[src_b] on the
        // compute stream, after the copies of buf[src_b] still in flight
        r = wait_io(ctx, src_b);
        if (r) return r;
        launch_state_to64(ctx->stream, ctx->N, ctx->c32[src_b], ctx->F32, ctx->buf[src_b], ctx->F,
                          !ctx->v64[src_b], fixed && !ctx->pr64);
        ctx->launches++;
        CK_LAUNCH();
        ctx->v64[src_b] = true;
        if (fixed) ctx->pr64 = true;
        CK(cudaEventRecord(ctx->ev_used[src_b], ctx->stream));
    }
    CK(cudaStreamWaitEvent(ctx->io_down, ctx->ev_used[src_b], 0));            // the step that wrote it
    if (fixed) {                                                              // p, R, ...: the last step
        CK(cudaEventRecord(ctx->ev_fixed, ctx->stream));
        CK(cudaStreamWaitEvent(ctx->io_down, ctx->ev_fixed, 0));
    }
    if (ctx->up_pending[src_b]) CK(cudaStreamWaitEvent(ctx->io_down, ctx->ev_up[src_b], 0));
    const sph_particles v = view_of_buf(ctx, src_b);
    for (const FieldDesc &fd : kFields) {
        void *dst = member<void *>(*host, fd.off_view);
        if (!dst) continue;
        const void *src = member<void *>(v, fd.off_view);
        CK(cudaMemcpyAsync(dst, src, (size_t)ctx->N * fd.width * (fd.is_int ? 4 : 8), cudaMemcpyDeviceToHost,
                           ctx->io_down));
    }
    CK(cudaEventRecord(ctx->ev_down[src_b], ctx->io_down));
    ctx->down_pending[src_b] = true;
    ctx->down_seq[src_b] = ++ctx->n_downloads;
    if (fixed) {
        CK(cudaEventRecord(ctx->ev_fixed, ctx->io_down));
        ctx->fixed_pending = true;
    }
    return SPH_OK;
}

int sph_get_cells(sph_ctx *ctx, int32_t **cell_start, int32_t **cell_end, int32_t *num_cell) {
    REQUIRE_CTX();
    if (cell_start) *cell_start = ctx->X.cell_start;
    if (cell_end) *cell_end = ctx->X.cell_end;
    if (num_cell) *num_cell = ctx->K.g.num_cell;
    return SPH_OK;
}

int sph_download_cells(sph_ctx *ctx, int32_t *cell_start, int32_t *cell_end) {
    REQUIRE_CTX();
    size_t b = sizeof(int32_t) * (size_t)ctx->K.g.num_cell;
    if (cell_start) CK(cudaMemcpyAsync(cell_start, ctx->X.cell_start, b, cudaMemcpyDeviceToHost, ctx->stream));
    if (cell_end) CK(cudaMemcpyAsync(cell_end, ctx->X.cell_end, b, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

// ---- grid ------------------------------------------------------------------------------------
int sph_update_geometry(sph_ctx *ctx) {
    REQUIRE_CTX();
    return SPH_OK;   // locked grid (grid.cu:88-91)
}

int sph_assign_hashes(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    launch_hash(ctx->stream, ctx->N, CUR(ctx), ctx->K.g);
    ctx->launches += 1;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_sort(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    const int N = ctx->N;
    launch_count(ctx->stream, N, CUR(ctx), ctx->X, ctx->K.g, ctx->W.status, false);
    launch_sort_rest(ctx->stream, N, ctx->X, ctx->K.g, ctx->F.idx, ctx->W.status);
    const int w = pick_out(ctx);
    launch_gather_plain(ctx->stream, N, ctx->F.idx, CUR(ctx), ctx->buf[w]);
    ctx->launches += 7;
    CK_LAUNCH();
    int rm = mark_used(ctx, ctx->cur, w);
    if (rm) return rm;
    ctx->last_in = ctx->cur;
    ctx->cur = w;   // double_buffer swap (grid_gpu_green.cu:152-182)
    ctx->counts_valid = false;
    ctx->in_cell_order = true;
    return SPH_OK;
}

// ---- leap frog --------------------------------------------------------------------------------
int sph_init(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    launch_init(ctx->stream, ctx->N, CUR(ctx), ctx->W);
    ctx->launches++;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_predict(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    REQUIRE_SINGLE_CASE();
    launch_predict_correct(ctx->stream, ctx->N, CUR(ctx), ctx->W, 0.5 * ctx->K.dt);
    ctx->launches++;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_correct(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    REQUIRE_SINGLE_CASE();
    launch_predict_correct(ctx->stream, ctx->N, CUR(ctx), ctx->W, ctx->K.dt);
    ctx->launches++;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

// ---- actions ----------------------------------------------------------------------------------
#define STAGE(name, call)                 \
    int name(sph_ctx *ctx) {              \
        REQUIRE_CTX();                    \
        REQUIRE_STATE(true);              \
        call;                             \
        ctx->launches++;                  \
        ctx->counts_valid = false;        \
        CK_LAUNCH();                      \
        return SPH_OK;                    \
    }

STAGE(sph_material_eos, launch_eos(ctx->stream, ctx->N, ctx->K, CUR(ctx), ctx->F))
STAGE(sph_corrector_artificial_stress, launch_artificial_stress(ctx->stream, ctx->N, ctx->K, CUR(ctx), ctx->F))
STAGE(sph_material_stress_rate_jaumann, launch_jaumann(ctx->stream, ctx->N, ctx->K, CUR(ctx), ctx->F))
STAGE(sph_contmech_continuity, launch_continuity(ctx->stream, ctx->N, CUR(ctx), ctx->F))
STAGE(sph_contmech_momentum, launch_momentum(ctx->stream, ctx->N, ctx->K, CUR(ctx), ctx->F))
STAGE(sph_contmech_advection, launch_advection(ctx->stream, ctx->N, CUR(ctx)))
STAGE(sph_perform_boundary_conditions, launch_bc(ctx->stream, ctx->N, CUR(ctx)))
STAGE(sph_debug_invalidate, launch_invalidate(ctx->stream, ctx->N, CUR(ctx), ctx->W.status))

int sph_perform_boundary_conditions_thermal(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    if (ctx->K.c.trml_tool.alpha == 0.) return SPH_OK;   // m_thermal off (actions_gpu.cu:881-886)
    launch_bc_thermal(ctx->stream, ctx->N, ctx->K, CUR(ctx));
    ctx->launches++;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_plasticity_johnson_cook(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    REQUIRE_SINGLE_CASE();
    if (!ctx->K.c.plastic) return SPH_OK;   // m_plastic off (actions_gpu.cu:874-879)
    launch_plasticity(ctx->stream, ctx->N, ctx->K, CUR(ctx), ctx->F, ctx->W);
    ctx->launches++;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_interactions_monaghan(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    REQUIRE_SINGLE_CASE();
    launch_build_records(ctx->stream, ctx->N, ctx->K, CUR(ctx), ctx->F, ctx->W);
    launch_interactions(ctx->stream, ctx->N, ctx->K, ctx->X.offsets, CUR(ctx), ctx->F, ctx->W, ctx->seg,
                        ctx->tool_dev, false);
    ctx->launches += 2;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

// ---- tool -------------------------------------------------------------------------------------
int sph_material_fric_heat_gen_fem(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    REQUIRE_SINGLE_CASE();
    REQUIRE_TOOL();
    SegDev sw = ctx->seg;
    sw.wear.T_nodes = ctx->fem.T;   // after calculate_temp(0.5 dt) in the staged sequence
    launch_fric_heat(ctx->stream, ctx->N, ctx->K, CUR(ctx), sw, ctx->tool_dev, ctx->W.status);
    ctx->launches++;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_compute_contact_forces_fem(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    REQUIRE_SINGLE_CASE();
    REQUIRE_TOOL();
    launch_contact(ctx->stream, ctx->N, ctx->K, CUR(ctx), ctx->seg, ctx->tool_dev, ctx->fem.T, ctx->W.status);
    ctx->launches += 3;   // segment y-bins, s1, s2
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_segments_update(sph_ctx *ctx, double dt) {
    REQUIRE_CTX();
    REQUIRE_SINGLE_CASE();
    REQUIRE_TOOL();
    launch_tool_move(ctx->stream, ctx->K, ctx->seg, ctx->fem, ctx->tool_dev, dt, 1, false);
    ctx->launches++;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_tool_update_fem(sph_ctx *ctx, double dt) {
    REQUIRE_CTX();
    REQUIRE_SINGLE_CASE();
    REQUIRE_TOOL();
    launch_tool_move(ctx->stream, ctx->K, ctx->seg, ctx->fem, ctx->tool_dev, dt, 2, false);
    ctx->launches++;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_fem_reset_server(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    int r = ensure_fem_temp(ctx);
    if (r) return r;
    launch_fem_reset(ctx->stream, ctx->fem, ctx->fem_T_old, ctx->fem_f_temp, ctx->fem_K_temp);
    ctx->launches++;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_fem_apply_robin(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    int r = ensure_fem_temp(ctx);
    if (r) return r;
    launch_fem_robin(ctx->stream, ctx->K, ctx->fem, ctx->seg, ctx->fem_f_temp, ctx->fem_K_temp);
    ctx->launches++;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_fem_calculate_temp_rate(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    int r = ensure_fem_temp(ctx);
    if (r) return r;
    launch_fem_rate(ctx->stream, ctx->fem, ctx->fem_f_temp, ctx->fem_K_temp);
    ctx->launches++;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_fem_calculate_temp(sph_ctx *ctx, double dt) {
    REQUIRE_CTX();
    REQUIRE_SINGLE_CASE();
    REQUIRE_TOOL();
    int r = ensure_fem_temp(ctx);
    if (r) return r;
    launch_fem_temp(ctx->stream, ctx->fem, ctx->fem_T_old, dt);
    ctx->launches++;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_set_tool_velocity(sph_ctx *ctx, double vx, double vy) {
    REQUIRE_CTX();
    REQUIRE_SINGLE_CASE();
    double v[2] = {vx, vy};
    CK(cudaMemcpyAsync(ctx->tool_dev, v, sizeof(v), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_get_tool_state(sph_ctx *ctx, sph_tool_state *out) {
    REQUIRE_CTX();
    if (!out) return SPH_ERR_INVALID;
    ToolDev td;
    CK(cudaMemcpyAsync(&td, ctx->tool_dev, sizeof(td), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    std::memset(out, 0, sizeof(*out));
    for (int a = 0; a < 2; a++) {
        out->vel[a] = td.vel[a];
        out->tl_point_ref[a] = td.tl_point_ref[a];
        out->br_point[a] = td.br_point[a];
    }
    out->ref_dist = td.ref_dist;
    out->lowest_point = td.lowest_point;
    out->right_point = td.right_point;
    out->n_segments = ctx->seg.n;
    out->n_cut_colors = ctx->tool_host.n_cut_colors;
    out->flank_retreat = td.flank_retreat;
    out->flank_contact = td.flank_contact;
    return SPH_OK;
}

int sph_get_segments(sph_ctx *ctx, sph_segments *v) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    if (!v) return SPH_ERR_INVALID;
    v->n = ctx->seg.n;
    v->left = (double *)ctx->seg.left;
    v->right = (double *)ctx->seg.right;
    v->normal = (double *)ctx->seg.normal;
    v->marks = (int32_t *)ctx->seg.marks;
    v->heat_exchange = (double *)ctx->seg.heat_exchange;
    v->fric_heat = ctx->seg.fric_heat;
    return SPH_OK;
}

int sph_download_segments(sph_ctx *ctx, sph_segments *h) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    if (!h || h->n != ctx->seg.n) return fail(ctx, SPH_ERR_INVALID, "download_segments: size mismatch");
    const size_t n = (size_t)ctx->seg.n;
    cudaStream_t s = ctx->stream;
    if (h->left) CK(cudaMemcpyAsync(h->left, ctx->seg.left, 16 * n, cudaMemcpyDeviceToHost, s));
    if (h->right) CK(cudaMemcpyAsync(h->right, ctx->seg.right, 16 * n, cudaMemcpyDeviceToHost, s));
    if (h->normal) CK(cudaMemcpyAsync(h->normal, ctx->seg.normal, 16 * n, cudaMemcpyDeviceToHost, s));
    if (h->marks) CK(cudaMemcpyAsync(h->marks, ctx->seg.marks, 16 * n, cudaMemcpyDeviceToHost, s));
    if (h->heat_exchange) CK(cudaMemcpyAsync(h->heat_exchange, ctx->seg.heat_exchange, 16 * n, cudaMemcpyDeviceToHost, s));
    if (h->fric_heat) CK(cudaMemcpyAsync(h->fric_heat, ctx->seg.fric_heat, 8 * n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return SPH_OK;
}

int sph_get_fem(sph_ctx *ctx, sph_fem *v) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    if (!v) return SPH_ERR_INVALID;
    v->n_nodes = ctx->fem.n_nodes;
    v->nnz = ctx->fem.nnz;
    v->position = (double *)ctx->fem.position;
    v->row_ptr = ctx->fem.row_ptr;
    v->col_ind = ctx->fem.col_ind;
    v->K = ctx->fem.K;
    v->M_inv = ctx->fem.M_inv;
    v->f = ctx->fem.f;
    v->T = ctx->fem.T;
    v->k = ctx->fem.k;
    return SPH_OK;
}

int sph_download_fem(sph_ctx *ctx, sph_fem *h) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    if (!h || h->n_nodes != ctx->fem.n_nodes || h->nnz != ctx->fem.nnz)
        return fail(ctx, SPH_ERR_INVALID, "download_fem: size mismatch");
    const size_t nn = (size_t)ctx->fem.n_nodes, nz = (size_t)ctx->fem.nnz;
    cudaStream_t s = ctx->stream;
    if (h->position) CK(cudaMemcpyAsync(h->position, ctx->fem.position, 16 * nn, cudaMemcpyDeviceToHost, s));
    if (h->row_ptr) CK(cudaMemcpyAsync(h->row_ptr, ctx->fem.row_ptr, 4 * (nn + 1), cudaMemcpyDeviceToHost, s));
    if (h->col_ind) CK(cudaMemcpyAsync(h->col_ind, ctx->fem.col_ind, 4 * nz, cudaMemcpyDeviceToHost, s));
    if (h->K) CK(cudaMemcpyAsync(h->K, ctx->fem.K, 8 * nz, cudaMemcpyDeviceToHost, s));
    if (h->M_inv) CK(cudaMemcpyAsync(h->M_inv, ctx->fem.M_inv, 8 * nn, cudaMemcpyDeviceToHost, s));
    if (h->f) CK(cudaMemcpyAsync(h->f, ctx->fem.f, 8 * nn, cudaMemcpyDeviceToHost, s));
    if (h->T) CK(cudaMemcpyAsync(h->T, ctx->fem.T, 8 * nn, cudaMemcpyDeviceToHost, s));
    if (h->k) CK(cudaMemcpyAsync(h->k, ctx->fem.k, 8 * nn, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return SPH_OK;
}

int sph_upload_fem_state(sph_ctx *ctx, const double *T, const double *k) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    const size_t nn = (size_t)ctx->fem.n_nodes;
    if (T) CK(cudaMemcpyAsync(ctx->fem.T, T, 8 * nn, cudaMemcpyHostToDevice, ctx->stream));
    if (k) CK(cudaMemcpyAsync(ctx->fem.k, k, 8 * nn, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

// ---- whole step -------------------------------------------------------------------------------
int sph_step(sph_ctx *ctx) {
    if (!ctx) return SPH_ERR_INVALID;
    cudaStream_t s = ctx->stream;
    const int w = pick_out(ctx);
    // only the copies into the input, out of (or into) the output, and of the derived fields;
    // an FP32K step writes the compact copy c32[w], which no copy touches (a download widens
    // it into buf[w] later, after the copies of buf[w])
    int r0 = wait_io(ctx, ctx->cur);
    if (r0 == SPH_OK && ctx->K.precision != SPH_PREC_FP32K) r0 = wait_io(ctx, w);
    if (r0) return r0;
    {
        int rc = count_current(ctx);
        if (rc) return rc;
    }
    const int p = ctx->cur;
    const bool f32 = ctx->K.precision == SPH_PREC_FP32K;
    const int src32 = f32 && ctx->v32[p] ? 1 : 0, pr32 = f32 && ctx->pr32 ? 1 : 0;
    cudaGraphExec_t &gexec = ctx->graph[p][w][src32][pr32];
    int64_t &glaunch = ctx->graph_launches[p][w][src32][pr32];
    if (ctx->use_graph) {
        if (!gexec) {
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            int64_t n = 0;
            int r = issue_fused_body(ctx, n, w);
            cudaError_t e = cudaStreamEndCapture(s, &g);
            if (r) {
                if (g) cudaGraphDestroy(g);
                return r;
            }
            if (e != cudaSuccess) return fail(ctx, SPH_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
            e = cudaGraphInstantiate(&gexec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return fail(ctx, SPH_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
            glaunch = n;
        }
        CK(cudaGraphLaunch(gexec, s));
        ctx->launches += glaunch;
    } else {
        int64_t n = 0;
        int r = issue_fused_body(ctx, n, w);
        if (r) return r;
        ctx->launches += n;
    }
    int r1 = mark_used(ctx, p, w);
    if (r1) return r1;
    finish_step(ctx, p, w);
    return SPH_OK;
}

int sph_profile_steps(sph_ctx *ctx, int32_t nsteps, float *stage_ms, int32_t *n_stages) {
    REQUIRE_CTX();
    constexpr int kStages = 7;
    if (!stage_ms || nsteps < 1) return SPH_ERR_INVALID;
    if (n_stages) *n_stages = kStages;
    cudaStream_t s = ctx->stream;
    cudaEvent_t ev[kStages + 1];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    for (int k = 0; k < kStages; k++) stage_ms[k] = 0.f;
    for (int step = 0; step < nsteps; step++) {
        const int w = pick_out(ctx);
        int r0 = wait_io(ctx, ctx->cur);
        if (r0 == SPH_OK) r0 = wait_io(ctx, w);
        if (r0) {
            for (auto &e : ev) cudaEventDestroy(e);
            return r0;
        }
        CK(cudaEventRecord(ev[0], s));
        int r1 = count_current(ctx);
        if (r1) return r1;
        CK(cudaEventRecord(ev[1], s));
        int64_t n = 0;
        r1 = issue_fused_body(ctx, n, w, ev + 2);
        if (r1) return r1;
        ctx->launches += n;
        CK(cudaEventSynchronize(ev[7]));
        for (int k = 0; k < kStages; k++) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
            stage_ms[k] += ms;
        }
        int rm = mark_used(ctx, ctx->cur, w);
        if (rm) return rm;
        finish_step(ctx, ctx->cur, w);
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return SPH_OK;
}

int sph_run(sph_ctx *ctx, int32_t nsteps) {
    REQUIRE_CTX();
    for (int i = 0; i < nsteps; i++) {
        int r = sph_step(ctx);
        if (r) return r;
    }
    return SPH_OK;
}

int sph_step_staged(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    REQUIRE_SINGLE_CASE();
    int r;
#define RUN(x)            \
    if ((r = (x)) != SPH_OK) return r;
    const double dt = ctx->K.dt;
    RUN(sph_update_geometry(ctx));
    RUN(sph_assign_hashes(ctx));
    RUN(sph_sort(ctx));
    RUN(sph_init(ctx));
    if (ctx->has_tool) RUN(sph_fem_reset_server(ctx));
    if (ctx->wear_mode != SPH_WEAR_OFF) RUN(sph_segments_wear_rate_reset(ctx));
    RUN(sph_predict(ctx));
    if (ctx->has_tool) RUN(sph_fem_calculate_temp(ctx, 0.5 * dt));
    RUN(sph_material_eos(ctx));
    RUN(sph_corrector_artificial_stress(ctx));
    RUN(sph_interactions_monaghan(ctx));
    if (ctx->K.thermal_pse) RUN(sph_interactions_heat_pse(ctx));
    RUN(sph_material_stress_rate_jaumann(ctx));
    RUN(sph_contmech_continuity(ctx));
    RUN(sph_contmech_momentum(ctx));
    RUN(sph_contmech_advection(ctx));
    RUN(sph_correct(ctx));
    if (ctx->has_tool) {
        RUN(sph_material_fric_heat_gen_fem(ctx));
        RUN(sph_fem_apply_robin(ctx));
        RUN(sph_fem_calculate_temp_rate(ctx));
        RUN(sph_fem_calculate_temp(ctx, dt));
    }
    if (ctx->K.rigid) RUN(sph_material_fric_heat_gen(ctx));
    RUN(sph_plasticity_johnson_cook(ctx));
    if (ctx->wear_mode == SPH_WEAR_SHIFT) RUN(sph_wear_adjustment(ctx));
    if (ctx->has_tool) {
        RUN(sph_segments_update(ctx, dt));
        RUN(sph_tool_update_fem(ctx, dt));
        RUN(sph_compute_contact_forces_fem(ctx));
    }
    if (ctx->K.rigid) {
        RUN(sph_rigid_tool_update(ctx));
        RUN(sph_compute_contact_forces(ctx));
    }
    RUN(sph_perform_boundary_conditions(ctx));
    RUN(sph_perform_boundary_conditions_thermal(ctx));
    RUN(sph_debug_invalidate(ctx));
#undef RUN
    return SPH_OK;
}

// ---- measurement hooks --------------------------------------------------------------------------
static int reduce_force_T(sph_ctx *ctx, double out[3]) {
    REQUIRE_STATE(false);
    launch_reduce_force_T(ctx->stream, ctx->N, CUR(ctx), ctx->W.reduce);
    ctx->launches++;
    CK_LAUNCH();
    const int nb = reduce_blocks();
    CK(cudaMemcpyAsync(ctx->h_reduce, ctx->W.reduce, sizeof(double) * 3 * nb, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    double fx = 0., fy = 0., tm = -1e300;
    for (int b = 0; b < nb; b++) {
        fx += ctx->h_reduce[3 * b];
        fy += ctx->h_reduce[3 * b + 1];
        tm = std::fmax(tm, ctx->h_reduce[3 * b + 2]);
    }
    out[0] = fx;
    out[1] = fy;
    out[2] = tm;
    return SPH_OK;
}

int sph_reduce_force(sph_ctx *ctx, double out[2]) {
    REQUIRE_CTX();
    if (!out) return SPH_ERR_INVALID;
    double r3[3];
    int r = reduce_force_T(ctx, r3);
    if (r) return r;
    out[0] = r3[0];
    out[1] = r3[1];
    return SPH_OK;
}

int sph_reduce_max_T(sph_ctx *ctx, double *out) {
    REQUIRE_CTX();
    if (!out) return SPH_ERR_INVALID;
    double r3[3];
    int r = reduce_force_T(ctx, r3);
    if (r) return r;
    *out = r3[2];
    return SPH_OK;
}

// ---- batched multi-case contexts ------------------------------------------------------------------
int sph_batch_create(const sph_constants *c, const sph_grid_params *cell, int32_t n_cases,
                     const sph_case_desc *cases, int32_t precision, int32_t device, sph_ctx **out) {
    if (!c || !cell || !cases || !out || n_cases < 1 || n_cases > 65535) return SPH_ERR_INVALID;
    *out = nullptr;
    if (precision != SPH_PREC_FP32K && precision != SPH_PREC_FP64) return SPH_ERR_INVALID;
    if (check_cell_params(cell)) return SPH_ERR_INVALID;
    const bool with_tool = cases[0].tool != nullptr;
    int64_t n_total = 0;
    for (int k = 0; k < n_cases; k++) {
        const sph_case_desc &d = cases[k];
        if (!d.host || d.host->N <= 0 || !(d.dt > 0)) return SPH_ERR_INVALID;
        if ((d.tool != nullptr) != with_tool) return SPH_ERR_INVALID;
        if (!(d.bbmax[0] > d.bbmin[0]) || !(d.bbmax[1] > d.bbmin[1])) return SPH_ERR_INVALID;
        n_total += d.host->N;
    }
    if (n_total > (int64_t)1 << 30) return SPH_ERR_INVALID;
    // layout: case k gets columns [col0[k], col0[k] + nx_k) of one global
    // grid, gaps of stencil + 1 columns between cases, bottoms aligned
    const double gx0 = cases[0].bbmin[0], gy0 = cases[0].bbmin[1];
    const int gap = cell->stencil + 1;
    std::vector<int> col0(n_cases), ncol(n_cases);
    std::vector<double> offs(2 * (size_t)n_cases);
    sph_geom_constants geo;
    geometry_from(*cell, geo);   // dx and stencil; extents set below
    int cols = 0, rows = 0;
    for (int k = 0; k < n_cases; k++) {
        sph_grid_params gk = *cell;
        for (int a = 0; a < 2; a++) {
            gk.bbmin[a] = cases[k].bbmin[a];
            gk.bbmax[a] = cases[k].bbmax[a];
        }
        sph_geom_constants ck;
        geometry_from(gk, ck);
        if (k) cols += gap;
        col0[k] = cols;
        ncol[k] = ck.nx;
        cols += ck.nx;
        rows = std::max(rows, ck.ny);
        offs[2 * k] = (gx0 + (double)col0[k] * geo.dx) - cases[k].bbmin[0];
        offs[2 * k + 1] = gy0 - cases[k].bbmin[1];
        if ((int64_t)cols * std::max(rows, 1) > (int64_t)1 << 30) return SPH_ERR_INVALID;
    }
    geo.nx = cols;
    geo.ny = rows;
    geo.bbmin_x = gx0 - 1e-6;
    geo.bbmin_y = gy0 - 1e-6;
    geo.num_cell = cols * rows;
    sph_grid_params g = *cell;
    g.bbmin[0] = gx0;
    g.bbmin[1] = gy0;
    g.bbmax[0] = gx0 + (double)cols * geo.dx - 2e-6;
    g.bbmax[1] = gy0 + (double)rows * geo.dx - 2e-6;
    int r = ctx_begin(c, &g, geo, (int)n_total, cases[0].dt, precision, device, out);
    sph_ctx *ctx = *out;
    if (r) return r;
    ctx->K.n_cases = n_cases;
    // tool models, each moved by its case offset and appended
    std::vector<ToolDev> tds(n_cases);
    ctx->case_seg_first.assign(n_cases, 0);
    ctx->case_seg_count.assign(n_cases, 0);
    ctx->case_node_first.assign(n_cases, 0);
    ctx->case_node_count.assign(n_cases, 0);
    for (int k = 0; k < n_cases; k++) {
        const sph_case_desc &d = cases[k];
        ToolDev td{};
        if (with_tool) {
            const sph_tool_mesh &m = *d.tool;
            if (m.n_nodes <= 0 || !m.nodes) return fail(ctx, SPH_ERR_INVALID, "batch: empty tool mesh");
            std::vector<double> nodes(2 * (size_t)m.n_nodes);
            for (int i = 0; i < m.n_nodes; i++) {
                nodes[2 * i] = m.nodes[2 * i] + offs[2 * k];
                nodes[2 * i + 1] = m.nodes[2 * i + 1] + offs[2 * k + 1];
            }
            sph_tool_mesh mk = m;
            mk.nodes = nodes.data();
            mk.tl[0] = m.tl[0] + offs[2 * k];
            mk.tl[1] = m.tl[1] + offs[2 * k + 1];
            ToolModelHost Mk;
            r = build_tool_model(mk, c->tool, Mk, ctx->err);
            if (r) return r;
            ctx->case_seg_first[k] = ctx->tool_host.n_seg;
            ctx->case_seg_count[k] = Mk.n_seg;
            ctx->case_node_first[k] = ctx->tool_host.n_nodes;
            ctx->case_node_count[k] = Mk.n_nodes;
            td = tool_state_of(Mk, d.dt, ctx->tool_host.n_seg);
            append_tool_model(ctx->tool_host, Mk);
        } else {
            set_case_dt(td, d.dt);
        }
        td.vel[0] = d.tool_vel[0];
        td.vel[1] = d.tool_vel[1];
        tds[k] = td;
    }
    // particles, concatenated in case order and moved by the case offsets
    const int N = (int)n_total;
    ctx->case_first.assign(n_cases, 0);
    ctx->case_count.assign(n_cases, 0);
    ctx->case_offset = offs;
    {
        int first = 0;
        for (int k = 0; k < n_cases; k++) {
            ctx->case_first[k] = first;
            ctx->case_count[k] = cases[k].host->N;
            first += cases[k].host->N;
        }
    }
    sph_particles cat;
    std::memset(&cat, 0, sizeof(cat));
    cat.N = N;
    std::vector<std::vector<char>> store;
    for (const FieldDesc &fd : kFields) {
        if (fd.off_view == offsetof(sph_particles, idx) || fd.off_view == offsetof(sph_particles, hash)) continue;
        bool any = false;
        for (int k = 0; k < n_cases; k++) any |= member<const void *>(*cases[k].host, fd.off_view) != nullptr;
        if (!any) continue;
        const size_t esz = (size_t)fd.width * (fd.is_int ? 4 : 8);
        store.emplace_back((size_t)N * esz, 0);
        char *dst = store.back().data();
        for (int k = 0; k < n_cases; k++) {
            const char *src = member<const char *>(*cases[k].host, fd.off_view);
            char *at = dst + (size_t)ctx->case_first[k] * esz;
            const size_t nk = (size_t)cases[k].host->N;
            if (src) std::memcpy(at, src, nk * esz);
            if (fd.off_view == offsetof(sph_particles, pos)) {
                double *p = (double *)at;
                for (size_t i = 0; i < nk; i++) {
                    p[2 * i] += offs[2 * k];
                    p[2 * i + 1] += offs[2 * k + 1];
                }
            } else if (fd.off_view == offsetof(sph_particles, on_seg) && src) {
                int32_t *q = (int32_t *)at;
                for (size_t i = 0; i < nk; i++)
                    if (q[i] >= 0) q[i] += ctx->case_seg_first[k];
            }
        }
        *(void **)((char *)&cat + fd.off_view) = (void *)dst;
    }
    r = sph_upload_particles(ctx, &cat);
    if (r) return r;
    r = ctx_upload_tool(ctx, with_tool, tds);
    if (r) return r;
    // case tables: columns split in the middle of each gap; nodes; segments
    ctx->case_of_col_h.assign(cols, 0);
    std::vector<int32_t> cell_bound(n_cases + 1);
    for (int k = 0; k < n_cases; k++) {
        int b = k ? col0[k] - (gap + 1) / 2 : 0;
        int e = (k + 1 < n_cases) ? col0[k + 1] - (gap + 1) / 2 : cols;
        for (int ix = b; ix < e; ix++) ctx->case_of_col_h[ix] = (uint16_t)k;
        cell_bound[k] = b * rows;
        if (k + 1 == n_cases) cell_bound[k + 1] = cols * rows;
    }
    uint16_t *d_col = nullptr, *d_node = nullptr, *d_seg = nullptr;
    DALLOC(d_col, (size_t)cols);
    CK(cudaMemcpy(d_col, ctx->case_of_col_h.data(), sizeof(uint16_t) * cols, cudaMemcpyHostToDevice));
    ctx->K.case_of_col = d_col;
    if (with_tool) {
        std::vector<uint16_t> cn(ctx->tool_host.n_nodes), cs(ctx->tool_host.n_seg);
        for (int k = 0; k < n_cases; k++) {
            for (int i = 0; i < ctx->case_node_count[k]; i++) cn[ctx->case_node_first[k] + i] = (uint16_t)k;
            for (int i = 0; i < ctx->case_seg_count[k]; i++) cs[ctx->case_seg_first[k] + i] = (uint16_t)k;
        }
        DALLOC(d_node, cn.size());
        DALLOC(d_seg, cs.size());
        CK(cudaMemcpy(d_node, cn.data(), sizeof(uint16_t) * cn.size(), cudaMemcpyHostToDevice));
        if (!cs.empty()) CK(cudaMemcpy(d_seg, cs.data(), sizeof(uint16_t) * cs.size(), cudaMemcpyHostToDevice));
        ctx->K.case_of_node = d_node;
        ctx->K.case_of_seg = d_seg;
    }
    return finish_cases(ctx, cell_bound);
}

int sph_batch_n_cases(const sph_ctx *ctx, int32_t *n_cases) {
    if (!ctx || !n_cases) return SPH_ERR_INVALID;
    *n_cases = ctx->K.n_cases;
    return SPH_OK;
}

int sph_batch_case_info(const sph_ctx *ctx, int32_t k, int32_t *first, int32_t *count, double offset[2],
                        int32_t *seg_first, int32_t *seg_count, int32_t *node_first, int32_t *node_count) {
    if (!ctx || k < 0 || k >= (int32_t)ctx->case_first.size()) return SPH_ERR_INVALID;
    if (first) *first = ctx->case_first[k];
    if (count) *count = ctx->case_count[k];
    if (offset) {
        offset[0] = ctx->case_offset[2 * k];
        offset[1] = ctx->case_offset[2 * k + 1];
    }
    if (seg_first) *seg_first = ctx->case_seg_first[k];
    if (seg_count) *seg_count = ctx->case_seg_count[k];
    if (node_first) *node_first = ctx->case_node_first[k];
    if (node_count) *node_count = ctx->case_node_count[k];
    return SPH_OK;
}

int sph_batch_reduce(sph_ctx *ctx, double *out) {
    REQUIRE_CTX();
    REQUIRE_STATE(false);
    if (!out) return SPH_ERR_INVALID;
    const int n = (int)ctx->case_first.size();
    launch_reduce_cases(ctx->stream, n, CUR(ctx), ctx->in_cell_order ? ctx->X.offsets : nullptr,
                        ctx->case_cell_bound, ctx->case_part_bound, ctx->case_reduce);
    ctx->launches++;
    CK_LAUNCH();
    CK(cudaMemcpyAsync(out, ctx->case_reduce, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_batch_case_of_particles(sph_ctx *ctx, int32_t *case_of) {
    REQUIRE_CTX();
    REQUIRE_STATE(false);
    if (!case_of) return SPH_ERR_INVALID;
    const int n = (int)ctx->case_first.size();
    if (!ctx->in_cell_order || n == 1) {
        for (int k = 0; k < n; k++)
            for (int i = 0; i < ctx->case_count[k]; i++) case_of[ctx->case_first[k] + i] = k;
        return SPH_OK;
    }
    CK(cudaMemcpyAsync(case_of, CUR(ctx).hash, sizeof(int32_t) * ctx->N, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const int nx = ctx->K.g.nx, ny = ctx->K.g.ny;
    for (int i = 0; i < ctx->N; i++) {   // the device's case_of_hash
        int ix = case_of[i] / ny;
        ix = ix < 0 ? 0 : (ix >= nx ? nx - 1 : ix);
        case_of[i] = ctx->case_of_col_h[ix];
    }
    return SPH_OK;
}

// ---- return-mapping log, statistics, learned warm start -------------------------------------------
int sph_jc_log_enable(sph_ctx *ctx, int64_t capacity) {
    REQUIRE_CTX();
    if (capacity < 0) return SPH_ERR_INVALID;
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->jc_log) {
        cudaFree(ctx->jc_log);
        ctx->allocs.erase(std::find(ctx->allocs.begin(), ctx->allocs.end(), (void *)ctx->jc_log));
        ctx->jc_log = nullptr;
    }
    if (!ctx->jc_log_count) DALLOC(ctx->jc_log_count, 1);
    CK(cudaMemset(ctx->jc_log_count, 0, sizeof(unsigned long long)));
    ctx->jc_log_cap = capacity;
    if (capacity > 0) DALLOC(ctx->jc_log, (size_t)capacity * kJcLogWidth);
    ctx->K.jc_log = ctx->jc_log;
    ctx->K.jc_log_count = ctx->jc_log_count;
    ctx->K.jc_log_cap = capacity;
    invalidate_graphs(ctx);
    return SPH_OK;
}

int sph_jc_log_read(sph_ctx *ctx, float *records, int64_t max_records, int64_t *n_offered) {
    REQUIRE_CTX();
    unsigned long long n = 0;
    if (ctx->jc_log_count) {
        CK(cudaMemcpyAsync(&n, ctx->jc_log_count, sizeof(n), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    if (n_offered) *n_offered = (int64_t)n;
    const int64_t held = std::min<int64_t>((int64_t)n, ctx->jc_log_cap);
    const int64_t m = std::min<int64_t>(held, max_records);
    if (records && m > 0) {
        CK(cudaMemcpyAsync(records, ctx->jc_log, sizeof(float) * kJcLogWidth * (size_t)m, cudaMemcpyDeviceToHost,
                           ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return SPH_OK;
}

int sph_jc_stats(sph_ctx *ctx, int32_t enable, int64_t *out, int32_t reset) {
    REQUIRE_CTX();
    unsigned long long h[2] = {0, 0};
    CK(cudaMemcpyAsync(h, ctx->jc_stats, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    if (reset) CK(cudaMemsetAsync(ctx->jc_stats, 0, sizeof(h), ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (out) {
        out[0] = (int64_t)h[0];
        out[1] = (int64_t)h[1];
    }
    unsigned long long *want = enable ? ctx->jc_stats : nullptr;
    if (ctx->K.jc_stats != want) {
        ctx->K.jc_stats = want;
        invalidate_graphs(ctx);
    }
    return SPH_OK;
}

int sph_mlp_attach(sph_ctx *ctx, const sph_mlp *m) {
    REQUIRE_CTX();
    CK(cudaStreamSynchronize(ctx->stream));
    if (!m) {
        ctx->mlp_on = false;
        ctx->K.jc_list = nullptr;
        ctx->K.jc_list_count = nullptr;
        invalidate_graphs(ctx);
        return SPH_OK;
    }
    if (ctx->K.precision != SPH_PREC_FP32K)
        return fail(ctx, SPH_ERR_STATE, "the learned warm start runs in the FP32K return mapping");
    if (m->device != ctx->device) return fail(ctx, SPH_ERR_INVALID, "network on another device");
    CK(mlp_configure());
    if (!ctx->mlp_params) {
        DALLOC(ctx->mlp_params, kMlpParams);
        DALLOC(ctx->mlp_wb, kMlpWb);
        DALLOC(ctx->jc_list, ctx->N);
        DALLOC(ctx->jc_list_count, 1);
    }
    CK(cudaStreamSynchronize(m->stream));
    CK(cudaMemcpy(ctx->mlp_params, m->params, sizeof(float) * kMlpParams, cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(ctx->mlp_wb, m->wb, sizeof(uint16_t) * kMlpWb, cudaMemcpyDeviceToDevice));
    ctx->mlp = mlp_view(m, ctx->mlp_params, ctx->mlp_wb);
    ctx->mlp_on = true;
    ctx->K.jc_list = ctx->jc_list;
    ctx->K.jc_list_count = ctx->jc_list_count;
    invalidate_graphs(ctx);
    return SPH_OK;
}

int sph_mlp_set_inference(sph_ctx *ctx, int32_t mode) {
    REQUIRE_CTX();
    if (mode != SPH_MLP_WARP && mode != SPH_MLP_TENSOR) return fail(ctx, SPH_ERR_INVALID, "unknown inference mode");
    if (mode != ctx->mlp_mode) {
        CK(cudaStreamSynchronize(ctx->stream));
        ctx->mlp_mode = mode;
        invalidate_graphs(ctx);
    }
    return SPH_OK;
}

// ---- launch shapes (autotuning) -------------------------------------------------------------------
int sph_launch_variants(int32_t *n, int32_t *block, int32_t *min_blocks, int32_t *staged_records,
                        int32_t *lanes_per_particle) {
    if (!n) return SPH_ERR_INVALID;
    const int nv = interact_variant_count();
    for (int v = 0; v < nv && v < *n; v++) {
        int b, m, st, l;
        interact_variant_shape(v, &b, &m, &st, &l);
        if (block) block[v] = b;
        if (min_blocks) min_blocks[v] = m;
        if (staged_records) staged_records[v] = st;
        if (lanes_per_particle) lanes_per_particle[v] = l;
    }
    *n = nv;
    return SPH_OK;
}

int sph_set_launch_config(sph_ctx *ctx, const sph_launch_config *cfg) {
    REQUIRE_CTX();
    if (!cfg || cfg->interact_variant < 0 || cfg->interact_variant >= interact_variant_count())
        return fail(ctx, SPH_ERR_INVALID, "unknown launch variant");
    if (cfg->step_form != SPH_STEP_LAUNCHES && cfg->step_form != SPH_STEP_PERSISTENT)
        return fail(ctx, SPH_ERR_INVALID, "unknown step form");
    if (cfg->step_form == SPH_STEP_PERSISTENT && ctx->K.precision != SPH_PREC_FP32K)
        return fail(ctx, SPH_ERR_STATE, "the persistent step runs the FP32K form");
    if (cfg->step_form == SPH_STEP_PERSISTENT && !ctx->grid_bar) {
        CK(cudaStreamSynchronize(ctx->stream));
        DALLOC(ctx->grid_bar, 4);
    }
    if (cfg->interact_variant != ctx->interact_variant || cfg->step_form != ctx->step_form) {
        CK(cudaStreamSynchronize(ctx->stream));
        ctx->interact_variant = cfg->interact_variant;
        ctx->step_form = cfg->step_form;
        invalidate_graphs(ctx);
    }
    return SPH_OK;
}

int sph_set_test_faults(sph_ctx *ctx, uint32_t faults, int32_t secant_cap) {
    REQUIRE_CTX();
    if (faults & ~(SPH_TEST_SKIP_BULK_COPY | SPH_TEST_SKIP_MMA | SPH_TEST_SKIP_GRID_ARRIVAL))
        return fail(ctx, SPH_ERR_INVALID, "unknown test fault");
    ctx->K.test_faults = faults;
    ctx->K.secant_cap = secant_cap >= 0 ? secant_cap : 100;
    invalidate_graphs(ctx);   // the graphs hold the constants by value
    return SPH_OK;
}

int sph_get_launch_config(const sph_ctx *ctx, sph_launch_config *cfg) {
    if (!ctx || !cfg) return SPH_ERR_INVALID;
    cfg->interact_variant = ctx->interact_variant;
    cfg->step_form = ctx->step_form;
    return SPH_OK;
}

// ---- output in the reference's formats (vtk_writer.cu, mfree_gpu.cpp) ------------------------------
namespace {
int write_fail(sph_ctx *ctx, FILE *fp, const std::string &what) {
    if (fp) fclose(fp);
    return fail(ctx, SPH_ERR_INVALID, what);
}
}  // namespace

int sph_write_vtk_particles(sph_ctx *ctx, const char *path) {
    REQUIRE_CTX();
    if (!path) return SPH_ERR_INVALID;
    const int n = ctx->N;
    std::vector<double> pos(2 * (size_t)n), vel(2 * (size_t)n), fc(2 * (size_t)n), ft(2 * (size_t)n),
        nrm(2 * (size_t)n), S(4 * (size_t)n), p(n), T(n), eps(n), blanked(n);
    std::vector<int32_t> on_seg(n);
    sph_particles h;
    std::memset(&h, 0, sizeof(h));
    h.N = n;
    h.pos = pos.data(); h.vel = vel.data(); h.fc = fc.data(); h.ft = ft.data(); h.n = nrm.data();
    h.S = S.data(); h.p = p.data(); h.T = T.data(); h.eps_pl = eps.data(); h.blanked = blanked.data();
    h.on_seg = on_seg.data();
    int r = sph_download_particles(ctx, &h);
    if (r) return r;
    if (sph_vtk_write_particles_host(&h, path) != SPH_OK) return fail(ctx, SPH_ERR_INVALID, std::string("cannot write ") + path);
    return SPH_OK;
}

int sph_write_vtk_tool(sph_ctx *ctx, const char *path, const double *tl_ref) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    if (!path) return SPH_ERR_INVALID;
    const ToolModelHost &M = ctx->tool_host;
    const int nn = ctx->fem.n_nodes;
    std::vector<double> position(2 * (size_t)nn), T(nn);
    CK(cudaMemcpyAsync(position.data(), ctx->fem.position, 16 * (size_t)nn, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(T.data(), ctx->fem.T, 8 * (size_t)nn, cudaMemcpyDeviceToHost, ctx->stream));
    double shift[2] = {0., 0.};
    if (tl_ref) {   // vtk_writer.cu:518-587: the tool moved back by its travel since tl_ref
        ToolDev td;
        CK(cudaMemcpyAsync(&td, ctx->tool_dev, sizeof(td), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        shift[0] = td.tl_point_ref[0] - tl_ref[0];
        shift[1] = td.tl_point_ref[1] - tl_ref[1];
    }
    CK(cudaStreamSynchronize(ctx->stream));
    const int ne = M.n_elements;
    std::vector<int32_t> el(4 * (size_t)ne);
    for (int e = 0; e < ne; e++) {
        el[4 * e] = M.elements[e].x;
        el[4 * e + 1] = M.elements[e].y;
        el[4 * e + 2] = M.elements[e].z;
        el[4 * e + 3] = M.elements[e].w;
    }
    if (sph_vtk_write_tool_host(nn, position.data(), T.data(), ne, el.data(), tl_ref ? shift : nullptr, path) != SPH_OK)
        return fail(ctx, SPH_ERR_INVALID, std::string("cannot write ") + path);
    return SPH_OK;
}

// vtk_writer.cu:368-516 vtk_writer_write_FEM_segments: every contact segment as a
// triangle (left, right, and right + |segment| n), with the wear statistics on
// the third point: mean pressure (GPa), sliding speed (m/s), segment
// temperature, frictional stress and wear rate (1e10 x).  Without gathered
// statistics the wear fields are zero.
int sph_write_vtk_segments(sph_ctx *ctx, const char *path) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    if (!path) return SPH_ERR_INVALID;
    const int ns = ctx->seg.n;
    std::vector<double> left(2 * (size_t)ns), right(2 * (size_t)ns), n(2 * (size_t)ns), wear(4 * (size_t)ns, 0.),
        sf(ns, 0.), wr(ns, 0.);
    CK(cudaMemcpyAsync(left.data(), ctx->seg.left, 16 * (size_t)ns, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(right.data(), ctx->seg.right, 16 * (size_t)ns, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(n.data(), ctx->seg.normal, 16 * (size_t)ns, cudaMemcpyDeviceToHost, ctx->stream));
    if (ctx->wear_ready) {
        CK(cudaMemcpyAsync(wear.data(), ctx->wear_pp, 32 * (size_t)ns, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(sf.data(), ctx->wear_sf, 8 * (size_t)ns, cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(wr.data(), ctx->seg.wear_rate, 8 * (size_t)ns, cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    const bool stats = ctx->wear_ready;
    if (sph_vtk_write_segments_host(ns, left.data(), right.data(), n.data(), stats ? wear.data() : nullptr,
                                    stats ? sf.data() : nullptr, stats ? wr.data() : nullptr, path) != SPH_OK)
        return fail(ctx, SPH_ERR_INVALID, std::string("cannot write ") + path);
    return SPH_OK;
}

int sph_append_force_log(sph_ctx *ctx, const char *path) {
    REQUIRE_CTX();
    if (!path) return SPH_ERR_INVALID;
    double f[2];
    int r = sph_reduce_force(ctx, f);
    if (r) return r;
    FILE *fp = fopen(path, "a");
    if (!fp) return fail(ctx, SPH_ERR_INVALID, std::string("cannot open ") + path);
    fprintf(fp, "%.9g %.9g\n", f[0], f[1]);   // mfree_gpu.cpp:336-338
    if (fclose(fp) != 0) return write_fail(ctx, nullptr, std::string("cannot write ") + path);
    return SPH_OK;
}

// ---- tool_wear::eval_usui (tool_wear.cu:14-54) --------------------------------------------------
int sph_eval_usui(sph_ctx *ctx, double K_usui, double alpha, const double tool_vel[2], double dt, double out[3],
                  double *accum_wear) {
    REQUIRE_CTX();
    REQUIRE_STATE(false);
    if (!tool_vel || !out) return SPH_ERR_INVALID;
    const int nb = reduce_blocks();
    std::vector<double> h(4 * (size_t)nb);
    double *dev = nullptr;
    if (!ctx->usui_scratch) DALLOC(ctx->usui_scratch, 4 * (size_t)nb);
    dev = ctx->usui_scratch;
    launch_usui(ctx->stream, ctx->N, CUR(ctx), K_usui, alpha, tool_vel[0], tool_vel[1], dev);
    ctx->launches++;
    CK_LAUNCH();
    CK(cudaMemcpyAsync(h.data(), dev, sizeof(double) * 4 * nb, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    double mn = 1.7976931348623157e308, mx = 0., sm = 0., cnt = 0.;
    for (int b = 0; b < nb; b++) {
        mn = std::fmin(mn, h[4 * b]);
        mx = std::fmax(mx, h[4 * b + 1]);
        sm += h[4 * b + 2];
        cnt += h[4 * b + 3];
    }
    out[0] = cnt == 0. ? 0. : mn;
    out[1] = mx;
    out[2] = cnt == 0. ? 0. : sm / cnt;
    if (accum_wear) *accum_wear += dt * out[2];
    return SPH_OK;
}


// ---- rigid (SPH-mode) tool and PSE conduction: leap_frog.cu:99-160 --------------------------------
int sph_set_rigid_tool(sph_ctx *ctx, const sph_rigid_tool *tool) {
    REQUIRE_CTX();
    REQUIRE_SINGLE_CASE();
    if (!tool) {   // remove it (the allocation stays with the context)
        if (ctx->K.rigid) {
            ctx->K.rigid = nullptr;
            invalidate_graphs(ctx);
        }
        return SPH_OK;
    }
    if (ctx->has_tool) return fail(ctx, SPH_ERR_STATE, "context has a FEM tool");
    if (tool->n_seg < 1 || tool->n_seg > SPH_RIGID_MAX_SEG)
        return fail(ctx, SPH_ERR_INVALID, "rigid tool: 1..5 segments");
    // tool_gpu.cu:83: a fillet exists exactly when the outline has 5 segments
    if ((tool->has_fillet != 0) != (tool->n_seg == SPH_RIGID_MAX_SEG))
        return fail(ctx, SPH_ERR_INVALID, "rigid tool: a fillet goes with 5 segments, and 5 segments with a fillet");
    if (!ctx->rigid_dev) DALLOC(ctx->rigid_dev, 1);
    CK(cudaMemcpyAsync(ctx->rigid_dev, tool, sizeof(sph_rigid_tool), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->K.rigid != ctx->rigid_dev) {
        ctx->K.rigid = ctx->rigid_dev;
        invalidate_graphs(ctx);
    }
    return SPH_OK;
}

int sph_get_rigid_tool(sph_ctx *ctx, sph_rigid_tool *tool) {
    REQUIRE_CTX();
    if (!tool) return SPH_ERR_INVALID;
    if (!ctx->K.rigid) return fail(ctx, SPH_ERR_STATE, "context has no rigid tool");
    CK(cudaMemcpyAsync(tool, ctx->K.rigid, sizeof(sph_rigid_tool), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

// tool_gpu.cu:266-305 tool_gpu_update_tool: segments and fillet (tool.cpp:202-212),
// then the tool particles (update_tool_particles), by the context's time step.
int sph_rigid_tool_update(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    if (!ctx->K.rigid) return fail(ctx, SPH_ERR_STATE, "context has no rigid tool");
    launch_rigid_move(ctx->stream, ctx->K.rigid, ctx->K.dt);
    launch_rigid_move_particles(ctx->stream, ctx->N, CUR(ctx), ctx->K.rigid, ctx->K.dt);
    ctx->launches += 2;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

// tool_gpu.cu:307-313 compute_contact_forces
int sph_compute_contact_forces(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    if (!ctx->K.rigid) return fail(ctx, SPH_ERR_STATE, "context has no rigid tool");
    launch_contact_rigid(ctx->stream, ctx->N, ctx->K, CUR(ctx));
    ctx->launches++;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

// actions_gpu.cu:955-965 material_fric_heat_gen (off while thermals_wp.eta == 0)
int sph_material_fric_heat_gen(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    if (!ctx->K.rigid) return fail(ctx, SPH_ERR_STATE, "context has no rigid tool");
    if (ctx->K.c.trml_wp.eta == 0.) return SPH_OK;
    launch_fric_heat_rigid(ctx->stream, ctx->N, ctx->K, CUR(ctx));
    ctx->launches++;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

// types.h:11-13,122-123: the thermal solver of the build, Brookshaw or PSE.  PSE
// sums over the reference's 5x5 block of cells of edge h, so it needs the
// reference's cell geometry (cell_factor 1).
int sph_set_thermal_model(sph_ctx *ctx, int32_t model) {
    REQUIRE_CTX();
    if (model != SPH_THERMAL_BROOKSHAW && model != SPH_THERMAL_PSE)
        return fail(ctx, SPH_ERR_INVALID, "unknown thermal model");
    const int32_t pse = model == SPH_THERMAL_PSE ? 1 : 0;
    if (pse) {
        if (ctx->grid.cell_factor != 1) return fail(ctx, SPH_ERR_STATE, "PSE conduction needs cells of edge h");
        if (ctx->K.n_cases > 1) return fail(ctx, SPH_ERR_STATE, "PSE conduction: single-case contexts only");
    }
    if (pse != ctx->K.thermal_pse) {
        ctx->K.thermal_pse = pse;
        invalidate_graphs(ctx);
    }
    return SPH_OK;
}

// interactions_gpu.cu:434-462 interactions_heat_pse on the current state
int sph_interactions_heat_pse(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_STATE(true);
    if (!ctx->K.thermal_pse) return fail(ctx, SPH_ERR_STATE, "thermal model is not PSE");
    if (ctx->K.c.trml_wp.alpha == 0.) return SPH_OK;
    launch_build_records(ctx->stream, ctx->N, ctx->K, CUR(ctx), ctx->F, ctx->W);
    launch_heat_pse(ctx->stream, ctx->N, ctx->K, ctx->X.offsets, ctx->W, CUR(ctx));
    ctx->launches += 2;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}


// ---- tool wear by nodal shift (WEAR_NODE_SHIFT) ---------------------------------------------------
namespace {
// Device layer data and per-segment statistics, allocated on first use.
int wear_setup(sph_ctx *ctx) {
    if (ctx->wear_ready) return SPH_OK;
    const ToolModelHost &M = ctx->tool_host;
    SegDev &S = ctx->seg;
    FemDev &Fm = ctx->fem;
    WearDev &W = ctx->wear;
    DALLOC(ctx->wear_pp, S.n);
    DALLOC(ctx->wear_sf, S.n);
    DALLOC(S.wear_rate, S.n);
    if (!Fm.M) DALLOC(Fm.M, Fm.n_nodes);   // the device assembly's lumped mass (after Dirichlet)
    int32_t *node = nullptr, *adj_ptr = nullptr;
    int4 *adj = nullptr, *slot = nullptr, *elements = ctx->fem_elements;
    DALLOC(node, M.wear_node.size());
    DALLOC(adj_ptr, M.wear_adj_ptr.size());
    DALLOC(adj, M.wear_adj.size());
    DALLOC(slot, M.wear_slot.size());
    if (!elements) DALLOC(elements, M.elements.size());
    DALLOC(W.seg_delta, S.n);
    int32_t *elem = nullptr;
    DALLOC(elem, M.wear_elem.size());
    DALLOC(W.mat_old, 10 * M.wear_elem.size());
    DALLOC(W.mat_new, 10 * M.wear_elem.size());
    if (!M.wear_elem.empty())
        CK(cudaMemcpyAsync(elem, M.wear_elem.data(), sizeof(int32_t) * M.wear_elem.size(), cudaMemcpyHostToDevice,
                           ctx->stream));
    CK(cudaMemsetAsync(ctx->wear_pp, 0, sizeof(dbl4) * S.n, ctx->stream));
    CK(cudaMemsetAsync(ctx->wear_sf, 0, sizeof(double) * S.n, ctx->stream));
    CK(cudaMemsetAsync(S.wear_rate, 0, sizeof(double) * S.n, ctx->stream));
    CK(cudaMemsetAsync(W.seg_delta, 0, sizeof(dbl4) * S.n, ctx->stream));
    if (!M.wear_node.empty()) {
        CK(cudaMemcpyAsync(node, M.wear_node.data(), sizeof(int32_t) * M.wear_node.size(), cudaMemcpyHostToDevice,
                           ctx->stream));
        CK(cudaMemcpyAsync(adj, M.wear_adj.data(), sizeof(int4) * M.wear_adj.size(), cudaMemcpyHostToDevice,
                           ctx->stream));
        CK(cudaMemcpyAsync(slot, M.wear_slot.data(), sizeof(int4) * M.wear_slot.size(), cudaMemcpyHostToDevice,
                           ctx->stream));
    }
    CK(cudaMemcpyAsync(adj_ptr, M.wear_adj_ptr.data(), sizeof(int32_t) * M.wear_adj_ptr.size(),
                       cudaMemcpyHostToDevice, ctx->stream));
    if (elements != ctx->fem_elements)
        CK(cudaMemcpyAsync(elements, M.elements.data(), sizeof(int4) * M.elements.size(), cudaMemcpyHostToDevice,
                           ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    W.n_elem = (int)M.wear_elem.size();
    W.elem = elem;
    W.n_nodes = (int)M.wear_node.size();
    W.node = node;
    W.adj_ptr = adj_ptr;
    W.adj = adj;
    W.slot = slot;
    W.elements = elements;
    S.wear.marks = S.marks;
    ctx->wear_ready = true;
    return SPH_OK;
}
}  // namespace

int sph_set_wear(sph_ctx *ctx, int32_t mode, const sph_wear_constants *wc) {
    REQUIRE_CTX();
    REQUIRE_SINGLE_CASE();
    REQUIRE_TOOL();
    if (mode != SPH_WEAR_OFF && mode != SPH_WEAR_ACCUMULATE && mode != SPH_WEAR_SHIFT)
        return fail(ctx, SPH_ERR_INVALID, "unknown wear mode");
    if (mode == SPH_WEAR_SHIFT && !wc) return fail(ctx, SPH_ERR_INVALID, "nodal shift needs the wear constants");
    if (mode != SPH_WEAR_OFF) {
        int r = wear_setup(ctx);
        if (r) return r;
    }
    WearDev &W = ctx->wear;
    bool changed = mode != ctx->wear_mode;
    if (wc && (wc->A != W.A || wc->B != W.B || wc->C != W.C || wc->D != W.D)) {
        W.A = wc->A; W.B = wc->B; W.C = wc->C; W.D = wc->D;
        changed = true;
    }
    ctx->wear_mode = mode;
    // the friction heat gathers the statistics only while wear is on
    const bool on = mode != SPH_WEAR_OFF;
    ctx->seg.wear.pp = on ? ctx->wear_pp : nullptr;
    ctx->seg.wear.sf = on ? ctx->wear_sf : nullptr;
    if (changed) invalidate_graphs(ctx);
    return SPH_OK;
}

int sph_remesh_low_level(sph_ctx *ctx, int32_t freq) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    REQUIRE_SINGLE_CASE();
    const ToolModelHost &M = ctx->tool_host;
    FemDev &Fm = ctx->fem;
    if (!ctx->fem_node_edge) {
        DALLOC(ctx->fem_node_edge, Fm.n_nodes);
        DALLOC(ctx->fem_pos_old, Fm.n_nodes);
        DALLOC(ctx->fem_T_map, Fm.n_nodes);
        CK(cudaMemcpyAsync(ctx->fem_node_edge, M.node_edge.data(), sizeof(int32_t) * Fm.n_nodes,
                           cudaMemcpyHostToDevice, ctx->stream));
    }
    launch_remesh_low_level(ctx->stream, Fm, ctx->fem_elements, M.n_elements, M.n_colors, ctx->fem_node_edge,
                            ctx->tool_dev, freq, ctx->fem_dir_elems, ctx->fem_dir_flags, ctx->fem_n_dir, ctx->K.c.tool,
                            ctx->fem_pos_old, ctx->fem_T_map);
    ctx->launches += M.n_colors + 5;
    CK_LAUNCH();
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_segments_wear_rate_reset(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    if (ctx->wear_mode == SPH_WEAR_OFF) return fail(ctx, SPH_ERR_STATE, "wear is off");
    launch_wear_reset(ctx->stream, ctx->seg);
    CK_LAUNCH();
    return SPH_OK;
}

int sph_wear_adjustment(sph_ctx *ctx) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    if (ctx->wear_mode != SPH_WEAR_SHIFT) return fail(ctx, SPH_ERR_STATE, "nodal-shift wear is off");
    launch_wear_adjustment(ctx->stream, ctx->K, ctx->fem, ctx->seg, ctx->wear, ctx->tool_dev, ctx->K.dt);
    ctx->launches += 6;
    ctx->counts_valid = false;
    CK_LAUNCH();
    return SPH_OK;
}

int sph_download_wear(sph_ctx *ctx, sph_wear_state *h) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    if (!h) return SPH_ERR_INVALID;
    const ToolModelHost &M = ctx->tool_host;
    h->n_elements = M.n_elements;
    h->n_seg = ctx->seg.n;
    const size_t ne = (size_t)M.n_elements, ns = (size_t)ctx->seg.n, nn = (size_t)ctx->fem.n_nodes;
    if (h->elements) std::memcpy(h->elements, M.elements.data(), sizeof(int32_t) * 4 * ne);
    if (h->layer)
        for (size_t e = 0; e < ne; e++) {
            h->layer[2 * e] = M.layer[e].x;
            h->layer[2 * e + 1] = M.layer[e].y;
        }
    const bool dev = ctx->wear_ready;
    if (h->M) {
        if (dev) CK(cudaMemcpyAsync(h->M, ctx->fem.M, sizeof(double) * nn, cudaMemcpyDeviceToHost, ctx->stream));
        else std::memcpy(h->M, M.M.data(), sizeof(double) * nn);
    }
    if (h->phys_para) {
        if (dev) CK(cudaMemcpyAsync(h->phys_para, ctx->wear_pp, sizeof(dbl4) * ns, cudaMemcpyDeviceToHost, ctx->stream));
        else std::memset(h->phys_para, 0, sizeof(double) * 4 * ns);
    }
    if (h->sliding_force) {
        if (dev) CK(cudaMemcpyAsync(h->sliding_force, ctx->wear_sf, sizeof(double) * ns, cudaMemcpyDeviceToHost,
                                    ctx->stream));
        else std::memset(h->sliding_force, 0, sizeof(double) * ns);
    }
    if (h->wear_nodes) {
        if (dev) CK(cudaMemcpyAsync(h->wear_nodes, ctx->seg.wear_rate, sizeof(double) * ns, cudaMemcpyDeviceToHost,
                                    ctx->stream));
        else std::memset(h->wear_nodes, 0, sizeof(double) * ns);
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_upload_wear(sph_ctx *ctx, const sph_wear_state *h) {
    REQUIRE_CTX();
    REQUIRE_TOOL();
    if (!h) return SPH_ERR_INVALID;
    if (!ctx->wear_ready) return fail(ctx, SPH_ERR_STATE, "wear was never switched on in this context");
    const size_t ns = (size_t)ctx->seg.n, nn = (size_t)ctx->fem.n_nodes;
    if (h->M) {
        CK(cudaMemcpyAsync(ctx->fem.M, h->M, sizeof(double) * nn, cudaMemcpyHostToDevice, ctx->stream));
    }
    if (h->phys_para)
        CK(cudaMemcpyAsync(ctx->wear_pp, h->phys_para, sizeof(dbl4) * ns, cudaMemcpyHostToDevice, ctx->stream));
    if (h->sliding_force)
        CK(cudaMemcpyAsync(ctx->wear_sf, h->sliding_force, sizeof(double) * ns, cudaMemcpyHostToDevice, ctx->stream));
    if (h->wear_nodes)
        CK(cudaMemcpyAsync(ctx->seg.wear_rate, h->wear_nodes, sizeof(double) * ns, cudaMemcpyHostToDevice,
                           ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

}  // extern "C"
