// state.cuh -- device-side layout of the particle state and step scratch.
#pragma once

#include "common.cuh"

namespace sphfem {

// The 20 fields reordered by the Green sort (grid_gpu_green.cu:55-113) plus
// the sort keys; two copies, swapped after each sort like the reference.
struct SortedFields {
    double2 *pos, *vel, *fc, *ft, *n;
    double *h, *rho, *eps_pl, *eps_pl_dot, *T, *fixed, *blanked, *tool_particle;
    dbl4 *S;
    double2 *pos_t, *vel_t;
    double *rho_t, *T_t;
    dbl4 *S_t;
    int32_t *on_seg;
    int32_t *hash;
};

// The same fields in the compact form of FP32K contexts: positions and density
// in FP64 (the corrector's x + dt*x_t and rho + dt*rho_t, where FP32 would lose
// the small increments), everything else in FP32; the 0/1 flags as floats.
// 148 bytes per particle instead of 284.  Every value the FP32K step computes
// for these fields is an FP32 value already, so storing them in FP32 changes
// no result of the step except the contact forces and normals, which the
// contact search still computes in FP64 and now rounds once to FP32.
struct SortedFields32 {
    double2 *pos;
    float2 *vel, *fc, *ft, *n;
    float *h;
    double *rho;
    float *eps_pl, *eps_pl_dot, *T, *fixed, *blanked, *tool_particle;
    float4 *S;
    float2 *pos_t, *vel_t;
    float *rho_t, *T_t;
    float4 *S_t;
    int32_t *on_seg;
    int32_t *hash;
};

// Arrays that are not reordered by the sort (particle_gpu fields the Green
// buffer does not carry: p, R, S_der, v_der, idx).
struct FixedFields {
    double *p;
    dbl4 *R;
    dbl4 *S_der, *v_der;
    int32_t *idx;
};

// p and R of the FP32K step (R.w unused); S_der, v_der and idx stay in FixedFields.
struct FixedFields32 {
    float *p;
    float4 *R;
};

// Scratch of the counting sort.
struct SortScratch {
    int32_t *key;        // [N] sort key of each particle (hash, or num_cell when out of range)
    int32_t *hash_next;  // [N] raw hash taken by the histogram pass (the fused step keeps the
                         //     visible hash array as the reference leaves it until the next sort)
    int32_t *arrival;    // [N] arrival slot inside its cell (atomic counter value)
    int32_t *counts;     // [num_cell+1] particles per cell (last = out-of-grid bucket)
    int32_t *offsets;    // [num_cell+2] exclusive scan of counts
    int32_t *slots;      // [N] particle ids grouped by cell, arbitrary order inside a cell
    int32_t *block_sums; // scan partials
    int32_t *cell_start, *cell_end;   // grid_gpu_green m_cell_start / m_cell_end
};

// Packed neighbour record: what a neighbour contributes to the pair sums.
// FP64: 16 doubles = 128 B; FP32K: 16 floats = 64 B (positions as offsets
// from the particle's cell corner; the last word packs the cell row and flags).
constexpr int kRecWords = 16;
// kFlagNonFinite: a value of an active particle's record is NaN or infinite
// (its pair terms are NaN even with the zero kernel weights outside the
// support); never set on blanked records.
enum : int { kFlagBlanked = 1 << 30, kFlagTool = 1 << 29, kFlagNonFinite = 1 << 28, kRowMask = (1 << 28) - 1 };

// FP32K candidate entry, one float2 per record in the same order: the record's
// (xr, yr) for the in-support test of the candidate scan, 8 bytes instead of
// the record's first 16.  The flags ride in the low mantissa bits: xr's two
// lowest bits hold kCandBlanked / kCandNonFinite, yr's three lowest bits the
// cell row modulo 8 (the row difference to the summing particle is at most the
// stencil half-width, 3).  Each coordinate moves by at most 7 units in the
// last place of a value below a cell edge, so the test's support boundary
// moves by at most 2^-20 of a cell, where the kernel and its gradient vanish to
// third and second order; the pair terms themselves use the full record.
enum : int { kCandBlanked = 1, kCandNonFinite = 2 };
__device__ __forceinline__ float2 cand_pack(float xr, float yr, int flags) {
    const int bx = (__float_as_int(xr) & ~3) | ((flags & kFlagBlanked) ? kCandBlanked : 0) |
                   ((flags & kFlagNonFinite) ? kCandNonFinite : 0);
    const int by = (__float_as_int(yr) & ~7) | (flags & 7);
    return make_float2(__int_as_float(bx), __int_as_float(by));
}

// Per-segment constants of the contact search, rebuilt each step with the
// y-bins (k_seg_bins), after the tool has moved: what on_segment_mesh and the
// first loop of find_shortest_distance_v1 (actions_gpu.cu:51-63, :139-180)
// form per particle from the segment alone, computed once with the same
// operations -- so every test gives the reference's result bit for bit.
struct __align__(64) SegGeo {
    long long kx0, kx1, ky0, ky1;     // order keys of xmin - 0.0008, xmax + 0.0008, ymin - 0.0008, ymax + 0.0008
    double ymin_f, ymax_f;            // fminf / fmaxf of the end points' y (float-rounded)
    double inv_slope;                 // (left.x - right.x) / (left.y - right.y), non-horizontal segments
    long long pad;
};

// Interface segments (segment_FEM_gpu, segment_FEM_gpu.h:31-56).
struct SegDev {
    int n;
    double2 *left, *right, *normal;
    int4 *marks;              // element, colour, node left, node right
    double2 *heat_exchange;   // (sum T*length, sum length)
    double *fric_heat;
    WearAcc wear;             // wear statistics (pp == NULL: off)
    double *wear_rate;        // wear_nodes: per-segment wear rate of the last nodal shift
    // y-bins of each case's segments for the contact's ray casting (k_seg_bins):
    // bin_count[case * kSegBins + b] segments listed, -1 when the bin overflowed
    // (then the full scan runs); bin_list[(case * kSegBins + b) * kSegBinCap + k]
    // the case-local segment index.  NULL: no bins, full scan.
    int32_t *bin_count;
    int32_t *bin_list;
    // with the bins: per segment, SegGeo; per bin, the order key of an x bound
    // right of which no segment of the bin has a crossing (an empty bin: the
    // lowest key)
    SegGeo *geo;
    long long *bin_xkey;
};
constexpr int kSegBins = 64;
constexpr int kSegBinCap = 256;

// FEM thermal system of the tool (FEM_thermal_2D_GPU, FEM_thermal_gpu.h:35-93).
// K, f are the assembled (post-Dirichlet) m_stiffness_matrix / m_f; the Robin
// terms of apply_robin_bdc are added on the fly from the segments touching a
// node (node_seg_ptr / node_seg), so no K_temp/f_temp copy is made per step.
struct FemDev {
    int n_nodes, nnz;
    double2 *position;
    int32_t *row_ptr, *col_ind, *diag;   // diag[i] = CSR slot of (i,i)
    double *K, *M_inv, *f, *T, *k;
    double *T_half;                      // T after calculate_temp(0.5 dt)
    int32_t *node_seg_ptr, *node_seg;    // segments whose left/right node is this node
    double *M;                           // lumped mass (m_mass_matrix); allocated with wear only
};

// Wear by nodal shift: the nodes of the two cutting-edge layers, each with its
// layer elements (x: element, y: the node's local index) and the CSR slots of
// (node, element node b), b = 0..2, for the atomic-free retreat / resume of the
// layers' mass and stiffness; the per-segment node shifts; the wear constants.
struct WearDev {
    int n_elem;                          // layer elements
    const int32_t *elem;                 // [n_elem] element ids
    double *mat_old, *mat_new;           // [n_elem][10]: lumped mass, stiffness (row-major) before / after the shift
    int n_nodes;                         // nodes of layer elements
    const int32_t *node;                 // [n_nodes] node ids
    const int32_t *adj_ptr;              // [n_nodes + 1]
    const int4 *adj;                     // (layer element index, local index)
    const int4 *slot;                    // CSR slots (x, y, z)
    const int4 *elements;                // [n_elements] node a, b, c, colour
    dbl4 *seg_delta;                     // [n_seg] shift of the left (x, y) and right (z, w) node
    double A, B, C, D;                   // wear constants (constants_structs.h:113-119)
};

struct StepScratch {
    dbl4 *rec64;      // [N][4] FP64 records
    float4 *rec32;       // [N][4] FP32 records
    float2 *cand32;      // [N] candidate entries of the FP32 records (cand_pack)
    double2 *pos_init, *vel_init;   // leap_frog snapshots (staged path)
    dbl4 *S_init;
    double *rho_init, *T_init;
    int32_t *secant_iters;          // [N] secant iterations of the last JC pass (0 = elastic)
    uint32_t *status;               // device status word
    double *reduce;                 // reduction scratch
};

// The learned warm start of the return mapping: a 4-64-64-64-1 SiLU MLP.
// Parameters in FP32 (layout kMlp* offsets); BF16 copies of the four weight
// matrices feed the tensor cores.  Features and target are standardised with
// the training set's moments.
constexpr int kMlpIn = 4, kMlpH = 64;
constexpr int kMlpOffW1 = 0, kMlpOffB1 = 256, kMlpOffW2 = 320, kMlpOffB2 = 4416, kMlpOffW3 = 4480,
              kMlpOffB3 = 8576, kMlpOffW4 = 8640, kMlpOffB4 = 8704, kMlpParams = 8705;
// BF16 weight copies: W1 [64][4], W2 [64][64], W3 [64][64], W4 [64]
constexpr int kMlpWbW1 = 0, kMlpWbW2 = 256, kMlpWbW3 = 4352, kMlpWbW4 = 8448, kMlpWb = 8512;

struct MlpDev {
    const float *params;      // [kMlpParams] FP32 (biases are read from here)
    const uint16_t *wb;       // [kMlpWb] BF16 bit patterns of the weights
    float x_mean[4], x_inv_std[4], y_mean, y_std;
};

}  // namespace sphfem
