// Test infrastructure: the reference pin on the GPU.  Compiles the reference's
// own interactions_gpu.cu (unmodified, from the read-only reference tree) into
// a cubin for sm_103a; oracle/ref_gpu.py loads it through the CUDA driver API.
// Its texture references become the device-side stand-ins of
// ref_shim/texture_ref.h, bound by ref_bind_interactions below with the
// pointers and byte sizes of the reference's host wrappers
// (interactions_gpu.cu:381-463); its __constant__ blocks become plain device
// globals that ref_set_interactions_constants fills.
#include <cuda_runtime.h>
#include "texture_ref.h"
#undef __constant__
#define __constant__ __device__
#include "interactions_gpu.cu"

extern "C" __global__ void ref_set_interactions_constants(phys_constants ph, corr_constants co, geom_constants ge,
                                                          trml_constants tw, trml_constants tt, tool_constants to) {
    physics = ph;
    correctors = co;
    geometry = ge;
    trml = tw;
    trml_tool = tt;
    tc = to;
}

// pointers in the order pos, vel, S, R, h, rho, p, T, hash, tool_particle, fc,
// cells_start, cells_end; N particles, num_cell cells
extern "C" __global__ void ref_bind_interactions(const void *pos, const void *vel, const void *S, const void *R,
                                                 const void *h, const void *rho, const void *p, const void *T,
                                                 const void *hash, const void *tool_particle, const void *fc,
                                                 const void *cells_start, const void *cells_end, int N, int num_cell) {
    const unsigned long long n = (unsigned long long)N, d = sizeof(double);
    texture_ref_bind(pos_tex, pos, d * n * 2);
    texture_ref_bind(vel_tex, vel, d * n * 2);
    texture_ref_bind(S_tex, S, d * n * 4);
    texture_ref_bind(R_tex, R, d * n * 4);
    texture_ref_bind(h_tex, h, d * n);
    texture_ref_bind(rho_tex, rho, d * n);
    texture_ref_bind(p_tex, p, d * n);
    texture_ref_bind(T_tex, T, d * n);
    texture_ref_bind(hashes_tex, hash, sizeof(int) * n);
    texture_ref_bind(tool_particle_tex, tool_particle, d * n);
#if defined(USE_FEM_TOOL) && defined(SURFACE)   // fc_tex exists only in that build (interactions_gpu.cu:39-43)
    texture_ref_bind(fc_tex, fc, d * n * 2);
#endif
    texture_ref_bind(cells_start_tex, cells_start, sizeof(int) * (unsigned long long)num_cell);
    texture_ref_bind(cells_end_tex, cells_end, sizeof(int) * (unsigned long long)num_cell);
}

// the bindings of interactions_heat_pse (interactions_gpu.cu:443-451), with its
// byte sizes: the tool flags are bound over N ints of the N-double array
extern "C" __global__ void ref_bind_interactions_pse(const void *pos, const void *h, const void *rho, const void *T,
                                                     const void *hash, const void *tool_particle,
                                                     const void *cells_start, const void *cells_end, int N,
                                                     int num_cell) {
    const unsigned long long n = (unsigned long long)N, d = sizeof(double);
    texture_ref_bind(pos_tex, pos, d * n * 2);
    texture_ref_bind(h_tex, h, d * n);
    texture_ref_bind(rho_tex, rho, d * n);
    texture_ref_bind(T_tex, T, d * n);
    texture_ref_bind(hashes_tex, hash, sizeof(int) * n);
    texture_ref_bind(tool_particle_tex, tool_particle, sizeof(int) * n);
    texture_ref_bind(cells_start_tex, cells_start, sizeof(int) * (unsigned long long)num_cell);
    texture_ref_bind(cells_end_tex, cells_end, sizeof(int) * (unsigned long long)num_cell);
}
