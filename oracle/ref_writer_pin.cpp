// ref_writer_pin.cpp -- runs the reference's OWN output code for the host to
// pin the product's writers (test infrastructure; built into oracle/_ref/ only,
// from the read-only reference tree: vtk_writer.cu and output.cu, compiled as
// host C++ with the stand-in headers of oracle/ref_shim).
//
// The reference's writers copy their inputs from device memory with
// cudaMemcpy; here the "device" arrays are host arrays and cudaMemcpy is the
// stand-in below (a plain copy).  The reference objects are built around the
// arrays in zeroed storage with only the members the writers read set (their
// constructors allocate device memory and are not linked here).
//
// Usage: ref_writer_pin <input file> (in a directory holding results/).
// Input (native byte order): int32 N, n_nodes, n_elements, n_seg; then double
// arrays pos[2N] vel[2N] fc[2N] ft[2N] n[2N] S[4N] p[N] T[N] eps_pl[N] rho[N]
// h[N] fixed[N], int32 idx[N] on_seg[N]; double node_pos[2 n_nodes]
// node_T[n_nodes], int32 elements[4 n_elements]; double left[2 n_seg]
// right[2 n_seg] normal[2 n_seg] phys_para[4 n_seg] sliding_force[n_seg]
// wear_rate[n_seg]; double tl_point_ref[2] tl_ref[2].
// Writes results/vtk_out_000000.vtk, vtk_tool_000000.vtk, vtk_seg_000000.vtk,
// vtk_tool_org_000000.vtk and prints report_force: "force %.17g %.17g".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "output.h"
#include "vtk_writer.h"

extern "C" cudaError_t cudaMemcpy(void *dst, const void *src, size_t count, enum cudaMemcpyKind) {
    std::memcpy(dst, src, count);
    return cudaSuccess;
}

template <class T>
static T *zeroed() {   // storage for a reference object whose members are set by hand
    void *p = std::calloc(1, sizeof(T) + 64);
    return reinterpret_cast<T *>(p);
}

template <class T>
static T *read_array(FILE *fp, size_t n) {
    T *a = static_cast<T *>(std::calloc(n ? n : 1, sizeof(T)));
    if (n && std::fread(a, sizeof(T), n, fp) != n) {
        std::fprintf(stderr, "short input\n");
        std::exit(2);
    }
    return a;
}

int main(int argc, char **argv) {
    if (argc != 2) return 1;
    FILE *fp = std::fopen(argv[1], "rb");
    if (!fp) return 1;
    int32_t hdr[4];
    if (std::fread(hdr, 4, 4, fp) != 4) return 2;
    const int N = hdr[0], nn = hdr[1], ne = hdr[2], ns = hdr[3];
    particle_gpu *P = zeroed<particle_gpu>();
    P->N = N;
    P->pos = read_array<float2_t>(fp, N);
    P->vel = read_array<float2_t>(fp, N);
    P->fc = read_array<float2_t>(fp, N);
    P->ft = read_array<float2_t>(fp, N);
    P->n = read_array<float2_t>(fp, N);
    P->S = read_array<float4_t>(fp, N);
    P->p = read_array<float_t>(fp, N);
    P->T = read_array<float_t>(fp, N);
    P->eps_pl = read_array<float_t>(fp, N);
    P->rho = read_array<float_t>(fp, N);
    P->h = read_array<float_t>(fp, N);
    P->fixed = read_array<float_t>(fp, N);
    P->idx = read_array<int>(fp, N);
    P->on_seg = read_array<int>(fp, N);
    mesh_GPU_m *mesh = zeroed<mesh_GPU_m>();
    mesh->position = read_array<float2_t>(fp, nn);
    FEM_thermal_2D_GPU *fem = zeroed<FEM_thermal_2D_GPU>();
    fem->m_T = read_array<float_t>(fp, nn);
    mesh->node_num = read_array<int4>(fp, ne);
    segment_FEM_gpu *seg = zeroed<segment_FEM_gpu>();
    seg->segment_num = ns;
    seg->left = read_array<float2_t>(fp, ns);
    seg->right = read_array<float2_t>(fp, ns);
    seg->n = read_array<float2_t>(fp, ns);
    seg->physical_para = read_array<float4_t>(fp, ns);
    seg->sliding_force = read_array<float_t>(fp, ns);
    seg->wear_nodes = read_array<float_t>(fp, ns);
    double tl[4];
    if (std::fread(tl, 8, 4, fp) != 4) return 2;
    std::fclose(fp);
    tool_FEM *t = zeroed<tool_FEM>();
    t->node_number = nn;
    t->element_number = ne;
    t->cutting_segment_size = ns;
    t->mesh_GPU = mesh;
    t->FEM_solver = fem;
    t->segments_FEM = seg;
    t->tl_point_ref = vec2_t(tl[0], tl[1]);
    float2_t tl_ref;
    tl_ref.x = tl[2];
    tl_ref.y = tl[3];
    vtk_writer_write(P, 0);
    vtk_writer_write_FEM_tool(t, 0);
    vtk_writer_write_FEM_segments(t, 0);
    vtk_writer_write_tool_org(t, 0, tl_ref);
    float2_t f = report_force(P);
    std::printf("force %.17g %.17g\n", f.x, f.y);
    return 0;
}
