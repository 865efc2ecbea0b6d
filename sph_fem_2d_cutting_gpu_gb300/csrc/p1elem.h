// p1elem.h -- element matrices of the linear triangle: lumped mass and
// conduction stiffness (do_mass_ele_matrix_construction_p1q3 and
// do_stiffness_ele_matrix_construction_p1q3, FEM_thermal_gpu.cu:71-109).
// Shared by the host assembly of the tool's thermal system, its device
// assembly (fem.cu) and the device update of the cutting-edge layers under
// wear.  Every product and sum is a separately rounded operation (no fused
// multiply-add on the device; host code is compiled without contraction), so
// host and device give the same bits.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define SPH_HD __host__ __device__
#else
#define SPH_HD
#endif

namespace sphfem {

#ifdef __CUDA_ARCH__
#define P1_MUL(a, b) __dmul_rn((a), (b))
#define P1_ADD(a, b) __dadd_rn((a), (b))
#else
#define P1_MUL(a, b) ((a) * (b))
#define P1_ADD(a, b) ((a) + (b))
#endif

// Nodes (x0, y0), (x1, y1), (x2, y2); cp, rho, k of the tool.  m: the lumped
// mass each node of the element receives; ke: element stiffness (symmetric).
SPH_HD inline void p1_element(double x0, double y0, double x1, double y1, double x2, double y2, double cp,
                              double rho, double k, double &m, double ke[3][3]) {
    const double weights = 1. / 3. * 0.5;
    // jacobian columns: x1 - x0, x2 - x0
    const double j00 = x1 - x0, j01 = y1 - y0, j10 = x2 - x0, j11 = y2 - y0;
    const double det_signed = P1_ADD(P1_MUL(j00, j11), -P1_MUL(j10, j01));
    const double determinant = fabs(det_signed);
    m = P1_MUL(P1_MUL(P1_MUL(weights, cp), rho), determinant);
    // physical gradients of (1 - xi - eta, xi, eta): J^-T * grad_ref, with
    // J = [[j00, j10], [j01, j11]] (rows x, y; columns xi, eta) and
    // J^-T = (1 / det) [[j11, -j01], [-j10, j00]]
    const double inv = 1.0 / det_signed;
    const double gref[3][2] = {{-1., -1.}, {1., 0.}, {0., 1.}};
    double g[3][2];
    for (int a = 0; a < 3; a++) {
        g[a][0] = P1_MUL(inv, P1_ADD(P1_MUL(j11, gref[a][0]), -P1_MUL(j01, gref[a][1])));
        g[a][1] = P1_MUL(inv, P1_ADD(P1_MUL(-j10, gref[a][0]), P1_MUL(j00, gref[a][1])));
    }
    const double s = P1_MUL(P1_MUL(weights, 3.), P1_MUL(k, determinant));
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++)
            ke[a][b] = P1_MUL(s, P1_ADD(P1_MUL(g[a][0], g[b][0]), P1_MUL(g[a][1], g[b][1])));
}

}  // namespace sphfem
