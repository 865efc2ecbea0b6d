// ref_pin.cpp -- runs the reference's OWN host-compilable arithmetic to pin the
// oracle (test infrastructure; built into oracle/_ref/ only).
//
// kernels.cuh (cubic_spline, __host__ __device__) and plasticity.cuh
// (sigma_yield, opt_fun, solve_secant, __device__) contain no CUDA-only
// constructs, so a host C++ compiler builds them as ordinary functions (the
// __device__ attribute is ignored).  This harness includes them from the
// reference tree at build time; no reference source is copied.
//
// Usage: ref_pin spline|yield|secant  < input lines  > output lines
//   spline: pix piy pjx pjy hi                      -> w wx wy
//   yield : A B C n m Tmelt Tref epsdotref eps epsdot T -> sigma
//   secant: A B C n m Tmelt Tref epsdotref init tol normS eps T dt mu -> dlambda
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>
#include "types.h"
#include "constants_structs.h"
#include "kernels.cuh"
#include "plasticity.cuh"

static joco_constants jc_from(const double *v) {
    joco_constants jc = make_joco_constants();
    jc.A = v[0]; jc.B = v[1]; jc.C = v[2]; jc.n = v[3]; jc.m = v[4];
    jc.Tmelt = v[5]; jc.Tref = v[6]; jc.eps_dot_ref = v[7];
    return jc;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    double v[16];
    if (!strcmp(argv[1], "spline")) {
        while (scanf("%lf %lf %lf %lf %lf", v, v + 1, v + 2, v + 3, v + 4) == 5) {
            double2 a = make_double2(v[0], v[1]), b = make_double2(v[2], v[3]);
            double3 w = cubic_spline(a, b, v[4]);
            printf("%.17g %.17g %.17g\n", w.x, w.y, w.z);
        }
    } else if (!strcmp(argv[1], "yield")) {
        while (scanf("%lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf", v, v + 1, v + 2, v + 3, v + 4, v + 5,
                     v + 6, v + 7, v + 8, v + 9, v + 10) == 11) {
            printf("%.17g\n", sigma_yield(jc_from(v), v[8], v[9], v[10]));
        }
    } else if (!strcmp(argv[1], "secant")) {
        while (scanf("%lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf", v, v + 1, v + 2, v + 3,
                     v + 4, v + 5, v + 6, v + 7, v + 8, v + 9, v + 10, v + 11, v + 12, v + 13, v + 14) == 15) {
            printf("%.17g\n", solve_secant(jc_from(v), v[8], v[9], v[10], v[11], v[12], v[13], v[14]));
        }
    } else {
        return 2;
    }
    return 0;
}
