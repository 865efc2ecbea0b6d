// rigid.cuh -- the reference's rigid (SPH-mode) tool: segment motion, contact
// search, penalty contact with LS-DYNA friction and the friction heat of
// do_material_fric_heat_gen, one particle at a time.
#pragma once

#include "common.cuh"

namespace sphfem {

constexpr double kRigidFltMax = 3.402823466385288598e38;   // FLT_MAX, the reference's "no distance"
constexpr double kRigidPi = 3.14159265358979323846;

// geometric_primitives.cpp:58-75 line(p1, p2): y = a x + b through two points,
// x = b when the points share x (|det| < 1e-12).  The reference evaluates this
// on the host without fused multiply-adds; the explicit roundings keep the
// device copy identical to it.
__device__ __forceinline__ void rigid_line(double p1x, double p1y, double p2x, double p2y, double &a, double &b,
                                           int32_t &vertical) {
    const double det = __dsub_rn(p1x, p2x);
    if (fabs(det) < 1e-12) {
        vertical = 1;
        a = 1.7976931348623157e308;
        b = p1x;
        return;
    }
    vertical = 0;
    a = __ddiv_rn(__dsub_rn(p1y, p2y), det);
    b = __ddiv_rn(__dsub_rn(__dmul_rn(p2y, p1x), __dmul_rn(p2x, p1y)), det);
}

// tool.cpp update_tool: every segment end and the fillet centre move by dt * vel,
// the segment lines are rebuilt, the normals stay.
__device__ __forceinline__ void rigid_move(sph_rigid_tool &t, double dt) {
    const double dx = __dmul_rn(dt, t.vel[0]), dy = __dmul_rn(dt, t.vel[1]);
    for (int i = 0; i < t.n_seg; i++) {
        t.left[i][0] = __dadd_rn(t.left[i][0], dx);
        t.left[i][1] = __dadd_rn(t.left[i][1], dy);
        t.right[i][0] = __dadd_rn(t.right[i][0], dx);
        t.right[i][1] = __dadd_rn(t.right[i][1], dy);
        rigid_line(t.left[i][0], t.left[i][1], t.right[i][0], t.right[i][1], t.la[i], t.lb[i], t.vertical[i]);
    }
    if (t.has_fillet) {
        t.fillet_p[0] = __dadd_rn(t.fillet_p[0], dx);
        t.fillet_p[1] = __dadd_rn(t.fillet_p[1], dy);
    }
}

// glm::normalize: v * (1 / sqrt(dot(v, v))).
__device__ __forceinline__ double2 rigid_normalize(double x, double y) {
    const double inv = 1.0 / sqrt(x * x + y * y);
    return make_double2(x * inv, y * inv);
}

// tool_gpu.cu:33-57 circle_segment_distance: distance to the fillet arc if the
// closest point on the circle lies inside the arc's angle range, else FLT_MAX.
__device__ __forceinline__ double rigid_fillet_distance(const sph_rigid_tool &t, double qx, double qy) {
    const double Ax = t.fillet_p[0], Ay = t.fillet_p[1], r = t.fillet_r;
    const double dBx = qx - Ax, dBy = qy - Ay;
    const double len = sqrt(dBx * dBx + dBy * dBy);
    const double Cx = Ax + r * dBx / len, Cy = Ay + r * dBy / len;
    double th = atan2(Ay - Cy, Ax - Cx);   // myatan2: angles in (0, 2 pi]
    if (!(th > 0.)) th = th + 2 * kRigidPi;
    const bool valid = th > fmin(t.fillet_t1, t.fillet_t2) && th < fmax(t.fillet_t1, t.fillet_t2);
    if (!valid) return kRigidFltMax;
    const double ex = Cx - qx, ey = Cy - qy;
    return sqrt(ex * ex + ey * ey);
}

// tool_gpu.cu:59-75 segment_closest_point (line::closest_point).
__device__ __forceinline__ double2 rigid_closest(const sph_rigid_tool &t, int i, double qx, double qy) {
    if (t.vertical[i]) return make_double2(t.lb[i], qy);
    const double bb = -1., cc = t.lb[i], aa = t.la[i];
    const double den = aa * aa + bb * bb;
    const double px = (bb * (bb * qx - aa * qy) - aa * cc) / den;
    const double py = (aa * (-bb * qx + aa * qy) - bb * cc) / den;
    return make_double2(px, py);
}

// tool_gpu.cu:81-130 establish_contact: inside every segment's half-plane (or the
// fillet disc), then the nearest primitive gives the contact point and normal.
__device__ __forceinline__ bool rigid_establish_contact(const sph_rigid_tool &t, double qx, double qy, double2 &cp,
                                                        double2 &n) {
    bool in = true;
    for (int i = 0; i < t.n_seg; i++)
        in = in && ((t.left[i][0] - qx) * t.n[i][0] + (t.left[i][1] - qy) * t.n[i][1] < 0.);
    if (t.has_fillet) {
        const double ex = t.fillet_p[0] - qx, ey = t.fillet_p[1] - qy;
        in = in || sqrt(ex * ex + ey * ey) < t.fillet_r;
    }
    if (!in) return false;
    double depth = kRigidFltMax;
    for (int i = 0; i < t.n_seg; i++) {
        double d;
        if (t.vertical[i]) {
            d = fabs(t.left[i][0] - qx);
            if (d < depth) {
                depth = d;
                n = rigid_normalize(t.left[i][0] - qx, 0.);
                cp = make_double2(t.left[i][0], qy);
            }
        } else if (t.has_fillet && i == 2) {   // the fillet replaces the third segment
            d = rigid_fillet_distance(t, qx, qy);
            if (d < depth) {
                depth = d;
                n = rigid_normalize(qx - t.fillet_p[0], qy - t.fillet_p[1]);
                cp = make_double2(t.fillet_p[0] + n.x * t.fillet_r, t.fillet_p[1] + n.y * t.fillet_r);
            }
        } else {
            const double2 p = rigid_closest(t, i, qx, qy);
            const double ex = p.x - qx, ey = p.y - qy;
            d = sqrt(ex * ex + ey * ey);
            if (d < depth) {
                depth = d;
                n = make_double2(-t.n[i][0], -t.n[i][1]);
                cp = p;
            }
        }
    }
    return true;
}

// tool_gpu.cu:142-198 do_compute_contact_forces for one (non-tool) particle:
// penalty normal force (slave mass, contact alpha) and the LS-DYNA friction
// update from the previous friction force.
__device__ __forceinline__ void rigid_contact_one(const KConsts &K, const sph_rigid_tool &t, double dt, double2 pos,
                                                  double2 vel, double2 &fc, double2 &ft, double2 &nrm) {
    double2 cp = make_double2(0., 0.), n = make_double2(0., 0.);
    if (!rigid_establish_contact(t, pos.x, pos.y, cp, n)) {
        fc = make_double2(0., 0.);
        ft = make_double2(0., 0.);
        nrm = make_double2(0., 0.);
        return;
    }
    const double ms = K.c.phys.mass, alpha = K.c.tool.contact_alpha;
    const double dt2 = dt * dt;
    const double gN = (pos.x - cp.x) * n.x + (pos.y - cp.y) * n.y;
    const double s = -ms * gN;
    const double2 fN = make_double2(s * n.x / dt2 * alpha, s * n.y / dt2 * alpha);
    double2 fT = make_double2(0., 0.);
    if (t.mu != 0.) {
        const double vx = vel.x - t.vel[0], vy = vel.y - t.vel[1];
        const double vrx = vx - vx * n.x, vry = vy - vy * n.y;   // v - v*n, component-wise (glm)
        const double am = alpha * ms;
        const double kx = am * vrx / dt, ky = am * vry / dt;
        const double fy = t.mu * sqrt(fN.x * fN.x + fN.y * fN.y);
        const double sx = ft.x - kx, sy = ft.y - ky;
        const double ls = sqrt(sx * sx + sy * sy);
        fT = (ls > fy) ? make_double2(fy * sx / ls, fy * sy / ls) : make_double2(sx, sy);
    }
    fc = fN;
    ft = fT;
    nrm = n;
}

// actions_gpu.cu:316-343 do_material_fric_heat_gen for one (non-tool) particle:
// T += eta dt |ft| |v_rel| / (cp m), |.| narrowed to float as the reference's sqrtf.
__device__ __forceinline__ void rigid_fric_heat_one(const KConsts &K, double dt, const double *vel_tool, double2 vel,
                                                    double2 ft, double2 nrm, double &T) {
    const double f = sqrtf_d(ft.x * ft.x + ft.y * ft.y);
    if (f == 0.) return;
    const double vdx = vel.x - vel_tool[0], vdy = vel.y - vel_tool[1];
    const double vdn = vdx * nrm.x + vdy * nrm.y;
    const double vrx = vdx - vdn * nrm.x, vry = vdy - vdn * nrm.y;
    const double v = sqrtf_d(vrx * vrx + vry * vry);
    T += K.c.trml_wp.eta * dt * f * v / (K.c.trml_wp.cp * K.c.phys.mass);
}

}  // namespace sphfem
