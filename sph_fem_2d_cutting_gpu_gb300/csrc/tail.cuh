// tail.cuh -- per-particle bodies of the step's contact with the FEM tool and
// of its fused tail (boundary conditions, invalidation, next histogram), and
// the per-case segment y-bins of the contact search; shared by their kernels
// (actions.cu) and the persistent step kernel (persistent.cu).
#pragma once

#include "launch.cuh"
#include "rigid.cuh"

namespace sphfem {

// ---- actions_gpu.cu:787-824 do_invalidate: the rates tested -----------------------------------------
__device__ __forceinline__ bool isnaninf(double v) { return is_nan_or_inf(v); }

__device__ __forceinline__ bool invalid_rates(double2 pt, double2 vt, dbl4 St, double rho_t, double T_t) {
    return isnaninf(pt.x) || isnaninf(pt.y) || isnaninf(vt.x) || isnaninf(vt.y) || isnaninf(St.x) ||
           isnaninf(St.y) || isnaninf(St.z) || isnaninf(St.w) || isnaninf(rho_t) || isnaninf(T_t);
}
// the compact FP32 state: the same test on its FP32 rates
__device__ __forceinline__ bool invalid_rates(float2 pt, float2 vt, float4 St, float rho_t, float T_t) {
    return is_nan_or_inf(pt.x) || is_nan_or_inf(pt.y) || is_nan_or_inf(vt.x) || is_nan_or_inf(vt.y) ||
           is_nan_or_inf(St.x) || is_nan_or_inf(St.y) || is_nan_or_inf(St.z) || is_nan_or_inf(St.w) ||
           is_nan_or_inf(rho_t) || is_nan_or_inf(T_t);
}

// ---- y-bins of the interface segments for the contact's ray casting ----------------------------
// A segment adds a crossing for a particle only if the particle's y lies in the
// segment's float-rounded y-range [lo, hi] (on_segment_mesh).  Each case's range
// [y0, y1] of those rounded values is cut into kSegBins bins, and every segment is
// listed in the bins its [lo, hi] overlaps (one more on each side).  The bin of a
// y is floor((y - y0) * scale); subtraction, the product and floor are monotone
// in y, so a particle's bin lies between the bins of lo and hi of any segment
// that can cross it.  Counting crossings over the particle's bin alone therefore
// gives the full scan's count (an integer sum: order does not matter).  A bin
// holding more than kSegBinCap segments is marked -1 and its particles scan all.
__device__ __forceinline__ int seg_bin_of(double y, double y0, double scale) {
    const double t = floor((y - y0) * scale);
    return t < 0. ? 0 : (t >= (double)(kSegBins - 1) ? kSegBins - 1 : (int)t);
}

// Case c's bins, by the whole block (any block size).
__device__ __forceinline__ void seg_bins_block(int c, const SegDev &seg, ToolDev *tool) {
    ToolDev &t = tool[c];
    __shared__ int cnt[kSegBins];
    __shared__ long long xkey[kSegBins];   // order key of the largest end-point x listed in the bin
    for (int b = threadIdx.x; b < kSegBins; b += blockDim.x) {
        cnt[b] = 0;
        xkey[b] = (long long)0x8000000000000000ull;
    }
    const double y0 = (double)(float)t.seg_ymin, y1 = (double)(float)t.seg_ymax;
    const double scale = (y1 > y0) ? (double)kSegBins / (y1 - y0) : 0.;
    int32_t *list = seg.bin_list + (size_t)c * kSegBins * kSegBinCap;
    __syncthreads();
    for (int i = threadIdx.x; i < t.seg_count; i += blockDim.x) {
        const double2 L = seg.left[t.seg_first + i], R = seg.right[t.seg_first + i];
        const int b0 = max(seg_bin_of(fminf_d(L.y, R.y), y0, scale) - 1, 0);
        const int b1 = min(seg_bin_of(fmaxf_d(L.y, R.y), y0, scale) + 1, kSegBins - 1);
        const long long kx = order_key(fmax(L.x, R.x));
        for (int b = b0; b <= b1; b++) {
            const int slot = atomicAdd(&cnt[b], 1);
            if (slot < kSegBinCap) list[b * kSegBinCap + slot] = i;
            if (seg.bin_xkey) atomicMax(&xkey[b], kx);
        }
    }
    // the per-segment constants of the contact search (SegGeo)
    if (seg.geo) {
        for (int i = threadIdx.x; i < t.seg_count; i += blockDim.x) {
            const double2 L = seg.left[t.seg_first + i], R = seg.right[t.seg_first + i];
            SegGeo g;
            g.ymin_f = fminf_d(L.y, R.y);
            g.ymax_f = fmaxf_d(L.y, R.y);
            g.inv_slope = fabs(L.y - R.y) != 0 ? (L.x - R.x) / (L.y - R.y) : 0.;
            const double xmax = find_max(L.x, R.x), xmin = find_min(L.x, R.x);
            const double ymax = find_max(L.y, R.y), ymin = find_min(L.y, R.y);
            g.kx0 = order_key(xmin - 0.0008);
            g.kx1 = order_key(xmax + 0.0008);
            g.ky0 = order_key(ymin - 0.0008);
            g.ky1 = order_key(ymax + 0.0008);
            g.pad = 0;
            seg.geo[t.seg_first + i] = g;
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kSegBins; b += blockDim.x) {
        seg.bin_count[c * kSegBins + b] = cnt[b] <= kSegBinCap ? cnt[b] : -1;
        if (seg.bin_xkey) {
            // A crossing of a segment lies within its x-range but for the float rounding
            // of its y-range (the pre-filter's bound below): right of the bin's largest
            // x by more than that, no segment of the bin counts.  An overflowed bin
            // takes the bound of all the case's segments.
            const double xm = cnt[b] > kSegBinCap ? t.seg_xmax : order_key_value(xkey[b]);
            seg.bin_xkey[c * kSegBins + b] =
                cnt[b] == 0 ? (long long)0x8000000000000000ull
                            : order_key(xm + t.seg_dxdy * fmax(fabs(t.seg_ymin), fabs(t.seg_ymax)) *
                                                 2.384185791015625e-7 + 1e-12);
        }
    }
    if (threadIdx.x == 0) {
        t.bin_y0 = y0;
        t.bin_scale = scale;
        t.key_y0 = order_key(y0);
        t.key_y1 = order_key(y1);
        t.key_x1 = order_key(t.seg_xmax + t.seg_dxdy * fmax(fabs(t.seg_ymin), fabs(t.seg_ymax)) *
                                              2.384185791015625e-7 + 1e-12);
    }
}

// on_segment_mesh (actions_gpu.cu:51-63) with the segment's float-rounded y-range
// and inverse slope from SegGeo: the same operations on the same values.
__device__ __forceinline__ int on_segment_mesh_geo(double2 left, double2 right, const SegGeo &g, double2 point) {
    if (point.y <= g.ymax_f && point.y >= g.ymin_f) {
        if (left.x == right.x && point.x < left.x) return 1;
        if (fabs(left.y - right.y) != 0) {
            double x_on_seg = right.x + g.inv_slope * (point.y - right.y);
            if (x_on_seg > point.x && x_on_seg != left.x) return 1;
        } else {
            if (point.x <= fmax(left.x, right.x)) return 1;
        }
    }
    return 0;
}

// inside_judgement over the particle's y-bin (the full scan when it overflowed);
// a particle right of the bin's x bound crosses none of its segments
__device__ __forceinline__ int inside_binned(double2 qp, const SegDev &seg, const ToolDev &tool) {
    const int b = seg_bin_of(qp.y, tool.bin_y0, tool.bin_scale);
    if (seg.bin_xkey && order_key(qp.x) > seg.bin_xkey[b]) return 0;
    const int n = seg.bin_count[b];
    int crossings = 0;
    if (n < 0) {
        if (!seg.geo) return inside_judgement(qp, seg.left, seg.right, seg.n);
        for (int i = 0; i < seg.n; i++)
            crossings += on_segment_mesh_geo(__ldg(seg.left + i), __ldg(seg.right + i), seg.geo[i], qp);
        return crossings & 1;
    }
    const int32_t *list = seg.bin_list + b * kSegBinCap;
    int k = 0;
    if (seg.geo) {   // two segments' loads in flight (the count is an integer sum: order-free)
        for (; k + 2 <= n; k += 2) {
            const int2 i2 = *reinterpret_cast<const int2 *>(list + k);
            const int ii[2] = {i2.x, i2.y};
            double2 L[2], R[2], Y[2];
            double Q[2];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                L[u] = __ldg(seg.left + ii[u]);
                R[u] = __ldg(seg.right + ii[u]);
                Y[u] = *reinterpret_cast<const double2 *>(&seg.geo[ii[u]].ymin_f);
                Q[u] = seg.geo[ii[u]].inv_slope;
            }
#pragma unroll
            for (int u = 0; u < 2; u++) {
                SegGeo g;
                g.ymin_f = Y[u].x;
                g.ymax_f = Y[u].y;
                g.inv_slope = Q[u];
                crossings += on_segment_mesh_geo(L[u], R[u], g, qp);
            }
        }
    }
    for (; k < n; k++) {
        const int i = list[k];
        crossings += seg.geo ? on_segment_mesh_geo(__ldg(seg.left + i), __ldg(seg.right + i), seg.geo[i], qp)
                             : on_segment_mesh(__ldg(seg.left + i), __ldg(seg.right + i), qp);
    }
    return crossings & 1;
}

// find_shortest_distance_v1 (actions_gpu.cu:139-220) with its first loop's
// bounding-box test on SegGeo's order keys (integer compares, exact for every
// non-NaN value and false for NaN, as the FP64 compares); the rest as the
// reference.
__device__ __forceinline__ int find_shortest_distance_geo(double2 qp, double &dN, double2 &n_re, const SegDev &seg) {
    const SegGeo *__restrict__ geo = seg.geo;
    const long long kx = order_key(qp.x), ky = order_key(qp.y);
    int sg = -1;
    double depth = FLT_MAX;
    const double limit_value = 2.5e-4;
    // the box tests of four segments per round (their keys loaded together), the
    // candidates then taken in index order as the reference's loop does
    for (int i0 = 0; i0 < seg.n; i0 += 4) {
      bool hit[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
          const int i = i0 + u;
          hit[u] = false;
          if (i < seg.n) {
              const longlong2 ka = reinterpret_cast<const longlong2 *>(geo + i)[0];   // kx0, kx1
              const longlong2 kb = reinterpret_cast<const longlong2 *>(geo + i)[1];   // ky0, ky1
              hit[u] = kx > ka.x && kx < ka.y && ky > kb.x && ky < kb.y;
          }
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int i = i0 + u;
        if (!hit[u]) continue;
        {
            const double2 L = __ldg(seg.left + i), Rr = __ldg(seg.right + i);
            const double ymax = find_max(L.y, Rr.y), ymin = find_min(L.y, Rr.y);
            const double xmax = find_max(L.x, Rr.x), xmin = find_min(L.x, Rr.x);
            const double2 ni = __ldg(seg.normal + i);
            const double d = (qp.x - L.x) * ni.x + (qp.y - L.y) * ni.y;
            if (d >= 0. && d < depth) {
                const double intersec_x = qp.x - d * ni.x;
                const double intersec_y = qp.y - d * ni.y;
                if (intersec_y <= ymax && intersec_y >= ymin && intersec_x <= xmax && intersec_x >= xmin) {
                    depth = d;
                    sg = i;
                }
            }
        }
      }
    }
    if (sg != -1 && depth <= limit_value) {
        const double2 ns = __ldg(seg.normal + sg);
        n_re = make_double2(-ns.x, -ns.y);
        dN = -depth;
        return sg;
    }
    return shortest_distance_fallback(qp, dN, n_re, seg.left, seg.right, seg.normal, seg.n, sg);
}

// The contact search's pre-filter (see contact_s1_one): false means no crossing,
// so the particle is outside the tool and out of contact.
__device__ __forceinline__ bool contact_near(double2 pos, const SegDev &seg, const ToolDev &tool) {
    if (seg.bin_count) {
        const long long ky = order_key(pos.y);
        return ky <= tool.key_y1 && ky >= tool.key_y0 && order_key(pos.x) <= tool.key_x1;
    }
    return pos.y <= (double)(float)tool.seg_ymax && pos.y >= (double)(float)tool.seg_ymin &&
           pos.x <= tool.seg_xmax + tool.seg_dxdy * fmax(fabs(tool.seg_ymin), fabs(tool.seg_ymax)) *
                                       2.384185791015625e-7 + 1e-12;
}

__device__ __forceinline__ uint32_t contact_s1_forces(const KConsts &K, double dt, const ToolDev &tool, double2 vel,
                                                      int seg_no, double gN, double2 n_, double2 &fc, double2 &ft,
                                                      double2 &nrm, int &on_seg, double &blanked);

// ---- contact, one particle: actions_gpu.cu:423-583 (s1) ------------------------------------------
// seg: the segments of the particle's case (and their y-bins); on_seg comes back
// as an index into them.
__device__ __forceinline__ uint32_t contact_s1_one(const KConsts &K, double dt, const SegDev &seg, const ToolDev &tool,
                                                   double2 pos, double2 vel, double2 &fc, double2 &ft, double2 &nrm,
                                                   int &on_seg, double &blanked) {
    int inside = 0;
    // A segment counts a crossing only if the particle's y lies in its float-rounded
    // y-range (on_segment_mesh); float rounding is monotone, so a particle outside the
    // rounded y-range of all segments has no crossing and the scan is skipped.
    // Likewise right of every segment: a crossing lies right of the segments' largest
    // x only by the float rounding of the y-range, which moves the interpolated
    // crossing by at most |dx/dy| * |y| * 2^-24 (bounded here with 2^-22 and an
    // absolute 1e-12).  (These tests first: all tests are pure, and they spare most
    // particles the FP64 sqrt.)
    // With the y-bins built (k_seg_bins), the two bounds come as order keys and the
    // tests run on the integer pipe.
    if (contact_near(pos, seg, tool)) {
        const double ddx = pos.x - tool.tl_point_ref[0], ddy = pos.y - tool.tl_point_ref[1];
        if (sqrt(ddx * ddx + ddy * ddy) < 1.05 * tool.ref_dist)
            inside = seg.bin_count ? inside_binned(pos, seg, tool) : inside_judgement(pos, seg.left, seg.right, seg.n);
    }
    if (inside == 0) {
        fc = make_double2(0., 0.); ft = make_double2(0., 0.); nrm = make_double2(0., 0.);
        on_seg = -1;
        return 0u;
    }
    double gN = 0.;
    double2 n_ = make_double2(0., 0.);
    int seg_no = seg.geo ? find_shortest_distance_geo(pos, gN, n_, seg)
                         : find_shortest_distance_v1(pos, gN, n_, seg.left, seg.right, seg.normal, seg.n);
    return contact_s1_forces(K, dt, tool, vel, seg_no, gN, n_, fc, ft, nrm, on_seg, blanked);
}

// The rest of s1 once the nearest segment is known (actions_gpu.cu:545-583).
__device__ __forceinline__ uint32_t contact_s1_forces(const KConsts &K, double dt, const ToolDev &tool, double2 vel,
                                                      int seg_no, double gN, double2 n_, double2 &fc, double2 &ft,
                                                      double2 &nrm, int &on_seg, double &blanked) {
    on_seg = seg_no;
    if (seg_no == -1) {
        fc = make_double2(0., 0.); ft = make_double2(0., 0.); nrm = make_double2(0., 0.);
        on_seg = -1;
        return SPH_STATUS_CONTACT_NOSEG;
    }
    if (gN < -0.00025) {
        blanked = 1.;
        fc = make_double2(0., 0.); ft = make_double2(0., 0.); nrm = make_double2(0., 0.);
        on_seg = -1;
        return SPH_STATUS_CONTACT_DEEP;
    }
    double dt2 = dt * dt;
    double s1 = -K.c.tool.slave_mass * gN;
    double2 fN = make_double2(s1 * n_.x / dt2 * K.c.tool.contact_alpha, s1 * n_.y / dt2 * K.c.tool.contact_alpha);
    double vx = vel.x - tool.vel[0], vy = vel.y - tool.vel[1];
    double vdn = vx * n_.x + vy * n_.y;
    double vrx = vx - n_.x * vdn, vry = vy - n_.y * vdn;
    double am = K.c.tool.contact_alpha * K.c.tool.slave_mass;
    double kx = am * vrx / dt, ky = am * vry / dt;
    double fy = K.c.tool.mu * sqrt(fN.x * fN.x + fN.y * fN.y);
    double fsx = ft.x - kx, fsy = ft.y - ky;
    double lfs = sqrt(fsx * fsx + fsy * fsy);
    if (lfs > fy) ft = make_double2(fy * fsx / lfs, fy * fsy / lfs);
    else ft = make_double2(fsx, fsy);
    fc = fN;
    nrm = n_;
    return 0u;
}

// ---- contact, one particle: actions_gpu.cu:585-617 (s2) ------------------------------------------
__device__ __forceinline__ void contact_s2_one(const KConsts &K, double dt, const SegDev &seg,
                                               const double *__restrict__ T_nodes, int seg_no, double rho, double &T) {
    int4 mk = seg.marks[seg_no];
    double T_ = T;
    double T_seg = 0.5 * (T_nodes[mk.z] + T_nodes[mk.w]);
    double delta_T = T_seg - T_;
    double length = sqrtf_d(K.c.tool.slave_mass / rho);
    atomicAdd(&seg.heat_exchange[seg_no].x, T_ * length);
    atomicAdd(&seg.heat_exchange[seg_no].y, length);
    double delta_T_part = delta_T * K.c.tool.h * length / K.c.trml_wp.cp / K.c.tool.slave_mass * dt;
    if (delta_T_part < 0) T += fmax(delta_T_part, delta_T);
    else T += fmin(delta_T_part, delta_T);
}

// ---- the FEM tool's contact of the fused step: actions_gpu.cu:423-617 (s1 + s2) -----------------------
// Its own pass before the tail: the contact search's registers would otherwise
// hold down the occupancy of the memory-bound tail for every particle, although
// only the particles near a tool reach it.  The tail that follows sees the
// contact's results (forces, segment id, blanking, temperature) in memory, in the
// order of the reference's step.
// SF: SortedFields (FP64 state) or SortedFields32 (the compact state of FP32K
// contexts); the contact search runs in FP64 either way.
// The segments of case c (indices case-local) and its y-bins.
__device__ __forceinline__ SegDev case_segments(const SegDev &seg, const ToolDev &tc, int c) {
    SegDev cs = seg;
    cs.left += tc.seg_first;
    cs.right += tc.seg_first;
    cs.normal += tc.seg_first;
    cs.n = tc.seg_count;
    if (cs.bin_count) {
        cs.bin_count += c * kSegBins;
        cs.bin_list += (size_t)c * kSegBins * kSegBinCap;
    }
    if (cs.geo) cs.geo += tc.seg_first;
    if (cs.bin_xkey) cs.bin_xkey += c * kSegBins;
    return cs;
}

template <class SF>
__device__ __forceinline__ void contact_fem_one(int i, const KConsts &K, const SF &A, const SegDev &seg,
                                                const ToolDev *__restrict__ tool, const double *__restrict__ T_nodes,
                                                uint32_t *status) {
    if (flag_is_one(A.blanked[i])) return;
    const double2 pos = A.pos[i];
    uint32_t st = 0;
    {
        // the particle's case: its tool, time step and interface segments
        const int c = case_of_hash(K, A.hash[i]);
        const ToolDev &tc = tool[c];
        const SegDev cs = case_segments(seg, tc, c);
        if (!contact_near(pos, cs, tc)) {   // the common case: out of contact, no FP64 work
            put(A.ft[i], make_double2(0., 0.));
            put(A.n[i], make_double2(0., 0.));
            A.on_seg[i] = -1;
            put(A.fc[i], make_double2(0., 0.));
            return;
        }
        double2 fc = d2(A.fc[i]), ft = d2(A.ft[i]), nrm = d2(A.n[i]);
        int on = A.on_seg[i];
        double bl = 0.;
        st |= contact_s1_one(K, tc.dt, cs, tc, pos, d2(A.vel[i]), fc, ft, nrm, on, bl);
        if (on >= 0) on += tc.seg_first;   // global segment id
        const bool blanked = flag_is_one(bl);
        if (blanked) put(A.blanked[i], 1.);
        put(A.ft[i], ft);
        put(A.n[i], nrm);
        A.on_seg[i] = on;
        put(A.fc[i], fc);   // zeroed for fixed particles by the tail (do_boundary_conditions)
        if (!blanked && on >= 0 && on < seg.n) {
            double T = A.T[i];
            contact_s2_one(K, tc.dt, seg, T_nodes, on, A.rho[i], T);
            put(A.T[i], T);
        }
    }
    if (st) set_status(status, st);
}

// ---- the same contact with the few particles at the tool searched by their whole warp --------------
// contact_fem_one's results, bit for bit: each segment test and distance is the
// reference's expression; the loops over a case's segments are spread over the
// 32 lanes (lane k takes segments k, k + 32, ...) and combined in the reference's
// order of preference -- the crossing count as a sum, the nearest segment as the
// smallest (distance, index), the first matching neighbour as the smallest index.
// Called by every lane of every warp (no lane may have left): 1-D blocks, a
// multiple of 32 threads.  Needs the y-bins and SegGeo (k_seg_bins).
constexpr unsigned kFullMask = 0xffffffffu;

__device__ __forceinline__ void warp_argmin(double &d, int &idx) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double d2 = __shfl_xor_sync(kFullMask, d, o);
        const int i2 = __shfl_xor_sync(kFullMask, idx, o);
        if (d2 < d || (d2 == d && i2 < idx)) {
            d = d2;
            idx = i2;
        }
    }
}

// inside_binned's crossing count over this lane's share of the segments
__device__ __forceinline__ int crossings_lanes(double2 qp, const SegDev &seg, const ToolDev &tool, int lane) {
    const int b = seg_bin_of(qp.y, tool.bin_y0, tool.bin_scale);
    if (order_key(qp.x) > seg.bin_xkey[b]) return 0;
    const int n = seg.bin_count[b];
    int crossings = 0;
    if (n < 0) {
        for (int i = lane; i < seg.n; i += 32)
            crossings += on_segment_mesh_geo(__ldg(seg.left + i), __ldg(seg.right + i), seg.geo[i], qp);
    } else {
        const int32_t *list = seg.bin_list + b * kSegBinCap;
        for (int k = lane; k < n; k += 32) {
            const int i = list[k];
            crossings += on_segment_mesh_geo(__ldg(seg.left + i), __ldg(seg.right + i), seg.geo[i], qp);
        }
    }
    return crossings;
}

// find_shortest_distance_v1 by the warp (every lane gets the result)
__device__ __forceinline__ int shortest_distance_lanes(double2 qp, double &dN, double2 &n_re, const SegDev &seg,
                                                       int lane) {
    const long long kx = order_key(qp.x), ky = order_key(qp.y);
    double best = FLT_MAX;
    int bi = 0x7fffffff;
    for (int i = lane; i < seg.n; i += 32) {
        const SegGeo &g = seg.geo[i];
        if (kx > g.kx0 && kx < g.kx1 && ky > g.ky0 && ky < g.ky1) {
            const double2 L = __ldg(seg.left + i), Rr = __ldg(seg.right + i);
            const double ymax = find_max(L.y, Rr.y), ymin = find_min(L.y, Rr.y);
            const double xmax = find_max(L.x, Rr.x), xmin = find_min(L.x, Rr.x);
            const double2 ni = __ldg(seg.normal + i);
            const double d = (qp.x - L.x) * ni.x + (qp.y - L.y) * ni.y;
            if (d >= 0. && d < best) {
                const double intersec_x = qp.x - d * ni.x;
                const double intersec_y = qp.y - d * ni.y;
                if (intersec_y <= ymax && intersec_y >= ymin && intersec_x <= xmax && intersec_x >= xmin) {
                    best = d;
                    bi = i;
                }
            }
        }
    }
    warp_argmin(best, bi);
    const int sg = bi == 0x7fffffff ? -1 : bi;
    const double depth = sg == -1 ? (double)FLT_MAX : best;
    if (sg != -1 && depth <= 2.5e-4) {
        const double2 ns = __ldg(seg.normal + sg);
        n_re = make_double2(-ns.x, -ns.y);
        dN = -depth;
        return sg;
    }
    // the fallback: the nearest right end point (strict <, so the first of equals)
    double bd = FLT_MAX;
    int bj = 0x7fffffff;
    for (int i = lane; i < seg.n; i += 32) {
        const double2 Rr = __ldg(seg.right + i);
        const double d_trial = sqrtf_d((qp.x - Rr.x) * (qp.x - Rr.x) + (qp.y - Rr.y) * (qp.y - Rr.y));
        if (d_trial < bd) {
            bd = d_trial;
            bj = i;
        }
    }
    warp_argmin(bd, bj);
    const int s_near = bj == 0x7fffffff ? sg : bj;
    const double dep = bj == 0x7fffffff ? (double)FLT_MAX : bd;
    if (s_near == -1) return -1;
    const double2 ns = __ldg(seg.normal + s_near);
    const double2 rs = __ldg(seg.right + s_near);
    int jm = 0x7fffffff;
    for (int j = lane; j < seg.n; j += 32) {
        const double2 Lj = __ldg(seg.left + j);
        if (Lj.y == rs.y && Lj.x == rs.x) {
            jm = j;
            break;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) jm = min(jm, __shfl_xor_sync(kFullMask, jm, o));
    double nsx = ns.x, nsy = ns.y;
    if (jm != 0x7fffffff) {
        const double2 nj = __ldg(seg.normal + jm);
        nsx = (nj.x + ns.x) / 2.;
        nsy = (nj.y + ns.y) / 2.;
    }
    const double n_length = sqrtf_d(nsx * nsx + nsy * nsy);
    n_re = make_double2(-nsx / n_length, -nsy / n_length);
    dN = -1.0 * dep;
    return s_near;
}

template <class SF>
__device__ __forceinline__ void contact_fem_warp(int i, int N, const KConsts &K, const SF &A, const SegDev &seg,
                                                 const ToolDev *__restrict__ tool,
                                                 const double *__restrict__ T_nodes, uint32_t *status) {
    const int lane = (int)(threadIdx.x & 31u);
    const bool live = i < N && !flag_is_one(A.blanked[i]);
    double2 pos = make_double2(0., 0.);
    int c = 0;
    bool near = false, probe = false;
    if (live) {
        pos = A.pos[i];
        c = case_of_hash(K, A.hash[i]);
        const ToolDev &tc = tool[c];
        near = contact_near(pos, case_segments(seg, tc, c), tc);
        if (!near) {   // out of contact: zeros, no FP64 work
            put(A.ft[i], make_double2(0., 0.));
            put(A.n[i], make_double2(0., 0.));
            A.on_seg[i] = -1;
            put(A.fc[i], make_double2(0., 0.));
        } else {
            const double ddx = pos.x - tc.tl_point_ref[0], ddy = pos.y - tc.tl_point_ref[1];
            // right of every segment of its y-bin a particle crosses none (no scan needed)
            probe = sqrt(ddx * ddx + ddy * ddy) < 1.05 * tc.ref_dist &&
                    order_key(pos.x) <= seg.bin_xkey[c * kSegBins + seg_bin_of(pos.y, tc.bin_y0, tc.bin_scale)];
        }
    }
    // the ray casting of each probing lane, by the warp
    int inside = 0;
    for (unsigned pend = __ballot_sync(kFullMask, probe); pend; pend &= pend - 1) {
        const int src = __ffs(pend) - 1;
        const double2 qp = make_double2(__shfl_sync(kFullMask, pos.x, src), __shfl_sync(kFullMask, pos.y, src));
        const int cc = __shfl_sync(kFullMask, c, src);
        const int cr = __reduce_add_sync(kFullMask, crossings_lanes(qp, case_segments(seg, tool[cc], cc), tool[cc], lane));
        if (lane == src) inside = cr & 1;
    }
    // the nearest segment of each lane inside the tool, by the warp
    int seg_no = -1;
    double gN = 0.;
    double2 n_ = make_double2(0., 0.);
    for (unsigned pend = __ballot_sync(kFullMask, inside != 0); pend; pend &= pend - 1) {
        const int src = __ffs(pend) - 1;
        const double2 qp = make_double2(__shfl_sync(kFullMask, pos.x, src), __shfl_sync(kFullMask, pos.y, src));
        const int cc = __shfl_sync(kFullMask, c, src);
        double dN;
        double2 nr;
        const int r = shortest_distance_lanes(qp, dN, nr, case_segments(seg, tool[cc], cc), lane);
        if (lane == src) {
            seg_no = r;
            gN = dN;
            n_ = nr;
        }
    }
    if (!near) return;
    const ToolDev &tc = tool[c];
    double2 fc = d2(A.fc[i]), ft = d2(A.ft[i]), nrm = d2(A.n[i]);
    int on = A.on_seg[i];
    double bl = 0.;
    uint32_t st = 0;
    if (inside == 0) {
        fc = make_double2(0., 0.); ft = make_double2(0., 0.); nrm = make_double2(0., 0.);
        on = -1;
    } else {
        st = contact_s1_forces(K, tc.dt, tc, d2(A.vel[i]), seg_no, gN, n_, fc, ft, nrm, on, bl);
    }
    if (on >= 0) on += tc.seg_first;   // global segment id
    const bool blanked = flag_is_one(bl);
    if (blanked) put(A.blanked[i], 1.);
    put(A.ft[i], ft);
    put(A.n[i], nrm);
    A.on_seg[i] = on;
    put(A.fc[i], fc);
    if (!blanked && on >= 0 && on < seg.n) {
        double T = A.T[i];
        contact_s2_one(K, tc.dt, seg, T_nodes, on, A.rho[i], T);
        put(A.T[i], T);
    }
    if (st) set_status(status, st);
}

// ---- fused tail of the step ----------------------------------------------------------------------
// The tool's contact for one particle -- kMode 2: rigid tool, update_tool_particles
// and do_compute_contact_forces (tool_gpu.cu:146-216); kMode 0: no tool, or the
// FEM tool whose contact k_contact_fem has applied just before -- then
// do_boundary_conditions, do_boundary_conditions_thermal, do_invalidate
// (actions_gpu.cu:756-824) and (kNextHash) the next step's compute_hashes and
// the counting-sort histogram (grid.cu:25-42) on the final state.
template <int kMode, bool kNextHash, class SF>
__device__ __forceinline__ void step_tail_one(int i, const KConsts &K, const SF &A, const SortScratch &X,
                                              uint32_t *status) {
    bool blanked = flag_is_one(A.blanked[i]);
    const bool bc_fixed = !flag_nonzero(A.tool_particle[i]) && flag_nonzero(A.fixed[i]);   // do_boundary_conditions
    const bool bc_thermal = K.thermal_bc && flag_is_one(A.fixed[i]);                         // ..._thermal
    uint32_t st = 0;
    double2 pos = A.pos[i];
    if (kMode == 2) {
        const sph_rigid_tool &rt = *K.rigid;
        if (flag_nonzero(A.tool_particle[i])) {   // update_tool_particles, blanked or not
            pos.x += K.dt * rt.vel[0];
            pos.y += K.dt * rt.vel[1];
            A.pos[i] = pos;
        } else {                                  // contact, blanked or not
            double2 fc, ft = d2(A.ft[i]), nrm;
            rigid_contact_one(K, rt, K.dt, pos, d2(A.vel[i]), fc, ft, nrm);
            put(A.ft[i], ft);
            put(A.n[i], nrm);
            if (bc_fixed) fc = make_double2(0., 0.);
            put(A.fc[i], fc);
        }
    } else if (bc_fixed) {
        put(A.fc[i], make_double2(0., 0.));
    }
    if (bc_fixed) {
        put(A.vel[i], make_double2(0., 0.));
        put(A.pos_t[i], make_double2(0., 0.));
        put(A.vel_t[i], make_double2(0., 0.));
    }
    if (bc_thermal) put(A.T[i], K.c.trml_wp.T_init);
    if (!blanked) {
        if (invalid_rates(A.pos_t[i], A.vel_t[i], A.S_t[i], A.rho_t[i], A.T_t[i])) {
            blanked = true;
            put(A.blanked[i], 1.);
            st |= SPH_STATUS_NAN_BLANKED;
        }
    }
    if (kNextHash) {
        int h;
        if (!blanked) {
            const sph_geom_constants &g = K.g;
            int ix = cell_coord(pos.x, g.bbmin_x, g.dx, K.f.inv_cell);
            int iy = cell_coord(pos.y, g.bbmin_y, g.dx, K.f.inv_cell);
            h = ix * g.ny + iy;
        } else {
            h = A.hash[i];   // blanked particles keep their stale hash
        }
        int key = h;
        if (h < 0 || h >= K.g.num_cell) {
            key = K.g.num_cell;
            st |= SPH_STATUS_OUT_OF_GRID;
        }
        X.key[i] = key;
        X.arrival[i] = histogram_slot(X.counts, key);
        X.hash_next[i] = h;   // the visible hash array changes only at the next sort
    }
    if (st) set_status(status, st);
}

}  // namespace sphfem
