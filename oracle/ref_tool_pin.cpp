// ref_tool_pin.cpp -- runs the reference's OWN host geometry of the rigid tool
// to pin the host-side restatement (test infrastructure; built into
// oracle/_ref/ only, from the read-only reference tree: tool.cpp and
// geometric_primitives.cpp, with the stand-in headers of oracle/ref_shim).
//
// Each input line: tlx tly length height rake clear r mu vel lo_x hi_y feed dx preload_time
// For it the harness builds tool(tl, length, height, rake, clear, r, mu)
// (tool.cpp:335-369), places it as setup_ref_cut does (benchmarks.cpp:388-412:
// front to lo_x, lowest point to hi_y - feed), moves it by preload_time at
// (vel, 0), samples it with spacing dx (tool.cpp:112-135) and prints
//   seg i left.x left.y right.x right.y n.x n.y a b vertical    (per segment)
//   fillet p.x p.y r t1 t2                                       (or "fillet none")
//   low v / front v / bb x0 x1 y0 y1 (safe_bb(0.1 dx)) / samples n, then n lines x y
//   end
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <vector>

#include "tool.h"

static void print_tool(tool &t, double dx) {
    std::vector<segment> segs = t.get_segments();
    for (size_t i = 0; i < segs.size(); i++) {
        const segment &s = segs[i];
        printf("seg %zu %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %d\n", i, s.left.x, s.left.y, s.right.x,
               s.right.y, s.n.x, s.n.y, s.l.a, s.l.b, s.l.vertical ? 1 : 0);
    }
    circle_segment *f = t.get_fillet();
    if (f)
        printf("fillet %.17g %.17g %.17g %.17g %.17g\n", f->p.x, f->p.y, f->r, f->t1, f->t2);
    else
        printf("fillet none\n");
    printf("low %.17g\nfront %.17g\n", t.low(), t.front());
    bbox b = t.safe_bb(0.1 * dx);
    printf("bb %.17g %.17g %.17g %.17g\n", b.bbmin_x, b.bbmax_x, b.bbmin_y, b.bbmax_y);
    std::vector<float2_t> smp = t.sample_tool(dx, 300., 4.43, 1.5);
    printf("samples %zu\n", smp.size());
    for (const float2_t &p : smp) printf("%.17g %.17g\n", p.x, p.y);
    printf("end\n");
}

int main() {
    double v[14];
    while (scanf("%lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf", v, v + 1, v + 2, v + 3, v + 4, v + 5,
                 v + 6, v + 7, v + 8, v + 9, v + 10, v + 11, v + 12, v + 13) == 14) {
        const double vel_tool = v[8], lo_x = v[9], hi_y = v[10], feed = v[11], dx = v[12], preload = v[13];
        tool t(glm::dvec2(v[0], v[1]), v[2], v[3], v[4], v[5], v[6], v[7]);
        // benchmarks.cpp:388-412
        double distance = t.front() - lo_x;
        double time = distance / vel_tool;
        t.set_vel(glm::dvec2(vel_tool, 0.));
        t.update_tool(-time);
        double current_feed = hi_y - t.low();
        double correction_time = fabs(current_feed - feed) / vel_tool;
        double sign = (current_feed > feed) ? 1 : -1.;
        t.set_vel(glm::dvec2(0., vel_tool));
        t.update_tool(correction_time * sign);
        t.set_vel(glm::dvec2(vel_tool, 0.));
        if (preload != 0.) t.update_tool(preload);
        print_tool(t, dx);
    }
    return 0;
}
