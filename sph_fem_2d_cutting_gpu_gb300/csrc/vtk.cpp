// vtk.cpp -- the reference's legacy-ASCII VTK output (vtk_writer.cu) from host
// arrays.  The device-context writers (sph_write_vtk_*) download the state and
// call these; they are also exported for callers holding host arrays.  Same
// records, field order and printf formats as the reference writers, so files
// compare byte for byte with the reference's own output, with one deliberate
// difference in the particle file: blanked particles are left out and the
// vertex cells number the written points 0..m-1 (the reference reads an
// uninitialised blanked array, vtk_writer.cu:67-82, and numbers its cells by
// particle index, vtk_writer.cu:101-104: the two agree when no particle is
// blanked).
#include <cmath>
#include <cstdio>

#include "../../include/sphfem.h"

extern "C" {

// vtk_writer.cu:11-220 vtk_writer_write(particle_gpu*, step): reads pos, vel,
// fc, ft, n, S, p, T, eps_pl, on_seg and blanked of h.
int sph_vtk_write_particles_host(const sph_particles *h, const char *path) {
    if (!h || !path || h->N < 0 || !h->pos || !h->vel || !h->fc || !h->ft || !h->n || !h->S || !h->p || !h->T ||
        !h->eps_pl || !h->on_seg || !h->blanked)
        return SPH_ERR_INVALID;
    const int n = h->N;
    const double *pos = h->pos, *vel = h->vel, *fc = h->fc, *ft = h->ft, *nrm = h->n, *S = h->S, *p = h->p,
                 *T = h->T, *eps = h->eps_pl, *blanked = h->blanked;
    const int32_t *on_seg = h->on_seg;
    FILE *fp = fopen(path, "w");
    if (!fp) return SPH_ERR_INVALID;
    int m = 0;
    for (int i = 0; i < n; i++) m += blanked[i] != 1.;
    // points of the non-blanked particles, one vertex cell each
    fprintf(fp, "# vtk DataFile Version 2.0\nmfree iwf\nASCII\n\nDATASET UNSTRUCTURED_GRID\nPOINTS %d float\n", m);
    for (int i = 0; i < n; i++)
        if (blanked[i] != 1.) fprintf(fp, "%f %f %f\n", pos[2 * i], pos[2 * i + 1], 0.);
    fprintf(fp, "\nCELLS %d %d\n", m, 2 * m);
    for (int k = 0; k < m; k++) fprintf(fp, "%d %d\n", 1, k);   // vertex k of the POINTS list
    fprintf(fp, "\nCELL_TYPES %d\n", m);
    for (int k = 0; k < m; k++) fprintf(fp, "%d\n", 1);
    fprintf(fp, "\nPOINT_DATA %d\n", m);
    fprintf(fp, "SCALARS Temperature float 1\nLOOKUP_TABLE default\n");
    for (int i = 0; i < n; i++)
        if (blanked[i] != 1.) fprintf(fp, "%f\n", T[i]);
    fprintf(fp, "\nSCALARS on_seg int 1\nLOOKUP_TABLE default\n");
    for (int i = 0; i < n; i++)
        if (blanked[i] != 1.) fprintf(fp, "%d\n", on_seg[i]);
    fprintf(fp, "\nSCALARS EquivAccumPlasticStrain float 1\nLOOKUP_TABLE default\n");
    for (int i = 0; i < n; i++)
        if (blanked[i] != 1.) fprintf(fp, "%f\n", eps[i]);
    fprintf(fp, "\nVECTORS Velocity float\n");
    for (int i = 0; i < n; i++)
        if (blanked[i] != 1.) fprintf(fp, "%f %f %f\n", vel[2 * i], vel[2 * i + 1], 0.);
    fprintf(fp, "\nVECTORS fc float\n");
    for (int i = 0; i < n; i++)
        if (blanked[i] != 1.) fprintf(fp, "%2f %2f %2f\n", 100000 * fc[2 * i], 100000 * fc[2 * i + 1], 0.);
    fprintf(fp, "\nVECTORS ft float\n");
    for (int i = 0; i < n; i++)
        if (blanked[i] != 1.) fprintf(fp, "%f %f %f\n", 100000 * ft[2 * i], 100000 * ft[2 * i + 1], 0.);
    fprintf(fp, "\nVECTORS normal float\n");
    for (int i = 0; i < n; i++)
        if (blanked[i] != 1.) fprintf(fp, "%f %f %f\n", nrm[2 * i], nrm[2 * i + 1], 0.);
    fprintf(fp, "\nSCALARS SvM float 1\nLOOKUP_TABLE default\n");
    for (int i = 0; i < n; i++) {
        if (blanked[i] == 1.) continue;
        const double cxx = S[4 * i] - p[i], cyy = S[4 * i + 2] - p[i], czz = S[4 * i + 3] - p[i], cxy = S[4 * i + 1];
        const double svm2 = (cxx * cxx + cyy * cyy + czz * czz) - cxx * cyy - cxx * czz - cyy * czz + 3.0 * cxy * cxy;
        fprintf(fp, "%f\n", svm2 > 0 ? std::sqrt(svm2) : 0.);
    }
    fprintf(fp, "\n");
    return fclose(fp) == 0 ? SPH_OK : SPH_ERR_INVALID;
}

// vtk_writer.cu:304-366 vtk_writer_write_FEM_tool (shift NULL) and :518-587
// vtk_writer_write_tool_org (shift = tl_point_ref - tl_ref: the tool moved
// back by its travel): nodes, triangles (elements [n][4]: nodes a, b, c and
// the colour, which is not written), nodal temperature.
int sph_vtk_write_tool_host(int32_t n_nodes, const double *position, const double *T, int32_t n_elements,
                            const int32_t *elements, const double *shift, const char *path) {
    if (!path || n_nodes < 0 || n_elements < 0 || (n_nodes && (!position || !T)) || (n_elements && !elements))
        return SPH_ERR_INVALID;
    const double sx = shift ? shift[0] : 0., sy = shift ? shift[1] : 0.;
    FILE *fp = fopen(path, "w");
    if (!fp) return SPH_ERR_INVALID;
    fprintf(fp, "# vtk DataFile Version 2.0\nmfree iwf\nASCII\n\nDATASET UNSTRUCTURED_GRID\nPOINTS %d float\n", n_nodes);
    for (int i = 0; i < n_nodes; i++) fprintf(fp, "%f %f %f\n", position[2 * i] - sx, position[2 * i + 1] - sy, 0.);
    fprintf(fp, "\nCELLS %d %d\n", n_elements, 4 * n_elements);
    for (int e = 0; e < n_elements; e++)
        fprintf(fp, "3 %d %d %d\n", elements[4 * e], elements[4 * e + 1], elements[4 * e + 2]);
    fprintf(fp, "\nCELL_TYPES %d\n", n_elements);
    for (int e = 0; e < n_elements; e++) fprintf(fp, "5\n");
    fprintf(fp, "POINT_DATA %d\nSCALARS temperature float 1\nLOOKUP_TABLE default\n", n_nodes);
    for (int i = 0; i < n_nodes; i++) fprintf(fp, "%f\n", T[i]);
    fprintf(fp, "\n");
    return fclose(fp) == 0 ? SPH_OK : SPH_ERR_INVALID;
}

// vtk_writer.cu:368-516 vtk_writer_write_FEM_segments: every contact segment
// as a triangle (left, right, and right + |segment| n), with the wear
// statistics on the third point: mean pressure (GPa), sliding speed (m/s),
// segment temperature, frictional stress and wear rate (1e10 x).  phys_para
// [n][4] (count, sum pressure, sum sliding speed, sum T), sliding_force and
// wear_rate [n]; NULL: no statistics gathered (all wear fields zero).
int sph_vtk_write_segments_host(int32_t n_seg, const double *left, const double *right, const double *normal,
                                const double *phys_para, const double *sliding_force, const double *wear_rate,
                                const char *path) {
    if (!path || n_seg < 0 || (n_seg && (!left || !right || !normal))) return SPH_ERR_INVALID;
    const int ns = n_seg;
    FILE *fp = fopen(path, "w");
    if (!fp) return SPH_ERR_INVALID;
    fprintf(fp, "# vtk DataFile Version 2.0\nmfree iwf\nASCII\n\nDATASET UNSTRUCTURED_GRID\nPOINTS %d float\n", 3 * ns);
    for (int i = 0; i < ns; i++) {
        const double lx = left[2 * i], ly = left[2 * i + 1], rx = right[2 * i], ry = right[2 * i + 1];
        fprintf(fp, "%f %f %f\n", lx, ly, 0.);
        fprintf(fp, "%f %f %f\n", rx, ry, 0.);
        const double dis = sqrt((lx - rx) * (lx - rx) + (ly - ry) * (ly - ry));
        fprintf(fp, "%f %f %f\n", rx + dis * normal[2 * i], ry + dis * normal[2 * i + 1], 0.);
    }
    fprintf(fp, "\nCELLS %d %d\n", ns, 4 * ns);
    for (int i = 0; i < ns; i++) fprintf(fp, "3 %d %d %d \n", 3 * i, 3 * i + 1, 3 * i + 2);
    fprintf(fp, "\nCELL_TYPES %d\n", ns);
    for (int i = 0; i < ns; i++) fprintf(fp, "5\n");
    fprintf(fp, "POINT_DATA %d\n", 3 * ns);
    // a segment's value on its third point, 0 where no particle contributed
    auto field = [&](const char *name, auto value) {
        fprintf(fp, "SCALARS %s float 1\nLOOKUP_TABLE default\n", name);
        for (int i = 0; i < ns; i++) {
            fprintf(fp, "%f\n%f\n", 0., 0.);
            const double cnt = phys_para ? phys_para[4 * i] : 0.;
            fprintf(fp, "%f\n", cnt != 0. ? value(i) : 0.);
        }
        fprintf(fp, "\n");
    };
    field("PressureGPa", [&](int i) { return phys_para[4 * i + 1] / phys_para[4 * i] * 100.; });
    field("Velocity", [&](int i) { return phys_para[4 * i + 2] / phys_para[4 * i] * 10000.; });
    field("Temperature", [&](int i) { return phys_para[4 * i + 3] / phys_para[4 * i]; });
    field("Frictional_stress", [&](int i) { return (sliding_force ? sliding_force[i] : 0.) / phys_para[4 * i] * 100.; });
    field("Wear_rate", [&](int i) { return (wear_rate ? wear_rate[i] : 0.) * 1e10; });
    return fclose(fp) == 0 ? SPH_OK : SPH_ERR_INVALID;
}

}  // extern "C"
