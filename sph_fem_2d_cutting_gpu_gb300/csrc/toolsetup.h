// toolsetup.h -- host-side set-up of the FEM tool: interface segments, element
// colouring, CSR pattern and the assembled thermal system.
#pragma once

#include <string>
#include <vector>

#include "../../include/sphfem.h"

namespace sphfem {

struct Int4 { int x, y, z, w; };

struct ToolModelHost {
    int n_nodes = 0, n_elements = 0;
    std::vector<double> pos;            // [n_nodes][2]
    std::vector<Int4> elements;         // node a, b, c, colour
    int n_colors = 0, n_cut_colors = 0;
    // CSR (zero-based, columns ascending per row)
    std::vector<int> row_ptr, col_ind, diag;
    std::vector<double> K, M, M_inv, f, T;
    // the Dirichlet elimination's processing order (colour by colour, then
    // element order): element and its fixed-edge flags (x, y, z; w unused)
    std::vector<int> dirichlet_elem;
    std::vector<Int4> dirichlet_flags;
    // per node: bit 0 on a cutting edge, bit 1 on a fixed edge (the mesh
    // reader's cutting_edge_flag / fixed_edge_flag, mesh_structure_GPU.cu:430-471)
    std::vector<int> node_edge;
    // interface segments
    int n_seg = 0;
    std::vector<double> left, right, normal;   // [n_seg][2]
    std::vector<Int4> marks;                   // element, colour, node left, node right
    std::vector<int> node_seg_ptr, node_seg;   // segments ending on each node
    // wear (WEAR_NODE_SHIFT): layer flags per element (x: layer 1, y: layer 2), the
    // layer elements, and per node of a layer element its layer elements
    // (x: index into wear_elem, y: local index) with the CSR slots of
    // (node, element node b), b = 0..2 (x, y, z)
    std::vector<Int4> layer;
    std::vector<int> wear_elem, wear_node, wear_adj_ptr;
    std::vector<Int4> wear_adj, wear_slot;
    // tool kinematics
    double tl_point_ref[2] = {0, 0}, br_point[2] = {0, 0};
    double ref_dist = 0, lowest_point = 0, right_point = 0;
};

// Builds the full tool model.  Returns SPH_OK or SPH_ERR_INVALID with *err set.
int build_tool_model(const sph_tool_mesh &mesh, const sph_tool_constants &tc, ToolModelHost &out, std::string &err);

}  // namespace sphfem
