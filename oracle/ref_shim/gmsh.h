// Stand-in for <gmsh.h> (reference-pin builds only).  gmsh is a third-party
// dependency of the reference that this image does not have.  The reference's
// headers include it and its tool remesher (tool_FEM.cu:1726-1801, host code)
// calls a few functions of gmsh's public API; the pins compile that host code
// only so that the file's device kernels can be built, and never run it.  So
// each function here has the API's name and parameter list and does nothing.
#pragma once

#include <string>
#include <vector>

namespace gmsh {
inline void initialize(int = 0, char ** = nullptr, bool = true, bool = false) {}
inline void finalize() {}
inline void write(const std::string &) {}
namespace option {
inline void setNumber(const std::string &, const double) {}
}  // namespace option
namespace model {
inline void add(const std::string &) {}
inline int addPhysicalGroup(const int, const std::vector<int> &, const int = -1, const std::string & = "") { return 0; }
namespace geo {
inline int addPoint(const double, const double, const double, const double = 0., const int = -1) { return 0; }
inline int addLine(const int, const int, const int = -1) { return 0; }
inline int addCurveLoop(const std::vector<int> &, const int = -1, const bool = false) { return 0; }
inline int addPlaneSurface(const std::vector<int> &, const int = -1) { return 0; }
inline void synchronize() {}
}  // namespace geo
namespace mesh {
inline void generate(const int = 3) {}
}  // namespace mesh
}  // namespace model
}  // namespace gmsh
