// Stand-in for <glm/matrix.hpp> (reference-pin builds only): the matrix
// types and functions of glm.hpp.
#pragma once
#include "glm.hpp"
