// Stand-in for <glm/gtc/matrix_integer.hpp> (reference-pin builds only):
// the reference includes it but uses no integer matrix type.
#pragma once
#include "../glm.hpp"
