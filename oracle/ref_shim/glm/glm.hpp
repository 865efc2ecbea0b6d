// Empty stand-in for <glm/glm.hpp>.  The reference's types.h includes GLM, but
// the two reference headers compiled by oracle/ref_pin.cpp (kernels.cuh and
// plasticity.cuh) use no GLM symbol, so nothing from GLM is needed to build them.
#pragma once
