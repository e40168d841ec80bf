// length2(v) = dot(v, v), the squared Euclidean length (see ../glm.hpp).
#ifndef FSIM_REF_GLM_SUBSET_NORM_HPP
#define FSIM_REF_GLM_SUBSET_NORM_HPP
#include "../glm.hpp"
namespace glm {
FSIM_GLM_FN float length2(const vec3 &a) { return dot(a, a); }
}  // namespace glm
#endif
