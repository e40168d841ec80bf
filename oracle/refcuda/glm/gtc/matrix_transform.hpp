// The reference includes this header but calls nothing from it beyond the
// core types (see ../glm.hpp).
#ifndef FSIM_REF_GLM_SUBSET_MATRIX_TRANSFORM_HPP
#define FSIM_REF_GLM_SUBSET_MATRIX_TRANSFORM_HPP
#include "../glm.hpp"
#endif
