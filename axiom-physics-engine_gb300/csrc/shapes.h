// shapes.h — shape predicates shared by host and device code.
#pragma once

#include <cstdint>

#include "../../include/axiom_c.h"

namespace axiom_gb300 {

// Shapes whose geometry is a hull in the world's vertex pool: convex bodies and the
// triangles of static meshes (three-point hulls).
#ifdef __CUDACC__
__host__ __device__
#endif
inline constexpr bool isHullShape(uint32_t s) {
    return s == AXIOM_SHAPE_CONVEX || s == AXIOM_SHAPE_MESH;
}

}  // namespace axiom_gb300
