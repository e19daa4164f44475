// host_math.h — host-side shape helpers shared by the world and the scene generators.
#pragma once

#include <cmath>
#include <cstdint>

#include "../../include/axiom_c.h"

namespace axiom_gb300 {

constexpr float kFourThirdsPi = 4.18879020f;
constexpr float kPi = 3.14159265f;

// Mass and body-frame diagonal inertia of a solid shape of the given density.
//  sphere  m = rho (4/3 pi r^3),              I = 0.4 m r^2
//  box     m = rho (8 hx hy hz),              I_x = m/3 (hy^2 + hz^2) (and cyclic)
//  capsule cylinder (2h) + two hemispheres;   I_y = mc r^2/2 + ms 0.4 r^2,
//          I_x = I_z = mc (h^2/3 + r^2/4) + ms (0.4 r^2 + h^2 + 0.75 h r)
//  cylinder m = rho (pi r^2 2h),              I_y = m r^2 / 2, I_x = I_z = m (3 r^2 + 4 h^2) / 12
//  (a convex hull takes the box formula with its bounding box's half-extents)
inline void massProperties(uint32_t shape, const float e[3], float density, float* mass,
                           float inertia[3]) {
    if (shape == AXIOM_SHAPE_SPHERE) {
        float r = e[0];
        float m = density * (kFourThirdsPi * r * r * r);
        float i = 0.4f * m * r * r;
        *mass = m;
        inertia[0] = inertia[1] = inertia[2] = i;
    } else if (shape == AXIOM_SHAPE_BOX) {
        float m = density * (8.0f * e[0] * e[1] * e[2]);
        float k = m / 3.0f;
        *mass = m;
        inertia[0] = k * (e[1] * e[1] + e[2] * e[2]);
        inertia[1] = k * (e[0] * e[0] + e[2] * e[2]);
        inertia[2] = k * (e[0] * e[0] + e[1] * e[1]);
    } else if (shape == AXIOM_SHAPE_CAPSULE) {
        float r = e[0], h = e[1];
        float mc = density * (kPi * r * r * (2.0f * h));
        float ms = density * (kFourThirdsPi * r * r * r);
        float iy = mc * r * r * 0.5f + ms * 0.4f * r * r;
        float ix = mc * (h * h / 3.0f + r * r * 0.25f) + ms * (0.4f * r * r + h * h + 0.75f * h * r);
        *mass = mc + ms;
        inertia[0] = ix;
        inertia[1] = iy;
        inertia[2] = ix;
    } else if (shape == AXIOM_SHAPE_CYLINDER) {
        float r = e[0], h = e[1];
        float m = density * (kPi * r * r * (2.0f * h));
        float iy = 0.5f * m * r * r;
        float ix = m * (3.0f * r * r + 4.0f * h * h) / 12.0f;
        *mass = m;
        inertia[0] = ix;
        inertia[1] = iy;
        inertia[2] = ix;
    } else {
        *mass = 0.0f;
        inertia[0] = inertia[1] = inertia[2] = 0.0f;
    }
}

// Radius of the smallest centred sphere that holds the shape.
inline float boundingRadius(uint32_t shape, const float e[3]) {
    switch (shape) {
        case AXIOM_SHAPE_SPHERE: return e[0];
        case AXIOM_SHAPE_BOX: return std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
        case AXIOM_SHAPE_CAPSULE: return e[0] + e[1];
        case AXIOM_SHAPE_CYLINDER: return std::sqrt(e[0] * e[0] + e[1] * e[1]);
        case AXIOM_SHAPE_CONVEX:
        case AXIOM_SHAPE_MESH: return e[0];  // packed hull extents: (radius, -, -)
        default: return 0.0f;
    }
}

// DeterministicRNG of include/axiom/math/random.hpp:19-64 (PCG-XSH-RR 64 -> 32).
class Pcg32 {
public:
    explicit Pcg32(uint64_t seed) : state_(seed | 1ULL) {
        for (int i = 0; i < 10; ++i) next();
    }
    uint32_t next() {
        uint64_t old = state_;
        state_ = old * 6364136223846793005ULL + 1442695040888963407ULL;
        uint32_t xs = static_cast<uint32_t>(((old >> 18U) ^ old) >> 27U);
        uint32_t rot = static_cast<uint32_t>(old >> 59U);
        return (xs >> rot) | (xs << ((~rot + 1U) & 31U));
    }
    float nextFloat() { return static_cast<float>(next()) / 4294967296.0f; }
    float nextFloat(float lo, float hi) { return lo + nextFloat() * (hi - lo); }

private:
    uint64_t state_;
};

}  // namespace axiom_gb300
