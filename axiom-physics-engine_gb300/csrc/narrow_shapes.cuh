// narrow_shapes.cuh — per-shape-pair contact generation (device).
#pragma once

#include "../../include/axiom_c.h"
#include "dmath.cuh"

namespace axiom_gb300 {

struct Geom {
    uint32_t shape;
    float4 pos, rot, ext;
};

struct Contact {
    uint32_t count;
    axd::f3 n;
    axd::f3 p[4];
    float depth[4];
};

// Sphere (ca, ra) against sphere (cb, rb); normal a -> b, point midway between surfaces.
__device__ __forceinline__ bool sphereSphere(axd::f3 ca, float ra, axd::f3 cb, float rb, Contact* c) {
    using namespace axd;
    const f3 d = sub(cb, ca);
    const float dist2 = dot(d, d);
    const float rs = ra + rb;
    if (dist2 > rs * rs) return false;
    const float dist = sqrtf(dist2);
    const f3 n = dist > 0.0f ? f3{d.x / dist, d.y / dist, d.z / dist} : f3{0.0f, 1.0f, 0.0f};
    const float depth = rs - dist;
    const float s = ra - 0.5f * depth;
    c->n = n;
    c->p[0] = f3{ca.x + n.x * s, ca.y + n.y * s, ca.z + n.z * s};
    c->depth[0] = depth;
    c->count = 1;
    return true;
}

// Sphere (centre cs, radius r) against the plane through pp with unit normal np.
__device__ __forceinline__ bool spherePlane(axd::f3 pp, axd::f3 np, axd::f3 cs, float r, Contact* c) {
    using namespace axd;
    const float s = dot(sub(cs, pp), np);
    if (s > r) return false;
    const float depth = r - s;
    const float k = r - 0.5f * depth;
    c->n = np;
    c->p[0] = f3{cs.x - np.x * k, cs.y - np.y * k, cs.z - np.z * k};
    c->depth[0] = depth;
    c->count = 1;
    return true;
}

__device__ __forceinline__ void collidePair(const Geom& a, const Geom& b, Contact* c) {
    using namespace axd;
    c->count = 0;
    if (a.shape == AXIOM_SHAPE_SPHERE && b.shape == AXIOM_SHAPE_SPHERE) {
        sphereSphere(mk(a.pos), a.ext.x, mk(b.pos), b.ext.x, c);
        return;
    }
}

__device__ __forceinline__ void collidePlane(axd::f3 pp, axd::f3 np, const Geom& g, Contact* c) {
    using namespace axd;
    c->count = 0;
    if (g.shape == AXIOM_SHAPE_SPHERE) {
        spherePlane(pp, np, mk(g.pos), g.ext.x, c);
        return;
    }
}

}  // namespace axiom_gb300
