// integrate_math.cuh — per-body integration and AABB arithmetic shared by the
// single-world kernels (integrate.cu) and the batched-world kernel (batch.cu).
//
// Semi-implicit Euler (the reference's toy step integrates explicitly,
// examples/profiling_example.cpp:35-41; this step integrates velocity first, solves
// contacts, then moves positions with the solved velocity).  Damping follows the
// linearDamping / angularDamping fields of gui::RigidBodyData (body_inspector.hpp:77-78)
// as v *= 1 / (1 + dt * damping).
#include "dmath.cuh"
#include "world.h"

#pragma once

namespace axiom_gb300 {

using namespace axd;

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Cell coordinate of one AABB min-corner component: floor(v / cell) clamped to
// [-2^16, 2^16] (monotone, so adjacent cells stay adjacent), then wrapped to 10 bits.
__device__ __forceinline__ uint32_t cellCoord(float v, float invCell) {
    float c = floorf(v * invCell);
    c = c > 65536.0f ? 65536.0f : c;
    c = c < -65536.0f ? -65536.0f : c;
    c = (c == c) ? c : -65536.0f;  // NaN
    return (uint32_t)((int32_t)c) & 0x3FFu;
}

__device__ __forceinline__ f3 halfExtentsWorld(uint32_t shape, float4 e, float4 q) {
    if (shape == AXIOM_SHAPE_SPHERE) return f3{e.x, e.x, e.x};
    if (shape == AXIOM_SHAPE_BOX) {
        m3 r = rotmat(q);
        return f3{fabsf(r.m[0][0]) * e.x + fabsf(r.m[0][1]) * e.y + fabsf(r.m[0][2]) * e.z,
                  fabsf(r.m[1][0]) * e.x + fabsf(r.m[1][1]) * e.y + fabsf(r.m[1][2]) * e.z,
                  fabsf(r.m[2][0]) * e.x + fabsf(r.m[2][1]) * e.y + fabsf(r.m[2][2]) * e.z};
    }
    if (shape == AXIOM_SHAPE_CAPSULE) {
        m3 r = rotmat(q);
        return f3{fabsf(r.m[0][1]) * e.y + e.x, fabsf(r.m[1][1]) * e.y + e.x,
                  fabsf(r.m[2][1]) * e.y + e.x};
    }
    if (shape == AXIOM_SHAPE_CYLINDER) {
        // axis u = column 1: |u_i| h + r sqrt(1 - u_i^2) (the cap disc's extent along axis i)
        m3 r = rotmat(q);
        float ext[3];
        for (int i = 0; i < 3; ++i) {
            const float u = r.m[i][1];
            const float s = 1.0f - u * u;
            ext[i] = fabsf(u) * e.y + e.x * sqrtf(s > 0.0f ? s : 0.0f);
        }
        return f3{ext[0], ext[1], ext[2]};
    }
    if (isHullShape(shape)) return f3{e.x, e.x, e.x};  // bounding sphere of the hull (or triangle)
    return f3{0.0f, 0.0f, 0.0f};
}

// Gravity and damping on body i (dynamic only) and its world inverse inertia.
__device__ __forceinline__ void velocityStep(uint32_t i, const StepParams& sp, const uint32_t* __restrict__ info,
                                             const float4* __restrict__ rot, SolverBody* __restrict__ sb,
                                             const float4* __restrict__ mat, const float4* __restrict__ iloc,
                                             float4* __restrict__ iw0, float4* __restrict__ iw1) {
    const uint32_t inf = info[i];
    const uint32_t type = inf & kInfoTypeMask;
    const uint32_t shape = (inf >> 4) & 0xFu;
    const float4 q = rot[i];
    if (type == AXIOM_BODY_DYNAMIC) {
        const float4 m = mat[i];
        float4 v = sb[i].v, w = sb[i].w;
        const float ld = 1.0f / (1.0f + sp.dt * m.z);
        const float ad = 1.0f / (1.0f + sp.dt * m.w);
        v.x = (v.x + sp.gx * sp.dt) * ld;
        v.y = (v.y + sp.gy * sp.dt) * ld;
        v.z = (v.z + sp.gz * sp.dt) * ld;
        w.x = w.x * ad;
        w.y = w.y * ad;
        w.z = w.z * ad;
        sb[i].v = v;
        sb[i].w = w;
        if (w.w < 0.0f) {
            const float4 il = iloc[i];
            const m3 r = rotmat(q);
            const f3 ii{il.x, il.y, il.z};
            iw0[i] = make_float4(inertiaEntry(r, ii, 0, 0), inertiaEntry(r, ii, 1, 1),
                                 inertiaEntry(r, ii, 2, 2), inertiaEntry(r, ii, 0, 1));
            iw1[i] = make_float4(inertiaEntry(r, ii, 0, 2), inertiaEntry(r, ii, 1, 2), 0.0f, 0.0f);
        }
    }
}

// AABB of body i (planes get their position as an empty box); returns the min corner.
__device__ __forceinline__ f3 bodyAabb(uint32_t i, const StepParams& sp, const uint32_t* __restrict__ info,
                                       const float4* __restrict__ pos, const float4* __restrict__ rot,
                                       const float4* __restrict__ shp, float4* __restrict__ aabbMin,
                                       float4* __restrict__ aabbMax) {
    const uint32_t shape = (info[i] >> 4) & 0xFu;
    const float4 q = rot[i];
    const float4 p = pos[i];
    f3 e = halfExtentsWorld(shape, shp[i], q);
    e = f3{e.x + sp.margin, e.y + sp.margin, e.z + sp.margin};
    const f3 mn{p.x - e.x, p.y - e.y, p.z - e.z};
    const f3 mx{p.x + e.x, p.y + e.y, p.z + e.z};
    aabbMin[i] = make_float4(mn.x, mn.y, mn.z, 0.0f);
    aabbMax[i] = make_float4(mx.x, mx.y, mx.z, 0.0f);
    return mn;
}

// Position and orientation update of body i (not static, not sleeping, not a plane).
__device__ __forceinline__ void positionStep(uint32_t i, const StepParams& sp, const uint32_t* __restrict__ info,
                                             float4* __restrict__ pos, float4* __restrict__ rot,
                                             const SolverBody* __restrict__ sb) {
    const uint32_t inf = info[i];
    const uint32_t type = inf & kInfoTypeMask;
    const uint32_t shape = (inf >> 4) & 0xFu;
    if (type == AXIOM_BODY_STATIC || type == kTypeSleeping || shape == AXIOM_SHAPE_PLANE) return;
    const float4 v = sb[i].v, o = sb[i].w;
    float4 p = pos[i];
    p.x = p.x + v.x * sp.dt;
    p.y = p.y + v.y * sp.dt;
    p.z = p.z + v.z * sp.dt;
    pos[i] = p;
    float4 q = rot[i];
    const float dx = o.x * q.w + (o.y * q.z - o.z * q.y);
    const float dy = o.y * q.w + (o.z * q.x - o.x * q.z);
    const float dz = o.z * q.w + (o.x * q.y - o.y * q.x);
    const float dw = -(o.x * q.x + o.y * q.y + o.z * q.z);
    q = make_float4(q.x + dx * sp.hdt, q.y + dy * sp.hdt, q.z + dz * sp.hdt, q.w + dw * sp.hdt);
    rot[i] = qnormalize(q);
}

}  // namespace axiom_gb300
