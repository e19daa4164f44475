// body_pack.h — validation and device layout of an axiom_body_soa (host code), shared by
// the single world (world.cu) and the batched worlds (batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "host_math.h"
#include "world.h"

namespace axiom_gb300 {

// Device shp of a convex body: (bounding radius, pool offset bits, vertex count bits, 0).
inline float4 convexShp(const HullInfo& h) {
    float4 v;
    v.x = h.radius;
    std::memcpy(&v.y, &h.offset, 4);
    std::memcpy(&v.z, &h.count, 4);
    v.w = 0.0f;
    return v;
}

struct PackedBodies {
    std::vector<float4> pos, rot, shp, mat, iloc;
    std::vector<SolverBody> body;
    std::vector<uint32_t> info;
    std::vector<uint4> filt;  // (category, mask, group, 0)
};

// True when every number given for body i is finite, the rotation has a length, and the
// quantities that cannot be negative (mass, inertia, density, friction, restitution,
// damping, rolling friction) are not.
inline bool finiteBody(const axiom_body_soa* b, uint32_t i) {
    auto fin = [](const float* a, uint32_t k) {
        for (uint32_t j = 0; j < k; ++j)
            if (!std::isfinite(a[j])) return false;
        return true;
    };
    auto nonneg = [](const float* a, uint32_t k) {
        for (uint32_t j = 0; j < k; ++j)
            if (!(a[j] >= 0.0f) || !std::isfinite(a[j])) return false;
        return true;
    };
    if (!fin(b->position + 3 * i, 3) || !fin(b->shape_extents + 3 * i, 3)) return false;
    if (b->rotation) {
        const float* q = b->rotation + 4 * i;
        if (!fin(q, 4) || !((q[0] * q[0] + q[1] * q[1]) + (q[2] * q[2] + q[3] * q[3]) > 0.0f)) return false;
    }
    if (b->linear_velocity && !fin(b->linear_velocity + 3 * i, 3)) return false;
    if (b->angular_velocity && !fin(b->angular_velocity + 3 * i, 3)) return false;
    if (b->mass && !nonneg(b->mass + i, 1)) return false;
    if (b->inertia && !nonneg(b->inertia + 3 * i, 3)) return false;
    if (b->density && !nonneg(b->density + i, 1)) return false;
    if (b->friction && !nonneg(b->friction + i, 1)) return false;
    if (b->restitution && !nonneg(b->restitution + i, 1)) return false;
    if (b->linear_damping && !nonneg(b->linear_damping + i, 1)) return false;
    if (b->angular_damping && !nonneg(b->angular_damping + i, 1)) return false;
    if (b->rolling_friction && !nonneg(b->rolling_friction + i, 1)) return false;
    return true;
}

// hullCount: hulls the world holds; a negative value (batched worlds) admits neither
// cylinders nor convex hulls.
inline int32_t validateBodies(const axiom_body_soa* b, uint32_t n, int64_t hullCount = -1) {
    if (!b) return AXIOM_NULL_POINTER;
    if (n == 0) return AXIOM_SUCCESS;
    if (!b->type || !b->shape || !b->position || !b->shape_extents) return AXIOM_NULL_POINTER;
    for (uint32_t i = 0; i < n; ++i) {
        if (b->type[i] > AXIOM_BODY_KINEMATIC || !finiteBody(b, i)) return AXIOM_INVALID_RIGID_BODY;
        const uint32_t s = b->shape[i];
        const bool extended = hullCount >= 0 && (s == AXIOM_SHAPE_CYLINDER || isHullShape(s));
        if (s != AXIOM_SHAPE_SPHERE && s != AXIOM_SHAPE_BOX && s != AXIOM_SHAPE_CAPSULE && s != AXIOM_SHAPE_PLANE &&
            !extended)
            return AXIOM_INVALID_SHAPE;
        if (s == AXIOM_SHAPE_MESH && b->type[i] == AXIOM_BODY_DYNAMIC) return AXIOM_INVALID_SHAPE;
        if (isHullShape(s)) {
            if (!b->convex_hull) return AXIOM_NULL_POINTER;
            if ((int64_t)b->convex_hull[i] >= hullCount) return AXIOM_INVALID_SHAPE;
            continue;
        }
        if (s == AXIOM_SHAPE_PLANE && b->type[i] == AXIOM_BODY_DYNAMIC) return AXIOM_INVALID_SHAPE;
        const float* e = b->shape_extents + 3 * i;
        if (s == AXIOM_SHAPE_SPHERE && !(e[0] > 0.0f)) return AXIOM_INVALID_SHAPE;
        if (s == AXIOM_SHAPE_BOX && !(e[0] > 0.0f && e[1] > 0.0f && e[2] > 0.0f)) return AXIOM_INVALID_SHAPE;
        if (s == AXIOM_SHAPE_CAPSULE && !(e[0] > 0.0f && e[1] >= 0.0f)) return AXIOM_INVALID_SHAPE;
        if (s == AXIOM_SHAPE_CYLINDER && !(e[0] > 0.0f && e[1] > 0.0f)) return AXIOM_INVALID_SHAPE;
    }
    return AXIOM_SUCCESS;
}

// Bodies [first, first + n) of the description, in the device layout of world.h.  With
// sleepEnabled (the world's allow_sleep), SleepInfo::isSleeping adds a dynamic body asleep
// and SleepInfo::allowSleep = 0 marks it as never sleeping; without it both are ignored.
inline void packBodies(const axiom_body_soa* b, uint32_t first, uint32_t n, PackedBodies* o,
                       bool sleepEnabled = false, const std::vector<HullInfo>* hulls = nullptr) {
    o->pos.resize(n);
    o->rot.resize(n);
    o->shp.resize(n);
    o->mat.resize(n);
    o->iloc.resize(n);
    o->body.resize(n);
    o->info.resize(n);
    o->filt.resize(n);
    for (uint32_t q = 0; q < n; ++q) {
        const uint32_t i = first + q;
        const uint32_t s = b->shape[i], t = b->type[i];
        const float* e = b->shape_extents + 3 * i;
        const float density = b->density ? b->density[i] : 1000.0f;
        float mass = 0.0f, inertia[3] = {0.0f, 0.0f, 0.0f};
        const HullInfo* hull = isHullShape(s) ? &(*hulls)[b->convex_hull[i]] : nullptr;
        if (hull) massProperties(AXIOM_SHAPE_BOX, hull->halfExtents, density, &mass, inertia);
        else massProperties(s, e, density, &mass, inertia);
        if (b->mass) mass = b->mass[i];
        if (b->inertia) {
            inertia[0] = b->inertia[3 * i];
            inertia[1] = b->inertia[3 * i + 1];
            inertia[2] = b->inertia[3 * i + 2];
        }
        const bool dyn = t == AXIOM_BODY_DYNAMIC && mass > 0.0f;
        const float invMass = dyn ? 1.0f / mass : 0.0f;
        float ii[3] = {0.0f, 0.0f, 0.0f};
        if (dyn)
            for (int k = 0; k < 3; ++k) ii[k] = inertia[k] > 0.0f ? 1.0f / inertia[k] : 0.0f;
        const bool iso = ii[0] == ii[1] && ii[1] == ii[2];
        o->pos[q] = make_float4(b->position[3 * i], b->position[3 * i + 1], b->position[3 * i + 2], 0.0f);
        o->rot[q] = b->rotation ? make_float4(b->rotation[4 * i], b->rotation[4 * i + 1], b->rotation[4 * i + 2],
                                              b->rotation[4 * i + 3])
                                : make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        const float* lv = b->linear_velocity ? b->linear_velocity + 3 * i : nullptr;
        const float* av = b->angular_velocity ? b->angular_velocity + 3 * i : nullptr;
        o->body[q].v = make_float4(lv ? lv[0] : 0.0f, lv ? lv[1] : 0.0f, lv ? lv[2] : 0.0f, invMass);
        o->body[q].w = make_float4(av ? av[0] : 0.0f, av ? av[1] : 0.0f, av ? av[2] : 0.0f, iso ? ii[0] : -1.0f);
        o->shp[q] = hull ? convexShp(*hull) : make_float4(e[0], e[1], e[2], 0.0f);
        o->mat[q] = make_float4(b->friction ? b->friction[i] : 0.5f, b->restitution ? b->restitution[i] : 0.5f,
                                b->linear_damping ? b->linear_damping[i] : 0.01f,
                                b->angular_damping ? b->angular_damping[i] : 0.05f);
        // .w carries MaterialInfo::rollingFriction (not applied by the solver)
        o->iloc[q] = make_float4(ii[0], ii[1], ii[2], b->rolling_friction ? b->rolling_friction[i] : 0.0f);
        const uint32_t cat = b->filter_category ? b->filter_category[i] : 0x0001u;
        const uint32_t msk = b->filter_mask ? b->filter_mask[i] : 0xFFFFu;
        const int32_t grp = b->filter_group ? (int32_t)b->filter_group[i] : 0;
        o->filt[q] = make_uint4(cat, msk, (uint32_t)grp, 0u);
        const bool filtered = cat != 0x0001u || msk != 0xFFFFu || grp != 0;
        uint32_t type = t;
        uint32_t sleepBits = 0u;
        if (sleepEnabled && t == AXIOM_BODY_DYNAMIC) {
            const bool allow = b->allow_sleep ? b->allow_sleep[i] != 0 : true;
            if (!allow) sleepBits = kInfoNoSleep;
            else if (b->is_sleeping && b->is_sleeping[i]) type = kTypeSleeping;
        }
        if (type == kTypeSleeping) {  // added asleep: at rest
            o->body[q].v = make_float4(0.0f, 0.0f, 0.0f, invMass);
            o->body[q].w = make_float4(0.0f, 0.0f, 0.0f, iso ? ii[0] : -1.0f);
        }
        o->info[q] = type | (s << 4) | (filtered ? kInfoFiltered : 0u) | sleepBits;
    }
}

}  // namespace axiom_gb300
