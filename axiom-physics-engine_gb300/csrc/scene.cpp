// scene.cpp — seeded synthetic scenes (host code; see include/axiom_scene.h).
#include "../../include/axiom_scene.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <unordered_map>
#include <vector>

#include "host_math.h"

using axiom_gb300::Pcg32;

namespace {

struct SceneBuilder {
    std::vector<uint32_t> type, shape;
    std::vector<float> pos, rot, ext, friction;

    void add(uint32_t t, uint32_t s, float x, float y, float z, const float q[4], float e0, float e1,
             float e2, float mu) {
        type.push_back(t);
        shape.push_back(s);
        pos.insert(pos.end(), {x, y, z});
        rot.insert(rot.end(), {q[0], q[1], q[2], q[3]});
        ext.insert(ext.end(), {e0, e1, e2});
        friction.push_back(mu);
    }

    void addGroundPlane(float mu) {
        const float q[4] = {0.0f, 0.0f, 0.0f, 1.0f};
        add(AXIOM_BODY_STATIC, AXIOM_SHAPE_PLANE, 0.0f, 0.0f, 0.0f, q, 0.0f, 0.0f, 0.0f, mu);
    }

    template <typename T>
    static T* copyOut(const std::vector<T>& v) {
        T* p = static_cast<T*>(std::malloc(sizeof(T) * (v.empty() ? 1 : v.size())));
        if (p && !v.empty()) std::memcpy(p, v.data(), sizeof(T) * v.size());
        return p;
    }

    int32_t finish(axiom_scene** out, uint32_t structures = 0) {
        const uint32_t n = static_cast<uint32_t>(type.size());
        axiom_scene* s = static_cast<axiom_scene*>(std::calloc(1, sizeof(axiom_scene)));
        if (!s) return AXIOM_OUT_OF_MEMORY;
        s->n = n;
        s->structures = structures;
        std::vector<float> zero3(3 * (size_t)n, 0.0f), mass(n), inertia(3 * (size_t)n),
            density(n, 1000.0f), zero1(n, 0.0f);
        for (uint32_t i = 0; i < n; ++i) {
            float m = 0.0f, in[3] = {0.0f, 0.0f, 0.0f};
            if (type[i] == AXIOM_BODY_DYNAMIC)
                axiom_gb300::massProperties(shape[i], &ext[3 * i], density[i], &m, in);
            mass[i] = m;
            inertia[3 * i] = in[0];
            inertia[3 * i + 1] = in[1];
            inertia[3 * i + 2] = in[2];
        }
        s->type = copyOut(type);
        s->shape = copyOut(shape);
        s->position = copyOut(pos);
        s->rotation = copyOut(rot);
        s->linear_velocity = copyOut(zero3);
        s->angular_velocity = copyOut(zero3);
        s->shape_extents = copyOut(ext);
        s->mass = copyOut(mass);
        s->inertia = copyOut(inertia);
        s->friction = copyOut(friction);
        s->restitution = copyOut(zero1);
        s->density = copyOut(density);
        s->linear_damping = copyOut(zero1);
        s->angular_damping = copyOut(zero1);
        if (!s->type || !s->shape || !s->position || !s->rotation || !s->linear_velocity ||
            !s->angular_velocity || !s->shape_extents || !s->mass || !s->inertia ||
            !s->friction || !s->restitution || !s->density || !s->linear_damping ||
            !s->angular_damping) {
            axiom_scene_free(s);
            return AXIOM_OUT_OF_MEMORY;
        }
        *out = s;
        return AXIOM_SUCCESS;
    }
};

// Uniform unit quaternion by Marsaglia (1972): two points uniform in the unit disc,
// q = (x1, y1, x2 k, y2 k) with k = sqrt((1 - s1) / s2); renormalised once.
void randomQuat(Pcg32& rng, float q[4]) {
    float x1, y1, s1, x2, y2, s2;
    do {
        x1 = rng.nextFloat(-1.0f, 1.0f);
        y1 = rng.nextFloat(-1.0f, 1.0f);
        s1 = x1 * x1 + y1 * y1;
    } while (!(s1 < 1.0f));
    do {
        x2 = rng.nextFloat(-1.0f, 1.0f);
        y2 = rng.nextFloat(-1.0f, 1.0f);
        s2 = x2 * x2 + y2 * y2;
    } while (!(s2 < 1.0f && s2 > 0.0f));
    float k = std::sqrt((1.0f - s1) / s2);
    float v[4] = {x1, y1, x2 * k, y2 * k};
    float len = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3]);
    float inv = 1.0f / len;
    for (int i = 0; i < 4; ++i) q[i] = v[i] * inv;
}

const float kIdentity[4] = {0.0f, 0.0f, 0.0f, 1.0f};

// nx * ny * nz spheres on a jittered cubic lattice, y outermost, then z, then x: body id =
// (j * nz + k) * nx + i; the bottom layer's centres at y = radius (+ jitter).
int32_t addLattice(SceneBuilder& b, uint64_t seed, uint32_t nx, uint32_t ny, uint32_t nz, float spacing,
                   float radius, float jitter, float friction) {
    if (nx == 0 || ny == 0 || nz == 0 || !(radius > 0.0f) || !(spacing > 0.0f) || !(jitter >= 0.0f))
        return AXIOM_INVALID_PARAMETER;
    if ((uint64_t)nx * ny * nz >= (1ull << 30)) return AXIOM_OUT_OF_RANGE;
    Pcg32 rng(seed);
    const size_t n = (size_t)nx * ny * nz;
    b.type.reserve(n + 5);
    b.shape.reserve(n + 5);
    b.pos.reserve(3 * n + 15);
    b.rot.reserve(4 * n + 20);
    b.ext.reserve(3 * n + 15);
    b.friction.reserve(n + 5);
    for (uint32_t j = 0; j < ny; ++j)
        for (uint32_t k = 0; k < nz; ++k)
            for (uint32_t i = 0; i < nx; ++i) {
                float jx = rng.nextFloat(-jitter, jitter);
                float jy = rng.nextFloat(-jitter, jitter);
                float jz = rng.nextFloat(-jitter, jitter);
                float x = (float)i * spacing + jx;
                float y = radius + (float)j * spacing + jy;
                float z = (float)k * spacing + jz;
                b.add(AXIOM_BODY_DYNAMIC, AXIOM_SHAPE_SPHERE, x, y, z, kIdentity, radius, 0.0f, 0.0f,
                      friction);
            }
    return AXIOM_SUCCESS;
}

}  // namespace

extern "C" {

AXIOM_API int32_t axiom_scene_sphere_drop(uint64_t seed, uint32_t count, float radius, float sx,
                                          float sy, float sz, float friction, axiom_scene** out) {
    if (!out) return AXIOM_NULL_POINTER;
    if (!(radius > 0.0f) || !(sx > 2.0f * radius) || !(sy > 2.0f * radius) || !(sz > 2.0f * radius))
        return AXIOM_INVALID_PARAMETER;
    Pcg32 rng(seed);
    SceneBuilder b;
    const float d2min = (2.0f * radius) * (2.0f * radius);
    const double cell = 2.0 * radius;
    std::unordered_map<uint64_t, std::vector<uint32_t>> grid;
    auto key = [](int64_t x, int64_t y, int64_t z) {
        return ((uint64_t)(x + 1048576) << 42) | ((uint64_t)(y + 1048576) << 21) | (uint64_t)(z + 1048576);
    };
    uint64_t attempts = 0;
    const uint64_t maxAttempts = 1000ull * count + 1000ull;
    while (b.type.size() < count) {
        if (++attempts > maxAttempts) return AXIOM_OUT_OF_RANGE;  // box too full
        float x = rng.nextFloat(radius, sx - radius);
        float y = rng.nextFloat(radius, sy - radius);
        float z = rng.nextFloat(radius, sz - radius);
        int64_t cx = (int64_t)std::floor(x / cell), cy = (int64_t)std::floor(y / cell),
                cz = (int64_t)std::floor(z / cell);
        bool ok = true;
        for (int dz = -1; dz <= 1 && ok; ++dz)
            for (int dy = -1; dy <= 1 && ok; ++dy)
                for (int dx = -1; dx <= 1 && ok; ++dx) {
                    auto it = grid.find(key(cx + dx, cy + dy, cz + dz));
                    if (it == grid.end()) continue;
                    for (uint32_t j : it->second) {
                        float ex = x - b.pos[3 * j], ey = y - b.pos[3 * j + 1], ez = z - b.pos[3 * j + 2];
                        if (ex * ex + ey * ey + ez * ez < d2min) {
                            ok = false;
                            break;
                        }
                    }
                }
        if (!ok) continue;
        grid[key(cx, cy, cz)].push_back((uint32_t)b.type.size());
        b.add(AXIOM_BODY_DYNAMIC, AXIOM_SHAPE_SPHERE, x, y, z, kIdentity, radius, 0.0f, 0.0f, friction);
    }
    b.addGroundPlane(friction);
    return b.finish(out);
}

AXIOM_API int32_t axiom_scene_sphere_lattice(uint64_t seed, uint32_t nx, uint32_t ny, uint32_t nz,
                                             float spacing, float radius, float jitter,
                                             float friction, axiom_scene** out) {
    if (!out) return AXIOM_NULL_POINTER;
    SceneBuilder b;
    const int32_t st = addLattice(b, seed, nx, ny, nz, spacing, radius, jitter, friction);
    if (st != AXIOM_SUCCESS) return st;
    b.addGroundPlane(friction);
    return b.finish(out);
}

AXIOM_API int32_t axiom_scene_sphere_pile(uint64_t seed, uint32_t nx, uint32_t ny, uint32_t nz,
                                          float spacing, float radius, float jitter, float friction,
                                          axiom_scene** out) {
    if (!out) return AXIOM_NULL_POINTER;
    SceneBuilder b;
    const int32_t st = addLattice(b, seed, nx, ny, nz, spacing, radius, jitter, friction);
    if (st != AXIOM_SUCCESS) return st;
    // four walls touching the unjittered outer spheres: x = -r, x = (nx-1)s + r, z = -r,
    // z = (nz-1)s + r, each plane's normal (rotation * +Y) pointing into the pile
    const float h = 0.70710677f;
    const float qxPos[4] = {0.0f, 0.0f, -h, h}, qxNeg[4] = {0.0f, 0.0f, h, h};
    const float qzPos[4] = {h, 0.0f, 0.0f, h}, qzNeg[4] = {-h, 0.0f, 0.0f, h};
    const float xHi = (float)(nx - 1) * spacing + radius, zHi = (float)(nz - 1) * spacing + radius;
    b.add(AXIOM_BODY_STATIC, AXIOM_SHAPE_PLANE, -radius, 0.0f, 0.0f, qxPos, 0.0f, 0.0f, 0.0f, friction);
    b.add(AXIOM_BODY_STATIC, AXIOM_SHAPE_PLANE, xHi, 0.0f, 0.0f, qxNeg, 0.0f, 0.0f, 0.0f, friction);
    b.add(AXIOM_BODY_STATIC, AXIOM_SHAPE_PLANE, 0.0f, 0.0f, -radius, qzPos, 0.0f, 0.0f, 0.0f, friction);
    b.add(AXIOM_BODY_STATIC, AXIOM_SHAPE_PLANE, 0.0f, 0.0f, zHi, qzNeg, 0.0f, 0.0f, 0.0f, friction);
    b.addGroundPlane(friction);
    return b.finish(out);
}

AXIOM_API int32_t axiom_scene_mixed(uint64_t seed, uint32_t count, float sx, float sy, float sz,
                                    float friction, axiom_scene** out) {
    if (!out) return AXIOM_NULL_POINTER;
    if (!(sx > 0.0f) || !(sy > 2.0f) || !(sz > 0.0f)) return AXIOM_INVALID_PARAMETER;
    Pcg32 rng(seed);
    SceneBuilder b;
    for (uint32_t i = 0; i < count; ++i) {
        float u = rng.nextFloat();
        float q[4] = {0.0f, 0.0f, 0.0f, 1.0f};
        float e[3] = {0.0f, 0.0f, 0.0f};
        uint32_t shape;
        if (u < 0.4f) {
            shape = AXIOM_SHAPE_SPHERE;
            e[0] = rng.nextFloat(0.2f, 0.6f);
        } else if (u < 0.8f) {
            shape = AXIOM_SHAPE_BOX;
            e[0] = rng.nextFloat(0.2f, 0.8f);
            e[1] = rng.nextFloat(0.2f, 0.8f);
            e[2] = rng.nextFloat(0.2f, 0.8f);
            randomQuat(rng, q);
        } else {
            shape = AXIOM_SHAPE_CAPSULE;
            e[0] = rng.nextFloat(0.1f, 0.3f);
            e[1] = rng.nextFloat(0.2f, 0.6f);
            randomQuat(rng, q);
        }
        float br = axiom_gb300::boundingRadius(shape, e);
        float x = rng.nextFloat(0.0f, sx);
        float y = rng.nextFloat(br, sy);
        float z = rng.nextFloat(0.0f, sz);
        b.add(AXIOM_BODY_DYNAMIC, shape, x, y, z, q, e[0], e[1], e[2], friction);
    }
    b.addGroundPlane(friction);
    return b.finish(out);
}

AXIOM_API int32_t axiom_scene_towers(uint64_t seed, uint32_t count, float friction, axiom_scene** out) {
    if (!out) return AXIOM_NULL_POINTER;
    if (count == 0) return AXIOM_INVALID_PARAMETER;
    Pcg32 rng(seed);
    SceneBuilder b;
    uint32_t side = 1;
    while ((uint64_t)side * side < count) ++side;
    const float spacing = 24.0f;
    for (uint32_t s = 0; s < count; ++s) {
        float ox = (float)(s % side) * spacing, oz = (float)(s / side) * spacing;
        uint32_t kind = rng.next() & 1u;
        if (kind == 0) {
            // pyramid: base 4..16 boxes along x, one box fewer per level
            uint32_t base = 4 + rng.next() % 13u;
            float y = 0.0f, prevHalf = 0.0f;
            for (uint32_t l = 0; l < base; ++l) {
                uint32_t cnt = base - l;
                std::vector<float> he(3 * (size_t)cnt);
                float maxHalf = 0.0f;
                for (uint32_t k = 0; k < cnt; ++k) {
                    for (int a = 0; a < 3; ++a) he[3 * k + a] = 0.5f * (1.0f + rng.nextFloat(-0.02f, 0.02f));
                    maxHalf = he[3 * k + 1] > maxHalf ? he[3 * k + 1] : maxHalf;
                }
                y = (l == 0) ? maxHalf : y + prevHalf + maxHalf;
                for (uint32_t k = 0; k < cnt; ++k) {
                    float x = ox + ((float)k - (float)(cnt - 1) * 0.5f) * 1.05f;
                    b.add(AXIOM_BODY_DYNAMIC, AXIOM_SHAPE_BOX, x, y, oz, kIdentity, he[3 * k],
                          he[3 * k + 1], he[3 * k + 2], friction);
                }
                prevHalf = maxHalf;
            }
        } else {
            // tower: a single column of 4..32 boxes
            uint32_t h = 4 + rng.next() % 29u;
            float y = 0.0f, prevHalf = 0.0f;
            for (uint32_t l = 0; l < h; ++l) {
                float e[3];
                for (int a = 0; a < 3; ++a) e[a] = 0.5f * (1.0f + rng.nextFloat(-0.02f, 0.02f));
                y = (l == 0) ? e[1] : y + prevHalf + e[1];
                b.add(AXIOM_BODY_DYNAMIC, AXIOM_SHAPE_BOX, ox, y, oz, kIdentity, e[0], e[1], e[2], friction);
                prevHalf = e[1];
            }
        }
    }
    b.addGroundPlane(friction);
    return b.finish(out, count);
}

AXIOM_API int32_t axiom_scene_batch(uint64_t seed, uint32_t worlds, float median, float sigma,
                                    uint32_t minBodies, uint32_t maxBodies, float friction, uint32_t* sizes,
                                    axiom_scene** out) {
    if (!out || !sizes) return AXIOM_NULL_POINTER;
    if (worlds == 0 || !(median > 0.0f) || !(sigma >= 0.0f) || minBodies < 2 || maxBodies < minBodies)
        return AXIOM_INVALID_PARAMETER;
    Pcg32 rng(seed);
    SceneBuilder b;
    for (uint32_t w = 0; w < worlds; ++w) {
        // standard normal by Box-Muller (double precision; only the rounded count is kept)
        double u1 = (double)rng.next() / 4294967296.0, u2 = (double)rng.next() / 4294967296.0;
        if (u1 < 1e-300) u1 = 1e-300;
        const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
        double c = std::floor((double)median * std::exp((double)sigma * z) + 0.5);
        c = c < minBodies ? minBodies : (c > maxBodies ? maxBodies : c);
        const uint32_t n = (uint32_t)c - 1u;  // the count includes the world's plane
        const uint32_t cols = (n + 5u) / 6u;
        uint32_t side = 1;
        while (side * side < cols) ++side;
        uint32_t placed = 0;
        for (uint32_t col = 0; col < cols; ++col) {
            const float cx = (float)(col % side) * 1.5f, cz = (float)(col / side) * 1.5f;
            float top = 0.0f;
            for (uint32_t k = 0; k < 6u && placed < n; ++k, ++placed) {
                const bool box = (rng.next() & 1u) != 0u;
                if (box) {
                    float e[3];
                    for (int a = 0; a < 3; ++a) e[a] = rng.nextFloat(0.3f, 0.45f);
                    const float y = top + e[1] + 0.005f;
                    b.add(AXIOM_BODY_DYNAMIC, AXIOM_SHAPE_BOX, cx, y, cz, kIdentity, e[0], e[1], e[2], friction);
                    top = y + e[1];
                } else {
                    const float r = rng.nextFloat(0.3f, 0.45f);
                    const float y = top + r + 0.005f;
                    b.add(AXIOM_BODY_DYNAMIC, AXIOM_SHAPE_SPHERE, cx, y, cz, kIdentity, r, 0.0f, 0.0f, friction);
                    top = y + r;
                }
            }
        }
        b.addGroundPlane(friction);
        sizes[w] = n + 1u;
    }
    return b.finish(out, worlds);
}

AXIOM_API void axiom_scene_free(axiom_scene* s) {
    if (!s) return;
    std::free(s->type);
    std::free(s->shape);
    std::free(s->position);
    std::free(s->rotation);
    std::free(s->linear_velocity);
    std::free(s->angular_velocity);
    std::free(s->shape_extents);
    std::free(s->mass);
    std::free(s->inertia);
    std::free(s->friction);
    std::free(s->restitution);
    std::free(s->density);
    std::free(s->linear_damping);
    std::free(s->angular_damping);
    std::free(s);
}

AXIOM_API void axiom_scene_as_soa(const axiom_scene* s, axiom_body_soa* o) {
    if (!s || !o) return;
    o->type = s->type;
    o->shape = s->shape;
    o->position = s->position;
    o->rotation = s->rotation;
    o->linear_velocity = s->linear_velocity;
    o->angular_velocity = s->angular_velocity;
    o->shape_extents = s->shape_extents;
    o->mass = s->mass;
    o->inertia = s->inertia;
    o->friction = s->friction;
    o->restitution = s->restitution;
    o->density = s->density;
    o->linear_damping = s->linear_damping;
    o->angular_damping = s->angular_damping;
    o->filter_category = nullptr;  // scenes use the default collision filter
    o->filter_mask = nullptr;
    o->filter_group = nullptr;
    o->allow_sleep = nullptr;
    o->is_sleeping = nullptr;
}

AXIOM_API void axiom_rng_u32(uint64_t seed, uint32_t count, uint32_t* out) {
    Pcg32 rng(seed);
    for (uint32_t i = 0; i < count; ++i) out[i] = rng.next();
}

AXIOM_API void axiom_rng_float(uint64_t seed, uint32_t count, float* out) {
    Pcg32 rng(seed);
    for (uint32_t i = 0; i < count; ++i) out[i] = rng.nextFloat();
}

AXIOM_API void axiom_rng_float_range(uint64_t seed, uint32_t count, float lo, float hi, float* out) {
    Pcg32 rng(seed);
    for (uint32_t i = 0; i < count; ++i) out[i] = rng.nextFloat(lo, hi);
}

}  // extern "C"
