// oracle_world.cpp — TEST INFRASTRUCTURE ONLY: the CPU oracle of the rigid-body step.
//
// This file is the checker for the CUDA library, never a fallback for it.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load oracle/liboracle.so.
//
// The reference (itsakeyfut/axiom-physics-engine) reserves src/collision and
// src/dynamics for this step and ships them empty (src/CMakeLists.txt:24-27), so there
// is no reference implementation to run.  This oracle is the step written out plainly,
// sequential where order matters, in the reference's stage order
// (examples/profiling_example.cpp:132-165: broadphase, narrowphase, solver,
// integration) and on the reference's math semantics (oracle_math.h).  It exports the
// C ABI of include/axiom_c.h so tests drive it and the GPU library through one binding.
//
// Every fp32 expression is written in the order the CUDA kernels use; both sides avoid
// fused multiply-add, so results are bit-identical, not merely close.
//
// Parity pinning: the math semantics it rests on are pinned by golden vectors made from
// the reference's own headers (tests/golden/ref_math.json, made by
// tests/golden/make_golden.py via oracle/ref_golden.cpp).  The step itself has no
// reference known-answer test (the reference has no step), so its trajectories are
// frozen as golden files by this project.
#include "../include/axiom_c.h"
#include "oracle_math.h"
#include "oracle_mlp.h"
#include "oracle_narrow.h"

#include <algorithm>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <functional>
#include <cstring>
#include <new>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace oracle;

namespace {

struct Imp3 {
    float v[3];
    uint32_t tag = 0;  // point 0 of a manifold: 1 + its colour in that step (0: none)
};

constexpr float kFourThirdsPi = 4.18879020f;
// a manifold at a dynamic body with more than kCrowdDegree manifolds is crowded: colour
// kCrowdColour, solved serially after the colours (as the GPU library does)
constexpr uint32_t kCrowdDegree = 32;
constexpr uint32_t kCrowdColour = 64;
// Type of a dynamic body while it sleeps (gui::SleepInfo::isSleeping): not dynamic for any
// stage until it wakes.  No island: static and kinematic bodies.
constexpr uint32_t kSleeping = 3u;
constexpr uint32_t kNoIsland = 0xFFFFFFFFu;
constexpr int kMaxWakePasses = 8;
constexpr uint32_t kNoHull = 0xFFFFFFFFu;
constexpr float kPi = 3.14159265f;

struct OWorld {
    axiom_world_config cfg;
    // body state (SoA)
    std::vector<uint32_t> type, shape;
    std::vector<V3> pos, vel, ang, ext, invInertia;
    std::vector<Q4> rot;
    std::vector<float> invMass, friction, restitution, linDamp, angDamp, boundRadius;
    std::vector<float> rollingFriction;  // MaterialInfo::rollingFriction (carried, not applied)
    std::vector<uint8_t> iso;  // inverse inertia isotropic -> scalar path
    std::vector<uint32_t> filterCategory, filterMask;  // gui::FilterInfo (body_inspector.hpp:38-42)
    std::vector<int32_t> filterGroup;
    // convex hulls (gui::ShapeType::Convex): points in the body frame; per body its hull
    std::vector<std::vector<V3>> hullPts;
    std::vector<float> hullRadius;
    std::vector<V3> hullHalf;  // half the body-frame bounding box
    std::vector<uint32_t> hullId;  // per body; kNoHull for other shapes
    // sleeping (gui::SleepInfo, body_inspector.hpp:45-51)
    std::vector<uint8_t> noSleep;   // allowSleep == false
    std::vector<float> sleepTime;
    std::vector<uint32_t> island;   // lowest body id of the island (kNoIsland: static / kinematic)
    uint32_t islandCount = 0;
    // speculative contacts: each body's displacement |v dt| this step (0 without sweeping)
    std::vector<float> sweep;
    // per-step products
    std::vector<V3> aabbMin, aabbMax;
    std::vector<Sym3> invIw;
    std::vector<uint32_t> pairs;  // 2 per pair
    std::vector<Manifold> manifolds;
    std::vector<uint32_t> colour;
    uint32_t colourCount = 0;
    uint32_t colourRounds = 0;  // longest chain of higher-priority neighbours (parallel rounds)
    std::vector<uint32_t> crowded;  // manifolds solved serially after the colours, by priority
    uint32_t gjkFailures = 0;   // pairs of the last narrowphase whose GJK ran out of iterations
    uint32_t epaFailures = 0;   // pairs whose EPA stopped at a cap before its tolerance
    // previous-step impulses by (pair key, point index)
    std::unordered_map<uint64_t, Imp3> prevImpulse;
    bool warmValid = false;  // a step has run since bodies were last added or loaded
    // learned warm start
    std::vector<float> mlp;
    int threads = 1;
    bool recording = false;     // keep features and impulses of the last step
    bool needFeatures = false;  // this step computes warm-start features
    float gdt = 0.0f;           // |g| * dt of this step
};

inline bool isPlane(const OWorld& w, uint32_t i) { return w.shape[i] == AXIOM_SHAPE_PLANE; }

inline BodyGeom geomOf(const OWorld& w, uint32_t i) {
    BodyGeom g{w.shape[i], w.pos[i], w.rot[i], w.ext[i]};
    g.sweep = w.sweep[i];
    if (isHull(w.shape[i])) {
        const auto& h = w.hullPts[w.hullId[i]];
        g.verts = h.data();
        g.nverts = (uint32_t)h.size();
    }
    return g;
}
inline bool isDynamic(const OWorld& w, uint32_t i) { return w.type[i] == AXIOM_BODY_DYNAMIC; }

// Bounding radius of a shape about its centre (for the grid cell size).
float boundingRadius(uint32_t shape, V3 e) {
    switch (shape) {
        case AXIOM_SHAPE_SPHERE: return e.x;
        case AXIOM_SHAPE_BOX: return std::sqrt(e.x * e.x + e.y * e.y + e.z * e.z);
        case AXIOM_SHAPE_CAPSULE: return e.x + e.y;
        case AXIOM_SHAPE_CYLINDER: return std::sqrt(e.x * e.x + e.y * e.y);
        case AXIOM_SHAPE_CONVEX:
        case AXIOM_SHAPE_MESH: return e.x;  // hull ext: (bounding radius, 0, 0)
        default: return 0.0f;
    }
}

// Mass and body-frame diagonal inertia from density (solid shapes).
void massProperties(uint32_t shape, V3 e, float density, float* mass, V3* inertia) {
    if (shape == AXIOM_SHAPE_SPHERE) {
        float r = e.x;
        float m = density * (kFourThirdsPi * r * r * r);
        float i = 0.4f * m * r * r;
        *mass = m;
        *inertia = V3{i, i, i};
    } else if (shape == AXIOM_SHAPE_BOX) {
        float m = density * (8.0f * e.x * e.y * e.z);
        float k = m / 3.0f;
        *mass = m;
        *inertia = V3{k * (e.y * e.y + e.z * e.z), k * (e.x * e.x + e.z * e.z),
                      k * (e.x * e.x + e.y * e.y)};
    } else if (shape == AXIOM_SHAPE_CAPSULE) {
        float r = e.x, h = e.y;
        float mc = density * (kPi * r * r * (2.0f * h));
        float ms = density * (kFourThirdsPi * r * r * r);
        float iy = mc * r * r * 0.5f + ms * 0.4f * r * r;
        float ix = mc * (h * h / 3.0f + r * r * 0.25f) + ms * (0.4f * r * r + h * h + 0.75f * h * r);
        *mass = mc + ms;
        *inertia = V3{ix, iy, ix};
    } else if (shape == AXIOM_SHAPE_CYLINDER) {
        // m = rho pi r^2 2h; I_y = m r^2 / 2; I_x = I_z = m (3 r^2 + 4 h^2) / 12
        float r = e.x, h = e.y;
        float m = density * (kPi * r * r * (2.0f * h));
        float iy = 0.5f * m * r * r;
        float ix = m * (3.0f * r * r + 4.0f * h * h) / 12.0f;
        *mass = m;
        *inertia = V3{ix, iy, ix};
    } else {
        *mass = 0.0f;
        *inertia = V3{0.0f, 0.0f, 0.0f};
    }
}

// ---- stage 1: velocity integration (semi-implicit Euler, gravity + damping) ----
void integrateBodyVelocity(OWorld& w, int64_t i, float dt) {
    const V3 g{w.cfg.gravity[0], w.cfg.gravity[1], w.cfg.gravity[2]};
    float ld = 1.0f / (1.0f + dt * w.linDamp[i]);
    float ad = 1.0f / (1.0f + dt * w.angDamp[i]);
    V3 v = w.vel[i];
    v.x = (v.x + g.x * dt) * ld;
    v.y = (v.y + g.y * dt) * ld;
    v.z = (v.z + g.z * dt) * ld;
    w.vel[i] = v;
    w.ang[i] = V3{w.ang[i].x * ad, w.ang[i].y * ad, w.ang[i].z * ad};
}

void integrateVelocities(OWorld& w, float dt) {
    const int64_t n = (int64_t)w.type.size();
#pragma omp parallel for num_threads(w.threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        if (w.type[i] == AXIOM_BODY_DYNAMIC) integrateBodyVelocity(w, i, dt);
        if (!w.iso[i]) w.invIw[i] = worldInvInertia(w.rot[i], w.invInertia[i]);
    }
}

// ---- stage 2: AABBs (AABB::fromCenterExtents, aabb.hpp:213-215, plus margin); with
// speculative contacts each moving body's AABB is swept by its displacement v dt and its
// sweep length |v dt| kept for the narrowphase ----
void computeAabbs(OWorld& w, float dt) {
    const float margin = w.cfg.aabb_margin;
    const bool spec = w.cfg.speculative_contacts != 0;
    const int64_t n = (int64_t)w.type.size();
#pragma omp parallel for num_threads(w.threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        V3 e = shapeHalfExtentsWorld(w.shape[i], w.ext[i], w.rot[i]);
        e = V3{e.x + margin, e.y + margin, e.z + margin};
        w.aabbMin[i] = sub(w.pos[i], e);
        w.aabbMax[i] = add(w.pos[i], e);
        w.sweep[i] = 0.0f;
        const uint32_t t = w.type[i];
        if (spec && (t == AXIOM_BODY_DYNAMIC || t == AXIOM_BODY_KINEMATIC) && !isPlane(w, (uint32_t)i)) {
            const V3 v = w.vel[i];
            const float dx = v.x * dt, dy = v.y * dt, dz = v.z * dt;
            V3& lo = w.aabbMin[i];
            V3& hi = w.aabbMax[i];
            lo = V3{lo.x + (dx < 0.0f ? dx : 0.0f), lo.y + (dy < 0.0f ? dy : 0.0f), lo.z + (dz < 0.0f ? dz : 0.0f)};
            hi = V3{hi.x + (dx > 0.0f ? dx : 0.0f), hi.y + (dy > 0.0f ? dy : 0.0f), hi.z + (dz > 0.0f ? dz : 0.0f)};
            w.sweep[i] = std::sqrt(dx * dx + dy * dy + dz * dz);
        }
    }
}

inline bool overlaps(const OWorld& w, uint32_t a, uint32_t b) {
    // AABB::intersects, inclusive (aabb.hpp:132-135).
    const V3 &amin = w.aabbMin[a], &amax = w.aabbMax[a];
    const V3 &bmin = w.aabbMin[b], &bmax = w.aabbMax[b];
    return amin.x <= bmax.x && amax.x >= bmin.x && amin.y <= bmax.y && amax.y >= bmin.y &&
           amin.z <= bmax.z && amax.z >= bmin.z;
}

// ---- stage 3: broadphase.  Pair set = every (a<b), neither a plane, at least one
// awake dynamic (or a sleeper and a moving kinematic body), whose AABBs intersect
// inclusively.  Enumerated through a uniform grid keyed on
// the AABB min corner (cell >= the widest AABB, so overlapping boxes sit in adjacent
// cells); the grid only enumerates candidates, the set is fixed by the overlap test.
// Collision filter (gui::FilterInfo): the same non-zero group decides alone (positive:
// collide, negative: never); otherwise each body's category must be in the other's mask.
// A kinematic body with a non-zero velocity: it wakes sleeping bodies it touches.
inline bool isMover(const OWorld& w, uint32_t i) {
    if (w.type[i] != AXIOM_BODY_KINEMATIC) return false;
    const V3 v = w.vel[i], o = w.ang[i];
    return v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || o.x != 0.0f || o.y != 0.0f || o.z != 0.0f;
}

// Broadphase admission: at least one awake dynamic body, or a sleeping body touched by a
// moving kinematic body (so that the contact can wake it).
inline bool admitPair(const OWorld& w, uint32_t a, uint32_t b) {
    if (isDynamic(w, a) || isDynamic(w, b)) return true;
    return (w.type[a] == kSleeping && isMover(w, b)) || (isMover(w, a) && w.type[b] == kSleeping);
}

inline bool shouldCollide(const OWorld& w, uint32_t a, uint32_t b) {
    const int32_t ga = w.filterGroup[a], gb = w.filterGroup[b];
    if (ga == gb && ga != 0) return ga > 0;
    return (w.filterMask[a] & w.filterCategory[b]) != 0u && (w.filterCategory[a] & w.filterMask[b]) != 0u;
}

void broadphase(OWorld& w) {
    w.pairs.clear();
    const uint32_t n = (uint32_t)w.type.size();
    std::vector<uint32_t> all;
    std::vector<float> width;
    all.reserve(n);
    for (uint32_t i = 0; i < n; ++i) {
        if (isPlane(w, i)) continue;
        all.push_back(i);
        width.push_back(maxf(maxf(w.aabbMax[i].x - w.aabbMin[i].x, w.aabbMax[i].y - w.aabbMin[i].y),
                             w.aabbMax[i].z - w.aabbMin[i].z));
    }
    if (all.empty()) return;
    // bodies far wider than the rest (wider than 8 x the median AABB width, at most 64)
    // stay out of the grid and are tested against every body; the pair set is the same
    float limit = FLT_MAX;
    if (all.size() >= 64) {
        std::vector<float> med(width);
        std::nth_element(med.begin(), med.begin() + med.size() / 2, med.end());
        std::vector<float> top(width);
        const size_t k = std::min<size_t>(65, top.size());
        std::partial_sort(top.begin(), top.begin() + k, top.end(), std::greater<float>());
        size_t taken = 0;
        while (taken < k - 1 && top[taken] > 8.0f * med[med.size() / 2]) ++taken;
        if (taken) limit = top[taken];
    }
    std::vector<uint32_t> ids, large;
    float maxw = 0.0f;
    for (size_t k = 0; k < all.size(); ++k) {
        if (width[k] > limit) {
            large.push_back(all[k]);
        } else {
            ids.push_back(all[k]);
            maxw = maxf(maxw, width[k]);
        }
    }
    for (uint32_t l : large)
        for (uint32_t j : all) {
            if (j == l) continue;
            const bool jLarge = std::binary_search(large.begin(), large.end(), j);
            if (jLarge && j < l) continue;  // reported from j's row
            const uint32_t a = l < j ? l : j, b = l < j ? j : l;
            if (admitPair(w, a, b) && overlaps(w, a, b) && shouldCollide(w, a, b)) {
                w.pairs.push_back(a);
                w.pairs.push_back(b);
            }
        }
    if (ids.empty()) return;
    double cell = (maxw > 0.0f ? (double)maxw : 1.0) * 1.0625 + 1e-6;
    // Cell coordinates clamp to +-(2^20 - 2): clamping is monotone and moves no two
    // coordinates further apart, so adjacent cells stay adjacent, and the packed key below
    // stays injective (21 bits per axis).
    const double lim = (double)((1 << 20) - 2);
    auto coord = [&](float v) -> int64_t {
        double c = std::floor((double)v / cell);
        if (!(c > -lim)) c = -lim;  // NaN and -inf clamp low
        if (c > lim) c = lim;
        return (int64_t)c;
    };
    auto cellKey = [](int64_t x, int64_t y, int64_t z) -> uint64_t {
        return ((uint64_t)(x + (1 << 20)) << 42) | ((uint64_t)(y + (1 << 20)) << 21) |
               (uint64_t)(z + (1 << 20));
    };
    struct Entry {
        int64_t cx, cy, cz;
        uint32_t id;
    };
    std::vector<Entry> ent(ids.size());
    for (size_t k = 0; k < ids.size(); ++k) {
        uint32_t i = ids[k];
        ent[k] = Entry{coord(w.aabbMin[i].x), coord(w.aabbMin[i].y), coord(w.aabbMin[i].z), i};
    }
    std::unordered_map<uint64_t, std::vector<uint32_t>> grid;
    grid.reserve(ent.size() * 2);
    for (const Entry& e : ent) grid[cellKey(e.cx, e.cy, e.cz)].push_back(e.id);
    // Each body looks at all 27 cells and keeps partners with a larger id.
    std::vector<std::vector<uint32_t>> local(w.threads);
    const int64_t m = (int64_t)ent.size();
#pragma omp parallel for num_threads(w.threads) schedule(dynamic, 1024)
    for (int64_t k = 0; k < m; ++k) {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        const Entry& e = ent[k];
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    auto it = grid.find(cellKey(e.cx + dx, e.cy + dy, e.cz + dz));
                    if (it == grid.end()) continue;
                    for (uint32_t j : it->second) {
                        if (j <= e.id) continue;
                        if (!admitPair(w, e.id, j)) continue;
                        if (overlaps(w, e.id, j) && shouldCollide(w, e.id, j)) {
                            local[t].push_back(e.id);
                            local[t].push_back(j);
                        }
                    }
                }
    }
    for (auto& v : local) w.pairs.insert(w.pairs.end(), v.begin(), v.end());
}

// ---- stage 4: narrowphase (pairs + planes) ----
void narrowphase(OWorld& w) {
    w.manifolds.clear();
    const int64_t np = (int64_t)w.pairs.size() / 2;
    const int64_t nb = (int64_t)w.type.size();
    std::vector<uint32_t> planes;
    for (uint32_t i = 0; i < w.type.size(); ++i)
        if (isPlane(w, i)) planes.push_back(i);
    // Manifold order is irrelevant downstream (colouring is by priority, PGS by colour),
    // so every thread keeps its own list.
    std::vector<std::vector<Manifold>> local(w.threads);
    std::vector<uint32_t> gjkFail(w.threads, 0u), epaFail(w.threads, 0u);
#pragma omp parallel num_threads(w.threads)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        std::vector<Manifold>& out = local[t];
#pragma omp for schedule(static)
        for (int64_t k = 0; k < np; ++k) {
            uint32_t a = w.pairs[2 * k], b = w.pairs[2 * k + 1];
            BodyGeom ga = geomOf(w, a);
            BodyGeom gb = geomOf(w, b);
            Manifold mf;
            uint32_t fail = 0;
            if (collide(a, ga, b, gb, &mf, &fail)) out.push_back(mf);
            gjkFail[t] += (fail & kFailGjk) ? 1u : 0u;
            epaFail[t] += (fail & kFailEpa) ? 1u : 0u;
        }
        // planes against every dynamic body
#pragma omp for schedule(static)
        for (int64_t i = 0; i < nb; ++i) {
            if (isPlane(w, (uint32_t)i) || !isDynamic(w, (uint32_t)i)) continue;
            BodyGeom gi = geomOf(w, (uint32_t)i);
            for (uint32_t p : planes) {
                if (!shouldCollide(w, p, (uint32_t)i)) continue;
                BodyGeom gp = geomOf(w, p);
                Manifold mf;
                if (collidePlane(p, gp, (uint32_t)i, gi, &mf)) out.push_back(mf);
            }
        }
    }
    w.gjkFailures = w.epaFailures = 0;
    for (int t = 0; t < w.threads; ++t) {
        w.gjkFailures += gjkFail[t];
        w.epaFailures += epaFail[t];
    }
    size_t total = 0;
    for (auto& v : local) total += v.size();
    w.manifolds.reserve(total);
    for (auto& v : local) w.manifolds.insert(w.manifolds.end(), v.begin(), v.end());
}

// ---- stage 5: deterministic colouring.  Manifolds are coloured greedily in descending
// priority mix64(pairKey); each takes the lowest colour unused at its dynamic bodies.
// This equals the parallel rounds the GPU runs (a manifold is coloured only once every
// higher-priority manifold sharing a dynamic body is coloured), and the number of rounds
// is the longest chain of such manifolds: round(m) = 1 + the latest round at its bodies.
// Temporally coherent mode (cfg.temporal_colouring): a manifold whose pair had a colour in
// the previous step keeps it unless a higher-priority manifold at a shared dynamic body had
// the same previous colour; the kept colours start the bodies' used masks, and only the
// other manifolds are coloured greedily (and counted in the rounds).
int colourContacts(OWorld& w) {
    const size_t m = w.manifolds.size();
    std::vector<std::pair<uint64_t, uint32_t>> order(m);
    for (size_t k = 0; k < m; ++k)
        order[k] = {mix64(pairKey(w.manifolds[k].a, w.manifolds[k].b)), (uint32_t)k};
    std::sort(order.begin(), order.end(),
              [](const auto& x, const auto& y) { return x.first > y.first; });
    std::vector<uint64_t> used(w.type.size(), 0);
    std::vector<uint32_t> lastRound(w.type.size(), 0);
    w.colour.assign(m, 0);
    std::vector<uint8_t> kept(m, 0);
    // crowded: a dynamic body with more than kCrowdDegree manifolds; such manifolds take no
    // colour and are solved serially after the colours, in descending priority
    std::vector<uint32_t> deg(w.type.size(), 0);
    for (const Manifold& mf : w.manifolds) {
        if (isDynamic(w, mf.a)) ++deg[mf.a];
        if (isDynamic(w, mf.b)) ++deg[mf.b];
    }
    std::vector<uint8_t> crowded(m, 0);
    w.crowded.clear();
    for (const auto& o : order) {
        const Manifold& mf = w.manifolds[o.second];
        if ((isDynamic(w, mf.a) && deg[mf.a] > kCrowdDegree) || (isDynamic(w, mf.b) && deg[mf.b] > kCrowdDegree)) {
            crowded[o.second] = 1;
            w.colour[o.second] = kCrowdColour;
            w.crowded.push_back(o.second);  // in descending priority
        }
    }
    if (w.cfg.temporal_colouring && w.warmValid) {
        constexpr uint32_t kNoColour = 0xFFFFFFFFu;
        std::vector<uint32_t> prev(m, kNoColour);
#pragma omp parallel for num_threads(w.threads) schedule(static)
        for (int64_t k = 0; k < (int64_t)m; ++k) {
            auto it = w.prevImpulse.find(pairKey(w.manifolds[k].a, w.manifolds[k].b) * 4u);
            if (it != w.prevImpulse.end() && it->second.tag) prev[k] = it->second.tag - 1u;
        }
        // in descending priority, seen[x] holds the previous colours of the higher-priority
        // manifolds at body x: a manifold whose previous colour is among them is recoloured
        std::vector<uint64_t> seen(w.type.size(), 0);
        for (const auto& o : order) {
            const uint32_t k = o.second;
            if (prev[k] == kNoColour || crowded[k]) continue;
            const Manifold& mf = w.manifolds[k];
            const bool da = isDynamic(w, mf.a), db = isDynamic(w, mf.b);
            const uint64_t bit = 1ull << prev[k];
            const bool dup = (da && (seen[mf.a] & bit)) || (db && (seen[mf.b] & bit));
            if (da) seen[mf.a] |= bit;
            if (db) seen[mf.b] |= bit;
            if (dup) continue;
            kept[k] = 1;
            w.colour[k] = prev[k];
            if (da) used[mf.a] |= bit;
            if (db) used[mf.b] |= bit;
        }
    }
    uint32_t ncol = 0, rounds = 0;
    for (size_t k = 0; k < m; ++k)
        if (kept[k] && w.colour[k] + 1 > ncol) ncol = w.colour[k] + 1;
    for (auto& o : order) {
        if (kept[o.second] || crowded[o.second]) continue;
        const Manifold& mf = w.manifolds[o.second];
        uint64_t mask = 0;
        bool da = isDynamic(w, mf.a), db = isDynamic(w, mf.b);
        if (da) mask |= used[mf.a];
        if (db) mask |= used[mf.b];
        if (mask == ~0ULL) return AXIOM_CONSTRAINT_SOLVER_FAILURE;  // > 64 colours
        uint32_t c = (uint32_t)__builtin_ctzll(~mask);
        w.colour[o.second] = c;
        if (da) used[mf.a] |= (1ULL << c);
        if (db) used[mf.b] |= (1ULL << c);
        if (c + 1 > ncol) ncol = c + 1;
        const uint32_t r = 1u + std::max(da ? lastRound[mf.a] : 0u, db ? lastRound[mf.b] : 0u);
        if (da) lastRound[mf.a] = r;
        if (db) lastRound[mf.b] = r;
        rounds = std::max(rounds, r);
    }
    w.colourCount = ncol;
    w.colourRounds = rounds;
    return AXIOM_SUCCESS;
}

// Inverse inertia applied to a vector: scalar path for isotropic bodies.
inline V3 applyInvI(const OWorld& w, uint32_t b, V3 v) {
    if (w.iso[b]) {
        float s = w.invInertia[b].x;
        return V3{s * v.x, s * v.y, s * v.z};
    }
    return mulSym(w.invIw[b], v);
}

// Apply impulse P at offsets rA/rB: A loses, B gains.  Static and kinematic bodies carry
// zero inverse mass/inertia and are never written.
inline void applyImpulse(OWorld& w, uint32_t a, uint32_t b, V3 rA, V3 rB, V3 P) {
    if (isDynamic(w, a)) {
        float m = w.invMass[a];
        w.vel[a] = V3{w.vel[a].x - m * P.x, w.vel[a].y - m * P.y, w.vel[a].z - m * P.z};
        V3 dw = applyInvI(w, a, cross(rA, P));
        w.ang[a] = V3{w.ang[a].x - dw.x, w.ang[a].y - dw.y, w.ang[a].z - dw.z};
    }
    if (isDynamic(w, b)) {
        float m = w.invMass[b];
        w.vel[b] = V3{w.vel[b].x + m * P.x, w.vel[b].y + m * P.y, w.vel[b].z + m * P.z};
        V3 dw = applyInvI(w, b, cross(rB, P));
        w.ang[b] = V3{w.ang[b].x + dw.x, w.ang[b].y + dw.y, w.ang[b].z + dw.z};
    }
}

inline V3 relVel(const OWorld& w, uint32_t a, uint32_t b, V3 rA, V3 rB) {
    V3 va = add(w.vel[a], cross(w.ang[a], rA));
    V3 vb = add(w.vel[b], cross(w.ang[b], rB));
    return sub(vb, va);
}

inline float invMassOf(const OWorld& w, uint32_t b) { return isDynamic(w, b) ? w.invMass[b] : 0.0f; }

// ---- stage 6: solver prep (effective masses, bias, warm-start impulses) ----
void prepare(OWorld& w, float dt) {
    const float invDt = 1.0f / dt;
    const float biasCoeff = w.cfg.baumgarte * invDt;
    const int64_t m = (int64_t)w.manifolds.size();
#pragma omp parallel for num_threads(w.threads) schedule(static)
    for (int64_t k = 0; k < m; ++k) {
        Manifold& mf = w.manifolds[k];
        const uint32_t a = mf.a, b = mf.b;
        const float mA = invMassOf(w, a), mB = invMassOf(w, b);
        const bool dA = isDynamic(w, a), dB = isDynamic(w, b);
        const float mu = std::sqrt(w.friction[a] * w.friction[b]);
        const float e = maxf(w.restitution[a], w.restitution[b]);
        for (uint32_t p = 0; p < mf.count; ++p) {
            ContactPoint& c = mf.pts[p];
            c.rA = sub(c.p, w.pos[a]);
            c.rB = sub(c.p, w.pos[b]);
            V3 t1, t2;
            tangentBasis(c.n, &t1, &t2);
            auto effMass = [&](V3 dir) {
                V3 ra = cross(c.rA, dir), rb = cross(c.rB, dir);
                float kA = dA ? dot(ra, applyInvI(w, a, ra)) : 0.0f;
                float kB = dB ? dot(rb, applyInvI(w, b, rb)) : 0.0f;
                float k = mA + mB + kA + kB;
                return k > 0.0f ? 1.0f / k : 0.0f;
            };
            c.kn = effMass(c.n);
            c.kt1 = effMass(t1);
            c.kt2 = effMass(t2);
            c.mu = mu;
            // touching: Baumgarte beyond the slop and restitution; speculative (a gap,
            // depth < 0): the point may close exactly its gap this step
            float bias = c.depth >= 0.0f ? biasCoeff * maxf(c.depth - w.cfg.linear_slop, 0.0f) : c.depth * invDt;
            if (e > 0.0f && c.depth >= 0.0f) {
                float vn0 = dot(relVel(w, a, b, c.rA, c.rB), c.n);
                if (vn0 < -w.cfg.restitution_threshold) bias = maxf(bias, -e * vn0);
            }
            c.bias = bias;
            // previous-step impulses of this (pair, point)
            c.prev[0] = c.prev[1] = c.prev[2] = 0.0f;
            auto it = w.prevImpulse.find(pairKey(a, b) * 4u + p);
            if (it != w.prevImpulse.end()) {
                c.prev[0] = it->second.v[0];
                c.prev[1] = it->second.v[1];
                c.prev[2] = it->second.v[2];
            }
            if (w.needFeatures) {
                // warm-start network features, dimensionless:
                //  relative velocity in the contact frame / (|g| dt), normal, depth / slop,
                //  inverse masses x kn, previous impulses / (kn |g| dt), linear share of
                //  the effective mass, friction
                V3 dv = relVel(w, a, b, c.rA, c.rB);
                const float vScale = w.gdt > 0.0f ? 1.0f / w.gdt : 1.0f;
                const float slop = w.cfg.linear_slop;
                const float sImp = c.kn * w.gdt;
                const float invImp = sImp > 0.0f ? 1.0f / sImp : 0.0f;
                c.feat[0] = dot(dv, c.n) * vScale;
                c.feat[1] = dot(dv, t1) * vScale;
                c.feat[2] = dot(dv, t2) * vScale;
                c.feat[3] = c.n.x;
                c.feat[4] = c.n.y;
                c.feat[5] = c.n.z;
                c.feat[6] = slop > 0.0f ? c.depth / slop : c.depth;
                c.feat[7] = mA * c.kn;
                c.feat[8] = mB * c.kn;
                c.feat[9] = c.prev[0] * invImp;
                c.feat[10] = c.prev[1] * invImp;
                c.feat[11] = c.prev[2] * invImp;
                c.feat[12] = (mA + mB) * c.kn;
                c.feat[13] = mu;
                c.impScale = sImp;
            }
        }
    }
}

void warmStartFromPrevious(OWorld& w) {
    const float f = w.cfg.warm_start_factor;
    const bool use = w.cfg.warm_start == AXIOM_WARM_START_PREVIOUS;
    for (Manifold& mf : w.manifolds)
        for (uint32_t p = 0; p < mf.count; ++p) {
            ContactPoint& c = mf.pts[p];
            c.lambda[0] = use ? c.prev[0] * f : 0.0f;
            c.lambda[1] = use ? c.prev[1] * f : 0.0f;
            c.lambda[2] = use ? c.prev[2] * f : 0.0f;
        }
}

// Learned warm start: the network (oracle_mlp.h) predicts the correction to the
// previous-step impulse in units of the contact's impulse scale; the start is
// factor x (prev + y * scale), clamped to the cone the solver enforces.
void warmStartLearned(OWorld& w) {
    std::vector<float> feat;
    std::vector<ContactPoint*> pts;
    for (Manifold& mf : w.manifolds)
        for (uint32_t p = 0; p < mf.count; ++p) {
            pts.push_back(&mf.pts[p]);
            feat.insert(feat.end(), mf.pts[p].feat, mf.pts[p].feat + 14);
        }
    MlpCache cache;
    if (w.mlp.size() == kMlpCount && !pts.empty()) mlpForward(w.mlp.data(), feat.data(), (uint32_t)pts.size(), &cache);
    const float f = w.cfg.warm_start_factor;
    for (size_t q = 0; q < pts.size(); ++q) {
        ContactPoint& c = *pts[q];
        if (w.mlp.size() != kMlpCount) {
            c.lambda[0] = c.lambda[1] = c.lambda[2] = 0.0f;
            continue;
        }
        float ln = c.prev[0] + (float)cache.y[3 * q] * c.impScale;
        ln = ln > 0.0f ? ln : 0.0f;
        const float mf = c.mu * ln;
        float l1 = c.prev[1] + (float)cache.y[3 * q + 1] * c.impScale;
        float l2 = c.prev[2] + (float)cache.y[3 * q + 2] * c.impScale;
        l1 = l1 > mf ? mf : (l1 < -mf ? -mf : l1);
        l2 = l2 > mf ? mf : (l2 < -mf ? -mf : l2);
        c.lambda[0] = ln * f;
        c.lambda[1] = l1 * f;
        c.lambda[2] = l2 * f;
    }
}

// Manifold indices grouped by colour (any order inside a colour gives the same result,
// since no two manifolds of one colour share a dynamic body).
// The colour batches, then the crowded batch (in descending priority) as the last one;
// serialFrom = the index of the crowded batch (batches.size() when there is none).
std::vector<std::vector<uint32_t>> colourBatches(const OWorld& w, size_t* serialFrom) {
    std::vector<std::vector<uint32_t>> batches(w.colourCount);
    for (uint32_t k = 0; k < w.manifolds.size(); ++k)
        if (w.colour[k] != kCrowdColour) batches[w.colour[k]].push_back(k);
    *serialFrom = batches.size();
    if (!w.crowded.empty()) batches.push_back(w.crowded);
    return batches;
}

void applyWarmStart(OWorld& w, const std::vector<std::vector<uint32_t>>& batches, size_t serialFrom) {
    for (size_t bi = 0; bi < batches.size(); ++bi) {
        const auto& batch = batches[bi];
        const int64_t nb = (int64_t)batch.size();
        const int threads = bi >= serialFrom ? 1 : w.threads;  // the crowded batch in order
#pragma omp parallel for num_threads(threads) schedule(static)
        for (int64_t q = 0; q < nb; ++q) {
            Manifold& mf = w.manifolds[batch[q]];
            for (uint32_t p = 0; p < mf.count; ++p) {
                ContactPoint& c = mf.pts[p];
                V3 t1, t2;
                tangentBasis(c.n, &t1, &t2);
                V3 P{c.n.x * c.lambda[0] + t1.x * c.lambda[1] + t2.x * c.lambda[2],
                     c.n.y * c.lambda[0] + t1.y * c.lambda[1] + t2.y * c.lambda[2],
                     c.n.z * c.lambda[0] + t1.z * c.lambda[1] + t2.z * c.lambda[2]};
                applyImpulse(w, mf.a, mf.b, c.rA, c.rB, P);
            }
        }
    }
}

// One PGS sweep; returns (max|dλ|, max|λ|) over all rows.
void solveSweep(OWorld& w, const std::vector<std::vector<uint32_t>>& batches, size_t serialFrom, float* maxDelta,
                float* maxLambda) {
    float gd = 0.0f, gl = 0.0f;
    for (size_t bi = 0; bi < batches.size(); ++bi) {
        const auto& batch = batches[bi];
        const int64_t nb = (int64_t)batch.size();
        const int threads = bi >= serialFrom ? 1 : w.threads;  // the crowded batch in order
#pragma omp parallel for num_threads(threads) schedule(static) reduction(max : gd, gl)
        for (int64_t q = 0; q < nb; ++q) {
            Manifold& mf = w.manifolds[batch[q]];
            const uint32_t a = mf.a, b = mf.b;
            for (uint32_t p = 0; p < mf.count; ++p) {
                ContactPoint& c = mf.pts[p];
                // normal row
                V3 dv = relVel(w, a, b, c.rA, c.rB);
                float vn = dot(dv, c.n);
                float lnOld = c.lambda[0];
                float ln = lnOld + c.kn * (c.bias - vn);
                ln = ln > 0.0f ? ln : 0.0f;
                float dn = ln - lnOld;
                c.lambda[0] = ln;
                applyImpulse(w, a, b, c.rA, c.rB, scale(c.n, dn));
                // friction rows (box clamp at mu * λn)
                V3 t1, t2;
                tangentBasis(c.n, &t1, &t2);
                dv = relVel(w, a, b, c.rA, c.rB);
                float vt1 = dot(dv, t1), vt2 = dot(dv, t2);
                float maxF = c.mu * ln;
                float l1 = c.lambda[1] - c.kt1 * vt1;
                float l2 = c.lambda[2] - c.kt2 * vt2;
                l1 = l1 > maxF ? maxF : (l1 < -maxF ? -maxF : l1);
                l2 = l2 > maxF ? maxF : (l2 < -maxF ? -maxF : l2);
                float d1 = l1 - c.lambda[1], d2 = l2 - c.lambda[2];
                c.lambda[1] = l1;
                c.lambda[2] = l2;
                V3 P{t1.x * d1 + t2.x * d2, t1.y * d1 + t2.y * d2, t1.z * d1 + t2.z * d2};
                applyImpulse(w, a, b, c.rA, c.rB, P);
                gd = maxf(gd, maxf(std::fabs(dn), maxf(std::fabs(d1), std::fabs(d2))));
                gl = maxf(gl, maxf(std::fabs(ln), maxf(std::fabs(l1), std::fabs(l2))));
            }
        }
    }
    *maxDelta = gd;
    *maxLambda = gl;
}

// ---- stage 8: position integration (x += v dt; q += 0.5 (ω,0)⊗q dt; normalise) ----
void integratePositions(OWorld& w, float dt) {
    const float hdt = 0.5f * dt;
    const int64_t n = (int64_t)w.type.size();
#pragma omp parallel for num_threads(w.threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        if (w.type[i] == AXIOM_BODY_STATIC || w.type[i] == kSleeping || isPlane(w, (uint32_t)i)) continue;
        V3 v = w.vel[i], o = w.ang[i];
        w.pos[i] = V3{w.pos[i].x + v.x * dt, w.pos[i].y + v.y * dt, w.pos[i].z + v.z * dt};
        Q4 q = w.rot[i];
        Q4 dq{o.x * q.w + (o.y * q.z - o.z * q.y), o.y * q.w + (o.z * q.x - o.x * q.z),
              o.z * q.w + (o.x * q.y - o.y * q.x), -(o.x * q.x + o.y * q.y + o.z * q.z)};
        q = Q4{q.x + dq.x * hdt, q.y + dq.y * hdt, q.z + dq.z * hdt, q.w + dq.w * hdt};
        w.rot[i] = qnormalize(q);
    }
}

// ---- wake (PhysicsWorldConfig::allowSleep): a contact between a sleeping body and an
// awake dynamic or a kinematic body (the broadphase pairs a sleeper with a kinematic body
// only while that one moves) wakes the sleeper's whole island in this step; woken bodies
// get this step's velocity integration.  Returns the number of woken bodies.
uint32_t wakePass(OWorld& w, float dt) {
    std::vector<uint8_t> mark(w.type.size(), 0);
    for (const Manifold& mf : w.manifolds) {
        const uint32_t ta = w.type[mf.a], tb = w.type[mf.b];
        if (ta == kSleeping && (tb == AXIOM_BODY_DYNAMIC || tb == AXIOM_BODY_KINEMATIC)) mark[w.island[mf.a]] = 1;
        if (tb == kSleeping && (ta == AXIOM_BODY_DYNAMIC || ta == AXIOM_BODY_KINEMATIC)) mark[w.island[mf.b]] = 1;
    }
    uint32_t woken = 0;
    for (size_t i = 0; i < w.type.size(); ++i) {
        if (w.type[i] != kSleeping || !mark[w.island[i]]) continue;
        w.type[i] = AXIOM_BODY_DYNAMIC;
        w.sleepTime[i] = 0.0f;
        integrateBodyVelocity(w, (int64_t)i, dt);
        ++woken;
    }
    return woken;
}

// ---- islands and sleeping (after position integration).  Sleep time grows by dt while
// |v|^2 and |w|^2 stay at or below the squared thresholds; islands are the connected
// components of the awake dynamic bodies under contacts between two of them, labelled by
// their lowest body id; an island whose every body has slept sleep_time_threshold falls
// asleep with zero velocities.
void islandsAndSleep(OWorld& w, float dt) {
    const size_t n = w.type.size();
    const float lin2 = w.cfg.sleep_linear_threshold * w.cfg.sleep_linear_threshold;
    const float ang2 = w.cfg.sleep_angular_threshold * w.cfg.sleep_angular_threshold;
    std::vector<uint32_t> parent(n);
    for (size_t i = 0; i < n; ++i) {
        parent[i] = (uint32_t)i;
        if (w.type[i] != AXIOM_BODY_DYNAMIC) continue;
        const V3 v = w.vel[i], o = w.ang[i];
        const float l2 = (v.x * v.x + v.y * v.y) + v.z * v.z;
        const float a2 = (o.x * o.x + o.y * o.y) + o.z * o.z;
        const bool moving = w.noSleep[i] || l2 > lin2 || a2 > ang2;
        w.sleepTime[i] = moving ? 0.0f : w.sleepTime[i] + dt;
    }
    auto find = [&](uint32_t x) {
        while (parent[x] != x) x = parent[x] = parent[parent[x]];
        return x;
    };
    for (const Manifold& mf : w.manifolds) {
        if (!isDynamic(w, mf.a) || !isDynamic(w, mf.b)) continue;
        uint32_t ra = find(mf.a), rb = find(mf.b);
        if (ra == rb) continue;
        if (ra > rb) std::swap(ra, rb);
        parent[rb] = ra;  // the lower id stays the root
    }
    std::vector<float> minSleep(n, INFINITY);
    uint32_t islands = 0;
    for (size_t i = 0; i < n; ++i) {
        if (w.type[i] != AXIOM_BODY_DYNAMIC) continue;
        const uint32_t r = find((uint32_t)i);
        w.island[i] = r;
        minSleep[r] = std::min(minSleep[r], w.sleepTime[i]);
        islands += r == i ? 1u : 0u;
    }
    for (size_t i = 0; i < n; ++i) {
        if (w.type[i] != AXIOM_BODY_DYNAMIC || !(minSleep[w.island[i]] >= w.cfg.sleep_time_threshold)) continue;
        w.type[i] = kSleeping;
        w.vel[i] = V3{0.0f, 0.0f, 0.0f};
        w.ang[i] = V3{0.0f, 0.0f, 0.0f};
    }
    w.islandCount = islands;
}

uint32_t countSleeping(const OWorld& w) {
    uint32_t k = 0;
    for (uint32_t t : w.type) k += t == kSleeping ? 1u : 0u;
    return k;
}

double nowMs() {
    return std::chrono::duration<double, std::milli>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

}  // namespace

extern "C" {

AXIOM_API void axiom_world_config_default(axiom_world_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));  // every field not set below (e.g. temporal_colouring) is 0
    c->gravity[0] = 0.0f;
    c->gravity[1] = -9.81f;
    c->gravity[2] = 0.0f;
    c->time_step = 1.0f / 60.0f;
    c->velocity_iterations = 8;
    c->position_iterations = 3;
    c->residual_tolerance = 0.0f;
    c->max_iterations = 200;
    c->baumgarte = 0.2f;
    c->linear_slop = 0.005f;
    c->aabb_margin = 0.0f;
    c->restitution_threshold = 1.0f;
    c->warm_start = AXIOM_WARM_START_PREVIOUS;
    c->warm_start_factor = 1.0f;
    c->pair_capacity = 0;
    c->contact_capacity = 0;
    c->device = -1;
    c->allow_sleep = 0;
    c->sleep_linear_threshold = 0.01f;
    c->sleep_angular_threshold = 0.01f;
    c->sleep_time_threshold = 0.5f;
    c->speculative_contacts = 0;
}

AXIOM_API int32_t axiom_world_create(const axiom_world_config* config, void** world) {
    if (!config || !world) return AXIOM_NULL_POINTER;
    if (!(config->time_step > 0.0f) || config->temporal_colouring > 1u) return AXIOM_INVALID_PARAMETER;
    if (config->allow_sleep && !(config->sleep_time_threshold > 0.0f && config->sleep_linear_threshold >= 0.0f &&
                                 config->sleep_angular_threshold >= 0.0f))
        return AXIOM_INVALID_PARAMETER;
    OWorld* w = new (std::nothrow) OWorld();
    if (!w) return AXIOM_OUT_OF_MEMORY;
    w->cfg = *config;
    *world = w;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_destroy(void* world) {
    delete static_cast<OWorld*>(world);
    return AXIOM_SUCCESS;
}

// Body i is admissible: every number finite, the rotation of non-zero length, and mass,
// inertia, density, friction, restitution and damping not negative.
static bool admissibleNumbers(const axiom_body_soa* b, uint32_t i) {
    auto ok = [](const float* a, uint32_t k, bool nonneg) {
        for (uint32_t j = 0; j < k; ++j) {
            if (!std::isfinite(a[j])) return false;
            if (nonneg && a[j] < 0.0f) return false;
        }
        return true;
    };
    if (!ok(b->position + 3 * i, 3, false) || !ok(b->shape_extents + 3 * i, 3, false)) return false;
    if (b->rotation) {
        const float* q = b->rotation + 4 * i;
        if (!ok(q, 4, false) || !((q[0] * q[0] + q[1] * q[1]) + (q[2] * q[2] + q[3] * q[3]) > 0.0f)) return false;
    }
    if (b->linear_velocity && !ok(b->linear_velocity + 3 * i, 3, false)) return false;
    if (b->angular_velocity && !ok(b->angular_velocity + 3 * i, 3, false)) return false;
    const float* scalars[] = {b->mass, b->density, b->friction, b->restitution, b->linear_damping,
                              b->angular_damping, b->rolling_friction};
    for (const float* a : scalars)
        if (a && !ok(a + i, 1, true)) return false;
    if (b->inertia && !ok(b->inertia + 3 * i, 3, true)) return false;
    return true;
}

// The checks of axiom_world_add_bodies, without adding anything.
static int32_t checkBodies(const OWorld* w, const axiom_body_soa* b, uint32_t n) {
    if (!b->type || !b->shape || !b->position || !b->shape_extents) return AXIOM_NULL_POINTER;
    for (uint32_t i = 0; i < n; ++i) {
        if (b->type[i] > AXIOM_BODY_KINEMATIC || !admissibleNumbers(b, i)) return AXIOM_INVALID_RIGID_BODY;
        uint32_t s = b->shape[i];
        if (s != AXIOM_SHAPE_SPHERE && s != AXIOM_SHAPE_BOX && s != AXIOM_SHAPE_CAPSULE &&
            s != AXIOM_SHAPE_PLANE && s != AXIOM_SHAPE_CYLINDER && !isHull(s))
            return AXIOM_INVALID_SHAPE;
        if (s == AXIOM_SHAPE_MESH && b->type[i] == AXIOM_BODY_DYNAMIC) return AXIOM_INVALID_SHAPE;
        if (isHull(s)) {
            if (!b->convex_hull) return AXIOM_NULL_POINTER;
            if (b->convex_hull[i] >= w->hullPts.size()) return AXIOM_INVALID_SHAPE;
            continue;
        }
        if (s == AXIOM_SHAPE_CYLINDER && !(b->shape_extents[3 * i] > 0.0f && b->shape_extents[3 * i + 1] > 0.0f))
            return AXIOM_INVALID_SHAPE;
        if (s == AXIOM_SHAPE_PLANE && b->type[i] == AXIOM_BODY_DYNAMIC) return AXIOM_INVALID_SHAPE;
        const float* e = b->shape_extents + 3 * i;
        if (s == AXIOM_SHAPE_SPHERE && !(e[0] > 0.0f)) return AXIOM_INVALID_SHAPE;
        if (s == AXIOM_SHAPE_BOX && !(e[0] > 0.0f && e[1] > 0.0f && e[2] > 0.0f))
            return AXIOM_INVALID_SHAPE;
        if (s == AXIOM_SHAPE_CAPSULE && !(e[0] > 0.0f && e[1] >= 0.0f)) return AXIOM_INVALID_SHAPE;
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_check_bodies(void* world, const axiom_body_soa* b, uint32_t n) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || !b) return AXIOM_NULL_POINTER;
    if (n == 0) return AXIOM_SUCCESS;
    return checkBodies(w, b, n);
}

AXIOM_API int32_t axiom_world_add_bodies(void* world, const axiom_body_soa* b, uint32_t n,
                                         uint32_t* first_id) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || !b) return AXIOM_NULL_POINTER;
    if (n == 0) {
        if (first_id) *first_id = (uint32_t)w->type.size();
        return AXIOM_SUCCESS;
    }
    if (const int32_t st = checkBodies(w, b, n); st != AXIOM_SUCCESS) return st;
    if (first_id) *first_id = (uint32_t)w->type.size();
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t s = b->shape[i];
        V3 e{b->shape_extents[3 * i], b->shape_extents[3 * i + 1], b->shape_extents[3 * i + 2]};
        const uint32_t hid = isHull(s) ? b->convex_hull[i] : kNoHull;
        if (hid != kNoHull) e = V3{w->hullRadius[hid], 0.0f, 0.0f};
        w->hullId.push_back(hid);
        const bool sleepOn = w->cfg.allow_sleep != 0 && b->type[i] == AXIOM_BODY_DYNAMIC;
        const bool noSleep = sleepOn && b->allow_sleep && !b->allow_sleep[i];
        const bool asleep = sleepOn && !noSleep && b->is_sleeping && b->is_sleeping[i];
        w->type.push_back(asleep ? kSleeping : b->type[i]);
        w->noSleep.push_back(noSleep ? 1 : 0);
        w->sleepTime.push_back(0.0f);
        w->island.push_back(asleep ? (uint32_t)(w->type.size() - 1) : kNoIsland);
        w->shape.push_back(s);
        w->pos.push_back(V3{b->position[3 * i], b->position[3 * i + 1], b->position[3 * i + 2]});
        w->rot.push_back(b->rotation ? Q4{b->rotation[4 * i], b->rotation[4 * i + 1],
                                          b->rotation[4 * i + 2], b->rotation[4 * i + 3]}
                                     : Q4{0.0f, 0.0f, 0.0f, 1.0f});
        w->vel.push_back(b->linear_velocity
                             ? V3{b->linear_velocity[3 * i], b->linear_velocity[3 * i + 1],
                                  b->linear_velocity[3 * i + 2]}
                             : V3{0.0f, 0.0f, 0.0f});
        w->ang.push_back(b->angular_velocity
                             ? V3{b->angular_velocity[3 * i], b->angular_velocity[3 * i + 1],
                                  b->angular_velocity[3 * i + 2]}
                             : V3{0.0f, 0.0f, 0.0f});
        if (asleep) {  // added asleep: at rest
            w->vel.back() = V3{0.0f, 0.0f, 0.0f};
            w->ang.back() = V3{0.0f, 0.0f, 0.0f};
        }
        w->ext.push_back(e);
        float density = b->density ? b->density[i] : 1000.0f;
        float mass;
        V3 inertia;
        if (hid != kNoHull) massProperties(AXIOM_SHAPE_BOX, w->hullHalf[hid], density, &mass, &inertia);
        else massProperties(s, e, density, &mass, &inertia);
        if (b->mass) mass = b->mass[i];
        if (b->inertia) inertia = V3{b->inertia[3 * i], b->inertia[3 * i + 1], b->inertia[3 * i + 2]};
        bool dyn = b->type[i] == AXIOM_BODY_DYNAMIC && mass > 0.0f;
        w->invMass.push_back(dyn ? 1.0f / mass : 0.0f);
        V3 ii{0.0f, 0.0f, 0.0f};
        if (dyn) {
            ii.x = inertia.x > 0.0f ? 1.0f / inertia.x : 0.0f;
            ii.y = inertia.y > 0.0f ? 1.0f / inertia.y : 0.0f;
            ii.z = inertia.z > 0.0f ? 1.0f / inertia.z : 0.0f;
        }
        w->invInertia.push_back(ii);
        w->iso.push_back(ii.x == ii.y && ii.y == ii.z ? 1 : 0);
        w->friction.push_back(b->friction ? b->friction[i] : 0.5f);
        w->restitution.push_back(b->restitution ? b->restitution[i] : 0.5f);
        w->linDamp.push_back(b->linear_damping ? b->linear_damping[i] : 0.01f);
        w->angDamp.push_back(b->angular_damping ? b->angular_damping[i] : 0.05f);
        w->rollingFriction.push_back(b->rolling_friction ? b->rolling_friction[i] : 0.0f);
        w->filterCategory.push_back(b->filter_category ? b->filter_category[i] : 0x0001u);
        w->filterMask.push_back(b->filter_mask ? b->filter_mask[i] : 0xFFFFu);
        w->filterGroup.push_back(b->filter_group ? (int32_t)b->filter_group[i] : 0);
        w->boundRadius.push_back(boundingRadius(s, e));
    }
    size_t N = w->type.size();
    w->prevImpulse.clear();  // as the GPU world: adding bodies restarts the warm start
    w->pairs.clear();        // ... and forgets the last step's pairs and contacts
    w->manifolds.clear();
    w->warmValid = false;
    w->aabbMin.resize(N);
    w->aabbMax.resize(N);
    w->invIw.resize(N);
    w->sweep.resize(N);
    return AXIOM_SUCCESS;
}

static int32_t oracleAddHull(OWorld* w, const float* points, uint32_t count, uint32_t minCount, uint32_t* hull_id);

AXIOM_API int32_t axiom_world_add_convex_hull(void* world, const float* points, uint32_t count, uint32_t* hull_id) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || !points) return AXIOM_NULL_POINTER;
    return oracleAddHull(w, points, count, 4, hull_id);
}

// Static triangle mesh: each triangle a static body of shape MESH at its centroid
// ((v0 + v1 + v2) / 3, in that order) holding its three points about it.
AXIOM_API int32_t axiom_world_add_triangle_mesh(void* world, const float* v, uint32_t nv, const uint32_t* tri,
                                                uint32_t nt, float friction, float restitution, uint32_t* first_id) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    if (first_id) *first_id = (uint32_t)w->type.size();
    if (nt == 0) return AXIOM_SUCCESS;
    if (!v || !tri) return AXIOM_NULL_POINTER;
    std::vector<float> centre(3ull * nt), pts(9ull * nt);
    for (uint32_t t = 0; t < nt; ++t) {
        const uint32_t i0 = tri[3 * t], i1 = tri[3 * t + 1], i2 = tri[3 * t + 2];
        if (i0 >= nv || i1 >= nv || i2 >= nv) return AXIOM_OUT_OF_RANGE;
        const float* a = v + 3ull * i0;
        const float* b = v + 3ull * i1;
        const float* c = v + 3ull * i2;
        for (int k = 0; k < 3; ++k)
            if (!std::isfinite(a[k]) || !std::isfinite(b[k]) || !std::isfinite(c[k])) return AXIOM_INVALID_SHAPE;
        const V3 e1{b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2{c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        const V3 n = cross(e1, e2);
        if (!((n.x * n.x + n.y * n.y) + n.z * n.z > 0.0f)) return AXIOM_INVALID_SHAPE;
        for (int k = 0; k < 3; ++k) {
            const float ce = ((a[k] + b[k]) + c[k]) / 3.0f;
            centre[3 * t + k] = ce;
            pts[9 * t + k] = a[k] - ce;
            pts[9 * t + 3 + k] = b[k] - ce;
            pts[9 * t + 6 + k] = c[k] - ce;
        }
    }
    const uint32_t firstHull = (uint32_t)w->hullPts.size();
    for (uint32_t t = 0; t < nt; ++t) {
        const int32_t st = oracleAddHull(w, pts.data() + 9ull * t, 3, 3, nullptr);
        if (st != AXIOM_SUCCESS) return st;
    }
    std::vector<uint32_t> type(nt, AXIOM_BODY_STATIC), shape(nt, AXIOM_SHAPE_MESH), hull(nt);
    std::vector<float> ext(3ull * nt, 0.0f), fr(nt, friction), re(nt, restitution);
    for (uint32_t t = 0; t < nt; ++t) hull[t] = firstHull + t;
    axiom_body_soa soa{};
    soa.type = type.data();
    soa.shape = shape.data();
    soa.position = centre.data();
    soa.shape_extents = ext.data();
    soa.friction = fr.data();
    soa.restitution = re.data();
    soa.convex_hull = hull.data();
    return axiom_world_add_bodies(world, &soa, nt, first_id);
}

static int32_t oracleAddHull(OWorld* w, const float* points, uint32_t count, uint32_t minCount, uint32_t* hull_id) {
    if (count < minCount || count > AXIOM_CONVEX_MAX_VERTICES) return AXIOM_INVALID_SHAPE;
    std::vector<V3> pts(count);
    float mn[3] = {0.0f, 0.0f, 0.0f}, mx[3] = {0.0f, 0.0f, 0.0f}, r2 = 0.0f;
    for (uint32_t i = 0; i < count; ++i) {
        const float* v = points + 3 * i;
        if (!std::isfinite(v[0]) || !std::isfinite(v[1]) || !std::isfinite(v[2])) return AXIOM_INVALID_SHAPE;
        for (int k = 0; k < 3; ++k) {
            mn[k] = i == 0 || v[k] < mn[k] ? v[k] : mn[k];
            mx[k] = i == 0 || v[k] > mx[k] ? v[k] : mx[k];
        }
        const float d2 = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
        r2 = d2 > r2 ? d2 : r2;
        pts[i] = V3{v[0], v[1], v[2]};
    }
    const float radius = std::sqrt(r2);
    if (!(radius > 0.0f)) return AXIOM_INVALID_SHAPE;
    if (hull_id) *hull_id = (uint32_t)w->hullPts.size();
    w->hullPts.push_back(std::move(pts));
    w->hullRadius.push_back(radius);
    w->hullHalf.push_back(V3{0.5f * (mx[0] - mn[0]), 0.5f * (mx[1] - mn[1]), 0.5f * (mx[2] - mn[2])});
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_body_count(void* world, uint32_t* n) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || !n) return AXIOM_NULL_POINTER;
    *n = (uint32_t)w->type.size();
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_step(void* world, float dt, axiom_step_stats* stats) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    if (!(dt > 0.0f)) dt = w->cfg.time_step;
    double t0 = nowMs();
    integrateVelocities(*w, dt);
    computeAabbs(*w, dt);
    broadphase(*w);
    double t1 = nowMs();
    narrowphase(*w);
    for (int pass = 0; w->cfg.allow_sleep && pass < kMaxWakePasses; ++pass) {
        if (countSleeping(*w) == 0 || wakePass(*w, dt) == 0) break;
        broadphase(*w);  // contacts again with the woken bodies awake
        narrowphase(*w);
    }
    double t2 = nowMs();
    int32_t status = colourContacts(*w);
    const bool coloured = status == AXIOM_SUCCESS;  // the GPU world keeps no impulses otherwise
    uint32_t iters = 0;
    float residual = 0.0f;
    if (status == AXIOM_SUCCESS && !w->manifolds.empty()) {
        w->needFeatures = w->recording || w->cfg.warm_start == AXIOM_WARM_START_LEARNED;
        {
            const float* g = w->cfg.gravity;
            w->gdt = std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) * dt;
        }
        prepare(*w, dt);
        if (w->cfg.warm_start == AXIOM_WARM_START_LEARNED)
            warmStartLearned(*w);
        else
            warmStartFromPrevious(*w);
        size_t serialFrom = 0;
        auto batches = colourBatches(*w, &serialFrom);
        applyWarmStart(*w, batches, serialFrom);
        const bool tolMode = w->cfg.residual_tolerance > 0.0f;
        const uint32_t maxIt = tolMode ? w->cfg.max_iterations : w->cfg.velocity_iterations;
        for (uint32_t it = 0; it < maxIt; ++it) {
            float md, ml;
            solveSweep(*w, batches, serialFrom, &md, &ml);
            residual = md / maxf(ml, 1e-6f);
            ++iters;
            if (tolMode && residual <= w->cfg.residual_tolerance) break;
        }
        if (tolMode && residual > w->cfg.residual_tolerance)
            status = AXIOM_CONSTRAINT_SOLVER_FAILURE;
    }
    double t3 = nowMs();
    integratePositions(*w, dt);
    if (w->cfg.allow_sleep) islandsAndSleep(*w, dt);
    // remember impulses for the next step's warm start
    w->prevImpulse.clear();
    w->prevImpulse.reserve(w->manifolds.size() * 2);
    w->warmValid = true;
    uint32_t points = 0;
    for (size_t mi = 0; mi < w->manifolds.size(); ++mi) {
        const Manifold& mf = w->manifolds[mi];
        uint64_t key = pairKey(mf.a, mf.b);
        for (uint32_t p = 0; p < mf.count && coloured; ++p) {
            Imp3 l;
            l.v[0] = mf.pts[p].lambda[0];
            l.v[1] = mf.pts[p].lambda[1];
            l.v[2] = mf.pts[p].lambda[2];
            l.tag = p == 0 && w->colour[mi] != kCrowdColour ? w->colour[mi] + 1u : 0u;
            w->prevImpulse[key * 4u + p] = l;
        }
        points += mf.count;
    }
    double t4 = nowMs();
    // the step completes either way; the status names the first convergence failure met
    if (status == AXIOM_SUCCESS && w->gjkFailures) status = AXIOM_GJK_FAILED_TO_CONVERGE;
    if (status == AXIOM_SUCCESS && w->epaFailures) status = AXIOM_EPA_FAILED_TO_CONVERGE;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        for (uint32_t t : w->type) {
            stats->static_bodies += t == AXIOM_BODY_STATIC;
            stats->dynamic_bodies += t == AXIOM_BODY_DYNAMIC || t == kSleeping;
            stats->kinematic_bodies += t == AXIOM_BODY_KINEMATIC;
            stats->sleeping_bodies += t == kSleeping;
        }
        stats->total_bodies = (uint32_t)w->type.size();
        stats->active_bodies = stats->dynamic_bodies - stats->sleeping_bodies;
        stats->island_count = w->cfg.allow_sleep ? w->islandCount : 0u;
        stats->contact_point_count = points;
        stats->total_step_time = (float)(t4 - t0);
        stats->broadphase_time = (float)(t1 - t0);
        stats->narrowphase_time = (float)(t2 - t1);
        stats->solver_time = (float)(t3 - t2);
        stats->integration_time = (float)(t4 - t3);
        stats->pair_count = (uint32_t)(w->pairs.size() / 2);
        stats->manifold_count = (uint32_t)w->manifolds.size();
        stats->colour_count = w->colourCount;
        stats->colour_rounds = w->colourRounds;
        stats->iterations = iters;
        stats->residual = residual;
        stats->status = status;
        stats->gjk_failures = w->gjkFailures;
        stats->epa_failures = w->epaFailures;
    }
    return status;
}

AXIOM_API int32_t axiom_world_read_state(void* world, float* position, float* rotation,
                                         float* linear_velocity, float* angular_velocity) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    for (size_t i = 0; i < w->type.size(); ++i) {
        if (position) std::memcpy(position + 3 * i, &w->pos[i], 12);
        if (rotation) std::memcpy(rotation + 4 * i, &w->rot[i], 16);
        if (linear_velocity) std::memcpy(linear_velocity + 3 * i, &w->vel[i], 12);
        if (angular_velocity) std::memcpy(angular_velocity + 3 * i, &w->ang[i], 12);
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_write_state(void* world, const float* position, const float* rotation,
                                          const float* linear_velocity,
                                          const float* angular_velocity) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    for (size_t i = 0; i < w->type.size(); ++i) {
        if (position) std::memcpy(&w->pos[i], position + 3 * i, 12);
        if (rotation) std::memcpy(&w->rot[i], rotation + 4 * i, 16);
        if (linear_velocity) std::memcpy(&w->vel[i], linear_velocity + 3 * i, 12);
        if (angular_velocity) std::memcpy(&w->ang[i], angular_velocity + 3 * i, 12);
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_sleep(void* world, uint8_t* sleeping, float* sleep_time, uint32_t* island) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    for (size_t i = 0; i < w->type.size(); ++i) {
        const bool dyn = w->cfg.allow_sleep && (w->type[i] == AXIOM_BODY_DYNAMIC || w->type[i] == kSleeping);
        if (sleeping) sleeping[i] = w->type[i] == kSleeping ? 1 : 0;
        if (sleep_time) sleep_time[i] = dyn ? w->sleepTime[i] : 0.0f;
        if (island) island[i] = dyn ? w->island[i] : kNoIsland;
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_set_sleeping(void* world, const uint32_t* ids, uint32_t n, int32_t sleeping) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || (n && !ids)) return AXIOM_NULL_POINTER;
    for (uint32_t k = 0; k < n; ++k)
        if (ids[k] >= w->type.size()) return AXIOM_OUT_OF_RANGE;
    if (sleeping && !w->cfg.allow_sleep) return AXIOM_INVALID_PARAMETER;
    for (uint32_t k = 0; k < n && w->cfg.allow_sleep; ++k) {
        const uint32_t i = ids[k];
        if (!sleeping && w->type[i] == kSleeping) {
            w->type[i] = AXIOM_BODY_DYNAMIC;
            w->sleepTime[i] = 0.0f;
        } else if (sleeping && w->type[i] == AXIOM_BODY_DYNAMIC) {
            w->type[i] = kSleeping;
            w->vel[i] = V3{0.0f, 0.0f, 0.0f};
            w->ang[i] = V3{0.0f, 0.0f, 0.0f};
            w->sleepTime[i] = 0.0f;
            w->island[i] = i;
        }
    }
    return AXIOM_SUCCESS;
}

// ---- snapshot (same byte layout as the GPU library's, include/axiom_c.h) ----
static const char kSnapMagic[8] = {'A', 'X', 'S', 'N', 'A', 'P', '0', '1'};

static std::vector<axiom_snapshot_contact> oracleWarmEntries(const OWorld& w) {
    std::vector<axiom_snapshot_contact> v;
    if (!w.warmValid) return v;
    v.reserve(w.prevImpulse.size());
    for (const auto& kv : w.prevImpulse) {
        axiom_snapshot_contact c;
        c.body_lo = (uint32_t)(kv.first >> 34);  // key = ((lo << 32) | hi) * 4 + point
        c.body_hi = (uint32_t)((kv.first >> 2) & 0xFFFFFFFFull);
        c.point = (uint32_t)(kv.first & 3u) | ((kv.second.tag & 0xFFu) << 8);  // tag: 1 + colour on point 0
        std::memcpy(c.impulse, kv.second.v, 12);
        v.push_back(c);
    }
    std::sort(v.begin(), v.end(), [](const axiom_snapshot_contact& a, const axiom_snapshot_contact& b) {
        if (a.body_lo != b.body_lo) return a.body_lo < b.body_lo;
        if (a.body_hi != b.body_hi) return a.body_hi < b.body_hi;
        return (a.point & 0xFFu) < (b.point & 0xFFu);
    });
    return v;
}

static uint64_t oracleHullBytes(const OWorld& w) {
    uint64_t pts = 0;
    for (const auto& h : w.hullPts) pts += h.size();
    return 4ull * w.hullPts.size() + 12ull * pts;
}

AXIOM_API int32_t axiom_world_snapshot_size(void* world, uint64_t* bytes) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || !bytes) return AXIOM_NULL_POINTER;
    *bytes = sizeof(axiom_snapshot_header) + sizeof(axiom_snapshot_body) * (uint64_t)w->type.size() +
             sizeof(axiom_snapshot_contact) * (uint64_t)oracleWarmEntries(*w).size() + oracleHullBytes(*w);
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_save_snapshot(void* world, void* buffer, uint64_t capacity, uint64_t* written) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || !buffer || !written) return AXIOM_NULL_POINTER;
    const auto warm = oracleWarmEntries(*w);
    const uint64_t n = w->type.size();
    const uint64_t total = sizeof(axiom_snapshot_header) + sizeof(axiom_snapshot_body) * n +
                           sizeof(axiom_snapshot_contact) * warm.size() + oracleHullBytes(*w);
    *written = total;
    if (capacity < total) return AXIOM_OUT_OF_RANGE;
    axiom_snapshot_header h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kSnapMagic, 8);
    h.version = AXIOM_SNAPSHOT_VERSION;
    h.body_count = (uint32_t)n;
    h.contact_count = (uint32_t)warm.size();
    h.flags = w->warmValid ? 1u : 0u;
    h.hull_count = (uint32_t)w->hullPts.size();
    for (const auto& hp : w->hullPts) h.hull_vertex_count += (uint32_t)hp.size();
    h.total_bytes = total;
    h.config = w->cfg;
    unsigned char* out = static_cast<unsigned char*>(buffer);
    std::memcpy(out, &h, sizeof(h));
    for (uint64_t i = 0; i < n; ++i) {
        axiom_snapshot_body r;
        const bool asleep = w->type[i] == kSleeping;
        const bool dyn = w->type[i] == AXIOM_BODY_DYNAMIC || asleep;
        r.type = asleep ? (uint32_t)AXIOM_BODY_DYNAMIC : w->type[i];
        r.shape = w->shape[i];
        r.flags = (asleep ? 1u : 0u) | (w->noSleep[i] ? 2u : 0u);
        r.island = w->cfg.allow_sleep && dyn ? w->island[i] : kNoIsland;
        std::memcpy(r.position, &w->pos[i], 12);
        std::memcpy(r.rotation, &w->rot[i], 16);
        std::memcpy(r.linear_velocity, &w->vel[i], 12);
        std::memcpy(r.angular_velocity, &w->ang[i], 12);
        std::memcpy(r.shape_extents, &w->ext[i], 12);
        if (isHull(w->shape[i])) std::memcpy(&r.shape_extents[1], &w->hullId[i], 4);
        r.inv_mass = w->invMass[i];
        std::memcpy(r.inv_inertia, &w->invInertia[i], 12);
        r.friction = w->friction[i];
        r.restitution = w->restitution[i];
        r.linear_damping = w->linDamp[i];
        r.angular_damping = w->angDamp[i];
        r.filter_category = w->filterCategory[i];
        r.filter_mask = w->filterMask[i];
        r.filter_group = w->filterGroup[i];
        r.sleep_time = w->cfg.allow_sleep && dyn ? w->sleepTime[i] : 0.0f;
        r.rolling_friction = w->rollingFriction[i];
        r.reserved[0] = r.reserved[1] = r.reserved[2] = 0u;
        std::memcpy(out + sizeof(h) + sizeof(r) * i, &r, sizeof(r));
    }
    unsigned char* tail = out + sizeof(h) + sizeof(axiom_snapshot_body) * n;
    if (!warm.empty()) std::memcpy(tail, warm.data(), sizeof(axiom_snapshot_contact) * warm.size());
    tail += sizeof(axiom_snapshot_contact) * warm.size();
    for (const auto& hp : w->hullPts) {
        const uint32_t c = (uint32_t)hp.size();
        std::memcpy(tail, &c, 4);
        tail += 4;
    }
    for (const auto& hp : w->hullPts)
        for (const V3& v : hp) {
            std::memcpy(tail, &v, 12);
            tail += 12;
        }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_load_snapshot(void* world, const void* buffer, uint64_t size) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || !buffer) return AXIOM_NULL_POINTER;
    if (size < sizeof(axiom_snapshot_header)) return AXIOM_INVALID_PARAMETER;
    axiom_snapshot_header h;
    std::memcpy(&h, buffer, sizeof(h));
    if (std::memcmp(h.magic, kSnapMagic, 8) != 0 || h.version != AXIOM_SNAPSHOT_VERSION) return AXIOM_INVALID_PARAMETER;
    const uint64_t n = h.body_count, m = h.contact_count;
    const uint64_t total = sizeof(h) + sizeof(axiom_snapshot_body) * n + sizeof(axiom_snapshot_contact) * m +
                           4ull * h.hull_count + 12ull * h.hull_vertex_count;
    if (h.total_bytes != total || size < total || n >= (1ull << 30)) return AXIOM_INVALID_PARAMETER;
    axiom_world_config cfg = h.config;
    cfg.device = w->cfg.device;
    cfg.pair_capacity = w->cfg.pair_capacity;
    cfg.contact_capacity = w->cfg.contact_capacity;
    if (!(cfg.time_step > 0.0f) || cfg.warm_start > AXIOM_WARM_START_LEARNED || cfg.temporal_colouring > 1u)
        return AXIOM_INVALID_PARAMETER;
    if (cfg.allow_sleep && !(cfg.sleep_time_threshold > 0.0f && cfg.sleep_linear_threshold >= 0.0f &&
                             cfg.sleep_angular_threshold >= 0.0f))
        return AXIOM_INVALID_PARAMETER;
    const unsigned char* in = static_cast<const unsigned char*>(buffer);
    std::vector<axiom_snapshot_body> rec(n);
    if (n) std::memcpy(rec.data(), in + sizeof(h), sizeof(axiom_snapshot_body) * n);
    std::vector<axiom_snapshot_contact> warm(m);
    if (m) std::memcpy(warm.data(), in + sizeof(h) + sizeof(axiom_snapshot_body) * n, sizeof(axiom_snapshot_contact) * m);
    // hull section: vertex counts, then the points
    const unsigned char* hsec = in + sizeof(h) + sizeof(axiom_snapshot_body) * n + sizeof(axiom_snapshot_contact) * m;
    std::vector<std::vector<V3>> hulls(h.hull_count);
    {
        uint64_t used = 0;
        const unsigned char* pts = hsec + 4ull * h.hull_count;
        for (uint32_t k = 0; k < h.hull_count; ++k) {
            uint32_t c;
            std::memcpy(&c, hsec + 4ull * k, 4);
            if (c < 3 || c > AXIOM_CONVEX_MAX_VERTICES || used + c > h.hull_vertex_count) return AXIOM_INVALID_PARAMETER;
            hulls[k].resize(c);
            std::memcpy(hulls[k].data(), pts + 12ull * used, 12ull * c);
            used += c;
        }
        if (used != h.hull_vertex_count) return AXIOM_INVALID_PARAMETER;
    }
    for (const auto& r : rec) {
        const uint32_t s = r.shape;
        const float* e = r.shape_extents;
        bool ok = r.type <= AXIOM_BODY_KINEMATIC && r.rolling_friction >= 0.0f && std::isfinite(r.rolling_friction) &&
                  (s == AXIOM_SHAPE_SPHERE || s == AXIOM_SHAPE_BOX || s == AXIOM_SHAPE_CAPSULE || s == AXIOM_SHAPE_PLANE ||
                   s == AXIOM_SHAPE_CYLINDER || isHull(s)) &&
                  !(s == AXIOM_SHAPE_PLANE && r.type == AXIOM_BODY_DYNAMIC) && !((r.flags & 1u) && r.type != AXIOM_BODY_DYNAMIC);
        if (ok && s == AXIOM_SHAPE_SPHERE) ok = e[0] > 0.0f;
        if (ok && s == AXIOM_SHAPE_BOX) ok = e[0] > 0.0f && e[1] > 0.0f && e[2] > 0.0f;
        if (ok && s == AXIOM_SHAPE_CAPSULE) ok = e[0] > 0.0f && e[1] >= 0.0f;
        if (ok && s == AXIOM_SHAPE_CYLINDER) ok = e[0] > 0.0f && e[1] > 0.0f;
        if (ok && s == AXIOM_SHAPE_MESH) ok = r.type != AXIOM_BODY_DYNAMIC;
        if (ok && isHull(s)) {
            uint32_t id;
            std::memcpy(&id, &e[1], 4);
            ok = id < h.hull_count;
        }
        if (!ok) return AXIOM_INVALID_PARAMETER;
    }
    for (const auto& c : warm)
        if (c.body_lo >= n || c.body_hi >= n || (c.point & 0xFFu) >= 4u || (c.point >> 8) > 64u ||
            ((c.point & 0xFFu) != 0u && (c.point >> 8) != 0u))
            return AXIOM_INVALID_PARAMETER;
    OWorld fresh;
    fresh.cfg = cfg;
    for (auto& hp : hulls) {  // radius and half box exactly as axiom_world_add_convex_hull computes them
        float mn[3] = {0.0f, 0.0f, 0.0f}, mx[3] = {0.0f, 0.0f, 0.0f}, r2 = 0.0f;
        for (size_t i = 0; i < hp.size(); ++i) {
            const float v[3] = {hp[i].x, hp[i].y, hp[i].z};
            for (int k = 0; k < 3; ++k) {
                mn[k] = i == 0 || v[k] < mn[k] ? v[k] : mn[k];
                mx[k] = i == 0 || v[k] > mx[k] ? v[k] : mx[k];
            }
            const float d2 = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
            r2 = d2 > r2 ? d2 : r2;
        }
        fresh.hullRadius.push_back(std::sqrt(r2));
        fresh.hullHalf.push_back(V3{0.5f * (mx[0] - mn[0]), 0.5f * (mx[1] - mn[1]), 0.5f * (mx[2] - mn[2])});
        fresh.hullPts.push_back(std::move(hp));
    }
    fresh.threads = w->threads;
    fresh.mlp = w->mlp;
    fresh.recording = w->recording;
    const bool sleepOn = cfg.allow_sleep != 0;
    for (const auto& r : rec) {
        const bool asleep = sleepOn && (r.flags & 1u);
        fresh.type.push_back(asleep ? kSleeping : r.type);
        fresh.shape.push_back(r.shape);
        fresh.noSleep.push_back(sleepOn && (r.flags & 2u) && r.type == AXIOM_BODY_DYNAMIC ? 1 : 0);
        fresh.sleepTime.push_back(r.sleep_time);
        fresh.island.push_back(r.island);
        fresh.pos.push_back(V3{r.position[0], r.position[1], r.position[2]});
        fresh.rot.push_back(Q4{r.rotation[0], r.rotation[1], r.rotation[2], r.rotation[3]});
        fresh.vel.push_back(V3{r.linear_velocity[0], r.linear_velocity[1], r.linear_velocity[2]});
        fresh.ang.push_back(V3{r.angular_velocity[0], r.angular_velocity[1], r.angular_velocity[2]});
        V3 e{r.shape_extents[0], r.shape_extents[1], r.shape_extents[2]};
        uint32_t hid = kNoHull;
        if (isHull(r.shape)) {
            std::memcpy(&hid, &r.shape_extents[1], 4);
            e = V3{fresh.hullRadius[hid], 0.0f, 0.0f};
        }
        fresh.hullId.push_back(hid);
        fresh.ext.push_back(e);
        fresh.invMass.push_back(r.inv_mass);
        const V3 ii{r.inv_inertia[0], r.inv_inertia[1], r.inv_inertia[2]};
        fresh.invInertia.push_back(ii);
        fresh.iso.push_back(ii.x == ii.y && ii.y == ii.z ? 1 : 0);
        fresh.friction.push_back(r.friction);
        fresh.restitution.push_back(r.restitution);
        fresh.linDamp.push_back(r.linear_damping);
        fresh.angDamp.push_back(r.angular_damping);
        fresh.rollingFriction.push_back(r.rolling_friction);
        fresh.filterCategory.push_back(r.filter_category);
        fresh.filterMask.push_back(r.filter_mask);
        fresh.filterGroup.push_back(r.filter_group);
        fresh.boundRadius.push_back(boundingRadius(r.shape, e));
    }
    fresh.aabbMin.resize(n);
    fresh.aabbMax.resize(n);
    fresh.invIw.resize(n);
    fresh.sweep.resize(n);
    if (h.flags & 1u) {
        for (const auto& c : warm) {
            Imp3 l;
            std::memcpy(l.v, c.impulse, 12);
            l.tag = c.point >> 8;
            fresh.prevImpulse[pairKey(c.body_lo, c.body_hi) * 4u + (c.point & 0xFFu)] = l;
        }
        fresh.warmValid = true;
    }
    *w = std::move(fresh);
    return AXIOM_SUCCESS;
}

// ---- debug feed (debug::PhysicsDebugDraw records, physics_debug_draw.hpp:97-132) ----
AXIOM_API int32_t axiom_world_read_debug(void* world, uint32_t flags, axiom_debug_body* bodies, uint32_t body_capacity,
                                         axiom_debug_contact* contacts, uint32_t contact_capacity,
                                         uint32_t* body_count, uint32_t* contact_count) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    const uint32_t n = (uint32_t)w->type.size();
    uint32_t pts = 0;
    if (flags & AXIOM_DEBUG_CONTACTS)
        for (const Manifold& mf : w->manifolds) pts += mf.count;
    if (body_count) *body_count = n;
    if (contact_count) *contact_count = pts;
    for (uint32_t i = 0; bodies && i < n && i < body_capacity; ++i) {
        axiom_debug_body r;
        std::memset(&r, 0, sizeof(r));
        const uint32_t t = w->type[i];
        if (flags & AXIOM_DEBUG_SHAPES) {
            std::memcpy(r.position, &w->pos[i], 12);
            std::memcpy(r.rotation, &w->rot[i], 16);
            r.shape = w->shape[i];
            std::memcpy(r.shape_extents, &w->ext[i], 12);
        }
        if (flags & AXIOM_DEBUG_AABBS) {
            std::memcpy(r.aabb_min, &w->aabbMin[i], 12);
            std::memcpy(r.aabb_max, &w->aabbMax[i], 12);
        }
        if (flags & AXIOM_DEBUG_VELOCITIES) {
            std::memcpy(r.linear_velocity, &w->vel[i], 12);
            std::memcpy(r.angular_velocity, &w->ang[i], 12);
        }
        if (flags & AXIOM_DEBUG_ISLANDS) {
            r.is_awake = (t == AXIOM_BODY_DYNAMIC || t == AXIOM_BODY_KINEMATIC) ? 1u : 0u;
            r.island_index = w->cfg.allow_sleep && (t == AXIOM_BODY_DYNAMIC || t == kSleeping) ? w->island[i] : kNoIsland;
        }
        bodies[i] = r;
    }
    uint32_t q = 0;
    for (const Manifold& mf : w->manifolds) {
        if (!contacts || !(flags & AXIOM_DEBUG_CONTACTS)) break;
        for (uint32_t k = 0; k < mf.count && q < contact_capacity; ++k, ++q) {
            axiom_debug_contact& c = contacts[q];
            std::memcpy(c.position, &mf.pts[k].p, 12);
            std::memcpy(c.normal, &mf.pts[k].n, 12);
            c.penetration_depth = mf.pts[k].depth;
            c.body_a = mf.a;
            c.body_b = mf.b;
        }
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_aabbs(void* world, float* aabb_min, float* aabb_max) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    for (size_t i = 0; i < w->type.size(); ++i) {
        if (aabb_min) std::memcpy(aabb_min + 3 * i, &w->aabbMin[i], 12);
        if (aabb_max) std::memcpy(aabb_max + 3 * i, &w->aabbMax[i], 12);
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_pairs(void* world, uint32_t* pairs, uint32_t capacity,
                                         uint32_t* count) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || !count) return AXIOM_NULL_POINTER;
    uint32_t total = (uint32_t)(w->pairs.size() / 2);
    *count = total;
    if (pairs) std::memcpy(pairs, w->pairs.data(), 8ull * std::min(total, capacity));
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_contacts(void* world, axiom_contact_point* out, uint32_t capacity,
                                            uint32_t* count) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || !count) return AXIOM_NULL_POINTER;
    uint32_t k = 0;
    for (size_t m = 0; m < w->manifolds.size(); ++m) {
        const Manifold& mf = w->manifolds[m];
        for (uint32_t p = 0; p < mf.count; ++p, ++k) {
            if (!out || k >= capacity) continue;
            const ContactPoint& c = mf.pts[p];
            axiom_contact_point& o = out[k];
            o.body_a = mf.a;
            o.body_b = mf.b;
            std::memcpy(o.position, &c.p, 12);
            std::memcpy(o.normal, &c.n, 12);
            o.penetration_depth = c.depth;
            o.impulse[0] = c.lambda[0];
            o.impulse[1] = c.lambda[1];
            o.impulse[2] = c.lambda[2];
            o.colour = w->colour.empty() ? 0 : w->colour[m];
            o.point_index = p;
        }
    }
    *count = k;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_set_recording(void* world, int32_t enable) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    w->recording = enable != 0;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_read_samples(void* world, float* features, float* targets, uint32_t* keys,
                                           uint32_t capacity, uint32_t* count) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || !count) return AXIOM_NULL_POINTER;
    if (!w->needFeatures) {
        *count = 0;
        return AXIOM_SUCCESS;
    }
    uint32_t q = 0;
    for (const Manifold& mf : w->manifolds)
        for (uint32_t p = 0; p < mf.count; ++p, ++q) {
            if (q >= capacity) continue;
            const ContactPoint& c = mf.pts[p];
            const float inv = c.impScale > 0.0f ? 1.0f / c.impScale : 0.0f;
            if (features) std::memcpy(features + 14ull * q, c.feat, 14 * 4);
            if (targets) {  // correction from the previous-step impulse, in impulse units
                targets[3ull * q] = c.lambda[0] * inv - c.feat[9];
                targets[3ull * q + 1] = c.lambda[1] * inv - c.feat[10];
                targets[3ull * q + 2] = c.lambda[2] * inv - c.feat[11];
            }
            if (keys) {
                keys[3ull * q] = mf.a;
                keys[3ull * q + 1] = mf.b;
                keys[3ull * q + 2] = p;
            }
        }
    *count = q;
    return AXIOM_SUCCESS;
}

// Oracle-only: the network's forward pass and its mean-squared-error gradient (double,
// bf16 rounding where the GPU rounds), for the GPU kernels' gradient check.
AXIOM_API int32_t oracle_mlp_forward(const float* params, const float* features, uint32_t n, float* out) {
    MlpCache c;
    mlpForward(params, features, n, &c);
    for (size_t i = 0; i < (size_t)n * 3; ++i) out[i] = (float)c.y[i];
    return AXIOM_SUCCESS;
}

AXIOM_API void oracle_mlp_set_rounding(int32_t on) { mlpRounding() = on != 0; }

AXIOM_API int32_t oracle_mlp_gradients(const float* params, const float* features, const float* targets,
                                       uint32_t n, double* grads, double* loss) {
    double l = mlpGradients(params, features, targets, n, grads);
    if (loss) *loss = l;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_world_set_warm_start_model(void* world, const float* params, uint32_t count) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w || !params) return AXIOM_NULL_POINTER;
    if (count != AXIOM_MLP_PARAM_COUNT) return AXIOM_INVALID_PARAMETER;
    w->mlp.assign(params, params + count);
    return AXIOM_SUCCESS;
}

// The oracle keeps no per-kernel profile: it reports stage times in axiom_step_stats.
AXIOM_API int32_t axiom_world_set_profiling(void* world, int32_t) {
    return world ? AXIOM_SUCCESS : AXIOM_NULL_POINTER;
}
AXIOM_API int32_t axiom_world_set_profiling_groups(void* world, uint32_t) {
    return world ? AXIOM_SUCCESS : AXIOM_NULL_POINTER;
}

AXIOM_API int32_t axiom_world_reset_profile(void* world) {
    return world ? AXIOM_SUCCESS : AXIOM_NULL_POINTER;
}
AXIOM_API int32_t axiom_world_read_profile(void* world, axiom_kernel_profile*, uint32_t, uint32_t* count) {
    if (!world || !count) return AXIOM_NULL_POINTER;
    *count = 0;
    return AXIOM_SUCCESS;
}

AXIOM_API const char* axiom_version(void) { return "axiom-oracle 0.1"; }

// ---- Oracle-only math probes, checked against the reference's golden vectors ----
AXIOM_API int32_t oracle_aabb_intersects(const float* amin, const float* amax, const float* bmin,
                                         const float* bmax) {
    return amin[0] <= bmax[0] && amax[0] >= bmin[0] && amin[1] <= bmax[1] && amax[1] >= bmin[1] &&
           amin[2] <= bmax[2] && amax[2] >= bmin[2];
}
// AABB::fromCenterExtents then expand(margin) as the step computes a sphere/box AABB.
AXIOM_API void oracle_aabb_from_center(const float* c, const float* e, float margin, float* mn, float* mx) {
    V3 ee{e[0] + margin, e[1] + margin, e[2] + margin};
    V3 lo = sub(V3{c[0], c[1], c[2]}, ee), hi = add(V3{c[0], c[1], c[2]}, ee);
    std::memcpy(mn, &lo, 12);
    std::memcpy(mx, &hi, 12);
}
AXIOM_API void oracle_vec3_ops(const float* a, const float* b, float* dotOut, float* crossOut,
                               float* normalizedOut) {
    V3 va{a[0], a[1], a[2]}, vb{b[0], b[1], b[2]};
    *dotOut = dot(va, vb);
    V3 c = cross(va, vb), n = normalized(va);
    std::memcpy(crossOut, &c, 12);
    std::memcpy(normalizedOut, &n, 12);
}
AXIOM_API void oracle_quat_rotate(const float* q, const float* v, float* out) {
    V3 r = rotate(Q4{q[0], q[1], q[2], q[3]}, V3{v[0], v[1], v[2]});
    std::memcpy(out, &r, 12);
}
AXIOM_API void oracle_quat_mul(const float* a, const float* b, float* out) {
    Q4 r = qmul(Q4{a[0], a[1], a[2], a[3]}, Q4{b[0], b[1], b[2], b[3]});
    std::memcpy(out, &r, 16);
}
AXIOM_API void oracle_quat_normalize(const float* q, float* out) {
    Q4 r = qnormalize(Q4{q[0], q[1], q[2], q[3]});
    std::memcpy(out, &r, 16);
}
AXIOM_API void oracle_quat_from_axis_angle(const float* axis, float angle, float* out) {
    Q4 r = qfromAxisAngle(V3{axis[0], axis[1], axis[2]}, angle);
    std::memcpy(out, &r, 16);
}

// Oracle-only: narrowphase of one shape pair (normal first -> second).  shape/pos/rot/ext
// describe each body as in axiom_body_soa; a plane is the second shape only.  Writes up
// to 4 points (p: 3 floats each, depth) and the normal; returns the point count.
AXIOM_API int32_t oracle_collide_shapes(uint32_t shapeA, const float* posA, const float* rotA,
                                        const float* extA, uint32_t shapeB, const float* posB,
                                        const float* rotB, const float* extB, float* normal,
                                        float* points, float* depths) {
    BodyGeom ga{shapeA, V3{posA[0], posA[1], posA[2]}, Q4{rotA[0], rotA[1], rotA[2], rotA[3]},
                V3{extA[0], extA[1], extA[2]}};
    BodyGeom gb{shapeB, V3{posB[0], posB[1], posB[2]}, Q4{rotB[0], rotB[1], rotB[2], rotB[3]},
                V3{extB[0], extB[1], extB[2]}};
    Manifold mf;
    bool hit = shapeB == AXIOM_SHAPE_PLANE ? collidePlane(1, gb, 0, ga, &mf) : collide(0, ga, 1, gb, &mf);
    if (!hit) return 0;
    std::memcpy(normal, &mf.pts[0].n, 12);
    for (uint32_t k = 0; k < mf.count; ++k) {
        std::memcpy(points + 3 * k, &mf.pts[k].p, 12);
        depths[k] = mf.pts[k].depth;
    }
    return (int32_t)mf.count;
}

// Oracle-only: number of OpenMP threads used by the parallel-safe loops.  Results do not
// depend on it (every parallel loop writes disjoint outputs; colouring is sequential).
AXIOM_API int32_t oracle_set_threads(void* world, int32_t threads) {
    OWorld* w = static_cast<OWorld*>(world);
    if (!w) return AXIOM_NULL_POINTER;
    w->threads = threads < 1 ? 1 : threads;
    return AXIOM_SUCCESS;
}

}  // extern "C"
