// batch_api_main.cpp — drives PhysicsWorldBatch of include/axiom_world.hpp (CUDA library
// only: batched worlds have no CPU implementation).
//
// Six worlds of different sizes (a jittered sphere column, a row of tilted boxes, a capsule,
// each on its own ground plane) step 60 times at dt = 1/120 s in one batch.  Every world's
// final state must equal, bit for bit, that of a PhysicsWorld holding the same bodies, and
// its last-step manifold and colour counts must equal that world's.  Mixed mass presence in
// setWorlds must come back as InvalidParameter.  Exits non-zero when a check fails.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "axiom_world.hpp"

using namespace axiom;
using dynamics::PhysicsWorld;
using dynamics::PhysicsWorldBatch;
using dynamics::RigidBodyDesc;

namespace {

constexpr float kDt = 1.0f / 120.0f;
constexpr int kSteps = 60;

std::vector<RigidBodyDesc> worldBodies(int w) {
    std::vector<RigidBodyDesc> b;
    for (int i = 0; i < 3 + 4 * w; ++i) {
        RigidBodyDesc d;
        d.shapeType = dynamics::ShapeType::Sphere;
        d.shapeExtents = {0.3f + 0.02f * (i % 3), 0.0f, 0.0f};
        d.position = {0.013f * (i % 5) - 0.02f * w, 0.4f + 0.75f * i, 0.011f * (i % 7)};
        b.push_back(d);
    }
    for (int i = 0; i < 2 + w; ++i) {
        RigidBodyDesc d;
        d.shapeType = dynamics::ShapeType::Box;
        d.shapeExtents = {0.3f, 0.25f, 0.35f};
        const float h = 0.1f * (i + w), s = std::sin(h), c = std::cos(h);
        d.rotation = {s, 0.0f, 0.0f, c};
        d.position = {2.0f + 0.9f * i, 0.6f + 0.1f * w, 0.0f};
        d.material.friction = 0.6f;
        b.push_back(d);
    }
    RigidBodyDesc cap;
    cap.shapeType = dynamics::ShapeType::Capsule;
    cap.shapeExtents = {0.2f, 0.35f, 0.0f};
    cap.position = {-1.5f, 1.0f, 0.2f * w};
    cap.angularVelocity = {0.4f, 0.0f, 0.2f};
    b.push_back(cap);
    RigidBodyDesc plane;
    plane.type = dynamics::BodyType::Static;
    plane.shapeType = dynamics::ShapeType::Plane;
    b.push_back(plane);
    return b;
}

bool sameBits(const void* a, const void* b, size_t bytes) { return std::memcmp(a, b, bytes) == 0; }

int fail(const char* what, int w = -1) {
    std::fprintf(stderr, "FAIL: %s (world %d)\n", what, w);
    return 1;
}

}  // namespace

int main() {
    constexpr int kWorlds = 6;
    dynamics::WorldConfig config;
    config.timeStep = kDt;
    config.velocityIterations = 10;

    std::vector<std::vector<RigidBodyDesc>> worlds;
    for (int w = 0; w < kWorlds; ++w) worlds.push_back(worldBodies(w));

    auto created = PhysicsWorldBatch::create(config);
    if (created.isFailure()) return fail("batch create");
    PhysicsWorldBatch& batch = *created.value();
    if (batch.setWorlds(worlds).isFailure()) return fail("setWorlds");
    if (batch.worldCount() != kWorlds) return fail("worldCount");
    // bodies in shared memory for every world: the results must not change
    if (batch.setStage(4096).isFailure() || batch.launch()[2] != 4096) return fail("setStage");
    for (int s = 0; s < kSteps; ++s)
        if (batch.step(kDt).isFailure()) return fail("batch step");
    auto bstate = batch.readState();
    auto bstats = batch.worldStats();
    if (bstate.isFailure() || bstats.isFailure()) return fail("batch read");
    const auto& off = batch.worldOffsets();

    uint32_t manifolds = 0;
    for (int w = 0; w < kWorlds; ++w) {
        auto single = PhysicsWorld::create(config);
        if (single.isFailure()) return fail("world create", w);
        PhysicsWorld& world = *single.value();
        if (world.createBodies(worlds[w].data(), worlds[w].size()).isFailure()) return fail("createBodies", w);
        for (int s = 0; s < kSteps; ++s)
            if (world.step(kDt).isFailure()) return fail("world step", w);
        auto st = world.readState();
        if (st.isFailure()) return fail("world readState", w);
        const size_t n = worlds[w].size(), lo = off[w];
        if (off[w + 1] - lo != n) return fail("world offsets", w);
        const auto& b = bstate.value();
        const auto& o = st.value();
        if (!sameBits(&b.position[lo], o.position.data(), 12 * n) ||
            !sameBits(&b.rotation[lo], o.rotation.data(), 16 * n) ||
            !sameBits(&b.linearVelocity[lo], o.linearVelocity.data(), 12 * n) ||
            !sameBits(&b.angularVelocity[lo], o.angularVelocity.data(), 12 * n))
            return fail("batch state differs from single world", w);
        const dynamics::BatchWorldStats& ws = bstats.value()[w];
        if (ws.manifolds != world.stepInfo().manifold_count || ws.colours != world.stepInfo().colour_count)
            return fail("batch counts differ from single world", w);
        if (ws.flags != 0) return fail("batch overflow flags", w);
        manifolds += ws.manifolds;
    }
    if (manifolds == 0) return fail("no contacts in the batch");

    std::vector<std::vector<RigidBodyDesc>> mixed = {worldBodies(0), worldBodies(1)};
    mixed[1][0].mass = 3.0f;
    auto bad = batch.setWorlds(mixed);
    if (bad.isSuccess() || bad.errorCode() != core::ErrorCode::InvalidParameter) return fail("mixed mass accepted");

    std::printf("batch worlds %d bodies %u manifolds %u\n", kWorlds, off.back(), manifolds);
    return 0;
}
