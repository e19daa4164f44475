// world_api_main.cpp — drives the C++ world API of include/axiom_world.hpp over whichever
// library it is linked with (the CUDA library or the CPU oracle, which export the same C ABI).
//
// Scene: 4x4x4 spheres (mass from density), 8 boxes (explicit mass and inertia, tilted), 4
// capsules (mass from density) and a static ground plane, dropped for 60 steps at
// dt = 1/120 s with 10 sweeps and friction 0.5.  The program checks, and exits non-zero
// when a check fails:
//   1. the same scene added through raw axiom_world_* calls steps to bit-identical state
//      (the wrapper maps every field and mass/inertia run correctly);
//   2. saving a snapshot at step 30, finishing, loading it and re-running the last 30 steps
//      gives bit-identical state;
//   3. the header's and the library's error paths return failures with the engine's codes.
// Then it prints the final state as float bits, one body per line, for comparison between
// libraries.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "axiom_world.hpp"

using namespace axiom;
using dynamics::Float3;
using dynamics::PhysicsWorld;
using dynamics::RigidBodyDesc;

namespace {

constexpr float kDt = 1.0f / 120.0f;
constexpr int kSteps = 60;

std::vector<RigidBodyDesc> sceneBodies() {
    std::vector<RigidBodyDesc> b;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            for (int k = 0; k < 4; ++k) {
                RigidBodyDesc d;
                d.shapeType = dynamics::ShapeType::Sphere;
                d.shapeExtents = {0.5f, 0.0f, 0.0f};
                d.position = {1.05f * i + 0.01f * j, 0.6f + 1.05f * j, 1.05f * k - 0.013f * i};
                d.material.restitution = 0.0f;
                b.push_back(d);
            }
    for (int i = 0; i < 8; ++i) {
        RigidBodyDesc d;
        d.shapeType = dynamics::ShapeType::Box;
        d.shapeExtents = {0.4f, 0.3f, 0.5f};
        d.position = {6.0f + 1.3f * (i % 4), 0.8f + 1.2f * (i / 4), 1.5f};
        const float h = 0.15f * (i + 1), s = std::sin(h), c = std::cos(h);
        d.rotation = {0.0f, 0.0f, s, c};
        d.mass = 12.0f;
        d.inertiaTensor = Float3{0.61f, 0.82f, 0.66f};
        d.material.restitution = 0.0f;
        b.push_back(d);
    }
    for (int i = 0; i < 4; ++i) {
        RigidBodyDesc d;
        d.shapeType = dynamics::ShapeType::Capsule;
        d.shapeExtents = {0.2f, 0.4f, 0.0f};
        d.position = {-2.0f, 0.8f + 1.3f * i, 0.5f * i};
        d.linearVelocity = {0.3f, 0.0f, -0.2f};
        d.angularVelocity = {0.0f, 0.5f, 0.1f * i};
        d.material.restitution = 0.0f;
        b.push_back(d);
    }
    RigidBodyDesc plane;
    plane.type = dynamics::BodyType::Static;
    plane.shapeType = dynamics::ShapeType::Plane;
    plane.position = {0.0f, 0.0f, 0.0f};
    b.push_back(plane);
    return b;
}

dynamics::WorldConfig sceneConfig() {
    dynamics::WorldConfig c;
    c.timeStep = kDt;
    c.velocityIterations = 10;
    return c;
}

// The same scene through the raw C ABI, one add_bodies call per mass/inertia run.
std::vector<float> rawRun(const std::vector<RigidBodyDesc>& bodies) {
    axiom_world_config c;
    axiom_world_config_default(&c);
    c.time_step = kDt;
    c.velocity_iterations = 10;
    void* w = nullptr;
    if (axiom_world_create(&c, &w) != AXIOM_SUCCESS) return {};
    size_t begin = 0;
    while (begin < bodies.size()) {
        size_t end = begin;
        while (end < bodies.size() && bodies[end].shapeType == bodies[begin].shapeType) ++end;
        const size_t n = end - begin;
        std::vector<uint32_t> type(n), shape(n);
        std::vector<float> pos(3 * n), rot(4 * n), lin(3 * n), ang(3 * n), ext(3 * n), mass(n), inertia(3 * n),
            rest(n);
        for (size_t i = 0; i < n; ++i) {
            const RigidBodyDesc& d = bodies[begin + i];
            type[i] = static_cast<uint32_t>(d.type);
            shape[i] = static_cast<uint32_t>(d.shapeType);
            const float p[3] = {d.position.x, d.position.y, d.position.z};
            const float q[4] = {d.rotation.x, d.rotation.y, d.rotation.z, d.rotation.w};
            const float v[3] = {d.linearVelocity.x, d.linearVelocity.y, d.linearVelocity.z};
            const float o[3] = {d.angularVelocity.x, d.angularVelocity.y, d.angularVelocity.z};
            const float e[3] = {d.shapeExtents.x, d.shapeExtents.y, d.shapeExtents.z};
            std::memcpy(&pos[3 * i], p, sizeof p);
            std::memcpy(&rot[4 * i], q, sizeof q);
            std::memcpy(&lin[3 * i], v, sizeof v);
            std::memcpy(&ang[3 * i], o, sizeof o);
            std::memcpy(&ext[3 * i], e, sizeof e);
            if (d.mass) mass[i] = *d.mass;
            if (d.inertiaTensor) {
                inertia[3 * i] = d.inertiaTensor->x;
                inertia[3 * i + 1] = d.inertiaTensor->y;
                inertia[3 * i + 2] = d.inertiaTensor->z;
            }
            rest[i] = d.material.restitution;
        }
        axiom_body_soa soa{};
        soa.type = type.data();
        soa.shape = shape.data();
        soa.position = pos.data();
        soa.rotation = rot.data();
        soa.linear_velocity = lin.data();
        soa.angular_velocity = ang.data();
        soa.shape_extents = ext.data();
        soa.mass = bodies[begin].mass ? mass.data() : nullptr;
        soa.inertia = bodies[begin].inertiaTensor ? inertia.data() : nullptr;
        soa.restitution = rest.data();
        if (axiom_world_add_bodies(w, &soa, static_cast<uint32_t>(n), nullptr) != AXIOM_SUCCESS) return {};
        begin = end;
    }
    for (int s = 0; s < kSteps; ++s)
        if (axiom_world_step(w, kDt, nullptr) != AXIOM_SUCCESS) return {};
    uint32_t n = 0;
    axiom_world_body_count(w, &n);
    std::vector<float> out(13ull * n);
    axiom_world_read_state(w, out.data(), out.data() + 3ull * n, out.data() + 7ull * n, out.data() + 10ull * n);
    axiom_world_destroy(w);
    return out;
}

std::vector<float> flatten(const dynamics::BodyStates& st) {
    const size_t n = st.position.size();
    std::vector<float> out(13 * n);
    std::memcpy(out.data(), st.position.data(), 12 * n);
    std::memcpy(out.data() + 3 * n, st.rotation.data(), 16 * n);
    std::memcpy(out.data() + 7 * n, st.linearVelocity.data(), 12 * n);
    std::memcpy(out.data() + 10 * n, st.angularVelocity.data(), 12 * n);
    return out;
}

bool sameBits(const std::vector<float>& a, const std::vector<float>& b) {
    return a.size() == b.size() && std::memcmp(a.data(), b.data(), 4 * a.size()) == 0;
}

int fail(const char* what) {
    std::fprintf(stderr, "FAIL: %s\n", what);
    return 1;
}

}  // namespace

int main() {
    const std::vector<RigidBodyDesc> bodies = sceneBodies();
    auto created = PhysicsWorld::create(sceneConfig());
    if (created.isFailure()) return fail("create");
    PhysicsWorld& world = *created.value();

    auto first = world.createBodies(bodies.data(), bodies.size());
    if (first.isFailure() || first.value() != 0) return fail("createBodies");
    if (world.bodyCount() != bodies.size()) return fail("bodyCount");

    std::vector<uint8_t> snap;
    uint32_t contactsAt30 = 0;
    for (int s = 0; s < kSteps; ++s) {
        if (world.step(kDt).isFailure()) return fail("step");
        if (s == kSteps / 2 - 1) {
            auto blob = world.saveSnapshot();
            if (blob.isFailure()) return fail("saveSnapshot");
            snap = std::move(blob).value();
            contactsAt30 = world.stats().contactPointCount;
        }
    }
    const gui::PhysicsWorldStats last = world.stats();
    const axiom_step_stats info = world.stepInfo();
    auto state = world.readState();
    if (state.isFailure()) return fail("readState");
    const std::vector<float> finalState = flatten(state.value());

    auto pairs = world.pairs();
    auto contacts = world.contacts();
    if (pairs.isFailure() || contacts.isFailure()) return fail("pairs/contacts");
    if (contacts.value().size() != last.contactPointCount) return fail("contact count");
    for (const auto& p : pairs.value())
        if (p[0] >= p[1] || p[1] >= world.bodyCount()) return fail("pair order");

    // 1. the wrapper against the raw C ABI
    if (!sameBits(finalState, rawRun(bodies))) return fail("wrapper and raw C ABI differ");

    // 2. snapshot resume
    if (world.loadSnapshot(snap).isFailure()) return fail("loadSnapshot");
    for (int s = kSteps / 2; s < kSteps; ++s)
        if (world.step(kDt).isFailure()) return fail("step after load");
    auto resumed = world.readState();
    if (resumed.isFailure() || !sameBits(finalState, flatten(resumed.value()))) return fail("resume differs");

    // 3. error paths: a size mismatch caught by the header, an unknown shape by the library
    dynamics::BodyStates wrong = resumed.value();
    wrong.position.pop_back();
    auto w1 = world.writeState(wrong);
    if (w1.isSuccess() || w1.errorCode() != core::ErrorCode::InvalidParameter) return fail("writeState sizes");
    RigidBodyDesc bad;
    bad.shapeType = static_cast<dynamics::ShapeType>(99u);
    auto w2 = world.createBody(bad);
    if (w2.isSuccess()) return fail("unknown shape accepted");
    if (world.bodyCount() != bodies.size()) return fail("failed add changed the world");
    if (world.createBodies(nullptr, 1).errorCode() != core::ErrorCode::NullPointer) return fail("null descs");

    std::printf("bodies %u dynamic %u static %u\n", last.totalBodies, last.dynamicBodies, last.staticBodies);
    std::printf("contacts_step30 %u contacts %u pairs %u manifolds %u colours %u sweeps %u\n", contactsAt30,
                last.contactPointCount, info.pair_count, info.manifold_count, info.colour_count, info.iterations);
    std::printf("bad_shape_code %d\n", static_cast<int>(w2.errorCode()));
    const size_t n = bodies.size();
    for (size_t i = 0; i < n; ++i) {
        std::printf("%zu", i);
        for (size_t f = 0; f < 13; ++f) {
            const size_t base = f < 3 ? 0 : f < 7 ? 3 * n : f < 10 ? 7 * n : 10 * n;
            const size_t width = f < 3 ? 3 : f < 7 ? 4 : 3;
            const size_t off = f < 3 ? f : f < 7 ? f - 3 : f < 10 ? f - 7 : f - 10;
            uint32_t bits;
            std::memcpy(&bits, &finalState[base + width * i + off], 4);
            std::printf(" %08x", bits);
        }
        std::printf("\n");
    }
    return 0;
}
