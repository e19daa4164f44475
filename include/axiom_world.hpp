// axiom_world.hpp — C++20 world / body / shape / step API over the C ABI of axiom_c.h.
//
// The reference engine declares the step's C++ surface in its dynamics layer: a
// PhysicsWorld built from gui::PhysicsWorldConfig (include/axiom/gui/physics_panel.hpp:34-43),
// bodies with the fields of gui::RigidBodyData (include/axiom/gui/body_inspector.hpp:57-90),
// a fixed step(dt) (CLAUDE.md:160-177 sketch, examples/profiling_example.cpp:132-165) and
// per-step gui::PhysicsWorldStats (physics_panel.hpp:11-30), with exception-free
// core::Result<T> returns (include/axiom/core/result.hpp:16) carrying core::ErrorCode values
// (include/axiom/core/error_code.hpp:21-57).  This header gives that surface with the
// engine's conventions (camelCase methods, member_ fields) and forwards every call to the
// C ABI, so any library exporting axiom_c.h (the CUDA library, libaxiom_gb300.so) serves it.
//
// Inside the engine, define before including this header:
//   AXIOM_GB300_ENGINE_RESULT  Result and ErrorCode are the engine's own
//                              (axiom/core/result.hpp, axiom/core/error_code.hpp);
//   AXIOM_GB300_ENGINE_STATS   PhysicsWorldStats is the engine's own
//                              (axiom/gui/physics_panel.hpp, which pulls in the debug-draw
//                              and Vulkan headers);
//   AXIOM_GB300_ENGINE_TYPES   both.
// Standalone, the header defines minimal equivalents with the same names, numeric codes and
// member functions.
//
// Threading follows the C ABI: a world is used from one thread at a time; every call runs
// on the world's own CUDA stream and returns once its results are in host memory.
#ifndef AXIOM_WORLD_HPP
#define AXIOM_WORLD_HPP

#include <array>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <optional>
#include <utility>
#include <vector>

#include "axiom_c.h"

#if defined(AXIOM_GB300_ENGINE_TYPES) && !defined(AXIOM_GB300_ENGINE_RESULT)
#define AXIOM_GB300_ENGINE_RESULT
#endif
#if defined(AXIOM_GB300_ENGINE_TYPES) && !defined(AXIOM_GB300_ENGINE_STATS)
#define AXIOM_GB300_ENGINE_STATS
#endif

#ifdef AXIOM_GB300_ENGINE_RESULT
#include "axiom/core/result.hpp"
#else
namespace axiom::core {

// Numeric values of the engine's ErrorCode; the C ABI returns the same numbers.
enum class ErrorCode : int32_t {
    Success = AXIOM_SUCCESS,
    DivisionByZero = AXIOM_DIVISION_BY_ZERO,
    OutOfMemory = AXIOM_OUT_OF_MEMORY,
    InvalidAllocation = AXIOM_INVALID_ALLOCATION,
    NullPointer = AXIOM_NULL_POINTER,
    InvalidShape = AXIOM_INVALID_SHAPE,
    GJKFailedToConverge = AXIOM_GJK_FAILED_TO_CONVERGE,
    EPAFailedToConverge = AXIOM_EPA_FAILED_TO_CONVERGE,
    InvalidRigidBody = AXIOM_INVALID_RIGID_BODY,
    ConstraintSolverFailure = AXIOM_CONSTRAINT_SOLVER_FAILURE,
    GPU_INVALID_OPERATION = AXIOM_GPU_INVALID_OPERATION,
    GPU_TIMEOUT = AXIOM_GPU_TIMEOUT,
    GPU_OPERATION_FAILED = AXIOM_GPU_OPERATION_FAILED,
    InvalidParameter = AXIOM_INVALID_PARAMETER,
    OutOfRange = AXIOM_OUT_OF_RANGE,
};

// A value or an error code with a static message; no exceptions.
template <typename T>
class Result {
public:
    static Result success(T value) { return Result(std::move(value)); }
    static Result failure(ErrorCode code, const char* message = nullptr) { return Result(code, message); }
    bool isSuccess() const noexcept { return value_.has_value(); }
    bool isFailure() const noexcept { return !value_.has_value(); }
    T& value() & { return *value_; }
    const T& value() const& { return *value_; }
    T&& value() && { return std::move(*value_); }
    T valueOr(const T& fallback) const& { return value_ ? *value_ : fallback; }
    ErrorCode errorCode() const noexcept { return code_; }
    const char* errorMessage() const noexcept { return message_; }

private:
    explicit Result(T v) : value_(std::move(v)) {}
    Result(ErrorCode c, const char* m) : code_(c), message_(m) {}
    std::optional<T> value_;
    ErrorCode code_ = ErrorCode::Success;
    const char* message_ = nullptr;
};

template <>
class Result<void> {
public:
    static Result success() { return Result(ErrorCode::Success, nullptr); }
    static Result failure(ErrorCode code, const char* message = nullptr) { return Result(code, message); }
    bool isSuccess() const noexcept { return code_ == ErrorCode::Success; }
    bool isFailure() const noexcept { return code_ != ErrorCode::Success; }
    ErrorCode errorCode() const noexcept { return code_; }
    const char* errorMessage() const noexcept { return message_; }

private:
    Result(ErrorCode c, const char* m) : code_(c), message_(m) {}
    ErrorCode code_;
    const char* message_;
};

}  // namespace axiom::core
#endif

#ifdef AXIOM_GB300_ENGINE_STATS
#include "axiom/gui/physics_panel.hpp"
#else
namespace axiom::gui {

// Field names of the engine's PhysicsWorldStats (times in milliseconds).
struct PhysicsWorldStats {
    uint32_t totalBodies = 0, activeBodies = 0, sleepingBodies = 0;
    uint32_t staticBodies = 0, dynamicBodies = 0, kinematicBodies = 0;
    uint32_t contactPointCount = 0, constraintCount = 0, islandCount = 0;
    float totalStepTime = 0.0f, broadphaseTime = 0.0f, narrowphaseTime = 0.0f;
    float solverTime = 0.0f, integrationTime = 0.0f;
};

}  // namespace axiom::gui
#endif

namespace axiom::dynamics {

using BodyId = uint32_t;

struct Float3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
};
struct Quat4 {  // unit quaternion (x, y, z, w), the engine's math::Quat order
    float x = 0.0f, y = 0.0f, z = 0.0f, w = 1.0f;
};
// readStates / writeState pass vectors of these as packed float arrays ([3n] and [4n])
static_assert(sizeof(Float3) == 3 * sizeof(float) && alignof(Float3) == alignof(float), "Float3 is 3 packed floats");
static_assert(sizeof(Quat4) == 4 * sizeof(float) && alignof(Quat4) == alignof(float), "Quat4 is 4 packed floats");

// gui::BodyType and gui::ShapeType numbering, plus the static plane of debug::ShapeType.
enum class BodyType : uint32_t {
    Static = AXIOM_BODY_STATIC,
    Dynamic = AXIOM_BODY_DYNAMIC,
    Kinematic = AXIOM_BODY_KINEMATIC,
};
enum class ShapeType : uint32_t {
    Sphere = AXIOM_SHAPE_SPHERE,
    Box = AXIOM_SHAPE_BOX,
    Capsule = AXIOM_SHAPE_CAPSULE,
    Cylinder = AXIOM_SHAPE_CYLINDER,
    Mesh = AXIOM_SHAPE_MESH,
    Convex = AXIOM_SHAPE_CONVEX,
    Plane = AXIOM_SHAPE_PLANE,
};
enum class WarmStart : uint32_t {
    None = AXIOM_WARM_START_NONE,
    Previous = AXIOM_WARM_START_PREVIOUS,
    Learned = AXIOM_WARM_START_LEARNED,
};

// gui::PhysicsWorldConfig plus the solver controls of axiom_world_config.  allowSleep is
// off by default here, as in the C ABI, so that a step's cost does not depend on the
// scene's history unless the caller asks (the engine's panel default is on).
struct WorldConfig {
    Float3 gravity{0.0f, -9.81f, 0.0f};
    float timeStep = 1.0f / 60.0f;
    uint32_t velocityIterations = 8;
    uint32_t positionIterations = 3;
    bool allowSleep = false;
    float sleepLinearThreshold = 0.01f;
    float sleepAngularThreshold = 0.01f;
    float sleepTimeThreshold = 0.5f;
    float residualTolerance = 0.0f;  // > 0: sweep until the residual is reached
    uint32_t maxIterations = 200;
    WarmStart warmStart = WarmStart::Previous;
    bool speculativeContacts = false;
    bool temporalColouring = false;  // keep last step's colours where they stay proper
    int32_t device = -1;  // CUDA device ordinal; -1 = the current device
};

// gui::MaterialInfo and gui::FilterInfo with the engine's defaults.
struct MaterialInfo {
    float restitution = 0.5f;
    float friction = 0.5f;
    float rollingFriction = 0.0f;  // carried with the body; not applied by the solver yet
    float density = 1000.0f;
};
struct FilterInfo {
    uint32_t categoryBits = 0x0001;
    uint32_t maskBits = 0xFFFF;
    int16_t groupIndex = 0;
};

// One body: the fields of gui::RigidBodyData.  A mass or inertia left empty is derived
// from the material density and the shape; shapeExtents follows AXIOM_SHAPE_* in axiom_c.h.
struct RigidBodyDesc {
    BodyType type = BodyType::Dynamic;
    Float3 position;
    Quat4 rotation;
    Float3 linearVelocity;
    Float3 angularVelocity;
    std::optional<float> mass;
    std::optional<Float3> inertiaTensor;
    float linearDamping = 0.01f;
    float angularDamping = 0.05f;
    ShapeType shapeType = ShapeType::Box;
    Float3 shapeExtents{1.0f, 1.0f, 1.0f};
    MaterialInfo material;
    FilterInfo filter;
    bool allowSleep = true;
    bool isSleeping = false;
    uint32_t convexHull = 0;  // hull id from PhysicsWorld::addConvexHull (ShapeType::Convex)
};

// Body state of a whole world, by body id.
struct BodyStates {
    std::vector<Float3> position;
    std::vector<Quat4> rotation;
    std::vector<Float3> linearVelocity;
    std::vector<Float3> angularVelocity;
};

namespace detail {

// Host SoA copy of n body descriptions in the layout of axiom_body_soa; mass and inertia
// arrays only when the bodies give them (else the library derives them).
struct BodyPack {
    std::vector<uint32_t> type, shape, category, mask, hull;
    std::vector<float> pos, rot, lin, ang, ext, mass, inertia, friction, restitution, density, linDamp, angDamp,
        rolling;
    std::vector<int16_t> group;
    std::vector<uint8_t> allowSleep, sleeping;
    axiom_body_soa soa{};

    BodyPack(const RigidBodyDesc* d, size_t n, bool hasMass, bool hasInertia)
        : type(n), shape(n), category(n), mask(n), hull(n), pos(3 * n), rot(4 * n), lin(3 * n), ang(3 * n),
          ext(3 * n), mass(hasMass ? n : 0), inertia(hasInertia ? 3 * n : 0), friction(n), restitution(n),
          density(n), linDamp(n), angDamp(n), rolling(n), group(n), allowSleep(n), sleeping(n) {
        auto put3 = [](std::vector<float>& v, size_t i, const Float3& f) {
            v[3 * i] = f.x;
            v[3 * i + 1] = f.y;
            v[3 * i + 2] = f.z;
        };
        for (size_t i = 0; i < n; ++i) {
            const RigidBodyDesc& b = d[i];
            type[i] = static_cast<uint32_t>(b.type);
            shape[i] = static_cast<uint32_t>(b.shapeType);
            put3(pos, i, b.position);
            rot[4 * i] = b.rotation.x;
            rot[4 * i + 1] = b.rotation.y;
            rot[4 * i + 2] = b.rotation.z;
            rot[4 * i + 3] = b.rotation.w;
            put3(lin, i, b.linearVelocity);
            put3(ang, i, b.angularVelocity);
            put3(ext, i, b.shapeExtents);
            if (hasMass) mass[i] = *b.mass;
            if (hasInertia) put3(inertia, i, *b.inertiaTensor);
            friction[i] = b.material.friction;
            restitution[i] = b.material.restitution;
            rolling[i] = b.material.rollingFriction;
            density[i] = b.material.density;
            linDamp[i] = b.linearDamping;
            angDamp[i] = b.angularDamping;
            category[i] = b.filter.categoryBits;
            mask[i] = b.filter.maskBits;
            group[i] = b.filter.groupIndex;
            allowSleep[i] = b.allowSleep ? 1u : 0u;
            sleeping[i] = b.isSleeping ? 1u : 0u;
            hull[i] = b.convexHull;
        }
        soa.type = type.data();
        soa.shape = shape.data();
        soa.position = pos.data();
        soa.rotation = rot.data();
        soa.linear_velocity = lin.data();
        soa.angular_velocity = ang.data();
        soa.shape_extents = ext.data();
        soa.mass = hasMass ? mass.data() : nullptr;
        soa.inertia = hasInertia ? inertia.data() : nullptr;
        soa.friction = friction.data();
        soa.restitution = restitution.data();
        soa.density = density.data();
        soa.linear_damping = linDamp.data();
        soa.angular_damping = angDamp.data();
        soa.filter_category = category.data();
        soa.filter_mask = mask.data();
        soa.filter_group = group.data();
        soa.allow_sleep = allowSleep.data();
        soa.is_sleeping = sleeping.data();
        soa.convex_hull = hull.data();
        soa.rolling_friction = rolling.data();
    }
    BodyPack(const BodyPack&) = delete;
    BodyPack& operator=(const BodyPack&) = delete;
};

// axiom_world_config from the C++ configuration (library defaults for the rest).
inline axiom_world_config toC(const WorldConfig& config) {
    axiom_world_config c;
    axiom_world_config_default(&c);
    c.gravity[0] = config.gravity.x;
    c.gravity[1] = config.gravity.y;
    c.gravity[2] = config.gravity.z;
    c.time_step = config.timeStep;
    c.velocity_iterations = config.velocityIterations;
    c.position_iterations = config.positionIterations;
    c.allow_sleep = config.allowSleep ? 1u : 0u;
    c.sleep_linear_threshold = config.sleepLinearThreshold;
    c.sleep_angular_threshold = config.sleepAngularThreshold;
    c.sleep_time_threshold = config.sleepTimeThreshold;
    c.residual_tolerance = config.residualTolerance;
    c.max_iterations = config.maxIterations;
    c.warm_start = static_cast<uint32_t>(config.warmStart);
    c.speculative_contacts = config.speculativeContacts ? 1u : 0u;
    c.temporal_colouring = config.temporalColouring ? 1u : 0u;
    c.device = config.device;
    return c;
}

inline core::ErrorCode code(int32_t s) { return static_cast<core::ErrorCode>(s); }

// Engine stats record from the step's counters.
inline void fillStats(const axiom_step_stats& in, gui::PhysicsWorldStats& out) {
    out.totalBodies = in.total_bodies;
    out.activeBodies = in.active_bodies;
    out.sleepingBodies = in.sleeping_bodies;
    out.staticBodies = in.static_bodies;
    out.dynamicBodies = in.dynamic_bodies;
    out.kinematicBodies = in.kinematic_bodies;
    out.contactPointCount = in.contact_point_count;
    out.constraintCount = in.constraint_count;
    out.islandCount = in.island_count;
    out.totalStepTime = in.total_step_time;
    out.broadphaseTime = in.broadphase_time;
    out.narrowphaseTime = in.narrowphase_time;
    out.solverTime = in.solver_time;
    out.integrationTime = in.integration_time;
}

// Reads n bodies' state through one of the read_state entry points.
template <typename ReadFn>
core::Result<BodyStates> readStates(size_t n, ReadFn read) {
    BodyStates st;
    st.position.resize(n);
    st.rotation.resize(n);
    st.linearVelocity.resize(n);
    st.angularVelocity.resize(n);
    if (n == 0) return core::Result<BodyStates>::success(std::move(st));
    const int32_t s = read(&st.position[0].x, &st.rotation[0].x, &st.linearVelocity[0].x, &st.angularVelocity[0].x);
    if (s != AXIOM_SUCCESS) return core::Result<BodyStates>::failure(code(s), "read_state");
    return core::Result<BodyStates>::success(std::move(st));
}

}  // namespace detail

class PhysicsWorld {
public:
    using Ptr = std::unique_ptr<PhysicsWorld>;

    static core::Result<Ptr> create(const WorldConfig& config = WorldConfig{}) {
        const axiom_world_config c = detail::toC(config);
        void* h = nullptr;
        if (const int32_t s = axiom_world_create(&c, &h); s != AXIOM_SUCCESS)
            return core::Result<Ptr>::failure(code(s), "axiom_world_create");
        return core::Result<Ptr>::success(Ptr(new PhysicsWorld(h)));
    }

    PhysicsWorld(const PhysicsWorld&) = delete;
    PhysicsWorld& operator=(const PhysicsWorld&) = delete;
    ~PhysicsWorld() { axiom_world_destroy(world_); }

    // Adds one body; returns its id.
    core::Result<BodyId> createBody(const RigidBodyDesc& desc) { return createBodies(&desc, 1); }

    // Adds count bodies with consecutive ids; returns the first id.  Bodies are uploaded in
    // runs that agree on whether mass and inertia are given (a run whose bodies leave them
    // empty lets the library derive them).  Every run is checked before the first upload,
    // so an invalid description adds no body; only a device failure during the uploads
    // (GPU_OPERATION_FAILED, OutOfMemory) can leave the runs before it added, which
    // bodyCount() then shows.
    core::Result<BodyId> createBodies(const RigidBodyDesc* descs, size_t count) {
        if (!descs && count) return core::Result<BodyId>::failure(core::ErrorCode::NullPointer, "createBodies");
        uint32_t first = 0;
        if (const int32_t s = axiom_world_body_count(world_, &first); s != AXIOM_SUCCESS)
            return core::Result<BodyId>::failure(code(s), "axiom_world_body_count");
        std::vector<std::unique_ptr<detail::BodyPack>> runs;
        std::vector<size_t> sizes;
        size_t begin = 0;
        while (begin < count) {
            const bool hasMass = descs[begin].mass.has_value();
            const bool hasInertia = descs[begin].inertiaTensor.has_value();
            size_t end = begin + 1;
            while (end < count && descs[end].mass.has_value() == hasMass &&
                   descs[end].inertiaTensor.has_value() == hasInertia)
                ++end;
            runs.push_back(std::make_unique<detail::BodyPack>(descs + begin, end - begin, hasMass, hasInertia));
            sizes.push_back(end - begin);
            const int32_t s = axiom_world_check_bodies(world_, &runs.back()->soa, static_cast<uint32_t>(end - begin));
            if (s != AXIOM_SUCCESS) return core::Result<BodyId>::failure(code(s), "createBodies: invalid body");
            begin = end;
        }
        for (size_t r = 0; r < runs.size(); ++r) {
            const int32_t s = axiom_world_add_bodies(world_, &runs[r]->soa, static_cast<uint32_t>(sizes[r]), nullptr);
            if (s != AXIOM_SUCCESS) return core::Result<BodyId>::failure(code(s), "axiom_world_add_bodies");
        }
        return core::Result<BodyId>::success(first);
    }

    // Convex hull for ShapeType::Convex bodies (4..AXIOM_CONVEX_MAX_VERTICES body-frame points).
    core::Result<uint32_t> addConvexHull(const std::vector<Float3>& points) {
        uint32_t id = 0;
        const int32_t s = axiom_world_add_convex_hull(world_, points.empty() ? nullptr : &points[0].x,
                                                      static_cast<uint32_t>(points.size()), &id);
        if (s != AXIOM_SUCCESS) return core::Result<uint32_t>::failure(code(s), "axiom_world_add_convex_hull");
        return core::Result<uint32_t>::success(id);
    }

    // One step: broadphase, narrowphase, coloured PGS, integration.  dt <= 0 uses timeStep.
    // GJKFailedToConverge / EPAFailedToConverge come back after a completed step (some
    // pair's contact is approximate; stepInfo() counts them), with the stats filled.
    core::Result<void> step(float dt = 0.0f) {
        const int32_t s = axiom_world_step(world_, dt, &info_);
        if (s == AXIOM_SUCCESS || s == AXIOM_GJK_FAILED_TO_CONVERGE || s == AXIOM_EPA_FAILED_TO_CONVERGE)
            detail::fillStats(info_, stats_);
        if (s != AXIOM_SUCCESS) return core::Result<void>::failure(code(s), "axiom_world_step");
        return core::Result<void>::success();
    }

    // Statistics of the last step, in the engine's record.
    const gui::PhysicsWorldStats& stats() const { return stats_; }
    // The step's own counters (pairs, manifolds, colours, sweeps, residual).
    const axiom_step_stats& stepInfo() const { return info_; }

    uint32_t bodyCount() const {
        uint32_t n = 0;
        axiom_world_body_count(world_, &n);
        return n;
    }

    core::Result<BodyStates> readState() const {
        return detail::readStates(bodyCount(), [this](float* p, float* r, float* l, float* a) {
            return axiom_world_read_state(world_, p, r, l, a);
        });
    }

    // Overwrites every body's pose and velocities (sizes must equal bodyCount()).
    core::Result<void> writeState(const BodyStates& st) {
        const size_t n = bodyCount();
        if (st.position.size() != n || st.rotation.size() != n || st.linearVelocity.size() != n ||
            st.angularVelocity.size() != n)
            return core::Result<void>::failure(core::ErrorCode::InvalidParameter, "writeState: sizes");
        if (n == 0) return core::Result<void>::success();
        const int32_t s = axiom_world_write_state(world_, &st.position[0].x, &st.rotation[0].x,
                                                  &st.linearVelocity[0].x, &st.angularVelocity[0].x);
        if (s != AXIOM_SUCCESS) return core::Result<void>::failure(code(s), "axiom_world_write_state");
        return core::Result<void>::success();
    }

    // Broadphase pairs of the last step, (a, b) with a < b, in no particular order.
    core::Result<std::vector<std::array<uint32_t, 2>>> pairs() const {
        using V = std::vector<std::array<uint32_t, 2>>;
        uint32_t total = 0;
        if (const int32_t s = axiom_world_read_pairs(world_, nullptr, 0, &total); s != AXIOM_SUCCESS)
            return core::Result<V>::failure(code(s), "axiom_world_read_pairs");
        V out(total);
        if (total) {
            const int32_t s = axiom_world_read_pairs(world_, out[0].data(), total, &total);
            if (s != AXIOM_SUCCESS) return core::Result<V>::failure(code(s), "axiom_world_read_pairs");
        }
        return core::Result<V>::success(std::move(out));
    }

    // Contact points of the last step with their impulses and colours, in no particular order.
    core::Result<std::vector<axiom_contact_point>> contacts() const {
        using V = std::vector<axiom_contact_point>;
        uint32_t total = 0;
        if (const int32_t s = axiom_world_read_contacts(world_, nullptr, 0, &total); s != AXIOM_SUCCESS)
            return core::Result<V>::failure(code(s), "axiom_world_read_contacts");
        V out(total);
        if (total) {
            const int32_t s = axiom_world_read_contacts(world_, out.data(), total, &total);
            if (s != AXIOM_SUCCESS) return core::Result<V>::failure(code(s), "axiom_world_read_contacts");
        }
        return core::Result<V>::success(std::move(out));
    }

    // Checkpoint / resume through the snapshot blob of axiom_c.h (the same bytes on every
    // library that exports the ABI).
    core::Result<std::vector<uint8_t>> saveSnapshot() const {
        using V = std::vector<uint8_t>;
        uint64_t size = 0, written = 0;
        if (const int32_t s = axiom_world_snapshot_size(world_, &size); s != AXIOM_SUCCESS)
            return core::Result<V>::failure(code(s), "axiom_world_snapshot_size");
        V blob(size);
        if (const int32_t s = axiom_world_save_snapshot(world_, blob.data(), size, &written); s != AXIOM_SUCCESS)
            return core::Result<V>::failure(code(s), "axiom_world_save_snapshot");
        blob.resize(written);
        return core::Result<V>::success(std::move(blob));
    }
    core::Result<void> loadSnapshot(const std::vector<uint8_t>& blob) {
        const int32_t s = axiom_world_load_snapshot(world_, blob.data(), blob.size());
        if (s != AXIOM_SUCCESS) return core::Result<void>::failure(code(s), "axiom_world_load_snapshot");
        return core::Result<void>::success();
    }

    // The C handle, for the axiom_world_* calls this class does not wrap.
    void* handle() const { return world_; }

private:
    explicit PhysicsWorld(void* h) : world_(h) {}

    static core::ErrorCode code(int32_t s) { return detail::code(s); }

    void* world_;
    gui::PhysicsWorldStats stats_{};
    axiom_step_stats info_{};
};


// Per-world counters of the last batched step (axiom_batch_read_world_stats).
struct BatchWorldStats {
    uint32_t pairs = 0, manifolds = 0, points = 0, colours = 0, colourRounds = 0, iterations = 0;
    uint32_t flags = 0;  // 1 pairs / 2 manifolds / 4 planes / 8 colours / 16 rounds overflow, 32 residual not reached
    uint32_t gjkPairs = 0;
    uint64_t stepNs = 0;  // device time of this world's step
    float residual = 0.0f;
};

// Thousands of independent worlds stepped together in one persistent launch (the batched
// form of PhysicsWorld::step; the reference has no batching).  Each world steps exactly as
// a PhysicsWorld holding the same bodies would.  Limits are the C ABI's: at most 8192
// bodies and 8 planes per world, warm start None or Previous, no sleeping.
class PhysicsWorldBatch {
public:
    using Ptr = std::unique_ptr<PhysicsWorldBatch>;

    static core::Result<Ptr> create(const WorldConfig& config = WorldConfig{}) {
        const axiom_world_config c = detail::toC(config);
        void* h = nullptr;
        if (const int32_t s = axiom_batch_create(&c, &h); s != AXIOM_SUCCESS)
            return core::Result<Ptr>::failure(detail::code(s), "axiom_batch_create");
        return core::Result<Ptr>::success(Ptr(new PhysicsWorldBatch(h)));
    }

    PhysicsWorldBatch(const PhysicsWorldBatch&) = delete;
    PhysicsWorldBatch& operator=(const PhysicsWorldBatch&) = delete;
    ~PhysicsWorldBatch() { axiom_batch_destroy(batch_); }

    // Replaces every world: world w holds worlds[w], with world-local body ids.  Mass and
    // inertia are given for every body of the batch or for none (one upload).
    core::Result<void> setWorlds(const std::vector<std::vector<RigidBodyDesc>>& worlds) {
        std::vector<RigidBodyDesc> all;
        std::vector<uint32_t> sizes;
        sizes.reserve(worlds.size());
        for (const auto& w : worlds) {
            sizes.push_back(static_cast<uint32_t>(w.size()));
            all.insert(all.end(), w.begin(), w.end());
        }
        if (all.empty()) return core::Result<void>::failure(core::ErrorCode::InvalidParameter, "setWorlds: no bodies");
        const bool hasMass = all[0].mass.has_value(), hasInertia = all[0].inertiaTensor.has_value();
        for (const RigidBodyDesc& d : all)
            if (d.mass.has_value() != hasMass || d.inertiaTensor.has_value() != hasInertia)
                return core::Result<void>::failure(core::ErrorCode::InvalidParameter,
                                                   "setWorlds: mass/inertia given for some bodies only");
        const detail::BodyPack pack(all.data(), all.size(), hasMass, hasInertia);
        const int32_t s =
            axiom_batch_set_worlds(batch_, &pack.soa, sizes.data(), static_cast<uint32_t>(sizes.size()));
        if (s != AXIOM_SUCCESS) return core::Result<void>::failure(detail::code(s), "axiom_batch_set_worlds");
        offsets_.assign(1, 0u);
        for (uint32_t n : sizes) offsets_.push_back(offsets_.back() + n);
        return core::Result<void>::success();
    }

    // One step of every world; dt <= 0 uses timeStep.  stats() then sums over the worlds
    // and totalStepTime is the device time of the whole batch.
    core::Result<void> step(float dt = 0.0f) {
        const int32_t s = axiom_batch_step(batch_, dt, &info_);
        if (s == AXIOM_SUCCESS || s == AXIOM_GJK_FAILED_TO_CONVERGE || s == AXIOM_EPA_FAILED_TO_CONVERGE)
            detail::fillStats(info_, stats_);
        if (s != AXIOM_SUCCESS) return core::Result<void>::failure(detail::code(s), "axiom_batch_step");
        return core::Result<void>::success();
    }

    const gui::PhysicsWorldStats& stats() const { return stats_; }
    const axiom_step_stats& stepInfo() const { return info_; }
    uint32_t worldCount() const { return offsets_.empty() ? 0u : static_cast<uint32_t>(offsets_.size() - 1); }
    // Body range of world w in readState(): [worldOffsets()[w], worldOffsets()[w + 1]).
    const std::vector<uint32_t>& worldOffsets() const { return offsets_; }

    core::Result<std::vector<BatchWorldStats>> worldStats() const {
        using V = std::vector<BatchWorldStats>;
        const uint32_t n = worldCount();
        std::vector<uint32_t> counts(8ull * n);
        std::vector<uint64_t> ns(n);
        std::vector<float> res(n);
        if (n) {
            const int32_t s = axiom_batch_read_world_stats(batch_, counts.data(), ns.data(), res.data());
            if (s != AXIOM_SUCCESS) return core::Result<V>::failure(detail::code(s), "axiom_batch_read_world_stats");
        }
        V out(n);
        for (uint32_t w = 0; w < n; ++w) {
            const uint32_t* c = &counts[8ull * w];
            out[w] = BatchWorldStats{c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], ns[w], res[w]};
        }
        return core::Result<V>::success(std::move(out));
    }

    // State of every body, world after world.
    core::Result<BodyStates> readState() const {
        const size_t n = offsets_.empty() ? 0 : offsets_.back();
        return detail::readStates(n, [this](float* p, float* r, float* l, float* a) {
            return axiom_batch_read_state(batch_, p, r, l, a);
        });
    }

    // Picks the fastest launch shape over trialSteps steps (state restored afterwards);
    // cachePath (may be null) stores and reuses the choice.  Returns {block, ctasPerSm}.
    core::Result<std::array<uint32_t, 2>> autotune(const char* cachePath = nullptr, uint32_t trialSteps = 3) {
        std::array<uint32_t, 2> shape{0, 0};
        if (const int32_t s = axiom_batch_autotune(batch_, cachePath, trialSteps, &shape[0], &shape[1]);
            s != AXIOM_SUCCESS)
            return core::Result<std::array<uint32_t, 2>>::failure(detail::code(s), "axiom_batch_autotune");
        return core::Result<std::array<uint32_t, 2>>::success(shape);
    }

    // Worlds of at most stageBodies bodies solve with their bodies in shared memory.
    core::Result<void> setStage(uint32_t stageBodies) {
        if (const int32_t s = axiom_batch_set_stage(batch_, stageBodies); s != AXIOM_SUCCESS)
            return core::Result<void>::failure(detail::code(s), "axiom_batch_set_stage");
        return core::Result<void>::success();
    }

    // {threads per world, CTAs per SM, staged bodies} of the persistent kernel.
    std::array<uint32_t, 3> launch() const {
        std::array<uint32_t, 3> l{0, 0, 0};
        axiom_batch_get_launch(batch_, &l[0], &l[1], &l[2]);
        return l;
    }

    void* handle() const { return batch_; }

private:
    explicit PhysicsWorldBatch(void* h) : batch_(h) {}
    void* batch_;
    std::vector<uint32_t> offsets_;
    gui::PhysicsWorldStats stats_{};
    axiom_step_stats info_{};
};

}  // namespace axiom::dynamics

#endif  // AXIOM_WORLD_HPP
