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
// Inside the engine, define AXIOM_GB300_ENGINE_TYPES before including this header: Result,
// ErrorCode and PhysicsWorldStats are then the engine's own (axiom/core/result.hpp,
// axiom/gui/physics_panel.hpp).  Standalone, the header defines minimal equivalents with
// the same names, numeric codes and member functions.
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

#ifdef AXIOM_GB300_ENGINE_TYPES
#include "axiom/core/result.hpp"
#include "axiom/gui/physics_panel.hpp"
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
    int32_t device = -1;  // CUDA device ordinal; -1 = the current device
};

// gui::MaterialInfo and gui::FilterInfo with the engine's defaults.
struct MaterialInfo {
    float restitution = 0.5f;
    float friction = 0.5f;
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

class PhysicsWorld {
public:
    using Ptr = std::unique_ptr<PhysicsWorld>;

    static core::Result<Ptr> create(const WorldConfig& config = WorldConfig{}) {
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
        c.device = config.device;
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
    // empty lets the library derive them).
    core::Result<BodyId> createBodies(const RigidBodyDesc* descs, size_t count) {
        if (!descs && count) return core::Result<BodyId>::failure(core::ErrorCode::NullPointer, "createBodies");
        uint32_t first = 0;
        if (const int32_t s = axiom_world_body_count(world_, &first); s != AXIOM_SUCCESS)
            return core::Result<BodyId>::failure(code(s), "axiom_world_body_count");
        size_t begin = 0;
        while (begin < count) {
            const bool hasMass = descs[begin].mass.has_value();
            const bool hasInertia = descs[begin].inertiaTensor.has_value();
            size_t end = begin + 1;
            while (end < count && descs[end].mass.has_value() == hasMass &&
                   descs[end].inertiaTensor.has_value() == hasInertia)
                ++end;
            if (const int32_t s = addRun(descs + begin, end - begin, hasMass, hasInertia); s != AXIOM_SUCCESS)
                return core::Result<BodyId>::failure(code(s), "axiom_world_add_bodies");
            begin = end;
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
    core::Result<void> step(float dt = 0.0f) {
        const int32_t s = axiom_world_step(world_, dt, &info_);
        if (s != AXIOM_SUCCESS) return core::Result<void>::failure(code(s), "axiom_world_step");
        stats_.totalBodies = info_.total_bodies;
        stats_.activeBodies = info_.active_bodies;
        stats_.sleepingBodies = info_.sleeping_bodies;
        stats_.staticBodies = info_.static_bodies;
        stats_.dynamicBodies = info_.dynamic_bodies;
        stats_.kinematicBodies = info_.kinematic_bodies;
        stats_.contactPointCount = info_.contact_point_count;
        stats_.constraintCount = info_.constraint_count;
        stats_.islandCount = info_.island_count;
        stats_.totalStepTime = info_.total_step_time;
        stats_.broadphaseTime = info_.broadphase_time;
        stats_.narrowphaseTime = info_.narrowphase_time;
        stats_.solverTime = info_.solver_time;
        stats_.integrationTime = info_.integration_time;
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
        BodyStates st;
        const uint32_t n = bodyCount();
        st.position.resize(n);
        st.rotation.resize(n);
        st.linearVelocity.resize(n);
        st.angularVelocity.resize(n);
        if (n == 0) return core::Result<BodyStates>::success(std::move(st));
        const int32_t s = axiom_world_read_state(world_, &st.position[0].x, &st.rotation[0].x,
                                                 &st.linearVelocity[0].x, &st.angularVelocity[0].x);
        if (s != AXIOM_SUCCESS) return core::Result<BodyStates>::failure(code(s), "axiom_world_read_state");
        return core::Result<BodyStates>::success(std::move(st));
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

    static core::ErrorCode code(int32_t s) { return static_cast<core::ErrorCode>(s); }

    int32_t addRun(const RigidBodyDesc* d, size_t n, bool hasMass, bool hasInertia) {
        std::vector<uint32_t> type(n), shape(n), category(n), mask(n), hull(n);
        std::vector<float> pos(3 * n), rot(4 * n), lin(3 * n), ang(3 * n), ext(3 * n), mass, inertia;
        std::vector<float> friction(n), restitution(n), density(n), linDamp(n), angDamp(n);
        std::vector<int16_t> group(n);
        std::vector<uint8_t> allowSleep(n), sleeping(n);
        if (hasMass) mass.resize(n);
        if (hasInertia) inertia.resize(3 * n);
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
        axiom_body_soa soa{};
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
        return axiom_world_add_bodies(world_, &soa, static_cast<uint32_t>(n), nullptr);
    }

    void* world_;
    gui::PhysicsWorldStats stats_{};
    axiom_step_stats info_{};
};

}  // namespace axiom::dynamics

#endif  // AXIOM_WORLD_HPP
