/*
 * axiom_c.h — C ABI of the GB300 rigid-body collision-and-contact step.
 *
 * The reference engine (itsakeyfut/axiom-physics-engine) reserves the collision and
 * dynamics layers for this path but ships them empty (src/collision/.gitkeep,
 * src/dynamics/.gitkeep; src/CMakeLists.txt:24-27), and it has no FFI of its own.
 * The entry points below are the binding a maintainer of that engine would add to
 * replace those layers: each one names the reference vocabulary it stands in for.
 *
 * Conventions
 *  - Every function returns an int32 status whose values are the reference's
 *    core::ErrorCode numbers (include/axiom/core/error_code.hpp:21-57); 0 is Success.
 *  - The caller owns every host array passed in or out.  A world owns all of its device
 *    memory and frees it in axiom_world_destroy.
 *  - A world is not thread-safe; calls on one world must be serialised by the caller
 *    (the reference's GUI records carry the same main-thread rule,
 *    include/axiom/gui/body_inspector.hpp:109-111).  Each world runs on its own CUDA stream.
 *  - No exception crosses this boundary.
 *  - Units are SI, y is up, quaternions are (x, y, z, w) like math::Quat
 *    (include/axiom/math/quat.hpp:29).
 *
 * The CPU oracle (oracle/liboracle.so) exports the same axiom_world_* symbols with the
 * same meaning, so a test can drive either implementation through this header.
 */
#ifndef AXIOM_C_H
#define AXIOM_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define AXIOM_API __declspec(dllexport)
#else
#define AXIOM_API __attribute__((visibility("default")))
#endif

/* ---- status codes: numeric values of core::ErrorCode (error_code.hpp:21-57) ---- */
enum {
    AXIOM_SUCCESS = 0,
    AXIOM_DIVISION_BY_ZERO = 100,
    AXIOM_OUT_OF_MEMORY = 200,
    AXIOM_INVALID_ALLOCATION = 201,
    AXIOM_NULL_POINTER = 202,
    AXIOM_INVALID_SHAPE = 300,
    AXIOM_GJK_FAILED_TO_CONVERGE = 301,
    AXIOM_EPA_FAILED_TO_CONVERGE = 302,
    AXIOM_INVALID_RIGID_BODY = 400,
    AXIOM_CONSTRAINT_SOLVER_FAILURE = 401,
    AXIOM_GPU_INVALID_OPERATION = 503,
    AXIOM_GPU_TIMEOUT = 504,
    AXIOM_GPU_OPERATION_FAILED = 505,
    AXIOM_INVALID_PARAMETER = 600,
    AXIOM_OUT_OF_RANGE = 601
};

/* gui::BodyType (include/axiom/gui/body_inspector.hpp:13-17) */
enum { AXIOM_BODY_STATIC = 0, AXIOM_BODY_DYNAMIC = 1, AXIOM_BODY_KINEMATIC = 2 };

/* gui::ShapeType values (body_inspector.hpp:20-27), plus the infinite plane of
 * debug::ShapeType::Plane (include/axiom/debug/physics_debug_draw.hpp:87-94).
 * shape_extents meaning: sphere (radius, -, -); box (half-extents x, y, z);
 * capsule (radius, half-height, -), its segment along local Y like the reference's
 * debug capsule (src/debug/physics_debug_draw.cpp:254-266); cylinder (radius,
 * half-height, -), axis along local Y; convex: ignored (the body names a hull added with
 * axiom_world_add_convex_hull in axiom_body_soa.convex_hull); plane: the plane passes
 * through the body position with normal = rotation * (0, 1, 0). */
enum {
    AXIOM_SHAPE_SPHERE = 0,
    AXIOM_SHAPE_BOX = 1,
    AXIOM_SHAPE_CAPSULE = 2,
    AXIOM_SHAPE_CYLINDER = 3,
    AXIOM_SHAPE_MESH = 4,     /* one triangle of a static mesh (axiom_world_add_triangle_mesh) */
    AXIOM_SHAPE_CONVEX = 5,
    AXIOM_SHAPE_PLANE = 6
};

/* Warm-start source for the PGS impulses of a step. */
enum {
    AXIOM_WARM_START_NONE = 0,     /* every contact starts at zero impulse            */
    AXIOM_WARM_START_PREVIOUS = 1, /* previous-step impulse of the same pair/point    */
    AXIOM_WARM_START_LEARNED = 2   /* MLP prediction from per-contact features        */
};

/* gui::PhysicsWorldConfig (include/axiom/gui/physics_panel.hpp:34-43) plus the solver
 * controls of this step. */
typedef struct axiom_world_config {
    float gravity[3];             /* default (0, -9.81, 0)                                 */
    float time_step;              /* default 1/60 s; used when step() is given dt <= 0     */
    uint32_t velocity_iterations; /* default 8: PGS sweeps when residual_tolerance == 0    */
    uint32_t position_iterations; /* default 3; accepted for API parity and ignored: there
                                     is no position-correction pass, penetration is fed
                                     back as a Baumgarte velocity bias (baumgarte, slop)  */
    float residual_tolerance;     /* > 0: sweep until residual <= tol or max_iterations     */
    uint32_t max_iterations;      /* cap for the tolerance mode (default 200)              */
    float baumgarte;              /* position-error feedback factor (default 0.2)          */
    float linear_slop;            /* allowed penetration (default 0.005 m)                 */
    float aabb_margin;            /* broadphase AABB inflation (default 0)                 */
    float restitution_threshold;  /* closing speed above which restitution applies (1 m/s) */
    uint32_t warm_start;          /* AXIOM_WARM_START_* (default PREVIOUS)                 */
    float warm_start_factor;      /* scale applied to warm-start impulses (default 1)      */
    uint32_t pair_capacity;       /* initial broadphase pair capacity (0: 16 per body)     */
    uint32_t contact_capacity;    /* initial manifold capacity (0: 4 per body; grows)      */
    int32_t device;               /* CUDA device ordinal; -1 (default) = current device    */
    /* Sleeping (PhysicsWorldConfig::allowSleep and thresholds, physics_panel.hpp:39-42).
     * The reference enables it by default; this library keeps it off (allow_sleep = 0) so
     * that a step's cost does not depend on the scene's history unless the caller asks.
     * A dynamic body whose speed stays at or below the linear threshold and whose angular
     * speed stays at or below the angular threshold accumulates sleep time; an island
     * (dynamic bodies linked by contacts) whose every body has slept for at least
     * sleep_time_threshold falls asleep: velocities zero, no integration, no contacts with
     * static or other sleeping bodies.  A sleeping island wakes, within the same step,
     * when an awake dynamic body or a moving kinematic body touches one of its bodies.  */
    uint32_t allow_sleep;          /* default 0 here (the reference's default is true)    */
    float sleep_linear_threshold;  /* m/s, default 0.01                                     */
    float sleep_angular_threshold; /* rad/s, default 0.01                                   */
    float sleep_time_threshold;    /* s, default 0.5                                        */
    /* Continuous collision ("prevents tunneling for fast-moving objects", the reference's
     * design notes, CLAUDE.md:136), by speculative contacts: each body's AABB is swept by
     * its displacement over the step, and every pair reports a contact while the gap is
     * within the two bodies' displacements (negative depth = separation): the analytic
     * pairs from their closest points, the support-mapped pairs (box-box, box-capsule and
     * every pair with a cylinder or a hull) by GJK-based CCD: GJK on one shape inflated
     * by that distance decides whether the gap is within it, EPA on the inflated pair
     * gives the normal, and the supporting features are clipped keeping the points within
     * the distance.  The solver lets such a point close exactly its gap in this step (no
     * restitution until it touches), so a fast body stops at the surface instead of
     * passing through.  Batched worlds ignore it.  Default 0 (off). */
    uint32_t speculative_contacts;
    /* Temporally coherent colouring (no reference counterpart: the reference has no
     * solver).  0 (default): every step colours the contact graph greedily in descending
     * manifold priority.  1: a manifold that existed in the previous step keeps its
     * previous colour unless a higher-priority manifold that also existed keeps the same
     * colour at a shared dynamic body; the others (new or conflicting) are coloured
     * greedily in descending priority around the kept colours.  A settled scene then
     * recolours only its new contacts.  The colouring stays proper and deterministic (the
     * CPU oracle computes the same colours); the solve order, and so the solver's
     * rounding, differ from mode 0.  Batched worlds reject it. */
    uint32_t temporal_colouring;
} axiom_world_config;

/* Structure-of-arrays body description, fields of gui::RigidBodyData
 * (body_inspector.hpp:57-90) and gui::MaterialInfo (:30-35).  NULL optional arrays take
 * the reference defaults: rotation identity, velocities zero, restitution 0.5,
 * friction 0.5, density 1000, linear damping 0.01, angular damping 0.05.  A NULL mass
 * (inertia) derives it from density and shape. */
typedef struct axiom_body_soa {
    const uint32_t* type;           /* [n]   AXIOM_BODY_*  (required)          */
    const uint32_t* shape;          /* [n]   AXIOM_SHAPE_* (required)          */
    const float* position;          /* [3n]  (required)                        */
    const float* rotation;          /* [4n]  (x, y, z, w)                      */
    const float* linear_velocity;   /* [3n]                                    */
    const float* angular_velocity;  /* [3n]                                    */
    const float* shape_extents;     /* [3n]  (required; see AXIOM_SHAPE_*)     */
    const float* mass;              /* [n]                                     */
    const float* inertia;           /* [3n]  diagonal, body frame              */
    const float* friction;          /* [n]                                     */
    const float* restitution;       /* [n]                                     */
    const float* density;           /* [n]                                     */
    const float* linear_damping;    /* [n]                                     */
    const float* angular_damping;   /* [n]                                     */
    /* gui::FilterInfo (body_inspector.hpp:38-42), defaults 0x0001 / 0xFFFF / 0.  Two
     * bodies with the same non-zero group always (group > 0) or never (group < 0)
     * collide; otherwise they collide when each one's category is in the other's mask. */
    const uint32_t* filter_category; /* [n]                                    */
    const uint32_t* filter_mask;     /* [n]                                    */
    const int16_t* filter_group;     /* [n]                                    */
    /* gui::SleepInfo (body_inspector.hpp:45-51): allowSleep (default 1) and isSleeping
     * (default 0: a dynamic body may be added asleep, e.g. a pre-settled pile).  Both are
     * ignored while the world's allow_sleep is 0. */
    const uint8_t* allow_sleep;      /* [n]                                    */
    const uint8_t* is_sleeping;      /* [n]                                    */
    /* Hull id (axiom_world_add_convex_hull) of each AXIOM_SHAPE_CONVEX body; required when
     * any body is convex, ignored for other shapes. */
    const uint32_t* convex_hull;     /* [n]                                    */
    /* MaterialInfo::rollingFriction (body_inspector.hpp:33), default 0, finite and >= 0.
     * Carried with the body (snapshots keep it); the solver does not apply rolling
     * resistance yet, so it has no effect on the step. */
    const float* rolling_friction;   /* [n]                                    */
} axiom_body_soa;

/* gui::PhysicsWorldStats (physics_panel.hpp:11-30) plus the counters of this step. */
typedef struct axiom_step_stats {
    uint32_t total_bodies, active_bodies, sleeping_bodies;
    uint32_t static_bodies, dynamic_bodies, kinematic_bodies;
    uint32_t contact_point_count, constraint_count, island_count;
    float total_step_time, broadphase_time, narrowphase_time, solver_time, integration_time;
    uint32_t pair_count;      /* broadphase pairs (inclusive AABB overlap)            */
    uint32_t manifold_count;  /* body pairs in contact                               */
    uint32_t colour_count;    /* colour batches of the contact graph                 */
    uint32_t iterations;      /* PGS sweeps performed                                */
    float residual;           /* max|dλ| / max(max|λ|, 1e-6) of the last sweep       */
    int32_t status;           /* status of the step                                  */
    uint32_t colour_rounds;   /* dependency depth of the colouring: the rounds a parallel (Jones-Plassmann) colouring takes */
    /* Convergence of the support-mapping narrowphase (core::ErrorCode GJKFailedToConverge /
     * EPAFailedToConverge, error_code.hpp:37-38): pairs whose GJK used all its iterations
     * without deciding (treated as separated), and pairs whose EPA stopped at its vertex,
     * face or iteration cap before its tolerance (the closest face found gives the contact).
     * The step still completes; its status is AXIOM_GJK_FAILED_TO_CONVERGE when the first
     * count is non-zero, else AXIOM_EPA_FAILED_TO_CONVERGE when the second is, unless an
     * earlier failure already set it. */
    uint32_t gjk_failures;
    uint32_t epa_failures;
} axiom_step_stats;

/* One contact point: debug::DebugContactPoint (physics_debug_draw.hpp:128-132) with the
 * solver's view of it.  The normal points from body_a to body_b. */
typedef struct axiom_contact_point {
    uint32_t body_a, body_b;
    float position[3];
    float normal[3];
    float penetration_depth;
    float impulse[3];         /* normal, tangent-1, tangent-2 impulse after the solve */
    uint32_t colour;          /* colour batch of the manifold                        */
    uint32_t point_index;     /* index of the point within its manifold              */
} axiom_contact_point;

/* ---- world lifetime: replaces PhysicsWorld construction (CLAUDE.md:160-177 sketch) ---- */
AXIOM_API void axiom_world_config_default(axiom_world_config* config);
AXIOM_API int32_t axiom_world_create(const axiom_world_config* config, void** world);
AXIOM_API int32_t axiom_world_destroy(void* world);

/* Appends n bodies; their ids are first_id .. first_id+n-1 (first_id may be NULL). */
AXIOM_API int32_t axiom_world_add_bodies(void* world, const axiom_body_soa* bodies, uint32_t n,
                                         uint32_t* first_id);
AXIOM_API int32_t axiom_world_body_count(void* world, uint32_t* n);
/* Checks n body descriptions as axiom_world_add_bodies would (the same status) without
 * adding them, so a caller that adds in several calls can check everything first. */
AXIOM_API int32_t axiom_world_check_bodies(void* world, const axiom_body_soa* bodies, uint32_t n);

/* One fixed step of the broadphase -> narrowphase -> solver -> integration order of
 * the reference's step (examples/profiling_example.cpp:132-165).  dt <= 0 uses
 * config.time_step.  stats may be NULL. */
AXIOM_API int32_t axiom_world_step(void* world, float dt, axiom_step_stats* stats);

/* Convex hull (gui::ShapeType::Convex, body_inspector.hpp:26) for AXIOM_SHAPE_CONVEX
 * bodies: count points [3 * count] in the body frame, about the body's centre of mass
 * (the step does not shift them), 4 <= count <= AXIOM_CONVEX_MAX_VERTICES.  The points
 * are used as given (every one is a vertex of the shape for support mapping; interior
 * points are harmless).  *hull_id receives the id bodies name in convex_hull.  A convex
 * body without mass (inertia) takes them from the hull's body-frame bounding box as a
 * solid box of its density.  Contacts: support mapping (GJK / EPA) and clipping of the
 * vertex set that lies on the supporting plane. */
#define AXIOM_CONVEX_MAX_VERTICES 64u
AXIOM_API int32_t axiom_world_add_convex_hull(void* world, const float* points, uint32_t count,
                                              uint32_t* hull_id);

/* Static triangle mesh (gui::ShapeType::Mesh, body_inspector.hpp:25): vertices
 * [3 * vertex_count] in world space (transform on the caller's side) and triangles
 * [3 * triangle_count] of vertex indices.  Each triangle becomes one static body of shape
 * AXIOM_SHAPE_MESH — a flat three-point hull about its centroid — with ids *first_id ..
 * *first_id + triangle_count - 1, the given friction and restitution and the default
 * collision filter; it collides with every other shape through GJK / EPA and the clipping
 * of supporting features (the triangle's face is a three-vertex polygon).  Triangles are
 * two-sided, and a body sliding across an edge shared by two triangles may catch on it.
 * The broadphase grid is as wide as the widest body, so large surfaces should be
 * tessellated into triangles comparable in size to the moving bodies.
 * Returns AXIOM_OUT_OF_RANGE for an index >= vertex_count and AXIOM_INVALID_SHAPE for a
 * triangle without area. */
AXIOM_API int32_t axiom_world_add_triangle_mesh(void* world, const float* vertices, uint32_t vertex_count,
                                                const uint32_t* triangles, uint32_t triangle_count,
                                                float friction, float restitution, uint32_t* first_id);

/* Body state in host memory; any pointer may be NULL. position/linear/angular are [3n],
 * rotation [4n]. */
AXIOM_API int32_t axiom_world_read_state(void* world, float* position, float* rotation,
                                         float* linear_velocity, float* angular_velocity);
AXIOM_API int32_t axiom_world_write_state(void* world, const float* position,
                                          const float* rotation, const float* linear_velocity,
                                          const float* angular_velocity);

/* Sleep state (gui::SleepInfo, body_inspector.hpp:45-51) per body; any pointer may be
 * NULL.  sleeping [n]: 1 while asleep; sleep_time [n]: seconds below the thresholds;
 * island [n]: the island of the last step, named by its lowest body id (the island a
 * sleeping body fell asleep with; 0xFFFFFFFF for static and kinematic bodies and while
 * the world's allow_sleep is 0).  PhysicsWorldStats::islandCount
 * (physics_panel.hpp:23) of a step is the number of islands of its awake bodies. */
AXIOM_API int32_t axiom_world_read_sleep(void* world, uint8_t* sleeping, float* sleep_time,
                                         uint32_t* island);
/* Wakes (sleeping = 0) or puts to sleep (sleeping = 1, velocities zeroed) the n bodies
 * listed in ids; static and kinematic bodies are left alone.  Waking resets the sleep
 * time; a woken body that touches the rest of its island wakes it at the next step.
 * Returns AXIOM_OUT_OF_RANGE for an id >= body count, AXIOM_INVALID_PARAMETER for
 * sleeping = 1 while the world's allow_sleep is 0. */
AXIOM_API int32_t axiom_world_set_sleeping(void* world, const uint32_t* ids, uint32_t n,
                                           int32_t sleeping);

/* AABBs of the last step ([3n] each). */
AXIOM_API int32_t axiom_world_read_aabbs(void* world, float* aabb_min, float* aabb_max);

/* Broadphase pairs of the last step as (a, b) with a < b, in no particular order.
 * Writes min(count, capacity) pairs ([2*capacity]); *count receives the total. */
AXIOM_API int32_t axiom_world_read_pairs(void* world, uint32_t* pairs, uint32_t capacity,
                                         uint32_t* count);

/* Contact points of the last step with their impulses and colours, in no particular
 * order.  Writes min(count, capacity) points; *count receives the total. */
AXIOM_API int32_t axiom_world_read_contacts(void* world, axiom_contact_point* points,
                                            uint32_t capacity, uint32_t* count);

/* ---- world snapshot: checkpoint / resume (no reference counterpart: the reference has no
 * world to save; its debug panel only displays PhysicsWorldStats) ----
 * A snapshot holds everything a world needs to continue bit for bit: the configuration,
 * every body (pose, velocities, mass properties, material, filter, sleep state) and the
 * previous-step impulses the warm start reads.  Layout, little-endian:
 *   axiom_snapshot_header, then header.body_count axiom_snapshot_body records (by body
 *   id), then header.contact_count axiom_snapshot_contact records sorted by
 *   (body_lo, body_hi, point), then the convex hulls: header.hull_count uint32 vertex
 *   counts and header.hull_vertex_count points of 3 floats, hull after hull.
 * The GPU library and the CPU oracle write and read the same format, so a snapshot taken
 * on one resumes on the other.  Not included: the learned warm-start network (set it
 * again), recording and profiling state. */
#define AXIOM_SNAPSHOT_VERSION 3u
typedef struct axiom_snapshot_header {
    char magic[8];                /* "AXSNAP01"                                         */
    uint32_t version;             /* AXIOM_SNAPSHOT_VERSION                             */
    uint32_t body_count;
    uint32_t contact_count;       /* warm-start entries                                 */
    uint32_t flags;               /* bit 0: warm-start entries valid (a step has run)   */
    uint32_t hull_count;          /* convex hulls                                       */
    uint32_t hull_vertex_count;   /* their points, all hulls                            */
    uint64_t total_bytes;         /* header + records                                   */
    axiom_world_config config;
} axiom_snapshot_header;

typedef struct axiom_snapshot_body {  /* 144 bytes */
    uint32_t type;                /* AXIOM_BODY_* (a sleeping body is DYNAMIC + flag)   */
    uint32_t shape;               /* AXIOM_SHAPE_*                                      */
    uint32_t flags;               /* bit 0 sleeping, bit 1 may not sleep                */
    uint32_t island;              /* island label (0xFFFFFFFF: none)                    */
    float position[3];
    float rotation[4];
    float linear_velocity[3];
    float angular_velocity[3];
    float shape_extents[3];       /* convex: (bounding radius, hull id as uint32 bits, 0) */
    float inv_mass;
    float inv_inertia[3];         /* body frame, diagonal                               */
    float friction, restitution, linear_damping, angular_damping;
    uint32_t filter_category, filter_mask;
    int32_t filter_group;
    float sleep_time;
    float rolling_friction;       /* MaterialInfo::rollingFriction                       */
    uint32_t reserved[3];         /* zero                                               */
} axiom_snapshot_body;

typedef struct axiom_snapshot_contact {  /* 24 bytes: a previous-step impulse */
    uint32_t body_lo, body_hi;    /* the pair, lower id first                           */
    uint32_t point;               /* bits 0-7: point index within the manifold; bits
                                     8-15 (point 0 only): 1 + the manifold's colour in
                                     that step (0: unknown), which temporally coherent
                                     colouring starts from                              */
    float impulse[3];             /* normal, tangent-1, tangent-2                       */
} axiom_snapshot_contact;

AXIOM_API int32_t axiom_world_snapshot_size(void* world, uint64_t* bytes);
/* Writes the snapshot into buffer (capacity bytes); *written receives its size.
 * Returns AXIOM_OUT_OF_RANGE (writing nothing) when capacity is too small. */
AXIOM_API int32_t axiom_world_save_snapshot(void* world, void* buffer, uint64_t capacity,
                                            uint64_t* written);
/* Replaces the world's bodies, configuration (except device and the initial capacities),
 * sleep state and warm-start impulses with the snapshot's.  Returns
 * AXIOM_INVALID_PARAMETER for a malformed snapshot (the world is then left empty). */
AXIOM_API int32_t axiom_world_load_snapshot(void* world, const void* buffer, uint64_t size);

/* ---- debug feed: the data of debug::PhysicsDebugDraw (physics_debug_draw.hpp:97-132)
 * for a headless consumer (a recorder, a remote viewer); the reference draws it with
 * Vulkan, which this library does not.  flags select what is filled, with the bit values
 * of debug::PhysicsDebugFlags (physics_debug_draw.hpp:27-40); unselected fields are 0. */
enum {
    AXIOM_DEBUG_SHAPES = 1u << 0,
    AXIOM_DEBUG_AABBS = 1u << 1,
    AXIOM_DEBUG_CONTACTS = 1u << 2,
    AXIOM_DEBUG_VELOCITIES = 1u << 4,
    AXIOM_DEBUG_ISLANDS = 1u << 7
};

typedef struct axiom_debug_body {  /* DebugRigidBody + DebugShape (physics_debug_draw.hpp:97-125) */
    float position[3];            /* SHAPES: transform (scale 1)                        */
    float rotation[4];
    uint32_t shape;               /* SHAPES: AXIOM_SHAPE_*                              */
    float shape_extents[3];       /* SHAPES: as in axiom_body_soa; convex: (bounding
                                     radius, 0, 0)                                       */
    float aabb_min[3], aabb_max[3];   /* AABBS: of the last step                        */
    float linear_velocity[3], angular_velocity[3];  /* VELOCITIES                       */
    uint32_t is_awake;            /* ISLANDS: 0 for static and sleeping bodies          */
    uint32_t island_index;        /* ISLANDS: island label (0xFFFFFFFF: none)           */
} axiom_debug_body;

typedef struct axiom_debug_contact {  /* DebugContactPoint (physics_debug_draw.hpp:128-132) */
    float position[3];
    float normal[3];              /* from body_a to body_b                              */
    float penetration_depth;
    uint32_t body_a, body_b;      /* the bodies in contact (not in DebugContactPoint)   */
} axiom_debug_contact;

/* Debug records of every body ([n], by id) and of the last step's contact points
 * (CONTACTS; in no particular order).  Writes min(count, capacity) of each; the counts
 * receive the totals.  Any array may be NULL. */
AXIOM_API int32_t axiom_world_read_debug(void* world, uint32_t flags, axiom_debug_body* bodies,
                                         uint32_t body_capacity, axiom_debug_contact* contacts,
                                         uint32_t contact_capacity, uint32_t* body_count,
                                         uint32_t* contact_count);

/* ---- learned warm start ----
 * The network maps 14 per-contact features to the initial (normal, tangent-1,
 * tangent-2) impulses; layers 14 -> 128 -> 128 -> 128 -> 3 with SiLU.  Parameters are a
 * flat fp32 array in the order W1[128x16] b1[128] W2[128x128] b2[128] W3[128x128]
 * b3[128] W4[3x128] b4[3] (row-major, output x input; the input width of W1 is padded
 * from 14 to 16 with zero columns). */
#define AXIOM_MLP_INPUTS 14
#define AXIOM_MLP_INPUTS_PADDED 16
#define AXIOM_MLP_HIDDEN 128
#define AXIOM_MLP_OUTPUTS 3
#define AXIOM_MLP_PARAM_COUNT \
    (128 * 16 + 128 + 128 * 128 + 128 + 128 * 128 + 128 + 3 * 128 + 3)

AXIOM_API int32_t axiom_world_set_warm_start_model(void* world, const float* params,
                                                   uint32_t count);

/* Per-contact network features (14 floats, dimensionless) and, as the target, the
 * correction the step's final impulses made to the previous-step impulses in the same
 * units (3 floats: normal, tangent-1, tangent-2), i.e. training samples for the
 * warm-start network, which starts PGS at prev + prediction x (kn |g| dt).  Recording
 * makes every step compute the features:
 *   0-2  relative velocity at the point in the (n, t1, t2) frame / (|g| dt)
 *   3-5  contact normal;  6  depth / linear_slop;  7-8  inverse masses x kn
 *   9-11 previous-step impulses / (kn |g| dt);  12 (invMassA + invMassB) x kn;  13 friction
 * (kn = normal effective mass).  keys ([3 * capacity], may be NULL) receives
 * (body_a, body_b, point_index) of each sample. */
AXIOM_API int32_t axiom_world_set_recording(void* world, int32_t enable);
AXIOM_API int32_t axiom_world_read_samples(void* world, float* features, float* targets,
                                           uint32_t* keys, uint32_t capacity, uint32_t* count);

/* The network itself, for training and inspection (host arrays; device work on the
 * network's own stream).  forward: features [n][14] -> impulses [n][3] in impulse-scale
 * units; gradients: mean squared error over n samples, grads [AXIOM_MLP_PARAM_COUNT];
 * train: Adam, shuffled minibatches (batch a multiple of 128), epochs passes. */
AXIOM_API int32_t axiom_mlp_create(int32_t device, void** mlp);
AXIOM_API int32_t axiom_mlp_destroy(void* mlp);
AXIOM_API int32_t axiom_mlp_set_params(void* mlp, const float* params, uint32_t count);
AXIOM_API int32_t axiom_mlp_get_params(void* mlp, float* params, uint32_t count);
AXIOM_API int32_t axiom_mlp_forward(void* mlp, const float* features, uint32_t n, float* out);
AXIOM_API int32_t axiom_mlp_gradients(void* mlp, const float* features, const float* targets,
                                      uint32_t n, float* grads, float* loss);
AXIOM_API int32_t axiom_mlp_train(void* mlp, const float* features, const float* targets,
                                  uint32_t n, uint32_t epochs, uint32_t batch, float lr,
                                  uint64_t seed, float* final_loss);

/* ---- batched worlds: thousands of independent worlds in one persistent launch ----
 * The reference has no batching; this is the batched form of PhysicsWorld::step
 * (CLAUDE.md:160-177 sketch).  World w owns bodies [sum(sizes[0..w)), + sizes[w]) of the
 * description passed to set_worlds, with world-local ids; at most 8192 bodies and 8
 * planes per world; warm start NONE or PREVIOUS; allow_sleep 0 (batched worlds do not
 * sleep; bodies' is_sleeping is ignored); temporal_colouring 0.  Each world steps exactly as a single
 * world holding the same bodies would.  step() replays a captured CUDA graph; its
 * stats->total_step_time is the device time of the whole batch, per-world times (ns,
 * from the GPU's global timer) come from read_world_stats; its gjk_failures / epa_failures
 * count the worlds with such a pair (flags 64 / 128 of read_world_stats name them). */
AXIOM_API int32_t axiom_batch_create(const axiom_world_config* config, void** batch);
AXIOM_API int32_t axiom_batch_destroy(void* batch);
AXIOM_API int32_t axiom_batch_set_worlds(void* batch, const axiom_body_soa* bodies,
                                         const uint32_t* sizes, uint32_t worlds);
AXIOM_API int32_t axiom_batch_step(void* batch, float dt, axiom_step_stats* stats);
/* counts [8 * worlds]: pairs, manifolds, points, colours, colouring rounds, iterations,
 * flags (1 pairs / 2 manifolds / 4 planes / 8 colours / 16 rounds overflow, 32 residual
 * not reached, 64 a GJK ran out of iterations, 128 an EPA stopped at a cap), GJK pairs; step_ns [worlds]; residual [worlds].  Any may be NULL. */
AXIOM_API int32_t axiom_batch_read_world_stats(void* batch, uint32_t* counts, uint64_t* step_ns,
                                               float* residual);
/* phase_ns [7 * worlds]: the last step's device time per phase of each world (global
 * timer at CTA barriers): 0 velocities + AABBs + sort, 1 sweep, 2 analytic narrowphase
 * and planes, 3 GJK/EPA, 4 colouring + grouping, 5 solver (prepare, warm start, sweeps),
 * 6 impulse storage + positions.  No reference counterpart (the reference's profiler
 * scopes, include/axiom/core/profiler.hpp:46-199, time whole host-side stages). */
AXIOM_API int32_t axiom_batch_read_phase_ns(void* batch, uint64_t* phase_ns);
AXIOM_API int32_t axiom_batch_read_state(void* batch, float* position, float* rotation,
                                         float* linear_velocity, float* angular_velocity);
/* Launch shape of the persistent kernel: threads per world (multiple of 32, <= 512) and
 * resident CTAs per SM. */
AXIOM_API int32_t axiom_batch_set_launch(void* batch, uint32_t block, uint32_t ctas_per_sm);
/* Colour-batch staging: worlds of at most stage_bodies bodies (<= 4096; default 2048; 0:
 * none) run their warm start and sweeps with the bodies in shared memory, 32 bytes a body
 * taken from the CTAs per SM the launch shape can have (AXIOM_OUT_OF_RANGE when the
 * current shape would no longer fit).  Results do not depend on it. */
AXIOM_API int32_t axiom_batch_set_stage(void* batch, uint32_t stage_bodies);
AXIOM_API int32_t axiom_batch_get_launch(void* batch, uint32_t* block, uint32_t* ctas_per_sm,
                                         uint32_t* stage_bodies);
/* Times trial_steps steps of every feasible (launch shape, staging) on a snapshot of the
 * state, in two interleaved rounds (a shape's better round counts), and keeps the fastest
 * (the state is restored); cache_path (may be NULL) stores and reuses the choice per
 * (worlds, bodies). */
AXIOM_API int32_t axiom_batch_autotune(void* batch, const char* cache_path, uint32_t trial_steps,
                                       uint32_t* block, uint32_t* ctas_per_sm);
/* Work-queue integrity.  Every step checks that each world was stepped exactly once (a
 * per-world step stamp) and that every queue entry the kernel popped named a world (the
 * kernel checks each entry before use and counts the bad ones); otherwise the step returns
 * AXIOM_GPU_INVALID_OPERATION (an entry named no world) or AXIOM_GPU_OPERATION_FAILED
 * (worlds left unstepped).  inject_queue_fault corrupts the next step's queue on the host
 * to test this: kind 1 starts the main lane's counter at `value` (its first `value` worlds
 * are skipped), kind 2 makes main-lane entry `value` name no world.  The queue is intact
 * again for the steps after.  Nothing faults: all accesses stay in bounds. */
AXIOM_API int32_t axiom_batch_inject_queue_fault(void* batch, uint32_t kind, uint32_t value);

/* ---- profiling: the per-stage scopes of the reference's Tracy profiler
 * (include/axiom/core/profiler.hpp:46-199; scope names Broadphase, Narrowphase, Solver,
 * Integration), as CUDA-event durations on the world's stream.  Launch counts are always
 * kept; durations only while profiling is enabled (it adds two events per range). */
typedef struct axiom_kernel_profile {
    char name[32];         /* kernel group, e.g. "pgs_colour"                        */
    uint64_t launches;     /* kernel launches of the group since the last reset      */
    uint64_t ranges;       /* timed ranges (each brackets one or more launches)      */
    double total_ms;       /* summed device time of the timed ranges                 */
} axiom_kernel_profile;

AXIOM_API int32_t axiom_world_set_profiling(void* world, int32_t enable);
/* Times only the kernel groups whose bit is set (bit g = the g-th entry that
 * axiom_world_read_profile reports); 0 turns timing off.  Each timed range adds two
 * events to the stream, so timing only the groups of interest keeps the step closer to
 * its unprofiled speed. */
AXIOM_API int32_t axiom_world_set_profiling_groups(void* world, uint32_t group_mask);
AXIOM_API int32_t axiom_world_reset_profile(void* world);
AXIOM_API int32_t axiom_world_read_profile(void* world, axiom_kernel_profile* out,
                                           uint32_t capacity, uint32_t* count);

/* ---- broadphase without allocation ----
 * No counterpart in the reference.  For callers that must not allocate GPU memory at
 * run time: code running inside a pre-sized memory pool, a real-time loop that may not
 * stall on cudaMalloc, or a plugin host that owns all device allocations.  It computes
 * the same pair set as the world's broadphase (every (a, b), a < b, whose AABBs
 * intersect inclusively and of which at least one is dynamic) for at most
 * AXIOM_BROADPHASE_STATIC_MAX_BODIES bodies, using a fixed scratch area that the library
 * reserves in device memory when it is loaded (about 6 MB on every GPU that loads it,
 * held until the process exits).  It calls no cudaMalloc, cudaFree or allocating
 * library routine.
 *
 * All pointers are device pointers.  aabb_min / aabb_max: [3n] floats (x, y, z per body);
 * dynamic: [n] flags (non-zero = dynamic) or NULL for all dynamic; pairs: [2 * capacity]
 * (8-byte aligned) receives (a, b) pairs in no particular order; *count (device) receives
 * the total pair count, which may exceed capacity (then only capacity pairs are written).
 * stream: a cudaStream_t, or NULL for the default stream.  Work is queued on the stream;
 * the call does not wait for it.
 *
 * Every call on one GPU shares the scratch area, and it keeps the last call's contents:
 * calls whose GPU work overlaps (different streams, or different host threads) race and
 * must be serialised by the caller.  The first call on each device looks up the scratch
 * address (cudaGetSymbolAddress) with that device current; make that first call before
 * any stream capture.  Returns AXIOM_INVALID_PARAMETER when n exceeds the maximum. */
#define AXIOM_BROADPHASE_STATIC_MAX_BODIES 65536u
AXIOM_API int32_t axiom_broadphase_pairs_static(const float* aabb_min, const float* aabb_max,
                                                const uint32_t* dynamic, uint32_t n,
                                                uint32_t* pairs, uint32_t capacity,
                                                uint32_t* count, void* stream);

/* Library version string. */
AXIOM_API const char* axiom_version(void);

#ifdef __cplusplus
}
#endif

#endif /* AXIOM_C_H */
