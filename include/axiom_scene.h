/*
 * axiom_scene.h — seeded synthetic scenes for the rigid-body step (host code).
 *
 * Every scene is drawn from the reference's DeterministicRNG (PCG-XSH-RR 64->32, state
 * seed|1, ten warm-up draws, nextFloat = u32 / 2^32, nextFloat(min,max) =
 * min + nextFloat()*(max-min); include/axiom/math/random.hpp:19-64), restated in
 * axiom_rng_* below and pinned against outputs of the reference header.  The generators
 * use no transcendental functions (unit quaternions come from Marsaglia's 1972 method,
 * which needs only square roots), so a seed gives the same bodies on any IEEE host.
 *
 * The scenes are the benchmark configurations of this step:
 *   sphere_drop     1,000 spheres r=0.5 m, rho=1000, rejection-sampled non-overlapping
 *                   centres in a 20x40x20 m box over a ground plane
 *   sphere_lattice  nx*ny*nz spheres on a jittered cubic lattice resting on a plane
 *                   (128x64x128, spacing 0.49 m, r=0.25 m, jitter +-0.002 m)
 *   sphere_pile     the same lattice held by four vertical wall planes touching its outer
 *                   spheres, so that it stays a dense pile (~6 contacts per body) instead
 *                   of spreading out sideways
 *   mixed           spheres / boxes / capsules (40/40/20 %) at random poses
 *   towers          box pyramids and towers of unit boxes with +-2 % size jitter
 * A ground plane (static, shape AXIOM_SHAPE_PLANE, normal +Y through the origin) is the
 * last body of every scene.
 */
#ifndef AXIOM_SCENE_H
#define AXIOM_SCENE_H

#include "axiom_c.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Host-owned scene: SoA arrays of n bodies, laid out like axiom_body_soa. */
typedef struct axiom_scene {
    uint32_t n;
    uint32_t* type;
    uint32_t* shape;
    float* position;          /* 3n */
    float* rotation;          /* 4n */
    float* linear_velocity;   /* 3n */
    float* angular_velocity;  /* 3n */
    float* shape_extents;     /* 3n */
    float* mass;              /* n  */
    float* inertia;           /* 3n */
    float* friction;          /* n  */
    float* restitution;       /* n  */
    float* density;           /* n  */
    float* linear_damping;    /* n  */
    float* angular_damping;   /* n  */
    uint32_t structures;      /* towers: number of structures; otherwise 0 */
} axiom_scene;

AXIOM_API int32_t axiom_scene_sphere_drop(uint64_t seed, uint32_t count, float radius,
                                          float size_x, float size_y, float size_z,
                                          float friction, axiom_scene** out);
AXIOM_API int32_t axiom_scene_sphere_lattice(uint64_t seed, uint32_t nx, uint32_t ny, uint32_t nz,
                                             float spacing, float radius, float jitter,
                                             float friction, axiom_scene** out);
/* The lattice of axiom_scene_sphere_lattice (same bodies, same ids), then four static wall
 * planes (normals +x, -x, +z, -z, through x = -radius, x = (nx-1)*spacing + radius,
 * z = -radius, z = (nz-1)*spacing + radius), then the ground plane. */
AXIOM_API int32_t axiom_scene_sphere_pile(uint64_t seed, uint32_t nx, uint32_t ny, uint32_t nz,
                                          float spacing, float radius, float jitter, float friction,
                                          axiom_scene** out);
AXIOM_API int32_t axiom_scene_mixed(uint64_t seed, uint32_t count, float size_x, float size_y,
                                    float size_z, float friction, axiom_scene** out);
AXIOM_API int32_t axiom_scene_towers(uint64_t seed, uint32_t count, float friction,
                                     axiom_scene** out);
/* Batched worlds: `worlds` worlds whose body counts (including the world's ground plane)
 * are round(median * exp(sigma * z)) clipped to [min_bodies, max_bodies] (z standard
 * normal, Box-Muller on the RNG); each world is a random stack of boxes and spheres in
 * columns of up to 6 on its own ground plane (the plane is the world's last body).
 * world_sizes[worlds] receives each world's body count; bodies of world w follow those of
 * world w - 1. */
AXIOM_API int32_t axiom_scene_batch(uint64_t seed, uint32_t worlds, float median, float sigma,
                                    uint32_t min_bodies, uint32_t max_bodies, float friction,
                                    uint32_t* world_sizes, axiom_scene** out);
AXIOM_API void axiom_scene_free(axiom_scene* scene);
/* Fills an axiom_body_soa that points into the scene's arrays. */
AXIOM_API void axiom_scene_as_soa(const axiom_scene* scene, axiom_body_soa* soa);

/* The restated DeterministicRNG: `count` raw draws / nextFloat draws after seeding. */
AXIOM_API void axiom_rng_u32(uint64_t seed, uint32_t count, uint32_t* out);
AXIOM_API void axiom_rng_float(uint64_t seed, uint32_t count, float* out);
AXIOM_API void axiom_rng_float_range(uint64_t seed, uint32_t count, float lo, float hi, float* out);

#ifdef __cplusplus
}
#endif

#endif /* AXIOM_SCENE_H */
