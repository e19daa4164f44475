// integrate.cu — velocity integration + AABB + cell keys, and position integration.
//
// Semi-implicit Euler (the reference's toy step integrates explicitly,
// examples/profiling_example.cpp:35-41; this step integrates velocity first, solves
// contacts, then moves positions with the solved velocity).  Damping follows the
// linearDamping / angularDamping fields of gui::RigidBodyData (body_inspector.hpp:77-78)
// as v *= 1 / (1 + dt * damping).
#include "dmath.cuh"
#include "world.h"

#include "integrate_math.cuh"

namespace axiom_gb300 {
namespace {

__global__ void __launch_bounds__(256) kIntegrateVelocities(
    uint32_t n, StepParams sp, const uint32_t* __restrict__ info, const float4* __restrict__ pos,
    const float4* __restrict__ rot, SolverBody* __restrict__ sb, const float4* __restrict__ shp,
    const float4* __restrict__ mat, const float4* __restrict__ iloc, float4* __restrict__ iw0,
    float4* __restrict__ iw1, float4* __restrict__ aabbMin, float4* __restrict__ aabbMax,
    uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    velocityStep(i, sp, info, rot, sb, mat, iloc, iw0, iw1);
    const f3 mn = bodyAabb(i, sp, info, pos, rot, shp, aabbMin, aabbMax);
    const uint32_t shape = (info[i] >> 4) & 0xFu;
    uint32_t key = kEmptyKey32;
    if (shape != AXIOM_SHAPE_PLANE) {
        key = spread10(cellCoord(mn.x, sp.invCell)) | (spread10(cellCoord(mn.y, sp.invCell)) << 1) |
              (spread10(cellCoord(mn.z, sp.invCell)) << 2);
    }
    keys[i] = key;
    vals[i] = i;
}

__global__ void __launch_bounds__(256) kIntegratePositions(uint32_t n, StepParams sp,
                                                           const uint32_t* __restrict__ info,
                                                           float4* __restrict__ pos,
                                                           float4* __restrict__ rot,
                                                           const SolverBody* __restrict__ sb) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    positionStep(i, sp, info, pos, rot, sb);
}

}  // namespace

void launchIntegrateVelocities(World& w, const StepParams& sp) {
    ProfRange pr(w, KG_INTEGRATE_VELOCITIES);
    w.prof.launches[KG_INTEGRATE_VELOCITIES] += 1;
    kIntegrateVelocities<<<gridFor(w.n, 256), 256, 0, w.stream>>>(
        w.n, sp, w.info.p, w.pos.p, w.rot.p, w.body.p, w.shp.p, w.mat.p, w.iloc.p, w.iw0.p,
        w.iw1.p, w.aabbMin.p, w.aabbMax.p, w.keyA.p, w.valA.p);
}

void launchIntegratePositions(World& w, const StepParams& sp) {
    ProfRange pr(w, KG_INTEGRATE_POSITIONS);
    w.prof.launches[KG_INTEGRATE_POSITIONS] += 1;
    kIntegratePositions<<<gridFor(w.n, 256), 256, 0, w.stream>>>(w.n, sp, w.info.p, w.pos.p,
                                                                  w.rot.p, w.body.p);
}

}  // namespace axiom_gb300
