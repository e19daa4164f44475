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
    NarrowBody* __restrict__ nbody, uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    velocityStep(i, sp, info, rot, sb, mat, iloc, iw0, iw1);
    const f3 mn = bodyAabb(i, sp, info, pos, rot, shp, aabbMin, aabbMax);
    const uint32_t inf = info[i];
    const float4 e = shp[i];
    nbody[i] = NarrowBody{pos[i], make_float4(e.x, e.y, e.z, __uint_as_float(inf))};
    const uint32_t shape = (inf >> 4) & 0xFu;
    uint32_t key = kEmptyKey32;
    if (shape != AXIOM_SHAPE_PLANE) {
        key = spread10(cellCoord(mn.x, sp.invCell)) | (spread10(cellCoord(mn.y, sp.invCell)) << 1) |
              (spread10(cellCoord(mn.z, sp.invCell)) << 2);
    }
    keys[i] = key;
    vals[i] = i;
}

// Speculative contacts, pass 1: velocities, AABB swept by this step's displacement v dt
// (dynamic and kinematic bodies), the sweep length |v dt| in pos.w, and the widest swept
// AABB of the step.
__global__ void __launch_bounds__(256) kIntegrateSwept(
    uint32_t n, StepParams sp, const uint32_t* __restrict__ info, float4* __restrict__ pos,
    const float4* __restrict__ rot, SolverBody* __restrict__ sb, const float4* __restrict__ shp,
    const float4* __restrict__ mat, const float4* __restrict__ iloc, float4* __restrict__ iw0,
    float4* __restrict__ iw1, float4* __restrict__ aabbMin, float4* __restrict__ aabbMax,
    NarrowBody* __restrict__ nbody, DevCounters* cnt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float width = 0.0f;
    if (i < n) {
        velocityStep(i, sp, info, rot, sb, mat, iloc, iw0, iw1);
        bodyAabb(i, sp, info, pos, rot, shp, aabbMin, aabbMax);
        const uint32_t inf = info[i];
        const uint32_t t = inf & kInfoTypeMask, shape = (inf >> 4) & 0xFu;
        float4 p = pos[i];
        p.w = 0.0f;
        if ((t == AXIOM_BODY_DYNAMIC || t == AXIOM_BODY_KINEMATIC) && shape != AXIOM_SHAPE_PLANE) {
            const float4 v = sb[i].v;
            const float dx = v.x * sp.dt, dy = v.y * sp.dt, dz = v.z * sp.dt;
            float4 lo = aabbMin[i], hi = aabbMax[i];
            lo.x = lo.x + (dx < 0.0f ? dx : 0.0f);
            lo.y = lo.y + (dy < 0.0f ? dy : 0.0f);
            lo.z = lo.z + (dz < 0.0f ? dz : 0.0f);
            hi.x = hi.x + (dx > 0.0f ? dx : 0.0f);
            hi.y = hi.y + (dy > 0.0f ? dy : 0.0f);
            hi.z = hi.z + (dz > 0.0f ? dz : 0.0f);
            aabbMin[i] = lo;
            aabbMax[i] = hi;
            p.w = sqrtf(dx * dx + dy * dy + dz * dz);
            width = fmaxf(hi.x - lo.x, fmaxf(hi.y - lo.y, hi.z - lo.z));
            width = width > 0.0f ? width : 0.0f;
        }
        pos[i] = p;
        const float4 e = shp[i];
        nbody[i] = NarrowBody{p, make_float4(e.x, e.y, e.z, __uint_as_float(inf))};
    }
    // non-negative floats order like their bit patterns: one atomic per warp
    const unsigned wbits = __reduce_max_sync(0xFFFFFFFFu, __float_as_uint(width));
    if ((threadIdx.x & 31u) == 0u && wbits) atomicMax(&cnt->sweptWidthBits, wbits);
}

// Speculative contacts, pass 2: cell keys on a grid wide enough for the widest swept AABB.
__global__ void __launch_bounds__(256) kSweptKeys(uint32_t n, StepParams sp, const uint32_t* __restrict__ info,
                                                  const float4* __restrict__ aabbMin, const DevCounters* cnt,
                                                  uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float swept = __uint_as_float(cnt->sweptWidthBits);
    const float widest = swept > sp.cellWidth ? swept : sp.cellWidth;
    const float invCell = 1.0f / (widest > 0.0f ? widest * 1.0625f : 1.0f);
    const uint32_t shape = (info[i] >> 4) & 0xFu;
    uint32_t key = kEmptyKey32;
    if (shape != AXIOM_SHAPE_PLANE) {
        const float4 mn = aabbMin[i];
        key = spread10(cellCoord(mn.x, invCell)) | (spread10(cellCoord(mn.y, invCell)) << 1) |
              (spread10(cellCoord(mn.z, invCell)) << 2);
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
    if (sp.spec) {
        w.prof.launches[KG_INTEGRATE_VELOCITIES] += 2;
        kIntegrateSwept<<<gridFor(w.n, 256), 256, 0, w.stream>>>(w.n, sp, w.info.p, w.pos.p, w.rot.p, w.body.p,
                                                                 w.shp.p, w.mat.p, w.iloc.p, w.iw0.p, w.iw1.p,
                                                                 w.aabbMin.p, w.aabbMax.p, w.nbody.p, w.dcnt);
        kSweptKeys<<<gridFor(w.n, 256), 256, 0, w.stream>>>(w.n, sp, w.info.p, w.aabbMin.p, w.dcnt, w.keyA.p,
                                                            w.valA.p);
        return;
    }
    w.prof.launches[KG_INTEGRATE_VELOCITIES] += 1;
    kIntegrateVelocities<<<gridFor(w.n, 256), 256, 0, w.stream>>>(
        w.n, sp, w.info.p, w.pos.p, w.rot.p, w.body.p, w.shp.p, w.mat.p, w.iloc.p, w.iw0.p,
        w.iw1.p, w.aabbMin.p, w.aabbMax.p, w.nbody.p, w.keyA.p, w.valA.p);
}

void launchIntegratePositions(World& w, const StepParams& sp) {
    ProfRange pr(w, KG_INTEGRATE_POSITIONS);
    w.prof.launches[KG_INTEGRATE_POSITIONS] += 1;
    kIntegratePositions<<<gridFor(w.n, 256), 256, 0, w.stream>>>(w.n, sp, w.info.p, w.pos.p,
                                                                  w.rot.p, w.body.p);
}

}  // namespace axiom_gb300
