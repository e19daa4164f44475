// sleep.cu — islands, sleeping and waking (PhysicsWorldConfig::allowSleep and its
// thresholds, include/axiom/gui/physics_panel.hpp:39-42; per-body gui::SleepInfo,
// include/axiom/gui/body_inspector.hpp:45-51; PhysicsWorldStats::islandCount and
// sleepingBodies, physics_panel.hpp:13-23).  The reference reserves this for its empty
// dynamics layer (src/dynamics/.gitkeep).
//
// Island / sleep pass (end of a step, after position integration):
//   1. every awake dynamic body updates its sleep time: reset to 0 when its speed or
//      angular speed exceeds the threshold (compared squared) or it may not sleep,
//      otherwise += dt;
//   2. islands = connected components of the awake dynamic bodies under the step's
//      contacts between two awake dynamic bodies (static and kinematic bodies do not link
//      islands).  Lock-free union-find: a root is hooked under the lower-id root by one
//      atomicCAS, so every island ends labelled by its lowest body id whatever order the
//      unions land in — the same labels a sequential union-find gives;
//   3. an island whose minimum sleep time is at least the threshold falls asleep: its
//      bodies take the internal type kTypeSleeping, velocities become zero, and each keeps
//      its island label.
// Wake pass (after the narrowphase, while any body sleeps): a contact between a sleeping
// body and an awake dynamic or a moving kinematic body marks the sleeper's island with
// the pass's generation number; every sleeping body whose island carries it wakes (type
// back to dynamic, sleep time 0) and receives this step's velocity integration, which it
// missed while asleep.  The caller then recomputes the step's contacts.
//
// Every loop below follows parent links, which always point to a lower id, or retries a
// CAS that failed because another thread hooked the root it wanted: all terminate.
#include "dmath.cuh"
#include "world.h"

#include "integrate_math.cuh"

namespace axiom_gb300 {
namespace {

// Root of x, shortening the path as it goes (each node is pointed at its grandparent).
// parent[v] <= v everywhere and parent[r] == r only at roots; the loads bypass L1 so a
// thread sees the links other SMs have made.
__device__ __forceinline__ uint32_t findRoot(uint32_t* parent, uint32_t x) {
    uint32_t cur = __ldcg(parent + x);
    if (cur == x) return x;
    uint32_t prev = x;
    uint32_t next;
    while (cur > (next = __ldcg(parent + cur))) {
        __stcg(parent + prev, next);  // next is an ancestor of prev: the link stays valid
        prev = cur;
        cur = next;
    }
    return cur;
}

__device__ __forceinline__ void unite(uint32_t* parent, uint32_t a, uint32_t b) {
    uint32_t ra = findRoot(parent, a), rb = findRoot(parent, b);
    while (ra != rb) {
        if (ra > rb) {
            const uint32_t t = ra;
            ra = rb;
            rb = t;
        }
        const uint32_t old = atomicCAS(parent + rb, rb, ra);  // hook the higher root under the lower
        if (old == rb) return;
        rb = findRoot(parent, old);  // rb was hooked meanwhile: continue from its new root
        ra = findRoot(parent, ra);
    }
}

__device__ __forceinline__ void warpCount(bool pred, uint32_t* counter) {
    const unsigned ballot = __ballot_sync(0xFFFFFFFFu, pred);
    if ((threadIdx.x & 31u) == 0u && ballot) atomicAdd(counter, (uint32_t)__popc(ballot));
}

__global__ void __launch_bounds__(256) kSleepPrep(uint32_t n, StepParams sp, const uint32_t* __restrict__ info,
                                                  const SolverBody* __restrict__ sb, float* __restrict__ sleepTime,
                                                  uint32_t* __restrict__ parent, uint32_t* __restrict__ islandMin) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t inf = info[i];
    if ((inf & kInfoTypeMask) != AXIOM_BODY_DYNAMIC) return;
    const float4 v = sb[i].v, w = sb[i].w;
    const float lin2 = (v.x * v.x + v.y * v.y) + v.z * v.z;
    const float ang2 = (w.x * w.x + w.y * w.y) + w.z * w.z;
    const bool moving = (inf & kInfoNoSleep) != 0u || lin2 > sp.sleepLin2 || ang2 > sp.sleepAng2;
    sleepTime[i] = moving ? 0.0f : sleepTime[i] + sp.dt;
    parent[i] = i;
    islandMin[i] = 0x7F800000u;  // +inf
}

__global__ void __launch_bounds__(256) kSleepUnion(uint32_t nM, const uint4* __restrict__ hdr,
                                                   uint32_t* __restrict__ parent) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nM) return;
    const uint4 h = hdr[m];
    if ((h.w & (kHdrDynA | kHdrDynB)) == (kHdrDynA | kHdrDynB)) unite(parent, h.x, h.y);
}

__global__ void __launch_bounds__(256) kSleepRoots(uint32_t n, const uint32_t* __restrict__ info,
                                                   uint32_t* __restrict__ parent, uint32_t* __restrict__ island,
                                                   const float* __restrict__ sleepTime,
                                                   uint32_t* __restrict__ islandMin, DevCounters* cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool root = false;
    if (i < n && (info[i] & kInfoTypeMask) == AXIOM_BODY_DYNAMIC) {
        const uint32_t r = findRoot(parent, i);
        island[i] = r;
        atomicMin(islandMin + r, __float_as_uint(sleepTime[i]));  // non-negative floats order as integers
        root = r == i;
    }
    warpCount(root, &cnt->islands);
}

__global__ void __launch_bounds__(256) kSleepApply(uint32_t n, StepParams sp, uint32_t* __restrict__ info,
                                                   const uint32_t* __restrict__ island,
                                                   const uint32_t* __restrict__ islandMin,
                                                   SolverBody* __restrict__ sb, DevCounters* cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool asleep = false;
    if (i < n) {
        const uint32_t inf = info[i];
        const uint32_t type = inf & kInfoTypeMask;
        asleep = type == kTypeSleeping;
        if (type == AXIOM_BODY_DYNAMIC && __uint_as_float(__ldcg(islandMin + island[i])) >= sp.sleepTime) {
            info[i] = (inf & ~kInfoTypeMask) | kTypeSleeping;
            SolverBody b = sb[i];
            b.v = make_float4(0.0f, 0.0f, 0.0f, b.v.w);
            b.w = make_float4(0.0f, 0.0f, 0.0f, b.w.w);
            sb[i] = b;
            asleep = true;
        }
    }
    warpCount(asleep, &cnt->sleeping);
}

// A contact between a sleeper and an awake dynamic body or a kinematic body (the
// broadphase pairs a sleeper with a kinematic body only while that one moves).
__global__ void __launch_bounds__(256) kWakeMark(uint32_t nM, const uint4* __restrict__ hdr,
                                                 const uint32_t* __restrict__ info,
                                                 const uint32_t* __restrict__ island, uint32_t* __restrict__ wakeGen,
                                                 uint32_t gen) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nM) return;
    const uint4 h = hdr[m];
    const uint32_t ta = info[h.x] & kInfoTypeMask, tb = info[h.y] & kInfoTypeMask;
    if (ta == kTypeSleeping && ((h.w & kHdrDynB) || tb == AXIOM_BODY_KINEMATIC)) wakeGen[island[h.x]] = gen;
    if (tb == kTypeSleeping && ((h.w & kHdrDynA) || ta == AXIOM_BODY_KINEMATIC)) wakeGen[island[h.y]] = gen;
}

__global__ void __launch_bounds__(256) kWakeBodies(uint32_t n, StepParams sp, uint32_t* __restrict__ info,
                                                   const uint32_t* __restrict__ island,
                                                   const uint32_t* __restrict__ wakeGen, uint32_t gen,
                                                   float* __restrict__ sleepTime, const float4* __restrict__ rot,
                                                   SolverBody* __restrict__ sb, const float4* __restrict__ mat,
                                                   const float4* __restrict__ iloc, float4* __restrict__ iw0,
                                                   float4* __restrict__ iw1, NarrowBody* __restrict__ nbody,
                                                   DevCounters* cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool woke = false;
    if (i < n) {
        const uint32_t inf = info[i];
        if ((inf & kInfoTypeMask) == kTypeSleeping && wakeGen[island[i]] == gen) {
            const uint32_t awake = (inf & ~kInfoTypeMask) | AXIOM_BODY_DYNAMIC;
            info[i] = awake;
            nbody[i].s.w = __uint_as_float(awake);
            sleepTime[i] = 0.0f;
            velocityStep(i, sp, info, rot, sb, mat, iloc, iw0, iw1);  // this step's gravity and damping
            woke = true;
        }
    }
    warpCount(woke, &cnt->woken);
}

__global__ void __launch_bounds__(256) kSetSleeping(uint32_t n, const uint32_t* __restrict__ ids, uint32_t sleeping,
                                                    uint32_t* __restrict__ info, SolverBody* __restrict__ sb,
                                                    float* __restrict__ sleepTime, uint32_t* __restrict__ island) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t i = ids[k];
    const uint32_t inf = info[i];
    const uint32_t type = inf & kInfoTypeMask;
    if (!sleeping && type == kTypeSleeping) {
        info[i] = (inf & ~kInfoTypeMask) | AXIOM_BODY_DYNAMIC;
        sleepTime[i] = 0.0f;
    } else if (sleeping && type == AXIOM_BODY_DYNAMIC) {
        info[i] = (inf & ~kInfoTypeMask) | kTypeSleeping;
        SolverBody b = sb[i];
        b.v = make_float4(0.0f, 0.0f, 0.0f, b.v.w);
        b.w = make_float4(0.0f, 0.0f, 0.0f, b.w.w);
        sb[i] = b;
        sleepTime[i] = 0.0f;
        island[i] = i;  // an island of its own until contacts wake it
    }
}

__global__ void __launch_bounds__(256) kCountSleeping(uint32_t n, const uint32_t* __restrict__ info, DevCounters* cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    warpCount(i < n && (info[i] & kInfoTypeMask) == kTypeSleeping, &cnt->sleeping);
}

}  // namespace

void launchWake(World& w, const StepParams& sp, uint32_t nM) {
    ProfRange pr(w, KG_SLEEP);
    w.prof.launches[KG_SLEEP] += 2;
    const uint32_t gen = ++w.wakeGeneration;
    cudaMemsetAsync(&w.dcnt->woken, 0, sizeof(uint32_t), w.stream);
    if (nM) kWakeMark<<<gridFor(nM, 256), 256, 0, w.stream>>>(nM, w.mhdr.p, w.info.p, w.island.p, w.wakeGen.p, gen);
    kWakeBodies<<<gridFor(w.n, 256), 256, 0, w.stream>>>(w.n, sp, w.info.p, w.island.p, w.wakeGen.p, gen,
                                                         w.sleepTime.p, w.rot.p, w.body.p, w.mat.p, w.iloc.p,
                                                         w.iw0.p, w.iw1.p, w.nbody.p, w.dcnt);
}

void launchIslands(World& w, const StepParams& sp, uint32_t nM) {
    ProfRange pr(w, KG_SLEEP);
    w.prof.launches[KG_SLEEP] += 4;
    const unsigned g = gridFor(w.n, 256);
    kSleepPrep<<<g, 256, 0, w.stream>>>(w.n, sp, w.info.p, w.body.p, w.sleepTime.p, w.ufParent.p, w.islandMin.p);
    if (nM) kSleepUnion<<<gridFor(nM, 256), 256, 0, w.stream>>>(nM, w.mhdr.p, w.ufParent.p);
    kSleepRoots<<<g, 256, 0, w.stream>>>(w.n, w.info.p, w.ufParent.p, w.island.p, w.sleepTime.p, w.islandMin.p,
                                         w.dcnt);
    kSleepApply<<<g, 256, 0, w.stream>>>(w.n, sp, w.info.p, w.island.p, w.islandMin.p, w.body.p, w.dcnt);
}

void launchSetSleeping(World& w, const uint32_t* ids, uint32_t n, bool sleeping) {
    if (!n) return;
    kSetSleeping<<<gridFor(n, 256), 256, 0, w.stream>>>(n, ids, sleeping ? 1u : 0u, w.info.p, w.body.p,
                                                        w.sleepTime.p, w.island.p);
}

void launchCountSleeping(World& w) {
    cudaMemsetAsync(&w.dcnt->sleeping, 0, sizeof(uint32_t), w.stream);
    kCountSleeping<<<gridFor(w.n, 256), 256, 0, w.stream>>>(w.n, w.info.p, w.dcnt);
}

}  // namespace axiom_gb300
