// narrowphase.cu — contact manifolds from broadphase pairs and from the ground planes.
//
// The reference's narrowphase is a sleep stub (examples/profiling_example.cpp:77-87);
// the contact record it intends is debug::DebugContactPoint (position, normal,
// penetrationDepth; include/axiom/debug/physics_debug_draw.hpp:128-132).  Contact model:
// pair manifolds have a < b and a normal from a to b; plane manifolds are (plane, body)
// with the plane normal; a point lies midway between the two surfaces and touching
// (depth 0) counts.  Manifolds are compacted with one warp-aggregated atomic per warp.
#include <algorithm>

#include "dmath.cuh"
#include "gjk_epa.cuh"
#include "narrow_shapes.cuh"
#include "world.h"

namespace axiom_gb300 {
namespace {

using namespace axd;

struct ManifoldOut {
    uint4* hdr;
    float4* n;
    float4* p0;
    float4* p1;
    float4* p2;
    float4* p3;
    uint32_t cap;
};

__device__ __forceinline__ uint32_t hdrDyn(uint32_t infoA, uint32_t infoB) {
    return ((infoA & kInfoTypeMask) == AXIOM_BODY_DYNAMIC ? kHdrDynA : 0u) |
           ((infoB & kInfoTypeMask) == AXIOM_BODY_DYNAMIC ? kHdrDynB : 0u);
}

// A sphere's contacts do not depend on its orientation: skip the gather.
__device__ __forceinline__ float4 shapeRot(const float4* __restrict__ rot, uint32_t i, uint32_t shape) {
    return shape == AXIOM_SHAPE_SPHERE ? make_float4(0.0f, 0.0f, 0.0f, 1.0f) : rot[i];
}

// Writes manifold idx (a reserved slot; past the capacity only counted).  Points are summed
// per thread in pts and added to the counter once at the end of the kernel.
__device__ __forceinline__ void writeManifold(uint32_t idx, uint32_t a, uint32_t b, uint32_t dyn, const Contact& c,
                                              const ManifoldOut& out, uint32_t& pts) {
    pts += c.count;
    if (idx >= out.cap) return;
    out.hdr[idx] = make_uint4(a, b, c.count, dyn);
    out.n[idx] = make_float4(c.n.x, c.n.y, c.n.z, 0.0f);
    out.p0[idx] = make_float4(c.p[0].x, c.p[0].y, c.p[0].z, c.depth[0]);
    if (c.count > 1) out.p1[idx] = make_float4(c.p[1].x, c.p[1].y, c.p[1].z, c.depth[1]);
    if (c.count > 2) out.p2[idx] = make_float4(c.p[2].x, c.p[2].y, c.p[2].z, c.depth[2]);
    if (c.count > 3) out.p3[idx] = make_float4(c.p[3].x, c.p[3].y, c.p[3].z, c.depth[3]);
}

// Block-aggregated append of one manifold per thread with hit; every thread of the block
// calls it (threads without a hit pass hit = false).
__device__ __forceinline__ void appendManifold(bool hit, uint32_t a, uint32_t b, uint32_t dyn,
                                               const Contact& c, const ManifoldOut& out,
                                               DevCounters* cnt, uint32_t& pts) {
    const uint32_t idx = blockReserve(hit ? 1u : 0u, &cnt->manifolds);
    if (hit) writeManifold(idx, a, b, dyn, c, out, pts);
}

// Sphere-sphere pairs, the bulk of most scenes, are collided here with the few registers
// they need; box-box and box-capsule pairs are queued for kGjkPairs (front of the queue)
// and the other analytic pairs for kPairsMixed (back of the queue), so that the general
// shape code's registers and local arrays do not slow the common case.
__global__ void __launch_bounds__(256) kPairs(uint32_t pairCap, const uint2* __restrict__ pairs,
                                              const NarrowBody* __restrict__ nbody, ManifoldOut out,
                                              uint2* __restrict__ queue, uint32_t queueCap,
                                              DevCounters* cnt) {
    // the pair count is read on the device (the sweep's counter; past the capacity only the
    // listed pairs, and the host redoes both stages with room for all)
    const uint32_t nPairs = min(cnt->pairs, pairCap);
    const uint32_t stride = gridDim.x * blockDim.x;
    // uniform trip count: every thread of the block reaches the block-wide appends
    const uint32_t trips = (nPairs + stride - 1) / stride;
    uint32_t pts = 0;
    for (uint32_t t = 0; t < trips; ++t) {
        const uint32_t k = t * stride + blockIdx.x * blockDim.x + threadIdx.x;
        Contact c;
        c.count = 0;
        uint32_t a = 0, b = 0, dyn = 0;
        bool gjkPair = false, mixed = false;
        if (k < nPairs) {
            const uint2 pr = pairs[k];
            a = pr.x;
            b = pr.y;
            const NarrowBody na = nbody[a], nb = nbody[b];
            const uint32_t ia = __float_as_uint(na.s.w), ib = __float_as_uint(nb.s.w);
            const uint32_t sa = (ia >> 4) & 0xFu, sb = (ib >> 4) & 0xFu;
            dyn = hdrDyn(ia, ib);
            if (sa == AXIOM_SHAPE_SPHERE && sb == AXIOM_SHAPE_SPHERE) {
                sphereSphere(axd::mk(na.p), na.s.x, axd::mk(nb.p), nb.s.x, &c, na.p.w + nb.p.w);
            } else if (isGjkPair(sa, sb)) {
                gjkPair = true;
            } else {
                mixed = true;
            }
        }
        // one pass reserves the GJK queue, the mixed queue and the manifold slots
        const bool hit = c.count > 0;
        const uint3 at = blockReserve3(gjkPair ? 1u : 0u, mixed ? 1u : 0u, hit ? 1u : 0u, &cnt->gjkPairs,
                                       &cnt->mixedPairs, &cnt->manifolds);
        if (gjkPair) queue[at.x] = make_uint2(a, b);
        if (mixed) queue[queueCap - 1u - at.y] = make_uint2(a, b);
        if (hit) writeManifold(at.z, a, b, dyn, c, out, pts);
    }
    blockReserve(pts, &cnt->points);
}

// The queued analytic pairs that are not sphere-sphere (sphere-box, sphere-capsule,
// capsule-capsule, sphere-cylinder).  The queue length is read on the device; every CTA sees the same.
__global__ void __launch_bounds__(256) kPairsMixed(const uint2* __restrict__ queue, uint32_t queueCap,
                                                   const uint32_t* __restrict__ info,
                                                   const float4* __restrict__ pos,
                                                   const float4* __restrict__ rot,
                                                   const float4* __restrict__ shp, ManifoldOut out,
                                                   DevCounters* cnt) {
    const uint32_t n = cnt->mixedPairs;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t trips = (n + stride - 1) / stride;
    uint32_t pts = 0;
    for (uint32_t t = 0; t < trips; ++t) {
        const uint32_t k = t * stride + blockIdx.x * blockDim.x + threadIdx.x;
        Contact c;
        c.count = 0;
        uint32_t a = 0, b = 0, dyn = 0;
        if (k < n) {
            const uint2 pr = queue[queueCap - 1u - k];
            a = pr.x;
            b = pr.y;
            const uint32_t ia = info[a], ib = info[b];
            const uint32_t sa = (ia >> 4) & 0xFu, sb = (ib >> 4) & 0xFu;
            dyn = hdrDyn(ia, ib);
            const Geom ga{sa, pos[a], shapeRot(rot, a, sa), shp[a]};
            const Geom gb{sb, pos[b], shapeRot(rot, b, sb), shp[b]};
            collidePair(ga, gb, &c);
        }
        appendManifold(c.count > 0, a, b, dyn, c, out, cnt, pts);
    }
    blockReserve(pts, &cnt->points);
}

// Plane contacts of every dynamic body.  Spheres, the bulk of most scenes, are tested here
// with the few registers a sphere needs; the other shapes are queued (the GJK queue is
// free again by now) for kPlanesMixed, so that the general shape code's registers do not
// slow the common case.  Each body meets every plane twice: first to count its manifolds
// (one block-wide reservation for all planes and the queue), then to write them (same
// inputs, same contacts).
__global__ void __launch_bounds__(256) kPlanes(uint32_t n, uint32_t nPlanes, const uint32_t* __restrict__ planes,
                                               const uint32_t* __restrict__ info, const float4* __restrict__ pos,
                                               const float4* __restrict__ rot, const float4* __restrict__ shp,
                                               const uint4* __restrict__ filt, uint2* __restrict__ queue,
                                               ManifoldOut out, DevCounters* cnt) {
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t trips = (n + stride - 1) / stride;
    uint32_t pts = 0;
    for (uint32_t t = 0; t < trips; ++t) {
        const uint32_t i = t * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool sphere = false, other = false, filtered = false;
        float4 ps = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float r = 0.0f;
        if (i < n) {
            const uint32_t inf = info[i];
            const uint32_t shape = (inf >> 4) & 0xFu;
            const bool body = (inf & kInfoTypeMask) == AXIOM_BODY_DYNAMIC && shape != AXIOM_SHAPE_PLANE;
            sphere = body && shape == AXIOM_SHAPE_SPHERE;
            other = body && !sphere;
            filtered = (inf & kInfoFiltered) != 0u;
            if (sphere) {
                ps = pos[i];  // centre and the sweep (planes do not move)
                r = shp[i].x;
            }
        }
        uint32_t hits = 0;
        uint3 at = make_uint3(0u, 0u, 0u);
        for (uint32_t pass = 0; pass < 2; ++pass) {
            if (pass == 1) at = blockReserve3(other ? 1u : 0u, 0u, hits, &cnt->planeQueue, &cnt->planeQueue,
                                              &cnt->manifolds);
            if (!sphere || (pass == 1 && hits == 0)) continue;
            for (uint32_t q = 0; q < nPlanes; ++q) {
                Contact c;
                c.count = 0;
                const uint32_t p = planes[q];
                bool admit = true;
                if (filtered || (info[p] & kInfoFiltered)) admit = filterPass(filt[p], filt[i]);
                if (admit) {
                    const float4 pp = pos[p];
                    const f3 np = rotate(rot[p], f3{0.0f, 1.0f, 0.0f});
                    spherePlaneAppend(f3{pp.x, pp.y, pp.z}, np, axd::mk(ps), r, &c, ps.w);
                }
                if (c.count == 0) continue;
                if (pass == 0) ++hits;
                else writeManifold(at.z++, p, i, kHdrDynB, c, out, pts);
            }
        }
        if (other) queue[at.x] = make_uint2(i, 0u);
    }
    blockReserve(pts, &cnt->points);
}

// Plane contacts of the queued dynamic bodies that are not spheres (the queue length is
// read on the device), against every plane.
__global__ void __launch_bounds__(256) kPlanesMixed(uint32_t nPlanes, const uint32_t* __restrict__ planes,
                                                    const uint2* __restrict__ queue,
                                                    const uint32_t* __restrict__ info,
                                                    const float4* __restrict__ pos, const float4* __restrict__ rot,
                                                    const float4* __restrict__ shp, const uint4* __restrict__ filt,
                                                    const float4* __restrict__ hullVerts, ManifoldOut out,
                                                    DevCounters* cnt) {
    const uint32_t nq = cnt->planeQueue;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t trips = (nq + stride - 1) / stride;
    uint32_t pts = 0;
    for (uint32_t t = 0; t < trips; ++t) {
        const uint32_t k = t * stride + blockIdx.x * blockDim.x + threadIdx.x;
        const bool body = k < nq;
        const uint32_t i = body ? queue[k].x : 0u;
        bool filtered = false;
        Geom gi{};
        if (body) {
            const uint32_t inf = info[i];
            const uint32_t shape = (inf >> 4) & 0xFu;
            filtered = (inf & kInfoFiltered) != 0u;
            gi = Geom{shape, pos[i], shapeRot(rot, i, shape), shp[i], hullVerts};
        }
        uint32_t hits = 0, at = 0;
        for (uint32_t pass = 0; pass < 2; ++pass) {
            if (pass == 1) at = blockReserve(hits, &cnt->manifolds);
            if (!body || (pass == 1 && hits == 0)) continue;
            for (uint32_t q = 0; q < nPlanes; ++q) {
                Contact c;
                c.count = 0;
                const uint32_t p = planes[q];
                bool admit = true;
                if (filtered || (info[p] & kInfoFiltered)) admit = filterPass(filt[p], filt[i]);
                if (admit) {
                    const float4 pp = pos[p];
                    const f3 np = rotate(rot[p], f3{0.0f, 1.0f, 0.0f});
                    collidePlane(f3{pp.x, pp.y, pp.z}, np, gi, &c);
                }
                if (c.count == 0) continue;
                if (pass == 0) ++hits;
                else writeManifold(at++, p, i, kHdrDynB, c, out, pts);
            }
        }
    }
    blockReserve(pts, &cnt->points);
}

constexpr int kGjkWarps = 4;

// The queued GJK pairs, up to 32 to a warp: GJK and the manifold per lane, EPA per warp
// (lanePairs); box-box and box-capsule with their shapes fixed at compile time.
__global__ void __launch_bounds__(32 * kGjkWarps) kGjkPairs(const uint2* __restrict__ queue,
                                                             const uint32_t* __restrict__ info,
                                                             const float4* __restrict__ pos,
                                                             const float4* __restrict__ rot,
                                                             const float4* __restrict__ shp,
                                                             const float4* __restrict__ hullVerts, ManifoldOut out,
                                                             DevCounters* cnt) {
    __shared__ EpaWarp ws[kGjkWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t count = cnt->gjkPairs;
    // pairs per warp: spread over every warp of the grid first, up to 32 when there are more
    const uint32_t warps = gridDim.x * kGjkWarps;
    const uint32_t per = min(32u, max(1u, (count + warps - 1u) / warps));
    for (uint32_t q0 = (blockIdx.x * kGjkWarps + warp) * per; q0 < count; q0 += warps * per) {
        const uint32_t q = q0 + lane;
        const bool active = (uint32_t)lane < per && q < count;
        uint32_t a = 0, b = 0, ia = 0, ib = 0, kind = kPairGeneric;
        bool flip = false;
        Geom ga{}, gb{};
        if (active) {
            const uint2 pr = queue[q];
            a = pr.x;
            b = pr.y;
            ia = info[a];
            ib = info[b];
            const uint32_t sa = (ia >> 4) & 0xFu, sb = (ib >> 4) & 0xFu;
            ga = Geom{sa, pos[a], shapeRot(rot, a, sa), shp[a], hullVerts};
            gb = Geom{sb, pos[b], shapeRot(rot, b, sb), shp[b], hullVerts};
            const bool boxBox = sa == AXIOM_SHAPE_BOX && sb == AXIOM_SHAPE_BOX;
            const bool boxCap = (sa == AXIOM_SHAPE_BOX && sb == AXIOM_SHAPE_CAPSULE) ||
                                (sa == AXIOM_SHAPE_CAPSULE && sb == AXIOM_SHAPE_BOX);
            flip = boxCap && sa == AXIOM_SHAPE_CAPSULE;  // (capsule, box): box goes first
            kind = boxBox ? kPairBoxBox : (boxCap ? kPairBoxCapsule : kPairGeneric);
        }
        uint32_t fail = 0;
        Contact c = lanePairs(active, kind, flip ? gb : ga, flip ? ga : gb, ws[warp], lane, &fail);
        if (flip) c.n = neg3(c.n);
        const unsigned gf = __ballot_sync(0xFFFFFFFFu, (fail & kFailGjk) != 0u);
        const unsigned ef = __ballot_sync(0xFFFFFFFFu, (fail & kFailEpa) != 0u);
        if (lane == 0 && gf) atomicAdd(&cnt->gjkFailures, (uint32_t)__popc(gf));
        if (lane == 0 && ef) atomicAdd(&cnt->epaFailures, (uint32_t)__popc(ef));
        // one reservation per warp for its manifolds and points
        const bool hit = c.count > 0;
        const unsigned hits = __ballot_sync(0xFFFFFFFFu, hit);
        uint32_t pts = hit ? c.count : 0u;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) pts += __shfl_xor_sync(0xFFFFFFFFu, pts, off);
        uint32_t base = 0;
        if (lane == 0 && hits) {
            base = atomicAdd(&cnt->manifolds, (uint32_t)__popc(hits));
            atomicAdd(&cnt->points, pts);
        }
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (hit) {
            const uint32_t idx = base + (uint32_t)__popc(hits & ((1u << lane) - 1u));
            uint32_t unused = 0;
            writeManifold(idx, a, b, hdrDyn(ia, ib), c, out, unused);
        }
    }
}

}  // namespace

// The pair count stays on the device: grids are sized for `expected` pairs (the host's
// estimate; the kernels stride over whatever the sweep listed), and idle CTAs exit at once.
void launchNarrowphase(World& w, const StepParams&, uint32_t expected) {
    ManifoldOut out{w.mhdr.p, w.mn.p, w.mp[0].p, w.mp[1].p, w.mp[2].p, w.mp[3].p, (uint32_t)w.mhdr.cap};
    const unsigned blocks = 152u * 8u;
    ProfRange pr(w, KG_NARROWPHASE);
    w.prof.launches[KG_NARROWPHASE] += 3 + (w.nPlanes ? 2 : 0);
    const uint32_t est = std::max<uint32_t>(expected, 1u);
    const uint32_t queueCap = (uint32_t)w.gjkQueue.cap;
    kPairs<<<min(gridFor(est, 256), blocks * 4u), 256, 0, w.stream>>>(
        (uint32_t)w.pairs.cap, w.pairs.p, w.nbody.p, out, w.gjkQueue.p, queueCap, w.dcnt);
    kPairsMixed<<<min(gridFor(est, 256), 152u * 4u), 256, 0, w.stream>>>(
        w.gjkQueue.p, queueCap, w.info.p, w.pos.p, w.rot.p, w.shp.p, out, w.dcnt);
    kGjkPairs<<<min(gridFor(est, 32u * kGjkWarps), 152u * 4u), 32 * kGjkWarps, 0, w.stream>>>(
        w.gjkQueue.p, w.info.p, w.pos.p, w.rot.p, w.shp.p, w.hullVerts.p, out, w.dcnt);
    if (w.nPlanes) {
        kPlanes<<<min(gridFor(w.n, 256), blocks * 4u), 256, 0, w.stream>>>(
            w.n, w.nPlanes, w.planes.p, w.info.p, w.pos.p, w.rot.p, w.shp.p, w.filt.p, w.gjkQueue.p, out, w.dcnt);
        kPlanesMixed<<<min(gridFor(w.n, 256), 152u * 4u), 256, 0, w.stream>>>(
            w.nPlanes, w.planes.p, w.gjkQueue.p, w.info.p, w.pos.p, w.rot.p, w.shp.p, w.filt.p, w.hullVerts.p, out,
            w.dcnt);
    }
}

}  // namespace axiom_gb300
