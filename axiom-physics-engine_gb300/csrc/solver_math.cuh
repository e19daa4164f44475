// solver_math.cuh — per-manifold PGS arithmetic shared by the single-world kernels
// (solver.cu) and the batched-world kernel (batch.cu), so both evaluate the same fp32
// expressions in the same order.  The rows, bias, clamps and residual are described in
// solver.cu.
#pragma once

#include "dmath.cuh"
#include "world.h"

namespace axiom_gb300 {

using namespace axd;

constexpr uint32_t kFlagDynA = 1u, kFlagDynB = 2u, kFlagAnisoA = 4u, kFlagAnisoB = 8u;

// Element k (< 4) of a per-slot pointer array, indexed only with constants: a runtime
// index into a kernel-parameter array would copy the array to local memory.
template <typename T>
__device__ __forceinline__ T* slot4(T* const (&arr)[kMaxPoints], uint32_t k) {
    return k == 0 ? arr[0] : (k == 1 ? arr[1] : (k == 2 ? arr[2] : arr[3]));
}

struct SolverPtrs {
    uint4* hdr;
    float4* n;
    float4* ra[kMaxPoints];
    float4* rb[kMaxPoints];
    float2* kt[kMaxPoints];
    float4* lam[kMaxPoints];
};

__device__ __forceinline__ f3 applyInvI(float4 w, float4 i0, float4 i1, bool aniso, f3 v) {
    if (!aniso) return f3{w.w * v.x, w.w * v.y, w.w * v.z};
    return mulSym(i0, i1, v);
}

__device__ __forceinline__ uint64_t warmKey(uint32_t a, uint32_t b, uint32_t k) {
    return pairKey(a, b) * 4ull + k;
}
__device__ __forceinline__ uint32_t warmHash(uint64_t key, uint32_t log2T) {
    return (uint32_t)((mix64(key) * 0x9E3779B97F4A7C15ull) >> (64u - log2T));
}

// Inserts (key, tag, val) into a tagged warm-start table at generation gen: a slot is
// taken by raising its claim to gen with one atomic max, which returns an older generation
// to exactly one thread (generations only grow between the table's clears, and keys are
// distinct within one generation, so a slot already claimed at gen holds another key);
// the taker then writes the slot's whole sector.  False when the table is full.
__device__ __forceinline__ bool warmInsert(WarmSlot* __restrict__ slots, uint32_t* __restrict__ claim,
                                           uint32_t log2T, uint32_t gen, unsigned long long key, uint32_t tag,
                                           float4 val) {
    const uint32_t mask = (1u << log2T) - 1u;
    uint32_t hh = warmHash(key, log2T);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        if (atomicMax(&claim[hh], gen) != gen) {
            uint4* sl = reinterpret_cast<uint4*>(slots + hh);
            sl[0] = make_uint4((uint32_t)key, (uint32_t)(key >> 32), gen, tag);
            sl[1] = make_uint4(__float_as_uint(val.x), __float_as_uint(val.y), __float_as_uint(val.z),
                               __float_as_uint(val.w));
            return true;
        }
        hh = (hh + 1u) & mask;
    }
    return false;
}

// Velocities of one body of a manifold.  The world inverse inertia of an anisotropic body
// is fetched where it is applied (it is read-only during the solve and stays in L1), so
// that the point loop keeps 16 fewer live registers per body.
struct BodyState {
    float4 v, w;
    uint32_t id;
};

struct InvInertia {
    const float4* __restrict__ i0;
    const float4* __restrict__ i1;
};

__device__ __forceinline__ f3 applyInvI(const BodyState& S, const InvInertia& I, bool aniso, f3 v) {
    if (!aniso) return f3{S.w.w * v.x, S.w.w * v.y, S.w.w * v.z};
    return mulSym(__ldg(&I.i0[S.id]), __ldg(&I.i1[S.id]), v);
}

__device__ __forceinline__ void applyImpulse(uint32_t flags, BodyState& A, BodyState& B, const InvInertia& I,
                                             f3 rA, f3 rB, f3 P) {
    if (flags & kFlagDynA) {
        const float m = A.v.w;
        A.v.x = A.v.x - m * P.x;
        A.v.y = A.v.y - m * P.y;
        A.v.z = A.v.z - m * P.z;
        const f3 dw = applyInvI(A, I, (flags & kFlagAnisoA) != 0u, cross(rA, P));
        A.w.x = A.w.x - dw.x;
        A.w.y = A.w.y - dw.y;
        A.w.z = A.w.z - dw.z;
    }
    if (flags & kFlagDynB) {
        const float m = B.v.w;
        B.v.x = B.v.x + m * P.x;
        B.v.y = B.v.y + m * P.y;
        B.v.z = B.v.z + m * P.z;
        const f3 dw = applyInvI(B, I, (flags & kFlagAnisoB) != 0u, cross(rB, P));
        B.w.x = B.w.x + dw.x;
        B.w.y = B.w.y + dw.y;
        B.w.z = B.w.z + dw.z;
    }
}

__device__ __forceinline__ f3 relVel(const BodyState& A, const BodyState& B, f3 rA, f3 rB) {
    const f3 va = add(f3{A.v.x, A.v.y, A.v.z}, cross(f3{A.w.x, A.w.y, A.w.z}, rA));
    const f3 vb = add(f3{B.v.x, B.v.y, B.v.z}, cross(f3{B.w.x, B.w.y, B.w.z}, rB));
    return sub(vb, va);
}

__device__ __forceinline__ void loadBodies(uint32_t a, uint32_t b, const SolverBody* sb, BodyState& A,
                                           BodyState& B) {
    A.v = sb[a].v;
    A.w = sb[a].w;
    A.id = a;
    B.v = sb[b].v;
    B.w = sb[b].w;
    B.id = b;
}

__device__ __forceinline__ void storeBodies(uint32_t a, uint32_t b, uint32_t flags, SolverBody* sb,
                                            const BodyState& A, const BodyState& B) {
    if (flags & kFlagDynA) {
        sb[a].v = A.v;
        sb[a].w = A.w;
    }
    if (flags & kFlagDynB) {
        sb[b].v = B.v;
        sb[b].w = B.w;
    }
}

// Solver constants of manifold m at colour-order position s (rA, rB, effective masses,
// bias, friction), its starting impulses and, when in.feat is set, the network features
// (row slot * nM + s).  Shared by the single-world and the batched step.
struct PrepIn {
    const uint4* mhdr;
    const float4* mn;
    const float4* mp[kMaxPoints];
    const uint32_t* info;
    const float4* pos;
    const SolverBody* sb;
    const float4* iw0;
    const float4* iw1;
    const float4* mat;
    const unsigned long long* wsKeys;  // split table (batched worlds): keys, kEmpty64 = empty
    const float4* wsVals;
    const WarmSlot* wsSlots;  // tagged table (single world), used when set
    const float4* warm0;      // point 0's previous impulses per manifold, found by the colouring (or null)
    uint32_t wsGen;           // the tagged table's current generation
    uint32_t wsLog2, lookup, usePrev;
    float* feat;
    uint32_t hdrDyn;  // mhdr.w carries the dynamic bits (single-world narrowphase): no info gathers
};

__device__ __forceinline__ void prepareManifold(uint32_t s, uint32_t m, uint32_t nM, const StepParams& sp,
                                                const PrepIn& in, SolverPtrs out) {
    const uint4* __restrict__ mhdr = in.mhdr;
    const float4* __restrict__ mn = in.mn;
    const float4* mp0 = in.mp[0];
    const float4* mp1 = in.mp[1];
    const float4* mp2 = in.mp[2];
    const float4* mp3 = in.mp[3];
    const uint32_t* __restrict__ info = in.info;
    const float4* __restrict__ pos = in.pos;
    const SolverBody* __restrict__ sb = in.sb;
    const float4* __restrict__ iw0 = in.iw0;
    const float4* __restrict__ iw1 = in.iw1;
    const float4* __restrict__ mat = in.mat;
    const unsigned long long* __restrict__ wsKeys = in.wsKeys;
    const float4* __restrict__ wsVals = in.wsVals;
    const uint32_t wsLog2 = in.wsLog2, lookup = in.lookup, usePrev = in.usePrev;
    float* __restrict__ feat = in.feat;
    const uint4 h = mhdr[m];
    const uint32_t a = h.x, b = h.y, npts = h.z;
    const bool dA = in.hdrDyn ? (h.w & kHdrDynA) != 0u : (info[a] & kInfoTypeMask) == AXIOM_BODY_DYNAMIC;
    const bool dB = in.hdrDyn ? (h.w & kHdrDynB) != 0u : (info[b] & kInfoTypeMask) == AXIOM_BODY_DYNAMIC;
    const float4 va = sb[a].v, vb = sb[b].v, wa = sb[a].w, wb = sb[b].w;
    const bool anA = dA && wa.w < 0.0f, anB = dB && wb.w < 0.0f;
    const float4 ia0 = anA ? iw0[a] : make_float4(0, 0, 0, 0), ia1 = anA ? iw1[a] : make_float4(0, 0, 0, 0);
    const float4 ib0 = anB ? iw0[b] : make_float4(0, 0, 0, 0), ib1 = anB ? iw1[b] : make_float4(0, 0, 0, 0);
    const float mA = dA ? va.w : 0.0f, mB = dB ? vb.w : 0.0f;
    const float4 matA = mat[a], matB = mat[b];
    const float mu = sqrtf(matA.x * matB.x);
    const float e = maxf(matA.y, matB.y);
    const float4 n4 = mn[m];
    const f3 n{n4.x, n4.y, n4.z};
    f3 t1, t2;
    tangentBasis(n, &t1, &t2);
    const float4 pa = pos[a], pb = pos[b];
    const uint32_t flags = (dA ? kFlagDynA : 0u) | (dB ? kFlagDynB : 0u) | (anA ? kFlagAnisoA : 0u) |
                           (anB ? kFlagAnisoB : 0u);
    out.hdr[s] = make_uint4(a, b, npts, flags);
    out.n[s] = make_float4(n.x, n.y, n.z, mu);
    for (uint32_t k = 0; k < npts; ++k) {
        const float4 p4 = (k == 0 ? mp0 : (k == 1 ? mp1 : (k == 2 ? mp2 : mp3)))[m];
        const f3 rA{p4.x - pa.x, p4.y - pa.y, p4.z - pa.z};
        const f3 rB{p4.x - pb.x, p4.y - pb.y, p4.z - pb.z};
        auto effMass = [&](f3 dir) {
            const f3 ra = cross(rA, dir), rb = cross(rB, dir);
            const float kA = dA ? dot(ra, applyInvI(wa, ia0, ia1, anA, ra)) : 0.0f;
            const float kB = dB ? dot(rb, applyInvI(wb, ib0, ib1, anB, rb)) : 0.0f;
            const float kk = mA + mB + kA + kB;
            return kk > 0.0f ? 1.0f / kk : 0.0f;
        };
        const float kn = effMass(n), kt1 = effMass(t1), kt2 = effMass(t2);
        // touching (depth >= 0): Baumgarte feedback beyond the slop, restitution above the
        // threshold; speculative (depth < 0, a gap): the point may close exactly its gap
        float bias = p4.w >= 0.0f ? sp.biasCoeff * maxf(p4.w - sp.slop, 0.0f) : p4.w * sp.invDt;
        if (e > 0.0f && p4.w >= 0.0f) {
            const f3 vA = add(f3{va.x, va.y, va.z}, cross(f3{wa.x, wa.y, wa.z}, rA));
            const f3 vB = add(f3{vb.x, vb.y, vb.z}, cross(f3{wb.x, wb.y, wb.z}, rB));
            const float vn0 = dot(sub(vB, vA), n);
            if (vn0 < -sp.restThreshold) bias = maxf(bias, -e * vn0);
        }
        // previous-step impulses of this (pair, point)
        float4 prev = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (lookup && k == 0 && in.warm0) {
            prev = in.warm0[m];
        } else if (lookup) {
            const uint64_t key = warmKey(a, b, k);
            const uint32_t mask = (1u << wsLog2) - 1u;
            uint32_t hh = warmHash(key, wsLog2);
            if (in.wsSlots) {
                // one sector per probe: key, generation and impulses together
                for (uint32_t probe = 0; probe <= mask; ++probe) {
                    const WarmSlot* sl = in.wsSlots + hh;
                    const uint4 head = *reinterpret_cast<const uint4*>(sl);
                    if (head.z != in.wsGen) break;
                    if (((unsigned long long)head.y << 32 | head.x) == key) {
                        prev = sl->val;
                        break;
                    }
                    hh = (hh + 1u) & mask;
                }
            } else {
                for (uint32_t probe = 0; probe <= mask; ++probe) {
                    const unsigned long long kk = wsKeys[hh];
                    if (kk == kEmpty64) break;
                    if (kk == key) {
                        prev = wsVals[hh];
                        break;
                    }
                    hh = (hh + 1u) & mask;
                }
            }
        }
        // PREVIOUS starts from factor x prev; LEARNED stores prev itself for kApplyLearned
        float4 lam = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (usePrev == 1u)
            lam = make_float4(prev.x * sp.warmFactor, prev.y * sp.warmFactor, prev.z * sp.warmFactor, 0.0f);
        else if (usePrev == 2u)
            lam = prev;
        if (feat) {
            // warm-start network features (dimensionless; the list is in include/axiom_c.h)
            const f3 vA = add(f3{va.x, va.y, va.z}, cross(f3{wa.x, wa.y, wa.z}, rA));
            const f3 vB = add(f3{vb.x, vb.y, vb.z}, cross(f3{wb.x, wb.y, wb.z}, rB));
            const f3 dv = sub(vB, vA);
            const float vScale = sp.gdt > 0.0f ? 1.0f / sp.gdt : 1.0f;
            const float sImp = kn * sp.gdt;
            const float invImp = sImp > 0.0f ? 1.0f / sImp : 0.0f;
            float* f = feat + ((size_t)k * nM + s) * 16u;
            f[0] = dot(dv, n) * vScale;
            f[1] = dot(dv, t1) * vScale;
            f[2] = dot(dv, t2) * vScale;
            f[3] = n.x;
            f[4] = n.y;
            f[5] = n.z;
            f[6] = sp.slop > 0.0f ? p4.w / sp.slop : p4.w;
            f[7] = mA * kn;
            f[8] = mB * kn;
            f[9] = prev.x * invImp;
            f[10] = prev.y * invImp;
            f[11] = prev.z * invImp;
            f[12] = (mA + mB) * kn;
            f[13] = mu;
            f[14] = sImp;
            f[15] = 1.0f;
        }
        slot4(out.ra, k)[s] = make_float4(rA.x, rA.y, rA.z, kn);
        slot4(out.rb, k)[s] = make_float4(rB.x, rB.y, rB.z, bias);
        slot4(out.kt, k)[s] = make_float2(kt1, kt2);
        slot4(out.lam, k)[s] = lam;
    }
    if (feat)
        for (uint32_t k = npts; k < (uint32_t)kMaxPoints; ++k) {
            float* f = feat + ((size_t)k * nM + s) * 16u;
            for (int j = 0; j < 16; ++j) f[j] = 0.0f;
        }
}

// The coalesced part of a manifold's solver data: header, normal and the constants and
// impulses of point slot 0 (every manifold has a point there).  It does not depend on
// the bodies, so a loop can fetch the next manifold's head while it solves this one.
struct ManifoldHead {
    uint4 h;
    float4 n4, ra4, rb4, l;
    float2 kt;
};

__device__ __forceinline__ ManifoldHead loadHead(uint32_t s, const SolverPtrs& sv) {
    ManifoldHead m;
    m.h = sv.hdr[s];
    m.n4 = sv.n[s];
    m.ra4 = sv.ra[0][s];
    m.rb4 = sv.rb[0][s];
    m.kt = sv.kt[0][s];
    m.l = sv.lam[0][s];
    return m;
}

// The same with evict-first (streaming) loads: in a world whose solver arrays exceed L2,
// each sweep streams them once, and they should not push the bodies (re-gathered by
// every colour) out of L2.
__device__ __forceinline__ ManifoldHead loadHeadStreaming(uint32_t s, const SolverPtrs& sv) {
    ManifoldHead m;
    m.h = __ldcs(&sv.hdr[s]);
    m.n4 = __ldcs(&sv.n[s]);
    m.ra4 = __ldcs(&sv.ra[0][s]);
    m.rb4 = __ldcs(&sv.rb[0][s]);
    m.kt = __ldcs(&sv.kt[0][s]);
    m.l = __ldcs(&sv.lam[0][s]);
    return m;
}

// The rest of a manifold's head once its header is known (streaming loads).
__device__ __forceinline__ void loadHeadRestStreaming(uint32_t s, const SolverPtrs& sv, ManifoldHead& m) {
    m.n4 = __ldcs(&sv.n[s]);
    m.ra4 = __ldcs(&sv.ra[0][s]);
    m.rb4 = __ldcs(&sv.rb[0][s]);
    m.kt = __ldcs(&sv.kt[0][s]);
    m.l = __ldcs(&sv.lam[0][s]);
}

// Applies the warm-start impulses of manifold s (head hd) to its bodies.
// Applies the warm-start impulses of manifold s (head hd) to its bodies A, B (velocities
// as loaded) and stores them back.
__device__ __forceinline__ void warmWithBodies(uint32_t s, const ManifoldHead& hd, BodyState A, BodyState B,
                                               const SolverPtrs& sv, SolverBody* __restrict__ sb,
                                               const float4* __restrict__ iw0, const float4* __restrict__ iw1) {
    const uint4 h = hd.h;
    const f3 n{hd.n4.x, hd.n4.y, hd.n4.z};
    f3 t1, t2;
    tangentBasis(n, &t1, &t2);
    const InvInertia I{iw0, iw1};
    // unrolled so that the slot index is a constant: the per-slot pointers stay in the
    // parameter bank instead of being copied to a local array for dynamic indexing
#pragma unroll
    for (uint32_t k = 0; k < (uint32_t)kMaxPoints; ++k) {
        if (k >= h.z) break;
        float4 ra = hd.ra4, rb = hd.rb4, l = hd.l;
        if (k > 0) {
            ra = sv.ra[k][s];
            rb = sv.rb[k][s];
            l = sv.lam[k][s];
        }
        const f3 P{n.x * l.x + t1.x * l.y + t2.x * l.z, n.y * l.x + t1.y * l.y + t2.y * l.z,
                   n.z * l.x + t1.z * l.y + t2.z * l.z};
        applyImpulse(h.w, A, B, I, f3{ra.x, ra.y, ra.z}, f3{rb.x, rb.y, rb.z}, P);
    }
    storeBodies(h.x, h.y, h.w, sb, A, B);
}

__device__ __forceinline__ void warmHead(uint32_t s, const ManifoldHead& hd, const SolverPtrs& sv,
                                         SolverBody* __restrict__ sb, const float4* __restrict__ iw0,
                                         const float4* __restrict__ iw1) {
    BodyState A, B;
    loadBodies(hd.h.x, hd.h.y, sb, A, B);
    warmWithBodies(s, hd, A, B, sv, sb, iw0, iw1);
}

__device__ __forceinline__ void warmManifold(uint32_t s, const SolverPtrs& sv, SolverBody* __restrict__ sb,
                                             const float4* __restrict__ iw0, const float4* __restrict__ iw1) {
    warmHead(s, loadHead(s, sv), sv, sb, iw0, iw1);
}

// One PGS pass over the points of manifold s whose head is hd; folds its max |dλ| and
// max |λ| into gd, gl.
// The bodies A, B (velocities as loaded) are given; they are stored back at the end.
// kStream: impulses and slots 1-3 move with streaming (evict-first) accesses.
// kHoist: the rows of points 1-3 are all loaded before the first point is solved (42 more
// live registers); otherwise each point's rows are loaded after the previous point's
// impulse store, which the compiler may not move them across, so that a four-point
// manifold waits three memory round trips inside its point loop.
template <bool kStream = false, bool kHoist = false>
__device__ __forceinline__ void solveWithBodies(uint32_t s, const ManifoldHead& hd, BodyState A, BodyState B,
                                                const SolverPtrs& sv, SolverBody* __restrict__ sb,
                                                const float4* __restrict__ iw0, const float4* __restrict__ iw1,
                                                float& gd, float& gl) {
    const uint4 h = hd.h;
    const float4 n4 = hd.n4;
    float4 ra4 = hd.ra4, rb4 = hd.rb4;
    float2 kt = hd.kt;
    float4 l = hd.l;
    float4 hra[kMaxPoints - 1], hrb[kMaxPoints - 1], hl[kMaxPoints - 1];
    float2 hkt[kMaxPoints - 1];
    if (kHoist) {
#pragma unroll
        for (uint32_t k = 1; k < (uint32_t)kMaxPoints; ++k) {
            if (k >= h.z) break;
            hra[k - 1] = kStream ? __ldcs(&sv.ra[k][s]) : sv.ra[k][s];
            hrb[k - 1] = kStream ? __ldcs(&sv.rb[k][s]) : sv.rb[k][s];
            hkt[k - 1] = kStream ? __ldcs(&sv.kt[k][s]) : sv.kt[k][s];
            hl[k - 1] = kStream ? __ldcs(&sv.lam[k][s]) : sv.lam[k][s];
        }
    }
    const f3 n{n4.x, n4.y, n4.z};
    const float mu = n4.w;
    f3 t1, t2;
    tangentBasis(n, &t1, &t2);
    const InvInertia I{iw0, iw1};
#pragma unroll
    for (uint32_t k = 0; k < (uint32_t)kMaxPoints; ++k) {
        if (k >= h.z) break;
        if (k > 0) {
            if (kHoist) {
                ra4 = hra[k - 1];
                rb4 = hrb[k - 1];
                kt = hkt[k - 1];
                l = hl[k - 1];
            } else if (kStream) {
                ra4 = __ldcs(&sv.ra[k][s]);
                rb4 = __ldcs(&sv.rb[k][s]);
                kt = __ldcs(&sv.kt[k][s]);
                l = __ldcs(&sv.lam[k][s]);
            } else {
                ra4 = sv.ra[k][s];
                rb4 = sv.rb[k][s];
                kt = sv.kt[k][s];
                l = sv.lam[k][s];
            }
        }
        const f3 rA{ra4.x, ra4.y, ra4.z}, rB{rb4.x, rb4.y, rb4.z};
        // normal row
        f3 dv = relVel(A, B, rA, rB);
        const float vn = dot(dv, n);
        const float lnOld = l.x;
        float ln = lnOld + ra4.w * (rb4.w - vn);
        ln = ln > 0.0f ? ln : 0.0f;
        const float dn = ln - lnOld;
        l.x = ln;
        applyImpulse(h.w, A, B, I, rA, rB, scale(n, dn));
        // friction rows
        dv = relVel(A, B, rA, rB);
        const float vt1 = dot(dv, t1), vt2 = dot(dv, t2);
        const float maxF = mu * ln;
        float l1 = l.y - kt.x * vt1;
        float l2 = l.z - kt.y * vt2;
        l1 = l1 > maxF ? maxF : (l1 < -maxF ? -maxF : l1);
        l2 = l2 > maxF ? maxF : (l2 < -maxF ? -maxF : l2);
        const float d1 = l1 - l.y, d2 = l2 - l.z;
        l.y = l1;
        l.z = l2;
        const f3 P{t1.x * d1 + t2.x * d2, t1.y * d1 + t2.y * d2, t1.z * d1 + t2.z * d2};
        applyImpulse(h.w, A, B, I, rA, rB, P);
        if (kStream) __stcs(&sv.lam[k][s], l);
        else sv.lam[k][s] = l;
        gd = maxf(gd, maxf(fabsf(dn), maxf(fabsf(d1), fabsf(d2))));
        gl = maxf(gl, maxf(fabsf(ln), maxf(fabsf(l1), fabsf(l2))));
    }
    storeBodies(h.x, h.y, h.w, sb, A, B);
}

template <bool kStream = false, bool kHoist = false>
__device__ __forceinline__ void solveHead(uint32_t s, const ManifoldHead& hd, const SolverPtrs& sv,
                                          SolverBody* __restrict__ sb, const float4* __restrict__ iw0,
                                          const float4* __restrict__ iw1, float& gd, float& gl) {
    BodyState A, B;
    loadBodies(hd.h.x, hd.h.y, sb, A, B);
    solveWithBodies<kStream, kHoist>(s, hd, A, B, sv, sb, iw0, iw1, gd, gl);
}

// One PGS pass over the points of manifold s; folds its max |dλ| and max |λ| into gd, gl.
__device__ __forceinline__ void solveManifold(uint32_t s, const SolverPtrs& sv, SolverBody* __restrict__ sb,
                                              const float4* __restrict__ iw0, const float4* __restrict__ iw1,
                                              float& gd, float& gl) {
    solveHead(s, loadHead(s, sv), sv, sb, iw0, iw1, gd, gl);
}

}  // namespace axiom_gb300
