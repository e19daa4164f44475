// gjk_epa.cuh — warp-per-pair GJK + EPA for box-box, box-capsule and the pairs with a
// cylinder or a convex hull (device).
//
// Boolean GJK (Gilbert, Johnson, Keerthi 1988) runs on every lane of the warp with the
// same data, so control flow stays uniform; it returns a tetrahedron holding the origin
// of the Minkowski difference.  The expanding polytope algorithm (van den Bergen 2001)
// keeps its polytope in the warp's shared memory: lanes split the closest-face search
// (arg-min with the lowest index on ties), the visibility test and the construction of
// the new faces; lane 0 alone edits the face list and the horizon so that faces keep a
// fixed order; the visibility scan and the compaction of the kept faces are lane-parallel
// (ballot prefix sums), so lane 0 only walks the few visible faces.  The manifold then comes from clipping the incident face against the
// reference face (Sutherland-Hodgman), or from one EPA witness point for edge contacts.
//
// Iteration caps (GJK 32, EPA 32) and polytope caps (40 vertices, 80 faces) bound every
// loop; a pair whose EPA stops on a cap keeps its best face so far.
#pragma once

#include <cfloat>

#include "narrow_shapes.cuh"

namespace axiom_gb300 {

constexpr int kGjkMaxIter = 32;
// convergence failures of a pair (lanePairs), counted per step
constexpr uint32_t kFailGjk = 1u, kFailEpa = 2u;
constexpr int kEpaMaxIter = 32;
constexpr int kEpaMaxVerts = 40;
constexpr int kEpaMaxFaces = 80;
constexpr float kEpaTolerance = 1e-4f;
constexpr float kFaceContactAlign = 0.9995f;
constexpr float kCapsuleParallel = 0.1f;

struct SupportPt {
    axd::f3 w, a, b;
};

// Index of the hull vertex (body frame) farthest along dl; the lowest index on ties.
__device__ __forceinline__ uint32_t hullSupportIndex(const Geom& g, axd::f3 dl) {
    using namespace axd;
    const float4* v = g.verts + hullOffset(g);
    const uint32_t n = hullCount(g);
    uint32_t bi = 0;
    float best = dot(mk(v[0]), dl);
    for (uint32_t i = 1; i < n; ++i) {
        const float t = dot(mk(v[i]), dl);
        if (t > best) {
            best = t;
            bi = i;
        }
    }
    return bi;
}

// Support point of g along d.  kShape >= 0 names g's shape at compile time (the pair
// kernels' box-box and box-capsule paths), so that only that shape's branch is compiled
// into their loops; kShape < 0 dispatches on g.shape.  Either way the same expressions run.
constexpr int kAnyShape = -1;

template <int kShape = kAnyShape>
__device__ __forceinline__ axd::f3 supportShape(const Geom& g, axd::f3 d) {
    using namespace axd;
    if (kShape == (int)AXIOM_SHAPE_BOX || (kShape < 0 && g.shape == AXIOM_SHAPE_BOX)) {
        const f3 dl = rotateInv(g.rot, d);
        const f3 vl{dl.x >= 0.0f ? g.ext.x : -g.ext.x, dl.y >= 0.0f ? g.ext.y : -g.ext.y,
                    dl.z >= 0.0f ? g.ext.z : -g.ext.z};
        return add(mk(g.pos), rotate(g.rot, vl));
    }
    if (kShape < 0 && isHullShape(g.shape)) {
        const f3 dl = rotateInv(g.rot, d);
        return add(mk(g.pos), rotate(g.rot, mk(g.verts[hullOffset(g) + hullSupportIndex(g, dl)])));
    }
    if (kShape < 0 && g.shape == AXIOM_SHAPE_SPHERE) {
        const float len = sqrtf(dot(d, d));
        if (!(len > 0.0f)) return mk(g.pos);
        const float k = g.ext.x / len;
        return f3{g.pos.x + d.x * k, g.pos.y + d.y * k, g.pos.z + d.z * k};
    }
    if (kShape < 0 && g.shape == AXIOM_SHAPE_CYLINDER) {
        // cap centre on the side of d, then the rim point in d's direction across the axis
        const f3 u = rotate(g.rot, f3{0.0f, 1.0f, 0.0f});
        const f3 ax = rotate(g.rot, f3{0.0f, g.ext.y, 0.0f});
        const f3 base = dot(d, ax) >= 0.0f ? add(mk(g.pos), ax) : sub(mk(g.pos), ax);
        const float du = dot(d, u);
        const f3 dp{d.x - u.x * du, d.y - u.y * du, d.z - u.z * du};
        const float len = sqrtf(dot(dp, dp));
        if (!(len > 0.0f)) return base;
        const float k = g.ext.x / len;
        return f3{base.x + dp.x * k, base.y + dp.y * k, base.z + dp.z * k};
    }
    const f3 ax = rotate(g.rot, f3{0.0f, g.ext.y, 0.0f});
    const f3 base = dot(d, ax) >= 0.0f ? add(mk(g.pos), ax) : sub(mk(g.pos), ax);
    const float len = sqrtf(dot(d, d));
    if (!(len > 0.0f)) return base;
    const float k = g.ext.x / len;
    return f3{base.x + d.x * k, base.y + d.y * k, base.z + d.z * k};
}

template <int KA = kAnyShape, int KB = kAnyShape>
__device__ __forceinline__ SupportPt minkowski(const Geom& A, const Geom& B, axd::f3 d) {
    SupportPt s;
    s.a = supportShape<KA>(A, d);
    if (A.margin > 0.0f) {  // A inflated by a sphere of radius margin
        const float len = sqrtf(axd::dot(d, d));
        if (len > 0.0f) {
            const float k = A.margin / len;
            s.a = axd::f3{s.a.x + d.x * k, s.a.y + d.y * k, s.a.z + d.z * k};
        }
    }
    s.b = supportShape<KB>(B, neg3(d));
    s.w = axd::sub(s.a, s.b);
    return s;
}

__device__ __forceinline__ bool sameDir(axd::f3 a, axd::f3 b) { return axd::dot(a, b) > 0.0f; }

// Search direction from segment ab towards the origin ao: (ab x ao) x ab.  When the
// origin lies on the segment's line this is the zero vector, and a zero direction would
// end GJK with "no contact" (two identical boxes stacked exactly on one axis do this);
// any normal of ab then serves, taken against the axis where ab is smallest.
__device__ __forceinline__ axd::f3 lineDir(axd::f3 ab, axd::f3 ao) {
    using namespace axd;
    f3 d = cross(cross(ab, ao), ab);
    if (d.x == 0.0f && d.y == 0.0f && d.z == 0.0f) {
        const float x = fabsf(ab.x), y = fabsf(ab.y), z = fabsf(ab.z);
        const f3 e = (x <= y && x <= z) ? f3{1.0f, 0.0f, 0.0f} : (y <= z ? f3{0.0f, 1.0f, 0.0f} : f3{0.0f, 0.0f, 1.0f});
        d = cross(ab, e);
    }
    return d;
}

// Line case of GJK on (sx[0], sx[1]).
__device__ __forceinline__ void gjkLine(SupportPt* sx, int* n, axd::f3* d) {
    using namespace axd;
    const f3 a = sx[0].w, ao = neg3(a);
    const f3 ab = sub(sx[1].w, a);
    *n = 2;
    if (sameDir(ab, ao)) {
        *d = lineDir(ab, ao);
    } else {
        *n = 1;
        *d = ao;
    }
}

// Boolean GJK.  On true, sx[0..3] is a tetrahedron holding the origin.  *exhausted is set
// when the iterations ran out without a decision (reported as separated).
template <int KA = kAnyShape, int KB = kAnyShape>
__device__ __forceinline__ bool gjk(const Geom& A, const Geom& B, SupportPt sx[4], bool* exhausted) {
    using namespace axd;
    *exhausted = false;
    f3 d = sub(mk(B.pos), mk(A.pos));
    if (!(dot(d, d) > 0.0f)) d = f3{1.0f, 0.0f, 0.0f};
    sx[0] = minkowski<KA, KB>(A, B, d);
    int n = 1;
    d = neg3(sx[0].w);
    for (int it = 0; it < kGjkMaxIter; ++it) {
        const SupportPt s = minkowski<KA, KB>(A, B, d);
        if (dot(s.w, d) <= 0.0f) return false;
        for (int k = n; k > 0; --k) sx[k] = sx[k - 1];
        sx[0] = s;
        ++n;
        const f3 a = sx[0].w, ao = neg3(a);
        if (n == 2) {
            gjkLine(sx, &n, &d);
        } else if (n == 3) {
            const f3 ab = sub(sx[1].w, a), ac = sub(sx[2].w, a);
            const f3 abc = cross(ab, ac);
            if (sameDir(cross(abc, ac), ao)) {
                if (sameDir(ac, ao)) {
                    sx[1] = sx[2];
                    n = 2;
                    d = lineDir(ac, ao);
                } else {
                    gjkLine(sx, &n, &d);
                }
            } else if (sameDir(cross(ab, abc), ao)) {
                gjkLine(sx, &n, &d);
            } else if (sameDir(abc, ao)) {
                d = abc;
            } else {
                const SupportPt t = sx[1];
                sx[1] = sx[2];
                sx[2] = t;
                d = neg3(abc);
            }
        } else {
            const f3 ab = sub(sx[1].w, a), ac = sub(sx[2].w, a), ad = sub(sx[3].w, a);
            const f3 abc = cross(ab, ac), acd = cross(ac, ad), adb = cross(ad, ab);
            int face = -1;
            if (sameDir(abc, ao)) face = 0;
            else if (sameDir(acd, ao)) face = 1;
            else if (sameDir(adb, ao)) face = 2;
            if (face < 0) return true;
            const SupportPt p = face == 0 ? sx[1] : (face == 1 ? sx[2] : sx[3]);
            const SupportPt q = face == 0 ? sx[2] : (face == 1 ? sx[3] : sx[1]);
            sx[1] = p;
            sx[2] = q;
            n = 3;
            const f3 tb = sub(sx[1].w, a), tc = sub(sx[2].w, a);
            const f3 tn = cross(tb, tc);
            if (sameDir(cross(tn, tc), ao)) {
                if (sameDir(tc, ao)) {
                    sx[1] = sx[2];
                    n = 2;
                    d = lineDir(tc, ao);
                } else {
                    gjkLine(sx, &n, &d);
                }
            } else if (sameDir(cross(tb, tn), ao)) {
                gjkLine(sx, &n, &d);
            } else {
                d = tn;
            }
        }
    }
    *exhausted = true;
    return false;
}

// Polytope of one warp in shared memory.
struct EpaWarp {
    float4 w[kEpaMaxVerts], a[kEpaMaxVerts], b[kEpaMaxVerts];
    int4 fi[kEpaMaxFaces];    // (i, j, k, -)
    float4 fn[kEpaMaxFaces];  // (n.xyz, dist)
    int2 edges[3 * kEpaMaxFaces];
    int visList[kEpaMaxFaces];  // faces that see the new support point, in face order
    int nv, nf, ne, keep;
};

__device__ __forceinline__ axd::f3 vw(const EpaWarp& s, int i) { return axd::mk(s.w[i]); }

// Face (i, j, k) of the polytope: unit outward normal and distance to the origin.
__device__ __forceinline__ void makeFace(const EpaWarp& s, int i, int j, int k, int4* fi, float4* fn) {
    using namespace axd;
    const f3 nn = cross(sub(vw(s, j), vw(s, i)), sub(vw(s, k), vw(s, i)));
    const float len = sqrtf(dot(nn, nn));
    if (!(len > 0.0f)) {
        *fi = make_int4(i, j, k, 0);
        *fn = make_float4(0.0f, 0.0f, 0.0f, FLT_MAX);
        return;
    }
    f3 n{nn.x / len, nn.y / len, nn.z / len};
    float dist = dot(n, vw(s, i));
    if (dist < 0.0f) {
        n = neg3(n);
        dist = -dist;
        *fi = make_int4(i, k, j, 0);
    } else {
        *fi = make_int4(i, j, k, 0);
    }
    *fn = make_float4(n.x, n.y, n.z, dist);
}

// Closest face: minimum distance, lowest index on ties (= the first minimum).
__device__ __forceinline__ int closestFace(const EpaWarp& s, int lane) {
    float bd = FLT_MAX;
    int bi = 0x7FFFFFFF;
    for (int k = lane; k < s.nf; k += 32) {
        const float d = s.fn[k].w;
        if (d < bd || (d == bd && k < bi)) {
            bd = d;
            bi = k;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float od = __shfl_xor_sync(0xFFFFFFFFu, bd, off);
        const int oi = __shfl_xor_sync(0xFFFFFFFFu, bi, off);
        if (od < bd || (od == bd && oi < bi)) {
            bd = od;
            bi = oi;
        }
    }
    return bi == 0x7FFFFFFF ? 0 : bi;
}

struct EpaResult {
    axd::f3 n;
    float depth;
    axd::f3 pa, pb;
    bool converged;  // stopped at the tolerance (not at a vertex, face or iteration cap)
};

__device__ __forceinline__ void barycentric(axd::f3 p, axd::f3 a, axd::f3 b, axd::f3 c, float* u, float* v,
                                            float* w) {
    using namespace axd;
    const f3 v0 = sub(b, a), v1 = sub(c, a), v2 = sub(p, a);
    const float d00 = dot(v0, v0), d01 = dot(v0, v1), d11 = dot(v1, v1);
    const float d20 = dot(v2, v0), d21 = dot(v2, v1);
    const float den = d00 * d11 - d01 * d01;
    if (!(den != 0.0f)) {
        *u = 1.0f;
        *v = 0.0f;
        *w = 0.0f;
        return;
    }
    *v = (d11 * d20 - d01 * d21) / den;
    *w = (d00 * d21 - d01 * d20) / den;
    *u = 1.0f - *v - *w;
}

// Warp-cooperative EPA from the GJK tetrahedron (all 32 lanes call it).
template <int KA = kAnyShape, int KB = kAnyShape>
__device__ inline EpaResult epaWarp(const Geom& A, const Geom& B, const SupportPt tet[4], EpaWarp& s, int lane) {
    using namespace axd;
    if (lane == 0) {
        for (int k = 0; k < 4; ++k) {
            s.w[k] = make_float4(tet[k].w.x, tet[k].w.y, tet[k].w.z, 0.0f);
            s.a[k] = make_float4(tet[k].a.x, tet[k].a.y, tet[k].a.z, 0.0f);
            s.b[k] = make_float4(tet[k].b.x, tet[k].b.y, tet[k].b.z, 0.0f);
        }
        s.nv = 4;
        s.nf = 4;
    }
    __syncwarp();
    if (lane < 4) {
        const int tri[4][3] = {{0, 1, 2}, {0, 3, 1}, {0, 2, 3}, {1, 3, 2}};
        makeFace(s, tri[lane][0], tri[lane][1], tri[lane][2], &s.fi[lane], &s.fn[lane]);
    }
    __syncwarp();
    bool converged = false;
    for (int it = 0; it < kEpaMaxIter; ++it) {
        const int best = closestFace(s, lane);
        const float4 bf = s.fn[best];
        if (!(bf.w < FLT_MAX)) break;
        const f3 bn{bf.x, bf.y, bf.z};
        const SupportPt sp = minkowski<KA, KB>(A, B, bn);
        const float sd = dot(bn, sp.w);
        if (sd - bf.w < kEpaTolerance) {
            converged = true;
            break;
        }
        if (s.nv >= kEpaMaxVerts) break;
        const int nvIdx = s.nv;
        const int nf = s.nf;
        // faces that see the new point (lane-parallel), listed in face order
        unsigned visMask[(kEpaMaxFaces + 31) / 32];
        int nvis = 0;
#pragma unroll
        for (int c = 0; c < (kEpaMaxFaces + 31) / 32; ++c) {
            const int k = c * 32 + lane;
            bool v = false;
            if (k < nf) {
                const float4 f = s.fn[k];
                v = dot(f3{f.x, f.y, f.z}, sub(sp.w, vw(s, s.fi[k].x))) > 0.0f;
            }
            visMask[c] = __ballot_sync(0xFFFFFFFFu, v);
            if (v) s.visList[nvis + __popc(visMask[c] & ((1u << lane) - 1u))] = k;
            nvis += __popc(visMask[c]);
        }
        __syncwarp();
        // horizon: edges of visible faces whose reverse is not also on a visible face, in
        // (face, edge) order of appearance.  When every directed edge of the visible faces
        // is distinct, an edge stays exactly when its reverse is absent, so the lanes test
        // the edges in parallel and compact the survivors in order; otherwise (a degenerate
        // polytope) lane 0 runs the sequential cancellation that defines the list.
        if (lane == 0) {
            s.w[nvIdx] = make_float4(sp.w.x, sp.w.y, sp.w.z, 0.0f);
            s.a[nvIdx] = make_float4(sp.a.x, sp.a.y, sp.a.z, 0.0f);
            s.b[nvIdx] = make_float4(sp.b.x, sp.b.y, sp.b.z, 0.0f);
            s.nv = nvIdx + 1;
        }
        const int nItems = 3 * nvis;
        auto edgeOf = [&](int k) {
            const int4 fk = s.fi[s.visList[k / 3]];
            const int q = k % 3;
            return q == 0 ? make_int2(fk.x, fk.y) : (q == 1 ? make_int2(fk.y, fk.z) : make_int2(fk.z, fk.x));
        };
        bool dup = false;
        int nePar = 0;
        for (int c0 = 0; c0 < nItems; c0 += 32) {
            const int k = c0 + lane;
            int2 e = make_int2(-1, -1);
            bool keepE = false;
            if (k < nItems) {
                e = edgeOf(k);
                bool rev = false;
                for (int j = 0; j < nItems; ++j) {
                    if (j == k) continue;
                    const int2 f = edgeOf(j);
                    dup |= f.x == e.x && f.y == e.y;
                    rev |= f.x == e.y && f.y == e.x;
                }
                keepE = !rev;
            }
            const unsigned km = __ballot_sync(0xFFFFFFFFu, keepE);
            if (keepE) s.edges[nePar + __popc(km & ((1u << lane) - 1u))] = e;
            nePar += __popc(km);
        }
        dup = __any_sync(0xFFFFFFFFu, dup);
        __syncwarp();
        if (!dup) {
            if (lane == 0) s.ne = nePar;
        } else if (lane == 0) {
            int ne = 0;
            for (int i = 0; i < nvis; ++i) {
                const int4 fk = s.fi[s.visList[i]];
                const int e[3][2] = {{fk.x, fk.y}, {fk.y, fk.z}, {fk.z, fk.x}};
                for (int q = 0; q < 3; ++q) {
                    int found = -1;
                    for (int h = 0; h < ne; ++h)
                        if (s.edges[h].x == e[q][1] && s.edges[h].y == e[q][0]) {
                            found = h;
                            break;
                        }
                    if (found >= 0) {
                        for (int h = found; h + 1 < ne; ++h) s.edges[h] = s.edges[h + 1];
                        --ne;
                    } else {
                        s.edges[ne] = make_int2(e[q][0], e[q][1]);
                        ++ne;
                    }
                }
            }
            s.ne = ne;
        }
        __syncwarp();
        // kept faces move down in order; a chunk is read whole before it is written, and
        // its destinations lie below the next chunk
        int keep = 0;
#pragma unroll
        for (int c = 0; c < (kEpaMaxFaces + 31) / 32; ++c) {
            const int k = c * 32 + lane;
            const bool kp = k < nf && !((visMask[c] >> lane) & 1u);
            int4 fk = make_int4(0, 0, 0, 0);
            float4 fnk = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (kp) {
                fk = s.fi[k];
                fnk = s.fn[k];
            }
            const unsigned km = __ballot_sync(0xFFFFFFFFu, kp);
            __syncwarp();
            if (kp) {
                const int d = keep + __popc(km & ((1u << lane) - 1u));
                s.fi[d] = fk;
                s.fn[d] = fnk;
            }
            keep += __popc(km);
            __syncwarp();
        }
        if (lane == 0) s.nf = keep;
        __syncwarp();
        if (s.nf + s.ne > kEpaMaxFaces) break;
        const int base = s.nf, ne = s.ne;
        for (int h = lane; h < ne; h += 32) makeFace(s, s.edges[h].x, s.edges[h].y, nvIdx, &s.fi[base + h], &s.fn[base + h]);
        __syncwarp();
        if (lane == 0) s.nf = base + ne;
        __syncwarp();
    }
    const int best = closestFace(s, lane);
    const float4 bf = s.fn[best];
    const int4 fb = s.fi[best];
    EpaResult r;
    r.converged = converged;
    r.n = f3{bf.x, bf.y, bf.z};
    r.depth = bf.w < FLT_MAX ? bf.w : 0.0f;
    const f3 proj = scale(r.n, r.depth);
    float u, vv, ww;
    barycentric(proj, vw(s, fb.x), vw(s, fb.y), vw(s, fb.z), &u, &vv, &ww);
    r.pa = add(add(scale(mk(s.a[fb.x]), u), scale(mk(s.a[fb.y]), vv)), scale(mk(s.a[fb.z]), ww));
    r.pb = add(add(scale(mk(s.b[fb.x]), u), scale(mk(s.b[fb.y]), vv)), scale(mk(s.b[fb.z]), ww));
    __syncwarp();
    return r;
}

__device__ __forceinline__ axd::f3 boxFaceNormal(const Geom& g, int f) {
    return axd::rotate(g.rot, axisVec(f >> 1, (f & 1) ? -1.0f : 1.0f));
}

__device__ __forceinline__ int bestFace(const Geom& g, axd::f3 d, float* align) {
    int bf = 0;
    float ba = axd::dot(boxFaceNormal(g, 0), d);
    for (int f = 1; f < 6; ++f) {
        const float a = axd::dot(boxFaceNormal(g, f), d);
        if (a > ba) {
            ba = a;
            bf = f;
        }
    }
    *align = ba;
    return bf;
}

__device__ __forceinline__ void boxFaceVerts(const Geom& g, int f, axd::f3 out[4]) {
    using namespace axd;
    const int k = f >> 1, u = (k + 1) % 3, w = (k + 2) % 3;
    const float s = (f & 1) ? -1.0f : 1.0f;
    const float su[4] = {1.0f, -1.0f, -1.0f, 1.0f}, sw[4] = {1.0f, 1.0f, -1.0f, -1.0f};
    const f3 e = mk(g.ext);
    for (int i = 0; i < 4; ++i) {
        float l[3];
        l[k] = s * comp3(e, k);
        l[u] = su[i] * comp3(e, u);
        l[w] = sw[i] * comp3(e, w);
        out[i] = add(mk(g.pos), rotate(g.rot, f3{l[0], l[1], l[2]}));
    }
}

__device__ __forceinline__ int clipPolygon(const axd::f3* in, int nin, axd::f3 n, float off, axd::f3* out) {
    using namespace axd;
    int no = 0;
    for (int i = 0; i < nin; ++i) {
        const f3 p = in[i], q = in[(i + 1) % nin];
        const float dp = dot(n, p) - off, dq = dot(n, q) - off;
        const bool ip = dp <= 0.0f, iq = dq <= 0.0f;
        if (ip) out[no++] = p;
        if (ip != iq) {
            const float t = dp / (dp - dq);
            out[no++] = add(p, scale(sub(q, p), t));
        }
    }
    return no;
}

__device__ __forceinline__ int reducePoints(axd::f3* p, float* depth, int n, axd::f3 nref) {
    using namespace axd;
    if (n <= 4) return n;
    int i0 = 0;
    for (int i = 1; i < n; ++i)
        if (depth[i] > depth[i0]) i0 = i;
    int i1 = -1;
    float bd = -1.0f;
    for (int i = 0; i < n; ++i) {
        const f3 d = sub(p[i], p[i0]);
        const float dd = dot(d, d);
        if (i != i0 && dd > bd) {
            bd = dd;
            i1 = i;
        }
    }
    int i2 = -1, i3 = -1;
    float amax = 0.0f, amin = 0.0f;
    const f3 e = sub(p[i1], p[i0]);
    for (int i = 0; i < n; ++i) {
        if (i == i0 || i == i1) continue;
        const float a = dot(cross(e, sub(p[i], p[i0])), nref);
        if (i2 < 0 || a > amax) {
            amax = a;
            i2 = i;
        }
    }
    for (int i = 0; i < n; ++i) {
        if (i == i0 || i == i1 || i == i2) continue;
        const float a = dot(cross(e, sub(p[i], p[i0])), nref);
        if (i3 < 0 || a < amin) {
            amin = a;
            i3 = i;
        }
    }
    const int idx[4] = {i0, i1, i2, i3};
    f3 tp[4];
    float td[4];
    int m = 0;
    for (int q = 0; q < 4; ++q) {
        if (idx[q] < 0) continue;
        tp[m] = p[idx[q]];
        td[m] = depth[idx[q]];
        ++m;
    }
    for (int q = 0; q < m; ++q) {
        p[q] = tp[q];
        depth[q] = td[q];
    }
    return m;
}

__device__ __forceinline__ void singlePoint(const EpaResult& e, Contact* out) {
    out->n = e.n;
    out->p[0] = axd::scale(axd::add(e.pa, e.pb), 0.5f);
    out->depth[0] = e.depth;
    out->count = 1;
}

// Manifold of box A against box B from the EPA result (normal A -> B).
// allow: feature points within this separation of the reference face are kept (0 for a
// touching pair; the speculative distance for a sweeping pair, whose separated points get
// negative depth).
__device__ __forceinline__ void boxBoxManifold(const Geom& A, const Geom& B, const EpaResult& e, float allow,
                                               Contact* out) {
    using namespace axd;
    float alA, alB;
    const int fA = bestFace(A, e.n, &alA);
    const int fB = bestFace(B, neg3(e.n), &alB);
    if (!(alA >= kFaceContactAlign || alB >= kFaceContactAlign)) {
        singlePoint(e, out);
        return;
    }
    const bool refA = alA >= alB - 1e-3f;
    const Geom& R = refA ? A : B;
    const Geom& I = refA ? B : A;
    const int fr = refA ? fA : fB;
    const f3 rn = boxFaceNormal(R, fr);
    float ia;
    const int fi = bestFace(I, neg3(rn), &ia);
    f3 poly[8], tmp[8];
    boxFaceVerts(I, fi, poly);
    int np = 4;
    const int k = fr >> 1;
    const int axes[2] = {(k + 1) % 3, (k + 2) % 3};
    const f3 rext = mk(R.ext);
    for (int a = 0; a < 2 && np > 0; ++a) {
        for (int sgn = 0; sgn < 2 && np > 0; ++sgn) {
            const int ax = axes[a];
            const f3 sn = rotate(R.rot, axisVec(ax, sgn ? -1.0f : 1.0f));
            const float off = dot(sn, mk(R.pos)) + comp3(rext, ax);
            np = clipPolygon(poly, np, sn, off, tmp);
            for (int q = 0; q < np; ++q) poly[q] = tmp[q];
        }
    }
    const float roff = dot(rn, mk(R.pos)) + comp3(rext, k);
    f3 pts[8];
    float dep[8];
    int m = 0;
    for (int q = 0; q < np; ++q) {
        const float sep = dot(rn, poly[q]) - roff;
        if (sep <= allow) {
            const float h = 0.5f * sep;
            pts[m] = f3{poly[q].x - rn.x * h, poly[q].y - rn.y * h, poly[q].z - rn.z * h};
            dep[m] = -sep;
            ++m;
        }
    }
    if (m == 0) {
        singlePoint(e, out);
        return;
    }
    m = reducePoints(pts, dep, m, rn);
    out->n = refA ? rn : neg3(rn);
    out->count = (uint32_t)m;
    for (int q = 0; q < m; ++q) {
        out->p[q] = pts[q];
        out->depth[q] = dep[q];
    }
}

// Manifold of box A against capsule B from the EPA result (normal A -> B).
__device__ __forceinline__ void boxCapsuleManifold(const Geom& A, const Geom& B, const EpaResult& e, float allow,
                                                   Contact* out) {
    using namespace axd;
    float al;
    const int fa = bestFace(A, e.n, &al);
    const f3 rn = boxFaceNormal(A, fa);
    f3 e0, e1;
    capsuleSegment(mk(B.pos), B.rot, B.ext.y, &e0, &e1);
    const f3 seg = sub(e1, e0);
    const float slen = sqrtf(dot(seg, seg));
    const bool parallel = slen > 0.0f && fabsf(dot(seg, rn)) < kCapsuleParallel * slen;
    if (al >= kFaceContactAlign && parallel) {
        float t0 = 0.0f, t1 = 1.0f;
        const int k = fa >> 1;
        const int axes[2] = {(k + 1) % 3, (k + 2) % 3};
        const f3 aext = mk(A.ext);
        for (int a = 0; a < 2; ++a)
            for (int sgn = 0; sgn < 2; ++sgn) {
                const int ax = axes[a];
                const f3 sn = rotate(A.rot, axisVec(ax, sgn ? -1.0f : 1.0f));
                const float off = dot(sn, mk(A.pos)) + comp3(aext, ax);
                const float d0 = dot(sn, e0) - off, d1 = dot(sn, e1) - off;
                if (d0 > 0.0f && d1 > 0.0f) {
                    t0 = 1.0f;
                    t1 = 0.0f;
                } else if (d0 > 0.0f) {
                    const float t = d0 / (d0 - d1);
                    t0 = t > t0 ? t : t0;
                } else if (d1 > 0.0f) {
                    const float t = d0 / (d0 - d1);
                    t1 = t < t1 ? t : t1;
                }
            }
        if (t0 <= t1) {
            const float roff = dot(rn, mk(A.pos)) + comp3(aext, k);
            const float ts[2] = {t0, t1};
            int m = 0;
            for (int q = 0; q < 2; ++q) {
                if (q == 1 && !(t1 > t0)) break;
                const f3 p = add(e0, scale(seg, ts[q]));
                const float sep = dot(rn, p) - roff - B.ext.x;
                if (sep <= allow) {
                    const float h = B.ext.x + 0.5f * sep;
                    out->p[m] = f3{p.x - rn.x * h, p.y - rn.y * h, p.z - rn.z * h};
                    out->depth[m] = -sep;
                    ++m;
                }
            }
            if (m > 0) {
                out->n = rn;
                out->count = (uint32_t)m;
                return;
            }
        }
    }
    singlePoint(e, out);
}

// ---- general manifold from supporting features (pairs with a cylinder or a convex hull) ----
//
// The feature of a shape in direction d is the part of its surface that is extreme along d:
// a polygon (box face, cylinder cap as an inscribed octagon, the hull vertices within a
// small tolerance of the supporting plane), a segment (capsule core or cylinder side line
// nearly perpendicular to d) or a point (the support point).  The manifold clips the other
// shape's feature against the side planes of the better-aligned polygon, keeps the points
// at or below that polygon's plane, and falls back to EPA's single point.

constexpr float kCylinderSide = 0.05f;   // |d . axis| below this: the side line is the feature
constexpr float kHullFeatureTol = 1e-3f;  // x bounding radius: hull vertices on the supporting plane
constexpr float kOct = 0.70710678f;

struct Feature {
    int n;            // 1 point, 2 segment, >= 3 polygon (convex, in order around normal)
    axd::f3 v[8];
    axd::f3 normal;   // polygon: its outward normal
    float radius;     // rounding of the surface around the feature (capsule, sphere)
};

// Two unit vectors spanning the plane normal to n.
__device__ __forceinline__ void planeBasis(axd::f3 n, axd::f3* t1, axd::f3* t2) {
    using namespace axd;
    const f3 a = fabsf(n.x) < 0.57735f ? f3{1.0f, 0.0f, 0.0f} : f3{0.0f, 1.0f, 0.0f};
    f3 t = cross(n, a);
    const float l = sqrtf(dot(t, t));
    t = f3{t.x / l, t.y / l, t.z / l};
    *t1 = t;
    *t2 = cross(n, t);
}

// Monotone stand-in for the angle of (x, y) (no transcendental function): [0, 4).
__device__ __forceinline__ float pseudoAngle(float x, float y) {
    const float s = fabsf(x) + fabsf(y);
    if (!(s > 0.0f)) return 0.0f;
    const float r = x / s;
    return y >= 0.0f ? 1.0f - r : 3.0f + r;
}

__device__ __forceinline__ void featureOf(const Geom& g, axd::f3 d, Feature* f) {
    using namespace axd;
    f->radius = 0.0f;
    f->normal = d;
    if (g.shape == AXIOM_SHAPE_SPHERE) {
        f->n = 1;
        f->v[0] = mk(g.pos);
        f->radius = g.ext.x;
        return;
    }
    if (g.shape == AXIOM_SHAPE_CAPSULE) {
        f3 e0, e1;
        capsuleSegment(mk(g.pos), g.rot, g.ext.y, &e0, &e1);
        const f3 seg = sub(e1, e0);
        const float slen = sqrtf(dot(seg, seg));
        const float ds = dot(seg, d);
        f->radius = g.ext.x;
        if (slen > 0.0f && fabsf(ds) < kCapsuleParallel * slen) {
            f->n = 2;
            f->v[0] = e0;
            f->v[1] = e1;
        } else {
            f->n = 1;
            f->v[0] = ds >= 0.0f ? e1 : e0;
        }
        return;
    }
    if (g.shape == AXIOM_SHAPE_BOX) {
        float al;
        const int fb = bestFace(g, d, &al);
        if (al >= kFaceContactAlign) {
            f->n = 4;
            boxFaceVerts(g, fb, f->v);
            f->normal = boxFaceNormal(g, fb);
        } else {
            f->n = 1;
            f->v[0] = supportShape(g, d);
        }
        return;
    }
    if (g.shape == AXIOM_SHAPE_CYLINDER) {
        const f3 u = rotate(g.rot, f3{0.0f, 1.0f, 0.0f});
        const f3 ax = rotate(g.rot, f3{0.0f, g.ext.y, 0.0f});
        const float du = dot(d, u);
        if (fabsf(du) >= kFaceContactAlign) {  // the cap: an inscribed octagon
            const f3 cc = du >= 0.0f ? add(mk(g.pos), ax) : sub(mk(g.pos), ax);
            const f3 e1 = rotate(g.rot, f3{g.ext.x, 0.0f, 0.0f});
            const f3 e2 = rotate(g.rot, f3{0.0f, 0.0f, g.ext.x});
            const float cs[8] = {1.0f, kOct, 0.0f, -kOct, -1.0f, -kOct, 0.0f, kOct};
            const float sn[8] = {0.0f, kOct, 1.0f, kOct, 0.0f, -kOct, -1.0f, -kOct};
            f->n = 8;
            for (int k = 0; k < 8; ++k)
                f->v[k] = f3{cc.x + e1.x * cs[k] + e2.x * sn[k], cc.y + e1.y * cs[k] + e2.y * sn[k],
                             cc.z + e1.z * cs[k] + e2.z * sn[k]};
            f->normal = du >= 0.0f ? u : neg3(u);
        } else if (fabsf(du) < kCylinderSide) {  // the side line facing d
            const f3 dp{d.x - u.x * du, d.y - u.y * du, d.z - u.z * du};
            const float len = sqrtf(dot(dp, dp));
            const float k = g.ext.x / len;
            const f3 rad{dp.x * k, dp.y * k, dp.z * k};
            f->n = 2;
            f->v[0] = add(sub(mk(g.pos), ax), rad);
            f->v[1] = add(add(mk(g.pos), ax), rad);
        } else {
            f->n = 1;
            f->v[0] = supportShape(g, d);
        }
        return;
    }
    // convex hull: the vertices within kHullFeatureTol x radius of the supporting plane
    const float4* v = g.verts + hullOffset(g);
    const uint32_t nv = hullCount(g);
    const f3 dl = rotateInv(g.rot, d);
    const float top = dot(mk(v[hullSupportIndex(g, dl)]), dl);
    const float tol = kHullFeatureTol * g.ext.x;
    int idx[8];
    int m = 0;
    for (uint32_t i = 0; i < nv && m < 8; ++i)
        if (dot(mk(v[i]), dl) >= top - tol) idx[m++] = (int)i;
    if (m >= 3) {
        f3 c = mk(v[idx[0]]);
        for (int i = 1; i < m; ++i) c = add(c, mk(v[idx[i]]));
        c = scale(c, 1.0f / (float)m);
        f3 t1, t2;
        planeBasis(dl, &t1, &t2);
        float ang[8];
        for (int i = 0; i < m; ++i) {
            const f3 r = sub(mk(v[idx[i]]), c);
            ang[i] = pseudoAngle(dot(r, t1), dot(r, t2));
        }
        for (int i = 1; i < m; ++i)  // by angle, then by vertex index
            for (int j = i; j > 0 && (ang[j] < ang[j - 1] || (ang[j] == ang[j - 1] && idx[j] < idx[j - 1])); --j) {
                const float ta = ang[j];
                ang[j] = ang[j - 1];
                ang[j - 1] = ta;
                const int ti = idx[j];
                idx[j] = idx[j - 1];
                idx[j - 1] = ti;
            }
    }
    f->n = m;
    for (int i = 0; i < m; ++i) f->v[i] = add(mk(g.pos), rotate(g.rot, mk(v[idx[i]])));
}

// Manifold of A against B from the EPA result (normal A -> B) through their features.
__device__ __forceinline__ void featureManifold(const Geom& A, const Geom& B, const EpaResult& e, float allow,
                                                Contact* out) {
    using namespace axd;
    Feature fa, fb;
    featureOf(A, e.n, &fa);
    featureOf(B, neg3(e.n), &fb);
    const bool pa = fa.n >= 3, pb = fb.n >= 3;
    if (!pa && !pb) {
        singlePoint(e, out);
        return;
    }
    const float ala = pa ? dot(fa.normal, e.n) : -2.0f;
    const float alb = pb ? dot(fb.normal, neg3(e.n)) : -2.0f;
    const bool refA = pa && (!pb || ala >= alb - 1e-3f);
    const Feature& R = refA ? fa : fb;
    const Feature& I = refA ? fb : fa;
    const f3 rn = R.normal;
    f3 cen = R.v[0];
    for (int i = 1; i < R.n; ++i) cen = add(cen, R.v[i]);
    cen = scale(cen, 1.0f / (float)R.n);
    f3 poly[16], tmp[16];
    int np = I.n;
    for (int i = 0; i < np; ++i) poly[i] = I.v[i];
    for (int i = 0; i < R.n && np > 0; ++i) {
        const f3 p0 = R.v[i], p1 = R.v[i + 1 < R.n ? i + 1 : 0];
        f3 sn = cross(sub(p1, p0), rn);
        if (dot(sn, sub(cen, p0)) > 0.0f) sn = neg3(sn);
        const float off = dot(sn, p0);
        if (np >= 3) {
            np = clipPolygon(poly, np, sn, off, tmp);
            for (int q = 0; q < np; ++q) poly[q] = tmp[q];
        } else if (np == 2) {
            const float d0 = dot(sn, poly[0]) - off, d1 = dot(sn, poly[1]) - off;
            if (d0 > 0.0f && d1 > 0.0f) {
                np = 0;
            } else if (d0 > 0.0f) {
                poly[0] = add(poly[0], scale(sub(poly[1], poly[0]), d0 / (d0 - d1)));
            } else if (d1 > 0.0f) {
                poly[1] = add(poly[0], scale(sub(poly[1], poly[0]), d0 / (d0 - d1)));
            }
        } else if (dot(sn, poly[0]) - off > 0.0f) {
            np = 0;
        }
    }
    const float roff = dot(rn, R.v[0]);
    f3 pts[16];
    float dep[16];
    int m = 0;
    for (int q = 0; q < np; ++q) {
        const float sep = dot(rn, poly[q]) - roff - I.radius;
        if (sep <= allow) {
            const float h = I.radius + 0.5f * sep;
            pts[m] = f3{poly[q].x - rn.x * h, poly[q].y - rn.y * h, poly[q].z - rn.z * h};
            dep[m] = -sep;
            ++m;
        }
    }
    if (m == 0) {
        singlePoint(e, out);
        return;
    }
    m = reducePoints(pts, dep, m, rn);
    out->n = refA ? rn : neg3(rn);
    out->count = (uint32_t)m;
    for (int q = 0; q < m; ++q) {
        out->p[q] = pts[q];
        out->depth[q] = dep[q];
    }
}

// ---- lane-parallel pairs: GJK and the manifold per lane, EPA per warp ----

enum : uint32_t { kPairBoxBox = 0u, kPairBoxCapsule = 1u, kPairGeneric = 2u };

__device__ __forceinline__ float4 shflF4(float4 v, int src) {
    return make_float4(__shfl_sync(0xFFFFFFFFu, v.x, src), __shfl_sync(0xFFFFFFFFu, v.y, src),
                       __shfl_sync(0xFFFFFFFFu, v.z, src), __shfl_sync(0xFFFFFFFFu, v.w, src));
}
__device__ __forceinline__ axd::f3 shflF3(axd::f3 v, int src) {
    return axd::f3{__shfl_sync(0xFFFFFFFFu, v.x, src), __shfl_sync(0xFFFFFFFFu, v.y, src),
                   __shfl_sync(0xFFFFFFFFu, v.z, src)};
}
__device__ __forceinline__ Geom shflGeom(const Geom& g, int src) {
    Geom r;
    r.shape = __shfl_sync(0xFFFFFFFFu, g.shape, src);
    r.pos = shflF4(g.pos, src);
    r.rot = shflF4(g.rot, src);
    r.ext = shflF4(g.ext, src);
    r.verts = reinterpret_cast<const float4*>(
        __shfl_sync(0xFFFFFFFFu, reinterpret_cast<unsigned long long>(g.verts), src));
    r.margin = __shfl_sync(0xFFFFFFFFu, g.margin, src);
    return r;
}

// Up to 32 pairs, one per lane (lanes with `active`): each lane runs GJK on its own pair
// (A, B) of kind `kind` (a box-capsule pair has the box as A); the warp then runs the
// cooperative EPA for every overlapping pair in lane order, with that pair's shapes and
// simplex broadcast from its lane; each lane finally builds its own manifold.  Every
// function runs the same expressions on the same inputs as when a whole warp handles one
// pair, so the contacts are the same.  All 32 lanes call it.  *fail receives the lane's
// kFailGjk (GJK ran out of iterations: treated as separated) and kFailEpa (EPA stopped at
// a cap: the closest face found gives the contact) bits.
__device__ inline Contact lanePairs(bool active, uint32_t kind, const Geom& A, const Geom& B, EpaWarp& ws,
                                    int lane, uint32_t* fail) {
    SupportPt tet[4];
    bool hit = false, exhausted = false;
    if (active) {
        if (kind == kPairBoxBox) hit = gjk<AXIOM_SHAPE_BOX, AXIOM_SHAPE_BOX>(A, B, tet, &exhausted);
        else if (kind == kPairBoxCapsule) hit = gjk<AXIOM_SHAPE_BOX, AXIOM_SHAPE_CAPSULE>(A, B, tet, &exhausted);
        else hit = gjk(A, B, tet, &exhausted);
    }
    // speculative contacts: a separated pair of sweeping bodies tries again with A inflated
    // by spec (the two bodies' displacements); if that meets, the gap is within spec
    const float spec = active ? A.pos.w + B.pos.w : 0.0f;
    Geom Ai = A;
    bool specHit = false, specExhausted = false;
    if (active && !hit && !exhausted && spec > 0.0f) {
        Ai.margin = spec;
        if (kind == kPairBoxBox) specHit = gjk<AXIOM_SHAPE_BOX, AXIOM_SHAPE_BOX>(Ai, B, tet, &specExhausted);
        else if (kind == kPairBoxCapsule)
            specHit = gjk<AXIOM_SHAPE_BOX, AXIOM_SHAPE_CAPSULE>(Ai, B, tet, &specExhausted);
        else specHit = gjk(Ai, B, tet, &specExhausted);
    }
    EpaResult mine{};
    for (unsigned pending = __ballot_sync(0xFFFFFFFFu, hit || specHit); pending; pending &= pending - 1u) {
        const int j = __ffs(pending) - 1;
        const uint32_t kj = __shfl_sync(0xFFFFFFFFu, kind, j);
        const Geom Aj = shflGeom(Ai, j), Bj = shflGeom(B, j);
        SupportPt tj[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            tj[k].w = shflF3(tet[k].w, j);
            tj[k].a = shflF3(tet[k].a, j);
            tj[k].b = shflF3(tet[k].b, j);
        }
        EpaResult r;
        if (kj == kPairBoxBox) r = epaWarp<AXIOM_SHAPE_BOX, AXIOM_SHAPE_BOX>(Aj, Bj, tj, ws, lane);
        else if (kj == kPairBoxCapsule) r = epaWarp<AXIOM_SHAPE_BOX, AXIOM_SHAPE_CAPSULE>(Aj, Bj, tj, ws, lane);
        else r = epaWarp(Aj, Bj, tj, ws, lane);
        if (lane == j) mine = r;
    }
    Contact c;
    c.count = 0;
    if (specHit) {
        // the inflated witness moves back to A's own surface; depth less spec = -(the gap)
        mine.pa = axd::f3{mine.pa.x - mine.n.x * spec, mine.pa.y - mine.n.y * spec, mine.pa.z - mine.n.z * spec};
        mine.depth = mine.depth - spec;
    }
    if (hit || specHit) {
        if (kind == kPairBoxBox) boxBoxManifold(A, B, mine, spec, &c);
        else if (kind == kPairBoxCapsule) boxCapsuleManifold(A, B, mine, spec, &c);
        else featureManifold(A, B, mine, spec, &c);
    }
    *fail = ((exhausted || specExhausted) ? kFailGjk : 0u) | (((hit || specHit) && !mine.converged) ? kFailEpa : 0u);
    return c;
}

}  // namespace axiom_gb300
