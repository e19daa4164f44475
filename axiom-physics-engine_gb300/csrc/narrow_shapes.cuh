// narrow_shapes.cuh — per-shape-pair contact generation (device).
//
// Contact model: a manifold of up to 4 points shares one unit normal pointing from the
// first shape to the second; a point lies midway between the two surfaces and touching
// (depth 0) counts.  Every function spells its fp32 operations in a fixed order (the
// library builds with --fmad=false), so results are reproducible bit for bit by a scalar
// CPU evaluation of the same expressions.
//
// Analytic pairs: sphere-sphere, sphere-plane, sphere-box (closest point in the box
// frame; a centre inside the box leaves through the nearest face), sphere-capsule
// (closest point on the segment), capsule-capsule (closest points of two segments,
// Ericson, Real-Time Collision Detection 5.1.9), box-plane (the <= 4 deepest vertices at
// or below the plane, emitted in vertex order), capsule-plane (the two end spheres).
// sphere-cylinder (closest point of the solid cylinder), cylinder-plane (rim points),
// convex-plane (deepest hull vertices).  Box-box, box-capsule and the other pairs with a
// cylinder or a convex hull go through GJK + EPA (gjk_epa.cuh).
#pragma once

#include "../../include/axiom_c.h"
#include "dmath.cuh"
#include "shapes.h"

namespace axiom_gb300 {

struct Geom {
    uint32_t shape;
    float4 pos, rot, ext;           // pos.w: the body's sweep length this step (speculative contacts)
    const float4* verts = nullptr;  // convex: the world's hull vertex pool
    float margin = 0.0f;            // support mapping inflated by this radius (speculative GJK)
};

// A convex body's ext packs (bounding radius, first pool vertex bits, vertex count bits, 0).
__device__ __forceinline__ uint32_t hullOffset(const Geom& g) { return __float_as_uint(g.ext.y); }
__device__ __forceinline__ uint32_t hullCount(const Geom& g) { return __float_as_uint(g.ext.z); }

struct Contact {
    uint32_t count;
    axd::f3 n;
    axd::f3 p[4];
    float depth[4];
};

__device__ __forceinline__ float clampf(float x, float lo, float hi) {
    return x < lo ? lo : (x > hi ? hi : x);
}
__device__ __forceinline__ axd::f3 neg3(axd::f3 a) { return axd::f3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float comp3(axd::f3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
__device__ __forceinline__ axd::f3 axisVec(int k, float s) {
    return axd::f3{k == 0 ? s : 0.0f, k == 1 ? s : 0.0f, k == 2 ? s : 0.0f};
}
__device__ __forceinline__ axd::f3 rotateInv(float4 q, axd::f3 v) { return axd::rotate(axd::conj(q), v); }

// Speculative contacts (continuous collision): every analytic pair also reports a contact
// while its gap is at most spec (the two bodies' displacements this step, 0 when the
// world does not sweep); such a contact has a negative depth (the separation).

// Sphere (ca, ra) against sphere (cb, rb); normal a -> b, point midway between surfaces.
__device__ __forceinline__ bool sphereSphere(axd::f3 ca, float ra, axd::f3 cb, float rb, Contact* c,
                                             float spec = 0.0f) {
    using namespace axd;
    const f3 d = sub(cb, ca);
    const float dist2 = dot(d, d);
    const float rs = ra + rb;
    const float lim = rs + spec;
    if (dist2 > lim * lim) return false;
    const float dist = sqrtf(dist2);
    const f3 n = dist > 0.0f ? f3{d.x / dist, d.y / dist, d.z / dist} : f3{0.0f, 1.0f, 0.0f};
    const float depth = rs - dist;
    const float s = ra - 0.5f * depth;
    c->n = n;
    c->p[0] = f3{ca.x + n.x * s, ca.y + n.y * s, ca.z + n.z * s};
    c->depth[0] = depth;
    c->count = 1;
    return true;
}

// Sphere (cs, r) against the plane through pp with unit normal np (contact normal np);
// appends one point to c.
__device__ __forceinline__ bool spherePlaneAppend(axd::f3 pp, axd::f3 np, axd::f3 cs, float r, Contact* c,
                                                  float spec = 0.0f) {
    using namespace axd;
    const float s = dot(sub(cs, pp), np);
    if (s > r + spec) return false;
    const float depth = r - s;
    const float k = r - 0.5f * depth;
    c->n = np;
    c->p[c->count] = f3{cs.x - np.x * k, cs.y - np.y * k, cs.z - np.z * k};
    c->depth[c->count] = depth;
    c->count += 1;
    return true;
}

// Sphere (c, r) against box (pb, qb, he); normal sphere -> box.
__device__ __forceinline__ bool sphereBox(axd::f3 c, float r, axd::f3 pb, float4 qb, axd::f3 he, Contact* out,
                                          float spec = 0.0f) {
    using namespace axd;
    const f3 cl = rotateInv(qb, sub(c, pb));
    const f3 q{clampf(cl.x, -he.x, he.x), clampf(cl.y, -he.y, he.y), clampf(cl.z, -he.z, he.z)};
    const f3 diff = sub(cl, q);
    const float dist2 = dot(diff, diff);
    const float lim = r + spec;
    if (dist2 > lim * lim) return false;
    f3 nl;
    float depth;
    if (dist2 > 0.0f) {
        const float dist = sqrtf(dist2);
        nl = f3{diff.x / dist, diff.y / dist, diff.z / dist};
        depth = r - dist;
    } else {
        int k = 0;
        float best = he.x - fabsf(cl.x);
        const float py = he.y - fabsf(cl.y), pz = he.z - fabsf(cl.z);
        if (py < best) {
            best = py;
            k = 1;
        }
        if (pz < best) {
            best = pz;
            k = 2;
        }
        nl = axisVec(k, comp3(cl, k) >= 0.0f ? 1.0f : -1.0f);
        depth = r + best;
    }
    const f3 nw = rotate(qb, nl);
    out->n = neg3(nw);
    const float k2 = r - 0.5f * depth;
    out->p[0] = f3{c.x - nw.x * k2, c.y - nw.y * k2, c.z - nw.z * k2};
    out->depth[0] = depth;
    out->count = 1;
    return true;
}

__device__ __forceinline__ void capsuleSegment(axd::f3 pc, float4 qc, float hh, axd::f3* e0, axd::f3* e1) {
    using namespace axd;
    const f3 ax = rotate(qc, f3{0.0f, hh, 0.0f});
    *e0 = sub(pc, ax);
    *e1 = add(pc, ax);
}

__device__ __forceinline__ axd::f3 closestOnSegment(axd::f3 p, axd::f3 e0, axd::f3 e1) {
    using namespace axd;
    const f3 seg = sub(e1, e0);
    const float len2 = dot(seg, seg);
    float t = len2 > 0.0f ? dot(sub(p, e0), seg) / len2 : 0.0f;
    t = clampf(t, 0.0f, 1.0f);
    return add(e0, scale(seg, t));
}

__device__ __forceinline__ void closestSegmentSegment(axd::f3 p1, axd::f3 q1, axd::f3 p2, axd::f3 q2,
                                                      axd::f3* c1, axd::f3* c2) {
    using namespace axd;
    const f3 d1 = sub(q1, p1), d2 = sub(q2, p2), r = sub(p1, p2);
    const float a = dot(d1, d1), e = dot(d2, d2), f = dot(d2, r);
    float s, t;
    if (a <= 0.0f && e <= 0.0f) {
        s = 0.0f;
        t = 0.0f;
    } else if (a <= 0.0f) {
        s = 0.0f;
        t = clampf(f / e, 0.0f, 1.0f);
    } else {
        const float c = dot(d1, r);
        if (e <= 0.0f) {
            t = 0.0f;
            s = clampf(-c / a, 0.0f, 1.0f);
        } else {
            const float b = dot(d1, d2);
            const float denom = a * e - b * b;
            s = denom != 0.0f ? clampf((b * f - c * e) / denom, 0.0f, 1.0f) : 0.0f;
            t = (b * s + f) / e;
            if (t < 0.0f) {
                t = 0.0f;
                s = clampf(-c / a, 0.0f, 1.0f);
            } else if (t > 1.0f) {
                t = 1.0f;
                s = clampf((b - c) / a, 0.0f, 1.0f);
            }
        }
    }
    *c1 = add(p1, scale(d1, s));
    *c2 = add(p2, scale(d2, t));
}

__device__ __forceinline__ axd::f3 boxVertex(const Geom& g, int v) {
    using namespace axd;
    const f3 l{(v & 1) ? g.ext.x : -g.ext.x, (v & 2) ? g.ext.y : -g.ext.y, (v & 4) ? g.ext.z : -g.ext.z};
    return add(mk(g.pos), rotate(g.rot, l));
}

__device__ __forceinline__ bool boxPlane(axd::f3 pp, axd::f3 np, const Geom& g, Contact* out, float spec = 0.0f) {
    using namespace axd;
    f3 vw[8];
    float depth[8];
    int cand[8], nc = 0;
    for (int v = 0; v < 8; ++v) {
        vw[v] = boxVertex(g, v);
        const float s = dot(sub(vw[v], pp), np);
        depth[v] = -s;
        if (s <= spec) cand[nc++] = v;
    }
    if (nc == 0) return false;
    for (int i = 0; i < nc; ++i) {
        int best = i;
        for (int j = i + 1; j < nc; ++j)
            if (depth[cand[j]] > depth[cand[best]]) best = j;
        const int t = cand[best];
        for (int j = best; j > i; --j) cand[j] = cand[j - 1];
        cand[i] = t;
    }
    const int keep = nc < 4 ? nc : 4;
    for (int i = 1; i < keep; ++i)
        for (int j = i; j > 0 && cand[j] < cand[j - 1]; --j) {
            const int t = cand[j];
            cand[j] = cand[j - 1];
            cand[j - 1] = t;
        }
    out->n = np;
    out->count = 0;
    for (int i = 0; i < keep; ++i) {
        const int v = cand[i];
        const float h = 0.5f * depth[v];
        out->p[i] = f3{vw[v].x + np.x * h, vw[v].y + np.y * h, vw[v].z + np.z * h};
        out->depth[i] = depth[v];
        out->count += 1;
    }
    return true;
}

__device__ __forceinline__ bool capsulePlane(axd::f3 pp, axd::f3 np, const Geom& g, Contact* out,
                                             float spec = 0.0f) {
    using namespace axd;
    f3 e0, e1;
    capsuleSegment(mk(g.pos), g.rot, g.ext.y, &e0, &e1);
    out->count = 0;
    spherePlaneAppend(pp, np, e0, g.ext.x, out, spec);
    spherePlaneAppend(pp, np, e1, g.ext.x, out, spec);
    return out->count > 0;
}

// Sphere (c, r) against cylinder (pc, qc, radius rc, half-height hc along local Y); normal
// sphere -> cylinder.  Closest point of the solid cylinder in its frame; a centre inside
// leaves through the nearer of the side and the cap (the cap on a tie).
__device__ __forceinline__ bool sphereCylinder(axd::f3 c, float r, axd::f3 pc, float4 qc, float rc, float hc,
                                               Contact* out, float spec = 0.0f) {
    using namespace axd;
    const f3 cl = rotateInv(qc, sub(c, pc));
    const float rho = sqrtf(cl.x * cl.x + cl.z * cl.z);
    f3 q{cl.x, clampf(cl.y, -hc, hc), cl.z};
    if (rho > rc) {
        const float k = rc / rho;
        q.x = cl.x * k;
        q.z = cl.z * k;
    }
    const f3 diff = sub(cl, q);
    const float dist2 = dot(diff, diff);
    const float lim = r + spec;
    if (dist2 > lim * lim) return false;
    f3 nl;
    float depth;
    if (dist2 > 0.0f) {
        const float dist = sqrtf(dist2);
        nl = f3{diff.x / dist, diff.y / dist, diff.z / dist};
        depth = r - dist;
    } else {
        const float side = rc - rho, cap = hc - fabsf(cl.y);
        if (cap <= side) {
            nl = f3{0.0f, cl.y >= 0.0f ? 1.0f : -1.0f, 0.0f};
            depth = r + cap;
        } else {
            nl = rho > 0.0f ? f3{cl.x / rho, 0.0f, cl.z / rho} : f3{1.0f, 0.0f, 0.0f};
            depth = r + side;
        }
    }
    const f3 nw = rotate(qc, nl);
    out->n = neg3(nw);
    const float k2 = r - 0.5f * depth;
    out->p[0] = f3{c.x - nw.x * k2, c.y - nw.y * k2, c.z - nw.z * k2};
    out->depth[0] = depth;
    out->count = 1;
    return true;
}

// Keeps the (at most 4) deepest candidates at or below the plane, deepest first with the
// lower index on ties, then emits them in index order, each midway between the surfaces.
// cand: world points; depth: signed depth below the plane.
__device__ __forceinline__ bool deepestBelowPlane(const axd::f3* cand, const float* depth, int n, axd::f3 np,
                                                  Contact* out, float spec = 0.0f) {
    using namespace axd;
    int best[4];
    int nb = 0;
    for (int v = 0; v < n; ++v) {
        if (!(depth[v] >= -spec)) continue;
        int at = nb;
        while (at > 0 && depth[v] > depth[best[at - 1]]) --at;  // stable: an equal depth stays behind
        if (at >= 4) continue;
        for (int j = (nb < 4 ? nb : 3); j > at; --j) best[j] = best[j - 1];
        best[at] = v;
        nb = nb < 4 ? nb + 1 : 4;
    }
    if (nb == 0) return false;
    for (int i = 1; i < nb; ++i)
        for (int j = i; j > 0 && best[j] < best[j - 1]; --j) {
            const int t = best[j];
            best[j] = best[j - 1];
            best[j - 1] = t;
        }
    out->n = np;
    out->count = (uint32_t)nb;
    for (int i = 0; i < nb; ++i) {
        const int v = best[i];
        const float h = 0.5f * depth[v];
        out->p[i] = f3{cand[v].x + np.x * h, cand[v].y + np.y * h, cand[v].z + np.z * h};
        out->depth[i] = depth[v];
    }
    return true;
}

// Cylinder against the plane (pp, np): four rim points of each cap, at 0, 90, 180 and 270
// degrees from the in-cap direction that dips deepest (-np without its axial part; the
// body's local X when the caps lie parallel to the plane); the deepest four are kept.
// A cylinder standing on a cap gets four rim points, one lying on its side two.
__device__ __forceinline__ bool cylinderPlane(axd::f3 pp, axd::f3 np, const Geom& g, Contact* out,
                                              float spec = 0.0f) {
    using namespace axd;
    const f3 u = rotate(g.rot, f3{0.0f, 1.0f, 0.0f});
    const f3 ax = rotate(g.rot, f3{0.0f, g.ext.y, 0.0f});
    const float nu = dot(np, u);
    f3 e1{u.x * nu - np.x, u.y * nu - np.y, u.z * nu - np.z};
    const float l2 = dot(e1, e1);
    if (l2 > 1e-12f) {
        const float l = sqrtf(l2);
        e1 = f3{e1.x / l, e1.y / l, e1.z / l};
    } else {
        e1 = rotate(g.rot, f3{1.0f, 0.0f, 0.0f});
    }
    const f3 e2 = cross(u, e1);
    const f3 c = mk(g.pos);
    f3 cand[8];
    float depth[8];
    for (int cap = 0; cap < 2; ++cap) {
        const f3 cc = cap ? add(c, ax) : sub(c, ax);
        for (int k = 0; k < 4; ++k) {
            const f3 dir = k == 0 ? e1 : (k == 1 ? e2 : (k == 2 ? neg3(e1) : neg3(e2)));
            const f3 v{cc.x + dir.x * g.ext.x, cc.y + dir.y * g.ext.x, cc.z + dir.z * g.ext.x};
            cand[cap * 4 + k] = v;
            depth[cap * 4 + k] = -dot(sub(v, pp), np);
        }
    }
    return deepestBelowPlane(cand, depth, 8, np, out, spec);
}

// Convex hull against the plane: its deepest four vertices at or below the plane.
__device__ __forceinline__ bool convexPlane(axd::f3 pp, axd::f3 np, const Geom& g, Contact* out,
                                            float spec = 0.0f) {
    using namespace axd;
    const float4* v = g.verts + hullOffset(g);
    const uint32_t n = hullCount(g);
    const f3 c = mk(g.pos);
    int best[4];
    float bd[4];
    int nb = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const f3 w = add(c, rotate(g.rot, mk(v[i])));
        const float d = -dot(sub(w, pp), np);
        if (!(d >= -spec)) continue;
        int at = nb;
        while (at > 0 && d > bd[at - 1]) --at;
        if (at >= 4) continue;
        for (int j = (nb < 4 ? nb : 3); j > at; --j) {
            best[j] = best[j - 1];
            bd[j] = bd[j - 1];
        }
        best[at] = (int)i;
        bd[at] = d;
        nb = nb < 4 ? nb + 1 : 4;
    }
    if (nb == 0) return false;
    for (int i = 1; i < nb; ++i)
        for (int j = i; j > 0 && best[j] < best[j - 1]; --j) {
            const int t = best[j];
            best[j] = best[j - 1];
            best[j - 1] = t;
            const float td = bd[j];
            bd[j] = bd[j - 1];
            bd[j - 1] = td;
        }
    out->n = np;
    out->count = (uint32_t)nb;
    for (int i = 0; i < nb; ++i) {
        const f3 w = add(c, rotate(g.rot, mk(v[best[i]])));
        const float h = 0.5f * bd[i];
        out->p[i] = f3{w.x + np.x * h, w.y + np.y * h, w.z + np.z * h};
        out->depth[i] = bd[i];
    }
    return true;
}

// Pairs that go through GJK + EPA: box-box, box-capsule, and every pair with a cylinder or
// a convex hull except sphere-cylinder (analytic).
__device__ __forceinline__ bool isGjkPair(uint32_t sa, uint32_t sb) {
    if (sa == AXIOM_SHAPE_PLANE || sb == AXIOM_SHAPE_PLANE) return false;
    const bool ext = sa == AXIOM_SHAPE_CYLINDER || sb == AXIOM_SHAPE_CYLINDER || isHullShape(sa) ||
                     isHullShape(sb);
    if (ext)
        return !((sa == AXIOM_SHAPE_SPHERE && sb == AXIOM_SHAPE_CYLINDER) ||
                 (sa == AXIOM_SHAPE_CYLINDER && sb == AXIOM_SHAPE_SPHERE));
    return (sa == AXIOM_SHAPE_BOX && (sb == AXIOM_SHAPE_BOX || sb == AXIOM_SHAPE_CAPSULE)) ||
           (sa == AXIOM_SHAPE_CAPSULE && sb == AXIOM_SHAPE_BOX);
}

// Analytic shape pairs; the normal points from a to b.  The GJK pairs are not handled here
// (isGjkPair).  spec: the speculative distance of the pair (pos.w holds each body's sweep).
__device__ __forceinline__ void collidePair(const Geom& a, const Geom& b, Contact* c) {
    using namespace axd;
    c->count = 0;
    const uint32_t sa = a.shape, sb = b.shape;
    const float spec = a.pos.w + b.pos.w;
    bool hit = false, flip = false;
    if (sa == AXIOM_SHAPE_SPHERE && sb == AXIOM_SHAPE_SPHERE) {
        hit = sphereSphere(mk(a.pos), a.ext.x, mk(b.pos), b.ext.x, c, spec);
    } else if (sa == AXIOM_SHAPE_SPHERE && sb == AXIOM_SHAPE_BOX) {
        hit = sphereBox(mk(a.pos), a.ext.x, mk(b.pos), b.rot, mk(b.ext), c, spec);
    } else if (sa == AXIOM_SHAPE_BOX && sb == AXIOM_SHAPE_SPHERE) {
        hit = sphereBox(mk(b.pos), b.ext.x, mk(a.pos), a.rot, mk(a.ext), c, spec);
        flip = true;
    } else if (sa == AXIOM_SHAPE_SPHERE && sb == AXIOM_SHAPE_CAPSULE) {
        f3 e0, e1;
        capsuleSegment(mk(b.pos), b.rot, b.ext.y, &e0, &e1);
        hit = sphereSphere(mk(a.pos), a.ext.x, closestOnSegment(mk(a.pos), e0, e1), b.ext.x, c, spec);
    } else if (sa == AXIOM_SHAPE_CAPSULE && sb == AXIOM_SHAPE_SPHERE) {
        f3 e0, e1;
        capsuleSegment(mk(a.pos), a.rot, a.ext.y, &e0, &e1);
        hit = sphereSphere(mk(b.pos), b.ext.x, closestOnSegment(mk(b.pos), e0, e1), a.ext.x, c, spec);
        flip = true;
    } else if (sa == AXIOM_SHAPE_CAPSULE && sb == AXIOM_SHAPE_CAPSULE) {
        f3 a0, a1, b0, b1, ca, cb;
        capsuleSegment(mk(a.pos), a.rot, a.ext.y, &a0, &a1);
        capsuleSegment(mk(b.pos), b.rot, b.ext.y, &b0, &b1);
        closestSegmentSegment(a0, a1, b0, b1, &ca, &cb);
        hit = sphereSphere(ca, a.ext.x, cb, b.ext.x, c, spec);
    } else if (sa == AXIOM_SHAPE_SPHERE && sb == AXIOM_SHAPE_CYLINDER) {
        hit = sphereCylinder(mk(a.pos), a.ext.x, mk(b.pos), b.rot, b.ext.x, b.ext.y, c, spec);
    } else if (sa == AXIOM_SHAPE_CYLINDER && sb == AXIOM_SHAPE_SPHERE) {
        hit = sphereCylinder(mk(b.pos), b.ext.x, mk(a.pos), a.rot, a.ext.x, a.ext.y, c, spec);
        flip = true;
    }
    if (hit && flip) c->n = neg3(c->n);
    if (!hit) c->count = 0;
}

// Plane (pp, np) against body g; the normal is the plane's (plane -> body).
__device__ __forceinline__ void collidePlane(axd::f3 pp, axd::f3 np, const Geom& g, Contact* c) {
    using namespace axd;
    c->count = 0;
    const float spec = g.pos.w;  // the body's sweep (planes do not move)
    if (g.shape == AXIOM_SHAPE_SPHERE) spherePlaneAppend(pp, np, mk(g.pos), g.ext.x, c, spec);
    else if (g.shape == AXIOM_SHAPE_BOX) boxPlane(pp, np, g, c, spec);
    else if (g.shape == AXIOM_SHAPE_CAPSULE) capsulePlane(pp, np, g, c, spec);
    else if (g.shape == AXIOM_SHAPE_CYLINDER) cylinderPlane(pp, np, g, c, spec);
    else if (isHullShape(g.shape)) convexPlane(pp, np, g, c, spec);
}

}  // namespace axiom_gb300
