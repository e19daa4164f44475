// batch.cu — thousands of independent worlds stepped by one persistent kernel.
//
// Each CTA pops a world from a queue ordered largest first (longest-processing-time
// order, so the big worlds do not finish last) and runs that world's whole step with
// CTA-local synchronisation: velocity integration and AABBs, an x-axis sweep-and-prune
// over a shared-memory bitonic sort of the AABB min corners, the narrowphase (analytic
// pairs per thread, GJK/EPA one warp per pair), Jones-Plassmann colouring, PGS prep, warm
// start, sweeps per colour, impulse storage and position integration.  Every phase uses
// the same device functions as the single-world step (integrate_math.cuh,
// narrow_shapes.cuh, gjk_epa.cuh, solver_math.cuh), so each world evolves exactly as a
// single world holding the same bodies.  The step is captured once as a CUDA graph and
// replayed; per-world step times come from %globaltimer.
//
// Limits: at most kBatchMaxBodies bodies and kBatchMaxPlanes planes per world (the sort
// lives in shared memory); the warm start is previous-step or none.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/axiom_c.h"
#include "body_pack.h"
#include "gjk_epa.cuh"
#include "integrate_math.cuh"
#include "solver_math.cuh"

namespace axiom_gb300 {
namespace {

constexpr uint32_t kBatchMaxBodies = 8192;
constexpr uint32_t kBatchMaxPlanes = 8;
constexpr uint32_t kBatchEpaWarps = 16;  // every warp of a 512-thread CTA runs GJK/EPA
constexpr uint32_t kBatchMaxRounds = 512;
// Worlds with at least this many bodies run in a lane of their own: a concurrent launch of
// 512-thread CTAs (one world each), so that the largest worlds, which bound the step, get
// the widest CTAs whatever launch shape suits the many small ones.
constexpr uint32_t kBigWorldBodies = 4096;
constexpr uint32_t kUnset = 0xFFFFFFFFu;
constexpr uint32_t kBadEntry = 0xFFFFFFFEu;  // a popped queue entry that names no world
constexpr size_t kSortBytes = sizeof(unsigned long long) * kBatchMaxBodies;
// Worlds of at most this many bodies can solve with their bodies in shared memory (the
// autotuner's largest staging choice; 32 bytes a body).
constexpr uint32_t kMaxStageBodies = 4096;
constexpr size_t kBatchSmemMax = 160u * 1024u;  // the kernel's dynamic shared memory opt-in

// Dynamic shared memory of a launch with `block` threads whose worlds have at most
// maxBodies bodies and stage up to stageBodies: the sort buffer (a power of two of 8-byte
// keys), one EPA polytope per warp, or the staged bodies, whichever is largest.  The
// phases use the region one after another.
inline size_t batchSmem(uint32_t block, uint32_t maxBodies, uint32_t stageBodies) {
    size_t p = 1;
    while (p < maxBodies) p <<= 1;
    const size_t warps = std::min<size_t>(block / 32u, kBatchEpaWarps);
    return std::max({sizeof(unsigned long long) * p, sizeof(EpaWarp) * warps, sizeof(SolverBody) * stageBodies});
}

enum : uint32_t {
    kWorldOverflowPairs = 1u,
    kWorldOverflowManifolds = 2u,
    kWorldOverflowPlanes = 4u,
    kWorldOverflowColours = 8u,
    kWorldOverflowRounds = 16u,
    kWorldNotConverged = 32u,
    kWorldGjkFailed = 64u,  // a pair's GJK ran out of iterations (treated as separated)
    kWorldEpaFailed = 128u  // a pair's EPA stopped at a cap (closest face found used)
};

struct WorldSlot {
    uint32_t bodyStart, bodyCount, pairStart, pairCap, manStart, manCap, tabStart, tabLog2;
};

constexpr int kBatchPhases = 7;  // see axiom_batch_read_phase_ns

struct WorldOut {
    uint32_t pairs, manifolds, points, colours, rounds, iterations, flags, gjk;
    float residual;
    uint32_t stamp;  // the step that wrote this record (a world left unstepped keeps an old one)
    unsigned long long ns;
    unsigned long long phase[kBatchPhases];
};

struct BatchDyn {  // changes every step; copied from pinned host memory inside the graph
    uint32_t wsCur, wsValid, stamp, pad;
};

// Work-queue counters: the two lanes' heads and the count of queue entries naming no world.
enum : uint32_t { kHeadMain = 0, kHeadBig = 1, kQueueBadEntries = 2, kQueueWords = 4 };

struct BatchPtrs {
    float4 *pos, *rot, *shp, *mat, *iloc, *iw0, *iw1, *aabbMin, *aabbMax;
    SolverBody* body;
    uint32_t* info;
    const uint4* filt;  // collision filters (read for bodies flagged kInfoFiltered)
    unsigned long long *prio0, *prio1, *mask;
    uint2 *pairs, *gjkq;
    uint4* mhdr;
    float4* mn;
    float4* mp[kMaxPoints];
    uint32_t* order;
    uint4* shdr;
    float4* sn;
    float4* sra[kMaxPoints];
    float4* srb[kMaxPoints];
    float2* skt[kMaxPoints];
    float4* slam[kMaxPoints];
    unsigned long long* wsKeys[2];
    float4* wsVals[2];
    const WorldSlot* worlds;
    WorldOut* out;
    const uint32_t* queueOrder;
    uint32_t* queueHead;
    uint32_t* queueBad;  // entries that named no world (a corrupted queue), counted and skipped
    const BatchDyn* dyn;
    uint32_t nWorlds, totalWorlds, warm, iterations, maxIterations, tolMode;
    uint32_t stageBodies;  // worlds of at most this many bodies solve with them in shared memory
    float tolerance;
};

__device__ __forceinline__ unsigned long long globalTimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t orderedBits(float x) {
    const uint32_t b = __float_as_uint(x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

struct BatchShared {
    uint32_t world, planeCount, planes[kBatchMaxPlanes];
    uint32_t pairs, gjk, manifolds, points, remain[2], maxColour, flags, rounds, iterations;
    uint32_t colStart[kMaxColours + 1], colCursor[kMaxColours];
    uint32_t delta, lambda;
    float residual;
    unsigned long long t0;
    unsigned long long tp[kBatchPhases];  // end of each phase (global timer)
};

// Marks the end of phase k; call right after a CTA barrier.
__device__ __forceinline__ void phaseMark(BatchShared& sh, int k) {
    if (threadIdx.x == 0) sh.tp[k] = globalTimer();
}

__device__ __forceinline__ void emitManifold(BatchShared& sh, const WorldSlot& W, const BatchPtrs& g, uint32_t a,
                                             uint32_t b, const Contact& c) {
    const uint32_t m = atomicAdd(&sh.manifolds, 1u);
    atomicAdd(&sh.points, c.count);
    if (m >= W.manCap) {
        atomicOr(&sh.flags, kWorldOverflowManifolds);
        return;
    }
    const uint32_t gm = W.manStart + m;
    g.mhdr[gm] = make_uint4(a, b, c.count, kUnset);
    g.mn[gm] = make_float4(c.n.x, c.n.y, c.n.z, 0.0f);
    for (uint32_t k = 0; k < c.count; ++k) g.mp[k][gm] = make_float4(c.p[k].x, c.p[k].y, c.p[k].z, c.depth[k]);
}

__global__ void __launch_bounds__(512) kBatchStep(BatchPtrs g, StepParams sp) {
    extern __shared__ __align__(16) unsigned char dynSmem[];
    unsigned long long* sortBuf = reinterpret_cast<unsigned long long*>(dynSmem);
    EpaWarp* epa = reinterpret_cast<EpaWarp*>(dynSmem);
    __shared__ BatchShared sh;
    const uint32_t tid = threadIdx.x, B = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t nWarps = B >> 5;
    const uint32_t wsCur = g.dyn->wsCur, wsValid = g.dyn->wsValid;
    for (;;) {
        if (tid == 0) {
            const uint32_t q = atomicAdd(g.queueHead, 1u);
            uint32_t wq = q < g.nWorlds ? g.queueOrder[q] : kUnset;
            if (wq != kUnset && wq >= g.totalWorlds) {
                atomicAdd(g.queueBad, 1u);
                wq = kBadEntry;
            }
            sh.world = wq;
            sh.t0 = globalTimer();
            sh.planeCount = sh.pairs = sh.gjk = sh.manifolds = sh.points = 0;
            sh.remain[0] = sh.remain[1] = 0;
            sh.maxColour = sh.flags = sh.rounds = sh.iterations = 0;
            sh.delta = sh.lambda = 0;
            sh.residual = 0.0f;
        }
        __syncthreads();
        const uint32_t wi = sh.world;
        if (wi == kUnset) break;
        if (wi == kBadEntry) {
            __syncthreads();  // every thread has read sh.world before thread 0 pops again
            continue;
        }
        const WorldSlot W = g.worlds[wi];
        const uint32_t n = W.bodyCount;
        float4* pos = g.pos + W.bodyStart;
        float4* rot = g.rot + W.bodyStart;
        const float4* shp = g.shp + W.bodyStart;
        const float4* mat = g.mat + W.bodyStart;
        const float4* iloc = g.iloc + W.bodyStart;
        float4* iw0 = g.iw0 + W.bodyStart;
        float4* iw1 = g.iw1 + W.bodyStart;
        float4* aabbMin = g.aabbMin + W.bodyStart;
        float4* aabbMax = g.aabbMax + W.bodyStart;
        SolverBody* sb = g.body + W.bodyStart;
        const uint32_t* info = g.info + W.bodyStart;
        const uint4* filt = g.filt + W.bodyStart;

        // ---- velocities, AABBs, sort keys (AABB min.x) ----
        for (uint32_t i = tid; i < n; i += B) {
            velocityStep(i, sp, info, rot, sb, mat, iloc, iw0, iw1);
            const f3 mn = bodyAabb(i, sp, info, pos, rot, shp, aabbMin, aabbMax);
            if (((info[i] >> 4) & 0xFu) == AXIOM_SHAPE_PLANE) {
                const uint32_t slot = atomicAdd(&sh.planeCount, 1u);
                if (slot < kBatchMaxPlanes) sh.planes[slot] = i;
                else atomicOr(&sh.flags, kWorldOverflowPlanes);
                sortBuf[i] = ~0ull;
            } else {
                sortBuf[i] = ((unsigned long long)orderedBits(mn.x) << 32) | i;
            }
        }
        uint32_t P = 2;
        while (P < n) P <<= 1;
        for (uint32_t i = n + tid; i < P; i += B) sortBuf[i] = ~0ull;
        __syncthreads();
        for (uint32_t k = 2; k <= P; k <<= 1)
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t i = tid; i < P; i += B) {
                    const uint32_t ixj = i ^ j;
                    if (ixj > i) {
                        const unsigned long long x = sortBuf[i], y = sortBuf[ixj];
                        const bool asc = (i & k) == 0;
                        if ((x > y) == asc) {
                            sortBuf[i] = y;
                            sortBuf[ixj] = x;
                        }
                    }
                }
                __syncthreads();
            }
        phaseMark(sh, 0);
        const uint32_t nPlanes = sh.planeCount < kBatchMaxPlanes ? sh.planeCount : kBatchMaxPlanes;
        const uint32_t nSorted = n - (sh.planeCount < n ? sh.planeCount : n);

        // ---- broadphase: sweep along x over the sorted min corners ----
        for (uint32_t i = tid; i < nSorted; i += B) {
            const uint32_t ia = (uint32_t)sortBuf[i];
            const float4 amn = aabbMin[ia], amx = aabbMax[ia];
            const bool dA = (info[ia] & kInfoTypeMask) == AXIOM_BODY_DYNAMIC;
            for (uint32_t j = i + 1; j < nSorted; ++j) {
                const uint32_t ib = (uint32_t)sortBuf[j];
                const float4 bmn = aabbMin[ib];
                if (bmn.x > amx.x) break;
                const float4 bmx = aabbMax[ib];
                const bool dB = (info[ib] & kInfoTypeMask) == AXIOM_BODY_DYNAMIC;
                if (!(dA || dB)) continue;
                if (amn.x <= bmx.x && amx.x >= bmn.x && amn.y <= bmx.y && amx.y >= bmn.y && amn.z <= bmx.z &&
                    amx.z >= bmn.z) {
                    if (((info[ia] | info[ib]) & kInfoFiltered) && !filterPass(filt[ia], filt[ib])) continue;
                    const uint32_t k = atomicAdd(&sh.pairs, 1u);
                    if (k < W.pairCap) g.pairs[W.pairStart + k] = make_uint2(ia < ib ? ia : ib, ia < ib ? ib : ia);
                    else atomicOr(&sh.flags, kWorldOverflowPairs);
                }
            }
        }
        __syncthreads();
        phaseMark(sh, 1);
        const uint32_t nPairs = sh.pairs < W.pairCap ? sh.pairs : W.pairCap;

        // ---- narrowphase: analytic pairs and planes per thread ----
        for (uint32_t k = tid; k < nPairs; k += B) {
            const uint2 pr = g.pairs[W.pairStart + k];
            const uint32_t sa = (info[pr.x] >> 4) & 0xFu, sb2 = (info[pr.y] >> 4) & 0xFu;
            if (isGjkPair(sa, sb2)) {
                const uint32_t q = atomicAdd(&sh.gjk, 1u);
                g.gjkq[W.pairStart + q] = pr;
                continue;
            }
            const Geom ga{sa, pos[pr.x], rot[pr.x], shp[pr.x]};
            const Geom gb{sb2, pos[pr.y], rot[pr.y], shp[pr.y]};
            Contact c;
            collidePair(ga, gb, &c);
            if (c.count) emitManifold(sh, W, g, pr.x, pr.y, c);
        }
        for (uint32_t i = tid; i < n; i += B) {
            const uint32_t inf = info[i];
            const uint32_t shape = (inf >> 4) & 0xFu;
            if ((inf & kInfoTypeMask) != AXIOM_BODY_DYNAMIC || shape == AXIOM_SHAPE_PLANE) continue;
            const Geom gi{shape, pos[i], rot[i], shp[i]};
            for (uint32_t q = 0; q < nPlanes; ++q) {
                const uint32_t p = sh.planes[q];
                if (((inf | info[p]) & kInfoFiltered) && !filterPass(filt[p], filt[i])) continue;
                const float4 pp = pos[p];
                const f3 np = rotate(rot[p], f3{0.0f, 1.0f, 0.0f});
                Contact c;
                collidePlane(f3{pp.x, pp.y, pp.z}, np, gi, &c);
                if (c.count) emitManifold(sh, W, g, p, i, c);
            }
        }
        __syncthreads();
        phaseMark(sh, 2);
        // ---- narrowphase: GJK + EPA, up to 32 pairs to a warp (GJK and the manifold per lane,
        // EPA per warp; the sort buffer is free now) ----
        {
            const uint32_t nG = sh.gjk;
            const uint32_t epaWarps = nWarps < kBatchEpaWarps ? nWarps : kBatchEpaWarps;
            // pairs per warp: spread over the warps first, up to 32 when there are more
            const uint32_t per = min(32u, max(1u, (nG + epaWarps - 1u) / epaWarps));
            if (warp < epaWarps)
                for (uint32_t q0 = warp * per; q0 < nG; q0 += epaWarps * per) {
                    const uint32_t q = q0 + lane;
                    const bool active = lane < per && q < nG;
                    uint2 pr = make_uint2(0u, 0u);
                    Geom ga{}, gb{};
                    bool flip = false;
                    if (active) {
                        pr = g.gjkq[W.pairStart + q];
                        ga = Geom{(info[pr.x] >> 4) & 0xFu, pos[pr.x], rot[pr.x], shp[pr.x]};
                        gb = Geom{(info[pr.y] >> 4) & 0xFu, pos[pr.y], rot[pr.y], shp[pr.y]};
                        flip = ga.shape == AXIOM_SHAPE_CAPSULE;
                    }
                    // A is a box: box-box or box-capsule
                    const Geom& A = flip ? gb : ga;
                    const Geom& Bg = flip ? ga : gb;
                    const uint32_t kind = Bg.shape == AXIOM_SHAPE_BOX ? kPairBoxBox : kPairBoxCapsule;
                    uint32_t fail = 0;
                    Contact c = lanePairs(active, kind, A, Bg, epa[warp], lane, &fail);
                    if (flip) c.n = neg3(c.n);
                    if (fail & kFailGjk) atomicOr(&sh.flags, kWorldGjkFailed);
                    if (fail & kFailEpa) atomicOr(&sh.flags, kWorldEpaFailed);
                    if (c.count > 0) emitManifold(sh, W, g, pr.x, pr.y, c);
                    __syncwarp();
                }
        }
        __syncthreads();
        phaseMark(sh, 3);
        const uint32_t nM = sh.manifolds < W.manCap ? sh.manifolds : W.manCap;

        // ---- colouring: Jones-Plassmann rounds with CTA barriers ----
        unsigned long long* prio[2] = {g.prio0 + W.bodyStart, g.prio1 + W.bodyStart};
        unsigned long long* mask = g.mask + W.bodyStart;
        uint4* mhdr = g.mhdr + W.manStart;
        for (uint32_t i = tid; i < n; i += B) {
            prio[0][i] = 0ull;
            prio[1][i] = 0ull;
            mask[i] = 0ull;
        }
        __syncthreads();
        uint32_t rounds = 0;
        for (uint32_t r = 0; r < kBatchMaxRounds && nM > 0; ++r) {
            unsigned long long* Pr = prio[r & 1u];
            unsigned long long* Pn = prio[(r + 1u) & 1u];
            if (tid == 0) sh.remain[r & 1u] = 0;
            for (uint32_t m = tid; m < nM; m += B) {
                const uint4 h = mhdr[m];
                if (h.w != kUnset) continue;
                const unsigned long long p = mix64(pairKey(h.x, h.y));
                if ((info[h.x] & kInfoTypeMask) == AXIOM_BODY_DYNAMIC) atomicMax(&Pr[h.x], p);
                if ((info[h.y] & kInfoTypeMask) == AXIOM_BODY_DYNAMIC) atomicMax(&Pr[h.y], p);
            }
            __syncthreads();
            for (uint32_t m = tid; m < nM; m += B) {
                const uint4 h = mhdr[m];
                if (h.w != kUnset) continue;
                const unsigned long long p = mix64(pairKey(h.x, h.y));
                const bool da = (info[h.x] & kInfoTypeMask) == AXIOM_BODY_DYNAMIC;
                const bool db = (info[h.y] & kInfoTypeMask) == AXIOM_BODY_DYNAMIC;
                if ((!da || Pr[h.x] == p) && (!db || Pr[h.y] == p)) {
                    const unsigned long long ma = da ? mask[h.x] : 0ull, mb = db ? mask[h.y] : 0ull;
                    const unsigned long long used = ma | mb;
                    uint32_t c;
                    if (used == ~0ull) {
                        atomicOr(&sh.flags, kWorldOverflowColours);
                        c = kMaxColours - 1;
                    } else {
                        c = (uint32_t)(__ffsll((long long)~used) - 1);
                    }
                    if (da) mask[h.x] = ma | (1ull << c);
                    if (db) mask[h.y] = mb | (1ull << c);
                    mhdr[m].w = c;
                    atomicMax(&sh.maxColour, c + 1u);
                } else {
                    Pn[h.x] = 0ull;
                    Pn[h.y] = 0ull;
                    atomicAdd(&sh.remain[r & 1u], 1u);
                }
            }
            __syncthreads();
            rounds = r + 1;
            if (sh.remain[r & 1u] == 0) break;
        }
        if (nM > 0 && rounds == kBatchMaxRounds && tid == 0) atomicOr(&sh.flags, kWorldOverflowRounds);
        const uint32_t nC = (nM > 0 && rounds == kBatchMaxRounds) ? (uint32_t)kMaxColours : sh.maxColour;

        // ---- manifolds grouped by colour ----
        uint32_t* order = g.order + W.manStart;
        if (tid < (uint32_t)kMaxColours) sh.colCursor[tid] = 0;
        __syncthreads();
        // a manifold left uncoloured by the round cap (flagged above) goes to the last colour
        auto colourOf = [&](uint32_t m) {
            const uint32_t c = mhdr[m].w;
            return c < (uint32_t)kMaxColours ? c : (uint32_t)kMaxColours - 1u;
        };
        for (uint32_t m = tid; m < nM; m += B) atomicAdd(&sh.colCursor[colourOf(m)], 1u);
        __syncthreads();
        if (tid == 0) {
            uint32_t run = 0;
            for (uint32_t c = 0; c < (uint32_t)kMaxColours; ++c) {
                sh.colStart[c] = run;
                const uint32_t cnt = sh.colCursor[c];
                sh.colCursor[c] = run;
                run += cnt;
            }
            sh.colStart[kMaxColours] = run;
        }
        __syncthreads();
        for (uint32_t m = tid; m < nM; m += B) order[atomicAdd(&sh.colCursor[colourOf(m)], 1u)] = m;
        __syncthreads();
        phaseMark(sh, 4);

        // ---- solver ----
        SolverPtrs sv;
        sv.hdr = g.shdr + W.manStart;
        sv.n = g.sn + W.manStart;
        for (int k = 0; k < kMaxPoints; ++k) {
            sv.ra[k] = g.sra[k] + W.manStart;
            sv.rb[k] = g.srb[k] + W.manStart;
            sv.kt[k] = g.skt[k] + W.manStart;
            sv.lam[k] = g.slam[k] + W.manStart;
        }
        const uint32_t prev = wsCur ^ 1u;
        PrepIn in{};
        in.mhdr = mhdr;
        in.mn = g.mn + W.manStart;
        for (int k = 0; k < kMaxPoints; ++k) in.mp[k] = g.mp[k] + W.manStart;
        in.info = info;
        in.pos = pos;
        in.sb = sb;
        in.iw0 = iw0;
        in.iw1 = iw1;
        in.mat = mat;
        in.wsKeys = g.wsKeys[prev] + W.tabStart;
        in.wsVals = g.wsVals[prev] + W.tabStart;
        in.wsLog2 = W.tabLog2;
        in.lookup = wsValid;
        in.usePrev = (g.warm == AXIOM_WARM_START_PREVIOUS && wsValid) ? 1u : 0u;
        in.feat = nullptr;
        for (uint32_t s = tid; s < nM; s += B) prepareManifold(s, order[s], nM, sp, in, sv);
        __syncthreads();
        // a world that fits solves with its bodies in the (now free) dynamic shared memory:
        // every body load and store of the warm start and the sweeps stays on chip
        SolverBody* vb = sb;
        if (n <= g.stageBodies) {
            SolverBody* staged = reinterpret_cast<SolverBody*>(dynSmem);
            for (uint32_t i = tid; i < n; i += B) staged[i] = sb[i];
            __syncthreads();
            vb = staged;
        }
        for (uint32_t c = 0; c < nC; ++c) {
            for (uint32_t s = sh.colStart[c] + tid; s < sh.colStart[c + 1]; s += B) warmManifold(s, sv, vb, iw0, iw1);
            __syncthreads();
        }
        const uint32_t maxIt = nM == 0 ? 0u : (g.tolMode ? g.maxIterations : g.iterations);
        uint32_t iters = 0;
        float residual = 0.0f;
        for (uint32_t it = 0; it < maxIt; ++it) {
            float gd = 0.0f, gl = 0.0f;
            for (uint32_t c = 0; c < nC; ++c) {
                for (uint32_t s = sh.colStart[c] + tid; s < sh.colStart[c + 1]; s += B)
                    solveManifold(s, sv, vb, iw0, iw1, gd, gl);
                __syncthreads();
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                gd = maxf(gd, __shfl_xor_sync(0xFFFFFFFFu, gd, off));
                gl = maxf(gl, __shfl_xor_sync(0xFFFFFFFFu, gl, off));
            }
            if (lane == 0) {
                atomicMax(&sh.delta, __float_as_uint(gd));
                atomicMax(&sh.lambda, __float_as_uint(gl));
            }
            __syncthreads();
            residual = __uint_as_float(sh.delta) / maxf(__uint_as_float(sh.lambda), 1e-6f);
            ++iters;
            __syncthreads();  // everyone has read the maxima
            if (tid == 0) {
                sh.delta = 0;
                sh.lambda = 0;
            }
            if (g.tolMode && residual <= g.tolerance) break;
        }
        if (g.tolMode && nM > 0 && residual > g.tolerance && tid == 0) atomicOr(&sh.flags, kWorldNotConverged);
        if (vb != sb) {
            __syncthreads();
            for (uint32_t i = tid; i < n; i += B) sb[i] = vb[i];
        }
        __syncthreads();
        phaseMark(sh, 5);

        // ---- impulses for the next step's warm start ----
        {
            unsigned long long* keys = g.wsKeys[wsCur] + W.tabStart;
            float4* vals = g.wsVals[wsCur] + W.tabStart;
            const uint32_t size = 1u << W.tabLog2, tmask = size - 1u;
            for (uint32_t i = tid; i < size; i += B) keys[i] = kEmpty64;
            __syncthreads();
            for (uint32_t s = tid; s < nM; s += B) {
                const uint4 h = sv.hdr[s];
                for (uint32_t k = 0; k < h.z; ++k) {
                    const uint64_t key = warmKey(h.x, h.y, k);
                    uint32_t hh = warmHash(key, W.tabLog2);
                    for (uint32_t probe = 0; probe <= tmask; ++probe) {
                        const unsigned long long old = atomicCAS(&keys[hh], kEmpty64, (unsigned long long)key);
                        if (old == kEmpty64 || old == key) {
                            vals[hh] = sv.lam[k][s];
                            break;
                        }
                        hh = (hh + 1u) & tmask;
                    }
                }
            }
        }
        // ---- positions ----
        for (uint32_t i = tid; i < n; i += B) positionStep(i, sp, info, pos, rot, sb);
        __syncthreads();
        if (tid == 0) {
            WorldOut o;
            o.pairs = sh.pairs;
            o.manifolds = sh.manifolds;
            o.points = sh.points;
            o.colours = nC;
            o.rounds = rounds;
            o.iterations = iters;
            o.flags = sh.flags;
            o.gjk = sh.gjk;
            o.residual = residual;
            o.stamp = g.dyn->stamp;
            const unsigned long long t1 = globalTimer();
            o.ns = t1 - sh.t0;
            sh.tp[kBatchPhases - 1] = t1;
            unsigned long long t = sh.t0;
            for (int k = 0; k < kBatchPhases; ++k) {
                o.phase[k] = sh.tp[k] - t;
                t = sh.tp[k];
            }
            g.out[wi] = o;
        }
    }
}

// ------------------------------------------------------------------ host side ----

struct Batch {
    axiom_world_config cfg{};
    cudaStream_t stream = nullptr;
    uint32_t nWorlds = 0, nBodies = 0;
    std::vector<WorldSlot> slots;
    std::vector<uint32_t> queueOrder;
    DevBuf<WorldSlot> dSlots;
    DevBuf<WorldOut> dOut;
    DevBuf<uint32_t> dQueue, dHead;
    DevBuf<BatchDyn> dDyn;
    BatchDyn* hDyn = nullptr;  // pinned
    DevBuf<float4> pos, rot, shp, mat, iloc, iw0, iw1, aabbMin, aabbMax;
    DevBuf<SolverBody> body;
    DevBuf<uint32_t> info, order;
    DevBuf<unsigned long long> prio0, prio1, mask, wsKeys[2];
    DevBuf<uint2> pairs, gjkq;
    DevBuf<uint4> mhdr, shdr, filt;
    DevBuf<float4> mn, sn, mp[kMaxPoints], sra[kMaxPoints], srb[kMaxPoints], slam[kMaxPoints], wsVals[2];
    DevBuf<float2> skt[kMaxPoints];
    uint64_t totalPairs = 0, totalMans = 0, totalTab = 0;
    uint32_t wsCur = 0;
    bool wsValid = false;
    uint32_t block = 256, ctasPerSm = 2;
    uint32_t stageBodies = 2048;        // main-lane worlds up to this size solve in shared memory
    uint32_t mainMaxBodies = 1, bigMaxBodies = 1;  // largest world of each lane
    uint32_t bigWorlds = 0;             // the first bigWorlds of queueOrder run in the big-world lane
    cudaStream_t side = nullptr;        // the big-world lane's stream
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaGraphExec_t graph = nullptr;
    float graphDt = 0.0f;
    uint32_t graphBlock = 0, graphCtas = 0, graphStage = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<WorldOut> hOut;
    uint32_t stamp = 0;                   // steps launched; each stepped world records it
    uint32_t hQueue[kQueueWords] = {};    // the queue counters after the last step
    uint32_t injectKind = 0, injectValue = 0;  // a queue fault to inject into the next step
};

// Dynamic shared memory of the main lane's launch.
inline size_t mainSmem(const Batch& b) {
    return batchSmem(b.block, b.mainMaxBodies, std::min(b.stageBodies, b.mainMaxBodies));
}

#define B_CUDA(call)                                                 \
    do {                                                             \
        if ((call) != cudaSuccess) return AXIOM_GPU_OPERATION_FAILED; \
    } while (0)

uint32_t log2Ceil(uint64_t v) {
    uint32_t l = 0;
    while ((1ull << l) < v) ++l;
    return l;
}

BatchPtrs makePtrs(Batch& b) {
    BatchPtrs g{};
    g.pos = b.pos.p;
    g.rot = b.rot.p;
    g.shp = b.shp.p;
    g.mat = b.mat.p;
    g.iloc = b.iloc.p;
    g.iw0 = b.iw0.p;
    g.iw1 = b.iw1.p;
    g.aabbMin = b.aabbMin.p;
    g.aabbMax = b.aabbMax.p;
    g.body = b.body.p;
    g.info = b.info.p;
    g.filt = b.filt.p;
    g.prio0 = b.prio0.p;
    g.prio1 = b.prio1.p;
    g.mask = b.mask.p;
    g.pairs = b.pairs.p;
    g.gjkq = b.gjkq.p;
    g.mhdr = b.mhdr.p;
    g.mn = b.mn.p;
    g.order = b.order.p;
    g.shdr = b.shdr.p;
    g.sn = b.sn.p;
    for (int k = 0; k < kMaxPoints; ++k) {
        g.mp[k] = b.mp[k].p;
        g.sra[k] = b.sra[k].p;
        g.srb[k] = b.srb[k].p;
        g.skt[k] = b.skt[k].p;
        g.slam[k] = b.slam[k].p;
    }
    for (int k = 0; k < 2; ++k) {
        g.wsKeys[k] = b.wsKeys[k].p;
        g.wsVals[k] = b.wsVals[k].p;
    }
    g.worlds = b.dSlots.p;
    g.out = b.dOut.p;
    g.queueOrder = b.dQueue.p;
    g.queueHead = b.dHead.p + kHeadMain;
    g.queueBad = b.dHead.p + kQueueBadEntries;
    g.dyn = b.dDyn.p;
    g.nWorlds = b.nWorlds;
    g.totalWorlds = b.nWorlds;
    g.warm = b.cfg.warm_start;
    g.iterations = b.cfg.velocity_iterations;
    g.maxIterations = b.cfg.max_iterations;
    g.tolMode = b.cfg.residual_tolerance > 0.0f ? 1u : 0u;
    g.tolerance = b.cfg.residual_tolerance;
    return g;
}

StepParams batchParams(const Batch& b, float dt) {
    StepParams sp{};
    sp.dt = dt;
    sp.invDt = 1.0f / dt;
    sp.hdt = 0.5f * dt;
    sp.gx = b.cfg.gravity[0];
    sp.gy = b.cfg.gravity[1];
    sp.gz = b.cfg.gravity[2];
    sp.biasCoeff = b.cfg.baumgarte * sp.invDt;
    sp.slop = b.cfg.linear_slop;
    sp.margin = b.cfg.aabb_margin;
    sp.restThreshold = b.cfg.restitution_threshold;
    sp.invCell = 1.0f;
    sp.warmFactor = b.cfg.warm_start_factor;
    sp.tolerance = b.cfg.residual_tolerance;
    sp.warmStart = b.cfg.warm_start;
    const float* gv = b.cfg.gravity;
    sp.gdt = sqrtf(gv[0] * gv[0] + gv[1] * gv[1] + gv[2] * gv[2]) * dt;
    return sp;
}

// headStart (uncaptured launches only) starts the main lane's queue counter there instead
// of at 0: the host-side queue fault of axiom_batch_inject_queue_fault.
int32_t launchStep(Batch& b, float dt, bool useGraph, const uint32_t* headStart = nullptr) {
    const StepParams sp = batchParams(b, dt);
    b.hDyn->wsCur = b.wsCur;
    b.hDyn->wsValid = b.wsValid ? 1u : 0u;
    b.hDyn->stamp = ++b.stamp;
    int dev = 0, sms = 0;
    B_CUDA(cudaGetDevice(&dev));
    B_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const uint32_t big = b.bigWorlds, rest = b.nWorlds - big;
    const uint32_t grid = std::min<uint32_t>((uint32_t)sms * b.ctasPerSm, std::max(rest, 1u));
    auto record = [&]() -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(b.dDyn.p, b.hDyn, sizeof(BatchDyn), cudaMemcpyHostToDevice, b.stream);
        if (e != cudaSuccess) return e;
        e = cudaMemsetAsync(b.dHead.p, 0, kQueueWords * sizeof(uint32_t), b.stream);
        if (e != cudaSuccess) return e;
        if (headStart) {
            e = cudaMemcpyAsync(b.dHead.p + kHeadMain, headStart, sizeof(uint32_t), cudaMemcpyHostToDevice, b.stream);
            if (e != cudaSuccess) return e;
        }
        if (big) {
            // the big-world lane: its own queue (the head of the largest-first order) and
            // counter, forked onto the side stream and joined before the step ends
            if ((e = cudaEventRecord(b.fork, b.stream)) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(b.side, b.fork, 0)) != cudaSuccess) return e;
            BatchPtrs gb = makePtrs(b);
            gb.nWorlds = big;
            gb.queueHead = b.dHead.p + kHeadBig;
            gb.stageBodies = 0;  // a world of 4,096 bodies or more does not fit
            kBatchStep<<<std::min<uint32_t>(big, (uint32_t)sms), 512, batchSmem(512, b.bigMaxBodies, 0), b.side>>>(
                gb, sp);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            if ((e = cudaEventRecord(b.join, b.side)) != cudaSuccess) return e;
        }
        if (rest) {
            BatchPtrs gm = makePtrs(b);
            gm.queueOrder += big;
            gm.nWorlds = rest;
            gm.stageBodies = std::min(b.stageBodies, b.mainMaxBodies);
            kBatchStep<<<grid, b.block, mainSmem(b), b.stream>>>(gm, sp);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        if (big) return cudaStreamWaitEvent(b.stream, b.join, 0);
        return cudaSuccess;
    };
    if (!useGraph || headStart) {
        B_CUDA(record());
        return AXIOM_SUCCESS;
    }
    if (!b.graph || b.graphDt != dt || b.graphBlock != b.block || b.graphCtas != b.ctasPerSm ||
        b.graphStage != b.stageBodies) {
        if (b.graph) cudaGraphExecDestroy(b.graph);
        b.graph = nullptr;
        cudaGraph_t gr = nullptr;
        B_CUDA(cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal));
        const cudaError_t e = record();
        const cudaError_t e2 = cudaStreamEndCapture(b.stream, &gr);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (gr) cudaGraphDestroy(gr);
            return AXIOM_GPU_OPERATION_FAILED;
        }
        const cudaError_t e3 = cudaGraphInstantiate(&b.graph, gr, 0);
        cudaGraphDestroy(gr);
        if (e3 != cudaSuccess) return AXIOM_GPU_OPERATION_FAILED;
        b.graphDt = dt;
        b.graphBlock = b.block;
        b.graphCtas = b.ctasPerSm;
        b.graphStage = b.stageBodies;
    }
    B_CUDA(cudaGraphLaunch(b.graph, b.stream));
    return AXIOM_SUCCESS;
}

// Device copies used by the autotuner to replay the same state for every candidate.
struct Snapshot {
    DevBuf<float4> pos, rot;
    DevBuf<SolverBody> body;
    DevBuf<unsigned long long> keys[2];
    DevBuf<float4> vals[2];
    uint32_t wsCur = 0;
    bool wsValid = false;
};

int32_t takeSnapshot(Batch& b, Snapshot& s, bool restore) {
    auto cp = [&](auto& dst, auto& src, size_t n) -> cudaError_t {
        return cudaMemcpyAsync(dst.p, src.p, n * sizeof(*src.p), cudaMemcpyDeviceToDevice, b.stream);
    };
    if (!restore) {
        B_CUDA(s.pos.reserve(b.nBodies));
        B_CUDA(s.rot.reserve(b.nBodies));
        B_CUDA(s.body.reserve(b.nBodies));
        for (int k = 0; k < 2; ++k) {
            B_CUDA(s.keys[k].reserve(b.totalTab));
            B_CUDA(s.vals[k].reserve(b.totalTab));
        }
        B_CUDA(cp(s.pos, b.pos, b.nBodies));
        B_CUDA(cp(s.rot, b.rot, b.nBodies));
        B_CUDA(cp(s.body, b.body, b.nBodies));
        for (int k = 0; k < 2; ++k) {
            B_CUDA(cp(s.keys[k], b.wsKeys[k], b.totalTab));
            B_CUDA(cp(s.vals[k], b.wsVals[k], b.totalTab));
        }
        s.wsCur = b.wsCur;
        s.wsValid = b.wsValid;
    } else {
        B_CUDA(cp(b.pos, s.pos, b.nBodies));
        B_CUDA(cp(b.rot, s.rot, b.nBodies));
        B_CUDA(cp(b.body, s.body, b.nBodies));
        for (int k = 0; k < 2; ++k) {
            B_CUDA(cp(b.wsKeys[k], s.keys[k], b.totalTab));
            B_CUDA(cp(b.wsVals[k], s.vals[k], b.totalTab));
        }
        b.wsCur = s.wsCur;
        b.wsValid = s.wsValid;
    }
    B_CUDA(cudaStreamSynchronize(b.stream));
    return AXIOM_SUCCESS;
}

}  // namespace
}  // namespace axiom_gb300

using namespace axiom_gb300;

extern "C" {

AXIOM_API int32_t axiom_batch_create(const axiom_world_config* config, void** batch) {
    if (!config || !batch) return AXIOM_NULL_POINTER;
    *batch = nullptr;
    // batched worlds do not sleep (a single world with the same bodies would)
    if (!(config->time_step > 0.0f) || config->warm_start == AXIOM_WARM_START_LEARNED || config->allow_sleep ||
        config->temporal_colouring)
        return AXIOM_INVALID_PARAMETER;
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) return AXIOM_GPU_OPERATION_FAILED;
    if (config->device >= dev) return AXIOM_INVALID_PARAMETER;
    if (config->device >= 0 && cudaSetDevice(config->device) != cudaSuccess) return AXIOM_GPU_OPERATION_FAILED;
    Batch* b = new (std::nothrow) Batch();
    if (!b) return AXIOM_OUT_OF_MEMORY;
    b->cfg = *config;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost(&b->hDyn, sizeof(BatchDyn)) != cudaSuccess || cudaEventCreate(&b->ev0) != cudaSuccess ||
        cudaEventCreate(&b->ev1) != cudaSuccess ||
        cudaFuncSetAttribute(kBatchStep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBatchSmemMax) !=
            cudaSuccess) {
        delete b;
        return AXIOM_GPU_OPERATION_FAILED;
    }
    *batch = b;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_batch_destroy(void* batch) {
    Batch* b = static_cast<Batch*>(batch);
    if (!b) return AXIOM_SUCCESS;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->join) cudaEventDestroy(b->join);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->hDyn) cudaFreeHost(b->hDyn);
    DevBuf<float4>* f4[] = {&b->pos, &b->rot, &b->shp, &b->mat, &b->iloc, &b->iw0, &b->iw1, &b->aabbMin,
                            &b->aabbMax, &b->mn, &b->sn, &b->wsVals[0], &b->wsVals[1]};
    for (auto* x : f4) x->release();
    for (int k = 0; k < kMaxPoints; ++k) {
        b->mp[k].release();
        b->sra[k].release();
        b->srb[k].release();
        b->slam[k].release();
        b->skt[k].release();
    }
    b->body.release();
    b->info.release();
    b->filt.release();
    b->order.release();
    b->prio0.release();
    b->prio1.release();
    b->mask.release();
    b->wsKeys[0].release();
    b->wsKeys[1].release();
    b->pairs.release();
    b->gjkq.release();
    b->mhdr.release();
    b->shdr.release();
    b->dSlots.release();
    b->dOut.release();
    b->dQueue.release();
    b->dHead.release();
    b->dDyn.release();
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return AXIOM_SUCCESS;
}

// Sets the worlds of the batch (replacing any previous ones): world w owns bodies
// [sum(sizes[0..w)), +sizes[w]) of the description, with world-local body ids.
AXIOM_API int32_t axiom_batch_set_worlds(void* batch, const axiom_body_soa* bodies, const uint32_t* sizes,
                                         uint32_t worlds) {
    Batch* b = static_cast<Batch*>(batch);
    if (!b || !bodies || !sizes) return AXIOM_NULL_POINTER;
    if (worlds == 0) return AXIOM_INVALID_PARAMETER;
    uint64_t total = 0;
    for (uint32_t w = 0; w < worlds; ++w) {
        if (sizes[w] == 0 || sizes[w] > kBatchMaxBodies) return AXIOM_INVALID_PARAMETER;
        total += sizes[w];
    }
    if (total >= (1ull << 31)) return AXIOM_OUT_OF_RANGE;
    int32_t st = validateBodies(bodies, (uint32_t)total);
    if (st != AXIOM_SUCCESS) return st;
    b->nWorlds = worlds;
    b->nBodies = (uint32_t)total;
    b->slots.resize(worlds);
    uint64_t body = 0, pairs = 0, mans = 0, tab = 0;
    for (uint32_t w = 0; w < worlds; ++w) {
        WorldSlot& s = b->slots[w];
        const uint32_t n = sizes[w];
        s.bodyStart = (uint32_t)body;
        s.bodyCount = n;
        s.pairStart = (uint32_t)pairs;
        s.pairCap = 24u * n + 32u;
        s.manStart = (uint32_t)mans;
        s.manCap = 4u * n + 32u;
        s.tabStart = (uint32_t)tab;
        s.tabLog2 = log2Ceil(8ull * s.manCap);
        body += n;
        pairs += s.pairCap;
        mans += s.manCap;
        tab += 1ull << s.tabLog2;
    }
    b->totalPairs = pairs;
    b->totalMans = mans;
    b->totalTab = tab;
    // largest first: the longest worlds start first so that they do not finish last
    b->queueOrder.resize(worlds);
    for (uint32_t w = 0; w < worlds; ++w) b->queueOrder[w] = w;
    std::stable_sort(b->queueOrder.begin(), b->queueOrder.end(),
                     [&](uint32_t x, uint32_t y) { return sizes[x] > sizes[y]; });
    b->bigWorlds = 0;
    while (b->bigWorlds < worlds && sizes[b->queueOrder[b->bigWorlds]] >= kBigWorldBodies) ++b->bigWorlds;
    b->bigMaxBodies = b->bigWorlds ? sizes[b->queueOrder[0]] : 1u;
    b->mainMaxBodies = b->bigWorlds < worlds ? sizes[b->queueOrder[b->bigWorlds]] : 1u;
    if (b->graph) cudaGraphExecDestroy(b->graph);  // the lanes changed
    b->graph = nullptr;
    PackedBodies pk;
    packBodies(bodies, 0, (uint32_t)total, &pk);
    const size_t N = total;
    DevBuf<float4>* bodyF4[] = {&b->pos, &b->rot, &b->shp, &b->mat, &b->iloc, &b->iw0, &b->iw1, &b->aabbMin, &b->aabbMax};
    for (auto* x : bodyF4) B_CUDA(x->reserve(N));
    B_CUDA(b->body.reserve(N));
    B_CUDA(b->info.reserve(N));
    B_CUDA(b->filt.reserve(N));
    B_CUDA(b->prio0.reserve(N));
    B_CUDA(b->prio1.reserve(N));
    B_CUDA(b->mask.reserve(N));
    B_CUDA(b->pairs.reserve(pairs));
    B_CUDA(b->gjkq.reserve(pairs));
    B_CUDA(b->mhdr.reserve(mans));
    B_CUDA(b->shdr.reserve(mans));
    B_CUDA(b->mn.reserve(mans));
    B_CUDA(b->sn.reserve(mans));
    B_CUDA(b->order.reserve(mans));
    for (int k = 0; k < kMaxPoints; ++k) {
        B_CUDA(b->mp[k].reserve(mans));
        B_CUDA(b->sra[k].reserve(mans));
        B_CUDA(b->srb[k].reserve(mans));
        B_CUDA(b->skt[k].reserve(mans));
        B_CUDA(b->slam[k].reserve(mans));
    }
    for (int k = 0; k < 2; ++k) {
        B_CUDA(b->wsKeys[k].reserve(tab));
        B_CUDA(b->wsVals[k].reserve(tab));
        B_CUDA(cudaMemsetAsync(b->wsKeys[k].p, 0xFF, tab * 8, b->stream));
    }
    B_CUDA(b->dSlots.reserve(worlds));
    B_CUDA(b->dOut.reserve(worlds));
    B_CUDA(b->dQueue.reserve(worlds));
    B_CUDA(b->dHead.reserve(kQueueWords));
    B_CUDA(b->dDyn.reserve(1));
    cudaStream_t s = b->stream;
    auto up = [&](auto& d, const auto& h) {
        return cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(h[0]), cudaMemcpyHostToDevice, s);
    };
    B_CUDA(up(b->pos, pk.pos));
    B_CUDA(up(b->rot, pk.rot));
    B_CUDA(up(b->shp, pk.shp));
    B_CUDA(up(b->mat, pk.mat));
    B_CUDA(up(b->iloc, pk.iloc));
    B_CUDA(up(b->body, pk.body));
    B_CUDA(up(b->info, pk.info));
    B_CUDA(up(b->filt, pk.filt));
    B_CUDA(cudaMemsetAsync(b->iw0.p, 0, N * 16, s));
    B_CUDA(cudaMemsetAsync(b->iw1.p, 0, N * 16, s));
    B_CUDA(up(b->dSlots, b->slots));
    B_CUDA(up(b->dQueue, b->queueOrder));
    B_CUDA(cudaStreamSynchronize(s));
    b->wsValid = false;
    b->wsCur = 0;
    b->hOut.assign(worlds, WorldOut{});
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return AXIOM_SUCCESS;
}

// One step of every world.  stats->total_step_time is the device time of the launch;
// per-world results are read with axiom_batch_read_world_stats.
AXIOM_API int32_t axiom_batch_step(void* batch, float dt, axiom_step_stats* stats) {
    Batch* b = static_cast<Batch*>(batch);
    if (!b) return AXIOM_NULL_POINTER;
    if (b->nWorlds == 0) return AXIOM_INVALID_PARAMETER;
    if (!(dt > 0.0f)) dt = b->cfg.time_step;
    const uint32_t inject = b->injectKind, injectValue = b->injectValue;
    b->injectKind = 0;
    const uint32_t badSlot = b->bigWorlds + injectValue;
    if (inject == 2) {  // host-side fault injection: one queue entry names no world
        const uint32_t bad = 0xFFFFFFF0u;
        B_CUDA(cudaMemcpyAsync(b->dQueue.p + badSlot, &bad, sizeof(uint32_t), cudaMemcpyHostToDevice, b->stream));
    }
    B_CUDA(cudaEventRecord(b->ev0, b->stream));
    int32_t st = launchStep(*b, dt, true, inject == 1 ? &injectValue : nullptr);
    if (st != AXIOM_SUCCESS) return st;
    B_CUDA(cudaEventRecord(b->ev1, b->stream));
    B_CUDA(cudaMemcpyAsync(b->hOut.data(), b->dOut.p, sizeof(WorldOut) * b->nWorlds, cudaMemcpyDeviceToHost,
                           b->stream));
    B_CUDA(cudaMemcpyAsync(b->hQueue, b->dHead.p, sizeof(b->hQueue), cudaMemcpyDeviceToHost, b->stream));
    if (inject == 2)
        B_CUDA(cudaMemcpyAsync(b->dQueue.p + badSlot, &b->queueOrder[badSlot], sizeof(uint32_t),
                               cudaMemcpyHostToDevice, b->stream));
    B_CUDA(cudaStreamSynchronize(b->stream));
    b->wsValid = true;
    b->wsCur ^= 1u;
    int32_t status = AXIOM_SUCCESS;
    axiom_step_stats o;
    std::memset(&o, 0, sizeof(o));
    o.total_bodies = b->nBodies;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    o.total_step_time = ms;
    o.solver_time = ms;
    float worst = 0.0f;
    for (const WorldOut& w : b->hOut) {
        o.pair_count += w.pairs;
        o.manifold_count += w.manifolds;
        o.contact_point_count += w.points;
        o.colour_count = std::max(o.colour_count, w.colours);
        o.iterations = std::max(o.iterations, w.iterations);
        o.colour_rounds = std::max(o.colour_rounds, w.rounds);
        worst = std::max(worst, w.residual);
        if (w.flags & (kWorldOverflowPairs | kWorldOverflowManifolds | kWorldOverflowPlanes | kWorldOverflowColours |
                       kWorldOverflowRounds))
            status = AXIOM_OUT_OF_RANGE;
        else if ((w.flags & kWorldNotConverged) && status == AXIOM_SUCCESS)
            status = AXIOM_CONSTRAINT_SOLVER_FAILURE;
        o.gjk_failures += (w.flags & kWorldGjkFailed) ? 1u : 0u;  // worlds with a failed pair
        o.epa_failures += (w.flags & kWorldEpaFailed) ? 1u : 0u;
    }
    if (status == AXIOM_SUCCESS && o.gjk_failures) status = AXIOM_GJK_FAILED_TO_CONVERGE;
    if (status == AXIOM_SUCCESS && o.epa_failures) status = AXIOM_EPA_FAILED_TO_CONVERGE;
    // work-queue integrity: every world stepped once, every popped entry named a world
    uint32_t unstepped = 0;
    for (const WorldOut& w : b->hOut) unstepped += w.stamp != b->stamp ? 1u : 0u;
    if (b->hQueue[kQueueBadEntries]) status = AXIOM_GPU_INVALID_OPERATION;
    else if (unstepped) status = AXIOM_GPU_OPERATION_FAILED;
    o.residual = worst;
    o.status = status;
    if (stats) *stats = o;
    return status;
}

// Host-side fault injection into the next step's work queue (tests of the failure checks
// above): kind 1 starts the main lane's counter at `value`, kind 2 makes main-lane entry
// `value` name no world.  Memory stays in bounds either way: the kernel checks each entry.
AXIOM_API int32_t axiom_batch_inject_queue_fault(void* batch, uint32_t kind, uint32_t value) {
    Batch* b = static_cast<Batch*>(batch);
    if (!b) return AXIOM_NULL_POINTER;
    if (b->nWorlds == 0) return AXIOM_INVALID_PARAMETER;
    const uint32_t lane = b->nWorlds - b->bigWorlds;
    if ((kind != 1 && kind != 2) || (kind == 2 && value >= lane)) return AXIOM_INVALID_PARAMETER;
    b->injectKind = kind;
    b->injectValue = value;
    return AXIOM_SUCCESS;
}

// Per-world results of the last step: counts [worlds][8] = (pairs, manifolds, points,
// colours, colouring rounds, iterations, flags, gjk pairs), step_ns [worlds], residual
// [worlds].  Any pointer may be NULL.
AXIOM_API int32_t axiom_batch_read_world_stats(void* batch, uint32_t* counts, uint64_t* step_ns, float* residual) {
    Batch* b = static_cast<Batch*>(batch);
    if (!b) return AXIOM_NULL_POINTER;
    for (uint32_t w = 0; w < b->nWorlds; ++w) {
        const WorldOut& o = b->hOut[w];
        if (counts) {
            uint32_t* c = counts + 8ull * w;
            c[0] = o.pairs;
            c[1] = o.manifolds;
            c[2] = o.points;
            c[3] = o.colours;
            c[4] = o.rounds;
            c[5] = o.iterations;
            c[6] = o.flags;
            c[7] = o.gjk;
        }
        if (step_ns) step_ns[w] = o.ns;
        if (residual) residual[w] = o.residual;
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_batch_read_phase_ns(void* batch, uint64_t* phase_ns) {
    Batch* b = static_cast<Batch*>(batch);
    if (!b) return AXIOM_NULL_POINTER;
    if (!phase_ns) return AXIOM_NULL_POINTER;
    for (uint32_t w = 0; w < b->nWorlds; ++w)
        for (int k = 0; k < kBatchPhases; ++k) phase_ns[(size_t)kBatchPhases * w + k] = b->hOut[w].phase[k];
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_batch_read_state(void* batch, float* position, float* rotation, float* linear_velocity,
                                         float* angular_velocity) {
    Batch* b = static_cast<Batch*>(batch);
    if (!b) return AXIOM_NULL_POINTER;
    const size_t N = b->nBodies;
    std::vector<float4> p(N), q(N);
    std::vector<SolverBody> v(N);
    B_CUDA(cudaMemcpyAsync(p.data(), b->pos.p, N * 16, cudaMemcpyDeviceToHost, b->stream));
    B_CUDA(cudaMemcpyAsync(q.data(), b->rot.p, N * 16, cudaMemcpyDeviceToHost, b->stream));
    B_CUDA(cudaMemcpyAsync(v.data(), b->body.p, N * sizeof(SolverBody), cudaMemcpyDeviceToHost, b->stream));
    B_CUDA(cudaStreamSynchronize(b->stream));
    for (size_t i = 0; i < N; ++i) {
        if (position) {
            position[3 * i] = p[i].x;
            position[3 * i + 1] = p[i].y;
            position[3 * i + 2] = p[i].z;
        }
        if (rotation) std::memcpy(rotation + 4 * i, &q[i], 16);
        if (linear_velocity) {
            linear_velocity[3 * i] = v[i].v.x;
            linear_velocity[3 * i + 1] = v[i].v.y;
            linear_velocity[3 * i + 2] = v[i].v.z;
        }
        if (angular_velocity) {
            angular_velocity[3 * i] = v[i].w.x;
            angular_velocity[3 * i + 1] = v[i].w.y;
            angular_velocity[3 * i + 2] = v[i].w.z;
        }
    }
    return AXIOM_SUCCESS;
}

// Launch shape: threads per world (CTA size, a multiple of 32 up to 512) and resident
// CTAs per SM of the persistent grid.
AXIOM_API int32_t axiom_batch_set_launch(void* batch, uint32_t block, uint32_t ctas_per_sm) {
    Batch* b = static_cast<Batch*>(batch);
    if (!b) return AXIOM_NULL_POINTER;
    if (block == 0 || block % 32u || block > 512u || ctas_per_sm == 0 || ctas_per_sm > 8u)
        return AXIOM_INVALID_PARAMETER;
    int active = 0;
    const uint32_t stage = std::min(b->stageBodies, b->mainMaxBodies);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&active, kBatchStep, (int)block,
                                                      batchSmem(block, b->mainMaxBodies, stage)) != cudaSuccess)
        return AXIOM_GPU_OPERATION_FAILED;
    if ((uint32_t)active < ctas_per_sm) return AXIOM_OUT_OF_RANGE;
    b->block = block;
    b->ctasPerSm = ctas_per_sm;
    return AXIOM_SUCCESS;
}

// Colour-batch staging of the main lane: worlds of at most stage_bodies bodies run their
// warm start and sweeps with the bodies in shared memory (32 bytes a body; 0: none).  The
// shared memory this takes counts against the CTAs per SM of the launch shape.
AXIOM_API int32_t axiom_batch_set_stage(void* batch, uint32_t stage_bodies) {
    Batch* b = static_cast<Batch*>(batch);
    if (!b) return AXIOM_NULL_POINTER;
    if (stage_bodies > kMaxStageBodies) return AXIOM_INVALID_PARAMETER;
    const uint32_t old = b->stageBodies;
    b->stageBodies = stage_bodies;
    int active = 0;
    const uint32_t stage = std::min(stage_bodies, b->mainMaxBodies);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&active, kBatchStep, (int)b->block,
                                                      batchSmem(b->block, b->mainMaxBodies, stage)) != cudaSuccess) {
        b->stageBodies = old;
        return AXIOM_GPU_OPERATION_FAILED;
    }
    if ((uint32_t)active < b->ctasPerSm) {
        b->stageBodies = old;
        return AXIOM_OUT_OF_RANGE;
    }
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_batch_get_launch(void* batch, uint32_t* block, uint32_t* ctas_per_sm,
                                         uint32_t* stage_bodies) {
    Batch* b = static_cast<Batch*>(batch);
    if (!b) return AXIOM_NULL_POINTER;
    if (block) *block = b->block;
    if (ctas_per_sm) *ctas_per_sm = b->ctasPerSm;
    if (stage_bodies) *stage_bodies = b->stageBodies;
    return AXIOM_SUCCESS;
}

// Autotuner: times `trial_steps` steps of every feasible (block, CTAs per SM, staged
// bodies) on a snapshot of the current state, twice (the better of two interleaved rounds
// counts), keeps the fastest, restores the state.  The
// three trade against each other: wider CTAs run a world's colour batches with more
// threads, more CTAs per SM overlap more worlds, and staging more bodies in shared memory
// keeps more worlds' sweeps on chip but takes shared memory from the other CTAs.  A cache
// file (one "worlds bodies block ctas stage" line per tuned batch shape) skips the search
// when the same shape was tuned before; cache_path may be NULL.
AXIOM_API int32_t axiom_batch_autotune(void* batch, const char* cache_path, uint32_t trial_steps, uint32_t* block,
                                       uint32_t* ctas_per_sm) {
    Batch* b = static_cast<Batch*>(batch);
    if (!b) return AXIOM_NULL_POINTER;
    if (b->nWorlds == 0) return AXIOM_INVALID_PARAMETER;
    auto apply = [&](uint32_t bl, uint32_t ct, uint32_t sg) {
        int active = 0;
        const size_t smem = batchSmem(bl, b->mainMaxBodies, std::min(sg, b->mainMaxBodies));
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&active, kBatchStep, (int)bl, smem) != cudaSuccess ||
            (uint32_t)active < ct)
            return false;
        b->block = bl;
        b->ctasPerSm = ct;
        b->stageBodies = sg;
        return true;
    };
    if (cache_path) {
        std::ifstream in(cache_path);
        std::string line;
        while (std::getline(in, line)) {
            std::istringstream ls(line);
            uint64_t w = 0, n = 0;
            uint32_t bl = 0, ct = 0, sg = 0;
            if ((ls >> w >> n >> bl >> ct >> sg) && w == b->nWorlds && n == b->nBodies && bl % 32u == 0u &&
                bl >= 32u && bl <= 512u && ct >= 1u && ct <= 8u && sg <= kMaxStageBodies && apply(bl, ct, sg)) {
                if (block) *block = bl;
                if (ctas_per_sm) *ctas_per_sm = ct;
                return AXIOM_SUCCESS;
            }
        }
    }
    if (trial_steps == 0) trial_steps = 2;
    Snapshot snap;
    int32_t st = takeSnapshot(*b, snap, false);
    if (st != AXIOM_SUCCESS) return st;
    // every feasible shape, timed in two interleaved rounds from the same snapshot; a shape
    // keeps its better round, so that one slow trial does not decide between close shapes
    struct Shape {
        uint32_t block, ctas, stage;
        float ms;
    };
    std::vector<Shape> shapes;
    const uint32_t blocks[3] = {128, 256, 512};
    const uint32_t stages[4] = {0, 1024, 2048, kMaxStageBodies};
    for (uint32_t si = 0; si < 4; ++si) {
        const uint32_t sg = stages[si];
        if (si > 0 && stages[si - 1] >= b->mainMaxBodies) continue;  // stages every world, like the previous
        for (uint32_t bl : blocks)
            for (uint32_t ct = 1; ct <= 4; ++ct)
                if (apply(bl, ct, sg)) shapes.push_back(Shape{bl, ct, sg, 1e30f});
    }
    for (int round = 0; round < 2; ++round)
        for (Shape& sh : shapes) {
            apply(sh.block, sh.ctas, sh.stage);
            if ((st = takeSnapshot(*b, snap, true)) != AXIOM_SUCCESS) return st;
            float total = 0.0f;
            for (uint32_t k = 0; k < trial_steps; ++k) {
                B_CUDA(cudaEventRecord(b->ev0, b->stream));
                if ((st = launchStep(*b, b->cfg.time_step, false)) != AXIOM_SUCCESS) return st;
                B_CUDA(cudaEventRecord(b->ev1, b->stream));
                B_CUDA(cudaStreamSynchronize(b->stream));
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, b->ev0, b->ev1);
                total += ms;
                b->wsValid = true;
                b->wsCur ^= 1u;
            }
            sh.ms = std::min(sh.ms, total);
        }
    float best = 1e30f;
    uint32_t bestBlock = b->block, bestCtas = b->ctasPerSm, bestStage = b->stageBodies;
    for (const Shape& sh : shapes)
        if (sh.ms < best) {
            best = sh.ms;
            bestBlock = sh.block;
            bestCtas = sh.ctas;
            bestStage = sh.stage;
        }
    if ((st = takeSnapshot(*b, snap, true)) != AXIOM_SUCCESS) return st;
    b->block = bestBlock;
    b->ctasPerSm = bestCtas;
    b->stageBodies = bestStage;
    if (cache_path) {
        std::ofstream out(cache_path, std::ios::app);
        out << b->nWorlds << " " << b->nBodies << " " << bestBlock << " " << bestCtas << " " << bestStage << "\n";
    }
    if (block) *block = bestBlock;
    if (ctas_per_sm) *ctas_per_sm = bestCtas;
    return AXIOM_SUCCESS;
}

}  // extern "C"
