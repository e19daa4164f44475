// solver.cu — graph-coloured projected Gauss-Seidel with warm starting.
//
// The reference's solver is a 10-iteration no-op stub (examples/profiling_example.cpp:95-111)
// with velocityIterations = 8 by default (include/axiom/gui/physics_panel.hpp:37) and
// a reserved ConstraintSolverFailure code (include/axiom/core/error_code.hpp:42).
//
// Per contact point: a normal row (λn >= 0, Baumgarte bias = β/dt · max(depth - slop, 0),
// restitution bias above the threshold) then two friction rows box-clamped to
// |λt| <= μ λn, with μ = sqrt(μa μb).  One thread owns one manifold and walks its points
// in order.  Manifolds of one colour share no dynamic body, so a colour is one launch
// with no atomics and the result does not depend on the order inside a colour.
//
// Residual of a sweep = max|dλ| / max(max|λ|, 1e-6) over all rows (the warp max is
// folded into one atomicMax on the float bits, exact since max is order-free).
#include <algorithm>
#include <cstring>

#include "solver_math.cuh"

namespace axiom_gb300 {
namespace {

// One thread per manifold in narrowphase order: its records are read coalesced and its
// bodies are gathered with the narrowphase's spatial locality; the solver rows are
// scattered to the manifold's colour-order position s = inv[m].
__global__ void __launch_bounds__(256, 3) kPrepare(uint32_t nM, StepParams sp, const uint32_t* __restrict__ inv,
                                                PrepIn in, SolverPtrs out) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nM) return;
    prepareManifold(inv[m], m, nM, sp, in, out);
}

// Learned warm start: the network predicts the correction to the previous-step impulse in
// impulse-scale units (row = slot * nM + s); the start is factor x (prev + Y sImp),
// clamped to the cone the solver enforces.
// The network's rows are the contact points only: row list rows[q] = k * nM + s for every
// point k of every manifold s (in any order; each row's prediction depends on its features
// alone), and rowOf[k * nM + s] = q.
__global__ void __launch_bounds__(256) kLearnRows(uint32_t nM, const uint4* __restrict__ hdr,
                                                  uint32_t* __restrict__ rows, uint32_t* __restrict__ rowOf,
                                                  uint32_t* __restrict__ counter) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t k = r < 4u * nM ? r / nM : 0u, s = r < 4u * nM ? r % nM : 0u;
    const bool live = r < 4u * nM && k < hdr[s].z;
    const uint32_t q = axd::blockReserve(live ? 1u : 0u, counter);
    if (!live) return;
    rows[q] = r;
    rowOf[r] = q;
}

__global__ void __launch_bounds__(256) kApplyLearned(uint32_t nM, const float* __restrict__ Y,
                                                     const uint32_t* __restrict__ rowOf,
                                                     const float* __restrict__ feat, float factor,
                                                     SolverPtrs sv) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= 4u * nM) return;
    const uint32_t k = r / nM, s = r % nM;
    if (k >= sv.hdr[s].z) return;
    const size_t q = rowOf[r];
    const float sImp = feat[(size_t)r * 16u + 14u];
    const float mu = sv.n[s].w;
    const float4 prev = sv.lam[k][s];
    float ln = prev.x + Y[q * 3u] * sImp;
    ln = ln > 0.0f ? ln : 0.0f;
    const float mf = mu * ln;
    float l1 = prev.y + Y[q * 3u + 1u] * sImp;
    float l2 = prev.z + Y[q * 3u + 2u] * sImp;
    l1 = l1 > mf ? mf : (l1 < -mf ? -mf : l1);
    l2 = l2 > mf ? mf : (l2 < -mf ? -mf : l2);
    sv.lam[k][s] = make_float4(ln * factor, l1 * factor, l2 * factor, 0.0f);
}

// Closes one sweep: residual, iteration count, convergence flag.
__device__ __forceinline__ void closeSweep(DevCounters* cnt, float tol, uint32_t tolMode) {
    const float md = __uint_as_float(atomicAdd(&cnt->maxDeltaBits, 0u));
    const float ml = __uint_as_float(atomicAdd(&cnt->maxLambdaBits, 0u));
    const float r = md / maxf(ml, 1e-6f);
    cnt->residual = r;
    cnt->iterations += 1u;
    cnt->maxDeltaBits = 0u;
    cnt->maxLambdaBits = 0u;
    if (tolMode && r <= tol) cnt->converged = 1u;
}

// Closes a sweep that launched no colour (a step without manifolds).
__global__ void kEndSweep(DevCounters* cnt, float tol, uint32_t tolMode) {
    if (tolMode && cnt->converged) return;
    closeSweep(cnt, tol, tolMode);
}

// One PGS pass over colour c, sorted positions [colourStart[c], colourStart[c + 1]) (read
// from the colouring's counters, which no kernel of the solve writes).  The grid is one
// resident wave (blocks per SM x SMs) and strides over the colour, so a colour larger than
// a wave does not leave a partial last wave, and the launch does not depend on the
// colour's size.  In the last colour of a sweep (closing != 0) the block that
// finishes last closes the sweep: every block folds its maxima with atomics, fences, then
// takes a ticket; the holder of the last ticket sees all maxima.  No block waits.
//
// kWarm: the same pipelined pass applies the warm-start impulses instead of solving (no
// residual, no closing).  kHoist (worlds with multi-point manifolds): the rows of a
// manifold's points 1-3 are loaded before its first point is solved, with the registers of
// one CTA per SM instead of two.
template <bool kWarm, bool kHoist = false>
__global__ void __launch_bounds__(256, kHoist ? 1 : 2) kSolveColour(uint32_t c, DevCounters* __restrict__ cnt, SolverPtrs sv,
                                                       SolverBody* __restrict__ sb,
                                                       const float4* __restrict__ iw0,
                                                       const float4* __restrict__ iw1, uint32_t tolMode,
                                                       uint32_t closing, float tol, uint32_t earlyHead) {
    float gd = 0.0f, gl = 0.0f;
    const uint32_t begin = cnt->colourStart[c], end = cnt->colourStart[c + 1];
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t s = begin + blockIdx.x * blockDim.x + threadIdx.x;
    // software pipeline: the next manifold's head is in flight while this one waits on
    // its body gathers.  The first head does not depend on the kernel launched just
    // before this one (the previous colour: other manifolds, other impulses) unless that
    // kernel was this same colour (a one-colour sweep, earlyHead = 0), so it is fetched
    // before the dependency wait, overlapping the previous colour's tail.
    //
    // Pipeline over a thread's manifolds s, s + stride, ...: while manifold i is solved,
    // the bodies and solver rows of manifold i + 1 and the header of manifold i + 2 are in
    // flight.  Fetching i + 1's bodies before i is solved is safe: manifolds of one colour
    // share no dynamic body, so no other manifold writes them during this launch.
    ManifoldHead cur;
    if (earlyHead && s < end) cur = loadHeadStreaming(s, sv);
    gridDependencyWait();
    launchDependents();
    if (!kWarm && tolMode && cnt->converged) return;
    if (!earlyHead && s < end) cur = loadHeadStreaming(s, sv);
    BodyState A, B;
    if (s < end) loadBodies(cur.h.x, cur.h.y, sb, A, B);
    uint32_t s1 = s + stride;
    uint4 nextHdr = make_uint4(0u, 0u, 0u, 0u);
    if (s1 < end) nextHdr = __ldcs(&sv.hdr[s1]);
    while (s < end) {
        ManifoldHead nxt;
        BodyState NA, NB;
        if (s1 < end) {
            nxt.h = nextHdr;
            loadBodies(nxt.h.x, nxt.h.y, sb, NA, NB);
            loadHeadRestStreaming(s1, sv, nxt);
        }
        const uint32_t s2 = s1 + stride;
        if (s2 < end) nextHdr = __ldcs(&sv.hdr[s2]);
        if (kWarm) warmWithBodies(s, cur, A, B, sv, sb, iw0, iw1);
        else solveWithBodies<true, kHoist>(s, cur, A, B, sv, sb, iw0, iw1, gd, gl);
        s = s1;
        s1 = s2;
        cur = nxt;
        A = NA;
        B = NB;
    }
    if (kWarm) return;
    // block maxima first: two atomics per block instead of two per warp on the same words
    __shared__ float wd[8], wl[8];
    __shared__ uint32_t isLast;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        gd = maxf(gd, __shfl_xor_sync(0xFFFFFFFFu, gd, off));
        gl = maxf(gl, __shfl_xor_sync(0xFFFFFFFFu, gl, off));
    }
    if ((threadIdx.x & 31) == 0) {
        wd[threadIdx.x >> 5] = gd;
        wl[threadIdx.x >> 5] = gl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < 8; ++k) {
            gd = maxf(gd, wd[k]);
            gl = maxf(gl, wl[k]);
        }
        if (gd > 0.0f || gl > 0.0f) {
            atomicMax(&cnt->maxDeltaBits, __float_as_uint(gd));
            atomicMax(&cnt->maxLambdaBits, __float_as_uint(gl));
        }
    }
    if (!closing) return;
    if (threadIdx.x == 0) {
        __threadfence();
        isLast = atomicAdd(&cnt->sweepDone, 1u) == gridDim.x - 1u ? 1u : 0u;
        if (isLast) {
            __threadfence();
            closeSweep(cnt, tol, tolMode);
            cnt->sweepDone = 0u;
        }
    }
}

// ---- small worlds: the whole solve in one CTA ----
//
// A world of at most kSmallSolve manifolds and bodies runs its warm start, every sweep and
// (tolerance mode) the convergence test in one launch of one CTA: the bodies are copied to
// shared memory, colours follow each other at CTA barriers, the crowded batch (sorted here
// by descending priority) runs in thread 0 after the colours, and the colour count, the
// bounds and the convergence stay on the device, so the host needs no colour-count sync and
// no per-chunk sync.  Per body the updates come in the same order as in the colour
// launches, so the results are the same bits.
constexpr uint32_t kSmallSolve = 4096;
constexpr uint32_t kSmallSolveThreads = 512;

size_t smallSolveSmem(uint32_t n) {
    return sizeof(SolverBody) * (size_t)n + (sizeof(unsigned long long) + sizeof(uint32_t)) * kSmallSolve;
}

__global__ void __launch_bounds__(kSmallSolveThreads) kSolveSmall(DevCounters* __restrict__ cnt, SolverPtrs sv,
                                                                  SolverBody* __restrict__ sb,
                                                                  const float4* __restrict__ iw0,
                                                                  const float4* __restrict__ iw1,
                                                                  const uint32_t* __restrict__ order,
                                                                  const uint4* __restrict__ rec, uint32_t n,
                                                                  uint32_t sweeps, uint32_t tolMode, float tol) {
    extern __shared__ __align__(16) unsigned char smem[];
    SolverBody* vb = reinterpret_cast<SolverBody*>(smem);
    unsigned long long* ckey = reinterpret_cast<unsigned long long*>(smem + sizeof(SolverBody) * (size_t)n);
    uint32_t* cpos = reinterpret_cast<uint32_t*>(ckey + kSmallSolve);
    __shared__ uint32_t bounds[kMaxColours + 2];
    __shared__ float wd[kSmallSolveThreads / 32], wl[kSmallSolveThreads / 32];
    const uint32_t tid = threadIdx.x, B = blockDim.x;
    if (cnt->colourOverflow) return;  // no solve after a failed colouring (the same for every thread)
    for (uint32_t i = tid; i < (uint32_t)kMaxColours + 2u; i += B) bounds[i] = cnt->colourStart[i];
    for (uint32_t i = tid; i < n; i += B) vb[i] = sb[i];
    const uint32_t nC = cnt->maxColour;
    __syncthreads();
    // crowded batch: positions by ascending ~priority (priorities are distinct)
    const uint32_t c0 = bounds[kMaxColours], K = bounds[kMaxColours + 1] - c0;
    if (K > 0u) {
        uint32_t P = 1;
        while (P < K) P <<= 1;
        for (uint32_t q = tid; q < P; q += B) {
            if (q < K) {
                const uint4 r = rec[order[c0 + q]];
                ckey[q] = ~((unsigned long long)r.y << 32 | r.x);
            } else {
                ckey[q] = ~0ull;
            }
            cpos[q] = q;
        }
        __syncthreads();
        for (uint32_t k = 2; k <= P; k <<= 1)
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t i = tid; i < P; i += B) {
                    const uint32_t p = i ^ j;
                    if (p > i) {
                        const unsigned long long a = ckey[i], b = ckey[p];
                        if ((a > b) == ((i & k) == 0u)) {
                            ckey[i] = b;
                            ckey[p] = a;
                            const uint32_t t = cpos[i];
                            cpos[i] = cpos[p];
                            cpos[p] = t;
                        }
                    }
                }
                __syncthreads();
            }
    }
    // warm start
    for (uint32_t c = 0; c < nC; ++c) {
        for (uint32_t s = bounds[c] + tid; s < bounds[c + 1]; s += B) warmManifold(s, sv, vb, iw0, iw1);
        __syncthreads();
    }
    if (tid == 0)
        for (uint32_t q = 0; q < K; ++q) warmManifold(c0 + cpos[q], sv, vb, iw0, iw1);
    __syncthreads();
    // sweeps
    for (uint32_t it = 0; it < sweeps; ++it) {
        float gd = 0.0f, gl = 0.0f;
        for (uint32_t c = 0; c < nC; ++c) {
            for (uint32_t s = bounds[c] + tid; s < bounds[c + 1]; s += B) solveManifold(s, sv, vb, iw0, iw1, gd, gl);
            __syncthreads();
        }
        if (tid == 0)
            for (uint32_t q = 0; q < K; ++q) solveManifold(c0 + cpos[q], sv, vb, iw0, iw1, gd, gl);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            gd = maxf(gd, __shfl_xor_sync(0xFFFFFFFFu, gd, off));
            gl = maxf(gl, __shfl_xor_sync(0xFFFFFFFFu, gl, off));
        }
        if ((tid & 31u) == 0u) {
            wd[tid >> 5] = gd;
            wl[tid >> 5] = gl;
        }
        __syncthreads();
        float md = 0.0f, ml = 0.0f;
        for (uint32_t w = 0; w < B / 32u; ++w) {
            md = maxf(md, wd[w]);
            ml = maxf(ml, wl[w]);
        }
        const float r = md / maxf(ml, 1e-6f);
        if (tid == 0) {
            cnt->residual = r;
            cnt->iterations += 1u;
            if (tolMode && r <= tol) cnt->converged = 1u;
        }
        __syncthreads();  // wd / wl are read before the next sweep writes them
        if (tolMode && r <= tol) break;
    }
    for (uint32_t i = tid; i < n; i += B) sb[i] = vb[i];
}

// ---- mid-size worlds: the whole solve in one thread-block cluster ----
//
// A world of more than kSmallSolve and at most kClusterSolve manifolds (kClusterSolveSingle
// when all are single-point) runs its warm start,
// every sweep and (tolerance mode) the convergence test in one launch of one cluster of
// CTAs.  Colours follow each other at cluster barriers (barrier.cluster: arrive releases,
// wait acquires, at cluster scope, so the bodies one CTA writes in a colour are seen by
// every CTA in the next; without a crowded batch the barrier of the sweep maxima closes the
// last colour); the crowded batch (sorted here by descending priority, in global
// scratch, by CTA 0) runs in thread 0 of CTA 0 after the colours; each CTA folds its sweep
// maxima into one of three rotating counter pairs, which every thread reads after the next
// barrier, so that all of them take the same convergence decision.  The pair of sweep
// it + 1 is cleared in sweep it before that barrier: after the reads of sweep it - 2 (the
// last users of that pair, which all come before the previous barrier) and before the
// atomics of sweep it + 1, whether or not a sweep has colour barriers.  The host
// needs no colour-count sync and no per-chunk sync, as for a small world, and every barrier
// sits on control flow that all threads of the cluster follow alike.  Per body the updates
// come in the same order as in the colour launches, so the results are the same bits.
constexpr uint32_t kClusterSolve = 32768;        // manifolds, when some have several points
constexpr uint32_t kClusterSolveSingle = 65536;  // manifolds, when all have one point
constexpr uint32_t kClusterThreads = 256;  // up to 255 registers: the point rows are hoisted

__device__ __forceinline__ void clusterSync() {
    asm volatile("barrier.cluster.arrive;\n\tbarrier.cluster.wait;" ::: "memory");
}
__device__ __forceinline__ void clusterArrive() { asm volatile("barrier.cluster.arrive;" ::: "memory"); }
__device__ __forceinline__ void clusterWait() { asm volatile("barrier.cluster.wait;" ::: "memory"); }

__global__ void __launch_bounds__(kClusterThreads, 1) kSolveCluster(DevCounters* __restrict__ cnt, SolverPtrs sv,
                                                                    SolverBody* __restrict__ sb,
                                                                    const float4* __restrict__ iw0,
                                                                    const float4* __restrict__ iw1,
                                                                    const uint32_t* __restrict__ order,
                                                                    const uint4* __restrict__ rec,
                                                                    unsigned long long* __restrict__ ckey,
                                                                    uint32_t* __restrict__ cpos, uint32_t sweeps,
                                                                    uint32_t tolMode, float tol) {
    __shared__ uint32_t bounds[kMaxColours + 2];
    __shared__ float wd[kClusterThreads / 32], wl[kClusterThreads / 32];
    const uint32_t tid = threadIdx.x, B = blockDim.x;
    const uint32_t g = blockIdx.x * B + tid, T = gridDim.x * B;
    const bool lead = blockIdx.x == 0u;  // the grid is one cluster: CTA 0 is its rank 0
    // written before this launch, so every thread reads the same flag: all leave together
    if (cnt->colourOverflow) return;
    for (uint32_t i = tid; i < (uint32_t)kMaxColours + 2u; i += B) bounds[i] = cnt->colourStart[i];
    const uint32_t nC = cnt->maxColour;
    __syncthreads();
    // crowded batch: positions by ascending ~priority (priorities are distinct), sorted by CTA
    // 0 alone while the others start the warm start's first colour
    const uint32_t c0 = bounds[kMaxColours], K = bounds[kMaxColours + 1] - c0;
    if (lead && K > 0u) {
        uint32_t P = 1;
        while (P < K) P <<= 1;
        for (uint32_t q = tid; q < P; q += B) {
            if (q < K) {
                const uint4 r = rec[order[c0 + q]];
                ckey[q] = ~((unsigned long long)r.y << 32 | r.x);
            } else {
                ckey[q] = ~0ull;
            }
            cpos[q] = q;
        }
        __syncthreads();
        for (uint32_t k = 2; k <= P; k <<= 1)
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t i = tid; i < P; i += B) {
                    const uint32_t p = i ^ j;
                    if (p > i) {
                        const unsigned long long a = ckey[i], b = ckey[p];
                        if ((a > b) == ((i & k) == 0u)) {
                            ckey[i] = b;
                            ckey[p] = a;
                            const uint32_t t = cpos[i];
                            cpos[i] = cpos[p];
                            cpos[p] = t;
                        }
                    }
                }
                __syncthreads();
            }
    }
    // warm start
    for (uint32_t c = 0; c < nC; ++c) {
        for (uint32_t s = bounds[c] + g; s < bounds[c + 1]; s += T) warmManifold(s, sv, sb, iw0, iw1);
        clusterSync();
    }
    if (lead && tid == 0)
        for (uint32_t q = 0; q < K; ++q) warmManifold(c0 + cpos[q], sv, sb, iw0, iw1);
    clusterSync();
    // sweeps.  Between arriving at a barrier and waiting on it, a thread loads the head of
    // its first manifold of the colour the barrier opens: the rows do not change during the
    // solve, and the impulses are the thread's own, so only the bodies need the barrier.
    ManifoldHead pre;
    bool havePre = false;
    for (uint32_t it = 0; it < sweeps; ++it) {
        float gd = 0.0f, gl = 0.0f;
        for (uint32_t c = 0; c < nC; ++c) {
            uint32_t s = bounds[c] + g;
            if (s < bounds[c + 1]) {
                solveHead<false, true>(s, havePre ? pre : loadHead(s, sv), sv, sb, iw0, iw1, gd, gl);
                for (s += T; s < bounds[c + 1]; s += T) solveHead<false, true>(s, loadHead(s, sv), sv, sb, iw0, iw1, gd, gl);
            }
            havePre = false;
            if (c + 1u < nC || K > 0u) {  // else the maxima's barrier closes the colour
                clusterArrive();
                if (c + 1u < nC && bounds[c + 1] + g < bounds[c + 2]) {
                    pre = loadHead(bounds[c + 1] + g, sv);
                    havePre = true;
                }
                clusterWait();
            }
        }
        if (lead && tid == 0)
            for (uint32_t q = 0; q < K; ++q) solveManifold(c0 + cpos[q], sv, sb, iw0, iw1, gd, gl);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            gd = maxf(gd, __shfl_xor_sync(0xFFFFFFFFu, gd, off));
            gl = maxf(gl, __shfl_xor_sync(0xFFFFFFFFu, gl, off));
        }
        if ((tid & 31u) == 0u) {
            wd[tid >> 5] = gd;
            wl[tid >> 5] = gl;
        }
        __syncthreads();
        uint32_t* slot = cnt->clusterMax + 2u * (it % 3u);
        if (tid == 0) {
            float md = 0.0f, ml = 0.0f;
            for (uint32_t w = 0; w < B / 32u; ++w) {
                md = maxf(md, wd[w]);
                ml = maxf(ml, wl[w]);
            }
            if (md > 0.0f) atomicMax(&slot[0], __float_as_uint(md));  // non-negative: bits order as values
            if (ml > 0.0f) atomicMax(&slot[1], __float_as_uint(ml));
            if (lead) {
                uint32_t* next = cnt->clusterMax + 2u * ((it + 1u) % 3u);
                next[0] = 0u;
                next[1] = 0u;
            }
        }
        clusterArrive();
        if (nC > 0u && bounds[0] + g < bounds[1]) {  // the next sweep's first colour
            pre = loadHead(bounds[0] + g, sv);
            havePre = true;
        }
        clusterWait();
        // every thread reads the same two words: no CTA changes them before the next barrier
        const float r = __uint_as_float(__ldcg(&slot[0])) / maxf(__uint_as_float(__ldcg(&slot[1])), 1e-6f);
        if (lead && tid == 0) {
            cnt->residual = r;
            cnt->iterations += 1u;
            if (tolMode && r <= tol) cnt->converged = 1u;
        }
        if (tolMode && r <= tol) break;
    }
}

// Inserts this step's impulses into the warm-start table for the next step (generation
// gen of that table), with the manifold's colour (tag = 1 + colour) on its point 0.  The
// colour of sorted position s is the last colour whose first position is <= s.
__global__ void __launch_bounds__(256) kStoreImpulses(uint32_t nM, SolverPtrs sv, WarmSlot* __restrict__ slots,
                                                      uint32_t* __restrict__ claim, uint32_t gen, uint32_t log2T,
                                                      DevCounters* cnt) {
    __shared__ uint32_t bounds[kMaxColours + 1];
    __shared__ uint32_t nColours;
    if (cnt->colourOverflow) return;  // nothing solved after a failed colouring (small worlds)
    for (uint32_t i = threadIdx.x; i <= (uint32_t)kMaxColours; i += blockDim.x) bounds[i] = cnt->colourStart[i];
    if (threadIdx.x == 0) nColours = cnt->maxColour;
    __syncthreads();
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nM) return;
    uint32_t lo = 0, hi = nColours > 0u ? nColours : 1u;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (bounds[mid] <= s) lo = mid;
        else hi = mid;
    }
    const uint32_t tag = s < bounds[kMaxColours] ? lo + 1u : 0u;  // crowded manifolds have no colour
    const uint4 h = sv.hdr[s];
    for (uint32_t k = 0; k < h.z; ++k)
        if (!warmInsert(slots, claim, log2T, gen, warmKey(h.x, h.y, k), k == 0 ? tag : 0u, sv.lam[k][s]))
            atomicOr(&cnt->errorFlags, 2u);
}

// The crowded batch (sorted positions [colourStart[64], colourStart[65]), in descending
// priority): one thread solves (or, kWarm, warm-starts) its manifolds one after another,
// each with freshly loaded bodies, since consecutive ones may share a body.  As the last
// launch of a sweep (closing) it folds its maxima and closes the sweep.
template <bool kWarm>
__global__ void kSolveCrowded(DevCounters* __restrict__ cnt, SolverPtrs sv, SolverBody* sb,
                              const float4* __restrict__ iw0, const float4* __restrict__ iw1, uint32_t tolMode,
                              uint32_t closing, float tol) {
    gridDependencyWait();
    launchDependents();
    if (threadIdx.x != 0) return;
    if (!kWarm && tolMode && cnt->converged) return;
    const uint32_t begin = cnt->colourStart[kMaxColours], end = cnt->colourStart[kMaxColours + 1];
    float gd = 0.0f, gl = 0.0f;
    for (uint32_t s = begin; s < end; ++s) {
        const ManifoldHead hd = loadHeadStreaming(s, sv);
        BodyState A, B;
        loadBodies(hd.h.x, hd.h.y, sb, A, B);
        if (kWarm) warmWithBodies(s, hd, A, B, sv, sb, iw0, iw1);
        else solveWithBodies<true>(s, hd, A, B, sv, sb, iw0, iw1, gd, gl);
    }
    if (kWarm) return;
    if (gd > 0.0f || gl > 0.0f) {
        atomicMax(&cnt->maxDeltaBits, __float_as_uint(gd));
        atomicMax(&cnt->maxLambdaBits, __float_as_uint(gl));
    }
    if (closing) {
        __threadfence();
        closeSweep(cnt, tol, tolMode);
    }
}

// Keys for the crowded batch's priority sort (descending priority = ascending ~prio):
// pass 0 the low 32 bits of ~prio with the manifold as value, pass 1 the high 32 bits of
// the (already low-sorted) values' ~prio.
__global__ void kCrowdKeys(uint32_t K, uint32_t pass, const DevCounters* __restrict__ cnt,
                           const uint32_t* __restrict__ order, const uint4* __restrict__ rec,
                           uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= K) return;
    const uint32_t m = pass == 0u ? order[cnt->colourStart[kMaxColours] + q] : vals[q];
    const uint4 r = rec[m];  // colouring record: priority lo, hi
    const unsigned long long k = ~((unsigned long long)r.y << 32 | r.x);
    keys[q] = pass == 0u ? (uint32_t)k : (uint32_t)(k >> 32);
    if (pass == 0u) vals[q] = m;
}

__global__ void kCrowdScatter(uint32_t K, const DevCounters* __restrict__ cnt, const uint32_t* __restrict__ vals,
                              uint32_t* __restrict__ order, uint32_t* __restrict__ inv) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= K) return;
    const uint32_t pos = cnt->colourStart[kMaxColours] + q, m = vals[q];
    order[pos] = m;
    inv[m] = pos;
}

SolverPtrs solverPtrs(World& w) {
    SolverPtrs p;
    p.hdr = w.shdr.p;
    p.n = w.sn.p;
    for (int k = 0; k < kMaxPoints; ++k) {
        p.ra[k] = w.sra[k].p;
        p.rb[k] = w.srb[k].p;
        p.kt[k] = w.skt[k].p;
        p.lam[k] = w.slam[k].p;
    }
    return p;
}

}  // namespace

void launchPrepare(World& w, const StepParams& sp, uint32_t nM) {
    if (!nM) return;
    const uint32_t prev = w.wsCur ^ 1u;
    const uint32_t lookup = w.wsValid ? 1u : 0u;
    const uint32_t usePrev = !w.wsValid ? 0u
                             : sp.warmStart == AXIOM_WARM_START_PREVIOUS ? 1u
                             : (sp.warmStart == AXIOM_WARM_START_LEARNED && w.mlpLoaded) ? 2u : 0u;
    float* feat = w.needFeatures ? w.feat.p : nullptr;
    ProfRange pr(w, KG_SOLVER_PREPARE);
    w.prof.launches[KG_SOLVER_PREPARE] += 1;
    PrepIn in{};
    in.mhdr = w.mhdr.p;
    in.mn = w.mn.p;
    for (int k = 0; k < kMaxPoints; ++k) in.mp[k] = w.mp[k].p;
    in.info = w.info.p;
    in.pos = w.pos.p;
    in.sb = w.body.p;
    in.iw0 = w.iw0.p;
    in.iw1 = w.iw1.p;
    in.mat = w.mat.p;
    in.wsSlots = w.wsSlots[prev].p;
    in.warm0 = w.warm0Valid ? w.warm0.p : nullptr;
    in.wsGen = w.wsGen[prev];
    in.wsLog2 = w.wsLog2[prev];
    in.lookup = lookup;
    in.usePrev = usePrev;
    in.feat = feat;
    in.hdrDyn = 1u;
    kPrepare<<<gridFor(nM, 256), 256, 0, w.stream>>>(nM, sp, w.orderInv.p, in, solverPtrs(w));
}

// Puts the K crowded manifolds (grouped last, in manifold order) into descending priority:
// two stable 32-bit radix sorts, low then high half of ~priority.
cudaError_t sortCrowded(World& w, uint32_t K) {
    if (K < 2u) return cudaSuccess;
    cudaError_t e;
    for (int k = 0; k < 2; ++k) {
        if ((e = w.crowdKey[k].reserve(K)) != cudaSuccess) return e;
        if ((e = w.crowdVal[k].reserve(K)) != cudaSuccess) return e;
    }
    if ((e = w.crowdHist.reserve(std::max<uint32_t>(radixHistWords(K), 1100u))) != cudaSuccess) return e;
    for (uint32_t pass = 0; pass < 2; ++pass) {
        kCrowdKeys<<<gridFor(K, 256), 256, 0, w.stream>>>(K, pass, w.dcnt, w.order.p, w.manRec.p, w.crowdKey[0].p,
                                                          w.crowdVal[0].p);
        radixSort(w.stream, w.crowdKey[0].p, w.crowdVal[0].p, w.crowdKey[1].p, w.crowdVal[1].p, w.crowdHist.p, K, 4);
    }
    kCrowdScatter<<<gridFor(K, 256), 256, 0, w.stream>>>(K, w.dcnt, w.crowdVal[0].p, w.order.p, w.orderInv.p);
    return cudaGetLastError();
}

void launchLearnRows(World& w, uint32_t nM) {
    if (!nM) return;
    kLearnRows<<<gridFor(4ull * nM, 256), 256, 0, w.stream>>>(nM, w.shdr.p, w.learnRows.p, w.learnRowOf.p,
                                                               &w.dcnt->learnRows);
}

void launchApplyLearned(World& w, const StepParams& sp, uint32_t nM, const float* Y) {
    if (!nM) return;
    kApplyLearned<<<gridFor(4ull * nM, 256), 256, 0, w.stream>>>(nM, Y, w.learnRowOf.p, w.feat.p, sp.warmFactor,
                                                                 solverPtrs(w));
}

// Replays `graph` when `key` matches the launches it holds; otherwise captures what
// `issue` launches on the world's stream into it first.  Returns false (nothing launched)
// when capture or instantiation fails; graphs are then left off for this world.
template <typename F>
static bool replayCached(World& w, CachedGraph& graph, const std::vector<uint64_t>& key, F issue) {
    if (w.graphsOff) return false;
    if (!graph.exec || graph.key != key) {
        if (graph.exec) cudaGraphExecDestroy(graph.exec);
        graph.exec = nullptr;
        cudaGraph_t g = nullptr;
        bool ok = cudaStreamBeginCapture(w.stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            issue();
            ok = cudaStreamEndCapture(w.stream, &g) == cudaSuccess && g;
        }
        if (ok) ok = cudaGraphInstantiate(&graph.exec, g, 0) == cudaSuccess;
        if (g) cudaGraphDestroy(g);
        if (!ok) {
            const cudaError_t e = cudaGetLastError();
            std::fprintf(stderr, "axiom_gb300: solve launches not capturable (%s); launching directly\n",
                         cudaGetErrorString(e));
            graph.exec = nullptr;
            w.graphsOff = true;
            return false;
        }
        graph.key = key;
    }
    return cudaGraphLaunch(graph.exec, w.stream) == cudaSuccess;
}

// What the solve's launches depend on: buffers, grids, colour count and parameters.
static std::vector<uint64_t> solveKey(World& w, uint32_t nColours, uint32_t sweeps, const std::vector<unsigned>& grids,
                                      float tol) {
    const SolverPtrs p = solverPtrs(w);
    std::vector<uint64_t> k = {nColours, sweeps, (uint64_t)(uintptr_t)w.body.p,
                               (uint64_t)(uintptr_t)w.iw0.p, (uint64_t)(uintptr_t)w.iw1.p,
                               (uint64_t)(uintptr_t)w.dcnt};
    uint32_t tb;
    std::memcpy(&tb, &tol, 4);
    k.push_back(tb);
    const uint64_t* words = reinterpret_cast<const uint64_t*>(&p);
    for (size_t i = 0; i < sizeof(p) / 8; ++i) k.push_back(words[i]);
    for (unsigned g : grids) k.push_back(g);
    return k;
}

// A grid for nM manifolds: at most `wave`, and the next power of two above what nM needs,
// so that the captured launches change only when nM crosses a power of two.
static unsigned solveGridFor(unsigned wave, uint32_t nM) {
    unsigned g = 1;
    while (g < wave && g < gridFor(nM, 256)) g <<= 1;
    return std::min(g, wave);
}

// The grid of each colour's launch, from the colour sizes of the last colour-count sync: a
// colour of a few thousand manifolds does not launch (and, closing a sweep, count in) the
// whole wave.  Power-of-two buckets keep the captured graphs stable from step to step.
static std::vector<unsigned> colourGrids(const World& w, uint32_t nColours, unsigned wave) {
    std::vector<unsigned> g(nColours);
    for (uint32_t c = 0; c < nColours; ++c)
        g[c] = solveGridFor(wave, w.hcnt->colourStart[c + 1] - w.hcnt->colourStart[c]);
    return g;
}

static void ensureSolveGrids(World& w) {
    if (w.solveGrid) return;
    int dev = 0, sms = 0, perSm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kSolveColour<false>, 256, 0);
    w.solveGrid = (unsigned)std::max(1, sms * std::max(1, perSm));
    perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kSolveColour<false, true>, 256, 0);
    w.solveGridHoist = (unsigned)std::max(1, sms * std::max(1, perSm));
}

// One launch per colour, chained with programmatic dependent launch (one profiler range
// for all of them: an event between two launches would serialise the chain).  The
// launches depend only on the colour count, so they are captured once per count and
// replayed as one graph.
void launchWarmStartApply(World& w, uint32_t nM, uint32_t nColours) {
    ProfRange pr(w, KG_WARM_START_APPLY);
    ensureSolveGrids(w);
    const std::vector<unsigned> grids = colourGrids(w, nColours, w.solveGrid);
    // the pipelined colour pass in its warm-start form; the first launch follows the
    // kernel that wrote the rows, so only the later ones fetch their first heads early
    const bool crowded = w.lastCrowded > 0;
    auto issue = [&]() {
        for (uint32_t c = 0; c < nColours; ++c)
            launchDependent(kSolveColour<true>, grids[c], 256, w.stream, c, w.dcnt, solverPtrs(w), w.body.p,
                            (const float4*)w.iw0.p, (const float4*)w.iw1.p, 0u, 0u, 0.0f, c > 0 ? 1u : 0u);
        if (crowded)
            launchDependent(kSolveCrowded<true>, 1u, 32, w.stream, w.dcnt, solverPtrs(w), w.body.p,
                            (const float4*)w.iw0.p, (const float4*)w.iw1.p, 0u, 0u, 0.0f);
    };
    w.prof.launches[KG_WARM_START_APPLY] += nColours + (crowded ? 1u : 0u);
    if (!replayCached(w, w.warmGraph, solveKey(w, nColours | (crowded ? 0x100u : 0u), 0, grids, 0.0f), issue))
        issue();
}

// `sweeps` PGS sweeps, one launch per colour (every colour below the colour count has
// manifolds: a first-fit colour c is only taken next to colours 0..c-1).  The last colour
// of a sweep closes it.  Captured once per (colour count, sweeps) and replayed as a graph.
void launchSweeps(World& w, const StepParams& sp, uint32_t nM, uint32_t nColours, uint32_t sweeps, bool tolMode) {
    (void)nM;
    ensureSolveGrids(w);
    const bool hoist = w.hoistRows;
    const std::vector<unsigned> grids = colourGrids(w, nColours, hoist ? w.solveGridHoist : w.solveGrid);
    const bool crowded = w.lastCrowded > 0;
    if (nColours == 0 && !crowded) {  // no manifolds: the sweeps still count
        for (uint32_t it = 0; it < sweeps; ++it)
            kEndSweep<<<1, 1, 0, w.stream>>>(w.dcnt, sp.tolerance, tolMode ? 1u : 0u);
        w.prof.launches[KG_PGS_COLOUR] += sweeps;
        return;
    }
    // a launch may fetch its first manifold heads before its dependency wait when the
    // kernel before it is another colour (which never touches these impulses); the
    // crowded batch, when there is one, is the last launch of each sweep and closes it
    const uint32_t earlyHead = nColours > 1u && !crowded ? 1u : 0u;
    auto issue = [&]() {
        for (uint32_t it = 0; it < sweeps; ++it) {
            for (uint32_t c = 0; c < nColours; ++c)
                launchDependent(hoist ? kSolveColour<false, true> : kSolveColour<false, false>, grids[c], 256,
                                w.stream, c, w.dcnt, solverPtrs(w), w.body.p, (const float4*)w.iw0.p,
                                (const float4*)w.iw1.p, tolMode ? 1u : 0u, c + 1u == nColours && !crowded ? 1u : 0u,
                                sp.tolerance, earlyHead);
            if (crowded)
                launchDependent(kSolveCrowded<false>, 1u, 32, w.stream, w.dcnt, solverPtrs(w), w.body.p,
                                (const float4*)w.iw0.p, (const float4*)w.iw1.p, tolMode ? 1u : 0u, 1u,
                                sp.tolerance);
        }
    };
    w.prof.launches[KG_PGS_COLOUR] += (uint64_t)sweeps * (nColours + (crowded ? 1u : 0u));
    const std::vector<uint64_t> key = solveKey(w, nColours | (crowded ? 0x100u : 0u) | (hoist ? 0x200u : 0u),
                                               sweeps | (tolMode ? 0x80000000u : 0u), grids, sp.tolerance);
    if (!replayCached(w, w.sweepGraph, key, issue)) issue();
}

bool smallSolve(const World& w, uint32_t nM) { return nM > 0u && nM <= kSmallSolve && w.n <= kSmallSolve; }

// The whole solve of a small world in one launch (kSolveSmall): warm start and `sweeps`
// sweeps, or up to `sweeps` sweeps to the tolerance.
cudaError_t launchSolveSmall(World& w, const StepParams& sp, uint32_t sweeps, bool tolMode) {
    if (!w.smallSolveReady) {  // the shared-memory opt-in, on this world's device
        const cudaError_t e = cudaFuncSetAttribute(kSolveSmall, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smallSolveSmem(kSmallSolve));
        if (e != cudaSuccess) return e;
        w.smallSolveReady = true;
    }
    ProfRange pr(w, KG_PGS_COLOUR);
    w.prof.launches[KG_PGS_COLOUR] += 1;
    kSolveSmall<<<1, kSmallSolveThreads, smallSolveSmem(w.n), w.stream>>>(
        w.dcnt, solverPtrs(w), w.body.p, (const float4*)w.iw0.p, (const float4*)w.iw1.p, w.order.p, w.manRec.p, w.n,
        sweeps, tolMode ? 1u : 0u, sp.tolerance);
    return cudaGetLastError();
}

// A world of at most kClusterSolve manifolds (kClusterSolveSingle when every manifold has one
// point: single-point colours take the cluster's rounds faster than four-point ones) on a
// device that can run the cluster: 16 CTAs (a non-portable size) where one such cluster
// fits, else 8, else none.  The step asks for it when a world is above the small-world
// bounds, or within them with more than 1,024 manifolds some of which have several points.
bool clusterSolve(World& w, uint32_t nM, bool multiPoint) {
    if (nM == 0u || nM > (multiPoint ? kClusterSolve : kClusterSolveSingle)) return false;
    if (w.clusterCtas < 0) {
        w.clusterCtas = 0;
        if (cudaFuncSetAttribute(kSolveCluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
            cudaGetLastError();
        for (int ctas : {16, 8}) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(ctas);
            cfg.blockDim = dim3(kClusterThreads);
            cudaLaunchAttribute at;
            at.id = cudaLaunchAttributeClusterDimension;
            at.val.clusterDim.x = ctas;
            at.val.clusterDim.y = 1;
            at.val.clusterDim.z = 1;
            cfg.attrs = &at;
            cfg.numAttrs = 1;
            int clusters = 0;
            if (cudaOccupancyMaxActiveClusters(&clusters, kSolveCluster, &cfg) == cudaSuccess && clusters >= 1) {
                w.clusterCtas = ctas;
                break;
            }
            cudaGetLastError();
        }
    }
    return w.clusterCtas > 0;
}

// The whole solve of a mid-size world in one cluster launch (kSolveCluster): warm start and
// `sweeps` sweeps, or up to `sweeps` sweeps to the tolerance.
cudaError_t launchSolveCluster(World& w, const StepParams& sp, uint32_t nM, uint32_t sweeps, bool tolMode) {
    uint32_t P = 1;
    while (P < nM) P <<= 1;
    cudaError_t e;
    if ((e = w.clusterKey.reserve(P)) != cudaSuccess) return e;
    if ((e = w.clusterPos.reserve(P)) != cudaSuccess) return e;
    ProfRange pr(w, KG_PGS_COLOUR);
    w.prof.launches[KG_PGS_COLOUR] += 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)w.clusterCtas);
    cfg.blockDim = dim3(kClusterThreads);
    cfg.stream = w.stream;
    cudaLaunchAttribute at;
    at.id = cudaLaunchAttributeClusterDimension;
    at.val.clusterDim.x = (unsigned)w.clusterCtas;
    at.val.clusterDim.y = 1;
    at.val.clusterDim.z = 1;
    cfg.attrs = &at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kSolveCluster, w.dcnt, solverPtrs(w), w.body.p, (const float4*)w.iw0.p,
                              (const float4*)w.iw1.p, (const uint32_t*)w.order.p, (const uint4*)w.manRec.p,
                              w.clusterKey.p, w.clusterPos.p, sweeps, tolMode ? 1u : 0u, sp.tolerance);
}

void launchStoreImpulses(World& w, uint32_t nM) {
    const uint32_t cur = w.wsCur;
    ProfRange pr(w, KG_STORE_IMPULSES);
    w.prof.launches[KG_STORE_IMPULSES] += nM ? 1 : 0;
    const uint32_t gen = nextWarmGen(w, cur);  // the table's older entries turn empty
    if (nM)
        kStoreImpulses<<<gridFor(nM, 256), 256, 0, w.stream>>>(nM, solverPtrs(w), w.wsSlots[cur].p,
                                                              w.wsClaim[cur].p, gen, w.wsLog2[cur], w.dcnt);
}

}  // namespace axiom_gb300
