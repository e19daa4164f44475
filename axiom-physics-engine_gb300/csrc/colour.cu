// colour.cu — deterministic colouring of the contact graph.
//
// Vertices are manifolds; two conflict when they share a dynamic body (static and
// kinematic bodies are never written by the solver, so they do not constrain colours).
// Priority of a manifold = SplitMix64(pairKey(a, b)), a bijection, so priorities are
// distinct.  The colouring is greedy first-fit in descending priority — what the CPU
// oracle computes sequentially: each manifold takes the lowest colour not used by a
// higher-priority manifold at either of its dynamic bodies.
//
// The manifolds at one body all conflict with each other, so at each dynamic body they
// form a chain in priority order, and a manifold only has to wait for its predecessor in
// the chain of each of its (at most two) dynamic bodies: once those are coloured, so is
// every higher-priority neighbour, and the body's colour mask holds exactly their
// colours.  The step (1) records every manifold in a fixed 64-slot list at each of its
// dynamic bodies (a body with more than 64 manifolds needs more than the 64 colours
// there are anyway), (2) links each manifold to its successor in each body's chain and
// counts its predecessors, (3) lists the seeds, the manifolds that have none, and
// (4) colours the chains as a dataflow: a coloured manifold releases its successors, and
// the thread that releases a successor's last predecessor queues it in its own CTA, which
// colours it in a later batch.  No CTA waits for another: each starts from its share of
// the seeds and stops when its own queue is empty.  A manifold is only ever queued after
// every higher-priority manifold at its bodies is coloured, and at most one manifold of a
// body's chain is in flight, so the mask updates are race-free and the colours do not
// depend on the order in which CTAs run.  Then a stable one-digit radix pass groups the
// manifolds by colour.
//
// The dependency depth (the number of Jones-Plassmann rounds the same colouring takes, as
// the oracle reports it) rides along in the predecessor counters: the low two bits count
// the predecessors left, and each predecessor adds its own level + 1 into the field of
// the body it shares, so the last one to finish reads both fields and knows the level.
//
// Temporally coherent mode (axiom_world_config.temporal_colouring): each manifold first
// looks up its previous-step colour (the tag of its point-0 slot in the previous warm-start
// table).  A manifold that has one keeps it unless a higher-priority manifold at a shared
// dynamic body has the same previous colour; the kept colours seed the body masks, and only
// the other manifolds (new or conflicting) go through the chains and the dataflow above,
// which then links and counts only them.  Kept manifolds share no colour at a dynamic body,
// and every recoloured one avoids the kept colours at its bodies, so the colouring stays
// proper; it depends only on the manifold set, the priorities and the previous colours.
//
// Crowded manifolds: a manifold with a dynamic body of more than kCrowdDegree manifolds
// (a box resting on dozens of spheres) takes no colour.  It stays out of the chains and
// the kept colours, and the solver runs all of them in one serial batch after the colours,
// in descending priority.  Every other manifold sees at most 2 x (kCrowdDegree - 1) other
// manifolds at its two bodies, so it always finds one of the 64 colours.
#include <algorithm>

#include "dmath.cuh"
#include "world.h"

namespace axiom_gb300 {
namespace {

using namespace axd;

constexpr uint32_t kSlots = kMaxColours;  // chain slots per dynamic body
constexpr uint32_t kSideB = 0x80000000u;    // slot / successor entry: manifold id | side bit
constexpr uint32_t kNone = 0xFFFFFFFFu;
// Chain record of a manifold (16 bytes, written once per colouring, read with one access
// wherever a body's list is scanned): priority (lo, hi), previous colour (kNone: none),
// flags.
constexpr uint32_t kFlagDropped = 1u;  // temporal mode: previous colour taken by a higher priority
constexpr uint32_t kFlagCrowded = 2u;  // a dynamic body with more than kCrowdDegree manifolds

__device__ __forceinline__ unsigned long long recPrio(uint4 r) { return (unsigned long long)r.y << 32 | r.x; }

// Predecessor counter of a manifold: bits 0-1 count the chain predecessors not yet
// coloured; bits 2-16 and 17-31 receive level + 1 of the predecessor through the
// manifold's body a and body b.
constexpr uint32_t kLevelShiftA = 2, kLevelShiftB = 17, kLevelMax = 0x7FFFu;

__device__ __forceinline__ uint32_t levelOf(uint32_t counter) {
    return max((counter >> kLevelShiftA) & kLevelMax, counter >> kLevelShiftB);
}

// Previous-step colours for the temporal mode: the previous warm-start table (slot tag =
// 1 + colour on point 0 of each manifold).  table == nullptr: none.
struct PrevColours {
    const WarmSlot* table;
    uint32_t log2T, gen;
};

// The previous-step slot of point 0 of manifold (a, b) (kNone: none), and its colour
// (kNone: none).
__device__ __forceinline__ uint32_t previousSlot(const PrevColours& pc, uint32_t a, uint32_t b, uint32_t& prevColour) {
    prevColour = kNone;
    if (!pc.table) return kNone;
    const uint32_t mask = (1u << pc.log2T) - 1u;
    const unsigned long long key = pairKey(a, b) * 4ull;
    uint32_t at = (uint32_t)((mix64(key) * 0x9E3779B97F4A7C15ull) >> (64u - pc.log2T));
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const uint4 hd = __ldcg(reinterpret_cast<const uint4*>(pc.table + at));  // key, gen, tag
        if (hd.z != pc.gen) return kNone;  // an empty slot: the key is absent
        if (((unsigned long long)hd.y << 32 | hd.x) == key) {
            prevColour = hd.w ? hd.w - 1u : kNone;
            return at;
        }
        at = (at + 1u) & mask;
    }
    return kNone;
}

// Kernels whose work is only needed when a flag set earlier in the step is up read it
// first (`gate`) and return at once otherwise; they stride over their range, so the idle
// launch is a few CTAs wide.
__device__ __forceinline__ bool gateClosed(const uint32_t* gate) { return gate && *((volatile const uint32_t*)gate) == 0u; }

// (1) priorities and previous colours (the chain records), and each manifold in the slot
// list of each of its dynamic bodies.  The lists are slot-major (slot k of body x at
// k * n + x), so that (2) reads them coalesced.  Also zeroes the predecessor counters, and
// raises `crowdSeen` when some body gets more than kCrowdDegree manifolds.  Successor
// links need no start value: (2) writes the one at every dynamic body of every manifold
// that enters a chain, and only those are read.
__device__ __forceinline__ void chainInit(uint32_t m, uint32_t nM, uint32_t n, const uint4* __restrict__ hdr,
                                          uint4* __restrict__ rec, uint32_t* __restrict__ deg,
                                          uint32_t* __restrict__ slots, uint32_t* __restrict__ colour,
                                          uint32_t* __restrict__ pending, const PrevColours& pc,
                                          float4* __restrict__ warm0, uint32_t* __restrict__ crowdSeen) {
    // the degree atomics are issued before the table probe, so that their round trips
    // overlap (more manifolds per thread measured slower: their registers halve the
    // resident threads, and this pass lives on memory latency)
    if (m >= nM) return;
    const uint4 h = hdr[m];
    const uint32_t ka = (h.w & kHdrDynA) ? atomicAdd(&deg[h.x], 1u) : kNone;
    const uint32_t kb = (h.w & kHdrDynB) ? atomicAdd(&deg[h.y], 1u) : kNone;
    uint32_t prev;
    const uint32_t slot = previousSlot(pc, h.x, h.y, prev);
    // point 0's previous impulses (same sector as the tag) for the solver preparation, which
    // then reads them in manifold order instead of probing the table again
    if (warm0) warm0[m] = slot != kNone ? __ldcg(&pc.table[slot].val) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const unsigned long long pr = mix64(pairKey(h.x, h.y));
    rec[m] = make_uint4((uint32_t)pr, (uint32_t)(pr >> 32), prev, 0u);
    colour[m] = prev;
    pending[m] = 0u;
    // a body beyond kSlots manifolds is crowded (kSlots > kCrowdDegree): its manifolds take
    // no chain, so the slots it cannot list are not needed
    if (ka < kSlots) slots[(size_t)ka * n + h.x] = m;
    if (kb < kSlots) slots[(size_t)kb * n + h.y] = m | kSideB;
    if (ka == kCrowdDegree || kb == kCrowdDegree) *crowdSeen = 1u;
}

__global__ void __launch_bounds__(256) kChainInit(uint32_t nM, uint32_t n, const uint4* __restrict__ hdr,
                                                  uint4* __restrict__ rec, uint32_t* __restrict__ deg,
                                                  uint32_t* __restrict__ slots, uint32_t* __restrict__ colour,
                                                  uint32_t* __restrict__ pending, PrevColours pc,
                                                  float4* __restrict__ warm0, uint32_t* __restrict__ crowdSeen) {
    chainInit(blockIdx.x * blockDim.x + threadIdx.x, nM, n, hdr, rec, deg, slots, colour, pending, pc, warm0,
              crowdSeen);
}

// (1a, gated by crowdSeen) per manifold, once the degrees are complete: flags it crowded
// when a dynamic body of it has more than kCrowdDegree manifolds.
__device__ __forceinline__ void chainFlags(uint32_t first, uint32_t step, uint32_t nM, const uint4* __restrict__ hdr,
                                           const uint32_t* __restrict__ deg, uint4* __restrict__ rec) {
    for (uint32_t m = first; m < nM; m += step) {
        const uint4 h = hdr[m];
        if (((h.w & kHdrDynA) && __ldcg(&deg[h.x]) > kCrowdDegree) ||
            ((h.w & kHdrDynB) && __ldcg(&deg[h.y]) > kCrowdDegree))
            rec[m].w = kFlagCrowded;
    }
}

__global__ void __launch_bounds__(256) kChainFlags(uint32_t nM, const uint4* __restrict__ hdr,
                                                   const uint32_t* __restrict__ deg, uint4* __restrict__ rec,
                                                   const uint32_t* __restrict__ gate) {
    if (gateClosed(gate)) return;
    chainFlags(blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, nM, hdr, deg, rec);
}

// (1b, temporal mode, gated by a conflict that (2) found) per dynamic body of at most
// kCrowdDegree manifolds (the others' are crowded): a manifold with a previous colour is
// dropped (to be recoloured) when a higher-priority manifold at this body has the same
// previous colour.  Crowded manifolds take no part.  Reads only the previous colours,
// priorities and crowded flags, so the result does not depend on order.
__device__ __forceinline__ void chainConflicts(uint32_t first, uint32_t step, uint32_t n,
                                               const uint32_t* __restrict__ deg, const uint32_t* __restrict__ slots,
                                               uint4* __restrict__ rec) {
    for (uint32_t x = first; x < n; x += step) {
        const uint32_t d = __ldcg(&deg[x]);
        if (d < 2u || d > kCrowdDegree) continue;
        const uint32_t* list = slots + x;
        for (uint32_t i = 0; i < d; ++i) {
            const uint32_t mi = list[(size_t)i * n] & ~kSideB;
            const uint4 ri = __ldcg(&rec[mi]);
            if (ri.z == kNone || (ri.w & kFlagCrowded)) continue;
            for (uint32_t j = 0; j < d; ++j) {
                const uint32_t mj = list[(size_t)j * n] & ~kSideB;
                const uint4 rj = __ldcg(&rec[mj]);
                if (mj != mi && rj.z == ri.z && recPrio(rj) > recPrio(ri) && !(rj.w & kFlagCrowded)) {
                    atomicOr(&rec[mi].w, kFlagDropped);
                    break;
                }
            }
        }
    }
}

__global__ void __launch_bounds__(256) kChainConflicts(uint32_t n, const uint32_t* __restrict__ deg,
                                                       const uint32_t* __restrict__ slots, uint4* __restrict__ rec,
                                                       const uint32_t* __restrict__ gate) {
    if (gateClosed(gate)) return;
    chainConflicts(blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, n, deg, slots, rec);
}

// (1c, gated like (1b)) the predecessor counters start again for the second linking pass.
__global__ void __launch_bounds__(256) kChainReset(uint32_t nM, uint32_t* __restrict__ pending,
                                                   const uint32_t* __restrict__ gate) {
    if (gateClosed(gate)) return;
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < nM; m += gridDim.x * blockDim.x) pending[m] = 0u;
}

// Kept in the temporal mode: a previous colour, not dropped, not crowded.
__device__ __forceinline__ bool keptColour(uint4 r, bool temporal) { return temporal && r.z != kNone && r.w == 0u; }
__device__ __forceinline__ bool crowdedRec(uint4 r) { return (r.w & kFlagCrowded) != 0u; }

constexpr uint32_t kLinkRegs = 16;  // bodies with at most this many manifolds link in registers

// best: the successor's slot entry (id | its side bit at this body), or kNone
__device__ __forceinline__ void linkOne(uint32_t e, uint32_t best, bool pred, uint2* __restrict__ succ,
                                        uint32_t* __restrict__ pending) {
    const uint32_t m = e & ~kSideB;
    if (e & kSideB) succ[m].y = best;
    else succ[m].x = best;
    if (pred) atomicAdd(&pending[m], 1u);
}

// (2) per dynamic body: each listed manifold's successor (the next lower priority) and
// whether it has a predecessor (some higher priority) in this body's chain.  Up to
// kLinkRegs entries are compared in registers (unrolled, so the arrays stay in registers);
// longer lists re-read their entries.  In the temporal mode the kept manifolds stay out of
// the chain and their colours start the body's mask.
//
// The temporal mode runs this pass before any manifold is dropped, with `conflict` set:
// two manifolds at one body with the same previous colour (neither crowded) raise it.
// Without such a pair nothing would be dropped, so the links are final.  Otherwise (1b)
// drops, (1c) resets the counters, and this pass runs again (gated by `conflict`), which
// rewrites every mask and every link it reads later.  A proper colouring last step leaves
// no such pair among manifolds that persist at a body whose dynamic state is unchanged, so
// the second pass is rare (bodies that woke or changed type).
__device__ __forceinline__ void chainLink(uint32_t first, uint32_t step, uint32_t n, const uint32_t* __restrict__ deg,
                                          const uint32_t* __restrict__ slots, const uint4* __restrict__ rec,
                                          uint32_t temporal, uint2* __restrict__ succ,
                                          uint32_t* __restrict__ pending, unsigned long long* __restrict__ mask,
                                          uint32_t* __restrict__ conflict) {
    for (uint32_t x = first; x < n; x += step) {
        // a body of more than kCrowdDegree manifolds has only crowded ones: no chain, no mask
        const uint32_t dx = __ldcg(&deg[x]), d = dx > kCrowdDegree ? 0u : dx;
        const uint32_t* list = slots + x;  // entry i at list[i * n]
        unsigned long long kept = 0ull;    // the body's colours before (4): the kept ones
        unsigned long long seen = 0ull;    // previous colours of the non-crowded manifolds
        bool clash = false;
        if (d <= kLinkRegs) {
            uint32_t e[kLinkRegs];
            unsigned long long p[kLinkRegs];
            bool live[kLinkRegs];  // in the chain (not kept)
#pragma unroll
            for (uint32_t i = 0; i < kLinkRegs; ++i) {
                e[i] = i < d ? list[(size_t)i * n] : kNone;
                const uint4 r = i < d ? __ldcg(&rec[e[i] & ~kSideB]) : make_uint4(0u, 0u, kNone, kFlagCrowded);
                p[i] = recPrio(r);
                const bool k = keptColour(r, temporal != 0u);
                if (k) kept |= 1ull << r.z;
                if (r.z != kNone && !crowdedRec(r)) {
                    clash = clash || ((seen >> r.z) & 1ull);
                    seen |= 1ull << r.z;
                }
                live[i] = i < d && !k && !crowdedRec(r);
            }
#pragma unroll
            for (uint32_t i = 0; i < kLinkRegs; ++i) {
                if (i >= d) break;
                if (!live[i]) continue;
                bool pred = false;
                unsigned long long bestP = 0ull;
                uint32_t best = kNone;
#pragma unroll
                for (uint32_t j = 0; j < kLinkRegs; ++j) {
                    if (live[j]) {
                        if (p[j] > p[i]) pred = true;
                        else if (p[j] < p[i] && (best == kNone || p[j] > bestP)) {
                            bestP = p[j];
                            best = e[j];
                        }
                    }
                }
                linkOne(e[i], best, pred, succ, pending);
            }
        } else {
            for (uint32_t i = 0; i < d; ++i) {
                const uint32_t ei = list[(size_t)i * n], mi = ei & ~kSideB;
                const uint4 ri = __ldcg(&rec[mi]);
                if (ri.z != kNone && !crowdedRec(ri)) {
                    clash = clash || ((seen >> ri.z) & 1ull);
                    seen |= 1ull << ri.z;
                }
                if (keptColour(ri, temporal != 0u)) {
                    kept |= 1ull << ri.z;
                    continue;
                }
                if (crowdedRec(ri)) continue;
                const unsigned long long pi = recPrio(ri);
                bool pred = false;
                unsigned long long bestP = 0ull;
                uint32_t best = kNone;
                for (uint32_t j = 0; j < d; ++j) {
                    const uint32_t ej = list[(size_t)j * n];
                    const uint4 rj = __ldcg(&rec[ej & ~kSideB]);
                    if (keptColour(rj, temporal != 0u) || crowdedRec(rj)) continue;
                    const unsigned long long pj = recPrio(rj);
                    if (pj > pi) pred = true;
                    else if (pj < pi && (best == kNone || pj > bestP)) {
                        bestP = pj;
                        best = ej;
                    }
                }
                linkOne(ei, best, pred, succ, pending);
            }
        }
        mask[x] = kept;
        if (conflict && temporal && clash) *conflict = 1u;
    }
}

// Three CTAs per SM (80 registers, a few bytes spilled): the pass waits on its record
// gathers, and the third CTA hides more of them than the spill costs.
__global__ void __launch_bounds__(256, 3) kChainLink(uint32_t n, const uint32_t* __restrict__ deg,
                                                  const uint32_t* __restrict__ slots, const uint4* __restrict__ rec,
                                                  uint32_t temporal, uint2* __restrict__ succ,
                                                  uint32_t* __restrict__ pending, unsigned long long* __restrict__ mask,
                                                  uint32_t* __restrict__ conflict, const uint32_t* __restrict__ gate) {
    if (gateClosed(gate)) return;
    chainLink(blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, n, deg, slots, rec, temporal, succ,
              pending, mask, conflict);
}

// (3) the seeds: manifolds without a predecessor at either body (and, in the temporal
// mode, not kept), listed with one reservation per block (a counter hit by every warp of
// the grid serialises in L2).
// Every thread of the block calls it (one block-wide reservation).
__device__ __forceinline__ void chainSeed(uint32_t m, uint32_t nM, const uint32_t* __restrict__ pending,
                                          uint32_t* __restrict__ colour, const uint4* __restrict__ rec,
                                          uint32_t temporal, uint32_t* __restrict__ seeds,
                                          uint32_t* __restrict__ count) {
    const uint4 r = m < nM ? __ldcg(&rec[m]) : make_uint4(0u, 0u, kNone, 0u);
    const bool crowded = m < nM && crowdedRec(r);
    if (crowded) colour[m] = kCrowdColour;
    const bool ready = m < nM && !crowded && __ldcg(&pending[m]) == 0u && !keptColour(r, temporal != 0u);
    const uint32_t at = blockReserve(ready ? 1u : 0u, count);
    if (ready) seeds[at] = m;
}

__global__ void __launch_bounds__(256) kChainSeed(uint32_t nM, const uint32_t* __restrict__ pending,
                                                  uint32_t* __restrict__ colour, const uint4* __restrict__ rec,
                                                  uint32_t temporal, uint32_t* __restrict__ seeds,
                                                  uint32_t* __restrict__ count) {
    chainSeed(blockIdx.x * blockDim.x + threadIdx.x, nM, pending, colour, rec, temporal, seeds, count);
}

// (4) the dataflow.  A CTA colours batches of up to kLocalThreads manifolds: first the
// queued successors it released, then more of its share of the seeds; it stops when both
// run out, and never waits for another CTA.  (Following a released successor at once in
// the releasing thread, or a queue per warp instead of per CTA, measured slower: the
// successors stay with the CTA that released them, and the smaller the agent the more the
// work drifts between agents.)  The queue is a FIFO of (manifold, level) entries in
// chunks taken from a pool; a batch consumes at most kLocalThreads entries and adds at
// most two per manifold, so it crosses at most one chunk boundary on either side, and the
// chunk after the write chunk is taken whenever the next batch could reach it.
constexpr uint32_t kLocalThreads = 512;
constexpr uint32_t kChunk = 2048;
static_assert(kChunk >= 2u * kLocalThreads && (kChunk & (kChunk - 1u)) == 0u, "chunk size");
constexpr uint32_t kErrColourPool = 4u;  // DevCounters::errorFlags: the queue chunk pool ran out

struct ChunkPool {
    uint2* entries;   // chunks of kChunk queue entries (manifold, level)
    uint32_t* next;   // next[c]: the chunk after chunk c in its CTA's queue
    uint32_t chunks;  // capacity in chunks; chunk b is CTA b's first
};

__device__ __forceinline__ void fenceAcqRel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

__device__ __forceinline__ uint32_t atomAddRelaxed(uint32_t* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.relaxed.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// What successor entry e (id | side bit) of a manifold at `level` adds to its counter.
__device__ __forceinline__ uint32_t releaseAdd(uint32_t e, uint32_t level) {
    return (min(level + 1u, kLevelMax) << ((e & kSideB) ? kLevelShiftB : kLevelShiftA)) - 1u;
}

// Colours manifold q.x (level q.y) and counts down its successors; r0 / r1 get the
// successors whose last predecessor it was.  The fence before the counts publishes this
// thread's mask stores to whoever colours a successor; the fence after them orders the
// other predecessors' mask stores before what this CTA reads after its next barrier.
__device__ __forceinline__ void colourOne(uint2 q, const uint4* __restrict__ hdr, const uint2* __restrict__ succ,
                                          uint32_t* __restrict__ pending, unsigned long long* __restrict__ mask,
                                          uint32_t* __restrict__ colour, DevCounters* cnt, bool& v0, uint2& r0,
                                          bool& v1, uint2& r1) {
    const uint32_t m = q.x;
    const uint4 h = hdr[m];
    const uint2 sc = succ[m];
    const bool da = (h.w & kHdrDynA) != 0u, db = (h.w & kHdrDynB) != 0u;
    const unsigned long long ma = da ? __ldcg(&mask[h.x]) : 0ull;
    const unsigned long long mb = db ? __ldcg(&mask[h.y]) : 0ull;
    const unsigned long long used = ma | mb;
    uint32_t c;
    if (used == ~0ull) {
        atomicOr(&cnt->colourOverflow, 1u);
        c = kMaxColours - 1;
    } else {
        c = (uint32_t)(__ffsll((long long)~used) - 1);
    }
    const unsigned long long bit = 1ull << c;
    if (da) mask[h.x] = ma | bit;
    if (db) mask[h.y] = mb | bit;
    colour[m] = c;  // the colour count comes from the grouping pass (groupByColour)
    const bool sa = da && sc.x != kNone, sb = db && sc.y != kNone;
    v0 = v1 = false;
    if (!sa && !sb) return;
    fenceAcqRel();
    const uint32_t addA = sa ? releaseAdd(sc.x, q.y) : 0u, addB = sb ? releaseAdd(sc.y, q.y) : 0u;
    const uint32_t oldA = sa ? atomAddRelaxed(&pending[sc.x & ~kSideB], addA) : 0u;
    const uint32_t oldB = sb ? atomAddRelaxed(&pending[sc.y & ~kSideB], addB) : 0u;
    v0 = sa && (oldA & 3u) == 1u;
    v1 = sb && (oldB & 3u) == 1u;
    if (v0) r0 = make_uint2(sc.x & ~kSideB, levelOf(oldA + addA));
    if (v1) r1 = make_uint2(sc.y & ~kSideB, levelOf(oldB + addB));
    if (v0 || v1) fenceAcqRel();
}

// One CTA (number `block` of `grid`, kLocalThreads threads) of the dataflow.
__device__ __forceinline__ void colourDataflow(uint32_t block, uint32_t grid, const uint32_t* __restrict__ seeds,
                                               const uint32_t* __restrict__ seedCount, const ChunkPool& pool,
                                               const uint4* __restrict__ hdr, const uint2* __restrict__ succ,
                                               uint32_t* __restrict__ pending, unsigned long long* __restrict__ mask,
                                               uint32_t* __restrict__ colour, DevCounters* cnt) {
    constexpr uint32_t kWarps = kLocalThreads / 32u;
    __shared__ uint32_t sHead, sTail, sSeedPos, sSeedEnd, sStop;
    __shared__ uint32_t sReadChunk, sReadBase, sReadNext, sWriteChunk, sWriteBase, sWriteNext;
    __shared__ uint32_t warpSum[kWarps];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        const uint32_t nSeeds = __ldcg(seedCount);  // counted by atomics, in L2
        sHead = sTail = 0u;
        sSeedPos = (uint32_t)((uint64_t)nSeeds * block / grid);
        sSeedEnd = (uint32_t)((uint64_t)nSeeds * (block + 1u) / grid);
        sReadChunk = sWriteChunk = block;
        sReadBase = sWriteBase = 0u;
        sReadNext = sWriteNext = kNone;
        sStop = 0u;
    }
    uint32_t levels = 0u;  // 1 + the highest level this thread coloured (0: none)
    for (;;) {
        __syncthreads();  // the previous batch's queue state and entries are final
        const uint32_t head = sHead, tail = sTail, seedPos = sSeedPos;
        const uint32_t r = min(tail - head, kLocalThreads);
        const uint32_t ns = min(kLocalThreads - r, sSeedEnd - seedPos);
        if (r + ns == 0u || sStop) break;
        const uint32_t writeChunk = sWriteChunk, writeBase = sWriteBase, writeNext = sWriteNext;
        const uint32_t t = threadIdx.x;
        uint2 cur = make_uint2(kNone, 0u);
        if (t < r) {
            const uint32_t off = head + t - sReadBase;
            const uint32_t ch = off < kChunk ? sReadChunk : sReadNext;
            cur = __ldcg(&pool.entries[(size_t)ch * kChunk + (off & (kChunk - 1u))]);
        } else if (t < r + ns) {
            cur = make_uint2(seeds[seedPos + (t - r)], 0u);
        }
        bool v0 = false, v1 = false;
        uint2 r0 = make_uint2(0u, 0u), r1 = r0;
        if (cur.x != kNone) {
            colourOne(cur, hdr, succ, pending, mask, colour, cnt, v0, r0, v1, r1);
            levels = max(levels, cur.y + 1u);
        }
        // queue positions of the released successors: block-wide exclusive scan
        const uint32_t k = (v0 ? 1u : 0u) + (v1 ? 1u : 0u);
        uint32_t x = k;
#pragma unroll
        for (uint32_t off = 1; off < 32u; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
            if (lane >= off) x += y;
        }
        if (lane == 31u) warpSum[warp] = x;
        __syncthreads();
        uint32_t before = 0u, total = 0u;
#pragma unroll
        for (uint32_t w = 0; w < kWarps; ++w) {
            const uint32_t cw = warpSum[w];
            if (w < warp) before += cw;
            total += cw;
        }
        uint32_t pos = tail + before + x - k;
        if (v0) {
            const uint32_t off = pos - writeBase;
            pool.entries[(size_t)(off < kChunk ? writeChunk : writeNext) * kChunk + (off & (kChunk - 1u))] = r0;
            ++pos;
        }
        if (v1) {
            const uint32_t off = pos - writeBase;
            pool.entries[(size_t)(off < kChunk ? writeChunk : writeNext) * kChunk + (off & (kChunk - 1u))] = r1;
        }
        if (threadIdx.x == 0) {
            // every thread read the queue state before the barrier above; it changes here
            const uint32_t newHead = head + r, newTail = tail + total;
            uint32_t wc = writeChunk, wb = writeBase, wn = writeNext;
            if (newTail - wb >= kChunk) {  // the write position moved into the chunk taken ahead
                wc = wn;
                wb += kChunk;
                wn = kNone;
            }
            if (wn == kNone && newTail + 2u * kLocalThreads - wb >= kChunk) {
                const uint32_t nc = grid + atomicAdd(&cnt->colourChunks, 1u);
                if (nc < pool.chunks) {
                    pool.next[wc] = nc;
                    wn = nc;
                } else {
                    atomicOr(&cnt->errorFlags, kErrColourPool);
                    sStop = 1u;
                }
            }
            uint32_t rc = sReadChunk, rb = sReadBase;
            if (newHead - rb >= kChunk) {  // the reader left its chunk: the writer linked the next one
                rc = pool.next[rc];
                rb += kChunk;
            }
            const uint32_t nextRead = min(newTail - newHead, kLocalThreads);
            sReadNext = newHead + nextRead - rb > kChunk ? pool.next[rc] : kNone;
            sReadChunk = rc;
            sReadBase = rb;
            sWriteChunk = wc;
            sWriteBase = wb;
            sWriteNext = wn;
            sHead = newHead;
            sTail = newTail;
            sSeedPos = seedPos + ns;
        }
    }
    // dependency depth: 1 + the highest level coloured
    const uint32_t wl = __reduce_max_sync(0xFFFFFFFFu, levels);
    if (lane == 0u) warpSum[warp] = wl;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t bl = 0u;
        for (uint32_t w = 0; w < kWarps; ++w) bl = max(bl, warpSum[w]);
        if (bl) atomicMax(&cnt->colourRounds, bl);
    }
}

__global__ void __launch_bounds__(kLocalThreads, 4) kChainLocal(const uint32_t* __restrict__ seeds,
                                                                const uint32_t* __restrict__ seedCount,
                                                                ChunkPool pool, const uint4* __restrict__ hdr,
                                                                const uint2* __restrict__ succ,
                                                                uint32_t* __restrict__ pending,
                                                                unsigned long long* __restrict__ mask,
                                                                uint32_t* __restrict__ colour, DevCounters* cnt) {
    colourDataflow(blockIdx.x, gridDim.x, seeds, seedCount, pool, hdr, succ, pending, mask, colour, cnt);
}

// ---- small worlds: the whole colouring in one CTA ----
//
// A world of at most kSmallColour manifolds and bodies runs every pass above in one launch
// of one kLocalThreads CTA, with CTA barriers between the passes instead of kernel
// boundaries (the gated passes are plain branches on the flags), and groups by colour with
// the stable counting sort below.  Same passes, same results.
constexpr uint32_t kSmallColour = 4096;

// Stable grouping by the low 8 bits of the colour (what the radix pass does: colours below
// 64, then the crowded batch (64), an uncoloured manifold of a failed colouring last),
// chunk by chunk in manifold order, ranks within a chunk from warp matches.  Writes the
// order, its inverse and the colour bounds and count.
__device__ __forceinline__ void groupSmall(const uint32_t* __restrict__ colour, uint32_t* __restrict__ order,
                                           uint32_t* __restrict__ inv, uint32_t nM, DevCounters* cnt) {
    constexpr uint32_t kWarps = kLocalThreads / 32u;
    __shared__ uint32_t total[256], run[256];
    __shared__ uint32_t wc[kWarps][256];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    for (uint32_t d = tid; d < 256u; d += kLocalThreads) total[d] = 0u;
    __syncthreads();
    for (uint32_t m = tid; m < nM; m += kLocalThreads) atomicAdd(&total[__ldcg(&colour[m]) & 0xFFu], 1u);
    __syncthreads();
    if (tid == 0) {
        uint32_t acc = 0u, maxC = 0u;
        for (uint32_t d = 0; d < 256u; ++d) {
            run[d] = acc;
            if (d <= (uint32_t)kMaxColours + 1u) cnt->colourStart[d] = acc;
            if (d < (uint32_t)kMaxColours && total[d] > 0u) maxC = d + 1u;
            acc += total[d];
        }
        cnt->maxColour = maxC;
    }
    for (uint32_t c0 = 0; c0 < nM; c0 += kLocalThreads) {
        for (uint32_t i = tid; i < kWarps * 256u; i += kLocalThreads) (&wc[0][0])[i] = 0u;
        __syncthreads();
        const uint32_t m = c0 + tid;
        const bool valid = m < nM;
        const uint32_t d = valid ? (__ldcg(&colour[m]) & 0xFFu) : 0x100u;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0u) wc[warp][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t pos = run[d] + rank;
            for (uint32_t w = 0; w < warp; ++w) pos += wc[w][d];
            order[pos] = m;
            inv[m] = pos;
        }
        __syncthreads();
        for (uint32_t dd = tid; dd < 256u; dd += kLocalThreads) {
            uint32_t add = 0u;
            for (uint32_t w = 0; w < kWarps; ++w) add += wc[w][dd];
            run[dd] += add;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kLocalThreads) kColourSmall(uint32_t nM, uint32_t n, const uint4* __restrict__ hdr,
                                                              uint4* __restrict__ rec, uint32_t* __restrict__ deg,
                                                              uint32_t* __restrict__ slots,
                                                              uint32_t* __restrict__ colour, uint2* __restrict__ succ,
                                                              uint32_t* __restrict__ pending,
                                                              unsigned long long* __restrict__ mask,
                                                              uint32_t* __restrict__ seeds,
                                                              uint32_t* __restrict__ seedCount, ChunkPool pool,
                                                              uint32_t* __restrict__ order,
                                                              uint32_t* __restrict__ inv, PrevColours pc,
                                                              float4* __restrict__ warm0, uint32_t temporal,
                                                              DevCounters* cnt) {
    const uint32_t tid = threadIdx.x, B = kLocalThreads;
    for (uint32_t x = tid; x < n; x += B) deg[x] = 0u;
    if (tid == 0) *seedCount = 0u;
    __syncthreads();
    for (uint32_t m0 = 0; m0 < nM; m0 += B)
        chainInit(m0 + tid, nM, n, hdr, rec, deg, slots, colour, pending, pc, warm0, &cnt->crowdSeen);
    __syncthreads();
    if (*((volatile const uint32_t*)&cnt->crowdSeen)) {
        chainFlags(tid, B, nM, hdr, deg, rec);
        __syncthreads();
    }
    chainLink(tid, B, n, deg, slots, rec, temporal, succ, pending, mask, temporal ? &cnt->colourConflict : nullptr);
    __syncthreads();
    if (temporal && *((volatile const uint32_t*)&cnt->colourConflict)) {
        chainConflicts(tid, B, n, deg, slots, rec);
        __syncthreads();
        for (uint32_t m = tid; m < nM; m += B) pending[m] = 0u;
        __syncthreads();
        chainLink(tid, B, n, deg, slots, rec, temporal, succ, pending, mask, nullptr);
        __syncthreads();
    }
    for (uint32_t m0 = 0; m0 < nM; m0 += B) chainSeed(m0 + tid, nM, pending, colour, rec, temporal, seeds, seedCount);
    __syncthreads();
    colourDataflow(0u, 1u, seeds, seedCount, pool, hdr, succ, pending, mask, colour, cnt);
    __syncthreads();
    groupSmall(colour, order, inv, nM, cnt);
}

}  // namespace

// Colours w.mhdr[0..nM) into w.mcolour, and leaves the colour-sorted manifold order in
// w.order with bounds in dcnt->colourStart.  Everything stays on the device; the
// dependency depth arrives with the counters (colourRounds).
cudaError_t colourManifolds(World& w, uint32_t nM) {
    ProfRange pr(w, KG_COLOURING);
    uint64_t& launches = w.prof.launches[KG_COLOURING];
    cudaStream_t s = w.stream;
    DevCounters* c = w.dcnt;
    w.warm0Valid = false;
    if (nM == 0) {
        cudaMemsetAsync(&c->maxColour, 0, sizeof(uint32_t), s);
        return cudaGetLastError();
    }
    if (!w.colourResident) {
        int dev = 0, sms = 0, perSm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kChainLocal, kLocalThreads, 0);
        w.colourResident = (unsigned)std::max(1, sms * std::max(perSm, 1));
    }
    const bool small = nM <= kSmallColour && w.n <= kSmallColour;
    // all CTAs resident, and no more than one per kLocalThreads manifolds
    const unsigned grid =
        small ? 1u : std::min<unsigned>(w.colourResident, std::max(1u, gridFor(nM, kLocalThreads)));
    // chunks: one first chunk per CTA, and per CTA at most one taken ahead beyond the
    // ceil(written / kChunk) it fills
    const size_t chunks = 2ull * grid + (nM + kChunk - 1u) / kChunk + 2u;
    cudaError_t e = w.colourPool.reserve(chunks * kChunk);
    if (e != cudaSuccess) return e;
    if ((e = w.colourChunkNext.reserve(chunks)) != cudaSuccess) return e;
    // the seed count lives in w.hist (reused scratch)
    uint32_t* seedCount = w.hist.p;
    // temporal mode: previous colours from the previous table
    const uint32_t prevSlot = w.wsCur ^ 1u;
    const PrevColours pc{w.cfg.temporal_colouring && w.wsValid ? w.wsSlots[prevSlot].p : nullptr,
                         w.wsLog2[prevSlot], w.wsGen[prevSlot]};
    const uint32_t temporal = pc.table ? 1u : 0u;
    uint4* rec = w.manRec.p;
    // with a previous table probed here, point 0's previous impulses go to warm0 for the
    // solver preparation
    float4* warm0 = nullptr;
    if (temporal) {
        cudaError_t ew = w.warm0.reserve(w.mhdr.cap);
        if (ew != cudaSuccess) return ew;
        warm0 = w.warm0.p;
    }
    w.warm0Valid = temporal != 0u;
    const ChunkPool pool{w.colourPool.p, w.colourChunkNext.p, (uint32_t)chunks};
    w.lastRounds = kRoundsFromCounters;
    if (small) {
        kColourSmall<<<1, kLocalThreads, 0, s>>>(nM, w.n, w.mhdr.p, rec, w.bodyDeg.p, w.bodySlots.p, w.mcolour.p,
                                                 w.manSucc.p, w.manPending.p, w.bodyMask.p, w.work0.p, seedCount,
                                                 pool, w.order.p, w.orderInv.p, pc, warm0, temporal, c);
        launches += 1;
        return cudaGetLastError();
    }
    cudaMemsetAsync(seedCount, 0, sizeof(uint32_t), s);
    cudaMemsetAsync(w.bodyDeg.p, 0, sizeof(uint32_t) * w.n, s);
    // the gated passes stride over their range with at most this many CTAs
    const unsigned gatedM = std::min<unsigned>(gridFor(nM, 256), 152u * 4u);
    const unsigned gatedN = std::min<unsigned>(gridFor(w.n, 256), 152u * 4u);
    kChainInit<<<gridFor(nM, 256), 256, 0, s>>>(nM, w.n, w.mhdr.p, rec, w.bodyDeg.p, w.bodySlots.p, w.mcolour.p,
                                                w.manPending.p, pc, warm0, &c->crowdSeen);
    kChainFlags<<<gatedM, 256, 0, s>>>(nM, w.mhdr.p, w.bodyDeg.p, rec, &c->crowdSeen);
    kChainLink<<<gridFor(w.n, 256), 256, 0, s>>>(w.n, w.bodyDeg.p, w.bodySlots.p, rec, temporal, w.manSucc.p,
                                                 w.manPending.p, w.bodyMask.p, temporal ? &c->colourConflict : nullptr,
                                                 nullptr);
    if (temporal) {
        kChainConflicts<<<gatedN, 256, 0, s>>>(w.n, w.bodyDeg.p, w.bodySlots.p, rec, &c->colourConflict);
        kChainReset<<<gatedM, 256, 0, s>>>(nM, w.manPending.p, &c->colourConflict);
        kChainLink<<<gatedN, 256, 0, s>>>(w.n, w.bodyDeg.p, w.bodySlots.p, rec, temporal, w.manSucc.p,
                                          w.manPending.p, w.bodyMask.p, nullptr, &c->colourConflict);
    }
    kChainSeed<<<gridFor(nM, 256), 256, 0, s>>>(nM, w.manPending.p, w.mcolour.p, rec, temporal, w.work0.p,
                                                seedCount);
    kChainLocal<<<grid, kLocalThreads, 0, s>>>(w.work0.p, seedCount, pool, w.mhdr.p, w.manSucc.p, w.manPending.p,
                                               w.bodyMask.p, w.mcolour.p, c);
    // group by colour: one stable 8-bit radix pass over the colours, which also writes the
    // inverse order and the colour bounds (maxColour is zero since the step began)
    groupByColour(s, w.mcolour.p, w.order.p, w.orderInv.p, w.hist.p, nM, c);
    launches += temporal ? 11 : 8;
    return cudaGetLastError();
}

}  // namespace axiom_gb300
