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
// counts its predecessors, (3) seeds the first frontier with the manifolds that have
// none, and (4) colours frontier after frontier: a coloured manifold releases its
// successors, and a successor whose last predecessor this was joins the next frontier.
// Frontier r holds exactly the manifolds a Jones-Plassmann round r would colour, but
// each manifold is visited once instead of once per round.  Manifolds of one frontier
// share no dynamic body, so the mask updates are race-free.  Then a stable one-digit
// radix pass groups the manifolds by colour.
#include <algorithm>
#include <vector>

#include "dmath.cuh"
#include "grid_sync.cuh"
#include "world.h"

namespace axiom_gb300 {
namespace {

using namespace axd;

constexpr uint32_t kMaxRounds = 1024;

constexpr uint32_t kSlots = kMaxColours;  // chain slots per dynamic body
constexpr uint32_t kRoundThreads = 1024;  // big CTAs: fewer arrivals on the shared counters
constexpr uint32_t kSideB = 0x80000000u;    // slot entry: manifold id | side bit
constexpr uint32_t kNone = 0xFFFFFFFFu;

// (1) priorities, and each manifold in the slot list of each of its dynamic bodies
__global__ void __launch_bounds__(256) kChainInit(uint32_t nM, const uint4* __restrict__ hdr,
                                                  unsigned long long* __restrict__ prio,
                                                  uint32_t* __restrict__ deg, uint32_t* __restrict__ slots,
                                                  uint32_t* __restrict__ colour, DevCounters* cnt) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nM) return;
    const uint4 h = hdr[m];
    prio[m] = mix64(pairKey(h.x, h.y));
    colour[m] = kNone;
    if (h.w & kHdrDynA) {
        const uint32_t k = atomicAdd(&deg[h.x], 1u);
        if (k < kSlots) slots[(size_t)h.x * kSlots + k] = m;
        else atomicOr(&cnt->colourOverflow, 1u);
    }
    if (h.w & kHdrDynB) {
        const uint32_t k = atomicAdd(&deg[h.y], 1u);
        if (k < kSlots) slots[(size_t)h.y * kSlots + k] = m | kSideB;
        else atomicOr(&cnt->colourOverflow, 1u);
    }
}

constexpr uint32_t kLinkRegs = 16;  // bodies with at most this many manifolds link in registers

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
// longer lists re-read their entries.
__global__ void __launch_bounds__(256) kChainLink(uint32_t n, const uint32_t* __restrict__ deg,
                                                  const uint32_t* __restrict__ slots,
                                                  const unsigned long long* __restrict__ prio,
                                                  uint2* __restrict__ succ, uint32_t* __restrict__ pending) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const uint32_t d = min(deg[x], kSlots);
    if (d == 0) return;
    const uint32_t* list = slots + (size_t)x * kSlots;
    if (d <= kLinkRegs) {
        uint32_t e[kLinkRegs];
        unsigned long long p[kLinkRegs];
#pragma unroll
        for (uint32_t i = 0; i < kLinkRegs; ++i) {
            e[i] = i < d ? list[i] : kNone;
            p[i] = i < d ? prio[e[i] & ~kSideB] : 0ull;
        }
#pragma unroll
        for (uint32_t i = 0; i < kLinkRegs; ++i) {
            if (i >= d) break;
            bool pred = false;
            unsigned long long bestP = 0ull;
            uint32_t best = kNone;
#pragma unroll
            for (uint32_t j = 0; j < kLinkRegs; ++j) {
                if (j < d) {
                    if (p[j] > p[i]) pred = true;
                    else if (p[j] < p[i] && (best == kNone || p[j] > bestP)) {
                        bestP = p[j];
                        best = e[j] & ~kSideB;
                    }
                }
            }
            linkOne(e[i], best, pred, succ, pending);
        }
        return;
    }
    for (uint32_t i = 0; i < d; ++i) {
        const uint32_t ei = list[i], mi = ei & ~kSideB;
        const unsigned long long pi = prio[mi];
        bool pred = false;
        unsigned long long bestP = 0ull;
        uint32_t best = kNone;
        for (uint32_t j = 0; j < d; ++j) {
            const uint32_t mj = list[j] & ~kSideB;
            const unsigned long long pj = prio[mj];
            if (pj > pi) pred = true;
            else if (pj < pi && (best == kNone || pj > bestP)) {
                bestP = pj;
                best = mj;
            }
        }
        linkOne(ei, best, pred, succ, pending);
    }
}

// Block-aggregated append of m to list[count++] for the threads with add set: one atomic
// per block (a frontier counter hit by every warp of the grid serialises in L2).  Every
// thread of the block calls it.
__device__ __forceinline__ void appendBlock(bool add, uint32_t m, uint32_t* list, uint32_t* count) {
    __shared__ uint32_t warpBase[32];
    __shared__ uint32_t blockBase;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned ballot = __ballot_sync(0xFFFFFFFFu, add);
    if (lane == 0) warpBase[warp] = (uint32_t)__popc(ballot);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t total = 0;
        for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) {
            const uint32_t c = warpBase[w];
            warpBase[w] = total;
            total += c;
        }
        blockBase = total ? atomicAdd(count, total) : 0u;
    }
    __syncthreads();
    if (add) list[blockBase + warpBase[warp] + __popc(ballot & ((1u << lane) - 1u))] = m;
    __syncthreads();  // warpBase / blockBase are reused by the next call
}

// (3) first frontier: manifolds without a predecessor at either body
__global__ void __launch_bounds__(256) kChainSeed(uint32_t nM, const uint32_t* __restrict__ pending,
                                                  uint32_t* __restrict__ front, uint32_t* __restrict__ count) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ready = m < nM && pending[m] == 0u;
    appendBlock(ready, m, front, count);
}

// (4) frontier r: colour, then release the successors.  Frontier entries, masks and
// counts are written by other CTAs within the persistent kernel, so they are read
// through L2 (ld.global.cg).
__device__ __forceinline__ void chainRound(uint32_t count, const uint32_t* __restrict__ front, uint32_t* nextCount,
                                           uint32_t* __restrict__ next, const uint4* __restrict__ hdr,
                                           const uint2* __restrict__ succ, uint32_t* __restrict__ pending,
                                           unsigned long long* __restrict__ mask, uint32_t* __restrict__ colour,
                                           DevCounters* cnt) {
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t trips = (count + stride - 1) / stride;
    for (uint32_t tr = 0; tr < trips; ++tr) {
        const uint32_t t = tr * stride + blockIdx.x * blockDim.x + threadIdx.x;
        uint32_t s0 = kNone, s1 = kNone;
        if (t < count) {
            const uint32_t m = __ldcg(&front[t]);
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
            colour[m] = c;  // the colour count comes from the sorted colours (kColourBounds)
            if (da && sc.x != kNone && atomicSub(&pending[sc.x], 1u) == 1u) s0 = sc.x;
            if (db && sc.y != kNone && atomicSub(&pending[sc.y], 1u) == 1u) s1 = sc.y;
        }
        // one reservation for both successors: a frontier counter that every CTA hits
        // serialises in L2, so CTAs reserve once per trip
        const uint32_t k = (s0 != kNone ? 1u : 0u) + (s1 != kNone ? 1u : 0u);
        uint32_t at = blockReserve(k, nextCount);
        if (s0 != kNone) next[at++] = s0;
        if (s1 != kNone) next[at] = s1;
    }
}

// One frontier round per launch (used when a cooperative launch is not available).
__global__ void __launch_bounds__(kRoundThreads) kChainRound(const uint32_t* __restrict__ front, uint32_t* __restrict__ wlCount,
                                                   uint32_t r, uint32_t* __restrict__ next,
                                                   const uint4* __restrict__ hdr, const uint2* __restrict__ succ,
                                                   uint32_t* __restrict__ pending,
                                                   unsigned long long* __restrict__ mask,
                                                   uint32_t* __restrict__ colour, DevCounters* cnt) {
    chainRound(wlCount[r], front, &wlCount[r + 1], next, hdr, succ, pending, mask, colour, cnt);
}

// All frontier rounds in one cooperative launch, a grid barrier between rounds; every CTA
// reads the next frontier's size after the barrier, so all stop at the same round.
__global__ void __launch_bounds__(kRoundThreads) kChainRounds(uint32_t* __restrict__ work0, uint32_t* __restrict__ work1,
                                                    uint32_t* __restrict__ wlCount, const uint4* __restrict__ hdr,
                                                    const uint2* __restrict__ succ, uint32_t* __restrict__ pending,
                                                    unsigned long long* __restrict__ mask,
                                                    uint32_t* __restrict__ colour, DevCounters* cnt) {
    uint32_t r = 0;
    for (; r < kMaxRounds; ++r) {
        const uint32_t count = __ldcg(&wlCount[r]);
        if (count == 0u) break;
        const uint32_t* front = (r & 1u) ? work1 : work0;
        uint32_t* next = (r & 1u) ? work0 : work1;
        chainRound(count, front, &wlCount[r + 1], next, hdr, succ, pending, mask, colour, cnt);
        if (!gridBarrier(&cnt->gridBar, (r + 1u) * gridDim.x, cnt)) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt->colourRounds = r;
}

__global__ void __launch_bounds__(256) kColourKeys(uint32_t nM, const uint32_t* __restrict__ colour,
                                                   uint32_t* __restrict__ keys,
                                                   uint32_t* __restrict__ vals) {
    uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nM) return;
    // a manifold left uncoloured (only after a colour overflow, which fails the step) goes
    // to the last colour so that the bounds stay inside the 64 colours
    const uint32_t c = colour[m];
    keys[m] = c < (uint32_t)kMaxColours ? c : (uint32_t)kMaxColours - 1u;
    vals[m] = m;
}

// inv[order[s]] = s: where each manifold (narrowphase order) sits in colour order.
__global__ void __launch_bounds__(256) kInvertOrder(uint32_t nM, const uint32_t* __restrict__ order,
                                                    uint32_t* __restrict__ inv) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nM) inv[order[s]] = s;
}

// colourStart[c] = first sorted position of colour c; maxColour = the last sorted colour
// + 1 and colourStart[maxColour] = nM.
__global__ void __launch_bounds__(256) kColourBounds(uint32_t nM, const uint32_t* __restrict__ sortedColour,
                                                     DevCounters* cnt) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nM) return;
    const uint32_t c = sortedColour[s];
    if (s == nM - 1u) {
        cnt->maxColour = c + 1u;
        cnt->colourStart[c + 1u] = nM;
    }
    if (s == 0) {
        for (uint32_t k = 0; k <= c; ++k) cnt->colourStart[k] = 0;
    } else {
        const uint32_t pc = sortedColour[s - 1];
        for (uint32_t k = pc + 1; k <= c; ++k) cnt->colourStart[k] = s;
    }
}

}  // namespace

// Frontier rounds as one launch per round, reading the frontier size every few rounds;
// sets w.lastRounds to the number of non-empty frontiers.
static cudaError_t roundsByLaunches(World& w, uint32_t nM, uint32_t* wlCount, uint64_t& launches) {
    cudaStream_t s = w.stream;
    uint32_t* cur = w.work0.p;
    uint32_t* nxt = w.work1.p;
    uint32_t known = nM;  // upper bound of the current frontier size
    uint32_t r = 0;
    uint32_t batch = 8;  // rounds launched between two reads of the frontier size
    while (known > 0) {
        if (r + batch >= kMaxRounds) return cudaErrorUnknown;
        for (uint32_t b = 0; b < batch; ++b, ++r) {
            const unsigned grid = min(gridFor(known, kRoundThreads), 152u * 2u);
            kChainRound<<<grid, kRoundThreads, 0, s>>>(cur, wlCount, r, nxt, w.mhdr.p, w.manSucc.p, w.manPending.p,
                                             w.bodyMask.p, w.mcolour.p, w.dcnt);
            launches += 1;
            uint32_t* t = cur;
            cur = nxt;
            nxt = t;
        }
        cudaMemcpyAsync(&w.hcnt->worklist, &wlCount[r], sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        known = w.hcnt->worklist;
        batch = 4;
    }
    std::vector<uint32_t> counts(r + 1);
    cudaMemcpy(counts.data(), wlCount, sizeof(uint32_t) * (r + 1), cudaMemcpyDeviceToHost);
    uint32_t depth = 0;
    while (depth <= r && counts[depth] != 0u) ++depth;
    w.lastRounds = depth;
    return cudaGetLastError();
}

// Colours w.mhdr[0..nM) into w.mcolour, and leaves the colour-sorted manifold order in
// w.order with bounds in dcnt->colourStart.  With a cooperative launch the rounds run on
// the device without host synchronisation (their count arrives in dcnt->colourRounds);
// otherwise one launch per round.
cudaError_t colourManifolds(World& w, uint32_t nM) {
    ProfRange pr(w, KG_COLOURING);
    uint64_t& launches = w.prof.launches[KG_COLOURING];
    cudaStream_t s = w.stream;
    DevCounters* c = w.dcnt;
    if (nM == 0) {
        cudaMemsetAsync(&c->maxColour, 0, sizeof(uint32_t), s);
        return cudaGetLastError();
    }
    // frontier sizes per round live in w.hist (reused, large enough: >= kMaxRounds + 1)
    uint32_t* wlCount = w.hist.p;
    cudaMemsetAsync(wlCount, 0, sizeof(uint32_t) * (kMaxRounds + 1), s);
    cudaMemsetAsync(w.bodyDeg.p, 0, sizeof(uint32_t) * w.n, s);
    cudaMemsetAsync(w.bodyMask.p, 0, sizeof(unsigned long long) * w.n, s);
    cudaMemsetAsync(w.manPending.p, 0, sizeof(uint32_t) * nM, s);
    cudaMemsetAsync(w.manSucc.p, 0xFF, sizeof(uint2) * nM, s);
    kChainInit<<<gridFor(nM, 256), 256, 0, s>>>(nM, w.mhdr.p, w.manPrio.p, w.bodyDeg.p, w.bodySlots.p,
                                                w.mcolour.p, c);
    kChainLink<<<gridFor(w.n, 256), 256, 0, s>>>(w.n, w.bodyDeg.p, w.bodySlots.p, w.manPrio.p, w.manSucc.p,
                                                 w.manPending.p);
    kChainSeed<<<gridFor(nM, 256), 256, 0, s>>>(nM, w.manPending.p, w.work0.p, wlCount);
    launches += 3;
    if (!w.colourGrid) {
        int dev = 0, sms = 0, perSm = 0, coop = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kChainRounds, kRoundThreads, 0);
        w.colourGrid = (coop && perSm > 0) ? (unsigned)(sms * perSm) : ~0u;
    }
    if (w.colourGrid != ~0u) {
        // every round in one cooperative launch; the round count comes back with the
        // counters (colourRounds)
        uint32_t* work0 = w.work0.p;
        uint32_t* work1 = w.work1.p;
        const uint4* hdr = w.mhdr.p;
        const uint2* succ = w.manSucc.p;
        uint32_t* pending = w.manPending.p;
        unsigned long long* mask = w.bodyMask.p;
        uint32_t* colour = w.mcolour.p;
        void* args[] = {&work0, &work1, &wlCount, &hdr, &succ, &pending, &mask, &colour, &c};
        const unsigned grid = std::min<unsigned>(w.colourGrid, std::max(1u, gridFor(nM, kRoundThreads)));
        if (cudaLaunchCooperativeKernel((const void*)kChainRounds, dim3(grid), dim3(kRoundThreads), args, 0, s) ==
            cudaSuccess) {
            launches += 1;
            w.lastRounds = kRoundsFromCounters;
        } else {
            cudaGetLastError();  // not sticky: use the per-round launches
            w.colourGrid = ~0u;
        }
    }
    if (w.colourGrid == ~0u) {
        const cudaError_t e = roundsByLaunches(w, nM, wlCount, launches);
        if (e != cudaSuccess) return e;
    }
    // group by colour: one stable 8-bit radix pass of (colour, manifold)
    kColourKeys<<<gridFor(nM, 256), 256, 0, s>>>(nM, w.mcolour.p, w.keyA.p, w.valA.p);
    radixSort(s, w.keyA.p, w.valA.p, w.keyB.p, w.order.p, w.hist.p, nM, 1);
    kColourBounds<<<gridFor(nM, 256), 256, 0, s>>>(nM, w.keyB.p, c);
    kInvertOrder<<<gridFor(nM, 256), 256, 0, s>>>(nM, w.order.p, w.orderInv.p);
    launches += 6;
    return cudaGetLastError();
}

}  // namespace axiom_gb300
