// colour.cu — deterministic colouring of the contact graph (Jones-Plassmann rounds).
//
// Vertices are manifolds; two conflict when they share a dynamic body (static and
// kinematic bodies are never written by the solver, so they do not constrain colours).
// Priority of a manifold = SplitMix64(pairKey(a, b)), a bijection, so priorities are
// distinct.  In each round every uncoloured manifold that holds the highest priority
// among the uncoloured manifolds of each of its dynamic bodies takes the lowest colour
// free at those bodies.  Winners of one round share no body, so the round is race-free,
// and the result equals greedy first-fit colouring in descending priority order — what
// the CPU oracle computes sequentially.  Then a stable one-digit radix pass groups the
// manifolds by colour.
#include "dmath.cuh"
#include "world.h"

namespace axiom_gb300 {
namespace {

using namespace axd;

constexpr uint32_t kMaxRounds = 1024;

// Worklist entry of manifold m: (a, b, m, dynamic bits of the header).
// Seed: every manifold enters round 0, and raises round 0's priority buffer at its
// dynamic bodies.
__global__ void __launch_bounds__(256) kColourSeed(uint32_t nM, const uint4* __restrict__ hdr,
                                                   uint4* __restrict__ work,
                                                   unsigned long long* __restrict__ prio0,
                                                   uint32_t* __restrict__ colour) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nM) return;
    const uint4 h = hdr[m];
    work[m] = make_uint4(h.x, h.y, m, h.w & (kHdrDynA | kHdrDynB));
    colour[m] = 0xFFFFFFFFu;
    const unsigned long long p = mix64(pairKey(h.x, h.y));
    if (h.w & kHdrDynA) atomicMax(&prio0[h.x], p);
    if (h.w & kHdrDynB) atomicMax(&prio0[h.y], p);
}

// Round r over the worklist wl (wlCount[r] entries), with three rotating priority buffers:
//   cur  = max priority over this round's manifolds at each body (raised by the previous
//          round's losers, or by the seed);
//   nxt  = raised here by this round's losers for round r + 1;
//   clr  = the buffer round r - 1 read; it becomes round r + 2's nxt, so it is cleared
//          here at the bodies of this round's manifolds.
// A manifold wins when it holds the maximum at each of its dynamic bodies.  Every entry
// of clr that round r - 1 read is cleared: the manifold that held the maximum at a body
// either lost and is in this round (clears it below) or won and cleared it in cur then.
// A winner clearing its own maximum in cur cannot change another manifold's outcome at
// that body: any other manifold there has a smaller (distinct, non-zero) priority and
// loses whether it reads the maximum or zero.  Winners take the lowest colour free at
// their bodies (winners of one round share no body); losers go to the next worklist.
__global__ void __launch_bounds__(256) kRound(const uint4* __restrict__ wl, uint32_t* __restrict__ wlCount,
                                              uint32_t r, uint4* __restrict__ next,
                                              unsigned long long* __restrict__ cur,
                                              unsigned long long* __restrict__ nxt,
                                              unsigned long long* __restrict__ clr,
                                              unsigned long long* __restrict__ mask,
                                              uint32_t* __restrict__ colour, DevCounters* cnt) {
    const uint32_t count = wlCount[r];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t trips = (count + stride - 1) / stride;
    const int lane = threadIdx.x & 31;
    for (uint32_t tr = 0; tr < trips; ++tr) {
        const uint32_t t = tr * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool lose = false;
        uint4 e = make_uint4(0u, 0u, 0u, 0u);
        if (t < count) {
            e = wl[t];
            const unsigned long long p = mix64(pairKey(e.x, e.y));
            const bool da = (e.w & kHdrDynA) != 0u, db = (e.w & kHdrDynB) != 0u;
            const bool win = (!da || cur[e.x] == p) && (!db || cur[e.y] == p);
            if (da) clr[e.x] = 0ull;
            if (db) clr[e.y] = 0ull;
            if (win) {
                const unsigned long long ma = da ? mask[e.x] : 0ull;
                const unsigned long long mb = db ? mask[e.y] : 0ull;
                const unsigned long long used = ma | mb;
                uint32_t c;
                if (used == ~0ull) {
                    atomicOr(&cnt->colourOverflow, 1u);
                    c = kMaxColours - 1;
                } else {
                    c = (uint32_t)(__ffsll((long long)~used) - 1);
                }
                const unsigned long long bit = 1ull << c;
                if (da) {
                    mask[e.x] = ma | bit;
                    cur[e.x] = 0ull;
                }
                if (db) {
                    mask[e.y] = mb | bit;
                    cur[e.y] = 0ull;
                }
                colour[e.z] = c;
                atomicMax(&cnt->maxColour, c + 1u);
            } else {
                lose = true;
                if (da) atomicMax(&nxt[e.x], p);
                if (db) atomicMax(&nxt[e.y], p);
            }
        }
        const unsigned ballot = __ballot_sync(0xFFFFFFFFu, lose);
        if (ballot) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&wlCount[r + 1], (uint32_t)__popc(ballot));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (lose) next[base + __popc(ballot & ((1u << lane) - 1u))] = e;
        }
    }
}

__global__ void __launch_bounds__(256) kColourKeys(uint32_t nM, const uint32_t* __restrict__ colour,
                                                   uint32_t* __restrict__ keys,
                                                   uint32_t* __restrict__ vals) {
    uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nM) return;
    keys[m] = colour[m];
    vals[m] = m;
}

// colourStart[c] = first sorted position of colour c; colourStart[maxColour] = nM.
__global__ void __launch_bounds__(256) kColourBounds(uint32_t nM, const uint32_t* __restrict__ sortedColour,
                                                     DevCounters* cnt) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) cnt->colourStart[cnt->maxColour] = nM;
    if (s >= nM) return;
    const uint32_t c = sortedColour[s];
    if (s == 0) {
        for (uint32_t k = 0; k <= c; ++k) cnt->colourStart[k] = 0;
    } else {
        const uint32_t pc = sortedColour[s - 1];
        for (uint32_t k = pc + 1; k <= c; ++k) cnt->colourStart[k] = s;
    }
}

}  // namespace

// Colours w.mhdr[0..nM) into w.mcolour, and leaves the colour-sorted manifold order in
// w.order with bounds in dcnt->colourStart.  Host-synchronising: it reads the worklist
// size every few rounds to stop launching.
cudaError_t colourManifolds(World& w, uint32_t nM) {
    ProfRange pr(w, KG_COLOURING);
    uint64_t& launches = w.prof.launches[KG_COLOURING];
    cudaStream_t s = w.stream;
    DevCounters* c = w.dcnt;
    if (nM == 0) {
        cudaMemsetAsync(&c->maxColour, 0, sizeof(uint32_t), s);
        return cudaGetLastError();
    }
    // worklist counts per round live in w.hist (reused, large enough: >= kMaxRounds + 1)
    uint32_t* wlCount = w.hist.p;
    cudaMemsetAsync(wlCount, 0, sizeof(uint32_t) * (kMaxRounds + 1), s);
    cudaMemcpyAsync(wlCount, &nM, sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    // three rotating priority buffers (3n words), see kRound
    cudaMemsetAsync(w.bodyPrio.p, 0, sizeof(unsigned long long) * 3ull * w.n, s);
    cudaMemsetAsync(w.bodyMask.p, 0, sizeof(unsigned long long) * w.n, s);
    unsigned long long* prio[3] = {w.bodyPrio.p, w.bodyPrio.p + w.n, w.bodyPrio.p + 2ull * w.n};
    kColourSeed<<<gridFor(nM, 256), 256, 0, s>>>(nM, w.mhdr.p, w.work0.p, prio[0], w.mcolour.p);
    launches += 1;
    uint4* cur = w.work0.p;
    uint4* nxt = w.work1.p;
    uint32_t known = nM;  // upper bound of the current worklist size
    uint32_t r = 0;
    uint32_t batch = 8;  // rounds launched between two reads of the worklist size
    while (known > 0) {
        if (r + batch >= kMaxRounds) return cudaErrorUnknown;
        for (uint32_t b = 0; b < batch; ++b, ++r) {
            const unsigned grid = min(gridFor(known, 256), 152u * 16u);
            kRound<<<grid, 256, 0, s>>>(cur, wlCount, r, nxt, prio[r % 3u], prio[(r + 1u) % 3u],
                                        prio[(r + 2u) % 3u], w.bodyMask.p, w.mcolour.p, c);
            launches += 1;
            uint4* t = cur;
            cur = nxt;
            nxt = t;
        }
        cudaMemcpyAsync(&w.hcnt->worklist, &wlCount[r], sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return e;
        known = w.hcnt->worklist;
        batch = 4;
    }
    w.lastRounds = r;
    // group by colour: one stable 8-bit radix pass of (colour, manifold)
    kColourKeys<<<gridFor(nM, 256), 256, 0, s>>>(nM, w.mcolour.p, w.keyA.p, w.valA.p);
    radixSort(s, w.keyA.p, w.valA.p, w.keyB.p, w.order.p, w.hist.p, nM, 1);
    kColourBounds<<<gridFor(nM, 256), 256, 0, s>>>(nM, w.keyB.p, c);
    launches += 5;
    return cudaGetLastError();
}

}  // namespace axiom_gb300
