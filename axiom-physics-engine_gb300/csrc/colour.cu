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

__global__ void __launch_bounds__(256) kColourInit(uint32_t nM, uint32_t* __restrict__ work,
                                                   uint32_t* __restrict__ colour) {
    uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nM) return;
    work[m] = m;
    colour[m] = 0xFFFFFFFFu;
}

// Round r: raise each dynamic body's max priority over its uncoloured manifolds.
__global__ void __launch_bounds__(256) kSelect(const uint32_t* __restrict__ wl,
                                               const uint32_t* __restrict__ wlCount, uint32_t r,
                                               const uint4* __restrict__ hdr,
                                               unsigned long long* __restrict__ prio) {
    const uint32_t count = wlCount[r];
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
        const uint4 h = hdr[wl[t]];
        const unsigned long long p = mix64(pairKey(h.x, h.y));
        if (h.w & kHdrDynA) atomicMax(&prio[h.x], p);
        if (h.w & kHdrDynB) atomicMax(&prio[h.y], p);
    }
}

// Winners take the lowest colour free at their bodies; losers go to the next list.
__global__ void __launch_bounds__(256) kAssign(const uint32_t* __restrict__ wl,
                                               uint32_t* __restrict__ wlCount, uint32_t r,
                                               uint32_t* __restrict__ next,
                                               const uint4* __restrict__ hdr,
                                               const unsigned long long* __restrict__ prio,
                                               unsigned long long* __restrict__ prioNext,
                                               unsigned long long* __restrict__ mask,
                                               uint32_t* __restrict__ colour, DevCounters* cnt) {
    const uint32_t count = wlCount[r];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t trips = (count + stride - 1) / stride;
    const int lane = threadIdx.x & 31;
    for (uint32_t tr = 0; tr < trips; ++tr) {
        const uint32_t t = tr * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool lose = false;
        uint32_t m = 0;
        if (t < count) {
            m = wl[t];
            const uint4 h = hdr[m];
            const unsigned long long p = mix64(pairKey(h.x, h.y));
            const bool da = (h.w & kHdrDynA) != 0u, db = (h.w & kHdrDynB) != 0u;
            const bool win = (!da || prio[h.x] == p) && (!db || prio[h.y] == p);
            if (win) {
                const unsigned long long ma = da ? mask[h.x] : 0ull;
                const unsigned long long mb = db ? mask[h.y] : 0ull;
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
                colour[m] = c;
                atomicMax(&cnt->maxColour, c + 1u);
            } else {
                // still uncoloured: clear its bodies in the next round's priority buffer
                lose = true;
                prioNext[h.x] = 0ull;
                prioNext[h.y] = 0ull;
            }
        }
        const unsigned ballot = __ballot_sync(0xFFFFFFFFu, lose);
        if (ballot) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&wlCount[r + 1], (uint32_t)__popc(ballot));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (lose) next[base + __popc(ballot & ((1u << lane) - 1u))] = m;
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
    // two priority buffers (2n words): round r raises buffer r&1 while its losers clear
    // their bodies in buffer (r+1)&1 for the next round
    cudaMemsetAsync(w.bodyPrio.p, 0, sizeof(unsigned long long) * 2ull * w.n, s);
    cudaMemsetAsync(w.bodyMask.p, 0, sizeof(unsigned long long) * w.n, s);
    kColourInit<<<gridFor(nM, 256), 256, 0, s>>>(nM, w.work0.p, w.mcolour.p);
    launches += 1;
    uint32_t* cur = w.work0.p;
    uint32_t* nxt = w.work1.p;
    unsigned long long* prio[2] = {w.bodyPrio.p, w.bodyPrio.p + w.n};
    uint32_t known = nM;  // upper bound of the current worklist size
    uint32_t r = 0;
    uint32_t batch = 8;  // rounds launched between two reads of the worklist size
    while (known > 0) {
        if (r + batch >= kMaxRounds) return cudaErrorUnknown;
        for (uint32_t b = 0; b < batch; ++b, ++r) {
            const unsigned grid = min(gridFor(known, 256), 152u * 16u);
            kSelect<<<grid, 256, 0, s>>>(cur, wlCount, r, w.mhdr.p, prio[r & 1u]);
            kAssign<<<grid, 256, 0, s>>>(cur, wlCount, r, nxt, w.mhdr.p, prio[r & 1u],
                                         prio[(r + 1u) & 1u], w.bodyMask.p, w.mcolour.p, c);
            launches += 2;
            uint32_t* t = cur;
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
