// broadphase.cu — Morton-ordered uniform-grid sweep over SoA AABBs.
//
// The reference's only broadphase is an O(N^2) toy (examples/profiling_example.cpp:49-69);
// its collision layer is empty.  Pair set produced here: every (a < b), neither a plane,
// at least one awake dynamic, whose AABBs intersect inclusively (AABB::intersects,
// include/axiom/math/aabb.hpp:132-135); also a sleeping body with a moving kinematic
// body, so that the contact can wake the sleeper.
//
// Method.  The cell size is >= the widest AABB, so two intersecting AABBs have min
// corners in the same or adjacent cells.  Bodies are radix-sorted by the 30-bit Morton
// code of their (wrapped, 10 bits per axis) min-corner cell, which puts each cell's
// bodies in one contiguous run and neighbouring cells close in memory.  A hash table maps
// a cell key to the start of its run.  Each body then sweeps its own run (partners after
// it) and the runs of the 13 "forward" neighbour cells, testing full AABB overlap; the
// forward half-stencil reports every pair exactly once.  Pairs whose collision filters
// reject each other (gui::FilterInfo, body_inspector.hpp:38-42) are not reported; the
// filters are read only when one of the two bodies has a non-default one.  Wrapping the coordinates can
// only put distant cells on one key, and those fail the AABB test.
//
// (A single-axis sweep-and-prune sorted on min.x would scan whole lattice layers on the
// dense 1M-sphere pile: about 12,000 candidates per body instead of about 14.)
//
// Hits are compacted through a per-block shared-memory stage and one global atomic per
// block; pair order is therefore not deterministic, but nothing downstream depends on it.
#include "dmath.cuh"
#include "world.h"

namespace axiom_gb300 {
namespace {

constexpr int kSweepThreads = 256;
constexpr int kStage = 4096;

__device__ __forceinline__ uint32_t compact10(uint32_t v) {
    v &= 0x09249249u;
    v = (v | (v >> 2)) & 0x030C30C3u;
    v = (v | (v >> 4)) & 0x0300F00Fu;
    v = (v | (v >> 8)) & 0x030000FFu;
    v = (v | (v >> 16)) & 0x000003FFu;
    return v;
}
__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__device__ __forceinline__ uint32_t cellHash(uint32_t key, uint32_t log2T) {
    return (key * 2654435761u) >> (32u - log2T);
}

// Gathers AABBs into sorted order (id and dynamic flag in the .w lanes) and registers the
// first position of every cell run in the hash table.
__global__ void __launch_bounds__(256) kGatherCells(uint32_t nAll, uint32_t nSorted,
                                                    const uint32_t* __restrict__ skey,
                                                    const uint32_t* __restrict__ sval,
                                                    const float4* __restrict__ aabbMin,
                                                    const float4* __restrict__ aabbMax,
                                                    const uint32_t* __restrict__ info,
                                                    const SolverBody* __restrict__ sb,
                                                    SortedBox* __restrict__ sbox,
                                                    unsigned long long* __restrict__ table,
                                                    uint32_t log2T, DevCounters* cnt) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nAll) return;
    const uint32_t id = sval[i];
    const float4 mn = aabbMin[id], mx = aabbMax[id];
    const uint32_t inf = info[id];
    const uint32_t type = inf & kInfoTypeMask;
    // .w of the max corner: kSweep* bits (awake dynamic, non-default filter, sleeping, moving
    // kinematic, and whether the next sorted box is in the same cell)
    uint32_t flags = (type == AXIOM_BODY_DYNAMIC ? kSweepDynamic : 0u) | ((inf & kInfoFiltered) ? kSweepFiltered : 0u) |
                     (type == kTypeSleeping ? kSweepSleeping : 0u);
    if (type == AXIOM_BODY_KINEMATIC) {
        const float4 v = sb[id].v, w = sb[id].w;
        if (v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || w.x != 0.0f || w.y != 0.0f || w.z != 0.0f)
            flags |= kSweepMover;
    }
    const uint32_t key = i < nSorted ? skey[i] : kEmptyKey32;
    if (i + 1u < nSorted && skey[i + 1u] == key) flags |= kSweepRunNext;
    sbox[i] = SortedBox{make_float4(mn.x, mn.y, mn.z, __uint_as_float(id)), make_float4(mx.x, mx.y, mx.z, __uint_as_float(flags))};
    if (i >= nSorted) return;
    if (i > 0 && skey[i - 1] == key) return;
    const uint32_t mask = (1u << log2T) - 1u;
    const unsigned long long entry = ((unsigned long long)key << 32) | i;
    uint32_t h = cellHash(key, log2T);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        unsigned long long prev = atomicCAS(&table[h], kEmpty64, entry);
        if (prev == kEmpty64) return;
        h = (h + 1u) & mask;
    }
    atomicOr(&cnt->errorFlags, 1u);  // table full: cannot happen with size >= 2 * bodies
}

__device__ __forceinline__ uint32_t lookupCell(const unsigned long long* __restrict__ table,
                                               uint32_t log2T, uint32_t key) {
    const uint32_t mask = (1u << log2T) - 1u;
    uint32_t h = cellHash(key, log2T);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long e = table[h];
        if (e == kEmpty64) return kEmptyKey32;
        if ((uint32_t)(e >> 32) == key) return (uint32_t)e;
        h = (h + 1u) & mask;
    }
    return kEmptyKey32;
}

struct SweepStage {
    uint2 buf[kStage];
    uint32_t count;
    uint32_t base;
};

__device__ __forceinline__ void emitPair(SweepStage& st, uint32_t a, uint32_t b,
                                         uint2* __restrict__ pairs, uint32_t cap, DevCounters* cnt) {
    const uint2 pr = make_uint2(a < b ? a : b, a < b ? b : a);
    const uint32_t slot = atomicAdd(&st.count, 1u);
    if (slot < (uint32_t)kStage) {
        st.buf[slot] = pr;
    } else {
        const uint32_t g = atomicAdd(&cnt->pairs, 1u);
        if (g < cap) pairs[g] = pr;
    }
}

// Five CTAs per SM (48 registers, 8 bytes spilled, against 60 and four CTAs): the sweep
// lives on the latency of its probes and run walks.
__global__ void __launch_bounds__(kSweepThreads, 5) kSweep(uint32_t nSorted, const uint32_t* __restrict__ skey,
                                                        const SortedBox* __restrict__ sbox,
                                                        const unsigned long long* __restrict__ table,
                                                        uint32_t log2T, const uint4* __restrict__ filt,
                                                        uint2* __restrict__ pairs, uint32_t cap, DevCounters* cnt) {
    __shared__ SweepStage st;
    if (threadIdx.x == 0) st.count = 0;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nSorted) {
        const uint32_t key = skey[i];
        const SortedBox me = sbox[i];
        const float4 mn = me.mn, mx = me.mx;
        const uint32_t id = __float_as_uint(mn.w);
        const uint32_t fi = __float_as_uint(mx.w);
        // tests candidate j; returns its flags (kSweepRunNext: its cell run continues)
        auto test = [&](uint32_t j) -> uint32_t {
            const SortedBox o = sbox[j];
            const float4 bn = o.mn, bx = o.mx;
            const uint32_t fj = __float_as_uint(bx.w);
            if (!((fi | fj) & kSweepDynamic)) {  // neither awake dynamic: only a mover touching a sleeper
                if (!(((fi & kSweepSleeping) && (fj & kSweepMover)) || ((fi & kSweepMover) && (fj & kSweepSleeping))))
                    return fj;
            }
            if (mn.x <= bx.x && mx.x >= bn.x && mn.y <= bx.y && mx.y >= bn.y && mn.z <= bx.z &&
                mx.z >= bn.z) {
                const uint32_t jd = __float_as_uint(bn.w);
                if (((fi | fj) & kSweepFiltered) && !filterPass(filt[id], filt[jd])) return fj;
                emitPair(st, id, jd, pairs, cap, cnt);
            }
            return fj;
        };
        // forward half of the 26 neighbours, (dz, dy, dx) > (0, 0, 0) lexicographically.
        // The 13 hash probes are independent, so they are all issued before any is used,
        // and so are the first entries of the 13 runs: a thread waits for two rounds of
        // loads instead of 13 chains of them.  Longer probes and runs continue serially.
        const uint32_t cx = compact10(key), cy = compact10(key >> 1), cz = compact10(key >> 2);
        const uint32_t mask = (1u << log2T) - 1u;
        uint32_t nk[13];
        unsigned long long e[13];
#pragma unroll
        for (int o = 0; o < 13; ++o) {
            const int dx = o == 0 ? 1 : (o < 4 ? o - 2 : (o - 4) % 3 - 1);
            const int dy = o == 0 ? 0 : (o < 4 ? 1 : (o - 4) / 3 - 1);
            const int dz = o < 4 ? 0 : 1;
            nk[o] = spread10((cx + (uint32_t)dx) & 0x3FFu) | (spread10((cy + (uint32_t)dy) & 0x3FFu) << 1) |
                    (spread10((cz + (uint32_t)dz) & 0x3FFu) << 2);
            e[o] = table[cellHash(nk[o], log2T)];
        }
        uint32_t start[13];
#pragma unroll
        for (int o = 0; o < 13; ++o) {
            start[o] = kEmptyKey32;
            if (e[o] == kEmpty64) continue;
            if ((uint32_t)(e[o] >> 32) == nk[o]) {
                start[o] = (uint32_t)e[o];
                continue;
            }
            uint32_t h = (cellHash(nk[o], log2T) + 1u) & mask;  // collision: keep probing
            for (uint32_t probe = 1; probe <= mask; ++probe) {
                const unsigned long long x = table[h];
                if (x == kEmpty64) break;
                if ((uint32_t)(x >> 32) == nk[o]) {
                    start[o] = (uint32_t)x;
                    break;
                }
                h = (h + 1u) & mask;
            }
        }
        // own cell: partners later in the run (each box says whether its run continues)
        if (fi & kSweepRunNext)
            for (uint32_t j = i + 1; test(j) & kSweepRunNext; ++j) {
            }
#pragma unroll
        for (int o = 0; o < 13; ++o) {
            const uint32_t j0 = start[o];
            if (j0 == kEmptyKey32) continue;
            for (uint32_t j = j0; test(j) & kSweepRunNext; ++j) {  // a registered run has at least one entry
            }
        }
    }
    __syncthreads();
    const uint32_t staged = st.count < (uint32_t)kStage ? st.count : (uint32_t)kStage;
    if (threadIdx.x == 0) st.base = staged ? atomicAdd(&cnt->pairs, staged) : 0u;
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < staged; k += blockDim.x) {
        const uint32_t g = st.base + k;
        if (g < cap) pairs[g] = st.buf[k];
    }
}

__global__ void kMarkLarge(uint32_t nLarge, const uint32_t* __restrict__ ids, uint32_t* __restrict__ keys) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nLarge) keys[ids[k]] = kEmptyKey32;
}

// Sweep flags of body i, as kGatherCells computes them (without the run bit).
__device__ __forceinline__ uint32_t bodySweepFlags(uint32_t inf, const SolverBody& b) {
    const uint32_t type = inf & kInfoTypeMask;
    uint32_t flags = (type == AXIOM_BODY_DYNAMIC ? kSweepDynamic : 0u) | ((inf & kInfoFiltered) ? kSweepFiltered : 0u) |
                     (type == kTypeSleeping ? kSweepSleeping : 0u);
    if (type == AXIOM_BODY_KINEMATIC) {
        const float4 v = b.v, w = b.w;
        if (v.x != 0.0f || v.y != 0.0f || v.z != 0.0f || w.x != 0.0f || w.y != 0.0f || w.z != 0.0f)
            flags |= kSweepMover;
    }
    return flags;
}

// Pairs of large body ids[blockIdx.y] with every body: the same test as the sweep's (one
// awake dynamic, or a sleeper with a moving kinematic; inclusive AABB overlap; filters).
// A pair of two large bodies is reported by the one with the lower id.
__global__ void __launch_bounds__(256) kLargePairs(uint32_t n, uint32_t nLarge, const uint32_t* __restrict__ ids,
                                                   const uint32_t* __restrict__ info,
                                                   const SolverBody* __restrict__ sb,
                                                   const float4* __restrict__ aabbMin,
                                                   const float4* __restrict__ aabbMax,
                                                   const uint4* __restrict__ filt, uint2* __restrict__ pairs,
                                                   uint32_t cap, DevCounters* cnt) {
    __shared__ uint32_t sIds[kMaxLarge];
    for (uint32_t k = threadIdx.x; k < nLarge; k += blockDim.x) sIds[k] = ids[k];
    __syncthreads();
    const uint32_t l = sIds[blockIdx.y];
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    bool hit = false;
    if (j < n && j != l) {
        const uint32_t ij = info[j];
        bool skip = ((ij >> 4) & 0xFu) == AXIOM_SHAPE_PLANE;
        if (!skip && j < l) {  // j large too: the pair belongs to j's row
            uint32_t lo = 0, hi = nLarge;
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (sIds[mid] < j) lo = mid + 1;
                else hi = mid;
            }
            skip = lo < nLarge && sIds[lo] == j;
        }
        if (!skip) {
            const uint32_t il = info[l];
            const uint32_t fi = bodySweepFlags(il, sb[l]), fj = bodySweepFlags(ij, sb[j]);
            bool admit = ((fi | fj) & kSweepDynamic) != 0u ||
                         ((fi & kSweepSleeping) && (fj & kSweepMover)) || ((fi & kSweepMover) && (fj & kSweepSleeping));
            if (admit) {
                const float4 mn = aabbMin[l], mx = aabbMax[l], bn = aabbMin[j], bx = aabbMax[j];
                admit = mn.x <= bx.x && mx.x >= bn.x && mn.y <= bx.y && mx.y >= bn.y && mn.z <= bx.z && mx.z >= bn.z;
            }
            if (admit && ((fi | fj) & kSweepFiltered)) admit = filterPass(filt[l], filt[j]);
            hit = admit;
        }
    }
    const uint32_t at = axd::blockReserve(hit ? 1u : 0u, &cnt->pairs);
    if (hit && at < cap) pairs[at] = make_uint2(l < j ? l : j, l < j ? j : l);
}

}  // namespace

void launchMarkLarge(World& w) {
    if (!w.nLarge) return;
    kMarkLarge<<<gridFor(w.nLarge, 64), 64, 0, w.stream>>>(w.nLarge, w.largeIds.p, w.keyA.p);
}

void launchLargePairs(World& w) {
    if (!w.nLarge) return;
    ProfRange pr(w, KG_BROADPHASE_SWEEP);
    w.prof.launches[KG_BROADPHASE_SWEEP] += 1;
    kLargePairs<<<dim3(gridFor(w.n, 256), w.nLarge), 256, 0, w.stream>>>(
        w.n, w.nLarge, w.largeIds.p, w.info.p, w.body.p, w.aabbMin.p, w.aabbMax.p, w.filt.p, w.pairs.p,
        (uint32_t)w.pairs.cap, w.dcnt);
}

void launchBroadphaseGather(World& w, uint32_t nSorted) {
    ProfRange pr(w, KG_BROADPHASE_GATHER);
    w.prof.launches[KG_BROADPHASE_GATHER] += 1;
    cudaMemsetAsync(w.cellTable.p, 0xFF, sizeof(unsigned long long) << w.cellTableLog2, w.stream);
    kGatherCells<<<gridFor(w.n, 256), 256, 0, w.stream>>>(w.n, nSorted, w.keyA.p, w.valA.p,
                                                          w.aabbMin.p, w.aabbMax.p, w.info.p, w.body.p, w.sbox.p,
                                                          w.cellTable.p, w.cellTableLog2, w.dcnt);
}

void launchBroadphase(World& w, const StepParams&, uint32_t nSorted) {
    ProfRange pr(w, KG_BROADPHASE_SWEEP);
    w.prof.launches[KG_BROADPHASE_SWEEP] += 1;
    kSweep<<<gridFor(nSorted, kSweepThreads), kSweepThreads, 0, w.stream>>>(
        nSorted, w.keyA.p, w.sbox.p, w.cellTable.p, w.cellTableLog2, w.filt.p, w.pairs.p,
        (uint32_t)w.pairs.cap, w.dcnt);
}

// The same sweep on caller-provided buffers (sorted keys and AABBs, cell table, output);
// no collision filters (the max corner's .w carries only the dynamic and run bits).
void launchSweepOnBuffers(cudaStream_t s, uint32_t nSorted, const uint32_t* skey, const SortedBox* sbox,
                          const unsigned long long* table, uint32_t log2T,
                          uint2* pairs, uint32_t cap, DevCounters* cnt) {
    kSweep<<<gridFor(nSorted, kSweepThreads), kSweepThreads, 0, s>>>(nSorted, skey, sbox, table,
                                                                      log2T, nullptr, pairs, cap, cnt);
}

}  // namespace axiom_gb300
