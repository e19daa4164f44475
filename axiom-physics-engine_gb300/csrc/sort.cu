// sort.cu — stable LSD radix sort of (uint32 key, uint32 value) pairs, 8-bit digits.
//
// Per pass: (1) each tile of 2048 keys counts its digits in shared memory and writes
// them digit-major to hist[digit * tiles + tile]; (2) one block scans hist exclusively;
// (3) each tile ranks its keys stably and scatters them.  Ranking is warp-major: warp w
// owns 256 consecutive keys of the tile and walks them in chunks of 32 with
// __match_any_sync, so the order inside a tile is (warp, chunk, lane) = input order and
// the sort is stable; a stable sort of distinct-priority keys makes the whole step
// deterministic.
//
// Up to kSmallSort pairs (small worlds) sort in one block instead: a bitonic sort of
// (key << 32 | input position) in shared memory, which is the same stable order, in one
// launch instead of twelve.
#include <algorithm>

#include "world.h"

namespace axiom_gb300 {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItemsPerWarp = 256;          // 8 chunks of 32
constexpr int kTile = kWarps * kItemsPerWarp;  // 2048
constexpr int kChunks = kItemsPerWarp / 32;

__global__ void __launch_bounds__(kThreads) kUpsweep(const uint32_t* __restrict__ keys, uint32_t n,
                                                     uint32_t shift, uint32_t tiles,
                                                     uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kTile;
#pragma unroll
    for (int k = 0; k < kTile / kThreads; ++k) {
        uint32_t i = base + k * kThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Block-wide exclusive scan of one value per thread (kThreads threads); returns the
// exclusive prefix and writes the block total to *total.
__device__ __forceinline__ uint32_t blockExclusiveScan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warpSums[kWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) warpSums[warp] = x;
    __syncthreads();
    uint32_t before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        const uint32_t s = warpSums[w];
        before += w < warp ? s : 0u;
        all += s;
    }
    __syncthreads();
    *total = all;
    return before + x - v;
}

// Row scan: block d turns hist[d * tiles + t] into the exclusive prefix over t and
// writes the row total to hist[256 * tiles + d].  Loads are coalesced along the row.
__global__ void __launch_bounds__(kThreads) kRowScan(uint32_t* __restrict__ hist, uint32_t tiles) {
    uint32_t* row = hist + (size_t)blockIdx.x * tiles;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < tiles; base += kThreads) {
        const uint32_t t = base + threadIdx.x;
        const uint32_t v = t < tiles ? row[t] : 0u;
        uint32_t total;
        const uint32_t ex = blockExclusiveScan(v, &total);
        if (t < tiles) row[t] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) hist[256u * tiles + blockIdx.x] = carry;
}

// kGroup: the colour grouping's pass — the values are the input positions (valsIn is not
// read), the sorted keys are not written, inv[value] receives the sorted position, and
// block 0 writes the colour bounds (colourStart = the digit bases, maxColour = the highest
// non-empty colour + 1).
template <bool kGroup>
__global__ void __launch_bounds__(kThreads) kDownsweep(const uint32_t* __restrict__ keysIn,
                                                       const uint32_t* __restrict__ valsIn,
                                                       uint32_t* __restrict__ keysOut,
                                                       uint32_t* __restrict__ valsOut, uint32_t n,
                                                       uint32_t shift, uint32_t tiles,
                                                       const uint32_t* __restrict__ hist,
                                                       uint32_t* __restrict__ inv, DevCounters* cnt) {
    __shared__ uint32_t wcount[kWarps][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < kWarps * 256; d += kThreads) (&wcount[0][0])[d] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kTile + warp * kItemsPerWarp;
    const unsigned ltmask = (1u << lane) - 1u;
    uint32_t key[kChunks], val[kChunks], local[kChunks];
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
        const uint32_t i = base + c * 32 + lane;
        const bool valid = i < n;
        key[c] = valid ? keysIn[i] : 0u;
        val[c] = kGroup ? i : (valid ? valsIn[i] : 0u);
        const uint32_t d = valid ? ((key[c] >> shift) & 0xFFu) : 0x100u;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank = __popc(peers & ltmask);
        const uint32_t before = valid ? wcount[warp][d] : 0u;
        local[c] = before + rank;
        __syncwarp();
        if (valid && rank == 0) wcount[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        const uint32_t d = threadIdx.x;  // kThreads == 256 digits
        // digit base = exclusive scan of the 256 row totals (recomputed by every tile)
        uint32_t total;
        const uint32_t digitTotal = hist[256u * tiles + d];
        const uint32_t digitBase = blockExclusiveScan(digitTotal, &total);
        if (kGroup && blockIdx.x == 0) {
            if (d <= (uint32_t)kMaxColours + 1u) cnt->colourStart[d] = digitBase;
            if (d < (uint32_t)kMaxColours && digitTotal > 0u) atomicMax(&cnt->maxColour, d + 1u);
        }
        uint32_t run = digitBase + hist[d * tiles + blockIdx.x];
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t c = wcount[w][d];
            wcount[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
        const uint32_t i = base + c * 32 + lane;
        if (i < n) {
            const uint32_t d = (key[c] >> shift) & 0xFFu;
            const uint32_t dst = wcount[warp][d] + local[c];
            if (kGroup) {
                valsOut[dst] = val[c];
                inv[val[c]] = dst;
            } else {
                keysOut[dst] = key[c];
                valsOut[dst] = val[c];
            }
        }
    }
}

// ---- one launch per pass: decoupled look-back ----
//
// The digit totals of all four passes come from one read of the keys (kDigitTotals).  Then
// each pass is one launch (kOnesweep): a CTA takes the next tile by ticket (so a tile's
// predecessors have all started), ranks its keys as kDownsweep does, publishes its digit
// counts, and finds each digit's offset by walking back over the predecessors' published
// words — an inclusive prefix ends the walk, an aggregate adds and walks on — then
// publishes its own inclusive prefix and scatters.  A status word is flag (2 bits) |
// count (30 bits).  Every wait is bounded; a wait that gives up raises kErrSortWait, and
// scatters outside [0, n) are dropped, so a failure costs a wrong order, never a stray
// write.
constexpr uint32_t kFlagAgg = 1u << 30, kFlagInc = 2u << 30, kCountMask = (1u << 30) - 1u;
constexpr uint32_t kSortSpins = 1u << 22;
constexpr uint32_t kErrSortWait = 8u;  // DevCounters::errorFlags: a look-back wait gave up

__global__ void __launch_bounds__(kThreads) kDigitTotals(const uint32_t* __restrict__ keys, uint32_t n,
                                                         uint32_t* __restrict__ totals) {
    __shared__ uint32_t h[4][256];
    for (int p = 0; p < 4; ++p) h[p][threadIdx.x] = 0u;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
#pragma unroll
        for (int p = 0; p < 4; ++p) atomicAdd(&h[p][(k >> (8 * p)) & 0xFFu], 1u);
    }
    __syncthreads();
    for (int p = 0; p < 4; ++p)
        if (h[p][threadIdx.x]) atomicAdd(&totals[p * 256 + threadIdx.x], h[p][threadIdx.x]);
}

__global__ void __launch_bounds__(kThreads) kOnesweep(const uint32_t* __restrict__ keysIn,
                                                      const uint32_t* __restrict__ valsIn,
                                                      uint32_t* __restrict__ keysOut, uint32_t* __restrict__ valsOut,
                                                      uint32_t n, uint32_t shift, const uint32_t* __restrict__ totals,
                                                      uint32_t* __restrict__ status, uint32_t* __restrict__ ticket,
                                                      uint32_t* __restrict__ errorFlags) {
    __shared__ uint32_t wcount[kWarps][256];
    __shared__ uint32_t tileOff[256], start[256];
    __shared__ uint32_t sKey[kTile], sVal[kTile];
    __shared__ uint32_t sTile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) sTile = atomicAdd(ticket, 1u);
    for (int d = threadIdx.x; d < kWarps * 256; d += kThreads) (&wcount[0][0])[d] = 0;
    __syncthreads();
    const uint32_t tile = sTile;
    const uint32_t base = tile * kTile + warp * kItemsPerWarp;
    const unsigned ltmask = (1u << lane) - 1u;
    uint32_t key[kChunks], val[kChunks], local[kChunks];
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
        const uint32_t i = base + c * 32 + lane;
        const bool valid = i < n;
        key[c] = valid ? keysIn[i] : 0u;
        val[c] = valid ? valsIn[i] : 0u;
        const uint32_t d = valid ? ((key[c] >> shift) & 0xFFu) : 0x100u;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank = __popc(peers & ltmask);
        const uint32_t before = valid ? wcount[warp][d] : 0u;
        local[c] = before + rank;
        __syncwarp();
        if (valid && rank == 0) wcount[warp][d] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    bool failed = false;
    {
        const uint32_t d = threadIdx.x;  // kThreads == 256 digits
        uint32_t all;
        const uint32_t digitBase = blockExclusiveScan(totals[d], &all);
        uint32_t count = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {  // per-warp counts -> exclusive prefix over the warps
            const uint32_t c = wcount[w][d];
            wcount[w][d] = count;
            count += c;
        }
        tileOff[d] = blockExclusiveScan(count, &all);  // the tile's keys, digit-major
        volatile uint32_t* st = status;
        uint32_t prefix = 0;
        if (tile == 0) {
            st[d] = kFlagInc | count;
        } else {
            st[(size_t)tile * 256u + d] = kFlagAgg | count;
            for (uint32_t p = tile; p-- > 0;) {
                uint32_t v = 0, spins = 0;
                while (((v = st[(size_t)p * 256u + d]) & (kFlagAgg | kFlagInc)) == 0u && ++spins < kSortSpins) {
                }
                if ((v & (kFlagAgg | kFlagInc)) == 0u) {
                    failed = true;
                    break;
                }
                prefix += v & kCountMask;
                if (v & kFlagInc) break;
            }
            st[(size_t)tile * 256u + d] = kFlagInc | ((prefix + count) & kCountMask);
        }
        start[d] = digitBase + prefix;  // global position of the tile's first key of digit d
    }
    if (__syncthreads_or(failed) && threadIdx.x == 0) atomicOr(errorFlags, kErrSortWait);
    // the tile sorted by digit in shared memory, then written out in runs: consecutive
    // threads write consecutive positions of a digit's run
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
        const uint32_t i = base + c * 32 + lane;
        if (i < n) {
            const uint32_t d = (key[c] >> shift) & 0xFFu;
            const uint32_t at = tileOff[d] + wcount[warp][d] + local[c];
            sKey[at] = key[c];
            sVal[at] = val[c];
        }
    }
    __syncthreads();
    const uint32_t inTile = min((uint32_t)kTile, n - tile * kTile);
    for (uint32_t j = threadIdx.x; j < inTile; j += kThreads) {
        const uint32_t k = sKey[j], d = (k >> shift) & 0xFFu;
        const uint32_t dst = start[d] + (j - tileOff[d]);
        if (dst < n) {
            keysOut[dst] = k;
            valsOut[dst] = sVal[j];
        }
    }
}

constexpr uint32_t kSmallSort = 4096;
constexpr uint32_t kSmallThreads = 1024;

// One block: keys / values [0, n) sorted stably by key, in place.  The composite
// (key << 32 | position) is unique, so any correct sort of it is the stable key order.
__global__ void __launch_bounds__(kSmallThreads) kSortSmall(uint32_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                                            uint32_t n) {
    __shared__ unsigned long long c[kSmallSort];
    __shared__ uint32_t v[kSmallSort];
    uint32_t m = 1;
    while (m < n) m <<= 1;
    if (m <= kSmallThreads) {
        // one composite per thread: partners closer than a warp are exchanged by shuffles,
        // the others through shared memory (two barriers per such stage)
        const uint32_t i = threadIdx.x;
        unsigned long long x = i < n ? ((unsigned long long)keys[i] << 32) | i : ~0ull;
        if (i < n) v[i] = vals[i];
        for (uint32_t k = 2; k <= m; k <<= 1)
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                unsigned long long y;
                if (j >= 32u) {
                    c[i] = x;
                    __syncthreads();
                    y = c[i ^ j];
                    __syncthreads();
                } else {
                    y = __shfl_xor_sync(0xFFFFFFFFu, x, j);
                }
                // the lower index of an ascending pair (or the upper of a descending one) keeps the minimum
                x = (((i & j) == 0u) == ((i & k) == 0u)) ? (x < y ? x : y) : (x < y ? y : x);
            }
        __syncthreads();  // v is complete
        if (i < n) {
            keys[i] = (uint32_t)(x >> 32);
            vals[i] = v[(uint32_t)x];
        }
        return;
    }
    for (uint32_t i = threadIdx.x; i < m; i += kSmallThreads) {
        c[i] = i < n ? ((unsigned long long)keys[i] << 32) | i : ~0ull;
        if (i < n) v[i] = vals[i];
    }
    __syncthreads();
    for (uint32_t k = 2; k <= m; k <<= 1)
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < m; i += kSmallThreads) {
                const uint32_t p = i ^ j;
                if (p > i) {
                    const unsigned long long a = c[i], b = c[p];
                    const bool up = (i & k) == 0u;
                    if ((a > b) == up) {
                        c[i] = b;
                        c[p] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (uint32_t i = threadIdx.x; i < n; i += kSmallThreads) {
        const unsigned long long x = c[i];
        keys[i] = (uint32_t)(x >> 32);
        vals[i] = v[(uint32_t)x];
    }
}

}  // namespace

// Sorts (kA, vA)[0..n) by the `passes` 8-bit digits starting at bit 0, ping-ponging
// through (kB, vB).  Returns true when the sorted result ends in (kA, vA).
bool radixSort(cudaStream_t s, uint32_t* kA, uint32_t* vA, uint32_t* kB, uint32_t* vB,
               uint32_t* hist, uint32_t n, uint32_t passes) {
    if (n == 0) return true;
    if (passes == 4u && n <= kSmallSort) {  // the full 32-bit sort of a small set: one block
        kSortSmall<<<1, kSmallThreads, 0, s>>>(kA, vA, n);
        return true;
    }
    const uint32_t tiles = (n + kTile - 1) / kTile;
    uint32_t *kin = kA, *vin = vA, *kout = kB, *vout = vB;
    for (uint32_t p = 0; p < passes; ++p) {
        const uint32_t shift = 8u * p;
        kUpsweep<<<tiles, kThreads, 0, s>>>(kin, n, shift, tiles, hist);
        kRowScan<<<256, kThreads, 0, s>>>(hist, tiles);
        kDownsweep<false><<<tiles, kThreads, 0, s>>>(kin, vin, kout, vout, n, shift, tiles, hist, nullptr, nullptr);
        uint32_t* t = kin;
        kin = kout;
        kout = t;
        t = vin;
        vin = vout;
        vout = t;
    }
    return (passes % 2u) == 0u;
}

// Groups manifolds by colour: one stable pass over the low 8 bits of colour[0..n) (colours
// are below 64, the crowded batch is 64 and follows them; an uncoloured manifold, only
// after a failed colouring, sorts last), order[s]
// = the manifold at colour-order position s, inv[m] = its position, and the colour bounds
// in cnt (maxColour must start at zero).  Three launches.
void groupByColour(cudaStream_t s, const uint32_t* colour, uint32_t* order, uint32_t* inv, uint32_t* hist,
                   uint32_t n, DevCounters* cnt) {
    if (n == 0) return;
    const uint32_t tiles = (n + kTile - 1) / kTile;
    kUpsweep<<<tiles, kThreads, 0, s>>>(colour, n, 0u, tiles, hist);
    kRowScan<<<256, kThreads, 0, s>>>(hist, tiles);
    kDownsweep<true><<<tiles, kThreads, 0, s>>>(colour, nullptr, nullptr, order, n, 0u, tiles, hist, inv, cnt);
}

// Words of scratch the one-launch-per-pass sort takes: the four passes' digit totals, their
// tickets and their status words (one per digit and tile).
uint32_t onesweepWords(uint32_t n) { return 4u * 256u + 8u + 4u * 256u * ((n + kTile - 1) / kTile); }

// Sorts (kA, vA)[0..n) by all 32 key bits through (kB, vB); the result is back in (kA, vA).
// Up to kSmallSort pairs sort in one block, more in 1 + 4 launches (digit totals, then one
// decoupled-look-back launch per 8-bit digit) after one memset of the scratch.
void radixSortFull(cudaStream_t s, uint32_t* kA, uint32_t* vA, uint32_t* kB, uint32_t* vB, uint32_t* scratch,
                   uint32_t n, uint32_t* errorFlags) {
    if (n == 0) return;
    if (n <= kSmallSort) {
        kSortSmall<<<1, kSmallThreads, 0, s>>>(kA, vA, n);
        return;
    }
    const uint32_t tiles = (n + kTile - 1) / kTile;
    uint32_t* totals = scratch;
    uint32_t* tickets = scratch + 4u * 256u;
    uint32_t* status = tickets + 8u;
    cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * onesweepWords(n), s);
    kDigitTotals<<<std::min<uint32_t>((n + kThreads - 1) / kThreads, 152u * 4u), kThreads, 0, s>>>(kA, n, totals);
    uint32_t *kin = kA, *vin = vA, *kout = kB, *vout = vB;
    for (uint32_t p = 0; p < 4; ++p) {
        kOnesweep<<<tiles, kThreads, 0, s>>>(kin, vin, kout, vout, n, 8u * p, totals + 256u * p,
                                             status + (size_t)256u * tiles * p, tickets + p, errorFlags);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
}

// Sorts w.keyA/w.valA[0..n) by all 32 key bits; the result is back in keyA/valA.
void radixSortPairs(World& w, uint32_t n) {
    ProfRange pr(w, KG_RADIX_SORT);
    w.prof.launches[KG_RADIX_SORT] += n ? (n <= kSmallSort ? 1 : 5) : 0;
    radixSortFull(w.stream, w.keyA.p, w.valA.p, w.keyB.p, w.valB.p, w.hist.p, n, &w.dcnt->errorFlags);
}

uint32_t radixHistWords(uint32_t n) { return std::max(256u * ((n + kTile - 1) / kTile) + 256u, onesweepWords(n)); }

}  // namespace axiom_gb300
