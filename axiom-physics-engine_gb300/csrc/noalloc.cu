// noalloc.cu — broadphase for callers that cannot allocate device memory.
//
// No counterpart in the reference.  Some callers of this library run where a
// cudaMalloc is not allowed: inside an engine whose device memory is carved out of one
// pool up front, in a fixed-rate loop that must not stall on the allocator, or as a
// plugin whose host owns every allocation.  axiom_broadphase_pairs_static serves them:
// it runs the world's broadphase (Morton keys, radix sort, cell table, forward-stencil
// sweep) on caller-owned inputs and outputs, with its scratch in the file-scope device
// array below instead of world-owned buffers.
//
// Limits and sharing (also stated in include/axiom_c.h):
//  - at most kStaticMaxBodies bodies; larger inputs are rejected with
//    AXIOM_INVALID_PARAMETER before any GPU work;
//  - the scratch (about 6 MB) exists on every GPU that loads the library until exit;
//  - all calls on a GPU share it and it keeps the last call's contents: the counters, the
//    widest extent and the cell table are cleared at the start of every call, and calls
//    whose GPU work overlaps race;
//  - the cell table has 2^17 slots, twice the maximum body count, and a cell run takes one
//    slot, so the insertion below always finds a free slot: its probe bound is a guard,
//    not a case the call can meet;
//  - host code cannot use the array's name as a device address; the first call on each
//    device obtains the address with cudaGetSymbolAddress (that device current) and
//    caches it, so that first call belongs before any stream capture.
#include <cstdint>
#include <mutex>

#include "dmath.cuh"
#include "world.h"

namespace axiom_gb300 {
namespace {

constexpr uint32_t kStaticMaxBodies = AXIOM_BROADPHASE_STATIC_MAX_BODIES;
constexpr uint32_t kStaticTableLog2 = 17;
static_assert((1u << kStaticTableLog2) >= 2u * kStaticMaxBodies, "the cell table holds every cell run");
constexpr uint32_t kStaticHistWords = 256u * ((kStaticMaxBodies + 2047u) / 2048u) + 256u;
constexpr int kMaxDevices = 64;

struct StaticScratch {
    float4 amin[kStaticMaxBodies];  // AABB min by body, .w = body id bits
    float4 amax[kStaticMaxBodies];  // AABB max by body, .w = dynamic flag bits
    SortedBox sbox[kStaticMaxBodies];  // the same in sorted order (run flag added)
    unsigned long long table[1u << kStaticTableLog2];
    uint32_t keys0[kStaticMaxBodies], vals0[kStaticMaxBodies];
    uint32_t keys1[kStaticMaxBodies], vals1[kStaticMaxBodies];
    uint32_t hist[kStaticHistWords];
    DevCounters cnt;
    uint32_t maxWidthBits;  // widest AABB extent (non-negative float bits)
};

static __device__ __align__(256) StaticScratch g_staticScratch;

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__device__ __forceinline__ uint32_t cellCoord(float v, float invCell) {
    float c = floorf(v * invCell);
    c = c > 65536.0f ? 65536.0f : c;
    c = c < -65536.0f ? -65536.0f : c;
    c = (c == c) ? c : -65536.0f;
    return (uint32_t)((int32_t)c) & 0x3FFu;
}
__device__ __forceinline__ uint32_t cellHash(uint32_t key, uint32_t log2T) {
    return (key * 2654435761u) >> (32u - log2T);
}

// Copies the caller's AABBs into float4 scratch and takes the widest extent.
__global__ void __launch_bounds__(256) kStaticLoad(uint32_t n, const float* __restrict__ mn3,
                                                   const float* __restrict__ mx3,
                                                   const uint32_t* __restrict__ dynamic,
                                                   StaticScratch* __restrict__ s) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x0 = mn3[3 * i], y0 = mn3[3 * i + 1], z0 = mn3[3 * i + 2];
    const float x1 = mx3[3 * i], y1 = mx3[3 * i + 1], z1 = mx3[3 * i + 2];
    const uint32_t dyn = dynamic ? (dynamic[i] != 0u ? 1u : 0u) : 1u;
    s->amin[i] = make_float4(x0, y0, z0, __uint_as_float(i));
    s->amax[i] = make_float4(x1, y1, z1, __uint_as_float(dyn));
    float wdt = axd::maxf(x1 - x0, axd::maxf(y1 - y0, z1 - z0));
    wdt = wdt > 0.0f ? wdt : 0.0f;  // also drops NaN
    atomicMax(&s->maxWidthBits, __float_as_uint(wdt));
}

__global__ void __launch_bounds__(256) kStaticKeys(uint32_t n, StaticScratch* __restrict__ s) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float maxw = __uint_as_float(s->maxWidthBits);
    const float invCell = 1.0f / (maxw > 0.0f ? maxw * 1.0625f : 1.0f);
    const float4 m = s->amin[i];
    s->keys0[i] = spread10(cellCoord(m.x, invCell)) | (spread10(cellCoord(m.y, invCell)) << 1) |
                  (spread10(cellCoord(m.z, invCell)) << 2);
    s->vals0[i] = i;
}

// Sorted-order AABBs and the first position of every cell run in the table.
__global__ void __launch_bounds__(256) kStaticGather(uint32_t n, StaticScratch* __restrict__ s) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = s->vals0[i];
    const uint32_t key = s->keys0[i];
    float4 mx = s->amax[id];
    if (i + 1u < n && s->keys0[i + 1u] == key) mx.w = __uint_as_float(__float_as_uint(mx.w) | kSweepRunNext);
    s->sbox[i] = SortedBox{s->amin[id], mx};
    if (i > 0 && s->keys0[i - 1] == key) return;
    const uint32_t mask = (1u << kStaticTableLog2) - 1u;
    const unsigned long long entry = ((unsigned long long)key << 32) | i;
    uint32_t h = cellHash(key, kStaticTableLog2);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        if (atomicCAS(&s->table[h], kEmpty64, entry) == kEmpty64) return;
        h = (h + 1u) & mask;
    }
    atomicOr(&s->cnt.errorFlags, 1u);
}

__global__ void kStaticCount(const StaticScratch* __restrict__ s, uint32_t* __restrict__ count) {
    *count = s->cnt.pairs;
}

std::mutex g_symbolMutex;
StaticScratch* g_symbolAddr[kMaxDevices] = {};

// Device address of g_staticScratch on the current device, looked up once per device.
cudaError_t staticScratchAddress(StaticScratch** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_symbolMutex);
    if (!g_symbolAddr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_staticScratch);
        if (e != cudaSuccess) return e;
        g_symbolAddr[dev] = static_cast<StaticScratch*>(p);
    }
    *out = g_symbolAddr[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace axiom_gb300

using namespace axiom_gb300;

extern "C" AXIOM_API int32_t axiom_broadphase_pairs_static(const float* aabb_min, const float* aabb_max,
                                                           const uint32_t* dynamic, uint32_t n,
                                                           uint32_t* pairs, uint32_t capacity,
                                                           uint32_t* count, void* stream) {
    if (!count || (n > 0 && (!aabb_min || !aabb_max)) || (capacity > 0 && !pairs))
        return AXIOM_NULL_POINTER;
    if (n > kStaticMaxBodies) return AXIOM_INVALID_PARAMETER;
    if (reinterpret_cast<uintptr_t>(pairs) % 8u != 0u) return AXIOM_INVALID_PARAMETER;
    StaticScratch* s = nullptr;
    if (staticScratchAddress(&s) != cudaSuccess) return AXIOM_GPU_OPERATION_FAILED;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // clear what must start at zero: counters, widest extent, cell table (each on its own, so
    // that no clear depends on the order of the scratch fields)
    if (cudaMemsetAsync(&s->cnt, 0, sizeof(DevCounters), st) != cudaSuccess ||
        cudaMemsetAsync(&s->maxWidthBits, 0, sizeof(uint32_t), st) != cudaSuccess ||
        cudaMemsetAsync(s->table, 0xFF, sizeof(s->table), st) != cudaSuccess)
        return AXIOM_GPU_OPERATION_FAILED;
    if (n > 0) {
        const unsigned grid = gridFor(n, 256);
        kStaticLoad<<<grid, 256, 0, st>>>(n, aabb_min, aabb_max, dynamic, s);
        kStaticKeys<<<grid, 256, 0, st>>>(n, s);
        radixSort(st, s->keys0, s->vals0, s->keys1, s->vals1, s->hist, n, 4);  // ends in keys0/vals0
        kStaticGather<<<grid, 256, 0, st>>>(n, s);
        launchSweepOnBuffers(st, n, s->keys0, s->sbox, s->table, kStaticTableLog2,
                             reinterpret_cast<uint2*>(pairs), capacity, &s->cnt);
    }
    kStaticCount<<<1, 1, 0, st>>>(s, count);
    return cudaGetLastError() == cudaSuccess ? AXIOM_SUCCESS : AXIOM_GPU_OPERATION_FAILED;
}
