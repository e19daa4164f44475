// mlp.cu — the learned PGS warm start: a 14 -> 128 -> 128 -> 128 -> 3 SiLU network,
// inference and training on the GPU with hand-written tcgen05 GEMMs (BF16 operands,
// FP32 accumulation in tensor memory).
//
// The reference has no learned component; this network only changes where PGS starts.
// The solver still iterates to the same residual threshold, so the accepted answer is
// the plain solver's.
//
// Layers 1-3 run through kGemm (C = A * B^T, M tiles of 128 rows, N = 16 or 128):
//   forward   Z_l = H_{l-1} W_l^T + b_l, H_l = SiLU(Z_l)            (EPI_SILU)
//   backward  dZ_l = (dZ_{l+1} W_{l+1}) * SiLU'(Z_l)                (EPI_DSILU, W^T copies)
//             dW_l += dZ_l^T H_{l-1}, split over the batch          (EPI_PARTIAL)
// Layer 4 (3 outputs), the loss and the first backward step are one CUDA-core kernel
// (kHead); bias gradients are column sums; Adam updates the fp32 master weights and
// refreshes the BF16 copies.  Every gradient is a sum in a fixed order (split partials and
// head-block partials are stored, then added up by one thread per element), so a seed and
// a data set give the same weights on every run.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/axiom_c.h"
#include "mlp.h"
#include "tcgen05.cuh"
#include "world.h"

namespace axiom_gb300 {
namespace {

using bf16 = __nv_bfloat16;

constexpr uint32_t kGemmThreads = 128;
constexpr uint32_t kKChunk = 64;
constexpr uint32_t kWaitSpins = 1u << 24;

enum Epi : uint32_t { EPI_SILU = 1, EPI_DSILU = 2, EPI_PARTIAL = 3 };

struct GemmArgs {
    const bf16* A;  // [M][K]
    const bf16* B;  // [N][K]
    uint32_t M, N, K;
    uint32_t kPerSplit;  // K handled by one blockIdx.z
    const float* bias;   // EPI_SILU: [N]
    float* C;            // EPI_PARTIAL: [splits][M][N], this split's [M][N] stored
    bf16* H;             // EPI_SILU: SiLU(z); EPI_DSILU: dz  -- [M][N]
    bf16* HT;            // the same transposed [N][M] (optional)
    float* Z;            // EPI_SILU: z [M][N] (optional)
    const float* Zin;    // EPI_DSILU: saved z [M][N]
    uint32_t* error;     // set on a timed-out wait
};

__device__ __forceinline__ float sigmoidf(float z) { return 1.0f / (1.0f + expf(-z)); }

template <uint32_t EPI, uint32_t BN>
__global__ void __launch_bounds__(kGemmThreads) kGemm(GemmArgs g) {
    __shared__ __align__(1024) uint8_t sA[128 * kKChunk * 2];
    __shared__ __align__(1024) uint8_t sB[BN * kKChunk * 2];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmemBase;
    __shared__ uint32_t failed;
    constexpr uint32_t kCols = BN < 32 ? 32 : BN;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t m0 = blockIdx.x * 128u, n0 = blockIdx.y * BN;
    const uint32_t kBeg = blockIdx.z * g.kPerSplit;
    const uint32_t kEnd = min(g.K, kBeg + g.kPerSplit);
    if (warp == 0) tc::tmemAlloc(&tmemBase, kCols);
    if (tid == 0) {
        tc::mbarInit(&mbar, 1);
        failed = 0;
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tmem = tmemBase;
    constexpr uint32_t idesc = tc::idescBf16F32(128, BN);
    uint32_t phase = 0;
    bool first = true;
    for (uint32_t k0 = kBeg; k0 < kEnd; k0 += kKChunk) {
        const uint32_t kc = min(kKChunk, kEnd - k0);  // multiple of 16
        const uint32_t pieces = kc >> 3;              // 16-byte pieces per row
        for (uint32_t p = tid; p < 128u * pieces; p += kGemmThreads) {
            const uint32_t r = p / pieces, c = p % pieces;
            const uint4 v = *reinterpret_cast<const uint4*>(g.A + (size_t)(m0 + r) * g.K + k0 + 8u * c);
            *reinterpret_cast<uint4*>(sA + tc::coreOffset(r, 8u * c)) = v;
        }
        for (uint32_t p = tid; p < BN * pieces; p += kGemmThreads) {
            const uint32_t r = p / pieces, c = p % pieces;
            const uint4 v = *reinterpret_cast<const uint4*>(g.B + (size_t)(n0 + r) * g.K + k0 + 8u * c);
            *reinterpret_cast<uint4*>(sB + tc::coreOffset(r, 8u * c)) = v;
        }
        tc::fenceProxyAsync();
        __syncthreads();
        if (tid == 0) {
            tc::fenceAfterSync();
            const uint32_t a = tc::smemAddr(sA), b = tc::smemAddr(sB);
            for (uint32_t j = 0; j < kc / 16u; ++j) {
                const uint64_t ad = tc::smemDesc(a + 256u * j, 128u, 1024u);
                const uint64_t bd = tc::smemDesc(b + 256u * j, 128u, 1024u);
                tc::mmaBf16(tmem, ad, bd, idesc, (first && j == 0) ? 0u : 1u);
            }
            tc::commit(&mbar);
        }
        first = false;
        // every thread waits before the shared tiles are overwritten
        if (!tc::mbarWait(&mbar, phase, kWaitSpins)) failed = 1;
        phase ^= 1u;
        __syncthreads();
        if (failed) break;
    }
    tc::fenceAfterSync();
    if (!failed && !first) {
        const uint32_t row = m0 + warp * 32u + lane;
        for (uint32_t c16 = 0; c16 < BN / 16u; ++c16) {
            float v[16];
            tc::tmemLoad16(tmem + ((warp * 32u) << 16) + c16 * 16u, v);
#pragma unroll
            for (uint32_t j = 0; j < 16; ++j) {
                const uint32_t col = n0 + c16 * 16u + j;
                const size_t idx = (size_t)row * g.N + col;
                if (EPI == EPI_PARTIAL) {
                    g.C[(size_t)blockIdx.z * g.M * g.N + idx] = v[j];
                } else if (EPI == EPI_SILU) {
                    const float z = v[j] + g.bias[col];
                    if (g.Z) g.Z[idx] = z;
                    const bf16 h = __float2bfloat16_rn(z * sigmoidf(z));
                    g.H[idx] = h;
                    if (g.HT) g.HT[(size_t)col * g.M + row] = h;
                } else {
                    const float z = g.Zin[idx];
                    const float s = sigmoidf(z);
                    const bf16 dz = __float2bfloat16_rn(v[j] * (s * (1.0f + z * (1.0f - s))));
                    g.H[idx] = dz;
                    if (g.HT) g.HT[(size_t)col * g.M + row] = dz;
                }
            }
        }
    }
    if (failed && tid == 0) atomicOr(g.error, 1u);
    tc::fenceBeforeSync();
    __syncthreads();
    if (warp == 0) tc::tmemDealloc(tmem, kCols);
}

// Features fp32 (first 14 of each row of `stride` floats; row r of X is feature row
// gather[r], or r without a gather list) -> X bf16 [Mpad][16] and X^T [16][Mpad]; padded
// rows and the two padding columns are zero.
__global__ void kPackFeatures(const float* __restrict__ f, uint32_t stride, uint32_t n, uint32_t mpad,
                              const uint32_t* __restrict__ gather, bf16* __restrict__ X, bf16* __restrict__ XT) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= mpad) return;
    const bool ok = r < n;
    const size_t src = ok ? (size_t)(gather ? gather[r] : r) : 0u;
    for (uint32_t j = 0; j < 16; ++j) {
        const float v = (ok && j < kMlpInputs) ? f[src * stride + j] : 0.0f;
        const bf16 b = __float2bfloat16_rn(v);
        X[(size_t)r * 16 + j] = b;
        if (XT) XT[(size_t)j * mpad + r] = b;
    }
}

// Layer 4 (+ loss and its backward when targets are given): one thread per row, block
// of 128 rows (mpad is a multiple of 128, so every thread has a row).  dW4 / db4 / loss
// are reduced over each warp with shuffles, then over the block in shared memory, and the
// block's sums are stored in its partial row (kReduceHead adds the rows up).
__global__ void __launch_bounds__(128) kHead(const bf16* __restrict__ H3, const float* __restrict__ Z3,
                                             const float* __restrict__ W4, const float* __restrict__ b4,
                                             uint32_t n, uint32_t mpad, const float* __restrict__ targets,
                                             float* __restrict__ Y, float* __restrict__ part,
                                             bf16* __restrict__ dZ3, bf16* __restrict__ dZ3T, float invCount) {
    __shared__ float sW4[3 * 128];
    __shared__ float sgW4[4][3 * 128];
    __shared__ float sgb4[4][4];
    for (uint32_t i = threadIdx.x; i < 384; i += blockDim.x) sW4[i] = W4[i];
    __syncthreads();
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = r < n;
    float y[3] = {b4[0], b4[1], b4[2]};
    for (uint32_t j = 0; j < 128; ++j) {
        const float h = __bfloat162float(H3[(size_t)r * 128 + j]);
        y[0] = y[0] + sW4[j] * h;
        y[1] = y[1] + sW4[128 + j] * h;
        y[2] = y[2] + sW4[256 + j] * h;
    }
    if (Y && live) {
        Y[(size_t)r * 3] = y[0];
        Y[(size_t)r * 3 + 1] = y[1];
        Y[(size_t)r * 3 + 2] = y[2];
    }
    if (!targets) return;
    float dy[3] = {0.0f, 0.0f, 0.0f};
    float l = 0.0f;
    if (live) {
        for (int o = 0; o < 3; ++o) {
            const float d = y[o] - targets[(size_t)r * 3 + o];
            l = l + d * d;
            dy[o] = 2.0f * d * invCount;
        }
    }
    for (uint32_t j = 0; j < 128; ++j) {
        const float h = __bfloat162float(H3[(size_t)r * 128 + j]);
        float g0 = dy[0] * h, g1 = dy[1] * h, g2 = dy[2] * h;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            g0 += __shfl_xor_sync(0xFFFFFFFFu, g0, off);
            g1 += __shfl_xor_sync(0xFFFFFFFFu, g1, off);
            g2 += __shfl_xor_sync(0xFFFFFFFFu, g2, off);
        }
        if (lane == 0) {
            sgW4[warp][j] = g0;
            sgW4[warp][128 + j] = g1;
            sgW4[warp][256 + j] = g2;
        }
        const float dh = sW4[j] * dy[0] + sW4[128 + j] * dy[1] + sW4[256 + j] * dy[2];
        const float z = Z3[(size_t)r * 128 + j];
        const float s = sigmoidf(z);
        const bf16 dz = __float2bfloat16_rn(dh * (s * (1.0f + z * (1.0f - s))));
        dZ3[(size_t)r * 128 + j] = dz;
        dZ3T[(size_t)j * mpad + r] = dz;
    }
    float b0 = dy[0], b1 = dy[1], b2 = dy[2];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        b0 += __shfl_xor_sync(0xFFFFFFFFu, b0, off);
        b1 += __shfl_xor_sync(0xFFFFFFFFu, b1, off);
        b2 += __shfl_xor_sync(0xFFFFFFFFu, b2, off);
        l += __shfl_xor_sync(0xFFFFFFFFu, l, off);
    }
    if (lane == 0) {
        sgb4[warp][0] = b0;
        sgb4[warp][1] = b1;
        sgb4[warp][2] = b2;
        sgb4[warp][3] = l;
    }
    __syncthreads();
    float* out = part + (size_t)blockIdx.x * kHeadPartials;
    for (uint32_t i = threadIdx.x; i < 384; i += blockDim.x)
        out[i] = ((sgW4[0][i] + sgW4[1][i]) + sgW4[2][i]) + sgW4[3][i];
    if (threadIdx.x < 4)
        out[384 + threadIdx.x] =
            ((sgb4[0][threadIdx.x] + sgb4[1][threadIdx.x]) + sgb4[2][threadIdx.x]) + sgb4[3][threadIdx.x];
}

// Head partials of `blocks` blocks added in block order: dW4 and db4 into the gradients,
// the loss (times invCount) into the loss accumulator.
__global__ void kReduceHead(const float* __restrict__ part, uint32_t blocks, float* __restrict__ gW4,
                            float* __restrict__ gb4, float* __restrict__ loss, float invCount) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kHeadPartials) return;
    float s = 0.0f;
    for (uint32_t b = 0; b < blocks; ++b) s += part[(size_t)b * kHeadPartials + i];
    if (i < 384) gW4[i] += s;
    else if (i < 387) gb4[i - 384] += s;
    else *loss += s * invCount;
}

// Split partials [splits][count] added in split order into out[count].
__global__ void kReduceSplits(const float* __restrict__ part, uint32_t splits, uint32_t count,
                              float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float s = 0.0f;
    for (uint32_t z = 0; z < splits; ++z) s += part[(size_t)z * count + i];
    out[i] += s;
}

// Bias gradient: out[j] += sum over rows of dZ^T[j][:] (one warp per column j).
__global__ void kColumnSums(const bf16* __restrict__ dZT, uint32_t cols, uint32_t mpad, float* __restrict__ out) {
    const uint32_t j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint32_t lane = threadIdx.x & 31;
    if (j >= cols) return;
    float s = 0.0f;
    for (uint32_t r = lane; r < mpad; r += 32) s += __bfloat162float(dZT[(size_t)j * mpad + r]);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, off);
    if (lane == 0) out[j] += s;
}

// BF16 copies of the master weights: W1 [128][16], W2, W3 [128][128], and W2^T, W3^T.
__global__ void kRefreshBf16(const float* __restrict__ p, bf16* __restrict__ w1, bf16* __restrict__ w2,
                             bf16* __restrict__ w3, bf16* __restrict__ w2t, bf16* __restrict__ w3t) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 128 * 16) w1[i] = __float2bfloat16_rn(p[kOffW1 + i]);
    if (i < 128 * 128) {
        const uint32_t o = i / 128, in = i % 128;
        const bf16 a = __float2bfloat16_rn(p[kOffW2 + i]);
        const bf16 b = __float2bfloat16_rn(p[kOffW3 + i]);
        w2[i] = a;
        w3[i] = b;
        w2t[in * 128 + o] = a;
        w3t[in * 128 + o] = b;
    }
}

__global__ void kAdam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                      const float* __restrict__ g, uint32_t n, float lr, float b1, float b2, float eps,
                      float c1, float c2) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// ---- fused inference: the whole network for 128-row tiles, hidden layers on chip ----
//
// Shared memory holds W1 (128 x 16), W2 and W3 (128 x 128) in the K-major canonical layout
// for the whole launch, and per tile the X tile (128 x 16) and one hidden tile H
// (128 x 128, the A operand of the next layer).  Per tile: X -> MMA (K = 16) -> TMEM ->
// bias + SiLU -> H (bf16) -> 8 MMAs (K = 128) -> ... -> the third hidden layer stays in
// registers for the 3-output head.  The MMA sequence (one K = 16 step per instruction, in K
// order), the epilogue expressions and the head's summation order are those of the
// unfused kGemm / kHead path, so the outputs are the same bits; the hidden layers never
// reach global memory.  Persistent: each CTA loads the weights once and loops over tiles.
constexpr uint32_t kInferThreads = 128;
constexpr uint32_t kSmemW1 = 128u * 16u * 2u, kSmemW = 128u * 128u * 2u, kSmemX = 128u * 16u * 2u;
constexpr uint32_t kInferSmem = kSmemW1 + 2u * kSmemW + kSmemX + kSmemW + (3u * 128u + 3u * 128u + 3u) * 4u;

// Byte offset of (row, k) in a K-major canonical tile whose rows hold `kw` K-elements.
__device__ __forceinline__ uint32_t canonOffset(uint32_t row, uint32_t k, uint32_t kw) {
    return (((row >> 3) * (kw >> 3) + (k >> 3)) * 128u) + ((row & 7u) * 16u) + ((k & 7u) * 2u);
}

// Copies a row-major bf16 [rows][kw] matrix into the canonical layout (16-byte pieces).
__device__ __forceinline__ void stageCanon(uint8_t* dst, const bf16* __restrict__ src, uint32_t rows, uint32_t kw) {
    const uint32_t pieces = kw >> 3;
    for (uint32_t p = threadIdx.x; p < rows * pieces; p += blockDim.x) {
        const uint32_t r = p / pieces, c = p % pieces;
        *reinterpret_cast<uint4*>(dst + canonOffset(r, 8u * c, kw)) =
            *reinterpret_cast<const uint4*>(src + (size_t)r * kw + 8u * c);
    }
}

// Waits for the tile's MMAs (bounded); false when the wait gave up.
__device__ __forceinline__ bool waitMma(uint64_t* mbar, uint32_t& phase) {
    const bool ok = tc::mbarWait(mbar, phase, kWaitSpins);
    phase ^= 1u;
    return ok;
}

// One layer's epilogue for this warp's 32 rows: z = acc + bias, h = bf16(z * sigmoid(z)),
// written to the H tile.
__device__ __forceinline__ void epilogueToSmem(uint32_t tmem, uint32_t warp, uint32_t lane, const float* bias,
                                               uint8_t* H) {
    const uint32_t row = warp * 32u + lane;
    for (uint32_t c16 = 0; c16 < 8u; ++c16) {
        float v[16];
        tc::tmemLoad16(tmem + ((warp * 32u) << 16) + c16 * 16u, v);
        __align__(16) bf16 hv[16];
#pragma unroll
        for (uint32_t j = 0; j < 16; ++j) {
            const float z = v[j] + bias[c16 * 16u + j];
            hv[j] = __float2bfloat16_rn(z * sigmoidf(z));
        }
        *reinterpret_cast<uint4*>(H + canonOffset(row, c16 * 16u, 128u)) = *reinterpret_cast<const uint4*>(&hv[0]);
        *reinterpret_cast<uint4*>(H + canonOffset(row, c16 * 16u + 8u, 128u)) =
            *reinterpret_cast<const uint4*>(&hv[8]);
    }
}

__global__ void __launch_bounds__(kInferThreads) kMlpInfer(const float* __restrict__ feat, uint32_t stride,
                                                           const uint32_t* __restrict__ gather, uint32_t n,
                                                           const bf16* __restrict__ w1, const bf16* __restrict__ w2,
                                                           const bf16* __restrict__ w3,
                                                           const float* __restrict__ params, float* __restrict__ Y,
                                                           uint32_t* error) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sW1 = smem;
    uint8_t* sW2 = sW1 + kSmemW1;
    uint8_t* sW3 = sW2 + kSmemW;
    uint8_t* sX = sW3 + kSmemW;
    uint8_t* sH = sX + kSmemX;
    float* sB = reinterpret_cast<float*>(sH + kSmemW);  // b1, b2, b3 [3][128]
    float* sW4 = sB + 3u * 128u;                        // [3][128]
    float* sB4 = sW4 + 3u * 128u;                       // [3]
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmemBase;
    __shared__ uint32_t failed;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    if (warp == 0) tc::tmemAlloc(&tmemBase, 128);
    if (tid == 0) {
        tc::mbarInit(&mbar, 1);
        failed = 0;
    }
    stageCanon(sW1, w1, 128u, 16u);
    stageCanon(sW2, w2, 128u, 128u);
    stageCanon(sW3, w3, 128u, 128u);
    for (uint32_t i = tid; i < 128u; i += kInferThreads) {
        sB[i] = params[kOffB1 + i];
        sB[128u + i] = params[kOffB2 + i];
        sB[256u + i] = params[kOffB3 + i];
    }
    for (uint32_t i = tid; i < 384u; i += kInferThreads) sW4[i] = params[kOffW4 + i];
    if (tid < 3u) sB4[tid] = params[kOffB4 + tid];
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tmem = tmemBase;
    constexpr uint32_t idesc = tc::idescBf16F32(128, 128);
    uint32_t phase = 0;
    const uint32_t tiles = (n + 127u) / 128u;
    for (uint32_t t = blockIdx.x; t < tiles && !failed; t += gridDim.x) {
        const uint32_t row = t * 128u + tid;  // this thread's row of the X tile
        {
            __align__(16) bf16 xv[16];
            const bool live = row < n;
            const size_t src = live ? (size_t)(gather ? gather[row] : row) : 0u;
#pragma unroll
            for (uint32_t j = 0; j < 16; ++j)
                xv[j] = __float2bfloat16_rn((live && j < kMlpInputs) ? feat[src * stride + j] : 0.0f);
            *reinterpret_cast<uint4*>(sX + canonOffset(tid, 0u, 16u)) = *reinterpret_cast<const uint4*>(&xv[0]);
            *reinterpret_cast<uint4*>(sX + canonOffset(tid, 8u, 16u)) = *reinterpret_cast<const uint4*>(&xv[8]);
        }
        const uint8_t* As[3] = {sX, sH, sH};
        const uint8_t* Bs[3] = {sW1, sW2, sW3};
        const uint32_t kw[3] = {16u, 128u, 128u};
        float y[3] = {sB4[0], sB4[1], sB4[2]};
        for (uint32_t l = 0; l < 3u; ++l) {
            // the operand tile is written, and every warp's TMEM reads of the last layer done
            tc::fenceProxyAsync();
            tc::fenceBeforeSync();
            __syncthreads();
            if (tid == 0) {
                tc::fenceAfterSync();
                const uint32_t a = tc::smemAddr(As[l]), b = tc::smemAddr(Bs[l]);
                const uint32_t sbo = kw[l] * 16u;  // 8 rows x kw/8 core matrices x 128 B
                for (uint32_t j = 0; j < kw[l] / 16u; ++j)
                    tc::mmaBf16(tmem, tc::smemDesc(a + 256u * j, 128u, sbo), tc::smemDesc(b + 256u * j, 128u, sbo),
                                idesc, j == 0 ? 0u : 1u);
                tc::commit(&mbar);
            }
            if (!waitMma(&mbar, phase)) failed = 1;
            __syncthreads();
            if (failed) break;
            tc::fenceAfterSync();
            if (l < 2u) {
                epilogueToSmem(tmem, warp, lane, sB + 128u * l, sH);
            } else {
                // third layer: SiLU in registers, then the head in column order
                for (uint32_t c16 = 0; c16 < 8u; ++c16) {
                    float v[16];
                    tc::tmemLoad16(tmem + ((warp * 32u) << 16) + c16 * 16u, v);
#pragma unroll
                    for (uint32_t j = 0; j < 16; ++j) {
                        const uint32_t col = c16 * 16u + j;
                        const float z = v[j] + sB[256u + col];
                        const float h = __bfloat162float(__float2bfloat16_rn(z * sigmoidf(z)));
                        y[0] = y[0] + sW4[col] * h;
                        y[1] = y[1] + sW4[128u + col] * h;
                        y[2] = y[2] + sW4[256u + col] * h;
                    }
                }
            }
        }
        if (failed) break;
        const uint32_t orow = t * 128u + warp * 32u + lane;
        if (orow < n) {
            Y[(size_t)orow * 3] = y[0];
            Y[(size_t)orow * 3 + 1] = y[1];
            Y[(size_t)orow * 3 + 2] = y[2];
        }
    }
    if (failed && tid == 0) atomicOr(error, 1u);
    tc::fenceBeforeSync();
    __syncthreads();
    if (warp == 0) tc::tmemDealloc(tmem, 128);
}

template <uint32_t EPI, uint32_t BN>
void launchGemm(const GemmArgs& g, uint32_t splits, cudaStream_t s) {
    dim3 grid(g.M / 128u, g.N / BN, splits);
    kGemm<EPI, BN><<<grid, kGemmThreads, 0, s>>>(g);
}

}  // namespace

// ---------------------------------------------------------------- MlpState ----

cudaError_t MlpState::reserveRows(uint32_t rows) {
    const uint32_t mpad = (rows + 127u) & ~127u;
    if (mpad <= cap) return cudaSuccess;
    uint32_t want = cap ? cap : 1024u;
    while (want < mpad) want *= 2;
    release(false);
    cap = want;
    const size_t r = want;
    cudaError_t e = cudaSuccess;
    auto al = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    al((void**)&X, r * 16 * 2);
    al((void**)&XT, r * 16 * 2);
    for (int l = 0; l < 3; ++l) {
        al((void**)&Z[l], r * 128 * 4);
        al((void**)&H[l], r * 128 * 2);
        al((void**)&HT[l], r * 128 * 2);
        al((void**)&dZ[l], r * 128 * 2);
        al((void**)&dZT[l], r * 128 * 2);
    }
    al((void**)&Y, r * 3 * 4);
    al((void**)&T, r * 3 * 4);
    al((void**)&F, r * 16 * 4);
    al((void**)&part, ((r + kMlpSplitRows - 1) / kMlpSplitRows) * 128 * 128 * 4);
    al((void**)&headPart, (r / 128) * kHeadPartials * 4);
    return e;
}

cudaError_t MlpState::init() {
    cudaError_t e = cudaSuccess;
    auto al = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    al((void**)&params, kMlpParams * 4);
    al((void**)&grads, kMlpParams * 4);
    al((void**)&adamM, kMlpParams * 4);
    al((void**)&adamV, kMlpParams * 4);
    al((void**)&w1, 128 * 16 * 2);
    al((void**)&w2, 128 * 128 * 2);
    al((void**)&w3, 128 * 128 * 2);
    al((void**)&w2t, 128 * 128 * 2);
    al((void**)&w3t, 128 * 128 * 2);
    al((void**)&scratch, 64 * 4);
    if (e == cudaSuccess) e = cudaMemset(adamM, 0, kMlpParams * 4);
    if (e == cudaSuccess) e = cudaMemset(adamV, 0, kMlpParams * 4);
    if (e == cudaSuccess) e = cudaMemset(scratch, 0, 64 * 4);
    return e;
}

void MlpState::release(bool all) {
    auto fr = [](void* p) {
        if (p) cudaFree(p);
    };
    fr(X);
    fr(XT);
    for (int l = 0; l < 3; ++l) {
        fr(Z[l]);
        fr(H[l]);
        fr(HT[l]);
        fr(dZ[l]);
        fr(dZT[l]);
        Z[l] = nullptr;
        H[l] = HT[l] = dZ[l] = dZT[l] = nullptr;
    }
    fr(Y);
    fr(T);
    fr(F);
    fr(part);
    fr(headPart);
    X = XT = nullptr;
    Y = T = F = nullptr;
    part = headPart = nullptr;
    cap = 0;
    if (all) {
        fr(params);
        fr(grads);
        fr(adamM);
        fr(adamV);
        fr(w1);
        fr(w2);
        fr(w3);
        fr(w2t);
        fr(w3t);
        fr(scratch);
        params = grads = adamM = adamV = nullptr;
        w1 = w2 = w3 = w2t = w3t = nullptr;
        scratch = nullptr;
    }
}

cudaError_t MlpState::setParams(const float* host, cudaStream_t s) {
    cudaError_t e = cudaMemcpyAsync(params, host, kMlpParams * 4, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    refresh(s);
    return cudaGetLastError();
}

void MlpState::refresh(cudaStream_t s) { kRefreshBf16<<<128, 128, 0, s>>>(params, w1, w2, w3, w2t, w3t); }

// Forward over rows already packed in X (mpad rows); training keeps Z/H/HT for backward.
void MlpState::forward(uint32_t mpad, bool training, cudaStream_t s) {
    GemmArgs g{};
    g.M = mpad;
    g.N = 128;
    g.error = reinterpret_cast<uint32_t*>(scratch + 1);
    // layer 1: K = 16
    g.A = X;
    g.B = w1;
    g.K = 16;
    g.kPerSplit = 16;
    g.bias = params + kOffB1;
    g.H = H[0];
    g.HT = training ? HT[0] : nullptr;
    g.Z = training ? Z[0] : nullptr;
    launchGemm<EPI_SILU, 128>(g, 1, s);
    // layers 2, 3: K = 128
    g.K = 128;
    g.kPerSplit = 128;
    g.A = H[0];
    g.B = w2;
    g.bias = params + kOffB2;
    g.H = H[1];
    g.HT = training ? HT[1] : nullptr;
    g.Z = training ? Z[1] : nullptr;
    launchGemm<EPI_SILU, 128>(g, 1, s);
    g.A = H[1];
    g.B = w3;
    g.bias = params + kOffB3;
    g.H = H[2];
    g.HT = nullptr;
    g.Z = Z[2];
    launchGemm<EPI_SILU, 128>(g, 1, s);
}

void MlpState::infer(const float* f, uint32_t stride, const uint32_t* gather, uint32_t n, cudaStream_t s) {
    if (n == 0) return;
    if (!inferGrid) {  // on this state's device: the shared-memory opt-in and one resident wave
        int dev = 0, sms = 0, perSm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(kMlpInfer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem);
        // all of the unified L1 as shared memory: two CTAs (each 128 TMEM columns of 512) per
        // SM, so one CTA's epilogue overlaps the other's MMAs and gathers
        cudaFuncSetAttribute(kMlpInfer, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kMlpInfer, kInferThreads, kInferSmem);
        inferGrid = (uint32_t)std::max(1, sms * std::max(1, perSm));
    }
    const uint32_t tiles = (n + 127u) / 128u;
    kMlpInfer<<<std::min<uint32_t>(tiles, inferGrid), kInferThreads, kInferSmem, s>>>(
        f, stride, gather, n, w1, w2, w3, params, Y, reinterpret_cast<uint32_t*>(scratch + 1));
}

void MlpState::head(uint32_t n, uint32_t mpad, const float* targets, cudaStream_t s) {
    const float invCount = n ? 1.0f / (3.0f * (float)n) : 0.0f;
    const uint32_t blocks = gridFor(mpad, 128);
    kHead<<<blocks, 128, 0, s>>>(H[2], Z[2], params + kOffW4, params + kOffB4, n, mpad, targets, Y, headPart,
                                 dZ[2], dZT[2], invCount);
    if (targets)
        kReduceHead<<<gridFor(kHeadPartials, 128), 128, 0, s>>>(headPart, blocks, grads + kOffW4, grads + kOffB4,
                                                                 scratch, invCount);
}

// Gradients of the mean squared error over n rows of X / targets (accumulated into grads).
void MlpState::backward(uint32_t n, uint32_t mpad, const float* targets, cudaStream_t s) {
    head(n, mpad, targets, s);
    const uint32_t splitRows = kMlpSplitRows;
    const uint32_t splits = (mpad + splitRows - 1) / splitRows;
    // dW3 = dZ3^T H2, db3
    GemmArgs g{};
    g.error = reinterpret_cast<uint32_t*>(scratch + 1);
    g.M = 128;
    g.N = 128;
    g.K = mpad;
    g.kPerSplit = splitRows;
    g.A = dZT[2];
    g.B = HT[1];
    g.C = part;
    launchGemm<EPI_PARTIAL, 128>(g, splits, s);
    kReduceSplits<<<gridFor(128 * 128, 256), 256, 0, s>>>(part, splits, 128 * 128, grads + kOffW3);
    kColumnSums<<<16, 256, 0, s>>>(dZT[2], 128, mpad, grads + kOffB3);
    // dZ2 = (dZ3 W3) * SiLU'(Z2)
    GemmArgs d{};
    d.error = reinterpret_cast<uint32_t*>(scratch + 1);
    d.M = mpad;
    d.N = 128;
    d.K = 128;
    d.kPerSplit = 128;
    d.A = dZ[2];
    d.B = w3t;
    d.Zin = Z[1];
    d.H = dZ[1];
    d.HT = dZT[1];
    launchGemm<EPI_DSILU, 128>(d, 1, s);
    g.A = dZT[1];
    g.B = HT[0];
    g.C = part;
    launchGemm<EPI_PARTIAL, 128>(g, splits, s);
    kReduceSplits<<<gridFor(128 * 128, 256), 256, 0, s>>>(part, splits, 128 * 128, grads + kOffW2);
    kColumnSums<<<16, 256, 0, s>>>(dZT[1], 128, mpad, grads + kOffB2);
    // dZ1 = (dZ2 W2) * SiLU'(Z1)
    d.A = dZ[1];
    d.B = w2t;
    d.Zin = Z[0];
    d.H = dZ[0];
    d.HT = dZT[0];
    launchGemm<EPI_DSILU, 128>(d, 1, s);
    // dW1 = dZ1^T X  (N = 16)
    g.N = 16;
    g.A = dZT[0];
    g.B = XT;
    g.C = part;
    launchGemm<EPI_PARTIAL, 16>(g, splits, s);
    kReduceSplits<<<gridFor(128 * 16, 256), 256, 0, s>>>(part, splits, 128 * 16, grads + kOffW1);
    kColumnSums<<<16, 256, 0, s>>>(dZT[0], 128, mpad, grads + kOffB1);
}

void MlpState::adam(float lr, cudaStream_t s) {
    ++adamStep;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)adamStep), c2 = 1.0f - powf(b2, (float)adamStep);
    kAdam<<<gridFor(kMlpParams, 256), 256, 0, s>>>(params, adamM, adamV, grads, kMlpParams, lr, b1, b2, 1e-8f, c1, c2);
    refresh(s);
}

void MlpState::pack(const float* f, uint32_t stride, uint32_t n, const uint32_t* gather, bool transposed,
                    cudaStream_t s) {
    const uint32_t mpad = (n + 127u) & ~127u;
    kPackFeatures<<<gridFor(mpad, 256), 256, 0, s>>>(f, stride, n, mpad, gather, X, transposed ? XT : nullptr);
}

}  // namespace axiom_gb300

// ------------------------------------------------------------------- C ABI ----

using namespace axiom_gb300;

namespace {
struct MlpHandle {
    MlpState st;
    cudaStream_t stream = nullptr;
};

#define MLP_CUDA(call)                                              \
    do {                                                            \
        if ((call) != cudaSuccess) return AXIOM_GPU_OPERATION_FAILED; \
    } while (0)

int32_t checkError(MlpHandle* h) {
    uint32_t err = 0;
    MLP_CUDA(cudaMemcpyAsync(&err, h->st.scratch + 1, 4, cudaMemcpyDeviceToHost, h->stream));
    MLP_CUDA(cudaStreamSynchronize(h->stream));
    return err ? AXIOM_GPU_TIMEOUT : AXIOM_SUCCESS;
}
}  // namespace

extern "C" {

AXIOM_API int32_t axiom_mlp_create(int32_t device, void** mlp) {
    if (!mlp) return AXIOM_NULL_POINTER;
    *mlp = nullptr;
    int dev = 0;
    if (cudaGetDeviceCount(&dev) != cudaSuccess || dev == 0) return AXIOM_GPU_OPERATION_FAILED;
    if (device >= dev) return AXIOM_INVALID_PARAMETER;
    if (device >= 0 && cudaSetDevice(device) != cudaSuccess) return AXIOM_GPU_OPERATION_FAILED;
    MlpHandle* h = new (std::nothrow) MlpHandle();
    if (!h) return AXIOM_OUT_OF_MEMORY;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess || h->st.init() != cudaSuccess) {
        h->st.release(true);
        if (h->stream) cudaStreamDestroy(h->stream);
        delete h;
        return AXIOM_GPU_OPERATION_FAILED;
    }
    *mlp = h;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_mlp_destroy(void* mlp) {
    MlpHandle* h = static_cast<MlpHandle*>(mlp);
    if (!h) return AXIOM_SUCCESS;
    cudaStreamSynchronize(h->stream);
    h->st.release(true);
    cudaStreamDestroy(h->stream);
    delete h;
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_mlp_set_params(void* mlp, const float* params, uint32_t count) {
    MlpHandle* h = static_cast<MlpHandle*>(mlp);
    if (!h || !params) return AXIOM_NULL_POINTER;
    if (count != AXIOM_MLP_PARAM_COUNT) return AXIOM_INVALID_PARAMETER;
    MLP_CUDA(h->st.setParams(params, h->stream));
    MLP_CUDA(cudaMemsetAsync(h->st.adamM, 0, kMlpParams * 4, h->stream));
    MLP_CUDA(cudaMemsetAsync(h->st.adamV, 0, kMlpParams * 4, h->stream));
    h->st.adamStep = 0;
    MLP_CUDA(cudaStreamSynchronize(h->stream));
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_mlp_get_params(void* mlp, float* params, uint32_t count) {
    MlpHandle* h = static_cast<MlpHandle*>(mlp);
    if (!h || !params) return AXIOM_NULL_POINTER;
    if (count != AXIOM_MLP_PARAM_COUNT) return AXIOM_INVALID_PARAMETER;
    MLP_CUDA(cudaMemcpyAsync(params, h->st.params, kMlpParams * 4, cudaMemcpyDeviceToHost, h->stream));
    MLP_CUDA(cudaStreamSynchronize(h->stream));
    return AXIOM_SUCCESS;
}

AXIOM_API int32_t axiom_mlp_forward(void* mlp, const float* features, uint32_t n, float* out) {
    MlpHandle* h = static_cast<MlpHandle*>(mlp);
    if (!h || (n && (!features || !out))) return AXIOM_NULL_POINTER;
    if (n == 0) return AXIOM_SUCCESS;
    MLP_CUDA(h->st.reserveRows(n));
    const uint32_t mpad = (n + 127u) & ~127u;
    MLP_CUDA(cudaMemcpyAsync(h->st.F, features, 4ull * kMlpInputs * n, cudaMemcpyHostToDevice, h->stream));
    h->st.infer(h->st.F, kMlpInputs, nullptr, n, h->stream);
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaMemcpyAsync(out, h->st.Y, 12ull * n, cudaMemcpyDeviceToHost, h->stream));
    return checkError(h);
}

AXIOM_API int32_t axiom_mlp_gradients(void* mlp, const float* features, const float* targets, uint32_t n,
                                      float* grads, float* loss) {
    MlpHandle* h = static_cast<MlpHandle*>(mlp);
    if (!h || !features || !targets || !grads) return AXIOM_NULL_POINTER;
    if (n == 0) return AXIOM_INVALID_PARAMETER;
    MLP_CUDA(h->st.reserveRows(n));
    const uint32_t mpad = (n + 127u) & ~127u;
    MLP_CUDA(cudaMemcpyAsync(h->st.F, features, 4ull * kMlpInputs * n, cudaMemcpyHostToDevice, h->stream));
    MLP_CUDA(cudaMemcpyAsync(h->st.T, targets, 12ull * n, cudaMemcpyHostToDevice, h->stream));
    MLP_CUDA(cudaMemsetAsync(h->st.grads, 0, kMlpParams * 4, h->stream));
    MLP_CUDA(cudaMemsetAsync(h->st.scratch, 0, 4, h->stream));
    h->st.pack(h->st.F, kMlpInputs, n, nullptr, true, h->stream);
    h->st.forward(mpad, true, h->stream);
    h->st.backward(n, mpad, h->st.T, h->stream);
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaMemcpyAsync(grads, h->st.grads, kMlpParams * 4, cudaMemcpyDeviceToHost, h->stream));
    if (loss) MLP_CUDA(cudaMemcpyAsync(loss, h->st.scratch, 4, cudaMemcpyDeviceToHost, h->stream));
    return checkError(h);
}

// Adam over the given data set (host arrays; each minibatch is gathered on the host and
// uploaded): `epochs` passes of
// shuffled minibatches of `batch` rows.  *final_loss = mean loss of the last epoch.
AXIOM_API int32_t axiom_mlp_train(void* mlp, const float* features, const float* targets, uint32_t n,
                                  uint32_t epochs, uint32_t batch, float lr, uint64_t seed, float* final_loss) {
    MlpHandle* h = static_cast<MlpHandle*>(mlp);
    if (!h || !features || !targets) return AXIOM_NULL_POINTER;
    if (n == 0 || batch == 0 || batch % 128u) return AXIOM_INVALID_PARAMETER;
    int32_t status = AXIOM_SUCCESS;
    std::vector<uint32_t> perm(n);
    for (uint32_t i = 0; i < n; ++i) perm[i] = i;
    std::vector<float> hf(4ull * kMlpInputs * std::min(n, batch)), ht(3ull * std::min(n, batch));
    uint64_t st = seed | 1ull;
    auto rnd = [&]() {
        st = st * 6364136223846793005ULL + 1442695040888963407ULL;
        return (uint32_t)(st >> 33);
    };
    float lastLoss = 0.0f;
    do {
        if (h->st.reserveRows(batch) != cudaSuccess) {
            status = AXIOM_GPU_OPERATION_FAILED;
            break;
        }
        for (uint32_t ep = 0; ep < epochs && status == AXIOM_SUCCESS; ++ep) {
            for (uint32_t i = n - 1; i > 0; --i) std::swap(perm[i], perm[rnd() % (i + 1)]);
            if (cudaMemsetAsync(h->st.scratch, 0, 4, h->stream) != cudaSuccess) status = AXIOM_GPU_OPERATION_FAILED;
            uint32_t batches = 0;
            for (uint32_t b0 = 0; b0 + batch <= n && status == AXIOM_SUCCESS; b0 += batch, ++batches) {
                // gather the minibatch on the host (pinned staging is not needed at this size)
                for (uint32_t r = 0; r < batch; ++r) {
                    std::memcpy(&hf[(size_t)r * kMlpInputs], features + (size_t)perm[b0 + r] * kMlpInputs,
                                4 * kMlpInputs);
                    std::memcpy(&ht[(size_t)r * 3], targets + (size_t)perm[b0 + r] * 3, 12);
                }
                if (cudaMemcpyAsync(h->st.F, hf.data(), 4ull * kMlpInputs * batch, cudaMemcpyHostToDevice,
                                    h->stream) != cudaSuccess ||
                    cudaMemcpyAsync(h->st.T, ht.data(), 12ull * batch, cudaMemcpyHostToDevice, h->stream) !=
                        cudaSuccess ||
                    cudaMemsetAsync(h->st.grads, 0, kMlpParams * 4, h->stream) != cudaSuccess) {
                    status = AXIOM_GPU_OPERATION_FAILED;
                    break;
                }
                h->st.pack(h->st.F, kMlpInputs, batch, nullptr, true, h->stream);
                h->st.forward(batch, true, h->stream);
                h->st.backward(batch, batch, h->st.T, h->stream);
                h->st.adam(lr, h->stream);
                // the host reuses hf / ht for the next batch: wait for this one's copies
                if (cudaStreamSynchronize(h->stream) != cudaSuccess) status = AXIOM_GPU_OPERATION_FAILED;
            }
            float sum = 0.0f;
            if (status == AXIOM_SUCCESS &&
                (cudaMemcpy(&sum, h->st.scratch, 4, cudaMemcpyDeviceToHost) != cudaSuccess))
                status = AXIOM_GPU_OPERATION_FAILED;
            lastLoss = batches ? sum / (float)batches : 0.0f;
        }
    } while (false);
    if (status == AXIOM_SUCCESS) status = checkError(h);
    if (final_loss) *final_loss = lastLoss;
    return status;
}

}  // extern "C"
