// mlp.h — device state of the warm-start network (mlp.cu).
//
// Parameter layout (fp32 master copy, the order of include/axiom_c.h):
//   W1 [128][16] (inputs 14 and 15 are zero padding), b1 [128], W2 [128][128], b2 [128],
//   W3 [128][128], b3 [128], W4 [3][128], b4 [3]; matrices are [out][in], row-major.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace axiom_gb300 {

constexpr uint32_t kMlpInputs = 14;
constexpr uint32_t kOffW1 = 0;
constexpr uint32_t kOffB1 = kOffW1 + 128 * 16;
constexpr uint32_t kOffW2 = kOffB1 + 128;
constexpr uint32_t kOffB2 = kOffW2 + 128 * 128;
constexpr uint32_t kOffW3 = kOffB2 + 128;
constexpr uint32_t kOffB3 = kOffW3 + 128 * 128;
constexpr uint32_t kOffW4 = kOffB3 + 128;
constexpr uint32_t kOffB4 = kOffW4 + 3 * 128;
constexpr uint32_t kMlpParams = kOffB4 + 3;
constexpr uint32_t kMlpSplitRows = 512;              // batch rows per weight-gradient split
constexpr uint32_t kHeadPartials = 3 * 128 + 3 + 1;  // dW4, db4, loss of one head block

struct MlpState {
    // parameters, gradients, Adam moments (fp32) and BF16 GEMM copies
    float* params = nullptr;
    float* grads = nullptr;
    float* adamM = nullptr;
    float* adamV = nullptr;
    __nv_bfloat16 *w1 = nullptr, *w2 = nullptr, *w3 = nullptr, *w2t = nullptr, *w3t = nullptr;
    float* scratch = nullptr;  // [0] loss accumulator, [1] error flag
    uint32_t adamStep = 0;
    uint32_t inferGrid = 0;  // resident CTAs of the fused inference kernel (0: not set up)
    // row buffers (capacity cap rows, a multiple of 128)
    uint32_t cap = 0;
    __nv_bfloat16 *X = nullptr, *XT = nullptr;
    float* Z[3] = {nullptr, nullptr, nullptr};
    __nv_bfloat16* H[3] = {nullptr, nullptr, nullptr};
    __nv_bfloat16* HT[3] = {nullptr, nullptr, nullptr};
    __nv_bfloat16* dZ[3] = {nullptr, nullptr, nullptr};
    __nv_bfloat16* dZT[3] = {nullptr, nullptr, nullptr};
    float* Y = nullptr;  // [rows][3]
    float* T = nullptr;  // targets [rows][3]
    float* F = nullptr;  // staged fp32 features [rows][16]
    // per-split weight-gradient partials [splits][128][128] and per-block head partials
    // [blocks][kHeadPartials], summed in a fixed order so that training is reproducible
    float* part = nullptr;
    float* headPart = nullptr;

    cudaError_t init();
    void release(bool all);
    cudaError_t reserveRows(uint32_t rows);
    cudaError_t setParams(const float* host, cudaStream_t s);
    void refresh(cudaStream_t s);
    // features fp32 rows of `stride` floats -> X (and X^T): row r of X is feature row
    // gather[r] (r itself when gather is null), n rows, zero padding to a multiple of 128
    void pack(const float* f, uint32_t stride, uint32_t n, const uint32_t* gather, bool transposed, cudaStream_t s);
    void forward(uint32_t mpad, bool training, cudaStream_t s);
    // inference of n feature rows (row r = f row gather[r], or r) into Y in one fused kernel
    void infer(const float* f, uint32_t stride, const uint32_t* gather, uint32_t n, cudaStream_t s);
    void head(uint32_t n, uint32_t mpad, const float* targets, cudaStream_t s);
    void backward(uint32_t n, uint32_t mpad, const float* targets, cudaStream_t s);
    void adam(float lr, cudaStream_t s);
};

}  // namespace axiom_gb300
