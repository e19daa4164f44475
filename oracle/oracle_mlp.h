// oracle_mlp.h — TEST INFRASTRUCTURE ONLY.  CPU reference of the warm-start network.
//
// 14 -> 128 -> 128 -> 128 -> 3 with SiLU, parameters in the layout of include/axiom_c.h.
// Evaluated in double, rounding to bf16 exactly where the GPU kernels do (inputs, W1-W3,
// the hidden activations H1-H3 and the back-propagated dZ1-dZ3), so GPU and CPU
// differ only by accumulation order.  W4 / b4 and the biases stay fp32, as on the GPU.
// The reference engine has no learned component; this is the checker for the project's
// own forward and backward kernels.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace oracle {

constexpr uint32_t kMlpIn = 14, kMlpH = 128;
constexpr uint32_t kOffW1 = 0, kOffB1 = 128 * 16, kOffW2 = kOffB1 + 128, kOffB2 = kOffW2 + 128 * 128,
                   kOffW3 = kOffB2 + 128, kOffB3 = kOffW3 + 128 * 128, kOffW4 = kOffB3 + 128,
                   kOffB4 = kOffW4 + 3 * 128, kMlpCount = kOffB4 + 3;

// When false the reference skips every bf16 rounding (plain fp64 network), which lets a
// test check its back-propagation against an independent autodiff.
inline bool& mlpRounding() {
    static bool on = true;
    return on;
}

// Round a float to bf16 (round to nearest, ties to even) and back.
inline float bf16r(float f) {
    if (!mlpRounding()) return f;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) == 0x7F800000u) return f;  // inf / nan unchanged
    uint32_t lsb = (u >> 16) & 1u;
    u += 0x7FFFu + lsb;
    u &= 0xFFFF0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

inline double sigm(double z) { return 1.0 / (1.0 + std::exp(-z)); }

struct MlpCache {
    std::vector<double> x, z1, h1, z2, h2, z3, h3, y;
};

// Forward pass of n rows; fills the cache used by the gradient.
inline void mlpForward(const float* p, const float* feat, uint32_t n, MlpCache* c) {
    c->x.assign((size_t)n * 16, 0.0);
    c->z1.resize((size_t)n * 128);
    c->h1.resize((size_t)n * 128);
    c->z2.resize((size_t)n * 128);
    c->h2.resize((size_t)n * 128);
    c->z3.resize((size_t)n * 128);
    c->h3.resize((size_t)n * 128);
    c->y.resize((size_t)n * 3);
    for (uint32_t r = 0; r < n; ++r)
        for (uint32_t j = 0; j < kMlpIn; ++j) c->x[(size_t)r * 16 + j] = bf16r(feat[(size_t)r * kMlpIn + j]);
    auto layer = [&](const std::vector<double>& in, uint32_t kin, uint32_t woff, uint32_t boff,
                     std::vector<double>& z, std::vector<double>& h) {
        for (uint32_t r = 0; r < n; ++r)
            for (uint32_t o = 0; o < 128; ++o) {
                double acc = 0.0;
                for (uint32_t k = 0; k < kin; ++k) acc += (double)bf16r(p[woff + o * kin + k]) * in[(size_t)r * kin + k];
                float zf = (float)acc + p[boff + o];
                z[(size_t)r * 128 + o] = zf;
                h[(size_t)r * 128 + o] = bf16r((float)(zf * sigm(zf)));
            }
    };
    layer(c->x, 16, kOffW1, kOffB1, c->z1, c->h1);
    layer(c->h1, 128, kOffW2, kOffB2, c->z2, c->h2);
    layer(c->h2, 128, kOffW3, kOffB3, c->z3, c->h3);
    for (uint32_t r = 0; r < n; ++r)
        for (uint32_t o = 0; o < 3; ++o) {
            double acc = p[kOffB4 + o];
            for (uint32_t k = 0; k < 128; ++k) acc += (double)p[kOffW4 + o * 128 + k] * c->h3[(size_t)r * 128 + k];
            c->y[(size_t)r * 3 + o] = acc;
        }
}

// Gradient of the mean squared error (mean over n rows x 3 outputs); returns the loss.
inline double mlpGradients(const float* p, const float* feat, const float* tgt, uint32_t n, double* g) {
    MlpCache c;
    mlpForward(p, feat, n, &c);
    for (uint32_t i = 0; i < kMlpCount; ++i) g[i] = 0.0;
    const double inv = 1.0 / (3.0 * n);
    double loss = 0.0;
    std::vector<double> dz3((size_t)n * 128), dz2((size_t)n * 128), dz1((size_t)n * 128);
    auto dsilu = [](double z) {
        double s = sigm(z);
        return s * (1.0 + z * (1.0 - s));
    };
    for (uint32_t r = 0; r < n; ++r) {
        double dy[3];
        for (int o = 0; o < 3; ++o) {
            double d = c.y[(size_t)r * 3 + o] - tgt[(size_t)r * 3 + o];
            loss += d * d * inv;
            dy[o] = 2.0 * d * inv;
            g[kOffB4 + o] += dy[o];
            for (uint32_t k = 0; k < 128; ++k) g[kOffW4 + o * 128 + k] += dy[o] * c.h3[(size_t)r * 128 + k];
        }
        for (uint32_t k = 0; k < 128; ++k) {
            double dh = p[kOffW4 + k] * dy[0] + p[kOffW4 + 128 + k] * dy[1] + p[kOffW4 + 256 + k] * dy[2];
            dz3[(size_t)r * 128 + k] = bf16r((float)(dh * dsilu(c.z3[(size_t)r * 128 + k])));
        }
    }
    // layer l weights: dW[o][k] = sum_r dz[r][o] * in[r][k]; dIn[r][k] = sum_o dz[r][o] W[o][k]
    auto back = [&](const std::vector<double>& dz, const std::vector<double>& in, uint32_t kin, uint32_t woff,
                    uint32_t boff, const std::vector<double>* zPrev, std::vector<double>* dzPrev) {
        for (uint32_t r = 0; r < n; ++r)
            for (uint32_t o = 0; o < 128; ++o) {
                double d = dz[(size_t)r * 128 + o];
                g[boff + o] += d;
                for (uint32_t k = 0; k < kin; ++k) g[woff + o * kin + k] += d * in[(size_t)r * kin + k];
            }
        if (!dzPrev) return;
        for (uint32_t r = 0; r < n; ++r)
            for (uint32_t k = 0; k < 128; ++k) {
                double acc = 0.0;
                for (uint32_t o = 0; o < 128; ++o) acc += dz[(size_t)r * 128 + o] * (double)bf16r(p[woff + o * kin + k]);
                (*dzPrev)[(size_t)r * 128 + k] = bf16r((float)(acc * dsilu((*zPrev)[(size_t)r * 128 + k])));
            }
    };
    back(dz3, c.h2, 128, kOffW3, kOffB3, &c.z2, &dz2);
    back(dz2, c.h1, 128, kOffW2, kOffB2, &c.z1, &dz1);
    back(dz1, c.x, 16, kOffW1, kOffB1, nullptr, nullptr);
    return loss;
}

}  // namespace oracle
