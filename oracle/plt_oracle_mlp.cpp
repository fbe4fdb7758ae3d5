// ORACLE -- test infrastructure only.  CPU forward / backward of the learned MIS proposal
// (pltfalcor_gb300/csrc/plt_mlp.cuh: 16 -> 64 -> 64 -> 64 -> 32, SiLU, 8-component Gaussian
// mixture on the unit disk, mean weighted negative log-likelihood).  Accumulation in double; with
// `round_bf16` the values the GPU stores in BF16 (weights, biases, inputs, pre-activations,
// activations, back-propagated gradients) are rounded the same way, so the GPU's gradients differ
// from these only by FP32 accumulation order.  Without it everything is double (finite-difference
// checks of the back-propagation).  The proposal has no counterpart in the reference.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>


#include "plt_oracle_mlp.hpp"

namespace {

using namespace plt_oracle_mlp;

// mixture NLL of one sample and d(loss)/d(out)
double nllGrad(const double* out, double tx, double ty, double w, double* d) {
    for (int j = 0; j < kOut; ++j) d[j] = 0.0;
    if (!(w > 0.0)) return 0.0;
    double lmax = -1e300;
    for (int k = 0; k < kComp; ++k) lmax = std::fmax(lmax, out[4 * k]);
    double lsum = 0.0;
    for (int k = 0; k < kComp; ++k) lsum += std::exp(out[4 * k] - lmax);
    const double lse = lmax + std::log(lsum);
    double a[kComp], d2s[kComp], amax = -1e300;
    for (int k = 0; k < kComp; ++k) {
        const double s = std::fmin(std::fmax(out[4 * k + 3], kLogSigmaMin), kLogSigmaMax);
        const double is2 = std::exp(-2.0 * s);
        const double dx = tx - out[4 * k + 1], dy = ty - out[4 * k + 2];
        d2s[k] = (dx * dx + dy * dy) * is2;
        a[k] = (out[4 * k] - lse) - 0.5 * d2s[k] - 2.0 * s - std::log(2.0 * M_PI);
        amax = std::fmax(amax, a[k]);
    }
    double asum = 0.0;
    for (int k = 0; k < kComp; ++k) asum += std::exp(a[k] - amax);
    const double lq = amax + std::log(asum);
    for (int k = 0; k < kComp; ++k) {
        const double r = std::exp(a[k] - lq);
        const double pik = std::exp(out[4 * k] - lse);
        const double s = out[4 * k + 3];
        const double is2 = std::exp(-2.0 * std::fmin(std::fmax(s, kLogSigmaMin), kLogSigmaMax));
        d[4 * k] = -w * (r - pik);
        d[4 * k + 1] = -w * r * (tx - out[4 * k + 1]) * is2;
        d[4 * k + 2] = -w * r * (ty - out[4 * k + 2]) * is2;
        d[4 * k + 3] = (s > kLogSigmaMin && s < kLogSigmaMax) ? -w * r * (d2s[k] - 2.0) : 0.0;
    }
    return -w * lq;
}

}  // namespace

extern "C" {

// outputs [n][32] of feature rows x [n][16] (bf16 bits)
void plto_mlp_forward(const float* params, const uint16_t* x, uint32_t n, int round_bf16, float* out) {
    const Net net(params, round_bf16 != 0);
    for (uint32_t s = 0; s < n; ++s) {
        double xi[kIn], z1[kHid], z2[kHid], z3[kHid], o[kOut];
        for (int i = 0; i < kIn; ++i) xi[i] = bf16Bits(x[(size_t)s * kIn + i]);
        net.forward(xi, z1, z2, z3, o);
        for (int j = 0; j < kOut; ++j) out[(size_t)s * kOut + j] = (float)o[j];
    }
}

// gradient [11488] of the mean weighted NLL over the batch and the loss; x may be given as
// float features (x_f32, used when non-null) for finite-difference checks in double.
double plto_mlp_gradient(const float* params, const uint16_t* x, const double* x_f64, const float* target, const float* weight,
                         uint32_t n, int round_bf16, double* grad) {
    const Net net(params, round_bf16 != 0);
    std::vector<double> g(kParams, 0.0);
    double loss = 0.0;
    for (uint32_t s = 0; s < n; ++s) {
        double xi[kIn], z1[kHid], z2[kHid], z3[kHid], o[kOut], d4[kOut];
        for (int i = 0; i < kIn; ++i) xi[i] = x_f64 ? x_f64[(size_t)s * kIn + i] : bf16Bits(x[(size_t)s * kIn + i]);
        net.forward(xi, z1, z2, z3, o);
        loss += nllGrad(o, target[2 * (size_t)s], target[2 * (size_t)s + 1], weight[s], d4);
        for (int j = 0; j < kOut; ++j) d4[j] = net.q(d4[j]);
        double h1[kHid], h2[kHid], h3[kHid];
        for (int i = 0; i < kHid; ++i) {
            h1[i] = net.q(net.silu(z1[i]));
            h2[i] = net.q(net.silu(z2[i]));
            h3[i] = net.q(net.silu(z3[i]));
        }
        double d3[kHid], d2[kHid], d1[kHid];
        for (int i = 0; i < kHid; ++i) {
            double a = 0.0;
            for (int o2 = 0; o2 < kOut; ++o2) a += d4[o2] * net.p[kW4 + o2 * kHid + i];
            d3[i] = net.q(a * net.siluGrad(z3[i]));
        }
        for (int i = 0; i < kHid; ++i) {
            double a = 0.0;
            for (int o2 = 0; o2 < kHid; ++o2) a += d3[o2] * net.p[kW3 + o2 * kHid + i];
            d2[i] = net.q(a * net.siluGrad(z2[i]));
        }
        for (int i = 0; i < kHid; ++i) {
            double a = 0.0;
            for (int o2 = 0; o2 < kHid; ++o2) a += d2[o2] * net.p[kW2 + o2 * kHid + i];
            d1[i] = net.q(a * net.siluGrad(z1[i]));
        }
        for (int o2 = 0; o2 < kOut; ++o2) {
            for (int i = 0; i < kHid; ++i) g[kW4 + o2 * kHid + i] += d4[o2] * h3[i];
            g[kB4 + o2] += d4[o2];
        }
        for (int o2 = 0; o2 < kHid; ++o2) {
            for (int i = 0; i < kHid; ++i) {
                g[kW3 + o2 * kHid + i] += d3[o2] * h2[i];
                g[kW2 + o2 * kHid + i] += d2[o2] * h1[i];
            }
            for (int i = 0; i < kIn; ++i) g[kW1 + o2 * kIn + i] += d1[o2] * xi[i];
            g[kB3 + o2] += d3[o2];
            g[kB2 + o2] += d2[o2];
            g[kB1 + o2] += d1[o2];
        }
    }
    const double inv = n ? 1.0 / (double)n : 0.0;
    for (int i = 0; i < kParams; ++i) grad[i] = g[i] * inv;
    return loss * inv;
}

}  // extern "C"
