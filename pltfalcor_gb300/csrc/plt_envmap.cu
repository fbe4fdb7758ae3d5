// The environment sampler's setup and test queries on the GPU: the importance map's base level
// (EnvMapSamplerSetup.cs.slang: the luminance of the lat-long map averaged over 8 x 8 subsamples
// of each texel of the equal-area octahedral map) and its mip chain (the 2 x 2 box average of
// Texture::generateMips, EnvMapSampler.cpp:113-117), and a query kernel that runs the sampler and
// the evaluation for given inputs.  Paths cited are inside ssteinberg/PLTFalcor.
#include "plt_envmap.cuh"

namespace pltdev {

// one thread per texel of the base level
__global__ void __launch_bounds__(256) envImportanceBaseKernel(const plt::EnvDev E, float* imp) {
    const uint32_t dim = E.impDim;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= dim * dim) return;
    const uint32_t px = i % dim, py = i / dim;
    constexpr uint32_t kS = 8;   // sqrt(kEnvImportanceSpp)
    const float invDimS = 1.f / (float)(dim * kS);
    float L = 0.f;
    for (uint32_t y = 0; y < kS; ++y)
        for (uint32_t x = 0; x < kS; ++x) {
            const f2 p{((float)(px * kS + x) + 0.5f) * invDimS, ((float)(py * kS + y) + 0.5f) * invDimS};
            const f3 c = envTexBilinear(E, worldToLatlong(octToNdirEqualAreaUnorm(p)));
            L += luminanceRgb(c.x, c.y, c.z);
        }
    imp[i] = L * (1.f / (float)(kS * kS));
}
// level mip + 1 from level mip
__global__ void __launch_bounds__(256) envImportanceMipKernel(float* imp, uint32_t srcOff, uint32_t dstOff, uint32_t dstDim) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= dstDim * dstDim) return;
    const uint32_t x = i % dstDim, y = i / dstDim, sd = 2 * dstDim;
    const float* s = imp + srcOff;
    const float a = s[(2 * y) * sd + 2 * x], b = s[(2 * y) * sd + 2 * x + 1];
    const float c = s[(2 * y + 1) * sd + 2 * x], d = s[(2 * y + 1) * sd + 2 * x + 1];
    imp[dstOff + i] = ((a + b) + (c + d)) * 0.25f;
}

// out[i][12]: sampled direction (3), its pdf, eval at it (3), evalPdf at it, then eval (3) and
// evalPdf of dirs[i] (zeros when dirs is null)
__global__ void __launch_bounds__(128) envQueryKernel(const plt::EnvDev E, const float* u, const float* dirs, uint32_t n, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float pdf;
    const f3 d = envSampleDir(E, u[2 * (size_t)i], u[2 * (size_t)i + 1], pdf);
    const f3 c = envEval(E, d);
    float* o = out + 12 * (size_t)i;
    o[0] = d.x; o[1] = d.y; o[2] = d.z; o[3] = pdf;
    o[4] = c.x; o[5] = c.y; o[6] = c.z; o[7] = envEvalPdf(E, d);
    if (dirs) {
        const f3 q = mk3(dirs[3 * (size_t)i], dirs[3 * (size_t)i + 1], dirs[3 * (size_t)i + 2]);
        const f3 cq = envEval(E, q);
        o[8] = cq.x; o[9] = cq.y; o[10] = cq.z; o[11] = envEvalPdf(E, q);
    } else {
        o[8] = o[9] = o[10] = o[11] = 0.f;
    }
}

}  // namespace pltdev

namespace plt {

cudaError_t launchEnvImportance(const EnvDev& env, cudaStream_t stream) {
    float* imp = const_cast<float*>(env.imp);
    const uint32_t dim = env.impDim;
    pltdev::envImportanceBaseKernel<<<(dim * dim + 255) / 256, 256, 0, stream>>>(env, imp);
    for (uint32_t mip = 0; mip < env.impBaseMip; ++mip) {
        const uint32_t dd = dim >> (mip + 1);
        pltdev::envImportanceMipKernel<<<(dd * dd + 255) / 256, 256, 0, stream>>>(imp, env.mipOff[mip], env.mipOff[mip + 1], dd);
    }
    return cudaGetLastError();
}

cudaError_t launchEnvQuery(const EnvDev& env, const float* u, const float* dirs, uint32_t n, float* out, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    pltdev::envQueryKernel<<<(n + 127) / 128, 128, 0, stream>>>(env, u, dirs, n, out);
    return cudaGetLastError();
}

}  // namespace plt
