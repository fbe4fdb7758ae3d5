// Host side of the learned MIS proposal (no counterpart in the reference): per-material features,
// parameter initialisation and transfer, training-batch generation from the exact samplers,
// gradients, Adam steps and the training loop.
#include <cmath>
#include <cstring>
#include <vector>

#include "plt_context.h"
#include "plt_nvtx.h"

namespace plt {
cudaError_t launchProposalData(const pltdev::DevMaterial* mats, const float4* matFeat, const uint2* matProps, const uint32_t* enabled,
                               uint32_t nEnabled, const pltdev::DevProfile* profiles, uint32_t nProfiles, uint32_t flags, uint32_t n,
                               uint32_t seed, void* x, float* target, float* weight, cudaStream_t stream);
cudaError_t launchProposalGrad(const void* params, const void* x, const float* target, const float* weight, uint32_t n, float* grad,
                               float* loss, cudaStream_t stream);
cudaError_t launchProposalForward(const void* params, const void* x, uint32_t n, float* out, cudaStream_t stream);
cudaError_t launchProposalAdam(float* p, float* m, float* v, const float* g, void* pb, float lr, uint32_t step, cudaStream_t stream);
cudaError_t launchProposalToBf16(const float* p, void* pb, cudaStream_t stream);
}  // namespace plt

namespace {

plt_status cudaFail(plt_context* ctx, cudaError_t e) {
    if (ctx) ctx->lastCudaError = (int)e;
    return e == cudaErrorMemoryAllocation ? PLT_OOM : PLT_CUDA_ERROR;
}
#define PLT_CUDA(ctx, call)                               \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cudaFail(ctx, e_);  \
    } while (0)

plt_status ensureProposal(plt_context* ctx) {
    if (ctx->dPropParams) return PLT_OK;
    const size_t P = PLT_PROPOSAL_PARAMS;
    PLT_CUDA(ctx, cudaMalloc(&ctx->dPropParams, 4 * P));
    PLT_CUDA(ctx, cudaMalloc(&ctx->dPropM, 4 * P));
    PLT_CUDA(ctx, cudaMalloc(&ctx->dPropV, 4 * P));
    PLT_CUDA(ctx, cudaMalloc(&ctx->dPropGrad, 4 * P));
    PLT_CUDA(ctx, cudaMalloc(&ctx->dPropBf16, 2 * P));
    PLT_CUDA(ctx, cudaMalloc(&ctx->dPropLoss, 4));
    return PLT_OK;
}

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

plt_status uploadParams(plt_context* ctx, const float* host) {
    plt_status s = ensureProposal(ctx);
    if (s != PLT_OK) return s;
    const size_t P = PLT_PROPOSAL_PARAMS;
    PLT_CUDA(ctx, cudaMemcpy(ctx->dPropParams, host, 4 * P, cudaMemcpyHostToDevice));
    PLT_CUDA(ctx, cudaMemset(ctx->dPropM, 0, 4 * P));
    PLT_CUDA(ctx, cudaMemset(ctx->dPropV, 0, 4 * P));
    PLT_CUDA(ctx, plt::launchProposalToBf16(ctx->dPropParams, ctx->dPropBf16, 0));
    PLT_CUDA(ctx, cudaDeviceSynchronize());
    ctx->propStep = 0;
    ctx->propReady = true;
    return PLT_OK;
}

}  // namespace

// Features of a material for the proposal: roughness (the surface's q), grating pitch (um / 5),
// class (conductor, dielectric, opaque dielectric, coated conductor, coated opaque dielectric,
// grated conductor, grated opaque dielectric, diffuse) and whether the proposal serves it (the
// material has non-delta scatter lobes; diffuse keeps its exact cosine sampler).
float4 pltProposalFeatures(const plt_material_record& r, const pltdev::DevMaterial& d) {
    float rough = 0.f, pitch = 0.f, cls = -1.f;
    bool scatter = false;
    switch (r.type) {
    case PLT_MATERIAL_CONDUCTOR: cls = 0.f; rough = d.p[pltdev::PF_Q]; scatter = true; break;
    case PLT_MATERIAL_DIELECTRIC: cls = 1.f; rough = d.p[pltdev::PG_Q]; scatter = rough != 0.f; break;
    case PLT_MATERIAL_OPAQUE_DIELECTRIC: cls = 2.f; rough = d.p[pltdev::PF_Q]; scatter = true; break;
    case PLT_MATERIAL_COATED_CONDUCTOR: cls = 3.f; rough = d.p[pltdev::PF_Q]; scatter = true; break;
    case PLT_MATERIAL_COATED_OPAQUE_DIELECTRIC: cls = 4.f; rough = d.p[pltdev::PF_Q]; scatter = true; break;
    case PLT_MATERIAL_GRATED_CONDUCTOR:
    case PLT_MATERIAL_GRATED_OPAQUE_DIELECTRIC:
        cls = r.type == PLT_MATERIAL_GRATED_CONDUCTOR ? 5.f : 6.f;
        rough = d.p[pltdev::PF_Q];
        pitch = d.p[pltdev::PD_IPX] > 0.f ? (1.f / d.p[pltdev::PD_IPX]) / 5.f : 0.f;
        scatter = true;
        break;
    case PLT_MATERIAL_DIFFUSE: cls = 7.f; rough = 1.f; break;
    default: break;
    }
    return make_float4(rough, pitch, cls, scatter ? 1.f : 0.f);
}

void pltReleaseProposal(plt_context* ctx) {
    void* ptrs[] = {ctx->dPropParams, ctx->dPropM, ctx->dPropV, ctx->dPropBf16, ctx->dPropGrad, ctx->dPropLoss,
                    ctx->dMatFeat, ctx->dPropEnabled, ctx->dPropBatch};
    for (void* p : ptrs) cudaFree(p);
}

extern "C" {

plt_status plt_proposal_init(plt_context* ctx, uint64_t seed) {
    if (!ctx) return PLT_INVALID_ARG;
    // Glorot-uniform weights, zero biases except the means (0.5, the centre of the primary-sample
    // square) and log sigma = -1 (sigma ~ 0.37)
    std::vector<float> h(PLT_PROPOSAL_PARAMS, 0.f);
    uint64_t st = seed ^ 0x5EEDu;
    const int fan[4][2] = {{16, 64}, {64, 64}, {64, 64}, {64, 32}};
    size_t off = 0;
    for (int l = 0; l < 4; ++l) {
        const float a = std::sqrt(6.f / (float)(fan[l][0] + fan[l][1]));
        for (int i = 0; i < fan[l][0] * fan[l][1]; ++i) {
            const float u = (float)(splitmix(st) >> 40) * 0x1p-24f;
            h[off + i] = (2.f * u - 1.f) * a;
        }
        // the two zero-padding inputs of layer 1 carry no weight
        if (l == 0)
            for (int o = 0; o < 64; ++o) h[off + o * 16 + 14] = h[off + o * 16 + 15] = 0.f;
        off += (size_t)fan[l][0] * fan[l][1];
    }
    const size_t b4 = off + 3 * 64;
    for (int k = 0; k < 8; ++k) {
        h[b4 + 4 * k + 1] = h[b4 + 4 * k + 2] = .5f;
        h[b4 + 4 * k + 3] = -1.f;
    }
    return uploadParams(ctx, h.data());
}

plt_status plt_proposal_set_params(plt_context* ctx, const float* params) {
    if (!ctx || !params) return PLT_INVALID_ARG;
    for (uint32_t i = 0; i < PLT_PROPOSAL_PARAMS; ++i)
        if (!std::isfinite(params[i])) return PLT_NAN_INPUT;
    return uploadParams(ctx, params);
}

plt_status plt_proposal_get_params(plt_context* ctx, float* params) {
    if (!ctx || !params || !ctx->propReady) return PLT_INVALID_ARG;
    PLT_CUDA(ctx, cudaDeviceSynchronize());
    PLT_CUDA(ctx, cudaMemcpy(params, ctx->dPropParams, 4 * (size_t)PLT_PROPOSAL_PARAMS, cudaMemcpyDeviceToHost));
    return PLT_OK;
}

plt_status plt_proposal_generate(plt_context* ctx, uint32_t n, uint32_t seed, uint16_t* x, float* target, float* weight, void* stream) {
    if (!ctx || (n && (!x || !target || !weight))) return PLT_INVALID_ARG;
    if (ctx->nPropEnabled == 0) return PLT_INVALID_ARG;   // no material with non-delta scatter lobes
    PLT_CUDA(ctx, plt::launchProposalData(ctx->dMats, ctx->dMatFeat, static_cast<const uint2*>(ctx->dMatProps), ctx->dPropEnabled,
                                          ctx->nPropEnabled, ctx->dProfiles, ctx->nProfiles, ctx->opt.flags, n, seed, x, target, weight,
                                          (cudaStream_t)stream));
    return PLT_OK;
}

plt_status plt_proposal_gradient(plt_context* ctx, uint32_t n, const uint16_t* x, const float* target, const float* weight, float* grad,
                                 float* loss, void* stream) {
    if (!ctx || !grad || !loss || (n && (!x || !target || !weight)) || !ctx->propReady) return PLT_INVALID_ARG;
    PLT_CUDA(ctx, plt::launchProposalGrad(ctx->dPropBf16, x, target, weight, n, grad, loss, (cudaStream_t)stream));
    return PLT_OK;
}

plt_status plt_proposal_forward(plt_context* ctx, uint32_t n, const uint16_t* x, float* out, void* stream) {
    if (!ctx || (n && (!x || !out)) || !ctx->propReady) return PLT_INVALID_ARG;
    PLT_CUDA(ctx, plt::launchProposalForward(ctx->dPropBf16, x, n, out, (cudaStream_t)stream));
    return PLT_OK;
}

plt_status plt_proposal_adam_step(plt_context* ctx, const float* grad, float lr, void* stream) {
    if (!ctx || !grad || !ctx->propReady || !(lr > 0.f)) return PLT_INVALID_ARG;
    ++ctx->propStep;
    PLT_CUDA(ctx, plt::launchProposalAdam(ctx->dPropParams, ctx->dPropM, ctx->dPropV, grad, ctx->dPropBf16, lr, ctx->propStep,
                                          (cudaStream_t)stream));
    return PLT_OK;
}

plt_status plt_proposal_train(plt_context* ctx, uint32_t steps, uint32_t batch, float lr, uint32_t seed, float* loss_history, void* stream) {
    const plt::NvtxRange range("proposal_train");
    if (!ctx || batch == 0 || !(lr > 0.f)) return PLT_INVALID_ARG;
    if (!ctx->propReady) {
        const plt_status s = plt_proposal_init(ctx, seed);
        if (s != PLT_OK) return s;
    }
    if (ctx->nPropEnabled == 0) return PLT_INVALID_ARG;
    const size_t need = (size_t)batch * (2 * 16 + 4 * 2 + 4);
    if (batch > ctx->propBatchCap) {
        cudaFree(ctx->dPropBatch);
        ctx->dPropBatch = nullptr;
        ctx->propBatchCap = 0;
        PLT_CUDA(ctx, cudaMalloc(&ctx->dPropBatch, need));
        ctx->propBatchCap = batch;
    }
    uint16_t* x = static_cast<uint16_t*>(ctx->dPropBatch);
    float* target = reinterpret_cast<float*>(x + (size_t)batch * 16);
    float* weight = target + 2 * (size_t)batch;
    const cudaStream_t st = (cudaStream_t)stream;
    for (uint32_t k = 0; k < steps; ++k) {
        plt_status s = plt_proposal_generate(ctx, batch, seed * 7919u + k + 1u, x, target, weight, stream);
        if (s != PLT_OK) return s;
        PLT_CUDA(ctx, plt::launchProposalGrad(ctx->dPropBf16, x, target, weight, batch, ctx->dPropGrad, ctx->dPropLoss, st));
        ++ctx->propStep;
        PLT_CUDA(ctx, plt::launchProposalAdam(ctx->dPropParams, ctx->dPropM, ctx->dPropV, ctx->dPropGrad, ctx->dPropBf16, lr, ctx->propStep, st));
        if (loss_history) PLT_CUDA(ctx, cudaMemcpyAsync(loss_history + k, ctx->dPropLoss, 4, cudaMemcpyDeviceToHost, st));
    }
    if (loss_history) PLT_CUDA(ctx, cudaStreamSynchronize(st));
    return PLT_OK;
}

}  // extern "C"
