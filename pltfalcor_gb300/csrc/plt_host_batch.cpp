// plt_bsdf_batch_host: the BSDF batch with host-resident queries and results.  The batch is cut
// into chunks of kHostChunk queries that flow through a three-stage pipeline: the chunk's input
// planes are copied to a device staging slot on an input copy stream, plt_bsdf_batch runs on a
// compute stream, and the output planes are copied back on an output copy stream, so the two copy
// directions and the kernels of different chunks overlap (GB300's host link carries both
// directions at once), also across consecutive calls.  Ordering with the caller's stream: the
// pipeline's streams first wait for everything queued on it before the call (so host inputs
// written by earlier work on that stream are read complete), and the caller's stream waits for the
// last output copy.  The chunk kernels sort through the pipeline's own scratch, never the
// context's, so they cannot race with plt_bsdf_batch calls on other streams.  Every chunk samples with rng_offset = the batch's rng_offset + its first
// query index, so the results equal one plt_bsdf_batch over the whole batch.  (Letting the kernels
// read pinned host memory directly measured 11x slower on GB300: the shade kernel's per-tile
// permuted accesses are latency-bound over the host link.)
#include <cstring>
#include <vector>

#include "plt_context.h"
#include "plt_nvtx.h"

namespace {

// Largest chunk.  The copies of a chunk are one 2-D copy per field (rows = the field's planes), and
// the host link moves long rows faster: the 2^22 mixed batch's copies alone (GB300, both directions
// at once, no kernels) take 2.00 ms per batch with 2^19-query chunks, 1.88 ms with 2^20 and 1.77 ms
// with 2^21, against 1.68 ms for one 285 MB and one 268 MB copy.  End to end with the kernels
// (slots rotating across calls): 2.05, 2.22, 2.33 and, with the whole batch as one chunk, 2.13 G
// queries/s.
#ifndef PLT_HOST_CHUNK_LOG2
#define PLT_HOST_CHUNK_LOG2 21
#endif
constexpr uint32_t kHostChunk = 1u << PLT_HOST_CHUNK_LOG2;
constexpr int kSlots = 4;   // 8 slots measured the same (2.07 G queries/s with 2^19-query chunks)

plt_status cudaFail(plt_context* ctx, cudaError_t e) {
    if (ctx) ctx->lastCudaError = (int)e;
    return e == cudaErrorMemoryAllocation ? PLT_OOM : PLT_CUDA_ERROR;
}
#define PLT_CUDA(ctx, call)                               \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cudaFail(ctx, e_);  \
    } while (0)

// One SoA field: its host pointer and plane count (planes of 4-byte values, stride n).
struct Field {
    const void* host;
    uint32_t planes;
    size_t off;      // byte offset of the field in a staging slot
};

}  // namespace

struct plt_host_pipeline {
    void* stage = nullptr;         // kSlots staging slots
    size_t slotBytes = 0;
    void* scratch = nullptr;       // sort scratch of the chunk kernels (one chunk; sComp runs them in order)
    cudaStream_t sIn = nullptr, sOut = nullptr, sComp = nullptr;
    cudaEvent_t evEntry = nullptr;  // the caller's stream at entry
    cudaEvent_t evIn[kSlots] = {}, evDone[kSlots] = {}, evOut[kSlots] = {};
    bool used[kSlots] = {};
    uint32_t nextSlot = 0;         // slots rotate across calls, so a call's first chunks do not wait on the previous call's last
};

void pltReleaseHostPipeline(plt_context* ctx) {
    plt_host_pipeline* hp = ctx->hostPipe;
    if (!hp) return;
    if (hp->sIn) cudaStreamSynchronize(hp->sIn);
    if (hp->sOut) cudaStreamSynchronize(hp->sOut);
    if (hp->sComp) cudaStreamSynchronize(hp->sComp);
    for (int k = 0; k < kSlots; ++k) {
        if (hp->evIn[k]) cudaEventDestroy(hp->evIn[k]);
        if (hp->evDone[k]) cudaEventDestroy(hp->evDone[k]);
        if (hp->evOut[k]) cudaEventDestroy(hp->evOut[k]);
    }
    if (hp->evEntry) cudaEventDestroy(hp->evEntry);
    if (hp->sIn) cudaStreamDestroy(hp->sIn);
    if (hp->sOut) cudaStreamDestroy(hp->sOut);
    if (hp->sComp) cudaStreamDestroy(hp->sComp);
    cudaFree(hp->stage);
    cudaFree(hp->scratch);
    delete hp;
    ctx->hostPipe = nullptr;
}

extern "C" {

plt_status plt_bsdf_batch_host(plt_context* ctx, const plt_bsdf_queries* hq, const plt_bsdf_results* hr, uint32_t ops, void* stream) {
    const plt::NvtxRange range("bsdf_batch_host");
    if (!ctx || !hq || !hr) return PLT_INVALID_ARG;
    if (hq->hwss < 1 || hq->hwss > PLT_MAX_HWSS) return PLT_INVALID_ARG;
    if (hq->hwss > 4 && hq->hwss != 8) return PLT_NOT_SUPPORTED;
    if (ops == 0 || (ops & ~0xFu)) return PLT_INVALID_ARG;
    const uint32_t n = hq->n, H = hq->hwss;
    if (n == 0) return PLT_OK;
    if (!hq->material || !hq->v || !hq->w || !hq->wavelengths || !hq->stokes || !hq->coherence) return PLT_INVALID_ARG;
    if (const plt_status ds = pltCheckDevice(ctx); ds != PLT_OK) return ds;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);

    // staging layout of one slot: the input fields, then the requested output fields
    std::vector<Field> in = {{hq->material, 1, 0}, {hq->v, 3, 0}, {hq->w, 3, 0}, {hq->lobe, 1, 0},
                             {hq->wavelengths, H, 0}, {hq->stokes, 4 * H, 0}, {hq->coherence, 4, 0}, {hq->beam_t, 3, 0}};
    const bool ev = (ops & PLT_OP_EVAL) != 0, pd = (ops & PLT_OP_PDF) != 0, sm = (ops & PLT_OP_SAMPLE) != 0,
               lp = (ops & PLT_OP_LAMBDA_PDF) != 0;
    std::vector<Field> out = {{ev ? hr->stokes : nullptr, 4 * H, 0},     {ev ? hr->coherence : nullptr, 4, 0},
                              {ev ? hr->beam_t : nullptr, 3, 0},         {pd ? hr->pdf : nullptr, 1, 0},
                              {lp ? hr->lambda_pdf : nullptr, H, 0},     {sm ? hr->sample_wo : nullptr, 3, 0},
                              {sm ? hr->sample_pdf : nullptr, 1, 0},     {sm ? hr->sample_weight : nullptr, 1, 0},
                              {sm ? hr->sample_lobe : nullptr, 1, 0},    {sm ? hr->sample_valid : nullptr, 1, 0}};
    // chunks of at most kHostChunk queries; a smaller batch is one chunk (slots sized for it)
    const uint32_t chunk = n < kHostChunk ? n : kHostChunk;
    size_t off = 0;
    auto place = [&](std::vector<Field>& fs) {
        for (Field& f : fs) {
            if (!f.host) continue;
            f.off = off;
            off += ((size_t)f.planes * chunk * 4 + 255) & ~(size_t)255;
        }
    };
    place(in);
    place(out);
    const size_t slotBytes = off;

    plt_host_pipeline* hp = ctx->hostPipe;
    if (!hp) {
        hp = new (std::nothrow) plt_host_pipeline();
        if (!hp) return PLT_OOM;
        ctx->hostPipe = hp;
        PLT_CUDA(ctx, cudaStreamCreateWithFlags(&hp->sIn, cudaStreamNonBlocking));
        PLT_CUDA(ctx, cudaStreamCreateWithFlags(&hp->sOut, cudaStreamNonBlocking));
        PLT_CUDA(ctx, cudaStreamCreateWithFlags(&hp->sComp, cudaStreamNonBlocking));
        PLT_CUDA(ctx, cudaEventCreateWithFlags(&hp->evEntry, cudaEventDisableTiming));
        PLT_CUDA(ctx, cudaMalloc(&hp->scratch, plt::bsdfScratchBytes(kHostChunk)));
        PLT_CUDA(ctx, cudaMemset(hp->scratch, 0, plt::bsdfScratchBytes(kHostChunk)));   // control words start at zero
        for (int k = 0; k < kSlots; ++k) {
            PLT_CUDA(ctx, cudaEventCreateWithFlags(&hp->evIn[k], cudaEventDisableTiming));
            PLT_CUDA(ctx, cudaEventCreateWithFlags(&hp->evDone[k], cudaEventDisableTiming));
            PLT_CUDA(ctx, cudaEventCreateWithFlags(&hp->evOut[k], cudaEventDisableTiming));
        }
    }
    if (hp->slotBytes < slotBytes) {
        // earlier calls may still be copying out of the slots
        PLT_CUDA(ctx, cudaStreamSynchronize(hp->sOut));
        PLT_CUDA(ctx, cudaStreamSynchronize(hp->sIn));
        PLT_CUDA(ctx, cudaStreamSynchronize(hp->sComp));
        cudaFree(hp->stage);
        hp->stage = nullptr;
        hp->slotBytes = 0;
        for (bool& u : hp->used) u = false;
        PLT_CUDA(ctx, cudaMalloc(&hp->stage, slotBytes * kSlots));
        hp->slotBytes = slotBytes;
    }
    const uint32_t nChunks = (n + chunk - 1) / chunk;
    // nothing of this call starts before the work already queued on the caller's stream
    PLT_CUDA(ctx, cudaEventRecord(hp->evEntry, cs));
    PLT_CUDA(ctx, cudaStreamWaitEvent(hp->sIn, hp->evEntry, 0));
    PLT_CUDA(ctx, cudaStreamWaitEvent(hp->sComp, hp->evEntry, 0));
    for (uint32_t j = 0; j < nChunks; ++j) {
        const int k = (int)((hp->nextSlot + j) % kSlots);
        const uint32_t b = j * chunk, m = n - b < chunk ? n - b : chunk;
        char* slot = static_cast<char*>(hp->stage) + (size_t)k * hp->slotBytes;
        // the slot's previous chunk has left it
        if (hp->used[k]) PLT_CUDA(ctx, cudaStreamWaitEvent(hp->sIn, hp->evOut[k], 0));
        for (const Field& f : in) {
            if (!f.host) continue;
            // planes of m values at stride m in the slot, from planes of stride n on the host
            PLT_CUDA(ctx, cudaMemcpy2DAsync(slot + f.off, (size_t)m * 4, static_cast<const char*>(f.host) + (size_t)b * 4, (size_t)n * 4,
                                            (size_t)m * 4, f.planes, cudaMemcpyHostToDevice, hp->sIn));
        }
        PLT_CUDA(ctx, cudaEventRecord(hp->evIn[k], hp->sIn));
        PLT_CUDA(ctx, cudaStreamWaitEvent(hp->sComp, hp->evIn[k], 0));
        auto dIn = [&](int i) -> const void* { return in[i].host ? slot + in[i].off : nullptr; };
        auto dOut = [&](int i) -> void* { return out[i].host ? slot + out[i].off : nullptr; };
        plt_bsdf_queries q{m, H, hq->rng_offset + b, hq->frame,
                           static_cast<const uint32_t*>(dIn(0)), static_cast<const float*>(dIn(1)), static_cast<const float*>(dIn(2)),
                           static_cast<const uint32_t*>(dIn(3)), static_cast<const float*>(dIn(4)), static_cast<const float*>(dIn(5)),
                           static_cast<const float*>(dIn(6)), static_cast<const float*>(dIn(7))};
        plt_bsdf_results r{static_cast<float*>(dOut(0)), static_cast<float*>(dOut(1)), static_cast<float*>(dOut(2)),
                           static_cast<float*>(dOut(3)), static_cast<float*>(dOut(4)), static_cast<float*>(dOut(5)),
                           static_cast<float*>(dOut(6)), static_cast<float*>(dOut(7)), static_cast<uint32_t*>(dOut(8)),
                           static_cast<uint32_t*>(dOut(9))};
        plt::BatchParams p{};
        int numSMs = 0;
        plt_status st = plt::fillBatchParams(ctx, &q, &r, ops, &p, &numSMs);
        for (void*& t : p.timing) t = nullptr;   // plt_set_timing_events times plt_bsdf_batch, not the chunks
        if (st == PLT_OK) st = pltLaunchBsdfBatch(ctx, p, hp->scratch, hp->sComp);
        if (st != PLT_OK) return st;
        PLT_CUDA(ctx, cudaEventRecord(hp->evDone[k], hp->sComp));
        PLT_CUDA(ctx, cudaStreamWaitEvent(hp->sOut, hp->evDone[k], 0));
        for (const Field& f : out) {
            if (!f.host) continue;
            PLT_CUDA(ctx, cudaMemcpy2DAsync(static_cast<char*>(const_cast<void*>(f.host)) + (size_t)b * 4, (size_t)n * 4, slot + f.off,
                                            (size_t)m * 4, (size_t)m * 4, f.planes, cudaMemcpyDeviceToHost, hp->sOut));
        }
        PLT_CUDA(ctx, cudaEventRecord(hp->evOut[k], hp->sOut));
        hp->used[k] = true;
    }
    // the caller's stream completes when the last results have reached the host
    PLT_CUDA(ctx, cudaStreamWaitEvent(cs, hp->evOut[(hp->nextSlot + nChunks - 1) % kSlots], 0));
    hp->nextSlot = (hp->nextSlot + nChunks) % kSlots;
    return PLT_OK;
}

}  // extern "C"
