// Batched BSDF kernels: one plt_bsdf_batch call serves eval / pdf / sample / lambdaPdf for
// queries of any mix of PLT materials (the batched form of IMaterialInstance,
// Source/Falcor/Rendering/Materials/IMaterialInstance.slang:122-184 in ssteinberg/PLTFalcor).
//
// Work layout on sm_103a, two launches:
//  1. classify: one CTA per tile of 2048 queries counting-sorts the tile by (material type, lobe
//     class) in shared memory and writes the tile's permutation (16-bit local indices) to the
//     scratch buffer; block 0 resets the shade kernel's work counter.
//  2. shade: a persistent, barrier-free grid.  Each warp takes 32-query units from one global
//     atomic counter.  Units are issued group by group (128 tiles = 262144 queries per group) and,
//     inside a group, slot-major: unit slot s of every tile before slot s + 1.  Slot s covers
//     sorted positions [32 s, 32 s + 32) of its tile, which hold the same (material, lobe) class
//     in every tile, so at any moment the GPU runs one or two materials' code paths (instruction
//     cache and SIMT coherence) while the group's inputs and outputs (~35 MB) stay L2-resident
//     between the eight material passes (DRAM traffic stays one read of the inputs and one write
//     of the outputs).  The spectral tables are staged into shared memory once per CTA by a bulk
//     asynchronous copy on an mbarrier.
#include "plt_bsdf_query.cuh"
#include "plt_ptx.cuh"

namespace pltdev {

constexpr uint32_t kLobeClasses = 10;                  // lowest set lobe bit (0..7), 8: none, 9: unused
constexpr uint32_t kBuckets = 16 * kLobeClasses;        // material type x lobe class
// Tiles per group: ~1,800 warps are in flight, so a group of G tiles keeps about 1800 / G slots
// (sorted positions x 32) busy at once; 128 tiles (262 K queries, 35 MB of inputs and outputs in
// L2) keeps them within one or two material classes.  Measured on the mixed-material batch: 64
// tiles 4.13, 128 tiles 4.84, 256 tiles 4.66, 512 tiles 3.38 G queries/s (beyond L2).
#ifndef PLT_GROUP_TILES
#define PLT_GROUP_TILES 128
#endif
constexpr uint32_t kGroupTiles = PLT_GROUP_TILES;
constexpr uint32_t kUnitsPerTile = plt::kBatchTile / 32;

PLT_DI uint32_t lobeClass(uint32_t lobe) {
    const uint32_t l = lobe & 0xFFu;
    return l ? (uint32_t)(__ffs((int)l) - 1) : 8u;
}

// internal linkage: each per-wavelength-count translation unit carries its own copy
static __global__ void __launch_bounds__(plt::kBatchThreads) bsdfClassifyKernel(const uint32_t* __restrict__ material,
                                                                         const uint32_t* __restrict__ lobes,
                                                                         const uint8_t* __restrict__ matType, uint32_t nMats,
                                                                         uint32_t n, uint16_t* __restrict__ perm,
                                                                         uint32_t* __restrict__ unitCounter) {
    using namespace plt;
    __shared__ uint32_t counts[kBuckets];
    __shared__ uint32_t offs[kBuckets];
    const uint32_t tid = threadIdx.x;
    const uint32_t base = blockIdx.x * kBatchTile;
    for (uint32_t b = tid; b < kBuckets; b += kBatchThreads) counts[b] = 0;
    __syncthreads();
    uint16_t key[kBatchItems], rank[kBatchItems];
#pragma unroll
    for (int k = 0; k < kBatchItems; ++k) {
        const uint32_t idx = base + k * kBatchThreads + tid;
        uint32_t b = kBuckets - 1;
        if (idx < n) {
            const uint32_t mid = __ldg(material + idx);
            const uint32_t t = mid < nMats ? __ldg(matType + mid) : 14u;
            b = (t & 15u) * kLobeClasses + lobeClass(lobes ? __ldg(lobes + idx) : 0xFFFFu);
        }
        key[k] = (uint16_t)b;
        rank[k] = (uint16_t)atomicAdd(&counts[b], 1u);
    }
    __syncthreads();
    if (tid < 32) {
        // exclusive scan of kBuckets counters by one warp: 5 consecutive buckets per lane
        constexpr uint32_t per = kBuckets / 32;
        uint32_t s = 0;
#pragma unroll
        for (uint32_t j = 0; j < per; ++j) s += counts[tid * per + j];
        uint32_t incl = s;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if ((int)tid >= d) incl += v;
        }
        uint32_t run = incl - s;
#pragma unroll
        for (uint32_t j = 0; j < per; ++j) {
            offs[tid * per + j] = run;
            run += counts[tid * per + j];
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kBatchItems; ++k) perm[base + offs[key[k]] + rank[k]] = (uint16_t)(k * kBatchThreads + tid);
    if (blockIdx.x == 0 && tid == 0) *unitCounter = 0u;
}

template <int H>
__global__ void __launch_bounds__(plt::kShadeThreads, plt::kShadeMinBlocks) bsdfShadeKernel(const BatchParams P) {
    using namespace plt;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    DevProfile* sprof = reinterpret_cast<DevProfile*>(smem);
    const uint32_t tid = threadIdx.x, lane = tid & 31u;

    // Stage the spectral profiles into shared memory with one bulk asynchronous copy.
    const uint32_t profBytes = P.nProfiles * (uint32_t)sizeof(DevProfile);
    if (profBytes > 0) {
        if (tid == 0) {
            mbar_init(&bar, 1);
            fence_mbar_init();
        }
        __syncthreads();
        if (tid == 0) {
            mbar_arrive_expect_tx(&bar, profBytes);
            bulk_g2s(sprof, P.profiles, profBytes, &bar);
        }
        const bool landed = mbar_wait_bounded(&bar, 0, 1u << 22);
        // every thread agrees before anyone leaves, so no barrier below waits on an exited thread
        if (!__syncthreads_and(landed)) {
            if (tid == 0) {
                atomicOr(P.status, kStatusCopyTimeout);
                mbar_wait_bounded(&bar, 0, 1u << 22);  // let a late copy land before the CTA leaves
            }
            return;
        }
    }
    const Ctx c{sprof, P.nProfiles, P.flags};

    const uint32_t n = P.q.n;
    const uint32_t nTiles = (n + kBatchTile - 1) / kBatchTile;
    // With PLT_SHADE_SPLIT_OPS each requested operation is its own slot-major pass over a group
    // (eval, then pdf, lambdaPdf, sample): a warp runs one operation of one material at a time,
    // a smaller code footprint per unit for the instruction caches, at the price of re-reading the
    // group's L2-resident inputs once per operation.
#if PLT_SHADE_SPLIT_OPS
    uint32_t opList[4], nOps = 0;
    for (uint32_t o : {PLT_OP_EVAL, PLT_OP_PDF, PLT_OP_LAMBDA_PDF, PLT_OP_SAMPLE})
        if (P.ops & o) opList[nOps++] = o;
#else
    const uint32_t opList[1] = {0xFFFFFFFFu}, nOps = 1;
#endif
    const uint32_t totalUnits = nTiles * kUnitsPerTile * nOps;
    for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(P.unitCounter, 1u);
        u = __shfl_sync(0xFFFFFFFFu, u, 0);
        if (u >= totalUnits) break;
        const uint32_t group = u / (kUnitsPerTile * kGroupTiles * nOps);
        uint32_t within = u - group * (kUnitsPerTile * kGroupTiles * nOps);
        const uint32_t gTiles = min(kGroupTiles, nTiles - group * kGroupTiles);
        const uint32_t op = within / (gTiles * kUnitsPerTile);
        within -= op * (gTiles * kUnitsPerTile);
        const uint32_t slot = within / gTiles;
        const uint32_t tile = group * kGroupTiles + (within - slot * gTiles);
        const uint32_t base = tile * kBatchTile;
        const uint32_t idx = base + __ldg(P.perm + base + slot * 32u + lane);
        if (idx < n) processQuery<H>(P, c, idx, opList[op]);
    }
}

}  // namespace pltdev

namespace plt {

// classify: one CTA per tile; shade: persistent grid of SM count x resident CTAs per SM
// (occupancy at this launch's shared memory).
template <int H>
cudaError_t launchBsdfBatchH(const BatchParams& p, int numSMs, cudaStream_t stream) {
    const uint32_t nTiles = (p.q.n + kBatchTile - 1) / kBatchTile;
    if (nTiles == 0) return cudaSuccess;
    if (p.timing[0]) cudaEventRecord((cudaEvent_t)p.timing[0], stream);
    pltdev::bsdfClassifyKernel<<<nTiles, kBatchThreads, 0, stream>>>(p.q.material, p.q.lobe, p.matType, p.nMats, p.q.n,
                                                                    p.perm, p.unitCounter);
    if (p.timing[1]) cudaEventRecord((cudaEvent_t)p.timing[1], stream);
    // at most 64 profiles x 528 B = 33 KB: below the 48 KB default limit, so no attribute is set
    const size_t smem = (size_t)p.nProfiles * sizeof(pltdev::DevProfile);
    static_assert(64 * sizeof(pltdev::DevProfile) <= 48 * 1024, "profile staging exceeds the default shared-memory limit");
    int blocksPerSM = 1;
    if (p.launch && p.launch->smem[H] == smem) {
        blocksPerSM = p.launch->blocks[H];
    } else {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, pltdev::bsdfShadeKernel<H>, kShadeThreads, smem) != cudaSuccess || b < 1) b = 1;
        blocksPerSM = b;
        if (p.launch) {
            p.launch->smem[H] = smem;
            p.launch->blocks[H] = b;
        }
    }
    uint32_t grid = (uint32_t)(numSMs * blocksPerSM);
    const uint32_t warpsNeeded = nTiles * (kBatchTile / 32);
    const uint32_t gridCap = (warpsNeeded + (kShadeThreads / 32) - 1) / (kShadeThreads / 32);
    if (grid > gridCap) grid = gridCap;
    pltdev::bsdfShadeKernel<H><<<grid, kShadeThreads, smem, stream>>>(p);
    if (p.timing[2]) cudaEventRecord((cudaEvent_t)p.timing[2], stream);
    return cudaGetLastError();
}

}  // namespace plt
