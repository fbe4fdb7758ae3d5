// Batched BSDF kernels: one plt_bsdf_batch call serves eval / pdf / sample / lambdaPdf for
// queries of any mix of PLT materials (the batched form of IMaterialInstance,
// Source/Falcor/Rendering/Materials/IMaterialInstance.slang:122-184 in ssteinberg/PLTFalcor).
//
// Work layout on sm_103a, two launches (one for a batch of at most kSmallBatchTiles tiles, shaded
// unsorted by the shade kernel alone):
//  1. classify: a persistent grid whose CTAs counting-sort tiles of 2048 queries by (material type,
//     lobe class) in shared memory, write each tile's permutation (16-bit local indices) and the
//     start of each material type's range in it, and add their tiles' per-type counts to the batch
//     totals.  The last CTA to finish builds the schedule from those totals: per material type, a queue of
//     work units (each a slice of one tile's range of that type, tiles in order) and, per SM, the
//     type it starts on, with SM shares proportional to each type's queries x relative cost.
//  2. shade: a persistent, barrier-free grid.  Every warp of an SM takes units from the queue of
//     its SM's type, so each SM runs one material's code at a time (the instruction caches hold
//     one material's eval + sample + pdf), and because every queue walks the tiles in order at a
//     rate matched to its SM share, all types work on the same few tiles at a time and each tile's
//     inputs and outputs stay L2-resident between the material passes over it (DRAM traffic stays
//     about one read of the inputs and one write of the outputs).  A warp whose queue runs dry
//     moves to the queue with the most work left.  Each unit's code is specialised for its type at
//     compile time.  The spectral tables are staged into shared memory once per CTA by a bulk
//     asynchronous copy on an mbarrier.
#include "plt_bounds.cuh"
#include "plt_bsdf_query.cuh"
#include "plt_ptx.cuh"

namespace pltdev {

using plt::kTypeSlots;
// Sub-buckets of a material type: 0..7 the lowest set lobe bit, 8 no lobe bit; a material whose
// type byte has bit 7 set is bucketed by its work class instead (bits 4..6: stack layers in fours
// for multilayers), 8..15, so a warp's lanes run loops of similar trip counts.  The last bucket
// (type 15, class 15) holds the padding.
constexpr uint32_t kLobeClasses = 16;
constexpr uint32_t kBuckets = kTypeSlots * kLobeClasses;  // material type x lobe / work class
constexpr uint32_t kPadBucket = kBuckets - 1;             // positions past the end of the batch

// Control words of a batch's schedule (BatchParams::ctrl).  C_COUNT, C_MAX and C_DONE are zero
// when a batch starts: the schedule builder zeroes them after reading them.
enum : uint32_t {
    C_COUNT = 0,    // [16] queries per type (classify atomics)
    C_MAX = 16,     // [16] largest per-tile count per type (classify atomics)
    C_NEXT = 32,    // [16] next unit of each type's queue (the shade kernel's work counters)
    C_DONE = 48,    // classify CTAs finished
    C_UNITS = 64,   // [16] units per tile of each type's queue
    C_USZ = 80,     // [16] queries per unit of each type (a multiple of 32)
    C_TOTAL = 96,   // [16] queries per type
    C_COST = 112,   // [16] measured cost per query of each type (float; exponential average over batches)
    C_CYC = 128,    // [16] x u64: warp cycles spent on each type's units in the last batch
    C_WORDS = 160
};
static_assert(C_WORDS * 4 <= plt::kBsdfCtrlBytes, "control words exceed their scratch block");

// entries of the sort permutation: whole tiles
PLT_DI size_t permSlots(uint32_t n) { return ((size_t)n + plt::kBatchTile - 1) / plt::kBatchTile * plt::kBatchTile; }

PLT_DI uint32_t lobeClass(uint32_t lobe) {
    const uint32_t l = lobe & 0xFFu;
    return l ? (uint32_t)(__ffs((int)l) - 1) : 8u;
}

PLT_DI uint32_t smId() {
    uint32_t s;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(s));
    return s;
}
PLT_DI uint32_t smIdCount() {
    uint32_t s;
    asm volatile("mov.u32 %0, %%nsmid;" : "=r"(s));
    return s;
}
PLT_DI uint32_t ldVolatile(const uint32_t* p) { return *reinterpret_cast<const volatile uint32_t*>(p); }

// A bound on how far a type's queue may lead the slowest one (tiles; 0 = none).  Measured on the
// 2^22 mixed batch (4 launches each): none 0.543 ms and 0.66-1.17 GB of DRAM traffic per launch;
// 32 tiles checked every 8 units 0.566 ms and 0.61-0.62 GB (1.11x the algorithmic bytes); 96 tiles
// 0.566 ms, 0.78-0.82 GB; 192 tiles 0.578 ms, 1.03-1.05 GB; checks every 16 or 32 units 0.68-0.71 ms
// (helping warps crowd the slowest queue).  Off: the batch's time is what counts.
#ifndef PLT_LEAD_TILES
#define PLT_LEAD_TILES 0
#endif
#ifndef PLT_LEAD_CHECK
#define PLT_LEAD_CHECK 8
#endif

// weight of the last batch's measured cost per query in each type's running average
// (0.2 and a minimum over the last two batches measured no better: per-launch DRAM traffic
// alternates between ~0.76 and ~1.15 GB with any of them)
#ifndef PLT_COST_EMA
#define PLT_COST_EMA 0.5f
#endif

// Schedule of a batch, built by the last classify CTA (all 256 threads) once every tile's counts
// are in: unit size and units per tile of each type, and the SM -> starting type table.
PLT_DI void buildSchedule(const BatchParams& P, uint32_t* sh) {
    using namespace plt;
    const uint32_t tid = threadIdx.x;
    uint32_t* count = sh;          // [16]
    float* cum = reinterpret_cast<float*>(sh + 16);   // [17] cumulative work
    float* cost = reinterpret_cast<float*>(sh + 33);  // [16] cost per query
    uint32_t* measured = sh + 49;  // 1 while every queried type has a measured cost
    uint32_t* mxs = sh + 50;       // [16] largest per-tile count per type
    if (tid == 0) *measured = 1u;
    // one round trip: the first warp reads the cost counters, the second takes the batch's counts
    unsigned long long cyc = 0ull;
    uint32_t prev = 0u, avgBits = 0u;
    if (tid < kTypeSlots) {
        cyc = atomicExch(reinterpret_cast<unsigned long long*>(P.ctrl + C_CYC) + tid, 0ull);
        prev = P.ctrl[C_TOTAL + tid];
        avgBits = P.ctrl[C_COST + tid];
    } else if (tid >= 32 && tid < 32 + kTypeSlots) {
        const uint32_t k = tid - 32;
        count[k] = atomicExch(P.ctrl + C_COUNT + k, 0u);
        mxs[k] = atomicExch(P.ctrl + C_MAX + k, 0u);
    }
    __syncthreads();
    if (tid < kTypeSlots) {
        // the previous batch's cycles per query of this type, folded into its running average
        float avg = __uint_as_float(avgBits);
        if (prev >= 1024u && cyc > 0ull) {
            const float m = (float)cyc / (float)prev;
            avg = avg > 0.f ? (1.f - PLT_COST_EMA) * avg + PLT_COST_EMA * m : m;
            P.ctrl[C_COST + tid] = __float_as_uint(avg);
        }
        cost[tid] = avg;
    } else if (tid >= 32 && tid < 32 + kTypeSlots) {
        const uint32_t k = tid - 32, mx = mxs[k];
        // units: slices of about unitQueries of one tile's range, at most ceil(max / unitQueries) per tile
        const uint32_t units = mx ? (mx + P.unitQueries - 1) / P.unitQueries : 0u;
        const uint32_t usz = units ? ((mx + units - 1) / units + 31u) & ~31u : 0u;
        P.ctrl[C_UNITS + k] = units;
        P.ctrl[C_USZ + k] = usz;
        P.ctrl[C_TOTAL + k] = count[k];
        P.ctrl[C_NEXT + k] = 0u;
    }
    __syncthreads();
#ifndef PLT_ADAPTIVE_COSTS
#define PLT_ADAPTIVE_COSTS 1
#endif
    if (tid < kTypeSlots && count[tid] > 0u && (!PLT_ADAPTIVE_COSTS || !(cost[tid] > 0.f))) atomicAnd(measured, 0u);
    __syncthreads();
    if (tid == 0) {
        // SM shares: queries x measured cost once every queried type has one, else the priors
        float s = 0.f;
        cum[0] = 0.f;
        for (uint32_t t = 0; t < kTypeSlots; ++t) {
            s += (float)count[t] * (*measured ? cost[t] : P.typeCost[t]);
            cum[t + 1] = s;
        }
        P.ctrl[C_DONE] = 0u;
    }
    __syncthreads();
    // SM s starts on the type whose share of the cumulative work holds (s + 1/2) / nsmid
    const uint32_t nsm = min(smIdCount(), kMaxSmIds);
    const float total = cum[kTypeSlots];
    for (uint32_t s = tid; s < kMaxSmIds; s += blockDim.x) {
        const float x = ((float)(s % nsm) + 0.5f) / (float)nsm * total;
        uint32_t t = 0;
        while (t + 1 < kTypeSlots && !(x < cum[t + 1])) ++t;
        while (t + 1 < kTypeSlots && count[t] == 0) ++t;   // never start on an empty queue
        P.smType[s] = (uint8_t)t;
    }
}

// The material ids and lobes of one tile's items (kBatchItems per thread).
PLT_DI void loadTileKeys(const BatchParams& P, uint32_t base, uint32_t* mid, uint32_t* lob) {
    using namespace plt;
    const uint32_t n = P.q.n;
#pragma unroll
    for (int k = 0; k < kBatchItems; ++k) {
        const uint32_t idx = base + k * kBatchThreads + threadIdx.x;
        mid[k] = idx < n ? __ldg(P.q.material + idx) : 0xFFFFFFFFu;
        lob[k] = idx < n && P.q.lobe ? __ldg(P.q.lobe + idx) : 0xFFFFu;
    }
}

// Persistent: each CTA sorts tiles blockIdx.x, blockIdx.x + gridDim.x, ... (a grid of the resident
// CTAs), loading the next tile's material ids and lobes while it sorts the current one, and adds
// its tiles' per-type counts to the batch totals once.  Measured on the 2^22 batch (2,048 tiles):
// one CTA per tile lived ~13 us (6 us of it waiting on its loads) and ran in three waves, 38 us.
#ifndef PLT_CLASSIFY_MIN_BLOCKS
#define PLT_CLASSIFY_MIN_BLOCKS 4
#endif
#ifndef PLT_CLASSIFY_MATCH
#define PLT_CLASSIFY_MATCH 0
#endif
// internal linkage: each per-wavelength-count translation unit carries its own copy
static __global__ void __launch_bounds__(plt::kBatchThreads, PLT_CLASSIFY_MIN_BLOCKS) bsdfClassifyKernel(const BatchParams P) {
    using namespace plt;
    __shared__ uint32_t counts[kBuckets];
    __shared__ uint32_t offs[kBuckets];
    __shared__ uint32_t sched[72];
    __shared__ uint32_t ctaCount[kTypeSlots], ctaMax[kTypeSlots];
    __shared__ __align__(16) uint16_t tilePerm[kBatchTile];   // the tile's permutation, stored coalesced
    __shared__ bool isLast;
    const uint32_t tid = threadIdx.x;
    const uint32_t n = P.q.n;
    const uint32_t nTiles = (n + kBatchTile - 1) / kBatchTile;
    // the shade kernel may be scheduled once every classify CTA has started: it stages its tables
    // and then waits for this grid to complete (programmatic dependent launch)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (tid < kTypeSlots) {
        ctaCount[tid] = 0u;
        ctaMax[tid] = 0u;
    }
    uint32_t mid[kBatchItems], lob[kBatchItems];
    loadTileKeys(P, blockIdx.x * kBatchTile, mid, lob);
    for (uint32_t tile = blockIdx.x; tile < nTiles; tile += gridDim.x) {
        const uint32_t base = tile * kBatchTile;
        for (uint32_t b = tid; b < kBuckets; b += kBatchThreads) counts[b] = 0;
        __syncthreads();
        // the material types of this tile's items, then the next tile's ids and lobes in flight
        // while this one is counted, scanned and scattered
        uint32_t key32[kBatchItems];
#pragma unroll
        for (int k = 0; k < kBatchItems; ++k) {
            const uint32_t t = mid[k] < P.nMats ? __ldg(P.matType + mid[k]) : 14u;
            uint32_t b = kPadBucket;
            if (base + k * kBatchThreads + tid < n) {
                const uint32_t cls = (t & 0x80u) ? 8u + ((t >> 4) & 7u) : lobeClass(lob[k]);
                b = (t & 15u) * kLobeClasses + cls;
            }
            key32[k] = b;
        }
        loadTileKeys(P, tile + gridDim.x < nTiles ? (tile + gridDim.x) * kBatchTile : n, mid, lob);
        // bucket << 16 | rank within the bucket
#if PLT_CLASSIFY_MATCH
        // one shared-memory atomic per distinct bucket of a warp (same-address atomics serialise)
        const uint32_t lane = tid & 31u, below = (1u << lane) - 1u;
#pragma unroll
        for (int k = 0; k < kBatchItems; ++k) {
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key32[k]);
            const uint32_t leader = (uint32_t)__ffs((int)peers) - 1u;
            uint32_t first = 0;
            if (lane == leader) first = atomicAdd(&counts[key32[k]], (uint32_t)__popc(peers));
            first = __shfl_sync(0xFFFFFFFFu, first, (int)leader);
            key32[k] = key32[k] << 16 | (first + (uint32_t)__popc(peers & below));
        }
#else
#pragma unroll
        for (int k = 0; k < kBatchItems; ++k) key32[k] = key32[k] << 16 | atomicAdd(&counts[key32[k]], 1u);
#endif
        __syncthreads();
        if (tid < 32) {
            // exclusive scan of kBuckets counters by one warp: 8 consecutive buckets per lane
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
        for (int k = 0; k < kBatchItems; ++k)
            tilePerm[pltIdx(P.status, offs[key32[k] >> 16] + (key32[k] & 0xFFFFu), (uint32_t)kBatchTile, kSitePerm)] = (uint16_t)(k * kBatchThreads + tid);
        // type t's range of this tile: [offs[t * kLobeClasses], start of type t + 1); the padding
        // bucket comes last, so its start is the tile's query count
        __syncthreads();
        // 16 bytes per thread: the tile's 2,048 16-bit entries in one coalesced store
        static_assert(kBatchTile * sizeof(uint16_t) == kBatchThreads * sizeof(uint4), "one 16-byte store per thread");
        reinterpret_cast<uint4*>(P.perm + base)[tid] = reinterpret_cast<const uint4*>(tilePerm)[tid];
        if (tid <= kTypeSlots) {
            const uint32_t start = tid < kTypeSlots ? offs[tid * kLobeClasses] : offs[kPadBucket];
            P.tileTypeOff[tile * (kTypeSlots + 1) + tid] = (uint16_t)start;
            if (tid < kTypeSlots) {
                const uint32_t end = tid + 1 < kTypeSlots ? offs[(tid + 1) * kLobeClasses] : offs[kPadBucket];
                ctaCount[tid] += end - start;
                ctaMax[tid] = max(ctaMax[tid], end - start);
            }
        }
        __syncthreads();   // counts and offs are rewritten for the next tile
    }
    if (tid < kTypeSlots && ctaCount[tid]) {
        atomicAdd(P.ctrl + C_COUNT + tid, ctaCount[tid]);
        atomicMax(P.ctrl + C_MAX + tid, ctaMax[tid]);
    }
    // the last CTA to finish builds the schedule: the barrier orders this CTA's count atomics
    // before thread 0's fence, so they are complete once every CTA has counted itself done (the
    // permutation's plain stores need no fence: the shade grid reads them after this grid ends)
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        isLast = atomicAdd(P.ctrl + C_DONE, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (isLast) {
        __threadfence();
        buildSchedule(P, sched);
    }
}

// One unit: positions [lo, hi) of the tile's sorted permutation, all of material type T (T = 0:
// a slot of invalid types or material ids, which only report their status and zero the outputs).
// One query of material type T (T = 0: an invalid type or material id, which only reports its
// status and zeroes the outputs), when `valid`.
template <int H, uint32_t T>
__device__ __forceinline__ void shadeUnit(const BatchParams& P, const Ctx& c, uint32_t idx, bool valid) {
    if (valid) processQueryTyped<H>(P, c, idx, 0xFFFFFFFFu, ldPlane(P.q.material + idx), T);
}

// The queue with the most estimated work left (remaining units x unit size x cost), or kTypeSlots
// when every queue is empty.  Whole warp.
PLT_DI uint32_t busiestQueue(const BatchParams& P, uint32_t nTiles, uint32_t lane) {
    float work = -1.f;
    if (lane < kTypeSlots) {
        const uint32_t units = min(ldVolatile(P.ctrl + C_UNITS + lane), (uint32_t)plt::kBatchTile / 32u) * nTiles;
        const uint32_t next = ldVolatile(P.ctrl + C_NEXT + lane);
        if (next < units) work = (float)(units - next) * (float)ldVolatile(P.ctrl + C_USZ + lane) * P.typeCost[lane];
    }
    uint32_t best = lane;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const float w2 = __shfl_xor_sync(0xFFFFFFFFu, work, d);
        const uint32_t b2 = __shfl_xor_sync(0xFFFFFFFFu, best, d);
        if (w2 > work || (w2 == work && b2 < best)) {
            work = w2;
            best = b2;
        }
    }
    return work > 0.f ? best : kTypeSlots;
}

// The queue whose next unit lies in the lowest tile among the queues with work left, packed as
// tile << 8 | type (0xFFFFFFFF when every queue is empty).  Whole warp; `unitsOf` is each lane's
// type's units per tile.
PLT_DI uint32_t slowestQueue(const BatchParams& P, uint32_t nTiles, uint32_t unitsOf, uint32_t lane) {
    uint32_t key = 0xFFFFFFFFu;
    if (lane < kTypeSlots && unitsOf) {
        const uint32_t next = ldVolatile(P.ctrl + C_NEXT + lane);
        if (next < unitsOf * nTiles) key = (next / unitsOf) << 8 | lane;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) key = min(key, __shfl_xor_sync(0xFFFFFFFFu, key, d));
    return key;
}

// Stages the spectral profiles into shared memory with one bulk asynchronous copy; false (after
// reporting the timeout and letting a late copy land) when the copy did not land within the poll
// budget.  All threads of the CTA.
PLT_DI bool stageProfiles(const BatchParams& P, DevProfile* sprof, uint64_t* bar) {
    using namespace plt;
    const uint32_t tid = threadIdx.x;
    const uint32_t profBytes = P.nProfiles * (uint32_t)sizeof(DevProfile);
    if (profBytes == 0) return true;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0) {
        mbar_arrive_expect_tx(bar, profBytes);
        bulk_g2s(sprof, P.profiles, profBytes, bar);
    }
    const bool landed = mbar_wait_bounded(bar, 0, P.copyPolls);
    // every thread agrees before anyone leaves, so no barrier below waits on an exited thread
    if (!__syncthreads_and(landed)) {
        if (tid == 0) {
            atomicOr(P.status, kStatusCopyTimeout);
            mbar_wait_bounded(bar, 0, 1u << 22);  // let a late copy land before the CTA leaves
        }
        return false;
    }
    return true;
}

// This lane's query (when `valid`), of material type t, with the code specialised for t at compile
// time.  The warp's lanes all pass the same t.
template <int H>
PLT_DI void shadeRange(const BatchParams& P, const Ctx& c, uint32_t t, uint32_t idx, bool v) {
    switch (t) {
    case kMatDielectric: shadeUnit<H, kMatDielectric>(P, c, idx, v); break;
    case kMatConductor: shadeUnit<H, kMatConductor>(P, c, idx, v); break;
    case kMatOpaqueDielectric: shadeUnit<H, kMatOpaqueDielectric>(P, c, idx, v); break;
    case kMatCoatedConductor: shadeUnit<H, kMatCoatedConductor>(P, c, idx, v); break;
    case kMatCoatedOpaque: shadeUnit<H, kMatCoatedOpaque>(P, c, idx, v); break;
    case kMatGratedConductor: shadeUnit<H, kMatGratedConductor>(P, c, idx, v); break;
    case kMatGratedOpaque: shadeUnit<H, kMatGratedOpaque>(P, c, idx, v); break;
    case kMatThin: shadeUnit<H, kMatThin>(P, c, idx, v); break;
    case kMatMultilayer: shadeUnit<H, kMatMultilayer>(P, c, idx, v); break;
    case kMatDiffuse: shadeUnit<H, kMatDiffuse>(P, c, idx, v); break;
    default: shadeUnit<H, 0u>(P, c, idx, v); break;
    }
}

// The shade kernel.  A batch of more than kSmallBatchTiles tiles is shaded from the per-type unit
// queues of the classify schedule.  A small batch is not classified (it is latency-bound and gains
// nothing from the queues or the sort): warp w takes the 32 consecutive queries of units w,
// w + warps, ..., and shades them once per material type among them, the lanes of that type
// active.  Both schedules end in the one call of the typed code, so a query gives the same bits in
// any batch.
template <int H>
__global__ void __launch_bounds__(plt::kShadeThreads, plt::shadeMinBlocks<H>()) bsdfShadeKernel(const BatchParams P) {
    using namespace plt;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ unsigned long long cycles[kTypeSlots];   // this CTA's warp cycles per type
    DevProfile* sprof = reinterpret_cast<DevProfile*>(smem);
    const uint32_t tid = threadIdx.x, lane = tid & 31u;
    if (tid < kTypeSlots) cycles[tid] = 0ull;
    if (!stageProfiles(P, sprof, &bar)) return;
    const Ctx c{sprof, P.nProfiles, P.flags};
    // the classify grid's permutation and schedule are complete and visible past this point
    // (a no-op when the kernel was not launched as a programmatic dependent)
    asm volatile("griddepcontrol.wait;" ::: "memory");

    const bool small = P.smallBatch != 0u;
    const uint32_t nTiles = (P.q.n + kBatchTile - 1) / kBatchTile;
    // the schedule never has more than kBatchTile / 32 units of at least 32 queries per tile; the
    // clamps keep every loop bounded whatever the control words hold
    constexpr uint32_t kMaxUnits = kBatchTile / 32;
    // each type's units per tile, one per lane (read together with this SM's type: one round trip)
    const uint32_t unitsOf = lane < kTypeSlots && !small ? min(__ldg(P.ctrl + C_UNITS + lane), kMaxUnits) : 0u;
    uint32_t t = small ? 0u : P.smType[smId() % kMaxSmIds] % kTypeSlots;
    uint32_t units = __shfl_sync(0xFFFFFFFFu, unitsOf, (int)t);
    // a small batch's current unit: its first query, its query count, this lane's material type
    // and the lanes not yet shaded
    const uint32_t warpId = blockIdx.x * (kShadeThreads / 32) + (tid >> 5), warps = gridDim.x * (kShadeThreads / 32);
    uint32_t sUnit = warpId, sBase = 0, sCount = 0, sType = 0, sLeft = 0;
    bool sStarted = false;
    uint32_t t0q = 0;   // the queue the current unit came from
#if PLT_LEAD_TILES
    // a warp whose own queue leads the slowest queue by more than PLT_LEAD_TILES tiles takes its
    // next PLT_LEAD_CHECK units from the slowest queue (checked every PLT_LEAD_CHECK units)
    uint32_t ownTile = 0, sinceCheck = 0, helpLeft = 0, helpType = 0;
#endif
    for (;;) {
        uint32_t tile, lo, hi, mask = 0xFFFFFFFFu;
        if (small) {
            if (sLeft == 0u) {
                if (sStarted) sUnit += warps;
                sStarted = true;
                if (sUnit >= (P.q.n + 31u) / 32u) break;
                sBase = sUnit * 32u;
                sCount = min(32u, P.q.n - sBase);
                if (lane < sCount) {
                    const uint32_t mid = ldPlane(P.q.material + sBase + lane);
                    sType = (mid < P.nMats ? (uint32_t)__ldg(P.matType + mid) : 14u) & 15u;
                }
                sLeft = __ballot_sync(0xFFFFFFFFu, lane < sCount);
            }
            // the type of the lowest lane not yet shaded, and every remaining lane of that type
            t = __shfl_sync(0xFFFFFFFFu, sType, __ffs((int)sLeft) - 1);
            mask = __ballot_sync(0xFFFFFFFFu, ((sLeft >> lane) & 1u) && sType == t);
            sLeft &= ~mask;
            tile = 0;
            lo = 0;
            hi = sCount;
        } else {
            uint32_t qt = t, qunits = units;
#if PLT_LEAD_TILES
            if (helpLeft) {
                qt = helpType;
                --helpLeft;
            } else if (++sinceCheck >= PLT_LEAD_CHECK) {
                sinceCheck = 0;
                const uint32_t slow = slowestQueue(P, nTiles, unitsOf, lane);
                if (slow != 0xFFFFFFFFu && (slow & 0xFFu) != t && ownTile > (slow >> 8) + PLT_LEAD_TILES) {
                    helpType = slow & 0xFFu;
                    helpLeft = PLT_LEAD_CHECK - 1;
                    qt = helpType;
                }
            }
            if (qt != t) qunits = __shfl_sync(0xFFFFFFFFu, unitsOf, (int)qt);
#endif
            uint32_t u = 0;
            if (lane == 0) u = atomicAdd(P.ctrl + C_NEXT + qt, 1u);
            u = __shfl_sync(0xFFFFFFFFu, u, 0);
            if (u >= qunits * nTiles) {
#if PLT_LEAD_TILES
                if (qt != t) {
                    helpLeft = 0;
                    continue;
                }
#endif
                t = busiestQueue(P, nTiles, lane);
                if (t >= kTypeSlots) break;
                units = __shfl_sync(0xFFFFFFFFu, unitsOf, (int)t);
                continue;
            }
            tile = u / qunits;
#if PLT_LEAD_TILES
            if (qt == t) ownTile = tile;
#endif
            const uint32_t sub = u - tile * qunits;
            const uint32_t usz = max(32u, min(__ldg(P.ctrl + C_USZ + qt), (uint32_t)kBatchTile));
            const uint16_t* off = P.tileTypeOff + tile * (kTypeSlots + 1);
            lo = __ldg(off + qt) + sub * usz;
            hi = min(min((uint32_t)__ldg(off + qt + 1), (uint32_t)kBatchTile), lo + usz);
            if (lo >= hi) continue;
            t0q = qt;
        }
        const uint32_t st = small ? t : t0q;
        const uint32_t base = small ? sBase : tile * kBatchTile;
        const long long t0 = clock64();
        // one pass for the schedule's 32-query units and for a small batch's unit
        for (uint32_t pos = lo; pos < hi; pos += 32) {
            const uint32_t k = pos + lane;
            const bool inUnit = k < hi && ((mask >> lane) & 1u);
            uint32_t idx = 0;
            if (inUnit) idx = small ? base + k : base + __ldg(P.perm + pltIdx(P.status, base + k, permSlots(P.q.n), kSitePerm));
            shadeRange<H>(P, c, st, idx, inUnit && idx < P.q.n);
        }
        __syncwarp();
        if (lane == 0 && !small) atomicAdd(&cycles[st], (unsigned long long)(clock64() - t0));
    }
    // the measured cost per type feeds the next batch's SM shares
    __syncthreads();
    if (tid < kTypeSlots && cycles[tid])
        atomicAdd(reinterpret_cast<unsigned long long*>(P.ctrl + C_CYC) + tid, cycles[tid]);
}

}  // namespace pltdev

namespace plt {

// Default relative cost per query of each material type (the schedule's SM shares): shade time
// per query in ns of each material's 2^19 queries of the mixed-material batch run alone on GB300
// (eval + sample + pdf, HWSS 1).  Opaque dielectric and diffuse are estimates.
inline float defaultTypeCost(uint32_t t) {
    using namespace pltdev;
    switch (t) {
    case kMatDielectric: return .105f;
    case kMatConductor: return .090f;
    case kMatCoatedOpaque: return .105f;
    case kMatCoatedConductor: return .117f;
    case kMatGratedOpaque: return .150f;
    case kMatGratedConductor: return .160f;
    case kMatThin: return .078f;
    case kMatMultilayer: return .156f;
    case kMatOpaqueDielectric: return .080f;
    case kMatDiffuse: return .050f;
    default: return .050f;
    }
}

// Batches of at most this many tiles (65,536 queries) are not classified: the classify launch, its
// last-CTA schedule build and the queue look-ups cost more latency than a few-tile batch loses to
// mixed-type warps (configuration 0, 65,536 single-material queries: 8.2 us per batch unclassified,
// 14.4 us classified).
constexpr uint32_t kSmallBatchTiles = 32;

// classify: one CTA per tile; shade: persistent grid of SM count x resident CTAs per SM
// (occupancy at this launch's shared memory).
template <int H>
cudaError_t launchBsdfBatchH(const BatchParams& p0, int numSMs, cudaStream_t stream) {
    const uint32_t nTiles = (p0.q.n + kBatchTile - 1) / kBatchTile;
    if (nTiles == 0) return cudaSuccess;
    // at most 64 profiles x 528 B = 33 KB: below the 48 KB default limit, so no attribute is set
    const size_t smem = (size_t)p0.nProfiles * sizeof(pltdev::DevProfile);
    static_assert(64 * sizeof(pltdev::DevProfile) <= 48 * 1024, "profile staging exceeds the default shared-memory limit");
    int blocksPerSM = 1;
    if (p0.launch && p0.launch->smem[H] == smem) {
        blocksPerSM = p0.launch->blocks[H];
    } else {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, pltdev::bsdfShadeKernel<H>, kShadeThreads, smem) != cudaSuccess || b < 1) b = 1;
        blocksPerSM = b;
        if (p0.launch) {
            p0.launch->smem[H] = smem;
            p0.launch->blocks[H] = b;
        }
    }
    uint32_t grid = (uint32_t)(numSMs * blocksPerSM);
    const uint32_t warpsNeeded = (p0.q.n + 31u) / 32u;
    const uint32_t gridCap = (warpsNeeded + (kShadeThreads / 32) - 1) / (kShadeThreads / 32);
    if (grid > gridCap) grid = gridCap;
    BatchParams p = p0;
    // units of one warp iteration (32 queries): a unit stays in flight for one iteration only, so the
    // tiles the GPU works on at a time stay few (L2 locality of the scattered loads and stores).
    // Measured on the 2^22 mixed batch: 32-query units 0.79 ms, 256-query units 0.86 ms per launch;
    // bounding each queue's lead over the slowest one (16 or 32 tiles) made it slower (1.2-2.0 ms),
    // since every unit then re-reads the contended queue counters and SMs leave their type
    p.unitQueries = 32;
    p.smallBatch = nTiles <= kSmallBatchTiles ? 1u : 0u;
    for (uint32_t t = 0; t < kTypeSlots; ++t)
        if (!(p.typeCost[t] > 0.f)) p.typeCost[t] = defaultTypeCost(t);
    // the classify grid: the resident CTAs (persistent over the tiles), at most one per tile
    int cb = p0.launch ? p0.launch->classifyBlocks[H] : 0;
    if (cb < 1) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cb, pltdev::bsdfClassifyKernel, kBatchThreads, 0) != cudaSuccess || cb < 1) cb = 1;
        if (p0.launch) p0.launch->classifyBlocks[H] = cb;
    }
    const uint32_t classifyGrid = min(nTiles, (uint32_t)(numSMs * cb));
    if (p.timing[0]) cudaEventRecord((cudaEvent_t)p.timing[0], stream);
    // a small batch is not classified: one ordinary launch of the shade kernel
    if (!p.smallBatch) pltdev::bsdfClassifyKernel<<<classifyGrid, kBatchThreads, 0, stream>>>(p);
    cudaError_t e = cudaSuccess;
    if (p.smallBatch) {
        if (p.timing[1]) cudaEventRecord((cudaEvent_t)p.timing[1], stream);
        pltdev::bsdfShadeKernel<H><<<grid, kShadeThreads, smem, stream>>>(p);
    } else if (p.timing[1]) {
        // per-kernel timing: an event between the kernels, so an ordinary launch
        cudaEventRecord((cudaEvent_t)p.timing[1], stream);
        pltdev::bsdfShadeKernel<H><<<grid, kShadeThreads, smem, stream>>>(p);
    } else {
        // programmatic dependent launch: the shade CTAs are scheduled while classify finishes and
        // stage their spectral tables before waiting on it (hides the launch gap of small batches)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(kShadeThreads);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, pltdev::bsdfShadeKernel<H>, p);
    }
    if (e != cudaSuccess) return e;
    if (p.timing[2]) cudaEventRecord((cudaEvent_t)p.timing[2], stream);
    return cudaGetLastError();
}

}  // namespace plt
