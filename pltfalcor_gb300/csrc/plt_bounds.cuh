// Index checks of the PLT_BOUNDS_CHECK build (-DPLT_BOUNDS_CHECK=1): the kernels' reads and writes
// of queue entries, path-state and bounce-record planes, triangles, materials, deferred tasks, the
// image accumulator and the batch's sort permutation go through pltIdx.  An index outside its buffer
// sets kStatusBoundsViolation, records the first violation (site, index, bound) in status[1..3] and
// is replaced by 0, so the access stays inside the buffer and the kernel runs to its end; the host
// reads the report through plt_check_status (PLT_BOUNDS_VIOLATION) and
// plt_last_bounds_violation.  In the default build pltIdx returns the index unchanged.  This is the
// project's substitute for a memory checker: it needs no tool and faults nothing.
#pragma once

#include <cstdint>

#include "plt_internal.h"

#ifndef PLT_BOUNDS_CHECK
#define PLT_BOUNDS_CHECK 0
#endif

namespace pltdev {

// where an index was checked (status[1] of a violation)
enum BoundsSite : uint32_t {
    kSiteQueue = 1,        // a segment queue entry or a solve-order entry
    kSitePath = 2,         // a path id (path-state planes)
    kSiteBounce = 3,       // a bounce-record offset
    kSitePrim = 4,         // a triangle id
    kSiteMaterial = 5,     // a material id
    kSiteTask = 6,         // a deferred walk or replay task, or its order entry
    kSiteAccum = 7,        // an image-accumulator path
    kSiteQuery = 8,        // a batch query index
    kSitePerm = 9,         // a position in a tile's sort permutation
};

__device__ __forceinline__ size_t pltIdx(uint32_t* status, size_t idx, size_t bound, uint32_t site) {
#if PLT_BOUNDS_CHECK
    if (idx < bound) return idx;
    if ((atomicOr(status, plt::kStatusBoundsViolation) & plt::kStatusBoundsViolation) == 0u) {
        status[1] = site;
        status[2] = (uint32_t)idx;
        status[3] = (uint32_t)bound;
    }
    return 0;
#else
    (void)status;
    (void)bound;
    (void)site;
    return idx;
#endif
}

}  // namespace pltdev
