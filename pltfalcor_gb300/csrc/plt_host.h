// Host-side internals of libplt_gb300.so.
#pragma once

#include <cstdint>

#include "../../include/plt_gb300.h"
#include "plt_layout.h"

namespace plt {

float halfToFloat(uint16_t h);
plt_status decodeMaterial(const plt_material_record& r, uint32_t nProfiles, pltdev::DevMaterial& d);
plt_status spectralProfileFromSamples(const float* wl, const float* val, uint32_t count, float scale, int computeIcdf,
                                      plt_spectral_profile* sp);

}  // namespace plt
