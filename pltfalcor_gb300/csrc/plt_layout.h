// Device-side record layouts shared by the host decoder (plt_materials.cpp) and the kernels.
#pragma once

#include <cstdint>

namespace pltdev {

// Device material record, 192 bytes, filled once per material by the host from the reference
// material record (setupMaterialInstance of the PLT*Material.slang files, evaluated ahead of
// time with the reference's float expressions).
struct alignas(16) DevMaterial {
    uint32_t type;          // plt_material_type
    uint32_t aux;           // grating: lobeCount | (gratingType << 8); multilayer: layer count
    uint32_t etaN, etaK;    // spectral profile ids (conductor bases)
    float m00a[12];         // rgbToSpectrum(primary rgb) per basis bin (specular / albedo / base colour)
    float m00b[12];         // rgbToSpectrum(transmission rgb) per basis bin (dielectric)
    float p[20];            // type-specific constants, see the P*_ indices
};
static_assert(sizeof(DevMaterial) == 192, "DevMaterial must stay 192 bytes");

// Device copy of a SpectralProfile's evaluation part, 528 bytes (a multiple of 16 so an array
// of them moves with one bulk copy).
struct alignas(16) DevProfile {
    float intensity, minl, maxl;
    uint32_t bins;
    float pdf[128];
};
static_assert(sizeof(DevProfile) == 528, "DevProfile must stay 528 bytes");

// Gaussian surface (dielectric)
enum { PG_SIGMA2 = 0, PG_Q = 1, PG_ETAINT = 2, PG_ETAEXT = 3, PG_B = 4, PG_INVSIGMA2 = 5 };
// Fractal surface block (conductor / opaque dielectric / coated / grated bases)
enum { PF_T = 0, PF_GAMMA = 1, PF_Q = 2, PF_EXPO = 3, PF_C = 4, PF_SEXP = 5, PF_IEXP = 6, PF_SQRTT = 7, PF_EXTETA = 8 };
// coated
enum { PC_COATIOR = 9, PC_TAU = 10, PC_COATETA = 11, PC_ETA1 = 12 };
// grating
enum { PD_GX = 9, PD_GY = 10, PD_IPX = 11, PD_IPY = 12, PD_Q = 13, PD_MULT = 14 };
// thin dielectric
enum { PT_OAX = 0, PT_OAY = 1, PT_OAZ = 2, PT_ETA = 3, PT_TAU = 4, PT_BIREF = 5, PT_EO = 6, PT_EE = 7, PT_TAUUM = 8 };
// multilayer
enum { PM_EXTETA = 0, PM_IOR1 = 1, PM_IOR2 = 2, PM_TH1 = 3, PM_TH2 = 4, PM_ETA1 = 5, PM_ETA2 = 6 };

}  // namespace pltdev
