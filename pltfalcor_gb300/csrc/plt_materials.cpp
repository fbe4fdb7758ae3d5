// Host-side material decode: reference material record -> DevMaterial.
//
// Restates setupMaterialInstance of each PLT material (paths inside ssteinberg/PLTFalcor,
// Source/Falcor/Rendering/Materials/PLT/PLT*Material.slang) plus the per-material constants of
// GaussianSurface.slang:42-59 and FractalSurface.slang:43-86, evaluated once per material with the
// same float expressions the shaders evaluate per call.  rgbToSpectrum
// (Utils/Color/SpectrumUtils.slang:106-198) is tabulated per basis bin.  Also the spectral-profile
// builder (SceneBuilder.cpp:911-960 with PiecewiseLinearSpectrum / SampledSpectrum).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "plt_host.h"

namespace plt {

float halfToFloat(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t exp = (h >> 10) & 0x1Fu, man = h & 0x3FFu, bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign;
        } else {
            int e = -1;
            do { ++e; man <<= 1; } while ((man & 0x400u) == 0);
            bits = sign | ((uint32_t)(127 - 15 - e) << 23) | ((man & 0x3FFu) << 13);
        }
    } else if (exp == 31) {
        bits = sign | 0x7F800000u | (man << 13);
    } else {
        bits = sign | ((exp - 15 + 127) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

namespace {

constexpr float kPi = 3.14159265358979323846f;
constexpr float k2Pi = 6.28318530717958647693f;
constexpr float k1_2Pi = 0.159154943091895335769f;

// 11-bin basis of SpectrumUtils.rgbToSpectrum (bin 10 is zero: lambda >= 720 nm)
const float kWhite[11] = {1.0000f, 1.0000f, 0.9999f, 0.9993f, 0.9992f, 0.9998f, 1.0000f, 1.0000f, 1.0000f, 1.0000f, 0.0f};
const float kCyan[11] = {0.9710f, 0.9426f, 1.0007f, 1.0007f, 1.0007f, 1.0007f, 0.1564f, 0.0000f, 0.0000f, 0.0000f, 0.0f};
const float kMagenta[11] = {1.0000f, 1.0000f, 0.968f, 0.22295f, 0.0000f, 0.0458f, 0.8369f, 1.0000f, 1.0000f, 0.9959f, 0.0f};
const float kYellow[11] = {0.0001f, 0.0000f, 0.1088f, 0.6651f, 1.0000f, 1.0000f, 0.9996f, 0.9586f, 0.9685f, 0.9840f, 0.0f};
const float kRed[11] = {0.1012f, 0.0515f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.8325f, 1.0149f, 1.0149f, 1.014f, 0.0f};
const float kGreen[11] = {0.0000f, 0.0000f, 0.0273f, 0.7937f, 1.0000f, 0.9418f, 0.1719f, 0.0000f, 0.0000f, 0.0025f, 0.0f};
const float kBlue[11] = {1.0000f, 1.0000f, 0.8916f, 0.3323f, 0.0000f, 0.0000f, 0.0003f, 0.0369f, 0.0483f, 0.0496f, 0.0f};

float rgbToSpectrumBin(const float rgb[3], int b) {
    float sd = 0.f;
    const float r = rgb[0], g = rgb[1], bl = rgb[2];
    if (r <= g && r <= bl) {
        sd += kWhite[b] * r;
        if (g <= bl) { sd += kCyan[b] * (g - r); sd += kBlue[b] * (bl - g); }
        else { sd += kCyan[b] * (bl - r); sd += kGreen[b] * (g - bl); }
    } else if (g <= r && g <= bl) {
        sd += kWhite[b] * g;
        if (r <= bl) { sd += kMagenta[b] * (r - g); sd += kBlue[b] * (bl - r); }
        else { sd += kMagenta[b] * (bl - g); sd += kRed[b] * (r - bl); }
    } else {
        sd += kWhite[b] * bl;
        if (r <= g) { sd += kYellow[b] * (r - bl); sd += kGreen[b] * (g - r); }
        else { sd += kYellow[b] * (g - bl); sd += kRed[b] * (r - g); }
    }
    return sd;
}
void tabulate(const float rgb[3], float* out) {
    for (int b = 0; b < 11; ++b) out[b] = rgbToSpectrumBin(rgb, b);
    out[11] = 0.f;
}

float meank() { return k2Pi / (550.0f * 1e-3f); }

// GaussianSurface(PSDroughness), GaussianSurface.slang:42-59
void gaussianConstants(float roughness, float* p) {
    auto toSigma2 = [](float r) { return std::pow(std::min(std::max(1.f - .5f * r, 0.f), 1.f), 28.f) * 2500.f; };
    const float s2 = toSigma2(roughness), s2max = toSigma2(0.1f), s2r0 = toSigma2(0.f);
    const float t = (s2r0 - s2) / (s2r0 - s2max);
    p[pltdev::PG_Q] = 0.f + (1.f - 0.f) * t;
    p[pltdev::PG_SIGMA2] = std::min(s2max, s2);
    p[pltdev::PG_INVSIGMA2] = 1.f / p[pltdev::PG_SIGMA2];
}
// FractalSurface(PSDroughness, gamma), FractalSurface.slang:43-86 and pGF/sample constants
void fractalConstants(float roughness, float gammaIn, float* p) {
    const float gamma = std::max(1.1f, gammaIn);
    const float mk = meank();
    const float a = std::min(std::max(roughness, 0.f), .75f);
    const float alpha2 = a * a;
    const float T = std::min(5000.f, (1.f - alpha2) / (4.f * (mk * mk) * alpha2));
    p[pltdev::PF_T] = T;
    p[pltdev::PF_GAMMA] = gamma;
    p[pltdev::PF_Q] = (1.f / std::sqrt(1.f + 4.f * (mk * mk) * T)) * 1.f;
    p[pltdev::PF_EXPO] = (gamma + 1.f) / 2.f;
    p[pltdev::PF_C] = k1_2Pi * (gamma - 1.f) * T;
    p[pltdev::PF_SEXP] = -(gamma - 1.f) / 2.f;
    p[pltdev::PF_IEXP] = -2.f / (gamma - 1.f);
    p[pltdev::PF_SQRTT] = std::sqrt(T);
}

}  // namespace

plt_status decodeMaterial(const plt_material_record& r, uint32_t nProfiles, pltdev::DevMaterial& d) {
    std::memset(&d, 0, sizeof(d));
    d.type = r.type;
    d.etaN = r.ior_n_spectral_id;
    d.etaK = r.ior_k_spectral_id;
    float base[4], spec[4], data1[4], data2[4], tran[3];
    for (int i = 0; i < 4; ++i) {
        base[i] = halfToFloat(r.base_color[i]);
        spec[i] = halfToFloat(r.specular[i]);
        data1[i] = halfToFloat(r.data1[i]);
        data2[i] = halfToFloat(r.data2[i]);
    }
    for (int i = 0; i < 3; ++i) tran[i] = halfToFloat(r.transmission[i]);
    const float ior = halfToFloat(r.ior);
    float* p = d.p;
    auto needProfiles = [&]() {
        return (r.ior_n_spectral_id == PLT_NO_SPECTRAL_PROFILE || r.ior_n_spectral_id < nProfiles) &&
               (r.ior_k_spectral_id == PLT_NO_SPECTRAL_PROFILE || r.ior_k_spectral_id < nProfiles);
    };
    tabulate(base, d.m00a);
    switch (r.type) {
    case PLT_MATERIAL_DIFFUSE: return PLT_OK;
    case PLT_MATERIAL_DIELECTRIC: {  // PLTDielectricMaterial.slang:40-57
        tabulate(tran, d.m00b);
        gaussianConstants(spec[1], p);
        const bool anyT = tran[0] > 0.f || tran[1] > 0.f || tran[2] > 0.f;
        const float B = anyT ? spec[0] : 0.f;
        p[pltdev::PG_ETAINT] = std::max(1.f, ior - 2.897f * B);
        p[pltdev::PG_ETAEXT] = spec[3];
        p[pltdev::PG_B] = B;
        return PLT_OK;
    }
    case PLT_MATERIAL_CONDUCTOR:  // PLTConductorMaterial.slang:40-57
        if (!needProfiles()) return PLT_INVALID_ARG;
        fractalConstants(spec[1], spec[0], p);
        p[pltdev::PF_EXTETA] = ior;
        return PLT_OK;
    case PLT_MATERIAL_OPAQUE_DIELECTRIC:  // PLTOpaqueDielectricMaterial.slang:40-52
        fractalConstants(spec[1], 3.f, p);
        return PLT_OK;
    case PLT_MATERIAL_COATED_CONDUCTOR:       // PLTCoatedConductorMaterial.slang:40-60
    case PLT_MATERIAL_COATED_OPAQUE_DIELECTRIC: {  // PLTCoatedOpaqueDielectricMaterial.slang:40-57
        if (r.type == PLT_MATERIAL_COATED_CONDUCTOR && !needProfiles()) return PLT_INVALID_ARG;
        fractalConstants(spec[1], 3.f, p);
        const float extEta = ior, tau = data1[0] * spec[2], coatIOR = data1[3];
        p[pltdev::PF_EXTETA] = extEta;
        p[pltdev::PC_COATIOR] = coatIOR;
        p[pltdev::PC_TAU] = tau;
        const float minTau = .05f;
        const float t = std::min(std::max(tau, 0.f), minTau) / minTau;
        const float coatior = extEta + (coatIOR - extEta) * t;
        p[pltdev::PC_COATETA] = coatior;
        p[pltdev::PC_ETA1] = coatior / extEta;
        return PLT_OK;
    }
    case PLT_MATERIAL_GRATED_CONDUCTOR:          // PLTDiffractionGratedConductorMaterial.slang:41-73
    case PLT_MATERIAL_GRATED_OPAQUE_DIELECTRIC: {  // PLTDiffractionGratedOpaqueDielectricMaterial.slang:41-69
        if (r.type == PLT_MATERIAL_GRATED_CONDUCTOR && !needProfiles()) return PLT_INVALID_ARG;
        fractalConstants(data2[1], 3.f, p);
        p[pltdev::PF_EXTETA] = ior;
        const float dir = data1[2];
        p[pltdev::PD_GX] = std::cos(dir);
        p[pltdev::PD_GY] = std::sin(dir);
        p[pltdev::PD_IPX] = data1[0] > 0.f ? 1.f / data1[0] : 0.f;
        p[pltdev::PD_IPY] = data1[1] > 0.f ? 1.f / data1[1] : 0.f;
        p[pltdev::PD_Q] = data2[0] * spec[0];
        p[pltdev::PD_MULT] = spec[1];
        const uint16_t tl = r.data1[3];
        const uint32_t lobes = std::min(std::max((uint32_t)(tl & 0xFFu), 1u), 8u);
        const uint32_t gtype = (uint32_t)(tl >> 8);
        if (gtype & 0x10u) return PLT_NOT_SUPPORTED;  // radial gratings need the surface uv
        d.aux = lobes | (gtype << 8);
        return PLT_OK;
    }
    case PLT_MATERIAL_THIN_DIELECTRIC: {  // PLTThinDielectricMaterial.slang:40-54
        const float ox = base[1], oy = base[2];
        p[pltdev::PT_OAX] = ox;
        p[pltdev::PT_OAY] = oy;
        p[pltdev::PT_OAZ] = std::sqrt(std::max(0.f, 1.f - (ox * ox + oy * oy)));
        p[pltdev::PT_ETA] = ior;
        p[pltdev::PT_TAU] = spec[3];
        const float biref = base[0] * spec[0];
        p[pltdev::PT_BIREF] = biref;
        p[pltdev::PT_EO] = ior - .5f * biref;
        p[pltdev::PT_EE] = ior + .5f * biref;
        p[pltdev::PT_TAUUM] = spec[3] * 1e+3f;
        return PLT_OK;
    }
    case PLT_MATERIAL_MULTILAYERED_STACK: {  // PLTMultiLayeredStackMaterial.slang:40-57
        p[pltdev::PM_EXTETA] = ior;
        p[pltdev::PM_IOR1] = data2[0];
        p[pltdev::PM_IOR2] = data2[1];
        p[pltdev::PM_TH1] = data1[0];
        p[pltdev::PM_TH2] = data1[1];
        p[pltdev::PM_ETA1] = data2[0] / ior;
        p[pltdev::PM_ETA2] = data2[1] / data2[0];
        d.aux = r.data1[3];
        return PLT_OK;
    }
    default: return PLT_BAD_MATERIAL;
    }
}

namespace {

// CIE 1931 XYZ multi-lobe Gaussian fit (Wyman, Sloan, Shirley 2013), as the shaders evaluate it
// (SpectrumUtils.slang:43-49)
float cieLobe(float x, float mu, float s1, float s2) {
    const float t = (x - mu) * (x < mu ? s1 : s2);
    return std::exp(-0.5f * t * t);
}
void cieXyz(float l, float& x, float& y, float& z) {
    x = 0.362f * cieLobe(l, 442.0f, 0.0624f, 0.0374f) + 1.056f * cieLobe(l, 599.8f, 0.0264f, 0.0323f) -
        0.065f * cieLobe(l, 501.1f, 0.0490f, 0.0382f);
    y = 0.821f * cieLobe(l, 568.8f, 0.0213f, 0.0247f) + 0.286f * cieLobe(l, 530.9f, 0.0613f, 0.0322f);
    z = 1.217f * cieLobe(l, 437.0f, 0.0845f, 0.0278f) + 0.681f * cieLobe(l, 459.0f, 0.0385f, 0.0725f);
}
// CIE D65 relative spectral power, 380-720 nm in 5 nm steps (the shaders' table,
// SpectrumUtils.slang:66-82), linearly interpolated; zero outside the range.
float d65(float l) {
    static const float t[69] = {49.9755f, 52.3118f, 54.6482f, 68.7015f, 82.7549f, 87.1204f, 91.486f, 92.4589f, 93.4318f,
                                90.057f, 86.6823f, 95.7736f, 104.865f, 110.936f, 117.008f, 117.41f, 117.812f, 116.336f,
                                114.861f, 115.392f, 115.923f, 112.367f, 108.811f, 109.082f, 109.354f, 108.578f, 107.802f,
                                106.296f, 104.79f, 106.239f, 107.689f, 106.047f, 104.405f, 104.225f, 104.046f, 102.023f,
                                100.f, 98.1671f, 96.3342f, 96.0611f, 95.788f, 92.2368f, 88.6856f, 89.3459f, 90.0062f,
                                89.8026f, 89.5991f, 88.6489f, 87.6987f, 85.4936f, 83.2886f, 83.4939f, 83.6992f, 81.863f,
                                80.0268f, 80.1207f, 80.2146f, 81.2462f, 82.2778f, 80.281f, 78.2842f, 74.0027f, 69.7213f,
                                70.6652f, 71.6091f, 72.979f, 74.349f, 67.9765f, 61.604f};
    if (!(l >= 380.0f && l <= 720.0f)) return 0.f;
    const float r = (l - 380.0f) * 0.2f;
    const int hi = int(std::ceil(r) + .5f), lo = int(std::floor(r) + .5f);
    const float w = r - float(lo);
    return t[hi] * w + t[lo] * (1.0f - w);
}

}  // namespace

plt_status spectralProfileFromSamples(const float* wl, const float* val, uint32_t count, float scale, int computeIcdf,
                                      plt_spectral_profile* sp) {
    if (!wl || !val || !sp || count == 0) return PLT_INVALID_ARG;
    for (uint32_t i = 1; i < count; ++i)
        if (!(wl[i] > wl[i - 1])) return PLT_INVALID_ARG;
    std::vector<float> w(wl, wl + count), v(val, val + count);
    for (auto& x : v) x *= scale;
    auto hlerp = [](float a, float b, float t) { return (1.f - t) * a + t * b; };
    auto pls = [&](float lambda) -> float {
        if (lambda < w.front() || lambda > w.back()) return 0.f;
        auto it = std::lower_bound(w.begin(), w.end(), lambda);
        if (it == w.begin()) return v.front();
        const size_t idx = (size_t)(it - w.begin()) - 1;
        return hlerp(v[idx], v[idx + 1], (lambda - w[idx]) / (w[idx + 1] - w[idx]));
    };
    float least = w.back() - w.front();
    for (size_t i = 1; i < w.size(); ++i) least = std::min(least, w[i] - w[i - 1]);
    const float binSize = std::max(5.f, least / 2.f);
    const float l0 = w.front(), l1 = w.back();
    const size_t ns = std::max<size_t>(1, (size_t)((l1 - l0) / binSize + .5f));
    std::vector<float> s(ns);
    for (size_t i = 0; i < ns; ++i) s[i] = pls(l0 + (l1 - l0) / float(ns - 1) * (float)i);
    auto ss = [&](float lambda) -> float {
        if (lambda < l0 || lambda > l1) return 0.f;
        const float x = ((lambda - l0) / (l1 - l0)) * (float(ns) - 1.0f);
        const size_t i = (size_t)std::floor(x);
        if (i + 1 >= ns) return s[ns - 1];
        return hlerp(s[i], s[i + 1], x - (float)i);
    };
    std::memset(sp, 0, sizeof(*sp));
    {
        // sp.rgb = toRGB_D65 of the sampled spectrum (SceneBuilder.cpp:913): trapezoid sum of
        // s * xyz * D65 over the samples, XYZ -> Rec.709 (ColorHelpers.slang:61-70), / 10567.0762.
        // The analytic CIE fit and the 380-720 nm D65 table stand in for the host's 1-nm tables.
        const float delta = ns > 1 ? (l1 - l0) / (float(ns) - 1.0f) : 0.f;
        float X = 0.f, Y = 0.f, Z = 0.f;
        for (size_t q = 0; q < ns; ++q) {
            const float l = std::min(l0 + delta * float(q), l1);
            float x, y, z;
            cieXyz(l, x, y, z);
            const float dd = d65(l);
            const float wq = ss(l) * delta * ((q == 0 || q == ns - 1) ? 0.5f : 1.0f);
            X += x * dd * wq;
            Y += y * dd * wq;
            Z += z * dd * wq;
        }
        const float k = 1.0f / 10567.0762f;
        sp->rgb[0] = (3.240969941904522f * X + -1.537383177570094f * Y + -0.4986107602930032f * Z) * k;
        sp->rgb[1] = (-0.9692436362808803f * X + 1.875967501507721f * Y + 0.04155505740717569f * Z) * k;
        sp->rgb[2] = (0.05563007969699373f * X + -0.2039769588889765f * Y + 1.056971514242878f * Z) * k;
    }
    sp->intensity = 1.f;
    sp->min_wavelength = std::max(l0, 380.0f);
    sp->max_wavelength = std::min(l1, 720.0f);
    sp->bins = std::min<uint32_t>(PLT_SPECTRAL_MAX_BINS, (uint32_t)(float(ns) * (sp->max_wavelength - sp->min_wavelength) / (l1 - l0) + .5f));
    if (sp->bins == 0) return PLT_OK;
    const float rr = sp->bins > 1 ? 1.f / float(sp->bins - 1) : 1.f;
    float sum = 0.f;
    for (uint32_t i = 0; i < sp->bins; ++i) {
        sp->pdf[i] = ss(hlerp(sp->min_wavelength, sp->max_wavelength, i * rr));
        sum += sp->pdf[i];
    }
    if (sum < 1.192092896e-07f || !computeIcdf) return PLT_OK;
    for (uint32_t i = 0; i < sp->bins; ++i) sp->pdf[i] /= sum;
    sp->intensity = sum;
    float cdfa = 0.f, cdfb = sp->pdf[0];
    for (uint32_t pdfi = 0, icdfi = 0; icdfi < sp->bins; ++icdfi) {
        const float cdf = icdfi * rr;
        while (cdf >= cdfb && pdfi + 1 < sp->bins) {
            cdfa = cdfb;
            ++pdfi;
            cdfb += sp->pdf[pdfi];
        }
        const float l = std::min(1.f, (cdf - cdfa) / (cdfb - cdfa));
        sp->icdf[icdfi] = hlerp((float)std::max<uint32_t>(1, pdfi) - 1.f, (float)pdfi, l) * rr;
    }
    return PLT_OK;
}

}  // namespace plt
