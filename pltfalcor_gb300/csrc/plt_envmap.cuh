// The environment light on the device: the lat-long map's evaluation (Scene/Lights/EnvMap.slang),
// the equal-area octahedral mapping and lat-long conversions (Utils/Math/MathHelpers.slang:106-128,
// 199-244), the hierarchical importance sampler and its pdf (Rendering/Lights/EnvMapSampler.slang),
// and rgbToSpectrum (Utils/Color/SpectrumUtils.slang:171-198).  Paths cited are inside
// ssteinberg/PLTFalcor.
//
// Texture filtering is restated in arithmetic: the map's sampler is bilinear with U wrapped and V
// clamped (EnvMap.cpp:123-126), the importance map's point-sampled with clamping
// (EnvMapSampler.cpp:75-76).  Filter weights are full FP32 (texture units quantise them).
#pragma once

#include "plt_device_math.cuh"
#include "plt_internal.h"

namespace pltdev {

constexpr float k2_Pi = 0.636619772367581343076f;    // M_2_PI
constexpr float kPi_4 = 0.785398163397448309616f;    // M_PI_4
constexpr float k1_4Pi = 0.0795774715459476678844f;  // M_1_4PI

// ndir_to_oct_equal_area_unorm, MathHelpers.slang:199-219
PLT_DI f2 ndirToOctEqualAreaUnorm(f3 n) {
    const float r = sqrtf(1.f - fabsf(n.z));
    const float phi = atan2f(fabsf(n.y), fabsf(n.x));
    f2 p;
    p.y = r * phi * k2_Pi;
    p.x = r - p.y;
    if (n.z < 0.f) p = f2{1.f - p.y, 1.f - p.x};
    p.x *= signf(n.x);
    p.y *= signf(n.y);
    return f2{p.x * 0.5f + 0.5f, p.y * 0.5f + 0.5f};
}
// oct_to_ndir_equal_area_unorm, MathHelpers.slang:225-244
PLT_DI f3 octToNdirEqualAreaUnorm(f2 u) {
    const f2 p{u.x * 2.f - 1.f, u.y * 2.f - 1.f};
    const float d = 1.f - (fabsf(p.x) + fabsf(p.y));
    const float r = 1.f - fabsf(d);
    const float phi = (r > 0.f) ? ((fabsf(p.y) - fabsf(p.x)) / r + 1.f) * kPi_4 : 0.f;
    const float f = r * sqrtf(2.f - r * r);
    const float x = f * signf(p.x) * cosf(phi);
    const float y = f * signf(p.y) * sinf(phi);
    const float z = signf(d) * (1.f - r * r);
    return mk3(x, y, z);
}
// world_to_latlong_map, MathHelpers.slang:106-113 (the map is centred on -z)
PLT_DI f2 worldToLatlong(f3 dir) {
    const f3 p = dir / sqrtf(dot(dir, dir));
    return f2{atan2f(p.x, -p.z) * k1_2Pi + 0.5f, acosf(p.y) * k1_Pi};
}
PLT_DI f3 mat3mul(const float* M, f3 v) {
    return mk3(M[0] * v.x + M[1] * v.y + M[2] * v.z, M[3] * v.x + M[4] * v.y + M[5] * v.z, M[6] * v.x + M[7] * v.y + M[8] * v.z);
}

// luminance, Utils/Color/ColorHelpers.slang (Rec.709 weights)
PLT_DI float luminanceRgb(float r, float g, float b) { return r * 0.2126f + g * 0.7152f + b * 0.0722f; }

// bilinear lookup of the raw map (no intensity): texel centres at (i + 0.5) / dim
PLT_DI f3 envTexBilinear(const plt::EnvDev& E, f2 uv) {
    const float x = uv.x * (float)E.width - 0.5f, y = uv.y * (float)E.height - 0.5f;
    const float fx0 = floorf(x), fy0 = floorf(y);
    const float fx = x - fx0, fy = y - fy0;
    const int W = (int)E.width, Hh = (int)E.height;
    int x0 = (int)fx0 % W;
    if (x0 < 0) x0 += W;
    const int x1 = (x0 + 1 == W) ? 0 : x0 + 1;
    const int y0 = min(max((int)fy0, 0), Hh - 1), y1 = min(max((int)fy0 + 1, 0), Hh - 1);
    const float4 a = __ldg(E.tex + (size_t)y0 * W + x0), b = __ldg(E.tex + (size_t)y0 * W + x1);
    const float4 c = __ldg(E.tex + (size_t)y1 * W + x0), d = __ldg(E.tex + (size_t)y1 * W + x1);
    const float w00 = (1.f - fx) * (1.f - fy), w10 = fx * (1.f - fy), w01 = (1.f - fx) * fy, w11 = fx * fy;
    return mk3(w00 * a.x + w10 * b.x + w01 * c.x + w11 * d.x, w00 * a.y + w10 * b.y + w01 * c.y + w11 * d.y,
               w00 * a.z + w10 * b.z + w01 * c.z + w11 * d.z);
}
// EnvMap.eval(dir): the map at worldToUv(dir) x intensity x tint
PLT_DI f3 envEval(const plt::EnvDev& E, f3 dirW) {
    const f3 c = envTexBilinear(E, worldToLatlong(mat3mul(E.toLocal, dirW)));
    return mk3(c.x * E.scale[0], c.y * E.scale[1], c.z * E.scale[2]);
}

PLT_DI float envImp(const plt::EnvDev& E, uint32_t mip, uint32_t x, uint32_t y) {
    return __ldg(E.imp + E.mipOff[mip] + (size_t)y * (E.impDim >> mip) + x);
}

// EnvMapSampler.sample, EnvMapSampler.slang:52-113: descend the mip chain from the 1x1 level,
// warping the random pair at each 2x2 choice; returns the world direction and its solid-angle pdf.
PLT_DI f3 envSampleDir(const plt::EnvDev& E, float ux, float uy, float& pdf) {
    float px = ux, py = uy;
    uint32_t posx = 0, posy = 0;
    for (int mip = (int)E.impBaseMip - 1; mip >= 0; --mip) {
        posx *= 2u;
        posy *= 2u;
        const float w0 = envImp(E, mip, posx, posy), w1 = envImp(E, mip, posx + 1, posy);
        const float w2 = envImp(E, mip, posx, posy + 1), w3 = envImp(E, mip, posx + 1, posy + 1);
        const float q0 = w0 + w2, q1 = w1 + w3;
        const float d = q0 / (q0 + q1);
        uint32_t offx, offy;
        if (px < d) { offx = 0; px = px / d; }
        else { offx = 1; px = (px - d) / (1.f - d); }
        const float e = offx == 0 ? (w0 / q0) : (w1 / q1);
        if (py < e) { offy = 0; py = py / e; }
        else { offy = 1; py = (py - e) / (1.f - e); }
        posx += offx;
        posy += offy;
    }
    const float inv = 1.f / (float)E.impDim;
    const f2 uv{((float)posx + px) * inv, ((float)posy + py) * inv};
    const f3 dir = octToNdirEqualAreaUnorm(uv);
    const float avgW = envImp(E, E.impBaseMip, 0, 0);
    pdf = (envImp(E, 0, posx, posy) / avgW) * k1_4Pi;
    return mat3mul(E.toWorld, dir);
}
// EnvMapSampler.evalPdf, EnvMapSampler.slang:121-127 (point sample, clamped)
PLT_DI float envEvalPdf(const plt::EnvDev& E, f3 dirW) {
    const f2 uv = ndirToOctEqualAreaUnorm(mat3mul(E.toLocal, dirW));
    const int dim = (int)E.impDim;
    const int x = min(max((int)floorf(uv.x * (float)dim), 0), dim - 1);
    const int y = min(max((int)floorf(uv.y * (float)dim), 0), dim - 1);
    const float avgW = envImp(E, E.impBaseMip, 0, 0);
    return (envImp(E, 0, x, y) / avgW) * (1.f / 12.5663706143591729539f);
}

// SpectrumUtils.rgbToSpectrum(float3, wavelength): the piecewise-constant 11-bin basis of white,
// cyan, magenta, yellow, red, green and blue, combined by the smallest channel
static __constant__ float kRgbBasis[7][11] = {
    {1.0000f, 1.0000f, 0.9999f, 0.9993f, 0.9992f, 0.9998f, 1.0000f, 1.0000f, 1.0000f, 1.0000f, 0.0f},
    {0.9710f, 0.9426f, 1.0007f, 1.0007f, 1.0007f, 1.0007f, 0.1564f, 0.0000f, 0.0000f, 0.0000f, 0.0f},
    {1.0000f, 1.0000f, 0.968f, 0.22295f, 0.0000f, 0.0458f, 0.8369f, 1.0000f, 1.0000f, 0.9959f, 0.0f},
    {0.0001f, 0.0000f, 0.1088f, 0.6651f, 1.0000f, 1.0000f, 0.9996f, 0.9586f, 0.9685f, 0.9840f, 0.0f},
    {0.1012f, 0.0515f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.8325f, 1.0149f, 1.0149f, 1.014f, 0.0f},
    {0.0000f, 0.0000f, 0.0273f, 0.7937f, 1.0000f, 0.9418f, 0.1719f, 0.0000f, 0.0000f, 0.0025f, 0.0f},
    {1.0000f, 1.0000f, 0.8916f, 0.3323f, 0.0000f, 0.0000f, 0.0003f, 0.0369f, 0.0483f, 0.0496f, 0.0f}};
PLT_DI float rgbToSpectrumAt(f3 rgb, float wl) {
    const int b = spectrumBin(wl);
    const float white = kRgbBasis[0][b], cyan = kRgbBasis[1][b], magenta = kRgbBasis[2][b], yellow = kRgbBasis[3][b];
    const float red = kRgbBasis[4][b], green = kRgbBasis[5][b], blue = kRgbBasis[6][b];
    float sd = 0.f;
    if (rgb.x <= rgb.y && rgb.x <= rgb.z) {
        sd += white * rgb.x;
        if (rgb.y <= rgb.z) { sd += cyan * (rgb.y - rgb.x); sd += blue * (rgb.z - rgb.y); }
        else { sd += cyan * (rgb.z - rgb.x); sd += green * (rgb.y - rgb.z); }
    } else if (rgb.y <= rgb.x && rgb.y <= rgb.z) {
        sd += white * rgb.y;
        if (rgb.x <= rgb.z) { sd += magenta * (rgb.x - rgb.y); sd += blue * (rgb.z - rgb.x); }
        else { sd += magenta * (rgb.z - rgb.y); sd += red * (rgb.x - rgb.z); }
    } else {
        sd += white * rgb.z;
        if (rgb.x <= rgb.y) { sd += yellow * (rgb.x - rgb.z); sd += green * (rgb.y - rgb.x); }
        else { sd += yellow * (rgb.y - rgb.z); sd += red * (rgb.x - rgb.y); }
    }
    return sd;
}

}  // namespace pltdev
