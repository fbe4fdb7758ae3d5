// Oracle (test infrastructure only): CPU restatement of the environment light for the render
// oracle -- EnvMap's evaluation (Scene/Lights/EnvMap.slang, EnvMap.cpp:60-126), the importance map
// (EnvMapSamplerSetup.cs.slang, EnvMapSampler.cpp:85-120) and the sampler
// (Rendering/Lights/EnvMapSampler.slang), with the lat-long and equal-area octahedral mappings of
// Utils/Math/MathHelpers.slang:106-128, 199-244.  Paths cited are inside ssteinberg/PLTFalcor.
//
// Texture filtering is restated in arithmetic: bilinear, U wrapped, V clamped for the map; point,
// clamped for the importance map; the mips are 2 x 2 box averages.
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

#include "plt_oracle_geom.hpp"

namespace plt_oracle_env {

struct EnvMap {
    bool present = false;
    uint32_t width = 0, height = 0;
    std::vector<float> rgb;                 // [height][width][3]
    float scale[3] = {1.f, 1.f, 1.f};       // intensity * tint
    float toWorld[9], toLocal[9];
    uint32_t dim = 512, baseMip = 9;
    std::vector<std::vector<float>> imp;    // mip chain, level 0 = dim x dim

    static void mul(const float* M, const float v[3], float out[3]) {
        out[0] = M[0] * v[0] + M[1] * v[1] + M[2] * v[2];
        out[1] = M[3] * v[0] + M[4] * v[1] + M[5] * v[2];
        out[2] = M[6] * v[0] + M[7] * v[1] + M[8] * v[2];
    }
    // EnvMap::setRotation: eulerAngleXYZ = Rx(x) Ry(y) Rz(z); toLocal = its inverse (transpose)
    void setRotation(const float deg[3]) {
        const float k = 3.14159265358979323846f / 180.f;
        const float a = deg[0] * k, b = deg[1] * k, c = deg[2] * k;
        const float ca = std::cos(a), sa = std::sin(a), cb = std::cos(b), sb = std::sin(b), cc = std::cos(c), sc = std::sin(c);
        const float M[9] = {cb * cc, -cb * sc, sb,
                            ca * sc + sa * sb * cc, ca * cc - sa * sb * sc, -sa * cb,
                            sa * sc - ca * sb * cc, sa * cc + ca * sb * sc, ca * cb};
        for (int r = 0; r < 3; ++r)
            for (int q = 0; q < 3; ++q) {
                toWorld[3 * r + q] = M[3 * r + q];
                toLocal[3 * r + q] = M[3 * q + r];
            }
    }
    // world_to_latlong_map
    static void latlong(const float d[3], float uv[2]) {
        const float len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        const float p[3] = {d[0] / len, d[1] / len, d[2] / len};
        uv[0] = std::atan2(p[0], -p[2]) * 0.159154943091895335769f + 0.5f;
        uv[1] = std::acos(p[1]) * 0.318309886183790671538f;
    }
    // the map without intensity, bilinear (texel centres at (i + 0.5) / dim)
    void texel(float u, float v, float out[3]) const {
        const float x = u * (float)width - 0.5f, y = v * (float)height - 0.5f;
        const float fx0 = std::floor(x), fy0 = std::floor(y);
        const float fx = x - fx0, fy = y - fy0;
        const int W = (int)width, Hh = (int)height;
        int x0 = (int)fx0 % W;
        if (x0 < 0) x0 += W;
        const int x1 = (x0 + 1 == W) ? 0 : x0 + 1;
        const int y0 = std::min(std::max((int)fy0, 0), Hh - 1), y1 = std::min(std::max((int)fy0 + 1, 0), Hh - 1);
        const float* a = &rgb[3 * ((size_t)y0 * W + x0)];
        const float* b = &rgb[3 * ((size_t)y0 * W + x1)];
        const float* c = &rgb[3 * ((size_t)y1 * W + x0)];
        const float* d = &rgb[3 * ((size_t)y1 * W + x1)];
        const float w00 = (1.f - fx) * (1.f - fy), w10 = fx * (1.f - fy), w01 = (1.f - fx) * fy, w11 = fx * fy;
        for (int k = 0; k < 3; ++k) out[k] = w00 * a[k] + w10 * b[k] + w01 * c[k] + w11 * d[k];
    }
    // EnvMap.eval(dir)
    void eval(const float dirW[3], float out[3]) const {
        float l[3], uv[2];
        mul(toLocal, dirW, l);
        latlong(l, uv);
        texel(uv[0], uv[1], out);
        for (int k = 0; k < 3; ++k) out[k] *= scale[k];
    }
    static void octUnormToDir(float u, float v, float n[3]) {
        const float p[2] = {u * 2.f - 1.f, v * 2.f - 1.f};
        plt_oracle::geom::octToNdirEqualArea(p, n);
    }
    // EnvMapSamplerSetup: luminance averaged over 8 x 8 subsamples per texel, then the mips
    void buildImportance() {
        imp.clear();
        std::vector<float> base((size_t)dim * dim);
        const uint32_t S = 8;
        const float invDimS = 1.f / (float)(dim * S);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)dim * dim; ++i) {
            const uint32_t px = (uint32_t)(i % dim), py = (uint32_t)(i / dim);
            float L = 0.f;
            for (uint32_t y = 0; y < S; ++y)
                for (uint32_t x = 0; x < S; ++x) {
                    float n[3], uv[2], c[3];
                    octUnormToDir(((float)(px * S + x) + 0.5f) * invDimS, ((float)(py * S + y) + 0.5f) * invDimS, n);
                    latlong(n, uv);
                    texel(uv[0], uv[1], c);
                    L += c[0] * 0.2126f + c[1] * 0.7152f + c[2] * 0.0722f;
                }
            base[i] = L * (1.f / (float)(S * S));
        }
        imp.push_back(std::move(base));
        for (uint32_t d = dim / 2; d >= 1; d /= 2) {
            const std::vector<float>& s = imp.back();
            std::vector<float> t((size_t)d * d);
            const uint32_t sd = 2 * d;
            for (uint32_t y = 0; y < d; ++y)
                for (uint32_t x = 0; x < d; ++x) {
                    const float a = s[(2 * y) * sd + 2 * x], b = s[(2 * y) * sd + 2 * x + 1];
                    const float c = s[(2 * y + 1) * sd + 2 * x], e = s[(2 * y + 1) * sd + 2 * x + 1];
                    t[(size_t)y * d + x] = ((a + b) + (c + e)) * 0.25f;
                }
            imp.push_back(std::move(t));
        }
        baseMip = (uint32_t)imp.size() - 1;
    }
    float at(uint32_t mip, uint32_t x, uint32_t y) const { return imp[mip][(size_t)y * (dim >> mip) + x]; }
    // EnvMapSampler.sample: the world direction and its solid-angle pdf
    void sample(float ux, float uy, float dirW[3], float& pdf) const {
        float px = ux, py = uy;
        uint32_t posx = 0, posy = 0;
        for (int mip = (int)baseMip - 1; mip >= 0; --mip) {
            posx *= 2u;
            posy *= 2u;
            const float w0 = at(mip, posx, posy), w1 = at(mip, posx + 1, posy);
            const float w2 = at(mip, posx, posy + 1), w3 = at(mip, posx + 1, posy + 1);
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
        const float inv = 1.f / (float)dim;
        float n[3];
        octUnormToDir(((float)posx + px) * inv, ((float)posy + py) * inv, n);
        pdf = (at(0, posx, posy) / at(baseMip, 0, 0)) * 0.0795774715459476678844f;   // M_1_4PI
        mul(toWorld, n, dirW);
    }
    // EnvMapSampler.evalPdf
    float evalPdf(const float dirW[3]) const {
        float l[3], p[2];
        mul(toLocal, dirW, l);
        plt_oracle::geom::ndirToOctEqualArea(l, p);
        const float u = p[0] * 0.5f + 0.5f, v = p[1] * 0.5f + 0.5f;
        const int D = (int)dim;
        const int x = std::min(std::max((int)std::floor(u * (float)D), 0), D - 1);
        const int y = std::min(std::max((int)std::floor(v * (float)D), 0), D - 1);
        return (at(0, x, y) / at(baseMip, 0, 0)) * (1.f / 12.5663706143591729539f);
    }
};

}  // namespace plt_oracle_env
