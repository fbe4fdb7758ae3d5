// Host-side input and output of the render pass: the .spd spectral-table loader feeding
// genSpectralProfile, and an OpenEXR writer for the accumulated image (the reference's pass graph
// ends in AccumulatePass and an EXR capture, scripts/PLTPathTracer.py:19-27).  Paths cited are
// inside ssteinberg/PLTFalcor.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "plt_context.h"

namespace {

// PiecewiseLinearSpectrum::fromFile (Source/Falcor/Utils/Color/Spectrum.cpp:89-111): '#' lines and
// blank lines are skipped; reading stops at the first line that does not start with two numbers.
bool parseSpd(const char* path, std::vector<float>& wl, std::vector<float>& val) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::string line;
    char buf[4096];
    bool more = true;
    while (more && std::fgets(buf, sizeof(buf), f)) {
        line = buf;
        size_t a = line.find_first_not_of(" \t\r\n");
        if (a == std::string::npos) continue;
        if (line[a] == '#') continue;
        const char* p = line.c_str() + a;
        char* e1 = nullptr;
        const double x = std::strtod(p, &e1);
        if (e1 == p) { more = false; break; }
        char* e2 = nullptr;
        const double y = std::strtod(e1, &e2);
        if (e2 == e1) { more = false; break; }
        wl.push_back((float)x);
        val.push_back((float)y);
    }
    std::fclose(f);
    return true;
}

void put32(std::vector<unsigned char>& o, uint32_t v) {
    for (int i = 0; i < 4; ++i) o.push_back((unsigned char)(v >> (8 * i)));
}
void put64(std::vector<unsigned char>& o, uint64_t v) {
    for (int i = 0; i < 8; ++i) o.push_back((unsigned char)(v >> (8 * i)));
}
void putStr(std::vector<unsigned char>& o, const char* s) {
    while (*s) o.push_back((unsigned char)*s++);
    o.push_back(0);
}
void putF32(std::vector<unsigned char>& o, float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    put32(o, u);
}
// an attribute: name, type, byte size, value
void attr(std::vector<unsigned char>& o, const char* name, const char* type, const std::vector<unsigned char>& value) {
    putStr(o, name);
    putStr(o, type);
    put32(o, (uint32_t)value.size());
    o.insert(o.end(), value.begin(), value.end());
}
uint16_t floatToHalf(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const int32_t e = (int32_t)((x >> 23) & 0xFF) - 127 + 15;
    uint32_t m = x & 0x7FFFFFu;
    if (((x >> 23) & 0xFF) == 0xFF) return (uint16_t)(sign | 0x7C00u | (m ? 0x200u : 0u));
    if (e >= 31) return (uint16_t)(sign | 0x7C00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        m |= 0x800000u;
        const int shift = 14 - e;
        uint32_t hm = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (hm & 1u))) ++hm;
        return (uint16_t)(sign | hm);
    }
    uint32_t h = ((uint32_t)e << 10) | (m >> 13);
    const uint32_t rem = m & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}

}  // namespace

extern "C" {

plt_status plt_spectral_profile_from_spd(const char* path, float scale, int compute_icdf, plt_spectral_profile* out) {
    if (!path || !out) return PLT_INVALID_ARG;
    std::vector<float> wl, val;
    if (!parseSpd(path, wl, val)) return PLT_INVALID_ARG;
    if (wl.size() < 2) return PLT_INVALID_ARG;
    return plt_spectral_profile_from_samples(wl.data(), val.data(), (uint32_t)wl.size(), scale, compute_icdf, out);
}

// SceneBuilder::addSpectralProfileFromMaterial (Scene/SceneBuilder.cpp:967-976): the real and
// imaginary IOR tables <tables>/ior/<name>.eta.spd and .k.spd, without inverse CDFs; "none" is the
// constant one-sample spectra n = 1, k = 0 over 380-720 nm.
plt_status plt_spectral_profiles_from_material(const char* tables_dir, const char* name, plt_spectral_profile* eta,
                                               plt_spectral_profile* k) {
    if (!tables_dir || !name || !eta || !k) return PLT_INVALID_ARG;
    if (std::strcmp(name, "none") == 0) {
        const float wl[2] = {380.0f, 720.0f};
        for (int i = 0; i < 2; ++i) {
            const float v[2] = {i == 0 ? 1.f : 0.f, i == 0 ? 1.f : 0.f};
            plt_spectral_profile* out = i == 0 ? eta : k;
            const plt_status s = plt_spectral_profile_from_samples(wl, v, 2, 1.f, 0, out);
            if (s != PLT_OK) return s;
            out->bins = 1;   // SampledSpectrum(value) holds one sample
            for (uint32_t b = 1; b < PLT_SPECTRAL_MAX_BINS; ++b) out->pdf[b] = 0.f;
            out->intensity = 1.f;
        }
        return PLT_OK;
    }
    const std::string base = std::string(tables_dir) + "/ior/" + name;
    const plt_status s = plt_spectral_profile_from_spd((base + ".eta.spd").c_str(), 1.f, 0, eta);
    if (s != PLT_OK) return s;
    return plt_spectral_profile_from_spd((base + ".k.spd").c_str(), 1.f, 0, k);
}

// SceneBuilder::addSpectralProfileForEmitterType (Scene/SceneBuilder.cpp:978-993): the emission
// table <tables>/emission/<name>.spd scaled by `scale`, with its inverse CDF.
plt_status plt_spectral_profile_for_emitter_type(const char* tables_dir, const char* name, float scale, plt_spectral_profile* out) {
    if (!tables_dir || !name || !out) return PLT_INVALID_ARG;
    const std::string path = std::string(tables_dir) + "/emission/" + name + ".spd";
    return plt_spectral_profile_from_spd(path.c_str(), scale, 1, out);
}

// OpenEXR 2 single-part scanline image, no compression, channels A, B, G, R (alphabetical, as the
// format requires), HALF or FLOAT; rgba is [height][width][4] on the host.
plt_status plt_write_exr(const char* path, const float* rgba, uint32_t width, uint32_t height, int half) {
    if (!path || !rgba || width == 0 || height == 0 || width > (1u << 20) || height > (1u << 20)) return PLT_INVALID_ARG;
    const uint32_t ptype = half ? 1u : 2u, bpc = half ? 2u : 4u;
    std::vector<unsigned char> o;
    put32(o, 20000630u);   // magic 0x762f3101
    put32(o, 2u);          // version 2, single-part scanline
    {
        std::vector<unsigned char> ch;
        for (const char* name : {"A", "B", "G", "R"}) {
            putStr(ch, name);
            put32(ch, ptype);
            ch.push_back(0);   // pLinear
            ch.push_back(0);
            ch.push_back(0);
            ch.push_back(0);
            put32(ch, 1u);     // x sampling
            put32(ch, 1u);     // y sampling
        }
        ch.push_back(0);
        attr(o, "channels", "chlist", ch);
    }
    attr(o, "compression", "compression", {0});
    std::vector<unsigned char> box;
    put32(box, 0u);
    put32(box, 0u);
    put32(box, width - 1);
    put32(box, height - 1);
    attr(o, "dataWindow", "box2i", box);
    attr(o, "displayWindow", "box2i", box);
    attr(o, "lineOrder", "lineOrder", {0});
    std::vector<unsigned char> v;
    putF32(v, 1.f);
    attr(o, "pixelAspectRatio", "float", v);
    v.clear();
    putF32(v, 0.f);
    putF32(v, 0.f);
    attr(o, "screenWindowCenter", "v2f", v);
    v.clear();
    putF32(v, 1.f);
    attr(o, "screenWindowWidth", "float", v);
    o.push_back(0);   // end of header
    const uint64_t rowBytes = 4ull * width * bpc;
    const uint64_t tableEnd = o.size() + 8ull * height;
    for (uint32_t y = 0; y < height; ++y) put64(o, tableEnd + (uint64_t)y * (8 + rowBytes));
    const int chanOfName[4] = {3, 2, 1, 0};   // A, B, G, R from RGBA
    for (uint32_t y = 0; y < height; ++y) {
        put32(o, y);
        put32(o, (uint32_t)rowBytes);
        for (int c = 0; c < 4; ++c)
            for (uint32_t x = 0; x < width; ++x) {
                const float f = rgba[(4ull * ((uint64_t)y * width + x)) + chanOfName[c]];
                if (half) {
                    const uint16_t h = floatToHalf(f);
                    o.push_back((unsigned char)(h & 0xFF));
                    o.push_back((unsigned char)(h >> 8));
                } else {
                    putF32(o, f);
                }
            }
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return PLT_INVALID_ARG;
    const size_t w = std::fwrite(o.data(), 1, o.size(), f);
    const int closed = std::fclose(f);
    return (w == o.size() && closed == 0) ? PLT_OK : PLT_INVALID_ARG;
}

}  // extern "C"
