// ORACLE -- test infrastructure only.  C entry points of the CPU oracle (liboracle_plt.so), loaded
// by tests/ and by bench.py's CPU-baseline leg through ctypes.  All pointers are HOST pointers.
#include "plt_oracle.hpp"

#include <vector>
#include <string>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace plt_oracle;

namespace {

uint64_t g_sr_seed = 1;
template <class R> inline void seedQuery(uint64_t) {}
template <> inline void seedQuery<SR>(uint64_t i) { sr_seed(g_sr_seed, i); }

template <class R>
int runBatch(const plt_material_record* mats, uint32_t nm, const plt_spectral_profile* profs, uint32_t np,
             const plt_bsdf_queries* q, const plt_bsdf_results* r, uint32_t ops, int threads, int fp64ml,
             uint64_t q_begin, uint64_t q_end) {
    SceneTables sc;
    sc.profiles = profs;
    sc.count = np;
    const uint32_t n = q->n, H = q->hwss;
    if (H < 1 || H > PLT_MAX_HWSS) return PLT_INVALID_ARG;
    int bad = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256) reduction(| : bad)
#endif
    for (long long ii = (long long)q_begin; ii < (long long)q_end; ++ii) {
        const uint32_t i = (uint32_t)ii;
        seedQuery<R>(i);
        const uint32_t mid = q->material[i];
        if (mid >= nm) { bad |= 1; continue; }
        const Material<R> m = decodeMaterial<R>(mats[mid]);
        const V3<R> V = {R(q->v[i]), R(q->v[n + i]), R(q->v[2 * n + i])};
        const V3<R> W = {R(q->w[i]), R(q->w[n + i]), R(q->w[2 * n + i])};
        const uint32_t lobe = q->lobe ? q->lobe[i] : LOBE_ALL;
        Beam<R> b;
        b.H = (int)H;
        for (uint32_t c = 0; c < 4; ++c)
            for (uint32_t j = 0; j < H; ++j) b.L[c][j] = R(q->stokes[(size_t)(c * H + j) * n + i]);
        for (uint32_t j = 0; j < H; ++j) { b.wl[j] = R(q->wavelengths[(size_t)j * n + i]); b.spdf[j] = R(1); }
        for (int c = 0; c < 3; ++c) b.D[c] = R(q->coherence[(size_t)c * n + i]);
        b.r_m = R(q->coherence[(size_t)3 * n + i]);
        b.posW = {R(0), R(0), R(0)};
        b.r = -V;
        b.t = q->beam_t ? V3<R>{R(q->beam_t[i]), R(q->beam_t[n + i]), R(q->beam_t[2 * n + i])} : canonical_tangent(b.r);
        b.distant = false;
        const uint32_t j = i + q->rng_offset;
        SampleGen sg(j & 0xFFFFu, j >> 16, q->frame);
        QueryResult<R> o;
        g_fp64ConductorGrazing = (fp64ml & PLT_OPTION_FP64_CONDUCTOR_GRAZING) != 0;
        const bool ok = queryMaterial(m, sc, ops, V, W, lobe, b, &sg, o, (fp64ml & PLT_OPTION_FP64_MULTILAYER) != 0);
        g_fp64ConductorGrazing = false;
        if (!ok) { bad |= 2; continue; }
        if (ops & PLT_OP_EVAL) {
            if (r->stokes)
                for (uint32_t c = 0; c < 4; ++c)
                    for (uint32_t jj = 0; jj < H; ++jj) r->stokes[(size_t)(c * H + jj) * n + i] = o_fval(o.stokes[c][jj]);
            if (r->coherence) {
                for (int c = 0; c < 3; ++c) r->coherence[(size_t)c * n + i] = o_fval(o.D[c]);
                r->coherence[(size_t)3 * n + i] = o_fval(o.r_m);
            }
            if (r->beam_t) {
                r->beam_t[i] = o_fval(o.t.x); r->beam_t[n + i] = o_fval(o.t.y); r->beam_t[2 * n + i] = o_fval(o.t.z);
            }
        }
        if ((ops & PLT_OP_PDF) && r->pdf) r->pdf[i] = o_fval(o.pdf);
        if ((ops & PLT_OP_LAMBDA_PDF) && r->lambda_pdf)
            for (uint32_t jj = 0; jj < H; ++jj) r->lambda_pdf[(size_t)jj * n + i] = o_fval(o.lambdaPdf[jj]);
        if (ops & PLT_OP_SAMPLE) {
            if (r->sample_wo) { r->sample_wo[i] = o_fval(o.sWo.x); r->sample_wo[n + i] = o_fval(o.sWo.y); r->sample_wo[2 * n + i] = o_fval(o.sWo.z); }
            if (r->sample_pdf) r->sample_pdf[i] = o_fval(o.sPdf);
            if (r->sample_weight) r->sample_weight[i] = o_fval(o.sWeight);
            if (r->sample_lobe) r->sample_lobe[i] = o.sLobe;
            if (r->sample_valid) r->sample_valid[i] = o.sValid;
        }
    }
    if (bad & 1) return PLT_INVALID_ARG;
    if (bad & 2) return PLT_BAD_MATERIAL;
    return PLT_OK;
}

}  // namespace

extern "C" {

// Seed of the random-rounding (Monte Carlo arithmetic) build, precision code 16.
void plto_set_sr_seed(uint64_t seed) { g_sr_seed = seed; }

// precision: 32 (FP32 reference), 64 (FP64 reference), 16 (FP32 with random rounding, seeded by
// plto_set_sr_seed).  fp64_multilayer: PLT_OPTION_FP64_MULTILAYER / PLT_OPTION_FP64_CONDUCTOR_GRAZING
// bits (a non-zero value without either bit, as older callers pass, means the multilayer option).
// Processes queries [begin, end).
int plto_bsdf_batch_range(int precision, int fp64_multilayer, const plt_material_record* mats, uint32_t nm,
                          const plt_spectral_profile* profs, uint32_t np, const plt_bsdf_queries* q,
                          const plt_bsdf_results* r, uint32_t ops, int threads, uint64_t begin, uint64_t end) {
    if (!mats || !q || !r || end > q->n || begin > end) return PLT_INVALID_ARG;
    if (fp64_multilayer && !(fp64_multilayer & (PLT_OPTION_FP64_MULTILAYER | PLT_OPTION_FP64_CONDUCTOR_GRAZING)))
        fp64_multilayer = PLT_OPTION_FP64_MULTILAYER;
    if (precision == 64) return runBatch<double>(mats, nm, profs, np, q, r, ops, threads, fp64_multilayer, begin, end);
    if (precision == 16) return runBatch<SR>(mats, nm, profs, np, q, r, ops, threads, fp64_multilayer, begin, end);
    return runBatch<float>(mats, nm, profs, np, q, r, ops, threads, fp64_multilayer, begin, end);
}
int plto_bsdf_batch(int precision, int fp64_multilayer, const plt_material_record* mats, uint32_t nm,
                    const plt_spectral_profile* profs, uint32_t np, const plt_bsdf_queries* q,
                    const plt_bsdf_results* r, uint32_t ops, int threads) {
    if (!q) return PLT_INVALID_ARG;
    return plto_bsdf_batch_range(precision, fp64_multilayer, mats, nm, profs, np, q, r, ops, threads, 0, q->n);
}

// Counting build: per-material-type mean FP32-pipe ops, SFU ops and divides of the requested ops
// (material setup excluded), over queries [0, n).  out[type*4 + {0,1,2,3}] = fp, sfu, div, count.
int plto_count_ops(const plt_material_record* mats, uint32_t nm, const plt_spectral_profile* profs, uint32_t np,
                   const plt_bsdf_queries* q, uint32_t ops, double* out) {
    SceneTables sc;
    sc.profiles = profs;
    sc.count = np;
    const uint32_t n = q->n, H = q->hwss;
    for (int t = 0; t < (int)PLT_MATERIAL_TYPE_COUNT * 4; ++t) out[t] = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t mid = q->material[i];
        if (mid >= nm) return PLT_INVALID_ARG;
        const Material<CF> m = decodeMaterial<CF>(mats[mid]);
        const V3<CF> V = {CF(q->v[i]), CF(q->v[n + i]), CF(q->v[2 * n + i])};
        const V3<CF> W = {CF(q->w[i]), CF(q->w[n + i]), CF(q->w[2 * n + i])};
        const uint32_t lobe = q->lobe ? q->lobe[i] : LOBE_ALL;
        Beam<CF> b;
        b.H = (int)H;
        for (uint32_t c = 0; c < 4; ++c)
            for (uint32_t j = 0; j < H; ++j) b.L[c][j] = CF(q->stokes[(size_t)(c * H + j) * n + i]);
        for (uint32_t j = 0; j < H; ++j) { b.wl[j] = CF(q->wavelengths[(size_t)j * n + i]); b.spdf[j] = CF(1); }
        for (int c = 0; c < 3; ++c) b.D[c] = CF(q->coherence[(size_t)c * n + i]);
        b.r_m = CF(q->coherence[(size_t)3 * n + i]);
        b.r = -V;
        b.t = q->beam_t ? V3<CF>{CF(q->beam_t[i]), CF(q->beam_t[n + i]), CF(q->beam_t[2 * n + i])} : canonical_tangent(b.r);
        const uint32_t j = i + q->rng_offset;
        QueryResult<CF> o;
        // setup-only pass (ops = 0) measured and subtracted: material constants are precomputed once
        SampleGen sg0(j & 0xFFFFu, j >> 16, q->frame);
        op_counts() = OpCounts();
        queryMaterial(m, sc, 0u, V, W, lobe, b, &sg0, o);
        const OpCounts setup = op_counts();
        SampleGen sg(j & 0xFFFFu, j >> 16, q->frame);
        op_counts() = OpCounts();
        queryMaterial(m, sc, ops, V, W, lobe, b, &sg, o);
        const OpCounts all = op_counts();
        const uint32_t t = m.type < PLT_MATERIAL_TYPE_COUNT ? m.type : 0;
        out[t * 4 + 0] += (double)(all.fp - setup.fp);
        out[t * 4 + 1] += (double)(all.sfu - setup.sfu);
        out[t * 4 + 2] += (double)(all.div - setup.div);
        out[t * 4 + 3] += 1.0;
    }
    for (int t = 0; t < (int)PLT_MATERIAL_TYPE_COUNT; ++t)
        if (out[t * 4 + 3] > 0)
            for (int c = 0; c < 3; ++c) out[t * 4 + c] /= out[t * 4 + 3];
    return PLT_OK;
}

// First `count` raw 32-bit outputs of UniformSampleGenerator(pixel, sampleNumber).
void plto_rng_stream(uint32_t px, uint32_t py, uint32_t sample_number, uint32_t count, uint32_t* out) {
    SampleGen sg(px, py, sample_number);
    for (uint32_t i = 0; i < count; ++i) out[i] = sg.next();
}

// the TinyUniformSampleGenerator stream of (pixel, sample number), for tests
void plto_rng_stream_tiny(uint32_t px, uint32_t py, uint32_t sample_number, uint32_t count, uint32_t* out) {
    SampleGen sg(px, py, sample_number, true);
    for (uint32_t i = 0; i < count; ++i) out[i] = sg.next();
}

float plto_half_to_float(uint16_t h) { return half_to_float(h); }

// rgbToSpectrum (SpectrumUtils.slang:106-198) for tests
float plto_rgb_to_spectrum(float r, float g, float b, float wavelength) {
    const float rgb[3] = {r, g, b};
    return rgbToSpectrum<float>(rgb, wavelength);
}

// Fresnel helpers for known-answer tests
void plto_fresnel_dielectric(float cos_i, float eta, float* out5) {
    float rs, rp, ts, tp, ct;
    fresnel_dielectric(cos_i, eta, rs, rp, ts, tp, ct);
    out5[0] = rs; out5[1] = rp; out5[2] = ts; out5[3] = tp; out5[4] = ct;
}
void plto_fresnel_conductor(double cos_i, double n, double k, double* out4) {
    V2<double> rs, rp;
    fresnel_conductor(cos_i, V2<double>{n, k}, rs, rp);
    out4[0] = rs.x; out4[1] = rs.y; out4[2] = rp.x; out4[3] = rp.y;
}
double plto_besselj(int nu, double x) { return BesselJ(nu, x); }
void plto_diffract(float wx, float wy, float wz, int lx, int ly, float lambda_um, float inv_pitch_x, float inv_pitch_y, float* out3) {
    DiffractionGrating<float> g{};
    g.invPitch = {inv_pitch_x, inv_pitch_y};
    const V3<float> o = g.diffract(V3<float>{wx, wy, wz}, lx, ly, lambda_um);
    out3[0] = o.x; out3[1] = o.y; out3[2] = o.z;
}

// Spectral profile from piecewise-linear samples: PiecewiseLinearSpectrum::eval
// (Utils/Color/Spectrum.h:88-107), SampledSpectrum(pls, 5 nm) (SampledSpectrum.h:64-73) and
// genSpectralProfile (Scene/SceneBuilder.cpp:911-960).  rgb is left at zero (display only).
int plto_spectral_profile_from_samples(const float* wl, const float* val, uint32_t count, float scale, int compute_icdf,
                                       plt_spectral_profile* sp) {
    if (!wl || !val || !sp || count == 0) return PLT_INVALID_ARG;
    std::vector<float> w(wl, wl + count), v(val, val + count);
    for (auto& x : v) x *= scale;
    // host lerp: (1-t)*a + t*b (Utils/Math/Common.h:53-57)
    auto hlerp = [](float a, float b, float t) { return (1.f - t) * a + t * b; };
    auto pls_eval = [&](float lambda) -> float {
        if (lambda < w.front() || lambda > w.back()) return 0.f;
        auto it = std::lower_bound(w.begin(), w.end(), lambda);
        if (it == w.begin()) return v.front();
        const size_t idx = (size_t)(it - w.begin()) - 1;
        const float t = (lambda - w[idx]) / (w[idx + 1] - w[idx]);
        return hlerp(v[idx], v[idx + 1], t);
    };
    float least = w.back() - w.front();
    for (size_t i = 1; i < w.size(); ++i) least = std::min(least, w[i] - w[i - 1]);
    const float binSize = std::max(5.f, least / 2.f);
    const float l0 = w.front(), l1 = w.back();
    const size_t ns = std::max<size_t>(1, (size_t)((l1 - l0) / binSize + .5f));
    std::vector<float> samples(ns);
    for (size_t i = 0; i < ns; ++i) samples[i] = pls_eval(l0 + (l1 - l0) / float(ns - 1) * (float)i);
    auto ss_eval = [&](float lambda) -> float {
        if (lambda < l0 || lambda > l1) return 0.f;
        const float x = ((lambda - l0) / (l1 - l0)) * (float(ns) - 1.0f);
        const size_t i = (size_t)std::floor(x);
        if (i + 1 >= ns) return samples[ns - 1];
        const float ww = x - (float)i;
        return hlerp(samples[i], samples[i + 1], ww);
    };
    std::memset(sp, 0, sizeof(*sp));
    profileRgb(l0, l1, ns, ss_eval, sp->rgb);
    sp->intensity = 1.f;
    sp->min_wavelength = std::max(l0, SPEC_MIN_WL);
    sp->max_wavelength = std::min(l1, SPEC_MAX_WL);
    sp->bins = std::min<uint32_t>(PLT_SPECTRAL_MAX_BINS,
                                  (uint32_t)(float(ns) * (sp->max_wavelength - sp->min_wavelength) / (l1 - l0) + .5f));
    if (sp->bins == 0) return PLT_OK;
    const float rr = sp->bins > 1 ? 1.f / float(sp->bins - 1) : 1.f;
    float sum = 0.f;
    for (uint32_t i = 0; i < sp->bins; ++i) {
        const float lam = hlerp(sp->min_wavelength, sp->max_wavelength, i * rr);
        sp->pdf[i] = ss_eval(lam);
        sum += sp->pdf[i];
    }
    if (sum < K_FLT_EPSILON || !compute_icdf) return PLT_OK;
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
        const float lo = (float)std::max<uint32_t>(1, pdfi) - 1.f, hi = (float)pdfi;
        sp->icdf[icdfi] = hlerp(lo, hi, l) * rr;
    }
    return PLT_OK;
}

}  // extern "C"
