// ORACLE -- test infrastructure only.  PLT BxDFs, material decode and the IMaterialInstance
// wrappers, restated from Source/Falcor/Rendering/Materials/PLT/*.slang (citations per block).
#pragma once

namespace plt_oracle {

constexpr uint32_t LOBE_ALL = 0xFFFFu;
constexpr uint32_t LOBE_DIFFUSE_REFLECTION = 0x01u, LOBE_SCATTER_REFLECTION = 0x02u, LOBE_DELTA_REFLECTION = 0x04u,
                   LOBE_DISPERSIVE_DELTA_REFLECTION = 0x08u, LOBE_SCATTER_TRANSMISSION = 0x20u,
                   LOBE_DELTA_TRANSMISSION = 0x40u, LOBE_DISPERSIVE_DELTA_TRANSMISSION = 0x80u, LOBE_DELTA = 0xCCu,
                   LOBE_NON_DELTA = 0x33u, LOBE_REFLECTION = 0x0Fu, LOBE_TRANSMISSION = 0xF0u;

// ---------------------------------------------------------------------------------------------
// Decoded material (setupMaterialInstance of each PLT*Material.slang, textures at their constants)
// ---------------------------------------------------------------------------------------------
template <class R> struct Material {
    uint32_t type = 0;
    R base[4], spec[4], data1[4], data2[4], tran[3], ior;
    uint16_t data1w_bits = 0;
    uint32_t etaN = PLT_NO_SPECTRAL_PROFILE, etaK = PLT_NO_SPECTRAL_PROFILE, emission = PLT_NO_SPECTRAL_PROFILE;
};
template <class R> inline Material<R> decodeMaterial(const plt_material_record& m) {
    Material<R> d;
    d.type = m.type;
    for (int i = 0; i < 4; ++i) {
        d.base[i] = R(half_to_float(m.base_color[i]));
        d.spec[i] = R(half_to_float(m.specular[i]));
        d.data1[i] = R(half_to_float(m.data1[i]));
        d.data2[i] = R(half_to_float(m.data2[i]));
    }
    for (int i = 0; i < 3; ++i) d.tran[i] = R(half_to_float(m.transmission[i]));
    d.ior = R(half_to_float(m.ior));
    d.data1w_bits = m.data1[3];
    d.etaN = m.ior_n_spectral_id;
    d.etaK = m.ior_k_spectral_id;
    d.emission = m.emission_spectral_id;
    return d;
}

template <class R> inline V3<R> reflectLocal(V3<R> wi) { return {-wi.x, -wi.y, wi.z}; }
template <class R> inline M2<R> scatterCoherenceTransform(V3<R> wo, bool isDirect) {
    // coherenceTransform of the rough BxDFs (e.g. PLTDielectricBSDF.slang:272-278)
    const R c = o_sqrt(o_max(R(1e-2), o_abs(wo.z)));
    return isDirect ? ident2<R>() : m2(c, R(0), R(0), R(1) / c);
}
template <class R> inline void kOf(const Beam<R>& b, R* k) { for (int j = 0; j < b.H; ++j) k[j] = R(K_2PI) / (R(1e-3) * b.wl[j]); }

// =============================================================================================
// PLTDielectric, PLTDielectricBSDF.slang:43-279, PLTDielectricMaterial.slang:40-57
// =============================================================================================
template <class R> struct Dielectric {
    R specular[3], transmission[3];
    GaussianSurface<R> gfs;
    R etaInt, etaExt, dispersionB;
    explicit Dielectric(const Material<R>& m) : gfs(m.spec[1]) {
        for (int i = 0; i < 3; ++i) { specular[i] = m.base[i]; transmission[i] = m.tran[i]; }
        etaExt = m.spec[3];
        const bool anyT = m.tran[0] > R(0) || m.tran[1] > R(0) || m.tran[2] > R(0);
        dispersionB = anyT ? m.spec[0] : R(0);
        etaInt = o_max(R(1), m.ior - R(2.897) * dispersionB);
    }
    R ior(R k) const { return (etaInt + dispersionB * sqr(k * R(K_1_2PI))) / etaExt; }
    bool isDispersive() const { return dispersionB != R(0); }
    static V3<R> refract(V3<R> wi, R cosThetaT, R eta) {
        const R scale = cosThetaT < R(0) ? R(1) / eta : eta;
        return {-scale * wi.x, -scale * wi.y, cosThetaT};
    }
    static V3<R> scattered_wo(V3<R> wo, R eta) {
        const R scale = wo.z > R(0) ? R(1) / eta : eta;
        const V2<R> xy = {wo.x * scale, wo.y * scale};
        const R l2 = dot(xy, xy);
        if (l2 > R(1)) return {R(0), R(0), R(0)};
        return {xy.x, xy.y, -o_sign(wo.z) * o_sqrt(o_max(R(0), R(1) - l2))};
    }
    void eval(V3<R> toLight, V3<R> toEye, uint32_t lobe, Beam<R>& beam) const {
        const bool isReflection = toLight.z * toEye.z > R(0);
        const bool isScatter = (lobe & LOBE_NON_DELTA) != 0;
        const bool isDirect = (lobe & LOBE_DELTA) != 0;
        const bool hasTransmission = (lobe & LOBE_TRANSMISSION) != 0;
        const bool hasReflection = (lobe & LOBE_REFLECTION) != 0;
        if (toLight.z * toEye.z == R(0) || (!isScatter && !isDirect) || (!hasTransmission && !isReflection) ||
            (!hasReflection && isReflection)) {
            beam.setZero();
            return;
        }
        R k[MAXH], m00[MAXH], eta[MAXH], relEta2[MAXH], a[MAXH];
        kOf(beam, k);
        for (int j = 0; j < beam.H; ++j) {
            m00[j] = isReflection ? rgbToSpectrum(specular, beam.wl[j]) : rgbToSpectrum(transmission, beam.wl[j]);
            eta[j] = ior(k[j]);
            relEta2[j] = sqr(toEye.z > R(0) ? eta[j] : R(1) / eta[j]);
        }
        const V3<R> toEyeUp = isReflection ? toEye : scattered_wo(toEye, eta[0]);
        const V3<R> toLightBeam = beam.toLocal(toLight);
        for (int j = 0; j < beam.H; ++j) a[j] = gfs.alpha(toLight, toEyeUp, k[j]);
        if (isScatter) {
            const V3<R> h = toLight + toEyeUp;
            const V3<R> m = normalize(h);
            const R LdotH = o_max(R(0), dot(toLight, m));
            const M2<R> Q = beam.Q();
            const M2<R> invTheta = beam.invTheta(R(1));
            for (int j = 0; j < beam.H; ++j) {
                const V4<R> SP = beam.getSP(j);
                const R J = isReflection ? R(1) : relEta2[j];
                const R D = gfs.eval(k[j], invTheta, Q, h);
                const M4<R> M1 = MuellerFresnelDielectric(o_sign(toLight.z) * LdotH, eta[j], isReflection);
                beam.setSP(j, (m00[j] * (R(1) - a[j]) * J * o_abs(toLight.z) * D) * mul(M1, SP));
            }
        } else {
            for (int j = 0; j < beam.H; ++j) {
                const V4<R> SP = beam.getSP(j);
                const R J = isReflection ? R(1) : relEta2[j];
                const M4<R> M0 = MuellerFresnelDielectric(toLight.z, eta[j], isReflection);
                R coh = R(1);
                if (!isReflection) {
                    R cosThetaT;
                    evalFresnelDielectric(eta[j], toEye.z, cosThetaT);
                    const V3<R> lobeWo = beam.toLocal(refract(toEye, cosThetaT, eta[j]));
                    coh = j == 0 ? R(1) : beam.mutualCoherenceAngular(lobeWo, toLightBeam);
                }
                beam.setSP(j, (m00[j] * a[j] * coh * J) * mul(M0, SP));
            }
        }
    }
    bool sample(V3<R> wi, V3<R>& wo, R& pdf, R& weight, uint32_t& lobe, SampleGen& sg, R wavelength, uint32_t lobeMask) const {
        const R k = R(K_2PI) / (R(1e-3) * wavelength);
        const R a = gfs.alpha(wi, k);
        const R eta = ior(k);
        const bool hasReflection = (lobeMask & LOBE_REFLECTION) != 0;
        const bool hasTransmission = (lobeMask & LOBE_TRANSMISSION) != 0;
        const bool hasDirect = (lobeMask & LOBE_DELTA) != 0;
        const bool hasScatter = (lobeMask & LOBE_NON_DELTA) != 0;
        if ((!hasReflection && !hasTransmission) || (!hasDirect && !hasScatter)) return false;
        const R pdfDirect = hasDirect && hasScatter ? a : hasDirect ? R(1) : R(0);
        bool isReflection;
        const bool isDirect = pdfDirect == R(1) || next1D<R>(sg) < pdfDirect;
        pdf = (hasDirect && hasScatter) ? (isDirect ? pdfDirect : R(1) - pdfDirect) : R(1);
        if (isDirect) {
            R cosThetaT;
            const R Fd = evalFresnelDielectric(eta, wi.z, cosThetaT);
            isReflection = hasReflection ? (Fd > R(0) && next1D<R>(sg) <= Fd) : false;
            wo = isReflection ? reflectLocal(wi) : refract(wi, cosThetaT, eta);
            pdf = pdf * ((hasReflection && hasTransmission) ? (isReflection ? Fd : R(1) - Fd) : R(1));
            lobe = isReflection ? LOBE_DELTA_REFLECTION : (isDispersive() ? LOBE_DISPERSIVE_DELTA_TRANSMISSION : LOBE_DELTA_TRANSMISSION);
        } else {
            R surfPdf;
            wo = gfs.sample(wi, sg, k, surfPdf);
            pdf = pdf * surfPdf;
            const V3<R> h = wi + wo;
            const V3<R> m = normalize(h);
            const R F = evalFresnelDielectric(eta, o_sign(wi.z) * dot(wi, m));
            isReflection = hasReflection ? (F > R(0) && next1D<R>(sg) <= F) : false;
            if (!isReflection) wo = scattered_wo(wo, eta);
            pdf = pdf * ((hasReflection && hasTransmission) ? (isReflection ? F : R(1) - F) : R(1));
            lobe = isReflection ? LOBE_SCATTER_REFLECTION : LOBE_SCATTER_TRANSMISSION;
        }
        weight = isReflection ? rgbToSpectrum(specular, wavelength) : rgbToSpectrum(transmission, wavelength);
        return (isReflection && wi.z * wo.z <= R(0)) ? false : (!isReflection && wi.z * wo.z >= R(0)) ? false : true;
    }
    R pdf(V3<R> wi, V3<R> woL, R wavelength) const {
        const R k = R(K_2PI) / (R(1e-3) * wavelength);
        const R a = gfs.alpha(wi, k);
        const R eta = ior(k);
        const R pdfDirect = a;
        const bool isReflection = wi.z * woL.z > R(0);
        const V3<R> wo = isReflection ? woL : scattered_wo(woL, eta);
        const V3<R> h = wi + wo;
        const V3<R> m = normalize(h);
        const R F = evalFresnelDielectric(eta, o_sign(wi.z) * dot(wi, m));
        const R pdfF = isReflection ? F : R(1) - F;
        return (R(1) - pdfDirect) * pdfF * gfs.pdf(wi, wo, k);
    }
    void lambdaPdf(V3<R> toLight, V3<R> toEye, uint32_t lobe, const Beam<R>& beam, R* out) const {
        const bool isReflection = toLight.z * toEye.z > R(0);
        const bool isScatter = (lobe & LOBE_NON_DELTA) != 0;
        const bool isDirect = (lobe & LOBE_DELTA) != 0;
        R k[MAXH];
        kOf(beam, k);
        const V3<R> toLightBeam = beam.toLocal(toLight);
        if (isDirect && !isReflection) {
            for (int j = 0; j < beam.H; ++j) {
                const R eta = ior(k[j]);
                R cosThetaT;
                evalFresnelDielectric(eta, toEye.z, cosThetaT);
                const V3<R> lobeWo = beam.toLocal(refract(toEye, cosThetaT, eta));
                out[j] = j == 0 ? R(1) : beam.mutualCoherenceAngular(lobeWo, toLightBeam);
            }
            return;
        }
        if (isScatter) {
            for (int j = 0; j < beam.H; ++j) {
                const R eta = ior(k[j]);
                const V3<R> wo = isReflection ? toLight : scattered_wo(toLight, eta);
                out[j] = gfs.pdf(toEye, wo, k[j]);
            }
            return;
        }
        for (int j = 0; j < beam.H; ++j) out[j] = R(1);
    }
    M2<R> coherenceTransform(V3<R>, V3<R> wo, uint32_t lobe) const { return scatterCoherenceTransform(wo, (lobe & LOBE_DELTA) != 0); }
};

// =============================================================================================
// PLTConductor, PLTConductorBSDF.slang:44-173, PLTConductorMaterial.slang:40-57
// =============================================================================================
template <class R> struct Conductor {
    R specular[3];
    FractalSurface<R> gfs;
    uint32_t etaN, etaK;
    R extEta;
    const SceneTables* sc;
    Conductor(const Material<R>& m, const SceneTables* s, bool gammaFromSpec = true)
        : gfs(gammaFromSpec ? FractalSurface<R>(m.spec[1], m.spec[0]) : FractalSurface<R>(m.data2[1])),
          etaN(m.etaN), etaK(m.etaK), extEta(m.ior), sc(s) {
        for (int i = 0; i < 3; ++i) specular[i] = m.base[i];
    }
    V2<R> iorAt(R wl) const { return {evalSpectrum(*sc, etaN, wl) / extEta, evalSpectrum(*sc, etaK, wl) / extEta}; }
    void eval(V3<R> toLight, V3<R> toEye, uint32_t lobe, Beam<R>& beam) const {
        const bool isScatter = (lobe & LOBE_SCATTER_REFLECTION) != 0;
        const bool isDirect = (lobe & LOBE_DELTA_REFLECTION) != 0;
        const bool hasReflection = (lobe & LOBE_REFLECTION) != 0;
        if ((!isScatter && !isDirect) || !hasReflection) { beam.setZero(); return; }
        R k[MAXH];
        kOf(beam, k);
        const V3<R> h = toLight + toEye;
        const V3<R> m = normalize(h);
        const R LdotH = o_max(R(0), dot(toLight, m));
        for (int j = 0; j < beam.H; ++j) {
            const R a = gfs.alpha(toLight, toEye, k[j]);
            const R m00 = rgbToSpectrum(specular, beam.wl[j]);
            const V4<R> SP = beam.getSP(j);
            const V2<R> ior = {evalSpectrum(*sc, etaN, beam.wl[j]) / extEta, evalSpectrum(*sc, etaK, beam.wl[j]) / extEta};
            V4<R> newSP;
            if (isScatter) {
                const M4<R> M1 = MuellerFresnelRConductor(LdotH, ior);
                const R D = gfs.eval(k[j], h);
                newSP = ((R(1) - a) * o_abs(toLight.z) * D) * mul(M1, SP);
            } else {
                const M4<R> M0 = MuellerFresnelRConductor(toLight.z, ior);
                newSP = a * mul(M0, SP);
            }
            beam.setSP(j, newSP * m00);
        }
    }
    bool sample(V3<R> wi, V3<R>& wo, R& pdf, R& weight, uint32_t& lobe, SampleGen& sg, R wavelength, uint32_t lobeMask) const {
        const bool hasReflection = (lobeMask & LOBE_REFLECTION) != 0;
        const bool hasDirect = (lobeMask & LOBE_DELTA) != 0;
        const bool hasScatter = (lobeMask & LOBE_NON_DELTA) != 0;
        if (!hasReflection || (!hasDirect && !hasScatter)) return false;
        const R k = R(K_2PI) / (R(1e-3) * wavelength);
        const R a = gfs.alpha(wi, k);
        const R m00 = rgbToSpectrum(specular, wavelength);
        pdf = R(1);
        bool isDirect = hasDirect;
        if (hasDirect && hasScatter) {
            const R pdfDirect = a;
            isDirect = pdfDirect == R(1) || next1D<R>(sg) < pdfDirect;
            pdf = isDirect ? pdfDirect : R(1) - pdfDirect;
        }
        weight = m00;
        if (isDirect) {
            wo = reflectLocal(wi);
            lobe = LOBE_DELTA_REFLECTION;
        } else {
            R surfPdf;
            wo = gfs.sample(wi, sg, k, surfPdf);
            pdf = pdf * surfPdf;
            lobe = LOBE_SCATTER_REFLECTION;
        }
        return true;
    }
    R pdf(V3<R> wi, V3<R> wo, R wavelength) const {
        const R k = R(K_2PI) / (R(1e-3) * wavelength);
        const R a = gfs.alpha(wi, k);
        return (R(1) - a) * gfs.pdf(wi, wo, k);
    }
    R weight(R wavelength) const { return rgbToSpectrum(specular, wavelength); }
    void lambdaPdf(V3<R> toLight, V3<R> toEye, uint32_t lobe, const Beam<R>& beam, R* out) const {
        const bool isScatter = (lobe & LOBE_NON_DELTA) != 0;
        R k[MAXH];
        kOf(beam, k);
        for (int j = 0; j < beam.H; ++j) out[j] = isScatter ? gfs.pdf(toEye, toLight, k[j]) : R(1);
    }
    M2<R> coherenceTransform(V3<R>, V3<R> wo, uint32_t lobe) const { return scatterCoherenceTransform(wo, (lobe & LOBE_DELTA) != 0); }
};

// =============================================================================================
// PLTOpaqueDielectric (base of the grated dielectric), PLTOpaqueDielectricBSDF.slang:43-147
// =============================================================================================
template <class R> struct OpaqueDielectric {
    R albedo[3];
    FractalSurface<R> gfs;
    explicit OpaqueDielectric(const Material<R>& m, bool fromData2 = false) : gfs(fromData2 ? m.data2[1] : m.spec[1]) {
        for (int i = 0; i < 3; ++i) albedo[i] = m.base[i];
    }
    void eval(V3<R> toLight, V3<R> toEye, uint32_t lobe, Beam<R>& beam) const {
        const bool hasReflection = (lobe & LOBE_REFLECTION) != 0;
        const bool isDirect = (lobe & LOBE_DELTA) != 0;
        const bool isScatter = (lobe & LOBE_NON_DELTA) != 0;
        if ((!isScatter && !isDirect) || !hasReflection) { beam.setZero(); return; }
        const R mk = meank<R>();
        const R a = gfs.alpha(toLight, toEye, mk);
        R M = a;
        if (isScatter) {
            const V3<R> h = toLight + toEye;
            const R D = gfs.eval(mk, h);
            M = (R(1) - a) * o_abs(toLight.z) * D;
        }
        for (int j = 0; j < beam.H; ++j) {
            const R m00 = rgbToSpectrum(albedo, beam.wl[j]);
            beam.setSP(j, (M * m00) * beam.getSP(j));
        }
    }
    bool sample(V3<R> wi, V3<R>& wo, R& pdf, R& weight, uint32_t& lobe, SampleGen& sg, R wavelength, uint32_t lobeMask) const {
        const bool hasReflection = (lobeMask & LOBE_REFLECTION) != 0;
        const bool hasDirect = (lobeMask & LOBE_DELTA) != 0;
        const bool hasScatter = (lobeMask & LOBE_NON_DELTA) != 0;
        if (!hasReflection || (!hasDirect && !hasScatter)) return false;
        const R mk = meank<R>();
        const R a = gfs.alpha(wi, mk);
        const R m00 = rgbToSpectrum(albedo, wavelength);
        pdf = R(1);
        bool isDirect = hasDirect;
        if (hasDirect && hasScatter) {
            isDirect = a == R(1) || next1D<R>(sg) < a;
            pdf = isDirect ? a : R(1) - a;
        }
        weight = m00;
        if (isDirect) {
            wo = reflectLocal(wi);
            lobe = LOBE_DELTA_REFLECTION;
        } else {
            R surfPdf;
            wo = gfs.sample(wi, sg, mk, surfPdf);
            pdf = pdf * surfPdf;
            lobe = LOBE_SCATTER_REFLECTION;
        }
        return true;
    }
    R pdf(V3<R> wi, V3<R> wo, R) const {
        const R mk = meank<R>();
        const R a = gfs.alpha(wi, mk);
        return (R(1) - a) * gfs.pdf(wi, wo, mk);
    }
    R weight(R wavelength) const { return rgbToSpectrum(albedo, wavelength); }
    void lambdaPdf(V3<R>, V3<R>, uint32_t, const Beam<R>& beam, R* out) const { for (int j = 0; j < beam.H; ++j) out[j] = R(1); }
    M2<R> coherenceTransform(V3<R>, V3<R> wo, uint32_t lobe) const { return scatterCoherenceTransform(wo, (lobe & LOBE_DELTA) != 0); }
};

// =============================================================================================
// Coated BxDFs: PLTCoatedOpaqueDielectricBSDF.slang:45-245 (+Material :40-60) and
// PLTCoatedConductorBSDF.slang:45-246 (+Material :40-60).  CONDUCTOR selects the base.
// =============================================================================================
template <class R, bool CONDUCTOR> struct Coated {
    R albedo[3];
    FractalSurface<R> gfs;
    uint32_t etaN, etaK;
    R extEta, coatIOR, tau;
    const SceneTables* sc;
    Coated(const Material<R>& m, const SceneTables* s) : gfs(m.spec[1]), etaN(m.etaN), etaK(m.etaK), sc(s) {
        for (int i = 0; i < 3; ++i) albedo[i] = m.base[i];
        extEta = m.ior;
        tau = m.data1[0] * m.spec[2];
        coatIOR = m.data1[3];
    }
    static V3<R> refractCoat(V3<R> wi, R eta, R cosThetaT) {
        const R scale = cosThetaT < R(0) ? R(1) / eta : eta;
        return {-scale * wi.x, -scale * wi.y, cosThetaT};
    }
    R coatEta() const {
        const R minTau = R(0.05);
        return lerp(extEta, coatIOR, o_clamp(tau, R(0), minTau) / minTau);
    }
    void eval(V3<R> toLight, V3<R> toEye, uint32_t lobe, Beam<R>& beam) const {
        const bool isReflection = toLight.z * toEye.z > R(0);
        const bool isScatter = (lobe & LOBE_SCATTER_REFLECTION) != 0;
        const bool isDirect = (lobe & LOBE_DELTA_REFLECTION) != 0;
        const R coatior = coatEta();
        const R eta1 = coatior / extEta;
        R cosThetaTin;
        evalFresnelDielectric(eta1, toLight.z, cosThetaTin);
        const V3<R> wiIn = -refractCoat(toLight, eta1, cosThetaTin);
        V3<R> woIn = reflectLocal(wiIn);
        if (!isDirect) {
            R cosThetaTout;
            evalFresnelDielectric(eta1, toEye.z, cosThetaTout);
            woIn = -refractCoat(toEye, eta1, cosThetaTout);
        }
        if (!isReflection || (!isScatter && !isDirect) || wiIn.z <= R(0) || woIn.z <= R(0)) { beam.setZero(); return; }
        R k[MAXH], mc[MAXH];
        kOf(beam, k);
        const V3<R> h = wiIn + woIn;
        const V3<R> m = normalize(h);
        const R LdotH = o_max(R(0), dot(wiIn, m));
        const V3<R> Z = beam.toLocal(V3<R>{R(0), R(0), R(1)});
        beam.mutualCoherenceH(k, Z * tau, mc);
        const M4<R> MiT = MuellerFresnelTDielectric(toLight.z, eta1);
        const M4<R> MoT = MuellerFresnelTDielectric(-woIn.z, eta1);
        if (!CONDUCTOR) {
            const M4<R> M = mul(MiT, MoT);
            for (int j = 0; j < beam.H; ++j) {
                const R a = gfs.alpha(wiIn, woIn, k[j]);
                const R m00 = rgbToSpectrum(albedo, beam.wl[j]);
                const R phase = phaseShiftH(coatior, R(2) * tau / wiIn.z, k[j]);
                const V4<R> SP = beam.getSP(j);
                V4<R> newSP = m00 * mul(M, SP);
                V4<R> SPreflcoat;
                if (isScatter) {
                    const M4<R> MiR = MuellerFresnelRDielectric(LdotH, eta1);
                    const R D = gfs.eval(k[j], h);
                    newSP = newSP * ((R(1) - a) * o_abs(toLight.z) * D);
                    SPreflcoat = ((R(1) - a) * o_abs(toLight.z) * D) * mul(MiR, SP);
                } else {
                    const M4<R> MiR = MuellerFresnelRDielectric(toLight.z, eta1);
                    newSP = newSP * a;
                    SPreflcoat = a * mul(MiR, SP);
                }
                beam.setSP(j, interfere(newSP, SPreflcoat, phase, phase, mc[j]));
            }
        } else {
            const M4<R> MiR = MuellerFresnelRDielectric(toLight.z, eta1);
            for (int j = 0; j < beam.H; ++j) {
                const R a = gfs.alpha(wiIn, woIn, k[j]);
                const R m00 = rgbToSpectrum(albedo, beam.wl[j]);
                V2<R> rs, rp;
                const V2<R> ior = {evalSpectrum(*sc, etaN, beam.wl[j]) / coatior, evalSpectrum(*sc, etaK, beam.wl[j]) / coatior};
                const M4<R> M2R = MuellerFresnelRConductor(LdotH, ior, rs, rp);
                const M4<R> M = mul(mul(MiT, M2R), MoT);
                const V4<R> SP = beam.getSP(j);
                V4<R> newSP = m00 * mul(M, SP);
                if (isScatter) {
                    const R D = gfs.eval(k[j], h);
                    newSP = newSP * ((R(1) - a) * o_abs(toLight.z) * D);
                } else {
                    const R pS = phaseShift(coatior, R(2) * tau / wiIn.z, k[j], rs);
                    const R pP = phaseShift(coatior, R(2) * tau / wiIn.z, k[j], rp);
                    newSP = interfere(a * newSP, mul(MiR, SP), pS, pP, mc[j]);
                }
                beam.setSP(j, newSP);
            }
        }
    }
    bool sample(V3<R> wi, V3<R>& wo, R& pdf, R& weight, uint32_t& lobe, SampleGen& sg, R wavelength, uint32_t lobeMask) const {
        const bool hasReflection = (lobeMask & LOBE_REFLECTION) != 0;
        const bool hasDirect = (lobeMask & LOBE_DELTA) != 0;
        const bool hasScatter = (lobeMask & LOBE_NON_DELTA) != 0;
        if (!hasReflection || (!hasDirect && !hasScatter) || wi.z <= R(0)) return false;
        const R k = R(K_2PI) / (R(1e-3) * wavelength);
        const R eta1 = coatEta() / extEta;
        R cosThetaT;
        const R Fd = evalFresnelDielectric(eta1, wi.z, cosThetaT);
        // "Fd == .1f" as written in the reference (PLTCoated*BSDF.slang:150-151)
        const bool isReflCoat = Fd == R(0.1f) || next1D<R>(sg) < Fd;
        weight = R(1);
        pdf = isReflCoat ? Fd : R(1) - Fd;
        if (isReflCoat) {
            wo = reflectLocal(wi);
            lobe = LOBE_DELTA_REFLECTION;
            return true;
        }
        const V3<R> wiIn = -refractCoat(wi, eta1, cosThetaT);
        if (wiIn.z == R(0)) return false;
        weight = rgbToSpectrum(albedo, wavelength);
        const R a = gfs.alpha(wiIn, k);
        const R pdfDirect = hasDirect && hasScatter ? a : hasDirect ? R(1) : R(0);
        const bool isDirect = pdfDirect == R(1) || next1D<R>(sg) < pdfDirect;
        if (hasDirect && hasScatter) pdf = pdf * (isDirect ? pdfDirect : R(1) - pdfDirect);
        if (isDirect) {
            wo = reflectLocal(wi);
            lobe = LOBE_DELTA_REFLECTION;
        } else {
            R surfPdf;
            const V3<R> woIn = gfs.sample(wiIn, sg, k, surfPdf);
            pdf = pdf * surfPdf;
            R cosThetaT1;
            evalFresnelDielectric(eta1, -woIn.z, cosThetaT1);
            wo = refractCoat(-woIn, eta1, cosThetaT1);
            lobe = LOBE_SCATTER_REFLECTION;
        }
        return wi.z * wo.z > R(0);
    }
    R pdf(V3<R> wi, V3<R> wo, R wavelength) const {
        if (wi.z <= R(0) || wo.z <= R(0)) return R(0);
        const R k = R(K_2PI) / (R(1e-3) * wavelength);
        const R eta1 = coatEta() / extEta;
        R cosThetaT, cosThetaT1;
        const R Fd = evalFresnelDielectric(eta1, wi.z, cosThetaT);
        evalFresnelDielectric(eta1, wo.z, cosThetaT1);
        const V3<R> wiIn = -refractCoat(wi, eta1, cosThetaT);
        const V3<R> woIn = -refractCoat(wo, eta1, cosThetaT1);
        const R a = gfs.alpha(wiIn, k);
        return wiIn.z * woIn.z == R(0) ? R(0) : (R(1) - a) * (R(1) - Fd) * gfs.pdf(wiIn, woIn, k);
    }
    void lambdaPdf(V3<R> toLight, V3<R> toEye, uint32_t lobe, const Beam<R>& beam, R* out) const {
        const bool isScatter = (lobe & LOBE_NON_DELTA) != 0;
        R k[MAXH];
        kOf(beam, k);
        const R eta1 = coatEta() / extEta;
        if (isScatter) {
            R cosThetaT, cosThetaT1;
            evalFresnelDielectric(eta1, toEye.z, cosThetaT);
            evalFresnelDielectric(eta1, toLight.z, cosThetaT1);
            const V3<R> wiIn = -refractCoat(toEye, eta1, cosThetaT);
            const V3<R> woIn = -refractCoat(toLight, eta1, cosThetaT1);
            for (int j = 0; j < beam.H; ++j) out[j] = gfs.pdf(wiIn, woIn, k[j]);
            return;
        }
        for (int j = 0; j < beam.H; ++j) out[j] = R(1);
    }
    M2<R> coherenceTransform(V3<R>, V3<R> wo, uint32_t lobe) const { return scatterCoherenceTransform(wo, (lobe & LOBE_DELTA) != 0); }
};

// =============================================================================================
// Diffraction-grated BxDFs: PLTDiffractionGratedOpaqueDielectricBSDF.slang:45-209 and
// PLTDiffractionGratedConductorBSDF.slang:45-213; setup in the matching *Material.slang.
// =============================================================================================
template <class R> inline DiffractionGrating<R> makeGrating(const Material<R>& m) {
    DiffractionGrating<R> g;
    const R pitchx = m.data1[0], pitchy = m.data1[1];
    g.invPitch = {pitchx > R(0) ? R(1) / pitchx : R(0), pitchy > R(0) ? R(1) / pitchy : R(0)};
    const R qscale = m.spec[0];
    g.q = m.data2[0] * qscale;
    g.intensityMultiplier = m.spec[1];
    const uint16_t tl = m.data1w_bits;
    g.lobeCount = std::min(std::max((unsigned)(tl & 0xFFu), 1u), 8u);
    g.type = (unsigned)(tl >> 8);
    const R dir = m.data1[2];
    g.gratingX = {o_cos(dir), o_sin(dir)};
    return g;
}
template <class R, bool CONDUCTOR> struct Grated {
    OpaqueDielectric<R> baseD;
    Conductor<R> baseC;
    DiffractionGrating<R> grating;
    Grated(const Material<R>& m, const SceneTables* s) : baseD(m, true), baseC(m, s, false), grating(makeGrating(m)) {}
    void eval(V3<R> toLight, V3<R> toEye, uint32_t bsdfLobe, Beam<R>& beam) const {
        const bool isDirect = (bsdfLobe & LOBE_DELTA) != 0;
        R lambdas[MAXH], k[MAXH], a[MAXH];
        bool anyPos = false, anyLt1 = false;
        for (int j = 0; j < beam.H; ++j) {
            lambdas[j] = R(1e-3) * beam.wl[j];
            k[j] = R(K_2PI) / lambdas[j];
            a[j] = grating.alpha(toLight, k[j]);
            anyPos = anyPos || a[j] > R(0);
            anyLt1 = anyLt1 || a[j] < R(1);
        }
        int lx, ly;
        decodeGratingLobe(bsdfLobe, lx, ly);
        const V3<R> toLightBeam = beam.toLocal(toLight);
        if (lx == 0 && ly == 0 && anyPos) {
            if (CONDUCTOR) baseC.eval(toLight, toEye, bsdfLobe, beam);
            else baseD.eval(toLight, toEye, bsdfLobe, beam);
            beam.scale(a);
        } else if ((lx != 0 || ly != 0) && anyLt1 && isDirect) {
            for (int j = 0; j < beam.H; ++j) {
                const V3<R> lobeWi = beam.toLocal(grating.diffract(toEye, lx, ly, lambdas[j]));
                const R coh = j == 0 ? R(1) : beam.mutualCoherenceAngular(lobeWi, toLightBeam);
                const R intensity = grating.lobeIntensity(lx, ly, toLight, lambdas[j]);
                if (CONDUCTOR) {
                    const R m00 = rgbToSpectrum(baseC.specular, beam.wl[j]);
                    const M4<R> M0 = MuellerFresnelRConductor(toLight.z, baseC.iorAt(beam.wl[j]));
                    beam.setSP(j, (m00 * (R(1) - a[j]) * coh * intensity) * mul(M0, beam.getSP(j)));
                } else {
                    const R m00 = rgbToSpectrum(baseD.albedo, beam.wl[j]);
                    beam.setSP(j, (m00 * (R(1) - a[j]) * coh * intensity) * beam.getSP(j));
                }
            }
        } else {
            beam.setZero();
        }
    }
    bool sample(V3<R> wi, V3<R>& wo, R& pdf, R& weight, uint32_t& bsdfLobe, SampleGen& sg, R wavelength, uint32_t lobeMask) const {
        const bool hasReflection = (lobeMask & LOBE_REFLECTION) != 0;
        const bool hasDirect = (lobeMask & LOBE_DELTA) != 0;
        const bool hasScatter = (lobeMask & LOBE_NON_DELTA) != 0;
        if (!hasReflection || (!hasDirect && !hasScatter)) return false;
        const R lambda = R(1e-3) * wavelength;
        const R k = R(K_2PI) / lambda;
        const R a = grating.alpha(wi, k);
        // No woHint in the batch API: hasHint = false.
        bool isDirect = hasDirect;
        if (hasDirect && hasScatter) {
            isDirect = a == R(1) || next1D<R>(sg) < a;
            pdf = isDirect ? a : R(1) - a;
        }
        if (isDirect) {
            R basePdf;
            if (CONDUCTOR) baseC.sample(wi, wo, basePdf, weight, bsdfLobe, sg, wavelength, lobeMask);
            else baseD.sample(wi, wo, basePdf, weight, bsdfLobe, sg, wavelength, lobeMask);
            pdf = pdf * basePdf;
            return true;
        }
        weight = CONDUCTOR ? baseC.weight(wavelength) : baseD.weight(wavelength);
        V2<R> lobePdf = {R(1), R(1)};
        int lx = 0, ly = 0;
        grating.sampleLobe(wi, lx, ly, lobePdf, lambda, sg);
        wo = grating.diffract(wi, lx, ly, lambda);
        bsdfLobe = LOBE_DISPERSIVE_DELTA_REFLECTION;
        encodeGratingLobe(lx, ly, bsdfLobe);
        pdf = pdf * (lobePdf.x * lobePdf.y);
        return true;
    }
    // sample with a direction hint (manifold walks), PLTDiffractionGrated*BSDF.slang:109-161
    bool sampleHint(V3<R> wi, V3<R>& wo, R& pdf, R& weight, uint32_t& bsdfLobe, SampleGen& sg, R wavelength, uint32_t lobeMask,
                    V3<R> woHint) const {
        const bool hasReflection = (lobeMask & LOBE_REFLECTION) != 0;
        const bool hasDirect = (lobeMask & LOBE_DELTA) != 0;
        const bool hasScatter = (lobeMask & LOBE_NON_DELTA) != 0;
        if (!hasReflection || (!hasDirect && !hasScatter)) return false;
        const R lambda = R(1e-3) * wavelength;
        const R k = R(K_2PI) / lambda;
        const R a = grating.alpha(wi, k);
        const bool hasHint = hasDirect && (woHint.x != R(0) || woHint.y != R(0) || woHint.z != R(0));
        int lx = 0, ly = 0;
        if (hasHint && a < R(1)) grating.closestLobeHint(wi, woHint, a, lambda, lx, ly);
        bool isDirect = hasDirect;
        if (hasHint) {
            isDirect = lx == 0 && ly == 0;
            pdf = R(1);
        } else if (hasDirect && hasScatter) {
            isDirect = a == R(1) || next1D<R>(sg) < a;
            pdf = isDirect ? a : R(1) - a;
        }
        if (isDirect) {
            R basePdf;
            if (CONDUCTOR) baseC.sample(wi, wo, basePdf, weight, bsdfLobe, sg, wavelength, lobeMask);
            else baseD.sample(wi, wo, basePdf, weight, bsdfLobe, sg, wavelength, lobeMask);
            pdf = pdf * basePdf;
            return true;
        }
        weight = CONDUCTOR ? baseC.weight(wavelength) : baseD.weight(wavelength);
        V2<R> lobePdf = {R(1), R(1)};
        if (!hasHint) grating.sampleLobe(wi, lx, ly, lobePdf, lambda, sg);
        wo = grating.diffract(wi, lx, ly, lambda);
        bsdfLobe = LOBE_DISPERSIVE_DELTA_REFLECTION;
        encodeGratingLobe(lx, ly, bsdfLobe);
        pdf = pdf * (lobePdf.x * lobePdf.y);
        return true;
    }
    R pdf(V3<R> wi, V3<R> wo, R wavelength) const {
        const R k = R(K_2PI) / (R(1e-3) * wavelength);
        const R a = grating.alpha(wi, k);
        return (CONDUCTOR ? baseC.pdf(wi, wo, wavelength) : baseD.pdf(wi, wo, wavelength)) * a;
    }
    void lambdaPdf(V3<R> toLight, V3<R> toEye, uint32_t bsdfLobe, const Beam<R>& beam, R* out) const {
        const bool isDirect = (bsdfLobe & LOBE_DELTA) != 0;
        R lambdas[MAXH], a[MAXH];
        bool anyLt1 = false;
        for (int j = 0; j < beam.H; ++j) {
            lambdas[j] = R(1e-3) * beam.wl[j];
            a[j] = grating.alpha(toLight, R(K_2PI) / lambdas[j]);
            anyLt1 = anyLt1 || a[j] < R(1);
        }
        int lx, ly;
        decodeGratingLobe(bsdfLobe, lx, ly);
        const V3<R> toLightBeam = beam.toLocal(toLight);
        if ((lx != 0 || ly != 0) && anyLt1 && isDirect) {
            for (int j = 0; j < beam.H; ++j) {
                const V3<R> lobeWi = beam.toLocal(grating.diffract(toEye, lx, ly, lambdas[j]));
                out[j] = j == 0 ? R(1) : beam.mutualCoherenceAngular(lobeWi, toLightBeam);
            }
            return;
        }
        for (int j = 0; j < beam.H; ++j) out[j] = R(1);
    }
    M2<R> coherenceTransform(V3<R> wi, V3<R> wo, uint32_t bsdfLobe) const {
        int lx, ly;
        decodeGratingLobe(bsdfLobe, lx, ly);
        if (lx == 0 && ly == 0) return CONDUCTOR ? baseC.coherenceTransform(wi, wo, bsdfLobe) : baseD.coherenceTransform(wi, wo, bsdfLobe);
        return ident2<R>();
    }
};

// =============================================================================================
// PLTThinDielectric (birefringent), PLTThinDielectricBSDF.slang:43-200, Material :40-54
// =============================================================================================
template <class R> struct ThinDielectric {
    V2<R> opticAxis_xy;
    R etaAvg, tau, birefringence;
    explicit ThinDielectric(const Material<R>& m) {
        opticAxis_xy = {m.base[1], m.base[2]};
        etaAvg = m.ior;
        tau = m.spec[3];
        birefringence = m.base[0] * m.spec[0];
    }
    V3<R> opticAxis() const {
        const R z = o_sqrt(o_max(R(0), R(1) - dot(opticAxis_xy, opticAxis_xy)));
        return {opticAxis_xy.x, opticAxis_xy.y, z};
    }
    void handle_birefringence(Beam<R>& beam, V3<R> wi, const R* k) const {
        using B = Biref<R>;
        const V3<R> OA = opticAxis();
        const R phii = o_atan2(wi.y, wi.x);
        const R phiA = o_atan2(OA.y, OA.x) - phii;
        const V3<R> I = {R(0), o_abs(wi.z), o_sqrt(R(1) - sqr(wi.z))};
        V3<R> A = {o_cos(phiA), R(0), o_sin(phiA)};
        A = A * o_sqrt(R(1) - sqr(OA.z));
        A.y = o_sign(wi.z) * OA.z;
        const V3<R> A2 = {A.x, -A.y, A.z};
        const V3<R> Z = beam.toLocal(V3<R>{o_cos(phii), o_sin(phii), R(0)});
        const R ei = R(1);
        const R eo = etaAvg - R(0.5) * birefringence;
        const R ee = etaAvg + R(0.5) * birefringence;
        const R tauum = tau * R(1e+3);
        V3<R> Io, Io2, Ie, Ie2;
        R e_eff, e_eff2;
        B::vectors_in_slab(I, ei, eo, ee, A, Io, Io2, Ie, Ie2, e_eff, e_eff2);
        R rss, rsp, tso, tse, rps, rpp, tpo, tpe, roo, roe, tos, top, reo, ree, tes, tep;
        B::fresnel_iso_aniso(I.y, I.z, ei, eo, ee, A, rss, rsp, tso, tse, rps, rpp, tpo, tpe);
        B::fresnel_aniso_iso(I.y, I.z, ei, eo, ee, A2, roo, roe, tos, top, reo, ree, tes, tep);
        const R ss = tso * tos + tse * tes;
        const R sp = tso * top + tse * tep;
        const R ps = tpo * tos + tpe * tes;
        const R pp = tpo * top + tpe * tep;
        const R Ioz = o_abs(tauum / Io.y) * Io.z;
        const R Iez = o_abs(tauum / Ie.y) * Ie.z;
        const R OPLo = o_abs(tauum / Io.y) * eo;
        const R OPLe = o_abs(tauum / Ie.y) * e_eff;
        const R oez = Ioz - Iez;
        R mc[MAXH];
        beam.mutualCoherenceH(k, Z * oez, mc);
        R nLx[MAXH], nLy[MAXH], newL[MAXH];
        bool allFinite = true, allPos = true;
        for (int j = 0; j < beam.H; ++j) {
            const R t = mc[j] * R(2) * o_sin(-k[j] * (ei * oez * I.z + OPLo - OPLe));
            const R Lx = R(0.5) * (beam.L[0][j] + beam.L[1][j]);
            const R Ly = R(0.5) * (beam.L[0][j] - beam.L[1][j]);
            const R sqrtLxLy = o_sqrt(Lx * Ly);
            nLx[j] = o_max(R(0), sqr(ss) * Lx + sqr(ps) * Ly + ss * ps * t * sqrtLxLy);
            nLy[j] = o_max(R(0), sqr(sp) * Lx + sqr(pp) * Ly + sp * pp * t * sqrtLxLy);
            newL[j] = nLx[j] + nLy[j];
            allFinite = allFinite && o_isfinite(newL[j]);
            allPos = allPos && beam.L[0][j] > R(1e-6);
        }
        for (int j = 0; j < beam.H; ++j) {
            const R norm = (allPos && allFinite) ? newL[j] / beam.L[0][j] : R(0);
            beam.L[0][j] = allFinite ? newL[j] : R(0);
            beam.L[1][j] = allFinite ? nLx[j] - nLy[j] : R(0);
            beam.L[2][j] *= norm;
            beam.L[3][j] *= norm;
        }
    }
    void eval(V3<R> toLight, V3<R> toEye, uint32_t lobe, Beam<R>& beam) const {
        const R eta = etaAvg / R(1);
        const bool isReflection = toLight.z * toEye.z > R(0);
        const bool isDirect = (lobe & LOBE_DELTA) != 0;
        const bool hasTransmission = (lobe & LOBE_TRANSMISSION) != 0;
        const bool hasReflection = (lobe & LOBE_REFLECTION) != 0;
        if ((isReflection && eta == R(1)) || toLight.z * toEye.z == R(0) || !isDirect || (!hasTransmission && !isReflection) ||
            (!hasReflection && isReflection)) {
            beam.setZero();
            return;
        }
        R k[MAXH];
        kOf(beam, k);
        const R ci = o_abs(toLight.z);
        const M4<R> Rm = MuellerFresnelRDielectric(ci, eta);
        const M4<R> iR = invOneMinusMuellerFresnelRDielectric(ci, eta);
        const M4<R> T = MuellerFresnelTDielectric(ci, eta);
        const M4<R> M = isReflection ? (iR.m[0][0] > R(0) ? Rm + mul(mul(T, Rm), mul(iR, T)) : Rm)
                                     : (iR.m[0][0] > R(0) ? mul(T, mul(iR, T)) : mul(T, T));
        if (birefringence > R(0) && !isReflection) handle_birefringence(beam, toLight, k);
        for (int j = 0; j < beam.H; ++j) beam.setSP(j, mul(M, beam.getSP(j)));
    }
    bool sample(V3<R> wi, V3<R>& wo, R& pdf, R& weight, uint32_t& lobe, SampleGen& sg, R, uint32_t lobeMask) const {
        const bool hasReflection = (lobeMask & LOBE_REFLECTION) != 0;
        const bool hasTransmission = (lobeMask & LOBE_TRANSMISSION) != 0;
        if (!hasReflection && !hasTransmission) return false;
        const R eta = etaAvg / R(1);
        const R Fd = evalFresnelDielectric(eta, o_abs(wi.z));
        const bool isReflection = hasReflection ? (Fd > R(0) && next1D<R>(sg) <= Fd) : false;
        wo = isReflection ? reflectLocal(wi) : -wi;
        weight = R(1);
        pdf = hasReflection && hasTransmission ? (isReflection ? Fd : R(1) - Fd) : R(1);
        lobe = isReflection ? LOBE_DELTA_REFLECTION : LOBE_DELTA_TRANSMISSION;
        return true;
    }
    R pdf(V3<R>, V3<R>, R) const { return R(0); }
    void lambdaPdf(V3<R>, V3<R>, uint32_t, const Beam<R>& beam, R* out) const { for (int j = 0; j < beam.H; ++j) out[j] = R(1); }
    M2<R> coherenceTransform(V3<R>, V3<R>, uint32_t) const { return ident2<R>(); }
};

// =============================================================================================
// PLTMultiLayeredStack, PLTMultiLayeredStackBSDF.slang:42-139, Material :40-57.
// RD is the arithmetic type of the layer recursion (R for the reference, double for the FP64
// transfer product option).
// =============================================================================================
template <class R> struct MultiLayer {
    R albedo[3];
    R extEta;
    V2<R> ior, thickness;
    unsigned layers;
    explicit MultiLayer(const Material<R>& m) {
        for (int i = 0; i < 3; ++i) albedo[i] = m.base[i];
        extEta = m.ior;
        ior = {m.data2[0], m.data2[1]};
        thickness = {m.data1[0], m.data1[1]};
        layers = m.data1w_bits;
    }
    template <class RD> static V2<RD> phasor(RD cosThetaT, RD thick, RD eta, RD k) {
        const RD d = RD(2) * thick / cosThetaT * k * eta;
        return {o_cos(d), o_sin(d)};
    }
    template <class RD> void evalT(V3<R> toLight, V3<R> toEye, uint32_t lobe, Beam<R>& beam) const {
        const bool isReflection = toLight.z * toEye.z > R(0);
        const bool isDirect = (lobe & LOBE_DELTA) != 0;
        if (!isDirect || !isReflection) { beam.setZero(); return; }
        R k[MAXH];
        kOf(beam, k);
        const R eta1 = ior.x / extEta;
        const R eta2 = ior.y / ior.x;
        V2<R> cosThetaT, r;
        const R Rout = o_sqrt(evalFresnelDielectric(eta1, toLight.z, cosThetaT.x));
        r.x = o_sqrt(evalFresnelDielectric(eta2, -cosThetaT.x, cosThetaT.y));
        r.y = o_sqrt(evalFresnelDielectric(eta2, cosThetaT.y));
        cosThetaT = {o_abs(cosThetaT.x), o_abs(cosThetaT.y)};
        const R cts[2] = {cosThetaT.x, cosThetaT.y}, ths[2] = {thickness.x, thickness.y}, iors[2] = {ior.x, ior.y},
                rr[2] = {r.x, r.y};
        for (int j = 0; j < beam.H; ++j) {
            const R m00 = rgbToSpectrum(albedo, beam.wl[j]);
            V2<RD> G = c_t(RD(o_sqrt(m00)));
            for (unsigned l = 0; l < layers; ++l) {
                const unsigned idx = l % 2;
                const V2<RD> p = phasor(RD(cts[idx]), RD(ths[idx]), RD(iors[idx]), RD(k[j]));
                const RD Rl = l == layers - 1 ? RD(Rout) : RD(rr[idx]);
                G = cmul(G, p);
                G = cdiv(c_t(Rl) + G, c_t(RD(1)) + G * Rl);
            }
            beam.setSP(j, R(sqr(G.x)) * beam.getSP(j));
        }
    }
    void eval(V3<R> toLight, V3<R> toEye, uint32_t lobe, Beam<R>& beam) const { evalT<R>(toLight, toEye, lobe, beam); }
    bool sample(V3<R> wi, V3<R>& wo, R& pdf, R& weight, uint32_t& lobe, SampleGen&, R wavelength, uint32_t lobeMask) const {
        const bool hasReflection = (lobeMask & LOBE_REFLECTION) != 0;
        const bool hasDirect = (lobeMask & LOBE_DELTA) != 0;
        if (!hasReflection || !hasDirect || wi.z <= R(0)) return false;
        pdf = R(1);
        wo = reflectLocal(wi);
        lobe = LOBE_DELTA_REFLECTION;
        weight = rgbToSpectrum(albedo, wavelength);
        return wi.z * wo.z > R(0);
    }
    R pdf(V3<R>, V3<R>, R) const { return R(0); }
    void lambdaPdf(V3<R>, V3<R>, uint32_t, const Beam<R>& beam, R* out) const { for (int j = 0; j < beam.H; ++j) out[j] = R(1); }
    M2<R> coherenceTransform(V3<R>, V3<R>, uint32_t) const { return ident2<R>(); }
};

// =============================================================================================
// PLTDiffuse, PLTDiffuseBSDF.slang:40-95
// =============================================================================================
template <class R> struct Diffuse {
    R albedo[3];
    explicit Diffuse(const Material<R>& m) { for (int i = 0; i < 3; ++i) albedo[i] = m.base[i]; }
    void eval(V3<R> toLight, V3<R>, uint32_t lobe, Beam<R>& beam) const {
        const bool valid = (lobe & LOBE_DIFFUSE_REFLECTION) != 0;
        for (int j = 0; j < beam.H; ++j) {
            const R colour = rgbToSpectrum(albedo, beam.wl[j]);
            const R w = valid ? o_abs(toLight.z) * R(K_1_PI) * colour : R(0);
            beam.L[0][j] *= w;
            beam.L[1][j] = beam.L[2][j] = beam.L[3][j] = R(0);
        }
    }
    bool sample(V3<R>, V3<R>& wo, R& pdf, R& weight, uint32_t& lobe, SampleGen& sg, R wavelength, uint32_t lobeMask) const {
        const bool has = (lobeMask & LOBE_DIFFUSE_REFLECTION) != 0;
        weight = rgbToSpectrum(albedo, wavelength);
        wo = sample_cosine_hemisphere_concentric(next2D<R>(sg), pdf);
        lobe = LOBE_DIFFUSE_REFLECTION;
        return has;
    }
    R pdf(V3<R>, V3<R> wo, R) const { return cosine_hemisphere_concentric_pdf(wo); }
    void lambdaPdf(V3<R>, V3<R>, uint32_t, const Beam<R>& beam, R* out) const { for (int j = 0; j < beam.H; ++j) out[j] = R(1); }
    M2<R> coherenceTransform(V3<R>, V3<R> wo, uint32_t) const {
        const R c = o_sqrt(o_max(R(1e-2), o_abs(wo.z)));
        return m2(c, R(0), R(0), R(1) / c);
    }
};

// =============================================================================================
// IMaterialInstance wrappers (e.g. PLTDielectricBSDF.slang:281-333): the batch API works in the
// local shading frame, so sd.toLocal is the identity except for the grated materials, which
// evaluate in the grating frame T = (gx, gy, 0), B = cross(N, T)
// (DiffractionGrating.slang:83-90, PLTDiffractionGrated*BSDF.slang:211-250).
// =============================================================================================
template <class R> struct Frame {
    V3<R> T, B, N;
    V3<R> toLocal(V3<R> v) const { return {dot(v, T), dot(v, B), dot(v, N)}; }
    V3<R> fromLocal(V3<R> v) const { return T * v.x + B * v.y + N * v.z; }
};
template <class R> inline Frame<R> identityFrame() {
    return {{R(1), R(0), R(0)}, {R(0), R(1), R(0)}, {R(0), R(0), R(1)}};
}
template <class R> inline Frame<R> gratingFrame(const DiffractionGrating<R>& g) {
    Frame<R> f;
    f.N = {R(0), R(0), R(1)};
    f.T = {g.gratingX.x, g.gratingX.y, R(0)};
    f.B = cross(f.N, f.T);
    return f;
}

template <class R, class BX> inline void wrapEval(const BX& bx, const Frame<R>& fr, V3<R> V, V3<R> W, uint32_t lobe, Beam<R>& beam) {
    beam.r = fr.toLocal(beam.r);
    beam.t = fr.toLocal(beam.t);
    const V3<R> wiL = fr.toLocal(V), woL = fr.toLocal(W);
    beam.constructLocalFrame(woL);
    bx.eval(wiL, woL, lobe, beam);
    beam.transformCoherence(bx.coherenceTransform(wiL, woL, lobe));
    beam.r = fr.fromLocal(beam.r);
    beam.t = fr.fromLocal(beam.t);
}

// One query of every op against one decoded material.
template <class R> struct QueryResult {
    R stokes[4][MAXH];
    R D[3], r_m;
    V3<R> t;
    R pdf;
    R lambdaPdf[MAXH];
    V3<R> sWo;
    R sPdf, sWeight;
    uint32_t sLobe, sValid;
};

template <class R, class BX>
inline void runOps(const BX& bx, const Frame<R>& evalFrame, const Frame<R>& lpFrame, uint32_t ops, V3<R> V, V3<R> W,
                   uint32_t lobe, const Beam<R>& beamIn, SampleGen* sg, QueryResult<R>& out, bool transmissiveForcing) {
    (void)transmissiveForcing;
    if (ops & PLT_OP_EVAL) {
        Beam<R> b = beamIn;
        wrapEval(bx, evalFrame, V, W, lobe, b);
        for (int c = 0; c < 4; ++c) for (int j = 0; j < b.H; ++j) out.stokes[c][j] = b.L[c][j];
        out.D[0] = b.D[0]; out.D[1] = b.D[1]; out.D[2] = b.D[2]; out.r_m = b.r_m;
        out.t = b.t;
    }
    if (ops & PLT_OP_PDF) out.pdf = bx.pdf(evalFrame.toLocal(W), evalFrame.toLocal(V), beamIn.wl[0]);
    if (ops & PLT_OP_LAMBDA_PDF) {
        // lambdaPdf takes the beam frame into sd-local coordinates (grated: sd, not the grating frame)
        Beam<R> b = beamIn;
        b.r = lpFrame.toLocal(b.r);
        b.t = lpFrame.toLocal(b.t);
        bx.lambdaPdf(lpFrame.toLocal(V), lpFrame.toLocal(W), lobe, b, out.lambdaPdf);
    }
    if (ops & PLT_OP_SAMPLE) {
        V3<R> wo = {R(0), R(0), R(0)};
        R pdf = R(0), weight = R(0);
        uint32_t sl = 0;
        const bool valid = bx.sample(evalFrame.toLocal(V), wo, pdf, weight, sl, *sg, beamIn.wl[0], LOBE_ALL);
        out.sWo = valid ? evalFrame.fromLocal(wo) : wo;
        out.sPdf = pdf;
        out.sWeight = weight;
        out.sLobe = sl;
        out.sValid = valid ? 1u : 0u;
    }
}

// Dispatch by material type (MaterialFactory.slang:79-130).  Returns false for unknown types.
template <class R>
inline bool queryMaterial(const Material<R>& m, const SceneTables& sc, uint32_t ops, V3<R> V, V3<R> W, uint32_t lobe,
                          const Beam<R>& beam, SampleGen* sg, QueryResult<R>& out, bool fp64Multilayer = false) {
    const Frame<R> id = identityFrame<R>();
    switch (m.type) {
    case PLT_MATERIAL_DIFFUSE: { Diffuse<R> b(m); runOps(b, id, id, ops, V, W, lobe, beam, sg, out, false); return true; }
    case PLT_MATERIAL_CONDUCTOR: { Conductor<R> b(m, &sc); runOps(b, id, id, ops, V, W, lobe, beam, sg, out, false); return true; }
    case PLT_MATERIAL_DIELECTRIC: {
        Dielectric<R> b(m);
        // PLTDielectricBSDF.sample restricts lobes by woHint; without a hint the mask is All.
        runOps(b, id, id, ops, V, W, lobe, beam, sg, out, true);
        return true;
    }
    case PLT_MATERIAL_OPAQUE_DIELECTRIC: { OpaqueDielectric<R> b(m); runOps(b, id, id, ops, V, W, lobe, beam, sg, out, false); return true; }
    case PLT_MATERIAL_THIN_DIELECTRIC: { ThinDielectric<R> b(m); runOps(b, id, id, ops, V, W, lobe, beam, sg, out, true); return true; }
    case PLT_MATERIAL_COATED_CONDUCTOR: { Coated<R, true> b(m, &sc); runOps(b, id, id, ops, V, W, lobe, beam, sg, out, false); return true; }
    case PLT_MATERIAL_COATED_OPAQUE_DIELECTRIC: { Coated<R, false> b(m, &sc); runOps(b, id, id, ops, V, W, lobe, beam, sg, out, false); return true; }
    case PLT_MATERIAL_GRATED_CONDUCTOR: {
        Grated<R, true> b(m, &sc);
        runOps(b, gratingFrame(b.grating), id, ops, V, W, lobe, beam, sg, out, false);
        return true;
    }
    case PLT_MATERIAL_GRATED_OPAQUE_DIELECTRIC: {
        Grated<R, false> b(m, &sc);
        runOps(b, gratingFrame(b.grating), id, ops, V, W, lobe, beam, sg, out, false);
        return true;
    }
    case PLT_MATERIAL_MULTILAYERED_STACK: {
        MultiLayer<R> b(m);
        if (fp64Multilayer && (ops & PLT_OP_EVAL)) {
            // FP64 recursion variant: same wrapper, double-precision layer loop
            struct ML64 {
                const MultiLayer<R>& ml;
                void eval(V3<R> a, V3<R> c, uint32_t l, Beam<R>& bm) const { ml.template evalT<double>(a, c, l, bm); }
                bool sample(V3<R> a, V3<R>& b2, R& c, R& d, uint32_t& e, SampleGen& f, R g, uint32_t h) const { return ml.sample(a, b2, c, d, e, f, g, h); }
                R pdf(V3<R> a, V3<R> c, R d) const { return ml.pdf(a, c, d); }
                void lambdaPdf(V3<R> a, V3<R> c, uint32_t d, const Beam<R>& e, R* f) const { ml.lambdaPdf(a, c, d, e, f); }
                M2<R> coherenceTransform(V3<R> a, V3<R> c, uint32_t d) const { return ml.coherenceTransform(a, c, d); }
            } w{b};
            runOps(w, id, id, ops, V, W, lobe, beam, sg, out, false);
        } else {
            runOps(b, id, id, ops, V, W, lobe, beam, sg, out, false);
        }
        return true;
    }
    default: return false;
    }
}

}  // namespace plt_oracle
