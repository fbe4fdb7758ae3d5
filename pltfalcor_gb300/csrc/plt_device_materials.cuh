// Device BxDFs of the ten PLT materials.  Each block cites the reference BxDF it restates
// (paths inside ssteinberg/PLTFalcor, Source/Falcor/Rendering/Materials/PLT/).
#pragma once

namespace pltdev {

// =============================================================================================
// PLTDielectric (PLTDielectricBSDF.slang:43-279)
// =============================================================================================
PLT_DI float dielIor(const float* __restrict__ p, float k) {
    const float x = k * k1_2Pi;
    return (__ldg(p + PG_ETAINT) + __ldg(p + PG_B) * (x * x)) / __ldg(p + PG_ETAEXT);
}
PLT_DI f3 dielRefract(f3 wi, float cosT, float eta) {
    const float s = cosT < 0.f ? 1.f / eta : eta;
    return mk3(-s * wi.x, -s * wi.y, cosT);
}
PLT_DI f3 dielScatteredWo(f3 wo, float eta) {
    const float s = wo.z > 0.f ? 1.f / eta : eta;
    const float x = wo.x * s, y = wo.y * s;
    const float l2 = x * x + y * y;
    if (l2 > 1.f) return mk3(0.f, 0.f, 0.f);
    return mk3(x, y, -signf(wo.z) * sqrtf(fmaxf(0.f, 1.f - l2)));
}
template <int H>
PLT_DI void dielEval(const DevMaterial* __restrict__ m, f3 toLight, f3 toEye, uint32_t lobe, DBeam<H>& b) {
    const float* p = m->p;
    const bool isReflection = toLight.z * toEye.z > 0.f;
    const bool isScatter = (lobe & kLobeNonDelta) != 0, isDirect = (lobe & kLobeDelta) != 0;
    const bool hasT = (lobe & kLobeTransmission) != 0, hasR = (lobe & kLobeReflection) != 0;
    if (toLight.z * toEye.z == 0.f || (!isScatter && !isDirect) || (!hasT && !isReflection) || (!hasR && isReflection)) {
        b.setZero();
        return;
    }
    const float* tab = isReflection ? m->m00a : m->m00b;
    float k[H], eta[H];
#pragma unroll
    for (int j = 0; j < H; ++j) { k[j] = kOfWl(b.wl[j]); eta[j] = dielIor(p, k[j]); }
    const f3 toEyeUp = isReflection ? toEye : dielScatteredWo(toEye, eta[0]);
    if (isScatter) {
        const f3 h = toLight + toEyeUp;
        const f3 mh = normalize(h);
        const float LdotH = fmaxf(0.f, dot(toLight, mh));
        const float cosM = signf(toLight.z) * LdotH;
#pragma unroll
        for (int j = 0; j < H; ++j) {
            const Alpha a = gaussAlpha(p, toLight, toEyeUp, k[j]);
            const float J = isReflection ? 1.f : sqr(toEye.z > 0.f ? eta[j] : 1.f / eta[j]);
            const float D = gaussEval(p, b, k[j], h);
            const FresnelD f = fresnel_dielectric(cosM, eta[j]);
            const MM M1 = isReflection ? muellerFresnelReal(f.rs, f.rp) : muellerFresnelReal(f.ts, f.tp);
            const float s = m00Of(tab, b.wl[j]) * a.om * J * fabsf(toLight.z) * D;
            b.setSP(j, s * mapply(M1, b.getSP(j)));
        }
    } else {
        const f3 toLightBeam = b.toLocal(toLight);
#pragma unroll
        for (int j = 0; j < H; ++j) {
            const float a = gaussAlpha(p, toLight, toEyeUp, k[j]).a;
            const float J = isReflection ? 1.f : sqr(toEye.z > 0.f ? eta[j] : 1.f / eta[j]);
            const FresnelD f = fresnel_dielectric(toLight.z, eta[j]);
            const MM M0 = isReflection ? muellerFresnelReal(f.rs, f.rp) : muellerFresnelReal(f.ts, f.tp);
            float coh = 1.f;
            if (!isReflection && j > 0) {
                const FresnelD fe = fresnel_dielectric(toEye.z, eta[j]);
                const f3 lobeWo = b.toLocal(dielRefract(toEye, fe.cosT, eta[j]));
                coh = b.mutualCoherenceAngular(lobeWo, toLightBeam);
            }
            const float s = m00Of(tab, b.wl[j]) * a * coh * J;
            b.setSP(j, s * mapply(M0, b.getSP(j)));
        }
    }
}
PLT_DI bool dielSample(const DevMaterial* __restrict__ m, f3 wi, f3& wo, float& pdf, float& weight, uint32_t& lobe,
                       SampleGen& sg, float wl, uint32_t lobeMask = kLobeAll, f2 uw = kNoWarp) {
    const bool hasR = (lobeMask & kLobeReflection) != 0, hasT = (lobeMask & kLobeTransmission) != 0;
    const bool hasD = (lobeMask & kLobeDelta) != 0, hasS = (lobeMask & kLobeNonDelta) != 0;
    if ((!hasR && !hasT) || (!hasD && !hasS)) return false;
    const float* p = m->p;
    const float k = kOfWl(wl);
    const Alpha a = gaussAlpha(p, wi, wi, k);
    const float eta = dielIor(p, k);
    bool isDirect;
    if (hasD && hasS) {
        isDirect = a.a == 1.f || sg.next1D() < a.a;
        pdf = isDirect ? a.a : a.om;
    } else {
        isDirect = hasD || sg.next1D() < 0.f;   // pdfDirect 1 (delta only) or 0 (scatter only: one draw)
        pdf = 1.f;
    }
    const bool both = hasR && hasT;
    bool isReflection;
    if (isDirect) {
        const FresnelD f = fresnel_dielectric(wi.z, eta);
        const float Fd = fresnelR(f);
        isReflection = hasR ? (Fd > 0.f && sg.next1D() <= Fd) : false;
        wo = isReflection ? reflectL(wi) : dielRefract(wi, f.cosT, eta);
        pdf *= both ? (isReflection ? Fd : 1.f - Fd) : 1.f;
        lobe = isReflection ? kLobeDeltaR : (__ldg(p + PG_B) != 0.f ? kLobeDispDeltaT : kLobeDeltaT);
    } else {
        float surfPdf;
        wo = gaussSample(p, wi, sg, k, surfPdf, uw);
        pdf *= surfPdf;
        const f3 mh = normalize(wi + wo);
        const float F = fresnelR(fresnel_dielectric(signf(wi.z) * dot(wi, mh), eta));
        isReflection = hasR ? (F > 0.f && sg.next1D() <= F) : false;
        if (!isReflection) wo = dielScatteredWo(wo, eta);
        pdf *= both ? (isReflection ? F : 1.f - F) : 1.f;
        lobe = isReflection ? kLobeScatterR : kLobeScatterT;
    }
    weight = m00Of(isReflection ? m->m00a : m->m00b, wl);
    return (isReflection && wi.z * wo.z <= 0.f) ? false : (!isReflection && wi.z * wo.z >= 0.f) ? false : true;
}
PLT_DI float dielPdf(const DevMaterial* __restrict__ m, f3 wi, f3 woL, float wl) {
    const float* p = m->p;
    const float k = kOfWl(wl);
    const Alpha a = gaussAlpha(p, wi, wi, k);
    const float eta = dielIor(p, k);
    const bool isReflection = wi.z * woL.z > 0.f;
    const f3 wo = isReflection ? woL : dielScatteredWo(woL, eta);
    const f3 mh = normalize(wi + wo);
    const float F = fresnelR(fresnel_dielectric(signf(wi.z) * dot(wi, mh), eta));
    const float pdfF = isReflection ? F : 1.f - F;
    return a.om * pdfF * gaussPdf(p, wi, wo, k);
}
template <int H>
PLT_DI void dielLambdaPdf(const DevMaterial* __restrict__ m, f3 toLight, f3 toEye, uint32_t lobe, const DBeam<H>& b, float* out) {
    const float* p = m->p;
    const bool isReflection = toLight.z * toEye.z > 0.f;
    const bool isScatter = (lobe & kLobeNonDelta) != 0, isDirect = (lobe & kLobeDelta) != 0;
    if (isDirect && !isReflection) {
        const f3 toLightBeam = b.toLocal(toLight);
#pragma unroll
        for (int j = 0; j < H; ++j) {
            if (j == 0) { out[0] = 1.f; continue; }
            const float eta = dielIor(p, kOfWl(b.wl[j]));
            const FresnelD fe = fresnel_dielectric(toEye.z, eta);
            out[j] = b.mutualCoherenceAngular(b.toLocal(dielRefract(toEye, fe.cosT, eta)), toLightBeam);
        }
        return;
    }
#pragma unroll
    for (int j = 0; j < H; ++j) {
        if (isScatter) {
            const float k = kOfWl(b.wl[j]);
            const float eta = dielIor(p, k);
            const f3 wo = isReflection ? toLight : dielScatteredWo(toLight, eta);
            out[j] = gaussPdf(p, toEye, wo, k);
        } else {
            out[j] = 1.f;
        }
    }
}

// =============================================================================================
// PLTConductor (PLTConductorBSDF.slang:44-173); also the base of the grated conductor
// =============================================================================================
PLT_DI f2 conductorIor(const DevMaterial* __restrict__ m, const Ctx& c, float wl, float div) {
    return f2{evalSpectrum(c.profiles, c.nprof, m->etaN, wl) / div, evalSpectrum(c.profiles, c.nprof, m->etaK, wl) / div};
}
template <int H>
PLT_DI void condEval(const DevMaterial* __restrict__ m, const Ctx& c, f3 toLight, f3 toEye, uint32_t lobe, DBeam<H>& b) {
    const float* p = m->p;
    const bool isScatter = (lobe & kLobeScatterR) != 0, isDirect = (lobe & kLobeDeltaR) != 0;
    if ((!isScatter && !isDirect) || (lobe & kLobeReflection) == 0) { b.setZero(); return; }
    const f3 h = toLight + toEye;
    const f3 mh = normalize(h);
    const float LdotH = fmaxf(0.f, dot(toLight, mh));
    const float extEta = __ldg(p + PF_EXTETA);
#pragma unroll
    for (int j = 0; j < H; ++j) {
        const float k = kOfWl(b.wl[j]);
        const Alpha a = fracAlpha(p, toLight, toEye, k);
        const f2 ior = conductorIor(m, c, b.wl[j], extEta);
        f2 rs, rp;
        float s;
        MM M;
        if (isScatter) {
            M = muellerRConductor(LdotH, ior, rs, rp, c.flags);
            s = a.om * fabsf(toLight.z) * fracPGF(p, k * h.x, k * h.y);
        } else {
            M = muellerRConductor(toLight.z, ior, rs, rp, c.flags);
            s = a.a;
        }
        const f4 v = s * mapply(M, b.getSP(j));
        const float m00 = m00Of(m->m00a, b.wl[j]);
        b.setSP(j, f4{v.x * m00, v.y * m00, v.z * m00, v.w * m00});
    }
}
PLT_DI bool condSample(const DevMaterial* __restrict__ m, f3 wi, f3& wo, float& pdf, float& weight, uint32_t& lobe,
                       SampleGen& sg, float wl, uint32_t lobeMask = kLobeAll, f2 uw = kNoWarp) {
    const bool hasR = (lobeMask & kLobeReflection) != 0;
    const bool hasD = (lobeMask & kLobeDelta) != 0, hasS = (lobeMask & kLobeNonDelta) != 0;
    if (!hasR || (!hasD && !hasS)) return false;
    const float* p = m->p;
    const float k = kOfWl(wl);
    bool isDirect = hasD;
    pdf = 1.f;
    if (hasD && hasS) {
        const Alpha a = fracAlpha(p, wi, wi, k);
        isDirect = a.a == 1.f || sg.next1D() < a.a;
        pdf = isDirect ? a.a : a.om;
    }
    weight = m00Of(m->m00a, wl);
    if (isDirect) {
        wo = reflectL(wi);
        lobe = kLobeDeltaR;
    } else {
        float sp;
        wo = fracSample(p, wi, sg, k, sp, uw);
        pdf *= sp;
        lobe = kLobeScatterR;
    }
    return true;
}
PLT_DI float condPdf(const DevMaterial* __restrict__ m, f3 wi, f3 wo, float wl) {
    const float k = kOfWl(wl);
    return fracAlpha(m->p, wi, wi, k).om * fracPdf(m->p, wi, wo, k);
}

// =============================================================================================
// PLTOpaqueDielectric (PLTOpaqueDielectricBSDF.slang:43-147): mean wavenumber, scalar Mueller
// =============================================================================================
template <int H>
PLT_DI void opaqEval(const DevMaterial* __restrict__ m, f3 toLight, f3 toEye, uint32_t lobe, DBeam<H>& b) {
    const float* p = m->p;
    const bool isDirect = (lobe & kLobeDelta) != 0, isScatter = (lobe & kLobeNonDelta) != 0;
    if ((!isScatter && !isDirect) || (lobe & kLobeReflection) == 0) { b.setZero(); return; }
    const float mk = meank();
    const Alpha a = fracAlpha(p, toLight, toEye, mk);
    float M = a.a;
    if (isScatter) {
        const f3 h = toLight + toEye;
        M = a.om * fabsf(toLight.z) * fracPGF(p, mk * h.x, mk * h.y);
    }
#pragma unroll
    for (int j = 0; j < H; ++j) b.setSP(j, (M * m00Of(m->m00a, b.wl[j])) * b.getSP(j));
}
PLT_DI bool opaqSample(const DevMaterial* __restrict__ m, f3 wi, f3& wo, float& pdf, float& weight, uint32_t& lobe,
                       SampleGen& sg, float wl, uint32_t lobeMask = kLobeAll, f2 uw = kNoWarp) {
    const bool hasR = (lobeMask & kLobeReflection) != 0;
    const bool hasD = (lobeMask & kLobeDelta) != 0, hasS = (lobeMask & kLobeNonDelta) != 0;
    if (!hasR || (!hasD && !hasS)) return false;
    const float* p = m->p;
    const float mk = meank();
    bool isDirect = hasD;
    pdf = 1.f;
    if (hasD && hasS) {
        const Alpha a = fracAlpha(p, wi, wi, mk);
        isDirect = a.a == 1.f || sg.next1D() < a.a;
        pdf = isDirect ? a.a : a.om;
    }
    weight = m00Of(m->m00a, wl);
    if (isDirect) {
        wo = reflectL(wi);
        lobe = kLobeDeltaR;
    } else {
        float sp;
        wo = fracSample(p, wi, sg, mk, sp, uw);
        pdf *= sp;
        lobe = kLobeScatterR;
    }
    return true;
}
PLT_DI float opaqPdf(const DevMaterial* __restrict__ m, f3 wi, f3 wo) {
    const float mk = meank();
    return fracAlpha(m->p, wi, wi, mk).om * fracPdf(m->p, wi, wo, mk);
}

// =============================================================================================
// Coated opaque dielectric / coated conductor (PLTCoatedOpaqueDielectricBSDF.slang:45-245,
// PLTCoatedConductorBSDF.slang:45-246)
// =============================================================================================
PLT_DI f3 coatRefract(f3 wi, float eta, float cosT) {
    const float s = cosT < 0.f ? 1.f / eta : eta;
    return mk3(-s * wi.x, -s * wi.y, cosT);
}
template <int H, bool CONDUCTOR>
PLT_DI void coatEval(const DevMaterial* __restrict__ m, const Ctx& c, f3 toLight, f3 toEye, uint32_t lobe, DBeam<H>& b) {
    const float* p = m->p;
    const bool isReflection = toLight.z * toEye.z > 0.f;
    const bool isScatter = (lobe & kLobeScatterR) != 0, isDirect = (lobe & kLobeDeltaR) != 0;
    const float coatior = __ldg(p + PC_COATETA), eta1 = __ldg(p + PC_ETA1), tau = __ldg(p + PC_TAU);
    const FresnelD fin = fresnel_dielectric(toLight.z, eta1);
    const f3 wiIn = -coatRefract(toLight, eta1, fin.cosT);
    f3 woIn = reflectL(wiIn);
    if (!isDirect) {
        const FresnelD fo = fresnel_dielectric(toEye.z, eta1);
        woIn = -coatRefract(toEye, eta1, fo.cosT);
    }
    if (!isReflection || (!isScatter && !isDirect) || wiIn.z <= 0.f || woIn.z <= 0.f) { b.setZero(); return; }
    const f3 h = wiIn + woIn;
    const f3 mh = normalize(h);
    const float LdotH = fmaxf(0.f, dot(wiIn, mh));
    const f3 Z = b.toLocal(mk3(0.f, 0.f, 1.f));
    const float quad = b.coherenceQuad(Z * tau);
    const MM MiT = muellerFresnelReal(fin.ts, fin.tp);
    const FresnelD fmo = fresnel_dielectric(-woIn.z, eta1);
    const MM MoT = muellerFresnelReal(fmo.ts, fmo.tp);
    const float dist = 2.f * tau / wiIn.z;
    if (!CONDUCTOR) {
        const MM M = mmul(MiT, MoT);
        const MM MiRs = isScatter ? muellerRDielectric(LdotH, eta1) : muellerFresnelReal(fin.rs, fin.rp);
#pragma unroll
        for (int j = 0; j < H; ++j) {
            const float k = kOfWl(b.wl[j]);
            const Alpha a = fracAlpha(p, wiIn, woIn, k);
            const float coh = b.mutualCoherenceK(k, quad);
            const float phase = sinf(dist * k * coatior);
            const f4 SP = b.getSP(j);
            f4 newSP = m00Of(m->m00a, b.wl[j]) * mapply(M, SP);
            f4 refl;
            if (isScatter) {
                const float w = a.om * fabsf(toLight.z) * fracPGF(p, k * h.x, k * h.y);
                newSP = w * newSP;
                refl = w * mapply(MiRs, SP);
            } else {
                newSP = a.a * newSP;
                refl = a.a * mapply(MiRs, SP);
            }
            b.setSP(j, interfere(newSP, refl, phase, phase, coh));
        }
    } else {
        const MM MiR = muellerFresnelReal(fin.rs, fin.rp);
#pragma unroll
        for (int j = 0; j < H; ++j) {
            const float k = kOfWl(b.wl[j]);
            const Alpha a = fracAlpha(p, wiIn, woIn, k);
            const float coh = b.mutualCoherenceK(k, quad);
            f2 rs, rp;
            const MM M2R = muellerRConductor(LdotH, conductorIor(m, c, b.wl[j], coatior), rs, rp, c.flags);
            const MM M = mmul(mmul(MiT, M2R), MoT);
            const f4 SP = b.getSP(j);
            f4 newSP = m00Of(m->m00a, b.wl[j]) * mapply(M, SP);
            if (isScatter) {
                newSP = (a.om * fabsf(toLight.z) * fracPGF(p, k * h.x, k * h.y)) * newSP;
            } else {
                const float pS = sinf(dist * k * coatior + atan2f(rs.y, rs.x));
                const float pP = sinf(dist * k * coatior + atan2f(rp.y, rp.x));
                newSP = interfere(a.a * newSP, mapply(MiR, SP), pS, pP, coh);
            }
            b.setSP(j, newSP);
        }
    }
}
PLT_DI bool coatSample(const DevMaterial* __restrict__ m, f3 wi, f3& wo, float& pdf, float& weight, uint32_t& lobe,
                       SampleGen& sg, float wl, uint32_t lobeMask = kLobeAll, f2 uw = kNoWarp) {
    const bool hasR = (lobeMask & kLobeReflection) != 0;
    const bool hasD = (lobeMask & kLobeDelta) != 0, hasS = (lobeMask & kLobeNonDelta) != 0;
    if (!hasR || (!hasD && !hasS)) return false;
    const float* p = m->p;
    if (wi.z <= 0.f) return false;
    const float k = kOfWl(wl);
    const float eta1 = __ldg(p + PC_ETA1);
    const FresnelD f = fresnel_dielectric(wi.z, eta1);
    const float Fd = fresnelR(f);
    // "Fd == .1f" is what the reference tests (PLTCoated*BSDF.slang:150-151)
    const bool isReflCoat = Fd == .1f || sg.next1D() < Fd;
    weight = 1.f;
    pdf = isReflCoat ? Fd : 1.f - Fd;
    if (isReflCoat) {
        wo = reflectL(wi);
        lobe = kLobeDeltaR;
        return true;
    }
    const f3 wiIn = -coatRefract(wi, eta1, f.cosT);
    if (wiIn.z == 0.f) return false;
    weight = m00Of(m->m00a, wl);
    bool isDirect;
    if (hasD && hasS) {
        const Alpha a = fracAlpha(p, wiIn, wiIn, k);
        isDirect = a.a == 1.f || sg.next1D() < a.a;
        pdf *= isDirect ? a.a : a.om;
    } else {
        isDirect = hasD || sg.next1D() < 0.f;
    }
    if (isDirect) {
        wo = reflectL(wi);
        lobe = kLobeDeltaR;
    } else {
        float sp;
        const f3 woIn = fracSample(p, wiIn, sg, k, sp, uw);
        pdf *= sp;
        const FresnelD f1 = fresnel_dielectric(-woIn.z, eta1);
        wo = coatRefract(-woIn, eta1, f1.cosT);
        lobe = kLobeScatterR;
    }
    return wi.z * wo.z > 0.f;
}
PLT_DI float coatPdf(const DevMaterial* __restrict__ m, f3 wi, f3 wo, float wl) {
    if (wi.z <= 0.f || wo.z <= 0.f) return 0.f;
    const float* p = m->p;
    const float k = kOfWl(wl);
    const float eta1 = __ldg(p + PC_ETA1);
    const FresnelD f = fresnel_dielectric(wi.z, eta1);
    const float Fd = fresnelR(f);
    const FresnelD f1 = fresnel_dielectric(wo.z, eta1);
    const f3 wiIn = -coatRefract(wi, eta1, f.cosT);
    const f3 woIn = -coatRefract(wo, eta1, f1.cosT);
    const float om = fracAlpha(p, wiIn, wiIn, k).om;
    return wiIn.z * woIn.z == 0.f ? 0.f : om * (1.f - Fd) * fracPdf(p, wiIn, woIn, k);
}
template <int H>
PLT_DI void coatLambdaPdf(const DevMaterial* __restrict__ m, f3 toLight, f3 toEye, uint32_t lobe, const DBeam<H>& b, float* out) {
    const float* p = m->p;
    if ((lobe & kLobeNonDelta) != 0) {
        const float eta1 = __ldg(p + PC_ETA1);
        const FresnelD f = fresnel_dielectric(toEye.z, eta1), f1 = fresnel_dielectric(toLight.z, eta1);
        const f3 wiIn = -coatRefract(toEye, eta1, f.cosT);
        const f3 woIn = -coatRefract(toLight, eta1, f1.cosT);
#pragma unroll
        for (int j = 0; j < H; ++j) out[j] = fracPdf(p, wiIn, woIn, kOfWl(b.wl[j]));
        return;
    }
#pragma unroll
    for (int j = 0; j < H; ++j) out[j] = 1.f;
}

// =============================================================================================
// Diffraction gratings (DiffractionGrating.slang:41-156) and the grated BxDFs
// (PLTDiffractionGratedOpaqueDielectricBSDF.slang:45-209, PLTDiffractionGratedConductorBSDF.slang:45-213)
// =============================================================================================
PLT_DI Alpha gratAlphaFull(const float* __restrict__ p, f3 wi, float k) { return alphaOf(sqr(wi.z * __ldg(p + PD_Q) * k)); }
PLT_DI float gratAlpha(const float* __restrict__ p, f3 wi, float k) { return expf(-sqr(wi.z * __ldg(p + PD_Q) * k)); }
PLT_NI float gratLobeIntensity(const DevMaterial* __restrict__ m, int lx, int ly, f3 wi, float lambda) {
    const float* p = m->p;
    const uint32_t gtype = (m->aux >> 8) & 0xFu;
    const bool is1D = __ldg(p + PD_IPY) == 0.f;
    const float a = k4Pi * __ldg(p + PD_Q) / (lambda * fabsf(wi.z));
    float ix, iy;
    if (gtype == 0u) {
        ix = iy = lx == 0 ? 1.f : besselJ(lx, a);
        if (!is1D) iy = ly == 0 ? 1.f : besselJ(ly, a);
    } else if (gtype == 1u) {
        const float sa = sinf(a / 2.f);
        ix = iy = lx == 0 ? 1.f : sa * (sinf(kPi * (float)lx / 2.f) / (kPi * (float)lx / 2.f));
        if (!is1D) iy = ly == 0 ? 1.f : sa * (sinf(kPi * (float)ly / 2.f) / (kPi * (float)ly / 2.f));
    } else {
        ix = iy = lx == 0 ? 1.f : 1.f / sqrtf((float)abs(lx));
        if (!is1D) iy = ly == 0 ? 1.f : 1.f / sqrtf((float)abs(ly));
    }
    return __ldg(p + PD_MULT) * ix * iy;
}
PLT_NI f3 gratDiffract(const float* __restrict__ p, f3 wi, int lx, int ly, float lambda) {
    const float px = sqrtf(wi.x * wi.x + wi.z * wi.z), py = sqrtf(wi.y * wi.y + wi.z * wi.z);
    const float sx = px > kFltEps ? wi.x / px : 0.f, sy = py > kFltEps ? wi.y / py : 0.f;
    const float a = lambda * (float)lx * __ldg(p + PD_IPX) - sx;
    const float bb = lambda * (float)ly * __ldg(p + PD_IPY) - sy;
    if (!(fabsf(a) <= 1.f && fabsf(bb) <= 1.f)) return mk3(0.f, 0.f, 0.f);
    const float mm = (a * a - 1.f) / (sqr(a * bb) - 1.f);
    const float q = 1.f - bb * bb * mm;
    return mk3(a * sqrtf(fmaxf(0.f, q)), bb * sqrtf(mm), sqrtf(fmaxf(0.f, 1.f - a * a * q - bb * bb * mm)));
}
PLT_DI void decodeGratingLobe(uint32_t code, int& lx, int& ly) {
    const int x = (int)code >> 8;
    lx = (x & 0x7) * (2 * ((x >> 6) & 1) - 1);
    ly = ((x >> 3) & 0x7) * (2 * ((x >> 7) & 1) - 1);
}
PLT_DI uint32_t encodeGratingLobe(int lx, int ly, uint32_t lobe) {
    const int sx = lx < 0 ? 0 : 1, sy = ly < 0 ? 0 : 1;
    const int ax = min(abs(lx), 7), ay = min(abs(ly), 7);
    return (lobe & ~kLobeMaterialSpecific) + (uint32_t)(((ay << 3) + ax + (sy << 7) + (sx << 6)) << 8);
}
template <int H, bool CONDUCTOR>
PLT_DI void gratEval(const DevMaterial* __restrict__ m, const Ctx& c, f3 toLight, f3 toEye, uint32_t bsdfLobe, DBeam<H>& b) {
    const float* p = m->p;
    const bool isDirect = (bsdfLobe & kLobeDelta) != 0;
    float a[H], om[H];
    bool anyPos = false, anyLt1 = false;
#pragma unroll
    for (int j = 0; j < H; ++j) {
        const Alpha al = gratAlphaFull(p, toLight, k2Pi / (1e-3f * b.wl[j]));
        a[j] = al.a;
        om[j] = al.om;
        anyPos |= a[j] > 0.f;
        anyLt1 |= a[j] < 1.f;
    }
    int lx, ly;
    decodeGratingLobe(bsdfLobe, lx, ly);
    if (lx == 0 && ly == 0 && anyPos) {
        if (CONDUCTOR) condEval<H>(m, c, toLight, toEye, bsdfLobe, b);
        else opaqEval<H>(m, toLight, toEye, bsdfLobe, b);
#pragma unroll
        for (int j = 0; j < H; ++j) { b.L[0][j] *= a[j]; b.L[1][j] *= a[j]; b.L[2][j] *= a[j]; b.L[3][j] *= a[j]; }
    } else if ((lx != 0 || ly != 0) && anyLt1 && isDirect) {
        const f3 toLightBeam = b.toLocal(toLight);
#pragma unroll
        for (int j = 0; j < H; ++j) {
            const float lambda = 1e-3f * b.wl[j];
            float coh = 1.f;
            if (j > 0) coh = b.mutualCoherenceAngular(b.toLocal(gratDiffract(p, toEye, lx, ly, lambda)), toLightBeam);
            const float inten = gratLobeIntensity(m, lx, ly, toLight, lambda);
            const float s = m00Of(m->m00a, b.wl[j]) * om[j] * coh * inten;
            if (CONDUCTOR) {
                f2 rs, rp;
                const MM M0 = muellerRConductor(toLight.z, conductorIor(m, c, b.wl[j], __ldg(p + PF_EXTETA)), rs, rp, c.flags);
                b.setSP(j, s * mapply(M0, b.getSP(j)));
            } else {
                b.setSP(j, s * b.getSP(j));
            }
        }
    } else {
        b.setZero();
    }
}
// DiffractionGrating.sampleLobe (:109-140)
PLT_DI void gratSampleLobe(const DevMaterial* __restrict__ m, f3 wi, int& lx, int& ly, float& px, float& py, float lambda, SampleGen& sg) {
    const int lobeCount = (int)(m->aux & 0xFFu);
    float inten[8];
    float total = 0.f;
#pragma unroll
    for (int l = 0; l < 8; ++l) {
        if (l < lobeCount) {
            inten[l] = gratLobeIntensity(m, l + 1, 0, wi, lambda);
            total += inten[l];
        }
    }
    const float rx = (sg.next1D() - .5f) * 2.f;
    const float ry = (sg.next1D() - .5f) * 2.f;
    float cdf = 0.f;
    lx = ly = 0;
    px = py = 0.f;
#pragma unroll
    for (int l = 0; l < 8; ++l) {
        if (l < lobeCount) {
            const float pr = inten[l] / total;
            cdf += pr;
            if (fabsf(rx) < cdf && lx == 0) { px = pr; lx = l + 1; }
            if (fabsf(ry) < cdf && ly == 0) { py = pr; ly = l + 1; }
        }
    }
    px /= 2.f;
    py /= 2.f;
    if (rx < 0.f) lx = -lx;
    if (ry < 0.f) ly = -ly;
    if (__ldg(m->p + PD_IPY) == 0.f) { ly = 0; py = 1.f; }
}
// closestLobeHint, DiffractionGrating.slang:92-107: the order whose direction is closest to -woHint
PLT_DI void gratClosestLobeHint(const DevMaterial* __restrict__ m, f3 wi, f3 woHint, float alpha, float lambda, int& lx, int& ly) {
    lx = ly = 0;
    if (alpha == 1.f) return;
    const float* p = m->p;
    const int lobeCount = (int)(m->aux & 0xFFu);
    const float li2x = wi.x * wi.x + wi.z * wi.z, li2y = wi.y * wi.y + wi.z * wi.z;
    const float lo2x = woHint.x * woHint.x + woHint.z * woHint.z, lo2y = woHint.y * woHint.y + woHint.z * woHint.z;
    const float six = li2x > kFltEps ? wi.x / sqrtf(li2x) : 0.f, siy = li2y > kFltEps ? wi.y / sqrtf(li2y) : 0.f;
    const float sox = lo2x > kFltEps ? -woHint.x / sqrtf(lo2x) : 0.f, soy = lo2y > kFltEps ? -woHint.y / sqrtf(lo2y) : 0.f;
    auto toLobe = [&](float l) {
        const float v = l + signf(l) * .5f;
        const int li = isfinite(v) ? (int)fmaxf(-1e9f, fminf(1e9f, v)) : 0;
        return max(-lobeCount, min(lobeCount, li));
    };
    const float l0 = (six - sox) / (__ldg(p + PD_IPX) * lambda);
    lx = toLobe(l0);
    if (alpha == 0.f && lx == 0) lx = (int)signf(l0);
    if (__ldg(p + PD_IPY) != 0.f) {
        const float l1 = (siy - soy) / (__ldg(p + PD_IPY) * lambda);
        ly = toLobe(l1);
        if (alpha == 0.f && ly == 0) ly = (int)signf(l1);
    }
}
template <bool CONDUCTOR>
PLT_DI bool gratSample(const DevMaterial* __restrict__ m, f3 wi, f3& wo, float& pdf, float& weight, uint32_t& lobe,
                       SampleGen& sg, float wl, uint32_t lobeMask = kLobeAll, f3 woHint = f3{0.f, 0.f, 0.f}, f2 uw = kNoWarp) {
    const bool hasR = (lobeMask & kLobeReflection) != 0;
    const bool hasD = (lobeMask & kLobeDelta) != 0, hasS = (lobeMask & kLobeNonDelta) != 0;
    if (!hasR || (!hasD && !hasS)) return false;
    const float* p = m->p;
    const float lambda = 1e-3f * wl;
    const Alpha a = gratAlphaFull(p, wi, k2Pi / lambda);
    const bool hasHint = hasD && (woHint.x != 0.f || woHint.y != 0.f || woHint.z != 0.f);
    int lx = 0, ly = 0;
    if (hasHint && a.a < 1.f) gratClosestLobeHint(m, wi, woHint, a.a, lambda, lx, ly);
    bool isDirect = hasD;
    if (hasHint) {
        isDirect = lx == 0 && ly == 0;
        pdf = 1.f;
    } else if (hasD && hasS) {
        isDirect = a.a == 1.f || sg.next1D() < a.a;
        pdf = isDirect ? a.a : a.om;
    }
    if (isDirect) {
        float bp = 0.f;
        if (CONDUCTOR) condSample(m, wi, wo, bp, weight, lobe, sg, wl, lobeMask, uw);
        else opaqSample(m, wi, wo, bp, weight, lobe, sg, wl, lobeMask, uw);
        pdf *= bp;
        return true;
    }
    weight = m00Of(m->m00a, wl);
    float px = 1.f, py = 1.f;
    if (!hasHint) gratSampleLobe(m, wi, lx, ly, px, py, lambda, sg);
    wo = gratDiffract(p, wi, lx, ly, lambda);
    lobe = encodeGratingLobe(lx, ly, kLobeDispDeltaR);
    pdf *= px * py;
    return true;
}
template <bool CONDUCTOR>
PLT_DI float gratPdf(const DevMaterial* __restrict__ m, f3 wi, f3 wo, float wl) {
    const float a = gratAlpha(m->p, wi, k2Pi / (1e-3f * wl));
    return (CONDUCTOR ? condPdf(m, wi, wo, wl) : opaqPdf(m, wi, wo)) * a;
}
template <int H>
PLT_DI void gratLambdaPdf(const DevMaterial* __restrict__ m, f3 toLight, f3 toEye, uint32_t bsdfLobe, const DBeam<H>& b, float* out) {
    const float* p = m->p;
    bool anyLt1 = false;
#pragma unroll
    for (int j = 0; j < H; ++j) anyLt1 |= gratAlpha(p, toLight, k2Pi / (1e-3f * b.wl[j])) < 1.f;
    int lx, ly;
    decodeGratingLobe(bsdfLobe, lx, ly);
    if ((lx != 0 || ly != 0) && anyLt1 && (bsdfLobe & kLobeDelta) != 0) {
        const f3 toLightBeam = b.toLocal(toLight);
#pragma unroll
        for (int j = 0; j < H; ++j)
            out[j] = j == 0 ? 1.f : b.mutualCoherenceAngular(b.toLocal(gratDiffract(p, toEye, lx, ly, 1e-3f * b.wl[j])), toLightBeam);
        return;
    }
#pragma unroll
    for (int j = 0; j < H; ++j) out[j] = 1.f;
}

// =============================================================================================
// PLTThinDielectric with birefringence (PLTThinDielectricBSDF.slang:43-200, Birefringence.slang)
// =============================================================================================
PLT_DI float bq_o(float eo, float K) { return sqrtf(eo * eo - K * K); }
PLT_DI f2 bq_e(float eo, float ee, f3 A, float K) {
    const float e = ee * ee - eo * eo;
    const float G = A.y * A.y * e + eo * eo;
    const float root = sqrtf(fmaxf(0.f, K * K * (A.x * A.x * e - ee * ee) + ee * ee * G));
    const float cb = A.z * A.y * K * e;
    return f2{(eo * root + cb) / G, (-eo * root + cb) / G};
}
PLT_DI f3 bE_e(float eo, f3 A, float K, float q) {
    return normalize(mk3(A.x * (eo * eo), K * A.z * q + A.y * (eo * eo - q * q), K * A.y * q + A.z * (eo * eo - K * K)));
}
PLT_DI f3 bE_o(f3 A, float K, float q) { return normalize(mk3(-A.y * K - A.z * q, A.x * K, A.x * q)); }
PLT_DI f3 bPoynting(float q, f3 E, float K) {
    return normalize(mk3(E.x * (K * E.z - q * E.y), K * E.z * E.y + q * (E.x * E.x + E.z * E.z), -q * E.z * E.y - K * (E.x * E.x + E.y * E.y)));
}
template <int H>
PLT_DI void thinBirefringence(const DevMaterial* __restrict__ m, DBeam<H>& b, f3 wi) {
    const float* p = m->p;
    const f3 OA = mk3(__ldg(p + PT_OAX), __ldg(p + PT_OAY), __ldg(p + PT_OAZ));
    const float phii = atan2f(wi.y, wi.x);
    const float phiA = atan2f(OA.y, OA.x) - phii;
    const f3 I = mk3(0.f, fabsf(wi.z), sqrtf(1.f - wi.z * wi.z));
    float sA, cA;
    sincosf(phiA, &sA, &cA);
    const float sOA = sqrtf(1.f - OA.z * OA.z);
    f3 A = mk3(cA * sOA, 0.f * sOA, sA * sOA);
    A.y = signf(wi.z) * OA.z;
    const f3 A2 = mk3(A.x, -A.y, A.z);
    float sp_, cp_;
    sincosf(phii, &sp_, &cp_);
    const f3 Z = b.toLocal(mk3(cp_, sp_, 0.f));
    const float ei = 1.f, eo = __ldg(p + PT_EO), ee = __ldg(p + PT_EE), tauum = __ldg(p + PT_TAUUM);
    // vectors_in_slab (Birefringence.slang:172-195)
    const float K = ei * I.z;
    const float qom = -bq_o(eo, K);
    const f2 qeK = bq_e(eo, ee, A, K);
    const f3 Eom = bE_o(A, K, qom);
    const f3 Eem = bE_e(eo, A, K, qeK.y);
    const f3 Io = bPoynting(qom, Eom, K);
    const f3 Ie = bPoynting(qeK.y, Eem, K);
    const f3 We = normalize(mk3(0.f, qeK.y, -K));
    const float e_eff = K / sqrtf(fmaxf(0.f, 1.f - We.y * We.y));
    // fresnel_iso_aniso(I.y, I.z, ei, eo, ee, A) (Birefringence.slang:109-136)
    float tso, tse, tpo, tpe;
    {
        const float cos_t = I.y, sin_t = I.z;
        const float Kk = ei * sin_t;
        const float qi = -bq_o(ei, Kk);
        const f2 q_e = bq_e(eo, ee, A, Kk);
        const float q2om = -bq_o(eo, Kk), q2em = q_e.y;
        const f3 E2om = bE_o(A, Kk, q2om);
        const f3 E2em = bE_e(eo, A, Kk, q2em);
        const float A_1 = -E2em.x * E2om.y * Kk * cos_t;
        const float A_2 = -E2em.y * E2om.x * Kk * cos_t;
        const float C_1 = qi * cos_t - Kk * sin_t;
        const float C_2 = E2em.x * E2om.z * (C_1 + q2om * cos_t) - A_1;
        const float C_3 = E2em.z * E2om.x * (C_1 + q2em * cos_t) - A_2;
        const float Ns = C_2 * (qi + q2em) - C_3 * (qi + q2om);
        tpo = -(2.f * E2em.x * cos_t * (q2em + qi) * C_1) / Ns;
        tpe = (2.f * E2om.x * cos_t * (q2om + qi) * C_1) / Ns;
        tso = -(2.f * qi * (E2em.y * Kk * cos_t + E2em.z * C_1 + E2em.z * q2em * cos_t)) / Ns;
        tse = (2.f * qi * (E2om.y * Kk * cos_t + E2om.z * C_1 + E2om.z * q2om * cos_t)) / Ns;
    }
    // fresnel_aniso_iso(I.y, I.z, ei, eo, ee, A2) (Birefringence.slang:137-169)
    float tos, top, tes, tep;
    {
        const float cos_p = I.y, sin_p = I.z;
        const float Kk = ei * sin_p;
        const float q2om = -bq_o(ei, Kk);
        const float qop = bq_o(eo, Kk);
        const f2 q_e = bq_e(eo, ee, A2, Kk);
        const float qep = q_e.x, qem = q_e.y;
        const f3 Eop = bE_o(A2, Kk, qop);
        const f3 Eep = bE_e(eo, A2, Kk, qep);
        const f3 Eom = bE_o(A2, Kk, -qop);
        const f3 Eem = bE_e(eo, A2, Kk, qem);
        const float B_1 = -Eep.x * Kk * cos_p * (q2om - qep);
        const float B_2 = -Eom.x * Kk * cos_p * (q2om + qop);
        const float B_3 = -Eop.x * Kk * cos_p * (qop - q2om);
        const float D_1 = Kk * sin_p - q2om * cos_p;
        const float D_2 = Eep.z * (D_1 + qep * cos_p);
        const float D_3 = Eem.z * (D_1 + qem * cos_p);
        const float D_4 = Eop.z * (D_1 + qop * cos_p);
        const float N2 = (Eep.x * (qep - q2om) * D_4 + Eop.x * (q2om - qop) * D_2 + Eop.y * B_1 + Eep.y * B_3);
        const float roo = -(Eep.x * Eom.z * (q2om - qep) * (qop * cos_p - D_1) + Eom.x * (q2om + qop) * D_2 + Eom.y * B_1 - Eep.y * B_2) / N2;
        const float roe = -(-Eom.x * Eop.z * (qop * (qop * cos_p + Kk * sin_p) + q2om * D_1) +
                            Eom.z * Eop.x * (qop * (qop * cos_p - Kk * sin_p) + q2om * D_1) + Eop.y * B_2 + Eom.y * B_3) / N2;
        tos = (Eep.x * qep * roe - Eom.x * qop + Eop.x * qop * roo) / q2om;
        top = -(Eom.z * qop - Eom.y * Kk - (Eep.y * Kk + Eep.z * qep) * roe - (Eop.y * Kk + Eop.z * qop) * roo) / D_1;
        const float reo = (Eem.x * (qem - q2om) * (D_2 + Eep.y * Kk * cos_p) + Eep.x * (q2om - qep) * (D_3 + Eem.y * Kk * cos_p)) / N2;
        const float ree = -(Eem.x * (qem - q2om) * D_4 - Eem.x * Eop.y * Kk * cos_p * (q2om - qem) + Eem.y * B_3 + Eop.x * (q2om - qop) * D_3) / N2;
        tes = (Eem.x * qem + Eep.x * qep * ree + Eop.x * qop * reo) / q2om;
        tep = -(Eem.z + Eep.z * ree + Eop.z * reo) / cos_p;
    }
    const float ss = tso * tos + tse * tes, sp = tso * top + tse * tep;
    const float ps = tpo * tos + tpe * tes, pp = tpo * top + tpe * tep;
    const float Ioz = fabsf(tauum / Io.y) * Io.z, Iez = fabsf(tauum / Ie.y) * Ie.z;
    const float OPLo = fabsf(tauum / Io.y) * eo, OPLe = fabsf(tauum / Ie.y) * e_eff;
    const float oez = Ioz - Iez;
    const float quad = b.coherenceQuad(Z * oez);
    const float opd = ei * oez * I.z + OPLo - OPLe;
    float nLx[H], nLy[H], newL[H];
    bool allFinite = true, allPos = true;
#pragma unroll
    for (int j = 0; j < H; ++j) {
        const float k = kOfWl(b.wl[j]);
        const float t = b.mutualCoherenceK(k, quad) * 2.f * sinf(-k * opd);
        const float Lx = .5f * (b.L[0][j] + b.L[1][j]), Ly = .5f * (b.L[0][j] - b.L[1][j]);
        const float sq = sqrtf(Lx * Ly);
        nLx[j] = fmaxf(0.f, ss * ss * Lx + ps * ps * Ly + ss * ps * t * sq);
        nLy[j] = fmaxf(0.f, sp * sp * Lx + pp * pp * Ly + sp * pp * t * sq);
        newL[j] = nLx[j] + nLy[j];
        allFinite &= isfinite(newL[j]);
        allPos &= b.L[0][j] > 1e-6f;
    }
#pragma unroll
    for (int j = 0; j < H; ++j) {
        const float norm = (allPos && allFinite) ? newL[j] / b.L[0][j] : 0.f;
        b.L[0][j] = allFinite ? newL[j] : 0.f;
        b.L[1][j] = allFinite ? nLx[j] - nLy[j] : 0.f;
        b.L[2][j] *= norm;
        b.L[3][j] *= norm;
    }
}
template <int H>
PLT_DI void thinEval(const DevMaterial* __restrict__ m, f3 toLight, f3 toEye, uint32_t lobe, DBeam<H>& b) {
    const float* p = m->p;
    const float eta = __ldg(p + PT_ETA) / 1.f;
    const bool isReflection = toLight.z * toEye.z > 0.f;
    const bool isDirect = (lobe & kLobeDelta) != 0;
    const bool hasT = (lobe & kLobeTransmission) != 0, hasR = (lobe & kLobeReflection) != 0;
    if ((isReflection && eta == 1.f) || toLight.z * toEye.z == 0.f || !isDirect || (!hasT && !isReflection) || (!hasR && isReflection)) {
        b.setZero();
        return;
    }
    const float ci = fabsf(toLight.z);
    const FresnelD f = fresnel_dielectric(ci, eta);
    const MM Rm = muellerFresnelReal(f.rs, f.rp), T = muellerFresnelReal(f.ts, f.tp);
    MM iR;
    invOneMinus(Rm, iR);
    const MM M = isReflection ? (iR.a > 0.f ? madd(Rm, mmul(mmul(T, Rm), mmul(iR, T))) : Rm)
                              : (iR.a > 0.f ? mmul(T, mmul(iR, T)) : mmul(T, T));
    if (__ldg(p + PT_BIREF) > 0.f && !isReflection) thinBirefringence<H>(m, b, toLight);
#pragma unroll
    for (int j = 0; j < H; ++j) b.setSP(j, mapply(M, b.getSP(j)));
}
PLT_DI bool thinSample(const DevMaterial* __restrict__ m, f3 wi, f3& wo, float& pdf, float& weight, uint32_t& lobe, SampleGen& sg,
                       uint32_t lobeMask = kLobeAll) {
    const bool hasR = (lobeMask & kLobeReflection) != 0, hasT = (lobeMask & kLobeTransmission) != 0;
    if (!hasR && !hasT) return false;
    const float eta = __ldg(m->p + PT_ETA) / 1.f;
    const float Fd = fresnelR(fresnel_dielectric(fabsf(wi.z), eta));
    const bool isReflection = hasR ? (Fd > 0.f && sg.next1D() <= Fd) : false;
    wo = isReflection ? reflectL(wi) : -wi;
    weight = 1.f;
    pdf = hasR && hasT ? (isReflection ? Fd : 1.f - Fd) : 1.f;
    lobe = isReflection ? kLobeDeltaR : kLobeDeltaT;
    return true;
}

// =============================================================================================
// PLTMultiLayeredStack (PLTMultiLayeredStackBSDF.slang:42-139): scalar Airy recursion, FP32 as
// the reference or FP64 (PLT_OPTION_FP64_MULTILAYER)
// =============================================================================================
struct MLLayer { float ct, th, ior, r; };  // one of the two alternating layers
template <typename RT>
PLT_NI float mlRecursion(float sqrtm00, uint32_t layers, MLLayer l0, MLLayer l1, float Rout, float k) {
    RT gx = (RT)sqrtm00, gy = (RT)0;
    for (uint32_t l = 0; l < layers; ++l) {
        const MLLayer L = (l & 1u) ? l1 : l0;
        const RT d = (RT)2 * (RT)L.th / (RT)L.ct * (RT)k * (RT)L.ior;
        RT sd, cd;
        if constexpr (sizeof(RT) == 8) sincos(d, &sd, &cd);
        else sincosReduced(d, &sd, &cd);
        const RT R = l == layers - 1 ? (RT)Rout : (RT)L.r;
        // G = G * p
        const RT x = gx * cd - gy * sd, y = gx * sd + gy * cd;
        // G = (R + G) / (1 + R G)
        const RT nx = R + x, ny = y;
        const RT dx = (RT)1 + x * R, dy = y * R;
        const RT n = dx * dx + dy * dy;
        if constexpr (sizeof(RT) == 8) {
            gx = (nx * dx + ny * dy) / n;
            gy = (ny * dx - nx * dy) / n;
        } else {  // correctly rounded: the recursion amplifies quotient errors near resonances
            gx = __fdiv_rn(nx * dx + ny * dy, n);
            gy = __fdiv_rn(ny * dx - nx * dy, n);
        }
    }
    return (float)(gx * gx);
}
template <int H>
PLT_DI void mlEval(const DevMaterial* __restrict__ m, const Ctx& c, f3 toLight, f3 toEye, uint32_t lobe, DBeam<H>& b) {
    const float* p = m->p;
    const bool isReflection = toLight.z * toEye.z > 0.f;
    if ((lobe & kLobeDelta) == 0 || !isReflection) { b.setZero(); return; }
    const float eta1 = __ldg(p + PM_ETA1), eta2 = __ldg(p + PM_ETA2);
    const FresnelD f0 = fresnel_dielectric(toLight.z, eta1);
    const float Rout = sqrtf(fresnelR(f0));
    const FresnelD f1 = fresnel_dielectric(-f0.cosT, eta2);
    const float r0 = sqrtf(fresnelR(f1));
    const float r1 = sqrtf(fresnelR(fresnel_dielectric(f1.cosT, eta2)));
    const MLLayer l0{fabsf(f0.cosT), __ldg(p + PM_TH1), __ldg(p + PM_IOR1), r0};
    const MLLayer l1{fabsf(f1.cosT), __ldg(p + PM_TH2), __ldg(p + PM_IOR2), r1};
    const uint32_t layers = m->aux;
#pragma unroll
    for (int j = 0; j < H; ++j) {
        const float sm = sqrtf(m00Of(m->m00a, b.wl[j]));
        const float k = kOfWl(b.wl[j]);
        const float g2 = (c.flags & 1u) ? mlRecursion<double>(sm, layers, l0, l1, Rout, k)
                                        : mlRecursion<float>(sm, layers, l0, l1, Rout, k);
        b.setSP(j, g2 * b.getSP(j));
    }
}

// =============================================================================================
// PLTDiffuse (PLTDiffuseBSDF.slang:40-95)
// =============================================================================================
template <int H>
PLT_DI void diffEval(const DevMaterial* __restrict__ m, f3 toLight, uint32_t lobe, DBeam<H>& b) {
    const bool valid = (lobe & kLobeDiffuseR) != 0;
#pragma unroll
    for (int j = 0; j < H; ++j) {
        const float w = valid ? fabsf(toLight.z) * k1_Pi * m00Of(m->m00a, b.wl[j]) : 0.f;
        b.L[0][j] *= w;
        b.L[1][j] = b.L[2][j] = b.L[3][j] = 0.f;
    }
}
PLT_DI bool diffSample(const DevMaterial* __restrict__ m, f3& wo, float& pdf, float& weight, uint32_t& lobe, SampleGen& sg, float wl) {
    weight = m00Of(m->m00a, wl);
    float ux = 2.f * sg.next1D() - 1.f, uy = 2.f * sg.next1D() - 1.f;
    float dx = ux, dy = uy;
    if (!(ux == 0.f && uy == 0.f)) {
        float r, phi;
        if (fabsf(ux) > fabsf(uy)) { r = ux; phi = (uy / ux) * (kPi / 4.f); }
        else { r = uy; phi = kPi / 2.f - (ux / uy) * (kPi / 4.f); }
        float s, c;
        sincosf(phi, &s, &c);
        dx = r * c;
        dy = r * s;
    }
    const float z = sqrtf(fmaxf(0.f, 1.f - (dx * dx + dy * dy)));
    pdf = z * k1_Pi;
    wo = mk3(dx, dy, z);
    lobe = kLobeDiffuseR;
    return true;
}

}  // namespace pltdev
