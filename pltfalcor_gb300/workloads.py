"""Seeded synthetic BSDF-query workloads.

All randomness is counter-based and portable: query i draws from the library's own sample
generator, UniformSampleGenerator(pixel = (i & 0xffff, i >> 16), sampleNumber = seed)
(SplitMix64-seeded xoshiro128**, Utils/Sampling/UniformSampleGenerator.slang:51-66 in the
reference), evaluated here with numpy integer arithmetic, so the same seed gives the same inputs on
every host.

rough_dielectric_batch: 65,536 PLTDielectric eval + pdf queries, seed 0 -- wi, wo uniform in solid
  angle over the upper hemisphere with cos >= 0.01; wavelength U[380, 780] nm; IoR 1.5, Cauchy
  B = 0.0042 um^2; roughness U[0.01, 0.5] mapped by the material's own GaussianSurface conversion;
  coherence area U[5, 50] um^2 at r = 1 m; unpolarised Stokes (1, 0, 0, 0); all lobes.
mixed_material_batch: 2^22 eval + sample + pdf queries, seed 1, split equally over the eight PLT
  types in shuffled order; each query carries one lobe of its material (the lobe a path tracer
  would pass to eval); conductors use the Au/Ag/Cu/Al tables; coatings 0.1-1 um, n 1.38-1.6;
  1-D sinusoidal gratings, pitch 0.5-5 um, depth 0.05-0.3 um, 5 lobes; multilayer stacks of 2-32
  alternating layers, n = 1.38 / 2.3, 0.05-0.5 um; birefringent thin film, delta-n 0.01-0.2,
  1 um thick; Stokes vectors uniform on the Poincare sphere with degree of polarisation U[0, 1].
"""
import numpy as np

from . import materials as M

U64 = np.uint64


def _interleave16(v):
    v = v.astype(np.uint32) & np.uint32(0xFFFF)
    v = (v | (v << np.uint32(8))) & np.uint32(0x00FF00FF)
    v = (v | (v << np.uint32(4))) & np.uint32(0x0F0F0F0F)
    v = (v | (v << np.uint32(2))) & np.uint32(0x33333333)
    v = (v | (v << np.uint32(1))) & np.uint32(0x55555555)
    return v


def _splitmix64(state):
    state = state + U64(0x9E3779B97F4A7C15)
    z = state
    z = (z ^ (z >> U64(30))) * U64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> U64(27))) * U64(0x94D049BB133111EB)
    return state, z ^ (z >> U64(31))


def _rotl(x, k):
    return (x << np.uint32(k)) | (x >> np.uint32(32 - k))


class CounterRNG:
    """Vectorised UniformSampleGenerator over query indices [offset, offset + n)."""

    def __init__(self, seed, n, offset=0):
        idx = np.arange(offset, offset + n, dtype=np.uint64)
        px = (idx & U64(0xFFFF)).astype(np.uint32)
        py = (idx >> U64(16)).astype(np.uint32)
        with np.errstate(over="ignore"):
            st = (U64(seed) << U64(32)) | (_interleave16(px) | (_interleave16(py) << np.uint32(1))).astype(np.uint64)
            st, a = _splitmix64(st)
            st, b = _splitmix64(st)
        self.s = [(a & U64(0xFFFFFFFF)).astype(np.uint32), (a >> U64(32)).astype(np.uint32),
                  (b & U64(0xFFFFFFFF)).astype(np.uint32), (b >> U64(32)).astype(np.uint32)]

    def next_u32(self):
        s0, s1, s2, s3 = self.s
        with np.errstate(over="ignore"):
            result = _rotl(s0 * np.uint32(5), 7) * np.uint32(9)
        t = s1 << np.uint32(9)
        s2 = s2 ^ s0
        s3 = s3 ^ s1
        s1 = s1 ^ s2
        s0 = s0 ^ s3
        s2 = s2 ^ t
        s3 = _rotl(s3, 11)
        self.s = [s0, s1, s2, s3]
        return result

    def uniform(self):
        """(bits >> 8) * 2^-24 as float32, SampleGeneratorInterface.slang:46-52."""
        return (self.next_u32() >> np.uint32(8)).astype(np.float32) * np.float32(2.0 ** -24)


def _hemisphere(rng, min_cos=0.01):
    z = min_cos + (1.0 - min_cos) * rng.uniform().astype(np.float64)
    phi = 2.0 * np.pi * rng.uniform().astype(np.float64)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return np.stack([s * np.cos(phi), s * np.sin(phi), z]).astype(np.float32)


def _coherence(rng, wavelengths_nm, r_m=1.0):
    """Isotropic diffusivity D = d I at distance r, with d = pi (lambda_um r_mm)^2 / A and the
    coherence area A ~ U[5, 50] um^2 (coherenceArea = pi sqrt(det Theta), PLT.slang:57-68,190-192)."""
    A = 5.0 + 45.0 * rng.uniform().astype(np.float64)
    lam_um = wavelengths_nm.astype(np.float64) * 1e-3
    d = np.pi * (lam_um * r_m * 1e3) ** 2 / A
    n = len(A)
    return np.stack([d, np.zeros(n), d, np.full(n, r_m)]).astype(np.float32)


class Workload:
    """SoA host arrays of one batch plus its material and spectral tables."""

    def __init__(self, name, n, hwss, material, v, w, lobe, wavelengths, stokes, coherence, records, profiles,
                 ops, frame=0, meta=None):
        self.name, self.n, self.hwss = name, n, hwss
        self.material = np.ascontiguousarray(material, np.uint32)
        self.v = np.ascontiguousarray(v, np.float32)
        self.w = np.ascontiguousarray(w, np.float32)
        self.lobe = None if lobe is None else np.ascontiguousarray(lobe, np.uint32)
        self.wavelengths = np.ascontiguousarray(wavelengths, np.float32)
        self.stokes = np.ascontiguousarray(stokes, np.float32)
        self.coherence = np.ascontiguousarray(coherence, np.float32)
        self.records = records
        self.profiles = profiles
        self.ops = ops
        self.frame = frame
        self.meta = meta or {}

    def input_bytes(self):
        b = self.material.nbytes + self.v.nbytes + self.w.nbytes + self.wavelengths.nbytes + self.stokes.nbytes + self.coherence.nbytes
        return b + (self.lobe.nbytes if self.lobe is not None else 0)

    def subset(self, idx):
        """Queries idx (kept with their materials), for oracle-sized checks."""
        idx = np.asarray(idx)
        n = len(idx)
        sl = lambda a, c: a.reshape(c, -1)[:, idx].reshape(-1)
        return Workload(self.name + "[subset]", n, self.hwss, self.material[idx], sl(self.v, 3), sl(self.w, 3),
                        None if self.lobe is None else self.lobe[idx], sl(self.wavelengths, self.hwss),
                        sl(self.stokes, 4 * self.hwss), sl(self.coherence, 4), self.records, self.profiles, self.ops,
                        self.frame, dict(self.meta))


def rough_dielectric_batch(n=65536, seed=0, profiles=None):
    rng = CounterRNG(seed, n)
    v = _hemisphere(rng)
    w = _hemisphere(rng)
    wl = (380.0 + 400.0 * rng.uniform().astype(np.float64)).astype(np.float32)
    rough = (0.01 + 0.49 * rng.uniform().astype(np.float64)).astype(np.float32)
    coh = _coherence(rng, wl)
    recs = M.dielectric(n, rough, ior=1.5, dispersion_b=0.0042)
    stokes = np.zeros((4, n), np.float32)
    stokes[0] = 1.0
    from . import capi
    return Workload("rough_dielectric_65536", n, 1, np.arange(n, dtype=np.uint32), v.reshape(-1), w.reshape(-1), None,
                    wl, stokes.reshape(-1), coh.reshape(-1), recs, profiles, capi.OP_EVAL | capi.OP_PDF, 0,
                    {"seed": seed})


def mixed_material_records(per_type=4096, seed=1):
    """per_type random materials of each BENCH_TYPES type, drawn with generator seed + 1000."""
    ntot = per_type * len(M.BENCH_TYPES)
    rng = CounterRNG(seed + 1000, ntot)
    u = [rng.uniform().astype(np.float64) for _ in range(12)]
    recs = []
    sl = lambda a, t: a[t * per_type:(t + 1) * per_type]
    for t, ty in enumerate(M.BENCH_TYPES):
        rough = 0.01 + 0.49 * sl(u[0], t)
        metal = np.minimum((sl(u[1], t) * 4).astype(np.int64), 3)
        albedo = np.stack([0.2 + 0.8 * sl(u[k], t) for k in (2, 3, 4)], 1)
        n = per_type
        if ty == M.DIELECTRIC:
            r = M.dielectric(n, rough, ior=1.5, dispersion_b=0.0042)
        elif ty == M.CONDUCTOR:
            r = M.conductor(n, rough, 2 * metal, 2 * metal + 1, specular=albedo)
        elif ty in (M.COATED_OPAQUE_DIELECTRIC, M.COATED_CONDUCTOR):
            tau = 0.1 + 0.9 * sl(u[5], t)
            cn = 1.38 + 0.22 * sl(u[6], t)
            cond = ty == M.COATED_CONDUCTOR
            r = M.coated(n, cond, rough, tau, cn, albedo=albedo, ior_n_id=2 * metal if cond else M.NO_PROFILE,
                         ior_k_id=2 * metal + 1 if cond else M.NO_PROFILE)
        elif ty in (M.GRATED_OPAQUE_DIELECTRIC, M.GRATED_CONDUCTOR):
            pitch = 0.5 + 4.5 * sl(u[5], t)
            depth = 0.05 + 0.25 * sl(u[6], t)
            direction = np.pi * sl(u[7], t)
            cond = ty == M.GRATED_CONDUCTOR
            r = M.grated(n, cond, pitch, depth, 0.0, direction, 1.0, 1.0, 5, M.GRATING_SINUSOIDAL, rough, albedo=albedo,
                         ior_n_id=2 * metal if cond else M.NO_PROFILE, ior_k_id=2 * metal + 1 if cond else M.NO_PROFILE)
        elif ty == M.THIN_DIELECTRIC:
            dn = 0.01 + 0.19 * sl(u[5], t)
            r = M.thin_dielectric(n, 1.5, thickness_mm=0.001, birefringence=dn)
        else:
            layers = 2 + np.minimum((sl(u[5], t) * 31).astype(np.int64), 30)
            d1 = 0.05 + 0.45 * sl(u[6], t)
            d2 = 0.05 + 0.45 * sl(u[7], t)
            r = M.multilayered_stack(n, layers, 1.38, 2.3, d1, d2, albedo=albedo)
        recs.append(r)
    return np.concatenate(recs)


def mixed_material_batch(n=1 << 22, seed=1, per_type=4096, profiles=None, hwss=1):
    from . import capi
    T = len(M.BENCH_TYPES)
    assert n % T == 0
    recs = mixed_material_records(per_type, seed)
    rng = CounterRNG(seed, n)
    # balanced types in shuffled order
    keys = rng.next_u32()
    order = np.argsort(keys, kind="stable")
    tsel = np.empty(n, np.int64)
    tsel[order] = np.arange(n) % T
    mat = (tsel * per_type + np.minimum((rng.uniform().astype(np.float64) * per_type).astype(np.int64), per_type - 1)).astype(np.uint32)
    v = _hemisphere(rng)
    w = _hemisphere(rng)
    # one lobe of the material per query
    ul = rng.uniform().astype(np.float64)
    uo = rng.uniform().astype(np.float64)
    lobe = np.zeros(n, np.uint32)
    for t, ty in enumerate(M.BENCH_TYPES):
        sel = tsel == t
        lobes = M.lobes_of(ty)
        k = np.minimum((ul[sel] * len(lobes)).astype(np.int64), len(lobes) - 1)
        lv = np.asarray(lobes, np.uint32)[k]
        if ty in (M.GRATED_CONDUCTOR, M.GRATED_OPAQUE_DIELECTRIC):
            dsel = lv == M.LOBE_DISP_DELTA_R
            order_m = 1 + np.minimum((uo[sel] * 10).astype(np.int64), 9)      # 1..10 -> +-1..5
            mval = np.where(order_m > 5, -(order_m - 5), order_m)
            lv = np.where(dsel, M.encode_grating_lobe(mval, 0), lv)
        lobe[sel] = lv
    # transmission lobes see the lower hemisphere
    trans = (lobe & 0xF0) != 0
    w[2, trans] = -w[2, trans]
    wl = np.empty((hwss, n), np.float32)
    wl[0] = (380.0 + 400.0 * rng.uniform().astype(np.float64)).astype(np.float32)
    for j in range(1, hwss):  # hero-wavelength stratification (SpectrumSampler.slang:38-54)
        x = wl[0].astype(np.float64) + j * 340.0 / hwss
        wl[j] = np.where(x > 720.0, x - 340.0, x).astype(np.float32)
    sz = 2.0 * rng.uniform().astype(np.float64) - 1.0
    sphi = 2.0 * np.pi * rng.uniform().astype(np.float64)
    dop = rng.uniform().astype(np.float64)
    sr = np.sqrt(np.maximum(0.0, 1 - sz * sz))
    stokes = np.zeros((4, hwss, n), np.float32)
    stokes[0] = 1.0
    stokes[1] = (dop * sr * np.cos(sphi)).astype(np.float32)
    stokes[2] = (dop * sr * np.sin(sphi)).astype(np.float32)
    stokes[3] = (dop * sz).astype(np.float32)
    coh = _coherence(rng, wl[0])
    return Workload("mixed_material_%d" % n, n, hwss, mat, v.reshape(-1), w.reshape(-1), lobe, wl.reshape(-1),
                    stokes.reshape(-1), coh.reshape(-1), recs, profiles, capi.OP_EVAL | capi.OP_SAMPLE | capi.OP_PDF,
                    1, {"seed": seed, "types": tsel.astype(np.uint8)})
