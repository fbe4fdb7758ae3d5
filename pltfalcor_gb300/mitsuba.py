"""Mitsuba 3 scene import for the render pass.

Follows the reference's importer (plugins/importers/MitsubaImporter/MitsubaImporter.cpp inside
ssteinberg/PLTFalcor), whose BSDFs map onto PLT materials (buildBSDF, MitsubaImporter.cpp:288-520):

- diffuse -> PLTDiffuse (baseColor = reflectance, default 0.5);
- dielectric / roughdielectric -> PLTDielectric: IoR and Abbe number from int_ior (a name of the
  IOR table or a float, default "bk7"), ext_ior (default "air"), specular_reflectance as base colour,
  specular_transmittance as transmission colour, roughness or convertGSSigma2(sigma2 = 100);
- thindielectric -> PLTThinDielectric: IoR from int_ior, thickness (default 0.001), optic_axis
  (default +z), birefringence_scale (default 1) and birefringence (default 0);
- conductor / roughconductor -> PLTConductor: specular_reflectance as base colour, the (n, k)
  profiles of a named material (Tables/ior/<name>.{eta,k}.spd) or of eta and k spectra, ext_ior,
  roughness;
- coated_conductor / coated_roughconductor -> PLTCoatedConductor from its nested conductor, coat
  IoR int_ior (default "bk7") and thickness (default 50);
- grating -> PLTDiffractionGratedConductor: (n, k) as the conductor, pitch (5), lobes (3), q (0.5),
  height 1, grating_direction (degrees), amplify (1), type;
- twosided -> its nested BSDF, double-sided; normalmap -> its nested BSDF (textures unsupported);
- anything else -> PLTDiffuse red (1, 0, 0), as the reference does, with a warning.

Emitters: an area emitter nested in a shape gives its material an emission profile (the
emission_profile table scaled by scale, else the radiance RGB through rgbToSpectrum); constant and
envmap (a .pfm image) become the environment map; point (sourcing area A) and directional lights
become analytic lights.  Sensor: perspective with fov (taken along x, as the reference's focal
length arithmetic does), to_world lookat, film width and height.  Shapes: obj, ply, rectangle,
cube, sphere, disk, with to_world transforms.
"""
import os
import xml.etree.ElementTree as ET

import numpy as np

from . import materials as M

INF = float("inf")
# MitsubaImporter/Tables.h: IOR name -> (IoR, Abbe number)
IOR_TABLE = {
    "vacuum": (1.0, INF), "helium": (1.000036, INF), "hydrogen": (1.000132, INF), "air": (1.000277, INF),
    "carbon dioxide": (1.00045, INF), "water": (1.3330, 55.0), "acetone": (1.36, 54.0), "ethanol": (1.361, 59.0),
    "carbon tetrachloride": (1.461, 49.0), "glycerol": (1.4729, INF), "benzene": (1.501, 30.3), "silicone oil": (1.52045, INF),
    "bromine": (1.661, 31.7), "water ice": (1.31, 64.0), "fused quartz": (1.458, 67.8), "pyrex": (1.470, 60.0),
    "acrylic glass": (1.49, INF), "polypropylene": (1.49, INF), "bk7": (1.5046, 64.0), "sodium chloride": (1.544, 42.9),
    "amber": (1.55, INF), "pet": (1.5750, INF), "diamond": (2.419, 55.3),
}
# 11-bin basis of SpectrumUtils::rgbToSpectrum (Utils/Color/SpectrumUtils.h:154-200)
_BASIS = {
    "white": (1.0, 1.0, 0.9999, 0.9993, 0.9992, 0.9998, 1.0, 1.0, 1.0, 1.0, 0.0),
    "cyan": (0.9710, 0.9426, 1.0007, 1.0007, 1.0007, 1.0007, 0.1564, 0.0, 0.0, 0.0, 0.0),
    "magenta": (1.0, 1.0, 0.968, 0.22295, 0.0, 0.0458, 0.8369, 1.0, 1.0, 0.9959, 0.0),
    "yellow": (0.0001, 0.0, 0.1088, 0.6651, 1.0, 1.0, 0.9996, 0.9586, 0.9685, 0.9840, 0.0),
    "red": (0.1012, 0.0515, 0.0, 0.0, 0.0, 0.0, 0.8325, 1.0149, 1.0149, 1.014, 0.0),
    "green": (0.0, 0.0, 0.0273, 0.7937, 1.0, 0.9418, 0.1719, 0.0, 0.0, 0.0025, 0.0),
    "blue": (1.0, 1.0, 0.8916, 0.3323, 0.0, 0.0, 0.0003, 0.0369, 0.0483, 0.0496, 0.0),
}


def lookup_ior(name):
    """lookupIOR: a table entry by lower-cased name; unknown names warn and give air."""
    return IOR_TABLE.get(str(name).lower())


def convert_gs_sigma2(sigma2):
    """convertGSSigma2 (MitsubaImporter.cpp:182-184)."""
    return float(np.clip(2.0 * (1.0 - max(0.0, sigma2 / 1000.0) ** (1.0 / 32.0)), 0.0, 1.0))


def rgb_to_spectrum_samples(rgb, samples=16):
    """SpectrumUtils::rgbToSpectrum<float>(rgb, 16): (wavelengths, values) over 380-720 nm."""
    r, g, b = (float(x) for x in rgb)
    wl = np.array([380.0 + (720.0 - 380.0) / (samples - 1) * i for i in range(samples)], np.float32)
    out = np.zeros(samples, np.float64)
    for i, w in enumerate(wl):
        k = min(10, max(0, int((w - 380.0) / (720.0 - 380.0) * 10.0)))
        B = {n: v[k] for n, v in _BASIS.items()}
        if r <= g and r <= b:
            s = B["white"] * r + (B["cyan"] * (g - r) + B["blue"] * (b - g) if g <= b else B["cyan"] * (b - r) + B["green"] * (g - b))
        elif g <= r and g <= b:
            s = B["white"] * g + (B["magenta"] * (r - g) + B["blue"] * (b - r) if r <= b else B["magenta"] * (b - g) + B["red"] * (r - b))
        else:
            s = B["white"] * b + (B["yellow"] * (r - b) + B["green"] * (g - r) if r <= g else B["yellow"] * (g - b) + B["red"] * (r - g))
        out[i] = s
    return wl, out.astype(np.float32)


def _f16(bits):
    return float(np.asarray(bits, np.uint16).view(np.float16))


def _vec(s):
    return [float(x) for x in str(s).replace(",", " ").split()]


def _rotation(axis, deg):
    a = np.radians(deg)
    k = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    m = np.eye(4)
    m[:3, :3] = np.eye(3) + np.sin(a) * K + (1 - np.cos(a)) * (K @ K)
    return m


class _Reader:
    """Mitsuba XML: objects with properties, references and nested objects; $name defaults."""

    def __init__(self, path):
        self.base = os.path.dirname(os.path.abspath(path))
        self.defaults = {}
        self.ids = {}
        root = ET.parse(path).getroot()
        self.root = root

    def attr(self, el, name, default=None):
        v = el.get(name, default)
        if isinstance(v, str) and v.startswith("$"):
            v = self.defaults.get(v[1:], v)
        return v

    def transform(self, el):
        m = np.eye(4)
        look = None
        for c in el:
            t = np.eye(4)
            if c.tag == "translate":
                v = _vec(self.attr(c, "value")) if c.get("value") else [float(self.attr(c, k, 0)) for k in "xyz"]
                t[:3, 3] = v
            elif c.tag == "scale":
                if c.get("value"):
                    v = _vec(self.attr(c, "value"))
                    v = v * 3 if len(v) == 1 else v
                else:
                    v = [float(self.attr(c, k, 1)) for k in "xyz"]
                t = np.diag(v + [1.0])
            elif c.tag == "rotate":
                axis = _vec(self.attr(c, "value")) if c.get("value") else [float(self.attr(c, k, 0)) for k in "xyz"]
                t = _rotation(axis, float(self.attr(c, "angle")))
            elif c.tag == "matrix":
                t = np.array(_vec(self.attr(c, "value")), np.float64).reshape(4, 4)
            elif c.tag == "lookat":
                o, tg = np.array(_vec(self.attr(c, "origin"))), np.array(_vec(self.attr(c, "target")))
                up = np.array(_vec(self.attr(c, "up", "0 1 0")))
                z = (tg - o) / np.linalg.norm(tg - o)
                x = np.cross(up, z)
                x /= np.linalg.norm(x)
                y = np.cross(z, x)
                t[:3, 0], t[:3, 1], t[:3, 2], t[:3, 3] = x, y, z, o
                look = (o, tg, up)
            m = t @ m
        return m, look

    def props(self, el):
        """(properties, nested objects, references) of an object element."""
        p, nested, refs = {}, [], []
        for c in el:
            name = self.attr(c, "name")
            if c.tag in ("float",):
                p[name] = float(self.attr(c, "value"))
            elif c.tag == "integer":
                p[name] = int(float(self.attr(c, "value")))
            elif c.tag == "boolean":
                p[name] = str(self.attr(c, "value")).lower() == "true"
            elif c.tag == "string":
                p[name] = self.attr(c, "value")
            elif c.tag in ("rgb", "color"):
                v = _vec(self.attr(c, "value"))
                p[name] = ("rgb", tuple(v * 3 if len(v) == 1 else v[:3]))
            elif c.tag == "spectrum":
                v = str(self.attr(c, "value", ""))
                if ":" in v:
                    pairs = [tuple(float(y) for y in x.split(":")) for x in v.replace(",", " ").split()]
                    p[name] = ("spectrum", pairs)
                elif v:
                    p[name] = ("rgb", (float(v),) * 3)
            elif c.tag in ("point", "vector"):
                p[name] = tuple(_vec(self.attr(c, "value"))) if c.get("value") else tuple(float(self.attr(c, k, 0)) for k in "xyz")
            elif c.tag == "transform":
                p[name] = self.transform(c)
            elif c.tag == "ref":
                refs.append((name, self.attr(c, "id")))
            elif c.tag in ("bsdf", "emitter", "shape", "texture", "film", "sampler", "rfilter", "medium"):
                nested.append(c)
        return p, nested, refs


class MitsubaScene:
    """Import result: geometry, material records, profile requests, camera, lights, environment."""

    def __init__(self):
        self.vertices, self.normals, self.indices, self.tri_material = [], [], [], []
        self.records = []
        self.profiles = []          # extra profiles after the standard ones: ("samples", wl, v, scale, icdf) | ("ior", name) | ("emission", name, scale)
        self.camera = None
        self.width, self.height = 768, 576
        self.lights = []            # (kind, dict)
        self.env = None
        self.emissive_materials = []
        self.warnings = []


_METALS = {"au": 0, "ag": 1, "cu": 2, "al": 3}   # standard_profiles order


class _Builder(_Reader):
    def __init__(self, path, out):
        super().__init__(path)
        self.out = out
        for c in self.root:
            if c.tag == "default":
                self.defaults[c.get("name")] = c.get("value")
        for el in self.root.iter():
            if el.get("id") is not None and el.tag != "ref":
                self.ids[el.get("id")] = el

    def warn(self, m):
        self.out.warnings.append(m)

    def profile(self, req):
        self.out.profiles.append(req)
        return 9 + len(self.out.profiles) - 1    # after the 9 standard profiles

    def rgb(self, p, name, default):
        v = p.get(name)
        if isinstance(v, tuple) and v and v[0] == "rgb":
            return v[1]
        return (v, v, v) if isinstance(v, float) else default

    def ior(self, p, name, default):
        """lookupIOR(props, name, default): a float (Abbe infinite) or a table name."""
        v = p.get(name, default)
        if isinstance(v, float):
            return v, INF
        e = lookup_ior(v)
        if e is None:
            self.warn("'%s' is not a valid IOR name" % v)
            return IOR_TABLE["air"]
        return e

    def nk(self, p, what):
        """(n, k) profile ids of a conductor: a named material or eta / k spectra."""
        if "material" in p:
            nm = str(p["material"]).lower()
            if nm in _METALS:
                return 2 * _METALS[nm], 2 * _METALS[nm] + 1
            i = self.profile(("ior", p["material"]))
            self.out.profiles.append(("ior_k", p["material"]))
            return i, i + 1
        if "eta" in p and "k" in p:
            ids = []
            for key in ("eta", "k"):
                v = p[key]
                if v[0] == "spectrum":
                    wl, vals = zip(*v[1])
                    ids.append(self.profile(("samples", np.array(wl, np.float32), np.array(vals, np.float32), 1.0, False)))
                else:
                    wl, vals = rgb_to_spectrum_samples(v[1])
                    ids.append(self.profile(("samples", wl, vals, 1.0, False)))
            return ids[0], ids[1]
        raise ValueError("'%s' BSDF must specify either 'eta' and 'k' IOR values or 'material' name." % what)

    def bsdf(self, el):
        ty = el.get("type")
        p, nested, refs = self.props(el)
        kids = [c for c in nested if c.tag == "bsdf"] + [self.ids[i] for _, i in refs if i in self.ids and self.ids[i].tag == "bsdf"]
        ext = self.ior(p, "ext_ior", "air")[0]
        if ty == "diffuse":
            return M.diffuse(1, albedo=self.rgb(p, "reflectance", (0.5, 0.5, 0.5)))
        if ty in ("dielectric", "roughdielectric"):
            eta, abbe = self.ior(p, "int_ior", "bk7")
            rough = p["roughness"] if "roughness" in p else convert_gs_sigma2(p.get("sigma2", 100.0))
            # setAbbeNumber after setIndexOfRefraction: Cauchy B = 0.52 (IoR - 1) / Abbe
            return M.dielectric(1, rough, ior=eta, ext_ior=ext, dispersion_b=0.52 * (eta - 1.0) / abbe,
                                specular=self.rgb(p, "specular_reflectance", (1, 1, 1)),
                                transmission=self.rgb(p, "specular_transmittance", (1, 1, 1)))
        if ty == "thindielectric":
            eta, _ = self.ior(p, "int_ior", "bk7")
            ax = np.asarray(p.get("optic_axis", (0.0, 0.0, 1.0)), np.float64)
            ax = ax / np.linalg.norm(ax)
            ax = -ax if ax[2] < 0 else ax
            bire = self.rgb(p, "birefringence", (0.0, 0.0, 0.0))[0] if "birefringence" in p and isinstance(p["birefringence"], tuple) \
                else float(p.get("birefringence", 0.0))
            return M.thin_dielectric(1, eta, thickness_mm=p.get("thickness", 0.001), birefringence=p.get("birefringence_scale", 1.0),
                                     birefringence_scale=bire, optic_axis_xy=(ax[0], ax[1]))
        if ty in ("conductor", "roughconductor"):
            n, k = self.nk(p, "conductor")
            return M.conductor(1, p.get("roughness", 0.0), n, k, ext_ior=ext, specular=self.rgb(p, "specular_reflectance", (1, 1, 1)))
        if ty in ("coated_conductor", "coated_roughconductor"):
            if len(kids) != 1 or kids[0].get("type") not in ("conductor", "roughconductor"):
                raise ValueError("'coatedConductor' BSDF must contain only a nested 'conductor' BSDF.")
            c = self.bsdf(kids[0])
            eta, _ = self.ior(p, "int_ior", "bk7")
            r = M.coated(1, True, _f16(c["specular"][0][1]), p.get("thickness", 50.0), eta, ext_ior=_f16(c["ior"][0]),
                         ior_n_id=int(c["ior_n_spectral_id"][0]), ior_k_id=int(c["ior_k_spectral_id"][0]))
            r["base_color"] = c["base_color"]
            return r
        if ty == "grating":
            n, k = self.nk(p, "grating")
            types = {"sinusoidal": M.GRATING_SINUSOIDAL, "rectangular": M.GRATING_RECTANGULAR, "linear": M.GRATING_LINEAR}
            gt = types.get(p.get("type", "sinusoidal"))
            if gt is None:
                raise ValueError("Unsupported 'type' name (radial gratings need surface uv).")
            return M.grated(1, True, p.get("pitch", 5.0), 1.0, direction=np.radians(p.get("grating_direction", 0.0)),
                            height_scale=p.get("q", 0.5), power_multiplier=p.get("amplify", 1.0), lobes=p.get("lobes", 3),
                            grating_type=gt, ext_ior=ext, ior_n_id=n, ior_k_id=k)
        if ty in ("twosided", "normalmap"):
            if len(kids) != 1:
                raise ValueError("'%s' BSDF must contain a single nested BSDF." % ty)
            r = self.bsdf(kids[0])
            if ty == "twosided":
                r["flags"] |= 1
            else:
                self.warn("normal map ignored (textures are not supported)")
            return r
        self.warn("BSDF %r mapped to PLTDiffuse red" % ty)
        return M.diffuse(1, albedo=(1.0, 0.0, 0.0))

    # ---- shapes ----
    def geometry(self, ty, p):
        from .scene import icosphere
        if ty in ("obj", "ply"):
            fn = os.path.join(self.base, p["filename"])
            if ty == "ply":
                from .pbrt import read_ply
                return read_ply(fn)
            return read_obj(fn)
        if ty == "rectangle":
            P = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float64)
            return P, np.array([[0, 1, 2], [0, 2, 3]]), np.tile([0.0, 0.0, 1.0], (4, 1))
        if ty == "disk":
            a = np.linspace(0, 2 * np.pi, 65)[:-1]
            P = np.concatenate([[[0.0, 0.0, 0.0]], np.stack([np.cos(a), np.sin(a), 0 * a], 1)])
            I = np.array([[0, 1 + i, 1 + (i + 1) % 64] for i in range(64)])
            return P, I, np.tile([0.0, 0.0, 1.0], (len(P), 1))
        if ty == "cube":
            P, I, N = [], [], []
            for ax in range(3):
                for s in (-1.0, 1.0):
                    u, v = [(ax + 1) % 3, (ax + 2) % 3]
                    q = np.zeros((4, 3))
                    q[:, ax] = s
                    q[:, u] = [-1, 1, 1, -1]
                    q[:, v] = [-1, -1, 1, 1]
                    n = np.zeros(3)
                    n[ax] = s
                    b = len(P) * 4
                    f = [[b, b + 1, b + 2], [b, b + 2, b + 3]] if s > 0 else [[b, b + 2, b + 1], [b, b + 3, b + 2]]
                    P.append(q)
                    N.append(np.tile(n, (4, 1)))
                    I += f
            return np.concatenate(P), np.array(I), np.concatenate(N)
        if ty == "sphere":
            v, f = icosphere(3)
            c = np.asarray(p.get("center", (0.0, 0.0, 0.0)), np.float64)
            return v * p.get("radius", 1.0) + c, f.astype(np.int64), v
        self.warn("shape %r not supported" % ty)
        return None

    def shape(self, el):
        p, nested, refs = self.props(el)
        g = self.geometry(el.get("type"), p)
        if g is None:
            return
        P, I, N = g
        bsdfs = [c for c in nested if c.tag == "bsdf"] + [self.ids[i] for _, i in refs if i in self.ids and self.ids[i].tag == "bsdf"]
        rec = self.bsdf(bsdfs[0]) if bsdfs else M.diffuse(1, albedo=(0.5, 0.5, 0.5))
        for em in [c for c in nested if c.tag == "emitter" and c.get("type") == "area"]:
            ep, _, _ = self.props(em)
            if "emission_profile" in ep:
                rec["emission_spectral_id"] = self.profile(("emission", ep["emission_profile"], ep.get("scale", 1.0)))
            else:
                wl, vals = rgb_to_spectrum_samples(self.rgb(ep, "radiance", (1.0, 1.0, 1.0)))
                rec["emission_spectral_id"] = self.profile(("samples", wl, vals, 1.0, True))
            if int(rec["type"][0]) != M.DIFFUSE:
                self.warn("emission on a non-PLTDiffuse material is ignored by the render pass")
            self.out.emissive_materials.append(len(self.out.records))
        self.out.records.append(rec)
        mi = len(self.out.records) - 1
        T = p.get("to_world", (np.eye(4), None))[0]
        W = (T @ np.concatenate([P, np.ones((len(P), 1))], 1).T).T[:, :3]
        if N is None:
            N = np.zeros_like(W)
            tri = W[I]
            fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
            for c in range(3):
                np.add.at(N, I[:, c], fn)
        else:
            N = (np.linalg.inv(T[:3, :3]).T @ np.asarray(N, np.float64).T).T
        N = N / np.maximum(np.linalg.norm(N, axis=1, keepdims=True), 1e-30)
        base = sum(len(v) for v in self.out.vertices)
        self.out.vertices.append(W)
        self.out.normals.append(N)
        self.out.indices.append(np.asarray(I, np.int64) + base)
        self.out.tri_material.append(np.full(len(I), mi, np.uint32))

    # ---- sensor and emitters ----
    def sensor(self, el):
        p, nested, _ = self.props(el)
        for c in nested:
            if c.tag == "film":
                fp, _, _ = self.props(c)
                self.out.width, self.out.height = int(fp.get("width", 768)), int(fp.get("height", 576))
        T, look = p.get("to_world", (np.eye(4), None))
        if look is None:
            eye = T[:3, 3]
            look = (eye, eye + T[:3, 2], T[:3, 1])
        if "fov_axis" in p:
            self.warn("fov_axis ignored (as the reference does)")
        self.out.camera = dict(eye=np.asarray(look[0]), target=np.asarray(look[1]), up=np.asarray(look[2]), fov=p.get("fov", 39.3077))

    def emitter(self, el):
        ty = el.get("type")
        p, _, _ = self.props(el)
        if ty == "area":
            raise ValueError("'area' emitter needs to be nested in a shape.")
        if ty == "constant":
            self.out.env = dict(rgb=np.array([[self.rgb(p, "radiance", (1.0, 1.0, 1.0))]], np.float32), intensity=1.0)
        elif ty == "envmap":
            fn = os.path.join(self.base, p["filename"])
            if fn.lower().endswith(".pfm"):
                from .pbrt import read_pfm
                self.out.env = dict(rgb=read_pfm(fn), intensity=p.get("scale", 1.0))
                if "to_world" in p:
                    self.warn("envmap rotation ignored")
            else:
                self.warn("envmap image %r not read (only .pfm)" % fn)
        elif ty in ("point", "directional"):
            key = "intensity" if ty == "point" else "irradiance"
            if "emission_profile" in p:
                sid = self.profile(("emission", p["emission_profile"], p.get("scale", 1.0)))
            else:
                wl, vals = rgb_to_spectrum_samples(self.rgb(p, key, (1.0, 1.0, 1.0)))
                sid = self.profile(("samples", wl, vals, 1.0, True))
            if ty == "point":
                if "A" not in p:
                    raise ValueError("Emitter must specify sourcing area 'A'.")
                pos = p["position"] if "position" in p else p.get("to_world", (np.eye(4), None))[0][:3, 3]
                self.out.lights.append(("point", dict(pos=np.asarray(pos, np.float64), spectrum=sid, area=p["A"])))
            else:
                self.out.lights.append(("directional", dict(dir=np.asarray(p.get("direction", (0.0, 0.0, 1.0)), np.float64), spectrum=sid)))
        else:
            self.warn("emitter %r not supported" % ty)

    def run(self):
        for c in self.root:
            if c.tag == "shape":
                self.shape(c)
            elif c.tag == "sensor":
                self.sensor(c)
            elif c.tag == "emitter":
                self.emitter(c)
            elif c.tag in ("default", "bsdf", "integrator", "texture", "medium"):
                pass
            else:
                self.warn("element %r ignored" % c.tag)


def read_obj(path):
    """Positions, triangles (polygons fanned) and per-vertex normals (when every face has them)."""
    V, VN, faces = [], [], []
    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "v":
                V.append([float(x) for x in t[1:4]])
            elif t[0] == "vn":
                VN.append([float(x) for x in t[1:4]])
            elif t[0] == "f":
                idx = []
                for w in t[1:]:
                    parts = w.split("/")
                    vi = int(parts[0])
                    ni = int(parts[2]) if len(parts) > 2 and parts[2] else None
                    idx.append((vi - 1 if vi > 0 else len(V) + vi, None if ni is None else (ni - 1 if ni > 0 else len(VN) + ni)))
                for j in range(1, len(idx) - 1):
                    faces.append((idx[0], idx[j], idx[j + 1]))
    P = np.asarray(V, np.float64)
    I = np.array([[a[0], b[0], c[0]] for a, b, c in faces], np.int64).reshape(-1, 3)
    N = None
    if VN and all(x[1] is not None for f in faces for x in f):
        N = np.zeros_like(P)
        for f in faces:
            for vi, ni in f:
                N[vi] = VN[ni]
    return P, I, N


def load(path):
    """Parses a Mitsuba XML scene into a MitsubaScene."""
    out = MitsubaScene()
    _Builder(path, out).run()
    return out


def build(ms, tables_dir=None, lib=None):
    """The render inputs of a MitsubaScene: (scene.Scene, profiles, camera, width, height, analytic
    lights, environment or None).  Named IOR and emission tables are read from `tables_dir` (the
    reference's Source/Tables layout); Au, Ag, Cu and Al come from the standard profiles."""
    from . import capi, spectra
    from . import scene as S
    prof, _ = spectra.standard_profiles(lib)
    extra = []
    pending = {}
    for req in ms.profiles:
        if req[0] == "samples":
            extra.append(spectra.profile_from_samples(req[1], req[2], req[3], req[4], lib))
        elif req[0] in ("ior", "ior_k"):
            if tables_dir is None:
                raise ValueError("material %r needs tables_dir" % req[1])
            if req[1] not in pending:
                pending[req[1]] = spectra.profiles_from_material(tables_dir, req[1], lib)
            extra.append(pending[req[1]][0 if req[0] == "ior" else 1])
        else:
            if tables_dir is None:
                raise ValueError("emission profile %r needs tables_dir" % req[1])
            extra.append(spectra.profile_for_emitter_type(tables_dir, req[1], req[2], lib))
    allp = (capi.SpectralProfile * (len(prof) + len(extra)))()
    for i in range(len(prof)):
        allp[i] = prof[i]
    for i, e in enumerate(extra):
        allp[len(prof) + i] = e
    if not ms.records:
        raise ValueError("no shapes in the scene")
    records = np.concatenate(ms.records)
    lights = []
    for kind, L in ms.lights:
        if kind == "point":
            li = S.point_light(L["pos"], L["spectrum"])
            li.surface_area = float(L["area"])
        else:
            li = S.directional_light(L["dir"], L["spectrum"])
        lights.append(li)
    V, F, Mt, Nv = (np.concatenate(x) for x in (ms.vertices, ms.indices, ms.tri_material, ms.normals))
    emissive = np.nonzero(np.isin(Mt, ms.emissive_materials))[0]
    inst = np.concatenate([np.full(len(f), i, np.uint32) for i, f in enumerate(ms.indices)])
    sc = S.Scene(V, F, Mt, records, emissive, ms.emissive_materials[0] if ms.emissive_materials else 0, 0,
                 (float(V.min()), float(V.max())), normals=Nv, tri_instance=inst)
    w, h = ms.width, ms.height
    cam = ms.camera or dict(eye=np.zeros(3), target=np.array([0.0, 0.0, 1.0]), up=np.array([0.0, 1.0, 0.0]), fov=39.3077)
    # the reference turns fov into a focal length over the film width: fov spans x
    fovy = 2.0 * np.arctan(np.tan(0.5 * np.radians(cam["fov"])) * h / w)
    camera = S.look_at_camera(cam["eye"], cam["target"], cam["up"], float(np.degrees(fovy)), w / h)
    return sc, allp, camera, w, h, lights, ms.env
