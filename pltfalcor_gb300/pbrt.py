"""PBRT-v4 scene import for the render pass.

Follows the reference's importer (plugins/importers/PBRTImporter/PBRTImporter.cpp inside
ssteinberg/PLTFalcor) with its PLT material mapping (usePBRTMaterials, PBRTImporter.cpp:969-1200):

- diffuse -> PLTDiffuse (baseColor = reflectance, default 0.5; double-sided);
- coateddiffuse -> PLTCoatedOpaqueDielectric (roughness, baseColor = reflectance; coat IOR 1.5,
  coat thickness 3 um as the material's defaults; double-sided);
- dielectric -> PLTDielectric (roughness, IoR = eta; Cauchy B 0.0026 from the constructor's Abbe
  number 100 at the default IoR 1.5, which setIndexOfRefraction does not update);
- thindielectric -> PLTThinDielectric (IoR = eta);
- diffusetransmission -> PLTDielectric (roughness 0.6, baseColor = reflectance, transmission =
  transmittance, default 0.25);
- conductor / coatedconductor -> PLTConductor / PLTCoatedConductor.  The reference sets their base
  colour to eta's RGB and no spectral IOR (left as a TODO there); here a named metal spectrum
  ("metal-Au-eta", "metal-Ag-eta", "metal-Cu-eta", "metal-Al-eta") selects that metal's (n, k)
  profiles and anything else falls back to aluminium.
- other material types -> PLTDiffuse 0.5, with a warning.

Roughness follows getRoughness (PBRTImporter.cpp:413-447) including its sum of u and v roughness
before the square-root remap.  As in the reference, area lights are not attached to PLT materials
(a warning); `area_lights=True` instead makes those shapes emissive PLTDiffuse with a D65 profile
scaled by the luminance of L.  Point, spot and distant lights become analytic lights (D65 scaled by
the luminance of I or L); "infinite" lights become the environment map (constant L, or a .pfm
lat-long image).

Shapes: trianglemesh, plymesh (ascii and binary little-endian, triangles and quads), bilinearmesh,
sphere (tessellated).  Transforms, AttributeBegin/End, Include/Import and named materials are
supported; textures are not (constants are used, as for the reference's non-constant fallbacks).
"""
import os
import struct

import numpy as np

from . import materials as M

METAL_NAMES = ("Au", "Ag", "Cu", "Al")


class PbrtScene:
    """Import result: geometry (arrays for scene.Scene), materials, camera, lights, environment."""

    def __init__(self):
        self.vertices, self.normals, self.indices, self.tri_material = [], [], [], []
        self.records = []
        self.camera = None          # dict(eye, target, up, fov) in world space
        self.width, self.height = 640, 480
        self.lights = []            # (kind, dict) of point / spot / distant lights
        self.env = None             # dict(rgb, intensity) for scene.Scene renders
        self.emitters = []          # (material index, luminance) of emissive area-light materials
        self.warnings = []


def _tokens(text):
    i, n = 0, len(text)
    while i < n:
        c = text[i]
        if c.isspace():
            i += 1
        elif c == "#":
            while i < n and text[i] != "\n":
                i += 1
        elif c == '"':
            j = text.index('"', i + 1)
            yield ("s", text[i + 1:j])
            i = j + 1
        elif c in "[]":
            yield (c, c)
            i += 1
        else:
            j = i
            while j < n and not text[j].isspace() and text[j] not in '[]"#':
                j += 1
            yield ("w", text[i:j])
            i = j


def _num(w):
    try:
        return float(w)
    except ValueError:
        return None


class _Parser:
    def __init__(self, out, area_lights):
        self.out, self.area_lights = out, area_lights
        self.ctm = np.eye(4)
        self.stack = []
        self.material = ("diffuse", {})
        self.named = {}
        self.area = None
        self.mat_cache = {}

    # ---- parameters: "type name" value | [values] ----
    def params(self, toks, k):
        p = {}
        while k < len(toks) and toks[k][0] == "s" and " " in toks[k][1].strip():
            ty, name = toks[k][1].split()
            k += 1
            vals = []
            if toks[k][0] == "[":
                k += 1
                while toks[k][0] != "]":
                    vals.append(toks[k][1] if toks[k][0] == "s" else _num(toks[k][1]))
                    k += 1
                k += 1
            else:
                vals.append(toks[k][1] if toks[k][0] == "s" else _num(toks[k][1]))
                k += 1
            if ty == "bool":
                vals = [v if isinstance(v, bool) else str(v).lower() == "true" for v in vals]
            p[name] = (ty, vals)
        return p, k

    def warn(self, msg):
        self.out.warnings.append(msg)

    # ---- transforms ----
    def apply(self, m):
        self.ctm = self.ctm @ m

    def parse_file(self, path):
        with open(path, "r") as f:
            toks = list(_tokens(f.read()))
        self.run(toks, os.path.dirname(os.path.abspath(path)))

    def run(self, toks, base):
        k = 0
        while k < len(toks):
            kind, d = toks[k]
            k += 1
            if kind != "w":
                raise ValueError("unexpected token %r" % (d,))
            nums = []
            while k < len(toks) and toks[k][0] == "w" and _num(toks[k][1]) is not None:
                nums.append(_num(toks[k][1]))
                k += 1
            if d in ("Transform", "ConcatTransform") and k < len(toks) and toks[k][0] == "[":
                k += 1
                while toks[k][0] != "]":
                    nums.append(_num(toks[k][1]))
                    k += 1
                k += 1
            args = []
            while k < len(toks) and toks[k][0] == "s" and " " not in toks[k][1].strip():
                args.append(toks[k][1])
                k += 1
            p, k = self.params(toks, k)
            self.directive(d, nums, args, p, base)

    def directive(self, d, nums, args, p, base):
        if d in ("Include", "Import"):
            self.parse_file(os.path.join(base, args[0]))
        elif d == "LookAt":
            e, l, u = np.array(nums[0:3]), np.array(nums[3:6]), np.array(nums[6:9])
            self.out.camera = dict(eye=e, target=l, up=u, fov=90.0)
            self.lookat = (e, l, u)
        elif d == "Camera":
            cam = self.out.camera or dict(eye=np.zeros(3), target=np.array([0.0, 0.0, 1.0]), up=np.array([0.0, 1.0, 0.0]))
            cam["fov"] = float(p.get("fov", ("float", [90.0]))[1][0])
            self.out.camera = cam
        elif d == "Film":
            self.out.width = int(p.get("xresolution", ("integer", [1280]))[1][0])
            self.out.height = int(p.get("yresolution", ("integer", [720]))[1][0])
        elif d == "WorldBegin":
            self.ctm = np.eye(4)
        elif d in ("AttributeBegin", "TransformBegin"):
            self.stack.append((self.ctm.copy(), self.material, self.area))
        elif d in ("AttributeEnd", "TransformEnd"):
            if self.stack:
                self.ctm, self.material, self.area = self.stack.pop()
        elif d == "Identity":
            self.ctm = np.eye(4)
        elif d == "Translate":
            m = np.eye(4)
            m[:3, 3] = nums[:3]
            self.apply(m)
        elif d == "Scale":
            self.apply(np.diag([nums[0], nums[1], nums[2], 1.0]))
        elif d == "Rotate":
            a = np.radians(nums[0])
            ax = np.array(nums[1:4]) / np.linalg.norm(nums[1:4])
            K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
            m = np.eye(4)
            m[:3, :3] = np.eye(3) + np.sin(a) * K + (1 - np.cos(a)) * (K @ K)
            self.apply(m)
        elif d == "Transform":
            self.ctm = np.array(nums, np.float64).reshape(4, 4).T
        elif d == "ConcatTransform":
            self.apply(np.array(nums, np.float64).reshape(4, 4).T)
        elif d == "Material":
            self.material = (args[0], p)
        elif d == "MakeNamedMaterial":
            self.named[args[0]] = (p.get("type", ("string", ["diffuse"]))[1][0], p)
        elif d == "NamedMaterial":
            self.material = self.named.get(args[0], ("diffuse", {}))
            if args[0] not in self.named:
                self.warn("unknown named material %r" % args[0])
        elif d == "AreaLightSource":
            self.area = p
        elif d == "LightSource":
            self.light(args[0], p, base)
        elif d == "Shape":
            self.shape(args[0], p, base)
        elif d in ("Sampler", "Integrator", "PixelFilter", "ColorSpace", "Option", "Accelerator", "ReverseOrientation",
                   "Attribute", "CoordinateSystem", "CoordSysTransform", "MakeNamedMedium", "MediumInterface"):
            pass
        else:
            self.warn("unsupported directive %s" % d)

    # ---- parameters helpers ----
    @staticmethod
    def f(p, name, default):
        return float(p[name][1][0]) if name in p else default

    @staticmethod
    def rgb(p, name, default):
        if name in p and p[name][0] == "rgb":
            return tuple(float(x) for x in p[name][1][:3])
        if name in p and p[name][0] == "float":
            return (float(p[name][1][0]),) * 3
        return default

    def roughness(self, p, r="roughness", u="uroughness", v="vroughness"):
        """getRoughness: (u + v), square-rooted when remaproughness (default true)."""
        ur = self.f(p, u, self.f(p, r, 0.0))
        vr = self.f(p, v, self.f(p, r, 0.0))
        s = ur + vr
        remap = p.get("remaproughness", ("bool", [True]))[1][0]
        return float(np.sqrt(s)) if remap else s

    def eta(self, p, name="eta"):
        if name in p and p[name][0] == "rgb":
            return sum(p[name][1][:3]) / 3.0
        return self.f(p, name, 1.5)

    def metal(self, p, name):
        if name in p and p[name][0] == "spectrum" and isinstance(p[name][1][0], str):
            for i, m in enumerate(METAL_NAMES):
                if "-%s-" % m in p[name][1][0]:
                    return i
        return METAL_NAMES.index("Al")

    # ---- materials ----
    def material_index(self, emissive_lum=None):
        ty, p = self.material
        key = (ty, repr(sorted((k, v[0], tuple(v[1])) for k, v in p.items())), emissive_lum)
        if key in self.mat_cache:
            return self.mat_cache[key]
        ds = 1  # PLT_MATERIAL_FLAG_DOUBLE_SIDED
        if emissive_lum is not None:
            r = M.diffuse(1, albedo=self.rgb(p, "reflectance", (0.5, 0.5, 0.5)))   # emission profile set by build()
            r["flags"] |= ds
            self.out.emitters.append((len(self.out.records), emissive_lum))
        elif ty == "diffuse":
            r = M.diffuse(1, albedo=self.rgb(p, "reflectance", (0.5, 0.5, 0.5)))
            r["flags"] |= ds
        elif ty == "coateddiffuse":
            r = M.coated(1, False, self.roughness(p), 3.0, 1.5, albedo=self.rgb(p, "reflectance", (0.5, 0.5, 0.5)))
            r["flags"] |= ds
        elif ty == "dielectric":
            r = M.dielectric(1, self.roughness(p), ior=self.eta(p), dispersion_b=0.52 * 0.5 / 100.0)
        elif ty == "thindielectric":
            r = M.thin_dielectric(1, self.eta(p))
        elif ty == "diffusetransmission":
            r = M.dielectric(1, 0.6, ior=1.5, dispersion_b=0.52 * 0.5 / 100.0, specular=self.rgb(p, "reflectance", (0.25,) * 3),
                             transmission=self.rgb(p, "transmittance", (0.25,) * 3))
        elif ty == "conductor":
            mi = self.metal(p, "eta")
            r = M.conductor(1, self.roughness(p), 2 * mi, 2 * mi + 1)
            r["flags"] |= ds
        elif ty == "coatedconductor":
            mi = self.metal(p, "conductor.eta")
            r = M.coated(1, True, self.roughness(p, "conductor.roughness", "conductor.uroughness", "conductor.vroughness"), 3.0,
                         self.eta(p, "interface.eta"), ior_n_id=2 * mi, ior_k_id=2 * mi + 1)
            r["flags"] |= ds
        else:
            self.warn("material %r mapped to PLTDiffuse 0.5" % ty)
            r = M.diffuse(1, albedo=(0.5, 0.5, 0.5))
            r["flags"] |= ds
        self.out.records.append(r)
        self.mat_cache[key] = len(self.out.records) - 1
        return self.mat_cache[key]

    # ---- lights ----
    @staticmethod
    def lum(rgb):
        return 0.2126 * rgb[0] + 0.7152 * rgb[1] + 0.0722 * rgb[2]

    def light(self, ty, p, base):
        sc = self.f(p, "scale", 1.0)
        X = lambda v: (self.ctm @ np.append(np.asarray(v, np.float64), 1.0))[:3]
        if ty == "point":
            self.out.lights.append(("point", dict(pos=X(p.get("from", ("point3", [0, 0, 0]))[1]), lum=sc * self.lum(self.rgb(p, "I", (1, 1, 1))))))
        elif ty == "spot":
            fr, to = X(p.get("from", ("point3", [0, 0, 0]))[1]), X(p.get("to", ("point3", [0, 0, 1]))[1])
            self.out.lights.append(("spot", dict(pos=fr, dir=to - fr, cone=np.radians(self.f(p, "coneangle", 30.0)),
                                                  delta=np.radians(self.f(p, "conedelta", 5.0)), lum=sc * self.lum(self.rgb(p, "I", (1, 1, 1))))))
        elif ty == "distant":
            fr, to = X(p.get("from", ("point3", [0, 0, 0]))[1]), X(p.get("to", ("point3", [0, 0, 1]))[1])
            self.out.lights.append(("distant", dict(dir=to - fr, lum=sc * self.lum(self.rgb(p, "L", (1, 1, 1))))))
        elif ty == "infinite":
            if "filename" in p:
                fn = os.path.join(base, p["filename"][1][0])
                if fn.lower().endswith(".pfm"):
                    self.out.env = dict(rgb=read_pfm(fn), intensity=sc)
                else:
                    self.warn("infinite light image %r not read (only .pfm)" % fn)
            else:
                self.out.env = dict(rgb=np.full((8, 16, 3), self.rgb(p, "L", (1, 1, 1)), np.float32), intensity=sc)
        else:
            self.warn("light %r not supported" % ty)

    # ---- shapes ----
    def shape(self, ty, p, base):
        if ty == "trianglemesh":
            P = np.asarray(p["P"][1], np.float64).reshape(-1, 3)
            I = np.asarray(p["indices"][1], np.int64).reshape(-1, 3) if "indices" in p else np.arange(len(P)).reshape(-1, 3)
            N = np.asarray(p["N"][1], np.float64).reshape(-1, 3) if "N" in p else None
        elif ty == "bilinearmesh":
            P = np.asarray(p["P"][1], np.float64).reshape(-1, 3)
            q = np.asarray(p["indices"][1], np.int64).reshape(-1, 4) if "indices" in p else np.arange(4).reshape(1, 4)
            I = np.concatenate([q[:, [0, 1, 3]], q[:, [0, 3, 2]]])
            N = None
        elif ty == "plymesh":
            P, I, N = read_ply(os.path.join(base, p["filename"][1][0]))
        elif ty == "sphere":
            from .scene import icosphere
            v, f = icosphere(3)
            P, I, N = v * self.f(p, "radius", 1.0), f.astype(np.int64), v
        else:
            self.warn("shape %r not supported" % ty)
            return
        em = None
        if self.area is not None:
            if self.area_lights:
                em = self.f(self.area, "scale", 1.0) * self.lum(self.rgb(self.area, "L", (1, 1, 1)))
            else:
                self.warn("area light on a PLT material ignored (as the reference's importer does)")
        mi = self.material_index(em)
        W = (self.ctm @ np.concatenate([P, np.ones((len(P), 1))], 1).T).T[:, :3]
        if N is None:
            N = np.zeros_like(P)
            tri = W[I]
            fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
            for c in range(3):
                np.add.at(N, I[:, c], fn)
            Nw = N
        else:
            Nw = (np.linalg.inv(self.ctm[:3, :3]).T @ N.T).T
        Nw = Nw / np.maximum(np.linalg.norm(Nw, axis=1, keepdims=True), 1e-30)
        base_v = sum(len(v) for v in self.out.vertices)
        self.out.vertices.append(W)
        self.out.normals.append(Nw)
        self.out.indices.append(I + base_v)
        self.out.tri_material.append(np.full(len(I), mi, np.uint32))


def read_pfm(path):
    """A PFM image (RGB 'PF' or grey 'Pf') as [height][width][3] float32, top row first."""
    with open(path, "rb") as f:
        kind = f.readline().strip()
        w, h = (int(x) for x in f.readline().split())
        scale = float(f.readline().strip())
        ch = 3 if kind == b"PF" else 1
        data = np.frombuffer(f.read(w * h * ch * 4), "<f4" if scale < 0 else ">f4").astype(np.float32)
    img = data.reshape(h, w, ch)[::-1]
    return np.ascontiguousarray(np.repeat(img, 3, axis=2) if ch == 1 else img)


def read_ply(path):
    """Vertices (x, y, z), faces (triangles; quads split) and optional normals of a PLY file."""
    with open(path, "rb") as f:
        assert f.readline().strip() == b"ply"
        fmt, elems, cur = None, [], None
        while True:
            line = f.readline().strip().decode()
            if line.startswith("format"):
                fmt = line.split()[1]
            elif line.startswith("element"):
                _, name, cnt = line.split()
                cur = [name, int(cnt), []]
                elems.append(cur)
            elif line.startswith("property"):
                cur[2].append(line.split()[1:])
            elif line == "end_header":
                break
        tmap = {"float": "f4", "float32": "f4", "double": "f8", "uchar": "u1", "uint8": "u1", "char": "i1", "int": "i4",
                "int32": "i4", "uint": "u4", "uint32": "u4", "short": "i2", "ushort": "u2"}
        verts, faces = None, []
        if fmt == "ascii":
            rest = f.read().decode().split()
            pos = 0
            for name, cnt, props in elems:
                if name == "vertex":
                    nprop = len(props)
                    verts = (np.asarray(rest[pos:pos + cnt * nprop], np.float64).reshape(cnt, nprop), [p[-1] for p in props])
                    pos += cnt * nprop
                else:
                    for _ in range(cnt):
                        k = int(rest[pos])
                        faces.append([int(x) for x in rest[pos + 1:pos + 1 + k]])
                        pos += 1 + k
        else:
            if fmt != "binary_little_endian":
                raise ValueError("PLY format %s not supported" % fmt)
            for name, cnt, props in elems:
                if name == "vertex":
                    dt = np.dtype([(p[-1], "<" + tmap[p[0]]) for p in props])
                    arr = np.frombuffer(f.read(dt.itemsize * cnt), dt)
                    verts = (np.stack([arr[p[-1]].astype(np.float64) for p in props], 1), [p[-1] for p in props])
                else:
                    lp = props[0]
                    ct, it = "<" + tmap[lp[1]], "<" + tmap[lp[2]]
                    for _ in range(cnt):
                        k = int(np.frombuffer(f.read(np.dtype(ct).itemsize), ct)[0])
                        faces.append(list(np.frombuffer(f.read(np.dtype(it).itemsize * k), it).astype(np.int64)))
    data, names = verts
    col = {n: i for i, n in enumerate(names)}
    P = data[:, [col["x"], col["y"], col["z"]]]
    N = data[:, [col["nx"], col["ny"], col["nz"]]] if "nx" in col else None
    tris = []
    for fc in faces:
        for j in range(1, len(fc) - 1):
            tris.append((fc[0], fc[j], fc[j + 1]))
    return P, np.asarray(tris, np.int64).reshape(-1, 3), N


def load(path, area_lights=False):
    """Parses a .pbrt file into a PbrtScene."""
    out = PbrtScene()
    _Parser(out, area_lights).parse_file(path)
    return out


def build(ps, lib=None):
    """The render inputs of a PbrtScene: (scene.Scene, profiles, camera, width, height, analytic
    lights, environment or None).  Profiles are the standard ones (Au, Ag, Cu, Al eta/k, D65) plus
    one D65 profile per light and emissive material, scaled by the luminance of its pbrt radiance
    (D65 is ~100 at 560 nm, hence the 1/100)."""
    import ctypes as C
    from . import capi, spectra
    from . import scene as S
    prof, _ = spectra.standard_profiles(lib)
    t = spectra.load_tables()
    extra = []

    def d65(lum):
        extra.append(spectra.profile_from_samples(t["D65"]["wavelength_nm"], t["D65"]["value"], float(lum) / 100.0, True, lib))
        return len(prof) + len(extra) - 1

    if not ps.records:
        raise ValueError("no shapes in the scene")
    records = np.concatenate(ps.records)
    for mi, lum in ps.emitters:
        records["emission_spectral_id"][mi] = d65(lum)
    lights = []
    for kind, L in ps.lights:
        sid = d65(L["lum"])
        if kind == "point":
            lights.append(S.point_light(L["pos"], sid))
        elif kind == "spot":
            lights.append(S.point_light(L["pos"], sid, L["dir"], L["cone"], L["delta"]))
        else:
            lights.append(S.distant_light(L["dir"], sid))
    allp = (capi.SpectralProfile * (len(prof) + len(extra)))()
    for i in range(len(prof)):
        allp[i] = prof[i]
    for i, e in enumerate(extra):
        allp[len(prof) + i] = e
    V = np.concatenate(ps.vertices)
    F = np.concatenate(ps.indices)
    Mt = np.concatenate(ps.tri_material)
    Nv = np.concatenate(ps.normals)
    emissive_mats = [mi for mi, _ in ps.emitters]
    emissive = np.nonzero(np.isin(Mt, emissive_mats))[0]
    inst = np.concatenate([np.full(len(f), i, np.uint32) for i, f in enumerate(ps.indices)])
    lo, hi = V.min(0), V.max(0)
    sc = S.Scene(V, F, Mt, records, emissive, emissive_mats[0] if emissive_mats else 0, 0, (float(lo.min()), float(hi.max())),
                 normals=Nv, tri_instance=inst)
    w, h = ps.width, ps.height
    cam = ps.camera or dict(eye=np.zeros(3), target=np.array([0.0, 0.0, 1.0]), up=np.array([0.0, 1.0, 0.0]), fov=90.0)
    fov = np.radians(cam["fov"])
    fovy = fov if w >= h else 2.0 * np.arctan(np.tan(0.5 * fov) * h / w)   # pbrt's fov spans the shorter axis
    camera = S.look_at_camera(cam["eye"], cam["target"], cam["up"], float(np.degrees(fovy)), w / h)
    return sc, allp, camera, w, h, lights, ps.env
