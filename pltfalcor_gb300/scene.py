"""Seeded procedural scenes for the traversal and path-tracing workloads.

`procedural_scene` builds the path-tracing test scene: a closed, subdivided box (the room),
`n_spheres` subdivided icospheres, `n_quads` randomly placed and oriented quads, one emissive
quad (PLTDiffuse with a spectral emission profile) under the ceiling and one smooth PLTDielectric
sphere (roughness 0, so manifold NEE applies) below it.  With the defaults (200 level-4
icospheres, 500 quads, 32x32 box faces) it holds about 1.04 M triangles.  Every other object gets a
material drawn uniformly from the eight PLT types with the mixed-material batch's parameter
ranges.  All randomness comes from the library's counter-based generator (workloads.CounterRNG),
so the scene is identical on every host.
"""
import numpy as np

from . import materials as M
from .workloads import CounterRNG, mixed_material_records


def icosphere(level):
    """Unit icosphere: 20 * 4^level triangles."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6],
                  [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
                  [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(level):
        edges = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
        uniq, inv = np.unique(edges, axis=0, return_inverse=True)
        mids = v[uniq[:, 0]] + v[uniq[:, 1]]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        m = inv.reshape(3, -1).T + len(v)
        v = np.concatenate([v, mids])
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)])
    return v, f


def grid_quad(corner, e1, e2, n):
    """n x n subdivided parallelogram corner + s e1 + t e2."""
    s = np.linspace(0.0, 1.0, n + 1)
    ss, tt = np.meshgrid(s, s, indexing="ij")
    v = corner[None, None, :] + ss[..., None] * e1[None, None, :] + tt[..., None] * e2[None, None, :]
    v = v.reshape(-1, 3)
    idx = lambda i, j: i * (n + 1) + j
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    i, j = i.ravel(), j.ravel()
    f = np.concatenate([np.stack([idx(i, j), idx(i + 1, j), idx(i + 1, j + 1)], 1), np.stack([idx(i, j), idx(i + 1, j + 1), idx(i, j + 1)], 1)])
    return v, f


class Scene:
    """Triangle soup with per-triangle material indices, material records and light data."""

    def __init__(self, vertices, indices, tri_material, records, emissive_tris, light_material, mnee_material, bounds,
                 normals=None, tri_instance=None):
        self.vertices = np.ascontiguousarray(vertices, np.float32)
        self.normals = None if normals is None else np.ascontiguousarray(normals, np.float32)
        self.tangents = None
        # geometry instance (mesh) of each triangle: manifold walks re-project onto the same instance
        self.tri_instance = None if tri_instance is None else np.ascontiguousarray(tri_instance, np.uint32)
        self.indices = np.ascontiguousarray(indices, np.uint32)
        self.tri_material = np.ascontiguousarray(tri_material, np.uint32)
        self.records = records
        self.emissive_tris = np.asarray(emissive_tris, np.uint32)
        self.light_material = light_material
        self.mnee_material = mnee_material
        self.bounds = bounds

    @property
    def n_tris(self):
        return len(self.indices)

    def triangle_vertices(self):
        """[n_tris][9] vertex coordinates."""
        return np.ascontiguousarray(self.vertices[self.indices].reshape(-1, 9))


def procedural_scene(seed=2, n_spheres=200, sphere_level=4, n_quads=500, box_subdiv=32, room=10.0, emission_id=8, walls=True,
                     emitter=True):
    """The procedural room: six subdivided walls (walls=False: the floor only, an open scene for an
    environment light), an area light under the ceiling (emitter=False: none), a smooth dielectric
    sphere below it, random icospheres and quads of the mixed PLT materials."""
    rng = CounterRNG(seed, max(n_spheres, n_quads, 1) * 16)
    u = lambda: rng.uniform().astype(np.float64)
    per_type = 512
    recs = mixed_material_records(per_type=per_type, seed=seed)
    # extra materials: the emitter, the smooth dielectric sphere, the room walls
    light = M.diffuse(1, albedo=(0.8, 0.8, 0.8), emission_id=emission_id)
    glass = M.dielectric(1, 0.0, ior=1.5, dispersion_b=0.0042)
    wall = M.opaque_dielectric(1, 0.3, albedo=(0.7, 0.7, 0.7))
    records = np.concatenate([recs, light, glass, wall])
    light_mat, glass_mat, wall_mat = len(recs), len(recs) + 1, len(recs) + 2
    verts, faces, mats, norms, insts = [], [], [], [], []
    nv = 0

    def add(v, f, m, n):
        nonlocal nv
        verts.append(v)
        faces.append(f + nv)
        mats.append(np.full(len(f), m, np.uint32))
        norms.append(np.broadcast_to(np.asarray(n, np.float64), v.shape))
        insts.append(np.full(len(f), len(insts), np.uint32))
        nv += len(v)

    # room: six subdivided faces of [-room, room]^3
    R = room
    corners = [(np.array([-R, -R, -R]), np.array([2 * R, 0, 0]), np.array([0, 2 * R, 0])),
               (np.array([-R, -R, R]), np.array([0, 2 * R, 0]), np.array([2 * R, 0, 0])),
               (np.array([-R, -R, -R]), np.array([0, 0, 2 * R]), np.array([2 * R, 0, 0])),
               (np.array([-R, R, -R]), np.array([2 * R, 0, 0]), np.array([0, 0, 2 * R])),
               (np.array([-R, -R, -R]), np.array([0, 2 * R, 0]), np.array([0, 0, 2 * R])),
               (np.array([R, -R, -R]), np.array([0, 0, 2 * R]), np.array([0, 2 * R, 0]))]
    for c, e1, e2 in (corners if walls else corners[:1]):
        v, f = grid_quad(c, e1, e2, box_subdiv)
        add(v, f, wall_mat, _unit(np.cross(e1, e2)))
    # area light under the ceiling (z = +R is the ceiling), emitting downwards
    e1, e2 = np.array([0, 3.0, 0]), np.array([3.0, 0, 0])
    v, f = grid_quad(np.array([-1.5, -1.5, R - 0.05]), e1, e2, 1)
    first_emissive = sum(len(x) for x in faces)
    if emitter:
        add(v, f, light_mat, _unit(np.cross(e1, e2)))
    emissive = np.arange(first_emissive, first_emissive + (len(f) if emitter else 0))
    # smooth dielectric sphere below the light (manifold NEE occluder)
    sv, sf = icosphere(min(sphere_level, 4))
    add(sv * 1.2 + np.array([0.0, 0.0, R - 4.0]), sf, glass_mat, sv)
    # random icospheres
    cx, cy, cz, rad, mt, mi = u(), u(), u(), u(), u(), u()
    for s in range(n_spheres):
        r = 0.25 + 0.75 * rad[s]
        c = np.array([(2 * cx[s] - 1) * (R - 1.5), (2 * cy[s] - 1) * (R - 1.5), (2 * cz[s] - 1) * (R - 6.0) - 1.0])
        t = min(int(mt[s] * 8), 7)
        add(sv * r + c, sf, t * per_type + min(int(mi[s] * per_type), per_type - 1), sv)
    # random quads
    qx, qy, qz, qa, qb, qs, qt, qm = u(), u(), u(), u(), u(), u(), u(), u()
    for q in range(n_quads):
        c = np.array([(2 * qx[q] - 1) * (R - 1.0), (2 * qy[q] - 1) * (R - 1.0), (2 * qz[q] - 1) * (R - 5.0) - 1.0])
        th, ph = np.pi * qa[q], 2 * np.pi * qb[q]
        nrm = np.array([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)])
        e1 = np.cross(nrm, [0.0, 0.0, 1.0] if abs(nrm[2]) < 0.9 else [1.0, 0.0, 0.0])
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(nrm, e1)
        size = 0.5 + 1.5 * qs[q]
        v, f = grid_quad(c - 0.5 * size * (e1 + e2), size * e1, size * e2, 1)
        t = min(int(qt[q] * 8), 7)
        add(v, f, t * per_type + min(int(qm[q] * per_type), per_type - 1), _unit(np.cross(size * e1, size * e2)))
    V = np.concatenate(verts).astype(np.float32)
    F = np.concatenate(faces).astype(np.uint32)
    Mt = np.concatenate(mats)
    Nv = np.concatenate(norms)
    Nv = (Nv / np.linalg.norm(Nv, axis=1, keepdims=True)).astype(np.float32)
    return Scene(V, F, Mt, records, emissive, light_mat, glass_mat, (-R, R), normals=Nv, tri_instance=np.concatenate(insts))


def small_scene(seed=3):
    """The procedural room at test size (about 8 K triangles): 12 level-2 icospheres, 40 quads,
    4x4 box faces, the light and the glass sphere."""
    return procedural_scene(seed=seed, n_spheres=12, sphere_level=2, n_quads=40, box_subdiv=4)


def open_scene(seed=5, emitter=True):
    """An open test scene (floor, objects, optional area light, no walls) for the environment light."""
    return procedural_scene(seed=seed, n_spheres=12, sphere_level=2, n_quads=30, box_subdiv=4, walls=False, emitter=emitter)


def sky_env(width=256, height=128, seed=1, sun=(0.35, 0.22), sun_radiance=200.0):
    """A synthetic HDR lat-long environment map [height][width][3]: a vertical sky gradient (map
    top = local +y), a warm ground, coloured smooth patches and a small bright sun disc at map
    coordinates `sun` (u, v)."""
    rng = np.random.default_rng(seed)
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    U, Vv = np.meshgrid(u, v)
    sky = np.stack([0.25 + 0.35 * Vv, 0.35 + 0.35 * Vv, 0.9 - 0.2 * Vv], -1)
    ground = np.stack([0.3 + 0 * Vv, 0.22 + 0 * Vv, 0.15 + 0 * Vv], -1)
    img = np.where((Vv > 0.5)[..., None], ground, sky)
    for _ in range(6):
        cu, cv, r = rng.uniform(0, 1), rng.uniform(0.1, 0.9), rng.uniform(0.03, 0.12)
        col = rng.uniform(0.0, 2.0, 3)
        d2 = np.minimum(np.abs(U - cu), 1 - np.abs(U - cu)) ** 2 + (Vv - cv) ** 2
        img = img + col * np.exp(-d2 / (2 * r * r))[..., None]
    d2 = np.minimum(np.abs(U - sun[0]), 1 - np.abs(U - sun[0])) ** 2 * 4 + (Vv - sun[1]) ** 2
    img = img + np.array([1.0, 0.95, 0.85]) * sun_radiance * (d2 < (1.5 / height) ** 2)[..., None]
    return img.astype(np.float32)


def floor_spheres_scene(emitter=True):
    """A diffuse floor (albedo 0.7) with closed spheres standing on it (every hit front-facing) and,
    optionally, a small emissive quad facing the floor."""
    verts, faces, mats, norms = [], [], [], []

    def add(v, f, m, n):
        faces.append(np.asarray(f) + sum(len(x) for x in verts))
        verts.append(np.asarray(v, np.float64))
        mats.append(np.full(len(f), m, np.uint32))
        norms.append(np.broadcast_to(np.asarray(n, np.float64), np.shape(v)))

    v, f = grid_quad(np.array([-60.0, -60.0, 0.0]), np.array([120.0, 0, 0]), np.array([0, 120.0, 0]), 4)
    add(v, f, 0, (0.0, 0.0, 1.0))
    sv, sf = icosphere(3)
    for c, r in (((-2.0, 1.0, 1.0), 1.0), ((1.5, 2.5, 1.5), 1.5), ((2.0, -1.5, 0.6), 0.6)):
        add(sv * r + np.array(c), sf, 0, sv)
    emissive = []
    if emitter:
        e1, e2 = np.array([0.0, 1.0, 0.0]), np.array([1.0, 0.0, 0.0])
        v, f = grid_quad(np.array([-0.5, -0.5, 6.0]), e1, e2, 1)
        emissive = list(range(sum(len(x) for x in faces), sum(len(x) for x in faces) + len(f)))
        add(v, f, 1, (0.0, 0.0, -1.0))
    recs = np.concatenate([M.diffuse(1, albedo=(0.7, 0.7, 0.7)), M.diffuse(1, albedo=(0.5, 0.5, 0.5), emission_id=8)])
    n = np.concatenate(norms)
    n = n / np.linalg.norm(n, axis=1, keepdims=True)
    return Scene(np.concatenate(verts), np.concatenate(faces), np.concatenate(mats), recs, emissive, 1, 0, (-60, 60),
                   normals=n, tri_instance=np.arange(len(faces)).repeat([len(x) for x in faces]).astype(np.uint32))


def _light(kind, spectrum, pos=(0.0, 0.0, 0.0), direction=(0.0, -1.0, 0.0), transform=None):
    from . import capi
    L = capi.AnalyticLight()
    L.type, L.intensity_spectral_id = kind, spectrum
    d = _unit(direction)
    for i in range(3):
        L.pos[i], L.dir[i] = float(pos[i]), float(d[i])
    # LightData defaults (Scene/Lights/LightData.slang:48-67)
    L.opening_angle, L.cos_opening_angle, L.penumbra_angle = float(np.pi), -1.0, 0.0
    L.cos_subtended_angle = 0.9999893
    T = np.eye(4)[:3] if transform is None else np.asarray(transform, np.float64).reshape(3, 4)
    for i in range(12):
        L.transform[i] = float(T.ravel()[i])
    return L, T


def point_light(pos, spectrum, direction=(0.0, -1.0, 0.0), opening_angle=np.pi, penumbra_angle=0.0):
    """PointLight (a spot light when opening_angle < pi): Light.cpp setOpeningAngle / setPenumbraAngle."""
    L, _ = _light(0, spectrum, pos, direction)
    L.opening_angle = float(opening_angle)
    L.cos_opening_angle = float(np.cos(np.float32(opening_angle)))
    L.penumbra_angle = float(penumbra_angle)
    return L


def directional_light(direction, spectrum):
    return _light(1, spectrum, direction=direction)[0]


def distant_light(direction, spectrum, half_angle=0.5 * np.pi / 180.0):
    """DistantLight: cosSubtendedAngle = cos(half angle), the frame rotating +z onto -dir
    (DistantLight::update, Light.cpp:295-312)."""
    d = _unit(direction)
    up = np.array([0.0, 0.0, 1.0])
    v = np.cross(up, -d)
    s = np.linalg.norm(v)
    R = np.eye(3)
    if s > 0:
        k = v / s
        c = np.dot(up, -d)
        K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
        R = np.eye(3) + s * K + (1 - c) * (K @ K)
    T = np.concatenate([R, np.zeros((3, 1))], 1)
    L, _ = _light(2, spectrum, direction=direction, transform=T)
    L.cos_subtended_angle = float(np.cos(half_angle))
    return L


def area_light(kind, transform, spectrum):
    """RectLight / DiscLight / SphereLight with a 3x4 model-to-world transform; surface area as the
    classes' update() computes it (Light.cpp:360-402)."""
    from . import capi
    L, T = _light({"rect": capi.LIGHT_RECT, "disc": capi.LIGHT_DISC, "sphere": capi.LIGHT_SPHERE}[kind], spectrum, transform=transform)
    rx, ry, rz = (float(np.linalg.norm(T[:, i])) for i in range(3))
    if kind == "rect":
        L.surface_area = 4.0 * rx * ry
    elif kind == "disc":
        L.surface_area = float(np.pi) * rx * ry
    else:
        L.surface_area = 4.0 * float(np.pi) * ((rx * ry) ** 1.6 + (ry * rz) ** 1.6 + (rx * rz) ** 1.6 / 3.0) ** (1.0 / 1.6)
    return L


def _unit(v):
    v = np.asarray(v, np.float64)
    return v / np.linalg.norm(v)


def look_at_camera(pos, target, up, fovy_deg, aspect, focal_distance=1.0):
    """plt_camera with Falcor's CameraData construction (Scene/Camera/Camera.cpp, calculateCameraParameters):
    W = normalize(target - pos) * focal distance, U/V orthonormal scaled by the image-plane half extents."""
    from . import capi
    pos = np.asarray(pos, np.float64)
    W = _unit(np.asarray(target, np.float64) - pos) * focal_distance
    U = _unit(np.cross(W, np.asarray(up, np.float64)))
    V = _unit(np.cross(U, W))
    vlen = focal_distance * np.tan(np.radians(fovy_deg) * 0.5)
    U = U * vlen * aspect
    V = V * vlen
    cam = capi.Camera()
    for name, val in (("pos", pos), ("u", U), ("v", V), ("w", W)):
        arr = getattr(cam, name)
        for i in range(3):
            arr[i] = float(val[i])
    return cam


def room_camera(width, height, room=10.0):
    """The benchmark view: from near the front wall towards the room centre, light and glass sphere in view."""
    return look_at_camera((0.0, -(room - 1.0), -1.0), (0.0, 0.0, 2.0), (0.0, 0.0, 1.0), 75.0, width / height)


def random_rays(n, seed, bounds, scene_tris=None):
    """n rays from random points inside the bounds in uniformly random directions; a fifth of them
    aimed exactly at triangle vertices or edge midpoints of `scene_tris` (watertightness)."""
    rng = CounterRNG(seed, n)
    lo, hi = bounds
    o = np.stack([lo + (hi - lo) * rng.uniform().astype(np.float64) for _ in range(3)])
    z = 2 * rng.uniform().astype(np.float64) - 1
    ph = 2 * np.pi * rng.uniform().astype(np.float64)
    s = np.sqrt(np.maximum(0, 1 - z * z))
    d = np.stack([s * np.cos(ph), s * np.sin(ph), z])
    if scene_tris is not None:
        k = rng.uniform().astype(np.float64)
        sel = k < 0.2
        pick = (rng.uniform().astype(np.float64) * len(scene_tris)).astype(np.int64) % len(scene_tris)
        which = (rng.uniform().astype(np.float64) * 6).astype(np.int64)
        tv = scene_tris[pick].reshape(-1, 3, 3).astype(np.float64)
        a, b, c = tv[:, 0], tv[:, 1], tv[:, 2]
        targets = np.select([which[:, None] == 0, which[:, None] == 1, which[:, None] == 2, which[:, None] == 3, which[:, None] == 4],
                            [a, b, c, 0.5 * (a + b), 0.5 * (b + c)], 0.5 * (c + a))
        dd = targets.T - o
        dd /= np.maximum(np.linalg.norm(dd, axis=0, keepdims=True), 1e-12)
        d = np.where(sel[None, :], dd, d)
    return np.ascontiguousarray(o.astype(np.float32).reshape(-1)), np.ascontiguousarray(d.astype(np.float32).reshape(-1))


def merged_materials(scenes):
    """One material table for a scene set: the scenes' records concatenated, and the offset of each
    scene's records (its tri_material indices shift by it)."""
    offsets, recs, n = [], [], 0
    for sc in scenes:
        offsets.append(n)
        recs.append(sc.records)
        n += len(sc.records)
    return np.concatenate(recs), offsets


def scene_set(seed=4, count=64, tris=(10_000, 500_000), rays=(4096, 1 << 20), sphere_level=3):
    """`count` independent procedural rooms of uneven size: triangle counts and primary-ray counts
    log-uniform in the given ranges (seeded), each room with its own materials over all eight PLT
    types (gratings and up to 32-layer stacks included), light and glass sphere.  Returns a list of
    (scene, width, height); width = height, a multiple of 8."""
    rng = CounterRNG(seed, count)
    ut, ur = rng.uniform().astype(np.float64), rng.uniform().astype(np.float64)
    per_sphere = 20 * 4 ** sphere_level
    box, quads = 16, 200
    base = 12 * box * box + 2 + 20 * 4 ** min(sphere_level, 4) + 2 * quads
    out = []
    for i in range(count):
        target = np.exp(np.log(tris[0]) + ut[i] * (np.log(tris[1]) - np.log(tris[0])))
        n_spheres = max(0, int(round((target - base) / per_sphere)))
        r = np.exp(np.log(rays[0]) + ur[i] * (np.log(rays[1]) - np.log(rays[0])))
        side = max(8, int(round(np.sqrt(r) / 8.0)) * 8)
        sc = procedural_scene(seed=1000 + seed * 131 + i, n_spheres=n_spheres, sphere_level=sphere_level, n_quads=quads,
                              box_subdiv=box)
        out.append((sc, side, side))
    return out
