"""Host-side PLT material packing: the float16 BasicMaterialData contract of the reference.

Mirrors the parameter setters of the reference's PLT*Material host classes (paths inside
ssteinberg/PLTFalcor, Source/Falcor/Rendering/Materials/PLT/PLT*Material.cpp): every parameter is
rounded to binary16 (round to nearest even) and stored in the BasicMaterialData field the setter
writes; integer fields (grating type and lobe count, layer count) are stored as raw 16-bit
patterns the way `asfloat16(uint16_t)` stores them.  Records are numpy structured arrays whose
layout is plt_material_record (80 bytes), so a table of any size is one contiguous buffer.
"""
import numpy as np

# plt_material_type (Source/Falcor/Scene/Material/MaterialTypes.slang:36-53)
DIFFUSE, CONDUCTOR, DIELECTRIC, OPAQUE_DIELECTRIC, THIN_DIELECTRIC = 2, 3, 4, 5, 6
COATED_CONDUCTOR, COATED_OPAQUE_DIELECTRIC, GRATED_CONDUCTOR, GRATED_OPAQUE_DIELECTRIC, MULTILAYERED_STACK = 7, 8, 9, 10, 11
TYPE_NAMES = {DIFFUSE: "PLTDiffuse", CONDUCTOR: "PLTConductor", DIELECTRIC: "PLTDielectric",
              OPAQUE_DIELECTRIC: "PLTOpaqueDielectric", THIN_DIELECTRIC: "PLTThinDielectric",
              COATED_CONDUCTOR: "PLTCoatedConductor", COATED_OPAQUE_DIELECTRIC: "PLTCoatedOpaqueDielectric",
              GRATED_CONDUCTOR: "PLTDiffractionGratedConductor",
              GRATED_OPAQUE_DIELECTRIC: "PLTDiffractionGratedOpaqueDielectric",
              MULTILAYERED_STACK: "PLTMultiLayeredStack"}
# the eight types of the mixed-material workload, in this order
BENCH_TYPES = [DIELECTRIC, CONDUCTOR, COATED_OPAQUE_DIELECTRIC, COATED_CONDUCTOR, GRATED_OPAQUE_DIELECTRIC,
               GRATED_CONDUCTOR, THIN_DIELECTRIC, MULTILAYERED_STACK]

# LobeType (Source/Falcor/Rendering/Materials/LobeType.slang:36-69)
LOBE_DIFFUSE_R, LOBE_SCATTER_R, LOBE_DELTA_R, LOBE_DISP_DELTA_R = 0x01, 0x02, 0x04, 0x08
LOBE_SCATTER_T, LOBE_DELTA_T, LOBE_DISP_DELTA_T = 0x20, 0x40, 0x80
LOBE_ALL = 0xFFFF

# DiffractionGratingType (DiffractionGrating.slangh:33-42)
GRATING_SINUSOIDAL, GRATING_RECTANGULAR, GRATING_LINEAR = 0, 1, 2

NO_PROFILE = 0xFFFFFFFF

MATERIAL_DTYPE = np.dtype([
    ("type", "<u4"), ("flags", "<u4"), ("base_color", "<u2", (4,)), ("specular", "<u2", (4,)),
    ("data1", "<u2", (4,)), ("data2", "<u2", (4,)), ("specular_transmission", "<u2"), ("transmission", "<u2", (3,)),
    ("diffuse_transmission", "<u2"), ("volume_scattering", "<u2", (3,)), ("ior", "<u2"),
    ("volume_absorption", "<u2", (3,)), ("volume_anisotropy", "<u2"), ("pad0", "<u2"),
    ("emission_spectral_id", "<u4"), ("ior_n_spectral_id", "<u4"), ("ior_k_spectral_id", "<u4")])
assert MATERIAL_DTYPE.itemsize == 80


def f16bits(x):
    """binary16 bit pattern of x (round to nearest even), as (float16_t)x does."""
    return np.asarray(x, dtype=np.float32).astype(np.float16).view(np.uint16)


def empty_records(n):
    """n records at the BasicMaterialData defaults (BasicMaterialData.slang:63-85)."""
    r = np.zeros(n, dtype=MATERIAL_DTYPE)
    r["base_color"] = f16bits(1.0)
    r["transmission"] = f16bits(1.0)
    r["ior"] = f16bits(1.5)
    r["emission_spectral_id"] = NO_PROFILE
    r["ior_n_spectral_id"] = NO_PROFILE
    r["ior_k_spectral_id"] = NO_PROFILE
    return r


def _rgb(x, n):
    a = np.asarray(x, dtype=np.float32)
    if a.ndim == 1:
        a = np.broadcast_to(a, (n, 3))
    return a


def dielectric(n, roughness, ior=1.5, ext_ior=1.0, dispersion_b=0.0, specular=(1, 1, 1), transmission=(1, 1, 1)):
    """PLTDielectricMaterial: specular[1] roughness, specular[3] ext IOR, specular[0] Cauchy B (um^2),
    IoR, baseColor specular colour, transmission colour (PLTDielectricMaterial.cpp:71-103)."""
    r = empty_records(n)
    r["type"] = DIELECTRIC
    r["base_color"][:, :3] = f16bits(_rgb(specular, n))
    r["transmission"] = f16bits(_rgb(transmission, n))
    r["specular"][:, 0] = f16bits(np.broadcast_to(dispersion_b, n))
    r["specular"][:, 1] = f16bits(np.broadcast_to(roughness, n))
    r["specular"][:, 3] = f16bits(np.broadcast_to(ext_ior, n))
    r["ior"] = f16bits(np.broadcast_to(ior, n))
    return r


def conductor(n, roughness, ior_n_id, ior_k_id, gamma=3.0, ext_ior=1.0, specular=(1, 1, 1)):
    """PLTConductorMaterial: specular[0] gamma, specular[1] roughness, IoR ext IOR, spectral (n, k)
    profile ids (PLTConductorMaterial.cpp:53-84)."""
    r = empty_records(n)
    r["type"] = CONDUCTOR
    r["base_color"][:, :3] = f16bits(_rgb(specular, n))
    r["specular"][:, 0] = f16bits(np.broadcast_to(gamma, n))
    r["specular"][:, 1] = f16bits(np.broadcast_to(roughness, n))
    r["ior"] = f16bits(np.broadcast_to(ext_ior, n))
    r["ior_n_spectral_id"] = ior_n_id
    r["ior_k_spectral_id"] = ior_k_id
    return r


def opaque_dielectric(n, roughness, albedo=(1, 1, 1)):
    """PLTOpaqueDielectricMaterial: specular[1] roughness, baseColor albedo."""
    r = empty_records(n)
    r["type"] = OPAQUE_DIELECTRIC
    r["base_color"][:, :3] = f16bits(_rgb(albedo, n))
    r["specular"][:, 1] = f16bits(np.broadcast_to(roughness, n))
    return r


def coated(n, conductor_base, roughness, coat_thickness_um, coat_ior, ext_ior=1.0, thickness_scale=1.0,
           albedo=(1, 1, 1), ior_n_id=NO_PROFILE, ior_k_id=NO_PROFILE):
    """PLTCoatedConductorMaterial / PLTCoatedOpaqueDielectricMaterial: specular[1] roughness,
    specular[2] thickness scale, data1[0] coat thickness (um), data1[3] coat IOR, IoR ext IOR
    (PLTCoatedConductorMaterial.cpp:54-102)."""
    r = empty_records(n)
    r["type"] = COATED_CONDUCTOR if conductor_base else COATED_OPAQUE_DIELECTRIC
    r["base_color"][:, :3] = f16bits(_rgb(albedo, n))
    r["specular"][:, 1] = f16bits(np.broadcast_to(roughness, n))
    r["specular"][:, 2] = f16bits(np.broadcast_to(thickness_scale, n))
    r["data1"][:, 0] = f16bits(np.broadcast_to(coat_thickness_um, n))
    r["data1"][:, 3] = f16bits(np.broadcast_to(coat_ior, n))
    r["ior"] = f16bits(np.broadcast_to(ext_ior, n))
    if conductor_base:
        r["ior_n_spectral_id"] = ior_n_id
        r["ior_k_spectral_id"] = ior_k_id
    return r


def grated(n, conductor_base, pitch_x_um, grating_height_um, pitch_y_um=0.0, direction=0.0, height_scale=1.0,
           power_multiplier=1.0, lobes=5, grating_type=GRATING_SINUSOIDAL, roughness=0.0, ext_ior=1.0,
           albedo=(1, 1, 1), ior_n_id=NO_PROFILE, ior_k_id=NO_PROFILE):
    """PLTDiffractionGrated{Conductor,OpaqueDielectric}Material: data1[0..1] pitch (um), data1[2]
    direction (rad), data1[3] = asfloat16(type << 8 | lobes), data2[0] height (um), data2[1]
    roughness, specular[0] height scale, specular[1] power multiplier
    (PLTDiffractionGratedConductorMaterial.cpp:55-146)."""
    r = empty_records(n)
    r["type"] = GRATED_CONDUCTOR if conductor_base else GRATED_OPAQUE_DIELECTRIC
    r["base_color"][:, :3] = f16bits(_rgb(albedo, n))
    r["data1"][:, 0] = f16bits(np.broadcast_to(pitch_x_um, n))
    r["data1"][:, 1] = f16bits(np.broadcast_to(pitch_y_um, n))
    r["data1"][:, 2] = f16bits(np.broadcast_to(direction, n))
    r["data1"][:, 3] = (np.broadcast_to(np.asarray(grating_type, np.uint32) << 8, n) |
                        np.broadcast_to(np.asarray(lobes, np.uint32), n)).astype(np.uint16)
    r["data2"][:, 0] = f16bits(np.broadcast_to(grating_height_um, n))
    r["data2"][:, 1] = f16bits(np.broadcast_to(roughness, n))
    r["specular"][:, 0] = f16bits(np.broadcast_to(height_scale, n))
    r["specular"][:, 1] = f16bits(np.broadcast_to(power_multiplier, n))
    r["ior"] = f16bits(np.broadcast_to(ext_ior, n))
    if conductor_base:
        r["ior_n_spectral_id"] = ior_n_id
        r["ior_k_spectral_id"] = ior_k_id
    return r


def thin_dielectric(n, ior, thickness_mm=0.0003, birefringence=0.0, birefringence_scale=1.0, optic_axis_xy=(0.15, 0.04)):
    """PLTThinDielectricMaterial: specular[3] thickness (mm), baseColor[0] birefringence,
    baseColor[1..2] optic axis xy, specular[0] birefringence scale, IoR (PLTThinDielectricMaterial.cpp:55-94)."""
    r = empty_records(n)
    r["type"] = THIN_DIELECTRIC
    r["specular"][:, 3] = f16bits(np.broadcast_to(thickness_mm, n))
    r["specular"][:, 0] = f16bits(np.broadcast_to(birefringence_scale, n))
    r["base_color"][:, 0] = f16bits(np.broadcast_to(birefringence, n))
    oa = np.asarray(optic_axis_xy, np.float32)
    r["base_color"][:, 1] = f16bits(np.broadcast_to(oa[..., 0], n))
    r["base_color"][:, 2] = f16bits(np.broadcast_to(oa[..., 1], n))
    r["ior"] = f16bits(np.broadcast_to(ior, n))
    return r


def multilayered_stack(n, layers, ior1, ior2, thickness1_um, thickness2_um, ext_ior=1.0, albedo=(1, 1, 1)):
    """PLTMultiLayeredStackMaterial: data1[0..1] thicknesses (um), data2[0..1] IORs,
    data1[3] = asfloat16(uint16 layer count), IoR ext IOR (PLTMultiLayeredStackMaterial.cpp:56-113)."""
    r = empty_records(n)
    r["type"] = MULTILAYERED_STACK
    r["base_color"][:, :3] = f16bits(_rgb(albedo, n))
    r["data1"][:, 0] = f16bits(np.broadcast_to(thickness1_um, n))
    r["data1"][:, 1] = f16bits(np.broadcast_to(thickness2_um, n))
    r["data1"][:, 3] = np.broadcast_to(np.asarray(layers, np.uint32), n).astype(np.uint16)
    r["data2"][:, 0] = f16bits(np.broadcast_to(ior1, n))
    r["data2"][:, 1] = f16bits(np.broadcast_to(ior2, n))
    r["ior"] = f16bits(np.broadcast_to(ext_ior, n))
    return r


def diffuse(n, albedo=(1, 1, 1), emission_id=NO_PROFILE):
    """PLTDiffuseMaterial: baseColor albedo, emission spectral profile id."""
    r = empty_records(n)
    r["type"] = DIFFUSE
    r["base_color"][:, :3] = f16bits(_rgb(albedo, n))
    r["emission_spectral_id"] = emission_id
    return r


def encode_grating_lobe(lx, ly, lobe=LOBE_DISP_DELTA_R):
    """LobeType::MaterialSpecific encoding of a diffraction order (PLTDiffractionGrated*BSDF.slang:54-60)."""
    lx = np.asarray(lx, np.int64)
    ly = np.asarray(ly, np.int64)
    sx = (lx >= 0).astype(np.int64)
    sy = (ly >= 0).astype(np.int64)
    ax = np.minimum(np.abs(lx), 7)
    ay = np.minimum(np.abs(ly), 7)
    code = ((ay << 3) + ax + (sy << 7) + (sx << 6)) << 8
    return ((np.asarray(lobe, np.int64) & ~0xFF00) + code).astype(np.uint32)


def lobes_of(type_id):
    """Single-lobe flags a material exposes (getLobes of each PLT*BSDF.slang)."""
    return {
        DIELECTRIC: [LOBE_DELTA_R, LOBE_DISP_DELTA_T, LOBE_SCATTER_R, LOBE_SCATTER_T],
        CONDUCTOR: [LOBE_DELTA_R, LOBE_SCATTER_R],
        OPAQUE_DIELECTRIC: [LOBE_DELTA_R, LOBE_SCATTER_R],
        COATED_CONDUCTOR: [LOBE_DELTA_R, LOBE_SCATTER_R],
        COATED_OPAQUE_DIELECTRIC: [LOBE_DELTA_R, LOBE_SCATTER_R],
        GRATED_CONDUCTOR: [LOBE_DELTA_R, LOBE_SCATTER_R, LOBE_DISP_DELTA_R],
        GRATED_OPAQUE_DIELECTRIC: [LOBE_DELTA_R, LOBE_SCATTER_R, LOBE_DISP_DELTA_R],
        THIN_DIELECTRIC: [LOBE_DELTA_R, LOBE_DELTA_T],
        MULTILAYERED_STACK: [LOBE_DELTA_R],
        DIFFUSE: [LOBE_DIFFUSE_R],
    }[type_id]
