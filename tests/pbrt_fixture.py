"""A small PBRT-v4 scene written by the import tests: every mapped material type, the supported
shapes (trianglemesh, sphere, ascii and binary PLY, bilinearmesh), point and infinite lights, an
area light and an unsupported material."""
import struct

SCENE = """LookAt 0 -8 3  0 0 1  0 0 1
Camera "perspective" "float fov" [ 45 ]
Film "rgb" "integer xresolution" [ 48 ] "integer yresolution" [ 32 ] "string filename" "x.exr"
WorldBegin
LightSource "infinite" "rgb L" [ 0.5 0.6 0.8 ]
LightSource "point" "point3 from" [ 0 0 6 ] "rgb I" [ 50 50 50 ]
MakeNamedMaterial "coat" "string type" "coateddiffuse" "rgb reflectance" [ 0.2 0.5 0.8 ] "float roughness" 0.1
AttributeBegin
  Material "diffuse" "rgb reflectance" [ 0.7 0.7 0.7 ]
  Shape "trianglemesh" "integer indices" [ 0 1 2 0 2 3 ] "point3 P" [ -10 -10 0  10 -10 0  10 10 0  -10 10 0 ]
AttributeEnd
AttributeBegin
  Translate 1 0 1
  Material "dielectric" "float eta" 1.33 "float roughness" 0.02 "bool remaproughness" false
  Shape "sphere" "float radius" 0.8
AttributeEnd
AttributeBegin
  NamedMaterial "coat"
  Translate -2 1 0
  Shape "plymesh" "string filename" "q.ply"
  Translate 0 0 2
  Shape "plymesh" "string filename" "qb.ply"
AttributeEnd
AttributeBegin
  Material "conductor" "spectrum eta" "metal-Cu-eta" "spectrum k" "metal-Cu-k" "float roughness" 0.05
  AreaLightSource "diffuse" "rgb L" [ 4 4 4 ]
  Translate 0 3 2
  Shape "bilinearmesh" "point3 P" [ -1 0 0  1 0 0  -1 0 1  1 0 1 ]
AttributeEnd
Material "measured" "string filename" "x.bsdf"
Shape "trianglemesh" "integer indices" [ 0 1 2 ] "point3 P" [ 3 3 0  4 3 0  3 4 0 ]
"""
QUAD = [(0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (1.0, 0.0, 1.0), (0.0, 0.0, 1.0)]


def write(d):
    (d / "s.pbrt").write_text(SCENE)
    with open(d / "q.ply", "w") as f:
        f.write("ply\nformat ascii 1.0\nelement vertex 4\nproperty float x\nproperty float y\nproperty float z\n"
                "element face 1\nproperty list uchar int vertex_indices\nend_header\n")
        for v in QUAD:
            f.write("%g %g %g\n" % v)
        f.write("4 0 1 2 3\n")
    with open(d / "qb.ply", "wb") as f:
        f.write(b"ply\nformat binary_little_endian 1.0\nelement vertex 4\nproperty float x\nproperty float y\nproperty float z\n"
                b"element face 1\nproperty list uchar int vertex_indices\nend_header\n")
        for v in QUAD:
            f.write(struct.pack("<3f", *v))
        f.write(struct.pack("<B4i", 4, 0, 1, 2, 3))
    return d / "s.pbrt"
