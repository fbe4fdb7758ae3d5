"""A small Mitsuba 3 scene written by the import tests: the mapped BSDF types (with a named and a
float IOR, a named metal, eta/k spectra, a nested coated conductor, a grating, twosided), obj / ply /
rectangle / cube / sphere / disk shapes, an area emitter with an RGB radiance, a constant emitter and
a point light."""

SCENE = """<scene version="3.0.0">
  <default name="res" value="32"/>
  <sensor type="perspective">
    <float name="fov" value="60"/>
    <transform name="to_world"><lookat origin="0, -8, 3" target="0, 0, 1" up="0, 0, 1"/></transform>
    <film type="hdrfilm"><integer name="width" value="48"/><integer name="height" value="$res"/></film>
  </sensor>
  <emitter type="constant"><rgb name="radiance" value="0.4, 0.5, 0.7"/></emitter>
  <emitter type="point"><point name="position" value="0, 0, 5"/><rgb name="intensity" value="20"/><float name="A" value="1"/></emitter>
  <bsdf type="twosided" id="floor"><bsdf type="diffuse"><rgb name="reflectance" value="0.6, 0.6, 0.6"/></bsdf></bsdf>
  <bsdf type="roughdielectric" id="glass"><string name="int_ior" value="bk7"/><float name="roughness" value="0.05"/></bsdf>
  <bsdf type="dielectric" id="water"><float name="int_ior" value="1.33"/></bsdf>
  <bsdf type="conductor" id="gold"><string name="material" value="Au"/><float name="roughness" value="0.1"/></bsdf>
  <bsdf type="roughconductor" id="custom"><spectrum name="eta" value="400:0.2, 700:0.3"/><spectrum name="k" value="400:3.0, 700:4.0"/></bsdf>
  <bsdf type="coated_conductor" id="coated"><float name="thickness" value="20"/>
    <bsdf type="conductor"><string name="material" value="Cu"/></bsdf></bsdf>
  <bsdf type="grating" id="grating"><string name="material" value="Al"/><float name="pitch" value="2"/><integer name="lobes" value="4"/></bsdf>
  <bsdf type="thindielectric" id="film"><float name="int_ior" value="1.4"/></bsdf>
  <bsdf type="plastic" id="plastic"/>
  <shape type="rectangle"><transform name="to_world"><scale value="10"/></transform><ref id="floor"/></shape>
  <shape type="sphere"><point name="center" value="1, 0, 1"/><float name="radius" value="0.8"/><ref id="glass"/></shape>
  <shape type="cube"><transform name="to_world"><scale value="0.5"/><translate x="-2" y="1" z="0.5"/></transform><ref id="gold"/></shape>
  <shape type="obj"><string name="filename" value="tri.obj"/><ref id="custom"/></shape>
  <shape type="ply"><string name="filename" value="q.ply"/><ref id="coated"/></shape>
  <shape type="disk"><transform name="to_world"><translate value="0 3 2"/></transform><ref id="grating"/></shape>
  <shape type="rectangle"><transform name="to_world"><rotate x="1" angle="180"/><translate z="6"/></transform>
    <bsdf type="diffuse"/><emitter type="area"><rgb name="radiance" value="5, 4, 3"/></emitter></shape>
  <shape type="rectangle"><transform name="to_world"><translate value="3 3 0.01"/></transform><ref id="film"/></shape>
  <shape type="rectangle"><transform name="to_world"><translate value="-3 3 0.01"/></transform><ref id="plastic"/></shape>
  <shape type="rectangle"><transform name="to_world"><translate value="-3 -3 0.01"/></transform><ref id="water"/></shape>
</scene>
"""


def write(d):
    (d / "s.xml").write_text(SCENE)
    (d / "tri.obj").write_text("v 3 3 0\nv 4 3 0\nv 3 4 1\nvn 0 0 1\nf 1//1 2//1 3//1\n")
    with open(d / "q.ply", "w") as f:
        f.write("ply\nformat ascii 1.0\nelement vertex 4\nproperty float x\nproperty float y\nproperty float z\n"
                "element face 1\nproperty list uchar int vertex_indices\nend_header\n0 0 0\n1 0 0\n1 0 1\n0 0 1\n4 0 1 2 3\n")
    return d / "s.xml"
