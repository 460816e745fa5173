"""PBRT and PLY loaders (gprt_pbrt_parse / gprt_pbrt_load / gprt_ply_load).

The cases restate the reference's loader tests (pkg/loaders/pbrt_test.go,
pbrt_graphics_state_test.go, pbrt_area_light_test.go,
pbrt_multiline_test.go, ply_test.go) and the conversion rules of
scene.NewPBRTScene (pkg/scene/pbrt_scene.go), checked on the scene
description the library builds.  No GPU is needed."""
import os
import struct
import tempfile

import numpy as np
import pytest


@pytest.fixture(scope="module")
def loaders(gprt_lib):
    from gprt import loaders
    return loaders


HEAD = '''Camera "perspective" "float fov" 40
Film "rgb" "string filename" "test.png" "integer xresolution" 200 "integer yresolution" 200
WorldBegin
'''


def shapes(desc):
    return [desc.shapes[k] for k in range(desc.n_shapes)]


def mat(desc, shape):
    return desc.materials[shape.material]


def albedo(desc, shape):
    return tuple(mat(desc, shape).albedo)


def test_graphics_state_global_and_local_materials(loaders):
    # TestGraphicsStateStack (pbrt_graphics_state_test.go:9-78)
    s = loaders.parse_pbrt(HEAD + '''
Material "diffuse" "rgb reflectance" [1.0 0.0 0.0]
Shape "sphere" "float radius" 0.5
Material "diffuse" "rgb reflectance" [0.0 1.0 0.0]
AttributeBegin
    Material "diffuse" "rgb reflectance" [0.0 0.0 1.0]
    Shape "sphere" "float radius" 0.3
AttributeEnd
Shape "sphere" "float radius" 0.7
WorldEnd''')
    d = s.desc
    got = [(sh.p[3], albedo(d, sh)) for sh in shapes(d)]
    # top-level shapes first, then the attribute block's (NewPBRTScene order)
    assert got == [(0.5, (1.0, 0.0, 0.0)), (0.7, (0.0, 1.0, 0.0)), (0.3, (0.0, 0.0, 1.0))]


def test_nested_attribute_blocks(loaders):
    # TestNestedAttributeBlocks (pbrt_graphics_state_test.go:80-167)
    s = loaders.parse_pbrt(HEAD + '''
Material "diffuse" "rgb reflectance" [1.0 0.0 0.0]
Shape "sphere" "float radius" 1.0
AttributeBegin
    Material "diffuse" "rgb reflectance" [0.0 1.0 0.0]
    Shape "sphere" "float radius" 0.8
    AttributeBegin
        Material "diffuse" "rgb reflectance" [0.0 0.0 1.0]
        Shape "sphere" "float radius" 0.6
    AttributeEnd
    Shape "sphere" "float radius" 0.4
AttributeEnd
Shape "sphere" "float radius" 0.2
WorldEnd''')
    d = s.desc
    got = [(round(sh.p[3], 6), albedo(d, sh)) for sh in shapes(d)]
    # global shapes, then blocks in completion order (the inner block first)
    assert got == [(1.0, (1, 0, 0)), (0.2, (1, 0, 0)), (0.6, (0, 0, 1)), (0.8, (0, 1, 0)), (0.4, (0, 1, 0))]


def test_material_state_restored_after_block(loaders):
    # TestMaterialStateRestoration (pbrt_graphics_state_test.go:169-236), without
    # the leading material-less shape (which NewPBRTScene rejects, below)
    s = loaders.parse_pbrt(HEAD + '''
Material "diffuse" "rgb reflectance" [1.0 0.0 0.0]
Shape "sphere" "float radius" 0.9
AttributeBegin
    Material "diffuse" "rgb reflectance" [0.0 1.0 0.0]
    Shape "sphere" "float radius" 0.8
AttributeEnd
Shape "sphere" "float radius" 0.7
Material "diffuse" "rgb reflectance" [0.0 0.0 1.0]
Shape "sphere" "float radius" 0.6
WorldEnd''')
    d = s.desc
    got = [(round(sh.p[3], 6), albedo(d, sh)) for sh in shapes(d)]
    assert got == [(0.9, (1, 0, 0)), (0.7, (1, 0, 0)), (0.6, (0, 0, 1)), (0.8, (0, 1, 0))]
    with pytest.raises(Exception, match="shape has no valid material"):
        loaders.parse_pbrt(HEAD + 'Shape "sphere" "float radius" 1.0\nWorldEnd')


def test_area_light_state_and_conversion(loaders):
    # TestAreaLightStateInheritance (pbrt_area_light_test.go:178-239) and
    # processAttributeBlock's area lights (pbrt_scene.go:397-468)
    from gprt import capi
    s = loaders.parse_pbrt('''
WorldBegin
AttributeBegin
  Material "diffuse" "rgb reflectance" [0.8 0.8 0.8]
  AreaLightSource "diffuse" "rgb L" [ 10 8 6 ]
  Shape "sphere" "float radius" [ 1.0 ]
  Shape "bilinearPatch" "point3 P00" [0 0 0] "point3 P01" [1 0 0] "point3 P10" [0 1 0] "point3 P11" [1 1 0]
AttributeEnd
WorldEnd''')
    d = s.desc
    sh = shapes(d)
    assert [x.kind for x in sh] == [capi.SHAPE_SPHERE, capi.SHAPE_QUAD]
    for x in sh:  # both shapes carry Emissive(L)
        m = mat(d, x)
        assert m.kind == capi.MAT_EMISSIVE and tuple(m.emission) == (10, 8, 6)
    assert list(sh[1].p[:9]) == [0, 0, 0, 1, 0, 0, 0, 1, 0]  # corner P00, u = P01 - P00, v = P10 - P00
    lights = [(d.lights[k].kind, d.lights[k].shape) for k in range(d.n_lights)]
    assert lights == [(capi.LIGHT_SPHERE, 0), (capi.LIGHT_QUAD, 1)]


def test_area_light_errors(loaders):
    # a top-level AreaLightSource is converted as a standalone light, which
    # NewPBRTScene refuses (pbrt_scene.go:391-392)
    with pytest.raises(Exception, match="AreaLightSource should be handled as graphics state"):
        loaders.parse_pbrt('WorldBegin\nAreaLightSource "diffuse" "rgb L" [1 1 1]\nWorldEnd')
    # area light on a shape that cannot be one (convertAreaLight, pbrt_scene.go:307-336)
    with pytest.raises(Exception, match="not supported as an area light"):
        loaders.parse_pbrt('''WorldBegin
AttributeBegin
  Material "diffuse"
  AreaLightSource "diffuse" "rgb L" [1 1 1]
  Shape "box" "point3 center" [0 0 0]
AttributeEnd
WorldEnd''')


def test_multiline_statements(loaders):
    # TestMultiLineParameterFormatting (pbrt_multiline_test.go:9-152)
    s = loaders.parse_pbrt('''Camera "perspective"
    "float fov" 40
Film "rgb"
    "string filename" "test.png"
    "integer xresolution" 320
    "integer yresolution" 160
WorldBegin
Material "diffuse"
    "rgb reflectance" [0.25 0.5 0.75]
Shape "trianglemesh"
    "point3 P" [ 0 0 0
                 1 0 0
                 0 1 0 ]
    "integer indices" [ 0 1 2 ]
LightSource "infinite-gradient"
    "rgb topColor" [0.1 0.2 0.3]
WorldEnd''')
    d = s.desc
    assert d.camera.vfov_deg == 40 and d.camera.width == 320 and d.camera.aspect_ratio == 2.0
    assert (d.sampling.width, d.sampling.height) == (320, 160)
    assert d.n_meshes == 1 and d.meshes[0].n_vertices == 3 and d.meshes[0].n_triangles == 1
    assert [d.meshes[0].vertices[k] for k in range(9)] == [0, 0, 0, 1, 0, 0, 0, 1, 0]
    assert albedo(d, shapes(d)[0]) == (0.25, 0.5, 0.75)
    g = d.lights[0]
    assert tuple(g.color_a) == (0.1, 0.2, 0.3) and tuple(g.color_b) == (1.0, 1.0, 1.0)  # default bottom
    with pytest.raises(Exception, match="unexpected continuation line"):
        loaders.parse_pbrt('WorldBegin\n"float radius" 1\nWorldEnd')


def test_block_and_parameter_edge_cases(loaders):
    from gprt import capi
    # processAttributeEnd with no open block does nothing; a block still open
    # at the end of the file never reaches the scene (pbrt.go:201-221)
    s = loaders.parse_pbrt('WorldBegin\nMaterial "diffuse"\nShape "sphere" "float radius" 2\nAttributeEnd\n'
                           'AttributeBegin\nShape "sphere" "float radius" 3\nWorldEnd')
    assert [sh.p[3] for sh in shapes(s.desc)] == [2.0]
    # a declaration that is not "type name" is skipped, and so is the bare
    # value after it; a later declaration of the same name wins
    s = loaders.parse_pbrt('WorldBegin\nMaterial "diffuse"\nShape "sphere" "radius" 5 "float radius" 4 '
                           '"point3 center" [1 2 3] "point3 center" [4 5 6]\nWorldEnd')
    sh = shapes(s.desc)[0]
    assert sh.p[3] == 4.0 and list(sh.p[:3]) == [4, 5, 6]
    # tabs separate tokens and list items, but a statement line must start
    # with the directive name and a space (isStatementStart, pbrt.go:707-722)
    s = loaders.parse_pbrt('WorldBegin\nMaterial "diffuse"\t"rgb reflectance"\t[0.1\t0.2 0.3]\n'
                           'Shape "sphere"\nWorldEnd')
    assert albedo(s.desc, shapes(s.desc)[0]) == (0.1, 0.2, 0.3)
    with pytest.raises(Exception, match="unexpected continuation line"):
        loaders.parse_pbrt('WorldBegin\nMaterial\t"diffuse"\nWorldEnd')
    # statements before WorldBegin other than Camera / Film / Sampler /
    # Integrator are read and dropped
    s = loaders.parse_pbrt('Material "diffuse"\nShape "sphere"\nWorldBegin\nWorldEnd')
    assert s.desc.n_shapes == 0 and s.desc.n_materials == 0
    # a directive with nothing after it is not a statement
    with pytest.raises(Exception, match="invalid statement format"):
        loaders.parse_pbrt('WorldBegin\nReverseOrientation\nWorldEnd')
    # the area light of an outer block applies to the shapes of blocks opened inside it
    s = loaders.parse_pbrt('WorldBegin\nMaterial "diffuse"\nAttributeBegin\n'
                           '  AreaLightSource "diffuse" "rgb L" [2 2 2]\n  AttributeBegin\n'
                           '    Shape "sphere" "float radius" 0.5\n  AttributeEnd\nAttributeEnd\nWorldEnd')
    assert mat(s.desc, shapes(s.desc)[0]).kind == capi.MAT_EMISSIVE
    assert [(s.desc.lights[k].kind, s.desc.lights[k].shape) for k in range(s.desc.n_lights)] == \
        [(capi.LIGHT_SPHERE, 0)]


def test_camera_defaults_lookat_and_override(loaders):
    # convertCamera (pbrt_scene.go:93-158) and parseLookAt (pbrt.go:435-490)
    from gprt.scene import CameraConfig
    s = loaders.parse_pbrt('WorldBegin\nWorldEnd')
    c = s.desc.camera
    assert tuple(c.center) == (0, 0, 0) and tuple(c.look_at) == (0, 0, -1) and c.vfov_deg == 90
    assert c.width == 400 and c.aspect_ratio == 1.0 and c.focus_distance == 1.0
    s = loaders.parse_pbrt('LookAt 1 2 3  4 5 6  0 0 1\nFilm "rgb" "integer xresolution" [300] '
                           '"integer yresolution" [200]\nWorldBegin\nWorldEnd',
                           camera=CameraConfig(width=150))
    c, sm = s.desc.camera, s.desc.sampling
    assert tuple(c.center) == (1, 2, 3) and tuple(c.look_at) == (4, 5, 6) and tuple(c.up) == (0, 0, 1)
    assert c.width == 150 and c.aspect_ratio == 1.5 and (sm.width, sm.height) == (150, 100)
    with pytest.raises(Exception, match="LookAt requires 9 values"):
        loaders.parse_pbrt('LookAt 1 2 3\nWorldBegin\nWorldEnd')
    with pytest.raises(Exception, match="invalid camera FOV"):
        loaders.parse_pbrt('Camera "perspective" "float fov" [180]\nWorldBegin\nWorldEnd')
    with pytest.raises(Exception, match="invalid image width"):
        loaders.parse_pbrt('Film "rgb" "integer xresolution" [9000]\nWorldBegin\nWorldEnd')


def test_materials_shapes_and_lights_conversion(loaders):
    from gprt import capi
    s = loaders.parse_pbrt('''WorldBegin
LightSource "point" "rgb I" [5 6 7] "point3 from" [1 2 3]
LightSource "distant"
Material "conductor" "rgb eta" [0.9 0.8 0.7] "float roughness" [0.25]
Shape "box" "point3 center" [0 1 0] "point3 size" [0.5 0.5 0.5] "point3 rotation" [0 0.3 0]
Material "dielectric"
Shape "sphere"
WorldEnd''')
    d = s.desc
    m0, m1 = d.materials[0], d.materials[1]
    assert m0.kind == capi.MAT_METAL and tuple(m0.albedo) == (0.9, 0.8, 0.7) and m0.fuzz == 0.25
    assert m1.kind == capi.MAT_DIELECTRIC and m1.ior == 1.5
    sh = shapes(d)
    assert sh[0].kind == capi.SHAPE_BOX and list(sh[0].p[:9]) == [0, 1, 0, 0.5, 0.5, 0.5, 0, 0.3, 0]
    assert sh[1].kind == capi.SHAPE_SPHERE and list(sh[1].p[:4]) == [0, 0, 0, 1]  # defaults
    pt, dist = d.lights[0], d.lights[1]
    # a 0.1-radius sphere light that is not a scene shape (pbrt_scene.go:340-349)
    assert pt.kind == capi.LIGHT_SPHERE and pt.shape == capi.NO_SHAPE and pt.radius == 0.1
    assert tuple(pt.from_) == (1, 2, 3) and tuple(pt.color_a) == (5, 6, 7)
    assert dist.kind == capi.LIGHT_UNIFORM_INFINITE and tuple(dist.color_a) == (3, 3, 3)
    for bad, msg in (('Material "plastic"', "unsupported material type"),
                     ('Material "conductor" "float roughness" [2]', "invalid metal roughness"),
                     ('Material "diffuse"\nShape "cylinder"', "unsupported shape type"),
                     ('Material "diffuse"\nShape "sphere" "float radius" [-1]', "invalid sphere radius"),
                     ('LightSource "spot"', "unsupported light type")):
        with pytest.raises(Exception, match=msg):
            loaders.parse_pbrt('WorldBegin\n' + bad + '\nWorldEnd')


def test_loaded_scene_validates_like_the_oracle(loaders, oracle):
    # the description the loader builds is one the library and the oracle both accept
    import ctypes as C
    import gprt
    s = loaders.parse_pbrt(HEAD + '''LightSource "point" "rgb I" [5 5 5] "point3 from" [0 4 0]
Material "diffuse" "rgb reflectance" [0.5 0.5 0.5]
Shape "bilinearPatch" "point3 P00" [-5 0 -5] "point3 P01" [5 0 -5] "point3 P10" [-5 0 5] "point3 P11" [5 0 5]
Shape "sphere" "float radius" [1] "point3 center" [0 1 0]
WorldEnd''')
    info = gprt.capi.SceneInfo()
    err = C.create_string_buffer(256)
    rc = gprt.capi.load().gprt_scene_validate(s.ptr(), C.byref(info), err, 256)
    assert rc == 0, err.value
    o = oracle.OracleScene(s)
    assert info.world_radius == pytest.approx(o.world_radius, rel=1e-12)
    assert (info.image_width, info.image_height) == (o.width, o.height) == (200, 200)


def test_load_pbrt_path_rules(loaders, tmp_path):
    # validateFilePath (pbrt.go:391-433)
    d = tempfile.mkdtemp()
    good = os.path.join(d, "scene.pbrt")
    with open(good, "w") as f:
        f.write(HEAD + 'Material "diffuse"\nShape "sphere"\nWorldEnd\n')
    assert loaders.load_pbrt(good).desc.n_shapes == 1
    bad = os.path.join(d, "scene.txt")
    with open(bad, "w") as f:
        f.write("WorldBegin\n")
    with pytest.raises(Exception, match="only .pbrt files"):
        loaders.load_pbrt(bad)
    with pytest.raises(Exception, match="must be in scenes/"):
        loaders.load_pbrt("/etc/x.pbrt")
    with pytest.raises(Exception, match="cannot be empty"):
        loaders.load_pbrt("")


# ------------------------------------------------------------------ PLY
def write_ply(path, verts, faces, normals=None, colors=None, count="uchar", index="int", extra_face=False,
              fmt="binary_little_endian"):
    head = ["ply", "format %s 1.0" % fmt, "comment made by the test", "element vertex %d" % len(verts),
            "property float x", "property float y", "property float z"]
    if normals is not None:
        head += ["property float nx", "property float ny", "property float nz"]
    if colors is not None:
        head += ["property uchar red", "property uchar green", "property uchar blue"]
    head += ["element face %d" % len(faces), "property list %s %s vertex_indices" % (count, index)]
    if extra_face:
        head += ["property uchar flags", "property list uchar float weights"]
    head += ["end_header"]
    body = b""
    for k, v in enumerate(verts):
        body += struct.pack("<3f", *v)
        if normals is not None:
            body += struct.pack("<3f", *normals[k])
        if colors is not None:
            body += struct.pack("<3B", *colors[k])
    for f in faces:
        body += struct.pack("<B" if count == "uchar" else "<i", len(f))
        body += struct.pack("<%d%s" % (len(f), "i" if index == "int" else "I"), *f)
        if extra_face:
            body += struct.pack("<B", 7) + struct.pack("<B2f", 2, 0.5, 0.25)
    with open(path, "wb") as fh:
        fh.write(("\n".join(head) + "\n").encode() + body)


def test_ply_basic_normals_colors(loaders, tmp_path):
    # TestLoadPLY_Basic / _WithNormals / _WithColors (ply_test.go:94-205)
    verts = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0.5)]
    faces = [(0, 1, 2), (1, 3, 2)]
    p = str(tmp_path / "a.ply")
    write_ply(p, verts, faces)
    d = loaders.load_ply(p)
    assert np.array_equal(d.vertices, np.array(verts, dtype=np.float64))
    assert np.array_equal(d.faces, np.array(faces))
    assert d.normals is None and d.colors is None
    nrm = [(0, 0, 1)] * 4
    col = [(255, 0, 0), (0, 255, 0), (0, 0, 255), (51, 102, 204)]
    write_ply(p, verts, faces, normals=nrm, colors=col, count="int", index="uint", extra_face=True)
    d = loaders.load_ply(p)
    assert np.array_equal(d.normals, np.array(nrm, dtype=np.float64))
    assert np.allclose(d.colors, np.array(col) / 255.0)
    assert np.array_equal(d.faces, np.array(faces))  # the extra face properties were skipped


def test_ply_errors(loaders, tmp_path):
    p = str(tmp_path / "b.ply")
    with pytest.raises(Exception, match="failed to open PLY file"):
        loaders.load_ply(str(tmp_path / "missing.ply"))  # TestLoadPLY_NonExistentFile
    write_ply(p, [(0, 0, 0)] * 4, [(0, 1, 2, 3)])
    with pytest.raises(Exception, match="only triangular faces supported"):
        loaders.load_ply(p)
    write_ply(p, [(0, 0, 0)] * 3, [(0, 1, 2)], fmt="ascii")
    with pytest.raises(Exception, match="ASCII PLY format not yet supported"):
        loaders.load_ply(p)
    write_ply(p, [(0, 0, 0)] * 3, [(0, 1, 2)], fmt="binary_big_endian")
    with pytest.raises(Exception, match="big-endian PLY format not yet implemented"):
        loaders.load_ply(p)
    write_ply(p, [(0, 0, 0)] * 3, [(0, 1, 7)])
    with pytest.raises(Exception, match="index out of range"):
        loaders.load_ply(p)


def test_ply_extra_elements_and_truncation(loaders, tmp_path):
    # elements other than vertex and face are skipped; a file that ends early
    # is an error, not a short mesh
    p = str(tmp_path / "c.ply")
    write_ply(p, [(0, 0, 0), (1, 0, 0), (0, 1, 0)], [(0, 1, 2)])
    head, body = open(p, "rb").read().split(b"end_header\n")
    head += b"element edge 1\nproperty int vertex1\nproperty int vertex2\n"
    open(p, "wb").write(head + b"end_header\n" + body + struct.pack("<2i", 0, 1))
    d = loaders.load_ply(p)
    assert np.array_equal(d.faces, np.array([(0, 1, 2)]))
    open(p, "wb").write(head + b"end_header\n" + body[:-5])
    with pytest.raises(Exception, match="unexpected EOF"):
        loaders.load_ply(p)


def _png(path, pixels, ctype, depth=8, palette=None, trns=None, filters=(0,)):
    import struct
    import zlib
    h, w = pixels.shape[:2]
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    raw = b""
    for y in range(h):
        f = filters[y % len(filters)]
        row = pixels[y].reshape(-1)
        data = row.astype(">u2").tobytes() if depth == 16 else row.astype(np.uint8).tobytes()
        line = np.frombuffer(data, dtype=np.uint8).astype(np.int64)
        bpp = ch * depth // 8
        if f == 1:  # Sub
            enc = line.copy()
            enc[bpp:] = (line[bpp:] - line[:-bpp]) & 0xFF
        else:
            enc = line
        raw += bytes([f]) + enc.astype(np.uint8).tobytes()

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    blob = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    if palette is not None:
        blob += chunk(b"PLTE", np.asarray(palette, dtype=np.uint8).tobytes())
    if trns is not None:
        blob += chunk(b"tRNS", bytes(trns))
    blob += chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b"")
    open(path, "wb").write(blob)


def test_load_image_png(loaders, tmp_path):
    # LoadImage (pkg/loaders/image.go:21-61, image_test.go): colour / 65535 of
    # the alpha-premultiplied 16-bit RGBA of each pixel, row 0 at the top
    p = str(tmp_path / "a.png")
    rgb = np.array([[[255, 0, 0], [0, 255, 0]], [[0, 0, 255], [128, 64, 32]]], dtype=np.int64)
    _png(p, rgb, 2, filters=(0, 1))
    t = loaders.load_image(p)
    assert t.width == 2 and t.height == 2
    assert np.allclose(t.pixels, rgb / 255.0)
    rgba = np.array([[[255, 255, 255, 128], [10, 20, 30, 255]]], dtype=np.int64)
    _png(p, rgba, 6)
    t = loaders.load_image(p)
    a = 128 * 257
    assert np.allclose(t.pixels[0, 0], np.floor(255 * 257 * a / 65535) / 65535)
    assert np.allclose(t.pixels[0, 1], np.array([10, 20, 30]) / 255.0)
    g16 = np.array([[[0], [65535], [4660]]], dtype=np.int64)
    _png(p, g16, 0, depth=16)
    t = loaders.load_image(p)
    assert np.allclose(t.pixels[0, :, 0], [0.0, 1.0, 4660 / 65535])
    _png(p, np.array([[[1], [0]]], dtype=np.int64), 3, palette=[[0, 0, 0], [200, 100, 50]], trns=[0, 255])
    t = loaders.load_image(p)
    assert np.allclose(t.pixels[0, 0], [200 / 255, 100 / 255, 50 / 255]) and np.allclose(t.pixels[0, 1], 0)
    open(p, "wb").write(b"\xff\xd8\xff not a png")
    with pytest.raises(ValueError, match="only PNG"):
        loaders.load_image(p)
    with pytest.raises(ValueError, match="failed to open image file"):
        loaders.load_image(str(tmp_path / "missing.png"))
