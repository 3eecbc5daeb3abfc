"""Scene ingestion on CPU: the PBRT lexer/parser/builder, Radiance .hdr and
glTF 2.0 readers (pyre_gb300.io).

The lexer and parser cases restate the reference's own unit tests
(crates/pyre/src/io/pbrt/lexer.rs:166-193, parser.rs:333-393). The builder is
checked by writing the built-in Cornell box as PBRT text and loading it back.
"""
import base64
import json
import struct

import numpy as np
import pytest

from pyre_gb300 import presets as P
from pyre_gb300.io import gltf as G
from pyre_gb300.io import hdr as H
from pyre_gb300.io import pbrt as B
from pyre_gb300.scene import DiffuseAreaQuadLight, DisneyBsdf, Lambertian

F32 = np.float32


# --------------------------------------------------------------- lexer KATs --
def test_tokenizes_lookat():
    toks = B.tokenize("LookAt 3 4 1.5 .5 .5 0 0 0 1")
    assert toks[0].kind == "ident" and toks[0].value == "LookAt"
    assert len(toks) == 10


def test_tokenizes_parameter_pair():
    toks = B.tokenize('Camera "perspective" "float fov" [39]')
    assert [(t.kind, t.value) for t in toks] == [("ident", "Camera"), ("string", "perspective"),
                                                 ("string", "float fov"), ("[", "["), ("int", 39), ("]", "]")]


def test_skips_comments():
    toks = B.tokenize("# only a comment\nLookAt 1 2 3 0 0 0 0 1 0")
    assert toks[0].kind == "ident" and toks[0].value == "LookAt" and toks[0].line == 2


@pytest.mark.parametrize("src", ['Shape "trianglemesh', "LookAt 1 2 $", 'X "a\nb"', "Translate 1-"])
def test_lex_errors(src):
    with pytest.raises(B.LexError):
        B.tokenize(src)


# -------------------------------------------------------------- parser KATs --
def test_parses_lookat():
    dirs = B.parse(B.tokenize("LookAt 3 4 1.5 0.5 0.5 0 0 1 0"))
    assert len(dirs) == 1 and dirs[0].keyword == "LookAt"
    assert len(dirs[0].positional) == 9 and abs(dirs[0].positional[0] - 3.0) < 1e-6


def test_parses_camera_with_param():
    d = B.parse(B.tokenize('Camera "perspective" "float fov" [39]'))[0]
    assert d.keyword == "Camera" and len(d.positional) == 1 and len(d.params) == 1
    p = d.params[0]
    assert (p.name, p.type_name, p.kind, p.values) == ("fov", "float", "floats", [39.0])


def test_parses_two_directives():
    dirs = B.parse(B.tokenize('LookAt 0 0 3 0 0 0 0 1 0\n   Camera "perspective" "float fov" [45]'))
    assert [d.keyword for d in dirs] == ["LookAt", "Camera"]


def test_parses_mixed_int_float_as_floats():
    p = B.parse(B.tokenize('X "rgb Kd" [0.5 0 1]'))[0].params[0]
    assert p.kind == "floats" and len(p.values) == 3


def test_parse_value_kinds():
    d = B.parse(B.tokenize('S "integer indices" [0 1 2] "string name" "a" "float r" 2 "integer n" [1 2.5]'))[0]
    kinds = {p.name: (p.kind, p.values) for p in d.params}
    assert kinds["indices"] == ("ints", [0, 1, 2])
    assert kinds["name"] == ("strings", ["a"])
    assert kinds["r"] == ("floats", [2.0])
    assert kinds["n"] == ("floats", [1.0, 2.5])  # an int list that meets a float becomes floats


@pytest.mark.parametrize("src", ['X "float a" [1 "b"]', "X ]", 'X "float " 1', 'X "float a" [1 2', "1 2 3"])
def test_parse_errors(src):
    with pytest.raises(B.ParseError):
        B.parse(B.tokenize(src))


# ----------------------------------------------------------------- builder --
def _fmt(v) -> str:
    return " ".join(repr(float(F32(x))) for x in np.asarray(v, F32).reshape(-1))


def scene_to_pbrt(scene, eye, target, up, fov, width, height) -> str:
    """Writes a scene of quads/meshes, matte or Disney materials and quad
    lights as PBRT text in the loader's subset (explicit normals)."""
    out = [f"LookAt {_fmt(eye)}  {_fmt(target)}  {_fmt(up)}", f'Camera "perspective" "float fov" [{fov}]',
           f'Film "image" "integer xresolution" [{width}] "integer yresolution" [{height}]', "WorldBegin"]
    for prim in scene.primitives:
        m = scene.materials[prim.material_id]
        mesh = prim.instance.mesh
        out.append("AttributeBegin")
        if isinstance(m, Lambertian):
            out.append(f'  Material "matte" "rgb Kd" [{_fmt(m.albedo)}]')
        else:
            assert m.metallic == 0.0
            out.append(f'  Material "plastic" "rgb Kd" [{_fmt(m.base_color)}] "rgb Ks" [{_fmt([m.specular] * 3)}] '
                       f'"float roughness" [{_fmt([m.roughness])}]')
        out.append(f'  Shape "trianglemesh" "point P" [{_fmt(mesh.positions)}]')
        if mesh.normals is not None:
            out.append(f'    "normal N" [{_fmt(mesh.normals)}]')
        out.append(f'    "integer indices" [{" ".join(str(int(i)) for i in mesh.indices)}]')
        out.append("AttributeEnd")
    for L in scene.lights:
        c = [L.p0, L.p0 + L.edge_u, L.p0 + L.edge_u + L.edge_v, L.p0 + L.edge_v]
        out += ["AttributeBegin", f'  AreaLightSource "diffuse" "rgb L" [{_fmt(L.emission)}]',
                f'  Shape "trianglemesh" "point P" [{_fmt(np.array(c, F32))}] "integer indices" [0 1 2 0 2 3]',
                "AttributeEnd"]
    out.append("WorldEnd")
    return "\n".join(out) + "\n"


def test_cornell_box_round_trip(tmp_path):
    sc = P.cornell_box()
    f = tmp_path / "cornell.pbrt"
    f.write_text(scene_to_pbrt(sc, (0, 0, 3), (0, 0, 0), (0, 1, 0), 45, 256, 256))
    ld = B.load_pbrt(f)
    assert ld.film.width == 256 and ld.film.height == 256 and ld.film.filename is None
    assert ld.camera.vfov_deg == 45.0 and np.array_equal(ld.camera.origin, [0, 0, 3])
    out = ld.scene
    assert len(out.primitives) == len(sc.primitives)
    for a, b in zip(out.primitives, sc.primitives):
        np.testing.assert_array_equal(a.instance.mesh.positions, b.instance.mesh.positions)
        np.testing.assert_array_equal(a.instance.mesh.indices, b.instance.mesh.indices)
        np.testing.assert_allclose(a.instance.mesh.normals, b.instance.mesh.normals, atol=1e-7)
        np.testing.assert_array_equal(out.materials[a.material_id].albedo, sc.materials[b.material_id].albedo)
    assert len(out.lights) == 1
    for k in ("p0", "edge_u", "edge_v", "emission"):
        np.testing.assert_allclose(getattr(out.lights[0], k), getattr(sc.lights[0], k), atol=1e-7)


def test_transforms_and_attribute_stack():
    src = """WorldBegin
    AttributeBegin
      Translate 1 2 3
      Scale 2 2 2
      Material "matte" "rgb Kd" [0.2 0.3 0.4]
      Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
    AttributeEnd
    Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
    AttributeBegin
      Rotate 90 0 0 1
      Shape "trianglemesh" "point P" [1 0 0 2 0 0 1 1 0] "integer indices" [0 1 2]
    AttributeEnd
    TransformBegin
      ConcatTransform [1 0 0 0  0 1 0 0  0 0 1 0  5 6 7 1]
      Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
    TransformEnd
    """
    with pytest.warns(UserWarning, match="gray"):
        sc = B.build(B.parse(B.tokenize(src))).scene
    p0, p1, p2, p3 = (pr.instance.mesh.positions for pr in sc.primitives)
    np.testing.assert_array_equal(p0, [[1, 2, 3], [3, 2, 3], [1, 4, 3]])    # translate then scale
    np.testing.assert_array_equal(p1, [[0, 0, 0], [1, 0, 0], [0, 1, 0]])    # attribute stack restored
    np.testing.assert_allclose(p2, [[0, 1, 0], [0, 2, 0], [-1, 1, 0]], atol=1e-6)  # +90 deg about z
    np.testing.assert_array_equal(p3, [[5, 6, 7], [6, 6, 7], [5, 7, 7]])    # column-major 16-float array
    assert isinstance(sc.materials[sc.primitives[0].material_id], Lambertian)
    # shapes without a current material get a fresh gray Lambertian each
    assert sc.primitives[1].material_id != 0
    np.testing.assert_array_equal(sc.materials[sc.primitives[1].material_id].albedo, [0.5, 0.5, 0.5])


def test_materials_lights_and_sphere(tmp_path):
    env = (np.arange(16 * 8 * 3, dtype=F32).reshape(8, 16, 3) % 7 + 1) / F32(4)
    (tmp_path / "sky.hdr").write_bytes(H.encode_hdr(env))
    src = """WorldBegin
    MakeNamedMaterial "gold" "string type" "metal" "float roughness" [0.3]
    MakeNamedMaterial "shiny" "string type" "plastic" "rgb Kd" [0.1 0.2 0.3]
    LightSource "infinite" "string mapname" "sky.hdr" "float scale" [2]
    NamedMaterial "gold"
    Shape "sphere" "float radius" [0.5]
    NamedMaterial "shiny"
    AttributeBegin
      AreaLightSource "diffuse" "rgb L" [4 5 6]
      Shape "trianglemesh" "point P" [0 1 0 1 1 0 1 1 1 0 1 1] "integer indices" [0 1 2 0 2 3]
    AttributeEnd
    """
    ld = B.build(B.parse(B.tokenize(src)), tmp_path)
    sc = ld.scene
    gold, shiny = sc.materials
    assert isinstance(gold, DisneyBsdf) and gold.metallic == 1.0 and gold.roughness == F32(0.3)
    np.testing.assert_array_equal(gold.base_color, F32([1.0, 0.766, 0.336]))
    assert isinstance(shiny, DisneyBsdf) and shiny.metallic == 0.0 and shiny.roughness == F32(0.2)
    assert shiny.specular == F32(0.5)
    mesh = sc.primitives[0].instance.mesh
    assert mesh.positions.shape == (49 * 25, 3) and mesh.triangle_count() == 48 * 24 * 2
    np.testing.assert_allclose(np.linalg.norm(mesh.positions, axis=1), 0.5, atol=1e-6)
    assert len(sc.lights) == 1 and isinstance(sc.lights[0], DiffuseAreaQuadLight)
    np.testing.assert_array_equal(sc.lights[0].edge_v, [0, 0, 1])
    np.testing.assert_array_equal(sc.lights[0].emission, [4, 5, 6])
    assert sc.env.width == 16 and sc.env.height == 8 and sc.env.intensity == 2.0
    ref = H.rgbe_to_float(H.float_to_rgbe(env))
    np.testing.assert_array_equal(sc.env.pixels, ref)
    assert ld.camera is None and ld.film is None


def test_constant_environment_and_defaults():
    sc = B.build(B.parse(B.tokenize('WorldBegin LightSource "infinite" "rgb L" [0.5 0.25 1]'))).scene
    assert sc.env.width == 1 and sc.env.height == 1 and sc.env.intensity == 1.0
    np.testing.assert_array_equal(sc.env.pixels.reshape(3), [0.5, 0.25, 1])
    ld = B.build(B.parse(B.tokenize('Film "image"  LookAt 0 0 1 0 0 0 0 1 0  Camera "perspective"')))
    assert (ld.film.width, ld.film.height) == (800, 600)
    assert ld.camera is None  # no fov given


@pytest.mark.parametrize("src,match", [
    ("AttributeEnd", "AttributeEnd"),
    ("TransformEnd", "TransformEnd"),
    ('NamedMaterial "nope"', "not declared"),
    ('WorldBegin Shape "trianglemesh" "integer indices" [0 1 2]', '"P"'),
    ('WorldBegin Shape "trianglemesh" "point P" [0 0 0 1] "integer indices" [0 1 2]', "multiple of 3"),
    ("Translate 1 2", "expected 3"),
    ("Transform [1 2 3]", "16-float"),
])
def test_build_errors(src, match):
    with pytest.raises(B.BuildError, match=match):
        B.build(B.parse(B.tokenize(src)))


def test_unsupported_directives_are_skipped():
    with pytest.warns(UserWarning):
        sc = B.build(B.parse(B.tokenize('Texture "t" "spectrum" "imagemap" WorldBegin Shape "disk"'))).scene
    assert not sc.primitives


# --------------------------------------------------------------------- hdr --
def test_rgbe_known_values():
    px = np.array([[128, 64, 32, 129], [0, 0, 0, 0], [255, 1, 0, 136], [200, 100, 50, 0]], np.uint8)
    out = H.rgbe_to_float(px)
    np.testing.assert_array_equal(out, F32([[1.0, 0.5, 0.25], [0, 0, 0], [255, 1, 0], [0, 0, 0]]))


def test_hdr_flat_and_rle_files():
    rgbe = np.array([[[128, 64, 32, 129], [10, 20, 30, 130]], [[1, 2, 3, 140], [0, 0, 0, 0]]], np.uint8)
    flat = b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 2 +X 2\n" + rgbe.tobytes()
    w, h, px = H.decode_hdr(flat)
    assert (w, h) == (2, 2)
    np.testing.assert_array_equal(px, H.rgbe_to_float(rgbe))
    # adaptive RLE, one scanline of 9 pixels: runs and literals per channel
    row = np.zeros((9, 4), np.uint8)
    row[:, 0] = [7] * 9
    row[:, 1] = np.arange(9)
    row[:, 2] = [1, 1, 1, 1, 2, 3, 3, 3, 3]
    row[:, 3] = 130
    enc = bytes([2, 2, 0, 9]) + bytes([128 + 9, 7]) + bytes([9]) + bytes(range(9)) \
        + bytes([128 + 4, 1, 1, 2, 128 + 4, 3]) + bytes([128 + 9, 130])
    w, h, px = H.decode_hdr(b"#?RADIANCE\n\n-Y 1 +X 9\n" + enc)
    np.testing.assert_array_equal(px[0], H.rgbe_to_float(row))


def test_hdr_round_trip_and_errors(tmp_path):
    rng = np.random.default_rng(3)
    img = (rng.random((5, 37, 3)) * 10).astype(F32)
    img[2, 3:20] = 0.5  # runs
    w, h, px = H.decode_hdr(H.encode_hdr(img))
    np.testing.assert_array_equal(px, H.rgbe_to_float(H.float_to_rgbe(img)))
    # one shared exponent per pixel: error below 1/128 of the pixel's largest channel
    assert np.all(np.abs(px - img) <= img.max(axis=-1, keepdims=True) / 128)
    with pytest.raises(H.HdrLoadError):
        H.decode_hdr(b"P6 not radiance")
    with pytest.raises(H.HdrLoadError):
        H.decode_hdr(b"#?RADIANCE\n\n+Y 2 +X 2\n" + bytes(16))
    with pytest.raises(H.HdrLoadError):
        H.decode_hdr(b"#?RADIANCE\n\n-Y 2 +X 2\n" + bytes(8))
    (tmp_path / "a.exr").write_bytes(b"")
    with pytest.raises(H.HdrLoadError, match="extension"):
        H.load_hdri(tmp_path / "a.exr", 1.0)


# -------------------------------------------------------------------- gltf --
def _gltf_doc(buffer_uri=None, mode=4):
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], F32)
    nor = np.array([[0, 0, 1]] * 3, F32)
    uv = np.array([[0, 0], [65535, 0], [0, 65535]], np.uint16)
    idx = np.array([0, 1, 2], np.uint16)
    blob = pos.tobytes() + nor.tobytes() + uv.tobytes() + idx.tobytes() + b"\0\0"
    doc = {
        "asset": {"version": "2.0"}, "scene": 0,
        "scenes": [{"nodes": [0]}],
        "nodes": [{"translation": [1, 2, 3], "scale": [2, 1, 1], "children": [1]},
                  {"matrix": [0, 1, 0, 0, -1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1], "mesh": 0}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "NORMAL": 1, "TEXCOORD_0": 2}, "indices": 3,
                                    "mode": mode}]}],
        "buffers": [{"byteLength": len(blob)}],
        "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": 36},
                        {"buffer": 0, "byteOffset": 36, "byteLength": 36},
                        {"buffer": 0, "byteOffset": 72, "byteLength": 12},
                        {"buffer": 0, "byteOffset": 84, "byteLength": 6}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": 3, "type": "VEC3"},
                      {"bufferView": 1, "componentType": 5126, "count": 3, "type": "VEC3"},
                      {"bufferView": 2, "componentType": 5123, "count": 3, "type": "VEC2", "normalized": True},
                      {"bufferView": 3, "componentType": 5123, "count": 3, "type": "SCALAR"}],
    }
    if buffer_uri:
        doc["buffers"][0]["uri"] = buffer_uri(blob)
    return doc, blob


def _check_mesh(meshes):
    assert len(meshes) == 1
    m = meshes[0]
    # child rotates +90 deg about z, parent scales x by 2 then translates
    np.testing.assert_allclose(m.positions, [[1, 2, 3], [1, 3, 3], [-1, 2, 3]], atol=1e-6)
    np.testing.assert_allclose(m.normals, [[0, 0, 1]] * 3, atol=1e-6)
    np.testing.assert_allclose(m.uvs, [[0, 0], [1, 0], [0, 1]])
    np.testing.assert_array_equal(m.indices, [0, 1, 2])


def test_gltf_data_uri_and_external_buffer(tmp_path):
    doc, _ = _gltf_doc(lambda b: "data:application/octet-stream;base64," + base64.b64encode(b).decode())
    (tmp_path / "a.gltf").write_text(json.dumps(doc))
    _check_mesh(G.load_gltf(tmp_path / "a.gltf"))
    doc, blob = _gltf_doc(lambda b: "a.bin")
    (tmp_path / "a.bin").write_bytes(blob)
    (tmp_path / "b.gltf").write_text(json.dumps(doc))
    _check_mesh(G.load_gltf(tmp_path / "b.gltf"))


def test_glb_and_normal_transform(tmp_path):
    doc, blob = _gltf_doc()
    js = json.dumps(doc).encode()
    js += b" " * (-len(js) % 4)
    blob += b"\0" * (-len(blob) % 4)
    data = struct.pack("<III", 0x46546C67, 2, 12 + 8 + len(js) + 8 + len(blob)) + struct.pack("<II", len(js),
                                                                                          0x4E4F534A) + js
    data += struct.pack("<II", len(blob), 0x004E4942) + blob
    (tmp_path / "a.glb").write_bytes(data)
    _check_mesh(G.load_gltf(tmp_path / "a.glb"))
    # a tilted normal under non-uniform scale follows the inverse transpose
    node = {"scale": [2, 1, 1]}
    m = G.node_matrix(node)
    n = np.array([1, 1, 0], F32) @ np.linalg.inv(m[:3, :3]).T.T
    n /= np.linalg.norm(n)
    np.testing.assert_allclose(n, [1 / np.sqrt(5), 2 / np.sqrt(5), 0], atol=1e-6)


def test_gltf_errors(tmp_path):
    doc, _ = _gltf_doc(lambda b: "data:;base64," + base64.b64encode(b).decode(), mode=1)
    (tmp_path / "lines.gltf").write_text(json.dumps(doc))
    with pytest.raises(G.GltfError, match="non-triangle"):
        G.load_gltf(tmp_path / "lines.gltf")
    doc, _ = _gltf_doc(lambda b: "data:;base64," + base64.b64encode(b).decode())
    del doc["meshes"][0]["primitives"][0]["attributes"]["POSITION"]
    (tmp_path / "nopos.gltf").write_text(json.dumps(doc))
    with pytest.raises(G.GltfError, match="positions"):
        G.load_gltf(tmp_path / "nopos.gltf")
    (tmp_path / "empty.gltf").write_text(json.dumps({"asset": {"version": "2.0"}}))
    assert G.load_gltf(tmp_path / "empty.gltf") == []


# ------------------------------------------------------------------- sinks --
def _film(w=13, h=7, seed=1):
    from pyre_gb300.scene import Film
    rng = np.random.default_rng(seed)
    f = Film(w, h)
    f.radiance[:] = (rng.random(f.radiance.shape) * 1.5 - 0.2).astype(F32)
    f.albedo[:] = rng.random(f.albedo.shape).astype(F32)
    f.normal[:] = (rng.random(f.normal.shape) * 2 - 1).astype(F32)
    d = (rng.random(f.depth.shape) * 5).astype(F32)
    d[d < 1] = 0.0  # misses
    f.depth[:] = d
    return f


def test_ldr_encodings():
    from pyre_gb300 import sinks as S
    x = F32([[-1.0, 0.0, 1e-3], [0.5, 1.0, 7.0]])
    got = S.encode_gamma8(x)
    want = [[0, 0, int(F32(np.power(F32(1e-3), F32(1) / F32(2.2))) * F32(255))],
            [int(F32(np.power(F32(0.5), F32(1) / F32(2.2))) * F32(255)), 255, 255]]
    np.testing.assert_array_equal(got, want)
    assert S.encode_gamma8(F32([0.5]))[0] == 186  # 0.5^(1/2.2) = 0.7297 -> 186.07 truncated
    np.testing.assert_array_equal(S.encode_normal8(F32([-1, 0, 1, 3])), [0, 127, 255, 255])
    d = S.encode_depth8(F32([0.0, 2.0, 4.0, 3.0]))
    np.testing.assert_array_equal(d, [0, 255, 0, 127])  # near bright, misses black


def test_png_sinks(tmp_path):
    from pyre_gb300 import sinks as S
    f = _film()
    S.save_png(f, tmp_path / "frame.png")
    img = S.read_png(tmp_path / "frame.png")
    np.testing.assert_array_equal(img, S.encode_gamma8(f.radiance.reshape(7, 13, 3)))
    paths = S.save_aov_pngs(f, tmp_path / "frame.png")
    assert [p.name for p in paths] == ["frame.albedo.png", "frame.normal.png", "frame.depth.png"]
    np.testing.assert_array_equal(S.read_png(paths[1]), S.encode_normal8(f.normal.reshape(7, 13, 3)))
    np.testing.assert_array_equal(S.read_png(paths[2]), S.encode_depth8(f.depth.reshape(7, 13)))


@pytest.mark.parametrize("comp", [0, 2, 3])
def test_exr_channels_round_trip(tmp_path, comp):
    from pyre_gb300 import sinks as S
    f = _film(w=21, h=37)
    if comp == 3:
        S.save_exr(f, tmp_path / "a.exr")
    else:
        rad = f.radiance.reshape(37, 21, 3)
        S.write_exr(tmp_path / "a.exr", {"R": rad[..., 0], "G": rad[..., 1], "B": rad[..., 2]}, 21, 37, comp)
    data = (tmp_path / "a.exr").read_bytes()
    assert struct.unpack_from("<ii", data) == (20000630, 2)
    planes = S.read_exr(tmp_path / "a.exr")
    names = list(planes)
    assert names == sorted(names)
    if comp == 3:
        assert names == ["B", "G", "N.X", "N.Y", "N.Z", "R", "Z", "albedo.B", "albedo.G", "albedo.R"]
        np.testing.assert_array_equal(planes["Z"], f.depth.reshape(37, 21))
        np.testing.assert_array_equal(planes["N.Y"], f.normal.reshape(37, 21, 3)[..., 1])
        np.testing.assert_array_equal(planes["albedo.R"], f.albedo.reshape(37, 21, 3)[..., 0])
    np.testing.assert_array_equal(planes["G"], f.radiance.reshape(37, 21, 3)[..., 1])
