"""PBRT scene-file loader (the directive subset of crates/pyre/src/io/pbrt).

Three layers, as in the reference:
  tokenize  text -> tokens                 (io/pbrt/lexer.rs:49-159)
  parse     tokens -> flat directive list  (io/pbrt/parser.rs:100-312)
  build     directives -> Scene + optional camera and film settings
            (io/pbrt/builder.rs:69-296)

Supported: LookAt, Camera "perspective" (fov), Film (xresolution,
yresolution, filename); Sampler / Integrator / Accelerator / PixelFilter are
parsed and ignored. Transforms Identity, Translate, Scale, Rotate, Transform,
ConcatTransform; AttributeBegin/End, TransformBegin/End, WorldBegin/End.
Materials matte -> Lambertian, plastic / metal / conductor -> DisneyBsdf
(builder.rs:303-356); Material, MakeNamedMaterial, NamedMaterial.
LightSource "infinite" (constant L or mapname .hdr), AreaLightSource
"diffuse" on a four-vertex two-triangle trianglemesh -> DiffuseAreaQuadLight.
Shapes sphere (48 x 24 UV tessellation, builder.rs:520-555) and
trianglemesh. Anything else is skipped with a warning, so partial scenes
still load. +Y is up (the reference's convention).

Matrix arithmetic is float32 with the glam conventions the reference uses:
column vectors, `ctm = ctm * M` for each transform, `transform_point3` =
x_axis * p.x + y_axis * p.y + z_axis * p.z + w_axis (left to right).
"""
from __future__ import annotations

import math
import warnings
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from ..scene import (DiffuseAreaQuadLight, DisneyBsdf, HdriEnvironmentLight, Lambertian, MeshInstance, Primitive,
                     Scene, TriangleMesh)

F32 = np.float32


# ------------------------------------------------------------------ lexer --
class PbrtError(Exception):
    """Any load failure (the reference's PbrtError: io, lex, parse, build)."""


class LexError(PbrtError):
    pass


class ParseError(PbrtError):
    pass


class BuildError(PbrtError):
    pass


@dataclass
class Token:
    kind: str     # "ident", "string", "int", "float", "[", "]"
    value: object
    line: int
    col: int


def _is_number_start(c: str) -> bool:
    return c.isdigit() or c in "-+."


def _is_number_body(c: str) -> bool:
    return c.isdigit() or c in "-+.eE"


def tokenize(src: str) -> list[Token]:
    """lexer.rs:49-159: whitespace and `#` comments skipped, strings in double
    quotes (no escapes, no newlines), numbers are floats when they contain
    `.`, `e` or `E`, else integers (floats when out of i64 range)."""
    out = []
    i, line, line_start, n = 0, 1, 0, len(src)
    while i < n:
        col = i - line_start + 1
        c = src[i]
        if c in " \t\r":
            i += 1
        elif c == "\n":
            line += 1
            i += 1
            line_start = i
        elif c == "#":
            while i < n and src[i] != "\n":
                i += 1
        elif c in "[]":
            out.append(Token(c, c, line, col))
            i += 1
        elif c == '"':
            i += 1
            start = i
            while i < n and src[i] != '"':
                if src[i] == "\n":
                    raise LexError(f"line {line}, col {col}: unterminated string literal")
                i += 1
            if i >= n:
                raise LexError(f"line {line}, col {col}: unterminated string literal")
            out.append(Token("string", src[start:i], line, col))
            i += 1
        elif _is_number_start(c):
            start = i
            while i < n and _is_number_body(src[i]):
                i += 1
            text = src[start:i]
            try:
                if any(ch in text for ch in ".eE"):
                    tok = Token("float", float(text), line, col)
                else:
                    v = int(text)
                    tok = Token("int", v, line, col) if -(1 << 63) <= v < (1 << 63) else Token("float", float(v),
                                                                                               line, col)
            except ValueError:
                raise LexError(f"line {line}, col {col}: invalid number {text!r}") from None
            out.append(tok)
        elif c.isascii() and (c.isalpha() or c == "_"):
            start = i
            while i < n and src[i].isascii() and (src[i].isalnum() or src[i] == "_"):
                i += 1
            out.append(Token("ident", src[start:i], line, col))
        else:
            raise LexError(f"line {line}, col {col}: unexpected character {c!r}")
    return out


# ----------------------------------------------------------------- parser --
FLOAT_TYPES = {"float", "rgb", "color", "spectrum", "blackbody", "point", "point2", "point3", "vector", "vector2",
               "vector3", "normal", "normal3", "xyz"}


@dataclass
class Param:
    type_name: str
    name: str
    kind: str          # "floats", "ints", "strings"
    values: list
    line: int


@dataclass
class Directive:
    keyword: str
    line: int
    positional: list = field(default_factory=list)   # float, str or list[float]
    params: list = field(default_factory=list)

    def param(self, name: str) -> Param | None:
        for p in self.params:
            if p.name == name:
                return p
        return None


def _param_values(toks, k, header: Token):
    """parser.rs:226-312: one value, or a bracketed list; ints and floats mix
    into floats, strings do not mix with numbers."""
    bracketed = k < len(toks) and toks[k].kind == "["
    if bracketed:
        k += 1
    seen, vals = None, []
    while True:
        if k >= len(toks):
            if bracketed:
                raise ParseError(f"line {toks[-1].line}: unexpected end of input")
            break
        t = toks[k]
        if t.kind == "]" and bracketed:
            k += 1
            break
        if t.kind == "float":
            if seen == "strings":
                raise ParseError(f"line {t.line}: mixed types in parameter array")
            if seen == "ints":
                vals = [float(v) for v in vals]
            seen = "floats"
            vals.append(float(t.value))
            k += 1
        elif t.kind == "int":
            if seen == "strings":
                raise ParseError(f"line {t.line}: mixed types in parameter array")
            if seen is None:
                seen = "ints"
            vals.append(float(t.value) if seen == "floats" else int(t.value))
            k += 1
        elif t.kind == "string":
            if seen not in (None, "strings"):
                raise ParseError(f"line {t.line}: mixed types in parameter array")
            seen = "strings"
            vals.append(t.value)
            k += 1
        else:
            if bracketed:
                raise ParseError(f"line {t.line}: expected value or `]`, found {t.kind}")
            break
        if not bracketed:
            break
    if seen is None:
        raise ParseError(f"line {header.line}: expected parameter value, found (empty)")
    return seen, vals, k


def parse(toks: list[Token]) -> list[Directive]:
    """parser.rs:100-205: a directive is a keyword followed by positional
    arguments (numbers, strings, [number arrays]) and `"type name" value`
    parameters, up to the next keyword."""
    out, k = [], 0
    while k < len(toks):
        head = toks[k]
        if head.kind != "ident":
            raise ParseError(f"line {head.line}: expected directive keyword, found {head.kind}")
        d = Directive(head.value, head.line)
        k += 1
        while k < len(toks):
            t = toks[k]
            if t.kind == "ident":
                break
            if t.kind == "string" and " " in t.value:
                parts = t.value.split(None, 1)
                if len(parts) != 2 or not parts[0].strip() or not parts[1].strip():
                    raise ParseError(f"line {t.line}: parameter header {t.value!r} must have form \"<type> <name>\"")
                type_name, name = parts[0].strip(), parts[1].strip()
                kind, vals, k = _param_values(toks, k + 1, t)
                if type_name in FLOAT_TYPES and kind == "ints":
                    kind, vals = "floats", [float(v) for v in vals]
                d.params.append(Param(type_name, name, kind, vals, t.line))
            elif t.kind == "string":
                d.positional.append(t.value)
                k += 1
            elif t.kind in ("int", "float"):
                d.positional.append(float(t.value))
                k += 1
            elif t.kind == "[":
                k += 1
                arr = []
                while True:
                    if k >= len(toks):
                        raise ParseError(f"line {toks[-1].line}: unexpected end of input")
                    u = toks[k]
                    if u.kind == "]":
                        k += 1
                        break
                    if u.kind not in ("int", "float"):
                        raise ParseError(f"line {u.line}: expected number or `]`, found {u.kind}")
                    arr.append(float(u.value))
                    k += 1
                d.positional.append(arr)
            else:
                raise ParseError(f"line {t.line}: expected directive arg, found `]`")
        out.append(d)
    return out


# ---------------------------------------------------------------- builder --
@dataclass
class CameraSettings:
    origin: np.ndarray
    target: np.ndarray
    up: np.ndarray
    vfov_deg: float


@dataclass
class FilmSettings:
    width: int
    height: int
    filename: str | None


@dataclass
class LoadedPbrt:
    scene: Scene
    camera: CameraSettings | None
    film: FilmSettings | None


def _mat_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """4x4 float32 product a * b (column-vector convention), each entry a
    left-to-right sum over k."""
    out = np.zeros((4, 4), F32)
    for i in range(4):
        for j in range(4):
            acc = F32(a[i, 0] * b[0, j])
            for k in range(1, 4):
                acc = F32(acc + F32(a[i, k] * b[k, j]))
            out[i, j] = acc
    return out


def _translation(v) -> np.ndarray:
    m = np.eye(4, dtype=F32)
    m[:3, 3] = v
    return m


def _scale(v) -> np.ndarray:
    return np.diag(np.array([v[0], v[1], v[2], 1.0], F32))


def _rotation(angle_deg: float, axis) -> np.ndarray:
    """Mat4::from_quat(Quat::from_axis_angle(axis.normalize(), radians))."""
    a = np.asarray(axis, F32)
    inv_len = F32(1.0) / F32(np.sqrt(F32(F32(a[0] * a[0]) + F32(a[1] * a[1])) + F32(a[2] * a[2])))
    a = (a * inv_len).astype(F32)
    ang = F32(F32(angle_deg) * F32(math.pi / 180.0))
    s, c = F32(math.sin(float(ang * F32(0.5)))), F32(math.cos(float(ang * F32(0.5))))
    x, y, z, w = a[0] * s, a[1] * s, a[2] * s, c
    x2, y2, z2 = x + x, y + y, z + z
    xx, xy, xz = x * x2, x * y2, x * z2
    yy, yz, zz = y * y2, y * z2, z * z2
    wx, wy, wz = w * x2, w * y2, w * z2
    m = np.eye(4, dtype=F32)
    m[:3, 0] = [F32(1.0) - (yy + zz), xy + wz, xz - wy]
    m[:3, 1] = [xy - wz, F32(1.0) - (xx + zz), yz + wx]
    m[:3, 2] = [xz + wy, yz - wx, F32(1.0) - (xx + yy)]
    return m


def _xform_points(m: np.ndarray, p: np.ndarray) -> np.ndarray:
    p = p.astype(F32)
    return (((m[:3, 0] * p[:, :1]).astype(F32) + (m[:3, 1] * p[:, 1:2]).astype(F32)).astype(F32)
            + (m[:3, 2] * p[:, 2:3]).astype(F32) + m[:3, 3]).astype(F32)


def _xform_vectors(m: np.ndarray, v: np.ndarray) -> np.ndarray:
    v = v.astype(F32)
    return (((m[:3, 0] * v[:, :1]).astype(F32) + (m[:3, 1] * v[:, 1:2]).astype(F32)).astype(F32)
            + (m[:3, 2] * v[:, 2:3]).astype(F32)).astype(F32)


def _normalize_rows(v: np.ndarray) -> np.ndarray:
    n2 = ((v[:, 0] * v[:, 0]).astype(F32) + (v[:, 1] * v[:, 1]).astype(F32)).astype(F32) + (v[:, 2] * v[:, 2])
    with np.errstate(divide="ignore", invalid="ignore"):
        return (v * (F32(1.0) / np.sqrt(n2.astype(F32)))[:, None]).astype(F32)


def _floats(p: Param | None):
    return p.values if p is not None and p.kind == "floats" else None


def _param_rgb(d: Directive, name: str):
    v = _floats(d.param(name))
    if v is None:
        return None
    if len(v) >= 3:
        return np.array(v[:3], F32)
    if len(v) == 1:
        return np.full(3, v[0], F32)
    return None


def _param_float(d: Directive, name: str):
    p = d.param(name)
    if p is None or p.kind not in ("floats", "ints") or not p.values:
        return None
    return float(F32(p.values[0]))


def _param_int(d: Directive, name: str):
    p = d.param(name)
    if p is None or p.kind not in ("floats", "ints") or not p.values:
        return None
    return int(p.values[0])


def _param_string(d: Directive, name: str):
    p = d.param(name)
    return p.values[0] if p is not None and p.kind == "strings" and p.values else None


def _expect_floats(d: Directive, n: int) -> list:
    f = [float(F32(a)) for a in d.positional if isinstance(a, float)]
    if len(f) < n:
        raise BuildError(f"malformed {d.keyword} on line {d.line}: expected {n} float positionals, got {len(f)}")
    return f


def _expect_string(d: Directive) -> str:
    for a in d.positional:
        if isinstance(a, str):
            return a
    raise BuildError(f"malformed {d.keyword} on line {d.line}: expected a positional string (type name)")


def _material(kind: str, d: Directive):
    """builder.rs:303-356."""
    if kind == "matte":
        kd = _param_rgb(d, "Kd")
        return Lambertian(kd if kd is not None else np.full(3, 0.5, F32))
    if kind == "plastic":
        kd = _param_rgb(d, "Kd")
        ks = _param_rgb(d, "Ks")
        kd = kd if kd is not None else np.full(3, 0.5, F32)
        ks = ks if ks is not None else np.full(3, 0.5, F32)
        rough = _param_float(d, "roughness")
        return DisneyBsdf(kd, 0.0, 0.2 if rough is None else rough,
                          float(F32(F32(F32(ks[0] + ks[1]) + ks[2]) / F32(3.0))))
    if kind in ("metal", "conductor"):
        base = _param_rgb(d, "Kr")
        if base is None:
            base = _param_rgb(d, "reflectance")
        if base is None:
            base = np.array([1.0, 0.766, 0.336], F32)
        rough = _param_float(d, "roughness")
        return DisneyBsdf(base, 1.0, 0.1 if rough is None else rough, 0.5)
    warnings.warn(f"PBRT material {kind!r} not supported; falling back to matte gray")
    return Lambertian(np.full(3, 0.5, F32))


def uv_sphere_mesh(radius: float, u_segments: int, v_segments: int, ctm: np.ndarray) -> TriangleMesh:
    """builder.rs:520-555: (u+1)(v+1) vertices, poles duplicated, world space."""
    pos, nor = [], []
    for v in range(v_segments + 1):
        phi = F32(F32(math.pi) * F32(v) / F32(v_segments))
        sp, cp = F32(math.sin(phi)), F32(math.cos(phi))
        for u in range(u_segments + 1):
            th = F32(F32(2.0 * math.pi) * F32(u) / F32(u_segments))
            n = np.array([sp * F32(math.cos(th)), cp, sp * F32(math.sin(th))], F32)
            nor.append(n)
            pos.append((F32(radius) * n).astype(F32))
    pos = _xform_points(ctm, np.array(pos, F32))
    nor = _normalize_rows(_xform_vectors(ctm, np.array(nor, F32)))
    row = u_segments + 1
    idx = []
    for v in range(v_segments):
        for u in range(u_segments):
            i00, i01 = v * row + u, v * row + u + 1
            i10, i11 = (v + 1) * row + u, (v + 1) * row + u + 1
            idx += [i00, i10, i11, i00, i11, i01]
    return TriangleMesh(pos, np.array(idx, np.uint32), nor)


def build(directives: list[Directive], base_dir: Path = Path(".")) -> LoadedPbrt:
    """builder.rs:69-296: walks the directives with a transform stack and an
    attribute stack (CTM, current material, pending area light)."""
    scene = Scene()
    named: dict[str, int] = {}
    cur = {"ctm": np.eye(4, dtype=F32), "material": None, "area": None}
    attr_stack, xf_stack = [], []
    lookat, vfov, film = None, None, None
    in_world = False

    def default_material() -> int:
        scene.materials.append(Lambertian(np.full(3, 0.5, F32)))
        return len(scene.materials) - 1

    for d in directives:
        kw = d.keyword
        if kw == "LookAt":
            f = _expect_floats(d, 9)
            lookat = (np.array(f[0:3], F32), np.array(f[3:6], F32), np.array(f[6:9], F32))
        elif kw == "Camera":
            if _expect_string(d) != "perspective":
                warnings.warn('only "perspective" Camera supported; ignoring others')
            vfov = _param_float(d, "fov")
        elif kw == "Film":
            w, h = _param_int(d, "xresolution"), _param_int(d, "yresolution")
            film = FilmSettings(800 if w is None else w, 600 if h is None else h, _param_string(d, "filename"))
        elif kw in ("Sampler", "Integrator", "Accelerator", "PixelFilter"):
            pass
        elif kw == "Identity":
            cur["ctm"] = np.eye(4, dtype=F32)
        elif kw == "Translate":
            cur["ctm"] = _mat_mul(cur["ctm"], _translation(_expect_floats(d, 3)[:3]))
        elif kw == "Scale":
            cur["ctm"] = _mat_mul(cur["ctm"], _scale(_expect_floats(d, 3)[:3]))
        elif kw == "Rotate":
            f = _expect_floats(d, 4)
            cur["ctm"] = _mat_mul(cur["ctm"], _rotation(f[0], f[1:4]))
        elif kw in ("Transform", "ConcatTransform"):
            arr = d.positional[0] if d.positional else None
            if not isinstance(arr, list) or len(arr) != 16:
                raise BuildError(f"malformed {kw} on line {d.line}: expected a 16-float array")
            m = np.array(arr, F32).reshape(4, 4).T  # 16 values, column by column
            cur["ctm"] = m if kw == "Transform" else _mat_mul(cur["ctm"], m)
        elif kw == "AttributeBegin":
            attr_stack.append(dict(cur))
        elif kw == "AttributeEnd":
            if not attr_stack:
                raise BuildError(f"AttributeEnd without matching AttributeBegin (line {d.line})")
            cur = attr_stack.pop()
        elif kw == "TransformBegin":
            xf_stack.append(cur["ctm"])
        elif kw == "TransformEnd":
            if not xf_stack:
                raise BuildError(f"TransformEnd without matching TransformBegin (line {d.line})")
            cur["ctm"] = xf_stack.pop()
        elif kw == "WorldBegin":
            in_world = True
            cur["ctm"] = np.eye(4, dtype=F32)
        elif kw == "WorldEnd":
            in_world = False
        elif kw == "Material":
            scene.materials.append(_material(_expect_string(d), d))
            cur["material"] = len(scene.materials) - 1
        elif kw == "MakeNamedMaterial":
            name = _expect_string(d)
            kind = _param_string(d, "type") or "matte"
            scene.materials.append(_material(kind, d))
            named[name] = len(scene.materials) - 1
        elif kw == "NamedMaterial":
            name = _expect_string(d)
            if name not in named:
                raise BuildError(f"named material {name!r} not declared")
            cur["material"] = named[name]
        elif kw == "AreaLightSource":
            if _expect_string(d) != "diffuse":
                warnings.warn('only "diffuse" area lights supported')
            L = _param_rgb(d, "L")
            cur["area"] = L if L is not None else np.ones(3, F32)
        elif kw == "LightSource":
            kind = _expect_string(d)
            if not in_world:
                warnings.warn(f"LightSource {kind!r} outside WorldBegin; placed anyway")
            if kind == "infinite":
                scale = _param_float(d, "scale")
                intensity = 1.0 if scale is None else scale
                mapname = _param_string(d, "mapname")
                if mapname is not None:
                    from .hdr import load_hdri
                    scene.env = load_hdri(Path(base_dir) / mapname, intensity)
                else:
                    L = _param_rgb(d, "L")
                    scene.env = HdriEnvironmentLight.constant(L if L is not None else np.ones(3, F32), intensity)
            else:
                warnings.warn(f"PBRT LightSource {kind!r} not supported; skipping")
        elif kw == "Shape":
            if not in_world:
                warnings.warn("Shape outside WorldBegin; ignoring")
                continue
            _add_shape(_expect_string(d), d, cur, scene, default_material)
        elif kw in ("Texture", "ObjectBegin", "ObjectEnd", "ObjectInstance", "Include", "ReverseOrientation",
                    "ActiveTransform", "CoordinateSystem", "CoordSysTransform", "MediumInterface",
                    "MakeNamedMedium"):
            warnings.warn(f"PBRT directive {kw} (line {d.line}) parsed but not implemented; skipping")
        else:
            warnings.warn(f"unknown PBRT directive {kw}; skipping")

    camera = None
    if lookat is not None and vfov is not None:
        camera = CameraSettings(lookat[0], lookat[1], lookat[2], vfov)
    return LoadedPbrt(scene, camera, film)


def _add_shape(kind: str, d: Directive, cur: dict, scene: Scene, default_material) -> None:
    """builder.rs:394-506."""
    if kind == "sphere":
        r = _param_float(d, "radius")
        mesh = uv_sphere_mesh(1.0 if r is None else r, 48, 24, cur["ctm"])
        if cur["area"] is not None:
            warnings.warn("AreaLightSource attached to a non-quad shape; emission ignored")
        mat = cur["material"] if cur["material"] is not None else default_material()
        scene.primitives.append(Primitive(MeshInstance.build(mesh), mat))
        return
    if kind != "trianglemesh":
        warnings.warn(f"PBRT Shape {kind!r} not supported; skipping")
        return
    P = _floats(d.param("P"))
    if P is None:
        raise BuildError('Shape "trianglemesh" requires parameter "P"')
    ip = d.param("indices")
    if ip is None or ip.kind != "ints":
        raise BuildError('Shape "trianglemesh" requires parameter "indices"')
    if len(P) % 3:
        raise BuildError(f"malformed trianglemesh on line {d.line}: P length not a multiple of 3")
    if len(ip.values) % 3:
        raise BuildError(f"malformed trianglemesh on line {d.line}: indices length not a multiple of 3")
    pos = _xform_points(cur["ctm"], np.array(P, F32).reshape(-1, 3))
    idx = np.array([v & 0xFFFFFFFF for v in ip.values], np.uint32)
    Nn = _floats(d.param("N"))
    nor = None
    if Nn is not None:
        nor = _normalize_rows(_xform_vectors(cur["ctm"], np.array(Nn, F32).reshape(-1, 3)))
    if cur["area"] is not None:
        if pos.shape[0] == 4 and idx.size == 6:
            scene.lights.append(DiffuseAreaQuadLight(pos[0], (pos[1] - pos[0]).astype(F32),
                                                     (pos[3] - pos[0]).astype(F32), cur["area"]))
            return
        warnings.warn(f"line {d.line}: AreaLightSource attached to non-quad trianglemesh; skipping emission")
    mat = cur["material"]
    if mat is None:
        warnings.warn(f"line {d.line}: Shape with no current Material; using gray")
        mat = default_material()
    scene.primitives.append(Primitive(MeshInstance.build(TriangleMesh(pos, idx, nor)), mat))


def load_pbrt(path) -> LoadedPbrt:
    """io/pbrt/mod.rs:63-76: read, tokenize, parse, build (relative map names
    resolve against the file's directory)."""
    path = Path(path)
    try:
        src = path.read_text()
    except OSError as e:
        raise PbrtError(f"io: {e}") from e
    return build(parse(tokenize(src)), path.parent)
