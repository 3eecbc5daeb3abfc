"""glTF 2.0 meshes (crates/pyre/src/io/gltf.rs:20-92).

load_gltf(path) -> list[TriangleMesh]: walks the default scene's node
hierarchy (or the first scene), accumulating node transforms, and emits one
mesh per primitive with positions and normals baked into world space.
Normals use the inverse transpose of the upper 3x3 and normalize_or_zero;
TEXCOORD_0 is kept as uvs; a primitive without indices uses 0..n-1. Only
mode 4 (TRIANGLES) is accepted, as in the reference. The reference reads
files through the `gltf` crate (Cargo.lock: gltf 1.4); this restates the
published glTF 2.0 container format: `.gltf` JSON with external or `data:`
URI buffers, and `.glb` binary (a JSON chunk then a BIN chunk).
"""
from __future__ import annotations

import base64
import json
import struct
from pathlib import Path

import numpy as np

from ..scene import TriangleMesh

F32 = np.float32


class GltfError(Exception):
    pass


_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}


def _read_document(path: Path):
    data = path.read_bytes()
    if data[:4] == b"glTF":
        version, length = struct.unpack_from("<II", data, 4)
        if version != 2:
            raise GltfError(f"unsupported glb version {version}")
        pos, doc, bin_chunk = 12, None, None
        while pos + 8 <= min(length, len(data)):
            clen, ctype = struct.unpack_from("<II", data, pos)
            chunk = data[pos + 8:pos + 8 + clen]
            if ctype == 0x4E4F534A:
                doc = json.loads(chunk.decode("utf-8"))
            elif ctype == 0x004E4942 and bin_chunk is None:
                bin_chunk = chunk
            pos += 8 + clen
        if doc is None:
            raise GltfError("glb without a JSON chunk")
    else:
        doc, bin_chunk = json.loads(data.decode("utf-8")), None
    buffers = []
    for k, b in enumerate(doc.get("buffers", [])):
        uri = b.get("uri")
        if uri is None:
            if bin_chunk is None:
                raise GltfError(f"buffer {k} has no uri and the file has no BIN chunk")
            buffers.append(bin_chunk)
        elif uri.startswith("data:"):
            buffers.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            buffers.append((path.parent / uri).read_bytes())
    return doc, buffers


def _accessor(doc, buffers, index: int, as_float: bool = False) -> np.ndarray:
    acc = doc["accessors"][index]
    if "sparse" in acc:
        raise GltfError("sparse accessors are not supported")
    dtype = np.dtype(_COMPONENT[acc["componentType"]]).newbyteorder("<")
    nc = _NCOMP[acc["type"]]
    count = acc["count"]
    if "bufferView" not in acc:
        arr = np.zeros((count, nc), dtype)
    else:
        view = doc["bufferViews"][acc["bufferView"]]
        buf = buffers[view["buffer"]]
        base = view.get("byteOffset", 0) + acc.get("byteOffset", 0)
        elem = dtype.itemsize * nc
        stride = view.get("byteStride", elem) or elem
        if count and base + (count - 1) * stride + elem > len(buf):
            raise GltfError(f"accessor {index} reads past its buffer")
        raw = np.frombuffer(buf, np.uint8, count=(count - 1) * stride + elem if count else 0, offset=base)
        rows = np.lib.stride_tricks.as_strided(raw, (count, elem), (stride, 1)) if count else np.zeros((0, elem),
                                                                                                     np.uint8)
        arr = np.ascontiguousarray(rows).view(dtype).reshape(count, nc)
    if as_float and arr.dtype != np.float32:
        if acc.get("normalized"):
            info = np.iinfo(arr.dtype)
            arr = np.maximum(arr.astype(F32) / F32(info.max), F32(-1.0))
        else:
            arr = arr.astype(F32)
    return arr


def _quat_matrix(q) -> np.ndarray:
    x, y, z, w = (F32(v) for v in q)
    m = np.eye(4, dtype=F32)
    m[:3, 0] = [F32(1) - F32(2) * (y * y + z * z), F32(2) * (x * y + w * z), F32(2) * (x * z - w * y)]
    m[:3, 1] = [F32(2) * (x * y - w * z), F32(1) - F32(2) * (x * x + z * z), F32(2) * (y * z + w * x)]
    m[:3, 2] = [F32(2) * (x * z + w * y), F32(2) * (y * z - w * x), F32(1) - F32(2) * (x * x + y * y)]
    return m


def node_matrix(node: dict) -> np.ndarray:
    """The node's local transform: `matrix` (16 values, column-major) or T * R * S."""
    if "matrix" in node:
        return np.array(node["matrix"], F32).reshape(4, 4).T
    t = np.eye(4, dtype=F32)
    t[:3, 3] = node.get("translation", [0.0, 0.0, 0.0])
    s = np.diag(np.array(list(node.get("scale", [1.0, 1.0, 1.0])) + [1.0], F32))
    r = _quat_matrix(node.get("rotation", [0.0, 0.0, 0.0, 1.0]))
    return (t @ r @ s).astype(F32)


def _primitive_mesh(doc, buffers, prim: dict, xform: np.ndarray) -> TriangleMesh:
    if prim.get("mode", 4) != 4:
        raise GltfError(f"non-triangle primitive (mode: {prim.get('mode')}); only Triangles is supported")
    attrs = prim.get("attributes", {})
    if "POSITION" not in attrs:
        raise GltfError("primitive has no positions attribute")
    p = _accessor(doc, buffers, attrs["POSITION"], as_float=True)[:, :3]
    pos = (p @ xform[:3, :3].T + xform[:3, 3]).astype(F32)
    if "indices" in prim:
        idx = _accessor(doc, buffers, prim["indices"]).reshape(-1).astype(np.uint32)
    else:
        idx = np.arange(pos.shape[0], dtype=np.uint32)
    normals = None
    if "NORMAL" in attrs:
        nx = np.linalg.inv(xform[:3, :3].astype(np.float64)).T.astype(F32)
        n = (_accessor(doc, buffers, attrs["NORMAL"], as_float=True)[:, :3] @ nx.T).astype(F32)
        ln = np.sqrt((n * n).sum(axis=1))
        with np.errstate(divide="ignore", invalid="ignore"):
            normals = np.where(ln[:, None] > 0, n / ln[:, None], F32(0.0)).astype(F32)
    uvs = _accessor(doc, buffers, attrs["TEXCOORD_0"], as_float=True)[:, :2] if "TEXCOORD_0" in attrs else None
    return TriangleMesh(pos, idx, normals, uvs)


def load_gltf(path) -> list[TriangleMesh]:
    path = Path(path)
    try:
        doc, buffers = _read_document(path)
    except (OSError, ValueError, KeyError) as e:
        raise GltfError(str(e)) from e
    scenes = doc.get("scenes", [])
    if not scenes:
        return []
    scene = scenes[doc.get("scene", 0)]
    nodes = doc.get("nodes", [])
    out: list[TriangleMesh] = []

    def walk(k: int, parent: np.ndarray) -> None:
        node = nodes[k]
        xform = (parent @ node_matrix(node)).astype(F32)
        if "mesh" in node:
            for prim in doc["meshes"][node["mesh"]]["primitives"]:
                out.append(_primitive_mesh(doc, buffers, prim, xform))
        for c in node.get("children", []):
            walk(c, xform)

    for k in scene.get("nodes", []):
        walk(k, np.eye(4, dtype=F32))
    return out
