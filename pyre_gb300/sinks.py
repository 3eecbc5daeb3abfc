"""Film sinks: PNG and OpenEXR files with the reference CLI's conventions
(crates/pyre/src/film.rs:117-264).

save_png         beauty, clamp to [0, 1], x^(1/2.2), * 255, truncated to u8
save_aov_pngs    <stem>.albedo.png (as beauty), <stem>.normal.png
                 (0.5 * (n + 1), linear), <stem>.depth.png (min-max over hit
                 pixels, near = bright, misses black)
save_exr         one layer, FP32 channels R, G, B and optionally albedo.R/G/B,
                 N.X/Y/Z, Z, sorted by name as OpenEXR requires; linear

PNG is written with zlib from the standard library (8-bit RGB / gray, one
IDAT). EXR is written as scanline blocks of 16 lines with ZIP compression
(the format's byte split + delta predictor + zlib); read_exr reads what
save_exr writes (NO, ZIPS and ZIP scanline compression). The reference
writes its EXR through the `exr` crate with run-length-coded 64 x 64 tiles;
block layout and compression differ, channel names, types and values are
the same.
"""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

F32 = np.float32


# ----------------------------------------------------------------- LDR maps --
def encode_gamma8(rgb: np.ndarray) -> np.ndarray:
    """film.rs:209-224: clamp(0, 1).powf(1 / 2.2) * 255 as u8 (truncation)."""
    x = np.clip(np.asarray(rgb, F32), F32(0.0), F32(1.0))
    return (np.power(x, F32(1.0) / F32(2.2)).astype(F32) * F32(255.0)).astype(np.uint8)


def encode_normal8(n: np.ndarray) -> np.ndarray:
    """film.rs:148-158: (n * 0.5 + 0.5).clamp(0, 1) * 255 as u8."""
    x = np.clip(np.asarray(n, F32) * F32(0.5) + F32(0.5), F32(0.0), F32(1.0))
    return (x * F32(255.0)).astype(np.uint8)


def encode_depth8(depth: np.ndarray) -> np.ndarray:
    """film.rs:161-186: min-max over depth > 0, (1 - (d - lo) / range) * 255,
    misses (depth 0) black."""
    d = np.asarray(depth, F32)
    hit = d > 0
    lo = d[hit].min() if hit.any() else F32(np.inf)
    hi = d[hit].max() if hit.any() else F32(0.0)
    rng = max(F32(hi - lo), F32(1e-6))
    with np.errstate(invalid="ignore"):
        v = np.clip(F32(1.0) - (d - lo) / rng, F32(0.0), F32(1.0))
    return np.where(hit, (v * F32(255.0)).astype(np.uint8), np.uint8(0))


# ---------------------------------------------------------------------- PNG --
def _png_chunk(tag: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def write_png(path, img: np.ndarray) -> None:
    """img: (h, w, 3) or (h, w) uint8."""
    img = np.ascontiguousarray(img, np.uint8)
    h, w = img.shape[:2]
    color = 2 if img.ndim == 3 else 0
    rows = img.reshape(h, -1)
    raw = np.concatenate([np.zeros((h, 1), np.uint8), rows], axis=1).tobytes()  # filter 0 per row
    data = b"\x89PNG\r\n\x1a\n" + _png_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, color, 0, 0, 0))
    data += _png_chunk(b"IDAT", zlib.compress(raw, 6)) + _png_chunk(b"IEND", b"")
    Path(path).write_bytes(data)


def read_png(path) -> np.ndarray:
    """Reads what write_png writes (8-bit, filter 0 rows)."""
    data = Path(path).read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h, color = 8, b"", 0, 0, 2
    while pos < len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h, _, color = struct.unpack(">IIBB", body[:10])
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    ch = 3 if color == 2 else 1
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + w * ch)
    if np.any(raw[:, 0]):
        raise ValueError("only unfiltered rows are supported")
    return raw[:, 1:].reshape((h, w, 3) if ch == 3 else (h, w))


def _film_arrays(film):
    h, w = film.height, film.width
    return (np.asarray(film.radiance, F32).reshape(h, w, 3), np.asarray(film.albedo, F32).reshape(h, w, 3),
            np.asarray(film.normal, F32).reshape(h, w, 3), np.asarray(film.depth, F32).reshape(h, w))


def save_png(film, path) -> None:
    write_png(path, encode_gamma8(_film_arrays(film)[0]))


def save_aov_pngs(film, base_path, albedo=True, normal=True, depth=True) -> list[Path]:
    base = Path(base_path)
    stem = base.stem or "render"
    _, alb, nor, dep = _film_arrays(film)
    out = []
    for on, name, img in ((albedo, "albedo", lambda: encode_gamma8(alb)), (normal, "normal", lambda: encode_normal8(nor)),
                          (depth, "depth", lambda: encode_depth8(dep))):
        if on:
            p = base.parent / f"{stem}.{name}.png"
            write_png(p, img())
            out.append(p)
    return out


# ---------------------------------------------------------------------- EXR --
_NO, _ZIPS, _ZIP = 0, 2, 3
_LINES = {_NO: 1, _ZIPS: 1, _ZIP: 16}


def _attr(name: str, typ: str, data: bytes) -> bytes:
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(data)) + data


def _zip_encode(raw: bytes) -> bytes:
    b = np.frombuffer(raw, np.uint8)
    t = np.concatenate([b[0::2], b[1::2]])
    d = t.copy()
    d[1:] = (t[1:].astype(np.int16) - t[:-1].astype(np.int16) + 128 + 256) % 256
    return zlib.compress(d.tobytes(), 6)


def _zip_decode(comp: bytes, size: int) -> bytes:
    d = np.frombuffer(zlib.decompress(comp), np.uint8).astype(np.int32)
    if d.size != size:
        raise ValueError("zip block size mismatch")
    t = (np.cumsum(np.concatenate([d[:1], d[1:] - 128])) % 256).astype(np.uint8)  # undo the delta predictor
    half = (size + 1) // 2
    out = np.empty(size, np.uint8)
    out[0::2], out[1::2] = t[:half], t[half:]
    return out.tobytes()


def write_exr(path, channels: dict, width: int, height: int, compression: int = _ZIP) -> None:
    """channels: name -> (h, w) float32 plane; written sorted by name."""
    names = sorted(channels)
    chlist = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", 2, 0, 1, 1) for n in names) + b"\0"
    hdr = struct.pack("<ii", 20000630, 2)
    hdr += _attr("channels", "chlist", chlist)
    hdr += _attr("compression", "compression", bytes([compression]))
    box = struct.pack("<iiii", 0, 0, width - 1, height - 1)
    hdr += _attr("dataWindow", "box2i", box) + _attr("displayWindow", "box2i", box)
    hdr += _attr("lineOrder", "lineOrder", b"\0")
    hdr += _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
    hdr += _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
    hdr += _attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) + b"\0"
    lines = _LINES[compression]
    n_blocks = (height + lines - 1) // lines
    planes = [np.ascontiguousarray(channels[n], "<f4").reshape(height, width) for n in names]
    blocks = []
    for b in range(n_blocks):
        y0, y1 = b * lines, min(height, (b + 1) * lines)
        raw = b"".join(p[y].tobytes() for y in range(y0, y1) for p in planes)  # per line: channel after channel
        if compression != _NO:
            comp = _zip_encode(raw)
            raw = comp if len(comp) < len(raw) else raw
        blocks.append(struct.pack("<ii", y0, len(raw)) + raw)
    table_at = len(hdr)
    offs, pos = [], table_at + 8 * n_blocks
    for blk in blocks:
        offs.append(pos)
        pos += len(blk)
    Path(path).write_bytes(hdr + struct.pack(f"<{n_blocks}Q", *offs) + b"".join(blocks))


def read_exr(path) -> dict:
    """Reads single-part scanline FP32 files (NO, ZIPS, ZIP): name -> (h, w)."""
    data = Path(path).read_bytes()
    magic, version = struct.unpack_from("<ii", data, 0)
    if magic != 20000630 or (version & 0xFF) != 2 or version & 0x200:
        raise ValueError("not a single-part scanline OpenEXR file")
    pos, attrs = 8, {}
    while data[pos] != 0:
        e = data.index(b"\0", pos)
        name = data[pos:e].decode()
        e2 = data.index(b"\0", e + 1)
        typ = data[e + 1:e2].decode()
        (size,) = struct.unpack_from("<i", data, e2 + 1)
        attrs[name] = (typ, data[e2 + 5:e2 + 5 + size])
        pos = e2 + 5 + size
    pos += 1
    chl, names, p = attrs["channels"][1], [], 0
    while chl[p] != 0:
        e = chl.index(b"\0", p)
        ptype = struct.unpack_from("<i", chl, e + 1)[0]
        if ptype != 2:
            raise ValueError("only FP32 channels are supported")
        names.append(chl[p:e].decode())
        p = e + 17
    comp = attrs["compression"][1][0]
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    lines = _LINES[comp]
    n_blocks = (h + lines - 1) // lines
    offs = struct.unpack_from(f"<{n_blocks}Q", data, pos)
    planes = {n: np.zeros((h, w), F32) for n in names}
    for off in offs:
        y, size = struct.unpack_from("<ii", data, off)
        body = data[off + 8:off + 8 + size]
        n_lines = min(lines, y1 + 1 - y)
        full = n_lines * len(names) * w * 4
        raw = body if (comp == _NO or size == full) else _zip_decode(body, full)
        arr = np.frombuffer(raw, "<f4").reshape(n_lines, len(names), w)
        for k, n in enumerate(names):
            planes[n][y - y0:y - y0 + n_lines] = arr[:, k]
    return planes


def save_exr(film, path, albedo=True, normal=True, depth=True) -> None:
    rad, alb, nor, dep = _film_arrays(film)
    ch = {"R": rad[..., 0], "G": rad[..., 1], "B": rad[..., 2]}
    if albedo:
        ch.update({"albedo.R": alb[..., 0], "albedo.G": alb[..., 1], "albedo.B": alb[..., 2]})
    if normal:
        ch.update({"N.X": nor[..., 0], "N.Y": nor[..., 1], "N.Z": nor[..., 2]})
    if depth:
        ch["Z"] = dep
    write_exr(path, ch, film.width, film.height)
