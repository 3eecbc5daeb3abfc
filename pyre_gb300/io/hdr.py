"""Radiance .hdr (RGBE) environment maps (crates/pyre/src/io/hdr.rs:23-50).

load_hdri(path, intensity) -> HdriEnvironmentLight, for `.hdr` / `.pic`
files; other extensions are rejected as in the reference. The reference
decodes through the `image` crate (Cargo.lock: image 0.25); the decoding
restated here is the published Radiance RGBE format: a text header ending in
an empty line, a `-Y <h> +X <w>` resolution line, then h scanlines stored
flat, with the old run-length scheme, or with the adaptive per-channel RLE
(a line starting 2, 2, w >> 8, w & 255). A pixel (r, g, b, e) decodes to
(r, g, b) * 2^(e - 136), and e = 0 to black.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from ..scene import HdriEnvironmentLight


class HdrLoadError(Exception):
    pass


def rgbe_to_float(rgbe: np.ndarray) -> np.ndarray:
    """(..., 4) uint8 -> (..., 3) float32; mantissa * 2^(e - 136)."""
    e = rgbe[..., 3].astype(np.int32)
    scale = np.where(e == 0, np.float32(0.0), np.ldexp(np.float32(1.0), e - 136).astype(np.float32))
    return (rgbe[..., :3].astype(np.float32) * scale[..., None]).astype(np.float32)


def float_to_rgbe(rgb: np.ndarray) -> np.ndarray:
    """(..., 3) float -> (..., 4) uint8, the usual encoder: shared exponent of
    the largest channel, mantissas floor(c * 256 / 2^e)."""
    rgb = np.asarray(rgb, np.float64)
    m = rgb.max(axis=-1)
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    ok = m > 1e-32
    mant, ex = np.frexp(np.where(ok, m, 1.0))
    f = np.where(ok, mant * 256.0 / np.where(ok, m, 1.0), 0.0)
    out[..., :3] = np.clip(np.floor(rgb * f[..., None]), 0, 255).astype(np.uint8)
    out[..., 3] = np.where(ok, ex + 128, 0).astype(np.uint8)
    return out


def _read_header(data: bytes):
    if not (data.startswith(b"#?RADIANCE") or data.startswith(b"#?RGBE")):
        raise HdrLoadError("decode: missing #?RADIANCE signature")
    pos = data.index(b"\n") + 1
    fmt = None
    while True:
        end = data.find(b"\n", pos)
        if end < 0:
            raise HdrLoadError("decode: header not terminated")
        line = data[pos:end].strip()
        pos = end + 1
        if not line:
            break
        if line.startswith(b"FORMAT="):
            fmt = line[7:].decode("ascii", "replace")
    if fmt not in (None, "32-bit_rle_rgbe"):
        raise HdrLoadError(f"decode: unsupported format {fmt}")
    end = data.find(b"\n", pos)
    parts = data[pos:end].split()
    if len(parts) != 4 or parts[0] != b"-Y" or parts[2] != b"+X":
        raise HdrLoadError("decode: only -Y h +X w images are supported")
    return int(parts[1]), int(parts[3]), end + 1


def _read_scanline(data: bytes, pos: int, w: int, out: np.ndarray) -> int:
    if 8 <= w <= 0x7FFF and data[pos] == 2 and data[pos + 1] == 2 and data[pos + 2] < 128:
        if (data[pos + 2] << 8 | data[pos + 3]) != w:
            raise HdrLoadError("decode: scanline width mismatch")
        pos += 4
        for c in range(4):
            x = 0
            while x < w:
                n = data[pos]
                pos += 1
                if n > 128:
                    n -= 128
                    if x + n > w:
                        raise HdrLoadError("decode: run overflows the scanline")
                    out[x:x + n, c] = data[pos]
                    pos += 1
                else:
                    if n == 0 or x + n > w:
                        raise HdrLoadError("decode: bad literal run")
                    out[x:x + n, c] = np.frombuffer(data, np.uint8, n, pos)
                    pos += n
                x += n
        return pos
    # flat pixels, with the old (1, 1, 1, count) repeat records
    x, shift = 0, 0
    while x < w:
        px = data[pos:pos + 4]
        if len(px) < 4:
            raise HdrLoadError("decode: truncated scanline")
        pos += 4
        if px[0] == 1 and px[1] == 1 and px[2] == 1:
            if x == 0:
                raise HdrLoadError("decode: repeat record at the start of a scanline")
            count = px[3] << shift
            if x + count > w:
                raise HdrLoadError("decode: repeat overflows the scanline")
            out[x:x + count] = out[x - 1]
            x += count
            shift += 8
        else:
            out[x] = np.frombuffer(px, np.uint8)
            x += 1
            shift = 0
    return pos


def decode_hdr(data: bytes) -> tuple[int, int, np.ndarray]:
    """Returns (width, height, (h, w, 3) float32 pixels, row 0 = top)."""
    h, w, pos = _read_header(data)
    rgbe = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        try:
            pos = _read_scanline(data, pos, w, rgbe[y])
        except IndexError:
            raise HdrLoadError("decode: truncated image data") from None
    return w, h, rgbe_to_float(rgbe)


def encode_hdr(pixels: np.ndarray) -> bytes:
    """Writes (h, w, 3) pixels as a Radiance file with adaptive RLE scanlines."""
    h, w, _ = pixels.shape
    rgbe = float_to_rgbe(pixels)
    out = bytearray(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n" + f"-Y {h} +X {w}\n".encode())
    for y in range(h):
        if not 8 <= w <= 0x7FFF:
            out += rgbe[y].tobytes()
            continue
        out += bytes([2, 2, w >> 8, w & 255])
        for c in range(4):
            ch = rgbe[y, :, c]
            x = 0
            while x < w:
                run = 1
                while x + run < w and run < 127 and ch[x + run] == ch[x]:
                    run += 1
                if run >= 3:
                    out += bytes([128 + run, ch[x]])
                    x += run
                    continue
                start = x
                while x < w and x - start < 128:
                    if x + 2 < w and ch[x] == ch[x + 1] == ch[x + 2]:
                        break
                    x += 1
                out += bytes([x - start]) + ch[start:x].tobytes()
    return bytes(out)


def load_hdri(path, intensity: float) -> HdriEnvironmentLight:
    path = Path(path)
    ext = path.suffix.lower().lstrip(".")
    if ext not in ("hdr", "pic"):
        raise HdrLoadError(f"unsupported environment-map extension: {ext}")
    try:
        data = path.read_bytes()
    except OSError as e:
        raise HdrLoadError(f"io: {e}") from e
    w, h, px = decode_hdr(data)
    return HdriEnvironmentLight(w, h, px, intensity)
