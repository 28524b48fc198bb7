"""Image I/O for the per-pixel pipeline, without OpenCV or Pillow.

The reference reads and writes its maps and photos with cv2 (src/imageio.py:11-76). Neither
cv2 nor Pillow is available here, so this module carries its own PNG codec (zlib + the
five PNG row filters, 8- and 16-bit grey/grey-alpha/RGB/RGBA, non-interlaced) and keeps the
reference's flag semantics:

* ``imread(path, flag, dim)``: float32 in [0, 1] (uint8 / 255, uint16 / 65535); "srgb" ->
  RGB (H, W, 3); "rough" -> mean of RGB or the grey plane (H, W); "normal" -> RGB*2-1
  normalised per pixel (src/imageio.py:11-51). ``dim`` = (width, height) resizes first.
* ``imwrite(im, path, flag)``: "srgb"/"rough" clip to [0, 1]; "normal" maps [-1, 1] to
  [0, 1]; stored as 8-bit (src/imageio.py:54-72).
* ``imresize``: separable Lanczos (a = 4, an 8x8 footprint, the kernel cv2's INTER_LANCZOS4
  names), computed with torch on any device. cv2 itself is absent, so its border and
  rounding details are not reproduced bit for bit.
"""
from __future__ import annotations

import math
import pathlib
import struct
import zlib

import numpy as np
import torch

_SIG = b"\x89PNG\r\n\x1a\n"
_CHANNELS = {0: 1, 2: 3, 4: 2, 6: 4}


def _chunks(data: bytes):
    pos = 8
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        kind = data[pos + 4:pos + 8]
        yield kind, data[pos + 8:pos + 8 + n]
        pos += 12 + n


def _unfilter(raw: np.ndarray, h: int, stride: int, bpp: int) -> np.ndarray:
    out = np.zeros((h, stride), dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int32)
    rows = raw.reshape(h, stride + 1)
    for y in range(h):
        ft = int(rows[y, 0])
        line = rows[y, 1:].astype(np.int32)
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 0xFF
        elif ft == 1 and stride % bpp == 0:
            # Sub: a running sum along each of the bpp interleaved byte lanes
            cur = (np.cumsum(line.reshape(-1, bpp), axis=0) & 0xFF).reshape(-1)
        elif ft in (1, 3, 4):
            cur = line.copy()
            # sequential dependency along the row, but only every bpp-th byte depends on
            # the one bpp bytes earlier: process bpp interleaved lanes together
            for x in range(0, stride, bpp):
                a = cur[x - bpp:x] if x >= bpp else np.zeros(bpp, np.int32)
                b = prev[x:x + bpp]
                if ft == 1:
                    pred = a
                elif ft == 3:
                    pred = (a + b) >> 1
                else:
                    c = prev[x - bpp:x] if x >= bpp else np.zeros(bpp, np.int32)
                    p = a + b - c
                    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
                    pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
                cur[x:x + bpp] = (cur[x:x + bpp] + pred) & 0xFF
        else:
            raise ValueError(f"bad PNG filter type {ft}")
        out[y] = cur.astype(np.uint8)
        prev = cur
    return out


def png_read(path) -> np.ndarray:
    """Decode a PNG to (H, W) or (H, W, C) uint8/uint16, channels in file order (RGB[A])."""
    data = pathlib.Path(path).read_bytes()
    if data[:8] != _SIG:
        raise ValueError(f"{path}: not a PNG")
    ihdr, idat = None, []
    for kind, body in _chunks(data):
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if ihdr is None:
        raise ValueError(f"{path}: no IHDR")
    w, h, depth, ctype, _, _, interlace = ihdr
    if ctype not in _CHANNELS or depth not in (8, 16) or interlace:
        raise ValueError(f"{path}: unsupported PNG (colour type {ctype}, depth {depth}, interlace {interlace})")
    ch = _CHANNELS[ctype]
    bpp = ch * depth // 8
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), dtype=np.uint8)
    px = _unfilter(raw, h, w * bpp, bpp)
    if depth == 16:
        px = px.reshape(h, w * ch, 2)
        arr = (px[..., 0].astype(np.uint16) << 8) | px[..., 1].astype(np.uint16)
    else:
        arr = px
    arr = arr.reshape(h, w, ch)
    return arr[..., 0] if ch == 1 else arr


def png_write(path, arr: np.ndarray) -> None:
    """Encode (H, W) or (H, W, 1|2|3|4) uint8 or uint16 as PNG (filter 0)."""
    a = np.asarray(arr)
    if a.dtype not in (np.uint8, np.uint16):
        raise ValueError("png_write needs uint8 or uint16")
    if a.ndim == 2:
        a = a[..., None]
    h, w, ch = a.shape
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}[ch]
    depth = 16 if a.dtype == np.uint16 else 8
    if depth == 16:
        rowbytes = a.astype(">u2").tobytes()
    else:
        rowbytes = a.tobytes()
    stride = w * ch * depth // 8
    raw = b"".join(b"\x00" + rowbytes[y * stride:(y + 1) * stride] for y in range(h))

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    out = _SIG + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    out += chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b"")
    pathlib.Path(path).write_bytes(out)


def _lanczos_matrix(n_in: int, n_out: int, a: int = 4) -> torch.Tensor:
    """(n_out, n_in) resampling matrix: centre-aligned, 2a taps, normalised, edge-clamped."""
    scale = n_in / n_out
    m = torch.zeros(n_out, n_in, dtype=torch.float64)
    for o in range(n_out):
        x = (o + 0.5) * scale - 0.5
        x0 = math.floor(x)
        taps = range(x0 - a + 1, x0 + a + 1)
        ws = []
        for t in taps:
            d = x - t
            w = 1.0 if abs(d) < 1e-12 else (a * math.sin(math.pi * d) * math.sin(math.pi * d / a)) / (math.pi * math.pi * d * d)
            ws.append(w)
        s = sum(ws)
        for t, w in zip(taps, ws):
            m[o, min(max(t, 0), n_in - 1)] += w / s
    return m


def imresize(im, dim, device=None):
    """Lanczos-resize an (H, W[, C]) array to dim = (width, height), like cv2.resize(...,
    INTER_LANCZOS4) (src/imageio.py:75-76). Works on numpy arrays or torch tensors."""
    w_out, h_out = int(dim[0]), int(dim[1])
    t = torch.as_tensor(np.asarray(im) if not torch.is_tensor(im) else im, dtype=torch.float32)
    if device is not None:
        t = t.to(device)
    h, w = t.shape[:2]
    if (h, w) == (h_out, w_out):
        return im
    my = _lanczos_matrix(h, h_out).to(t.device, torch.float32)
    mx = _lanczos_matrix(w, w_out).to(t.device, torch.float32)
    flat = t.reshape(h, w, -1)
    r = torch.einsum("oh,hwc->owc", my, flat)
    r = torch.einsum("pw,owc->opc", mx, r)
    r = r.reshape(h_out, w_out, *t.shape[2:])
    return r if torch.is_tensor(im) else r.cpu().numpy()


def imread(filename, flag=None, dim=None) -> np.ndarray:
    """src/imageio.py:11-51 without cv2: returns float32, RGB order."""
    im = png_read(filename)
    scale = 65535.0 if im.dtype == np.uint16 else 255.0
    im = im.astype(np.float32) / np.float32(scale)
    if dim is not None:
        im = imresize(im, dim).astype(np.float32)
    if flag == "srgb":
        if im.ndim != 3 or im.shape[2] < 3:
            raise ValueError(f"{filename} should be a 3 channel image")
        im = im[:, :, :3]
    elif flag == "rough":
        if im.ndim == 3 and im.shape[2] >= 3:
            im = im[:, :, :3].mean(axis=2)
        elif im.ndim != 2:
            raise ValueError(f"{filename} should be a 3 or 1 channel image")
    elif flag == "normal":
        if im.ndim != 3 or im.shape[2] < 3:
            raise ValueError(f"{filename} should be a 3 channel image")
        im = im[:, :, :3] * 2 - 1
        im = im / np.linalg.norm(im, axis=2, keepdims=True)
    return im.astype(np.float32)


def imwrite(im, filename, flag=None, dim=None) -> None:
    """src/imageio.py:54-72 without cv2: 8-bit PNG, RGB order."""
    im = np.asarray(im, dtype=np.float32)
    if dim is not None:
        im = imresize(im, dim)
    if flag in ("srgb", "rough"):
        im = im.clip(0, 1)
    elif flag == "normal":
        im = (im.clip(-1, 1) + 1) / 2
    png_write(filename, (im * 255).astype(np.uint8))
