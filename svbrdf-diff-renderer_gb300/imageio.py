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


# ---------------------------------------------------------------- OpenEXR (scanline)
# The reference lights its novel-view video with an OpenEXR environment map
# (src/scripts.py:47, fig/ennis.exr, read by Mitsuba). This is a reader and writer of
# single-part scanline OpenEXR files, following the published file layout: magic 20000630,
# version 2, the attribute header (channels, compression, dataWindow, ...), an offset table
# of 64-bit chunk positions, then chunks of (y, size, data) holding per line each channel's
# samples in channel-name order. Supported: HALF and FLOAT channels, compressions NONE,
# ZIPS (one line per chunk) and ZIP (16 lines): zlib over bytes that were delta-coded
# (d[i] = b[i] - b[i-1] + 128) and split into even and odd halves. Tiled, deep, multi-part
# and the other compressions are refused with a clear error.

_EXR_MAGIC = 20000630
_EXR_LINES = {0: 1, 2: 1, 3: 16}  # compression -> scanlines per chunk
_EXR_TYPES = {1: np.float16, 2: np.float32}


def _exr_unpredict(t: np.ndarray) -> np.ndarray:
    """Inverse of the ZIP predictor: b[0] = d[0], b[i] = (b[i-1] + d[i] - 128) mod 256."""
    out = np.empty_like(t)
    if t.size:
        out[0] = t[0]
        out[1:] = (t[0] + np.cumsum(t[1:].astype(np.int64) - 128)) % 256
    return out


def _exr_deinterleave(t: np.ndarray) -> np.ndarray:
    """The predictor's input was bytes 0, 2, 4, ... followed by bytes 1, 3, 5, ..."""
    half = (t.size + 1) // 2
    out = np.empty_like(t)
    out[0::2] = t[:half]
    out[1::2] = t[half:]
    return out


def _exr_decode_zip(data: bytes, raw_size: int) -> bytes:
    if len(data) == raw_size:
        return data
    t = np.frombuffer(zlib.decompress(data), dtype=np.uint8)
    if t.size != raw_size:
        raise ValueError("EXR chunk decompresses to the wrong size")
    return _exr_deinterleave(_exr_unpredict(t)).astype(np.uint8).tobytes()


def _exr_encode_zip(raw: bytes) -> bytes:
    b = np.frombuffer(raw, dtype=np.uint8)
    t = np.concatenate([b[0::2], b[1::2]]).astype(np.int64)
    d = t.copy()
    d[1:] = (t[1:] - t[:-1] + 128) % 256
    z = zlib.compress(d.astype(np.uint8).tobytes(), 6)
    return z if len(z) < len(raw) else raw


def exr_read(path) -> np.ndarray:
    """[H, W, 3] float32 RGB of a scanline OpenEXR file (a single Y channel is repeated)."""
    buf = pathlib.Path(path).read_bytes()
    if len(buf) < 8 or struct.unpack_from("<i", buf, 0)[0] != _EXR_MAGIC:
        raise ValueError(f"{path}: not an OpenEXR file")
    version = struct.unpack_from("<i", buf, 4)[0]
    if version & 0xFF != 2 or version & (0x200 | 0x800 | 0x1000):
        raise ValueError(f"{path}: only single-part scanline OpenEXR files are supported")
    pos, attrs = 8, {}
    while True:
        end = buf.index(b"\0", pos)
        name = buf[pos:end].decode()
        pos = end + 1
        if not name:
            break
        end = buf.index(b"\0", pos)
        typ = buf[pos:end].decode()
        size = struct.unpack_from("<i", buf, end + 1)[0]
        attrs[name] = (typ, buf[end + 5:end + 5 + size])
        pos = end + 5 + size
    chans = []
    raw = attrs["channels"][1]
    q = 0
    while raw[q] != 0:
        end = raw.index(b"\0", q)
        cname = raw[q:end].decode()
        ptype, _, xs, ys = struct.unpack_from("<iB3xii", raw, end + 1)
        if ptype not in _EXR_TYPES or xs != 1 or ys != 1:
            raise ValueError(f"{path}: channel {cname}: only unsubsampled HALF/FLOAT channels are supported")
        chans.append((cname, _EXR_TYPES[ptype]))
        q = end + 1 + 16
    comp = attrs["compression"][1][0]
    if comp not in _EXR_LINES:
        raise ValueError(f"{path}: compression {comp} is not supported (NONE, ZIPS and ZIP are)")
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    lines = _EXR_LINES[comp]
    nchunks = (h + lines - 1) // lines
    offsets = struct.unpack_from(f"<{nchunks}Q", buf, pos)
    line_bytes = sum(np.dtype(t).itemsize for _, t in chans) * w
    planes = {c: np.zeros((h, w), np.float32) for c, _ in chans}
    for off in offsets:
        y, size = struct.unpack_from("<ii", buf, off)
        first = y - y0
        n = min(lines, h - first)
        data = buf[off + 8:off + 8 + size]
        block = data if comp == 0 else _exr_decode_zip(data, n * line_bytes)
        p = 0
        for r in range(n):
            for c, t in chans:
                nb = np.dtype(t).itemsize * w
                planes[c][first + r] = np.frombuffer(block, dtype=np.dtype(t).newbyteorder("<"), count=w, offset=p)
                p += nb
    if all(c in planes for c in "RGB"):
        return np.stack([planes["R"], planes["G"], planes["B"]], -1)
    if "Y" in planes:
        return np.repeat(planes["Y"][..., None], 3, -1)
    raise ValueError(f"{path}: no R, G, B or Y channels")


def exr_write(path, rgb: np.ndarray, half: bool = True, compression: str = "zip") -> None:
    """Write [H, W, 3] RGB as a scanline OpenEXR file (HALF or FLOAT; "none", "zips", "zip")."""
    rgb = np.asarray(rgb, dtype=np.float32)
    h, w = rgb.shape[:2]
    comp = {"none": 0, "zips": 2, "zip": 3}[compression]
    dt = np.float16 if half else np.float32

    def attr(name, typ, value):
        return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(value)) + value

    chl = b"".join(c.encode() + b"\0" + struct.pack("<iB3xii", 1 if half else 2, 0, 1, 1) for c in "BGR") + b"\0"
    header = (struct.pack("<ii", _EXR_MAGIC, 2) + attr("channels", "chlist", chl) +
              attr("compression", "compression", bytes([comp])) +
              attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)) +
              attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)) +
              attr("lineOrder", "lineOrder", bytes([0])) + attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)) +
              attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0)) +
              attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) + b"\0")
    lines = _EXR_LINES[comp]
    chunks = []
    for y in range(0, h, lines):
        block = b"".join(rgb[r, :, ci].astype(dt).astype(np.dtype(dt).newbyteorder("<")).tobytes()
                         for r in range(y, min(h, y + lines)) for ci in (2, 1, 0))
        data = block if comp == 0 else _exr_encode_zip(block)
        chunks.append(struct.pack("<ii", y, len(data)) + data)
    pos = len(header) + 8 * len(chunks)
    offsets = []
    for c in chunks:
        offsets.append(pos)
        pos += len(c)
    pathlib.Path(path).write_bytes(header + struct.pack(f"<{len(offsets)}Q", *offsets) + b"".join(chunks))


# ---------------------------------------------------------------- mosaics and GIFs
def imconcat(im_list, size=(2, 2)):
    """w x h mosaic of equally sized images, row by row (src/imageio.py:79-89)."""
    w, h = size
    rows = [np.concatenate([np.asarray(im_list[i * w + j]) for j in range(w)], 1) for i in range(h)]
    return np.concatenate(rows, 0)


def img9to1(folder, names=None):
    """all.png: the 3 x 3 mosaic of a folder's nine renders (src/imageio.py:92-98);
    ``names`` lists the nine files (default 00.png .. 08.png, as the reference reads)."""
    folder = pathlib.Path(folder)
    names = names or [f"{i:02d}.png" for i in range(9)]
    imwrite(imconcat([imread(folder / n) for n in names], (3, 3)), folder / "all.png")


def tex4to1(folder):
    """tex.png: the 2 x 2 mosaic normal | diffuse / specular | roughness (src/imageio.py:101-111)."""
    folder = pathlib.Path(folder)
    normal, diffuse = imread(folder / "nom.png"), imread(folder / "dif.png")
    specular, roughness = imread(folder / "spe.png"), imread(folder / "rgh.png")
    if roughness.ndim == 2:
        roughness = np.dstack((roughness, roughness, roughness))
    imwrite(imconcat([normal, diffuse, specular, roughness]), folder / "tex.png")


def _gif_palette() -> np.ndarray:
    """3-3-2 palette: index = r3 << 5 | g3 << 2 | b2, each level spread over 0..255."""
    i = np.arange(256)
    r, g, b = (i >> 5) & 7, (i >> 2) & 7, i & 3
    return np.stack([r * 255 // 7, g * 255 // 7, b * 255 // 3], 1).astype(np.uint8)


def _gif_indices(rgb: np.ndarray) -> np.ndarray:
    q = rgb.astype(np.uint16)
    r = (q[..., 0] * 7 + 127) // 255
    g = (q[..., 1] * 7 + 127) // 255
    b = (q[..., 2] * 3 + 127) // 255
    return ((r << 5) | (g << 2) | b).astype(np.uint8)


def _gif_lzw(indices: np.ndarray) -> bytes:
    """The image data of one frame: minimum code size 8, then 9-bit codes (clear, up to 250
    literals, clear, ...), end code, in sub-blocks of at most 255 bytes. Literal codes and a
    clear before the code table would outgrow 9 bits make a valid, uncompressed LZW stream."""
    px = indices.reshape(-1).astype(np.uint16)
    run = 250
    n = px.size
    groups = (n + run - 1) // run
    codes = np.full(groups * (run + 1), 0xFFFF, np.uint16)
    codes[0::run + 1] = 256  # a clear code before each run
    body = codes.reshape(groups, run + 1)
    padded = np.full(groups * run, 0xFFFF, np.uint16)
    padded[:n] = px
    body[:, 1:] = padded.reshape(groups, run)
    codes = np.concatenate([codes[codes != 0xFFFF], np.array([257], np.uint16)])
    bits = ((codes[:, None] >> np.arange(9)) & 1).astype(np.uint8).reshape(-1)
    data = np.packbits(bits, bitorder="little").tobytes()
    out = bytearray([8])
    for k in range(0, len(data), 255):
        chunk = data[k:k + 255]
        out += bytes([len(chunk)]) + chunk
    out += b"\0"
    return bytes(out)


def gif_write(frames, path, delay_ms: int = 40, loop: int = 0) -> None:
    """Animated GIF89a of RGB frames (uint8, or floats in [0, 1]) with a 3-3-2 palette."""
    frames = [np.asarray(f) for f in frames]
    if not frames:
        raise ValueError("no frames")
    h, w = frames[0].shape[:2]
    out = bytearray(b"GIF89a")
    out += struct.pack("<HHBBB", w, h, 0xF7, 0, 0) + _gif_palette().tobytes()
    out += b"\x21\xff\x0bNETSCAPE2.0\x03\x01" + struct.pack("<H", loop) + b"\0"
    for f in frames:
        if f.dtype == np.uint16:
            f = (f >> 8).astype(np.uint8)
        elif f.dtype != np.uint8:
            f = (np.clip(f, 0, 1) * 255 + 0.5).astype(np.uint8)
        if f.ndim == 2:
            f = np.dstack((f, f, f))
        if f.shape[:2] != (h, w):
            raise ValueError("all frames must have the same size")
        out += b"\x21\xf9\x04\x00" + struct.pack("<H", max(delay_ms // 10, 1)) + b"\x00\x00"
        out += b"\x2c" + struct.pack("<HHHHB", 0, 0, w, h, 0) + _gif_lzw(_gif_indices(f[..., :3]))
    out += b"\x3b"
    pathlib.Path(path).write_bytes(bytes(out))


def img2gif(in_filenames, out_filename, method="Pillow"):
    """GIF of PNG frames, 40 ms each, looping (src/imageio.py:114-123). ``method`` is
    accepted for the reference's signature; the encoder is this module's own either way."""
    gif_write([png_read(f) for f in in_filenames], out_filename, delay_ms=40)
