"""PNG codec, imread/imwrite flags (src/imageio.py:11-76 semantics), Lanczos resize and
SvbrdfIO (src/svbrdf.py:86-221) on the host."""
import json
import struct
import zlib

import numpy as np
import pytest
import torch


def _encode_filtered(arr, filters):
    """Reference PNG encoder that applies the given filter type per row."""
    h, w, ch = arr.shape
    bpp = ch
    rows = arr.reshape(h, w * ch).astype(np.int32)
    out = []
    prev = np.zeros(w * ch, np.int32)
    for y in range(h):
        ft = filters[y % len(filters)]
        cur = rows[y]
        a = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        c = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        b = prev
        if ft == 0:
            f = cur
        elif ft == 1:
            f = cur - a
        elif ft == 2:
            f = cur - b
        elif ft == 3:
            f = cur - ((a + b) >> 1)
        else:
            p = a + b - c
            pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
            f = cur - np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))
        out.append(bytes([ft]) + (f & 0xFF).astype(np.uint8).tobytes())
        prev = cur
    raw = b"".join(out)

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    ctype = {1: 0, 3: 2, 4: 6}[ch]
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))


@pytest.mark.parametrize("ch", [1, 3, 4])
def test_png_decoder_all_filters(svb, tmp_path, ch):
    rng = np.random.default_rng(ch)
    arr = rng.integers(0, 256, (13, 17, ch), dtype=np.uint8)
    p = tmp_path / "f.png"
    p.write_bytes(_encode_filtered(arr, [0, 1, 2, 3, 4]))
    got = svb.imageio.png_read(p)
    assert np.array_equal(got.reshape(arr.shape), arr)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
def test_png_roundtrip(svb, tmp_path, dtype):
    rng = np.random.default_rng(1)
    arr = rng.integers(0, np.iinfo(dtype).max, (7, 9, 3)).astype(dtype)
    svb.imageio.png_write(tmp_path / "a.png", arr)
    assert np.array_equal(svb.imageio.png_read(tmp_path / "a.png"), arr)


def test_imread_flags(svb, tmp_path):
    io = svb.imageio
    rng = np.random.default_rng(2)
    rgb = rng.integers(0, 256, (8, 8, 3), dtype=np.uint8)
    io.png_write(tmp_path / "c.png", rgb)
    s = io.imread(tmp_path / "c.png", "srgb")
    assert s.dtype == np.float32 and np.allclose(s, rgb / 255.0)
    r = io.imread(tmp_path / "c.png", "rough")
    assert r.shape == (8, 8) and np.allclose(r, (rgb / 255.0).mean(2), atol=1e-6)
    n = io.imread(tmp_path / "c.png", "normal")
    assert np.allclose(np.linalg.norm(n, axis=2), 1.0, atol=1e-5)
    # imwrite normal maps [-1, 1] to 8 bits and back
    nn = np.zeros((4, 4, 3), np.float32)
    nn[..., 2] = 1.0
    io.imwrite(nn, tmp_path / "n.png", "normal")
    back = io.imread(tmp_path / "n.png", "normal")
    assert np.allclose(back[..., 2], 1.0, atol=1e-2)


def test_lanczos_properties(svb):
    io = svb.imageio
    const = np.full((16, 16, 3), 0.25, np.float32)
    up = io.imresize(const, (32, 32))
    assert up.shape == (32, 32, 3) and np.allclose(up, 0.25, atol=1e-6)
    ramp = np.tile(np.linspace(0, 1, 32, dtype=np.float32), (32, 1))
    down = io.imresize(ramp, (16, 16))
    # a linear ramp stays (nearly) linear and keeps its mean
    assert abs(down.mean() - ramp.mean()) < 1e-3
    assert np.all(np.diff(down[8]) > 0)
    assert io.imresize(ramp, (32, 32)) is ramp


def test_svbrdfio_roundtrip(svb, tmp_path):
    cams = [[-3, 3, 16], [0, 3, 16], [3, 3, 16], [-3, 0, 16]]
    cfg = {"reference_dir": "ref", "target_dir": "tgt", "optimize_dir": "opt", "rerender_dir": "rr",
           "im_size": 6.5, "idx": [0, 2, 3], "camera_pos": cams, "light_pos": cams, "light_pow": [1400, 1500, 1600]}
    j = tmp_path / "scene.json"
    j.write_text(json.dumps(cfg))
    io = svb.SvbrdfIO(j, "cpu")
    assert io.n_of_imgs == 3 and io.im_size == 6.5
    assert torch.equal(io.cl[0], torch.tensor([cams[0], cams[2], cams[3]], dtype=torch.float32))
    assert torch.equal(io.cl[2], torch.tensor([1400.0, 1500.0, 1600.0]))
    tex = svb.scenes.make_material(16, 1000)
    io.save_textures_th(tex, io.reference_dir)
    back = io.load_textures_th(io.reference_dir, 16)
    assert back.shape == (1, 9, 16, 16)
    # 8-bit quantisation of [-1, 1] maps: within 2/255 (+ normal renormalisation)
    assert (back[:, [0, 1, 2, 5, 6, 7, 8]] - tex[:, [0, 1, 2, 5, 6, 7, 8]]).abs().max() < 2.5 / 255
    assert (back[:, 3:5] - tex[:, 3:5]).abs().max() < 0.02
    imgs = torch.rand(3, 3, 16, 16)
    io.save_images_th(imgs, io.target_dir)
    got = io.load_images_th(io.target_dir, 16)
    assert (got - imgs).abs().max() <= 1.0 / 255 + 1e-6
    with pytest.raises(FileNotFoundError):
        svb.SvbrdfIO(tmp_path / "missing.json", "cpu")


@pytest.mark.parametrize("half", [True, False])
@pytest.mark.parametrize("compression", ["none", "zips", "zip"])
def test_exr_round_trip(svb, tmp_path, half, compression):
    """Scanline OpenEXR write -> read, 37 lines (ZIP: two full 16-line chunks and a partial one)."""
    IO = svb.imageio
    g = np.random.default_rng(5)
    img = (g.random((37, 23, 3)) * 40.0).astype(np.float32)
    img[0, 0] = [0.0, 1e-3, 65000.0 if half else 1e6]
    p = tmp_path / f"env_{compression}_{half}.exr"
    IO.exr_write(p, img, half=half, compression=compression)
    back = IO.exr_read(p)
    want = img.astype(np.float16).astype(np.float32) if half else img
    assert back.shape == (37, 23, 3) and back.dtype == np.float32
    assert np.array_equal(back, want)  # random values do not compress: those chunks are stored raw
    if compression != "none":
        # a smooth map compresses, and still reads back exactly
        yy, xx = np.mgrid[0:37, 0:23].astype(np.float32)
        smooth = np.stack([xx / 23, yy / 37, (xx + yy) / 60], -1)
        q = tmp_path / "smooth.exr"
        IO.exr_write(q, smooth, half=half, compression=compression)
        assert q.stat().st_size < 37 * 23 * 3 * (2 if half else 4)
        ws = smooth.astype(np.float16).astype(np.float32) if half else smooth
        assert np.array_equal(IO.exr_read(q), ws)


def test_exr_hand_built_file(svb, tmp_path):
    """A file assembled field by field from the published layout (not by exr_write): one
    uncompressed FLOAT line pair with channels B, G, R."""
    import struct

    def attr(name, typ, value):
        return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(value)) + value

    chl = b"".join(c + b"\0" + struct.pack("<iB3xii", 2, 0, 1, 1) for c in (b"B", b"G", b"R")) + b"\0"
    hdr = struct.pack("<ii", 20000630, 2) + attr("channels", "chlist", chl) + attr("compression", "compression", b"\0")
    hdr += attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, 1, 1)) + b"\0"
    rows = []
    for y in range(2):
        vals = {c: [10 * y + x + (0.25 if c == "G" else 0.5 if c == "B" else 0.0) for x in range(2)] for c in "BGR"}
        data = b"".join(struct.pack("<2f", *vals[c]) for c in "BGR")
        rows.append(struct.pack("<ii", y, len(data)) + data)
    start = len(hdr) + 16
    offs = struct.pack("<2Q", start, start + len(rows[0]))
    p = tmp_path / "hand.exr"
    p.write_bytes(hdr + offs + b"".join(rows))
    img = svb.imageio.exr_read(p)
    assert img.shape == (2, 2, 3)
    assert np.allclose(img[1, 0], [10.0, 10.25, 10.5]) and np.allclose(img[0, 1], [1.0, 1.25, 1.5])


def test_exr_rejects_unsupported(svb, tmp_path):
    p = tmp_path / "bad.exr"
    p.write_bytes(b"\x76\x2f\x31\x01" + (2 | 0x200).to_bytes(4, "little"))  # tiled flag
    with pytest.raises(ValueError):
        svb.imageio.exr_read(p)
    p.write_bytes(b"PNG not exr")
    with pytest.raises(ValueError):
        svb.imageio.exr_read(p)


def test_envmap_renderer_reads_exr_path(svb, tmp_path):
    """EnvmapRenderer takes an environment file path, as MitsubaRender takes fig/ennis.exr."""
    env = svb.envmap.synthetic_envmap(8, 16, seed=1)
    p = tmp_path / "sky.exr"
    svb.imageio.exr_write(p, env, half=False)
    r = svb.EnvmapRenderer([16, 16], p, torch.zeros(9, 4, 4), device="cpu")
    assert np.array_equal(r.env_np, env)
    assert r.tables_np[0].shape == (9,)


def test_render_envmap_writes_the_video_frames(svb, tmp_path, monkeypatch):
    """render_envmap (src/scripts.py:44-59): maps read from the folder at their own size,
    116 frames written as vid/000.png .. 115.png. The renderer is replaced by a stand-in here
    (no GPU on this machine); its own kernel is tested on the GPU."""
    g = np.random.default_rng(0)
    svb.imageio.imwrite(g.random((12, 10, 3)), tmp_path / "dif.png", flag="srgb")
    svb.imageio.imwrite(g.random((12, 10, 3)), tmp_path / "spe.png", flag="srgb")
    svb.imageio.imwrite(g.random((12, 10)), tmp_path / "rgh.png", flag="rough")
    n = np.zeros((12, 10, 3)); n[..., 2] = 1.0
    svb.imageio.imwrite(n, tmp_path / "nom.png", flag="normal")
    seen = {}

    def fake_video(self, n=59, light_intensity=0.5):
        seen["tex"] = tuple(self.textures.shape)
        seen["args"] = (n, light_intensity)
        fwd = [np.full((8, 8, 3), k / 60.0, np.float32) for k in range(n)]
        return fwd + fwd[-2:0:-1]

    monkeypatch.setattr(svb.envmap.EnvmapRenderer, "render_video", fake_video)
    frames = svb.render_envmap(tmp_path, 8, envmap=np.ones((4, 8, 3), np.float32), device="cpu")
    assert seen["tex"] == (9, 12, 10) and seen["args"] == (59, 0.5)
    assert len(frames) == 116
    files = sorted((tmp_path / "vid").glob("*.png"))
    assert [f.name for f in files[:2]] == ["000.png", "001.png"] and len(files) == 116
    assert np.allclose(svb.imageio.imread(files[115], "srgb"), 1 / 60.0, atol=1 / 255)


def _gif_decode(data):
    """A plain GIF89a reader for the tests: global palette, per-frame LZW (any code widths)."""
    import struct
    assert data[:6] == b"GIF89a"
    w, h, packed = struct.unpack_from("<HHB", data, 6)
    p = 13
    pal = None
    if packed & 0x80:
        n = 2 << (packed & 7)
        pal = np.frombuffer(data[p:p + 3 * n], np.uint8).reshape(n, 3)
        p += 3 * n
    frames, delays, loops = [], [], None
    while data[p] != 0x3B:
        if data[p] == 0x21:
            label = data[p + 1]
            q = p + 2
            blocks = []
            while data[q]:
                blocks.append(data[q + 1:q + 1 + data[q]])
                q += 1 + data[q]
            if label == 0xF9:
                delays.append(struct.unpack_from("<H", blocks[0], 1)[0])
            if label == 0xFF and blocks[0] == b"NETSCAPE2.0":
                loops = struct.unpack_from("<H", blocks[1], 1)[0]
            p = q + 1
        elif data[p] == 0x2C:
            fw, fh = struct.unpack_from("<HH", data, p + 5)
            mcs = data[p + 10]
            q = p + 11
            raw = bytearray()
            while data[q]:
                raw += data[q + 1:q + 1 + data[q]]
                q += 1 + data[q]
            p = q + 1
            bits = np.unpackbits(np.frombuffer(bytes(raw), np.uint8), bitorder="little")
            clear, end = 1 << mcs, (1 << mcs) + 1
            width, pos, out, table, prev = mcs + 1, 0, [], None, None
            while True:
                code = int(sum(int(bits[pos + k]) << k for k in range(width)))
                pos += width
                if code == clear:
                    table = [[i] for i in range(clear)] + [[], []]
                    width, prev = mcs + 1, None
                    continue
                if code == end:
                    break
                if prev is None:
                    entry = table[code]
                else:
                    entry = table[code] if code < len(table) else table[prev] + table[prev][:1]
                    table.append(table[prev] + entry[:1])
                    if len(table) == (1 << width) and width < 12:
                        width += 1
                out += entry
                prev = code
            frames.append(pal[np.array(out, np.int64)].reshape(fh, fw, 3))
        else:
            raise AssertionError(f"unexpected GIF block {data[p]:#x}")
    return frames, delays, loops


def test_gif_write_and_img2gif(svb, tmp_path):
    IO = svb.imageio
    g = np.random.default_rng(3)
    frames = [(g.random((21, 34, 3)) * 255).astype(np.uint8) for _ in range(3)]
    IO.gif_write(frames, tmp_path / "a.gif", delay_ms=40)
    dec, delays, loops = _gif_decode((tmp_path / "a.gif").read_bytes())
    assert len(dec) == 3 and delays == [4, 4, 4] and loops == 0
    pal = IO._gif_palette()
    for f, d in zip(frames, dec):
        assert np.array_equal(d, pal[IO._gif_indices(f)])  # the 3-3-2 quantisation, losslessly coded
        assert np.abs(d.astype(int) - f.astype(int)).max() <= 43  # within half a blue level
    names = []
    for i, f in enumerate(frames):
        names.append(tmp_path / f"{i:03d}.png")
        IO.png_write(names[-1], f)
    IO.img2gif(names, tmp_path / "b.gif")
    assert _gif_decode((tmp_path / "b.gif").read_bytes())[0][2].shape == (21, 34, 3)


def test_mosaics(svb, tmp_path):
    IO = svb.imageio
    ims = [np.full((4, 5, 3), k / 10.0, np.float32) for k in range(9)]
    for k, im in enumerate(ims):
        IO.imwrite(im, tmp_path / f"{k:02d}.png")
    IO.img9to1(tmp_path)
    allp = IO.imread(tmp_path / "all.png")
    assert allp.shape == (12, 15, 3) and np.allclose(allp[4, 5], 0.4, atol=1 / 255)  # row 1, column 1
    m = IO.imconcat([np.zeros((2, 3)), np.ones((2, 3)), np.ones((2, 3)) * 2, np.ones((2, 3)) * 3])
    assert m.shape == (4, 6) and m[3, 5] == 3 and m[0, 4] == 1


def test_savers_write_the_reference_mosaics(svb, tmp_path):
    """save_textures_th adds tex.png and save_images_th (nine views) all.png, as the reference does."""
    cfg = {"reference_dir": "ref", "target_dir": "target", "optimize_dir": "optim", "rerender_dir": "rerender",
           "im_size": 17.0, "idx": list(range(9)), "camera_pos": [[0, 0, 30]] * 9, "light_pos": [[0, 0, 30]] * 9,
           "light_pow": [1500, 1500, 1500]}
    j = tmp_path / "scene.json"
    j.write_text(json.dumps(cfg))
    io = svb.SvbrdfIO(j, "cpu")
    io.save_textures_th(svb.scenes.make_material(32, 5), io.reference_dir)
    assert (tmp_path / "ref" / "tex.png").exists()
    assert IO_shape(svb, tmp_path / "ref" / "tex.png") == (64, 64, 3)
    io.save_images_th(torch.rand(9, 3, 6, 6), io.target_dir)
    assert IO_shape(svb, tmp_path / "target" / "all.png") == (18, 18, 3)


def IO_shape(svb, p):
    return svb.imageio.imread(p).shape
