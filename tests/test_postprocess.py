"""Post-process and export (postprocess.glsl, Export.h): the oracle against a float32 numpy
restatement of the shader's formulas (CPU), the GPU pass against the oracle bit for bit, and
the PNG / PFM writers by reading the files back."""
import struct
import zlib

import numpy as np
import pytest

import lavaframe_gb300 as lf
import oracle
from tests import scenes

F = np.float32


def np_texture(img, u, v):
    """GL_LINEAR + GL_REPEAT sampling of an (H, W, 3) image at (u, v) arrays."""
    h, w = img.shape[:2]
    xf = u * F(w) - F(0.5)
    yf = v * F(h) - F(0.5)
    fx, fy = np.floor(xf), np.floor(yf)
    a, b = (xf - fx)[..., None], (yf - fy)[..., None]
    x0, y0 = fx.astype(np.int64) % w, fy.astype(np.int64) % h
    x1, y1 = (x0 + 1) % w, (y0 + 1) % h
    top = img[y0, x0] * (F(1) - a) + img[y0, x1] * a
    bot = img[y1, x0] * (F(1) - a) + img[y1, x1] * a
    return top * (F(1) - b) + bot * b


def np_post(acc, p, samples):
    h, w = acc.shape[:2]
    u = ((np.arange(w, dtype=F) + F(0.5)) / F(w))[None, :].repeat(h, 0)
    v = ((np.arange(h, dtype=F) + F(0.5)) / F(h))[:, None].repeat(w, 1)
    inv = F(1.0) / F(samples)
    if p.use_ca and not p.preview:
        dist = np.sqrt((u - F(p.ca_p3)) ** 2 + (v - F(p.ca_p3)) ** 2).astype(F) ** F(p.ca_p1) * F(p.ca_p2)
        s = F(p.ca_distance) * dist if p.use_ca_distortion else np.full_like(u, F(p.ca_distance) * F(0.025) * F(p.ca_p2))
        c = np.stack([np_texture(acc, u + s, v + s)[..., 0], np_texture(acc, u, v)[..., 1],
                      np_texture(acc, u - s, v - s)[..., 2]], -1) * inv
    else:
        c = np_texture(acc, u, v) * inv
    g = F(1.0) / F(2.2)
    t = p.tonemap
    if t == 1:
        lum = F(0.3) * c[..., 0] + F(0.6) * c[..., 1] + F(0.1) * c[..., 2]
        c = (c / (F(1) + lum / F(2))[..., None]) ** g
    elif t == 2:
        c = np.clip((c * (F(2.51) * c + F(0.03))) / (c * (F(2.43) * c + F(0.59)) + F(0.14)), 0, 1) ** g
    elif t == 3:
        c = np.clip(c / (c + F(1)), 0, 1) ** g
    elif t == 4:
        c = ((c * (c * (F(1.2295) * c + F(0.3135)) + F(1.1935) * F(0.4655))) /
             (c * (F(1.1935) * c + F(0.4655)) + F(0.073))) ** F(1.7)
        c = np.clip(c ** (F(1) / F(0.8)) * F(0.8), 0, 1) ** g
    elif t == 5:
        c = np.maximum(F(0), c - F(0.004))
        c = (c * (F(6.2) * c + F(0.5))) / (c * (F(6.2) * c + F(1.7)) + F(0.06))
    elif t == 6:
        c = ((c * (F(0.15) * c + F(0.05)) + F(0.004)) / (c * (F(0.15) * c + F(0.5)) + F(0.06)) - F(0.02) / F(0.3))
        c = c ** g * F(1.75)
    if p.use_vignette:
        d = F(1) - np.sqrt((u - F(0.5)) ** 2 + (v - F(0.5)) ** 2) ** F(p.vignette_power) * F(p.vignette_intensity)
        c = c * d[..., None]
    return c.astype(F)


def settings():
    from tests.golden.cases import post_settings

    return post_settings()


def test_oracle_postprocess_matches_the_shader_formulas():
    rng = np.random.default_rng(0)
    acc = (rng.gamma(1.5, 1.0, (24, 40, 3)) * 16).astype(np.float32)
    for p in settings():
        _, got = oracle.postprocess(acc, p, 16)
        ref = np_post(acc, p, 16)
        np.testing.assert_allclose(got, ref, rtol=2e-5, atol=2e-6, err_msg=str(p.tonemap))


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        assert zlib.crc32(typ + body) == struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    n = 3 * w
    out = np.zeros((h, n), np.int64)
    for y in range(h):   # undo the row filters (PNG specification section 9)
        f = raw[y * (n + 1)]
        line = np.frombuffer(raw[y * (n + 1) + 1:(y + 1) * (n + 1)], np.uint8).astype(np.int64)
        up = out[y - 1] if y else np.zeros(n, np.int64)
        for i in range(n):
            a = out[y, i - 3] if i >= 3 else 0
            b, c = up[i], (up[i - 3] if i >= 3 else 0)
            if f == 0:
                pred = 0
            elif f == 1:
                pred = a
            elif f == 2:
                pred = b
            elif f == 3:
                pred = (a + b) // 2
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            out[y, i] = (line[i] + pred) % 256
    return out.astype(np.uint8).reshape(h, w, 3)


def test_png_and_pfm_writers_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    img8 = rng.integers(0, 256, (70, 300, 3), dtype=np.uint8)   # > 64 KiB: several stored blocks
    lf.write_image(tmp_path / "a.png", img8)
    back = read_png(tmp_path / "a.png")
    assert np.array_equal(back, img8[::-1])                      # written top row first
    imgf = rng.normal(size=(5, 7, 3)).astype(np.float32)
    lf.write_image(tmp_path / "a.pfm", imgf)
    raw = open(tmp_path / "a.pfm", "rb").read()
    hdr = b"PF\n7 5\n-1.0\n"
    assert raw.startswith(hdr)
    assert np.array_equal(np.frombuffer(raw[len(hdr):], "<f4").reshape(5, 7, 3), imgf)


def read_bmp(path):
    """24-bit BI_RGB reader (BITMAPFILEHEADER + BITMAPINFOHEADER), rows returned bottom-first."""
    data = open(path, "rb").read()
    assert data[:2] == b"BM" and struct.unpack("<I", data[2:6])[0] == len(data)
    off, hsize, w, h, planes, bpp, comp = struct.unpack("<I I i i H H I", data[10:34])
    assert (hsize, planes, bpp, comp) == (40, 1, 24, 0) and h > 0
    stride = (3 * w + 3) // 4 * 4
    rows = [np.frombuffer(data[off + y * stride: off + y * stride + 3 * w], np.uint8).reshape(w, 3)[:, ::-1]
            for y in range(h)]
    return np.stack(rows)


def read_tga(path):
    """Type-10 (run-length true colour, 24-bit) reader, rows returned bottom-first."""
    data = open(path, "rb").read()
    idlen, cmtype, typ = data[0], data[1], data[2]
    w, h, bpp, desc = struct.unpack("<HHBB", data[12:18])
    assert (cmtype, typ, bpp) == (0, 10, 24) and not desc & 0x20   # bottom-left origin
    pos, px = 18 + idlen, []
    while len(px) < w * h:
        c = data[pos]
        pos += 1
        n = (c & 0x7F) + 1
        if c & 0x80:
            px += [data[pos:pos + 3]] * n
            pos += 3
        else:
            px += [data[pos + 3 * k:pos + 3 * k + 3] for k in range(n)]
            pos += 3 * n
    assert len(px) == w * h and data[pos:] == b"\0" * 8 + b"TRUEVISION-XFILE.\0"
    return np.frombuffer(b"".join(px), np.uint8).reshape(h, w, 3)[:, :, ::-1]


def read_exr(path):
    """Single-part scanline OpenEXR reader for 32-bit float channels: uncompressed, RLE, ZIPS or
    ZIP (run-length or zlib decoding, then the byte predictor and the even/odd split undone)."""
    data = open(path, "rb").read()
    assert data[:4] == bytes([0x76, 0x2F, 0x31, 0x01]) and data[4] == 2
    pos, attrs = 8, {}
    while data[pos] != 0:
        name_end = data.index(0, pos)
        type_end = data.index(0, name_end + 1)
        size = struct.unpack("<i", data[type_end + 1:type_end + 5])[0]
        attrs[data[pos:name_end].decode()] = (data[name_end + 1:type_end].decode(),
                                                data[type_end + 5:type_end + 5 + size])
        pos = type_end + 5 + size
    pos += 1
    comp = attrs["compression"][1][0]
    assert comp in (0, 1, 2, 3)
    lines = 16 if comp == 3 else 1
    ch, chans = attrs["channels"][1], []
    i = 0
    while ch[i] != 0:
        e = ch.index(0, i)
        ptype, _, xs, ys = struct.unpack("<iiii", ch[e + 1:e + 17])
        assert ptype == 2 and xs == ys == 1
        chans.append(ch[i:e].decode())
        i = e + 17
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    nblocks = (h + lines - 1) // lines
    offsets = struct.unpack(f"<{nblocks}Q", data[pos:pos + 8 * nblocks])
    img = np.zeros((h, w, len(chans)), np.float32)
    for off in offsets:
        y, n = struct.unpack("<ii", data[off:off + 8])
        rows = min(lines, y0 + h - y)
        size = 4 * w * len(chans) * rows
        blk = data[off + 8:off + 8 + n]
        if n < size:
            if comp == 1:
                dec, k = bytearray(), 0
                while k < len(blk):
                    c = struct.unpack("b", blk[k:k + 1])[0]
                    if c < 0:
                        dec += blk[k + 1:k + 1 - c]
                        k += 1 - c
                    else:
                        dec += blk[k + 1:k + 2] * (c + 1)
                        k += 2
                blk = bytes(dec)
            else:
                blk = zlib.decompress(blk)
            t = np.frombuffer(blk, np.uint8).astype(np.int64)
            t = (np.cumsum(t - 128) + 128) % 256    # t[i] = t[i-1] + d[i] - 128, t[0] = d[0]
            half = (size + 1) // 2
            raw = np.empty(size, np.uint8)
            raw[0::2], raw[1::2] = t[:half], t[half:]
            blk = raw.tobytes()
        assert len(blk) == size
        block = np.frombuffer(blk, "<f4").reshape(rows, len(chans), w)
        img[y - y0:y - y0 + rows] = block.transpose(0, 2, 1)
    return chans, img


def test_png_and_exr_are_deflated(tmp_path):
    # the writers' own deflate (fixed Huffman codes, LZ77) must round-trip through zlib and
    # shrink smooth images; noise may stay near its raw size
    yy, xx = np.mgrid[0:200, 0:300]
    smooth = np.stack([xx % 256, yy % 256, (xx // 8 + yy // 8) % 256], -1).astype(np.uint8)
    lf.write_image(tmp_path / "s.png", smooth)
    assert np.array_equal(read_png(tmp_path / "s.png"), smooth[::-1])
    assert (tmp_path / "s.png").stat().st_size < smooth.nbytes / 4
    imgf = (smooth / 255.0).astype(np.float32)
    lf.write_image(tmp_path / "s.exr", imgf)
    chans, back = read_exr(tmp_path / "s.exr")
    assert back[:, :, ::-1].tobytes() == imgf.tobytes()
    assert (tmp_path / "s.exr").stat().st_size < imgf.nbytes / 2
    for comp in (0, 1, 2, 3):   # none, RLE, ZIPS, ZIP
        lf.write_image(tmp_path / f"c{comp}.exr", imgf, exr_compression=comp)
        _, back = read_exr(tmp_path / f"c{comp}.exr")
        assert back[:, :, ::-1].tobytes() == imgf.tobytes(), comp
    # long runs for the run-length code (a constant like 0.25 leaves the predictor's odd-byte
    # half alternating, which run-length coding cannot shorten)
    flat = np.zeros((40, 50, 3), np.float32)
    flat[5:9, 10:20] = 1.0
    lf.write_image(tmp_path / "f.exr", flat, exr_compression=1)
    assert read_exr(tmp_path / "f.exr")[1].tobytes() == flat.tobytes()
    assert (tmp_path / "f.exr").stat().st_size < flat.nbytes / 10
    noise = np.random.default_rng(7).integers(0, 256, (64, 65, 3), dtype=np.uint8)
    lf.write_image(tmp_path / "n.png", noise)
    assert np.array_equal(read_png(tmp_path / "n.png"), noise[::-1])


def test_bmp_tga_exr_writers_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    for h, w in ((5, 7), (33, 130)):   # odd widths: BMP row padding; TGA packets within rows
        img8 = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
        img8[1, 2:40] = (10, 20, 30)                 # runs for the TGA run-length packets
        img8[-1] = 255
        lf.write_image(tmp_path / "a.bmp", img8)
        assert np.array_equal(read_bmp(tmp_path / "a.bmp"), img8)   # stored bottom-up
        lf.write_image(tmp_path / "a.tga", img8)
        assert np.array_equal(read_tga(tmp_path / "a.tga"), img8)
        imgf = rng.normal(size=(h, w, 3)).astype(np.float32)
        imgf[0, 0] = (np.inf, -0.0, 1e-40)
        lf.write_image(tmp_path / "a.exr", imgf)
        chans, back = read_exr(tmp_path / "a.exr")
        assert chans == ["B", "G", "R"]
        # rows in the order given, channels by name: bit for bit
        assert back[:, :, ::-1].tobytes() == imgf.tobytes()


def read_jpg(path):
    """Baseline sequential JPEG decoder (ITU-T T.81, 8-bit, 1x1 sampling), rows returned top down."""
    data = open(path, "rb").read()
    assert data[:2] == b"\xff\xd8"
    pos, qt, huff, comps, scan = 2, {}, {}, None, None
    while True:
        assert data[pos] == 0xFF
        m = data[pos + 1]
        pos += 2
        if m == 0xD9:
            break
        n = struct.unpack(">H", data[pos:pos + 2])[0]
        seg = data[pos + 2:pos + n]
        pos += n
        if m == 0xDB:
            i = 0
            while i < len(seg):
                assert seg[i] >> 4 == 0
                qt[seg[i] & 15] = np.frombuffer(seg[i + 1:i + 65], np.uint8).astype(np.float64)
                i += 65
        elif m == 0xC0:
            assert seg[0] == 8
            h, w = struct.unpack(">HH", seg[1:5])
            comps = [(seg[6 + 3 * k], seg[7 + 3 * k], seg[8 + 3 * k]) for k in range(seg[5])]
            assert all(c[1] == 0x11 for c in comps)
        elif m == 0xC4:
            i = 0
            while i < len(seg):
                bits, k, code, table = seg[i + 1:i + 17], 0, 0, {}
                vals = seg[i + 17:i + 17 + sum(bits)]
                for length in range(1, 17):
                    for _ in range(bits[length - 1]):
                        table[(length, code)] = vals[k]
                        code, k = code + 1, k + 1
                    code <<= 1
                huff[seg[i]] = table
                i += 17 + sum(bits)
        elif m == 0xDA:
            scan = [(seg[1 + 2 * k], seg[2 + 2 * k]) for k in range(seg[0])]
            end = pos
            while not (data[end] == 0xFF and data[end + 1] != 0):
                end += 1
            ecs = data[pos:end].replace(b"\xff\x00", b"\xff")
            pos = end
    bitstr = "".join(f"{b:08b}" for b in ecs)
    bp = 0

    def receive(nbits):
        nonlocal bp
        v = int(bitstr[bp:bp + nbits], 2) if nbits else 0
        bp += nbits
        return v

    def decode(table):
        code = 0
        for length in range(1, 17):
            code = (code << 1) | receive(1)
            if (length, code) in table:
                return table[(length, code)]
        raise AssertionError("bad Huffman code")

    def extend(v, t):
        return v - (1 << t) + 1 if t and v < (1 << (t - 1)) else v

    order = sorted(range(64), key=lambda i: (i // 8 + i % 8, i // 8 if (i // 8 + i % 8) % 2 else -(i // 8)))
    cu = np.array([np.sqrt(0.5)] + [1.0] * 7)
    M = np.array([[cu[u] / 2 * np.cos((2 * x + 1) * u * np.pi / 16) for x in range(8)] for u in range(8)])
    bw, bh = (w + 7) // 8, (h + 7) // 8
    planes = np.zeros((3, bh * 8, bw * 8))
    pred = [0, 0, 0]
    qsel = {c[0]: c[2] for c in comps}
    for by in range(bh):
        for bx in range(bw):
            for ci, (cid, tables) in enumerate(scan):
                coef = np.zeros(64)
                t = decode(huff[0x00 | (tables >> 4)])
                pred[ci] += extend(receive(t), t)
                coef[0] = pred[ci]
                k = 1
                while k < 64:
                    rs = decode(huff[0x10 | (tables & 15)])
                    r, sz = rs >> 4, rs & 15
                    if sz == 0:
                        if r != 15:
                            break
                        k += 16
                        continue
                    k += r
                    coef[k] = extend(receive(sz), sz)
                    k += 1
                F = np.zeros(64)
                F[order] = coef * qt[qsel[cid]]
                planes[ci, by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] = M.T @ F.reshape(8, 8) @ M
    Y, Cb, Cr = planes[0] + 128, planes[1], planes[2]
    rgb = np.stack([Y + 1.402 * Cr, Y - 0.344136 * Cb - 0.714136 * Cr, Y + 1.772 * Cb], -1)
    return np.clip(np.rint(rgb), 0, 255)[:h, :w]


def test_jpg_writer_decodes_to_the_image(tmp_path):
    rng = np.random.default_rng(3)
    for h, w in ((21, 37), (48, 64)):   # partial edge blocks, and whole ones
        yy, xx = np.mgrid[0:h, 0:w]
        smooth = np.stack([xx * 255 / w, yy * 255 / h, (xx + yy) * 127 / (w + h) + 60], -1)
        img8 = np.clip(smooth + rng.normal(0, 3, smooth.shape), 0, 255).astype(np.uint8)
        sizes = {}
        for q in (50, 95, 100):
            lf.write_image(tmp_path / f"a{q}.jpg", img8, jpg_quality=q)
            sizes[q] = (tmp_path / f"a{q}.jpg").stat().st_size
            back = read_jpg(tmp_path / f"a{q}.jpg")
            err = np.abs(back - img8[::-1].astype(np.float64))   # shown upright: top row first
            # noise of sigma 3 sits in the coefficients that quality 50 and 95 quantise
            assert err.mean() < {50: 4.0, 95: 3.0, 100: 0.5}[q], (q, err.mean())
            assert err.max() <= {50: 25, 95: 16, 100: 3}[q], (q, err.max())
        assert sizes[50] < sizes[95] < sizes[100]


@pytest.mark.gpu
def test_gpu_postprocess_is_bit_exact(ctx):
    s = scenes.build("cornell")
    p = s.render_params()
    p.width, p.height = 80, 56
    ds = ctx.upload(s)
    f = lf.Frame(ctx, ds, p)
    f.render(0, 8)
    f.sync()
    acc = f.accum()
    try:
        for pp in settings():
            rgb8, rgbf = f.postprocess(8, pp)
            o8, of = oracle.postprocess(acc, pp, 8)
            assert rgbf.view(np.uint32).tobytes() == of.view(np.uint32).tobytes(), pp.tonemap
            assert np.array_equal(rgb8, o8)
    finally:
        f.close()
        ds.close()
