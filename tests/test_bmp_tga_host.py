"""BMP, TGA, GIF and Radiance HDR texture decoding on the host (the formats stbi_load reads besides PNG and JPEG, behind
Scene::defineTexture, src/graphics/Image.cpp:10-41): the test writes seeded images in each layout itself
— BMP with 1/4/8-bit palettes, 16-bit 5-5-5 and bit fields, 24-bit, 32-bit with and without alpha,
bottom-up and top-down; TGA true-colour 16/24/32-bit, grey, colour-mapped, uncompressed and run-length
encoded, both origins; GIF through its own LZW encoder (growing code widths, a full table cleared,
transparency, interlacing, local tables, an offset image); HDR with flat and run-length scanlines — and requires the decoded RGBA8 (rows
top to bottom) to equal the image it wrote (HDR: its tone mapping restated in numpy, within one level)."""
import struct

import numpy as np
import pytest


def rgba_image(H, W, seed, alpha=True):
    rng = np.random.default_rng(seed)
    img = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    if not alpha:
        img[..., 3] = 255
    return img


def bmp(img, bpp=24, top_down=False, palette=None, fields=None):
    H, W = img.shape[:2]
    rows = []
    for y in range(H):
        px = img[y]
        if bpp == 24:
            raw = px[:, [2, 1, 0]].tobytes()
        elif bpp == 32:
            raw = px[:, [2, 1, 0, 3]].tobytes()
        elif bpp == 16:
            v = ((px[:, 0].astype(np.uint32) >> 3) << 10) | ((px[:, 1].astype(np.uint32) >> 3) << 5) | (px[:, 2] >> 3)
            if fields:   # 5-6-5
                v = ((px[:, 0].astype(np.uint32) >> 3) << 11) | ((px[:, 1].astype(np.uint32) >> 2) << 5) | (px[:, 2] >> 3)
            raw = v.astype("<u2").tobytes()
        else:   # indices into `palette` (image holds palette colours)
            idx = [palette.index(tuple(int(c) for c in p[:3])) for p in px]
            bits = "".join(format(i, f"0{bpp}b") for i in idx)
            bits += "0" * (-len(bits) % 8)
            raw = bytes(int(bits[k:k + 8], 2) for k in range(0, len(bits), 8))
        raw += b"\0" * (-len(raw) % 4)
        rows.append(raw)
    if not top_down:
        rows = rows[::-1]
    pal = b"".join(bytes([b, g, r, 0]) for r, g, b in (palette or []))
    masks = struct.pack("<III", *fields) if fields else b""
    offset = 14 + 40 + len(masks) + len(pal)
    data = b"".join(rows)
    hdr = b"BM" + struct.pack("<IHHI", offset + len(data), 0, 0, offset)
    dib = struct.pack("<IiiHHIIiiII", 40, W, -H if top_down else H, 1, bpp, 3 if fields else 0, len(data), 2835, 2835,
                      len(palette or []), 0)
    return hdr + dib + masks + pal + data


def to5(c):
    return (((c.astype(np.uint32) >> 3) * 255 + 15) // 31).astype(np.uint8)


def to6(c):
    return (((c.astype(np.uint32) >> 2) * 255 + 31) // 63).astype(np.uint8)


def tga(img, kind="rgb32", rle=False, top_left=False):
    H, W = img.shape[:2]
    rows = list(img) if top_left else list(img[::-1])
    cmap = b""
    cmap_type, cmap_len, cmap_bits = 0, 0, 0
    if kind == "rgb32":
        vals = [bytes([p[2], p[1], p[0], p[3]]) for r in rows for p in r]
        itype, depth, desc = 2, 32, 8
    elif kind == "rgb24":
        vals = [bytes([p[2], p[1], p[0]]) for r in rows for p in r]
        itype, depth, desc = 2, 24, 0
    elif kind == "rgb16":
        vals = [struct.pack("<H", ((int(p[0]) >> 3) << 10) | ((int(p[1]) >> 3) << 5) | (int(p[2]) >> 3)) for r in rows for p in r]
        itype, depth, desc = 2, 16, 0
    elif kind == "gray":
        vals = [bytes([p[0]]) for r in rows for p in r]
        itype, depth, desc = 3, 8, 0
    else:   # colour-mapped, 24-bit entries
        colours = sorted({tuple(int(c) for c in p[:3]) for r in rows for p in r})
        cmap = b"".join(bytes([b, g, r]) for r, g, b in colours)
        vals = [bytes([colours.index(tuple(int(c) for c in p[:3]))]) for r in rows for p in r]
        itype, depth, desc = 1, 8, 0
        cmap_type, cmap_len, cmap_bits = 1, len(colours), 24
    if top_left:
        desc |= 0x20
    body = b""
    if not rle:
        body = b"".join(vals)
    else:
        i = 0
        while i < len(vals):   # runs of equal values as run packets, the rest as raw packets (<= 128)
            j = i
            while j + 1 < len(vals) and vals[j + 1] == vals[i] and j + 1 - i < 128:
                j += 1
            if j > i:
                body += bytes([0x80 | (j - i)]) + vals[i]
                i = j + 1
            else:
                k = i
                while k + 1 < len(vals) and vals[k + 1] != vals[k] and k + 1 - i < 128:
                    k += 1
                body += bytes([k - i]) + b"".join(vals[i:k + 1])
                i = k + 1
        itype += 8
    hdr = struct.pack("<BBBHHBHHHHBB", 0, cmap_type, itype, 0, cmap_len, cmap_bits, 0, 0, W, H, depth, desc)
    return hdr + cmap + body


@pytest.mark.parametrize("H,W", [(5, 7), (16, 16), (1, 3), (9, 1)])
def test_bmp_layouts(R, H, W):
    img = rgba_image(H, W, H * 31 + W)
    opaque = img.copy()
    opaque[..., 3] = 255
    assert np.array_equal(R.decode_image(bmp(img, 24)), opaque)
    assert np.array_equal(R.decode_image(bmp(img, 24, top_down=True)), opaque)
    assert np.array_equal(R.decode_image(bmp(img, 32)), img)
    no_alpha = img.copy()
    no_alpha[..., 3] = 0   # an unused alpha channel decodes opaque
    assert np.array_equal(R.decode_image(bmp(no_alpha, 32, top_down=True)), opaque)
    want16 = np.stack([to5(img[..., 0]), to5(img[..., 1]), to5(img[..., 2]), np.full((H, W), 255, np.uint8)], -1)
    assert np.array_equal(R.decode_image(bmp(img, 16)), want16)
    want565 = np.stack([to5(img[..., 0]), to6(img[..., 1]), to5(img[..., 2]), np.full((H, W), 255, np.uint8)], -1)
    assert np.array_equal(R.decode_image(bmp(img, 16, fields=(0xF800, 0x07E0, 0x001F))), want565)
    for bpp in (1, 4, 8):
        rng = np.random.default_rng(bpp)
        palette = [tuple(int(c) for c in rng.integers(0, 256, 3)) for _ in range(1 << bpp)]
        pal_img = np.zeros((H, W, 4), np.uint8)
        pal_img[..., 3] = 255
        idx = rng.integers(0, 1 << bpp, (H, W))
        for y in range(H):
            for x in range(W):
                pal_img[y, x, :3] = palette[idx[y, x]]
        assert np.array_equal(R.decode_image(bmp(pal_img, bpp, palette=palette)), pal_img), bpp


@pytest.mark.parametrize("rle", [False, True])
@pytest.mark.parametrize("top_left", [False, True])
def test_tga_layouts(R, rle, top_left):
    H, W = 11, 13
    img = rgba_image(H, W, 7 + rle + 2 * top_left)
    img[3:6, 2:9] = img[3, 2]   # runs for the run-length packets
    opaque = img.copy()
    opaque[..., 3] = 255
    assert np.array_equal(R.decode_image(tga(img, "rgb32", rle, top_left)), img)
    assert np.array_equal(R.decode_image(tga(img, "rgb24", rle, top_left)), opaque)
    want16 = np.stack([to5(img[..., 0]), to5(img[..., 1]), to5(img[..., 2]), np.full((H, W), 255, np.uint8)], -1)
    assert np.array_equal(R.decode_image(tga(img, "rgb16", rle, top_left)), want16)
    gray = np.stack([img[..., 0]] * 3 + [np.full((H, W), 255, np.uint8)], -1)
    assert np.array_equal(R.decode_image(tga(img, "gray", rle, top_left)), gray)
    few = img.copy()
    few[..., :3] = (few[..., :3] // 64) * 64   # at most 64 colours for the colour map
    few[..., 3] = 255
    assert np.array_equal(R.decode_image(tga(few, "mapped", rle, top_left)), few)


def test_bmp_tga_malformed(R):
    img = rgba_image(4, 4, 1)
    good_bmp, good_tga = bmp(img, 24), tga(img, "rgb32", rle=True)
    bad = [good_bmp[:40], good_bmp[:-5], good_tga[:-3], good_bmp[:30] + struct.pack("<I", 1) + good_bmp[34:]]
    for data in bad:
        with pytest.raises(R.ReinaError) as e:
            R.decode_image(data)
        assert e.value.code == R.REINA_ERR_IO


def hdr_file(rgbe, rle):
    H, W = rgbe.shape[:2]
    out = b"#?RADIANCE\n# written by the test\nFORMAT=32-bit_rle_rgbe\n\n" + f"-Y {H} +X {W}\n".encode()
    for y in range(H):
        if not rle:
            out += rgbe[y].tobytes()
            continue
        out += bytes([2, 2, W >> 8, W & 255])
        for c in range(4):   # runs of >= 3 equal bytes as run codes, the rest as literals (<= 128 / 127)
            ch = rgbe[y, :, c].tolist()
            x = 0
            while x < W:
                r = 1
                while x + r < W and ch[x + r] == ch[x] and r < 127:
                    r += 1
                if r >= 3:
                    out += bytes([128 + r, ch[x]])
                    x += r
                    continue
                lit = 1
                while x + lit < W and lit < 128 and not (x + lit + 2 < W and ch[x + lit] == ch[x + lit + 1] == ch[x + lit + 2]):
                    lit += 1
                out += bytes([lit]) + bytes(ch[x:x + lit])
                x += lit
    return out


@pytest.mark.parametrize("rle", [False, True])
def test_hdr_rgbe(R, rle):
    """Radiance RGBE read as an 8-bit texture the way stbi_load does (gamma 1/2.2, scale 1)."""
    rng = np.random.default_rng(5 + rle)
    H, W = 9, 40
    rgbe = np.zeros((H, W, 4), np.uint8)
    rgbe[..., :3] = rng.integers(0, 256, (H, W, 3))
    rgbe[..., 3] = rng.integers(124, 140, (H, W))
    rgbe[2, 5:30] = rgbe[2, 5]   # runs for the run-length scanlines
    rgbe[4, :, 3] = 0            # exponent 0: black
    got = R.decode_image(hdr_file(rgbe, rle))
    f = rgbe[..., :3].astype(np.float32) * np.ldexp(np.float32(1), rgbe[..., 3:4].astype(np.int32) - 136).astype(np.float32)
    want = np.clip(np.floor(np.power(f, np.float32(1 / 2.2)) * 255 + 0.5), 0, 255).astype(np.int64)
    want[rgbe[..., 3] == 0] = 0
    assert got.shape == (H, W, 4) and (got[..., 3] == 255).all()
    d = np.abs(got[..., :3].astype(np.int64) - want)
    assert d.max() <= 1 and (d == 0).mean() >= 0.99, (d.max(), (d == 0).mean())


def test_hdr_malformed(R):
    rgbe = np.full((3, 8, 4), 128, np.uint8)
    good = hdr_file(rgbe, True)
    for data in (good[:-4], good.replace(b"-Y 3 +X 8", b"+Y 3 +X 8"), good.replace(b"rle_rgbe", b"rle_xyze")):
        with pytest.raises(R.ReinaError) as e:
            R.decode_image(data)
        assert e.value.code == R.REINA_ERR_IO


def lzw_gif(indices, min_size):
    """GIF's LZW: codes of min_size + 1 bits growing to 12, a clear code first and when the table fills."""
    clear, end = 1 << min_size, (1 << min_size) + 1
    codes = [(clear, min_size + 1)]
    size, nxt = min_size + 1, end + 1
    table = {(i,): i for i in range(clear)}
    w = ()
    for k in indices:
        wk = w + (int(k),)
        if wk in table:
            w = wk
            continue
        codes.append((table[w], size))
        table[wk] = nxt
        nxt += 1
        if nxt - 1 == (1 << size) and size < 12:   # the decoder adds its entries one code later
            size += 1
        if nxt == 4096:
            codes.append((clear, size))
            table = {(i,): i for i in range(clear)}
            size, nxt = min_size + 1, end + 1
        w = (int(k),)
    if w:
        codes.append((table[w], size))
    if nxt == (1 << size) and size < 12:
        size += 1
    codes.append((end, size))
    acc, nbits, out = 0, 0, bytearray()
    for c, s in codes:
        acc |= c << nbits
        nbits += s
        while nbits >= 8:
            out.append(acc & 255)
            acc >>= 8
            nbits -= 8
    if nbits:
        out.append(acc & 255)
    return bytes(out)


def gif_file(idx, palette, W, H, left=0, top=0, transparent=None, interlace=False, local=False):
    ih, iw = idx.shape
    bits = max(1, (len(palette) - 1).bit_length())
    table = b"".join(bytes(c) for c in palette) + b"\0" * (3 * (1 << bits) - 3 * len(palette))
    out = b"GIF89a" + struct.pack("<HHBBB", W, H, 0 if local else 0x80 | (bits - 1), 0, 0)
    if not local:
        out += table
    if transparent is not None:
        out += b"\x21\xf9\x04" + bytes([1, 0, 0, transparent, 0])
    out += b"\x2c" + struct.pack("<HHHHB", left, top, iw, ih, (0x80 | (bits - 1) if local else 0) | (0x40 if interlace else 0))
    if local:
        out += table
    rows = list(range(ih))
    if interlace:
        rows = list(range(0, ih, 8)) + list(range(4, ih, 8)) + list(range(2, ih, 4)) + list(range(1, ih, 2))
    min_size = max(2, bits)
    data = lzw_gif(idx[rows].reshape(-1), min_size)
    out += bytes([min_size])
    for k in range(0, len(data), 255):
        out += bytes([len(data[k:k + 255])]) + data[k:k + 255]
    return out + b"\x00\x3b"


@pytest.mark.parametrize("case", range(5))
def test_gif_first_frame(R, case):
    W, H, ncol, left, top, transp, inter, local = [
        (17, 13, 4, 0, 0, None, False, False),
        (64, 40, 16, 3, 5, 2, False, True),
        (33, 29, 4, 0, 0, None, True, False),
        (90, 80, 256, 0, 0, 7, False, False),    # random colours: the code table fills and is cleared
        (40, 40, 2, 4, 4, None, True, True),
    ][case]
    rng = np.random.default_rng(case)
    palette = [tuple(int(c) for c in rng.integers(0, 256, 3)) for _ in range(ncol)]
    iw, ih = W - left, H - top
    idx = rng.integers(0, ncol, (ih, iw)).astype(np.uint8)
    if ncol <= 16:   # runs, so that LZW strings repeat
        idx[: ih // 2] = idx[0, 0]
    got = R.decode_image(gif_file(idx, palette, W, H, left, top, transp, inter, local))
    want = np.zeros((H, W, 4), np.uint8)
    for y in range(ih):
        for x in range(iw):
            if idx[y, x] != transp:
                want[top + y, left + x] = (*palette[idx[y, x]], 255)
    assert np.array_equal(got, want)


def test_gif_malformed(R):
    idx = np.zeros((4, 4), np.uint8)
    good = gif_file(idx, [(1, 2, 3), (4, 5, 6)], 4, 4)
    for data in (good[:12], good[:-10], good.replace(b"\x2c", b"\x99", 1), b"GIF89a" + good[6:13] + b"\x3b"):
        with pytest.raises(R.ReinaError) as e:
            R.decode_image(data)
        assert e.value.code == R.REINA_ERR_IO


def test_oversized_headers_are_rejected_before_allocating(R):
    """A few bytes that declare a 65535 x 65535 image (2^32 pixels, 17 GB as RGBA8) fail at once, before the
    decoder reserves the canvas: the cap is 2^28 pixels, as for PNG, JPEG, BMP and HDR."""
    big_gif = b"GIF89a" + struct.pack("<HHBBB", 0xFFFF, 0xFFFF, 0x80, 0, 0) + b"\0" * 6 + b"\x2c" + b"\0" * 9 + b"\x02\x00\x3b"
    small_screen_big_frame = (b"GIF89a" + struct.pack("<HHBBB", 4, 4, 0x80, 0, 0) + b"\0" * 6 + b"\x2c" +
                              struct.pack("<HHHHB", 0, 0, 0xFFFF, 0xFFFF, 0) + b"\x02\x00\x3b")
    big_tga = struct.pack("<BBBHHBHHHHBB", 0, 0, 2, 0, 0, 0, 0, 0, 0xFFFF, 0xFFFF, 32, 0) + b"\0" * 8
    big_tga_rle = struct.pack("<BBBHHBHHHHBB", 0, 0, 10, 0, 0, 0, 0, 0, 0xFFFF, 0xFFFF, 32, 0) + b"\0" * 8
    short_tga = struct.pack("<BBBHHBHHHHBB", 0, 0, 2, 0, 0, 0, 0, 0, 100, 100, 32, 0) + b"\0" * 64
    for data in (big_gif, small_screen_big_frame, big_tga, big_tga_rle, short_tga):
        with pytest.raises(R.ReinaError) as e:
            R.decode_image(data)
        assert e.value.code == R.REINA_ERR_IO


def test_hdr_mode_is_decided_by_the_first_scanline(R):
    """A flat file whose later row starts with the bytes of a run-length header (2, 2, W >> 8, W & 255) reads
    that row as pixels, as stbi_load does; a run-length file whose later scanline lacks the header fails."""
    H, W = 3, 8
    rgbe = np.full((H, W, 4), 130, np.uint8)
    rgbe[1, 0] = (2, 2, 0, W)            # pixel bytes equal to a run-length header
    rgbe[1, 1] = (200, 10, 10, 129)
    got = R.decode_image(hdr_file(rgbe, False))
    assert got.shape == (H, W, 4)
    f = rgbe[..., :3].astype(np.float32) * np.ldexp(np.float32(1), rgbe[..., 3:4].astype(np.int32) - 136).astype(np.float32)
    want = np.clip(np.floor(np.power(f, np.float32(1 / 2.2)) * 255 + 0.5), 0, 255).astype(np.int64)
    assert np.abs(got[..., :3].astype(np.int64) - want).max() <= 1
    rle = hdr_file(np.full((H, W, 4), 130, np.uint8), True)
    head, body = rle.split(b"+X 8\n", 1)
    rows = body.split(bytes([2, 2, 0, W]))[1:]
    broken = head + b"+X 8\n" + bytes([2, 2, 0, W]) + rows[0] + bytes(rgbe[1].tobytes()) + bytes([2, 2, 0, W]) + rows[2]
    with pytest.raises(R.ReinaError) as e:
        R.decode_image(broken)
    assert e.value.code == R.REINA_ERR_IO


def test_bmp_full_width_bit_field(R):
    """A 32-bit bit-field BMP whose red mask is all 32 bits: red scales from 32 bits (no shift by 32)."""
    H, W = 2, 3
    px = np.array([[0, 0xFFFFFFFF, 0x80000000], [0x7FFFFFFF, 1, 0xC0000000]], np.uint32)
    data = px.astype("<u4").tobytes()
    masks = struct.pack("<III", 0xFFFFFFFF, 0, 0)
    offset = 14 + 40 + len(masks)
    hdr = b"BM" + struct.pack("<IHHI", offset + len(data), 0, 0, offset)
    dib = struct.pack("<IiiHHIIiiII", 40, W, -H, 1, 32, 3, len(data), 2835, 2835, 0, 0)
    got = R.decode_image(hdr + dib + masks + data)
    top = 0xFFFFFFFF
    want_r = (px.astype(np.uint64) * 255 + top // 2) // top
    assert np.array_equal(got[..., 0], want_r.astype(np.uint8))
    assert (got[..., 1] == 0).all() and (got[..., 2] == 0).all()
