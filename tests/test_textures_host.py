"""Texture input on the host: the PNG decoder behind reina_decode_image / reina_scene_define_texture_* against
an independent restatement (Python's zlib for inflate, numpy for the row filters and the RGBA8
conversion stbi_load(..., 4) applies), over synthetic PNGs of every colour type, bit depth, filter,
compression level and interlacing, and over the reference's own texture files when they are present;
plus the texture-id checks of reina_scene_build."""
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

import scenes
from conftest import reference_dir

REF_TEXTURES = reference_dir("textures")

CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]


def chunk(t: bytes, d: bytes) -> bytes:
    return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)


def pack_row(samples: np.ndarray, depth: int) -> bytes:
    """One row of samples (flattened channel values) at a bit depth, MSB first."""
    s = samples.astype(np.uint32).reshape(-1)
    if depth == 16:
        return s.astype(">u2").tobytes()
    if depth == 8:
        return s.astype(np.uint8).tobytes()
    per = 8 // depth
    pad = (-len(s)) % per
    s = np.concatenate([s, np.zeros(pad, np.uint32)]).reshape(-1, per)
    shifts = (8 - depth * (np.arange(per) + 1)).astype(np.uint32)
    return (s << shifts).sum(axis=1).astype(np.uint8).tobytes()


def filter_rows(rows: list, bpp: int, rng) -> bytes:
    """Applies a random PNG filter type to each row (PNG specification section 9)."""
    out = bytearray()
    prev = bytes(len(rows[0])) if rows else b""
    for r in rows:
        ft = int(rng.integers(0, 5))
        cur = np.frombuffer(r, np.uint8).astype(np.int32)
        up = np.frombuffer(prev, np.uint8).astype(np.int32)
        f = np.zeros_like(cur)
        for i in range(len(cur)):
            a = cur[i - bpp] if i >= bpp else 0
            b = up[i]
            c = up[i - bpp] if i >= bpp else 0
            if ft == 0:
                pred = 0
            elif ft == 1:
                pred = a
            elif ft == 2:
                pred = b
            elif ft == 3:
                pred = (a + b) >> 1
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            f[i] = (cur[i] - pred) & 255
        out += bytes([ft]) + f.astype(np.uint8).tobytes()
        prev = r
    return bytes(out)


def encode_png(samples: np.ndarray, ctype: int, depth: int, interlace: int = 0, palette=None, trns=None,
               level: int = 6, seed: int = 0) -> bytes:
    """samples: (H, W, channels) integer samples at `depth`."""
    rng = np.random.default_rng(seed)
    H, W = samples.shape[:2]
    ch = CHANNELS[ctype]
    bpp = max(1, ch * depth // 8)
    raw = bytearray()
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    for x0, y0, dx, dy in passes:
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        raw += filter_rows([pack_row(sub[y], depth) for y in range(sub.shape[0])], bpp, rng)
    out = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", W, H, depth, ctype, 0, 0, interlace))
    if palette is not None:
        out += chunk(b"PLTE", np.asarray(palette, np.uint8).tobytes())
    if trns is not None:
        out += chunk(b"tRNS", trns)
    out += chunk(b"tEXt", b"Comment\x00ancillary chunks are skipped")
    comp = zlib.compress(bytes(raw), level)
    # split the image data over several IDAT chunks
    for k in range(0, len(comp), 997):
        out += chunk(b"IDAT", comp[k:k + 997])
    return out + chunk(b"IEND", b"")


def expected_rgba(samples: np.ndarray, ctype: int, depth: int, palette=None, trns=None) -> np.ndarray:
    """The RGBA8 conversion stbi_load(..., 4) applies."""
    s = samples.astype(np.uint32)
    H, W = s.shape[:2]
    out = np.zeros((H, W, 4), np.uint8)

    def to8(v):
        if depth == 16:
            return (v >> 8).astype(np.uint8)
        if depth == 8:
            return v.astype(np.uint8)
        return (v * (255 // ((1 << depth) - 1))).astype(np.uint8)

    if ctype == 3:
        pal = np.asarray(palette, np.uint8).reshape(-1, 3)
        alpha = np.full(len(pal), 255, np.uint8)
        if trns is not None:
            alpha[:len(trns)] = np.frombuffer(trns, np.uint8)
        out[..., :3] = pal[s[..., 0]]
        out[..., 3] = alpha[s[..., 0]]
        return out
    if ctype in (0, 4):
        g = to8(s[..., 0])
        out[..., 0] = out[..., 1] = out[..., 2] = g
        out[..., 3] = to8(s[..., 1]) if ctype == 4 else 255
    else:
        for c in range(ctype == 6 and 4 or 3):
            out[..., c] = to8(s[..., c])
        if ctype == 2:
            out[..., 3] = 255
    if trns is not None and ctype in (0, 2):
        key = np.frombuffer(trns, ">u2").astype(np.uint32)
        hit = np.all(s[..., :len(key)] == key, axis=-1)
        out[..., 3][hit] = 0
    return out


CASES = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8), (4, 8), (4, 16),
         (6, 8), (6, 16)]


@pytest.mark.parametrize("ctype,depth", CASES)
@pytest.mark.parametrize("interlace", [0, 1])
def test_png_decode_matches_restatement(R, ctype, depth, interlace):
    rng = np.random.default_rng(ctype * 100 + depth + 7 * interlace)
    H, W = (int(rng.integers(1, 40)), int(rng.integers(1, 40)))
    ch = CHANNELS[ctype]
    top = (1 << depth) - 1
    palette = trns = None
    if ctype == 3:
        n = int(rng.integers(1, (1 << depth) + 1))
        palette = rng.integers(0, 256, (n, 3))
        samples = rng.integers(0, n, (H, W, 1))
        trns = rng.integers(0, 256, int(rng.integers(0, n + 1))).astype(np.uint8).tobytes() or None
    else:
        samples = rng.integers(0, top + 1, (H, W, ch))
        if ctype in (0, 2) and rng.uniform() < 0.7:
            key = samples[0, 0, :ch]   # a key colour that occurs
            trns = np.asarray(key, ">u2").tobytes()
    for level in (0, 1, 9):
        data = encode_png(samples, ctype, depth, interlace, palette, trns, level, seed=level)
        got = R.decode_image(data)
        want = expected_rgba(samples, ctype, depth, palette, trns)
        assert got.shape == want.shape
        assert np.array_equal(got, want), (ctype, depth, interlace, level)


def test_png_large_dynamic_blocks(R):
    """A 300x200 RGBA image with long runs and noise: dynamic Huffman blocks with long codes and
    back-references across rows, at every compression level."""
    rng = np.random.default_rng(3)
    img = np.zeros((200, 300, 4), np.int64)
    img[..., 0] = (np.arange(300)[None, :] // 7) % 256
    img[..., 1] = rng.integers(0, 256, (200, 300))
    img[..., 2] = (np.arange(200)[:, None] * 3) % 256
    img[..., 3] = np.where(rng.uniform(size=(200, 300)) < 0.9, 255, rng.integers(0, 256, (200, 300)))
    for level in range(10):
        got = R.decode_image(encode_png(img, 6, 8, 0, level=level, seed=level))
        assert np.array_equal(got, img.astype(np.uint8)), level


def numpy_png_decode(data: bytes) -> np.ndarray:
    """Independent decode of a non-interlaced 8-bit PNG (colour types 2, 3 at depth <= 8, 6) with Python's
    zlib, for the reference's texture files."""
    p = 8
    idat = b""
    pal = trns = None
    while p < len(data):
        n = struct.unpack(">I", data[p:p + 4])[0]
        t = data[p + 4:p + 8]
        d = data[p + 8:p + 8 + n]
        if t == b"IHDR":
            W, H, depth, ctype, _, _, il = struct.unpack(">IIBBBBB", d)
        elif t == b"PLTE":
            pal = np.frombuffer(d, np.uint8).reshape(-1, 3)
        elif t == b"tRNS":
            trns = d
        elif t == b"IDAT":
            idat += d
        p += 12 + n
    assert il == 0
    raw = np.frombuffer(zlib.decompress(idat), np.uint8)
    ch = CHANNELS[ctype]
    stride = (W * ch * depth + 7) // 8
    bpp = max(1, ch * depth // 8)
    rows = raw.reshape(H, stride + 1)
    out = np.zeros((H, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    for y in range(H):
        ft, cur = rows[y, 0], rows[y, 1:].astype(np.int32)
        if ft == 0:
            rec = cur
        elif ft == 2:
            rec = (cur + prev) & 255
        else:
            rec = np.zeros(stride, np.int32)
            for i in range(stride):
                a = rec[i - bpp] if i >= bpp else 0
                b = prev[i]
                c = prev[i - bpp] if i >= bpp else 0
                if ft == 1:
                    pr = a
                elif ft == 3:
                    pr = (a + b) >> 1
                else:
                    q = a + b - c
                    pa, pb, pc = abs(q - a), abs(q - b), abs(q - c)
                    pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                rec[i] = (cur[i] + pr) & 255
        out[y] = rec
        prev = rec
    if depth < 8:
        per = 8 // depth
        bits = np.stack([(out >> (8 - depth * (k + 1))) & ((1 << depth) - 1) for k in range(per)], -1)
        samples = bits.reshape(H, -1)[:, :W * ch].reshape(H, W, ch)
    else:
        samples = out.reshape(H, W, ch)
    return expected_rgba(samples, ctype, depth, pal, trns)


@pytest.mark.skipif(REF_TEXTURES is None, reason="REINA_REFERENCE_DIR unset or without textures/")
@pytest.mark.parametrize("name", ["toybox/diffuse.png", "toybox/parallax.png", "bricks2/normal.png",
                                  "cornell_texture.png", "brick_normal.png"])
def test_png_reference_textures(R, name):
    data = (REF_TEXTURES / name).read_bytes()
    assert np.array_equal(R.decode_image(data), numpy_png_decode(data))


def test_png_malformed_inputs(R):
    good = encode_png(np.zeros((4, 4, 3), np.int64), 2, 8)
    bad = [
        b"",
        good[:8],
        good[:40],                                   # truncated inside IDAT
        good.replace(b"IHDR", b"IHDX", 1),           # unknown critical chunk first
        b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", 4, 4, 3, 2, 0, 0, 0)) + chunk(b"IEND", b""),
        b"\xff\xd8\xff\xe0 not decoded",             # JPEG
        b"GIF89a",
    ]
    # corrupt deflate data: flip bits in the middle of the zlib stream
    i = good.index(b"IDAT") + 8
    corrupt = bytearray(good)
    corrupt[i] ^= 0xFF
    bad.append(bytes(corrupt))
    for k, d in enumerate(bad):
        with pytest.raises(R.ReinaError) as e:
            R.decode_image(d)
        assert e.value.code == R.REINA_ERR_IO, k


def test_texture_ids_checked_at_build(R):
    ctx = R.Context(-1)
    v, i = scenes.quad((0, 0, 0), (1, 0, 0), (0, 1, 0))
    s = R.Scene(ctx)
    s.add_object(v, i, material=R.Material(texture_id=0))
    with pytest.raises(R.ReinaError) as e:
        s.build()
    assert e.value.code == R.REINA_ERR_INVALID
    s2 = R.Scene(ctx)
    s2.add_object(v, i, material=R.Material(texture_id=0, normal_map_id=1, bump_map_id=0))
    assert s2.define_texture_rgba8(np.zeros((2, 3, 4), np.uint8)) == 0
    assert s2.define_texture_encoded(encode_png(np.zeros((5, 7, 4), np.int64), 6, 8)) == 1
    assert s2.texture_count() == 2
    s2.build()
    with pytest.raises(R.ReinaError):
        s2.define_texture_rgba8(np.zeros((2, 2, 4), np.uint8))   # built
    with pytest.raises(R.ReinaError) as e:
        R.Scene(ctx).define_texture(Path("/nonexistent/texture.png"))
    assert e.value.code == R.REINA_ERR_IO
    ctx.close()


def test_texture_sources_and_flip(R, tmp_path):
    """A file is loaded with its rows flipped (stbi_set_flip_vertically_on_load(true) for paths); encoded
    bytes and raw texels are kept as given."""
    ctx = R.Context(-1)
    rng = np.random.default_rng(11)
    img = rng.integers(0, 256, (5, 7, 4))
    data = encode_png(img, 6, 8)
    p = tmp_path / "t.png"
    p.write_bytes(data)
    s = R.Scene(ctx)
    assert s.define_texture(p) == 0
    assert s.define_texture_encoded(data) == 1
    assert s.define_texture_rgba8(img.astype(np.uint8)) == 2
    assert np.array_equal(s.export_texture(0), img[::-1].astype(np.uint8))
    assert np.array_equal(s.export_texture(1), img.astype(np.uint8))
    assert np.array_equal(s.export_texture(2), img.astype(np.uint8))
    with pytest.raises(R.ReinaError):
        s.export_texture(3)
    ctx.close()
