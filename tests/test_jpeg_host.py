"""JPEG texture decoding on the host: the test encodes seeded images as sequential (baseline) JPEG itself —
its own forward DCT, quantization tables and Huffman tables built from the symbol frequencies, every
chroma subsampling the decoder handles, restart intervals, single- and multi-scan files — and checks
the library's decoding against the reconstruction of the coefficients it wrote (dequantization, the 8x8
inverse DCT, the triangle-filter chroma upsampling and the JFIF YCbCr -> RGB conversion, restated in
numpy), plus the reference's own JPEG textures when they are present.  The same coefficients are also
written as progressive JPEG (spectral selection and successive approximation) and must decode to the
sequential file's pixels exactly."""
import heapq
import struct
from pathlib import Path

import numpy as np
import pytest
from conftest import reference_dir

REF_TEXTURES = reference_dir("textures")

ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13,
                   6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52, 45,
                   38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])

_u = np.arange(8)
COS = np.cos((2 * _u[:, None] + 1) * _u[None, :] * np.pi / 16) * np.where(_u == 0, np.sqrt(0.5), 1.0)[None, :]


def fdct(block):   # 8x8 forward DCT (T.81 A.3.3)
    return COS.T @ block @ COS / 4.0


def idct(F):
    return COS @ F @ COS.T / 4.0


def huff_lengths(freq: dict) -> dict:
    """Code lengths (<= 16) for the symbols of `freq`, with one reserved longest code (never all ones)."""
    f = dict(freq)
    while True:
        items = [(c, i, [s]) for i, (s, c) in enumerate(sorted(f.items()))] + [(1, -1, [256])]
        heapq.heapify(items)
        depth = {s: 0 for _, _, ss in items for s in ss}
        k = len(items)
        while len(items) > 1:
            a, b = heapq.heappop(items), heapq.heappop(items)
            for s in a[2] + b[2]:
                depth[s] += 1
            k += 1
            heapq.heappush(items, (a[0] + b[0], k, a[2] + b[2]))
        if max(depth.values()) <= 16:
            depth.pop(256)
            return depth
        f = {s: (c + 1) // 2 for s, c in f.items()}


def canonical(lengths: dict):
    """(counts per length 1..16, symbols in code order, code table symbol -> (code, length))."""
    order = sorted(lengths, key=lambda s: (lengths[s], s))
    counts = [0] * 17
    for s in order:
        counts[lengths[s]] += 1
    codes, code, prev = {}, 0, 0
    for s in order:
        code <<= lengths[s] - prev
        prev = lengths[s]
        codes[s] = (code, lengths[s])
        code += 1
    return counts[1:], order, codes


class BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, v, n):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((v >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = self.n = 0

    def flush(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)


def category(v):
    return 0 if v == 0 else int(abs(v)).bit_length()


def bits_of(v, c):
    return v if v >= 0 else v + (1 << c) - 1


def encode_jpeg(rgb, sampling=((2, 2), (1, 1), (1, 1)), gray=False, restart=0, scans="interleaved", quality_step=1,
                seed=0):
    """Returns (file bytes, per-component quantized coefficient blocks, quant tables, component layout)."""
    rng = np.random.default_rng(seed)
    H, W = rgb.shape[:2]
    x = rgb.astype(np.float64)
    if gray:
        planes = [0.299 * x[..., 0] + 0.587 * x[..., 1] + 0.114 * x[..., 2]]
        sampling = ((1, 1),)
    else:
        Y = 0.299 * x[..., 0] + 0.587 * x[..., 1] + 0.114 * x[..., 2]
        Cb = -0.168736 * x[..., 0] - 0.331264 * x[..., 1] + 0.5 * x[..., 2] + 128
        Cr = 0.5 * x[..., 0] - 0.418688 * x[..., 1] - 0.081312 * x[..., 2] + 128
        planes = [Y, Cb, Cr]
    hmax = max(h for h, _ in sampling)
    vmax = max(v for _, v in sampling)
    mcux, mcuy = -(-W // (8 * hmax)), -(-H // (8 * vmax))
    qts = [np.clip(1 + quality_step * (np.arange(64) // 3) + rng.integers(0, 3, 64), 1, 255).astype(np.int64)
           for _ in range(2)]
    comps = []
    for ci, (p, (h, v)) in enumerate(zip(planes, sampling)):
        sx, sy = hmax // h, vmax // v
        cw, ch = -(-W // sx), -(-H // sy)
        # subsample by averaging, pad by edge replication to whole MCUs
        pp = np.pad(p, ((0, (-H) % sy), (0, (-W) % sx)), mode="edge")
        sub = pp.reshape(pp.shape[0] // sy, sy, pp.shape[1] // sx, sx).mean(axis=(1, 3))[:ch, :cw]
        bw, bh = mcux * h, mcuy * v
        full = np.pad(sub, ((0, bh * 8 - ch), (0, bw * 8 - cw)), mode="edge")
        q = qts[0 if ci == 0 else 1]
        blocks = np.zeros((bh, bw, 64), np.int64)
        for by in range(bh):
            for bx in range(bw):
                F = fdct(full[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] - 128.0).reshape(64)[ZIGZAG]
                blocks[by, bx] = np.round(F / q).astype(np.int64)
        comps.append(dict(id=ci + 1, h=h, v=v, tq=0 if ci == 0 else 1, blocks=blocks, cw=cw, ch=ch, bw=bw, bh=bh))

    def units(scan_comps):
        """Blocks of a scan in coding order: (component index, block x, block y, mcu index)."""
        out = []
        if len(scan_comps) == 1:
            c = comps[scan_comps[0]]
            ux, uy = -(-c["cw"] // 8), -(-c["ch"] // 8)
            for by in range(uy):
                for bx in range(ux):
                    out.append((scan_comps[0], bx, by, by * ux + bx))
        else:
            for my in range(mcuy):
                for mx in range(mcux):
                    for ci in scan_comps:
                        c = comps[ci]
                        for vv in range(c["v"]):
                            for hh in range(c["h"]):
                                out.append((ci, mx * c["h"] + hh, my * c["v"] + vv, my * mcux + mx))
        return out

    scan_list = [list(range(len(comps)))] if scans == "interleaved" else [[c] for c in range(len(comps))]
    seg = bytearray(b"\xff\xd8")
    seg += b"\xff\xe0" + struct.pack(">H", 16) + b"JFIF\x00\x01\x01\x00\x00\x01\x00\x01\x00\x00"
    for t, q in enumerate(qts[: 1 if gray else 2]):
        seg += b"\xff\xdb" + struct.pack(">HB", 67, t) + bytes(q.astype(np.uint8))
    seg += b"\xff\xc0" + struct.pack(">HBHHB", 8 + 3 * len(comps), 8, H, W, len(comps))
    for c in comps:
        seg += bytes([c["id"], c["h"] << 4 | c["v"], c["tq"]])
    if restart:
        seg += b"\xff\xdd" + struct.pack(">HH", 4, restart)
    for sc in scan_list:
        # symbols of this scan for the frequency-built tables (DC table per component class, AC likewise)
        seq = units(sc)
        syms = []
        preds = {ci: 0 for ci in sc}
        last_mcu = -1
        n_mcu = 0
        for ci, bx, by, mcu in seq:
            if mcu != last_mcu:
                if restart and n_mcu and n_mcu % restart == 0:
                    preds = {c: 0 for c in sc}
                    syms.append(("RST", None, None))
                last_mcu = mcu
                n_mcu += 1
            blk = comps[ci]["blocks"][by, bx]
            diff = int(blk[0]) - preds[ci]
            preds[ci] = int(blk[0])
            cls = 0 if ci == 0 else 1
            syms.append(("DC", cls, (category(diff), diff)))
            run = 0
            last_nz = max([k for k in range(1, 64) if blk[k] != 0], default=0)
            for k in range(1, last_nz + 1):
                if blk[k] == 0:
                    run += 1
                    continue
                while run > 15:
                    syms.append(("AC", cls, (0xF0, None)))
                    run -= 16
                c = category(int(blk[k]))
                syms.append(("AC", cls, ((run << 4) | c, int(blk[k]))))
                run = 0
            if last_nz < 63:
                syms.append(("AC", cls, (0x00, None)))
        tables = {}
        for kind in ("DC", "AC"):
            for cls in (0, 1):
                freq = {}
                for k, c, v in syms:
                    if k == kind and c == cls:
                        freq[v[0]] = freq.get(v[0], 0) + 1
                if freq:
                    tables[(kind, cls)] = canonical(huff_lengths(freq))
        for (kind, cls), (counts, order, _) in tables.items():
            tc = 0 if kind == "DC" else 1
            seg += b"\xff\xc4" + struct.pack(">HB", 2 + 1 + 16 + len(order), tc << 4 | cls) + bytes(counts) + bytes(order)
        seg += b"\xff\xda" + struct.pack(">HB", 6 + 2 * len(sc), len(sc))
        for ci in sc:
            cls = 0 if ci == 0 else 1
            seg += bytes([comps[ci]["id"], cls << 4 | cls])
        seg += bytes([0, 63, 0])
        bw = BitWriter()
        rst = 0
        for kind, cls, v in syms:
            if kind == "RST":
                bw.flush()
                seg += bw.out
                bw = BitWriter()
                seg += bytes([0xFF, 0xD0 + rst])
                rst = (rst + 1) % 8
                continue
            code, n = tables[(kind, cls)][2][v[0]]
            bw.put(code, n)
            if kind == "DC":
                if v[0]:
                    bw.put(bits_of(v[1], v[0]), v[0])
            elif v[1] is not None:
                bw.put(bits_of(v[1], v[0] & 15), v[0] & 15)
        bw.flush()
        seg += bw.out
    seg += b"\xff\xd9"
    return bytes(seg), comps, qts, (hmax, vmax, mcux, mcuy)


def reconstruct(comps, qts, layout, W, H, gray):
    """The decoder's definitions restated: dequantize, IDCT (double), level shift, round, clamp; 2:1
    triangle-filter upsampling (replication otherwise); JFIF YCbCr -> RGB with rounding."""
    hmax, vmax, mcux, mcuy = layout
    fw, fh = mcux * hmax * 8, mcuy * vmax * 8
    full = []
    for c in comps:
        q = qts[c["tq"]]
        plane = np.zeros((c["bh"] * 8, c["bw"] * 8), np.int64)
        for by in range(c["bh"]):
            for bx in range(c["bw"]):
                F = np.zeros(64)
                F[ZIGZAG] = c["blocks"][by, bx] * q
                f = np.floor(idct(F.reshape(8, 8)) + 128.0 + 0.5)
                plane[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] = np.clip(f, 0, 255)
        sx, sy = hmax // c["h"], vmax // c["v"]
        if sx == 1 and sy == 1:
            full.append(plane)
            continue
        if sx > 2 or sy > 2:   # replication
            ys, xs = np.arange(fh) // sy, np.arange(fw) // sx
            full.append(plane[np.minimum(ys, plane.shape[0] - 1)[:, None], np.minimum(xs, plane.shape[1] - 1)[None, :]])
            continue
        uw = max(1, min(plane.shape[1], -(-(W * c["h"]) // hmax)))
        uh = max(1, min(plane.shape[0], -(-(H * c["v"]) // vmax)))
        ys, xs = np.arange(fh), np.arange(fw)
        yc = ys // sy if sy == 2 else ys
        xc = xs // sx if sx == 2 else xs
        yf = np.where(ys % 2 == 1, yc + 1, yc - 1) if sy == 2 else yc
        xf = np.where(xs % 2 == 1, xc + 1, xc - 1) if sx == 2 else xc
        S = lambda yy, xx: plane[np.clip(yy, 0, uh - 1)[:, None], np.clip(xx, 0, uw - 1)[None, :]]
        if sx == 2 and sy == 2:
            out = (3 * (3 * S(yc, xc) + S(yf, xc)) + (3 * S(yc, xf) + S(yf, xf)) + 8) >> 4
        elif sx == 2:
            out = (3 * S(yc, xc) + S(yc, xf) + 2) >> 2
        else:
            out = (3 * S(yc, xc) + S(yf, xc) + 2) >> 2
        full.append(out)
    rgba = np.full((H, W, 4), 255, np.uint8)
    if gray:
        rgba[..., :3] = full[0][:H, :W, None]
        return rgba
    Y, cb, cr = (p[:H, :W].astype(np.float64) for p in full)
    cb, cr = cb - 128.0, cr - 128.0
    q = lambda v: np.clip(np.floor(v + 0.5), 0, 255).astype(np.uint8)
    rgba[..., 0] = q(Y + 1.402 * cr)
    rgba[..., 1] = q(Y - 0.344136 * cb - 0.714136 * cr)
    rgba[..., 2] = q(Y + 1.772 * cb)
    return rgba


def sample_image(H, W, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:H, 0:W]
    img = np.stack([128 + 100 * np.sin(x / 7.0 + seed), 128 + 90 * np.cos(y / 5.0), (x * 3 + y * 2) % 256], -1)
    img += rng.normal(0, 12, img.shape)
    return np.clip(img, 0, 255).astype(np.uint8)


CASES = [
    dict(sampling=((1, 1), (1, 1), (1, 1))),                 # 4:4:4
    dict(sampling=((2, 1), (1, 1), (1, 1))),                 # 4:2:2
    dict(sampling=((2, 2), (1, 1), (1, 1))),                 # 4:2:0
    dict(sampling=((1, 2), (1, 1), (1, 1))),                 # 4:4:0
    dict(sampling=((4, 1), (1, 1), (1, 1))),                 # 4:1:1 (replicated chroma)
    dict(sampling=((2, 2), (1, 1), (1, 1)), restart=3),
    dict(sampling=((2, 2), (1, 1), (1, 1)), scans="separate"),
    dict(sampling=((1, 1), (1, 1), (1, 1)), scans="separate", restart=5),
    dict(gray=True),
    dict(gray=True, restart=1),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_jpeg_decode_matches_restatement(R, case):
    kw = CASES[case]
    for seed, (H, W) in enumerate([(37, 53), (64, 64), (8, 9), (1, 17)]):
        img = sample_image(H, W, seed + 10 * case)
        data, comps, qts, layout = encode_jpeg(img, seed=seed, **kw)
        got = R.decode_image(data)
        want = reconstruct(comps, qts, layout, W, H, kw.get("gray", False))
        assert got.shape == want.shape
        d = np.abs(got.astype(np.int64) - want.astype(np.int64))
        # the library sums the IDCT in another order: a value on a rounding boundary may move by one
        assert d.max() <= 1 and (d == 0).mean() >= 0.999, (case, seed, d.max(), (d == 0).mean())
        if not kw.get("gray"):
            err = np.abs(got[..., :3].astype(np.int64) - img.astype(np.int64))
            assert err.mean() < 12   # a lossy round trip, not a different image


def test_jpeg_malformed_and_unsupported(R):
    img = sample_image(16, 16, 1)
    data = encode_jpeg(img)[0]
    prog = data.replace(b"\xff\xc0", b"\xff\xc2", 1)   # progressive frame marker
    cut = data[: len(data) // 2]
    for bad in (prog, cut, data[:4] + b"\xff\xd9", b"\xff\xd8\xff\xc0\x00\x0b\x0c\x00\x10\x00\x10\x01\x01\x11\x00\xff\xd9"):
        with pytest.raises(R.ReinaError) as e:
            R.decode_image(bad)
        assert e.value.code == R.REINA_ERR_IO


@pytest.mark.skipif(REF_TEXTURES is None, reason="REINA_REFERENCE_DIR unset or without textures/")
def test_jpeg_reference_textures(R):
    """The reference's JPEG textures decode; the tangent-space normal map points mostly along +z."""
    alb = R.decode_image((REF_TEXTURES / "qgdpH_2K_Albedo.jpg").read_bytes())
    nrm = R.decode_image((REF_TEXTURES / "qgdpH_2K_Normal.jpg").read_bytes())
    assert alb.shape == (2048, 2048, 4) and nrm.shape == (2048, 2048, 4)
    assert nrm[..., 2].mean() > 240 and abs(nrm[..., 0].mean() - 128) < 8 and abs(nrm[..., 1].mean() - 128) < 8
    assert alb[..., 1].mean() > alb[..., 2].mean()   # a green-dominated albedo


# ------------------------------------------------------------------------------------------------
# Progressive JPEG (T.81 Annex G): the same quantized coefficients written as progressive scans —
# spectral selection (DC, then AC bands of one component each) and successive approximation (a first
# scan at a reduced bit level, then one refinement scan per bit), with end-of-band runs, zero-run
# codes, correction bits and restart intervals — must decode to exactly the pixels of the sequential
# file.

def units_of(comps, layout, scan_comps):
    """Blocks of a scan in coding order: (component index, block x, block y, mcu index)."""
    hmax, vmax, mcux, mcuy = layout
    out = []
    if len(scan_comps) == 1:
        c = comps[scan_comps[0]]
        ux, uy = -(-c["cw"] // 8), -(-c["ch"] // 8)
        for by in range(uy):
            for bx in range(ux):
                out.append((scan_comps[0], bx, by, by * ux + bx))
    else:
        for my in range(mcuy):
            for mx in range(mcux):
                for ci in scan_comps:
                    c = comps[ci]
                    for vv in range(c["v"]):
                        for hh in range(c["h"]):
                            out.append((ci, mx * c["h"] + hh, my * c["v"] + vv, my * mcux + mx))
    return out


def ac_point(v, al):   # AC point transform: magnitude shifted, sign kept (division toward zero)
    return -((-v) >> al) if v < 0 else v >> al


def progressive_events(comps, layout, sc, ss, se, ah, al, restart):
    """One scan as a list of ("S", kind, class, symbol) / ("B", value, nbits) / ("R",) events."""
    ev = []
    acls = 0 if sc[0] == 0 else 1
    st = {"eobrun": 0, "be": []}

    def flush_eob():
        n = st["eobrun"]
        if n:
            r = n.bit_length() - 1
            ev.append(("S", "AC", acls, r << 4))
            if r:
                ev.append(("B", n - (1 << r), r))
            ev.extend(("B", b, 1) for b in st["be"])
            st["eobrun"], st["be"] = 0, []

    preds = {ci: 0 for ci in sc}
    last_mcu, n_mcu = -1, 0
    for ci, bx, by, mcu in units_of(comps, layout, sc):
        cls = 0 if ci == 0 else 1
        if mcu != last_mcu:
            if restart and n_mcu and n_mcu % restart == 0:
                flush_eob()
                ev.append(("R",))
                preds = {c: 0 for c in sc}
            last_mcu, n_mcu = mcu, n_mcu + 1
        blk = comps[ci]["blocks"][by, bx]
        if ss == 0:
            if ah == 0:
                v = int(blk[0]) >> al
                diff, preds[ci] = v - preds[ci], v
                cat = category(diff)
                ev.append(("S", "DC", cls, cat))
                if cat:
                    ev.append(("B", bits_of(diff, cat), cat))
            else:
                ev.append(("B", (int(blk[0]) >> al) & 1, 1))
            continue
        band = [int(blk[k]) for k in range(ss, se + 1)]
        if ah == 0:   # first scan of the band
            vals = [ac_point(v, al) for v in band]
            nz = [i for i, v in enumerate(vals) if v]
            if nz:
                flush_eob()
                run = 0
                for i in range(nz[-1] + 1):
                    if vals[i] == 0:
                        run += 1
                        continue
                    while run > 15:
                        ev.append(("S", "AC", cls, 0xF0))
                        run -= 16
                    cat = category(vals[i])
                    ev.append(("S", "AC", cls, (run << 4) | cat))
                    ev.append(("B", bits_of(vals[i], cat), cat))
                    run = 0
            if not nz or nz[-1] < len(vals) - 1:
                st["eobrun"] += 1
                if st["eobrun"] == 0x7FFF:
                    flush_eob()
            continue
        # refinement: one more bit of every coefficient of the band
        absv = [abs(v) >> al for v in band]
        news = [i for i, a in enumerate(absv) if a == 1]
        last_new = news[-1] if news else -1
        run, br = 0, []
        for i, a in enumerate(absv):
            if a == 0:
                run += 1
                continue
            while run > 15 and i <= last_new:
                flush_eob()
                ev.append(("S", "AC", cls, 0xF0))
                run -= 16
                ev.extend(("B", b, 1) for b in br)
                br = []
            if a > 1:   # already nonzero: a correction bit
                br.append(a & 1)
                continue
            flush_eob()
            ev.append(("S", "AC", cls, (run << 4) | 1))
            ev.append(("B", 0 if band[i] < 0 else 1, 1))
            ev.extend(("B", b, 1) for b in br)
            run, br = 0, []
        if run > 0 or br:
            st["eobrun"] += 1
            st["be"] += br
            if st["eobrun"] == 0x7FFF or len(st["be"]) > 900:
                flush_eob()
    flush_eob()
    return ev


SCRIPT_SA = ("dc:0:1", "ac:1:5:0:2", "ac:6:63:0:1", "dc:1:0", "ac:1:5:2:1", "ac:1:5:1:0", "ac:6:63:1:0")
SCRIPT_SPECTRAL = ("dc:0:0", "ac:1:2:0:0", "ac:3:20:0:0", "ac:21:63:0:0")


def encode_progressive(comps, qts, layout, H, W, gray, restart=0, script=SCRIPT_SA):
    """The coefficients of `comps` as a progressive JPEG (SOF2) following `script`."""
    seg = bytearray(b"\xff\xd8")
    for t, q in enumerate(qts[: 1 if gray else 2]):
        seg += b"\xff\xdb" + struct.pack(">HB", 67, t) + bytes(q.astype(np.uint8))
    seg += b"\xff\xc2" + struct.pack(">HBHHB", 8 + 3 * len(comps), 8, H, W, len(comps))
    for c in comps:
        seg += bytes([c["id"], c["h"] << 4 | c["v"], c["tq"]])
    if restart:
        seg += b"\xff\xdd" + struct.pack(">HH", 4, restart)
    scans = []
    for item in script:
        f = item.split(":")
        if f[0] == "dc":
            scans.append((list(range(len(comps))), 0, 0, int(f[1]), int(f[2])))
        else:
            for ci in range(len(comps)):
                scans.append(([ci], int(f[1]), int(f[2]), int(f[3]), int(f[4])))
    for sc, ss, se, ah, al in scans:
        ev = progressive_events(comps, layout, sc, ss, se, ah, al, restart)
        tables = {}
        for kind in ("DC", "AC"):
            for cls in (0, 1):
                freq = {}
                for e in ev:
                    if e[0] == "S" and e[1] == kind and e[2] == cls:
                        freq[e[3]] = freq.get(e[3], 0) + 1
                if freq:
                    tables[(kind, cls)] = canonical(huff_lengths(freq))
        for (kind, cls), (counts, order, _) in tables.items():
            tc = 0 if kind == "DC" else 1
            seg += b"\xff\xc4" + struct.pack(">HB", 2 + 1 + 16 + len(order), tc << 4 | cls) + bytes(counts) + bytes(order)
        seg += b"\xff\xda" + struct.pack(">HB", 6 + 2 * len(sc), len(sc))
        for ci in sc:
            cls = 0 if ci == 0 else 1
            seg += bytes([comps[ci]["id"], cls << 4 | cls])
        seg += bytes([ss, se, ah << 4 | al])
        bw = BitWriter()
        rst = 0
        for e in ev:
            if e[0] == "R":
                bw.flush()
                seg += bw.out
                bw = BitWriter()
                seg += bytes([0xFF, 0xD0 + rst])
                rst = (rst + 1) % 8
            elif e[0] == "S":
                code, n = tables[(e[1], e[2])][2][e[3]]
                bw.put(code, n)
            else:
                bw.put(e[1], e[2])
        bw.flush()
        seg += bw.out
    seg += b"\xff\xd9"
    return bytes(seg)


PROGRESSIVE_CASES = [
    dict(gray=True),
    dict(sampling=((2, 2), (1, 1), (1, 1))),
    dict(sampling=((1, 1), (1, 1), (1, 1)), restart=2),
    dict(sampling=((2, 1), (1, 1), (1, 1)), script=SCRIPT_SPECTRAL),
    dict(gray=True, restart=1, script=SCRIPT_SPECTRAL),
]


@pytest.mark.parametrize("case", range(len(PROGRESSIVE_CASES)))
def test_progressive_jpeg_equals_sequential(R, case):
    kw = dict(PROGRESSIVE_CASES[case])
    script = kw.pop("script", SCRIPT_SA)
    restart = kw.get("restart", 0)
    gray = kw.get("gray", False)
    for seed, (H, W) in enumerate([(37, 53), (64, 64), (8, 9), (1, 17), (96, 40)]):
        img = sample_image(H, W, seed + 7 * case)
        # quality_step 0: fine quantization, so many coefficients are large (several refinement bits)
        data, comps, qts, layout = encode_jpeg(img, seed=seed, quality_step=0, **kw)
        prog = encode_progressive(comps, qts, layout, H, W, gray, restart=restart, script=script)
        assert prog[2:] != data[2:] and b"\xff\xc2" in prog
        assert np.array_equal(R.decode_image(prog), R.decode_image(data)), (case, seed)


def test_progressive_jpeg_refinements_matter(R):
    """Leaving out any refinement scan (AC high band, AC low band, DC) changes the decoded pixels: the
    refinement paths of the decoder are exercised, not bypassed."""
    img = sample_image(64, 64, 3)
    data, comps, qts, layout = encode_jpeg(img, seed=1, quality_step=0, sampling=((2, 2), (1, 1), (1, 1)))
    full = R.decode_image(data)
    for drop in ("ac:6:63:1:0", "ac:1:5:1:0", "dc:1:0"):
        script = tuple(s for s in SCRIPT_SA if s != drop)
        got = R.decode_image(encode_progressive(comps, qts, layout, 64, 64, False, script=script))
        assert not np.array_equal(got, full), drop
