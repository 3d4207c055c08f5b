// PNG decoding (PNG specification, ISO/IEC 15948) over an RFC 1950/1951 inflater, producing the RGBA8
// texels the reference gets from stbi_load(..., 4) (src/graphics/Image.cpp:15, 29-33).
#include "image.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>

#include "errors.h"

namespace rt {

namespace {

[[noreturn]] void bad(const std::string& what) { fail(REINA_ERR_IO, what); }

// ---- inflate -------------------------------------------------------------------------------------

class Bits {
public:
    Bits(const uint8_t* p, size_t n) : p_(p), n_(n) {}
    // Tops the bit buffer up to at least 57 bits (zeros past the end of the input; real_ counts the rest).
    void fill() {
        while (cnt_ <= 56) {
            const uint64_t b = pos_ < n_ ? p_[pos_] : 0u;
            if (pos_ < n_) real_ += 8;
            ++pos_;
            buf_ |= b << cnt_;
            cnt_ += 8;
        }
    }
    uint32_t peek(int k) {
        if (cnt_ < k) fill();
        return (uint32_t)(buf_ & ((1ull << k) - 1ull));
    }
    void drop(int k) {
        if (k > real_) bad("truncated deflate stream");
        buf_ >>= k;
        cnt_ -= k;
        real_ -= k;
    }
    uint32_t get(int k) {
        if (k == 0) return 0;
        const uint32_t v = peek(k);
        drop(k);
        return v;
    }
    void align() {
        const int k = cnt_ & 7;
        buf_ >>= k;
        cnt_ -= k;
        real_ = std::max(0, real_ - k);
    }
    // Byte-aligned input position (after align()).
    size_t byte_pos() const { return pos_ - (size_t)(cnt_ / 8); }
    void skip_to(size_t byte) {
        pos_ = byte;
        buf_ = 0;
        cnt_ = 0;
        real_ = 0;
    }
    size_t size() const { return n_; }
    const uint8_t* data() const { return p_; }

private:
    const uint8_t* p_;
    size_t n_;
    size_t pos_ = 0;
    uint64_t buf_ = 0;
    int cnt_ = 0;    // bits in buf_
    int real_ = 0;   // of which come from the input
};

// Canonical Huffman code: a 9-bit direct table for short codes plus the per-length walk for longer ones.
class Huffman {
public:
    static constexpr int kFast = 9;
    void build(const uint8_t* lengths, int n) {
        std::memset(count_, 0, sizeof(count_));
        for (int s = 0; s < n; ++s) count_[lengths[s]]++;
        count_[0] = 0;
        int left = 1;
        for (int l = 1; l <= 15; ++l) {
            left = left * 2 - count_[l];
            if (left < 0) bad("over-subscribed Huffman code");
        }
        int offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + count_[l];
        sym_.assign((size_t)n, 0);
        for (int s = 0; s < n; ++s)
            if (lengths[s]) sym_[(size_t)offs[lengths[s]]++] = (uint16_t)s;
        // direct table: canonical codes assigned in (length, symbol) order, stored bit-reversed
        std::fill(std::begin(fast_), std::end(fast_), (uint16_t)0);
        int code = 0, idx = 0;
        for (int l = 1; l <= kFast; ++l) {
            for (int k = 0; k < count_[l]; ++k, ++idx, ++code) {
                int rev = 0;
                for (int b = 0; b < l; ++b) rev |= ((code >> b) & 1) << (l - 1 - b);
                for (int fill = rev; fill < (1 << kFast); fill += 1 << l)
                    fast_[fill] = (uint16_t)((sym_[(size_t)idx] << 4) | l);
            }
            code <<= 1;
        }
    }
    int decode(Bits& in) const {
        const uint16_t e = fast_[in.peek(kFast)];
        if (e) {
            in.drop(e & 15);
            return e >> 4;
        }
        int code = 0, first = 0, index = 0;
        for (int l = 1; l <= 15; ++l) {
            code |= (int)in.get(1);
            const int c = count_[l];
            if (code - first < c) return sym_[(size_t)(index + code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        bad("invalid Huffman code");
    }

private:
    int count_[16];
    std::vector<uint16_t> sym_;
    uint16_t fast_[1 << kFast];
};

// RFC 1951 section 3.2.5 length and distance tables.
constexpr uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                                   35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193,
                                    257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// Order of the code-length code lengths (section 3.2.7).
constexpr uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

void inflate_block(Bits& in, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out, size_t limit) {
    for (;;) {
        const int s = lit.decode(in);
        if (s < 256) {
            if (out.size() >= limit) bad("decompressed data larger than expected");
            out.push_back((uint8_t)s);
        } else if (s == 256) {
            return;
        } else {
            if (s > 285) bad("invalid length symbol");
            const size_t len = kLenBase[s - 257] + in.get(kLenExtra[s - 257]);
            const int ds = dist.decode(in);
            if (ds >= 30) bad("invalid distance symbol");
            const size_t d = kDistBase[ds] + in.get(kDistExtra[ds]);
            if (d > out.size()) bad("distance before the start of the output");
            if (out.size() + len > limit) bad("decompressed data larger than expected");
            const size_t from = out.size() - d;
            for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
        }
    }
}

}  // namespace

std::vector<uint8_t> zlib_inflate(const uint8_t* data, size_t n, size_t limit) {
    if (n < 2) bad("truncated zlib stream");
    const uint8_t cmf = data[0], flg = data[1];
    if ((cmf & 15) != 8 || (cmf >> 4) > 7) bad("zlib stream is not deflate");
    if (((cmf << 8) | flg) % 31 != 0) bad("bad zlib header check");
    if (flg & 32) bad("zlib preset dictionary not supported");
    Bits in(data + 2, n - 2);
    std::vector<uint8_t> out;
    out.reserve(std::min<size_t>(limit, 1u << 26));
    Huffman lit, dist;
    bool fixed_built = false;
    Huffman flit, fdist;
    for (;;) {
        const uint32_t final_block = in.get(1);
        const uint32_t type = in.get(2);
        if (type == 0) {
            in.align();
            const size_t p = in.byte_pos();
            if (p + 4 > in.size()) bad("truncated stored block");
            const uint8_t* d = in.data() + p;
            const uint32_t len = d[0] | (d[1] << 8), nlen = d[2] | (d[3] << 8);
            if ((len ^ 0xFFFFu) != nlen) bad("stored block length check failed");
            if (p + 4 + len > in.size()) bad("truncated stored block");
            if (out.size() + len > limit) bad("decompressed data larger than expected");
            out.insert(out.end(), d + 4, d + 4 + len);
            in.skip_to(p + 4 + len);
        } else if (type == 1) {
            if (!fixed_built) {
                uint8_t l[288];
                for (int s = 0; s < 288; ++s) l[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
                flit.build(l, 288);
                uint8_t d[30];
                std::fill(d, d + 30, (uint8_t)5);
                fdist.build(d, 30);
                fixed_built = true;
            }
            inflate_block(in, flit, fdist, out, limit);
        } else if (type == 2) {
            const int hlit = (int)in.get(5) + 257, hdist = (int)in.get(5) + 1, hclen = (int)in.get(4) + 4;
            uint8_t cl[19] = {0};
            for (int k = 0; k < hclen; ++k) cl[kClOrder[k]] = (uint8_t)in.get(3);
            Huffman clh;
            clh.build(cl, 19);
            uint8_t lens[288 + 32] = {0};
            int k = 0;
            while (k < hlit + hdist) {
                const int s = clh.decode(in);
                if (s < 16) {
                    lens[k++] = (uint8_t)s;
                } else {
                    int rep = 0;
                    uint8_t val = 0;
                    if (s == 16) {
                        if (k == 0) bad("repeat of a code length before the first");
                        val = lens[k - 1];
                        rep = 3 + (int)in.get(2);
                    } else if (s == 17) {
                        rep = 3 + (int)in.get(3);
                    } else {
                        rep = 11 + (int)in.get(7);
                    }
                    if (k + rep > hlit + hdist) bad("code lengths overflow");
                    while (rep--) lens[k++] = val;
                }
            }
            if (lens[256] == 0) bad("no end-of-block code");
            lit.build(lens, hlit);
            dist.build(lens + hlit, hdist);
            inflate_block(in, lit, dist, out, limit);
        } else {
            bad("invalid deflate block type");
        }
        if (final_block) break;
    }
    // Adler-32 of the output (RFC 1950 section 2.2) follows the deflate data, byte aligned.
    in.align();
    const size_t p = in.byte_pos();
    if (p + 4 <= in.size()) {
        uint32_t a = 1, b = 0;
        for (uint8_t c : out) {
            a = (a + c) % 65521u;
            b = (b + a) % 65521u;
        }
        const uint8_t* d = in.data() + p;
        const uint32_t want = ((uint32_t)d[0] << 24) | ((uint32_t)d[1] << 16) | ((uint32_t)d[2] << 8) | d[3];
        if (want != ((b << 16) | a)) bad("zlib Adler-32 check failed");
    }
    return out;
}

namespace {

// ---- PNG -----------------------------------------------------------------------------------------

uint32_t be32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

uint8_t paeth(int a, int b, int c) {
    const int p = a + b - c;
    const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return (uint8_t)a;
    if (pb <= pc) return (uint8_t)b;
    return (uint8_t)c;
}

// Reverses the row filters of one (sub)image in place; `rows` holds height * (1 + stride) bytes.
void unfilter(uint8_t* rows, uint32_t height, size_t stride, size_t bpp, std::vector<uint8_t>& out) {
    out.assign((size_t)height * stride, 0);
    for (uint32_t y = 0; y < height; ++y) {
        const uint8_t ft = rows[(size_t)y * (stride + 1)];
        const uint8_t* src = rows + (size_t)y * (stride + 1) + 1;
        uint8_t* cur = out.data() + (size_t)y * stride;
        const uint8_t* prev = y ? cur - stride : nullptr;
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= bpp ? cur[i - bpp] : 0;
            const int b = prev ? prev[i] : 0;
            const int c = (prev && i >= bpp) ? prev[i - bpp] : 0;
            int v = src[i];
            switch (ft) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: bad("invalid PNG filter type " + std::to_string(ft));
            }
            cur[i] = (uint8_t)v;
        }
    }
}

struct PngInfo {
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = 0, interlace = 0;
    int channels = 0;
    uint8_t palette[256][4];
    int pal_len = 0;
    bool has_key = false;
    uint16_t key[3] = {0, 0, 0};
};

// One sample (channel value at its bit depth) of row `row` at sample index `i`.
inline uint32_t sample(const uint8_t* row, size_t i, int depth) {
    if (depth == 8) return row[i];
    if (depth == 16) return ((uint32_t)row[2 * i] << 8) | row[2 * i + 1];
    const size_t bit = i * (size_t)depth;
    const int shift = 8 - depth - (int)(bit & 7);
    return (row[bit >> 3] >> shift) & ((1u << depth) - 1u);
}

inline uint8_t to8(uint32_t v, int depth) {
    if (depth == 16) return (uint8_t)(v >> 8);
    if (depth == 8) return (uint8_t)v;
    return (uint8_t)(v * (255u / ((1u << depth) - 1u)));
}

// Converts one unfiltered (sub)image row of `n` pixels to RGBA8 at out[0], out[step], ...
void convert_row(const PngInfo& pi, const uint8_t* row, uint32_t n, uint8_t* out, size_t step) {
    for (uint32_t x = 0; x < n; ++x, out += step) {
        const size_t s = (size_t)x * pi.channels;
        switch (pi.ctype) {
            case 0: {
                const uint32_t g = sample(row, s, pi.depth);
                out[0] = out[1] = out[2] = to8(g, pi.depth);
                out[3] = (pi.has_key && g == pi.key[0]) ? 0 : 255;
                break;
            }
            case 2: {
                const uint32_t r = sample(row, s, pi.depth), g = sample(row, s + 1, pi.depth), b = sample(row, s + 2, pi.depth);
                out[0] = to8(r, pi.depth);
                out[1] = to8(g, pi.depth);
                out[2] = to8(b, pi.depth);
                out[3] = (pi.has_key && r == pi.key[0] && g == pi.key[1] && b == pi.key[2]) ? 0 : 255;
                break;
            }
            case 3: {
                const uint32_t k = sample(row, s, pi.depth);
                if ((int)k < pi.pal_len) std::memcpy(out, pi.palette[k], 4);
                else out[0] = out[1] = out[2] = 0, out[3] = 255;   // index past the palette: opaque black
                break;
            }
            case 4: {
                out[0] = out[1] = out[2] = to8(sample(row, s, pi.depth), pi.depth);
                out[3] = to8(sample(row, s + 1, pi.depth), pi.depth);
                break;
            }
            default: {
                for (int c = 0; c < 4; ++c) out[c] = to8(sample(row, s + c, pi.depth), pi.depth);
                break;
            }
        }
    }
}

Image decode_png(const uint8_t* data, size_t n) {
    PngInfo pi;
    std::vector<uint8_t> idat;
    size_t p = 8;
    bool seen_ihdr = false, seen_iend = false;
    while (p + 8 <= n && !seen_iend) {
        const uint32_t len = be32(data + p);
        const uint8_t* type = data + p + 4;
        if (len > n - p - 8 || n - p - 8 - len < 4) bad("truncated PNG chunk");
        const uint8_t* d = data + p + 8;
        const std::string t(reinterpret_cast<const char*>(type), 4);
        if (!seen_ihdr && t != "IHDR") bad("PNG does not start with IHDR");
        if (t == "IHDR") {
            if (len != 13) bad("bad IHDR length");
            pi.w = be32(d);
            pi.h = be32(d + 4);
            pi.depth = d[8];
            pi.ctype = d[9];
            if (d[10] != 0 || d[11] != 0) bad("unknown PNG compression or filter method");
            pi.interlace = d[12];
            if (pi.interlace > 1) bad("unknown PNG interlace method");
            if (pi.w == 0 || pi.h == 0) bad("PNG has zero size");
            if (pi.w > (1u << 24) || pi.h > (1u << 24) || (uint64_t)pi.w * pi.h > (1ull << 28))
                bad("PNG too large (more than 2^28 pixels)");
            const int dp = pi.depth, ct = pi.ctype;
            const bool ok = (ct == 0 && (dp == 1 || dp == 2 || dp == 4 || dp == 8 || dp == 16)) ||
                            (ct == 3 && (dp == 1 || dp == 2 || dp == 4 || dp == 8)) ||
                            ((ct == 2 || ct == 4 || ct == 6) && (dp == 8 || dp == 16));
            if (!ok) bad("invalid PNG colour type / bit depth");
            pi.channels = ct == 0 ? 1 : ct == 2 ? 3 : ct == 3 ? 1 : ct == 4 ? 2 : 4;
            seen_ihdr = true;
        } else if (t == "PLTE") {
            if (len % 3 != 0 || len / 3 > 256) bad("bad PLTE chunk");
            pi.pal_len = (int)(len / 3);
            for (int k = 0; k < pi.pal_len; ++k) {
                pi.palette[k][0] = d[3 * k];
                pi.palette[k][1] = d[3 * k + 1];
                pi.palette[k][2] = d[3 * k + 2];
                pi.palette[k][3] = 255;
            }
        } else if (t == "tRNS") {
            if (!idat.empty()) bad("tRNS after IDAT");
            if (pi.ctype == 3) {
                if (pi.pal_len == 0) bad("tRNS before PLTE");
                if ((int)len > pi.pal_len) bad("tRNS longer than the palette");
                for (uint32_t k = 0; k < len; ++k) pi.palette[k][3] = d[k];
            } else if (pi.ctype == 0 || pi.ctype == 2) {
                const uint32_t want = pi.ctype == 0 ? 2u : 6u;
                if (len != want) bad("bad tRNS length");
                for (uint32_t k = 0; k < want / 2; ++k) pi.key[k] = (uint16_t)((d[2 * k] << 8) | d[2 * k + 1]);
                pi.has_key = true;
            } else {
                bad("tRNS on a PNG with an alpha channel");
            }
        } else if (t == "IDAT") {
            idat.insert(idat.end(), d, d + len);
        } else if (t == "IEND") {
            seen_iend = true;
        } else if (!(type[0] & 32)) {
            bad("unknown critical PNG chunk " + t);
        }
        p += 12 + (size_t)len;
    }
    if (!seen_ihdr) bad("PNG has no IHDR");
    if (pi.ctype == 3 && pi.pal_len == 0) bad("palette PNG without PLTE");
    if (idat.empty()) bad("PNG has no image data");

    const size_t bits_pp = (size_t)pi.channels * pi.depth;
    const size_t bpp = std::max<size_t>(1, bits_pp / 8);
    // passes (x0, y0, dx, dy): the whole image, or the seven Adam7 passes
    static const int kAdam7[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4}, {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    static const int kWhole[1][4] = {{0, 0, 1, 1}};
    const int (*passes)[4] = pi.interlace ? kAdam7 : kWhole;
    const int npass = pi.interlace ? 7 : 1;
    size_t expect = 0;
    for (int k = 0; k < npass; ++k) {
        const uint64_t pw = (pi.w + (uint32_t)(passes[k][2] - 1 - passes[k][0])) / (uint32_t)passes[k][2];
        const uint64_t ph = (pi.h + (uint32_t)(passes[k][3] - 1 - passes[k][1])) / (uint32_t)passes[k][3];
        if (pw && ph) expect += (size_t)ph * (1 + (size_t)((pw * bits_pp + 7) / 8));
    }
    std::vector<uint8_t> raw = zlib_inflate(idat.data(), idat.size(), expect);
    if (raw.size() < expect) bad("PNG image data too short");

    Image img;
    img.width = pi.w;
    img.height = pi.h;
    img.rgba.assign((size_t)pi.w * pi.h * 4, 0);
    size_t off = 0;
    std::vector<uint8_t> sub;
    for (int k = 0; k < npass; ++k) {
        const uint32_t x0 = (uint32_t)passes[k][0], y0 = (uint32_t)passes[k][1];
        const uint32_t dx = (uint32_t)passes[k][2], dy = (uint32_t)passes[k][3];
        const uint32_t pw = (pi.w + dx - 1 - x0) / dx, ph = (pi.h + dy - 1 - y0) / dy;
        if (!pw || !ph) continue;
        const size_t stride = ((size_t)pw * bits_pp + 7) / 8;
        unfilter(raw.data() + off, ph, stride, bpp, sub);
        off += (size_t)ph * (stride + 1);
        for (uint32_t y = 0; y < ph; ++y)
            convert_row(pi, sub.data() + (size_t)y * stride, pw,
                        img.rgba.data() + (((size_t)(y0 + y * dy) * pi.w) + x0) * 4, (size_t)dx * 4);
    }
    return img;
}

// ---- JPEG (ITU-T T.81: baseline and extended sequential Huffman, 8-bit samples) -----------------------

// Natural (row-major) index of the k-th coefficient in zigzag order (T.81 figure A.6).
constexpr uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                                 12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                                 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                                 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct JpegHuff {
    bool defined = false;
    int count[17] = {0};
    std::vector<uint8_t> vals;
    // canonical decoding (T.81 F.2.2.3): per length the first code and the index of its first value
    int32_t mincode[17], maxcode[18], valptr[17];
    void derive() {
        int code = 0, k = 0;
        for (int l = 1; l <= 16; ++l) {
            valptr[l] = k;
            mincode[l] = code;
            code += count[l];
            k += count[l];
            maxcode[l] = count[l] ? code - 1 : -1;
            code <<= 1;
        }
        maxcode[17] = 0x7FFFFFFF;
        defined = true;
    }
};

struct JpegComp {
    int id = 0, h = 1, v = 1, tq = 0, td = 0, ta = 0;
    int bw = 0, bh = 0;       // blocks across / down (padded to whole MCUs)
    std::vector<uint8_t> plane;
    std::vector<int16_t> coef;   // progressive frames: quantized coefficients, 64 per block in zigzag order
    int pred = 0;
};

class JpegBits {
public:
    JpegBits(const uint8_t* p, size_t n, size_t pos) : p_(p), n_(n), pos_(pos) {}
    int bit() {
        if (cnt_ == 0) fill();
        --cnt_;
        return (int)((buf_ >> cnt_) & 1u);
    }
    int bits(int k) {
        int v = 0;
        for (int i = 0; i < k; ++i) v = (v << 1) | bit();
        return v;
    }
    // After a restart interval: skip to the RSTn marker and past it.
    void restart() {
        cnt_ = 0;
        marker_ = false;
        while (pos_ + 1 < n_ && !(p_[pos_] == 0xFF && p_[pos_ + 1] >= 0xD0 && p_[pos_ + 1] <= 0xD7)) ++pos_;
        if (pos_ + 1 >= n_) bad("JPEG: missing restart marker");
        pos_ += 2;
    }
    size_t pos() const { return pos_; }

private:
    void fill() {
        // past a marker (or the end) the decoder reads zero bits; a valid stream never needs them
        uint8_t b = 0;
        if (!marker_ && pos_ < n_) {
            b = p_[pos_];
            if (b == 0xFF) {
                const uint8_t nx = pos_ + 1 < n_ ? p_[pos_ + 1] : 0xD9;
                if (nx == 0x00) pos_ += 2;
                else { marker_ = true; b = 0; }
            } else {
                ++pos_;
            }
        }
        buf_ = b;
        cnt_ = 8;
    }
    const uint8_t* p_;
    size_t n_, pos_;
    uint32_t buf_ = 0;
    int cnt_ = 0;
    bool marker_ = false;
};

int huff_decode(JpegBits& in, const JpegHuff& h) {
    int code = in.bit();
    for (int l = 1; l <= 16; ++l) {
        if (code <= h.maxcode[l]) return h.vals[(size_t)(h.valptr[l] + code - h.mincode[l])];
        code = (code << 1) | in.bit();
    }
    bad("JPEG: invalid Huffman code");
}

inline int extend(int v, int t) { return t == 0 ? 0 : (v < (1 << (t - 1)) ? v - (1 << t) + 1 : v); }   // T.81 F.2.2.1

// Separable 8x8 inverse DCT in double precision: f(x, y) = 1/4 sum C(u) C(v) F(u, v) cos((2x+1)u pi/16)
// cos((2y+1)v pi/16) with C(0) = 1/sqrt(2), level-shifted by 128, rounded to nearest and clamped.
void idct8x8(const double* F, uint8_t* out, int stride) {
    struct Table {
        double v[8][8];
        Table() {
            for (int x = 0; x < 8; ++x)
                for (int u = 0; u < 8; ++u)
                    v[x][u] = (u == 0 ? std::sqrt(0.5) : 1.0) * std::cos((2 * x + 1) * u * 3.14159265358979323846 / 16.0);
        }
    };
    static const Table table;   // built once, thread-safely (a function-local static)
    const auto& cosv = table.v;
    double tmp[64];
    for (int v = 0; v < 8; ++v)   // rows of F: inverse over u for every x
        for (int x = 0; x < 8; ++x) {
            double s = 0.0;
            for (int u = 0; u < 8; ++u) s += cosv[x][u] * F[v * 8 + u];
            tmp[v * 8 + x] = s;
        }
    for (int y = 0; y < 8; ++y)
        for (int x = 0; x < 8; ++x) {
            double s = 0.0;
            for (int v = 0; v < 8; ++v) s += cosv[y][v] * tmp[v * 8 + x];
            const double val = std::floor(s / 4.0 + 128.0 + 0.5);
            out[y * stride + x] = (uint8_t)std::min(255.0, std::max(0.0, val));
        }
}

Image decode_jpeg(const uint8_t* d, size_t n) {
    uint16_t qt[4][64];
    bool qt_def[4] = {false, false, false, false};
    JpegHuff dc[4], ac[4];
    std::vector<JpegComp> comps;
    int W = 0, H = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
    int restart = 0;
    int adobe_transform = -1;
    bool frame = false, seen_scan = false, progressive = false;
    size_t p = 2;
    auto u16 = [&](size_t at) {
        if (at + 2 > n) bad("JPEG: truncated");
        return (int)((d[at] << 8) | d[at + 1]);
    };
    for (;;) {
        while (p < n && d[p] != 0xFF) ++p;   // tolerate fill bytes between segments
        while (p < n && d[p] == 0xFF) ++p;
        if (p >= n) bad("JPEG: truncated (no EOI)");
        const uint8_t m = d[p++];
        if (m == 0xD9) break;   // EOI
        if (m == 0xD8 || (m >= 0xD0 && m <= 0xD7) || m == 0x01) continue;
        const int len = u16(p);
        if (len < 2 || p + (size_t)len > n) bad("JPEG: truncated segment");
        const uint8_t* s = d + p + 2;
        const size_t sl = (size_t)len - 2;
        if (m == 0xDB) {   // DQT
            size_t k = 0;
            while (k < sl) {
                const int pq = s[k] >> 4, tq = s[k] & 15;
                if (tq > 3 || pq > 1) bad("JPEG: bad quantization table");
                ++k;
                if (k + (pq ? 128u : 64u) > sl) bad("JPEG: truncated quantization table");
                for (int i = 0; i < 64; ++i) qt[tq][i] = pq ? (uint16_t)((s[k + 2 * i] << 8) | s[k + 2 * i + 1]) : s[k + i];
                k += pq ? 128 : 64;
                qt_def[tq] = true;
            }
        } else if (m == 0xC4) {   // DHT
            size_t k = 0;
            while (k < sl) {
                const int tc = s[k] >> 4, th = s[k] & 15;
                if (tc > 1 || th > 3 || k + 17 > sl) bad("JPEG: bad Huffman table");
                JpegHuff& h = tc ? ac[th] : dc[th];
                int total = 0;
                h.count[0] = 0;
                for (int l = 1; l <= 16; ++l) total += (h.count[l] = s[k + (size_t)l]);
                if (total > 256 || k + 17 + (size_t)total > sl) bad("JPEG: bad Huffman table");
                h.vals.assign(s + k + 17, s + k + 17 + total);
                h.derive();
                k += 17 + (size_t)total;
            }
        } else if (m == 0xC0 || m == 0xC1 || m == 0xC2) {   // SOF0 / SOF1 sequential, SOF2 progressive (Huffman)
            if (frame) bad("JPEG: more than one frame");
            progressive = m == 0xC2;
            if (sl < 6 || s[0] != 8) bad("JPEG: only 8-bit samples are supported");
            H = (s[1] << 8) | s[2];
            W = (s[3] << 8) | s[4];
            const int nc = s[5];
            if (W == 0 || H == 0) bad("JPEG: zero size (DNL not supported)");
            if ((uint64_t)W * H > (1ull << 28)) bad("JPEG too large (more than 2^28 pixels)");
            if ((nc != 1 && nc != 3) || sl < 6 + 3 * (size_t)nc) bad("JPEG: only 1 or 3 components are supported");
            comps.resize((size_t)nc);
            for (int c = 0; c < nc; ++c) {
                comps[c].id = s[6 + 3 * c];
                comps[c].h = s[7 + 3 * c] >> 4;
                comps[c].v = s[7 + 3 * c] & 15;
                comps[c].tq = s[8 + 3 * c];
                if (comps[c].h < 1 || comps[c].h > 4 || comps[c].v < 1 || comps[c].v > 4 || comps[c].tq > 3)
                    bad("JPEG: bad component parameters");
                hmax = std::max(hmax, comps[c].h);
                vmax = std::max(vmax, comps[c].v);
            }
            mcux = (W + 8 * hmax - 1) / (8 * hmax);
            mcuy = (H + 8 * vmax - 1) / (8 * vmax);
            for (JpegComp& c : comps) {
                c.bw = mcux * c.h;
                c.bh = mcuy * c.v;
                c.plane.assign((size_t)c.bw * 8 * c.bh * 8, 0);
                if (progressive) c.coef.assign((size_t)c.bw * c.bh * 64, 0);
            }
            frame = true;
        } else if (m == 0xC3 || (m >= 0xC5 && m <= 0xCF && m != 0xC8 && m != 0xCC)) {
            bad("JPEG: lossless, hierarchical and arithmetic-coded JPEG are not supported");
        } else if (m == 0xDD) {   // DRI
            restart = u16(p + 2);
        } else if (m == 0xEE) {   // APP14 (Adobe): colour transform flag
            if (sl >= 12 && std::memcmp(s, "Adobe", 5) == 0) adobe_transform = s[11];
        } else if (m == 0xDA) {   // SOS
            if (!frame) bad("JPEG: scan before frame");
            const int ns = s[0];
            if (ns < 1 || ns > 4 || sl < 1 + 2 * (size_t)ns + 3) bad("JPEG: bad scan header");
            std::vector<JpegComp*> sc;
            for (int k = 0; k < ns; ++k) {
                JpegComp* c = nullptr;
                for (JpegComp& cc : comps)
                    if (cc.id == s[1 + 2 * k]) c = &cc;
                if (!c) bad("JPEG: scan references an unknown component");
                c->td = s[2 + 2 * k] >> 4;
                c->ta = s[2 + 2 * k] & 15;
                if (c->td > 3 || c->ta > 3) bad("JPEG: bad Huffman table selector");
                if (!qt_def[c->tq]) bad("JPEG: missing quantization table");
                c->pred = 0;
                sc.push_back(c);
            }
            const int ss = s[1 + 2 * ns], se = s[2 + 2 * ns], ah = s[3 + 2 * ns] >> 4, al = s[3 + 2 * ns] & 15;
            if (!progressive) {
                if (ss != 0 || se != 63 || ah != 0 || al != 0) bad("JPEG: not a sequential scan");
                for (JpegComp* c : sc)
                    if (!dc[c->td].defined || !ac[c->ta].defined) bad("JPEG: missing Huffman table");
            } else {
                // T.81 G.1.1.1: a DC scan (Ss = Se = 0) may interleave components; an AC scan
                // (1 <= Ss <= Se <= 63) holds one; a refinement scan lowers the point transform by one bit
                const bool dc_scan = ss == 0;
                if (dc_scan ? se != 0 : (se < ss || se > 63 || ns != 1)) bad("JPEG: bad progressive scan band");
                if (al > 13 || (ah != 0 && ah != al + 1)) bad("JPEG: bad successive-approximation parameters");
                for (JpegComp* c : sc) {
                    if (dc_scan && ah == 0 && !dc[c->td].defined) bad("JPEG: missing Huffman table");
                    if (!dc_scan && !ac[c->ta].defined) bad("JPEG: missing Huffman table");
                }
            }
            int eobrun = 0;   // progressive AC scans: blocks left in the current end-of-band run
            JpegBits in(d, n, p + (size_t)len);
            // blocks of one MCU: interleaved scans take h x v blocks per component; a single-component scan
            // takes the component's blocks one at a time in raster order over its own (unpadded) extent
            const bool single = ns == 1;
            int units_x = mcux, units_y = mcuy;
            if (single) {
                const JpegComp& c = *sc[0];
                units_x = ((W * c.h + hmax - 1) / hmax + 7) / 8;
                units_y = ((H * c.v + vmax - 1) / vmax + 7) / 8;
            }
            double F[64];
            auto block = [&](JpegComp& c, int bx, int by) {
                std::fill(F, F + 64, 0.0);
                const uint16_t* q = qt[c.tq];
                const int t = huff_decode(in, dc[c.td]);
                if (t > 11) bad("JPEG: bad DC difference");
                c.pred += extend(in.bits(t), t);
                F[0] = (double)c.pred * q[0];
                for (int k = 1; k < 64;) {
                    const int rs = huff_decode(in, ac[c.ta]);
                    const int r = rs >> 4, sz = rs & 15;
                    if (sz == 0) {
                        if (r != 15) break;   // end of block
                        k += 16;
                        continue;
                    }
                    k += r;
                    if (k > 63) bad("JPEG: coefficient index past 63");
                    F[kZigzag[k]] = (double)extend(in.bits(sz), sz) * q[k];
                    ++k;
                }
                const int stride = c.bw * 8;
                idct8x8(F, c.plane.data() + (size_t)by * 8 * stride + (size_t)bx * 8, stride);
            };
            // progressive scans (T.81 G.1.2): one band of one bit level of the coefficients per scan
            const int p1 = 1 << al, m1 = -(1 << al);
            auto refine = [&](int16_t& c) {   // a correction bit for a coefficient already nonzero
                if (in.bit() && (c & p1) == 0) c = (int16_t)(c + (c >= 0 ? p1 : m1));
            };
            auto pblock = [&](JpegComp& c, int bx, int by) {
                int16_t* blk = c.coef.data() + ((size_t)by * c.bw + bx) * 64;
                if (ss == 0) {
                    if (ah == 0) {   // DC first: difference of the point-transformed DC
                        const int t = huff_decode(in, dc[c.td]);
                        if (t > 11) bad("JPEG: bad DC difference");
                        c.pred += extend(in.bits(t), t);
                        blk[0] = (int16_t)(c.pred * (1 << al));
                    } else if (in.bit()) {   // DC refinement: one more bit
                        blk[0] = (int16_t)(blk[0] | p1);
                    }
                    return;
                }
                int k = ss;
                if (ah == 0) {   // AC first: run/size symbols and end-of-band runs
                    if (eobrun > 0) {
                        --eobrun;
                        return;
                    }
                    for (; k <= se; ++k) {
                        const int rs = huff_decode(in, ac[c.ta]);
                        const int r = rs >> 4, sz = rs & 15;
                        if (sz == 0) {
                            if (r == 15) {   // sixteen zeros
                                k += 15;
                                continue;
                            }
                            eobrun = (1 << r) - 1 + (r ? in.bits(r) : 0);   // this block and eobrun more
                            break;
                        }
                        k += r;
                        if (k > se) bad("JPEG: coefficient index past the band");
                        blk[k] = (int16_t)(extend(in.bits(sz), sz) * (1 << al));
                    }
                    return;
                }
                // AC refinement: newly nonzero coefficients (magnitude 1 at this bit level) with their
                // zero runs, and a correction bit for every coefficient that was already nonzero
                if (eobrun == 0) {
                    for (; k <= se; ++k) {
                        const int rs = huff_decode(in, ac[c.ta]);
                        int r = rs >> 4;
                        const int sz = rs & 15;
                        int val = 0;
                        if (sz != 0) {
                            if (sz != 1) bad("JPEG: bad refinement coefficient size");
                            val = in.bit() ? p1 : m1;
                        } else if (r != 15) {
                            eobrun = (1 << r) + (r ? in.bits(r) : 0);
                            break;
                        }
                        // pass r zero coefficients (correcting the nonzero ones on the way); stop at the
                        // next zero, where a new coefficient goes (a run of sixteen leaves it zero)
                        for (; k <= se; ++k) {
                            if (blk[k] != 0) refine(blk[k]);
                            else if (r == 0) break;
                            else --r;
                        }
                        if (val != 0) {
                            if (k > se) bad("JPEG: coefficient index past the band");
                            blk[k] = (int16_t)val;
                        }
                    }
                }
                if (eobrun > 0) {   // the rest of the band is in an end-of-band run: corrections only
                    for (; k <= se; ++k)
                        if (blk[k] != 0) refine(blk[k]);
                    --eobrun;
                }
            };
            auto unit = [&](JpegComp& c, int bx, int by) {
                if (progressive) pblock(c, bx, by);
                else block(c, bx, by);
            };
            int todo = restart;
            for (int my = 0; my < units_y; ++my)
                for (int mx = 0; mx < units_x; ++mx) {
                    if (restart && todo == 0) {
                        in.restart();
                        for (JpegComp* c : sc) c->pred = 0;
                        eobrun = 0;
                        todo = restart;
                    }
                    if (single) {
                        unit(*sc[0], mx, my);
                    } else {
                        for (JpegComp* c : sc)
                            for (int v = 0; v < c->v; ++v)
                                for (int h = 0; h < c->h; ++h) unit(*c, mx * c->h + h, my * c->v + v);
                    }
                    if (restart) --todo;
                }
            seen_scan = true;
            p = in.pos();
            continue;
        }
        p += (size_t)len;
    }
    if (!frame || !seen_scan) bad("JPEG: no image data");
    if (progressive) {   // every scan is in: dequantize and transform each block once
        double F[64];
        for (JpegComp& c : comps) {
            const uint16_t* q = qt[c.tq];
            const int stride = c.bw * 8;
            for (int by = 0; by < c.bh; ++by)
                for (int bx = 0; bx < c.bw; ++bx) {
                    const int16_t* blk = c.coef.data() + ((size_t)by * c.bw + bx) * 64;
                    for (int k = 0; k < 64; ++k) F[kZigzag[k]] = (double)blk[k] * q[k];
                    idct8x8(F, c.plane.data() + (size_t)by * 8 * stride + (size_t)bx * 8, stride);
                }
        }
    }

    // upsample every component to the full grid: 2:1 by the triangle filter (3/4 nearer + 1/4 farther
    // sample, JFIF co-sited centres), other ratios by replication
    const int fw = mcux * hmax * 8, fh = mcuy * vmax * 8;
    std::vector<std::vector<uint8_t>> full(comps.size());
    for (size_t ci = 0; ci < comps.size(); ++ci) {
        const JpegComp& c = comps[ci];
        const int cw = c.bw * 8, ch = c.bh * 8;
        const int sx = hmax / c.h, sy = vmax / c.v;
        if (hmax % c.h || vmax % c.v) bad("JPEG: non-integral sampling ratio");
        std::vector<uint8_t>& o = full[ci];
        o.assign((size_t)fw * fh, 0);
        if (sx == 1 && sy == 1) {
            o = c.plane;
            continue;
        }
        if ((sx == 2 || sx == 1) && (sy == 2 || sy == 1)) {
            // vertical then horizontal, in 16ths (2x2) or quarters (one direction)
            const int used_w = (W * c.h + hmax - 1) / hmax, used_h = (H * c.v + vmax - 1) / vmax;
            const int uw = std::max(1, std::min(cw, used_w)), uh = std::max(1, std::min(ch, used_h));
            auto S = [&](int x, int y) { return (int)c.plane[(size_t)std::min(std::max(y, 0), uh - 1) * cw + std::min(std::max(x, 0), uw - 1)]; };
            for (int y = 0; y < fh; ++y) {
                const int yc = sy == 2 ? y / 2 : y;
                const int yf = sy == 2 ? (y % 2 ? yc + 1 : yc - 1) : yc;   // farther row
                for (int x = 0; x < fw; ++x) {
                    const int xc = sx == 2 ? x / 2 : x;
                    const int xf = sx == 2 ? (x % 2 ? xc + 1 : xc - 1) : xc;
                    int val;
                    if (sx == 2 && sy == 2) {
                        const int t_near = 3 * S(xc, yc) + S(xc, yf), t_far = 3 * S(xf, yc) + S(xf, yf);
                        val = (3 * t_near + t_far + 8) >> 4;
                    } else if (sx == 2) {
                        val = (3 * S(xc, yc) + S(xf, yc) + 2) >> 2;
                    } else {
                        val = (3 * S(xc, yc) + S(xc, yf) + 2) >> 2;
                    }
                    o[(size_t)y * fw + x] = (uint8_t)val;
                }
            }
            continue;
        }
        for (int y = 0; y < fh; ++y)
            for (int x = 0; x < fw; ++x) o[(size_t)y * fw + x] = c.plane[(size_t)std::min(y / sy, ch - 1) * cw + std::min(x / sx, cw - 1)];
    }

    Image img;
    img.width = (uint32_t)W;
    img.height = (uint32_t)H;
    img.rgba.assign((size_t)W * H * 4, 255);
    const bool rgb = comps.size() == 3 && (adobe_transform == 0 || (comps[0].id == 'R' && comps[1].id == 'G' && comps[2].id == 'B'));
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            uint8_t* o = &img.rgba[((size_t)y * W + x) * 4];
            const size_t i = (size_t)y * fw + x;
            if (comps.size() == 1) {
                o[0] = o[1] = o[2] = full[0][i];
            } else if (rgb) {
                o[0] = full[0][i];
                o[1] = full[1][i];
                o[2] = full[2][i];
            } else {   // JFIF YCbCr -> RGB
                const double Y = full[0][i], cb = full[1][i] - 128.0, cr = full[2][i] - 128.0;
                auto q = [](double v) { return (uint8_t)std::min(255.0, std::max(0.0, std::floor(v + 0.5))); };
                o[0] = q(Y + 1.402 * cr);
                o[1] = q(Y - 0.344136 * cb - 0.714136 * cr);
                o[2] = q(Y + 1.772 * cb);
            }
        }
    return img;
}

}  // namespace

namespace {

uint32_t le16(const uint8_t* p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
uint32_t le32(const uint8_t* p) { return le16(p) | (le16(p + 2) << 16); }

// Value of the bits of `v` under `mask`, scaled to 0..255 (a mask of zero gives `none`).
uint8_t masked(uint32_t v, uint32_t mask, uint8_t none) {
    if (mask == 0) return none;
    int shift = 0;
    while (((mask >> shift) & 1u) == 0) ++shift;
    const uint32_t m = mask >> shift;
    int bits = 0;
    while (bits < 32 && ((m >> bits) & 1u)) ++bits;
    // 64-bit arithmetic: a full 32-bit mask has top = 2^32 - 1 and x * 255 needs more than 32 bits
    const uint64_t x = (v & mask) >> shift, top = bits >= 32 ? 0xFFFFFFFFull : (1ull << bits) - 1ull;
    return (uint8_t)((x * 255ull + top / 2) / top);
}

// Windows / OS/2 bitmap: 1, 4, 8 (palette), 16 (5-5-5 or bit fields), 24 and 32 (BGRA or bit fields) bits
// per pixel, bottom-up or top-down, uncompressed.  32-bit pixels whose alpha is zero everywhere are opaque.
Image decode_bmp(const uint8_t* d, size_t n) {
    if (n < 26) bad("BMP: truncated");
    const uint32_t offset = le32(d + 10), hsize = le32(d + 14);
    int64_t w, h;
    uint32_t bpp, comp = 0, ncolors = 0;
    size_t pal_entry = 4;
    if (hsize == 12) {   // OS/2 core header
        w = le16(d + 18);
        h = le16(d + 20);
        bpp = le16(d + 24);
        pal_entry = 3;
    } else if (hsize >= 40 && n >= 14 + 40) {
        w = (int32_t)le32(d + 18);
        h = (int32_t)le32(d + 22);
        bpp = le16(d + 28);
        comp = le32(d + 30);
        ncolors = le32(d + 46);
    } else {
        bad("BMP: unsupported header");
    }
    const bool top_down = h < 0;
    if (h < 0) h = -h;
    if (w <= 0 || h <= 0 || (uint64_t)w * (uint64_t)h > (1ull << 28)) bad("BMP: bad size");
    if (comp != 0 && comp != 3) bad("BMP: compressed bitmaps are not supported");
    if (bpp != 1 && bpp != 4 && bpp != 8 && bpp != 16 && bpp != 24 && bpp != 32) bad("BMP: unsupported bit depth");
    uint32_t mr = 0, mg = 0, mb = 0, ma = 0;
    if (bpp == 16) { mr = 0x7C00; mg = 0x03E0; mb = 0x001F; }
    if (bpp == 32) { mr = 0x00FF0000; mg = 0x0000FF00; mb = 0x000000FF; ma = 0xFF000000; }
    if (comp == 3) {
        if (bpp != 16 && bpp != 32) bad("BMP: bit fields need 16 or 32 bits per pixel");
        if (n < 14 + 40 + 12) bad("BMP: truncated");
        mr = le32(d + 54);
        mg = le32(d + 58);
        mb = le32(d + 62);
        ma = hsize >= 56 && n >= 14 + 56 ? le32(d + 66) : 0;
    }
    std::vector<uint8_t> pal;   // RGBA
    if (bpp <= 8) {
        const uint32_t count = ncolors ? ncolors : (1u << bpp);
        if (count > 256) bad("BMP: bad palette size");
        const size_t at = 14 + hsize;
        if (at + count * pal_entry > n) bad("BMP: truncated palette");
        pal.resize((size_t)count * 4);
        for (uint32_t i = 0; i < count; ++i) {
            const uint8_t* e = d + at + i * pal_entry;
            pal[4 * i + 0] = e[2];
            pal[4 * i + 1] = e[1];
            pal[4 * i + 2] = e[0];
            pal[4 * i + 3] = 255;
        }
    }
    const size_t stride = (((size_t)w * bpp + 31) / 32) * 4;
    if (offset > n || (size_t)h * stride > n - offset) bad("BMP: truncated pixel data");
    Image img;
    img.width = (uint32_t)w;
    img.height = (uint32_t)h;
    img.rgba.assign((size_t)w * h * 4, 255);
    bool any_alpha = false;
    for (int64_t y = 0; y < h; ++y) {
        const uint8_t* row = d + offset + (size_t)(top_down ? y : h - 1 - y) * stride;
        uint8_t* o = &img.rgba[(size_t)y * w * 4];
        for (int64_t x = 0; x < w; ++x, o += 4) {
            if (bpp <= 8) {
                const size_t bit = (size_t)x * bpp;
                const uint32_t idx = (row[bit / 8] >> (8 - bpp - bit % 8)) & ((1u << bpp) - 1u);
                if ((size_t)idx * 4 >= pal.size()) bad("BMP: palette index out of range");
                std::memcpy(o, &pal[(size_t)idx * 4], 4);
            } else if (bpp == 24) {
                o[0] = row[3 * x + 2];
                o[1] = row[3 * x + 1];
                o[2] = row[3 * x + 0];
            } else {
                const uint32_t v = bpp == 16 ? le16(row + 2 * x) : le32(row + 4 * x);
                o[0] = masked(v, mr, 0);
                o[1] = masked(v, mg, 0);
                o[2] = masked(v, mb, 0);
                o[3] = masked(v, ma, 255);
                any_alpha = any_alpha || o[3] != 0;
            }
        }
    }
    if (bpp == 32 && ma != 0 && !any_alpha)   // an unused alpha channel: opaque
        for (size_t i = 3; i < img.rgba.size(); i += 4) img.rgba[i] = 255;
    return img;
}

// Truevision TGA: colour-mapped (8-bit indices into 15/16/24/32-bit entries), true-colour (15/16, 24, 32
// bits) and grey (8 bits) images, uncompressed or run-length encoded, either origin.
bool looks_like_tga(const uint8_t* d, size_t n) {
    if (n < 18) return false;
    const int cmap = d[1], type = d[2], depth = d[16];
    if (cmap > 1) return false;
    if (type != 1 && type != 2 && type != 3 && type != 9 && type != 10 && type != 11) return false;
    if ((type == 1 || type == 9) ? (cmap != 1 || depth != 8) : (depth != 8 && depth != 15 && depth != 16 && depth != 24 && depth != 32))
        return false;
    return le16(d + 12) > 0 && le16(d + 14) > 0;
}

Image decode_tga(const uint8_t* d, size_t n) {
    if (!looks_like_tga(d, n)) bad("TGA: bad header");
    const uint32_t id_len = d[0], cmap_type = d[1], type = d[2];
    const uint32_t cmap_first = le16(d + 3), cmap_len = le16(d + 5), cmap_bits = d[7];
    const uint32_t w = le16(d + 12), h = le16(d + 14), depth = d[16], desc = d[17];
    const bool rle = type >= 9, gray = type == 3 || type == 11, mapped = type == 1 || type == 9;
    size_t p = 18 + id_len;
    auto texel = [](const uint8_t* e, uint32_t bits, uint8_t* o) {   // one stored value -> RGBA
        if (bits == 15 || bits == 16) {
            const uint32_t v = le16(e);
            o[0] = (uint8_t)((((v >> 10) & 31u) * 255u + 15u) / 31u);
            o[1] = (uint8_t)((((v >> 5) & 31u) * 255u + 15u) / 31u);
            o[2] = (uint8_t)(((v & 31u) * 255u + 15u) / 31u);
            o[3] = 255;
        } else {
            o[0] = e[2];
            o[1] = e[1];
            o[2] = e[0];
            o[3] = bits == 32 ? e[3] : 255;
        }
    };
    std::vector<uint8_t> pal;
    if (cmap_type == 1) {
        if (cmap_bits != 15 && cmap_bits != 16 && cmap_bits != 24 && cmap_bits != 32) bad("TGA: bad colour map");
        const size_t eb = (cmap_bits + 7) / 8;
        if (p + cmap_len * eb > n) bad("TGA: truncated colour map");
        pal.resize((size_t)(cmap_first + cmap_len) * 4, 0);
        for (uint32_t i = 0; i < cmap_len; ++i) texel(d + p + i * eb, cmap_bits, &pal[(size_t)(cmap_first + i) * 4]);
        p += cmap_len * eb;
    }
    const size_t pb = (depth + 7) / 8;
    if ((uint64_t)w * h > (1ull << 28)) bad("TGA: too large (more than 2^28 pixels)");
    if (!rle && p + (size_t)w * h * pb > n) bad("TGA: truncated pixel data");
    Image img;
    img.width = w;
    img.height = h;
    img.rgba.assign((size_t)w * h * 4, 255);
    auto put = [&](const uint8_t* e, size_t i) {
        uint8_t* o = &img.rgba[i * 4];
        if (mapped) {
            if ((size_t)e[0] * 4 + 4 > pal.size()) bad("TGA: colour index out of range");
            std::memcpy(o, &pal[(size_t)e[0] * 4], 4);
        } else if (gray) {
            o[0] = o[1] = o[2] = e[0];
        } else {
            texel(e, depth, o);
        }
    };
    const size_t total = (size_t)w * h;
    size_t i = 0;
    while (i < total) {
        if (!rle) {
            if (p + pb > n) bad("TGA: truncated pixel data");
            put(d + p, i++);
            p += pb;
            continue;
        }
        if (p >= n) bad("TGA: truncated pixel data");
        const uint32_t hdr = d[p++], count = (hdr & 0x7F) + 1;
        if (i + count > total) bad("TGA: run past the image");
        if (hdr & 0x80) {   // one value repeated
            if (p + pb > n) bad("TGA: truncated pixel data");
            for (uint32_t k = 0; k < count; ++k) put(d + p, i++);
            p += pb;
        } else {
            if (p + count * pb > n) bad("TGA: truncated pixel data");
            for (uint32_t k = 0; k < count; ++k, p += pb) put(d + p, i++);
        }
    }
    if ((desc & 0x20) == 0) flip_rows(img);   // stored bottom row first
    return img;
}

// Radiance RGBE (.hdr): "-Y H +X W" scanlines, flat or run-length encoded per channel.  A texture read
// as 8-bit RGBA is tone mapped like stbi_load does for HDR files (its documented defaults): each channel
// m * 2^(e - 136), then 255 * x^(1/2.2) + 0.5 truncated and clamped; alpha 255.
Image decode_hdr(const uint8_t* d, size_t n) {
    size_t p = 0;
    auto line = [&]() {
        std::string l;
        while (p < n && d[p] != '\n') l.push_back((char)d[p++]);
        if (p >= n) bad("HDR: truncated header");
        ++p;
        return l;
    };
    const std::string magic = line();
    if (magic != "#?RADIANCE" && magic != "#?RGBE") bad("HDR: bad signature");
    for (;;) {
        const std::string l = line();
        if (l.empty()) break;
        if (l.rfind("FORMAT=", 0) == 0 && l != "FORMAT=32-bit_rle_rgbe") bad("HDR: only 32-bit_rle_rgbe is supported");
    }
    int H = 0, W = 0;
    {
        const std::string res = line();
        char ya[3] = {0}, xa[3] = {0};
        if (std::sscanf(res.c_str(), "%2s %d %2s %d", ya, &H, xa, &W) != 4 || std::string(ya) != "-Y" ||
            std::string(xa) != "+X")
            bad("HDR: only -Y H +X W orientation is supported");
    }
    if (W <= 0 || H <= 0 || (uint64_t)W * H > (1ull << 28)) bad("HDR: bad size");
    Image img;
    img.width = (uint32_t)W;
    img.height = (uint32_t)H;
    img.rgba.assign((size_t)W * H * 4, 255);
    std::vector<uint8_t> scan((size_t)W * 4);
    auto to8 = [](uint8_t m, uint8_t e) {
        if (e == 0) return (uint8_t)0;
        const float f = std::ldexp((float)m, (int)e - 136);
        const float z = std::pow(f, 1.0f / 2.2f) * 255.0f + 0.5f;
        return (uint8_t)(z < 0.0f ? 0.0f : (z > 255.0f ? 255.0f : z));
    };
    // Run-length or flat is decided once, by the first scanline, as stbi_load decides it: widths outside
    // [8, 32768) are always flat; otherwise the file is run-length encoded when the first scanline starts
    // with 2, 2 and a length byte below 128.  A flat file is then read flat to the end (a later row that
    // happens to start with those bytes is pixels), and in a run-length file every scanline must carry the
    // header with the image's width (stbi_load fails on a wrong length and restarts its flat decoding from
    // the first pixel on a missing header; both are rejected here).
    const bool rle_file = W >= 8 && W < 32768 && p + 3 <= n && d[p] == 2 && d[p + 1] == 2 && (d[p + 2] & 0x80) == 0;
    for (int y = 0; y < H; ++y) {
        if (rle_file) {
            if (p + 4 > n) bad("HDR: truncated scanline");
            if (d[p] != 2 || d[p + 1] != 2 || (d[p + 2] & 0x80) != 0) bad("HDR: scanline without a run-length header");
            if ((((int)d[p + 2] << 8) | d[p + 3]) != W) bad("HDR: invalid decoded scanline length");
            p += 4;
            for (int c = 0; c < 4; ++c) {   // each channel of the scanline in turn
                int x = 0;
                while (x < W) {
                    if (p >= n) bad("HDR: truncated scanline");
                    int count = d[p++];
                    if (count > 128) {
                        count -= 128;
                        if (p >= n || x + count > W) bad("HDR: bad run");
                        for (int k = 0; k < count; ++k) scan[(size_t)(x + k) * 4 + c] = d[p];
                        ++p;
                    } else {
                        if (count == 0 || x + count > W || p + (size_t)count > n) bad("HDR: bad literal run");
                        for (int k = 0; k < count; ++k) scan[(size_t)(x + k) * 4 + c] = d[p++];
                    }
                    x += count;
                }
            }
        } else {
            if (p + (size_t)W * 4 > n) bad("HDR: truncated scanline");
            std::memcpy(scan.data(), d + p, (size_t)W * 4);
            p += (size_t)W * 4;
        }
        for (int x = 0; x < W; ++x) {
            const uint8_t* e = &scan[(size_t)x * 4];
            uint8_t* o = &img.rgba[((size_t)y * W + x) * 4];
            for (int c = 0; c < 3; ++c) o[c] = to8(e[c], e[3]);
        }
    }
    return img;
}

// GIF (87a / 89a): the first image, placed on a canvas of the logical screen size that starts transparent
// black; global or local colour table, the graphic-control transparent index, interlaced rows.  LZW codes
// grow from min size + 1 bits to 12 as the table fills (clear and end codes as the format defines).
Image decode_gif(const uint8_t* d, size_t n) {
    if (n < 13 || (std::memcmp(d, "GIF87a", 6) != 0 && std::memcmp(d, "GIF89a", 6) != 0)) bad("GIF: bad signature");
    const uint32_t W = le16(d + 6), H = le16(d + 8), flags = d[10];
    if (W == 0 || H == 0) bad("GIF: bad size");
    if ((uint64_t)W * H > (1ull << 28)) bad("GIF: too large (more than 2^28 pixels)");
    size_t p = 13;
    std::vector<uint8_t> gct;
    if (flags & 0x80) {
        const size_t sz = 3u << ((flags & 7) + 1);
        if (p + sz > n) bad("GIF: truncated colour table");
        gct.assign(d + p, d + p + sz);
        p += sz;
    }
    int transparent = -1;
    for (;;) {
        if (p >= n) bad("GIF: truncated");
        const uint8_t b = d[p++];
        if (b == 0x3B) bad("GIF: no image");
        if (b == 0x21) {   // extension: graphic control keeps the transparent index; the rest is skipped
            if (p >= n) bad("GIF: truncated extension");
            const uint8_t label = d[p++];
            bool first = true;
            for (;;) {
                if (p >= n) bad("GIF: truncated extension");
                const uint8_t len = d[p++];
                if (len == 0) break;
                if (p + len > n) bad("GIF: truncated extension");
                if (label == 0xF9 && first && len >= 4 && (d[p] & 1)) transparent = d[p + 3];
                first = false;
                p += len;
            }
            continue;
        }
        if (b != 0x2C) bad("GIF: unknown block");
        if (p + 9 > n) bad("GIF: truncated image descriptor");
        const uint32_t left = le16(d + p), top = le16(d + p + 2), iw = le16(d + p + 4), ih = le16(d + p + 6), f = d[p + 8];
        p += 9;
        if ((uint64_t)iw * ih > (1ull << 28)) bad("GIF: image too large (more than 2^28 pixels)");
        std::vector<uint8_t> table = gct;
        if (f & 0x80) {
            const size_t sz = 3u << ((f & 7) + 1);
            if (p + sz > n) bad("GIF: truncated colour table");
            table.assign(d + p, d + p + sz);
            p += sz;
        }
        if (table.empty()) bad("GIF: no colour table");
        if (p >= n) bad("GIF: truncated image data");
        const int min_size = d[p++];
        if (min_size < 2 || min_size > 8) bad("GIF: bad LZW code size");
        std::vector<uint8_t> lzw;   // the data sub-blocks joined
        for (;;) {
            if (p >= n) bad("GIF: truncated image data");
            const uint8_t len = d[p++];
            if (len == 0) break;
            if (p + len > n) bad("GIF: truncated image data");
            lzw.insert(lzw.end(), d + p, d + p + len);
            p += len;
        }
        // LZW: table entries as (prefix code, last byte); strings are rebuilt back to front
        const int clear = 1 << min_size, end = clear + 1;
        std::vector<uint16_t> prefix(4096);
        std::vector<uint8_t> suffix(4096), first_byte(4096), stack;
        std::vector<uint16_t> length(4096);
        for (int c = 0; c < clear; ++c) { prefix[c] = 0xFFFF; suffix[c] = first_byte[c] = (uint8_t)c; length[c] = 1; }
        std::vector<uint8_t> idx;
        idx.reserve((size_t)iw * ih);
        int size = min_size + 1, next = end + 1, prev = -1;
        size_t bitpos = 0;
        const size_t total_bits = lzw.size() * 8;
        while (idx.size() < (size_t)iw * ih) {
            if (bitpos + (size_t)size > total_bits) break;   // short data: the rest stays transparent
            int code = 0;
            for (int k = 0; k < size; ++k, ++bitpos) code |= ((lzw[bitpos / 8] >> (bitpos % 8)) & 1) << k;
            if (code == clear) {
                size = min_size + 1;
                next = end + 1;
                prev = -1;
                continue;
            }
            if (code == end) break;
            if (prev < 0) {
                if (code >= clear) bad("GIF: bad first code");
                idx.push_back((uint8_t)code);
                prev = code;
                continue;
            }
            int out = code;
            uint8_t fb;
            if (code < next) {
                fb = first_byte[code];
            } else if (code == next) {   // the string being defined: previous string + its first byte
                fb = first_byte[prev];
            } else {
                bad("GIF: bad LZW code");
            }
            if (next < 4096) {
                prefix[next] = (uint16_t)prev;
                suffix[next] = fb;
                first_byte[next] = first_byte[prev];
                length[next] = (uint16_t)(length[prev] + 1);
                ++next;
                if (next == (1 << size) && size < 12) ++size;
            }
            stack.clear();
            for (int c = out; c != 0xFFFF; c = prefix[c]) stack.push_back(suffix[c]);
            for (size_t k = stack.size(); k-- > 0;) idx.push_back(stack[k]);
            prev = code;
        }
        Image img;
        img.width = W;
        img.height = H;
        img.rgba.assign((size_t)W * H * 4, 0);
        const bool interlaced = (f & 0x40) != 0;
        std::vector<uint32_t> rows(ih);
        if (interlaced) {
            uint32_t r = 0;
            for (const auto& pass : {std::make_pair(0u, 8u), std::make_pair(4u, 8u), std::make_pair(2u, 4u), std::make_pair(1u, 2u)})
                for (uint32_t y = pass.first; y < ih; y += pass.second) rows[r++] = y;
        } else {
            for (uint32_t y = 0; y < ih; ++y) rows[y] = y;
        }
        for (size_t i = 0; i < idx.size() && i < (size_t)iw * ih; ++i) {
            const uint32_t x = left + (uint32_t)(i % iw), y = top + rows[i / iw];
            if (x >= W || y >= H || idx[i] == transparent) continue;
            if ((size_t)idx[i] * 3 + 3 > table.size()) bad("GIF: colour index out of range");
            uint8_t* o = &img.rgba[((size_t)y * W + x) * 4];
            o[0] = table[idx[i] * 3u];
            o[1] = table[idx[i] * 3u + 1];
            o[2] = table[idx[i] * 3u + 2];
            o[3] = 255;
        }
        return img;
    }
}

}  // namespace

Image decode_image(const uint8_t* data, size_t n) {
    static const uint8_t kPngSig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (n >= 8 && std::memcmp(data, kPngSig, 8) == 0) return decode_png(data, n);
    if (n >= 3 && data[0] == 0xFF && data[1] == 0xD8 && data[2] == 0xFF) return decode_jpeg(data, n);
    if (n >= 2 && data[0] == 'B' && data[1] == 'M') return decode_bmp(data, n);
    if (n >= 6 && (std::memcmp(data, "#?RADIANCE", std::min<size_t>(n, 10)) == 0 || std::memcmp(data, "#?RGBE", 6) == 0))
        return decode_hdr(data, n);
    if (n >= 6 && (std::memcmp(data, "GIF87a", 6) == 0 || std::memcmp(data, "GIF89a", 6) == 0)) return decode_gif(data, n);
    if (looks_like_tga(data, n)) return decode_tga(data, n);   // TGA has no signature: a plausible header
    bad("unknown image format (PNG, JPEG, BMP, GIF, TGA or HDR expected)");
}

void flip_rows(Image& img) {
    const size_t stride = (size_t)img.width * 4;
    for (uint32_t y = 0; y < img.height / 2; ++y)
        std::swap_ranges(img.rgba.begin() + (ptrdiff_t)(y * stride), img.rgba.begin() + (ptrdiff_t)((y + 1) * stride),
                         img.rgba.begin() + (ptrdiff_t)((img.height - 1 - y) * stride));
}

Image load_image(const std::string& path, bool flip_vertically) {
    std::ifstream f(path, std::ios::binary);
    if (!f) fail(REINA_ERR_IO, "Could not load image at path: " + path);
    std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    Image img;
    try {
        img = decode_image(bytes.data(), bytes.size());
    } catch (const Error& e) {
        fail(e.code, "Could not load image at path: " + path + ": " + e.what());
    }
    if (flip_vertically) flip_rows(img);
    return img;
}

}  // namespace rt
