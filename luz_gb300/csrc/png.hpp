// png.hpp — PNG decoding to RGBA8 for the scene importers (glTF images, OBJ texture
// maps). Written from the specifications: zlib stream (RFC 1950) with DEFLATE blocks
// (RFC 1951: stored, fixed and dynamic Huffman), PNG chunks, the five scanline
// filters and Adam7 interlacing (PNG, ISO/IEC 15948). All colour types and bit
// depths; 16-bit samples keep their high byte, sub-byte grey samples are scaled to
// 0..255, tRNS becomes alpha.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace luz {
namespace png {

[[noreturn]] inline void fail(const char* what) { throw std::runtime_error(std::string("PNG: ") + what); }

// ---------------------------------------------------------------- inflate
class BitReader {
public:
    BitReader(const uint8_t* p, size_t n) : p_(p), n_(n) {}
    uint32_t bits(int k) {   // k <= 24
        while (cnt_ < k) {
            if (pos_ >= n_) fail("truncated deflate stream");
            acc_ |= (uint32_t)p_[pos_++] << cnt_;
            cnt_ += 8;
        }
        uint32_t v = acc_ & ((1u << k) - 1u);
        acc_ >>= k;
        cnt_ -= k;
        return v;
    }
    void align() { acc_ = 0; cnt_ = 0; }
    size_t pos() const { return pos_; }
    void skip(size_t k) { pos_ += k; }
    const uint8_t* data() const { return p_; }
    size_t size() const { return n_; }

private:
    const uint8_t* p_;
    size_t n_, pos_ = 0;
    uint32_t acc_ = 0;
    int cnt_ = 0;
};

// Canonical Huffman code: counts per length and symbols sorted by code.
struct Huffman {
    uint16_t count[16] = {};
    std::vector<uint16_t> symbol;
    void build(const uint8_t* lengths, int n) {
        memset(count, 0, sizeof count);
        for (int s = 0; s < n; ++s) count[lengths[s]]++;
        count[0] = 0;
        uint16_t offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + count[l];
        symbol.assign(n, 0);
        for (int s = 0; s < n; ++s)
            if (lengths[s]) symbol[offs[lengths[s]]++] = (uint16_t)s;
    }
    int decode(BitReader& br) const {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; ++l) {
            code |= (int)br.bits(1);
            int c = count[l];
            if (code - c < first) return symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
        }
        fail("bad Huffman code");
    }
};

// Decodes one Huffman block into out; stops early once out holds `limit` bytes (it
// may then hold up to one match, 258 bytes, more).
inline void inflate_block(BitReader& br, std::vector<uint8_t>& out, const Huffman& lit, const Huffman& dist,
                          size_t limit) {
    static const uint16_t lbase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                                       35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
    static const uint8_t lextra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2,
                                       3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    static const uint16_t dbase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                       193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097,
                                       6145, 8193, 12289, 16385, 24577};
    static const uint8_t dextra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6,
                                       6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
    while (out.size() < limit) {
        int sym = lit.decode(br);
        if (sym < 256) { out.push_back((uint8_t)sym); continue; }
        if (sym == 256) return;
        sym -= 257;
        if (sym >= 29) fail("bad length symbol");
        size_t len = lbase[sym] + br.bits(lextra[sym]);
        int ds = dist.decode(br);
        if (ds >= 30) fail("bad distance symbol");
        size_t d = dbase[ds] + br.bits(dextra[ds]);
        if (d > out.size()) fail("distance beyond output");
        size_t from = out.size() - d;
        for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
    }
}

// zlib stream -> its first `limit` bytes: decoding stops there, so a stream that
// expands beyond what the image needs costs no more memory than the image.
inline std::vector<uint8_t> inflate_zlib(const uint8_t* p, size_t n, size_t limit) {
    if (n < 2) fail("short zlib stream");
    if ((p[0] & 0x0F) != 8 || ((p[0] << 8) | p[1]) % 31 != 0 || (p[1] & 0x20)) fail("bad zlib header");
    BitReader br(p + 2, n - 2);
    std::vector<uint8_t> out;
    Huffman fl, fd;
    {
        uint8_t l[288];
        for (int s = 0; s < 144; ++s) l[s] = 8;
        for (int s = 144; s < 256; ++s) l[s] = 9;
        for (int s = 256; s < 280; ++s) l[s] = 7;
        for (int s = 280; s < 288; ++s) l[s] = 8;
        fl.build(l, 288);
        uint8_t d[30];
        for (int s = 0; s < 30; ++s) d[s] = 5;
        fd.build(d, 30);
    }
    for (;;) {
        uint32_t last = br.bits(1), type = br.bits(2);
        if (type == 0) {
            br.align();
            size_t pos = br.pos();
            if (pos + 4 > br.size()) fail("truncated stored block");
            const uint8_t* q = br.data() + pos;
            uint32_t len = q[0] | (q[1] << 8), nlen = q[2] | (q[3] << 8);
            if ((len ^ 0xFFFFu) != nlen) fail("stored block length check");
            if (pos + 4 + len > br.size()) fail("truncated stored block");
            out.insert(out.end(), q + 4, q + 4 + std::min<size_t>(len, limit - out.size()));
            br.skip(4 + len);
        } else if (type == 1) {
            inflate_block(br, out, fl, fd, limit);
        } else if (type == 2) {
            int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int k = 0; k < hclen; ++k) cl[order[k]] = (uint8_t)br.bits(3);
            Huffman ch;
            ch.build(cl, 19);
            uint8_t lens[320] = {};
            int k = 0;
            while (k < hlit + hdist) {
                int sym = ch.decode(br);
                if (sym < 16) { lens[k++] = (uint8_t)sym; continue; }
                int rep = 0;
                uint8_t val = 0;
                if (sym == 16) {
                    if (k == 0) fail("repeat without a length");
                    val = lens[k - 1];
                    rep = 3 + (int)br.bits(2);
                } else if (sym == 17) {
                    rep = 3 + (int)br.bits(3);
                } else {
                    rep = 11 + (int)br.bits(7);
                }
                if (k + rep > hlit + hdist) fail("code lengths overflow");
                while (rep--) lens[k++] = val;
            }
            Huffman dl, dd;
            dl.build(lens, hlit);
            dd.build(lens + hlit, hdist);
            inflate_block(br, out, dl, dd, limit);
        } else {
            fail("bad block type");
        }
        if (last || out.size() >= limit) break;
    }
    if (out.size() > limit) out.resize(limit);
    return out;
}

// ---------------------------------------------------------------- PNG
inline uint32_t be32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

inline uint8_t paeth(int a, int b, int c) {
    int p = a + b - c;
    int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    if (pa <= pb && pa <= pc) return (uint8_t)a;
    if (pb <= pc) return (uint8_t)b;
    return (uint8_t)c;
}

// Undoes the scanline filters of one (sub)image in place; returns the filtered-out rows.
inline void unfilter(uint8_t* data, uint32_t rows, size_t stride, size_t bpp, std::vector<uint8_t>& out) {
    out.assign(rows * stride, 0);
    std::vector<uint8_t> zero(stride, 0);
    for (uint32_t y = 0; y < rows; ++y) {
        const uint8_t* in = data + y * (stride + 1);
        uint8_t f = in[0];
        ++in;
        uint8_t* cur = out.data() + y * stride;
        const uint8_t* prev = y ? out.data() + (y - 1) * stride : zero.data();
        for (size_t x = 0; x < stride; ++x) {
            int a = x >= bpp ? cur[x - bpp] : 0, b = prev[x], c = x >= bpp ? prev[x - bpp] : 0;
            int v = in[x];
            switch (f) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: fail("bad filter type");
            }
            cur[x] = (uint8_t)v;
        }
    }
}

struct Image {
    uint32_t width = 0, height = 0;
    std::vector<uint8_t> rgba;   // width * height * 4
};

inline bool is_png(const uint8_t* p, size_t n) {
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    return n >= 8 && memcmp(p, sig, 8) == 0;
}

inline Image decode(const uint8_t* p, size_t n) {
    if (!is_png(p, n)) fail("not a PNG file");
    size_t pos = 8;
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte, trns;
    while (pos + 12 <= n) {
        uint32_t len = be32(p + pos);
        const uint8_t* type = p + pos + 4;
        const uint8_t* d = p + pos + 8;
        if (pos + 12 + (size_t)len > n) fail("truncated chunk");
        if (!memcmp(type, "IHDR", 4)) {
            if (len < 13) fail("short IHDR");
            w = be32(d);
            h = be32(d + 4);
            depth = d[8];
            ctype = d[9];
            if (d[10] != 0 || d[11] != 0) fail("unknown compression or filter method");
            interlace = d[12];
        } else if (!memcmp(type, "PLTE", 4)) {
            plte.assign(d, d + len);
        } else if (!memcmp(type, "tRNS", 4)) {
            trns.assign(d, d + len);
        } else if (!memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), d, d + len);
        } else if (!memcmp(type, "IEND", 4)) {
            break;
        }
        pos += 12 + len;
    }
    if (w == 0 || h == 0 || w > (1u << 16) || h > (1u << 16)) fail("bad image size");
    int channels;
    switch (ctype) {
        case 0: channels = 1; break;
        case 2: channels = 3; break;
        case 3: channels = 1; break;
        case 4: channels = 2; break;
        case 6: channels = 4; break;
        default: fail("bad colour type");
    }
    bool ok_depth = depth == 8 || depth == 16 || ((ctype == 0 || ctype == 3) && (depth == 1 || depth == 2 || depth == 4));
    if (!ok_depth || (ctype == 3 && depth == 16)) fail("bad bit depth");
    if (ctype == 3 && plte.empty()) fail("palette image without PLTE");
    const size_t bits_pp = (size_t)channels * depth;
    const size_t bpp = bits_pp < 8 ? 1 : bits_pp / 8;
    static const int x0[7] = {0, 4, 0, 2, 0, 1, 0}, y0[7] = {0, 0, 4, 0, 2, 0, 1};
    static const int dx[7] = {8, 8, 4, 4, 2, 2, 1}, dy[7] = {8, 8, 8, 4, 4, 2, 2};
    auto pass_size = [&](int pass, uint32_t& pw, uint32_t& ph) {   // Adam7 pass extent
        pw = w > (uint32_t)x0[pass] ? (w - x0[pass] + dx[pass] - 1) / dx[pass] : 0;
        ph = h > (uint32_t)y0[pass] ? (h - y0[pass] + dy[pass] - 1) / dy[pass] : 0;
    };
    // The filtered scanlines the header implies: the image data is decoded up to that
    // size, and nothing of the image's own size is allocated before it is there.
    size_t expected = 0;
    if (!interlace) {
        expected = (((size_t)w * bits_pp + 7) / 8 + 1) * h;
    } else {
        for (int pass = 0; pass < 7; ++pass) {
            uint32_t pw, ph;
            pass_size(pass, pw, ph);
            if (pw && ph) expected += (((size_t)pw * bits_pp + 7) / 8 + 1) * ph;
        }
    }
    std::vector<uint8_t> raw = inflate_zlib(idat.data(), idat.size(), expected);
    if (raw.size() < expected) fail("short image data");

    Image img;
    img.width = w;
    img.height = h;
    img.rgba.assign((size_t)w * h * 4, 0);

    // sample k of a pixel at x in an unfiltered row
    auto sample = [&](const uint8_t* row, uint32_t x, int k) -> uint32_t {
        if (depth == 8) return row[x * channels + k];
        if (depth == 16) return row[(x * channels + k) * 2];     // high byte
        size_t bit = (size_t)x * depth;                        // channels == 1 here
        uint32_t v = (row[bit >> 3] >> (8 - depth - (bit & 7))) & ((1u << depth) - 1u);
        return v;
    };
    auto sample16 = [&](const uint8_t* row, uint32_t x, int k) -> uint32_t {
        return depth == 16 ? ((uint32_t)row[(x * channels + k) * 2] << 8) | row[(x * channels + k) * 2 + 1] : 0u;
    };
    auto put = [&](uint32_t X, uint32_t Y, const uint8_t* row, uint32_t x) {
        uint8_t* o = img.rgba.data() + ((size_t)Y * w + X) * 4;
        const uint32_t scale = depth == 1 ? 255 : depth == 2 ? 0x55 : depth == 4 ? 0x11 : 1;
        if (ctype == 3) {
            uint32_t i = sample(row, x, 0);
            if ((size_t)i * 3 + 2 >= plte.size()) fail("palette index out of range");
            o[0] = plte[i * 3];
            o[1] = plte[i * 3 + 1];
            o[2] = plte[i * 3 + 2];
            o[3] = i < trns.size() ? trns[i] : 255;
        } else if (ctype == 0 || ctype == 4) {
            uint32_t g = sample(row, x, 0);
            uint8_t gv = (uint8_t)(depth < 8 ? g * scale : g);
            o[0] = o[1] = o[2] = gv;
            if (ctype == 4) {
                o[3] = (uint8_t)sample(row, x, 1);
            } else {
                uint32_t key = trns.size() >= 2 ? ((uint32_t)trns[0] << 8) | trns[1] : 0x10000u;
                uint32_t full = depth == 16 ? sample16(row, x, 0) : g;
                o[3] = (trns.size() >= 2 && full == key) ? 0 : 255;
            }
        } else {
            o[0] = (uint8_t)sample(row, x, 0);
            o[1] = (uint8_t)sample(row, x, 1);
            o[2] = (uint8_t)sample(row, x, 2);
            if (ctype == 6) {
                o[3] = (uint8_t)sample(row, x, 3);
            } else {
                bool keyed = false;
                if (trns.size() >= 6) {
                    uint32_t kr = ((uint32_t)trns[0] << 8) | trns[1], kg = ((uint32_t)trns[2] << 8) | trns[3],
                             kb = ((uint32_t)trns[4] << 8) | trns[5];
                    uint32_t r = depth == 16 ? sample16(row, x, 0) : o[0], g2 = depth == 16 ? sample16(row, x, 1) : o[1],
                             b = depth == 16 ? sample16(row, x, 2) : o[2];
                    keyed = r == kr && g2 == kg && b == kb;
                }
                o[3] = keyed ? 0 : 255;
            }
        }
    };

    std::vector<uint8_t> rows;
    if (!interlace) {
        size_t stride = ((size_t)w * bits_pp + 7) / 8;
        if (raw.size() < (stride + 1) * h) fail("short image data");
        unfilter(raw.data(), h, stride, bpp, rows);
        for (uint32_t y = 0; y < h; ++y)
            for (uint32_t x = 0; x < w; ++x) put(x, y, rows.data() + y * stride, x);
    } else {
        size_t off = 0;
        for (int pass = 0; pass < 7; ++pass) {
            uint32_t pw, ph;
            pass_size(pass, pw, ph);
            if (!pw || !ph) continue;
            size_t stride = ((size_t)pw * bits_pp + 7) / 8;
            if (raw.size() < off + (stride + 1) * ph) fail("short interlaced data");
            unfilter(raw.data() + off, ph, stride, bpp, rows);
            off += (stride + 1) * ph;
            for (uint32_t y = 0; y < ph; ++y)
                for (uint32_t x = 0; x < pw; ++x)
                    put(x0[pass] + x * dx[pass], y0[pass] + y * dy[pass], rows.data() + y * stride, x);
        }
    }
    return img;
}

}  // namespace png
}  // namespace luz
