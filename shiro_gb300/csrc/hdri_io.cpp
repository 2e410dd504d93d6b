// hdri_io.cpp - environment images from disk without OpenImageIO, for C and
// C++ hosts (shiro_hdri_load / shiro_hdri_decode in include/shiro_gpu.h).
//
// The reference loads a dome light's image with OpenImageIO
// (EnvironmentMap::Load, src/render/EnvironmentMap.cpp:49-92): any readable
// image becomes float RGB texels, row 0 at the top, channel 0 as red, channel
// 1 (else red) as green, channel 2 (else green) as blue.  Built without
// OpenImageIO it loads nothing.  This reader covers the two formats HDR
// environments ship in, with the same results as shiro_gb300/hdri.py:
//  * Radiance RGBE: "#?" signature, FORMAT=32-bit_rle_rgbe (or none), all
//    eight resolution-line orientations, flat, old-style (1,1,1,n) and
//    new-style per-component run-length scanlines; a texel reads as
//    mantissa * 2^(exponent - 136), exponent 0 black (rgbe.c's convention);
//  * OpenEXR: single-part scanline files, HALF / FLOAT / UINT channels,
//    compression NONE, RLE, ZIPS, ZIP (the zlib stream decoded by the
//    inflater below, then OpenEXR's delta predictor and byte interleave
//    undone); PIZ, PXR24, B44 and DWA are refused.  R, G, B are used when
//    present (a missing one repeats the previous), else Y, else the first
//    non-alpha channels in name order.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/shiro_gpu.h"

namespace {

struct HdriError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

using Bytes = std::vector<uint8_t>;

// ---- DEFLATE (RFC 1951) inside a zlib stream (RFC 1950) ----------------------
class Inflater {
public:
    Inflater(const uint8_t* p, size_t n) : p_(p), n_(n) {}

    Bytes Run(size_t expect) {
        if (n_ < 2) throw HdriError("zlib stream too short");
        const uint32_t cmf = p_[0], flg = p_[1];
        if ((cmf & 0x0f) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20))
            throw HdriError("not a zlib deflate stream");
        pos_ = 16;  // bit position after the two header bytes
        out_.reserve(expect);
        bool last = false;
        while (!last) {
            last = Bits(1) != 0;
            const uint32_t type = Bits(2);
            if (type == 0) Stored();
            else if (type == 1) Fixed();
            else if (type == 2) Dynamic();
            else throw HdriError("invalid deflate block type");
            if (out_.size() > expect) throw HdriError("zip chunk decodes past its size");
        }
        return std::move(out_);
    }

private:
    struct Huffman {
        uint16_t count[16] = {};
        std::vector<uint16_t> symbol;
    };

    uint32_t Bits(int k) {
        uint32_t v = 0;
        for (int i = 0; i < k; ++i, ++pos_) {
            const size_t byte = pos_ >> 3;
            if (byte >= n_) throw HdriError("zlib stream ends early");
            v |= static_cast<uint32_t>((p_[byte] >> (pos_ & 7)) & 1u) << i;
        }
        return v;
    }

    static Huffman Build(const uint8_t* lengths, int n) {
        Huffman h;
        h.symbol.assign(n, 0);
        for (int i = 0; i < n; ++i) h.count[lengths[i]]++;
        h.count[0] = 0;
        uint16_t offs[16] = {};
        for (int l = 1; l < 16; ++l) offs[l] = static_cast<uint16_t>(offs[l - 1] + h.count[l - 1]);
        for (int i = 0; i < n; ++i)
            if (lengths[i]) h.symbol[offs[lengths[i]]++] = static_cast<uint16_t>(i);
        return h;
    }

    // canonical decoding, one bit at a time (codes are read MSB first)
    int Decode(const Huffman& h) {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= static_cast<int>(Bits(1));
            const int count = h.count[len];
            if (code - count < first) return h.symbol[index + (code - first)];
            index += count;
            first = (first + count) << 1;
            code <<= 1;
        }
        throw HdriError("invalid deflate code");
    }

    void Stored() {
        pos_ = (pos_ + 7) & ~static_cast<size_t>(7);
        const uint32_t len = Bits(16), nlen = Bits(16);
        if ((len ^ 0xffffu) != nlen) throw HdriError("corrupt stored deflate block");
        const size_t byte = pos_ >> 3;
        if (byte + len > n_) throw HdriError("zlib stream ends early");
        out_.insert(out_.end(), p_ + byte, p_ + byte + len);
        pos_ += 8ull * len;
    }

    void Codes(const Huffman& lit, const Huffman& dist) {
        static const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                              31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
        static const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                                              2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
        static const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,
                                               33,  49,  65,  97,  129, 193,  257,  385,  513,  769,
                                               1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
        static const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                               6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
        for (;;) {
            const int sym = Decode(lit);
            if (sym < 256) {
                out_.push_back(static_cast<uint8_t>(sym));
            } else if (sym == 256) {
                return;
            } else {
                const int li = sym - 257;
                if (li >= 29) throw HdriError("invalid deflate length code");
                const size_t len = kLenBase[li] + Bits(kLenExtra[li]);
                const int di = Decode(dist);
                if (di >= 30) throw HdriError("invalid deflate distance code");
                const size_t d = kDistBase[di] + Bits(kDistExtra[di]);
                if (d > out_.size()) throw HdriError("deflate distance before the start");
                const size_t from = out_.size() - d;
                for (size_t k = 0; k < len; ++k) out_.push_back(out_[from + k]);
            }
        }
    }

    void Fixed() {
        uint8_t l[288], d[30];
        for (int i = 0; i < 144; ++i) l[i] = 8;
        for (int i = 144; i < 256; ++i) l[i] = 9;
        for (int i = 256; i < 280; ++i) l[i] = 7;
        for (int i = 280; i < 288; ++i) l[i] = 8;
        for (int i = 0; i < 30; ++i) d[i] = 5;
        Codes(Build(l, 288), Build(d, 30));
    }

    void Dynamic() {
        const int hlit = static_cast<int>(Bits(5)) + 257, hdist = static_cast<int>(Bits(5)) + 1,
                  hclen = static_cast<int>(Bits(4)) + 4;
        static const uint8_t kOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
        uint8_t cl[19] = {};
        for (int i = 0; i < hclen; ++i) cl[kOrder[i]] = static_cast<uint8_t>(Bits(3));
        const Huffman clh = Build(cl, 19);
        uint8_t lens[320] = {};
        int i = 0;
        while (i < hlit + hdist) {
            const int sym = Decode(clh);
            if (sym < 16) {
                lens[i++] = static_cast<uint8_t>(sym);
                continue;
            }
            int rep;
            uint8_t val = 0;
            if (sym == 16) {
                if (i == 0) throw HdriError("deflate repeat with no previous length");
                val = lens[i - 1];
                rep = 3 + static_cast<int>(Bits(2));
            } else if (sym == 17) {
                rep = 3 + static_cast<int>(Bits(3));
            } else {
                rep = 11 + static_cast<int>(Bits(7));
            }
            if (i + rep > hlit + hdist) throw HdriError("deflate code lengths overflow");
            while (rep--) lens[i++] = val;
        }
        Codes(Build(lens, hlit), Build(lens + hlit, hdist));
    }

    const uint8_t* p_;
    size_t n_;
    size_t pos_ = 0;
    Bytes out_;
};

// ---- Radiance RGBE -----------------------------------------------------------
struct Reader {
    const uint8_t* p;
    size_t n;
};

std::string Line(const Reader& r, size_t* pos) {
    size_t end = *pos;
    while (end < r.n && r.p[end] != '\n') ++end;
    if (end >= r.n) throw HdriError("Radiance header is not terminated");
    std::string s(reinterpret_cast<const char*>(r.p + *pos), end - *pos);
    *pos = end + 1;
    // strip surrounding white space
    size_t a = 0, b = s.size();
    while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) ++a;
    while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) --b;
    return s.substr(a, b - a);
}

void Scanline(const Reader& r, size_t* pos, uint32_t width, uint8_t* quads) {
    size_t p = *pos;
    if (width >= 8 && width <= 0x7fff && p + 4 <= r.n && r.p[p] == 2 && r.p[p + 1] == 2 && !(r.p[p + 2] & 0x80)) {
        if (((static_cast<uint32_t>(r.p[p + 2]) << 8) | r.p[p + 3]) != width)
            throw HdriError("RGBE scanline length does not match the image width");
        p += 4;
        for (int c = 0; c < 4; ++c) {
            uint32_t x = 0;
            while (x < width) {
                if (p >= r.n) throw HdriError("RGBE data ends inside a scanline");
                const uint32_t code = r.p[p++];
                if (code > 128) {
                    const uint32_t count = code - 128;
                    if (x + count > width || p >= r.n) throw HdriError("RGBE run overflows its scanline");
                    for (uint32_t k = 0; k < count; ++k) quads[4 * (x + k) + c] = r.p[p];
                    ++p;
                    x += count;
                } else {
                    const uint32_t count = code;
                    if (count == 0 || x + count > width || p + count > r.n)
                        throw HdriError("RGBE dump overflows its scanline");
                    for (uint32_t k = 0; k < count; ++k) quads[4 * (x + k) + c] = r.p[p + k];
                    p += count;
                    x += count;
                }
            }
        }
        *pos = p;
        return;
    }
    uint32_t x = 0;
    int shift = 0;
    while (x < width) {
        if (p + 4 > r.n) throw HdriError("RGBE data ends inside a scanline");
        const uint8_t* q = r.p + p;
        p += 4;
        if (q[0] == 1 && q[1] == 1 && q[2] == 1) {
            if (x == 0) throw HdriError("RGBE run at the start of a scanline");
            const uint64_t count = static_cast<uint64_t>(q[3]) << shift;
            if (x + count > width) throw HdriError("RGBE run overflows its scanline");
            for (uint64_t k = 0; k < count; ++k) std::memcpy(quads + 4 * (x + k), quads + 4 * (x - 1), 4);
            x += static_cast<uint32_t>(count);
            shift += 8;
        } else {
            std::memcpy(quads + 4 * x, q, 4);
            ++x;
            shift = 0;
        }
    }
    *pos = p;
}

void LoadHdr(const Reader& r, uint32_t* wOut, uint32_t* hOut, std::vector<float>* out) {
    if (r.n < 2 || r.p[0] != '#' || r.p[1] != '?') throw HdriError("not a Radiance file (no #? signature)");
    size_t pos = 0;
    std::string fmt;
    bool haveFmt = false;
    for (;;) {
        const std::string line = Line(r, &pos);
        if (line.empty()) break;
        if (line.compare(0, 7, "FORMAT=") == 0) {
            fmt = line.substr(7);
            while (!fmt.empty() && std::isspace(static_cast<unsigned char>(fmt.back()))) fmt.pop_back();
            while (!fmt.empty() && std::isspace(static_cast<unsigned char>(fmt.front()))) fmt.erase(fmt.begin());
            haveFmt = true;
        }
    }
    if (haveFmt && fmt != "32-bit_rle_rgbe") throw HdriError("unsupported Radiance pixel format " + fmt);
    size_t end = pos;
    while (end < r.n && r.p[end] != '\n') ++end;
    if (end >= r.n) throw HdriError("Radiance resolution line missing");
    const std::string res = Line(r, &pos);
    char s1, a1, s2, a2;
    long n1, n2;
    char tail;
    if (std::sscanf(res.c_str(), "%c%c %ld %c%c %ld%c", &s1, &a1, &n1, &s2, &a2, &n2, &tail) != 6 ||
        (s1 != '-' && s1 != '+') || (s2 != '-' && s2 != '+') || (a1 != 'X' && a1 != 'Y') || (a2 != 'X' && a2 != 'Y') ||
        a1 == a2)
        throw HdriError("malformed Radiance resolution line");
    if (n1 <= 0 || n2 <= 0) throw HdriError("empty Radiance image");
    if (n1 > (1L << 20) || n2 > (1L << 20)) throw HdriError("Radiance image too large");
    std::vector<uint8_t> quads(4 * static_cast<size_t>(n2));
    const uint32_t rows = a1 == 'Y' ? static_cast<uint32_t>(n1) : static_cast<uint32_t>(n2);
    const uint32_t cols = a1 == 'Y' ? static_cast<uint32_t>(n2) : static_cast<uint32_t>(n1);
    out->assign(3 * static_cast<size_t>(rows) * cols, 0.0f);
    for (long k = 0; k < n1; ++k) {
        Scanline(r, &pos, static_cast<uint32_t>(n2), quads.data());
        for (long m = 0; m < n2; ++m) {
            // scanline k, position m -> row / column, the picture's Y axis up
            long row, col;
            if (a1 == 'Y') {
                row = s1 == '+' ? n1 - 1 - k : k;
                col = s2 == '-' ? n2 - 1 - m : m;
            } else {
                col = s1 == '-' ? n1 - 1 - k : k;
                row = s2 == '+' ? n2 - 1 - m : m;
            }
            const uint8_t* q = &quads[4 * m];
            float* o = &(*out)[3 * (static_cast<size_t>(row) * cols + static_cast<size_t>(col))];
            const float scale = q[3] > 0 ? std::ldexp(1.0f, static_cast<int>(q[3]) - 136) : 0.0f;
            for (int c = 0; c < 3; ++c) o[c] = static_cast<float>(q[c]) * scale;
        }
    }
    *wOut = cols;
    *hOut = rows;
}

// ---- OpenEXR -----------------------------------------------------------------
float HalfToFloat(uint16_t h) {
    const uint32_t sign = static_cast<uint32_t>(h >> 15) << 31;
    const uint32_t exp = (h >> 10) & 0x1fu, man = h & 0x3ffu;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign;
        } else {  // subnormal half: normalise
            int e = -1;
            uint32_t m = man;
            do {
                ++e;
                m <<= 1;
            } while (!(m & 0x400u));
            bits = sign | (static_cast<uint32_t>(127 - 15 - e) << 23) | ((m & 0x3ffu) << 13);
        }
    } else if (exp == 31) {
        bits = sign | 0x7f800000u | (man << 13);
    } else {
        bits = sign | ((exp + 112u) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

template <typename T>
T Le(const uint8_t* p) {
    T v;
    std::memcpy(&v, p, sizeof(T));
    return v;
}

struct ExrChannel {
    std::string name;
    int32_t type;
};

Bytes Unpredict(const Bytes& t) {
    Bytes b(t.size());
    if (t.empty()) return b;
    b[0] = t[0];
    for (size_t i = 1; i < t.size(); ++i) b[i] = static_cast<uint8_t>(b[i - 1] + t[i] - 128);
    Bytes out(t.size());
    const size_t half = (b.size() + 1) / 2;
    for (size_t i = 0; i < half; ++i) out[2 * i] = b[i];
    for (size_t i = half; i < b.size(); ++i) out[2 * (i - half) + 1] = b[i];
    return out;
}

Bytes RleDecode(const uint8_t* p, size_t n, size_t expect) {
    Bytes out;
    size_t pos = 0;
    while (pos < n) {
        const int count = static_cast<int8_t>(p[pos++]);
        if (count < 0) {
            if (pos + static_cast<size_t>(-count) > n) throw HdriError("OpenEXR RLE literal overflows its chunk");
            out.insert(out.end(), p + pos, p + pos - count);
            pos += static_cast<size_t>(-count);
        } else {
            if (pos >= n) throw HdriError("OpenEXR RLE run overflows its chunk");
            out.insert(out.end(), static_cast<size_t>(count) + 1, p[pos]);
            ++pos;
        }
        if (out.size() > expect) throw HdriError("OpenEXR RLE chunk decodes past its size");
    }
    return out;
}

Bytes Decompress(int comp, const uint8_t* p, size_t n, size_t expect) {
    if (n >= expect) return Bytes(p, p + expect);  // stored raw when compression would not shrink it
    if (comp == 0) throw HdriError("truncated OpenEXR chunk");
    Bytes tmp;
    if (comp == 2 || comp == 3) tmp = Inflater(p, n).Run(expect);
    else if (comp == 1) tmp = RleDecode(p, n, expect);
    else throw HdriError("OpenEXR compression not supported");
    if (tmp.size() != expect) throw HdriError("OpenEXR chunk decodes to the wrong size");
    return Unpredict(tmp);
}

std::string Suffix(const std::string& n) {
    const size_t d = n.rfind('.');
    return d == std::string::npos ? n : n.substr(d + 1);
}

void PickChannels(const std::vector<ExrChannel>& ch, int pick[3]) {
    auto find = [&](const char* want) -> int {
        for (size_t i = 0; i < ch.size(); ++i)
            if (ch[i].name == want) return static_cast<int>(i);
        for (size_t i = 0; i < ch.size(); ++i)
            if (Suffix(ch[i].name) == want) return static_cast<int>(i);
        return -1;
    };
    const int r = find("R"), g = find("G"), b = find("B");
    if (r >= 0) {
        pick[0] = r;
        pick[1] = g >= 0 ? g : r;
        pick[2] = b >= 0 ? b : pick[1];
        return;
    }
    const int y = find("Y");
    if (y >= 0) {
        pick[0] = pick[1] = pick[2] = y;
        return;
    }
    std::vector<int> order;
    for (size_t i = 0; i < ch.size(); ++i)
        if (Suffix(ch[i].name) != "A") order.push_back(static_cast<int>(i));
    if (order.empty())
        for (size_t i = 0; i < ch.size(); ++i) order.push_back(static_cast<int>(i));
    pick[0] = order[0];
    pick[1] = order.size() > 1 ? order[1] : pick[0];
    pick[2] = order.size() > 2 ? order[2] : pick[1];
}

void LoadExr(const Reader& r, uint32_t* wOut, uint32_t* hOut, std::vector<float>* out) {
    if (r.n < 8) throw HdriError("not an OpenEXR file");
    if (Le<int32_t>(r.p) != 20000630) throw HdriError("not an OpenEXR file (bad magic number)");
    const int32_t version = Le<int32_t>(r.p + 4);
    if ((version & 0xff) != 2) throw HdriError("unsupported OpenEXR version");
    if (version & 0x200) throw HdriError("tiled OpenEXR images are not supported");
    if (version & (0x800 | 0x1000)) throw HdriError("deep or multi-part OpenEXR images are not supported");
    size_t pos = 8;
    const uint8_t *chRaw = nullptr, *dwRaw = nullptr;
    int32_t chSize = 0;
    int comp = -1;
    auto cstr = [&](size_t at, size_t* end) {
        size_t e = at;
        while (e < r.n && r.p[e]) ++e;
        if (e >= r.n) throw HdriError("OpenEXR header is not terminated");
        *end = e;
        return std::string(reinterpret_cast<const char*>(r.p + at), e - at);
    };
    for (;;) {
        size_t e;
        const std::string name = cstr(pos, &e);
        pos = e + 1;
        if (name.empty()) break;
        const std::string type = cstr(pos, &e);
        pos = e + 1;
        if (pos + 4 > r.n) throw HdriError("truncated OpenEXR attribute");
        const int32_t size = Le<int32_t>(r.p + pos);
        pos += 4;
        if (size < 0 || pos + static_cast<size_t>(size) > r.n) throw HdriError("truncated OpenEXR attribute value");
        if (name == "channels") {
            chRaw = r.p + pos;
            chSize = size;
        } else if (name == "compression" && size >= 1) {
            comp = r.p[pos];
        } else if (name == "dataWindow" && size >= 16) {
            dwRaw = r.p + pos;
        }
        pos += static_cast<size_t>(size);
    }
    if (!chRaw) throw HdriError("OpenEXR header lacks 'channels'");
    if (comp < 0) throw HdriError("OpenEXR header lacks 'compression'");
    if (!dwRaw) throw HdriError("OpenEXR header lacks 'dataWindow'");
    std::vector<ExrChannel> ch;
    for (size_t q = 0; q < static_cast<size_t>(chSize);) {
        size_t e = q;
        while (e < static_cast<size_t>(chSize) && chRaw[e]) ++e;
        if (e >= static_cast<size_t>(chSize)) throw HdriError("malformed OpenEXR channel list");
        const std::string name(reinterpret_cast<const char*>(chRaw + q), e - q);
        q = e + 1;
        if (name.empty()) break;
        if (q + 16 > static_cast<size_t>(chSize)) throw HdriError("malformed OpenEXR channel list");
        const int32_t type = Le<int32_t>(chRaw + q), xs = Le<int32_t>(chRaw + q + 8), ys = Le<int32_t>(chRaw + q + 12);
        q += 16;
        if (type < 0 || type > 2) throw HdriError("OpenEXR channel " + name + ": unknown pixel type");
        if (xs != 1 || ys != 1) throw HdriError("OpenEXR channel " + name + ": subsampled channels are not supported");
        ch.push_back({name, type});
    }
    if (ch.empty()) throw HdriError("OpenEXR image has no channels");
    if (comp > 3) throw HdriError("OpenEXR compression " + std::to_string(comp) + " is not supported");
    const int32_t x0 = Le<int32_t>(dwRaw), y0 = Le<int32_t>(dwRaw + 4), x1 = Le<int32_t>(dwRaw + 8),
                  y1 = Le<int32_t>(dwRaw + 12);
    const int64_t width = static_cast<int64_t>(x1) - x0 + 1, height = static_cast<int64_t>(y1) - y0 + 1;
    if (width <= 0 || height <= 0) throw HdriError("empty OpenEXR data window");
    if (width > (1 << 20) || height > (1 << 20)) throw HdriError("OpenEXR image too large");
    const int64_t lpc = comp == 3 ? 16 : 1;
    const int64_t nchunks = (height + lpc - 1) / lpc;
    if (pos + 8 * static_cast<size_t>(nchunks) > r.n) throw HdriError("truncated OpenEXR offset table");
    size_t lineBytes = 0;
    for (const ExrChannel& c : ch) lineBytes += static_cast<size_t>(width) * (c.type == 1 ? 2u : 4u);
    std::vector<std::vector<float>> planes(ch.size(), std::vector<float>(static_cast<size_t>(width * height), 0.0f));
    for (int64_t k = 0; k < nchunks; ++k) {
        const uint64_t off = Le<uint64_t>(r.p + pos + 8 * k);
        if (off + 8 > r.n) throw HdriError("OpenEXR chunk offset past the end of the file");
        const int32_t y = Le<int32_t>(r.p + off), size = Le<int32_t>(r.p + off + 4);
        const int64_t first = static_cast<int64_t>(y) - y0;
        if (first < 0 || first >= height || first % lpc || size < 0 || off + 8 + static_cast<uint64_t>(size) > r.n)
            throw HdriError("malformed OpenEXR chunk");
        const int64_t lines = std::min(lpc, height - first);
        const Bytes raw = Decompress(comp, r.p + off + 8, static_cast<size_t>(size), static_cast<size_t>(lines) * lineBytes);
        size_t p = 0;
        for (int64_t l = 0; l < lines; ++l)
            for (size_t c = 0; c < ch.size(); ++c) {
                float* dst = &planes[c][static_cast<size_t>((first + l) * width)];
                for (int64_t x = 0; x < width; ++x) {
                    if (ch[c].type == 1) {
                        dst[x] = HalfToFloat(Le<uint16_t>(&raw[p]));
                        p += 2;
                    } else if (ch[c].type == 2) {
                        dst[x] = Le<float>(&raw[p]);
                        p += 4;
                    } else {
                        dst[x] = static_cast<float>(Le<uint32_t>(&raw[p]));
                        p += 4;
                    }
                }
            }
    }
    int pick[3];
    PickChannels(ch, pick);
    const size_t n = static_cast<size_t>(width * height);
    out->assign(3 * n, 0.0f);
    for (size_t i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) (*out)[3 * i + c] = planes[static_cast<size_t>(pick[c])][i];
    *wOut = static_cast<uint32_t>(width);
    *hOut = static_cast<uint32_t>(height);
}

int Decode(const uint8_t* data, size_t size, uint32_t* w, uint32_t* h, float** pixels, char* error, size_t errorSize) {
    auto say = [&](const std::string& m) {
        if (error && errorSize) std::snprintf(error, errorSize, "%s", m.c_str());
    };
    if (!w || !h || !pixels || (!data && size)) {
        say("null argument");
        return SHIRO_ERR_INVALID_ARGUMENT;
    }
    *pixels = nullptr;
    *w = *h = 0;
    try {
        const Reader r{data, size};
        std::vector<float> out;
        uint32_t ww = 0, hh = 0;
        if (size >= 4 && Le<int32_t>(data) == 20000630) LoadExr(r, &ww, &hh, &out);
        else if (size >= 2 && data[0] == '#' && data[1] == '?') LoadHdr(r, &ww, &hh, &out);
        else throw HdriError("unrecognised image format (expected Radiance .hdr or OpenEXR .exr)");
        float* buf = static_cast<float*>(std::malloc(std::max<size_t>(out.size(), 1) * sizeof(float)));
        if (!buf) {
            say("out of host memory");
            return SHIRO_ERR_OUT_OF_MEMORY;
        }
        std::memcpy(buf, out.data(), out.size() * sizeof(float));
        *pixels = buf;
        *w = ww;
        *h = hh;
        say("");
        return SHIRO_OK;
    } catch (const std::exception& e) {
        say(e.what());
        return SHIRO_ERR_INVALID_ARGUMENT;
    }
}

}  // namespace

extern "C" {

int shiro_hdri_decode(const void* data, size_t size, uint32_t* width, uint32_t* height, float** pixels, char* error,
                      size_t error_size) {
    return Decode(static_cast<const uint8_t*>(data), size, width, height, pixels, error, error_size);
}

int shiro_hdri_load(const char* path, uint32_t* width, uint32_t* height, float** pixels, char* error, size_t error_size) {
    if (!path) {
        if (error && error_size) std::snprintf(error, error_size, "null path");
        return SHIRO_ERR_INVALID_ARGUMENT;
    }
    std::FILE* f = std::fopen(path, "rb");
    if (!f) {
        if (error && error_size) std::snprintf(error, error_size, "cannot open %s", path);
        return SHIRO_ERR_INVALID_ARGUMENT;
    }
    std::vector<uint8_t> data;
    uint8_t buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) data.insert(data.end(), buf, buf + got);
    std::fclose(f);
    return Decode(data.data(), data.size(), width, height, pixels, error, error_size);
}

void shiro_hdri_free(float* pixels) { std::free(pixels); }

}  // extern "C"
