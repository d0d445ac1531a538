// dem.cpp — DEM height fields of XML projects, read without GDAL.
//
// The reference opens the project's <DEM> with GDAL, reads band 1 as
// float32, replaces non-finite and nodata cells by the minimum of the valid
// ones and samples it bilinearly, stretched over the scene domain, for the
// ground grid and for every object placement (readDemHeightField and
// DemHeightField::heightAboveMinimum, facetrtcore.cpp:2618-2697, used at
// :2836-2878 and :2989-2993).  This file restates that, with the same float
// operations, over two raster formats read here:
//   - ESRI ASCII grids (GDAL's AAIGrid: a header of ncols, nrows,
//     xll/yll corner or center, cellsize or dx/dy, optional nodata_value,
//     keys in any case, then the rows from north to south);
//   - baseline GeoTIFF (classic and BigTIFF, either byte order; strips or
//     tiles; chunky or planar; no compression, LZW, deflate or PackBits;
//     predictors 1, 2 and 3; unsigned, signed and IEEE samples of 8-64 bits
//     with float16; the GDAL_NODATA tag 42113).  Band 1 of the first image
//     is read, as GDAL reads it;
//   - non-interlaced PNG of 8 or 16 bits (gray, RGB, palette indices, gray
//     + alpha, RGBA), for textures.
// Any other file fails as the reference's GDALOpen failure does ("Cannot
// open DEM: <path>"); a file that opens but cannot be decoded fails as its
// RasterIO failure does ("Cannot read DEM elevations: <path>").
//
// The decoders follow the published formats: TIFF 6.0 (section 13 for LZW,
// section 14 for the horizontal predictor; the floating-point predictor of
// Adobe's TIFF technical note 3), RFC 1950/1951 for deflate streams.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <climits>
#include <cstdint>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iterator>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/facetcu.h"
#include "host_scene.h"

void facetcu_set_host_error(const std::string& message);

namespace facetcu {
namespace dem {
namespace {

struct OpenError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct ReadError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// A raster as GDAL hands it over: band 1 converted to float32, its nodata.
struct Raster {
    int width = 0, height = 0;
    int bands = 1;  // raster bands (samples per pixel)
    bool has_nodata = false;
    double nodata = 0.0;
    std::vector<float> values;
};

// ---- ASCII grid --------------------------------------------------------------
bool ascii_key(const std::string& word, const char* key)
{
    if (word.size() != std::strlen(key)) return false;
    for (size_t i = 0; i < word.size(); ++i)
        if (std::tolower(static_cast<unsigned char>(word[i])) != key[i]) return false;
    return true;
}

bool looks_ascii_grid(const std::string& text)
{
    size_t at = 0;
    while (at < text.size() && std::isspace(static_cast<unsigned char>(text[at]))) ++at;
    std::string word;
    while (at < text.size() && !std::isspace(static_cast<unsigned char>(text[at])))
        word += text[at++];
    for (const char* k : {"ncols", "nrows", "xllcorner", "yllcorner", "xllcenter", "yllcenter",
                          "dx", "dy", "cellsize"})
        if (ascii_key(word, k)) return true;
    return false;
}

double parse_number(const std::string& token, bool& ok)
{
    char* end = nullptr;
    const double v = std::strtod(token.c_str(), &end);
    ok = end && *end == 0 && !token.empty();
    return v;
}

Raster read_ascii_grid(const std::string& text)
{
    Raster r;
    size_t at = 0;
    auto next = [&](std::string& token) {
        while (at < text.size() && std::isspace(static_cast<unsigned char>(text[at]))) ++at;
        token.clear();
        while (at < text.size() && !std::isspace(static_cast<unsigned char>(text[at])))
            token += text[at++];
        return !token.empty();
    };
    bool cols = false, rows = false, xll = false, yll = false, cell = false, dx = false,
         dy = false;
    std::string key, value;
    size_t data_at = 0;
    while (true) {
        const size_t mark = at;
        if (!next(key)) throw OpenError("no data");
        const char c = key[0];
        if (std::isdigit(static_cast<unsigned char>(c)) || c == '-' || c == '+' || c == '.') {
            data_at = mark;
            break;
        }
        if (!next(value)) throw OpenError("header");
        bool ok = false;
        const double v = parse_number(value, ok);
        if (!ok) throw OpenError("header value");
        if (ascii_key(key, "ncols")) cols = true, r.width = int(v);
        else if (ascii_key(key, "nrows")) rows = true, r.height = int(v);
        else if (ascii_key(key, "xllcorner") || ascii_key(key, "xllcenter")) xll = true;
        else if (ascii_key(key, "yllcorner") || ascii_key(key, "yllcenter")) yll = true;
        else if (ascii_key(key, "cellsize")) cell = true;
        else if (ascii_key(key, "dx")) dx = true;
        else if (ascii_key(key, "dy")) dy = true;
        else if (ascii_key(key, "nodata_value")) r.has_nodata = true, r.nodata = v;
        else throw OpenError("header key");
    }
    if (!cols || !rows || !xll || !yll || !(cell || (dx && dy)) || r.width <= 0 || r.height <= 0)
        throw OpenError("incomplete header");
    const size_t n = size_t(r.width) * size_t(r.height);
    if (n > (size_t(1) << 31)) throw OpenError("too large");
    at = data_at;
    r.values.resize(n);
    std::string token;
    for (size_t i = 0; i < n; ++i) {
        bool ok = false;
        if (!next(token)) throw ReadError("short data");
        const double v = parse_number(token, ok);
        if (!ok) throw ReadError("bad value");
        r.values[i] = float(v);
    }
    return r;
}

// ---- deflate (RFC 1951) inside a zlib stream (RFC 1950) ----------------------
class BitReader {
public:
    BitReader(const uint8_t* p, size_t n) : p_(p), n_(n) {}
    uint32_t bits(int count)
    {
        while (have_ < count) {
            if (at_ >= n_) throw ReadError("deflate: truncated");
            acc_ |= uint64_t(p_[at_++]) << have_;
            have_ += 8;
        }
        const uint32_t v = uint32_t(acc_ & ((uint64_t(1) << count) - 1));
        acc_ >>= count;
        have_ -= count;
        return v;
    }
    void align()
    {
        acc_ >>= (have_ & 7);
        have_ -= (have_ & 7);
    }
    size_t byte_position() const { return at_ - size_t(have_ / 8); }
    void skip_to(size_t pos)
    {
        at_ = pos;
        acc_ = 0;
        have_ = 0;
    }

private:
    const uint8_t* p_;
    size_t n_, at_ = 0;
    uint64_t acc_ = 0;
    int have_ = 0;
};

// Canonical Huffman code (RFC 1951 3.2.2): symbols ordered by code length,
// then by value; decoded one bit at a time.
struct Huffman {
    uint16_t count[16]{};
    std::vector<uint16_t> symbol;
    void build(const uint8_t* lengths, int n)
    {
        std::fill(std::begin(count), std::end(count), 0);
        for (int i = 0; i < n; ++i) ++count[lengths[i]];
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; ++len) {
            left = left * 2 - count[len];
            if (left < 0) throw ReadError("deflate: oversubscribed code");
        }
        uint16_t offset[16]{};
        for (int len = 1; len < 15; ++len) offset[len + 1] = uint16_t(offset[len] + count[len]);
        symbol.assign(size_t(n), 0);
        for (int i = 0; i < n; ++i)
            if (lengths[i]) symbol[offset[lengths[i]]++] = uint16_t(i);
    }
    int decode(BitReader& in) const
    {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= int(in.bits(1));
            const int c = count[len];
            if (code - first < c) return symbol[size_t(index + code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        throw ReadError("deflate: bad code");
    }
};

void length_tables(uint16_t* len_base, uint8_t* len_extra, uint16_t* dist_base,
                   uint8_t* dist_extra)
{
    // lengths 257..284: eight codes of 0 extra bits, then four each of 1..5;
    // 285 is 258 with none.  distances 0..29: four of 0, then two each of 1..13.
    int base = 3;
    for (int i = 0; i < 28; ++i) {
        const int extra = i < 8 ? 0 : (i - 4) / 4;
        len_base[i] = uint16_t(base);
        len_extra[i] = uint8_t(extra);
        base += 1 << extra;
    }
    len_base[28] = 258;
    len_extra[28] = 0;
    base = 1;
    for (int i = 0; i < 30; ++i) {
        const int extra = i < 4 ? 0 : (i - 2) / 2;
        dist_base[i] = uint16_t(base);
        dist_extra[i] = uint8_t(extra);
        base += 1 << extra;
    }
}

std::vector<uint8_t> inflate_zlib(const uint8_t* p, size_t n, size_t expect)
{
    if (n < 6) throw ReadError("zlib: short");
    const int cmf = p[0], flg = p[1];
    if ((cmf & 15) != 8 || (cmf * 256 + flg) % 31 != 0 || (flg & 32))
        throw ReadError("zlib: header");
    uint16_t len_base[29], dist_base[30];
    uint8_t len_extra[29], dist_extra[30];
    length_tables(len_base, len_extra, dist_base, dist_extra);
    static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5,
                                      11, 4, 12, 3, 13, 2, 14, 1, 15};
    std::vector<uint8_t> out;
    out.reserve(expect);
    BitReader in(p + 2, n - 2);
    Huffman lit, dist;
    bool last = false;
    while (!last) {
        last = in.bits(1) != 0;
        const uint32_t type = in.bits(2);
        if (type == 0) {
            in.align();
            const uint32_t len = in.bits(16), nlen = in.bits(16);
            if ((len ^ 0xffffu) != nlen) throw ReadError("deflate: stored length");
            const size_t at = in.byte_position() + 2;
            if (at + len > n) throw ReadError("deflate: truncated");
            out.insert(out.end(), p + at, p + at + len);
            in.skip_to(at + len - 2);
            continue;
        }
        uint8_t lengths[320];
        if (type == 1) {
            for (int i = 0; i < 288; ++i) lengths[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
            lit.build(lengths, 288);
            for (int i = 0; i < 30; ++i) lengths[i] = 5;
            dist.build(lengths, 30);
        } else if (type == 2) {
            const int hlit = int(in.bits(5)) + 257, hdist = int(in.bits(5)) + 1,
                      hclen = int(in.bits(4)) + 4;
            uint8_t cl[19]{};
            for (int i = 0; i < hclen; ++i) cl[order[i]] = uint8_t(in.bits(3));
            Huffman clh;
            clh.build(cl, 19);
            int i = 0;
            while (i < hlit + hdist) {
                const int s = clh.decode(in);
                if (s < 16) {
                    lengths[i++] = uint8_t(s);
                    continue;
                }
                int rep = 0;
                uint8_t v = 0;
                if (s == 16) {
                    if (i == 0) throw ReadError("deflate: repeat without length");
                    v = lengths[i - 1];
                    rep = 3 + int(in.bits(2));
                } else if (s == 17) {
                    rep = 3 + int(in.bits(3));
                } else {
                    rep = 11 + int(in.bits(7));
                }
                if (i + rep > hlit + hdist) throw ReadError("deflate: lengths overrun");
                while (rep--) lengths[i++] = v;
            }
            lit.build(lengths, hlit);
            dist.build(lengths + hlit, hdist);
        } else {
            throw ReadError("deflate: block type");
        }
        while (true) {
            const int s = lit.decode(in);
            if (s < 256) {
                out.push_back(uint8_t(s));
            } else if (s == 256) {
                break;
            } else {
                if (s > 285) throw ReadError("deflate: length code");
                const size_t len = len_base[s - 257] + in.bits(len_extra[s - 257]);
                const int d = dist.decode(in);
                if (d > 29) throw ReadError("deflate: distance code");
                const size_t back = dist_base[d] + in.bits(dist_extra[d]);
                if (back > out.size()) throw ReadError("deflate: distance too far");
                const size_t from = out.size() - back;
                for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
            }
            if (out.size() > expect + (size_t(1) << 20)) throw ReadError("deflate: too long");
        }
    }
    // Adler-32 of the output (RFC 1950 section 8)
    in.align();
    const size_t at = in.byte_position() + 2;
    if (at + 4 <= n) {
        uint32_t a = 1, b = 0;
        for (const uint8_t c : out) {
            a = (a + c) % 65521u;
            b = (b + a) % 65521u;
        }
        const uint32_t want =
            uint32_t(p[at]) << 24 | uint32_t(p[at + 1]) << 16 | uint32_t(p[at + 2]) << 8 | p[at + 3];
        if (want != (b << 16 | a)) throw ReadError("zlib: checksum");
    }
    return out;
}

// ---- LZW (TIFF 6.0 section 13) ------------------------------------------------
std::vector<uint8_t> lzw_decode(const uint8_t* p, size_t n, size_t expect)
{
    constexpr int kClear = 256, kEnd = 257, kMax = 4096;
    std::vector<uint16_t> prefix(kMax);
    std::vector<uint8_t> suffix(kMax), first(kMax);
    std::vector<uint16_t> length(kMax);
    for (int i = 0; i < 256; ++i) {
        suffix[size_t(i)] = first[size_t(i)] = uint8_t(i);
        length[size_t(i)] = 1;
    }
    std::vector<uint8_t> out;
    out.reserve(expect);
    size_t bitpos = 0;
    const size_t total = n * 8;
    auto read = [&](int width) -> int {
        if (bitpos + size_t(width) > total) return kEnd;  // a missing end code
        int v = 0;
        for (int k = 0; k < width; ++k, ++bitpos)
            v = (v << 1) | ((p[bitpos >> 3] >> (7 - (bitpos & 7))) & 1);
        return v;
    };
    auto emit = [&](int code) {
        const size_t len = length[size_t(code)], at = out.size();
        out.resize(at + len);
        for (size_t k = len; k-- > 0;) {
            out[at + k] = suffix[size_t(code)];
            code = prefix[size_t(code)];
        }
    };
    int width = 9, next = 258, old = -1;
    while (true) {
        const int code = read(width);
        if (code == kEnd) break;
        if (code == kClear) {
            width = 9;
            next = 258;
            old = -1;
            continue;
        }
        if (old < 0) {
            if (code > 255) throw ReadError("lzw: first code");
            emit(code);
            old = code;
            continue;
        }
        if (code < next) {
            emit(code);
            if (next < kMax) {
                prefix[size_t(next)] = uint16_t(old);
                suffix[size_t(next)] = first[size_t(code)];
                first[size_t(next)] = first[size_t(old)];
                length[size_t(next)] = uint16_t(length[size_t(old)] + 1);
                ++next;
            }
        } else if (code == next && next < kMax) {
            prefix[size_t(next)] = uint16_t(old);
            suffix[size_t(next)] = first[size_t(old)];
            first[size_t(next)] = first[size_t(old)];
            length[size_t(next)] = uint16_t(length[size_t(old)] + 1);
            ++next;
            emit(code);
        } else {
            throw ReadError("lzw: code out of range");
        }
        old = code;
        // the code width grows one code early (TIFF 6.0 LZW)
        if (next >= (1 << width) - 1 && width < 12) ++width;
        if (out.size() > expect + (size_t(1) << 20)) throw ReadError("lzw: too long");
    }
    return out;
}

std::vector<uint8_t> packbits_decode(const uint8_t* p, size_t n, size_t expect)
{
    std::vector<uint8_t> out;
    out.reserve(expect);
    size_t at = 0;
    while (at < n && out.size() < expect) {
        const int c = int(int8_t(p[at++]));
        if (c >= 0) {
            if (at + size_t(c) + 1 > n) throw ReadError("packbits: truncated");
            out.insert(out.end(), p + at, p + at + c + 1);
            at += size_t(c) + 1;
        } else if (c != -128) {
            if (at >= n) throw ReadError("packbits: truncated");
            out.insert(out.end(), size_t(1 - c), p[at++]);
        }
    }
    return out;
}

// ---- TIFF ----------------------------------------------------------------------
struct Tiff {
    const std::vector<uint8_t>& b;
    bool big_endian = false, big_tiff = false;

    uint64_t u(size_t at, int bytes) const
    {
        if (at + size_t(bytes) > b.size()) throw OpenError("tiff: truncated");
        uint64_t v = 0;
        for (int k = 0; k < bytes; ++k) {
            const uint64_t c = b[at + size_t(k)];
            v |= big_endian ? c << (8 * (bytes - 1 - k)) : c << (8 * k);
        }
        return v;
    }
};

struct Entry {
    uint16_t type = 0;
    uint64_t count = 0, data = 0;  // data = the value's offset in the file
};

int type_size(uint16_t type)
{
    switch (type) {
    case 1: case 2: case 6: case 7: return 1;
    case 3: case 8: return 2;
    case 4: case 9: case 11: case 13: return 4;
    case 5: case 10: case 12: case 16: case 17: case 18: return 8;
    default: return 0;
    }
}

std::vector<uint64_t> entry_values(const Tiff& t, const Entry& e)
{
    const int sz = type_size(e.type);
    if (e.type != 1 && e.type != 3 && e.type != 4 && e.type != 16 && e.type != 13 && e.type != 18)
        throw OpenError("tiff: integer tag expected");
    if (e.count > (uint64_t(1) << 26)) throw OpenError("tiff: tag too long");
    std::vector<uint64_t> v(size_t(e.count));
    for (size_t i = 0; i < v.size(); ++i) v[i] = t.u(size_t(e.data) + i * size_t(sz), sz);
    return v;
}

float half_to_float(uint16_t h)
{
    const int sign = h >> 15, exp = (h >> 10) & 31, man = h & 1023;
    float v;
    if (exp == 0) v = std::ldexp(float(man), -24);
    else if (exp == 31) v = man ? std::numeric_limits<float>::quiet_NaN()
                                : std::numeric_limits<float>::infinity();
    else v = std::ldexp(float(man | 1024), exp - 25);
    return sign ? -v : v;
}

// float32 as GDAL's RasterIO converts it: integers rounded to nearest, doubles
// narrowed (out-of-range finite values saturate at the largest float).
float double_to_float(double d)
{
    if (std::isfinite(d) && std::fabs(d) > double(std::numeric_limits<float>::max()))
        return d > 0 ? std::numeric_limits<float>::max() : -std::numeric_limits<float>::max();
    return float(d);
}

Raster read_tiff(const std::vector<uint8_t>& bytes, int band)
{
    Tiff t{bytes};
    t.big_endian = bytes[0] == 'M';
    const uint64_t magic = t.u(2, 2);
    uint64_t ifd = 0;
    if (magic == 42) {
        ifd = t.u(4, 4);
    } else if (magic == 43) {
        t.big_tiff = true;
        if (t.u(4, 2) != 8 || t.u(6, 2) != 0) throw OpenError("bigtiff header");
        ifd = t.u(8, 8);
    } else {
        throw OpenError("tiff magic");
    }
    const uint64_t entries = t.u(size_t(ifd), t.big_tiff ? 8 : 2);
    const size_t head = t.big_tiff ? 8 : 2, stride = t.big_tiff ? 20 : 12;
    const int inline_bytes = t.big_tiff ? 8 : 4;
    Entry tags[16];  // only the tags below are kept
    auto slot = [](uint32_t tag) -> int {
        switch (tag) {
        case 256: return 0; case 257: return 1; case 258: return 2; case 259: return 3;
        case 273: return 4; case 277: return 5; case 278: return 6; case 279: return 7;
        case 284: return 8; case 317: return 9; case 322: return 10; case 323: return 11;
        case 324: return 12; case 325: return 13; case 339: return 14; case 42113: return 15;
        default: return -1;
        }
    };
    bool seen[16]{};
    for (uint64_t i = 0; i < entries; ++i) {
        const size_t at = size_t(ifd) + head + size_t(i) * stride;
        const uint32_t tag = uint32_t(t.u(at, 2));
        const int s = slot(tag);
        if (s < 0) continue;
        Entry e;
        e.type = uint16_t(t.u(at + 2, 2));
        e.count = t.u(at + 4, t.big_tiff ? 8 : 4);
        const int sz = type_size(e.type);
        if (!sz) throw OpenError("tiff: tag type");
        const size_t value_at = at + (t.big_tiff ? 12 : 8);
        e.data = e.count * uint64_t(sz) <= uint64_t(inline_bytes) ? value_at
                                                                   : t.u(value_at, inline_bytes);
        if (e.data + e.count * uint64_t(sz) > bytes.size()) throw OpenError("tiff: tag data");
        tags[s] = e;
        seen[s] = true;
    }
    auto one = [&](int s, uint64_t fallback) -> uint64_t {
        if (!seen[s]) return fallback;
        const std::vector<uint64_t> v = entry_values(t, tags[s]);
        return v.empty() ? fallback : v[0];
    };
    if (!seen[0] || !seen[1]) throw OpenError("tiff: no size");
    const uint64_t width = one(0, 0), height = one(1, 0);
    const uint64_t spp = one(5, 1);
    const uint64_t compression = one(3, 1), planar = one(8, 1), predictor = one(9, 1);
    std::vector<uint64_t> bps_all = seen[2] ? entry_values(t, tags[2]) : std::vector<uint64_t>{1};
    std::vector<uint64_t> fmt_all = seen[14] ? entry_values(t, tags[14]) : std::vector<uint64_t>{1};
    const uint64_t bps = bps_all.empty() ? 1 : bps_all[0];
    const uint64_t format = fmt_all.empty() ? 1 : fmt_all[0];
    for (uint64_t v : bps_all)
        if (v != bps) throw OpenError("tiff: mixed sample sizes");
    if (width == 0 || height == 0 || spp == 0 || spp > 64) throw OpenError("tiff: size");
    if (width * height > (uint64_t(1) << 31)) throw OpenError("tiff: too large");
    if (planar != 1 && planar != 2) throw OpenError("tiff: planar configuration");
    const bool ok_type = (format == 1 || format == 2)
                             ? (bps == 8 || bps == 16 || bps == 32 || bps == 64)
                             : format == 3 && (bps == 16 || bps == 32 || bps == 64);
    if (!ok_type) throw OpenError("tiff: sample type");
    if (compression != 1 && compression != 5 && compression != 8 && compression != 32946 &&
        compression != 32773)
        throw OpenError("tiff: compression");
    if (predictor != 1 && predictor != 2 && predictor != 3) throw OpenError("tiff: predictor");
    if (predictor == 3 && format != 3) throw OpenError("tiff: predictor 3 on integers");

    const bool tiled = seen[10] || seen[11] || seen[12];
    const uint64_t cw = tiled ? one(10, 0) : width;
    const uint64_t ch = tiled ? one(11, 0) : std::min<uint64_t>(one(6, height), height);
    if (cw == 0 || ch == 0) throw OpenError("tiff: block size");
    const int off_slot = tiled ? 12 : 4, cnt_slot = tiled ? 13 : 7;
    if (!seen[off_slot]) throw OpenError("tiff: no data offsets");
    const std::vector<uint64_t> offsets = entry_values(t, tags[off_slot]);
    std::vector<uint64_t> counts;
    if (seen[cnt_slot]) counts = entry_values(t, tags[cnt_slot]);
    const uint64_t across = (width + cw - 1) / cw, down = (height + ch - 1) / ch;
    const uint64_t per_plane = across * down;
    const uint64_t block_spp = planar == 1 ? spp : 1;
    const size_t sample_bytes = size_t(bps / 8);
    const size_t pixel_bytes = size_t(block_spp) * sample_bytes;
    const size_t row_bytes = size_t(cw) * pixel_bytes;
    const size_t block_bytes = row_bytes * size_t(ch);
    if (offsets.size() < per_plane * (planar == 1 ? 1 : spp)) throw OpenError("tiff: offsets");
    if (!counts.empty() && counts.size() < per_plane * (planar == 1 ? 1 : spp))
        throw OpenError("tiff: byte counts");
    if (counts.empty() && compression != 1) throw OpenError("tiff: byte counts");

    if (band < 0 || uint64_t(band) >= spp) throw ReadError("tiff: band");
    Raster r;
    r.width = int(width);
    r.height = int(height);
    r.bands = int(spp);
    if (seen[15] && tags[15].type == 2) {
        std::string s(reinterpret_cast<const char*>(bytes.data() + tags[15].data),
                      size_t(tags[15].count));
        s = s.substr(0, s.find('\0'));
        r.has_nodata = true;
        r.nodata = std::strtod(s.c_str(), nullptr);
    }
    r.values.assign(size_t(width) * size_t(height), 0.0f);
    // the band's plane (planar) or its sample within each pixel (chunky)
    const uint64_t plane0 = planar == 2 ? uint64_t(band) * per_plane : 0;
    const size_t sample0 = planar == 2 ? 0 : size_t(band) * sample_bytes;
    for (uint64_t bi = 0; bi < per_plane; ++bi) {
        const uint64_t off = offsets[size_t(plane0 + bi)];
        const uint64_t rows_here =
            tiled ? ch : std::min<uint64_t>(ch, height - (bi / across) * ch);
        const size_t want = tiled ? block_bytes : row_bytes * size_t(rows_here);
        const uint64_t cnt = counts.empty() ? want : counts[size_t(plane0 + bi)];
        if (off + cnt > bytes.size()) throw ReadError("tiff: block outside the file");
        const uint8_t* src = bytes.data() + off;
        std::vector<uint8_t> block;
        switch (compression) {
        case 1: block.assign(src, src + std::min<uint64_t>(cnt, want)); break;
        case 5: block = lzw_decode(src, size_t(cnt), want); break;
        case 8: case 32946: block = inflate_zlib(src, size_t(cnt), want); break;
        default: block = packbits_decode(src, size_t(cnt), want); break;
        }
        if (block.size() < want) throw ReadError("tiff: short block");
        block.resize(want);
        // undo the predictor, row by row
        const size_t rows = size_t(tiled ? ch : rows_here);
        for (size_t y = 0; y < rows; ++y) {
            uint8_t* row = block.data() + y * row_bytes;
            const size_t n = size_t(cw) * size_t(block_spp);  // samples in the row
            if (predictor == 2) {
                const size_t st = size_t(block_spp);
                for (size_t i = st; i < n; ++i) {
                    uint64_t prev = 0, cur = 0;
                    for (size_t k = 0; k < sample_bytes; ++k) {
                        const size_t kk = t.big_endian ? sample_bytes - 1 - k : k;
                        prev |= uint64_t(row[(i - st) * sample_bytes + kk]) << (8 * k);
                        cur |= uint64_t(row[i * sample_bytes + kk]) << (8 * k);
                    }
                    const uint64_t sum = prev + cur;
                    for (size_t k = 0; k < sample_bytes; ++k) {
                        const size_t kk = t.big_endian ? sample_bytes - 1 - k : k;
                        row[i * sample_bytes + kk] = uint8_t(sum >> (8 * k));
                    }
                }
            } else if (predictor == 3) {
                // byte-wise differences over the row (stride = samples per
                // pixel), then the bytes of sample i are in planes of n bytes,
                // most significant first; rewritten here in file byte order
                const size_t st = size_t(block_spp), nb = n * sample_bytes;
                for (size_t i = st; i < nb; ++i) row[i] = uint8_t(row[i] + row[i - st]);
                std::vector<uint8_t> tmp(row, row + nb);
                for (size_t i = 0; i < n; ++i)
                    for (size_t k = 0; k < sample_bytes; ++k) {
                        const size_t kk = t.big_endian ? k : sample_bytes - 1 - k;
                        row[i * sample_bytes + kk] = tmp[k * n + i];
                    }
            }
        }
        const uint64_t bx = (bi % across) * cw, by = (bi / across) * ch;
        for (size_t y = 0; y < rows; ++y) {
            if (by + y >= height) break;
            for (size_t x = 0; x < size_t(cw); ++x) {
                if (bx + x >= width) break;
                const size_t at = y * row_bytes + x * pixel_bytes + sample0;
                uint64_t raw = 0;
                for (size_t k = 0; k < sample_bytes; ++k) {
                    const size_t kk = t.big_endian ? sample_bytes - 1 - k : k;
                    raw |= uint64_t(block[at + kk]) << (8 * k);
                }
                float v = 0.0f;
                if (format == 3) {
                    if (bps == 16) {
                        v = half_to_float(uint16_t(raw));
                    } else if (bps == 32) {
                        const uint32_t w = uint32_t(raw);
                        std::memcpy(&v, &w, 4);
                    } else {
                        double d;
                        std::memcpy(&d, &raw, 8);
                        v = double_to_float(d);
                    }
                } else if (format == 2) {
                    const int shift = int(64 - bps);
                    const int64_t s = int64_t(raw << shift) >> shift;
                    v = float(s);
                } else {
                    v = float(raw);
                }
                r.values[size_t(by + y) * size_t(width) + size_t(bx + x)] = v;
            }
        }
    }
    return r;
}

// ---- PNG (ISO/IEC 15948) -----------------------------------------------------
// Non-interlaced PNG of bit depth 8 or 16: gray (1 band), RGB (3), palette
// (1 band of palette indices, as GDAL exposes it), gray + alpha (2), RGBA
// (4); the five row filters undone after inflating the IDAT stream.
Raster read_png(const std::vector<uint8_t>& b, int band)
{
    auto be32 = [&](size_t at) {
        if (at + 4 > b.size()) throw OpenError("png: truncated");
        return uint32_t(b[at]) << 24 | uint32_t(b[at + 1]) << 16 | uint32_t(b[at + 2]) << 8 | b[at + 3];
    };
    size_t at = 8;
    uint32_t width = 0, height = 0;
    int depth = 0, color = -1, interlace = 0;
    std::vector<uint8_t> idat;
    while (at + 8 <= b.size()) {
        const uint32_t len = be32(at);
        const std::string type(reinterpret_cast<const char*>(b.data() + at + 4), 4);
        if (at + 12 + size_t(len) > b.size()) throw OpenError("png: chunk");
        const uint8_t* d = b.data() + at + 8;
        if (type == "IHDR") {
            if (len < 13) throw OpenError("png: header");
            width = be32(at + 8);
            height = be32(at + 12);
            depth = d[8];
            color = d[9];
            interlace = d[12];
        } else if (type == "IDAT") {
            idat.insert(idat.end(), d, d + len);
        } else if (type == "IEND") {
            break;
        }
        at += 12 + size_t(len);
    }
    const int channels = color == 0 ? 1 : color == 2 ? 3 : color == 3 ? 1 : color == 4 ? 2
                         : color == 6 ? 4 : 0;
    if (!channels || (depth != 8 && depth != 16) || interlace != 0 || width == 0 || height == 0 ||
        width > uint32_t(INT_MAX) || height > uint32_t(INT_MAX) ||
        uint64_t(width) * height > (uint64_t(1) << 31) || (color == 3 && depth != 8))
        throw OpenError("png: unsupported");
    if (band < 0 || band >= channels) throw ReadError("png: band");
    const size_t bpp = size_t(channels) * size_t(depth / 8), stride = size_t(width) * bpp;
    std::vector<uint8_t> raw = inflate_zlib(idat.data(), idat.size(), (stride + 1) * height);
    if (raw.size() < (stride + 1) * height) throw ReadError("png: short image data");
    std::vector<uint8_t> prev(stride, 0), cur(stride);
    Raster r;
    r.width = int(width);
    r.height = int(height);
    r.bands = channels;
    r.values.resize(size_t(width) * height);
    for (uint32_t y = 0; y < height; ++y) {
        const uint8_t filter = raw[y * (stride + 1)];
        const uint8_t* src = raw.data() + y * (stride + 1) + 1;
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= bpp ? cur[i - bpp] : 0, up = prev[i];
            const int c = i >= bpp ? prev[i - bpp] : 0;
            int pred = 0;
            switch (filter) {
            case 0: pred = 0; break;
            case 1: pred = a; break;
            case 2: pred = up; break;
            case 3: pred = (a + up) / 2; break;
            case 4: {
                const int p = a + up - c, pa = std::abs(p - a), pb = std::abs(p - up),
                          pc = std::abs(p - c);
                pred = pa <= pb && pa <= pc ? a : pb <= pc ? up : c;
                break;
            }
            default: throw ReadError("png: filter");
            }
            cur[i] = uint8_t(src[i] + pred);
        }
        for (uint32_t x = 0; x < width; ++x) {
            const size_t o = size_t(x) * bpp + size_t(band) * size_t(depth / 8);
            const float v = depth == 8 ? float(cur[o]) : float(uint32_t(cur[o]) << 8 | cur[o + 1]);
            r.values[size_t(y) * width + x] = v;
        }
        std::swap(prev, cur);
    }
    return r;
}

Raster read_raster(const std::filesystem::path& path, int band = 0)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) throw OpenError("cannot open");
    const std::vector<uint8_t> bytes{std::istreambuf_iterator<char>(in),
                                     std::istreambuf_iterator<char>()};
    if (bytes.size() >= 8 && ((bytes[0] == 'I' && bytes[1] == 'I') ||
                              (bytes[0] == 'M' && bytes[1] == 'M')))
        return read_tiff(bytes, band);
    static const uint8_t kPng[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    if (bytes.size() >= 8 && std::memcmp(bytes.data(), kPng, 8) == 0) return read_png(bytes, band);
    const std::string text(bytes.begin(), bytes.end());
    if (looks_ascii_grid(text)) {
        if (band != 0) throw ReadError("ascii grid: one band");
        return read_ascii_grid(text);
    }
    throw OpenError("not a raster");
}

}  // namespace

HeightField read_height_field(const std::filesystem::path& path)
{
    const std::string name = path.string();
    Raster r;
    try {
        r = read_raster(path);
    } catch (const ReadError&) {
        throw std::runtime_error("Cannot read DEM elevations: " + name);
    } catch (const std::exception&) {
        throw std::runtime_error("Cannot open DEM: " + name);
    }
    if (r.width < 2 || r.height < 2)
        throw std::runtime_error("DEM must contain at least 2 x 2 cells: " + name);
    HeightField h;
    h.width = r.width;
    h.height = r.height;
    h.values = std::move(r.values);
    const float nodata = float(r.nodata);
    h.minimum = std::numeric_limits<float>::infinity();
    for (const float v : h.values) {
        if (!std::isfinite(v) || (r.has_nodata && v == nodata)) continue;
        h.minimum = std::min(h.minimum, v);
    }
    if (!std::isfinite(h.minimum))
        throw std::runtime_error("DEM contains no valid elevations: " + name);
    for (float& v : h.values)
        if (!std::isfinite(v) || (r.has_nodata && v == nodata)) v = h.minimum;
    return h;
}

// Up to `max_bands` bands as bytes, as a GDAL RasterIO into GDT_Byte
// converts them: rounded to the nearest integer (halves up) and clamped to
// [0, 255], NaN as 0.
ByteBands read_byte_bands(const std::filesystem::path& path, int max_bands,
                          const std::string& open_error, const std::string& read_error)
{
    const std::string name = path.string();
    ByteBands out;
    try {
        Raster first = read_raster(path, 0);
        out.width = first.width;
        out.height = first.height;
        out.count = std::min(max_bands, first.bands);
        for (int b = 0; b < out.count; ++b) {
            const Raster r = b == 0 ? std::move(first) : read_raster(path, b);
            std::vector<uint8_t>& v = out.values[size_t(b)];
            v.resize(r.values.size());
            for (size_t i = 0; i < v.size(); ++i) {
                const float x = r.values[i];
                v[i] = std::isnan(x) ? 0 : x >= 255.0f ? 255 : x <= 0.0f ? 0 : uint8_t(x + 0.5f);
            }
        }
    } catch (const ReadError&) {
        throw std::runtime_error(read_error + name);
    } catch (const std::exception&) {
        throw std::runtime_error(open_error + name);
    }
    return out;
}

// DemHeightField::heightAboveMinimum (facetrtcore.cpp:2630-2649): GeoTIFF
// columns run east (+Z), rows south (-X); the raster is stretched over the
// scene domain and sampled bilinearly.
float HeightField::above_minimum(float north_x, float east_z, float scene_width,
                                 float scene_depth) const
{
    if (!valid()) return 0.0f;
    const float u = std::clamp(east_z / scene_depth, 0.0f, 1.0f) * float(width - 1);
    const float v = (1.0f - std::clamp(north_x / scene_width, 0.0f, 1.0f)) * float(height - 1);
    const int x0 = int(std::floor(u)), y0 = int(std::floor(v));
    const int x1 = std::min(width - 1, x0 + 1), y1 = std::min(height - 1, y0 + 1);
    const auto at = [this](int c, int r) { return values[size_t(r) * size_t(width) + size_t(c)]; };
    const float dx = u - float(x0), dy = v - float(y0);
    const float top = at(x0, y0) * (1.0f - dx) + at(x1, y0) * dx;
    const float bottom = at(x0, y1) * (1.0f - dx) + at(x1, y1) * dx;
    return std::max(0.0f, top * (1.0f - dy) + bottom * dy - minimum);
}

}  // namespace dem
}  // namespace facetcu

extern "C" {

int facetcu_dem_height_field(const char* path, int32_t* width, int32_t* height, float* minimum,
                             float* values, uint64_t capacity)
{
    facetcu_set_host_error("");
    if (!path || !width || !height) {
        facetcu_set_host_error("path, width and height are required");
        return FACETCU_INVALID_ARGUMENT;
    }
    try {
        const facetcu::dem::HeightField h = facetcu::dem::read_height_field(path);
        *width = h.width;
        *height = h.height;
        if (minimum) *minimum = h.minimum;
        if (values) {
            if (capacity < h.values.size()) {
                facetcu_set_host_error("values: capacity below width * height");
                return FACETCU_INVALID_ARGUMENT;
            }
            std::memcpy(values, h.values.data(), h.values.size() * sizeof(float));
        }
        return FACETCU_OK;
    } catch (const std::exception& e) {
        facetcu_set_host_error(e.what());
        return FACETCU_RUNTIME_ERROR;
    }
}

}  // extern "C"
