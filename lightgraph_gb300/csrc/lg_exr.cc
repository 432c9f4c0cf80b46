// Uncompressed OpenEXR scanline files without the OpenEXR library: the
// writer of the renderer's 13 AOV channels (the layout of src/Image.h:47-62)
// and a reader of environment maps as Imf::RgbaInputFile hands them to
// readExr (src/Sampling.h:175-189): R, G, B, A of the data window, each
// rounded to half precision (Imf::Rgba stores half), missing colour channels
// 0 and a missing alpha 1. Only NO_COMPRESSION files are read.
//
// File layout (OpenEXR 2 single-part scanline): magic 20000630, version 2,
// attributes (name, type, size, value) ending with an empty name, a line
// offset table (one uint64 per scanline block), then per block the int32 y,
// the int32 data size and, per channel in name order, the row's values.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "lightgraph_c.h"

namespace {

uint16_t float_to_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7FFFFFFFu;
    if (ax >= 0x7F800000u) return (uint16_t)(sign | 0x7C00u | (ax > 0x7F800000u ? 0x200u : 0u));  // inf / nan
    if (ax >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);  // rounds past the largest half: inf
    if (ax < 0x38800000u) {
        // subnormal half (or zero): value / 2^-24 rounded to nearest even
        if (ax < 0x33000000u) return (uint16_t)sign;  // below half of the smallest subnormal
        const uint32_t mant = (ax & 0x7FFFFFu) | 0x800000u;
        const int shift = 126 - (int)(ax >> 23);  // 14 .. 24
        const uint32_t q = mant >> shift, rem = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
        const uint32_t r = q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u);
        return (uint16_t)(sign | r);
    }
    // normal: rebias the exponent, round the 13 dropped mantissa bits to even
    const uint32_t e = (ax >> 23) - 112u, m = ax & 0x7FFFFFu;
    uint32_t h = (e << 10) | (m >> 13);
    const uint32_t rem = m & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;  // may carry into the exponent (still correct)
    return (uint16_t)(sign | h);
}

float half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 0x1Fu, m = h & 0x3FFu;
    uint32_t x;
    if (e == 0) {
        if (m == 0) {
            x = sign;
        } else {  // subnormal: normalise
            int s = 0;
            uint32_t mm = m;
            while (!(mm & 0x400u)) { mm <<= 1; ++s; }
            x = sign | ((uint32_t)(113 - s) << 23) | ((mm & 0x3FFu) << 13);
        }
    } else if (e == 31) {
        x = sign | 0x7F800000u | (m << 13);
    } else {
        x = sign | ((e + 112u) << 23) | (m << 13);
    }
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

}  // namespace

extern "C" lg_status lg_write_exr(const char* path, int w, int h, int n_channels, const char* const* names,
                                  const float* const* planes) {
    if (!path || w <= 0 || h <= 0 || n_channels <= 0 || !names || !planes) return LG_ERR_INVALID;
    std::vector<int> order(n_channels);
    for (int k = 0; k < n_channels; ++k) order[k] = k;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return std::strcmp(names[a], names[b]) < 0; });
    std::vector<char> hdr;
    auto put = [&](const void* p, size_t n) { hdr.insert(hdr.end(), (const char*)p, (const char*)p + n); };
    auto put_i32 = [&](int32_t v) { put(&v, 4); };
    auto put_str = [&](const std::string& s) { put(s.c_str(), s.size() + 1); };
    auto attr = [&](const std::string& name, const std::string& type, const std::vector<char>& val) {
        put_str(name);
        put_str(type);
        put_i32((int32_t)val.size());
        put(val.data(), val.size());
    };
    put_i32(20000630);
    put_i32(2);
    std::vector<char> chl;
    for (int k : order) {
        chl.insert(chl.end(), names[k], names[k] + std::strlen(names[k]) + 1);
        const int32_t pix_type = 2, sx = 1, sy = 1;  // FLOAT
        const uint8_t plinear_res[4] = {0, 0, 0, 0};
        chl.insert(chl.end(), (const char*)&pix_type, (const char*)&pix_type + 4);
        chl.insert(chl.end(), (const char*)plinear_res, (const char*)plinear_res + 4);
        chl.insert(chl.end(), (const char*)&sx, (const char*)&sx + 4);
        chl.insert(chl.end(), (const char*)&sy, (const char*)&sy + 4);
    }
    chl.push_back(0);
    attr("channels", "chlist", chl);
    attr("compression", "compression", std::vector<char>{0});
    const int32_t box[4] = {0, 0, w - 1, h - 1};
    const std::vector<char> bx((const char*)box, (const char*)box + 16);
    attr("dataWindow", "box2i", bx);
    attr("displayWindow", "box2i", bx);
    attr("lineOrder", "lineOrder", std::vector<char>{0});
    const float par = 1.0f, swc[2] = {0.f, 0.f}, sww = 1.0f;
    attr("pixelAspectRatio", "float", std::vector<char>((const char*)&par, (const char*)&par + 4));
    attr("screenWindowCenter", "v2f", std::vector<char>((const char*)swc, (const char*)swc + 8));
    attr("screenWindowWidth", "float", std::vector<char>((const char*)&sww, (const char*)&sww + 4));
    hdr.push_back(0);
    std::ofstream f(path, std::ios::binary);
    if (!f) return LG_ERR_INVALID;
    f.write(hdr.data(), (std::streamsize)hdr.size());
    const uint64_t line_bytes = 8 + (uint64_t)w * 4 * n_channels;
    uint64_t off = hdr.size() + 8ull * h;
    for (int y = 0; y < h; ++y) {
        f.write((const char*)&off, 8);
        off += line_bytes;
    }
    for (int y = 0; y < h; ++y) {
        const int32_t yy = y, sz = (int32_t)(w * 4 * n_channels);
        f.write((const char*)&yy, 4);
        f.write((const char*)&sz, 4);
        for (int k : order) f.write((const char*)(planes[k] + (int64_t)y * w), 4 * (std::streamsize)w);
    }
    return f ? LG_OK : LG_ERR_INVALID;
}

extern "C" lg_status lg_read_exr_rgba(const char* path, int32_t* width, int32_t* height, float* rgba) {
    if (!path || !width || !height) return LG_ERR_INVALID;
    std::ifstream f(path, std::ios::binary);
    if (!f) return LG_ERR_INVALID;
    std::vector<char> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    size_t pos = 0;
    auto rd = [&](void* dst, size_t n) {
        if (pos + n > buf.size()) return false;
        std::memcpy(dst, buf.data() + pos, n);
        pos += n;
        return true;
    };
    auto rd_str = [&](std::string& s) {
        s.clear();
        while (pos < buf.size() && buf[pos]) s.push_back(buf[pos++]);
        if (pos >= buf.size()) return false;
        ++pos;
        return true;
    };
    int32_t magic = 0, version = 0;
    if (!rd(&magic, 4) || !rd(&version, 4) || magic != 20000630) return LG_ERR_INVALID;
    if (version & 0x1200) return LG_ERR_INVALID;  // tiled or multi-part files
    struct Ch { std::string name; int32_t type; };
    std::vector<Ch> chans;
    int32_t dw[4] = {0, 0, -1, -1};
    int compression = -1;
    for (;;) {
        std::string name, type;
        if (!rd_str(name)) return LG_ERR_INVALID;
        if (name.empty()) break;
        int32_t size = 0;
        if (!rd_str(type) || !rd(&size, 4) || size < 0 || pos + (size_t)size > buf.size()) return LG_ERR_INVALID;
        const size_t end = pos + (size_t)size;
        if (name == "channels") {
            while (pos < end && buf[pos]) {
                Ch c;
                if (!rd_str(c.name) || !rd(&c.type, 4)) return LG_ERR_INVALID;
                pos += 12;  // pLinear, reserved, xSampling, ySampling
                chans.push_back(c);
            }
        } else if (name == "compression") {
            compression = (uint8_t)buf[pos];
        } else if (name == "dataWindow") {
            std::memcpy(dw, buf.data() + pos, 16);
        }
        pos = end;
    }
    if (compression != 0) return LG_ERR_INVALID;  // only NO_COMPRESSION without the OpenEXR library
    const int w = dw[2] - dw[0] + 1, h = dw[3] - dw[1] + 1;
    if (w <= 0 || h <= 0 || chans.empty()) return LG_ERR_INVALID;
    *width = w;
    *height = h;
    if (!rgba) return LG_OK;
    std::sort(chans.begin(), chans.end(), [](const Ch& a, const Ch& b) { return a.name < b.name; });
    int slot[64];
    size_t px_bytes = 0;
    for (size_t k = 0; k < chans.size() && k < 64; ++k) {
        const std::string& n = chans[k].name;
        slot[k] = n == "R" ? 0 : n == "G" ? 1 : n == "B" ? 2 : n == "A" ? 3 : -1;
        px_bytes += chans[k].type == 1 ? 2 : 4;
    }
    for (int64_t p = 0; p < (int64_t)w * h; ++p) {
        rgba[4 * p] = rgba[4 * p + 1] = rgba[4 * p + 2] = 0.f;
        rgba[4 * p + 3] = 1.f;
    }
    std::vector<uint64_t> offsets(h);
    if (!rd(offsets.data(), 8ull * h)) return LG_ERR_INVALID;
    for (int b = 0; b < h; ++b) {
        pos = offsets[b];
        int32_t y = 0, size = 0;
        if (!rd(&y, 4) || !rd(&size, 4)) return LG_ERR_INVALID;
        const int row = y - dw[1];
        if (row < 0 || row >= h || (size_t)size < px_bytes * w || pos + (size_t)size > buf.size())
            return LG_ERR_INVALID;
        for (size_t k = 0; k < chans.size(); ++k) {
            for (int x = 0; x < w; ++x) {
                float v;
                if (chans[k].type == 1) {
                    uint16_t hv;
                    rd(&hv, 2);
                    v = half_to_float(hv);
                } else if (chans[k].type == 2) {
                    rd(&v, 4);
                } else {
                    uint32_t u;
                    rd(&u, 4);
                    v = (float)u;
                }
                if (k < 64 && slot[k] >= 0)
                    rgba[4 * ((int64_t)row * w + x) + slot[k]] = half_to_float(float_to_half(v));
            }
        }
    }
    return LG_OK;
}
