// Minimal OpenEXR 2.0 writer (single part, scanline, NO_COMPRESSION), written
// from the published file-layout description: magic, version, header
// attributes, line-offset table, one scanline per chunk.
#include "sb_exr.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace sb {

unsigned short float_to_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t exp = (x >> 23) & 0xffu;
    uint32_t man = x & 0x7fffffu;
    if (exp == 0xffu) return (unsigned short)(sign | 0x7c00u | (man ? 0x200u : 0u));  // inf / nan
    int e = (int)exp - 127 + 15;
    if (e >= 0x1f) return (unsigned short)(sign | 0x7c00u);  // overflow -> inf
    if (e <= 0) {
        // subnormal half (or zero)
        if (e < -10) return (unsigned short)sign;
        man |= 0x800000u;
        const int shift = 14 - e;  // 24-bit mantissa -> 10-bit at exponent 1
        uint32_t h = man >> shift;
        const uint32_t rem = man & ((1u << shift) - 1u);
        const uint32_t half = 1u << (shift - 1);
        if (rem > half || (rem == half && (h & 1u))) ++h;
        return (unsigned short)(sign | h);
    }
    uint32_t h = ((uint32_t)e << 10) | (man >> 13);
    const uint32_t rem = man & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;  // may carry into the exponent
    return (unsigned short)(sign | h);
}

namespace {

void put_u32(std::vector<unsigned char>& v, uint32_t x) {
    for (int k = 0; k < 4; ++k) v.push_back((unsigned char)(x >> (8 * k)));
}
void put_u64(std::vector<unsigned char>& v, uint64_t x) {
    for (int k = 0; k < 8; ++k) v.push_back((unsigned char)(x >> (8 * k)));
}
void put_f32(std::vector<unsigned char>& v, float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    put_u32(v, x);
}
void put_str(std::vector<unsigned char>& v, const char* s) {
    v.insert(v.end(), s, s + std::strlen(s));
    v.push_back(0);
}
void attr(std::vector<unsigned char>& v, const char* name, const char* type, uint32_t size) {
    put_str(v, name);
    put_str(v, type);
    put_u32(v, size);
}

}  // namespace

bool write_exr_gray3(const char* path, int width, int height, const float* img) {
    std::vector<unsigned char> h;
    h.push_back(0x76); h.push_back(0x2f); h.push_back(0x31); h.push_back(0x01);
    put_u32(h, 2u);  // version 2, single-part scanline
    const char* chans[3] = {"B", "G", "R"};
    attr(h, "channels", "chlist", 3 * (2 + 16) + 1);
    for (const char* c : chans) {
        put_str(h, c);
        put_u32(h, 1u);  // HALF
        h.push_back(0); h.push_back(0); h.push_back(0); h.push_back(0);  // pLinear + reserved
        put_u32(h, 1u);
        put_u32(h, 1u);
    }
    h.push_back(0);
    attr(h, "compression", "compression", 1);
    h.push_back(0);
    attr(h, "dataWindow", "box2i", 16);
    put_u32(h, 0); put_u32(h, 0); put_u32(h, (uint32_t)(width - 1)); put_u32(h, (uint32_t)(height - 1));
    attr(h, "displayWindow", "box2i", 16);
    put_u32(h, 0); put_u32(h, 0); put_u32(h, (uint32_t)(width - 1)); put_u32(h, (uint32_t)(height - 1));
    attr(h, "lineOrder", "lineOrder", 1);
    h.push_back(0);
    attr(h, "pixelAspectRatio", "float", 4);
    put_f32(h, 1.0f);
    attr(h, "screenWindowCenter", "v2f", 8);
    put_f32(h, 0.0f); put_f32(h, 0.0f);
    attr(h, "screenWindowWidth", "float", 4);
    put_f32(h, 1.0f);
    h.push_back(0);  // end of header

    const uint64_t chunk = 8 + (uint64_t)width * 3 * 2;
    const uint64_t first = h.size() + 8ull * (uint64_t)height;
    for (int y = 0; y < height; ++y) put_u64(h, first + chunk * (uint64_t)y);
    std::vector<unsigned short> row((size_t)width);
    std::FILE* fp = std::fopen(path, "wb");
    if (!fp) return false;
    bool ok = std::fwrite(h.data(), 1, h.size(), fp) == h.size();
    std::vector<unsigned char> blk;
    for (int y = 0; y < height && ok; ++y) {
        blk.clear();
        put_u32(blk, (uint32_t)y);
        put_u32(blk, (uint32_t)(width * 3 * 2));
        for (int x = 0; x < width; ++x) row[x] = float_to_half(img[(size_t)y * width + x]);
        for (int c = 0; c < 3; ++c)
            for (int x = 0; x < width; ++x) {
                blk.push_back((unsigned char)(row[x] & 0xff));
                blk.push_back((unsigned char)(row[x] >> 8));
            }
        ok = std::fwrite(blk.data(), 1, blk.size(), fp) == blk.size();
    }
    ok = (std::fclose(fp) == 0) && ok;
    return ok;
}

}  // namespace sb
