// Minimal OpenEXR 2.0 writer and reader (single part, scanline,
// NO_COMPRESSION), written from the published file-layout description:
// magic, version, header attributes, line-offset table, one scanline per
// chunk.  Plus the bilinear resampling the reference applies to its input
// textures.
#include "sb_exr.h"

#include <cmath>
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
    return write_exr_bgr(path, width, height, img, img, img);
}

bool write_exr_bgr(const char* path, int width, int height, const float* b, const float* g,
                   const float* r) {
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
    const float* planes[3] = {b, g, r};  // channel order B, G, R
    std::FILE* fp = std::fopen(path, "wb");
    if (!fp) return false;
    bool ok = std::fwrite(h.data(), 1, h.size(), fp) == h.size();
    std::vector<unsigned char> blk;
    for (int y = 0; y < height && ok; ++y) {
        blk.clear();
        put_u32(blk, (uint32_t)y);
        put_u32(blk, (uint32_t)(width * 3 * 2));
        for (int c = 0; c < 3; ++c)
            for (int x = 0; x < width; ++x) {
                const unsigned short v = float_to_half(planes[c][(size_t)y * width + x]);
                blk.push_back((unsigned char)(v & 0xff));
                blk.push_back((unsigned char)(v >> 8));
            }
        ok = std::fwrite(blk.data(), 1, blk.size(), fp) == blk.size();
    }
    ok = (std::fclose(fp) == 0) && ok;
    return ok;
}

float half_to_float(unsigned short h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t exp = (h >> 10) & 0x1fu;
    uint32_t man = h & 0x3ffu;
    uint32_t x;
    if (exp == 0x1fu) {
        x = sign | 0x7f800000u | (man << 13);  // inf / nan
    } else if (exp == 0) {
        if (man == 0) {
            x = sign;
        } else {
            // subnormal half: normalise
            int e = -1;
            do {
                ++e;
                man <<= 1;
            } while (!(man & 0x400u));
            x = sign | ((uint32_t)(127 - 15 - e) << 23) | ((man & 0x3ffu) << 13);
        }
    } else {
        x = sign | ((exp - 15 + 127) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

namespace {

uint32_t get_u32(const unsigned char* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

uint64_t get_u64(const unsigned char* p) {
    return (uint64_t)get_u32(p) | ((uint64_t)get_u32(p + 4) << 32);
}

}  // namespace

bool read_exr_channel(const char* path, const char* channel, int* width, int* height,
                      std::vector<float>& out, std::string& err) {
    std::FILE* fp = std::fopen(path, "rb");
    if (!fp) {
        err = std::string("cannot open ") + path;
        return false;
    }
    std::vector<unsigned char> d;
    unsigned char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), fp)) > 0) d.insert(d.end(), buf, buf + n);
    std::fclose(fp);
    auto bad = [&](const char* why) {
        err = std::string(path) + ": " + why;
        return false;
    };
    if (d.size() < 8 || d[0] != 0x76 || d[1] != 0x2f || d[2] != 0x31 || d[3] != 0x01)
        return bad("not an OpenEXR file");
    const uint32_t version = get_u32(&d[4]);
    if ((version & 0xffu) != 2u || (version & 0x1e00u) != 0u)
        return bad("only single-part scanline files are read");
    // header attributes
    struct Chan { std::string name; int type; };
    std::vector<Chan> chans;
    int comp = -1, x0 = 0, y0 = 0, x1 = -1, y1 = -1, order = 0;
    size_t i = 8;
    auto cstr = [&](std::string& s) {
        const size_t e = i;
        while (i < d.size() && d[i] != 0) ++i;
        if (i >= d.size()) return false;
        s.assign((const char*)&d[e], i - e);
        ++i;
        return true;
    };
    for (;;) {
        std::string name, type;
        if (!cstr(name)) return bad("truncated header");
        if (name.empty()) break;
        if (!cstr(type) || i + 4 > d.size()) return bad("truncated header");
        const uint32_t size = get_u32(&d[i]);
        i += 4;
        if (i + size > d.size()) return bad("truncated header");
        const unsigned char* v = &d[i];
        if (name == "channels") {
            size_t k = 0;
            while (k < size && v[k] != 0) {
                size_t e = k;
                while (e < size && v[e] != 0) ++e;
                if (e + 17 > size) return bad("bad channel list");
                chans.push_back({std::string((const char*)v + k, e - k), (int)get_u32(v + e + 1)});
                const int xs = (int)get_u32(v + e + 9), ys = (int)get_u32(v + e + 13);
                if (xs != 1 || ys != 1) return bad("subsampled channels are not read");
                k = e + 17;
            }
        } else if (name == "compression") {
            comp = v[0];
        } else if (name == "dataWindow") {
            x0 = (int)get_u32(v); y0 = (int)get_u32(v + 4);
            x1 = (int)get_u32(v + 8); y1 = (int)get_u32(v + 12);
        } else if (name == "lineOrder") {
            order = v[0];
        }
        i += size;
    }
    if (comp != 0) return bad("only uncompressed files are read");
    if (order != 0 && order != 1) return bad("random line order is not read");
    const int w = x1 - x0 + 1, h = y1 - y0 + 1;
    if (w <= 0 || h <= 0 || (long long)w * h > (1ll << 28)) return bad("bad data window");
    // channels are stored in the listed (alphabetical) order within a scanline
    int want = -1;
    size_t offset = 0, line = 0;
    for (size_t c = 0; c < chans.size(); ++c) {
        const int bytes = chans[c].type == 1 ? 2 : 4;  // HALF, else UINT / FLOAT
        if (chans[c].type < 0 || chans[c].type > 2) return bad("unknown pixel type");
        if (chans[c].name == channel) {
            want = (int)c;
            offset = line;
        }
        line += (size_t)bytes * w;
    }
    if (want < 0) return bad((std::string("no channel ") + channel).c_str());
    const int type = chans[want].type;
    // line-offset table, then one scanline per chunk: y, size, data
    if (i + 8ull * h > d.size()) return bad("truncated offset table");
    out.assign((size_t)w * h, 0.0f);
    for (int r = 0; r < h; ++r) {
        const uint64_t at = get_u64(&d[i + 8ull * r]);
        if (at + 8 > d.size()) return bad("bad chunk offset");
        const int y = (int)get_u32(&d[at]) - y0;
        const uint32_t size = get_u32(&d[at + 4]);
        if (y < 0 || y >= h || size != line || at + 8 + size > d.size()) return bad("bad chunk");
        const unsigned char* p = &d[at + 8 + offset];
        float* o = &out[(size_t)y * w];
        for (int x = 0; x < w; ++x) {
            if (type == 1) {
                o[x] = half_to_float((unsigned short)(p[2 * x] | (p[2 * x + 1] << 8)));
            } else {
                const uint32_t u = get_u32(p + 4 * x);
                if (type == 2) {
                    std::memcpy(&o[x], &u, 4);
                } else {
                    o[x] = (float)u;
                }
            }
        }
    }
    *width = w;
    *height = h;
    return true;
}

void resize_linear(const float* src, int sw, int sh, float* dst, int dw, int dh) {
    // source index and weight of every destination column / row
    auto taps = [](int s, int dn, std::vector<int>& i0, std::vector<float>& w1) {
        const double scale = (double)s / dn;
        i0.resize(dn);
        w1.resize(dn);
        for (int k = 0; k < dn; ++k) {
            float f = (float)((k + 0.5) * scale - 0.5);
            int i = (int)std::floor(f);
            f -= (float)i;
            if (i < 0) {
                i = 0;
                f = 0.0f;
            }
            if (i >= s - 1) {
                i = s - 1;
                f = 0.0f;
            }
            i0[k] = i;
            w1[k] = f;
        }
    };
    std::vector<int> xi, yi;
    std::vector<float> xw, yw;
    taps(sw, dw, xi, xw);
    taps(sh, dh, yi, yw);
    for (int y = 0; y < dh; ++y) {
        const float* r0 = src + (size_t)yi[y] * sw;
        const float* r1 = src + (size_t)(yi[y] + 1 < sh ? yi[y] + 1 : yi[y]) * sw;
        const float b = yw[y];
        for (int x = 0; x < dw; ++x) {
            const int i = xi[x], j = i + 1 < sw ? i + 1 : i;
            const float a = xw[x];
            const float top = r0[i] * (1.0f - a) + r0[j] * a;
            const float bot = r1[i] * (1.0f - a) + r1[j] * a;
            dst[(size_t)y * dw + x] = top * (1.0f - b) + bot * b;
        }
    }
}

}  // namespace sb
