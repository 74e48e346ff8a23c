// Image export: PNG (zlib stream of stored deflate blocks, CRC-32 and Adler-32 per the PNG and
// zlib specifications), BMP (24-bit, uncompressed), TGA (run-length encoded true colour, the
// form stb_image_write writes by default), OpenEXR (single-part scanline, 32-bit float B, G, R
// channels, no compression), binary PPM and PFM. Replaces the stb_image_write / tinyexr calls
// of Export.h:14-151 (JPG and tinyexr's compressors are not written here).
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../../include/lavaframe_gb300.h"

namespace
{
uint32_t crc32(const uint8_t* p, size_t n, uint32_t crc = 0)
{
    static uint32_t table[256];
    static bool init = false;
    if (!init)
    {
        for (uint32_t i = 0; i < 256; ++i)
        {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        init = true;
    }
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
    return ~crc;
}

void put32(std::vector<uint8_t>& v, uint32_t x)
{
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data)
{
    put32(out, (uint32_t)data.size());
    std::vector<uint8_t> td(type, type + 4);
    td.insert(td.end(), data.begin(), data.end());
    out.insert(out.end(), td.begin(), td.end());
    put32(out, crc32(td.data(), td.size()));
}

void put_le(std::vector<uint8_t>& v, uint64_t x, int bytes)
{
    for (int k = 0; k < bytes; ++k) v.push_back((uint8_t)(x >> (8 * k)));
}

void put_f32(std::vector<uint8_t>& v, float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    put_le(v, u, 4);
}

// OpenEXR header attribute: name, type name, byte size, value
void exr_attr(std::vector<uint8_t>& v, const char* name, const char* type, const std::vector<uint8_t>& value)
{
    v.insert(v.end(), name, name + std::strlen(name) + 1);
    v.insert(v.end(), type, type + std::strlen(type) + 1);
    put_le(v, value.size(), 4);
    v.insert(v.end(), value.begin(), value.end());
}

bool write_file(const char* path, const void* data, size_t n)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    const bool ok = std::fwrite(data, 1, n, f) == n;
    return std::fclose(f) == 0 && ok;
}
}

extern "C" {

lf_status lf_write_png(const char* path, const uint8_t* rgb8, int32_t w, int32_t h)
{
    if (!path || !rgb8 || w <= 0 || h <= 0) return LF_ERR_INVALID;
    // raw scanlines, top row first, filter type 0
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (1 + (size_t)w * 3));
    for (int y = h - 1; y >= 0; --y)
    {
        raw.push_back(0);
        const uint8_t* row = rgb8 + (size_t)y * w * 3;
        raw.insert(raw.end(), row, row + (size_t)w * 3);
    }
    // zlib: header, stored blocks of at most 65535 bytes, Adler-32
    std::vector<uint8_t> z{0x78, 0x01};
    size_t pos = 0;
    do
    {
        const size_t len = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(len & 0xff));
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)(~len & 0xff));
        z.push_back((uint8_t)((~len >> 8) & 0xff));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
        pos += len;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw)
    {
        a = (a + c) % 65521;
        b = (b + a) % 65521;
    }
    put32(z, (b << 16) | a);
    std::vector<uint8_t> png{0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
    std::vector<uint8_t> ihdr;
    put32(ihdr, (uint32_t)w);
    put32(ihdr, (uint32_t)h);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});   // 8-bit RGB, deflate, no filter method, no interlace
    chunk(png, "IHDR", ihdr);
    chunk(png, "IDAT", z);
    chunk(png, "IEND", {});
    return write_file(path, png.data(), png.size()) ? LF_OK : LF_ERR_IO;
}

lf_status lf_write_bmp(const char* path, const uint8_t* rgb8, int32_t w, int32_t h)
{
    if (!path || !rgb8 || w <= 0 || h <= 0) return LF_ERR_INVALID;
    const size_t stride = ((size_t)w * 3 + 3) / 4 * 4;   // rows padded to 4 bytes
    const size_t pixels = stride * h;
    std::vector<uint8_t> out;
    out.reserve(54 + pixels);
    // BITMAPFILEHEADER
    out.push_back('B');
    out.push_back('M');
    put_le(out, 54 + pixels, 4);
    put_le(out, 0, 4);
    put_le(out, 54, 4);
    // BITMAPINFOHEADER: positive height = rows stored bottom-up, 24 bits, BI_RGB
    put_le(out, 40, 4);
    put_le(out, (uint32_t)w, 4);
    put_le(out, (uint32_t)h, 4);
    put_le(out, 1, 2);
    put_le(out, 24, 2);
    put_le(out, 0, 4);
    put_le(out, pixels, 4);
    put_le(out, 2835, 4);   // 72 dpi
    put_le(out, 2835, 4);
    put_le(out, 0, 4);
    put_le(out, 0, 4);
    for (int y = 0; y < h; ++y)   // the input's bottom row first, as BMP stores it
    {
        const uint8_t* row = rgb8 + (size_t)y * w * 3;
        for (int x = 0; x < w; ++x)
        {
            out.push_back(row[x * 3 + 2]);
            out.push_back(row[x * 3 + 1]);
            out.push_back(row[x * 3 + 0]);
        }
        for (size_t k = (size_t)w * 3; k < stride; ++k) out.push_back(0);
    }
    return write_file(path, out.data(), out.size()) ? LF_OK : LF_ERR_IO;
}

lf_status lf_write_tga(const char* path, const uint8_t* rgb8, int32_t w, int32_t h)
{
    if (!path || !rgb8 || w <= 0 || h <= 0 || w > 65535 || h > 65535) return LF_ERR_INVALID;
    std::vector<uint8_t> out;
    // header: no id, no colour map, type 10 (run-length true colour), origin bottom left
    const uint8_t hdr[18] = {0, 0, 10, 0, 0, 0, 0, 0, 0, 0, 0, 0, (uint8_t)w, (uint8_t)(w >> 8), (uint8_t)h,
                             (uint8_t)(h >> 8), 24, 0};
    out.insert(out.end(), hdr, hdr + 18);
    auto px = [&](const uint8_t* p) {
        out.push_back(p[2]);
        out.push_back(p[1]);
        out.push_back(p[0]);
    };
    for (int y = 0; y < h; ++y)   // bottom row first; packets never cross a row
    {
        const uint8_t* row = rgb8 + (size_t)y * w * 3;
        int x = 0;
        while (x < w)
        {
            int run = 1;   // equal pixels from x
            while (x + run < w && run < 128 && std::memcmp(row + (x + run) * 3, row + x * 3, 3) == 0) ++run;
            if (run > 1)
            {
                out.push_back((uint8_t)(0x80 | (run - 1)));
                px(row + x * 3);
                x += run;
                continue;
            }
            int lit = 1;   // pixels up to the next pair of equal ones
            while (x + lit < w && lit < 128 &&
                   !(x + lit + 1 < w && std::memcmp(row + (x + lit) * 3, row + (x + lit + 1) * 3, 3) == 0))
                ++lit;
            out.push_back((uint8_t)(lit - 1));
            for (int k = 0; k < lit; ++k) px(row + (x + k) * 3);
            x += lit;
        }
    }
    const char footer[] = "\0\0\0\0\0\0\0\0TRUEVISION-XFILE.";   // TGA 2.0: no extension or developer area
    out.insert(out.end(), footer, footer + sizeof footer);
    return write_file(path, out.data(), out.size()) ? LF_OK : LF_ERR_IO;
}

lf_status lf_write_exr(const char* path, const float* rgbf, int32_t w, int32_t h)
{
    if (!path || !rgbf || w <= 0 || h <= 0) return LF_ERR_INVALID;
    std::vector<uint8_t> out{0x76, 0x2f, 0x31, 0x01, 2, 0, 0, 0};   // magic, version 2, scanline
    std::vector<uint8_t> v;
    for (const char* c : {"B", "G", "R"})   // channel list in name order, 32-bit float, 1x1 sampling
    {
        v.push_back((uint8_t)c[0]);
        v.push_back(0);
        put_le(v, 2, 4);
        put_le(v, 0, 4);   // pLinear + reserved
        put_le(v, 1, 4);
        put_le(v, 1, 4);
    }
    v.push_back(0);
    exr_attr(out, "channels", "chlist", v);
    exr_attr(out, "compression", "compression", {0});
    v.clear();
    for (int32_t k : {0, 0, w - 1, h - 1}) put_le(v, (uint32_t)k, 4);
    exr_attr(out, "dataWindow", "box2i", v);
    exr_attr(out, "displayWindow", "box2i", v);
    exr_attr(out, "lineOrder", "lineOrder", {0});
    v.clear();
    put_f32(v, 1.0f);
    exr_attr(out, "pixelAspectRatio", "float", v);
    v.clear();
    put_f32(v, 0.0f);
    put_f32(v, 0.0f);
    exr_attr(out, "screenWindowCenter", "v2f", v);
    v.clear();
    put_f32(v, 1.0f);
    exr_attr(out, "screenWindowWidth", "float", v);
    out.push_back(0);
    // one scanline per block: the offset table, then y, byte count and the B, G and R rows.
    // Rows go out in the order given (the reference writes the bottom-first GL buffer as is).
    const size_t rowBytes = (size_t)w * 3 * 4;
    const size_t table = out.size();
    for (int y = 0; y < h; ++y) put_le(out, table + (size_t)h * 8 + (size_t)y * (8 + rowBytes), 8);
    for (int y = 0; y < h; ++y)
    {
        put_le(out, (uint32_t)y, 4);
        put_le(out, rowBytes, 4);
        const float* row = rgbf + (size_t)y * w * 3;
        for (int c = 2; c >= 0; --c)
            for (int x = 0; x < w; ++x) put_f32(out, row[x * 3 + c]);
    }
    return write_file(path, out.data(), out.size()) ? LF_OK : LF_ERR_IO;
}

lf_status lf_write_ppm(const char* path, const uint8_t* rgb8, int32_t w, int32_t h)
{
    if (!path || !rgb8 || w <= 0 || h <= 0) return LF_ERR_INVALID;
    char hdr[64];
    const int n = std::snprintf(hdr, sizeof hdr, "P6\n%d %d\n255\n", w, h);
    std::vector<uint8_t> out(hdr, hdr + n);
    for (int y = h - 1; y >= 0; --y)
    {
        const uint8_t* row = rgb8 + (size_t)y * w * 3;
        out.insert(out.end(), row, row + (size_t)w * 3);
    }
    return write_file(path, out.data(), out.size()) ? LF_OK : LF_ERR_IO;
}

lf_status lf_write_pfm(const char* path, const float* rgbf, int32_t w, int32_t h)
{
    if (!path || !rgbf || w <= 0 || h <= 0) return LF_ERR_INVALID;
    char hdr[64];
    const int n = std::snprintf(hdr, sizeof hdr, "PF\n%d %d\n-1.0\n", w, h);   // negative scale: little endian
    std::vector<uint8_t> out(hdr, hdr + n);
    const size_t bytes = (size_t)w * h * 3 * sizeof(float);
    const size_t off = out.size();
    out.resize(off + bytes);
    // stored as the host's floats; the scale's sign says little endian, so convert on big-endian hosts
    for (size_t i = 0; i < (size_t)w * h * 3; ++i)
    {
        uint32_t u;
        std::memcpy(&u, rgbf + i, 4);
        out[off + i * 4 + 0] = (uint8_t)u;
        out[off + i * 4 + 1] = (uint8_t)(u >> 8);
        out[off + i * 4 + 2] = (uint8_t)(u >> 16);
        out[off + i * 4 + 3] = (uint8_t)(u >> 24);
    }
    return write_file(path, out.data(), out.size()) ? LF_OK : LF_ERR_IO;
}
}
