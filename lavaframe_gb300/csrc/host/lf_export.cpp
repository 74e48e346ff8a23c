// Image export: PNG (zlib stream of stored deflate blocks, CRC-32 and Adler-32 per the PNG and
// zlib specifications), binary PPM and PFM. Replaces the stb_image_write / tinyexr calls of
// Export.h:14-151 for the formats a headless render needs.
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
