// Image export: PNG (row filters chosen per row, deflated; CRC-32 and Adler-32 per the PNG and
// zlib specifications), BMP (24-bit, uncompressed), TGA (run-length encoded true colour, the
// form stb_image_write writes by default), OpenEXR (single-part scanline, 32-bit float B, G, R
// channels; none, RLE, ZIPS or ZIP compression, ZIP by default as in the reference), baseline JPEG (ITU-T T.81: 4:4:4 YCbCr, quality-scaled Annex K
// quantisation tables, Huffman tables built for each image by the Annex K.2 procedure), binary
// PPM and PFM. Replaces the stb_image_write / tinyexr calls of Export.h:14-151 (tinyexr's PIZ
// and ZFP compressors are not written here). Deflate is this file's own: one block with the fixed
// Huffman codes of RFC 1951 and hash-chain LZ77 matches.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
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

// ---------------------------------------------------------------- zlib / deflate (RFC 1950/1951)
// One deflate block with the fixed Huffman codes of RFC 1951 section 3.2.6 and LZ77 matches
// found through hash chains over 3-byte prefixes (32 KiB window, at most 64 candidates).
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

struct LsbWriter   // deflate packs bits from the least significant end
{
    std::vector<uint8_t>& out;
    uint64_t acc = 0;
    int n = 0;
    void bits(uint32_t v, int len)
    {
        acc |= (uint64_t)v << n;
        n += len;
        while (n >= 8)
        {
            out.push_back((uint8_t)acc);
            acc >>= 8;
            n -= 8;
        }
    }
    void code(uint32_t c, int len)   // Huffman codes go most significant bit first
    {
        uint32_t r = 0;
        for (int i = 0; i < len; ++i) r |= ((c >> i) & 1u) << (len - 1 - i);
        bits(r, len);
    }
    void flush()
    {
        if (n) out.push_back((uint8_t)acc);
        acc = 0;
        n = 0;
    }
};

void fixed_symbol(LsbWriter& w, int sym)
{
    if (sym < 144) w.code(0x30 + sym, 8);
    else if (sym < 256) w.code(0x190 + (sym - 144), 9);
    else if (sym < 280) w.code(sym - 256, 7);
    else w.code(0xC0 + (sym - 280), 8);
}

std::vector<uint8_t> zlib_compress(const std::vector<uint8_t>& in)
{
    std::vector<uint8_t> out{0x78, 0x01};
    LsbWriter w{out};
    w.bits(1, 1);   // final block
    w.bits(1, 2);   // fixed Huffman codes
    const int kWindow = 32768, kHash = 1 << 15, kChain = 64;
    std::vector<int> head(kHash, -1), prev(kWindow, -1);
    auto hash3 = [&](size_t i) { return ((in[i] << 10) ^ (in[i + 1] << 5) ^ in[i + 2]) & (kHash - 1); };
    auto insert = [&](size_t i) {
        if (i + 2 >= in.size()) return;
        const int h = hash3(i);
        prev[i & (kWindow - 1)] = head[h];
        head[h] = (int)i;
    };
    size_t i = 0;
    while (i < in.size())
    {
        int bestLen = 0, bestDist = 0;
        if (i + 2 < in.size())
        {
            int cand = head[hash3(i)];
            for (int k = 0; k < kChain && cand >= 0 && (int)i - cand <= kWindow - 1; ++k)
            {
                const size_t maxLen = std::min<size_t>(258, in.size() - i);
                size_t l = 0;
                while (l < maxLen && in[cand + l] == in[i + l]) ++l;
                if ((int)l > bestLen)
                {
                    bestLen = (int)l;
                    bestDist = (int)i - cand;
                    if (l == maxLen) break;
                }
                const int nxt = prev[cand & (kWindow - 1)];
                if (nxt >= cand) break;   // the chain slot was reused by a newer position
                cand = nxt;
            }
        }
        if (bestLen >= 3)
        {
            int lc = 28;
            while (kLenBase[lc] > bestLen) --lc;
            fixed_symbol(w, 257 + lc);
            w.bits((uint32_t)(bestLen - kLenBase[lc]), kLenExtra[lc]);
            int dc = 29;
            while (kDistBase[dc] > bestDist) --dc;
            w.code((uint32_t)dc, 5);
            w.bits((uint32_t)(bestDist - kDistBase[dc]), kDistExtra[dc]);
            for (int k = 0; k < bestLen; ++k) insert(i + k);
            i += bestLen;
        }
        else
        {
            fixed_symbol(w, in[i]);
            insert(i);
            ++i;
        }
    }
    fixed_symbol(w, 256);   // end of block
    w.flush();
    uint32_t a = 1, b = 0;
    for (uint8_t c : in)
    {
        a = (a + c) % 65521;
        b = (b + a) % 65521;
    }
    put32(out, (b << 16) | a);
    return out;
}

// OpenEXR's run-length code: a run of 3 to 128 equal bytes is (count - 1, byte); other bytes go
// in literal groups of up to 128 as (-count, bytes...).
std::vector<uint8_t> rle_compress(const std::vector<uint8_t>& in)
{
    std::vector<uint8_t> out;
    size_t i = 0;
    while (i < in.size())
    {
        size_t run = 1;
        while (i + run < in.size() && run < 128 && in[i + run] == in[i]) ++run;
        if (run >= 3)
        {
            out.push_back((uint8_t)(run - 1));
            out.push_back(in[i]);
            i += run;
            continue;
        }
        size_t lit = 0;   // up to the next run of three
        while (i + lit < in.size() && lit < 128 &&
               !(i + lit + 2 < in.size() && in[i + lit] == in[i + lit + 1] && in[i + lit] == in[i + lit + 2]))
            ++lit;
        out.push_back((uint8_t)(-(int)lit));
        out.insert(out.end(), in.begin() + (long)i, in.begin() + (long)(i + lit));
        i += lit;
    }
    return out;
}

// ---------------------------------------------------------------- baseline JPEG (ITU-T T.81)
// Example quantisation tables of T.81 Annex K.1 (natural order), scaled by quality the way the
// IJG library does: scale = 5000 / q below 50, 200 - 2 q from there.
const uint8_t kLumaQ[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                            14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                            18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                            49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
const uint8_t kChromaQ[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99,
                              24, 26, 56, 99, 99, 99, 99, 99, 47, 66, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};

// zigzag position k -> natural index (row * 8 + column)
void zigzag(int zz[64])
{
    int k = 0;
    for (int s = 0; s < 15; ++s)
        for (int i = 0; i < 8; ++i)
        {
            const int r = (s % 2) ? i : s - i;   // odd diagonals run down-left, even ones up-right
            const int c = s - r;
            if (r < 0 || r > 7 || c < 0 || c > 7) continue;
            zz[k++] = r * 8 + c;
        }
}

int category(int v)
{
    int a = v < 0 ? -v : v, n = 0;
    while (a) { ++n; a >>= 1; }
    return n;
}

// Code lengths for the symbols with nonzero counts (Annex K.2: Huffman procedure with one
// reserved code point so that no code is all ones, lengths limited to 16 bits), returned as
// the DHT BITS / HUFFVAL lists and per-symbol code and length.
struct HuffTable
{
    uint8_t bits[17] = {};
    std::vector<uint8_t> vals;
    uint16_t code[256] = {};
    uint8_t len[256] = {};
};

void build_huffman(const uint32_t freqIn[256], HuffTable& t)
{
    long long freq[257];
    int codesize[257], others[257];
    for (int i = 0; i < 256; ++i) freq[i] = freqIn[i];
    freq[256] = 1;   // reserved point
    for (int i = 0; i < 257; ++i)
    {
        codesize[i] = 0;
        others[i] = -1;
    }
    while (true)   // Figure K.1
    {
        int v1 = -1, v2 = -1;
        for (int i = 0; i < 257; ++i)
            if (freq[i] > 0 && (v1 < 0 || freq[i] <= freq[v1])) v1 = i;
        for (int i = 0; i < 257; ++i)
            if (freq[i] > 0 && i != v1 && (v2 < 0 || freq[i] <= freq[v2])) v2 = i;
        if (v2 < 0) break;
        freq[v1] += freq[v2];
        freq[v2] = 0;
        for (++codesize[v1]; others[v1] >= 0; ++codesize[v1]) v1 = others[v1];
        others[v1] = v2;
        for (++codesize[v2]; others[v2] >= 0; ++codesize[v2]) v2 = others[v2];
    }
    int bits[258] = {};   // code sizes reach at most 256 with 257 points
    for (int i = 0; i < 257; ++i)
        if (codesize[i]) ++bits[codesize[i]];
    for (int i = 257; i > 16; --i)   // Figure K.3: limit to 16 bits
        while (bits[i] > 0)
        {
            int j = i - 2;
            while (bits[j] == 0) --j;
            bits[i] -= 2;
            ++bits[i - 1];
            bits[j + 1] += 2;
            --bits[j];
        }
    int last = 16;
    while (bits[last] == 0) --last;
    --bits[last];   // drop the reserved point
    // symbols by code size, then value (Figure K.4); the reserved point sorts last
    t.vals.clear();
    for (int size = 1; size <= 257; ++size)
        for (int i = 0; i < 256; ++i)
            if (codesize[i] == size) t.vals.push_back((uint8_t)i);
    for (int i = 1; i <= 16; ++i) t.bits[i] = (uint8_t)bits[i];
    // canonical codes (Annex C)
    int k = 0;
    uint16_t code = 0;
    for (int l = 1; l <= 16; ++l)
    {
        for (int n = 0; n < bits[l]; ++n, ++k)
        {
            t.code[t.vals[k]] = code++;
            t.len[t.vals[k]] = (uint8_t)l;
        }
        code <<= 1;
    }
    t.vals.resize(k);
}

struct BitWriter
{
    std::vector<uint8_t>& out;
    uint32_t acc = 0;
    int n = 0;
    void put(uint32_t bits, int len)
    {
        for (int i = len - 1; i >= 0; --i)
        {
            acc = (acc << 1) | ((bits >> i) & 1u);
            if (++n == 8)
            {
                out.push_back((uint8_t)acc);
                if (acc == 0xFF) out.push_back(0);   // byte stuffing
                acc = 0;
                n = 0;
            }
        }
    }
    void flush()
    {
        while (n) put(1, 1);   // pad with ones
    }
};

void marker(std::vector<uint8_t>& o, uint8_t m, const std::vector<uint8_t>& body)
{
    o.push_back(0xFF);
    o.push_back(m);
    o.push_back((uint8_t)((body.size() + 2) >> 8));
    o.push_back((uint8_t)(body.size() + 2));
    o.insert(o.end(), body.begin(), body.end());
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
    // scanlines top row first, each with the filter (none, sub, up, average, Paeth; PNG
    // specification section 9) whose output has the smallest sum of absolute signed values
    const size_t n = (size_t)w * 3;
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (1 + n));
    std::vector<uint8_t> zero(n, 0), cand[5];
    for (auto& c : cand) c.resize(n);
    for (int y = h - 1; y >= 0; --y)
    {
        const uint8_t* row = rgb8 + (size_t)y * n;
        const uint8_t* up = y + 1 < h ? rgb8 + (size_t)(y + 1) * n : zero.data();
        for (size_t i = 0; i < n; ++i)
        {
            const int x = row[i], a = i >= 3 ? row[i - 3] : 0, b = up[i], c = i >= 3 ? up[i - 3] : 0;
            const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
            const int paeth = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
            cand[0][i] = (uint8_t)x;
            cand[1][i] = (uint8_t)(x - a);
            cand[2][i] = (uint8_t)(x - b);
            cand[3][i] = (uint8_t)(x - ((a + b) >> 1));
            cand[4][i] = (uint8_t)(x - paeth);
        }
        int best = 0;
        long long bestSum = -1;
        for (int f = 0; f < 5; ++f)
        {
            long long sum = 0;
            for (size_t i = 0; i < n; ++i) sum += std::abs((int)(int8_t)cand[f][i]);
            if (bestSum < 0 || sum < bestSum)
            {
                bestSum = sum;
                best = f;
            }
        }
        raw.push_back((uint8_t)best);
        raw.insert(raw.end(), cand[best].begin(), cand[best].end());
    }
    const std::vector<uint8_t> z = zlib_compress(raw);
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

lf_status lf_write_exr_compressed(const char* path, const float* rgbf, int32_t w, int32_t h, int32_t compression)
{
    if (!path || !rgbf || w <= 0 || h <= 0 || compression < 0 || compression > 3) return LF_ERR_INVALID;
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
    // 0 none and 1 RLE (one scanline per block), 2 ZIPS (one), 3 ZIP (16)
    exr_attr(out, "compression", "compression", {(uint8_t)compression});
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
    // blocks of scanlines: the offset table, then per block its first y, byte count and data.
    // Rows go out in the order given (the reference writes the bottom-first GL buffer as is).
    // A block's data is its rows' B, G and R channels; RLE and ZIP split the bytes into even and
    // odd positions and difference them (d[i] - d[i-1] + 128), then run-length code or deflate
    // them; when that is not smaller, the raw rows are stored.
    const int lines = compression == 3 ? 16 : 1;
    const int nBlocks = (h + lines - 1) / lines;
    const size_t table = out.size();
    out.resize(table + (size_t)nBlocks * 8);
    std::vector<uint8_t> raw, mixed;
    for (int blk = 0; blk < nBlocks; ++blk)
    {
        const int y0 = blk * lines, y1 = std::min(h, y0 + lines);
        raw.clear();
        for (int y = y0; y < y1; ++y)
        {
            const float* row = rgbf + (size_t)y * w * 3;
            for (int c = 2; c >= 0; --c)
                for (int x = 0; x < w; ++x) put_f32(raw, row[x * 3 + c]);
        }
        std::vector<uint8_t> z;
        if (compression > 0)
        {
            mixed.resize(raw.size());
            const size_t half = (raw.size() + 1) / 2;
            for (size_t k = 0; k < raw.size(); ++k) mixed[(k & 1) ? half + k / 2 : k / 2] = raw[k];
            for (size_t k = mixed.size() - 1; k > 0; --k) mixed[k] = (uint8_t)(mixed[k] - mixed[k - 1] + 128);
            z = compression == 1 ? rle_compress(mixed) : zlib_compress(mixed);
        }
        const std::vector<uint8_t>& data = compression > 0 && z.size() < raw.size() ? z : raw;
        const size_t at = out.size();
        for (int k = 0; k < 8; ++k) out[table + (size_t)blk * 8 + k] = (uint8_t)((uint64_t)at >> (8 * k));
        put_le(out, (uint32_t)y0, 4);
        put_le(out, data.size(), 4);
        out.insert(out.end(), data.begin(), data.end());
    }
    return write_file(path, out.data(), out.size()) ? LF_OK : LF_ERR_IO;
}

lf_status lf_write_exr(const char* path, const float* rgbf, int32_t w, int32_t h)
{
    return lf_write_exr_compressed(path, rgbf, w, h, 3);
}

lf_status lf_write_jpg(const char* path, const uint8_t* rgb8, int32_t w, int32_t h, int32_t quality)
{
    if (!path || !rgb8 || w <= 0 || h <= 0 || w > 65535 || h > 65535) return LF_ERR_INVALID;
    const int q = std::max(1, std::min(100, quality));
    const int scale = q < 50 ? 5000 / q : 200 - 2 * q;
    int zz[64];
    zigzag(zz);
    uint8_t qt[2][64];
    for (int i = 0; i < 64; ++i)
    {
        qt[0][i] = (uint8_t)std::max(1, std::min(255, (kLumaQ[i] * scale + 50) / 100));
        qt[1][i] = (uint8_t)std::max(1, std::min(255, (kChromaQ[i] * scale + 50) / 100));
    }
    double cosv[8][8];
    for (int x = 0; x < 8; ++x)
        for (int u = 0; u < 8; ++u) cosv[x][u] = std::cos((2 * x + 1) * u * 3.14159265358979323846 / 16.0);
    // quantised coefficients of every block, zigzag order; components interleaved per block
    const int bw = (w + 7) / 8, bh = (h + 7) / 8;
    std::vector<int16_t> coef((size_t)bw * bh * 3 * 64);
    for (int by = 0; by < bh; ++by)
        for (int bx = 0; bx < bw; ++bx)
        {
            double ycc[3][64];
            for (int y = 0; y < 8; ++y)
                for (int x = 0; x < 8; ++x)
                {
                    // JPEG rows run top down; the input's row 0 is the bottom. Edges repeat.
                    const int iy = std::min(h - 1, by * 8 + y), ix = std::min(w - 1, bx * 8 + x);
                    const uint8_t* p = rgb8 + ((size_t)(h - 1 - iy) * w + ix) * 3;
                    const double r = p[0], g = p[1], b = p[2];
                    ycc[0][y * 8 + x] = 0.299 * r + 0.587 * g + 0.114 * b - 128.0;   // JFIF YCbCr, level shift
                    ycc[1][y * 8 + x] = -0.168736 * r - 0.331264 * g + 0.5 * b;
                    ycc[2][y * 8 + x] = 0.5 * r - 0.418688 * g - 0.081312 * b;
                }
            for (int c = 0; c < 3; ++c)
            {
                // separable DCT-II: along rows (x -> u), then along columns (y -> v)
                double row[8][8], dct[8][8];
                for (int y = 0; y < 8; ++y)
                    for (int u = 0; u < 8; ++u)
                    {
                        double sum = 0.0;
                        for (int x = 0; x < 8; ++x) sum += ycc[c][y * 8 + x] * cosv[x][u];
                        row[y][u] = sum;
                    }
                for (int v = 0; v < 8; ++v)
                    for (int u = 0; u < 8; ++u)
                    {
                        double sum = 0.0;
                        for (int y = 0; y < 8; ++y) sum += row[y][u] * cosv[y][v];
                        const double cu = u ? 1.0 : 1.0 / std::sqrt(2.0), cv = v ? 1.0 : 1.0 / std::sqrt(2.0);
                        dct[v][u] = 0.25 * cu * cv * sum;
                    }
                int16_t* out = &coef[(((size_t)by * bw + bx) * 3 + c) * 64];
                for (int k = 0; k < 64; ++k)
                    out[k] = (int16_t)std::lround(dct[zz[k] >> 3][zz[k] & 7] / qt[c ? 1 : 0][zz[k]]);
            }
        }
    // symbol statistics, then Huffman tables (DC and AC for luma and for chroma)
    uint32_t freq[4][256] = {};
    auto walk = [&](auto&& emit) {
        int pred[3] = {0, 0, 0};
        for (size_t blk = 0; blk < (size_t)bw * bh; ++blk)
            for (int c = 0; c < 3; ++c)
            {
                const int16_t* cf = &coef[(blk * 3 + c) * 64];
                const int t = c ? 1 : 0;
                const int diff = cf[0] - pred[c];
                pred[c] = cf[0];
                emit(t * 2, category(diff), diff);
                int run = 0;
                for (int k = 1; k < 64; ++k)
                {
                    if (cf[k] == 0)
                    {
                        ++run;
                        continue;
                    }
                    while (run > 15)
                    {
                        emit(t * 2 + 1, 0xF0, 0);   // ZRL
                        run -= 16;
                    }
                    const int sz = category(cf[k]);
                    emit(t * 2 + 1, (run << 4) | sz, cf[k]);
                    run = 0;
                }
                if (run) emit(t * 2 + 1, 0x00, 0);   // EOB
            }
    };
    walk([&](int table, int sym, int) { ++freq[table][sym]; });
    HuffTable ht[4];
    for (int i = 0; i < 4; ++i) build_huffman(freq[i], ht[i]);

    std::vector<uint8_t> o{0xFF, 0xD8};
    marker(o, 0xE0, {'J', 'F', 'I', 'F', 0, 1, 1, 0, 0, 1, 0, 1, 0, 0});   // JFIF 1.01, aspect 1:1
    for (int t = 0; t < 2; ++t)
    {
        std::vector<uint8_t> body{(uint8_t)t};
        for (int k = 0; k < 64; ++k) body.push_back(qt[t][zz[k]]);
        marker(o, 0xDB, body);
    }
    marker(o, 0xC0, {8, (uint8_t)(h >> 8), (uint8_t)h, (uint8_t)(w >> 8), (uint8_t)w, 3, 1, 0x11, 0, 2, 0x11, 1, 3,
                     0x11, 1});
    const uint8_t classId[4] = {0x00, 0x10, 0x01, 0x11};   // DC luma, AC luma, DC chroma, AC chroma
    for (int i = 0; i < 4; ++i)
    {
        std::vector<uint8_t> body{classId[i]};
        body.insert(body.end(), ht[i].bits + 1, ht[i].bits + 17);
        body.insert(body.end(), ht[i].vals.begin(), ht[i].vals.end());
        marker(o, 0xC4, body);
    }
    marker(o, 0xDA, {3, 1, 0x00, 2, 0x11, 3, 0x11, 0, 63, 0});
    BitWriter bw8{o};
    walk([&](int table, int sym, int v) {
        bw8.put(ht[table].code[sym], ht[table].len[sym]);
        const int sz = (table & 1) ? (sym & 15) : sym;
        if (sz) bw8.put((uint32_t)(v < 0 ? v - 1 : v) & ((1u << sz) - 1u), sz);
    });
    bw8.flush();
    o.push_back(0xFF);
    o.push_back(0xD9);
    return write_file(path, o.data(), o.size()) ? LF_OK : LF_ERR_IO;
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
