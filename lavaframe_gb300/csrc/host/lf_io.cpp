// Scene file loader, OBJ reader and Radiance HDR reader for the host scene layer.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "lf_scene.h"

namespace LavaFrame
{
namespace
{
    int QuietLog(const char*, ...) { return 0; }
}

// The reference logs through printf (Loader.cpp:42); the library is quiet unless the caller
// installs a logger.
int (*Log)(const char* szFormat, ...) = QuietLog;

// ============================================================== OBJ
namespace
{
    // Decimal-to-double conversion used by tinyobjloader (the OBJ reader vendored by the
    // reference, LavaFrame/tiny_obj_loader.h:866-1003): integer digits accumulate as
    // m = m*10 + d, fraction digits add d*10^-k (k < 8 from a table of double constants,
    // beyond that 10^-k from pow), and an exponent e is applied as ldexp(m * 5^e, e).
    // Parsing the same way keeps the float vertex bits identical to the reference's meshes.
    bool ParseObjDouble(const char* s, const char* end, double* result)
    {
        if (s >= end) return false;
        static const double kFrac[] = {1.0, 0.1, 0.01, 0.001, 0.0001, 0.00001, 0.000001, 0.0000001};
        double mant = 0.0;
        int expo = 0;
        bool neg = false, neg_exp = false, dot_first = false;
        const char* c = s;
        if (*c == '+' || *c == '-')
        {
            neg = (*c == '-');
            ++c;
            if (c != end && *c == '.') dot_first = true;
        }
        else if (*c == '.')
            dot_first = true;
        else if (!(*c >= '0' && *c <= '9'))
            return false;

        int nread = 0;
        if (!dot_first)
        {
            while (c != end && *c >= '0' && *c <= '9')
            {
                mant *= 10;
                mant += (int)(*c - '0');
                ++c;
                ++nread;
            }
            if (nread == 0) return false;
        }
        if (c == end) goto done;
        if (*c == '.')
        {
            ++c;
            int k = 1;
            while (c != end && *c >= '0' && *c <= '9')
            {
                mant += (int)(*c - '0') * (k < 8 ? kFrac[k] : std::pow(10.0, -k));
                ++k;
                ++c;
            }
        }
        else if (!(*c == 'e' || *c == 'E'))
            goto done;
        if (c == end) goto done;
        if (*c == 'e' || *c == 'E')
        {
            ++c;
            if (c != end && (*c == '+' || *c == '-'))
            {
                neg_exp = (*c == '-');
                ++c;
            }
            else if (c == end || !(*c >= '0' && *c <= '9'))
                return false;
            nread = 0;
            while (c != end && *c >= '0' && *c <= '9')
            {
                if (expo > 2147483647 / 10) return false;
                expo = expo * 10 + (int)(*c - '0');
                ++c;
                ++nread;
            }
            if (neg_exp) expo = -expo;
            if (nread == 0) return false;
        }
    done:
        *result = (neg ? -1 : 1) * (expo ? std::ldexp(mant * std::pow(5.0, expo), expo) : mant);
        return true;
    }

    float ParseObjReal(const char*& p, double dflt)
    {
        p += std::strspn(p, " \t");
        const char* e = p + std::strcspn(p, " \t\r\n");
        double v = dflt;
        ParseObjDouble(p, e, &v);
        p = e;
        return (float)v;
    }

    bool ParseObjIndex(const char*& p, int count, int* out)
    {
        char* endp = nullptr;
        long v = std::strtol(p, &endp, 10);
        if (endp == p) return false;
        p = endp;
        if (v > 0) *out = (int)v - 1;
        else if (v < 0) *out = count + (int)v;
        else return false;
        return *out >= 0 && *out < count;
    }

    struct ObjCorner
    {
        int v, vt, vn;
    };
}

namespace
{
    // Corner order of the triangles tinyobjloader emits for one face when the reference
    // builds it with TINYOBJLOADER_USE_MAPBOX_EARCUT (tiny_obj_loader.h:1441-1690):
    //  - quads are split along the shorter diagonal: (0,1,2)(0,2,3) or (0,1,3)(1,2,3);
    //  - every other polygon goes through mapbox earcut in a 2D projection chosen from the
    //    first non-degenerate corner. For a triangle earcut links the corners in its
    //    clockwise order and cuts the single ear at the last linked corner, which yields
    //    (1,2,0) or (1,0,2); a triangle whose projection is degenerate yields nothing.
    //  - polygons with more than four corners are fan-triangulated here (earcut's full
    //    ear-clipping search is not restated).
    std::vector<int> TriangulateFace(const std::vector<ObjCorner>& face, const std::vector<float>& pos)
    {
        const size_t n = face.size();
        auto P = [&](int corner, int axis) { return pos[(size_t)face[corner].v * 3 + axis]; };
        if (n == 4)
        {
            float e02x = P(2, 0) - P(0, 0), e02y = P(2, 1) - P(0, 1), e02z = P(2, 2) - P(0, 2);
            float e13x = P(3, 0) - P(1, 0), e13y = P(3, 1) - P(1, 1), e13z = P(3, 2) - P(1, 2);
            float sqr02 = e02x * e02x + e02y * e02y + e02z * e02z;
            float sqr13 = e13x * e13x + e13y * e13y + e13z * e13z;
            if (sqr02 < sqr13) return {0, 1, 2, 0, 2, 3};
            return {0, 1, 3, 1, 2, 3};
        }
        if (n > 4)
        {
            std::vector<int> out;
            for (size_t k = 1; k + 1 < n; ++k) out.insert(out.end(), {0, (int)k, (int)k + 1});
            return out;
        }
        int axes[2] = {1, 2};
        for (size_t k = 0; k < n; ++k)
        {
            int a = (int)k, b = (int)((k + 1) % n), c = (int)((k + 2) % n);
            float e0x = P(b, 0) - P(a, 0), e0y = P(b, 1) - P(a, 1), e0z = P(b, 2) - P(a, 2);
            float e1x = P(c, 0) - P(b, 0), e1y = P(c, 1) - P(b, 1), e1z = P(c, 2) - P(b, 2);
            float cx = std::fabs(e0y * e1z - e0z * e1y);
            float cy = std::fabs(e0z * e1x - e0x * e1z);
            float cz = std::fabs(e0x * e1y - e0y * e1x);
            const float eps = 1.1920929e-7f;
            if (cx > eps || cy > eps || cz > eps)
            {
                if (!(cx > cy && cx > cz))
                {
                    axes[0] = 0;
                    if (cz > cx && cz > cy) axes[1] = 1;
                }
                break;
            }
        }
        double x[3], y[3];
        for (int k = 0; k < 3; ++k)
        {
            x[k] = (double)P(k, axes[0]);
            y[k] = (double)P(k, axes[1]);
        }
        double sum = 0;
        for (int i = 0, j = 2; i < 3; j = i++)
            sum += (x[j] - x[i]) * (y[i] + y[j]);
        auto area = [&](int p, int q, int r) { return (y[q] - y[p]) * (x[r] - x[q]) - (x[q] - x[p]) * (y[r] - y[q]); };
        auto same = [&](int p, int q) { return x[p] == x[q] && y[p] == y[q]; };
        if (same(0, 2) || same(0, 1) || same(1, 2)) return {};
        if (sum > 0)
            return area(1, 2, 0) < 0 ? std::vector<int>{1, 2, 0} : std::vector<int>{};
        return area(1, 0, 2) < 0 ? std::vector<int>{1, 0, 2} : std::vector<int>{};
    }
}

// OBJ to un-indexed triangle lists (Mesh.cpp:28-90). Triangles come out in file order.
// Polygons with more than three corners are fan-triangulated; faces without a normal
// index get the geometric face normal (the reference reads out of bounds there).
bool Mesh::LoadFromFile(const std::string& filename)
{
    name = filename;
    FILE* f = std::fopen(filename.c_str(), "rb");
    if (!f)
    {
        Log("Unable to load geometry.\n");
        return false;
    }
    std::vector<float> pos, nrm, uv;
    std::vector<ObjCorner> face;
    std::vector<char> buf(1 << 16);
    std::string line;
    bool ok = true;
    verticesUVX.clear();
    normalsUVY.clear();
    while (ok)
    {
        line.clear();
        bool got = false;
        while (std::fgets(buf.data(), (int)buf.size(), f))
        {
            got = true;
            line += buf.data();
            if (!line.empty() && line.back() == '\n') break;
        }
        if (!got) break;
        const char* p = line.c_str();
        p += std::strspn(p, " \t");
        if (p[0] == 'v' && (p[1] == ' ' || p[1] == '\t'))
        {
            p += 2;
            float x = ParseObjReal(p, 0.0), y = ParseObjReal(p, 0.0), z = ParseObjReal(p, 0.0);
            pos.push_back(x); pos.push_back(y); pos.push_back(z);
        }
        else if (p[0] == 'v' && p[1] == 'n' && (p[2] == ' ' || p[2] == '\t'))
        {
            p += 3;
            float x = ParseObjReal(p, 0.0), y = ParseObjReal(p, 0.0), z = ParseObjReal(p, 0.0);
            nrm.push_back(x); nrm.push_back(y); nrm.push_back(z);
        }
        else if (p[0] == 'v' && p[1] == 't' && (p[2] == ' ' || p[2] == '\t'))
        {
            p += 3;
            float u = ParseObjReal(p, 0.0), v = ParseObjReal(p, 0.0);
            uv.push_back(u); uv.push_back(v);
        }
        else if (p[0] == 'f' && (p[1] == ' ' || p[1] == '\t'))
        {
            p += 2;
            face.clear();
            const int nv = (int)(pos.size() / 3), nt = (int)(uv.size() / 2), nn = (int)(nrm.size() / 3);
            while (true)
            {
                p += std::strspn(p, " \t");
                if (*p == '\0' || *p == '\r' || *p == '\n') break;
                ObjCorner c{-1, -1, -1};
                if (!ParseObjIndex(p, nv, &c.v)) { ok = false; break; }
                if (*p == '/')
                {
                    ++p;
                    if (*p != '/')
                    {
                        if (!ParseObjIndex(p, nt, &c.vt)) { ok = false; break; }
                    }
                    if (*p == '/')
                    {
                        ++p;
                        if (!ParseObjIndex(p, nn, &c.vn)) { ok = false; break; }
                    }
                }
                face.push_back(c);
                p += std::strcspn(p, " \t\r\n");
            }
            if (!ok || face.size() < 3) continue;
            std::vector<int> order = TriangulateFace(face, pos);
            for (size_t k = 0; k + 2 < order.size(); k += 3)
            {
                const ObjCorner tri[3] = {face[order[k]], face[order[k + 1]], face[order[k + 2]]};
                Vec3 gn(0, 0, 0);
                if (tri[0].vn < 0 || tri[1].vn < 0 || tri[2].vn < 0)
                {
                    Vec3 a(pos[tri[0].v * 3], pos[tri[0].v * 3 + 1], pos[tri[0].v * 3 + 2]);
                    Vec3 b(pos[tri[1].v * 3], pos[tri[1].v * 3 + 1], pos[tri[1].v * 3 + 2]);
                    Vec3 c(pos[tri[2].v * 3], pos[tri[2].v * 3 + 1], pos[tri[2].v * 3 + 2]);
                    gn = Vec3::Normalize(Vec3::Cross(b - a, c - a));
                }
                for (int j = 0; j < 3; ++j)
                {
                    const ObjCorner& cc = tri[j];
                    float tx = 0.f, ty = 0.f;
                    if (!uv.empty() && cc.vt >= 0)
                    {
                        tx = uv[cc.vt * 2 + 0];
                        ty = uv[cc.vt * 2 + 1];
                    }
                    Vec3 n = cc.vn >= 0 ? Vec3(nrm[cc.vn * 3], nrm[cc.vn * 3 + 1], nrm[cc.vn * 3 + 2]) : gn;
                    verticesUVX.push_back(Vec4(pos[cc.v * 3], pos[cc.v * 3 + 1], pos[cc.v * 3 + 2], tx));
                    normalsUVY.push_back(Vec4(n.x, n.y, n.z, ty));
                }
            }
        }
    }
    std::fclose(f);
    if (!ok || verticesUVX.empty())
    {
        Log("Unable to load geometry.\n");
        return false;
    }
    return true;
}

// ============================================================== HDR
namespace
{
    float Luminance(float r, float g, float b) { return r * 0.3f + g * 0.6f + b * 0.1f; }

    int LowerBound(const float* a, int lo, int hi, float value)
    {
        while (lo < hi)
        {
            int mid = lo + (hi - lo) / 2;
            if (a[mid] < value) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    }

    // Reads one RGBE scanline: new-style run-length encoding when the line starts with
    // (2, 2, hi, lo), otherwise flat pixels with the old (1,1,1,count) repeat marker.
    bool ReadScanline(FILE* f, unsigned char* line, int w)
    {
        auto read_flat = [&](unsigned char* dst, int len, int shift_start) {
            int shift = shift_start;
            while (len > 0)
            {
                int r = std::fgetc(f), g = std::fgetc(f), b = std::fgetc(f), e = std::fgetc(f);
                if (e == EOF) return false;
                if (r == 1 && g == 1 && b == 1)
                {
                    if (dst == line) return false;   // repeat marker with nothing to repeat
                    for (int i = e << shift; i > 0 && len > 0; --i)
                    {
                        std::memcpy(dst, dst - 4, 4);
                        dst += 4;
                        --len;
                    }
                    shift += 8;
                }
                else
                {
                    dst[0] = (unsigned char)r; dst[1] = (unsigned char)g; dst[2] = (unsigned char)b; dst[3] = (unsigned char)e;
                    dst += 4;
                    --len;
                    shift = 0;
                }
            }
            return true;
        };
        if (w < 8 || w > 0x7fff) return read_flat(line, w, 0);
        int c0 = std::fgetc(f);
        if (c0 == EOF) return false;
        if (c0 != 2)
        {
            std::ungetc(c0, f);
            return read_flat(line, w, 0);
        }
        int c1 = std::fgetc(f), c2 = std::fgetc(f), c3 = std::fgetc(f);
        if (c3 == EOF) return false;
        if (c1 != 2 || (c2 & 128))
        {
            line[0] = 2; line[1] = (unsigned char)c1; line[2] = (unsigned char)c2; line[3] = (unsigned char)c3;
            return read_flat(line + 4, w - 1, 0);
        }
        for (int ch = 0; ch < 4; ++ch)
        {
            for (int x = 0; x < w;)
            {
                int code = std::fgetc(f);
                if (code == EOF) return false;
                if (code > 128)
                {
                    code &= 127;
                    int val = std::fgetc(f);
                    if (val == EOF || x + code > w) return false;
                    while (code--) line[(x++) * 4 + ch] = (unsigned char)val;
                }
                else
                {
                    if (code == 0 || x + code > w) return false;
                    while (code--)
                    {
                        int val = std::fgetc(f);
                        if (val == EOF) return false;
                        line[(x++) * 4 + ch] = (unsigned char)val;
                    }
                }
            }
        }
        return true;
    }
}

void HDRLoader::buildDistributions(HDRData* res)
{
    const int width = res->width, height = res->height;
    std::vector<float> pdf2D((size_t)width * height), cdf2D((size_t)width * height);
    std::vector<float> pdf1D(height), cdf1D(height);
    delete[] res->marginalDistData;
    delete[] res->conditionalDistData;
    res->marginalDistData = new Vec2[height];
    res->conditionalDistData = new Vec2[(size_t)width * height];

    float colWeightSum = 0.0f;
    for (int j = 0; j < height; j++)
    {
        float rowWeightSum = 0.0f;
        for (int i = 0; i < width; ++i)
        {
            const float* c = res->cols + ((size_t)j * width + i) * 3;
            float weight = Luminance(c[0], c[1], c[2]);
            rowWeightSum += weight;
            pdf2D[(size_t)j * width + i] = weight;
            cdf2D[(size_t)j * width + i] = rowWeightSum;
        }
        for (int i = 0; i < width; i++)
        {
            pdf2D[(size_t)j * width + i] /= rowWeightSum;
            cdf2D[(size_t)j * width + i] /= rowWeightSum;
        }
        colWeightSum += rowWeightSum;
        pdf1D[j] = rowWeightSum;
        cdf1D[j] = colWeightSum;
    }
    for (int j = 0; j < height; j++)
    {
        cdf1D[j] /= colWeightSum;
        pdf1D[j] /= colWeightSum;
    }
    for (int i = 0; i < height; i++)
    {
        float target = (float)(i + 1) / height;
        int row = LowerBound(cdf1D.data(), 0, height, target);
        res->marginalDistData[i].x = row / (float)height;
        res->marginalDistData[i].y = pdf1D[i];
    }
    for (int j = 0; j < height; j++)
        for (int i = 0; i < width; i++)
        {
            float target = (float)(i + 1) / width;
            int col = LowerBound(cdf2D.data(), j * width, (j + 1) * width, target) - j * width;
            res->conditionalDistData[(size_t)j * width + i].x = col / (float)width;
            res->conditionalDistData[(size_t)j * width + i].y = pdf2D[(size_t)j * width + i];
        }
}

HDRData* HDRLoader::FromRGB(const float* rgb, int width, int height)
{
    if (!rgb || width <= 0 || height <= 0) return nullptr;
    HDRData* res = new HDRData;
    res->width = width;
    res->height = height;
    res->cols = new float[(size_t)width * height * 3];
    std::memcpy(res->cols, rgb, sizeof(float) * (size_t)width * height * 3);
    buildDistributions(res);
    return res;
}

HDRData* HDRLoader::load(const char* fileName)
{
    FILE* f = std::fopen(fileName, "rb");
    if (!f) return nullptr;
    char magic[10];
    if (std::fread(magic, 10, 1, f) != 1 || std::memcmp(magic, "#?RADIANCE", 10) != 0)
    {
        std::fclose(f);
        return nullptr;
    }
    // Header lines end with an empty line; the resolution line follows.
    int prev = 0, c = 0;
    while ((c = std::fgetc(f)) != EOF)
    {
        if (c == '\n' && prev == '\n') break;
        prev = c;
    }
    char reso[256] = {0};
    if (!std::fgets(reso, sizeof reso, f))
    {
        std::fclose(f);
        return nullptr;
    }
    int w = 0, h = 0;
    if (std::sscanf(reso, "-Y %d +X %d", &h, &w) != 2 || w <= 0 || h <= 0)
    {
        std::fclose(f);
        return nullptr;
    }
    HDRData* res = new HDRData;
    res->width = w;
    res->height = h;
    res->cols = new float[(size_t)w * h * 3]();
    std::vector<unsigned char> line((size_t)w * 4);
    for (int y = 0; y < h; ++y)
    {
        if (!ReadScanline(f, line.data(), w))
            break;
        float* dst = res->cols + (size_t)y * w * 3;
        for (int x = 0; x < w; ++x)
        {
            int e = (int)line[x * 4 + 3] - 128;
            float d = (float)std::pow(2.0, e);
            dst[x * 3 + 0] = (line[x * 4 + 0] / 256.0f) * d;
            dst[x * 3 + 1] = (line[x * 4 + 1] / 256.0f) * d;
            dst[x * 3 + 2] = (line[x * 4 + 2] / 256.0f) * d;
        }
    }
    std::fclose(f);
    buildDistributions(res);
    return res;
}

// ============================================================== .scene loader
// Line-oriented block parser with the keys and matching rules of Loader.cpp:45-385.
// Block headers are matched the same way (a `material <name>` line, or any line that
// contains "light", "Camera", "Renderer" or "mesh"), so the same files give the same
// scenes. Differences: a path without a directory resolves next to the working directory
// (the reference appends '/' to the file name), integer flags read into ints, not bools,
// and an unknown light type is kept as a quad with zero area.
bool LoadSceneFromFile(const std::string& filename, Scene* scene, RenderOptions& renderOptions)
{
    FILE* file = std::fopen(filename.c_str(), "r");
    if (!file)
    {
        Log("Couldn't open scene file %s for reading\n", filename.c_str());
        return false;
    }
    Log("Loading scene %s ...\n", filename.c_str());

    struct MaterialData
    {
        Material mat;
        int id;
    };
    std::map<std::string, MaterialData> materialMap;
    size_t sep = filename.find_last_of("/\\");
    std::string path = sep == std::string::npos ? std::string() : filename.substr(0, sep) + "/";

    const int kMaxLine = 2048;
    char line[kMaxLine];
    Material defaultMat;
    scene->AddMaterial(defaultMat);
    bool cameraAdded = false;
    bool overrideTileSize = false;
    int legacyAces = 2;

    while (std::fgets(line, kMaxLine, file))
    {
        if (line[0] == '#')
            continue;
        char name[kMaxLine] = {0};

        if (std::sscanf(line, " material %s", name) == 1)
        {
            Material material;
            char albedoTex[100] = "None", mrTex[100] = "None", normalTex[100] = "None", emissionTex[100] = "None";
            while (std::fgets(line, kMaxLine, file))
            {
                if (std::strchr(line, '}'))
                    break;
                std::sscanf(line, " name %s", name);
                std::sscanf(line, " color %f %f %f", &material.albedo.x, &material.albedo.y, &material.albedo.z);
                std::sscanf(line, " albedo %f %f %f", &material.albedo.x, &material.albedo.y, &material.albedo.z);
                std::sscanf(line, " emission %f %f %f", &material.emission.x, &material.emission.y, &material.emission.z);
                std::sscanf(line, " metallic %f", &material.metallic);
                std::sscanf(line, " roughness %f", &material.roughness);
                std::sscanf(line, " subsurface %f", &material.subsurface);
                std::sscanf(line, " specular %f", &material.specular);
                std::sscanf(line, " specularTint %f", &material.specularTint);
                std::sscanf(line, " anisotropic %f", &material.anisotropic);
                std::sscanf(line, " sheen %f", &material.sheen);
                std::sscanf(line, " sheenTint %f", &material.sheenTint);
                std::sscanf(line, " clearcoat %f", &material.clearcoat);
                std::sscanf(line, " clearcoatRoughness %f", &material.clearcoatRoughness);
                std::sscanf(line, " transmission %f", &material.transmission);
                std::sscanf(line, " ior %f", &material.ior);
                std::sscanf(line, " extinction %f %f %f", &material.extinction.x, &material.extinction.y, &material.extinction.z);
                std::sscanf(line, " albedoTexture %99s", albedoTex);
                std::sscanf(line, " metallicRoughnessTexture %99s", mrTex);
                std::sscanf(line, " normalTexture %99s", normalTex);
                std::sscanf(line, " emissionTexture %99s", emissionTex);
            }
            if (std::strcmp(albedoTex, "None") != 0) material.albedoTexID = (float)scene->AddTexture(path + albedoTex);
            if (std::strcmp(mrTex, "None") != 0) material.metallicRoughnessTexID = (float)scene->AddTexture(path + mrTex);
            if (std::strcmp(normalTex, "None") != 0) material.normalmapTexID = (float)scene->AddTexture(path + normalTex);
            if (std::strcmp(emissionTex, "None") != 0) material.emissionmapTexID = (float)scene->AddTexture(path + emissionTex);
            if (materialMap.find(name) == materialMap.end())
            {
                int id = scene->AddMaterial(material);
                materialMap[name] = MaterialData{material, id};
            }
        }

        if (std::strstr(line, "light"))
        {
            Light light;
            Vec3 v1, v2;
            char type[20] = "None";
            while (std::fgets(line, kMaxLine, file))
            {
                if (std::strchr(line, '}'))
                    break;
                std::sscanf(line, " position %f %f %f", &light.position.x, &light.position.y, &light.position.z);
                std::sscanf(line, " emission %f %f %f", &light.emission.x, &light.emission.y, &light.emission.z);
                std::sscanf(line, " radius %f", &light.radius);
                std::sscanf(line, " v1 %f %f %f", &v1.x, &v1.y, &v1.z);
                std::sscanf(line, " v2 %f %f %f", &v2.x, &v2.y, &v2.z);
                std::sscanf(line, " type %19s", type);
            }
            if (std::strcmp(type, "Quad") == 0)
            {
                light.type = (float)RectLight;
                light.u = v1 - light.position;
                light.v = v2 - light.position;
                light.area = Vec3::Length(Vec3::Cross(light.u, light.v));
            }
            else if (std::strcmp(type, "Sphere") == 0)
            {
                light.type = (float)SphereLight;
                light.area = 4.0f * LF_PI * light.radius * light.radius;
            }
            scene->AddLight(light);
        }

        if (std::strstr(line, "Camera"))
        {
            Vec3 position, lookAt;
            float fov = 35.f, aperture = 0, focalDist = 1;
            while (std::fgets(line, kMaxLine, file))
            {
                if (std::strchr(line, '}'))
                    break;
                std::sscanf(line, " position %f %f %f", &position.x, &position.y, &position.z);
                std::sscanf(line, " lookAt %f %f %f", &lookAt.x, &lookAt.y, &lookAt.z);
                std::sscanf(line, " aperture %f ", &aperture);
                std::sscanf(line, " focalDistance %f", &focalDist);
                std::sscanf(line, " focaldist %f", &focalDist);
                std::sscanf(line, " fov %f", &fov);
            }
            scene->AddCamera(position, lookAt, fov);
            scene->camera->aperture = aperture;
            scene->camera->focalDist = focalDist;
            cameraAdded = true;
        }

        if (std::strstr(line, "Renderer"))
        {
            char envMap[200] = "None";
            char enableRR[10] = "None";
            while (std::fgets(line, kMaxLine, file))
            {
                if (std::strchr(line, '}'))
                    break;
                int iv = 0;
                std::sscanf(line, " envMap %199s", envMap);
                std::sscanf(line, " hdriMap %199s", envMap);
                std::sscanf(line, " resolution %d %d", &renderOptions.resolution.x, &renderOptions.resolution.y);
                std::sscanf(line, " hdrMultiplier %f", &renderOptions.hdrMultiplier);
                std::sscanf(line, " hdriMultiplier %f", &renderOptions.hdrMultiplier);
                std::sscanf(line, " maxDepth %i", &renderOptions.maxDepth);
                if (std::sscanf(line, " tileWidth %i", &renderOptions.tileWidth) == 1) overrideTileSize = true;
                if (std::sscanf(line, " tileHeight %i", &renderOptions.tileHeight) == 1) overrideTileSize = true;
                std::sscanf(line, " enableRR %9s", enableRR);
                std::sscanf(line, " RRDepth %i", &renderOptions.RRDepth);
                std::sscanf(line, " tonemapIndex %i", &renderOptions.tonemapIndex);
                std::sscanf(line, " useAces %i", &legacyAces);
                if (legacyAces == 1) renderOptions.tonemapIndex = 1;
                if (legacyAces == 0) renderOptions.tonemapIndex = 0;
                if (std::sscanf(line, " useChromaticAberration %i", &iv) == 1) renderOptions.useCA = iv != 0;
                std::sscanf(line, " CADistance %f", &renderOptions.caDistance);
                if (std::sscanf(line, " useCAdistortion %i", &iv) == 1) renderOptions.useCADistortion = iv != 0;
                std::sscanf(line, " CAAngularity %f", &renderOptions.caP1);
                std::sscanf(line, " CADirectionality %f", &renderOptions.caP2);
                std::sscanf(line, " CACenter %f", &renderOptions.caP3);
                if (std::sscanf(line, " useVignette %i", &iv) == 1) renderOptions.useVignette = iv != 0;
                std::sscanf(line, " vignetteIntensity %f", &renderOptions.vignetteIntensity);
                std::sscanf(line, " vignettePower %f", &renderOptions.vignettePower);
            }
            if (std::strcmp(envMap, "None") != 0)
            {
                scene->AddHDR(path + envMap);
                renderOptions.useEnvMap = true;
            }
            if (std::strcmp(enableRR, "False") == 0) renderOptions.enableRR = false;
            else if (std::strcmp(enableRR, "True") == 0) renderOptions.enableRR = true;
        }

        if (std::strstr(line, "mesh"))
        {
            std::string meshFile;
            Mat4 xform;
            int material_id = 0;
            char meshName[200] = "None";
            while (std::fgets(line, kMaxLine, file))
            {
                if (std::strchr(line, '}'))
                    break;
                char fileTok[2048];
                char matName[100];
                std::sscanf(line, " name %199[^\t\n]", meshName);
                if (std::sscanf(line, " file %2047s", fileTok) == 1)
                    meshFile = path + fileTok;
                if (std::sscanf(line, " material %99s", matName) == 1)
                {
                    auto it = materialMap.find(matName);
                    if (it != materialMap.end()) material_id = it->second.id;
                    else Log("Could not find material %s\n", matName);
                }
                std::sscanf(line, " position %f %f %f", &xform[3][0], &xform[3][1], &xform[3][2]);
                std::sscanf(line, " scale %f %f %f", &xform[0][0], &xform[1][1], &xform[2][2]);
            }
            if (!meshFile.empty())
            {
                int mesh_id = scene->AddMesh(meshFile);
                if (mesh_id != -1)
                {
                    std::string instanceName;
                    if (std::strcmp(meshName, "None") != 0)
                        instanceName = meshName;
                    else
                        instanceName = meshFile.substr(meshFile.find_last_of("/\\") + 1);
                    scene->AddMeshInstance(MeshInstance(instanceName, mesh_id, xform, material_id));
                }
            }
        }
    }
    std::fclose(file);

    if (!overrideTileSize)
    {
        renderOptions.tileHeight = renderOptions.resolution.y;
        renderOptions.tileWidth = renderOptions.resolution.x;
    }
    if (!cameraAdded)
        scene->AddCamera(Vec3(0.0f, 0.0f, 10.0f), Vec3(0.0f, 0.0f, -10.0f), 35.0f);

    scene->CreateAccelerationStructures();
    Log("Scene loaded.\n");
    return scene->built;
}
}
