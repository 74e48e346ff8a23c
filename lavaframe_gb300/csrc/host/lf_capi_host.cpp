// C ABI over the host scene layer (LavaFrame::Scene and LoadSceneFromFile) and the
// procedural workload generators. Generators use only IEEE basic operations and the
// contract functions (lf_contract.h) so they produce the same bits on every host.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../../include/lavaframe_gb300.h"
#include "../lf_vec.h"
#include "lf_scene.h"

using namespace LavaFrame;

struct lf_hscene
{
    Scene scene;
    RenderOptions options;
    std::string err;
};

namespace
{
lf_status herr(lf_hscene* s, lf_status st, const std::string& m)
{
    if (s) s->err = m;
    return st;
}

// ------------------------------------------------------------------ deterministic RNG
struct SplitMix
{
    uint64_t x;
    explicit SplitMix(uint64_t seed) : x(seed) {}
    uint64_t next()
    {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // uniform in [0, 1) with 24 random bits
    float uniform() { return (float)(next() >> 40) * (1.0f / 16777216.0f); }
    // standard normal, Box-Muller on contract functions
    float normal()
    {
        float u1 = ((float)(next() >> 40) + 1.0f) * (1.0f / 16777216.0f);   // (0, 1]
        float u2 = uniform();
        float r = sqrtf(-2.0f * lfc::log_c(u1));
        float s, c;
        lfc::sincos_c(6.28318548f * u2, &s, &c);
        return r * c;
    }
};

Vec4 V4(lfc::v3 a, float w) { return Vec4(a.x, a.y, a.z, w); }

void push_tri(std::vector<Vec4>& v, std::vector<Vec4>& n, lfc::v3 a, lfc::v3 b, lfc::v3 c)
{
    lfc::v3 fn = lfc::normalize(lfc::cross(b - a, c - a));
    v.push_back(V4(a, 0.f)); v.push_back(V4(b, 0.f)); v.push_back(V4(c, 0.f));
    n.push_back(V4(fn, 0.f)); n.push_back(V4(fn, 0.f)); n.push_back(V4(fn, 0.f));
}

// quad a-b-c-d (counter-clockwise seen from the side the normal points to)
void push_quad(std::vector<Vec4>& v, std::vector<Vec4>& n, lfc::v3 a, lfc::v3 b, lfc::v3 c, lfc::v3 d)
{
    push_tri(v, n, a, b, c);
    push_tri(v, n, a, c, d);
}

// Quad a-b-c-d split into k x k quads (2 triangles each); k = 1 is push_quad itself. Grid
// points interpolate the corners with weights (1 - t, t), which reproduce the corners exactly.
void push_quad_grid(std::vector<Vec4>& v, std::vector<Vec4>& n, lfc::v3 a, lfc::v3 b, lfc::v3 c, lfc::v3 d, int k)
{
    using lfc::v3;
    if (k <= 1)
    {
        push_quad(v, n, a, b, c, d);
        return;
    }
    auto lerp = [](v3 x, v3 y, float t) { return x * (1.0f - t) + y * t; };
    auto at = [&](int i, int j) {
        const float u = (float)i / (float)k, w = (float)j / (float)k;
        return lerp(lerp(a, b, u), lerp(d, c, u), w);
    };
    for (int j = 0; j < k; ++j)
        for (int i = 0; i < k; ++i) push_quad(v, n, at(i, j), at(i + 1, j), at(i + 1, j + 1), at(i, j + 1));
}

// Axis-aligned box [lo, hi] with outward normals (12 triangles, or 12 k^2 with k x k faces).
void push_box(std::vector<Vec4>& v, std::vector<Vec4>& n, lfc::v3 lo, lfc::v3 hi, int k = 1)
{
    using lfc::v3;
    v3 p000(lo.x, lo.y, lo.z), p100(hi.x, lo.y, lo.z), p010(lo.x, hi.y, lo.z), p110(hi.x, hi.y, lo.z);
    v3 p001(lo.x, lo.y, hi.z), p101(hi.x, lo.y, hi.z), p011(lo.x, hi.y, hi.z), p111(hi.x, hi.y, hi.z);
    push_quad_grid(v, n, p000, p010, p110, p100, k);   // -z
    push_quad_grid(v, n, p001, p101, p111, p011, k);   // +z
    push_quad_grid(v, n, p000, p001, p011, p010, k);   // -x
    push_quad_grid(v, n, p100, p110, p111, p101, k);   // +x
    push_quad_grid(v, n, p000, p100, p101, p001, k);   // -y
    push_quad_grid(v, n, p010, p011, p111, p110, k);   // +y
}

Mat4 rigid_y(float angleDeg, lfc::v3 t)
{
    float s, c;
    lfc::sincos_c(angleDeg * (3.14159265f / 180.0f), &s, &c);
    Mat4 m;
    m[0][0] = c;  m[0][1] = 0; m[0][2] = -s; m[0][3] = 0;
    m[1][0] = 0;  m[1][1] = 1; m[1][2] = 0;  m[1][3] = 0;
    m[2][0] = s;  m[2][1] = 0; m[2][2] = c;  m[2][3] = 0;
    m[3][0] = t.x; m[3][1] = t.y; m[3][2] = t.z; m[3][3] = 1;
    return m;
}

Material diffuse(float r, float g, float b)
{
    Material m;
    m.albedo = Vec3(r, g, b);
    m.roughness = 1.0f;
    m.metallic = 0.0f;
    return m;
}

// ------------------------------------------------------------------ value noise
uint32_t hash3(int x, int y, int z, uint32_t seed)
{
    uint32_t h = seed ^ 0x27d4eb2du;
    h ^= (uint32_t)x * 0x8da6b343u;
    h = (h ^ (h >> 13)) * 0x85ebca6bu;
    h ^= (uint32_t)y * 0xd8163841u;
    h = (h ^ (h >> 13)) * 0xc2b2ae35u;
    h ^= (uint32_t)z * 0xcb1ab31fu;
    h = (h ^ (h >> 16)) * 0x85ebca6bu;
    return h ^ (h >> 15);
}

float lattice(int x, int y, int z, uint32_t seed) { return (float)(hash3(x, y, z, seed) >> 8) * (2.0f / 16777216.0f) - 1.0f; }

float smooth(float t) { return t * t * (3.0f - 2.0f * t); }

float value_noise(lfc::v3 p, uint32_t seed)
{
    float fx = floorf(p.x), fy = floorf(p.y), fz = floorf(p.z);
    int ix = (int)fx, iy = (int)fy, iz = (int)fz;
    float tx = smooth(p.x - fx), ty = smooth(p.y - fy), tz = smooth(p.z - fz);
    float c[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int d = 0; d < 2; ++d) c[a][b][d] = lattice(ix + a, iy + b, iz + d, seed);
    float x00 = c[0][0][0] + (c[1][0][0] - c[0][0][0]) * tx;
    float x10 = c[0][1][0] + (c[1][1][0] - c[0][1][0]) * tx;
    float x01 = c[0][0][1] + (c[1][0][1] - c[0][0][1]) * tx;
    float x11 = c[0][1][1] + (c[1][1][1] - c[0][1][1]) * tx;
    float y0 = x00 + (x10 - x00) * ty;
    float y1 = x01 + (x11 - x01) * ty;
    return y0 + (y1 - y0) * tz;
}

float fbm4(lfc::v3 p, uint32_t seed)
{
    float sum = 0.f, amp = 0.5f;
    for (int o = 0; o < 4; ++o)
    {
        sum = sum + amp * value_noise(p, seed + (uint32_t)o * 1013u);
        p = p * 2.0f;
        amp = amp * 0.5f;
    }
    return sum;
}

// Indexed unit icosphere subdivided `level` times.
void icosphere(int level, std::vector<lfc::v3>& pts, std::vector<int>& tri)
{
    using lfc::v3;
    const float t = 1.61803398875f;
    v3 base[12] = {v3(-1, t, 0), v3(1, t, 0), v3(-1, -t, 0), v3(1, -t, 0), v3(0, -1, t), v3(0, 1, t),
                   v3(0, -1, -t), v3(0, 1, -t), v3(t, 0, -1), v3(t, 0, 1), v3(-t, 0, -1), v3(-t, 0, 1)};
    const int faces[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                              {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                              {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    pts.clear();
    for (auto& b : base) pts.push_back(lfc::normalize(b));
    tri.clear();
    for (auto& f : faces) tri.insert(tri.end(), {f[0], f[1], f[2]});
    for (int l = 0; l < level; ++l)
    {
        std::unordered_map<uint64_t, int> mid;
        auto midpoint = [&](int a, int b) {
            uint64_t key = a < b ? ((uint64_t)a << 32 | (uint32_t)b) : ((uint64_t)b << 32 | (uint32_t)a);
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            v3 m = lfc::normalize((pts[a] + pts[b]) * 0.5f);
            pts.push_back(m);
            int id = (int)pts.size() - 1;
            mid.emplace(key, id);
            return id;
        };
        std::vector<int> nt;
        nt.reserve(tri.size() * 4);
        for (size_t i = 0; i < tri.size(); i += 3)
        {
            int a = tri[i], b = tri[i + 1], c = tri[i + 2];
            int ab = midpoint(a, b), bc = midpoint(b, c), ca = midpoint(c, a);
            nt.insert(nt.end(), {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca});
        }
        tri.swap(nt);
    }
}

// Rotation from a uniform random unit quaternion (Shoemake).
Mat4 random_rigid(SplitMix& r, float half)
{
    float u1 = r.uniform(), u2 = r.uniform(), u3 = r.uniform();
    float a = sqrtf(1.0f - u1), b = sqrtf(u1);
    float s2, c2, s3, c3;
    lfc::sincos_c(6.28318548f * u2, &s2, &c2);
    lfc::sincos_c(6.28318548f * u3, &s3, &c3);
    float qx = a * s2, qy = a * c2, qz = b * s3, qw = b * c3;
    Mat4 m;
    // column-major rotation: data[col][row]
    m[0][0] = 1 - 2 * (qy * qy + qz * qz); m[0][1] = 2 * (qx * qy + qz * qw);     m[0][2] = 2 * (qx * qz - qy * qw);
    m[1][0] = 2 * (qx * qy - qz * qw);     m[1][1] = 1 - 2 * (qx * qx + qz * qz); m[1][2] = 2 * (qy * qz + qx * qw);
    m[2][0] = 2 * (qx * qz + qy * qw);     m[2][1] = 2 * (qy * qz - qx * qw);     m[2][2] = 1 - 2 * (qx * qx + qy * qy);
    m[0][3] = m[1][3] = m[2][3] = 0.f;
    m[3][0] = (r.uniform() * 2.0f - 1.0f) * half;
    m[3][1] = (r.uniform() * 2.0f - 1.0f) * half;
    m[3][2] = (r.uniform() * 2.0f - 1.0f) * half;
    m[3][3] = 1.f;
    return m;
}
}

extern "C" {

lf_status lf_hscene_create(lf_hscene** out)
{
    if (!out) return LF_ERR_INVALID;
    *out = new lf_hscene;
    return LF_OK;
}

void lf_hscene_destroy(lf_hscene* s) { delete s; }

const char* lf_hscene_last_error(const lf_hscene* s) { return s ? s->err.c_str() : "null scene"; }

lf_status lf_hscene_load_file(lf_hscene* s, const char* path)
{
    if (!s || !path) return LF_ERR_INVALID;
    bool ok = LoadSceneFromFile(path, &s->scene, s->options);
    s->scene.renderOptions = s->options;
    if (!ok) return herr(s, LF_ERR_IO, s->scene.LastError().empty() ? std::string("cannot load ") + path : s->scene.LastError());
    return LF_OK;
}

int32_t lf_hscene_add_mesh(lf_hscene* s, const float* v, const float* n, int32_t nv)
{
    if (!s || !v || !n) return -1;
    int id = s->scene.AddMeshData("mesh" + std::to_string(s->scene.meshes.size()), reinterpret_cast<const Vec4*>(v),
                                  reinterpret_cast<const Vec4*>(n), nv);
    if (id < 0) s->err = s->scene.LastError();
    return id;
}

int32_t lf_hscene_add_mesh_file(lf_hscene* s, const char* path)
{
    if (!s || !path) return -1;
    int id = s->scene.AddMesh(path);
    if (id < 0) s->err = s->scene.LastError();
    return id;
}

int32_t lf_hscene_add_material(lf_hscene* s, const float* m28)
{
    if (!s || !m28) return -1;
    static_assert(std::is_trivially_copyable<Material>::value && sizeof(Material) == 28 * sizeof(float),
                  "Material is the 112-byte float record");
    Material m;
    std::memcpy(static_cast<void*>(&m), m28, sizeof(Material));
    return s->scene.AddMaterial(m);
}

int32_t lf_hscene_add_instance(lf_hscene* s, int32_t mesh, const float* xf, int32_t mat)
{
    if (!s || !xf) return -1;
    Mat4 m;
    std::memcpy(m.data, xf, sizeof(float) * 16);
    return s->scene.AddMeshInstance(MeshInstance("instance" + std::to_string(s->scene.meshInstances.size()), mesh, m, mat));
}

int32_t lf_hscene_add_light(lf_hscene* s, const float* l15)
{
    if (!s || !l15) return -1;
    static_assert(std::is_trivially_copyable<Light>::value && sizeof(Light) == 15 * sizeof(float),
                  "Light is the 60-byte float record");
    Light l;
    std::memcpy(static_cast<void*>(&l), l15, sizeof(Light));
    return s->scene.AddLight(l);
}

lf_status lf_hscene_set_camera(lf_hscene* s, const float eye[3], const float at[3], float fov, float aperture, float focal)
{
    if (!s || !eye || !at) return LF_ERR_INVALID;
    s->scene.AddCamera(Vec3(eye[0], eye[1], eye[2]), Vec3(at[0], at[1], at[2]), fov);
    s->scene.camera->aperture = aperture;
    s->scene.camera->focalDist = focal;
    return LF_OK;
}

lf_status lf_hscene_add_hdr_file(lf_hscene* s, const char* path)
{
    if (!s || !path) return LF_ERR_INVALID;
    s->scene.AddHDR(path);
    if (!s->scene.hdrData) return herr(s, LF_ERR_IO, std::string("cannot load HDR ") + path);
    s->options.useEnvMap = true;
    return LF_OK;
}

lf_status lf_hscene_add_hdr(lf_hscene* s, const float* rgb, int32_t w, int32_t h)
{
    if (!s || !rgb || w <= 0 || h <= 0) return LF_ERR_INVALID;
    if (!s->scene.AddHDRData(rgb, w, h)) return herr(s, LF_ERR_INVALID, s->scene.LastError());
    s->options.useEnvMap = true;
    return LF_OK;
}

lf_status lf_hscene_build(lf_hscene* s, int32_t threads)
{
    if (!s) return LF_ERR_INVALID;
    SetBuildThreads(threads);
    if (!s->scene.camera) s->scene.AddCamera(Vec3(0.0f, 0.0f, 10.0f), Vec3(0.0f, 0.0f, -10.0f), 35.0f);
    s->scene.renderOptions = s->options;
    s->scene.CreateAccelerationStructures();
    if (!s->scene.built) return herr(s, LF_ERR_INVALID, s->scene.LastError());
    return LF_OK;
}

lf_status lf_hscene_set_instance(lf_hscene* s, int32_t i, const float* xf, int32_t mat)
{
    if (!s || !xf || i < 0 || i >= (int)s->scene.meshInstances.size()) return LF_ERR_INVALID;
    if (mat < 0 || mat >= (int)s->scene.materials.size()) return LF_ERR_INVALID;
    std::memcpy(s->scene.meshInstances[i].transform.data, xf, sizeof(float) * 16);
    s->scene.meshInstances[i].materialID = mat;
    return LF_OK;
}

lf_status lf_hscene_rebuild_instances(lf_hscene* s)
{
    if (!s || !s->scene.built) return LF_ERR_STATE;
    s->scene.RebuildInstances();
    return LF_OK;
}

lf_status lf_hscene_view(const lf_hscene* s, lf_scene_view* out)
{
    if (!s || !out) return LF_ERR_INVALID;
    if (!s->scene.built) return LF_ERR_STATE;
    const Scene& sc = s->scene;
    std::memset(out, 0, sizeof *out);
    out->nodes = reinterpret_cast<const float*>(sc.bvhTranslator.nodes.data());
    out->num_nodes = (int32_t)sc.bvhTranslator.nodes.size();
    out->top_level_index = sc.bvhTranslator.topLevelIndex;
    out->vert_indices = reinterpret_cast<const int32_t*>(sc.vertIndices.data());
    out->num_tris = (int32_t)sc.vertIndices.size();
    out->vertices_uvx = reinterpret_cast<const float*>(sc.verticesUVX.data());
    out->normals_uvy = reinterpret_cast<const float*>(sc.normalsUVY.data());
    out->num_vertices = (int32_t)sc.verticesUVX.size();
    out->materials = reinterpret_cast<const float*>(sc.materials.data());
    out->num_materials = (int32_t)sc.materials.size();
    out->transforms = reinterpret_cast<const float*>(sc.transforms.data());
    out->num_instances = (int32_t)sc.transforms.size();
    out->lights = sc.lights.empty() ? nullptr : reinterpret_cast<const float*>(sc.lights.data());
    out->num_lights = (int32_t)sc.lights.size();
    if (sc.hdrData)
    {
        out->env_rgb = sc.hdrData->cols;
        out->env_marginal = reinterpret_cast<const float*>(sc.hdrData->marginalDistData);
        out->env_conditional = reinterpret_cast<const float*>(sc.hdrData->conditionalDistData);
        out->env_width = sc.hdrData->width;
        out->env_height = sc.hdrData->height;
    }
    if (!sc.textures.empty())
    {
        out->textures = sc.textureMapsArray.data();
        out->tex_width = sc.texWidth;
        out->tex_height = sc.texHeight;
        out->num_textures = (int32_t)sc.textures.size();
    }
    return LF_OK;
}

lf_status lf_hscene_counts(const lf_hscene* s, int32_t counts[4])
{
    if (!s || !counts) return LF_ERR_INVALID;
    counts[0] = (int32_t)s->scene.meshes.size();
    counts[1] = (int32_t)s->scene.meshInstances.size();
    counts[2] = (int32_t)s->scene.materials.size();
    counts[3] = (int32_t)s->scene.lights.size();
    return LF_OK;
}

lf_status lf_hscene_layout(const lf_hscene* s, int32_t* mesh_vertex_counts, int32_t* instance_mesh, int32_t* instance_material)
{
    if (!s) return LF_ERR_INVALID;
    for (size_t i = 0; mesh_vertex_counts && i < s->scene.meshes.size(); ++i)
        mesh_vertex_counts[i] = (int32_t)s->scene.meshes[i]->verticesUVX.size();
    for (size_t i = 0; i < s->scene.meshInstances.size(); ++i)
    {
        if (instance_mesh) instance_mesh[i] = s->scene.meshInstances[i].meshID;
        if (instance_material) instance_material[i] = s->scene.meshInstances[i].materialID;
    }
    return LF_OK;
}

lf_status lf_hscene_render_params(const lf_hscene* s, lf_render_params* p)
{
    if (!s || !p) return LF_ERR_INVALID;
    const RenderOptions& o = s->options;
    const Camera* cam = s->scene.camera;
    if (!cam) return LF_ERR_STATE;
    std::memset(p, 0, sizeof *p);
    p->width = o.resolution.x;
    p->height = o.resolution.y;
    p->max_depth = o.maxDepth;
    p->enable_rr = o.enableRR ? 1 : 0;
    p->rr_depth = o.RRDepth;
    p->use_env_map = (o.useEnvMap && s->scene.hdrData) ? 1 : 0;
    p->use_constant_bg = o.useConstantBg ? 1 : 0;
    p->bg_color[0] = o.bgColor.x; p->bg_color[1] = o.bgColor.y; p->bg_color[2] = o.bgColor.z;
    p->hdr_multiplier = o.hdrMultiplier;
    const Vec3* vs[4] = {&cam->position, &cam->right, &cam->up, &cam->forward};
    float* dst[4] = {p->cam_position, p->cam_right, p->cam_up, p->cam_forward};
    for (int k = 0; k < 4; ++k)
    {
        dst[k][0] = vs[k]->x; dst[k][1] = vs[k]->y; dst[k][2] = vs[k]->z;
    }
    p->cam_fov = cam->fov;
    p->cam_focal_dist = cam->focalDist;
    p->cam_aperture = cam->aperture;
    p->seed = 0;
    p->frame_base = 1;
    p->tile_width = 0;
    p->tile_height = 0;
    return LF_OK;
}

// Procedural Cornell box: 1 m box open at z = 0, tall box 0.3x0.6x0.3 at 15 degrees,
// short box 0.3x0.3x0.3 at -18 degrees, 0.25 m quad light 1 mm below the ceiling with
// radiance (17, 12, 4), diffuse Disney materials, pinhole 45 degrees, depth 4, RR on.
// subdiv > 1 splits every wall and box face into subdiv x subdiv quads (34 subdiv^2
// triangles; the same surfaces), so the scene can be scaled for the serving mix.
lf_status lf_gen_cornell_tess(lf_hscene* s, int32_t width, int32_t height, int32_t subdiv)
{
    using lfc::v3;
    if (!s || width <= 0 || height <= 0 || subdiv < 1 || subdiv > 4096) return LF_ERR_INVALID;
    Scene& sc = s->scene;
    if (sc.materials.empty()) sc.AddMaterial(Material());   // default material 0, as the loader
    int white = sc.AddMaterial(diffuse(0.73f, 0.73f, 0.73f));
    int red = sc.AddMaterial(diffuse(0.63f, 0.065f, 0.05f));
    int green = sc.AddMaterial(diffuse(0.14f, 0.45f, 0.09f));
    struct Wall
    {
        v3 a, b, c, d;
        int mat;
    };
    // normals face into the box
    Wall walls[5] = {
        {v3(0, 0, 0), v3(0, 0, 1), v3(1, 0, 1), v3(1, 0, 0), white},   // floor, +y
        {v3(0, 1, 0), v3(1, 1, 0), v3(1, 1, 1), v3(0, 1, 1), white},   // ceiling, -y
        {v3(0, 0, 1), v3(0, 1, 1), v3(1, 1, 1), v3(1, 0, 1), white},   // back, -z
        {v3(0, 0, 0), v3(0, 1, 0), v3(0, 1, 1), v3(0, 0, 1), red},     // left x=0, +x
        {v3(1, 0, 0), v3(1, 0, 1), v3(1, 1, 1), v3(1, 1, 0), green},   // right x=1, -x
    };
    for (const Wall& w : walls)
    {
        std::vector<Vec4> v, n;
        push_quad_grid(v, n, w.a, w.b, w.c, w.d, subdiv);
        int mid = sc.AddMeshData("wall", v.data(), n.data(), (int)v.size());
        sc.AddMeshInstance(MeshInstance("wall", mid, Mat4(), w.mat));
    }
    {
        std::vector<Vec4> v, n;
        push_box(v, n, v3(-0.15f, -0.3f, -0.15f), v3(0.15f, 0.3f, 0.15f), subdiv);
        int mid = sc.AddMeshData("tallbox", v.data(), n.data(), (int)v.size());
        sc.AddMeshInstance(MeshInstance("tallbox", mid, rigid_y(15.0f, v3(0.66f, 0.3f, 0.66f)), white));
    }
    {
        std::vector<Vec4> v, n;
        push_box(v, n, v3(-0.15f, -0.15f, -0.15f), v3(0.15f, 0.15f, 0.15f), subdiv);
        int mid = sc.AddMeshData("shortbox", v.data(), n.data(), (int)v.size());
        sc.AddMeshInstance(MeshInstance("shortbox", mid, rigid_y(-18.0f, v3(0.33f, 0.15f, 0.35f)), white));
    }
    Light L;
    L.position = Vec3(0.375f, 0.999f, 0.375f);
    L.u = Vec3(0.25f, 0.f, 0.f);
    L.v = Vec3(0.f, 0.f, 0.25f);
    L.emission = Vec3(17.f, 12.f, 4.f);
    L.area = Vec3::Length(Vec3::Cross(L.u, L.v));
    L.type = (float)RectLight;
    L.radius = 0.f;
    sc.AddLight(L);
    sc.AddCamera(Vec3(0.5f, 0.5f, -1.3f), Vec3(0.5f, 0.5f, 0.5f), 45.0f);
    s->options.resolution = iVec2(width, height);
    s->options.maxDepth = 4;
    s->options.enableRR = true;
    s->options.RRDepth = 2;
    s->options.tileWidth = width;
    s->options.tileHeight = height;
    return LF_OK;
}

lf_status lf_gen_cornell(lf_hscene* s, int32_t width, int32_t height)
{
    return lf_gen_cornell_tess(s, width, height, 1);
}

// Intersection microbench: `instances` meshes of `tris` random triangles each; every mesh
// has one centroid uniform in [0,100]^3 and its triangle vertices are that centroid plus
// N(0, 0.5^2) offsets per coordinate; identity transforms.
lf_status lf_gen_soup(lf_hscene* s, int32_t instances, int32_t tris, uint64_t seed)
{
    using lfc::v3;
    if (!s || instances <= 0 || tris <= 0) return LF_ERR_INVALID;
    Scene& sc = s->scene;
    if (sc.materials.empty()) sc.AddMaterial(Material());
    int mat = sc.AddMaterial(diffuse(0.7f, 0.7f, 0.7f));
    SplitMix r(seed);
    std::vector<Vec4> v, n;
    sc.meshes.reserve(sc.meshes.size() + instances);
    sc.meshInstances.reserve(sc.meshInstances.size() + instances);
    for (int i = 0; i < instances; ++i)
    {
        v.clear();
        n.clear();
        const float cx = r.uniform() * 100.0f, cy = r.uniform() * 100.0f, cz = r.uniform() * 100.0f;
        const v3 c(cx, cy, cz);   // draws sequenced: argument order is unspecified in C++
        for (int t = 0; t < tris; ++t)
        {
            v3 p[3];
            for (int k = 0; k < 3; ++k)
            {
                float ox = r.normal() * 0.5f, oy = r.normal() * 0.5f, oz = r.normal() * 0.5f;
                p[k] = c + v3(ox, oy, oz);
            }
            push_tri(v, n, p[0], p[1], p[2]);
        }
        int mid = sc.AddMeshData("soup", v.data(), n.data(), (int)v.size());
        sc.AddMeshInstance(MeshInstance("soup", mid, Mat4(), mat));
    }
    sc.AddCamera(Vec3(50.f, 50.f, -80.f), Vec3(50.f, 50.f, 50.f), 45.0f);
    s->options.resolution = iVec2(1024, 1024);
    return LF_OK;
}

// Displaced icospheres: `instances` distinct meshes of a level-`level` icosphere
// (radius 5 m, radial displacement 0.1 x fBm of 4 octaves of seeded value noise),
// uniform random rotations, translations uniform in a 50 m cube, per-instance Disney
// materials, and a procedural sky + sun environment of env_w x env_h texels.
lf_status lf_gen_icospheres(lf_hscene* s, int32_t instances, int32_t level, uint64_t seed, int32_t env_w, int32_t env_h)
{
    using lfc::v3;
    if (!s || instances <= 0 || level < 0 || level > 8 || env_w <= 0 || env_h <= 0) return LF_ERR_INVALID;
    Scene& sc = s->scene;
    if (sc.materials.empty()) sc.AddMaterial(Material());
    SplitMix r(seed);
    std::vector<v3> pts;
    std::vector<int> tri;
    icosphere(level, pts, tri);
    const float R = 5.0f;
    std::vector<Vec4> v, n;
    std::vector<v3> disp(pts.size());
    for (int i = 0; i < instances; ++i)
    {
        uint32_t nseed = (uint32_t)(r.next() >> 32);
        const float ox = r.uniform() * 64.0f, oy = r.uniform() * 64.0f, oz = r.uniform() * 64.0f;
        const v3 off(ox, oy, oz);
        for (size_t k = 0; k < pts.size(); ++k)
        {
            float h = fbm4(pts[k] * 2.0f + off, nseed);
            disp[k] = pts[k] * (R * (1.0f + 0.1f * h));
        }
        v.clear();
        n.clear();
        v.reserve(tri.size());
        n.reserve(tri.size());
        for (size_t k = 0; k < tri.size(); k += 3) push_tri(v, n, disp[tri[k]], disp[tri[k + 1]], disp[tri[k + 2]]);
        int mid = sc.AddMeshData("icosphere", v.data(), n.data(), (int)v.size());
        Material m;
        const float ar = r.uniform(), ag = r.uniform(), ab = r.uniform();
        m.albedo = Vec3(ar, ag, ab);
        m.metallic = r.uniform();
        m.roughness = 0.05f + 0.95f * r.uniform();
        m.transmission = r.uniform() < 0.2f ? 1.0f : 0.0f;
        m.ior = 1.5f;
        int mat = sc.AddMaterial(m);
        sc.AddMeshInstance(MeshInstance("icosphere", mid, random_rigid(r, 25.0f), mat));
    }
    // sky gradient + 0.5 degree sun of radiance 1e4, in the shader's (u, v) mapping
    std::vector<float> rgb((size_t)env_w * env_h * 3);
    v3 sun = lfc::normalize(v3(0.3f, 0.6f, 0.4f));
    const float cosSun = lfc::cos_c(0.5f * 3.14159265f / 180.0f);
    for (int y = 0; y < env_h; ++y)
        for (int x = 0; x < env_w; ++x)
        {
            float u = ((float)x + 0.5f) / (float)env_w, vv = ((float)y + 0.5f) / (float)env_h;
            float st, ct, sp, cp;
            lfc::sincos_c(vv * 3.14159265f, &st, &ct);
            lfc::sincos_c(u * 6.28318548f, &sp, &cp);
            v3 d(-st * cp, ct, -st * sp);
            v3 col;
            if (d.y > 0.f)
                col = lfc::mix(v3(0.9f, 0.85f, 0.8f), v3(0.25f, 0.45f, 0.9f), d.y);
            else
                col = v3(0.2f, 0.18f, 0.16f);
            if (lfc::dot(d, sun) >= cosSun) col = v3(10000.f, 9500.f, 9000.f);
            float* o = &rgb[((size_t)y * env_w + x) * 3];
            o[0] = col.x; o[1] = col.y; o[2] = col.z;
        }
    sc.AddHDRData(rgb.data(), env_w, env_h);
    s->options.useEnvMap = true;
    sc.AddCamera(Vec3(0.f, 18.f, 62.f), Vec3(0.f, 0.f, 0.f), 45.0f);
    s->options.resolution = iVec2(1920, 1080);
    s->options.tileWidth = 1920;
    s->options.tileHeight = 1080;
    s->options.maxDepth = 8;
    s->options.enableRR = true;
    s->options.RRDepth = 2;
    return LF_OK;
}

// Occluded-light interior: a closed 10 x 4 x 10 m room filled with `boxes` random boxes,
// lit only through a 1 x 1 m doorway by a 2000-radiance quad light in the adjacent room.
lf_status lf_gen_room(lf_hscene* s, int32_t boxes, uint64_t seed)
{
    using lfc::v3;
    if (!s || boxes < 0) return LF_ERR_INVALID;
    Scene& sc = s->scene;
    if (sc.materials.empty()) sc.AddMaterial(Material());
    int white = sc.AddMaterial(diffuse(0.75f, 0.75f, 0.75f));
    int wood = sc.AddMaterial(diffuse(0.55f, 0.4f, 0.25f));
    std::vector<Vec4> v, n;
    // main room [0,10] x [0,4] x [0,10], normals inward
    push_quad(v, n, v3(0, 0, 0), v3(0, 0, 10), v3(10, 0, 10), v3(10, 0, 0));     // floor
    push_quad(v, n, v3(0, 4, 0), v3(10, 4, 0), v3(10, 4, 10), v3(0, 4, 10));     // ceiling
    push_quad(v, n, v3(0, 0, 0), v3(10, 0, 0), v3(10, 4, 0), v3(0, 4, 0));       // z = 0
    push_quad(v, n, v3(0, 0, 10), v3(0, 4, 10), v3(10, 4, 10), v3(10, 0, 10));   // z = 10
    push_quad(v, n, v3(0, 0, 0), v3(0, 4, 0), v3(0, 4, 10), v3(0, 0, 10));       // x = 0
    // x = 10 wall with a doorway z in [4.5, 5.5], y in [0, 1] (normal -x)
    auto wallx = [&](float z0, float z1, float y0, float y1) {
        push_quad(v, n, v3(10, y0, z0), v3(10, y0, z1), v3(10, y1, z1), v3(10, y1, z0));
    };
    wallx(0.f, 4.5f, 0.f, 4.f);
    wallx(5.5f, 10.f, 0.f, 4.f);
    wallx(4.5f, 5.5f, 1.f, 4.f);
    // adjacent room [10.2, 14] x [0, 4] x [0, 10] with its own doorway wall at x = 10.2
    push_quad(v, n, v3(10.2f, 0, 0), v3(10.2f, 0, 10), v3(14, 0, 10), v3(14, 0, 0));
    push_quad(v, n, v3(10.2f, 4, 0), v3(14, 4, 0), v3(14, 4, 10), v3(10.2f, 4, 10));
    push_quad(v, n, v3(10.2f, 0, 0), v3(14, 0, 0), v3(14, 4, 0), v3(10.2f, 4, 0));
    push_quad(v, n, v3(10.2f, 0, 10), v3(10.2f, 4, 10), v3(14, 4, 10), v3(14, 0, 10));
    push_quad(v, n, v3(14, 0, 0), v3(14, 0, 10), v3(14, 4, 10), v3(14, 4, 0));
    auto wallx2 = [&](float z0, float z1, float y0, float y1) {   // normal +x
        push_quad(v, n, v3(10.2f, y0, z0), v3(10.2f, y1, z0), v3(10.2f, y1, z1), v3(10.2f, y0, z1));
    };
    wallx2(0.f, 4.5f, 0.f, 4.f);
    wallx2(5.5f, 10.f, 0.f, 4.f);
    wallx2(4.5f, 5.5f, 1.f, 4.f);
    // door jambs between the two walls
    push_quad(v, n, v3(10, 0, 4.5f), v3(10, 1, 4.5f), v3(10.2f, 1, 4.5f), v3(10.2f, 0, 4.5f));
    push_quad(v, n, v3(10, 0, 5.5f), v3(10.2f, 0, 5.5f), v3(10.2f, 1, 5.5f), v3(10, 1, 5.5f));
    push_quad(v, n, v3(10, 1, 4.5f), v3(10, 1, 5.5f), v3(10.2f, 1, 5.5f), v3(10.2f, 1, 4.5f));
    int shell = sc.AddMeshData("room", v.data(), n.data(), (int)v.size());
    sc.AddMeshInstance(MeshInstance("room", shell, Mat4(), white));

    SplitMix r(seed);
    struct Box
    {
        v3 lo, hi;
    };
    std::vector<Box> all((size_t)boxes);
    for (int b = 0; b < boxes; ++b)
    {
        // small clutter (2-14 cm wide, up to 30 cm high), so that 200k triangles leave the
        // room navigable for light entering through the doorway
        float sx = 0.02f + 0.12f * r.uniform(), sy = 0.02f + 0.28f * r.uniform(), sz = 0.02f + 0.12f * r.uniform();
        float x = 0.3f + (9.4f - sx) * r.uniform(), z = 0.3f + (9.4f - sz) * r.uniform();
        if (x > 8.0f && z > 3.5f && z < 6.5f) x = x - 7.5f;   // keep the way to the doorway clear
        float y = r.uniform() < 0.9f ? 0.0f : 0.3f + 3.0f * r.uniform();
        all[(size_t)b] = {v3(x, y, z), v3(x + sx, y + sy, z + sz)};
    }
    // Meshes of at most 512 boxes. Beyond one mesh, boxes are grouped by floor position (Morton
    // order of a 64 x 64 grid over the room), so every furniture mesh covers a compact patch of
    // floor instead of the whole room.
    const int perMesh = 512;
    if (boxes > perMesh)
    {
        auto key = [](const Box& bx) {
            auto cell = [](float c) {
                int q = (int)(c * (64.0f / 10.0f));
                return (uint32_t)(q < 0 ? 0 : (q > 63 ? 63 : q));
            };
            auto spread = [](uint32_t x) {
                x = (x | (x << 4)) & 0x0F0Fu;
                x = (x | (x << 2)) & 0x3333u;
                x = (x | (x << 1)) & 0x5555u;
                return x;
            };
            return (spread(cell(bx.lo.x)) << 1) | spread(cell(bx.lo.z));
        };
        std::stable_sort(all.begin(), all.end(), [&](const Box& a, const Box& b) { return key(a) < key(b); });
    }
    for (int b0 = 0; b0 < boxes; b0 += perMesh)
    {
        v.clear();
        n.clear();
        int nb = boxes - b0 < perMesh ? boxes - b0 : perMesh;
        for (int b = 0; b < nb; ++b) push_box(v, n, all[(size_t)(b0 + b)].lo, all[(size_t)(b0 + b)].hi);
        int mid = sc.AddMeshData("furniture", v.data(), n.data(), (int)v.size());
        sc.AddMeshInstance(MeshInstance("furniture", mid, Mat4(), wood));
    }
    Light L;
    L.position = Vec3(12.0f, 3.99f, 4.0f);
    L.u = Vec3(1.0f, 0.f, 0.f);
    L.v = Vec3(0.f, 0.f, 2.0f);
    L.emission = Vec3(2000.f, 2000.f, 2000.f);
    L.area = Vec3::Length(Vec3::Cross(L.u, L.v));
    L.type = (float)RectLight;
    // the light must face down: cross(u, v) = (0, -2, 0)
    sc.AddLight(L);
    sc.AddCamera(Vec3(1.0f, 1.7f, 1.0f), Vec3(9.0f, 1.0f, 6.0f), 60.0f);
    s->options.resolution = iVec2(1280, 720);
    s->options.tileWidth = 1280;
    s->options.tileHeight = 720;
    s->options.maxDepth = 10;
    s->options.enableRR = true;
    s->options.RRDepth = 2;
    return LF_OK;
}

lf_status lf_gen_rays(const float lo[3], const float hi[3], int64_t nrays, uint64_t seed, float tmax, float* out)
{
    if (!lo || !hi || nrays < 0 || (nrays > 0 && !out)) return LF_ERR_INVALID;
    SplitMix r(seed);
    for (int64_t i = 0; i < nrays; ++i)
    {
        float* o = out + i * 8;
        for (int k = 0; k < 3; ++k) o[k] = lo[k] + (hi[k] - lo[k]) * r.uniform();
        o[3] = 0.f;
        lfc::v3 d;
        float len;
        do
        {
            const float dx = r.normal(), dy = r.normal(), dz = r.normal();
            d = lfc::v3(dx, dy, dz);
            len = lfc::dot(d, d);
        } while (len < 1e-12f);
        d = lfc::normalize(d);
        o[4] = d.x; o[5] = d.y; o[6] = d.z;
        o[7] = tmax;
    }
    return LF_OK;
}
}
