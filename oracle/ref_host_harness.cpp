// Test infrastructure: a C-ABI harness around the reference's own host code (compiled from
// the reference checkout by oracle/build_ref.py into oracle/_ref/). It builds scenes with
// the reference classes (LavaFrame::Scene, RadeonRays BVH, BvhTranslator, Loader,
// HDRLoader, Camera) so that the product's host layer can be compared byte for byte.
// Nothing in the product links or loads this file.
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#define STB_IMAGE_IMPLEMENTATION
#include "stb_image.h"
#define private public
#include "hdrloader.h"
#undef private
#include "GlobalState.h"
#include "Loader.h"
#include "Scene.h"

LavaFrameState GlobalState;

using namespace LavaFrame;

namespace
{
int QuietPrintf(const char*, ...) { return 0; }
}

struct RefScene
{
    Scene* scene = nullptr;
    RenderOptions options;
};

extern "C" {

RefScene* ref_scene_load(const char* path)
{
    Log = QuietPrintf;
    RefScene* r = new RefScene;
    r->scene = new Scene();
    if (!LoadSceneFromFile(path, r->scene, r->options))
    {
        delete r->scene;
        delete r;
        return nullptr;
    }
    return r;
}

// meshes: counts[i] vertices each (multiple of 3), concatenated xyzu / xyzv float4s.
RefScene* ref_scene_build(int nmeshes, const int* counts, const float* verts, const float* normals, int ninst,
                          const int* inst_mesh, const float* inst_xf, const int* inst_mat, int nmat, const float* mats)
{
    RefScene* r = new RefScene;
    r->scene = new Scene();
    size_t off = 0;
    for (int i = 0; i < nmeshes; ++i)
    {
        Mesh* m = new Mesh;
        m->name = "mesh" + std::to_string(i);
        for (int k = 0; k < counts[i]; ++k)
        {
            const float* v = verts + (off + k) * 4;
            const float* n = normals + (off + k) * 4;
            m->verticesUVX.push_back(Vec4(v[0], v[1], v[2], v[3]));
            m->normalsUVY.push_back(Vec4(n[0], n[1], n[2], n[3]));
        }
        off += counts[i];
        r->scene->meshes.push_back(m);
    }
    for (int i = 0; i < nmat; ++i)
    {
        Material m;
        std::memcpy(&m, mats + (size_t)i * 28, sizeof(Material));
        r->scene->AddMaterial(m);
    }
    for (int i = 0; i < ninst; ++i)
    {
        Mat4 xf;
        std::memcpy(xf.data, inst_xf + (size_t)i * 16, 64);
        r->scene->AddMeshInstance(MeshInstance("inst", inst_mesh[i], xf, inst_mat[i]));
    }
    r->scene->AddCamera(Vec3(0, 0, 10), Vec3(0, 0, -10), 35.0f);
    r->scene->CreateAccelerationStructures();
    return r;
}

// Scene::RebuildInstances (Scene.cpp:165-178) after new transforms and materials for the
// first n instances: a fresh TLAS, BvhTranslator::UpdateTLAS over the TLAS part of the node
// array, transforms copied - the host half of an instance move.
void ref_scene_move_instances(RefScene* r, int n, const float* xf, const int* mat)
{
    for (int i = 0; i < n && i < (int)r->scene->meshInstances.size(); ++i)
    {
        std::memcpy(r->scene->meshInstances[i].transform.data, xf + (size_t)i * 16, 64);
        r->scene->meshInstances[i].materialID = mat[i];
    }
    r->scene->RebuildInstances();
}

void ref_scene_free(RefScene* r)
{
    if (!r) return;
    delete r->scene;
    delete r;
}

// which: 0 nodes (9 floats), 1 vertIndices (3 ints), 2 verticesUVX, 3 normalsUVY,
// 4 transforms (16 floats), 5 materials (28 floats), 6 lights (15 floats)
const void* ref_scene_array(RefScene* r, int which, long long* count)
{
    Scene* s = r->scene;
    switch (which)
    {
    case 0: *count = (long long)s->bvhTranslator.nodes.size(); return s->bvhTranslator.nodes.data();
    case 1: *count = (long long)s->vertIndices.size(); return s->vertIndices.data();
    case 2: *count = (long long)s->verticesUVX.size(); return s->verticesUVX.data();
    case 3: *count = (long long)s->normalsUVY.size(); return s->normalsUVY.data();
    case 4: *count = (long long)s->transforms.size(); return s->transforms.data();
    case 5: *count = (long long)s->materials.size(); return s->materials.data();
    case 6: *count = (long long)s->lights.size(); return s->lights.data();
    }
    *count = 0;
    return nullptr;
}

int ref_scene_top_level_index(RefScene* r) { return r->scene->bvhTranslator.topLevelIndex; }

// camera basis after loading: position, right, up, forward (12 floats), fov, focalDist,
// aperture; render options: width, height, maxDepth, enableRR, RRDepth
void ref_scene_camera(RefScene* r, float* out15, int* opts5)
{
    Camera* c = r->scene->camera;
    const Vec3* v[4] = {&c->position, &c->right, &c->up, &c->forward};
    for (int k = 0; k < 4; ++k)
    {
        out15[k * 3 + 0] = v[k]->x;
        out15[k * 3 + 1] = v[k]->y;
        out15[k * 3 + 2] = v[k]->z;
    }
    out15[12] = c->fov;
    out15[13] = c->focalDist;
    out15[14] = c->aperture;
    opts5[0] = r->options.resolution.x;
    opts5[1] = r->options.resolution.y;
    opts5[2] = r->options.maxDepth;
    opts5[3] = r->options.enableRR ? 1 : 0;
    opts5[4] = r->options.RRDepth;
}

void ref_camera(const float* eye, const float* at, float fov, float* out15)
{
    Camera c(Vec3(eye[0], eye[1], eye[2]), Vec3(at[0], at[1], at[2]), fov);
    const Vec3* v[4] = {&c.position, &c.right, &c.up, &c.forward};
    for (int k = 0; k < 4; ++k)
    {
        out15[k * 3 + 0] = v[k]->x;
        out15[k * 3 + 1] = v[k]->y;
        out15[k * 3 + 2] = v[k]->z;
    }
    out15[12] = c.fov;
    out15[13] = c.focalDist;
    out15[14] = c.aperture;
}

// Reference sampling tables for an RGB32F image: marginal (h x 2), conditional (w*h x 2).
void ref_hdr_tables(const float* rgb, int w, int h, float* marginal, float* conditional)
{
    HDRData d;
    d.width = w;
    d.height = h;
    d.cols = new float[(size_t)w * h * 3];
    std::memcpy(d.cols, rgb, sizeof(float) * (size_t)w * h * 3);
    HDRLoader::buildDistributions(&d);
    std::memcpy(marginal, d.marginalDistData, sizeof(float) * 2 * h);
    std::memcpy(conditional, d.conditionalDistData, sizeof(float) * 2 * (size_t)w * h);
    delete[] d.cols;
    d.cols = nullptr;
    delete[] d.marginalDistData;
    d.marginalDistData = nullptr;
    delete[] d.conditionalDistData;
    d.conditionalDistData = nullptr;
}

// Mesh::LoadFromFile: returns the vertex count (0 on failure); arrays must hold `cap` float4s.
int ref_load_obj(const char* path, float* verts, float* normals, int cap)
{
    Mesh m;
    if (!m.LoadFromFile(path)) return 0;
    int n = (int)m.verticesUVX.size();
    if (n > cap) return -n;
    std::memcpy(verts, m.verticesUVX.data(), sizeof(Vec4) * n);
    std::memcpy(normals, m.normalsUVY.data(), sizeof(Vec4) * n);
    return n;
}
}
