// Scene container, camera, acceleration-structure build and flatten.
#include "lf_scene.h"

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <thread>

namespace LavaFrame
{
namespace
{
    std::atomic<int> g_build_threads{0};

    // Runs fn(i) for i in [0, n) on a small pool; work is claimed in chunks.
    template <class Fn>
    void ParallelFor(int n, Fn fn, int chunk = 64)
    {
        int nt = GetBuildThreads();
        if (n <= chunk || nt <= 1)
        {
            for (int i = 0; i < n; ++i) fn(i);
            return;
        }
        std::atomic<int> next{0};
        auto worker = [&]() {
            for (;;)
            {
                int b = next.fetch_add(chunk);
                if (b >= n) break;
                int e = b + chunk < n ? b + chunk : n;
                for (int i = b; i < e; ++i) fn(i);
            }
        };
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
        worker();
        for (auto& th : pool) th.join();
    }
}

void SetBuildThreads(int n) { g_build_threads = n; }

int GetBuildThreads()
{
    int n = g_build_threads.load();
    if (n > 0) return n;
    unsigned hc = std::thread::hardware_concurrency();
    return hc ? (int)hc : 1;
}

// ---------------------------------------------------------------- Camera
// Same construction as Camera.cpp:101-117,157-169. The trigonometry runs in double
// precision (the reference calls the unsuffixed C functions on float arguments).
Camera::Camera(Vec3 eye, Vec3 lookat, float fov_deg)
{
    position = eye;
    pivot = lookat;
    worldUp = Vec3(0, 1, 0);

    Vec3 dir = Vec3::Normalize(pivot - position);
    pitch = Math::Degrees((float)::asin((double)dir.y));
    yaw = Math::Degrees((float)::atan2((double)dir.z, (double)dir.x));

    radius = Vec3::Distance(eye, lookat);

    fov = Math::Radians(fov_deg);
    focalDist = 0.1f;
    aperture = 0.0f;
    UpdateCamera();
}

Camera::Camera(const Camera& other)
    : position(other.position), up(other.up), right(other.right), forward(other.forward),
      focalDist(other.focalDist), aperture(other.aperture), fov(other.fov),
      chromaticAberration(other.chromaticAberration), isMoving(false), worldUp(other.worldUp),
      pivot(other.pivot), pitch(other.pitch), radius(other.radius), yaw(other.yaw)
{
}

// Assignment copies the public view state and flags a change, like Camera.cpp:124-130
// (which compares and copies the bytes from `position` up to `isMoving`).
Camera& Camera::operator=(const Camera& other)
{
    bool changed = std::memcmp(&position, &other.position,
                               (const char*)&other.isMoving - (const char*)&other.position) != 0;
    position = other.position;
    up = other.up;
    right = other.right;
    forward = other.forward;
    focalDist = other.focalDist;
    aperture = other.aperture;
    fov = other.fov;
    chromaticAberration = other.chromaticAberration;
    isMoving = changed;
    return *this;
}

void Camera::OffsetOrientation(float dx, float dy)
{
    pitch -= dy;
    yaw += dx;
    UpdateCamera();
}

void Camera::Strafe(float dx, float dy)
{
    Vec3 translation = right * -dx + up * dy;
    pivot = pivot + translation;
    UpdateCamera();
}

void Camera::SetRadius(float dr)
{
    radius += dr;
    UpdateCamera();
}

void Camera::SetFov(float val) { fov = Math::Radians(val); }

void Camera::UpdateCamera()
{
    Vec3 f;
    double ry = (double)Math::Radians(yaw);
    double rp = (double)Math::Radians(pitch);
    f.x = (float)(::cos(ry) * ::cos(rp));
    f.y = (float)::sin(rp);
    f.z = (float)(::sin(ry) * ::cos(rp));

    forward = Vec3::Normalize(f);
    position = pivot + (forward * -1.0f) * radius;
    right = Vec3::Normalize(Vec3::Cross(forward, worldUp));
    up = Vec3::Normalize(Vec3::Cross(right, forward));
}

// ---------------------------------------------------------------- Mesh
void Mesh::BuildBVH()
{
    const int numTris = (int)(verticesUVX.size() / 3);
    std::vector<lfbvh::bbox> bounds(numTris);
    for (int i = 0; i < numTris; ++i)
    {
        bounds[i].grow(Vec3(verticesUVX[i * 3 + 0]));
        bounds[i].grow(Vec3(verticesUVX[i * 3 + 1]));
        bounds[i].grow(Vec3(verticesUVX[i * 3 + 2]));
    }
    lfbvh::BuildMeshBvh(bounds.data(), numTris, bvh);
}

// ---------------------------------------------------------------- HDR data
HDRData::~HDRData()
{
    delete[] cols;
    delete[] marginalDistData;
    delete[] conditionalDistData;
}

// ---------------------------------------------------------------- BvhTranslator
void BvhTranslator::Process(const lfbvh::BuiltBvh& tlas, const std::vector<Mesh*>& meshes,
                            const std::vector<MeshInstance>& instances)
{
    const int nm = (int)meshes.size();
    bvhRootStartIndices.assign(nm, 0);
    triStartIndices.assign(nm, 0);
    int nodeCnt = 0, triCnt = 0;
    for (int i = 0; i < nm; ++i)
    {
        bvhRootStartIndices[i] = nodeCnt;
        triStartIndices[i] = triCnt;
        nodeCnt += meshes[i]->bvh.NodeCount();
        triCnt += (int)meshes[i]->bvh.packed.size();
    }
    topLevelIndex = nodeCnt;
    nodes.assign((size_t)nodeCnt + 2 * instances.size(), Node{});

    Node* out = nodes.data();
    ParallelFor(nm, [&](int i) {
        lfbvh::FlattenMesh(meshes[i]->bvh, bvhRootStartIndices[i], triStartIndices[i], out);
    }, 256);
    UpdateTLAS(tlas, instances);
}

void BvhTranslator::UpdateTLAS(const lfbvh::BuiltBvh& tlas, const std::vector<MeshInstance>& instances)
{
    std::vector<int> root(instances.size()), mat(instances.size());
    for (size_t i = 0; i < instances.size(); ++i)
    {
        root[i] = bvhRootStartIndices[instances[i].meshID];
        mat[i] = instances[i].materialID;
    }
    lfbvh::FlattenInstances(tlas, topLevelIndex, root.data(), mat.data(), nodes.data());
}

// ---------------------------------------------------------------- Scene
Scene::Scene() {}

Scene::~Scene()
{
    delete camera;
    delete hdrData;
    for (Mesh* m : meshes) delete m;
    for (Texture* t : textures) delete t;
}

void Scene::AddCamera(Vec3 pos, Vec3 lookAt, float fov)
{
    delete camera;
    camera = new Camera(pos, lookAt, fov);
}

int Scene::AddMesh(const std::string& filename)
{
    for (size_t i = 0; i < meshes.size(); ++i)
        if (meshes[i]->name == filename)
            return (int)i;
    Mesh* mesh = new Mesh;
    if (!mesh->LoadFromFile(filename))
    {
        delete mesh;
        lastError = "unable to load geometry " + filename;
        return -1;
    }
    meshes.push_back(mesh);
    return (int)meshes.size() - 1;
}

int Scene::AddMeshData(const std::string& name, const Vec4* v, const Vec4* n, int numVertices)
{
    if (numVertices <= 0 || numVertices % 3 != 0)
    {
        lastError = "AddMeshData: vertex count must be a positive multiple of 3";
        return -1;
    }
    Mesh* mesh = new Mesh;
    mesh->name = name;
    mesh->verticesUVX.assign(v, v + numVertices);
    mesh->normalsUVY.assign(n, n + numVertices);
    meshes.push_back(mesh);
    return (int)meshes.size() - 1;
}

int Scene::AddTexture(const std::string& filename)
{
    for (size_t i = 0; i < textures.size(); ++i)
        if (textures[i]->name == filename)
            return (int)i;
    Texture* t = new Texture;
    if (!t->LoadTexture(filename))
    {
        delete t;
        lastError = "unable to load texture " + filename;
        return -1;
    }
    textures.push_back(t);
    return (int)textures.size() - 1;
}

int Scene::AddMaterial(const Material& material)
{
    materials.push_back(material);
    return (int)materials.size() - 1;
}

void Scene::AddHDR(const std::string& filename)
{
    delete hdrData;
    hdrData = HDRLoader::load(filename.c_str());
    if (hdrData == nullptr)
    {
        lastError = "unable to load HDRI " + filename;
        Log("Unable to load HDRI\n");
    }
    else
        renderOptions.useEnvMap = true;
}

bool Scene::AddHDRData(const float* rgb, int width, int height)
{
    delete hdrData;
    hdrData = HDRLoader::FromRGB(rgb, width, height);
    if (!hdrData)
    {
        lastError = "AddHDRData: invalid image";
        return false;
    }
    renderOptions.useEnvMap = true;
    return true;
}

int Scene::AddMeshInstance(const MeshInstance& meshInstance)
{
    meshInstances.push_back(meshInstance);
    return (int)meshInstances.size() - 1;
}

int Scene::AddLight(const Light& light)
{
    lights.push_back(light);
    return (int)lights.size() - 1;
}

// Instance-level boxes: the mesh box mapped through each transform by the per-axis
// min/max of the scaled basis rows (Scene.cpp:106-146).
void Scene::createTLAS()
{
    const int ni = (int)meshInstances.size();
    std::vector<lfbvh::bbox> bounds(ni);
    ParallelFor(ni, [&](int i) {
        const lfbvh::bbox& b = meshes[meshInstances[i].meshID]->bvh.bounds;
        const Mat4& m = meshInstances[i].transform;
        Vec3 minBound = b.pmin, maxBound = b.pmax;
        Vec3 right(m[0][0], m[0][1], m[0][2]);
        Vec3 up(m[1][0], m[1][1], m[1][2]);
        Vec3 forward(m[2][0], m[2][1], m[2][2]);
        Vec3 translation(m[3][0], m[3][1], m[3][2]);
        Vec3 xa = right * minBound.x, xb = right * maxBound.x;
        Vec3 ya = up * minBound.y, yb = up * maxBound.y;
        Vec3 za = forward * minBound.z, zb = forward * maxBound.z;
        lfbvh::bbox out;
        out.pmin = Vec3::Min(xa, xb) + Vec3::Min(ya, yb) + Vec3::Min(za, zb) + translation;
        out.pmax = Vec3::Max(xa, xb) + Vec3::Max(ya, yb) + Vec3::Max(za, zb) + translation;
        bounds[i] = out;
    }, 4096);
    lfbvh::BuildInstanceBvh(bounds.data(), ni, sceneBvh);
    sceneBounds = sceneBvh.bounds;
}

void Scene::createBLAS()
{
    ParallelFor((int)meshes.size(), [&](int i) { meshes[i]->BuildBVH(); }, 1);
}

bool Scene::ValidateForDevice()
{
    if (meshes.empty() || meshInstances.empty())
    {
        lastError = "scene has no meshes or no mesh instances";
        return false;
    }
    for (size_t i = 0; i < meshes.size(); ++i)
        if (meshes[i]->verticesUVX.size() < 3 || meshes[i]->verticesUVX.size() % 3 != 0 ||
            meshes[i]->normalsUVY.size() != meshes[i]->verticesUVX.size())
        {
            lastError = "mesh " + std::to_string(i) + " has no triangles or mismatched normals";
            return false;
        }
    for (size_t i = 0; i < meshInstances.size(); ++i)
    {
        const MeshInstance& mi = meshInstances[i];
        if (mi.meshID < 0 || mi.meshID >= (int)meshes.size() || mi.materialID < 0 ||
            mi.materialID >= (int)materials.size())
        {
            lastError = "instance " + std::to_string(i) + " refers to a missing mesh or material";
            return false;
        }
    }
    if (materials.empty())
    {
        lastError = "scene has no materials";
        return false;
    }
    size_t tris = 0;
    for (Mesh* m : meshes) tris += m->verticesUVX.size() / 3;
    const size_t kExact = (size_t)1 << 24;   // indices are stored as floats in the nodes
    if (tris >= kExact || meshInstances.size() >= kExact)
    {
        lastError = "scene exceeds 2^24 triangles or instances (float-encoded indices)";
        return false;
    }
    return true;
}

void Scene::CreateAccelerationStructures()
{
    built = false;
    if (!ValidateForDevice())
    {
        Log("CreateAccelerationStructures: %s\n", lastError.c_str());
        return;
    }
    createBLAS();
    size_t meshNodes = 0;
    for (Mesh* m : meshes) meshNodes += (size_t)m->bvh.NodeCount();
    if (meshNodes + 2 * meshInstances.size() >= ((size_t)1 << 24))
    {
        lastError = "scene exceeds 2^24 BVH nodes (float-encoded indices)";
        Log("CreateAccelerationStructures: %s\n", lastError.c_str());
        return;
    }
    createTLAS();
    bvhTranslator.Process(sceneBvh, meshes, meshInstances);

    // Concatenate per-mesh data; triangle indices come from the packed BVH order
    // (Scene.cpp:195-215).
    const int nm = (int)meshes.size();
    std::vector<size_t> vbase(nm + 1, 0), ibase(nm + 1, 0);
    for (int i = 0; i < nm; ++i)
    {
        vbase[i + 1] = vbase[i] + meshes[i]->verticesUVX.size();
        ibase[i + 1] = ibase[i] + meshes[i]->bvh.packed.size();
    }
    vertIndices.resize(ibase[nm]);
    verticesUVX.resize(vbase[nm]);
    normalsUVY.resize(vbase[nm]);
    ParallelFor(nm, [&](int i) {
        const Mesh* m = meshes[i];
        const int vc = (int)vbase[i];
        for (size_t j = 0; j < m->bvh.packed.size(); ++j)
        {
            int index = m->bvh.packed[j];
            vertIndices[ibase[i] + j] = Indices{index * 3 + 0 + vc, index * 3 + 1 + vc, index * 3 + 2 + vc};
        }
        std::memcpy(&verticesUVX[vbase[i]], m->verticesUVX.data(), m->verticesUVX.size() * sizeof(Vec4));
        std::memcpy(&normalsUVY[vbase[i]], m->normalsUVY.data(), m->normalsUVY.size() * sizeof(Vec4));
    }, 256);

    transforms.resize(meshInstances.size());
    for (size_t i = 0; i < meshInstances.size(); ++i)
        transforms[i] = meshInstances[i].transform;

    textureMapsArray.clear();
    for (Texture* t : textures)
    {
        texWidth = t->width;
        texHeight = t->height;
        textureMapsArray.insert(textureMapsArray.end(), t->texData, t->texData + (size_t)t->width * t->height * 4);
    }
    built = true;
}

void Scene::RebuildInstances()
{
    createTLAS();
    bvhTranslator.UpdateTLAS(sceneBvh, meshInstances);
    for (size_t i = 0; i < meshInstances.size(); ++i)
        transforms[i] = meshInstances[i].transform;
    instancesModified = true;
}

// ---------------------------------------------------------------- Texture
bool Texture::LoadTexture(const std::string& filename)
{
    name = filename;
    FILE* f = std::fopen(filename.c_str(), "rb");
    if (!f) return false;
    char magic[3] = {0};
    int w = 0, h = 0, maxv = 0;
    bool ok = std::fscanf(f, "%2s %d %d %d", magic, &w, &h, &maxv) == 4 && std::strcmp(magic, "P6") == 0 &&
              w > 0 && h > 0 && maxv == 255;
    if (ok)
    {
        std::fgetc(f);
        std::vector<unsigned char> rgb((size_t)w * h * 3);
        ok = std::fread(rgb.data(), 1, rgb.size(), f) == rgb.size();
        if (ok)
        {
            delete[] texData;
            texData = new unsigned char[(size_t)w * h * 4];
            for (size_t i = 0; i < (size_t)w * h; ++i)
            {
                texData[i * 4 + 0] = rgb[i * 3 + 0];
                texData[i * 4 + 1] = rgb[i * 3 + 1];
                texData[i * 4 + 2] = rgb[i * 3 + 2];
                texData[i * 4 + 3] = 255;
            }
            width = w;
            height = h;
        }
    }
    std::fclose(f);
    return ok;
}
}
