// LavaFrame scene API, rebuilt as the drop-in host surface of the GB300 path tracer.
//
// Class and member names, value layouts and call semantics follow the reference so that
// code written against it (Loader, Main, export) compiles and behaves the same:
//   Material          LavaFrame/Material.h:13-77      (112 bytes, 7 x vec4)
//   Light, Indices    LavaFrame/Scene.h:31-45          (60 and 12 bytes)
//   Camera            LavaFrame/Camera.h:14-47, Camera.cpp:101-169
//   Mesh/MeshInstance LavaFrame/Mesh.h:13-51, Mesh.cpp:28-111
//   RenderOptions     LavaFrame/Renderer.h:18-67
//   HDRData/HDRLoader LavaFrame/hdrloader.h:19-33, hdrloader.cpp:57-204
//   Scene             LavaFrame/Scene.h:47-107, Scene.cpp
// Additions (no reference counterpart): in-memory mesh and environment input
// (AddMeshData, AddHDRData), the aliases AddEnvMap/ProcessScene, and
// ValidateForDevice. Errors are reported through return values and LastError(), never by
// aborting.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "lf_bvh.h"
#include "lf_types.h"

namespace LavaFrame
{
    class Material
    {
    public:
        Material()
        {
            albedo = Vec3(1.0f, 1.0f, 1.0f);
            specular = 0.5f;
            emission = Vec3(0.0f, 0.0f, 0.0f);
            anisotropic = 0.0f;
            metallic = 0.0f;
            roughness = 0.5f;
            subsurface = 0.0f;
            specularTint = 0.0f;
            sheen = 0.0f;
            sheenTint = 0.0f;
            clearcoat = 0.0f;
            clearcoatRoughness = 0.0f;
            transmission = 0.0f;
            ior = 1.45f;
            atDistance = 1.0f;
            padding1 = 0.0f;
            extinction = Vec3(1.0f, 1.0f, 1.0f);
            padding2 = 0.0f;
            albedoTexID = -1.0f;
            metallicRoughnessTexID = -1.0f;
            normalmapTexID = -1.0f;
            emissionmapTexID = -1.0f;
        }

        Vec3 albedo;
        float specular;
        Vec3 emission;
        float anisotropic;
        float metallic;
        float roughness;
        float subsurface;
        float specularTint;
        float sheen;
        float sheenTint;
        float clearcoat;
        float clearcoatRoughness;
        float transmission;
        float ior;
        float atDistance;
        float padding1;
        Vec3 extinction;
        float padding2;
        float albedoTexID;
        float metallicRoughnessTexID;
        float normalmapTexID;
        float emissionmapTexID;
    };
    static_assert(sizeof(Material) == 112, "Material must stay 7 x vec4");

    enum LightType
    {
        RectLight,
        SphereLight,
        DistantLight
    };

    struct Light
    {
        Vec3 position;
        Vec3 emission;
        Vec3 u;
        Vec3 v;
        float radius = 0.f;
        float area = 0.f;
        float type = 0.f;
    };
    static_assert(sizeof(Light) == 60, "Light must stay 5 x vec3");

    struct Indices
    {
        int x, y, z;
    };

    class Camera
    {
    public:
        Camera(Vec3 eye, Vec3 lookat, float fov);
        Camera(const Camera& other);
        Camera& operator=(const Camera& other);

        void OffsetOrientation(float dx, float dy);
        void Strafe(float dx, float dy);
        void SetRadius(float dr);
        void SetFov(float val);

        Vec3 position;
        Vec3 up;
        Vec3 right;
        Vec3 forward;

        float focalDist;
        float aperture;
        float fov;   // radians

        bool chromaticAberration = false;
        bool isMoving = false;

    private:
        void UpdateCamera();

        Vec3 worldUp;
        Vec3 pivot;
        float pitch;
        float radius;
        float yaw;
    };

    class Mesh
    {
    public:
        void BuildBVH();
        bool LoadFromFile(const std::string& filename);

        std::vector<Vec4> verticesUVX;   // xyz + u
        std::vector<Vec4> normalsUVY;    // xyz + v
        lfbvh::BuiltBvh bvh;
        std::string name;
    };

    class MeshInstance
    {
    public:
        MeshInstance(std::string name_, int meshId, Mat4 xform, int matId)
            : transform(xform), name(std::move(name_)), materialID(matId), meshID(meshId)
        {
        }
        Mat4 transform;
        std::string name;
        int materialID;
        int meshID;
    };

    struct RenderOptions
    {
        RenderOptions()
        {
            maxDepth = 2;
            tileWidth = 512;
            tileHeight = 512;
            useEnvMap = false;
            resolution = iVec2(1280, 720);
            hdrMultiplier = 1.0f;
            enableRR = true;
            useConstantBg = false;
            RRDepth = 2;
            bgColor = Vec3(0.5f, 0.5f, 0.5f);
            denoiserFrameCnt = 50;
            enableAutomaticDenoise = false;
            tonemapIndex = 2;
            useCA = false;
            caDistance = 0.05f;
            caP1 = 5;
            caP2 = -0.5f;
            caP3 = 0.5f;
            useCADistortion = false;
            // The reference constructor shadows these three with locals
            // (Renderer.h:41-43) and leaves the members unset; they are defined here.
            useVignette = false;
            vignetteIntensity = 0.f;
            vignettePower = 1.f;
        }
        iVec2 resolution;
        int maxDepth;
        int tileWidth;
        int tileHeight;
        bool useEnvMap;
        bool enableRR;
        bool enableAutomaticDenoise;
        bool useConstantBg;
        bool useCA;
        bool useCADistortion;
        bool useVignette;
        int RRDepth;
        int denoiserFrameCnt;
        int tonemapIndex;
        float hdrMultiplier;
        float caDistance;
        float caP1;
        float caP2;
        float caP3;
        float vignetteIntensity;
        float vignettePower;
        Vec3 bgColor;
    };

    class HDRData
    {
    public:
        HDRData() = default;
        ~HDRData();
        HDRData(const HDRData&) = delete;
        HDRData& operator=(const HDRData&) = delete;

        int width = 0, height = 0;
        float* cols = nullptr;                 // RGB32F, row 0 first
        Vec2* marginalDistData = nullptr;      // x: inverted-CDF row coordinate, y: pdf
        Vec2* conditionalDistData = nullptr;   // x: inverted-CDF column coordinate, y: pdf
    };

    class HDRLoader
    {
    public:
        // Radiance .hdr (RGBE, flat or RLE scanlines); nullptr on failure.
        static HDRData* load(const char* fileName);
        // In-memory RGB32F image (copied). Builds the sampling tables.
        static HDRData* FromRGB(const float* rgb, int width, int height);
        // Marginal/conditional tables with precomputed inverted-CDF lookups
        // (hdrloader.cpp:57-131).
        static void buildDistributions(HDRData* res);
    };

    class Texture
    {
    public:
        ~Texture() { delete[] texData; }
        // Binary PPM (P6) only: decoded to RGBA8. Other formats return false.
        bool LoadTexture(const std::string& filename);
        int width = 0;
        int height = 0;
        unsigned char* texData = nullptr;
        std::string name;
    };

    // Flattened BVH: the 36-byte node array plus where the instance level starts.
    class BvhTranslator
    {
    public:
        using Node = lfbvh::FlatNode;

        // Flattens every mesh tree and the instance tree (bvh_translator.cpp:91-140).
        void Process(const lfbvh::BuiltBvh& tlas, const std::vector<Mesh*>& meshes,
                     const std::vector<MeshInstance>& instances);
        // Rewrites the instance level after a rebuild (bvh_translator.cpp:125-131).
        void UpdateTLAS(const lfbvh::BuiltBvh& tlas, const std::vector<MeshInstance>& instances);

        int topLevelIndex = 0;
        std::vector<Node> nodes;
        int nodeTexWidth = 0;
        std::vector<int> bvhRootStartIndices;   // per mesh
        std::vector<int> triStartIndices;       // per mesh, into the packed triangles
    };

    class Scene
    {
    public:
        Scene();
        ~Scene();
        Scene(const Scene&) = delete;
        Scene& operator=(const Scene&) = delete;

        int AddMesh(const std::string& filename);
        int AddTexture(const std::string& filename);
        int AddMaterial(const Material& material);
        int AddMeshInstance(const MeshInstance& meshInstance);
        int AddLight(const Light& light);
        void AddCamera(Vec3 eye, Vec3 lookat, float fov);
        void AddHDR(const std::string& filename);

        // In-memory inputs. Vertices are un-indexed (three per triangle), xyz + uv.
        int AddMeshData(const std::string& name, const Vec4* verticesUVX, const Vec4* normalsUVY, int numVertices);
        bool AddHDRData(const float* rgb, int width, int height);

        void CreateAccelerationStructures();
        void RebuildInstances();

        // Names used by the GB300 build plan for the same operations.
        void AddEnvMap(const std::string& filename) { AddHDR(filename); }
        void ProcessScene() { CreateAccelerationStructures(); }

        // Checks the limits the device layout relies on (indices exact as float, non-empty
        // meshes, valid mesh/material references). Returns false and sets LastError().
        bool ValidateForDevice();
        const std::string& LastError() const { return lastError; }

        RenderOptions renderOptions;
        std::vector<Mesh*> meshes;

        std::vector<Indices> vertIndices;
        std::vector<Vec4> verticesUVX;
        std::vector<Vec4> normalsUVY;
        std::vector<Mat4> transforms;

        std::vector<Material> materials;
        std::vector<MeshInstance> meshInstances;
        bool instancesModified = false;

        std::vector<Light> lights;
        HDRData* hdrData = nullptr;
        Camera* camera = nullptr;

        BvhTranslator bvhTranslator;
        lfbvh::bbox sceneBounds;

        std::vector<Texture*> textures;
        std::vector<unsigned char> textureMapsArray;
        int texWidth = 0;
        int texHeight = 0;

        bool built = false;

    private:
        void createBLAS();
        void createTLAS();
        lfbvh::BuiltBvh sceneBvh;
        std::string lastError;
    };

    // `.scene`/`.lfs` text format (Loader.cpp:45-385). Builds the acceleration structures
    // at the end, like the reference.
    bool LoadSceneFromFile(const std::string& filename, Scene* scene, RenderOptions& renderOptions);
    extern int (*Log)(const char* szFormat, ...);

    // Number of worker threads used for per-mesh BVH builds (0 = hardware concurrency).
    void SetBuildThreads(int n);
    int GetBuildThreads();
}
