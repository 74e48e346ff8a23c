// Test infrastructure: drives a CPU-compiled variant of the reference fragment shader
// (see ref_shader_gen.py) over a frame the way TiledRenderer does - one invocation of main()
// per pixel and sample with the uniforms of TiledRenderer::Init/Update, TexCoords at the
// pixel centre of the tile viewport - and accumulates the returned colours in sample order.
#pragma once

#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "glsl_shim.h"

extern "C" {
// Same fields as lf_scene_view / lf_render_params in include/lavaframe_gb300.h.
struct lfo_view
{
    const float* nodes;
    int32_t num_nodes;
    int32_t top_level_index;
    const int32_t* vert_indices;
    int32_t num_tris;
    const float* vertices_uvx;
    const float* normals_uvy;
    int32_t num_vertices;
    const float* materials;
    int32_t num_materials;
    const float* transforms;
    int32_t num_instances;
    const float* lights;
    int32_t num_lights;
    const float* env_rgb;
    const float* env_marginal;
    const float* env_conditional;
    int32_t env_width, env_height;
    const uint8_t* textures;
    int32_t tex_width, tex_height, num_textures;
};

struct lfo_params
{
    int32_t width, height;
    int32_t max_depth;
    int32_t enable_rr, rr_depth;
    int32_t use_env_map;
    int32_t use_constant_bg;
    float bg_color[3];
    float hdr_multiplier;
    float cam_position[3], cam_right[3], cam_up[3], cam_forward[3];
    float cam_fov, cam_focal_dist, cam_aperture;
    uint32_t seed;
    int32_t frame_base;
    int32_t tile_width, tile_height;
};
}

namespace refsh
{
template <class S>
int render(const lfo_view* v, const lfo_params* p, int first, int n, float* accum, float* paths, int threads)
{
    using namespace glsl;
    const int W = p->width, H = p->height;
    const int tileW = p->tile_width > 0 ? p->tile_width : W;
    const int tileH = p->tile_height > 0 ? p->tile_height : H;
    const bool env = v->env_rgb && v->env_width > 0;
    if (threads <= 0)
    {
        unsigned hc = std::thread::hardware_concurrency();
        threads = hc ? (int)hc : 1;
    }
    std::atomic<int> nextRow{0};
    auto work = [&]() {
        for (;;)
        {
            int gy = nextRow.fetch_add(1);
            if (gy >= H) break;
            int ty = gy / tileH, ly = gy - ty * tileH;
            for (int gx = 0; gx < W; ++gx)
            {
                int tx = gx / tileW, lx = gx - tx * tileW;
                float* acc = accum + ((size_t)gy * W + gx) * 3;
                for (int s = 0; s < n; ++s)
                {
                    S sh{};
                    sh.rrDepthValue = p->rr_depth;
                    sh.BVH = samplerBuffer{v->nodes, 3, (long long)v->num_nodes * 3};
                    sh.vertexIndicesTex = isamplerBuffer{v->vert_indices, 3, (long long)v->num_tris};
                    sh.verticesTex = samplerBuffer{v->vertices_uvx, 4, (long long)v->num_vertices};
                    sh.normalsTex = samplerBuffer{v->normals_uvy, 4, (long long)v->num_vertices};
                    sh.materialsTex = sampler2D{v->materials, 7 * v->num_materials, 1, 4, false};
                    sh.transformsTex = sampler2D{v->transforms, 4 * v->num_instances, 1, 4, false};
                    sh.lightsTex = sampler2D{v->lights, 5 * v->num_lights, 1, 3, false};
                    sh.textureMapsArrayTex = sampler2DArray{v->textures, v->tex_width, v->tex_height, v->num_textures};
                    if (env)
                    {
                        sh.hdrTex = sampler2D{v->env_rgb, v->env_width, v->env_height, 3, true};
                        sh.hdrMarginalDistTex = sampler2D{v->env_marginal, v->env_height, 1, 2, false};
                        sh.hdrCondDistTex = sampler2D{v->env_conditional, v->env_width, v->env_height, 2, false};
                    }
                    sh.accumTexture = sampler2D{};
                    // TiledRenderer::Init uniforms (TiledRenderer.cpp:221-233)
                    sh.hdrResolution = env ? (float)(v->env_width * v->env_height) : 0.0f;
                    sh.topBVHIndex = v->top_level_index;
                    sh.screenResolution = vec2((float)W, (float)H);
                    sh.numOfLights = v->num_lights;
                    sh.invNumTilesX = 1.0f / ((float)W / (float)tileW);
                    sh.invNumTilesY = 1.0f / ((float)H / (float)tileH);
                    // TiledRenderer::Update uniforms (TiledRenderer.cpp:506-520)
                    sh.camera.position = vec3(p->cam_position[0], p->cam_position[1], p->cam_position[2]);
                    sh.camera.right = vec3(p->cam_right[0], p->cam_right[1], p->cam_right[2]);
                    sh.camera.up = vec3(p->cam_up[0], p->cam_up[1], p->cam_up[2]);
                    sh.camera.forward = vec3(p->cam_forward[0], p->cam_forward[1], p->cam_forward[2]);
                    sh.camera.fov = p->cam_fov;
                    sh.camera.focalDist = p->cam_focal_dist;
                    sh.camera.aperture = p->cam_aperture;
                    sh.useEnvMap = env && p->use_env_map;
                    sh.hdrMultiplier = p->hdr_multiplier;
                    sh.maxDepth = p->max_depth;
                    sh.tileX = tx;
                    sh.tileY = ty;
                    sh.bgColor = vec3(p->bg_color[0], p->bg_color[1], p->bg_color[2]);
                    sh.frame = p->frame_base + first + s;
                    sh.TexCoords = vec2(((float)lx + 0.5f) / (float)tileW, ((float)ly + 0.5f) / (float)tileH);
                    sh.main();
                    vec3 col = sh.color;
                    acc[0] = acc[0] + col.x;
                    acc[1] = acc[1] + col.y;
                    acc[2] = acc[2] + col.z;
                    if (paths)
                    {
                        float* o = paths + (((size_t)s * H + gy) * W + gx) * 3;
                        o[0] = col.x;
                        o[1] = col.y;
                        o[2] = col.z;
                    }
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    return 0;
}
}
