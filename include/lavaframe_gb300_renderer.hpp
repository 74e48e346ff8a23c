// C++ drop-in renderer over the GB300 C ABI.
//
// LavaFrame's application code drives rendering through the abstract Renderer interface
// (LavaFrame/Renderer.h:71-117): Init, Finish, Render, Present, Update, GetProgress,
// GetSampleCount, GetOutputBuffer, GetOutputBufferHDR, SetViewport, Denoise. CudaRenderer
// implements it for a LavaFrame::Scene built with this library's scene layer
// (lavaframe_gb300/csrc/host/lf_scene.h) and keeps the frame bookkeeping of TiledRenderer
// (TiledRenderer.cpp:48-554):
//  - one Render() call renders one tile; tiles advance left to right, top tile row first;
//  - the shader `frame` counter advances per tile and starts at 2 for the first tile
//    (Init sets it to 1, every Update increments it before the next Render);
//  - sampleCounter advances after the last tile of a pass; GetOutputBufferHDR divides the
//    accumulation by it, like postprocess.glsl's invSampleCounter;
//  - a moved camera or edited instances reset the accumulation (TiledRenderer.cpp:471-484).
// There is no GL: Present/SetViewport are no-ops returning 0, Denoise is not available
// (the reference's OIDN binary is not part of this library) and returns 0.
//
// The base class is a template parameter. Inside the LavaFrame application it is the
// reference's own abstract renderer, so the object drops into `GlobalState.renderer`
// (a `LavaFrame::Renderer*`, GlobalState.h:7) unchanged:
//     new LavaFrame::CudaRenderer<LavaFrame::Scene, LavaFrame::Renderer>(scene, 0)
// The base is then constructed with (scene, "") and its GL state is never initialised
// (its destructor releases GL objects only when initialised, Renderer.cpp:44-48). Without
// the reference headers the default base is RendererInterface, the same virtuals without the
// GL handles.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "lavaframe_gb300.h"

namespace LavaFrame
{
class Scene;

// Interface of the reference Renderer without its GL handles.
class RendererInterface
{
public:
    virtual ~RendererInterface() = default;
    virtual void Init() = 0;
    virtual void Finish() = 0;
    virtual void Render() = 0;
    virtual void Present() const = 0;
    virtual void Update(float secondsElapsed) = 0;
    virtual float GetProgress() const = 0;
    virtual int GetSampleCount() const = 0;
    virtual void GetOutputBuffer(unsigned char** data, int& w, int& h) = 0;
    virtual void GetOutputBufferHDR(float** data, int& w, int& h) = 0;
    virtual uint32_t SetViewport(int width, int height) = 0;
    virtual uint32_t Denoise() = 0;
};

// Flat-array view of a built scene, as consumed by lf_scene_upload (Renderer.cpp:76-188).
template <class SceneT>
inline lf_scene_view MakeSceneView(const SceneT& sc)
{
    lf_scene_view v;
    std::memset(&v, 0, sizeof v);
    v.nodes = reinterpret_cast<const float*>(sc.bvhTranslator.nodes.data());
    v.num_nodes = (int32_t)sc.bvhTranslator.nodes.size();
    v.top_level_index = sc.bvhTranslator.topLevelIndex;
    v.vert_indices = reinterpret_cast<const int32_t*>(sc.vertIndices.data());
    v.num_tris = (int32_t)sc.vertIndices.size();
    v.vertices_uvx = reinterpret_cast<const float*>(sc.verticesUVX.data());
    v.normals_uvy = reinterpret_cast<const float*>(sc.normalsUVY.data());
    v.num_vertices = (int32_t)sc.verticesUVX.size();
    v.materials = reinterpret_cast<const float*>(sc.materials.data());
    v.num_materials = (int32_t)sc.materials.size();
    v.transforms = reinterpret_cast<const float*>(sc.transforms.data());
    v.num_instances = (int32_t)sc.transforms.size();
    v.lights = sc.lights.empty() ? nullptr : reinterpret_cast<const float*>(sc.lights.data());
    v.num_lights = (int32_t)sc.lights.size();
    if (sc.hdrData)
    {
        v.env_rgb = sc.hdrData->cols;
        v.env_marginal = reinterpret_cast<const float*>(sc.hdrData->marginalDistData);
        v.env_conditional = reinterpret_cast<const float*>(sc.hdrData->conditionalDistData);
        v.env_width = sc.hdrData->width;
        v.env_height = sc.hdrData->height;
    }
    if (!sc.textures.empty())
    {
        v.textures = sc.textureMapsArray.data();
        v.tex_width = sc.texWidth;
        v.tex_height = sc.texHeight;
        v.num_textures = (int32_t)sc.textures.size();
    }
    return v;
}

namespace detail
{
// Constructs the renderer base: (scene, shaders directory) for LavaFrame::Renderer
// (Renderer.h:100), default construction for RendererInterface.
template <class Base, class SceneT, bool = std::is_same<Base, RendererInterface>::value>
struct RendererBase : Base
{
    explicit RendererBase(SceneT* scene) : Base(scene, std::string()) {}
};
template <class Base, class SceneT>
struct RendererBase<Base, SceneT, true> : Base
{
    explicit RendererBase(SceneT*) {}
};
}

template <class SceneT, class Base = RendererInterface>
class CudaRenderer : public detail::RendererBase<Base, SceneT>
{
public:
    CudaRenderer(SceneT* scene, int device = 0)
        : detail::RendererBase<Base, SceneT>(scene), scene_(scene), device_(device)
    {
    }
    ~CudaRenderer() override { Finish(); }

    void Init() override
    {
        if (initialized_) return;
        if (!scene_ || !scene_->camera) throw std::runtime_error("CudaRenderer: no scene");
        check(lf_ctx_create(device_, &ctx_), "lf_ctx_create");
        lf_scene_view v = MakeSceneView(*scene_);
        check(lf_scene_upload(ctx_, &v, &dscene_), "lf_scene_upload");
        const auto& o = scene_->renderOptions;
        w_ = o.resolution.x;
        h_ = o.resolution.y;
        tileW_ = o.tileWidth > 0 ? o.tileWidth : w_;
        tileH_ = o.tileHeight > 0 ? o.tileHeight : h_;
        numTilesX_ = (w_ + tileW_ - 1) / tileW_;
        numTilesY_ = (h_ + tileH_ - 1) / tileH_;
        sampleCounter_ = 1;
        frameCounter_ = 1;
        tileX_ = -1;
        tileY_ = numTilesY_ - 1;
        makeFrame();
        initialized_ = true;
    }

    void Finish() override
    {
        if (frame_) lf_frame_release(frame_);
        if (dscene_) lf_scene_release(dscene_);
        if (ctx_) lf_ctx_destroy(ctx_);
        frame_ = nullptr;
        dscene_ = nullptr;
        ctx_ = nullptr;
        initialized_ = false;
    }

    // Renders the current tile; with the frame created as frame_base = 2 and per-tile
    // frame keying, tile k of pass s is rendered with frame 2 + s * tiles + k, the value of
    // TiledRenderer's frameCounter for that tile.
    void Render() override
    {
        if (!initialized_ || tileX_ < 0) return;
        check(lf_frame_render_tile(frame_, sampleCounter_ - 1, tileX_, tileY_), "lf_frame_render_tile");
        check(lf_frame_sync(frame_), "lf_frame_sync");
    }

    void Present() const override {}

    void Update(float) override
    {
        if (!initialized_) return;
        if (scene_->instancesModified)
        {
            lf_scene_view v = MakeSceneView(*scene_);
            check(lf_scene_update_instances(dscene_, &v), "lf_scene_update_instances");
        }
        if (scene_->camera->isMoving || scene_->instancesModified)
        {
            tileX_ = -1;
            tileY_ = numTilesY_ - 1;
            sampleCounter_ = 1;
            frameCounter_ = 1;
            check(lf_frame_reset(frame_), "lf_frame_reset");
            scene_->instancesModified = false;
        }
        else
        {
            frameCounter_++;
            tileX_++;
            if (tileX_ >= numTilesX_)
            {
                tileX_ = 0;
                tileY_--;
                if (tileY_ < 0)
                {
                    tileX_ = 0;
                    tileY_ = numTilesY_ - 1;
                    sampleCounter_++;
                }
            }
        }
    }

    float GetProgress() const override
    {
        return float((numTilesY_ - tileY_ - 1) * numTilesX_ + tileX_) / float(numTilesX_ * numTilesY_);
    }
    int GetSampleCount() const override { return sampleCounter_; }

    // Mean radiance of the accumulated passes, RGB32F, row 0 at the bottom (caller
    // delete[]s). The reference reads back its post-processed buffer here; the linear mean
    // is what that post-processing starts from.
    void GetOutputBufferHDR(float** data, int& w, int& h) override
    {
        w = w_;
        h = h_;
        *data = new float[(size_t)w_ * h_ * 3];
        check(lf_frame_read_accum(frame_, *data), "lf_frame_read_accum");
        float inv = 1.0f / (float)sampleCounter_;
        for (size_t i = 0; i < (size_t)w_ * h_ * 3; ++i) (*data)[i] = (*data)[i] * inv;
    }

    // 8-bit output of the display pass (postprocess.glsl:26-171) with the scene's RenderOptions:
    // tone map, chromatic aberration and vignette, row 0 at the bottom (caller delete[]s).
    void GetOutputBuffer(unsigned char** data, int& w, int& h) override
    {
        w = w_;
        h = h_;
        const auto& o = scene_->renderOptions;
        lf_post_params pp;
        pp.tonemap = o.tonemapIndex;
        pp.use_ca = o.useCA ? 1 : 0;
        pp.use_ca_distortion = o.useCADistortion ? 1 : 0;
        pp.use_vignette = o.useVignette ? 1 : 0;
        pp.preview = 0;
        pp.ca_distance = o.caDistance;
        pp.ca_p1 = o.caP1;
        pp.ca_p2 = o.caP2;
        pp.ca_p3 = o.caP3;
        pp.vignette_intensity = o.vignetteIntensity;
        pp.vignette_power = o.vignettePower;
        *data = new unsigned char[(size_t)w_ * h_ * 3];
        check(lf_frame_postprocess(frame_, &pp, sampleCounter_, *data, nullptr), "lf_frame_postprocess");
    }

    uint32_t SetViewport(int, int) override { return 0; }
    uint32_t Denoise() override { return 0; }

    // Renders `passes` full sample passes at once (all tiles), keeping the same RNG keying
    // as calling Update()+Render() once per tile.
    void RenderPasses(int passes)
    {
        if (!initialized_ || passes <= 0) return;
        check(lf_frame_render(frame_, sampleCounter_ - 1, passes), "lf_frame_render");
        check(lf_frame_sync(frame_), "lf_frame_sync");
        sampleCounter_ += passes;
    }

    lf_ctx* context() { return ctx_; }

private:
    lf_render_params params() const
    {
        lf_render_params p;
        std::memset(&p, 0, sizeof p);
        const auto& o = scene_->renderOptions;
        const auto* c = scene_->camera;
        p.width = w_;
        p.height = h_;
        p.max_depth = o.maxDepth;
        p.enable_rr = o.enableRR ? 1 : 0;
        p.rr_depth = o.RRDepth;
        p.use_env_map = (o.useEnvMap && scene_->hdrData) ? 1 : 0;
        p.use_constant_bg = o.useConstantBg ? 1 : 0;
        p.bg_color[0] = o.bgColor.x; p.bg_color[1] = o.bgColor.y; p.bg_color[2] = o.bgColor.z;
        p.hdr_multiplier = o.hdrMultiplier;
        const float* src[4] = {&c->position.x, &c->right.x, &c->up.x, &c->forward.x};
        float* dst[4] = {p.cam_position, p.cam_right, p.cam_up, p.cam_forward};
        for (int k = 0; k < 4; ++k) std::memcpy(dst[k], src[k], 3 * sizeof(float));
        p.cam_fov = c->fov;
        p.cam_focal_dist = c->focalDist;
        p.cam_aperture = c->aperture;
        p.frame_base = 1;
        return p;
    }

    void makeFrame()
    {
        lf_render_params p = params();
        p.tile_width = tileW_;
        p.tile_height = tileH_;
        p.frame_base = 2;
        check(lf_frame_create(ctx_, dscene_, &p, LF_FRAME_TILED_FRAMES, &frame_), "lf_frame_create");
    }

    void check(lf_status st, const char* what)
    {
        if (st != LF_OK)
            throw std::runtime_error(std::string(what) + ": " + (ctx_ ? lf_ctx_last_error(ctx_) : "no context"));
    }

    SceneT* scene_;
    int device_;
    lf_ctx* ctx_ = nullptr;
    lf_scene* dscene_ = nullptr;
    lf_frame* frame_ = nullptr;
    bool initialized_ = false;
    int w_ = 0, h_ = 0, tileW_ = 0, tileH_ = 0, numTilesX_ = 1, numTilesY_ = 1;
    int tileX_ = -1, tileY_ = 0, sampleCounter_ = 1, frameCounter_ = 1;
};
}
