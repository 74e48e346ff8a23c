/*
 * lavaframe_gb300.h - C ABI of the GB300 path-tracing core for LavaFrame.
 *
 * This ABI replaces the OpenGL renderer boundary of the reference (the abstract
 * LavaFrame::Renderer in LavaFrame/Renderer.h:71-117 and TiledRenderer in
 * LavaFrame/TiledRenderer.h:15-72) and exposes the host scene layer (LavaFrame::Scene,
 * LavaFrame/Scene.h:47-107) to non-C++ callers. Plain pointers and sizes only.
 *
 * Conventions
 *  - Every function returns lf_status (0 = LF_OK) unless stated otherwise; failures never
 *    abort the process. The text of the last error is available from lf_ctx_last_error /
 *    lf_hscene_last_error.
 *  - The caller owns all host buffers; the library owns all device memory it allocates.
 *  - One lf_ctx drives one GPU through one CUDA stream; calls on the same context are
 *    serialised by an internal lock.
 *  - Device-side failures (BVH stack overflow, step limit, queue overflow) are reported as
 *    LF_ERR_DEVICE with the bits in lf_ctx_device_errors; no kernel traps or spins without
 *    an iteration limit.
 *  - Flat scene arrays use the reference layouts byte for byte: 36-byte BVH nodes
 *    (bvh_translator.h:48-53), int3 triangle indices, float4 vertices/normals, 112-byte
 *    materials (Material.h:13-77), 64-byte Mat4 transforms (row i = GL column i), 60-byte
 *    lights (Scene.h:31-40), RGB32F environment with its marginal/conditional tables
 *    (hdrloader.h:19-28), RGBA8 texture layers.
 */
#ifndef LAVAFRAME_GB300_H
#define LAVAFRAME_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LF_ABI_VERSION 1

typedef enum lf_status
{
    LF_OK = 0,
    LF_ERR_INVALID = 1,    /* bad argument or inconsistent scene data */
    LF_ERR_CUDA = 2,       /* CUDA runtime error (no device, launch failure, ...) */
    LF_ERR_OOM = 3,        /* device allocation failed */
    LF_ERR_DEVICE = 4,     /* a kernel reported an error bit (see lf_ctx_device_errors) */
    LF_ERR_TIMEOUT = 5,    /* wait deadline passed; work is still in flight */
    LF_ERR_STATE = 6,      /* call not valid in the object's current state */
    LF_ERR_IO = 7,         /* file could not be read */
    LF_ERR_BUDGET = 8      /* admission refused: memory budget exhausted */
} lf_status;

/* Device-side error bits. */
#define LF_DEVERR_STACK 0x1u   /* BVH stack (64 entries) overflowed; the ray was ended */
#define LF_DEVERR_STEPS 0x2u   /* traversal step limit reached */
#define LF_DEVERR_QUEUE 0x4u   /* wavefront queue overflow */
#define LF_DEVERR_INDEX 0x8u   /* out-of-range index caught by a device bounds check */
#define LF_DEVERR_GUIDE_TIMEOUT 0x10u /* a tensor-core guide kernel's bounded wait ran out; its CTAs returned */

typedef struct lf_ctx lf_ctx;
typedef struct lf_scene lf_scene;     /* device-resident scene */
typedef struct lf_frame lf_frame;     /* render target: accumulation + wavefront state */
typedef struct lf_hscene lf_hscene;   /* host scene (LavaFrame::Scene) */

/* ------------------------------------------------------------------ host scene
 * Mirrors LavaFrame::Scene (Scene.h:47-107) and LoadSceneFromFile (Loader.h:15). */

/* new Scene() */
lf_status lf_hscene_create(lf_hscene** out);
/* Scene::~Scene */
void lf_hscene_destroy(lf_hscene* s);
const char* lf_hscene_last_error(const lf_hscene* s);
/* LoadSceneFromFile(filename, scene, renderOptions) (Loader.cpp:45-385); builds the
 * acceleration structures like the reference. */
lf_status lf_hscene_load_file(lf_hscene* s, const char* path);
/* Scene::AddMesh (Scene.cpp:21-40) from memory: num_vertices = 3 x triangles, 4 floats
 * each (xyz + u, xyz + v). Returns the mesh id, or -1. */
int32_t lf_hscene_add_mesh(lf_hscene* s, const float* vertices_uvx, const float* normals_uvy, int32_t num_vertices);
/* Scene::AddMesh(filename) with an OBJ file. Returns the mesh id, or -1. */
int32_t lf_hscene_add_mesh_file(lf_hscene* s, const char* path);
/* Scene::AddMaterial (Scene.cpp:70-75): 28 floats in Material order. Returns the id. */
int32_t lf_hscene_add_material(lf_hscene* s, const float* material28);
/* Scene::AddMeshInstance (Scene.cpp:92-97): transform = 16 floats (Mat4 data order). */
int32_t lf_hscene_add_instance(lf_hscene* s, int32_t mesh_id, const float* transform16, int32_t material_id);
/* Scene::AddLight (Scene.cpp:99-104): 15 floats in Light order. */
int32_t lf_hscene_add_light(lf_hscene* s, const float* light15);
/* Scene::AddCamera (Scene.cpp:15-19) plus the aperture/focal distance the loader sets. */
lf_status lf_hscene_set_camera(lf_hscene* s, const float eye[3], const float lookat[3], float fov_degrees,
                               float aperture, float focal_dist);
/* Scene::AddHDR (Scene.cpp:77-90), from a Radiance .hdr file or from RGB32F memory. */
lf_status lf_hscene_add_hdr_file(lf_hscene* s, const char* path);
lf_status lf_hscene_add_hdr(lf_hscene* s, const float* rgb, int32_t width, int32_t height);
/* Scene::CreateAccelerationStructures (Scene.cpp:180-231) - named ProcessScene in the
 * build plan. Mesh-level builds run in parallel on `threads` host threads (0 = all). */
lf_status lf_hscene_build(lf_hscene* s, int32_t threads);
/* Scene::RebuildInstances (Scene.cpp:165-178) after editing instances. */
lf_status lf_hscene_set_instance(lf_hscene* s, int32_t instance, const float* transform16, int32_t material_id);
lf_status lf_hscene_rebuild_instances(lf_hscene* s);

/* Pointers into the built scene, valid until the next build or destroy. */
typedef struct lf_scene_view
{
    const float* nodes;            /* 9 floats per node */
    int32_t num_nodes;
    int32_t top_level_index;
    const int32_t* vert_indices;   /* 3 ints per packed triangle */
    int32_t num_tris;
    const float* vertices_uvx;     /* 4 floats per vertex */
    const float* normals_uvy;      /* 4 floats per vertex */
    int32_t num_vertices;
    const float* materials;        /* 28 floats per material */
    int32_t num_materials;
    const float* transforms;       /* 16 floats per instance */
    int32_t num_instances;
    const float* lights;           /* 15 floats per light */
    int32_t num_lights;
    const float* env_rgb;          /* width*height*3, may be NULL */
    const float* env_marginal;     /* height*2 */
    const float* env_conditional;  /* width*height*2 */
    int32_t env_width, env_height;
    const uint8_t* textures;       /* num_textures * tex_width * tex_height * 4 */
    int32_t tex_width, tex_height, num_textures;
} lf_scene_view;

lf_status lf_hscene_view(const lf_hscene* s, lf_scene_view* out);

/* Scene contents before flattening: counts[0..3] = meshes, instances, materials, lights.
 * Optional arrays (may be NULL): vertex count per mesh, mesh id and material id per
 * instance (Scene::meshes, Scene::meshInstances). */
lf_status lf_hscene_counts(const lf_hscene* s, int32_t counts[4]);
lf_status lf_hscene_layout(const lf_hscene* s, int32_t* mesh_vertex_counts, int32_t* instance_mesh,
                           int32_t* instance_material);

/* Per-render parameters: RenderOptions (Renderer.h:18-67), the Camera uniforms
 * (TiledRenderer.cpp:506-520) and the RNG keying. */
typedef struct lf_render_params
{
    int32_t width, height;
    int32_t max_depth;
    int32_t enable_rr, rr_depth;
    int32_t use_env_map;       /* ENVMAP (requires environment data) */
    int32_t use_constant_bg;   /* CONSTANT_BG */
    float bg_color[3];
    float hdr_multiplier;
    float cam_position[3], cam_right[3], cam_up[3], cam_forward[3];
    float cam_fov;             /* radians, as Camera::fov */
    float cam_focal_dist, cam_aperture;
    uint32_t seed;             /* 0 reproduces the reference's per-pixel seeding */
    int32_t frame_base;        /* shader `frame` for sample 0; sample s uses frame_base + s */
    int32_t tile_width, tile_height;   /* 0 = whole frame; else TiledRenderer tiling */
} lf_render_params;

/* Fills params from the scene's RenderOptions and camera. */
lf_status lf_hscene_render_params(const lf_hscene* s, lf_render_params* out);

/* Procedural workloads (seeded, deterministic on every host). */
lf_status lf_gen_cornell(lf_hscene* s, int32_t width, int32_t height);
/* The same box with every wall and box face split into subdiv x subdiv quads (34 subdiv^2
 * triangles): the Cornell generator scaled for the serving mix. */
lf_status lf_gen_cornell_tess(lf_hscene* s, int32_t width, int32_t height, int32_t subdiv);
lf_status lf_gen_soup(lf_hscene* s, int32_t instances, int32_t tris_per_instance, uint64_t seed);
lf_status lf_gen_icospheres(lf_hscene* s, int32_t instances, int32_t level, uint64_t seed, int32_t env_width,
                            int32_t env_height);
lf_status lf_gen_room(lf_hscene* s, int32_t boxes, uint64_t seed);
/* Rays for the intersection microbench: origins uniform in [lo, hi], directions uniform on
 * the sphere; 8 floats per ray (origin xyz, 0, direction xyz, tmax). */
lf_status lf_gen_rays(const float lo[3], const float hi[3], int64_t n, uint64_t seed, float tmax, float* rays_out);

/* ------------------------------------------------------------------ device context */
lf_status lf_ctx_create(int32_t device, lf_ctx** out);
void lf_ctx_destroy(lf_ctx* c);
const char* lf_ctx_last_error(const lf_ctx* c);
uint32_t lf_ctx_device_errors(const lf_ctx* c);
lf_status lf_ctx_sync(lf_ctx* c);
/* CUDA-event timing on the context stream: start records an event, stop records a second
 * one, waits for it and returns the elapsed device time in milliseconds. */
lf_status lf_ctx_timer_start(lf_ctx* c);
lf_status lf_ctx_timer_stop(lf_ctx* c, float* ms);

/* Renderer::Init upload set (Renderer.cpp:76-188): copies the flat arrays to HBM and
 * re-encodes them for the kernels. */
lf_status lf_scene_upload(lf_ctx* c, const lf_scene_view* view, lf_scene** out);
/* Renderer::Update partial re-upload (Renderer.cpp:190-205): transforms, materials and
 * the instance-level nodes from top_level_index on. */
lf_status lf_scene_update_instances(lf_scene* sc, const lf_scene_view* view);
lf_status lf_scene_release(lf_scene* sc);
/* Culling margins of the traversal (relative, absolute); rel < 0 turns culling off. */
lf_status lf_scene_set_culling(lf_scene* sc, float rel, float abs_margin);
/* Traversal of the scene's queries and renders: 1 = the 4-wide tree collapsed from the
 * reference BVH (default), 0 = the reference's binary tree. Both return the reference's
 * hits: the wide tree tests the same leaves and resolves equal distances by the reference's
 * depth-first order. */
lf_status lf_scene_set_traversal(lf_scene* sc, int32_t wide);
size_t lf_scene_device_bytes(const lf_scene* sc);

/* ------------------------------------------------------------------ ray queries
 * ClosestHit / AnyHit (closest_hit.glsl:7-205, anyhit.glsl:7-173) as batched queries.
 * Ray: 8 floats (origin xyz, unused, direction xyz, tmax). tmax is the initial t of the
 * closest-hit query (the shader uses INFINITY = 1e6) and maxDist of the any-hit query. */
typedef struct lf_hit
{
    float t;          /* 1e6 when nothing was hit */
    int32_t instance; /* instance index, -1 for none (or an analytic light hit) */
    int32_t prim;     /* packed triangle index (row of vert_indices), -1 for none */
    int32_t light;    /* analytic light index when a light is the closest hit, else -1 */
} lf_hit;

#define LF_TRACE_LIGHTS 0x1   /* include analytic lights, as the LIGHTS shader define */
#define LF_TRACE_STATS 0x2    /* count node visits / triangle tests (slower) */
#define LF_TRACE_UNSORTED 0x4 /* trace in input order (no binning by origin cell and octant) */
#define LF_TRACE_SIMPLE 0x8   /* one thread per ray, no persistent warps */

/* Host buffers: copies rays in, traces, copies hits out (synchronous). When the output lies
 * in one block from lf_host_alloc of this context, the kernels write the results there and
 * nothing is copied back. */
lf_status lf_trace_closest(lf_ctx* c, lf_scene* sc, const float* rays, int64_t n, lf_hit* hits, uint32_t flags);
/* occluded[i] = 1 when something lies closer than tmax. */
lf_status lf_trace_any(lf_ctx* c, lf_scene* sc, const float* rays, int64_t n, uint8_t* occluded, uint32_t flags);
/* Host-buffer queries split the rays into `chunks` pieces (1..8; 0 = automatic, the
 * default: two pieces from 2^24 rays up, else one): piece k+1 is copied in and piece k-1
 * copied out while piece k is sorted and traced. Every ray's result is the same for any
 * setting; LF_TRACE_STATS queries run whole. */
lf_status lf_ctx_set_host_chunks(lf_ctx* c, int32_t chunks);
/* Device buffers, asynchronous on the context stream (lf_ctx_sync to wait). */
lf_status lf_trace_closest_device(lf_ctx* c, lf_scene* sc, const void* d_rays, int64_t n, void* d_hits,
                                  uint32_t flags);
lf_status lf_trace_any_device(lf_ctx* c, lf_scene* sc, const void* d_rays, int64_t n, void* d_occluded,
                              uint32_t flags);
/* Traversal counters of the last LF_TRACE_STATS query: node visits, triangle tests,
 * leaf visits (sums over all rays). */
lf_status lf_trace_stats(const lf_ctx* c, uint64_t out3[3]);

/* Traversal-kernel timer (no counterpart in the reference; measurement aid): while on, the
 * device ray queries (lf_trace_closest_device / lf_trace_any_device, binned path) record a
 * CUDA event pair on the context's stream around the traversal kernel alone. _read waits for
 * the recorded launches and returns their summed duration and count, then starts over. */
lf_status lf_ctx_kernel_timer(lf_ctx* c, int32_t on);
/* Streaming multiprocessors and maximum SM clock (MHz) of the context's device. */
lf_status lf_ctx_device_attrs(lf_ctx* c, int32_t* sm_count, int32_t* max_sm_mhz);
lf_status lf_ctx_kernel_timer_read(lf_ctx* c, double* total_ms, int64_t* launches);
/* Page-locked host memory, mapped into the device's address space (fast host<->device
 * copies; host queries write their results straight into it), e.g. for ray and hit buffers. */
lf_status lf_host_alloc(lf_ctx* c, size_t bytes, void** out);
lf_status lf_host_free(lf_ctx* c, void* p);
/* Device memory helpers for callers without their own allocator. */
lf_status lf_device_alloc(lf_ctx* c, size_t bytes, void** out);
lf_status lf_device_free(lf_ctx* c, void* p);
lf_status lf_copy_to_device(lf_ctx* c, void* dst, const void* src, size_t bytes);
lf_status lf_copy_to_host(lf_ctx* c, void* dst, const void* src, size_t bytes);

/* ------------------------------------------------------------------ progressive render
 * One render target with its accumulation buffer: TiledRenderer::Render/Update
 * (TiledRenderer.cpp:317-554) without the GL passes. Samples accumulate in sample order,
 * so results do not depend on how calls are batched. */
#define LF_FRAME_FP64_ACCUM 0x1   /* also accumulate in double precision */
#define LF_FRAME_USE_GRAPH 0x2    /* per-batch pipeline: record each batch (generate, bounces,
                                     accumulate) as a CUDA graph and replay it; the engine
                                     pipeline always replays graph-captured steps */
#define LF_FRAME_TILED_FRAMES 0x4 /* TiledRenderer RNG keying: the shader `frame` advances per
                                     tile (TiledRenderer.cpp:486-501): frame = frame_base +
                                     sample * tiles + tile, tiles counted from the top row */
#define LF_FRAME_PER_BATCH 0x8    /* lf_frame_render runs bounce-synchronous batches (every
                                     path of a batch advances one bounce per launch) instead of
                                     the context's multi-job engine (paths regenerate in a fixed
                                     slot pool). Results are identical; only speed differs. */

lf_status lf_frame_create(lf_ctx* c, lf_scene* sc, const lf_render_params* p, uint32_t flags, lf_frame** out);
/* Queue samples [first_sample, first_sample + count) (asynchronous). */
lf_status lf_frame_render(lf_frame* f, int32_t first_sample, int32_t count);
/* One sample of one tile (TiledRenderer::Render, TiledRenderer.cpp:317-352): tile
 * (tile_x, tile_y) of the frame's tiling, tile_y counted from the bottom as in GL. */
lf_status lf_frame_render_tile(lf_frame* f, int32_t sample, int32_t tile_x, int32_t tile_y);
/* Wait for queued work and report device errors. */
lf_status lf_frame_sync(lf_frame* f);
/* GetOutputBufferHDR (TiledRenderer.cpp:399-414): accumulated radiance sum, RGB32F,
 * row 0 = bottom row as in GL. Divide by the sample count for the mean. */
lf_status lf_frame_read_accum(lf_frame* f, float* rgb);
lf_status lf_frame_read_accum64(lf_frame* f, double* rgb);
/* Per-sample, per-pixel path radiance of the most recent batch, RGB32F,
 * [sample][pixel], for path-level comparisons. */
lf_status lf_frame_read_paths(lf_frame* f, float* rgb, int32_t max_samples);
lf_status lf_frame_reset(lf_frame* f);
/* Counters since creation/reset: [0] camera paths, [1] extension rays, [2] shadow rays,
 * [3] light-index clamps (rand() == 1). */
lf_status lf_frame_counters(lf_frame* f, uint64_t out4[4]);
/* Samples per wavefront batch (per-batch pipeline) or per engine pass (memory/parallelism
 * trade-off); 0 = default. */
lf_status lf_frame_set_batch(lf_frame* f, int32_t samples_per_batch);
lf_status lf_frame_release(lf_frame* f);

/* Engine of the context (no counterpart in the reference; the reference renders one tile per
 * GL draw). `slots` = path slots in the pool (0 keeps the current pool), block sizes of the
 * extend / shade / shadow kernels (0 = default 128; multiples of 32 up to 1024, shade up to
 * 256), and the register cap of the shade kernel as the threads per SM it must fit (0 = none,
 * 512, 768 or 1024). The engine starts with 2^24 slots and a cap of 512. Fails with LF_ERR_STATE
 * while passes are in flight. */
lf_status lf_ctx_configure_engine(lf_ctx* c, int32_t slots, int32_t block_extend, int32_t block_shade,
                                  int32_t block_shadow, int32_t shade_threads_per_sm);
/* Sort-by-material in the engine (no counterpart in the reference, whose shader shades each
 * fragment where it lands, pathtrace.glsl:246-291): 1 = the extend kernel buckets the paths
 * that hit a surface by the class of their material's shading code (opaque dielectric, metal,
 * transmissive, textured) and shade takes the buckets one after the other, so that a warp
 * runs one class; 0 = hits in the order extend finished them; 2 (default) = sorted in the
 * steps of a single job whose scene has instances of more than one class, unsorted otherwise
 * (multi-job steps, single-class scenes). Results are unchanged either way. The buckets take
 * 16 B per path slot, allocated on first use. Fails with LF_ERR_STATE while passes are in
 * flight. */
lf_status lf_ctx_set_engine_sort(lf_ctx* c, int32_t sort_by_material);
/* Engine drain threshold (no counterpart in the reference): once every path id of a frame run
 * is issued and at most `paths` paths are still in flight, the run finishes them with one
 * kernel that takes each path through its remaining bounces instead of a further step pair per
 * bounce (default 2^22; 0 = never). Results are unchanged. */
lf_status lf_ctx_set_engine_drain(lf_ctx* c, int64_t paths);
/* Current pool size and device bytes of the engine (0, 0 before first use). */
lf_status lf_ctx_engine_info(lf_ctx* c, int64_t* slots, int64_t* device_bytes);

/* ------------------------------------------------------------------ post-process and export
 * The display pass (postprocess.glsl:26-171 with TiledRenderer's uniforms): accumulated sum /
 * samples (optionally with chromatic aberration), tone map 0..6 (none, linear, ACES,
 * Reinhard, Kanjero, Hejl-Richard, Uncharted 2) with the shader's gamma, optional vignette,
 * then the 8-bit conversion GetOutputBuffer reads (clamp to [0, 1], round to nearest). Fields
 * follow RenderOptions (Renderer.h:18-67); `preview` is the camera-moving flag (no CA). */
typedef struct lf_post_params
{
    int32_t tonemap;
    int32_t use_ca, use_ca_distortion, use_vignette, preview;
    float ca_distance, ca_p1, ca_p2, ca_p3;
    float vignette_intensity, vignette_power;
} lf_post_params;

/* rgb8 (W*H*3 bytes) and/or rgbf (W*H*3 floats, after tone map and vignette, before the
 * 8-bit conversion); row 0 = bottom as in GL. `samples` = the accumulated sample count. */
lf_status lf_frame_postprocess(lf_frame* f, const lf_post_params* p, int32_t samples, uint8_t* rgb8, float* rgbf);
/* Image export (Export.h:14-151 writes through stb/tinyexr; here): PNG, BMP, TGA, JPEG and PPM
 * (8-bit RGB), PFM and OpenEXR (float RGB). Input rows are bottom-first as the frame buffers;
 * PNG, BMP, TGA and PPM show the image upright (the reference flips on write; BMP and TGA store
 * rows bottom-up), PFM stores rows bottom-first as the format wants, and EXR stores the rows in
 * the order given, as the reference's SaveFrameEXR does with the GL buffer (Export.h:56-151:
 * channels B, G, R as 32-bit float, ZIP compression). TGA is run-length encoded
 * (stb_image_write's default); PNG rows are filtered and deflated. */
lf_status lf_write_png(const char* path, const uint8_t* rgb8, int32_t width, int32_t height);
lf_status lf_write_bmp(const char* path, const uint8_t* rgb8, int32_t width, int32_t height);
lf_status lf_write_tga(const char* path, const uint8_t* rgb8, int32_t width, int32_t height);
lf_status lf_write_ppm(const char* path, const uint8_t* rgb8, int32_t width, int32_t height);
lf_status lf_write_pfm(const char* path, const float* rgbf, int32_t width, int32_t height);
lf_status lf_write_exr(const char* path, const float* rgbf, int32_t width, int32_t height);
/* EXR with a chosen compression: 0 none, 1 RLE, 2 ZIPS (one-line ZIP blocks), 3 ZIP (the
 * default of lf_write_exr); PIZ and ZFP are not written. */
lf_status lf_write_exr_compressed(const char* path, const float* rgbf, int32_t width, int32_t height,
                                  int32_t compression);
/* Baseline JPEG (SaveFrameJPG, Export.h:37-46): `quality` 1..100 scales the quantisation
 * tables; 4:4:4 YCbCr; Huffman tables built for the image. Shown upright like PNG. */
lf_status lf_write_jpg(const char* path, const uint8_t* rgb8, int32_t width, int32_t height, int32_t quality);

/* Render without allocating (no counterpart in the reference). For callers that cannot
 * allocate device memory while they render: plugin hosts that give the renderer a fixed
 * device arena and account for every byte on the GPU themselves, and real-time frame loops
 * that forbid allocation inside a frame (cudaMalloc/cudaFree can synchronise the device and
 * stall the frame, and can fail once another allocator holds the memory). Accumulates
 * samples [first_sample, first_sample + count) of `p` into the caller's device buffer
 * `d_accum` (width*height float4 RGBA32F, row 0 = bottom, A unused; zero it before the first
 * call), in sample order; the sums are bit-identical to lf_frame_render's.
 * All wavefront state lives in one fixed device array of the library (30 MiB + 256 B, i.e.
 * 31.5 MB, on every GPU that loads it, held until exit): one tile (tile_width x tile_height,
 * or the whole frame) may have at most 131072 pixels, larger tiles are rejected with
 * LF_ERR_INVALID. The call makes no cudaMalloc/cudaFree and no allocating library call.
 * The first call on a device resolves the array's address (cudaGetSymbolAddress); make it
 * before any stream capture. Every call reuses the same array and clears the queue sizes,
 * status word and counters it keeps at the start: calls that overlap on the GPU (other
 * threads, other contexts on the same device) race. Returns after the GPU has finished. */
lf_status lf_render_noalloc(lf_scene* sc, const lf_render_params* p, int32_t first_sample, int32_t count,
                            void* d_accum);

/* ------------------------------------------------------------------ serving loop
 * No counterpart in the reference (one scene per GL context, one frame at a time). A
 * scheduler thread admits render jobs of registered scenes under a device-memory budget,
 * keeps scenes resident (uploading on admission, evicting idle scenes least recently used
 * first) and runs the sample passes of all admitted jobs in the same engine launches, so
 * jobs that arrive while others run start as soon as memory allows. A job's image is the
 * one lf_frame_render gives for the same scene, parameters and samples, bit for bit. */
typedef struct lf_server lf_server;

typedef struct lf_server_config
{
    uint64_t memory_budget;    /* device bytes: resident scenes, engine pool, accumulation and
                                  pass buffers (0 = 150 GiB) */
    int32_t paths_per_pass;    /* target paths per pass (0 = the engine pool size) */
    int32_t passes_per_job;    /* passes of one job in flight at once (0 = 2) */
} lf_server_config;

#define LF_JOB_QUEUED 0
#define LF_JOB_RUNNING 1
#define LF_JOB_DONE 2
#define LF_JOB_FAILED 3

typedef struct lf_job_info
{
    int32_t state;             /* LF_JOB_* */
    int32_t samples_done;      /* samples accumulated so far */
    double submit_ms, start_ms, finish_ms;   /* server clock: ms since lf_server_create */
} lf_job_info;

typedef struct lf_server_stats
{
    uint64_t jobs_submitted, jobs_done;
    uint64_t paths, ext_rays, shadow_rays;
    uint64_t scene_uploads, scene_evictions;
    uint64_t device_bytes;     /* what the budget counts now */
    int32_t scenes_resident, jobs_running, jobs_queued;
} lf_server_stats;

lf_status lf_server_create(lf_ctx* c, const lf_server_config* cfg, lf_server** out);
/* Registers a scene by its flat arrays; the arrays must stay valid until the scene is
 * removed (they are uploaded again after an eviction). */
lf_status lf_server_add_scene(lf_server* s, const lf_scene_view* v, int64_t* scene_id);
/* LF_ERR_STATE while queued or running jobs use the scene. */
lf_status lf_server_remove_scene(lf_server* s, int64_t scene_id);
/* Queues `spp` samples of `p` (samples 0 .. spp-1). LF_ERR_BUDGET if the job could never fit
 * the budget. */
lf_status lf_server_submit(lf_server* s, int64_t scene_id, const lf_render_params* p, int32_t spp, int64_t* job_id);
lf_status lf_server_job_info(lf_server* s, int64_t job_id, lf_job_info* out);
/* Waits until the job is done or failed; LF_ERR_TIMEOUT after timeout_ms (< 0: no limit). */
lf_status lf_server_wait(lf_server* s, int64_t job_id, int32_t timeout_ms);
/* Accumulated radiance sum of a done job, RGB32F, row 0 = bottom. */
lf_status lf_server_read(lf_server* s, int64_t job_id, float* rgb);
/* Frees a finished job's buffers (queued jobs are cancelled; running ones: LF_ERR_STATE). */
lf_status lf_server_release_job(lf_server* s, int64_t job_id);
lf_status lf_server_get_stats(lf_server* s, lf_server_stats* out);
/* Stops the scheduler after the running jobs finish; queued jobs are dropped. */
lf_status lf_server_destroy(lf_server* s);

/* ------------------------------------------------------------------ learned path guiding
 * No counterpart in the reference (directions come from DisneySample only). A hash-grid +
 * MLP model (8 levels x 4 FP16 features, 64-64-64-64-48 ReLU network with FP16 weights and
 * FP32 accumulation on the tensor cores) maps (position, outgoing direction, normal) to an
 * 8-lobe von Mises-Fisher mixture over incident directions. Trained online with Adam on
 * directions the tracer sampled, weighted by the luminance they carried over their pdf.
 * Training sample / query record: 16 floats = position xyz, outgoing direction xyz, normal
 * xyz, sampled direction xyz, weight, 3 unused. Parameter arrays: 15360 weights (W1 64x64,
 * W2, W3, W4 48x64, each [out][in]) and 8 x 16384 x 4 grid values. */
typedef struct lf_guide lf_guide;

#define LF_GUIDE_WEIGHTS 15360
#define LF_GUIDE_GRID_PARAMS (8 * 16384 * 4)
#define LF_GUIDE_SAMPLE_FLOATS 16
#define LF_GUIDE_MIX_FLOATS 40 /* per lobe: mu xyz, kappa, cumulative lobe weight */

/* Positions are normalised to the box [scene_lo, scene_hi]; parameters start from `seed`. */
lf_status lf_guide_create(lf_ctx* c, const float scene_lo[3], const float scene_hi[3], uint64_t seed,
                          lf_guide** out);
lf_status lf_guide_release(lf_guide* g);
/* FP32 master copies of the parameters (host buffers of LF_GUIDE_WEIGHTS and
 * LF_GUIDE_GRID_PARAMS floats); setting them also refreshes the FP16 working copies. */
lf_status lf_guide_get_params(lf_guide* g, float* weights, float* grid);
lf_status lf_guide_set_params(lf_guide* g, const float* weights, const float* grid);
/* Loss (mean over the n samples) and its gradients, without changing the parameters. */
lf_status lf_guide_gradients(lf_guide* g, const float* samples, int32_t n, float* dweights, float* dgrid,
                             float* loss);
/* One Adam step (beta 0.9 / 0.99) on n samples in host memory (loss optional) or device memory. */
lf_status lf_guide_train(lf_guide* g, const float* samples, int32_t n, float lr, float* loss);
lf_status lf_guide_train_device(lf_guide* g, const float* d_samples, int32_t n, float lr);
/* Mixture per query (n x LF_GUIDE_MIX_FLOATS, may be NULL) and its pdf at the record's
 * direction (n floats, may be NULL). */
lf_status lf_guide_eval(lf_guide* g, const float* queries, int32_t n, float* mix, float* pdf);
/* The guide's MLP on the tcgen05 tensor cores (1): inference (lf_guide_eval, guided
 * rendering) and training (lf_guide_train*, lf_guide_gradients) in 128-sample tiles, FP16
 * operands from shared memory, FP32 accumulators in tensor memory (default); or the warp-level
 * mma.sync kernels (0). Same encoding and FP16 roundings; the FP32 sums differ only in
 * summation order. */
lf_status lf_guide_set_tensor_path(lf_guide* g, int32_t tcgen05);
/* Guided rendering of a frame (g = NULL detaches): at every surface hit a direction comes from
 * the guide's mixture with probability `alpha` and from DisneySample otherwise, weighted by
 * one-sample MIS so the estimator stays unbiased; next-event MIS uses the same combined pdf.
 * Guided frames run the per-batch pipeline in batches of lf_frame_set_batch samples; every
 * `train_every`-th batch (0 = never) records its path vertices and then trains the guide with
 * Adam (learning rate `lr`) on the directions they sampled. The guide must outlive the frame's
 * renders. */
lf_status lf_frame_set_guide(lf_frame* f, lf_guide* g, float alpha, int32_t train_every, float lr);
/* Adam steps and training samples used by the frame's guide so far. */
lf_status lf_frame_guide_stats(lf_frame* f, uint64_t* steps, uint64_t* samples);

#ifdef __cplusplus
}
#endif

#endif
