// Post-process (postprocess.glsl:26-171 with TiledRenderer's uniforms, TiledRenderer.cpp:540-552):
// mean of the accumulated radiance (optionally with chromatic aberration), one of the seven
// tone maps with the shader's gamma, optional vignette, then the 8-bit framebuffer conversion
// (clamp to [0, 1], round to nearest) that GetOutputBuffer reads back. The accumulation buffer
// is sampled as the shader's GL_LINEAR / GL_REPEAT texture, with the filtering contract of the
// environment map (texel centres at +0.5, float weights).
#include "lf_internal.h"

#include "../lf_contract.h"

namespace lfd
{
namespace
{
struct PostParams
{
    int tonemap;
    int useCA, useCADistortion, useVignette, preview;
    float caDistance, caP1, caP2, caP3, vignetteIntensity, vignettePower;
    float invSamples;
};

__device__ __forceinline__ int wrapi(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

// texture(pathTraceTexture, uv): bilinear, GL_REPEAT, channel c of the RGB sums.
__device__ __forceinline__ float tex_bilinear(const float4* t, int w, int h, float u, float v, int c)
{
    const float xf = u * (float)w - 0.5f, yf = v * (float)h - 0.5f;
    const float fx0 = floorf(xf), fy0 = floorf(yf);
    const float a = xf - fx0, b = yf - fy0;
    const int x0 = wrapi((int)fx0, w), x1 = wrapi((int)fx0 + 1, w);
    const int y0 = wrapi((int)fy0, h), y1 = wrapi((int)fy0 + 1, h);
    auto at = [&](int x, int y) {
        const float4 p = t[(size_t)y * w + x];
        return c == 0 ? p.x : (c == 1 ? p.y : p.z);
    };
    const float ia = 1.0f - a, ib = 1.0f - b;
    const float top = at(x0, y0) * ia + at(x1, y0) * a;
    const float bot = at(x0, y1) * ia + at(x1, y1) * a;
    return top * ib + bot * b;
}

__device__ __forceinline__ float distance2(float ax, float ay, float bx, float by)
{
    const float dx = ax - bx, dy = ay - by;
    return sqrtf(dx * dx + dy * dy);
}

__device__ __forceinline__ float clamp01(float x) { return lfc::clamp_g(x, 0.0f, 1.0f); }

__device__ void tonemap(int idx, float c[4])
{
    const float g = 1.0f / 2.2f;
    if (idx == 1)
    {
        // tonemap(c, 2): c * 1.0 / (1.0 + luminance / limit)
        const float lum = 0.3f * c[0] + 0.6f * c[1] + 0.1f * c[2];
        const float den = 1.0f + lum / 2.0f;
        for (int k = 0; k < 4; ++k) c[k] = lfc::pow_c(c[k] * 1.0f / den, g);
    }
    else if (idx == 2)
    {
        const float a = 2.51f, b = 0.03f, y = 2.43f, d = 0.59f, e = 0.14f;
        for (int k = 0; k < 4; ++k)
            c[k] = lfc::pow_c(clamp01((c[k] * (a * c[k] + b)) / (c[k] * (y * c[k] + d) + e)), g);
    }
    else if (idx == 3)
    {
        for (int k = 0; k < 4; ++k) c[k] = lfc::pow_c(clamp01(c[k] / (c[k] + 1.0f)), g);
    }
    else if (idx == 4)
    {
        const float a = 1.2295f, b = 0.3135f, y = 1.1935f, d = 0.4655f, e = 0.073f;
        for (int k = 0; k < 4; ++k)
        {
            float v = lfc::pow_c((c[k] * (c[k] * (a * c[k] + b) + y * d) / (c[k] * (y * c[k] + d) + e)), 1.7f);
            if (k < 3) v = lfc::pow_c(v, 1.0f / 0.8f);
            v = v * 0.8f;
            c[k] = lfc::pow_c(clamp01(v), g);
        }
    }
    else if (idx == 5)
    {
        for (int k = 0; k < 4; ++k)
        {
            const float v = lfc::fmax_g(0.0f, c[k] - 0.004f);
            c[k] = (v * (6.2f * v + 0.5f)) / (v * (6.2f * v + 1.7f) + 0.06f);
        }
    }
    else if (idx == 6)
    {
        const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
        for (int k = 0; k < 4; ++k)
        {
            const float v = ((c[k] * (A * c[k] + C * B) + D * E) / (c[k] * (A * c[k] + B) + D * F)) - E / F;
            c[k] = lfc::pow_c(v, g) * 1.75f;
        }
    }
}
}

__global__ void postprocess_kernel(const float4* accum, int W, int H, PostParams P, uchar4* out8, float4* outf)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < W * H; i += gridDim.x * blockDim.x)
    {
        const int x = i % W, y = i / W;
        const float u = ((float)x + 0.5f) / (float)W, v = ((float)y + 0.5f) / (float)H;
        float c[4];
        if (!P.preview && P.useCA)
        {
            float offset = P.caDistance;
            const float dist = 0.0f + lfc::pow_c(distance2(u, v, P.caP3, P.caP3), P.caP1) * P.caP2;
            float su, sv;
            if (P.useCADistortion)
                su = sv = offset * dist;
            else
            {
                offset = offset * 0.025f;
                su = sv = offset * P.caP2;
            }
            c[0] = tex_bilinear(accum, W, H, u + su, v + sv, 0) * P.invSamples;
            c[1] = tex_bilinear(accum, W, H, u, v, 1) * P.invSamples;
            c[2] = tex_bilinear(accum, W, H, u - su, v - sv, 2) * P.invSamples;
            c[3] = 0.0f;
        }
        else
        {
            for (int k = 0; k < 3; ++k) c[k] = tex_bilinear(accum, W, H, u, v, k) * P.invSamples;
            c[3] = 0.0f;
        }
        tonemap(P.tonemap, c);
        if (P.useVignette)
        {
            const float dist = 1.0f - lfc::pow_c(distance2(u, v, 0.5f, 0.5f), P.vignettePower) * P.vignetteIntensity;
            for (int k = 0; k < 4; ++k) c[k] = c[k] * dist;
        }
        if (outf) outf[i] = make_float4(c[0], c[1], c[2], c[3]);
        if (out8)
        {
            unsigned char q[3];
            for (int k = 0; k < 3; ++k) q[k] = (unsigned char)rintf(clamp01(c[k]) * 255.0f);
            out8[i] = make_uchar4(q[0], q[1], q[2], 255);
        }
    }
}
}

using namespace lfrt;

extern "C" lf_status lf_frame_postprocess(lf_frame* f, const lf_post_params* pp, int32_t samples, uint8_t* rgb8,
                                          float* rgbf)
{
    if (!f || !pp || samples <= 0 || (!rgb8 && !rgbf) || pp->tonemap < 0 || pp->tonemap > 6) return LF_ERR_INVALID;
    lf_ctx* c = f->ctx;
    std::lock_guard<std::recursive_mutex> lk(c->mu);
    cudaSetDevice(c->device);
    const size_t pix = (size_t)f->W * f->H;
    uchar4* d8 = nullptr;
    float4* df = nullptr;
    cudaError_t e = cudaSuccess;
    if (rgb8) e = cudaMallocAsync((void**)&d8, pix * sizeof(uchar4), c->stream);
    if (e == cudaSuccess && rgbf) e = cudaMallocAsync((void**)&df, pix * sizeof(float4), c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "post-process buffers");
    PostParams P;
    P.tonemap = pp->tonemap;
    P.useCA = pp->use_ca;
    P.useCADistortion = pp->use_ca_distortion;
    P.useVignette = pp->use_vignette;
    P.preview = pp->preview;
    P.caDistance = pp->ca_distance;
    P.caP1 = pp->ca_p1;
    P.caP2 = pp->ca_p2;
    P.caP3 = pp->ca_p3;
    P.vignetteIntensity = pp->vignette_intensity;
    P.vignettePower = pp->vignette_power;
    P.invSamples = 1.0f / (float)samples;
    const int B = 256;
    const int grid = (int)std::min<size_t>((pix + B - 1) / B, 152 * 16);
    postprocess_kernel<<<grid, B, 0, c->stream>>>(f->accum, f->W, f->H, P, d8, df);
    e = cudaGetLastError();
    std::vector<uchar4> h8(rgb8 ? pix : 0);
    std::vector<float4> hf(rgbf ? pix : 0);
    if (e == cudaSuccess && rgb8) e = cudaMemcpyAsync(h8.data(), d8, pix * sizeof(uchar4), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && rgbf) e = cudaMemcpyAsync(hf.data(), df, pix * sizeof(float4), cudaMemcpyDeviceToHost, c->stream);
    if (d8) cudaFreeAsync(d8, c->stream);
    if (df) cudaFreeAsync(df, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "post-process");
    for (size_t i = 0; i < pix; ++i)
    {
        if (rgb8)
        {
            rgb8[i * 3 + 0] = h8[i].x;
            rgb8[i * 3 + 1] = h8[i].y;
            rgb8[i * 3 + 2] = h8[i].z;
        }
        if (rgbf)
        {
            rgbf[i * 3 + 0] = hf[i].x;
            rgbf[i * 3 + 1] = hf[i].y;
            rgbf[i * 3 + 2] = hf[i].z;
        }
    }
    return check_device(c);
}
