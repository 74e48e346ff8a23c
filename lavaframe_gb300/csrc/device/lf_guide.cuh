// Learned path guiding: the model shared by the training and inference kernels (lf_guide.cu)
// and the guided path kernels. No reference counterpart: the reference samples directions from
// the BSDF only (disney.glsl:128-225).
//
// Model: hash-grid encoding of the position (8 levels x 4 FP16 features) plus one-blob
// encodings of the outgoing direction and the shading normal (32 values) -> MLP
// 64-64-64-64-48 with ReLU, FP16 weights, FP32 accumulation on the tensor cores -> 8 von
// Mises-Fisher lobes (outputs 0..39: mu_raw xyz, kappa_raw, logit per lobe).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace lfd
{
namespace guide
{
constexpr int kLevels = 8;
constexpr int kFeatures = 4;
constexpr int kLog2T = 14;
constexpr int kT = 1 << kLog2T;
constexpr int kBlobBins = 8;
constexpr int kLobes = 8;
constexpr int kIn = 64;
constexpr int kHidden = 64;
constexpr int kOut = 48;          // 40 used
constexpr int kW1 = 0, kW2 = 64 * 64, kW3 = 2 * 64 * 64, kW4 = 3 * 64 * 64;
constexpr int kWeights = 3 * 64 * 64 + kOut * 64;   // 15360
constexpr int kGridParams = kLevels * kT * kFeatures;
constexpr int kSampleFloats = 16;  // p xyz, wo xyz, n xyz, direction xyz, weight, 3 unused
constexpr int kMixFloats = 40;     // per query: per lobe mu xyz, kappa, cumulative weight
constexpr float kBlobSigma = 1.0f / 8.0f;

struct Net
{
    const __half* W;      // [W1 | W2 | W3 | W4], each [out][in] row-major
    const __half* grid;   // [level][entry][feature]
    int res[kLevels];     // grid resolution per level
    float lo[3];          // scene box -> [0, 1]^3
    float invExt[3];
};

// Level l: the 8 corner entries and trilinear weights of position p01 in [0, 1]^3 (corner c =
// dx + 2 dy + 4 dz). A corner (x, y, z) of a level with n = res + 1 vertices per axis has the
// dense entry x + y n + z n^2 while n^3 fits the table, else the spatial hash
// (x * 1) ^ (y * 2654435761) ^ (z * 805459861) mod T (uint32 arithmetic); both are formed from
// per-axis terms. The weights are (wx * wy) * wz.
__device__ __forceinline__ void grid_corners(int res, const float p01[3], uint32_t idx[8], float w[8])
{
    uint32_t i0[3];
    float fr[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        const float q = fminf(fmaxf(p01[a], 0.f), 1.f) * (float)res;
        int i = (int)floorf(q);
        i = i > res - 1 ? res - 1 : i;
        i0[a] = (uint32_t)i;
        fr[a] = q - (float)i;
    }
    const uint32_t n = (uint32_t)res + 1u;
    uint32_t hx[2], hy[2], hz[2];
    if ((unsigned long long)n * n * n <= (unsigned long long)kT)
    {
        // dense: x + y n + z n^2
        hx[0] = i0[0];
        hy[0] = i0[1] * n;
        hz[0] = i0[2] * n * n;
        hx[1] = hx[0] + 1u;
        hy[1] = hy[0] + n;
        hz[1] = hz[0] + n * n;
#pragma unroll
        for (int c = 0; c < 8; ++c) idx[c] = hx[c & 1] + hy[(c >> 1) & 1] + hz[c >> 2];
    }
    else
    {
        // spatial hash: (x * 1) ^ (y * 2654435761) ^ (z * 805459861) mod T
        hx[0] = i0[0];
        hy[0] = i0[1] * 2654435761u;
        hz[0] = i0[2] * 805459861u;
        hx[1] = hx[0] + 1u;
        hy[1] = hy[0] + 2654435761u;
        hz[1] = hz[0] + 805459861u;
#pragma unroll
        for (int c = 0; c < 8; ++c) idx[c] = (hx[c & 1] ^ hy[(c >> 1) & 1] ^ hz[c >> 2]) & (uint32_t)(kT - 1);
    }
    const float wx[2] = {1.f - fr[0], fr[0]}, wy[2] = {1.f - fr[1], fr[1]}, wz[2] = {1.f - fr[2], fr[2]};
    float wxy[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) wxy[c] = wx[c & 1] * wy[c >> 1];
#pragma unroll
    for (int c = 0; c < 8; ++c) w[c] = wxy[c & 3] * wz[c >> 2];
}

// The 4 features of level l at p01: trilinear sum of the corner entries (FP16 table, FP32
// fused multiply-adds in corner order).
__device__ __forceinline__ void level_features(const Net& net, int l, const float p01[3], float acc[4])
{
    uint32_t idx[8];
    float w[8];
    grid_corners(net.res[l], p01, idx, w);
    const __half* tab = net.grid + (size_t)l * kT * kFeatures;
    uint2 v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) v[c] = *reinterpret_cast<const uint2*>(tab + (size_t)idx[c] * kFeatures);
#pragma unroll
    for (int f = 0; f < 4; ++f) acc[f] = 0.f;
#pragma unroll
    for (int c = 0; c < 8; ++c)
    {
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&v[c].x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&v[c].y));
        acc[0] = __fmaf_rn(w[c], a.x, acc[0]);
        acc[1] = __fmaf_rn(w[c], a.y, acc[1]);
        acc[2] = __fmaf_rn(w[c], b.x, acc[2]);
        acc[3] = __fmaf_rn(w[c], b.y, acc[3]);
    }
}

__device__ __forceinline__ void sph01(float x, float y, float z, float* th, float* ph)
{
    *th = acosf(fminf(fmaxf(z, -1.f), 1.f)) * 0.318309886f;
    *ph = (atan2f(y, x) + 3.14159265f) * 0.159154943f;
}

__device__ __forceinline__ float blob(float s, int k)
{
    const float c = ((float)k + 0.5f) * (1.0f / kBlobBins);
    const float u = (s - c) * (1.0f / kBlobSigma);
    return __expf(-0.5f * u * u);
}

// Feature f (0..63) of a query: 0..31 grid (level-major), 32..63 one-blob bins.
__device__ __forceinline__ float grid_feature(const Net& net, const float p01[3], int l, int f)
{
    uint32_t idx[8];
    float w[8];
    grid_corners(net.res[l], p01, idx, w);
    const __half* tab = net.grid + (size_t)l * kT * kFeatures;
    float acc = 0.f;
    for (int c = 0; c < 8; ++c) acc = __fmaf_rn(w[c], __half2float(tab[idx[c] * kFeatures + f]), acc);
    return acc;
}

__device__ __forceinline__ void position01(const Net& net, const float p[3], float p01[3])
{
    for (int a = 0; a < 3; ++a) p01[a] = (p[a] - net.lo[a]) * net.invExt[a];
}

// von Mises-Fisher lobe of the sampling mixture from raw outputs (the oracle's `pdf`): the mean
// direction is normalised exactly (a raw vector of zero length gives +z), so that mix_sample
// draws unit directions whose density is exactly mix_pdf. The training loss keeps the
// regularised mean mu_raw / sqrt(|mu_raw|^2 + 1e-6) (sample_loss_grad); the two differ only for
// near-zero raw vectors, whose lobes would otherwise sample directions of less than unit length.
__device__ __forceinline__ void lobe_params(const float* o5, float mu[3], float* kappa)
{
    const float len = sqrtf(o5[0] * o5[0] + o5[1] * o5[1] + o5[2] * o5[2]);
    if (len > 1e-30f)
    {
        const float inv = 1.f / len;
        mu[0] = o5[0] * inv;
        mu[1] = o5[1] * inv;
        mu[2] = o5[2] * inv;
    }
    else
    {
        mu[0] = 0.f;
        mu[1] = 0.f;
        mu[2] = 1.f;
    }
    *kappa = __expf(fminf(fmaxf(o5[3], -3.f), 7.f));
}

__device__ __forceinline__ float vmf_norm(float k) { return __fdividef(k, 6.28318531f * (1.f - __expf(-2.f * k))); }

// Mixture pdf from the compact per-query form (mu xyz, kappa, cumulative weight per lobe).
__device__ __forceinline__ float mix_pdf(const float* mix, float wx, float wy, float wz)
{
    float p = 0.f, prev = 0.f;
    for (int i = 0; i < kLobes; ++i)
    {
        const float* q = mix + 5 * i;
        const float pi = q[4] - prev;
        prev = q[4];
        const float dot = q[0] * wx + q[1] * wy + q[2] * wz;
        p += pi * vmf_norm(q[3]) * __expf(q[3] * (dot - 1.f));
    }
    return p;
}

// Loss of one sample and d loss / d outputs (without the 1/N of the mean), clamped to the
// FP16 range. Mirrors oracle/guide.py loss_and_grads.
__device__ __forceinline__ float sample_loss_grad(const float* out, const float dir[3], float weight, float* d_out)
{
    float mu[kLobes][3], kap[kLobes], f[kLobes], dot[kLobes], pi[kLobes], nrm[kLobes];
    float mx = -1e30f;
    for (int i = 0; i < kLobes; ++i) mx = fmaxf(mx, out[5 * i + 4]);
    float es = 0.f;
    for (int i = 0; i < kLobes; ++i)
    {
        pi[i] = __expf(out[5 * i + 4] - mx);
        es += pi[i];
    }
    float q = 0.f;
    for (int i = 0; i < kLobes; ++i)
    {
        pi[i] /= es;
        const float* o = out + 5 * i;
        nrm[i] = sqrtf(o[0] * o[0] + o[1] * o[1] + o[2] * o[2] + 1e-6f);
        mu[i][0] = o[0] / nrm[i];
        mu[i][1] = o[1] / nrm[i];
        mu[i][2] = o[2] / nrm[i];
        kap[i] = __expf(fminf(fmaxf(o[3], -3.f), 7.f));
        dot[i] = mu[i][0] * dir[0] + mu[i][1] * dir[1] + mu[i][2] * dir[2];
        f[i] = vmf_norm(kap[i]) * __expf(kap[i] * (dot[i] - 1.f));
        q += pi[i] * f[i];
    }
    const float dq = -weight / (q + 1e-12f);
    float gpi_avg = 0.f;
    for (int i = 0; i < kLobes; ++i) gpi_avg += pi[i] * (dq * f[i]);
    for (int i = 0; i < kLobes; ++i)
    {
        const float* o = out + 5 * i;
        const float gpi = dq * f[i];
        const float glg = pi[i] * (gpi - gpi_avg);
        const float gf = dq * pi[i];
        const float e2 = __expf(-2.f * kap[i]);
        const float dlogf = 1.f / kap[i] - 2.f * e2 / (1.f - e2) + (dot[i] - 1.f);
        const float gk = gf * f[i] * dlogf;
        const float gkr = (o[3] > -3.f && o[3] < 7.f) ? gk * kap[i] : 0.f;
        const float gm = gf * f[i] * kap[i];
        const float gmx = gm * dir[0], gmy = gm * dir[1], gmz = gm * dir[2];
        const float proj = gmx * mu[i][0] + gmy * mu[i][1] + gmz * mu[i][2];
        float* d = d_out + 5 * i;
        d[0] = (gmx - mu[i][0] * proj) / nrm[i];
        d[1] = (gmy - mu[i][1] * proj) / nrm[i];
        d[2] = (gmz - mu[i][2] * proj) / nrm[i];
        d[3] = gkr;
        d[4] = glg;
    }
    for (int k = 0; k < 40; ++k) d_out[k] = fminf(fmaxf(d_out[k], -60000.f), 60000.f);
    return -weight * __logf(q + 1e-12f);
}

// Mixture of every query record (16 floats: position, outgoing direction, normal, ...) into
// mix (kMixFloats each); the count is read from nDev. Launched on `st`; returns a CUDA error.
int launch_infer(const Net& net, const float* queries, const int* nDev, int cap, float* mix, cudaStream_t st);
// The same on the tcgen05 tensor cores (lf_guide_tc.cu): tiles of 128 queries, accumulators in
// TMEM. A bounded wait that runs out sets LF_DEVERR_GUIDE_TIMEOUT in `status`.
int launch_infer_tc(const Net& net, const float* queries, const int* nDev, int cap, float* mix, uint32_t* status,
                    cudaStream_t st);
// One training pass on tcgen05 (lf_guide_tc.cu): the per-sample weight and grid gradients of n
// sample records summed into gW / gGrid and the loss into `loss`, as the warp-level kernel.
int launch_train_tc(const Net& net, const float* samples, int n, float* gW, float* gGrid, float* loss, uint32_t* status,
                    cudaStream_t st);

// Samples a direction from the compact mixture with uniforms u0 (lobe), u1, u2.
__device__ __forceinline__ void mix_sample(const float* mix, float u0, float u1, float u2, float* wx, float* wy,
                                           float* wz)
{
    int i = 0;
    while (i < kLobes - 1 && u0 > mix[5 * i + 4]) ++i;
    const float* q = mix + 5 * i;
    const float k = q[3];
    // w = 1 + log(u1 + (1 - u1) e^{-2k}) / k  (cosine to the lobe axis)
    const float w = fminf(fmaxf(1.f + __logf(u1 + (1.f - u1) * __expf(-2.f * k)) / k, -1.f), 1.f);
    const float s = sqrtf(fmaxf(0.f, 1.f - w * w));
    float sp, cp;
    __sincosf(6.28318531f * u2, &sp, &cp);
    // frame around mu
    const float mx = q[0], my = q[1], mz = q[2];
    const float sign = mz >= 0.f ? 1.f : -1.f;
    const float a = -1.f / (sign + mz);
    const float b = mx * my * a;
    const float tx = 1.f + sign * mx * mx * a, ty = sign * b, tz = -sign * mx;
    const float bx = b, by = sign + my * my * a, bz = -my;
    *wx = s * cp * tx + s * sp * bx + w * mx;
    *wy = s * cp * ty + s * sp * by + w * my;
    *wz = s * cp * tz + s * sp * bz + w * mz;
}
}
}
