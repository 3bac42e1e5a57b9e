// enb_adjoint.cu -- adjoint of the float enfuse (no counterpart in the
// reference): gradients of a mean-squared loss against a target image with
// respect to the exposure-weight parameters (optimum, width), the weight
// coefficients (exposure, saturation, contrast) and a per-exposure additive
// logit map.
//
// The differentiated forward model is enfuseMain's float path
// (src/enfuse.h:1217-1617) with continuous masks: per exposure the weight
// w_k = W_exp f((y - opt) / width') + W_con sigma + W_sat s of
// src/enfuse.h:623-829, w~_k = w_k exp(a_k) with the logit map a_k,
// m_k = w~_k / sum_j w~_j (the soft mask, src/enfuse.h:1526-1535, without
// its 9.15 fixed-point quantisation), the mask Gaussian pyramids and image
// Laplacian pyramids of the opaque images (src/pyramid.h:1468-1747), the
// merge R[l] = sum_k LP_k[l] M_k[l] (src/enfuse.h:601-620, 1576-1588), the
// collapse (src/pyramid.h:1758-1784) and the mapping back
// (src/fixmath.h:320-329).  Entropy weights, hard masks and wrap-around are
// not differentiated.
//
// Backward, for each level from the output down the pyramids:
//   gC0 = dL/dout phi'(C0); gR[l] = gC[l], gC[l+1] = E^T gC[l]  (collapse)
//   gM_k[l] = sum_c gR[l]_c LP_k[l]_c                          (merge)
//   gm_k = gM_k[0] + Rd^T(gM_k[1] + Rd^T(...))                  (mask pyramid)
//   gw~_k = (gm_k - sum_j gm_j m_j) / S, ga_k = gw~_k w~_k     (normalisation)
//   gw_k = gw~_k exp(a_k) -> d/d(opt, width, W_exp, W_sat, W_con)
// where E^T and Rd^T are the transposes of the expand and of the
// normalised (opaque) reduce, written as gathers with the forward
// operators' per-position weights and divisors.
//
// The image pyramids hold G - 1 rather than the log-mapped G itself
// (log1p(v) for v >= 0, v / (1 - v) below): reduce and expand are
// normalised, so every level and every Laplacian but the top one is the
// same, the collapse yields C - 1 and the top level's Laplacian differs by
// the same amount for every exposure, which the normalisation's backward
// cancels.  In FP32 this keeps the fine Laplacians, small differences of
// values near 1 to 1.7, a few times more accurate.
#include <cuda_runtime.h>
#include <stdint.h>

#include "enb_device.cuh"
#include "enb_fweights.cuh"
#include "enb_internal.h"

namespace enb {

namespace {

inline dim3 row_grid(int w, int h) { return dim3((unsigned)((w + 255) / 256), (unsigned)h); }
inline double npix(int w, int h) { return (double)w * (double)h; }

// In-image weight sum of the 5-tap binomial centred at 2I (the reduce's
// divisor factor along one axis, opaque, no wrap).
__device__ __forceinline__ int reduce_den1(int I, int n)
{
    const int W5[5] = {1, 4, 6, 4, 1};
    int d = 0;
#pragma unroll
    for (int t = -2; t <= 2; ++t) {
        const int x = 2 * I + t;
        d += (x >= 0 && x < n) ? W5[t + 2] : 0;
    }
    return d;
}

}  // namespace

// ---- forward pieces ---------------------------------------------------------

// w~_k = w_k exp(a_k), m_k = w~_k / S (S = sum_k w~_k; 1/K where S == 0).
__global__ void __launch_bounds__(256) k_adj_norm(int K, const float* __restrict__ w, const float* __restrict__ a,
                                                  float* __restrict__ m, int64_t pitch, int64_t plane, int width)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= width) {
        return;
    }
    const int64_t o = (int64_t)blockIdx.y * pitch + x;
    float S = 0.0f;
    for (int k = 0; k < K; ++k) {
        S += w[k * plane + o] * (a ? expf(a[k * plane + o]) : 1.0f);
    }
    for (int k = 0; k < K; ++k) {
        const float wt = w[k * plane + o] * (a ? expf(a[k * plane + o]) : 1.0f);
        m[k * plane + o] = S > 0.0f ? wt / S : 1.0f / (float)K;
    }
}

// R[l] (+)= LP[l] * M[l] over the three planes.
__global__ void __launch_bounds__(256) k_adj_merge(const float* __restrict__ lp, const float* __restrict__ mk,
                                                   float* __restrict__ r, int64_t pitch, int64_t plane, int w,
                                                   int first)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= w) {
        return;
    }
    const int64_t o = (int64_t)blockIdx.y * pitch + x;
    const float mv = mk[o];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float v = lp[c * plane + o] * mv;
        r[c * plane + o] = first ? v : r[c * plane + o] + v;
    }
}

// Level 0 of an image pyramid in the offset form G - 1 (see above) from
// interleaved float RGB.
__global__ void __launch_bounds__(256) k_adj_to_pyramid(FloatPixelView img, float* __restrict__ g, int64_t pitch,
                                                        int64_t plane)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= img.w) {
        return;
    }
    const int y = blockIdx.y;
    const float* px = img.p + (int64_t)y * img.pitch + (int64_t)x * img.stride;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float v = px[c];
        g[c * plane + (int64_t)y * pitch + x] = v >= 0.0f ? log1pf(v) : __fdiv_rn(v, 1.0f - v);
    }
}

// out = phi(C0) with C0 - 1 given (expm1 above 0, u / (1 + u) below);
// loss += (out - T)^2; gC0 = 2 (out - T) / N * phi'(C0).
__global__ void __launch_bounds__(256) k_adj_loss(const float* __restrict__ c0, int64_t pitch, int64_t plane,
                                                  const float* __restrict__ tgt, int64_t tpitch, int tstride,
                                                  float* __restrict__ out, int64_t opitch, int ostride,
                                                  float* __restrict__ g0, int w, float inv_n, double* loss)
{
    __shared__ double part[8];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (x < w) {
        const int y = blockIdx.y;
        const int64_t o = (int64_t)y * pitch + x;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float u = c0[c * plane + o];  // C0 - 1
            const float ov = u >= 0.0f ? expm1f(u) : __fdiv_rn(u, 1.0f + u);
            const float d = ov - tgt[(int64_t)y * tpitch + (int64_t)x * tstride + c];
            l += (double)d * d;
            const float dphi = u >= 0.0f ? expf(u) : 1.0f / ((1.0f + u) * (1.0f + u));
            g0[c * plane + o] = 2.0f * d * inv_n * dphi;
            if (out) {
                out[(int64_t)y * opitch + (int64_t)x * ostride + c] = ov;
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        l += __shfl_down_sync(0xffffffffu, l, off);
    }
    if ((threadIdx.x & 31) == 0) {
        part[threadIdx.x >> 5] = l;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
            s += part[i];
        }
        atomicAdd(loss, s);
    }
}

// ---- transposed operators -------------------------------------------------------

// gc = E^T g: coarse (i, j) gathers from the fine pixels whose expand uses it
// (taps (X >> 1) - 1 .. (X >> 1) + 1 with expand_hweights / expand_vweights,
// no wrap).
__global__ void __launch_bounds__(256) k_expand_T(const float* __restrict__ g, int64_t gpitch, int64_t gplane, int fw,
                                                  int fh, float* __restrict__ gc, int64_t cpitch, int64_t cplane,
                                                  int cw, int ch, int C)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= cw) {
        return;
    }
    float acc[3] = {0.0f, 0.0f, 0.0f};
    for (int Y = max(2 * j - 2, 0); Y <= min(2 * j + 3, fh - 1); ++Y) {
        int vw[3], vden;
        expand_vweights(Y, ch, vw, vden);
        const int b = j - (Y >> 1) + 1;
        if (b < 0 || b > 2 || vw[b] == 0) {
            continue;
        }
        for (int X = max(2 * i - 2, 0); X <= min(2 * i + 3, fw - 1); ++X) {
            int hw[3], hden;
            expand_hweights(X, cw, fw, 0, hw, hden);
            const int a = i - (X >> 1) + 1;
            if (a < 0 || a > 2 || hw[a] == 0) {
                continue;
            }
            const float f = (float)(hw[a] * vw[b]) / (float)(hden * vden);
            for (int c = 0; c < C; ++c) {
                acc[c] += f * g[c * gplane + (int64_t)Y * gpitch + X];
            }
        }
    }
    for (int c = 0; c < C; ++c) {
        gc[c * cplane + (int64_t)j * cpitch + i] = acc[c];
    }
}

// acc[l] = sum_c gR[l]_c LP[l]_c + Rd^T(acc[l+1]): the mask pyramid's
// adjoint at one level.  Rd^T gathers from the coarse pixels (I, J) whose
// 5x5 window holds (x, y), with the forward's weights over its in-image
// divisor (opaque, no wrap).
__global__ void __launch_bounds__(256) k_adj_mask_level(const float* __restrict__ gr, const float* __restrict__ lp,
                                                        int64_t pitch, int64_t plane, int w, int h,
                                                        const float* __restrict__ nxt, int64_t npitch, int nw, int nh,
                                                        float* __restrict__ acc)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const int64_t o = (int64_t)y * pitch + x;
    float v = gr[o] * lp[o] + gr[plane + o] * lp[plane + o] + gr[2 * plane + o] * lp[2 * plane + o];
    if (nxt) {
        const int W5[5] = {1, 4, 6, 4, 1};
        float s = 0.0f;
        for (int J = max((y - 1) >> 1, 0); J <= min((y + 2) >> 1, nh - 1); ++J) {
            const int ty = y - 2 * J;
            if (ty < -2 || ty > 2) {
                continue;
            }
            const float vy = (float)W5[ty + 2] / (float)reduce_den1(J, h);
            for (int I = max((x - 1) >> 1, 0); I <= min((x + 2) >> 1, nw - 1); ++I) {
                const int tx = x - 2 * I;
                if (tx < -2 || tx > 2) {
                    continue;
                }
                s += vy * (float)W5[tx + 2] / (float)reduce_den1(I, w) * nxt[(int64_t)J * npitch + I];
            }
        }
        v += s;
    }
    acc[o] = v;
}

// ---- normalisation, logits and weight functions ---------------------------------

// gw~_k = (gm_k - sum_j gm_j m_j) / S; ga_k = gw~_k w~_k; gw_k = gw~_k exp(a_k).
__global__ void __launch_bounds__(256) k_adj_norm_bw(int K, const float* __restrict__ w, const float* __restrict__ a,
                                                     const float* __restrict__ gm, float* __restrict__ gw,
                                                     float* __restrict__ ga, int64_t pitch, int64_t plane, int width)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= width) {
        return;
    }
    const int64_t o = (int64_t)blockIdx.y * pitch + x;
    float S = 0.0f;
    for (int k = 0; k < K; ++k) {
        S += w[k * plane + o] * (a ? expf(a[k * plane + o]) : 1.0f);
    }
    if (!(S > 0.0f)) {
        for (int k = 0; k < K; ++k) {
            gw[k * plane + o] = 0.0f;
            if (ga) {
                ga[k * plane + o] = 0.0f;
            }
        }
        return;
    }
    float dot = 0.0f;
    for (int k = 0; k < K; ++k) {
        const float wt = w[k * plane + o] * (a ? expf(a[k * plane + o]) : 1.0f);
        dot += gm[k * plane + o] * (wt / S);
    }
    for (int k = 0; k < K; ++k) {
        const float e = a ? expf(a[k * plane + o]) : 1.0f;
        const float gwt = (gm[k * plane + o] - dot) / S;
        gw[k * plane + o] = gwt * e;
        if (ga) {
            ga[k * plane + o] = gwt * w[k * plane + o] * e;
        }
    }
}

// Derivative of the built-in exposure weight functions (src/exposure_weight.h:44-128).
__device__ __forceinline__ float exposure_dfdz(int fn, float z)
{
    switch (fn) {
    case ENB_EXP_LORENTZIAN: {
        const float q = 1.0f + 0.5f * z * z;
        return -z / (q * q);
    }
    case ENB_EXP_HALF_SINE: return fabsf(z) <= 1.57079632679489661923f ? -sinf(z) : 0.0f;
    case ENB_EXP_FULL_SINE: return fabsf(z) <= 3.14159265358979323846f ? -0.5f * sinf(z) : 0.0f;
    case ENB_EXP_BISQUARE: return fabsf(z) <= 1.0f ? -4.0f * z * z * z : 0.0f;
    default: return -z * expf(-0.5f * z * z);
    }
}

// Per pixel of exposure k: dL/dw_k times the partial derivatives of w_k,
// summed into d[0..4] = d/d(optimum, width, W_exp, W_sat, W_con).  A 16x16
// tile of the image (with the contrast window's halo) is staged in shared
// memory as the forward weight kernel stages it, and sigma is recomputed
// from it with the forward's arithmetic.
template <int CW>
__global__ void __launch_bounds__(256) k_adj_weights_bw(FloatPixelView img, const float* __restrict__ gw,
                                                        int64_t gpitch, FloatWeightParams wp, float inv_width,
                                                        float width, float w_exp, double* d)
{
    extern __shared__ __align__(16) unsigned char asmem[];
    __shared__ double part[5][8];
    const int halo = wp.contrast_window / 2;
    FloatWeightParams tp = wp;
    tp.repeat_slots = 0;
    const FTile t = ftile_carve(asmem, 16 + 2 * halo, 0);
    const int opaque = ftile_load(t, tp, img.p, img.pitch, img.stride, img.w, img.h, 3, nullptr, 0,
                                  blockIdx.x * 16 - halo, blockIdx.y * 16 - halo);
    const int lx = threadIdx.x % 16, ly = threadIdx.x / 16;
    const int x = blockIdx.x * 16 + lx, y = blockIdx.y * 16 + ly;
    // per pixel and per warp in float (a warp's sum of 32 terms: ~1e-6
    // relative), per block and across blocks in double
    float s[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (x < img.w && y < img.h) {
        const int ci = (ly + halo) * t.TW + (lx + halo);
        const float g = gw[(int64_t)y * gpitch + x];
        const float gray = t.gray[ci];
        // exposure: z = (y - opt) / width'; dz/dopt = -1/width', dz/dwidth = -z/width
        const float yv = __fdiv_rn(gray, wp.range);
        const float z = (yv - (wp.opt_hi + wp.opt_lo)) * inv_width;
        const float df = exposure_dfdz(wp.exp_function, z);
        s[0] = g * w_exp * df * (-inv_width);
        s[1] = g * w_exp * df * (-z / width);
        s[2] = g * exposure_f(wp, gray);
        // saturation (max_value 1.0)
        const int TT = t.TW * t.TW;
        const float r = t.raw[ci], gg = t.raw[TT + ci], b = t.raw[2 * TT + ci];
        const float mx = fmaxf(r, fmaxf(gg, b)), mn = fminf(r, fminf(gg, b));
        float sat = 0.0f;
        if (mx != mn) {
            const float sum = mx + mn, diff = mx - mn;
            sat = __fdiv_rn(diff, sum <= 1.0f ? sum : (1.0f - mx) + (1.0f - mn));
        }
        s[3] = g * sat;
        // contrast: the window's sample standard deviation (border strip 0)
        float sd = 0.0f;
        if (x >= halo && x < img.w - halo && y >= halo && y < img.h - halo) {
            sd = window_stddev<CW>(t, ci, halo, opaque != 0);
        }
        s[4] = g * sd;
    }
    for (int i = 0; i < 5; ++i) {
        for (int off = 16; off > 0; off >>= 1) {
            s[i] += __shfl_down_sync(0xffffffffu, s[i], off);
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int i = 0; i < 5; ++i) {
            part[i][threadIdx.x >> 5] = (double)s[i];
        }
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double tot = 0.0;
        for (int j = 0; j < (int)(blockDim.x >> 5); ++j) {
            tot += part[threadIdx.x][j];
        }
        atomicAdd(&d[threadIdx.x], tot);
    }
}

// ---- launchers ---------------------------------------------------------------------

cudaError_t launch_adj_norm(int K, const float* w, const float* a, float* m, int64_t pitch, int64_t plane, int width,
                            int height, cudaStream_t st)
{
    note_launch("adj_norm", npix(width, height) * K * (a ? 12.0 : 8.0));
    k_adj_norm<<<row_grid(width, height), 256, 0, st>>>(K, w, a, m, pitch, plane, width);
    return cudaGetLastError();
}

cudaError_t launch_adj_merge(const PlanarView& lp, const PlanarView& m, const PlanarView& r, int first, cudaStream_t st)
{
    note_launch("adj_merge", npix(lp.w, lp.h) * (12.0 + 4.0 + (first ? 12.0 : 24.0)));
    k_adj_merge<<<row_grid(lp.w, lp.h), 256, 0, st>>>((const float*)lp.p, (const float*)m.p, (float*)r.p, lp.pitch,
                                                      lp.plane, lp.w, first);
    return cudaGetLastError();
}

cudaError_t launch_adj_to_pyramid(const FloatPixelView& img, const PlanarView& g, cudaStream_t st)
{
    note_launch("adj_to_pyramid", npix(img.w, img.h) * (4.0 * img.stride + 12.0));
    k_adj_to_pyramid<<<row_grid(img.w, img.h), 256, 0, st>>>(img, (float*)g.p, g.pitch, g.plane);
    return cudaGetLastError();
}

cudaError_t launch_adj_loss(const PlanarView& c0, const float* tgt, int64_t tpitch, int tstride, float* out,
                            int64_t opitch, int ostride, const PlanarView& g0, double* loss, cudaStream_t st)
{
    note_launch("adj_loss", npix(c0.w, c0.h) * (12.0 + 12.0 + 12.0 + (out ? 12.0 : 0.0)));
    const float inv_n = (float)(1.0 / (3.0 * c0.w * (double)c0.h));
    k_adj_loss<<<row_grid(c0.w, c0.h), 256, 0, st>>>((const float*)c0.p, c0.pitch, c0.plane, tgt, tpitch, tstride, out,
                                                     opitch, ostride, (float*)g0.p, c0.w, inv_n, loss);
    return cudaGetLastError();
}

cudaError_t launch_expand_T(const PlanarView& fine, const PlanarView& coarse, cudaStream_t st)
{
    note_launch("expand_T", 4.0 * fine.C * (npix(fine.w, fine.h) + npix(coarse.w, coarse.h)));
    k_expand_T<<<row_grid(coarse.w, coarse.h), 256, 0, st>>>((const float*)fine.p, fine.pitch, fine.plane, fine.w,
                                                             fine.h, (float*)coarse.p, coarse.pitch, coarse.plane,
                                                             coarse.w, coarse.h, coarse.C);
    return cudaGetLastError();
}

cudaError_t launch_adj_mask_level(const PlanarView& gr, const PlanarView& lp, const PlanarView* next,
                                  const PlanarView& acc, cudaStream_t st)
{
    note_launch("adj_mask_level", npix(gr.w, gr.h) * (24.0 + 4.0) + (next ? 4.0 * npix(next->w, next->h) : 0.0));
    k_adj_mask_level<<<row_grid(gr.w, gr.h), 256, 0, st>>>(
        (const float*)gr.p, (const float*)lp.p, gr.pitch, gr.plane, gr.w, gr.h, next ? (const float*)next->p : nullptr,
        next ? next->pitch : 0, next ? next->w : 0, next ? next->h : 0, (float*)acc.p);
    return cudaGetLastError();
}

cudaError_t launch_adj_norm_bw(int K, const float* w, const float* a, const float* gm, float* gw, float* ga,
                               int64_t pitch, int64_t plane, int width, int height, cudaStream_t st)
{
    note_launch("adj_norm_bw", npix(width, height) * K * (a ? 20.0 : 12.0));
    k_adj_norm_bw<<<row_grid(width, height), 256, 0, st>>>(K, w, a, gm, gw, ga, pitch, plane, width);
    return cudaGetLastError();
}

cudaError_t launch_adj_weights_bw(const FloatPixelView& img, const float* gw, int64_t gpitch, const FloatWeightParams& wp,
                                  float inv_width, float width, float w_exp, int cwin, double* d, cudaStream_t st)
{
    note_launch("adj_weights_bw", npix(img.w, img.h) * (img.stride * 4.0 + 4.0));
    FloatWeightParams p = wp;
    p.contrast_window = cwin;
    const int TW = 16 + 2 * (cwin / 2);
    const size_t smem = ftile_bytes(TW, 0);
    const dim3 g((unsigned)((img.w + 15) / 16), (unsigned)((img.h + 15) / 16));
    if (cwin == 5) {
        k_adj_weights_bw<5><<<g, 256, smem, st>>>(img, gw, gpitch, p, inv_width, width, w_exp, d);
    } else {
        if (smem > 48 * 1024) {
            cudaFuncSetAttribute(k_adj_weights_bw<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        }
        k_adj_weights_bw<0><<<g, 256, smem, st>>>(img, gw, gpitch, p, inv_width, width, w_exp, d);
    }
    return cudaGetLastError();
}

}  // namespace enb
