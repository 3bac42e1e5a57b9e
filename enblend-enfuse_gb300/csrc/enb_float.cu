// enb_float.cu -- the float-image path: FP32 pyramids standing in for the
// reference's double pyramids of float images (src/numerictraits.h:185,
// float row: pyramid double 8.0, mask pyramid Int32 9.15).
//
// The reference maps float samples logarithmically into the pyramid
// (src/fixmath.h:165-187: v >= 0 ? 1 + log1p(v) : 1 / (1 - v), with the float
// overload of log1p), reduces and expands them with real divisions, merges in
// double and maps level 0 back (src/fixmath.h:320-329).  Here every pyramid
// value is a float; the results agree with the double pyramids to float
// rounding (the tests bound the difference).  Mask pyramids stay Int32 9.15
// and use the fixed-point kernels.
#include <cuda_runtime.h>
#include <stdint.h>

#include "enb_device.cuh"
#include "enb_fpair.cuh"
#include "enb_fweights.cuh"
#include "enb_internal.h"

namespace enb {

namespace {

inline dim3 row_grid(int w, int h) { return dim3((unsigned)((w + 255) / 256), (unsigned)h); }
inline double npix(int w, int h) { return (double)w * (double)h; }

}  // namespace

// ---------------------------------------------------------------------------
// Conversions (src/fixmath.h:165-187, 320-329)
// ---------------------------------------------------------------------------

template <int C>
__global__ void __launch_bounds__(256) k_f_to_pyramid(const float* __restrict__ src, int64_t spitch, int stride,
                                                      float* __restrict__ dst, int64_t dpitch, int64_t dplane, int w,
                                                      int h)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const float* s = src + (int64_t)y * spitch + (int64_t)x * stride;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        dst[(int64_t)c * dplane + (int64_t)y * dpitch + x] = to_pyramid_value(__ldg(&s[c]));
    }
}

template <int C>
__global__ void __launch_bounds__(256) k_f_from_pyramid(const float* __restrict__ src, int64_t spitch,
                                                        int64_t splane, const uint8_t* __restrict__ alpha,
                                                        int64_t apitch, float* __restrict__ dst, int64_t dpitch,
                                                        int dstride, int w, int h)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w || !alpha[(int64_t)y * apitch + x]) {
        return;
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
        dst[(int64_t)y * dpitch + (int64_t)x * dstride + c] =
            from_pyramid_value(src[(int64_t)c * splane + (int64_t)y * spitch + x]);
    }
}

// ---------------------------------------------------------------------------
// Expand (src/pyramid.h:875-1457) with real divisions
// ---------------------------------------------------------------------------

template <bool ADD>
__device__ __forceinline__ void f_combine(float* d, float e)
{
    *d = ADD ? __fadd_rn(*d, e) : __fsub_rn(*d, e);
}

template <int C, bool ADD>
__global__ void __launch_bounds__(256) k_f_expand(const float* __restrict__ src, int64_t spitch, int64_t splane,
                                                  int sw, int sh, float* __restrict__ dst, int64_t dpitch,
                                                  int64_t dplane, int dw, int dh, int wrap)
{
    __shared__ float ss[C][ESH][ESW];
    const int X0 = blockIdx.x * ETW, Y0 = blockIdx.y * ETH;
    const int I0 = X0 >> 1, J0 = Y0 >> 1;
    const int tid = threadIdx.x;

    for (int k = tid; k < ESH * ESW; k += 256) {
        const int r = k / ESW, c = k - r * ESW;
        const int j = J0 - 1 + r;
        int i = I0 - 1 + c;
        if (wrap) {
            i = imod(i, sw);
        }
        const bool in = j >= 0 && j < sh && i >= 0 && i < sw;
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            ss[ch][r][c] = in ? src[(int64_t)ch * splane + (int64_t)j * spitch + i] : 0.0f;
        }
    }
    __syncthreads();

    const int qx = tid % 32, qy = tid / 32;
    const int i = I0 + qx, j = J0 + qy;
    const int X = 2 * i, Y = 2 * j;
    if (X >= dw || Y >= dh) {
        return;
    }
    const bool has_x1 = X + 1 < dw, has_y1 = Y + 1 < dh;
    const bool interior = i >= 1 && i + 1 < sw && j >= 1 && j + 1 < sh;

    if (interior) {
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            const float* a = &ss[ch][qy][qx];
            const float* b = &ss[ch][qy + 1][qx];
            const float* c = &ss[ch][qy + 2][qx];
            const float hea = a[0] + 6.0f * a[1] + a[2], heb = b[0] + 6.0f * b[1] + b[2],
                        hec = c[0] + 6.0f * c[1] + c[2];
            const float hoa = 4.0f * (a[1] + a[2]), hob = 4.0f * (b[1] + b[2]), hoc = 4.0f * (c[1] + c[2]);
            float* d0 = dst + (int64_t)ch * dplane + (int64_t)Y * dpitch + X;
            // divisors 64 and 16 are powers of two: the products are exact divisions
            f_combine<ADD>(d0, (hea + 6.0f * heb + hec) * 0.015625f);
            if (has_x1) {
                f_combine<ADD>(d0 + 1, (hoa + 6.0f * hob + hoc) * 0.015625f);
            }
            if (has_y1) {
                float* d1 = d0 + dpitch;
                f_combine<ADD>(d1, (heb + hec) * 0.0625f);
                if (has_x1) {
                    f_combine<ADD>(d1 + 1, (hob + hoc) * 0.0625f);
                }
            }
        }
        return;
    }

#pragma unroll
    for (int oy = 0; oy < 2; ++oy) {
        const int YY = Y + oy;
        if (YY >= dh) {
            continue;
        }
        int vw[3], vden;
        expand_vweights(YY, sh, vw, vden);
#pragma unroll
        for (int ox = 0; ox < 2; ++ox) {
            const int XX = X + ox;
            if (XX >= dw) {
                continue;
            }
            int hw[3], hden;
            expand_hweights(XX, sw, dw, wrap, hw, hden);
            const float den = (float)(hden * vden);
#pragma unroll
            for (int ch = 0; ch < C; ++ch) {
                float num = 0.0f;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const float* row = &ss[ch][qy + a][qx];
                    num += (float)vw[a] * ((float)hw[0] * row[0] + (float)hw[1] * row[1] + (float)hw[2] * row[2]);
                }
                f_combine<ADD>(dst + (int64_t)ch * dplane + (int64_t)YY * dpitch + XX, __fdiv_rn(num, den));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Merge operators on FP32 levels with Int32 mask levels
// ---------------------------------------------------------------------------

// CartesianBlendFunctor (src/blend.h:41-76): c = mask / white; c >= 1 keeps
// white, c <= 0 keeps black, otherwise c * white + (1 - c) * black.
template <int C>
__global__ void __launch_bounds__(256) k_f_blend(const int32_t* __restrict__ mask, int64_t mpitch,
                                                 const float* __restrict__ white, int64_t wpitch, int64_t wplane,
                                                 float* __restrict__ black, int64_t bpitch, int64_t bplane, int w,
                                                 int h, int32_t white_value)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const int32_t m = mask[(int64_t)y * mpitch + x];
    if (m <= 0) {
        return;
    }
    if (m >= white_value) {
#pragma unroll
        for (int c = 0; c < C; ++c) {
            black[(int64_t)c * bplane + (int64_t)y * bpitch + x] = white[(int64_t)c * wplane + (int64_t)y * wpitch + x];
        }
        return;
    }
    const float wc = __fdiv_rn((float)m, (float)white_value), bc = 1.0f - wc;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        float* b = &black[(int64_t)c * bplane + (int64_t)y * bpitch + x];
        *b = wc * white[(int64_t)c * wplane + (int64_t)y * wpitch + x] + bc * *b;
    }
}

// ImageMaskMultiplyFunctor (src/enfuse.h:601-620) and the accumulation into
// the result pyramid (src/enfuse.h:1576-1588).
template <int C>
__global__ void __launch_bounds__(256) k_f_mask_mul_acc(const float* __restrict__ lp, int64_t lpitch, int64_t lplane,
                                                        const int32_t* __restrict__ mask, int64_t mpitch,
                                                        float inv_divisor, float* __restrict__ res, int64_t rpitch,
                                                        int64_t rplane, int w, int h, int accumulate)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    // each product and sum rounded on its own (no fused multiply-add), as
    // the batched merge rounds them
    const float coeff = __fmul_rn((float)mask[(int64_t)y * mpitch + x], inv_divisor);
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const float v = __fmul_rn(lp[(int64_t)c * lplane + (int64_t)y * lpitch + x], coeff);
        float* r = &res[(int64_t)c * rplane + (int64_t)y * rpitch + x];
        *r = accumulate ? __fadd_rn(*r, v) : v;
    }
}

template <int C>
__global__ void __launch_bounds__(256) k_f_copy_level0(const float* __restrict__ src, int64_t spitch, int64_t splane,
                                                       float* __restrict__ dst, int w, int h)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
        dst[((int64_t)y * w + x) * C + c] = src[(int64_t)c * splane + (int64_t)y * spitch + x];
    }
}

// ---------------------------------------------------------------------------
// enfuse weights of float images (src/enfuse.h:962-1212), enb_fweights.cuh
// ---------------------------------------------------------------------------

constexpr int FWT = 16;  // 16x16 weight pixels per CTA

template <int CW, int EW>
__global__ void __launch_bounds__(256) k_f_enfuse_mask(FloatPixelView img, const uint8_t* __restrict__ alpha,
                                                       int64_t apitch, FloatWeightParams wp, WeightTables tab,
                                                       float* __restrict__ out, int64_t opitch)
{
    extern __shared__ __align__(16) unsigned char fsmem[];
    const int halo = fweight_halo(wp);
    const FTile t = ftile_carve(fsmem, FWT + 2 * halo, wp.repeat_slots, wp.ent_cut);
    const int opaque = ftile_load(t, wp, img.p, img.pitch, img.stride, img.w, img.h, img.C, alpha, apitch,
                                  blockIdx.x * FWT - halo, blockIdx.y * FWT - halo);
    const int lx = threadIdx.x % FWT, ly = threadIdx.x / FWT;
    const int x = blockIdx.x * FWT + lx, y = blockIdx.y * FWT + ly;
    if (x >= img.w || y >= img.h) {
        return;
    }
    const int ci = (ly + halo) * t.TW + (lx + halo);
    out[(int64_t)y * opitch + x] = f_pixel_weight<CW, EW>(t, wp, tab, ci, x, y, img.w, img.h, img.C, opaque != 0);
}

// The weights of one image, two output pixels per thread on 32x16 tiles
// (enb_fpair.cuh), for the window sizes of the pair path.
template <int CW, int EW, int C>
__global__ void __launch_bounds__(FPT, 4) k_f_enfuse_mask_pair(FloatPixelView img, const uint8_t* __restrict__ alpha,
                                                                int64_t apitch, FloatWeightParams wp, WeightTables tab,
                                                                float* __restrict__ out, int64_t opitch)
{
    constexpr int HALO = fpair_halo(CW, EW), HX = fpair_halo_x(HALO);
    constexpr int TW = fpair_tw(CW, EW), TT = TW * fpair_th(CW, EW), NP = (TT + 255) / 256;
    extern __shared__ __align__(16) unsigned char fsmem[];
    const FTileP t = fpair_carve(fsmem, TW, TT, wp.repeat_slots, wp.ent_cut);
    if (t.slots) {
        fpair_clear_tables<C>(t);
        __syncthreads();
    }
    const int opaque = fpair_load<NP, C, TW, TT>(t, wp, img.p, img.pitch, img.stride, img.w, img.h, alpha, apitch,
                                                 blockIdx.x * FPX - HX, blockIdx.y * FPY - HALO);
    const int px = threadIdx.x % (FPX / 2), py = threadIdx.x / (FPX / 2);
    const int x = blockIdx.x * FPX + 2 * px, y = blockIdx.y * FPY + py;
    if (x >= img.w || y >= img.h) {
        return;
    }
    float w0, w1;
    fpair_weights<CW, EW, C>(t, wp, tab, HX + 2 * px, HALO + py, x, y, img.w, img.h, opaque != 0, w0, w1);
    float* o = out + (int64_t)y * opitch + x;
    o[0] = w0;
    if (x + 1 < img.w) {
        o[1] = w1;
    }
}

// H of every window whose only repeated samples are clip values, by
// entropy_clip_bins (the function that evaluates such windows in the
// per-pixel weight path), so that the pair path's table lookups agree with
// it bit for bit.
__global__ void k_clip_entropy_table(WeightTables tab, int nmax, float* __restrict__ out)
{
    const int m = nmax + 1, total = m * m * m;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int n = i / (m * m), m1 = (i / m) % m, m0 = i % m;
        out[i] = m1 + m0 <= n ? entropy_clip_bins(n, m1, m0, tab, nmax) : 0.0f;
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

cudaError_t launch_clip_entropy_table(const WeightTables& tab, int nmax, float* out, cudaStream_t st)
{
    const int m = nmax + 1;
    note_launch("clip_entropy_table", (double)m * m * m * 4.0);
    k_clip_entropy_table<<<(unsigned)((m * m * m + 255) / 256), 256, 0, st>>>(tab, nmax, out);
    return cudaGetLastError();
}

cudaError_t launch_f_to_pyramid(const FloatPixelView& s, const PlanarView& d, cudaStream_t st)
{
    note_launch("f_to_pyramid", npix(s.w, s.h) * s.C * 8.0);
    const dim3 g = row_grid(s.w, s.h);
    if (s.C == 1) {
        k_f_to_pyramid<1><<<g, 256, 0, st>>>(s.p, s.pitch, s.stride, (float*)d.p, d.pitch, d.plane, s.w, s.h);
    } else {
        k_f_to_pyramid<3><<<g, 256, 0, st>>>(s.p, s.pitch, s.stride, (float*)d.p, d.pitch, d.plane, s.w, s.h);
    }
    return cudaGetLastError();
}

cudaError_t launch_f_from_pyramid(const PlanarView& s, const BytePlane& a, float* dst, int64_t dpitch, int dstride,
                                  cudaStream_t st)
{
    note_launch("f_from_pyramid", npix(s.w, s.h) * (1.0 + s.C * 8.0));
    const dim3 g = row_grid(s.w, s.h);
    if (s.C == 1) {
        k_f_from_pyramid<1><<<g, 256, 0, st>>>((const float*)s.p, s.pitch, s.plane, a.p, a.pitch, dst, dpitch, dstride,
                                               s.w, s.h);
    } else {
        k_f_from_pyramid<3><<<g, 256, 0, st>>>((const float*)s.p, s.pitch, s.plane, a.p, a.pitch, dst, dpitch, dstride,
                                               s.w, s.h);
    }
    return cudaGetLastError();
}

cudaError_t launch_f_expand(int add, int wrap, const PlanarView& s, const PlanarView& d, cudaStream_t st)
{
    note_launch(add ? "f_expand_add" : "f_expand_sub", 4.0 * (npix(s.w, s.h) + 2.0 * npix(d.w, d.h)) * d.C);
    const dim3 g = grid2d(d.w, d.h, ETW, ETH);
    const float* sp = (const float*)s.p;
    float* dp = (float*)d.p;
    if (s.C == 1) {
        add ? k_f_expand<1, true><<<g, 256, 0, st>>>(sp, s.pitch, s.plane, s.w, s.h, dp, d.pitch, d.plane, d.w, d.h, wrap)
            : k_f_expand<1, false><<<g, 256, 0, st>>>(sp, s.pitch, s.plane, s.w, s.h, dp, d.pitch, d.plane, d.w, d.h, wrap);
    } else {
        add ? k_f_expand<3, true><<<g, 256, 0, st>>>(sp, s.pitch, s.plane, s.w, s.h, dp, d.pitch, d.plane, d.w, d.h, wrap)
            : k_f_expand<3, false><<<g, 256, 0, st>>>(sp, s.pitch, s.plane, s.w, s.h, dp, d.pitch, d.plane, d.w, d.h, wrap);
    }
    return cudaGetLastError();
}

cudaError_t launch_f_blend(const PlanarView& m, const PlanarView& wt, const PlanarView& b, int32_t wv, cudaStream_t st)
{
    note_launch("f_blend", npix(b.w, b.h) * (4.0 + 12.0 * b.C));
    const dim3 g = row_grid(b.w, b.h);
    if (b.C == 1) {
        k_f_blend<1><<<g, 256, 0, st>>>((const int32_t*)m.p, m.pitch, (const float*)wt.p, wt.pitch, wt.plane,
                                        (float*)b.p, b.pitch, b.plane, b.w, b.h, wv);
    } else {
        k_f_blend<3><<<g, 256, 0, st>>>((const int32_t*)m.p, m.pitch, (const float*)wt.p, wt.pitch, wt.plane,
                                        (float*)b.p, b.pitch, b.plane, b.w, b.h, wv);
    }
    return cudaGetLastError();
}

cudaError_t launch_f_mask_mul_acc(const PlanarView& lp, const PlanarView& m, int32_t divisor, const PlanarView& r,
                                  int acc, cudaStream_t st)
{
    note_launch("f_mask_mul_acc", npix(lp.w, lp.h) * (4.0 + 4.0 * lp.C * (acc ? 3.0 : 2.0)));
    const dim3 g = row_grid(lp.w, lp.h);
    const float inv = (float)(1.0 / (double)divisor);
    if (lp.C == 1) {
        k_f_mask_mul_acc<1><<<g, 256, 0, st>>>((const float*)lp.p, lp.pitch, lp.plane, (const int32_t*)m.p, m.pitch,
                                               inv, (float*)r.p, r.pitch, r.plane, lp.w, lp.h, acc);
    } else {
        k_f_mask_mul_acc<3><<<g, 256, 0, st>>>((const float*)lp.p, lp.pitch, lp.plane, (const int32_t*)m.p, m.pitch,
                                               inv, (float*)r.p, r.pitch, r.plane, lp.w, lp.h, acc);
    }
    return cudaGetLastError();
}

cudaError_t launch_f_copy_level0(const PlanarView& s, float* dst, cudaStream_t st)
{
    note_launch("f_copy_level0", npix(s.w, s.h) * s.C * 8.0);
    const dim3 g = row_grid(s.w, s.h);
    if (s.C == 1) {
        k_f_copy_level0<1><<<g, 256, 0, st>>>((const float*)s.p, s.pitch, s.plane, dst, s.w, s.h);
    } else {
        k_f_copy_level0<3><<<g, 256, 0, st>>>((const float*)s.p, s.pitch, s.plane, dst, s.w, s.h);
    }
    return cudaGetLastError();
}

cudaError_t launch_f_enfuse_mask(const FloatPixelView& img, const BytePlane& alpha, const FloatWeightParams& wp,
                                 const WeightTables& tab, const FloatPlane& out, cudaStream_t st)
{
    note_launch("f_enfuse_mask", npix(img.w, img.h) * (img.stride * 4.0 + 1.0 + 4.0));
    if (fpair_path(wp) && (!wp.use_entropy || tab.clip_h)) {
        const int cw = wp.use_contrast ? wp.contrast_window : 0, ew = wp.use_entropy ? wp.entropy_window : 0;
        const int TT = fpair_tw(cw, ew) * fpair_th(cw, ew);
        FloatWeightParams p = wp;
        p.repeat_slots = fpair_slots(wp, TT);
        const size_t smem = fpair_tile_bytes(TT, p.repeat_slots, p.ent_cut);
        const dim3 g = grid2d(img.w, img.h, FPX, FPY);
        ENB_FPAIR_DISPATCH(p, {
            auto k = img.C == 1 ? k_f_enfuse_mask_pair<CWV, EWV, 1> : k_f_enfuse_mask_pair<CWV, EWV, 3>;
            if (smem > 48 * 1024) {
                cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            }
            // as many CTAs per SM as the shared memory holds
            cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
            k<<<g, FPT, smem, st>>>(img, alpha.p, alpha.pitch, p, tab, out.p, out.pitch);
        });
        return cudaGetLastError();
    }
    const int TW = FWT + 2 * fweight_halo(wp);
    FloatWeightParams p = wp;
    p.repeat_slots = fweight_slots(wp, TW);
    const size_t smem = ftile_bytes(TW, p.repeat_slots, p.ent_cut);
    const int cw = p.use_contrast ? p.contrast_window : 5, ew = p.use_entropy ? p.entropy_window : 5;
    void (*k)(FloatPixelView, const uint8_t*, int64_t, FloatWeightParams, WeightTables, float*, int64_t) =
        k_f_enfuse_mask<0, 0>;
    if (cw == 5 && ew == 5) {
        k = k_f_enfuse_mask<5, 5>;
    } else if (cw == 5 && ew == 3) {
        k = k_f_enfuse_mask<5, 3>;
    } else if (cw == 3 && ew == 3) {
        k = k_f_enfuse_mask<3, 3>;
    } else if (ew == 5) {
        k = k_f_enfuse_mask<0, 5>;
    } else if (ew == 3) {
        k = k_f_enfuse_mask<0, 3>;
    }
    if (smem > 48 * 1024) {
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    k<<<grid2d(img.w, img.h, FWT, FWT), FWT * FWT, smem, st>>>(img, alpha.p, alpha.pitch, p, tab, out.p, out.pitch);
    return cudaGetLastError();
}

}  // namespace enb
