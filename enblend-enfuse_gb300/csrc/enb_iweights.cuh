// enb_iweights.cuh -- enfuse weights of 8/16-bit images (src/enfuse.h:
// 962-1212 with integer pixels): the gray projectors, the rounding of the
// window statistics, a shared-memory tile of one exposure and the weight of
// one pixel of it.  Used by the per-image weight kernel (enb_kernels.cu) and
// by the fused enfuse (enb_efuse.cu).
#pragma once

#include <stdint.h>

#include "enb_device.cuh"
#include "enb_entropy.cuh"
#include "enb_internal.h"

namespace enb {

__device__ __forceinline__ int alpha_at(const AlphaSrc& a, int x, int y)
{
    if (a.mode == kAlphaOpaque) {
        return 1;
    }
    if (a.mode == kAlphaPlane) {
        return a.plane.p[(int64_t)y * a.plane.pitch + x] != 0;
    }
    const int64_t i = (int64_t)y * a.pix.pitch + (int64_t)x * a.pix.stride + 3;
    if (a.pix.dtype == ENB_F32) {
        const float f = reinterpret_cast<const float*>(a.pix.p)[i];
        return f >= a.flo && f <= a.fhi;
    }
    const uint32_t v = load_sample(a.pix.p, a.pix.dtype, i);
    return v >= a.lo && v <= a.hi;
}

constexpr int WT = 16;  // 16x16 weight pixels per CTA

// MultiGrayscaleAccessor::project for integer RGB (src/mga.h:185-222):
// average = fromRealPromote((r+g+b)/3.0) = (r+g+b+1)/3 and lightness =
// fromRealPromote((min+max)/2.0) = (min+max+1)/2 exactly for non-negative
// integers; luminance and the mixer evaluate the reference's double sums.
__device__ __forceinline__ int32_t gray_proj(int projector, const WeightParams& wp, uint32_t r, uint32_t g, uint32_t b)
{
    switch (projector) {
    case ENB_GRAY_VALUE: return (int32_t)max(r, max(g, b));
    case ENB_GRAY_ANTI_VALUE: return (int32_t)min(r, min(g, b));
    case ENB_GRAY_LIGHTNESS: return (int32_t)((min(r, min(g, b)) + max(r, max(g, b)) + 1) >> 1);
    case ENB_GRAY_LUMINANCE: {
        const double s = __dadd_rn(__dadd_rn(__dmul_rn(0.3, (double)r), __dmul_rn(0.59, (double)g)),
                                   __dmul_rn(0.11, (double)b));
        return (int32_t)frp_unsigned(s, wp.maxv);
    }
    case ENB_GRAY_MIXER: {
        const double s = __dadd_rn(__dadd_rn(__dmul_rn(wp.mixer[0], (double)r), __dmul_rn(wp.mixer[1], (double)g)),
                                   __dmul_rn(wp.mixer[2], (double)b));
        return (int32_t)frp_unsigned(s, wp.maxv);
    }
    default: return (int32_t)((r + g + b + 1u) / 3u);
    }
}

__device__ __forceinline__ int32_t gray_of(const WeightParams& wp, uint32_t r, uint32_t g, uint32_t b)
{
    return gray_proj(wp.gray_projector, wp, r, g, b);
}

// ClampingFunctor of the entropy cutoff (src/enfuse.h:893-925): x <= lo -> 0,
// x >= hi -> max, else x; the third sample is judged low by the first.
__device__ __forceinline__ void entropy_clamp(const WeightParams& wp, uint32_t (&rgb)[3], int C)
{
    const bool red_low = (int32_t)rgb[0] <= wp.ent_lo;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        if (ch < C) {
            const bool low = (C == 3 && ch == 2) ? red_low : (int32_t)rgb[ch] <= wp.ent_lo;
            rgb[ch] = low ? 0u : ((int32_t)rgb[ch] >= wp.ent_hi ? wp.maxv : rgb[ch]);
        }
    }
}

// fromRealPromote(sqrt((Q - S*S/n) / (n-1))) of the window sums
// (src/enfuse.h:154-160).  With num = n Q - S^2 and nn = n (n-1) (exact
// integers), the rounded deviation is the m with
//   (2m-1)^2 nn <= 4 num < (2m+1)^2 nn,
// found from a float estimate (within one of m) and checked in 64-bit
// integers.  The reference's double expression can round differently only
// where 4 num lies within its rounding error of a boundary: within tol =
// 2^-45 num + 2^-48 n Q + 4 of one (a bound on those errors, larger than
// them by a factor of two or more), and at exact ties, the double expression
// is evaluated as the reference writes it.
__device__ __forceinline__ int32_t stddev_round(int64_t S, int64_t Q, int n)
{
    if (n <= 1) {
        return 0;
    }
    const int64_t num = (int64_t)n * Q - S * S;
    const int64_t nn = (int64_t)n * (n - 1);
    const int64_t num4 = 4 * num;
    int64_t m = (int64_t)floorf(sqrtf(__fdiv_rn((float)num, (float)nn)) + 0.5f);
    if (m > 0 && (2 * m - 1) * (2 * m - 1) * nn > num4) {
        --m;
    } else if ((2 * m + 1) * (2 * m + 1) * nn <= num4) {
        ++m;
    }
    const int64_t dlo = m > 0 ? num4 - (2 * m - 1) * (2 * m - 1) * nn : INT64_MAX;
    const int64_t dhi = (2 * m + 1) * (2 * m + 1) * nn - num4;
    const int64_t tol = (num >> 45) + (((int64_t)n * Q) >> 48) + 4;
    if (dlo >= tol && dhi >= tol) {
        return (int32_t)m;
    }
    const double sum = (double)S;
    const double var = __ddiv_rn(__dadd_rn((double)Q, -__ddiv_rn(__dmul_rn(sum, sum), (double)n)), (double)(n - 1));
    const double sd = __dsqrt_rn(var);
    return __double2int_rz(__dadd_rn(sd, 0.5));
}

// Histogram::entropyOfChannel of n sorted samples (src/enfuse.h:346-375),
// scaled by the channel maximum and rounded (Histogram::entropyFun).  The
// sum of p log p is accumulated exactly in 2^-56 fixed point and rounded by
// entropy_fx_round; near a rounding boundary the reference's double sum
// (bins in ascending key order) is evaluated.
__device__ __noinline__ static int32_t entropy_round(const uint16_t* v, int n, const WeightTables& tab, int nmax, uint32_t maxv)
{
    if (n == 0) {
        return 0;
    }
    int bins = 0;
    long long acc = 0;
    const long long* fx = tab.plogp_fx + (int64_t)n * (nmax + 1);
    int i = 0;
    while (i < n) {
        int j = i + 1;
        while (j < n && v[j] == v[i]) {
            ++j;
        }
        acc += fx[j - i];
        ++bins;
        i = j;
    }
    if (bins <= 1) {
        return 0;
    }
    bool near;
    const uint32_t r = entropy_fx_round(acc, bins, n, tab, maxv, near);
    if (!near) {
        return (int32_t)r;
    }
    const double* pl = tab.plogp + (int64_t)n * (nmax + 1);
    double es = 0.0;
    i = 0;
    while (i < n) {
        int j = i + 1;
        while (j < n && v[j] == v[i]) {
            ++j;
        }
        es = __dadd_rn(es, pl[j - i]);
        i = j;
    }
    const double H = __ddiv_rn(-es, tab.logb[bins]);
    return (int32_t)frp_unsigned(__dmul_rn(H, (double)maxv), maxv);
}

// (float)(w * s) with s = fl(d / S) in double, d < S integers
// (SaturationFunctor, src/enfuse.h:755-776), via a float-float product;
// near a float rounding midpoint the double expression is evaluated.
__device__ __forceinline__ float saturation_weight(const WeightParams& wp, uint32_t d, uint32_t S)
{
    const float fd = (float)d, fS = (float)S;
    const float q1 = __fdiv_rn(fd, fS);
    const float rem = __fmaf_rn(-q1, fS, fd);       // exact remainder
    const float q2 = __fdiv_rn(rem, fS);
    const float p_hi = __fmul_rn(wp.w_sat_hi, q1);
    const float e1 = __fmaf_rn(wp.w_sat_hi, q1, -p_hi);
    const float p_lo = __fadd_rn(e1, __fadd_rn(__fmul_rn(wp.w_sat_hi, q2), __fmul_rn(wp.w_sat_lo, q1)));
    const float s = __fadd_rn(p_hi, p_lo);
    // residual of the float-float value against its rounding s
    const float t = __fadd_rn(__fadd_rn(p_hi, -s), p_lo);
    const float ulp = __int_as_float(__float_as_int(s) + 1) - s;
    const float dist = fabsf(fabsf(t) - 0.5f * ulp);
    const bool pow2 = (__float_as_int(s) & 0x7fffff) == 0;  // ulp below s is half as large
    if (dist > 1.0e-5f * ulp && s > 1.0e-30f && !pow2) {
        return s;
    }
    const double sd = __ddiv_rn((double)d, (double)S);
    return (float)__dmul_rn(wp.w_saturation, sd);
}

// ---- one exposure's tile in shared memory -----------------------------------

// Tile of (TW x TW) input pixels around 16x16 output pixels: gray, the
// samples (clamped by the entropy cutoff when it is active) and the alpha.
struct ITile {
    int32_t* gray;   // [TW*TW]
    uint16_t* raw;   // [3][TW*TW]
    uint8_t* a;      // [TW*TW]
    int TW;
};

__host__ __device__ inline size_t itile_bytes(int TW) { return (size_t)TW * TW * (sizeof(int32_t) + 3 * sizeof(uint16_t) + 1); }

__host__ __device__ inline int iweight_halo(const WeightParams& wp)
{
    const int hc = wp.use_contrast ? wp.contrast_window / 2 : 0, he = wp.use_entropy ? wp.entropy_window / 2 : 0;
    return hc > he ? hc : he;
}

__device__ __forceinline__ ITile itile_carve(unsigned char* smem, int TW)
{
    ITile t;
    t.TW = TW;
    t.gray = reinterpret_cast<int32_t*>(smem);
    t.raw = reinterpret_cast<uint16_t*>(t.gray + TW * TW);
    t.a = reinterpret_cast<uint8_t*>(t.raw + 3 * TW * TW);
    return t;
}

// Loads the tile whose top-left input pixel is (x0, y0): zero and
// transparent outside the image.  All threads call; the caller syncs.
__device__ __forceinline__ void itile_load(const ITile& t, const WeightParams& wp, const PixelView& img,
                                           const AlphaSrc& alpha, int x0, int y0)
{
    const int TW = t.TW, TT = TW * TW;
    const int w = img.w, h = img.h, C = img.C;
    for (int k = threadIdx.x; k < TT; k += blockDim.x) {
        const int r = k / TW, c = k - r * TW;
        const int gx = x0 + c, gy = y0 + r;
        int32_t g = 0;
        uint8_t a = 0;
        uint32_t rgb[3] = {0, 0, 0};
        if (gx >= 0 && gx < w && gy >= 0 && gy < h) {
            const int64_t base = (int64_t)gy * img.pitch + (int64_t)gx * img.stride;
            for (int ch = 0; ch < C; ++ch) {
                rgb[ch] = load_sample(img.p, img.dtype, base + ch);
            }
            g = C == 1 ? (int32_t)rgb[0] : gray_of(wp, rgb[0], rgb[1], rgb[2]);
            a = (uint8_t)alpha_at(alpha, gx, gy);
            if (wp.ent_cut) {
                // the tile's samples feed only the entropy windows then; the
                // saturation reloads its pixel
                entropy_clamp(wp, rgb, C);
            }
        }
        t.gray[k] = g;
        t.a[k] = a;
        for (int ch = 0; ch < 3; ++ch) {
            t.raw[ch * TT + k] = (uint16_t)rgb[ch];
        }
    }
}

// The enfuseMask weight of the output pixel (x, y) at tile index ci:
// exposure (assigned, with the cutoff), + contrast, + saturation, + entropy
// (the reference's float adds, src/enfuse.h:1119-1120, 1133-1134, 1208-1209).
__device__ __forceinline__ float i_pixel_weight(const ITile& t, const WeightParams& wp, const WeightTables& tab,
                                                const PixelView& img, int ci, int x, int y)
{
    const int TW = t.TW;
    const int w = img.w, h = img.h, C = img.C;
    const int32_t* s_gray = t.gray;
    const uint16_t* s_raw = t.raw;
    const uint8_t* s_a = t.a;
    float result = 0.0f;
    if (s_a[ci]) {
        const int32_t g = s_gray[ci];
        if (wp.use_exposure) {
            bool pass = true;
            if (wp.exp_cut) {
                int32_t lv = g, uv = g;
                if (C == 3) {
                    // the unclamped samples of this pixel
                    const int64_t base = (int64_t)y * img.pitch + (int64_t)x * img.stride;
                    const uint32_t r = load_sample(img.p, img.dtype, base), gg = load_sample(img.p, img.dtype, base + 1),
                                   bb = load_sample(img.p, img.dtype, base + 2);
                    lv = gray_proj(wp.cut_proj[0], wp, r, gg, bb);
                    uv = gray_proj(wp.cut_proj[1], wp, r, gg, bb);
                }
                pass = lv >= wp.cut_lo && uv <= wp.cut_hi;
            }
            result = pass ? tab.exposure[g] : 0.0f;
        }
        if (wp.use_contrast) {
            const int b = wp.contrast_window / 2;
            uint32_t gc = 0;
            if (x >= b && x < w - b && y >= b && y < h - b) {
                int64_t S = 0, Q = 0;
                int n = 0;
                for (int dy = -b; dy <= b; ++dy) {
                    const int row = ci + dy * TW;
                    for (int dx = -b; dx <= b; ++dx) {
                        if (s_a[row + dx]) {
                            const int64_t v = s_gray[row + dx];
                            S += v;
                            Q += v * v;
                            ++n;
                        }
                    }
                }
                // the combine lambda receives the gradient as the pixel's scalar type
                gc = (uint32_t)stddev_round(S, Q, n) & wp.maxv;
            }
            result = __fadd_rn(tab.contrast[gc], result);
        }
        if (wp.use_saturation && C == 3) {
            uint32_t r = s_raw[ci], gg = s_raw[TW * TW + ci], bb = s_raw[2 * TW * TW + ci];
            if (wp.ent_cut) {
                const int64_t base = (int64_t)y * img.pitch + (int64_t)x * img.stride;
                r = load_sample(img.p, img.dtype, base);
                gg = load_sample(img.p, img.dtype, base + 1);
                bb = load_sample(img.p, img.dtype, base + 2);
            }
            const uint32_t mx = max(r, max(gg, bb)), mn = min(r, min(gg, bb));
            float sw = 0.0f;
            if (mx != mn) {
                const uint32_t sum = mx + mn;
                const uint32_t S = sum <= wp.maxv ? sum : 2u * wp.maxv - sum;
                sw = saturation_weight(wp, mx - mn, S);
            }
            result = __fadd_rn(sw, result);
        }
        if (wp.use_entropy) {
            const int b = wp.entropy_window / 2;
            uint32_t emin = 0;
            if (x >= b && x < w - b && y >= b && y < h - b) {
                uint16_t vals[kMaxEntropyWindow * kMaxEntropyWindow];
                const int nmax = wp.entropy_window * wp.entropy_window;
                emin = wp.maxv;
                for (int ch = 0; ch < C; ++ch) {
                    if (wp.entropy_window == 5 || wp.entropy_window == 3) {
                        const uint16_t* raw = s_raw + ch * TW * TW;
                        const uint32_t e = wp.entropy_window == 5
                                               ? entropy_window_int<5>(raw, s_a, TW, ci, tab, wp.maxv)
                                               : entropy_window_int<3>(raw, s_a, TW, ci, tab, wp.maxv);
                        emin = min(emin, e);
                        continue;
                    }
                    int n = 0;
                    for (int dy = -b; dy <= b; ++dy) {
                        const int row = ci + dy * TW;
                        for (int dx = -b; dx <= b; ++dx) {
                            if (s_a[row + dx]) {
                                // insertion into the sorted prefix
                                const uint16_t v = s_raw[ch * TW * TW + row + dx];
                                int p = n++;
                                while (p > 0 && vals[p - 1] > v) {
                                    vals[p] = vals[p - 1];
                                    --p;
                                }
                                vals[p] = v;
                            }
                        }
                    }
                    const uint32_t e = (uint32_t)entropy_round(vals, n, tab, nmax, wp.maxv);
                    emin = min(emin, e);
                }
            }
            result = __fadd_rn(tab.entropy[emin], result);
        }
    }
    return result;
}


}  // namespace enb
