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
    int32_t* gray;   // [TT]
    uint16_t* raw;   // [3][TT]
    uint8_t* a;      // [TT]
    int TW;          // row pitch (pixels)
    int TT;          // plane size: TW * rows
};

__host__ __device__ inline size_t itile_bytes(int TW) { return (size_t)TW * TW * (sizeof(int32_t) + 3 * sizeof(uint16_t) + 1); }
__host__ __device__ inline size_t itile_bytes_rect(int TW, int TH)
{
    return (size_t)TW * TH * (sizeof(int32_t) + 3 * sizeof(uint16_t) + 1);
}

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
    t.TT = TW * TW;
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
            uint32_t r = s_raw[ci], gg = s_raw[t.TT + ci], bb = s_raw[2 * t.TT + ci];
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
                        const uint16_t* raw = s_raw + ch * t.TT;
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
                                const uint16_t v = s_raw[ch * t.TT + row + dx];
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


// ---- rectangular tiles and pairs of output pixels --------------------------

__device__ __forceinline__ ITile itile_carve_rect(unsigned char* smem, int TW, int TH)
{
    ITile t;
    t.TW = TW;
    t.TT = TW * TH;
    t.gray = reinterpret_cast<int32_t*>(smem);
    t.raw = reinterpret_cast<uint16_t*>(t.gray + t.TT);
    t.a = reinterpret_cast<uint8_t*>(t.raw + 3 * t.TT);
    return t;
}

// Loads the TW x TH tile whose top-left input pixel is (x0, y0) as
// itile_load does (all threads call); ends with a barrier and returns
// nonzero when every tile pixel lies in the image and is opaque.
__device__ __forceinline__ int itile_load_rect(const ITile& t, const WeightParams& wp, const PixelView& img,
                                               const AlphaSrc& alpha, int x0, int y0)
{
    const int TW = t.TW, TT = t.TT;
    const int w = img.w, h = img.h, C = img.C;
    int mine = 1;
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
                entropy_clamp(wp, rgb, C);
            }
        }
        mine &= a;
        t.gray[k] = g;
        t.a[k] = a;
        for (int ch = 0; ch < 3; ++ch) {
            t.raw[ch * TT + k] = (uint16_t)rgb[ch];
        }
    }
    return __syncthreads_and(mine);
}

// Keys of the W x W entropy windows (W = 3 or 5) of two horizontally
// adjacent pixels, the left one at tile position (cx, cy) with cx even, in
// a plane of 16-bit samples with an even row pitch TW: key j of a row holds
// the left pixel's tap in its low half and the right pixel's in its high
// half, which are the two samples of one word (an aligned word or the
// middle of two), so a row of five keys takes three word loads.
template <int W>
__device__ __forceinline__ void pair_window_keys(const uint16_t* plane, int TW, int cx, int cy, uint32_t (&k)[W * W])
{
    constexpr int B = W / 2;
#pragma unroll
    for (int dy = 0; dy < W; ++dy) {
        const uint32_t* row = reinterpret_cast<const uint32_t*>(plane + (cy + dy - B) * TW + cx - 2);
        const uint32_t w0 = row[0], w1 = row[1], w2 = row[2];  // columns cx-2 .. cx+3
        const uint32_t m01 = __byte_perm(w0, w1, 0x5432), m12 = __byte_perm(w1, w2, 0x5432);
        if (W == 5) {
            k[dy * W + 0] = w0;
            k[dy * W + 1] = m01;
            k[dy * W + 2] = w1;
            k[dy * W + 3] = m12;
            k[dy * W + 4] = w2;
        } else {
            k[dy * W + 0] = m01;
            k[dy * W + 1] = w1;
            k[dy * W + W - 1] = m12;
        }
    }
}

// Histogram::entropyOfChannel of M = W * W opaque samples from the bit mask
// of their sorted order (bit i set: sample i differs from sample i - 1):
// popc + 1 bins, and each run of set-free bits of length c - 1 a bin of c
// equal samples.  fx: the 2^-56 fixed-point p log p terms of n = M (in shared
// memory).  near: the result lies too close to a rounding boundary; the
// caller then evaluates the reference's double sum.
template <int M>
__device__ __forceinline__ uint32_t entropy_from_boundaries(uint32_t bnd, const long long* fx,
                                                            const WeightTables& tab, uint32_t maxv, bool& near)
{
    near = false;
    const int bins = __popc(bnd) + 1;
    if (bins <= 1) {
        return 0u;
    }
    long long acc = (long long)bins * fx[1];
    uint32_t eq = ~bnd & (((1u << M) - 1u) & ~1u);  // sample i equals sample i - 1
    while (eq) {
        const int s0 = __ffs(eq) - 1;
        const int len = __ffs(~(eq >> s0)) - 1;  // a bin of len + 1 equal samples
        acc += fx[len + 1] - fx[1];
        eq &= ~(((1u << len) - 1u) << s0);
    }
    return entropy_fx_round(acc, bins, M, tab, maxv, near);
}

// The reference's double expression for one half of the sorted pair keys
// (the rare rounding-boundary case).
template <int M>
__device__ __noinline__ static uint32_t entropy_half_exact(const uint32_t (&k)[M], int half, const WeightTables& tab,
                                                           uint32_t maxv)
{
    uint32_t v[M];
    int bins = 1;
#pragma unroll
    for (int i = 0; i < M; ++i) {
        v[i] = (k[i] >> (16 * half)) & 0xffffu;
        bins += (i > 0 && v[i] != v[i - 1]) ? 1 : 0;
    }
    const double es = entropy_sum_double<M>(v, M, tab.plogp + (int64_t)M * (M + 1));
    const double H = __ddiv_rn(-es, tab.logb[bins]);
    return frp_unsigned(__dmul_rn(H, (double)maxv), maxv);
}

// fromRealPromote(H * max) of the W x W windows of two adjacent pixels in
// one channel: both windows sorted at once, one per half word (the samples
// are at most 16 bits wide), then the bins of each from its boundary mask.
template <int W>
__device__ __forceinline__ void entropy_pair(const uint16_t* plane, int TW, int cx, int cy, const long long* fx,
                                             const WeightTables& tab, uint32_t maxv, uint32_t& e0, uint32_t& e1)
{
    constexpr int M = W * W;
    uint32_t k[M];
    pair_window_keys<W>(plane, TW, cx, cy, k);
    sortnet(k, CeU16x2());
    uint32_t b0 = 0, b1 = 0;
#pragma unroll
    for (int i = 1; i < M; ++i) {
        // each half is sorted, so the word difference is the two halves'
        // differences without a borrow; min(d, 1) per half: 1 where they differ
        const uint32_t d = k[i] - k[i - 1];
        uint32_t nz;
        asm("min.u16x2 %0, %1, %2;" : "=r"(nz) : "r"(d), "r"(0x00010001u));
        b0 |= (nz & 1u) << i;
        b1 |= (nz >> 16) << i;
    }
    bool near0, near1;
    e0 = entropy_from_boundaries<M>(b0, fx, tab, maxv, near0);
    e1 = entropy_from_boundaries<M>(b1, fx, tab, maxv, near1);
    if (near0) {
        e0 = entropy_half_exact<M>(k, 0, tab, maxv);
    }
    if (near1) {
        e1 = entropy_half_exact<M>(k, 1, tab, maxv);
    }
}

// The rounded window deviations (localStdDevIf) of two adjacent pixels
// whose CW x CW windows are opaque: column sums of gray and gray^2 over
// the CW + 1 columns of both windows, each column summed once.
template <int CW>
__device__ __forceinline__ void contrast_pair(const int32_t* gray, int TW, int cx, int cy, uint32_t maxv, uint32_t& g0,
                                              uint32_t& g1)
{
    constexpr int B = CW / 2, NC = CW + 1;
    uint32_t S[NC];
    uint64_t Q[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        S[c] = 0u;
        Q[c] = 0ull;
    }
#pragma unroll
    for (int dy = 0; dy < CW; ++dy) {
        const int32_t* row = gray + (cy + dy - B) * TW + cx - B;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const uint32_t v = (uint32_t)row[c];
            S[c] += v;
            Q[c] += (uint64_t)v * v;
        }
    }
    uint32_t s0 = 0u;
    uint64_t q0 = 0ull;
#pragma unroll
    for (int c = 0; c < CW; ++c) {
        s0 += S[c];
        q0 += Q[c];
    }
    const uint32_t s1 = s0 - S[0] + S[CW];
    const uint64_t q1 = q0 - Q[0] + Q[CW];
    g0 = (uint32_t)stddev_round((int64_t)s0, (int64_t)q0, CW * CW) & maxv;
    g1 = (uint32_t)stddev_round((int64_t)s1, (int64_t)q1, CW * CW) & maxv;
}

// SaturationFunctor of an integer RGB pixel (src/enfuse.h:733-780), as
// i_pixel_weight evaluates it.
__device__ __forceinline__ float saturation_of(const WeightParams& wp, uint32_t r, uint32_t g, uint32_t b)
{
    const uint32_t mx = max(r, max(g, b)), mn = min(r, min(g, b));
    if (mx == mn) {
        return 0.0f;
    }
    const uint32_t sum = mx + mn;
    const uint32_t S = sum <= wp.maxv ? sum : 2u * wp.maxv - sum;
    return saturation_weight(wp, mx - mn, S);
}

// Whether the pair path can weight a tile whose pixels are all opaque and
// inside the image: entropy windows of 3 or 5, contrast windows of 3, 5 or
// 7, no cutoff (the cutoffs need the unclamped samples of a pixel).
__host__ __device__ inline bool iweight_pair_path(const WeightParams& wp)
{
    return !wp.exp_cut && !wp.ent_cut && (!wp.use_entropy || wp.entropy_window == 3 || wp.entropy_window == 5) &&
           (!wp.use_contrast || wp.contrast_window == 3 || wp.contrast_window == 5 || wp.contrast_window == 7);
}

// The weights of the pixel pair at tile position (cx, cy) of a fully opaque
// tile, in the reference's order of float adds (as i_pixel_weight).
template <int CW, int EW>
__device__ __forceinline__ void pair_weights_t(const ITile& t, const WeightParams& wp, const WeightTables& tab,
                                               const long long* fx, int C, int cx, int cy, float& w0, float& w1)
{
    const int ci = cy * t.TW + cx;
    float r0 = 0.0f, r1 = 0.0f;
    if (wp.use_exposure) {
        r0 = tab.exposure[t.gray[ci]];
        r1 = tab.exposure[t.gray[ci + 1]];
    }
    if (CW > 0) {
        uint32_t g0, g1;
        contrast_pair<(CW > 0 ? CW : 3)>(t.gray, t.TW, cx, cy, wp.maxv, g0, g1);
        r0 = __fadd_rn(tab.contrast[g0], r0);
        r1 = __fadd_rn(tab.contrast[g1], r1);
    }
    if (wp.use_saturation && C == 3) {
        const uint16_t* raw = t.raw;
        r0 = __fadd_rn(saturation_of(wp, raw[ci], raw[t.TT + ci], raw[2 * t.TT + ci]), r0);
        r1 = __fadd_rn(saturation_of(wp, raw[ci + 1], raw[t.TT + ci + 1], raw[2 * t.TT + ci + 1]), r1);
    }
    if (EW > 0) {
        uint32_t m0 = wp.maxv, m1 = wp.maxv;
        for (int ch = 0; ch < C; ++ch) {
            uint32_t e0, e1;
            entropy_pair<(EW > 0 ? EW : 3)>(t.raw + ch * t.TT, t.TW, cx, cy, fx, tab, wp.maxv, e0, e1);
            m0 = min(m0, e0);
            m1 = min(m1, e1);
        }
        r0 = __fadd_rn(tab.entropy[m0], r0);
        r1 = __fadd_rn(tab.entropy[m1], r1);
    }
    w0 = r0;
    w1 = r1;
}

__device__ __forceinline__ void pair_weights(const ITile& t, const WeightParams& wp, const WeightTables& tab,
                                             const long long* fx, int C, int cx, int cy, float& w0, float& w1)
{
    const int cw = wp.use_contrast ? wp.contrast_window : 0, ew = wp.use_entropy ? wp.entropy_window : 0;
#define ENB_PW(CWV, EWV)                                                          \
    if (cw == CWV && ew == EWV) {                                                 \
        pair_weights_t<CWV, EWV>(t, wp, tab, fx, C, cx, cy, w0, w1);              \
        return;                                                                   \
    }
    ENB_PW(5, 5) ENB_PW(5, 3) ENB_PW(3, 3) ENB_PW(3, 5) ENB_PW(7, 5) ENB_PW(7, 3)
    ENB_PW(0, 5) ENB_PW(0, 3) ENB_PW(5, 0) ENB_PW(3, 0) ENB_PW(7, 0) ENB_PW(0, 0)
#undef ENB_PW
    w0 = w1 = 0.0f;
}

}  // namespace enb
