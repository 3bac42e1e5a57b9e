// enb_fweights.cuh -- enfuse weights of float images (src/enfuse.h:962-1212
// with float pixels): the per-pixel functions, a shared-memory tile of one
// exposure and the weight of one pixel of it.  Used by the per-image weight
// kernel (enb_float.cu) and by the batched stack fuse (enb_batch.cu).
#pragma once

#include <stdint.h>

#include "enb_device.cuh"
#include "enb_entropy.cuh"
#include "enb_internal.h"

namespace enb {

// The logarithmic mapping of float samples into the pyramid and back
// (src/fixmath.h:165-187, 320-329).
__device__ __forceinline__ float to_pyramid_value(float v)
{
    return v >= 0.0f ? __fadd_rn(1.0f, log1pf(v)) : __fdiv_rn(1.0f, __fsub_rn(1.0f, v));
}

__device__ __forceinline__ float from_pyramid_value(float v)
{
    return v >= 1.0f ? expm1f(__fsub_rn(v, 1.0f)) : __fsub_rn(1.0f, __fdiv_rn(1.0f, v));
}

// fl(fl_double(s / 3)) of a float s, the reference's (float)(s / 3.0), in
// float arithmetic.  q = s * fl(1/3) corrected once by its exact remainder
// (fmaf) approximates s / 3 to within an ulp; the remainder r = s - 3 q of
// the corrected q (exact) then locates s / 3 = q + r / 3 relative to q.
// Where |s / 3 - q| lies clearly below half an ulp, q is the correctly
// rounded quotient and no rounding through double can differ (s / 3 is no
// float midpoint nor within 2^-29 ulp of one); everywhere else (q off by an
// ulp, s / 3 near a midpoint, q a power of two) the double expression
// decides.
// The double expression of third_of's rare cases, out of line.
static __device__ __noinline__ float third_of_double(float s) { return __double2float_rn((double)s / 3.0); }

__device__ __forceinline__ float third_of(float s)
{
    if (s == 0.0f) {
        return s;
    }
    constexpr float kThird = 0.333333343267440796f;  // fl(1/3)
    const float q0 = __fmul_rn(s, kThird);
    const float q = __fmaf_rn(__fmaf_rn(-3.0f, q0, s), kThird, q0);
    const float rem = __fmaf_rn(-3.0f, q, s);  // s - 3 q, exact
    if (rem == 0.0f) {
        return q;  // s / 3 is a float: every rounding gives it (white pixels: 3 / 3)
    }
    // s / 3 - q = rem / 3; a midpoint sits at +-ulp/2
    const float ulp = fabsf(__int_as_float(__float_as_int(q) + 1) - q);
    const float d = fabsf(rem) - 1.5f * ulp;  // 3 (|s/3 - q| - ulp/2), exact or nearly
    if (d < -1.0e-6f * ulp && (__float_as_int(q) & 0x7fffff) != 0) {
        return q;
    }
    return third_of_double(s);
}

// MultiGrayscaleAccessor on float RGB (src/mga.h:184-222).  The reference's
// RealPromote of float is float: the average adds the samples in float and
// divides by 3.0 in double, the lightness adds min and max in float;
// luminance (0.3/0.59/0.11) and the channel mixer are double expressions.
// m0 r + m1 g + m2 b in double (the luminance and channel-mixer projectors),
// out of line: the weight kernels' common projectors stay in float.
static __device__ __noinline__ float gray_mix_double(double m0, double m1, double m2, float r, float g, float b)
{
    return __double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(m0, (double)r), __dmul_rn(m1, (double)g)),
                                       __dmul_rn(m2, (double)b)));
}

// The projector with the channel-mixer weights m0..m2.
__device__ __forceinline__ float gray_proj_m(int projector, double m0, double m1, double m2, float r, float g, float b)
{
    switch (projector) {
    case ENB_GRAY_VALUE: return fmaxf(r, fmaxf(g, b));
    case ENB_GRAY_ANTI_VALUE: return fminf(r, fminf(g, b));
    case ENB_GRAY_LIGHTNESS: return 0.5f * __fadd_rn(fminf(r, fminf(g, b)), fmaxf(r, fmaxf(g, b)));
    case ENB_GRAY_LUMINANCE: return gray_mix_double(0.3, 0.59, 0.11, r, g, b);
    case ENB_GRAY_MIXER: return gray_mix_double(m0, m1, m2, r, g, b);
    default: return third_of(__fadd_rn(__fadd_rn(r, g), b));
    }
}

__device__ __forceinline__ float gray_proj_f(int projector, const FloatWeightParams& p, float r, float g, float b)
{
    return gray_proj_m(projector, p.mixer[0], p.mixer[1], p.mixer[2], r, g, b);
}

__device__ __forceinline__ float gray_of_f(const FloatWeightParams& p, float r, float g, float b)
{
    return gray_proj_f(p.gray_projector, p, r, g, b);
}

// ClampingFunctor of the entropy cutoff (src/enfuse.h:893-925) on float
// samples: x <= lo -> 0, x >= hi -> range, else x; the third sample is
// judged low by the first.
__device__ __forceinline__ void entropy_clamp_f(const FloatWeightParams& p, float (&rgb)[3], int C)
{
    const bool red_low = rgb[0] <= p.ent_lo;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        if (ch < C) {
            const bool low = (C == 3 && ch == 2) ? red_low : rgb[ch] <= p.ent_lo;
            rgb[ch] = low ? 0.0f : (rgb[ch] >= p.ent_hi ? p.range : rgb[ch]);
        }
    }
}

// The built-in exposure weight functions (src/exposure_weight.h:44-128).
// The reference forms y = gray / max in float (both operands are float) and
// z = (y - optimum) / width in double.  The Gaussian and the Lorentzian are
// evaluated from z in float (relative error of z a few ulps, of the weight at
// most that times z^2 / 2, where the Gaussian has fallen to exp(-z^2 / 2)).
// For the functions that vanish at the edge of their support (half-sine,
// full-sine, bisquare) z is carried as a float-float pair zh + zl (error
// ~1e-14 relative) so that they keep their relative accuracy there; each is
// then evaluated in float with a first-order correction for zl.
// The functions that vanish at the edge of their support, from y = gray /
// max (out of line: rare, and large with their sines).
static __device__ __noinline__ float exposure_f_support(int fn, float y, float opt_hi, float opt_lo, float inv_hi, float inv_lo)
{
    // d = y - (opt_hi + opt_lo) as dh + dl: TwoSum(y, -opt_hi), then opt_lo
    const float s = __fsub_rn(y, opt_hi);
    const float bv = __fsub_rn(s, y);
    const float e = __fadd_rn(__fsub_rn(y, __fsub_rn(s, bv)), __fsub_rn(-opt_hi, bv));
    const float dl0 = __fsub_rn(e, opt_lo);
    const float dh = __fadd_rn(s, dl0);
    const float dl = __fsub_rn(dl0, __fsub_rn(dh, s));
    // z = d * (inv_hi + inv_lo)
    const float zh = __fmul_rn(dh, inv_hi);
    const float zl = __fadd_rn(__fmaf_rn(dh, inv_hi, -zh), __fmaf_rn(dh, inv_lo, __fmul_rn(dl, inv_hi)));
    const float az = fabsf(zh);
    switch (fn) {
    case ENB_EXP_LORENTZIAN: return __fdiv_rn(1.0f, __fmaf_rn(0.5f * zh, zh, 1.0f));
    case ENB_EXP_HALF_SINE: {
        if (az > 1.57079632679489661923f) {
            return 0.0f;
        }
        float sn, cs;
        sincosf(zh, &sn, &cs);
        return fmaxf(__fmaf_rn(-sn, zl, cs), 0.0f);
    }
    case ENB_EXP_FULL_SINE: {
        if (az > 3.14159265358979323846f) {
            return 0.0f;
        }
        // 0.5 + cos(z) / 2 = cos(z / 2)^2, without the cancellation near z = pi
        float sn, cs;
        sincosf(0.5f * zh, &sn, &cs);
        const float c = __fmaf_rn(-sn, 0.5f * zl, cs);
        return c * c;
    }
    case ENB_EXP_BISQUARE: {
        if (az > 1.0f) {
            return 0.0f;
        }
        // (1 - z^2)(1 + z^2) with 1 - z^2 = (1 - zh)(1 + zh) - 2 zh zl
        const float one_minus = __fmaf_rn(-2.0f * zh, zl, __fmul_rn(1.0f - zh, 1.0f + zh));
        const float one_plus = __fmaf_rn(zh, zh, __fmul_rn(2.0f * zh, zl)) + 1.0f;
        return fmaxf(one_minus, 0.0f) * one_plus;
    }
    default: {
        // exp(-z^2 / 2) with z^2 / 2 = qh + ql
        const float qh = __fmul_rn(0.5f * zh, zh);
        const float ql = __fmaf_rn(0.5f * zh, zh, -qh) + zh * zl;
        return expf(-qh) * (1.0f - ql);
    }
    }
}


__device__ __forceinline__ float exposure_f(const FloatWeightParams& p, float gray)
{
    const float y = p.range == 1.0f ? gray : __fdiv_rn(gray, p.range);
    if (p.exp_function == ENB_EXP_GAUSSIAN || p.exp_function == ENB_EXP_LORENTZIAN) {
        const float z = __fmul_rn(__fsub_rn(y, p.opt_hi), p.inv_hi);
        const float q = __fmul_rn(__fmul_rn(0.5f, z), z);
        return p.exp_function == ENB_EXP_GAUSSIAN ? expf(-q) : __fdiv_rn(1.0f, __fadd_rn(1.0f, q));
    }
    return exposure_f_support(p.exp_function, y, p.opt_hi, p.opt_lo, p.inv_hi, p.inv_lo);
}

// Histogram::entropyOfChannel of n float keys sorted by bit pattern (equal
// floats are adjacent; -0 was folded into +0), src/enfuse.h:346-375.  The
// sum of p log p is exact in 2^-56 fixed point (host table; the tables of
// float images are built with max 1, so scale_logb[b] = 1 / log b); H <= 1.
__device__ __forceinline__ float entropy_f(const uint32_t* v, int n, const WeightTables& tab, int nmax)
{
    if (n == 0) {
        return 0.0f;
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
        return 0.0f;
    }
    const float H = __fmul_rn(-(float)acc * 1.3877787807814457e-17f, tab.scale_logb[bins]);  // 2^-56
    return fminf(H, 1.0f);
}


// ---- one exposure's tile in shared memory -----------------------------------

__host__ __device__ inline size_t align16_sz(size_t n) { return (n + 15) & ~(size_t)15; }

// Tile of (TW x TW) input pixels around a block of output pixels: gray,
// the three samples, the window counters (clip values, repeat marks, opaque
// flags; enb_entropy.cuh), the repeat hash tables and the opaque flags.
// TW is even (16 + 2 * halo), which keeps every array 16-byte aligned.
// With the entropy cutoff the entropy windows read their own, clamped
// copy of the samples (eraw); else eraw is raw.
struct FTile {
    float* gray;     // [TW*TW]
    float* raw;      // [3][TW*TW]
    uint64_t* cnt;   // [TW*TW]
    uint32_t* table; // [3][slots]
    uint8_t* flags;  // [3][slots]
    uint8_t* a;      // [TW*TW]
    float* eraw;     // [3][TW*TW] (entropy cutoff) or raw
    int TW, slots;
};

__host__ __device__ inline size_t ftile_bytes(int TW, int slots, int ent_cut = 0)
{
    return align16_sz((size_t)TW * TW * (4 * sizeof(float) + sizeof(uint64_t) + 1) + (size_t)slots * 3 * 5) +
           (ent_cut ? (size_t)TW * TW * 3 * sizeof(float) : 0);
}

__host__ __device__ inline size_t align16(size_t n) { return (n + 15) & ~(size_t)15; }

__device__ __forceinline__ FTile ftile_carve(unsigned char* smem, int TW, int slots, int ent_cut = 0)
{
    FTile t;
    t.TW = TW;
    t.slots = slots;
    t.gray = reinterpret_cast<float*>(smem);
    t.raw = t.gray + TW * TW;
    t.cnt = reinterpret_cast<uint64_t*>(t.raw + 3 * TW * TW);
    t.table = reinterpret_cast<uint32_t*>(t.cnt + TW * TW);
    t.flags = reinterpret_cast<uint8_t*>(t.table + 3 * slots);
    t.a = t.flags + 3 * slots;
    t.eraw = ent_cut ? reinterpret_cast<float*>(smem + ftile_bytes(TW, slots, 0)) : t.raw;
    return t;
}

// Writes tile pixel k from its samples and opaque flag.
__device__ __forceinline__ void ftile_put_px(const FTile& t, const FloatWeightParams& wp, int k, const float (&rgb)[3],
                                             uint8_t a, int C)
{
    const int TT = t.TW * t.TW;
    t.gray[k] = C == 1 ? rgb[0] : gray_of_f(wp, rgb[0], rgb[1], rgb[2]);
    t.a[k] = a;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        t.raw[ch * TT + k] = rgb[ch];
    }
    if (!wp.use_entropy) {
        return;  // the window counters and the clamped samples feed only the entropy
    }
    if (wp.ent_cut) {
        float e[3] = {rgb[0], rgb[1], rgb[2]};
        entropy_clamp_f(wp, e, C);
        t.cnt[k] = a ? (uint64_t)clip_counts(e, C) | (1ull << kCntOpaque) : 0ull;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            t.eraw[ch * TT + k] = e[ch];
        }
    } else {
        t.cnt[k] = a ? (uint64_t)clip_counts(rgb, C) | (1ull << kCntOpaque) : 0ull;
    }
}

// Samples and opaque flag of input pixel (gx, gy); zero and transparent
// outside the image.
__device__ __forceinline__ void ftile_fetch_px(float (&rgb)[3], uint8_t& a, const float* img, int64_t pitch, int stride,
                                               int w, int h, int C, const uint8_t* alpha, int64_t apitch, int gx, int gy)
{
    rgb[0] = rgb[1] = rgb[2] = 0.0f;
    a = 0;
    if (gx >= 0 && gx < w && gy >= 0 && gy < h) {
        const float* px = img + (int64_t)gy * pitch + (int64_t)gx * stride;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            if (ch < C) {
                rgb[ch] = __ldg(&px[ch]);
            }
        }
        a = alpha ? (__ldg(&alpha[(int64_t)gy * apitch + gx]) != 0) : 1;
    }
}

// Loads the tile whose top-left input pixel is (x0, y0) (all threads call;
// ends with the tile and its repeat marks complete in shared memory; the
// tile and its tables must be out of use since the block's previous
// barrier).  alpha == nullptr: opaque.  Returns nonzero when every tile
// pixel is opaque (and inside the image).
__device__ __forceinline__ int ftile_load(const FTile& t, const FloatWeightParams& wp, const float* img, int64_t pitch,
                                          int stride, int w, int h, int C, const uint8_t* alpha, int64_t apitch,
                                          int x0, int y0)
{
    const int TW = t.TW, TT = TW * TW;
    if (t.slots) {
        // the tables were last read before the block's previous barrier
        repeat_tables_clear(t.table, t.flags, C, t.slots);
    }
    // tile pixel k = r * TW + c, walked with a stride of blockDim.x
    const int dr = (int)blockDim.x / TW, dc = (int)blockDim.x - dr * TW;
    int r = (int)threadIdx.x / TW, c = (int)threadIdx.x - r * TW;
    int mine = 1;
    for (int k = threadIdx.x; k < TT; k += blockDim.x) {
        float rgb[3];
        uint8_t a;
        ftile_fetch_px(rgb, a, img, pitch, stride, w, h, C, alpha, apitch, x0 + c, y0 + r);
        ftile_put_px(t, wp, k, rgb, a, C);
        mine &= a;
        c += dc;
        r += dr;
        if (c >= TW) {
            c -= TW;
            ++r;
        }
    }
    const int opaque = __syncthreads_and(mine);
    if (t.slots) {
        if (TT <= 2 * (int)blockDim.x) {
            mark_repeats<2>(t.eraw, TT, t.a, TT, C, t.table, t.flags, t.slots, t.cnt);
        } else {
            mark_repeats<0>(t.eraw, TT, t.a, TT, C, t.table, t.flags, t.slots, t.cnt);
        }
    }
    return opaque;
}

// Sample standard deviation of the opaque window pixels (localStdDevIf,
// src/enfuse.h:75-219) in two passes around the float mean.  CW > 0: the
// window size at compile time; CW == 0: b is the runtime half-width.
// opaque: every tile pixel is opaque, so no tap is skipped (the same sums).
template <int CW>
__device__ __forceinline__ float window_stddev(const FTile& t, int ci, int bdyn, bool opaque)
{
    const int TW = t.TW;
    if (CW > 0 && opaque) {
        constexpr int B = CW / 2, N = (CW > 0 ? CW * CW : 1);
        float v[N];
        float sum = 0.0f;
#pragma unroll
        for (int dy = -B; dy <= B; ++dy) {
#pragma unroll
            for (int dx = -B; dx <= B; ++dx) {
                v[(dy + B) * CW + dx + B] = t.gray[ci + dy * TW + dx];
                sum += v[(dy + B) * CW + dx + B];
            }
        }
        const float mean = __fdiv_rn(sum, (float)N);
        float s1 = 0.0f, s2 = 0.0f;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const float d = v[i] - mean;
            s1 += d;
            s2 = fmaf(d, d, s2);
        }
        const float var = __fdiv_rn(s2 - __fdiv_rn(s1 * s1, (float)N), (float)(N - 1));
        return sqrtf(fmaxf(var, 0.0f));
    }
    const int b = CW > 0 ? CW / 2 : bdyn;
    float sum = 0.0f;
    int n = 0;
#pragma unroll
    for (int dy = -b; dy <= b; ++dy) {
#pragma unroll
        for (int dx = -b; dx <= b; ++dx) {
            const int idx = ci + dy * TW + dx;
            const bool on = t.a[idx] != 0;
            sum += on ? t.gray[idx] : 0.0f;
            n += on ? 1 : 0;
        }
    }
    if (n <= 1) {
        return 0.0f;
    }
    const float mean = __fdiv_rn(sum, (float)n);
    float s1 = 0.0f, s2 = 0.0f;
#pragma unroll
    for (int dy = -b; dy <= b; ++dy) {
#pragma unroll
        for (int dx = -b; dx <= b; ++dx) {
            const int idx = ci + dy * TW + dx;
            const float d = t.a[idx] ? t.gray[idx] - mean : 0.0f;
            s1 += d;
            s2 = fmaf(d, d, s2);
        }
    }
    const float var = __fdiv_rn(s2 - __fdiv_rn(s1 * s1, (float)n), (float)(n - 1));
    return sqrtf(fmaxf(var, 0.0f));
}

// H of channel ch of the entropy window at ci (EW: 3 or 5 at compile time,
// 0: the runtime window wp.entropy_window through an insertion sort).
template <int EW>
__device__ __forceinline__ float window_entropy(const FTile& t, const FloatWeightParams& wp, const WeightTables& tab,
                                                int ci, int ch, int nwin, uint32_t marks, uint32_t clips)
{
    const float* raw = t.eraw + ch * t.TW * t.TW;
    const int nmax = (EW > 0 ? EW * EW : wp.entropy_window * wp.entropy_window);
    if (EW > 0) {
        if (!(marks & (1u << ch))) {
            // no repeated sample besides the clip values: three counts
            return entropy_clip_bins(nwin, (int)((clips >> (5 * ch)) & 31u), (int)((clips >> (15 + 5 * ch)) & 31u),
                                     tab, nmax);
        }
        return entropy_window_float<(EW > 0 ? EW : 3)>(raw, t.a, t.TW, ci, tab);
    }
    const int b = wp.entropy_window / 2;
    uint32_t vals[kMaxEntropyWindow * kMaxEntropyWindow];
    int n = 0;
    for (int dy = -b; dy <= b; ++dy) {
        for (int dx = -b; dx <= b; ++dx) {
            const int idx = ci + dy * t.TW + dx;
            if (t.a[idx]) {
                const uint32_t v = float_key(raw[idx]);
                int q = n++;
                while (q > 0 && vals[q - 1] > v) {
                    vals[q] = vals[q - 1];
                    --q;
                }
                vals[q] = v;
            }
        }
    }
    return entropy_f(vals, n, tab, nmax);
}

// The enfuseMask weight of the output pixel (x, y) whose tile index is ci:
// exposure (assigned), + contrast, + saturation, + entropy, float adds in
// the reference's order (src/enfuse.h:1119-1120, 1133-1134, 1208-1209).
template <int CW, int EW>
__device__ __forceinline__ float f_pixel_weight(const FTile& t, const FloatWeightParams& wp, const WeightTables& tab,
                                                int ci, int x, int y, int w, int h, int C, bool opaque)
{
    if (!t.a[ci]) {
        return 0.0f;
    }
    float result = 0.0f;
    if (wp.use_exposure) {
        bool pass = true;
        if (wp.exp_cut) {
            float lv = t.gray[ci], uv = lv;
            if (C == 3) {
                const int TT = t.TW * t.TW;
                const float r = t.raw[ci], g = t.raw[TT + ci], bb = t.raw[2 * TT + ci];
                lv = gray_proj_f(wp.cut_proj[0], wp, r, g, bb);
                uv = gray_proj_f(wp.cut_proj[1], wp, r, g, bb);
            }
            pass = lv >= wp.cut_lo && uv <= wp.cut_hi;
        }
        result = pass ? wp.w_exposure * exposure_f(wp, t.gray[ci]) : 0.0f;
    }
    if (wp.use_contrast) {
        const int b = wp.contrast_window / 2;
        float sd = 0.0f;  // the border strip is not written (0)
        if (x >= b && x < w - b && y >= b && y < h - b) {
            sd = window_stddev<CW>(t, ci, b, opaque);
        }
        result = wp.w_contrast * sd + result;
    }
    if (wp.use_saturation && C == 3) {
        // SaturationFunctor with max_value 1.0 (src/enfuse.h:733-780);
        // 2 - (max + min) is formed as (1 - max) + (1 - min), whose terms
        // are exact near white
        const int TT = t.TW * t.TW;
        const float r = t.raw[ci], g = t.raw[TT + ci], bb = t.raw[2 * TT + ci];
        const float mx = fmaxf(r, fmaxf(g, bb)), mn = fminf(r, fminf(g, bb));
        float sw = 0.0f;
        if (mx != mn) {
            const float sum = mx + mn, diff = mx - mn;
            const float den = sum <= 1.0f ? sum : (1.0f - mx) + (1.0f - mn);
            sw = wp.w_saturation * __fdiv_rn(diff, den);
        }
        result = sw + result;
    }
    if (wp.use_entropy) {
        const int b = wp.entropy_window / 2;
        float emin = 0.0f;
        if (x >= b && x < w - b && y >= b && y < h - b) {
            int nwin = 0;
            uint32_t marks = 0xffu, clips = 0;
            if (EW > 0 && t.slots) {
                window_counts<(EW > 0 ? EW : 3)>(t.cnt, t.TW, ci, nwin, marks, clips);
            }
            emin = 3.402823466e38f;
            for (int ch = 0; ch < C; ++ch) {
                // fromRealPromote<float>(H * max): the entropy image pixel
                emin = fminf(emin, __fmul_rn(window_entropy<EW>(t, wp, tab, ci, ch, nwin, marks, clips), wp.range));
            }
        }
        result = __fmul_rn(wp.w_entropy, emin) + result;
    }
    return result;
}

// Halo of the weight windows and the hash slots of the repeat marks.
__host__ __device__ inline int fweight_halo(const FloatWeightParams& wp)
{
    const int hc = wp.use_contrast ? wp.contrast_window / 2 : 0, he = wp.use_entropy ? wp.entropy_window / 2 : 0;
    return hc > he ? hc : he;
}

inline int fweight_slots(const FloatWeightParams& wp, int TW)
{
    if (!wp.use_entropy || (wp.entropy_window != 3 && wp.entropy_window != 5)) {
        return 0;
    }
    int slots = 64;
    while (slots < 2 * TW * TW) {
        slots <<= 1;
    }
    return slots;
}

}  // namespace enb
