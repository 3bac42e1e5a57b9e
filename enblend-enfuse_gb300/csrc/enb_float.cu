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
#include "enb_internal.h"

namespace enb {

namespace {

inline dim3 row_grid(int w, int h) { return dim3((unsigned)((w + 255) / 256), (unsigned)h); }
inline double npix(int w, int h) { return (double)w * (double)h; }

}  // namespace

// ---------------------------------------------------------------------------
// Conversions (src/fixmath.h:165-187, 320-329)
// ---------------------------------------------------------------------------

__device__ __forceinline__ float to_pyramid_value(float v)
{
    return v >= 0.0f ? __fadd_rn(1.0f, log1pf(v)) : __fdiv_rn(1.0f, __fsub_rn(1.0f, v));
}

__device__ __forceinline__ float from_pyramid_value(float v)
{
    return v >= 1.0f ? expm1f(__fsub_rn(v, 1.0f)) : __fsub_rn(1.0f, __fdiv_rn(1.0f, v));
}

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
    const float coeff = (float)mask[(int64_t)y * mpitch + x] * inv_divisor;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const float v = lp[(int64_t)c * lplane + (int64_t)y * lpitch + x] * coeff;
        float* r = &res[(int64_t)c * rplane + (int64_t)y * rpitch + x];
        *r = accumulate ? *r + v : v;
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
// enfuse weights of float images (src/enfuse.h:962-1212)
// ---------------------------------------------------------------------------

constexpr int FWT = 16;  // 16x16 weight pixels per CTA

// fl(fl_double(s / 3)) of a float s, the reference's (float)(s / 3.0), in
// float arithmetic: q1 = fl(s / 3) is the correctly rounded quotient, which
// is the result unless s / 3 lies within 2^-29 ulp of a float rounding
// midpoint (where rounding through double could differ).  The remainder
// s - 3 q1 is exact (fmaf) and locates s / 3 relative to q1; near a midpoint
// the double expression decides.
__device__ __forceinline__ float third_of(float s)
{
    if (s == 0.0f) {
        return s;
    }
    const float q1 = __fdiv_rn(s, 3.0f);
    const float rem = __fmaf_rn(-3.0f, q1, s);  // s - 3 q1, exact
    // s / 3 - q1 = rem / 3; a midpoint sits at +-ulp/2
    const float ulp = fabsf(__int_as_float(__float_as_int(q1) + 1) - q1);
    const float d = fabsf(rem) - 1.5f * ulp;  // 3 (|s/3 - q1| - ulp/2), exact or nearly
    if (fabsf(d) > 1.0e-6f * ulp && (__float_as_int(q1) & 0x7fffff) != 0) {
        return q1;
    }
    return __double2float_rn((double)s / 3.0);
}

// MultiGrayscaleAccessor on float RGB (src/mga.h:184-222).  The reference's
// RealPromote of float is float: the average adds the samples in float and
// divides by 3.0 in double, the lightness adds min and max in float;
// luminance (0.3/0.59/0.11) and the channel mixer are double expressions.
__device__ __forceinline__ float gray_of_f(const FloatWeightParams& p, float r, float g, float b)
{
    switch (p.gray_projector) {
    case ENB_GRAY_VALUE: return fmaxf(r, fmaxf(g, b));
    case ENB_GRAY_ANTI_VALUE: return fminf(r, fminf(g, b));
    case ENB_GRAY_LIGHTNESS: return 0.5f * __fadd_rn(fminf(r, fminf(g, b)), fmaxf(r, fmaxf(g, b)));
    case ENB_GRAY_LUMINANCE:
        return __double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(0.3, (double)r), __dmul_rn(0.59, (double)g)),
                                           __dmul_rn(0.11, (double)b)));
    case ENB_GRAY_MIXER:
        return __double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(p.mixer[0], (double)r), __dmul_rn(p.mixer[1], (double)g)),
                                           __dmul_rn(p.mixer[2], (double)b)));
    default: return third_of(__fadd_rn(__fadd_rn(r, g), b));
    }
}

// The built-in exposure weight functions (src/exposure_weight.h:44-128).
// The reference forms y = gray / max in float (both operands are float) and
// z = (y - optimum) / width in double.  Here z is carried as a float-float
// pair zh + zl (error ~1e-14 relative), so that the functions that vanish at
// the edge of their support (half-sine, full-sine, bisquare) keep their
// relative accuracy there; each function is then evaluated in float with a
// first-order correction for zl.
__device__ __forceinline__ float exposure_f(const FloatWeightParams& p, float gray)
{
    const float y = __fdiv_rn(gray, p.range);
    // d = y - (opt_hi + opt_lo) as dh + dl: TwoSum(y, -opt_hi), then opt_lo
    const float s = __fsub_rn(y, p.opt_hi);
    const float bv = __fsub_rn(s, y);
    const float e = __fadd_rn(__fsub_rn(y, __fsub_rn(s, bv)), __fsub_rn(-p.opt_hi, bv));
    const float dl0 = __fsub_rn(e, p.opt_lo);
    const float dh = __fadd_rn(s, dl0);
    const float dl = __fsub_rn(dl0, __fsub_rn(dh, s));
    // z = d * (inv_hi + inv_lo)
    const float zh = __fmul_rn(dh, p.inv_hi);
    const float zl = __fadd_rn(__fmaf_rn(dh, p.inv_hi, -zh), __fmaf_rn(dh, p.inv_lo, __fmul_rn(dl, p.inv_hi)));
    const float az = fabsf(zh);
    switch (p.exp_function) {
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

// Histogram::entropyOfChannel of n float keys sorted by bit pattern (equal
// floats are adjacent; -0 was folded into +0), src/enfuse.h:346-375.  The
// sum of p log p is exact in 2^-56 fixed point (host table; the tables of
// float images are built with max 1, so scale_logb[b] = 1 / log b); H <= 1.
__device__ float entropy_f(const uint32_t* v, int n, const WeightTables& tab, int nmax)
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

__global__ void __launch_bounds__(256) k_f_enfuse_mask(FloatPixelView img, const uint8_t* __restrict__ alpha,
                                                       int64_t apitch, FloatWeightParams wp, WeightTables tab,
                                                       float* __restrict__ out, int64_t opitch)
{
    extern __shared__ __align__(16) unsigned char fsmem[];
    const int halo = max(wp.use_contrast ? wp.contrast_window / 2 : 0, wp.use_entropy ? wp.entropy_window / 2 : 0);
    const int TW = FWT + 2 * halo;
    float* s_gray = reinterpret_cast<float*>(fsmem);
    float* s_raw = s_gray + TW * TW;  // [3][TW*TW]
    uint8_t* s_a = reinterpret_cast<uint8_t*>(s_raw + 3 * TW * TW);

    const int x0 = blockIdx.x * FWT - halo, y0 = blockIdx.y * FWT - halo;
    const int w = img.w, h = img.h, C = img.C;
    for (int k = threadIdx.x; k < TW * TW; k += blockDim.x) {
        const int r = k / TW, c = k - r * TW;
        const int gx = x0 + c, gy = y0 + r;
        float rgb[3] = {0.0f, 0.0f, 0.0f};
        uint8_t a = 0;
        if (gx >= 0 && gx < w && gy >= 0 && gy < h) {
            const float* px = img.p + (int64_t)gy * img.pitch + (int64_t)gx * img.stride;
            for (int ch = 0; ch < C; ++ch) {
                rgb[ch] = __ldg(&px[ch]);
            }
            a = alpha[(int64_t)gy * apitch + gx] != 0;
        }
        s_gray[k] = C == 1 ? rgb[0] : gray_of_f(wp, rgb[0], rgb[1], rgb[2]);
        s_a[k] = a;
        for (int ch = 0; ch < 3; ++ch) {
            s_raw[ch * TW * TW + k] = rgb[ch];
        }
    }
    __syncthreads();

    const int lx = threadIdx.x % FWT, ly = threadIdx.x / FWT;
    const int x = blockIdx.x * FWT + lx, y = blockIdx.y * FWT + ly;
    if (x >= w || y >= h) {
        return;
    }
    const int ci = (ly + halo) * TW + (lx + halo);
    float result = 0.0f;
    if (s_a[ci]) {
        if (wp.use_exposure) {
            result = wp.w_exposure * exposure_f(wp, s_gray[ci]);
        }
        if (wp.use_contrast) {
            // sample standard deviation of the opaque window pixels
            // (localStdDevIf, src/enfuse.h:75-219), two passes around the
            // float mean; the border strip is not written (0)
            const int b = wp.contrast_window / 2;
            float sd = 0.0f;
            if (x >= b && x < w - b && y >= b && y < h - b) {
                float sum = 0.0f;
                int n = 0;
                for (int dy = -b; dy <= b; ++dy) {
                    const int row = (ly + halo + dy) * TW + lx + halo;
                    for (int dx = -b; dx <= b; ++dx) {
                        if (s_a[row + dx]) {
                            sum += s_gray[row + dx];
                            ++n;
                        }
                    }
                }
                if (n > 1) {
                    const float mean = __fdiv_rn(sum, (float)n);
                    float s1 = 0.0f, s2 = 0.0f;
                    for (int dy = -b; dy <= b; ++dy) {
                        const int row = (ly + halo + dy) * TW + lx + halo;
                        for (int dx = -b; dx <= b; ++dx) {
                            if (s_a[row + dx]) {
                                const float d = s_gray[row + dx] - mean;
                                s1 += d;
                                s2 = fmaf(d, d, s2);
                            }
                        }
                    }
                    const float var = __fdiv_rn(s2 - __fdiv_rn(s1 * s1, (float)n), (float)(n - 1));
                    sd = sqrtf(fmaxf(var, 0.0f));
                }
            }
            result = wp.w_contrast * sd + result;
        }
        if (wp.use_saturation && C == 3) {
            // SaturationFunctor with max_value 1.0 (src/enfuse.h:733-780);
            // 2 - (max + min) is formed as (1 - max) + (1 - min), whose terms
            // are exact near white
            const float r = s_raw[ci], g = s_raw[TW * TW + ci], bb = s_raw[2 * TW * TW + ci];
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
                uint32_t vals[kMaxEntropyWindow * kMaxEntropyWindow];
                const int nmax = wp.entropy_window * wp.entropy_window;
                emin = 3.402823466e38f;
                for (int ch = 0; ch < C; ++ch) {
                    int n = 0;
                    for (int dy = -b; dy <= b; ++dy) {
                        const int row = (ly + halo + dy) * TW + lx + halo;
                        for (int dx = -b; dx <= b; ++dx) {
                            if (s_a[row + dx]) {
                                const float f = s_raw[ch * TW * TW + row + dx];
                                const uint32_t v = __float_as_uint(f == 0.0f ? 0.0f : f);
                                int q = n++;
                                while (q > 0 && vals[q - 1] > v) {
                                    vals[q] = vals[q - 1];
                                    --q;
                                }
                                vals[q] = v;
                            }
                        }
                    }
                    // fromRealPromote<float>(H * max): the entropy image pixel
                    emin = fminf(emin, __fmul_rn(entropy_f(vals, n, tab, nmax), wp.range));
                }
            }
            result = __fmul_rn(wp.w_entropy, emin) + result;
        }
    }
    out[(int64_t)y * opitch + x] = result;
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

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
    const int halo = max(wp.use_contrast ? wp.contrast_window / 2 : 0, wp.use_entropy ? wp.entropy_window / 2 : 0);
    const int TW = FWT + 2 * halo;
    const size_t smem = (size_t)TW * TW * (4 * sizeof(float) + 1);
    note_launch("f_enfuse_mask", npix(img.w, img.h) * (img.stride * 4.0 + 1.0 + 4.0));
    if (smem > 48 * 1024) {
        cudaFuncSetAttribute(k_f_enfuse_mask, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    k_f_enfuse_mask<<<grid2d(img.w, img.h, FWT, FWT), FWT * FWT, smem, st>>>(img, alpha.p, alpha.pitch, wp, tab, out.p,
                                                                             out.pitch);
    return cudaGetLastError();
}

}  // namespace enb
