// enb_device.cuh -- device helpers shared by the kernels of the
// enblend/enfuse path: VIGRA conversion semantics, expand weights, tile
// geometry and the dither hash.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "enbgpu.h"

namespace enb {

// Reduce tiles: 32x8 destination pixels from a 67x19 source window.
constexpr int RTW = 32, RTH = 8;
constexpr int RIW = 2 * RTW + 3, RIH = 2 * RTH + 3;
// Expand tiles: 64x16 destination pixels (2x2 quads of 32x8 source pixels)
// from a 34x10 source window.
constexpr int ETW = 64, ETH = 16;
constexpr int ESW = ETW / 2 + 2, ESH = ETH / 2 + 2;

template <typename T>
__device__ __forceinline__ T cast_store(int64_t v);  // static_cast into the pyramid type

template <>
__device__ __forceinline__ int16_t cast_store<int16_t>(int64_t v) { return (int16_t)(uint16_t)(v & 0xffff); }

template <>
__device__ __forceinline__ int32_t cast_store<int32_t>(int64_t v) { return (int32_t)(uint32_t)(v & 0xffffffffu); }

// NumericTraits<T>::fromPromote: saturate Int16, identity for Int32.
template <typename T>
__device__ __forceinline__ T sat_store(int32_t v);

template <>
__device__ __forceinline__ int16_t sat_store<int16_t>(int32_t v) { return (int16_t)min(max(v, -32768), 32767); }

template <>
__device__ __forceinline__ int32_t sat_store<int32_t>(int32_t v) { return v; }

// NumericTraits<T>::fromRealPromote of a double: +-0.5 and a truncating
// cast, saturating at the type limits.
template <typename T>
__device__ __forceinline__ T frp_store(double v);

template <>
__device__ __forceinline__ int32_t frp_store<int32_t>(double v)
{
    if (v < 0.0) {
        return v < -2147483648.0 ? INT32_MIN : __double2int_rz(__dadd_rn(v, -0.5));
    }
    return v > 2147483647.0 ? INT32_MAX : __double2int_rz(__dadd_rn(v, 0.5));
}

template <>
__device__ __forceinline__ int16_t frp_store<int16_t>(double v)
{
    if (v < 0.0) {
        return v < -32768.0 ? (int16_t)-32768 : (int16_t)__double2int_rz(__dadd_rn(v, -0.5));
    }
    return v > 32767.0 ? (int16_t)32767 : (int16_t)__double2int_rz(__dadd_rn(v, 0.5));
}

__device__ __forceinline__ uint32_t frp_unsigned(double v, uint32_t maxv)
{
    if (v < 0.0) {
        return 0u;
    }
    return v > (double)maxv ? maxv : (uint32_t)__double2uint_rz(__dadd_rn(v, 0.5));
}

__host__ __device__ __forceinline__ int imod(int a, int m)
{
    int r = a % m;
    return r < 0 ? r + m : r;
}

__device__ __forceinline__ uint32_t load_sample(const void* p, int dtype, int64_t i)
{
    return dtype == ENB_U8 ? (uint32_t)reinterpret_cast<const uint8_t*>(p)[i]
                           : (uint32_t)reinterpret_cast<const uint16_t*>(p)[i];
}

template <typename TIn, int S>
__device__ __forceinline__ void load_pixel(const TIn* px, TIn (&p)[S])
{
#pragma unroll
    for (int c = 0; c < S; ++c) {
        p[c] = px[c];
    }
}

template <typename TIn, int S>
__device__ __forceinline__ void store_pixel(TIn* px, const TIn (&p)[S])
{
#pragma unroll
    for (int c = 0; c < S; ++c) {
        px[c] = p[c];
    }
}

static inline dim3 grid2d(int w, int h, int tw, int th)
{
    return dim3((unsigned)((w + tw - 1) / tw), (unsigned)((h + th - 1) / th));
}

// Horizontal expand weights on source offsets (-1, 0, +1) of destination
// column X and their divisor; the SKIPSM scale tables of
// src/pyramid.h:1227-1411 factor into these per-axis divisors.
__device__ __forceinline__ void expand_hweights(int X, int sw, int dw, int wrap, int w[3], int& den)
{
    const int i = X >> 1;
    if ((X & 1) == 0) {
        if (wrap && sw == 1) {
            // single source column: the wrapped left state joins the
            // numerator over the plain divisor (src/pyramid.h:1233-1236,1304-1307)
            w[0] = 0;
            w[1] = (dw & 1) ? 10 : 7;
            w[2] = 0;
            den = 6;
            return;
        }
        w[0] = 1;
        w[1] = 6;
        w[2] = 1;
        if (wrap) {
            if (dw & 1) {
                if (i == 0) {
                    w[0] = 4;
                }
                if (i == sw - 1) {
                    w[2] = 4;
                }
            }
        } else {
            if (i == 0) {
                w[0] = 0;
            }
            if (i + 1 >= sw) {
                w[2] = 0;
            }
        }
    } else {
        w[0] = 0;
        w[1] = 4;
        w[2] = (i + 1 < sw || (wrap && sw > 1)) ? 4 : 0;
    }
    den = w[0] + w[1] + w[2];
}

__device__ __forceinline__ void expand_vweights(int Y, int sh, int w[3], int& den)
{
    const int j = Y >> 1;
    if ((Y & 1) == 0) {
        w[0] = j > 0 ? 1 : 0;
        w[1] = 6;
        w[2] = j + 1 < sh ? 1 : 0;
    } else {
        w[0] = 0;
        w[1] = 1;
        w[2] = j + 1 < sh ? 1 : 0;
    }
    den = w[0] + w[1] + w[2];
}

// Truncating division by a divisor known only at run time, kept out of line so
// that the compiler branches around it instead of predicating it into the
// common path (the divisor is a power-of-two constant there).
static __device__ __noinline__ int32_t div_any(int32_t num, int32_t den) { return num / den; }

__device__ __forceinline__ int32_t div_den(int32_t num, int den)
{
    if (den == 64) {
        return num / 64;
    }
    if (den == 16) {
        return num / 16;
    }
    return div_any(num, den);
}

// 32-bit integer finaliser (public-domain "lowbias32" constants by C. Wellons).
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// Random bits of the dither (same rule as the oracle): one hash per pixel,
// 8 bits per channel when the rule needs at most 8 bits per sample and the
// pixel has at most four samples, otherwise one hash per sample.  The pixel
// index wraps at 2^32.
__host__ __device__ __forceinline__ uint32_t dither_key(uint64_t seed)
{
    return mix32((uint32_t)(seed >> 32) ^ 0x9e3779b9u) ^ (uint32_t)seed;
}

__device__ __forceinline__ bool dither_per_pixel(int C, int frac) { return frac - 1 <= 8 && C <= 4; }

__device__ __forceinline__ uint32_t dither_sample_bits(uint32_t key, uint32_t pixbits, uint64_t pixel, int C, int c,
                                                       int frac)
{
    return dither_per_pixel(C, frac) ? pixbits >> (8 * c)
                                     : mix32((uint32_t)(pixel * (uint64_t)C + (uint64_t)c) ^ key);
}

// The conversion rule of SpecializedConvertPyramidToScalarFunctor
// (src/fixmath.h:251-277): q = v >> F, fraction f; f < 1/4 -> q,
// f >= 3/4 -> q+1, in between q+1 iff (random & (2^(F-1)-1)) + 1/4 <= f;
// then fromPromote into [0, maxv].  `bits` is consumed only in the band.
__device__ __forceinline__ int32_t dither_rule(int32_t v, int frac, int nearest, uint32_t bits, int32_t maxv)
{
    const int32_t q = v >> frac;
    const int32_t f = v & ((1 << frac) - 1);
    const int32_t quarter = 1 << (frac - 2);
    int32_t r;
    if (nearest) {
        r = f >= (1 << (frac - 1)) ? q + 1 : q;
    } else if (f >= quarter && f < 3 * quarter) {
        const int32_t rnd = (int32_t)(bits & (uint32_t)((1 << (frac - 1)) - 1)) + quarter;
        r = rnd <= f ? q + 1 : q;
    } else {
        r = f >= quarter ? q + 1 : q;
    }
    return min(max(r, 0), maxv);
}

// Second half of the reduce with alpha: separable [1 4 6 4 1] sums over the
// staged window (values already zero where transparent), normalisation by the
// opaque weight sum with a truncating division, destination alpha 255/0.
template <typename TD, int C>
__device__ __forceinline__ void reduce_alpha_finish(int32_t (*sv)[RIH][RIW], int32_t (*sm)[RIW],
                                                    int32_t (*hv)[RIH][RTW], int32_t (*hm)[RTW], int X0, int Y0,
                                                    TD* __restrict__ dst, int64_t dpitch, int64_t dplane, int dw,
                                                    int dh, uint8_t* __restrict__ da, int64_t dapitch)
{
    const int tid = threadIdx.x;
    for (int i = tid; i < RIH * RTW; i += 256) {
        const int r = i / RTW, j = i - r * RTW;
        const int c0 = 2 * j;
        hm[r][j] = sm[r][c0] + 4 * sm[r][c0 + 1] + 6 * sm[r][c0 + 2] + 4 * sm[r][c0 + 3] + sm[r][c0 + 4];
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            hv[ch][r][j] = sv[ch][r][c0] + 4 * sv[ch][r][c0 + 1] + 6 * sv[ch][r][c0 + 2] +
                           4 * sv[ch][r][c0 + 3] + sv[ch][r][c0 + 4];
        }
    }
    __syncthreads();
    const int tx = tid % RTW, ty = tid / RTW;
    const int X = X0 + tx, Y = Y0 + ty;
    if (X >= dw || Y >= dh) {
        return;
    }
    const int r0 = 2 * ty;
    const int den = hm[r0][tx] + 4 * hm[r0 + 1][tx] + 6 * hm[r0 + 2][tx] + 4 * hm[r0 + 3][tx] + hm[r0 + 4][tx];
    if (den > 0) {
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            const int32_t num = hv[ch][r0][tx] + 4 * hv[ch][r0 + 1][tx] + 6 * hv[ch][r0 + 2][tx] +
                                4 * hv[ch][r0 + 3][tx] + hv[ch][r0 + 4][tx];
            const int32_t q = den == 256 ? num / 256 : num / den;
            dst[(int64_t)ch * dplane + (int64_t)Y * dpitch + X] = cast_store<TD>(q);
        }
        da[(int64_t)Y * dapitch + X] = 255;
    } else {
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            dst[(int64_t)ch * dplane + (int64_t)Y * dpitch + X] = (TD)0;
        }
        da[(int64_t)Y * dapitch + X] = 0;
    }
}

// Second half of the alpha-free reduce: separable sums, /256.
template <typename TD, int C>
__device__ __forceinline__ void reduce_noalpha_finish(int32_t (*sv)[RIH][RIW], int32_t (*hv)[RIH][RTW], int X0,
                                                      int Y0, TD* __restrict__ dst, int64_t dpitch, int64_t dplane,
                                                      int dw, int dh)
{
    const int tid = threadIdx.x;
    for (int i = tid; i < RIH * RTW; i += 256) {
        const int r = i / RTW, j = i - r * RTW;
        const int c0 = 2 * j;
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            hv[ch][r][j] = sv[ch][r][c0] + 4 * sv[ch][r][c0 + 1] + 6 * sv[ch][r][c0 + 2] +
                           4 * sv[ch][r][c0 + 3] + sv[ch][r][c0 + 4];
        }
    }
    __syncthreads();
    const int tx = tid % RTW, ty = tid / RTW;
    const int X = X0 + tx, Y = Y0 + ty;
    if (X >= dw || Y >= dh) {
        return;
    }
    const int r0 = 2 * ty;
#pragma unroll
    for (int ch = 0; ch < C; ++ch) {
        const int32_t num = hv[ch][r0][tx] + 4 * hv[ch][r0 + 1][tx] + 6 * hv[ch][r0 + 2][tx] +
                            4 * hv[ch][r0 + 3][tx] + hv[ch][r0 + 4][tx];
        dst[(int64_t)ch * dplane + (int64_t)Y * dpitch + X] = cast_store<TD>(num / 256);
    }
}

}  // namespace enb
