// enb_device.cuh -- device helpers shared by the kernels of the
// enblend/enfuse path: VIGRA conversion semantics, expand weights, tile
// geometry and the dither hash.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "enbgpu.h"

namespace enb {

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

// Exact fromRealPromote(m * 2^frac) for 0 <= m * 2^frac < 2^23 in float
// arithmetic: the product is exact, floor and the fractional part are exact.
template <typename TD>
__device__ __forceinline__ TD mask_to_fixed(float m, int frac)
{
    const float v = m * (float)(1u << frac);
    if (v >= 0.0f && v < 8388608.0f) {
        const float fl = floorf(v);
        const int r = (int)fl + ((v - fl) >= 0.5f ? 1 : 0);
        return (TD)r;
    }
    return frp_store<TD>(__dmul_rn((double)m, (double)(1u << frac)));
}

// fromRealPromote(lp * fl(m / D)) with D = 255 * 2^F (src/enfuse.h:601-620).
//
// For 0 < m < D the exact value t = lp*m/D has denominator 2D after adding
// 1/2, so its distance to the rounding boundary is either 0 or >= 1/(2D);
// the double expression differs from t by < 2^-26, which is smaller.  Hence
// round-half-away(t) is the reference's result unless t is exactly a
// half-integer, in which case the double expression is evaluated as is.
template <typename T, int F>
__device__ __forceinline__ T mask_multiply(int32_t lp, int32_t m)
{
    constexpr int32_t D = 255 << F;
    if (m == 0) {
        return (T)0;  // lp * 0.0 rounds to 0
    }
    if (m == D) {
        return (T)lp;  // coefficient exactly 1.0
    }
    const uint32_t a = lp < 0 ? (uint32_t)(-(int64_t)lp) : (uint32_t)lp;
    if (m > 0 && m < D && a < (1u << 24)) {
        const uint64_t N = 2ull * (uint64_t)a * (uint64_t)m + (uint64_t)D;
        const uint32_t hi = (uint32_t)(N >> (F + 1));
        const uint32_t lo = (uint32_t)(N & ((1ull << (F + 1)) - 1));
        const uint32_t q = hi / 255u;
        const bool tie = lo == 0 && hi == q * 255u;
        if (!tie) {
            const int32_t r = lp < 0 ? -(int32_t)q : (int32_t)q;
            return sizeof(T) == 2 ? (T)min(max(r, -32768), 32767) : (T)r;
        }
    }
    const double coeff = __ddiv_rn((double)m, (double)D);
    return frp_store<T>(__dmul_rn((double)lp, coeff));
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

// Global load through the read-only path (NC: no thread of the launch writes
// the data) or a load cached in L2 only (the data was written earlier in the
// same launch, possibly by another SM, and is read only after the barrier or
// the release/acquire counter that follows the write; L2 is coherent across
// SMs, the SMs' L1 caches are not).
template <bool NC, typename T>
__device__ __forceinline__ T ld_src(const T* p)
{
    if (NC) {
        return __ldg(p);
    }
    return __ldcg(p);
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

// Truncating division by a divisor d in [1, 256] known only at run time, as a
// multiplication (division by invariant integers, Granlund & Montgomery
// 1994): with l = ceil(log2 d) and m = floor(2^(31+l) / d) + 1 < 2^32,
// floor(x / d) = (x * m) >> (31 + l) for every 0 <= x < 2^31.  The table
// holds m | (31 + l) << 32 per divisor; it is read through the read-only
// cache, so lanes with different divisors do not serialise.
struct DivTable {
    uint64_t e[257];
};

constexpr DivTable make_div_table()
{
    DivTable t{};
    for (int d = 1; d <= 256; ++d) {
        int l = 0;
        while ((1 << l) < d) {
            ++l;
        }
        const uint64_t m = ((uint64_t)1 << (31 + l)) / (uint64_t)d + 1;
        t.e[d] = m | ((uint64_t)(31 + l) << 32);
    }
    return t;
}

static __device__ const DivTable g_div_table = make_div_table();

__device__ __forceinline__ int32_t div_any(int32_t num, int32_t den)
{
    const uint32_t a = num < 0 ? 0u - (uint32_t)num : (uint32_t)num;
    if (den < 1 || den > 256 || a >= 0x80000000u) {
        return num / den;
    }
    const uint64_t e = __ldg(&g_div_table.e[den]);
    const uint32_t q = (uint32_t)(((uint64_t)a * (uint32_t)e) >> (uint32_t)(e >> 32));
    return num < 0 ? -(int32_t)q : (int32_t)q;
}

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

// Programmatic dependent launch: a kernel launched with the programmatic
// stream serialization attribute may start while its predecessor on the
// stream drains; griddep_wait() blocks (in hardware) until the predecessor
// has completed and its writes are visible, and must precede every access to
// data the predecessor wrote.  griddep_launch() lets the successor be
// scheduled.  Both are no-ops for kernels launched without the attribute.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

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
// (src/fixmath.h:251-277): q = v >> F, fraction f, Q = 2^(F-2); f < Q -> q,
// f >= 3Q -> q+1, in between q+1 iff (random & (2Q-1)) + Q <= f; then
// fromPromote into [0, maxv].  With t = (random & (2Q-1)) + Q, which lies in
// [Q, 3Q-1], all three cases are "q+1 iff f >= t", i.e. (v + 4Q - t) >> F;
// round-to-nearest is t = 2Q.  v is capped below 2^31 - 4Q first (F <= 15 and
// maxv <= 65535 keep the result at maxv there).
__device__ __forceinline__ int32_t dither_rule(int32_t v, int frac, int nearest, uint32_t bits, int32_t maxv)
{
    const int32_t Q = 1 << (frac - 2);
    const int32_t t = nearest ? 2 * Q : (int32_t)(bits & (uint32_t)(2 * Q - 1)) + Q;
    const int32_t vc = min(v, INT32_MAX - 4 * Q);
    return min(max((vc + 4 * Q - t) >> frac, 0), maxv);
}

// CartesianBlendFunctor of one sample (src/blend.h:41-76) in integers.
//
// The reference evaluates fromRealPromote(wc*lw + (1-wc)*lb) in double with
// wc = fl(m/W).  For 0 < m < W the exact value v = N/W, N = m*lw + (W-m)*lb,
// is either a half-integer or at least 1/(2W) away from one.  The double
// evaluation, including the +-0.5 of the conversion, stays within
// 7.2 * M * 2^-53 of v (M = max(|lw|, |lb|)): below 1/(2W) whenever
// M*W < 2^48.  Then rounding v half away from zero is the reference's result;
// exact half-integers and larger operands take the reference's double
// expression.  floor(t / (255*2^k)) = floor(floor(t / 2^k) / 255), and
// floor(x / 255) = mulhi(x, 0x8080808080808081) >> 7 for all 64-bit x.
template <typename T>
__device__ __forceinline__ int32_t blend_sample(int32_t m, int32_t W, int32_t lw, int32_t lb)
{
    if (m >= W) {
        return lw;
    }
    if (m <= 0) {
        return lb;
    }
    const uint32_t aw = lw < 0 ? 0u - (uint32_t)lw : (uint32_t)lw;
    const uint32_t ab = lb < 0 ? 0u - (uint32_t)lb : (uint32_t)lb;
    if ((uint64_t)max(aw, ab) * (uint64_t)W < (1ull << 48)) {
        const int64_t n = (int64_t)m * lw + (int64_t)(W - m) * lb;
        const uint64_t t = 2ull * (uint64_t)(n < 0 ? -n : n) + (uint64_t)W;
        const uint64_t d = 2ull * (uint64_t)W;
        const int wf = __ffs(W) - 1;
        const uint64_t q =
            (W >> wf) == 255 ? __umul64hi(t >> (wf + 1), 0x8080808080808081ull) >> 7 : t / d;
        if (t != q * d) {
            return n < 0 ? -(int32_t)q : (int32_t)q;
        }
    }
    const double wc = __ddiv_rn((double)m, (double)W);
    const double bc = __dadd_rn(1.0, -wc);
    return (int32_t)frp_store<T>(__dadd_rn(__dmul_rn(wc, (double)lw), __dmul_rn(bc, (double)lb)));
}

}  // namespace enb
