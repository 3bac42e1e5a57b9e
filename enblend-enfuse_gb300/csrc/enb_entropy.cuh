// enb_entropy.cuh -- local entropy of one window channel
// (Histogram::entropyOfChannel, src/enfuse.h:346-375) for the 3x3 and 5x5
// windows: the window's keys are sorted in registers by a branch-free
// sorting network (enb_sortnet.cuh), so every lane of a warp runs the same
// instructions whatever the data; runs of equal keys are the histogram bins,
// visited in ascending key order as the reference's std::map visits them.
// Transparent taps carry the maximum key and sort behind the n opaque ones.
#pragma once

#include <stdint.h>

#include "enb_device.cuh"
#include "enb_internal.h"
#include "enb_sortnet.cuh"

namespace enb {

constexpr uint32_t kEntropyPad = 0xffffffffu;

template <int M>
__device__ __forceinline__ void sortnet(uint32_t (&k)[M]);
template <>
__device__ __forceinline__ void sortnet<9>(uint32_t (&k)[9]) { sortnet9(k); }
template <>
__device__ __forceinline__ void sortnet<25>(uint32_t (&k)[25]) { sortnet25(k); }

// Keys of the W x W window centred at smem index ci of a TW-wide tile
// (transparent taps -> kEntropyPad); returns the number of opaque taps.
template <int W, typename TK, typename KeyFn>
__device__ __forceinline__ int window_keys(const TK* v, const uint8_t* a, int TW, int ci, uint32_t (&k)[W * W],
                                           KeyFn key)
{
    int n = 0;
#pragma unroll
    for (int dy = 0; dy < W; ++dy) {
#pragma unroll
        for (int dx = 0; dx < W; ++dx) {
            const int idx = ci + (dy - W / 2) * TW + (dx - W / 2);
            const bool on = a[idx] != 0;
            k[dy * W + dx] = on ? key(v[idx]) : kEntropyPad;
            n += on ? 1 : 0;
        }
    }
    return n;
}

// Sum of the 2^-56 fixed-point p log p terms (p = c / n) over the bins of the
// sorted keys k[0..n-1], and the number of bins.
template <int M>
__device__ __forceinline__ void entropy_bins(const uint32_t (&k)[M], int n, const long long* fx, long long& acc,
                                             int& bins)
{
    acc = 0;
    bins = 0;
    int run = 1;
#pragma unroll
    for (int i = 1; i < M; ++i) {
        if (i < n) {
            if (k[i] != k[i - 1]) {
                acc += fx[run];
                ++bins;
                run = 1;
            } else {
                ++run;
            }
        }
    }
    if (n > 0) {
        acc += fx[run];
        ++bins;
    }
}

// The reference's double sum of p log p in ascending key order (the exact
// fallback of the integer path).
template <int M>
__device__ __forceinline__ double entropy_sum_double(const uint32_t (&k)[M], int n, const double* pl)
{
    double es = 0.0;
    int run = 1;
#pragma unroll
    for (int i = 1; i < M; ++i) {
        if (i < n) {
            if (k[i] != k[i - 1]) {
                es = __dadd_rn(es, pl[run]);
                run = 1;
            } else {
                ++run;
            }
        }
    }
    return n > 0 ? __dadd_rn(es, pl[run]) : es;
}

// Integer images: fromRealPromote(H * max) of the window (Histogram::entropyFun).
// A float estimate from the exact fixed-point sum decides the rounding
// unless it lies within 0.03 of a boundary; then the reference's double
// expression is evaluated.
template <int W>
__device__ __forceinline__ uint32_t entropy_window_int(const uint16_t* raw, const uint8_t* a, int TW, int ci, const WeightTables& tab,
                                       uint32_t maxv)
{
    constexpr int M = W * W;
    uint32_t k[M];
    const int n = window_keys<W>(raw, a, TW, ci, k, [](uint16_t x) { return (uint32_t)x; });
    if (n == 0) {
        return 0;
    }
    sortnet<M>(k);
    long long acc;
    int bins;
    entropy_bins<M>(k, n, tab.plogp_fx + (int64_t)n * (M + 1), acc, bins);
    if (bins <= 1) {
        return 0;
    }
    const float e = -(float)acc * 1.3877787807814457e-17f;  // 2^-56
    const float val = __fmul_rn(e, tab.scale_logb[bins]);
    const float x = val + 0.5f;
    const float fl = floorf(x);
    const float d = x - fl;
    if (d > 0.03f && d < 0.97f) {
        return min((uint32_t)max(fl, 0.0f), maxv);
    }
    const double es = entropy_sum_double<M>(k, n, tab.plogp + (int64_t)n * (M + 1));
    const double H = __ddiv_rn(-es, tab.logb[bins]);
    return frp_unsigned(__dmul_rn(H, (double)maxv), maxv);
}

// Float images: H of the window in float (keys: the sample's bit pattern with
// -0 folded into +0, so that equal floats share a bin); tables built with
// max 1 (scale_logb[b] = 1 / log b).  H <= 1.
template <int W>
__device__ __forceinline__ float entropy_window_float(const float* raw, const uint8_t* a, int TW, int ci, const WeightTables& tab)
{
    constexpr int M = W * W;
    uint32_t k[M];
    const int n = window_keys<W>(raw, a, TW, ci, k, [](float f) { return __float_as_uint(f == 0.0f ? 0.0f : f); });
    if (n == 0) {
        return 0.0f;
    }
    sortnet<M>(k);
    long long acc;
    int bins;
    entropy_bins<M>(k, n, tab.plogp_fx + (int64_t)n * (M + 1), acc, bins);
    if (bins <= 1) {
        return 0.0f;
    }
    const float H = __fmul_rn(-(float)acc * 1.3877787807814457e-17f, tab.scale_logb[bins]);
    return fminf(H, 1.0f);
}

}  // namespace enb

namespace enb {

// ---- repeated-sample marks of a float tile ----------------------------------
//
// Float samples rarely repeat except at the clip values 0 and 1.  The
// samples equal to 0.0 or 1.0 are counted per window (two bins whose sizes
// are those counts); all other opaque samples go through the repeat marks
// below, and a window without marks has only singletons besides the two
// clip bins, so its H follows from three counts.  Every opaque sample of the
// tile (halo included) goes into a shared-memory hash table per channel; a
// second insertion of an equal key marks the slot.  meta[p] then carries bit
// c when sample c of pixel p occurs more than once in the tile, and bit 7
// when p is opaque.  A window with no mark in channel c has all-distinct
// keys in that channel (marks from matches elsewhere in the tile only send a
// window down the exact sorting path, they never change a result).

__device__ __forceinline__ uint32_t dup_hash(uint32_t k, int shift) { return (k * 0x9E3779B1u) >> shift; }

// All threads of the block call this.  table: C * slots words, flags: C *
// slots bytes, slots a power of two >= 2 * npx.
template <typename KeyOf>
__device__ __forceinline__ void mark_repeats(const float* raw, int plane, const uint8_t* a, int npx, int C, uint32_t* table,
                             uint8_t* flags, int slots, uint8_t* meta, KeyOf key)
{
    const int shift = 32 - (31 - __clz(slots));
    for (int i = threadIdx.x; i < C * slots; i += blockDim.x) {
        table[i] = kEntropyPad;
        flags[i] = 0;
    }
    __syncthreads();
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
        if (!a[p]) {
            continue;
        }
        for (int c = 0; c < C; ++c) {
            const float fv = raw[c * plane + p];
            if (fv == 0.0f || fv == 1.0f) {
                continue;  // clip values are counted per window, not hashed
            }
            const uint32_t k = key(fv);
            uint32_t* t = table + c * slots;
            uint32_t h = dup_hash(k, shift);
            for (int probe = 0; probe < slots; ++probe) {
                const uint32_t old = atomicCAS(&t[h], kEntropyPad, k);
                if (old == kEntropyPad) {
                    break;
                }
                if (old == k) {
                    flags[c * slots + h] = 1;
                    break;
                }
                h = (h + 1) & (uint32_t)(slots - 1);
            }
        }
    }
    __syncthreads();
    for (int p = threadIdx.x; p < npx; p += blockDim.x) {
        uint8_t m = 0;
        if (a[p]) {
            m = 0x80;
            for (int c = 0; c < C; ++c) {
                const float fv = raw[c * plane + p];
                if (fv == 0.0f || fv == 1.0f) {
                    continue;
                }
                const uint32_t k = key(fv);
                const uint32_t* t = table + c * slots;
                uint32_t h = dup_hash(k, shift);
                for (int probe = 0; probe < slots && t[h] != k; ++probe) {
                    h = (h + 1) & (uint32_t)(slots - 1);
                }
                m |= flags[c * slots + h] ? (uint8_t)(1u << c) : (uint8_t)0;
            }
        }
        meta[p] = m;
    }
    __syncthreads();
}

// Opaque-tap count and OR of the repeat marks of the W x W window at ci.
template <int W>
__device__ __forceinline__ void window_marks(const uint8_t* meta, int TW, int ci, int& n, uint32_t& marks)
{
    n = 0;
    marks = 0;
#pragma unroll
    for (int dy = 0; dy < W; ++dy) {
#pragma unroll
        for (int dx = 0; dx < W; ++dx) {
            const uint32_t m = meta[ci + (dy - W / 2) * TW + (dx - W / 2)];
            n += (int)(m >> 7);
            marks |= m;
        }
    }
}

// Per-pixel clip counters of a float tile: 5-bit fields, samples equal to 1.0
// for channels 0..2 at bits 0, 5, 10 and equal to 0.0 at bits 15, 20, 25
// (opaque pixels only); a window's sum keeps every field below 32.
__device__ __forceinline__ uint32_t clip_counts(const float* rgb, int C)
{
    uint32_t m = 0;
    for (int c = 0; c < C; ++c) {
        m |= (rgb[c] == 1.0f ? 1u : 0u) << (5 * c);
        m |= (rgb[c] == 0.0f ? 1u : 0u) << (15 + 5 * c);
    }
    return m;
}

// Opaque-tap count, OR of the repeat marks and sum of the clip counters of
// the W x W window at ci.
template <int W>
__device__ __forceinline__ void window_counts(const uint8_t* meta, const uint32_t* cnt, int TW, int ci, int& n,
                                              uint32_t& marks, uint32_t& clips)
{
    n = 0;
    marks = 0;
    clips = 0;
#pragma unroll
    for (int dy = 0; dy < W; ++dy) {
#pragma unroll
        for (int dx = 0; dx < W; ++dx) {
            const int idx = ci + (dy - W / 2) * TW + (dx - W / 2);
            const uint32_t m = meta[idx];
            n += (int)(m >> 7);
            marks |= m;
            clips += cnt[idx];
        }
    }
}

// H of a window channel without repeat marks: n - m1 - m0 singletons and the
// bins of the m1 samples equal to 1.0 and the m0 equal to 0.0 (the value the
// sorting path computes for such a window).
__device__ __forceinline__ float entropy_clip_bins(int n, int m1, int m0, const WeightTables& tab, int nmax)
{
    const int bins = n - m1 - m0 + (m1 > 0 ? 1 : 0) + (m0 > 0 ? 1 : 0);
    if (n == 0 || bins <= 1) {
        return 0.0f;
    }
    const long long* fx = tab.plogp_fx + (int64_t)n * (nmax + 1);
    const long long acc = (long long)(n - m1 - m0) * fx[1] + (m1 > 0 ? fx[m1] : 0) + (m0 > 0 ? fx[m0] : 0);
    return fminf(__fmul_rn(-(float)acc * 1.3877787807814457e-17f, tab.scale_logb[bins]), 1.0f);
}

// H of n all-distinct keys, the value entropy_window_float computes for them.
__device__ __forceinline__ float entropy_distinct(int n, const WeightTables& tab, int nmax)
{
    if (n <= 1) {
        return 0.0f;
    }
    const long long acc = (long long)n * tab.plogp_fx[(int64_t)n * (nmax + 1) + 1];
    const float H = __fmul_rn(-(float)acc * 1.3877787807814457e-17f, tab.scale_logb[n]);
    return fminf(H, 1.0f);
}

}  // namespace enb

namespace enb {

// H of a float window channel whose marked taps (bit `bit` of meta) all carry
// one key: n - m singletons and one bin of m.  Returns false when the marked
// taps hold more than one key (the caller then sorts the window).
template <int W, typename KeyOf>
__device__ __forceinline__ bool entropy_one_repeat(const float* raw, const uint8_t* meta, int TW, int ci,
                                                   uint32_t bit, int n, const WeightTables& tab, int nmax,
                                                   KeyOf key, float& H)
{
    uint32_t first = kEntropyPad;
    int m = 0;
    bool single = true;
#pragma unroll
    for (int dy = 0; dy < W; ++dy) {
#pragma unroll
        for (int dx = 0; dx < W; ++dx) {
            const int idx = ci + (dy - W / 2) * TW + (dx - W / 2);
            const uint32_t mk = meta[idx];
            if ((mk & 0x80u) && (mk & bit)) {
                const uint32_t k = key(raw[idx]);
                single = single && (m == 0 || k == first);
                first = m == 0 ? k : first;
                ++m;
            }
        }
    }
    if (!single) {
        return false;
    }
    const int bins = n - m + 1;
    if (bins <= 1) {
        H = 0.0f;
        return true;
    }
    const long long* fx = tab.plogp_fx + (int64_t)n * (nmax + 1);
    const long long acc = (long long)(n - m) * fx[1] + fx[m];
    H = fminf(__fmul_rn(-(float)acc * 1.3877787807814457e-17f, tab.scale_logb[bins]), 1.0f);
    return true;
}

}  // namespace enb
