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

template <class CE = CeU32>
__device__ __forceinline__ void sortnet(uint32_t (&k)[9], CE ce = CE()) { sortnet9(k, ce); }
template <class CE = CeU32>
__device__ __forceinline__ void sortnet(uint32_t (&k)[25], CE ce = CE()) { sortnet25(k, ce); }

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

// fromRealPromote(H * max) with H = -sum p log p / log(bins) from the 2^-56
// fixed-point sum acc (each term rounded once, so |acc 2^-56 - sum| <=
// bins 2^-57): the 128-bit product of -acc and max / log(bins) in 2^-40
// fixed point is H * max in 2^-96 fixed point, whose top 32 fraction bits
// decide the rounding to within 1e-10.  The reference sums the n <= 225
// terms in double (error below n 2^-53 log n, times max / log 2 at most
// n 2^-33 after scaling); where H * max lies within (n + 8) 2^-32 of a
// half-integer, `near` is set and the caller evaluates the reference's
// double expression.
__device__ __forceinline__ uint32_t entropy_fx_round(long long acc, int bins, int n, const WeightTables& tab,
                                                     uint32_t maxv, bool& near)
{
    const unsigned long long A = (unsigned long long)(-acc);  // p log p <= 0
    const unsigned long long hi = __umul64hi(A, tab.scale_fx[bins]);
    const uint32_t frac = (uint32_t)hi;
    const uint32_t dist = frac >= 0x80000000u ? frac - 0x80000000u : 0x80000000u - frac;
    near = dist <= (uint32_t)(n + 8);
    const uint32_t m = (uint32_t)(hi >> 32) + (frac >= 0x80000000u ? 1u : 0u);
    return min(m, maxv);
}

// Integer images: fromRealPromote(H * max) of the window (Histogram::entropyFun),
// rounded by entropy_fx_round, with the reference's double expression near
// a rounding boundary.
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
    sortnet(k);
    long long acc;
    int bins;
    entropy_bins<M>(k, n, tab.plogp_fx + (int64_t)n * (M + 1), acc, bins);
    if (bins <= 1) {
        return 0;
    }
    bool near;
    const uint32_t r = entropy_fx_round(acc, bins, n, tab, maxv, near);
    if (!near) {
        return r;
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
    sortnet(k);
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
// second insertion of an equal key flags the slot.  A sample whose slot is
// flagged occurs more than once in the tile and gets a repeat mark.  A
// window with no mark in channel c has all-distinct keys in that channel
// (marks from matches elsewhere in the tile only send a window down the
// exact sorting path, they never change a result).
//
// Per-pixel counters (one 64-bit word per tile pixel, summed over a window):
//   bits  0..14  samples equal to 1.0, channels 0..2 (5 bits each)
//   bits 15..29  samples equal to 0.0
//   bits 32..46  repeat marks
//   bits 47..51  opaque pixels
// A 5x5 window's sum keeps every field below 32, and no field crosses bit
// 32, so the two 32-bit halves of a sum can be added separately.
constexpr int kCntMark = 32, kCntOpaque = 47;

// Histogram key of a float sample: its bit pattern, -0 folded into +0.
__device__ __forceinline__ uint32_t float_key(float f) { return __float_as_uint(f == 0.0f ? 0.0f : f); }

// Clip-value counters of one opaque pixel (bits 0..29 of its word).
__device__ __forceinline__ uint32_t clip_counts(const float (&rgb)[3], int C)
{
    uint32_t m = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (c < C) {
            m |= (rgb[c] == 1.0f ? 1u : 0u) << (5 * c);
            m |= (rgb[c] == 0.0f ? 1u : 0u) << (15 + 5 * c);
        }
    }
    return m;
}

__device__ __forceinline__ uint32_t dup_hash(uint32_t k, int shift) { return (k * 0x9E3779B1u) >> shift; }

// Empties the C hash tables (C * slots key words, C * slots flag bytes;
// slots a multiple of 64, table and flags 16-byte aligned).
__device__ __forceinline__ void repeat_tables_clear(uint32_t* table, uint8_t* flags, int C, int slots)
{
    uint4* t4 = reinterpret_cast<uint4*>(table);
    const uint4 pad = make_uint4(kEntropyPad, kEntropyPad, kEntropyPad, kEntropyPad);
    for (int i = threadIdx.x; i < C * slots / 4; i += blockDim.x) {
        t4[i] = pad;
    }
    uint4* f4 = reinterpret_cast<uint4*>(flags);
    for (int i = threadIdx.x; i < C * slots / 16; i += blockDim.x) {
        f4[i] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// Marks of a complete tile (all threads call after the barrier that
// completes the tile; the tables were emptied before that barrier by
// repeat_tables_clear; ends with a barrier).  Pixel p is handled by thread
// p % blockDim.x.  NP > 0 (npx <= NP * blockDim.x):
// the keys of a thread probe in lock step, one CAS per pending key a round,
// so its NP * C insertions are in flight together, and the slot where each
// key ended up is kept, so that its flag is read without probing again;
// NP == 0: one key after the other, and a second probe per key to find its
// slot's flag.  slots: a power of two >= 2 * npx, so every probe sequence
// meets an empty slot.
template <int NP>
__device__ __forceinline__ void mark_repeats(const float* raw, int plane, const uint8_t* a, int npx, int C,
                                             uint32_t* table, uint8_t* flags, int slots, uint64_t* cnt)
{
    const int shift = 32 - (31 - __clz(slots));
    if constexpr (NP > 0) {
        constexpr int N = NP;
        uint32_t kk[N][3], h[N][3];
        uint32_t pend = 0;  // bit j * 3 + c: key (j, c) still probing
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const int p = (int)threadIdx.x + j * (int)blockDim.x;
            const bool on = p < npx && a[p] != 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float fv = on && c < C ? raw[c * plane + p] : 0.0f;
                kk[j][c] = float_key(fv);
                h[j][c] = (uint32_t)c * (uint32_t)slots + dup_hash(kk[j][c], shift);
                // clip values are counted per window, not hashed
                pend |= (on && c < C && fv != 0.0f && fv != 1.0f) ? 1u << (j * 3 + c) : 0u;
            }
        }
        const uint32_t hashed = pend;
        for (int round = 0; pend && round < slots; ++round) {
#pragma unroll
            for (int j = 0; j < N; ++j) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const uint32_t bit = 1u << (j * 3 + c);
                    if (pend & bit) {
                        const uint32_t old = atomicCAS(&table[h[j][c]], kEntropyPad, kk[j][c]);
                        if (old == kEntropyPad || old == kk[j][c]) {
                            if (old != kEntropyPad) {
                                flags[h[j][c]] = 1;
                            }
                            pend &= ~bit;
                        } else {
                            const uint32_t base = (uint32_t)c * (uint32_t)slots;
                            h[j][c] = base + ((h[j][c] - base + 1u) & (uint32_t)(slots - 1));
                        }
                    }
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < N; ++j) {
            const int p = (int)threadIdx.x + j * (int)blockDim.x;
            uint64_t m = 0;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if ((hashed >> (j * 3 + c)) & 1u) {
                    m |= flags[h[j][c]] ? 1ull << (kCntMark + 5 * c) : 0ull;
                }
            }
            if (m) {
                cnt[p] |= m;
            }
        }
        __syncthreads();
    } else {
        for (int p = threadIdx.x; p < npx; p += blockDim.x) {
            if (!a[p]) {
                continue;
            }
            for (int c = 0; c < C; ++c) {
                const float fv = raw[c * plane + p];
                if (fv == 0.0f || fv == 1.0f) {
                    continue;
                }
                const uint32_t k = float_key(fv);
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
            if (!a[p]) {
                continue;
            }
            uint64_t m = 0;
            for (int c = 0; c < C; ++c) {
                const float fv = raw[c * plane + p];
                if (fv == 0.0f || fv == 1.0f) {
                    continue;
                }
                const uint32_t k = float_key(fv);
                const uint32_t* t = table + c * slots;
                uint32_t h = dup_hash(k, shift);
                for (int probe = 0; probe < slots && t[h] != k; ++probe) {
                    h = (h + 1) & (uint32_t)(slots - 1);
                }
                m |= flags[c * slots + h] ? 1ull << (kCntMark + 5 * c) : 0ull;
            }
            if (m) {
                cnt[p] |= m;
            }
        }
        __syncthreads();
    }
}

// Opaque-tap count, repeat marks (bit c: some tap of channel c is marked)
// and clip counters (bits 0..29) of the W x W window at ci.
template <int W>
__device__ __forceinline__ void window_counts(const uint64_t* cnt, int TW, int ci, int& n, uint32_t& marks,
                                              uint32_t& clips)
{
    uint64_t sum = 0;
#pragma unroll
    for (int dy = 0; dy < W; ++dy) {
#pragma unroll
        for (int dx = 0; dx < W; ++dx) {
            sum += cnt[ci + (dy - W / 2) * TW + (dx - W / 2)];
        }
    }
    n = (int)((sum >> kCntOpaque) & 31u);
    clips = (uint32_t)sum & 0x3fffffffu;
    marks = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        marks |= ((sum >> (kCntMark + 5 * c)) & 31u) ? 1u << c : 0u;
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

}  // namespace enb
