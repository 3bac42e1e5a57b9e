// enb_fpair.cuh -- enfuse weights of float images, two horizontally adjacent
// output pixels per thread (src/enfuse.h:962-1212 with float pixels): a CTA
// of 256 threads weights 32x16 output pixels from a shared-memory tile of
// their windows.  The two windows of a pair share all but one column, so
// every window statistic is formed from per-column sums computed once:
//
// * local contrast (localStdDevIf, src/enfuse.h:75-219): the window's sample
//   deviation sqrt((S2 - S1^2 / n) / (n - 1)) from the sums S1, S2 of
//   d = g - c and d^2, where the shift c is the gray value of an opaque pixel
//   of the pair (inside both windows).  Shifting by a sample of the window
//   bounds the cancellation in S2 - S1^2 / n to a factor n, so the result
//   stays within a few 1e-7 of the window's exact deviation (the reference's
//   running float sums of g and g^2 cancel without that bound);
// * local entropy (Histogram::entropyOfChannel, src/enfuse.h:346-375): the
//   window counters of enb_entropy.cuh (opaque taps, taps equal to 1.0 or
//   0.0, repeat marks) summed per column; a channel without repeat marks has
//   only singletons besides the two clip bins, and its H is read from a
//   table indexed by (n, m1, m0) built by the same function that evaluates
//   such a window (entropy_clip_bins); a marked channel counts its bins
//   exactly from its marked taps (fpair_entropy_marked).
//
// Each statistic is summed in one fixed order (columns top to bottom, then
// the window's columns left to right), whichever tile, kernel or thread
// evaluates a window, so the per-image weight kernel (enb_float.cu) and the
// batched stack fuse (enb_batch.cu) give bit-identical weights.
#pragma once

#include <stdint.h>

#include "enb_fweights.cuh"

namespace enb {

constexpr int FPX = 32, FPY = 16;  // output pixels of a pair tile
constexpr int FPT = 256;           // threads of a pair CTA: FPX / 2 x FPY

// Halo of windows of sizes CW and EW (0: that weight is off) and the tile's
// left margin: the halo rounded up to even, so that the left pixel of every
// pair sits at an even tile column (aligned vector loads of a pair's columns).
__host__ __device__ constexpr int fpair_halo(int CW, int EW) { return (CW > EW ? CW : EW) / 2; }
__host__ __device__ constexpr int fpair_halo_x(int halo) { return (halo + 1) & ~1; }
__host__ __device__ constexpr int fpair_tw(int CW, int EW) { return FPX + 2 * fpair_halo_x(fpair_halo(CW, EW)); }
__host__ __device__ constexpr int fpair_th(int CW, int EW) { return FPY + 2 * fpair_halo(CW, EW); }

// Tile of TW x TH input pixels (TW and TH even, so TT is a multiple of 4
// and every array below starts on a 16-byte boundary).
struct FTileP {
    uint64_t* cnt;    // [TT] window counters (enb_entropy.cuh)
    float* gray;      // [TT]
    float* raw;       // [3][TT]
    float* eraw;      // [3][TT]: the entropy cutoff's clamped samples, else raw
    uint32_t* table;     // [3][slots] repeat hash
    uint64_t* markrow;   // [3][FPMAXROWS] of the exposure being weighted: bit x of row y: pixel (x, y)
                         // has a repeat mark in that channel (two such buffers, by exposure parity)
    uint8_t* a;          // [TT] opaque flags
    int TW, TT, slots;
};

// Rows of a tile of at most FPY + 2 * 3 rows (windows up to 7).
constexpr int FPMAXROWS = FPY + 6;

__host__ __device__ inline size_t fpair_tile_bytes(int TT, int slots, int ent_cut)
{
    return (size_t)TT * (8 + 4 + 12 + (ent_cut ? 12 : 0)) + (size_t)slots * 12 + (size_t)2 * 3 * FPMAXROWS * 8 +
           align16_sz((size_t)TT);
}

// Hash slots per channel of a tile of TT pixels: a power of two >= 2 TT
// (0: no entropy windows of 3 or 5).
inline int fpair_slots(const FloatWeightParams& wp, int TT)
{
    if (!wp.use_entropy || (wp.entropy_window != 3 && wp.entropy_window != 5)) {
        return 0;
    }
    int slots = 64;
    while (slots < 2 * TT) {
        slots <<= 1;
    }
    return slots;
}

// Whether the pair kernels weight with these parameters: contrast windows of
// 3 or 5, entropy windows of 3 or 5 (either weight may be off).
__host__ __device__ inline bool fpair_path(const FloatWeightParams& wp)
{
    return (!wp.use_contrast || wp.contrast_window == 3 || wp.contrast_window == 5) &&
           (!wp.use_entropy || wp.entropy_window == 3 || wp.entropy_window == 5);
}

__device__ __forceinline__ FTileP fpair_carve(unsigned char* smem, int TW, int TT, int slots, int ent_cut)
{
    FTileP t;
    t.TW = TW;
    t.TT = TT;
    t.slots = slots;
    t.cnt = reinterpret_cast<uint64_t*>(smem);
    t.gray = reinterpret_cast<float*>(t.cnt + TT);
    t.raw = t.gray + TT;
    t.eraw = ent_cut ? t.raw + 3 * TT : t.raw;
    t.table = reinterpret_cast<uint32_t*>(t.raw + (ent_cut ? 6 : 3) * TT);
    t.markrow = reinterpret_cast<uint64_t*>(t.table + 3 * slots);
    t.a = reinterpret_cast<uint8_t*>(t.markrow + 2 * 3 * FPMAXROWS);
    return t;
}

// Tile t with the row-mask buffer of exposure k.
__device__ __forceinline__ FTileP fpair_for_exposure(FTileP t, int k)
{
    t.markrow += (k & 1) * 3 * FPMAXROWS;
    return t;
}

// Empties the C hash tables of the repeat marks and the row masks of t
// (t.markrow: the buffer to be filled next).  The tables are used only while
// a tile is loaded; the row masks are read while its windows are weighted,
// so the kernels alternate two row-mask buffers and empty the one that no
// thread reads.
template <int C>
__device__ __forceinline__ void fpair_clear_tables(const FTileP& t)
{
    uint4* t4 = reinterpret_cast<uint4*>(t.table);
    const uint4 pad = make_uint4(kEntropyPad, kEntropyPad, kEntropyPad, kEntropyPad);
    for (int i = threadIdx.x; i < C * t.slots / 4; i += FPT) {
        t4[i] = pad;
    }
    if (threadIdx.x < 3 * FPMAXROWS) {
        t.markrow[threadIdx.x] = 0ull;
    }
}

// Records a repeat mark of channel c at tile pixel p in its counters and in
// the channel's row mask (the owner of p only).
template <int TW>
__device__ __forceinline__ void fpair_mark(const FTileP& t, int p, int c)
{
    t.cnt[p] |= 1ull << (kCntMark + 5 * c);
    const int r = p / TW;
    atomicOr(reinterpret_cast<unsigned long long*>(&t.markrow[c * FPMAXROWS + r]), 1ull << (p - r * TW));
}

// A thread's NP tile pixels (pixel p = threadIdx.x + j * FPT) as fetched
// from an exposure: samples, opaque flags (bit j) and whether the pixel lies
// in the image (bit 8 + j).
template <int NP>
struct FpairFetch {
    float v[NP][3];
    uint32_t fl;
};

// Issues the loads of the thread's pixels of the TW-wide tile of TT pixels
// whose top-left input pixel is (x0, y0) (zeros and transparent outside the
// image); the values are used by fpair_store.
template <int NP, int C, int TW, int TT>
__device__ __forceinline__ void fpair_fetch(FpairFetch<NP>& f, const float* img, int64_t pitch, int stride, int w,
                                            int h, const uint8_t* alpha, int64_t apitch, int x0, int y0)
{
    f.fl = 0;
#pragma unroll
    for (int j = 0; j < NP; ++j) {
        const int p = (int)threadIdx.x + j * FPT;
        const int r = p / TW, c = p - r * TW;
        const int gx = x0 + c, gy = y0 + r;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            f.v[j][ch] = 0.0f;
        }
        if ((j * FPT + FPT <= TT || p < TT) && gx >= 0 && gx < w && gy >= 0 && gy < h) {
            const float* px = img + (int64_t)gy * pitch + (int64_t)gx * stride;
#pragma unroll
            for (int ch = 0; ch < C; ++ch) {
                f.v[j][ch] = __ldg(&px[ch]);
            }
            const bool a = alpha ? __ldg(&alpha[(int64_t)gy * apitch + gx]) != 0 : true;
            f.fl |= (a ? 1u : 0u) << j | 1u << (8 + j);
        }
    }
}

// Writes the thread's fetched pixels into tile t and, with hash slots,
// issues the first probe of each of their repeat-mark keys (old: the
// probed slots' previous contents; kEntropyPad where no key was inserted
// or the slot was empty).  The tables must be empty.  Returns 1 when every
// one of the pixels that lies in the image is opaque.
//
// Repeat marks: every opaque sample that is no clip value goes into its
// channel's hash table (open addressing, linear probing); an insertion
// that meets its own key marks its pixel.  Of every set of equal samples
// all but the first inserted are marked, so a window holding two equal
// samples holds a marked one.  Only the thread that owns a pixel writes
// its counters.  slots: a power of two >= 2 TT, so every probe sequence
// meets an empty slot.
template <int NP, int C, int TT>
__device__ __forceinline__ int fpair_store(const FTileP& t, const FloatWeightParams& wp, const FpairFetch<NP>& f,
                                           uint32_t (&old)[NP][3])
{
    const int slots = t.slots;
    const int shift = slots ? 32 - (31 - __clz(slots)) : 0;
    int mine = 1;
#pragma unroll
    for (int j = 0; j < NP; ++j) {
        const int p = (int)threadIdx.x + j * FPT;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            old[j][c] = kEntropyPad;
        }
        if (j * FPT + FPT <= TT || p < TT) {
            const bool a = (f.fl >> j) & 1u;
            float rgb[3] = {f.v[j][0], f.v[j][1], f.v[j][2]};
            t.gray[p] = C == 1 ? rgb[0] : gray_of_f(wp, rgb[0], rgb[1], rgb[2]);
            t.a[p] = a ? 1 : 0;
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
                t.raw[ch * TT + p] = rgb[ch];
            }
            if (wp.use_entropy) {
                if (wp.ent_cut) {
                    entropy_clamp_f(wp, rgb, C);
#pragma unroll
                    for (int ch = 0; ch < 3; ++ch) {
                        t.eraw[ch * TT + p] = rgb[ch];
                    }
                }
                t.cnt[p] = a ? (uint64_t)clip_counts(rgb, C) | (1ull << kCntOpaque) : 0ull;
                if (slots && a) {
#pragma unroll
                    for (int c = 0; c < C; ++c) {
                        // clip values are counted per window, not hashed
                        if (rgb[c] != 0.0f && rgb[c] != 1.0f) {
                            const uint32_t key = float_key(rgb[c]);
                            old[j][c] = atomicCAS(&t.table[(uint32_t)c * (uint32_t)slots + dup_hash(key, shift)],
                                                  kEntropyPad, key);
                        }
                    }
                }
            }
            mine &= (a || !((f.fl >> (8 + j)) & 1u)) ? 1 : 0;
        }
    }
    return mine;
}

// Completes the repeat marks of the thread's pixels of tile t from the first
// probes' results (fpair_store): a probe that met its own key marks the
// pixel; keys whose slot held another key probe on, one after the other.
template <int NP, int C, int TW, int TT>
__device__ __forceinline__ void fpair_hash_finish(const FTileP& t, const uint32_t (&old)[NP][3])
{
    const int slots = t.slots;
    const int shift = 32 - (31 - __clz(slots));
    uint32_t pend = 0;  // bit j * 3 + c: key (j, c) found its slot taken
#pragma unroll
    for (int j = 0; j < NP; ++j) {
        const int p = (int)threadIdx.x + j * FPT;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            if (old[j][c] != kEntropyPad) {
                if (old[j][c] == float_key(t.eraw[c * TT + p])) {
                    fpair_mark<TW>(t, p, c);
                } else {
                    pend |= 1u << (j * 3 + c);
                }
            }
        }
    }
    while (pend) {
        const int b = __ffs(pend) - 1;
        pend &= pend - 1u;
        const int j = b / 3, c = b - 3 * j;
        const int p = (int)threadIdx.x + j * FPT;
        const uint32_t key = float_key(t.eraw[c * TT + p]);
        uint32_t* tab = t.table + c * slots;
        uint32_t h = dup_hash(key, shift);
        for (int probe = 1; probe < slots; ++probe) {
            h = (h + 1u) & (uint32_t)(slots - 1);
            const uint32_t o = atomicCAS(&tab[h], kEntropyPad, key);
            if (o == kEntropyPad) {
                break;
            }
            if (o == key) {
                fpair_mark<TW>(t, p, c);
                break;
            }
        }
    }
}

// Loads tile t whole (fetch, store, repeat marks) as the first step of a
// kernel; the tables must be empty since the block's previous barrier.
// Ends with a barrier; returns nonzero when every tile pixel inside the
// image is opaque (then every window that is evaluated, which lies inside
// the image, is opaque).
template <int NP, int C, int TW, int TT>
__device__ __forceinline__ int fpair_load(const FTileP& t, const FloatWeightParams& wp, const float* img, int64_t pitch,
                                          int stride, int w, int h, const uint8_t* alpha, int64_t apitch, int x0, int y0)
{
    FpairFetch<NP> f;
    fpair_fetch<NP, C, TW, TT>(f, img, pitch, stride, w, h, alpha, apitch, x0, y0);
    uint32_t old[NP][3];
    const int mine = fpair_store<NP, C, TT>(t, wp, f, old);
    if (t.slots) {
        fpair_hash_finish<NP, C, TW, TT>(t, old);
    }
    return __syncthreads_and(mine);
}

// The W x W window counters of the pair at (cx, cy), cx even: column sums
// of the two 32-bit halves (no field crosses bit 32 and none overflows).
template <int W>
__device__ __forceinline__ void fpair_counts(const uint64_t* cnt, int TW, int cx, int cy, uint2& left, uint2& right)
{
    constexpr int B = W / 2, NC = W + 1;
    uint32_t lo[NC], hi[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        lo[j] = 0u;
        hi[j] = 0u;
    }
#pragma unroll
    for (int dy = 0; dy < W; ++dy) {
        const uint64_t* row = cnt + (cy + dy - B) * TW + cx - B;
        if constexpr ((B & 1) == 0) {
            // cx - B is even: 16-byte aligned pairs of words
#pragma unroll
            for (int j = 0; j < NC / 2; ++j) {
                const uint4 v = reinterpret_cast<const uint4*>(row)[j];
                lo[2 * j] += v.x;
                hi[2 * j] += v.y;
                lo[2 * j + 1] += v.z;
                hi[2 * j + 1] += v.w;
            }
        } else {
#pragma unroll
            for (int j = 0; j < NC; ++j) {
                const uint2 v = reinterpret_cast<const uint2*>(row)[j];
                lo[j] += v.x;
                hi[j] += v.y;
            }
        }
    }
    uint32_t l0 = 0u, l1 = 0u, r0 = 0u, r1 = 0u;
#pragma unroll
    for (int j = 0; j < W; ++j) {
        l0 += lo[j];
        l1 += hi[j];
        r0 += lo[j + 1];
        r1 += hi[j + 1];
    }
    left = make_uint2(l0, l1);
    right = make_uint2(r0, r1);
}

// Columns cx - B .. cx + B + 1 of row `row` (a tile row's first pixel) into
// v[0 .. 2B+1], with 8-byte loads where the column is even.
template <int B>
__device__ __forceinline__ void fpair_row(const float* row, int cx, float (&v)[2 * B + 2])
{
    constexpr int NC = 2 * B + 2;
    if constexpr ((B & 1) == 0) {
#pragma unroll
        for (int j = 0; j < NC / 2; ++j) {
            const float2 p = reinterpret_cast<const float2*>(row + cx - B)[j];
            v[2 * j] = p.x;
            v[2 * j + 1] = p.y;
        }
    } else {
        v[0] = row[cx - B];
#pragma unroll
        for (int j = 0; j < NC / 2 - 1; ++j) {
            const float2 p = reinterpret_cast<const float2*>(row + cx - B + 1)[j];
            v[2 * j + 1] = p.x;
            v[2 * j + 2] = p.y;
        }
        v[NC - 1] = row[cx + B + 1];
    }
}

// Sample deviation from the shifted sums of n taps.
// fpair_sd of a whole window of N taps, with the reciprocals of N and N - 1
// as constants (their correctly rounded floats, as __frcp_rn gives them).
template <int N>
__device__ __forceinline__ float fpair_sd_full(float s1, float s2)
{
    constexpr float rn = (float)(1.0 / N), rn1 = (float)(1.0 / (N - 1));
    const float var = __fmul_rn(__fsub_rn(s2, __fmul_rn(__fmul_rn(s1, s1), rn)), rn1);
    return var > 0.0f ? __fsqrt_rn(var) : 0.0f;
}

__device__ __forceinline__ float fpair_sd(float s1, float s2, int n)
{
    if (n <= 1) {
        return 0.0f;
    }
    const float nf = (float)n;
    const float var = __fmul_rn(__fsub_rn(s2, __fmul_rn(__fmul_rn(s1, s1), __frcp_rn(nf))), __frcp_rn(nf - 1.0f));
    return var > 0.0f ? __fsqrt_rn(var) : 0.0f;
}

// Local contrast of the pair at (cx, cy): sd[q] of the CW x CW window of
// pixel q, from the deviations of the gray values from c.  OPAQUE: every
// tap of both windows is opaque (no per-tap test; the same sums).
template <int CW, bool OPAQUE>
__device__ __forceinline__ void fpair_contrast(const FTileP& t, int cx, int cy, float c, float (&sd)[2])
{
    constexpr int B = CW / 2, NC = CW + 1;
    float s[NC], q[NC];
    int n[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        s[j] = 0.0f;
        q[j] = 0.0f;
        n[j] = 0;
    }
#pragma unroll
    for (int dy = 0; dy < CW; ++dy) {
        const int rbase = (cy + dy - B) * t.TW;
        float v[NC];
        fpair_row<B>(t.gray + rbase, cx, v);
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            float d = __fsub_rn(v[j], c);
            if (!OPAQUE) {
                const bool on = t.a[rbase + cx - B + j] != 0;
                d = on ? d : 0.0f;
                n[j] += on ? 1 : 0;
            }
            s[j] = __fadd_rn(s[j], d);
            q[j] = __fmaf_rn(d, d, q[j]);
        }
    }
    float s0 = s[0], q0 = q[0], s1 = s[1], q1 = q[1];
    int n0 = n[0], n1 = n[1];
#pragma unroll
    for (int j = 1; j < CW; ++j) {
        s0 = __fadd_rn(s0, s[j]);
        q0 = __fadd_rn(q0, q[j]);
        s1 = __fadd_rn(s1, s[j + 1]);
        q1 = __fadd_rn(q1, q[j + 1]);
        n0 += n[j];
        n1 += n[j + 1];
    }
    if (OPAQUE) {
        sd[0] = fpair_sd_full<CW * CW>(s0, q0);
        sd[1] = fpair_sd_full<CW * CW>(s1, q1);
    } else {
        // a window of all CW * CW taps gives the same value as fpair_sd_full
        sd[0] = n0 == CW * CW ? fpair_sd_full<CW * CW>(s0, q0) : fpair_sd(s0, q0, n0);
        sd[1] = n1 == CW * CW ? fpair_sd_full<CW * CW>(s1, q1) : fpair_sd(s1, q1, n1);
    }
}

// fpair_contrast of windows with transparent taps (tiles at the edge of an
// alpha mask), out of line.
template <int CW>
__device__ __noinline__ float2 fpair_contrast_alpha(const float* gray, const uint8_t* a, int TW, int cx, int cy, float c)
{
    FTileP t{};
    t.gray = const_cast<float*>(gray);
    t.a = const_cast<uint8_t*>(a);
    t.TW = TW;
    float sd[2];
    fpair_contrast<CW, false>(t, cx, cy, c, sd);
    return make_float2(sd[0], sd[1]);
}

// The exposure term of a pixel (as f_pixel_weight): W_exp * f(gray), or 0
// where the exposure cutoff rejects the pixel.
// Whether an RGB pixel passes the exposure cutoff (lower projection >= lo,
// upper projection <= hi), out of line.
static __device__ __noinline__ bool exposure_cut_rgb(int p0, int p1, double m0, double m1, double m2, float lo,
                                                     float hi, float r, float g, float b)
{
    return gray_proj_m(p0, m0, m1, m2, r, g, b) >= lo && gray_proj_m(p1, m0, m1, m2, r, g, b) <= hi;
}

__device__ __forceinline__ float f_exposure_term(const FloatWeightParams& wp, float gray, float r, float g, float b,
                                                 int C)
{
    bool pass = true;
    if (wp.exp_cut) {
        pass = C == 3 ? exposure_cut_rgb(wp.cut_proj[0], wp.cut_proj[1], wp.mixer[0], wp.mixer[1], wp.mixer[2],
                                         wp.cut_lo, wp.cut_hi, r, g, b)
                      : gray >= wp.cut_lo && gray <= wp.cut_hi;
    }
    return pass ? __fmul_rn(wp.w_exposure, exposure_f(wp, gray)) : 0.0f;
}

// W_sat * saturation of an RGB pixel (SaturationFunctor with max_value 1.0,
// src/enfuse.h:733-780; 2 - (max + min) formed as (1 - max) + (1 - min)).
__device__ __forceinline__ float f_saturation_term(const FloatWeightParams& wp, float r, float g, float b)
{
    const float mx = fmaxf(r, fmaxf(g, b)), mn = fminf(r, fminf(g, b));
    if (mx == mn) {
        return 0.0f;
    }
    const float sum = __fadd_rn(mx, mn), diff = __fsub_rn(mx, mn);
    const float den = sum <= 1.0f ? sum : __fadd_rn(__fsub_rn(1.0f, mx), __fsub_rn(1.0f, mn));
    return __fmul_rn(wp.w_saturation, __fdiv_rn(diff, den));
}

// H of a window channel with repeat marks (rare), from its bins: every
// repeated key of the window has a marked tap (of equal samples all but the
// first inserted are marked), so the bins are the two clip bins (m1 taps at
// 1.0, m0 at 0.0), one bin per distinct key of the marked taps, sized by
// comparing that key with the window's taps, and singletons for the other
// opaque taps: the same bin sizes, hence the same sum of p log p terms and
// the same H, as sorting the window's keys.  (x0, y0): the window's top-left
// tile pixel; raw, markrow: the channel's samples and row masks.
template <int EW>
__device__ __noinline__ float fpair_entropy_marked(const float* raw, const uint8_t* a, const uint64_t* markrow, int TW,
                                                   int x0, int y0, int n, int m1, int m0, const long long* fx,
                                                   const float* scale_logb)
{
    constexpr int W = EW, M = W * W;
    uint32_t marked = 0;  // bit dy * W + dx
#pragma unroll
    for (int dy = 0; dy < W; ++dy) {
        marked |= ((uint32_t)(markrow[y0 + dy] >> x0) & ((1u << W) - 1u)) << (dy * W);
    }
    uint32_t done = 0;
    long long acc = 0;
    int bins = 0, rep = 0;
    while (marked) {
        const int i = __ffs(marked) - 1;
        marked &= marked - 1u;
        if ((done >> i) & 1u) {
            continue;  // in the bin of an earlier marked tap
        }
        const int iy = i / W;
        // a marked key is never that of 0.0 or -0.0, so the samples' bit
        // patterns compare as their keys; with n = W * W every tap is opaque
        const uint32_t k = __float_as_uint(raw[(y0 + iy) * TW + x0 + i - iy * W]);
        const uint32_t* bits = reinterpret_cast<const uint32_t*>(raw);
        uint32_t same = 0;
        if (n == M) {
#pragma unroll
            for (int j = 0; j < M; ++j) {
                same |= bits[(y0 + j / W) * TW + x0 + j % W] == k ? 1u << j : 0u;
            }
        } else {
#pragma unroll
            for (int j = 0; j < M; ++j) {
                const int idx = (y0 + j / W) * TW + x0 + j % W;
                same |= (a[idx] && bits[idx] == k) ? 1u << j : 0u;
            }
        }
        done |= same;
        const int c = __popc(same);
        acc += fx[c];
        ++bins;
        rep += c;
    }
    const int single = n - m1 - m0 - rep;
    acc += (long long)single * fx[1] + (m1 > 0 ? fx[m1] : 0) + (m0 > 0 ? fx[m0] : 0);
    bins += single + (m1 > 0 ? 1 : 0) + (m0 > 0 ? 1 : 0);
    if (n == 0 || bins <= 1) {
        return 0.0f;
    }
    return fminf(__fmul_rn(-(float)acc * 1.3877787807814457e-17f, scale_logb[bins]), 1.0f);
}

// min over the channels of H * range for the entropy window of tile pixel ci
// with the window's counter sums cs (low and high halves).
template <int EW, int C>
__device__ __forceinline__ float fpair_entropy(const FTileP& t, const FloatWeightParams& wp, const WeightTables& tab,
                                               int ci, uint2 cs)
{
    constexpr int M = EW * EW;
    const int n = (int)((cs.y >> (kCntOpaque - 32)) & 31u);
    float emin = 3.402823466e38f;
#pragma unroll
    for (int ch = 0; ch < C; ++ch) {
        float H;
        const int m1 = (int)((cs.x >> (5 * ch)) & 31u), m0 = (int)((cs.x >> (15 + 5 * ch)) & 31u);
        if ((cs.y >> (kCntMark - 32 + 5 * ch)) & 31u) {
            const int cy = ci / t.TW, cx = ci - cy * t.TW;
            H = fpair_entropy_marked<EW>(t.eraw + ch * t.TT, t.a, t.markrow + ch * FPMAXROWS, t.TW, cx - EW / 2,
                                         cy - EW / 2, n, m1, m0, tab.plogp_fx + (int64_t)n * (M + 1), tab.scale_logb);
        } else {
            H = __ldg(&tab.clip_h[(n * (M + 1) + m1) * (M + 1) + m0]);
        }
        emin = fminf(emin, __fmul_rn(H, wp.range));
    }
    return emin;
}

// The enfuseMask weights (w0, w1) of the output pixels (x, y), (x + 1, y) at
// tile position (cx, cy): exposure, + contrast, + saturation, + entropy, in
// the reference's order of the float adds (src/enfuse.h:1119-1120,
// 1133-1134, 1208-1209); 0 for pixels that are transparent or outside the
// image.  opaque: as fpair_load returned.
template <int CW, int EW, int C>
__device__ __forceinline__ void fpair_weights(const FTileP& t, const FloatWeightParams& wp, const WeightTables& tab,
                                              int cx, int cy, int x, int y, int w, int h, bool opaque, float& w0,
                                              float& w1)
{
    const int TT = t.TT, ci = cy * t.TW + cx;
    const bool a[2] = {t.a[ci] != 0, t.a[ci + 1] != 0};
    float res[2] = {0.0f, 0.0f};
    if (!a[0] && !a[1]) {
        w0 = w1 = 0.0f;
        return;
    }
    if (wp.use_exposure) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (a[q]) {
                res[q] = f_exposure_term(wp, t.gray[ci + q], t.raw[ci + q], t.raw[TT + ci + q], t.raw[2 * TT + ci + q], C);
            }
        }
    }
    if constexpr (CW > 0) {
        constexpr int B = CW / 2;
        const bool rows = y >= B && y < h - B;
        const bool need0 = a[0] && rows && x >= B && x < w - B;
        const bool need1 = a[1] && rows && x + 1 >= B && x + 1 < w - B;
        float sd[2] = {0.0f, 0.0f};
        if (need0 || need1) {
            const float c = a[0] ? t.gray[ci] : t.gray[ci + 1];
            if (opaque) {
                fpair_contrast<CW, true>(t, cx, cy, c, sd);
            } else {
                const float2 v = fpair_contrast_alpha<CW>(t.gray, t.a, t.TW, cx, cy, c);
                sd[0] = v.x;
                sd[1] = v.y;
            }
        }
        // the border strip is not written (0)
        res[0] = __fmaf_rn(wp.w_contrast, need0 ? sd[0] : 0.0f, res[0]);
        res[1] = __fmaf_rn(wp.w_contrast, need1 ? sd[1] : 0.0f, res[1]);
    }
    if (wp.use_saturation && C == 3) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            if (a[q]) {
                res[q] = __fadd_rn(f_saturation_term(wp, t.raw[ci + q], t.raw[TT + ci + q], t.raw[2 * TT + ci + q]), res[q]);
            }
        }
    }
    if constexpr (EW > 0) {
        constexpr int B = EW / 2;
        const bool rows = y >= B && y < h - B;
        const bool need0 = a[0] && rows && x >= B && x < w - B;
        const bool need1 = a[1] && rows && x + 1 >= B && x + 1 < w - B;
        if (need0 || need1) {
            uint2 cl, cr;
            fpair_counts<EW>(t.cnt, t.TW, cx, cy, cl, cr);
            const float e0 = need0 ? fpair_entropy<EW, C>(t, wp, tab, ci, cl) : 0.0f;
            const float e1 = need1 ? fpair_entropy<EW, C>(t, wp, tab, ci + 1, cr) : 0.0f;
            res[0] = __fadd_rn(__fmul_rn(wp.w_entropy, e0), res[0]);
            res[1] = __fadd_rn(__fmul_rn(wp.w_entropy, e1), res[1]);
        }
    }
    w0 = a[0] ? res[0] : 0.0f;
    w1 = a[1] ? res[1] : 0.0f;
}

// Runs the statement(s) after wp with the compile-time window sizes
// (CWV, EWV) of the pair path for the parameters' windows (0 where a weight
// is off).
#define ENB_FPAIR_DISPATCH(wp, ...)                                                        \
    do {                                                                                   \
        const int cw_ = (wp).use_contrast ? (wp).contrast_window : 0;                      \
        const int ew_ = (wp).use_entropy ? (wp).entropy_window : 0;                        \
        if (cw_ == 5 && ew_ == 5) { constexpr int CWV = 5, EWV = 5; __VA_ARGS__; }         \
        else if (cw_ == 5 && ew_ == 3) { constexpr int CWV = 5, EWV = 3; __VA_ARGS__; }    \
        else if (cw_ == 3 && ew_ == 3) { constexpr int CWV = 3, EWV = 3; __VA_ARGS__; }    \
        else if (cw_ == 3 && ew_ == 5) { constexpr int CWV = 3, EWV = 5; __VA_ARGS__; }    \
        else if (cw_ == 0 && ew_ == 5) { constexpr int CWV = 0, EWV = 5; __VA_ARGS__; }    \
        else if (cw_ == 0 && ew_ == 3) { constexpr int CWV = 0, EWV = 3; __VA_ARGS__; }    \
        else if (cw_ == 5 && ew_ == 0) { constexpr int CWV = 5, EWV = 0; __VA_ARGS__; }    \
        else if (cw_ == 3 && ew_ == 0) { constexpr int CWV = 3, EWV = 0; __VA_ARGS__; }    \
        else { constexpr int CWV = 0, EWV = 0; __VA_ARGS__; }                              \
    } while (0)

}  // namespace enb
