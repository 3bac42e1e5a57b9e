// enb_efuse.cu -- fused level passes of enfuse for 8/16-bit images.
//
// The reference (src/enfuse.h:1281-1617) computes each exposure's weight
// map, sums them, then per exposure builds the full Laplacian pyramid of the
// image and the Gaussian pyramid of its normalised mask, multiplies them
// level by level and adds the product into the result pyramid, and finally
// collapses it: the result pyramid is read and written once per exposure and
// every level of every pyramid is materialised.  Here
//   * one pass computes the weights of all K exposures per 16x16 tile, their
//     sum, the normalised (or hard) masks as level 0 of the mask pyramids and
//     the union alpha;
//   * level 0 of no image pyramid is stored: the level-1 reduce reads the
//     interleaved pixels and converts them to fixed point on the fly; each
//     reduce launch covers the K exposures (blockIdx.z);
//   * each level l >= 1 is one pass: R_l = fromPromote(sum_k
//     fromRealPromote((G_k,l - E(G_k,l+1)) * M_k,l / D) + E(R_l+1)), the sum
//     wrapping in the pyramid type as the reference's accumulation does (the
//     order of the exposures does not change a modular sum);
//   * level 0 is one pass from the K images and level-0 masks and the
//     level-1 pyramids straight to the dithered output pixels.
// Every value is the same integer the reference computes: only the order of
// the passes over memory changes.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "enb_device.cuh"
#include "enb_internal.h"
#include "enb_iweights.cuh"
#include "enb_pixels.cuh"
#include "enb_reduce.cuh"
#include "enb_tiles.cuh"

namespace enb {

// ---------------------------------------------------------------------------
// weights of all exposures, normalisation, level-0 masks, union alpha
// ---------------------------------------------------------------------------

template <typename TM>
struct EfWeightsArgs {
    int K, w, h, hard, mfrac;
    PixelView img[kEfuseMaxK];
    AlphaSrc alpha[kEfuseMaxK];
    const float* min[kEfuseMaxK];
    int64_t mipitch[kEfuseMaxK];
    WeightParams wp;
    WeightTables tab;
    TM* m0[kEfuseMaxK];
    int64_t mpitch;
    uint8_t* u0;
    int64_t upitch;
};

// Output tile of the weight pass: 32 x 16 pixels, a pair of horizontally
// adjacent pixels per thread.
constexpr int EWX = 32, EWY = 16;

// Left and top margins of the weight tile: the windows' halo, the left one
// rounded up to even so that pair keys are word loads.
__host__ __device__ inline int ef_halo_x(const WeightParams& wp) { return (iweight_halo(wp) + 1) & ~1; }

template <typename TM>
__global__ void __launch_bounds__(256, 3) k_ef_weights(const __grid_constant__ EfWeightsArgs<TM> a)
{
    extern __shared__ __align__(16) unsigned char esmem[];
    const int halo = iweight_halo(a.wp), hx = ef_halo_x(a.wp);
    const int TW = EWX + 2 * hx, TH = EWY + 2 * halo;
    const ITile t = itile_carve_rect(esmem, TW, TH);
    long long* fx = reinterpret_cast<long long*>(esmem + ((itile_bytes_rect(TW, TH) + 15) & ~(size_t)15));  // [32]
    float2* wk = reinterpret_cast<float2*>(fx + 32) + threadIdx.x;  // [K][256]
    const int px = threadIdx.x % (EWX / 2), py = threadIdx.x / (EWX / 2);
    const int x = blockIdx.x * EWX + 2 * px, y = blockIdx.y * EWY + py;
    const bool in0 = x < a.w && y < a.h, in1 = x + 1 < a.w && y < a.h;
    const int cx = hx + 2 * px, cy = halo + py;
    const int ci = cy * TW + cx;
    const int K = a.K;
    const bool pair_path = iweight_pair_path(a.wp);
    if (a.wp.use_entropy && pair_path && (int)threadIdx.x <= a.wp.entropy_window * a.wp.entropy_window) {
        // the p log p terms of full windows (n = W * W)
        const int M = a.wp.entropy_window * a.wp.entropy_window;
        fx[threadIdx.x] = a.tab.plogp_fx[(int64_t)M * (M + 1) + threadIdx.x];
    }
    uint32_t ua0 = 0, ua1 = 0;
    for (int k = 0; k < K; ++k) {
        if (a.min[k]) {
            // --load-masks: the loaded weight replaces enfuseMask (src/enfuse.h:1288-1331)
            const float* mrow = a.min[k] + (int64_t)y * a.mipitch[k];
            wk[k * 256] = make_float2(in0 ? __ldg(&mrow[x]) : 0.0f, in1 ? __ldg(&mrow[x + 1]) : 0.0f);
            ua0 |= in0 ? (uint32_t)alpha_at(a.alpha[k], x, y) : 0u;
            ua1 |= in1 ? (uint32_t)alpha_at(a.alpha[k], x + 1, y) : 0u;
            continue;
        }
        // ends with a barrier (which also publishes fx)
        const int opaque = itile_load_rect(t, a.wp, a.img[k], a.alpha[k], blockIdx.x * EWX - hx, blockIdx.y * EWY - halo);
        float w0 = 0.0f, w1 = 0.0f;
        if (opaque && pair_path) {
            // every window of the tile is whole and opaque: both pixels at once
            pair_weights(t, a.wp, a.tab, fx, a.img[k].C, cx, cy, w0, w1);
        } else {
            w0 = in0 ? i_pixel_weight(t, a.wp, a.tab, a.img[k], ci, x, y) : 0.0f;
            w1 = in1 ? i_pixel_weight(t, a.wp, a.tab, a.img[k], ci + 1, x + 1, y) : 0.0f;
        }
        wk[k * 256] = make_float2(w0, w1);
        ua0 |= t.a[ci];
        ua1 |= t.a[ci + 1];
        __syncthreads();  // the next exposure's load overwrites the tile
    }
    // normalisation (src/enfuse.h:1382-1385 sum in exposure order, 1399-1442
    // hard mask, 1526-1535 soft mask: float 255 * w / sum, integer 255 / K
    // where every weight is 0), then fromRealPromote(m * 2^F) into the mask
    // pyramid's level 0
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        if (!(q == 0 ? in0 : in1)) {
            continue;
        }
        const float* wq = reinterpret_cast<const float*>(wk) + q;
        const int64_t o = (int64_t)y * a.mpitch + x + q;
        if (a.hard) {
            float mx = 0.0f;
            int mi = 0;
            for (int k = 0; k < K; ++k) {
                if (wq[k * 512] > mx) {
                    mx = wq[k * 512];
                    mi = k;
                }
            }
            const float fallback = __fdiv_rn(255.0f, (float)K);
            for (int k = 0; k < K; ++k) {
                const float m = mx == 0.0f ? fallback : (k == mi ? 255.0f : 0.0f);
                a.m0[k][o] = mask_to_fixed<TM>(m, a.mfrac);
            }
        } else {
            float norm = 0.0f;
            for (int k = 0; k < K; ++k) {
                norm = __fadd_rn(wq[k * 512], norm);
            }
            const float fallback = (float)(255 / K);
            for (int k = 0; k < K; ++k) {
                const float m = norm > 0.0f ? __fdiv_rn(__fmul_rn(255.0f, wq[k * 512]), norm) : fallback;
                a.m0[k][o] = mask_to_fixed<TM>(m, a.mfrac);
            }
        }
        a.u0[(int64_t)y * a.upitch + x + q] = (q == 0 ? ua0 : ua1) ? 255 : 0;
    }
}

// ---------------------------------------------------------------------------
// staging and expansion of coarse windows
// ---------------------------------------------------------------------------

// Stages the (ESH x ESW) window of one coarse plane at (I0 - 1, J0 - 1):
// zero outside the level, x periodic when wrap.  All threads call.
template <typename T>
__device__ __forceinline__ void ef_stage(int32_t (*ss)[ESW], const T* __restrict__ p, int64_t pitch, int cw, int ch,
                                         int I0, int J0, int wrap)
{
    for (int k = threadIdx.x; k < ESH * ESW; k += blockDim.x) {
        const int r = k / ESW, c = k - r * ESW;
        const int j = J0 - 1 + r;
        int i = I0 - 1 + c;
        if (wrap) {
            i = imod(i, cw);
        }
        const bool in = j >= 0 && j < ch && i >= 0 && i < cw;
        const int64_t o = (int64_t)min(max(j, 0), ch - 1) * pitch + min(max(i, 0), cw - 1);
        const int32_t v = (int32_t)__ldg(&p[o]);
        ss[r][c] = in ? v : 0;
    }
}

// Expansion of the quad at (qx, qy) of a staged window: the interior formula
// when the whole tile's neighbourhoods lie inside the coarse level, else the
// per-position border weights and divisors.
template <bool NONNEG>
__device__ __forceinline__ void ef_expand(const int32_t (*s)[ESW], bool interior, int qx, int qy, int X, int Y,
                                          int cw, int ch, int dw, int dh, int wrap, int32_t e[4])
{
    if (interior) {
        int32_t v[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                v[r][c] = s[qy + r][qx + c];
            }
        }
        expand9<NONNEG>(v, e);
        return;
    }
    expand_quad(s, qx, qy, X, Y, cw, ch, dw, dh, wrap, e);
}

// Two horizontally adjacent pixels (the first at an even x) of an
// interleaved image as 2*S*sizeof(TIn) / UNIT words of UNIT bytes (UNIT: the
// largest power of two, at most 16, dividing the pair's size; the caller
// checks that the image's base and row pitch are multiples of it).
template <int U> struct PairWord;
template <> struct PairWord<2> { typedef uint16_t type; };
template <> struct PairWord<4> { typedef uint32_t type; };
template <> struct PairWord<8> { typedef uint2 type; };
template <> struct PairWord<16> { typedef uint4 type; };

template <typename TIn, int S>
struct PixelPair {
    static constexpr int BYTES = 2 * S * (int)sizeof(TIn);
    static constexpr int UNIT = (BYTES % 16 == 0) ? 16 : (BYTES % 8 == 0) ? 8 : (BYTES % 4 == 0) ? 4 : 2;
    static constexpr int NW = BYTES / UNIT;
    typedef typename PairWord<UNIT>::type W;
    __device__ __forceinline__ static void load(const TIn* p, TIn (&px)[2][S])
    {
        union {
            W w[NW];
            TIn s[2 * S];
        } u;
#pragma unroll
        for (int i = 0; i < NW; ++i) {
            u.w[i] = __ldg(reinterpret_cast<const W*>(p) + i);
        }
#pragma unroll
        for (int i = 0; i < S; ++i) {
            px[0][i] = u.s[i];
            px[1][i] = u.s[S + i];
        }
    }
};

// Two adjacent samples of a planar level or mask (x even), as ld2 of the
// enblend tiles through the read-only path.
template <typename T>
__device__ __forceinline__ void ld_pair(const T* p, int32_t& a, int32_t& b)
{
    ld2<T, true>(p, a, b);
}

// ---------------------------------------------------------------------------
// top level: R = sum_k fromRealPromote(G_k * M_k / D)
// ---------------------------------------------------------------------------

template <typename T, typename TM>
struct EfLevelArgs {
    int K, C, dw, dh, cw, ch, wrap, mfrac;
    const T* g[kEfuseMaxK];   // level l of the image pyramids
    const T* gc[kEfuseMaxK];  // level l + 1
    const TM* m[kEfuseMaxK];  // level l of the mask pyramids
    const T* rc;              // R[l + 1]
    T* r;                     // R[l]
    int64_t pitch, plane, cpitch, cplane;
};

template <typename T, typename TM, int F>
__global__ void __launch_bounds__(256) k_ef_top(const __grid_constant__ EfLevelArgs<T, TM> a)
{
    griddep_wait();
    griddep_launch();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= a.dw) {
        return;
    }
    const int64_t o = (int64_t)y * a.pitch + x;
    for (int c = 0; c < a.C; ++c) {
        int32_t acc = 0;
        for (int k = 0; k < a.K; ++k) {
            acc += (int32_t)mask_multiply<T, F>((int32_t)a.g[k][c * a.plane + o], (int32_t)a.m[k][o]);
        }
        a.r[c * a.plane + o] = cast_store<T>(acc);
    }
}

// ---------------------------------------------------------------------------
// levels L-2 .. 1: Laplacians, mask products, accumulation and collapse
// ---------------------------------------------------------------------------

// One 64x16 tile of level l (256 threads, one 2x2 quad each).  The K + 1
// coarse windows of every channel are staged together (one barrier);
// ss holds (K + 1) * C windows.
template <typename T, typename TM, int C, int F>
__global__ void __launch_bounds__(256, 3) k_ef_up(const __grid_constant__ EfLevelArgs<T, TM> a)
{
    extern __shared__ __align__(16) int32_t ewin[];
    int32_t (*ss)[ESH][ESW] = reinterpret_cast<int32_t (*)[ESH][ESW]>(ewin);
    griddep_wait();
    griddep_launch();
    const int K = a.K;
    const int X0 = blockIdx.x * ETW, Y0 = blockIdx.y * ETH;
    const int I0 = X0 >> 1, J0 = Y0 >> 1;
    const int qx = threadIdx.x % 32, qy = threadIdx.x / 32;
    const int i = I0 + qx, j = J0 + qy;
    const int X = 2 * i, Y = 2 * j;
    for (int k = 0; k <= K; ++k) {
        const T* src = k < K ? a.gc[k] : a.rc;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            ef_stage<T>(ss[k * C + c], src + c * a.cplane, a.cpitch, a.cw, a.ch, I0, J0, a.wrap);
        }
    }
    __syncthreads();
    if (X >= a.dw || Y >= a.dh) {
        return;
    }
    const bool interior = interior_tile(X0, Y0, a.dw, a.dh, I0, J0, a.cw, a.ch);
    int32_t acc[C][4];
#pragma unroll
    for (int c = 0; c < C; ++c) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            acc[c][q] = 0;
        }
    }
    int64_t off[4];
    bool ok[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int XX = X + (q & 1), YY = Y + (q >> 1);
        ok[q] = XX < a.dw && YY < a.dh;
        off[q] = (int64_t)min(YY, a.dh - 1) * a.pitch + min(XX, a.dw - 1);
    }
    // both pixels of a quad row in one paired load where x + 1 is inside
    const bool pair = X + 1 < a.dw;
    // the fine values of exposure k: mask m[4], image g[C][4]
    const auto fetch = [&](int k, int32_t (&m)[4], int32_t (&g)[C][4]) {
        if (pair) {
            ld_pair<TM>(a.m[k] + off[0], m[0], m[1]);
            ld_pair<TM>(a.m[k] + off[2], m[2], m[3]);
#pragma unroll
            for (int c = 0; c < C; ++c) {
                ld_pair<T>(a.g[k] + c * a.plane + off[0], g[c][0], g[c][1]);
                ld_pair<T>(a.g[k] + c * a.plane + off[2], g[c][2], g[c][3]);
            }
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                m[q] = (int32_t)__ldg(&a.m[k][off[q]]);
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    g[c][q] = (int32_t)__ldg(&a.g[k][c * a.plane + off[q]]);
                }
            }
        }
    };
    int32_t m[4], g[C][4];
    fetch(0, m, g);
    for (int k = 0; k < K; ++k) {
        int32_t mn[4], gn[C][4];
        if (k + 1 < K) {
            fetch(k + 1, mn, gn);  // in flight while exposure k is merged
        }
#pragma unroll
        for (int c = 0; c < C; ++c) {
            int32_t e[4];
            ef_expand<true>(ss[k * C + c], interior, qx, qy, X, Y, a.cw, a.ch, a.dw, a.dh, a.wrap, e);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int32_t lp = (int32_t)cast_store<T>((int64_t)g[c][q] - e[q]);
                acc[c][q] += (int32_t)mask_multiply<T, F>(lp, m[q]);
            }
        }
        if (k + 1 < K) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                m[q] = mn[q];
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    g[c][q] = gn[c][q];
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
        int32_t e[4];
        ef_expand<false>(ss[K * C + c], interior, qx, qy, X, Y, a.cw, a.ch, a.dw, a.dh, a.wrap, e);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (ok[q]) {
                a.r[c * a.plane + off[q]] = sat_store<T>((int32_t)cast_store<T>(acc[c][q]) + e[q]);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// level 0: from the K images and level-0 masks to the output pixels
// ---------------------------------------------------------------------------

template <typename TIn, typename T, typename TM>
struct EfOut0Args {
    int K, w, h, cw, ch, wrap;
    const TIn* img[kEfuseMaxK];
    int64_t ipitch[kEfuseMaxK];  // elements
    const TM* m0[kEfuseMaxK];
    int64_t mpitch;
    const T* g1[kEfuseMaxK];
    const T* r1;
    int64_t cpitch, cplane;
    const uint8_t* u0;
    int64_t upitch;
    TIn* out;
    int64_t opitch;
    int32_t* level0;
    int dither;
    uint32_t key;
    int32_t maxv;
    int vec;  // the images' bases and pitches allow the paired pixel loads
};

template <typename TIn, typename T, typename TM, int C, int S, int F>
__global__ void __launch_bounds__(256, 3) k_ef_out0(const __grid_constant__ EfOut0Args<TIn, T, TM> a)
{
    extern __shared__ __align__(16) int32_t ewin[];
    int32_t (*ss)[ESH][ESW] = reinterpret_cast<int32_t (*)[ESH][ESW]>(ewin);
    griddep_wait();
    griddep_launch();
    const int K = a.K;
    const int X0 = blockIdx.x * ETW, Y0 = blockIdx.y * ETH;
    const int I0 = X0 >> 1, J0 = Y0 >> 1;
    const int qx = threadIdx.x % 32, qy = threadIdx.x / 32;
    const int i = I0 + qx, j = J0 + qy;
    const int X = 2 * i, Y = 2 * j;
    for (int k = 0; k <= K; ++k) {
        const T* src = k < K ? a.g1[k] : a.r1;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            ef_stage<T>(ss[k * C + c], src + c * a.cplane, a.cpitch, a.cw, a.ch, I0, J0, a.wrap);
        }
    }
    __syncthreads();
    if (X >= a.w || Y >= a.h) {
        return;
    }
    const bool interior = interior_tile(X0, Y0, a.w, a.h, I0, J0, a.cw, a.ch);
    int32_t acc[C][4];
#pragma unroll
    for (int c = 0; c < C; ++c) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            acc[c][q] = 0;
        }
    }
    int XX[4], YY[4];
    bool ok[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        XX[q] = X + (q & 1);
        YY[q] = Y + (q >> 1);
        ok[q] = XX[q] < a.w && YY[q] < a.h;
        XX[q] = min(XX[q], a.w - 1);
        YY[q] = min(YY[q], a.h - 1);
    }
    // both pixels of a quad row in one paired load where x + 1 is inside and
    // the images are aligned for it
    const bool pair = a.vec && X + 1 < a.w;
    const auto fetch = [&](int k, int32_t (&m)[4], TIn (&px)[4][S]) {
        if (pair) {
            ld_pair<TM>(a.m0[k] + (int64_t)YY[0] * a.mpitch + X, m[0], m[1]);
            ld_pair<TM>(a.m0[k] + (int64_t)YY[2] * a.mpitch + X, m[2], m[3]);
            TIn pp[2][S];
            PixelPair<TIn, S>::load(a.img[k] + (int64_t)YY[0] * a.ipitch[k] + (int64_t)X * S, pp);
#pragma unroll
            for (int s = 0; s < S; ++s) {
                px[0][s] = pp[0][s];
                px[1][s] = pp[1][s];
            }
            PixelPair<TIn, S>::load(a.img[k] + (int64_t)YY[2] * a.ipitch[k] + (int64_t)X * S, pp);
#pragma unroll
            for (int s = 0; s < S; ++s) {
                px[2][s] = pp[0][s];
                px[3][s] = pp[1][s];
            }
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                m[q] = (int32_t)__ldg(&a.m0[k][(int64_t)YY[q] * a.mpitch + XX[q]]);
                const TIn* p = a.img[k] + (int64_t)YY[q] * a.ipitch[k] + (int64_t)XX[q] * S;
#pragma unroll
                for (int s = 0; s < S; ++s) {
                    px[q][s] = __ldg(&p[s]);
                }
            }
        }
    };
    int32_t m[4];
    TIn px[4][S];
    fetch(0, m, px);
    for (int k = 0; k < K; ++k) {
        int32_t mn[4];
        TIn pn[4][S];
        if (k + 1 < K) {
            fetch(k + 1, mn, pn);  // in flight while exposure k is merged
        }
#pragma unroll
        for (int c = 0; c < C; ++c) {
            int32_t e[4];
            ef_expand<true>(ss[k * C + c], interior, qx, qy, X, Y, a.cw, a.ch, a.w, a.h, a.wrap, e);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                // copyToPyramidImage: v << 7 (src/fixmath.h:197-202)
                const int32_t lp = (int32_t)cast_store<T>(((int64_t)px[q][c] << 7) - e[q]);
                acc[c][q] += (int32_t)mask_multiply<T, F>(lp, m[q]);
            }
        }
        if (k + 1 < K) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                m[q] = mn[q];
#pragma unroll
                for (int s = 0; s < S; ++s) {
                    px[q][s] = pn[q][s];
                }
            }
        }
    }
    int32_t res[C][4];
#pragma unroll
    for (int c = 0; c < C; ++c) {
        int32_t e[4];
        ef_expand<false>(ss[K * C + c], interior, qx, qy, X, Y, a.cw, a.ch, a.w, a.h, a.wrap, e);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            res[c][q] = (int32_t)sat_store<T>((int32_t)cast_store<T>(acc[c][q]) + e[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (!ok[q]) {
            continue;
        }
        const int64_t pix = (int64_t)YY[q] * a.w + XX[q];
        if (a.level0) {
#pragma unroll
            for (int c = 0; c < C; ++c) {
                a.level0[pix * C + c] = res[c][q];
            }
        }
        // copyFromPyramidImageIf (src/fixmath.h:2158-2294): the dither rule
        // where the union alpha is set, 0 elsewhere; an RGBA result's 4th
        // component is the union alpha
        const bool on = __ldg(&a.u0[(int64_t)YY[q] * a.upitch + XX[q]]) != 0;
        const uint32_t pixbits = mix32((uint32_t)pix ^ a.key);
        TIn o[S];
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const uint32_t bits = dither_sample_bits(a.key, pixbits, (uint64_t)pix, C, c, 7);
            o[c] = on ? (TIn)dither_rule(res[c][q], 7, a.dither == ENB_DITHER_NEAREST, bits, a.maxv) : (TIn)0;
        }
        if (S == 4) {
            o[S - 1] = on ? (TIn)a.maxv : (TIn)0;
        }
        TIn* dst = a.out + (int64_t)YY[q] * a.opitch + (int64_t)XX[q] * S;
#pragma unroll
        for (int s = 0; s < S; ++s) {
            dst[s] = o[s];
        }
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

static inline double esz_b(int dt) { return dt == ENB_U8 ? 1.0 : 2.0; }

static size_t win_smem(int K, int C) { return (size_t)(K + 1) * C * ESH * ESW * sizeof(int32_t); }

template <typename K_>
static void allow_smem(K_ kernel, size_t smem)
{
    if (smem > 48 * 1024) {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
}

template <typename TM>
static cudaError_t ef_weights_t(const EfuseHost& h, cudaStream_t st)
{
    EfWeightsArgs<TM> a{};
    a.K = h.K;
    a.w = h.w;
    a.h = h.h;
    a.hard = h.hard;
    a.mfrac = h.dtype == ENB_U8 ? 7 : 15;
    for (int k = 0; k < h.K; ++k) {
        a.img[k] = h.img[k];
        a.alpha[k] = h.alpha[k];
        a.min[k] = h.masks_in[k];
        a.mipitch[k] = h.mipitch[k];
        a.m0[k] = (TM*)h.m[k][0];
    }
    a.wp = h.wp;
    a.tab = h.tab;
    a.mpitch = h.pitch[0];
    a.u0 = h.u[0];
    a.upitch = h.upitch0;
    const int TW = EWX + 2 * ef_halo_x(h.wp), TH = EWY + 2 * iweight_halo(h.wp);
    const size_t smem = ((itile_bytes_rect(TW, TH) + 15) & ~(size_t)15) + 32 * sizeof(long long) +
                        (size_t)h.K * 256 * sizeof(float2);
    allow_smem(k_ef_weights<TM>, smem);
    const dim3 g((unsigned)((h.w + EWX - 1) / EWX), (unsigned)((h.h + EWY - 1) / EWY));
    return launch_pdl_smem(k_ef_weights<TM>, g, dim3(256), smem, st, a);
}

cudaError_t launch_ef_weights(const EfuseHost& h, cudaStream_t st)
{
    const double px = (double)h.w * h.h;
    double in = 0.0;
    for (int k = 0; k < h.K; ++k) {
        in += h.masks_in[k] ? 4.0 : h.S * esz_b(h.dtype) + (h.alpha[k].mode == kAlphaPlane ? 1.0 : 0.0);
    }
    note_launch("ef_weights", px * (in + h.K * (h.dtype == ENB_U8 ? 2.0 : 4.0) + 1.0));
    return h.dtype == ENB_U8 ? ef_weights_t<int16_t>(h, st) : ef_weights_t<int32_t>(h, st);
}

// Level-1 reduce of the K images straight from their pixels (PixelSourceV).
struct EfReduce0 {
    const EfuseHost& h;
    cudaStream_t st;
    cudaError_t err;
    template <typename TIn, typename T, int C, int S, int AM, bool VEC>
    void operator()()
    {
        using Src = PixelSourceV<TIn, C, S, AM, VEC>;
        ReduceJobsN<Src, T> jobs{};
        for (int k = 0; k < h.K; ++k) {
            const AlphaSrc& al = h.alpha[k];
            jobs.j[k] = ReduceJob<Src, T>{
                Src{(const TIn*)h.img[k].p, h.img[k].pitch, al.mode == kAlphaPlane ? al.plane.p : nullptr,
                    al.mode == kAlphaPlane ? al.plane.pitch : 0, al.lo, al.hi, 7},
                (T*)h.g[k][1], h.pitch[1], h.pitch[1] * h.lh[1], h.a[k][1], h.apitch[1]};
        }
        err = launch_reduce_n<Src, T, C, true>(jobs, h.K, h.w, h.h, h.lw[1], h.lh[1], h.wrap, st);
    }
};

template <typename T, int C>
static cudaError_t ef_reduce_images(const EfuseHost& h, int l, cudaStream_t st)
{
    using Src = PlanarSource<T, C, true>;
    ReduceJobsN<Src, T> jobs{};
    for (int k = 0; k < h.K; ++k) {
        jobs.j[k] = ReduceJob<Src, T>{Src{(const T*)h.g[k][l], h.pitch[l], h.pitch[l] * h.lh[l], h.a[k][l], h.apitch[l]},
                                      (T*)h.g[k][l + 1], h.pitch[l + 1], h.pitch[l + 1] * h.lh[l + 1], h.a[k][l + 1],
                                      h.apitch[l + 1]};
    }
    return launch_reduce_n<Src, T, C, true>(jobs, h.K, h.lw[l], h.lh[l], h.lw[l + 1], h.lh[l + 1], h.wrap, st);
}

template <typename TM>
static cudaError_t ef_reduce_masks(const EfuseHost& h, int l, cudaStream_t st)
{
    using Src = PlanarSource<TM, 1, true>;
    ReduceJobsN<Src, TM> jobs{};
    const int64_t ap = l == 0 ? h.upitch0 : h.apitch[l];
    for (int k = 0; k < h.K; ++k) {
        jobs.j[k] = ReduceJob<Src, TM>{Src{(const TM*)h.m[k][l], h.pitch[l], h.pitch[l] * h.lh[l], h.u[l], ap},
                                       (TM*)h.m[k][l + 1], h.pitch[l + 1], h.pitch[l + 1] * h.lh[l + 1], h.u[l + 1],
                                       h.apitch[l + 1]};
    }
    return launch_reduce_n<Src, TM, 1, true>(jobs, h.K, h.lw[l], h.lh[l], h.lw[l + 1], h.lh[l + 1], h.wrap, st);
}

cudaError_t launch_ef_reduce(const EfuseHost& h, int l, int masks, cudaStream_t st)
{
    const double sp = (double)h.lw[l] * h.lh[l], dp = (double)h.lw[l + 1] * h.lh[l + 1];
    const double ps = h.dtype == ENB_U8 ? 2.0 : 4.0;
    if (masks) {
        note_launch(l == 0 ? "ef_reduce0_mask" : "ef_reduce_mask", h.K * (sp * ps + dp * ps + dp) + sp);
        return h.dtype == ENB_U8 ? ef_reduce_masks<int16_t>(h, l, st) : ef_reduce_masks<int32_t>(h, l, st);
    }
    if (l == 0) {
        double in = 0.0;
        for (int k = 0; k < h.K; ++k) {
            in += sp * (h.S * esz_b(h.dtype) + (h.alpha[k].mode == kAlphaPlane ? 1.0 : 0.0));
        }
        note_launch("ef_reduce0", in + h.K * dp * (h.C * ps + 1.0));
        const PixelView& v = h.img[0];
        bool vec = h.S == 4;
        for (int k = 0; k < h.K; ++k) {
            const size_t px = (size_t)h.S * (size_t)esz_b(h.dtype);
            vec = vec && ((uintptr_t)h.img[k].p % px) == 0 && ((size_t)h.img[k].pitch * (size_t)esz_b(h.dtype)) % px == 0;
        }
        const int am = h.alpha[0].mode == kAlphaPlane ? 0 : (h.alpha[0].mode == kAlphaOpaque ? 1 : 2);
        EfReduce0 f{h, st, cudaErrorInvalidValue};
#define ENB_EF_CASE(TIN, TP, CC, SS, AMM, VV)                  \
    if (v.C == CC && h.S == SS && am == AMM && vec == VV) {    \
        f.template operator()<TIN, TP, CC, SS, AMM, VV>();     \
        return f.err;                                          \
    }
#define ENB_EF_TYPE(TIN, TP)                                   \
    ENB_EF_CASE(TIN, TP, 1, 1, 0, false)                       \
    ENB_EF_CASE(TIN, TP, 1, 1, 1, false)                       \
    ENB_EF_CASE(TIN, TP, 3, 3, 0, false)                       \
    ENB_EF_CASE(TIN, TP, 3, 3, 1, false)                       \
    ENB_EF_CASE(TIN, TP, 3, 4, 0, false)                       \
    ENB_EF_CASE(TIN, TP, 3, 4, 1, false)                       \
    ENB_EF_CASE(TIN, TP, 3, 4, 2, false)                       \
    ENB_EF_CASE(TIN, TP, 3, 4, 0, true)                        \
    ENB_EF_CASE(TIN, TP, 3, 4, 1, true)                        \
    ENB_EF_CASE(TIN, TP, 3, 4, 2, true)
        if (h.dtype == ENB_U8) {
            ENB_EF_TYPE(uint8_t, int16_t)
        } else {
            ENB_EF_TYPE(uint16_t, int32_t)
        }
#undef ENB_EF_TYPE
#undef ENB_EF_CASE
        return cudaErrorInvalidValue;
    }
    note_launch("ef_reduce", h.K * (sp * (h.C * ps + 1.0) + dp * (h.C * ps + 1.0)));
    if (h.dtype == ENB_U8) {
        return h.C == 1 ? ef_reduce_images<int16_t, 1>(h, l, st) : ef_reduce_images<int16_t, 3>(h, l, st);
    }
    return h.C == 1 ? ef_reduce_images<int32_t, 1>(h, l, st) : ef_reduce_images<int32_t, 3>(h, l, st);
}

template <typename T, typename TM>
static EfLevelArgs<T, TM> level_args(const EfuseHost& h, int l)
{
    EfLevelArgs<T, TM> a{};
    const bool top = l == h.L - 1;
    a.K = h.K;
    a.C = h.C;
    a.dw = h.lw[l];
    a.dh = h.lh[l];
    a.cw = top ? 1 : h.lw[l + 1];
    a.ch = top ? 1 : h.lh[l + 1];
    a.wrap = h.wrap;
    a.mfrac = h.dtype == ENB_U8 ? 7 : 15;
    for (int k = 0; k < h.K; ++k) {
        a.g[k] = (const T*)h.g[k][l];
        a.gc[k] = top ? nullptr : (const T*)h.g[k][l + 1];
        a.m[k] = (const TM*)h.m[k][l];
    }
    a.rc = top ? nullptr : (const T*)h.r[l + 1];
    a.r = (T*)h.r[l];
    a.pitch = h.pitch[l];
    a.plane = h.pitch[l] * h.lh[l];
    a.cpitch = top ? 0 : h.pitch[l + 1];
    a.cplane = top ? 0 : h.pitch[l + 1] * h.lh[l + 1];
    return a;
}

cudaError_t launch_ef_top(const EfuseHost& h, cudaStream_t st)
{
    const int l = h.L - 1;
    const double px = (double)h.lw[l] * h.lh[l], ps = h.dtype == ENB_U8 ? 2.0 : 4.0;
    note_launch("ef_top", px * (h.K * (h.C * ps + ps) + h.C * ps));
    const dim3 g((unsigned)((h.lw[l] + 255) / 256), (unsigned)h.lh[l]);
    if (h.dtype == ENB_U8) {
        return launch_pdl(k_ef_top<int16_t, int16_t, 7>, g, dim3(256), st, level_args<int16_t, int16_t>(h, l));
    }
    return launch_pdl(k_ef_top<int32_t, int32_t, 15>, g, dim3(256), st, level_args<int32_t, int32_t>(h, l));
}

template <typename T, typename TM, int C, int F>
static cudaError_t ef_up_t(const EfuseHost& h, int l, cudaStream_t st)
{
    const size_t smem = win_smem(h.K, C);
    allow_smem(k_ef_up<T, TM, C, F>, smem);
    const dim3 g((unsigned)((h.lw[l] + ETW - 1) / ETW), (unsigned)((h.lh[l] + ETH - 1) / ETH));
    return launch_pdl_smem(k_ef_up<T, TM, C, F>, g, dim3(256), smem, st, level_args<T, TM>(h, l));
}

cudaError_t launch_ef_up(const EfuseHost& h, int l, cudaStream_t st)
{
    const double px = (double)h.lw[l] * h.lh[l], cp = (double)h.lw[l + 1] * h.lh[l + 1];
    const double ps = h.dtype == ENB_U8 ? 2.0 : 4.0;
    note_launch("ef_up", px * (h.K * (h.C * ps + ps) + h.C * ps) + cp * (h.K + 1) * h.C * ps);
    if (h.dtype == ENB_U8) {
        return h.C == 1 ? ef_up_t<int16_t, int16_t, 1, 7>(h, l, st) : ef_up_t<int16_t, int16_t, 3, 7>(h, l, st);
    }
    return h.C == 1 ? ef_up_t<int32_t, int32_t, 1, 15>(h, l, st) : ef_up_t<int32_t, int32_t, 3, 15>(h, l, st);
}

template <typename TIn, typename T, typename TM, int C, int S, int F>
static cudaError_t ef_out0_t(const EfuseHost& h, cudaStream_t st)
{
    EfOut0Args<TIn, T, TM> a{};
    a.K = h.K;
    a.w = h.w;
    a.h = h.h;
    a.cw = h.lw[1];
    a.ch = h.lh[1];
    a.wrap = h.wrap;
    for (int k = 0; k < h.K; ++k) {
        a.img[k] = (const TIn*)h.img[k].p;
        a.ipitch[k] = h.img[k].pitch;
        a.m0[k] = (const TM*)h.m[k][0];
        a.g1[k] = (const T*)h.g[k][1];
    }
    a.mpitch = h.pitch[0];
    a.r1 = (const T*)h.r[1];
    a.cpitch = h.pitch[1];
    a.cplane = h.pitch[1] * h.lh[1];
    a.u0 = h.u[0];
    a.upitch = h.upitch0;
    a.out = (TIn*)h.out;
    a.opitch = h.opitch;
    a.level0 = h.level0;
    a.dither = h.dither;
    a.key = dither_key(h.seed);
    a.maxv = sizeof(TIn) == 1 ? 255 : 65535;
    a.vec = 1;
    for (int k = 0; k < h.K; ++k) {
        const size_t unit = (size_t)PixelPair<TIn, S>::UNIT;
        a.vec &= ((uintptr_t)h.img[k].p % unit) == 0 && ((size_t)h.img[k].pitch * sizeof(TIn)) % unit == 0;
    }
    const size_t smem = win_smem(h.K, C);
    allow_smem(k_ef_out0<TIn, T, TM, C, S, F>, smem);
    const dim3 g((unsigned)((h.w + ETW - 1) / ETW), (unsigned)((h.h + ETH - 1) / ETH));
    return launch_pdl_smem(k_ef_out0<TIn, T, TM, C, S, F>, g, dim3(256), smem, st, a);
}

cudaError_t launch_ef_out0(const EfuseHost& h, cudaStream_t st)
{
    const double px = (double)h.w * h.h, cp = (double)h.lw[1] * h.lh[1];
    const double ps = h.dtype == ENB_U8 ? 2.0 : 4.0, ss = esz_b(h.dtype);
    note_launch("ef_out0", px * (h.K * (h.S * ss + ps) + 1.0 + h.S * ss) + cp * (h.K + 1) * h.C * ps +
                               (h.level0 ? px * h.C * 4.0 : 0.0));
#define ENB_EF_OUT(TIN, TP, CC, SS, FF)                                    \
    if (h.C == CC && h.S == SS) {                                          \
        return ef_out0_t<TIN, TP, TP, CC, SS, FF>(h, st);                  \
    }
    if (h.dtype == ENB_U8) {
        ENB_EF_OUT(uint8_t, int16_t, 1, 1, 7)
        ENB_EF_OUT(uint8_t, int16_t, 3, 3, 7)
        ENB_EF_OUT(uint8_t, int16_t, 3, 4, 7)
    } else {
        ENB_EF_OUT(uint16_t, int32_t, 1, 1, 15)
        ENB_EF_OUT(uint16_t, int32_t, 3, 3, 15)
        ENB_EF_OUT(uint16_t, int32_t, 3, 4, 15)
    }
#undef ENB_EF_OUT
    return cudaErrorInvalidValue;
}

}  // namespace enb
