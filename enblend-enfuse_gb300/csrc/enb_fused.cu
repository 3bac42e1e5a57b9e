// enb_fused.cu -- fused level kernels of the enblend pyramid blend.
//
// The reference builds the white and black Laplacian pyramids and the mask
// Gaussian pyramid in full, blends level by level and collapses
// (src/enblend.h:384-510): every level crosses memory several times.  Here
//   * level 0 is never materialised: the first reduce reads the interleaved
//     RGBA pixels and converts them to fixed point on the fly;
//   * each coarser level l is one pass that forms both Laplacians
//     G_l - E(G_{l+1}), blends them under the mask pyramid and adds the
//     expansion of the collapsed level l+1 (the collapse recursion
//     R_l = fromPromote(B_l + E(R_{l+1})), src/pyramid.h:1758-1784);
//   * level 0 is one pass from the two images, the seam mask and the three
//     level-1 pyramids straight to the dithered output pixels.
// The integer results are the reference's: each step is the same operation on
// the same integers, only the order of the passes over memory changes.
//
// Kernel structure: a CTA covers a 64x16 destination tile as 2x2 quads (one
// per thread).  Each thread first issues its global loads (fine-level values
// or image pixels), then the CTA stages the 34x10 coarse neighbourhoods of the
// three level-(l+1) pyramids in shared memory.  Tiles inside the image take a
// path without bounds or border weights, expand only the planes the quad's
// seam mask selects, and use paired/vector loads and stores.  Level 0 of RGBA
// images runs instead as one persistent launch (k_out0_tma): the border ring
// through the same tile code, then the interior tiles through a two-stage
// pipeline fed by TMA (coarse planes; image and mask rows when they start on
// 16-byte boundaries) or per-thread cp.async (image rows off that grid).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "enb_device.cuh"
#include "enb_internal.h"
#include "enb_reduce.cuh"
#include "enb_pixels.cuh"
#include "enb_tiles.cuh"
#include "enb_tma.cuh"

namespace enb {

// ---------------------------------------------------------------------------
// Merge helpers
// ---------------------------------------------------------------------------

// Top level: R = blend(M, Gw, Gb) (the top Laplacian level is the Gaussian).
template <typename T, typename TM, int C>
__global__ void __launch_bounds__(256) k_blend_into(const TM* __restrict__ mask, int64_t mpitch,
                                                    const T* __restrict__ gw, const T* __restrict__ gb,
                                                    T* __restrict__ r, int64_t pitch, int64_t plane, int w, int h,
                                                    int32_t white_value)
{
    griddep_wait();
    griddep_launch();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const int64_t o = (int64_t)y * pitch + x;
    const int32_t m = (int32_t)mask[(int64_t)y * mpitch + x];
#pragma unroll
    for (int c = 0; c < C; ++c) {
        r[c * plane + o] = (T)blend1<T>(m, white_value, gw[c * plane + o], gb[c * plane + o]);
    }
}

// ---------------------------------------------------------------------------
// Coarse level l (1 <= l <= L-2): Laplacians, blend, collapse in one pass
// ---------------------------------------------------------------------------

template <typename T, typename TM, int C>
__global__ void __launch_bounds__(256) k_up_level(CoarseLevels cl, const TM* __restrict__ mask, int64_t mpitch,
                                                  const T* __restrict__ gw, const T* __restrict__ gb,
                                                  T* __restrict__ r, int64_t pitch, int64_t plane, int w, int h,
                                                  int32_t white_value, int wrap)
{
    __shared__ int4 sbuf[C][ESH][ESW];
    griddep_wait();
    griddep_launch();
    up_tile<T, TM, C, true, 256>(cl, mask, mpitch, gw, gb, r, pitch, plane, w, h, white_value, wrap,
                                 blockIdx.x * ETW, blockIdx.y * ETH, sbuf);
}

// ---------------------------------------------------------------------------
// Level 0: images, seam mask and level-1 pyramids -> dithered output pixels
// ---------------------------------------------------------------------------

struct Out0Args {
    const void* white;
    const void* black;
    int64_t wpitch, bpitch;      // elements
    const uint8_t* wa;           // alpha planes (AM 0) or null
    const uint8_t* ba;
    int64_t wapitch, bapitch;
    uint32_t alo, ahi;           // channel-3 threshold (AM 2)
    const uint8_t* mask;
    int64_t mpitch;
    int mfrac;
    int32_t white_value;
    void* out;
    int64_t opitch;              // elements
    uint8_t* out_alpha;          // union alpha plane or null
    int64_t oapitch;
    int32_t* level0;             // collapsed level 0 (interleaved int32) or null
    int w, h, frac, dither, has_coarse, wrap;
    uint64_t seed;
    uint32_t key;                // dither_key(seed)
    int32_t maxv;
    int tx0, ty0;                // first tile column (64 pixels) and row (16 rows) of the launch
    unsigned int* err;           // device error word (bit 0: a tile wait timed out)
    uint32_t tx_extra;           // bytes each stage's barrier expects beyond its
                                 // copies (0; > 0 only to test the timeout path)
};

// Coarse taps of an interior tile packed as (Gw, Gb, R) int4 per position
// and channel (the staging of k_out0).
struct PackedTaps {
    const int4 (*s)[ESH][ESW];
    __device__ __forceinline__ void operator()(int c, int qx, int qy, int kind, int32_t (&ew)[4], int32_t (&eb)[4],
                                               int32_t (&er)[4]) const
    {
        expand_packed(s[c], qx, qy, kind, ew, eb, er);
    }
};

// Level-0 output of the interior quad (X, Y) (tile position qx, qy) from its
// loaded pixels and seam mask and the packed coarse taps of the tile.
template <typename TIn, typename T, int C, int S, int AM, bool VEC, typename Taps>
__device__ __forceinline__ void out0_quad(const Out0Args& a, const Taps& taps, int X, int Y, int qx, int qy,
                                          const TIn (&wp)[4][S], const TIn (&bp)[4][S], const int32_t (&mk)[4])
{
    constexpr int F = 7;
    constexpr int MF = sizeof(TIn) == 1 ? 7 : 15;
    constexpr int32_t WV = 255 << MF;
    constexpr int32_t MAXV = sizeof(TIn) == 1 ? 255 : 65535;
    const bool nearest = a.dither == ENB_DITHER_NEAREST;
    bool uni[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int XX = X + (q & 1), YY = Y + (q >> 1);
        uni[q] = pixel_alpha<AM, TIn, S>(wp[q], a.wa, a.wapitch, XX, YY, a.alo, a.ahi) ||
                 pixel_alpha<AM, TIn, S>(bp[q], a.ba, a.bapitch, XX, YY, a.alo, a.ahi);
    }
    const int kind = quad_kind(mk, WV);
    const uint32_t pix0 = (uint32_t)Y * (uint32_t)a.w + (uint32_t)X;
    const uint32_t pixq[4] = {pix0, pix0 + 1, pix0 + (uint32_t)a.w, pix0 + (uint32_t)a.w + 1};
    int32_t res[C][4];
#pragma unroll
    for (int c = 0; c < C; ++c) {
        int32_t ew[4], eb[4], er[4];
        taps(c, qx, qy, kind, ew, eb, er);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            res[c][q] = merge_sample<T>(kind, mk[q], WV, (int32_t)wp[q][c] << F, ew[q], (int32_t)bp[q][c] << F,
                                        eb[q], er[q]);
        }
    }
    if (a.level0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
            for (int c = 0; c < C; ++c) {
                a.level0[(uint64_t)pixq[q] * C + c] = res[c][q];
            }
        }
    }
    TIn* out0 = reinterpret_cast<TIn*>(a.out) + (int64_t)Y * a.opitch + (int64_t)X * S;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint32_t pb = mix32(pixq[q] ^ a.key);
        TIn o[S];
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const int32_t d = dither_rule(res[c][q], F, nearest, pb >> (8 * c), MAXV);
            o[c] = uni[q] ? (TIn)d : bp[q][c];
        }
        if (S == 4) {
            o[S - 1] = uni[q] ? (TIn)MAXV : (TIn)0;
        }
        st_px<TIn, S, VEC>(out0 + (q >> 1) * a.opitch + (q & 1) * S, o);
    }
    if (a.out_alpha) {
        uint8_t* oa = a.out_alpha + (int64_t)Y * a.oapitch + X;
        oa[0] = uni[0] ? 255 : 0;
        oa[1] = uni[1] ? 255 : 0;
        oa[a.oapitch] = uni[2] ? 255 : 0;
        oa[a.oapitch + 1] = uni[3] ? 255 : 0;
    }
}

// Level-0 output of any tile (X0, Y0) (border tiles, or a single level): the
// quads' pixels from clamped positions, the coarse planes staged in ss with
// the border and wrap rules of stage_coarse.  All threads of the CTA call
// (it contains a barrier); ss must be free on entry.
template <typename TIn, typename T, int C, int S, int AM, bool VEC>
__device__ __forceinline__ void out0_border_tile(const CoarseLevels& cl, const Out0Args& a, int X0, int Y0,
                                                 int32_t (*ss)[ESH][ESW])
{
    constexpr int F = 7;
    constexpr int MF = sizeof(TIn) == 1 ? 7 : 15;
    constexpr int32_t WV = 255 << MF;
    constexpr int32_t MAXV = sizeof(TIn) == 1 ? 255 : 65535;
    const int I0 = X0 >> 1, J0 = Y0 >> 1;
    const int qx = threadIdx.x % 32, qy = threadIdx.x / 32;
    const int X = 2 * (I0 + qx), Y = 2 * (J0 + qy);
    const bool nearest = a.dither == ENB_DITHER_NEAREST;
    // the quad's pixels, loaded (from
    // clamped positions, unconditionally) before the barrier
    TIn wp[4][S], bp[4][S];
    int32_t mk[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int XX = min(X + (q & 1), a.w - 1), YY = min(Y + (q >> 1), a.h - 1);
        ld_px<TIn, S, VEC>(reinterpret_cast<const TIn*>(a.white) + (int64_t)YY * a.wpitch + (int64_t)XX * S, wp[q]);
        ld_px<TIn, S, VEC>(reinterpret_cast<const TIn*>(a.black) + (int64_t)YY * a.bpitch + (int64_t)XX * S, bp[q]);
        mk[q] = (int32_t)__ldg(&a.mask[(int64_t)YY * a.mpitch + XX]) << MF;
    }
    if (a.has_coarse) {
        stage_coarse<3 * C, T, true, 256>(ss, cl, I0, J0, a.wrap);
        __syncthreads();
    }
    if (X >= a.w || Y >= a.h) {
        return;
    }
    bool uni[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        // clamped like the loads above; pixels outside the image are not stored
        const int XX = min(X + (q & 1), a.w - 1), YY = min(Y + (q >> 1), a.h - 1);
        uni[q] = pixel_alpha<AM, TIn, S>(wp[q], a.wa, a.wapitch, XX, YY, a.alo, a.ahi) ||
                 pixel_alpha<AM, TIn, S>(bp[q], a.ba, a.bapitch, XX, YY, a.alo, a.ahi);
    }
    TIn o[4][S];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int c = 0; c < S; ++c) {
            o[q][c] = bp[q][c];
        }
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
        int32_t ew[4] = {0, 0, 0, 0}, eb[4] = {0, 0, 0, 0}, er[4] = {0, 0, 0, 0};
        if (a.has_coarse) {
            expand_quad(ss[c], qx, qy, X, Y, cl.w, cl.h, a.w, a.h, a.wrap, ew);
            expand_quad(ss[C + c], qx, qy, X, Y, cl.w, cl.h, a.w, a.h, a.wrap, eb);
            expand_quad(ss[2 * C + c], qx, qy, X, Y, cl.w, cl.h, a.w, a.h, a.wrap, er);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int XX = X + (q & 1), YY = Y + (q >> 1);
            if (XX >= a.w || YY >= a.h) {
                continue;
            }
            const int32_t lw = (int32_t)cast_store<T>((int64_t)((int32_t)wp[q][c] << F) - ew[q]);
            const int32_t lb = (int32_t)cast_store<T>((int64_t)((int32_t)bp[q][c] << F) - eb[q]);
            const int32_t res = (int32_t)sat_store<T>(blend1<T>(mk[q], WV, lw, lb) + er[q]);
            const uint64_t pix = (uint64_t)YY * (uint64_t)a.w + (uint64_t)XX;
            if (a.level0) {
                a.level0[pix * C + c] = res;
            }
            if (uni[q]) {
                const uint32_t bits = mix32((uint32_t)pix ^ a.key) >> (8 * c);
                o[q][c] = (TIn)dither_rule(res, F, nearest, bits, MAXV);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int XX = X + (q & 1), YY = Y + (q >> 1);
        if (XX >= a.w || YY >= a.h) {
            continue;
        }
        if (S == 4) {
            o[q][S - 1] = uni[q] ? (TIn)MAXV : (TIn)0;
        }
        st_px<TIn, S, VEC>(reinterpret_cast<TIn*>(a.out) + (int64_t)YY * a.opitch + (int64_t)XX * S, o[q]);
        if (a.out_alpha) {
            a.out_alpha[(int64_t)YY * a.oapitch + XX] = uni[q] ? 255 : 0;
        }
    }
}

template <typename TIn, typename T, int C, int S, int AM, bool VEC>
__global__ void __launch_bounds__(256, 3) k_out0(CoarseLevels cl, Out0Args a)
{
    // fixed-point formats of the enblend pyramids (the host checks a.frac,
    // a.mfrac, a.white_value and a.maxv against these): image 9.7 / 17.7,
    // mask 9.7 (8-bit) / 9.15 (16-bit); one hash per pixel covers the dither
    // bits of all its samples (F - 1 <= 8, C <= 4)
    constexpr int MF = sizeof(TIn) == 1 ? 7 : 15;
    static_assert(C <= 4, "per-pixel dither bits");
    // packed int4 taps for interior tiles, 3C int32 planes for border tiles
    __shared__ int4 sbuf[C][ESH][ESW];
    int32_t (*ss)[ESH][ESW] = reinterpret_cast<int32_t (*)[ESH][ESW]>(&sbuf[0][0][0]);
    griddep_wait();
    griddep_launch();
    const int X0 = (blockIdx.x + a.tx0) * ETW, Y0 = (blockIdx.y + a.ty0) * ETH;
    const int I0 = X0 >> 1, J0 = Y0 >> 1;
    const int qx = threadIdx.x % 32, qy = threadIdx.x / 32;
    const int i = I0 + qx, j = J0 + qy;
    const int X = 2 * i, Y = 2 * j;

    if (a.has_coarse && interior_tile(X0, Y0, a.w, a.h, I0, J0, cl.w, cl.h)) {
        // interior tile: no bounds, packed taps, only the expansions the seam
        // mask of the quad selects
        TIn wp[4][S], bp[4][S];
        const TIn* w0 = reinterpret_cast<const TIn*>(a.white) + (int64_t)Y * a.wpitch + (int64_t)X * S;
        const TIn* b0 = reinterpret_cast<const TIn*>(a.black) + (int64_t)Y * a.bpitch + (int64_t)X * S;
        ld_px<TIn, S, VEC>(w0, wp[0]);
        ld_px<TIn, S, VEC>(w0 + S, wp[1]);
        ld_px<TIn, S, VEC>(w0 + a.wpitch, wp[2]);
        ld_px<TIn, S, VEC>(w0 + a.wpitch + S, wp[3]);
        ld_px<TIn, S, VEC>(b0, bp[0]);
        ld_px<TIn, S, VEC>(b0 + S, bp[1]);
        ld_px<TIn, S, VEC>(b0 + a.bpitch, bp[2]);
        ld_px<TIn, S, VEC>(b0 + a.bpitch + S, bp[3]);
        const uint8_t* m0 = a.mask + (int64_t)Y * a.mpitch + X;
        const int32_t mk[4] = {(int32_t)__ldg(m0) << MF, (int32_t)__ldg(m0 + 1) << MF,
                               (int32_t)__ldg(m0 + a.mpitch) << MF, (int32_t)__ldg(m0 + a.mpitch + 1) << MF};
        stage_coarse4_interior<C, T, true, 256>(sbuf, cl, I0, J0);
        __syncthreads();
        out0_quad<TIn, T, C, S, AM, VEC>(a, PackedTaps{sbuf}, X, Y, qx, qy, wp, bp, mk);
        return;
    }

    out0_border_tile<TIn, T, C, S, AM, VEC>(cl, a, X0, Y0, ss);
}

// ---------------------------------------------------------------------------
// Level 0 on the interior tiles: persistent CTAs fed by a TMA pipeline
// ---------------------------------------------------------------------------
//
// Each CTA walks its share of the interior tiles (blockIdx.x, + gridDim.x,
// ...) with two shared-memory stages: while the quads of one tile are
// merged, the TMA unit copies the next tile's image rows, seam-mask rows and
// coarse neighbourhoods into the other stage, so that the loads of a tile
// are in flight during the arithmetic of the previous one and no thread
// spends registers or issue slots on them.  The merge of a quad is
// out0_quad's, with the coarse taps read from the planar TMA boxes.

// Tensor maps of one launch: the interleaved images as 2-D arrays of w * S
// samples by h rows and the seam mask (used when their rows start on 16-byte
// boundaries), and the 3C coarse planes (128-byte aligned rows).
struct Out0Maps {
    CUtensorMap white, black, mask;
    CUtensorMap coarse[9];
};

// How the fine level reaches a stage: OUT0_TMA_ROWS, one 2-D TMA box per
// image and one for the mask rows; OUT0_CP_ASYNC, each thread copies its own
// quad's eight pixels with cp.async, a row's pixel pair in one copy where it
// is aligned to its size (any pixel-aligned row pitch), and reads its four
// mask bytes into registers one tile ahead.
constexpr int OUT0_TMA_ROWS = 0, OUT0_CP_ASYNC = 1;

// One stage: the fine-level pixels of both images (MODE 0: the tile's 16 rows
// of 64 pixels; MODE 1: pixel-pair slots [image][quad row][thread]), the mask
// rows (MODE 0) and, per coarse plane, ESH rows
// of CBW samples that start XOFF samples left of the tile's first coarse
// column I0 (a TMA box starts on a 16-byte boundary; the taps used are I0-1
// .. I0+32).  Every part is a multiple of 128 bytes.
template <typename TIn, typename T, int C, int S, int MODE>
struct Out0Stage {
    static constexpr int XOFF = 16 / (int)sizeof(T);
    static constexpr int CBW = (ESW - 1 + XOFF + XOFF - 1) / XOFF * XOFF;
    static constexpr int PXB = S * (int)sizeof(TIn);
    static constexpr int IMG = ETH * ETW * PXB;
    static constexpr int MSK = MODE == OUT0_TMA_ROWS ? ETH * ETW : 0;
    static constexpr int PLANE_BYTES = ESH * CBW * (int)sizeof(T);
    static constexpr int PLANE = (PLANE_BYTES + 127) / 128 * 128;
    static constexpr int BYTES = 2 * IMG + MSK + 3 * C * PLANE;
    // bytes the TMA writes per stage
    static constexpr uint32_t TX = (uint32_t)((MODE == OUT0_TMA_ROWS ? 2 * IMG + MSK : 0) + 3 * C * PLANE_BYTES);
    static_assert(IMG % 128 == 0 && MSK % 128 == 0, "stage parts stay 128-byte aligned");
};

// Coarse taps of an interior quad from the planar boxes (plane q at p + q *
// PS samples, rows of CBW samples; column 0 is coarse column I0 - XOFF).
template <typename T, int C, int CBW, int PS, int XOFF>
struct PlanarTaps {
    const T* p;
    __device__ __forceinline__ void load(int q, int off, int32_t (&v)[3][3]) const
    {
        const T* b = p + q * PS + off;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                v[r][c] = (int32_t)b[r * CBW + c];
            }
        }
    }
    __device__ __forceinline__ void operator()(int c, int qx, int qy, int kind, int32_t (&ew)[4], int32_t (&eb)[4],
                                               int32_t (&er)[4]) const
    {
        const int off = qy * CBW + qx + XOFF - 1;
        int32_t v[3][3];
        load(2 * C + c, off, v);
        expand9<false>(v, er);
        if (kind != 2) {
            load(c, off, v);
            expand9<true>(v, ew);
        }
        if (kind != 1) {
            load(C + c, off, v);
            expand9<true>(v, eb);
        }
    }
};

// Two horizontally adjacent interleaved pixels from shared memory (S == 4:
// one 16-byte (u16) or 8-byte (u8) access).
template <typename TIn, int S>
__device__ __forceinline__ void lds_pixel_pair(const TIn* p, TIn (&a)[S], TIn (&b)[S])
{
    static_assert(S == 4, "RGBA pixels");
    if (sizeof(TIn) == 2) {
        const uint4 v = *reinterpret_cast<const uint4*>(p);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            a[2 * c] = (TIn)(w[c] & 0xffffu);
            a[2 * c + 1] = (TIn)(w[c] >> 16);
            b[2 * c] = (TIn)(w[2 + c] & 0xffffu);
            b[2 * c + 1] = (TIn)(w[2 + c] >> 16);
        }
    } else {
        const uint2 v = *reinterpret_cast<const uint2*>(p);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            a[c] = (TIn)((v.x >> (8 * c)) & 0xffu);
            b[c] = (TIn)((v.y >> (8 * c)) & 0xffu);
        }
    }
}

// The tiles of one level-0 launch over tile rows [ty0, ty0 + nty) and tile
// columns [0, cols): the interior rectangle of columns bx0 .. bx0 + nbx - 1
// (bx0 = 1) and rows by0 .. by0 + nby - 1, and the ring around it in the
// band -- the first column, the columns right of the rectangle, and the band
// rows above and below it.
struct Out0Ring {
    int bx0, nbx, by0, nby;  // interior rectangle
    int ty0, nty, cols;      // band
    __host__ __device__ int right() const { return cols - bx0 - nbx; }
    __host__ __device__ int above() const { return by0 - ty0; }
    __host__ __device__ int below() const { return ty0 + nty - by0 - nby; }
    __host__ __device__ int count() const { return nty * (bx0 + right()) + nbx * (above() + below()); }
    // tile (column, row) of ring tile t
    __device__ void tile(int t, int& bx, int& by) const
    {
        const int nl = nty * bx0, nr = nty * right(), na = nbx * above();
        if (t < nl) {
            bx = t % bx0;
            by = ty0 + t / bx0;
        } else if ((t -= nl) < nr) {
            bx = bx0 + nbx + t % right();
            by = ty0 + t / right();
        } else if ((t -= nr) < na) {
            bx = bx0 + t % nbx;
            by = ty0 + t / nbx;
        } else {
            t -= na;
            bx = bx0 + t % nbx;
            by = by0 + nby + t / nbx;
        }
    }
};

// The ring tiles go first, through out0_border_tile with their coarse planes
// staged in stage 1, while the copies of the CTA's first interior tile land
// in stage 0; then the pipelined interior tiles.
template <typename TIn, typename T, int C, int S, int AM, int MODE>
__global__ void __launch_bounds__(256, 3) k_out0_tma(const __grid_constant__ Out0Maps maps, CoarseLevels cl, Out0Args a,
                                                     Out0Ring ring)
{
    const int bx0 = ring.bx0, nbx = ring.nbx, by0 = ring.by0, nby = ring.nby;
    using St = Out0Stage<TIn, T, C, S, MODE>;
    constexpr int MF = sizeof(TIn) == 1 ? 7 : 15;
    extern __shared__ __align__(128) unsigned char osm[];
    __shared__ __align__(8) uint64_t bar[2];
    const int ntiles = nbx * nby;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_init_fence();
        if (MODE == OUT0_TMA_ROWS) {
            tma_prefetch_map(&maps.white);
            tma_prefetch_map(&maps.black);
            tma_prefetch_map(&maps.mask);
        }
    }
    __syncthreads();
    griddep_wait();
    griddep_launch();
    const int qx = threadIdx.x % 32, qy = threadIdx.x / 32;
    const auto origin = [&](int t, int& X0, int& Y0) {
        X0 = (bx0 + t % nbx) * ETW;
        Y0 = (by0 + t / nbx) * ETH;
    };
    // the TMA part of a tile's copies (thread 0 arms the stage's barrier,
    // warp 0 issues)
    const auto issue_tma = [&](int t, int s) {
        int X0, Y0;
        origin(t, X0, Y0);
        const int I0 = X0 >> 1, J0 = Y0 >> 1, l = threadIdx.x;
        unsigned char* st = osm + s * St::BYTES;
        if (l == 0) {
            mbar_arrive_expect_tx(&bar[s], St::TX + a.tx_extra);
            if (MODE == OUT0_TMA_ROWS) {
                tma_load_2d(st, &maps.white, X0 * S, Y0, &bar[s]);
                tma_load_2d(st + St::IMG, &maps.black, X0 * S, Y0, &bar[s]);
                tma_load_2d(st + 2 * St::IMG, &maps.mask, X0, Y0, &bar[s]);
            }
        }
        __syncwarp();
        if (l < 3 * C) {
            tma_load_2d(st + 2 * St::IMG + St::MSK + l * St::PLANE, &maps.coarse[l], I0 - St::XOFF, J0 - 1, &bar[s]);
        }
    };
    // MODE 1: this thread's eight pixels of a tile (one commit group) and
    // its four mask bytes
    const auto issue_own = [&](int t, int s) {
        int X0, Y0;
        origin(t, X0, Y0);
        unsigned char* st = osm + s * St::BYTES;
        // the two pixels of a quad row: one copy when the pair is aligned to
        // its size (on the rows that start on such a boundary), else two
        const auto pair = [&](unsigned char* dst, const TIn* src) {
            if (((uintptr_t)src & (2 * St::PXB - 1)) == 0) {
                cp_async_bytes<2 * St::PXB>(dst, src);
            } else {
                cp_async_bytes<St::PXB>(dst, src);
                cp_async_bytes<St::PXB>(dst + St::PXB, src + S);
            }
        };
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int64_t y = Y0 + 2 * qy + h, x = X0 + 2 * qx;
            const int slot = (h * 256 + (int)threadIdx.x) * 2 * St::PXB;
            pair(st + slot, reinterpret_cast<const TIn*>(a.white) + y * a.wpitch + x * S);
            pair(st + St::IMG + slot, reinterpret_cast<const TIn*>(a.black) + y * a.bpitch + x * S);
        }
        cp_async_commit();
    };
    const auto mask4 = [&](int t) -> uint32_t {
        int X0, Y0;
        origin(t, X0, Y0);
        const uint8_t* m0 = a.mask + (int64_t)(Y0 + 2 * qy) * a.mpitch + X0 + 2 * qx;
        return (uint32_t)__ldg(m0) | (uint32_t)__ldg(m0 + 1) << 8 | (uint32_t)__ldg(m0 + a.mpitch) << 16 |
               (uint32_t)__ldg(m0 + a.mpitch + 1) << 24;
    };
    int t = blockIdx.x;
    uint32_t mreg = 0;
    if (t < ntiles) {
        if (threadIdx.x < 32) {
            issue_tma(t, 0);
        }
        if (MODE == OUT0_CP_ASYNC) {
            issue_own(t, 0);
            mreg = mask4(t);
        }
    }
    {
        static_assert(St::BYTES >= (int)sizeof(int32_t) * 3 * C * ESH * ESW, "ring staging fits");
        int32_t (*ss)[ESH][ESW] = reinterpret_cast<int32_t (*)[ESH][ESW]>(osm + St::BYTES);
        const int nring = ring.count();
        for (int r = blockIdx.x; r < nring; r += gridDim.x) {
            int bx, by;
            ring.tile(r, bx, by);
            __syncthreads();  // the previous ring tile's readers of ss are done
            out0_border_tile<TIn, T, C, S, AM, true>(cl, a, bx * ETW, by * ETH, ss);
        }
        __syncthreads();  // stage 1 is free for the copies
    }
    for (int it = 0; t < ntiles; ++it, t += gridDim.x) {
        const int s = it & 1;
        const bool next = t + (int)gridDim.x < ntiles;
        uint32_t mnext = 0;
        if (next) {
            // the other stage was last read before the previous barrier
            if (threadIdx.x < 32) {
                fence_proxy_async();
                issue_tma(t + gridDim.x, s ^ 1);
            }
            if (MODE == OUT0_CP_ASYNC) {
                issue_own(t + gridDim.x, s ^ 1);
                mnext = mask4(t + gridDim.x);
            }
        }
        const bool ok = mbar_wait_bounded(&bar[s], (uint32_t)(it >> 1) & 1u);
        int X0, Y0;
        origin(t, X0, Y0);
        const int X = X0 + 2 * qx, Y = Y0 + 2 * qy;
        const unsigned char* st = osm + s * St::BYTES;
        TIn wp[4][S], bp[4][S];
        int32_t mk[4];
        if (MODE == OUT0_TMA_ROWS) {
            const TIn* ws = reinterpret_cast<const TIn*>(st) + (2 * qy * ETW + 2 * qx) * S;
            const TIn* bs = reinterpret_cast<const TIn*>(st + St::IMG) + (2 * qy * ETW + 2 * qx) * S;
            const uint8_t* ms = st + 2 * St::IMG + 2 * qy * ETW + 2 * qx;
            lds_pixel_pair<TIn, S>(ws, wp[0], wp[1]);
            lds_pixel_pair<TIn, S>(ws + ETW * S, wp[2], wp[3]);
            lds_pixel_pair<TIn, S>(bs, bp[0], bp[1]);
            lds_pixel_pair<TIn, S>(bs + ETW * S, bp[2], bp[3]);
            const uint32_t m01 = *reinterpret_cast<const uint16_t*>(ms);
            const uint32_t m23 = *reinterpret_cast<const uint16_t*>(ms + ETW);
            mreg = m01 | m23 << 16;
        } else {
            // this thread's own copies of this tile are complete
            if (next) {
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int slot = (h * 256 + (int)threadIdx.x) * 2 * St::PXB;
                lds_pixel_pair<TIn, S>(reinterpret_cast<const TIn*>(st + slot), wp[2 * h], wp[2 * h + 1]);
                lds_pixel_pair<TIn, S>(reinterpret_cast<const TIn*>(st + St::IMG + slot), bp[2 * h], bp[2 * h + 1]);
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            mk[q] = (int32_t)((mreg >> (8 * q)) & 0xffu) << MF;
        }
        const PlanarTaps<T, C, St::CBW, St::PLANE / (int)sizeof(T), St::XOFF> taps{
            reinterpret_cast<const T*>(st + 2 * St::IMG + St::MSK)};
        // a completed phase means every copy of the stage landed; a thread
        // whose wait ran out writes nothing, so the tiles of a failed launch
        // keep their previous output
        if (ok) {
            out0_quad<TIn, T, C, S, AM, true>(a, taps, X, Y, qx, qy, wp, bp, mk);
        }
        mreg = mnext;
        if (!__syncthreads_and(ok)) {
            // a stage never completed: report it, let the copies of the next
            // stage (if any) land, and stop
            if (MODE == OUT0_CP_ASYNC) {
                cp_async_wait<0>();
            }
            if (threadIdx.x == 0) {
                atomicOr(a.err, 1u);
                if (next) {
                    (void)mbar_wait_bounded(&bar[s ^ 1], (uint32_t)((it + 1) >> 1) & 1u);
                }
            }
            return;
        }
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

static inline double esz_f(int dt) { return dt == ENB_U8 ? 1.0 : ((dt == ENB_U16 || dt == ENB_I16) ? 2.0 : 4.0); }
static inline double npix_f(int w, int h) { return (double)w * (double)h; }
static inline double pbytes(const PlanarView& v) { return npix_f(v.w, v.h) * v.C * esz_f(v.dtype); }

struct Reduce0Launch {
    const PixelView* s[2];
    const uint8_t* ap[2];
    int64_t apitch[2];
    uint32_t lo[2], hi[2];
    const PlanarView* d[2];
    const BytePlane* da[2];
    int n;
    int frac;
    int wrap;
    cudaStream_t st;
    int ty0, nty;
    template <typename TIn, typename T, int C, int S, int AM, bool VEC>
    void operator()() const
    {
        using Src = PixelSourceV<TIn, C, S, AM, VEC>;
        ReduceJobs<Src, T> jobs{};
        for (int i = 0; i < 2; ++i) {
            const int k = i < n ? i : 0;
            jobs.j[i] = ReduceJob<Src, T>{Src{(const TIn*)s[k]->p, s[k]->pitch, ap[k], apitch[k], lo[k], hi[k], frac},
                                          (T*)d[k]->p, d[k]->pitch, d[k]->plane, da[k]->p, da[k]->pitch};
        }
        launch_reduce_jobs<Src, T, C, true>(jobs, n, s[0]->w, s[0]->h, d[0]->w, d[0]->h, wrap, st, ty0, nty);
    }
};

struct Out0Launch {
    const CoarseLevels& cl;
    const Out0Args& a;
    dim3 g;
    cudaStream_t st;
    template <typename TIn, typename T, int C, int S, int AM, bool VEC>
    void operator()() const
    {
        (void)launch_pdl(k_out0<TIn, T, C, S, AM, VEC>, g, dim3(256), st, cl, a);
    }
};

// Calls f.operator()<TIn, T, C, S, AM, VEC>() for the runtime combination
// (the pyramid type follows the sample type: U8 -> Int16, U16 -> Int32).
template <typename F>
static cudaError_t dispatch_pixels(int dtype, int C, int S, int AM, bool vec, F&& f)
{
#define ENB_PX_CASE(TIN, TP, CC, SS, AMM, VV)                      \
    if (C == CC && S == SS && AM == AMM && vec == VV) {            \
        f.template operator()<TIN, TP, CC, SS, AMM, VV>();         \
        return cudaGetLastError();                                 \
    }
#define ENB_PX_TYPE(TIN, TP)                                       \
    ENB_PX_CASE(TIN, TP, 1, 1, 0, false)                           \
    ENB_PX_CASE(TIN, TP, 1, 1, 1, false)                           \
    ENB_PX_CASE(TIN, TP, 3, 3, 0, false)                           \
    ENB_PX_CASE(TIN, TP, 3, 3, 1, false)                           \
    ENB_PX_CASE(TIN, TP, 3, 4, 0, false)                           \
    ENB_PX_CASE(TIN, TP, 3, 4, 1, false)                           \
    ENB_PX_CASE(TIN, TP, 3, 4, 2, false)                           \
    ENB_PX_CASE(TIN, TP, 3, 4, 0, true)                            \
    ENB_PX_CASE(TIN, TP, 3, 4, 1, true)                            \
    ENB_PX_CASE(TIN, TP, 3, 4, 2, true)
    if (dtype == ENB_U8) {
        ENB_PX_TYPE(uint8_t, int16_t)
    } else {
        ENB_PX_TYPE(uint16_t, int32_t)
    }
#undef ENB_PX_TYPE
#undef ENB_PX_CASE
    return cudaErrorInvalidValue;
}

static bool vec_ok(const void* p, int64_t pitch_elems, int dtype, int S)
{
    const size_t bytes = (size_t)S * (dtype == ENB_U8 ? 1 : 2);
    return S == 4 && ((uintptr_t)p % bytes) == 0 && ((size_t)pitch_elems * (dtype == ENB_U8 ? 1 : 2)) % bytes == 0;
}

static int alpha_mode_code(const AlphaSrc& a)
{
    return a.mode == kAlphaPlane ? 0 : (a.mode == kAlphaOpaque ? 1 : 2);
}

static double reduce0_bytes(const PixelView& s, const AlphaSrc& a, const PlanarView& d)
{
    return npix_f(s.w, s.h) * s.stride * esz_f(s.dtype) + (a.mode == kAlphaPlane ? npix_f(s.w, s.h) : 0.0) +
           pbytes(d) + npix_f(d.w, d.h);
}

// Share of a level's tile rows a banded launch covers (for the byte counts).
static double row_share(int dh, int ty0, int nty)
{
    const int total = reduce_tile_rows(dh);
    const int n = nty < 0 ? total - ty0 : nty;
    return total > 0 ? (double)std::max(n, 0) / total : 0.0;
}

int reduce_tile_rows_of(int dh) { return reduce_tile_rows(dh); }

int reduce_tile_rows_ready(int sh, int dh, int rows_ready)
{
    // destination tile row ty reads source rows up to 2 * (16 ty + 15) + 2
    if (rows_ready >= sh) {
        return reduce_tile_rows(dh);
    }
    const int n = rows_ready >= 2 * RDH + 1 ? (rows_ready - (2 * RDH + 1)) / (2 * RDH) + 1 : 0;
    return std::min(n, reduce_tile_rows(dh));
}

static cudaError_t reduce0_launch(int n, const PixelView* const* s, const AlphaSrc* const* a, const PlanarView* const* d,
                                  const BytePlane* const* da, int frac, int wrap, cudaStream_t st, int ty0, int nty)
{
    Reduce0Launch l{};
    double bytes = 0.0;
    bool vec = true;
    for (int i = 0; i < n; ++i) {
        l.s[i] = s[i];
        l.ap[i] = a[i]->mode == kAlphaPlane ? a[i]->plane.p : nullptr;
        l.apitch[i] = a[i]->mode == kAlphaPlane ? a[i]->plane.pitch : 0;
        l.lo[i] = a[i]->lo;
        l.hi[i] = a[i]->hi;
        l.d[i] = d[i];
        l.da[i] = da[i];
        bytes += reduce0_bytes(*s[i], *a[i], *d[i]);
        vec = vec && vec_ok(s[i]->p, s[i]->pitch, s[i]->dtype, s[i]->stride);
    }
    l.n = n;
    l.frac = frac;
    l.wrap = wrap;
    l.st = st;
    l.ty0 = ty0;
    l.nty = nty;
    note_launch("reduce0_alpha", bytes * row_share(d[0]->h, ty0, nty));
    return dispatch_pixels(s[0]->dtype, s[0]->C, s[0]->stride, alpha_mode_code(*a[0]), vec, l);
}

static cudaError_t reduce0_single(const PixelView& s, const AlphaSrc& a, int frac, const PlanarView& d,
                                  const BytePlane& da, int wrap, cudaStream_t st, int ty0, int nty)
{
    const PixelView* sv[1] = {&s};
    const AlphaSrc* av[1] = {&a};
    const PlanarView* dv[1] = {&d};
    const BytePlane* dav[1] = {&da};
    return reduce0_launch(1, sv, av, dv, dav, frac, wrap, st, ty0, nty);
}

cudaError_t launch_reduce0_alpha(const PixelView& s, const AlphaSrc& a, int frac, const PlanarView& d,
                                 const BytePlane& da, int wrap, cudaStream_t st)
{
    return reduce0_single(s, a, frac, d, da, wrap, st, 0, -1);
}

cudaError_t launch_reduce0_alpha2(const PixelView& s0, const AlphaSrc& a0, const PlanarView& d0, const BytePlane& da0,
                                  const PixelView& s1, const AlphaSrc& a1, const PlanarView& d1, const BytePlane& da1,
                                  int frac, int wrap, cudaStream_t st, int ty0, int nty)
{
    const bool same = s0.w == s1.w && s0.h == s1.h && s0.dtype == s1.dtype && s0.C == s1.C &&
                      s0.stride == s1.stride && a0.mode == a1.mode && a0.lo == a1.lo && a0.hi == a1.hi &&
                      d0.w == d1.w && d0.h == d1.h && d0.dtype == d1.dtype && d0.C == d1.C;
    if (!same) {
        const cudaError_t e = reduce0_single(s0, a0, frac, d0, da0, wrap, st, ty0, nty);
        return e != cudaSuccess ? e : reduce0_single(s1, a1, frac, d1, da1, wrap, st, ty0, nty);
    }
    const PixelView* sv[2] = {&s0, &s1};
    const AlphaSrc* av[2] = {&a0, &a1};
    const PlanarView* dv[2] = {&d0, &d1};
    const BytePlane* dav[2] = {&da0, &da1};
    return reduce0_launch(2, sv, av, dv, dav, frac, wrap, st, ty0, nty);
}

template <typename TD>
static void reduce0_bytes_launch(const BytePlane& s, int frac, const PlanarView& d, int wrap, cudaStream_t st, int ty0,
                                 int nty)
{
    ReduceJobs<ByteSource, TD> jobs{};
    jobs.j[0] = ReduceJob<ByteSource, TD>{ByteSource{s.p, s.pitch, frac}, (TD*)d.p, d.pitch, 0, nullptr, 0};
    jobs.j[1] = jobs.j[0];
    launch_reduce_jobs<ByteSource, TD, 1, false>(jobs, 1, s.w, s.h, d.w, d.h, wrap, st, ty0, nty);
}

cudaError_t launch_reduce0_bytes(const BytePlane& s, int frac, const PlanarView& d, int wrap, cudaStream_t st, int ty0,
                                 int nty)
{
    note_launch("reduce0_mask", (npix_f(s.w, s.h) + pbytes(d)) * row_share(d.h, ty0, nty));
    if (d.dtype == ENB_I16) {
        reduce0_bytes_launch<int16_t>(s, frac, d, wrap, st, ty0, nty);
    } else {
        reduce0_bytes_launch<int32_t>(s, frac, d, wrap, st, ty0, nty);
    }
    return cudaGetLastError();
}

cudaError_t launch_blend_into(const PlanarView& m, const PlanarView& gw, const PlanarView& gb, const PlanarView& r,
                              int32_t wv, cudaStream_t st)
{
    note_launch("blend_top", pbytes(m) + pbytes(gw) + pbytes(gb) + pbytes(r));
    const dim3 g((unsigned)((r.w + 255) / 256), (unsigned)r.h);
    const bool m16 = m.dtype == ENB_I16;
#define ENB_BI(T, TM, CC)                                                                                    \
    (void)launch_pdl(k_blend_into<T, TM, CC>, g, dim3(256), st, (const TM*)m.p, m.pitch, (const T*)gw.p,         \
                     (const T*)gb.p, (T*)r.p, r.pitch, r.plane, r.w, r.h, wv)
    if (r.dtype == ENB_I16) {
        if (r.C == 1) {
            if (m16) ENB_BI(int16_t, int16_t, 1); else ENB_BI(int16_t, int32_t, 1);
        } else {
            if (m16) ENB_BI(int16_t, int16_t, 3); else ENB_BI(int16_t, int32_t, 3);
        }
    } else {
        if (r.C == 1) {
            if (m16) ENB_BI(int32_t, int16_t, 1); else ENB_BI(int32_t, int32_t, 1);
        } else {
            if (m16) ENB_BI(int32_t, int16_t, 3); else ENB_BI(int32_t, int32_t, 3);
        }
    }
#undef ENB_BI
    return cudaGetLastError();
}

static CoarseLevels coarse_of(const PlanarView& gw, const PlanarView& gb, const PlanarView& r)
{
    CoarseLevels cl{};
    const size_t es = gw.dtype == ENB_I16 ? 2 : 4;
    for (int c = 0; c < gw.C; ++c) {
        cl.p[c] = (const char*)gw.p + (size_t)c * gw.plane * es;
        cl.p[gw.C + c] = (const char*)gb.p + (size_t)c * gb.plane * es;
        cl.p[2 * gw.C + c] = (const char*)r.p + (size_t)c * r.plane * es;
    }
    cl.pitch = gw.pitch;
    cl.w = gw.w;
    cl.h = gw.h;
    return cl;
}

cudaError_t launch_up_level(const PlanarView& gw1, const PlanarView& gb1, const PlanarView& r1, const PlanarView& m,
                            const PlanarView& gw, const PlanarView& gb, const PlanarView& r, int32_t wv, int wrap,
                            cudaStream_t st)
{
    if (gw1.pitch != gb1.pitch || gw1.pitch != r1.pitch || gw.pitch != gb.pitch || gw.pitch != r.pitch ||
        gw.plane != gb.plane || gw.plane != r.plane) {
        return cudaErrorInvalidValue;
    }
    note_launch("up_level", 3.0 * pbytes(gw1) + pbytes(m) + 3.0 * pbytes(gw));
    const CoarseLevels cl = coarse_of(gw1, gb1, r1);
    const dim3 g = grid2d(r.w, r.h, ETW, ETH);
    const bool m16 = m.dtype == ENB_I16;
#define ENB_UL(T, TM, CC)                                                                                    \
    (void)launch_pdl(k_up_level<T, TM, CC>, g, dim3(256), st, cl, (const TM*)m.p, m.pitch, (const T*)gw.p,       \
                     (const T*)gb.p, (T*)r.p, r.pitch, r.plane, r.w, r.h, wv, wrap)
    if (r.dtype == ENB_I16) {
        if (r.C == 1) {
            if (m16) ENB_UL(int16_t, int16_t, 1); else ENB_UL(int16_t, int32_t, 1);
        } else {
            if (m16) ENB_UL(int16_t, int16_t, 3); else ENB_UL(int16_t, int32_t, 3);
        }
    } else {
        if (r.C == 1) {
            if (m16) ENB_UL(int32_t, int16_t, 1); else ENB_UL(int32_t, int32_t, 1);
        } else {
            if (m16) ENB_UL(int32_t, int16_t, 3); else ENB_UL(int32_t, int32_t, 3);
        }
    }
#undef ENB_UL
    return cudaGetLastError();
}

// ---- TMA tensor maps ---------------------------------------------------------

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled of the driver (through the runtime's entry-point
// query, so that the library needs no link against libcuda); null when the
// driver has none.
static EncodeTiledFn encode_tiled()
{
    static const EncodeTiledFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (EncodeTiledFn) nullptr;
        }
        return (EncodeTiledFn)f;
    }();
    return fn;
}

// A 2-D map of w x h elements with a row pitch in bytes and a bw x bh box;
// false when the layout does not meet the TMA rules (16-byte aligned base
// and pitch, box rows a multiple of 16 bytes).
static bool map2d(CUtensorMap* m, CUtensorMapDataType dt, int esz, const void* base, int64_t w, int64_t h,
                  int64_t pitch_bytes, int bw, int bh)
{
    const EncodeTiledFn fn = encode_tiled();
    if (!fn || ((uintptr_t)base & 15) || (pitch_bytes & 15) || pitch_bytes < w * esz || (bw * esz) % 16 ||
        bw > 256 || bh > 256) {
        return false;
    }
    const cuuint64_t dims[2] = {(cuuint64_t)w, (cuuint64_t)h};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, dt, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static int sm_count()
{
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
}

// The TMA level-0 kernel over the interior rectangle [bx0, bx0 + nbx) x
// [by0, by0 + nby) of tiles; false when this format or layout has no TMA
// path (the caller then runs k_out0 there).
template <typename TIn, typename T, int AM, int MODE>
static bool out0_tma_run(const Out0Maps& maps, const CoarseLevels& cl, const Out0Args& a, const Out0Ring& ring,
                         cudaStream_t st)
{
    using St = Out0Stage<TIn, T, 3, 4, MODE>;
    auto kern = k_out0_tma<TIn, T, 3, 4, AM, MODE>;
    // per call: the attribute belongs to the current device
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * St::BYTES) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    const int grid = std::min(ring.nbx * ring.nby, 3 * sm_count());
    if (launch_pdl_smem(kern, dim3((unsigned)grid), dim3(256), (size_t)(2 * St::BYTES), st, maps, cl, a, ring) !=
        cudaSuccess) {
        cudaGetLastError();  // the caller runs k_out0 instead
        return false;
    }
    return true;
}

// The level-0 kernel with the TMA pipeline over the interior rectangle and
// the ring of the band; false when the coarse planes do not meet the TMA
// rules (the caller then runs k_out0).  Images and mask go through 2-D TMA
// boxes when their rows start on 16-byte boundaries, else through
// per-thread cp.async copies.
template <typename TIn, typename T, int AM>
static bool out0_tma_launch(const CoarseLevels& cl, const Out0Args& a, const Out0Ring& ring, cudaStream_t st)
{
    constexpr int C = 3, S = 4;
    using St0 = Out0Stage<TIn, T, C, S, OUT0_TMA_ROWS>;
    const CUtensorMapDataType dimg = sizeof(TIn) == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_UINT16;
    const CUtensorMapDataType dpl = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_INT32 : CU_TENSOR_MAP_DATA_TYPE_UINT16;
    Out0Maps maps;
    for (int q = 0; q < 3 * C; ++q) {
        if (!map2d(&maps.coarse[q], dpl, sizeof(T), cl.p[q], cl.w, cl.h, cl.pitch * (int64_t)sizeof(T), St0::CBW,
                   ESH)) {
            return false;
        }
    }
    const bool rows = map2d(&maps.white, dimg, sizeof(TIn), a.white, (int64_t)a.w * S, a.h,
                            a.wpitch * (int64_t)sizeof(TIn), ETW * S, ETH) &&
                      map2d(&maps.black, dimg, sizeof(TIn), a.black, (int64_t)a.w * S, a.h,
                            a.bpitch * (int64_t)sizeof(TIn), ETW * S, ETH) &&
                      map2d(&maps.mask, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, a.mask, a.w, a.h, a.mpitch, ETW, ETH);
    return rows ? out0_tma_run<TIn, T, AM, OUT0_TMA_ROWS>(maps, cl, a, ring, st)
                : out0_tma_run<TIn, T, AM, OUT0_CP_ASYNC>(maps, cl, a, ring, st);
}

cudaError_t launch_out0(const PlanarView* gw1, const PlanarView* gb1, const PlanarView* r1, const Out0Host& h,
                        cudaStream_t st, int ty0, int nty)
{
    const PixelView& wv = h.white;
    Out0Args a{};
    a.white = wv.p;
    a.black = h.black.p;
    a.wpitch = wv.pitch;
    a.bpitch = h.black.pitch;
    a.wa = h.white_alpha.mode == kAlphaPlane ? h.white_alpha.plane.p : nullptr;
    a.ba = h.black_alpha.mode == kAlphaPlane ? h.black_alpha.plane.p : nullptr;
    a.wapitch = h.white_alpha.mode == kAlphaPlane ? h.white_alpha.plane.pitch : 0;
    a.bapitch = h.black_alpha.mode == kAlphaPlane ? h.black_alpha.plane.pitch : 0;
    a.alo = h.white_alpha.lo;
    a.ahi = h.white_alpha.hi;
    a.mask = h.mask.p;
    a.mpitch = h.mask.pitch;
    a.mfrac = h.mfrac;
    a.white_value = h.white_value;
    a.out = h.out;
    a.opitch = h.opitch;
    a.out_alpha = h.out_alpha.p;
    a.oapitch = h.out_alpha.pitch;
    a.level0 = h.level0;
    a.w = wv.w;
    a.h = wv.h;
    a.frac = h.frac;
    a.dither = h.dither;
    a.has_coarse = gw1 != nullptr;
    a.wrap = h.wrap;
    a.seed = h.seed;
    a.key = dither_key(h.seed);
    a.maxv = wv.dtype == ENB_U8 ? 255 : 65535;
    a.err = h.err;
    a.tx_extra = h.tx_extra;
    // k_out0 compiles these formats in
    const int mf_expect = wv.dtype == ENB_U8 ? 7 : 15;
    if (a.frac != 7 || a.mfrac != mf_expect || a.white_value != (255 << mf_expect) || wv.C > 4) {
        return cudaErrorInvalidValue;
    }
    CoarseLevels cl{};
    if (gw1) {
        cl = coarse_of(*gw1, *gb1, *r1);
    }
    const double px = npix_f(wv.w, wv.h);
    const int rows = (wv.h + ETH - 1) / ETH, cols = (wv.w + ETW - 1) / ETW;
    {
        const double share = (double)(nty < 0 ? rows - ty0 : nty) / rows;
        note_launch("out0", share * (px * (3.0 * wv.stride * esz_f(wv.dtype) + 1.0 + (h.out_alpha.p ? 1.0 : 0.0)) +
                                     (gw1 ? 3.0 * pbytes(*gw1) : 0.0)));
    }
    const bool vec = vec_ok(wv.p, wv.pitch, wv.dtype, wv.stride) &&
                     vec_ok(h.black.p, h.black.pitch, wv.dtype, wv.stride) && vec_ok(h.out, h.opitch, wv.dtype, wv.stride);
    const int am = alpha_mode_code(h.white_alpha);
    if (nty < 0) {
        nty = rows - ty0;
    }
    if (nty <= 0) {
        return cudaSuccess;
    }
    // k_out0 over the rectangle [tx0, tx0 + ncol) x [ry0, ry0 + nrow) of tiles
    const auto legacy = [&](int tx0, int ncol, int ry0, int nrow) -> cudaError_t {
        Out0Args b = a;
        b.tx0 = tx0;
        b.ty0 = ry0;
        Out0Launch l{cl, b, dim3((unsigned)ncol, (unsigned)nrow), st};
        return dispatch_pixels(wv.dtype, wv.C, wv.stride, am, vec, l);
    };
    // interior tiles (interior_tile): columns 1 .. bx1, rows 1 .. by1
    const int bx1 = gw1 ? std::min((wv.w - ETW) / ETW, (cl.w - ESW + 1) / (ETW / 2)) : 0;
    const int by1 = gw1 ? std::min((wv.h - ETH) / ETH, (cl.h - ESH + 1) / (ETH / 2)) : 0;
    const int iy0 = std::max(ty0, 1), iy1 = std::min(ty0 + nty - 1, by1);
    bool tma = false;
    if (bx1 >= 1 && iy1 >= iy0 && vec && wv.C == 3 && wv.stride == 4 && h.err &&
        (wv.dtype == ENB_U16 || wv.dtype == ENB_U8)) {
        const Out0Ring ring{1, bx1, iy0, iy1 - iy0 + 1, ty0, nty, cols};
        if (wv.dtype == ENB_U16) {
            tma = am == 0   ? out0_tma_launch<uint16_t, int32_t, 0>(cl, a, ring, st)
                  : am == 1 ? out0_tma_launch<uint16_t, int32_t, 1>(cl, a, ring, st)
                            : out0_tma_launch<uint16_t, int32_t, 2>(cl, a, ring, st);
        } else {
            tma = am == 0   ? out0_tma_launch<uint8_t, int16_t, 0>(cl, a, ring, st)
                  : am == 1 ? out0_tma_launch<uint8_t, int16_t, 1>(cl, a, ring, st)
                            : out0_tma_launch<uint8_t, int16_t, 2>(cl, a, ring, st);
        }
    }
    if (tma) {
        last_launch().name = "out0_tma";
        return cudaSuccess;
    }
    return legacy(0, cols, ty0, nty);
}

}  // namespace enb
