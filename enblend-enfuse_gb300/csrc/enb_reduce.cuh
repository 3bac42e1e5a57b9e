// enb_reduce.cuh -- the Burt-Adelson reduce (src/pyramid.h:166-848) as one
// tiled kernel over pluggable sources.
//
// One CTA of 256 threads computes a 32x16 tile of destination pixels from the
// 67x35 source window around it (2 pixels of halo).  All global loads of the
// window are issued up front (unrolled, independent of the alpha test) so
// that each thread keeps ~10 loads in flight.  Tiles whose window lies inside
// the image (almost all) take a path without bounds, clamp or wrap logic.  The
// window is then filtered with the separable [1 4 6 4 1] kernel in shared
// memory, first along x at the even source columns (consecutive threads take
// consecutive rows, so the odd 67-word row stride spreads them over all
// banks), then along y.  Integer sums are exact, so the order of the taps does
// not matter.
//   with alpha: normalised convolution over the opaque taps, taps outside the
//               image dropped, x periodic when wrap (pyramid.h:166-573);
//   no alpha:   clamp-to-edge replication in y (and x unless wrap), /256
//               (pyramid.h:601-848).
#pragma once

#include "enb_device.cuh"

namespace enb {

constexpr int R2W = 32, R2H = 16;                      // destination tile
constexpr int R2IW = 2 * R2W + 3, R2IH = 2 * R2H + 3;  // 67 x 35 source window
constexpr int R2N = R2IW * R2IH;
constexpr int R2ITER = (R2N + 255) / 256;
constexpr int R2HP = R2W + 1;                          // padded row of the x-filtered window

// Planar pyramid level (+ optional 8-bit alpha plane).
template <typename TS, int C>
struct PlanarSource {
    const TS* p;
    int64_t pitch, plane;   // elements
    const uint8_t* a;
    int64_t apitch;
    __device__ __forceinline__ void load(int gy, int gx, int32_t (&v)[C], int& al) const
    {
        const int64_t o = (int64_t)gy * pitch + gx;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            v[c] = (int32_t)p[c * plane + o];
        }
        al = a ? (a[(int64_t)gy * apitch + gx] != 0) : 1;
    }
};

// 8-bit seam mask converted to fixed point on the fly.
struct ByteSource {
    const uint8_t* p;
    int64_t pitch;
    int frac;
    __device__ __forceinline__ void load(int gy, int gx, int32_t (&v)[1], int& al) const
    {
        v[0] = (int32_t)p[(int64_t)gy * pitch + gx] << frac;
        al = 1;
    }
};

template <class Src, int C, bool ALPHA>
__device__ __forceinline__ void reduce_stage(const Src& src, int gy, int gx, int r, int c, int32_t (*sv)[R2IH][R2IW],
                                             uint8_t (*sa)[R2IW + 1])
{
    int32_t v[C];
    int al = 1;
    src.load(gy, gx, v, al);
#pragma unroll
    for (int ch = 0; ch < C; ++ch) {
        sv[ch][r][c] = (ALPHA && !al) ? 0 : v[ch];
    }
    if (ALPHA) {
        sa[r][c] = (uint8_t)al;
    }
}

template <class Src, typename TD, int C, bool ALPHA>
__global__ void __launch_bounds__(256) k_reduce_tiles(Src src, int sw, int sh, TD* __restrict__ dst, int64_t dpitch,
                                                      int64_t dplane, int dw, int dh, uint8_t* __restrict__ da,
                                                      int64_t dapitch, int wrap)
{
    __shared__ int32_t sv[C][R2IH][R2IW];
    __shared__ uint8_t sa[ALPHA ? R2IH : 1][R2IW + 1];
    __shared__ int32_t hv[C][R2IH][R2HP];
    __shared__ uint8_t ha[ALPHA ? R2IH : 1][R2HP];

    const int X0 = blockIdx.x * R2W, Y0 = blockIdx.y * R2H;
    const int gx0 = 2 * X0 - 2, gy0 = 2 * Y0 - 2;
    const int tid = threadIdx.x;

    if (gx0 >= 0 && gy0 >= 0 && gx0 + R2IW <= sw && gy0 + R2IH <= sh) {
        // interior window: thread -> column tid%64 (+64 for the last 3), rows tid/64 + 4k
        const int c = tid & 63, rg = tid >> 6;
#pragma unroll
        for (int k = 0; k < (R2IH + 3) / 4; ++k) {
            const int r = rg + 4 * k;
            if (r < R2IH) {
                reduce_stage<Src, C, ALPHA>(src, gy0 + r, gx0 + c, r, c, sv, sa);
                if (c < R2IW - 64) {
                    reduce_stage<Src, C, ALPHA>(src, gy0 + r, gx0 + 64 + c, r, 64 + c, sv, sa);
                }
            }
        }
    } else {
#pragma unroll
        for (int it = 0; it < R2ITER; ++it) {
            const int i = tid + it * 256;
            if (i < R2N) {
                const int r = i / R2IW, c = i - r * R2IW;
                int gy = gy0 + r, gx = gx0 + c;
                if (ALPHA) {
                    if (wrap) {
                        gx = imod(gx, sw);
                    }
                    if (gy >= 0 && gy < sh && gx >= 0 && gx < sw) {
                        reduce_stage<Src, C, ALPHA>(src, gy, gx, r, c, sv, sa);
                    } else {
#pragma unroll
                        for (int ch = 0; ch < C; ++ch) {
                            sv[ch][r][c] = 0;
                        }
                        sa[r][c] = 0;
                    }
                } else {
                    gy = min(max(gy, 0), sh - 1);
                    gx = wrap ? imod(gx, sw) : min(max(gx, 0), sw - 1);
                    reduce_stage<Src, C, ALPHA>(src, gy, gx, r, c, sv, sa);
                }
            }
        }
    }
    __syncthreads();

    // x pass at the even source columns; consecutive threads take consecutive rows
    for (int i = tid; i < R2IH * R2W; i += 256) {
        const int j = i / R2IH, r = i - j * R2IH;
        const int c0 = 2 * j;
        if (ALPHA) {
            ha[r][j] = (uint8_t)(sa[r][c0] + 4 * sa[r][c0 + 1] + 6 * sa[r][c0 + 2] + 4 * sa[r][c0 + 3] + sa[r][c0 + 4]);
        }
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            const int32_t* s = &sv[ch][r][c0];
            hv[ch][r][j] = s[0] + 4 * s[1] + 6 * s[2] + 4 * s[3] + s[4];
        }
    }
    __syncthreads();

    // y pass: two destination rows per thread
    const int tx = tid % R2W;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const int ty = tid / R2W + 8 * half;
        const int X = X0 + tx, Y = Y0 + ty;
        if (X >= dw || Y >= dh) {
            continue;
        }
        const int r0 = 2 * ty;
        const int64_t o = (int64_t)Y * dpitch + X;
        if (ALPHA) {
            const int den = ha[r0][tx] + 4 * ha[r0 + 1][tx] + 6 * ha[r0 + 2][tx] + 4 * ha[r0 + 3][tx] + ha[r0 + 4][tx];
            if (den > 0) {
#pragma unroll
                for (int ch = 0; ch < C; ++ch) {
                    const int32_t num = hv[ch][r0][tx] + 4 * hv[ch][r0 + 1][tx] + 6 * hv[ch][r0 + 2][tx] +
                                        4 * hv[ch][r0 + 3][tx] + hv[ch][r0 + 4][tx];
                    dst[ch * dplane + o] = cast_store<TD>(den == 256 ? num / 256 : div_any(num, den));
                }
                da[(int64_t)Y * dapitch + X] = 255;
            } else {
#pragma unroll
                for (int ch = 0; ch < C; ++ch) {
                    dst[ch * dplane + o] = (TD)0;
                }
                da[(int64_t)Y * dapitch + X] = 0;
            }
        } else {
#pragma unroll
            for (int ch = 0; ch < C; ++ch) {
                const int32_t num = hv[ch][r0][tx] + 4 * hv[ch][r0 + 1][tx] + 6 * hv[ch][r0 + 2][tx] +
                                    4 * hv[ch][r0 + 3][tx] + hv[ch][r0 + 4][tx];
                dst[ch * dplane + o] = cast_store<TD>(num / 256);
            }
        }
    }
}

template <class Src, typename TD, int C, bool ALPHA>
inline void launch_reduce_tiles(const Src& src, int sw, int sh, TD* dst, int64_t dpitch, int64_t dplane, int dw,
                                int dh, uint8_t* da, int64_t dapitch, int wrap, cudaStream_t st)
{
    const dim3 g((unsigned)((dw + R2W - 1) / R2W), (unsigned)((dh + R2H - 1) / R2H));
    k_reduce_tiles<Src, TD, C, ALPHA><<<g, 256, 0, st>>>(src, sw, sh, dst, dpitch, dplane, dw, dh, da, dapitch, wrap);
}

}  // namespace enb
