// enb_tiles.cuh -- tile machinery shared by the per-level kernels and the
// coarse-level cluster kernel of the enblend blend: staging of the coarse
// neighbourhood of a 64x16 destination tile, the expansion (src/pyramid.h
// SKIPSM expand, 1227-1411) of its quads, and the per-tile Laplacian + blend
// + collapse step.  NC selects the read-only load path (data no thread of the
// launch writes) or plain loads (levels written earlier in the same launch);
// NT is the CTA's thread count.
#pragma once

#include "enb_device.cuh"

namespace enb {

// CartesianBlendFunctor of one sample (src/blend.h:41-76).
template <typename T>
__device__ __forceinline__ int32_t blend1(int32_t m, int32_t white_value, int32_t lw, int32_t lb)
{
    return blend_sample<T>(m, white_value, lw, lb);
}


// ---------------------------------------------------------------------------
// Tiled expansion of coarse planes
// ---------------------------------------------------------------------------

struct CoarseLevels {
    // plane pointers of Gw_{l+1}, Gb_{l+1}, R_{l+1}, channel-major: [which*C + c]
    const void* p[9];
    int64_t pitch;  // elements
    int w, h;
};

// Stage the 34x10 coarse neighbourhoods of a 64x16 destination tile for NP
// planes; loads unrolled and independent of each other.
template <int NP, typename T, bool NC, int NT>
__device__ __forceinline__ void stage_coarse(int32_t (*ss)[ESH][ESW], const CoarseLevels& cl, int I0, int J0,
                                             int wrap)
{
    constexpr int N = ESH * ESW;
    constexpr int IT = (N + NT - 1) / NT;
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const int k = threadIdx.x + it * NT;
        if (k < N) {
            const int r = k / ESW, c = k - r * ESW;
            const int j = J0 - 1 + r;
            int i = I0 - 1 + c;
            if (wrap) {
                i = imod(i, cl.w);
            }
            const bool in = j >= 0 && j < cl.h && i >= 0 && i < cl.w;
            // clamped position: the loads are unconditional, the taps outside
            // the level are zeroed afterwards
            const int64_t o = (int64_t)min(max(j, 0), cl.h - 1) * cl.pitch + min(max(i, 0), cl.w - 1);
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const int32_t v = (int32_t)ld_src<NC>(&reinterpret_cast<const T*>(cl.p[p])[o]);
                ss[p][r][c] = in ? v : 0;
            }
        }
    }
}

// Expansion of the four destination pixels of the quad at tile position
// (qx, qy) from one staged coarse plane (the 3x3 source neighbourhood), with
// the border weights and divisors of expand_hweights / expand_vweights.
__device__ __forceinline__ void expand_quad(const int32_t (*s)[ESW], int qx, int qy, int X, int Y, int sw, int sh,
                                            int dw, int dh, int wrap, int32_t e[4])
{
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int XX = X + (q & 1), YY = Y + (q >> 1);
        e[q] = 0;
        if (XX >= dw || YY >= dh) {
            continue;
        }
        int vw[3], vden, hw[3], hden;
        expand_vweights(YY, sh, vw, vden);
        expand_hweights(XX, sw, dw, wrap, hw, hden);
        int32_t num = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int32_t* row = &s[qy + a][qx];
            num += vw[a] * (hw[0] * row[0] + hw[1] * row[1] + hw[2] * row[2]);
        }
        e[q] = div_den(num, hden * vden);
    }
}

// Staging of an interior tile with the three planes of a channel packed into
// one int4 per tap ({Gw, Gb, R, 0}): a quad's nine taps of all three planes
// are then nine 16-byte shared loads (a warp's loads are 512 contiguous
// bytes, four wavefronts, no bank conflicts).
template <int C, typename T, bool NC, int NT>
__device__ __forceinline__ void stage_coarse4_interior(int4 (*s4)[ESH][ESW], const CoarseLevels& cl, int I0, int J0)
{
    constexpr int N = ESH * ESW;
    constexpr int IT = (N + NT - 1) / NT;
    const T* base[3 * C];
#pragma unroll
    for (int p = 0; p < 3 * C; ++p) {
        base[p] = reinterpret_cast<const T*>(cl.p[p]) + (int64_t)(J0 - 1) * cl.pitch + (I0 - 1);
    }
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const int k = threadIdx.x + it * NT;
        if (k < N) {
            const int r = k / ESW, c = k - r * ESW;
            const int o = r * (int)cl.pitch + c;
#pragma unroll
            for (int ch = 0; ch < C; ++ch) {
                s4[ch][r][c] = make_int4((int32_t)ld_src<NC>(&base[ch][o]), (int32_t)ld_src<NC>(&base[C + ch][o]),
                                         (int32_t)ld_src<NC>(&base[2 * C + ch][o]), 0);
            }
        }
    }
}

// Expansion of an interior quad (all taps inside the level) from its 3x3
// source neighbourhood v.  The (4,4) taps enter without their common factor
// 4, which is folded into the divisors: trunc(4n/64) = trunc(n/16) and
// trunc(4n/16) = trunc(n/4).  NONNEG: the source is a Gaussian level of an
// unsigned image (all values >= 0), so the truncating divisions are shifts.
template <bool NONNEG>
__device__ __forceinline__ void expand9(const int32_t (&v)[3][3], int32_t e[4])
{
    const int32_t hea = v[0][0] + 6 * v[0][1] + v[0][2], heb = v[1][0] + 6 * v[1][1] + v[1][2],
                  hec = v[2][0] + 6 * v[2][1] + v[2][2];
    const int32_t hoa = v[0][1] + v[0][2], hob = v[1][1] + v[1][2], hoc = v[2][1] + v[2][2];
    const int32_t n0 = hea + 6 * heb + hec, n1 = hoa + 6 * hob + hoc, n2 = heb + hec, n3 = hob + hoc;
    if (NONNEG) {
        e[0] = (int32_t)((uint32_t)n0 >> 6);
        e[1] = (int32_t)((uint32_t)n1 >> 4);
        e[2] = (int32_t)((uint32_t)n2 >> 4);
        e[3] = (int32_t)((uint32_t)n3 >> 2);
    } else {
        e[0] = n0 / 64;
        e[1] = n1 / 16;
        e[2] = n2 / 16;
        e[3] = n3 / 4;
    }
}

// One 16-byte shared load (all four words, so that it stays one access).
__device__ __forceinline__ int4 lds128(const int4* p)
{
    int4 v;
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ld.shared.v4.s32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "r"(a)
                 : "memory");
    return v;
}

// Expansions of one channel's planes at an interior quad from the packed
// taps: er always, ew / eb where the quad's seam mask needs them
// (kind 1: all white, 2: all black, 0: mixed).
__device__ __forceinline__ void expand_packed(const int4 (*s)[ESW], int qx, int qy, int kind, int32_t ew[4],
                                              int32_t eb[4], int32_t er[4])
{
    int4 t[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            t[a][b] = lds128(&s[qy + a][qx + b]);
        }
    }
    int32_t v[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            v[a][b] = t[a][b].z;
        }
    }
    expand9<false>(v, er);
    if (kind != 2) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                v[a][b] = t[a][b].x;
            }
        }
        expand9<true>(v, ew);
    }
    if (kind != 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                v[a][b] = t[a][b].y;
            }
        }
        expand9<true>(v, eb);
    }
}

// Collapsed value of one sample: fromPromote(blend(m, Lw, Lb) + E(R)), with
// the blend resolved without the mask test when the whole quad is white (1)
// or black (2).
template <typename T>
__device__ __forceinline__ int32_t merge_sample(int kind, int32_t m, int32_t W, int32_t fw, int32_t ew, int32_t fb,
                                                int32_t eb, int32_t er)
{
    if (kind == 1) {
        return (int32_t)sat_store<T>((int32_t)cast_store<T>((int64_t)fw - ew) + er);
    }
    if (kind == 2) {
        return (int32_t)sat_store<T>((int32_t)cast_store<T>((int64_t)fb - eb) + er);
    }
    const int32_t lw = (int32_t)cast_store<T>((int64_t)fw - ew);
    const int32_t lb = (int32_t)cast_store<T>((int64_t)fb - eb);
    return (int32_t)sat_store<T>(blend_sample<T>(m, W, lw, lb) + er);
}

__device__ __forceinline__ int quad_kind(const int32_t (&m)[4], int32_t W)
{
    if (m[0] >= W && m[1] >= W && m[2] >= W && m[3] >= W) {
        return 1;
    }
    if (m[0] <= 0 && m[1] <= 0 && m[2] <= 0 && m[3] <= 0) {
        return 2;
    }
    return 0;
}

// Two horizontally adjacent samples of a planar level (even x: 4- or 8-byte aligned).
template <typename T, bool NC>
__device__ __forceinline__ void ld2(const T* p, int32_t& a, int32_t& b)
{
    if (sizeof(T) == 4) {
        const int2 v = ld_src<NC>(reinterpret_cast<const int2*>(p));
        a = v.x;
        b = v.y;
    } else {
        const int v = ld_src<NC>(reinterpret_cast<const int*>(p));
        a = (int32_t)(int16_t)(v & 0xffff);
        b = v >> 16;
    }
}

template <typename T>
__device__ __forceinline__ void st2(T* p, T a, T b)
{
    if (sizeof(T) == 4) {
        *reinterpret_cast<int2*>(p) = make_int2((int32_t)a, (int32_t)b);
    } else {
        *reinterpret_cast<int*>(p) = (int)(((uint32_t)(uint16_t)a) | ((uint32_t)(uint16_t)b << 16));
    }
}

// CTA-uniform test: the 64x16 destination tile lies inside the level and
// every quad's 3x3 coarse neighbourhood lies inside the coarse level.
__device__ __forceinline__ bool interior_tile(int X0, int Y0, int w, int h, int I0, int J0, int cw, int ch)
{
    return X0 + ETW <= w && Y0 + ETH <= h && I0 >= 1 && I0 + ETW / 2 < cw && J0 >= 1 && J0 + ETH / 2 < ch;
}

// ---------------------------------------------------------------------------
// One 64x16 tile of a coarse level l: Laplacians, blend, collapse
// ---------------------------------------------------------------------------

// R_l = fromPromote(blend(M_l, Gw_l - E(Gw_{l+1}), Gb_l - E(Gb_{l+1})) + E(R_{l+1}))
// on the tile at (X0, Y0), quads on threads 0..255 (threads NT > 256 only
// take part in the staging and the barrier).  sbuf: C*ESH*ESW int4.
template <typename T, typename TM, int C, bool NC, int NT>
__device__ __forceinline__ void up_tile(const CoarseLevels& cl, const TM* __restrict__ mask, int64_t mpitch,
                                        const T* __restrict__ gw, const T* __restrict__ gb, T* __restrict__ r,
                                        int64_t pitch, int64_t plane, int w, int h, int32_t white_value, int wrap,
                                        int X0, int Y0, int4 (*sbuf)[ESH][ESW])
{
    static_assert(NT >= 256, "one thread per quad of the 64x16 tile");
    int32_t (*ss)[ESH][ESW] = reinterpret_cast<int32_t (*)[ESH][ESW]>(&sbuf[0][0][0]);
    const int I0 = X0 >> 1, J0 = Y0 >> 1;
    const bool active = threadIdx.x < 256;
    const int qx = threadIdx.x % 32, qy = (threadIdx.x / 32) & 7;
    const int i = I0 + qx, j = J0 + qy;
    const int X = 2 * i, Y = 2 * j;

    if (interior_tile(X0, Y0, w, h, I0, J0, cl.w, cl.h)) {
        // interior tile: no bounds, paired loads and stores, packed taps,
        // only the expansions the quad's mask values select
        const int64_t o0 = (int64_t)Y * pitch + X;
        int32_t fw[C][4], fb[C][4], fm[4];
        if (active) {
            ld2<TM, NC>(mask + (int64_t)Y * mpitch + X, fm[0], fm[1]);
            ld2<TM, NC>(mask + (int64_t)(Y + 1) * mpitch + X, fm[2], fm[3]);
#pragma unroll
            for (int c = 0; c < C; ++c) {
                ld2<T, NC>(gw + c * plane + o0, fw[c][0], fw[c][1]);
                ld2<T, NC>(gw + c * plane + o0 + pitch, fw[c][2], fw[c][3]);
                ld2<T, NC>(gb + c * plane + o0, fb[c][0], fb[c][1]);
                ld2<T, NC>(gb + c * plane + o0 + pitch, fb[c][2], fb[c][3]);
            }
        }
        stage_coarse4_interior<C, T, NC, NT>(sbuf, cl, I0, J0);
        __syncthreads();
        if (active) {
            const int kind = quad_kind(fm, white_value);
#pragma unroll
            for (int c = 0; c < C; ++c) {
                int32_t ew[4], eb[4], er[4];
                expand_packed(sbuf[c], qx, qy, kind, ew, eb, er);
                T res[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    res[q] = (T)merge_sample<T>(kind, fm[q], white_value, fw[c][q], ew[q], fb[c][q], eb[q], er[q]);
                }
                st2<T>(r + c * plane + o0, res[0], res[1]);
                st2<T>(r + c * plane + o0 + pitch, res[2], res[3]);
            }
        }
        return;
    }

    // border tile: fine-level values of the quad, loaded (from clamped
    // positions, unconditionally) before the barrier
    int32_t fw[C][4], fb[C][4], fm[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int XX = min(X + (q & 1), w - 1), YY = min(Y + (q >> 1), h - 1);
        const int64_t o = (int64_t)YY * pitch + XX;
        fm[q] = (int32_t)ld_src<NC>(&mask[(int64_t)YY * mpitch + XX]);
#pragma unroll
        for (int c = 0; c < C; ++c) {
            fw[c][q] = (int32_t)ld_src<NC>(&gw[c * plane + o]);
            fb[c][q] = (int32_t)ld_src<NC>(&gb[c * plane + o]);
        }
    }
    stage_coarse<3 * C, T, NC, NT>(ss, cl, I0, J0, wrap);
    __syncthreads();
    if (!active || X >= w || Y >= h) {
        return;
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
        int32_t ew[4], eb[4], er[4];
        expand_quad(ss[c], qx, qy, X, Y, cl.w, cl.h, w, h, wrap, ew);
        expand_quad(ss[C + c], qx, qy, X, Y, cl.w, cl.h, w, h, wrap, eb);
        expand_quad(ss[2 * C + c], qx, qy, X, Y, cl.w, cl.h, w, h, wrap, er);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int XX = X + (q & 1), YY = Y + (q >> 1);
            if (XX >= w || YY >= h) {
                continue;
            }
            const int32_t lw = (int32_t)cast_store<T>((int64_t)fw[c][q] - ew[q]);
            const int32_t lb = (int32_t)cast_store<T>((int64_t)fb[c][q] - eb[q]);
            const int32_t bl = blend1<T>(fm[q], white_value, lw, lb);
            r[c * plane + (int64_t)YY * pitch + XX] = sat_store<T>(bl + er[q]);
        }
    }
}

}  // namespace enb
