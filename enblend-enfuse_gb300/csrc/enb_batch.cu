// enb_batch.cu -- batched fuse of many float exposure stacks of uneven sizes.
//
// Every stack is enfuseMain's float path (src/enfuse.h:1217-1617 on float
// images, FP32 pyramids for the reference's double ones): weights and their
// normalisation, per exposure a Laplacian image pyramid and an Int32 9.15
// mask pyramid with the union alpha, the masked merge, the collapse and the
// conversion back.  The whole batch runs as one short sequence of launches,
// each covering every stack and exposure at one pyramid level:
//
//   weights   one CTA per 16x16 tile of a stack: the K weights of each pixel
//             (enb_fweights.cuh), their sum, the soft (or hard) masks as
//             level 0 of the mask pyramids, the union alpha, and level 0 of
//             the image pyramids;
//   down l    one CTA per 64x16 destination tile of level l+1 of one
//             exposure's image or mask pyramid (reduce with alpha); level 0
//             of each image pyramid (the log mapping) is written by the
//             weights kernel, which reads the input anyway;
//   coarse    a persistent kernel walking a device work queue of (stack,
//             level, tile) items: every reduce tile of the levels below
//             ~64x64 of every stack and exposure, then every up tile, each
//             item waiting (bounded) for the step before it in its stack;
//   up l      one CTA per 64x16 tile of level l of a stack: the collapsed
//             result C[l] = sum_k (G_k[l] - E(G_k[l+1])) m_k[l] / D + E(C[l+1])
//             (the Laplacian, the mask multiply, the accumulation and the
//             collapse of the reference fused); at level 0 the output pixels
//             are written instead (v >= 1 ? expm1(v - 1) : 1 - 1/v).
//
// Jobs are (stack, kind, tile) entries of host-built tables; a launch's
// grid is its job count.  The host side (the C ABI in enb_api.cu) captures
// the launch sequence into a CUDA graph per batch geometry.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "enb_device.cuh"
#include "enb_fpair.cuh"
#include "enb_fweights.cuh"
#include "enb_internal.h"
#include "enb_reduce.cuh"

namespace enb {

// Per-stack geometry and buffers (device table, one entry per stack).
struct BatchStack {
    int K, w, h, L, Lc;  // exposures, size, levels, first level of the coarse kernel
    int istride[kBatchMaxK];
    const float* img[kBatchMaxK];
    int64_t ipitch[kBatchMaxK];  // floats
    const uint8_t* alpha[kBatchMaxK];
    int64_t apitch[kBatchMaxK];
    float* out;
    int64_t opitch;  // floats
    int ostride;
    uint8_t* oalpha;  // optional
    int64_t oapitch;
    // workspace: levels 0..L-1 at off0 (masks, union alpha), levels 1..L-1
    // at off1 (image levels, image alphas, collapsed result); pitches in
    // elements, planes of pitch * height
    int32_t* m;   // K * s0
    uint8_t* u;   // s0
    float* g;     // K * 3 * s1 (C planes used)
    uint8_t* a;   // K * s1
    float* r;     // 3 * s1
    float* g0;    // K * 3 * s0 (level 0 of the image pyramids, written by the weights kernel)
    int64_t s0, s1;
    int64_t off0[kMaxLevels], off1[kMaxLevels];
    int pitch[kMaxLevels], lw[kMaxLevels], lh[kMaxLevels];
};

namespace {

__device__ __forceinline__ float* g_level(const BatchStack& s, int k, int l, int C)
{
    return s.g + (int64_t)k * C * s.s1 + (int64_t)C * s.off1[l];
}
__device__ __forceinline__ uint8_t* a_level(const BatchStack& s, int k, int l)
{
    return s.a + (int64_t)k * s.s1 + s.off1[l];
}
__device__ __forceinline__ int32_t* m_level(const BatchStack& s, int k, int l)
{
    return s.m + (int64_t)k * s.s0 + s.off0[l];
}
__device__ __forceinline__ float* r_level(const BatchStack& s, int l, int C)
{
    return s.r + (int64_t)C * s.off1[l];
}
// Level 0 of exposure k's image pyramid (planes of pitch[0] * h).
__device__ __forceinline__ float* g0_level(const BatchStack& s, int k, int C)
{
    return s.g0 + (int64_t)k * C * s.s0;
}

// Level 0 of an exposure's image pyramid (planar floats) with the input's
// alpha plane, or opaque when there is none.
template <int C>
struct Level0Source {
    const float* p;
    int64_t pitch, plane;
    const uint8_t* a;  // nullptr: opaque
    int64_t apitch;
    template <typename AC>
    __device__ __forceinline__ void load(int gy, int gx, AC (&v)[C], int& al) const
    {
        const int64_t o = (int64_t)gy * pitch + gx;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            v[c] = __ldg(&p[c * plane + o]);
        }
        al = a ? (__ldg(&a[(int64_t)gy * apitch + gx]) != 0) : 1;
    }
};

}  // namespace

// ---------------------------------------------------------------------------
// weights, normalisation, mask level 0, union alpha
// ---------------------------------------------------------------------------

constexpr int BWT = 16;

// Normalisation of the K weights wk[k * ws] of output pixel (x, y) of stack
// s (src/enfuse.h:1382-1385 sum in exposure order, :1399-1442 hard mask,
// :1526-1535 soft mask) into level 0 of the mask pyramids, and the union
// alpha ua.
__device__ __forceinline__ void batch_normalise(const BatchStack& s, const float* wk, int ws, int x, int y, int hard,
                                                uint8_t ua)
{
    const int K = s.K;
    const int64_t o = (int64_t)y * s.pitch[0] + x;
    if (hard) {
        float mx = 0.0f;
        int mi = 0;
        for (int k = 0; k < K; ++k) {
            if (wk[k * ws] > mx) {
                mx = wk[k * ws];
                mi = k;
            }
        }
        const float fallback = __fdiv_rn(255.0f, (float)K);
        for (int k = 0; k < K; ++k) {
            const float m = mx == 0.0f ? fallback : (k == mi ? 255.0f : 0.0f);
            m_level(s, k, 0)[o] = mask_to_fixed<int32_t>(m, 15);
        }
    } else {
        float norm = 0.0f;
        for (int k = 0; k < K; ++k) {
            norm = __fadd_rn(wk[k * ws], norm);
        }
        const float fallback = (float)(255 / K);
        for (int k = 0; k < K; ++k) {
            const float m = norm > 0.0f ? __fdiv_rn(__fmul_rn(255.0f, wk[k * ws]), norm) : fallback;
            m_level(s, k, 0)[o] = mask_to_fixed<int32_t>(m, 15);
        }
    }
    const uint8_t uv = ua ? 255 : 0;
    s.u[s.off0[0] + o] = uv;
    if (s.oalpha) {
        s.oalpha[(int64_t)y * s.oapitch + x] = uv;
    }
}

// Weights of window sizes that the pair kernel does not take: one output
// pixel per thread on 16x16 tiles (enb_fweights.cuh).
template <int CW, int EW>
__global__ void __launch_bounds__(256, 4) k_batch_weights(const BatchStack* __restrict__ stacks,
                                                       const int4* __restrict__ jobs, FloatWeightParams wp,
                                                       WeightTables tab, int hard, int C)
{
    extern __shared__ __align__(16) unsigned char bsmem[];
    const int4 job = jobs[blockIdx.x];
    const BatchStack& s = stacks[job.x];
    const int halo = fweight_halo(wp);
    const FTile t = ftile_carve(bsmem, BWT + 2 * halo, wp.repeat_slots, wp.ent_cut);
    float* wk = reinterpret_cast<float*>(bsmem + align16(ftile_bytes(t.TW, t.slots, wp.ent_cut))) + threadIdx.x;  // [K][BWT * BWT]
    const int lx = threadIdx.x % BWT, ly = threadIdx.x / BWT;
    const int x = job.y * BWT + lx, y = job.z * BWT + ly;
    const bool inside = x < s.w && y < s.h;
    const int ci = (ly + halo) * t.TW + (lx + halo);
    const int K = s.K;
    const int x0 = job.y * BWT - halo, y0 = job.z * BWT - halo;
    uint8_t ua = 0;
    for (int k = 0; k < K; ++k) {
        const int opaque =
            ftile_load(t, wp, s.img[k], s.ipitch[k], s.istride[k], s.w, s.h, C, s.alpha[k], s.apitch[k], x0, y0);
        wk[k * BWT * BWT] = inside ? f_pixel_weight<CW, EW>(t, wp, tab, ci, x, y, s.w, s.h, C, opaque != 0) : 0.0f;
        ua |= t.a[ci];
        if (inside) {
            // level 0 of the exposure's image pyramid: the log mapping, once
            float* g0 = g0_level(s, k, C);
            const int TT = t.TW * t.TW;
            for (int c = 0; c < C; ++c) {
                g0[(int64_t)c * s.pitch[0] * s.h + (int64_t)y * s.pitch[0] + x] = to_pyramid_value(t.raw[c * TT + ci]);
            }
        }
        __syncthreads();  // the next exposure's load overwrites the tile
    }
    if (inside) {
        batch_normalise(s, wk, BWT * BWT, x, y, hard, ua);
    }
}

// Weights, normalisation, level 0 of the image pyramids and of the mask
// pyramids, and the union alpha of a 32x16 tile of a stack, two output
// pixels per thread (enb_fpair.cuh).  The exposures' tiles come in turn; a
// pixel's weight waits in its exposure's level-0 mask plane (as float bits)
// until the normalisation replaces it.  Five CTAs per SM (48 registers;
// the 42.6 KB tile of 5x5 windows fits five times): the warps hide the
// kernel's latencies better than more registers would.
template <int CW, int EW, int C>
__global__ void __launch_bounds__(FPT, 5) k_batch_weights_pair(const BatchStack* __restrict__ stacks,
                                                            const int4* __restrict__ jobs, FloatWeightParams wp,
                                                            WeightTables tab, int hard)
{
    constexpr int HALO = fpair_halo(CW, EW), HX = fpair_halo_x(HALO);
    constexpr int TW = fpair_tw(CW, EW), TT = TW * fpair_th(CW, EW), NP = (TT + FPT - 1) / FPT;
    extern __shared__ __align__(16) unsigned char bsmem[];
    const int4 job = jobs[blockIdx.x];
    const BatchStack& s = stacks[job.x];
    const FTileP t0 = fpair_carve(bsmem, TW, TT, wp.repeat_slots, wp.ent_cut);
    const int px = threadIdx.x % (FPX / 2), py = threadIdx.x / (FPX / 2);
    const int x = job.y * FPX + 2 * px, y = job.z * FPY + py;
    const bool in0 = x < s.w && y < s.h, in1 = x + 1 < s.w && y < s.h;
    const int cx = HX + 2 * px, cy = HALO + py, ci = cy * TW + cx;
    const int K = s.K;
    const int64_t plane = (int64_t)s.pitch[0] * s.h, o = (int64_t)y * s.pitch[0] + x;
    const int x0 = job.y * FPX - HX, y0 = job.z * FPY - HALO;
    uint8_t ua0 = 0, ua1 = 0;
    if (t0.slots) {
        fpair_clear_tables<C>(fpair_for_exposure(t0, 0));
        __syncthreads();
    }
    for (int k = 0; k < K; ++k) {
        const FTileP t = fpair_for_exposure(t0, k);
        const int opaque = fpair_load<NP, C, TW, TT>(t, wp, s.img[k], s.ipitch[k], s.istride[k], s.w, s.h, s.alpha[k],
                                                     s.apitch[k], x0, y0);
        if (in0) {
            float w0, w1;
            fpair_weights<CW, EW, C>(t, wp, tab, cx, cy, x, y, s.w, s.h, opaque != 0, w0, w1);
            int32_t* m0 = m_level(s, k, 0) + o;
            float* g0 = g0_level(s, k, C) + o;
            if (in1) {
                // x is even and rows start on 128-byte boundaries
                *reinterpret_cast<int2*>(m0) = make_int2(__float_as_int(w0), __float_as_int(w1));
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    // level 0 of the exposure's image pyramid: the log mapping, once
                    *reinterpret_cast<float2*>(g0 + c * plane) =
                        make_float2(to_pyramid_value(t.raw[c * TT + ci]), to_pyramid_value(t.raw[c * TT + ci + 1]));
                }
            } else {
                m0[0] = __float_as_int(w0);
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    g0[c * plane] = to_pyramid_value(t.raw[c * TT + ci]);
                }
            }
        }
        ua0 |= t.a[ci];
        ua1 |= t.a[ci + 1];
        if (t.slots && k + 1 < K) {
            // the tables for exposure k + 1 (the load of exposure k has ended
            // with a barrier; exposure k - 1's row masks were read before
            // the previous barrier)
            fpair_clear_tables<C>(fpair_for_exposure(t0, k + 1));
        }
        __syncthreads();  // the next exposure's load overwrites the tile; its tables are empty
    }
    // the union alpha; k_batch_normalise turns the weights into masks
    if (in0) {
        const uint8_t u0 = ua0 ? 255 : 0, u1 = ua1 ? 255 : 0;
        s.u[s.off0[0] + o] = u0;
        if (in1) {
            s.u[s.off0[0] + o + 1] = u1;
        }
        if (s.oalpha) {
            uint8_t* oa = s.oalpha + (int64_t)y * s.oapitch + x;
            oa[0] = u0;
            if (in1) {
                oa[1] = u1;
            }
        }
    }
}

// Normalisation of the weights that k_batch_weights_pair left in the level-0
// mask planes (float bits) of a 32x16 tile of a stack, two output pixels per
// thread: src/enfuse.h:1382-1385 (sum in exposure order), :1399-1442 (hard
// mask), :1526-1535 (soft mask), into Int32 9.15 masks.
__global__ void __launch_bounds__(256) k_batch_normalise(const BatchStack* __restrict__ stacks,
                                                         const int4* __restrict__ jobs, int hard)
{
    const int4 job = jobs[blockIdx.x];
    const BatchStack& s = stacks[job.x];
    const int px = threadIdx.x % (FPX / 2), py = threadIdx.x / (FPX / 2);
    const int x = job.y * FPX + 2 * px, y = job.z * FPY + py;
    if (x >= s.w || y >= s.h) {
        return;
    }
    const int K = s.K;
    const int64_t o = (int64_t)y * s.pitch[0] + x;
    const bool pair = x + 1 < s.w;
    const auto wt = [&](int k) {
        const int32_t* m = m_level(s, k, 0) + o;
        // x is even and rows start on 128-byte boundaries
        return pair ? __ldcg(reinterpret_cast<const float2*>(m)) : make_float2(__int_as_float(__ldcg(m)), 0.0f);
    };
    const auto put = [&](int k, float m0, float m1) {
        int32_t* m = m_level(s, k, 0) + o;
        if (pair) {
            *reinterpret_cast<int2*>(m) = make_int2(mask_to_fixed<int32_t>(m0, 15), mask_to_fixed<int32_t>(m1, 15));
        } else {
            m[0] = mask_to_fixed<int32_t>(m0, 15);
        }
    };
    if (hard) {
        float mx0 = 0.0f, mx1 = 0.0f;
        int mi0 = 0, mi1 = 0;
        for (int k = 0; k < K; ++k) {
            const float2 w = wt(k);
            if (w.x > mx0) {
                mx0 = w.x;
                mi0 = k;
            }
            if (w.y > mx1) {
                mx1 = w.y;
                mi1 = k;
            }
        }
        const float fallback = __fdiv_rn(255.0f, (float)K);
        for (int k = 0; k < K; ++k) {
            put(k, mx0 == 0.0f ? fallback : (k == mi0 ? 255.0f : 0.0f), mx1 == 0.0f ? fallback : (k == mi1 ? 255.0f : 0.0f));
        }
    } else {
        float n0 = 0.0f, n1 = 0.0f;
        for (int k = 0; k < K; ++k) {
            const float2 w = wt(k);
            n0 = __fadd_rn(w.x, n0);
            n1 = __fadd_rn(w.y, n1);
        }
        const float fallback = (float)(255 / K);
        for (int k = 0; k < K; ++k) {
            const float2 w = wt(k);
            put(k, n0 > 0.0f ? __fdiv_rn(__fmul_rn(255.0f, w.x), n0) : fallback,
                n1 > 0.0f ? __fdiv_rn(__fmul_rn(255.0f, w.y), n1) : fallback);
        }
    }
}

// ---------------------------------------------------------------------------
// reduce of one image or mask tile (down sweep)
// ---------------------------------------------------------------------------

// Job kind k < K: exposure k's image; K <= kind < 2K: exposure kind-K's mask.
// NC: the source levels are read through the read-only path (they were
// written by an earlier launch); false inside the coarse kernel, which reads
// levels it wrote itself.
template <int C, bool NC>
__device__ __forceinline__ void batch_reduce_tile(const BatchStack& s, int kind, int l, int X0, int Y0, int wrap,
                                                  unsigned char* smem)
{
    const int sw = s.lw[l], sh = s.lh[l], dw = s.lw[l + 1], dh = s.lh[l + 1];
    if (kind < s.K) {
        const int k = kind;
        float* dst = g_level(s, k, l + 1, C);
        const int64_t dplane = (int64_t)s.pitch[l + 1] * dh;
        float(*V)[RDH][RVP] = reinterpret_cast<float(*)[RDH][RVP]>(smem);
        if (l == 0) {
            using Src = Level0Source<C>;
            const ReduceJob<Src, float> job{
                Src{g0_level(s, k, C), s.pitch[0], (int64_t)s.pitch[0] * sh, s.alpha[k], s.apitch[k]}, dst,
                s.pitch[l + 1], dplane, a_level(s, k, l + 1), s.pitch[l + 1]};
            reduce_tile<Src, float, C, true, float>(job, X0, Y0, sw, sh, dw, dh, wrap, V);
        } else {
            using Src = PlanarSource<float, C, true, NC>;
            const ReduceJob<Src, float> job{
                Src{g_level(s, k, l, C), s.pitch[l], (int64_t)s.pitch[l] * sh, a_level(s, k, l), s.pitch[l]}, dst,
                s.pitch[l + 1], dplane, a_level(s, k, l + 1), s.pitch[l + 1]};
            reduce_tile<Src, float, C, true, float>(job, X0, Y0, sw, sh, dw, dh, wrap, V);
        }
    } else {
        const int k = kind - s.K;
        using Src = PlanarSource<int32_t, 1, true, NC>;
        int32_t(*V)[RDH][RVP] = reinterpret_cast<int32_t(*)[RDH][RVP]>(smem);
        const ReduceJob<Src, int32_t> job{
            Src{m_level(s, k, l), s.pitch[l], (int64_t)s.pitch[l] * sh, s.u + s.off0[l], s.pitch[l]},
            m_level(s, k, l + 1), s.pitch[l + 1], (int64_t)s.pitch[l + 1] * dh, s.u + s.off0[l + 1], s.pitch[l + 1]};
        reduce_tile<Src, int32_t, 1, true, int32_t>(job, X0, Y0, sw, sh, dw, dh, wrap, V);
    }
}

constexpr int kBatchReduceSmem = ReduceSmem<3, true>::WORDS * 4;

// Image jobs (kind < K) and mask jobs (kind >= K) of a level run as two
// launches, each with the registers its path needs.
template <int C>
__global__ void __launch_bounds__(RTHREADS, 3) k_batch_reduce(const BatchStack* __restrict__ stacks,
                                                              const int4* __restrict__ jobs, int l, int wrap)
{
    __shared__ __align__(16) unsigned char smem[kBatchReduceSmem];
    const int4 job = jobs[blockIdx.x];
    batch_reduce_tile<C, true>(stacks[job.x], job.y, l, job.z * RDW, job.w * RDH, wrap, smem);
}

__global__ void __launch_bounds__(RTHREADS, 4) k_batch_reduce_mask(const BatchStack* __restrict__ stacks,
                                                                   const int4* __restrict__ jobs, int l, int wrap)
{
    __shared__ __align__(16) int32_t V[ReduceSmem<1, true>::NV][RDH][RVP];
    const int4 job = jobs[blockIdx.x];
    const BatchStack& s = stacks[job.x];
    const int k = job.y - s.K;
    const int sw = s.lw[l], sh = s.lh[l], dw = s.lw[l + 1], dh = s.lh[l + 1];
    using Src = PlanarSource<int32_t, 1, true, true>;
    const ReduceJob<Src, int32_t> rj{
        Src{m_level(s, k, l), s.pitch[l], (int64_t)s.pitch[l] * sh, s.u + s.off0[l], s.pitch[l]}, m_level(s, k, l + 1),
        s.pitch[l + 1], (int64_t)s.pitch[l + 1] * dh, s.u + s.off0[l + 1], s.pitch[l + 1]};
    reduce_tile<Src, int32_t, 1, true, int32_t>(rj, job.z * RDW, job.w * RDH, sw, sh, dw, dh, wrap, V);
}

// ---------------------------------------------------------------------------
// merge and collapse of one level tile (up sweep)
// ---------------------------------------------------------------------------

// Expand (src/pyramid.h:875-1457, real division) of the quad (X, Y)..(X+1,
// Y+1) of destination pixels at source position (i, j) = (X/2, Y/2), from a
// window staged at source (I0 - 1, J0 - 1); e[q][c] for q = (0,0), (1,0),
// (0,1), (1,1).
template <int C>
__device__ __forceinline__ void expand_quad_f(const float (*ss)[ESH][ESW], int qx, int qy, int i, int j, int sw,
                                              int sh, int dw, int wrap, float (&e)[4][C])
{
    const int X = 2 * i, Y = 2 * j;
    if (i >= 1 && i + 1 < sw && j >= 1 && j + 1 < sh) {
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const float* a = &ss[c][qy][qx];
            const float* b = &ss[c][qy + 1][qx];
            const float* d = &ss[c][qy + 2][qx];
            const float hea = a[0] + 6.0f * a[1] + a[2], heb = b[0] + 6.0f * b[1] + b[2],
                        hec = d[0] + 6.0f * d[1] + d[2];
            const float hoa = 4.0f * (a[1] + a[2]), hob = 4.0f * (b[1] + b[2]), hoc = 4.0f * (d[1] + d[2]);
            e[0][c] = (hea + 6.0f * heb + hec) * 0.015625f;
            e[1][c] = (hoa + 6.0f * hob + hoc) * 0.015625f;
            e[2][c] = (heb + hec) * 0.0625f;
            e[3][c] = (hob + hoc) * 0.0625f;
        }
        return;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int XX = X + (q & 1), YY = Y + (q >> 1);
        int vw[3], vden, hw[3], hden;
        expand_vweights(YY, sh, vw, vden);
        expand_hweights(XX, sw, dw, wrap, hw, hden);
        const float den = (float)(hden * vden);
#pragma unroll
        for (int c = 0; c < C; ++c) {
            float num = 0.0f;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float* row = &ss[c][qy + a][qx];
                num += (float)vw[a] * ((float)hw[0] * row[0] + (float)hw[1] * row[1] + (float)hw[2] * row[2]);
            }
            e[q][c] = __fdiv_rn(num, den);
        }
    }
}

// Stages the (ESH x ESW) source window at (I0 - 1, J0 - 1) of a planar level
// (zero outside; x periodic when wrap).  All threads of the CTA call it.
template <int C>
__device__ __forceinline__ void stage_window(float (*ss)[ESH][ESW], const float* src, int64_t pitch, int64_t plane,
                                             int sw, int sh, int I0, int J0, int wrap)
{
    // element k = r * ESW + c, walked with a stride of blockDim.x
    int r = (int)threadIdx.x / ESW, c = (int)threadIdx.x - r * ESW;
    const int dr = (int)blockDim.x / ESW, dc = (int)blockDim.x - dr * ESW;
    for (; r < ESH;) {
        const int jj = J0 - 1 + r;
        int ii = I0 - 1 + c;
        if (wrap) {
            ii = imod(ii, sw);
        }
        const bool in = jj >= 0 && jj < sh && ii >= 0 && ii < sw;
        const int64_t o = (int64_t)jj * pitch + ii;
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            ss[ch][r][c] = in ? src[(int64_t)ch * plane + o] : 0.0f;
        }
        c += dc;
        r += dr;
        if (c >= ESW) {
            c -= ESW;
            ++r;
        }
    }
}

// stage_window by asynchronous 4-byte copies (zero-filled outside the level;
// the caller commits and waits): for levels written by an earlier launch.
template <int C>
__device__ __forceinline__ void stage_window_async(float (*ss)[ESH][ESW], const float* src, int64_t pitch, int64_t plane,
                                                   int sw, int sh, int I0, int J0, int wrap)
{
    int r = (int)threadIdx.x / ESW, c = (int)threadIdx.x - r * ESW;
    const int dr = (int)blockDim.x / ESW, dc = (int)blockDim.x - dr * ESW;
    for (; r < ESH;) {
        const int jj = J0 - 1 + r;
        int ii = I0 - 1 + c;
        if (wrap) {
            ii = imod(ii, sw);
        }
        const bool in = jj >= 0 && jj < sh && ii >= 0 && ii < sw;
        const float* p = in ? src + (int64_t)jj * pitch + ii : src;  // a valid address where nothing is read
        const unsigned n = in ? 4u : 0u;
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            const unsigned sa = (unsigned)__cvta_generic_to_shared(&ss[ch][r][c]);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(p + (in ? (int64_t)ch * plane : 0)),
                         "r"(n)
                         : "memory");
        }
        c += dc;
        r += dr;
        if (c >= ESW) {
            c -= ESW;
            ++r;
        }
    }
}

// One 64x16 tile of level l of a stack (256 working threads, 2x2 quads):
// C[l] = sum_k (G_k[l] - E(G_k[l+1])) m_k[l] / D + E(C[l+1]), written to
// the result level (l >= 1) or converted into the output pixels (l == 0).
// At the stack's top level the expand terms are absent.  The coarse kernel
// runs it on levels written in the same launch, so the levels >= 1 are read
// through the coherent path.  The level-(l+1) windows of all K exposures and
// of C[l+1] are staged together (one barrier); ss holds (K + 1) * C windows.
template <int C>
__device__ __forceinline__ void batch_up_tile(const BatchStack& s, int l, int X0, int Y0, int wrap, float inv_d,
                                              float (*ss)[ESH][ESW])
{
    const bool top = l == s.L - 1;
    const int K = s.K;
    const int dw = s.lw[l], dh = s.lh[l];
    const int sw = top ? 1 : s.lw[l + 1], sh = top ? 1 : s.lh[l + 1];
    const int I0 = X0 >> 1, J0 = Y0 >> 1;
    const int tid = threadIdx.x;
    const int qx = tid % 32, qy = tid / 32;
    const int i = I0 + qx, j = J0 + qy;
    const int X = 2 * i, Y = 2 * j;
    const bool active = tid < 256 && X < dw && Y < dh;
    const int64_t dp = s.pitch[l];
    const int64_t gplane = (int64_t)dp * dh;
    if (!top) {
        const int64_t sp = s.pitch[l + 1], splane = sp * sh;
        for (int k = 0; k <= K; ++k) {
            const float* src = k < K ? g_level(s, k, l + 1, C) : r_level(s, l + 1, C);
            stage_window<C>(ss + k * C, src, sp, splane, sw, sh, I0, J0, wrap);
        }
    }
    __syncthreads();
    if (!active) {
        return;
    }
    // channel by channel (fewer live registers): the K exposures' terms of
    // the four quad pixels, then the expand of C[l+1]
    for (int c = 0; c < C; ++c) {
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 2
        for (int k = 0; k < K; ++k) {
            float g[4], coeff[4];
            const int32_t* mk = m_level(s, k, l);
            const float* gk = l > 0 ? g_level(s, k, l, C) + (int64_t)c * gplane : nullptr;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int XX = min(X + (q & 1), dw - 1), YY = min(Y + (q >> 1), dh - 1);
                coeff[q] = __fmul_rn((float)ld_src<false>(&mk[(int64_t)YY * dp + XX]), inv_d);
                if (l == 0) {
                    g[q] = __ldg(&g0_level(s, k, C)[(int64_t)c * gplane + (int64_t)YY * dp + XX]);
                } else {
                    g[q] = ld_src<false>(&gk[(int64_t)YY * dp + XX]);
                }
            }
            float e[4][1] = {{0.0f}, {0.0f}, {0.0f}, {0.0f}};
            if (!top) {
                expand_quad_f<1>(ss + k * C + c, qx, qy, i, j, sw, sh, dw, wrap, e);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                // rounded like the per-stack merge (k_f_mask_mul_acc)
                acc[q] = __fadd_rn(acc[q], __fmul_rn(__fsub_rn(g[q], e[q][0]), coeff[q]));
            }
        }
        if (!top) {
            float e[4][1];
            expand_quad_f<1>(ss + K * C + c, qx, qy, i, j, sw, sh, dw, wrap, e);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                acc[q] = __fadd_rn(acc[q], e[q][0]);
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int XX = X + (q & 1), YY = Y + (q >> 1);
            if (XX >= dw || YY >= dh) {
                continue;
            }
            if (l > 0) {
                r_level(s, l, C)[(int64_t)c * gplane + (int64_t)YY * dp + XX] = acc[q];
            } else {
                float* o = s.out + (int64_t)YY * s.opitch + (int64_t)XX * s.ostride;
                const bool on = s.u[(int64_t)YY * dp + XX] != 0;
                o[c] = on ? from_pyramid_value(acc[q]) : 0.0f;
                if (c == 0 && s.ostride == 4) {
                    o[3] = on ? 1.0f : 0.0f;  // AlphaTraits<float>::max()
                }
            }
        }
    }
}

// Level 0 with the exposures' level-0 and mask tiles streamed through shared
// memory: while exposure k is merged from one buffer, exposure k+1's 64x16
// pyramid values and mask values are copied into the other (cp.async), so the
// loads of the next exposure are in flight during this one's arithmetic.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all_but_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Issues the copies of exposure k's level-0 tile (C planes) and mask tile.
template <int C>
__device__ __forceinline__ void up0_issue(const BatchStack& s, int k, int l, int X0, int Y0, int dw, int dh,
                                          float* g_tile, int32_t* mask_tile)
{
    const int nx = min(ETW, dw - X0), ny = min(ETH, dh - Y0);
    const float* g0 = l == 0 ? g0_level(s, k, C) : g_level(s, k, l, C);
    const int64_t plane = (int64_t)s.pitch[l] * dh, lp = s.pitch[l];
    if (nx == ETW) {
        // whole rows: 16-byte copies (rows of the level start on 128-byte
        // boundaries and a tile on a 256-byte one)
        constexpr int Q = ETW / 4;  // chunks of a row
        const int32_t* m = m_level(s, k, l);
        for (int e = threadIdx.x; e < (C + 1) * ETH * Q; e += blockDim.x) {
            const int c = e / (ETH * Q), rc = e - c * (ETH * Q), r = rc / Q, x = (rc - r * Q) * 4;
            if (r < ny) {
                if (c < C) {
                    cp_async16(&g_tile[(c * ETH + r) * ETW + x], &g0[c * plane + (int64_t)(Y0 + r) * lp + X0 + x]);
                } else {
                    cp_async16(&mask_tile[r * ETW + x], &m[(int64_t)(Y0 + r) * lp + X0 + x]);
                }
            }
        }
        return;
    }
    for (int e = threadIdx.x; e < C * ETH * ETW; e += blockDim.x) {
        const int c = e / (ETH * ETW), rc = e - c * (ETH * ETW), r = rc / ETW, x = rc - r * ETW;
        if (r < ny && x < nx) {
            cp_async4(&g_tile[e], &g0[c * plane + (int64_t)(Y0 + r) * lp + X0 + x]);
        }
    }
    const int32_t* m = m_level(s, k, l);
    for (int e = threadIdx.x; e < ETH * ETW; e += blockDim.x) {
        const int r = e / ETW, x = e - r * ETW;
        if (r < ny && x < nx) {
            cp_async4(&mask_tile[e], &m[(int64_t)(Y0 + r) * lp + X0 + x]);
        }
    }
}

// Stages of the level-0 merge: an exposure's level-0 tile (C planes), its
// mask tile and its level-1 window.
constexpr int kUp0Stages = 3;
template <int C>
__host__ __device__ constexpr int up0_stage_floats()
{
    return C * ETH * ETW + ETH * ETW + C * ESH * ESW;
}

// Level l of a stack (one 64x16 tile, 2x2 quads): level 0 converts the
// result into the output pixels, levels >= 1 write the result level
// (batch_up_tile's computation with the tiles streamed through the stages).
template <int C, bool L0>
__global__ void __launch_bounds__(256, 3) k_batch_up0(const BatchStack* __restrict__ stacks,
                                                     const int4* __restrict__ jobs, int l, int wrap, float inv_d)
{
    extern __shared__ __align__(16) float up0smem[];
    const int4 job = jobs[blockIdx.x];
    const BatchStack& s = stacks[job.x];
    if (L0) {
        l = 0;
    }
    const int K = s.K;
    const bool top = l == s.L - 1;
    const int X0 = job.y * ETW, Y0 = job.z * ETH;
    const int dw = s.lw[l], dh = s.lh[l];
    const int sw = top ? 1 : s.lw[l + 1], sh = top ? 1 : s.lh[l + 1];
    const int I0 = X0 >> 1, J0 = Y0 >> 1;
    const int64_t sp = top ? 0 : s.pitch[l + 1], splane = sp * sh;
    // stage b: [C planes of the level-0 tile][mask tile][C planes of the level-1 window];
    // after the stages, the window of C[1]
    const auto g_tile = [&](int b) { return up0smem + b * up0_stage_floats<C>(); };
    const auto mask_tile = [&](int b) { return reinterpret_cast<int32_t*>(g_tile(b) + C * ETH * ETW); };
    const auto window = [&](int b) {
        return reinterpret_cast<float(*)[ESH][ESW]>(g_tile(b) + C * ETH * ETW + ETH * ETW);
    };
    float(*rwin)[ESH][ESW] = reinterpret_cast<float(*)[ESH][ESW]>(up0smem + kUp0Stages * up0_stage_floats<C>());
    const auto issue = [&](int k) {
        const int b = k % kUp0Stages;
        if (!top) {
            stage_window_async<C>(window(b), g_level(s, k, l + 1, C), sp, splane, sw, sh, I0, J0, wrap);
        }
        up0_issue<C>(s, k, l, X0, Y0, dw, dh, g_tile(b), mask_tile(b));
    };
    // exposures 0 and 1 (with the window of C[1]) in flight before the first merge
    if (!top) {
        stage_window_async<C>(rwin, r_level(s, l + 1, C), sp, splane, sw, sh, I0, J0, wrap);
    }
    issue(0);
    cp_async_commit();
    if (K > 1) {
        issue(1);
    }
    cp_async_commit();
    const int tid = threadIdx.x;
    const int qx = tid % 32, qy = tid / 32;
    const int i = I0 + qx, j = J0 + qy;
    const int X = 2 * i, Y = 2 * j;
    const bool active = X < dw && Y < dh;
    float acc[4][C];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int c = 0; c < C; ++c) {
            acc[q][c] = 0.0f;
        }
    }
    for (int k = 0; k < K; ++k) {
        // the stage of exposure k + 2 was last read while merging exposure
        // k - 1, before the previous barrier
        if (k + 2 < K) {
            issue(k + 2);
        }
        cp_async_commit();
        asm volatile("cp.async.wait_group 2;\n" ::: "memory");  // exposure k's group has landed
        __syncthreads();
        if (active) {
            const int b = k % kUp0Stages;
            const float* gt = g_tile(b);
            const int32_t* mt = mask_tile(b);
            float e[4][C];
            if (!top) {
                expand_quad_f<C>(window(b), qx, qy, i, j, sw, sh, dw, wrap, e);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int xx = min(X + (q & 1), dw - 1) - X0, yy = min(Y + (q >> 1), dh - 1) - Y0;
                const float coeff = __fmul_rn((float)mt[yy * ETW + xx], inv_d);
#pragma unroll
                for (int c = 0; c < C; ++c) {
                    const float g = gt[c * ETH * ETW + yy * ETW + xx];
                    // rounded like the per-stack merge (k_f_mask_mul_acc)
                    acc[q][c] = __fadd_rn(acc[q][c], __fmul_rn(top ? g : __fsub_rn(g, e[q][c]), coeff));
                }
            }
        }
        __syncthreads();  // this stage is refilled for exposure k + 3
    }
    if (!active) {
        return;
    }
    float e[4][C];
    if (!top) {
        expand_quad_f<C>(rwin, qx, qy, i, j, sw, sh, dw, wrap, e);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int XX = X + (q & 1), YY = Y + (q >> 1);
        if (XX >= dw || YY >= dh) {
            continue;
        }
        if (!L0) {
            float* r = r_level(s, l, C) + (int64_t)YY * s.pitch[l] + XX;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                r[(int64_t)c * s.pitch[l] * dh] = top ? acc[q][c] : __fadd_rn(acc[q][c], e[q][c]);
            }
            continue;
        }
        float* o = s.out + (int64_t)YY * s.opitch + (int64_t)XX * s.ostride;
        const bool on = s.u[(int64_t)YY * s.pitch[0] + XX] != 0;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            o[c] = on ? from_pyramid_value(top ? acc[q][c] : __fadd_rn(acc[q][c], e[q][c])) : 0.0f;
        }
        if (s.ostride == 4) {
            o[3] = on ? 1.0f : 0.0f;  // AlphaTraits<float>::max()
        }
    }
}

// ---------------------------------------------------------------------------
// coarse levels: a persistent kernel walking (stack, level, tile) items
// ---------------------------------------------------------------------------
//
// The coarse end of every stack (its levels of at most coarse_pixels pixels)
// is a list of items, each one tile of one step: a reduce tile of one
// exposure's image or mask pyramid (down, level l -> l + 1), or an up tile
// (Laplacians, masks, merge and collapse of level l).  The items of a step
// depend on the whole previous step of the same stack (a tile's halo reaches
// into its neighbours), which a per-(stack, step) counter records: an item
// waits until the counter of its predecessor step reaches that step's item
// count, and counts itself in its own step's counter when done.  The host
// orders the device queue step by step across the stacks (step 0 of every
// stack, then step 1, ...), so an item's predecessors always come earlier in
// the queue; the CTAs take items in queue order, so every item an item waits
// for is held by a running CTA, and no wait depends on a CTA that has not
// started.  Waits are bounded (about a second); a CTA whose wait runs out
// sets bit 1 of the context's error word and stops, and the items that
// depend on its own item then run out too: the launch ends, and the host
// fails the call.

struct CoarseItem {
    int stack, up, level, kind, tile;  // up = 0: reduce tile of `kind` (image k < K, mask K + k)
    int wait_ctr, wait_count;          // predecessor step's counter (-1: none) and its item count
    int sig_ctr;                       // this step's counter
};

constexpr long long kCoarseWaitSpins = 1ll << 23;  // x ~128 ns sleeps: about a second

template <int C>
__global__ void __launch_bounds__(RTHREADS) k_batch_coarse(const BatchStack* __restrict__ stacks,
                                                           const CoarseItem* __restrict__ items, int nitems,
                                                           int* __restrict__ queue, int* ctrs, unsigned int* err,
                                                           int wrap, float inv_d)
{
    extern __shared__ __align__(16) unsigned char smem[];  // max(reduce tile, (K + 1) * C windows)
    __shared__ int item;
    __shared__ int ready;
    for (;;) {
        if (threadIdx.x == 0) {
            const int it = atomicAdd(queue, 1);
            int ok = 1;
            if (it < nitems) {
                const int wc = items[it].wait_ctr, need = items[it].wait_count;
                if (wc >= 0) {
                    long long spins = 0;
                    while (atomicAdd(&ctrs[wc], 0) < need) {
                        if (++spins > kCoarseWaitSpins) {
                            ok = 0;
                            break;
                        }
                        __nanosleep(128);
                    }
                    __threadfence();  // the predecessor step's writes before this item's reads
                }
            }
            item = it;
            ready = ok;
        }
        __syncthreads();
        const int it = item;
        const int ok = ready;
        __syncthreads();
        if (it >= nitems) {
            return;
        }
        if (!ok) {
            if (threadIdx.x == 0) {
                atomicOr(err, 2u);
            }
            return;
        }
        const CoarseItem ci = items[it];
        const BatchStack& s = stacks[ci.stack];
        if (!ci.up) {
            const int tx = (s.lw[ci.level + 1] + RDW - 1) / RDW;
            batch_reduce_tile<C, false>(s, ci.kind, ci.level, (ci.tile % tx) * RDW, (ci.tile / tx) * RDH, wrap, smem);
        } else {
            float(*ss)[ESH][ESW] = reinterpret_cast<float(*)[ESH][ESW]>(smem);
            const int tx = (s.lw[ci.level] + ETW - 1) / ETW;
            batch_up_tile<C>(s, ci.level, (ci.tile % tx) * ETW, (ci.tile / tx) * ETH, wrap, inv_d, ss);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();  // this item's writes before its count
            atomicAdd(&ctrs[ci.sig_ctr], 1);
        }
    }
}

// ---------------------------------------------------------------------------
// host: plan of a batch and its launches
// ---------------------------------------------------------------------------

struct BatchPlan {
    int C = 3;
    int nstacks = 0;
    int wrap = 0, hard = 0;
    FloatWeightParams wp{};
    WeightTables tab{};
    size_t wsmem = 0;
    void* work = nullptr;         // workspace of all stacks
    BatchStack* dstacks = nullptr;
    int4* djobs = nullptr;
    CoarseItem* ditems = nullptr;  // the coarse items in queue order
    int* dqueue = nullptr;         // queue position, then one counter per (stack, coarse step)
    int nitems = 0, nctrs = 0;
    unsigned int* err = nullptr;   // the context's device error word
    int maxK = 1;
    bool pair_weights = false;  // the weights step runs k_batch_weights_pair
    struct Step {
        int kind;  // 0 weights, 5 normalisation, 1 image reduce, 4 mask reduce, 2 coarse, 3 up
        int level;
        int64_t job0, njobs;
        double bytes;
    };
    std::vector<Step> steps;
    int64_t coarse_pixels = 4096;
    double pixels = 0.0;  // sum of K * w * h
};

namespace {

void level_geometry(BatchStack& s, int64_t coarse_pixels)
{
    int lw = s.w, lh = s.h;
    int64_t o0 = 0, o1 = 0;
    s.Lc = s.L;
    for (int l = 0; l < s.L; ++l) {
        s.lw[l] = lw;
        s.lh[l] = lh;
        s.pitch[l] = (int)((lw + 31) / 32 * 32);
        s.off0[l] = o0;
        s.off1[l] = l >= 1 ? o1 : 0;
        o0 += (int64_t)s.pitch[l] * lh;
        if (l >= 1) {
            o1 += (int64_t)s.pitch[l] * lh;
            if (s.Lc == s.L && (int64_t)lw * lh <= coarse_pixels) {
                s.Lc = l;
            }
        }
        lw = (lw + 1) >> 1;
        lh = (lh + 1) >> 1;
    }
    s.s0 = o0;
    s.s1 = o1 > 0 ? o1 : 1;
}

}  // namespace

void batch_plan_destroy(BatchPlan* p)
{
    if (!p) {
        return;
    }
    cudaFree(p->work);
    delete p;
}

cudaError_t batch_plan_create(const std::vector<BatchStackHost>& hs, const FloatWeightParams& wp,
                              const WeightTables& tab, int levels, int wrap, int hard, int64_t coarse_pixels,
                              unsigned int* err, cudaStream_t st, BatchPlan** out)
{
    BatchPlan* p = new BatchPlan();
    p->err = err;
    p->nstacks = (int)hs.size();
    p->wrap = wrap;
    p->hard = hard;
    p->wp = wp;
    p->tab = tab;
    p->C = hs.empty() ? 3 : hs[0].C;
    p->coarse_pixels = coarse_pixels;
    std::vector<BatchStack> stacks(hs.size());
    size_t bytes = 0;
    auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
    std::vector<size_t> base(hs.size());
    for (size_t i = 0; i < hs.size(); ++i) {
        BatchStack& s = stacks[i];
        std::memset(&s, 0, sizeof s);
        const BatchStackHost& h = hs[i];
        s.K = h.K;
        s.w = h.w;
        s.h = h.h;
        s.L = enb_num_levels(h.w, h.h, 1, levels);
        for (int k = 0; k < h.K; ++k) {
            s.img[k] = h.img[k];
            s.ipitch[k] = h.ipitch[k];
            s.istride[k] = h.istride[k];
            s.alpha[k] = h.alpha[k];
            s.apitch[k] = h.apitch[k];
        }
        s.out = h.out;
        s.opitch = h.opitch;
        s.ostride = h.ostride;
        s.oalpha = h.oalpha;
        s.oapitch = h.oapitch;
        level_geometry(s, coarse_pixels);
        base[i] = bytes;
        bytes += align((size_t)s.K * s.s0 * 4) + align((size_t)s.s0) + align((size_t)s.K * p->C * s.s1 * 4) +
                 align((size_t)s.K * s.s1) + align((size_t)p->C * s.s1 * 4) + align((size_t)s.K * p->C * s.s0 * 4);
        p->pixels += (double)h.K * h.w * h.h;
        p->maxK = std::max(p->maxK, h.K);
    }
    // job tables
    std::vector<int4> jobs;
    auto add_step = [&](int kind, int level, double b) {
        p->steps.push_back(BatchPlan::Step{kind, level, 0, 0, b});
        p->steps.back().job0 = (int64_t)jobs.size();
    };
    // the tile, then the K weights of each output pixel
    p->pair_weights = fpair_path(wp);
    int wtx = BWT, wty = BWT;
    if (p->pair_weights) {
        const int cw = wp.use_contrast ? wp.contrast_window : 0, ew = wp.use_entropy ? wp.entropy_window : 0;
        const int TT = fpair_tw(cw, ew) * fpair_th(cw, ew);
        p->wp.repeat_slots = fpair_slots(wp, TT);
        p->wsmem = fpair_tile_bytes(TT, p->wp.repeat_slots, p->wp.ent_cut);
        wtx = FPX;
        wty = FPY;
    } else {
        const int TW = BWT + 2 * fweight_halo(wp);
        p->wp.repeat_slots = fweight_slots(wp, TW);
        p->wsmem = align16(ftile_bytes(TW, p->wp.repeat_slots, p->wp.ent_cut)) + (size_t)p->maxK * BWT * BWT * sizeof(float);
    }
    double b = 0.0;
    add_step(0, 0, 0.0);
    for (int i = 0; i < p->nstacks; ++i) {
        const BatchStack& s = stacks[i];
        for (int ty = 0; ty < (s.h + wty - 1) / wty; ++ty) {
            for (int tx = 0; tx < (s.w + wtx - 1) / wtx; ++tx) {
                jobs.push_back(make_int4(i, tx, ty, 0));
            }
        }
        b += (double)s.K * s.w * s.h * (4.0 * hs[i].istride[0] + 4.0) + (double)s.w * s.h;
    }
    p->steps.back().njobs = (int64_t)jobs.size() - p->steps.back().job0;
    p->steps.back().bytes = b;
    if (p->pair_weights) {
        // the normalisation, over the weights step's tiles
        const BatchPlan::Step w = p->steps.back();
        double nb = 0.0;
        for (const BatchStack& s : stacks) {
            nb += (double)s.K * s.w * s.h * 12.0;
        }
        p->steps.push_back(BatchPlan::Step{5, 0, w.job0, w.njobs, nb});
    }
    int maxL = 0;
    for (const BatchStack& s : stacks) {
        maxL = std::max(maxL, s.L);
    }
    for (int l = 0; l + 1 < maxL; ++l) {
        add_step(1, l, 0.0);
        b = 0.0;
        for (int i = 0; i < p->nstacks; ++i) {
            const BatchStack& s = stacks[i];
            if (l + 1 > std::min(s.Lc, s.L - 1)) {
                continue;
            }
            const int tx = (s.lw[l + 1] + RDW - 1) / RDW, ty = (s.lh[l + 1] + RDH - 1) / RDH;
            for (int kind = 0; kind < s.K; ++kind) {
                for (int y = 0; y < ty; ++y) {
                    for (int x = 0; x < tx; ++x) {
                        jobs.push_back(make_int4(i, kind, x, y));
                    }
                }
            }
            const double src = (double)s.lw[l] * s.lh[l], dst = (double)s.lw[l + 1] * s.lh[l + 1];
            b += s.K * (src * (l == 0 ? 4.0 * hs[i].istride[0] : 4.0 * p->C + 1.0) + dst * (4.0 * p->C + 1.0));
        }
        p->steps.back().njobs = (int64_t)jobs.size() - p->steps.back().job0;
        p->steps.back().bytes = b;
        if (p->steps.back().njobs == 0) {
            p->steps.pop_back();
        }
        add_step(4, l, 0.0);
        b = 0.0;
        for (int i = 0; i < p->nstacks; ++i) {
            const BatchStack& s = stacks[i];
            if (l + 1 > std::min(s.Lc, s.L - 1)) {
                continue;
            }
            const int tx = (s.lw[l + 1] + RDW - 1) / RDW, ty = (s.lh[l + 1] + RDH - 1) / RDH;
            for (int kind = s.K; kind < 2 * s.K; ++kind) {
                for (int y = 0; y < ty; ++y) {
                    for (int x = 0; x < tx; ++x) {
                        jobs.push_back(make_int4(i, kind, x, y));
                    }
                }
            }
            const double src = (double)s.lw[l] * s.lh[l], dst = (double)s.lw[l + 1] * s.lh[l + 1];
            b += s.K * (src * 4.0 + dst * 4.0) + src + dst;
        }
        p->steps.back().njobs = (int64_t)jobs.size() - p->steps.back().job0;
        p->steps.back().bytes = b;
        if (p->steps.back().njobs == 0) {
            p->steps.pop_back();
        }
    }
    // the coarse items: per stack, the down steps (source levels Lc .. L-2,
    // each all exposures' image and mask tiles) then the up steps (levels
    // L-1 .. Lc); queued step by step across the stacks
    std::vector<CoarseItem> items;
    {
        struct StackSteps {
            int stack, base;                       // first counter
            std::vector<std::vector<CoarseItem>> steps;
        };
        std::vector<StackSteps> ss;
        int nctr = 0;
        for (int i = 0; i < p->nstacks; ++i) {
            const BatchStack& s = stacks[i];
            if (s.Lc >= s.L) {
                continue;
            }
            StackSteps st{i, nctr, {}};
            for (int l = s.Lc; l + 1 < s.L; ++l) {
                std::vector<CoarseItem> step;
                const int t = ((s.lw[l + 1] + RDW - 1) / RDW) * ((s.lh[l + 1] + RDH - 1) / RDH);
                for (int kind = 0; kind < 2 * s.K; ++kind) {
                    for (int j = 0; j < t; ++j) {
                        step.push_back(CoarseItem{i, 0, l, kind, j, -1, 0, 0});
                    }
                }
                st.steps.push_back(step);
            }
            for (int l = s.L - 1; l >= s.Lc; --l) {
                std::vector<CoarseItem> step;
                const int t = ((s.lw[l] + ETW - 1) / ETW) * ((s.lh[l] + ETH - 1) / ETH);
                for (int j = 0; j < t; ++j) {
                    step.push_back(CoarseItem{i, 1, l, 0, j, -1, 0, 0});
                }
                st.steps.push_back(step);
            }
            for (size_t k = 0; k < st.steps.size(); ++k) {
                for (CoarseItem& it : st.steps[k]) {
                    it.sig_ctr = st.base + (int)k;
                    if (k > 0) {
                        it.wait_ctr = st.base + (int)k - 1;
                        it.wait_count = (int)st.steps[k - 1].size();
                    }
                }
            }
            nctr += (int)st.steps.size();
            ss.push_back(std::move(st));
        }
        for (size_t k = 0;; ++k) {
            bool any = false;
            for (const StackSteps& st : ss) {
                if (k < st.steps.size()) {
                    items.insert(items.end(), st.steps[k].begin(), st.steps[k].end());
                    any = true;
                }
            }
            if (!any) {
                break;
            }
        }
        p->nitems = (int)items.size();
        p->nctrs = nctr;
    }
    if (p->nitems) {
        add_step(2, 0, 0.0);
    }
    for (int l = maxL - 1; l >= 0; --l) {
        add_step(3, l, 0.0);
        b = 0.0;
        for (int i = 0; i < p->nstacks; ++i) {
            const BatchStack& s = stacks[i];
            if (l > std::min(s.Lc, s.L) - 1) {
                continue;
            }
            const int tx = (s.lw[l] + ETW - 1) / ETW, ty = (s.lh[l] + ETH - 1) / ETH;
            for (int y = 0; y < ty; ++y) {
                for (int x = 0; x < tx; ++x) {
                    jobs.push_back(make_int4(i, x, y, 0));
                }
            }
            const double px = (double)s.lw[l] * s.lh[l], up = l + 1 < s.L ? (double)s.lw[l + 1] * s.lh[l + 1] : 0.0;
            b += s.K * (px * ((l == 0 ? 4.0 * hs[i].istride[0] : 4.0 * p->C) + 4.0) + up * 4.0 * p->C) +
                 up * 4.0 * p->C + px * (l == 0 ? 4.0 * hs[i].ostride + 1.0 : 4.0 * p->C);
        }
        p->steps.back().njobs = (int64_t)jobs.size() - p->steps.back().job0;
        p->steps.back().bytes = b;
        if (p->steps.back().njobs == 0) {
            p->steps.pop_back();
        }
    }
    // device memory: workspace, stack table, jobs, coarse list, queue counter
    const size_t o_st = align(bytes), o_jobs = o_st + align(sizeof(BatchStack) * stacks.size()),
                 o_coarse = o_jobs + align(sizeof(int4) * std::max<size_t>(jobs.size(), 1)),
                 o_queue = o_coarse + align(sizeof(CoarseItem) * std::max<size_t>(items.size(), 1)),
                 total = o_queue + align(sizeof(int) * (size_t)(1 + p->nctrs));
    cudaError_t e = cudaMalloc(&p->work, total);
    if (e != cudaSuccess) {
        delete p;
        return e;
    }
    char* w = (char*)p->work;
    for (size_t i = 0; i < stacks.size(); ++i) {
        BatchStack& s = stacks[i];
        char* q = w + base[i];
        s.m = (int32_t*)q;
        q += align((size_t)s.K * s.s0 * 4);
        s.u = (uint8_t*)q;
        q += align((size_t)s.s0);
        s.g = (float*)q;
        q += align((size_t)s.K * p->C * s.s1 * 4);
        s.a = (uint8_t*)q;
        q += align((size_t)s.K * s.s1);
        s.r = (float*)q;
        q += align((size_t)p->C * s.s1 * 4);
        s.g0 = (float*)q;
    }
    p->dstacks = (BatchStack*)(w + o_st);
    p->djobs = (int4*)(w + o_jobs);
    p->ditems = (CoarseItem*)(w + o_coarse);
    p->dqueue = (int*)(w + o_queue);
    e = cudaMemcpyAsync(p->dstacks, stacks.data(), sizeof(BatchStack) * stacks.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !jobs.empty()) {
        e = cudaMemcpyAsync(p->djobs, jobs.data(), sizeof(int4) * jobs.size(), cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess && !items.empty()) {
        e = cudaMemcpyAsync(p->ditems, items.data(), sizeof(CoarseItem) * items.size(), cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(st);  // the host tables go out of scope
    }
    if (e != cudaSuccess) {
        batch_plan_destroy(p);
        return e;
    }
    *out = p;
    return cudaSuccess;
}

int batch_plan_steps(const BatchPlan* p) { return (int)p->steps.size(); }
double batch_plan_pixels(const BatchPlan* p) { return p->pixels; }

// Shared memory of an up tile: the windows of K exposures and of C[l+1].
static size_t up_smem_bytes(int K, int C) { return (size_t)(K + 1) * C * ESH * ESW * sizeof(float); }

template <int C>
static cudaError_t launch_step(const BatchPlan* p, const BatchPlan::Step& s, cudaStream_t st)
{
    const int4* jobs = p->djobs + s.job0;
    const float inv_d = (float)(1.0 / (double)(255 << 15));
    switch (s.kind) {
    case 0: {
        note_launch("batch_weights", s.bytes);
        if (p->pair_weights) {
            ENB_FPAIR_DISPATCH(p->wp, {
                auto k = k_batch_weights_pair<CWV, EWV, C>;
                if (p->wsmem > 48 * 1024) {
                    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->wsmem);
                }
                // as many CTAs per SM as the shared memory holds
                cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
                k<<<(unsigned)s.njobs, FPT, p->wsmem, st>>>(p->dstacks, jobs, p->wp, p->tab, p->hard);
            });
            break;
        }
        const int cw = p->wp.use_contrast ? p->wp.contrast_window : 5;
        const int ew = p->wp.use_entropy ? p->wp.entropy_window : 5;
        void (*k)(const BatchStack*, const int4*, FloatWeightParams, WeightTables, int, int) = k_batch_weights<0, 0>;
        if (cw == 5 && ew == 5) {
            k = k_batch_weights<5, 5>;
        } else if (cw == 5 && ew == 3) {
            k = k_batch_weights<5, 3>;
        } else if (cw == 3 && ew == 3) {
            k = k_batch_weights<3, 3>;
        } else if (ew == 5) {
            k = k_batch_weights<0, 5>;
        } else if (ew == 3) {
            k = k_batch_weights<0, 3>;
        }
        if (p->wsmem > 48 * 1024) {
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->wsmem);
        }
        k<<<(unsigned)s.njobs, BWT * BWT, p->wsmem, st>>>(p->dstacks, jobs, p->wp, p->tab, p->hard, C);
        break;
    }
    case 5:
        note_launch("batch_normalise", s.bytes);
        k_batch_normalise<<<(unsigned)s.njobs, 256, 0, st>>>(p->dstacks, jobs, p->hard);
        break;
    case 1:
        note_launch("batch_reduce", s.bytes);
        k_batch_reduce<C><<<(unsigned)s.njobs, RTHREADS, 0, st>>>(p->dstacks, jobs, s.level, p->wrap);
        break;
    case 4:
        note_launch("batch_reduce_mask", s.bytes);
        k_batch_reduce_mask<<<(unsigned)s.njobs, RTHREADS, 0, st>>>(p->dstacks, jobs, s.level, p->wrap);
        break;
    case 2: {
        note_launch("batch_coarse", 0.0);
        // the queue position and the step counters start at 0 on every run
        cudaError_t e = cudaMemsetAsync(p->dqueue, 0, sizeof(int) * (size_t)(1 + p->nctrs), st);
        if (e != cudaSuccess) {
            return e;
        }
        int sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int grid = std::max(1, std::min(p->nitems, 2 * sms));
        const size_t smem = std::max((size_t)kBatchReduceSmem, up_smem_bytes(p->maxK, C));
        if (smem > 48 * 1024) {
            cudaFuncSetAttribute(k_batch_coarse<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        }
        k_batch_coarse<C><<<grid, RTHREADS, smem, st>>>(p->dstacks, p->ditems, p->nitems, p->dqueue, p->dqueue + 1,
                                                        p->err, p->wrap, inv_d);
        break;
    }
    default: {
        note_launch(s.level == 0 ? "batch_up0" : "batch_up", s.bytes);
        if (s.level == 0) {
            const size_t smem = ((size_t)kUp0Stages * up0_stage_floats<C>() + (size_t)C * ESH * ESW) * sizeof(float);
            if (smem > 48 * 1024) {
                cudaFuncSetAttribute(k_batch_up0<C, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            }
            k_batch_up0<C, true><<<(unsigned)s.njobs, 256, smem, st>>>(p->dstacks, jobs, 0, p->wrap, inv_d);
            break;
        }
        const size_t smem = ((size_t)kUp0Stages * up0_stage_floats<C>() + (size_t)C * ESH * ESW) * sizeof(float);
        if (smem > 48 * 1024) {
            cudaFuncSetAttribute(k_batch_up0<C, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        }
        k_batch_up0<C, false><<<(unsigned)s.njobs, 256, smem, st>>>(p->dstacks, jobs, s.level, p->wrap, inv_d);
        break;
    }
    }
    return cudaGetLastError();
}

cudaError_t batch_plan_launch(const BatchPlan* p, int i, cudaStream_t st)
{
    const BatchPlan::Step& s = p->steps[(size_t)i];
    return p->C == 1 ? launch_step<1>(p, s, st) : launch_step<3>(p, s, st);
}

}  // namespace enb
