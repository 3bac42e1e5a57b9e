// enb_reduce.cuh -- the Burt-Adelson reduce (src/pyramid.h:166-848) as one
// tiled kernel over pluggable sources.
//
// A CTA computes a 64x16 tile of destination pixels from the 131x35 source
// window around it (2 pixels of halo), in two phases:
//   1. column sums: 262 threads each take one source column and 8
//      destination rows, load the column's 19 source rows into registers (all
//      loads issued before any arithmetic, so that a thread keeps ~19 loads in
//      flight) and form the vertical [1 4 6 4 1] sums at the even rows;
//   2. row sums: 256 threads each take 4 adjacent destination pixels of one
//      row, read the 11 column sums they need with three 16-byte shared loads
//      per channel and form the horizontal [1 4 6 4 1] sums.
// The weights are separable and the sums exact integers, so the order of the
// taps does not change the result.
//   with alpha: normalised convolution over the opaque taps, taps outside the
//               image dropped, x periodic when wrap (pyramid.h:166-573);
//   no alpha:   clamp-to-edge replication in y (and x unless wrap), /256
//               (pyramid.h:601-848).
// blockIdx.z selects one of up to two jobs of the same geometry (the white and
// black pyramids of a level), so a level of both images is one launch.
#pragma once

#include "enb_device.cuh"
#include "enb_internal.h"

namespace enb {

constexpr int RDW = 64, RDH = 16;        // destination tile
constexpr int RSW = 2 * RDW + 3;         // 131 source columns
constexpr int RSH = 2 * RDH + 3;         // 35 source rows
constexpr int RGR = 8;                   // destination rows of a column item
constexpr int RGN = 2 * RGR + 3;         // 19 source rows of a column item
constexpr int RITEMS = RSW * (RDH / RGR);  // 262 column items
constexpr int RTHREADS = 288;
constexpr int RVP = 148;                 // padded row of column sums

// Column c of a row of column sums sits at c + 4*(c/32): the 16-byte reads of
// phase 2 (8 threads at a stride of 8 words) then hit 32 distinct banks.
__device__ __forceinline__ int rphys(int c) { return c + ((c >> 5) << 2); }

// Planar pyramid level (+ an 8-bit alpha plane when A); NC: read-only load
// path (the level is not written by the launch).  Samples are delivered in
// the accumulator type of the reduce (int32 for fixed point, float for the
// FP32 pyramids of float images).
template <typename TS, int C, bool A, bool NC = true>
struct PlanarSource {
    const TS* p;
    int64_t pitch, plane;   // elements
    const uint8_t* a;
    int64_t apitch;
    template <typename AC>
    __device__ __forceinline__ void load(int gy, int gx, AC (&v)[C], int& al) const
    {
        const int64_t o = (int64_t)gy * pitch + gx;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            v[c] = (AC)ld_src<NC>(&p[c * plane + o]);
        }
        al = A ? (ld_src<NC>(&a[(int64_t)gy * apitch + gx]) != 0) : 1;
    }
};

// 8-bit seam mask converted to fixed point on the fly.
struct ByteSource {
    const uint8_t* p;
    int64_t pitch;
    int frac;
    template <typename AC>
    __device__ __forceinline__ void load(int gy, int gx, AC (&v)[1], int& al) const
    {
        v[0] = (int32_t)__ldg(&p[(int64_t)gy * pitch + gx]) << frac;
        al = 1;
    }
};

template <class Src, typename TD>
struct ReduceJob {
    Src src;
    TD* dst;
    int64_t dpitch, dplane;  // elements
    uint8_t* da;             // destination alpha (with alpha) or null
    int64_t dapitch;
};

template <class Src, typename TD>
struct ReduceJobs {
    ReduceJob<Src, TD> j[2];
    int ty0;  // first destination tile row of the launch
};

// Phase 1 for one column item: vertical sums of destination rows r0..r0+7.
// Border items load from clamped (always valid) positions and zero the taps
// outside the image afterwards, so that no load waits behind a branch and
// all 19 rows are in flight at once.
template <class Src, int C, bool ALPHA, bool INTERIOR, typename AC>
__device__ __forceinline__ void reduce_column(const Src& src, int gx, int gyb, int sw, int sh, int wrap,
                                              AC (*V)[RDH][RVP], int col, int r0)
{
    constexpr int NV = C + (ALPHA ? 1 : 0);
    bool colok = true;
    if (!INTERIOR) {
        if (wrap) {
            gx = imod(gx, sw);
        } else {
            colok = gx >= 0 && gx < sw;
            gx = min(max(gx, 0), sw - 1);
        }
    }
    AC x[RGN][NV];
#pragma unroll
    for (int k = 0; k < RGN; ++k) {
        int gy = gyb + k;
        bool ok = true;
        if (!INTERIOR) {
            ok = colok && gy >= 0 && gy < sh;
            gy = min(max(gy, 0), sh - 1);
        }
        AC v[C];
        int al = 1;
        src.load(gy, gx, v, al);
        if (ALPHA) {
            al = ok ? al : 0;   // taps outside the image are dropped
        }
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            x[k][ch] = (ALPHA && !al) ? (AC)0 : v[ch];   // without alpha: clamp-to-edge
        }
        if (ALPHA) {
            x[k][NV - 1] = (AC)al;
        }
    }
    const int pc = rphys(col);
#pragma unroll
    for (int r = 0; r < RGR; ++r) {
#pragma unroll
        for (int ch = 0; ch < NV; ++ch) {
            V[ch][r0 + r][pc] = x[2 * r][ch] + (AC)4 * x[2 * r + 1][ch] + (AC)6 * x[2 * r + 2][ch] +
                                (AC)4 * x[2 * r + 3][ch] + x[2 * r + 4][ch];
        }
    }
}

__device__ __forceinline__ void store4(float* p, const float (&v)[4], int n)
{
    if (n == 4 && ((uintptr_t)p & 15) == 0) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (q < n) {
                p[q] = v[q];
            }
        }
    }
}

template <typename TD>
__device__ __forceinline__ void store4(TD* p, const int32_t (&v)[4], int n)
{
    if (n == 4 && ((uintptr_t)p & (4 * sizeof(TD) - 1)) == 0) {
        if (sizeof(TD) == 4) {
            *reinterpret_cast<int4*>(p) = make_int4(v[0], v[1], v[2], v[3]);
        } else {
            *reinterpret_cast<uint2*>(p) = make_uint2((uint32_t)(uint16_t)v[0] | ((uint32_t)(uint16_t)v[1] << 16),
                                                      (uint32_t)(uint16_t)v[2] | ((uint32_t)(uint16_t)v[3] << 16));
        }
    } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (q < n) {
                p[q] = cast_store<TD>(v[q]);
            }
        }
    }
}

// Shared memory of one reduce tile: NV planes of 16 rows of column sums.
template <int C, bool ALPHA>
struct ReduceSmem {
    static constexpr int NV = C + (ALPHA ? 1 : 0);
    static constexpr int WORDS = NV * RDH * RVP;
};

// Normalisation of a tap sum by the opaque weight sum den > 0: truncating
// integer division for fixed point (pyramid.h:242-250), real division for
// the float pyramids (SKIPSMImagePixelType double in the reference).
__device__ __forceinline__ int32_t reduce_norm(int32_t s, int32_t den)
{
    return den == 256 ? s / 256 : div_any(s, den);
}
__device__ __forceinline__ float reduce_norm(float s, float den) { return __fdiv_rn(s, den); }
__device__ __forceinline__ int32_t reduce_256(int32_t s) { return s / 256; }
__device__ __forceinline__ float reduce_256(float s) { return s * 0.00390625f; }

// One 64x16 destination tile at (X0, Y0) of a reduce job (RTHREADS threads;
// V holds ReduceSmem<C, ALPHA>::WORDS 16-byte aligned words of the
// accumulator type AC: int32 for fixed point, float for FP32 levels).
template <class Src, typename TD, int C, bool ALPHA, typename AC = int32_t>
__device__ __forceinline__ void reduce_tile(const ReduceJob<Src, TD>& job, int X0, int Y0, int sw, int sh, int dw,
                                            int dh, int wrap, AC (*V)[RDH][RVP])
{
    constexpr int NV = C + (ALPHA ? 1 : 0);
    const int gx0 = 2 * X0 - 2, gy0 = 2 * Y0 - 2;
    const int tid = threadIdx.x;

    if (tid < RITEMS) {
        const int g = tid >= RSW ? 1 : 0;
        const int col = tid - g * RSW;
        const int gyb = gy0 + 2 * RGR * g;
        if (gx0 >= 0 && gy0 >= 0 && gx0 + RSW <= sw && gy0 + RSH <= sh) {
            reduce_column<Src, C, ALPHA, true, AC>(job.src, gx0 + col, gyb, sw, sh, wrap, V, col, RGR * g);
        } else {
            reduce_column<Src, C, ALPHA, false, AC>(job.src, gx0 + col, gyb, sw, sh, wrap, V, col, RGR * g);
        }
    }
    __syncthreads();

    const int r = tid >> 4, k = tid & 15;
    const int Y = Y0 + r, Xb = X0 + 4 * k;
    if (tid >= RDH * (RDW / 4) || Y >= dh || Xb >= dw) {
        return;
    }
    const int n = min(4, dw - Xb);
    AC s[NV][4];
#pragma unroll
    for (int ch = 0; ch < NV; ++ch) {
        const AC* row = &V[ch][r][0];
        AC v[12];
        *reinterpret_cast<int4*>(&v[0]) = *reinterpret_cast<const int4*>(row + rphys(8 * k));
        *reinterpret_cast<int4*>(&v[4]) = *reinterpret_cast<const int4*>(row + rphys(8 * k + 4));
        *reinterpret_cast<int4*>(&v[8]) = *reinterpret_cast<const int4*>(row + rphys(8 * k + 8));
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            s[ch][q] = v[2 * q] + (AC)4 * v[2 * q + 1] + (AC)6 * v[2 * q + 2] + (AC)4 * v[2 * q + 3] + v[2 * q + 4];
        }
    }
    const int64_t o = (int64_t)Y * job.dpitch + Xb;
    if (ALPHA) {
        AC out[C][4];
        uint32_t abits = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const AC den = s[NV - 1][q];
#pragma unroll
            for (int ch = 0; ch < C; ++ch) {
                out[ch][q] = den <= (AC)0 ? (AC)0 : reduce_norm(s[ch][q], den);
            }
            abits |= (den > (AC)0 ? 255u : 0u) << (8 * q);
        }
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            store4(job.dst + ch * job.dplane + o, out[ch], n);
        }
        uint8_t* ap = job.da + (int64_t)Y * job.dapitch + Xb;
        if (n == 4 && ((uintptr_t)ap & 3) == 0) {
            *reinterpret_cast<uint32_t*>(ap) = abits;
        } else {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (q < n) {
                    ap[q] = (uint8_t)(abits >> (8 * q));
                }
            }
        }
    } else {
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            AC out[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                out[q] = reduce_256(s[ch][q]);
            }
            store4(job.dst + ch * job.dplane + o, out, n);
        }
    }
}

// Accumulator of a reduce into destination type TD.
template <typename TD> struct ReduceAcc { typedef int32_t type; };
template <> struct ReduceAcc<float> { typedef float type; };

template <class Src, typename TD, int C, bool ALPHA>
__global__ void __launch_bounds__(RTHREADS, 3) k_reduce(ReduceJobs<Src, TD> jobs, int sw, int sh, int dw, int dh,
                                                        int wrap)
{
    typedef typename ReduceAcc<TD>::type AC;
    __shared__ __align__(16) AC V[ReduceSmem<C, ALPHA>::NV][RDH][RVP];
    griddep_wait();
    griddep_launch();
    const ReduceJob<Src, TD> job = blockIdx.z == 0 ? jobs.j[0] : jobs.j[1];
    reduce_tile<Src, TD, C, ALPHA, AC>(job, blockIdx.x * RDW, (blockIdx.y + jobs.ty0) * RDH, sw, sh, dw, dh, wrap, V);
}

// Destination tile rows of the reduce (16 rows each).
inline int reduce_tile_rows(int dh) { return (dh + RDH - 1) / RDH; }

// One level of enblend's down sweep in one launch: the white and black image
// reduces with alpha (blockIdx.z 0 and 1) and the seam mask's reduce without
// (blockIdx.z 2), so that the three Gaussian pyramids advance together
// (src/enblend.h:384-446).
template <class SrcI, typename TI, int C, class SrcM, typename TM>
__global__ void __launch_bounds__(RTHREADS, 3) k_reduce_img2_mask(const __grid_constant__ ReduceJobs<SrcI, TI> img,
                                                                  const __grid_constant__ ReduceJob<SrcM, TM> msk,
                                                                  int sw, int sh, int dw, int dh, int wrap)
{
    typedef typename ReduceAcc<TI>::type ACI;
    typedef typename ReduceAcc<TM>::type ACM;
    constexpr size_t BI = sizeof(ACI) * ReduceSmem<C, true>::NV * RDH * RVP;
    constexpr size_t BM = sizeof(ACM) * ReduceSmem<1, false>::NV * RDH * RVP;
    __shared__ __align__(16) unsigned char V[BI > BM ? BI : BM];
    griddep_wait();
    griddep_launch();
    if (blockIdx.z < 2) {
        reduce_tile<SrcI, TI, C, true, ACI>(img.j[blockIdx.z], blockIdx.x * RDW, blockIdx.y * RDH, sw, sh, dw, dh,
                                            wrap, reinterpret_cast<ACI(*)[RDH][RVP]>(V));
    } else {
        reduce_tile<SrcM, TM, 1, false, ACM>(msk, blockIdx.x * RDW, blockIdx.y * RDH, sw, sh, dw, dh, wrap,
                                             reinterpret_cast<ACM(*)[RDH][RVP]>(V));
    }
}

// One launch over njobs (1 or 2) jobs of the same geometry, covering the
// destination tile rows [ty0, ty0 + nty) (nty < 0: all).
template <class Src, typename TD, int C, bool ALPHA>
inline void launch_reduce_jobs(ReduceJobs<Src, TD> jobs, int njobs, int sw, int sh, int dw, int dh, int wrap,
                               cudaStream_t st, int ty0 = 0, int nty = -1)
{
    if (nty < 0) {
        nty = reduce_tile_rows(dh) - ty0;
    }
    if (nty <= 0) {
        return;
    }
    jobs.ty0 = ty0;
    const dim3 g((unsigned)((dw + RDW - 1) / RDW), (unsigned)nty, (unsigned)njobs);
    (void)launch_pdl(k_reduce<Src, TD, C, ALPHA>, g, dim3(RTHREADS), st, jobs, sw, sh, dw, dh, wrap);
}

// Up to kReduceMaxJobs jobs of one geometry in one launch (blockIdx.z = job):
// the K exposures of a fused enfuse level.
constexpr int kReduceMaxJobs = 16;

template <class Src, typename TD>
struct ReduceJobsN {
    ReduceJob<Src, TD> j[kReduceMaxJobs];
};

template <class Src, typename TD, int C, bool ALPHA>
__global__ void __launch_bounds__(RTHREADS, 3) k_reduce_n(const __grid_constant__ ReduceJobsN<Src, TD> jobs, int sw,
                                                          int sh, int dw, int dh, int wrap)
{
    typedef typename ReduceAcc<TD>::type AC;
    __shared__ __align__(16) AC V[ReduceSmem<C, ALPHA>::NV][RDH][RVP];
    griddep_wait();
    griddep_launch();
    reduce_tile<Src, TD, C, ALPHA, AC>(jobs.j[blockIdx.z], blockIdx.x * RDW, blockIdx.y * RDH, sw, sh, dw, dh, wrap,
                                       V);
}

template <class Src, typename TD, int C, bool ALPHA>
inline cudaError_t launch_reduce_n(const ReduceJobsN<Src, TD>& jobs, int njobs, int sw, int sh, int dw, int dh,
                                   int wrap, cudaStream_t st)
{
    const dim3 g((unsigned)((dw + RDW - 1) / RDW), (unsigned)reduce_tile_rows(dh), (unsigned)njobs);
    return launch_pdl(k_reduce_n<Src, TD, C, ALPHA>, g, dim3(RTHREADS), st, jobs, sw, sh, dw, dh, wrap);
}

template <class Src, typename TD, int C, bool ALPHA>
inline void launch_reduce_tiles(const Src& src, int sw, int sh, TD* dst, int64_t dpitch, int64_t dplane, int dw,
                                int dh, uint8_t* da, int64_t dapitch, int wrap, cudaStream_t st)
{
    ReduceJobs<Src, TD> jobs{};
    jobs.j[0] = ReduceJob<Src, TD>{src, dst, dpitch, dplane, da, dapitch};
    jobs.j[1] = jobs.j[0];
    launch_reduce_jobs<Src, TD, C, ALPHA>(jobs, 1, sw, sh, dw, dh, wrap, st);
}

}  // namespace enb
