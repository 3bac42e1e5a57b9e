// enb_pixels.cuh -- interleaved pixel I/O shared by the fused enblend and
// enfuse kernels: vector pixel loads and stores, the pixel's alpha (8-bit
// plane, opaque, or the thresholded 4th component, src/assemble.h:240-253)
// and the reduce source that converts pixels to fixed point on the fly.
#pragma once

#include <stdint.h>

#include "enb_device.cuh"

namespace enb {

// ---------------------------------------------------------------------------
// Pixel I/O
// ---------------------------------------------------------------------------

// Interleaved pixel load/store; VEC packs the 4 samples of an RGBA pixel in
// one 4- or 8-byte access (the caller checks the alignment).
template <typename TIn, int S, bool VEC>
__device__ __forceinline__ void ld_px(const TIn* p, TIn (&o)[S])
{
    if (VEC && S == 4 && sizeof(TIn) == 2) {
        const uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
        o[0] = (TIn)(v.x & 0xffffu);
        o[1] = (TIn)(v.x >> 16);
        o[2] = (TIn)(v.y & 0xffffu);
        o[S - 1] = (TIn)(v.y >> 16);
    } else if (VEC && S == 4 && sizeof(TIn) == 1) {
        const uint32_t v = __ldg(reinterpret_cast<const uint32_t*>(p));
        o[0] = (TIn)(v & 0xffu);
        o[1] = (TIn)((v >> 8) & 0xffu);
        o[2] = (TIn)((v >> 16) & 0xffu);
        o[S - 1] = (TIn)(v >> 24);
    } else {
#pragma unroll
        for (int c = 0; c < S; ++c) {
            o[c] = __ldg(&p[c]);
        }
    }
}

template <typename TIn, int S, bool VEC>
__device__ __forceinline__ void st_px(TIn* p, const TIn (&o)[S])
{
    if (VEC && S == 4 && sizeof(TIn) == 2) {
        uint2 v;
        v.x = (uint32_t)o[0] | ((uint32_t)o[1] << 16);
        v.y = (uint32_t)o[2] | ((uint32_t)o[S - 1] << 16);
        *reinterpret_cast<uint2*>(p) = v;
    } else if (VEC && S == 4 && sizeof(TIn) == 1) {
        *reinterpret_cast<uint32_t*>(p) =
            (uint32_t)o[0] | ((uint32_t)o[1] << 8) | ((uint32_t)o[2] << 16) | ((uint32_t)o[S - 1] << 24);
    } else {
#pragma unroll
        for (int c = 0; c < S; ++c) {
            p[c] = o[c];
        }
    }
}

// Alpha of an interleaved pixel: 8-bit plane (AM 0), opaque (AM 1) or the
// thresholded 4th component (AM 2, src/assemble.h:240-253).
template <int AM, typename TIn, int S>
__device__ __forceinline__ int pixel_alpha(const TIn (&px)[S], const uint8_t* ap, int64_t apitch, int x, int y,
                                           uint32_t alo, uint32_t ahi)
{
    if (AM == 0) {
        return __ldg(&ap[(int64_t)y * apitch + x]) != 0;
    }
    if (AM == 1) {
        return 1;
    }
    const uint32_t v = px[S - 1];
    return v >= alo && v <= ahi;
}

// Source of the tiled reduce: interleaved pixels converted to fixed point
// on the fly (copyToPyramidImage, src/fixmath.h:197-202).
template <typename TIn, int C, int S, int AM, bool VEC>
struct PixelSourceV {
    const TIn* p;
    int64_t pitch;
    const uint8_t* a;
    int64_t apitch;
    uint32_t lo, hi;
    int frac;
    __device__ __forceinline__ void load(int gy, int gx, int32_t (&v)[C], int& al) const
    {
        TIn px[S];
        ld_px<TIn, S, VEC>(p + (int64_t)gy * pitch + (int64_t)gx * S, px);
#pragma unroll
        for (int c = 0; c < C; ++c) {
            v[c] = (int32_t)px[c] << frac;
        }
        al = pixel_alpha<AM, TIn, S>(px, a, apitch, gx, gy, lo, hi);
    }
};

}  // namespace enb
