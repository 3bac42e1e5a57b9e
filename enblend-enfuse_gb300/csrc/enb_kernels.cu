// enb_kernels.cu -- sm_103a kernels of the enblend/enfuse multiresolution path.
//
// Integer stages reproduce the reference's fixed-point arithmetic exactly
// (src/pyramid.h, src/fixmath.h, src/blend.h, src/enfuse.h:601-620).  Where the
// reference rounds an IEEE double expression, the kernels either evaluate it
// with the same round-to-nearest double operations (__dmul_rn/__dadd_rn/
// __ddiv_rn, never contracted into FMAs) or with an exact integer/float
// formulation that provably yields the same result, falling back to the double
// expression in the rare cases the fast path cannot decide.
#include <cuda_runtime.h>
#include <stdint.h>

#include "enb_device.cuh"
#include "enb_internal.h"
#include "enb_entropy.cuh"
#include "enb_iweights.cuh"
#include "enb_reduce.cuh"

namespace enb {

// ---------------------------------------------------------------------------
// Conversions to fixed point (src/fixmath.h:116-206)
// ---------------------------------------------------------------------------

template <typename TS, typename TD>
__global__ void __launch_bounds__(256) k_to_fixed(const TS* __restrict__ src, int64_t spitch, int stride, int C,
                                                  TD* __restrict__ dst, int64_t dpitch, int64_t dplane,
                                                  int w, int h, int frac)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const TS* s = src + (int64_t)y * spitch + (int64_t)x * stride;
    for (int c = 0; c < C; ++c) {
        dst[(int64_t)c * dplane + (int64_t)y * dpitch + x] = (TD)((int32_t)s[c] << frac);
    }
}

template <typename TD>
__global__ void __launch_bounds__(256) k_float_to_fixed(const float* __restrict__ src, int64_t spitch,
                                                        TD* __restrict__ dst, int64_t dpitch, int w, int h,
                                                        int frac)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const double v = __dmul_rn((double)src[(int64_t)y * spitch + x], (double)(1u << frac));
    dst[(int64_t)y * dpitch + x] = frp_store<TD>(v);
}

// Soft-mask normalisation fused with the conversion of the mask to fixed
// point (src/enfuse.h:1526-1535 then fixmath.h:189-195).
template <typename TD>
__global__ void __launch_bounds__(256) k_soft_mask_to_fixed(const float* __restrict__ mask, int64_t mpitch,
                                                            const float* __restrict__ norm, int64_t npitch,
                                                            float fallback, TD* __restrict__ dst,
                                                            int64_t dpitch, int w, int h, int frac)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const float n = norm[(int64_t)y * npitch + x];
    const float m = n > 0.0f ? __fdiv_rn(__fmul_rn(255.0f, mask[(int64_t)y * mpitch + x]), n) : fallback;
    dst[(int64_t)y * dpitch + x] = mask_to_fixed<TD>(m, frac);
}

template <typename TD>
__global__ void __launch_bounds__(256) k_bytes_to_fixed(const uint8_t* __restrict__ src, int64_t spitch,
                                                        TD* __restrict__ dst, int64_t dpitch, int w, int h,
                                                        int frac)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    dst[(int64_t)y * dpitch + x] = (TD)((int32_t)src[(int64_t)y * spitch + x] << frac);
}

__global__ void __launch_bounds__(256) k_alpha_extract(AlphaSrc a, uint8_t* __restrict__ dst, int64_t dpitch,
                                                       int w, int h)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    dst[(int64_t)y * dpitch + x] = alpha_at(a, x, y) ? 255 : 0;
}

// Reduce (src/pyramid.h:166-848): k_reduce_tiles in enb_reduce.cuh.

// ---------------------------------------------------------------------------
// Expand (src/pyramid.h:875-1457)
// ---------------------------------------------------------------------------
//
// Destination pixel (X, Y) is a separable interpolation of the source:
// horizontally (1,6,1) at even X and (4,4) at odd X, vertically (1,6,1) at
// even Y and (1,1) at odd Y, divided by the product of the in-image weight
// sums (64 or 16 inside the image; 56, 49, 14, 8, ... at the borders).  One
// thread handles the 2x2 destination quad of one source pixel.

template <typename T, bool ADD>
__device__ __forceinline__ void expand_combine(T* d, int32_t e)
{
    if (ADD) {
        *d = sat_store<T>((int32_t)*d + e);
    } else {
        *d = cast_store<T>((int64_t)*d - e);
    }
}

template <typename T, int C, bool ADD>
__global__ void __launch_bounds__(256) k_expand(const T* __restrict__ src, int64_t spitch, int64_t splane, int sw,
                                                int sh, T* __restrict__ dst, int64_t dpitch, int64_t dplane, int dw,
                                                int dh, int wrap)
{
    __shared__ int32_t ss[C][ESH][ESW];
    const int X0 = blockIdx.x * ETW, Y0 = blockIdx.y * ETH;
    const int I0 = X0 >> 1, J0 = Y0 >> 1;
    const int tid = threadIdx.x;

    for (int k = tid; k < ESH * ESW; k += 256) {
        const int r = k / ESW, c = k - r * ESW;
        const int j = J0 - 1 + r;
        int i = I0 - 1 + c;
        if (wrap) {
            i = imod(i, sw);
        }
        const bool in = j >= 0 && j < sh && i >= 0 && i < sw;
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            ss[ch][r][c] = in ? (int32_t)src[(int64_t)ch * splane + (int64_t)j * spitch + i] : 0;
        }
    }
    __syncthreads();

    const int qx = tid % 32, qy = tid / 32;
    const int i = I0 + qx, j = J0 + qy;
    const int X = 2 * i, Y = 2 * j;
    if (X >= dw || Y >= dh) {
        return;
    }
    const bool has_x1 = X + 1 < dw, has_y1 = Y + 1 < dh;
    const bool interior = i >= 1 && i + 1 < sw && j >= 1 && j + 1 < sh;

    if (interior) {
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            const int32_t* a = &ss[ch][qy][qx];
            const int32_t* b = &ss[ch][qy + 1][qx];
            const int32_t* c = &ss[ch][qy + 2][qx];
            const int32_t hea = a[0] + 6 * a[1] + a[2], heb = b[0] + 6 * b[1] + b[2], hec = c[0] + 6 * c[1] + c[2];
            const int32_t hoa = 4 * (a[1] + a[2]), hob = 4 * (b[1] + b[2]), hoc = 4 * (c[1] + c[2]);
            T* d0 = reinterpret_cast<T*>(dst) + (int64_t)ch * dplane + (int64_t)Y * dpitch + X;
            expand_combine<T, ADD>(d0, (hea + 6 * heb + hec) / 64);
            if (has_x1) {
                expand_combine<T, ADD>(d0 + 1, (hoa + 6 * hob + hoc) / 64);
            }
            if (has_y1) {
                T* d1 = d0 + dpitch;
                expand_combine<T, ADD>(d1, (heb + hec) / 16);
                if (has_x1) {
                    expand_combine<T, ADD>(d1 + 1, (hob + hoc) / 16);
                }
            }
        }
        return;
    }

    // Border quads: per-position weights and divisors.
#pragma unroll
    for (int oy = 0; oy < 2; ++oy) {
        const int YY = Y + oy;
        if (YY >= dh) {
            continue;
        }
        int vw[3], vden;
        expand_vweights(YY, sh, vw, vden);
#pragma unroll
        for (int ox = 0; ox < 2; ++ox) {
            const int XX = X + ox;
            if (XX >= dw) {
                continue;
            }
            int hw[3], hden;
            expand_hweights(XX, sw, dw, wrap, hw, hden);
            const int den = hden * vden;
#pragma unroll
            for (int ch = 0; ch < C; ++ch) {
                int32_t num = 0;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const int32_t* row = &ss[ch][qy + a][qx];
                    num += vw[a] * (hw[0] * row[0] + hw[1] * row[1] + hw[2] * row[2]);
                }
                T* d = reinterpret_cast<T*>(dst) + (int64_t)ch * dplane + (int64_t)YY * dpitch + XX;
                expand_combine<T, ADD>(d, div_den(num, den));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Merge operators
// ---------------------------------------------------------------------------

// CartesianBlendFunctor (src/blend.h:41-76) in place on the black level,
// evaluated by blend_sample (exact integer rounding, double only at ties).
template <typename T, typename TM, int C>
__global__ void __launch_bounds__(256) k_blend(const TM* __restrict__ mask, int64_t mpitch,
                                               const T* __restrict__ white, int64_t wpitch, int64_t wplane,
                                               T* __restrict__ black, int64_t bpitch, int64_t bplane, int w,
                                               int h, int32_t white_value)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const int32_t m = (int32_t)mask[(int64_t)y * mpitch + x];
    if (m <= 0) {
        return;
    }
    if (m >= white_value) {
#pragma unroll
        for (int c = 0; c < C; ++c) {
            black[(int64_t)c * bplane + (int64_t)y * bpitch + x] = white[(int64_t)c * wplane + (int64_t)y * wpitch + x];
        }
        return;
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
        T* b = &black[(int64_t)c * bplane + (int64_t)y * bpitch + x];
        *b = (T)blend_sample<T>(m, white_value, (int32_t)white[(int64_t)c * wplane + (int64_t)y * wpitch + x],
                                (int32_t)*b);
    }
}

template <typename T, typename TM, int C, int F>
__global__ void __launch_bounds__(256) k_mask_mul_acc(const T* __restrict__ lp, int64_t lpitch, int64_t lplane,
                                                      const TM* __restrict__ mask, int64_t mpitch,
                                                      T* __restrict__ res, int64_t rpitch, int64_t rplane, int w,
                                                      int h, int accumulate)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const int32_t m = (int32_t)mask[(int64_t)y * mpitch + x];
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const T v = mask_multiply<T, F>((int32_t)lp[(int64_t)c * lplane + (int64_t)y * lpitch + x], m);
        T* r = &res[(int64_t)c * rplane + (int64_t)y * rpitch + x];
        *r = accumulate ? cast_store<T>((int64_t)*r + v) : v;
    }
}

// Generic (non-constant divisor) variant for the primitive entry point.
template <typename T, typename TM, int C>
__global__ void __launch_bounds__(256) k_mask_mul_acc_generic(const T* __restrict__ lp, int64_t lpitch,
                                                              int64_t lplane, const TM* __restrict__ mask,
                                                              int64_t mpitch, int32_t divisor,
                                                              T* __restrict__ res, int64_t rpitch, int64_t rplane,
                                                              int w, int h, int accumulate)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const double coeff = __ddiv_rn((double)mask[(int64_t)y * mpitch + x], (double)divisor);
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const T v = frp_store<T>(__dmul_rn((double)lp[(int64_t)c * lplane + (int64_t)y * lpitch + x], coeff));
        T* r = &res[(int64_t)c * rplane + (int64_t)y * rpitch + x];
        *r = accumulate ? cast_store<T>((int64_t)*r + v) : v;
    }
}

// ---------------------------------------------------------------------------
// Conversion from fixed point (src/fixmath.h:241-277)
// ---------------------------------------------------------------------------

template <typename TS, typename TD>
__global__ void __launch_bounds__(256) k_from_fixed(const TS* __restrict__ src, int64_t spitch, int64_t splane, int C,
                                                    const uint8_t* __restrict__ alpha, int64_t apitch,
                                                    TD* __restrict__ dst, int64_t dpitch, int dstride, int w, int h,
                                                    int frac, int dither, uint64_t seed, int32_t maxv)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w || !alpha[(int64_t)y * apitch + x]) {
        return;
    }
    const uint32_t key = dither_key(seed);
    const uint64_t pix = (uint64_t)y * (uint64_t)w + (uint64_t)x;
    const uint32_t pixbits = mix32((uint32_t)pix ^ key);
    for (int c = 0; c < C; ++c) {
        const int32_t v = (int32_t)src[(int64_t)c * splane + (int64_t)y * spitch + x];
        const uint32_t bits = dither_sample_bits(key, pixbits, pix, C, c, frac);
        dst[(int64_t)y * dpitch + (int64_t)x * dstride + c] =
            (TD)dither_rule(v, frac, dither == ENB_DITHER_NEAREST, bits, maxv);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_copy_pixels(const T* __restrict__ src, int64_t spitch,
                                                     T* __restrict__ dst, int64_t dpitch, int rowlen, int h)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x < rowlen) {
        dst[(int64_t)y * dpitch + x] = src[(int64_t)y * spitch + x];
    }
}

// 4th component of an RGBA result: the union alpha scaled to the sample type,
// as the output writer stores the alpha image (src/assemble.h:133-225).
template <typename T>
__global__ void __launch_bounds__(256) k_alpha_component(const uint8_t* __restrict__ a, int64_t apitch,
                                                         T* __restrict__ dst, int64_t dpitch, int w, int h, T maxv)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x < w) {
        dst[(int64_t)y * dpitch + (int64_t)x * 4 + 3] = a[(int64_t)y * apitch + x] ? maxv : (T)0;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_copy_level0(const T* __restrict__ src, int64_t spitch, int64_t splane,
                                                     int C, int32_t* __restrict__ dst, int w, int h)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    for (int c = 0; c < C; ++c) {
        dst[((int64_t)y * w + x) * C + c] = (int32_t)src[(int64_t)c * splane + (int64_t)y * spitch + x];
    }
}

// ---------------------------------------------------------------------------
// enfuse weights (src/enfuse.h:962-1212)
// ---------------------------------------------------------------------------

// 32 x 16 output pixels per CTA, a pair of horizontally adjacent pixels per
// thread: fully opaque tiles take the pair path (enb_iweights.cuh), the
// others the per-pixel weight.
constexpr int EMX = 32, EMY = 16;

__host__ __device__ inline int emask_halo_x(const WeightParams& wp) { return (iweight_halo(wp) + 1) & ~1; }

__global__ void __launch_bounds__(256, 3) k_enfuse_mask(PixelView img, AlphaSrc alpha, WeightParams wp,
                                                        WeightTables tab, float* __restrict__ out, int64_t opitch)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int halo = iweight_halo(wp), hx = emask_halo_x(wp);
    const int TW = EMX + 2 * hx, TH = EMY + 2 * halo;
    const ITile t = itile_carve_rect(smem, TW, TH);
    long long* fx = reinterpret_cast<long long*>(smem + ((itile_bytes_rect(TW, TH) + 15) & ~(size_t)15));  // [32]
    const bool pair_path = iweight_pair_path(wp);
    if (wp.use_entropy && pair_path && (int)threadIdx.x <= wp.entropy_window * wp.entropy_window) {
        const int M = wp.entropy_window * wp.entropy_window;
        fx[threadIdx.x] = tab.plogp_fx[(int64_t)M * (M + 1) + threadIdx.x];
    }
    // ends with a barrier (which also publishes fx)
    const int opaque = itile_load_rect(t, wp, img, alpha, blockIdx.x * EMX - hx, blockIdx.y * EMY - halo);
    const int px = threadIdx.x % (EMX / 2), py = threadIdx.x / (EMX / 2);
    const int x = blockIdx.x * EMX + 2 * px, y = blockIdx.y * EMY + py;
    const int cx = hx + 2 * px, cy = halo + py;
    if (opaque && pair_path) {
        float w0, w1;
        pair_weights(t, wp, tab, fx, img.C, cx, cy, w0, w1);
        out[(int64_t)y * opitch + x] = w0;
        out[(int64_t)y * opitch + x + 1] = w1;
        return;
    }
    const int ci = cy * TW + cx;
    if (y < img.h && x < img.w) {
        out[(int64_t)y * opitch + x] = i_pixel_weight(t, wp, tab, img, ci, x, y);
    }
    if (y < img.h && x + 1 < img.w) {
        out[(int64_t)y * opitch + x + 1] = i_pixel_weight(t, wp, tab, img, ci + 1, x + 1, y);
    }
}

__global__ void __launch_bounds__(256) k_norm_accumulate(const float* __restrict__ m, int64_t mpitch,
                                                         float* __restrict__ norm, int64_t npitch, int w, int h,
                                                         int first)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const float v = m[(int64_t)y * mpitch + x];
    float* n = &norm[(int64_t)y * npitch + x];
    *n = first ? __fadd_rn(v, 0.0f) : __fadd_rn(v, *n);
}

__global__ void __launch_bounds__(256) k_union_alpha(const uint8_t* __restrict__ a, int64_t apitch,
                                                     uint8_t* __restrict__ u, int64_t upitch, int w, int h,
                                                     int first)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const uint8_t v = a[(int64_t)y * apitch + x];
    uint8_t* d = &u[(int64_t)y * upitch + x];
    if (first) {
        *d = v;
    } else if (v) {
        *d = v;
    }
}

constexpr int kMaxHardMasks = 64;
struct HardMaskArgs {
    float* p[kMaxHardMasks];
    int64_t pitch[kMaxHardMasks];
};

// Hard mask: argmax (first maximum) -> 255, others 0; all-zero -> 255/K
// (src/enfuse.h:1402-1442).
__global__ void __launch_bounds__(256) k_hard_mask(HardMaskArgs m, int K, int w, int h)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    float mx = 0.0f;
    int mi = 0;
    for (int k = 0; k < K; ++k) {
        const float v = m.p[k][(int64_t)y * m.pitch[k] + x];
        if (v > mx) {
            mx = v;
            mi = k;
        }
    }
    const float fallback = __fdiv_rn(255.0f, (float)K);
    for (int k = 0; k < K; ++k) {
        m.p[k][(int64_t)y * m.pitch[k] + x] = mx == 0.0f ? fallback : (k == mi ? 255.0f : 0.0f);
    }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

static inline dim3 row_grid(int w, int h) { return dim3((unsigned)((w + 255) / 256), (unsigned)h); }

LaunchInfo& last_launch()
{
    static thread_local LaunchInfo li{"", 0.0, 1};
    return li;
}

static inline double esz(int dt) { return dt == ENB_U8 ? 1.0 : ((dt == ENB_U16 || dt == ENB_I16) ? 2.0 : 4.0); }
static inline double npix(int w, int h) { return (double)w * (double)h; }
static inline double planar_bytes(const PlanarView& v) { return npix(v.w, v.h) * v.C * esz(v.dtype); }
static inline void note(const char* name, double bytes) { last_launch() = LaunchInfo{name, bytes, 1}; }

cudaError_t launch_to_fixed(const PixelView& s, const PlanarView& d, int frac, cudaStream_t st)
{
    if (s.dtype == ENB_F32 || d.dtype == ENB_F32) {
        if (s.dtype != d.dtype) {
            return cudaErrorInvalidValue;
        }
        return launch_f_to_pyramid(FloatPixelView{(const float*)s.p, s.pitch, s.w, s.h, s.C, s.stride}, d, st);
    }
    note("to_fixed", npix(s.w, s.h) * s.C * esz(s.dtype) + planar_bytes(d));
    const dim3 g = row_grid(s.w, s.h);
    if (s.dtype == ENB_U8 && d.dtype == ENB_I16) {
        k_to_fixed<uint8_t, int16_t><<<g, 256, 0, st>>>((const uint8_t*)s.p, s.pitch, s.stride, s.C, (int16_t*)d.p,
                                                        d.pitch, d.plane, s.w, s.h, frac);
    } else if (s.dtype == ENB_U8 && d.dtype == ENB_I32) {
        k_to_fixed<uint8_t, int32_t><<<g, 256, 0, st>>>((const uint8_t*)s.p, s.pitch, s.stride, s.C, (int32_t*)d.p,
                                                        d.pitch, d.plane, s.w, s.h, frac);
    } else if (s.dtype == ENB_U16 && d.dtype == ENB_I32) {
        k_to_fixed<uint16_t, int32_t><<<g, 256, 0, st>>>((const uint16_t*)s.p, s.pitch, s.stride, s.C,
                                                         (int32_t*)d.p, d.pitch, d.plane, s.w, s.h, frac);
    } else if (s.dtype == ENB_U16 && d.dtype == ENB_I16) {
        k_to_fixed<uint16_t, int16_t><<<g, 256, 0, st>>>((const uint16_t*)s.p, s.pitch, s.stride, s.C,
                                                         (int16_t*)d.p, d.pitch, d.plane, s.w, s.h, frac);
    } else {
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_bytes_to_fixed(const BytePlane& s, const PlanarView& d, int frac, cudaStream_t st)
{
    note("bytes_to_fixed", npix(s.w, s.h) + planar_bytes(d));
    const dim3 g = row_grid(s.w, s.h);
    if (d.dtype == ENB_I16) {
        k_bytes_to_fixed<int16_t><<<g, 256, 0, st>>>(s.p, s.pitch, (int16_t*)d.p, d.pitch, s.w, s.h, frac);
    } else {
        k_bytes_to_fixed<int32_t><<<g, 256, 0, st>>>(s.p, s.pitch, (int32_t*)d.p, d.pitch, s.w, s.h, frac);
    }
    return cudaGetLastError();
}

cudaError_t launch_float_to_fixed(const FloatPlane& s, const PlanarView& d, int frac, cudaStream_t st)
{
    note("float_to_fixed", 4.0 * npix(s.w, s.h) + planar_bytes(d));
    const dim3 g = row_grid(s.w, s.h);
    if (d.dtype == ENB_I16) {
        k_float_to_fixed<int16_t><<<g, 256, 0, st>>>(s.p, s.pitch, (int16_t*)d.p, d.pitch, s.w, s.h, frac);
    } else {
        k_float_to_fixed<int32_t><<<g, 256, 0, st>>>(s.p, s.pitch, (int32_t*)d.p, d.pitch, s.w, s.h, frac);
    }
    return cudaGetLastError();
}

cudaError_t launch_soft_mask_to_fixed(const FloatPlane& m, const FloatPlane& n, int K, const PlanarView& d,
                                      int frac, cudaStream_t st)
{
    note("soft_mask_to_fixed", 8.0 * npix(m.w, m.h) + planar_bytes(d));
    const dim3 g = row_grid(m.w, m.h);
    const float fallback = (float)(255 / K);  // integer division, src/enfuse.h:1534
    if (d.dtype == ENB_I16) {
        k_soft_mask_to_fixed<int16_t><<<g, 256, 0, st>>>(m.p, m.pitch, n.p, n.pitch, fallback, (int16_t*)d.p, d.pitch,
                                                         m.w, m.h, frac);
    } else {
        k_soft_mask_to_fixed<int32_t><<<g, 256, 0, st>>>(m.p, m.pitch, n.p, n.pitch, fallback, (int32_t*)d.p, d.pitch,
                                                         m.w, m.h, frac);
    }
    return cudaGetLastError();
}

cudaError_t launch_alpha_extract(const AlphaSrc& a, const BytePlane& d, cudaStream_t st)
{
    note("alpha_extract", npix(d.w, d.h) * (a.mode == kAlphaChannel3 ? 1.0 + esz(a.pix.dtype) : 1.0));
    k_alpha_extract<<<row_grid(d.w, d.h), 256, 0, st>>>(a, d.p, d.pitch, d.w, d.h);
    return cudaGetLastError();
}

template <typename TS, typename TD, int C>
static void reduce_dispatch(int wrap, int n, const PlanarView* const* s, const BytePlane* const* sa,
                            const PlanarView* const* d, const BytePlane* const* da, cudaStream_t st)
{
    if (sa[0]) {
        using Src = PlanarSource<TS, C, true>;
        ReduceJobs<Src, TD> jobs{};
        for (int i = 0; i < 2; ++i) {
            const int k = i < n ? i : 0;
            jobs.j[i] = ReduceJob<Src, TD>{Src{(const TS*)s[k]->p, s[k]->pitch, s[k]->plane, sa[k]->p, sa[k]->pitch},
                                           (TD*)d[k]->p, d[k]->pitch, d[k]->plane, da[k]->p, da[k]->pitch};
        }
        launch_reduce_jobs<Src, TD, C, true>(jobs, n, s[0]->w, s[0]->h, d[0]->w, d[0]->h, wrap, st);
    } else {
        using Src = PlanarSource<TS, C, false>;
        ReduceJobs<Src, TD> jobs{};
        for (int i = 0; i < 2; ++i) {
            const int k = i < n ? i : 0;
            jobs.j[i] = ReduceJob<Src, TD>{Src{(const TS*)s[k]->p, s[k]->pitch, s[k]->plane, nullptr, 0},
                                           (TD*)d[k]->p, d[k]->pitch, d[k]->plane, nullptr, 0};
        }
        launch_reduce_jobs<Src, TD, C, false>(jobs, n, s[0]->w, s[0]->h, d[0]->w, d[0]->h, wrap, st);
    }
}

static cudaError_t reduce_jobs(int wrap, int n, const PlanarView* const* s, const BytePlane* const* sa,
                               const PlanarView* const* d, const BytePlane* const* da, cudaStream_t st)
{
    double bytes = 0.0;
    for (int i = 0; i < n; ++i) {
        if (s[i]->dtype != d[i]->dtype || s[i]->C != d[i]->C || (sa[i] == nullptr) != (da[i] == nullptr)) {
            return cudaErrorInvalidValue;
        }
        bytes += planar_bytes(*s[i]) + planar_bytes(*d[i]) +
                 (sa[i] ? npix(s[i]->w, s[i]->h) + npix(d[i]->w, d[i]->h) : 0.0);
    }
    note(sa[0] ? "reduce_alpha" : "reduce", bytes);
    if (s[0]->dtype == ENB_F32) {
        if (s[0]->C == 1) {
            reduce_dispatch<float, float, 1>(wrap, n, s, sa, d, da, st);
        } else {
            reduce_dispatch<float, float, 3>(wrap, n, s, sa, d, da, st);
        }
    } else if (s[0]->dtype == ENB_I16) {
        if (s[0]->C == 1) {
            reduce_dispatch<int16_t, int16_t, 1>(wrap, n, s, sa, d, da, st);
        } else {
            reduce_dispatch<int16_t, int16_t, 3>(wrap, n, s, sa, d, da, st);
        }
    } else {
        if (s[0]->C == 1) {
            reduce_dispatch<int32_t, int32_t, 1>(wrap, n, s, sa, d, da, st);
        } else {
            reduce_dispatch<int32_t, int32_t, 3>(wrap, n, s, sa, d, da, st);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_reduce(int wrap, const PlanarView& s, const BytePlane* sa, const PlanarView& d,
                          const BytePlane* da, cudaStream_t st)
{
    const PlanarView* sv[1] = {&s};
    const PlanarView* dv[1] = {&d};
    const BytePlane* sav[1] = {sa};
    const BytePlane* dav[1] = {da};
    return reduce_jobs(wrap, 1, sv, sav, dv, dav, st);
}

cudaError_t launch_reduce2(int wrap, const PlanarView& s0, const BytePlane* sa0, const PlanarView& d0,
                           const BytePlane* da0, const PlanarView& s1, const BytePlane* sa1, const PlanarView& d1,
                           const BytePlane* da1, cudaStream_t st)
{
    const bool same = s0.w == s1.w && s0.h == s1.h && d0.w == d1.w && d0.h == d1.h && s0.dtype == s1.dtype &&
                      s0.C == s1.C && d0.dtype == d1.dtype && d0.C == d1.C && (sa0 == nullptr) == (sa1 == nullptr) &&
                      (da0 == nullptr) == (da1 == nullptr);
    if (!same) {
        const cudaError_t e = launch_reduce(wrap, s0, sa0, d0, da0, st);
        return e != cudaSuccess ? e : launch_reduce(wrap, s1, sa1, d1, da1, st);
    }
    const PlanarView* sv[2] = {&s0, &s1};
    const PlanarView* dv[2] = {&d0, &d1};
    const BytePlane* sav[2] = {sa0, sa1};
    const BytePlane* dav[2] = {da0, da1};
    return reduce_jobs(wrap, 2, sv, sav, dv, dav, st);
}

template <typename T, typename TM, int C>
static void reduce_img2_mask_t(int wrap, const PlanarView& s0, const BytePlane& sa0, const PlanarView& d0,
                               const BytePlane& da0, const PlanarView& s1, const BytePlane& sa1, const PlanarView& d1,
                               const BytePlane& da1, const PlanarView& ms, const PlanarView& md, cudaStream_t st)
{
    using SrcI = PlanarSource<T, C, true>;
    using SrcM = PlanarSource<TM, 1, false>;
    ReduceJobs<SrcI, T> img{};
    img.j[0] = ReduceJob<SrcI, T>{SrcI{(const T*)s0.p, s0.pitch, s0.plane, sa0.p, sa0.pitch}, (T*)d0.p, d0.pitch,
                                  d0.plane, da0.p, da0.pitch};
    img.j[1] = ReduceJob<SrcI, T>{SrcI{(const T*)s1.p, s1.pitch, s1.plane, sa1.p, sa1.pitch}, (T*)d1.p, d1.pitch,
                                  d1.plane, da1.p, da1.pitch};
    const ReduceJob<SrcM, TM> msk{SrcM{(const TM*)ms.p, ms.pitch, ms.plane, nullptr, 0}, (TM*)md.p, md.pitch, md.plane,
                                  nullptr, 0};
    const dim3 g((unsigned)((d0.w + RDW - 1) / RDW), (unsigned)reduce_tile_rows(d0.h), 3u);
    (void)launch_pdl(k_reduce_img2_mask<SrcI, T, C, SrcM, TM>, g, dim3(RTHREADS), st, img, msk, s0.w, s0.h, d0.w,
                     d0.h, wrap);
}

cudaError_t launch_reduce_img2_mask(int wrap, const PlanarView& s0, const BytePlane& sa0, const PlanarView& d0,
                                    const BytePlane& da0, const PlanarView& s1, const BytePlane& sa1,
                                    const PlanarView& d1, const BytePlane& da1, const PlanarView& ms,
                                    const PlanarView& md, cudaStream_t st)
{
    const bool same = s0.w == s1.w && s0.h == s1.h && s0.w == ms.w && s0.h == ms.h && d0.w == d1.w && d0.h == d1.h &&
                      d0.w == md.w && d0.h == md.h && s0.dtype == s1.dtype && s0.dtype == d0.dtype &&
                      d1.dtype == d0.dtype && s0.C == s1.C && s0.C == d0.C && d1.C == d0.C && ms.C == 1 && md.C == 1 &&
                      ms.dtype == md.dtype && (s0.dtype == ENB_I16 || s0.dtype == ENB_I32) &&
                      (ms.dtype == ENB_I16 || ms.dtype == ENB_I32) && (s0.C == 1 || s0.C == 3);
    if (!same) {
        return cudaErrorInvalidValue;
    }
    note("reduce_level", planar_bytes(s0) + planar_bytes(d0) + planar_bytes(s1) + planar_bytes(d1) +
                             2.0 * (npix(s0.w, s0.h) + npix(d0.w, d0.h)) + planar_bytes(ms) + planar_bytes(md));
#define ENB_RIM(T, TM, CC) reduce_img2_mask_t<T, TM, CC>(wrap, s0, sa0, d0, da0, s1, sa1, d1, da1, ms, md, st)
    const bool m16 = ms.dtype == ENB_I16;
    if (s0.dtype == ENB_I16) {
        if (s0.C == 1) {
            if (m16) ENB_RIM(int16_t, int16_t, 1); else ENB_RIM(int16_t, int32_t, 1);
        } else {
            if (m16) ENB_RIM(int16_t, int16_t, 3); else ENB_RIM(int16_t, int32_t, 3);
        }
    } else {
        if (s0.C == 1) {
            if (m16) ENB_RIM(int32_t, int16_t, 1); else ENB_RIM(int32_t, int32_t, 1);
        } else {
            if (m16) ENB_RIM(int32_t, int16_t, 3); else ENB_RIM(int32_t, int32_t, 3);
        }
    }
#undef ENB_RIM
    return cudaGetLastError();
}

template <typename T, int C>
static void expand_dispatch(int add, int wrap, const PlanarView& s, const PlanarView& d, cudaStream_t st)
{
    const dim3 g = grid2d(d.w, d.h, ETW, ETH);
    if (add) {
        k_expand<T, C, true><<<g, 256, 0, st>>>((const T*)s.p, s.pitch, s.plane, s.w, s.h, (T*)d.p, d.pitch, d.plane,
                                                d.w, d.h, wrap);
    } else {
        k_expand<T, C, false><<<g, 256, 0, st>>>((const T*)s.p, s.pitch, s.plane, s.w, s.h, (T*)d.p, d.pitch, d.plane,
                                                 d.w, d.h, wrap);
    }
}

cudaError_t launch_expand(int add, int wrap, const PlanarView& s, const PlanarView& d, cudaStream_t st)
{
    if (s.dtype != d.dtype || s.C != d.C) {
        return cudaErrorInvalidValue;
    }
    if (s.dtype == ENB_F32) {
        return launch_f_expand(add, wrap, s, d, st);
    }
    note(add ? "expand_add" : "expand_sub", planar_bytes(s) + 2.0 * planar_bytes(d));
    if (s.dtype == ENB_I16) {
        if (s.C == 1) {
            expand_dispatch<int16_t, 1>(add, wrap, s, d, st);
        } else {
            expand_dispatch<int16_t, 3>(add, wrap, s, d, st);
        }
    } else {
        if (s.C == 1) {
            expand_dispatch<int32_t, 1>(add, wrap, s, d, st);
        } else {
            expand_dispatch<int32_t, 3>(add, wrap, s, d, st);
        }
    }
    return cudaGetLastError();
}

template <typename T, typename TM, int C>
static void blend_dispatch(const PlanarView& m, const PlanarView& wt, const PlanarView& b, int32_t wv,
                           cudaStream_t st)
{
    k_blend<T, TM, C><<<row_grid(b.w, b.h), 256, 0, st>>>((const TM*)m.p, m.pitch, (const T*)wt.p, wt.pitch, wt.plane,
                                                          (T*)b.p, b.pitch, b.plane, b.w, b.h, wv);
}

cudaError_t launch_blend(const PlanarView& m, const PlanarView& wt, const PlanarView& b, int32_t wv,
                         cudaStream_t st)
{
    if (wt.dtype != b.dtype || wt.C != b.C) {
        return cudaErrorInvalidValue;
    }
    if (b.dtype == ENB_F32) {
        return m.dtype == ENB_I32 ? launch_f_blend(m, wt, b, wv, st) : cudaErrorInvalidValue;
    }
    note("blend", planar_bytes(m) + planar_bytes(wt) + 2.0 * planar_bytes(b));
    const bool m16 = m.dtype == ENB_I16;
    if (b.dtype == ENB_I16) {
        if (b.C == 1) {
            m16 ? blend_dispatch<int16_t, int16_t, 1>(m, wt, b, wv, st) : blend_dispatch<int16_t, int32_t, 1>(m, wt, b, wv, st);
        } else {
            m16 ? blend_dispatch<int16_t, int16_t, 3>(m, wt, b, wv, st) : blend_dispatch<int16_t, int32_t, 3>(m, wt, b, wv, st);
        }
    } else {
        if (b.C == 1) {
            m16 ? blend_dispatch<int32_t, int16_t, 1>(m, wt, b, wv, st) : blend_dispatch<int32_t, int32_t, 1>(m, wt, b, wv, st);
        } else {
            m16 ? blend_dispatch<int32_t, int16_t, 3>(m, wt, b, wv, st) : blend_dispatch<int32_t, int32_t, 3>(m, wt, b, wv, st);
        }
    }
    return cudaGetLastError();
}

template <typename T, typename TM, int C>
static void mma_dispatch(const PlanarView& lp, const PlanarView& m, int32_t divisor, const PlanarView& r, int acc,
                         cudaStream_t st)
{
    const dim3 g = row_grid(lp.w, lp.h);
    if (divisor == (255 << 15)) {
        k_mask_mul_acc<T, TM, C, 15><<<g, 256, 0, st>>>((const T*)lp.p, lp.pitch, lp.plane, (const TM*)m.p, m.pitch,
                                                        (T*)r.p, r.pitch, r.plane, lp.w, lp.h, acc);
    } else if (divisor == (255 << 7)) {
        k_mask_mul_acc<T, TM, C, 7><<<g, 256, 0, st>>>((const T*)lp.p, lp.pitch, lp.plane, (const TM*)m.p, m.pitch,
                                                       (T*)r.p, r.pitch, r.plane, lp.w, lp.h, acc);
    } else {
        k_mask_mul_acc_generic<T, TM, C><<<g, 256, 0, st>>>((const T*)lp.p, lp.pitch, lp.plane, (const TM*)m.p,
                                                            m.pitch, divisor, (T*)r.p, r.pitch, r.plane, lp.w, lp.h,
                                                            acc);
    }
}

cudaError_t launch_mask_mul_acc(const PlanarView& lp, const PlanarView& m, int32_t divisor, const PlanarView& r,
                                int acc, cudaStream_t st)
{
    if (lp.dtype != r.dtype || lp.C != r.C) {
        return cudaErrorInvalidValue;
    }
    if (lp.dtype == ENB_F32) {
        return m.dtype == ENB_I32 ? launch_f_mask_mul_acc(lp, m, divisor, r, acc, st) : cudaErrorInvalidValue;
    }
    note("mask_mul_acc", planar_bytes(lp) + planar_bytes(m) + (acc ? 2.0 : 1.0) * planar_bytes(r));
    const bool m16 = m.dtype == ENB_I16;
    if (lp.dtype == ENB_I16) {
        if (lp.C == 1) {
            m16 ? mma_dispatch<int16_t, int16_t, 1>(lp, m, divisor, r, acc, st) : mma_dispatch<int16_t, int32_t, 1>(lp, m, divisor, r, acc, st);
        } else {
            m16 ? mma_dispatch<int16_t, int16_t, 3>(lp, m, divisor, r, acc, st) : mma_dispatch<int16_t, int32_t, 3>(lp, m, divisor, r, acc, st);
        }
    } else {
        if (lp.C == 1) {
            m16 ? mma_dispatch<int32_t, int16_t, 1>(lp, m, divisor, r, acc, st) : mma_dispatch<int32_t, int32_t, 1>(lp, m, divisor, r, acc, st);
        } else {
            m16 ? mma_dispatch<int32_t, int16_t, 3>(lp, m, divisor, r, acc, st) : mma_dispatch<int32_t, int32_t, 3>(lp, m, divisor, r, acc, st);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_from_fixed(const PlanarView& s, const BytePlane& a, void* dst, int64_t dpitch, int ddtype,
                              int dstride, int frac, int dither, uint64_t seed, cudaStream_t st)
{
    if (s.dtype == ENB_F32 || ddtype == ENB_F32) {
        if (s.dtype != ddtype) {
            return cudaErrorInvalidValue;
        }
        return launch_f_from_pyramid(s, a, (float*)dst, dpitch, dstride, st);
    }
    note("from_fixed", planar_bytes(s) + npix(s.w, s.h) * (1.0 + s.C * esz(ddtype)));
    const dim3 g = row_grid(s.w, s.h);
    if (s.dtype == ENB_I16) {
        if (ddtype == ENB_U8) {
            k_from_fixed<int16_t, uint8_t><<<g, 256, 0, st>>>((const int16_t*)s.p, s.pitch, s.plane, s.C, a.p, a.pitch,
                                                              (uint8_t*)dst, dpitch, dstride, s.w, s.h, frac, dither,
                                                              seed, 255);
        } else {
            k_from_fixed<int16_t, uint16_t><<<g, 256, 0, st>>>((const int16_t*)s.p, s.pitch, s.plane, s.C, a.p, a.pitch,
                                                               (uint16_t*)dst, dpitch, dstride, s.w, s.h, frac, dither,
                                                               seed, 65535);
        }
    } else {
        if (ddtype == ENB_U8) {
            k_from_fixed<int32_t, uint8_t><<<g, 256, 0, st>>>((const int32_t*)s.p, s.pitch, s.plane, s.C, a.p, a.pitch,
                                                              (uint8_t*)dst, dpitch, dstride, s.w, s.h, frac, dither,
                                                              seed, 255);
        } else {
            k_from_fixed<int32_t, uint16_t><<<g, 256, 0, st>>>((const int32_t*)s.p, s.pitch, s.plane, s.C, a.p, a.pitch,
                                                               (uint16_t*)dst, dpitch, dstride, s.w, s.h, frac, dither,
                                                               seed, 65535);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_copy_pixels(const PixelView& s, void* dst, int64_t dpitch, cudaStream_t st)
{
    const int rowlen = s.w * s.stride;
    note("copy_pixels", 2.0 * npix(rowlen, s.h) * esz(s.dtype));
    const dim3 g = row_grid(rowlen, s.h);
    if (s.dtype == ENB_U8) {
        k_copy_pixels<uint8_t><<<g, 256, 0, st>>>((const uint8_t*)s.p, s.pitch, (uint8_t*)dst, dpitch, rowlen, s.h);
    } else if (s.dtype == ENB_F32) {
        k_copy_pixels<uint32_t><<<g, 256, 0, st>>>((const uint32_t*)s.p, s.pitch, (uint32_t*)dst, dpitch, rowlen, s.h);
    } else {
        k_copy_pixels<uint16_t><<<g, 256, 0, st>>>((const uint16_t*)s.p, s.pitch, (uint16_t*)dst, dpitch, rowlen, s.h);
    }
    return cudaGetLastError();
}

cudaError_t launch_alpha_component(const BytePlane& a, void* dst, int64_t dpitch, int ddtype, cudaStream_t st)
{
    note("alpha_component", npix(a.w, a.h) * (1.0 + esz(ddtype)));
    const dim3 g = row_grid(a.w, a.h);
    if (ddtype == ENB_U8) {
        k_alpha_component<uint8_t><<<g, 256, 0, st>>>(a.p, a.pitch, (uint8_t*)dst, dpitch, a.w, a.h, (uint8_t)255);
    } else if (ddtype == ENB_F32) {
        // AlphaTraits<float>::max() = 1.0 (src/numerictraits.h:247)
        k_alpha_component<float><<<g, 256, 0, st>>>(a.p, a.pitch, (float*)dst, dpitch, a.w, a.h, 1.0f);
    } else {
        k_alpha_component<uint16_t><<<g, 256, 0, st>>>(a.p, a.pitch, (uint16_t*)dst, dpitch, a.w, a.h, (uint16_t)65535);
    }
    return cudaGetLastError();
}

cudaError_t launch_copy_level0(const PlanarView& s, int32_t* dst, cudaStream_t st)
{
    if (s.dtype == ENB_F32) {
        return launch_f_copy_level0(s, reinterpret_cast<float*>(dst), st);
    }
    note("copy_level0", planar_bytes(s) + 4.0 * npix(s.w, s.h) * s.C);
    const dim3 g = row_grid(s.w, s.h);
    if (s.dtype == ENB_I16) {
        k_copy_level0<int16_t><<<g, 256, 0, st>>>((const int16_t*)s.p, s.pitch, s.plane, s.C, dst, s.w, s.h);
    } else {
        k_copy_level0<int32_t><<<g, 256, 0, st>>>((const int32_t*)s.p, s.pitch, s.plane, s.C, dst, s.w, s.h);
    }
    return cudaGetLastError();
}

cudaError_t launch_enfuse_mask(const PixelView& img, const AlphaSrc& alpha, const WeightParams& wp,
                               const WeightTables& tab, const FloatPlane& out, cudaStream_t st)
{
    const int TW = EMX + 2 * emask_halo_x(wp), TH = EMY + 2 * iweight_halo(wp);
    const size_t smem = ((itile_bytes_rect(TW, TH) + 15) & ~(size_t)15) + 32 * sizeof(long long);
    note("enfuse_mask", npix(img.w, img.h) * (img.stride * esz(img.dtype) + (alpha.mode == kAlphaPlane ? 1.0 : 0.0) + 4.0));
    if (smem > 48 * 1024) {
        cudaFuncSetAttribute(k_enfuse_mask, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    k_enfuse_mask<<<grid2d(img.w, img.h, EMX, EMY), 256, smem, st>>>(img, alpha, wp, tab, out.p, out.pitch);
    return cudaGetLastError();
}

cudaError_t launch_norm_accumulate(const FloatPlane& m, const FloatPlane& n, int first, cudaStream_t st)
{
    note("norm_accumulate", npix(m.w, m.h) * (first ? 8.0 : 12.0));
    k_norm_accumulate<<<row_grid(m.w, m.h), 256, 0, st>>>(m.p, m.pitch, n.p, n.pitch, m.w, m.h, first);
    return cudaGetLastError();
}

cudaError_t launch_union_alpha(const BytePlane& a, const BytePlane& u, int first, cudaStream_t st)
{
    note("union_alpha", npix(a.w, a.h) * (first ? 2.0 : 3.0));
    k_union_alpha<<<row_grid(a.w, a.h), 256, 0, st>>>(a.p, a.pitch, u.p, u.pitch, a.w, a.h, first);
    return cudaGetLastError();
}

cudaError_t launch_hard_mask(const FloatPlane* masks, int K, cudaStream_t st)
{
    if (K > kMaxHardMasks) {
        return cudaErrorInvalidValue;
    }
    note("hard_mask", 8.0 * K * npix(masks[0].w, masks[0].h));
    HardMaskArgs a;
    for (int k = 0; k < K; ++k) {
        a.p[k] = masks[k].p;
        a.pitch[k] = masks[k].pitch;
    }
    k_hard_mask<<<row_grid(masks[0].w, masks[0].h), 256, 0, st>>>(a, K, masks[0].w, masks[0].h);
    return cudaGetLastError();
}

}  // namespace enb
