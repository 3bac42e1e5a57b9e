// enb_coarse.cu -- the coarse end of the enblend pyramid blend in one launch.
//
// Below a few tens of thousands of pixels a pyramid level is too small to
// fill the GPU: a launch per level and pyramid costs more in launch latency,
// instruction fetch and the dependent load chain of a lone CTA than the level
// costs in memory traffic.  One cluster of CTAs therefore runs every coarse
// level of the blend in a single launch, separated by hardware cluster
// barriers (barrier.cluster, no software spin):
//   1. the Gaussian levels of the white and black images (with alpha) and of
//      the seam mask (without) down to the top (src/enblend.h:384-446,
//      gaussianPyramid, src/pyramid.h:1500-1610);
//   2. the top level blend, R_top = blend(M, Gw, Gb) (src/blend.h:81-121);
//   3. for each coarse level l, top-1 down to the finest level produced here:
//      R_l = fromPromote(blend(M_l, Gw_l - E(Gw_{l+1}), Gb_l - E(Gb_{l+1}))
//                        + E(R_{l+1}))
//      (Laplacians, blend and collapse, src/pyramid.h:1758-1784).
// The finer levels stay with the tiled kernels.  Each thread computes whole
// destination pixels with the reference's integer arithmetic (the same
// operations as the tiled kernels): normalised 5x5 reduce over opaque taps,
// clamp-to-edge reduce of the mask, expansion with the border weights of
// expand_hweights / expand_vweights.  Every level is read only after the
// barrier that follows its last write, and no SM touches a level before it is
// written, so plain (L1-cached) loads see the written values; the read-only
// (non-coherent) load path is never used for them.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>

#include "enb_device.cuh"
#include "enb_internal.h"

namespace enb {

namespace cg = cooperative_groups;

constexpr int kCoarseThreads = 1024;

struct CoarseArgs {
    // slot 0: the finest level (input); slots 1..n-1: produced here
    char* gw[kMaxLevels];
    char* gb[kMaxLevels];
    char* rr[kMaxLevels];
    char* mg[kMaxLevels];
    uint8_t* aw[kMaxLevels];
    uint8_t* ab[kMaxLevels];
    int64_t pitch[kMaxLevels], plane[kMaxLevels];  // elements of T (gw, gb, rr)
    int64_t mpitch[kMaxLevels];                    // elements of TM
    int64_t apitch[kMaxLevels];                    // bytes (aw, ab)
    int w[kMaxLevels], h[kMaxLevels];
    int n;
    int32_t white_value;
    int wrap;
};

template <typename T>
__device__ __forceinline__ T ld_level(const T* p)
{
    return *p;
}

__device__ __forceinline__ int tap5(int k) { return k == 2 ? 6 : ((k & 1) ? 4 : 1); }

// Reduce with alpha of one destination pixel (X, Y).
template <typename T, int C>
__device__ __forceinline__ void coarse_reduce_alpha(const T* s, int64_t sp, int64_t spl, const uint8_t* sa,
                                                    int64_t sap, int sw, int sh, T* d, int64_t dp, int64_t dpl,
                                                    uint8_t* da, int64_t dap, int X, int Y, int wrap)
{
    int32_t num[C];
#pragma unroll
    for (int c = 0; c < C; ++c) {
        num[c] = 0;
    }
    int32_t den = 0;
#pragma unroll
    for (int a = 0; a < 5; ++a) {
        const int gy = 2 * Y - 2 + a;
        const bool rok = gy >= 0 && gy < sh;
        const int gyc = min(max(gy, 0), sh - 1);
#pragma unroll
        for (int b = 0; b < 5; ++b) {
            int gx = 2 * X - 2 + b;
            bool ok = rok;
            if (wrap) {
                gx = imod(gx, sw);
            } else {
                ok = ok && gx >= 0 && gx < sw;
                gx = min(max(gx, 0), sw - 1);
            }
            const int64_t o = (int64_t)gyc * sp + gx;
            // unconditional load from the clamped position, dropped afterwards
            const uint8_t al = ld_level(&sa[(int64_t)gyc * sap + gx]);
            const int32_t wt = (ok && al != 0) ? tap5(a) * tap5(b) : 0;
            den += wt;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                num[c] += wt * (int32_t)ld_level(&s[c * spl + o]);
            }
        }
    }
    const int64_t o = (int64_t)Y * dp + X;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        d[c * dpl + o] = den <= 0 ? (T)0 : cast_store<T>(den == 256 ? num[c] / 256 : div_any(num[c], den));
    }
    da[(int64_t)Y * dap + X] = den > 0 ? 255 : 0;
}

// Alpha-free (clamp-to-edge) reduce of one mask pixel.
template <typename TM>
__device__ __forceinline__ void coarse_reduce_mask(const TM* s, int64_t sp, int sw, int sh, TM* d, int64_t dp, int X,
                                                   int Y, int wrap)
{
    int32_t num = 0;
#pragma unroll
    for (int a = 0; a < 5; ++a) {
        const int gy = min(max(2 * Y - 2 + a, 0), sh - 1);
        const TM* row = s + (int64_t)gy * sp;
        int32_t hs = 0;
#pragma unroll
        for (int b = 0; b < 5; ++b) {
            const int t = 2 * X - 2 + b;
            const int gx = wrap ? imod(t, sw) : min(max(t, 0), sw - 1);
            hs += tap5(b) * (int32_t)ld_level(&row[gx]);
        }
        num += tap5(a) * hs;
    }
    d[(int64_t)Y * dp + X] = cast_store<TM>(num / 256);
}

// Source taps and weights of the expansion at destination pixel (X, Y); taps
// of weight 0 point at a valid sample so that every load is unconditional.
struct ExpandTaps {
    int jj[3], ii[3], vw[3], hw[3], den;
};

__device__ __forceinline__ ExpandTaps expand_taps(int X, int Y, int sw, int sh, int dw, int wrap)
{
    ExpandTaps t;
    int vden, hden;
    expand_vweights(Y, sh, t.vw, vden);
    expand_hweights(X, sw, dw, wrap, t.hw, hden);
    t.den = vden * hden;
    const int i = X >> 1, j = Y >> 1;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        t.jj[k] = min(max(j - 1 + k, 0), sh - 1);
        const int c = i - 1 + k;
        t.ii[k] = wrap ? imod(c, sw) : min(max(c, 0), sw - 1);
    }
    return t;
}

template <typename T>
__device__ __forceinline__ int32_t expand_at(const T* s, int64_t pitch, const ExpandTaps& t)
{
    int32_t num = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T* row = s + (int64_t)t.jj[a] * pitch;
        num += t.vw[a] * (t.hw[0] * (int32_t)ld_level(&row[t.ii[0]]) + t.hw[1] * (int32_t)ld_level(&row[t.ii[1]]) +
                          t.hw[2] * (int32_t)ld_level(&row[t.ii[2]]));
    }
    return div_den(num, t.den);
}

__device__ __forceinline__ void coarse_sync(cg::cluster_group& cluster)
{
    __threadfence();
    cluster.sync();
}

// Launched as one cluster (16 CTAs where the GPU allows that cluster size,
// else the portable 8) of kCoarseThreads threads.
template <typename T, typename TM, int C>
__global__ void __launch_bounds__(kCoarseThreads, 1) k_coarse(CoarseArgs a)
{
    cg::cluster_group cluster = cg::this_cluster();
    const int nt = (int)cluster.num_blocks() * kCoarseThreads;
    const int gt = (int)cluster.block_rank() * kCoarseThreads + (int)threadIdx.x;
    const int32_t W = a.white_value;

    // 1. Gaussian levels 1..n-1 of the white, black and mask pyramids
    for (int l = 1; l < a.n; ++l) {
        const int dw = a.w[l], dh = a.h[l], sw = a.w[l - 1], sh = a.h[l - 1];
        const int np = dw * dh;
        for (int k = gt; k < 3 * np; k += nt) {
            const int job = k / np;
            const int p = k - job * np;
            const int Y = p / dw, X = p - Y * dw;
            if (job < 2) {
                const T* s = reinterpret_cast<const T*>(job == 0 ? a.gw[l - 1] : a.gb[l - 1]);
                T* d = reinterpret_cast<T*>(job == 0 ? a.gw[l] : a.gb[l]);
                coarse_reduce_alpha<T, C>(s, a.pitch[l - 1], a.plane[l - 1], job == 0 ? a.aw[l - 1] : a.ab[l - 1],
                                          a.apitch[l - 1], sw, sh, d, a.pitch[l], a.plane[l],
                                          job == 0 ? a.aw[l] : a.ab[l], a.apitch[l], X, Y, a.wrap);
            } else {
                coarse_reduce_mask<TM>(reinterpret_cast<const TM*>(a.mg[l - 1]), a.mpitch[l - 1], sw, sh,
                                       reinterpret_cast<TM*>(a.mg[l]), a.mpitch[l], X, Y, a.wrap);
            }
        }
        coarse_sync(cluster);
    }

    // 2. top level: R = blend(M, Gw, Gb)
    {
        const int l = a.n - 1;
        const int dw = a.w[l], np = dw * a.h[l];
        const T* gw = reinterpret_cast<const T*>(a.gw[l]);
        const T* gb = reinterpret_cast<const T*>(a.gb[l]);
        T* rr = reinterpret_cast<T*>(a.rr[l]);
        const TM* mg = reinterpret_cast<const TM*>(a.mg[l]);
        for (int p = gt; p < np; p += nt) {
            const int Y = p / dw, X = p - Y * dw;
            const int32_t m = (int32_t)ld_level(&mg[(int64_t)Y * a.mpitch[l] + X]);
            const int64_t o = (int64_t)Y * a.pitch[l] + X;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                rr[c * a.plane[l] + o] = (T)blend_sample<T>(m, W, (int32_t)ld_level(&gw[c * a.plane[l] + o]),
                                                            (int32_t)ld_level(&gb[c * a.plane[l] + o]));
            }
        }
    }

    // 3. Laplacians + blend + collapse, levels n-2 .. 1
    for (int l = a.n - 2; l >= 1; --l) {
        coarse_sync(cluster);
        const int dw = a.w[l], np = dw * a.h[l];
        const int sw = a.w[l + 1], sh = a.h[l + 1];
        const T* gw = reinterpret_cast<const T*>(a.gw[l]);
        const T* gb = reinterpret_cast<const T*>(a.gb[l]);
        T* rr = reinterpret_cast<T*>(a.rr[l]);
        const TM* mg = reinterpret_cast<const TM*>(a.mg[l]);
        const T* cw = reinterpret_cast<const T*>(a.gw[l + 1]);
        const T* cb = reinterpret_cast<const T*>(a.gb[l + 1]);
        const T* cr = reinterpret_cast<const T*>(a.rr[l + 1]);
        for (int p = gt; p < np; p += nt) {
            const int Y = p / dw, X = p - Y * dw;
            const ExpandTaps t = expand_taps(X, Y, sw, sh, dw, a.wrap);
            const int32_t m = (int32_t)ld_level(&mg[(int64_t)Y * a.mpitch[l] + X]);
            const int64_t o = (int64_t)Y * a.pitch[l] + X;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const int64_t cpl = c * a.plane[l + 1];
                const int32_t ew = expand_at<T>(cw + cpl, a.pitch[l + 1], t);
                const int32_t eb = expand_at<T>(cb + cpl, a.pitch[l + 1], t);
                const int32_t er = expand_at<T>(cr + cpl, a.pitch[l + 1], t);
                const int32_t lw = (int32_t)cast_store<T>((int64_t)ld_level(&gw[c * a.plane[l] + o]) - ew);
                const int32_t lb = (int32_t)cast_store<T>((int64_t)ld_level(&gb[c * a.plane[l] + o]) - eb);
                rr[c * a.plane[l] + o] = sat_store<T>(blend_sample<T>(m, W, lw, lb) + er);
            }
        }
    }
}

// One cluster of 16 CTAs when the device can schedule it (non-portable size),
// otherwise 8; decided once per kernel instantiation.
static cudaError_t coarse_launch(void (*kernel)(CoarseArgs), const CoarseArgs& a, cudaStream_t st)
{
    static std::mutex mu;
    static std::map<void*, int> sizes;
    int cs = 8;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = sizes.find((void*)kernel);
        if (it == sizes.end()) {
            int n = 0;
            cudaLaunchConfig_t q{};
            cudaLaunchAttribute qa{};
            q.gridDim = dim3(16);
            q.blockDim = dim3(kCoarseThreads);
            qa.id = cudaLaunchAttributeClusterDimension;
            qa.val.clusterDim.x = 16;
            qa.val.clusterDim.y = 1;
            qa.val.clusterDim.z = 1;
            q.attrs = &qa;
            q.numAttrs = 1;
            if (cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
                cudaOccupancyMaxActiveClusters(&n, kernel, &q) == cudaSuccess && n > 0) {
                cs = 16;
            }
            (void)cudaGetLastError();
            sizes[(void*)kernel] = cs;
        } else {
            cs = it->second;
        }
    }
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr{};
    cfg.gridDim = dim3((unsigned)cs);
    cfg.blockDim = dim3(kCoarseThreads);
    cfg.stream = st;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = (unsigned)cs;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, a);
}

static double pbytes_c(const PlanarView& v) { return (double)v.w * v.h * v.C * (v.dtype == ENB_I16 ? 2.0 : 4.0); }

cudaError_t launch_coarse(const CoarseHost& h, cudaStream_t st)
{
    if (h.n < 2 || h.n > kMaxLevels) {
        return cudaErrorInvalidValue;
    }
    CoarseArgs a{};
    double bytes = 0.0;
    for (int l = 0; l < h.n; ++l) {
        if (h.gw[l].pitch != h.gb[l].pitch || h.gw[l].pitch != h.rr[l].pitch || h.gw[l].plane != h.gb[l].plane ||
            h.gw[l].plane != h.rr[l].plane || h.aw[l].pitch != h.ab[l].pitch) {
            return cudaErrorInvalidValue;
        }
        a.gw[l] = (char*)h.gw[l].p;
        a.gb[l] = (char*)h.gb[l].p;
        a.rr[l] = (char*)h.rr[l].p;
        a.mg[l] = (char*)h.mg[l].p;
        a.aw[l] = h.aw[l].p;
        a.ab[l] = h.ab[l].p;
        a.pitch[l] = h.gw[l].pitch;
        a.plane[l] = h.gw[l].plane;
        a.mpitch[l] = h.mg[l].pitch;
        a.apitch[l] = h.aw[l].pitch;
        a.w[l] = h.gw[l].w;
        a.h[l] = h.gw[l].h;
        const double px = (double)a.w[l] * a.h[l];
        // each level is written once and read by the next reduce, the top
        // blend or the up sweep: count its bytes twice (once for slot 0)
        bytes += (l == 0 ? 1.0 : 2.0) * (2.0 * pbytes_c(h.gw[l]) + 2.0 * px + pbytes_c(h.mg[l]));
        bytes += l >= 1 ? 2.0 * pbytes_c(h.rr[l]) : 0.0;
    }
    a.n = h.n;
    a.white_value = h.white_value;
    a.wrap = h.wrap;
    note_launch("coarse", bytes);
    const PlanarView& r = h.rr[0];
    const bool m16 = h.mg[0].dtype == ENB_I16;
#define ENB_CO(T, TM, CC) return coarse_launch(k_coarse<T, TM, CC>, a, st)
    if (r.dtype == ENB_I16) {
        if (r.C == 1) {
            if (m16) ENB_CO(int16_t, int16_t, 1); else ENB_CO(int16_t, int32_t, 1);
        } else {
            if (m16) ENB_CO(int16_t, int16_t, 3); else ENB_CO(int16_t, int32_t, 3);
        }
    } else {
        if (r.C == 1) {
            if (m16) ENB_CO(int32_t, int16_t, 1); else ENB_CO(int32_t, int32_t, 1);
        } else {
            if (m16) ENB_CO(int32_t, int16_t, 3); else ENB_CO(int32_t, int32_t, 3);
        }
    }
#undef ENB_CO
}

}  // namespace enb
