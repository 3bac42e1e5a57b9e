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
// The CTAs of the cluster share out the 64x16 tiles of each step and run the
// same tile code as the per-level kernels (reduce_tile, up_tile), so the
// integer results are theirs.  Every level is read only after the barrier that
// follows its last write, and no SM touches a level before it is written, so
// plain (L1-cached) loads see the written values; the read-only
// (non-coherent) load path is never used for them.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>

#include "enb_device.cuh"
#include "enb_internal.h"
#include "enb_reduce.cuh"
#include "enb_tiles.cuh"

namespace enb {

namespace cg = cooperative_groups;


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

__device__ __forceinline__ void coarse_sync(cg::cluster_group& cluster)
{
    __threadfence();
    cluster.sync();
}

constexpr int kCoarseThreads = RTHREADS;
constexpr int kCoarseWords = ReduceSmem<3, true>::WORDS;   // the largest tile buffer
static_assert(kCoarseWords * 4 >= 3 * ESH * ESW * 16, "up_tile staging fits the reduce buffer");

// Launched as one cluster (16 CTAs where the GPU allows that cluster size,
// else the portable 8) of kCoarseThreads threads.
template <typename T, typename TM, int C>
__global__ void __launch_bounds__(kCoarseThreads, 1) k_coarse(CoarseArgs a)
{
    __shared__ __align__(16) int32_t sm[kCoarseWords];
    int32_t (*V)[RDH][RVP] = reinterpret_cast<int32_t (*)[RDH][RVP]>(sm);
    int4 (*S4)[ESH][ESW] = reinterpret_cast<int4 (*)[ESH][ESW]>(sm);
    griddep_wait();
    griddep_launch();
    cg::cluster_group cluster = cg::this_cluster();
    const int nb = (int)cluster.num_blocks();
    const int rank = (int)cluster.block_rank();
    const int32_t W = a.white_value;
    using SrcI = PlanarSource<T, C, true, false>;
    using SrcM = PlanarSource<TM, 1, false, false>;

    // 1. Gaussian levels 1..n-1: white and black (with alpha), mask
    for (int l = 1; l < a.n; ++l) {
        const int dw = a.w[l], dh = a.h[l], sw = a.w[l - 1], sh = a.h[l - 1];
        const int tx = (dw + RDW - 1) / RDW, nt = tx * ((dh + RDH - 1) / RDH);
        for (int t = rank; t < 3 * nt; t += nb) {
            const int job = t / nt, tile = t - job * nt;
            const int X0 = (tile % tx) * RDW, Y0 = (tile / tx) * RDH;
            __syncthreads();  // the previous tile's readers of sm are done
            if (job < 2) {
                const ReduceJob<SrcI, T> rj{
                    SrcI{reinterpret_cast<const T*>(job == 0 ? a.gw[l - 1] : a.gb[l - 1]), a.pitch[l - 1],
                         a.plane[l - 1], job == 0 ? a.aw[l - 1] : a.ab[l - 1], a.apitch[l - 1]},
                    reinterpret_cast<T*>(job == 0 ? a.gw[l] : a.gb[l]), a.pitch[l], a.plane[l],
                    job == 0 ? a.aw[l] : a.ab[l], a.apitch[l]};
                reduce_tile<SrcI, T, C, true>(rj, X0, Y0, sw, sh, dw, dh, a.wrap, V);
            } else {
                const ReduceJob<SrcM, TM> rj{
                    SrcM{reinterpret_cast<const TM*>(a.mg[l - 1]), a.mpitch[l - 1], 0, nullptr, 0},
                    reinterpret_cast<TM*>(a.mg[l]), a.mpitch[l], 0, nullptr, 0};
                reduce_tile<SrcM, TM, 1, false>(rj, X0, Y0, sw, sh, dw, dh, a.wrap, V);
            }
        }
        coarse_sync(cluster);
    }

    // 2. top level: R = blend(M, Gw, Gb), one pixel per thread
    {
        const int l = a.n - 1;
        const int dw = a.w[l], np = dw * a.h[l];
        const T* gw = reinterpret_cast<const T*>(a.gw[l]);
        const T* gb = reinterpret_cast<const T*>(a.gb[l]);
        T* rr = reinterpret_cast<T*>(a.rr[l]);
        const TM* mg = reinterpret_cast<const TM*>(a.mg[l]);
        for (int p = rank * kCoarseThreads + (int)threadIdx.x; p < np; p += nb * kCoarseThreads) {
            const int Y = p / dw, X = p - Y * dw;
            const int32_t m = (int32_t)mg[(int64_t)Y * a.mpitch[l] + X];
            const int64_t o = (int64_t)Y * a.pitch[l] + X;
#pragma unroll
            for (int c = 0; c < C; ++c) {
                rr[c * a.plane[l] + o] =
                    (T)blend_sample<T>(m, W, (int32_t)gw[c * a.plane[l] + o], (int32_t)gb[c * a.plane[l] + o]);
            }
        }
    }

    // 3. Laplacians + blend + collapse, levels n-2 .. 1
    for (int l = a.n - 2; l >= 1; --l) {
        coarse_sync(cluster);
        CoarseLevels cl{};
#pragma unroll
        for (int c = 0; c < C; ++c) {
            cl.p[c] = reinterpret_cast<const T*>(a.gw[l + 1]) + c * a.plane[l + 1];
            cl.p[C + c] = reinterpret_cast<const T*>(a.gb[l + 1]) + c * a.plane[l + 1];
            cl.p[2 * C + c] = reinterpret_cast<const T*>(a.rr[l + 1]) + c * a.plane[l + 1];
        }
        cl.pitch = a.pitch[l + 1];
        cl.w = a.w[l + 1];
        cl.h = a.h[l + 1];
        const int dw = a.w[l], dh = a.h[l];
        const int tx = (dw + ETW - 1) / ETW, nt = tx * ((dh + ETH - 1) / ETH);
        for (int t = rank; t < nt; t += nb) {
            __syncthreads();  // the previous tile's readers of sm are done
            up_tile<T, TM, C, false, kCoarseThreads>(
                cl, reinterpret_cast<const TM*>(a.mg[l]), a.mpitch[l], reinterpret_cast<const T*>(a.gw[l]),
                reinterpret_cast<const T*>(a.gb[l]), reinterpret_cast<T*>(a.rr[l]), a.pitch[l], a.plane[l], dw, dh, W,
                a.wrap, (t % tx) * ETW, (t / tx) * ETH, S4);
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
    cudaLaunchAttribute attr[2];
    cfg.gridDim = dim3((unsigned)cs);
    cfg.blockDim = dim3(kCoarseThreads);
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
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
