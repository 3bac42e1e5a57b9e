// enb_nft.cu -- enblend's nearest-feature seam mask (src/nearest.h:427-553)
// on the GPU: the mask of `enblend --fine-mask --no-optimize`
// (src/mask.h:1101-1180), 255 where the nearest pixel that only the white
// image covers is nearer than the nearest pixel that only the black image
// covers, else 0.
//
// The distances are the Euclidean distance transform of Felzenszwalb and
// Huttenlocher as the reference's OpenMP build computes it
// (src/openmp_vigra.h:257-433): a 1-D lower envelope of parabolas along
// every column of the feature image (0 on features, FLT_MAX elsewhere), then
// along every row of that result, then sqrt.  Every float operation is the
// reference's, in its order and rounding (no contraction into fused
// multiply-adds), so the masks are bit-identical.  One thread walks one line
// (the envelope is sequential); its envelope (vertex indices v, boundaries
// z) lives in global scratch interleaved across the threads of a launch.
//
// Wrap-around (--wrap horizontal): the reference transforms the image
// doubled horizontally and keeps, for x < w/2, column w + x and, for the
// other columns, column x (src/nearest.h:136-342).
#include <cuda_runtime.h>
#include <float.h>
#include <math_constants.h>
#include <stdint.h>

#include "enb_internal.h"

namespace enb {

namespace {

// The 1-D transform of n samples f(q) (src/openmp_vigra.h:300-351); out(q,
// d) receives the squared distances.  v, z: this line's envelope in scratch
// with a stride of ss elements between consecutive entries.
template <class F, class Out>
__device__ __forceinline__ void fh_line(int n, const F& f, const Out& out, int* v, float* z, int64_t ss)
{
    int k = 0;
    v[0] = 0;
    z[0] = -CUDART_INF_F;
    z[ss] = CUDART_INF_F;
    for (int q = 1; q < n; ++q) {
        const float qf = (float)q;
        const float sum_q = __fadd_rn(f(q), __fmul_rn(qf, qf));
        int vk = v[k * ss];
        float s = __fdiv_rn(__fsub_rn(sum_q, __fadd_rn(f(vk), (float)(vk * vk))), (float)(2 * (q - vk)));
        while (s <= z[k * ss]) {
            --k;
            vk = v[k * ss];
            s = __fdiv_rn(__fsub_rn(sum_q, __fadd_rn(f(vk), (float)(vk * vk))), (float)(2 * (q - vk)));
        }
        ++k;
        v[k * ss] = q;
        z[k * ss] = s;
        z[(k + 1) * ss] = CUDART_INF_F;
    }
    k = 0;
    for (int q = 0; q < n; ++q) {
        while (z[(k + 1) * ss] < (float)q) {
            ++k;
        }
        const int vk = v[k * ss];
        out(q, __fadd_rn((float)((q - vk) * (q - vk)), f(vk)));
    }
}

struct NftArgs {
    const uint8_t* white;
    const uint8_t* black;
    int64_t wpitch, bpitch;
    int w, h;
    float* inter;        // [2][h][ipitch]: column pass of the two transforms
    int64_t ipitch;
    float* dist;         // [2][h][ipitch]: distances of the kept columns
    int* v;              // envelope scratch
    float* z;
    unsigned int* tally; // [2]: pixels only white covers, only black covers
    int wrap;
};

// Whether (x, y) is a feature of transform t: covered by the white image
// only (t = 0, saturating white - black != 0) or by the black one only.
__device__ __forceinline__ bool nft_feature(const NftArgs& a, int t, int x, int y)
{
    const uint8_t wv = a.white[(int64_t)y * a.wpitch + x], bv = a.black[(int64_t)y * a.bpitch + x];
    return t == 0 ? wv > bv : bv > wv;
}

// Column pass: thread (x, t) for x < w, t = blockIdx.y.  With wrap the
// doubled image's columns repeat, so each column is transformed once.
__global__ void __launch_bounds__(128) k_nft_columns(const NftArgs a)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = blockIdx.y;
    if (x >= a.w) {
        return;
    }
    const int64_t line = (int64_t)t * a.w + x, ss = 2 * (int64_t)a.w;
    int* v = a.v + line;
    float* z = a.z + line;
    unsigned int count = 0;
    const auto f = [&](int y) { return nft_feature(a, t, x, y) ? 0.0f : FLT_MAX; };
    float* col = a.inter + (int64_t)t * a.h * a.ipitch + x;
    fh_line(a.h, f, [&](int y, float d) { col[(int64_t)y * a.ipitch] = d; }, v, z, ss);
    for (int y = 0; y < a.h; ++y) {
        count += nft_feature(a, t, x, y) ? 1u : 0u;
    }
    atomicAdd(&a.tally[t], count);
}

// Row pass: thread (y, t).  The row has w samples, or 2w with wrap (the
// column pass repeated); the kept samples are written as distances.
__global__ void __launch_bounds__(128) k_nft_rows(const NftArgs a)
{
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = blockIdx.y;
    if (y >= a.h) {
        return;
    }
    const int n = a.wrap ? 2 * a.w : a.w;
    const int64_t line = (int64_t)t * a.h + y, ss = 2 * (int64_t)a.h;
    int* v = a.v + line;
    float* z = a.z + line;
    const float* row = a.inter + ((int64_t)t * a.h + y) * a.ipitch;
    float* drow = a.dist + ((int64_t)t * a.h + y) * a.ipitch;
    const int w = a.w, half = a.w / 2;
    const auto f = [&](int q) { return row[q < w ? q : q - w]; };
    if (a.wrap) {
        // keep columns w/2 .. w + w/2 - 1 of the doubled row, as column q mod w
        fh_line(n, f, [&](int q, float d) {
            if (q >= half && q < w + half) {
                drow[q < w ? q : q - w] = sqrtf(d);
            }
        }, v, z, ss);
    } else {
        fh_line(n, f, [&](int q, float d) { drow[q] = sqrtf(d); }, v, z, ss);
    }
}

__global__ void __launch_bounds__(256) k_nft_mask(const float* __restrict__ dist, int64_t ipitch, int w, int h,
                                                  uint8_t* __restrict__ mask, int64_t mpitch)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= w) {
        return;
    }
    const float d12 = dist[(int64_t)y * ipitch + x], d21 = dist[((int64_t)h + y) * ipitch + x];
    mask[(int64_t)y * mpitch + x] = d12 < d21 ? 255 : 0;
}

}  // namespace

size_t nft_scratch_bytes(int w, int h, int wrap)
{
    const int64_t ipitch = (w + 31) / 32 * 32;
    const int64_t n_col = 2 * (int64_t)w * ((int64_t)h + 1), n_row = 2 * (int64_t)h * ((wrap ? 2 : 1) * (int64_t)w + 1);
    const int64_t n_env = n_col > n_row ? n_col : n_row;
    return (size_t)(4 * ipitch * h * sizeof(float) + n_env * (sizeof(int) + sizeof(float)) + 256);
}

// Stage 0: the column pass and the tallies; 1: the row pass; 2: the mask.
cudaError_t launch_nft_stage(int stage, const BytePlane& white, const BytePlane& black, const BytePlane& mask,
                             int wrap, void* scratch, unsigned int* tally, cudaStream_t st)
{
    const int w = white.w, h = white.h;
    NftArgs a{};
    a.white = white.p;
    a.black = black.p;
    a.wpitch = white.pitch;
    a.bpitch = black.pitch;
    a.w = w;
    a.h = h;
    a.wrap = wrap;
    a.ipitch = (w + 31) / 32 * 32;
    a.inter = static_cast<float*>(scratch);
    a.dist = a.inter + 2 * a.ipitch * h;
    const int64_t n_col = 2 * (int64_t)w * ((int64_t)h + 1), n_row = 2 * (int64_t)h * ((wrap ? 2 : 1) * (int64_t)w + 1);
    const int64_t n_env = n_col > n_row ? n_col : n_row;
    a.v = reinterpret_cast<int*>(a.dist + 2 * a.ipitch * h);
    a.z = reinterpret_cast<float*>(a.v + n_env);
    a.tally = tally;
    if (stage == 0) {
        note_launch("nft_columns", 2.0 * w * h * (2.0 + 4.0));
        k_nft_columns<<<dim3((unsigned)((w + 127) / 128), 2), 128, 0, st>>>(a);
    } else if (stage == 1) {
        note_launch("nft_rows", 2.0 * w * h * 8.0);
        k_nft_rows<<<dim3((unsigned)((h + 127) / 128), 2), 128, 0, st>>>(a);
    } else {
        note_launch("nft_mask", (double)w * h * 9.0);
        k_nft_mask<<<dim3((unsigned)((w + 255) / 256), (unsigned)h), 256, 0, st>>>(a.dist, a.ipitch, w, h, mask.p,
                                                                               mask.pitch);
    }
    return cudaGetLastError();
}

}  // namespace enb
