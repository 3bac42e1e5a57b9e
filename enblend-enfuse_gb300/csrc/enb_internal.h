// enb_internal.h -- shared declarations of the CUDA kernels and the C ABI layer.
#pragma once

#include <cuda_runtime.h>

#include <utility>
#include <stdint.h>

#include <string>
#include <vector>

#include "enbgpu.h"

namespace enb {

constexpr int kMaxLevels = 29;  // MAX_PYRAMID_LEVELS, src/common.h:55
constexpr int kMaxEntropyWindow = 15;
constexpr int kMaxContrastWindow = 31;

// A planar level: `C` planes of h rows; pitch and plane strides in elements.
struct PlanarView {
    void* p;
    int64_t pitch;
    int64_t plane;
    int w, h, C;
    int dtype;  // ENB_I16 / ENB_I32 / ENB_F32
};

// An interleaved pixel image; pitch in elements of the sample type.
struct PixelView {
    const void* p;
    int64_t pitch;
    int w, h, C, stride;
    int dtype;  // ENB_U8 / ENB_U16 / ENB_F32
};

// An interleaved float image (the float-image path); pitch in floats.
struct FloatPixelView {
    const float* p;
    int64_t pitch;
    int w, h, C, stride;
};

// An 8-bit plane (alpha, seam mask).
struct BytePlane {
    uint8_t* p;
    int64_t pitch;
    int w, h;
};

// A float plane (weights).
struct FloatPlane {
    float* p;
    int64_t pitch;
    int w, h;
};

// Where the alpha of a pixel comes from.
enum AlphaMode { kAlphaPlane = 0, kAlphaOpaque = 1, kAlphaChannel3 = 2 };

struct AlphaSrc {
    int mode;
    BytePlane plane;  // kAlphaPlane
    PixelView pix;    // kAlphaChannel3: 4th component thresholded at [lo, hi]
    uint32_t lo, hi;  // integer samples
    float flo, fhi;   // float samples (pix.dtype == ENB_F32)
};

// Device-side constant tables of the enfuse weights.
struct WeightTables {
    const float* exposure;    // [max+1]: (float)(W_exp * f(g / max))
    const float* contrast;    // [max+1]: (float)(W_con * g / max)
    const float* entropy;     // [max+1]: (float)(W_ent * (double)(float)m)
    const double* plogp;      // [(n_max+1)*(n_max+1)]: p log p, p = c / n
    const long long* plogp_fx;// same in 2^-56 fixed point
    const double* logb;       // [n_max+1]: log(b)
    const float* scale_logb;  // [n_max+1]: max / log(b) as float
    const unsigned long long* scale_fx;  // [n_max+1]: max / log(b) in 2^-40 fixed point
    // float images, entropy windows of 3 or 5 (n_max = 9 or 25): H of a window
    // of n opaque taps whose only repeated samples are m1 taps at 1.0 and m0
    // at 0.0, at [(n * (n_max + 1) + m1) * (n_max + 1) + m0]; else nullptr
    const float* clip_h;
};

struct WeightParams {
    int use_exposure, use_contrast, use_saturation, use_entropy;
    int contrast_window, entropy_window;
    int gray_projector;
    double mixer[3];          // normalised channel-mixer weights
    double w_saturation;
    float w_sat_hi, w_sat_lo; // w_saturation split into two floats
    uint32_t maxv;
    // exposure cutoff (src/enfuse.h:652-730): exposure weight only where
    // cut_lo <= lower projection and upper projection <= cut_hi
    int exp_cut;
    int cut_proj[2];
    int32_t cut_lo, cut_hi;
    // entropy cutoff (src/enfuse.h:1143-1192): samples <= ent_lo -> 0,
    // >= ent_hi -> maxv before the entropy windows
    int ent_cut;
    int32_t ent_lo, ent_hi;
};

// Weights of float images (src/enfuse.h:962-1212 with float pixels).
// range stands for NumericTraits<float>::max() in the exposure and entropy
// weights (FLT_MAX: the reference, 1.0: normalised-float mode).
struct FloatWeightParams {
    int use_exposure, use_contrast, use_saturation, use_entropy;
    int contrast_window, entropy_window;
    int gray_projector, exp_function;
    double mixer[3];  // normalised channel-mixer weights
    float w_exposure, w_contrast, w_saturation, w_entropy;
    float range;
    float opt_hi, opt_lo;  // exposure optimum as a sum of two floats
    float inv_hi, inv_lo;  // 1 / effective width of the weight function, ditto
    int repeat_slots;      // hash slots per channel of the repeated-sample marks (0: none)
    // exposure cutoff (src/enfuse.h:652-730) and entropy cutoff (src/enfuse.h:
    // 1143-1192), as in WeightParams with float limits (upper clamp value:
    // range)
    int exp_cut;
    int cut_proj[2];
    float cut_lo, cut_hi;
    int ent_cut;
    float ent_lo, ent_hi;
};

// Name and algorithmic bytes of the most recent launch on this host thread;
// each launcher sets it (read by the profiler of the C ABI layer).
struct LaunchInfo {
    const char* name;
    double bytes;
    int kernels;  // kernel launches the launcher made (1 unless it says otherwise)
};
LaunchInfo& last_launch();
inline void note_launch(const char* name, double bytes) { last_launch() = LaunchInfo{name, bytes, 1}; }

// Level-0 pass of the fused enblend (enb_fused.cu).
struct Out0Host {
    PixelView white, black;
    AlphaSrc white_alpha, black_alpha;  // same mode for both
    BytePlane mask;
    int mfrac;
    int32_t white_value;
    void* out;
    int64_t opitch;       // elements
    BytePlane out_alpha;  // p == nullptr: not written
    int32_t* level0;      // collapsed level 0 (interleaved int32) or nullptr
    int frac, dither, wrap;
    uint64_t seed;
    unsigned int* err;    // device error word of the context (bit 0: a tile wait timed out)
    uint32_t tx_extra;    // bytes the level-0 pipeline's stage barriers expect
                          // beyond their copies: 0, except to test the timeout
};

// Coarse end of the fused enblend blend (one launch): slot 0 is the finest
// level handed over by the tiled kernels, slots 1..n-1 are reduced, blended
// and collapsed here; R of slots 1..n-1 is produced.
struct CoarseHost {
    int n;
    PlanarView gw[kMaxLevels], gb[kMaxLevels], rr[kMaxLevels], mg[kMaxLevels];
    BytePlane aw[kMaxLevels], ab[kMaxLevels];
    int32_t white_value;
    int wrap;
};

// Default of enb_fuse_options.coarse_pixels == 0: no coarse launch.  With
// programmatic dependent launch the per-level kernels finish the coarse
// levels sooner than the cluster launch (measured on the 2x4096x3072 blend:
// 0.617 ms per call against 0.635-0.648 ms with the cluster launch from
// 2048, 8192 or 32768 pixels down).
constexpr int64_t kCoarsePixels = -1;

// Launch with programmatic stream serialization: the kernel may be scheduled
// while its predecessor on the stream drains, and calls griddep_wait() before
// it reads anything the predecessor wrote.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args&&... args)
{
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// The same with dynamic shared memory.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl_smem(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                   Args&&... args)
{
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// ---- launchers (all queue on `st` and return the CUDA launch status) ------
cudaError_t launch_to_fixed(const PixelView& src, const PlanarView& dst, int frac, cudaStream_t st);
cudaError_t launch_bytes_to_fixed(const BytePlane& src, const PlanarView& dst, int frac, cudaStream_t st);
cudaError_t launch_float_to_fixed(const FloatPlane& src, const PlanarView& dst, int frac,
                                  cudaStream_t st);
cudaError_t launch_alpha_extract(const AlphaSrc& a, const BytePlane& dst, cudaStream_t st);
cudaError_t launch_reduce(int wrap, const PlanarView& src, const BytePlane* src_alpha,
                          const PlanarView& dst, const BytePlane* dst_alpha, cudaStream_t st);
// The same reduce of two levels of equal geometry and type (the white and
// black pyramids of one level) as one launch; falls back to two launches when
// the geometries differ.
// white and black images with alpha and the seam mask without, one level of
// the enblend down sweep in one launch (integer pyramids)
cudaError_t launch_reduce_img2_mask(int wrap, const PlanarView& s0, const BytePlane& sa0, const PlanarView& d0,
                                    const BytePlane& da0, const PlanarView& s1, const BytePlane& sa1,
                                    const PlanarView& d1, const BytePlane& da1, const PlanarView& ms,
                                    const PlanarView& md, cudaStream_t st);
cudaError_t launch_reduce2(int wrap, const PlanarView& s0, const BytePlane* sa0, const PlanarView& d0,
                           const BytePlane* da0, const PlanarView& s1, const BytePlane* sa1, const PlanarView& d1,
                           const BytePlane* da1, cudaStream_t st);
cudaError_t launch_expand(int add, int wrap, const PlanarView& src, const PlanarView& dst,
                          cudaStream_t st);
cudaError_t launch_blend(const PlanarView& mask, const PlanarView& white, const PlanarView& black,
                         int32_t white_value, cudaStream_t st);
cudaError_t launch_mask_mul_acc(const PlanarView& lp, const PlanarView& mask, int32_t divisor,
                                const PlanarView& result, int accumulate, cudaStream_t st);
cudaError_t launch_from_fixed(const PlanarView& src, const BytePlane& alpha, void* dst,
                              int64_t dst_pitch, int dst_dtype, int dst_stride, int frac,
                              int dither, uint64_t seed, cudaStream_t st);
cudaError_t launch_copy_pixels(const PixelView& src, void* dst, int64_t dst_pitch, cudaStream_t st);
cudaError_t launch_enfuse_mask(const PixelView& img, const AlphaSrc& alpha, const WeightParams& wp,
                               const WeightTables& tab, const FloatPlane& out, cudaStream_t st);
cudaError_t launch_norm_accumulate(const FloatPlane& mask, const FloatPlane& norm, int first,
                                   cudaStream_t st);
cudaError_t launch_union_alpha(const BytePlane& a, const BytePlane& uni, int first, cudaStream_t st);
cudaError_t launch_hard_mask(const FloatPlane* masks, int K, cudaStream_t st);
cudaError_t launch_soft_mask_to_fixed(const FloatPlane& mask, const FloatPlane& norm, int K,
                                      const PlanarView& dst, int frac, cudaStream_t st);
cudaError_t launch_copy_level0(const PlanarView& src, int32_t* dst, cudaStream_t st);
cudaError_t launch_alpha_component(const BytePlane& alpha, void* dst, int64_t dst_pitch, int dst_dtype,
                                   cudaStream_t st);

// fused enblend passes (enb_fused.cu)
cudaError_t launch_reduce0_alpha(const PixelView& src, const AlphaSrc& a, int frac, const PlanarView& dst,
                                 const BytePlane& dst_alpha, int wrap, cudaStream_t st);
// Level-0 reduce of the white and black images in one launch (two launches
// when their formats, alpha sources or geometries differ).
cudaError_t launch_reduce0_alpha2(const PixelView& s0, const AlphaSrc& a0, const PlanarView& d0, const BytePlane& da0,
                                  const PixelView& s1, const AlphaSrc& a1, const PlanarView& d1, const BytePlane& da1,
                                  int frac, int wrap, cudaStream_t st, int ty0 = 0, int nty = -1);
cudaError_t launch_reduce0_bytes(const BytePlane& src, int frac, const PlanarView& dst, int wrap, cudaStream_t st,
                                 int ty0 = 0, int nty = -1);
// Destination tile rows (16 each) of a reduce into a level of height dh.
int reduce_tile_rows_of(int dh);
// A reduced level's tile rows whose source rows [0, rows_ready) are all
// present (rows_ready >= sh: every tile row).
int reduce_tile_rows_ready(int sh, int dh, int rows_ready);
cudaError_t launch_blend_into(const PlanarView& mask, const PlanarView& gw, const PlanarView& gb,
                              const PlanarView& r, int32_t white_value, cudaStream_t st);
cudaError_t launch_up_level(const PlanarView& gw1, const PlanarView& gb1, const PlanarView& r1,
                            const PlanarView& mask, const PlanarView& gw, const PlanarView& gb,
                            const PlanarView& r, int32_t white_value, int wrap, cudaStream_t st);
cudaError_t launch_out0(const PlanarView* gw1, const PlanarView* gb1, const PlanarView* r1, const Out0Host& h,
                        cudaStream_t st, int ty0 = 0, int nty = -1);
cudaError_t launch_coarse(const CoarseHost& h, cudaStream_t st);

// fused enfuse of K 8/16-bit images (enb_efuse.cu): the level passes of
// enfuseMain's pyramids (src/enfuse.h:1501-1617) with the weights of all
// exposures per tile, no level 0 of any image pyramid stored, one up pass
// per level and level 0 straight to the output pixels.
constexpr int kEfuseMaxK = 16;
struct EfuseHost {
    int K, L, w, h, C, S, dtype;   // exposures, levels, canvas, colour samples, samples a pixel, ENB_U8/U16
    PixelView img[kEfuseMaxK];
    AlphaSrc alpha[kEfuseMaxK];
    const float* masks_in[kEfuseMaxK];  // --load-masks planes or null
    int64_t mipitch[kEfuseMaxK];        // floats
    int hard;
    WeightParams wp;
    WeightTables tab;
    int lw[kMaxLevels], lh[kMaxLevels];
    int64_t pitch[kMaxLevels];     // elements of every image/mask/result plane of level l
    int64_t apitch[kMaxLevels];    // bytes of the alpha planes of level l
    void* m[kEfuseMaxK][kMaxLevels];      // mask pyramids M_k[l] (Int16 9.7 / Int32 9.15)
    void* g[kEfuseMaxK][kMaxLevels];      // image pyramids G_k[l], l >= 1 (C planes)
    uint8_t* a[kEfuseMaxK][kMaxLevels];   // their alpha, l >= 1
    uint8_t* u[kMaxLevels];               // union alpha U[l] (U[0]: the output alpha plane)
    int64_t upitch0;                      // bytes of U[0]
    void* r[kMaxLevels];                  // result levels R[l], l >= 1 (C planes)
    void* out;                            // output pixels (the input type, S samples a pixel)
    int64_t opitch;                       // elements
    int32_t* level0;                      // collapsed level 0 (interleaved int32) or null
    int wrap, dither;
    uint64_t seed;
};
cudaError_t launch_ef_weights(const EfuseHost& h, cudaStream_t st);
cudaError_t launch_ef_reduce(const EfuseHost& h, int l, int masks, cudaStream_t st);
cudaError_t launch_ef_top(const EfuseHost& h, cudaStream_t st);
cudaError_t launch_ef_up(const EfuseHost& h, int l, cudaStream_t st);
cudaError_t launch_ef_out0(const EfuseHost& h, cudaStream_t st);

// batched fuse of float stacks (enb_batch.cu)
constexpr int kBatchMaxK = 16;
struct BatchStackHost {
    int K, w, h, C;
    const float* img[kBatchMaxK];
    int64_t ipitch[kBatchMaxK];  // floats
    int istride[kBatchMaxK];
    const uint8_t* alpha[kBatchMaxK];  // nullptr: opaque
    int64_t apitch[kBatchMaxK];
    float* out;
    int64_t opitch;  // floats
    int ostride;
    uint8_t* oalpha;  // nullptr: not written
    int64_t oapitch;
};
struct BatchPlan;
// err: the context's device error word (bit 1: a coarse item's wait ran out)
cudaError_t batch_plan_create(const std::vector<BatchStackHost>& stacks, const FloatWeightParams& wp,
                              const WeightTables& tab, int levels, int wrap, int hard, int64_t coarse_pixels,
                              unsigned int* err, cudaStream_t st, BatchPlan** out);
void batch_plan_destroy(BatchPlan* p);
int batch_plan_steps(const BatchPlan* p);
double batch_plan_pixels(const BatchPlan* p);
cudaError_t batch_plan_launch(const BatchPlan* p, int step, cudaStream_t st);

// nearest-feature seam mask (enb_nft.cu): scratch bytes for a w x h
// canvas, and the three stages (0 columns and tallies, 1 rows, 2 mask)
size_t nft_scratch_bytes(int w, int h, int wrap);
cudaError_t launch_nft_stage(int stage, const BytePlane& white, const BytePlane& black, const BytePlane& mask,
                             int wrap, void* scratch, unsigned int* tally, cudaStream_t st);

// adjoint of the float enfuse (enb_adjoint.cu)
cudaError_t launch_adj_norm(int K, const float* w, const float* a, float* m, int64_t pitch, int64_t plane, int width,
                            int height, cudaStream_t st);
cudaError_t launch_adj_merge(const PlanarView& lp, const PlanarView& m, const PlanarView& r, int first, cudaStream_t st);
// level 0 of an image pyramid in the adjoint's offset form (G - 1)
cudaError_t launch_adj_to_pyramid(const FloatPixelView& img, const PlanarView& g, cudaStream_t st);
cudaError_t launch_adj_loss(const PlanarView& c0, const float* tgt, int64_t tpitch, int tstride, float* out,
                            int64_t opitch, int ostride, const PlanarView& g0, double* loss, cudaStream_t st);
cudaError_t launch_expand_T(const PlanarView& fine, const PlanarView& coarse, cudaStream_t st);
cudaError_t launch_adj_mask_level(const PlanarView& gr, const PlanarView& lp, const PlanarView* next,
                                  const PlanarView& acc, cudaStream_t st);
cudaError_t launch_adj_norm_bw(int K, const float* w, const float* a, const float* gm, float* gw, float* ga,
                               int64_t pitch, int64_t plane, int width, int height, cudaStream_t st);
cudaError_t launch_adj_weights_bw(const FloatPixelView& img, const float* gw, int64_t gpitch, const FloatWeightParams& wp,
                                  float inv_width, float width, float w_exp, int cwin, double* d, cudaStream_t st);

// float-image path (enb_float.cu): FP32 pyramid levels (dtype ENB_F32)
cudaError_t launch_f_to_pyramid(const FloatPixelView& s, const PlanarView& d, cudaStream_t st);
cudaError_t launch_f_from_pyramid(const PlanarView& s, const BytePlane& a, float* dst, int64_t dpitch, int dstride,
                                  cudaStream_t st);
cudaError_t launch_f_expand(int add, int wrap, const PlanarView& s, const PlanarView& d, cudaStream_t st);
cudaError_t launch_f_blend(const PlanarView& m, const PlanarView& wt, const PlanarView& b, int32_t wv,
                           cudaStream_t st);
cudaError_t launch_f_mask_mul_acc(const PlanarView& lp, const PlanarView& m, int32_t divisor, const PlanarView& r,
                                  int acc, cudaStream_t st);
cudaError_t launch_f_copy_level0(const PlanarView& s, float* dst, cudaStream_t st);
// Fills WeightTables.clip_h (tab's other tables on the device) for windows
// of nmax taps.
cudaError_t launch_clip_entropy_table(const WeightTables& tab, int nmax, float* out, cudaStream_t st);

cudaError_t launch_f_enfuse_mask(const FloatPixelView& img, const BytePlane& alpha, const FloatWeightParams& wp,
                                 const WeightTables& tab, const FloatPlane& out, cudaStream_t st);

}  // namespace enb
