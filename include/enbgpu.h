/*
 * enbgpu.h -- C ABI of the GB300 (sm_103a) enblend/enfuse multiresolution path.
 *
 * Each entry point replaces one internal call of enblend-enfuse 4.3 on the
 * pyramid / blend / weight path; the reference interface it stands in for is
 * cited beside it (file:line in the reference source tree).  The reference's
 * templates take VIGRA iterator/accessor triples and `new` their pyramids; here
 * images are plain descriptors of device memory, pyramids are device-resident
 * handles, errors are status codes (the reference throws from
 * vigra_precondition or calls exit(1)), and all work is queued on the
 * context's CUDA stream.  Nothing is synchronous unless a call says so.
 *
 * There is no CPU fallback: without a usable CUDA device every compute entry
 * point fails with ENB_ERR_CUDA.
 */
#ifndef ENBGPU_H
#define ENBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ENBGPU_ABI_VERSION 6

typedef enum {
    ENB_OK = 0,
    ENB_ERR_INVALID = 1,     /* bad argument (the reference's vigra_precondition) */
    ENB_ERR_UNSUPPORTED = 2, /* valid in the reference but not implemented here */
    ENB_ERR_CUDA = 3,        /* CUDA runtime error or no device */
    ENB_ERR_NOMEM = 4        /* device allocation failed */
} enb_status;

typedef enum {
    ENB_U8 = 0,   /* 8-bit unsigned samples */
    ENB_U16 = 1,  /* 16-bit unsigned samples */
    ENB_F32 = 2,  /* 32-bit float: float images (interleaved), weight masks,
                     and the FP32 pyramid levels of float images, which stand
                     in for the reference's double pyramids
                     (src/numerictraits.h:185) */
    ENB_I16 = 3,  /* 16-bit signed fixed point (pyramids of 8-bit images) */
    ENB_I32 = 4   /* 32-bit signed fixed point (pyramids of 16-bit images, masks) */
} enb_dtype;

/* Dither rule of the fixed-point -> pixel conversion. */
typedef enum {
    ENB_DITHER_HASH = 0,    /* the reference's rule (src/fixmath.h:251-277), random
                               bits from a counter hash of (seed, sample index) */
    ENB_DITHER_NEAREST = 1  /* no dither: round half up */
} enb_dither;

/* Exposure weight functions, src/exposure_weight.h:44-128. */
typedef enum {
    ENB_EXP_GAUSSIAN = 0,
    ENB_EXP_LORENTZIAN = 1,
    ENB_EXP_HALF_SINE = 2,
    ENB_EXP_FULL_SINE = 3,
    ENB_EXP_BISQUARE = 4
} enb_exposure_function;

/* Grayscale projectors, src/mga.h:78-87 (l-star and pl-star are not provided). */
typedef enum {
    ENB_GRAY_AVERAGE = 0,
    ENB_GRAY_VALUE = 1,
    ENB_GRAY_ANTI_VALUE = 2,
    ENB_GRAY_LIGHTNESS = 3,
    ENB_GRAY_LUMINANCE = 4,
    ENB_GRAY_MIXER = 5
} enb_gray_projector;

/* An image in device memory (host memory for the drivers when
 * enb_fuse_options.host_buffers is set).
 *   interleaved pixel images: `channels` colour samples out of `pix_stride`
 *     components per pixel, rows `pitch` bytes apart (RGB: 3/3, RGBA: 3/4);
 *   planar pyramid levels: `channels` planes of `height` rows, rows `pitch`
 *     bytes apart, planes `plane_pitch` bytes apart (pix_stride ignored);
 *   alpha and mask planes: channels = 1, U8 (0 transparent, else opaque). */
typedef struct {
    void* data;
    int64_t pitch;
    int64_t plane_pitch;
    int32_t width;
    int32_t height;
    int32_t channels;
    int32_t pix_stride;
    int32_t dtype;   /* enb_dtype */
    int32_t planar;  /* 0 interleaved, 1 planar */
} enb_image;

/* enfuse weighting parameters; defaults as in src/enfuse.cc:117-140. */
typedef struct {
    double w_exposure;      /* --exposure-weight, default 1.0 */
    double w_saturation;    /* --saturation-weight, default 0.0 */
    double w_contrast;      /* --contrast-weight, default 0.0 */
    double w_entropy;       /* --entropy-weight, default 0.0 */
    double exp_optimum;     /* --exposure-optimum, default 0.5 */
    double exp_width;       /* --exposure-width, default 0.2 */
    int32_t exp_function;   /* --exposure-weight-function, enb_exposure_function */
    int32_t contrast_window;/* --contrast-window-size, odd >= 3, default 5 */
    int32_t entropy_window; /* --entropy-window-size, odd 3..15, default 3 */
    int32_t gray_projector; /* --gray-projector, enb_gray_projector */
    double mixer[3];        /* channel-mixer weights (unnormalised) */
    double float_range;     /* float images: the value the reference takes as
                               NumericTraits<float>::max() in the exposure
                               (y = gray / max, src/enfuse.h:638) and entropy
                               (H * max) weights.  0 (default): FLT_MAX, the
                               reference's behaviour, which makes the exposure
                               weight constant and the entropy weight huge;
                               > 0: normalised-float mode, e.g. 1.0 for images
                               in [0, 1].  Saturation (max 1.0) and contrast
                               (W * sigma) are the same in both modes. */
    /* --exposure-cutoff LOWER[:UPPER[:LOWERPROJ[:UPPERPROJ]]]
     * (src/enfuse.cc:1272-1340, CutoffExposureFunctor src/enfuse.h:652-730):
     * a pixel whose lower projection lies below the lower limit, or whose
     * upper projection lies above the upper limit, gets exposure weight 0.
     * A limit with its *_pct flag set is a percentage of the sample maximum
     * (of float_range's scale for float images), else an absolute sample
     * value; integer limits truncate toward zero; a negative upper limit
     * counts down from the maximum.  Defaults: 0 % / 100 % (off), projectors
     * anti-value / value (enb_gray_projector). */
    double exp_cutoff_lower, exp_cutoff_upper;
    int32_t exp_cutoff_lower_pct, exp_cutoff_upper_pct;
    int32_t exp_cutoff_lower_projector, exp_cutoff_upper_projector;
    /* --entropy-cutoff LOWER[:UPPER] (src/enfuse.cc:1213-1270, src/enfuse.h:
     * 1143-1192): before the entropy windows, samples at or below the lower
     * limit become 0 and samples at or above the upper limit the maximum
     * (the third sample is judged low by the first sample, as the reference
     * does).  Limits as for the exposure cutoff; defaults 0 % / 100 % (off). */
    double ent_cutoff_lower, ent_cutoff_upper;
    int32_t ent_cutoff_lower_pct, ent_cutoff_upper_pct;
    /* User-defined exposure weight function (--exposure-weight-function=
     * SHARED-OBJECT:SYMBOL[:ARGUMENT...], src/exposure_weight.cc:44-129):
     * the function's weight(y) tabulated by the caller at y = g / max for
     * every sample value g = 0..max of the images' type, exposure_table_size
     * = max + 1 (256 for 8-bit, 65536 for 16-bit images).  It replaces the
     * built-in exp_function in W_exp * weight(y) (src/enfuse.h:624-651),
     * also under the exposure cutoff.  NULL (default): exp_function.  Float
     * images, whose y is no sample index, reject a table
     * (ENB_ERR_UNSUPPORTED).  The caller keeps the table alive for the call. */
    const double* exposure_table;
    int32_t exposure_table_size;
} enb_enfuse_params;

/* Options of the fuse drivers. */
typedef struct {
    int32_t levels;        /* 0: automatic (roiBounds, src/bounds.h:97-177); >0 --levels */
    int32_t wrap;          /* --wrap horizontal (periodic x) */
    int32_t hard_mask;     /* enfuse --hard-mask */
    int32_t dither;        /* enb_dither */
    uint64_t seed;         /* dither seed */
    int32_t host_buffers;  /* 1: all image pointers are host memory; copies are
                              done on the context stream and the call returns
                              after the result is back in host memory */
    int32_t plain;         /* 1: run the reference's pass structure (one kernel
                              per reference operation, every level materialised)
                              instead of the fused level passes; same result,
                              for comparisons */
    void* level0_out;      /* optional device buffer (host if host_buffers):
                              collapsed level 0 before conversion, int32
                              (float for F32 images), interleaved
                              width*height*channels */
    int32_t coarse_pixels; /* enblend: pyramid levels of at most this many
                              pixels run in one cluster launch; 0: default
                              (none), < 0: every level in its own launches.
                              enb_fuse_stacks: levels of at most this many
                              pixels run in the persistent coarse kernel;
                              0: the threshold enb_fuse_stacks_tune chose for
                              the batch geometry, else 64 x 64; < 0: none */
    int32_t graph;         /* enb_fuse_stacks: 1 (default) replays a CUDA
                              graph of the launch sequence, captured once per
                              batch geometry; 0 launches directly */
} enb_fuse_options;

typedef struct enb_ctx enb_ctx;
typedef struct enb_pyramid enb_pyramid;

/* ---- context ----------------------------------------------------------- */
int enb_abi_version(void);
enb_status enb_create(int device, enb_ctx** ctx);
enb_status enb_destroy(enb_ctx* ctx);
/* Queue all later work on `cuda_stream` (a cudaStream_t; NULL = legacy default). */
enb_status enb_set_stream(enb_ctx* ctx, void* cuda_stream);
/* Wait for the context's stream.  ENB_ERR_CUDA also when a kernel queued
 * since the last synchronisation gave up a bounded wait for its tile copies
 * (the level-0 pipeline of enb_enblend); enb_last_error says which. */
enb_status enb_synchronize(enb_ctx* ctx);
/* Message of the last failed call on this context (never NULL). */
const char* enb_last_error(const enb_ctx* ctx);
/* Test hook of the bounded waits (no counterpart in the reference): with
 * extra_bytes in 1..4096, the level-0 tile pipeline of later enb_enblend
 * calls on this context arms each stage's barrier for that many bytes more
 * than its copies deliver, so every wait for a stage runs out (after about
 * half a second of SM clock), the kernel records the timeout in the
 * context's error word and returns without writing the waiting tiles, and
 * the next synchronising call fails with ENB_ERR_CUDA.  Nothing faults and
 * nothing waits without a limit; the context stays usable.  0 (the default)
 * restores normal operation. */
enb_status enb_debug_overarm_tile_waits(enb_ctx* ctx, uint32_t extra_bytes);
/* Kernels launched on this context since creation (a counter, for profiling). */
uint64_t enb_launch_count(const enb_ctx* ctx);
void enb_default_enfuse_params(enb_enfuse_params* p);
void enb_default_fuse_options(enb_fuse_options* o);

/* Per-kernel timing with CUDA events around every launch on the context
 * stream, with the algorithmic bytes each launch must move (the role of
 * ShowProfileData for the reference's OpenCL kernels, src/opencl.h:199).
 * Enabling (or disabling) clears the records.  enb_profile_entry
 * synchronises the stream and returns kernel i's launch count, summed device
 * time and summed algorithmic bytes. */
enb_status enb_profile_enable(enb_ctx* ctx, int enable);
int enb_profile_count(enb_ctx* ctx);
enb_status enb_profile_entry(enb_ctx* ctx, int i, const char** name, uint64_t* launches,
                             double* total_ms, double* bytes);

/* roiBounds level count (src/bounds.h:97-177). */
int enb_num_levels(int width, int height, int min_levels, int exact_levels);

/* ---- pyramids (std::vector<PyramidImageType*>*, src/pyramid.h:1471) ----- */
/* Device-resident pyramid: `levels` planar levels of `channels` planes of
 * dtype ENB_I16, ENB_I32 or ENB_F32, level l of size ((w+1)>>1)^l.  The
 * primitives below accept F32 image levels with I32 (9.15) mask levels, the
 * pyramid types of float images.  Ownership stays
 * with the caller (the reference's `delete` of each level and the vector,
 * src/enfuse.h:1568-1570 -> enb_pyramid_free). */
enb_status enb_pyramid_create(enb_ctx* ctx, int levels, int width, int height, int channels,
                              int dtype, enb_pyramid** out);
enb_status enb_pyramid_free(enb_ctx* ctx, enb_pyramid* pyr);
int enb_pyramid_levels(const enb_pyramid* pyr);
enb_status enb_pyramid_level(const enb_pyramid* pyr, int level, enb_image* out);
/* Copy one level to / from dense host memory laid out as channels x height x
 * width samples of the pyramid dtype; synchronous.  The debugging role of
 * exportPyramid (src/pyramid.h:1788-1857). */
enb_status enb_pyramid_read_level(enb_ctx* ctx, const enb_pyramid* pyr, int level, void* host_dst);
enb_status enb_pyramid_write_level(enb_ctx* ctx, enb_pyramid* pyr, int level, const void* host_src);

/* ---- primitives (device images) ---------------------------------------- */
/* copyToPyramidImage / ConvertScalarToPyramidFunctor (src/fixmath.h:116-206,
 * 2019-2147): U8/U16 samples -> `v << frac_bits` into a planar I16/I32 level;
 * an F32 plane (a weight mask) into an I16/I32 level -> fromRealPromote(v *
 * 2^frac_bits); an interleaved F32 image into an F32 level -> the
 * logarithmic mapping v >= 0 ? 1 + log1p(v) : 1 / (1 - v) (frac_bits ignored). */
enb_status enb_to_pyramid(enb_ctx* ctx, const enb_image* src, const enb_image* dst, int frac_bits);

/* reduce (src/pyramid.h:166-573 with alpha, :601-848 without).  src_alpha ==
 * NULL selects the alpha-free operator (clamp-to-edge, /256); otherwise
 * dst_alpha receives 255 where any opaque tap contributed. */
enb_status enb_reduce(enb_ctx* ctx, int wraparound, const enb_image* src, const enb_image* src_alpha,
                      const enb_image* dst, const enb_image* dst_alpha);

/* expand (src/pyramid.h:1102-1457): add == 0: dst -= E(src) (laplacian build);
 * add != 0: dst = fromPromote(dst + E(src)) (collapse). */
enb_status enb_expand(enb_ctx* ctx, int add, int wraparound, const enb_image* src,
                      const enb_image* dst);

/* CartesianBlendFunctor over one level (src/blend.h:41-76): black := blend of
 * white and black under mask / white_value. */
enb_status enb_blend(enb_ctx* ctx, const enb_image* mask, const enb_image* white,
                     const enb_image* black, int32_t white_value);

/* ImageMaskMultiplyFunctor and accumulation (src/enfuse.h:601-620,
 * 1554-1588): result = (accumulate ? result : 0) + fromRealPromote(lp * mask / divisor). */
enb_status enb_mask_multiply_accumulate(enb_ctx* ctx, const enb_image* lp, const enb_image* mask,
                                        int32_t divisor, const enb_image* result, int accumulate);

/* copyFromPyramidImageIf (src/fixmath.h:2158-2294, rule :251-277): planar
 * fixed point -> interleaved U8/U16 pixels where alpha != 0; an F32 level ->
 * F32 pixels by v >= 1 ? expm1(v - 1) : 1 - 1/v (src/fixmath.h:320-329;
 * frac_bits, dither and seed ignored). */
enb_status enb_from_pyramid(enb_ctx* ctx, const enb_image* src, const enb_image* alpha,
                            const enb_image* dst, int frac_bits, int dither, uint64_t seed);

/* ---- pyramid builders --------------------------------------------------- */
/* gaussianPyramid (src/pyramid.h:1468-1636); alpha NULL -> alpha-free reduce. */
enb_status enb_gaussian_pyramid(enb_ctx* ctx, int wraparound, const enb_image* src,
                                const enb_image* alpha, int frac_bits, enb_pyramid* pyr);
/* No counterpart in the reference.  Same result as enb_gaussian_pyramid, but
 * the call allocates nothing: for callers that must not allocate device
 * memory while they run, such as an application that reserves its whole GPU
 * budget up front in its own pool and forbids allocations in its processing
 * callbacks (cudaMalloc can block the device and can fail mid-run), or a
 * fixed-budget embedded pipeline.  The alpha planes of levels 1..L-1 live in
 * a file-scope device array of ENB_NOALLOC_SCRATCH_BYTES (16 MiB, about
 * 48 Mpx at level 0) that every GPU loading the library holds until exit;
 * larger images are rejected with ENB_ERR_INVALID.  It accepts the same
 * sources as enb_gaussian_pyramid (level 0 converted as by enb_to_pyramid).
 * The first call on each device looks up that array's device address (make
 * that first call before any stream capture) and keeps it for the life of
 * the process, so a cudaDeviceReset after that first call is not supported.
 * All calls share the array: calls that overlap on the GPU (other streams,
 * other threads) race on it. */
#define ENB_NOALLOC_SCRATCH_BYTES (16u << 20)
enb_status enb_gaussian_pyramid_noalloc(enb_ctx* ctx, int wraparound, const enb_image* src,
                                        const enb_image* alpha, int frac_bits, enb_pyramid* pyr);
/* laplacianPyramid (src/pyramid.h:1647-1747). */
enb_status enb_laplacian_pyramid(enb_ctx* ctx, int wraparound, const enb_image* src,
                                 const enb_image* alpha, int frac_bits, enb_pyramid* pyr);
/* collapsePyramid (src/pyramid.h:1758-1784); level 0 receives the result. */
enb_status enb_collapse_pyramid(enb_ctx* ctx, int wraparound, enb_pyramid* pyr);
/* blend (src/blend.h:81-121): black_lp := per-level CartesianBlend. */
enb_status enb_blend_pyramids(enb_ctx* ctx, const enb_pyramid* mask_gp, const enb_pyramid* white_lp,
                              enb_pyramid* black_lp, int32_t white_value);

/* ---- enfuse weights ----------------------------------------------------- */
/* enfuseMask (src/enfuse.h:962-1212): F32 weight plane of an U8/U16/F32 image. */
enb_status enb_enfuse_mask(enb_ctx* ctx, const enb_enfuse_params* params, const enb_image* src,
                           const enb_image* alpha, const enb_image* mask_out);

/* ---- drivers ------------------------------------------------------------ */
/* enfuseMain's weighting, normalisation, pyramids, merge, collapse and
 * output conversion (src/enfuse.h:1217-1617) for K union-sized U8, U16 or
 * F32 images (F32: FP32 pyramids in place of the reference's double ones;
 * the 4th component of an RGBA F32 image is thresholded at [0.5, 1]).
 * alphas: K alpha planes or NULL (for RGBA images the alpha is then the
 * thresholded 4th component as imported by src/assemble.h:240-253, else fully
 * opaque).  masks_in: K F32 weight planes replacing enfuseMask (--load-masks),
 * or NULL.  out: interleaved image of the input type (zero where out_alpha is
 * 0); out_alpha: U8 union alpha, may be NULL. */
enb_status enb_enfuse(enb_ctx* ctx, const enb_enfuse_params* params, int K, const enb_image* images,
                      const enb_image* alphas, const enb_image* masks_in, const enb_image* out,
                      const enb_image* out_alpha, const enb_fuse_options* opt);

/* enblend's seam mask from the nearest-feature transform
 * (nearestFeatureTransform, src/nearest.h:427-553; the mask of --fine-mask
 * --no-optimize, src/mask.h:1101-1180): mask = 255 where the nearest pixel
 * covered by the white image only (white_alpha > black_alpha) is nearer than
 * the nearest pixel covered by the black image only, else 0, with the
 * reference's Euclidean distance transform in float (the Felzenszwalb-
 * Huttenlocher transform of its OpenMP build, src/openmp_vigra.h:257-433),
 * bit-identical.  opt: wrap (the horizontally periodic transform,
 * src/nearest.h:293-342) and host_buffers; other fields are ignored.  The
 * call synchronises.  ENB_ERR_INVALID when fewer than 4 (w + h) pixels are
 * covered by one image only in both directions (the reference's "excessive
 * image overlap" exit); the mask is then unspecified. */
enb_status enb_nft_mask(enb_ctx* ctx, const enb_image* white_alpha, const enb_image* black_alpha,
                        const enb_image* mask, const enb_fuse_options* opt);

/* enblendMain's pyramid section (src/enblend.h:330-510): blend `white` into
 * `black` under the 0/255 seam mask over the whole canvas.  out receives the
 * black image with the blended pixels where the union alpha is set (for RGBA
 * images the 4th component becomes the union alpha, 0 or the type maximum,
 * 1.0 for F32); out may be the black image itself.  F32 images always take
 * the per-operation pass structure (the fused passes are fixed point). */
enb_status enb_enblend(enb_ctx* ctx, const enb_image* white, const enb_image* white_alpha,
                       const enb_image* black, const enb_image* black_alpha, const enb_image* mask,
                       const enb_image* out, const enb_image* out_alpha, const enb_fuse_options* opt);

/* ---- batched stacks (no counterpart in the reference) ------------------- */
/* One exposure stack of a batched fuse. */
#define ENB_BATCH_MAX_K 16
typedef struct {
    int32_t K;                  /* exposures, 1..ENB_BATCH_MAX_K */
    const enb_image* images;    /* K interleaved F32 images of one geometry */
    const enb_image* alphas;    /* K U8 alpha planes, or NULL (thresholded 4th
                                   component of RGBA images, else opaque) */
    const enb_image* out;       /* interleaved F32 result of the geometry */
    const enb_image* out_alpha; /* U8 union alpha, or NULL */
} enb_stack;

/* enfuseMain (src/enfuse.h:1217-1617) of n independent float stacks of
 * arbitrary, different sizes and exposure counts as one batch: every launch
 * covers all stacks at one pyramid level, the levels of at most
 * opt->coarse_pixels pixels run in one persistent kernel, and the sequence
 * is replayed as a CUDA graph.  Each stack's result is that of enb_enfuse on
 * it (same FP32 arithmetic up to the order of float additions).  masks are
 * computed (no --load-masks); opt->plain = 1 runs enb_enfuse stack by stack
 * instead (for comparisons).  The workspace and graph of the last batch
 * geometry stay cached in the context. */
enb_status enb_fuse_stacks(enb_ctx* ctx, const enb_enfuse_params* params, int n_stacks, const enb_stack* stacks,
                           const enb_fuse_options* opt);

/* Autotuner of the batched fuse's level schedule (which levels run in the
 * persistent coarse kernel, which in per-level launches): runs
 * enb_fuse_stacks on this batch once per candidate coarse threshold to warm
 * up and then `reps` times under CUDA events, and keeps the fastest for the
 * batch's geometry (stack sizes and exposure counts, parameters, options;
 * not the buffers).  Later enb_fuse_stacks calls on a batch of that
 * geometry with opt->coarse_pixels == 0 use it.  candidates: n_candidates
 * thresholds in pixels (< 0: no coarse kernel), or NULL for the built-in
 * list {-1, 1024, 4096, 16384, 65536}; times_ms (optional) receives the
 * mean milliseconds per call of each candidate, best the chosen threshold.
 * The outputs hold the last call's result (every schedule gives the same
 * bits). */
enb_status enb_fuse_stacks_tune(enb_ctx* ctx, const enb_enfuse_params* params, int n_stacks, const enb_stack* stacks,
                                const enb_fuse_options* opt, const int32_t* candidates, int n_candidates, int reps,
                                float* times_ms, int32_t* best);

/* ---- adjoint (no counterpart in the reference) --------------------------- */
/* Loss and gradients of the float enfuse against a target image. */
typedef struct {
    double loss;            /* mean over pixels and channels of (out - target)^2 */
    double d_exp_optimum;   /* dL/d exp_optimum */
    double d_exp_width;     /* dL/d exp_width */
    double d_w_exposure;    /* dL/d w_exposure */
    double d_w_saturation;  /* dL/d w_saturation */
    double d_w_contrast;    /* dL/d w_contrast */
} enb_fuse_grad_result;

/* The float enfuse of K opaque RGB images (src/enfuse.h:1217-1617 with
 * continuous soft masks: each weight w_k, from params, is scaled by
 * exp(logit_k), normalised over the K exposures, and used as a mask without
 * its 9.15 quantisation), the loss against `target`, and its gradients:
 * the scalars in `res` and, when grad_logits is given, dL/d logit_k per
 * pixel.  logits: K F32 planes or NULL (all 0).  out: optional F32 image
 * receiving the forward result.  Entropy weights, the exposure cutoff, hard
 * masks and wrap-around are not differentiated (ENB_ERR_UNSUPPORTED).  The backward rebuilds each
 * exposure's Laplacian pyramid instead of keeping K of them, so the memory
 * held is one pyramid per kind whatever K.  Device buffers; synchronous. */
enb_status enb_fuse_grad(enb_ctx* ctx, const enb_enfuse_params* params, int K, const enb_image* images,
                         const enb_image* logits, const enb_image* target, const enb_image* out,
                         const enb_image* grad_logits, enb_fuse_grad_result* res, const enb_fuse_options* opt);

#ifdef __cplusplus
}
#endif

#endif /* ENBGPU_H */
