/*
 * enb_oracle.h -- CPU restatement of the enblend/enfuse multiresolution hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * path and the timed CPU baseline ("port") of bench.py.  Only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline leg may load it.  The
 * product library (libenbgpu.so) never links or calls it.
 *
 * Every function restates an algorithm of the reference (enblend-enfuse 4.3,
 * src/...) from its observable semantics; the file:line of the reference
 * code it follows is given at each function.  Pyramid values are held as
 * int32 arrays; `bits` (16 or 32) selects the storage semantics of the
 * reference's pyramid pixel type (Int16 for 8-bit images, Int32 for 16-bit
 * images, src/numerictraits.h:159-163): static_cast wrap-around where the
 * reference assigns through a plain cast, saturation where it uses
 * fromPromote / fromRealPromote.
 *
 * Pixel images are interleaved: `C` colour channels out of `pix_stride`
 * components per pixel (3/3 for RGB, 3/4 for RGBA, 1/1 for gray).  Alpha is a
 * separate 8-bit plane (0 = transparent, anything else = opaque), which is
 * what the reference's importer produces after thresholding
 * (src/assemble.h:240-253).
 */
#ifndef ENB_ORACLE_H
#define ENB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_U8 = 0, ORC_U16 = 1, ORC_F32 = 2 };

enum { ORC_DITHER_HASH = 0, ORC_DITHER_NEAREST = 1 };

enum {
    ORC_EXP_GAUSSIAN = 0,
    ORC_EXP_LORENTZIAN = 1,
    ORC_EXP_HALF_SINE = 2,
    ORC_EXP_FULL_SINE = 3,
    ORC_EXP_BISQUARE = 4
};

enum {
    ORC_GRAY_AVERAGE = 0,
    ORC_GRAY_VALUE = 1,
    ORC_GRAY_ANTI_VALUE = 2,
    ORC_GRAY_LIGHTNESS = 3,
    ORC_GRAY_LUMINANCE = 4,
    ORC_GRAY_MIXER = 5
};

typedef struct {
    double w_exposure;      /* --exposure-weight   (enfuse.cc:117) */
    double w_saturation;    /* --saturation-weight (enfuse.cc:130) */
    double w_contrast;      /* --contrast-weight   (enfuse.cc:129) */
    double w_entropy;       /* --entropy-weight    (enfuse.cc:131) */
    double exp_optimum;     /* --exposure-optimum  (enfuse.cc:118) */
    double exp_width;       /* --exposure-width    (enfuse.cc:119) */
    int exp_function;       /* ORC_EXP_*           (exposure_weight.h:44-128) */
    int contrast_window;    /* --contrast-window-size, odd >= 3 (enfuse.cc:132) */
    int entropy_window;     /* --entropy-window-size, odd >= 3 (enfuse.cc:140) */
    int gray_projector;     /* ORC_GRAY_*          (mga.h:78-87) */
    double mixer[3];        /* channel-mixer weights (mga.h:107-116) */
    /* --exposure-cutoff (enfuse.cc:1272-1340): lower / upper cutoff values,
     * each a percentage of the type's maximum or an absolute value, and the
     * gray projectors (ORC_GRAY_*) that judge them; {0 %, 100 %} is off */
    double exp_cutoff[2];
    int exp_cutoff_pct[2];
    int exp_cutoff_proj[2];
    /* --entropy-cutoff (enfuse.cc:1213-1270): lower / upper clamp of the
     * samples before the entropy windows; {0 %, 100 %} is off */
    double ent_cutoff[2];
    int ent_cutoff_pct[2];
    /* float images: 1 forms the contrast windows' sums as the reference does
     * (float running sums along each row, src/enfuse.h:105-217) instead of
     * exact double window sums */
    int float_sliding_sums;
    /* a user-defined exposure weight function (exposure_weight.cc:44-129)
     * as its values at y = g / max, g = 0..max (integer images); NULL: the
     * built-in exp_function */
    const double* exposure_table;
} orc_enfuse_params;

/* roiBounds level count (src/bounds.h:97-177) for an ROI of w x h. */
int orc_num_levels(int w, int h, int min_levels, int exact_levels);

/* Integer pixel -> fixed point, `v << frac` (src/fixmath.h:197-202). */
void orc_fixed_from_int(const void* src, int dtype, int64_t npix, int C, int pix_stride,
                        int32_t* dst, int frac);

/* Real value -> fixed point, fromRealPromote(v * 2^frac) (src/fixmath.h:189-195). */
void orc_fixed_from_float(const float* src, int64_t n, int32_t* dst, int frac, int bits);

/* Burt-Adelson reduce with alpha (src/pyramid.h:166-573). */
int orc_reduce_alpha(int wrap, const int32_t* src, const uint8_t* alpha, int sw, int sh, int C,
                     int32_t* dst, uint8_t* dst_alpha, int bits);

/* Burt-Adelson reduce without alpha (src/pyramid.h:601-848). */
int orc_reduce(int wrap, const int32_t* src, int sw, int sh, int C, int32_t* dst, int bits);

/* Burt-Adelson expand; add=0: dst -= E(src), add=1: dst = fromPromote(dst + E(src))
 * (src/pyramid.h:875-1457). */
int orc_expand(int add, int wrap, const int32_t* src, int sw, int sh,
               int32_t* dst, int dw, int dh, int C, int bits);

/* enblend's CartesianBlendFunctor over one level; result written into black
 * (src/blend.h:41-121). */
void orc_blend(const int32_t* mask, const int32_t* white, int32_t* black, int64_t npix, int C,
               int32_t white_value, int bits);

/* enfuse's ImageMaskMultiplyFunctor (src/enfuse.h:601-620). */
void orc_mask_multiply(int32_t* lp, const int32_t* mask, int64_t npix, int C, int32_t divisor,
                       int bits);

/* resultLP += imageLP with the pyramid type's cast (src/enfuse.h:1576-1588). */
void orc_accumulate(const int32_t* lp, int32_t* res, int64_t n, int bits);

/* Fixed point -> integer pixel with the reference's dither rule, written only
 * where alpha != 0 (src/fixmath.h:241-277, 2158-2294). */
void orc_from_fixed(const int32_t* src, const uint8_t* alpha, int64_t npix, int C,
                    void* dst, int dtype, int pix_stride, int frac, int dither_mode, uint64_t seed);

/* Dither random bits of sample c of pixel `pixel` (shared rule with the CUDA
 * path; only the low frac-1 bits are used). */
uint32_t orc_dither_bits(uint64_t seed, uint64_t pixel, int C, int c, int frac);

/* enfuseMask: exposure, contrast, saturation and entropy weights (src/enfuse.h:962-1212). */
int orc_enfuse_mask(const void* img, int dtype, int w, int h, int C, int pix_stride,
                    const uint8_t* alpha, const orc_enfuse_params* p, float* out);

/* Local standard deviation of the gray image, integer result (src/enfuse.h:75-219). */
int orc_local_stddev(const int32_t* gray, const uint8_t* alpha, int w, int h, int window,
                     int32_t* out);

/* Local entropy per channel, scaled by the channel maximum (src/enfuse.h:222-566). */
int orc_local_entropy(const void* img, int dtype, int w, int h, int C, int pix_stride,
                      const uint8_t* alpha, int window, double* out);

/* Full enfuse fuse (src/enfuse.h:1217-1617), identity colour space.
 * masks_in: optional K float weight maps that replace enfuseMask (--load-masks).
 * level0_out: optional int32 buffer (w*h*C) receiving the collapsed level 0 before
 * the conversion to pixels.  Returns 0 on success. */
int orc_enfuse(int K, const void* const* imgs, const uint8_t* const* alphas, int dtype,
               int w, int h, int C, int pix_stride, const orc_enfuse_params* p,
               int levels, int wrap, int hard_mask, const float* const* masks_in,
               void* out, uint8_t* out_alpha, int dither_mode, uint64_t seed,
               int32_t* level0_out, float* masks_out);

/* enblend's pyramid blend of a white and a black image under a 0/255 seam mask
 * (src/enblend.h:330-510). out receives the black image with the blended ROI. */
int orc_enblend(const void* white, const uint8_t* white_alpha, const void* black,
                const uint8_t* black_alpha, const uint8_t* mask, int dtype, int w, int h,
                int C, int pix_stride, int levels, int wrap, void* out, uint8_t* out_alpha,
                int dither_mode, uint64_t seed, int32_t* level0_out);

/* ---- float images: double pyramids (src/numerictraits.h:185) -------------- */

/* v >= 0 ? 1 + log1p(v) : 1 / (1 - v) (src/fixmath.h:165-187). */
void orc_real_to_pyramid(const float* src, int64_t npix, int C, int pix_stride, double* dst);

/* v >= 1 ? expm1(v - 1) : 1 - 1/v where alpha != 0 (src/fixmath.h:320-329). */
void orc_real_from_pyramid(const double* src, const uint8_t* alpha, int64_t npix, int C, float* dst,
                           int pix_stride);

/* Reduce with alpha of a double level (src/pyramid.h:166-573, real division). */
int orc_reduce_alpha_d(int wrap, const double* src, const uint8_t* alpha, int sw, int sh, int C, double* dst,
                       uint8_t* dst_alpha);

/* Expand into a double level; add=0: dst -= E(src), add=1: dst += E(src). */
int orc_expand_d(int add, int wrap, const double* src, int sw, int sh, double* dst, int dw, int dh, int C);

/* CartesianBlendFunctor on a double level (src/blend.h:41-76). */
void orc_blend_d(const int32_t* mask, const double* white, double* black, int64_t npix, int C, int32_t white_value);

/* ImageMaskMultiplyFunctor on a double level, accumulated into res when res != NULL. */
void orc_mask_multiply_d(double* lp, const int32_t* mask, int64_t npix, int C, int32_t divisor, double* res);

/* enfuseMask of a float image; range replaces NumericTraits<float>::max() in
 * the exposure and entropy weights (FLT_MAX: reference, 1.0: normalised). */
int orc_enfuse_mask_f(const float* img, int w, int h, int C, int pix_stride, const uint8_t* alpha,
                      const orc_enfuse_params* p, double range, float* out);

/* enfuse of float images (double pyramids); level0_out: optional double (h, w, C). */
int orc_enfuse_f(int K, const float* const* imgs, const uint8_t* const* alphas, int w, int h, int C, int pix_stride,
                 const orc_enfuse_params* p, double range, int levels, int wrap, int hard_mask,
                 const float* const* masks_in, float* out, uint8_t* out_alpha, double* level0_out, float* masks_out);

/* enblend of float images (double pyramids); level0_out: optional double (h, w, C). */
int orc_enblend_f(const float* white, const uint8_t* white_alpha, const float* black, const uint8_t* black_alpha,
                  const uint8_t* mask, int w, int h, int C, int pix_stride, int levels, int wrap, float* out,
                  uint8_t* out_alpha, double* level0_out);

/* Seam mask of enblend's nearest-feature transform (src/nearest.h:427-553,
 * the fine mask without optimisation, src/mask.h:1101-1180): 255 where the
 * nearest pixel opaque in white only is nearer than the nearest pixel opaque
 * in black only (Euclidean distances from the Felzenszwalb-Huttenlocher
 * transform in float, src/openmp_vigra.h:257-433), else 0; wrap: the
 * horizontally periodic transform (src/nearest.h:293-342).  Returns 0, or 2
 * when fewer than 4 (w + h) pixels are opaque in one image only in both
 * directions (the reference's "excessive image overlap" exit). */
int orc_nft_mask(const uint8_t* white, const uint8_t* black, int w, int h, int wrap, uint8_t* mask);

#ifdef __cplusplus
}
#endif

#endif /* ENB_ORACLE_H */
