/*
 * enb_oracle.c -- CPU restatement of the enblend/enfuse multiresolution hot path.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline); see
 * enb_oracle.h.  The reduce/expand operators are written as direct per-pixel
 * formulas (weights and divisors per output position) rather than the
 * reference's SKIPSM raster state machines; the divisor tables they produce are
 * the ones implied by src/pyramid.h:875-1419.  Pyramid passes run serially and
 * pointwise passes under OpenMP, which is the parallel structure of the
 * reference (src/pyramid.h has no OpenMP; src/openmp_vigra.h parallelises the
 * pointwise wrappers).
 *
 * Must be compiled with -ffp-contract=off and without -ffast-math: several
 * steps reproduce the reference's IEEE double expressions exactly.
 */
#include "enb_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* VIGRA NumericTraits conversions used by the reference.                     */
/* ------------------------------------------------------------------------- */

/* NumericTraits<int>::fromRealPromote: round half away from zero via +-0.5 and a
 * truncating cast, saturating at the type limits. */
static inline int32_t frp_i32(double v)
{
    if (v < 0.0) {
        return v < (double)INT_MIN ? INT_MIN : (int32_t)(v - 0.5);
    }
    return v > (double)INT_MAX ? INT_MAX : (int32_t)(v + 0.5);
}

static inline int32_t frp_i16(double v)
{
    if (v < 0.0) {
        return v < (double)SHRT_MIN ? SHRT_MIN : (int32_t)(short)(v - 0.5);
    }
    return v > (double)SHRT_MAX ? SHRT_MAX : (int32_t)(short)(v + 0.5);
}

static inline int32_t frp_bits(double v, int bits) { return bits == 16 ? frp_i16(v) : frp_i32(v); }

static inline uint32_t frp_unsigned(double v, uint32_t maxv)
{
    if (v < 0.0) {
        return 0u;
    }
    return v > (double)maxv ? maxv : (uint32_t)(v + 0.5);
}

/* Assignment through the pyramid accessor: static_cast to the pyramid type. */
static inline int32_t cast_bits(int64_t v, int bits)
{
    return bits == 16 ? (int32_t)(int16_t)(uint16_t)(v & 0xffff) : (int32_t)(uint32_t)(v & 0xffffffffu);
}

/* NumericTraits<PyramidType>::fromPromote: saturate for Int16, identity for Int32. */
static inline int32_t fp_bits(int64_t v, int bits)
{
    if (bits == 16) {
        return v < SHRT_MIN ? SHRT_MIN : (v > SHRT_MAX ? SHRT_MAX : (int32_t)v);
    }
    return (int32_t)v;
}

static inline int imod(int a, int m)
{
    int r = a % m;
    return r < 0 ? r + m : r;
}

static inline uint32_t sample_int(const void* src, int dtype, int64_t i)
{
    return dtype == ORC_U8 ? ((const uint8_t*)src)[i] : ((const uint16_t*)src)[i];
}

/* ------------------------------------------------------------------------- */
/* roiBounds level count, src/bounds.h:121-133.                              */
/* ------------------------------------------------------------------------- */

int orc_num_levels(int w, int h, int min_levels, int exact_levels)
{
    const int max_levels = 29; /* MAX_PYRAMID_LEVELS, src/common.h:55 */
    unsigned int shortdim = (unsigned int)(w < h ? w : h);
    int allowable = min_levels;
    while (allowable <= max_levels) {
        if (shortdim <= 8u) {
            break;
        }
        shortdim = (shortdim + 1u) >> 1;
        ++allowable;
    }
    if (allowable > min_levels) {
        if (exact_levels >= 1) {
            if (exact_levels < allowable) {
                allowable = exact_levels;
            }
        } else if (exact_levels < 0) {
            if (allowable + exact_levels >= min_levels) {
                allowable += exact_levels;
            } else {
                allowable = min_levels;
            }
        }
    }
    return allowable;
}

/* ------------------------------------------------------------------------- */
/* Conversions to fixed point, src/fixmath.h:189-202.                        */
/* ------------------------------------------------------------------------- */

void orc_fixed_from_int(const void* src, int dtype, int64_t npix, int C, int pix_stride,
                        int32_t* dst, int frac)
{
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npix; ++p) {
        for (int c = 0; c < C; ++c) {
            dst[p * C + c] = (int32_t)(sample_int(src, dtype, p * pix_stride + c) << frac);
        }
    }
}

void orc_fixed_from_float(const float* src, int64_t n, int32_t* dst, int frac, int bits)
{
    const double scale = (double)(1u << frac);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        dst[i] = frp_bits((double)src[i] * scale, bits);
    }
}

/* ------------------------------------------------------------------------- */
/* Reduce, src/pyramid.h:166-848.                                             */
/* ------------------------------------------------------------------------- */

static const int W5[5] = {1, 4, 6, 4, 1};

/* Normalised 5x5 binomial over the opaque taps; taps outside the image are
 * dropped, columns wrap when `wrap` (periodic x, src/pyramid.h:234-244). */
int orc_reduce_alpha(int wrap, const int32_t* src, const uint8_t* alpha, int sw, int sh, int C,
                     int32_t* dst, uint8_t* dst_alpha, int bits)
{
    if (sw <= 1 || sh <= 1 || C > 4) {
        return -1; /* vigra_precondition "src image too small in reduce" */
    }
    const int dw = (sw + 1) >> 1, dh = (sh + 1) >> 1;
    for (int Y = 0; Y < dh; ++Y) {
        for (int X = 0; X < dw; ++X) {
            int64_t num[4] = {0, 0, 0, 0};
            int64_t den = 0;
            for (int j = -2; j <= 2; ++j) {
                const int y = 2 * Y + j;
                if (y < 0 || y >= sh) {
                    continue;
                }
                for (int i = -2; i <= 2; ++i) {
                    int x = 2 * X + i;
                    if (wrap) {
                        x = imod(x, sw);
                    } else if (x < 0 || x >= sw) {
                        continue;
                    }
                    const int64_t p = (int64_t)y * sw + x;
                    if (alpha[p]) {
                        const int wgt = W5[j + 2] * W5[i + 2];
                        den += wgt;
                        for (int c = 0; c < C; ++c) {
                            num[c] += (int64_t)wgt * src[p * C + c];
                        }
                    }
                }
            }
            const int64_t q = (int64_t)Y * dw + X;
            if (den > 0) {
                for (int c = 0; c < C; ++c) {
                    dst[q * C + c] = cast_bits(num[c] / den, bits);
                }
                dst_alpha[q] = 255;
            } else {
                for (int c = 0; c < C; ++c) {
                    dst[q * C + c] = 0;
                }
                dst_alpha[q] = 0;
            }
        }
    }
    return 0;
}

/* 5x5 binomial / 256 with clamp-to-edge replication in y (and in x unless
 * `wrap`), src/pyramid.h:646-847. */
int orc_reduce(int wrap, const int32_t* src, int sw, int sh, int C, int32_t* dst, int bits)
{
    if (sw <= 1 || sh <= 1 || C > 4) {
        return -1;
    }
    const int dw = (sw + 1) >> 1, dh = (sh + 1) >> 1;
    for (int Y = 0; Y < dh; ++Y) {
        for (int X = 0; X < dw; ++X) {
            int64_t num[4] = {0, 0, 0, 0};
            for (int j = -2; j <= 2; ++j) {
                int y = 2 * Y + j;
                y = y < 0 ? 0 : (y >= sh ? sh - 1 : y);
                for (int i = -2; i <= 2; ++i) {
                    int x = 2 * X + i;
                    if (wrap) {
                        x = imod(x, sw);
                    } else {
                        x = x < 0 ? 0 : (x >= sw ? sw - 1 : x);
                    }
                    const int wgt = W5[j + 2] * W5[i + 2];
                    for (int c = 0; c < C; ++c) {
                        num[c] += (int64_t)wgt * src[((int64_t)y * sw + x) * C + c];
                    }
                }
            }
            for (int c = 0; c < C; ++c) {
                dst[((int64_t)Y * dw + X) * C + c] = cast_bits(num[c] / 256, bits);
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Expand, src/pyramid.h:875-1457.                                            */
/* ------------------------------------------------------------------------- */

/* Horizontal taps of destination column X.  Even columns interpolate with
 * (1,6,1), odd columns with (4,4); the divisor is the sum of the weights whose
 * taps lie inside the source.  With wrap-around, an odd destination width puts
 * weight 4 on the wrapped neighbour of the first and the last even column
 * (divisor 11, src/pyramid.h:1058-1078, 1153-1161), and a one-column source
 * keeps the wrapped state as an extra numerator term over the plain divisor 6
 * (src/pyramid.h:1233-1236, 1304-1307). */
static void expand_htaps(int X, int sw, int dw, int wrap, int idx[3], int wt[3], int* n, int* den)
{
    const int i = X >> 1;
    int cnt = 0, d = 0;
    if ((X & 1) == 0) {
        if (wrap && sw == 1) {
            idx[0] = 0;
            wt[0] = (dw & 1) ? 10 : 7;
            *n = 1;
            *den = 6;
            return;
        }
        int cand[3] = {i - 1, i, i + 1};
        int cw[3] = {1, 6, 1};
        if (wrap && (dw & 1)) {
            if (i == 0) {
                cw[0] = 4;
            }
            if (i == sw - 1) {
                cw[2] = 4;
            }
        }
        for (int k = 0; k < 3; ++k) {
            int t = cand[k];
            if (wrap) {
                t = imod(t, sw);
            } else if (t < 0 || t >= sw) {
                continue;
            }
            idx[cnt] = t;
            wt[cnt] = cw[k];
            d += cw[k];
            ++cnt;
        }
    } else {
        int cand[2] = {i, i + 1};
        for (int k = 0; k < 2; ++k) {
            int t = cand[k];
            if (wrap && sw > 1) {
                t = imod(t, sw);
            } else if (t < 0 || t >= sw) {
                continue;
            }
            idx[cnt] = t;
            wt[cnt] = 4;
            d += 4;
            ++cnt;
        }
    }
    *n = cnt;
    *den = d;
}

/* Vertical taps of destination row Y: (1,6,1) for even rows, (1,1) for odd
 * rows, taps outside the source dropped (no wrap-around in y). */
static void expand_vtaps(int Y, int sh, int idx[3], int wt[3], int* n, int* den)
{
    const int j = Y >> 1;
    int cnt = 0, d = 0;
    if ((Y & 1) == 0) {
        const int cand[3] = {j - 1, j, j + 1};
        const int cw[3] = {1, 6, 1};
        for (int k = 0; k < 3; ++k) {
            if (cand[k] >= 0 && cand[k] < sh) {
                idx[cnt] = cand[k];
                wt[cnt] = cw[k];
                d += cw[k];
                ++cnt;
            }
        }
    } else {
        const int cand[2] = {j, j + 1};
        for (int k = 0; k < 2; ++k) {
            if (cand[k] >= 0 && cand[k] < sh) {
                idx[cnt] = cand[k];
                wt[cnt] = 1;
                d += 1;
                ++cnt;
            }
        }
    }
    *n = cnt;
    *den = d;
}

int orc_expand(int add, int wrap, const int32_t* src, int sw, int sh,
               int32_t* dst, int dw, int dh, int C, int bits)
{
    if (sw < 1 || sh < 1 || sw != ((dw + 1) >> 1) || sh != ((dh + 1) >> 1) || C > 4) {
        return -1;
    }
    for (int Y = 0; Y < dh; ++Y) {
        int vi[3], vw[3], vn, vd;
        expand_vtaps(Y, sh, vi, vw, &vn, &vd);
        for (int X = 0; X < dw; ++X) {
            int hi[3], hw[3], hn, hd;
            expand_htaps(X, sw, dw, wrap, hi, hw, &hn, &hd);
            const int64_t den = (int64_t)hd * vd;
            for (int c = 0; c < C; ++c) {
                int64_t num = 0;
                for (int a = 0; a < vn; ++a) {
                    int64_t row = 0;
                    for (int b = 0; b < hn; ++b) {
                        row += (int64_t)hw[b] * src[((int64_t)vi[a] * sw + hi[b]) * C + c];
                    }
                    num += vw[a] * row;
                }
                const int64_t e = num / den;
                int32_t* d = &dst[((int64_t)Y * dw + X) * C + c];
                *d = add ? fp_bits((int64_t)*d + e, bits) : cast_bits((int64_t)*d - e, bits);
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Merge operators.                                                           */
/* ------------------------------------------------------------------------- */

/* CartesianBlendFunctor, src/blend.h:41-76. */
void orc_blend(const int32_t* mask, const int32_t* white, int32_t* black, int64_t npix, int C,
               int32_t white_value, int bits)
{
    const double wv = (double)white_value;
#pragma omp parallel for schedule(guided)
    for (int64_t p = 0; p < npix; ++p) {
        const double wc = (double)mask[p] / wv;
        if (wc >= 1.0) {
            for (int c = 0; c < C; ++c) {
                black[p * C + c] = white[p * C + c];
            }
        } else if (wc <= 0.0) {
            /* keep black */
        } else {
            const double bc = 1.0 - wc;
            for (int c = 0; c < C; ++c) {
                const double a = wc * (double)white[p * C + c];
                const double b = bc * (double)black[p * C + c];
                black[p * C + c] = frp_bits(a + b, bits);
            }
        }
    }
}

/* ImageMaskMultiplyFunctor, src/enfuse.h:601-620. */
void orc_mask_multiply(int32_t* lp, const int32_t* mask, int64_t npix, int C, int32_t divisor,
                       int bits)
{
    const double dv = (double)divisor;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npix; ++p) {
        const double coeff = (double)mask[p] / dv;
        for (int c = 0; c < C; ++c) {
            lp[p * C + c] = frp_bits((double)lp[p * C + c] * coeff, bits);
        }
    }
}

/* vigra Arg1()+Arg2() into the pyramid type (static_cast), src/enfuse.h:1579-1582. */
void orc_accumulate(const int32_t* lp, int32_t* res, int64_t n, int bits)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        res[i] = cast_bits((int64_t)lp[i] + res[i], bits);
    }
}

/* ------------------------------------------------------------------------- */
/* Conversion from fixed point, src/fixmath.h:241-277.                        */
/* ------------------------------------------------------------------------- */

/* 32-bit integer finaliser (public-domain "lowbias32" constants by C. Wellons). */
static inline uint32_t mix32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

/* Random bits of the dither: one hash per pixel, 8 bits per channel when
 * the rule needs at most 8 bits per sample and the pixel has at most four
 * samples, otherwise one hash per sample.  The pixel index wraps at 2^32. */
static inline uint32_t dither_key(uint64_t seed)
{
    return mix32((uint32_t)(seed >> 32) ^ 0x9e3779b9u) ^ (uint32_t)seed;
}

uint32_t orc_dither_bits(uint64_t seed, uint64_t pixel, int C, int c, int frac)
{
    const uint32_t key = dither_key(seed);
    if (frac - 1 <= 8 && C <= 4) {
        return mix32((uint32_t)pixel ^ key) >> (8 * c);
    }
    return mix32((uint32_t)(pixel * (uint64_t)C + (uint64_t)c) ^ key);
}

void orc_from_fixed(const int32_t* src, const uint8_t* alpha, int64_t npix, int C,
                    void* dst, int dtype, int pix_stride, int frac, int dither_mode, uint64_t seed)
{
    const int32_t half_m1 = (1 << (frac - 1)) - 1;
    const int32_t quarter = 1 << (frac - 2);
    const int32_t three_quarter = 3 << (frac - 2);
    const int32_t half = 1 << (frac - 1);
    const int32_t maxv = dtype == ORC_U8 ? 255 : 65535;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npix; ++p) {
        if (!alpha[p]) {
            continue;
        }
        for (int c = 0; c < C; ++c) {
            const int32_t v = src[p * C + c];
            const int32_t q = v >> frac;            /* arithmetic shift: floor */
            const int32_t f = v & ((1 << frac) - 1);
            int32_t r;
            if (dither_mode == ORC_DITHER_NEAREST) {
                r = f >= half ? q + 1 : q;
            } else if (f >= quarter && f < three_quarter) {
                const int32_t rnd =
                    (int32_t)(orc_dither_bits(seed, (uint64_t)p, C, c, frac) & (uint32_t)half_m1) + quarter;
                r = rnd <= f ? q + 1 : q;
            } else if (f >= quarter) {
                r = q + 1;
            } else {
                r = q;
            }
            r = r < 0 ? 0 : (r > maxv ? maxv : r); /* fromPromote */
            if (dtype == ORC_U8) {
                ((uint8_t*)dst)[p * pix_stride + c] = (uint8_t)r;
            } else {
                ((uint16_t*)dst)[p * pix_stride + c] = (uint16_t)r;
            }
        }
    }
}

/* The alpha component of an RGBA result: the union alpha scaled to the
 * sample type, as the output writer stores the alpha image
 * (src/assemble.h:133-225). */
static void write_alpha_component(void* dst, int dtype, int64_t npix, const uint8_t* alpha)
{
    if (dtype == ORC_U8) {
        for (int64_t p = 0; p < npix; ++p) {
            ((uint8_t*)dst)[p * 4 + 3] = alpha[p] ? 255 : 0;
        }
    } else {
        for (int64_t p = 0; p < npix; ++p) {
            ((uint16_t*)dst)[p * 4 + 3] = alpha[p] ? 65535 : 0;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Pyramid builders, src/pyramid.h:1468-1784.                                */
/* ------------------------------------------------------------------------- */

typedef struct {
    int levels;
    int C;
    int w[30], h[30];
    int32_t* lv[30];
} pyr_t;

static void pyr_alloc(pyr_t* p, int levels, int w, int h, int C)
{
    p->levels = levels;
    p->C = C;
    for (int l = 0; l < levels; ++l) {
        p->w[l] = w;
        p->h[l] = h;
        p->lv[l] = (int32_t*)calloc((size_t)w * h * C, sizeof(int32_t));
        w = (w + 1) >> 1;
        h = (h + 1) >> 1;
    }
}

static void pyr_free(pyr_t* p)
{
    for (int l = 0; l < p->levels; ++l) {
        free(p->lv[l]);
    }
}

/* gaussianPyramid with alpha: level 0 already in p->lv[0]; the first reduce
 * uses the given alpha, later ones the reduced binary alpha (pyramid.h:1500-1530). */
static int gaussian_alpha(pyr_t* p, const uint8_t* alpha0, int wrap, int bits)
{
    const uint8_t* a = alpha0;
    uint8_t* owned = NULL;
    for (int l = 1; l < p->levels; ++l) {
        uint8_t* na = (uint8_t*)malloc((size_t)p->w[l] * p->h[l]);
        const int rc = orc_reduce_alpha(wrap, p->lv[l - 1], a, p->w[l - 1], p->h[l - 1], p->C,
                                        p->lv[l], na, bits);
        free(owned);
        owned = na;
        a = na;
        if (rc) {
            free(owned);
            return rc;
        }
    }
    free(owned);
    return 0;
}

static int gaussian_noalpha(pyr_t* p, int wrap, int bits)
{
    for (int l = 1; l < p->levels; ++l) {
        const int rc = orc_reduce(wrap, p->lv[l - 1], p->w[l - 1], p->h[l - 1], p->C, p->lv[l], bits);
        if (rc) {
            return rc;
        }
    }
    return 0;
}

/* laplacianPyramid: gp[l] -= expand(gp[l+1]) for l = 0..L-2 (pyramid.h:1672-1736). */
static int laplacian_inplace(pyr_t* p, int wrap, int bits)
{
    for (int l = 0; l + 1 < p->levels; ++l) {
        const int rc = orc_expand(0, wrap, p->lv[l + 1], p->w[l + 1], p->h[l + 1], p->lv[l],
                                  p->w[l], p->h[l], p->C, bits);
        if (rc) {
            return rc;
        }
    }
    return 0;
}

/* collapsePyramid: p[l] = fromPromote(p[l] + expand(p[l+1])), l = L-2..0 (pyramid.h:1758-1784). */
static int collapse(pyr_t* p, int wrap, int bits)
{
    for (int l = p->levels - 2; l >= 0; --l) {
        const int rc = orc_expand(1, wrap, p->lv[l + 1], p->w[l + 1], p->h[l + 1], p->lv[l],
                                  p->w[l], p->h[l], p->C, bits);
        if (rc) {
            return rc;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Enfuse weights, src/enfuse.h:64-1212 and src/mga.h.                       */
/* ------------------------------------------------------------------------- */

#define FWHM_GAUSSIAN_C 2.3548200450309493820231386529193992755
#define FWHM_LORENTZIAN_C 2.8284271247461900976033774484193961571
#define FWHM_HALFSINE_C 2.0943951023931954923084289221863352561
#define FWHM_FULLSINE_C 3.14159265358979323846
#define FWHM_BISQUARE_C 1.6817928305074290860622509524664297901

/* Effective width of the built-in exposure weight functions: each rescales the
 * user width to the Gaussian's FWHM (exposure_weight.h:56-116). */
static double exposure_effective_width(int fn, double width)
{
    switch (fn) {
    case ORC_EXP_LORENTZIAN: return width * FWHM_GAUSSIAN_C / FWHM_LORENTZIAN_C;
    case ORC_EXP_HALF_SINE: return width * FWHM_GAUSSIAN_C / FWHM_HALFSINE_C;
    case ORC_EXP_FULL_SINE: return width * FWHM_GAUSSIAN_C / FWHM_FULLSINE_C;
    case ORC_EXP_BISQUARE: return width * FWHM_GAUSSIAN_C / FWHM_BISQUARE_C;
    default: return width;
    }
}

/* ExposureWeight::weight of the built-ins (exposure_weight.h:44-128). */
static double exposure_weight(int fn, double y, double opt, double eff_width)
{
    const double z = (y - opt) / eff_width;
    switch (fn) {
    case ORC_EXP_LORENTZIAN: return 1.0 / (1.0 + 0.5 * z * z);
    case ORC_EXP_HALF_SINE: return fabs(z) <= 1.57079632679489661923 ? cos(z) : 0.0;
    case ORC_EXP_FULL_SINE: return fabs(z) <= 3.14159265358979323846 ? 0.5 + cos(z) / 2.0 : 0.0;
    case ORC_EXP_BISQUARE:
        if (fabs(z) <= 1.0) {
            const double z2 = z * z;
            return (1.0 - z2) * (1.0 + z2);
        }
        return 0.0;
    default: return exp(-0.5 * z * z);
    }
}

/* MultiGrayscaleAccessor::project for integer RGB pixels, result rounded to
 * an integer by fromRealPromote (mga.h:185-222). */
static int32_t gray_int(const orc_enfuse_params* prm, int32_t r, int32_t g, int32_t b,
                        uint32_t maxv, double mw0, double mw1, double mw2)
{
    switch (prm->gray_projector) {
    case ORC_GRAY_VALUE: {
        int32_t m = r > g ? r : g;
        return m > b ? m : b;
    }
    case ORC_GRAY_ANTI_VALUE: {
        int32_t m = r < g ? r : g;
        return m < b ? m : b;
    }
    case ORC_GRAY_LIGHTNESS: {
        int32_t mn = r < g ? r : g;
        mn = mn < b ? mn : b;
        int32_t mx = r > g ? r : g;
        mx = mx > b ? mx : b;
        return (int32_t)frp_unsigned((double)(mn + mx) / 2.0, maxv);
    }
    case ORC_GRAY_LUMINANCE:
        return (int32_t)frp_unsigned(0.3 * r + 0.59 * g + 0.11 * b, maxv);
    case ORC_GRAY_MIXER:
        return (int32_t)frp_unsigned(mw0 * (double)r + mw1 * (double)g + mw2 * (double)b, maxv);
    default:
        return (int32_t)frp_unsigned(((double)r + (double)g + (double)b) / 3.0, maxv);
    }
}

/* AlternativePercentage / CompactifiedAlternativePercentage
 * (src/alternativepercentage.h:31-97): is_effective<t> and instantiate<t>
 * for a sample type whose maximum is `maxv` (the float maximum for float
 * images).  instantiate converts to the sample type: truncation toward zero
 * for the integer types, rounding to float for float images. */
static int cutoff_effective(double v, int pct, double maxv, int compactified)
{
    if (compactified) {
        return v != 0.0 && ((pct && fabs(v) != 100.0) || (!pct && v != maxv));
    }
    return v > 0.0 && ((pct && v < 100.0) || (!pct && v < maxv));
}

static double cutoff_value(double v, int pct, double maxv, int integral, int compactified)
{
    double c;
    if (compactified) {
        c = pct ? (v >= 0.0 ? v : 100.0 + v) * maxv / 100.0 : (v >= 0.0 ? v : maxv + v);
    } else {
        c = pct ? v * maxv / 100.0 : v;
    }
    return integral ? trunc(c) : (double)(float)c;
}

/* The exposure cutoff of one image type: *active, and the lower and upper
 * limits (src/enfuse.h:655-690).  The upper limit is a compactified
 * percentage, a negative value counting down from the maximum, as the
 * option is documented (doc/enfuse-expert-fusion-options.tex:184-185) and as
 * the reference judges its activity; the reference's functor instantiates it
 * through the plain base class instead, which converts a negative limit to
 * the unsigned sample type (undefined behaviour), so the two agree for every
 * non-negative limit.  -3 for the reference's fatal cases (negative limits,
 * lower above upper). */
static int exposure_cutoffs(const orc_enfuse_params* prm, double maxv, int integral, int* active, double* lo,
                            double* hi)
{
    *active = cutoff_effective(prm->exp_cutoff[0], prm->exp_cutoff_pct[0], maxv, 0) ||
              cutoff_effective(prm->exp_cutoff[1], prm->exp_cutoff_pct[1], maxv, 1);
    if (!*active) {
        return 0;
    }
    *lo = cutoff_value(prm->exp_cutoff[0], prm->exp_cutoff_pct[0], maxv, integral, 0);
    *hi = cutoff_value(prm->exp_cutoff[1], prm->exp_cutoff_pct[1], maxv, integral, 1);
    return (*lo < 0.0 || *hi < 0.0 || *lo > *hi) ? -3 : 0;
}

/* The entropy cutoff (src/enfuse.h:1145-1192): lower as a plain, upper as a
 * compactified AlternativePercentage. */
static int entropy_cutoffs(const orc_enfuse_params* prm, double maxv, int integral, int* active, double* lo,
                           double* hi)
{
    *active = cutoff_effective(prm->ent_cutoff[0], prm->ent_cutoff_pct[0], maxv, 0) ||
              cutoff_effective(prm->ent_cutoff[1], prm->ent_cutoff_pct[1], maxv, 1);
    if (!*active) {
        return 0;
    }
    *lo = cutoff_value(prm->ent_cutoff[0], prm->ent_cutoff_pct[0], maxv, integral, 0);
    *hi = cutoff_value(prm->ent_cutoff[1], prm->ent_cutoff_pct[1], maxv, integral, 1);
    return (*lo < 0.0 || *hi < 0.0 || *lo > *hi) ? -3 : 0;
}

/* ClampingFunctor of the entropy cutoff (src/enfuse.h:893-925): per sample
 * x <= lo -> 0, x >= hi -> max, else x; the third (blue) sample is tested
 * against the first sample's lower limit, as the reference does. */
static void clamp_rgb_u32(uint32_t* px, int C, double lo, double hi, uint32_t maxv)
{
    const int red_low = (double)px[0] <= lo;
    for (int c = 0; c < C; ++c) {
        const int low = (C == 3 && c == 2) ? red_low : ((double)px[c] <= lo);
        px[c] = low ? 0u : ((double)px[c] >= hi ? maxv : px[c]);
    }
}

int orc_local_stddev(const int32_t* gray, const uint8_t* alpha, int w, int h, int window,
                     int32_t* out)
{
    if (window < 2 || w < window || h < window) {
        return -1;
    }
    const int b = window / 2;
#pragma omp parallel for schedule(static)
    for (int y = b; y < h - b; ++y) {
        for (int x = b; x < w - b; ++x) {
            if (!alpha[(int64_t)y * w + x]) {
                continue;
            }
            double sum = 0.0, sumsq = 0.0;
            size_t n = 0;
            for (int yy = y - b; yy <= y + b; ++yy) {
                for (int xx = x - b; xx <= x + b; ++xx) {
                    const int64_t p = (int64_t)yy * w + xx;
                    if (alpha[p]) {
                        const double v = (double)gray[p];
                        sum += v;
                        sumsq += v * v;
                        ++n;
                    }
                }
            }
            const double r = n <= 1 ? 0.0 : sqrt((sumsq - sum * sum / (double)n) / (double)(n - 1));
            out[(int64_t)y * w + x] = frp_i32(r);
        }
    }
    return 0;
}

static int cmp_u32(const void* a, const void* b)
{
    const uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* Histogram::entropyOfChannel (enfuse.h:346-375): bins visited in ascending
 * key order, p = count/total, H = -sum(p log p) / log(#bins). */
static double entropy_of(uint32_t* vals, int n)
{
    if (n == 0) {
        return 0.0;
    }
    qsort(vals, (size_t)n, sizeof(uint32_t), cmp_u32);
    int bins = 1;
    for (int i = 1; i < n; ++i) {
        bins += vals[i] != vals[i - 1];
    }
    if (bins <= 1) {
        return 0.0;
    }
    double e = 0.0;
    int i = 0;
    while (i < n) {
        int j = i;
        while (j < n && vals[j] == vals[i]) {
            ++j;
        }
        const double p = (double)(unsigned)(j - i) / (double)(unsigned)n;
        e += p * log(p);
        i = j;
    }
    return -e / log((double)bins);
}

static int local_entropy_clamped(const void* img, int dtype, int w, int h, int C, int pix_stride,
                                 const uint8_t* alpha, int window, int clamp, double lo, double hi, double* out);

int orc_local_entropy(const void* img, int dtype, int w, int h, int C, int pix_stride,
                      const uint8_t* alpha, int window, double* out)
{
    return local_entropy_clamped(img, dtype, w, h, C, pix_stride, alpha, window, 0, 0.0, 0.0, out);
}

/* localEntropyIf (src/enfuse.h:458-566) of the image, its samples first
 * clamped by the entropy cutoff when `clamp` is set. */
static int local_entropy_clamped(const void* img, int dtype, int w, int h, int C, int pix_stride,
                                 const uint8_t* alpha, int window, int clamp, double lo, double hi, double* out)
{
    if (w < window || h < window || dtype == ORC_F32) {
        return -1;
    }
    const int b = window / 2;
    const double maxv = dtype == ORC_U8 ? 255.0 : 65535.0;
#pragma omp parallel
    {
        uint32_t* vals = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)window * window);
#pragma omp for schedule(static)
        for (int y = b; y < h - b; ++y) {
            for (int x = b; x < w - b; ++x) {
                if (!alpha[(int64_t)y * w + x]) {
                    continue;
                }
                for (int c = 0; c < C; ++c) {
                    int n = 0;
                    for (int yy = y - b; yy <= y + b; ++yy) {
                        for (int xx = x - b; xx <= x + b; ++xx) {
                            const int64_t p = (int64_t)yy * w + xx;
                            if (alpha[p]) {
                                if (clamp) {
                                    uint32_t px[3];
                                    for (int k = 0; k < C; ++k) {
                                        px[k] = sample_int(img, dtype, p * pix_stride + k);
                                    }
                                    clamp_rgb_u32(px, C, lo, hi, (uint32_t)maxv);
                                    vals[n++] = px[c];
                                } else {
                                    vals[n++] = sample_int(img, dtype, p * pix_stride + c);
                                }
                            }
                        }
                    }
                    out[((int64_t)y * w + x) * C + c] = entropy_of(vals, n) * maxv;
                }
            }
        }
        free(vals);
    }
    return 0;
}

int orc_enfuse_mask(const void* img, int dtype, int w, int h, int C, int pix_stride,
                    const uint8_t* alpha, const orc_enfuse_params* prm, float* out)
{
    if (dtype == ORC_F32 || (C != 1 && C != 3)) {
        return -2; /* float images are handled by the float path */
    }
    const int64_t npix = (int64_t)w * h;
    const uint32_t maxv = dtype == ORC_U8 ? 255u : 65535u;
    double mw0 = 0, mw1 = 0, mw2 = 0;
    if (prm->gray_projector == ORC_GRAY_MIXER) {
        const double s = prm->mixer[0] + prm->mixer[1] + prm->mixer[2];
        mw0 = prm->mixer[0] / s;
        mw1 = prm->mixer[1] / s;
        mw2 = prm->mixer[2] / s;
    }
    int32_t* gray = (int32_t*)malloc(sizeof(int32_t) * (size_t)npix);
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npix; ++p) {
        if (C == 1) {
            gray[p] = (int32_t)sample_int(img, dtype, p * pix_stride);
        } else {
            gray[p] = gray_int(prm, (int32_t)sample_int(img, dtype, p * pix_stride),
                               (int32_t)sample_int(img, dtype, p * pix_stride + 1),
                               (int32_t)sample_int(img, dtype, p * pix_stride + 2), maxv, mw0, mw1, mw2);
        }
    }
    memset(out, 0, sizeof(float) * (size_t)npix);

    /* Exposure (enfuse.h:974-1010, 623-730), with the cutoff when active. */
    if (prm->w_exposure > 0.0) {
        const double ew = exposure_effective_width(prm->exp_function, prm->exp_width);
        int cut = 0;
        double lo = 0.0, hi = 0.0;
        const int rc = exposure_cutoffs(prm, (double)maxv, 1, &cut, &lo, &hi);
        if (rc) {
            free(gray);
            return rc;
        }
        /* the projectors that judge the lower and the upper limit
         * (enfuse.h:982-986; the caller resolves the reference's fallbacks
         * between empty projector names) */
        orc_enfuse_params lp = *prm, up = *prm;
        lp.gray_projector = prm->exp_cutoff_proj[0];
        up.gray_projector = prm->exp_cutoff_proj[1];
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < npix; ++p) {
            if (!alpha[p]) {
                continue;
            }
            if (cut) {
                double lv, uv;
                if (C == 1) {
                    lv = uv = (double)gray[p];
                } else {
                    const int32_t r = (int32_t)sample_int(img, dtype, p * pix_stride);
                    const int32_t g = (int32_t)sample_int(img, dtype, p * pix_stride + 1);
                    const int32_t b = (int32_t)sample_int(img, dtype, p * pix_stride + 2);
                    lv = (double)gray_int(&lp, r, g, b, maxv, mw0, mw1, mw2);
                    uv = (double)gray_int(&up, r, g, b, maxv, mw0, mw1, mw2);
                }
                if (!(lv >= lo && uv <= hi)) {
                    out[p] = 0.0f;
                    continue;
                }
            }
            const double y = (double)gray[p] / (double)maxv;
            /* weight_function_->weight(y): the user's function through its
             * values at the sample values */
            const double f = prm->exposure_table ? prm->exposure_table[gray[p]]
                                                 : exposure_weight(prm->exp_function, y, prm->exp_optimum, ew);
            out[p] = (float)(prm->w_exposure * f);
        }
    }

    /* Contrast (enfuse.h:1013-1122, 783-829). */
    if (prm->w_contrast > 0.0) {
        int32_t* grad = (int32_t*)calloc((size_t)npix, sizeof(int32_t));
        const int rc = orc_local_stddev(gray, alpha, w, h, prm->contrast_window, grad);
        if (rc) {
            free(grad);
            free(gray);
            return rc;
        }
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < npix; ++p) {
            if (alpha[p]) {
                /* the combine lambda takes the gradient as the pixel's scalar type */
                const uint32_t g = dtype == ORC_U8 ? (uint32_t)(uint8_t)grad[p] : (uint32_t)(uint16_t)grad[p];
                const float cw = (float)(prm->w_contrast * (double)(int32_t)g / (double)maxv);
                out[p] = cw + out[p];
            }
        }
        free(grad);
    }

    /* Saturation (enfuse.h:1125-1136, 733-780). */
    if (prm->w_saturation > 0.0 && C == 3) {
        const double max_value = (double)maxv;
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < npix; ++p) {
            if (!alpha[p]) {
                continue;
            }
            const uint32_t r = sample_int(img, dtype, p * pix_stride);
            const uint32_t g = sample_int(img, dtype, p * pix_stride + 1);
            const uint32_t b = sample_int(img, dtype, p * pix_stride + 2);
            uint32_t mx = r > g ? r : g;
            mx = mx > b ? mx : b;
            uint32_t mn = r < g ? r : g;
            mn = mn < b ? mn : b;
            float sw = 0.0f;
            if (mx != mn) {
                const double sum = (double)mx + (double)mn;
                const double diff = (double)mx - (double)mn;
                const double s = sum <= max_value ? diff / sum : diff / (2.0 * max_value - sum);
                sw = (float)(prm->w_saturation * s);
            }
            out[p] = sw + out[p];
        }
    }

    /* Entropy (enfuse.h:1139-1211, 832-861). */
    if (prm->w_entropy > 0.0) {
        int cut = 0;
        double lo = 0.0, hi = 0.0;
        int rc = entropy_cutoffs(prm, (double)maxv, 1, &cut, &lo, &hi);
        if (rc) {
            free(gray);
            return rc;
        }
        double* ent = (double*)calloc((size_t)npix * C, sizeof(double));
        rc = local_entropy_clamped(img, dtype, w, h, C, pix_stride, alpha, prm->entropy_window, cut, lo, hi, ent);
        if (rc) {
            free(ent);
            free(gray);
            return rc;
        }
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < npix; ++p) {
            if (!alpha[p]) {
                continue;
            }
            uint32_t mn = maxv;
            for (int c = 0; c < C; ++c) {
                /* entropy image pixel = fromRealPromote<T>(H * max) */
                const uint32_t e = frp_unsigned(ent[p * C + c], maxv);
                mn = e < mn ? e : mn;
            }
            const float ew = (float)(prm->w_entropy * (double)(float)mn);
            out[p] = ew + out[p];
        }
        free(ent);
    }
    free(gray);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Drivers.                                                                   */
/* ------------------------------------------------------------------------- */

int orc_enfuse(int K, const void* const* imgs, const uint8_t* const* alphas, int dtype,
               int w, int h, int C, int pix_stride, const orc_enfuse_params* prm,
               int levels, int wrap, int hard_mask, const float* const* masks_in,
               void* out, uint8_t* out_alpha, int dither_mode, uint64_t seed,
               int32_t* level0_out, float* masks_out)
{
    if (K < 1 || dtype == ORC_F32 || (C != 1 && C != 3)) {
        return -2;
    }
    const int64_t npix = (int64_t)w * h;
    const int bits = dtype == ORC_U8 ? 16 : 32;      /* numerictraits.h:159-163 */
    const int frac = 7;
    const int mbits = dtype == ORC_U8 ? 16 : 32;
    const int mfrac = dtype == ORC_U8 ? 7 : 15;
    const int32_t max_mask_pyr = 255 << mfrac;       /* enfuse.h:1554-1558 */
    int rc = 0;

    float** masks = (float**)malloc(sizeof(float*) * (size_t)K);
    float* norm = (float*)calloc((size_t)npix, sizeof(float));
    memset(out_alpha, 0, (size_t)npix);
    for (int k = 0; k < K; ++k) {
        masks[k] = (float*)malloc(sizeof(float) * (size_t)npix);
        if (masks_in) {
            memcpy(masks[k], masks_in[k], sizeof(float) * (size_t)npix);
        } else {
            rc = orc_enfuse_mask(imgs[k], dtype, w, h, C, pix_stride, alphas[k], prm, masks[k]);
            if (rc) {
                goto done;
            }
        }
        for (int64_t p = 0; p < npix; ++p) {
            if (alphas[k][p]) {
                out_alpha[p] = alphas[k][p];            /* copyImageIf, enfuse.h:1377-1379 */
            }
            norm[p] = masks[k][p] + norm[p];            /* enfuse.h:1382-1385 */
        }
    }

    if (hard_mask) {                                    /* enfuse.h:1399-1442 */
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < npix; ++p) {
            float mx = 0.0f;
            int mi = 0;
            for (int k = 0; k < K; ++k) {
                if (masks[k][p] > mx) {
                    mx = masks[k][p];
                    mi = k;
                }
            }
            for (int k = 0; k < K; ++k) {
                masks[k][p] = mx == 0.0f ? 255.0f / (float)K : (k == mi ? 255.0f : 0.0f);
            }
        }
    }

    levels = levels > 0 ? levels : orc_num_levels(w, h, 1, 0);
    pyr_t result;
    memset(&result, 0, sizeof(result));
    for (int k = 0; k < K && rc == 0; ++k) {
        pyr_t lp, mg;
        pyr_alloc(&lp, levels, w, h, C);
        orc_fixed_from_int(imgs[k], dtype, npix, C, pix_stride, lp.lv[0], frac);
        rc = gaussian_alpha(&lp, alphas[k], wrap, bits);
        if (!rc) {
            rc = laplacian_inplace(&lp, wrap, bits);
        }
        if (!hard_mask) {                               /* enfuse.h:1526-1535 */
            const float fallback = (float)(255 / K);
#pragma omp parallel for schedule(static)
            for (int64_t p = 0; p < npix; ++p) {
                masks[k][p] = norm[p] > 0.0f ? (255.0f * masks[k][p]) / norm[p] : fallback;
            }
        }
        if (masks_out) {
            memcpy(masks_out + (size_t)k * npix, masks[k], sizeof(float) * (size_t)npix);
        }
        pyr_alloc(&mg, levels, w, h, 1);
        orc_fixed_from_float(masks[k], npix, mg.lv[0], mfrac, mbits);
        if (!rc) {
            rc = gaussian_alpha(&mg, out_alpha, wrap, mbits);   /* enfuse.h:1539-1546 */
        }
        for (int l = 0; l < levels && !rc; ++l) {
            orc_mask_multiply(lp.lv[l], mg.lv[l], (int64_t)lp.w[l] * lp.h[l], C, max_mask_pyr, bits);
        }
        pyr_free(&mg);
        if (k == 0) {
            result = lp;
        } else {
            for (int l = 0; l < levels; ++l) {
                orc_accumulate(lp.lv[l], result.lv[l], (int64_t)lp.w[l] * lp.h[l] * C, bits);
            }
            pyr_free(&lp);
        }
    }
    if (!rc) {
        rc = collapse(&result, wrap, bits);
    }
    if (!rc) {
        if (level0_out) {
            memcpy(level0_out, result.lv[0], sizeof(int32_t) * (size_t)npix * C);
        }
        const size_t esz = dtype == ORC_U8 ? 1 : 2;
        memset(out, 0, esz * (size_t)npix * pix_stride);
        orc_from_fixed(result.lv[0], out_alpha, npix, C, out, dtype, pix_stride, frac, dither_mode, seed);
        if (pix_stride == 4) {
            write_alpha_component(out, dtype, npix, out_alpha);
        }
    }
    pyr_free(&result);
done:
    for (int k = 0; k < K; ++k) {
        if (masks[k]) {
            free(masks[k]);
        }
    }
    free(masks);
    free(norm);
    return rc;
}

int orc_enblend(const void* white, const uint8_t* white_alpha, const void* black,
                const uint8_t* black_alpha, const uint8_t* mask, int dtype, int w, int h,
                int C, int pix_stride, int levels, int wrap, void* out, uint8_t* out_alpha,
                int dither_mode, uint64_t seed, int32_t* level0_out)
{
    if (dtype == ORC_F32 || C > 4) {
        return -2;
    }
    const int64_t npix = (int64_t)w * h;
    const int bits = dtype == ORC_U8 ? 16 : 32;
    const int frac = 7;
    const int mbits = dtype == ORC_U8 ? 16 : 32;
    const int mfrac = dtype == ORC_U8 ? 7 : 15;
    int rc;
    levels = levels > 0 ? levels : orc_num_levels(w, h, 1, 0);

    /* Mask Gaussian pyramid without alpha (enblend.h:384-388). */
    pyr_t mg, wl, bl;
    pyr_alloc(&mg, levels, w, h, 1);
    orc_fixed_from_int(mask, ORC_U8, npix, 1, 1, mg.lv[0], mfrac);
    rc = gaussian_noalpha(&mg, wrap, mbits);

    /* White and black Laplacian pyramids (enblend.h:418-446). */
    pyr_alloc(&wl, levels, w, h, C);
    pyr_alloc(&bl, levels, w, h, C);
    orc_fixed_from_int(white, dtype, npix, C, pix_stride, wl.lv[0], frac);
    orc_fixed_from_int(black, dtype, npix, C, pix_stride, bl.lv[0], frac);
    if (!rc) {
        rc = gaussian_alpha(&wl, white_alpha, wrap, bits);
    }
    if (!rc) {
        rc = laplacian_inplace(&wl, wrap, bits);
    }
    if (!rc) {
        rc = gaussian_alpha(&bl, black_alpha, wrap, bits);
    }
    if (!rc) {
        rc = laplacian_inplace(&bl, wrap, bits);
    }
    /* Black alpha becomes the union (enblend.h:461-464). */
    for (int64_t p = 0; p < npix; ++p) {
        out_alpha[p] = white_alpha[p] ? 255 : black_alpha[p];
    }
    if (!rc) {
        for (int l = 0; l < levels; ++l) {             /* blend.h:81-121 */
            orc_blend(mg.lv[l], wl.lv[l], bl.lv[l], (int64_t)bl.w[l] * bl.h[l], C, 255 << mfrac, bits);
        }
        rc = collapse(&bl, wrap, bits);                 /* enblend.h:503 */
    }
    if (!rc) {
        if (level0_out) {
            memcpy(level0_out, bl.lv[0], sizeof(int32_t) * (size_t)npix * C);
        }
        const size_t esz = dtype == ORC_U8 ? 1 : 2;
        memcpy(out, black, esz * (size_t)npix * pix_stride);
        orc_from_fixed(bl.lv[0], out_alpha, npix, C, out, dtype, pix_stride, frac, dither_mode, seed);
        if (pix_stride == 4) {
            write_alpha_component(out, dtype, npix, out_alpha);
        }
    }
    pyr_free(&mg);
    pyr_free(&wl);
    pyr_free(&bl);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* Float images: double pyramids (src/numerictraits.h:185, float row).        */
/*                                                                            */
/* The reference builds the image pyramids of float images in double with a   */
/* logarithmic mapping, reduces and expands them with real divisions, merges  */
/* them in double and maps level 0 back (src/fixmath.h:165-187, 320-329).     */
/* The mask pyramids stay Int32 9.15 (the integer operators above).  The      */
/* weights of float images are evaluated here in double from their            */
/* definitions; where the reference keeps a running float sum (the sliding   */
/* window of localStdDevIf, src/enfuse.h:75-219) this restatement computes    */
/* the exact window statistics instead.                                       */
/* ------------------------------------------------------------------------- */

/* ConvertScalarToPyramidFunctor, real -> real (src/fixmath.h:165-187).  The
 * functor's argument is the float sample, so the C++ overload log1p(float)
 * is the one called: the logarithm is a float, the sum 1.0 + it a double
 * (this reproduces the reference's double pyramid to the last bit). */
void orc_real_to_pyramid(const float* src, int64_t npix, int C, int pix_stride, double* dst)
{
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npix; ++p) {
        for (int c = 0; c < C; ++c) {
            const double v = (double)src[p * pix_stride + c];
            dst[p * C + c] = v >= 0.0 ? 1.0 + (double)log1pf((float)v) : 1.0 / (1.0 - v);
        }
    }
}

/* SpecializedConvertPyramidToScalarFunctor, real -> real (src/fixmath.h:320-329),
 * written where alpha != 0 (copyFromPyramidImageIf, src/fixmath.h:2259-2294);
 * NumericTraits<float>::fromRealPromote is the plain conversion to float. */
void orc_real_from_pyramid(const double* src, const uint8_t* alpha, int64_t npix, int C, float* dst,
                           int pix_stride)
{
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npix; ++p) {
        if (!alpha[p]) {
            continue;
        }
        for (int c = 0; c < C; ++c) {
            const double v = src[p * C + c];
            dst[p * pix_stride + c] = (float)(v >= 1.0 ? expm1(v - 1.0) : 1.0 - 1.0 / v);
        }
    }
}

/* reduce with alpha over a double pyramid (src/pyramid.h:166-573 with
 * SKIPSMImagePixelType double): the normalised 5x5 binomial with a real
 * division; zero where no opaque tap contributes. */
int orc_reduce_alpha_d(int wrap, const double* src, const uint8_t* alpha, int sw, int sh, int C, double* dst,
                       uint8_t* dst_alpha)
{
    if (sw <= 1 || sh <= 1 || C > 4) {
        return -1;
    }
    const int dw = (sw + 1) >> 1, dh = (sh + 1) >> 1;
#pragma omp parallel for schedule(static)
    for (int Y = 0; Y < dh; ++Y) {
        for (int X = 0; X < dw; ++X) {
            double num[4] = {0, 0, 0, 0};
            int den = 0;
            for (int j = -2; j <= 2; ++j) {
                const int y = 2 * Y + j;
                if (y < 0 || y >= sh) {
                    continue;
                }
                for (int i = -2; i <= 2; ++i) {
                    int x = 2 * X + i;
                    if (wrap) {
                        x = imod(x, sw);
                    } else if (x < 0 || x >= sw) {
                        continue;
                    }
                    const int64_t p = (int64_t)y * sw + x;
                    if (alpha[p]) {
                        const int wgt = W5[j + 2] * W5[i + 2];
                        den += wgt;
                        for (int c = 0; c < C; ++c) {
                            num[c] += (double)wgt * src[p * C + c];
                        }
                    }
                }
            }
            const int64_t q = (int64_t)Y * dw + X;
            for (int c = 0; c < C; ++c) {
                dst[q * C + c] = den > 0 ? num[c] / (double)den : 0.0;
            }
            dst_alpha[q] = den > 0 ? 255 : 0;
        }
    }
    return 0;
}

/* expand over a double pyramid (src/pyramid.h:875-1457): add = 0: dst -= E,
 * add = 1: dst += E (fromPromote is the identity for double). */
int orc_expand_d(int add, int wrap, const double* src, int sw, int sh, double* dst, int dw, int dh, int C)
{
    if (sw < 1 || sh < 1 || sw != ((dw + 1) >> 1) || sh != ((dh + 1) >> 1) || C > 4) {
        return -1;
    }
#pragma omp parallel for schedule(static)
    for (int Y = 0; Y < dh; ++Y) {
        int vi[3], vw[3], vn, vd;
        expand_vtaps(Y, sh, vi, vw, &vn, &vd);
        for (int X = 0; X < dw; ++X) {
            int hi[3], hw[3], hn, hd;
            expand_htaps(X, sw, dw, wrap, hi, hw, &hn, &hd);
            const double den = (double)(hd * vd);
            for (int c = 0; c < C; ++c) {
                double num = 0.0;
                for (int a = 0; a < vn; ++a) {
                    double row = 0.0;
                    for (int b = 0; b < hn; ++b) {
                        row += (double)hw[b] * src[((int64_t)vi[a] * sw + hi[b]) * C + c];
                    }
                    num += (double)vw[a] * row;
                }
                double* d = &dst[((int64_t)Y * dw + X) * C + c];
                *d = add ? *d + num / den : *d - num / den;
            }
        }
    }
    return 0;
}

/* CartesianBlendFunctor on double pixels (src/blend.h:41-76). */
void orc_blend_d(const int32_t* mask, const double* white, double* black, int64_t npix, int C, int32_t white_value)
{
    const double wv = (double)white_value;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npix; ++p) {
        const double wc = (double)mask[p] / wv;
        if (wc >= 1.0) {
            for (int c = 0; c < C; ++c) {
                black[p * C + c] = white[p * C + c];
            }
        } else if (wc > 0.0) {
            const double bc = 1.0 - wc;
            for (int c = 0; c < C; ++c) {
                black[p * C + c] = wc * white[p * C + c] + bc * black[p * C + c];
            }
        }
    }
}

/* ImageMaskMultiplyFunctor on double pixels (src/enfuse.h:601-620), then the
 * accumulation into the result pyramid (src/enfuse.h:1576-1588); res = NULL
 * multiplies in place only. */
void orc_mask_multiply_d(double* lp, const int32_t* mask, int64_t npix, int C, int32_t divisor, double* res)
{
    const double dv = (double)divisor;
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npix; ++p) {
        const double coeff = (double)mask[p] / dv;
        for (int c = 0; c < C; ++c) {
            const double v = lp[p * C + c] * coeff;
            lp[p * C + c] = v;
            if (res) {
                res[p * C + c] += v;
            }
        }
    }
}

typedef struct {
    int levels;
    int C;
    int w[30], h[30];
    double* lv[30];
} pyrd_t;

static void pyrd_alloc(pyrd_t* p, int levels, int w, int h, int C)
{
    p->levels = levels;
    p->C = C;
    for (int l = 0; l < levels; ++l) {
        p->w[l] = w;
        p->h[l] = h;
        p->lv[l] = (double*)calloc((size_t)w * h * C, sizeof(double));
        w = (w + 1) >> 1;
        h = (h + 1) >> 1;
    }
}

static void pyrd_free(pyrd_t* p)
{
    for (int l = 0; l < p->levels; ++l) {
        free(p->lv[l]);
    }
}

/* laplacianPyramid of a float image (src/pyramid.h:1647-1747): log mapping,
 * Gaussian levels with alpha, then gp[l] -= expand(gp[l+1]). */
static int laplacian_d(pyrd_t* p, const float* img, int pix_stride, const uint8_t* alpha0, int wrap)
{
    orc_real_to_pyramid(img, (int64_t)p->w[0] * p->h[0], p->C, pix_stride, p->lv[0]);
    const uint8_t* a = alpha0;
    uint8_t* owned = NULL;
    int rc = 0;
    for (int l = 1; l < p->levels && !rc; ++l) {
        uint8_t* na = (uint8_t*)malloc((size_t)p->w[l] * p->h[l]);
        rc = orc_reduce_alpha_d(wrap, p->lv[l - 1], a, p->w[l - 1], p->h[l - 1], p->C, p->lv[l], na);
        free(owned);
        owned = na;
        a = na;
    }
    free(owned);
    for (int l = 0; l + 1 < p->levels && !rc; ++l) {
        rc = orc_expand_d(0, wrap, p->lv[l + 1], p->w[l + 1], p->h[l + 1], p->lv[l], p->w[l], p->h[l], p->C);
    }
    return rc;
}

static int collapse_d(pyrd_t* p, int wrap)
{
    for (int l = p->levels - 2; l >= 0; --l) {
        const int rc = orc_expand_d(1, wrap, p->lv[l + 1], p->w[l + 1], p->h[l + 1], p->lv[l], p->w[l], p->h[l],
                                    p->C);
        if (rc) {
            return rc;
        }
    }
    return 0;
}

/* MultiGrayscaleAccessor on float RGB (src/mga.h:184-222), stored as float
 * (fromRealPromote<float>).  NumericTraits<float>::RealPromote is float, so
 * the average adds the three samples in float before the double division by
 * 3.0, and the lightness adds min and max in float; luminance
 * (RGBValue::luminance, 0.3/0.59/0.11 in double) and the mixer (double
 * weights) are double expressions. */
static float gray_float(const orc_enfuse_params* prm, float r, float g, float b, double mw0, double mw1, double mw2)
{
    const float mx = r > g ? (r > b ? r : b) : (g > b ? g : b);
    const float mn = r < g ? (r < b ? r : b) : (g < b ? g : b);
    switch (prm->gray_projector) {
    case ORC_GRAY_VALUE: return mx;
    case ORC_GRAY_ANTI_VALUE: return mn;
    case ORC_GRAY_LIGHTNESS: {
        const float s = mn + mx;
        return (float)((double)s / 2.0);
    }
    case ORC_GRAY_LUMINANCE: return (float)(0.3 * r + 0.59 * g + 0.11 * b);
    case ORC_GRAY_MIXER: return (float)(mw0 * (double)r + mw1 * (double)g + mw2 * (double)b);
    default: {
        const float s = (r + g) + b;
        return (float)((double)s / 3.0);
    }
    }
}

static int cmp_f32(const void* a, const void* b)
{
    const float x = *(const float*)a, y = *(const float*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* Histogram::entropyOfChannel over raw float keys (src/enfuse.h:346-375);
 * keys compare as floats (-0 and +0 are one bin). */
static double entropy_of_f(float* vals, int n)
{
    if (n == 0) {
        return 0.0;
    }
    qsort(vals, (size_t)n, sizeof(float), cmp_f32);
    int bins = 1;
    for (int i = 1; i < n; ++i) {
        bins += vals[i] != vals[i - 1];
    }
    if (bins <= 1) {
        return 0.0;
    }
    double e = 0.0;
    int i = 0;
    while (i < n) {
        int j = i;
        while (j < n && vals[j] == vals[i]) {
            ++j;
        }
        const double p = (double)(j - i) / (double)n;
        e += p * log(p);
        i = j;
    }
    return -e / log((double)bins);
}

/* localStdDevIf (src/enfuse.h:75-219) for a float gray image, with the
 * reference's own rounding: per row, float column sums of the masked window
 * rows, a float running sum along the row updated by (new column - old
 * column), and sqrt((sumSqr - sum^2 / n) / (n - 1)) in float.  Rows are
 * independent (each starts from its own column sums), so the result does not
 * depend on how rows are shared among threads.  Pixels outside the interior
 * or without alpha stay 0. */
static void stddev_sliding_f(const float* gray, const uint8_t* alpha, int w, int h, int win, float* sd)
{
    const int b = win / 2;
#pragma omp parallel
    {
        float* csum = (float*)malloc(sizeof(float) * (size_t)(w + 1));
        float* csq = (float*)malloc(sizeof(float) * (size_t)(w + 1));
        size_t* cn = (size_t*)malloc(sizeof(size_t) * (size_t)(w + 1));
#pragma omp for schedule(static)
        for (int y = b; y < h - b; ++y) {
            float sum = 0.0f, sumsq = 0.0f;
            size_t n = 0;
            for (int i = 0; i <= 2 * b; ++i) {        /* columns 0 .. 2b */
                float s0 = 0.0f, q0 = 0.0f;
                size_t n0 = 0;
                for (int yy = y - b; yy <= y + b; ++yy) {
                    const int64_t q = (int64_t)yy * w + i;
                    if (alpha[q]) {
                        const float v = gray[q];
                        s0 += v;
                        q0 += v * v;
                        ++n0;
                    }
                }
                csum[i] = s0;
                csq[i] = q0;
                cn[i] = n0;
                sum += s0;
                sumsq += q0;
                n += n0;
            }
            int old = 0, next = win;
            for (int x = b;; ++x) {
                const int64_t p = (int64_t)y * w + x;
                if (alpha[p]) {
                    sd[p] = n <= 1 ? 0.0f : sqrtf((sumsq - sum * sum / (float)n) / (float)(n - 1));
                }
                if (x == w - b - 1) {
                    break;
                }
                const int cx = x + b + 1;
                float s0 = 0.0f, q0 = 0.0f;
                size_t n0 = 0;
                for (int yy = y - b; yy <= y + b; ++yy) {
                    const int64_t q = (int64_t)yy * w + cx;
                    if (alpha[q]) {
                        const float v = gray[q];
                        s0 += v;
                        q0 += v * v;
                        ++n0;
                    }
                }
                csum[next] = s0;
                csq[next] = q0;
                cn[next] = n0;
                sum += s0 - csum[old];
                sumsq += q0 - csq[old];
                n += n0 - cn[old];
                ++old;
                ++next;
            }
        }
        free(csum);
        free(csq);
        free(cn);
    }
}

/* enfuseMask for float images (src/enfuse.h:962-1212).  `range` stands for
 * NumericTraits<float>::max() in the exposure (y = gray / max, :638) and
 * entropy (H * max) weights: FLT_MAX is the reference's behaviour, 1.0 the
 * normalised-float mode for images in [0, 1].  Saturation uses max_value 1.0
 * (:758-761); contrast is W * sigma without a scale (:800-804, 818-823). */
int orc_enfuse_mask_f(const float* img, int w, int h, int C, int pix_stride, const uint8_t* alpha,
                      const orc_enfuse_params* prm, double range, float* out)
{
    if (C != 1 && C != 3) {
        return -2;
    }
    const int64_t npix = (int64_t)w * h;
    double mw0 = 0, mw1 = 0, mw2 = 0;
    if (prm->gray_projector == ORC_GRAY_MIXER) {
        const double s = prm->mixer[0] + prm->mixer[1] + prm->mixer[2];
        mw0 = prm->mixer[0] / s;
        mw1 = prm->mixer[1] / s;
        mw2 = prm->mixer[2] / s;
    }
    float* gray = (float*)malloc(sizeof(float) * (size_t)npix);
#pragma omp parallel for schedule(static)
    for (int64_t p = 0; p < npix; ++p) {
        const float* px = img + p * pix_stride;
        gray[p] = C == 1 ? px[0] : gray_float(prm, px[0], px[1], px[2], mw0, mw1, mw2);
    }
    memset(out, 0, sizeof(float) * (size_t)npix);

    if (prm->w_exposure > 0.0) {
        const double ew = exposure_effective_width(prm->exp_function, prm->exp_width);
        /* the cutoff limits are fractions of the same `range` (enfuse.h:655-690) */
        int cut = 0;
        double lo = 0.0, hi = 0.0;
        const int rc = exposure_cutoffs(prm, range, 0, &cut, &lo, &hi);
        if (rc) {
            free(gray);
            return rc;
        }
        orc_enfuse_params lp = *prm, up = *prm;
        lp.gray_projector = prm->exp_cutoff_proj[0];
        up.gray_projector = prm->exp_cutoff_proj[1];
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < npix; ++p) {
            if (alpha[p]) {
                if (cut) {
                    const float* px = img + p * pix_stride;
                    const float lv = C == 1 ? gray[p] : gray_float(&lp, px[0], px[1], px[2], mw0, mw1, mw2);
                    const float uv = C == 1 ? gray[p] : gray_float(&up, px[0], px[1], px[2], mw0, mw1, mw2);
                    if (!((double)lv >= lo && (double)uv <= hi)) {
                        out[p] = 0.0f;
                        continue;
                    }
                }
                /* toRealPromote(float) / max(): a float division (enfuse.h:638) */
                const double y = (double)(gray[p] / (float)range);
                out[p] = (float)(prm->w_exposure * exposure_weight(prm->exp_function, y, prm->exp_optimum, ew));
            }
        }
    }

    if (prm->w_contrast > 0.0 && prm->float_sliding_sums) {
        const int win = prm->contrast_window;
        if (win < 2 || w < win || h < win) {
            free(gray);
            return -1;
        }
        float* sd = (float*)calloc((size_t)npix, sizeof(float));
        stddev_sliding_f(gray, alpha, w, h, win, sd);
        for (int64_t p = 0; p < npix; ++p) {
            if (alpha[p]) {
                out[p] = (float)(prm->w_contrast * (double)sd[p]) + out[p];
            }
        }
        free(sd);
    } else if (prm->w_contrast > 0.0) {
        const int win = prm->contrast_window, b = win / 2;
        if (win < 2 || w < win || h < win) {
            free(gray);
            return -1;
        }
#pragma omp parallel for schedule(static)
        for (int y = b; y < h - b; ++y) {
            for (int x = b; x < w - b; ++x) {
                if (!alpha[(int64_t)y * w + x]) {
                    continue;
                }
                double sum = 0.0;
                int n = 0;
                for (int yy = y - b; yy <= y + b; ++yy) {
                    for (int xx = x - b; xx <= x + b; ++xx) {
                        if (alpha[(int64_t)yy * w + xx]) {
                            sum += gray[(int64_t)yy * w + xx];
                            ++n;
                        }
                    }
                }
                float sd = 0.0f;
                if (n > 1) {
                    const double mean = sum / n;
                    double ss = 0.0;
                    for (int yy = y - b; yy <= y + b; ++yy) {
                        for (int xx = x - b; xx <= x + b; ++xx) {
                            if (alpha[(int64_t)yy * w + xx]) {
                                const double d = gray[(int64_t)yy * w + xx] - mean;
                                ss += d * d;
                            }
                        }
                    }
                    sd = (float)sqrt(ss / (double)(n - 1));
                }
                const int64_t p = (int64_t)y * w + x;
                out[p] = (float)(prm->w_contrast * (double)sd) + out[p];
            }
        }
    }

    if (prm->w_saturation > 0.0 && C == 3) {
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < npix; ++p) {
            if (!alpha[p]) {
                continue;
            }
            const float* px = img + p * pix_stride;
            const float mx = px[0] > px[1] ? (px[0] > px[2] ? px[0] : px[2]) : (px[1] > px[2] ? px[1] : px[2]);
            const float mn = px[0] < px[1] ? (px[0] < px[2] ? px[0] : px[2]) : (px[1] < px[2] ? px[1] : px[2]);
            float sw = 0.0f;
            if (mx != mn) {
                const double sum = (double)mx + (double)mn;
                const double diff = (double)mx - (double)mn;
                const double s = sum <= 1.0 ? diff / sum : diff / (2.0 - sum);
                sw = (float)(prm->w_saturation * s);
            }
            out[p] = sw + out[p];
        }
    }

    if (prm->w_entropy > 0.0) {
        const int win = prm->entropy_window, b = win / 2;
        if (w < win || h < win) {
            free(gray);
            return -1;
        }
        int cut = 0;
        double lo = 0.0, hi = 0.0;
        const int rc = entropy_cutoffs(prm, range, 0, &cut, &lo, &hi);
        if (rc) {
            free(gray);
            return rc;
        }
#pragma omp parallel
        {
            float* vals = (float*)malloc(sizeof(float) * (size_t)win * win);
#pragma omp for schedule(static)
            for (int y = b; y < h - b; ++y) {
                for (int x = b; x < w - b; ++x) {
                    if (!alpha[(int64_t)y * w + x]) {
                        continue;
                    }
                    float mn = FLT_MAX;
                    for (int c = 0; c < C; ++c) {
                        int n = 0;
                        for (int yy = y - b; yy <= y + b; ++yy) {
                            for (int xx = x - b; xx <= x + b; ++xx) {
                                const int64_t q = (int64_t)yy * w + xx;
                                if (alpha[q]) {
                                    float v = img[q * pix_stride + c];
                                    if (cut) {
                                        /* ClampingFunctor (enfuse.h:893-925), the third
                                         * sample judged low by the first */
                                        const float* px = img + q * pix_stride;
                                        const int low = (C == 3 && c == 2) ? ((double)px[0] <= lo) : ((double)v <= lo);
                                        v = low ? 0.0f : ((double)v >= hi ? (float)range : v);
                                    }
                                    vals[n++] = v == 0.0f ? 0.0f : v;
                                }
                            }
                        }
                        const float e = (float)(entropy_of_f(vals, n) * range);
                        mn = e < mn ? e : mn;
                    }
                    const int64_t p = (int64_t)y * w + x;
                    out[p] = (float)(prm->w_entropy * (double)mn) + out[p];
                }
            }
            free(vals);
        }
    }
    free(gray);
    return 0;
}

/* enfuseMain for float images (src/enfuse.h:1217-1617): weights (or
 * masks_in), normalisation, double Laplacian pyramids, Int32 9.15 mask
 * pyramids with the union alpha, merge, collapse, conversion back.
 * level0_out: optional (h, w, C) double buffer of the collapsed level 0. */
int orc_enfuse_f(int K, const float* const* imgs, const uint8_t* const* alphas, int w, int h, int C, int pix_stride,
                 const orc_enfuse_params* prm, double range, int levels, int wrap, int hard_mask,
                 const float* const* masks_in, float* out, uint8_t* out_alpha, double* level0_out, float* masks_out)
{
    if (K < 1 || (C != 1 && C != 3)) {
        return -2;
    }
    const int64_t npix = (int64_t)w * h;
    const int mfrac = 15;
    const int32_t max_mask_pyr = 255 << mfrac;
    int rc = 0;
    float** masks = (float**)calloc((size_t)K, sizeof(float*));
    float* norm = (float*)calloc((size_t)npix, sizeof(float));
    memset(out_alpha, 0, (size_t)npix);
    for (int k = 0; k < K && !rc; ++k) {
        masks[k] = (float*)malloc(sizeof(float) * (size_t)npix);
        if (masks_in) {
            memcpy(masks[k], masks_in[k], sizeof(float) * (size_t)npix);
        } else {
            rc = orc_enfuse_mask_f(imgs[k], w, h, C, pix_stride, alphas[k], prm, range, masks[k]);
        }
        for (int64_t p = 0; p < npix && !rc; ++p) {
            if (alphas[k][p]) {
                out_alpha[p] = alphas[k][p];
            }
            norm[p] = masks[k][p] + norm[p];
        }
    }
    if (!rc && hard_mask) {
#pragma omp parallel for schedule(static)
        for (int64_t p = 0; p < npix; ++p) {
            float mx = 0.0f;
            int mi = 0;
            for (int k = 0; k < K; ++k) {
                if (masks[k][p] > mx) {
                    mx = masks[k][p];
                    mi = k;
                }
            }
            for (int k = 0; k < K; ++k) {
                masks[k][p] = mx == 0.0f ? 255.0f / (float)K : (k == mi ? 255.0f : 0.0f);
            }
        }
    }
    levels = levels > 0 ? levels : orc_num_levels(w, h, 1, 0);
    pyrd_t result;
    pyrd_alloc(&result, levels, w, h, C);
    for (int k = 0; k < K && !rc; ++k) {
        pyrd_t lp;
        pyr_t mg;
        pyrd_alloc(&lp, levels, w, h, C);
        rc = laplacian_d(&lp, imgs[k], pix_stride, alphas[k], wrap);
        if (!hard_mask) {
            const float fallback = (float)(255 / K);
#pragma omp parallel for schedule(static)
            for (int64_t p = 0; p < npix; ++p) {
                masks[k][p] = norm[p] > 0.0f ? (255.0f * masks[k][p]) / norm[p] : fallback;
            }
        }
        if (masks_out) {
            memcpy(masks_out + (size_t)k * npix, masks[k], sizeof(float) * (size_t)npix);
        }
        pyr_alloc(&mg, levels, w, h, 1);
        orc_fixed_from_float(masks[k], npix, mg.lv[0], mfrac, 32);
        if (!rc) {
            rc = gaussian_alpha(&mg, out_alpha, wrap, 32);
        }
        for (int l = 0; l < levels && !rc; ++l) {
            orc_mask_multiply_d(lp.lv[l], mg.lv[l], (int64_t)lp.w[l] * lp.h[l], C, max_mask_pyr, result.lv[l]);
        }
        pyr_free(&mg);
        pyrd_free(&lp);
    }
    if (!rc) {
        rc = collapse_d(&result, wrap);
    }
    if (!rc) {
        if (level0_out) {
            memcpy(level0_out, result.lv[0], sizeof(double) * (size_t)npix * C);
        }
        memset(out, 0, sizeof(float) * (size_t)npix * pix_stride);
        orc_real_from_pyramid(result.lv[0], out_alpha, npix, C, out, pix_stride);
        if (pix_stride == 4) {
            for (int64_t p = 0; p < npix; ++p) {
                out[p * 4 + 3] = out_alpha[p] ? 1.0f : 0.0f;
            }
        }
    }
    pyrd_free(&result);
    for (int k = 0; k < K; ++k) {
        free(masks[k]);
    }
    free(masks);
    free(norm);
    return rc;
}

/* enblendMain's pyramid section for float images (src/enblend.h:330-510):
 * Int32 9.15 mask Gaussian pyramid, double white/black Laplacian pyramids,
 * blend, collapse, conversion back where the union alpha is set. */
int orc_enblend_f(const float* white, const uint8_t* white_alpha, const float* black, const uint8_t* black_alpha,
                  const uint8_t* mask, int w, int h, int C, int pix_stride, int levels, int wrap, float* out,
                  uint8_t* out_alpha, double* level0_out)
{
    if (C > 4) {
        return -2;
    }
    const int64_t npix = (int64_t)w * h;
    const int mfrac = 15;
    levels = levels > 0 ? levels : orc_num_levels(w, h, 1, 0);
    pyr_t mg;
    pyrd_t wl, bl;
    pyr_alloc(&mg, levels, w, h, 1);
    orc_fixed_from_int(mask, ORC_U8, npix, 1, 1, mg.lv[0], mfrac);
    int rc = gaussian_noalpha(&mg, wrap, 32);
    pyrd_alloc(&wl, levels, w, h, C);
    pyrd_alloc(&bl, levels, w, h, C);
    if (!rc) {
        rc = laplacian_d(&wl, white, pix_stride, white_alpha, wrap);
    }
    if (!rc) {
        rc = laplacian_d(&bl, black, pix_stride, black_alpha, wrap);
    }
    for (int64_t p = 0; p < npix; ++p) {
        out_alpha[p] = white_alpha[p] ? 255 : black_alpha[p];
    }
    if (!rc) {
        for (int l = 0; l < levels; ++l) {
            orc_blend_d(mg.lv[l], wl.lv[l], bl.lv[l], (int64_t)bl.w[l] * bl.h[l], C, 255 << mfrac);
        }
        rc = collapse_d(&bl, wrap);
    }
    if (!rc) {
        if (level0_out) {
            memcpy(level0_out, bl.lv[0], sizeof(double) * (size_t)npix * C);
        }
        memcpy(out, black, sizeof(float) * (size_t)npix * pix_stride);
        orc_real_from_pyramid(bl.lv[0], out_alpha, npix, C, out, pix_stride);
        if (pix_stride == 4) {
            for (int64_t p = 0; p < npix; ++p) {
                out[p * 4 + 3] = out_alpha[p] ? 1.0f : 0.0f;
            }
        }
    }
    pyr_free(&mg);
    pyrd_free(&wl);
    pyrd_free(&bl);
    return rc;
}


/* ---- nearest-feature seam mask (src/nearest.h, src/openmp_vigra.h) ---------- */

/* The 1-D squared Euclidean transform of Felzenszwalb and Huttenlocher as the
 * reference writes it (src/openmp_vigra.h:300-351): lower envelope of the
 * parabolas q^2 + f(q), float arithmetic, with the sample index squared as an
 * int where the reference squares an int (v[k]) and as a float where it
 * squares a float (q). */
static void nft_fh1d(float* d, const float* f, int n, int* v, float* z)
{
    int k = 0;
    v[0] = 0;
    z[0] = -INFINITY;
    z[1] = INFINITY;
    for (int q = 1; q < n; ++q) {
        const float qf = (float)q;
        const float sum_q = f[q] + qf * qf;
        float s = (sum_q - (f[v[k]] + (float)(v[k] * v[k]))) / (float)(2 * (q - v[k]));
        while (s <= z[k]) {
            --k;
            s = (sum_q - (f[v[k]] + (float)(v[k] * v[k]))) / (float)(2 * (q - v[k]));
        }
        ++k;
        v[k] = q;
        z[k] = s;
        z[k + 1] = INFINITY;
    }
    k = 0;
    for (int q = 0; q < n; ++q) {
        while (z[k + 1] < (float)q) {
            ++k;
        }
        d[q] = (float)((q - v[k]) * (q - v[k])) + f[v[k]];
    }
}

/* Euclidean distance to the nearest feature (feat != 0) of a w x h image,
 * columns first, then rows, sqrt in float (src/openmp_vigra.h:355-433). */
static void nft_distance(const uint8_t* feat, int w, int h, float* dist)
{
    const int n = w > h ? w : h;
    float* inter = (float*)malloc(sizeof(float) * (size_t)w * h);
    float* f = (float*)malloc(sizeof(float) * (size_t)n);
    float* d = (float*)malloc(sizeof(float) * (size_t)n);
    int* v = (int*)malloc(sizeof(int) * (size_t)n);
    float* z = (float*)malloc(sizeof(float) * (size_t)(n + 1));
    for (int x = 0; x < w; ++x) {
        for (int y = 0; y < h; ++y) {
            f[y] = feat[(size_t)y * w + x] ? 0.0f : FLT_MAX;
        }
        nft_fh1d(d, f, h, v, z);
        for (int y = 0; y < h; ++y) {
            inter[(size_t)y * w + x] = d[y];
        }
    }
    for (int y = 0; y < h; ++y) {
        nft_fh1d(d, inter + (size_t)y * w, w, v, z);
        for (int x = 0; x < w; ++x) {
            dist[(size_t)y * w + x] = sqrtf(d[x]);
        }
    }
    free(z);
    free(v);
    free(d);
    free(f);
    free(inter);
}

int orc_nft_mask(const uint8_t* white, const uint8_t* black, int w, int h, int wrap, uint8_t* mask)
{
    const size_t npix = (size_t)w * h;
    /* saturating_subtract (src/nearest.h:358-372): white - black where white
     * exceeds black; quick_tally counts such pixels up to the threshold
     * (src/nearest.h:375-395, 465-470, 531-545) */
    const unsigned threshold = 2u * 2u * ((unsigned)h + (unsigned)w);
    unsigned t12 = 0, t21 = 0;
    for (size_t i = 0; i < npix; ++i) {
        t12 += (white[i] > black[i] && t12 < threshold) ? 1u : 0u;
        t21 += (black[i] > white[i] && t21 < threshold) ? 1u : 0u;
    }
    if ((t12 > t21 ? t12 : t21) < threshold) {
        return 2;
    }
    /* the periodic transform doubles the image horizontally and keeps the
     * middle columns: x < w/2 from column w + x, the rest from column x
     * (quadruple_image / quater_image, src/nearest.h:136-290) */
    const int W = wrap ? 2 * w : w;
    uint8_t* f12 = (uint8_t*)malloc((size_t)W * h);
    uint8_t* f21 = (uint8_t*)malloc((size_t)W * h);
    float* d12 = (float*)malloc(sizeof(float) * (size_t)W * h);
    float* d21 = (float*)malloc(sizeof(float) * (size_t)W * h);
    for (int y = 0; y < h; ++y) {
        for (int X = 0; X < W; ++X) {
            const size_t i = (size_t)y * w + (X % w);
            f12[(size_t)y * W + X] = white[i] > black[i];
            f21[(size_t)y * W + X] = black[i] > white[i];
        }
    }
    nft_distance(f12, W, h, d12);
    nft_distance(f21, W, h, d21);
    const int half = w / 2;
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            const int X = wrap ? (x < half ? w + x : x) : x;
            const size_t j = (size_t)y * W + X;
            mask[(size_t)y * w + x] = d12[j] < d21[j] ? 255 : 0;
        }
    }
    free(d21);
    free(d12);
    free(f21);
    free(f12);
    return 0;
}
