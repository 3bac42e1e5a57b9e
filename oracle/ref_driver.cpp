// ref_driver.cpp -- C entry points over the reference's own pyramid, blend
// and fixed-point code (src/pyramid.h, src/blend.h, src/fixmath.h,
// src/numerictraits.h, src/openmp_vigra.h of enblend-enfuse, compiled
// unmodified from the reference tree against the VIGRA/GSL/LCMS2 shims in
// refshim/).  Test oracle only: it pins the C restatement in enb_oracle.c to
// the reference's code.  Built by reference_build.py into _ref/.
//
// Buffers are plain row-major arrays: pixel images interleaved (H, W, S)
// with S = C (RGB or gray) samples, pyramid levels interleaved (h, w, C)
// int16/int32, alpha and mask planes (H, W) uint8.

#include <config.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "global.h"
#include "common.h"

// Colour-space globals of enblend.cc; the oracle blends in the identity space.
blend_colorspace_t BlendColorspace = IdentitySpace;
cmsHPROFILE InputProfile = nullptr;

#include "openmp_def.h"
#include "openmp_vigra.h"
#include "numerictraits.h"
#include "fixmath.h"
#include "pyramid.h"
#include "blend.h"

// ---- globals the reference's translation units define --------------------------
const std::string command("enblend-oracle");
int Verbose = 0;
cmsHTRANSFORM InputToXYZTransform = nullptr;
cmsHTRANSFORM XYZToInputTransform = nullptr;
cmsHTRANSFORM InputToLabTransform = nullptr;
cmsHTRANSFORM LabToInputTransform = nullptr;
cmsHANDLE CIECAMTransform = nullptr;

// ---- definitions behind the shim declarations (never reached) -------------------
[[noreturn]] static void shim_abort(const char* what)
{
    std::cerr << "reference oracle: " << what << " is not available" << std::endl;
    std::abort();
}

void cmsDoTransform(cmsHTRANSFORM, const void*, void*, cmsUInt32Number) { shim_abort("cmsDoTransform"); }
cmsUInt32Number cmsGetProfileInfoASCII(cmsHPROFILE, cmsInfoType, const char*, const char*, char*, cmsUInt32Number)
{
    shim_abort("cmsGetProfileInfoASCII");
}
cmsColorSpaceSignature cmsGetColorSpace(cmsHPROFILE) { shim_abort("cmsGetColorSpace"); }
cmsUInt32Number cmsChannelsOf(cmsColorSpaceSignature) { shim_abort("cmsChannelsOf"); }
double cmsCMCdeltaE(const cmsCIELab*, const cmsCIELab*, double, double) { shim_abort("cmsCMCdeltaE"); }
void cmsCIECAM02Forward(cmsHANDLE, const cmsCIEXYZ*, cmsJCh*) { shim_abort("cmsCIECAM02Forward"); }
void cmsCIECAM02Reverse(cmsHANDLE, const cmsJCh*, cmsCIEXYZ*) { shim_abort("cmsCIECAM02Reverse"); }

namespace enblend {
std::string extractBasename(const std::string& f)
{
    const size_t slash = f.rfind('/');
    const std::string b = slash == std::string::npos ? f : f.substr(slash + 1);
    const size_t dot = b.rfind('.');
    return dot == std::string::npos ? b : b.substr(0, dot);
}
std::string extractDirname(const std::string& f)
{
    const size_t slash = f.rfind('/');
    return slash == std::string::npos ? std::string(".") : f.substr(0, slash);
}
std::string extractFilename(const std::string& f)
{
    const size_t slash = f.rfind('/');
    return slash == std::string::npos ? f : f.substr(slash + 1);
}
std::string extractExtension(const std::string& f)
{
    const size_t dot = f.rfind('.');
    return dot == std::string::npos ? std::string() : f.substr(dot);
}
std::string errorMessage(int e) { return "error " + std::to_string(e); }
}  // namespace enblend

namespace parameter {
bool exists(const std::string&) { return false; }
unsigned as_unsigned(const std::string&, unsigned d) { return d; }
int as_integer(const std::string&, int d) { return d; }
double as_double(const std::string&, double d) { return d; }
bool as_boolean(const std::string&, bool d) { return d; }
std::string as_string(const std::string&, const std::string& d) { return d; }
}  // namespace parameter

using namespace enblend;

namespace {

template <class P>
void to_image(const P* src, int w, int h, vigra::BasicImage<P>& img)
{
    img.resize(w, h);
    std::memcpy(img.data(), src, sizeof(P) * (size_t)w * h);
}

template <class P>
void to_image(const P* src, int w, int h, vigra::BasicImage<vigra::RGBValue<P>>& img)
{
    img.resize(w, h);
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        img.data()[i] = vigra::RGBValue<P>(src[3 * i], src[3 * i + 1], src[3 * i + 2]);
    }
}

template <class P>
void from_image(const vigra::BasicImage<P>& img, P* dst)
{
    std::memcpy(dst, img.data(), sizeof(P) * (size_t)img.width() * img.height());
}

template <class P>
void from_image(const vigra::BasicImage<vigra::RGBValue<P>>& img, P* dst)
{
    for (size_t i = 0; i < (size_t)img.width() * img.height(); ++i) {
        dst[3 * i] = img.data()[i].red();
        dst[3 * i + 1] = img.data()[i].green();
        dst[3 * i + 2] = img.data()[i].blue();
    }
}

// Pixel image of the reference for sample type T and C (1 or 3) channels.
template <class T, int C>
struct Pix;
template <class T>
struct Pix<T, 1> {
    typedef T type;
};
template <class T>
struct Pix<T, 3> {
    typedef vigra::RGBValue<T> type;
};

template <class T, int C>
int run_reduce(int alpha, int wrap, const void* src, const uint8_t* sa, int sw, int sh, void* dst, uint8_t* da)
{
    typedef EnblendNumericTraits<typename Pix<T, C>::type> Tr;
    typedef typename Tr::ImagePyramidType PyrImg;
    typedef typename Tr::ImagePyramidPixelComponentType PC;
    PyrImg s, d((sw + 1) >> 1, (sh + 1) >> 1);
    to_image((const PC*)src, sw, sh, s);
    if (alpha) {
        vigra::BasicImage<vigra::UInt8> a, ad(d.width(), d.height());
        to_image(sa, sw, sh, a);
        reduce<typename Tr::SKIPSMImagePixelType, typename Tr::SKIPSMAlphaPixelType>(
            wrap != 0, s.upperLeft(), s.lowerRight(), s.accessor(), a.upperLeft(), a.accessor(), d.upperLeft(),
            d.lowerRight(), d.accessor(), ad.upperLeft(), ad.lowerRight(), ad.accessor());
        from_image(ad, da);
    } else {
        reduce<typename Tr::SKIPSMImagePixelType>(wrap != 0, s.upperLeft(), s.lowerRight(), s.accessor(),
                                                  d.upperLeft(), d.lowerRight(), d.accessor());
    }
    from_image(d, (PC*)dst);
    return 0;
}

template <class T, int C>
int run_expand(int add, int wrap, const void* src, int sw, int sh, void* dst, int dw, int dh)
{
    typedef EnblendNumericTraits<typename Pix<T, C>::type> Tr;
    typedef typename Tr::ImagePyramidType PyrImg;
    typedef typename Tr::ImagePyramidPixelComponentType PC;
    PyrImg s, d;
    to_image((const PC*)src, sw, sh, s);
    to_image((const PC*)dst, dw, dh, d);
    expand<typename Tr::SKIPSMImagePixelType>(add != 0, wrap != 0, vigra::srcImageRange(s), vigra::destImageRange(d));
    from_image(d, (PC*)dst);
    return 0;
}

// enblendMain's pyramid section (src/enblend.h:384-510) over the whole
// canvas: mask Gaussian pyramid, white and black Laplacian pyramids with
// alpha, blend, collapse.  Writes the collapsed level 0 (int32, (h, w, C)).
template <class T, int C, class L0>
int run_enblend(int levels, int wrap, const T* white, const uint8_t* wa, const T* black, const uint8_t* ba,
                const uint8_t* mask, int w, int h, L0* level0)
{
    typedef EnblendNumericTraits<typename Pix<T, C>::type> Tr;
    typedef typename Tr::ImageType ImageType;
    typedef typename Tr::AlphaType AlphaType;
    typedef typename Tr::MaskType MaskType;
    typedef typename Tr::ImagePyramidType ImagePyramidType;
    typedef typename Tr::MaskPyramidType MaskPyramidType;
    typedef typename Tr::MaskPixelType MaskPixelType;
    typedef typename Tr::MaskPyramidPixelType MaskPyramidPixelType;
    typedef typename Tr::ImagePixelComponentType IC;
    typedef typename Tr::ImagePyramidPixelComponentType PC;

    ImageType wi, bi;
    AlphaType wai, bai;
    MaskType mi;
    to_image((const IC*)white, w, h, wi);
    to_image((const IC*)black, w, h, bi);
    to_image(wa, w, h, wai);
    to_image(ba, w, h, bai);
    to_image(mask, w, h, mi);

    std::vector<MaskPyramidType*>* maskGP =
        gaussianPyramid<MaskType, MaskPyramidType, Tr::MaskPyramidIntegerBits, Tr::MaskPyramidFractionBits,
                        typename Tr::SKIPSMMaskPixelType>(levels, wrap != 0, vigra::srcImageRange(mi));
    std::vector<ImagePyramidType*>* whiteLP =
        laplacianPyramid<ImageType, AlphaType, ImagePyramidType, Tr::ImagePyramidIntegerBits,
                         Tr::ImagePyramidFractionBits, typename Tr::SKIPSMImagePixelType,
                         typename Tr::SKIPSMAlphaPixelType>("whiteGP", levels, wrap != 0, vigra::srcImageRange(wi),
                                                            vigra::maskImage(wai));
    std::vector<ImagePyramidType*>* blackLP =
        laplacianPyramid<ImageType, AlphaType, ImagePyramidType, Tr::ImagePyramidIntegerBits,
                         Tr::ImagePyramidFractionBits, typename Tr::SKIPSMImagePixelType,
                         typename Tr::SKIPSMAlphaPixelType>("blackGP", levels, wrap != 0, vigra::srcImageRange(bi),
                                                            vigra::maskImage(bai));
    ConvertScalarToPyramidFunctor<MaskPixelType, MaskPyramidPixelType, Tr::MaskPyramidIntegerBits,
                                  Tr::MaskPyramidFractionBits>
        whiteMask;
    blend(maskGP, whiteLP, blackLP, whiteMask(vigra::NumericTraits<MaskPixelType>::max()));
    collapsePyramid<typename Tr::SKIPSMImagePixelType>(wrap != 0, blackLP);

    const ImagePyramidType& l0 = *(*blackLP)[0];
    std::vector<PC> tmp((size_t)w * h * C);
    from_image(l0, tmp.data());
    for (size_t i = 0; i < tmp.size(); ++i) {
        level0[i] = (L0)tmp[i];
    }
    for (auto* p : *maskGP) delete p;
    for (auto* p : *whiteLP) delete p;
    for (auto* p : *blackLP) delete p;
    delete maskGP;
    delete whiteLP;
    delete blackLP;
    return 0;
}

// copyFromPyramidImageIf (src/fixmath.h:2158-2294): the collapsed level 0
// (int32, (h, w, 3)) to RGB pixels where the alpha plane is nonzero, with the
// reference's dithering conversion (Mersenne Twister draws).
template <class T, class L0>
int run_from_pyramid(const L0* level0, const uint8_t* alpha, int w, int h, T* out)
{
    typedef EnblendNumericTraits<vigra::RGBValue<T>> Tr;
    typedef typename Tr::ImagePyramidType ImagePyramidType;
    typedef typename Tr::MaskType MaskType;
    typedef typename Tr::ImageType ImageType;
    typedef typename Tr::ImagePyramidPixelComponentType PC;
    std::vector<PC> tmp((size_t)w * h * 3);
    for (size_t i = 0; i < tmp.size(); ++i) {
        tmp[i] = (PC)level0[i];
    }
    ImagePyramidType pyr;
    MaskType a;
    ImageType o;
    to_image(tmp.data(), w, h, pyr);
    to_image(alpha, w, h, a);
    to_image(out, w, h, o);
    copyFromPyramidImageIf<ImagePyramidType, MaskType, ImageType, Tr::ImagePyramidIntegerBits,
                           Tr::ImagePyramidFractionBits>(vigra::srcImageRange(pyr), vigra::maskImage(a),
                                                         vigra::destImage(o));
    from_image(o, out);
    return 0;
}

}  // namespace

extern "C" {

// The conversion of a collapsed level 0 to RGB output pixels (bits 8 or 16).
int ref_from_pyramid(int bits, const int32_t* level0, const uint8_t* alpha, int w, int h, void* out)
{
    try {
        return bits == 8 ? run_from_pyramid<vigra::UInt8, int32_t>(level0, alpha, w, h, (vigra::UInt8*)out)
                         : run_from_pyramid<vigra::UInt16, int32_t>(level0, alpha, w, h, (vigra::UInt16*)out);
    } catch (const std::exception& e) {
        std::cerr << "ref_from_pyramid: " << e.what() << std::endl;
        return 1;
    }
}

// Reduce of one level (pyramid.h:166-573 with alpha, :601-848 without).
// bits: 8 or 16 (pyramid Int16 9.7 or Int32 17.7); C: 1 or 3.
int ref_reduce(int bits, int C, int alpha, int wrap, const void* src, const uint8_t* src_alpha, int sw, int sh,
               void* dst, uint8_t* dst_alpha)
{
    try {
        if (bits == 8) {
            return C == 1 ? run_reduce<vigra::UInt8, 1>(alpha, wrap, src, src_alpha, sw, sh, dst, dst_alpha)
                          : run_reduce<vigra::UInt8, 3>(alpha, wrap, src, src_alpha, sw, sh, dst, dst_alpha);
        }
        return C == 1 ? run_reduce<vigra::UInt16, 1>(alpha, wrap, src, src_alpha, sw, sh, dst, dst_alpha)
                      : run_reduce<vigra::UInt16, 3>(alpha, wrap, src, src_alpha, sw, sh, dst, dst_alpha);
    } catch (const std::exception& e) {
        std::cerr << "ref_reduce: " << e.what() << std::endl;
        return 1;
    }
}

// Expand of one level into dst (pyramid.h:1102-1457): add = 1 collapses
// (dst = fromPromote(dst + E)), add = 0 forms a Laplacian (dst -= E).
int ref_expand(int bits, int C, int add, int wrap, const void* src, int sw, int sh, void* dst, int dw, int dh)
{
    try {
        if (bits == 8) {
            return C == 1 ? run_expand<vigra::UInt8, 1>(add, wrap, src, sw, sh, dst, dw, dh)
                          : run_expand<vigra::UInt8, 3>(add, wrap, src, sw, sh, dst, dw, dh);
        }
        return C == 1 ? run_expand<vigra::UInt16, 1>(add, wrap, src, sw, sh, dst, dw, dh)
                      : run_expand<vigra::UInt16, 3>(add, wrap, src, sw, sh, dst, dw, dh);
    } catch (const std::exception& e) {
        std::cerr << "ref_expand: " << e.what() << std::endl;
        return 1;
    }
}

// The pyramid section of enblendMain on RGB images (bits 8 or 16).
int ref_enblend(int bits, int levels, int wrap, const void* white, const uint8_t* white_alpha, const void* black,
                const uint8_t* black_alpha, const uint8_t* mask, int w, int h, int32_t* level0)
{
    try {
        if (bits == 8) {
            return run_enblend<vigra::UInt8, 3>(levels, wrap, (const vigra::UInt8*)white, white_alpha,
                                                (const vigra::UInt8*)black, black_alpha, mask, w, h, level0);
        }
        return run_enblend<vigra::UInt16, 3>(levels, wrap, (const vigra::UInt16*)white, white_alpha,
                                             (const vigra::UInt16*)black, black_alpha, mask, w, h, level0);
    } catch (const std::exception& e) {
        std::cerr << "ref_enblend: " << e.what() << std::endl;
        return 1;
    }
}

// ---- float images: double pyramids (src/numerictraits.h:185) --------------
// Pyramid levels are (h, w, C) double arrays, pixel images (H, W, 3) float.

// Reduce of one double level (pyramid.h:166-573 with SKIPSMImagePixelType double).
int ref_reduce_f(int C, int alpha, int wrap, const double* src, const uint8_t* src_alpha, int sw, int sh,
                 double* dst, uint8_t* dst_alpha)
{
    try {
        return C == 1 ? run_reduce<float, 1>(alpha, wrap, src, src_alpha, sw, sh, dst, dst_alpha)
                      : run_reduce<float, 3>(alpha, wrap, src, src_alpha, sw, sh, dst, dst_alpha);
    } catch (const std::exception& e) {
        std::cerr << "ref_reduce_f: " << e.what() << std::endl;
        return 1;
    }
}

// Expand of one double level into dst (pyramid.h:1102-1457).
int ref_expand_f(int C, int add, int wrap, const double* src, int sw, int sh, double* dst, int dw, int dh)
{
    try {
        return C == 1 ? run_expand<float, 1>(add, wrap, src, sw, sh, dst, dw, dh)
                      : run_expand<float, 3>(add, wrap, src, sw, sh, dst, dw, dh);
    } catch (const std::exception& e) {
        std::cerr << "ref_expand_f: " << e.what() << std::endl;
        return 1;
    }
}

// The pyramid section of enblendMain on float RGB images: collapsed level 0
// (double, (h, w, 3)) and the float pixels copyFromPyramidImageIf makes of
// it where the union alpha is set (out keeps its values elsewhere).
int ref_enblend_f(int levels, int wrap, const float* white, const uint8_t* white_alpha, const float* black,
                  const uint8_t* black_alpha, const uint8_t* mask, int w, int h, double* level0, float* out)
{
    try {
        const int rc = run_enblend<float, 3, double>(levels, wrap, white, white_alpha, black, black_alpha, mask, w,
                                                     h, level0);
        if (rc) {
            return rc;
        }
        std::vector<uint8_t> ua((size_t)w * h);
        for (size_t i = 0; i < ua.size(); ++i) {
            ua[i] = white_alpha[i] ? 255 : black_alpha[i];
        }
        return run_from_pyramid<float, double>(level0, ua.data(), w, h, out);
    } catch (const std::exception& e) {
        std::cerr << "ref_enblend_f: " << e.what() << std::endl;
        return 1;
    }
}

}  // extern "C"
