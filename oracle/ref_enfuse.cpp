// ref_enfuse.cpp -- C entry points over the reference's own enfuse code:
// src/enfuse.h (enfuseMask and its functors, localStdDevIf, localEntropyIf,
// and enfuseMain itself: weights, normalisation, hard mask, pyramids,
// ImageMaskMultiplyFunctor, accumulation, collapse, dithered output),
// src/assemble.h (image import with the alpha threshold, checkpoint),
// src/mga.h, src/exposure_weight.h and src/alternativepercentage.cc of
// enblend-enfuse, compiled unmodified from the reference tree against the
// VIGRA/GSL/LCMS2 shims in refshim/.  Test oracle only: it pins the C
// restatement in enb_oracle.c to the reference's code.  Built by
// reference_build.py into _ref/ (a library of its own, because src/common.h
// defines functions that the enblend driver's library defines as well).
//
// Images cross this boundary as plain interleaved arrays; enfuseMain reads
// its inputs and writes its output and masks through the shim's in-memory
// image files (vigra::memfile_put / memfile_get), so no file is read or
// written except the empty placeholders that the reference's mask loader
// checks with can_open_file.

#include <config.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <list>
#include <optional>
#include <string>
#include <vector>

#include <unistd.h>

#include "alternativepercentage.h"
#include "exposure_weight.h"
#include "global.h"
#include "parameter.h"
#include "selector.h"

// ---- the globals of enfuse.cc that src/enfuse.h and src/assemble.h read -------------
// (names and types as declared at src/enfuse.cc:99-160; values are set per call)
const std::string command("enfuse-oracle");
std::string OutputFileName("a.tif");
std::optional<std::string> OutputMaskFileName;
int Verbose = 0;
int ExactLevels = 0;
bool OneAtATime = true;
boundary_t WrapAround = OpenBoundaries;
blend_colorspace_t BlendColorspace = IdentitySpace;
double WExposure = 1.0;
double ExposureOptimum = 0.5;
double ExposureWidth = 0.2;
ExposureWeight* ExposureWeightFunction = nullptr;
AlternativePercentage ExposureLowerCutoff(0.0, true);
CompactifiedAlternativePercentage ExposureUpperCutoff(100.0, true);
std::string ExposureLowerCutoffGrayscaleProjector("anti-value");
std::string ExposureUpperCutoffGrayscaleProjector("value");
double WContrast = 0.0;
double WSaturation = 0.0;
double WEntropy = 0.0;
int ContrastWindowSize = 5;
std::string GrayscaleProjector;
struct EdgeFilterConfiguration {
    double edgeScale, lceScale, lceFactor;
} FilterConfig = {0.0, 0.0, 0.0};
AlternativePercentage MinCurvature(0.0, false);
int EntropyWindowSize = 3;
AlternativePercentage EntropyLowerCutoff(0.0, true);
CompactifiedAlternativePercentage EntropyUpperCutoff(100.0, true);
bool UseHardMask = false;
bool SaveMasks = false;
bool StopAfterMaskGeneration = false;
bool LoadMasks = false;
std::string SoftMaskTemplate("softmask-%n.tif");
std::string HardMaskTemplate("hardmask-%n.tif");
TiffResolution ImageResolution;
bool OutputIsValid = true;
cmsHPROFILE InputProfile = nullptr;
cmsHTRANSFORM InputToXYZTransform = nullptr;
cmsHTRANSFORM XYZToInputTransform = nullptr;
cmsHTRANSFORM InputToLabTransform = nullptr;
cmsHTRANSFORM LabToInputTransform = nullptr;
cmsHANDLE CIECAMTransform = nullptr;

#include <vigra/imageinfo.hxx>
#include <vigra/impex.hxx>

#include "common.h"
#include "filespec.h"
#include "enfuse.h"

// ---- definitions behind declarations the included headers make ------------------------
// The static tables of enblend::Histogram (defined by enfuse.cc, src/enfuse.cc:199-205).
template <typename InputPixelType, typename ResultPixelType>
size_t enblend::Histogram<InputPixelType, ResultPixelType>::precomputedSize = 0;
template <typename InputPixelType, typename ResultPixelType>
double* enblend::Histogram<InputPixelType, ResultPixelType>::precomputedLog = nullptr;
template <typename InputPixelType, typename ResultPixelType>
double* enblend::Histogram<InputPixelType, ResultPixelType>::precomputedEntropy = nullptr;

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
}  // namespace enblend

// Constant dither draws (gsl_shim.cpp): < 0 keeps the Mersenne Twister.
extern "C" void gsl_shim_set_constant(long long value);

// ---- parameters of one call -----------------------------------------------------------------
extern "C" {

// enfuse's weighting options (src/enfuse.cc:117-160); cutoffs as the
// AlternativePercentage pairs --exposure-cutoff / --entropy-cutoff set.
typedef struct {
    double w_exposure, w_saturation, w_contrast, w_entropy;
    double exp_optimum, exp_width;
    int32_t exp_function;     // 0 gaussian, 1 lorentzian, 2 half-sine, 3 full-sine, 4 bisquare
    int32_t contrast_window, entropy_window;
    int32_t hard_mask;
    double exp_cutoff[2];     // lower, upper
    int32_t exp_cutoff_pct[2];
    double ent_cutoff[2];
    int32_t ent_cutoff_pct[2];
    char gray_projector[96];  // --gray-projector ("" = default)
    char exp_cutoff_projector[2][32];
} ref_enfuse_params;

}  // extern "C"

namespace {

ExposureWeight* make_function(int fn, double opt, double width)
{
    switch (fn) {
    case 1: return new exposure_weight::Lorentzian(opt, width);
    case 2: return new exposure_weight::HalfSinusodial(opt, width);
    case 3: return new exposure_weight::FullSinusodial(opt, width);
    case 4: return new exposure_weight::Bisquare(opt, width);
    default: return new exposure_weight::Gaussian(opt, width);
    }
}

void set_globals(const ref_enfuse_params* p)
{
    WExposure = p->w_exposure;
    WSaturation = p->w_saturation;
    WContrast = p->w_contrast;
    WEntropy = p->w_entropy;
    ExposureOptimum = p->exp_optimum;
    ExposureWidth = p->exp_width;
    delete ExposureWeightFunction;
    ExposureWeightFunction = make_function(p->exp_function, p->exp_optimum, p->exp_width);
    ContrastWindowSize = p->contrast_window;
    EntropyWindowSize = p->entropy_window;
    UseHardMask = p->hard_mask != 0;
    ExposureLowerCutoff.set_value(p->exp_cutoff[0]);
    ExposureLowerCutoff.set_percentage(p->exp_cutoff_pct[0] != 0);
    ExposureUpperCutoff.set_value(p->exp_cutoff[1]);
    ExposureUpperCutoff.set_percentage(p->exp_cutoff_pct[1] != 0);
    EntropyLowerCutoff.set_value(p->ent_cutoff[0]);
    EntropyLowerCutoff.set_percentage(p->ent_cutoff_pct[0] != 0);
    EntropyUpperCutoff.set_value(p->ent_cutoff[1]);
    EntropyUpperCutoff.set_percentage(p->ent_cutoff_pct[1] != 0);
    GrayscaleProjector = p->gray_projector;
    ExposureLowerCutoffGrayscaleProjector = p->exp_cutoff_projector[0];
    ExposureUpperCutoffGrayscaleProjector = p->exp_cutoff_projector[1];
}

const char* pixel_type_of(int depth) { return depth == 8 ? "UINT8" : (depth == 16 ? "UINT16" : "FLOAT"); }

double sample_at(const void* p, int depth, size_t i)
{
    if (depth == 8) {
        return static_cast<const uint8_t*>(p)[i];
    }
    if (depth == 16) {
        return static_cast<const uint16_t*>(p)[i];
    }
    return static_cast<const float*>(p)[i];
}

void store_at(void* p, int depth, size_t i, double v)
{
    if (depth == 8) {
        static_cast<uint8_t*>(p)[i] = (uint8_t)v;
    } else if (depth == 16) {
        static_cast<uint16_t*>(p)[i] = (uint16_t)v;
    } else {
        static_cast<float*>(p)[i] = (float)v;
    }
}

// An interleaved image as an in-memory file: S samples a pixel, the 4th (or
// 2nd of gray + alpha) being the extra band.
vigra::MemFile memfile_of(const void* img, int depth, int S, int w, int h)
{
    vigra::MemFile f;
    f.width = w;
    f.height = h;
    f.bands = S;
    f.extra = (S == 2 || S == 4) ? 1 : 0;
    f.pixel_type = pixel_type_of(depth);
    f.samples.resize((size_t)w * h * S);
    for (size_t i = 0; i < f.samples.size(); ++i) {
        f.samples[i] = sample_at(img, depth, i);
    }
    return f;
}

template <class Pixel>
struct PixelIO;

template <class T>
struct PixelIO<vigra::RGBValue<T>> {
    static vigra::RGBValue<T> get(const void* p, int depth, size_t i)
    {
        return vigra::RGBValue<T>((T)sample_at(p, depth, 3 * i), (T)sample_at(p, depth, 3 * i + 1),
                                  (T)sample_at(p, depth, 3 * i + 2));
    }
};

template <class T>
struct PixelIO {
    static T get(const void* p, int depth, size_t i) { return (T)sample_at(p, depth, i); }
};

// enfuseMask on one image (its colour samples interleaved, alpha a plane).
template <class Pixel>
int enfuse_mask_impl(int depth, const void* img, const uint8_t* alpha, int w, int h, float* out)
{
    typedef vigra::BasicImage<Pixel> ImageType;
    typedef vigra::BasicImage<vigra::UInt8> AlphaType;
    typedef vigra::BasicImage<float> MaskType;
    ImageType image(w, h);
    AlphaType a(w, h);
    MaskType mask(w, h);
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            const size_t i = (size_t)y * w + x;
            image(x, y) = PixelIO<Pixel>::get(img, depth, i);
            a(x, y) = alpha ? alpha[i] : 255;
        }
    }
    enblend::enfuseMask<ImageType, AlphaType, MaskType>(srcImageRange(image), srcImage(a), destImage(mask));
    std::memcpy(out, mask.data(), sizeof(float) * (size_t)w * h);
    return 0;
}

std::string scratch_dir()
{
    static std::string dir;
    if (dir.empty()) {
        char tmpl[] = "/tmp/enb_ref_enfuse_XXXXXX";
        const char* d = mkdtemp(tmpl);
        dir = d ? d : "/tmp";
    }
    return dir;
}

template <class Pixel>
int enfuse_main_impl(int depth, int S, int K, const void* const* imgs, int w, int h,
                     const float* const* load_masks, void* out, float* saved_masks)
{
    vigra::memfile_clear();
    const std::string dir = scratch_dir();
    enblend::FileNameList names;
    std::list<vigra::ImageImportInfo*> infos;
    for (int k = 0; k < K; ++k) {
        const std::string name = dir + "/input-" + std::to_string(k) + ".tif";
        vigra::memfile_put(name, memfile_of(imgs[k], depth, S, w, h));
        names.push_back(name);
    }
    for (const std::string& n : names) {
        infos.push_back(new vigra::ImageImportInfo(n.c_str()));
    }
    SoftMaskTemplate = dir + "/softmask-%n.tif";
    HardMaskTemplate = dir + "/hardmask-%n.tif";
    OutputFileName = dir + "/output.tif";
    LoadMasks = load_masks != nullptr;
    SaveMasks = saved_masks != nullptr;
    if (LoadMasks) {
        for (int k = 0; k < K; ++k) {
            const std::string mname = enblend::expandFilenameTemplate(UseHardMask ? HardMaskTemplate : SoftMaskTemplate,
                                                                      K, *std::next(names.begin(), k), OutputFileName, k);
            vigra::memfile_put(mname, memfile_of(load_masks[k], 32, 1, w, h));
            FILE* placeholder = std::fopen(mname.c_str(), "w");  // for can_open_file
            if (placeholder) {
                std::fclose(placeholder);
            }
        }
    }
    vigra::ImageExportInfo out_info(OutputFileName.c_str());
    out_info.setPixelType(pixel_type_of(depth));
    vigra::Rect2D input_union(vigra::Size2D(w, h));
    enblend::enfuseMain<Pixel>(names, infos, out_info, input_union);
    for (vigra::ImageImportInfo* i : infos) {
        delete i;
    }
    vigra::MemFile o;
    if (!vigra::memfile_get(OutputFileName, o)) {
        return -2;
    }
    for (size_t i = 0; i < o.samples.size(); ++i) {
        store_at(out, depth, i, o.samples[i]);
    }
    if (saved_masks) {
        for (int k = 0; k < K; ++k) {
            const std::string mname = enblend::expandFilenameTemplate(UseHardMask ? HardMaskTemplate : SoftMaskTemplate,
                                                                      K, *std::next(names.begin(), k), OutputFileName, k);
            vigra::MemFile m;
            if (!vigra::memfile_get(mname, m) || m.bands != 1) {
                return -3;
            }
            for (size_t i = 0; i < (size_t)w * h; ++i) {
                saved_masks[(size_t)k * w * h + i] = (float)m.samples[i];
            }
        }
    }
    return 0;
}

}  // namespace

extern "C" {

// enfuseMask (src/enfuse.h:962-1212) of one image: depth 8/16 (integers) or
// 32 (float), C = 1 (gray) or 3 (RGB) colour samples a pixel, alpha plane
// (or NULL: opaque); out: w*h weights.  0 on success.
int ref_enfuse_mask(const ref_enfuse_params* p, int depth, int C, const void* img, const uint8_t* alpha, int w, int h,
                    float* out)
{
    try {
        set_globals(p);
        if (C == 3) {
            return depth == 8    ? enfuse_mask_impl<vigra::RGBValue<vigra::UInt8>>(depth, img, alpha, w, h, out)
                   : depth == 16 ? enfuse_mask_impl<vigra::RGBValue<vigra::UInt16>>(depth, img, alpha, w, h, out)
                                 : enfuse_mask_impl<vigra::RGBValue<float>>(depth, img, alpha, w, h, out);
        }
        return depth == 8    ? enfuse_mask_impl<vigra::UInt8>(depth, img, alpha, w, h, out)
               : depth == 16 ? enfuse_mask_impl<vigra::UInt16>(depth, img, alpha, w, h, out)
                             : enfuse_mask_impl<float>(depth, img, alpha, w, h, out);
    } catch (const std::exception& e) {
        std::cerr << "ref_enfuse_mask: " << e.what() << std::endl;
        return -1;
    }
}

// enfuseMain (src/enfuse.h:1217-1617) on K union-sized images of S samples a
// pixel (3 RGB, 4 RGBA with the alpha thresholded on import, 1 gray, 2 gray +
// alpha), all at the canvas origin.  levels: --levels (0 automatic); wrap:
// --wrap=horizontal.  load_masks: K weight planes for --load-masks, or NULL.
// dither: < 0 the Mersenne Twister, else every draw returns this value.
// out: w*h*(C+1) samples, the output image with its alpha band (0 or the
// type's maximum) as the reference's checkpoint writes it.  saved_masks:
// K*w*h floats, the soft (or, with the hard mask, the hard) masks written by
// --save-masks, or NULL.  0 on success.
int ref_enfuse_main(const ref_enfuse_params* p, int depth, int S, int K, const void* const* imgs, int w, int h,
                    int levels, int wrap, const float* const* load_masks, long long dither, void* out,
                    float* saved_masks)
{
    try {
        set_globals(p);
        ExactLevels = levels;
        WrapAround = wrap ? HorizontalStrip : OpenBoundaries;
        gsl_shim_set_constant(dither);
        const int C = (S == 3 || S == 4) ? 3 : 1;
        int rc;
        if (C == 3) {
            rc = depth == 8    ? enfuse_main_impl<vigra::RGBValue<vigra::UInt8>>(depth, S, K, imgs, w, h, load_masks,
                                                                                 out, saved_masks)
                 : depth == 16 ? enfuse_main_impl<vigra::RGBValue<vigra::UInt16>>(depth, S, K, imgs, w, h, load_masks,
                                                                                  out, saved_masks)
                               : enfuse_main_impl<vigra::RGBValue<float>>(depth, S, K, imgs, w, h, load_masks, out,
                                                                         saved_masks);
        } else {
            rc = depth == 8    ? enfuse_main_impl<vigra::UInt8>(depth, S, K, imgs, w, h, load_masks, out, saved_masks)
                 : depth == 16 ? enfuse_main_impl<vigra::UInt16>(depth, S, K, imgs, w, h, load_masks, out, saved_masks)
                               : enfuse_main_impl<float>(depth, S, K, imgs, w, h, load_masks, out, saved_masks);
        }
        gsl_shim_set_constant(-1);
        return rc;
    } catch (const std::exception& e) {
        gsl_shim_set_constant(-1);
        std::cerr << "ref_enfuse_main: " << e.what() << std::endl;
        return -1;
    }
}

}  // extern "C"
