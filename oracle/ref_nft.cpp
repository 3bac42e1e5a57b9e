// ref_nft.cpp -- C entry point over the reference's own nearest-feature
// transform (src/nearest.h: nearestFeatureTransform, periodicDistanceTransform,
// quick_tally; src/openmp_vigra.h: the Felzenszwalb-Huttenlocher distance
// transform of its OpenMP build) of enblend-enfuse, compiled unmodified from
// the reference tree against the VIGRA shims in refshim/ with OPENMP defined
// (the reference's OpenMP build; without OpenMP it calls VIGRA's own distance
// transform instead).  Test oracle only: it pins the C restatement in
// enb_oracle.c.  Built by reference_build.py into _ref/.
//
// The seam mask of `enblend --fine-mask --no-optimize` (src/mask.h:1130-1180):
// 255 where the nearest white-only pixel is nearer than the nearest
// black-only pixel, else 0, over the union canvas; wrap: the horizontally
// periodic transform.

#include <config.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>

#include "global.h"
#include "common.h"

// globals of enblend.cc that src/nearest.h reads (names and types as declared
// at src/enblend.cc:133-134; only its verbose messages use them)
extern bool CoarseMask;
extern unsigned CoarsenessFactor;

#include "openmp_def.h"
#include "openmp_vigra.h"
#include "parameter.h"
#include "nearest.h"

const std::string command("enblend-oracle");
int Verbose = 0;
bool CoarseMask = false;
unsigned CoarsenessFactor = 8U;
cmsHTRANSFORM InputToXYZTransform = nullptr;
cmsHTRANSFORM XYZToInputTransform = nullptr;
cmsHTRANSFORM InputToLabTransform = nullptr;
cmsHTRANSFORM LabToInputTransform = nullptr;
cmsHANDLE CIECAMTransform = nullptr;

extern "C" {

// mask (h, w) of the alpha planes white (h, w) and black (h, w), 0/255 each.
// Returns 0, or 2 when the reference rejects the pair for too much overlap
// (it exits there; here the process continues).
int ref_nft_mask(const uint8_t* white, const uint8_t* black, int w, int h, int wrap, uint8_t* mask)
{
    typedef vigra::BasicImage<vigra::UInt8> Img;
    Img wa(w, h), ba(w, h), out(w, h);
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            wa(x, y) = white[(size_t)y * w + x];
            ba(x, y) = black[(size_t)y * w + x];
        }
    }
    // the overlap check exits the process; evaluate it first as the reference does
    const unsigned threshold = 2U * 2U * (static_cast<unsigned>(h) + static_cast<unsigned>(w));
    unsigned t12 = 0U, t21 = 0U;
    for (size_t i = 0; i < (size_t)w * h && (t12 < threshold || t21 < threshold); ++i) {
        t12 += (white[i] > black[i]) ? 1U : 0U;
        t21 += (black[i] > white[i]) ? 1U : 0U;
    }
    if (std::max(std::min(t12, threshold), std::min(t21, threshold)) < threshold) {
        return 2;
    }
    enblend::nearestFeatureTransform(srcImageRange(wa), srcImage(ba), destImage(out), enblend::EuclideanDistance,
                                     wrap ? HorizontalStrip : OpenBoundaries);
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            mask[(size_t)y * w + x] = out(x, y);
        }
    }
    return 0;
}

}  // extern "C"
