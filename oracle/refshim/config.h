/* config.h for compiling the reference's pyramid/blend/fixmath headers
 * unmodified against the project's VIGRA/GSL/LCMS2 shims (test oracle only).
 * The build defines HAVE_CONFIG_H so that every reference header includes
 * this file first. */
#ifndef ENB_REFSHIM_CONFIG_H
#define ENB_REFSHIM_CONFIG_H

#define PACKAGE "enblend"
#define VERSION "shim"

#include <lcms2.h>

/* Standard facilities the reference's configure step detects. */
#define HAVE_OPTIONAL 1
#define HAVE_DECL_STRERROR_R 1
#define STRERROR_R_CHAR_P 1

#ifdef __cplusplus
#include <functional>
#include <string>
/* Globals of enblend.cc that the headers use. */
extern const std::string command;
extern int Verbose;
#endif

/* Colour-space transforms of enblend.cc/enfuse.cc; only the identity colour
 * space is used by the oracle, so they stay null. */
extern cmsHTRANSFORM InputToXYZTransform;
extern cmsHTRANSFORM XYZToInputTransform;
extern cmsHTRANSFORM InputToLabTransform;
extern cmsHTRANSFORM LabToInputTransform;
extern cmsHANDLE CIECAMTransform;

#endif

#define RESTRICT __restrict__

/* Image container of the reference's numerictraits.h macros. */
#define IMAGETYPE vigra::BasicImage
