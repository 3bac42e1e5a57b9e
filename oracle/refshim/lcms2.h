/* Minimal LCMS2 declarations for the reference's fixmath.h (test oracle
 * only): the non-identity colour spaces that call these are never used;
 * the definitions in ref_driver.cpp abort. */
#ifndef ENB_REFSHIM_LCMS2_H
#define ENB_REFSHIM_LCMS2_H

#include <cstdint>

typedef void* cmsHTRANSFORM;
typedef void* cmsHANDLE;
typedef void* cmsHPROFILE;
typedef uint32_t cmsUInt32Number;
typedef double cmsFloat64Number;
typedef int cmsBool;

typedef struct { double X, Y, Z; } cmsCIEXYZ;
typedef struct { double L, a, b; } cmsCIELab;
typedef struct { double J, C, h; } cmsJCh;
typedef struct { double x, y, Y; } cmsCIExyY;

typedef enum { cmsInfoDescription = 0, cmsInfoManufacturer = 1, cmsInfoModel = 2, cmsInfoCopyright = 3 } cmsInfoType;
typedef uint32_t cmsColorSpaceSignature;
#define cmsNoLanguage "\0\0"
#define cmsNoCountry "\0\0"
#define cmsFLAGS_NOCACHE 0x0040
#define cmsFLAGS_HIGHRESPRECALC 0x0400
#define INTENT_PERCEPTUAL 0

cmsUInt32Number cmsGetProfileInfoASCII(cmsHPROFILE, cmsInfoType, const char*, const char*, char*, cmsUInt32Number);
cmsColorSpaceSignature cmsGetColorSpace(cmsHPROFILE);
cmsUInt32Number cmsChannelsOf(cmsColorSpaceSignature);
void cmsDoTransform(cmsHTRANSFORM, const void*, void*, cmsUInt32Number);
double cmsCMCdeltaE(const cmsCIELab*, const cmsCIELab*, double, double);
void cmsCIECAM02Forward(cmsHANDLE, const cmsCIEXYZ*, cmsJCh*);
void cmsCIECAM02Reverse(cmsHANDLE, const cmsJCh*, cmsCIEXYZ*);

#endif
