// enb_sortnet.cuh -- generated by gen_sortnet.py (Batcher's odd-even merge
// sort, pruned to the live keys); do not edit by hand.
#pragma once

#include <stdint.h>

namespace enb {

// Compare-exchange of two 32-bit keys (ascending).
struct CeU32 {
    __device__ __forceinline__ void operator()(uint32_t& a, uint32_t& b) const
    {
        const uint32_t lo = min(a, b);
        b = max(a, b);
        a = lo;
    }
};

// Compare-exchange of the two 16-bit halves of two words independently
// (two windows sorted at once, one per half).
struct CeU16x2 {
    __device__ __forceinline__ void operator()(uint32_t& a, uint32_t& b) const
    {
        uint32_t lo, hi;
        asm("min.u16x2 %0, %1, %2;" : "=r"(lo) : "r"(a), "r"(b));
        asm("max.u16x2 %0, %1, %2;" : "=r"(hi) : "r"(a), "r"(b));
        a = lo;
        b = hi;
    }
};

// Sorts k[0..8] ascending (28 comparators).
template <class CE = CeU32>
__device__ __forceinline__ void sortnet9(uint32_t (&k)[9], CE ce = CE())
{
    ce(k[0], k[1]);
    ce(k[2], k[3]);
    ce(k[4], k[5]);
    ce(k[6], k[7]);
    ce(k[0], k[2]);
    ce(k[1], k[3]);
    ce(k[4], k[6]);
    ce(k[5], k[7]);
    ce(k[1], k[2]);
    ce(k[5], k[6]);
    ce(k[0], k[4]);
    ce(k[1], k[5]);
    ce(k[2], k[6]);
    ce(k[3], k[7]);
    ce(k[2], k[4]);
    ce(k[3], k[5]);
    ce(k[1], k[2]);
    ce(k[3], k[4]);
    ce(k[5], k[6]);
    ce(k[0], k[8]);
    ce(k[4], k[8]);
    ce(k[2], k[4]);
    ce(k[3], k[5]);
    ce(k[6], k[8]);
    ce(k[1], k[2]);
    ce(k[3], k[4]);
    ce(k[5], k[6]);
    ce(k[7], k[8]);
}

// Sorts k[0..24] ascending (140 comparators).
template <class CE = CeU32>
__device__ __forceinline__ void sortnet25(uint32_t (&k)[25], CE ce = CE())
{
    ce(k[0], k[1]);
    ce(k[2], k[3]);
    ce(k[4], k[5]);
    ce(k[6], k[7]);
    ce(k[8], k[9]);
    ce(k[10], k[11]);
    ce(k[12], k[13]);
    ce(k[14], k[15]);
    ce(k[16], k[17]);
    ce(k[18], k[19]);
    ce(k[20], k[21]);
    ce(k[22], k[23]);
    ce(k[0], k[2]);
    ce(k[1], k[3]);
    ce(k[4], k[6]);
    ce(k[5], k[7]);
    ce(k[8], k[10]);
    ce(k[9], k[11]);
    ce(k[12], k[14]);
    ce(k[13], k[15]);
    ce(k[16], k[18]);
    ce(k[17], k[19]);
    ce(k[20], k[22]);
    ce(k[21], k[23]);
    ce(k[1], k[2]);
    ce(k[5], k[6]);
    ce(k[9], k[10]);
    ce(k[13], k[14]);
    ce(k[17], k[18]);
    ce(k[21], k[22]);
    ce(k[0], k[4]);
    ce(k[1], k[5]);
    ce(k[2], k[6]);
    ce(k[3], k[7]);
    ce(k[8], k[12]);
    ce(k[9], k[13]);
    ce(k[10], k[14]);
    ce(k[11], k[15]);
    ce(k[16], k[20]);
    ce(k[17], k[21]);
    ce(k[18], k[22]);
    ce(k[19], k[23]);
    ce(k[2], k[4]);
    ce(k[3], k[5]);
    ce(k[10], k[12]);
    ce(k[11], k[13]);
    ce(k[18], k[20]);
    ce(k[19], k[21]);
    ce(k[1], k[2]);
    ce(k[3], k[4]);
    ce(k[5], k[6]);
    ce(k[9], k[10]);
    ce(k[11], k[12]);
    ce(k[13], k[14]);
    ce(k[17], k[18]);
    ce(k[19], k[20]);
    ce(k[21], k[22]);
    ce(k[0], k[8]);
    ce(k[1], k[9]);
    ce(k[2], k[10]);
    ce(k[3], k[11]);
    ce(k[4], k[12]);
    ce(k[5], k[13]);
    ce(k[6], k[14]);
    ce(k[7], k[15]);
    ce(k[16], k[24]);
    ce(k[4], k[8]);
    ce(k[5], k[9]);
    ce(k[6], k[10]);
    ce(k[7], k[11]);
    ce(k[20], k[24]);
    ce(k[2], k[4]);
    ce(k[3], k[5]);
    ce(k[6], k[8]);
    ce(k[7], k[9]);
    ce(k[10], k[12]);
    ce(k[11], k[13]);
    ce(k[18], k[20]);
    ce(k[19], k[21]);
    ce(k[22], k[24]);
    ce(k[1], k[2]);
    ce(k[3], k[4]);
    ce(k[5], k[6]);
    ce(k[7], k[8]);
    ce(k[9], k[10]);
    ce(k[11], k[12]);
    ce(k[13], k[14]);
    ce(k[17], k[18]);
    ce(k[19], k[20]);
    ce(k[21], k[22]);
    ce(k[23], k[24]);
    ce(k[0], k[16]);
    ce(k[1], k[17]);
    ce(k[2], k[18]);
    ce(k[3], k[19]);
    ce(k[4], k[20]);
    ce(k[5], k[21]);
    ce(k[6], k[22]);
    ce(k[7], k[23]);
    ce(k[8], k[24]);
    ce(k[8], k[16]);
    ce(k[9], k[17]);
    ce(k[10], k[18]);
    ce(k[11], k[19]);
    ce(k[12], k[20]);
    ce(k[13], k[21]);
    ce(k[14], k[22]);
    ce(k[15], k[23]);
    ce(k[4], k[8]);
    ce(k[5], k[9]);
    ce(k[6], k[10]);
    ce(k[7], k[11]);
    ce(k[12], k[16]);
    ce(k[13], k[17]);
    ce(k[14], k[18]);
    ce(k[15], k[19]);
    ce(k[20], k[24]);
    ce(k[2], k[4]);
    ce(k[3], k[5]);
    ce(k[6], k[8]);
    ce(k[7], k[9]);
    ce(k[10], k[12]);
    ce(k[11], k[13]);
    ce(k[14], k[16]);
    ce(k[15], k[17]);
    ce(k[18], k[20]);
    ce(k[19], k[21]);
    ce(k[22], k[24]);
    ce(k[1], k[2]);
    ce(k[3], k[4]);
    ce(k[5], k[6]);
    ce(k[7], k[8]);
    ce(k[9], k[10]);
    ce(k[11], k[12]);
    ce(k[13], k[14]);
    ce(k[15], k[16]);
    ce(k[17], k[18]);
    ce(k[19], k[20]);
    ce(k[21], k[22]);
    ce(k[23], k[24]);
}

}  // namespace enb
