// enb_sortnet.cuh -- generated by gen_sortnet.py (Batcher's odd-even merge
// sort, pruned to the live keys); do not edit by hand.
#pragma once

#include <stdint.h>

namespace enb {

__device__ __forceinline__ void sortnet_ce(uint32_t& a, uint32_t& b)
{
    const uint32_t lo = min(a, b);
    b = max(a, b);
    a = lo;
}

// Sorts k[0..8] ascending (28 comparators).
__device__ __forceinline__ void sortnet9(uint32_t (&k)[9])
{
    sortnet_ce(k[0], k[1]);
    sortnet_ce(k[2], k[3]);
    sortnet_ce(k[4], k[5]);
    sortnet_ce(k[6], k[7]);
    sortnet_ce(k[0], k[2]);
    sortnet_ce(k[1], k[3]);
    sortnet_ce(k[4], k[6]);
    sortnet_ce(k[5], k[7]);
    sortnet_ce(k[1], k[2]);
    sortnet_ce(k[5], k[6]);
    sortnet_ce(k[0], k[4]);
    sortnet_ce(k[1], k[5]);
    sortnet_ce(k[2], k[6]);
    sortnet_ce(k[3], k[7]);
    sortnet_ce(k[2], k[4]);
    sortnet_ce(k[3], k[5]);
    sortnet_ce(k[1], k[2]);
    sortnet_ce(k[3], k[4]);
    sortnet_ce(k[5], k[6]);
    sortnet_ce(k[0], k[8]);
    sortnet_ce(k[4], k[8]);
    sortnet_ce(k[2], k[4]);
    sortnet_ce(k[3], k[5]);
    sortnet_ce(k[6], k[8]);
    sortnet_ce(k[1], k[2]);
    sortnet_ce(k[3], k[4]);
    sortnet_ce(k[5], k[6]);
    sortnet_ce(k[7], k[8]);
}

// Sorts k[0..24] ascending (140 comparators).
__device__ __forceinline__ void sortnet25(uint32_t (&k)[25])
{
    sortnet_ce(k[0], k[1]);
    sortnet_ce(k[2], k[3]);
    sortnet_ce(k[4], k[5]);
    sortnet_ce(k[6], k[7]);
    sortnet_ce(k[8], k[9]);
    sortnet_ce(k[10], k[11]);
    sortnet_ce(k[12], k[13]);
    sortnet_ce(k[14], k[15]);
    sortnet_ce(k[16], k[17]);
    sortnet_ce(k[18], k[19]);
    sortnet_ce(k[20], k[21]);
    sortnet_ce(k[22], k[23]);
    sortnet_ce(k[0], k[2]);
    sortnet_ce(k[1], k[3]);
    sortnet_ce(k[4], k[6]);
    sortnet_ce(k[5], k[7]);
    sortnet_ce(k[8], k[10]);
    sortnet_ce(k[9], k[11]);
    sortnet_ce(k[12], k[14]);
    sortnet_ce(k[13], k[15]);
    sortnet_ce(k[16], k[18]);
    sortnet_ce(k[17], k[19]);
    sortnet_ce(k[20], k[22]);
    sortnet_ce(k[21], k[23]);
    sortnet_ce(k[1], k[2]);
    sortnet_ce(k[5], k[6]);
    sortnet_ce(k[9], k[10]);
    sortnet_ce(k[13], k[14]);
    sortnet_ce(k[17], k[18]);
    sortnet_ce(k[21], k[22]);
    sortnet_ce(k[0], k[4]);
    sortnet_ce(k[1], k[5]);
    sortnet_ce(k[2], k[6]);
    sortnet_ce(k[3], k[7]);
    sortnet_ce(k[8], k[12]);
    sortnet_ce(k[9], k[13]);
    sortnet_ce(k[10], k[14]);
    sortnet_ce(k[11], k[15]);
    sortnet_ce(k[16], k[20]);
    sortnet_ce(k[17], k[21]);
    sortnet_ce(k[18], k[22]);
    sortnet_ce(k[19], k[23]);
    sortnet_ce(k[2], k[4]);
    sortnet_ce(k[3], k[5]);
    sortnet_ce(k[10], k[12]);
    sortnet_ce(k[11], k[13]);
    sortnet_ce(k[18], k[20]);
    sortnet_ce(k[19], k[21]);
    sortnet_ce(k[1], k[2]);
    sortnet_ce(k[3], k[4]);
    sortnet_ce(k[5], k[6]);
    sortnet_ce(k[9], k[10]);
    sortnet_ce(k[11], k[12]);
    sortnet_ce(k[13], k[14]);
    sortnet_ce(k[17], k[18]);
    sortnet_ce(k[19], k[20]);
    sortnet_ce(k[21], k[22]);
    sortnet_ce(k[0], k[8]);
    sortnet_ce(k[1], k[9]);
    sortnet_ce(k[2], k[10]);
    sortnet_ce(k[3], k[11]);
    sortnet_ce(k[4], k[12]);
    sortnet_ce(k[5], k[13]);
    sortnet_ce(k[6], k[14]);
    sortnet_ce(k[7], k[15]);
    sortnet_ce(k[16], k[24]);
    sortnet_ce(k[4], k[8]);
    sortnet_ce(k[5], k[9]);
    sortnet_ce(k[6], k[10]);
    sortnet_ce(k[7], k[11]);
    sortnet_ce(k[20], k[24]);
    sortnet_ce(k[2], k[4]);
    sortnet_ce(k[3], k[5]);
    sortnet_ce(k[6], k[8]);
    sortnet_ce(k[7], k[9]);
    sortnet_ce(k[10], k[12]);
    sortnet_ce(k[11], k[13]);
    sortnet_ce(k[18], k[20]);
    sortnet_ce(k[19], k[21]);
    sortnet_ce(k[22], k[24]);
    sortnet_ce(k[1], k[2]);
    sortnet_ce(k[3], k[4]);
    sortnet_ce(k[5], k[6]);
    sortnet_ce(k[7], k[8]);
    sortnet_ce(k[9], k[10]);
    sortnet_ce(k[11], k[12]);
    sortnet_ce(k[13], k[14]);
    sortnet_ce(k[17], k[18]);
    sortnet_ce(k[19], k[20]);
    sortnet_ce(k[21], k[22]);
    sortnet_ce(k[23], k[24]);
    sortnet_ce(k[0], k[16]);
    sortnet_ce(k[1], k[17]);
    sortnet_ce(k[2], k[18]);
    sortnet_ce(k[3], k[19]);
    sortnet_ce(k[4], k[20]);
    sortnet_ce(k[5], k[21]);
    sortnet_ce(k[6], k[22]);
    sortnet_ce(k[7], k[23]);
    sortnet_ce(k[8], k[24]);
    sortnet_ce(k[8], k[16]);
    sortnet_ce(k[9], k[17]);
    sortnet_ce(k[10], k[18]);
    sortnet_ce(k[11], k[19]);
    sortnet_ce(k[12], k[20]);
    sortnet_ce(k[13], k[21]);
    sortnet_ce(k[14], k[22]);
    sortnet_ce(k[15], k[23]);
    sortnet_ce(k[4], k[8]);
    sortnet_ce(k[5], k[9]);
    sortnet_ce(k[6], k[10]);
    sortnet_ce(k[7], k[11]);
    sortnet_ce(k[12], k[16]);
    sortnet_ce(k[13], k[17]);
    sortnet_ce(k[14], k[18]);
    sortnet_ce(k[15], k[19]);
    sortnet_ce(k[20], k[24]);
    sortnet_ce(k[2], k[4]);
    sortnet_ce(k[3], k[5]);
    sortnet_ce(k[6], k[8]);
    sortnet_ce(k[7], k[9]);
    sortnet_ce(k[10], k[12]);
    sortnet_ce(k[11], k[13]);
    sortnet_ce(k[14], k[16]);
    sortnet_ce(k[15], k[17]);
    sortnet_ce(k[18], k[20]);
    sortnet_ce(k[19], k[21]);
    sortnet_ce(k[22], k[24]);
    sortnet_ce(k[1], k[2]);
    sortnet_ce(k[3], k[4]);
    sortnet_ce(k[5], k[6]);
    sortnet_ce(k[7], k[8]);
    sortnet_ce(k[9], k[10]);
    sortnet_ce(k[11], k[12]);
    sortnet_ce(k[13], k[14]);
    sortnet_ce(k[15], k[16]);
    sortnet_ce(k[17], k[18]);
    sortnet_ce(k[19], k[20]);
    sortnet_ce(k[21], k[22]);
    sortnet_ce(k[23], k[24]);
}

}  // namespace enb
