"""Generate enb_sortnet.cuh: Batcher's odd-even merge sorting networks for the
local-entropy windows (3x3 = 9 and 5x5 = 25 keys), padded to 16 and 32 keys
and pruned of every comparator that touches a padding position (padding keys
are the maximum key, so such comparators never exchange).

Usage: python gen_sortnet.py > enb_sortnet.cuh
"""


def batcher(n_pow2: int, live: int):
    pairs = []
    p = 1
    while p < n_pow2:
        k = p
        while k >= 1:
            j = k % p
            while j + k < n_pow2:
                for i in range(k):
                    a, b = i + j, i + j + k
                    if a // (2 * p) == b // (2 * p) and b < live:
                        pairs.append((a, b))
                j += 2 * k
            k //= 2
        p *= 2
    return pairs


def check(pairs, live):
    import itertools
    import random
    rnd = random.Random(1)
    for _ in range(20000):
        v = [rnd.randrange(6) for _ in range(live)]
        for a, b in pairs:
            if v[a] > v[b]:
                v[a], v[b] = v[b], v[a]
        assert v == sorted(v)


def main():
    print("// enb_sortnet.cuh -- generated by gen_sortnet.py (Batcher's odd-even merge")
    print("// sort, pruned to the live keys); do not edit by hand.")
    print("#pragma once")
    print()
    print("#include <stdint.h>")
    print()
    print("namespace enb {")
    print()
    print("// Compare-exchange of two 32-bit keys (ascending).")
    print("struct CeU32 {")
    print("    __device__ __forceinline__ void operator()(uint32_t& a, uint32_t& b) const")
    print("    {")
    print("        const uint32_t lo = min(a, b);")
    print("        b = max(a, b);")
    print("        a = lo;")
    print("    }")
    print("};")
    print()
    print("// Compare-exchange of the two 16-bit halves of two words independently")
    print("// (two windows sorted at once, one per half).")
    print("struct CeU16x2 {")
    print("    __device__ __forceinline__ void operator()(uint32_t& a, uint32_t& b) const")
    print("    {")
    print("        uint32_t lo, hi;")
    print('        asm("min.u16x2 %0, %1, %2;" : "=r"(lo) : "r"(a), "r"(b));')
    print('        asm("max.u16x2 %0, %1, %2;" : "=r"(hi) : "r"(a), "r"(b));')
    print("        a = lo;")
    print("        b = hi;")
    print("    }")
    print("};")
    for live, n in ((9, 16), (25, 32)):
        pairs = batcher(n, live)
        check(pairs, live)
        print()
        print(f"// Sorts k[0..{live - 1}] ascending ({len(pairs)} comparators).")
        print("template <class CE = CeU32>")
        print(f"__device__ __forceinline__ void sortnet{live}(uint32_t (&k)[{live}], CE ce = CE())")
        print("{")
        for a, b in pairs:
            print(f"    ce(k[{a}], k[{b}]);")
        print("}")
    print()
    print("}  // namespace enb")


if __name__ == "__main__":
    main()
