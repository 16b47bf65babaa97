// Fingerprints of the device hash table's keys (region, kind, position and
// key bytes), shared by the pileup kernels and the realigner's patch kernel.
#pragma once
#include "rv_internal.h"

namespace rv {

// MurmurHash3 64-bit finalizer (public-domain mixing function)
__device__ __forceinline__ unsigned long long fmix64(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

// h1: the slot fingerprint (never 0), h2: an independent hash for the
// collision check
__device__ inline void key_hashes(int region, int kind, int pos, const char *k, int n, unsigned long long &h1,
                                  unsigned long long &h2) {
    unsigned long long a = fmix64(((unsigned long long)(uint32_t)region << 32) ^ (uint32_t)pos ^
                                  ((unsigned long long)kind << 58) ^ ((unsigned long long)n << 44));
    unsigned long long b = fmix64(a ^ 0x9e3779b97f4a7c15ULL);
    int i = 0;
    while (i < n) {
        unsigned long long w = 0;
        int m = n - i < 8 ? n - i : 8;
        for (int j = 0; j < m; j++) w |= (unsigned long long)(uint8_t)k[i + j] << (8 * j);
        a = fmix64(a ^ w) + 0x632be59bd9b4e019ULL;
        b = fmix64(b + w * 0x94d049bb133111ebULL);
        i += m;
    }
    h1 = a ? a : 1;
    h2 = b;
}

}  // namespace rv
