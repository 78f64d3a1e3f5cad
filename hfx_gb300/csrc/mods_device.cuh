// Variable-modification isoforms on the device (stage e).
//
// Restates, for one (peptide, modification combination, isoform rank):
//   modable-acid counts over [tc, tn)          filter_by_mod.cu:216-230
//   isoform count prod C(D_i, d_i), suffix products  calc_mod_cands.cu:49-66
//   mixed-radix split of the rank              gen_mod_pep.cu:127-157
//   combination unranking (dual-rank shortcut) combinatorics.h:59-134
//   which residues carry the modification      mion_series.cu:244-286
// all in uint32 arithmetic exactly as the reference.
#pragma once
#include <cstdint>
#include "hfx_internal.h"
#include "device_common.cuh"

namespace hfx {

constexpr int kMaxMa = 8;

// C(n <= 42, k <= 11), combinatorics.h:13-57 (values fit in uint32).
struct BinomTable {
    uint32_t v[43][12];
    constexpr BinomTable() : v() {
        for (int n = 0; n < 43; ++n)
            for (int k = 0; k < 12; ++k)
                v[n][k] = (k > n) ? 0u : (k == 0 || k == n) ? 1u : v[n - 1][k - 1] + v[n - 1][k];
    }
};
__constant__ const BinomTable kBinom = BinomTable();

// combinatorics.h:59-88 (the loop form outside the table, uint32 wrap-around).
__device__ __forceinline__ uint32_t choose_dev(uint32_t n, uint32_t k) {
    if (n <= 42 && k <= 11) return kBinom.v[n][k];
    if (k == 0 || n == k) return 1u;
    if (n < k) return 0u;
    uint32_t t = 1u;
    if (k < n - k) {
        for (uint32_t i = n; i >= n - k + 1; --i) t = t * i / (n - i + 1);
    } else {
        for (uint32_t i = n; i >= k + 1; --i) t = t * i / (n - i + 1);
    }
    return t;
}

// combinatorics.h:90-134: the k indices of combination `rank` of n, as a bit
// mask.  Returns false if an index does not fit in 64 bits.
__device__ __forceinline__ bool unrank_comb_mask(uint32_t n, uint32_t k, uint32_t rank, uint64_t &mask) {
    mask = 0ull;
    uint32_t a = n, b = k;
    const uint32_t total = choose_dev(n, k);
    uint32_t x;
    bool dual = false;
    if ((total / 2u) >= rank) x = rank;
    else { x = total - 1u - rank; dual = true; }
    bool ok = true;
    for (uint32_t i = 0; i < k; ++i) {
        uint32_t v = a - 1u;
        for (int guard = 0; guard < 256 && choose_dev(v, b) > x; ++guard) --v;
        x = x - choose_dev(v, b);
        a = v;
        b = b - 1u;
        const uint32_t ans = dual ? (n - 1u) - v : v;
        if (ans < 64u) mask |= 1ull << ans;
        else ok = false;
    }
    return ok;
}

// Modable-acid counts of the residues [tc, tn) (warp-cooperative; result
// identical in every lane).  The packed residue's mod field (utils.h:97)
// names the acid.
__device__ __forceinline__ void modable_counts(const uint8_t *__restrict__ ions, uint32_t tc, uint32_t tn,
                                               int num_ma, uint32_t (&D)[kMaxMa]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < kMaxMa; ++i) D[i] = 0u;
    for (uint32_t base = tc; base < tn; base += 32) {
        const uint32_t j = base + lane;
        const uint32_t t = (j < tn) ? ((uint32_t)__ldg(ions + j) >> 5) & 7u : 0u;
#pragma unroll
        for (int i = 0; i < kMaxMa; ++i)
            if (i < num_ma) D[i] += __popc(__ballot_sync(kFullMask, t == (uint32_t)(i + 1)));
    }
}

// Isoform count and suffix products (calc_mod_cands.cu:49-66).
__device__ __forceinline__ uint32_t isoform_count(const uint32_t (&D)[kMaxMa], const int32_t *__restrict__ dcount,
                                                  int num_ma, uint32_t (&scan)[kMaxMa]) {
    // fully unrolled over the acid slots so that D and scan stay in registers
    uint32_t num = 1u;
#pragma unroll
    for (int i = kMaxMa - 1; i >= 0; --i) {
        if (i < num_ma) {
            num *= choose_dev(D[i], (uint32_t)dcount[i]);
            scan[i] = num;
        } else {
            scan[i] = 1u;
        }
    }
    return num;
}

// The residues that carry the modification in isoform `rank`: per acid a
// bit mask of the selected occurrence indices (gen_mod_pep.cu:127-227).
__device__ __forceinline__ bool isoform_masks(const uint32_t (&D)[kMaxMa], const uint32_t (&scan)[kMaxMa],
                                              const int32_t *__restrict__ dcount, int num_ma, uint32_t rank,
                                              uint64_t (&mask)[kMaxMa]) {
    uint32_t x = rank;
    bool ok = true;
#pragma unroll
    for (int i = 0; i < kMaxMa; ++i) {
        mask[i] = 0ull;
        if (i >= num_ma) continue;
        uint32_t r;
        if (i != num_ma - 1) {
            const uint32_t nx = scan[i + 1];
            if (x >= nx) { r = x / nx; x = x % nx; }
            else r = 0u;
        } else {
            r = x;
        }
        if (dcount[i] != 0) ok &= unrank_comb_mask(D[i], (uint32_t)dcount[i], r, mask[i]);
    }
    return ok;
}

// Residue-mass hook for build_planes: adds the acid's modification mass to
// the residues the isoform modifies.  The i-th-acid counter is the
// reference kernel's (every modable residue counts, mion_series.cu:252-269)
// unless per_type (the serial checker's per-acid counter,
// check_series.cu:62-100).
struct ModIsoform {
    uint64_t mask[kMaxMa];
    float ma_mass[kMaxMa];
    int num_ma;
    int per_type;
    uint32_t seen_any;
    uint32_t seen[kMaxMa];

    __device__ __forceinline__ void reset() {
        seen_any = 0u;
#pragma unroll
        for (int i = 0; i < kMaxMa; ++i) seen[i] = 0u;
    }

    __device__ __forceinline__ float chunk_add(uint32_t byte, bool valid) {
        const int lane = threadIdx.x & 31;
        const uint32_t lt = (1u << lane) - 1u;
        const uint32_t t = valid ? (byte >> 5) & 7u : 0u;
        const uint32_t any = __ballot_sync(kFullMask, t != 0u);
        uint32_t k = seen_any + __popc(any & lt);
        seen_any += __popc(any);
        uint32_t mytype_seen = 0;
        uint64_t m = 0ull;
        float add = 0.0f;
#pragma unroll
        for (int i = 0; i < kMaxMa; ++i) {
            if (i >= num_ma) continue;
            const uint32_t bi = __ballot_sync(kFullMask, t == (uint32_t)(i + 1));
            if (t == (uint32_t)(i + 1)) {
                mytype_seen = seen[i] + __popc(bi & lt);
                m = mask[i];
                add = ma_mass[i];
            }
            seen[i] += __popc(bi);
        }
        if (per_type) k = mytype_seen;
        if (t == 0u || (int)t > num_ma) return 0.0f;
        const bool modded = k < 64u && ((m >> k) & 1ull);
        return modded ? add : 0.0f;
    }
};

// Residue-mass hook for build_planes over an isoform's modified residues
// (one bit per residue in 32-residue words, as k_iso_positions writes them;
// the same decision as ModIsoform::chunk_add): lane i of ma_lane holds acid
// i+1's modification mass.  Passed by value, so every build starts at the
// first 32-residue chunk.
struct ModPositions {
    const uint32_t *bits;
    float ma_lane;
    uint32_t c;

    __device__ __forceinline__ float chunk_add(uint32_t byte, bool valid) {
        const int lane = threadIdx.x & 31;
        const uint32_t w = bits[c++];
        const uint32_t t = (byte >> 5) & 7u;
        const float add = __shfl_sync(kFullMask, ma_lane, (int)((t + 7u) & 7u));
        return valid && ((w >> lane) & 1u) ? add : 0.0f;
    }
};

// Ordering key of a modified match (Search.hs:119-123 over the reference's
// enumeration order: combination, mass-order position, isoform rank).
__device__ __forceinline__ uint64_t mod_key(int mod, uint32_t pos, uint32_t rank) {
    return (1ull << 63) | ((uint64_t)mod << 54) | ((uint64_t)pos << 27) | (uint64_t)rank;
}

}  // namespace hfx
