// List-based batched scoring (the default batched path for unmodified
// candidates).
//
// Within one search step every candidate peptide is scored against many
// spectra (the +-tolerance windows of neighbouring spectra overlap).  So the
// step first builds, ONCE per (peptide, ion-charge level) that some spectrum
// of the batch needs, the ascending list of distinct ion bins with their
// intensity levels (ion_series.cu:78-123 with the max-dedupe of
// ion_series.cu:71-75), and stores it in HBM.  The scorer then streams a
// candidate's list -- entry i read by lane i % 32, which is exactly the
// canonical accumulation order -- and gathers the group tile in shared
// memory.  Nothing is reused across steps: the lists are rebuilt by every
// search.
//
// Which (peptide, level) pairs are needed: every spectrum adds its window
// [begin, end) to a difference array of its level; a prefix sum marks the
// covered peptides.
#include "hfx_internal.h"
#include "device_common.cuh"
#include "batched.h"
#include "lists.h"
#include "lists_device.cuh"
#include <algorithm>
#include <type_traits>
#include "batched_common.cuh"

namespace hfx {

constexpr int kScanTile = 4096;

// ---- multi-block inclusive scan of int32 (reduce, scan partials, apply) ----
__global__ void k_scan_reduce(const int32_t *__restrict__ a, int64_t n, int32_t *__restrict__ partial) {
    __shared__ int32_t red[32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int32_t s = 0;
    for (int i = threadIdx.x; i < kScanTile; i += blockDim.x)
        if (base + i < n) s += a[base + i];
    s = __reduce_add_sync(kFullMask, s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        int32_t v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0;
        v = __reduce_add_sync(kFullMask, v);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

__global__ void k_scan_partials(int32_t *__restrict__ partial, int32_t nb) {
    // single CTA, exclusive scan in place
    __shared__ int32_t ws[32];
    __shared__ int32_t carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int32_t b0 = 0; b0 < nb; b0 += blockDim.x) {
        const int32_t i = b0 + threadIdx.x;
        const int32_t v = i < nb ? partial[i] : 0;
        const int32_t x = warp_incl_scan(v);
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int32_t w = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
            w = warp_incl_scan(w);
            ws[lane] = w;
        }
        __syncthreads();
        const int32_t before = carry + (warp ? ws[warp - 1] : 0);
        if (i < nb) partial[i] = before + x - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + x;
        __syncthreads();
    }
}

// Inclusive scan of one tile with its block offset: out[i] = sum a[0..i].
__global__ void k_scan_apply(const int32_t *__restrict__ a, int64_t n, const int32_t *__restrict__ partial,
                             int32_t *__restrict__ out) {
    __shared__ int32_t ws[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    const int per = kScanTile / blockDim.x;  // consecutive elements per thread
    int32_t loc[16];
    int32_t s = 0;
    for (int k = 0; k < per; ++k) {
        const int64_t i = base + (int64_t)threadIdx.x * per + k;
        loc[k] = i < n ? a[i] : 0;
        s += loc[k];
    }
    const int32_t x = warp_incl_scan(s);
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int32_t w = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0;
        w = warp_incl_scan(w);
        ws[lane] = w;
    }
    __syncthreads();
    int32_t run = partial[blockIdx.x] + (warp ? ws[warp - 1] : 0) + x - s;
    for (int k = 0; k < per; ++k) {
        const int64_t i = base + (int64_t)threadIdx.x * per + k;
        run += loc[k];
        if (i < n) out[i] = run;
    }
}

// ---- which (peptide, level) lists the batch needs ----
__global__ void k_mark_levels(const SpecMeta *__restrict__ meta, const uint32_t *__restrict__ wb,
                              const uint32_t *__restrict__ we, int32_t nspec, int64_t npep1,
                              int32_t *__restrict__ diff) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nspec) return;
    const SpecMeta m = meta[s];
    const int z = m.charges_plain;
    if (m.status != 0 || z < 1 || z > kLevels || we[s] <= wb[s]) return;
    atomicAdd(&diff[(int64_t)(z - 1) * npep1 + wb[s]], 1);
    atomicAdd(&diff[(int64_t)(z - 1) * npep1 + we[s]], -1);
}


// One warp per candidate peptide: for every charge level some spectrum of
// the batch needs, the sorted distinct-bin list, built incrementally (the
// level-z planes are the level-(z-1) planes plus the charge-z ions).
template <bool FastDiv>
__global__ void __launch_bounds__(256) k_gen_lists(DevDB db, const int32_t *__restrict__ cover, int64_t npep1,
                                                   int32_t nbins, const uint32_t *__restrict__ lstart,
                                                   uint64_t total10, uint16_t *__restrict__ lists,
                                                   uint16_t *__restrict__ list_len, int32_t list_cap,
                                                   unsigned long long *__restrict__ stats,
                                                   uint32_t *__restrict__ err) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int32_t words = (nbins + 31) / 32;
    uint32_t *planes = reinterpret_cast<uint32_t *>(smem) + (size_t)warp * 3 * words;
    uint16_t *list = reinterpret_cast<uint16_t *>(reinterpret_cast<uint32_t *>(smem) + (size_t)nw * 3 * words) +
                     (size_t)warp * list_cap;
    __shared__ unsigned long long s_stats[3];
    if (threadIdx.x < 3) s_stats[threadIdx.x] = 0ull;
    for (int32_t i = lane; i < 3 * words; i += 32) planes[i] = 0u;
    __syncthreads();
    const Planes pl{planes, planes + words, planes + 2 * words};
    const float mt_lane = db.mt[lane];
    unsigned long long my_lists = 0, my_entries = 0, my_res = 0;
    for (int64_t t = (int64_t)blockIdx.x * nw + warp; t < (int64_t)db.num_pep; t += (int64_t)gridDim.x * nw) {
        const uint32_t p = (uint32_t)t;
        uint32_t need = 0;
        if (lane < kLevels && cover[(int64_t)lane * npep1 + p] > 0) need = 1u;
        need = __ballot_sync(kFullMask, need) & ((1u << kLevels) - 1u);
        if (lane < kLevels && !((need >> lane) & 1u)) list_len[(size_t)lane * db.num_pep + p] = 0;
        if (!need) continue;
        const int zmax = 32 - __clz(need);
        const uint32_t tc = db.tc_sorted[p], tn = db.tn_sorted[p];
        const float r = db.r_sorted[p];
        my_res += tn > tc ? tn - tc : 0u;
        WordRange all{0x7FFFFFFF, 0};
        // the level-z list from the planes, when some spectrum needs it
        auto emit_level = [&](int z) {
            if (!((need >> (z - 1)) & 1u)) return;
            const WordRange use = all.hi > all.lo ? all : WordRange{0, 0};
            const uint64_t off = list_offset(lstart, total10, z, p);
            const int room = (int)((lstart[p + 1] - lstart[p]) * (uint32_t)z);  // the slot, >= 10 (tn - tc) z
            int n = compact_planes(pl, use, z == zmax, list, list_cap, lists + off, room);
            if (n > room) {
                if (lane == 0) atomicOr(err, kErrListOverflow);
                n = room;
            }
            if (n <= list_cap) {
                // 16-byte copies: the slot and the staging list start on
                // 16-byte boundaries and hold n rounded up to 8 entries
                const uint4 *src = reinterpret_cast<const uint4 *>(list);
                uint4 *dst = reinterpret_cast<uint4 *>(lists + off);
                for (int i = lane; i < ((n + 7) >> 3); i += 32) dst[i] = src[i];
            }
            if (lane == 0) list_len[(size_t)(z - 1) * db.num_pep + p] = (uint16_t)n;
            my_lists += 1;
            my_entries += (unsigned long long)n;
            __syncwarp();
        };
        auto widen = [&](WordRange wr) {
            if (wr.hi > wr.lo) {
                all.lo = min(all.lo, wr.lo);
                all.hi = max(all.hi, wr.hi);
            }
        };
        for (int z = 1; z <= zmax; ++z) {
            widen(build_planes_range<FastDiv>(pl, db.ions, tc, tn, r, z, z, nbins, mt_lane, NoMods{}));
            emit_level(z);
        }
    }
    if (stats) {
        if (lane == 0) {
            atomicAdd(&s_stats[0], my_lists);
            atomicAdd(&s_stats[1], my_entries);
            atomicAdd(&s_stats[2], my_res);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            atomicAdd(&stats[0], s_stats[0]);
            atomicAdd(&stats[1], s_stats[1]);
            atomicAdd(&stats[6], s_stats[2]);
        }
    }
}

// ---- long rows: 32-bit list entries built by sorting ----
//
// With ~10^5 bins per row the three bit planes no longer fit in shared
// memory.  Instead, for every needed (peptide, level z) the warp writes the
// ten keys (bin << 2 | level) of every (prefix, charge 1..z) into a per-warp
// buffer (ion_series.cu:78-123, the same arithmetic as emit_ions), sorts the
// buffer, and keeps the last key of each bin, i.e. its highest level -- the
// reference's atomicMax into the dense row (ion_series.cu:71-75).
constexpr int kLongKeys = 4096;  // keys per warp: 32-prefix chunks x charges x 10

// rint(mz / width): the mono width as in bin_of, or a custom ion width
// (ibw > 0, the 0.02 Da switch) by IEEE division (__fdividef with FastDiv).
template <bool FastDiv>
__device__ __forceinline__ int32_t bin_w(float mz, float ibw) {
    if (ibw > 0.0f) return sat_bin(rintf(FastDiv ? __fdividef(mz, ibw) : __fdiv_rn(mz, ibw)));
    return bin_of<FastDiv>(mz);
}

template <bool FastDiv>
__device__ __forceinline__ void emit_keys(float b, float y, const ChargeConst &k, int32_t nbins, float ibw,
                                          uint32_t *out) {
    auto key = [&](int32_t x, uint32_t lvl) -> uint32_t {
        return (x >= 0 && x < nbins) ? (((uint32_t)x << 2) | lvl) : 0xFFFFFFFFu;
    };
    // A ion
    out[0] = key(bin_w<FastDiv>(div_charge<FastDiv>(__fadd_rn(__fsub_rn(b, kCO), k.hc), k.c), ibw), 1u);
    // B ions: x-1, x, x+1 at 25/50/25, and the water and ammonia losses at 10
    float m = div_charge<FastDiv>(__fadd_rn(b, k.hc), k.c);
    int32_t x = bin_w<FastDiv>(m, ibw);
    out[1] = key(x - 1, 2u);
    out[2] = key(x, 3u);
    out[3] = key(x + 1, 2u);
    out[4] = key(bin_w<FastDiv>(__fsub_rn(m, k.dh2o), ibw), 1u);
    out[5] = key(bin_w<FastDiv>(__fsub_rn(m, k.dnh3), ibw), 1u);
    // Y ions
    m = div_charge<FastDiv>(__fadd_rn(__fadd_rn(y, kH2O), k.hc), k.c);
    x = bin_w<FastDiv>(m, ibw);
    out[6] = key(x - 1, 2u);
    out[7] = key(x, 3u);
    out[8] = key(x + 1, 2u);
    out[9] = key(bin_w<FastDiv>(__fsub_rn(m, k.dnh3), ibw), 1u);
}

// Warp-wide bitonic sort of n2 (a power of two) keys in shared memory,
// ascending (or descending).
__device__ __forceinline__ void warp_bitonic_sort(uint32_t *kb, int32_t n2, bool descending = false) {
    const int lane = threadIdx.x & 31;
    for (int32_t kk = 2; kk <= n2; kk <<= 1) {
        for (int32_t j = kk >> 1; j > 0; j >>= 1) {
            for (int32_t i = lane; i < n2; i += 32) {
                const int32_t l = i ^ j;
                if (l > i) {
                    const uint32_t a = kb[i], b = kb[l];
                    if ((a > b) == (((i & kk) == 0) != descending)) {
                        kb[i] = b;
                        kb[l] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// Ascending bitonic merge of n2 keys whose first half ascends and second
// half descends.
__device__ __forceinline__ void warp_bitonic_merge(uint32_t *kb, int32_t n2) {
    const int lane = threadIdx.x & 31;
    for (int32_t j = n2 >> 1; j > 0; j >>= 1) {
        for (int32_t i = lane; i < n2; i += 32) {
            const int32_t l = i ^ j;
            if (l > i) {
                const uint32_t a = kb[i], b = kb[l];
                if (a > b) {
                    kb[i] = b;
                    kb[l] = a;
                }
            }
        }
        __syncwarp();
    }
}

// Keeps the last key of each bin (its highest level) of the ascending keys
// kb[0, n2), packed in order at kb[0, n) (in place: a round reads its keys
// before it writes, and writes only at or below them), and, when out is
// given, at out[0, min(n, cap)).  Returns n.
__device__ __forceinline__ int32_t warp_keep_highest(uint32_t *kb, int32_t n2, uint32_t *out, int32_t cap) {
    const int lane = threadIdx.x & 31;
    int32_t n = 0;
    for (int32_t i0 = 0; i0 < n2; i0 += 32) {
        const int32_t i = i0 + lane;
        const uint32_t k = i < n2 ? kb[i] : 0xFFFFFFFFu;
        const bool keep = k != 0xFFFFFFFFu && (i + 1 >= n2 || (kb[i + 1] >> 2) != (k >> 2));
        const uint32_t bal = __ballot_sync(kFullMask, keep);
        const int32_t at = n + __popc(bal & ((1u << lane) - 1u));
        if (keep) {
            kb[at] = k;
            if (out && at < cap) out[at] = k;
        }
        n += __popc(bal);
    }
    __syncwarp();
    return n;
}

template <bool FastDiv>
__global__ void __launch_bounds__(256) k_gen_lists_long(DevDB db, const int32_t *__restrict__ cover, int64_t npep1,
                                                        int32_t nbins, const uint32_t *__restrict__ lstart,
                                                        uint64_t total10, uint32_t *__restrict__ lists,
                                                        uint16_t *__restrict__ list_len, float ibw,
                                                        unsigned long long *__restrict__ stats,
                                                        uint32_t *__restrict__ err) {
    extern __shared__ __align__(16) uint32_t keybuf[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t *kb = keybuf + (size_t)warp * kLongKeys;
    __shared__ unsigned long long s_stats[3];
    if (threadIdx.x < 3) s_stats[threadIdx.x] = 0ull;
    __syncthreads();
    const float mt_lane = db.mt[lane];
    uint32_t my_lists = 0, my_entries = 0, my_res = 0;
    for (int64_t t = (int64_t)blockIdx.x * nw + warp; t < (int64_t)db.num_pep; t += (int64_t)gridDim.x * nw) {
        const uint32_t p = (uint32_t)t;
        uint32_t need = 0;
        if (lane < kLevels && cover[(int64_t)lane * npep1 + p] > 0) need = 1u;
        need = __ballot_sync(kFullMask, need) & ((1u << kLevels) - 1u);
        if (lane < kLevels && !((need >> lane) & 1u)) list_len[(size_t)lane * db.num_pep + p] = 0;
        if (!need) continue;
        const int zmax = 32 - __clz(need);
        const uint32_t tc = db.tc_sorted[p], tn = db.tn_sorted[p];
        const float r = db.r_sorted[p];
        my_res += tn > tc ? tn - tc : 0u;
        const uint32_t nchunk = (tn - tc + 31u) / 32u;
        // keys of (prefix k, charge c) at 10 (k z + c - 1), padded to a power of two
        uint32_t nmax = 32u;
        while (tn >= tc && nmax < (tn - tc) * (uint32_t)zmax * 10u) nmax <<= 1;
        if (tn < tc || nmax > (uint32_t)kLongKeys) {
            if (lane == 0) atomicOr(err, kErrTooLong);
            if (lane < kLevels && ((need >> lane) & 1u)) list_len[(size_t)lane * db.num_pep + p] = 0;
            continue;
        }
        // Incremental levels where they fit: the level-z list is the
        // level-(z-1) list (ascending, in the lower half) merged with the
        // sorted charge-z keys (descending, in the upper half) by one bitonic
        // merge, then reduced to each bin's highest level -- the same list as
        // sorting every charge <= z at once, with a tenth of the
        // compare-exchanges.  A peptide whose lists outgrow half the buffer
        // takes the full sort below.
        const int32_t nk = 10 * (int32_t)(tn - tc);  // keys of one charge
        int32_t hmax = 32;
        while (hmax < max(nk, nk * (zmax - 1))) hmax <<= 1;
        if (2 * hmax <= kLongKeys) {
            int32_t n_prev = 0;
            for (int z = 1; z <= zmax; ++z) {
                int32_t h = 32;
                while (h < max(nk, n_prev)) h <<= 1;
                const int32_t lo = z == 1 ? 0 : h;  // where the charge-z keys go
                const int32_t n2 = z == 1 ? h : 2 * h;
                for (int32_t i = n_prev + lane; i < n2; i += 32) kb[i] = 0xFFFFFFFFu;
                __syncwarp();
                float carry = 0.0f;
                for (uint32_t ci = 0; ci < nchunk; ++ci) {
                    const uint32_t base = tc + 32u * ci;
                    const int cnt = (int)min(32u, tn - base);
                    uint32_t byte = 0;
                    if (lane < cnt) byte = __ldg(db.ions + base + lane);
                    float v = residue_mass(mt_lane, byte);
                    if (lane >= cnt) v = 0.0f;
                    if (lane == 0) v = __fadd_rn(v, carry);
#pragma unroll
                    for (int d = 1; d < 32; d <<= 1) {
                        const float u = __shfl_up_sync(kFullMask, v, d);
                        if (lane >= d) v = __fadd_rn(v, u);
                    }
                    carry = __shfl_sync(kFullMask, v, cnt - 1);
                    if (lane < cnt)
                        emit_keys<FastDiv>(v, __fsub_rn(r, v), charge_const<FastDiv>(z), nbins, ibw,
                                           kb + lo + (size_t)(32u * ci + (uint32_t)lane) * 10);
                }
                __syncwarp();
                if (z == 1) {
                    warp_bitonic_sort(kb, n2);
                } else {
                    warp_bitonic_sort(kb + h, h, true);
                    warp_bitonic_merge(kb, n2);
                }
                const bool needed = (need >> (z - 1)) & 1u;
                const int32_t slot = 10 * z * (int32_t)(tn - tc);
                int32_t n = warp_keep_highest(kb, n2, needed ? lists + list_offset(lstart, total10, z, p) : nullptr,
                                              slot);
                n_prev = n;
                if (!needed) continue;
                if (n > slot) {
                    if (lane == 0) atomicOr(err, kErrListOverflow);
                    n = slot;
                }
                if (lane == 0) list_len[(size_t)(z - 1) * db.num_pep + p] = (uint16_t)min(n, 65535);
                my_lists += 1u;
                my_entries += (uint32_t)n;
                __syncwarp();
            }
            continue;
        }
        for (int z = 1; z <= zmax; ++z) {
            if (!((need >> (z - 1)) & 1u)) continue;
            const int32_t nslot = (int32_t)(tn - tc) * z * 10;
            int32_t n2 = 32;
            while (n2 < nslot) n2 <<= 1;
            for (int32_t i = lane; i < n2; i += 32) kb[i] = 0xFFFFFFFFu;
            __syncwarp();
            // the b-ladder: the reference warp scan per 32-residue chunk
            float carry = 0.0f;
            for (uint32_t ci = 0; ci < nchunk; ++ci) {
                const uint32_t base = tc + 32u * ci;
                const int cnt = (int)min(32u, tn - base);
                uint32_t byte = 0;
                if (lane < cnt) byte = __ldg(db.ions + base + lane);
                float v = residue_mass(mt_lane, byte);
                if (lane >= cnt) v = 0.0f;
                if (lane == 0) v = __fadd_rn(v, carry);
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const float u = __shfl_up_sync(kFullMask, v, d);
                    if (lane >= d) v = __fadd_rn(v, u);
                }
                carry = __shfl_sync(kFullMask, v, cnt - 1);
                if (lane < cnt) {
                    const float y = __fsub_rn(r, v);
                    const uint32_t k = 32u * ci + (uint32_t)lane;
                    for (int c = 1; c <= z; ++c)
                        emit_keys<FastDiv>(v, y, charge_const<FastDiv>(c), nbins, ibw,
                                           kb + ((size_t)k * z + (c - 1)) * 10);
                }
            }
            __syncwarp();
            warp_bitonic_sort(kb, n2);
            // keep the last key of each bin (its highest level), in order
            const uint64_t off = list_offset(lstart, total10, z, p);
            const int32_t slot = 10 * z * (int32_t)(tn - tc);
            int32_t n = 0;
            for (int32_t i0 = 0; i0 < n2; i0 += 32) {
                const int32_t i = i0 + lane;
                const uint32_t k = kb[i];
                const bool keep = k != 0xFFFFFFFFu && (i + 1 == n2 || (kb[i + 1] >> 2) != (k >> 2));
                const uint32_t bal = __ballot_sync(kFullMask, keep);
                const int32_t at = n + __popc(bal & ((1u << lane) - 1u));
                if (keep && at < slot) lists[off + at] = k;
                n += __popc(bal);
            }
            if (n > slot) {
                if (lane == 0) atomicOr(err, kErrListOverflow);
                n = slot;
            }
            if (lane == 0) list_len[(size_t)(z - 1) * db.num_pep + p] = (uint16_t)min(n, 65535);
            my_lists += 1u;
            my_entries += (uint32_t)n;
            __syncwarp();
        }
    }
    if (stats) {
        if (lane == 0) {
            atomicAdd(&s_stats[0], (unsigned long long)my_lists);
            atomicAdd(&s_stats[1], (unsigned long long)my_entries);
            atomicAdd(&s_stats[2], (unsigned long long)my_res);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            atomicAdd(&stats[0], s_stats[0]);
            atomicAdd(&stats[1], s_stats[1]);
            atomicAdd(&stats[6], s_stats[2]);
        }
    }
}

// FP32 rescoring of kept unmodified candidates from their lists and the
// FP32 row in global memory (long rows), canonical order: entry i by lane
// i % 32, XOR butterfly.  One CTA per spectrum.
template <typename E>
__global__ void __launch_bounds__(256) k_rescore_lists(const E *__restrict__ lists,
                                                       const uint32_t *__restrict__ lstart, uint64_t total10,
                                                       const uint16_t *__restrict__ list_len, uint32_t num_pep,
                                                       const uint32_t *__restrict__ idx_sorted,
                                                       const float *__restrict__ rows32, int64_t stride,
                                                       const SpecMeta *__restrict__ meta,
                                                       const uint64_t *__restrict__ kept_k, int32_t K, int32_t topn,
                                                       float *__restrict__ out_s, uint64_t *__restrict__ out_k,
                                                       uint32_t *__restrict__ out_pep, uint32_t *__restrict__ err) {
    __shared__ float res_s[kMaxKept];
    __shared__ uint64_t res_k[kMaxKept];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int32_t s = blockIdx.x;
    const SpecMeta m = meta[s];
    const float *row = rows32 + (size_t)s * stride;
    const int z = m.charges_plain;
    for (int t = warp; t < K; t += nw) {
        const uint64_t kk = kept_k[(size_t)s * K + t];
        float sc = -INFINITY;
        if (kk != ~0ull) {
            float acc = 0.0f;
            if (!(kk >> 63) && z >= 1 && kk < num_pep) {
                const uint32_t p = (uint32_t)kk;
                const int n = list_len[(size_t)(z - 1) * num_pep + p];
                const E *lp = lists + list_offset(lstart, total10, z, p);
                // four entries per lane in flight, then their row values,
                // then the sums in the lane's ascending entry order
                for (int i0 = lane; i0 < n; i0 += 128) {
                    uint32_t e[4];
                    float x[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) e[k] = i0 + 32 * k < n ? (uint32_t)__ldg(lp + i0 + 32 * k) : ~0u;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const uint32_t bin = e[k] >> 2;
                        x[k] = (i0 + 32 * k < n && (int32_t)bin < m.len) ? __ldg(row + bin) : 0.0f;
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k)
                        if (i0 + 32 * k < n && (int32_t)(e[k] >> 2) < m.len)
                            acc = __fmaf_rn(level_weight(e[k] & 3u), x[k], acc);
                }
            } else if (kk >> 63) {
                if (lane == 0) atomicOr(err, kErrBounds);
            }
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(kFullMask, acc, o));
            sc = acc;
        }
        if (lane == 0) {
            res_s[t] = sc;
            res_k[t] = kk;
        }
    }
    __syncthreads();
    if (warp == 0) {
        WarpTopK tk;
        tk.init();
        for (int t = 0; t < K; ++t)
            if (res_k[t] != ~0ull) tk.insert(res_s[t], res_k[t], topn);
        if (lane < topn) {
            out_s[(size_t)s * topn + lane] = tk.s;
            out_k[(size_t)s * topn + lane] = tk.k;
            out_pep[(size_t)s * topn + lane] = (tk.k != ~0ull && tk.k < num_pep) ? idx_sorted[tk.k] : ~0u;
        }
    }
}

// Scorer over precomputed lists: a persistent grid pulls work items (group x
// candidate chunk); the group's interleaved tile is staged by one bulk copy;
// a warp streams each candidate's list (entry i by lane i % 32, four loads
// in flight per lane) and gathers the tile; CTA-wide top-K per member.
// E = list entry type (uint16_t up to 16,383 bins, uint32_t for long rows);
// kGlobal: the group tile is read from global memory (L2) instead of being
// staged in shared memory (rows too long for shared memory).
// kC: candidates per warp (1, 2 or 4), one per group of 32 / kC lanes (entry
// i of a list by lane i % (32 / kC) of its group).  The per-candidate work
// around the list -- the claim, the reduction, the admission -- is then
// shared by kC candidates.  In FP32 with four candidates each lane keeps four
// partial-sum sets (entry k of every round of 32 in set k) and adds them as
// the 32-lane butterfly would, so the sums keep the canonical order; the
// BF16/FP16 pass sums in one set (its scores only pick the candidates that
// FP32 rescoring orders).
template <typename T, int G, typename E, bool kGlobal, int kC, int L>
__global__ void __launch_bounds__(1024, 1)
k_score_lists(const E *__restrict__ lists, const uint32_t *__restrict__ lstart, uint64_t total10,
              uint64_t list_total, const uint16_t *__restrict__ list_len, uint32_t num_pep,
              const T *__restrict__ tiles, int64_t stride,
              const uint32_t *__restrict__ wb, const uint32_t *__restrict__ we, const int32_t *__restrict__ perm,
              const GroupInfo *__restrict__ groups, const uint32_t *__restrict__ item_off,
              const uint32_t *__restrict__ ngroups_p, int32_t K, uint32_t *__restrict__ counter,
              float *__restrict__ part_s, uint64_t *__restrict__ part_k, unsigned long long *__restrict__ stats,
              float *__restrict__ sink, const uint64_t *__restrict__ sink_off, uint32_t qoff,
              uint32_t *__restrict__ err) {
    static_assert(kC == 1 || kC == 2 || kC == 4, "1, 2 or 4 candidates per warp");
    constexpr int kW = 32 / kC;  // lanes per candidate
    // FP32 with several candidates per warp: four partial-sum sets per lane
    constexpr bool kSets4 = std::is_same<T, float>::value && kC > 1;
    static_assert(!kSets4 || kW == 8, "the FP32 partial-sum sets assume 8 lanes per candidate");
    static_assert(G <= kW, "a lane group takes up to one spectrum of the group per lane");
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int hl = lane & (kW - 1), half = lane / kW;  // `half`: the lane's candidate group
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    T *stile = reinterpret_cast<T *>(smem + 128);
    const T *tile = stile;
    __shared__ int32_t s_item;
    __shared__ uint32_t s_next;
    __shared__ uint32_t s_wb[G], s_we[G];
    __shared__ uint64_t s_off[G];  // with a sink: where each member's window starts in it
    __shared__ uint32_t thr_u[G], s_lock[G];
    __shared__ float s_ls[G * L];
    __shared__ uint32_t s_lk[G * L];
    __shared__ unsigned long long s_stats[5];

    const int32_t ngroups = (int32_t)*ngroups_p;
    const uint32_t total = item_off[ngroups];
    if (threadIdx.x == 0) mbar_init(bar, 1);
    if (threadIdx.x < 5) s_stats[threadIdx.x] = 0ull;
    __syncthreads();
    const int my_slot = reduce_slot_of_lane<G>(lane);
    uint32_t my_cand = 0, my_entries = 0, my_psm = 0, my_claims = 0;
    uint32_t phase = 0;
    CtaSlots<G, uint32_t, cta_queue_len(G), L> slots;
    slots.bind(s_ls, s_lk, s_lock, thr_u, smem + qoff + (size_t)warp * CtaSlots<G>::warp_bytes(), err);
    while (true) {
        if (threadIdx.x == 0) s_item = (int32_t)atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t item = (uint32_t)s_item;
        if (item >= total) break;
        const int32_t g = find_group(item_off, ngroups, item);
        const GroupInfo gi = groups[g];
        const uint32_t p0 = gi.lo + (item - item_off[g]) * gi.chunk;
        const uint32_t p1 = min(gi.hi, p0 + gi.chunk);
        const int cnt_members = (int)gi.count;
        if (threadIdx.x < G) {
            const int j = threadIdx.x;
            uint32_t b = 0, e = 0;
            uint64_t o = 0;
            if (j < cnt_members) {
                const int32_t s = perm[gi.pos0 + j];
                b = wb[s];
                e = we[s];
                if (sink) o = sink_off[s];
            }
            s_off[j] = o;
            s_wb[j] = b;
            s_we[j] = e;
        }
        slots.reset_shared();
        const int32_t nb = tile_bins(gi.maxlen);
        if (threadIdx.x == 0) {
            s_next = p0;
            my_claims += p1 - p0;
            if (stats && !kGlobal) s_stats[4] += (unsigned long long)nb * G * sizeof(T);
        }
        if constexpr (kGlobal) {
            tile = tiles + (size_t)g * stride * G;
            __syncthreads();
        } else {
            if (threadIdx.x == 0) {
                fence_proxy_async();
                const uint32_t bytes = (uint32_t)((size_t)nb * G * sizeof(T));
                mbar_arrive_expect_tx(bar, bytes);
                bulk_g2s(stile, tiles + (size_t)g * stride * G, bytes, bar);
            }
            // bins [nb, stride + 8) of the shared tile read as zero: every
            // list bin (< stride) and the pad entry (bin = stride) may be
            // gathered without a bounds test
            {
                uint4 *z = reinterpret_cast<uint4 *>(stile);
                const size_t z0 = (size_t)nb * G * sizeof(T) / 16, z1 = (size_t)(stride + 8) * G * sizeof(T) / 16;
                for (size_t i = z0 + threadIdx.x; i < z1; i += blockDim.x) z[i] = make_uint4(0u, 0u, 0u, 0u);
                fence_proxy_async();  // before a later item's bulk copy overwrites these bytes
            }
            __syncthreads();
            if (!mbar_wait(bar, phase, kWaitLimit)) {
                if (threadIdx.x == 0) atomicOr(err, kErrTimeout);
                return;
            }
            phase ^= 1u;
        }
        // member hl's window, in each half
        const uint32_t my_b = hl < G ? s_wb[hl] : 0u, my_e = hl < G ? s_we[hl] : 0u;
        // entry past a list's end: the zero bin `stride` of the shared tile
        // (beyond every group's bins, so it also ends the scan), or an
        // out-of-range bin for tiles in global memory
        const uint32_t pad = kGlobal ? 0xFFFFFFFFu : ((uint32_t)stride << 2);
        const int z = (int)gi.charges;
        const uint16_t *llen = list_len + (size_t)(z >= 1 ? z - 1 : 0) * num_pep;
        // Three-stage software pipeline over the warp's candidates: while
        // candidate i is scored, candidate i+1's first list entries are in
        // flight and candidate i+2 is claimed with its list length and
        // offset loads in flight, so no stage waits on a dependent load.
        // Per lane: its half's candidate; `live` (warp-uniform) while any
        // candidate was claimed.
        struct Meta {
            uint32_t p, act, n, ls;
            bool live;
        };
        struct Cand {
            uint32_t p, act;
            int n;
            bool live;
            const E *lp;
            uint32_t e[4];
        };
        auto claim = [&]() {
            Meta m;
            m.act = 0u;
            m.n = 0u;
            m.ls = 0u;
            while (true) {
                uint32_t q = 0;
                if (lane == 0) q = atomicAdd(&s_next, (uint32_t)kC);
                const uint32_t base = __shfl_sync(kFullMask, q, 0);
                m.live = base < p1;
                m.p = base + (uint32_t)half;
                if (!m.live) break;
                const uint32_t bal =
                    __ballot_sync(kFullMask, hl < G && m.p < p1 && my_b <= m.p && m.p < my_e);
                m.act = (bal >> (kW * half)) & ((1u << G) - 1u);
                if (bal) break;
            }
            if (m.act && z >= 1 && m.p < num_pep) {
                m.n = llen[m.p];
                m.ls = lstart[m.p];
            }
            return m;
        };
        auto issue = [&](const Meta &m) {
            Cand c;
            c.p = m.p;
            c.act = m.act;
            c.n = (int)m.n;
            c.live = m.live;
            c.lp = lists;
            if (m.act && z >= 1) {
                const uint64_t off = total10 * (uint64_t)(z * (z - 1) / 2) + (uint64_t)z * m.ls;
                if (m.p >= num_pep || off + (uint64_t)c.n > list_total) {
                    if (hl == 0) atomicOr(err, kErrBounds);
                    c.n = 0;
                } else {
                    c.lp = lists + off;
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int i = kW * k + hl;
                c.e[k] = i < c.n ? (uint32_t)__ldg(c.lp + i) : pad;
            }
            return c;
        };
        Meta ahead = claim();
        Cand nxt = issue(ahead);
        if (nxt.live) ahead = claim();
        while (nxt.live) {
            const Cand cur = nxt;
            nxt = issue(ahead);
            if (nxt.live) ahead = claim();
            float acc[G];
#pragma unroll
            for (int j = 0; j < G; ++j) acc[j] = 0.0f;
            // FP32 with four candidates per warp keeps the canonical order:
            // entry i of a list goes to partial sum i % 32, and with 8 lanes
            // per candidate entry k of each round of 32 is partial 8 k + lane,
            // so each lane keeps four partial-sum sets and adds them as the
            // 32-lane butterfly's offsets 16 and 8 do
            float acc4[kSets4 ? 4 : 1][G];
#pragma unroll
            for (int k = 0; k < (kSets4 ? 4 : 1); ++k)
#pragma unroll
                for (int j = 0; j < G; ++j) acc4[k][j] = 0.0f;
            const int n = cur.n;
            int nmax = n;
#pragma unroll
            for (int o = kW; o < 32; o <<= 1) nmax = max(nmax, __shfl_xor_sync(kFullMask, nmax, o));
            // entries [i0, i0 + 4 kW) in e, the next 4 kW already in flight in f
            uint32_t e[4], f[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                e[k] = cur.e[k];
                const int i = 4 * kW + kW * k + hl;
                f[k] = i < n ? (uint32_t)__ldg(cur.lp + i) : pad;
            }
            for (int i0 = 0; i0 < nmax; i0 += 4 * kW) {
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t bin = e[k] >> 2;
                    float *a = acc;
                    if constexpr (kSets4) a = acc4[k];
                    if constexpr (kGlobal) {
                        if ((int32_t)bin < nb)
                            TileFma<T, G>::fma(tile, bin, e[k] & 3u, *reinterpret_cast<float(*)[G]>(a));
                    } else {
                        // zero beyond nb
                        TileFma<T, G>::fma(tile, bin, e[k] & 3u, *reinterpret_cast<float(*)[G]>(a));
                    }
                }
                // lists ascend: once an entry lies beyond the tile, so do the rest
                const uint32_t last = __shfl_sync(kFullMask, e[3], (lane & ~(kW - 1)) | (kW - 1));
                if (__all_sync(kFullMask, (last >> 2) >= (uint32_t)nb)) break;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    e[k] = f[k];
                    const int i = i0 + 8 * kW + kW * k + hl;
                    f[k] = i < n ? (uint32_t)__ldg(cur.lp + i) : pad;
                }
            }
            if constexpr (kSets4) {
                // offsets 16 (partials l and l + 16, l + 8 and l + 24) and 8
#pragma unroll
                for (int j = 0; j < G; ++j)
                    acc[j] = __fadd_rn(__fadd_rn(acc4[0][j], acc4[2][j]), __fadd_rn(acc4[1][j], acc4[3][j]));
            }
            if constexpr (kC > 1) {
                const float sc = reduce_scatter_lanes<G, kW>(acc);
                const bool owner = (lane & (32 / G - 1)) == 0;
#pragma unroll
                for (int q = 0; q < kC; ++q) {
                    const uint32_t act_q = __shfl_sync(kFullMask, cur.act, q * kW);
                    const uint32_t p_q = __shfl_sync(kFullMask, cur.p, q * kW);
                    const int n_q = __shfl_sync(kFullMask, n, q * kW);
                    my_cand += act_q != 0u;
                    my_entries += (uint32_t)n_q;
                    my_psm += (uint32_t)__popc(act_q);
                    // member j's sums sit in lanes j * kW / G of candidate q's
                    // group; its admission lane is j * 32 / G
                    const float sc_q = __shfl_sync(kFullMask, sc, q * kW + (lane / (32 / G)) * (kW / G));
                    // every pair's score, at its member's window offset
                    // (E-values; FP32 only, the host refuses a sink otherwise)
                    if constexpr (std::is_same<T, float>::value) {
                        if (sink && owner && ((act_q >> my_slot) & 1u))
                            sink[s_off[my_slot] + (p_q - s_wb[my_slot])] = sc_q;
                    }
                    const bool want = owner && ((act_q >> my_slot) & 1u) &&
                                      score_order(sc_q) >= *(volatile uint32_t *)(thr_u + my_slot);
                    slots.offer(want, sc_q, p_q, my_slot, K);
                }
            } else {
                my_cand += 1u;
                my_entries += (uint32_t)n;
                my_psm += (uint32_t)__popc(cur.act);
                const float sc = reduce_scatter<G>(acc);
                if (sink) {
                    // every pair's score, at its member's window offset (the
                    // admission below still keeps the top-K)
                    if ((lane & (32 / G - 1)) == 0 && ((cur.act >> my_slot) & 1u))
                        sink[s_off[my_slot] + (cur.p - s_wb[my_slot])] = sc;
                }
                const bool want = (lane & (32 / G - 1)) == 0 && ((cur.act >> my_slot) & 1u) &&
                                  score_order(sc) >= *(volatile uint32_t *)(thr_u + my_slot);
                slots.offer(want, sc, cur.p, my_slot, K);
            }
        }
        slots.drain(K);
        __syncthreads();  // every warp has merged its queues
        for (int j = warp; j < cnt_members; j += nw) {
            const size_t o = ((size_t)item * G + j) * K;
            slots.result(j, K, part_s + o, part_k + o);
        }
        __syncthreads();
    }
    if (stats) {
        if (lane == 0) {
            atomicAdd(&s_stats[0], (unsigned long long)my_cand);
            atomicAdd(&s_stats[1], (unsigned long long)my_entries);
            atomicAdd(&s_stats[2], (unsigned long long)my_psm);
            atomicAdd(&s_stats[3], (unsigned long long)my_claims);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            atomicAdd(&stats[2], s_stats[0]);
            atomicAdd(&stats[3], s_stats[1]);
            atomicAdd(&stats[4], s_stats[2]);
            atomicAdd(&stats[5], s_stats[3]);
            atomicAdd(&stats[7], s_stats[4]);
        }
    }
}

}  // namespace hfx

using namespace hfx;

int hfx_scan_inclusive(const int32_t *in, int64_t n, int32_t *out, int32_t *partial, cudaStream_t st) {
    if (n <= 0) return 0;
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    k_scan_reduce<<<(unsigned)nb, 512, 0, st>>>(in, n, partial);
    k_scan_partials<<<1, 1024, 0, st>>>(partial, (int32_t)nb);
    k_scan_apply<<<(unsigned)nb, 256, 0, st>>>(in, n, partial, out);
    return (int)cudaGetLastError();
}

int64_t hfx_scan_partials_needed(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

int hfx_lists_mark(const SpecMeta *meta, const uint32_t *wb, const uint32_t *we, int32_t nspec, int64_t npep1,
                   int32_t *diff, cudaStream_t st) {
    cudaMemsetAsync(diff, 0, sizeof(int32_t) * (size_t)kLevels * npep1, st);
    if (nspec > 0) k_mark_levels<<<(nspec + 255) / 256, 256, 0, st>>>(meta, wb, we, nspec, npep1, diff);
    return (int)cudaGetLastError();
}

int hfx_lists_generate(const DevDB &db, const int32_t *cover, int64_t npep1, int32_t nbins, const uint32_t *lstart,
                       uint64_t total10, uint16_t *lists, uint16_t *list_len, int32_t list_cap, int fastdiv,
                       unsigned long long *stats, uint32_t *err, cudaStream_t st) {
    const int nw = 8;
    const int32_t words = (nbins + 31) / 32;
    // 16-byte staging lists of up to kStageCap entries (longer lists are
    // written directly)
    list_cap = (std::max(32, std::min(list_cap, kStageCap)) + 7) & ~7;
    // per warp: three bit planes and a staging list of list_cap entries
    const size_t smem = (size_t)nw * 3 * words * 4 + (size_t)nw * list_cap * 2;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto f = fastdiv ? k_gen_lists<true> : k_gen_lists<false>;
    cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, nw * 32, smem);
    f<<<sms * (per > 0 ? per : 1), nw * 32, smem, st>>>(db, cover, npep1, nbins, lstart, total10, lists, list_len,
                                                        list_cap, stats, err);
    return (int)cudaGetLastError();
}

// Candidates per warp with groups of up to 8 spectra (FP32 and BF16/FP16).
constexpr int kLowpCands = 4;

// Warps per list-scorer CTA: 16 (two CTAs per SM) up to 8 spectra per
// group, 32 (one CTA per SM, the tile taking most of shared memory) for 16.
constexpr int list_warps(int G) { return G >= 16 ? 32 : 16; }

// Dynamic shared memory of the list scorer: an mbarrier, the group tile
// (none when it is read from global memory), then the warps' queues.
static size_t lists_queue_offset(bool global_tile, int64_t stride, int G, size_t elem_bytes) {
    // the shared tile holds stride + 8 bins: the zero bins after the group's
    // rows and the pad entry's bin
    return 128 + (global_tile ? 0 : (((size_t)(stride + 8) * G * elem_bytes + 15) & ~(size_t)15));
}

template <typename T, int G, typename E, bool kGlobal, int kC, int L>
static int launch_lists_t(const E *lists, const uint32_t *lstart, uint64_t total10, const uint16_t *list_len,
                          uint32_t num_pep, int64_t stride, const uint32_t *wb, const uint32_t *we,
                          const BatchedWs &ws, void *tiles, int32_t K, int nw,
                          float *part_s, uint64_t *part_k, unsigned long long *stats, float *sink,
                          const uint64_t *sink_off, uint32_t *err, cudaStream_t st) {
    int dev = 0, sms = 0, smem_max = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (nw <= 0) nw = list_warps(G);
    const size_t qoff = lists_queue_offset(kGlobal, stride, G, sizeof(T));
    const size_t smem = qoff + (size_t)nw * CtaSlots<G>::warp_bytes();
    if (smem > (size_t)smem_max) return (int)cudaErrorInvalidValue;
    auto fn = k_score_lists<T, G, E, kGlobal, kC, L>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, nw * 32, smem);
    const int grid = sms * (per > 0 ? per : 1);
    cudaMemsetAsync(ws.counter, 0, 4, st);
    fn<<<grid, nw * 32, smem, st>>>(lists, lstart, total10, total10 * 10, list_len, num_pep, (const T *)tiles,
                                    stride, wb, we, ws.perm, ws.groups, ws.item_off, ws.ngroups, K,
                                    ws.counter, part_s, part_k, stats, sink, sink_off, (uint32_t)qoff, err);
    return (int)cudaGetLastError();
}

int hfx_lists_group_fits(int32_t G, int long_rows, int64_t stride, int elem_bytes) {
    if (G != 16) return 1;
    int dev = 0, smem_max = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    const cudaError_t e =
        long_rows ? cudaFuncGetAttributes(&fa, k_score_lists<__nv_bfloat16, 16, uint32_t, true, 1, 32>)
                  : cudaFuncGetAttributes(&fa, k_score_lists<__nv_bfloat16, 16, uint16_t, false, 1, 32>);
    if (e != cudaSuccess) return 0;
    const size_t smem = lists_queue_offset(long_rows != 0, stride, 16, (size_t)elem_bytes) +
                        (size_t)list_warps(16) * CtaSlots<16>::warp_bytes();
    return smem + fa.sharedSizeBytes <= (size_t)smem_max ? 1 : 0;
}

int hfx_lists_score(const void *lists, int long_rows, const uint32_t *lstart, uint64_t total10,
                    const uint16_t *list_len, uint32_t num_pep, int elem_kind, int64_t stride, const uint32_t *wb,
                    const uint32_t *we, const BatchedWs &ws, void *tiles, int32_t G, int32_t K, int nw,
                    float *part_s, uint64_t *part_k, unsigned long long *stats, uint32_t *err, cudaStream_t st,
                    float *sink, const uint64_t *sink_off) {
    // groups of up to 8 spectra score four candidates per warp (FP32 in the
    // canonical order, with or without a sink; BF16/FP16 scores only choose
    // what FP32 rescoring orders)
    if (elem_kind != 0 && sink) return (int)cudaErrorInvalidValue;
    // up to 64 kept candidates per member in the BF16/FP16 pass
    if (K > kMaxKept || (K > 32 && (elem_kind == 0 || G > 8))) return (int)cudaErrorInvalidValue;
#define HFX_LL(T, GG, LL)                                                                                      \
    do {                                                                                                       \
        constexpr int kP = GG > 8 ? 1 : kLowpCands;                                                            \
        if (long_rows)                                                                                         \
            return launch_lists_t<T, GG, uint32_t, true, kP, LL>((const uint32_t *)lists, lstart, total10,     \
                                                                 list_len, num_pep, stride, wb, we, ws, tiles, \
                                                                 K, nw, part_s, part_k, stats, sink, sink_off, \
                                                                 err, st);                                     \
        return launch_lists_t<T, GG, uint16_t, false, kP, LL>((const uint16_t *)lists, lstart, total10,        \
                                                              list_len, num_pep, stride, wb, we, ws, tiles, K, \
                                                              nw, part_s, part_k, stats, sink, sink_off, err,  \
                                                              st);                                             \
    } while (0)
#define HFX_L(T, GG) HFX_LL(T, GG, 32)
#define HFX_L64(T, GG)                 \
    do {                               \
        if (K > 32) HFX_LL(T, GG, 64); \
        HFX_LL(T, GG, 32);             \
    } while (0)
    if (elem_kind == 0) {
        if (G == 4) HFX_L(float, 4);
        if (G == 8) HFX_L(float, 8);
        if (G == 2) HFX_L(float, 2);
        if (G == 1) HFX_L(float, 1);
    } else if (elem_kind == 1) {
        if (G == 8) HFX_L64(__nv_bfloat16, 8);
        if (G == 16) HFX_L(__nv_bfloat16, 16);
        if (G == 4) HFX_L64(__nv_bfloat16, 4);
        if (G == 2) HFX_L64(__nv_bfloat16, 2);
        if (G == 1) HFX_L64(__nv_bfloat16, 1);
    } else {
        if (G == 8) HFX_L64(__half, 8);
        if (G == 16) HFX_L(__half, 16);
        if (G == 4) HFX_L64(__half, 4);
        if (G == 2) HFX_L64(__half, 2);
        if (G == 1) HFX_L64(__half, 1);
    }
#undef HFX_L64
#undef HFX_LL
#undef HFX_L
    return (int)cudaErrorInvalidValue;
}

int hfx_lists_generate_long(const DevDB &db, const int32_t *cover, int64_t npep1, int32_t nbins,
                            const uint32_t *lstart, uint64_t total10, uint32_t *lists, uint16_t *list_len,
                            int fastdiv, float ion_bw, unsigned long long *stats, uint32_t *err,
                            cudaStream_t st) {
    const int nw = 8;
    const size_t smem = (size_t)nw * kLongKeys * 4;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto f = fastdiv ? k_gen_lists_long<true> : k_gen_lists_long<false>;
    cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, nw * 32, smem);
    f<<<sms * (per > 0 ? per : 1), nw * 32, smem, st>>>(db, cover, npep1, nbins, lstart, total10, lists, list_len,
                                                        ion_bw, stats, err);
    return (int)cudaGetLastError();
}

int hfx_rescore_lists(const void *lists, int long_rows, const uint32_t *lstart, uint64_t total10,
                      const uint16_t *list_len, uint32_t num_pep, const uint32_t *idx_sorted, const float *rows32,
                      int64_t stride, const SpecMeta *meta, const uint64_t *kept_k, int32_t nspec, int32_t K,
                      int32_t topn, float *out_s, uint64_t *out_k, uint32_t *out_pep, uint32_t *err,
                      cudaStream_t st) {
    if (nspec <= 0) return 0;
    if (long_rows)
        k_rescore_lists<uint32_t><<<nspec, 256, 0, st>>>((const uint32_t *)lists, lstart, total10, list_len, num_pep,
                                                         idx_sorted, rows32, stride, meta, kept_k, K, topn, out_s,
                                                         out_k, out_pep, err);
    else
        k_rescore_lists<uint16_t><<<nspec, 256, 0, st>>>((const uint16_t *)lists, lstart, total10, list_len, num_pep,
                                                         idx_sorted, rows32, stride, meta, kept_k, K, topn, out_s,
                                                         out_k, out_pep, err);
    return (int)cudaGetLastError();
}
