// Per-step ion lists of modified isoforms (the batched modification search
// over lists, batch_mode 1).
//
// The reference enumerates every modified candidate of a spectrum
// (filter_by_mod.cu:145-378, calc_mod_cands.cu, prepare_gen_mod.cu,
// gen_mod_pep.cu) and builds its theoretical row (mion_series.cu:174-328)
// once per spectrum.  The fused scorer (mods.cu) rebuilds an isoform's ions
// for every work item whose spectra cover it.  Here, as for unmodified
// candidates (lists.cu), the step first builds each needed isoform's ion
// list once, per charge level, and the scorer streams the lists:
//   1. which (combination, position, level) the batch needs: every
//      spectrum adds its combination windows [mb, me) to a difference array
//      per (combination, modified ion-charge level); a scan marks coverage;
//   2. per (combination, position) with coverage: the modable-acid counts
//      over [tc, tn) and the isoform count (filter_by_mod.cu:216-261,
//      calc_mod_cands.cu:49-66), and the slot the isoforms' lists take;
//      scans give every isoform a global index and every slot an offset;
//   3. one record per isoform: its ordering key (combination, position,
//      rank; Search.hs:119-123) and its slot;
//   4. one thread per isoform: unrank the modified residues
//      (gen_mod_pep.cu:127-227, combinatorics.h:90-134) into a bit per
//      residue; then one warp per isoform: build the bit planes of charges
//      1..zmax with the modified masses (residual + delta, residue mass +
//      acid delta) and write the distinct-bin list of every needed level
//      (the list format of lists.cu);
//   5. the scorer: work items (spectrum group, combination, chunk of
//      positions) as in the fused path; an item's isoforms are a contiguous
//      index range; each is streamed against the group's tile.
// Spectra whose charge gives no modified ion charges (mion_series.cu:425-438)
// still enumerate their isoforms, each scored 0 over an empty list.
#include <algorithm>

#include "hfx_internal.h"
#include "device_common.cuh"
#include "batched.h"
#include "batched_common.cuh"
#include "lists.h"
#include "lists_device.cuh"
#include "mods_device.cuh"
#include "iso_lists.h"

namespace hfx {

// 1. coverage: diff[(mu * kLevels + z - 1) * npep1 + p]
__global__ void k_mark_mod_levels(const SpecMeta *__restrict__ meta, const uint32_t *__restrict__ mb,
                                  const uint32_t *__restrict__ me, int32_t nspec, int32_t num_mod, int64_t npep1,
                                  int32_t *__restrict__ diff) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nspec * num_mod) return;
    const int32_t s = (int32_t)(t / num_mod), mu = (int32_t)(t % num_mod);
    const SpecMeta m = meta[s];
    const uint32_t b = mb[t], e = me[t];
    if (m.status != 0 || e <= b) return;
    // no modified ion charges: the isoforms still exist (score 0); level 1 marks them
    const int z = m.charges_mod >= 1 ? min(m.charges_mod, kLevels) : 1;
    int32_t *d = diff + ((int64_t)mu * kLevels + (z - 1)) * npep1;
    atomicAdd(d + b, 1);
    atomicAdd(d + e, -1);
}

__device__ __forceinline__ uint32_t need_levels(const int32_t *__restrict__ cover, int64_t npep1, int32_t mu,
                                                uint32_t p) {
    uint32_t need = 0;
#pragma unroll
    for (int z = 0; z < kLevels; ++z)
        if (cover[((int64_t)mu * kLevels + z) * npep1 + p] > 0) need |= 1u << z;
    return need;
}

// Entries of one isoform's slot: the level-z list at unit * z(z-1)/2 for
// z = 1..zmax, unit = the position's rounded 10 (tn - tc).
__device__ __forceinline__ uint64_t iso_slot(uint32_t unit, int zmax) {
    return (uint64_t)unit * (uint64_t)(zmax * (zmax + 1) / 2);
}

// 2. per (combination, position): the isoform count and the slot entries of
// all its isoforms (one thread each).  count has n + 1 entries (the last 0).
__global__ void k_iso_count(DevDB db, DevMods mods, const int32_t *__restrict__ cover, int64_t npep1,
                            const uint32_t *__restrict__ lstart, int64_t n, int32_t *__restrict__ count,
                            unsigned long long *__restrict__ units) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    if (i == n) {
        count[n] = 0;
        return;
    }
    const int32_t mu = (int32_t)(i / db.num_pep);
    const uint32_t p = (uint32_t)(i % db.num_pep);
    const uint32_t need = need_levels(cover, npep1, mu, p);
    uint32_t niso = 0;
    int zmax = 0;
    if (need) {
        zmax = 32 - __clz(need);
        const uint32_t tc = db.tc_sorted[p], tn = db.tn_sorted[p];
        // modable-acid counts over [tc, tn) (filter_by_mod.cu:216-230)
        uint32_t D[kMaxMa];
#pragma unroll
        for (int k = 0; k < kMaxMa; ++k) D[k] = 0u;
        for (uint32_t j = tc; j < tn; ++j) {
            const uint32_t t = ((uint32_t)__ldg(db.ions + j) >> 5) & 7u;
#pragma unroll
            for (int k = 0; k < kMaxMa; ++k) D[k] += (t == (uint32_t)(k + 1)) ? 1u : 0u;
        }
        const int32_t *dcount = mods.counts + (size_t)mu * mods.num_ma;
        bool modable = true;
#pragma unroll
        for (int k = 0; k < kMaxMa; ++k)
            if (k < mods.num_ma) modable &= D[k] >= (uint32_t)dcount[k];
        if (modable) {
            uint32_t scan[kMaxMa];
            niso = isoform_count(D, dcount, mods.num_ma, scan);
        }
    }
    count[i] = (int32_t)niso;
    units[i] = niso ? (unsigned long long)niso * iso_slot(lstart[p + 1] - lstart[p], zmax) : 0ull;
}

// 3. the isoform records: key (combination, position, rank) and slot
// offset; isoforms past the capacities are dropped and reported.
__global__ void k_iso_expand(DevDB db, const int32_t *__restrict__ count, const int32_t *__restrict__ incl,
                             const unsigned long long *__restrict__ units,
                             const unsigned long long *__restrict__ incl_units, const int32_t *__restrict__ cover,
                             int64_t npep1, const uint32_t *__restrict__ lstart, int64_t n, uint32_t cap_iso,
                             uint64_t cap_entries, uint64_t *__restrict__ iso_key, uint64_t *__restrict__ iso_off,
                             uint32_t *__restrict__ err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t c = count[i];
    if (c <= 0) return;
    const int32_t mu = (int32_t)(i / db.num_pep);
    const uint32_t p = (uint32_t)(i % db.num_pep);
    const uint32_t base = (uint32_t)(incl[i] - c);
    const uint64_t off0 = incl_units[i] - units[i];
    const int zmax = 32 - __clz(need_levels(cover, npep1, mu, p));
    const uint64_t slot = iso_slot(lstart[p + 1] - lstart[p], zmax);
    // a key holds position and rank in 27 bits each, the combination in 9
    const bool fits = p < (1u << 27) && (uint32_t)c < (1u << 27) && mu < 512;
    if (!fits) atomicOr(err, kErrKeyOverflow);
    for (int32_t r = 0; r < c; ++r) {
        const uint32_t t = base + (uint32_t)r;
        if (t >= cap_iso) {  // beyond the records' capacity (graph replays)
            atomicOr(err, kErrBounds);
            return;
        }
        const uint64_t o = off0 + (uint64_t)r * slot;
        if (!fits || o + slot > cap_entries) {  // a record that is skipped (no slot, or no key)
            if (fits) atomicOr(err, kErrBounds);
            iso_key[t] = ~0ull;
            iso_off[t] = 0;
            continue;
        }
        iso_key[t] = mod_key(mu, p, (uint32_t)r);
        iso_off[t] = o;
    }
}

// 4a. one thread per isoform: the residues it modifies (modable-acid
// counts, isoform count, unranking, gen_mod_pep.cu:127-227, and the i-th
// acid counter of mion_series.cu:244-286 / check_series.cu:62-100),
// pos_words words per record in iso_pos.  The per-residue decision is
// ModIsoform::chunk_add's, residue by residue; consecutive records are
// mostly the ranks of one (combination, peptide), so a warp's threads run
// the same loops.
__global__ void __launch_bounds__(256) k_iso_positions(DevDB db, DevMods mods, const int32_t *__restrict__ total_p,
                                                       uint32_t cap_iso, const uint64_t *__restrict__ iso_key,
                                                       int32_t pos_words, uint32_t *__restrict__ iso_pos,
                                                       uint32_t *__restrict__ err) {
    const uint32_t total = min((uint32_t)*total_p, cap_iso);
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const uint64_t key = iso_key[t];
    const int32_t mu = (int32_t)((key >> 54) & 0x1FFu);
    const uint32_t p = (uint32_t)((key >> 27) & 0x7FFFFFFu), rank = (uint32_t)(key & 0x7FFFFFFu);
    uint32_t *bits = iso_pos + (size_t)t * pos_words;
    if (key == ~0ull || p >= db.num_pep || mu >= mods.num_mod) return;  // a skipped record
    const uint32_t tc = db.tc_sorted[p], tn = db.tn_sorted[p];
    const int num_ma = mods.num_ma;
    if (tn > tc && (int64_t)(tn - tc) > 32ll * pos_words) {  // longer than the database's longest peptide
        atomicOr(err, kErrBounds);
        for (int i = 0; i < pos_words; ++i) bits[i] = 0u;
        return;
    }
    // modable-acid counts (filter_by_mod.cu:216-230)
    uint32_t D[kMaxMa];
#pragma unroll
    for (int i = 0; i < kMaxMa; ++i) D[i] = 0u;
    for (uint32_t j = tc; j < tn; ++j) {
        const uint32_t ty = ((uint32_t)__ldg(db.ions + j) >> 5) & 7u;
#pragma unroll
        for (int i = 0; i < kMaxMa; ++i) D[i] += (i < num_ma && ty == (uint32_t)(i + 1)) ? 1u : 0u;
    }
    const int32_t *dcount = mods.counts + (size_t)mu * num_ma;
    uint32_t scan[kMaxMa];
    uint64_t mask[kMaxMa];
    const uint32_t niso = isoform_count(D, dcount, num_ma, scan);
    if (rank >= niso || !isoform_masks(D, scan, dcount, num_ma, rank, mask)) {
        atomicOr(err, kErrKeyOverflow);
        for (int i = 0; i < pos_words; ++i) bits[i] = 0u;
        return;
    }
    // the i-th acid counter, in peptide order
    uint32_t seen_any = 0u, seen[kMaxMa];
#pragma unroll
    for (int i = 0; i < kMaxMa; ++i) seen[i] = 0u;
    uint32_t word = 0u;
    for (uint32_t j = tc; j < tn; ++j) {
        const uint32_t ty = ((uint32_t)__ldg(db.ions + j) >> 5) & 7u;
        uint32_t k = seen_any, ts = 0u;
        uint64_t m = 0ull;
#pragma unroll
        for (int i = 0; i < kMaxMa; ++i) {
            if (i < num_ma && ty == (uint32_t)(i + 1)) {
                ts = seen[i];
                m = mask[i];
                seen[i] += 1u;
            }
        }
        if (mods.per_type) k = ts;
        seen_any += ty != 0u ? 1u : 0u;
        const bool modded = ty != 0u && (int)ty <= num_ma && k < 64u && ((m >> k) & 1ull);
        const uint32_t r = j - tc;
        word |= (modded ? 1u : 0u) << (r & 31u);
        if ((r & 31u) == 31u || j + 1 == tn) {
            bits[r >> 5] = word;
            word = 0u;
        }
    }
}

// 4b. one warp per isoform: the distinct-bin list of every needed level.
template <bool FastDiv>
__global__ void __launch_bounds__(256) k_gen_iso_lists(DevDB db, DevMods mods, const int32_t *__restrict__ cover,
                                                       int64_t npep1, int32_t nbins,
                                                       const uint32_t *__restrict__ lstart,
                                                       const int32_t *__restrict__ total_p, uint32_t cap_iso,
                                                       const uint64_t *__restrict__ iso_key,
                                                       const uint64_t *__restrict__ iso_off, uint16_t *__restrict__ lists,
                                                       uint64_t list_total, uint16_t *__restrict__ iso_len,
                                                       int32_t list_cap, int32_t pos_words,
                                                       const uint32_t *__restrict__ iso_pos,
                                                       unsigned long long *__restrict__ stats,
                                                       uint32_t *__restrict__ err) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int32_t words = (nbins + 31) / 32;
    uint32_t *planes = reinterpret_cast<uint32_t *>(smem) + (size_t)warp * 3 * words;
    uint16_t *list = reinterpret_cast<uint16_t *>(reinterpret_cast<uint32_t *>(smem) + (size_t)nw * 3 * words) +
                     (size_t)warp * list_cap;
    for (int32_t i = lane; i < 3 * words; i += 32) planes[i] = 0u;
    __syncwarp();
    const Planes pl{planes, planes + words, planes + 2 * words};
    const float mt_lane = db.mt[lane];
    float ma_lane = 0.0f;
#pragma unroll
    for (int i = 0; i < kMaxMa; ++i)
        if (lane == i && i < mods.num_ma) ma_lane = mods.ma_mass[i];
    const uint32_t total = min((uint32_t)*total_p, cap_iso);
    // per-warp work counters (a warp's share of one launch fits 32 bits)
    uint32_t my_lists = 0, my_entries = 0, my_iso = 0, my_res = 0;
    for (uint32_t t = blockIdx.x * nw + warp; t < total; t += gridDim.x * nw) {
        const uint64_t key = iso_key[t];
        const int32_t mu = (int32_t)((key >> 54) & 0x1FFu);
        const uint32_t p = (uint32_t)((key >> 27) & 0x7FFFFFFu);
        if (key == ~0ull || p >= db.num_pep || mu >= mods.num_mod) {  // a skipped record
            if (lane < kLevels) iso_len[(size_t)t * kLevels + lane] = 0;
            continue;
        }
        const uint32_t need = need_levels(cover, npep1, mu, p);
        const int zmax = 32 - __clz(need);
        const uint32_t tc = db.tc_sorted[p], tn = db.tn_sorted[p];
        const uint32_t unit = lstart[p + 1] - lstart[p];
        const uint64_t off = iso_off[t];
        if (off + iso_slot(unit, zmax) > list_total ||
            (tn > tc && (int64_t)(tn - tc) > 32ll * pos_words)) {  // neither happens for an expanded record
            if (lane == 0) atomicOr(err, kErrBounds);
            if (lane < kLevels) iso_len[(size_t)t * kLevels + lane] = 0;
            continue;
        }
        // the residues this isoform modifies (k_iso_positions)
        const ModPositions iso{iso_pos + (size_t)t * pos_words, ma_lane, 0u};
        my_iso += 1;
        my_res += tn > tc ? tn - tc : 0u;
        // mion_series.cu:226: residual + delta
        const float residual = __fadd_rn(db.r_sorted[p], mods.delta[mu]);
        WordRange all{0x7FFFFFFF, 0};
        // the level-z list from the planes, when some spectrum needs it
        auto emit_level = [&](int z) {
            if (!((need >> (z - 1)) & 1u)) return;
            const WordRange use = all.hi > all.lo ? all : WordRange{0, 0};
            uint16_t *slot = lists + off + (uint64_t)unit * (uint64_t)(z * (z - 1) / 2);
            const int room = (int)(unit * (uint32_t)z);  // >= 10 (tn - tc) z distinct bins
            int nl = compact_planes(pl, use, z == zmax, list, list_cap, slot, room);
            if (nl > room) {
                if (lane == 0) atomicOr(err, kErrListOverflow);
                nl = room;
            }
            if (nl <= list_cap) {
                const uint4 *src = reinterpret_cast<const uint4 *>(list);
                uint4 *dst = reinterpret_cast<uint4 *>(slot);
                for (int i = lane; i < ((nl + 7) >> 3); i += 32) dst[i] = src[i];
            }
            if (lane == 0) iso_len[(size_t)t * kLevels + (z - 1)] = (uint16_t)nl;
            my_lists += 1;
            my_entries += (uint32_t)nl;
            __syncwarp();
        };
        auto widen = [&](WordRange wr) {
            if (wr.hi > wr.lo) {
                all.lo = min(all.lo, wr.lo);
                all.hi = max(all.hi, wr.hi);
            }
        };
        for (int z = 1; z <= zmax; ++z) {
            widen(build_planes_range<FastDiv>(pl, db.ions, tc, tn, residual, z, z, nbins, mt_lane, iso));
            emit_level(z);
        }
        if (lane >= zmax && lane < kLevels) iso_len[(size_t)t * kLevels + lane] = 0;
        if (lane < zmax && !((need >> lane) & 1u)) iso_len[(size_t)t * kLevels + lane] = 0;
    }
    if (stats && lane == 0) {
        atomicAdd(&stats[0], (unsigned long long)my_lists);
        atomicAdd(&stats[1], (unsigned long long)my_entries);
        atomicAdd(&stats[5], (unsigned long long)my_iso);
        atomicAdd(&stats[6], (unsigned long long)my_res);
    }
}

// 5. the scorer over the isoform lists: a persistent grid pulls work items
// (group, combination, chunk of positions); the group's tile is staged by
// one bulk copy; an item's isoforms are [index(mu, p0), index(mu, p1)); kC
// isoforms per warp (32 / kC lanes each, entry i of a list by lane i % (32 /
// kC)); in FP32 each lane keeps four partial-sum sets, the canonical order.
template <typename T, int G, int kC>
__global__ void __launch_bounds__(512, 1)
k_score_iso_lists(const uint16_t *__restrict__ lists, uint64_t list_total, const uint32_t *__restrict__ lstart,
                  const uint64_t *__restrict__ iso_key, const uint64_t *__restrict__ iso_off,
                  const uint16_t *__restrict__ iso_len, const int32_t *__restrict__ count,
                  const int32_t *__restrict__ incl, uint32_t num_pep, uint32_t cap_iso, const T *__restrict__ tiles,
                  int64_t stride, const uint32_t *__restrict__ mb, const uint32_t *__restrict__ me, int32_t num_mod,
                  const int32_t *__restrict__ perm, const GroupInfo *__restrict__ groups,
                  const uint32_t *__restrict__ mlo, const uint32_t *__restrict__ mhi,
                  const uint32_t *__restrict__ mchunk, const uint32_t *__restrict__ item_off, int32_t n_gm, int32_t K,
                  uint32_t *__restrict__ counter, float *__restrict__ part_s, uint64_t *__restrict__ part_k,
                  unsigned long long *__restrict__ ncand, unsigned long long *__restrict__ stats, uint32_t qoff,
                  uint32_t *__restrict__ err) {
    static_assert(kC == 1 || kC == 4, "1 or 4 isoforms per warp");
    constexpr int kW = 32 / kC;
    // FP32 with four isoforms per warp keeps the canonical order: entry i of
    // a list goes to partial sum i % 32, i.e. entry k of each round of 32 to
    // this lane's partial set k (8 lanes per isoform)
    constexpr bool kSets4 = std::is_same<T, float>::value && kC > 1;
    static_assert(G <= kW, "a lane group takes up to one spectrum of the group per lane");
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int hl = lane & (kW - 1), quad = lane / kW;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    T *stile = reinterpret_cast<T *>(smem + 128);
    __shared__ int32_t s_item;
    __shared__ uint32_t s_next;
    __shared__ uint32_t s_wb[G], s_we[G];
    __shared__ int32_t s_spec[G];
    __shared__ uint32_t thr_u[G], s_lock[G];
    __shared__ float s_ls[G * 32];
    __shared__ uint64_t s_lk[G * 32];

    const uint32_t total = item_off[n_gm];
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    const int my_slot = reduce_slot_of_lane<G>(lane);
    uint32_t phase = 0;
    unsigned long long my_cand = 0, my_entries = 0, my_psm = 0, my_tile = 0;
    CtaSlots<G, uint64_t> slots;
    slots.bind(s_ls, s_lk, s_lock, thr_u, smem + qoff + (size_t)warp * CtaSlots<G, uint64_t>::warp_bytes(), err);
    while (true) {
        if (threadIdx.x == 0) s_item = (int32_t)atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t item = (uint32_t)s_item;
        if (item >= total) break;
        const int32_t gm = find_group(item_off, n_gm, item);
        const int32_t g = gm / num_mod, mu = gm % num_mod;
        const GroupInfo gi = groups[g];
        const uint32_t p0 = mlo[gm] + (item - item_off[gm]) * mchunk[gm];
        const uint32_t p1 = min(mhi[gm], p0 + mchunk[gm]);
        const int64_t row = (int64_t)mu * num_pep;
        // the item's isoforms (index = inclusive scan - count)
        const uint32_t t0 = min((uint32_t)(incl[row + p0] - count[row + p0]), cap_iso);
        const uint32_t t1 = min((uint32_t)(incl[row + p1] - count[row + p1]), cap_iso);
        const int cnt_members = (int)gi.count;
        if (threadIdx.x < G) {
            const int j = threadIdx.x;
            uint32_t b = 0, e = 0;
            int32_t s = -1;
            if (j < cnt_members) {
                s = perm[gi.pos0 + j];
                b = mb[(size_t)s * num_mod + mu];
                e = me[(size_t)s * num_mod + mu];
            }
            s_wb[j] = b;
            s_we[j] = e;
            s_spec[j] = s;
        }
        slots.reset_shared();
        const int32_t nb = tile_bins(gi.maxlen);
        if (threadIdx.x == 0) {
            s_next = t0;
            fence_proxy_async();
            const uint32_t bytes = (uint32_t)((size_t)nb * G * sizeof(T));
            mbar_arrive_expect_tx(bar, bytes);
            bulk_g2s(stile, tiles + (size_t)g * stride * G, bytes, bar);
            my_tile += bytes;
        }
        {
            // bins [nb, stride + 8) read as zero (the pad entry's bin is stride)
            uint4 *zt = reinterpret_cast<uint4 *>(stile);
            const size_t z0 = (size_t)nb * G * sizeof(T) / 16, z1 = (size_t)(stride + 8) * G * sizeof(T) / 16;
            for (size_t i = z0 + threadIdx.x; i < z1; i += blockDim.x) zt[i] = make_uint4(0u, 0u, 0u, 0u);
            fence_proxy_async();
        }
        __syncthreads();
        if (!mbar_wait(bar, phase, kWaitLimit)) {
            if (threadIdx.x == 0) atomicOr(err, kErrTimeout);
            return;
        }
        phase ^= 1u;
        const uint32_t my_b = hl < G ? s_wb[hl] : 0u, my_e = hl < G ? s_we[hl] : 0u;
        const int32_t my_s = hl < G ? s_spec[hl] : -1;
        const uint32_t pad = (uint32_t)stride << 2;
        const int z = (int)gi.charges_mod;
        while (true) {
            uint32_t q = 0;
            if (lane == 0) q = atomicAdd(&s_next, (uint32_t)kC);
            const uint32_t base = __shfl_sync(kFullMask, q, 0);
            if (base >= t1) break;
            const uint32_t t = base + (uint32_t)quad;
            const bool have = t < t1;
            uint64_t key = ~0ull;
            uint32_t p = 0, rank = 0;
            if (have) {
                key = iso_key[t];
                p = (uint32_t)((key >> 27) & 0x7FFFFFFu);
                rank = (uint32_t)(key & 0x7FFFFFFu);
            }
            const bool valid = have && key != ~0ull && p < num_pep;  // skipped records score nothing
            const uint32_t bal = __ballot_sync(kFullMask, valid && hl < G && my_b <= p && p < my_e);
            const uint32_t act = (bal >> (kW * quad)) & ((1u << G) - 1u);
            // every isoform of a position is one pair per member spectrum
            if (ncand && act && rank == 0 && hl < G && ((act >> hl) & 1u))
                atomicAdd(ncand + my_s, (unsigned long long)count[row + p]);
            int n = 0;
            const uint16_t *lp = lists;
            if (act && z >= 1) {
                const uint64_t off =
                    iso_off[t] + (uint64_t)(lstart[p + 1] - lstart[p]) * (uint64_t)(z * (z - 1) / 2);
                n = iso_len[(size_t)t * kLevels + (z - 1)];
                if (off + (uint64_t)n > list_total) {
                    if (hl == 0) atomicOr(err, kErrBounds);
                    n = 0;
                } else {
                    lp = lists + off;
                }
            }
            float acc[G];
#pragma unroll
            for (int j = 0; j < G; ++j) acc[j] = 0.0f;
            float acc4[kSets4 ? 4 : 1][G];
#pragma unroll
            for (int k = 0; k < (kSets4 ? 4 : 1); ++k)
#pragma unroll
                for (int j = 0; j < G; ++j) acc4[k][j] = 0.0f;
            int nmax = n;
#pragma unroll
            for (int o = kW; o < 32; o <<= 1) nmax = max(nmax, __shfl_xor_sync(kFullMask, nmax, o));
            for (int i0 = 0; i0 < nmax; i0 += 4 * kW) {
                uint32_t e[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int i = i0 + kW * k + hl;
                    e[k] = i < n ? (uint32_t)__ldg(lp + i) : pad;
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    float *a = acc;
                    if constexpr (kSets4) a = acc4[k];
                    TileFma<T, G>::fma(stile, e[k] >> 2, e[k] & 3u, *reinterpret_cast<float(*)[G]>(a));
                }
            }
            if constexpr (kSets4) {
                // the 32-lane butterfly's offsets 16 and 8, within the lane
#pragma unroll
                for (int j = 0; j < G; ++j)
                    acc[j] = __fadd_rn(__fadd_rn(acc4[0][j], acc4[2][j]), __fadd_rn(acc4[1][j], acc4[3][j]));
            }
            float sc;
            if constexpr (kC == 1) sc = reduce_scatter<G>(acc);
            else sc = reduce_scatter_lanes<G, kW>(acc);
            const bool owner = (lane & (32 / G - 1)) == 0;
#pragma unroll
            for (int c = 0; c < kC; ++c) {
                const uint32_t act_c = __shfl_sync(kFullMask, act, c * kW);
                const uint64_t key_c = __shfl_sync(kFullMask, key, c * kW);
                const int n_c = __shfl_sync(kFullMask, n, c * kW);
                my_cand += act_c != 0u;
                my_entries += (unsigned long long)n_c;
                my_psm += (unsigned long long)__popc(act_c);
                const float sc_c =
                    kC == 1 ? sc : __shfl_sync(kFullMask, sc, c * kW + (lane / (32 / G)) * (kW / G));
                const bool want = owner && ((act_c >> my_slot) & 1u) &&
                                  score_order(sc_c) >= *(volatile uint32_t *)(thr_u + my_slot);
                slots.offer(want, sc_c, key_c, my_slot, K);
            }
        }
        slots.drain(K);
        __syncthreads();
        const int nw = blockDim.x >> 5;
        for (int j = warp; j < cnt_members; j += nw) {
            const size_t o = ((size_t)item * G + j) * K;
            slots.result(j, K, part_s + o, part_k + o);
        }
        __syncthreads();
    }
    if (stats && lane == 0) {
        atomicAdd(&stats[2], my_cand);
        atomicAdd(&stats[3], my_entries);
        atomicAdd(&stats[4], my_psm);
        if (threadIdx.x == 0) atomicAdd(&stats[7], my_tile);
    }
}

// ---- inclusive scan of 64-bit values (reduce, scan partials, apply) ----
constexpr int kScan64Tile = 4096;

__global__ void k_scan64_reduce(const unsigned long long *__restrict__ a, int64_t n,
                                unsigned long long *__restrict__ partial) {
    __shared__ unsigned long long red[32];
    const int64_t base = (int64_t)blockIdx.x * kScan64Tile;
    unsigned long long s = 0;
    for (int i = threadIdx.x; i < kScan64Tile; i += blockDim.x)
        if (base + i < n) s += a[base + i];
    for (int o = 16; o >= 1; o >>= 1) s += __shfl_xor_sync(kFullMask, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned long long v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0ull;
        for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

__device__ __forceinline__ unsigned long long warp_incl_scan64(unsigned long long v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long t = __shfl_up_sync(kFullMask, v, d);
        if (lane >= d) v += t;
    }
    return v;
}

// single CTA: exclusive scan of the partials in place
__global__ void k_scan64_partials(unsigned long long *__restrict__ partial, int64_t nb) {
    __shared__ unsigned long long ws[32];
    __shared__ unsigned long long carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
        const int64_t i = b0 + threadIdx.x;
        const unsigned long long v = i < nb ? partial[i] : 0ull;
        const unsigned long long x = warp_incl_scan64(v);
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned long long w = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0ull;
            w = warp_incl_scan64(w);
            ws[lane] = w;
        }
        __syncthreads();
        const unsigned long long before = carry + (warp ? ws[warp - 1] : 0ull);
        if (i < nb) partial[i] = before + x - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + x;
        __syncthreads();
    }
}

__global__ void k_scan64_apply(const unsigned long long *__restrict__ a, int64_t n,
                               const unsigned long long *__restrict__ partial, unsigned long long *__restrict__ out) {
    __shared__ unsigned long long ws[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kScan64Tile;
    const int per = kScan64Tile / blockDim.x;
    unsigned long long loc[16];
    unsigned long long s = 0;
    for (int k = 0; k < per; ++k) {
        const int64_t i = base + (int64_t)threadIdx.x * per + k;
        loc[k] = i < n ? a[i] : 0ull;
        s += loc[k];
    }
    const unsigned long long x = warp_incl_scan64(s);
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0ull;
        w = warp_incl_scan64(w);
        ws[lane] = w;
    }
    __syncthreads();
    unsigned long long run = partial[blockIdx.x] + (warp ? ws[warp - 1] : 0ull) + x - s;
    for (int k = 0; k < per; ++k) {
        const int64_t i = base + (int64_t)threadIdx.x * per + k;
        run += loc[k];
        if (i < n) out[i] = run;
    }
}

}  // namespace hfx

using namespace hfx;

int64_t hfx_iso_scan64_partials_needed(int64_t n) { return (n + kScan64Tile - 1) / kScan64Tile + 1; }

int hfx_iso_plan(const DevDB &db, const DevMods &m, const SpecMeta *meta, int32_t nspec, const uint32_t *mb,
                 const uint32_t *me, const uint32_t *lstart, int32_t *cover, int32_t *cover_partial,
                 int32_t *count, int32_t *incl, int32_t *count_partial, unsigned long long *units,
                 unsigned long long *incl_units, unsigned long long *units_partial, cudaStream_t st) {
    const int64_t npep1 = (int64_t)db.num_pep + 1;
    const int64_t ncover = (int64_t)m.num_mod * kLevels * npep1;
    const int64_t n = (int64_t)m.num_mod * db.num_pep;
    cudaError_t e = cudaMemsetAsync(cover, 0, sizeof(int32_t) * (size_t)ncover, st);
    if (e != cudaSuccess) return (int)e;
    const int64_t nt = (int64_t)nspec * m.num_mod;
    if (nt > 0)
        k_mark_mod_levels<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(meta, mb, me, nspec, m.num_mod, npep1, cover);
    int rc = hfx_scan_inclusive(cover, ncover, cover, cover_partial, st);  // in place
    if (rc) return rc;
    k_iso_count<<<(unsigned)((n + 1 + 255) / 256), 256, 0, st>>>(db, m, cover, npep1, lstart, n, count, units);
    rc = hfx_scan_inclusive(count, n + 1, incl, count_partial, st);
    if (rc) return rc;
    if (n > 0) {
        const int64_t nb = (n + kScan64Tile - 1) / kScan64Tile;
        k_scan64_reduce<<<(unsigned)nb, 512, 0, st>>>(units, n, units_partial);
        k_scan64_partials<<<1, 1024, 0, st>>>(units_partial, nb);
        k_scan64_apply<<<(unsigned)nb, 256, 0, st>>>(units, n, units_partial, incl_units);
    }
    return (int)cudaGetLastError();
}

int hfx_iso_expand(const DevDB &db, const DevMods &m, const int32_t *cover, const uint32_t *lstart,
                   const int32_t *count, const int32_t *incl, const unsigned long long *units,
                   const unsigned long long *incl_units, uint32_t cap_iso, uint64_t cap_entries, uint64_t *iso_key,
                   uint64_t *iso_off, uint32_t *err, cudaStream_t st) {
    const int64_t n = (int64_t)m.num_mod * db.num_pep;
    if (n <= 0) return 0;
    k_iso_expand<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(db, count, incl, units, incl_units, cover,
                                                               (int64_t)db.num_pep + 1, lstart, n, cap_iso,
                                                               cap_entries, iso_key, iso_off, err);
    return (int)cudaGetLastError();
}

int hfx_iso_generate(const DevDB &db, const DevMods &m, const int32_t *cover, int32_t nbins, const uint32_t *lstart,
                     const int32_t *total_p, uint32_t cap_iso, const uint64_t *iso_key, const uint64_t *iso_off,
                     uint16_t *lists, uint64_t list_total, uint16_t *iso_len, int32_t list_cap, int32_t pos_words,
                     uint32_t *iso_pos, int fastdiv, unsigned long long *stats, uint32_t *err, cudaStream_t st) {
    if (cap_iso == 0) return 0;
    const int nw = 8;
    const int32_t words = (nbins + 31) / 32;
    // 16-byte staging lists of up to kStageCap entries (longer lists are
    // written directly)
    list_cap = (std::max(32, std::min(list_cap, kStageCap)) + 7) & ~7;
    const size_t smem = (size_t)nw * 3 * words * 4 + (size_t)nw * list_cap * 2;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_iso_positions<<<(unsigned)((cap_iso + 255) / 256), 256, 0, st>>>(db, m, total_p, cap_iso, iso_key, pos_words,
                                                                        iso_pos, err);
    auto f = fastdiv ? k_gen_iso_lists<true> : k_gen_iso_lists<false>;
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, f, nw * 32, smem);
    f<<<sms * (per > 0 ? per : 1), nw * 32, smem, st>>>(db, m, cover, (int64_t)db.num_pep + 1, nbins, lstart, total_p,
                                                        cap_iso, iso_key, iso_off, lists, list_total, iso_len,
                                                        list_cap, pos_words, iso_pos, stats, err);
    return (int)cudaGetLastError();
}

template <typename T, int G, int kC>
static int launch_iso_score(const uint16_t *lists, uint64_t list_total, const uint32_t *lstart,
                            const uint64_t *iso_key, const uint64_t *iso_off, const uint16_t *iso_len,
                            const int32_t *count, const int32_t *incl, uint32_t num_pep, uint32_t cap_iso,
                            const void *tiles, int64_t stride, const uint32_t *mb, const uint32_t *me,
                            int32_t num_mod, const BatchedWs &ws, const uint32_t *mlo, const uint32_t *mhi,
                            const uint32_t *mchunk, const uint32_t *item_off, int32_t n_gm, int32_t K, float *ps,
                            uint64_t *pk, unsigned long long *ncand, unsigned long long *stats, uint32_t *err,
                            cudaStream_t st) {
    int dev = 0, sms = 0, smem_max = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const int nw = 16;
    const size_t qoff = 128 + (((size_t)(stride + 8) * G * sizeof(T) + 15) & ~(size_t)15);
    const size_t smem = qoff + (size_t)nw * CtaSlots<G, uint64_t>::warp_bytes();
    auto fn = k_score_iso_lists<T, G, kC>;
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, fn);
    if (smem + fa.sharedSizeBytes > (size_t)smem_max) return (int)cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, nw * 32, smem);
    cudaMemsetAsync(ws.counter, 0, 4, st);
    fn<<<sms * (per > 0 ? per : 1), nw * 32, smem, st>>>(lists, list_total, lstart, iso_key, iso_off, iso_len, count,
                                                         incl, num_pep, cap_iso, (const T *)tiles, stride, mb, me,
                                                         num_mod, ws.perm, ws.groups, mlo, mhi, mchunk, item_off,
                                                         n_gm, K, ws.counter, ps, pk, ncand, stats, (uint32_t)qoff,
                                                         err);
    return (int)cudaGetLastError();
}

int hfx_iso_score(const uint16_t *lists, uint64_t list_total, const uint32_t *lstart, const uint64_t *iso_key,
                  const uint64_t *iso_off, const uint16_t *iso_len, const int32_t *count, const int32_t *incl,
                  uint32_t num_pep, uint32_t cap_iso, int elem_kind, const void *tiles, int64_t stride,
                  const uint32_t *mb, const uint32_t *me, int32_t num_mod, const BatchedWs &ws, const uint32_t *mlo,
                  const uint32_t *mhi, const uint32_t *mchunk, const uint32_t *item_off, int32_t n_gm, int32_t G,
                  int32_t K, float *ps, uint64_t *pk, unsigned long long *ncand, unsigned long long *stats,
                  uint32_t *err, cudaStream_t st) {
    if (n_gm <= 0) return 0;
    if (K > 32) return (int)cudaErrorInvalidValue;
#define HFX_IS(T, GG, CC)                                                                                         \
    return launch_iso_score<T, GG, CC>(lists, list_total, lstart, iso_key, iso_off, iso_len, count, incl,       \
                                       num_pep, cap_iso, tiles, stride, mb, me, num_mod, ws, mlo, mhi, mchunk,  \
                                       item_off, n_gm, K, ps, pk, ncand, stats, err, st)
    if (elem_kind == 0) {
        if (G == 4) HFX_IS(float, 4, 4);
        if (G == 8) HFX_IS(float, 8, 4);
        if (G == 2) HFX_IS(float, 2, 4);
        if (G == 1) HFX_IS(float, 1, 4);
    } else if (elem_kind == 1) {
        if (G == 8) HFX_IS(__nv_bfloat16, 8, 4);
        if (G == 4) HFX_IS(__nv_bfloat16, 4, 4);
        if (G == 2) HFX_IS(__nv_bfloat16, 2, 4);
        if (G == 1) HFX_IS(__nv_bfloat16, 1, 4);
    } else {
        if (G == 8) HFX_IS(__half, 8, 4);
        if (G == 4) HFX_IS(__half, 4, 4);
        if (G == 2) HFX_IS(__half, 2, 4);
        if (G == 1) HFX_IS(__half, 1, 4);
    }
#undef HFX_IS
    return (int)cudaErrorInvalidValue;
}
