// Batched search: every spectrum of a batch in one persistent, work-stealing
// launch.  Replaces the reference's host loops over spectra
// (Search.hs:195-201, :232-245) and its per-spectrum b40c sort + full score
// copy-back (Search.hs:250-276).
//
// Planning (all on the device):
//   1. spectra are bucketed by (ion charges, wide/narrow window, 1 Da of
//      precursor residual mass) with a counting sort;
//   2. consecutive spectra of one class form groups of up to G;
//   3. a group's work is the union of its members' candidate windows, cut
//      into chunks of C candidates -- one work item each;
//   4. a persistent grid pulls items from an atomic counter.
// A work item stages its G spectrum rows in shared memory with one bulk
// copy per row (cp.async.bulk + mbarrier), then each warp builds a
// candidate's ion list once and gathers it against every member spectrum
// whose window contains the candidate.  Each warp keeps a register top-K
// per member; the CTA merges them and writes the item's partial lists; a
// merge kernel reduces them per spectrum, and (BF16/FP16 rows) a rescore
// kernel recomputes the kept candidates from the FP32 row.
#include "hfx_internal.h"
#include "device_common.cuh"
#include "batched.h"
#include "batched_common.cuh"
#include "mods_device.cuh"
#include <type_traits>

namespace hfx {

constexpr int kMassBuckets = 8192;   // 1 Da buckets of residual mass
constexpr int kClasses = 12;         // (ion charge class 0..5) x (narrow, wide)
constexpr float kWideEps = 1.0f;     // windows wider than this are "wide"

__device__ __forceinline__ int spec_class(const SpecMeta &m) {
    // charge class: plain charges 1..4 (modified ones equal them), 5 = no
    // plain ions but modified ions (charge 6..11), 0 = none
    const int cc = m.charges_plain > 0 ? m.charges_plain : (m.charges_mod > 0 ? 5 : 0);
    return cc * 2 + (m.eps > kWideEps ? 1 : 0);
}
__device__ __forceinline__ int spec_bucket(const SpecMeta &m) {
    int mb = (int)fminf(fmaxf(m.mass, 0.0f), (float)(kMassBuckets - 1));
    return spec_class(m) * kMassBuckets + mb;
}

__global__ void k_bucket_count(const SpecMeta *__restrict__ meta, int32_t nspec, uint32_t *__restrict__ hist) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nspec) return;
    const SpecMeta m = meta[s];
    if (m.status != 0) return;
    atomicAdd(&hist[spec_bucket(m)], 1u);
}

// Single-CTA exclusive scan of n counters (in place), total in *total.
__global__ void k_scan_u32(uint32_t *__restrict__ a, int32_t n, uint32_t *__restrict__ total) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int32_t base = 0; base < n; base += blockDim.x) {
        const int32_t i = base + tid;
        const uint32_t v = (i < n) ? a[i] : 0u;
        uint32_t x = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t t = __shfl_up_sync(kFullMask, x, d);
            if (lane >= d) x += t;
        }
        if (lane == 31) warp_sums[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0u;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                uint32_t t = __shfl_up_sync(kFullMask, w, d);
                if (lane >= d) w += t;
            }
            warp_sums[lane] = w;
        }
        __syncthreads();
        const uint32_t before = carry + (warp ? warp_sums[warp - 1] : 0u);
        if (i < n) a[i] = before + x - v;
        __syncthreads();
        if (tid == blockDim.x - 1) carry = before + x;
        __syncthreads();
    }
    if (tid == 0 && total) *total = carry;
}

__global__ void k_bucket_scatter(const SpecMeta *__restrict__ meta, int32_t nspec, uint32_t *__restrict__ cursor,
                                 int32_t *__restrict__ perm) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nspec) return;
    const SpecMeta m = meta[s];
    if (m.status != 0) return;
    const uint32_t pos = atomicAdd(&cursor[spec_bucket(m)], 1u);
    perm[pos] = s;
}

// One thread per group: members, union window, chunk count.
// class_off[c] = first sorted position of class c (from the bucket scan).
__global__ void k_groups(const uint32_t *__restrict__ bucket_off, const uint32_t *__restrict__ n_sorted,
                         const int32_t *__restrict__ perm, const uint32_t *__restrict__ wb,
                         const uint32_t *__restrict__ we, const SpecMeta *__restrict__ meta, int32_t G,
                         int32_t chunk, int32_t max_groups, GroupInfo *__restrict__ groups,
                         uint32_t *__restrict__ nchunks, int32_t *__restrict__ group_of,
                         int32_t *__restrict__ slot_of, uint32_t *__restrict__ ngroups_out) {
    __shared__ uint32_t cls_start[kClasses + 1], grp_start[kClasses + 1];
    if (threadIdx.x == 0) {
        uint32_t gs = 0;
        for (int c = 0; c < kClasses; ++c) {
            cls_start[c] = bucket_off[c * kMassBuckets];
            const uint32_t end = (c + 1 < kClasses) ? bucket_off[(c + 1) * kMassBuckets] : *n_sorted;
            grp_start[c] = gs;
            gs += (end - cls_start[c] + G - 1) / G;
        }
        cls_start[kClasses] = *n_sorted;
        grp_start[kClasses] = gs;
        if (blockIdx.x == 0) *ngroups_out = gs;
    }
    __syncthreads();
    const int32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= max_groups) return;
    if ((uint32_t)g >= grp_start[kClasses]) {
        nchunks[g] = 0;
        return;
    }
    int c = 0;
    while (c + 1 < kClasses && (uint32_t)g >= grp_start[c + 1]) ++c;
    const uint32_t pos0 = cls_start[c] + ((uint32_t)g - grp_start[c]) * (uint32_t)G;
    const uint32_t cnt = min((uint32_t)G, cls_start[c + 1] - pos0);
    GroupInfo gi;
    gi.pos0 = pos0;
    gi.count = cnt;
    gi.lo = 0xFFFFFFFFu;
    gi.hi = 0u;
    gi.maxlen = 0;
    gi.charges = 0;
    gi.charges_mod = 0;
    for (uint32_t j = 0; j < cnt; ++j) {
        const int32_t s = perm[pos0 + j];
        group_of[s] = g;
        slot_of[s] = (int32_t)j;
        const uint32_t b = wb[s], e = we[s];
        if (e > b) {
            gi.lo = min(gi.lo, b);
            gi.hi = max(gi.hi, e);
        }
        gi.maxlen = max(gi.maxlen, meta[s].len);
        gi.charges = meta[s].charges_plain;
        gi.charges_mod = meta[s].charges_mod;
    }
    if (gi.hi <= gi.lo) {
        gi.lo = gi.hi = 0;
    }
    // wide windows (open search) are cut into at most ~16 items per group;
    // the groups dispensed last take shorter items (the last quarter 1/4,
    // the last sixteenth 1/16 of the chunk), so the grid ends evenly
    const uint32_t ng = grp_start[kClasses];
    const int32_t cg = (uint32_t)g >= ng - ng / 16 ? max(chunk / 16, 256)
                       : (uint32_t)g >= ng - ng / 4 ? max(chunk / 4, 256)
                                                    : chunk;
    gi.chunk = group_chunk(gi.hi - gi.lo, cg);
    groups[g] = gi;
    nchunks[g] = (gi.hi - gi.lo + gi.chunk - 1) / gi.chunk;
}

template <bool FastDiv, typename T, int G>
__global__ void __launch_bounds__(768, 1)
k_score_batched(DevDB db, const T *__restrict__ tiles, int64_t stride, const uint32_t *__restrict__ wb,
                const uint32_t *__restrict__ we, const int32_t *__restrict__ perm,
                const GroupInfo *__restrict__ groups, const uint32_t *__restrict__ item_off,
                const uint32_t *__restrict__ ngroups_p, int32_t chunk, int32_t K, uint32_t *__restrict__ counter,
                float *__restrict__ part_s, uint64_t *__restrict__ part_k, uint32_t *__restrict__ err) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int32_t words_cap = (int32_t)((stride + 31) / 32);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    T *stile = reinterpret_cast<T *>(smem + 128);
    constexpr size_t kQueue = CtaSlots<G>::warp_bytes();
    uint8_t *wbase = smem + 128 + fused_tile_bytes(stride, sizeof(T), G) +
                     (size_t)warp * fused_warp_bytes(words_cap, kQueue);
    uint8_t *my_queue = wbase + fused_queue_offset(words_cap);
    uint32_t *planes = reinterpret_cast<uint32_t *>(wbase);
    uint16_t *list = reinterpret_cast<uint16_t *>(planes + 3 * words_cap);
    __shared__ int32_t s_item;
    __shared__ uint32_t s_next;
    __shared__ uint32_t s_wb[G], s_we[G];
    __shared__ uint32_t thr_u[G], s_lock[G];
    __shared__ float s_ls[G * 32];
    __shared__ uint32_t s_lk[G * 32];

    const int32_t ngroups = (int32_t)*ngroups_p;
    const uint32_t total = item_off[ngroups];
    if (threadIdx.x == 0) mbar_init(bar, 1);
    for (int32_t i = lane; i < 3 * words_cap; i += 32) planes[i] = 0u;
    __syncthreads();
    const Planes pl{planes, planes + words_cap, planes + 2 * words_cap};
    const float mt_lane = db.mt[lane];
    const int my_slot = reduce_slot_of_lane<G>(lane);
    uint32_t phase = 0;
    CtaSlots<G> slots;
    slots.bind(s_ls, s_lk, s_lock, thr_u, my_queue, err);

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
            if (j < cnt_members) {
                const int32_t s = perm[gi.pos0 + j];
                b = wb[s];
                e = we[s];
            }
            s_wb[j] = b;
            s_we[j] = e;
        }
        slots.reset_shared();
        if (threadIdx.x == 0) s_next = p0;
        const int32_t nb = tile_bins(gi.maxlen);
        if (threadIdx.x == 0) {
            fence_proxy_async();
            const uint32_t bytes = (uint32_t)((size_t)nb * G * sizeof(T));
            mbar_arrive_expect_tx(bar, bytes);
            bulk_g2s(stile, tiles + (size_t)g * stride * G, bytes, bar);
        }
        __syncthreads();
        if (!mbar_wait(bar, phase, kWaitLimit)) {
            if (threadIdx.x == 0) atomicOr(err, kErrTimeout);
            return;
        }
        phase ^= 1u;
        const uint32_t my_b = lane < G ? s_wb[lane] : 0u, my_e = lane < G ? s_we[lane] : 0u;
        const TileDot<T, G> dot{stile};
        while (true) {
            // candidates are handed out one at a time so that warps finish together
            uint32_t p = 0;
            if (lane == 0) p = atomicAdd(&s_next, 1u);
            p = __shfl_sync(kFullMask, p, 0);
            if (p >= p1) break;
            const uint32_t act = __ballot_sync(kFullMask, lane < G && my_b <= p && p < my_e) & ((1u << G) - 1u);
            if (!act) continue;
            const WordRange wr = build_planes<FastDiv>(pl, db.ions, db.tc_sorted[p], db.tn_sorted[p],
                                                       db.r_sorted[p], (int)gi.charges, gi.maxlen, mt_lane,
                                                       NoMods{});
            float acc[G];
            planes_accumulate<G>(pl, list, wr, dot, acc);
            const float sc = reduce_scatter<G>(acc);
            const bool want = (lane & (32 / G - 1)) == 0 && ((act >> my_slot) & 1u) &&
                              score_order(sc) >= *(volatile uint32_t *)(thr_u + my_slot);
            slots.offer(want, sc, p, my_slot, K);
        }
        slots.drain(K);
        __syncthreads();  // every warp has merged its queues
        for (int j = warp; j < cnt_members; j += nw) {
            const size_t o = ((size_t)item * G + j) * K;
            slots.result(j, K, part_s + o, part_k + o);
        }
        __syncthreads();
    }
}

// Per spectrum: merge its slot of every item of its group.
// R = 1: up to 32 kept per spectrum (WarpTopK), R = 2: up to 64 (WarpTopK64).
template <int R>
__global__ void k_merge_items(const float *__restrict__ part_s, const uint64_t *__restrict__ part_k,
                              const uint32_t *__restrict__ item_off, const int32_t *__restrict__ group_of,
                              const int32_t *__restrict__ slot_of, const SpecMeta *__restrict__ meta, int32_t nspec,
                              int32_t G, int32_t K, int32_t kout, float *__restrict__ out_s,
                              uint64_t *__restrict__ out_k) {
    const int lane = threadIdx.x & 31;
    const int32_t s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= nspec) return;
    typename std::conditional<R == 1, WarpTopK, WarpTopK64>::type tk;
    tk.init();
    if (meta[s].status == 0) {
        const int32_t g = group_of[s], j = slot_of[s];
        for (uint32_t it = item_off[g]; it < item_off[g + 1]; ++it) {
            const size_t o = ((size_t)it * G + j) * K;
            bool done = false;
            for (int r = 0; r < R && !done; ++r) {
                const int i = 32 * r + lane;
                const float sc = i < K ? part_s[o + i] : -INFINITY;
                const uint64_t kk = i < K ? part_k[o + i] : ~0ull;
                for (int t = 0; t < 32 && 32 * r + t < K; ++t) {
                    const float ts = __shfl_sync(kFullMask, sc, t);
                    const uint64_t tk2 = __shfl_sync(kFullMask, kk, t);
                    if (tk2 == ~0ull) {
                        done = true;  // the item's list ends here
                        break;
                    }
                    tk.insert(ts, tk2, kout);
                }
            }
        }
    }
    if constexpr (R == 1) {
        if (lane < kout) {
            out_s[(size_t)s * kout + lane] = tk.s;
            out_k[(size_t)s * kout + lane] = tk.k;
        }
    } else {
        if (lane < kout) {
            out_s[(size_t)s * kout + lane] = tk.s0;
            out_k[(size_t)s * kout + lane] = tk.k0;
        }
        if (32 + lane < kout) {
            out_s[(size_t)s * kout + 32 + lane] = tk.s1;
            out_k[(size_t)s * kout + 32 + lane] = tk.k1;
        }
    }
}

// FP32 rescoring of the kept candidates (BF16/FP16-stored rows): one CTA
// per spectrum, each warp recomputes kept entries from the FP32 row, then
// the CTA orders them and writes the top-N.
template <bool FastDiv>
__global__ void __launch_bounds__(256) k_rescore(DevDB db, DevMods mods, const float *__restrict__ rows32,
                                                 int64_t stride, const SpecMeta *__restrict__ meta,
                                                 const float *__restrict__ kept_s,
                                                 const uint64_t *__restrict__ kept_k, int32_t K, int32_t topn,
                                                 float *__restrict__ out_s, uint64_t *__restrict__ out_k,
                                                 uint32_t *__restrict__ out_pep) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int32_t s = blockIdx.x;
    const SpecMeta m = meta[s];
    const int32_t words = (int32_t)((stride + 31) / 32);
    uint32_t *planes = reinterpret_cast<uint32_t *>(smem);
    uint16_t *lists = reinterpret_cast<uint16_t *>(planes + (size_t)nw * 3 * words);
    float *res_s = reinterpret_cast<float *>(lists + (size_t)nw * kListCap);
    uint64_t *res_k = reinterpret_cast<uint64_t *>(res_s + 64);
    for (int32_t i = threadIdx.x; i < nw * 3 * words; i += blockDim.x) planes[i] = 0u;
    __syncthreads();
    Planes pl{planes + (size_t)warp * 3 * words, planes + (size_t)warp * 3 * words + words,
              planes + (size_t)warp * 3 * words + 2 * words};
    uint16_t *list = lists + (size_t)warp * kListCap;
    const float mt_lane = db.mt[lane];
    SpecSet<float, 1> ss;
    ss.row[0] = rows32 + (size_t)s * stride;
    ss.len[0] = m.len;
    ss.active = 1u;
    for (int t = warp; t < K; t += nw) {
        const uint64_t kk = kept_k[(size_t)s * K + t];
        float sc = -INFINITY;
        if (kk != ~0ull && !(kk >> 63)) {
            const uint32_t p = (uint32_t)kk;
            const WordRange wr = build_planes<FastDiv>(pl, db.ions, db.tc_sorted[p], db.tn_sorted[p],
                                                       db.r_sorted[p], m.charges_plain, m.len, mt_lane, NoMods{});
            float acc[1];
            planes_dot<float, 1>(pl, list, wr, ss, acc);
            sc = acc[0];
        } else if (kk != ~0ull) {
            // modified match: combination, mass-order position and isoform rank from the key
            const int32_t mu = (int32_t)((kk >> 54) & 511u);
            const uint32_t p = (uint32_t)((kk >> 27) & ((1u << 27) - 1u));
            const uint32_t rank = (uint32_t)(kk & ((1u << 27) - 1u));
            const uint32_t tc = db.tc_sorted[p], tn = db.tn_sorted[p];
            const int32_t *dcount = mods.counts + (size_t)mu * mods.num_ma;
            uint32_t D[kMaxMa], scan[kMaxMa];
            modable_counts(db.ions, tc, tn, mods.num_ma, D);
            isoform_count(D, dcount, mods.num_ma, scan);
            ModIsoform iso;
            iso.num_ma = mods.num_ma;
            iso.per_type = mods.per_type;
#pragma unroll
            for (int i = 0; i < kMaxMa; ++i) iso.ma_mass[i] = mods.ma_mass[i];
            isoform_masks(D, scan, dcount, mods.num_ma, rank, iso.mask);
            iso.reset();
            const float residual = __fadd_rn(db.r_sorted[p], mods.delta[mu]);
            const WordRange wr = build_planes<FastDiv>(pl, db.ions, tc, tn, residual, m.charges_mod, m.len, mt_lane,
                                                       iso);
            float acc[1];
            planes_dot<float, 1>(pl, list, wr, ss, acc);
            sc = acc[0];
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
            const uint64_t pos = (tk.k >> 63) ? ((tk.k >> 27) & ((1ull << 27) - 1)) : tk.k;
            out_pep[(size_t)s * topn + lane] = (tk.k != ~0ull) ? db.idx_sorted[pos] : ~0u;
        }
    }
}

__global__ void k_finish(const float *__restrict__ in_s, const uint64_t *__restrict__ in_k, int32_t nspec,
                         int32_t topn, const uint32_t *__restrict__ idx_sorted, const uint32_t *__restrict__ wb,
                         const uint32_t *__restrict__ we, const SpecMeta *__restrict__ meta, float *__restrict__ out_s,
                         uint64_t *__restrict__ out_k, uint32_t *__restrict__ out_pep, int32_t plain,
                         const unsigned long long *__restrict__ ncand_mod, int64_t *__restrict__ ncand) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (int64_t)nspec * topn) {
        const uint64_t k = in_k[i];
        out_s[i] = in_s[i];
        out_k[i] = k;
        uint32_t pep = ~0u;
        if (k != ~0ull) {
            const uint64_t pos = (k >> 63) ? ((k >> 27) & ((1ull << 27) - 1)) : k;
            pep = idx_sorted[pos];
        }
        out_pep[i] = pep;
    }
    if (ncand && i < nspec)
        ncand[i] = ((meta[i].status == 0 && plain) ? (int64_t)(we[i] - wb[i]) : 0) +
                   (ncand_mod ? (int64_t)ncand_mod[i] : 0);
}

__global__ void k_ncand(const uint32_t *__restrict__ wb, const uint32_t *__restrict__ we,
                        const SpecMeta *__restrict__ meta, int32_t nspec, int32_t plain,
                        const unsigned long long *__restrict__ ncand_mod, int64_t *__restrict__ ncand) {
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nspec)
        ncand[i] = ((meta[i].status == 0 && plain) ? (int64_t)(we[i] - wb[i]) : 0) +
                   (ncand_mod ? (int64_t)ncand_mod[i] : 0);
}

}  // namespace hfx

using namespace hfx;

size_t hfx_batched_smem(int64_t stride, int elem_bytes, int G, int nw, int K) {
    (void)K;
    return fused_smem_bytes(stride, elem_bytes, G, nw, cta_queue_bytes(G, 4));
}

int hfx_batched_plan(const SpecMeta *meta, int32_t nspec, const uint32_t *wb, const uint32_t *we, int32_t G,
                     int32_t chunk, const BatchedWs &ws, cudaStream_t st) {
    const int nbk = kClasses * kMassBuckets;
    cudaMemsetAsync(ws.hist, 0, sizeof(uint32_t) * (nbk + 1), st);
    cudaMemsetAsync(ws.item_off, 0, sizeof(uint32_t) * (nspec + 1), st);
    k_bucket_count<<<(nspec + 255) / 256, 256, 0, st>>>(meta, nspec, ws.hist);
    k_scan_u32<<<1, 1024, 0, st>>>(ws.hist, nbk, ws.n_sorted);
    cudaMemcpyAsync(ws.cursor, ws.hist, sizeof(uint32_t) * nbk, cudaMemcpyDeviceToDevice, st);
    k_bucket_scatter<<<(nspec + 255) / 256, 256, 0, st>>>(meta, nspec, ws.cursor, ws.perm);
    const int32_t max_groups = nspec;  // each class adds at most one partial group
    k_groups<<<(max_groups + 255) / 256, 256, 0, st>>>(ws.hist, ws.n_sorted, ws.perm, wb, we, meta, G, chunk,
                                                       max_groups, ws.groups, ws.item_off, ws.group_of, ws.slot_of,
                                                       ws.ngroups);
    k_scan_u32<<<1, 1024, 0, st>>>(ws.item_off, max_groups + 1, ws.total_items);
    return (int)cudaGetLastError();
}

template <bool F, typename T, int G>
static int launch_batched_t(const DevDB &db, const T *rows, int64_t stride, const SpecMeta *meta, const uint32_t *wb,
                            const uint32_t *we, const BatchedWs &ws, void *tiles, uint32_t ngroups, int32_t chunk,
                            int32_t K, int nw, int grid, float *part_s, uint64_t *part_k, uint32_t *err,
                            cudaStream_t st) {
    (void)rows;
    int dev = 0, sms = 0, smem_max = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    auto fn = k_score_batched<F, T, G>;
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, fn);  // static shared memory counts against the same limit
    const size_t avail = (size_t)smem_max > fa.sharedSizeBytes ? (size_t)smem_max - fa.sharedSizeBytes : 0;
    if (nw <= 0) nw = std::min(fused_warps(stride, sizeof(T), G, cta_queue_bytes(G, 4), avail), 24);
    if (nw < 1) return (int)cudaErrorInvalidValue;
    const size_t smem = hfx_batched_smem(stride, sizeof(T), G, nw, K);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    if (grid <= 0) {
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, nw * 32, smem);
        grid = sms * (per > 0 ? per : 1);
    }
    fn<<<grid, nw * 32, smem, st>>>(db, (const T *)tiles, stride, wb, we, ws.perm, ws.groups, ws.item_off,
                                    ws.ngroups, chunk, K, ws.counter, part_s, part_k, err);
    return (int)cudaGetLastError();
}

template <bool F, typename T>
static int launch_batched_g(int G, const DevDB &db, const T *rows, int64_t stride, const SpecMeta *meta,
                            const uint32_t *wb, const uint32_t *we, const BatchedWs &ws, void *tiles, uint32_t ng,
                            int32_t chunk, int32_t K, int nw, int grid, float *ps, uint64_t *pk, uint32_t *err,
                            cudaStream_t st) {
    switch (G) {
    case 1: return launch_batched_t<F, T, 1>(db, rows, stride, meta, wb, we, ws, tiles, ng, chunk, K, nw, grid, ps, pk, err, st);
    case 2: return launch_batched_t<F, T, 2>(db, rows, stride, meta, wb, we, ws, tiles, ng, chunk, K, nw, grid, ps, pk, err, st);
    case 4: return launch_batched_t<F, T, 4>(db, rows, stride, meta, wb, we, ws, tiles, ng, chunk, K, nw, grid, ps, pk, err, st);
    case 8: return launch_batched_t<F, T, 8>(db, rows, stride, meta, wb, we, ws, tiles, ng, chunk, K, nw, grid, ps, pk, err, st);
    default: return (int)cudaErrorInvalidValue;
    }
}

int hfx_batched_score(const DevDB &db, const void *rows, int elem_kind, int64_t stride, const SpecMeta *meta,
                      const uint32_t *wb, const uint32_t *we, const BatchedWs &ws, void *tiles, uint32_t ngroups,
                      int32_t G, int32_t chunk, int32_t K, int nw, int grid, int fastdiv, float *part_s,
                      uint64_t *part_k, uint32_t *err, cudaStream_t st) {
    cudaMemsetAsync(ws.counter, 0, 4, st);
    if (elem_kind == 0) {
        const float *r = (const float *)rows;
        return fastdiv ? launch_batched_g<true, float>(G, db, r, stride, meta, wb, we, ws, tiles, ngroups, chunk, K,
                                                       nw, grid, part_s, part_k, err, st)
                       : launch_batched_g<false, float>(G, db, r, stride, meta, wb, we, ws, tiles, ngroups, chunk, K,
                                                        nw, grid, part_s, part_k, err, st);
    } else if (elem_kind == 1) {
        const __nv_bfloat16 *r = (const __nv_bfloat16 *)rows;
        return fastdiv ? launch_batched_g<true, __nv_bfloat16>(G, db, r, stride, meta, wb, we, ws, tiles, ngroups,
                                                               chunk, K, nw, grid, part_s, part_k, err, st)
                       : launch_batched_g<false, __nv_bfloat16>(G, db, r, stride, meta, wb, we, ws, tiles, ngroups,
                                                                chunk, K, nw, grid, part_s, part_k, err, st);
    } else {
        const __half *r = (const __half *)rows;
        return fastdiv ? launch_batched_g<true, __half>(G, db, r, stride, meta, wb, we, ws, tiles, ngroups, chunk, K,
                                                        nw, grid, part_s, part_k, err, st)
                       : launch_batched_g<false, __half>(G, db, r, stride, meta, wb, we, ws, tiles, ngroups, chunk,
                                                         K, nw, grid, part_s, part_k, err, st);
    }
}

// Graph replays size the work-item buffers from an earlier run: clamp the
// item offsets to that capacity and report an overflow (the host re-plans).
__global__ void k_clamp_items(uint32_t *__restrict__ off, int64_t n1, uint32_t cap, uint32_t *__restrict__ err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n1) return;
    const uint32_t v = off[i];
    if (v > cap) {
        off[i] = cap;
        if (i == n1 - 1) atomicOr(err, kErrBounds);
    }
}

__global__ void k_clamp_groups(uint32_t *__restrict__ ngroups, uint32_t cap, uint32_t *__restrict__ err) {
    if (threadIdx.x == 0 && *ngroups > cap) {
        *ngroups = cap;
        atomicOr(err, kErrBounds);
    }
}

int hfx_clamp_groups(uint32_t *ngroups, uint32_t cap, uint32_t *err, cudaStream_t st) {
    k_clamp_groups<<<1, 32, 0, st>>>(ngroups, cap, err);
    return (int)cudaGetLastError();
}

int hfx_clamp_items(uint32_t *off, int64_t n1, uint32_t cap, uint32_t *err, cudaStream_t st) {
    if (n1 <= 0) return 0;
    k_clamp_items<<<(unsigned)((n1 + 255) / 256), 256, 0, st>>>(off, n1, cap, err);
    return (int)cudaGetLastError();
}

int hfx_batched_merge(const float *part_s, const uint64_t *part_k, const BatchedWs &ws, const SpecMeta *meta,
                      int32_t nspec, int32_t G, int32_t K, int32_t kout, float *out_s, uint64_t *out_k,
                      cudaStream_t st) {
    if (kout > kMaxKept || K > kMaxKept) return (int)cudaErrorInvalidValue;
    if (kout > 32 || K > 32)
        k_merge_items<2><<<(nspec + 3) / 4, 128, 0, st>>>(part_s, part_k, ws.item_off, ws.group_of, ws.slot_of, meta,
                                                          nspec, G, K, kout, out_s, out_k);
    else
        k_merge_items<1><<<(nspec + 3) / 4, 128, 0, st>>>(part_s, part_k, ws.item_off, ws.group_of, ws.slot_of, meta,
                                                          nspec, G, K, kout, out_s, out_k);
    return (int)cudaGetLastError();
}

int hfx_rescore(const DevDB &db, const DevMods &mods, const float *rows32, int64_t stride, const SpecMeta *meta,
                const float *kept_s,
                const uint64_t *kept_k, int32_t nspec, int32_t K, int32_t topn, int fastdiv, float *out_s,
                uint64_t *out_k, uint32_t *out_pep, cudaStream_t st) {
    const int nw = 8;
    const int32_t words = (int32_t)((stride + 31) / 32);
    const size_t smem = (size_t)nw * 3 * words * 4 + (size_t)nw * kListCap * 2 + 64 * 4 + 64 * 8;
    auto f = fastdiv ? k_rescore<true> : k_rescore<false>;
    cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    f<<<nspec, nw * 32, smem, st>>>(db, mods, rows32, stride, meta, kept_s, kept_k, K, topn, out_s, out_k, out_pep);
    return (int)cudaGetLastError();
}

int hfx_finish(const float *in_s, const uint64_t *in_k, int32_t nspec, int32_t topn, const uint32_t *idx_sorted,
               const uint32_t *wb, const uint32_t *we, const SpecMeta *meta, float *out_s, uint64_t *out_k,
               uint32_t *out_pep, int32_t plain, const unsigned long long *ncand_mod, int64_t *ncand,
               cudaStream_t st) {
    const int64_t n = std::max<int64_t>((int64_t)nspec * topn, nspec);
    k_finish<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in_s, in_k, nspec, topn, idx_sorted, wb, we, meta, out_s,
                                                          out_k, out_pep, plain, ncand_mod, ncand);
    return (int)cudaGetLastError();
}

int hfx_ncand(const uint32_t *wb, const uint32_t *we, const SpecMeta *meta, int32_t nspec, int32_t plain,
              const unsigned long long *ncand_mod, int64_t *ncand, cudaStream_t st) {
    k_ncand<<<(nspec + 255) / 256, 256, 0, st>>>(wb, we, meta, nspec, plain, ncand_mod, ncand);
    return (int)cudaGetLastError();
}

template <typename T>
static int pack_tiles_g(int32_t G, const void *rows, int64_t stride, const SpecMeta *meta, const BatchedWs &ws,
                        void *tiles, uint32_t ngroups, cudaStream_t st) {
    if (ngroups == 0) return 0;
    const T *r = (const T *)rows;
    if (G == 16) hfx_pack_tiles_launch<T, 16>(r, stride, meta, ws, (T *)tiles, ngroups, st);
    else if (G == 8) hfx_pack_tiles_launch<T, 8>(r, stride, meta, ws, (T *)tiles, ngroups, st);
    else if (G == 4) hfx_pack_tiles_launch<T, 4>(r, stride, meta, ws, (T *)tiles, ngroups, st);
    else if (G == 2) hfx_pack_tiles_launch<T, 2>(r, stride, meta, ws, (T *)tiles, ngroups, st);
    else if (G == 1) hfx_pack_tiles_launch<T, 1>(r, stride, meta, ws, (T *)tiles, ngroups, st);
    else return (int)cudaErrorInvalidValue;
    return (int)cudaGetLastError();
}

int hfx_pack_tiles(const void *rows, int elem_kind, int64_t stride, const SpecMeta *meta, const BatchedWs &ws,
                   void *tiles, uint32_t ngroups, int32_t G, cudaStream_t st) {
    if (elem_kind == 0) return pack_tiles_g<float>(G, rows, stride, meta, ws, tiles, ngroups, st);
    if (elem_kind == 1) return pack_tiles_g<__nv_bfloat16>(G, rows, stride, meta, ws, tiles, ngroups, st);
    return pack_tiles_g<__half>(G, rows, stride, meta, ws, tiles, ngroups, st);
}
