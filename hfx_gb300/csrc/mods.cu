// Stage (e): variable-modification search on the device.
//
// The reference enumerates modified candidates per spectrum on the host
// side of the FFI in five steps -- per-combination windows (filter_by_mod.cu:
// 35-143), modable filter and compaction (:145-378), isoform counts
// (calc_mod_cands.cu), expansion (prepare_gen_mod.cu) and unranking
// (gen_mod_pep.cu) -- then scores every isoform with a dense theoretical row
// (mion_series.cu) and cuBLAS sgemv.  Here the same enumeration is fused into
// the batched scorer: a work item is (spectrum group, combination, chunk of
// the group's union window for that combination); a warp takes one
// candidate, counts its modable acids, and for each isoform rank unranks the
// modified residues, builds the modified ion list (residual + delta,
// residue mass + acid delta) and gathers it against every member spectrum
// whose combination window contains the candidate.  Modified matches use
// the key (1<<63 | combination<<54 | position<<27 | rank), which orders ties
// exactly as the reference's merge (Search.hs:119-123).
#include "hfx_internal.h"
#include "device_common.cuh"
#include "batched.h"
#include "batched_common.cuh"
#include "mods_device.cuh"
#include "mods.h"
#include "lists.h"
#include <algorithm>

namespace hfx {

// Warps per CTA of the modification scorer: the isoform state (masks, counts,
// suffix products) needs ~120 registers per thread.
constexpr int kModWarps = 16;

// filter_by_mod.cu:72-80: lower_bound((m - eps) - delta), upper_bound((m + eps) - delta)
__global__ void k_mod_windows(const float *__restrict__ r_sorted, uint32_t n, const SpecMeta *__restrict__ meta,
                              int32_t nspec, const float *__restrict__ delta, int32_t num_mod,
                              uint32_t *__restrict__ mb, uint32_t *__restrict__ me) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)nspec * num_mod) return;
    const int32_t s = (int32_t)(t / num_mod), mu = (int32_t)(t % num_mod);
    const SpecMeta m = meta[s];
    uint32_t b = 0, e = 0;
    // spectra whose charge gives no modified ion charges (mion_series.cu:425-438)
    // still enumerate their isoforms, each with an empty ion list (score 0)
    if (m.status == 0) {
        const float lo = __fsub_rn(m.lo, delta[mu]), hi = __fsub_rn(m.hi, delta[mu]);
        uint32_t a = 0, z = n;
        while (a < z) { const uint32_t c = (a + z) >> 1; if (r_sorted[c] < lo) a = c + 1; else z = c; }
        b = a;
        a = 0; z = n;
        while (a < z) { const uint32_t c = (a + z) >> 1; if (hi < r_sorted[c]) z = c; else a = c + 1; }
        e = a < b ? b : a;
    }
    mb[t] = b;
    me[t] = e;
}

// One thread per (group, combination): the union of the members' windows
// for that combination, in chunks.
__global__ void k_mod_groups(const GroupInfo *__restrict__ groups, const uint32_t *__restrict__ ngroups_p,
                             const int32_t *__restrict__ perm, const uint32_t *__restrict__ mb,
                             const uint32_t *__restrict__ me, int32_t num_mod, int32_t chunk, int32_t max_gm,
                             uint32_t *__restrict__ mlo, uint32_t *__restrict__ mhi, uint32_t *__restrict__ mchunk,
                             int32_t *__restrict__ nchunks) {
    const int32_t gm = blockIdx.x * blockDim.x + threadIdx.x;
    if (gm >= max_gm) return;
    const uint32_t ng = *ngroups_p;
    const int32_t g = gm / num_mod, mu = gm % num_mod;
    uint32_t lo = 0xFFFFFFFFu, hi = 0u;
    if ((uint32_t)g < ng) {
        const GroupInfo gi = groups[g];
        for (uint32_t j = 0; j < gi.count; ++j) {
            const int32_t s = perm[gi.pos0 + j];
            const uint32_t b = mb[(size_t)s * num_mod + mu], e = me[(size_t)s * num_mod + mu];
            if (e > b) {
                lo = min(lo, b);
                hi = max(hi, e);
            }
        }
    }
    if (hi <= lo) lo = hi = 0u;
    const uint32_t c = group_chunk(hi - lo, chunk);
    mlo[gm] = lo;
    mhi[gm] = hi;
    mchunk[gm] = c;
    nchunks[gm] = (int32_t)((hi - lo + c - 1) / c);
}

template <bool FastDiv, typename T, int G>
__global__ void __launch_bounds__(kModWarps * 32, 1)
k_score_mods(DevDB db, DevMods mods, const T *__restrict__ tiles, int64_t stride, const uint32_t *__restrict__ mb,
             const uint32_t *__restrict__ me, const int32_t *__restrict__ perm,
             const GroupInfo *__restrict__ groups, const uint32_t *__restrict__ mlo, const uint32_t *__restrict__ mhi,
             const uint32_t *__restrict__ mchunk, const uint32_t *__restrict__ item_off, int32_t n_gm, int32_t K,
             uint32_t *__restrict__ counter, float *__restrict__ part_s, uint64_t *__restrict__ part_k,
             unsigned long long *__restrict__ ncand, float *__restrict__ sink, unsigned long long *__restrict__ cursor,
             const uint64_t *__restrict__ sink_end, uint32_t *__restrict__ err) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int32_t words_cap = (int32_t)((stride + 31) / 32);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    T *stile = reinterpret_cast<T *>(smem + 128);
    constexpr size_t kQueue = CtaSlots<G, uint64_t>::warp_bytes();
    uint8_t *wbase = smem + 128 + fused_tile_bytes(stride, sizeof(T), G) +
                     (size_t)warp * fused_warp_bytes(words_cap, kQueue);
    uint8_t *my_queue = wbase + fused_queue_offset(words_cap);
    uint32_t *planes = reinterpret_cast<uint32_t *>(wbase);
    uint16_t *list = reinterpret_cast<uint16_t *>(planes + 3 * words_cap);
    __shared__ int32_t s_item;
    __shared__ uint32_t s_next;
    __shared__ uint32_t s_wb[G], s_we[G];
    __shared__ int32_t s_spec[G];
    __shared__ uint32_t thr_u[G], s_lock[G];
    __shared__ float s_ls[G * 32];
    __shared__ uint64_t s_lk[G * 32];

    const uint32_t total = item_off[n_gm];
    if (threadIdx.x == 0) mbar_init(bar, 1);
    for (int32_t i = lane; i < 3 * words_cap; i += 32) planes[i] = 0u;
    __syncthreads();
    const Planes pl{planes, planes + words_cap, planes + 2 * words_cap};
    const float mt_lane = db.mt[lane];
    const int my_slot = reduce_slot_of_lane<G>(lane);
    uint32_t phase = 0;
    ModIsoform iso;
    iso.num_ma = mods.num_ma;
    iso.per_type = mods.per_type;
#pragma unroll
    for (int i = 0; i < kMaxMa; ++i) iso.ma_mass[i] = mods.ma_mass[i];
    CtaSlots<G, uint64_t> slots;
    slots.bind(s_ls, s_lk, s_lock, thr_u, my_queue, err);

    while (true) {
        if (threadIdx.x == 0) s_item = (int32_t)atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t item = (uint32_t)s_item;
        if (item >= total) break;
        const int32_t gm = find_group(item_off, n_gm, item);
        const int32_t g = gm / mods.num_mod, mu = gm % mods.num_mod;
        const GroupInfo gi = groups[g];
        const uint32_t p0 = mlo[gm] + (item - item_off[gm]) * mchunk[gm];
        const uint32_t p1 = min(mhi[gm], p0 + mchunk[gm]);
        const int cnt_members = (int)gi.count;
        if (threadIdx.x < G) {
            const int j = threadIdx.x;
            uint32_t b = 0, e = 0;
            int32_t s = -1;
            if (j < cnt_members) {
                s = perm[gi.pos0 + j];
                b = mb[(size_t)s * mods.num_mod + mu];
                e = me[(size_t)s * mods.num_mod + mu];
            }
            s_wb[j] = b;
            s_we[j] = e;
            s_spec[j] = s;
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
        const int32_t *dcount = mods.counts + (size_t)mu * mods.num_ma;
        const float delta = mods.delta[mu];
        while (true) {
            uint32_t p = 0;
            if (lane == 0) p = atomicAdd(&s_next, 1u);
            p = __shfl_sync(kFullMask, p, 0);
            if (p >= p1) break;
            const uint32_t act = __ballot_sync(kFullMask, lane < G && my_b <= p && p < my_e) & ((1u << G) - 1u);
            if (!act) continue;
            const uint32_t tc = db.tc_sorted[p], tn = db.tn_sorted[p];
            uint32_t D[kMaxMa];
            modable_counts(db.ions, tc, tn, mods.num_ma, D);
            bool modable = true;
#pragma unroll
            for (int i = 0; i < kMaxMa; ++i)  // filter_by_mod.cu:251-261
                if (i < mods.num_ma) modable &= D[i] >= (uint32_t)dcount[i];
            if (!modable) continue;
            uint32_t scan[kMaxMa];
            const uint32_t niso = isoform_count(D, dcount, mods.num_ma, scan);
            // candidates counted per member spectrum: one per isoform
            if (ncand && lane < G && ((act >> lane) & 1u) && niso)
                atomicAdd(ncand + s_spec[lane], (unsigned long long)niso);
            // score sink (E-values): niso consecutive entries of the member's
            // segment, claimed at once; the fit reads them as a multiset
            unsigned long long sbase = ~0ull;
            if (sink) {
                if (lane < G && ((act >> lane) & 1u) && niso) {
                    const int32_t s = s_spec[lane];
                    const unsigned long long b0 = atomicAdd(cursor + s, (unsigned long long)niso);
                    if (b0 + niso <= sink_end[s]) sbase = b0;
                    else atomicOr(err, kErrBounds);
                }
                sbase = __shfl_sync(kFullMask, sbase, my_slot);
            }
            // mion_series.cu:226: residual + delta
            const float residual = __fadd_rn(db.r_sorted[p], delta);
            for (uint32_t rank = 0; rank < niso; ++rank) {
                if (p >= (1u << 27) || rank >= (1u << 27)) {
                    if (lane == 0) atomicOr(err, kErrKeyOverflow);
                    break;
                }
                if (!isoform_masks(D, scan, dcount, mods.num_ma, rank, iso.mask)) {
                    if (lane == 0) atomicOr(err, kErrKeyOverflow);
                }
                iso.reset();
                const WordRange wr = build_planes<FastDiv>(pl, db.ions, tc, tn, residual, (int)gi.charges_mod,
                                                           gi.maxlen, mt_lane, iso);
                float acc[G];
                planes_accumulate<G>(pl, list, wr, dot, acc);
                const float sc = reduce_scatter<G>(acc);
                if (sbase != ~0ull && (lane & (32 / G - 1)) == 0 && ((act >> my_slot) & 1u)) sink[sbase + rank] = sc;
                const bool want = (lane & (32 / G - 1)) == 0 && ((act >> my_slot) & 1u) &&
                                  score_order(sc) >= *(volatile uint32_t *)(thr_u + my_slot);
                slots.offer(want, sc, mod_key(mu, p, rank), my_slot, K);
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
}

// Per spectrum: merge its slot of the unmodified items of its group and of
// the modified items of every (group, combination).
__global__ void k_merge_with_mods(const float *__restrict__ ps, const uint64_t *__restrict__ pk,
                                  const uint32_t *__restrict__ item_off, const float *__restrict__ ms,
                                  const uint64_t *__restrict__ mk, const uint32_t *__restrict__ mitem_off,
                                  int32_t num_mod, const int32_t *__restrict__ group_of,
                                  const int32_t *__restrict__ slot_of, const SpecMeta *__restrict__ meta,
                                  int32_t nspec, int32_t G, int32_t K, int32_t plain, float *__restrict__ out_s,
                                  uint64_t *__restrict__ out_k) {
    const int lane = threadIdx.x & 31;
    const int32_t s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= nspec) return;
    WarpTopK tk;
    tk.init();
    if (meta[s].status == 0) {
        const int32_t g = group_of[s], j = slot_of[s];
        for (int pass = 0; pass < 2; ++pass) {
            const float *sp = pass ? ms : ps;
            const uint64_t *kp = pass ? mk : pk;
            uint32_t a, b;
            if (pass == 0) {
                if (!plain) continue;
                a = item_off[g];
                b = item_off[g + 1];
            } else {
                if (num_mod <= 0) continue;
                a = mitem_off[(size_t)g * num_mod];
                b = mitem_off[(size_t)(g + 1) * num_mod];
            }
            for (uint32_t it = a; it < b; ++it) {
                const size_t o = ((size_t)it * G + j) * K;
                const float sc = lane < K ? sp[o + lane] : -INFINITY;
                const uint64_t kk = lane < K ? kp[o + lane] : ~0ull;
                const int nvalid = __popc(__ballot_sync(kFullMask, kk != ~0ull));
                for (int t = 0; t < nvalid; ++t)
                    tk.insert(__shfl_sync(kFullMask, sc, t), __shfl_sync(kFullMask, kk, t), K);
            }
        }
    }
    if (lane < K) {
        out_s[(size_t)s * K + lane] = tk.s;
        out_k[(size_t)s * K + lane] = tk.k;
    }
}

// Isoform export for parity checks: for queries (mass-order position,
// combination, rank): isoform count, and for rank < count the unrank row
// (occurrence indices per acid, ascending acid order, each acid's values in
// unrankComb order) and the per-residue modified flags.
__global__ void k_mod_isoforms(DevDB db, DevMods mods, const uint32_t *__restrict__ pos,
                               const int32_t *__restrict__ mu_q, const uint32_t *__restrict__ rank_q, int32_t n,
                               int32_t cap, uint32_t *__restrict__ out_count, uint32_t *__restrict__ out_unrank,
                               uint8_t *__restrict__ out_modded) {
    const int lane = threadIdx.x & 31;
    const int32_t q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (q >= n) return;
    const uint32_t p = pos[q];
    const int32_t mu = mu_q[q];
    const int32_t *dcount = mods.counts + (size_t)mu * mods.num_ma;
    const uint32_t tc = db.tc_sorted[p], tn = db.tn_sorted[p];
    uint32_t D[kMaxMa];
    modable_counts(db.ions, tc, tn, mods.num_ma, D);
    bool modable = true;
    for (int i = 0; i < mods.num_ma; ++i) modable &= D[i] >= (uint32_t)dcount[i];
    uint32_t scan[kMaxMa];
    const uint32_t niso = modable ? isoform_count(D, dcount, mods.num_ma, scan) : 0u;
    if (lane == 0) out_count[q] = niso;
    const uint32_t rank = rank_q[q];
    if (rank >= niso) return;
    // unrank values in the reference's order (combinatorics.h:120-131)
    if (lane == 0) {
        uint32_t x = rank, o = 0;
        for (int i = 0; i < mods.num_ma; ++i) {
            uint32_t r;
            if (i != mods.num_ma - 1) {
                const uint32_t nx = scan[i + 1];
                if (x >= nx) { r = x / nx; x = x % nx; } else r = 0u;
            } else r = x;
            const uint32_t k = (uint32_t)dcount[i];
            if (k == 0) continue;
            const uint32_t nn = D[i];
            uint32_t a = nn, b = k;
            const uint32_t total = choose_dev(nn, k);
            uint32_t y;
            bool dual = false;
            if ((total / 2u) >= r) y = r; else { y = total - 1u - r; dual = true; }
            for (uint32_t t = 0; t < k; ++t) {
                uint32_t v = a - 1u;
                for (int guard = 0; guard < 256 && choose_dev(v, b) > y; ++guard) --v;
                y -= choose_dev(v, b);
                a = v;
                b -= 1u;
                if (o < 8) out_unrank[(size_t)q * 8 + o] = dual ? (nn - 1u) - v : v;
                ++o;
            }
        }
    }
    ModIsoform iso;
    iso.num_ma = mods.num_ma;
    iso.per_type = mods.per_type;
#pragma unroll
    for (int i = 0; i < kMaxMa; ++i) iso.ma_mass[i] = (float)(i + 1);  // marker values
    isoform_masks(D, scan, dcount, mods.num_ma, rank, iso.mask);
    iso.reset();
    for (uint32_t base = tc; base < tn; base += 32) {
        const uint32_t j = base + lane;
        const uint32_t byte = j < tn ? (uint32_t)__ldg(db.ions + j) : 0u;
        const float add = iso.chunk_add(byte, j < tn);
        if (j < tn && (int32_t)(j - tc) < cap) out_modded[(size_t)q * cap + (j - tc)] = add != 0.0f ? 1 : 0;
    }
}

}  // namespace hfx

using namespace hfx;

int hfx_mods_windows(const float *r_sorted, uint32_t num_pep, const SpecMeta *meta, int32_t nspec, const DevMods &m,
                     uint32_t *mb, uint32_t *me, cudaStream_t st) {
    const int64_t n = (int64_t)nspec * m.num_mod;
    if (n <= 0) return 0;
    k_mod_windows<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(r_sorted, num_pep, meta, nspec, m.delta, m.num_mod, mb,
                                                               me);
    return (int)cudaGetLastError();
}

int hfx_mods_plan(const BatchedWs &ws, uint32_t ngroups, const uint32_t *mb, const uint32_t *me, int32_t num_mod,
                  int32_t chunk, uint32_t *mlo, uint32_t *mhi, uint32_t *mchunk, int32_t *nchunks,
                  uint32_t *item_off, int32_t *partial, cudaStream_t st) {
    const int32_t n_gm = (int32_t)ngroups * num_mod;
    if (n_gm <= 0) return 0;
    k_mod_groups<<<(n_gm + 255) / 256, 256, 0, st>>>(ws.groups, ws.ngroups, ws.perm, mb, me, num_mod, chunk, n_gm,
                                                     mlo, mhi, mchunk, nchunks);
    cudaMemsetAsync(item_off, 0, sizeof(uint32_t), st);
    return hfx_scan_inclusive(nchunks, n_gm, (int32_t *)(item_off + 1), partial, st);
}

template <bool F, typename T, int G>
static int launch_mods_t(const DevDB &db, const DevMods &m, const void *tiles, int64_t stride, const uint32_t *mb,
                         const uint32_t *me, const BatchedWs &ws, const uint32_t *mlo, const uint32_t *mhi,
                         const uint32_t *mchunk, const uint32_t *item_off, int32_t n_gm, int32_t K, float *ps,
                         uint64_t *pk, unsigned long long *ncand, float *sink, unsigned long long *cursor,
                         const uint64_t *sink_end, uint32_t *err, cudaStream_t st) {
    int dev = 0, sms = 0, smem_max = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t qb = CtaSlots<G, uint64_t>::warp_bytes();
    auto fn = k_score_mods<F, T, G>;
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, fn);  // static shared memory counts against the same limit
    const size_t avail = (size_t)smem_max > fa.sharedSizeBytes ? (size_t)smem_max - fa.sharedSizeBytes : 0;
    const int nw = std::min(kModWarps, fused_warps(stride, sizeof(T), G, qb, avail));
    if (nw < 1) return (int)cudaErrorInvalidValue;
    const size_t smem = fused_smem_bytes(stride, sizeof(T), G, nw, qb);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, nw * 32, smem);
    cudaMemsetAsync(ws.counter, 0, 4, st);
    fn<<<sms * (occ > 0 ? occ : 1), nw * 32, smem, st>>>(db, m, (const T *)tiles, stride, mb, me, ws.perm, ws.groups,
                                                         mlo, mhi, mchunk, item_off, n_gm, K, ws.counter, ps, pk,
                                                         ncand, sink, cursor, sink_end, err);
    return (int)cudaGetLastError();
}

int hfx_mods_score(const DevDB &db, const DevMods &m, const void *tiles, int elem_kind, int64_t stride,
                   const uint32_t *mb, const uint32_t *me, const BatchedWs &ws, const uint32_t *mlo,
                   const uint32_t *mhi, const uint32_t *mchunk, const uint32_t *item_off, int32_t n_gm, int32_t G,
                   int32_t K, int fastdiv, float *ps, uint64_t *pk, unsigned long long *ncand, uint32_t *err,
                   cudaStream_t st, float *sink, unsigned long long *cursor, const uint64_t *sink_end) {
    if (n_gm <= 0) return 0;
    if (sink && (!cursor || !sink_end)) return (int)cudaErrorInvalidValue;
#define HFX_M(F, T, GG)                                                                                            \
    return launch_mods_t<F, T, GG>(db, m, tiles, stride, mb, me, ws, mlo, mhi, mchunk, item_off, n_gm, K, ps, pk, \
                                   ncand, sink, cursor, sink_end, err, st)
#define HFX_MG(F, T)              \
    do {                          \
        if (G == 8) HFX_M(F, T, 8); \
        if (G == 4) HFX_M(F, T, 4); \
        if (G == 2) HFX_M(F, T, 2); \
        if (G == 1) HFX_M(F, T, 1); \
    } while (0)
    if (elem_kind == 0) { if (fastdiv) HFX_MG(true, float); else HFX_MG(false, float); }
    else if (elem_kind == 1) { if (fastdiv) HFX_MG(true, __nv_bfloat16); else HFX_MG(false, __nv_bfloat16); }
    else { if (fastdiv) HFX_MG(true, __half); else HFX_MG(false, __half); }
#undef HFX_MG
#undef HFX_M
    return (int)cudaErrorInvalidValue;
}

int hfx_merge_with_mods(const float *ps, const uint64_t *pk, const uint32_t *item_off, const float *ms,
                        const uint64_t *mk, const uint32_t *mitem_off, int32_t num_mod, const BatchedWs &ws,
                        const SpecMeta *meta, int32_t nspec, int32_t G, int32_t K, int32_t plain, float *out_s,
                        uint64_t *out_k, cudaStream_t st) {
    k_merge_with_mods<<<(nspec + 3) / 4, 128, 0, st>>>(ps, pk, item_off, ms, mk, mitem_off, num_mod, ws.group_of,
                                                       ws.slot_of, meta, nspec, G, K, plain, out_s, out_k);
    return (int)cudaGetLastError();
}

int hfx_mods_isoforms(const DevDB &db, const DevMods &m, const uint32_t *pos, const int32_t *mu, const uint32_t *rank,
                      int32_t n, int32_t cap, uint32_t *out_count, uint32_t *out_unrank, uint8_t *out_modded,
                      cudaStream_t st) {
    if (n <= 0) return 0;
    k_mod_isoforms<<<(n + 3) / 4, 128, 0, st>>>(db, m, pos, mu, rank, n, cap, out_count, out_unrank, out_modded);
    return (int)cudaGetLastError();
}
