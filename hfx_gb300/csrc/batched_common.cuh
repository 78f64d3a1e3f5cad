// Pieces shared by the two batched scorers (fused ion generation,
// batched.cu; precomputed ion lists, lists.cu).
#pragma once
#include "hfx_internal.h"
#include "device_common.cuh"
#include "batched.h"

namespace hfx {

constexpr uint32_t kWaitLimit = 1u << 24;  // mbarrier polls before reporting a timeout
constexpr uint32_t kLockLimit = 1u << 20;  // lock attempts before reporting a timeout

// Candidates per work item for a union window of `width` candidates: the
// requested chunk, or width/16 when that is larger (open-search windows of
// 10^5-10^6 candidates would otherwise need 10^5+ items per group).
__host__ __device__ __forceinline__ uint32_t group_chunk(uint32_t width, int32_t chunk) {
    const uint32_t c = (uint32_t)(chunk > 0 ? chunk : 1);
    const uint32_t w = (width + 15u) / 16u;
    return w > c ? w : c;
}

// Bins of a group tile that the scorer copies (a multiple of 8 keeps every
// bulk copy a multiple of 16 bytes).
__host__ __device__ __forceinline__ int32_t tile_bins(int32_t maxlen) { return (maxlen + 7) & ~7; }


__device__ __forceinline__ int32_t find_group(const uint32_t *__restrict__ item_off, int32_t ngroups, uint32_t item) {
    // last g with item_off[g] <= item
    int32_t lo = 0, hi = ngroups;
    while (hi - lo > 1) {
        const int32_t mid = (lo + hi) >> 1;
        if (item_off[mid] <= item) lo = mid; else hi = mid;
    }
    return lo;
}

// Interleave each group's member rows bin-major, tile[g][bin][G]: zero
// rows for empty slots and zeros beyond each member's length, so that the
// scorer needs neither a per-member length test nor a per-member load.
template <typename T> __device__ __forceinline__ T zero_of();
template <> __device__ __forceinline__ float zero_of<float>() { return 0.0f; }
template <> __device__ __forceinline__ __nv_bfloat16 zero_of<__nv_bfloat16>() { return __float2bfloat16_rn(0.0f); }
template <> __device__ __forceinline__ __half zero_of<__half>() { return __float2half_rn(0.0f); }

template <typename T, int G>
struct alignas((G * sizeof(T) >= 16) ? 16 : G * sizeof(T)) TilePack {
    T v[G];
};

template <typename T, int G>
__global__ void k_pack_tiles(const T *__restrict__ rows, int64_t stride, const SpecMeta *__restrict__ meta,
                             const int32_t *__restrict__ perm, const GroupInfo *__restrict__ groups,
                             const uint32_t *__restrict__ ngroups_p, T *__restrict__ tiles) {
    const uint32_t g = blockIdx.x;
    if (g >= *ngroups_p) return;
    const GroupInfo gi = groups[g];
    __shared__ int32_t s_spec[G], s_len[G];
    if (threadIdx.x < G) {
        const int j = threadIdx.x;
        const int32_t s = j < (int)gi.count ? perm[gi.pos0 + j] : -1;
        s_spec[j] = s;
        s_len[j] = s >= 0 ? meta[s].len : 0;
    }
    __syncthreads();
    T *tile = tiles + (size_t)g * stride * G;
    const int32_t nb = tile_bins(gi.maxlen);
    for (int32_t b = threadIdx.x; b < nb; b += blockDim.x) {
        TilePack<T, G> pk;
#pragma unroll
        for (int j = 0; j < G; ++j)
            pk.v[j] = (s_spec[j] >= 0 && b < s_len[j]) ? rows[(size_t)s_spec[j] * stride + b] : zero_of<T>();
        *reinterpret_cast<TilePack<T, G> *>(tile + (size_t)b * G) = pk;
    }
}

// Shared-memory layout of the fused scorers (unmodified and modified): an
// mbarrier, the group tile, and per warp three bit planes, a list and the
// warp's admission queue (queue_bytes).
__host__ __device__ __forceinline__ size_t fused_queue_offset(int32_t words) {
    return ((size_t)3 * words * 4 + (size_t)kListCap * 2 + 15) & ~(size_t)15;
}
__host__ __device__ __forceinline__ size_t fused_warp_bytes(int32_t words, size_t queue_bytes) {
    return (fused_queue_offset(words) + queue_bytes + 15) & ~(size_t)15;
}
__host__ __device__ __forceinline__ size_t fused_tile_bytes(int64_t stride, int elem_bytes, int G) {
    return ((size_t)stride * G * elem_bytes + 15) & ~(size_t)15;
}
__host__ __device__ __forceinline__ size_t fused_smem_bytes(int64_t stride, int elem_bytes, int G, int nw,
                                                            size_t queue_bytes) {
    return 128 + fused_tile_bytes(stride, elem_bytes, G) +
           (size_t)nw * fused_warp_bytes((int32_t)((stride + 31) / 32), queue_bytes);
}
// Largest warp count (<= 24) whose layout fits in smem_max bytes, 0 if none.
inline int fused_warps(int64_t stride, int elem_bytes, int G, size_t queue_bytes, size_t smem_max) {
    for (int nw = 24; nw >= 1; --nw)
        if (fused_smem_bytes(stride, elem_bytes, G, nw, queue_bytes) <= smem_max) return nw;
    return 0;
}

// Order-preserving map of a float score to uint32 (for atomicMax thresholds).
__device__ __forceinline__ uint32_t score_order(float s) {
    const uint32_t b = __float_as_uint(s);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Lane that holds member slot j's score after reduce_scatter<G>.
template <int G> __host__ __device__ constexpr int slot_lane(int j) { return j * (32 / G); }

// Queue entries per member slot of a warp, and a warp's queue bytes.
__host__ __device__ constexpr int cta_queue_len(int G) { return G >= 16 ? 8 : 16; }
__host__ __device__ constexpr size_t cta_queue_bytes(int G, int key_bytes) {
    return (size_t)G * cta_queue_len(G) * (4 + key_bytes);
}

// L: entries per member list (32, or 64 to keep up to 64 candidates: each
// lane then holds list entries lane and 32 + lane).
template <int G, typename Key = uint32_t, int Q = cta_queue_len(G), int L = 32>
struct CtaSlots {
    static_assert(L == 32 || L == 64, "member lists hold 32 or 64 entries");
    static constexpr int kQ = Q;
    static constexpr Key kNone = ~Key(0);
    float *ls;       // [G][L] scores of the CTA's lists
    Key *lk;         // [G][L] keys
    uint32_t *lock;  // [G]
    uint32_t *thr;   // [G] score_order of each list's K-th (0 = none yet)
    float *qs;       // this warp's queues: [G][kQ] scores, then [G][kQ] keys
    Key *qk;
    uint32_t qn;     // slot lanes: entries queued for the lane's slot
    uint32_t *err;
    // lock hold test (the word after the error word; 0 = off): member 0's
    // lock starts held by nobody, so every merge into it gives up after
    // kLockLimit attempts
    uint32_t test_hold;

    __host__ __device__ static constexpr size_t warp_bytes() { return cta_queue_bytes(G, (int)sizeof(Key)); }
    static_assert(Q == cta_queue_len(G), "queue length and cta_queue_bytes disagree");

    __device__ __forceinline__ void bind(float *ls_, Key *lk_, uint32_t *lock_, uint32_t *thr_, uint8_t *queue,
                                         uint32_t *err_) {
        ls = ls_;
        lk = lk_;
        lock = lock_;
        thr = thr_;
        qs = reinterpret_cast<float *>(queue);
        qk = reinterpret_cast<Key *>(queue + (size_t)G * kQ * 4);
        qn = 0u;
        err = err_;
        test_hold = err_[1] & 0xFFu;
    }
    // Item start, by threads [0, L G) of the CTA (a barrier must follow).
    __device__ __forceinline__ void reset_shared() {
        for (int t = threadIdx.x; t < G * L; t += blockDim.x) {
            ls[t] = -INFINITY;
            lk[t] = kNone;
        }
        if (threadIdx.x < G) {
            lock[threadIdx.x] = (test_hold != 0u && threadIdx.x == 0) ? 2u : 0u;
            thr[threadIdx.x] = 0u;
        }
    }

    __device__ __forceinline__ static bool better(float a, Key ka, float b, Key kb) {
        return a > b || (a == b && ka < kb);
    }
    // Compare-exchange with lane ^ d: the lower lane keeps the better entry
    // when `desc`, the worse one otherwise.
    __device__ __forceinline__ static void cx(float &v, Key &kv, int d, bool desc) {
        const int lane = threadIdx.x & 31;
        const float ov = __shfl_xor_sync(kFullMask, v, d);
        const Key ok = __shfl_xor_sync(kFullMask, kv, d);
        const bool lower = (lane & d) == 0;
        const bool mine = better(v, kv, ov, ok);
        if (mine != (lower == desc)) {
            v = ov;
            kv = ok;
        }
    }

    // Merge the first `cnt` queued entries of slot j (warp-wide).
    __device__ __forceinline__ void merge(int j, int cnt, int K) {
        const int lane = threadIdx.x & 31;
        float ns = -INFINITY;
        Key nk = kNone;
        if (lane < cnt) {
            ns = qs[j * kQ + lane];
            nk = qk[j * kQ + lane];
        }
        // lanes 0..kQ-1 sorted best first; lanes kQ..31 hold nothing
#pragma unroll
        for (int b = 2; b <= kQ; b <<= 1)
#pragma unroll
            for (int d = b >> 1; d > 0; d >>= 1) cx(ns, nk, d, (lane & b) == 0);
        const float rs = __shfl_sync(kFullMask, ns, 31 - lane);
        const Key rk = __shfl_sync(kFullMask, nk, 31 - lane);
        uint32_t got = 0u;
        if (lane == 0) {
            // a constant bound: a variable one measurably slowed every kernel
            // that merges here (the modification scorer by a sixth)
            for (uint32_t i = 0; i < kLockLimit; ++i)
                if (atomicCAS(lock + j, 0u, 1u) == 0u) {
                    got = 1u;
                    break;
                }
        }
        got = __shfl_sync(kFullMask, got, 0);
        if (!got) {
            if (lane == 0) atomicOr(err, kErrTimeout);
            return;
        }
        __threadfence_block();
        float kth;
        if constexpr (L == 32) {
            float ws = *(volatile float *)(ls + j * 32 + lane);
            Key wk = *(volatile Key *)(lk + j * 32 + lane);
            // the top 32 of both lists as a bitonic sequence, then sorted best first
            if (better(rs, rk, ws, wk)) {
                ws = rs;
                wk = rk;
            }
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) cx(ws, wk, d, true);
            *(volatile float *)(ls + j * 32 + lane) = ws;
            *(volatile Key *)(lk + j * 32 + lane) = wk;
            kth = __shfl_sync(kFullMask, ws, K - 1);
        } else {
            // entries lane (w0) and 32 + lane (w1); the queue, ascending, fills
            // the last 16 of 64 positions (w1 of lanes 16..31, which rs holds)
            float w0 = *(volatile float *)(ls + j * 64 + lane), w1 = *(volatile float *)(ls + j * 64 + 32 + lane);
            Key k0 = *(volatile Key *)(lk + j * 64 + lane), k1 = *(volatile Key *)(lk + j * 64 + 32 + lane);
            if (better(rs, rk, w1, k1)) {
                w1 = rs;
                k1 = rk;
            }
            // bitonic merge of the 64: positions i and i + 32 in the lane,
            // then each half across lanes
            if (better(w1, k1, w0, k0)) {
                const float ts = w0;
                const Key tk = k0;
                w0 = w1;
                k0 = k1;
                w1 = ts;
                k1 = tk;
            }
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
                cx(w0, k0, d, true);
                cx(w1, k1, d, true);
            }
            *(volatile float *)(ls + j * 64 + lane) = w0;
            *(volatile float *)(ls + j * 64 + 32 + lane) = w1;
            *(volatile Key *)(lk + j * 64 + lane) = k0;
            *(volatile Key *)(lk + j * 64 + 32 + lane) = k1;
            const float a = __shfl_sync(kFullMask, w0, (K - 1) & 31), b = __shfl_sync(kFullMask, w1, (K - 1) & 31);
            kth = K > 32 ? b : a;
        }
        if (lane == 0 && kth != -INFINITY) *(volatile uint32_t *)(thr + j) = score_order(kth);
        __threadfence_block();
        __syncwarp();
        if (lane == 0) atomicExch(lock + j, 0u);
    }

    // Offer candidate `key`: the lane of slot `my_slot` appends (sc, key) to
    // the slot's queue when `want`; full queues are merged.
    __device__ __forceinline__ void offer(bool want, float sc, Key key, int my_slot, int K) {
        if (want) {
            qs[my_slot * kQ + qn] = sc;
            qk[my_slot * kQ + qn] = key;
            ++qn;
        }
        uint32_t full = __ballot_sync(kFullMask, want && qn == (uint32_t)kQ);
        while (full) {
            const int l = __ffs(full) - 1;
            full &= full - 1u;
            __syncwarp();
            merge(l / (32 / G), kQ, K);
            if ((threadIdx.x & 31) == l) qn = 0u;
        }
    }

    // Item end: merge what is still queued.
    __device__ __forceinline__ void drain(int K) {
        uint32_t own = 0u;
#pragma unroll
        for (int j = 0; j < G; ++j) own |= 1u << slot_lane<G>(j);
        uint32_t pend = __ballot_sync(kFullMask, qn != 0u) & own;
        __syncwarp();
        while (pend) {
            const int l = __ffs(pend) - 1;
            pend &= pend - 1u;
            merge(l / (32 / G), (int)__shfl_sync(kFullMask, qn, l), K);
        }
        qn = 0u;
    }

    // After a barrier: slot j's top-K (entries < K; warp-wide).
    __device__ __forceinline__ void result(int j, int K, float *out_s, uint64_t *out_k) const {
        const int lane = threadIdx.x & 31;
#pragma unroll
        for (int r = 0; r < L / 32; ++r) {
            const int i = 32 * r + lane;
            if (i < K) {
                const Key k = lk[j * L + i];
                out_s[i] = ls[j * L + i];
                out_k[i] = k == kNone ? ~0ull : (uint64_t)k;
            }
        }
    }
};

}  // namespace hfx

template <typename T, int G>
inline void hfx_pack_tiles_launch(const T *rows, int64_t stride, const hfx::SpecMeta *meta, const hfx::BatchedWs &ws,
                                  T *tiles, uint32_t ngroups, cudaStream_t st) {
    hfx::k_pack_tiles<T, G><<<ngroups, 256, 0, st>>>(rows, stride, meta, ws.perm, ws.groups, ws.ngroups, tiles);
}

