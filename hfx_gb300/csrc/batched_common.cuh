// Pieces shared by the two batched scorers (fused ion generation,
// batched.cu; precomputed ion lists, lists.cu).
#pragma once
#include "hfx_internal.h"
#include "device_common.cuh"
#include "batched.h"

namespace hfx {

constexpr uint32_t kWaitLimit = 1u << 24;  // mbarrier polls before reporting a timeout
constexpr uint32_t kLockLimit = 1u << 20;  // lock attempts before reporting a timeout

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

// Warp-cooperative insert into a sorted shared-memory list (entry i at
// lane i); returns the new K-th score (the admission threshold).
__device__ __forceinline__ float smem_topk_insert(float *ks, uint64_t *kk, float ns, uint64_t nk, int K) {
    const int lane = threadIdx.x & 31;
    const float cs = lane < K ? ks[lane] : -INFINITY;
    const uint64_t ck = lane < K ? kk[lane] : ~0ull;
    const bool mine_better = (lane < K) && better(cs, ck, ns, nk);
    const int pos = __popc(__ballot_sync(kFullMask, mine_better));
    const float us = __shfl_up_sync(kFullMask, cs, 1);
    const uint64_t uk = __shfl_up_sync(kFullMask, ck, 1);
    float out = cs;
    __syncwarp();
    if (pos < K) {
        if (lane == pos) { ks[lane] = ns; kk[lane] = nk; out = ns; }
        else if (lane > pos && lane < K) { ks[lane] = us; kk[lane] = uk; out = us; }
    }
    __syncwarp();
    return __shfl_sync(kFullMask, out, K - 1);
}

template <int G>
__device__ __forceinline__ uint32_t slot_owner_mask() {
    // one lane per slot among the lanes that hold the same reduced slot
    if constexpr (G == 8) return 0x11111111u;
    else if constexpr (G == 4) return 0x01010101u;
    else if constexpr (G == 2) return 0x00010001u;
    else return 0x1u;
}


}  // namespace hfx

template <typename T, int G>
inline void hfx_pack_tiles_launch(const T *rows, int64_t stride, const hfx::SpecMeta *meta, const hfx::BatchedWs &ws,
                                  T *tiles, uint32_t ngroups, cudaStream_t st) {
    hfx::k_pack_tiles<T, G><<<ngroups, 256, 0, st>>>(rows, stride, meta, ws.perm, ws.groups, ws.ngroups, tiles);
}

