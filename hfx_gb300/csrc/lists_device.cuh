// Device helpers of the per-step ion lists, shared by the list kernels of
// unmodified candidates (lists.cu) and of modified isoforms (iso_lists.cu).
#pragma once
#include <cstdint>
#include "device_common.cuh"

namespace hfx {

// Entries of one lane's plane words [w0, w1) from list position pos on;
// clears the words when `clear`.  kChecked drops entries at or beyond cap
// (a list longer than its destination); otherwise the caller has checked
// that the whole list fits.  Inlined once per destination so that a staging
// list in shared memory is written with shared-memory stores.
template <bool kChecked>
__device__ __forceinline__ void emit_plane_entries(const Planes &pl, int w0, int w1, bool clear, int pos,
                                                   uint16_t *list, int cap) {
    for (int w = w0; w < w1; ++w) {
        const uint32_t h = pl.H[w], tt = pl.T[w];
        uint32_t a = pl.A[w] | h;
        if (clear) {
            pl.A[w] = 0u;
            pl.H[w] = 0u;
            pl.T[w] = 0u;
        }
        const uint32_t base = (uint32_t)w << 7 | 1u;  // (w * 32) << 2, level 1
        while (a) {
            const int b = __ffs(a) - 1;
            a &= a - 1u;
            const uint32_t key = base + ((uint32_t)b << 2) + ((h >> b) & 1u) + ((tt >> b) & 1u);
            if (!kChecked || pos < cap) list[pos] = (uint16_t)key;
            ++pos;
        }
    }
}

// Warp-cooperative compaction of plane words [wr.lo, wr.hi) into the
// ascending distinct-bin list (entries (bin << 2) | level); clears the
// words when `clear`.  Lane l takes k = ceil(words / 32) consecutive words,
// so one scan places every lane's entries and the serial bit loop runs as
// long as the fullest lane's k words, not a 32-word stripe's fullest word
// per stripe.  A list of up to `stage_cap` entries goes to the shared-memory
// staging list `stage` (the caller copies it out in 16-byte pieces); a
// longer one straight to `direct` (global memory, room for `direct_cap`
// entries).  Returns the number of distinct bins (entries beyond the
// destination's room are dropped).
__device__ __forceinline__ int compact_planes(const Planes &pl, WordRange wr, bool clear, uint16_t *stage,
                                              int stage_cap, uint16_t *direct, int direct_cap) {
    const int lane = threadIdx.x & 31;
    const int nwords = wr.hi - wr.lo;
    if (nwords <= 0) return 0;
    const int k = (nwords + 31) >> 5;
    const int w0 = wr.lo + lane * k;
    const int w1 = min(w0 + k, wr.hi);
    int pc = 0;
    for (int w = w0; w < w1; ++w) pc += __popc(pl.A[w] | pl.H[w]);
    const int incl = warp_incl_scan(pc);
    const int total = __shfl_sync(kFullMask, incl, 31);
    if (total <= stage_cap) emit_plane_entries<false>(pl, w0, w1, clear, incl - pc, stage, stage_cap);
    else if (total <= direct_cap) emit_plane_entries<false>(pl, w0, w1, clear, incl - pc, direct, direct_cap);
    else emit_plane_entries<true>(pl, w0, w1, clear, incl - pc, direct, direct_cap);
    __syncwarp();
    return total;
}

// Room of the shared-memory staging list of one warp (entries): lists up to
// this long are copied out in 16-byte pieces, longer ones written directly.
constexpr int kStageCap = 1024;

// Offset of the list of (level z, mass-order position p): every level has a
// static region; position p's slot holds z * (10 (tn - tc) rounded up to 8)
// entries and starts on a 16-byte boundary.
__device__ __forceinline__ uint64_t list_offset(const uint32_t *__restrict__ lstart, uint64_t total10, int z,
                                                uint32_t p) {
    return total10 * (uint64_t)(z * (z - 1) / 2) + (uint64_t)z * lstart[p];
}

}  // namespace hfx
