// Batched (persistent) search: workspace and launch wrappers.
#pragma once
#include "hfx_internal.h"

namespace hfx {
struct GroupInfo {
    uint32_t pos0, count;  // members: perm[pos0 .. pos0+count)
    uint32_t lo, hi;       // union of the members' candidate windows
    int32_t maxlen;        // longest member row
    int32_t charges;       // ion charges shared by the members (unmodified)
    int32_t charges_mod;   // ion charges of the members' modified candidates
    uint32_t chunk;        // candidates per work item of this group
};

struct BatchedWs {
    uint32_t *hist;         // [classes*buckets + 1] bucket counts -> offsets
    uint32_t *cursor;       // [classes*buckets] scatter cursors
    uint32_t *n_sorted;     // [1] spectra placed
    int32_t *perm;          // [nspec] sorted position -> spectrum
    GroupInfo *groups;      // [nspec]
    uint32_t *item_off;     // [nspec+1] first work item of each group
    uint32_t *ngroups;      // [1]
    uint32_t *total_items;  // [1]
    int32_t *group_of;      // [nspec]
    int32_t *slot_of;       // [nspec]
    uint32_t *counter;      // [1] work-stealing cursor
};

constexpr int kBucketCount = 12 * 8192;
}  // namespace hfx

size_t hfx_batched_smem(int64_t stride, int elem_bytes, int G, int nw, int K);
int hfx_batched_plan(const hfx::SpecMeta *meta, int32_t nspec, const uint32_t *wb, const uint32_t *we, int32_t G,
                     int32_t chunk, const hfx::BatchedWs &ws, cudaStream_t st);
// Runs the persistent scorer over the group tiles packed by hfx_pack_tiles
// (tiles: ngroups * stride * G elements); nw = warps per CTA (0 = as many as shared memory holds,
// at most 16), grid = CTAs (0 = one wave).
int hfx_batched_score(const hfx::DevDB &db, const void *rows, int elem_kind, int64_t stride,
                      const hfx::SpecMeta *meta, const uint32_t *wb, const uint32_t *we, const hfx::BatchedWs &ws,
                      void *tiles, uint32_t ngroups, int32_t G, int32_t chunk, int32_t K, int nw, int grid,
                      int fastdiv, float *part_s, uint64_t *part_k, uint32_t *err, cudaStream_t st);
int hfx_clamp_items(uint32_t *off, int64_t n1, uint32_t cap, uint32_t *err, cudaStream_t st);
// Graph replays: a planned group count above the tiles' capacity is cut to
// it and sets kErrBounds in the error word.
int hfx_clamp_groups(uint32_t *ngroups, uint32_t cap, uint32_t *err, cudaStream_t st);
int hfx_batched_merge(const float *part_s, const uint64_t *part_k, const hfx::BatchedWs &ws,
                      const hfx::SpecMeta *meta, int32_t nspec, int32_t G, int32_t K, int32_t kout, float *out_s,
                      uint64_t *out_k, cudaStream_t st);
// FP32 rescoring of the kept low-precision matches (unmodified and modified
// keys) and the final top-N.
int hfx_rescore(const hfx::DevDB &db, const hfx::DevMods &mods, const float *rows32, int64_t stride,
                const hfx::SpecMeta *meta, const float *kept_s, const uint64_t *kept_k, int32_t nspec, int32_t K,
                int32_t topn, int fastdiv, float *out_s, uint64_t *out_k, uint32_t *out_pep, cudaStream_t st);
// Peptide ids of the top-N and candidate counts: the unmodified window
// (when plain) plus the modified isoforms counted by the scorer (ncand_mod,
// may be null).
int hfx_finish(const float *in_s, const uint64_t *in_k, int32_t nspec, int32_t topn, const uint32_t *idx_sorted,
               const uint32_t *wb, const uint32_t *we, const hfx::SpecMeta *meta, float *out_s, uint64_t *out_k,
               uint32_t *out_pep, int32_t plain, const unsigned long long *ncand_mod, int64_t *ncand,
               cudaStream_t st);
int hfx_ncand(const uint32_t *wb, const uint32_t *we, const hfx::SpecMeta *meta, int32_t nspec, int32_t plain,
              const unsigned long long *ncand_mod, int64_t *ncand, cudaStream_t st);
// Interleaved group tiles only (the scorers pack their own otherwise).
int hfx_pack_tiles(const void *rows, int elem_kind, int64_t stride, const hfx::SpecMeta *meta,
                   const hfx::BatchedWs &ws, void *tiles, uint32_t ngroups, int32_t G, cudaStream_t st);
