// Variable-modification search (stage e): launch wrappers.
#pragma once
#include "hfx_internal.h"
#include "batched.h"

// Candidate window of every (spectrum, combination): mb/me [nspec][num_mod].
int hfx_mods_windows(const float *r_sorted, uint32_t num_pep, const hfx::SpecMeta *meta, int32_t nspec,
                     const hfx::DevMods &m, uint32_t *mb, uint32_t *me, cudaStream_t st);
// Union window of every (group, combination) and the work-item offsets
// item_off [ngroups*num_mod + 1]; partial = hfx_scan_partials_needed(n) ints.
int hfx_mods_plan(const hfx::BatchedWs &ws, uint32_t ngroups, const uint32_t *mb, const uint32_t *me,
                  int32_t num_mod, int32_t chunk, uint32_t *mlo, uint32_t *mhi, uint32_t *mchunk, int32_t *nchunks,
                  uint32_t *item_off, int32_t *partial, cudaStream_t st);
// Persistent scorer of the modified isoforms over the packed group tiles;
// ncand (may be null) gains one per isoform per member spectrum.  With a
// sink, every isoform's score also goes to sink[cursor[s]++] (per member
// spectrum s; an entry at or past sink_end[s] sets kErrBounds instead).
int hfx_mods_score(const hfx::DevDB &db, const hfx::DevMods &m, const void *tiles, int elem_kind, int64_t stride,
                   const uint32_t *mb, const uint32_t *me, const hfx::BatchedWs &ws, const uint32_t *mlo,
                   const uint32_t *mhi, const uint32_t *mchunk, const uint32_t *item_off, int32_t n_gm, int32_t G,
                   int32_t K, int fastdiv, float *ps, uint64_t *pk, unsigned long long *ncand, uint32_t *err,
                   cudaStream_t st, float *sink = nullptr, unsigned long long *cursor = nullptr,
                   const uint64_t *sink_end = nullptr);
// Per spectrum: the best K of its unmodified items (when plain) and of its
// modified items.
int hfx_merge_with_mods(const float *ps, const uint64_t *pk, const uint32_t *item_off, const float *ms,
                        const uint64_t *mk, const uint32_t *mitem_off, int32_t num_mod, const hfx::BatchedWs &ws,
                        const hfx::SpecMeta *meta, int32_t nspec, int32_t G, int32_t K, int32_t plain, float *out_s,
                        uint64_t *out_k, cudaStream_t st);
// Isoform export for parity checks (see k_mod_isoforms).
int hfx_mods_isoforms(const hfx::DevDB &db, const hfx::DevMods &m, const uint32_t *pos, const int32_t *mu,
                      const uint32_t *rank, int32_t n, int32_t cap, uint32_t *out_count, uint32_t *out_unrank,
                      uint8_t *out_modded, cudaStream_t st);
