// Per-step ion lists of modified isoforms (iso_lists.cu): launch wrappers.
#pragma once
#include "hfx_internal.h"
#include "batched.h"

// Scan partials the 64-bit scan of n values needs.
int64_t hfx_iso_scan64_partials_needed(int64_t n);
// Coverage and isoform counts: cover [num_mod * kLevels * (num_pep + 1)]
// (difference arrays scanned in place; cover_partial for that scan), count
// and incl [num_mod * num_pep + 1] (isoforms per (combination, position)
// and their inclusive scan; incl[n] = total isoforms), units and incl_units
// [num_mod * num_pep] (list entries of their slots and the inclusive scan).
int hfx_iso_plan(const hfx::DevDB &db, const hfx::DevMods &m, const hfx::SpecMeta *meta, int32_t nspec,
                 const uint32_t *mb, const uint32_t *me, const uint32_t *lstart, int32_t *cover, int32_t *cover_partial,
                 int32_t *count, int32_t *incl, int32_t *count_partial, unsigned long long *units,
                 unsigned long long *incl_units, unsigned long long *units_partial, cudaStream_t st);
// One record per isoform (key, list slot offset); records past cap_iso or
// slots past cap_entries set kErrBounds (skipped slots get the key ~0).
int hfx_iso_expand(const hfx::DevDB &db, const hfx::DevMods &m, const int32_t *cover, const uint32_t *lstart,
                   const int32_t *count, const int32_t *incl, const unsigned long long *units,
                   const unsigned long long *incl_units, uint32_t cap_iso, uint64_t cap_entries, uint64_t *iso_key,
                   uint64_t *iso_off, uint32_t *err, cudaStream_t st);
// The isoforms' ion lists (u16 entries bin << 2 | level, ascending) of every
// needed level; iso_len [isoform][kLevels].  total_p: the device total.
// First the residues each isoform modifies (iso_pos, pos_words words per
// record, at least the longest peptide's residues / 32).
// stats (nullable, 8 counters): [0] lists, [1] entries, [5] isoform records,
// [6] residues read.
int hfx_iso_generate(const hfx::DevDB &db, const hfx::DevMods &m, const int32_t *cover, int32_t nbins,
                     const uint32_t *lstart, const int32_t *total_p, uint32_t cap_iso, const uint64_t *iso_key,
                     const uint64_t *iso_off, uint16_t *lists, uint64_t list_total, uint16_t *iso_len,
                     int32_t list_cap, int32_t pos_words, uint32_t *iso_pos, int fastdiv,
                     unsigned long long *stats, uint32_t *err, cudaStream_t st);
// The scorer over the isoform lists and the group tiles; work items and
// partial outputs as hfx_mods_score's (without a score sink).  stats
// (nullable): [2] isoform hand-outs, [3] list entries streamed, [4] pairs,
// [7] tile bytes staged.
int hfx_iso_score(const uint16_t *lists, uint64_t list_total, const uint32_t *lstart, const uint64_t *iso_key,
                  const uint64_t *iso_off, const uint16_t *iso_len, const int32_t *count, const int32_t *incl,
                  uint32_t num_pep, uint32_t cap_iso, int elem_kind, const void *tiles, int64_t stride,
                  const uint32_t *mb, const uint32_t *me, int32_t num_mod, const hfx::BatchedWs &ws,
                  const uint32_t *mlo, const uint32_t *mhi, const uint32_t *mchunk, const uint32_t *item_off,
                  int32_t n_gm, int32_t G, int32_t K, float *ps, uint64_t *pk, unsigned long long *ncand,
                  unsigned long long *stats, uint32_t *err, cudaStream_t st);
