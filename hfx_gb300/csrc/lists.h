// Precomputed ion lists (lists.cu): declarations.
#pragma once
#include "hfx_internal.h"
#include "batched.h"

namespace hfx {
constexpr int kLevels = 4;          // ion-charge levels 1..4 (Search.hs:182, ion_series.cu:301-309)
constexpr int kMaxListLen = 4096;   // distinct bins kept per (peptide, level)
}  // namespace hfx

int hfx_scan_inclusive(const int32_t *in, int64_t n, int32_t *out, int32_t *partial, cudaStream_t st);
int64_t hfx_scan_partials_needed(int64_t n);
int hfx_lists_mark(const hfx::SpecMeta *meta, const uint32_t *wb, const uint32_t *we, int32_t nspec, int64_t npep1,
                   int32_t *diff, cudaStream_t st);
// lstart[p] = 10 * sum_{q<p} (tn_q - tc_q) in mass order; total10 = 10 * sum
// over all peptides; the level-z list of p starts at
// total10 * z(z-1)/2 + z * lstart[p].  stats (nullable, 8 counters): [0] lists
// built, [1] list entries, [2] candidates scored, [3] entries streamed,
// [4] peptide-spectrum pairs.
int hfx_lists_generate(const hfx::DevDB &db, const int32_t *cover, int64_t npep1, int32_t nbins,
                       const uint32_t *lstart, uint64_t total10, uint16_t *lists, uint16_t *list_len,
                       int32_t list_cap, int fastdiv, unsigned long long *stats, uint32_t *err, cudaStream_t st);
// Scorer over the lists; long_rows: 32-bit entries and group tiles read
// from global memory (rows too long for shared memory), else 16-bit entries
// and tiles staged in shared memory.
// With a sink, every pair's score is written to sink[sink_off[s] + p - wb[s]]
// instead of the top-K.
int hfx_lists_score(const void *lists, int long_rows, const uint32_t *lstart, uint64_t total10,
                    const uint16_t *list_len, uint32_t num_pep, int elem_kind, int64_t stride, const uint32_t *wb,
                    const uint32_t *we, const hfx::BatchedWs &ws, void *tiles, int32_t G, int32_t K, int nw,
                    float *part_s, uint64_t *part_k, unsigned long long *stats, uint32_t *err, cudaStream_t st,
                    float *sink = nullptr, const uint64_t *sink_off = nullptr);
// Whether a G-spectrum group tile of rows `stride` bins long (and the
// scorer's queues) fits in shared memory; always 1 for G <= 8.
int hfx_lists_group_fits(int32_t G, int long_rows, int64_t stride, int elem_bytes);
// Long rows: 32-bit lists built by sorting each (peptide, level)'s ion keys,
// and FP32 rescoring of kept unmodified candidates from those lists.
int hfx_lists_generate_long(const hfx::DevDB &db, const int32_t *cover, int64_t npep1, int32_t nbins,
                            const uint32_t *lstart, uint64_t total10, uint32_t *lists, uint16_t *list_len,
                            int fastdiv, float ion_bw, unsigned long long *stats, uint32_t *err,
                            cudaStream_t st);
// FP32 rescoring of kept unmodified candidates from the step's lists (32-bit
// entries for long rows, else 16-bit) and the FP32 rows.
int hfx_rescore_lists(const void *lists, int long_rows, const uint32_t *lstart, uint64_t total10,
                      const uint16_t *list_len, uint32_t num_pep, const uint32_t *idx_sorted, const float *rows32,
                      int64_t stride, const hfx::SpecMeta *meta, const uint64_t *kept_k, int32_t nspec, int32_t K,
                      int32_t topn, float *out_s, uint64_t *out_k, uint32_t *out_pep, uint32_t *err,
                      cudaStream_t st);
