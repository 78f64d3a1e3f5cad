// Launch wrappers of the search kernels (called by the C++ host code).
#pragma once
#include "hfx_internal.h"

int hfx_launch_windows(const float *r_sorted, uint32_t n, const hfx::SpecMeta *meta, int32_t nspec,
                       uint32_t *wb, uint32_t *we, cudaStream_t st);
int hfx_launch_score_spectrum(const hfx::DevDB &db, const float *row, int32_t len, int32_t charges,
                              uint32_t begin, uint32_t end, int32_t K, int32_t nblocks, int fastdiv,
                              float *part_s, uint64_t *part_k, uint32_t *err, cudaStream_t st);
int hfx_launch_merge_parts(const float *part_s, const uint64_t *part_k, const int64_t *part_off,
                           int32_t nspec, int32_t K, int32_t topn, const uint32_t *idx_sorted,
                           float *out_s, uint64_t *out_k, uint32_t *out_pep, cudaStream_t st);
int hfx_launch_ion_bins(const hfx::DevDB &db, const uint32_t *pos, const int32_t *charges,
                        const int32_t *lens, int32_t n, int32_t maxlen, int32_t cap, int fastdiv,
                        uint32_t *out_bins, uint8_t *out_lvl, int32_t *out_n, cudaStream_t st);
