// E-values of the matches on the device (evalues.cu): launch wrappers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

// Per spectrum the number of candidates -- unmodified (we - wb, when plain)
// plus modified isoforms (isoforms[s], may be null) -- their exclusive scan,
// the segment ends and the first entry after the unmodified ones (cursor,
// may be null).
int hfx_evalue_offsets(const uint32_t *wb, const uint32_t *we, int plain, const unsigned long long *isoforms,
                       int32_t ns, uint64_t *size, uint64_t *off, uint64_t *end, unsigned long long *cursor,
                       cudaStream_t st);
// fit[s] = (alpha, beta, histogram points) of spectrum s, from its unsorted
// scores scores[off[s] .. off[s] + size[s]) (order statistics by radix
// select, histogram in shared memory).
int hfx_evalue_select_fit(const float *scores, const uint64_t *off, const uint64_t *size, int32_t ns,
                          int32_t bin_width, float cutoff_perc, double *fit, cudaStream_t st);
// ev[s][i] = 10 ** (alpha + beta * out_s[s][i] / 10000) (NaN for empty slots).
int hfx_evalue_apply(const float *out_s, const uint64_t *out_k, const double *fit, int32_t ns, int32_t topn,
                     double *ev, cudaStream_t st);
