// The "Ions" column of the matches (ions.cu): launch wrapper.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "hfx_internal.h"

// Dynamic shared memory of the kernel for rows of this stride.
size_t hfx_match_ions_smem(int64_t stride);
// out_m / out_t [nspec][topn]: matched and total ions of each result key
// (0 / 0 for empty slots) against the spectra's preprocessed rows.
int hfx_match_ions_launch(const hfx::DevDB &db, const hfx::DevMods &mods, uint64_t nion, const hfx::SpecMeta *meta,
                          const float *rows, int64_t stride, const float *z, float bw, const uint64_t *keys,
                          int32_t nspec, int32_t topn, int32_t *out_m, int32_t *out_t, uint32_t *err,
                          cudaStream_t st);
