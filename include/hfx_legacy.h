/* Per-stage C ABI of the reference, served by libhfx_gpu.so.
 *
 * The reference's Haskell host binds these symbols with `foreign import
 * ccall` (src/haskell/Foreign/CUDA/Algorithms.hs:44-371) from
 * src/common/include/algorithms.h:80-325.  They are declared here with the
 * same names, argument order, types and return values, so a host built
 * against algorithms.h links against libhfx_gpu.so unchanged.  Every pointer
 * named d_* is device memory owned by the caller; work runs on the legacy
 * default stream (addModIons: on `stream`), as the reference's does.
 * Functions that return a count synchronise.
 *
 * The engine's own entry points (include/hfx_gpu.h) replace whole stages at
 * once; these shims are for hosts that keep the reference's stage-by-stage
 * call sequence, dense theoretical spectra included.
 */
#ifndef HFX_LEGACY_H
#define HFX_LEGACY_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *cudaStream_t;
typedef struct cublasContext *cublasHandle_t;

/* prepare_ions.cu:105-132: pack residue letters in place, byte =
 * (c - 'A') | (1 + index of c in d_ma) << 5.  As in the reference, a
 * database of fewer than 512 residues is left unpacked. */
void prepare_ions(uint8_t *d_ions, uint32_t N, uint8_t *d_ma, uint32_t num_ma);

/* filter.cu:40-66: indices i (ascending) with min <= d_in[i] <= max;
 * returns their number. */
uint32_t findIndicesInRange_f(const float *d_in, uint32_t *d_out, const uint32_t length, const float min,
                              const float max);

/* filter.cu:75-127: per spectrum the window [lower_bound(m - eps),
 * upper_bound(m + eps)) over d_r[d_pep_idx_r_sorted[.]], its size, and the
 * total (uint32). */
uint32_t findSpecCandsByMass(uint32_t *d_spec_begin_raw, uint32_t *d_spec_end_raw, uint32_t *d_spec_num_pep_raw,
                             const float *d_r_raw, const uint32_t *d_pep_idx_r_sorted_raw, const uint32_t num_pep,
                             const float *d_spec_masses_raw, const uint32_t num_spec, const float eps);

/* filter_by_mod.cu:35-143: for one spectrum mass, per modification the
 * window for (mass - eps) - delta .. (mass + eps) - delta, the exclusive scan
 * of the window sizes, and the total. */
uint32_t findBeginEnd_f(uint32_t *d_begin_raw, uint32_t *d_end_raw, uint32_t *d_num_pep_scan_raw,
                        const float *d_r_raw, const uint32_t *d_pep_idx_r_sorted_raw, const uint32_t num_pep,
                        const float *d_mod_delta_raw, const uint32_t num_mod, const float mass_, const float eps);

/* filter_by_mod.cu:265-378: expand every (spectrum, modification) window
 * into (fragment, modification) rows, count each modable acid over [tc, tn),
 * keep the rows that have enough of every acid (stable), and per spectrum
 * the number of kept rows before its first; returns the kept rows. */
uint32_t findModablePeptides(uint32_t *d_out_pep_idx_raw, uint32_t *d_out_pep_mod_idx_raw,
                             uint32_t *d_out_pep_ma_count_raw, uint32_t *d_out_spec_num_valid_scan,
                             const uint32_t *d_spec_num_cand_scan, const uint32_t num_spec, uint32_t num_cand_total,
                             const uint8_t *d_ions, const uint32_t *d_tc, const uint32_t *d_tn,
                             const uint32_t *d_pep_idx_r_sorted_raw, const uint32_t *d_begin_raw,
                             const uint32_t *d_end_raw, const uint32_t *d_num_pep_scan_raw,
                             const uint32_t *d_mod_ma_count, const uint32_t num_mod, const uint8_t *d_ma,
                             const uint32_t num_ma);

/* calc_mod_cands.cu:76-119: per row the isoform count prod C(D_i, d_i) and
 * its suffix products; returns the total (uint32). */
uint32_t calcTotalModCands(uint32_t *d_out_pep_num_mpep_raw, uint32_t *d_out_pep_ma_num_comb_scan_raw,
                           const uint32_t *d_mod_ma_count_raw, const uint32_t *d_pep_idx_raw,
                           const uint32_t *d_pep_mod_idx_raw, const uint32_t *d_pep_ma_count_raw,
                           const uint32_t nPep, const uint32_t num_mod, const uint32_t num_ma);

/* prepare_gen_mod.cu:79-129: one row per isoform (fragment, modification,
 * rank, source row) and the exclusive scan of the modification sizes;
 * returns the total unrank length. */
uint32_t prepareGenMod(uint32_t *d_out_mpep_pep_idx, uint32_t *d_out_mpep_pep_mod_idx, uint32_t *d_out_mpep_rank,
                       uint32_t *d_out_mpep_ith_valid, uint32_t *d_out_mpep_mod_ma_count_sum_scan,
                       const uint32_t *d_mod_ma_count_sum, const uint32_t *d_pep_idx, const uint32_t *d_pep_mod_idx,
                       const uint32_t *d_pep_num_mpep, const uint32_t num_pep, const uint32_t num_mpep);

/* gen_mod_pep.cu:127-312: per isoform the occurrence indices of every
 * modified acid (mixed-radix rank split, combination unranking with the
 * reference's dual-rank shortcut); num_ma 1..10. */
void genModCands(uint32_t *d_out_mpep_unrank, const uint32_t *d_mod_ma_count, const uint32_t *d_mpep_ith_valid,
                 const uint32_t *d_mpep_rank, const uint32_t *d_mpep_mod_ma_count_sum_scan,
                 const uint32_t *d_pep_mod_idx, const uint32_t *d_pep_ma_count,
                 const uint32_t *d_pep_ma_num_comb_scan, const uint32_t total, const uint32_t mod_num_ma);

/* mion_series.cu:174-558: dense theoretical spectra of modified
 * candidates, rows of len_spec floats (the caller zeroes d_out_mspec);
 * ion charges 1..min(max_charge, 4) for max_charge 1..10, num_ma 1..10. */
void addModIons(float *d_out_mspec, const float *d_residual, const float *d_mass, const uint8_t *d_ions,
                const uint32_t *d_tc, const uint32_t *d_tn, const uint32_t *d_mpep_pep_idx,
                const uint32_t *d_mpep_pep_mod_idx, const uint32_t *d_mpep_unrank,
                const uint32_t *d_mpep_mod_ma_count_sum_scan, const uint32_t len_unrank, const uint32_t num_mpep,
                const uint32_t *d_mod_ma_count, const float *d_mod_delta, const uint8_t *d_ma,
                const float *d_ma_mass, const uint32_t num_ma, const uint32_t len_spec, const uint32_t max_charge,
                cudaStream_t stream);

/* ion_series.cu:150-310: dense theoretical spectra, one row of len_spec
 * floats per d_idx entry (the caller zeroes d_spec); max_charge 1..4. */
void addIons(float *d_spec, const float *d_residual, const float *d_mass, const uint8_t *d_ions,
             const uint32_t *d_tc, const uint32_t *d_tn, const uint32_t *d_idx, const uint32_t num_idx,
             const uint32_t max_charge, const uint32_t len_spec);

/* prepare_scoring.cu:47-67: the concatenated candidate lists
 * d_pep_idx_r_sorted[begin[s] .. begin[s] + num[s]). */
void prepare_scoring(uint32_t *d_out_spec_pep_idx, const uint32_t *d_pep_idx_r_sorted_raw,
                     const uint32_t *d_spec_begin, const uint32_t *d_spec_num_pep, const uint32_t num_spec);

/* sort.cu:28-76, sort_b40c.cu:34-41: stable key-value sorts in place,
 * ascending (sort_val_f, sort_idx_f, sort_b40c_f) or descending (sort_rf,
 * sort_idx_rf); the _idx forms first fill the values with init, init+1, ... */
void sort_val_f(float *d_keys, uint32_t *d_vals, uint32_t N);
void sort_idx_f(float *d_keys_raw, uint32_t *d_idx_raw, uint32_t N, uint32_t init);
void sort_rf(float *d_keys, uint32_t *d_vals, uint32_t N);
void sort_idx_rf(float *d_keys_raw, uint32_t *d_idx_raw, uint32_t N, uint32_t init);
void sort_b40c_f(float *d_keys, uint32_t *d_vals, uint32_t N);

/* mvm.cu:22-56 (cublasSgemv, CUBLAS_OP_T): d_y[i] = sum_j d_A[i*n + j] *
 * d_x[j] for i < m, computed by the library's own kernel (the handle is
 * accepted and not used). */
void mvm_ff(cublasHandle_t handle, float *d_y, const float *d_A, const float *d_x, const uint32_t m,
            const uint32_t n);

#ifdef __cplusplus
}
#endif
#endif
