/*
 * CPU oracle for the SEQUEST search hot path (TEST INFRASTRUCTURE ONLY).
 *
 * This library is the checker, not the product.  Only tests/, the smoke test
 * in __graft_entry__.py and the cpu_baseline leg of bench.py may load it.
 * The product (hfx_gb300/, libhfx_gpu.so) never links or calls it.
 *
 * It restates, step by step, the reference's search arithmetic:
 *   stage (a) Spectrum/Correlation.hs:29-109, Spectrum/Data.hs:58-59
 *   digest    Sequence/Fragment.hs:197-233, 363-405, Config.hs:266-272, 415-431
 *   stage (b) cuda/filter/filter.cu:75-127, cuda/filter/filter_by_mod.cu:35-143
 *   stage (c) cuda/ion_series/ion_series.cu:25-232, ion_series.h:16-26,
 *             cuda/ion_series/mion_series.cu:143-328
 *   stage (e) Sequence/Fragment.hs:260-289, filter_by_mod.cu:145-378,
 *             gen_mod_pep/calc_mod_cands.cu:27-119, prepare_gen_mod.cu:23-129,
 *             gen_mod_pep.cu:127-312, common/include/combinatorics.h:13-134,
 *             misc/prepare_ions.cu:29-132, common/include/utils.h:92-101
 *   order     Sequence/Search.hs:118-124, 247-276, 565-617 (b40c + sortBy)
 *
 * Two numeric modes: "ref32" (FP32, the reference's operation order, IEEE
 * division where the device used __fdividef) and "fp64" (same integer
 * decisions, values in double).  Parity against the running reference is
 * unpinned for the Haskell and cuBLAS parts (neither can run here); the
 * combinatorics are pinned against the reference's own header compiled from
 * its sources (oracle/Makefile, target ref).
 */
#ifndef HFX_ORACLE_H
#define HFX_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Config.hs:266-272: table[c] = static_add[c] + residue mass (mono/avg). */
void hfxo_mass_table(int mono, const float *static_add26, float *out26);

/* Fragment.hs:363-405 digest of concatenated proteins seq[seg[i]..seg[i+1]).
 * Returns fragment count (or -1 if cap exceeded).  true_len receives the
 * number of residues of each fragment. */
int64_t hfxo_digest(const uint8_t *seq, const uint32_t *seg, int32_t nprot,
                    const float *mt26, int rule, int missed, float min_mass,
                    float max_mass, int proline_rule, int min_len, int max_len,
                    float *r, uint32_t *tc, uint32_t *tn, int64_t cap);

/* sort.cu:28-35 stable key-value sort of residual masses with iota. */
void hfxo_sort_idx(const float *r, int64_t n, uint32_t *idx);

/* prepare_ions.cu:29-132 packing, byte = (c-'A') | (ma_index+1)<<5.
 * reference_quirk=1 reproduces the zero-block launch for n < 512 (no-op). */
void hfxo_pack_ions(uint8_t *ions, int64_t n, const uint8_t *ma, int num_ma,
                    int reference_quirk);

/* Spectrum/Data.hs:58-59 */
float hfxo_ms2_mass(float pcr, float z);

/* Correlation.hs:58-67: vector length 75 + ceiling cutoff (custom_bw: the
 * cutoff is divided by the bin width first).  -1 on an empty spectrum. */
int32_t hfxo_spec_len(const float *mz, int32_t npk, float pcr, float z,
                      float bw, int custom_bw);

/* Correlation.hs:37-109.  Writes len values to out32 (ref32) and/or out64
 * (fp64 values with the ref32 integer decisions).  Returns len or <0. */
int32_t hfxo_preprocess(const float *mz, const float *it, int32_t npk,
                        float pcr, float z, float bw, int custom_bw,
                        int remove_pcr, float *out32, double *out64,
                        int32_t cap);

/* filter.cu:101-115 lower_bound(lo) / upper_bound(hi) on the sorted masses. */
void hfxo_windows(const float *r_sorted, int64_t n, const float *lo,
                  const float *hi, int64_t nq, uint32_t *begin, uint32_t *end);

/* ion_series.cu:150-232 (mods: mion_series.cu:215-307).  Sorted distinct
 * in-range bins (ascending) with level 1/2/3 = weight 10/25/50.  res_add is
 * NULL or per-residue added mass (modified residues).  charges = number of
 * charges (0 = none).  Returns count or -1 if cap exceeded. */
int32_t hfxo_ion_bins(const uint8_t *ions, const float *mt26, uint32_t tc,
                      uint32_t tn, float residual, int32_t charges,
                      int32_t len, const float *res_add, const uint8_t *modded,
                      uint32_t *bins, uint8_t *lvl, int32_t cap);

/* Ion charges used for a spectrum charge z (Search.hs:182, ion_series.cu:301,
 * mion_series.cu:425-438). */
int32_t hfxo_ion_charges(float z, int is_mod);

/* Canonical score: entry i accumulated by lane i%32 with fmaf, then an XOR
 * butterfly (16,8,4,2,1).  x32 is the stored row converted to float. */
float hfxo_score32(const uint32_t *bins, const uint8_t *lvl, int32_t n,
                   const float *x);
double hfxo_score64(const uint32_t *bins, const uint8_t *lvl, int32_t n,
                    const double *x);

/* combinatorics.h:59-134 */
uint32_t hfxo_choose(uint32_t n, uint32_t k);
void hfxo_unrank_comb(uint32_t *ans, uint32_t n, uint32_t k, uint32_t rank);

/* Fragment.hs:260-289 makeModInfo.  counts[num_mod][num_ma], sums, deltas.
 * Returns num_mod (or -1 if cap exceeded). */
int32_t hfxo_mod_combos(int32_t num_ma, int32_t max_ma, const float *ma_mass,
                        int32_t *counts, int32_t *sums, float *deltas,
                        int32_t cap);

/* One modified isoform: count of each modable acid in [tc,tn)
 * (filter_by_mod.cu:216-230), isoform count and per-acid suffix products
 * (calc_mod_cands.cu:49-66), and for rank < count the unrank row
 * (gen_mod_pep.cu:127-227) plus the per-residue modified flags
 * (mion_series.cu:244-286; per_type=1 uses the serial checker's per-type
 * counter, check_series.cu:62-100).  Returns the isoform count, 0 if not
 * modable. */
uint32_t hfxo_mod_isoform(const uint8_t *ions, uint32_t tc, uint32_t tn,
                          const uint8_t *ma, int32_t num_ma,
                          const int32_t *mod_counts, uint32_t rank,
                          int per_type, uint32_t *unrank_out,
                          uint8_t *modded_out);

/* Full search (Search.hs:98-124).  Results per spectrum: top-n entries in
 * final order; key = position in mass order for plain matches, or
 * 1<<63 | mod<<54 | pos<<27 | rank for modified ones.
 * prec: 0 = ref32 canonical FP32, 1 = bf16-stored row, 2 = fp16-stored row,
 * 3 = fp64 (score64 cast to float in out_score, exact in out_score64).
 * tol: per spectrum tolerance; ppm != 0 means tolerance in ppm. */
typedef struct {
    float bw;            /* spectrum bin width (Correlation.hs:29-30)          */
    int32_t custom_bw;   /* 1: bw is a custom width (len formula divides)      */
    int32_t remove_pcr;  /* remove-precursor-peak (Config.hs:63)               */
    int32_t ppm;         /* 0 Da, 1 ppm, 2 per spectrum: negative = ppm (new) */
    int32_t topn;        /* entries kept per spectrum                          */
    int32_t prec;        /* see above                                          */
    int32_t num_ma;      /* variable modifications: 0 = none                   */
    int32_t max_ma;
    int32_t per_type;    /* i-th acid counter: 0 reference, 1 per type         */
    int32_t plain;       /* 1: score unmodified candidates                     */
    uint8_t ma[16];
    float ma_mass[16];
    float ion_bw;        /* 0: ion bins use the mono width (ion_series.cu:68); */
                         /* > 0: ion bins use this width (new, 0.02 Da rows)   */
} hfxo_params;

int32_t hfxo_search(const uint8_t *ions, const float *mt26, const float *r,
                    const uint32_t *tc, const uint32_t *tn,
                    const uint32_t *idx_sorted, int64_t num_pep,
                    const float *mz, const float *it, const int64_t *off,
                    const float *pcr, const float *z, const float *tol,
                    int32_t nspec, const hfxo_params *p, int32_t nthreads,
                    float *out_score, double *out_score64, uint64_t *out_key,
                    uint32_t *out_pep, int64_t *out_ncand);

/* The "Ions" column of one match (Match.hs:36-44 scoreSP over
 * IonSeries.hs:87-147 extractPeaks / matchIonSequence / bions):
 *   peaks: the 200 largest values of the spectrum's sequestXCorr vector x
 *          (ties: lower index first), each max'ed (from 0) into bin i/3 of
 *          len/3 + 1 bins;
 *   ions:  for charge c = 1, 2, ... while c <= max(1, z-1) + 1/2 (Float
 *          enumeration), the ladder of prefix sums of the peptide's residue
 *          masses (mt26, the last one the whole peptide), each as
 *          (m + H*c) / c (host H);
 *   b = every ion but the last of the whole list, y = mh - ion for every
 *   ion but the first; an ion matches when round((v / bw) / 3) (halves to
 *   even) is a peak bin with a value above 0;
 *   matched = matching b + y; total = (text length - 5) * 2 with the text
 *   "X.PEPTIDE.Y" plus one '*' per modified residue (nstar).
 * pep[L]: the letters of the unmodified peptide; mh: its (M+H)+
 * ((res + H) + H2O, host masses). */
void hfxo_match_ions(const float *x, int32_t len, float z, float bw,
                     const uint8_t *pep, int32_t L, const float *mt26, float mh,
                     int32_t nstar, int32_t *matched, int32_t *total);

/* As hfxo_search, and also every candidate's score (plain candidates in
 * mass order, then modified isoforms by combination, position and rank) at
 * sink[sink_off[s] ...]: the score list the reference hands to its E-value
 * fit (Search.hs:116-121, every match of the spectrum, modified or not).
 * sink_off per spectrum: exclusive prefix sum of out_ncand. */
int32_t hfxo_search_scores(const uint8_t *ions, const float *mt26, const float *r,
                           const uint32_t *tc, const uint32_t *tn,
                           const uint32_t *idx_sorted, int64_t num_pep,
                           const float *mz, const float *it, const int64_t *off,
                           const float *pcr, const float *z, const float *tol,
                           int32_t nspec, const hfxo_params *p, int32_t nthreads,
                           float *out_score, double *out_score64, uint64_t *out_key,
                           uint32_t *out_pep, int64_t *out_ncand,
                           const int64_t *sink_off, float *sink);

#ifdef __cplusplus
}
#endif
#endif
