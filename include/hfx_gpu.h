/*
 * hfx_gpu.h -- C ABI of the GB300 SEQUEST search engine (libhfx_gpu.so).
 *
 * This is the drop-in boundary for the search path of kevyin/hfx.  In the
 * reference the Haskell host calls CUDA through `foreign import ccall`
 * (src/haskell/Foreign/CUDA/Algorithms.hs:44-371) into the functions declared
 * in src/common/include/algorithms.h:80-325, plus cuBLAS sgemv called
 * directly from Sequence/Search.hs:245 and :529.  Here the same work is
 * behind a context-based API: plain pointers and sizes, int32 status codes,
 * no C++ or torch types.  Each function names the reference interface it
 * replaces.
 *
 * Status codes: every call returns HFX_OK or an error; hfx_last_error()
 * gives the message.  (The reference checks no errors: utils.h:27-76.)
 */
#ifndef HFX_GPU_H
#define HFX_GPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define HFX_OK 0
#define HFX_ERR_ARG 1
#define HFX_ERR_OOM 2
#define HFX_ERR_CUDA 3
#define HFX_ERR_TIMEOUT 4
#define HFX_ERR_UNSUPPORTED 5

typedef struct hfx_ctx hfx_ctx;

/* Search parameters: the hfx.params / command-line keys that reach the
 * search path (Config.hs:55-104), plus the keys of the new engine. */
typedef struct hfx_search_params {
    float bin_width;               /* Correlation.hs:29-30: 1.0005079 mono, 1.0011413 average */
    int32_t custom_bin_width;      /* 1: bin_width is a custom width (e.g. 0.02 Da)           */
    int32_t remove_precursor_peak; /* remove-precursor-peak (Config.hs:312-317)               */
    int32_t tol_ppm;               /* 0: mass-tolerance in Da (Config.hs:308); 1: ppm; 2: per
                                      spectrum, tol < 0 is |tol| ppm, tol >= 0 is Da           */
    int32_t top_n;                 /* matches kept per spectrum, 1..32                         */
    int32_t precision;             /* 0 FP32 rows; 1 BF16 rows + FP32 rescore; 2 FP16 + rescore */
    int32_t rescore_k;             /* candidates rescored in FP32 (>= top_n; <= 64 when only   */
                                   /* unmodified candidates are list-scored, else <= 32)       */
    int32_t batch_mode;            /* 0 one launch per spectrum; 1 batched over per-step ion
                                      lists; 2 batched with ion lists rebuilt per work item    */
    int32_t fastdiv;               /* 1: __fdividef in ion m/z, as ion_series.cu:59-69         */
    int32_t search_plain;          /* score unmodified candidates                              */
    int32_t search_mods;           /* score variable-modification isoforms (needs hfx_set_mods) */
    int32_t group_size;            /* spectra per work item: 1, 2, 4, 8, or 16 (BF16/FP16 list
                                      scoring without modifications); 0 = default               */
    int32_t chunk;                 /* candidates per batched work item, 0 = default            */
    int32_t max_len;               /* longest spectrum row accepted, 0 = default (262,144)     */
    int32_t ion_bins_custom;       /* 1: ion bins use bin_width too (new; the reference bins
                                      ions with the mono width, ion_series.cu:68); rows longer
                                      than 8,192 bins only                                     */
    int32_t use_graph;             /* 1: replay the search as one CUDA graph while the batch
                                      shape, buffers and parameters repeat (batched modes)     */
} hfx_search_params;

/* Fill p with the engine defaults (reference behaviour where it has one). */
void hfx_default_params(hfx_search_params *p);

/* Create a context on CUDA device `device`.  All work is issued on the
 * context's stream (hfx_set_stream).  Replaces Execution.hs:49-53
 * withExecutionPlan (cuBLAS handle + streams). */
int32_t hfx_ctx_create(int32_t device, hfx_ctx **out);
int32_t hfx_ctx_destroy(hfx_ctx *ctx);
/* stream: a cudaStream_t passed as a pointer; NULL = the context's own. */
int32_t hfx_set_stream(hfx_ctx *ctx, void *stream);
const char *hfx_last_error(const hfx_ctx *ctx);

/* Stage timing: with profiling on, every search records CUDA events around
 * each stage on the context stream.  hfx_stage_stats returns, per stage,
 * accumulated milliseconds, kernel launches and units processed (spectra,
 * or peptide-spectrum pairs for the scoring stage).  New; the reference's
 * only timer is CPU time around the whole search (Util/Time.hs:42-47). */
#define HFX_STAGE_LAYOUT 0      /* per-spectrum layout, mass, window bounds */
#define HFX_STAGE_PREPROCESS 1  /* stage (a)                                */
#define HFX_STAGE_WINDOWS 2     /* stage (b), work planning                 */
#define HFX_STAGE_SCORE 3       /* stages (c)+(d): ion ladders, gather-dot  */
#define HFX_STAGE_TOPN 4        /* stage (e): top-N merge                   */
#define HFX_STAGE_RESCORE 5     /* FP32 rescoring of the kept candidates    */
#define HFX_STAGE_MODS 6        /* scoring of the modified isoforms         */
#define HFX_STAGE_LISTS 7       /* per-peptide ion lists of the batch       */
#define HFX_STAGE_PACK 8        /* interleaved spectrum tiles of the groups */
#define HFX_STAGE_MOD_LISTS 9   /* isoform windows, planning, ion lists     */
#define HFX_NSTAGES 10
int32_t hfx_set_profiling(hfx_ctx *ctx, int32_t on);
/* Caps the bytes of the context's search workspaces (new; the reference
 * sizes its dense matrices to the free memory, Search.hs:427-433): a call
 * whose workspaces would grow the context beyond `bytes` allocates nothing
 * more and returns HFX_ERR_OOM, and the context stays usable (raise the cap
 * and call again).  0 = no cap.  in_use (nullable) receives the bytes held
 * now.  The database and the per-call host staging are not counted. */
int32_t hfx_set_workspace_limit(hfx_ctx *ctx, uint64_t bytes, uint64_t *in_use);
int32_t hfx_stage_stats(hfx_ctx *ctx, double *ms, int64_t *launches, int64_t *units, int32_t reset);
/* Work counters of the batched list path, accumulated while profiling is on:
 * [0] ion lists built, [1] list entries built, [2] candidates scored,
 * [3] list entries streamed by the scorer, [4] peptide-spectrum pairs,
 * [5] candidate positions in the scorer's work items (active or not),
 * [6] residues read by the list generator (one peptide's once per step),
 * [7] spectrum-tile bytes staged into shared memory by the scorer. */
int32_t hfx_search_counters(hfx_ctx *ctx, uint64_t *out8, int32_t reset);
/* Work counters of the modification search over isoform lists
 * (batch_mode 1), accumulated while profiling is on: [0] isoform ion lists
 * built, [1] their entries, [2] isoforms handed to the scorer, [3] list
 * entries streamed by the scorer, [4] modified peptide-spectrum pairs,
 * [5] isoform records built, [6] residues read by the isoform-list
 * generator, [7] spectrum-tile bytes staged by the scorer. */
int32_t hfx_mod_counters(hfx_ctx *ctx, uint64_t *out8, int32_t reset);

/* Digest proteins into the search database and upload it.  Replaces
 * Fragment.hs:197-233 makeSeqDB + :239-258 withDeviceDB + sort.cu:28-35
 * sort_idx_f + prepare_ions.cu:105-132 prepare_ions.  seq: concatenated
 * upper-case residues, seg[nprot+1] protein offsets.  static_add26: add_X
 * static modifications (Config.hs:204-218), mono: aa-mass-type.
 * proline_rule / min_len / max_len extend the reference digest (its rule 1
 * ignores P and it has no length filter; 0 = off). */
/* The same digest on the device (new; the reference digests on the host,
 * Fragment.hs:197-233, 363-405): every residue that starts a piece walks
 * it, every piece start walks its joins, the kept fragments are placed by a
 * scan of their counts, so the output equals hfx_digest's element for
 * element (order, masses, tc, tn).  Host buffers in and out; r == NULL
 * returns the count only.  Returns the fragment count, -1 on bad arguments
 * or a CUDA failure (hfx_last_error says which), -2 when cap is too small.
 * hfx_build_db digests with it. */
int64_t hfx_digest_gpu(hfx_ctx *ctx, const uint8_t *seq, const uint32_t *seg, int32_t nprot, const float *mt26,
                       int32_t rule, int32_t missed, float min_mass, float max_mass, int32_t proline_rule,
                       int32_t min_len, int32_t max_len, float *r, uint32_t *tc, uint32_t *tn, int64_t cap);
int32_t hfx_build_db(hfx_ctx *ctx, const uint8_t *seq, const uint32_t *seg, int32_t nprot,
                     const float *static_add26, int32_t mono, int32_t rule, int32_t missed,
                     float min_mass, float max_mass, int32_t proline_rule, int32_t min_len,
                     int32_t max_len);
/* Host-only helpers (no device work), the two host steps of the database
 * build: the digest of Fragment.hs:363-405 into r/tc/tn (returns the
 * fragment count, -2 if cap is exceeded; pass r = NULL to count), and the
 * residue packing of prepare_ions.cu:29-52 (byte = (c-'A') | (ma index+1)<<5). */
int64_t hfx_digest(const uint8_t *seq, const uint32_t *seg, int32_t nprot, const float *mass_table26,
                   int32_t rule, int32_t missed, float min_mass, float max_mass, int32_t proline_rule,
                   int32_t min_len, int32_t max_len, float *r, uint32_t *tc, uint32_t *tn, int64_t cap);
int32_t hfx_pack_ions(const uint8_t *ascii, uint64_t n, const uint8_t *ma, int32_t num_ma, uint8_t *out);
/* Host-only: the residue mass table of Config.hs:266-272 (initializeAAMasses):
 * out26[c] = static_add26[c] (nullable: 0) + the mono or average mass of c. */
int32_t hfx_mass_table(int32_t mono, const float *static_add26, float *out26);

/* Upload a prebuilt database (r, tc, tn per fragment, ASCII residues) --
 * the SequenceDB fields of Fragment.hs:151-158. */
int32_t hfx_upload_db(hfx_ctx *ctx, const uint8_t *ions_ascii, uint64_t num_ions, const float *r,
                      const uint32_t *tc, const uint32_t *tn, uint64_t num_pep,
                      const float *mass_table26);
/* Database sizes and host copies: r, tc, tn per fragment in digest order,
 * idx_sorted[q] = the fragment at residual-mass position q. */
int32_t hfx_db_info(const hfx_ctx *ctx, uint64_t *num_ions, uint64_t *num_pep);
int32_t hfx_db_export(const hfx_ctx *ctx, float *r, uint32_t *tc, uint32_t *tn, uint32_t *idx_sorted,
                      float *mass_table26);

/* Variable modifications: mod_X keys (Config.hs:204-218) and
 * max-modable-acids; builds the combination table of Fragment.hs:260-289
 * and repacks the residues (prepare_ions.cu:105-132).  num_ma = 0 clears.
 * per_type selects the i-th acid counter: 0 = the reference kernel's
 * (mion_series.cu:252-269), 1 = per acid type (check_series.cu:62-100). */
int32_t hfx_set_mods(hfx_ctx *ctx, int32_t num_ma, const uint8_t *ma, const float *ma_mass,
                     int32_t max_ma, int32_t per_type);
int32_t hfx_mod_table(const hfx_ctx *ctx, int32_t *num_mod, int32_t *counts, float *deltas,
                      int32_t cap);

/* Full search of a batch of spectra, HOST buffers in and out (the host
 * copies are part of the call).  Replaces Search.hs:98-124 searchForMatches
 * (stages a-e and the per-spectrum sort).  Spectrum i has peaks
 * [off[i], off[i+1]) of mz/it (sorted by m/z), precursor m/z pcr[i],
 * charge z[i], tolerance tol[i].  Outputs, top_n per spectrum in final
 * order: score (raw XCorr; the displayed value is score/10000,
 * Search.hs:122), key (position in mass order for plain matches;
 * 1<<63 | mod<<54 | position<<27 | isoform rank for modified ones), pep
 * (fragment index), ncand[i] = candidates scored. */
int32_t hfx_search_host(hfx_ctx *ctx, const hfx_search_params *p, const float *mz, const float *it,
                        const int64_t *off, const float *pcr, const float *z, const float *tol,
                        int32_t nspec, float *out_score, uint64_t *out_key, uint32_t *out_pep,
                        int64_t *out_ncand);
/* The same with DEVICE buffers (inputs resident in HBM). */
int32_t hfx_search_device(hfx_ctx *ctx, const hfx_search_params *p, const float *mz, const float *it,
                          const int64_t *off, const float *pcr, const float *z, const float *tol,
                          int32_t nspec, float *out_score, uint64_t *out_key, uint32_t *out_pep,
                          int64_t *out_ncand);
/* The device-buffer search plus E-values (Util/Statistics.hs:37-100, applied
 * per spectrum at Search.hs:119-123): every candidate's FP32 score -- the
 * unmodified candidates and, in a modification search, every modified
 * isoform, as the reference fits over all matches of the spectrum
 * (Search.hs:116-121) -- is computed on the device, each spectrum's ascending scores are sliced at
 * round(0.3 n) .. round((1 - cutoff_perc/100) n), shifted by 1 - min, kept
 * above 4000 and binned by bin_width; an ordinary least-squares line through
 * (bin centre / 10000, log10(count / bin_width)) gives alpha and beta, and a
 * result of score s gets 10 ** (alpha + beta * s / 10000).  out_ev [nspec]
 * [top_n] (NaN for empty slots), out_fit [nspec][3] = alpha, beta, histogram
 * points.  The reference's defaults are bin_width 350 and cutoff_perc 3.
 * Without modifications the search runs as one FP32 pass over the step's
 * ion lists whatever p->precision asks (its top-N equals the BF16/FP16
 * search rescored in FP32; group_size is chosen for FP32); with
 * modifications the requested search runs first and a second FP32 pass
 * scores every pair. */
int32_t hfx_search_evalues(hfx_ctx *ctx, const hfx_search_params *p, const float *mz, const float *it,
                           const int64_t *off, const float *pcr, const float *z, const float *tol, int32_t nspec,
                           int32_t bin_width, float cutoff_perc, float *out_score, uint64_t *out_key,
                           uint32_t *out_pep, int64_t *out_ncand, double *out_ev, double *out_fit);
/* The "Ions" column of the results (Match.hs:36-44 scoreSP over
 * IonSeries.hs:87-147), device buffers: for each result key of the last
 * search on this context (hfx_search, hfx_search_device or
 * hfx_search_evalues over the same nspec spectra; z the same charges and p
 * the same bin width), out_matched / out_total [nspec][top_n] = matched b
 * and y ions / (peptide text length - 5) * 2.  The peaks are the 200 largest
 * values of the spectrum's preprocessed row (ties at the 200th value taken
 * in index order), binned by index / 3; the ions are the b ladder of the
 * unmodified peptide for charges 1 .. max(1, z-1) as (m + H*c) / c and
 * (M+H)+ minus each, binned by round(mz / bin_width / 3) (host masses).
 * Empty slots get 0 / 0. */
int32_t hfx_match_ions(hfx_ctx *ctx, const hfx_search_params *p, const float *z, int32_t nspec,
                       const uint64_t *keys, int32_t top_n, int32_t *out_matched, int32_t *out_total);
/* Result record of one match (Match.hs:17-27): Location.hs:42-58 lookup --
 * the peptide text "X.PEPTIDE.Y" with its flanking residues ('-' at a
 * protein end) and (M+H)+ = residual + H + H2O (host masses) -- and for a
 * modified key Fragment.hs:84-106 modifyFragment: the combination's mass
 * added and '*' after each modified residue (the i-th occurrence of its acid
 * in the text, i from the isoform's unrank row).  key/pep as returned by the
 * search; protein (nullable) receives the protein index.  Proteins come from
 * hfx_build_db's segments (hfx_set_protein_segments after hfx_upload_db). */
int32_t hfx_match_peptide(hfx_ctx *ctx, uint64_t key, uint32_t pep, char *text, int32_t cap, float *mh,
                          int32_t *protein);
int32_t hfx_set_protein_segments(hfx_ctx *ctx, const uint32_t *seg, int32_t nprot);
/* Autotuner (new): times the batched search of this batch (device buffers,
 * as hfx_search_device) for each spectra-per-group size G and work-item
 * size (candidates per item) it supports, `reps` timed runs each after one
 * warm-up, and writes the fastest into p->group_size and p->chunk.  The
 * outputs hold the last search's results.  ms_out (nullable) receives the
 * best time per search.  With the environment variable HFX_AUTOTUNE_FILE
 * naming a text file, the choice is persisted there per batch shape (the
 * device, database and batch sizes, and the settings that pick the
 * kernels): a later call with the same shape, in any process, reads it back
 * and runs one search instead of timing them all. */
int32_t hfx_autotune(hfx_ctx *ctx, hfx_search_params *p, const float *mz, const float *it, const int64_t *off,
                     const float *pcr, const float *z, const float *tol, int32_t nspec, float *out_score,
                     uint64_t *out_key, uint32_t *out_pep, int64_t *out_ncand, int32_t reps, float *ms_out);

/* Stage (a) alone, device buffers: Correlation.hs:37-109 sequestXCorr.
 * rows[nspec][stride] FP32 (+ optional BF16 / FP16 copies), lens[nspec]
 * (0 for a rejected spectrum), masses[nspec] = ms2Mass (Data.hs:58-59). */
int32_t hfx_preprocess(hfx_ctx *ctx, const hfx_search_params *p, const float *mz, const float *it,
                       const int64_t *off, const float *pcr, const float *z, int32_t nspec,
                       int64_t stride, float *rows, void *rows_bf16, void *rows_fp16, int32_t *lens,
                       float *masses);
/* Stage (b) alone, device buffers: filter.cu:75-127 findSpecCandsByMass
 * (windows in residual-mass order, end exclusive). */
int32_t hfx_find_windows(hfx_ctx *ctx, const hfx_search_params *p, const float *mz, const int64_t *off,
                         const float *pcr, const float *z, const float *tol, int32_t nspec,
                         uint32_t *begin, uint32_t *end);
/* Stage (c) alone, device buffers: the distinct ion bins of candidates at
 * mass-order positions pos[n] (ion_series.cu:150-232 addIons without the
 * dense row): bins ascending, level 1/2/3 = intensity 10/25/50, capped at
 * cap per candidate; count[i] may exceed cap. */
int32_t hfx_ion_bins(hfx_ctx *ctx, const uint32_t *pos, const int32_t *charges, const int32_t *lens,
                     int32_t n, int32_t cap, int32_t fastdiv, uint32_t *bins, uint8_t *levels,
                     int32_t *count);
/* Stage (e) alone, device buffers: for queries (mass-order position pos[i],
 * combination mod[i] of hfx_mod_table, isoform rank[i]) the isoform count
 * of the candidate (0 when not modable; filter_by_mod.cu:216-261,
 * calc_mod_cands.cu:49-66), and when rank[i] < count the unranked
 * occurrence indices (unrank[i*8 ..], acids ascending, each acid's indices in
 * the order of combinatorics.h:90-134; gen_mod_pep.cu:127-227) and the
 * per-residue modified flags (modded[i*cap + residue], mion_series.cu:244-286). */
int32_t hfx_mod_isoforms(hfx_ctx *ctx, const uint32_t *pos, const int32_t *mod, const uint32_t *rank,
                         int32_t n, int32_t cap, uint32_t *count, uint32_t *unrank, uint8_t *modded);

/* Allocation-free scoring of ONE spectrum.  It has no counterpart in the
 * reference.  It is for callers that cannot call cudaMalloc: code running
 * inside another framework's memory pool or allocator hooks, host runtimes
 * whose only device memory is what they were handed, and latency-critical
 * paths that must not take the allocator's locks.  It needs no context; the
 * caller passes every input and output as a device buffer:
 *   ions, r_sorted, tc_sorted, tn_sorted, idx_sorted[num_pep]: the
 *     database in residual-mass order (hfx_db_export gives the host copies,
 *     hfx_pack_ions the packed residues); mass_table26 is a HOST array;
 *   row[len]: the spectrum's FP32 row (hfx_preprocess), len <= 8192;
 *   charges: ion charges 1..4 (0 = none); [begin, end): the candidate window
 *     in mass order (hfx_find_windows);
 *   out_score / out_key / out_pep[top_n]: the top_n matches in final order,
 *     top_n <= 32, with the keys and scores of hfx_search_* (plain matches).
 * Its only scratch is a file-scope device array of
 * HFX_NOALLOC_MAX_BLOCKS * 32 * 12 bytes (117 KB) that every GPU loading the
 * library holds until exit.  Every call looks up that array's device
 * address (cudaGetSymbolAddress) and sets the kernels' shared-memory limit,
 * host calls that allocate nothing, so a call stays correct after a device
 * reset; the first call on a device also loads the kernels there: make it
 * before any stream capture.  Every call shares the one array, so calls
 * that overlap on the GPU (two streams, two threads) race: serialize them.
 * Work is issued on `stream` (a cudaStream_t; NULL = the legacy default
 * stream) and is asynchronous.  Returns HFX_ERR_ARG for sizes beyond these
 * limits, and HFX_ERR_CUDA without launching anything when a CUDA error of
 * earlier work is already pending on the calling thread (that error is left
 * pending for its owner). */
#define HFX_NOALLOC_MAX_BLOCKS 304
int32_t hfx_score_spectrum_noalloc(const uint8_t *ions, const float *r_sorted, const uint32_t *tc_sorted,
                                   const uint32_t *tn_sorted, const uint32_t *idx_sorted, uint32_t num_pep,
                                   const float *mass_table26, const float *row, int32_t len, int32_t charges,
                                   uint32_t begin, uint32_t end, int32_t top_n, int32_t fastdiv, void *stream,
                                   float *out_score, uint64_t *out_key, uint32_t *out_pep);

#ifdef __cplusplus
}
#endif
#endif
