/* The reference's text output (Util/PrettyPrint.hs:83-180), served by
 * libhfx_gpu.so (host code only).
 *
 * Every function writes the text (NUL-terminated, truncated to cap bytes)
 * and returns its full length in bytes, so a first call with cap = 0 sizes
 * the buffer.  Numbers follow GHC's Numeric: shortest round-trip digits,
 * then rounding of those digits (halves up) to the shown places.
 */
#ifndef HFX_REPORT_H
#define HFX_REPORT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One match as printResults shows it (toDoc, PrettyPrint.hs:110-125). */
typedef struct {
    float mh;                /* fragmass: (M+H)+ of the (modified) fragment          */
    float xcorr;             /* scoreXC as shown: the raw score / 10000              */
    int32_t ions_matched;    /* scoreSP (hfx_match_ions)                             */
    int32_t ions_total;
    const char *reference;   /* fraglabel: first word of the protein header          */
    const char *peptide;     /* fragdata: "X.PEPTIDE.Y", '*' after modified residues */
    double evalue;
    const char *scan;        /* ms2info (printAllResults only)                       */
    const char *file;        /* the spectrum file (printAllResults only)             */
} hfx_result_row;

/* printResults (all = 0: # (M+H)+ deltCn XCorr Ions Reference Peptide
 * E-value) or printAllResults (all = 1: the same plus Scan details and File),
 * rows in the order given; deltCn = (s0 - XCorr) / s0 with s0 the first
 * row's XCorr. */
int64_t hfx_format_results(const hfx_result_row *rows, int32_t n, int32_t all, char *out, int64_t cap);
/* printConfig (PrettyPrint.hs:83-97): Title, Spectrum, Database, Enzyme and
 * "(M+H)+ Mass :: m ~ tol (+z)" with m = pcr * z - (z * H - 1); enzyme:
 * the words printed after the rule number. */
int64_t hfx_format_config(const char *title, const char *spectrum, const char *database, const char *enzyme,
                          float pcr, float charge, float tol, char *out, int64_t cap);
/* printResultsDetail (PrettyPrint.hs:127-133): each protein header
 * flowed into 95 columns beside its right-aligned number. */
int64_t hfx_format_detail(const char *const *headers, int32_t n, char *out, int64_t cap);
/* ppAsRows q (PrettyPrint.hs:199-211) over nrows x ncols cells, row-major. */
int64_t hfx_format_rows(const char *const *cells, int32_t nrows, int32_t ncols, int32_t q, char *out, int64_t cap);
/* One number: kind 0 = show (Float), 1 = showFFloat (Just 4) of a Float,
 * 2 = showFFloat (Just 4) of a Double, 3 = showEFloat (Just 4) of a
 * Double. */
int64_t hfx_format_number(double x, int32_t kind, char *out, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
