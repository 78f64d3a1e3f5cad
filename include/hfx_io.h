/* Input formats on both sides of the search, served by libhfx_gpu.so (host
 * code only; no call here touches the GPU).
 *
 *   spectra   Spectrum.hs:38-47 readMS2Data, by file suffix:
 *             "dta"  Spectrum/DTA.hs:35-68  (first line "(M+H)+ charge", then peaks)
 *             "mgf"  Spectrum/MGF.hs:31-75 (BEGIN IONS / TITLE, CHARGE, PEPMASS / peaks / END IONS)
 *             with the value grammar of Util/Parsec.hs:25-85
 *   proteins  Sequence/Fasta.hs:27-36 readFasta (".gz" inflated), laid out as
 *             makeSeqDB does (Sequence/Fragment.hs:197-233, 336-352): residues
 *             concatenated, segments = running sum of the protein lengths
 *   index     Sequence/Index.hs:40-82 writeIndex / readIndex: the options
 *             text, then gzip of the serialised SequenceDB (Fragment.hs:165-172)
 *
 * Results are owned by opaque handles; the accessors return pointers into
 * them, valid until the handle is freed.  Every call returns HFX_OK (0) or
 * HFX_ERR_ARG (1) with a message in err (nullable, errcap bytes).
 */
#ifndef HFX_IO_H
#define HFX_IO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hfx_spectra hfx_spectra;
typedef struct hfx_proteins hfx_proteins;
typedef struct hfx_index hfx_index;

/* readMS2Data on a file (suffix, any case: dta or mgf). */
int32_t hfx_read_spectra(const char *path, hfx_spectra **out, char *err, int32_t errcap);
/* The same on text in memory; kind 0 = DTA, 1 = MGF. */
int32_t hfx_parse_spectra(const char *text, int64_t n, int32_t kind, hfx_spectra **out, char *err, int32_t errcap);
/* Spectra, peaks in file order: mz/it [peaks], off [count + 1], precursor
 * m/z and charge [count] (MS2Data, Spectrum/Data.hs:47-53). */
int64_t hfx_spectra_count(const hfx_spectra *s);
void hfx_spectra_arrays(const hfx_spectra *s, const float **mz, const float **it, const int64_t **off,
                        const float **pcr, const float **z);
/* ms2info: the MGF TITLE (empty for DTA); len receives its length. */
const char *hfx_spectra_title(const hfx_spectra *s, int64_t i, int64_t *len);
void hfx_spectra_free(hfx_spectra *s);

/* readFasta on a file (inflated when the name ends in ".gz"). */
int32_t hfx_read_fasta(const char *path, hfx_proteins **out, char *err, int32_t errcap);
/* The same on bytes in memory (gz: gzip-compressed). */
int32_t hfx_parse_fasta(const uint8_t *data, int64_t n, int32_t gz, hfx_proteins **out, char *err, int32_t errcap);
/* seq [seg[count]] residues, seg [count + 1] (dbIon, dbIonSeg). */
int64_t hfx_proteins_count(const hfx_proteins *p);
void hfx_proteins_arrays(const hfx_proteins *p, const uint8_t **seq, const uint32_t **seg);
/* dbHeader: the header line after '>'. */
const char *hfx_proteins_header(const hfx_proteins *p, int64_t i, int64_t *len);
void hfx_proteins_free(hfx_proteins *p);

/* readIndex: the options text (key = value lines, Index.hs:47-57) and the
 * database (SeqDB: headers, ions, ion segments, fragments (r, c, n),
 * fragment segments). */
int32_t hfx_read_index(const char *path, hfx_index **out, char *err, int32_t errcap);
int32_t hfx_parse_index(const uint8_t *data, int64_t n, hfx_index **out, char *err, int32_t errcap);
const char *hfx_index_options(const hfx_index *x, int64_t *len);
void hfx_index_sizes(const hfx_index *x, int64_t *num_headers, int64_t *num_ions, int64_t *num_frags);
const char *hfx_index_header(const hfx_index *x, int64_t i, int64_t *len);
void hfx_index_arrays(const hfx_index *x, const uint8_t **ions, const uint32_t **ion_seg, const float **r,
                      const uint32_t **c, const uint32_t **n, const uint32_t **frag_seg);
void hfx_index_free(hfx_index *x);
/* writeIndex: the same layout, the database gzip-compressed with stored
 * (uncompressed) deflate blocks.  headers: num_headers strings. */
int32_t hfx_write_index(const char *path, const char *options, int64_t num_headers, const char *const *headers,
                        const uint8_t *ions, int64_t num_ions, const uint32_t *ion_seg, const float *r,
                        const uint32_t *c, const uint32_t *n, int64_t num_frags, const uint32_t *frag_seg,
                        char *err, int32_t errcap);

#ifdef __cplusplus
}
#endif
#endif
