// The protein digest of the database build on the device (hfx_digest_gpu).
//
// The reference digests on the host while it builds its sequence database:
// `makeSeqDB` / `digest` / `fragment` / `splice` (Sequence/Fragment.hs:197-233,
// 363-405) with the cleavage rules of Config.hs:415-431.  A protein is cut
// after every residue of the rule's set (with the optional proline rule:
// not before P); the pieces are joined with up to `missed` following pieces;
// a joined fragment is kept when (M + H2O) + H lies in [min, max] (host
// masses, Mass.hs:20-25) and, optionally, its length in [min_len, max_len].
// A fragment's residues are [tc, tn] for a piece ending at a cut residue
// (tn = that residue's index, so the ion ladder over [tc, tn) skips it) and
// [tc, tn) with tn one past the protein's end for its last piece.
//
// Here every residue is a thread: a residue that starts a piece (the
// protein's first residue, or the one after a cut) walks to its piece's end,
// summing the residue masses in order (the reference's left fold); then
// every piece start walks the joins of up to `missed` following pieces,
// counting (pass 1) and writing (pass 2) the fragments it keeps, at offsets
// from a scan of the counts, so the output order is the reference's:
// protein, piece, number of joined pieces.
#include <algorithm>

#include "hfx_internal.h"
#include "../../include/hfx_gpu.h"

namespace hfx {
namespace {

constexpr uint32_t kNoPiece = 0xFFFFFFFFu;
constexpr float kDigestH2O = 18.010565f;  // Mass.hs:20
constexpr float kDigestH = 1.007276f;     // Mass.hs:25

struct DigestArgs {
    const uint8_t *seq;   // upper-case residues 'A'..'Z'
    const uint32_t *seg;  // nprot + 1 protein offsets
    int32_t nprot;
    uint32_t nres;
    float mt[26];
    uint32_t rule_mask;   // bit c - 'A': cleave after residue c
    int32_t proline, missed, min_len, max_len;
    float min_mass, max_mass;
};

__device__ __forceinline__ uint32_t protein_end(const DigestArgs &a, uint32_t j, uint32_t *start) {
    // last protein whose offset is <= j (upper bound - 1)
    int32_t lo = 0, hi = a.nprot;
    while (hi - lo > 1) {
        const int32_t mid = (lo + hi) >> 1;
        if (a.seg[mid] <= j) lo = mid;
        else hi = mid;
    }
    *start = a.seg[lo];
    return a.seg[lo + 1];
}

__device__ __forceinline__ bool cut_after(const DigestArgs &a, uint32_t i, uint32_t y) {
    if (!((a.rule_mask >> (a.seq[i] - 'A')) & 1u)) return false;
    return !(a.proline && i + 1 < y && a.seq[i + 1] == 'P');
}

// Pieces: for every residue that starts one, its mass, tn, length and the
// next piece's start (kNoPiece after the protein's last piece).
__global__ void k_digest_pieces(DigestArgs a, float *__restrict__ pm, uint32_t *__restrict__ ptn,
                                uint32_t *__restrict__ plen, uint32_t *__restrict__ pnext) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < a.nres; j += gridDim.x * blockDim.x) {
        plen[j] = 0u;
        if (j < a.seg[0]) continue;  // before the first protein
        uint32_t s0 = 0;
        const uint32_t y = protein_end(a, j, &s0);
        if (!(j == s0 || cut_after(a, j - 1, y))) continue;
        float m = 0.0f;
        uint32_t i = j;
        for (; i < y; ++i) {
            m = __fadd_rn(m, a.mt[a.seq[i] - 'A']);
            if (cut_after(a, i, y)) break;
        }
        pm[j] = m;
        if (i == y) {
            ptn[j] = y;
            plen[j] = y - j;
            pnext[j] = kNoPiece;
        } else {
            ptn[j] = i;
            plen[j] = i - j + 1;
            pnext[j] = i + 1 < y ? i + 1 : kNoPiece;
        }
    }
}

// The fragments a piece start keeps: itself joined with 0..missed following
// pieces.  Pass 1 counts them into cnt[j]; pass 2 writes them from the
// inclusive scan of the counts.
template <bool kWrite>
__global__ void k_digest_splice(DigestArgs a, const float *__restrict__ pm, const uint32_t *__restrict__ ptn,
                                const uint32_t *__restrict__ plen, const uint32_t *__restrict__ pnext,
                                int32_t *__restrict__ cnt, const int32_t *__restrict__ incl, float *__restrict__ r,
                                uint32_t *__restrict__ tc, uint32_t *__restrict__ tn, int64_t cap) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < a.nres; j += gridDim.x * blockDim.x) {
        int32_t n = 0;
        int64_t at = 0;
        if constexpr (kWrite) at = (int64_t)incl[j] - cnt[j];
        if (plen[j]) {
            uint32_t q = j;
            float m = pm[j];
            uint32_t len = plen[j];
            for (int k = 0; k <= a.missed; ++k) {
                if (k) {
                    q = pnext[q];
                    if (q == kNoPiece) break;
                    m = __fadd_rn(m, pm[q]);
                    len += plen[q];
                }
                const float mm = __fadd_rn(__fadd_rn(m, kDigestH2O), kDigestH);
                if (!(a.min_mass <= mm && mm <= a.max_mass)) continue;
                if (a.min_len > 0 && (int32_t)len < a.min_len) continue;
                if (a.max_len > 0 && (int32_t)len > a.max_len) continue;
                if constexpr (kWrite) {
                    if (at < cap) {
                        r[at] = m;
                        tc[at] = j;
                        tn[at] = ptn[q];
                    }
                    ++at;
                }
                ++n;
            }
        }
        if constexpr (!kWrite) cnt[j] = n;
    }
}

}  // namespace
}  // namespace hfx

using namespace hfx;

int hfx_scan_inclusive(const int32_t *in, int64_t n, int32_t *out, int32_t *partial, cudaStream_t st);

int hfx_digest_launch(const uint8_t *d_seq, const uint32_t *d_seg, int32_t nprot, uint32_t nres, const float *mt26,
                      int32_t rule_mask, int32_t missed, float min_mass, float max_mass, int32_t proline,
                      int32_t min_len, int32_t max_len, float *pm, uint32_t *ptn, uint32_t *plen, uint32_t *pnext,
                      int32_t *cnt, int32_t *incl, int32_t *partial, float *r, uint32_t *tc, uint32_t *tn,
                      int64_t cap, int pass, cudaStream_t st) {
    DigestArgs a;
    a.seq = d_seq;
    a.seg = d_seg;
    a.nprot = nprot;
    a.nres = nres;
    for (int i = 0; i < 26; ++i) a.mt[i] = mt26[i];
    a.rule_mask = (uint32_t)rule_mask;
    a.proline = proline;
    a.missed = missed;
    a.min_len = min_len;
    a.max_len = max_len;
    a.min_mass = min_mass;
    a.max_mass = max_mass;
    if (nres == 0 || nprot <= 0) return 0;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned grid = (unsigned)std::min<uint64_t>((nres + 255) / 256, (uint64_t)sms * 16);
    if (pass == 1) {
        k_digest_pieces<<<grid, 256, 0, st>>>(a, pm, ptn, plen, pnext);
        k_digest_splice<false><<<grid, 256, 0, st>>>(a, pm, ptn, plen, pnext, cnt, nullptr, nullptr, nullptr, nullptr,
                                                     0);
        const int rc = (int)cudaGetLastError();
        if (rc) return rc;
        return hfx_scan_inclusive(cnt, (int64_t)nres, incl, partial, st);
    }
    k_digest_splice<true><<<grid, 256, 0, st>>>(a, pm, ptn, plen, pnext, cnt, incl, r, tc, tn, cap);
    return (int)cudaGetLastError();
}
