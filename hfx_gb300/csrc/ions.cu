// The "Ions" column of the matches (Match.hs:36-44 scoreSP over
// IonSeries.hs:87-147), computed on the device from the search's own
// preprocessed rows.  The reference builds it on the host for every match
// it keeps (Search.hs:137-139, 296-299).
//
// Per spectrum (one CTA):
//   peaks   extractPeaks: the 200 largest values of the sequestXCorr row,
//           each max'ed (from 0) into bin i/3 of len/3 + 1 bins; only
//           values above 0 can make a bin count, so the CTA radix-selects
//           the 200th largest positive value (8 bits a pass over the IEEE
//           bit pattern, which orders positive floats) and takes ties at
//           that value in index order;
//   per match (one thread): bions over the peptide text -- ladder prefix
//           sums of the residue masses for charges 1, 2, ... while
//           c <= max(1, z-1) + 1/2, each as (m + H*c) / c -- and
//           matchIonSequence: b = every ion but the last, y = (M+H)+ - ion
//           for every ion but the first, matching when round((v / w) / 3)
//           is a peak bin; total = (text length - 5) * 2, the text of a
//           modified match carrying one '*' per modified residue
//           (Fragment.hs:84-106), while the ions come from the unmodified
//           fragment (Search.hs:297).
// All arithmetic is single precision, one IEEE operation at a time, as the
// reference's Float code; H and H2O are the host masses (Mass.hs:20-25).
#include <cstdint>
#include "hfx_internal.h"
#include "ions.h"

namespace hfx {

constexpr int kIonThreads = 256;
constexpr int kTopPeaks = 200;            // IonSeries.hs:105-106
constexpr int kMaxIonCharges = 4096;      // bound on the charge loop (z is data)
constexpr float kIonH = 1.007276f;        // Mass.hs:25
constexpr float kIonH2O = 18.010565f;     // Mass.hs:20

__global__ void __launch_bounds__(kIonThreads)
k_match_ions(DevDB db, DevMods mods, uint64_t nion, const SpecMeta *__restrict__ meta,
             const float *__restrict__ rows, int64_t stride, const float *__restrict__ z, float bw,
             const uint64_t *__restrict__ keys, int32_t topn, int32_t *__restrict__ out_m,
             int32_t *__restrict__ out_t, uint32_t *__restrict__ err) {
    extern __shared__ uint32_t s_mask[];  // one bit per peak bin
    __shared__ uint32_t s_hist[256];
    __shared__ uint32_t s_warp[kIonThreads / 32];
    __shared__ uint32_t s_pos, s_sel, s_need, s_base;
    const int32_t s = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const SpecMeta m = meta[s];
    const int32_t len = m.status == 0 ? m.len : 0;
    const float *x = rows + (size_t)s * stride;
    const int32_t np = len / 3 + 1;
    const int32_t words = (np + 31) / 32;
    for (int32_t i = tid; i < words; i += blockDim.x) s_mask[i] = 0u;
    if (tid == 0) s_pos = 0u;
    __syncthreads();
    for (int32_t i = tid; i < len; i += blockDim.x)
        if (x[i] > 0.0f) atomicAdd(&s_pos, 1u);
    __syncthreads();
    const bool all = s_pos <= (uint32_t)kTopPeaks;
    // radix select of the 200th largest positive value: T and how many of
    // the values equal to T are among the 200
    uint32_t prefix = 0u, pmask = 0u, need = kTopPeaks, eq_count = 0u;
    if (!all) {
        for (int shift = 24; shift >= 0; shift -= 8) {
            for (int i = tid; i < 256; i += blockDim.x) s_hist[i] = 0u;
            __syncthreads();
            for (int32_t i = tid; i < len; i += blockDim.x) {
                const float v = x[i];
                const uint32_t u = __float_as_uint(v);
                if (v > 0.0f && (u & pmask) == prefix) atomicAdd(&s_hist[(u >> shift) & 255u], 1u);
            }
            __syncthreads();
            if (tid == 0) {
                uint32_t acc = 0u;
                int d = 255;
                for (; d > 0; --d) {
                    if (acc + s_hist[d] >= need) break;
                    acc += s_hist[d];
                }
                s_sel = (uint32_t)d;
                s_need = need - acc;
            }
            __syncthreads();
            prefix |= s_sel << shift;
            pmask |= 255u << shift;
            need = s_need;
            eq_count = s_hist[s_sel];
            __syncthreads();
        }
    }
    const uint32_t T = prefix;
    const bool take_all_eq = all || need >= eq_count;
    for (int32_t i = tid; i < len; i += blockDim.x) {
        const float v = x[i];
        const uint32_t u = __float_as_uint(v);
        if (v > 0.0f && (all || u > T || (u == T && take_all_eq))) {
            const int32_t b = i / 3;
            atomicOr(&s_mask[b >> 5], 1u << (b & 31));
        }
    }
    if (!take_all_eq) {
        // ties at T: the first `need` of them in index order
        if (tid == 0) s_base = 0u;
        __syncthreads();
        for (int32_t base = 0; base < len; base += blockDim.x) {
            const int32_t i = base + tid;
            const bool eq = i < len && x[i] > 0.0f && __float_as_uint(x[i]) == T;
            const uint32_t bal = __ballot_sync(0xFFFFFFFFu, eq);
            if (lane == 0) s_warp[warp] = __popc(bal);
            __syncthreads();
            uint32_t before = s_base;
            for (int w = 0; w < warp; ++w) before += s_warp[w];
            const uint32_t rank = before + __popc(bal & ((1u << lane) - 1u));
            if (eq && rank < need) {
                const int32_t b = i / 3;
                atomicOr(&s_mask[b >> 5], 1u << (b & 31));
            }
            __syncthreads();
            if (tid == 0)
                for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s_base += s_warp[w];
            __syncthreads();
        }
    }
    __syncthreads();
    for (int32_t j = tid; j < topn; j += blockDim.x) {
        const size_t o = (size_t)s * topn + j;
        const uint64_t key = keys[o];
        int32_t matched = 0, total = 0;
        if (key != ~0ull && len > 0) {
            const bool modded = (key >> 63) != 0ull;
            const uint32_t pos = modded ? (uint32_t)((key >> 27) & ((1u << 27) - 1u)) : (uint32_t)key;
            if (pos >= db.num_pep || (!modded && key >= (uint64_t)db.num_pep)) {
                atomicOr(err, kErrBounds);
            } else {
                const uint32_t tc = db.tc_sorted[pos], tn = db.tn_sorted[pos];
                // Location.hs:50-58: the text holds residue n too, except at
                // the end of the database
                const int32_t L = (int32_t)((uint64_t)tn < nion ? tn - tc + 1u : tn - tc);
                int32_t nstar = 0;
                if (modded) {
                    const int32_t mu = (int32_t)((key >> 54) & 511u);
                    if (mu < mods.num_mod)
                        for (int a = 0; a < mods.num_ma; ++a) nstar += mods.counts[(size_t)mu * mods.num_ma + a];
                }
                const float mh = __fadd_rn(__fadd_rn(db.r_sorted[pos], kIonH), kIonH2O);
                const float stop = __fadd_rn(fmaxf(1.0f, __fsub_rn(z[s], 1.0f)), 0.5f);
                int32_t nch = 0;
                for (float c = 1.0f; c <= stop && nch < kMaxIonCharges; c = __fadd_rn(c, 1.0f)) ++nch;
                const int64_t n = (int64_t)nch * L;
                auto hit = [&](float v) -> int32_t {
                    const float q = rintf(__fdiv_rn(__fdiv_rn(v, bw), 3.0f));
                    if (!(q >= 0.0f && q < (float)np)) return 0;
                    const int32_t b = (int32_t)q;
                    return (int32_t)((s_mask[b >> 5] >> (b & 31)) & 1u);
                };
                int64_t k = 0;
                float c = 1.0f;
                for (int32_t ci = 0; ci < nch; ++ci, c = __fadd_rn(c, 1.0f)) {
                    const float hc = __fmul_rn(kIonH, c);
                    float lad = 0.0f;
                    for (int32_t a = 0; a < L; ++a, ++k) {
                        lad = __fadd_rn(lad, db.mt[db.ions[tc + a] & 31u]);
                        const float ion = __fdiv_rn(__fadd_rn(lad, hc), c);
                        if (k != n - 1) matched += hit(ion);              // init: b
                        if (k != 0) matched += hit(__fsub_rn(mh, ion));   // tail: y
                    }
                }
                total = (L + 4 + nstar - 5) * 2;
            }
        }
        out_m[o] = matched;
        out_t[o] = total;
    }
}

}  // namespace hfx

using namespace hfx;

size_t hfx_match_ions_smem(int64_t stride) { return (size_t)((stride / 3 + 1 + 31) / 32) * 4u; }

int hfx_match_ions_launch(const DevDB &db, const DevMods &mods, uint64_t nion, const SpecMeta *meta,
                          const float *rows, int64_t stride, const float *z, float bw, const uint64_t *keys,
                          int32_t nspec, int32_t topn, int32_t *out_m, int32_t *out_t, uint32_t *err,
                          cudaStream_t st) {
    if (nspec <= 0 || topn <= 0) return 0;
    const size_t smem = hfx_match_ions_smem(stride);
    int dev = 0, smem_max = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, k_match_ions);
    if (smem + fa.sharedSizeBytes > (size_t)smem_max) return (int)cudaErrorInvalidValue;
    if (smem > 48u * 1024u) {
        const cudaError_t e = cudaFuncSetAttribute(k_match_ions, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem);
        if (e != cudaSuccess) return (int)e;
    }
    k_match_ions<<<nspec, kIonThreads, smem, st>>>(db, mods, nion, meta, rows, stride, z, bw, keys, topn, out_m,
                                                   out_t, err);
    return (int)cudaGetLastError();
}
