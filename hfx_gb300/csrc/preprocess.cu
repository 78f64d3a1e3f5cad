// Stage (a): XCorr spectrum preprocessing, one CTA per spectrum.
//
// Restates Spectrum/Correlation.hs:37-109 (observedIntensity,
// normaliseByRegion, crossCorrolation) and Spectrum/Data.hs:58-59 (ms2Mass)
// with every float operation an explicit IEEE-rounded intrinsic, so the FP32
// row is bit-identical to the reference's host computation:
//   bin   = round(mz / binWidth)        (ties to even, Haskell `round`)
//   value = max over the bin of sqrt(intensity)
//   norm  = 50 * (e / regionMax)  when regionMax > 1e-6 and i < sel*10
//   x[i]  = norm[i] - (sequential sum of norm over take 151 (drop (i-75)))/150
// The row lives in shared memory while it is built; the output is written
// once as FP32 and, optionally, as BF16 and FP16 copies (round to nearest).
#include "hfx_internal.h"

namespace hfx {

// Host masses, Mass.hs:19-25.
constexpr float kHostH2O = 18.010565f;
constexpr float kHostH = 1.007276f;

__device__ __forceinline__ float spec_cutoff(float last_mz, float pcr, float z) {
    // Correlation.hs:65-67: min (50 + pcr*z) (fromInteger (truncate (last/10) * 10))
    const float mzcut = __fadd_rn(50.0f, __fmul_rn(pcr, z));
    const double t = trunc((double)__fdiv_rn(last_mz, 10.0f));
    const float mzlim = (float)(t * 10.0);
    return (mzcut <= mzlim) ? mzcut : mzlim;
}

// Per-spectrum layout and search window (one thread per spectrum).
__global__ void k_layout(const float *__restrict__ mz, const int64_t *__restrict__ off,
                         const float *__restrict__ pcr, const float *__restrict__ z,
                         const float *__restrict__ tol, int32_t nspec, LayoutParams lp,
                         SpecMeta *__restrict__ meta, uint32_t *__restrict__ max_len, uint32_t *__restrict__ err) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nspec) return;
    SpecMeta m;
    const int64_t o0 = off[s], o1 = off[s + 1];
    const float zs = z[s], ps = pcr[s];
    m.npk = (int32_t)(o1 - o0);
    m.status = 0;
    m.len = 0;
    m.cutoff = 0.0f;
    if (m.npk <= 0) {
        m.status = 1;  // empty spectrum: G.last fails in the reference
    } else {
        m.cutoff = spec_cutoff(mz[o1 - 1], ps, zs);
        const float c = lp.custom_bw ? __fdiv_rn(m.cutoff, lp.bw) : m.cutoff;
        const double len = 75.0 + ceil((double)c);
        if (!(len >= 76.0) || len > (double)lp.max_len) {
            m.status = 2;
        } else if (lp.cap_len > 0 && len > (double)lp.cap_len) {
            if (err) atomicOr(err, kErrTooLong);
            m.status = 2;
        } else {
            m.len = (int32_t)len;
            if ((m.len - 75) / 10 <= 0) m.status = 3;  // sel = 0: div by zero
        }
    }
    // Spectrum/Data.hs:58-59 ms2Mass with host constants
    m.mass = __fsub_rn(__fsub_rn(__fmul_rn(ps, zs), __fmul_rn(__fsub_rn(zs, 1.0f), kHostH)),
                       __fadd_rn(kHostH, kHostH2O));
    // tolerance unit: Da (filter.cu:105), ppm, or per spectrum (negative = ppm)
    const float ts = tol[s];
    const bool in_ppm = lp.ppm == 1 || (lp.ppm == 2 && ts < 0.0f);
    const float eps = in_ppm ? __fmul_rn(m.mass, __fmul_rn(lp.ppm == 2 ? -ts : ts, 1e-6f)) : ts;
    m.eps = eps;
    m.lo = __fsub_rn(m.mass, eps);  // filter.cu:103-115 (m - eps), (m + eps)
    m.hi = __fadd_rn(m.mass, eps);
    // Search.hs:182 max_chs = round (max 1 (chrg - 1)); ion_series.cu:301-309
    const float zm = __fsub_rn(zs, 1.0f);
    const float mc = (1.0f <= zm) ? zm : 1.0f;
    const float rr = rintf(mc);
    int32_t ch = (rr >= 1.0f) ? (rr > 1000.0f ? 1000 : (int32_t)rr) : 0;
    m.charges_plain = (ch >= 1 && ch <= 4) ? ch : 0;
    m.charges_mod = (ch >= 1 && ch <= 10) ? min(ch, 4) : 0;  // mion_series.cu:303-306, 425-438
    meta[s] = m;
    if (m.status == 0) atomicMax(max_len, (uint32_t)m.len);
}

// One CTA per spectrum; the whole row sits in shared memory.
// Block-wide exclusive scan of one value per thread (blockDim.x <= 1024).
__device__ __forceinline__ int32_t block_excl_scan(int32_t v, int32_t *warp_tot, int32_t &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int32_t t = __shfl_up_sync(0xFFFFFFFFu, x, d);
        if (lane >= d) x += t;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int32_t w = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int32_t t = __shfl_up_sync(0xFFFFFFFFu, w, d);
            if (lane >= d) w += t;
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    total = warp_tot[nw - 1];
    const int32_t before = (warp ? warp_tot[warp - 1] : 0) + x - v;
    __syncthreads();
    return before;
}

__global__ void __launch_bounds__(256) k_preprocess(const float *__restrict__ mz, const float *__restrict__ it,
                                                    const int64_t *__restrict__ off,
                                                    const float *__restrict__ pcr, LayoutParams lp,
                                                    const SpecMeta *__restrict__ meta, int64_t stride,
                                                    float *__restrict__ out32, __nv_bfloat16 *__restrict__ outbf,
                                                    __half *__restrict__ outh, int fold_nonzero) {
    extern __shared__ float sh[];
    const int32_t s = blockIdx.x;
    const SpecMeta m = meta[s];
    float *e = sh;                      // [len]
    __shared__ float rmax[11];
    const int tid = threadIdx.x;
    const int32_t len = (m.status == 0) ? m.len : 0;
    float *o32 = out32 + (int64_t)s * stride;
    if (m.status != 0) {
        for (int64_t i = tid; i < stride; i += blockDim.x) {
            o32[i] = 0.0f;
            if (outbf) outbf[(int64_t)s * stride + i] = __float2bfloat16_rn(0.0f);
            if (outh) outh[(int64_t)s * stride + i] = __float2half_rn(0.0f);
        }
        return;
    }
    for (int32_t i = tid; i < len; i += blockDim.x) e[i] = 0.0f;
    if (tid < 11) rmax[tid] = 0.0f;
    __syncthreads();
    // observedIntensity, Correlation.hs:58-71
    const float ps = pcr[s];
    const float plo = __fsub_rn(ps, 15.0f), phi = __fadd_rn(ps, 15.0f);
    const int64_t o0 = off[s];
    for (int32_t i = tid; i < m.npk; i += blockDim.x) {
        const float x = mz[o0 + i];
        const bool keep = lp.remove_pcr ? (x <= m.cutoff && (x <= plo || phi <= x)) : (x <= m.cutoff);
        if (!keep) continue;
        const float q = rintf(__fdiv_rn(x, lp.bw));
        if (!(q >= 0.0f) || q >= (float)len) continue;  // the reference raises here
        const float v = __fsqrt_rn(it[o0 + i]);
        if (v >= 0.0f) atomicMax((int *)&e[(int32_t)q], __float_as_int(v));
    }
    __syncthreads();
    // normaliseByRegion, Correlation.hs:84-96
    const int32_t sel = (len - 75) / 10;
    for (int32_t i = tid; i < len; i += blockDim.x) {
        const int32_t g = min(10, i / sel);
        const float v = e[i];
        if (v > 0.0f) atomicMax((int *)&rmax[g], __float_as_int(v));
    }
    __syncthreads();
    for (int32_t i = tid; i < len; i += blockDim.x) {
        const int32_t g = min(10, i / sel);
        const float mx = rmax[g];
        e[i] = (mx > 1e-6f && i < sel * 10) ? __fmul_rn(50.0f, __fdiv_rn(e[i], mx)) : 0.0f;
    }
    __syncthreads();
    // crossCorrolation, Correlation.hs:105-109.  Every e is >= 0, so the
    // left fold over a window equals the left fold over its nonzero bins
    // (adding +0 is exact and the sum never is -0); with fold_nonzero the
    // nonzero bins are listed once in bin order (nz_val) with, per bin, how
    // many precede it (nz_before), and each window folds only those.
    float *nz_val = e + stride;
    int32_t *nz_before = reinterpret_cast<int32_t *>(e + 2 * stride);
    if (fold_nonzero) {
        __shared__ int32_t warp_tot[32];
        const int32_t per = (len + (int32_t)blockDim.x - 1) / (int32_t)blockDim.x;
        const int32_t j0 = min(len, tid * per), j1 = min(len, j0 + per);
        int32_t c = 0;
        for (int32_t j = j0; j < j1; ++j) c += e[j] > 0.0f ? 1 : 0;
        int32_t total = 0;
        int32_t pos = block_excl_scan(c, warp_tot, total);
        for (int32_t j = j0; j < j1; ++j) {
            nz_before[j] = pos;
            if (e[j] > 0.0f) nz_val[pos++] = e[j];
        }
        if (tid == 0) nz_before[len] = total;
        __syncthreads();
    }
    __nv_bfloat16 *obf = outbf ? outbf + (int64_t)s * stride : nullptr;
    __half *oh = outh ? outh + (int64_t)s * stride : nullptr;
    for (int64_t i = tid; i < stride; i += blockDim.x) {
        float x = 0.0f;
        if (i < len) {
            const int32_t lo = max(0, (int32_t)i - 75);
            const int32_t hi = min(len, lo + 151);
            float acc = 0.0f;
            if (fold_nonzero) {
                for (int32_t t = nz_before[lo]; t < nz_before[hi]; ++t) acc = __fadd_rn(acc, nz_val[t]);
            } else {
                for (int32_t j = lo; j < hi; ++j) acc = __fadd_rn(acc, e[j]);
            }
            x = __fsub_rn(e[i], __fdiv_rn(acc, 150.0f));
        }
        o32[i] = x;
        if (obf) obf[i] = __float2bfloat16_rn(x);
        if (oh) oh[i] = __float2half_rn(x);
    }
}

// ---- long rows (e.g. 0.02 Da bins, ~10^5 bins): the same row, computed sparsely ----
//
// A row that does not fit in shared memory is built from its nonzero bins
// only.  The binned values are the kept peaks' sqrt intensities, max per bin
// (sort the (bin, value) keys, keep the last of each bin); normalisation
// touches only those bins; and x[i] is nonzero only where the 151-bin window
// of i holds a nonzero bin or e[i] != 0.  Every e is >= 0, so the reference's
// left fold over the window equals the left fold over the window's nonzero
// bins (adding +0 is exact and the sum never is -0): the row is bit-identical
// to the dense computation.
constexpr int kSparsePeaks = 4096;
constexpr size_t kDenseRowBytes = 200 * 1024;  // rows up to 51,200 bins are built densely in shared memory


__global__ void __launch_bounds__(256) k_preprocess_sparse(const float *__restrict__ mz, const float *__restrict__ it,
                                                           const int64_t *__restrict__ off,
                                                           const float *__restrict__ pcr, LayoutParams lp,
                                                           const SpecMeta *__restrict__ meta, int64_t stride,
                                                           float *__restrict__ out32,
                                                           __nv_bfloat16 *__restrict__ outbf,
                                                           __half *__restrict__ outh, uint32_t *__restrict__ err) {
    extern __shared__ __align__(16) uint8_t sm_sparse[];
    unsigned long long *keys = reinterpret_cast<unsigned long long *>(sm_sparse);  // [kSparsePeaks]
    int32_t *nzk = reinterpret_cast<int32_t *>(keys + kSparsePeaks);               // [kSparsePeaks]
    float *nze = reinterpret_cast<float *>(nzk + kSparsePeaks);                    // [kSparsePeaks]
    int32_t *ivs = reinterpret_cast<int32_t *>(nze + kSparsePeaks);                // [kSparsePeaks + 1]
    __shared__ int32_t warp_tot[32];
    __shared__ float rmax[11];
    const int32_t s = blockIdx.x;
    const SpecMeta m = meta[s];
    const int tid = threadIdx.x, nt = blockDim.x;
    float *o32 = out32 + (int64_t)s * stride;
    __nv_bfloat16 *obf = outbf ? outbf + (int64_t)s * stride : nullptr;
    __half *oh = outh ? outh + (int64_t)s * stride : nullptr;
    // zero rows (stride is a multiple of 16 elements, rows 16-byte aligned)
    for (int64_t i = (int64_t)tid * 4; i < stride; i += (int64_t)nt * 4)
        *reinterpret_cast<float4 *>(o32 + i) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int64_t i = (int64_t)tid * 8; i < stride; i += (int64_t)nt * 8) {
        if (obf) *reinterpret_cast<uint4 *>(obf + i) = make_uint4(0u, 0u, 0u, 0u);
        if (oh) *reinterpret_cast<uint4 *>(oh + i) = make_uint4(0u, 0u, 0u, 0u);
    }
    if (m.status != 0) return;
    if (m.npk > kSparsePeaks) {
        if (tid == 0) atomicOr(err, kErrTooLong);
        return;
    }
    const int32_t len = m.len;
    // observedIntensity, Correlation.hs:58-71: (bin, sqrt intensity) keys
    const float ps = pcr[s];
    const float plo = __fsub_rn(ps, 15.0f), phi = __fadd_rn(ps, 15.0f);
    const int64_t o0 = off[s];
    int32_t n2 = 1;
    while (n2 < m.npk) n2 <<= 1;
    for (int32_t i = tid; i < n2; i += nt) {
        unsigned long long k = ~0ull;
        if (i < m.npk) {
            const float x = mz[o0 + i];
            const bool keep = lp.remove_pcr ? (x <= m.cutoff && (x <= plo || phi <= x)) : (x <= m.cutoff);
            if (keep) {
                const float q = rintf(__fdiv_rn(x, lp.bw));
                const float v = __fsqrt_rn(it[o0 + i]);
                if (q >= 0.0f && q < (float)len && v >= 0.0f)
                    k = ((unsigned long long)(uint32_t)(int32_t)q << 32) | __float_as_uint(v);
            }
        }
        keys[i] = k;
    }
    if (tid < 11) rmax[tid] = 0.0f;
    __syncthreads();
    // bitonic sort, ascending (bin, then value: non-negative floats order as their bits)
    for (int32_t kk = 2; kk <= n2; kk <<= 1) {
        for (int32_t j = kk >> 1; j > 0; j >>= 1) {
            for (int32_t i = tid; i < n2; i += nt) {
                const int32_t l = i ^ j;
                if (l > i) {
                    const unsigned long long a = keys[i], b = keys[l];
                    const bool up = (i & kk) == 0;
                    if ((a > b) == up) {
                        keys[i] = b;
                        keys[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    // the last key of each bin carries the bin's max; compact them in order
    int32_t nnz = 0;
    for (int32_t base = 0; base < n2; base += nt) {
        const int32_t i = base + tid;
        const unsigned long long k = i < n2 ? keys[i] : ~0ull;
        const bool last = k != ~0ull && (i + 1 >= n2 || (keys[i + 1] >> 32) != (k >> 32));
        int32_t tot = 0;
        const int32_t at = nnz + block_excl_scan(last ? 1 : 0, warp_tot, tot);
        if (last) {
            nzk[at] = (int32_t)(k >> 32);
            nze[at] = __uint_as_float((uint32_t)k);
        }
        nnz += tot;
    }
    __syncthreads();
    // normaliseByRegion, Correlation.hs:84-96
    const int32_t sel = (len - 75) / 10;
    for (int32_t j = tid; j < nnz; j += nt) {
        const float v = nze[j];
        if (v > 0.0f) atomicMax((int *)&rmax[min(10, nzk[j] / sel)], __float_as_int(v));
    }
    __syncthreads();
    for (int32_t j = tid; j < nnz; j += nt) {
        const int32_t k = nzk[j];
        const float mx = rmax[min(10, k / sel)];
        nze[j] = (mx > 1e-6f && k < sel * 10) ? __fmul_rn(50.0f, __fdiv_rn(nze[j], mx)) : 0.0f;
    }
    // positions whose window holds a nonzero bin: [0, 75), and per nonzero
    // bin k the positions i >= 75 with |i - k| <= 75, minus the previous
    // bin's (bins ascending, so the pieces are disjoint)
    const int32_t head = min(75, len);
    int32_t tot = 0;
    for (int32_t base = 0; base < nnz; base += nt) {
        const int32_t j = base + tid;
        int32_t c = 0;
        if (j < nnz) {
            const int32_t k = nzk[j];
            int32_t a = max(head, k - 75);
            if (j > 0) a = max(a, nzk[j - 1] + 76);
            const int32_t b = min(len, k + 76);
            c = max(0, b - a);
        }
        int32_t t = 0;
        const int32_t at = tot + block_excl_scan(c, warp_tot, t);
        if (j < nnz) ivs[j] = at;
        tot += t;
    }
    if (tid == 0) ivs[nnz] = tot;
    __syncthreads();
    // crossCorrolation, Correlation.hs:105-109, at those positions only
    for (int32_t u = tid; u < head + tot; u += nt) {
        int32_t i;
        if (u < head) {
            i = u;
        } else {
            const int32_t v = u - head;
            int32_t lo = 0, hi = nnz;  // last j with ivs[j] <= v
            while (hi - lo > 1) {
                const int32_t mid = (lo + hi) >> 1;
                if (ivs[mid] <= v) lo = mid; else hi = mid;
            }
            const int32_t k = nzk[lo];
            int32_t a = max(head, k - 75);
            if (lo > 0) a = max(a, nzk[lo - 1] + 76);
            i = a + (v - ivs[lo]);
        }
        const int32_t wlo = max(0, i - 75);
        const int32_t whi = min(len, wlo + 151);
        int32_t a = 0, b = nnz;  // first nonzero bin >= wlo
        while (a < b) {
            const int32_t mid = (a + b) >> 1;
            if (nzk[mid] < wlo) a = mid + 1; else b = mid;
        }
        float acc = 0.0f, ei = 0.0f;
        for (int32_t j = a; j < nnz && nzk[j] < whi; ++j) {
            acc = __fadd_rn(acc, nze[j]);
            if (nzk[j] == i) ei = nze[j];
        }
        const float x = __fsub_rn(ei, __fdiv_rn(acc, 150.0f));
        o32[i] = x;
        if (obf) obf[i] = __float2bfloat16_rn(x);
        if (oh) oh[i] = __float2half_rn(x);
    }
}

}  // namespace hfx

using namespace hfx;

int hfx_launch_layout(const float *mz, const int64_t *off, const float *pcr, const float *z,
                      const float *tol, int32_t nspec, const LayoutParams &lp, SpecMeta *meta,
                      uint32_t *max_len, uint32_t *err, cudaStream_t st) {
    if (nspec <= 0) return 0;
    k_layout<<<(nspec + 127) / 128, 128, 0, st>>>(mz, off, pcr, z, tol, nspec, lp, meta, max_len, err);
    return (int)cudaGetLastError();
}

int hfx_launch_preprocess(const float *mz, const float *it, const int64_t *off, const float *pcr,
                          const LayoutParams &lp, const SpecMeta *meta, int32_t nspec, int64_t stride,
                          float *out32, __nv_bfloat16 *outbf, __half *outh, uint32_t *err, cudaStream_t st) {
    if (nspec <= 0) return 0;
    size_t smem = (size_t)stride * sizeof(float);
    if (smem > kDenseRowBytes) {
        // long rows: the sparse form (needs the error word for its peak limit)
        if (!err) return (int)cudaErrorInvalidValue;
        const size_t sm = (size_t)kSparsePeaks * (8 + 4 + 4 + 4) + 16;
        cudaFuncSetAttribute(k_preprocess_sparse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_preprocess_sparse<<<nspec, 256, sm, st>>>(mz, it, off, pcr, lp, meta, stride, out32, outbf, outh, err);
        return (int)cudaGetLastError();
    }
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_preprocess, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDenseRowBytes);
        attr_set = true;
    }
    // the row, its nonzero values and their running count (stride + 1 ints)
    // when they fit; otherwise every window folds all its bins
    const size_t smem3 = (size_t)stride * 8 + ((size_t)stride + 1) * 4;
    const int fold_nonzero = smem3 <= kDenseRowBytes ? 1 : 0;
    if (fold_nonzero) smem = smem3;
    k_preprocess<<<nspec, 256, smem, st>>>(mz, it, off, pcr, lp, meta, stride, out32, outbf, outh, fold_nonzero);
    return (int)cudaGetLastError();
}
