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
                         SpecMeta *__restrict__ meta, uint32_t *__restrict__ max_len) {
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
__global__ void __launch_bounds__(256) k_preprocess(const float *__restrict__ mz, const float *__restrict__ it,
                                                    const int64_t *__restrict__ off,
                                                    const float *__restrict__ pcr, LayoutParams lp,
                                                    const SpecMeta *__restrict__ meta, int64_t stride,
                                                    float *__restrict__ out32, __nv_bfloat16 *__restrict__ outbf,
                                                    __half *__restrict__ outh) {
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
    // crossCorrolation, Correlation.hs:105-109
    __nv_bfloat16 *obf = outbf ? outbf + (int64_t)s * stride : nullptr;
    __half *oh = outh ? outh + (int64_t)s * stride : nullptr;
    for (int64_t i = tid; i < stride; i += blockDim.x) {
        float x = 0.0f;
        if (i < len) {
            const int32_t lo = max(0, (int32_t)i - 75);
            const int32_t hi = min(len, lo + 151);
            float acc = 0.0f;
            for (int32_t j = lo; j < hi; ++j) acc = __fadd_rn(acc, e[j]);
            x = __fsub_rn(e[i], __fdiv_rn(acc, 150.0f));
        }
        o32[i] = x;
        if (obf) obf[i] = __float2bfloat16_rn(x);
        if (oh) oh[i] = __float2half_rn(x);
    }
}

}  // namespace hfx

using namespace hfx;

int hfx_launch_layout(const float *mz, const int64_t *off, const float *pcr, const float *z,
                      const float *tol, int32_t nspec, const LayoutParams &lp, SpecMeta *meta,
                      uint32_t *max_len, cudaStream_t st) {
    if (nspec <= 0) return 0;
    k_layout<<<(nspec + 127) / 128, 128, 0, st>>>(mz, off, pcr, z, tol, nspec, lp, meta, max_len);
    return (int)cudaGetLastError();
}

int hfx_launch_preprocess(const float *mz, const float *it, const int64_t *off, const float *pcr,
                          const LayoutParams &lp, const SpecMeta *meta, int32_t nspec, int64_t stride,
                          float *out32, __nv_bfloat16 *outbf, __half *outh, cudaStream_t st) {
    if (nspec <= 0) return 0;
    const size_t smem = (size_t)stride * sizeof(float);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_preprocess, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    if (smem > 200 * 1024) return (int)cudaErrorInvalidValue;
    k_preprocess<<<nspec, 256, smem, st>>>(mz, it, off, pcr, lp, meta, stride, out32, outbf, outh);
    return (int)cudaGetLastError();
}
