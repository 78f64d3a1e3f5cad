// E-values of the matches (Util/Statistics.hs:37-100, called per spectrum at
// Search.hs:119-123), computed on the device from every candidate's FP32
// score -- the unmodified candidates and, in a modification search, every
// modified isoform -- instead of copying all scores to the host.
//
// Per spectrum, over its n candidate scores sorted ascending:
//   cut_end = round((1 - p/100) * n)   in single precision (p = evalueCutOffPerc, a Float)
//   cut_beg = round(0.3 * n)           in double precision
//   the scores of ranks [cut_beg, cut_end), shifted to x + 1 - min, keeping x > 4000;
//   histogram bins ceiling(x / w) (w = evalueBinWidth), points
//   (bin * w - w/2) / 10000 against log10(count / w);
//   an ordinary least-squares line log10 h = alpha + beta * x;
// and a match of score s gets E = 10 ** (alpha + beta * s / 10000).
// round is Haskell's (halves to even).  The regression restates
// statistics-linreg's linearRegression as plain OLS with sequential sums:
// that package is not in the reference tree, so its summation order is not
// reproduced (results agree to rounding).
#include <cmath>
#include <cstdint>
#include "hfx_internal.h"
#include "evalues.h"

namespace hfx {

__device__ __forceinline__ uint64_t plain_count(const uint32_t *wb, const uint32_t *we, int plain, int32_t s) {
    return plain && we[s] > wb[s] ? (uint64_t)(we[s] - wb[s]) : 0ull;
}

__global__ void k_window_sizes64(const uint32_t *__restrict__ wb, const uint32_t *__restrict__ we, int plain,
                                 const unsigned long long *__restrict__ isoforms, int32_t ns,
                                 uint64_t *__restrict__ size) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < ns) size[s] = plain_count(wb, we, plain, s) + (isoforms ? (uint64_t)isoforms[s] : 0ull);
}

// Exclusive scan of ns 64-bit sizes by one CTA of 1024 threads, in chunks.
__global__ void __launch_bounds__(1024) k_scan_sizes(const uint64_t *__restrict__ size, int32_t ns,
                                                     uint64_t *__restrict__ off) {
    __shared__ uint64_t ws[32];
    __shared__ uint64_t carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int32_t b0 = 0; b0 < ns; b0 += blockDim.x) {
        const int32_t i = b0 + threadIdx.x;
        const uint64_t v = i < ns ? size[i] : 0ull;
        uint64_t x = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t t = __shfl_up_sync(0xFFFFFFFFu, x, d);
            if (lane >= d) x += t;
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0) {
            uint64_t w = lane < (int)(blockDim.x >> 5) ? ws[lane] : 0ull;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint64_t t = __shfl_up_sync(0xFFFFFFFFu, w, d);
                if (lane >= d) w += t;
            }
            ws[lane] = w;
        }
        __syncthreads();
        const uint64_t before = carry + (warp ? ws[warp - 1] : 0ull);
        if (i < ns) off[i] = before + x - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + x;
        __syncthreads();
    }
}

__global__ void k_segment_ends(const uint32_t *__restrict__ wb, const uint32_t *__restrict__ we, int plain,
                               const uint64_t *__restrict__ off, const uint64_t *__restrict__ size, int32_t ns,
                               uint64_t *__restrict__ end, unsigned long long *__restrict__ cursor) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    end[s] = off[s] + size[s];
    if (cursor) cursor[s] = off[s] + plain_count(wb, we, plain, s);
}

// ---- the fit from the unsorted scores: order statistics by radix select ----
//
// The slice [cut_beg, cut_end) of the sorted scores is a multiset: every
// score strictly between the values at ranks cut_beg and cut_end - 1, plus
// the copies of those two values that fall inside the rank range.  A radix
// select (four 8-bit digits, most significant first, over order-preserving
// keys of the floats) finds both boundary values and how many scores lie
// below / at them; the minimum (the shift) comes from a block reduction; the
// histogram of ceil(t / w) is then counted in shared memory and read in
// ascending bin order, so the least squares see the points of the sorted
// slice in bin order, without sorting the scores.

__device__ __forceinline__ uint32_t score_key(float x) {
    const uint32_t u = __float_as_uint(x);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_score(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

constexpr int kEvThreads = 256;
constexpr int kEvHistCap = 4096;  // histogram bins per pass over the scores

// One CTA per spectrum over its unsorted scores sc[off[s] .. off[s] + size[s]).
__global__ void __launch_bounds__(kEvThreads) k_evalue_select_fit(const float *__restrict__ scores,
                                                                  const uint64_t *__restrict__ off,
                                                                  const uint64_t *__restrict__ size, double width,
                                                                  float cutoff_perc, double *__restrict__ fit) {
    __shared__ uint32_t hist[2][256];
    __shared__ uint32_t bins[kEvHistCap];
    __shared__ uint32_t s_red[kEvThreads / 32];
    __shared__ uint32_t s_pick[2], s_below[2], s_at[2];
    const int32_t s = blockIdx.x;
    const uint64_t n = size[s];
    double *f = fit + (size_t)s * 3;
    if (n == 0) {
        if (threadIdx.x == 0) {
            f[0] = f[1] = NAN;
            f[2] = 0.0;
        }
        return;
    }
    const float *sc = scores + off[s];
    const float keep = __fsub_rn(1.0f, __fdiv_rn(cutoff_perc, 100.0f));
    const int64_t cut_end = (int64_t)rintf(__fmul_rn(keep, (float)n));
    const int64_t cut_beg = (int64_t)rint(__dmul_rn(0.3, (double)n));
    const int64_t hi_i = cut_end < 0 ? 0 : (cut_end > (int64_t)n ? (int64_t)n : cut_end);
    const int64_t lo_i = cut_beg < 0 ? 0 : (cut_beg > hi_i ? hi_i : cut_beg);
    const uint64_t hi = (uint64_t)hi_i, lo = (uint64_t)lo_i;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // the minimum score
    uint32_t kmin = 0xFFFFFFFFu;
    for (uint64_t i = threadIdx.x; i < n; i += kEvThreads) kmin = min(kmin, score_key(sc[i]));
    kmin = __reduce_min_sync(0xFFFFFFFFu, kmin);
    if (lane == 0) s_red[warp] = kmin;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t v = threadIdx.x < kEvThreads / 32 ? s_red[threadIdx.x] : 0xFFFFFFFFu;
        v = __reduce_min_sync(0xFFFFFFFFu, v);
        if (threadIdx.x == 0) s_red[0] = v;
    }
    __syncthreads();
    const double head = (double)key_score(s_red[0]);
    // keys at ranks lo and hi - 1 (target 0 and 1), digit by digit
    const bool any = hi > lo;
    uint64_t rank[2] = {lo, any ? hi - 1 : lo};
    uint32_t prefix[2] = {0u, 0u}, below[2] = {0u, 0u};
    for (int d = 3; d >= 0; --d) {
        const int shift = 8 * d;
        const uint32_t hmask = d == 3 ? 0u : (0xFFFFFFFFu << (shift + 8));
        for (int i = threadIdx.x; i < 512; i += kEvThreads) (&hist[0][0])[i] = 0u;
        __syncthreads();
        for (uint64_t i = threadIdx.x; i < n; i += kEvThreads) {
            const uint32_t k = score_key(sc[i]);
            const uint32_t dig = (k >> shift) & 0xFFu;
            if ((k & hmask) == prefix[0]) atomicAdd(&hist[0][dig], 1u);
            if ((k & hmask) == prefix[1]) atomicAdd(&hist[1][dig], 1u);
        }
        __syncthreads();
        if (threadIdx.x < 2) {
            const int t = threadIdx.x;
            uint64_t acc = 0;
            int dig = 0;
            for (; dig < 256; ++dig) {
                if (acc + hist[t][dig] > rank[t]) break;
                acc += hist[t][dig];
            }
            s_pick[t] = (uint32_t)dig;
            s_below[t] = (uint32_t)acc;
            s_at[t] = hist[t][dig < 256 ? dig : 255];
        }
        __syncthreads();
        for (int t = 0; t < 2; ++t) {
            prefix[t] |= s_pick[t] << shift;
            rank[t] -= s_below[t];
            below[t] += s_below[t];
        }
        __syncthreads();
    }
    // below[t] = scores under the key, s_at[t] = scores equal to it (an
    // empty slice keeps no score: k1 = k2 = 0 admits none)
    const uint32_t k1 = any ? prefix[0] : 0u, k2 = any ? prefix[1] : 0u;
    const uint64_t le1 = (uint64_t)below[0] + s_at[0], lt2 = below[1];
    const double v1 = (double)key_score(k1), v2 = (double)key_score(k2);
    // copies of v1 and v2 inside the rank range
    uint64_t c1 = 0, c2 = 0;
    if (any) {
        if (k1 == k2) {
            c1 = hi - lo;
        } else {
            c1 = (le1 < hi ? le1 : hi) - lo;
            c2 = hi - (lt2 > lo ? lt2 : lo);
        }
    }
    // histogram bins of t = (x + 1) - head, t > 4000, in chunks of kEvHistCap
    const double tmax = (v2 + 1.0) + (-head);
    const int64_t b_lo = (int64_t)floor(4000.0 / width);
    const int64_t b_hi = any && tmax > 4000.0 ? (int64_t)ceil(tmax / width) : b_lo;
    double m = 0.0, sx = 0.0, sy = 0.0, mx = 0.0, my = 0.0, sxy = 0.0, sxx = 0.0;
    const bool one_chunk = b_hi - b_lo < kEvHistCap;  // counted once, read twice
    for (int pass = 0; pass < 2; ++pass) {
        for (int64_t c0 = b_lo; c0 <= b_hi; c0 += kEvHistCap) {
            if (!(one_chunk && pass == 1)) {
                for (int i = threadIdx.x; i < kEvHistCap; i += kEvThreads) bins[i] = 0u;
                __syncthreads();
                auto add = [&](double x, uint32_t cnt) {
                    const double t = (x + 1.0) + (-head);
                    if (!(t > 4000.0)) return;
                    const int64_t b = (int64_t)ceil(t / width) - c0;
                    if (b >= 0 && b < kEvHistCap) atomicAdd(&bins[b], cnt);
                };
                for (uint64_t i = threadIdx.x; i < n; i += kEvThreads) {
                    const float x = sc[i];
                    const uint32_t k = score_key(x);
                    if (k > k1 && k < k2) add((double)x, 1u);
                }
                if (threadIdx.x == 0) {
                    if (c1) add(v1, (uint32_t)c1);
                    if (c2) add(v2, (uint32_t)c2);
                }
                __syncthreads();
            }
            if (threadIdx.x == 0) {
                // the points in ascending bin order: pass 0 the means, pass 1
                // the centred sums (the sorted path's order)
                for (int i = 0; i < kEvHistCap && c0 + i <= b_hi; ++i) {
                    if (!bins[i]) continue;
                    const double x = ((double)(c0 + i) * width - width / 2.0) / 10000.0;
                    const double y = log((double)bins[i] / width) / log(10.0);
                    if (pass == 0) {
                        m += 1.0;
                        sx += x;
                        sy += y;
                    } else {
                        sxy += (x - mx) * (y - my);
                        sxx += (x - mx) * (x - mx);
                    }
                }
            }
            __syncthreads();
        }
        if (pass == 0) {
            mx = sx / m;
            my = sy / m;
        }
    }
    if (threadIdx.x == 0) {
        const double beta = sxy / sxx;
        f[0] = my - beta * mx;
        f[1] = beta;
        f[2] = m;
    }
}

__global__ void k_evalue_apply(const float *__restrict__ out_s, const uint64_t *__restrict__ out_k,
                               const double *__restrict__ fit, int32_t ns, int32_t topn, double *__restrict__ ev) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)ns * topn) return;
    const int32_t s = (int32_t)(i / topn);
    const double *f = fit + (size_t)s * 3;
    ev[i] = out_k[i] == ~0ull ? NAN : pow(10.0, f[0] + f[1] * ((double)out_s[i] / 10000.0));
}

}  // namespace hfx

using namespace hfx;

int hfx_evalue_offsets(const uint32_t *wb, const uint32_t *we, int plain, const unsigned long long *isoforms,
                       int32_t ns, uint64_t *size, uint64_t *off, uint64_t *end, unsigned long long *cursor,
                       cudaStream_t st) {
    if (ns <= 0) return 0;
    k_window_sizes64<<<(ns + 255) / 256, 256, 0, st>>>(wb, we, plain, isoforms, ns, size);
    k_scan_sizes<<<1, 1024, 0, st>>>(size, ns, off);
    k_segment_ends<<<(ns + 255) / 256, 256, 0, st>>>(wb, we, plain, off, size, ns, end, cursor);
    return (int)cudaGetLastError();
}

int hfx_evalue_select_fit(const float *scores, const uint64_t *off, const uint64_t *size, int32_t ns,
                          int32_t bin_width, float cutoff_perc, double *fit, cudaStream_t st) {
    if (ns <= 0) return 0;
    k_evalue_select_fit<<<ns, kEvThreads, 0, st>>>(scores, off, size, (double)bin_width, cutoff_perc, fit);
    return (int)cudaGetLastError();
}

int hfx_evalue_apply(const float *out_s, const uint64_t *out_k, const double *fit, int32_t ns, int32_t topn,
                     double *ev, cudaStream_t st) {
    const int64_t n = (int64_t)ns * topn;
    if (n <= 0) return 0;
    k_evalue_apply<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out_s, out_k, fit, ns, topn, ev);
    return (int)cudaGetLastError();
}
