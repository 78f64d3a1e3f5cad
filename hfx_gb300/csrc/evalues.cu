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
#include <cub/cub.cuh>
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

__global__ void k_segment_ends(const uint32_t *__restrict__ wb, const uint32_t *__restrict__ we, int plain,
                               const uint64_t *__restrict__ off, const uint64_t *__restrict__ size, int32_t ns,
                               uint64_t *__restrict__ end, unsigned long long *__restrict__ cursor) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    end[s] = off[s] + size[s];
    if (cursor) cursor[s] = off[s] + plain_count(wb, we, plain, s);
}

// The histogram points of one spectrum's slice, in ascending bin order;
// visit(x, y) per point.
template <typename Visit>
__device__ void evalue_points(const float *__restrict__ sc, uint64_t lo, uint64_t hi, double head, double width,
                              Visit visit) {
    int64_t cur = INT64_MIN;
    double cnt = 0.0;
    auto flush = [&]() {
        if (cnt > 0.0) {
            const double x = ((double)cur * width - width / 2.0) / 10000.0;
            const double y = log(cnt / width) / log(10.0);
            visit(x, y);
        }
    };
    for (uint64_t i = lo; i < hi; ++i) {
        const double t = ((double)sc[i] + 1.0) + (-head);
        if (!(t > 4000.0)) continue;
        const int64_t b = (int64_t)ceil(t / width);
        if (b != cur) {
            flush();
            cur = b;
            cnt = 0.0;
        }
        cnt += 1.0;
    }
    flush();
}

__global__ void k_evalue_fit(const float *__restrict__ sorted, const uint64_t *__restrict__ off,
                             const uint64_t *__restrict__ size, int32_t ns, double width, float cutoff_perc,
                             double *__restrict__ fit) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    const uint64_t n = size[s];
    double *f = fit + (size_t)s * 3;
    if (n == 0) {
        f[0] = f[1] = NAN;
        f[2] = 0.0;
        return;
    }
    const float *sc = sorted + off[s];
    const double head = (double)sc[0];
    const float keep = __fsub_rn(1.0f, __fdiv_rn(cutoff_perc, 100.0f));
    const int64_t cut_end = (int64_t)rintf(__fmul_rn(keep, (float)n));
    const int64_t cut_beg = (int64_t)rint(__dmul_rn(0.3, (double)n));
    const int64_t hi_i = cut_end < 0 ? 0 : (cut_end > (int64_t)n ? (int64_t)n : cut_end);
    const int64_t lo_i = cut_beg < 0 ? 0 : (cut_beg > hi_i ? hi_i : cut_beg);
    const uint64_t hi = (uint64_t)hi_i, lo = (uint64_t)lo_i;
    double m = 0.0, sx = 0.0, sy = 0.0;
    evalue_points(sc, lo, hi, head, width, [&](double x, double y) {
        m += 1.0;
        sx += x;
        sy += y;
    });
    const double mx = sx / m, my = sy / m;
    double sxy = 0.0, sxx = 0.0;
    evalue_points(sc, lo, hi, head, width, [&](double x, double y) {
        sxy += (x - mx) * (y - my);
        sxx += (x - mx) * (x - mx);
    });
    const double beta = sxy / sxx;
    f[0] = my - beta * mx;
    f[1] = beta;
    f[2] = m;
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
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, size, off, ns, st);
    void *tmp = nullptr;
    if (cudaMallocAsync(&tmp, bytes, st) != cudaSuccess) return (int)cudaErrorMemoryAllocation;
    cub::DeviceScan::ExclusiveSum(tmp, bytes, size, off, ns, st);
    cudaFreeAsync(tmp, st);
    k_segment_ends<<<(ns + 255) / 256, 256, 0, st>>>(wb, we, plain, off, size, ns, end, cursor);
    return (int)cudaGetLastError();
}

int hfx_evalue_sort(const float *scores, float *sorted, uint64_t total, const uint64_t *off, const uint64_t *end,
                    int32_t ns, cudaStream_t st) {
    if (ns <= 0 || total == 0) return 0;
    size_t bytes = 0;
    cub::DeviceSegmentedSort::SortKeys(nullptr, bytes, scores, sorted, (int64_t)total, ns, off, end, st);
    void *tmp = nullptr;
    if (cudaMallocAsync(&tmp, bytes, st) != cudaSuccess) return (int)cudaErrorMemoryAllocation;
    cub::DeviceSegmentedSort::SortKeys(tmp, bytes, scores, sorted, (int64_t)total, ns, off, end, st);
    cudaFreeAsync(tmp, st);
    return (int)cudaGetLastError();
}

int hfx_evalue_fit(const float *sorted, const uint64_t *off, const uint64_t *size, int32_t ns, int32_t bin_width,
                   float cutoff_perc, double *fit, cudaStream_t st) {
    if (ns <= 0) return 0;
    k_evalue_fit<<<(ns + 127) / 128, 128, 0, st>>>(sorted, off, size, ns, (double)bin_width, cutoff_perc, fit);
    return (int)cudaGetLastError();
}

int hfx_evalue_apply(const float *out_s, const uint64_t *out_k, const double *fit, int32_t ns, int32_t topn,
                     double *ev, cudaStream_t st) {
    const int64_t n = (int64_t)ns * topn;
    if (n <= 0) return 0;
    k_evalue_apply<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out_s, out_k, fit, ns, topn, ev);
    return (int)cudaGetLastError();
}
