// Stages (b)-(e) for unmodified candidates: mass windows, the fused
// ion-ladder + gather-dot scorer, top-K selection and merging.
#include "hfx_internal.h"
#include "device_common.cuh"
#include "search_kernels.h"

namespace hfx {

// Stage (b), filter.cu:75-127: begin = lower_bound(r_sorted, m - eps),
// end = upper_bound(r_sorted, m + eps), both bounds inclusive.
__device__ __forceinline__ uint32_t lower_bound_f(const float *a, uint32_t n, float v) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ uint32_t upper_bound_f(const float *a, uint32_t n, float v) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (v < a[mid]) hi = mid; else lo = mid + 1;
    }
    return lo;
}

__global__ void k_windows(const float *__restrict__ r_sorted, uint32_t n, const SpecMeta *__restrict__ meta,
                          int32_t nspec, uint32_t *__restrict__ wb, uint32_t *__restrict__ we) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nspec) return;
    const SpecMeta m = meta[s];
    uint32_t b = 0, e = 0;
    if (m.status == 0) {
        b = lower_bound_f(r_sorted, n, m.lo);
        e = upper_bound_f(r_sorted, n, m.hi);
        if (e < b) e = b;
    }
    wb[s] = b;
    we[s] = e;
}

// Write every warp's list to shared memory and merge them in warp 0.
__device__ __forceinline__ void cta_merge(WarpTopK &tk, int K, float *sm_s, uint64_t *sm_k) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane < K) {
        sm_s[warp * K + lane] = tk.s;
        sm_k[warp * K + lane] = tk.k;
    }
    __syncthreads();
    if (warp == 0) {
        tk.init();
        for (int j = 0; j < nw * K; ++j) {
            const float s = sm_s[j];
            const uint64_t k = sm_k[j];
            if (k != ~0ull) tk.insert(s, k, K);
        }
    }
    __syncthreads();
}

// Plain path: one launch per spectrum, FP32 row staged in shared memory.
template <bool FastDiv>
__global__ void __launch_bounds__(256) k_score_spectrum(DevDB db, const float *__restrict__ row, int32_t len,
                                                        int32_t charges, uint32_t begin, uint32_t end,
                                                        int32_t words, int32_t K, float *__restrict__ part_s,
                                                        uint64_t *__restrict__ part_k, uint32_t *__restrict__ err) {
    extern __shared__ __align__(16) uint8_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float *srow = reinterpret_cast<float *>(smem);
    const int32_t len4 = (len + 3) & ~3;
    uint32_t *planes = reinterpret_cast<uint32_t *>(srow + len4);
    uint16_t *lists = reinterpret_cast<uint16_t *>(planes + (size_t)nw * 3 * words);
    for (int32_t i = threadIdx.x; i < len4; i += blockDim.x) srow[i] = (i < len) ? row[i] : 0.0f;
    for (int32_t i = threadIdx.x; i < nw * 3 * words; i += blockDim.x) planes[i] = 0u;
    __syncthreads();
    Planes pl{planes + (size_t)warp * 3 * words, planes + (size_t)warp * 3 * words + words,
              planes + (size_t)warp * 3 * words + 2 * words};
    uint16_t *list = lists + (size_t)warp * kListCap;
    const float mt_lane = db.mt[lane];
    WarpTopK tk;
    tk.init();
    SpecSet<float, 1> ss;
    ss.row[0] = srow;
    ss.len[0] = len;
    ss.active = 1u;
    for (uint32_t p = begin + blockIdx.x * nw + warp; p < end; p += gridDim.x * nw) {
        const uint32_t tc = db.tc_sorted[p], tn = db.tn_sorted[p];
        const float r = db.r_sorted[p];
        const WordRange wr = build_planes<FastDiv>(pl, db.ions, tc, tn, r, charges, len, mt_lane, NoMods{});
        float acc[1];
        planes_dot<float, 1>(pl, list, wr, ss, acc);
        tk.insert(acc[0], (uint64_t)p, K);
    }
    __syncthreads();
    float *sm_s = reinterpret_cast<float *>(planes);
    uint64_t *sm_k = reinterpret_cast<uint64_t *>(planes) + (size_t)nw * K;
    cta_merge(tk, K, sm_s, sm_k);
    if (warp == 0 && lane < K) {
        part_s[(size_t)blockIdx.x * K + lane] = tk.s;
        part_k[(size_t)blockIdx.x * K + lane] = tk.k;
    }
    (void)err;
}

// Merge per-spectrum partial lists into the final top-N.
__global__ void k_merge_parts(const float *__restrict__ part_s, const uint64_t *__restrict__ part_k,
                              const int64_t *__restrict__ part_off, int32_t nspec, int32_t K, int32_t topn,
                              const uint32_t *__restrict__ idx_sorted, float *__restrict__ out_s,
                              uint64_t *__restrict__ out_k, uint32_t *__restrict__ out_pep) {
    const int lane = threadIdx.x & 31;
    const int32_t s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= nspec) return;
    WarpTopK tk;
    tk.init();
    const int64_t p0 = part_off[s], p1 = part_off[s + 1];
    for (int64_t j0 = p0 * K; j0 < p1 * K; j0 += 32) {
        const int64_t j = j0 + lane;
        float sc = -INFINITY;
        uint64_t kk = ~0ull;
        if (j < p1 * K) { sc = part_s[j]; kk = part_k[j]; }
        const int m = (int)min((int64_t)32, p1 * K - j0);
        for (int t = 0; t < m; ++t) {
            const float ts = __shfl_sync(kFullMask, sc, t);
            const uint64_t tk2 = __shfl_sync(kFullMask, kk, t);
            if (tk2 != ~0ull) tk.insert(ts, tk2, topn);
        }
    }
    if (lane < topn) {
        out_s[(size_t)s * topn + lane] = tk.s;
        out_k[(size_t)s * topn + lane] = tk.k;
        uint32_t pep = ~0u;
        if (tk.k != ~0ull) {
            const uint64_t pos = (tk.k >> 63) ? ((tk.k >> 27) & ((1ull << 27) - 1)) : tk.k;
            pep = idx_sorted[pos];
        }
        out_pep[(size_t)s * topn + lane] = pep;
    }
}

// Ion-bin export for parity checks: the sorted distinct list of candidate
// positions pos[i] at `charges` and row length len[i].
template <bool FastDiv>
__global__ void k_ion_bins(DevDB db, const uint32_t *__restrict__ pos, const int32_t *__restrict__ charges,
                           const int32_t *__restrict__ lens, int32_t n, int32_t words, int32_t cap,
                           uint32_t *__restrict__ out_bins, uint8_t *__restrict__ out_lvl,
                           int32_t *__restrict__ out_n) {
    extern __shared__ __align__(16) uint8_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t *planes = reinterpret_cast<uint32_t *>(smem);
    uint16_t *lists = reinterpret_cast<uint16_t *>(planes + (size_t)nw * 3 * words);
    for (int32_t i = threadIdx.x; i < nw * 3 * words; i += blockDim.x) planes[i] = 0u;
    __syncthreads();
    Planes pl{planes + (size_t)warp * 3 * words, planes + (size_t)warp * 3 * words + words,
              planes + (size_t)warp * 3 * words + 2 * words};
    uint16_t *list = lists + (size_t)warp * kListCap;
    const float mt_lane = db.mt[lane];
    for (int32_t i = blockIdx.x * nw + warp; i < n; i += gridDim.x * nw) {
        const uint32_t p = pos[i];
        const int32_t len = min(lens[i], words * 32);
        build_planes<FastDiv>(pl, db.ions, db.tc_sorted[p], db.tn_sorted[p], db.r_sorted[p], charges[i], len,
                              mt_lane, NoMods{});
        // compact without a dot: same pass as planes_dot, writing the list out
        int cnt = 0;
        for (int w0 = 0; w0 < words; w0 += 32) {
            const int w = w0 + lane;
            uint32_t a = 0, h = 0, t = 0;
            if (w < words) {
                h = pl.H[w];
                t = pl.T[w];
                a = pl.A[w] | h;
                pl.A[w] = pl.H[w] = pl.T[w] = 0u;
            }
            const int pc = __popc(a);
            const int incl = warp_incl_scan(pc);
            int o = cnt + incl - pc;
            while (a) {
                const int b = __ffs(a) - 1;
                a &= a - 1u;
                if (o < cap) {
                    out_bins[(size_t)i * cap + o] = (uint32_t)(w * 32 + b);
                    out_lvl[(size_t)i * cap + o] = ((t >> b) & 1u) ? 3 : (((h >> b) & 1u) ? 2 : 1);
                }
                ++o;
            }
            cnt += __shfl_sync(kFullMask, incl, 31);
        }
        __syncwarp();
        if (lane == 0) out_n[i] = cnt;
        (void)list;
    }
}

}  // namespace hfx

using namespace hfx;

static size_t score_smem_bytes(int32_t len, int32_t words, int nw, int K) {
    size_t b = (size_t)((len + 3) & ~3) * 4 + (size_t)nw * 3 * words * 4 + (size_t)nw * kListCap * 2;
    size_t merge = (size_t)nw * K * 16;
    size_t planes = (size_t)nw * 3 * words * 4 + (size_t)nw * kListCap * 2;
    if (merge > planes) b += merge - planes;
    return b;
}

int hfx_launch_windows(const float *r_sorted, uint32_t n, const SpecMeta *meta, int32_t nspec, uint32_t *wb,
                       uint32_t *we, cudaStream_t st) {
    if (nspec <= 0) return 0;
    k_windows<<<(nspec + 127) / 128, 128, 0, st>>>(r_sorted, n, meta, nspec, wb, we);
    return (int)cudaGetLastError();
}

int hfx_launch_score_spectrum(const DevDB &db, const float *row, int32_t len, int32_t charges, uint32_t begin,
                              uint32_t end, int32_t K, int32_t nblocks, int fastdiv, float *part_s,
                              uint64_t *part_k, uint32_t *err, cudaStream_t st) {
    const int nw = 8;
    const int32_t words = (len + 31) / 32;
    if (words > kMaxWords) return (int)cudaErrorInvalidValue;
    const size_t smem = score_smem_bytes(len, words, nw, K);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_score_spectrum<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_score_spectrum<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    if (fastdiv)
        k_score_spectrum<true><<<nblocks, nw * 32, smem, st>>>(db, row, len, charges, begin, end, words, K, part_s,
                                                               part_k, err);
    else
        k_score_spectrum<false><<<nblocks, nw * 32, smem, st>>>(db, row, len, charges, begin, end, words, K, part_s,
                                                                part_k, err);
    return (int)cudaGetLastError();
}

int hfx_launch_merge_parts(const float *part_s, const uint64_t *part_k, const int64_t *part_off, int32_t nspec,
                           int32_t K, int32_t topn, const uint32_t *idx_sorted, float *out_s, uint64_t *out_k,
                           uint32_t *out_pep, cudaStream_t st) {
    if (nspec <= 0) return 0;
    k_merge_parts<<<(nspec + 3) / 4, 128, 0, st>>>(part_s, part_k, part_off, nspec, K, topn, idx_sorted, out_s,
                                                   out_k, out_pep);
    return (int)cudaGetLastError();
}

int hfx_launch_ion_bins(const DevDB &db, const uint32_t *pos, const int32_t *charges, const int32_t *lens,
                        int32_t n, int32_t maxlen, int32_t cap, int fastdiv, uint32_t *out_bins,
                        uint8_t *out_lvl, int32_t *out_n, cudaStream_t st) {
    if (n <= 0) return 0;
    const int nw = 4;
    const int32_t words = (maxlen + 31) / 32;
    if (words > kMaxWords) return (int)cudaErrorInvalidValue;
    const size_t smem = (size_t)nw * 3 * words * 4 + (size_t)nw * kListCap * 2;
    const int blocks = (n + nw - 1) / nw < 1024 ? (n + nw - 1) / nw : 1024;
    if (fastdiv)
        k_ion_bins<true><<<blocks, nw * 32, smem, st>>>(db, pos, charges, lens, n, words, cap, out_bins, out_lvl,
                                                        out_n);
    else
        k_ion_bins<false><<<blocks, nw * 32, smem, st>>>(db, pos, charges, lens, n, words, cap, out_bins, out_lvl,
                                                         out_n);
    return (int)cudaGetLastError();
}

