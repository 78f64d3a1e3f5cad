// Per-stage C ABI of the reference (include/hfx_legacy.h: the symbols of
// src/common/include/algorithms.h, bound by src/haskell/Foreign/CUDA/
// Algorithms.hs:44-371), served by kernels of this library so that a host
// built for the reference links unchanged.  Semantics follow each
// function's reference file (cited per function); the integer outputs are
// the reference's, the ion arithmetic is the reference's source
// (__fdividef m/z and bins), and the dense rows carry 10 / 25 / 50.
//
// Work runs on the legacy default stream (addModIons on its stream), and a
// function that returns a count synchronises, as the reference's Thrust
// calls do.  Scratch memory is allocated per call, as Thrust did.
#include <cub/cub.cuh>
#include <algorithm>
#include <cstdint>
#include <vector>
#include "hfx_legacy.h"
#include "device_common.cuh"
#include "mods_device.cuh"

namespace hfx {
namespace legacy {

constexpr int kThreads = 256;
constexpr int kLegacyMaxMa = 10;  // gen_mod_pep.cu:287-300, mion_series.cu:488-499

inline unsigned grid_for(uint64_t n, int threads = kThreads) {
    const uint64_t b = (n + (uint64_t)threads - 1) / (uint64_t)threads;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(b, 65535ull * 16));
}

// Device scratch that frees itself.
struct Scratch {
    void *p = nullptr;
    explicit Scratch(size_t bytes) {
        if (bytes && cudaMalloc(&p, bytes) != cudaSuccess) p = nullptr;
    }
    ~Scratch() {
        if (p) cudaFree(p);
    }
    template <typename T> T *as() const { return static_cast<T *>(p); }
    bool ok() const { return p != nullptr; }
};

uint32_t read_u32(const uint32_t *d) {
    uint32_t h = 0;
    cudaMemcpy(&h, d, 4, cudaMemcpyDeviceToHost);
    return h;
}

// out[0..n) = exclusive prefix sums of in (uint32, wrapping).
bool exclusive_scan(const uint32_t *in, uint32_t *out, uint32_t n) {
    if (n == 0) return true;
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, (int64_t)n);
    Scratch tmp(bytes);
    if (!tmp.ok()) return false;
    return cub::DeviceScan::ExclusiveSum(tmp.p, bytes, in, out, (int64_t)n) == cudaSuccess;
}

// ---- prepare_ions (prepare_ions.cu:29-132) ----
__global__ void k_pack(uint8_t *ions, uint32_t n, const uint8_t *ma, uint32_t num_ma) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint8_t c = ions[i];
        uint32_t mod = 0;
        for (uint32_t j = 0; j < num_ma; ++j)
            if (ma[j] == c) {
                mod = j + 1;
                break;
            }
        ions[i] = (uint8_t)((uint8_t)(c - 'A') | (uint8_t)(mod << 5));
    }
}

// ---- findIndicesInRange_f (filter.cu:40-66) ----
__global__ void k_flag_range(const float *in, uint32_t n, float lo, float hi, uint32_t *flag) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        flag[i] = (lo <= in[i] && in[i] <= hi) ? 1u : 0u;
}
__global__ void k_scatter_index(const uint32_t *flag, const uint32_t *pos, uint32_t n, uint32_t *out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        if (flag[i]) out[pos[i]] = i;
}

// ---- windows (filter.cu:75-127, filter_by_mod.cu:35-86) ----
// First k in [0, n) with !(r[idx[k]] < key), resp. key < r[idx[k]].
__device__ __forceinline__ uint32_t lower_bound_perm(const float *r, const uint32_t *idx, uint32_t n, float key) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if (r[idx[mid]] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ uint32_t upper_bound_perm(const float *r, const uint32_t *idx, uint32_t n, float key) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if (!(key < r[idx[mid]])) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}
__global__ void k_spec_windows(const float *r, const uint32_t *idx, uint32_t num_pep, const float *masses,
                               uint32_t num_spec, float eps, uint32_t *begin, uint32_t *end, uint32_t *num,
                               uint32_t *total) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < num_spec; s += gridDim.x * blockDim.x) {
        const float m = masses[s];
        const uint32_t b = lower_bound_perm(r, idx, num_pep, __fsub_rn(m, eps));
        const uint32_t e = upper_bound_perm(r, idx, num_pep, __fadd_rn(m, eps));
        begin[s] = b;
        end[s] = e;
        num[s] = e - b;
        atomicAdd(total, e - b);
    }
}
// lo0 = mass - eps and hi0 = mass + eps (computed on the host in FP32, as
// the reference's host expression is); the keys are lo0 - delta, hi0 - delta.
__global__ void k_mod_windows(const float *r, const uint32_t *idx, uint32_t num_pep, const float *delta,
                              uint32_t num_mod, float lo0, float hi0, uint32_t *begin, uint32_t *end) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < num_mod; i += gridDim.x * blockDim.x) {
        begin[i] = lower_bound_perm(r, idx, num_pep, __fsub_rn(lo0, delta[i]));
        end[i] = upper_bound_perm(r, idx, num_pep, __fsub_rn(hi0, delta[i]));
    }
}
__global__ void k_window_sizes(const uint32_t *begin, const uint32_t *end, uint32_t n, uint32_t *size) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        size[i] = end[i] - begin[i];
}

// ---- findModablePeptides (filter_by_mod.cu:145-378) ----
__global__ void k_fill_rows(uint32_t *pep, uint32_t *mod, const uint32_t *idx, const uint32_t *begin,
                            const uint32_t *end, const uint32_t *num_pep_scan, const uint32_t *spec_num_cand_scan,
                            uint32_t num_spec, uint32_t num_mod, uint32_t num_rows) {
    const uint64_t n = (uint64_t)num_spec * num_mod;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t m = (uint32_t)(t % num_mod), s = (uint32_t)(t / num_mod);
        uint32_t out = num_pep_scan[t] + spec_num_cand_scan[s];
        for (uint32_t i = begin[t]; i != end[t] && out < num_rows; ++i, ++out) {
            pep[out] = idx[i];
            mod[out] = m;
        }
    }
}
// utils.h:92: the letter of a packed residue is (byte & 0x1F) + 'A'.
__global__ void k_ma_counts(const uint32_t *pep, uint32_t num_rows, const uint8_t *ions, const uint32_t *tc,
                            const uint32_t *tn, const uint8_t *ma, uint32_t num_ma, uint32_t *count) {
    const uint64_t n = (uint64_t)num_rows * num_ma;
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t row = (uint32_t)(t / num_ma), a = (uint32_t)(t % num_ma);
        const uint32_t p = pep[row];
        const uint8_t acid = ma[a];
        uint32_t c = 0;
        for (uint32_t j = tc[p]; j < tn[p]; ++j) c += (uint8_t)((ions[j] & 0x1Fu) + 'A') == acid ? 1u : 0u;
        count[t] = c;
    }
}
__global__ void k_modable(const uint32_t *count, const uint32_t *mod, const uint32_t *mod_ma_count,
                          uint32_t num_rows, uint32_t num_ma, uint32_t *flag) {
    for (uint32_t row = blockIdx.x * blockDim.x + threadIdx.x; row < num_rows; row += gridDim.x * blockDim.x) {
        uint32_t ok = 1u;
        for (uint32_t a = 0; a < num_ma; ++a)
            if (count[(size_t)row * num_ma + a] < mod_ma_count[(size_t)mod[row] * num_ma + a]) ok = 0u;
        flag[row] = ok;
    }
}
__global__ void k_compact_rows(const uint32_t *flag, const uint32_t *pos, uint32_t num_rows, uint32_t num_ma,
                               const uint32_t *pep, const uint32_t *mod, const uint32_t *count, uint32_t *out_pep,
                               uint32_t *out_mod, uint32_t *out_count) {
    for (uint32_t row = blockIdx.x * blockDim.x + threadIdx.x; row < num_rows; row += gridDim.x * blockDim.x) {
        if (!flag[row]) continue;
        const uint32_t o = pos[row];
        out_pep[o] = pep[row];
        out_mod[o] = mod[row];
        for (uint32_t a = 0; a < num_ma; ++a) out_count[(size_t)o * num_ma + a] = count[(size_t)row * num_ma + a];
    }
}
// The kept rows before spectrum s's first row (the reference's lower_bound
// of the compacted source indices).
__global__ void k_valid_scan(const uint32_t *spec_num_cand_scan, uint32_t num_spec, const uint32_t *pos,
                             uint32_t num_rows, uint32_t kept, uint32_t *out) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < num_spec; s += gridDim.x * blockDim.x) {
        const uint32_t c = spec_num_cand_scan[s];
        out[s] = c < num_rows ? pos[c] : kept;
    }
}

// ---- calcTotalModCands (calc_mod_cands.cu:27-119) ----
__global__ void k_num_isoforms(uint32_t *out_num, uint32_t *out_scan, const uint32_t *mod_ma_count,
                               const uint32_t *pep_mod_idx, const uint32_t *pep_ma_count, uint32_t n_rows,
                               uint32_t num_ma, uint32_t *total) {
    for (uint32_t row = blockIdx.x * blockDim.x + threadIdx.x; row < n_rows; row += gridDim.x * blockDim.x) {
        const uint32_t m = pep_mod_idx[row];
        uint32_t num = 1u;
        for (int32_t i = (int32_t)num_ma - 1; i >= 0; --i) {
            num *= choose_dev(pep_ma_count[(size_t)num_ma * row + i], mod_ma_count[(size_t)num_ma * m + i]);
            out_scan[(size_t)row * num_ma + i] = num;
        }
        out_num[row] = num;
        atomicAdd(total, num);
    }
}

// ---- prepareGenMod (prepare_gen_mod.cu:23-129) ----
__global__ void k_expand_isoforms(uint32_t *o_pep, uint32_t *o_mod, uint32_t *o_rank, uint32_t *o_ith,
                                  uint32_t *o_size, const uint32_t *mod_ma_count_sum, const uint32_t *pep_idx,
                                  const uint32_t *pep_mod_idx, const uint32_t *pep_num_mpep, const uint32_t *start,
                                  uint32_t num_cand, uint32_t num_mpep) {
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < num_cand; c += gridDim.x * blockDim.x) {
        const uint32_t p = pep_idx[c], m = pep_mod_idx[c], size = mod_ma_count_sum[m];
        for (uint32_t i = 0, o = start[c]; i < pep_num_mpep[c] && o < num_mpep; ++i, ++o) {
            o_pep[o] = p;
            o_mod[o] = m;
            o_rank[o] = i;
            o_ith[o] = c;
            o_size[o] = size;
        }
    }
}

// ---- genModCands (gen_mod_pep.cu:127-312, combinatorics.h:90-134) ----
// The k occurrence indices of combination `rank` of n, written in the
// reference's order (largest first, mirrored under the dual rank).
__device__ void unrank_into(uint32_t *ans, uint32_t n, uint32_t k, uint32_t rank) {
    uint32_t a = n, b = k;
    const uint32_t total = choose_dev(n, k);
    uint32_t x;
    bool dual = false;
    if ((total / 2u) >= rank) x = rank;
    else { x = total - 1u - rank; dual = true; }
    for (uint32_t i = 0; i < k; ++i) {
        uint32_t v = a - 1u;
        // bounded: v never needs to pass below b
        for (uint32_t guard = 0; guard <= a && choose_dev(v, b) > x; ++guard) --v;
        ans[i] = v;
        x = x - choose_dev(v, b);
        a = v;
        b = b - 1u;
    }
    if (dual)
        for (uint32_t i = 0; i < k; ++i) ans[i] = (n - 1u) - ans[i];
}
__global__ void k_unrank(uint32_t *out, const uint32_t *mod_ma_count, const uint32_t *ith_valid,
                         const uint32_t *mpep_rank, const uint32_t *sum_scan, const uint32_t *pep_mod_idx,
                         const uint32_t *pep_ma_count, const uint32_t *comb_scan, uint32_t total, uint32_t num_ma) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const uint32_t ith = ith_valid[t];
        const uint32_t m = pep_mod_idx[ith];
        const uint32_t *cs = comb_scan + (size_t)ith * num_ma;
        uint32_t ranks[kLegacyMaxMa];
        uint32_t x = mpep_rank[t];
        for (uint32_t i = 0; i < num_ma; ++i) {
            if (i != num_ma - 1) {
                const uint32_t nxt = cs[i + 1];
                if (nxt != 0u && x >= nxt) {
                    ranks[i] = x / nxt;
                    x = x % nxt;
                } else {
                    ranks[i] = 0u;
                }
            } else {
                ranks[i] = x;
            }
        }
        uint32_t pos = sum_scan[t];
        for (uint32_t i = 0; i < num_ma; ++i) {
            const uint32_t k = mod_ma_count[(size_t)m * num_ma + i];
            if (k != 0u) {
                unrank_into(out + pos, pep_ma_count[(size_t)ith * num_ma + i], k, ranks[i]);
                pos += k;
            }
        }
    }
}

// ---- addIons / addModIons (ion_series.cu:59-232, mion_series.cu:143-328) ----
__device__ __forceinline__ void add_ion(uint32_t *spec, uint32_t n, int32_t x, uint32_t w) {
    if (0 <= x && (uint32_t)x < n) atomicMax(spec + x, w);
}
// ionMZ (ion_series.cu:59-63) and binMZ (:65-69) of the reference source.
__device__ __forceinline__ float ion_mz(float m, float c) { return __fdividef(__fadd_rn(m, __fmul_rn(kH, c)), c); }
__device__ __forceinline__ void dense_ions(uint32_t *spec, uint32_t n, float b, float y, int charge) {
    const float c = (float)charge;
    // A and B ions (addIonsAB)
    add_ion(spec, n, bin_of<true>(ion_mz(__fsub_rn(b, kCO), c)), 10u);
    float m = ion_mz(b, c);
    int32_t x = bin_of<true>(m);
    add_ion(spec, n, x, 50u);
    add_ion(spec, n, x + 1, 25u);
    add_ion(spec, n, x - 1, 25u);
    add_ion(spec, n, bin_of<true>(__fsub_rn(m, __fdividef(kH2O, c))), 10u);
    add_ion(spec, n, bin_of<true>(__fsub_rn(m, __fdividef(kNH3, c))), 10u);
    // Y ions (addIonsY)
    m = ion_mz(__fadd_rn(y, kH2O), c);
    x = bin_of<true>(m);
    add_ion(spec, n, x, 50u);
    add_ion(spec, n, x + 1, 25u);
    add_ion(spec, n, x - 1, 25u);
    add_ion(spec, n, bin_of<true>(__fsub_rn(m, __fdividef(kNH3, c))), 10u);
}
// Residue mass of a packed byte: the table entry of its letter; letters past
// the 26-entry table read 0 (the reference's texture fetch).
__device__ __forceinline__ float legacy_mass(const float *mass, uint8_t byte) {
    const uint32_t i = byte & 0x1Fu;
    return i < 26u ? __ldg(mass + i) : 0.0f;
}
// Warp-inclusive scan of one 32-residue chunk with the previous chunk's
// total added by lane 0 (the reference's scan_warp order).
template <typename V> __device__ __forceinline__ V chunk_scan(V v, V carry) {
    const int lane = threadIdx.x & 31;
    if (lane == 0) v = v + carry;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const V t = __shfl_up_sync(kFullMask, v, d);
        if (lane >= d) v = v + t;
    }
    return v;
}

__global__ void k_dense_ions(uint32_t *spec, const float *residual, const float *mass, const uint8_t *ions,
                             const uint32_t *tc, const uint32_t *tn, const uint32_t *idx, uint32_t num_idx,
                             uint32_t charges, uint32_t len_spec) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < num_idx; row += warps) {
        const uint32_t p = idx[row];
        const uint32_t t0 = tc[p], t1 = tn[p];
        const float res = residual[p];
        uint32_t *out = spec + (size_t)row * len_spec;
        float carry = 0.0f;
        for (uint32_t base = t0; base < t1; base += 32) {
            const int cnt = (int)min(32u, t1 - base);
            const float m = lane < cnt ? legacy_mass(mass, ions[base + lane]) : 0.0f;
            const float b = chunk_scan(m, carry);
            carry = __shfl_sync(kFullMask, b, cnt - 1);
            if (lane < cnt) {
                const float y = __fsub_rn(res, b);
                for (uint32_t c = 1; c <= charges; ++c) dense_ions(out, len_spec, b, y, (int)c);
            }
        }
    }
}

// isToBeModded (mion_series.cu:143-160): occurrence ith of acid ma_idx is
// among the acid's unranked indices.
__device__ __forceinline__ bool to_be_modded(const uint32_t *unrank, const uint32_t *mod_ma_count, uint32_t ma_idx,
                                             uint32_t ith) {
    uint32_t off = 0;
    for (uint32_t i = 0; i < ma_idx; ++i) off += mod_ma_count[i];
    bool res = false;
    for (uint32_t i = 0; i < mod_ma_count[ma_idx]; ++i)
        if (unrank[off + i] == ith) res = true;
    return res;
}
__global__ void k_dense_mod_ions(uint32_t *spec, const float *residual, const float *mass, const uint8_t *ions,
                                 const uint32_t *tc, const uint32_t *tn, const uint32_t *mpep_pep,
                                 const uint32_t *mpep_mod, const uint32_t *unrank, const uint32_t *sum_scan,
                                 uint32_t num_mpep, const uint32_t *mod_ma_count_all, const float *mod_delta,
                                 const float *ma_mass, uint32_t num_ma, uint32_t len_spec, uint32_t charges) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < num_mpep; row += warps) {
        const uint32_t p = mpep_pep[row], m = mpep_mod[row];
        const uint32_t *ur = unrank + sum_scan[row];
        const uint32_t *mc = mod_ma_count_all + (size_t)m * num_ma;
        const uint32_t t0 = tc[p], t1 = tn[p];
        const float res = __fadd_rn(residual[p], mod_delta[m]);
        uint32_t *out = spec + (size_t)row * len_spec;
        float carry = 0.0f;
        uint32_t carry_n = 0u;
        for (uint32_t base = t0; base < t1; base += 32) {
            const int cnt = (int)min(32u, t1 - base);
            const uint8_t byte = lane < cnt ? ions[base + lane] : (uint8_t)0;
            const uint32_t tag = ((uint32_t)byte & 0xE0u) >> 5;
            // the i-th counter counts every modable residue, whatever its acid
            // (mion_series.cu:252-269)
            const uint32_t n_incl = chunk_scan<uint32_t>(lane < cnt && tag != 0u ? 1u : 0u, carry_n);
            carry_n = __shfl_sync(kFullMask, n_incl, cnt - 1);
            float mres = lane < cnt ? legacy_mass(mass, byte) : 0.0f;
            if (lane < cnt && tag != 0u && tag - 1u < num_ma && to_be_modded(ur, mc, tag - 1u, n_incl - 1u))
                mres = __fadd_rn(mres, ma_mass[tag - 1u]);
            const float b = chunk_scan(mres, carry);
            carry = __shfl_sync(kFullMask, b, cnt - 1);
            if (lane < cnt) {
                const float y = __fsub_rn(res, b);
                for (uint32_t c = 1; c <= charges; ++c) dense_ions(out, len_spec, b, y, (int)c);
            }
        }
    }
}
// The dense rows hold uint32 intensities until this pass makes them floats.
__global__ void k_int_to_float(float *spec, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        spec[i] = __int2float_rn(__float_as_int(spec[i]));
}

// ---- prepare_scoring (prepare_scoring.cu:22-67) ----
__global__ void k_gather_cands(uint32_t *out, const uint32_t *idx, const uint32_t *begin, const uint32_t *num,
                               const uint32_t *start, uint32_t num_spec) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < num_spec; s += gridDim.x * blockDim.x)
        for (uint32_t i = 0; i < num[s]; ++i) out[start[s] + i] = idx[begin[s] + i];
}

// ---- sorts (sort.cu, sort_b40c.cu) ----
__global__ void k_iota(uint32_t *v, uint32_t n, uint32_t init) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = init + i;
}
void sort_pairs(float *keys, uint32_t *vals, uint32_t n, bool descending) {
    if (n < 2) return;
    Scratch alt_k((size_t)n * 4), alt_v((size_t)n * 4);
    if (!alt_k.ok() || !alt_v.ok()) return;
    cub::DoubleBuffer<float> dk(keys, alt_k.as<float>());
    cub::DoubleBuffer<uint32_t> dv(vals, alt_v.as<uint32_t>());
    size_t bytes = 0;
    if (descending) cub::DeviceRadixSort::SortPairsDescending(nullptr, bytes, dk, dv, (int64_t)n);
    else cub::DeviceRadixSort::SortPairs(nullptr, bytes, dk, dv, (int64_t)n);
    Scratch tmp(bytes);
    if (!tmp.ok()) return;
    if (descending) cub::DeviceRadixSort::SortPairsDescending(tmp.p, bytes, dk, dv, (int64_t)n);
    else cub::DeviceRadixSort::SortPairs(tmp.p, bytes, dk, dv, (int64_t)n);
    if (dk.Current() != keys) cudaMemcpy(keys, dk.Current(), (size_t)n * 4, cudaMemcpyDeviceToDevice);
    if (dv.Current() != vals) cudaMemcpy(vals, dv.Current(), (size_t)n * 4, cudaMemcpyDeviceToDevice);
}

// ---- mvm_ff (mvm.cu:22-56) ----
__global__ void k_gemv_t(float *y, const float *A, const float *x, uint32_t m, uint32_t n) {
    const int lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < m; i += warps) {
        const float *row = A + (size_t)i * n;
        float acc = 0.0f;
        for (uint32_t j = lane; j < n; j += 32) acc = __fmaf_rn(row[j], x[j], acc);
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(kFullMask, acc, o));
        if (lane == 0) y[i] = acc;
    }
}

}  // namespace legacy
}  // namespace hfx

using namespace hfx;
using namespace hfx::legacy;

extern "C" {

void prepare_ions(uint8_t *d_ions, uint32_t N, uint8_t *d_ma, uint32_t num_ma) {
    // prepare_ions.cu:98-103: fewer than threads x 4 residues launch no block
    if (N < 512u) return;
    k_pack<<<grid_for(N), kThreads>>>(d_ions, N, d_ma, num_ma);
}

uint32_t findIndicesInRange_f(const float *d_in, uint32_t *d_out, const uint32_t length, const float min,
                              const float max) {
    if (length == 0) return 0;
    Scratch flag((size_t)length * 4), pos((size_t)length * 4);
    if (!flag.ok() || !pos.ok()) return 0;
    k_flag_range<<<grid_for(length), kThreads>>>(d_in, length, min, max, flag.as<uint32_t>());
    if (!exclusive_scan(flag.as<uint32_t>(), pos.as<uint32_t>(), length)) return 0;
    k_scatter_index<<<grid_for(length), kThreads>>>(flag.as<uint32_t>(), pos.as<uint32_t>(), length, d_out);
    return read_u32(pos.as<uint32_t>() + length - 1) + read_u32(flag.as<uint32_t>() + length - 1);
}

uint32_t findSpecCandsByMass(uint32_t *d_spec_begin_raw, uint32_t *d_spec_end_raw, uint32_t *d_spec_num_pep_raw,
                             const float *d_r_raw, const uint32_t *d_pep_idx_r_sorted_raw, const uint32_t num_pep,
                             const float *d_spec_masses_raw, const uint32_t num_spec, const float eps) {
    if (num_spec == 0) return 0;
    Scratch total(4);
    if (!total.ok()) return 0;
    cudaMemset(total.p, 0, 4);
    k_spec_windows<<<grid_for(num_spec), kThreads>>>(d_r_raw, d_pep_idx_r_sorted_raw, num_pep, d_spec_masses_raw,
                                                      num_spec, eps, d_spec_begin_raw, d_spec_end_raw,
                                                      d_spec_num_pep_raw, total.as<uint32_t>());
    return read_u32(total.as<uint32_t>());
}

uint32_t findBeginEnd_f(uint32_t *d_begin_raw, uint32_t *d_end_raw, uint32_t *d_num_pep_scan_raw,
                        const float *d_r_raw, const uint32_t *d_pep_idx_r_sorted_raw, const uint32_t num_pep,
                        const float *d_mod_delta_raw, const uint32_t num_mod, const float mass_, const float eps) {
    if (num_mod == 0) return 0;
    const float lo0 = mass_ - eps, hi0 = mass_ + eps;
    k_mod_windows<<<grid_for(num_mod), kThreads>>>(d_r_raw, d_pep_idx_r_sorted_raw, num_pep, d_mod_delta_raw,
                                                    num_mod, lo0, hi0, d_begin_raw, d_end_raw);
    Scratch size((size_t)num_mod * 4);
    if (!size.ok()) return 0;
    k_window_sizes<<<grid_for(num_mod), kThreads>>>(d_begin_raw, d_end_raw, num_mod, size.as<uint32_t>());
    if (!exclusive_scan(size.as<uint32_t>(), d_num_pep_scan_raw, num_mod)) return 0;
    return read_u32(d_num_pep_scan_raw + num_mod - 1) + read_u32(size.as<uint32_t>() + num_mod - 1);
}

uint32_t findModablePeptides(uint32_t *d_out_pep_idx_raw, uint32_t *d_out_pep_mod_idx_raw,
                             uint32_t *d_out_pep_ma_count_raw, uint32_t *d_out_spec_num_valid_scan,
                             const uint32_t *d_spec_num_cand_scan, const uint32_t num_spec, uint32_t num_cand_total,
                             const uint8_t *d_ions, const uint32_t *d_tc, const uint32_t *d_tn,
                             const uint32_t *d_pep_idx_r_sorted_raw, const uint32_t *d_begin_raw,
                             const uint32_t *d_end_raw, const uint32_t *d_num_pep_scan_raw,
                             const uint32_t *d_mod_ma_count, const uint32_t num_mod, const uint8_t *d_ma,
                             const uint32_t num_ma) {
    const uint32_t n = num_cand_total;
    if (n == 0 || num_mod == 0) {
        if (num_spec) cudaMemset(d_out_spec_num_valid_scan, 0, (size_t)num_spec * 4);
        return 0;
    }
    const size_t nc = (size_t)n * std::max<uint32_t>(num_ma, 1u);
    Scratch pep((size_t)n * 4), mod((size_t)n * 4), cnt(nc * 4), flag((size_t)n * 4), pos((size_t)n * 4);
    if (!pep.ok() || !mod.ok() || !cnt.ok() || !flag.ok() || !pos.ok()) return 0;
    // rows the windows do not reach (a total larger than their sum) read as
    // (fragment 0, modification 0)
    cudaMemset(pep.p, 0, (size_t)n * 4);
    cudaMemset(mod.p, 0, (size_t)n * 4);
    k_fill_rows<<<grid_for((uint64_t)num_spec * num_mod), kThreads>>>(
        pep.as<uint32_t>(), mod.as<uint32_t>(), d_pep_idx_r_sorted_raw, d_begin_raw, d_end_raw, d_num_pep_scan_raw,
        d_spec_num_cand_scan, num_spec, num_mod, n);
    if (num_ma)
        k_ma_counts<<<grid_for((uint64_t)n * num_ma), kThreads>>>(pep.as<uint32_t>(), n, d_ions, d_tc, d_tn, d_ma,
                                                                  num_ma, cnt.as<uint32_t>());
    k_modable<<<grid_for(n), kThreads>>>(cnt.as<uint32_t>(), mod.as<uint32_t>(), d_mod_ma_count, n, num_ma,
                                          flag.as<uint32_t>());
    if (!exclusive_scan(flag.as<uint32_t>(), pos.as<uint32_t>(), n)) return 0;
    const uint32_t kept = read_u32(pos.as<uint32_t>() + n - 1) + read_u32(flag.as<uint32_t>() + n - 1);
    k_compact_rows<<<grid_for(n), kThreads>>>(flag.as<uint32_t>(), pos.as<uint32_t>(), n, num_ma, pep.as<uint32_t>(),
                                               mod.as<uint32_t>(), cnt.as<uint32_t>(), d_out_pep_idx_raw,
                                               d_out_pep_mod_idx_raw, d_out_pep_ma_count_raw);
    if (num_spec)
        k_valid_scan<<<grid_for(num_spec), kThreads>>>(d_spec_num_cand_scan, num_spec, pos.as<uint32_t>(), n, kept,
                                                        d_out_spec_num_valid_scan);
    cudaDeviceSynchronize();
    return kept;
}

uint32_t calcTotalModCands(uint32_t *d_out_pep_num_mpep_raw, uint32_t *d_out_pep_ma_num_comb_scan_raw,
                           const uint32_t *d_mod_ma_count_raw, const uint32_t *d_pep_idx_raw,
                           const uint32_t *d_pep_mod_idx_raw, const uint32_t *d_pep_ma_count_raw,
                           const uint32_t nPep, const uint32_t num_mod, const uint32_t num_ma) {
    (void)d_pep_idx_raw;
    (void)num_mod;
    if (nPep == 0) return 0;
    Scratch total(4);
    if (!total.ok()) return 0;
    cudaMemset(total.p, 0, 4);
    k_num_isoforms<<<grid_for(nPep), kThreads>>>(d_out_pep_num_mpep_raw, d_out_pep_ma_num_comb_scan_raw,
                                                  d_mod_ma_count_raw, d_pep_mod_idx_raw, d_pep_ma_count_raw, nPep,
                                                  num_ma, total.as<uint32_t>());
    return read_u32(total.as<uint32_t>());
}

uint32_t prepareGenMod(uint32_t *d_out_mpep_pep_idx, uint32_t *d_out_mpep_pep_mod_idx, uint32_t *d_out_mpep_rank,
                       uint32_t *d_out_mpep_ith_valid, uint32_t *d_out_mpep_mod_ma_count_sum_scan,
                       const uint32_t *d_mod_ma_count_sum, const uint32_t *d_pep_idx, const uint32_t *d_pep_mod_idx,
                       const uint32_t *d_pep_num_mpep, const uint32_t num_pep, const uint32_t num_mpep) {
    if (num_pep == 0 || num_mpep == 0) return 0;
    Scratch start((size_t)num_pep * 4), size((size_t)num_mpep * 4);
    if (!start.ok() || !size.ok()) return 0;
    if (!exclusive_scan(d_pep_num_mpep, start.as<uint32_t>(), num_pep)) return 0;
    k_expand_isoforms<<<grid_for(num_pep), kThreads>>>(d_out_mpep_pep_idx, d_out_mpep_pep_mod_idx, d_out_mpep_rank,
                                                        d_out_mpep_ith_valid, size.as<uint32_t>(), d_mod_ma_count_sum,
                                                        d_pep_idx, d_pep_mod_idx, d_pep_num_mpep,
                                                        start.as<uint32_t>(), num_pep, num_mpep);
    if (!exclusive_scan(size.as<uint32_t>(), d_out_mpep_mod_ma_count_sum_scan, num_mpep)) return 0;
    return read_u32(d_out_mpep_mod_ma_count_sum_scan + num_mpep - 1) + read_u32(size.as<uint32_t>() + num_mpep - 1);
}

void genModCands(uint32_t *d_out_mpep_unrank, const uint32_t *d_mod_ma_count, const uint32_t *d_mpep_ith_valid,
                 const uint32_t *d_mpep_rank, const uint32_t *d_mpep_mod_ma_count_sum_scan,
                 const uint32_t *d_pep_mod_idx, const uint32_t *d_pep_ma_count,
                 const uint32_t *d_pep_ma_num_comb_scan, const uint32_t total, const uint32_t mod_num_ma) {
    if (total == 0 || mod_num_ma < 1 || mod_num_ma > (uint32_t)kLegacyMaxMa) return;
    k_unrank<<<grid_for(total), kThreads>>>(d_out_mpep_unrank, d_mod_ma_count, d_mpep_ith_valid, d_mpep_rank,
                                             d_mpep_mod_ma_count_sum_scan, d_pep_mod_idx, d_pep_ma_count,
                                             d_pep_ma_num_comb_scan, total, mod_num_ma);
}

void addModIons(float *d_out_mspec, const float *d_residual, const float *d_mass, const uint8_t *d_ions,
                const uint32_t *d_tc, const uint32_t *d_tn, const uint32_t *d_mpep_pep_idx,
                const uint32_t *d_mpep_pep_mod_idx, const uint32_t *d_mpep_unrank,
                const uint32_t *d_mpep_mod_ma_count_sum_scan, const uint32_t len_unrank, const uint32_t num_mpep,
                const uint32_t *d_mod_ma_count, const float *d_mod_delta, const uint8_t *d_ma,
                const float *d_ma_mass, const uint32_t num_ma, const uint32_t len_spec, const uint32_t max_charge,
                cudaStream_t stream) {
    (void)len_unrank;
    (void)d_ma;
    if (num_mpep == 0 || num_ma < 1 || num_ma > (uint32_t)kLegacyMaxMa || max_charge < 1 || max_charge > 10) return;
    // the ion loop of mion_series.cu:317-320 stops at charge 4
    const uint32_t charges = std::min<uint32_t>(max_charge, 4u);
    k_dense_mod_ions<<<grid_for((uint64_t)num_mpep * 32), kThreads, 0, stream>>>(
        reinterpret_cast<uint32_t *>(d_out_mspec), d_residual, d_mass, d_ions, d_tc, d_tn, d_mpep_pep_idx,
        d_mpep_pep_mod_idx, d_mpep_unrank, d_mpep_mod_ma_count_sum_scan, num_mpep, d_mod_ma_count, d_mod_delta,
        d_ma_mass, num_ma, len_spec, charges);
    const uint64_t n = (uint64_t)num_mpep * len_spec;
    k_int_to_float<<<grid_for(n), kThreads, 0, stream>>>(d_out_mspec, n);
}

void addIons(float *d_spec, const float *d_residual, const float *d_mass, const uint8_t *d_ions,
             const uint32_t *d_tc, const uint32_t *d_tn, const uint32_t *d_idx, const uint32_t num_idx,
             const uint32_t max_charge, const uint32_t len_spec) {
    if (num_idx == 0 || max_charge < 1 || max_charge > 4) return;
    k_dense_ions<<<grid_for((uint64_t)num_idx * 32), kThreads>>>(reinterpret_cast<uint32_t *>(d_spec), d_residual,
                                                                  d_mass, d_ions, d_tc, d_tn, d_idx, num_idx,
                                                                  max_charge, len_spec);
    const uint64_t n = (uint64_t)num_idx * len_spec;
    k_int_to_float<<<grid_for(n), kThreads>>>(d_spec, n);
}

void prepare_scoring(uint32_t *d_out_spec_pep_idx, const uint32_t *d_pep_idx_r_sorted_raw,
                     const uint32_t *d_spec_begin, const uint32_t *d_spec_num_pep, const uint32_t num_spec) {
    if (num_spec == 0) return;
    Scratch start((size_t)num_spec * 4);
    if (!start.ok() || !exclusive_scan(d_spec_num_pep, start.as<uint32_t>(), num_spec)) return;
    k_gather_cands<<<grid_for(num_spec), kThreads>>>(d_out_spec_pep_idx, d_pep_idx_r_sorted_raw, d_spec_begin,
                                                      d_spec_num_pep, start.as<uint32_t>(), num_spec);
    cudaDeviceSynchronize();  // the scratch scan is freed on return
}

void sort_val_f(float *d_keys, uint32_t *d_vals, uint32_t N) { sort_pairs(d_keys, d_vals, N, false); }
void sort_rf(float *d_keys, uint32_t *d_vals, uint32_t N) { sort_pairs(d_keys, d_vals, N, true); }
void sort_b40c_f(float *d_keys, uint32_t *d_vals, uint32_t N) { sort_pairs(d_keys, d_vals, N, false); }
void sort_idx_f(float *d_keys_raw, uint32_t *d_idx_raw, uint32_t N, uint32_t init) {
    if (N == 0) return;
    k_iota<<<grid_for(N), kThreads>>>(d_idx_raw, N, init);
    sort_pairs(d_keys_raw, d_idx_raw, N, false);
}
void sort_idx_rf(float *d_keys_raw, uint32_t *d_idx_raw, uint32_t N, uint32_t init) {
    if (N == 0) return;
    k_iota<<<grid_for(N), kThreads>>>(d_idx_raw, N, init);
    sort_pairs(d_keys_raw, d_idx_raw, N, true);
}

void mvm_ff(cublasHandle_t handle, float *d_y, const float *d_A, const float *d_x, const uint32_t m,
            const uint32_t n) {
    (void)handle;
    if (m == 0) return;
    k_gemv_t<<<grid_for((uint64_t)m * 32), kThreads>>>(d_y, d_A, d_x, m, n);
}

}  // extern "C"
