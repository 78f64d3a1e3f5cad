// Device building blocks shared by the search kernels (sm_103a).
//
// One warp scores one candidate peptide.  The warp
//   1. builds the b-ion mass ladder with the same FP32 Hillis-Steele order as
//      the reference warp scan (ion_series.cu:25-56, 176-213),
//   2. turns every (prefix, charge) into its ten ion bins
//      (ion_series.cu:78-123) and ORs them into three per-warp bit planes in
//      shared memory -- "any ion", "weight >= 25", "weight 50" -- which is the
//      reference's atomicMax-into-a-dense-row (ion_series.cu:71-75) without
//      the dense row,
//   3. compacts the planes into the ascending list of distinct bins and
//      gathers the spectrum at those bins (the sparse form of the reference's
//      cuBLAS sgemv over the dense row, Search.hs:245).
// Canonical FP32 order of the gather-dot: list entry i is accumulated by lane
// i % 32 with fmaf in ascending i; the 32 partial sums are combined by an XOR
// butterfly with offsets 16, 8, 4, 2, 1.  The oracle computes the same order.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include "hfx_internal.h"

namespace hfx {

// Device masses, ion_series.h:16-26 (they differ from the host masses).
constexpr float kH2O = 18.01056f;
constexpr float kNH3 = 17.02655f;
constexpr float kCO = 27.9949f;
constexpr float kH = 1.0078246f;
constexpr float kBinMono = 1.0005079f;

constexpr uint32_t kFullMask = 0xFFFFFFFFu;

// ion_series.cu:59-69: ionMZ and binMZ.  IEEE division unless FastDiv, which
// calls __fdividef exactly where the reference did.
template <bool FastDiv>
__device__ __forceinline__ float dev_div(float a, float b) {
    if constexpr (FastDiv) return __fdividef(a, b);
    else return __fdiv_rn(a, b);
}

// The IEEE quotient a / c for an ion charge c in 1..4: the powers of two are
// exact scalings, only c = 3 needs a division.
template <bool FastDiv>
__device__ __forceinline__ float div_charge(float a, int c) {
    if constexpr (FastDiv) return __fdividef(a, (float)c);
    if (c == 3) return __fdiv_rn(a, 3.0f);
    return __fmul_rn(a, c == 1 ? 1.0f : (c == 2 ? 0.5f : 0.25f));
}

// float -> uint32 conversion (saturating, NaN -> 0) reinterpreted as int32.
__device__ __forceinline__ int32_t sat_bin(float r) {
    return (int32_t)__float2uint_rz(r);
}

// rint(fl(mz / 1.0005079)).  A multiply by the rounded reciprocal lies within
// 2^-22 relative of the IEEE quotient, i.e. within 2^-8 for |q| < 2^14; when
// it is farther than 1/128 from a half-integer -- its distance to the nearest
// integer, |q - rint(q)| (exact), is below 1/2 - 1/128 -- both round to the
// same integer, otherwise the IEEE quotient itself is computed.  Exact.
constexpr float kInvBinMono = 1.0f / 1.0005079f;
template <bool FastDiv>
__device__ __forceinline__ int32_t bin_of(float mz) {
    if constexpr (FastDiv) return sat_bin(rintf(__fdividef(mz, kBinMono)));
    const float q = __fmul_rn(mz, kInvBinMono);
    const float r = rintf(q);
    if (fabsf(q) < 16384.0f && fabsf(__fsub_rn(q, r)) < 0.4921875f) return sat_bin(r);
    return sat_bin(rintf(__fdiv_rn(mz, kBinMono)));
}

struct ChargeConst {
    int c;
    float hc, dh2o, dnh3;
};

template <bool FastDiv>
__device__ __forceinline__ ChargeConst charge_const(int c) {
    ChargeConst k;
    k.c = c;
    k.hc = __fmul_rn(kH, (float)c);
    k.dh2o = div_charge<FastDiv>(kH2O, c);
    k.dnh3 = div_charge<FastDiv>(kNH3, c);
    return k;
}

// Bit planes of one warp: A = any ion, H = weight >= 25, T = weight 50.
// (Weight 25 and 50 bins are only ever set through H and T; "any" is A|H.)
struct Planes {
    uint32_t *A, *H, *T;
};

__device__ __forceinline__ void set_bit(uint32_t *p, int32_t x) {
    atomicOr(&p[x >> 5], 1u << (x & 31));
}

// Range of bins a lane has set, for the compaction pass.
struct BinRange {
    int32_t lo = 0x7FFFFFFF, hi = -1;
    __device__ __forceinline__ void add(int32_t a, int32_t b) {
        lo = min(lo, a);
        hi = max(hi, b);
    }
};

// x-1, x, x+1 at weight 25/50/25 (ion_series.cu:92-94, 109-111).
__device__ __forceinline__ void set_triplet(const Planes &pl, int32_t x, int32_t nbins, BinRange &br) {
    if (x >= 1 && x + 1 < nbins && (x & 31) != 0 && (x & 31) != 31) {
        atomicOr(&pl.H[x >> 5], 7u << ((x - 1) & 31));
        atomicOr(&pl.T[x >> 5], 1u << (x & 31));
        br.add(x - 1, x + 1);
        return;
    }
    if (0 <= x - 1 && x - 1 < nbins) { set_bit(pl.H, x - 1); br.add(x - 1, x - 1); }
    if (0 <= x + 1 && x + 1 < nbins) { set_bit(pl.H, x + 1); br.add(x + 1, x + 1); }
    if (0 <= x && x < nbins) { set_bit(pl.H, x); set_bit(pl.T, x); br.add(x, x); }
}

__device__ __forceinline__ void set_single(const Planes &pl, int32_t x, int32_t nbins, BinRange &br) {
    if (0 <= x && x < nbins) { set_bit(pl.A, x); br.add(x, x); }
}

// The ten ions of one (b, y, charge), ion_series.cu:78-123.
template <bool FastDiv>
__device__ __forceinline__ void emit_ions(const Planes &pl, float b, float y, const ChargeConst &k,
                                          int32_t nbins, BinRange &br) {
    // A ion
    set_single(pl, bin_of<FastDiv>(div_charge<FastDiv>(__fadd_rn(__fsub_rn(b, kCO), k.hc), k.c)), nbins, br);
    // B ions
    float m = div_charge<FastDiv>(__fadd_rn(b, k.hc), k.c);
    set_triplet(pl, bin_of<FastDiv>(m), nbins, br);
    set_single(pl, bin_of<FastDiv>(__fsub_rn(m, k.dh2o)), nbins, br);
    set_single(pl, bin_of<FastDiv>(__fsub_rn(m, k.dnh3)), nbins, br);
    // Y ions
    m = div_charge<FastDiv>(__fadd_rn(__fadd_rn(y, kH2O), k.hc), k.c);
    set_triplet(pl, bin_of<FastDiv>(m), nbins, br);
    set_single(pl, bin_of<FastDiv>(__fsub_rn(m, k.dnh3)), nbins, br);
}

// Mass of one packed residue byte (utils.h:92-101; an out-of-range texture
// fetch of an unpacked byte reads 0).  mt_lane: lane l holds mass[l].
__device__ __forceinline__ float residue_mass(float mt_lane, uint32_t byte) {
    uint32_t i = byte & 0x1Fu;
    float m = __shfl_sync(kFullMask, mt_lane, (int)i);
    return i < 26u ? m : 0.0f;
}

// Per-residue modification hook, called by every lane once per 32-residue
// chunk in peptide order: returns the mass to add to this lane's residue
// (0 = unmodified).  `valid` is false for lanes past the peptide's end.
struct NoMods {
    __device__ __forceinline__ float chunk_add(uint32_t /*byte*/, bool /*valid*/) { return 0.0f; }
};

// Words [lo, hi) of the bit planes that hold set bits.
struct WordRange {
    int32_t lo, hi;
};

template <bool FastDiv, typename Mods>
__device__ __forceinline__ WordRange build_planes_range(const Planes &pl, const uint8_t *__restrict__ ions,
                                                        uint32_t tc, uint32_t tn, float residual, int c_first,
                                                        int c_last, int32_t nbins, float mt_lane,
                                                        Mods mods);

// Build the ion bit planes of one candidate.  Residues [tc, tn) of `ions`,
// `charges` ion charges (0 = none), bins >= nbins dropped.  Returns the
// range of plane words that may hold set bits (warp-uniform).
template <bool FastDiv, typename Mods>
__device__ __forceinline__ WordRange build_planes(const Planes &pl, const uint8_t *__restrict__ ions,
                                                  uint32_t tc, uint32_t tn, float residual,
                                                  int charges, int32_t nbins, float mt_lane,
                                                  Mods mods) {
    return build_planes_range<FastDiv>(pl, ions, tc, tn, residual, 1, charges, nbins, mt_lane, mods);
}

// The same for ion charges c_first..c_last only (bits accumulate in the
// planes, so successive calls build the cumulative charge levels).
template <bool FastDiv, typename Mods>
__device__ __forceinline__ WordRange build_planes_range(const Planes &pl, const uint8_t *__restrict__ ions,
                                                        uint32_t tc, uint32_t tn, float residual, int c_first,
                                                        int c_last, int32_t nbins, float mt_lane,
                                                        Mods mods) {
    const int lane = threadIdx.x & 31;
    BinRange br;
    const int charges = c_last - c_first + 1;
    if (c_last <= 0 || charges <= 0) return WordRange{0, 0};
    float carry = 0.0f;
    for (uint32_t base = tc; base < tn; base += 32) {
        const int cnt = (int)min(32u, tn - base);
        uint32_t byte = 0;
        if (lane < cnt) byte = __ldg(ions + base + lane);
        float v = residue_mass(mt_lane, byte);
        {
            const float add = mods.chunk_add(byte, lane < cnt);
            if (add != 0.0f) v = __fadd_rn(v, add);
        }
        if (lane >= cnt) v = 0.0f;
        if (lane == 0) v = __fadd_rn(v, carry);
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            float t = __shfl_up_sync(kFullMask, v, d);
            if (lane >= d) v = __fadd_rn(v, t);
        }
        carry = __shfl_sync(kFullMask, v, cnt - 1);
        const float y = __fsub_rn(residual, v);
        // balanced (prefix, charge) items: item = (c-1)*cnt + k
        const int items = cnt * charges;
        const uint32_t inv = (65536u + (uint32_t)cnt - 1u) / (uint32_t)cnt;
        for (int it0 = 0; it0 < items; it0 += 32) {
            const int it = it0 + lane;
            const int cm1 = (int)(((uint32_t)it * inv) >> 16);
            const int k = it - cm1 * cnt;
            const float bk = __shfl_sync(kFullMask, v, k & 31);
            const float yk = __shfl_sync(kFullMask, y, k & 31);
            if (it < items) {
                const ChargeConst kc = charge_const<FastDiv>(c_first + cm1);
                emit_ions<FastDiv>(pl, bk, yk, kc, nbins, br);
            }
        }
    }
    __syncwarp();
    const int32_t lo = __reduce_min_sync(kFullMask, br.lo);
    const int32_t hi = __reduce_max_sync(kFullMask, br.hi);
    if (hi < 0) return WordRange{0, 0};
    return WordRange{lo >> 5, (hi >> 5) + 1};
}

// Warp-wide inclusive scan of an int.
__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int t = __shfl_up_sync(kFullMask, v, d);
        if (lane >= d) v += t;
    }
    return v;
}

template <typename T> __device__ __forceinline__ float load_x(const T *row, uint32_t i);
template <> __device__ __forceinline__ float load_x<float>(const float *row, uint32_t i) { return row[i]; }
template <> __device__ __forceinline__ float load_x<__nv_bfloat16>(const __nv_bfloat16 *row, uint32_t i) {
    return __bfloat162float(row[i]);
}
template <> __device__ __forceinline__ float load_x<__half>(const __half *row, uint32_t i) {
    return __half2float(row[i]);
}

// Weight of a list entry's level: 10, 25, 50 for levels 1, 2, 3 (0 for
// level 0).  The three values share their low 16 bits (zero) and differ in
// two bytes, which one byte permute picks by level: bytes 1..3 of `lo` and
// 5..7 of `hi` are the third and fourth bytes of 10.0f, 25.0f, 50.0f.
__device__ __forceinline__ uint32_t level_weight_hi16(uint32_t lvl) {
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(0x48C82000u), "r"(0x42414100u), "r"(lvl * 0x11u + 0x40u));
    return r & 0xFFFFu;  // the bf16 (upper half) bits of the weight
}
__device__ __forceinline__ float level_weight(uint32_t lvl) { return __uint_as_float(level_weight_hi16(lvl) << 16); }

// A set of spectra scored against the same candidate list.
template <typename T, int G>
struct SpecSet {
    const T *row[G];
    int32_t len[G];
    uint32_t active;     // bit g set: score this candidate against spectrum g
};

// Accumulate list entries [0, n) into acc[] (entry i by lane i%32): rows
// given separately, with a length and an active flag per spectrum.
template <typename T, int G>
struct RowDot {
    const SpecSet<T, G> &ss;
    __device__ __forceinline__ void operator()(const uint16_t *list, int n, float (&acc)[G]) const {
        const int lane = threadIdx.x & 31;
        for (int i = lane; i < n; i += 32) {
            const uint32_t e = list[i];
            const uint32_t bin = e >> 2;
            const float w = level_weight(e & 3u);
#pragma unroll
            for (int g = 0; g < G; ++g) {
                if (((ss.active >> g) & 1u) && (int32_t)bin < ss.len[g])
                    acc[g] = __fmaf_rn(w, load_x<T>(ss.row[g], bin), acc[g]);
            }
        }
    }
};

// The same over a tile of G zero-padded rows interleaved bin-major
// (tile[bin*G + g]): one vector load per entry feeds all G spectra.  Rows
// are zero beyond their length and fmaf(w, +0, acc) == acc (acc is never
// -0), so no per-spectrum length test is needed.
template <typename T, int G> struct TileLoad {
    __device__ __forceinline__ static void load(const T *t, uint32_t bin, float (&x)[G]) {
#pragma unroll
        for (int g = 0; g < G; ++g) x[g] = load_x<T>(t, bin * G + g);
    }
};
template <> struct TileLoad<__nv_bfloat16, 8> {
    __device__ __forceinline__ static void load(const __nv_bfloat16 *t, uint32_t bin, float (&x)[8]) {
        const uint4 v = *reinterpret_cast<const uint4 *>(t + (size_t)bin * 8);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            x[2 * i] = __uint_as_float(w[i] << 16);
            x[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
        }
    }
};
template <> struct TileLoad<__nv_bfloat16, 4> {
    __device__ __forceinline__ static void load(const __nv_bfloat16 *t, uint32_t bin, float (&x)[4]) {
        const uint2 v = *reinterpret_cast<const uint2 *>(t + (size_t)bin * 4);
        x[0] = __uint_as_float(v.x << 16);
        x[1] = __uint_as_float(v.x & 0xFFFF0000u);
        x[2] = __uint_as_float(v.y << 16);
        x[3] = __uint_as_float(v.y & 0xFFFF0000u);
    }
};
template <> struct TileLoad<__half, 8> {
    __device__ __forceinline__ static void load(const __half *t, uint32_t bin, float (&x)[8]) {
        const uint4 v = *reinterpret_cast<const uint4 *>(t + (size_t)bin * 8);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const __half2 h = *reinterpret_cast<const __half2 *>(&w[i]);
            const float2 f = __half22float2(h);
            x[2 * i] = f.x;
            x[2 * i + 1] = f.y;
        }
    }
};
template <> struct TileLoad<__half, 4> {
    __device__ __forceinline__ static void load(const __half *t, uint32_t bin, float (&x)[4]) {
        const uint2 v = *reinterpret_cast<const uint2 *>(t + (size_t)bin * 4);
        const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&v.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&v.y));
        x[0] = a.x; x[1] = a.y; x[2] = b.x; x[3] = b.y;
    }
};
template <> struct TileLoad<float, 4> {
    __device__ __forceinline__ static void load(const float *t, uint32_t bin, float (&x)[4]) {
        const float4 v = *reinterpret_cast<const float4 *>(t + (size_t)bin * 4);
        x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
    }
};
template <> struct TileLoad<float, 8> {
    __device__ __forceinline__ static void load(const float *t, uint32_t bin, float (&x)[8]) {
        const float4 a = *reinterpret_cast<const float4 *>(t + (size_t)bin * 8);
        const float4 b = *reinterpret_cast<const float4 *>(t + (size_t)bin * 8 + 4);
        x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
        x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
    }
};

// acc[g] += weight(level) * tile[bin][g] for the G spectra of a group tile.
// BF16/FP16 tiles use the mixed-precision FMA (fma.rn.f32.bf16 / .f16:
// 16-bit multiplicands, FP32 addend and result).  The 16-bit weight and tile
// value multiply exactly in FP32, so each step rounds once, exactly like
// fmaf(weight, float(x), acc): bit-identical to the FP32 path, without the
// conversions.
__device__ __forceinline__ uint16_t level_weight_bf16(uint32_t lvl) {
    return (uint16_t)level_weight_hi16(lvl);  // 0x4120, 0x41C8, 0x4248 = 10, 25, 50
}
__device__ __forceinline__ uint16_t level_weight_f16(uint32_t lvl) {
    // 0x4900, 0x4E40, 0x5240 = 10, 25, 50 in FP16, by the same byte permute
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(0x40400000u), "r"(0x524E4900u), "r"(lvl * 0x11u + 0x40u));
    return (uint16_t)(r & 0xFFFFu);
}

template <typename T, int G>
struct TileFma {
    __device__ __forceinline__ static void fma(const T *t, uint32_t bin, uint32_t lvl, float (&acc)[G]) {
        const float w = level_weight(lvl);
        float x[G];
        TileLoad<T, G>::load(t, bin, x);
#pragma unroll
        for (int g = 0; g < G; ++g) acc[g] = __fmaf_rn(w, x[g], acc[g]);
    }
};

#define HFX_MIXED_FMA8(TY)                                                                                      \
    asm("{\n\t.reg .b16 l0, h0, l1, h1, l2, h2, l3, h3;\n\t"                                                   \
        "mov.b32 {l0, h0}, %8;\n\tmov.b32 {l1, h1}, %9;\n\tmov.b32 {l2, h2}, %10;\n\tmov.b32 {l3, h3}, %11;\n\t" \
        "fma.rn.f32." TY " %0, %12, l0, %0;\n\tfma.rn.f32." TY " %1, %12, h0, %1;\n\t"                          \
        "fma.rn.f32." TY " %2, %12, l1, %2;\n\tfma.rn.f32." TY " %3, %12, h1, %3;\n\t"                          \
        "fma.rn.f32." TY " %4, %12, l2, %4;\n\tfma.rn.f32." TY " %5, %12, h2, %5;\n\t"                          \
        "fma.rn.f32." TY " %6, %12, l3, %6;\n\tfma.rn.f32." TY " %7, %12, h3, %7;\n\t}"                          \
        : "+f"(acc[0]), "+f"(acc[1]), "+f"(acc[2]), "+f"(acc[3]), "+f"(acc[4]), "+f"(acc[5]), "+f"(acc[6]),    \
          "+f"(acc[7])                                                                                          \
        : "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "h"(w))
#define HFX_MIXED_FMA4(TY)                                                                                      \
    asm("{\n\t.reg .b16 l0, h0, l1, h1;\n\t"                                                                   \
        "mov.b32 {l0, h0}, %4;\n\tmov.b32 {l1, h1}, %5;\n\t"                                                    \
        "fma.rn.f32." TY " %0, %6, l0, %0;\n\tfma.rn.f32." TY " %1, %6, h0, %1;\n\t"                            \
        "fma.rn.f32." TY " %2, %6, l1, %2;\n\tfma.rn.f32." TY " %3, %6, h1, %3;\n\t}"                            \
        : "+f"(acc[0]), "+f"(acc[1]), "+f"(acc[2]), "+f"(acc[3])                                                \
        : "r"(v.x), "r"(v.y), "h"(w))

template <> struct TileFma<__nv_bfloat16, 8> {
    __device__ __forceinline__ static void fma(const __nv_bfloat16 *t, uint32_t bin, uint32_t lvl, float (&acc)[8]) {
        const uint4 v = *reinterpret_cast<const uint4 *>(t + (size_t)bin * 8);
        const uint16_t w = level_weight_bf16(lvl);
        HFX_MIXED_FMA8("bf16");
    }
};
template <> struct TileFma<__half, 8> {
    __device__ __forceinline__ static void fma(const __half *t, uint32_t bin, uint32_t lvl, float (&acc)[8]) {
        const uint4 v = *reinterpret_cast<const uint4 *>(t + (size_t)bin * 8);
        const uint16_t w = level_weight_f16(lvl);
        HFX_MIXED_FMA8("f16");
    }
};
// 16 spectra: two 16-byte loads, the same per-element FMAs.
template <> struct TileFma<__nv_bfloat16, 16> {
    __device__ __forceinline__ static void fma(const __nv_bfloat16 *t, uint32_t bin, uint32_t lvl, float (&a)[16]) {
        const uint4 v0 = *reinterpret_cast<const uint4 *>(t + (size_t)bin * 16);
        const uint4 v1 = *reinterpret_cast<const uint4 *>(t + (size_t)bin * 16 + 8);
        const uint16_t w = level_weight_bf16(lvl);
        {
            float(&acc)[8] = *reinterpret_cast<float(*)[8]>(&a[0]);
            const uint4 v = v0;
            HFX_MIXED_FMA8("bf16");
        }
        {
            float(&acc)[8] = *reinterpret_cast<float(*)[8]>(&a[8]);
            const uint4 v = v1;
            HFX_MIXED_FMA8("bf16");
        }
    }
};
template <> struct TileFma<__half, 16> {
    __device__ __forceinline__ static void fma(const __half *t, uint32_t bin, uint32_t lvl, float (&a)[16]) {
        const uint4 v0 = *reinterpret_cast<const uint4 *>(t + (size_t)bin * 16);
        const uint4 v1 = *reinterpret_cast<const uint4 *>(t + (size_t)bin * 16 + 8);
        const uint16_t w = level_weight_f16(lvl);
        {
            float(&acc)[8] = *reinterpret_cast<float(*)[8]>(&a[0]);
            const uint4 v = v0;
            HFX_MIXED_FMA8("f16");
        }
        {
            float(&acc)[8] = *reinterpret_cast<float(*)[8]>(&a[8]);
            const uint4 v = v1;
            HFX_MIXED_FMA8("f16");
        }
    }
};
template <> struct TileFma<__nv_bfloat16, 4> {
    __device__ __forceinline__ static void fma(const __nv_bfloat16 *t, uint32_t bin, uint32_t lvl, float (&acc)[4]) {
        const uint2 v = *reinterpret_cast<const uint2 *>(t + (size_t)bin * 4);
        const uint16_t w = level_weight_bf16(lvl);
        HFX_MIXED_FMA4("bf16");
    }
};
template <> struct TileFma<__half, 4> {
    __device__ __forceinline__ static void fma(const __half *t, uint32_t bin, uint32_t lvl, float (&acc)[4]) {
        const uint2 v = *reinterpret_cast<const uint2 *>(t + (size_t)bin * 4);
        const uint16_t w = level_weight_f16(lvl);
        HFX_MIXED_FMA4("f16");
    }
};
#undef HFX_MIXED_FMA8
#undef HFX_MIXED_FMA4

template <typename T, int G>
struct TileDot {
    const T *tile;
    __device__ __forceinline__ void operator()(const uint16_t *list, int n, float (&acc)[G]) const {
        const int lane = threadIdx.x & 31;
        for (int i = lane; i < n; i += 32) {
            const uint32_t e = list[i];
            TileFma<T, G>::fma(tile, e >> 2, e & 3u, acc);
        }
    }
};

// Compact plane words [wr.lo, wr.hi) (clearing them) into the ascending list
// of distinct bins and feed it to `dot` in lane order (entry i -> lane i%32).
// acc[] holds each lane's partial sums afterwards (no cross-lane reduction).
template <int G, typename Dot>
__device__ __forceinline__ int planes_accumulate(const Planes &pl, uint16_t *list, WordRange wr, const Dot &dot,
                                                 float (&acc)[G]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int g = 0; g < G; ++g) acc[g] = 0.0f;
    int nbuf = 0;
    int ntot = 0;
    for (int w0 = wr.lo; w0 < wr.hi; w0 += 32) {
        const int w = w0 + lane;
        uint32_t a = 0, h = 0, t = 0;
        if (w < wr.hi) {
            h = pl.H[w];
            t = pl.T[w];
            a = pl.A[w] | h;
            pl.A[w] = 0u;
            pl.H[w] = 0u;
            pl.T[w] = 0u;
        }
        const int pc = __popc(a);
        const int incl = warp_incl_scan(pc);
        const int total = __shfl_sync(kFullMask, incl, 31);
        if (nbuf + total > kListCap) {
            // flush whole multiples of 32 so that lane = global rank % 32 holds
            const int full = nbuf & ~31;
            dot(list, full, acc);
            __syncwarp();
            const int rem = nbuf - full;
            uint16_t keep = 0;
            if (lane < rem) keep = list[full + lane];
            __syncwarp();
            if (lane < rem) list[lane] = keep;
            __syncwarp();
            nbuf = rem;
        }
        int pos = nbuf + incl - pc;
        while (a) {
            const int b = __ffs(a) - 1;
            a &= a - 1u;
            const uint32_t lvl = ((t >> b) & 1u) ? 3u : (((h >> b) & 1u) ? 2u : 1u);
            list[pos++] = (uint16_t)((((uint32_t)w << 5 | (uint32_t)b) << 2) | lvl);
        }
        nbuf += total;
        ntot += total;
        __syncwarp();
    }
    dot(list, nbuf, acc);
    __syncwarp();
    return ntot;
}

// XOR butterfly (16, 8, 4, 2, 1) of every accumulator: all lanes end with the
// canonical sums.
template <int G>
__device__ __forceinline__ void butterfly_all(float (&acc)[G]) {
#pragma unroll
    for (int g = 0; g < G; ++g) {
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1)
            acc[g] = __fadd_rn(acc[g], __shfl_xor_sync(kFullMask, acc[g], off));
    }
}

// The same sums as butterfly_all, as a reduce-scatter: at offsets 16, 8, 4
// (and 2 for G = 16) each lane keeps half of its accumulators and receives
// its partner's copy of them, so every addition pairs the same operands as
// the full butterfly.  Returns the sum of accumulator slot_of_lane(lane);
// lanes differing only in bit 0 (G = 16), bits 0-1 (G = 8), 0-2 (G = 4),
// 0-3 (G = 2) hold the same slot.
template <int G>
__device__ __forceinline__ int reduce_slot_of_lane(int lane) {
    if constexpr (G == 16) return ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
    else if constexpr (G == 8) return ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
    else if constexpr (G == 4) return ((lane >> 4) & 1) * 2 + ((lane >> 3) & 1);
    else if constexpr (G == 2) return (lane >> 4) & 1;
    else return 0;
}
template <int G>
__device__ __forceinline__ float reduce_scatter(float (&acc)[G]) {
    const int lane = threadIdx.x & 31;
    float v[G];
#pragma unroll
    for (int g = 0; g < G; ++g) v[g] = acc[g];
    int n = G;
    int off = 16;
#pragma unroll
    for (int step = 0; step < 4; ++step) {
        if (n == 1) break;
        const int half = n / 2;
        const bool hi = (lane & off) != 0;
#pragma unroll
        for (int k = 0; k < G / 2; ++k) {
            if (k < half) {
                const float send = hi ? v[k] : v[half + k];
                const float keep = hi ? v[half + k] : v[k];
                v[k] = __fadd_rn(keep, __shfl_xor_sync(kFullMask, send, off));
            }
        }
        n = half;
        off >>= 1;
    }
    float s = v[0];
    for (; off >= 1; off >>= 1) s = __fadd_rn(s, __shfl_xor_sync(kFullMask, s, off));
    return s;
}

// reduce_scatter<G> within each group of W lanes (W = 32, 16 or 8: one
// candidate per group; the groups reduce separately): member j's sum ends in
// lanes j * W / G .. (j + 1) * W / G - 1 of each group.
template <int G, int W>
__device__ __forceinline__ float reduce_scatter_lanes(float (&acc)[G]) {
    static_assert(G <= W, "a lane group holds at most one sum per lane");
    const int lane = threadIdx.x & 31;
    float v[G];
#pragma unroll
    for (int g = 0; g < G; ++g) v[g] = acc[g];
    int n = G;
    int off = W / 2;
#pragma unroll
    for (int step = 0; step < 5; ++step) {
        if (n == 1 || off == 0) break;
        const int half = n / 2;
        const bool hi = (lane & off) != 0;
#pragma unroll
        for (int k = 0; k < G / 2; ++k) {
            if (k < half) {
                const float send = hi ? v[k] : v[half + k];
                const float keep = hi ? v[half + k] : v[k];
                v[k] = __fadd_rn(keep, __shfl_xor_sync(kFullMask, send, off));
            }
        }
        n = half;
        off >>= 1;
    }
    float s = v[0];
    for (; off >= 1; off >>= 1) s = __fadd_rn(s, __shfl_xor_sync(kFullMask, s, off));
    return s;
}

// Within each half-warp (lanes 0-15 and 16-31 reduce separately).
template <int G>
__device__ __forceinline__ float reduce_scatter16(float (&acc)[G]) {
    return reduce_scatter_lanes<G, 16>(acc);
}

// Compact the planes (clearing them) into the sorted distinct-bin list and
// accumulate the gather-dot for every active spectrum; every lane ends with
// the canonical sums.
template <typename T, int G>
__device__ __forceinline__ void planes_dot(const Planes &pl, uint16_t *list, WordRange wr,
                                           const SpecSet<T, G> &ss, float (&acc)[G],
                                           int *n_distinct = nullptr) {
    const int nt = planes_accumulate<G>(pl, list, wr, RowDot<T, G>{ss}, acc);
    butterfly_all<G>(acc);
    if (n_distinct) *n_distinct = nt;
}

// ---------------------------------------------------------------- top-K ---
// Final order (Search.hs:118-124 over b40c + sortBy): score descending, then
// the smaller key (plain keys < modified keys; position/rank ascending).
__device__ __forceinline__ bool better(float sa, uint64_t ka, float sb, uint64_t kb) {
    return sa > sb || (sa == sb && ka < kb);
}

// Warp-distributed sorted list: lane i holds entry i (i < K).
struct WarpTopK {
    float s;
    uint64_t k;
    __device__ __forceinline__ void init() {
        s = -INFINITY;
        k = ~0ull;
    }
    // Insert (ns, nk); all lanes pass the same values.
    __device__ __forceinline__ void insert(float ns, uint64_t nk, int K) {
        const int lane = threadIdx.x & 31;
        const bool mine_better = (lane < K) && better(s, k, ns, nk);
        const uint32_t bal = __ballot_sync(kFullMask, mine_better);
        const int pos = __popc(bal);
        const float us = __shfl_up_sync(kFullMask, s, 1);
        const uint64_t uk = __shfl_up_sync(kFullMask, k, 1);
        if (pos < K) {
            if (lane == pos) { s = ns; k = nk; }
            else if (lane > pos && lane < K) { s = us; k = uk; }
        }
    }
};

// The same for up to 64 entries: lane l holds entries l (s0, k0) and
// 32 + l (s1, k1).
struct WarpTopK64 {
    float s0, s1;
    uint64_t k0, k1;
    __device__ __forceinline__ void init() {
        s0 = s1 = -INFINITY;
        k0 = k1 = ~0ull;
    }
    __device__ __forceinline__ void insert(float ns, uint64_t nk, int K) {
        const int lane = threadIdx.x & 31;
        const int i0 = lane, i1 = 32 + lane;
        const uint32_t b0 = __ballot_sync(kFullMask, i0 < K && better(s0, k0, ns, nk));
        const uint32_t b1 = __ballot_sync(kFullMask, i1 < K && better(s1, k1, ns, nk));
        const int pos = __popc(b0) + __popc(b1);
        // entry i moves to i + 1 for pos <= i < K - 1
        const float u0 = __shfl_up_sync(kFullMask, s0, 1), u1 = __shfl_up_sync(kFullMask, s1, 1);
        const uint64_t v0 = __shfl_up_sync(kFullMask, k0, 1), v1 = __shfl_up_sync(kFullMask, k1, 1);
        const float c = __shfl_sync(kFullMask, s0, 31);  // entry 31 becomes entry 32
        const uint64_t ck = __shfl_sync(kFullMask, k0, 31);
        if (pos < K) {
            if (i0 == pos) { s0 = ns; k0 = nk; }
            else if (i0 > pos && i0 < K) { s0 = u0; k0 = v0; }
            if (i1 == pos) { s1 = ns; k1 = nk; }
            else if (i1 > pos && i1 < K) {
                s1 = lane == 0 ? c : u1;
                k1 = lane == 0 ? ck : v1;
            }
        }
    }
};

// Bounded spin on an mbarrier phase: returns false after max_iter tries.
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t phase, uint32_t max_iter) {
    for (uint32_t i = 0; i < max_iter; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(phase)
            : "memory");
        if (ok) return true;
    }
    return false;
}

}  // namespace hfx
