/*
 * CPU oracle for the SEQUEST search hot path (TEST INFRASTRUCTURE ONLY).
 * See hfx_oracle.h for the file-by-file list of reference code it restates.
 * Must be compiled with -ffp-contract=off and without -ffast-math: every
 * float operation below is one IEEE single-precision operation.
 */
#include "hfx_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

/* Host masses, Mass.hs:19-25 */
const float kHostH2O = 18.010565f;
const float kHostH = 1.007276f;
/* Device masses, ion_series.h:16-26 (they differ from the host's). */
const float kDevH2O = 18.01056f;
const float kDevNH3 = 17.02655f;
const float kDevCO = 27.9949f;
const float kDevH = 1.0078246f;
const float kBinMono = 1.0005079f;

/* Mass.hs:37-69 monoisotopic, :76-103 average; index c-'A'. */
const float kMono[26] = {
    71.037114f,  114.53494f, 103.009185f, 115.026943f, 129.042593f,
    147.068414f, 57.021464f, 137.058912f, 113.084064f, 113.16472f,
    128.094963f, 113.084064f, 131.040485f, 114.042927f, 114.07931f,
    97.052764f,  128.058578f, 156.101111f, 87.032028f,  101.047679f,
    150.04344f,  99.068414f,  186.079313f, 113.08406f,  163.06332f,
    128.55059f};
const float kAvg[26] = {
    71.0788f,  114.5962f, 103.1388f, 115.0886f, 129.1155f, 147.1766f,
    57.0519f,  137.1411f, 113.1594f, 113.240178f, 128.1741f, 113.1594f,
    131.1926f, 114.1038f, 114.1472f, 97.1167f,  128.1307f, 156.1875f,
    87.0782f,  101.1051f, 150.0388f, 99.1326f,  186.2132f, 113.1594f,
    163.1760f, 128.6231f};

/* Config.hs:415-431 digestion rules (cleave after these residues). */
bool rule_match(int rule, uint8_t c) {
    switch (rule) {
    case 0: return false;
    case 1: return c == 'K' || c == 'R';
    case 2: return c == 'F' || c == 'W' || c == 'Y';
    case 3: return c == 'R';
    case 4: return c == 'M';
    case 5: return c == 'W';
    case 6: return c == 'P';
    case 7: return c == 'E';
    case 8: return c == 'K';
    case 9: return c == 'R';
    case 10: return c == 'D';
    case 11: return c == 'F' || c == 'W' || c == 'Y' || c == 'L';
    case 12: return c == 'A' || c == 'L' || c == 'I' || c == 'V';
    case 13:
        return c == 'A' || c == 'L' || c == 'I' || c == 'V' || c == 'K' ||
               c == 'R' || c == 'W' || c == 'F' || c == 'Y';
    default: return false;
    }
}

/* float -> uint32 conversion as the device performs it (saturating, NaN->0);
 * the value is then reinterpreted as int32 (ion_series.cu:65-75). */
inline int32_t sat_bin(float r) {
    uint32_t u;
    if (!(r > 0.0f)) u = 0u;                       /* negatives, -0, NaN */
    else if (r >= 4294967296.0f) u = 0xFFFFFFFFu;
    else u = (uint32_t)r;
    return (int32_t)u;
}

/* ion_series.cu:59-69 with IEEE division in place of __fdividef. */
inline float ion_mz(float m, float c, float hc) { return (m + hc) / c; }
/* ion_series.cu:65-69 bins every ion with the mono width (H3); ibw > 0 is
 * the new switch that bins ions with a custom width instead (0.02 Da rows). */
inline int32_t bin_mz(float mz, float ibw) { return sat_bin(std::rint(mz / (ibw > 0.0f ? ibw : kBinMono))); }

struct Hist {
    /* dense max-level row over [0,len) + touched list: the reference's
     * atomicMax into a zeroed row (ion_series.cu:71-75) */
    std::vector<uint8_t> lvl;
    std::vector<uint32_t> touched;
    void reset(int32_t len) {
        if ((int32_t)lvl.size() < len) lvl.assign(len, 0);
        touched.clear();
    }
    inline void add(int32_t x, uint8_t l, int32_t len) {
        if (0 <= x && x < len) {
            uint8_t &v = lvl[x];
            if (v == 0) touched.push_back((uint32_t)x);
            if (l > v) v = l;
        }
    }
};

/* ion_series.cu:78-123: the 10 ions of one (b, y, charge). */
inline void add_ions(Hist &h, float b, float y, int c, int32_t len, float ibw) {
    const float cf = (float)c;
    const float hc = kDevH * cf;           /* MASS_H * charge (compile-time) */
    const float dh2o = kDevH2O / cf;
    const float dnh3 = kDevNH3 / cf;
    /* A ion */
    h.add(bin_mz(ion_mz(b - kDevCO, cf, hc), ibw), 1, len);
    /* B ions */
    float m = ion_mz(b, cf, hc);
    int32_t x = bin_mz(m, ibw);
    h.add(x, 3, len);
    h.add(x + 1, 2, len);
    h.add(x - 1, 2, len);
    h.add(bin_mz(m - dh2o, ibw), 1, len);
    h.add(bin_mz(m - dnh3, ibw), 1, len);
    /* Y ions */
    m = ion_mz(y + kDevH2O, cf, hc);
    x = bin_mz(m, ibw);
    h.add(x, 3, len);
    h.add(x + 1, 2, len);
    h.add(x - 1, 2, len);
    h.add(bin_mz(m - dnh3, ibw), 1, len);
}

/* ion_series.cu:176-213: per 32-residue chunk, lane 0 adds the previous
 * chunk's last prefix, then a Hillis-Steele inclusive scan (strides
 * 1,2,4,8,16) in FP32; y = residual - b. */
void gen_ions(Hist &h, const uint8_t *ions, const float *mt, uint32_t tc,
              uint32_t tn, float residual, int charges, int32_t len,
              const float *res_add, const uint8_t *modded, float ibw = 0.0f) {
    h.reset(len);
    if (charges <= 0) return;
    float carry = 0.0f;
    float v[32], nv[32];
    for (uint32_t base = tc; base < tn; base += 32) {
        int cnt = (int)std::min<uint32_t>(32u, tn - base);
        for (int l = 0; l < cnt; ++l) {
            uint8_t byte = ions[base + l];
            /* out-of-range texture fetches (unpacked bytes) read 0 */
            float m = (byte & 0x1Fu) < 26u ? mt[byte & 0x1Fu] : 0.0f;
            if (modded && modded[base + l - tc]) m = m + res_add[base + l - tc];
            v[l] = m;
        }
        v[0] = v[0] + carry;
        for (int d = 1; d < 32; d <<= 1) {
            for (int l = 0; l < cnt; ++l) nv[l] = (l >= d) ? v[l] + v[l - d] : v[l];
            for (int l = 0; l < cnt; ++l) v[l] = nv[l];
        }
        carry = v[cnt - 1];
        for (int l = 0; l < cnt; ++l) {
            const float b = v[l];
            const float y = residual - b;
            for (int c = 1; c <= charges; ++c) add_ions(h, b, y, c, len, ibw);
        }
    }
}

int32_t collect(Hist &h, uint32_t *bins, uint8_t *lvl, int32_t cap) {
    std::sort(h.touched.begin(), h.touched.end());
    int32_t n = (int32_t)h.touched.size();
    if (n > cap) return -1;
    for (int32_t i = 0; i < n; ++i) {
        bins[i] = h.touched[i];
        lvl[i] = h.lvl[h.touched[i]];
        h.lvl[h.touched[i]] = 0;
    }
    return n;
}

const float kW[4] = {0.0f, 10.0f, 25.0f, 50.0f};

template <typename T, typename F>
T canonical_dot(const uint32_t *bins, const uint8_t *lvl, int32_t n, F xat) {
    T acc[32];
    for (int l = 0; l < 32; ++l) acc[l] = (T)0;
    for (int32_t i = 0; i < n; ++i) {
        T w = (T)kW[lvl[i]];
        if constexpr (sizeof(T) == 4) acc[i & 31] = std::fmaf(w, xat(bins[i]), acc[i & 31]);
        else acc[i & 31] = std::fma(w, xat(bins[i]), acc[i & 31]);
    }
    T tmp[32];
    for (int off = 16; off >= 1; off >>= 1) {
        for (int l = 0; l < 32; ++l) tmp[l] = acc[l] + acc[l ^ off];
        for (int l = 0; l < 32; ++l) acc[l] = tmp[l];
    }
    return acc[0];
}

/* combinatorics.h:59-88 */
uint32_t choose_slow(uint32_t n, uint32_t k) {
    if (k == 0 || n == k) return 1;
    if (n < k) return 0;
    uint32_t i, t = 1;
    if (k < n - k) {
        for (i = n; i >= n - k + 1; --i) t = t * i / (n - i + 1);
    } else {
        for (i = n; i >= k + 1; --i) t = t * i / (n - i + 1);
    }
    return t;
}
uint32_t binom_table(uint32_t n, uint32_t k) {
    /* the reference tabulates C(n<=42, k<=11) exactly (values fit in u32) */
    if (k > n) return 0;
    uint64_t t = 1;
    for (uint32_t i = 1; i <= k; ++i) t = t * (n - k + i) / i;
    return (uint32_t)t;
}

/* bf16 / fp16 round-to-nearest-even storage of a float */
float to_bf16(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7F800000u) == 0x7F800000u) return x;
    uint32_t lsb = (u >> 16) & 1u;
    u = (u + 0x7FFFu + lsb) & 0xFFFF0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
float to_fp16(float x) {
    /* IEEE binary16, round to nearest even, via exact scaling in double */
    if (std::isnan(x)) return x;
    double a = std::fabs((double)x);
    if (a >= 65520.0) return std::copysign(INFINITY, x);
    int e;
    std::frexp(a, &e);                 /* a = f * 2^e, f in [0.5,1) */
    int exp = e - 1;                   /* a in [2^exp, 2^(exp+1)) */
    if (exp < -14) exp = -14;          /* subnormal spacing 2^-24 */
    double q = std::ldexp(1.0, exp - 10);
    double r = std::nearbyint(a / q) * q;
    return (float)std::copysign(r, (double)x);
}

struct Entry {
    float s;
    double s64;
    uint64_t key;
    uint32_t pep;
};
inline bool better(const Entry &a, const Entry &b) {
    if (a.s != b.s) return a.s > b.s;
    return a.key < b.key;
}

} // namespace

extern "C" {

void hfxo_mass_table(int mono, const float *add, float *out) {
    for (int i = 0; i < 26; ++i) out[i] = add[i] + (mono ? kMono[i] : kAvg[i]);
}

int64_t hfxo_digest(const uint8_t *seq, const uint32_t *seg, int32_t nprot,
                    const float *mt, int rule, int missed, float min_mass,
                    float max_mass, int proline_rule, int min_len, int max_len,
                    float *r, uint32_t *tc, uint32_t *tn, int64_t cap) {
    int64_t nf = 0;
    struct F { float m; uint32_t c, n, len; };
    std::vector<F> frags;
    for (int32_t p = 0; p < nprot; ++p) {
        const uint32_t x = seg[p], y = seg[p + 1];
        /* Fragment.hs:376-390 fragment: unfoldr over the segment */
        frags.clear();
        uint32_t c = x;
        while (c < y) {
            uint32_t len = y - c;
            int64_t found = -1;
            for (uint32_t i = 0; i < len; ++i) {
                if (rule_match(rule, seq[c + i])) {
                    if (proline_rule && i + 1 < len && seq[c + i + 1] == 'P') continue;
                    found = i;
                    break;
                }
            }
            if (found < 0) {
                float m = 0.0f;
                for (uint32_t i = 0; i < len; ++i) m = m + mt[seq[c + i] - 'A'];
                frags.push_back({m, c, c + len, len});      /* tn one past */
                break;
            }
            uint32_t n = (uint32_t)found;
            float m = 0.0f;
            for (uint32_t i = 0; i <= n; ++i) m = m + mt[seq[c + i] - 'A'];
            frags.push_back({m, c, c + n, n + 1});           /* tn inclusive */
            c = c + n + 1;
        }
        /* Fragment.hs:397-405 splice: scanl fuse p (take n ps) ++ loop ps */
        for (size_t i = 0; i < frags.size(); ++i) {
            F acc = frags[i];
            for (int k = 0; k <= missed && i + k < frags.size(); ++k) {
                if (k > 0) {
                    const F &b = frags[i + k];
                    acc = {acc.m + b.m, acc.c, b.n, acc.len + b.len};
                }
                /* Fragment.hs:365-369 mass filter on res + H2O + H */
                float mm = (acc.m + kHostH2O) + kHostH;
                bool ok = (min_mass <= mm && mm <= max_mass);
                if (min_len > 0 && (int)acc.len < min_len) ok = false;
                if (max_len > 0 && (int)acc.len > max_len) ok = false;
                if (ok) {
                    if (nf >= cap) return -1;
                    r[nf] = acc.m;
                    tc[nf] = acc.c;
                    tn[nf] = acc.n;
                    ++nf;
                }
            }
        }
    }
    return nf;
}

void hfxo_sort_idx(const float *r, int64_t n, uint32_t *idx) {
    std::vector<uint32_t> v(n);
    std::iota(v.begin(), v.end(), 0u);
    std::stable_sort(v.begin(), v.end(), [&](uint32_t a, uint32_t b) { return r[a] < r[b]; });
    std::memcpy(idx, v.data(), n * sizeof(uint32_t));
}

void hfxo_pack_ions(uint8_t *ions, int64_t n, const uint8_t *ma, int num_ma,
                    int quirk) {
    /* prepare_ions.cu:98-103: blocks = n / (threads*4) is zero for n < 512,
     * so the reference leaves such a database unpacked. */
    if (quirk && n < 512) return;
    for (int64_t i = 0; i < n; ++i) {
        uint8_t c = ions[i];
        uint8_t mod = 0;
        for (int j = 0; j < num_ma; ++j)
            if (ma[j] == c) { mod = (uint8_t)(j + 1); break; }
        ions[i] = (uint8_t)((uint8_t)(c - 'A') | (uint8_t)(mod << 5));
    }
}

float hfxo_ms2_mass(float pcr, float z) {
    /* Spectrum/Data.hs:58-59 */
    return ((pcr * z) - ((z - 1.0f) * kHostH)) - (kHostH + kHostH2O);
}

static float spec_cutoff(const float *mz, int32_t npk, float pcr, float z) {
    /* Correlation.hs:65-67 */
    float mzcut = 50.0f + pcr * z;
    double t = std::trunc((double)(mz[npk - 1] / 10.0f));
    float mzlim = (float)(t * 10.0);
    return (mzcut <= mzlim) ? mzcut : mzlim;
}

int32_t hfxo_spec_len(const float *mz, int32_t npk, float pcr, float z,
                      float bw, int custom_bw) {
    if (npk <= 0) return -1;
    float cutoff = spec_cutoff(mz, npk, pcr, z);
    float c = custom_bw ? cutoff / bw : cutoff;
    double len = 75.0 + std::ceil((double)c);
    if (!(len >= 76.0) || len > 2.0e9) return -1;
    return (int32_t)len;
}

int32_t hfxo_preprocess(const float *mz, const float *it, int32_t npk,
                        float pcr, float z, float bw, int custom_bw,
                        int remove_pcr, float *out32, double *out64,
                        int32_t cap) {
    const int32_t len = hfxo_spec_len(mz, npk, pcr, z, bw, custom_bw);
    if (len < 0) return -1;
    if (len > cap) return -4;
    const float cutoff = spec_cutoff(mz, npk, pcr, z);
    const float plo = pcr - 15.0f, phi = pcr + 15.0f;
    std::vector<float> e(len, 0.0f);
    std::vector<double> e64(len, 0.0);
    /* Correlation.hs:58-71 observedIntensity */
    for (int32_t i = 0; i < npk; ++i) {
        const float x = mz[i];
        bool keep = remove_pcr ? (x <= cutoff && (x <= plo || phi <= x)) : (x <= cutoff);
        if (!keep) continue;
        const float q = std::rint(x / bw);
        if (!(q >= 0.0f) || q >= (float)len) return -2;
        const int32_t b = (int32_t)q;
        const float v = std::sqrt(it[i]);
        if (e[b] <= v) e[b] = v;                      /* max old new */
        const double v64 = std::sqrt((double)it[i]);
        if (e64[b] <= v64) e64[b] = v64;
    }
    /* Correlation.hs:84-96 normaliseByRegion */
    const int32_t cut = len - 75;
    const int32_t sel = cut / 10;
    if (sel <= 0) return -3;
    float rmax[11] = {0};
    double rmax64[11] = {0};
    for (int32_t i = 0; i < len; ++i) {
        int32_t g = std::min(10, i / sel);
        if (rmax[g] <= e[i]) rmax[g] = e[i];
        if (rmax64[g] <= e64[i]) rmax64[g] = e64[i];
    }
    std::vector<float> a(len);
    std::vector<double> a64(len);
    for (int32_t i = 0; i < len; ++i) {
        int32_t g = std::min(10, i / sel);
        const float m = rmax[g];
        a[i] = (m > 1e-6f && i < sel * 10) ? 50.0f * (e[i] / m) : 0.0f;
        const double m64 = rmax64[g];
        a64[i] = (m64 > 1e-6 && i < sel * 10) ? 50.0 * (e64[i] / m64) : 0.0;
    }
    /* Correlation.hs:105-109 crossCorrolation: sequential left fold from 0
     * over take 151 (drop (i-75) a), divided by 150. */
    for (int32_t i = 0; i < len; ++i) {
        int32_t lo = std::max(0, i - 75);
        int32_t hi = std::min(len, lo + 151);
        if (out32) {
            float s = 0.0f;
            for (int32_t j = lo; j < hi; ++j) s = s + a[j];
            out32[i] = a[i] - s / 150.0f;
        }
        if (out64) {
            double s = 0.0;
            for (int32_t j = lo; j < hi; ++j) s = s + a64[j];
            out64[i] = a64[i] - s / 150.0;
        }
    }
    return len;
}

void hfxo_windows(const float *rs, int64_t n, const float *lo, const float *hi,
                  int64_t nq, uint32_t *begin, uint32_t *end) {
    for (int64_t q = 0; q < nq; ++q) {
        begin[q] = (uint32_t)(std::lower_bound(rs, rs + n, lo[q]) - rs);
        end[q] = (uint32_t)(std::upper_bound(rs, rs + n, hi[q]) - rs);
    }
}

int32_t hfxo_ion_charges(float z, int is_mod) {
    /* Search.hs:182 max_chs = round (max 1 (chrg - 1)) */
    float zm = z - 1.0f;
    float mc = (1.0f <= zm) ? zm : 1.0f;
    float rr = std::rint(mc);
    if (!(rr >= 1.0f)) return 0;
    int32_t ch = (rr > 1000.0f) ? 1000 : (int32_t)rr;
    if (!is_mod) return (ch <= 4) ? ch : 0;             /* ion_series.cu:301-309 */
    if (ch > 10) return 0;                               /* mion_series.cu:425-438 */
    return std::min(ch, 4);                              /* mion_series.cu:303-306 */
}

int32_t hfxo_ion_bins(const uint8_t *ions, const float *mt, uint32_t tc,
                      uint32_t tn, float residual, int32_t charges, int32_t len,
                      const float *res_add, const uint8_t *modded,
                      uint32_t *bins, uint8_t *lvl, int32_t cap) {
    Hist h;
    gen_ions(h, ions, mt, tc, tn, residual, charges, len, res_add, modded);
    return collect(h, bins, lvl, cap);
}

float hfxo_score32(const uint32_t *bins, const uint8_t *lvl, int32_t n,
                   const float *x) {
    return canonical_dot<float>(bins, lvl, n, [&](uint32_t b) { return x[b]; });
}
double hfxo_score64(const uint32_t *bins, const uint8_t *lvl, int32_t n,
                    const double *x) {
    return canonical_dot<double>(bins, lvl, n, [&](uint32_t b) { return x[b]; });
}

uint32_t hfxo_choose(uint32_t n, uint32_t k) {
    if (n > 42 || k > 11) return choose_slow(n, k);
    return binom_table(n, k);
}

void hfxo_unrank_comb(uint32_t *ans, uint32_t n, uint32_t k, uint32_t rank) {
    /* combinatorics.h:90-134 */
    uint32_t a = n, b = k;
    uint32_t total = hfxo_choose(n, k);
    uint32_t x;
    bool dual = false;
    if ((total / 2) >= rank) x = rank;
    else { x = total - 1 - rank; dual = true; }
    for (uint32_t i = 0; i < k; ++i) {
        uint32_t v = a - 1;
        while (hfxo_choose(v, b) > x) --v;
        ans[i] = v;
        x = x - hfxo_choose(ans[i], b);
        a = ans[i];
        b = b - 1;
    }
    if (dual)
        for (uint32_t i = 0; i < k; ++i) ans[i] = (n - 1) - ans[i];
}

int32_t hfxo_mod_combos(int32_t num_ma, int32_t max_ma, const float *ma_mass,
                        int32_t *counts, int32_t *sums, float *deltas,
                        int32_t cap) {
    /* Fragment.hs:275-289: all count vectors over 0..max_ma, expanded with
     * dimension 0 outermost (lexicographic, dim 0 most significant), the
     * all-zero vector dropped, kept when sum < max_ma (strict). */
    if (num_ma <= 0) return 0;
    std::vector<int32_t> c(num_ma, 0);
    int32_t nm = 0;
    while (true) {
        /* odometer increment with the last dimension fastest */
        int d = num_ma - 1;
        while (d >= 0) {
            if (c[d] < max_ma) { ++c[d]; break; }
            c[d] = 0;
            --d;
        }
        if (d < 0) break;
        int32_t s = 0;
        for (int i = 0; i < num_ma; ++i) s += c[i];
        if (s < max_ma) {
            if (nm >= cap) return -1;
            float delta = 0.0f;                           /* U.sum: foldl' (+) 0 */
            for (int i = 0; i < num_ma; ++i) delta = delta + ma_mass[i] * (float)c[i];
            for (int i = 0; i < num_ma; ++i) counts[nm * num_ma + i] = c[i];
            sums[nm] = s;
            deltas[nm] = delta;
            ++nm;
        }
    }
    return nm;
}

uint32_t hfxo_mod_isoform(const uint8_t *ions, uint32_t tc, uint32_t tn,
                          const uint8_t *ma, int32_t num_ma,
                          const int32_t *mc, uint32_t rank, int per_type,
                          uint32_t *unrank_out, uint8_t *modded_out) {
    (void)ma;
    uint32_t D[16] = {0};
    /* filter_by_mod.cu:216-230 (the packed byte's mod field names the acid) */
    for (uint32_t a = tc; a < tn; ++a) {
        uint32_t mod = (ions[a] >> 5) & 7u;
        if (mod) D[mod - 1]++;
    }
    /* filter_by_mod.cu:251-261 checkModable */
    for (int i = 0; i < num_ma; ++i)
        if (D[i] < (uint32_t)mc[i]) return 0;
    /* calc_mod_cands.cu:49-66 suffix products */
    uint32_t scan[16];
    uint32_t num = 1;
    for (int i = num_ma - 1; i >= 0; --i) {
        num *= hfxo_choose(D[i], (uint32_t)mc[i]);
        scan[i] = num;
    }
    if (rank >= num || !unrank_out) return num;
    /* gen_mod_pep.cu:127-157 add_ma_ranks */
    uint32_t mar[16];
    uint32_t x = rank;
    for (int i = 0; i < num_ma; ++i) {
        if (i != num_ma - 1) {
            uint32_t nx = scan[i + 1];
            if (x >= nx) { mar[i] = x / nx; x = x % nx; }
            else mar[i] = 0;
        } else mar[i] = x;
    }
    /* gen_mod_pep.cu:208-222 */
    uint32_t pos = 0;
    uint32_t start[16];
    for (int i = 0; i < num_ma; ++i) {
        start[i] = pos;
        if (mc[i] != 0) {
            hfxo_unrank_comb(unrank_out + pos, D[i], (uint32_t)mc[i], mar[i]);
            pos += (uint32_t)mc[i];
        }
    }
    if (modded_out) {
        /* mion_series.cu:244-286: ith = (number of modable residues seen so
         * far, of any acid) - 1; per_type counts the same acid only
         * (check_series.cu:62-100). */
        uint32_t seen_any = 0, seen[16] = {0};
        for (uint32_t a = tc; a < tn; ++a) {
            uint32_t mod = (ions[a] >> 5) & 7u;
            uint8_t f = 0;
            if (mod) {
                uint32_t t = mod - 1;
                uint32_t ith = per_type ? seen[t] : seen_any;
                seen[t]++;
                seen_any++;
                for (int l = 0; l < mc[t]; ++l)
                    if (unrank_out[start[t] + l] == ith) f = 1;
            }
            modded_out[a - tc] = f;
        }
    }
    return num;
}

int32_t hfxo_search_scores(const uint8_t *ions, const float *mt, const float *r,
                           const uint32_t *tc, const uint32_t *tn,
                           const uint32_t *idx, int64_t num_pep, const float *mz,
                           const float *it, const int64_t *off, const float *pcr,
                           const float *z, const float *tol, int32_t nspec,
                           const hfxo_params *p, int32_t nthreads, float *out_score,
                           double *out_score64, uint64_t *out_key, uint32_t *out_pep,
                           int64_t *out_ncand, const int64_t *sink_off, float *sink) {
    const int32_t topn = p->topn;
    std::vector<float> rs(num_pep);
    for (int64_t i = 0; i < num_pep; ++i) rs[i] = r[idx[i]];
    /* modification table */
    int32_t num_mod = 0;
    std::vector<int32_t> mcount, msum;
    std::vector<float> mdelta;
    if (p->num_ma > 0) {
        const int cap = 1 << 16;
        mcount.resize((size_t)cap * p->num_ma);
        msum.resize(cap);
        mdelta.resize(cap);
        num_mod = hfxo_mod_combos(p->num_ma, p->max_ma, p->ma_mass, mcount.data(),
                                  msum.data(), mdelta.data(), cap);
        if (num_mod < 0) return -1;
    }
    const float ppm_scale = 1e-6f;
    int32_t status = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        Hist h;
        std::vector<uint32_t> bins(1 << 16);
        std::vector<uint8_t> lv(1 << 16);
        std::vector<float> x32;
        std::vector<double> x64;
        std::vector<float> xs;
        std::vector<Entry> top;
        std::vector<uint32_t> unrank(256);
        std::vector<uint8_t> modded(4096);
        std::vector<float> radd(4096);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int32_t s = 0; s < nspec; ++s) {
            const int64_t o = off[s];
            const int32_t npk = (int32_t)(off[s + 1] - o);
            top.clear();
            int64_t ncand = 0;
            int32_t len = hfxo_spec_len(mz + o, npk, pcr[s], z[s], p->bw, p->custom_bw);
            if (len > 0) {
                x32.assign(len, 0.0f);
                x64.assign(len, 0.0);
                int32_t l2 = hfxo_preprocess(mz + o, it + o, npk, pcr[s], z[s], p->bw,
                                             p->custom_bw, p->remove_pcr, x32.data(),
                                             p->prec == 3 ? x64.data() : nullptr, len);
                if (l2 != len) len = -1;
            }
            if (len > 0) {
                xs.resize(len);
                for (int32_t i = 0; i < len; ++i)
                    xs[i] = p->prec == 1 ? to_bf16(x32[i]) : p->prec == 2 ? to_fp16(x32[i]) : x32[i];
                const float mass = hfxo_ms2_mass(pcr[s], z[s]);
                const float ts = tol[s];
                const bool in_ppm = p->ppm == 1 || (p->ppm == 2 && ts < 0.0f);
                const float eps = in_ppm ? mass * ((p->ppm == 2 ? -ts : ts) * ppm_scale) : ts;
                const float lo = mass - eps, hi = mass + eps;
                auto score_list = [&](int32_t n, Entry &e) {
                    e.s = hfxo_score32(bins.data(), lv.data(), n, xs.data());
                    e.s64 = p->prec == 3 ? hfxo_score64(bins.data(), lv.data(), n, x64.data()) : (double)e.s;
                    if (p->prec == 3) e.s = (float)e.s64;
                };
                auto push = [&](const Entry &e) {
                    if (sink) sink[sink_off[s] + ncand] = e.s;
                    if ((int32_t)top.size() < topn) {
                        top.push_back(e);
                        std::push_heap(top.begin(), top.end(), better);
                    } else if (better(e, top.front())) {
                        std::pop_heap(top.begin(), top.end(), better);
                        top.back() = e;
                        std::push_heap(top.begin(), top.end(), better);
                    }
                };
                if (p->plain) {
                    const int32_t ch = hfxo_ion_charges(z[s], 0);
                    uint32_t b = (uint32_t)(std::lower_bound(rs.begin(), rs.end(), lo) - rs.begin());
                    uint32_t e = (uint32_t)(std::upper_bound(rs.begin(), rs.end(), hi) - rs.begin());
                    for (uint32_t q = b; q < e; ++q) {
                        const uint32_t pi = idx[q];
                        gen_ions(h, ions, mt, tc[pi], tn[pi], r[pi], ch, len, nullptr, nullptr, p->ion_bw);
                        int32_t n = collect(h, bins.data(), lv.data(), (int32_t)bins.size());
                        Entry en;
                        if (n < 0) { status = -2; n = 0; }
                        score_list(n, en);
                        en.key = q;
                        en.pep = pi;
                        push(en);
                        ++ncand;
                    }
                }
                if (num_mod > 0) {
                    const int32_t ch = hfxo_ion_charges(z[s], 1);
                    for (int32_t mi = 0; mi < num_mod; ++mi) {
                        /* filter_by_mod.cu:72-80: ((m-eps) - delta), ((m+eps) - delta) */
                        const float mlo = lo - mdelta[mi], mhi = hi - mdelta[mi];
                        uint32_t b = (uint32_t)(std::lower_bound(rs.begin(), rs.end(), mlo) - rs.begin());
                        uint32_t e = (uint32_t)(std::upper_bound(rs.begin(), rs.end(), mhi) - rs.begin());
                        const int32_t *mc = &mcount[(size_t)mi * p->num_ma];
                        for (uint32_t q = b; q < e; ++q) {
                            const uint32_t pi = idx[q];
                            const uint32_t L = tn[pi] - tc[pi];
                            if (L > modded.size()) { status = -3; continue; }
                            uint32_t niso = hfxo_mod_isoform(ions, tc[pi], tn[pi], p->ma, p->num_ma,
                                                             mc, UINT32_MAX, p->per_type, nullptr, nullptr);
                            /* mion_series.cu:226 residual + delta */
                            const float resid = r[pi] + mdelta[mi];
                            for (uint32_t rk = 0; rk < niso; ++rk) {
                                hfxo_mod_isoform(ions, tc[pi], tn[pi], p->ma, p->num_ma, mc, rk,
                                                 p->per_type, unrank.data(), modded.data());
                                for (uint32_t a = 0; a < L; ++a) {
                                    uint32_t mod = (ions[tc[pi] + a] >> 5) & 7u;
                                    radd[a] = mod ? p->ma_mass[mod - 1] : 0.0f;
                                }
                                gen_ions(h, ions, mt, tc[pi], tn[pi], resid, ch, len, radd.data(), modded.data(),
                                         p->ion_bw);
                                int32_t n = collect(h, bins.data(), lv.data(), (int32_t)bins.size());
                                Entry en;
                                if (n < 0) { status = -2; n = 0; }
                                if (mi >= 512 || q >= (1u << 27) || rk >= (1u << 27)) status = -4;
                                score_list(n, en);
                                en.key = (1ull << 63) | ((uint64_t)mi << 54) | ((uint64_t)q << 27) | (uint64_t)rk;
                                en.pep = pi;
                                push(en);
                                ++ncand;
                            }
                        }
                    }
                }
            }
            std::sort(top.begin(), top.end(), better);
            for (int32_t k = 0; k < topn; ++k) {
                const size_t w = (size_t)s * topn + k;
                if (k < (int32_t)top.size()) {
                    out_score[w] = top[k].s;
                    if (out_score64) out_score64[w] = top[k].s64;
                    out_key[w] = top[k].key;
                    out_pep[w] = top[k].pep;
                } else {
                    out_score[w] = -INFINITY;
                    if (out_score64) out_score64[w] = -INFINITY;
                    out_key[w] = UINT64_MAX;
                    out_pep[w] = UINT32_MAX;
                }
            }
            if (out_ncand) out_ncand[s] = ncand;
        }
    }
    return status;
}

void hfxo_match_ions(const float *x, int32_t len, float z, float bw,
                     const uint8_t *pep, int32_t L, const float *mt, float mh,
                     int32_t nstar, int32_t *matched, int32_t *total) {
    /* IonSeries.hs:99-109 extractPeaks */
    std::vector<int32_t> order((size_t)std::max(len, 0));
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return x[a] > x[b]; });
    const int32_t np = len / 3 + 1;
    std::vector<float> peaks((size_t)np, 0.0f);
    for (int32_t k = 0; k < std::min(len, 200); ++k) {
        const int32_t i = order[k];
        peaks[i / 3] = std::max(peaks[i / 3], x[i]);
    }
    /* IonSeries.hs:87-91 bions: charges [1 .. max 1 (charge-1)] */
    std::vector<float> ions;
    const float lim = std::max(1.0f, z - 1.0f);
    for (float c = 1.0f; c <= lim + 0.5f; c = c + 1.0f) {
        float m = 0.0f;
        for (int32_t a = 0; a < L; ++a) {
            m = m + mt[pep[a] - 'A'];
            ions.push_back((m + kHostH * c) / c);   /* IonSeries.hs:44 ionMZ */
        }
    }
    /* IonSeries.hs:132-147 matchIonSequence */
    auto hit = [&](float v) {
        const float q = (v / bw) / 3.0f;
        const double rq = (double)std::nearbyint(q);
        if (!(rq >= 0.0 && rq < (double)np)) return 0;
        return peaks[(size_t)rq] > 0.0f ? 1 : 0;
    };
    int32_t cnt = 0;
    const size_t n = ions.size();
    for (size_t k = 0; k + 1 < n; ++k) cnt += hit(ions[k]);      /* init (b) */
    for (size_t k = 1; k < n; ++k) cnt += hit(mh - ions[k]);     /* tail (y) */
    *matched = cnt;
    *total = (L + 4 + nstar - 5) * 2;                            /* Match.hs:41 */
}

int32_t hfxo_search(const uint8_t *ions, const float *mt, const float *r,
                    const uint32_t *tc, const uint32_t *tn,
                    const uint32_t *idx, int64_t num_pep, const float *mz,
                    const float *it, const int64_t *off, const float *pcr,
                    const float *z, const float *tol, int32_t nspec,
                    const hfxo_params *p, int32_t nthreads, float *out_score,
                    double *out_score64, uint64_t *out_key, uint32_t *out_pep,
                    int64_t *out_ncand) {
    return hfxo_search_scores(ions, mt, r, tc, tn, idx, num_pep, mz, it, off, pcr, z, tol, nspec, p,
                              nthreads, out_score, out_score64, out_key, out_pep, out_ncand, nullptr,
                              nullptr);
}

} // extern "C"
