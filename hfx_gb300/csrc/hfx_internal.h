// Internal declarations shared by the CUDA translation units and the C++ host.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace hfx {

constexpr int kListCap = 1056;   // u16 distinct-bin list entries per warp (1024 + 32)
constexpr int kMaxWords = 256;   // bit-plane words per plane (8192 bins)
constexpr int kMaxTopK = 32;     // per-warp top-K kept in registers
constexpr int kMaxKept = 64;     // candidates kept per spectrum for FP32 rescoring (list scoring)

struct LayoutParams {
    float bw;           // spectrum bin width (Correlation.hs:29-30)
    int32_t custom_bw;  // 1: custom width, the length formula divides the cutoff
    int32_t remove_pcr; // remove-precursor-peak (Correlation.hs:69-71)
    int32_t ppm;        // 0 Da, 1 ppm, 2 per spectrum: negative = ppm (new; the reference has Da only)
    int32_t max_len;    // longest row accepted (longer spectra get status 2 and score nothing)
    int32_t cap_len;    // > 0: an accepted row longer than this sets kErrTooLong (graph replays,
                        // whose row stride is fixed at capture)
};

// Per-spectrum metadata computed on the device (k_layout).
struct SpecMeta {
    int32_t npk, len, status;
    float cutoff, mass, eps, lo, hi;
    int32_t charges_plain, charges_mod;
};

// Search database on the device, in residual-mass order.
struct DevDB {
    const uint8_t *ions;        // packed residues (prepare_ions.cu encoding)
    const float *r_sorted;      // residual masses, ascending (stable)
    const uint32_t *tc_sorted;  // first residue
    const uint32_t *tn_sorted;  // end of the ion ladder (exclusive)
    const uint32_t *idx_sorted; // fragment index (sort.cu:28-35)
    uint32_t num_pep;
    float mt[32];               // residue masses by (byte & 31); 0 beyond 'Z'
};

// Variable modifications (Fragment.hs:260-289) on the device.
struct DevMods {
    int32_t num_ma, num_mod;
    float ma_mass[8];
    const int32_t *counts;  // [num_mod][num_ma]
    const float *delta;     // [num_mod]
    int32_t per_type;       // i-th acid counter: 0 reference, 1 per acid type
};

// Error bits written to the device error word.
enum : uint32_t {
    kErrListOverflow = 1u,
    kErrTimeout = 2u,
    kErrKeyOverflow = 4u,
    kErrTooLong = 8u,
    kErrBounds = 16u,
};

}  // namespace hfx

int hfx_launch_layout(const float *mz, const int64_t *off, const float *pcr, const float *z,
                      const float *tol, int32_t nspec, const hfx::LayoutParams &lp,
                      hfx::SpecMeta *meta, uint32_t *max_len, uint32_t *err, cudaStream_t st);
int hfx_launch_preprocess(const float *mz, const float *it, const int64_t *off, const float *pcr,
                          const hfx::LayoutParams &lp, const hfx::SpecMeta *meta, int32_t nspec,
                          int64_t stride, float *out32, __nv_bfloat16 *outbf, __half *outh, uint32_t *err,
                          cudaStream_t st);
