// Allocation-free scoring of one spectrum (hfx_score_spectrum_noalloc).
//
// Some callers cannot call cudaMalloc: code that runs inside another
// framework's memory pool or allocator hooks, host runtimes whose only
// device memory is what they were handed, or latency-critical paths that
// must not take the allocator's locks.  For them this entry point scores one
// spectrum against caller-provided device buffers and allocates nothing: its
// only scratch -- the per-block partial top-K lists that the regular path
// keeps in a context workspace -- lives in the file-scope device array
// below, of fixed size, which every GPU that loads the library holds until
// the process exits.
//
// The kernels are variants of the per-spectrum scorer and merge of search.cu
// (same device routines, same canonical FP32 order), so the results equal
// the regular per-spectrum path's bit for bit.
#include <algorithm>

#include "hfx_internal.h"
#include "device_common.cuh"
#include "../../include/hfx_gpu.h"

namespace hfx {
namespace {

constexpr int kNaMaxBlocks = HFX_NOALLOC_MAX_BLOCKS;
constexpr int kNaMaxK = 32;
constexpr int kNaWarps = 8;
constexpr size_t kNaScoreBytes = (size_t)kNaMaxBlocks * kNaMaxK * sizeof(float);
constexpr size_t kNaKeyBytes = (size_t)kNaMaxBlocks * kNaMaxK * sizeof(uint64_t);

// The scratch: partial lists (scores, then keys) of the last call's blocks.
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNaScoreBytes + kNaKeyBytes];

template <bool FastDiv>
__global__ void __launch_bounds__(256) k_score_spectrum_na(DevDB db, const float *__restrict__ row, int32_t len,
                                                           int32_t charges, uint32_t begin, uint32_t end,
                                                           int32_t words, int32_t K, uint8_t *__restrict__ scratch) {
    extern __shared__ __align__(16) uint8_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float *part_s = reinterpret_cast<float *>(scratch);
    uint64_t *part_k = reinterpret_cast<uint64_t *>(scratch + kNaScoreBytes);
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
        const WordRange wr = build_planes<FastDiv>(pl, db.ions, db.tc_sorted[p], db.tn_sorted[p],
                                                   db.r_sorted[p], charges, len, mt_lane, NoMods{});
        float acc[1];
        planes_dot<float, 1>(pl, list, wr, ss, acc);
        tk.insert(acc[0], (uint64_t)p, K);
    }
    __syncthreads();
    // merge the warps' lists in shared memory (planes reused as scratch)
    float *sm_s = reinterpret_cast<float *>(planes);
    uint64_t *sm_k = reinterpret_cast<uint64_t *>(planes) + (size_t)nw * K;
    if (lane < K) {
        sm_s[warp * K + lane] = tk.s;
        sm_k[warp * K + lane] = tk.k;
    }
    __syncthreads();
    if (warp == 0) {
        tk.init();
        for (int j = 0; j < nw * K; ++j)
            if (sm_k[j] != ~0ull) tk.insert(sm_s[j], sm_k[j], K);
        if (lane < K) {
            part_s[(size_t)blockIdx.x * K + lane] = tk.s;
            part_k[(size_t)blockIdx.x * K + lane] = tk.k;
        }
    }
}

// One warp merges the blocks' lists of this call into the caller's outputs.
__global__ void k_merge_na(const uint8_t *__restrict__ scratch, int32_t nblocks, int32_t K,
                           const uint32_t *__restrict__ idx_sorted, float *__restrict__ out_s,
                           uint64_t *__restrict__ out_k, uint32_t *__restrict__ out_pep) {
    const int lane = threadIdx.x & 31;
    const float *part_s = reinterpret_cast<const float *>(scratch);
    const uint64_t *part_k = reinterpret_cast<const uint64_t *>(scratch + kNaScoreBytes);
    WarpTopK tk;
    tk.init();
    for (int32_t j0 = 0; j0 < nblocks * K; j0 += 32) {
        const int32_t j = j0 + lane;
        const float sc = j < nblocks * K ? part_s[j] : -INFINITY;
        const uint64_t kk = j < nblocks * K ? part_k[j] : ~0ull;
        const int m = min(32, nblocks * K - j0);
        for (int t = 0; t < m; ++t) {
            const float ts = __shfl_sync(kFullMask, sc, t);
            const uint64_t tk2 = __shfl_sync(kFullMask, kk, t);
            if (tk2 != ~0ull) tk.insert(ts, tk2, K);
        }
    }
    if (lane < K) {
        out_s[lane] = tk.s;
        out_k[lane] = tk.k;
        out_pep[lane] = (tk.k != ~0ull) ? idx_sorted[(uint32_t)tk.k] : ~0u;
    }
}

// Dynamic shared memory of one launch: the row, then the larger of the
// warps' bit planes with their staging lists and the block's merge buffer.
size_t smem_bytes(int32_t len, int32_t top_n) {
    const size_t words = (size_t)(len + 31) / 32;
    return (size_t)((len + 3) & ~3) * 4 +
           std::max((size_t)kNaWarps * 3 * words * 4 + (size_t)kNaWarps * kListCap * 2,
                    (size_t)kNaWarps * top_n * 16);
}

// Set-up, with the device current: the scratch array's device address (the
// host-side name of a __device__ array is not a device address) and the
// kernels' shared-memory limit, sized for the largest launch this entry
// point makes.  It runs on every call: both are host calls that allocate
// nothing, and redoing them keeps a call correct after a device reset or
// under another context on the same device, where the module is loaded
// anew.
int32_t setup_device(uint8_t **scratch, int *smem_limit) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HFX_ERR_CUDA;
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return HFX_ERR_CUDA;
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
        return HFX_ERR_CUDA;
    const int want = (int)std::min<size_t>(smem_bytes(kMaxWords * 32, kNaMaxK), (size_t)optin);
    if (cudaFuncSetAttribute(k_score_spectrum_na<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, want) !=
            cudaSuccess ||
        cudaFuncSetAttribute(k_score_spectrum_na<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, want) !=
            cudaSuccess)
        return HFX_ERR_CUDA;
    *scratch = static_cast<uint8_t *>(p);
    *smem_limit = want;
    return HFX_OK;
}

}  // namespace
}  // namespace hfx

using namespace hfx;

extern "C" int32_t hfx_score_spectrum_noalloc(const uint8_t *ions, const float *r_sorted, const uint32_t *tc_sorted,
                                              const uint32_t *tn_sorted, const uint32_t *idx_sorted,
                                              uint32_t num_pep, const float *mass_table26, const float *row,
                                              int32_t len, int32_t charges, uint32_t begin, uint32_t end,
                                              int32_t top_n, int32_t fastdiv, void *stream, float *out_score,
                                              uint64_t *out_key, uint32_t *out_pep) {
    if (!ions || !r_sorted || !tc_sorted || !tn_sorted || !idx_sorted || !mass_table26 || !row || !out_score ||
        !out_key || !out_pep)
        return HFX_ERR_ARG;
    if (top_n < 1 || top_n > kNaMaxK) return HFX_ERR_ARG;              // scratch holds 32 per block
    if (len < 1 || len > kMaxWords * 32) return HFX_ERR_ARG;           // rows of at most 8192 bins
    if (charges < 0 || charges > 4) return HFX_ERR_ARG;
    if (end < begin || end > num_pep) return HFX_ERR_ARG;
    // an error left pending by the caller's own work is not taken for this
    // call's: it stays pending and nothing is launched
    if (cudaPeekAtLastError() != cudaSuccess) return HFX_ERR_CUDA;
    uint8_t *scratch = nullptr;
    int smem_limit = 0;
    int32_t rc = setup_device(&scratch, &smem_limit);
    if (rc != HFX_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    DevDB db;
    db.ions = ions;
    db.r_sorted = r_sorted;
    db.tc_sorted = tc_sorted;
    db.tn_sorted = tn_sorted;
    db.idx_sorted = idx_sorted;
    db.num_pep = num_pep;
    for (int i = 0; i < 32; ++i) db.mt[i] = i < 26 ? mass_table26[i] : 0.0f;
    const uint32_t ncand = end - begin;
    const int32_t nblocks = ncand == 0 ? 1 : (int32_t)min((ncand + 31u) / 32u, (uint32_t)kNaMaxBlocks);
    const int32_t words = (len + 31) / 32;
    const size_t smem = smem_bytes(len, top_n);
    if (smem > (size_t)smem_limit) return HFX_ERR_UNSUPPORTED;  // a device with less shared memory
    if (fastdiv)
        k_score_spectrum_na<true><<<nblocks, kNaWarps * 32, smem, st>>>(db, row, len, charges, begin, end, words,
                                                                       top_n, scratch);
    else
        k_score_spectrum_na<false><<<nblocks, kNaWarps * 32, smem, st>>>(db, row, len, charges, begin, end, words,
                                                                        top_n, scratch);
    if (cudaGetLastError() != cudaSuccess) return HFX_ERR_CUDA;
    k_merge_na<<<1, 32, 0, st>>>(scratch, nblocks, top_n, idx_sorted, out_score, out_key, out_pep);
    if (cudaGetLastError() != cudaSuccess) return HFX_ERR_CUDA;
    return HFX_OK;
}
