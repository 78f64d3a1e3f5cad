// C++ host side of libhfx_gpu.so: context, database build and upload,
// orchestration of the search kernels and the C ABI (include/hfx_gpu.h).
//
// Mirrors the reference's Haskell host for the search path:
//   makeSeqDB / withDeviceDB      Sequence/Fragment.hs:197-258
//   makeModInfo                   Sequence/Fragment.hs:260-289
//   searchForMatches              Sequence/Search.hs:98-277
// with the per-spectrum Haskell loops replaced by device kernels.
#include "hfx_internal.h"
#include "search_kernels.h"
#include "batched.h"
#include "lists.h"
#include "mods.h"
#include "evalues.h"
#include "ions.h"
#include "iso_lists.h"

int hfx_digest_launch(const uint8_t *d_seq, const uint32_t *d_seg, int32_t nprot, uint32_t nres, const float *mt26,
                      int32_t rule_mask, int32_t missed, float min_mass, float max_mass, int32_t proline,
                      int32_t min_len, int32_t max_len, float *pm, uint32_t *ptn, uint32_t *plen, uint32_t *pnext,
                      int32_t *cnt, int32_t *incl, int32_t *partial, float *r, uint32_t *tc, uint32_t *tn,
                      int64_t cap, int pass, cudaStream_t st);
#include "../../include/hfx_gpu.h"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

using namespace hfx;

namespace {

// Residue masses, Mass.hs:37-69 (mono) and :76-103 (average), by c - 'A'.
const float kMonoMass[26] = {
    71.037114f,  114.53494f, 103.009185f, 115.026943f, 129.042593f, 147.068414f, 57.021464f,
    137.058912f, 113.084064f, 113.16472f, 128.094963f, 113.084064f, 131.040485f, 114.042927f,
    114.07931f,  97.052764f, 128.058578f, 156.101111f, 87.032028f,  101.047679f, 150.04344f,
    99.068414f,  186.079313f, 113.08406f, 163.06332f, 128.55059f};
const float kAvgMass[26] = {
    71.0788f,  114.5962f, 103.1388f, 115.0886f, 129.1155f, 147.1766f, 57.0519f,  137.1411f, 113.1594f,
    113.240178f, 128.1741f, 113.1594f, 131.1926f, 114.1038f, 114.1472f, 97.1167f, 128.1307f, 156.1875f,
    87.0782f,  101.1051f, 150.0388f, 99.1326f,  186.2132f, 113.1594f, 163.1760f, 128.6231f};
const float kHostH2O = 18.010565f;  // Mass.hs:20
const float kHostH = 1.007276f;     // Mass.hs:25

bool cleaves_after(int rule, uint8_t c) {  // Config.hs:415-431
    static const char *const sets[14] = {"",  "KR", "FWY", "R", "M", "W", "P",
                                         "E", "K",  "R",   "D", "FWYL", "ALIV", "ALIVKRWFY"};
    if (rule < 0 || rule > 13) return false;
    return c != 0 && std::strchr(sets[rule], (int)c) != nullptr;
}

// Grow-only device buffer.
struct DBuf {
    void *p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        size_t want = bytes < 256 ? 256 : bytes;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) n = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
};

}  // namespace

namespace {
const char *const kStageNames[HFX_NSTAGES] = {"layout", "preprocess", "windows", "score", "topn",
                                              "rescore", "mods", "lists", "pack", "mod_lists"};
}  // namespace

struct hfx_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    // database (residual-mass order on the device)
    uint64_t num_ions = 0, num_pep = 0;
    uint64_t ladder_residues = 0;  // sum over fragments of (tn - tc)
    uint64_t list_units = 0;       // sum over fragments of 10 (tn - tc) rounded up to 8 entries
    uint32_t max_ladder = 0;       // max over fragments of (tn - tc)
    DBuf d_lstart;                 // per mass-order position: 10 * prefix sum of (tn - tc)
    unsigned long long counters[8] = {0};
    unsigned long long mod_counters[8] = {0};  // the modification path's (hfx_mod_counters)
    float mt[26] = {0};
    std::vector<uint8_t> h_ascii;
    std::vector<uint32_t> h_seg;   // protein residue starts (+ end); one segment if unknown
    std::vector<float> h_r;        // fragment order
    std::vector<uint32_t> h_tc, h_tn;
    std::vector<uint32_t> h_idx;   // mass order -> fragment
    DBuf d_ions, d_r, d_tc, d_tn, d_idx;
    // variable modifications
    int32_t num_ma = 0, max_ma = 0, per_type = 0, num_mod = 0;
    uint8_t ma[8] = {0};
    float ma_mass[8] = {0};
    std::vector<int32_t> mod_counts;
    std::vector<float> mod_delta;
    DBuf d_mod_counts, d_mod_delta;
    // workspace
    std::map<std::string, DBuf> ws;
    DBuf d_err;
    // stage timing (CUDA events on the context stream) and launch counts
    bool profile = false;
    cudaEvent_t ev[HFX_NSTAGES][2] = {};
    bool ev_pending[HFX_NSTAGES] = {};
    double stage_ms[HFX_NSTAGES] = {0};
    int64_t stage_launches[HFX_NSTAGES] = {0};
    int64_t stage_units[HFX_NSTAGES] = {0};

    // NVTX ranges, one per stage, for timeline tools (no-ops without one)
    int nvtx_depth = 0;
    void stage_begin(int s) {
        nvtxRangePushA(kStageNames[s]);
        ++nvtx_depth;
        if (!profile || gmode == 2) return;
        if (!ev[s][0]) { cudaEventCreate(&ev[s][0]); cudaEventCreate(&ev[s][1]); }
        cudaEventRecord(ev[s][0], stream);
    }
    // CUDA-graph replay (params.use_graph): 0 eager, 1 eager with buffers
    // sized to the capacities, 2 capturing (no host synchronisation; sizes
    // from the capacities; device-side overflow checks)
    int gmode = 0;
    int64_t cap_stride = 0;
    int32_t last_G = 0;  // spectra per group of the last batched search (after every adjustment)
    uint32_t cap_groups = 0, cap_items = 0, cap_mitems = 0;
    uint64_t cap_iso = 0, cap_iso_entries = 0, last_iso = 0, last_iso_entries = 0;  // isoform lists
    int64_t last_stride = 0;
    // the preprocessed rows ("rows32", "meta") of the last search: their stride and spectrum count
    int64_t rows_stride = 0;
    int32_t rows_nspec = 0;
    uint32_t last_items = 0, last_mitems = 0;
    bool graph_valid = false;
    cudaGraphExec_t graph_exec = nullptr;
    cudaStream_t graph_stream = nullptr;  // captures and replays run here (never the legacy stream)
    cudaEvent_t graph_event = nullptr;
    std::vector<uint8_t> graph_key;
    void graph_reset() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        graph_exec = nullptr;
        graph_valid = false;
        graph_key.clear();
    }

    // HFX_DEBUG_SYNC=1: synchronize after every stage and remember the first
    // stage whose kernels reported an error (for locating device faults)
    // hfx_search_evalues without modifications: the FP32 list search also
    // writes every pair's score into the E-value sink (one scoring pass)
    bool ev_single = false;
    float *ev_sink = nullptr;

    bool debug_sync = false;
    std::string fault_stage;
    std::string err_stage;  // with debug_sync: the first stage after which the device error word was set
    void nvtx_close() {
        for (; nvtx_depth > 0; --nvtx_depth) nvtxRangePop();
    }
    void stage_end(int s, int64_t launches, int64_t units = 0) {
        if (nvtx_depth > 0) {
            nvtxRangePop();
            --nvtx_depth;
        }
        if (gmode == 2) return;
        stage_launches[s] += launches;
        stage_units[s] += units;
        if (debug_sync && fault_stage.empty()) {
            const cudaError_t e = cudaStreamSynchronize(stream);
            if (e != cudaSuccess) fault_stage = kStageNames[s];
            uint32_t w = 0;
            if (e == cudaSuccess && err_stage.empty() && d_err.p &&
                cudaMemcpy(&w, d_err.p, 4, cudaMemcpyDeviceToHost) == cudaSuccess && w)
                err_stage = std::string(kStageNames[s]) + " (word " + std::to_string(w) + ")";
        }
        if (!profile) return;
        cudaEventRecord(ev[s][1], stream);
        ev_pending[s] = true;
    }
    void stage_collect() {
        for (int s = 0; s < HFX_NSTAGES; ++s) {
            if (!ev_pending[s]) continue;
            float ms = 0.0f;
            cudaEventSynchronize(ev[s][1]);
            cudaEventElapsedTime(&ms, ev[s][0], ev[s][1]);
            stage_ms[s] += ms;
            ev_pending[s] = false;
        }
    }

    // Workspace byte cap (hfx_set_workspace_limit; 0 = none): a workspace
    // that would take the context's total beyond it is not allocated and the
    // call reports HFX_ERR_OOM, as when cudaMalloc itself fails.
    size_t ws_limit = 0;
    size_t ws_total() const {
        size_t t = 0;
        for (const auto &kv : ws) t += kv.second.n;
        return t;
    }
    // Frees a workspace (one-time scratch such as the digest's).
    void drop(const char *name) {
        auto it = ws.find(name);
        if (it == ws.end()) return;
        it->second.release();
        ws.erase(it);
    }
    template <typename T> T *buf(const char *name, size_t count, cudaError_t &e) {
        DBuf &b = ws[name];
        const size_t want = count * sizeof(T) + 16;
        if (ws_limit && want > b.n && ws_total() - b.n + std::max<size_t>(want, 256) > ws_limit) {
            e = cudaErrorMemoryAllocation;
            return nullptr;
        }
        e = b.ensure(want);
        return b.as<T>();
    }
    DevDB devdb() const {
        DevDB db;
        db.ions = d_ions.as<uint8_t>();
        db.r_sorted = d_r.as<float>();
        db.tc_sorted = d_tc.as<uint32_t>();
        db.tn_sorted = d_tn.as<uint32_t>();
        db.idx_sorted = d_idx.as<uint32_t>();
        db.num_pep = (uint32_t)num_pep;
        for (int i = 0; i < 32; ++i) db.mt[i] = i < 26 ? mt[i] : 0.0f;
        return db;
    }
    DevMods devmods() const {
        DevMods m;
        m.num_ma = num_ma;
        m.num_mod = num_mod;
        for (int i = 0; i < 8; ++i) m.ma_mass[i] = i < num_ma ? ma_mass[i] : 0.0f;
        m.counts = num_mod > 0 ? d_mod_counts.as<int32_t>() : nullptr;
        m.delta = num_mod > 0 ? d_mod_delta.as<float>() : nullptr;
        m.per_type = per_type;
        return m;
    }
};

namespace {

int32_t fail(hfx_ctx *c, int32_t code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}
int32_t cuda_fail(hfx_ctx *c, cudaError_t e, const char *where) {
    if (e == cudaErrorMemoryAllocation)
        return fail(c, HFX_ERR_OOM, std::string(where) + ": " + cudaGetErrorString(e));
    std::string msg = std::string(where) + ": " + cudaGetErrorString(e);
    if (c && !c->fault_stage.empty()) msg += " (first failing stage: " + c->fault_stage + ")";
    if (c && !c->err_stage.empty()) msg += " (error word first set after stage: " + c->err_stage + ")";
    return fail(c, HFX_ERR_CUDA, msg);
}
#define HFX_CUDA(call, where)                         \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, where); \
    } while (0)

// prepare_ions.cu:29-52 packing: (c - 'A') | (index of c in ma + 1) << 5.
void pack_ions(const std::vector<uint8_t> &ascii, const uint8_t *ma, int num_ma, std::vector<uint8_t> &out) {
    out.resize(ascii.size());
    uint8_t code[256];
    for (int c = 0; c < 256; ++c) {
        uint8_t mod = 0;
        for (int j = 0; j < num_ma; ++j)
            if (ma[j] == c) { mod = (uint8_t)(j + 1); break; }
        code[c] = (uint8_t)((uint8_t)(c - 'A') | (uint8_t)(mod << 5));
    }
    for (size_t i = 0; i < ascii.size(); ++i) out[i] = code[ascii[i]];
}

int32_t upload_db(hfx_ctx *ctx) {
    ctx->graph_reset();
    const uint64_t np = ctx->num_pep;
    ctx->h_idx.resize(np);
    std::iota(ctx->h_idx.begin(), ctx->h_idx.end(), 0u);
    // sort.cu:28-35: key-value sort of residual masses with iota (stable)
    std::stable_sort(ctx->h_idx.begin(), ctx->h_idx.end(),
                     [&](uint32_t a, uint32_t b) { return ctx->h_r[a] < ctx->h_r[b]; });
    std::vector<float> rs(np);
    std::vector<uint32_t> tcs(np), tns(np);
    ctx->ladder_residues = 0;
    ctx->list_units = 0;
    ctx->max_ladder = 0;
    // list slots: 10 entries per prefix, rounded up to 8 entries so that every
    // (level, fragment) slot starts on a 16-byte boundary
    std::vector<uint32_t> lstart(np);
    for (uint64_t i = 0; i < np; ++i) {
        rs[i] = ctx->h_r[ctx->h_idx[i]];
        tcs[i] = ctx->h_tc[ctx->h_idx[i]];
        tns[i] = ctx->h_tn[ctx->h_idx[i]];
        if (tns[i] < tcs[i] || tns[i] > ctx->num_ions) return fail(ctx, HFX_ERR_ARG, "fragment outside the residues");
        if (ctx->list_units > 0xFFFFFFFFull)
            return fail(ctx, HFX_ERR_UNSUPPORTED, "ion-list offsets exceed 32 bits");
        lstart[i] = (uint32_t)ctx->list_units;
        ctx->ladder_residues += tns[i] - tcs[i];
        ctx->list_units += (10ull * (tns[i] - tcs[i]) + 7ull) & ~7ull;
        ctx->max_ladder = std::max(ctx->max_ladder, tns[i] - tcs[i]);
    }
    if (ctx->list_units > 0xFFFFFFFFull) return fail(ctx, HFX_ERR_UNSUPPORTED, "ion-list offsets exceed 32 bits");
    std::vector<uint8_t> packed;
    pack_ions(ctx->h_ascii, ctx->ma, ctx->num_ma, packed);
    HFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    HFX_CUDA(ctx->d_ions.ensure(packed.size() + 64), "alloc ions");
    HFX_CUDA(ctx->d_r.ensure(np * 4 + 16), "alloc r");
    HFX_CUDA(ctx->d_tc.ensure(np * 4 + 16), "alloc tc");
    HFX_CUDA(ctx->d_tn.ensure(np * 4 + 16), "alloc tn");
    HFX_CUDA(ctx->d_idx.ensure(np * 4 + 16), "alloc idx");
    HFX_CUDA(cudaMemcpy(ctx->d_ions.p, packed.data(), packed.size(), cudaMemcpyHostToDevice), "H2D ions");
    HFX_CUDA(cudaMemcpy(ctx->d_r.p, rs.data(), np * 4, cudaMemcpyHostToDevice), "H2D r");
    HFX_CUDA(cudaMemcpy(ctx->d_tc.p, tcs.data(), np * 4, cudaMemcpyHostToDevice), "H2D tc");
    HFX_CUDA(cudaMemcpy(ctx->d_tn.p, tns.data(), np * 4, cudaMemcpyHostToDevice), "H2D tn");
    HFX_CUDA(cudaMemcpy(ctx->d_idx.p, ctx->h_idx.data(), np * 4, cudaMemcpyHostToDevice), "H2D idx");
    // one entry past the last position: the end of its slot (slot sizes by difference)
    lstart.push_back((uint32_t)ctx->list_units);
    HFX_CUDA(ctx->d_lstart.ensure(np * 4 + 16), "alloc lstart");
    HFX_CUDA(cudaMemcpy(ctx->d_lstart.p, lstart.data(), (np + 1) * 4, cudaMemcpyHostToDevice), "H2D lstart");
    return HFX_OK;
}

// Fragment.hs:260-289 makeModInfo: count vectors over 0..max_ma with
// dimension 0 most significant, all-zero dropped, sum < max_ma kept.
void make_mod_table(hfx_ctx *ctx) {
    ctx->mod_counts.clear();
    ctx->mod_delta.clear();
    ctx->num_mod = 0;
    const int n = ctx->num_ma;
    if (n <= 0) return;
    std::vector<int32_t> c(n, 0);
    for (;;) {
        int d = n - 1;
        while (d >= 0 && c[d] == ctx->max_ma) c[d--] = 0;
        if (d < 0) break;
        ++c[d];
        int s = 0;
        for (int i = 0; i < n; ++i) s += c[i];
        if (s >= ctx->max_ma) continue;
        float delta = 0.0f;
        for (int i = 0; i < n; ++i) delta = delta + ctx->ma_mass[i] * (float)c[i];
        ctx->mod_counts.insert(ctx->mod_counts.end(), c.begin(), c.end());
        ctx->mod_delta.push_back(delta);
        ++ctx->num_mod;
    }
}

// Longest spectrum row accepted by default (0.02 Da bins over 0-5000 m/z).
constexpr int32_t kDefaultMaxLen = 262144;

struct Batch {
    const float *mz, *it, *pcr, *z, *tol;
    const int64_t *off;
    int32_t nspec;
};

int32_t check_params(hfx_ctx *ctx, const hfx_search_params *p) {
    if (!p) return fail(ctx, HFX_ERR_ARG, "null params");
    if (p->top_n < 1 || p->top_n > kMaxTopK) return fail(ctx, HFX_ERR_ARG, "top_n must be 1..32");
    if (!(p->bin_width > 0.0f)) return fail(ctx, HFX_ERR_ARG, "bin_width must be > 0");
    if (p->precision < 0 || p->precision > 2) return fail(ctx, HFX_ERR_ARG, "precision must be 0, 1 or 2");
    if (ctx->num_pep == 0) return fail(ctx, HFX_ERR_ARG, "no database uploaded");
    return HFX_OK;
}

LayoutParams layout_params(const hfx_search_params *p) {
    LayoutParams lp;
    lp.bw = p->bin_width;
    lp.custom_bw = p->custom_bin_width;
    lp.remove_pcr = p->remove_precursor_peak;
    lp.ppm = p->tol_ppm;
    lp.max_len = p->max_len > 0 ? p->max_len : kDefaultMaxLen;
    lp.cap_len = 0;
    return lp;
}

// Layout + preprocess a batch into the workspace rows.  Returns stride.
int32_t run_stage_a(hfx_ctx *ctx, const hfx_search_params *p, const Batch &b, int64_t &stride,
                    SpecMeta *&meta, float *&rows, __nv_bfloat16 *&rows_bf, __half *&rows_h, bool want_bf,
                    bool want_h) {
    cudaError_t e;
    LayoutParams lp = layout_params(p);
    if (ctx->gmode >= 1) {
        // graph replays keep the row stride of the capture: longer accepted
        // rows are reported (and the batch re-planned)
        lp.cap_len = (int32_t)std::min<int64_t>(lp.max_len, ctx->cap_stride);
    }
    meta = ctx->buf<SpecMeta>("meta", b.nspec, e);
    if (e) return cuda_fail(ctx, e, "alloc meta");
    uint32_t *d_max = ctx->buf<uint32_t>("maxlen", 4, e);
    if (e) return cuda_fail(ctx, e, "alloc maxlen");
    HFX_CUDA(cudaMemsetAsync(d_max, 0, 4, ctx->stream), "memset");
    ctx->stage_begin(HFX_STAGE_LAYOUT);
    int rc = hfx_launch_layout(b.mz, b.off, b.pcr, b.z, b.tol, b.nspec, lp, meta, d_max, ctx->d_err.as<uint32_t>(),
                               ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_layout");
    ctx->stage_end(HFX_STAGE_LAYOUT, 1, b.nspec);
    if (ctx->gmode >= 1) {
        stride = ctx->cap_stride;
    } else {
        uint32_t maxlen = 0;
        HFX_CUDA(cudaMemcpyAsync(&maxlen, d_max, 4, cudaMemcpyDeviceToHost, ctx->stream), "D2H maxlen");
        HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        if (maxlen == 0) maxlen = 16;
        stride = ((int64_t)maxlen + 15) & ~(int64_t)15;
        ctx->last_stride = stride;
    }
    rows = ctx->buf<float>("rows32", (size_t)b.nspec * stride, e);
    if (e) return cuda_fail(ctx, e, "alloc rows");
    ctx->rows_stride = stride;
    ctx->rows_nspec = b.nspec;
    rows_bf = nullptr;
    rows_h = nullptr;
    if (want_bf) {
        rows_bf = ctx->buf<__nv_bfloat16>("rowsbf", (size_t)b.nspec * stride, e);
        if (e) return cuda_fail(ctx, e, "alloc rows bf16");
    }
    if (want_h) {
        rows_h = ctx->buf<__half>("rowsh", (size_t)b.nspec * stride, e);
        if (e) return cuda_fail(ctx, e, "alloc rows fp16");
    }
    ctx->stage_begin(HFX_STAGE_PREPROCESS);
    rc = hfx_launch_preprocess(b.mz, b.it, b.off, b.pcr, lp, meta, b.nspec, stride, rows, rows_bf, rows_h,
                               ctx->d_err.as<uint32_t>(), ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_preprocess");
    ctx->stage_end(HFX_STAGE_PREPROCESS, 1, b.nspec);
    return HFX_OK;
}

int32_t search_plain_per_spectrum(hfx_ctx *ctx, const hfx_search_params *p, const Batch &b, const SpecMeta *meta,
                                  const float *rows, int64_t stride, float *out_s, uint64_t *out_k,
                                  uint32_t *out_pep, int64_t *out_ncand) {
    cudaError_t e;
    uint32_t *wb = ctx->buf<uint32_t>("wb", b.nspec, e);
    if (e) return cuda_fail(ctx, e, "alloc wb");
    uint32_t *we = ctx->buf<uint32_t>("we", b.nspec, e);
    if (e) return cuda_fail(ctx, e, "alloc we");
    ctx->stage_begin(HFX_STAGE_WINDOWS);
    int rc = hfx_launch_windows(ctx->d_r.as<float>(), (uint32_t)ctx->num_pep, meta, b.nspec, wb, we, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_windows");
    ctx->stage_end(HFX_STAGE_WINDOWS, 1, b.nspec);
    // Search.hs:184-185 peeks the counts to the host; so does the plain path.
    std::vector<uint32_t> hb(b.nspec), he(b.nspec);
    std::vector<SpecMeta> hm(b.nspec);
    HFX_CUDA(cudaMemcpyAsync(hb.data(), wb, 4ull * b.nspec, cudaMemcpyDeviceToHost, ctx->stream), "D2H wb");
    HFX_CUDA(cudaMemcpyAsync(he.data(), we, 4ull * b.nspec, cudaMemcpyDeviceToHost, ctx->stream), "D2H we");
    HFX_CUDA(cudaMemcpyAsync(hm.data(), meta, sizeof(SpecMeta) * b.nspec, cudaMemcpyDeviceToHost, ctx->stream),
             "D2H meta");
    HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    const int32_t K = std::max(p->top_n, std::min(p->rescore_k > 0 ? p->rescore_k : p->top_n, kMaxTopK));
    std::vector<int64_t> part_off(b.nspec + 1, 0);
    std::vector<int32_t> nblk(b.nspec, 0);
    for (int32_t s = 0; s < b.nspec; ++s) {
        const uint32_t nc = he[s] - hb[s];
        int32_t nb = 0;
        if (nc > 0 && hm[s].status == 0) nb = (int32_t)std::min<uint32_t>((nc + 31) / 32, 304u);
        nblk[s] = nb;
        part_off[s + 1] = part_off[s] + nb;
    }
    float *ps = ctx->buf<float>("part_s", (size_t)part_off[b.nspec] * K + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc parts");
    uint64_t *pk = ctx->buf<uint64_t>("part_k", (size_t)part_off[b.nspec] * K + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc parts");
    int64_t *d_off = ctx->buf<int64_t>("part_off", b.nspec + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc part_off");
    HFX_CUDA(cudaMemcpyAsync(d_off, part_off.data(), 8ull * (b.nspec + 1), cudaMemcpyHostToDevice, ctx->stream),
             "H2D part_off");
    const DevDB db = ctx->devdb();
    int64_t nl = 0, psm = 0;
    ctx->stage_begin(HFX_STAGE_SCORE);
    for (int32_t s = 0; s < b.nspec; ++s) {
        if (nblk[s] == 0) continue;
        ++nl;
        psm += he[s] - hb[s];
        const int32_t ch = hm[s].charges_plain;
        rc = hfx_launch_score_spectrum(db, rows + (size_t)s * stride, hm[s].len, ch, hb[s], he[s], K, nblk[s],
                                       p->fastdiv, ps + part_off[s] * K, pk + part_off[s] * K,
                                       ctx->d_err.as<uint32_t>(), ctx->stream);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_score_spectrum");
    }
    ctx->stage_end(HFX_STAGE_SCORE, nl, psm);
    ctx->stage_begin(HFX_STAGE_TOPN);
    rc = hfx_launch_merge_parts(ps, pk, d_off, b.nspec, K, p->top_n, ctx->d_idx.as<uint32_t>(), out_s, out_k,
                                out_pep, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_merge_parts");
    ctx->stage_end(HFX_STAGE_TOPN, 1, b.nspec);
    if (out_ncand) {
        std::vector<int64_t> nc(b.nspec);
        for (int32_t s = 0; s < b.nspec; ++s) nc[s] = (hm[s].status == 0) ? (int64_t)(he[s] - hb[s]) : 0;
        HFX_CUDA(cudaMemcpyAsync(out_ncand, nc.data(), 8ull * b.nspec, cudaMemcpyHostToDevice, ctx->stream),
                 "H2D ncand");
        HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    }
    return HFX_OK;
}

// The modification search over isoform lists (iso_lists.cu): coverage and
// isoform counts, one record per isoform, their ion lists, the scorer.  The
// totals come back to the host in eager searches; graph replays use the
// capacities of their capture and report a batch that outgrows them.
int32_t search_isoform_lists(hfx_ctx *ctx, const hfx_search_params *p, const SpecMeta *meta, int32_t ns,
                             const uint32_t *mb, const uint32_t *me, const BatchedWs &ws, const uint32_t *mlo,
                             const uint32_t *mhi, const uint32_t *mch, const uint32_t *mitem_off, int32_t n_gm,
                             int elem_kind, const void *tiles, int64_t stride, int32_t G, int32_t K, float *ms,
                             uint64_t *mk, unsigned long long *ncm) {
    cudaError_t e;
    unsigned long long *stats = nullptr;
    if (ctx->profile) {
        stats = ctx->buf<unsigned long long>("i_stats", 8, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        HFX_CUDA(cudaMemsetAsync(stats, 0, 64, ctx->stream), "memset");
    }
    const DevDB db = ctx->devdb();
    const DevMods dm = ctx->devmods();
    const int64_t npep1 = (int64_t)ctx->num_pep + 1;
    const int64_t ncover = (int64_t)ctx->num_mod * kLevels * npep1;
    const int64_t n = (int64_t)ctx->num_mod * (int64_t)ctx->num_pep;
    int32_t *cover = ctx->buf<int32_t>("i_cover", (size_t)ncover, e);
    int32_t *cpart = e ? nullptr : ctx->buf<int32_t>("i_cpart", hfx_scan_partials_needed(ncover), e);
    int32_t *count = e ? nullptr : ctx->buf<int32_t>("i_count", (size_t)n + 1, e);
    int32_t *incl = e ? nullptr : ctx->buf<int32_t>("i_incl", (size_t)n + 1, e);
    int32_t *npart = e ? nullptr : ctx->buf<int32_t>("i_npart", hfx_scan_partials_needed(n + 1), e);
    unsigned long long *units = e ? nullptr : ctx->buf<unsigned long long>("i_units", (size_t)n, e);
    unsigned long long *iunits = e ? nullptr : ctx->buf<unsigned long long>("i_iunits", (size_t)n, e);
    unsigned long long *upart =
        e ? nullptr : ctx->buf<unsigned long long>("i_upart", hfx_iso_scan64_partials_needed(n), e);
    if (e) return cuda_fail(ctx, e, "alloc isoform plan");
    int rc = hfx_iso_plan(db, dm, meta, ns, mb, me, ctx->d_lstart.as<uint32_t>(), cover, cpart, count, incl, npart,
                          units, iunits, upart, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "isoform plan");
    uint64_t cap_iso = 0, cap_entries = 0;
    if (ctx->gmode >= 1) {
        cap_iso = ctx->cap_iso;
        cap_entries = ctx->cap_iso_entries;
    } else {
        int32_t total = 0;
        unsigned long long entries = 0;
        HFX_CUDA(cudaMemcpyAsync(&total, incl + n, 4, cudaMemcpyDeviceToHost, ctx->stream), "D2H isoforms");
        if (n > 0)
            HFX_CUDA(cudaMemcpyAsync(&entries, iunits + n - 1, 8, cudaMemcpyDeviceToHost, ctx->stream), "D2H entries");
        HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        if (total < 0) return fail(ctx, HFX_ERR_UNSUPPORTED, "more than 2^31 modified isoforms in one batch");
        cap_iso = (uint64_t)total;
        cap_entries = entries;
        ctx->last_iso = cap_iso;
        ctx->last_iso_entries = cap_entries;
    }
    if (cap_iso > 0xFFFFFFF0ull) return fail(ctx, HFX_ERR_UNSUPPORTED, "more than 2^32 modified isoforms");
    uint64_t *key = ctx->buf<uint64_t>("i_key", cap_iso + 1, e);
    uint64_t *off = e ? nullptr : ctx->buf<uint64_t>("i_off", cap_iso + 1, e);
    uint16_t *len = e ? nullptr : ctx->buf<uint16_t>("i_len", (cap_iso + 1) * kLevels, e);
    uint16_t *lists = e ? nullptr : ctx->buf<uint16_t>("i_lists", cap_entries + 64, e);
    const int32_t pos_words = (int32_t)((ctx->max_ladder + 31) / 32 + 1);
    uint32_t *pos = e ? nullptr : ctx->buf<uint32_t>("i_pos", (cap_iso + 1) * (size_t)pos_words, e);
    if (e) return cuda_fail(ctx, e, "alloc isoform lists");
    rc = hfx_iso_expand(db, dm, cover, ctx->d_lstart.as<uint32_t>(), count, incl, units, iunits, (uint32_t)cap_iso,
                        cap_entries, key, off, ctx->d_err.as<uint32_t>(), ctx->stream);
    if (!rc)
        rc = hfx_iso_generate(db, dm, cover, (int32_t)std::min<int64_t>(stride, kMaxWords * 32),
                              ctx->d_lstart.as<uint32_t>(), incl + n, (uint32_t)cap_iso, key, off, lists, cap_entries,
                              len, (int32_t)std::min<uint64_t>(40ull * ctx->max_ladder, kMaxListLen), pos_words,
                              pos, p->fastdiv, stats, ctx->d_err.as<uint32_t>(), ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "isoform lists");
    ctx->stage_end(HFX_STAGE_MOD_LISTS, 17, (int64_t)cap_iso);  // windows, planning, 12 isoform-list kernels
    ctx->stage_begin(HFX_STAGE_MODS);
    rc = hfx_iso_score(lists, cap_entries, ctx->d_lstart.as<uint32_t>(), key, off, len, count, incl,
                       (uint32_t)ctx->num_pep, (uint32_t)cap_iso, elem_kind, tiles, stride, mb, me, ctx->num_mod, ws,
                       mlo, mhi, mch, mitem_off, n_gm, G, K, ms, mk, ncm, stats, ctx->d_err.as<uint32_t>(),
                       ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_score_iso_lists");
    if (stats) {
        unsigned long long h[8];
        HFX_CUDA(cudaMemcpyAsync(h, stats, 64, cudaMemcpyDeviceToHost, ctx->stream), "D2H stats");
        HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        for (int i = 0; i < 8; ++i) ctx->mod_counters[i] += h[i];
    }
    return HFX_OK;
}

int32_t search_batched(hfx_ctx *ctx, const hfx_search_params *p, const Batch &b, const SpecMeta *meta,
                       const float *rows, const void *rows_lo, int elem_kind, int64_t stride, float *out_s,
                       uint64_t *out_k, uint32_t *out_pep, int64_t *out_ncand) {
    cudaError_t e;
    const int32_t ns = b.nspec;
    // one 16-byte tile load per bin: 8 BF16/FP16 or 4 FP32 spectra per group
    int32_t G = p->group_size > 0 ? p->group_size : (elem_kind == 0 ? 4 : 8);
    const int32_t chunk = p->chunk > 0 ? p->chunk : 4096;
    if (G != 1 && G != 2 && G != 4 && G != 8 && G != 16)
        return fail(ctx, HFX_ERR_ARG, "group_size must be 1, 2, 4, 8 or 16");
    // rows longer than the shared-memory bit planes: 32-bit sorted lists,
    // tiles read from global memory, list-based rescoring; no fused or
    // modification scoring
    const bool long_rows = stride > (int64_t)kMaxWords * 32;
    // candidates kept for FP32 rescoring: up to 64 when unmodified candidates
    // alone are list-scored in groups of up to 8, else up to 32
    const bool lists_only = (p->batch_mode == 1 || long_rows) && !(p->search_mods != 0 && ctx->num_mod > 0);
    const int32_t K = elem_kind == 0 ? p->top_n
                                     : std::max(p->top_n, std::min(p->rescore_k > 0 ? p->rescore_k : 32,
                                                                   lists_only ? kMaxKept : kMaxTopK));
    if (K > 32 && G == 16) G = 8;
    if (G == 16) {
        // two 16-byte loads per bin: list scoring of BF16/FP16 rows only
        if (elem_kind == 0 || (p->batch_mode != 1 && !long_rows) || (p->search_mods != 0 && ctx->num_mod > 0))
            return fail(ctx, HFX_ERR_UNSUPPORTED,
                        "group_size 16 needs BF16/FP16 rows, list scoring and no modification search");
        // a 16-spectrum tile of the longest row must fit in shared memory
        if (!hfx_lists_group_fits(16, long_rows ? 1 : 0, stride, 2)) G = 8;
    }
    if (long_rows && p->search_mods && ctx->num_mod > 0)
        return fail(ctx, HFX_ERR_UNSUPPORTED, "modification search on rows longer than 8192 bins");
    ctx->last_G = G;
    if (p->ion_bins_custom && !long_rows)
        return fail(ctx, HFX_ERR_UNSUPPORTED, "custom ion bin width needs rows longer than 8192 bins");
    uint32_t *wb = ctx->buf<uint32_t>("wb", ns, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    uint32_t *we = ctx->buf<uint32_t>("we", ns, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    BatchedWs ws;
    ws.hist = ctx->buf<uint32_t>("b_hist", kBucketCount + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    ws.cursor = ctx->buf<uint32_t>("b_cursor", kBucketCount, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    uint32_t *scal = ctx->buf<uint32_t>("b_scal", 8, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    ws.n_sorted = scal;
    ws.ngroups = scal + 1;
    ws.total_items = scal + 2;
    ws.counter = scal + 3;
    ws.perm = ctx->buf<int32_t>("b_perm", ns, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    ws.groups = ctx->buf<GroupInfo>("b_groups", ns, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    ws.item_off = ctx->buf<uint32_t>("b_itemoff", ns + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    ws.group_of = ctx->buf<int32_t>("b_groupof", ns, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    ws.slot_of = ctx->buf<int32_t>("b_slotof", ns, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    ctx->stage_begin(HFX_STAGE_WINDOWS);
    int rc = hfx_launch_windows(ctx->d_r.as<float>(), (uint32_t)ctx->num_pep, meta, ns, wb, we, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_windows");
    rc = hfx_batched_plan(meta, ns, wb, we, G, chunk, ws, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "plan");
    ctx->stage_end(HFX_STAGE_WINDOWS, 6, ns);  // k_windows + 5 planning kernels
    uint32_t ngroups = 0, total_items = 0;
    if (ctx->gmode >= 1) {
        // capacities of the graph; a batch that needs more is reported (k_clamp_items)
        ngroups = ctx->cap_groups;
        total_items = ctx->cap_items;
        // a batch with more groups than the tiles were sized for is cut to
        // the capacity and reported (the replay is then planned again)
        rc = hfx_clamp_groups(ws.ngroups, ngroups, ctx->d_err.as<uint32_t>(), ctx->stream);
        if (!rc)
            rc = hfx_clamp_items(ws.item_off, (int64_t)ns + 1, total_items, ctx->d_err.as<uint32_t>(), ctx->stream);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_clamp_items");
    } else {
        uint32_t hs[4];
        HFX_CUDA(cudaMemcpyAsync(hs, scal, 16, cudaMemcpyDeviceToHost, ctx->stream), "D2H plan");
        HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        ngroups = hs[1];
        total_items = hs[2];
        ctx->last_items = total_items;
    }
    const size_t esz = elem_kind == 0 ? 4 : 2;
    void *tiles = ctx->buf<uint8_t>("tiles", (size_t)ngroups * stride * G * esz + 64, e);
    if (e) return cuda_fail(ctx, e, "alloc tiles");
    float *ps = ctx->buf<float>("part_s", (size_t)total_items * G * K + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc parts");
    uint64_t *pk = ctx->buf<uint64_t>("part_k", (size_t)total_items * G * K + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc parts");
    const DevDB db = ctx->devdb();
    const void *src_rows = elem_kind == 0 ? (const void *)rows : rows_lo;
    const bool plain_on = p->search_plain != 0;
    const void *lists_out = nullptr;  // the step's lists, which the FP32 rescoring reads
    const uint16_t *llen_out = nullptr;
    uint64_t total10_out = 0;
    const int32_t list_cap = (int32_t)std::min<uint64_t>(40ull * ctx->max_ladder, kMaxListLen);
    const bool mods_on = p->search_mods != 0 && ctx->num_mod > 0;
    ctx->stage_begin(HFX_STAGE_PACK);
    rc = hfx_pack_tiles(src_rows, elem_kind, stride, meta, ws, tiles, ngroups, G, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_pack_tiles");
    ctx->stage_end(HFX_STAGE_PACK, ngroups > 0 ? 1 : 0, ngroups);
    if (!plain_on) {
    } else if (p->batch_mode != 1 && !long_rows) {
        // fused: every work item rebuilds its candidates' ion lists
        ctx->stage_begin(HFX_STAGE_SCORE);
        rc = hfx_batched_score(db, src_rows, elem_kind, stride, meta, wb, we, ws, tiles, ngroups, G, chunk, K, 0, 0,
                               p->fastdiv, ps, pk, ctx->d_err.as<uint32_t>(), ctx->stream);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_score_batched");
        ctx->stage_end(HFX_STAGE_SCORE, 1, 0);
    } else {
        // lists: one ion list per needed (peptide, charge level), then scoring
        const int64_t npep1 = (int64_t)ctx->num_pep + 1;
        int32_t *diff = ctx->buf<int32_t>("l_diff", (size_t)kLevels * npep1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        int32_t *cover = ctx->buf<int32_t>("l_cover", (size_t)kLevels * npep1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        int32_t *partial = ctx->buf<int32_t>("l_partial", hfx_scan_partials_needed(kLevels * npep1), e);
        if (e) return cuda_fail(ctx, e, "alloc");
        uint16_t *llen = ctx->buf<uint16_t>("l_len", (size_t)kLevels * ctx->num_pep, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        // static slots: 10 ions per prefix and charge (rounded up to 8
        // entries per fragment), levels 1..4 (1+2+3+4)
        const uint64_t total10 = ctx->list_units;
        void *lists = long_rows ? (void *)ctx->buf<uint32_t>("l_lists32", total10 * 10 + 64, e)
                                : (void *)ctx->buf<uint16_t>("l_lists", total10 * 10 + 64, e);
        if (e) return cuda_fail(ctx, e, "alloc lists");
        lists_out = lists;
        llen_out = llen;
        total10_out = total10;
        unsigned long long *stats = nullptr;
        if (ctx->profile) {
            stats = ctx->buf<unsigned long long>("l_stats", 8, e);
            if (e) return cuda_fail(ctx, e, "alloc");
            HFX_CUDA(cudaMemsetAsync(stats, 0, 64, ctx->stream), "memset");
        }
        ctx->stage_begin(HFX_STAGE_LISTS);
        rc = hfx_lists_mark(meta, wb, we, ns, npep1, diff, ctx->stream);
        if (!rc) rc = hfx_scan_inclusive(diff, kLevels * npep1, cover, partial, ctx->stream);
        if (!rc && long_rows)
            rc = hfx_lists_generate_long(db, cover, npep1, (int32_t)stride, ctx->d_lstart.as<uint32_t>(), total10,
                                         (uint32_t *)lists, llen, p->fastdiv,
                                         p->ion_bins_custom ? p->bin_width : 0.0f, stats,
                                         ctx->d_err.as<uint32_t>(), ctx->stream);
        else if (!rc)
            rc = hfx_lists_generate(db, cover, npep1, (int32_t)std::min<int64_t>(stride, kMaxWords * 32),
                                    ctx->d_lstart.as<uint32_t>(), total10, (uint16_t *)lists, llen, list_cap,
                                    p->fastdiv, stats, ctx->d_err.as<uint32_t>(), ctx->stream);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "ion lists");
        ctx->stage_end(HFX_STAGE_LISTS, 5, 0);
        ctx->stage_begin(HFX_STAGE_SCORE);
        float *sink = nullptr;
        const uint64_t *sink_off = nullptr;
        if (ctx->ev_single && elem_kind == 0 && ctx->gmode == 0) {
            // E-values in the same pass: each spectrum's window of scores
            // at its offset in the sink (Search.hs:116-121)
            uint64_t *size = ctx->buf<uint64_t>("e_size", ns, e);
            uint64_t *soff = e ? nullptr : ctx->buf<uint64_t>("e_off", ns, e);
            uint64_t *send = e ? nullptr : ctx->buf<uint64_t>("e_end", ns, e);
            unsigned long long *cur = e ? nullptr : ctx->buf<unsigned long long>("e_cursor", ns, e);
            if (e) return cuda_fail(ctx, e, "alloc");
            rc = hfx_evalue_offsets(wb, we, 1, nullptr, ns, size, soff, send, cur, ctx->stream);
            if (rc) return cuda_fail(ctx, (cudaError_t)rc, "E-value offsets");
            uint64_t total = 0;
            HFX_CUDA(cudaMemcpyAsync(&total, send + ns - 1, 8, cudaMemcpyDeviceToHost, ctx->stream), "D2H total");
            HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
            sink = ctx->buf<float>("e_sink", total + 1, e);
            if (e) return cuda_fail(ctx, e, "alloc E-value scores");
            sink_off = soff;
            ctx->ev_sink = sink;
        }
        rc = hfx_lists_score(lists, long_rows, ctx->d_lstart.as<uint32_t>(), total10, llen, (uint32_t)ctx->num_pep,
                             elem_kind, stride, wb, we, ws, tiles, G, K, 0, ps, pk, stats,
                             ctx->d_err.as<uint32_t>(), ctx->stream, sink, sink_off);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_score_lists");
        ctx->stage_end(HFX_STAGE_SCORE, 1, 0);
        if (stats) {
            unsigned long long h[8];
            HFX_CUDA(cudaMemcpyAsync(h, stats, 64, cudaMemcpyDeviceToHost, ctx->stream), "D2H stats");
            HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
            for (int i = 0; i < 8; ++i) ctx->counters[i] += h[i];
        }
    }
    // modified isoforms: fused enumeration + scoring over the same group tiles
    const DevMods dm = ctx->devmods();
    float *ms = nullptr;
    uint64_t *mk = nullptr;
    uint32_t *mitem_off = nullptr;
    unsigned long long *ncm = nullptr;
    if (mods_on) {
        const int32_t nm = ctx->num_mod;
        const int32_t n_gm = (int32_t)ngroups * nm;
        uint32_t *mb = ctx->buf<uint32_t>("m_wb", (size_t)ns * nm, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        uint32_t *me = ctx->buf<uint32_t>("m_we", (size_t)ns * nm, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        uint32_t *mlo = ctx->buf<uint32_t>("m_lo", (size_t)n_gm + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        uint32_t *mhi = ctx->buf<uint32_t>("m_hi", (size_t)n_gm + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        uint32_t *mch = ctx->buf<uint32_t>("m_chunk", (size_t)n_gm + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        int32_t *nch = ctx->buf<int32_t>("m_nchunks", (size_t)n_gm + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        mitem_off = ctx->buf<uint32_t>("m_itemoff", (size_t)n_gm + 2, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        int32_t *partial = ctx->buf<int32_t>("m_partial", hfx_scan_partials_needed(n_gm + 1) + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        ncm = ctx->buf<unsigned long long>("m_ncand", (size_t)ns, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        HFX_CUDA(cudaMemsetAsync(ncm, 0, 8ull * ns, ctx->stream), "memset");
        // "mod_lists": windows, planning and (batch_mode 1) the isoform
        // lists; "mods": the scorer
        ctx->stage_begin(HFX_STAGE_MOD_LISTS);
        rc = hfx_mods_windows(ctx->d_r.as<float>(), (uint32_t)ctx->num_pep, meta, ns, dm, mb, me, ctx->stream);
        if (!rc) rc = hfx_mods_plan(ws, ngroups, mb, me, nm, chunk, mlo, mhi, mch, nch, mitem_off, partial,
                                    ctx->stream);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "modification plan");
        uint32_t mtotal = 0;
        if (ctx->gmode >= 1) {
            mtotal = ctx->cap_mitems;
            if (n_gm > 0) {
                rc = hfx_clamp_items(mitem_off, (int64_t)n_gm + 1, mtotal, ctx->d_err.as<uint32_t>(), ctx->stream);
                if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_clamp_items");
            }
        } else if (n_gm > 0) {
            HFX_CUDA(cudaMemcpyAsync(&mtotal, mitem_off + n_gm, 4, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
            HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
            ctx->last_mitems = mtotal;
        }
        ms = ctx->buf<float>("m_part_s", (size_t)mtotal * G * K + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc mod parts");
        mk = ctx->buf<uint64_t>("m_part_k", (size_t)mtotal * G * K + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc mod parts");
        if (mtotal > 0 && p->batch_mode == 1) {
            // isoform lists: every needed isoform's ion lists built once for
            // the batch, then streamed by the scorer (which ends the
            // mod_lists stage and begins the mods stage)
            rc = search_isoform_lists(ctx, p, meta, ns, mb, me, ws, mlo, mhi, mch, mitem_off, n_gm, elem_kind, tiles,
                                      stride, G, K, ms, mk, ncm);
            if (rc) return rc;
            ctx->stage_end(HFX_STAGE_MODS, 1, mtotal);
        } else {
            ctx->stage_end(HFX_STAGE_MOD_LISTS, n_gm > 0 ? 5 : 1, 0);  // k_mod_windows, k_mod_groups, 3 scans
            if (mtotal > 0) {
                // fused: every work item enumerates and builds its isoforms
                ctx->stage_begin(HFX_STAGE_MODS);
                rc = hfx_mods_score(db, dm, tiles, elem_kind, stride, mb, me, ws, mlo, mhi, mch, mitem_off, n_gm, G,
                                    K, p->fastdiv, ms, mk, ncm, ctx->d_err.as<uint32_t>(), ctx->stream);
                if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_score_mods");
                ctx->stage_end(HFX_STAGE_MODS, 1, mtotal);
            }
        }
    }
    float *ks = ctx->buf<float>("kept_s", (size_t)ns * K, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    uint64_t *kk = ctx->buf<uint64_t>("kept_k", (size_t)ns * K, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    ctx->stage_begin(HFX_STAGE_TOPN);
    if (mods_on)
        rc = hfx_merge_with_mods(ps, pk, ws.item_off, ms, mk, mitem_off, ctx->num_mod, ws, meta, ns, G, K, plain_on,
                                 ks, kk, ctx->stream);
    else
        rc = hfx_batched_merge(ps, pk, ws, meta, ns, G, K, K, ks, kk, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_merge_items");
    if (elem_kind == 0) {
        rc = hfx_finish(ks, kk, ns, p->top_n, ctx->d_idx.as<uint32_t>(), wb, we, meta, out_s, out_k, out_pep,
                        plain_on, ncm, out_ncand, ctx->stream);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_finish");
        ctx->stage_end(HFX_STAGE_TOPN, 2, ns);
    } else {
        ctx->stage_end(HFX_STAGE_TOPN, 1, ns);
        ctx->stage_begin(HFX_STAGE_RESCORE);
        // unmodified keys only: rescore from the step's lists; modified keys
        // (and the fused mode, which keeps no lists) rebuild their ions
        if (lists_out && (long_rows || !mods_on))
            rc = hfx_rescore_lists(lists_out, long_rows, ctx->d_lstart.as<uint32_t>(), total10_out, llen_out,
                                   (uint32_t)ctx->num_pep, ctx->d_idx.as<uint32_t>(), rows, stride, meta, kk, ns, K,
                                   p->top_n, out_s, out_k, out_pep, ctx->d_err.as<uint32_t>(), ctx->stream);
        else
            rc = hfx_rescore(db, dm, rows, stride, meta, ks, kk, ns, K, p->top_n, p->fastdiv, out_s, out_k,
                             out_pep, ctx->stream);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_rescore");
        if (out_ncand) {
            rc = hfx_ncand(wb, we, meta, ns, plain_on, ncm, out_ncand, ctx->stream);
            if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_ncand");
        }
        ctx->stage_end(HFX_STAGE_RESCORE, out_ncand ? 2 : 1, (int64_t)ns * K);
    }
    return HFX_OK;
}

// Failure-detection test: HFX_TEST_HOLD_LOCK=1 makes every scorer CTA start
// with member 0's admission lock held by nobody, so each merge into it gives
// up after its bounded number of attempts (2^20), the CTA records a timeout
// in the error word and goes on, and the search returns HFX_ERR_TIMEOUT.
// Read at each search (eager searches; a captured graph keeps the value of
// its capture).  Off (0) by default.
int test_lock_attempts() {
    const char *v = std::getenv("HFX_TEST_HOLD_LOCK");
    if (!v || !*v) return 0;
    const int n = std::atoi(v);
    return n < 0 ? 0 : (n > 255 ? 255 : n);
}

// Clears the device error word and sets the word after it, which the
// scorers read as the lock hold test (0 = off).
cudaError_t clear_err(hfx_ctx *ctx) {
    cudaError_t e = cudaMemsetAsync(ctx->d_err.p, 0, 4, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(static_cast<uint8_t *>(ctx->d_err.p) + 4, test_lock_attempts(), 4, ctx->stream);
    return e;
}

// Everything a search enqueues, from clearing the error word to the last
// kernel; in gmode 2 this is what the CUDA graph captures.
int32_t search_enqueue(hfx_ctx *ctx, const hfx_search_params *p, const Batch &b, float *out_s, uint64_t *out_k,
                       uint32_t *out_pep, int64_t *out_ncand) {
    int32_t rc = 0;
    ctx->nvtx_close();
    HFX_CUDA(clear_err(ctx), "memset err");
    int64_t stride = 0;
    SpecMeta *meta = nullptr;
    float *rows = nullptr;
    __nv_bfloat16 *rows_bf = nullptr;
    __half *rows_h = nullptr;
    rc = run_stage_a(ctx, p, b, stride, meta, rows, rows_bf, rows_h, p->precision == 1, p->precision == 2);
    if (rc) return rc;
    // the modified isoforms are scored by the batched engine only: with
    // modifications on, batch_mode 0 runs the fused batched path
    if (p->batch_mode || (p->search_mods && ctx->num_mod > 0) || !p->search_plain ||
        stride > (int64_t)kMaxWords * 32)
        rc = search_batched(ctx, p, b, meta, rows, p->precision == 1 ? (const void *)rows_bf : (const void *)rows_h,
                            p->precision, stride, out_s, out_k, out_pep, out_ncand);
    else if (p->precision != 0)
        return fail(ctx, HFX_ERR_UNSUPPORTED, "per-spectrum launches use FP32 rows only");
    else
        rc = search_plain_per_spectrum(ctx, p, b, meta, rows, stride, out_s, out_k, out_pep, out_ncand);
    return rc;
}

// Waits for the search and turns the device error word into a status.
int32_t search_finish(hfx_ctx *ctx, uint32_t *herr_out = nullptr) {
    uint32_t herr = 0;
    HFX_CUDA(cudaMemcpyAsync(&herr, ctx->d_err.p, 4, cudaMemcpyDeviceToHost, ctx->stream), "D2H err");
    HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    ctx->stage_collect();
    if (herr_out) *herr_out = herr;
    if (herr & kErrTimeout) return fail(ctx, HFX_ERR_TIMEOUT, "device wait timed out");
    if (herr) return fail(ctx, HFX_ERR_UNSUPPORTED, "device error word " + std::to_string(herr));
    return HFX_OK;
}

// CUDA-graph search: the first call for a batch shape runs eagerly to learn
// the sizes, again with buffers at 1.25x those sizes, and then captures the
// whole enqueue sequence (no host synchronisation inside) into a graph;
// later calls with the same shape, buffers and parameters replay it.  A
// replay whose batch needs more than the capacities is reported on the
// device (row stride, work items) and re-planned eagerly.
int32_t search_graph(hfx_ctx *ctx, const hfx_search_params *p, const Batch &b, float *out_s, uint64_t *out_k,
                     uint32_t *out_pep, int64_t *out_ncand) {
    std::vector<uint8_t> key(sizeof(hfx_search_params) + sizeof(Batch) + 4 * sizeof(void *));
    uint8_t *kp = key.data();
    std::memcpy(kp, p, sizeof(hfx_search_params));
    kp += sizeof(hfx_search_params);
    std::memcpy(kp, &b, sizeof(Batch));
    kp += sizeof(Batch);
    const void *outs[4] = {out_s, out_k, out_pep, out_ncand};
    std::memcpy(kp, outs, sizeof(outs));
    // all graph work runs on the context's own graph stream, after the work
    // already queued on the caller's stream
    if (!ctx->graph_stream) {
        HFX_CUDA(cudaStreamCreateWithFlags(&ctx->graph_stream, cudaStreamNonBlocking), "graph stream");
        HFX_CUDA(cudaEventCreateWithFlags(&ctx->graph_event, cudaEventDisableTiming), "graph event");
    }
    HFX_CUDA(cudaEventRecord(ctx->graph_event, ctx->stream), "event");
    HFX_CUDA(cudaStreamWaitEvent(ctx->graph_stream, ctx->graph_event, 0), "wait event");
    struct StreamSwap {
        hfx_ctx *c;
        cudaStream_t saved;
        explicit StreamSwap(hfx_ctx *c_) : c(c_), saved(c_->stream) { c->stream = c->graph_stream; }
        ~StreamSwap() { c->stream = saved; }
    } swap(ctx);
    if (ctx->graph_valid && key == ctx->graph_key) {
        HFX_CUDA(cudaGraphLaunch(ctx->graph_exec, ctx->stream), "cudaGraphLaunch");
        uint32_t herr = 0;
        const int32_t rc = search_finish(ctx, &herr);
        if (!(herr & (kErrBounds | kErrTooLong))) return rc;
    }
    ctx->graph_reset();  // no graph yet, another shape, or the batch outgrew the capture
    const bool prof = ctx->profile;
    ctx->profile = false;
    auto restore = [&](int32_t rc) {
        ctx->gmode = 0;
        ctx->profile = prof;
        return rc;
    };
    ctx->gmode = 0;
    int32_t rc = search_enqueue(ctx, p, b, out_s, out_k, out_pep, out_ncand);
    if (!rc) rc = search_finish(ctx);
    if (rc) return restore(rc);
    // the group size the eager search used (a requested 16 falls back to 8
    // when more than 32 candidates are kept or the tile does not fit)
    const int32_t G = ctx->last_G > 0 ? ctx->last_G : (p->precision == 0 ? 4 : 8);
    ctx->cap_stride = ctx->last_stride;
    ctx->cap_groups = (uint32_t)((b.nspec + G - 1) / G + 24);  // <= one partial group per class
    ctx->cap_items = ctx->last_items + ctx->last_items / 4 + 64;
    ctx->cap_mitems = ctx->last_mitems + ctx->last_mitems / 4 + 64;
    ctx->cap_iso = ctx->last_iso + ctx->last_iso / 4 + 64;
    ctx->cap_iso_entries = ctx->last_iso_entries + ctx->last_iso_entries / 4 + 4096;
    ctx->gmode = 1;
    rc = search_enqueue(ctx, p, b, out_s, out_k, out_pep, out_ncand);
    if (!rc) rc = search_finish(ctx);
    if (rc) return restore(rc);
    ctx->gmode = 2;
    cudaGraph_t graph = nullptr;
    HFX_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed), "capture");
    rc = search_enqueue(ctx, p, b, out_s, out_k, out_pep, out_ncand);
    const cudaError_t ec = cudaStreamEndCapture(ctx->stream, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return restore(rc);
    }
    if (ec != cudaSuccess) return restore(cuda_fail(ctx, ec, "cudaStreamEndCapture"));
    const cudaError_t ei = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        ctx->graph_exec = nullptr;
        return restore(cuda_fail(ctx, ei, "cudaGraphInstantiate"));
    }
    ctx->graph_valid = true;
    ctx->graph_key = key;
    return restore(HFX_OK);
}

int32_t search_device(hfx_ctx *ctx, const hfx_search_params *p, const Batch &b, float *out_s, uint64_t *out_k,
                      uint32_t *out_pep, int64_t *out_ncand) {
    int32_t rc = check_params(ctx, p);
    if (rc) return rc;
    if (b.nspec <= 0) return HFX_OK;
    HFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    HFX_CUDA(ctx->d_err.ensure(16), "alloc err");
    if (p->use_graph) {
        if (!p->batch_mode && !(p->search_mods && ctx->num_mod > 0))
            return fail(ctx, HFX_ERR_UNSUPPORTED, "graph replay needs a batched mode (batch_mode 1 or 2)");
        return search_graph(ctx, p, b, out_s, out_k, out_pep, out_ncand);
    }
    rc = search_enqueue(ctx, p, b, out_s, out_k, out_pep, out_ncand);
    if (rc) return rc;
    return search_finish(ctx);
}

}  // namespace

extern "C" {

void hfx_default_params(hfx_search_params *p) {
    std::memset(p, 0, sizeof(*p));
    p->bin_width = 1.0005079f;
    p->custom_bin_width = 0;
    p->remove_precursor_peak = 1;
    p->tol_ppm = 0;
    p->top_n = 10;
    p->precision = 0;
    p->rescore_k = 0;
    p->batch_mode = 0;
    p->fastdiv = 0;
    p->search_plain = 1;
    p->search_mods = 1;
    p->group_size = 0;
    p->chunk = 0;
    p->max_len = 0;
    p->ion_bins_custom = 0;
    p->use_graph = 0;
}

int32_t hfx_ctx_create(int32_t device, hfx_ctx **out) {
    if (!out) return HFX_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return HFX_ERR_CUDA;
    hfx_ctx *c = new hfx_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) {
        delete c;
        return HFX_ERR_CUDA;
    }
    c->own_stream = true;
    const char *dbg = std::getenv("HFX_DEBUG_SYNC");
    c->debug_sync = dbg && dbg[0] == '1';
    *out = c;
    return HFX_OK;
}

int32_t hfx_ctx_destroy(hfx_ctx *ctx) {
    if (!ctx) return HFX_ERR_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->graph_reset();
    if (ctx->graph_stream) {
        cudaStreamSynchronize(ctx->graph_stream);
        cudaStreamDestroy(ctx->graph_stream);
    }
    if (ctx->graph_event) cudaEventDestroy(ctx->graph_event);
    for (auto &kv : ctx->ws) kv.second.release();
    ctx->d_ions.release();
    ctx->d_r.release();
    ctx->d_tc.release();
    ctx->d_tn.release();
    ctx->d_idx.release();
    ctx->d_lstart.release();
    ctx->d_mod_counts.release();
    ctx->d_mod_delta.release();
    ctx->d_err.release();
    for (int s = 0; s < HFX_NSTAGES; ++s)
        if (ctx->ev[s][0]) { cudaEventDestroy(ctx->ev[s][0]); cudaEventDestroy(ctx->ev[s][1]); }
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return HFX_OK;
}

int32_t hfx_set_stream(hfx_ctx *ctx, void *stream) {
    if (!ctx) return HFX_ERR_ARG;
    if (!stream) return HFX_OK;
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    ctx->stream = (cudaStream_t)stream;
    ctx->own_stream = false;
    return HFX_OK;
}

const char *hfx_last_error(const hfx_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int32_t hfx_set_profiling(hfx_ctx *ctx, int32_t on) {
    if (!ctx) return HFX_ERR_ARG;
    ctx->profile = on != 0;
    return HFX_OK;
}

int32_t hfx_set_workspace_limit(hfx_ctx *ctx, uint64_t bytes, uint64_t *in_use) {
    if (!ctx) return HFX_ERR_ARG;
    ctx->ws_limit = (size_t)bytes;
    if (in_use) *in_use = ctx->ws_total();
    return HFX_OK;
}

int32_t hfx_search_counters(hfx_ctx *ctx, uint64_t *out8, int32_t reset) {
    if (!ctx || !out8) return HFX_ERR_ARG;
    for (int i = 0; i < 8; ++i) {
        out8[i] = ctx->counters[i];
        if (reset) ctx->counters[i] = 0;
    }
    return HFX_OK;
}

int32_t hfx_mod_counters(hfx_ctx *ctx, uint64_t *out8, int32_t reset) {
    if (!ctx || !out8) return HFX_ERR_ARG;
    for (int i = 0; i < 8; ++i) {
        out8[i] = ctx->mod_counters[i];
        if (reset) ctx->mod_counters[i] = 0;
    }
    return HFX_OK;
}

int32_t hfx_stage_stats(hfx_ctx *ctx, double *ms, int64_t *launches, int64_t *units, int32_t reset) {
    if (!ctx) return HFX_ERR_ARG;
    ctx->stage_collect();
    for (int s = 0; s < HFX_NSTAGES; ++s) {
        if (ms) ms[s] = ctx->stage_ms[s];
        if (launches) launches[s] = ctx->stage_launches[s];
        if (units) units[s] = ctx->stage_units[s];
        if (reset) {
            ctx->stage_ms[s] = 0.0;
            ctx->stage_launches[s] = 0;
            ctx->stage_units[s] = 0;
        }
    }
    return HFX_OK;
}

int64_t hfx_digest(const uint8_t *seq, const uint32_t *seg, int32_t nprot, const float *mt26, int32_t rule,
                   int32_t missed, float min_mass, float max_mass, int32_t proline_rule, int32_t min_len,
                   int32_t max_len, float *r, uint32_t *tc, uint32_t *tn, int64_t cap) {
    if (!seq || !seg || !mt26 || nprot < 0 || missed < 0 || rule < 0 || rule > 13) return -1;
    struct Frag { float m; uint32_t c, n, len; };
    std::vector<Frag> fr;
    int64_t nf = 0;
    for (int32_t pi = 0; pi < nprot; ++pi) {
        // Fragment.hs:376-390: split after each cleavage residue; the last
        // piece of a protein ends one past its final residue.
        fr.clear();
        uint32_t c = seg[pi];
        const uint32_t y = seg[pi + 1];
        while (c < y) {
            uint32_t i = c;
            for (; i < y; ++i) {
                if (!cleaves_after(rule, seq[i])) continue;
                if (proline_rule && i + 1 < y && seq[i + 1] == 'P') continue;
                break;
            }
            float m = 0.0f;  // G.foldl' (+) 0
            if (i == y) {
                for (uint32_t j = c; j < y; ++j) m = m + mt26[seq[j] - 'A'];
                fr.push_back({m, c, y, y - c});
                break;
            }
            for (uint32_t j = c; j <= i; ++j) m = m + mt26[seq[j] - 'A'];
            fr.push_back({m, c, i, i - c + 1});
            c = i + 1;
        }
        // Fragment.hs:397-405 splice, :365-369 mass filter
        for (size_t i = 0; i < fr.size(); ++i) {
            Frag a = fr[i];
            for (int k = 0; k <= missed && i + k < fr.size(); ++k) {
                if (k) a = {a.m + fr[i + k].m, a.c, fr[i + k].n, a.len + fr[i + k].len};
                const float mm = (a.m + kHostH2O) + kHostH;
                if (!(min_mass <= mm && mm <= max_mass)) continue;
                if (min_len > 0 && (int32_t)a.len < min_len) continue;
                if (max_len > 0 && (int32_t)a.len > max_len) continue;
                if (r) {
                    if (nf >= cap) return -2;
                    r[nf] = a.m;
                    tc[nf] = a.c;
                    tn[nf] = a.n;
                }
                ++nf;
            }
        }
    }
    return nf;
}

namespace {

uint32_t rule_mask(int rule) {
    uint32_t m = 0;
    for (int c = 'A'; c <= 'Z'; ++c)
        if (cleaves_after(rule, (uint8_t)c)) m |= 1u << (c - 'A');
    return m;
}

// The digest on the device (digest.cu): counts, then, with `r`, resizes
// the three host vectors and fills them.  Returns the fragment count, -1 for
// bad arguments or -3 for a CUDA failure (ctx->err says which).
int64_t digest_device_run(hfx_ctx *ctx, const uint8_t *seq, const uint32_t *seg, int32_t nprot, const float *mt26,
                          int32_t rule, int32_t missed, float min_mass, float max_mass, int32_t proline_rule,
                          int32_t min_len, int32_t max_len, std::vector<float> *r, std::vector<uint32_t> *tc,
                          std::vector<uint32_t> *tn);

// The digest's scratch is freed when it returns (a one-time step of the
// database build, not a search workspace).
int64_t digest_device(hfx_ctx *ctx, const uint8_t *seq, const uint32_t *seg, int32_t nprot, const float *mt26,
                      int32_t rule, int32_t missed, float min_mass, float max_mass, int32_t proline_rule,
                      int32_t min_len, int32_t max_len, std::vector<float> *r, std::vector<uint32_t> *tc,
                      std::vector<uint32_t> *tn) {
    const int64_t n = digest_device_run(ctx, seq, seg, nprot, mt26, rule, missed, min_mass, max_mass, proline_rule,
                                        min_len, max_len, r, tc, tn);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (const char *name : {"dg_seq", "dg_seg", "dg_pm", "dg_ptn", "dg_plen", "dg_pnext", "dg_cnt", "dg_incl",
                             "dg_partial", "dg_r", "dg_tc", "dg_tn"})
        ctx->drop(name);
    return n;
}

int64_t digest_device_run(hfx_ctx *ctx, const uint8_t *seq, const uint32_t *seg, int32_t nprot, const float *mt26,
                          int32_t rule, int32_t missed, float min_mass, float max_mass, int32_t proline_rule,
                          int32_t min_len, int32_t max_len, std::vector<float> *r, std::vector<uint32_t> *tc,
                          std::vector<uint32_t> *tn) {
    const uint32_t nres = nprot > 0 ? seg[nprot] : 0u;
    for (int32_t p = 0; p < nprot; ++p)
        if (seg[p + 1] < seg[p]) return fail(ctx, HFX_ERR_ARG, "protein offsets must not decrease"), -1;
    for (uint32_t i = nprot > 0 ? seg[0] : 0u; i < nres; ++i)
        if (seq[i] < 'A' || seq[i] > 'Z') return fail(ctx, HFX_ERR_ARG, "residue outside A-Z"), -1;
    if (nres == 0) {
        if (r) r->clear(), tc->clear(), tn->clear();
        return 0;
    }
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, HFX_ERR_CUDA, "cudaSetDevice"), -3;
    cudaError_t e;
    uint8_t *d_seq = ctx->buf<uint8_t>("dg_seq", nres, e);
    uint32_t *d_seg = e ? nullptr : ctx->buf<uint32_t>("dg_seg", (size_t)nprot + 1, e);
    float *pm = e ? nullptr : ctx->buf<float>("dg_pm", nres, e);
    uint32_t *ptn = e ? nullptr : ctx->buf<uint32_t>("dg_ptn", nres, e);
    uint32_t *plen = e ? nullptr : ctx->buf<uint32_t>("dg_plen", nres, e);
    uint32_t *pnext = e ? nullptr : ctx->buf<uint32_t>("dg_pnext", nres, e);
    int32_t *cnt = e ? nullptr : ctx->buf<int32_t>("dg_cnt", nres, e);
    int32_t *incl = e ? nullptr : ctx->buf<int32_t>("dg_incl", nres, e);
    int32_t *partial = e ? nullptr : ctx->buf<int32_t>("dg_partial", hfx_scan_partials_needed(nres), e);
    if (e) return cuda_fail(ctx, e, "alloc digest"), -3;
    if ((e = cudaMemcpyAsync(d_seq, seq, nres, cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_seg, seg, 4ull * (nprot + 1), cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "H2D digest"), -3;
    const int32_t mask = (int32_t)rule_mask(rule);
    int rc = hfx_digest_launch(d_seq, d_seg, nprot, nres, mt26, mask, missed, min_mass, max_mass, proline_rule,
                               min_len, max_len, pm, ptn, plen, pnext, cnt, incl, partial, nullptr, nullptr, nullptr,
                               0, 1, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_digest"), -3;
    int32_t total = 0;
    if ((e = cudaMemcpyAsync(&total, incl + nres - 1, 4, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "digest count"), -3;
    if (!r) return total;
    r->resize(total);
    tc->resize(total);
    tn->resize(total);
    if (total == 0) return 0;
    float *d_r = ctx->buf<float>("dg_r", total, e);
    uint32_t *d_tc = e ? nullptr : ctx->buf<uint32_t>("dg_tc", total, e);
    uint32_t *d_tn = e ? nullptr : ctx->buf<uint32_t>("dg_tn", total, e);
    if (e) return cuda_fail(ctx, e, "alloc digest output"), -3;
    rc = hfx_digest_launch(d_seq, d_seg, nprot, nres, mt26, mask, missed, min_mass, max_mass, proline_rule, min_len,
                           max_len, pm, ptn, plen, pnext, cnt, incl, partial, d_r, d_tc, d_tn, total, 2, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_digest_splice"), -3;
    if ((e = cudaMemcpyAsync(r->data(), d_r, 4ull * total, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(tc->data(), d_tc, 4ull * total, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(tn->data(), d_tn, 4ull * total, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
        return cuda_fail(ctx, e, "D2H digest"), -3;
    return total;
}

}  // namespace

int64_t hfx_digest_gpu(hfx_ctx *ctx, const uint8_t *seq, const uint32_t *seg, int32_t nprot, const float *mt26,
                       int32_t rule, int32_t missed, float min_mass, float max_mass, int32_t proline_rule,
                       int32_t min_len, int32_t max_len, float *r, uint32_t *tc, uint32_t *tn, int64_t cap) {
    if (!ctx || !seq || !seg || !mt26 || nprot < 0 || missed < 0 || rule < 0 || rule > 13) {
        if (ctx) fail(ctx, HFX_ERR_ARG, "bad hfx_digest_gpu arguments");
        return -1;
    }
    if (!r) {
        const int64_t n = digest_device(ctx, seq, seg, nprot, mt26, rule, missed, min_mass, max_mass, proline_rule,
                                        min_len, max_len, nullptr, nullptr, nullptr);
        return n < 0 ? -1 : n;
    }
    if (!tc || !tn) return fail(ctx, HFX_ERR_ARG, "bad hfx_digest_gpu arguments"), -1;
    std::vector<float> hr;
    std::vector<uint32_t> htc, htn;
    const int64_t n = digest_device(ctx, seq, seg, nprot, mt26, rule, missed, min_mass, max_mass, proline_rule,
                                    min_len, max_len, &hr, &htc, &htn);
    if (n < 0) return -1;
    if (n > cap) return fail(ctx, HFX_ERR_ARG, "output capacity below the fragment count"), -2;
    std::memcpy(r, hr.data(), 4ull * n);
    std::memcpy(tc, htc.data(), 4ull * n);
    std::memcpy(tn, htn.data(), 4ull * n);
    return n;
}

int32_t hfx_pack_ions(const uint8_t *ascii, uint64_t n, const uint8_t *ma, int32_t num_ma, uint8_t *out) {
    if (!ascii || !out || num_ma < 0 || num_ma > 7) return HFX_ERR_ARG;
    std::vector<uint8_t> in(ascii, ascii + n), packed;
    pack_ions(in, ma, num_ma, packed);
    std::memcpy(out, packed.data(), n);
    return HFX_OK;
}

int32_t hfx_mass_table(int32_t mono, const float *add26, float *out26) {
    if (!out26) return HFX_ERR_ARG;
    // Config.hs:266-272 initializeAAMasses: static add + residue mass
    for (int i = 0; i < 26; ++i) out26[i] = (add26 ? add26[i] : 0.0f) + (mono ? kMonoMass[i] : kAvgMass[i]);
    return HFX_OK;
}

int32_t hfx_build_db(hfx_ctx *ctx, const uint8_t *seq, const uint32_t *seg, int32_t nprot, const float *add26,
                     int32_t mono, int32_t rule, int32_t missed, float min_mass, float max_mass,
                     int32_t proline_rule, int32_t min_len, int32_t max_len) {
    if (!ctx || !seq || !seg || nprot < 0 || missed < 0 || rule < 0 || rule > 13)
        return fail(ctx, HFX_ERR_ARG, "bad hfx_build_db arguments");
    hfx_mass_table(mono, add26, ctx->mt);
    const uint32_t nion = seg[nprot];
    for (uint32_t i = 0; i < nion; ++i)
        if (seq[i] < 'A' || seq[i] > 'Z') return fail(ctx, HFX_ERR_ARG, "residue outside A-Z");
    // the digest runs on the device; its fragments come back for the
    // mass-order sort and the list layout of upload_db
    const int64_t nf = digest_device(ctx, seq, seg, nprot, ctx->mt, rule, missed, min_mass, max_mass, proline_rule,
                                     min_len, max_len, &ctx->h_r, &ctx->h_tc, &ctx->h_tn);
    if (nf < 0) return nf == -1 ? HFX_ERR_ARG : HFX_ERR_CUDA;
    if (nf >= (1ll << 27)) return fail(ctx, HFX_ERR_UNSUPPORTED, "more than 2^27 fragments");
    ctx->h_ascii.assign(seq, seq + nion);
    ctx->h_seg.assign(seg, seg + nprot + 1);
    ctx->num_ions = nion;
    ctx->num_pep = (uint64_t)nf;
    return upload_db(ctx);
}

int32_t hfx_upload_db(hfx_ctx *ctx, const uint8_t *ions, uint64_t num_ions, const float *r, const uint32_t *tc,
                      const uint32_t *tn, uint64_t num_pep, const float *mt26) {
    if (!ctx || !ions || !r || !tc || !tn || !mt26) return fail(ctx, HFX_ERR_ARG, "bad hfx_upload_db arguments");
    if (num_pep >= (1ull << 27)) return fail(ctx, HFX_ERR_UNSUPPORTED, "more than 2^27 fragments");
    ctx->h_ascii.assign(ions, ions + num_ions);
    ctx->h_seg = {0u, (uint32_t)num_ions};
    ctx->h_r.assign(r, r + num_pep);
    ctx->h_tc.assign(tc, tc + num_pep);
    ctx->h_tn.assign(tn, tn + num_pep);
    std::memcpy(ctx->mt, mt26, sizeof(ctx->mt));
    ctx->num_ions = num_ions;
    ctx->num_pep = num_pep;
    return upload_db(ctx);
}

int32_t hfx_db_info(const hfx_ctx *ctx, uint64_t *num_ions, uint64_t *num_pep) {
    if (!ctx) return HFX_ERR_ARG;
    if (num_ions) *num_ions = ctx->num_ions;
    if (num_pep) *num_pep = ctx->num_pep;
    return HFX_OK;
}

int32_t hfx_db_export(const hfx_ctx *ctx, float *r, uint32_t *tc, uint32_t *tn, uint32_t *idx, float *mt26) {
    if (!ctx) return HFX_ERR_ARG;
    const size_t n = ctx->num_pep;
    if (r) std::memcpy(r, ctx->h_r.data(), n * 4);
    if (tc) std::memcpy(tc, ctx->h_tc.data(), n * 4);
    if (tn) std::memcpy(tn, ctx->h_tn.data(), n * 4);
    if (idx) std::memcpy(idx, ctx->h_idx.data(), n * 4);
    if (mt26) std::memcpy(mt26, ctx->mt, sizeof(ctx->mt));
    return HFX_OK;
}

int32_t hfx_set_mods(hfx_ctx *ctx, int32_t num_ma, const uint8_t *ma, const float *ma_mass, int32_t max_ma,
                     int32_t per_type) {
    if (!ctx || num_ma < 0 || num_ma > 7 || (num_ma > 0 && (!ma || !ma_mass)))
        return fail(ctx, HFX_ERR_ARG, "num_ma must be 0..7 (3-bit field, utils.h:97)");
    ctx->graph_reset();
    ctx->num_ma = num_ma;
    ctx->max_ma = max_ma;
    ctx->per_type = per_type;
    for (int i = 0; i < num_ma; ++i) {
        ctx->ma[i] = ma[i];
        ctx->ma_mass[i] = ma_mass[i];
    }
    make_mod_table(ctx);
    if (ctx->num_mod >= 512) return fail(ctx, HFX_ERR_UNSUPPORTED, "more than 511 modification combinations");
    if (ctx->num_mod > 0) {
        HFX_CUDA(ctx->d_mod_counts.ensure(ctx->mod_counts.size() * 4 + 16), "alloc mods");
        HFX_CUDA(ctx->d_mod_delta.ensure(ctx->mod_delta.size() * 4 + 16), "alloc mods");
        HFX_CUDA(cudaMemcpy(ctx->d_mod_counts.p, ctx->mod_counts.data(), ctx->mod_counts.size() * 4,
                            cudaMemcpyHostToDevice), "H2D mods");
        HFX_CUDA(cudaMemcpy(ctx->d_mod_delta.p, ctx->mod_delta.data(), ctx->mod_delta.size() * 4,
                            cudaMemcpyHostToDevice), "H2D mods");
    }
    if (ctx->num_pep > 0) return upload_db(ctx);
    return HFX_OK;
}

int32_t hfx_mod_table(const hfx_ctx *ctx, int32_t *num_mod, int32_t *counts, float *deltas, int32_t cap) {
    if (!ctx) return HFX_ERR_ARG;
    if (num_mod) *num_mod = ctx->num_mod;
    if (ctx->num_mod > cap) return HFX_ERR_ARG;
    if (counts) std::memcpy(counts, ctx->mod_counts.data(), ctx->mod_counts.size() * 4);
    if (deltas) std::memcpy(deltas, ctx->mod_delta.data(), ctx->mod_delta.size() * 4);
    return HFX_OK;
}

int32_t hfx_search_device(hfx_ctx *ctx, const hfx_search_params *p, const float *mz, const float *it,
                          const int64_t *off, const float *pcr, const float *z, const float *tol, int32_t nspec,
                          float *out_s, uint64_t *out_k, uint32_t *out_pep, int64_t *out_ncand) {
    if (!ctx) return HFX_ERR_ARG;
    Batch b{mz, it, pcr, z, tol, off, nspec};
    return search_device(ctx, p, b, out_s, out_k, out_pep, out_ncand);
}

int32_t hfx_search_evalues(hfx_ctx *ctx, const hfx_search_params *p, const float *mz, const float *it,
                           const int64_t *off, const float *pcr, const float *z, const float *tol, int32_t nspec,
                           int32_t bin_width, float cutoff_perc, float *out_s, uint64_t *out_k, uint32_t *out_pep,
                           int64_t *out_ncand, double *out_ev, double *out_fit) {
    if (!ctx || !p || nspec < 0 || !out_s || !out_k || !out_ev || !out_fit)
        return fail(ctx, HFX_ERR_ARG, "bad hfx_search_evalues arguments");
    if (bin_width < 1 || !(cutoff_perc >= 0.0f && cutoff_perc <= 100.0f))
        return fail(ctx, HFX_ERR_ARG, "E-value bin width must be >= 1 and the cut-off 0..100 %");
    if (nspec == 0) return HFX_OK;
    const bool mods_on = p->search_mods != 0 && ctx->num_mod > 0;
    const bool plain_on = p->search_plain != 0;
    Batch b{mz, it, pcr, z, tol, off, nspec};
    if (!mods_on && plain_on) {
        // one FP32 pass over the step's ion lists scores every pair into the
        // sink and keeps the top-N: the same top-N as a BF16/FP16 search
        // rescored in FP32 (both are the FP32 search's), without a second
        // scoring pass
        hfx_search_params q = *p;
        q.batch_mode = 1;
        q.use_graph = 0;
        q.precision = 0;
        q.group_size = 0;
        ctx->ev_single = true;
        ctx->ev_sink = nullptr;
        int32_t rc = search_device(ctx, &q, b, out_s, out_k, out_pep, out_ncand);
        ctx->ev_single = false;
        if (rc) return rc;
        if (!ctx->ev_sink) return fail(ctx, HFX_ERR_UNSUPPORTED, "E-value scores were not written");
        cudaError_t e;
        const uint64_t *soff = ctx->buf<uint64_t>("e_off", nspec, e);
        const uint64_t *size = e ? nullptr : ctx->buf<uint64_t>("e_size", nspec, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        rc = hfx_evalue_select_fit(ctx->ev_sink, soff, size, nspec, bin_width, cutoff_perc, out_fit, ctx->stream);
        if (!rc) rc = hfx_evalue_apply(out_s, out_k, out_fit, nspec, p->top_n, out_ev, ctx->stream);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "E-values");
        return search_finish(ctx);
    }
    // the search over the step's ion lists, eagerly
    hfx_search_params q = *p;
    q.batch_mode = 1;
    q.use_graph = 0;
    int32_t rc = search_device(ctx, &q, b, out_s, out_k, out_pep, out_ncand);
    if (rc) return rc;
    // every candidate's FP32 score (Search.hs:116-121: the unmodified
    // candidates and every modified isoform), from the step's lists, the
    // modification scorer and the FP32 rows
    cudaError_t e;
    const int32_t ns = nspec;
    const int64_t stride = ctx->last_stride;
    const bool long_rows = stride > (int64_t)kMaxWords * 32;
    const int32_t G = 4, K = p->top_n;
    const int32_t chunk = p->chunk > 0 ? p->chunk : 4096;
    SpecMeta *meta = ctx->buf<SpecMeta>("meta", ns, e);
    float *rows = ctx->buf<float>("rows32", (size_t)ns * stride, e);
    uint32_t *wb = ctx->buf<uint32_t>("wb", ns, e);
    uint32_t *we = ctx->buf<uint32_t>("we", ns, e);
    uint64_t *size = ctx->buf<uint64_t>("e_size", ns, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    uint64_t *soff = ctx->buf<uint64_t>("e_off", ns, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    uint64_t *send = ctx->buf<uint64_t>("e_end", ns, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    unsigned long long *cursor = ctx->buf<unsigned long long>("e_cursor", ns, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    // isoforms per spectrum, counted by the search's modification scorer
    unsigned long long *niso = mods_on ? ctx->buf<unsigned long long>("m_ncand", ns, e) : nullptr;
    if (e) return cuda_fail(ctx, e, "alloc");
    HFX_CUDA(clear_err(ctx), "memset err");
    rc = hfx_evalue_offsets(wb, we, plain_on ? 1 : 0, niso, ns, size, soff, send, cursor, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "E-value offsets");
    uint64_t total = 0;
    HFX_CUDA(cudaMemcpyAsync(&total, send + ns - 1, 8, cudaMemcpyDeviceToHost, ctx->stream), "D2H total");
    HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    float *sink = ctx->buf<float>("e_sink", total + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc E-value scores");
    // re-plan with FP32 groups of 4 over the search's workspace
    BatchedWs ws;
    ws.hist = ctx->buf<uint32_t>("b_hist", kBucketCount + 1, e);
    ws.cursor = ctx->buf<uint32_t>("b_cursor", kBucketCount, e);
    uint32_t *scal = ctx->buf<uint32_t>("b_scal", 8, e);
    ws.n_sorted = scal;
    ws.ngroups = scal + 1;
    ws.total_items = scal + 2;
    ws.counter = scal + 3;
    ws.perm = ctx->buf<int32_t>("b_perm", ns, e);
    ws.groups = ctx->buf<GroupInfo>("b_groups", ns, e);
    ws.item_off = ctx->buf<uint32_t>("b_itemoff", ns + 1, e);
    ws.group_of = ctx->buf<int32_t>("b_groupof", ns, e);
    ws.slot_of = ctx->buf<int32_t>("b_slotof", ns, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    rc = hfx_batched_plan(meta, ns, wb, we, G, chunk, ws, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "plan");
    uint32_t hs[4];
    HFX_CUDA(cudaMemcpyAsync(hs, scal, 16, cudaMemcpyDeviceToHost, ctx->stream), "D2H plan");
    HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    const uint32_t ngroups = hs[1], items = hs[2];
    void *tiles = ctx->buf<uint8_t>("e_tiles", (size_t)ngroups * stride * G * 4 + 64, e);
    if (e) return cuda_fail(ctx, e, "alloc tiles");
    float *ps = ctx->buf<float>("e_ps", (size_t)items * G * K + 1, e);
    uint64_t *pk = ctx->buf<uint64_t>("e_pk", (size_t)items * G * K + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    rc = hfx_pack_tiles(rows, 0, stride, meta, ws, tiles, ngroups, G, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_pack_tiles");
    if (plain_on) {
        const uint64_t total10 = ctx->list_units;
        const void *lists = long_rows ? (const void *)ctx->buf<uint32_t>("l_lists32", total10 * 10 + 64, e)
                                      : (const void *)ctx->buf<uint16_t>("l_lists", total10 * 10 + 64, e);
        const uint16_t *llen = ctx->buf<uint16_t>("l_len", (size_t)kLevels * ctx->num_pep, e);
        if (e) return cuda_fail(ctx, e, "lists");
        rc = hfx_lists_score(lists, long_rows, ctx->d_lstart.as<uint32_t>(), total10, llen, (uint32_t)ctx->num_pep,
                             0, stride, wb, we, ws, tiles, G, K, 0, ps, pk, nullptr, ctx->d_err.as<uint32_t>(),
                             ctx->stream, sink, soff);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_score_lists (all pairs)");
    }
    if (mods_on) {
        // the isoforms again, FP32 groups of 4, each score appended to its
        // spectrum's segment after the unmodified ones
        const int32_t nm = ctx->num_mod;
        const int32_t n_gm = (int32_t)ngroups * nm;
        const uint32_t *mb = ctx->buf<uint32_t>("m_wb", (size_t)ns * nm, e);
        const uint32_t *me = ctx->buf<uint32_t>("m_we", (size_t)ns * nm, e);
        uint32_t *mlo = ctx->buf<uint32_t>("m_lo", (size_t)n_gm + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        uint32_t *mhi = ctx->buf<uint32_t>("m_hi", (size_t)n_gm + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        uint32_t *mch = ctx->buf<uint32_t>("m_chunk", (size_t)n_gm + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        int32_t *nch = ctx->buf<int32_t>("m_nchunks", (size_t)n_gm + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        uint32_t *mitem_off = ctx->buf<uint32_t>("m_itemoff", (size_t)n_gm + 2, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        int32_t *partial = ctx->buf<int32_t>("m_partial", hfx_scan_partials_needed(n_gm + 1) + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        rc = hfx_mods_plan(ws, ngroups, mb, me, nm, chunk, mlo, mhi, mch, nch, mitem_off, partial, ctx->stream);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "modification plan (all pairs)");
        uint32_t mtotal = 0;
        if (n_gm > 0) {
            HFX_CUDA(cudaMemcpyAsync(&mtotal, mitem_off + n_gm, 4, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
            HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        }
        float *mps = ctx->buf<float>("e_mps", (size_t)mtotal * G * K + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        uint64_t *mpk = ctx->buf<uint64_t>("e_mpk", (size_t)mtotal * G * K + 1, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        if (mtotal > 0) {
            rc = hfx_mods_score(ctx->devdb(), ctx->devmods(), tiles, 0, stride, mb, me, ws, mlo, mhi, mch, mitem_off,
                                n_gm, G, K, p->fastdiv, mps, mpk, nullptr, ctx->d_err.as<uint32_t>(), ctx->stream,
                                sink, cursor, send);
            if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_score_mods (all pairs)");
        }
    }
    rc = hfx_evalue_select_fit(sink, soff, size, ns, bin_width, cutoff_perc, out_fit, ctx->stream);
    if (!rc) rc = hfx_evalue_apply(out_s, out_k, out_fit, ns, p->top_n, out_ev, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "E-values");
    return search_finish(ctx);
}

int32_t hfx_match_ions(hfx_ctx *ctx, const hfx_search_params *p, const float *z, int32_t nspec,
                       const uint64_t *keys, int32_t top_n, int32_t *out_matched, int32_t *out_total) {
    if (!ctx || !p || nspec < 0 || top_n < 1 || !z || !keys || !out_matched || !out_total)
        return fail(ctx, HFX_ERR_ARG, "bad hfx_match_ions arguments");
    if (nspec == 0) return HFX_OK;
    if (nspec != ctx->rows_nspec || ctx->rows_stride <= 0)
        return fail(ctx, HFX_ERR_ARG, "hfx_match_ions needs the spectra of the last search on this context");
    HFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaError_t e;
    const SpecMeta *meta = ctx->buf<SpecMeta>("meta", nspec, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    const float *rows = ctx->buf<float>("rows32", (size_t)nspec * ctx->rows_stride, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    HFX_CUDA(ctx->d_err.ensure(16), "alloc err");
    HFX_CUDA(clear_err(ctx), "memset err");
    // the spectrum bin width (IonSeries.hs:139 binWidth cp)
    const int rc = hfx_match_ions_launch(ctx->devdb(), ctx->devmods(), ctx->num_ions, meta, rows, ctx->rows_stride,
                                         z, p->bin_width, keys, nspec, top_n, out_matched, out_total,
                                         ctx->d_err.as<uint32_t>(), ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_match_ions");
    return search_finish(ctx);
}

int32_t hfx_set_protein_segments(hfx_ctx *ctx, const uint32_t *seg, int32_t nprot) {
    if (!ctx || !seg || nprot < 1 || seg[0] != 0 || seg[nprot] != ctx->h_ascii.size())
        return fail(ctx, HFX_ERR_ARG, "segments must start at 0 and end at the residue count");
    for (int32_t i = 0; i < nprot; ++i)
        if (seg[i + 1] < seg[i]) return fail(ctx, HFX_ERR_ARG, "segments must ascend");
    ctx->h_seg.assign(seg, seg + nprot + 1);
    return HFX_OK;
}

int32_t hfx_match_peptide(hfx_ctx *ctx, uint64_t key, uint32_t pep, char *text, int32_t cap, float *mh,
                          int32_t *protein) {
    if (!ctx || !text || cap < 8) return fail(ctx, HFX_ERR_ARG, "bad hfx_match_peptide arguments");
    if (pep >= ctx->num_pep) return fail(ctx, HFX_ERR_ARG, "fragment index out of range");
    // Location.hs:42-58 lookup: the protein holding the fragment, its
    // residues [c, n] (n itself unless it is the database's last residue),
    // the flanking residues or '-', and (M+H)+ = residual + H + H2O
    const uint32_t c = ctx->h_tc[pep], n = ctx->h_tn[pep];
    const uint32_t nion = (uint32_t)ctx->h_ascii.size();
    const size_t pi = (size_t)(std::upper_bound(ctx->h_seg.begin(), ctx->h_seg.end(), c) - ctx->h_seg.begin()) - 1;
    const uint32_t a = ctx->h_seg[pi], b = ctx->h_seg[pi + 1];
    const uint32_t ntake = n < nion ? n - c + 1 : n - c;
    std::string s;
    s.push_back(c > a ? (char)ctx->h_ascii[c - 1] : '-');
    s.push_back('.');
    for (uint32_t i = 0; i < ntake; ++i) s.push_back((char)ctx->h_ascii[c + i]);
    s.push_back('.');
    s.push_back(n + 1 < b ? (char)ctx->h_ascii[n + 1] : '-');
    float mass = (ctx->h_r[pep] + kHostH) + kHostH2O;
    if (key != ~0ull && (key >> 63)) {
        // Fragment.hs:84-106 modifyFragment: mass + sum(count * mass), and a
        // '*' after the i-th occurrence of each modified acid (i from the
        // isoform's unrank row; occurrences of that acid in the peptide text)
        const int32_t mu = (int32_t)((key >> 54) & 511u);
        const uint32_t pos = (uint32_t)((key >> 27) & ((1u << 27) - 1u));
        const uint32_t rank = (uint32_t)(key & ((1u << 27) - 1u));
        if (mu >= ctx->num_mod || pos >= ctx->num_pep || ctx->h_idx[pos] != pep)
            return fail(ctx, HFX_ERR_ARG, "modified key does not match the fragment");
        const int32_t *cnt = ctx->mod_counts.data() + (size_t)mu * ctx->num_ma;
        float add = 0.0f;
        for (int32_t i = 0; i < ctx->num_ma; ++i) add = add + (float)cnt[i] * ctx->ma_mass[i];
        mass = mass + add;
        // the unrank row, computed on the device by the enumeration kernel
        cudaError_t e;
        uint32_t *q = ctx->buf<uint32_t>("mq", 16, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        uint32_t hq[16] = {pos, (uint32_t)mu, rank};
        HFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
        HFX_CUDA(cudaMemcpy(q, hq, 12, cudaMemcpyHostToDevice), "H2D");
        uint8_t *mod = ctx->buf<uint8_t>("mq_mod", 64, e);
        if (e) return cuda_fail(ctx, e, "alloc");
        int rc = hfx_mods_isoforms(ctx->devdb(), ctx->devmods(), q, (const int32_t *)(q + 1), q + 2, 1, 64, q + 4,
                                   q + 8, mod, ctx->stream);
        if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_mod_isoforms");
        HFX_CUDA(cudaMemcpyAsync(hq, q, 64, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
        HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
        if (rank >= hq[4]) return fail(ctx, HFX_ERR_ARG, "isoform rank out of range");
        std::vector<uint8_t> star(s.size(), 0);
        int32_t u = 0;
        for (int32_t i = 0; i < ctx->num_ma; ++i) {
            std::vector<size_t> occ;
            for (size_t j = 2; j + 2 < s.size(); ++j)
                if ((uint8_t)s[j] == ctx->ma[i]) occ.push_back(j);
            for (int32_t t = 0; t < cnt[i]; ++t, ++u) {
                const uint32_t ith = u < 8 ? hq[8 + u] : ~0u;
                if (ith < occ.size()) star[occ[ith]] = 1;
            }
        }
        std::string m;
        for (size_t j = 0; j < s.size(); ++j) {
            m.push_back(s[j]);
            if (star[j]) m.push_back('*');
        }
        s.swap(m);
    }
    if ((int32_t)s.size() >= cap) return fail(ctx, HFX_ERR_ARG, "text buffer too small");
    std::memcpy(text, s.c_str(), s.size() + 1);
    if (mh) *mh = mass;
    if (protein) *protein = (int32_t)pi;
    return HFX_OK;
}

namespace {

// The persisted choices of hfx_autotune: a text file of lines
// "<batch shape key>\t<group size>\t<chunk>\t<ms>", named by the
// HFX_AUTOTUNE_FILE environment variable.  The key holds what the choice
// depends on: the device, the database and batch sizes and the search
// settings that select the kernels.
std::string autotune_key(const hfx_ctx *ctx, const hfx_search_params *p, int32_t nspec, int64_t npeaks) {
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, ctx->device) != cudaSuccess) return std::string();
    char buf[512];
    std::snprintf(buf, sizeof buf,
                  "%s/sm%d%d/%d SMs|pep %llu|spectra %d|peaks %lld|prec %d|mode %d|mods %d|bw %.7g/%d/%d|"
                  "tol %d|top %d|rescore %d|fastdiv %d|maxlen %d",
                  prop.name, prop.major, prop.minor, prop.multiProcessorCount, (unsigned long long)ctx->num_pep,
                  nspec, (long long)npeaks, p->precision, p->batch_mode,
                  (p->search_mods != 0 && ctx->num_mod > 0) ? ctx->num_mod : 0, (double)p->bin_width,
                  p->custom_bin_width, p->ion_bins_custom, p->tol_ppm, p->top_n, p->rescore_k, p->fastdiv,
                  p->max_len);
    std::string k(buf);
    for (char &c : k)
        if (c == '\t' || c == '\n') c = ' ';
    return k;
}

bool autotune_lookup(const char *path, const std::string &key, int32_t *g, int32_t *c, float *ms) {
    FILE *f = std::fopen(path, "r");
    if (!f) return false;
    char line[1024];
    bool found = false;
    while (std::fgets(line, sizeof line, f)) {
        char *t1 = std::strchr(line, '\t');
        if (!t1 || (size_t)(t1 - line) != key.size() || std::strncmp(line, key.c_str(), key.size()) != 0) continue;
        int gg = 0, cc = 0;
        float mm = 0.0f;
        if (std::sscanf(t1 + 1, "%d\t%d\t%f", &gg, &cc, &mm) == 3 && gg > 0 && cc > 0) {
            *g = gg;  // the last matching line wins
            *c = cc;
            *ms = mm;
            found = true;
        }
    }
    std::fclose(f);
    return found;
}

}  // namespace

int32_t hfx_autotune(hfx_ctx *ctx, hfx_search_params *p, const float *mz, const float *it, const int64_t *off,
                     const float *pcr, const float *z, const float *tol, int32_t nspec, float *out_s,
                     uint64_t *out_k, uint32_t *out_pep, int64_t *out_ncand, int32_t reps, float *ms_out) {
    if (!ctx || !p || nspec <= 0) return fail(ctx, HFX_ERR_ARG, "bad hfx_autotune arguments");
    if (p->batch_mode == 0) return fail(ctx, HFX_ERR_ARG, "hfx_autotune tunes the batched modes");
    HFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    Batch b{mz, it, pcr, z, tol, off, nspec};
    // a choice persisted for this batch shape is reused without timing
    const char *cache = std::getenv("HFX_AUTOTUNE_FILE");
    std::string key;
    if (cache && *cache) {
        int64_t npk = 0;
        HFX_CUDA(cudaMemcpy(&npk, off + nspec, 8, cudaMemcpyDeviceToHost), "D2H peak count");
        key = autotune_key(ctx, p, nspec, npk);
        int32_t g = 0, c = 0;
        float ms = 0.0f;
        if (!key.empty() && autotune_lookup(cache, key, &g, &c, &ms)) {
            p->group_size = g;
            p->chunk = c;
            if (ms_out) *ms_out = ms;
            return search_device(ctx, p, b, out_s, out_k, out_pep, out_ncand);
        }
    }
    hfx_search_params q = *p;
    q.use_graph = 0;
    // one 16-byte shared-memory load per bin: 8 BF16/FP16 or 4 FP32 spectra
    // per group are the natural sizes; half of that is the alternative, and
    // BF16/FP16 list scoring without modifications also tries 16
    const bool g16 = p->precision != 0 && p->batch_mode == 1 && !(p->search_mods != 0 && ctx->num_mod > 0);
    const int32_t gs[3] = {p->precision == 0 ? 4 : 8, p->precision == 0 ? 2 : 4, 16};
    const int ngs = g16 ? 3 : 2;
    const int32_t chunks[5] = {1024, 2048, 4096, 8192, 16384};
    cudaEvent_t e0, e1;
    HFX_CUDA(cudaEventCreate(&e0), "event");
    HFX_CUDA(cudaEventCreate(&e1), "event");
    float best = 1e30f;
    int32_t best_g = gs[0], best_c = chunks[2];
    int32_t rc = HFX_OK;
    for (int gi = 0; gi < ngs && rc == HFX_OK; ++gi) {
        for (int ci = 0; ci < 5 && rc == HFX_OK; ++ci) {
            q.group_size = gs[gi];
            q.chunk = chunks[ci];
            rc = search_device(ctx, &q, b, out_s, out_k, out_pep, out_ncand);
            float tot = 0.0f;
            for (int r = 0; r < std::max(1, reps) && rc == HFX_OK; ++r) {
                cudaEventRecord(e0, ctx->stream);
                rc = search_device(ctx, &q, b, out_s, out_k, out_pep, out_ncand);
                cudaEventRecord(e1, ctx->stream);
                cudaEventSynchronize(e1);
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, e0, e1);
                tot += ms;
            }
            const float avg = tot / std::max(1, reps);
            if (rc == HFX_OK && avg < best) {
                best = avg;
                best_g = gs[gi];
                best_c = chunks[ci];
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    p->group_size = best_g;
    p->chunk = best_c;
    if (ms_out) *ms_out = best;
    if (!key.empty()) {
        FILE *f = std::fopen(cache, "a");
        if (f) {
            std::fprintf(f, "%s\t%d\t%d\t%.4f\n", key.c_str(), best_g, best_c, (double)best);
            std::fclose(f);
        }
    }
    return HFX_OK;
}

int32_t hfx_search_host(hfx_ctx *ctx, const hfx_search_params *p, const float *mz, const float *it,
                        const int64_t *off, const float *pcr, const float *z, const float *tol, int32_t nspec,
                        float *out_s, uint64_t *out_k, uint32_t *out_pep, int64_t *out_ncand) {
    if (!ctx || nspec < 0 || !off) return fail(ctx, HFX_ERR_ARG, "bad hfx_search_host arguments");
    HFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int64_t npk = off[nspec];
    cudaError_t e;
    float *d_mz = ctx->buf<float>("in_mz", npk + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    float *d_it = ctx->buf<float>("in_it", npk + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    int64_t *d_off = ctx->buf<int64_t>("in_off", nspec + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    float *d_meta = ctx->buf<float>("in_pzt", 3ull * nspec + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    const int32_t topn = p ? p->top_n : 0;
    float *d_os = ctx->buf<float>("out_s", (size_t)nspec * topn + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    uint64_t *d_ok = ctx->buf<uint64_t>("out_k", (size_t)nspec * topn + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    uint32_t *d_op = ctx->buf<uint32_t>("out_p", (size_t)nspec * topn + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    int64_t *d_nc = ctx->buf<int64_t>("out_nc", nspec + 1, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    cudaStream_t st = ctx->stream;
    HFX_CUDA(cudaMemcpyAsync(d_mz, mz, 4ull * npk, cudaMemcpyHostToDevice, st), "H2D mz");
    HFX_CUDA(cudaMemcpyAsync(d_it, it, 4ull * npk, cudaMemcpyHostToDevice, st), "H2D it");
    HFX_CUDA(cudaMemcpyAsync(d_off, off, 8ull * (nspec + 1), cudaMemcpyHostToDevice, st), "H2D off");
    HFX_CUDA(cudaMemcpyAsync(d_meta, pcr, 4ull * nspec, cudaMemcpyHostToDevice, st), "H2D pcr");
    HFX_CUDA(cudaMemcpyAsync(d_meta + nspec, z, 4ull * nspec, cudaMemcpyHostToDevice, st), "H2D z");
    HFX_CUDA(cudaMemcpyAsync(d_meta + 2 * nspec, tol, 4ull * nspec, cudaMemcpyHostToDevice, st), "H2D tol");
    Batch b{d_mz, d_it, d_meta, d_meta + nspec, d_meta + 2 * nspec, d_off, nspec};
    int32_t rc = search_device(ctx, p, b, d_os, d_ok, d_op, out_ncand ? d_nc : nullptr);
    if (rc) return rc;
    HFX_CUDA(cudaMemcpyAsync(out_s, d_os, 4ull * nspec * topn, cudaMemcpyDeviceToHost, st), "D2H score");
    HFX_CUDA(cudaMemcpyAsync(out_k, d_ok, 8ull * nspec * topn, cudaMemcpyDeviceToHost, st), "D2H key");
    if (out_pep) HFX_CUDA(cudaMemcpyAsync(out_pep, d_op, 4ull * nspec * topn, cudaMemcpyDeviceToHost, st), "D2H pep");
    if (out_ncand) HFX_CUDA(cudaMemcpyAsync(out_ncand, d_nc, 8ull * nspec, cudaMemcpyDeviceToHost, st), "D2H nc");
    HFX_CUDA(cudaStreamSynchronize(st), "sync");
    return HFX_OK;
}

int32_t hfx_preprocess(hfx_ctx *ctx, const hfx_search_params *p, const float *mz, const float *it,
                       const int64_t *off, const float *pcr, const float *z, int32_t nspec, int64_t stride,
                       float *rows, void *rows_bf16, void *rows_fp16, int32_t *lens, float *masses) {
    if (!ctx || !p || nspec < 0 || !rows) return fail(ctx, HFX_ERR_ARG, "bad hfx_preprocess arguments");
    if (nspec == 0) return HFX_OK;
    HFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaError_t e;
    LayoutParams lp = layout_params(p);
    lp.max_len = (int32_t)std::min<int64_t>(stride, lp.max_len > stride ? stride : lp.max_len);
    lp.max_len = (int32_t)stride;
    SpecMeta *meta = ctx->buf<SpecMeta>("meta", nspec, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    uint32_t *d_max = ctx->buf<uint32_t>("maxlen", 4, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    float *tol = ctx->buf<float>("tol0", nspec, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    HFX_CUDA(cudaMemsetAsync(tol, 0, 4ull * nspec, ctx->stream), "memset");
    int rc = hfx_launch_layout(mz, off, pcr, z, tol, nspec, lp, meta, d_max, nullptr, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_layout");
    HFX_CUDA(ctx->d_err.ensure(16), "alloc err");
    HFX_CUDA(clear_err(ctx), "memset err");
    rc = hfx_launch_preprocess(mz, it, off, pcr, lp, meta, nspec, stride, rows, (__nv_bfloat16 *)rows_bf16,
                               (__half *)rows_fp16, ctx->d_err.as<uint32_t>(), ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_preprocess");
    std::vector<SpecMeta> hm(nspec);
    HFX_CUDA(cudaMemcpyAsync(hm.data(), meta, sizeof(SpecMeta) * nspec, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    std::vector<int32_t> hl(nspec);
    std::vector<float> hmass(nspec);
    for (int32_t s = 0; s < nspec; ++s) {
        hl[s] = hm[s].status == 0 ? hm[s].len : 0;
        hmass[s] = hm[s].mass;
    }
    if (lens) HFX_CUDA(cudaMemcpy(lens, hl.data(), 4ull * nspec, cudaMemcpyHostToDevice), "H2D lens");
    if (masses) HFX_CUDA(cudaMemcpy(masses, hmass.data(), 4ull * nspec, cudaMemcpyHostToDevice), "H2D masses");
    return HFX_OK;
}

int32_t hfx_find_windows(hfx_ctx *ctx, const hfx_search_params *p, const float *mz, const int64_t *off,
                         const float *pcr, const float *z, const float *tol, int32_t nspec, uint32_t *begin,
                         uint32_t *end) {
    if (!ctx || !p || nspec < 0 || !begin || !end) return fail(ctx, HFX_ERR_ARG, "bad hfx_find_windows arguments");
    if (nspec == 0) return HFX_OK;
    HFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaError_t e;
    const LayoutParams lp = layout_params(p);
    SpecMeta *meta = ctx->buf<SpecMeta>("meta", nspec, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    uint32_t *d_max = ctx->buf<uint32_t>("maxlen", 4, e);
    if (e) return cuda_fail(ctx, e, "alloc");
    int rc = hfx_launch_layout(mz, off, pcr, z, tol, nspec, lp, meta, d_max, nullptr, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_layout");
    rc = hfx_launch_windows(ctx->d_r.as<float>(), (uint32_t)ctx->num_pep, meta, nspec, begin, end, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_windows");
    HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    return HFX_OK;
}

int32_t hfx_ion_bins(hfx_ctx *ctx, const uint32_t *pos, const int32_t *charges, const int32_t *lens, int32_t n,
                     int32_t cap, int32_t fastdiv, uint32_t *bins, uint8_t *levels, int32_t *count) {
    if (!ctx || n < 0 || !pos || !charges || !lens || !bins || !levels || !count)
        return fail(ctx, HFX_ERR_ARG, "bad hfx_ion_bins arguments");
    if (n == 0) return HFX_OK;
    HFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    int rc = hfx_launch_ion_bins(ctx->devdb(), pos, charges, lens, n, kMaxWords * 32, cap, fastdiv, bins, levels,
                                 count, ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_ion_bins");
    HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    return HFX_OK;
}

int32_t hfx_mod_isoforms(hfx_ctx *ctx, const uint32_t *pos, const int32_t *mod, const uint32_t *rank, int32_t n,
                         int32_t cap, uint32_t *count, uint32_t *unrank, uint8_t *modded) {
    if (!ctx || n < 0 || cap < 0 || !pos || !mod || !rank || !count || !unrank || !modded)
        return fail(ctx, HFX_ERR_ARG, "bad hfx_mod_isoforms arguments");
    if (ctx->num_mod <= 0) return fail(ctx, HFX_ERR_ARG, "no modification table (hfx_set_mods)");
    if (n == 0) return HFX_OK;
    // queries are checked on the host: positions and combinations index device tables
    std::vector<uint32_t> hp(n);
    std::vector<int32_t> hm(n);
    HFX_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    HFX_CUDA(cudaMemcpy(hp.data(), pos, 4ull * n, cudaMemcpyDeviceToHost), "D2H pos");
    HFX_CUDA(cudaMemcpy(hm.data(), mod, 4ull * n, cudaMemcpyDeviceToHost), "D2H mod");
    for (int32_t i = 0; i < n; ++i)
        if (hp[i] >= ctx->num_pep || hm[i] < 0 || hm[i] >= ctx->num_mod)
            return fail(ctx, HFX_ERR_ARG, "query out of range");
    int rc = hfx_mods_isoforms(ctx->devdb(), ctx->devmods(), pos, mod, rank, n, cap, count, unrank, modded,
                               ctx->stream);
    if (rc) return cuda_fail(ctx, (cudaError_t)rc, "k_mod_isoforms");
    HFX_CUDA(cudaStreamSynchronize(ctx->stream), "sync");
    return HFX_OK;
}

}  // extern "C"
