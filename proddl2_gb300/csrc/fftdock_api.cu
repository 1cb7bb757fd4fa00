// C ABI of libfftdock.so (declared in include/fftdock.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <mutex>
#include <vector>

#include "fft_core.cuh"
#include "fftdock.h"
#include "internal.h"

namespace fftdock {
const SizeOps* size_ops_small(int n);
const SizeOps* size_ops_mid(int n);
const SizeOps* size_ops_big(int n);
const SizeOps* size_ops_n128(int n);
const SizeOps* size_ops_n144(int n);

const SizeOps* size_ops(int n) {
    const SizeOps* o = nullptr;
    if ((o = size_ops_small(n))) return o;
    if ((o = size_ops_mid(n))) return o;
    if ((o = size_ops_big(n))) return o;
    if ((o = size_ops_n128(n))) return o;
    if ((o = size_ops_n144(n))) return o;
    return nullptr;
}

constexpr int kKC = 16;
constexpr int kMaxEntries = 32768;
constexpr size_t kMaxSmem = 227 * 1024;
}  // namespace fftdock

using fftdock::BatchArgs;
using fftdock::SizeOps;

struct fftdock_ctx {
    fftdock_config cfg{};
    std::vector<double> ace;
    const SizeOps* ops = nullptr;
    int N = 0, H = 0, PP = 0, K = 0, B = 0;
    size_t V = 0;
    double h = 0, zero_h = 0, center0 = 0;
    // per-axis sizes and geometry (all N on a cubic grid); box: the box-grid
    // path (box_grid.cu) with its per-axis twiddle tables [Nx | Ny | Nz]
    int dims[3] = {0, 0, 0};
    fftdock::Geo geo{};
    bool box = false;
    float2* btw32 = nullptr;
    double2* btw64 = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;

    float2* tw32 = nullptr;
    double2* tw64 = nullptr;
    void* spec = nullptr;       // float2 or __nv_bfloat162 pairs (cfg.precision)
    double* rgrid = nullptr;
    double* emat = nullptr;

    bool have_rec = false, have_lig = false;
    int n_ent = 0;
    double* lig_xyz = nullptr;
    int32_t* lig_term = nullptr;
    // weighted entries (the LJ term sets)
    bool lj = false;
    float* lig_w32 = nullptr;
    double* lig_w64 = nullptr;
    float* ent_w = nullptr;
    int32_t* ent_idx = nullptr;

    // work: ent/offs/cand (and ent_w/ent_idx) per group of G rotations,
    // g2 per batch of B
    int G = 0;
    uint32_t* ent = nullptr;
    int32_t* offs = nullptr;
    float2* g2 = nullptr;
    float2* g2t = nullptr;   // tensor stage output (x-quads)
    float* cand_v = nullptr;
    int32_t* cand_i = nullptr;

    // per-call buffers (grown on demand)
    int cap_rot = 0;
    double* rot_all = nullptr;
    int32_t* status_all = nullptr;
    fftdock_peak* peaks_all = nullptr;
    int32_t* npeaks_all = nullptr;
    int cap_status_dev = 0;
    int32_t* status_dev = nullptr;

    // tensor-core pencil stage
    bool use_tc = false;
    float2* circ = nullptr;
    int8_t* cscale = nullptr;
    float2* tc_slots = nullptr;  // running sums of the tensor stage (tc_slot_count slots of 128 x 128)
    int tc_n_slots = 0;
    int* err_dev = nullptr;
    int x0 = 0, W = 0;
    bool tc_ready = false;       // the ligand fits the tensor stage (window, terms, unweighted)
    uint32_t* ent_t = nullptr;   // [G/128][n_pad][128]
    int32_t* tinfo = nullptr;    // non-empty terms: padded entry starts, then term ids
    int32_t* tpad = nullptr;     // [K] padded start - start per term
    int n_tc_terms = 0, n_pad = 0;

    // the no-allocation scan's work array, resolved at creation
    void* noalloc_scratch = nullptr;

    // queue + clustering path (cfg.cluster_trans)
    fftdock::WideArgs wide{};

    // kernel timing (fftdock_profile): event pool and (stage, from, to)
    // records of pool indices
    bool profiling = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    struct EvRec {
        int stage;
        size_t from, to;
    };
    std::vector<EvRec> ev_recs;
};

namespace {

int fail(fftdock_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(fftdock_ctx* c, cudaError_t e, const char* where) {
    return fail(c, FFTDOCK_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(expr)                                                   \
    do {                                                           \
        cudaError_t e_ = (expr);                                   \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #expr);   \
    } while (0)

template <typename T> cudaError_t dalloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    return cudaMalloc((void**)p, n * sizeof(T));
}

template <typename T> void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

bool finite3(const double* p, int n) {
    for (int i = 0; i < 3 * n; ++i)
        if (!std::isfinite(p[i])) return false;
    return true;
}

int grow_call_buffers(fftdock_ctx* ctx, int n_rot) {
    if (n_rot <= ctx->cap_rot) return FFTDOCK_OK;
    dfree(ctx->rot_all);
    dfree(ctx->status_all);
    dfree(ctx->peaks_all);
    dfree(ctx->npeaks_all);
    ctx->cap_rot = 0;
    CK(dalloc(&ctx->rot_all, (size_t)n_rot * 9));
    CK(dalloc(&ctx->status_all, (size_t)n_rot));
    CK(dalloc(&ctx->peaks_all, (size_t)n_rot * ctx->cfg.peaks_per_rot));
    CK(dalloc(&ctx->npeaks_all, (size_t)n_rot));
    ctx->cap_rot = n_rot;
    return FFTDOCK_OK;
}

int grow_status(fftdock_ctx* ctx, int n_rot) {
    if (n_rot <= ctx->cap_status_dev) return FFTDOCK_OK;
    dfree(ctx->status_dev);
    ctx->cap_status_dev = 0;
    CK(dalloc(&ctx->status_dev, (size_t)n_rot));
    ctx->cap_status_dev = n_rot;
    return FFTDOCK_OK;
}

BatchArgs batch_args(fftdock_ctx* ctx) {
    BatchArgs a{};
    a.lig_xyz = ctx->lig_xyz;
    a.lig_term = ctx->lig_term;
    a.lig_w32 = ctx->lig_w32;
    a.lig_w64 = ctx->lig_w64;
    a.ent_w = ctx->ent_w;
    a.ent_idx = ctx->ent_idx;
    a.spec = ctx->spec;
    a.spec_bf16 = ctx->cfg.precision == FFTDOCK_PREC_BF16_SPECTRA ? 1 : 0;
    a.rgrid = ctx->rgrid;
    a.tw32 = ctx->tw32;
    a.n_ent = ctx->n_ent;
    a.K = ctx->K;
    a.PP = ctx->PP;
    a.h = ctx->h;
    a.zero_h = ctx->zero_h;
    a.center0 = ctx->center0;
    a.ent = ctx->ent;
    a.offs = ctx->offs;
    a.g2 = ctx->g2;
    a.g2t = ctx->g2t;
    a.cand_v = ctx->cand_v;
    a.cand_i = ctx->cand_i;
    a.peak_stride = ctx->cfg.peaks_per_rot;
    a.k_out = std::min(ctx->cfg.peaks_per_rot, ctx->cfg.max_trans_inp);
    a.max_val = ctx->cfg.max_val_corr;
    a.circ = ctx->circ;
    a.cscale = ctx->cscale;
    a.x0 = ctx->x0;
    a.W = ctx->W;
    a.use_tc = ctx->use_tc && ctx->tc_ready ? 1 : 0;
    a.ent_t = ctx->ent_t;
    a.tinfo = ctx->tinfo;
    a.tpad = ctx->tpad;
    a.n_tc_terms = ctx->n_tc_terms;
    a.tc_group = ctx->cfg.tc_terms_per_sum;
    a.tc_slots = ctx->tc_slots;
    a.tc_n_slots = ctx->tc_n_slots;
    a.n_pad = ctx->n_pad;
    a.err = ctx->err_dev;
    a.wide = ctx->wide;
    a.box = ctx->box ? ctx->geo : fftdock::Geo{};
    a.box_tw32 = ctx->btw32;
    return a;
}

// nonzero device error word -> FFTDOCK_ECUDA (after a synchronisation)
int check_pipeline(fftdock_ctx* ctx) {
    int err = 0;
    CK(cudaMemcpy(&err, ctx->err_dev, sizeof(int), cudaMemcpyDeviceToHost));
    if (err != 0) {
        cudaMemset(ctx->err_dev, 0, sizeof(int));
        // bits 2, 4, 16: a bounded wait on a pipeline barrier ran out; 32: a
        // CTA found no running-sum slot for its SM (an SM id at or above %nsmid)
        const std::string what = (err & 32) && !(err & 23) ? "tensor pencil stage found no running-sum slot"
                                                           : "tensor pencil stage timed out waiting on a pipeline barrier";
        return fail(ctx, FFTDOCK_ECUDA, what + " (code " + std::to_string(err) + ")");
    }
    return FFTDOCK_OK;
}

// n events from the profiling pool; returns the index of the first
int take_events(fftdock_ctx* ctx, size_t n, size_t* first) {
    while (ctx->ev_pool.size() < ctx->ev_used + n) {
        cudaEvent_t ev;
        cudaError_t e = cudaEventCreate(&ev);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaEventCreate");
        ctx->ev_pool.push_back(ev);
    }
    *first = ctx->ev_used;
    ctx->ev_used += n;
    return FFTDOCK_OK;
}

// Rotations per group: ligand prep and finalize run once per group (full-GPU
// launches), pencil and plane once per batch of B.
int group_size(int B) { return B * std::max(1, 1024 / B); }

// queue every batch of a call; rot/peaks/npeaks/status are device arrays
// covering the whole call
int run_batches(fftdock_ctx* ctx, int n_rot, const double* rot, int first_id, fftdock_peak* peaks,
                int32_t* npeaks, int32_t* status, cudaStream_t s, float* dbg, float* pool_v, int32_t* pool_i) {
    const BatchArgs a = batch_args(ctx);
    const int N = ctx->N, stride = ctx->cfg.peaks_per_rot;
    int rc;
    size_t ev = 0;
    for (int g0 = 0; g0 < n_rot; g0 += ctx->G) {
        BatchArgs ga = a;
        ga.ev = nullptr;
        ga.n_rot = std::min(ctx->G, n_rot - g0);
        ga.rot = rot + (size_t)g0 * 9;
        ga.status = status + g0;
        ga.peaks = peaks + (size_t)g0 * stride;
        ga.n_peaks = npeaks + g0;
        ga.first_rot_id = first_id + g0;
        ga.dbg_corr = dbg ? dbg + (size_t)g0 * ctx->V : nullptr;
        ga.pool_v = pool_v ? pool_v + (size_t)g0 * fftdock::kKC : nullptr;
        ga.pool_i = pool_i ? pool_i + (size_t)g0 * fftdock::kKC : nullptr;
        cudaError_t e;
        if (ctx->profiling) {
            if ((rc = take_events(ctx, 2, &ev))) return rc;
            if ((e = cudaEventRecord(ctx->ev_pool[ev], s)) != cudaSuccess) return cuda_fail(ctx, e, "event");
        }
        if ((e = ctx->ops->prep(ga, s)) != cudaSuccess) return cuda_fail(ctx, e, "ligand prep launch");
        if (ctx->profiling) {
            if ((e = cudaEventRecord(ctx->ev_pool[ev + 1], s)) != cudaSuccess) return cuda_fail(ctx, e, "event");
            ctx->ev_recs.push_back({0, ev, ev + 1});
        }
        for (int j = 0; j < ga.n_rot; j += ctx->B) {
            BatchArgs b = ga;
            b.n_rot = std::min(ctx->B, ga.n_rot - j);
            b.rot += (size_t)j * 9;
            b.status += j;
            b.peaks += (size_t)j * stride;
            b.n_peaks += j;
            b.first_rot_id += j;
            if (b.dbg_corr) b.dbg_corr += (size_t)j * ctx->V;
            if (b.pool_v) b.pool_v += (size_t)j * fftdock::kKC;
            if (b.pool_i) b.pool_i += (size_t)j * fftdock::kKC;
            b.ent += (size_t)j * ctx->n_ent;
            b.offs += (size_t)j * (ctx->K * N + 1);
            b.cand_v += (size_t)j * N * fftdock::kKC;
            b.cand_i += (size_t)j * N * fftdock::kKC;
            if (b.ent_w) b.ent_w += (size_t)j * ctx->n_ent;
            if (b.ent_idx) b.ent_idx += (size_t)j * ctx->n_ent;
            if (b.ent_t) b.ent_t += (size_t)j * ctx->n_pad;  // j is a multiple of 128 on the tensor path
            cudaEvent_t evs[4];
            const bool wide = b.wide.corr != nullptr;
            if (ctx->profiling) {
                const size_t n_ev = wide ? 4 : 3;
                if ((rc = take_events(ctx, n_ev, &ev))) return rc;
                for (size_t k = 0; k < n_ev; ++k) evs[k] = ctx->ev_pool[ev + k];
                b.ev = evs;
                ctx->ev_recs.push_back({1, ev, ev + 1});
                ctx->ev_recs.push_back({2, ev + 1, ev + 2});
                if (wide) ctx->ev_recs.push_back({3, ev + 2, ev + 3});
            }
            if ((e = ctx->ops->middle(b, s)) != cudaSuccess) return cuda_fail(ctx, e, "scan batch launch");
        }
        if (ga.wide.corr) continue;
        if (ctx->profiling) {
            if ((rc = take_events(ctx, 2, &ev))) return rc;
            if ((e = cudaEventRecord(ctx->ev_pool[ev], s)) != cudaSuccess) return cuda_fail(ctx, e, "event");
        }
        if ((e = ctx->ops->finish(ga, s)) != cudaSuccess) return cuda_fail(ctx, e, "finalize launch");
        if (ctx->profiling) {
            if ((e = cudaEventRecord(ctx->ev_pool[ev + 1], s)) != cudaSuccess) return cuda_fail(ctx, e, "event");
            ctx->ev_recs.push_back({3, ev, ev + 1});
        }
    }
    return FFTDOCK_OK;
}

int check_ready(fftdock_ctx* ctx) {
    if (!ctx) return FFTDOCK_EINVAL;
    if (!ctx->have_rec) return fail(ctx, FFTDOCK_ESTATE, "fftdock_set_receptor has not been called");
    if (!ctx->have_lig) return fail(ctx, FFTDOCK_ESTATE, "fftdock_set_ligand has not been called");
    return FFTDOCK_OK;
}

}  // namespace

namespace fftdock {

namespace {
__global__ void fill_u32_kernel(uint32_t* p, uint32_t v, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}
}  // namespace

cudaError_t fill_padding(uint32_t* ent_t, int W, size_t n, cudaStream_t s) {
    fill_u32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(ent_t, (uint32_t)W << 24, n);
    return cudaGetLastError();
}

namespace {
__global__ void nsmid_kernel(int* out) {
    uint32_t v;
    asm volatile("mov.u32 %0, %%nsmid;" : "=r"(v));
    *out = (int)v;
}
}  // namespace

cudaError_t tc_slot_count(int* n_slots) {
    static std::mutex mu;
    static std::vector<int> cache;  // per device ordinal
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
    if (cache[dev] == 0) {
        int* d = nullptr;
        if ((e = cudaMalloc(&d, sizeof(int))) != cudaSuccess) return e;
        nsmid_kernel<<<1, 1>>>(d);
        int h = 0;
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
        cudaFree(d);
        if (e != cudaSuccess) return e;
        if (h < 1) return cudaErrorUnknown;
        cache[dev] = h;
    }
    *n_slots = 2 * cache[dev];
    return cudaSuccess;
}

TcTables tc_tables(const double* xyz, const int32_t* term, int n, int K, int N, double h, double zero_h) {
    TcTables t;
    // window of x cells that holds the ligand under every rotation about the
    // origin: |R p| <= max |p|, with a cell of margin on each side
    double rmax = 0.0;
    for (int i = 0; i < n; ++i) {
        const double r2 = xyz[3 * i] * xyz[3 * i] + xyz[3 * i + 1] * xyz[3 * i + 1] + xyz[3 * i + 2] * xyz[3 * i + 2];
        rmax = std::max(rmax, std::sqrt(r2));
    }
    rmax = rmax * (1.0 + 1e-9) + 1e-9;
    long lo = (long)std::floor((-rmax - zero_h) / h) - 2;
    long hi = (long)std::floor((rmax - zero_h) / h) + 0;
    lo = std::max(lo, 0L);
    hi = std::min(hi, (long)N - 1);
    // a multiple of 8 cells (whole MMA chunks); on a box grid whose Nx is
    // not one, the window may run past Nx: those rows hold no entries
    // (the ligand's cells lie in [lo, hi]) and their circulant index wraps
    const int n_pad8 = (N + 7) / 8 * 8;
    int W = (int)((hi - lo + 1 + 7) / 8 * 8);
    if (W > n_pad8) W = n_pad8;
    long x0 = lo;
    if (x0 + W > N) x0 = std::max(0L, (long)N - W);
    t.x0 = (int)x0;
    t.W = W;
    // rows of the transposed entries: each non-empty term's range padded to 8
    std::vector<int32_t> cnt(K, 0);
    for (int i = 0; i < n; ++i) ++cnt[term[i]];
    std::vector<int32_t> starts, ids;
    t.tpad.assign(K, 0);
    int run = 0, prun = 0;
    for (int k = 0; k < K; ++k) {
        if (cnt[k] == 0) continue;
        starts.push_back(prun);
        ids.push_back(k);
        t.tpad[k] = prun - run;
        run += cnt[k];
        prun += (cnt[k] + 7) / 8 * 8;
    }
    starts.push_back(prun);
    t.ka = (int)ids.size();
    t.n_pad = prun;
    t.info = starts;
    t.info.insert(t.info.end(), ids.begin(), ids.end());
    t.ok = W / 8 <= kTcMaxChunks && t.ka <= kTcMaxTerms && t.ka >= 1 &&
           cubic_tc_smem(N, W / 8, t.ka) <= kMaxSmem;
    return t;
}

// Inputs of a scan held by a ready context, for entry points that bring
// their own work memory.
int ctx_scan_inputs(fftdock_ctx* ctx, ScanInputs* in) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    in->args = batch_args(ctx);
    in->ops = ctx->ops;
    in->device = ctx->cfg.device;
    in->stream = ctx->stream;
    in->N = ctx->N;
    in->K = ctx->K;
    in->PP = ctx->PP;
    in->B = ctx->B;
    in->n_ent = ctx->n_ent;
    in->noalloc_scratch = ctx->noalloc_scratch;
    in->box = ctx->box;
    return FFTDOCK_OK;
}

int ctx_fail(fftdock_ctx* ctx, int code, const char* msg) { return fail(ctx, code, msg); }

}  // namespace fftdock

extern "C" {

void fftdock_config_init(fftdock_config* cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->struct_size = (int32_t)sizeof(fftdock_config);
    cfg->grid_n = 128;
    cfg->grid_step = 1.2;
    cfg->term_set = FFTDOCK_TERMS_SHAPE_ACE;
    cfg->peaks_per_rot = 4;
    cfg->max_trans_inp = 10000;
    cfg->max_val_corr = INFINITY;
    cfg->rot_batch = 64;
    cfg->precision = FFTDOCK_PREC_FP32;
    cfg->device = 0;
    cfg->n_types = 18;
    cfg->ace_matrix = nullptr;
    cfg->shape_core_radius = 2.2;
    cfg->shape_surface_width = 1.8;
    cfg->ace_b = 7.0;
    cfg->ace_k = 0.15;
    cfg->ace_a = 0.6;
    cfg->ace_cut = 6.0;
    cfg->cluster_trans = 0;
    cfg->cluster_order = FFTDOCK_CLUSTER_ORDER_REFERENCE;
    cfg->cluster_radius = 5.0;
    cfg->lj_mix = 1;
    cfg->lj_cut = 9.0;
}

int fftdock_supported_grid(int32_t n) { return fftdock::size_ops(n) != nullptr ? 1 : 0; }

int fftdock_find_best_size(int32_t start_n, int32_t* result) {
    if (!result) return FFTDOCK_EINVAL;
    static const int primes[6] = {2, 3, 5, 7, 11, 13};
    for (long n = start_n <= 1 ? 2 : start_n; n < 2147483647L; ++n) {
        long rem = n;
        int e[6] = {0, 0, 0, 0, 0, 0};
        for (int i = 0; i < 6 && rem != 1; ++i)
            while (rem % primes[i] == 0) { rem /= primes[i]; ++e[i]; }
        if (rem == 1 && e[4] + e[5] <= 1) {
            *result = (int32_t)n;
            return FFTDOCK_OK;
        }
    }
    return FFTDOCK_EINVAL;
}

const char* fftdock_last_error(const fftdock_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int fftdock_grid_n(const fftdock_ctx* ctx) { return ctx ? ctx->N : 0; }

int fftdock_grid_dims(const fftdock_ctx* ctx, int32_t* dims3) {
    if (!ctx || !dims3) return FFTDOCK_EINVAL;
    for (int d = 0; d < 3; ++d) dims3[d] = ctx->dims[d];
    return FFTDOCK_OK;
}

int fftdock_supported_dims(int32_t nx, int32_t ny, int32_t nz) {
    if (nx == ny && ny == nz && fftdock::size_ops(nx)) return 1;
    const int n[3] = {nx, ny, nz};
    for (int d = 0; d < 3; ++d) {
        fftdock::BoxPlan pl;
        if (n[d] < fftdock::kBoxMin || n[d] > fftdock::kBoxMax || !fftdock::box_plan(n[d], &pl)) return 0;
    }
    return 1;
}

int fftdock_get_scan_info(const fftdock_ctx* ctx, fftdock_scan_info* out) {
    if (!ctx || !out) return FFTDOCK_EINVAL;
    out->grid_n = ctx->N;
    out->n_terms = ctx->K;
    out->pencil_path = ctx->use_tc && ctx->tc_ready ? FFTDOCK_PENCIL_TENSOR : FFTDOCK_PENCIL_FFT;
    out->rot_batch = ctx->B;
    out->n_entries = ctx->have_lig ? ctx->n_ent : 0;
    out->window_x0 = ctx->x0;
    out->window_w = ctx->W;
    return FFTDOCK_OK;
}
int fftdock_n_terms(const fftdock_ctx* ctx) { return ctx ? ctx->K : 0; }

void fftdock_destroy(fftdock_ctx* ctx) {
    if (!ctx) return;
    dfree(ctx->tw32);
    dfree(ctx->tw64);
    dfree(ctx->btw32);
    dfree(ctx->btw64);
    dfree(ctx->spec);
    dfree(ctx->rgrid);
    dfree(ctx->emat);
    dfree(ctx->lig_xyz);
    dfree(ctx->lig_term);
    dfree(ctx->lig_w32);
    dfree(ctx->lig_w64);
    dfree(ctx->ent_w);
    dfree(ctx->ent_idx);
    dfree(ctx->ent);
    dfree(ctx->offs);
    dfree(ctx->g2);
    dfree(ctx->g2t);
    dfree(ctx->cand_v);
    dfree(ctx->cand_i);
    dfree(ctx->rot_all);
    dfree(ctx->status_all);
    dfree(ctx->peaks_all);
    dfree(ctx->npeaks_all);
    dfree(ctx->status_dev);
    dfree(ctx->circ);
    dfree(ctx->cscale);
    dfree(ctx->tc_slots);
    dfree(ctx->ent_t);
    dfree(ctx->tinfo);
    dfree(ctx->tpad);
    dfree(ctx->err_dev);
    dfree(ctx->wide.corr);
    dfree(ctx->wide.hist);
    dfree(ctx->wide.st);
    dfree(ctx->wide.cand);
    dfree(ctx->wide.cnt);
    for (cudaEvent_t ev : ctx->ev_pool) cudaEventDestroy(ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int fftdock_create(const fftdock_config* cfg_in, fftdock_ctx** out) {
    if (!out) return FFTDOCK_EINVAL;
    *out = nullptr;
    fftdock_ctx* ctx = new (std::nothrow) fftdock_ctx();
    if (!ctx) return FFTDOCK_ENOMEM;
    *out = ctx;
    if (!cfg_in) return fail(ctx, FFTDOCK_EINVAL, "null configuration");
    if (cfg_in->struct_size != (int32_t)sizeof(fftdock_config))
        return fail(ctx, FFTDOCK_EINVAL, "fftdock_config.struct_size does not match this library");
    fftdock_config& c = ctx->cfg;
    c = *cfg_in;
    // FFT sizes per axis: a compiled cubic edge runs the cubic kernels, any
    // other sizes the box-grid kernels
    int dims[3] = {c.grid_n, c.grid_n, c.grid_n};
    if (c.grid_nx != 0 || c.grid_ny != 0 || c.grid_nz != 0) {
        dims[0] = c.grid_nx;
        dims[1] = c.grid_ny;
        dims[2] = c.grid_nz;
    }
    const std::string dims_s = std::to_string(dims[0]) + " x " + std::to_string(dims[1]) + " x " +
                               std::to_string(dims[2]);
    if (dims[0] == dims[1] && dims[1] == dims[2]) ctx->ops = fftdock::size_ops(dims[0]);
    if (!ctx->ops) {
        if (!fftdock_supported_dims(dims[0], dims[1], dims[2]))
            return fail(ctx, FFTDOCK_EUNSUPPORTED, "grid " + dims_s + " is not supported: each size must be in [" +
                                                       std::to_string(fftdock::kBoxMin) + ", " +
                                                       std::to_string(fftdock::kBoxMax) +
                                                       "] with no prime factor above 13");
        ctx->ops = fftdock::box_ops();
        ctx->box = true;
        if (c.pencil_mode == FFTDOCK_PENCIL_TENSOR && dims[0] > 2 * fftdock::kTcRot)
            return fail(ctx, FFTDOCK_EUNSUPPORTED,
                        "the tensor-core pencil stage covers x sizes up to 256 (grid " + dims_s + ")");
        if (c.precision != FFTDOCK_PREC_FP32)
            return fail(ctx, FFTDOCK_EUNSUPPORTED, "box grids keep FP32 receptor spectra");
        if (c.cluster_trans || c.peaks_per_rot > fftdock::kKC)
            return fail(ctx, FFTDOCK_EUNSUPPORTED,
                        "box grids keep up to 16 peaks per rotation without clustering (grid " + dims_s + ")");
    }
    if (!(c.grid_step > 0.0) || !std::isfinite(c.grid_step)) return fail(ctx, FFTDOCK_EINVAL, "grid_step must be > 0");
    if (c.peaks_per_rot < 1 || c.peaks_per_rot > FFTDOCK_MAX_PEAKS)
        return fail(ctx, FFTDOCK_EINVAL, "peaks_per_rot must be in [1, " + std::to_string(FFTDOCK_MAX_PEAKS) + "]");
    if (c.max_trans_inp < 1) return fail(ctx, FFTDOCK_EINVAL, "max_trans_inp must be >= 1");
    if (c.rot_batch < 1 || c.rot_batch > 1024) return fail(ctx, FFTDOCK_EINVAL, "rot_batch must be in [1, 1024]");
    if (c.precision != FFTDOCK_PREC_FP32 && c.precision != FFTDOCK_PREC_BF16_SPECTRA)
        return fail(ctx, FFTDOCK_EUNSUPPORTED, "precision mode not built");
    if (std::isnan(c.max_val_corr)) return fail(ctx, FFTDOCK_EINVAL, "max_val_corr is NaN");
    if (c.pencil_mode < FFTDOCK_PENCIL_AUTO || c.pencil_mode > FFTDOCK_PENCIL_TENSOR)
        return fail(ctx, FFTDOCK_EINVAL, "unknown pencil_mode");
    if (c.tc_terms_per_sum < 0 || c.tc_terms_per_sum > fftdock::kTcMaxTerms)
        return fail(ctx, FFTDOCK_EINVAL, "tc_terms_per_sum must be in [0, 64]");
    // the tensor form: cubic edges and box grids with Nx up to 256 (two
    // 128-row output tiles above 128)
    const bool has_tc = ctx->box ? dims[0] <= 2 * fftdock::kTcRot : ctx->ops->has_tc;
    if (c.pencil_mode == FFTDOCK_PENCIL_TENSOR && !has_tc)
        return fail(ctx, FFTDOCK_EUNSUPPORTED, "the tensor-core pencil stage covers grid edges up to 256");
    // AUTO runs the tensor form where it is the faster one with many terms:
    // cubic edges up to 128 (one 128-row x tile; at 144 the second tile is
    // 7/8 empty and the FFT form wins) and every box grid it covers (the box
    // FFT pencil kernel is the generic runtime-radix one).  The FFT form
    // keeps the more accurate FP32 candidate values.
    const bool lj_set = c.term_set == FFTDOCK_TERMS_LJ_COMP || c.term_set == FFTDOCK_TERMS_LJ_AVG;
    const int k_terms = c.term_set == FFTDOCK_TERMS_SHAPE_ACE ? c.n_types : 1;
    const bool tc_faster = ctx->box || dims[0] <= fftdock::kTcRot;
    ctx->use_tc = c.pencil_mode == FFTDOCK_PENCIL_TENSOR ||
                  (c.pencil_mode == FFTDOCK_PENCIL_AUTO && has_tc && tc_faster && !lj_set &&
                   c.precision == FFTDOCK_PREC_FP32 && k_terms >= fftdock::kTcMinTerms);
    if (!(c.shape_core_radius >= 0.0) || !(c.shape_surface_width >= 0.0))
        return fail(ctx, FFTDOCK_EINVAL, "shape radii must be >= 0");
    if (c.cluster_trans != 0 && c.cluster_trans != 1) return fail(ctx, FFTDOCK_EINVAL, "cluster_trans must be 0 or 1");
    if (c.cluster_trans) {
        if (c.max_trans_inp > FFTDOCK_MAX_QUEUE_CLUSTERED)
            return fail(ctx, FFTDOCK_EINVAL, "with cluster_trans, max_trans_inp must be <= " +
                                                 std::to_string(FFTDOCK_MAX_QUEUE_CLUSTERED));
        if (c.cluster_order != FFTDOCK_CLUSTER_ORDER_REFERENCE && c.cluster_order != FFTDOCK_CLUSTER_ORDER_BEST_FIRST)
            return fail(ctx, FFTDOCK_EINVAL, "unknown cluster_order");
        if (!(c.cluster_radius >= 0.0) || !std::isfinite(c.cluster_radius))
            return fail(ctx, FFTDOCK_EINVAL, "cluster_radius must be finite and >= 0");
    }
    if (c.term_set == FFTDOCK_TERMS_SHAPE) {
        ctx->K = 1;
    } else if (c.term_set == FFTDOCK_TERMS_SHAPE_ACE) {
        if (c.n_types < 1 || c.n_types > 32) return fail(ctx, FFTDOCK_EINVAL, "n_types must be in [1, 32]");
        if (!c.ace_matrix) return fail(ctx, FFTDOCK_EINVAL, "ace_matrix is required for the shape+ACE term set");
        if (!(c.ace_cut > 0.0)) return fail(ctx, FFTDOCK_EINVAL, "ace_cut must be > 0");
        ctx->ace.assign(c.ace_matrix, c.ace_matrix + (size_t)c.n_types * c.n_types);
        for (double v : ctx->ace)
            if (!std::isfinite(v)) return fail(ctx, FFTDOCK_EINVAL, "ace_matrix has a non-finite entry");
        ctx->K = c.n_types;
    } else if (c.term_set == FFTDOCK_TERMS_LJ_COMP || c.term_set == FFTDOCK_TERMS_LJ_AVG) {
        if (c.lj_mix != 0 && c.lj_mix != 1) return fail(ctx, FFTDOCK_EINVAL, "lj_mix must be 0 or 1");
        if (c.term_set == FFTDOCK_TERMS_LJ_COMP && c.lj_mix != 1)
            return fail(ctx, FFTDOCK_EINVAL, "ljComp requires the geometric sigma rule (lj_mix 1)");
        if (!(c.lj_cut > 0.0) || !std::isfinite(c.lj_cut)) return fail(ctx, FFTDOCK_EINVAL, "lj_cut must be > 0");
        if (c.pencil_mode == FFTDOCK_PENCIL_TENSOR)
            return fail(ctx, FFTDOCK_EUNSUPPORTED, "the LJ term sets run with the FFT pencil stage");
        if (c.precision != FFTDOCK_PREC_FP32)
            return fail(ctx, FFTDOCK_EUNSUPPORTED, "the LJ term sets keep FP32 receptor spectra");
        ctx->K = c.term_set == FFTDOCK_TERMS_LJ_COMP ? 2 : 1;
        ctx->lj = true;
    } else {
        return fail(ctx, FFTDOCK_EINVAL, "unknown term_set");
    }
    c.ace_matrix = nullptr;
    const int N = dims[0];
    ctx->N = N;
    for (int d = 0; d < 3; ++d) ctx->dims[d] = dims[d];
    ctx->H = dims[2] / 2 + 1;
    ctx->PP = ctx->box ? (dims[1] * ctx->H + 31) / 32 * 32 : fftdock::pencil_pitch(N);
    ctx->V = (size_t)dims[0] * dims[1] * dims[2];
    ctx->B = c.rot_batch;
    // the tensor stage takes rotations in groups of 128
    if (ctx->use_tc) ctx->B = (ctx->B + fftdock::kTcRot - 1) / fftdock::kTcRot * fftdock::kTcRot;
    ctx->G = group_size(ctx->B);
    // centred geometry exactly as UniformCubicGeometry(step, logicalSize)
    const double h = c.grid_step;
    const double s_size = h + h * (double)(N - 1);
    const double zero = (-1.0 * s_size) / 2.0;
    ctx->h = h;
    ctx->zero_h = zero - h;
    ctx->center0 = zero + h / 2.0;
    ctx->geo = fftdock::make_geo(h, dims[0], dims[1], dims[2]);

    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(ctx, FFTDOCK_ECUDA, "no CUDA device available");
    if (c.device < 0 || c.device >= ndev) return fail(ctx, FFTDOCK_EINVAL, "device ordinal out of range");
    fftdock::DeviceScope dev_scope(c.device);
    CK(dev_scope.status());
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, c.device));
    if (prop.major != 10 || prop.minor != 3)
        return fail(ctx, FFTDOCK_EUNSUPPORTED, std::string("libfftdock is built for sm_103a only; device is ") +
                                                   prop.name);
    CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    // commit the no-allocation scan's array and load the kernels it runs now,
    // so that its calls allocate nothing
    CK(fftdock::noalloc_scratch_address(&ctx->noalloc_scratch));
    CK(ctx->ops->load_fft_form(c.precision == FFTDOCK_PREC_BF16_SPECTRA ? 1 : 0));

    std::vector<float2> tw32(N);
    std::vector<double2> tw64(N);
    for (int k = 0; k < N; ++k) {
        const double cr = fftdock::cos2pi(k, N), si = -fftdock::sin2pi(k, N);
        tw32[k] = make_float2((float)cr, (float)si);
        tw64[k] = make_double2(cr, si);
    }
    CK(dalloc(&ctx->tw32, N));
    CK(dalloc(&ctx->tw64, N));
    CK(cudaMemcpy(ctx->tw32, tw32.data(), N * sizeof(float2), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->tw64, tw64.data(), N * sizeof(double2), cudaMemcpyHostToDevice));
    if (ctx->box) {
        // one table per axis, e^{-2 pi i k / n_d}, concatenated [Nx | Ny | Nz]
        const int nt = dims[0] + dims[1] + dims[2];
        std::vector<float2> b32;
        std::vector<double2> b64;
        for (int d = 0; d < 3; ++d)
            for (int k = 0; k < dims[d]; ++k) {
                const double cr = fftdock::cos2pi(k, dims[d]), si = -fftdock::sin2pi(k, dims[d]);
                b32.push_back(make_float2((float)cr, (float)si));
                b64.push_back(make_double2(cr, si));
            }
        CK(dalloc(&ctx->btw32, nt));
        CK(dalloc(&ctx->btw64, nt));
        CK(cudaMemcpy(ctx->btw32, b32.data(), nt * sizeof(float2), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->btw64, b64.data(), nt * sizeof(double2), cudaMemcpyHostToDevice));
    }
    if (!ctx->ace.empty()) {
        CK(dalloc(&ctx->emat, ctx->ace.size()));
        CK(cudaMemcpy(ctx->emat, ctx->ace.data(), ctx->ace.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    {
        const size_t elem = c.precision == FFTDOCK_PREC_BF16_SPECTRA ? 4 : 8;
        unsigned char* sp = nullptr;
        CK(dalloc(&sp, (size_t)ctx->K * N * ctx->PP * elem));
        ctx->spec = sp;
    }
    CK(dalloc(&ctx->rgrid, (size_t)ctx->K * ctx->V));
    CK(dalloc(&ctx->offs, (size_t)ctx->G * (ctx->K * N + 1)));
    CK(dalloc(&ctx->g2, (size_t)ctx->B * N * ctx->PP));
    // pencils (ky, kz) and the x extent of the tensor stage's x-quads
    const size_t n_pencils = (size_t)dims[1] * ctx->H;
    const size_t nx_quads = (size_t)(dims[0] + 3) / 4 * 4;
    if (ctx->use_tc) CK(dalloc(&ctx->g2t, (size_t)ctx->B * nx_quads * n_pencils));
    CK(dalloc(&ctx->cand_v, (size_t)ctx->G * N * fftdock::kKC));
    CK(dalloc(&ctx->cand_i, (size_t)ctx->G * N * fftdock::kKC));
    CK(dalloc(&ctx->err_dev, 1));
    CK(cudaMemset(ctx->err_dev, 0, sizeof(int)));
    if (ctx->use_tc) {
        CK(dalloc(&ctx->circ, (size_t)ctx->K * n_pencils * dims[0]));
        CK(dalloc(&ctx->cscale, n_pencils));
        CK(fftdock::tc_slot_count(&ctx->tc_n_slots));
        CK(dalloc(&ctx->tc_slots, (size_t)ctx->tc_n_slots * fftdock::kTcRot * 128));
    }
    // more peaks per rotation than the per-plane pools hold: the exact-queue
    // path, without clustering, over the first peaks_per_rot + 16 cells of
    // the queue (CorrelationProcessor's queue of maxNTransInp cells, of which
    // getTranValuesFilled keeps the first maxNTrans; docking_fft.hpp:430-468)
    const bool deep = !c.cluster_trans && c.peaks_per_rot > fftdock::kKC;
    if (c.cluster_trans || deep) {
        fftdock::WideArgs& w = ctx->wide;
        CK(dalloc(&w.corr, (size_t)ctx->B * ctx->V));
        CK(dalloc(&w.hist, (size_t)ctx->B * fftdock::kWideBins));
        CK(dalloc(&w.st, (size_t)ctx->B));
        CK(dalloc(&w.cand, (size_t)ctx->B * fftdock::kWideMax));
        CK(dalloc(&w.cnt, (size_t)ctx->B));
        w.m = deep ? std::min(c.max_trans_inp, c.peaks_per_rot + fftdock::kKC) : c.max_trans_inp;
        w.order = deep ? fftdock::kWideNoClustering : c.cluster_order;
        // ClusterMatrix::cluster: cutoff2 = r^2 * 3 columns, cutoff = sqrt,
        // compared as cutoff * cutoff (Geom/cluster.hpp:153-156)
        const double cut = std::sqrt((c.cluster_radius * c.cluster_radius) * 3.0);
        w.rad2 = cut * cut;
    }
    return FFTDOCK_OK;
}

int fftdock_set_receptor(fftdock_ctx* ctx, int32_t n, const double* xyz, const int32_t* type) {
    if (!ctx) return FFTDOCK_EINVAL;
    if (!ctx->ops) return fail(ctx, FFTDOCK_ESTATE, "context was not created successfully");
    if (ctx->lj) return fail(ctx, FFTDOCK_EINVAL, "the LJ term sets take their atoms through fftdock_set_pair_lj");
    if (n < 0 || (n > 0 && !xyz)) return fail(ctx, FFTDOCK_EINVAL, "bad receptor atom arrays");
    if (!finite3(xyz, n)) return fail(ctx, FFTDOCK_EINVAL, "receptor coordinates must be finite");
    const fftdock_config& c = ctx->cfg;
    const bool ace = c.term_set == FFTDOCK_TERMS_SHAPE_ACE;
    if (ace) {
        if (n > 0 && !type) return fail(ctx, FFTDOCK_EINVAL, "receptor atom types are required");
        for (int i = 0; i < n; ++i)
            if (type[i] < 0 || type[i] >= c.n_types) return fail(ctx, FFTDOCK_EINVAL, "receptor type out of range");
    }
    fftdock::DeviceScope dev_scope(c.device);
    CK(dev_scope.status());
    ctx->have_rec = false;
    const int N = ctx->N;
    const size_t V = ctx->V;
    cudaStream_t s = ctx->stream;
    const fftdock::Geo g = ctx->geo;
    double* d_xyz = nullptr;
    int32_t* d_type = nullptr;
    int* flags = nullptr;
    double* dens = nullptr;
    double2* cbuf = nullptr;
    double2* hbuf = nullptr;
    int* bin_start = nullptr;
    int* bin_atoms = nullptr;
    int* box = nullptr;
    int rc = FFTDOCK_OK;
    auto cleanup = [&]() {
        cudaStreamSynchronize(s);
        dfree(d_xyz);
        dfree(d_type);
        dfree(flags);
        dfree(dens);
        dfree(cbuf);
        dfree(hbuf);
        dfree(bin_start);
        dfree(bin_atoms);
        dfree(box);
    };
#define CKR(expr)                                 \
    do {                                          \
        cudaError_t e_ = (expr);                  \
        if (e_ != cudaSuccess) {                  \
            rc = cuda_fail(ctx, e_, #expr);       \
            cleanup();                            \
            return rc;                            \
        }                                         \
    } while (0)
    CKR(dalloc(&d_xyz, (size_t)n * 3));
    CKR(dalloc(&d_type, (size_t)n));
    CKR(dalloc(&flags, V));
    if (n > 0) {
        CKR(cudaMemcpyAsync(d_xyz, xyz, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice, s));
        if (ace) CKR(cudaMemcpyAsync(d_type, type, (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    }
    fftdock::HostAtomBins hb;
    if (ace) {
        CKR(dalloc(&dens, (size_t)c.n_types * V));
        fftdock::bin_atoms(xyz, n, c.ace_cut, hb);
        CKR(dalloc(&bin_start, hb.start.size()));
        CKR(dalloc(&bin_atoms, hb.atoms.size()));
        CKR(dalloc(&box, (size_t)6 * n));
        CKR(cudaMemcpyAsync(bin_start, hb.start.data(), hb.start.size() * sizeof(int), cudaMemcpyHostToDevice, s));
        if (n > 0)
            CKR(cudaMemcpyAsync(bin_atoms, hb.atoms.data(), hb.atoms.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    }
    {
        fftdock::ReceptorGridArgs ra{};
        ra.xyz = d_xyz;
        ra.type = d_type;
        ra.n = n;
        for (int d = 0; d < 3; ++d) {
            ra.bins.lo[d] = hb.lo[d];
            ra.bins.nb[d] = hb.nb[d];
        }
        ra.bins.size = hb.size;
        ra.bins.start = bin_start;
        ra.bins.atoms = bin_atoms;
        ra.box = box;
        ra.geo = g;
        ra.term_set = c.term_set;
        ra.n_types = c.n_types;
        ra.K = ctx->K;
        ra.shape_core = c.shape_core_radius;
        ra.shape_width = c.shape_surface_width;
        ra.ace_b = c.ace_b;
        ra.ace_k = c.ace_k;
        ra.ace_a = c.ace_a;
        ra.ace_cut = c.ace_cut;
        ra.emat = ctx->emat;
        ra.flags = flags;
        ra.dens = dens;
        ra.rgrid = ctx->rgrid;
        CKR(fftdock::build_receptor_grids(ra, s));
    }
    CKR(dalloc(&cbuf, V));
    CKR(dalloc(&hbuf, (size_t)ctx->dims[0] * ctx->dims[1] * ctx->H));
    for (int t = 0; t < ctx->K; ++t) {
        const size_t elem = c.precision == FFTDOCK_PREC_BF16_SPECTRA ? 4 : 8;
        void* spec_t = static_cast<unsigned char*>(ctx->spec) + (size_t)t * N * ctx->PP * elem;
        // the tensor stage's circulant samples of term t: [pencils][Nx]
        float2* circ_t = ctx->use_tc ? ctx->circ + (size_t)t * ctx->dims[1] * ctx->H * ctx->dims[0] : nullptr;
        if (ctx->box)
            CKR(fftdock::box_receptor_fft(ctx->rgrid + (size_t)t * V, cbuf, hbuf, ctx->btw64, ctx->dims, spec_t,
                                          ctx->PP, circ_t, s));
        else
            CKR(ctx->ops->receptor_fft(ctx->rgrid + (size_t)t * V, cbuf, hbuf, ctx->tw64, spec_t,
                                       c.precision == FFTDOCK_PREC_BF16_SPECTRA ? 1 : 0, ctx->PP, circ_t, s));
    }
    if (ctx->use_tc) {
        if (ctx->box)
            CKR(fftdock::box_circ_scales(ctx->circ, ctx->K, ctx->dims[1] * ctx->H, ctx->dims[0], ctx->cscale, s));
        else
            CKR(ctx->ops->circ_scales(ctx->circ, ctx->K, ctx->cscale, s));
    }
    CKR(cudaStreamSynchronize(s));
    cleanup();
#undef CKR
    ctx->have_rec = true;
    return FFTDOCK_OK;
}

int fftdock_set_ligand(fftdock_ctx* ctx, int32_t n, const double* xyz, const int32_t* type) {
    if (!ctx) return FFTDOCK_EINVAL;
    if (!ctx->ops) return fail(ctx, FFTDOCK_ESTATE, "context was not created successfully");
    if (ctx->lj) return fail(ctx, FFTDOCK_EINVAL, "the LJ term sets take their atoms through fftdock_set_pair_lj");
    if (n < 1 || !xyz) return fail(ctx, FFTDOCK_EINVAL, "the ligand needs at least one atom");
    if (n > fftdock::kMaxEntries) return fail(ctx, FFTDOCK_EINVAL, "ligand has more than 32768 atoms");
    if (!finite3(xyz, n)) return fail(ctx, FFTDOCK_EINVAL, "ligand coordinates must be finite");
    const fftdock_config& c = ctx->cfg;
    std::vector<int32_t> term(n, 0);
    if (c.term_set == FFTDOCK_TERMS_SHAPE_ACE) {
        if (!type) return fail(ctx, FFTDOCK_EINVAL, "ligand atom types are required");
        for (int i = 0; i < n; ++i) {
            if (type[i] < 0 || type[i] >= c.n_types) return fail(ctx, FFTDOCK_EINVAL, "ligand type out of range");
            term[i] = type[i];
        }
    }
    const size_t smem = ctx->box ? fftdock::box_pencil_smem(ctx->dims[0], ctx->dims[1], ctx->dims[2], ctx->K, n, false)
                                 : ctx->ops->pencil_smem(ctx->K, n);
    if (smem > fftdock::kMaxSmem)
        return fail(ctx, FFTDOCK_EINVAL, "ligand too large for the pencil kernel's shared memory");
    fftdock::DeviceScope dev_scope(c.device);
    CK(dev_scope.status());
    ctx->have_lig = false;
    CK(cudaStreamSynchronize(ctx->stream));
    dfree(ctx->lig_xyz);
    dfree(ctx->lig_term);
    dfree(ctx->ent);
    CK(dalloc(&ctx->lig_xyz, (size_t)n * 3));
    CK(dalloc(&ctx->lig_term, (size_t)n));
    CK(dalloc(&ctx->ent, (size_t)ctx->G * n));
    CK(cudaMemcpy(ctx->lig_xyz, xyz, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->lig_term, term.data(), (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice));
    fftdock::TcTables tt = fftdock::tc_tables(xyz, term.data(), n, ctx->K, ctx->N, ctx->h, ctx->zero_h);
    // box grids: the tensor stage's phase tables grow with Ny + Nz
    if (ctx->box && tt.ok && fftdock::box_tc_smem(ctx->dims, tt.W / 8, tt.ka) > fftdock::kMaxSmem) tt.ok = false;
    ctx->x0 = tt.x0;
    ctx->W = tt.W;
    ctx->n_ent = n;
    // tensor stage: entry ranges of the non-empty terms (the same in every
    // rotation: entries are sorted by term first)
    ctx->tc_ready = false;
    dfree(ctx->ent_t);
    dfree(ctx->tinfo);
    dfree(ctx->tpad);
    if (ctx->use_tc && tt.ok) {
        // 16 spare rows of 128 at the end: the tensor stage's loads run up
        // to 16 rows past a range
        const size_t n_t = (size_t)ctx->G * tt.n_pad + 16 * fftdock::kTcRot;
        CK(dalloc(&ctx->ent_t, n_t));
        CK(fftdock::fill_padding(ctx->ent_t, tt.W, n_t, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        CK(dalloc(&ctx->tinfo, tt.info.size()));
        CK(dalloc(&ctx->tpad, tt.tpad.size()));
        CK(cudaMemcpy(ctx->tinfo, tt.info.data(), tt.info.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->tpad, tt.tpad.data(), tt.tpad.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        ctx->n_tc_terms = tt.ka;
        ctx->n_pad = tt.n_pad;
        ctx->tc_ready = true;
    }
    ctx->have_lig = true;
    return FFTDOCK_OK;
}

// per receptor atom (as6, 4es6, 4es12, fshift, gshift) of its LJ field, in
// the reference's operation order (SoftCoreLJRep/SoftCoreLJAttr for ljComp,
// potentials_inc.hpp:247-354; SoftCoreLJ with CUT_POLICY_SHIFT_FORCE for
// ljAvg, :142-245; parameters as MolForceLJComp / MolForceLJ combine them,
// docking_molforce.hpp:375-600)
static double lj_pow3(double x) { return (x * x) * x; }
static double lj_pow6(double x) {
    const double t = (x * x) * x;
    return t * t;
}
static double lj_mean(const double* v, int n) {
    double t = 0.0;
    for (int i = 0; i < n; ++i) t = t + v[i];
    return t / (double)n;
}

int fftdock_set_pair_lj(fftdock_ctx* ctx, int32_t n_rec, const double* rec_xyz, const double* rec_sigma,
                                   const double* rec_eps, const double* rec_alpha, int32_t n_lig,
                                   const double* lig_xyz, const double* lig_sigma, const double* lig_eps) {
    if (!ctx) return FFTDOCK_EINVAL;
    if (!ctx->ops) return fail(ctx, FFTDOCK_ESTATE, "context was not created successfully");
    if (!ctx->lj) return fail(ctx, FFTDOCK_EINVAL, "fftdock_set_pair_lj needs an LJ term set");
    if (n_rec < 0 || (n_rec > 0 && (!rec_xyz || !rec_sigma || !rec_eps || !rec_alpha)))
        return fail(ctx, FFTDOCK_EINVAL, "bad receptor arrays");
    if (n_lig < 1 || !lig_xyz || !lig_sigma || !lig_eps) return fail(ctx, FFTDOCK_EINVAL, "bad ligand arrays");
    if (!finite3(rec_xyz, n_rec) || !finite3(lig_xyz, n_lig))
        return fail(ctx, FFTDOCK_EINVAL, "coordinates must be finite");
    for (int i = 0; i < n_rec; ++i)
        if (!(rec_sigma[i] > 0.0) || !(rec_eps[i] >= 0.0) || !(rec_alpha[i] >= 0.0) || !std::isfinite(rec_sigma[i]) ||
            !std::isfinite(rec_eps[i]) || !std::isfinite(rec_alpha[i]))
            return fail(ctx, FFTDOCK_EINVAL, "receptor sigma must be > 0, eps and alpha >= 0, all finite");
    for (int i = 0; i < n_lig; ++i)
        if (!(lig_sigma[i] > 0.0) || !(lig_eps[i] >= 0.0) || !std::isfinite(lig_sigma[i]) || !std::isfinite(lig_eps[i]))
            return fail(ctx, FFTDOCK_EINVAL, "ligand sigma must be > 0, eps >= 0, all finite");
    const fftdock_config& c = ctx->cfg;
    const bool comp = c.term_set == FFTDOCK_TERMS_LJ_COMP;
    const int n_ent = comp ? 2 * n_lig : n_lig;
    if (n_ent > fftdock::kMaxEntries) return fail(ctx, FFTDOCK_EINVAL, "too many ligand entries (2 per atom for ljComp)");
    const size_t smem = ctx->box ? fftdock::box_pencil_smem(ctx->dims[0], ctx->dims[1], ctx->dims[2], ctx->K, n_ent,
                                                            comp)
                                 : ctx->ops->pencil_smem(ctx->K, n_ent) + (comp ? (size_t)n_ent * sizeof(float) : 0);
    if (smem > fftdock::kMaxSmem)
        return fail(ctx, FFTDOCK_EINVAL, "ligand too large for the pencil kernel's shared memory");

    // receptor field constants
    const double sig_l = lj_mean(lig_sigma, n_lig);
    const double eps_l = lj_mean(lig_eps, n_lig);
    const double cut = c.lj_cut, cut2 = cut * cut;
    std::vector<double> lc((size_t)5 * n_rec);
    for (int i = 0; i < n_rec; ++i) {
        double* p = &lc[(size_t)5 * i];
        if (comp) {
            const double sigma = std::sqrt(rec_sigma[i]);
            const double sigma_alpha = std::sqrt(rec_sigma[i] * sig_l);
            const double eps = std::sqrt(rec_eps[i]);
            const double s6 = lj_pow6(sigma);
            p[0] = rec_alpha[i] * lj_pow6(sigma_alpha);
            p[1] = 4. * eps * s6;
            p[2] = p[1] * s6;
            p[3] = 0.0;
            p[4] = 0.0;
        } else {
            const double sigma = c.lj_mix == 0 ? (rec_sigma[i] + sig_l) / 2. : std::sqrt(rec_sigma[i] * sig_l);
            const double eps = std::sqrt(rec_eps[i] * eps_l);
            const double s6 = lj_pow6(sigma);
            const double as6 = rec_alpha[i] * s6;
            const double e6 = 4. * eps * s6;
            const double e12 = e6 * s6;
            const double r6 = lj_pow3(cut2);
            const double A = r6 + as6;
            const double B = s6 / (r6 + as6) - 1.;
            const double C = -6. * (cut2 * cut2) * (e6 * A * B + e12) / lj_pow3(A);
            const double gcut = cut * C + cut * (0.0 / std::sqrt(cut2));
            double fshift = -((e12 / A - e6) / A + 0.0 + 0.0 * std::sqrt(cut2));
            const double gshift = -gcut;
            fshift = fshift - gshift * cut;
            p[0] = as6;
            p[1] = e6;
            p[2] = e12;
            p[3] = fshift;
            p[4] = gshift;
        }
    }
    fftdock::DeviceScope dev_scope(c.device);
    CK(dev_scope.status());
    ctx->have_rec = ctx->have_lig = false;
    CK(cudaStreamSynchronize(ctx->stream));
    const int N = ctx->N;
    const size_t V = ctx->V;
    cudaStream_t s = ctx->stream;
    double* d_xyz = nullptr;
    double* d_lc = nullptr;
    int* bin_start = nullptr;
    int* bin_atoms = nullptr;
    int* box = nullptr;
    double2* cbuf = nullptr;
    double2* hbuf = nullptr;
    int rc = FFTDOCK_OK;
    auto cleanup = [&]() {
        cudaStreamSynchronize(s);
        dfree(d_xyz);
        dfree(d_lc);
        dfree(bin_start);
        dfree(bin_atoms);
        dfree(box);
        dfree(cbuf);
        dfree(hbuf);
    };
#define CKR(expr)                                 \
    do {                                          \
        cudaError_t e_ = (expr);                  \
        if (e_ != cudaSuccess) {                  \
            rc = cuda_fail(ctx, e_, #expr);       \
            cleanup();                            \
            return rc;                            \
        }                                         \
    } while (0)
    fftdock::HostAtomBins hb;
    fftdock::bin_atoms(rec_xyz, n_rec, cut, hb);
    CKR(dalloc(&d_xyz, (size_t)n_rec * 3));
    CKR(dalloc(&d_lc, lc.size()));
    CKR(dalloc(&bin_start, hb.start.size()));
    CKR(dalloc(&bin_atoms, hb.atoms.size()));
    CKR(dalloc(&box, (size_t)6 * n_rec));
    CKR(cudaMemcpyAsync(bin_start, hb.start.data(), hb.start.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    if (n_rec > 0) {
        CKR(cudaMemcpyAsync(d_xyz, rec_xyz, (size_t)n_rec * 3 * sizeof(double), cudaMemcpyHostToDevice, s));
        CKR(cudaMemcpyAsync(d_lc, lc.data(), lc.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        CKR(cudaMemcpyAsync(bin_atoms, hb.atoms.data(), hb.atoms.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    }
    {
        fftdock::ReceptorGridArgs ra{};
        ra.xyz = d_xyz;
        ra.n = n_rec;
        ra.geo = ctx->geo;
        ra.term_set = c.term_set;
        ra.K = ctx->K;
        for (int d = 0; d < 3; ++d) {
            ra.bins.lo[d] = hb.lo[d];
            ra.bins.nb[d] = hb.nb[d];
        }
        ra.bins.size = hb.size;
        ra.bins.start = bin_start;
        ra.bins.atoms = bin_atoms;
        ra.box = box;
        ra.lj_c = d_lc;
        ra.lj_cut = cut;
        ra.rgrid = ctx->rgrid;
        CKR(fftdock::build_receptor_grids(ra, s));
    }
    CKR(dalloc(&cbuf, V));
    CKR(dalloc(&hbuf, (size_t)ctx->dims[0] * ctx->dims[1] * ctx->H));
    for (int t = 0; t < ctx->K; ++t) {
        void* spec_t = static_cast<unsigned char*>(ctx->spec) + (size_t)t * N * ctx->PP * 8;
        if (ctx->box)
            CKR(fftdock::box_receptor_fft(ctx->rgrid + (size_t)t * V, cbuf, hbuf, ctx->btw64, ctx->dims, spec_t,
                                          ctx->PP, nullptr, s));
        else
            CKR(ctx->ops->receptor_fft(ctx->rgrid + (size_t)t * V, cbuf, hbuf, ctx->tw64, spec_t, 0, ctx->PP,
                                       nullptr, s));
    }
    CKR(cudaStreamSynchronize(s));
    cleanup();
#undef CKR

    // ligand entries: one per (atom, term); ljComp weighs each atom into both
    // terms, ljAvg has unit weights (the unweighted path)
    std::vector<double> exyz((size_t)3 * n_ent), w64;
    std::vector<float> w32;
    std::vector<int32_t> term(n_ent, 0);
    for (int k = 0; k < (comp ? 2 : 1); ++k)
        for (int i = 0; i < n_lig; ++i) {
            const int e = k * n_lig + i;
            std::memcpy(&exyz[(size_t)3 * e], lig_xyz + (size_t)3 * i, 3 * sizeof(double));
            term[e] = k;
        }
    if (comp) {
        w64.resize(n_ent);
        w32.resize(n_ent);
        for (int i = 0; i < n_lig; ++i) {
            const double se = std::sqrt(lig_eps[i]);
            w64[i] = se * lj_pow6(lig_sigma[i]);
            w64[n_lig + i] = se * lj_pow3(lig_sigma[i]);
        }
        for (int e = 0; e < n_ent; ++e) w32[e] = (float)w64[e];
    }
    dfree(ctx->lig_xyz);
    dfree(ctx->lig_term);
    dfree(ctx->lig_w32);
    dfree(ctx->lig_w64);
    dfree(ctx->ent);
    dfree(ctx->ent_w);
    dfree(ctx->ent_idx);
    CK(dalloc(&ctx->lig_xyz, exyz.size()));
    CK(dalloc(&ctx->lig_term, (size_t)n_ent));
    CK(dalloc(&ctx->ent, (size_t)ctx->G * n_ent));
    CK(cudaMemcpy(ctx->lig_xyz, exyz.data(), exyz.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->lig_term, term.data(), (size_t)n_ent * sizeof(int32_t), cudaMemcpyHostToDevice));
    if (comp) {
        CK(dalloc(&ctx->lig_w32, (size_t)n_ent));
        CK(dalloc(&ctx->lig_w64, (size_t)n_ent));
        CK(dalloc(&ctx->ent_w, (size_t)ctx->G * n_ent));
        CK(dalloc(&ctx->ent_idx, (size_t)ctx->G * n_ent));
        CK(cudaMemcpy(ctx->lig_w32, w32.data(), (size_t)n_ent * sizeof(float), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(ctx->lig_w64, w64.data(), (size_t)n_ent * sizeof(double), cudaMemcpyHostToDevice));
    }
    ctx->n_ent = n_ent;
    ctx->x0 = 0;
    ctx->W = N;
    ctx->have_rec = ctx->have_lig = true;
    return FFTDOCK_OK;
}

int fftdock_scan(fftdock_ctx* ctx, int32_t n_rot, const double* rot, int32_t first_rot_id, fftdock_peak* peaks,
                 int32_t* n_peaks) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (n_rot < 0 || (n_rot > 0 && (!rot || !peaks || !n_peaks))) return fail(ctx, FFTDOCK_EINVAL, "bad arguments");
    if (n_rot == 0) return FFTDOCK_OK;
    fftdock::DeviceScope dev_scope(ctx->cfg.device);
    CK(dev_scope.status());
    if ((rc = grow_call_buffers(ctx, n_rot))) return rc;
    cudaStream_t s = ctx->stream;
    const int P = ctx->cfg.peaks_per_rot;
    CK(cudaMemcpyAsync(ctx->rot_all, rot, (size_t)n_rot * 9 * sizeof(double), cudaMemcpyHostToDevice, s));
    if ((rc = run_batches(ctx, n_rot, ctx->rot_all, first_rot_id, ctx->peaks_all, ctx->npeaks_all, ctx->status_all,
                          s, nullptr, nullptr, nullptr)))
        return rc;
    CK(cudaMemcpyAsync(peaks, ctx->peaks_all, (size_t)n_rot * P * sizeof(fftdock_peak), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(n_peaks, ctx->npeaks_all, (size_t)n_rot * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    std::vector<int32_t> status(n_rot);
    CK(cudaMemcpyAsync(status.data(), ctx->status_all, (size_t)n_rot * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if ((rc = check_pipeline(ctx))) return rc;
    for (int i = 0; i < n_rot; ++i) {
        if (status[i] != 0)
            return fail(ctx, FFTDOCK_EOUT_OF_GRID,
                        "rotation " + std::to_string(first_rot_id + i) + " moves a ligand atom outside the grid");
    }
    return FFTDOCK_OK;
}

int fftdock_scan_device(fftdock_ctx* ctx, int32_t n_rot, const double* d_rot, int32_t first_rot_id,
                        fftdock_peak* d_peaks, int32_t* d_n_peaks, void* stream) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (n_rot < 0 || (n_rot > 0 && (!d_rot || !d_peaks || !d_n_peaks))) return fail(ctx, FFTDOCK_EINVAL, "bad arguments");
    if (n_rot == 0) return FFTDOCK_OK;
    fftdock::DeviceScope dev_scope(ctx->cfg.device);
    CK(dev_scope.status());
    if ((rc = grow_status(ctx, n_rot))) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    return run_batches(ctx, n_rot, d_rot, first_rot_id, d_peaks, d_n_peaks, ctx->status_dev, s, nullptr, nullptr,
                       nullptr);
}

int fftdock_get_receptor_grid(fftdock_ctx* ctx, int32_t term, double* out) {
    if (!ctx || !out) return FFTDOCK_EINVAL;
    if (!ctx->have_rec) return fail(ctx, FFTDOCK_ESTATE, "fftdock_set_receptor has not been called");
    if (term < 0 || term >= ctx->K) return fail(ctx, FFTDOCK_EINVAL, "term out of range");
    fftdock::DeviceScope dev_scope(ctx->cfg.device);
    CK(dev_scope.status());
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(out, ctx->rgrid + (size_t)term * ctx->V, ctx->V * sizeof(double), cudaMemcpyDeviceToHost));
    return FFTDOCK_OK;
}

int fftdock_correlation_grid(fftdock_ctx* ctx, const double* rot, float* out) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (!rot || !out) return fail(ctx, FFTDOCK_EINVAL, "bad arguments");
    fftdock::DeviceScope dev_scope(ctx->cfg.device);
    CK(dev_scope.status());
    if ((rc = grow_call_buffers(ctx, 1))) return rc;
    cudaStream_t s = ctx->stream;
    float* dbg = nullptr;
    CK(dalloc(&dbg, ctx->V));
    CK(cudaMemcpyAsync(ctx->rot_all, rot, 9 * sizeof(double), cudaMemcpyHostToDevice, s));
    rc = run_batches(ctx, 1, ctx->rot_all, 0, ctx->peaks_all, ctx->npeaks_all, ctx->status_all, s, dbg, nullptr,
                     nullptr);
    cudaError_t e = rc ? cudaSuccess : cudaMemcpyAsync(out, dbg, ctx->V * sizeof(float), cudaMemcpyDeviceToHost, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(dbg);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "copy correlation grid");
    if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "synchronize");
    return FFTDOCK_OK;
}

int fftdock_scan_candidates(fftdock_ctx* ctx, int32_t n_rot, const double* rot, float* values, int32_t* offsets) {
    int rc = check_ready(ctx);
    if (rc) return rc;
    if (n_rot < 1 || !rot || !values || !offsets) return fail(ctx, FFTDOCK_EINVAL, "bad arguments");
    if (ctx->wide.corr)
        return fail(ctx, FFTDOCK_EUNSUPPORTED, "a clustering context keeps no per-plane candidate pools");
    fftdock::DeviceScope dev_scope(ctx->cfg.device);
    CK(dev_scope.status());
    if ((rc = grow_call_buffers(ctx, n_rot))) return rc;
    cudaStream_t s = ctx->stream;
    float* pv = nullptr;
    int32_t* pi = nullptr;
    CK(dalloc(&pv, (size_t)n_rot * fftdock::kKC));
    cudaError_t e = dalloc(&pi, (size_t)n_rot * fftdock::kKC);
    if (e != cudaSuccess) {
        cudaFree(pv);
        return cuda_fail(ctx, e, "alloc candidate pool");
    }
    e = cudaMemcpyAsync(ctx->rot_all, rot, (size_t)n_rot * 9 * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        rc = run_batches(ctx, n_rot, ctx->rot_all, 0, ctx->peaks_all, ctx->npeaks_all, ctx->status_all, s, nullptr,
                         pv, pi);
    if (e == cudaSuccess && !rc)
        e = cudaMemcpyAsync(values, pv, (size_t)n_rot * fftdock::kKC * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && !rc)
        e = cudaMemcpyAsync(offsets, pi, (size_t)n_rot * fftdock::kKC * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(pv);
    cudaFree(pi);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "candidate pool");
    if (e2 != cudaSuccess) return cuda_fail(ctx, e2, "synchronize");
    return FFTDOCK_OK;
}

int fftdock_profile(fftdock_ctx* ctx, int32_t enable) {
    if (!ctx) return FFTDOCK_EINVAL;
    ctx->profiling = enable != 0;
    if (enable) {
        ctx->ev_used = 0;
        ctx->ev_recs.clear();
    }
    return FFTDOCK_OK;
}

int fftdock_get_kernel_stats(fftdock_ctx* ctx, fftdock_kernel_stats* out) {
    if (!ctx || !out) return FFTDOCK_EINVAL;
    std::memset(out, 0, sizeof(*out));
    if (ctx->ev_used == 0) return FFTDOCK_OK;
    fftdock::DeviceScope dev_scope(ctx->cfg.device);
    CK(dev_scope.status());
    CK(cudaEventSynchronize(ctx->ev_pool[ctx->ev_used - 1]));
    for (const auto& r : ctx->ev_recs) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ctx->ev_pool[r.from], ctx->ev_pool[r.to]));
        out->launches[r.stage] += 1;
        out->total_ms[r.stage] += ms;
    }
    return FFTDOCK_OK;
}

int fftdock_write_scan_records(const char* path, int32_t n_rot, const double* rot, int32_t peaks_per_rot,
                               const fftdock_peak* peaks, const int32_t* n_peaks, int32_t append) {
    if (!path || n_rot < 0 || peaks_per_rot < 1 || (n_rot > 0 && (!rot || !peaks || !n_peaks)))
        return FFTDOCK_EINVAL;
    FILE* f = std::fopen(path, append ? "ab" : "wb");
    if (!f) return FFTDOCK_EIO;
    const int32_t sig = 2014011401;
    bool ok = true;
    for (int i = 0; i < n_rot && ok; ++i) {
        const int32_t np = n_peaks[i];
        if (np < 0 || np > peaks_per_rot) { ok = false; break; }
        ok = ok && std::fwrite(&sig, sizeof(sig), 1, f) == 1;
        ok = ok && std::fwrite(rot + (size_t)9 * i, sizeof(double), 9, f) == 9;
        const uint64_t nn = (uint64_t)np;
        ok = ok && std::fwrite(&nn, sizeof(nn), 1, f) == 1;
        for (int j = 0; j < np && ok; ++j) {
            const fftdock_peak& p = peaks[(size_t)i * peaks_per_rot + j];
            const double rec[4] = {p.t[0], p.t[1], p.t[2], p.score};
            ok = std::fwrite(rec, sizeof(double), 4, f) == 4;
        }
    }
    if (std::fclose(f) != 0) ok = false;
    return ok ? FFTDOCK_OK : FFTDOCK_EIO;
}

}  // extern "C"
