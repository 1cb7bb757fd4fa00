// Many docking pairs of uneven grid sizes in one CUDA graph.
//
// The single-pair entry points allocate, copy and synchronise per call; for
// a workload of hundreds of small pairs that host traffic and the launch
// gaps between pairs cost as much as the scans.  fftdock_scan_pairs stages
// every pair's atoms and rotations on the device once, keeps one set of work
// buffers per (queue, grid size), and captures the whole workload -- per pair:
// receptor grids, receptor transforms, ligand binning and the scan batches --
// into one CUDA graph over several streams ("queues", pairs spread by
// longest-processing-time first), launched once.  Grid edges up to 128 run
// the tensor form of the pencil stage under the same rule as the single-pair
// contexts (AUTO: term sets of at least kTcMinTerms terms).  The autotuner picks,
// for each grid size, the pencil-stage form (tensor-core GEMM or radix FFT,
// where AUTO could run either) and the rotations per launch (timed probe
// scans of the pair's own kernels), and the number of queues (timed probe
// graphs over a subset of the pairs).  Each form's radix plan is fixed at
// compile time.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "fft_core.cuh"
#include "fftdock.h"
#include "internal.h"

namespace fftdock {
const SizeOps* size_ops(int n);
}

namespace {

using fftdock::BatchArgs;
using fftdock::SizeOps;

constexpr int kKC = 16;
constexpr int kMaxEntries = 32768;
constexpr size_t kMaxSmem = 227 * 1024;
constexpr int kSizes[FFTDOCK_N_SIZES] = {16, 24, 32, 48, 64, 80, 96, 112, 128, 144};
constexpr int kMaxQueues = 8;

int size_slot(int n) {
    for (int i = 0; i < FFTDOCK_N_SIZES; ++i)
        if (kSizes[i] == n) return i;
    return -1;
}

template <typename T> cudaError_t dalloc(T** p, size_t n) {
    *p = nullptr;
    return cudaMalloc((void**)p, (n ? n : 1) * sizeof(T));
}
template <typename T> void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// per grid size: geometry and twiddles shared by every queue
struct SizeData {
    int N = 0, H = 0, PP = 0;
    size_t V = 0;
    double zero_h = 0, center0 = 0;
    const SizeOps* ops = nullptr;
    float2* tw32 = nullptr;
    double2* tw64 = nullptr;
    int batch = 64;
    int max_lig = 1;
    int max_rec = 1;
    bool tc = false;      // tensor form of the pencil stage (the form that runs)
    bool tc_ok = false;   // the tensor form is available for this edge (the tuner may choose it)
    int max_pad = 16;     // largest padded entry rows per rotation among its pairs
};

// work buffers of one queue for one grid size
struct Work {
    double* rgrid = nullptr;
    void* spec = nullptr;
    int* flags = nullptr;
    double* dens = nullptr;
    double2* cbuf = nullptr;
    double2* hbuf = nullptr;
    uint32_t* ent = nullptr;
    int32_t* offs = nullptr;
    float2* g2 = nullptr;
    float* cand_v = nullptr;
    int32_t* cand_i = nullptr;
    int* err = nullptr;
    int* box = nullptr;
    // tensor form
    float2* circ = nullptr;
    int8_t* cscale = nullptr;
    uint32_t* ent_t = nullptr;
    float2* g2t = nullptr;
    void release() {
        dfree(circ);
        dfree(cscale);
        dfree(ent_t);
        dfree(g2t);
        dfree(box);
        dfree(rgrid);
        if (spec) cudaFree(spec);
        spec = nullptr;
        dfree(flags);
        dfree(dens);
        dfree(cbuf);
        dfree(hbuf);
        dfree(ent);
        dfree(offs);
        dfree(g2);
        dfree(cand_v);
        dfree(cand_i);
        dfree(err);
    }
};

struct Staged {
    double* rec_xyz = nullptr;
    int32_t* rec_type = nullptr;
    double* lig_xyz = nullptr;
    int32_t* lig_term = nullptr;
    double* rot = nullptr;
    fftdock_peak* peaks = nullptr;
    int32_t* npeaks = nullptr;
    int32_t* status = nullptr;
    double* emat = nullptr;
    int* bin_start = nullptr;   // all pairs' cell lists, concatenated
    int* bin_atoms = nullptr;
    int* box = nullptr;         // [sum n_rec][6]
    std::vector<size_t> rec_off, lig_off, rot_off, bin_off;
    std::vector<fftdock::HostAtomBins> bins;
    // tensor form: per pair its window and entry tables (concatenated on the device)
    std::vector<fftdock::TcTables> tct;
    std::vector<size_t> info_off, tpad_off;
    int32_t* tinfo = nullptr;
    int32_t* tpad = nullptr;
    void release() {
        dfree(tinfo);
        dfree(tpad);
        dfree(bin_start);
        dfree(bin_atoms);
        dfree(box);
        dfree(rec_xyz);
        dfree(rec_type);
        dfree(lig_xyz);
        dfree(lig_term);
        dfree(rot);
        dfree(peaks);
        dfree(npeaks);
        dfree(status);
        dfree(emat);
    }
};

struct Run {
    fftdock_config cfg{};
    int K = 1;
    bool ace = false;
    bool tc = false;      // the tensor form where the grid edge allows it
    std::map<int, SizeData> sizes;
    std::vector<std::vector<Work>> work;  // [queue][slot]
    Staged st;
    std::string err;
    // running sums of the tensor stage: shared by every queue (a slot is
    // owned by the CTA holding that SM's tensor-memory half)
    float2* tc_slots = nullptr;
    int tc_n_slots = 0;
    ~Run() {
        dfree(tc_slots);
        for (auto& q : work)
            for (auto& w : q) w.release();
        for (auto& kv : sizes) {
            dfree(kv.second.tw32);
            dfree(kv.second.tw64);
        }
        st.release();
    }
};

thread_local std::string g_pairs_err;

int fail(int code, const std::string& msg) {
    g_pairs_err = msg;
    return code;
}

#define PCK(expr)                                                                              \
    do {                                                                                       \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess) return fail(FFTDOCK_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int alloc_work(Run& r, Work& w, const SizeData& sd, int B) {
    const size_t V = sd.V;
    const int K = r.K, N = sd.N;
    const size_t elem = r.cfg.precision == FFTDOCK_PREC_BF16_SPECTRA ? 4 : 8;
    PCK(dalloc(&w.rgrid, (size_t)K * V));
    {
        unsigned char* sp = nullptr;
        PCK(dalloc(&sp, (size_t)K * N * sd.PP * elem));
        w.spec = sp;
    }
    PCK(dalloc(&w.flags, V));
    if (r.ace) {
        PCK(dalloc(&w.dens, (size_t)r.cfg.n_types * V));
        PCK(dalloc(&w.box, (size_t)6 * sd.max_rec));
    }
    PCK(dalloc(&w.cbuf, V));
    PCK(dalloc(&w.hbuf, (size_t)N * N * sd.H));
    PCK(dalloc(&w.ent, (size_t)B * sd.max_lig));
    PCK(dalloc(&w.offs, (size_t)B * (K * N + 1)));
    PCK(dalloc(&w.g2, (size_t)B * N * sd.PP));
    PCK(dalloc(&w.cand_v, (size_t)B * N * kKC));
    PCK(dalloc(&w.cand_i, (size_t)B * N * kKC));
    PCK(dalloc(&w.err, 1));
    PCK(cudaMemset(w.err, 0, sizeof(int)));
    if (sd.tc) {
        const size_t nh = (size_t)N * sd.H;
        PCK(dalloc(&w.circ, (size_t)K * nh * N));
        PCK(dalloc(&w.cscale, nh));
        PCK(dalloc(&w.g2t, (size_t)B * nh * N));
        // 16 spare rows of 128: the tensor stage's loads run up to 16 rows past a range
        PCK(dalloc(&w.ent_t, (size_t)B * sd.max_pad + 16 * fftdock::kTcRot));
    }
    return FFTDOCK_OK;
}

// enqueue one pair (receptor set-up, then the scan batches) on stream s;
// rot_lo/rot_n select a part of the pair's rotations (probes)
cudaError_t enqueue_pair(Run& r, const fftdock_pair& p, int i, Work& w, const SizeData& sd, int B, int rot_lo,
                         int rot_n, cudaStream_t s) {
    const fftdock_config& c = r.cfg;
    const int N = sd.N;
    const fftdock::Geo g = fftdock::make_geo(c.grid_step, N, N, N);
    fftdock::ReceptorGridArgs ra{};
    ra.xyz = r.st.rec_xyz + 3 * r.st.rec_off[i];
    ra.type = r.ace ? r.st.rec_type + r.st.rec_off[i] : nullptr;
    ra.n = p.n_rec;
    ra.geo = g;
    ra.term_set = c.term_set;
    ra.n_types = c.n_types;
    ra.K = r.K;
    ra.shape_core = c.shape_core_radius;
    ra.shape_width = c.shape_surface_width;
    ra.ace_b = c.ace_b;
    ra.ace_k = c.ace_k;
    ra.ace_a = c.ace_a;
    ra.ace_cut = c.ace_cut;
    ra.emat = r.st.emat;
    if (r.ace) {
        const fftdock::HostAtomBins& hb = r.st.bins[i];
        for (int d = 0; d < 3; ++d) {
            ra.bins.lo[d] = hb.lo[d];
            ra.bins.nb[d] = hb.nb[d];
        }
        ra.bins.size = hb.size;
        ra.bins.start = r.st.bin_start + r.st.bin_off[i];
        ra.bins.atoms = r.st.bin_atoms + r.st.rec_off[i];
        ra.box = w.box;
    }
    ra.flags = w.flags;
    ra.dens = w.dens;
    ra.rgrid = w.rgrid;
    cudaError_t e = fftdock::build_receptor_grids(ra, s);
    if (e != cudaSuccess) return e;
    const bool bf = c.precision == FFTDOCK_PREC_BF16_SPECTRA;
    const size_t elem = bf ? 4 : 8;
    const bool tc = sd.tc && r.st.tct[i].ok;
    const size_t nh = (size_t)N * sd.H;
    for (int t = 0; t < r.K; ++t) {
        e = sd.ops->receptor_fft(w.rgrid + (size_t)t * sd.V, w.cbuf, w.hbuf, sd.tw64,
                                 static_cast<unsigned char*>(w.spec) + (size_t)t * N * sd.PP * elem, bf ? 1 : 0,
                                 sd.PP, tc ? w.circ + (size_t)t * nh * N : nullptr, s);
        if (e != cudaSuccess) return e;
    }
    if (tc) {
        if ((e = sd.ops->circ_scales(w.circ, r.K, w.cscale, s)) != cudaSuccess) return e;
        const fftdock::TcTables& tt = r.st.tct[i];
        // this pair's padding rows (x' = its window width) over the rows its batches use
        e = fftdock::fill_padding(w.ent_t, tt.W, (size_t)B * tt.n_pad + 16 * fftdock::kTcRot, s);
        if (e != cudaSuccess) return e;
    }
    BatchArgs a{};
    a.lig_xyz = r.st.lig_xyz + 3 * r.st.lig_off[i];
    a.lig_term = r.st.lig_term + r.st.lig_off[i];
    a.spec = w.spec;
    a.spec_bf16 = bf ? 1 : 0;
    a.rgrid = w.rgrid;
    a.tw32 = sd.tw32;
    a.n_ent = p.n_lig;
    a.K = r.K;
    a.PP = sd.PP;
    a.h = c.grid_step;
    a.zero_h = sd.zero_h;
    a.center0 = sd.center0;
    a.ent = w.ent;
    a.offs = w.offs;
    a.g2 = w.g2;
    a.cand_v = w.cand_v;
    a.cand_i = w.cand_i;
    a.peak_stride = c.peaks_per_rot;
    a.k_out = std::min(c.peaks_per_rot, c.max_trans_inp);
    a.max_val = c.max_val_corr;
    a.err = w.err;
    if (tc) {
        const fftdock::TcTables& tt = r.st.tct[i];
        a.use_tc = 1;
        a.circ = w.circ;
        a.cscale = w.cscale;
        a.tc_slots = r.tc_slots;
        a.tc_n_slots = r.tc_n_slots;
        a.x0 = tt.x0;
        a.W = tt.W;
        a.ent_t = w.ent_t;
        a.tinfo = r.st.tinfo + r.st.info_off[i];
        a.tpad = r.st.tpad + r.st.tpad_off[i];
        a.n_tc_terms = tt.ka;
        a.n_pad = tt.n_pad;
        a.g2t = w.g2t;
    }
    const size_t ro = r.st.rot_off[i] + rot_lo;
    for (int b0 = 0; b0 < rot_n; b0 += B) {
        const int nb = std::min(B, rot_n - b0);
        a.rot = r.st.rot + 9 * (ro + b0);
        a.n_rot = nb;
        a.status = r.st.status + ro + b0;
        a.peaks = r.st.peaks + (ro + b0) * c.peaks_per_rot;
        a.n_peaks = r.st.npeaks + ro + b0;
        a.first_rot_id = p.first_rot_id + rot_lo + b0;
        if ((e = sd.ops->scan_batch(a, s)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// longest-processing-time assignment of pairs to queues
std::vector<std::vector<int>> assign(const Run& r, const std::vector<int>& ids, const fftdock_pair* pairs,
                                     int queues) {
    std::vector<std::pair<double, int>> cost;
    for (int i : ids) {
        const double n = pairs[i].grid_n;
        cost.push_back({n * n * n * (double)(pairs[i].n_rot + 200) * r.K, i});
    }
    std::stable_sort(cost.begin(), cost.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    std::vector<std::vector<int>> out(queues);
    std::vector<double> load(queues, 0.0);
    for (auto& ci : cost) {
        const int q = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        out[q].push_back(ci.second);
        load[q] += ci.first;
    }
    return out;
}

int ensure_work(Run& r, int queues) {
    while ((int)r.work.size() < queues) r.work.emplace_back(FFTDOCK_N_SIZES);
    for (int q = 0; q < queues; ++q)
        for (auto& kv : r.sizes) {
            Work& w = r.work[q][size_slot(kv.first)];
            if (!w.rgrid) {
                int rc = alloc_work(r, w, kv.second, kv.second.batch);
                if (rc) return rc;
            }
        }
    return FFTDOCK_OK;
}

// capture the given pairs (each fully, or the probe part) over `queues`
// streams into one graph; returns it instantiated
int capture(Run& r, const fftdock_pair* pairs, const std::vector<int>& ids, int queues, bool probe,
            cudaStream_t* streams, cudaEvent_t* evs, cudaGraphExec_t* exec) {
    int rc = ensure_work(r, queues);
    if (rc) return rc;
    const auto plan = assign(r, ids, pairs, queues);
    cudaGraph_t graph = nullptr;
    PCK(cudaStreamBeginCapture(streams[0], cudaStreamCaptureModeRelaxed));
    cudaError_t e = cudaEventRecord(evs[0], streams[0]);
    for (int q = 1; q < queues && e == cudaSuccess; ++q) e = cudaStreamWaitEvent(streams[q], evs[0], 0);
    for (int q = 0; q < queues && e == cudaSuccess; ++q) {
        for (int i : plan[q]) {
            const fftdock_pair& p = pairs[i];
            const SizeData& sd = r.sizes.at(p.grid_n);
            const int n = probe ? std::min(p.n_rot, sd.batch) : p.n_rot;
            e = enqueue_pair(r, p, i, r.work[q][size_slot(p.grid_n)], sd, sd.batch, 0, n, streams[q]);
            if (e != cudaSuccess) break;
        }
    }
    for (int q = 1; q < queues && e == cudaSuccess; ++q) {
        e = cudaEventRecord(evs[q], streams[q]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(streams[0], evs[q], 0);
    }
    cudaError_t e2 = cudaStreamEndCapture(streams[0], &graph);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail(FFTDOCK_ECUDA, std::string("capture of the pair graph: ") +
                                       cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(FFTDOCK_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    return FFTDOCK_OK;
}

int time_graph(cudaGraphExec_t g, cudaStream_t s, cudaEvent_t a, cudaEvent_t b, float* ms) {
    PCK(cudaEventRecord(a, s));
    PCK(cudaGraphLaunch(g, s));
    PCK(cudaEventRecord(b, s));
    PCK(cudaEventSynchronize(b));
    PCK(cudaEventElapsedTime(ms, a, b));
    return FFTDOCK_OK;
}

double host_ms(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

int check_pair(const fftdock_config& c, const fftdock_pair& p, int i, int K, bool ace) {
    const std::string w = "pair " + std::to_string(i) + ": ";
    if (size_slot(p.grid_n) < 0 || !fftdock::size_ops(p.grid_n))
        return fail(FFTDOCK_EUNSUPPORTED, w + "grid_n " + std::to_string(p.grid_n) + " is not built");
    if (p.n_rec < 0 || (p.n_rec > 0 && !p.rec_xyz)) return fail(FFTDOCK_EINVAL, w + "bad receptor arrays");
    if (p.n_lig < 1 || p.n_lig > kMaxEntries || !p.lig_xyz) return fail(FFTDOCK_EINVAL, w + "bad ligand arrays");
    if (p.n_rot < 0 || (p.n_rot > 0 && (!p.rot || !p.peaks || !p.n_peaks)))
        return fail(FFTDOCK_EINVAL, w + "bad rotation or output arrays");
    for (int k = 0; k < 3 * p.n_rec; ++k)
        if (!std::isfinite(p.rec_xyz[k])) return fail(FFTDOCK_EINVAL, w + "receptor coordinates must be finite");
    for (int k = 0; k < 3 * p.n_lig; ++k)
        if (!std::isfinite(p.lig_xyz[k])) return fail(FFTDOCK_EINVAL, w + "ligand coordinates must be finite");
    if (ace) {
        if ((p.n_rec > 0 && !p.rec_type) || !p.lig_type) return fail(FFTDOCK_EINVAL, w + "atom types are required");
        for (int k = 0; k < p.n_rec; ++k)
            if (p.rec_type[k] < 0 || p.rec_type[k] >= c.n_types)
                return fail(FFTDOCK_EINVAL, w + "receptor type out of range");
        for (int k = 0; k < p.n_lig; ++k)
            if (p.lig_type[k] < 0 || p.lig_type[k] >= c.n_types)
                return fail(FFTDOCK_EINVAL, w + "ligand type out of range");
    }
    if (fftdock::size_ops(p.grid_n)->pencil_smem(K, p.n_lig) > kMaxSmem)
        return fail(FFTDOCK_EINVAL, w + "ligand too large for the pencil kernel's shared memory");
    return FFTDOCK_OK;
}

int stage(Run& r, int n_pairs, const fftdock_pair* pairs) {
    Staged& st = r.st;
    size_t nr = 0, nl = 0, no = 0;
    for (int i = 0; i < n_pairs; ++i) {
        st.rec_off.push_back(nr);
        st.lig_off.push_back(nl);
        st.rot_off.push_back(no);
        nr += pairs[i].n_rec;
        nl += pairs[i].n_lig;
        no += pairs[i].n_rot;
    }
    std::vector<double> rx(3 * nr), lx(3 * nl), ro(9 * no);
    std::vector<int32_t> rt(r.ace ? nr : 0), lt(nl, 0);
    for (int i = 0; i < n_pairs; ++i) {
        const fftdock_pair& p = pairs[i];
        std::memcpy(rx.data() + 3 * st.rec_off[i], p.rec_xyz, sizeof(double) * 3 * p.n_rec);
        std::memcpy(lx.data() + 3 * st.lig_off[i], p.lig_xyz, sizeof(double) * 3 * p.n_lig);
        if (p.n_rot) std::memcpy(ro.data() + 9 * st.rot_off[i], p.rot, sizeof(double) * 9 * p.n_rot);
        if (r.ace) {
            std::memcpy(rt.data() + st.rec_off[i], p.rec_type, sizeof(int32_t) * p.n_rec);
            std::memcpy(lt.data() + st.lig_off[i], p.lig_type, sizeof(int32_t) * p.n_lig);
        }
    }
    PCK(dalloc(&st.rec_xyz, rx.size()));
    PCK(dalloc(&st.lig_xyz, lx.size()));
    PCK(dalloc(&st.lig_term, lt.size()));
    PCK(dalloc(&st.rot, ro.size()));
    PCK(dalloc(&st.peaks, no * r.cfg.peaks_per_rot));
    PCK(dalloc(&st.npeaks, no));
    PCK(dalloc(&st.status, no));
    PCK(cudaMemcpy(st.rec_xyz, rx.data(), rx.size() * sizeof(double), cudaMemcpyHostToDevice));
    PCK(cudaMemcpy(st.lig_xyz, lx.data(), lx.size() * sizeof(double), cudaMemcpyHostToDevice));
    PCK(cudaMemcpy(st.lig_term, lt.data(), lt.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    PCK(cudaMemcpy(st.rot, ro.data(), ro.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (r.ace) {
        std::vector<int> bs, ba;
        st.bins.resize(n_pairs);
        for (int i = 0; i < n_pairs; ++i) {
            fftdock::bin_atoms(pairs[i].rec_xyz, pairs[i].n_rec, r.cfg.ace_cut, st.bins[i]);
            st.bin_off.push_back(bs.size());
            bs.insert(bs.end(), st.bins[i].start.begin(), st.bins[i].start.end());
            ba.insert(ba.end(), st.bins[i].atoms.begin(), st.bins[i].atoms.end());
        }
        PCK(dalloc(&st.bin_start, bs.size()));
        PCK(dalloc(&st.bin_atoms, ba.size()));
        PCK(cudaMemcpy(st.bin_start, bs.data(), bs.size() * sizeof(int), cudaMemcpyHostToDevice));
        if (!ba.empty()) PCK(cudaMemcpy(st.bin_atoms, ba.data(), ba.size() * sizeof(int), cudaMemcpyHostToDevice));
        PCK(dalloc(&st.rec_type, rt.size()));
        PCK(cudaMemcpy(st.rec_type, rt.data(), rt.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        const size_t ne = (size_t)r.cfg.n_types * r.cfg.n_types;
        PCK(dalloc(&st.emat, ne));
        PCK(cudaMemcpy(st.emat, r.cfg.ace_matrix, ne * sizeof(double), cudaMemcpyHostToDevice));
    }
    // tensor form: each pair's window and entry tables, for the grid edges that run it
    st.tct.assign(n_pairs, fftdock::TcTables{});
    std::vector<int32_t> info_all, tpad_all;
    for (int i = 0; i < n_pairs; ++i) {
        SizeData& sd = r.sizes[pairs[i].grid_n];
        st.info_off.push_back(info_all.size());
        st.tpad_off.push_back(tpad_all.size());
        if (!sd.tc_ok) continue;
        st.tct[i] = fftdock::tc_tables(pairs[i].lig_xyz, lt.data() + st.lig_off[i], pairs[i].n_lig, r.K, sd.N,
                                      r.cfg.grid_step, sd.zero_h);
        if (!st.tct[i].ok) continue;
        info_all.insert(info_all.end(), st.tct[i].info.begin(), st.tct[i].info.end());
        tpad_all.insert(tpad_all.end(), st.tct[i].tpad.begin(), st.tct[i].tpad.end());
        sd.max_pad = std::max(sd.max_pad, st.tct[i].n_pad);
    }
    if (!info_all.empty()) {
        PCK(dalloc(&st.tinfo, info_all.size()));
        PCK(dalloc(&st.tpad, tpad_all.size()));
        PCK(cudaMemcpy(st.tinfo, info_all.data(), info_all.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        PCK(cudaMemcpy(st.tpad, tpad_all.data(), tpad_all.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    return FFTDOCK_OK;
}

int setup_sizes(Run& r, int n_pairs, const fftdock_pair* pairs) {
    for (int i = 0; i < n_pairs; ++i) {
        SizeData& sd = r.sizes[pairs[i].grid_n];
        sd.max_lig = std::max(sd.max_lig, pairs[i].n_lig);
        sd.max_rec = std::max(sd.max_rec, pairs[i].n_rec);
    }
    for (auto& kv : r.sizes) {
        SizeData& sd = kv.second;
        const int N = kv.first;
        sd.N = N;
        sd.H = N / 2 + 1;
        sd.PP = fftdock::pencil_pitch(N);
        sd.V = (size_t)N * N * N;
        const double h = r.cfg.grid_step;
        const double zero = (-1.0 * (h + h * (double)(N - 1))) / 2.0;
        sd.zero_h = zero - h;
        sd.center0 = zero + h / 2.0;
        sd.ops = fftdock::size_ops(N);
        sd.batch = r.cfg.rot_batch;
        // AUTO keeps the FFT form above 128 (the tensor form's second x tile
        // is mostly empty there); TENSOR asks for it wherever it is built;
        // the autotuner times both forms wherever AUTO could run either
        sd.tc_ok = r.tc && sd.ops->has_tc;
        sd.tc = sd.tc_ok && (r.cfg.pencil_mode == FFTDOCK_PENCIL_TENSOR || N <= fftdock::kTcRot);
        // the tensor form takes rotations in groups of 128
        if (sd.tc) sd.batch = (sd.batch + fftdock::kTcRot - 1) / fftdock::kTcRot * fftdock::kTcRot;
        std::vector<float2> t32(N);
        std::vector<double2> t64(N);
        for (int k = 0; k < N; ++k) {
            const double cr = fftdock::cos2pi(k, N), si = -fftdock::sin2pi(k, N);
            t32[k] = make_float2((float)cr, (float)si);
            t64[k] = make_double2(cr, si);
        }
        PCK(dalloc(&sd.tw32, N));
        PCK(dalloc(&sd.tw64, N));
        PCK(cudaMemcpy(sd.tw32, t32.data(), N * sizeof(float2), cudaMemcpyHostToDevice));
        PCK(cudaMemcpy(sd.tw64, t64.data(), N * sizeof(double2), cudaMemcpyHostToDevice));
    }
    return FFTDOCK_OK;
}

// plan of one grid size: the pencil-stage form (the tensor-core GEMM form or
// the radix-FFT form, both where AUTO could run either) and the rotations
// per launch.  For each candidate, the first pair of that size is timed
// with its set-up alone and with a probe of rotations; the candidate with
// the least set-up + (the pair's rotations x the probe's time per rotation)
// wins.
int tune_batch(Run& r, const fftdock_pair* pairs, int n_pairs, int N, cudaStream_t s, cudaEvent_t a, cudaEvent_t b) {
    static const int cand[] = {32, 64, 128, 256};
    SizeData& sd = r.sizes.at(N);
    int pi = -1;
    for (int i = 0; i < n_pairs && pi < 0; ++i)
        if (pairs[i].grid_n == N && pairs[i].n_rot > 0) pi = i;
    if (pi < 0) return FFTDOCK_OK;
    const int n_probe = std::min(pairs[pi].n_rot, 512);
    double best = 1e300;
    int best_b = sd.batch;
    bool best_tc = sd.tc;
    // the forms to time: both when AUTO could run either and the pair has
    // the tensor form's tables, else the one set up
    const bool both = sd.tc_ok && r.cfg.pencil_mode == FFTDOCK_PENCIL_AUTO && r.st.tct[pi].ok;
    for (int f = 0; f < (both ? 2 : 1); ++f)
    for (int B : cand) {
        const bool tc = both ? f == 0 : sd.tc;
        // rotations per launch: multiples of 128 for the tensor form
        if (B > 1024 || (tc && B % fftdock::kTcRot)) continue;
        Work w;
        SizeData tmp = sd;
        tmp.tc = tc;
        int rc = alloc_work(r, w, tmp, B);
        if (rc) {
            w.release();
            return rc;
        }
        // warm-up (also sets kernel attributes before any capture), then
        // time the set-up alone and with the probe's rotations
        cudaError_t e = enqueue_pair(r, pairs[pi], pi, w, tmp, B, 0, n_probe, s);
        float ms = 0.f, ms0 = 0.f;
        auto timed = [&](int n, float* out) {
            if (e == cudaSuccess) e = cudaEventRecord(a, s);
            if (e == cudaSuccess) e = enqueue_pair(r, pairs[pi], pi, w, tmp, B, 0, n, s);
            if (e == cudaSuccess) e = cudaEventRecord(b, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(b);
            if (e == cudaSuccess) e = cudaEventElapsedTime(out, a, b);
        };
        timed(n_probe, &ms);
        timed(0, &ms0);
        w.release();
        if (e != cudaSuccess) return fail(FFTDOCK_ECUDA, std::string("batch probe: ") + cudaGetErrorString(e));
        const double per = ms0 + (double)pairs[pi].n_rot * std::max(0.0, (double)(ms - ms0)) / n_probe;
        if (per < best * 0.98) {
            best = per;
            best_b = B;
            best_tc = tc;
        }
    }
    sd.batch = best_b;
    sd.tc = best_tc;
    return FFTDOCK_OK;
}

}  // namespace

extern "C" {

const char* fftdock_pairs_last_error(void) { return g_pairs_err.c_str(); }

int fftdock_pair_grid(int32_t n_rec, const double* rec_xyz, int32_t n_lig, const double* lig_xyz, double step,
                      double margin, int32_t* grid_n) {
    if (!grid_n || n_rec < 0 || n_lig < 1 || (n_rec > 0 && !rec_xyz) || !lig_xyz || !(step > 0.0) ||
        !(margin >= 0.0))
        return fail(FFTDOCK_EINVAL, "bad arguments");
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int i = 0; i < n_rec; ++i)
        for (int d = 0; d < 3; ++d) {
            const double v = rec_xyz[3 * i + d];
            if (i == 0 || v < lo[d]) lo[d] = v;
            if (i == 0 || v > hi[d]) hi[d] = v;
        }
    double rr = 0.0, rl = 0.0;
    for (int i = 0; i < n_rec; ++i) {
        double s = 0.0;
        for (int d = 0; d < 3; ++d) {
            const double t = rec_xyz[3 * i + d] - 0.5 * (lo[d] + hi[d]);
            s += t * t;
        }
        rr = std::max(rr, std::sqrt(s));
    }
    for (int i = 0; i < n_lig; ++i) {
        double s = 0.0;
        for (int d = 0; d < 3; ++d) s += lig_xyz[3 * i + d] * lig_xyz[3 * i + d];
        rl = std::max(rl, std::sqrt(s));
    }
    const double need = std::ceil((2.0 * rr + 2.0 * rl + 2.0 * margin) / step);
    for (int n : kSizes)
        if (n >= 48 && n >= need && fftdock::size_ops(n)) {
            *grid_n = n;
            return FFTDOCK_OK;
        }
    return fail(FFTDOCK_EUNSUPPORTED, "the pair needs a grid edge above 144");
}

int fftdock_scan_pairs(const fftdock_config* cfg, int32_t n_pairs, const fftdock_pair* pairs, int32_t tune,
                       fftdock_pairs_report* report) {
    g_pairs_err.clear();
    if (!cfg || n_pairs < 0 || (n_pairs > 0 && !pairs)) return fail(FFTDOCK_EINVAL, "bad arguments");
    if (cfg->struct_size != (int32_t)sizeof(fftdock_config))
        return fail(FFTDOCK_EINVAL, "fftdock_config.struct_size does not match this library");
    Run r;
    r.cfg = *cfg;
    const fftdock_config& c = r.cfg;
    if (c.cluster_trans) return fail(FFTDOCK_EUNSUPPORTED, "translational clustering is not part of the pair batch");
    if (c.pencil_mode < FFTDOCK_PENCIL_AUTO || c.pencil_mode > FFTDOCK_PENCIL_TENSOR)
        return fail(FFTDOCK_EINVAL, "unknown pencil_mode");
    if (c.peaks_per_rot < 1 || c.peaks_per_rot > kKC) return fail(FFTDOCK_EINVAL, "peaks_per_rot must be in [1, 16]");
    if (c.max_trans_inp < 1) return fail(FFTDOCK_EINVAL, "max_trans_inp must be >= 1");
    if (c.rot_batch < 1 || c.rot_batch > 1024) return fail(FFTDOCK_EINVAL, "rot_batch must be in [1, 1024]");
    if (!(c.grid_step > 0.0) || std::isnan(c.max_val_corr)) return fail(FFTDOCK_EINVAL, "bad grid_step or max_val_corr");
    if (c.precision != FFTDOCK_PREC_FP32 && c.precision != FFTDOCK_PREC_BF16_SPECTRA)
        return fail(FFTDOCK_EUNSUPPORTED, "precision mode not built");
    if (c.term_set == FFTDOCK_TERMS_LJ_COMP || c.term_set == FFTDOCK_TERMS_LJ_AVG)
        return fail(FFTDOCK_EUNSUPPORTED, "the LJ term sets are not part of the pair batch");
    if (c.term_set == FFTDOCK_TERMS_SHAPE) {
        r.K = 1;
    } else if (c.term_set == FFTDOCK_TERMS_SHAPE_ACE) {
        if (c.n_types < 1 || c.n_types > 32 || !c.ace_matrix) return fail(FFTDOCK_EINVAL, "bad ACE configuration");
        for (int k = 0; k < c.n_types * c.n_types; ++k)
            if (!std::isfinite(c.ace_matrix[k])) return fail(FFTDOCK_EINVAL, "ace_matrix has a non-finite entry");
        r.K = c.n_types;
        r.ace = true;
    } else {
        return fail(FFTDOCK_EINVAL, "unknown term_set");
    }
    r.tc = c.precision == FFTDOCK_PREC_FP32 &&
           (c.pencil_mode == FFTDOCK_PENCIL_TENSOR ||
            (c.pencil_mode == FFTDOCK_PENCIL_AUTO && r.K >= fftdock::kTcMinTerms));
    for (int i = 0; i < n_pairs; ++i) {
        int rc = check_pair(c, pairs[i], i, r.K, r.ace);
        if (rc) return rc;
    }
    fftdock_pairs_report rep{};
    for (int i = 0; i < FFTDOCK_N_SIZES; ++i) rep.grid_sizes[i] = kSizes[i];
    if (n_pairs == 0) {
        if (report) *report = rep;
        return FFTDOCK_OK;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(FFTDOCK_ECUDA, "no CUDA device available");
    if (c.device < 0 || c.device >= ndev) return fail(FFTDOCK_EINVAL, "device ordinal out of range");
    fftdock::DeviceScope dev_scope(c.device);
    PCK(dev_scope.status());
    cudaDeviceProp prop;
    PCK(cudaGetDeviceProperties(&prop, c.device));
    if (prop.major != 10 || prop.minor != 3)
        return fail(FFTDOCK_EUNSUPPORTED, std::string("libfftdock is built for sm_103a only; device is ") + prop.name);

    const auto t_setup = std::chrono::steady_clock::now();
    if (r.tc) {
        PCK(fftdock::tc_slot_count(&r.tc_n_slots));
        PCK(dalloc(&r.tc_slots, (size_t)r.tc_n_slots * fftdock::kTcRot * 128));
    }
    int rc = setup_sizes(r, n_pairs, pairs);
    if (!rc) rc = stage(r, n_pairs, pairs);
    if (rc) return rc;
    cudaStream_t streams[kMaxQueues] = {};
    cudaEvent_t evs[kMaxQueues] = {};
    cudaEvent_t ta = nullptr, tb = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        for (int q = 0; q < kMaxQueues; ++q) {
            if (streams[q]) cudaStreamDestroy(streams[q]);
            if (evs[q]) cudaEventDestroy(evs[q]);
        }
        if (ta) cudaEventDestroy(ta);
        if (tb) cudaEventDestroy(tb);
    };
    auto run = [&]() -> int {
        for (int q = 0; q < kMaxQueues; ++q) {
            PCK(cudaStreamCreateWithFlags(&streams[q], cudaStreamNonBlocking));
            PCK(cudaEventCreateWithFlags(&evs[q], cudaEventDisableTiming));
        }
        PCK(cudaEventCreate(&ta));
        PCK(cudaEventCreate(&tb));
        int queues = 1;
        std::vector<int> all(n_pairs);
        for (int i = 0; i < n_pairs; ++i) all[i] = i;
        if (!tune && report && report->n_streams > 0) {
            // the plan of an earlier tuned call
            queues = std::min(std::max(1, (int)report->n_streams), kMaxQueues);
            for (auto& kv : r.sizes) {
                const int b = report->rot_batch[size_slot(kv.first)];
                if (b >= 1 && b <= 1024) kv.second.batch = b;
                // the planned pencil form, where AUTO could run either
                const int form = report->pencil_form[size_slot(kv.first)];
                if (kv.second.tc_ok && r.cfg.pencil_mode == FFTDOCK_PENCIL_AUTO &&
                    (form == FFTDOCK_PENCIL_FFT || form == FFTDOCK_PENCIL_TENSOR))
                    kv.second.tc = form == FFTDOCK_PENCIL_TENSOR;
                if (kv.second.tc)
                    kv.second.batch = (kv.second.batch + fftdock::kTcRot - 1) / fftdock::kTcRot * fftdock::kTcRot;
            }
        }
        if (tune) {
            const auto t_tune = std::chrono::steady_clock::now();
            for (auto& kv : r.sizes) {
                int rc2 = tune_batch(r, pairs, n_pairs, kv.first, streams[0], ta, tb);
                if (rc2) return rc2;
            }
            // queues: time probe graphs (every pair's set-up plus one batch)
            static const int qc[] = {1, 2, 4};
            float best = 1e30f;
            for (int q : qc) {
                cudaGraphExec_t g = nullptr;
                int rc2 = capture(r, pairs, all, q, true, streams, evs, &g);
                float ms = 0.f;
                if (!rc2) rc2 = time_graph(g, streams[0], ta, tb, &ms);  // warm
                if (!rc2) rc2 = time_graph(g, streams[0], ta, tb, &ms);
                if (g) cudaGraphExecDestroy(g);
                if (rc2) return rc2;
                if (ms < best * 0.97f) {
                    best = ms;
                    queues = q;
                }
            }
            rep.tune_ms = host_ms(t_tune);
        }
        const auto t_cap = std::chrono::steady_clock::now();
        int rc2 = capture(r, pairs, all, queues, false, streams, evs, &exec);
        if (rc2) return rc2;
        rep.capture_ms = host_ms(t_cap);
        float ms = 0.f;
        rc2 = time_graph(exec, streams[0], ta, tb, &ms);
        if (rc2) return rc2;
        rep.run_ms = ms;
        rep.n_streams = queues;
        for (auto& kv : r.sizes) {
            rep.rot_batch[size_slot(kv.first)] = kv.second.batch;
            rep.pencil_form[size_slot(kv.first)] = kv.second.tc ? FFTDOCK_PENCIL_TENSOR : FFTDOCK_PENCIL_FFT;
        }
        // outputs
        size_t no = 0;
        for (int i = 0; i < n_pairs; ++i) no += pairs[i].n_rot;
        const int P = c.peaks_per_rot;
        std::vector<fftdock_peak> pk(no * P);
        std::vector<int32_t> np(no), stv(no);
        PCK(cudaMemcpy(pk.data(), r.st.peaks, pk.size() * sizeof(fftdock_peak), cudaMemcpyDeviceToHost));
        PCK(cudaMemcpy(np.data(), r.st.npeaks, no * sizeof(int32_t), cudaMemcpyDeviceToHost));
        PCK(cudaMemcpy(stv.data(), r.st.status, no * sizeof(int32_t), cudaMemcpyDeviceToHost));
        int first_bad = -1;
        for (int i = 0; i < n_pairs; ++i) {
            const fftdock_pair& p = pairs[i];
            const size_t o = r.st.rot_off[i];
            for (int k = 0; k < p.n_rot; ++k) {
                p.n_peaks[k] = np[o + k];
                std::memcpy(p.peaks + (size_t)k * P, pk.data() + (o + k) * P, sizeof(fftdock_peak) * P);
                if (stv[o + k] != 0) {
                    ++rep.n_out_of_grid;
                    if (first_bad < 0) first_bad = i;
                }
            }
            rep.rotations += p.n_rot;
        }
        if (first_bad >= 0)
            return fail(FFTDOCK_EOUT_OF_GRID, std::to_string(rep.n_out_of_grid) +
                                                  " rotations place a ligand atom outside the grid (first in pair " +
                                                  std::to_string(first_bad) + "); they report no peaks");
        return FFTDOCK_OK;
    };
    rc = run();
    rep.setup_ms = host_ms(t_setup);
    cleanup();
    if (report) *report = rep;
    return rc;
}

}  // extern "C"
