// Internal declarations shared by the C ABI implementation and the per-size
// kernel translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "fftdock.h"

namespace fftdock {

// Makes a context's device current for one entry point and puts the caller's
// current device back when the entry point returns, so that no call leaves
// the library's device selected on the calling thread (nothing is restored
// when the two are the same device).
class DeviceScope {
  public:
    explicit DeviceScope(int device) : dev_(device) {
        if (cudaGetDevice(&prev_) != cudaSuccess) prev_ = -1;
        err_ = prev_ == device ? cudaSuccess : cudaSetDevice(device);
    }
    ~DeviceScope() {
        if (prev_ >= 0 && prev_ != dev_) cudaSetDevice(prev_);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
    cudaError_t status() const { return err_; }

  private:
    int dev_;
    int prev_ = -1;
    cudaError_t err_ = cudaSuccess;
};

// pencils per x-plane, N (N/2 + 1), rounded up to whole 32-lane tiles
__host__ __device__ constexpr int pencil_pitch(int n) { return (n * (n / 2 + 1) + 31) / 32 * 32; }

// Grid geometry of the reference's centred UniformCubicGeometry
// (include/PRODDL/Grid/gridcoord.hpp:127-191): cubic cells of step h, a
// logical size per axis (fftSize, docking_fft.hpp:541-553), centred per axis.
struct Geo {
    double h;           // step
    double zero_h[3];   // per axis: spatial zero - h (toLogical)
    double center0[3];  // per axis: centre of cell 0 (toSpatial)
    int n[3];           // logical size per axis
};
// UniformCubicGeometry(step, logicalSize): per axis zero = -(h + h (n - 1)) / 2
inline Geo make_geo(double h, int nx, int ny, int nz) {
    Geo g{};
    g.h = h;
    const int n[3] = {nx, ny, nz};
    for (int d = 0; d < 3; ++d) {
        const double s_size = h + h * (double)(n[d] - 1);
        const double zero = (-1.0 * s_size) / 2.0;
        g.zero_h[d] = zero - h;
        g.center0[d] = zero + h / 2.0;
        g.n[d] = n[d];
    }
    return g;
}

// Receptor atoms sorted into cubic bins of edge >= the desolvation cutoff
// (host-built counting sort, atoms in index order inside each bin), so that
// every grid cell gathers its atoms in one fixed order.
struct AtomBins {
    double lo[3];          // corner of bin (0, 0, 0)
    double size;           // bin edge
    int nb[3];             // bins per axis
    const int* start;      // [nbins + 1]
    const int* atoms;      // [n] atom indexes
};
struct HostAtomBins {
    double lo[3] = {0, 0, 0};
    double size = 1.0;
    int nb[3] = {1, 1, 1};
    std::vector<int> start, atoms;
};
void bin_atoms(const double* xyz, int n, double cut, HostAtomBins& out);

struct ReceptorGridArgs {
    const double* xyz;     // [n][3]
    const int32_t* type;   // [n]
    int n;
    AtomBins bins;         // shape+ACE and LJ: cell list of the atoms (device arrays)
    int* box;              // shape+ACE and LJ: [n][6] work (each atom's projection box)
    const double* lj_c;    // LJ: [n][5] per-atom field constants (as6, 4es6, 4es12, fshift, gshift)
    double lj_cut;         // LJ: field cutoff
    Geo geo;
    int term_set;
    int n_types;
    int K;
    double shape_core, shape_width;
    double ace_b, ace_k, ace_a, ace_cut;
    const double* emat;    // [n_types][n_types]
    int* flags;            // [N^3] work
    double* dens;          // [n_types][N^3] work (shape+ACE)
    double* rgrid;         // [K][N^3] out
};

cudaError_t build_receptor_grids(const ReceptorGridArgs& a, cudaStream_t s);

// Exact per-rotation queue of up to kWideMax entries ("maxNTransInp") and
// the translational clustering applied to it (TranClust,
// include/PRODDL/docking_fft.hpp:30-140).  The correlation grid of every
// rotation of the batch is written out; the cells at or below an upper bound
// of the queue's last value (taken from the per-plane top-KC pools) are
// gathered in one pass, sorted and clustered per rotation.  When the bound is
// missing or too loose, a radix select over 64-bit keys (ordered float bits
// << 32 | cell offset, so ties go to the lower offset) narrows the set first.
// tensor pencil stage: rotations per CTA (the MMA's N), largest window in
// 8-cell chunks, most non-empty terms
constexpr int kTcRot = 128;
constexpr int kTcMaxChunks = 32;  // the whole x range at N = 256 (two 128-row output tiles)
constexpr int kTcMaxTerms = 64;

constexpr int kWideMax = 16384;
constexpr int kWideBins = 4096;  // 12-bit digits

struct WideState {
    unsigned long long pfx;  // resolved key prefix (radix path)
    int nres;                // resolved key bits
    int need;                // entries still to take from the prefix's bin
    int below;               // entries with a key below the bin (all kept)
    int active;              // another digit pass is needed
    int flags;               // kWideAll | kWideRadix
    float thr;               // upper bound of the queue's values (+inf: none)
};
constexpr int kWideAll = 1;    // fewer than m cells pass: keep them all
constexpr int kWideRadix = 2;  // the bound was too loose: radix path
// The same exact queue without clustering serves more than KC peaks per
// rotation: the whole queue (at most kWidePool cells) is rescored in FP64,
// sorted by (energy, offset) and the first peaks_per_rot below maxValCorr
// are kept, like the per-plane pool path does for up to KC peaks.
constexpr int kWideNoClustering = -1;
constexpr int kWidePool = 512;

struct WideArgs {
    float* corr;               // [B][N^3] correlation grids (nullptr: wide path off)
    uint32_t* hist;            // [B][kWideBins]
    WideState* st;             // [B]
    unsigned long long* cand;  // [B][kWideMax] gathered keys
    int32_t* cnt;              // [B]
    int m;                     // queue bound, 1..kWideMax
    int order;                 // FFTDOCK_CLUSTER_ORDER_*, or kWideNoClustering
    double rad2;               // squared neighbour radius of the clustering
};

// Mixed-radix plan of one transform length of the box-grid path: radices in
// Stockham stage order (4, 2, 3, 5, 7, 11, 13).
constexpr int kBoxMaxFactors = 12;
struct BoxPlan {
    int n;
    int nf;
    int f[kBoxMaxFactors];
};
// Box-grid sizes each axis may take: [kBoxMin, kBoxMax], factors 2..13.
constexpr int kBoxMin = 8;
constexpr int kBoxMax = 256;

// Everything one device batch of rotations needs.
struct BatchArgs {
    // inputs
    const double* rot;          // [B][9]
    const double* lig_xyz;      // [n_ent][3]
    const int32_t* lig_term;    // [n_ent]
    const float* lig_w32;       // optional [n_ent] entry weights (weighted term sets), FP32 for the sums
    const double* lig_w64;      // optional [n_ent] the same weights in FP64 for the rescoring
    const void* spec;           // [K][N][PP] float2, or __nv_bfloat162 when spec_bf16
    int spec_bf16;
    const double* rgrid;        // [K][N^3]
    const float2* tw32;         // [N]
    int n_rot;                  // rotations in this batch (<= B)
    int n_ent;
    int K;
    int PP;
    double h, zero_h, center0;
    // work
    uint32_t* ent;              // [B][n_ent]
    float* ent_w;               // weighted: [B][n_ent] weights in sorted order
    int32_t* ent_idx;           // weighted: [B][n_ent] entry index in sorted order
    int32_t* offs;              // [B][K*N+1]
    int32_t* status;            // [B]
    float2* g2;                 // [B][N][PP]
    float* cand_v;              // [B][N][KC]
    int32_t* cand_i;
    // outputs
    fftdock_peak* peaks;        // [B][peak_stride]
    int32_t* n_peaks;           // [B]
    int peak_stride;
    int k_out;
    double max_val;
    int first_rot_id;
    float* dbg_corr;            // optional [B][N^3]
    float* pool_v;              // optional [B][KC]
    int32_t* pool_i;
    cudaEvent_t* ev;            // optional: events recorded by the middle stage (see SizeOps::middle)
    // tensor-core pencil stage (use_tc): it writes g2t as x-quads
    // [B][N/4][N*H][4] (four consecutive x per pencil), which the plane stage
    // reads in clusters of 4 CTAs
    float2* g2t;
    int use_tc;
    const float2* circ;         // [K][N*H][N] receptor circulant samples
    const int8_t* cscale;       // [N*H] power-of-two scale exponents
    int x0, W;                  // ligand window along x
    uint32_t* ent_t;            // [B/128][n_pad][128] entries transposed per group of 128 rotations
    const int32_t* tinfo;       // padded entry starts of the n_tc_terms non-empty terms, then their term ids
    const int32_t* tpad;        // [K] padded start - start of each term's entries
    int n_tc_terms;
    int tc_group;               // terms per tensor-memory sum (<= 0: FFTDOCK_TC_TERMS_PER_SUM_DEFAULT)
    float2* tc_slots;           // [tc_n_slots][128][128] running sums of the tensor stage's CTAs
    int tc_n_slots;             // 2 per SM id (tc_slot_count)
    int n_pad;                  // entries per rotation with every term padded to a multiple of 8
    int* err;                   // device word: nonzero after a pipeline timeout
    WideArgs wide;              // queue + clustering path (wide.corr != nullptr)
    // box-grid path (box.n[0] > 0): per-axis geometry and the FP32 twiddle
    // tables of the three axes, [Nx | Ny | Nz]
    Geo box;
    const float2* box_tw32;
};

// The tensor pencil stage's per-ligand tables: the x window [x0, x0 + W)
// that holds the ligand's cells under every rotation about the origin, and
// the rows of the transposed entries (each non-empty term's range padded to
// 8).  ok = the window and the term count fit the stage.
struct TcTables {
    int x0 = 0, W = 0;
    int n_pad = 0;                 // padded rows per rotation
    int ka = 0;                    // non-empty terms
    std::vector<int32_t> info;     // [ka + 1] padded starts, then [ka] term ids
    std::vector<int32_t> tpad;     // [K] padded start - start of each term
    bool ok = false;
};
TcTables tc_tables(const double* xyz, const int32_t* term, int n, int K, int N, double h, double zero_h);
// the padding rows of the transposed entries: x' = W (the tensor stage's
// dummy staging row), y = z = 0
cudaError_t fill_padding(uint32_t* ent_t, int W, size_t n, cudaStream_t s);
// slots of the tensor stage's running sums on the current device: two per SM
// id (%nsmid, which bounds %smid), one per tensor-memory half
cudaError_t tc_slot_count(int* n_slots);
// AUTO selection of the tensor form: grid edge <= 128 (has_tc), FP32
// spectra, an unweighted term set with at least kTcMinTerms terms (at 64^3
// with the single shape term the FFT form measured faster)
constexpr int kTcMinTerms = 4;

// queue + clustering stage of one batch, after the correlation grids of the
// batch are in a.wide.corr; writes a.peaks / a.n_peaks
cudaError_t wide_select_batch(const BatchArgs& a, int N, cudaStream_t s);

struct SizeOps {
    int n;
    // forward 3-D FFT of one real FP64 term grid into spec_t ([N][PP], scaled 1/V)
    cudaError_t (*receptor_fft)(const double* rgrid_t, double2* cbuf, double2* hbuf, const double2* tw64,
                                void* spec_t, int spec_bf16, int PP, float2* circ_t, cudaStream_t s);
    // per-pencil scale exponents of the circulant samples (tensor path)
    cudaError_t (*circ_scales)(const float2* circ, int K, int8_t* cscale, cudaStream_t s);
    bool has_tc;
    cudaError_t (*scan_batch)(const BatchArgs& a, cudaStream_t s);
    // shared-memory bytes of the pencil kernel for (K, n_ent)
    size_t (*pencil_smem)(int K, int n_ent);
    // the pipeline's stages: ligand prep, pencil + plane (+ clustering
    // selection), finalize; scan_batch = all three for one batch
    cudaError_t (*prep)(const BatchArgs& a, cudaStream_t s);
    cudaError_t (*middle)(const BatchArgs& a, cudaStream_t s);
    cudaError_t (*finish)(const BatchArgs& a, cudaStream_t s);
    // load the code of the FFT-form kernels (the ones the no-allocation scan
    // runs) into the current CUDA context, so that their first launch loads
    // nothing
    cudaError_t (*load_fft_form)(int spec_bf16);
};

const SizeOps* size_ops(int n);

// Box grids (box_grid.cu): sizes per axis, any length of factors 2..13 in
// [kBoxMin, kBoxMax]; the pipeline's stages read the sizes from BatchArgs.box.
const SizeOps* box_ops();
bool box_plan(int n, BoxPlan* pl);
// largest dynamic shared memory of the box-grid kernels for a ligand
size_t box_pencil_smem(int nx, int ny, int nz, int K, int n_ent, bool weighted);
// forward transform of one real FP64 term grid into spec_t ([Nx][PP] float2,
// scaled 1/V); tw64 = the FP64 twiddle tables [Nx | Ny | Nz]; circ_t (tensor
// form): the term's circulant samples [Ny Hz][Nx] (the grid transformed
// along z and y only, conjugated, / (Ny Nz))
cudaError_t box_receptor_fft(const double* rgrid_t, double2* cbuf, double2* hbuf, const double2* tw64,
                             const int dims[3], void* spec_t, int PP, float2* circ_t, cudaStream_t s);
// per-pencil scale exponents of the box grid's circulant samples
cudaError_t box_circ_scales(const float2* circ, int K, int nh, int nx, int8_t* cscale, cudaStream_t s);
// dynamic shared memory of the tensor pencil stage on a box grid, and on a
// cubic grid of edge n
size_t box_tc_smem(const int dims[3], int n_chunks, int n_terms);
size_t cubic_tc_smem(int n, int n_chunks, int n_terms);

// Read-only view of a ready context's scan inputs (receptor spectra and
// grids, ligand, geometry); the work pointers of `args` are the context's own.
struct ScanInputs {
    BatchArgs args;
    const SizeOps* ops;
    int device;
    cudaStream_t stream;
    int N, K, PP, B, n_ent;
    void* noalloc_scratch;  // the no-allocation scan's array in the context's CUDA context
    bool box;               // a box-grid context
};
int ctx_scan_inputs(fftdock_ctx* ctx, ScanInputs* in);
// Device address, in the current CUDA context, of the no-allocation scan's
// work array (noalloc.cu); resolving it loads the library's module for that
// file, which commits the array on the device.  Called by fftdock_create.
cudaError_t noalloc_scratch_address(void** addr);
int ctx_fail(fftdock_ctx* ctx, int code, const char* msg);

}  // namespace fftdock
