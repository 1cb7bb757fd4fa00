/*
 * fftdock.h -- C ABI of the GB300 FFT rotational/translational correlation
 * scan (libfftdock.so).
 *
 * This library replaces the in-process C++ template API of the PRODDL2
 * `rot-scan` worker for one ligand/receptor pair:
 *   MolForce::{projectMol, collectTotal, nGrids}
 *       include/PRODDL/docking_molforce.hpp:38-104
 *   FFTCorrelators::{preprocessReceptor, correlate}
 *       include/PRODDL/docking_fft.hpp:767-883
 *   CorrelationProcessor::{init, selectFromFFT, getTranValuesFilled}
 *       include/PRODDL/docking_fft.hpp:283-447
 * as orchestrated by Worker::{init, prepareReceptor, scanRotation, run}
 *       include/PRODDL/docking_app.hpp:326-513.
 *
 * Ownership: the caller owns every host buffer passed in; the library copies
 * what it needs before returning.  The context owns all device memory.
 * Threading: one context per host thread; calls on one context are not
 * re-entrant, separate contexts are independent.  Everything runs on one GPU;
 * there is no CPU fallback: on a machine without a usable GPU every call that
 * needs one returns FFTDOCK_ECUDA.
 * Errors: every entry point returns an FFTDOCK_* status; the text of the last
 * error is available from fftdock_last_error(ctx).  No C++ exception crosses
 * this boundary.
 */
#ifndef FFTDOCK_H_
#define FFTDOCK_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFTDOCK_ABI_VERSION 1

/* status codes; the reference signals the same conditions with C++
 * exceptions caught at main (src/PRODDL/docking_main.cpp:143,155) or leaves
 * them undefined (ligand atoms outside the grid, docking_molforce.hpp:360-364) */
enum {
    FFTDOCK_OK = 0,
    FFTDOCK_EINVAL = 1,        /* bad argument or configuration */
    FFTDOCK_EOUT_OF_GRID = 2,  /* a rotated ligand atom falls outside the grid */
    FFTDOCK_ECUDA = 3,         /* CUDA error or no usable GPU */
    FFTDOCK_ENOMEM = 4,        /* device or host allocation failed */
    FFTDOCK_ESTATE = 5,        /* call order (scan before receptor/ligand) */
    FFTDOCK_EUNSUPPORTED = 6,  /* grid size or option not built into this library */
    FFTDOCK_EIO = 7            /* scan-record file I/O */
};

/* correlation term sets (the reference's "potentialName",
 * docking_app.hpp:54-66, plus this library's shape/desolvation terms) */
enum {
    FFTDOCK_TERMS_SHAPE = 1,     /* surface +1 / core -15 receptor grid, unit ligand weights; K = 1 */
    FFTDOCK_TERMS_SHAPE_ACE = 2, /* shape + n_types ACE-style desolvation grids, folded to K = n_types */
    FFTDOCK_TERMS_LJ_COMP = 3,   /* the reference's "ljComp": soft-core LJ repulsion + attraction
                                    (MolForceLJComp, docking_molforce.hpp:456-600), K = 2; atoms and
                                    parameters through fftdock_set_pair_lj */
    FFTDOCK_TERMS_LJ_AVG = 4     /* the reference's "ljAvg": soft-core LJ with ligand-averaged
                                    parameters (MolForceLJ, docking_molforce.hpp:375-455), K = 1 */
};

/* precision of the stored receptor spectra (FFT pencil stage): FP32 pairs,
 * or BF16 pairs widened to FP32 for the spectrum product (half the
 * spectrum memory and traffic; candidate values then carry BF16-level
 * error, and the FP64 rescoring still fixes the reported scores) */
enum {
    FFTDOCK_PREC_FP32 = 0,
    FFTDOCK_PREC_BF16_SPECTRA = 1
};

/* how the per-pencil x stage (x transforms and the spectrum product summed
 * over terms) runs.  FFT: FP32 x-FFTs on the CUDA cores.  TENSOR (x sizes
 * <= 256, one or two 128-row output tiles; unweighted term sets) restates the stage as a circular
 * correlation along x computed with split-FP16 tcgen05 GEMMs (hi*hi + hi*lo
 * + lo*hi, FP32 accumulate) over ligand bins summed on the CUDA cores; the
 * scan then takes rotations in groups of 128 (rot_batch is rounded up).  The
 * tensor core's FP32 accumulation error grows with the chain of MMAs into one
 * accumulator, so the accumulator restarts every tc_terms_per_sum terms and
 * the groups are summed in FP32 with round-to-nearest: with the default 6 the
 * FP32 candidate values stay within 1e-4 relative of FP64 (measured 8.4e-5
 * at 128^3 with 18 terms; one group of all 18 terms: 2.3e-4; FFT: 3.8e-5);
 * reported scores are FP64 direct-space energies either way.  AUTO = TENSOR
 * where it is the faster form (cubic edges <= 128 and box grids with Nx <=
 * 256, FP32 spectra, an unweighted term set with at least 4 terms: at 64^3
 * with the single shape term, and at 144^3, the FFT form is faster), else FFT; a ligand whose window exceeds the tensor stage's shared
 * memory runs the FFT form.  The no-allocation scan always runs the FFT form;
 * fftdock_scan_pairs follows the same rule per grid edge. */
enum {
    FFTDOCK_PENCIL_AUTO = 0,
    FFTDOCK_PENCIL_FFT = 1,     /* FP32 x-FFTs on the CUDA cores */
    FFTDOCK_PENCIL_TENSOR = 2   /* circular correlation as split-FP16 tcgen05 GEMMs, FP32 accumulate */
};

/* translational clustering of each rotation's queue ("doClusterTranslations",
 * TranClust, include/PRODDL/docking_fft.hpp:30-140 over ClusterMatrix,
 * include/PRODDL/Geom/cluster.hpp:121-477).  With clustering on, the scan
 * keeps the exact max_trans_inp lowest cells of every rotation (at most
 * FFTDOCK_MAX_QUEUE_CLUSTERED), walks them in the chosen order and makes a
 * cell a cluster leader unless it lies within the neighbour radius of an
 * earlier leader; the first peaks_per_rot leaders are the rotation's peaks,
 * in walk order.  The reference's walk starts from the queue's worst value
 * (its density is overridden by the weight -value and sorted ascending,
 * cluster.hpp:238-253); BEST_FIRST walks from the best value instead.  The
 * neighbour radius tested is sqrt(3) * cluster_radius, as in the reference
 * (three clustered columns). */
enum {
    FFTDOCK_CLUSTER_ORDER_REFERENCE = 0,
    FFTDOCK_CLUSTER_ORDER_BEST_FIRST = 1
};
#define FFTDOCK_MAX_QUEUE_CLUSTERED 16384
#define FFTDOCK_MAX_PEAKS 256

typedef struct fftdock_config {
    int32_t struct_size;         /* sizeof(fftdock_config) */
    int32_t grid_n;              /* FFT grid edge N (cubic); see fftdock_supported_grid() */
    double grid_step;            /* h in Angstrom ("gridStep") */
    int32_t term_set;            /* FFTDOCK_TERMS_* ("potentialName") */
    int32_t peaks_per_rot;       /* translations kept per rotation ("maxNTrans"), 1..FFTDOCK_MAX_PEAKS;
                                    above 16 (the per-plane candidate pools) the scan keeps each
                                    rotation's exact queue like cluster_trans does, without the
                                    clustering: its first peaks_per_rot + 16 cells are rescored in
                                    FP64 and the best peaks_per_rot kept */
    int32_t max_trans_inp;       /* bound of the per-rotation queue ("maxNTransInp") */
    double max_val_corr;         /* only scores strictly below this are kept ("maxValCorr") */
    int32_t rot_batch;           /* rotations per device batch, 1..1024 */
    int32_t precision;           /* FFTDOCK_PREC_* */
    int32_t device;              /* CUDA device ordinal */
    int32_t n_types;             /* desolvation atom types (FFTDOCK_TERMS_SHAPE_ACE) */
    const double* ace_matrix;    /* n_types x n_types row-major; copied by fftdock_create */
    double shape_core_radius;    /* core if a cell centre is within this of an atom (A) */
    double shape_surface_width;  /* surface shell width beyond the core radius (A) */
    double ace_b, ace_k, ace_a;  /* sigmoid 1/(1+exp(b(k r - a))) (potentials_inc.hpp:394-397) */
    double ace_cut;              /* cutoff of the desolvation field (A) */
    int32_t pencil_mode;         /* FFTDOCK_PENCIL_* */
    int32_t cluster_trans;       /* 1: cluster each rotation's queue ("doClusterTranslations") */
    int32_t cluster_order;       /* FFTDOCK_CLUSTER_ORDER_* */
    double cluster_radius;       /* "clusterRadiusTrans" (A), reference default 5 */
    int32_t lj_mix;              /* LJ term sets: sigma combination rule (PotentialsT::LJ_MIX_0 = 0:
                                    arithmetic, LJ_MIX_1 = 1: geometric; ljComp requires 1) */
    double lj_cut;               /* LJ term sets: field cutoff ("cutOffFft"), grid length units */
    int32_t tc_terms_per_sum;    /* tensor pencil stage: the terms are split into ceil(K / this) groups
                                    of equal size, each accumulated in a fresh tensor-memory sum, and the
                                    groups' sums are added in FP32 (round to nearest); the tensor core's
                                    own accumulation error grows with the group size.
                                    0 = the library default (FFTDOCK_TC_TERMS_PER_SUM_DEFAULT) */
    int32_t grid_nx, grid_ny, grid_nz; /* FFT sizes per axis (the reference's fftSize, each axis from
                                    findBestSize over the padded receptor box, docking_fft.hpp:541-553);
                                    all 0 = grid_n on every axis.  A cubic size with compiled plans
                                    (fftdock_supported_grid) runs the cubic kernels; any other sizes,
                                    each in [8, 256] with no prime factor above 13, run the box-grid
                                    kernels (the tensor pencil stage for Nx <= 256, else the FFT form; up to
                                    16 peaks per rotation, FP32 spectra,
                                    no clustering, no pair graph, no no-allocation scan) */
} fftdock_config;
#define FFTDOCK_TC_TERMS_PER_SUM_DEFAULT 6

/* one selected translation; the reference's TranValue
 * (include/PRODDL/types.hpp:68-84) plus the rotation id and the raw
 * correlation cell. */
typedef struct fftdock_peak {
    int32_t rot_id;   /* first_rot_id + index of the rotation in the call */
    int32_t cell[3];  /* correlation offset s (FFT output index, [0, N)^3) */
    double t[3];      /* translation h * unwrap(s) (docking_fft.hpp:368-389) */
    double score;     /* correlation energy, FP64 direct-space rescored; lower is better */
} fftdock_peak;

typedef struct fftdock_ctx fftdock_ctx;

/* Fill *cfg with defaults: N 128, h 1.2, shape+ACE with 18 types (matrix
 * must still be supplied), 4 peaks, queue 10000, maxValCorr +inf, batch 64. */
void fftdock_config_init(fftdock_config* cfg);

/* Cubic grid edges with compiled plans in this library (1 if supported). */
int fftdock_supported_grid(int32_t n);

/* 1 if this library scans a grid of these per-axis FFT sizes: a compiled
 * cubic edge, or box-grid sizes (each in [8, 256], no prime factor above 13;
 * every findBestSize result in that range qualifies).  Replaces the sizing of
 * FFTCorrelator::init (include/PRODDL/docking_fft.hpp:541-553), which takes
 * fftSize per axis. */
int fftdock_supported_dims(int32_t nx, int32_t ny, int32_t nz);

/* FFTW_Size::findBestSize (include/PRODDL/Math/fft.hpp:141-151): smallest
 * size >= start_n over primes {2,3,5,7,11,13} with e11 + e13 <= 1. */
int fftdock_find_best_size(int32_t start_n, int32_t* result);

/* Create a context (Worker::init, docking_app.hpp:326-404, minus rotation
 * file loading): validates the configuration and allocates device memory. */
int fftdock_create(const fftdock_config* cfg, fftdock_ctx** out);
void fftdock_destroy(fftdock_ctx* ctx);
const char* fftdock_last_error(const fftdock_ctx* ctx);

/* The LJ term sets' inputs (the reference's MolForceParams pos/eps/sigma/
 * alpha of both molecules): receptor atoms in the grid frame with sigma,
 * eps, alpha; ligand atoms (rotation centre at the origin) with sigma, eps.
 * Builds the receptor fields -- per atom SoftCoreLJRep/SoftCoreLJAttr
 * (ljComp) or SoftCoreLJ with the force-shifted cutoff (ljAvg) against the
 * ligand's mean sigma/eps, projected like ProjectorRadialField -- and the
 * ligand weights (ljComp: sqrt(eps) sigma^6 and sqrt(eps) sigma^3; ljAvg:
 * 1).  Replaces fftdock_set_receptor / fftdock_set_ligand for these sets. */
int fftdock_set_pair_lj(fftdock_ctx* ctx, int32_t n_rec, const double* rec_xyz, const double* rec_sigma,
                        const double* rec_eps, const double* rec_alpha, int32_t n_lig, const double* lig_xyz,
                        const double* lig_sigma, const double* lig_eps);

/* Receptor atoms in the grid frame (grid centred on the origin).  Builds the
 * K receptor term grids and keeps their spectra on the device
 * (Worker::prepareReceptor, docking_app.hpp:406-415, and
 * FFTCorrelator::preprocessReceptor, docking_fft.hpp:614-618). */
int fftdock_set_receptor(fftdock_ctx* ctx, int32_t n, const double* xyz, const int32_t* type);

/* Ligand atoms in the ligand frame (rotations are applied about the origin,
 * docking_app.hpp:454-456).  type[i] in [0, n_types) for shape+ACE. */
int fftdock_set_ligand(fftdock_ctx* ctx, int32_t n, const double* xyz, const int32_t* type);

/* Scan n_rot rotations (row-major 3x3 doubles, host memory).  For rotation i,
 * peaks[i*peaks_per_rot + j] for j < n_peaks[i] hold the selected
 * translations in ascending score order (Worker::scanRotation,
 * docking_app.hpp:450-466).  Returns FFTDOCK_EOUT_OF_GRID if any rotated
 * ligand atom leaves the grid; those rotations report n_peaks = 0. */
int fftdock_scan(fftdock_ctx* ctx, int32_t n_rot, const double* rot, int32_t first_rot_id,
                 fftdock_peak* peaks, int32_t* n_peaks);

/* Same with device pointers on the given CUDA stream (NULL = the context's
 * stream); the call returns after queueing the work and does not report
 * out-of-grid rotations (their n_peaks is 0). */
int fftdock_scan_device(fftdock_ctx* ctx, int32_t n_rot, const double* d_rot, int32_t first_rot_id,
                        fftdock_peak* d_peaks, int32_t* d_n_peaks, void* stream);

/* Scan without allocating device memory (no counterpart in the reference,
 * whose scan runs in its own process and allocates freely).  For callers that
 * cannot allocate at scan time: a host whose memory pool already owns the
 * GPU, or a pipeline that forbids allocation once running.  Same arguments
 * and results as fftdock_scan_device, but the per-batch work memory lives in
 * one 16 MiB array compiled into the library instead of the context's
 * buffers; the context must already hold a receptor and a ligand.  The array
 * exists once per CUDA context that loads the library (for this library's
 * contexts: the primary context of their device) and stays until that
 * context ends.  fftdock_create commits it on the device and looks up its
 * address, so the scan call itself allocates nothing and looks nothing up;
 * create contexts at start-up, before the host's pool takes the GPU and
 * before any stream capture.  Batches shrink to fit the array; a context
 * whose single rotation needs more than 16 MiB is rejected with
 * FFTDOCK_EINVAL.  All calls in one CUDA context share the array: calls whose
 * GPU work overlaps race and must be serialised by the caller. */
int fftdock_scan_device_noalloc(fftdock_ctx* ctx, int32_t n_rot, const double* d_rot, int32_t first_rot_id,
                                fftdock_peak* d_peaks, int32_t* d_n_peaks, void* stream);

/* Introspection.  fftdock_grid_n: the x size (the edge of a cubic grid);
 * fftdock_grid_dims: the three sizes. */
int fftdock_grid_n(const fftdock_ctx* ctx);
int fftdock_grid_dims(const fftdock_ctx* ctx, int32_t* dims3);
int fftdock_n_terms(const fftdock_ctx* ctx);

typedef struct fftdock_scan_info {
    int32_t grid_n;
    int32_t n_terms;       /* K correlation terms */
    int32_t pencil_path;   /* FFTDOCK_PENCIL_FFT or FFTDOCK_PENCIL_TENSOR (the form that runs) */
    int32_t rot_batch;     /* rotations per device batch */
    int32_t n_entries;     /* ligand entries (0 before fftdock_set_ligand) */
    int32_t window_x0;     /* tensor path: first x cell of the ligand window */
    int32_t window_w;      /* tensor path: window width in cells (multiple of 8) */
} fftdock_scan_info;
int fftdock_get_scan_info(const fftdock_ctx* ctx, fftdock_scan_info* out);

/* Copy receptor term grid `term` (real space, FP64, N^3 C order) to host. */
int fftdock_get_receptor_grid(fftdock_ctx* ctx, int32_t term, double* out);

/* Diagnostic: the FP32 correlation grid sum_t corr(R_t, L_t) for one
 * rotation (N^3 floats, C order), as produced before selection. */
int fftdock_correlation_grid(fftdock_ctx* ctx, const double* rot, float* out);

/* Diagnostic: per-rotation FP32 candidate pool (16 smallest values and their
 * flat offsets, ascending) before FP64 rescoring.  FFTDOCK_EUNSUPPORTED on a
 * clustering context (cluster_trans), which keeps no such pool. */
int fftdock_scan_candidates(fftdock_ctx* ctx, int32_t n_rot, const double* rot,
                            float* values, int32_t* offsets);

/* Per-kernel device time of the scan, from CUDA events recorded on the
 * launching stream around each kernel of every batch while profiling is on.
 * Kernels: 0 ligand rotate/bin/sort, 1 pencil (forward x transform, spectrum
 * product over terms, inverse x transform), 2 plane (inverse y, real z,
 * top-k), 3 finalize (merge, FP64 rescoring, translations). */
typedef struct fftdock_kernel_stats {
    int64_t launches[4];
    double total_ms[4];
} fftdock_kernel_stats;

/* Start (enable != 0) or stop recording kernel events; starting clears the record. */
int fftdock_profile(fftdock_ctx* ctx, int32_t enable);

/* Synchronise the context's work and sum the recorded kernel times. */
int fftdock_get_kernel_stats(fftdock_ctx* ctx, fftdock_kernel_stats* out);

/* One docking pose of the gathered result: the reference's RotTranValue
 * (include/PRODDL/types.hpp:80-84), a rotation applied first then a
 * translation, with its score. */
typedef struct fftdock_pose {
    double value;
    double rot[9];   /* row-major */
    double t[3];
} fftdock_pose;

/* Foreman::run (include/PRODDL/docking_app.hpp:174-220): read the
 * RotFftScanIO_Bin files in order, turn every translation t of a record with
 * rotation R into the pose (R, t), keep the max_matches smallest values below
 * 1e16 and return them ascending (ties in file order).  out holds max_matches
 * poses; *n_out receives the count.  FFTDOCK_EIO on a missing file or a
 * signature mismatch. */
int fftdock_gather_records(const char* const* paths, int32_t n_paths, int32_t max_matches, fftdock_pose* out,
                           int32_t* n_out);

/* Same over a list file of record-file paths, one per line
 * (RotFftScanIO_Collector, docking_io_bin.hpp:81-116). */
int fftdock_gather_list(const char* list_path, int32_t max_matches, fftdock_pose* out, int32_t* n_out);

/* Foreman::writeResults (docking_app.hpp:269-281): move each pose to the
 * original frame, rec_frame^-1 * pose * lig_frame (docking_molstruct.hpp:
 * 31-51; each frame is 12 doubles, row-major rotation then vector, NULL =
 * identity), and write IORigid records (IO/rigid.hpp:115-176): binary
 * [int32 2005052501][int32 n][n x float32 {value, euler[3], xyz[3]}] or, if
 * text != 0, the reference's tab-separated text form. */
int fftdock_write_rigid(const char* path, const fftdock_pose* poses, int32_t n, const double* rec_frame,
                        const double* lig_frame, int32_t text);

/* Append one RotFftScanIO_Bin record per rotation to `path`
 * (include/PRODDL/docking_io_bin.hpp:55-71): [int32 2014011401][3x3 double
 * rotation][size_t n][n x {double t[3], double value}]. */
int fftdock_write_scan_records(const char* path, int32_t n_rot, const double* rot, int32_t peaks_per_rot,
                               const fftdock_peak* peaks, const int32_t* n_peaks, int32_t append);

/* ------------------------------------------------------------------------
 * Pre-scan frame set-up of a pair (host only): MolStruct::
 * moveIntoReferencePositions (include/PRODDL/docking_molstruct.hpp:199-252)
 * and the FFT size rule of FFTCorrelator::init (docking_fft.hpp:535-553).
 * Spins the ligand about its centre of mass by the Euler angles (s, 3.7877 s,
 * -4.513432 s), moves both molecules into the receptor box's frame, moves
 * the ligand's diameter centre to the origin, pads the box by 2 h + ligand
 * size / 2 + cutOffFft and sizes the grid per axis.  The receptor box is
 * axis-aligned (FFTDOCK_BOX_AXES: the reference's Box with fixed
 * directions) or given by the caller (FFTDOCK_BOX_GIVEN: e.g. the minimum-
 * volume box the reference gets from its gdiam library: 3 direction rows and
 * the corners (0,0,0) and (1,1,1)).  The frames written out are the ones
 * fftdock_write_rigid undoes.
 * ------------------------------------------------------------------------ */
enum {
    FFTDOCK_BOX_AXES = 0,
    FFTDOCK_BOX_GIVEN = 1,
    FFTDOCK_BOX_MIN_VOLUME = 2   /* the minimum-volume box computed by fftdock_min_volume_box (grid 5) */
};

/* Minimum-volume bounding box of n points (the receptor), as the reference's
 * Geom::Bounding::Box computes it through gdiam's grid search
 * (include/PRODDL/Geom/bounding.hpp:137-172): Barequet and Har-Peled's
 * approximation -- a box on the diameter and the projected diameter, boxes
 * from the minimum-area rectangles of the points projected across each box
 * direction, and a search over the primitive integer combinations of the box
 * directions up to `grid` (the reference uses 5).  dirs: 3 direction rows;
 * corners: vertex (0,0,0) then vertex (1,1,1), in the points' frame. */
int fftdock_min_volume_box(int32_t n, const double* xyz, int32_t grid, double* dirs, double* corners);

typedef struct fftdock_frame_setup_in {
    int32_t n_rec;
    const double* rec_xyz;       /* [n_rec][3], original frame */
    int32_t n_lig;
    const double* lig_xyz;       /* [n_lig][3], original frame */
    const double* lig_mass;      /* [n_lig] or NULL (unit masses) */
    double grid_step;            /* gridStep */
    double cut_off_fft;          /* cutOffFft */
    double starting_spin;        /* startingSpin (radians; reference default 23.3734432) */
    int32_t box_mode;            /* FFTDOCK_BOX_* */
    const double* box_dirs;      /* GIVEN: [3][3] direction rows */
    const double* box_corners;   /* GIVEN: corner (0,0,0) then corner (1,1,1), original frame */
    const double* lig_diam;      /* optional: the ligand diameter's end points (6 doubles, frame after
                                    step 2); NULL: the exact farthest pair */
} fftdock_frame_setup_in;

typedef struct fftdock_frame {
    double rec_frame[12];        /* original -> scan frame (row-major rotation, then vector) */
    double lig_frame[12];
    double lig_size;             /* ligand diameter */
    double min_box[6];           /* padded receptor box in the scan frame: low xyz, high xyz */
    int32_t fft_size[3];         /* FFTW_Size::findBestSize per axis */
    int32_t grid_n;              /* smallest built cubic edge >= the largest fft_size (0: none) */
} fftdock_frame;

/* rec_out [n_rec][3] and lig_out [n_lig][3] receive the moved atoms. */
int fftdock_frame_setup(const fftdock_frame_setup_in* in, double* rec_out, double* lig_out, fftdock_frame* out);

/* ------------------------------------------------------------------------
 * Many pairs in one CUDA graph.  No counterpart in the reference (it runs
 * one pair per process).  Every pair's atoms and rotations are staged on the
 * device once; the whole workload -- per pair the receptor grids and
 * transforms, then the scan batches -- is captured into one CUDA graph over
 * one or more streams and launched once.  With tune != 0 an autotuner picks
 * the rotations per launch of each grid size and the number of streams from
 * timed probes.  cfg supplies everything but the grid edge (term set, ACE
 * matrix, peaks, limits, precision, device); clustering and the tensor-core
 * pencil form are not part of the batch.
 * ------------------------------------------------------------------------ */
#define FFTDOCK_N_SIZES 10   /* built grid edges: 16 24 32 48 64 80 96 112 128 144 */

typedef struct fftdock_pair {
    int32_t grid_n;              /* built grid edge of this pair */
    int32_t n_rec;
    const double* rec_xyz;       /* [n_rec][3], grid frame */
    const int32_t* rec_type;     /* [n_rec], shape+ACE only */
    int32_t n_lig;
    const double* lig_xyz;       /* [n_lig][3], rotation centre at the origin */
    const int32_t* lig_type;     /* [n_lig], shape+ACE only */
    int32_t n_rot;
    const double* rot;           /* [n_rot][9] row-major */
    int32_t first_rot_id;
    fftdock_peak* peaks;         /* out, host: [n_rot][peaks_per_rot] */
    int32_t* n_peaks;            /* out, host: [n_rot] */
} fftdock_pair;

typedef struct fftdock_pairs_report {
    int32_t n_streams;                    /* streams the graph used */
    int32_t grid_sizes[FFTDOCK_N_SIZES];  /* the edge each slot below stands for */
    int32_t rot_batch[FFTDOCK_N_SIZES];   /* rotations per launch used per edge (0: edge unused) */
    double setup_ms;                      /* whole call, host clock */
    double tune_ms;                       /* autotuner probes, host clock */
    double capture_ms;                    /* capture + instantiation, host clock */
    double run_ms;                        /* the graph's execution, CUDA events */
    int64_t rotations;                    /* rotations scanned */
    int32_t n_out_of_grid;                /* rotations that left the grid (no peaks) */
    int32_t pencil_form[FFTDOCK_N_SIZES]; /* pencil-stage form used per edge: FFTDOCK_PENCIL_FFT or
                                             FFTDOCK_PENCIL_TENSOR (0: edge unused); under AUTO the
                                             autotuner times both where either can run */
} fftdock_pairs_report;

/* Scan every pair; FFTDOCK_EOUT_OF_GRID (outputs still written) if any
 * rotation put a ligand atom outside its grid.  Errors are described by
 * fftdock_pairs_last_error() (per calling thread).  With tune == 0, a report
 * whose n_streams > 0 is read as the plan to use (streams, and per edge the
 * rotations per launch and, under AUTO, the pencil form; e.g. from an
 * earlier tuned call); otherwise one stream, cfg->rot_batch and the AUTO
 * rule. */
int fftdock_scan_pairs(const fftdock_config* cfg, int32_t n_pairs, const fftdock_pair* pairs, int32_t tune,
                       fftdock_pairs_report* report);
const char* fftdock_pairs_last_error(void);

/* Grid edge for a pair: the smallest built edge >= 48 that covers
 * ceil((2 r_rec + 2 r_lig + 2 margin) / step) cells, r_rec the receptor's
 * largest atom distance from its bounding-box centre and r_lig the ligand's
 * from the origin (the rotation centre). */
int fftdock_pair_grid(int32_t n_rec, const double* rec_xyz, int32_t n_lig, const double* lig_xyz, double step,
                      double margin, int32_t* grid_n);

/* ------------------------------------------------------------------------
 * Learned rotation proposal.  No counterpart in the reference: a small
 * network predicts each rotation's best (lowest) scan score from a 16^3
 * occupancy grid of the rotated ligand and a 128-value receptor descriptor,
 * so that a caller can scan only the rotations it ranks best; the
 * exhaustive scan (fftdock_scan) stays the fallback and the measure of its
 * recall.  Network: three 3^3 stride-2 convolutions (16, 32, 64 channels,
 * ReLU) -> 512 features + descriptor -> 256 ReLU -> 1.  Every layer, forward
 * and backward, is a batched BF16 tensor-core GEMM with FP32 accumulation
 * (convolutions through im2col); BF16 weights, activations and activation
 * gradients, FP32 master weights trained with Adam; the training step runs as
 * one captured CUDA graph.  Calls on one network are ordered on its own
 * stream (prediction on a caller's stream is fenced against it with events).
 * ------------------------------------------------------------------------ */
#define FFTDOCK_PROPOSAL_DESC 128

typedef struct fftdock_proposal fftdock_proposal;

/* New network with He-normal weights drawn from `seed` on `device`. */
int fftdock_proposal_create(int32_t device, uint64_t seed, fftdock_proposal** out);
void fftdock_proposal_destroy(fftdock_proposal* p);
const char* fftdock_proposal_last_error(const fftdock_proposal* p);

/* Parameter count and the FP32 master weights (layout: conv1 w[16][1][27],
 * b[16]; conv2 w[32][16][27], b[32]; conv3 w[64][32][27], b[64]; fc1
 * w[640][256] input-major, b[256]; fc2 w[256], b).  Setting the weights
 * resets the optimiser state. */
int32_t fftdock_proposal_n_params(void);
int fftdock_proposal_get_params(fftdock_proposal* p, float* out);
int fftdock_proposal_set_params(fftdock_proposal* p, const float* in);

/* Register one docking pair: the ligand's atoms (in the scan frame, rotation
 * centre at the origin) and the receptor's descriptor; returns its id. */
int fftdock_proposal_add_ligand(fftdock_proposal* p, int32_t n_atoms, const double* xyz, const float* rec_desc,
                                int32_t* id);

/* Training samples of a registered pair: rotations (row-major 3x3) and the
 * regression targets (the caller's scale, e.g. standardised best scores). */
int fftdock_proposal_add_samples(fftdock_proposal* p, int32_t lig, int32_t n, const double* rot,
                                 const float* target);
int fftdock_proposal_clear_samples(fftdock_proposal* p);

/* `steps` Adam steps (betas 0.9 / 0.999, eps 1e-8) on minibatches of
 * `batch` samples drawn with replacement by a hash of (seed, step); the
 * mean squared error over the steps is returned in *mean_loss. */
int fftdock_proposal_train(fftdock_proposal* p, int32_t steps, int32_t batch, float lr, uint64_t seed,
                           float* mean_loss);

/* Gradient of the mean squared error of the given samples with respect to
 * every parameter (no update): the check against a CPU restatement. */
int fftdock_proposal_gradients(fftdock_proposal* p, int32_t n, const int32_t* lig, const double* rot,
                               const float* target, float* grads, float* loss);

/* Predicted best score of pair `lig` for each rotation: host buffers, or
 * device buffers ordered on `stream` (NULL: the library's own stream). */
int fftdock_proposal_predict(fftdock_proposal* p, int32_t lig, int32_t n, const double* rot, float* out);
int fftdock_proposal_predict_device(fftdock_proposal* p, int32_t lig, int32_t n, const double* d_rot, float* d_out,
                                    void* stream);

/* Receptor descriptor: per element (0 C, 1 N, 2 O, 3 S) a 32-shell radial
 * histogram (1.5 A shells about the bounding-box centre, the last shell
 * open-ended) divided by the atom count.  Host only. */
int fftdock_receptor_descriptor(int32_t n, const double* xyz, const int32_t* element, float* out);
/* Oriented alternative (no counterpart in the reference): the receptor's
 * occupancy in the scan frame, 4 x 4 x 4 cells of the cube about its box
 * centre (half-width = the box's largest half-extent), all atoms (values
 * 0..63) and the outer atoms (64..127), as fractions of the atom count; with
 * it the network sees both molecules in one frame. */
int fftdock_receptor_descriptor_oriented(int32_t n, const double* xyz, float* out);

#ifdef __cplusplus
}
#endif

#endif /* FFTDOCK_H_ */
