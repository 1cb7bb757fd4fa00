// Scan entry point that allocates no device memory.
//
// fftdock_scan_device() keeps its per-batch work memory (ligand entries, bin
// offsets, x-inverse planes, candidate pools, status words) in buffers the
// context allocates.  Some callers cannot allocate at scan time: hosts whose
// memory pool has already reserved the whole GPU (a cudaMalloc would fail or
// fragment their pool), or real-time pipelines whose policy forbids
// allocation once they are running.  fftdock_scan_device_noalloc() runs the
// same kernels with that work memory in one fixed-size array compiled into
// this library instead.
//
// The array (kScratchBytes, 16 MiB) exists once per CUDA context that loads
// this file's module (for the library's contexts: the primary context of
// their device) and lives until that context ends.  Its address in the
// current context is resolved by noalloc_scratch_address(), which
// fftdock_create calls with the context's device current: resolving it loads
// the module, which is when the driver commits the array on the device.  So
// the scan call itself neither allocates nor looks anything up; callers
// create their contexts at start-up, before their own pool takes the GPU and
// before any stream capture.  Every call uses the same array and nothing in it
// needs to start at zero (each batch writes every word it later reads), so
// calls whose GPU work overlaps -- on two streams, or from two library
// contexts in one CUDA context -- race and must be serialised by the caller.
#include <cuda_runtime.h>

#include <string>

#include "fftdock.h"
#include "internal.h"

namespace {

constexpr size_t kScratchBytes = size_t(16) << 20;
constexpr int kKC = 16;

static __device__ __align__(256) unsigned char g_scan_scratch[kScratchBytes];

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// bytes of work memory for a batch of b rotations
size_t scratch_bytes(const fftdock::ScanInputs& in, int b) {
    size_t s = 0;
    s += align256(sizeof(int32_t) * (size_t)b);                                  // status
    s += align256(sizeof(uint32_t) * (size_t)b * in.n_ent);                      // entries
    s += align256(sizeof(int32_t) * (size_t)b * ((size_t)in.K * in.N + 1));      // bin offsets
    s += align256(sizeof(float) * (size_t)b * in.N * kKC);                       // pool values
    s += align256(sizeof(int32_t) * (size_t)b * in.N * kKC);                     // pool offsets
    s += align256(sizeof(float2) * (size_t)b * in.N * in.PP);                    // x-inverse planes
    return s;
}

}  // namespace

namespace fftdock {

// The host-side name g_scan_scratch stands for the array but is not its
// device address; kernels get the address resolved here.
cudaError_t noalloc_scratch_address(void** addr) {
    *addr = nullptr;
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scan_scratch);
    if (e != cudaSuccess) return e;
    if (!p) return cudaErrorInvalidSymbol;
    *addr = p;
    return cudaSuccess;
}

}  // namespace fftdock

extern "C" int fftdock_scan_device_noalloc(fftdock_ctx* ctx, int32_t n_rot, const double* d_rot,
                                           int32_t first_rot_id, fftdock_peak* d_peaks, int32_t* d_n_peaks,
                                           void* stream) {
    if (!ctx) return FFTDOCK_EINVAL;
    fftdock::ScanInputs in;
    int rc = fftdock::ctx_scan_inputs(ctx, &in);
    if (rc) return rc;
    if (n_rot < 0 || (n_rot > 0 && (!d_rot || !d_peaks || !d_n_peaks)))
        return fftdock::ctx_fail(ctx, FFTDOCK_EINVAL, "bad arguments");
    if (n_rot == 0) return FFTDOCK_OK;
    if (in.args.lig_w32)
        return fftdock::ctx_fail(ctx, FFTDOCK_EUNSUPPORTED,
                                 "weighted ligand entries (ljComp) are not covered by the no-allocation scan");
    if (in.box)
        return fftdock::ctx_fail(ctx, FFTDOCK_EUNSUPPORTED, "box grids are not covered by the no-allocation scan");
    if (in.args.wide.corr)
        return fftdock::ctx_fail(ctx, FFTDOCK_EUNSUPPORTED,
                                 "translational clustering needs a full correlation grid per rotation; the "
                                 "no-allocation scan does not cover it");
    if (scratch_bytes(in, 1) > kScratchBytes) {
        const std::string msg = "one rotation of this context needs " + std::to_string(scratch_bytes(in, 1)) +
                                " bytes of work memory; the no-allocation scan has " +
                                std::to_string(kScratchBytes);
        return fftdock::ctx_fail(ctx, FFTDOCK_EINVAL, msg.c_str());
    }
    if (!in.noalloc_scratch)
        return fftdock::ctx_fail(ctx, FFTDOCK_ECUDA, "the no-allocation scan's array was not resolved");
    fftdock::DeviceScope dev_scope(in.device);
    cudaError_t e = dev_scope.status();
    if (e != cudaSuccess) return fftdock::ctx_fail(ctx, FFTDOCK_ECUDA, cudaGetErrorString(e));
    unsigned char* base = static_cast<unsigned char*>(in.noalloc_scratch);
    int b = in.B;
    while (b > 1 && scratch_bytes(in, b) > kScratchBytes) --b;

    fftdock::BatchArgs a = in.args;
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        unsigned char* p = base + off;
        off += align256(bytes);
        return p;
    };
    int32_t* status = reinterpret_cast<int32_t*>(carve(sizeof(int32_t) * (size_t)b));
    a.ent = reinterpret_cast<uint32_t*>(carve(sizeof(uint32_t) * (size_t)b * in.n_ent));
    a.offs = reinterpret_cast<int32_t*>(carve(sizeof(int32_t) * (size_t)b * ((size_t)in.K * in.N + 1)));
    a.cand_v = reinterpret_cast<float*>(carve(sizeof(float) * (size_t)b * in.N * kKC));
    a.cand_i = reinterpret_cast<int32_t*>(carve(sizeof(int32_t) * (size_t)b * in.N * kKC));
    a.g2 = reinterpret_cast<float2*>(carve(sizeof(float2) * (size_t)b * in.N * in.PP));
    a.dbg_corr = nullptr;
    a.pool_v = nullptr;
    a.pool_i = nullptr;
    a.ev = nullptr;
    // the FFT form of the pencil stage: its work memory fits the static array
    a.use_tc = 0;
    a.ent_t = nullptr;
    cudaStream_t s = stream ? (cudaStream_t)stream : in.stream;
    for (int b0 = 0; b0 < n_rot; b0 += b) {
        a.n_rot = n_rot - b0 < b ? n_rot - b0 : b;
        a.rot = d_rot + (size_t)b0 * 9;
        a.status = status;
        a.peaks = d_peaks + (size_t)b0 * a.peak_stride;
        a.n_peaks = d_n_peaks + b0;
        a.first_rot_id = first_rot_id + b0;
        e = in.ops->scan_batch(a, s);
        if (e != cudaSuccess)
            return fftdock::ctx_fail(ctx, FFTDOCK_ECUDA, (std::string("scan batch: ") + cudaGetErrorString(e)).c_str());
    }
    return FFTDOCK_OK;
}
