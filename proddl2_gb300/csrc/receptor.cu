// Receptor term grids in real space (once per pair, FP64): shape flags,
// per-type desolvation densities and their mixing into the K folded terms.
#include <cuda_runtime.h>

#include "internal.h"
#include "scan_kernels.cuh"

namespace fftdock {
namespace {

// ---------------------------------------------------------------------------
// Receptor builders (once per pair; FP64)
// ---------------------------------------------------------------------------
// Cells of the cropped toLogical(c +- cut) box (project.hpp:87-98).
struct Box {
    int lo[3], hi[3];
};
__device__ __forceinline__ bool projection_box(const double* c, double cut, const Geo& g, Box& b) {
    for (int d = 0; d < 3; ++d) {
        int lo = logical_q(__dsub_rn(c[d], cut), g) - 1;
        int hi = logical_q(__dadd_rn(c[d], cut), g) - 1;
        b.lo[d] = max(lo, 0);
        b.hi[d] = min(hi, g.n - 1);
        if (b.lo[d] > b.hi[d]) return false;
    }
    return true;
}

__device__ __forceinline__ double dist2(const double* c, int ix, int iy, int iz, const Geo& g) {
    const double dx = __dsub_rn(cell_centre(ix, g), c[0]);
    const double dy = __dsub_rn(cell_centre(iy, g), c[1]);
    const double dz = __dsub_rn(cell_centre(iz, g), c[2]);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// shape term flags: 2 = core (r^2 <= rc2), 1 = surface (r^2 <= rs2)
__global__ void shape_flags_kernel(const double* __restrict__ xyz, int n, Geo g, double cut, double rc2, double rs2,
                                   int* __restrict__ flags) {
    const int a = blockIdx.x;
    if (a >= n) return;
    const double c[3] = {xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]};
    Box b;
    if (!projection_box(c, cut, g, b)) return;
    const int nx = b.hi[0] - b.lo[0] + 1, ny = b.hi[1] - b.lo[1] + 1, nz = b.hi[2] - b.lo[2] + 1;
    const int tot = nx * ny * nz;
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
        const int ix = b.lo[0] + i / (ny * nz), iy = b.lo[1] + (i / nz) % ny, iz = b.lo[2] + i % nz;
        const double r2 = dist2(c, ix, iy, iz, g);
        const int f = r2 <= rc2 ? 2 : (r2 <= rs2 ? 1 : 0);
        if (f) atomicMax(&flags[((size_t)ix * g.n + iy) * g.n + iz], f);
    }
}

// per-type desolvation density G_tau(x) = sum_i g(r) (PotAce::f2,
// potentials_inc.hpp:394-397; projection as project.hpp:143-159)
__global__ void ace_density_kernel(const double* __restrict__ xyz, const int32_t* __restrict__ type, int n, Geo g,
                                   double cut, double cut2, double mind2, double ab, double ak, double aa,
                                   double* __restrict__ dens) {
    const int a = blockIdx.x;
    if (a >= n) return;
    const double c[3] = {xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]};
    Box b;
    if (!projection_box(c, cut, g, b)) return;
    const size_t V = (size_t)g.n * g.n * g.n;
    double* dt = dens + (size_t)type[a] * V;
    const int nx = b.hi[0] - b.lo[0] + 1, ny = b.hi[1] - b.lo[1] + 1, nz = b.hi[2] - b.lo[2] + 1;
    const int tot = nx * ny * nz;
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
        const int ix = b.lo[0] + i / (ny * nz), iy = b.lo[1] + (i / nz) % ny, iz = b.lo[2] + i % nz;
        double r2 = dist2(c, ix, iy, iz, g);
        if (r2 <= cut2) {
            if (r2 < mind2) r2 = mind2;
            const double r = sqrt(r2);
            const double val = __ddiv_rn(1.0, __dadd_rn(1.0, exp(__dmul_rn(ab, __dsub_rn(__dmul_rn(ak, r), aa)))));
            atomicAdd(&dt[((size_t)ix * g.n + iy) * g.n + iz], val);
        }
    }
}

// R_t = sum_u E[u][t] G_u - S (shape+ACE, folded) or R_0 = -S (shape)
__global__ void mix_terms_kernel(const int* __restrict__ flags, const double* __restrict__ dens,
                                 const double* __restrict__ emat, int n_types, int K, int term_set, size_t V,
                                 double* __restrict__ rgrid) {
    const size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= V) return;
    const int f = flags[cell];
    const double s = f == 2 ? -15.0 : (f == 1 ? 1.0 : 0.0);
    if (term_set == FFTDOCK_TERMS_SHAPE) {
        rgrid[cell] = -s;
        return;
    }
    for (int t = 0; t < K; ++t) {
        double d = 0.0;
        for (int u = 0; u < n_types; ++u) d = __dadd_rn(d, __dmul_rn(emat[u * n_types + t], dens[(size_t)u * V + cell]));
        rgrid[(size_t)t * V + cell] = __dsub_rn(d, s);
    }
}

}  // namespace

cudaError_t build_receptor_grids(const ReceptorGridArgs& a, cudaStream_t s) {
    const size_t V = (size_t)a.geo.n * a.geo.n * a.geo.n;
    cudaError_t e = cudaMemsetAsync(a.flags, 0, V * sizeof(int), s);
    if (e != cudaSuccess) return e;
    if (a.n > 0) {
        const double cut = a.shape_core + a.shape_width;
        shape_flags_kernel<<<a.n, 128, 0, s>>>(a.xyz, a.n, a.geo, cut, a.shape_core * a.shape_core, cut * cut,
                                               a.flags);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (a.term_set == FFTDOCK_TERMS_SHAPE_ACE) {
        e = cudaMemsetAsync(a.dens, 0, (size_t)a.n_types * V * sizeof(double), s);
        if (e != cudaSuccess) return e;
        const double md = a.geo.h / 4.0;
        if (a.n > 0) {
            ace_density_kernel<<<a.n, 256, 0, s>>>(a.xyz, a.type, a.n, a.geo, a.ace_cut, a.ace_cut * a.ace_cut,
                                                   md * md, a.ace_b, a.ace_k, a.ace_a, a.dens);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
    }
    mix_terms_kernel<<<(unsigned)((V + 255) / 256), 256, 0, s>>>(a.flags, a.dens, a.emat, a.n_types, a.K,
                                                                  a.term_set, V, a.rgrid);
    return cudaGetLastError();
}

}  // namespace fftdock
