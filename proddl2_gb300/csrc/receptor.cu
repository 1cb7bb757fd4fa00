// Receptor term grids in real space (once per pair, FP64): shape flags,
// per-type desolvation densities and their mixing into the K folded terms.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

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
        int lo = logical_q(__dsub_rn(c[d], cut), g, d) - 1;
        int hi = logical_q(__dadd_rn(c[d], cut), g, d) - 1;
        b.lo[d] = max(lo, 0);
        b.hi[d] = min(hi, g.n[d] - 1);
        if (b.lo[d] > b.hi[d]) return false;
    }
    return true;
}

__device__ __forceinline__ double dist2(const double* c, int ix, int iy, int iz, const Geo& g) {
    const double dx = __dsub_rn(cell_centre(ix, g, 0), c[0]);
    const double dy = __dsub_rn(cell_centre(iy, g, 1), c[1]);
    const double dz = __dsub_rn(cell_centre(iz, g, 2), c[2]);
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
        if (f) atomicMax(&flags[((size_t)ix * g.n[1] + iy) * g.n[2] + iz], f);
    }
}

// each atom's cropped projection box (project.hpp:87-98); empty boxes get
// lo > hi
__global__ void atom_box_kernel(const double* __restrict__ xyz, int n, Geo g, double cut, int* __restrict__ box) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const double c[3] = {xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]};
    Box b;
    const bool ok = projection_box(c, cut, g, b);
    for (int d = 0; d < 3; ++d) {
        box[6 * a + d] = ok ? b.lo[d] : 1;
        box[6 * a + 3 + d] = ok ? b.hi[d] : 0;
    }
}

// per-type desolvation density G_tau(x) = sum_i g(r) (PotAce::f2,
// potentials_inc.hpp:394-397; projection as project.hpp:143-159: atom i
// reaches cell x if x lies in i's cropped box and r^2 <= cut^2, r^2 clamped
// to minDist^2).  Gathered per cell over the atoms of the 27 neighbouring
// bins, bins and atoms in a fixed order: the sums do not depend on thread
// scheduling.
__global__ void ace_density_kernel(const double* __restrict__ xyz, const int32_t* __restrict__ type,
                                   const int* __restrict__ box, AtomBins bins, Geo g, double cut2, double mind2,
                                   double ab, double ak, double aa, double* __restrict__ dens) {
    const size_t V = (size_t)g.n[0] * g.n[1] * g.n[2];
    const size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= V) return;
    const int ix = (int)(cell / ((size_t)g.n[1] * g.n[2])), iy = (int)((cell / g.n[2]) % g.n[1]),
              iz = (int)(cell % g.n[2]);
    const int ic[3] = {ix, iy, iz};
    int b0[3];
    for (int d = 0; d < 3; ++d) {
        const double t = floor((cell_centre(ic[d], g, d) - bins.lo[d]) / bins.size);
        b0[d] = t < -2.0 ? -2 : (t > (double)bins.nb[d] + 1.0 ? bins.nb[d] + 1 : (int)t);
    }
    for (int bx = max(b0[0] - 1, 0); bx <= min(b0[0] + 1, bins.nb[0] - 1); ++bx)
        for (int by = max(b0[1] - 1, 0); by <= min(b0[1] + 1, bins.nb[1] - 1); ++by)
            for (int bz = max(b0[2] - 1, 0); bz <= min(b0[2] + 1, bins.nb[2] - 1); ++bz) {
                const int bin = (bx * bins.nb[1] + by) * bins.nb[2] + bz;
                for (int k = bins.start[bin]; k < bins.start[bin + 1]; ++k) {
                    const int a = bins.atoms[k];
                    const int* bb = box + 6 * a;
                    if (ix < bb[0] || ix > bb[3] || iy < bb[1] || iy > bb[4] || iz < bb[2] || iz > bb[5]) continue;
                    const double c[3] = {xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]};
                    double r2 = dist2(c, ix, iy, iz, g);
                    if (r2 <= cut2) {
                        if (r2 < mind2) r2 = mind2;
                        const double r = sqrt(r2);
                        const double val =
                            __ddiv_rn(1.0, __dadd_rn(1.0, exp(__dmul_rn(ab, __dsub_rn(__dmul_rn(ak, r), aa)))));
                        double* dt = dens + (size_t)type[a] * V + cell;
                        *dt = __dadd_rn(*dt, val);
                    }
                }
            }
}

// The reference's LJ fields (SoftCoreLJRep / SoftCoreLJAttr for ljComp,
// SoftCoreLJ with the force-shifted cutoff for ljAvg; potentials_inc.hpp:
// 142-354), projected like ProjectorRadialField::projectFields
// (project.hpp:143-176): each cell gathers, in a fixed bin and atom order,
// f2(max(r^2, minDist^2)) of every atom whose cropped box holds it and with
// r^2 <= cut^2.  K = 2 (ljComp: repulsion, attraction) or 1 (ljAvg).
template <int K>
__global__ void lj_field_kernel(const double* __restrict__ xyz, const double* __restrict__ lc,
                                const int* __restrict__ box, AtomBins bins, Geo g, double cut2, double mind2,
                                double* __restrict__ rgrid) {
    const size_t V = (size_t)g.n[0] * g.n[1] * g.n[2];
    const size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= V) return;
    const int ix = (int)(cell / ((size_t)g.n[1] * g.n[2])), iy = (int)((cell / g.n[2]) % g.n[1]),
              iz = (int)(cell % g.n[2]);
    const int ic[3] = {ix, iy, iz};
    int b0[3];
    for (int d = 0; d < 3; ++d) {
        const double t = floor((cell_centre(ic[d], g, d) - bins.lo[d]) / bins.size);
        b0[d] = t < -2.0 ? -2 : (t > (double)bins.nb[d] + 1.0 ? bins.nb[d] + 1 : (int)t);
    }
    double acc0 = 0.0, acc1 = 0.0;
    for (int bx = max(b0[0] - 1, 0); bx <= min(b0[0] + 1, bins.nb[0] - 1); ++bx)
        for (int by = max(b0[1] - 1, 0); by <= min(b0[1] + 1, bins.nb[1] - 1); ++by)
            for (int bz = max(b0[2] - 1, 0); bz <= min(b0[2] + 1, bins.nb[2] - 1); ++bz) {
                const int bin = (bx * bins.nb[1] + by) * bins.nb[2] + bz;
                for (int k = bins.start[bin]; k < bins.start[bin + 1]; ++k) {
                    const int a = bins.atoms[k];
                    const int* bb = box + 6 * a;
                    if (ix < bb[0] || ix > bb[3] || iy < bb[1] || iy > bb[4] || iz < bb[2] || iz > bb[5]) continue;
                    const double c[3] = {xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]};
                    double r2 = dist2(c, ix, iy, iz, g);
                    if (r2 <= cut2) {
                        if (r2 < mind2) r2 = mind2;
                        const double* p = lc + 5 * a;  // as6, 4es6, 4es12, fshift, gshift
                        const double A = __dadd_rn(__dmul_rn(__dmul_rn(r2, r2), r2), p[0]);
                        if constexpr (K == 2) {
                            acc0 = __dadd_rn(acc0, __ddiv_rn(__ddiv_rn(p[2], A), A));
                            acc1 = __dadd_rn(acc1, __ddiv_rn(-p[1], A));
                        } else {
                            const double f = __dadd_rn(
                                __dadd_rn(__ddiv_rn(__dsub_rn(__ddiv_rn(p[2], A), p[1]), A), p[3]),
                                __dmul_rn(p[4], sqrt(r2)));
                            acc0 = __dadd_rn(acc0, f);
                        }
                    }
                }
            }
    rgrid[cell] = acc0;
    if constexpr (K == 2) rgrid[V + cell] = acc1;
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
    const size_t V = (size_t)a.geo.n[0] * a.geo.n[1] * a.geo.n[2];
    if (a.term_set == FFTDOCK_TERMS_LJ_COMP || a.term_set == FFTDOCK_TERMS_LJ_AVG) {
        const double md = a.geo.h / 4.0;
        cudaError_t e = cudaSuccess;
        if (a.n > 0) {
            atom_box_kernel<<<(a.n + 127) / 128, 128, 0, s>>>(a.xyz, a.n, a.geo, a.lj_cut, a.box);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        const unsigned blocks = (unsigned)((V + 255) / 256);
        if (a.term_set == FFTDOCK_TERMS_LJ_COMP)
            lj_field_kernel<2><<<blocks, 256, 0, s>>>(a.xyz, a.lj_c, a.box, a.bins, a.geo, a.lj_cut * a.lj_cut,
                                                       md * md, a.rgrid);
        else
            lj_field_kernel<1><<<blocks, 256, 0, s>>>(a.xyz, a.lj_c, a.box, a.bins, a.geo, a.lj_cut * a.lj_cut,
                                                       md * md, a.rgrid);
        return cudaGetLastError();
    }
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
            atom_box_kernel<<<(a.n + 127) / 128, 128, 0, s>>>(a.xyz, a.n, a.geo, a.ace_cut, a.box);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            ace_density_kernel<<<(unsigned)((V + 255) / 256), 256, 0, s>>>(
                a.xyz, a.type, a.box, a.bins, a.geo, a.ace_cut * a.ace_cut, md * md, a.ace_b, a.ace_k, a.ace_a,
                a.dens);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
    }
    mix_terms_kernel<<<(unsigned)((V + 255) / 256), 256, 0, s>>>(a.flags, a.dens, a.emat, a.n_types, a.K,
                                                                  a.term_set, V, a.rgrid);
    return cudaGetLastError();
}

// counting sort of the atoms into bins of edge cut * (1 + 1e-6) (at least
// 1e-3 A), atoms in index order inside each bin
void bin_atoms(const double* xyz, int n, double cut, HostAtomBins& out) {
    out.size = std::max(cut * (1.0 + 1e-6), 1e-3);
    double hi[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d) out.lo[d] = n > 0 ? xyz[d] : 0.0;
    for (int d = 0; d < 3; ++d) hi[d] = out.lo[d];
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            out.lo[d] = std::min(out.lo[d], xyz[3 * i + d]);
            hi[d] = std::max(hi[d], xyz[3 * i + d]);
        }
    for (int d = 0; d < 3; ++d) out.nb[d] = (int)std::floor((hi[d] - out.lo[d]) / out.size) + 1;
    const int nbins = out.nb[0] * out.nb[1] * out.nb[2];
    std::vector<int> bin(n);
    out.start.assign(nbins + 1, 0);
    for (int i = 0; i < n; ++i) {
        int b[3];
        for (int d = 0; d < 3; ++d) {
            b[d] = (int)std::floor((xyz[3 * i + d] - out.lo[d]) / out.size);
            b[d] = std::min(std::max(b[d], 0), out.nb[d] - 1);
        }
        bin[i] = (b[0] * out.nb[1] + b[1]) * out.nb[2] + b[2];
        ++out.start[bin[i] + 1];
    }
    for (int k = 0; k < nbins; ++k) out.start[k + 1] += out.start[k];
    out.atoms.assign(n, 0);
    std::vector<int> fill(out.start.begin(), out.start.end() - 1);
    for (int i = 0; i < n; ++i) out.atoms[fill[bin[i]]++] = i;
}

}  // namespace fftdock
