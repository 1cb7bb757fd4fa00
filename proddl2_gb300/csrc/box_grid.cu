// The scan on box grids: FFT sizes chosen per axis (Nx, Ny, Nz), as the
// reference sizes its grid (findBestSize<N_dim> per axis over the padded
// receptor box, include/PRODDL/docking_fft.hpp:541-553 and
// include/PRODDL/Math/fft.hpp:141-168), and cubic edges without a compiled
// plan.  Same pipeline and conventions as the cubic kernels -- ligand prep
// (rotate, toLogical per axis, stable sort by (term, x)), pencil stage
// (y/z stages as direct sums over the ligand's entries, x transform,
// spectrum product summed over terms, inverse x transform), plane stage
// (inverse y transform, real inverse z transform, exact per-plane top 16),
// finalize (merge, FP64 direct-space rescoring, sort, maxValCorr, unwrap per
// axis) -- with every transform length a runtime value: one warp per line
// runs a mixed-radix Stockham FFT (radices 4, 6, 2, 9, 3, 5, 7, 11, 13 in
// that order of preference) out of shared memory with a twiddle table per
// axis (even-length plane rows: two lines per warp, 16 lanes each).  The receptor's transforms
// run the same line FFT in FP64.
//
// Layout (Hz = Nz/2 + 1, pencil p = ky Hz + kz, PP = Ny Hz rounded up to 32):
//   spec  [K][PP][Nx]  float2  R^_t(kx, p) / V (pencil-major: coalesced along kx)
//   rgrid [K][V]       double  real-space receptor terms (FP64 rescoring)
//   ent   [B][n_ent]   uint32  t << 24 | x << 16 | y << 8 | z, sorted by (t, x)
//   offs  [B][K Nx+1]  int32   start of bin (t, x)
//   g2    [B][Nx][PP]  float2  per-x complex (ky, kz) planes
//   cand  [B][Nx][16]          per-plane FP32 candidate pools
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "fft_core.cuh"
#include "internal.h"
#include "pencil_tc.cuh"
#include "scan_kernels.cuh"

namespace fftdock {

namespace {

constexpr int kBoxWarps = 8;  // lines (pencils, columns, rows) per CTA

// radices in Stockham stage order; false if n has another prime factor
bool factor_plan(int n, BoxPlan& pl) {
    static const int radices[] = {4, 6, 2, 9, 3, 5, 7, 11, 13};
    pl.n = n;
    pl.nf = 0;
    int m = n;
    for (int r : radices)
        while (m % r == 0 && pl.nf < kBoxMaxFactors) {
            pl.f[pl.nf++] = r;
            m /= r;
        }
    return m == 1 && n >= 2;
}

template <typename T2> __device__ __forceinline__ T2 c_mul(T2 a, T2 b) {
    T2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
// table entry W_n^m = e^{-2 pi i m / n}, conjugated for the inverse transform
template <typename T2, int SIGN> __device__ __forceinline__ T2 tw_at(const T2* tw, int m) {
    T2 w = tw[m];
    if (SIGN > 0) w.y = -w.y;
    return w;
}

// one Stockham stage of radix R over a line of n points held in src:
// butterfly j reads src[j + r n/R], applies the twiddles W^(j mod Ns) r n/(Ns R),
// and writes its R-point DFT to dst[(j / Ns) Ns R + j mod Ns + k Ns].  The
// twiddle index (j mod Ns) r n/(Ns R) stays below n; the R-th roots of unity
// are held in registers for the whole stage, radices 2 and 4 need none, 6
// is two 3-point DFTs joined by W6 twiddles.  LS lanes share one line
// (butterflies j = lane, lane + LS, ..).
template <typename T2, int SIGN, int R, int LS = 32>
__device__ __forceinline__ void stockham_stage(const T2* src, T2* dst, const T2* tw, int n, int ns, int lane) {
    using S = decltype(T2::x);
    const int nb = n / R;
    const int tstep = n / (ns * R);
    // j / ns as a multiply-high by ceil(2^32 / ns) (ns > 1): exact for
    // j < 2^32 / ns^2 (here j < 256 and ns <= 256)
    const unsigned magic = ns > 1 ? 0xffffffffu / (unsigned)ns + 1u : 0u;
    T2 root[R];
    root[0].x = 1;  // W^0 (a composite odd radix pairs some q k = 0 mod R)
    root[0].y = 0;
#pragma unroll
    for (int m = 1; m < R; ++m) root[m] = tw_at<T2, SIGN>(tw, m * nb);
    for (int j = lane; j < nb; j += LS) {
        T2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = src[j + r * nb];
        const int jq = ns > 1 ? (int)__umulhi((unsigned)j, magic) : j;
        const int jm = j - jq * ns;
        const int step = jm * tstep;
#pragma unroll
        for (int r = 1; r < R; ++r) v[r] = c_mul(v[r], tw_at<T2, SIGN>(tw, step * r));
        T2* out = dst + jq * ns * R + jm;
        if constexpr (R == 2) {
            T2 o0 = v[0], o1 = v[0];
            o0.x += v[1].x; o0.y += v[1].y;
            o1.x -= v[1].x; o1.y -= v[1].y;
            out[0] = o0;
            out[ns] = o1;
        } else if constexpr (R == 6) {
            // two 3-point DFTs of the even and odd inputs, the odd ones
            // turned by W6^k (W6 = e^(SIGN i pi / 3)): out_k = e_k + W6^k o_k,
            // out_(k+3) = e_k - W6^k o_k
            constexpr S c3 = (S)0.86602540378443864676;  // sin(pi / 3)
            constexpr S sg = SIGN < 0 ? (S)-1 : (S)1;
            T2 e3[3], o3[3];
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                const T2 x0 = v[t], x1 = v[t + 2], x2 = v[t + 4];
                T2 sm, df, u;
                sm.x = x1.x + x2.x; sm.y = x1.y + x2.y;
                df.x = sg * c3 * (x1.x - x2.x); df.y = sg * c3 * (x1.y - x2.y);
                u.x = x0.x - (S)0.5 * sm.x; u.y = x0.y - (S)0.5 * sm.y;
                T2* y = t == 0 ? e3 : o3;
                y[0].x = x0.x + sm.x; y[0].y = x0.y + sm.y;
                // y1 = u + i df, y2 = u - i df
                y[1].x = u.x - df.y; y[1].y = u.y + df.x;
                y[2].x = u.x + df.y; y[2].y = u.y - df.x;
            }
            // W6 = (1/2, sg c3), W6^2 = (-1/2, sg c3)
            T2 t1, t2;
            t1.x = (S)0.5 * o3[1].x - sg * c3 * o3[1].y; t1.y = (S)0.5 * o3[1].y + sg * c3 * o3[1].x;
            t2.x = (S)-0.5 * o3[2].x - sg * c3 * o3[2].y; t2.y = (S)-0.5 * o3[2].y + sg * c3 * o3[2].x;
            T2 o;
            o.x = e3[0].x + o3[0].x; o.y = e3[0].y + o3[0].y; out[0] = o;
            o.x = e3[1].x + t1.x; o.y = e3[1].y + t1.y; out[ns] = o;
            o.x = e3[2].x + t2.x; o.y = e3[2].y + t2.y; out[2 * ns] = o;
            o.x = e3[0].x - o3[0].x; o.y = e3[0].y - o3[0].y; out[3 * ns] = o;
            o.x = e3[1].x - t1.x; o.y = e3[1].y - t1.y; out[4 * ns] = o;
            o.x = e3[2].x - t2.x; o.y = e3[2].y - t2.y; out[5 * ns] = o;
        } else if constexpr (R == 4) {
            // W4 = e^(SIGN i pi / 2): out1 = (v0 - v2) + W4 (v1 - v3), out3 = (v0 - v2) - W4 (v1 - v3)
            T2 a, b, c, d, e;
            a.x = v[0].x + v[2].x; a.y = v[0].y + v[2].y;
            b.x = v[0].x - v[2].x; b.y = v[0].y - v[2].y;
            c.x = v[1].x + v[3].x; c.y = v[1].y + v[3].y;
            e.x = v[1].x - v[3].x; e.y = v[1].y - v[3].y;
            if (SIGN < 0) { d.x = e.y; d.y = -e.x; } else { d.x = -e.y; d.y = e.x; }
            T2 o;
            o.x = a.x + c.x; o.y = a.y + c.y; out[0] = o;
            o.x = b.x + d.x; o.y = b.y + d.y; out[ns] = o;
            o.x = a.x - c.x; o.y = a.y - c.y; out[2 * ns] = o;
            o.x = b.x - d.x; o.y = b.y - d.y; out[3 * ns] = o;
        } else {
            // odd R: pairs a_q = v_q + v_(R-q), b_q = v_q - v_(R-q); with
            // root[m] = (cos, s sin) of the stage's direction,
            // out_k = v0 + sum_q cos(qk) a_q + i sum_q s sin(qk) b_q and
            // out_(R-k) the same with - i
            constexpr int P = (R - 1) / 2;
            T2 o0 = v[0];
#pragma unroll
            for (int q = 1; q <= P; ++q) {
                o0.x += v[q].x + v[R - q].x;
                o0.y += v[q].y + v[R - q].y;
            }
            out[0] = o0;
#pragma unroll
            for (int k = 1; k <= P; ++k) {
                T2 re = v[0];
                S ix = 0, iy = 0;
#pragma unroll
                for (int q = 1; q <= P; ++q) {
                    const T2 w = root[(q * k) % R];
                    re.x += w.x * (v[q].x + v[R - q].x);
                    re.y += w.x * (v[q].y + v[R - q].y);
                    ix += w.y * (v[q].x - v[R - q].x);
                    iy += w.y * (v[q].y - v[R - q].y);
                }
                // i (ix + i iy) = (-iy, ix)
                T2 o;
                o.x = re.x - iy; o.y = re.y + ix; out[k * ns] = o;
                o.x = re.x + iy; o.y = re.y - ix; out[(R - k) * ns] = o;
            }
        }
    }
}

// Unnormalised DFT of the warp's line in a (n points), b a second buffer of
// n points; returns the buffer that holds the result.  SIGN -1: forward
// e^{-2 pi i jk/n}; +1: inverse.  Ends with __syncwarp.  MAXR < 11: the plan
// has no factor 11 or 13 (those stages are not compiled: fewer registers).
// LS = 16: two lines per warp, lane = the thread's index within its half
// (each half passes its own line's buffers).
template <typename T2, int SIGN, int MAXR = 13, int LS = 32>
__device__ T2* warp_fft(T2* a, T2* b, const T2* tw, const BoxPlan& pl, int lane) {
    T2* src = a;
    T2* dst = b;
    int ns = 1;
    __syncwarp();
    for (int s = 0; s < pl.nf; ++s) {
        const int R = pl.f[s];
        switch (R) {
            case 4: stockham_stage<T2, SIGN, 4, LS>(src, dst, tw, pl.n, ns, lane); break;
            case 6: stockham_stage<T2, SIGN, 6, LS>(src, dst, tw, pl.n, ns, lane); break;
            case 2: stockham_stage<T2, SIGN, 2, LS>(src, dst, tw, pl.n, ns, lane); break;
            case 3: stockham_stage<T2, SIGN, 3, LS>(src, dst, tw, pl.n, ns, lane); break;
            case 5: stockham_stage<T2, SIGN, 5, LS>(src, dst, tw, pl.n, ns, lane); break;
            case 7: stockham_stage<T2, SIGN, 7, LS>(src, dst, tw, pl.n, ns, lane); break;
            case 9: stockham_stage<T2, SIGN, 9, LS>(src, dst, tw, pl.n, ns, lane); break;
            default:
                if constexpr (MAXR >= 11) {
                    if (R == 11) stockham_stage<T2, SIGN, 11, LS>(src, dst, tw, pl.n, ns, lane);
                    else stockham_stage<T2, SIGN, 13, LS>(src, dst, tw, pl.n, ns, lane);
                }
                break;
        }
        __syncwarp();
        T2* t = src;
        src = dst;
        dst = t;
        ns *= R;
    }
    return src;
}

// ---------------------------------------------------------------------------
// receptor transforms (FP64), one warp per line: line L starts at
// (L / inner_count) outer_stride + (L % inner_count) inner_stride, element e
// at + e elem_stride; in place
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32 * kBoxWarps) box_line_fft64_kernel(double2* __restrict__ data,
                                                                       const double2* __restrict__ tw, BoxPlan pl,
                                                                       long n_lines, long elem_stride,
                                                                       long inner_count, long inner_stride,
                                                                       long outer_stride) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = pl.n;
    double2* tws = reinterpret_cast<double2*>(smem_raw);  // [n]
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double2* a = tws + n + (size_t)w * 2 * n;
    double2* b = a + n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) tws[i] = tw[i];
    __syncthreads();
    const long L = (long)blockIdx.x * kBoxWarps + w;
    if (L >= n_lines) return;
    double2* line = data + (L / inner_count) * outer_stride + (L % inner_count) * inner_stride;
    for (int e = lane; e < n; e += 32) a[e] = line[(long)e * elem_stride];
    const double2* r = warp_fft<double2, -1>(a, b, tws, pl, lane);
    for (int e = lane; e < n; e += 32) line[(long)e * elem_stride] = r[e];
}

// half spectrum [Nx][Ny Hz] (FP64) -> the pencil stage's spectra [PP][Nx]
// (FP32, scaled; pencils past Ny Hz are zero): a warp reads one pencil's
// kx values as consecutive words
__global__ void box_pack_spectrum_kernel(const double2* __restrict__ half, float2* __restrict__ spec, int nx,
                                         int nh, int pp, double scale) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t tot = (size_t)nx * pp;
    if (i >= tot) return;
    const size_t p = i / nx;
    const int kx = (int)(i - p * nx);
    float2 o = make_float2(0.f, 0.f);
    if (p < (size_t)nh) {
        const double2 v = half[(size_t)kx * nh + p];
        o = make_float2((float)(v.x * scale), (float)(v.y * scale));
    }
    spec[i] = o;
}

// [Nx][Ny][Nz] complex -> [Nx][Ny][Hz]
__global__ void box_half_extract_kernel(const double2* __restrict__ full, double2* __restrict__ half, int nx, int ny,
                                        int nz, int hz) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t tot = (size_t)nx * ny * hz;
    if (i >= tot) return;
    const size_t row = i / hz;
    const int kz = (int)(i - row * hz);
    half[i] = full[row * nz + kz];
}

// ---------------------------------------------------------------------------
// ligand prep: rotate (the reference's operation order, no FMA), toLogical
// per axis, bins (t, x), stable sort (one CTA per rotation)
// ---------------------------------------------------------------------------
// ent_t (tensor form): the transposed entries of ligand_prep_kernel
__global__ void __launch_bounds__(256) box_prep_kernel(const double* __restrict__ rot,
                                                       const double* __restrict__ lig_xyz,
                                                       const int32_t* __restrict__ lig_term, int n_ent, int K, Geo geo,
                                                       uint32_t* __restrict__ ent_out, int32_t* __restrict__ offs_out,
                                                       int32_t* __restrict__ status, const float* __restrict__ w_in,
                                                       float* __restrict__ w_out, int32_t* __restrict__ idx_out,
                                                       uint32_t* __restrict__ ent_t, const int32_t* __restrict__ tpad,
                                                       int n_pad, int x0, int W) {
    extern __shared__ unsigned char smem_raw[];
    const int nx = geo.n[0], ny = geo.n[1], nz = geo.n[2];
    const int nbins = K * nx;
    int32_t* cnt = reinterpret_cast<int32_t*>(smem_raw);           // [K*Nx + 1]
    uint32_t* keys = reinterpret_cast<uint32_t*>(cnt + nbins + 1);  // [n_ent]
    __shared__ int bad;
    __shared__ int wsum[8];
    const int q = blockIdx.x;
    const int tid = threadIdx.x;
    for (int i = tid; i <= nbins; i += blockDim.x) cnt[i] = 0;
    if (tid == 0) bad = 0;
    __syncthreads();
    const double* m = rot + 9 * (size_t)q;
    for (int i = tid; i < n_ent; i += blockDim.x) {
        const double x0 = lig_xyz[3 * i], x1 = lig_xyz[3 * i + 1], x2 = lig_xyz[3 * i + 2];
        const double p0 = __dadd_rn(__dadd_rn(__dmul_rn(m[0], x0), __dmul_rn(m[1], x1)), __dmul_rn(m[2], x2));
        const double p1 = __dadd_rn(__dadd_rn(__dmul_rn(m[3], x0), __dmul_rn(m[4], x1)), __dmul_rn(m[5], x2));
        const double p2 = __dadd_rn(__dadd_rn(__dmul_rn(m[6], x0), __dmul_rn(m[7], x1)), __dmul_rn(m[8], x2));
        int c0 = logical_q(p0, geo, 0), c1 = logical_q(p1, geo, 1), c2 = logical_q(p2, geo, 2);
        const bool ok = c0 >= 1 && c0 <= nx && c1 >= 1 && c1 <= ny && c2 >= 1 && c2 <= nz;
        if (!ok) atomicOr(&bad, 1);
        // out-of-grid atoms are clamped for memory safety; the rotation is
        // reported and gives no peaks
        c0 = min(max(c0 - 1, 0), nx - 1);
        c1 = min(max(c1 - 1, 0), ny - 1);
        c2 = min(max(c2 - 1, 0), nz - 1);
        const int t = lig_term[i];
        keys[i] = ((uint32_t)t << 24) | ((uint32_t)c0 << 16) | ((uint32_t)c1 << 8) | (uint32_t)c2;
        atomicAdd(&cnt[t * nx + c0], 1);
    }
    __syncthreads();
    {
        const int per = (nbins + blockDim.x - 1) / blockDim.x;
        const int b0 = min(tid * per, nbins), b1 = min(b0 + per, nbins);
        int local = 0;
        for (int i = b0; i < b1; ++i) local += cnt[i];
        const int lane = tid & 31, wid = tid >> 5;
        int incl = local;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        int wbase = 0;
        for (int k = 0; k < wid; ++k) wbase += wsum[k];
        int run = wbase + incl - local;
        for (int i = b0; i < b1; ++i) {
            const int c = cnt[i];
            cnt[i] = run;
            run += c;
        }
        __syncthreads();
        if (tid == 0) cnt[nbins] = n_ent;
        __syncthreads();
    }
    int32_t* offs = offs_out + (size_t)q * (nbins + 1);
    for (int i = tid; i <= nbins; i += blockDim.x) offs[i] = cnt[i];
    __syncthreads();
    if (tid < 32) {
        uint32_t* ent = ent_out + (size_t)q * n_ent;
        for (int base = 0; base < n_ent; base += 32) {
            const int i = base + tid;
            const bool act = i < n_ent;
            const uint32_t key = act ? keys[i] : 0xffffffffu;
            const int bin = act ? (int)((key >> 24) * nx + ((key >> 16) & 255u)) : -1;
            const unsigned peers = __match_any_sync(0xffffffffu, bin);
            const int rank = __popc(peers & ((1u << tid) - 1u));
            const int leader = __ffs(peers) - 1;
            int dst = 0;
            if (act) dst = cnt[bin] + rank;
            __syncwarp();
            if (act) ent[dst] = key;
            // [q / 128][row / 4][q % 128][row % 4], x relative to x0 (cells
            // outside the window at the dummy row W), as in ligand_prep_kernel
            if (act && ent_t) {
                const size_t row = (size_t)(dst + __ldg(tpad + (key >> 24)));
                ent_t[(((size_t)(q >> 7) * (n_pad >> 2) + (row >> 2)) * 128 + (q & 127)) * 4 + (row & 3)] =
                    (min(((key >> 16) - (uint32_t)x0) & 255u, (uint32_t)W) << 24) | (((key >> 8) & 255u) << 16) |
                    (key & 255u);
            }
            if (act && w_out) {
                w_out[(size_t)q * n_ent + dst] = w_in[i];
                idx_out[(size_t)q * n_ent + dst] = i;
            }
            if (act && tid == leader) cnt[bin] += __popc(peers);
            __syncwarp();
        }
    }
    if (tid == 0) status[q] = bad;
}

// ---------------------------------------------------------------------------
// pencil stage: CTA = one rotation x 8 pencils, one warp per pencil (ky, kz):
//   F(x) = sum over entries of bin (t, x) of w e^{-2 pi i (ky y / Ny + kz z / Nz)}
//   S(kx) += conj(R^_t(kx)) FFT_x(F)(kx)   over the terms
//   g2[x][p] = IFFT_x(S)(x)
// The warp first tabulates its pencil's phases along y and z (Ny + Nz
// values), so an entry costs two lookups and a complex product.  The lanes
// take a term's entries 32 at a time; entries are sorted by x, so a
// segmented scan over the lanes sums each x bin's entries and the last lane
// of each bin adds the sum into F(x): every lane has work whatever the bin
// sizes, and the additions happen in one fixed order.
// ---------------------------------------------------------------------------
template <bool WEIGHTED>
__global__ void __launch_bounds__(32 * kBoxWarps, 2) box_pencil_kernel(
    const float2* __restrict__ spec, const uint32_t* __restrict__ ent, const int32_t* __restrict__ offs,
    const float* __restrict__ ent_w, const float2* __restrict__ twx_g, const float2* __restrict__ twy_g,
    const float2* __restrict__ twz_g, BoxPlan plx, float2* __restrict__ g2, int K, int n_ent, int ny, int nz, int pp) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nx = plx.n, hz = nz / 2 + 1, np = ny * hz;
    const int wstride = ny + nz + 3 * nx;
    float2* twx = reinterpret_cast<float2*>(smem_raw);  // [nx]
    float2* twy = twx + nx;                             // [ny]
    float2* twz = twy + ny;                             // [nz]
    float2* wbuf = twz + nz;                            // [8][ny + nz + 3 nx]
    float2* otile = wbuf + kBoxWarps * wstride;         // [nx][8]
    uint32_t* ent_s = reinterpret_cast<uint32_t*>(otile + kBoxWarps * nx);  // [n_ent]
    float* w_s = reinterpret_cast<float*>(ent_s + n_ent);                     // WEIGHTED: [n_ent]
    int32_t* tstart = reinterpret_cast<int32_t*>(w_s + (WEIGHTED ? n_ent : 0));  // [K + 1]

    const int q = blockIdx.x;
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    for (int i = tid; i < nx; i += blockDim.x) twx[i] = twx_g[i];
    for (int i = tid; i < ny; i += blockDim.x) twy[i] = twy_g[i];
    for (int i = tid; i < nz; i += blockDim.x) twz[i] = twz_g[i];
    const uint32_t* eq = ent + (size_t)q * n_ent;
    for (int i = tid; i < n_ent; i += blockDim.x) {
        ent_s[i] = eq[i];
        if (WEIGHTED) w_s[i] = ent_w[(size_t)q * n_ent + i];
    }
    // entries of term t: [tstart[t], tstart[t + 1]) (sorted by (t, x))
    const int32_t* oq = offs + (size_t)q * (K * nx + 1);
    for (int t = tid; t <= K; t += blockDim.x) tstart[t] = t < K ? oq[t * nx] : n_ent;
    __syncthreads();

    const int p = blockIdx.y * kBoxWarps + w;
    if (p < np) {
        const int ky = p / hz, kz = p - (p / hz) * hz;
        float2* phy = wbuf + (size_t)w * wstride;  // [ny] e^{-2 pi i ky y / Ny}
        float2* phz = phy + ny;                     // [nz] e^{-2 pi i kz z / Nz}
        float2* a = phz + nz;
        float2* b = a + nx;
        float2* acc = b + nx;
        for (int y = lane; y < ny; y += 32) phy[y] = twy[(ky * y) % ny];
        for (int z = lane; z < nz; z += 32) phz[z] = twz[(kz * z) % nz];
        for (int x = lane; x < nx; x += 32) acc[x] = make_float2(0.f, 0.f);
        for (int t = 0; t < K; ++t) {
            for (int x = lane; x < nx; x += 32) a[x] = make_float2(0.f, 0.f);
            __syncwarp();
            const int j1 = tstart[t + 1];
            for (int base = tstart[t]; base < j1; base += 32) {
                const int j = base + lane;
                const bool act = j < j1;
                const uint32_t e = act ? ent_s[j] : 0u;
                const int xk = act ? (int)((e >> 16) & 255u) : -1;
                float2 v = make_float2(0.f, 0.f);
                if (act) {
                    v = c_mul(phy[(e >> 8) & 255u], phz[e & 255u]);
                    if (WEIGHTED) {
                        const float wj = w_s[j];
                        v.x *= wj;
                        v.y *= wj;
                    }
                }
                // segmented inclusive scan over lanes with equal x (contiguous: sorted)
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const float ux = __shfl_up_sync(0xffffffffu, v.x, o);
                    const float uy = __shfl_up_sync(0xffffffffu, v.y, o);
                    const int uk = __shfl_up_sync(0xffffffffu, xk, o);
                    if (lane >= o && uk == xk) {
                        v.x += ux;
                        v.y += uy;
                    }
                }
                const int nk = __shfl_down_sync(0xffffffffu, xk, 1);
                if (act && (lane == 31 || nk != xk)) {
                    float2 f = a[xk];
                    f.x += v.x;
                    f.y += v.y;
                    a[xk] = f;
                }
                __syncwarp();
            }
            const float2* fx = warp_fft<float2, -1>(a, b, twx, plx, lane);
            const float2* sp = spec + ((size_t)t * pp + p) * nx;
            for (int kx = lane; kx < nx; kx += 32) {
                const float2 f = fx[kx];
                const float2 rv = __ldg(sp + kx);
                float2 s = acc[kx];
                s.x += f.x * rv.x + f.y * rv.y;
                s.y += f.y * rv.x - f.x * rv.y;
                acc[kx] = s;
            }
            __syncwarp();
        }
        for (int x = lane; x < nx; x += 32) a[x] = acc[x];
        const float2* out = warp_fft<float2, +1>(a, b, twx, plx, lane);
        for (int x = lane; x < nx; x += 32) otile[x * kBoxWarps + w] = out[x];
    }
    __syncthreads();
    // the CTA's 8 pencils of every x plane: 64 contiguous bytes per plane
    float2* dst = g2 + (size_t)q * nx * pp + (size_t)blockIdx.y * kBoxWarps;
    for (int i = tid; i < nx * kBoxWarps; i += blockDim.x) {
        const int x = i / kBoxWarps, ww = i - x * kBoxWarps;
        if (blockIdx.y * kBoxWarps + ww < np) dst[(size_t)x * pp + ww] = otile[i];
    }
}

// ---------------------------------------------------------------------------
// plane stage: CTA = one (rotation, x) plane.  Inverse y transform of every
// kz column, then each row's real inverse z transform (the half spectrum
// extended by Hermitian symmetry, a complex inverse transform, the real
// part); every warp keeps the KC smallest (value, offset) of its rows, and
// warp 0 merges them into the plane's pool.
// ---------------------------------------------------------------------------
// QUAD: input = the tensor pencil stage's x-quads [B][nxp / 4][nh][4]
// plh (plh.n = nz / 2 for even nz, else 0): each row's real inverse
// transform as one nz/2-point complex transform of the Hermitian-folded half
// spectrum, Y[k] = A + i w^k B with A = X[k] + conj(X[nz/2 - k]),
// B = X[k] - conj(X[nz/2 - k]), w = e^{2 pi i / nz}: output m holds the real
// values of z = 2m and 2m + 1.
// PW warps; MAXR: the largest radix of the y and z plans (9: none of 11, 13)
template <bool DBG, bool QUAD, int PW, int MAXR>
__global__ void __launch_bounds__(32 * PW, 2) box_plane_kernel(const float2* __restrict__ g2,
                                                                  const float2* __restrict__ twy_g,
                                                                  const float2* __restrict__ twz_g, BoxPlan ply,
                                                                  BoxPlan plz, BoxPlan plh, int nx, int pp,
                                                                  float* __restrict__ cand_v,
                                                                  int32_t* __restrict__ cand_i,
                                                                  float* __restrict__ dbg, int nxp) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ny = ply.n, nz = plz.n, hz = nz / 2 + 1;
    const int lmax = ny > nz ? ny : nz;
    const int ns = plh.n;
    // rows of an odd pitch: a half-warp reading a column hits 16 bank pairs
    const int pitch = hz | 1;
    float2* plane = reinterpret_cast<float2*>(smem_raw);  // [Ny][pitch]
    float2* twy = plane + (size_t)ny * pitch;             // [ny]
    float2* twz = twy + ny;                               // [nz]
    float2* twh = twz + nz;                               // [nz / 2]: e^{-2 pi i m / (nz / 2)}
    float2* wbuf = twh + nz / 2;                          // [8][2][lmax]
    __shared__ float lv_s[PW * KC];
    __shared__ int li_s[PW * KC];

    const int x = blockIdx.x, q = blockIdx.y;
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    for (int i = tid; i < ny; i += blockDim.x) twy[i] = twy_g[i];
    for (int i = tid; i < nz; i += blockDim.x) twz[i] = twz_g[i];
    for (int i = tid; i < ns; i += blockDim.x) twh[i] = twz_g[2 * i];
    {
        // the plane's values, 8 loads in flight per thread before their stores
        const size_t nh = (size_t)ny * hz;
        const float2* src = QUAD ? g2 + (size_t)q * nxp * nh + (size_t)(x >> 2) * nh * 4 + (x & 3)
                                 : g2 + ((size_t)q * nx + x) * pp;
        const int step = QUAD ? 4 : 1;
        const int tot = ny * hz;
        // i / hz as a multiply-high by ceil(2^32 / hz): exact for i < 2^32 / hz
        const unsigned mhz = 0xffffffffu / (unsigned)hz + 1u;
        for (int i0 = tid; i0 < tot; i0 += 8 * blockDim.x) {
            float2 v[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int i = i0 + k * blockDim.x;
                if (i < tot) v[k] = src[(size_t)i * step];
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int i = i0 + k * blockDim.x;
                if (i < tot) {
                    const int yq = (int)__umulhi((unsigned)i, mhz);
                    plane[yq * pitch + (i - yq * hz)] = v[k];
                }
            }
        }
    }
    __syncthreads();
    float2* a = wbuf + (size_t)w * 2 * lmax;
    float2* b = a + lmax;
    // columns kz: inverse transform along ky
    for (int kz = w; kz < hz; kz += PW) {
        __syncwarp();
        for (int k = lane; k < ny; k += 32) a[k] = plane[k * pitch + kz];
        const float2* o = warp_fft<float2, +1, MAXR>(a, b, twy, ply, lane);
        for (int y = lane; y < ny; y += 32) plane[y * pitch + kz] = o[y];
    }
    __syncthreads();
    // rows y: real inverse transform along kz, and the warp's top KC.  Even
    // nz: two rows per warp, 16 lanes each (the short nz/2-point transforms
    // leave most of a warp idle in their larger-radix stages); each half's
    // line sits at offset line * ns of the warp's two buffers.
    WarpTopK tk;
    tk.init();
    const size_t row0 = (size_t)x * ny;
    const int line = lane >> 4, li = lane & 15;
    for (int y0 = 2 * w; y0 < ny && ns > 0; y0 += 2 * PW) {
        __syncwarp();
        const int y = y0 + line < ny ? y0 + line : y0;  // an odd last row: both halves take it
        const float2* row = plane + (size_t)y * pitch;
        float2* al = a + line * ns;
        for (int k = li; k < ns; k += 16) {
            const float2 X = row[k], Xm = row[ns - k];
            const float2 A = make_float2(X.x + Xm.x, X.y - Xm.y);
            const float2 B = make_float2(X.x - Xm.x, X.y + Xm.y);
            const float2 wk = twz[k];  // conj(w^k)
            const float2 cb = make_float2(B.x * wk.x + B.y * wk.y, B.y * wk.x - B.x * wk.y);  // B w^k
            al[k] = make_float2(A.x - cb.y, A.y + cb.x);
        }
        const float2* o = warp_fft<float2, +1, MAXR, 16>(al, b + line * ns, twh, plh, li);
        // the same plan in both halves: both results in a, or both in b
        const float2* res = (o == al ? a : b);
#pragma unroll 1
        for (int hl = 0; hl < 2 && y0 + hl < ny; ++hl) {
            const float2* ol = res + hl * ns;
            const int yy = y0 + hl;
            for (int z0 = 0; z0 < nz; z0 += 32) {
                const int z = z0 + lane;
                const bool ok = z < nz;
                const float2 c = ol[ok ? z >> 1 : 0];
                const float v = ok ? ((z & 1) ? c.y : c.x) : INFINITY;
                const int idx = ok ? (int)((row0 + yy) * nz + z) : 0x7fffffff;
                if (DBG && ok) dbg[(size_t)q * nx * ny * nz + (size_t)idx] = v;
                tk.offer(v, idx, lane);
            }
        }
    }
    for (int y = w; y < ny && ns == 0; y += PW) {
        __syncwarp();
        const float2* row = plane + (size_t)y * pitch;
        for (int k = lane; k < nz; k += 32) {
            if (k < hz) {
                a[k] = row[k];
            } else {
                const float2 c = row[nz - k];
                a[k] = make_float2(c.x, -c.y);
            }
        }
        const float2* o = warp_fft<float2, +1, MAXR>(a, b, twz, plz, lane);
        for (int z0 = 0; z0 < nz; z0 += 32) {
            const int z = z0 + lane;
            const bool ok = z < nz;
            const float v = ok ? o[z].x : INFINITY;
            const int idx = ok ? (int)((row0 + y) * nz + z) : 0x7fffffff;
            if (DBG && ok) dbg[(size_t)q * nx * ny * nz + (size_t)idx] = v;
            tk.offer(v, idx, lane);
        }
    }
    if (lane < KC) {
        lv_s[w * KC + lane] = tk.lv;
        li_s[w * KC + lane] = tk.li;
    }
    // the warps' sorted lists merged pairwise over log2(PW) levels into
    // list 0 (warp w merges list w + step into list w)
    for (int step = 1; step < PW; step <<= 1) {
        __syncthreads();
        if ((w & (2 * step - 1)) == 0 && w + step < PW) {
            float sv = lane < KC ? lv_s[w * KC + lane] : lv_s[(w + step) * KC + 31 - lane];
            int si = lane < KC ? li_s[w * KC + lane] : li_s[(w + step) * KC + 31 - lane];
            warp_merge32(sv, si, lane);
            if (lane < KC) {
                lv_s[w * KC + lane] = sv;
                li_s[w * KC + lane] = si;
            }
        }
    }
    __syncthreads();
    if (w == 0 && lane < KC) {
        cand_v[((size_t)q * nx + x) * KC + lane] = lv_s[lane];
        cand_i[((size_t)q * nx + x) * KC + lane] = li_s[lane];
    }
}

// ---------------------------------------------------------------------------
// finalize: merge the Nx x KC pools, FP64 direct-space rescoring of the KC
// best cells (mod each axis' size), sort by (energy, offset), maxValCorr,
// translation = h unwrap(cell) per axis.  One CTA per rotation.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) box_finalize_kernel(
    const float* __restrict__ cand_v, const int32_t* __restrict__ cand_i, const uint32_t* __restrict__ ent,
    const int32_t* __restrict__ status, const double* __restrict__ rgrid, int n_ent, int nx, int ny, int nz,
    int peak_stride, int k_out, double max_val, double h, int first_rot_id, fftdock_peak* __restrict__ peaks,
    int32_t* __restrict__ n_peaks, float* __restrict__ pool_v, int32_t* __restrict__ pool_i,
    const double* __restrict__ w64, const int32_t* __restrict__ ent_idx) {
    __shared__ float lv_s[8 * KC];
    __shared__ int li_s[8 * KC];
    __shared__ double score_s[KC];
    const int q = blockIdx.x;
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
    const long V = (long)nx * ny * nz;
    const int ncand = nx * KC;
    WarpTopK tk;
    tk.init();
    const float* cv = cand_v + (size_t)q * ncand;
    const int32_t* ci = cand_i + (size_t)q * ncand;
    for (int base = w * 32; base < ncand; base += 256) {
        const int e = base + l;
        tk.offer(e < ncand ? cv[e] : INFINITY, e < ncand ? ci[e] : 0x7fffffff, l);
    }
    if (l < KC) {
        lv_s[w * KC + l] = tk.lv;
        li_s[w * KC + l] = tk.li;
    }
    __syncthreads();
    if (w == 0) {
        merge_lists(lv_s, li_s, 8 * KC, tk, l);
        __syncwarp();
        if (l < KC) {
            lv_s[l] = tk.lv;
            li_s[l] = tk.li;
        }
    }
    __syncthreads();
    if (pool_v != nullptr && tid < KC) {
        pool_v[(size_t)q * KC + tid] = lv_s[tid];
        pool_i[(size_t)q * KC + tid] = li_s[tid];
    }
    const uint32_t* e_q = ent + (size_t)q * n_ent;
    for (int c = w; c < KC; c += 8) {
        const int off = li_s[c];
        double sum = 0.0;
        const bool ok = off >= 0 && off < V;
        if (ok) {
            const int sx = off / (ny * nz), sy = (off / nz) % ny, sz = off % nz;
            for (int j = l; j < n_ent; j += 32) {
                const uint32_t u = e_q[j];
                const int t = (int)(u >> 24);
                const int ax = (int)((u >> 16) & 255u), ay = (int)((u >> 8) & 255u), az = (int)(u & 255u);
                const int gx = ax - sx < 0 ? ax - sx + nx : ax - sx;
                const int gy = ay - sy < 0 ? ay - sy + ny : ay - sy;
                const int gz = az - sz < 0 ? az - sz + nz : az - sz;
                const double rv = rgrid[(size_t)t * V + ((size_t)gx * ny + gy) * nz + gz];
                sum = __dadd_rn(sum, w64 ? __dmul_rn(w64[ent_idx[(size_t)q * n_ent + j]], rv) : rv);
            }
            for (int o = 16; o > 0; o >>= 1) sum = __dadd_rn(sum, __shfl_xor_sync(0xffffffffu, sum, o));
        }
        if (l == 0) score_s[c] = ok ? sum : INFINITY;
    }
    __syncthreads();
    if (tid == 0) {
        double sc[KC];
        int of[KC];
        for (int c = 0; c < KC; ++c) {
            sc[c] = score_s[c];
            of[c] = li_s[c];
        }
        for (int a2 = 1; a2 < KC; ++a2) {
            const double s = sc[a2];
            const int o = of[a2];
            int b2 = a2 - 1;
            while (b2 >= 0 && (sc[b2] > s || (sc[b2] == s && of[b2] > o))) {
                sc[b2 + 1] = sc[b2];
                of[b2 + 1] = of[b2];
                --b2;
            }
            sc[b2 + 1] = s;
            of[b2 + 1] = o;
        }
        int n = 0;
        if (status[q] == 0) {
            const int dims[3] = {nx, ny, nz};
            for (int c = 0; c < KC && n < k_out; ++c) {
                if (!(sc[c] < max_val) || of[c] < 0 || of[c] >= V) continue;
                fftdock_peak pk;
                pk.rot_id = first_rot_id + q;
                pk.cell[0] = of[c] / (ny * nz);
                pk.cell[1] = (of[c] / nz) % ny;
                pk.cell[2] = of[c] % nz;
                for (int d = 0; d < 3; ++d) {
                    int yv = -pk.cell[d];
                    if (yv < -(dims[d] / 2)) yv += dims[d];
                    pk.t[d] = h * (double)yv;
                }
                pk.score = sc[c];
                peaks[(size_t)q * peak_stride + n] = pk;
                ++n;
            }
        }
        n_peaks[q] = n;
    }
}

size_t pencil_smem_bytes(int nx, int ny, int nz, int K, int n_ent, bool weighted) {
    return (size_t)(nx + ny + nz) * sizeof(float2) + (size_t)kBoxWarps * (ny + nz + 3 * nx) * sizeof(float2) +
           (size_t)kBoxWarps * nx * sizeof(float2) + (size_t)n_ent * sizeof(uint32_t) * (weighted ? 2 : 1) +
           ((size_t)K + 1) * sizeof(int32_t);
}
size_t plane_smem_bytes(int ny, int nz) {
    const int hz = nz / 2 + 1, lmax = std::max(ny, nz);
    // up to 16 warps (plans without factors 11 and 13)
    return ((size_t)ny * (hz | 1) + ny + nz + nz / 2 + (size_t)16 * 2 * lmax) * sizeof(float2);
}
size_t prep_smem_bytes(int nx, int K, int n_ent) {
    return ((size_t)K * nx + 1) * sizeof(int32_t) + (size_t)n_ent * sizeof(uint32_t);
}

cudaError_t set_smem(const void* fn, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

cudaError_t box_prep(const BatchArgs& a, cudaStream_t s) {
    const int nb = a.n_rot;
    if (nb <= 0) return cudaSuccess;
    const size_t sm = prep_smem_bytes(a.box.n[0], a.K, a.n_ent);
    cudaError_t e = set_smem((const void*)box_prep_kernel, sm);
    if (e != cudaSuccess) return e;
    box_prep_kernel<<<nb, 256, sm, s>>>(a.rot, a.lig_xyz, a.lig_term, a.n_ent, a.K, a.box, a.ent, a.offs, a.status,
                                        a.lig_w32, a.lig_w32 ? a.ent_w : nullptr, a.ent_idx,
                                        a.use_tc ? a.ent_t : nullptr, a.tpad, a.n_pad, a.x0, a.W);
    return cudaGetLastError();
}

bool big_radix(const BoxPlan& pl) {
    for (int i = 0; i < pl.nf; ++i)
        if (pl.f[i] > 9) return true;
    return false;
}

template <bool DBG, bool QUAD, int PW, int MAXR>
cudaError_t box_plane_launch(dim3 grid, size_t sm, const float2* src, const float2* twy, const float2* twz,
                             const BoxPlan& py, const BoxPlan& pz, const BoxPlan& ph, int nx, const BatchArgs& a,
                             float* dbg, int nxp, cudaStream_t s) {
    cudaError_t e = set_smem((const void*)box_plane_kernel<DBG, QUAD, PW, MAXR>, sm);
    if (e != cudaSuccess) return e;
    box_plane_kernel<DBG, QUAD, PW, MAXR><<<grid, 32 * PW, sm, s>>>(src, twy, twz, py, pz, ph, nx, a.PP, a.cand_v,
                                                                    a.cand_i, dbg, nxp);
    return cudaGetLastError();
}

// plans without factors 11 and 13 run 16 warps per CTA (the smaller
// stages fit 64 registers), others 8
template <bool DBG, bool QUAD>
cudaError_t box_plane(dim3 grid, size_t sm, const float2* src, const float2* twy, const float2* twz, const BoxPlan& py,
                      const BoxPlan& pz, int nx, const BatchArgs& a, float* dbg, int nxp, cudaStream_t s) {
    // even nz: rows through the half-length transform
    BoxPlan ph{};
    if (pz.n % 2 == 0 && !factor_plan(pz.n / 2, ph)) ph = BoxPlan{};
    if (big_radix(py) || big_radix(pz))
        return box_plane_launch<DBG, QUAD, 8, 13>(grid, sm, src, twy, twz, py, pz, ph, nx, a, dbg, nxp, s);
    return box_plane_launch<DBG, QUAD, 16, 9>(grid, sm, src, twy, twz, py, pz, ph, nx, a, dbg, nxp, s);
}

cudaError_t box_middle(const BatchArgs& a, cudaStream_t s) {
    const int nb = a.n_rot;
    if (nb <= 0) return cudaSuccess;
    const int nx = a.box.n[0], ny = a.box.n[1], nz = a.box.n[2];
    BoxPlan px, py, pz;
    if (!factor_plan(nx, px) || !factor_plan(ny, py) || !factor_plan(nz, pz)) return cudaErrorInvalidValue;
    const float2* twx = a.box_tw32;
    const float2* twy = twx + nx;
    const float2* twz = twy + ny;
    cudaError_t e;
    if (a.ev && (e = cudaEventRecord(a.ev[0], s)) != cudaSuccess) return e;
    const bool weighted = a.lig_w32 != nullptr;
    const size_t sm2 = pencil_smem_bytes(nx, ny, nz, a.K, a.n_ent, weighted);
    const int np = ny * (nz / 2 + 1);
    const size_t sm3 = plane_smem_bytes(ny, nz);
    dim3 grid3(nx, nb);
    if (a.use_tc) {
        // tensor form: the x stage as split-FP16 tcgen05 GEMMs over 128
        // rotations per CTA, then the plane stage from its x-quads
        const int nxp = (nx + 3) / 4 * 4;
        const size_t smt = tc_smem_bytes_box(nx, ny, nz, a.W / 8, a.n_tc_terms);
        dim3 gridt(np, (nb + TC_ROT - 1) / TC_ROT);
        const int tg = a.tc_group > 0 ? a.tc_group : FFTDOCK_TC_TERMS_PER_SUM_DEFAULT;
        const TcBox bx{nx, ny, nz, nz / 2 + 1, np, nxp, twy, twz};
        if (tc_tiles(nx) == 1) {
            if ((e = set_smem((const void*)pencil_tc_kernel<0, 1>, smt)) != cudaSuccess) return e;
            pencil_tc_kernel<0, 1><<<gridt, TC_THREADS, smt, s>>>(a.circ, a.cscale, a.ent_t, a.tinfo, a.n_tc_terms,
                                                                 nullptr, a.g2t, a.n_pad, nb, a.x0, a.W, tg,
                                                                 a.tc_slots, a.tc_n_slots, bx, a.err);
        } else {
            if ((e = set_smem((const void*)pencil_tc_kernel<0, 2>, smt)) != cudaSuccess) return e;
            pencil_tc_kernel<0, 2><<<gridt, TC_THREADS, smt, s>>>(a.circ, a.cscale, a.ent_t, a.tinfo, a.n_tc_terms,
                                                                 nullptr, a.g2t, a.n_pad, nb, a.x0, a.W, tg,
                                                                 a.tc_slots, a.tc_n_slots, bx, a.err);
        }
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if (a.ev && (e = cudaEventRecord(a.ev[1], s)) != cudaSuccess) return e;
        e = a.dbg_corr ? box_plane<true, true>(grid3, sm3, a.g2t, twy, twz, py, pz, nx, a, a.dbg_corr, nxp, s)
                       : box_plane<false, true>(grid3, sm3, a.g2t, twy, twz, py, pz, nx, a, nullptr, nxp, s);
        if (e != cudaSuccess) return e;
        if (a.ev && (e = cudaEventRecord(a.ev[2], s)) != cudaSuccess) return e;
        return cudaSuccess;
    }
    dim3 grid2(nb, (np + kBoxWarps - 1) / kBoxWarps);
    if (weighted) {
        if ((e = set_smem((const void*)box_pencil_kernel<true>, sm2)) != cudaSuccess) return e;
        box_pencil_kernel<true><<<grid2, 32 * kBoxWarps, sm2, s>>>(static_cast<const float2*>(a.spec), a.ent, a.offs,
                                                                  a.ent_w, twx, twy, twz, px, a.g2, a.K, a.n_ent, ny,
                                                                  nz, a.PP);
    } else {
        if ((e = set_smem((const void*)box_pencil_kernel<false>, sm2)) != cudaSuccess) return e;
        box_pencil_kernel<false><<<grid2, 32 * kBoxWarps, sm2, s>>>(static_cast<const float2*>(a.spec), a.ent,
                                                                   a.offs, nullptr, twx, twy, twz, px, a.g2, a.K,
                                                                   a.n_ent, ny, nz, a.PP);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (a.ev && (e = cudaEventRecord(a.ev[1], s)) != cudaSuccess) return e;
    e = a.dbg_corr ? box_plane<true, false>(grid3, sm3, a.g2, twy, twz, py, pz, nx, a, a.dbg_corr, nx, s)
                   : box_plane<false, false>(grid3, sm3, a.g2, twy, twz, py, pz, nx, a, nullptr, nx, s);
    if (e != cudaSuccess) return e;
    if (a.ev && (e = cudaEventRecord(a.ev[2], s)) != cudaSuccess) return e;
    return cudaSuccess;
}

cudaError_t box_finish(const BatchArgs& a, cudaStream_t s) {
    const int nb = a.n_rot;
    if (nb <= 0) return cudaSuccess;
    box_finalize_kernel<<<nb, 256, 0, s>>>(a.cand_v, a.cand_i, a.ent, a.status, a.rgrid, a.n_ent, a.box.n[0],
                                           a.box.n[1], a.box.n[2], a.peak_stride, a.k_out, a.max_val, a.h,
                                           a.first_rot_id, a.peaks, a.n_peaks, a.pool_v, a.pool_i, a.lig_w64,
                                           a.lig_w64 ? a.ent_idx : nullptr);
    return cudaGetLastError();
}

cudaError_t box_scan_batch(const BatchArgs& a, cudaStream_t s) {
    cudaError_t e = box_prep(a, s);
    if (e != cudaSuccess) return e;
    BatchArgs m = a;
    m.ev = nullptr;
    if ((e = box_middle(m, s)) != cudaSuccess) return e;
    return box_finish(a, s);
}

size_t box_pencil_smem_unknown(int, int) { return 0; }

cudaError_t box_load_kernels(int) {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, (const void*)box_prep_kernel);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void*)box_pencil_kernel<false>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void*)box_plane_kernel<false, false, 16, 9>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void*)box_finalize_kernel);
    return e;
}

}  // namespace

bool box_plan(int n, BoxPlan* pl) { return factor_plan(n, *pl); }

size_t box_pencil_smem(int nx, int ny, int nz, int K, int n_ent, bool weighted) {
    return std::max(pencil_smem_bytes(nx, ny, nz, K, n_ent, weighted),
                    std::max(plane_smem_bytes(ny, nz), prep_smem_bytes(nx, K, n_ent)));
}

// Forward transform of one real FP64 term grid [Nx][Ny][Nz] into spec_t
// ([Nx][PP] float2, scaled 1 / V): complex z transforms, the half spectrum
// kz < Hz, then y and x transforms, each a batch of line FFTs.
cudaError_t box_receptor_fft(const double* rgrid_t, double2* cbuf, double2* hbuf, const double2* tw64,
                             const int dims[3], void* spec_t, int PP, float2* circ_t, cudaStream_t s) {
    const int nx = dims[0], ny = dims[1], nz = dims[2], hz = nz / 2 + 1;
    BoxPlan px, py, pz;
    if (!factor_plan(nx, px) || !factor_plan(ny, py) || !factor_plan(nz, pz)) return cudaErrorInvalidValue;
    const double2* twx = tw64;
    const double2* twy = twx + nx;
    const double2* twz = twy + ny;
    const size_t V = (size_t)nx * ny * nz;
    complexify_kernel<<<(unsigned)((V + 255) / 256), 256, 0, s>>>(rgrid_t, cbuf, V);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    auto lines = [&](double2* data, const double2* tw, const BoxPlan& pl, long n_lines, long es, long ic, long is,
                     long os) -> cudaError_t {
        const size_t sm = ((size_t)pl.n + (size_t)kBoxWarps * 2 * pl.n) * sizeof(double2);
        cudaError_t e2 = set_smem((const void*)box_line_fft64_kernel, sm);
        if (e2 != cudaSuccess) return e2;
        const long blocks = (n_lines + kBoxWarps - 1) / kBoxWarps;
        box_line_fft64_kernel<<<(unsigned)blocks, 32 * kBoxWarps, sm, s>>>(data, tw, pl, n_lines, es, ic, is, os);
        return cudaGetLastError();
    };
    // z: lines (x, y), contiguous
    if ((e = lines(cbuf, twz, pz, (long)nx * ny, 1, 1, 0, nz)) != cudaSuccess) return e;
    const size_t nh = (size_t)nx * ny * hz;
    box_half_extract_kernel<<<(unsigned)((nh + 255) / 256), 256, 0, s>>>(cbuf, hbuf, nx, ny, nz, hz);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // y: lines (x, kz) of [Nx][Ny][Hz]
    if ((e = lines(hbuf, twy, py, (long)nx * hz, hz, hz, 1, (long)ny * hz)) != cudaSuccess) return e;
    if (circ_t) {
        // transformed along z and y only: the tensor stage's circulant samples
        const size_t tot = (size_t)nx * ny * hz;
        pack_circ_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(hbuf, circ_t, nx, ny * hz,
                                                                     1.0 / ((double)ny * nz));
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    // x: lines p = (ky, kz)
    if ((e = lines(hbuf, twx, px, (long)ny * hz, (long)ny * hz, (long)ny * hz, 1, 0)) != cudaSuccess) return e;
    const size_t tot = (size_t)nx * PP;
    box_pack_spectrum_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(hbuf, static_cast<float2*>(spec_t), nx,
                                                                           ny * hz, PP, 1.0 / (double)V);
    return cudaGetLastError();
}

cudaError_t box_circ_scales(const float2* circ, int K, int nh, int nx, int8_t* cscale, cudaStream_t s) {
    circ_scale_box_kernel<<<(nh + 127) / 128, 128, 0, s>>>(circ, K, nh, nx, cscale);
    return cudaGetLastError();
}

size_t box_tc_smem(const int dims[3], int n_chunks, int n_terms) {
    return tc_smem_bytes_box(dims[0], dims[1], dims[2], n_chunks, n_terms);
}

size_t cubic_tc_smem(int n, int n_chunks, int n_terms) { return tc_smem_bytes(n, n_chunks, n_terms); }

const SizeOps* box_ops() {
    static const SizeOps o{0, nullptr, nullptr, false, &box_scan_batch, &box_pencil_smem_unknown, &box_prep,
                           &box_middle, &box_finish, &box_load_kernels};
    return &o;
}

}  // namespace fftdock
