// Device kernels of the correlation scan.  Templated on the grid edge N;
// instantiated per N by kernels_nXX.cu through dispatch_impl.cuh.
//
// Data layout in HBM (N = grid edge, H = N/2+1, PP = N*H rounded up to 32,
// pencil index p = ky*H + kz):
//   spec  [K][N][PP]   float2  receptor spectra R^_t(kx, p) / N^3
//   rgrid [K][N^3]     double  real-space receptor terms (FP64 rescoring)
//   ent   [B][n_ent]   uint32  per-rotation ligand entries t<<24|x<<16|y<<8|z,
//                              sorted by (t, x), atom order inside a bin
//   offs  [B][K*N+1]   int32   start of bin (t, x) at offs[t*N + x]
//   g2    [B][N][PP]   float2  sum_t conj(R^_t) L^_t inverse-transformed
//                              along x: one complex (ky, kz) plane per x
//   cand  [B][N][KC]           per-plane FP32 candidate pools
#pragma once

#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include "fft_core.cuh"
#include "fftdock.h"
#include "internal.h"

namespace fftdock {

constexpr int KC = 16;  // FP32 candidates kept per plane / per rotation

// Warps per line transform along x/y (G) and along the half rows (GR);
// G*G | N and GR*GR | N/2, GR | G.
template <int N> struct SizeTraits;
template <> struct SizeTraits<16> { static constexpr int G = 4, GR = 2; };
template <> struct SizeTraits<24> { static constexpr int G = 2, GR = 2; };
template <> struct SizeTraits<32> { static constexpr int G = 4, GR = 4; };
template <> struct SizeTraits<48> { static constexpr int G = 4, GR = 2; };
template <> struct SizeTraits<64> { static constexpr int G = 8, GR = 4; };
template <> struct SizeTraits<80> { static constexpr int G = 4, GR = 2; };
template <> struct SizeTraits<96> { static constexpr int G = 4, GR = 4; };
template <> struct SizeTraits<112> { static constexpr int G = 4, GR = 2; };
template <> struct SizeTraits<128> { static constexpr int G = 8, GR = 8; };
template <> struct SizeTraits<144> { static constexpr int G = 12, GR = 6; };

// Pencil kernel occupancy: exchange buffers (2: one barrier per term; 1: two
// barriers per term but N*32 complex less shared memory) and the CTAs per SM
// its launch bounds ask for (which caps the registers).  Chosen per edge from
// timed scans on GB300 (shape + 18 terms; pencil-kernel time against the
// two-buffer, unbounded form): 64 -22 %, 80 -11 %, 96 -12 %, 128 -6 %,
// 144 -25 %; 112 gained nothing.
template <int N> struct PencilTraits { static constexpr int BUFS = 2, MINB = 1; };
template <> struct PencilTraits<64> { static constexpr int BUFS = 1, MINB = 4; };
template <> struct PencilTraits<80> { static constexpr int BUFS = 1, MINB = 4; };
template <> struct PencilTraits<96> { static constexpr int BUFS = 1, MINB = 4; };
template <> struct PencilTraits<128> { static constexpr int BUFS = 1, MINB = 3; };
template <> struct PencilTraits<144> { static constexpr int BUFS = 2, MINB = 2; };


// toLogical: int((x - zero_h) / h) - 1, truncation toward zero, no FMA.
// Returns the truncated quotient; the cell is q - 1.
__device__ __forceinline__ int logical_q(double x, const Geo& g, int d) {
    return __double2int_rz(__ddiv_rn(__dsub_rn(x, g.zero_h[d]), g.h));
}
__device__ __forceinline__ double cell_centre(int i, const Geo& g, int d) {
    return __dadd_rn(g.center0[d], __dmul_rn(g.h, (double)i));
}

// ---------------------------------------------------------------------------
// warp top-k (KC smallest by (value, index); lanes < KC hold the sorted list)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool better(float a, int ia, float b, int ib) {
    return a < b || (a == b && ia < ib);
}

// Compare-exchange with lane ^ j under better(): this lane keeps the better
// of the two pairs when keep_min, else the other one.
__device__ __forceinline__ void warp_cmp_swap(float& v, int& i, int j, bool keep_min) {
    const float pv = __shfl_xor_sync(0xffffffffu, v, j);
    const int pi = __shfl_xor_sync(0xffffffffu, i, j);
    if (better(pv, pi, v, i) == keep_min) {
        v = pv;
        i = pi;
    }
}

// Bitonic sort of one (value, index) pair per lane, ascending by better()
// across the warp (15 compare-exchange steps).
__device__ __forceinline__ void warp_sort32(float& v, int& i, int lane) {
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) warp_cmp_swap(v, i, j, ((lane & k) == 0) == ((lane & j) == 0));
}

// Lanes 0..15 ascending and lanes 16..31 descending (a bitonic sequence) ->
// all 32 ascending: lanes < 16 then hold the 16 best of both halves.
__device__ __forceinline__ void warp_merge32(float& v, int& i, int lane) {
#pragma unroll
    for (int j = 16; j > 0; j >>= 1) warp_cmp_swap(v, i, j, (lane & j) == 0);
}

struct WarpTopK {
    float lv;
    int li;
    float tv;  // current KC-th value (threshold)
    int ti;
    __device__ __forceinline__ void init() { lv = INFINITY; li = 0x7fffffff; tv = INFINITY; ti = 0x7fffffff; }
    // offer one candidate per lane (all lanes of the warp must call)
    __device__ __forceinline__ void offer(float v, int idx, int lane) {
        // v <= tv is necessary for (v, idx) < (tv, ti); the exact test runs
        // only on the rare candidates
        if (__ballot_sync(0xffffffffu, v <= tv) == 0u) return;
        unsigned mask = __ballot_sync(0xffffffffu, better(v, idx, tv, ti));
        if (__popc(mask) > 6) {
            // many at once: sort the qualifying offers and merge them with
            // the list (lanes < KC ascending, the best KC offers descending
            // above them: one bitonic sequence) -- the same KC best by
            // (value, index) as one insertion each
            static_assert(KC == 16, "the batch merge takes lists of 16");
            float sv = (mask >> lane) & 1u ? v : INFINITY;
            int si = (mask >> lane) & 1u ? idx : 0x7fffffff;
            warp_sort32(sv, si, lane);
            const float rv = __shfl_sync(0xffffffffu, sv, 31 - lane);
            const int ri = __shfl_sync(0xffffffffu, si, 31 - lane);
            float mv = lane < KC ? lv : rv;
            int mi = lane < KC ? li : ri;
            warp_merge32(mv, mi, lane);
            lv = mv;
            li = mi;
            tv = __shfl_sync(0xffffffffu, lv, KC - 1);
            ti = __shfl_sync(0xffffffffu, li, KC - 1);
            return;
        }
        while (mask) {
            const int src = __ffs(mask) - 1;
            const float cv = __shfl_sync(0xffffffffu, v, src);
            const int ci = __shfl_sync(0xffffffffu, idx, src);
            const unsigned below = __ballot_sync(0xffffffffu, lane < KC && better(lv, li, cv, ci));
            const int pos = __popc(below);
            const float upv = __shfl_up_sync(0xffffffffu, lv, 1);
            const int upi = __shfl_up_sync(0xffffffffu, li, 1);
            if (pos < KC) {
                if (lane == pos) { lv = cv; li = ci; }
                else if (lane > pos && lane < KC) { lv = upv; li = upi; }
            }
            tv = __shfl_sync(0xffffffffu, lv, KC - 1);
            ti = __shfl_sync(0xffffffffu, li, KC - 1);
            mask &= ~(1u << src);
            mask &= __ballot_sync(0xffffffffu, better(v, idx, tv, ti));
        }
    }
};

// Merge per-warp lists staged in shared memory (nw lists of KC) into warp 0's
// list; the caller syncs before and reads lanes < KC of warp 0 after.
__device__ __forceinline__ void merge_lists(const float* sv, const int* si, int n, WarpTopK& tk, int lane) {
    tk.init();
    for (int base = 0; base < n; base += 32) {
        const int e = base + lane;
        const float v = e < n ? sv[e] : INFINITY;
        const int i = e < n ? si[e] : 0x7fffffff;
        tk.offer(v, i, lane);
    }
}

// ---------------------------------------------------------------------------
// K1: rotate + bin + stable sort of the ligand entries of one rotation
// (MolForceRadial::projectLigand, docking_molforce.hpp:351-368, with
// Rotation::operator(), transformation.hpp:206-222).  One CTA per rotation.
// ---------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(256) ligand_prep_kernel(
    const double* __restrict__ rot, const double* __restrict__ lig_xyz, const int32_t* __restrict__ lig_term,
    int n_ent, int K, Geo geo, uint32_t* __restrict__ ent_out, int32_t* __restrict__ offs_out,
    int32_t* __restrict__ status, const float* __restrict__ w_in, float* __restrict__ w_out,
    int32_t* __restrict__ idx_out, uint32_t* __restrict__ ent_t, const int32_t* __restrict__ tpad, int n_pad,
    int x0, int W) {
    extern __shared__ unsigned char smem_raw[];
    int32_t* cnt = reinterpret_cast<int32_t*>(smem_raw);          // [K*N + 1]
    uint32_t* keys = reinterpret_cast<uint32_t*>(cnt + K * N + 1);  // [n_ent]
    __shared__ int bad;
    __shared__ int wsum[8];
    const int q = blockIdx.x;
    const int tid = threadIdx.x;
    const int nbins = K * N;
    for (int i = tid; i <= nbins; i += blockDim.x) cnt[i] = 0;
    if (tid == 0) bad = 0;
    __syncthreads();
    const double* m = rot + 9 * (size_t)q;
    const double m00 = m[0], m01 = m[1], m02 = m[2], m10 = m[3], m11 = m[4], m12 = m[5], m20 = m[6], m21 = m[7],
                 m22 = m[8];
    for (int i = tid; i < n_ent; i += blockDim.x) {
        const double x0 = lig_xyz[3 * i], x1 = lig_xyz[3 * i + 1], x2 = lig_xyz[3 * i + 2];
        // y_i = ((m_i0 x0) + m_i1 x1) + m_i2 x2, each product rounded (no FMA)
        const double p0 = __dadd_rn(__dadd_rn(__dmul_rn(m00, x0), __dmul_rn(m01, x1)), __dmul_rn(m02, x2));
        const double p1 = __dadd_rn(__dadd_rn(__dmul_rn(m10, x0), __dmul_rn(m11, x1)), __dmul_rn(m12, x2));
        const double p2 = __dadd_rn(__dadd_rn(__dmul_rn(m20, x0), __dmul_rn(m21, x1)), __dmul_rn(m22, x2));
        int c0 = logical_q(p0, geo, 0), c1 = logical_q(p1, geo, 1), c2 = logical_q(p2, geo, 2);
        const bool ok = c0 >= 1 && c0 <= N && c1 >= 1 && c1 <= N && c2 >= 1 && c2 <= N;
        if (!ok) atomicOr(&bad, 1);
        c0 = min(max(c0 - 1, 0), N - 1);
        c1 = min(max(c1 - 1, 0), N - 1);
        c2 = min(max(c2 - 1, 0), N - 1);
        const int t = lig_term[i];
        keys[i] = ((uint32_t)t << 24) | ((uint32_t)c0 << 16) | ((uint32_t)c1 << 8) | (uint32_t)c2;
        atomicAdd(&cnt[t * N + c0], 1);
    }
    __syncthreads();
    // exclusive scan of cnt[0..nbins) -> starts; cnt[nbins] = n_ent
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
    // stable scatter by one warp: ranks within equal keys follow atom order
    if (tid < 32) {
        uint32_t* ent = ent_out + (size_t)q * n_ent;
        for (int base = 0; base < n_ent; base += 32) {
            const int i = base + tid;
            const bool act = i < n_ent;
            const uint32_t key = act ? keys[i] : 0xffffffffu;
            const int bin = act ? (int)((key >> 24) * N + ((key >> 16) & 255u)) : -1;
            const unsigned peers = __match_any_sync(0xffffffffu, bin);
            const int rank = __popc(peers & ((1u << tid) - 1u));
            const int leader = __ffs(peers) - 1;
            int dst = 0;
            if (act) dst = cnt[bin] + rank;
            __syncwarp();
            if (act) ent[dst] = key;
            // transposed copy for the tensor pencil stage,
            // [q / 128][row / 4][q % 128][row % 4], with each term's rows
            // padded to a multiple of 8; the term is implied by the row and
            // x is stored relative to the window start x0 (mod 256: cells
            // outside the window stay outside it); entry = x' << 24 | y << 16
            // | z, so that one multiply by kz << 16 | ky gives the phase
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
// K2: pencil kernel.  CTA = one rotation x 32 consecutive pencils (ky, kz),
// G warps.  For every term t:
//   F(x) = sum over entries of bin (t, x) of w^(ky*y + kz*z)   (the y and z
//          stages of the forward transform, as direct sums over atoms)
//   L^_t(kx) = FFT_x(F); S(kx) += conj(R^_t(kx)) L^_t(kx)
// then S is inverse-transformed along x and written as one column of g2.
// (FFTCorrelator::correlate, docking_fft.hpp:622-633, summed over terms as
// MolForceComp::collectTotal does in real space, docking_molforce.hpp:172-184.)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 spec_load(const float2* p) { return __ldg(p); }
__device__ __forceinline__ float2 spec_load(const __nv_bfloat162* p) { return __bfloat1622float2(*p); }

template <int N, typename SpecT, bool WEIGHTED = false>
__global__ void __launch_bounds__(32 * SizeTraits<N>::G, PencilTraits<N>::MINB) pencil_kernel(
    const SpecT* __restrict__ spec, const uint32_t* __restrict__ ent, const int32_t* __restrict__ offs,
    const float2* __restrict__ tw, float2* __restrict__ g2, int K, int n_ent, const float* __restrict__ ent_w) {
    using P = LinePlan<N, SizeTraits<N>::G>;
    constexpr int G = P::G, R1 = P::R1, H = N / 2 + 1;
    constexpr int PP = pencil_pitch(N);
    constexpr int BUFS = PencilTraits<N>::BUFS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* xbuf = reinterpret_cast<float2*>(smem_raw);  // [BUFS][N][32]
    float2* tws = xbuf + BUFS * N * 32;                  // [N]
    // the phase table once per half-warp lane ([phase][16]): a warp's lanes
    // are consecutive pencils, whose phases for one entry step by its z, so
    // a single table would put lanes on the same banks whenever z is even
    float2* twr = tws + N;                                  // [N][16]
    // entries ([n_ent]; weighted: [n_ent] pairs of entry and weight bits, one
    // 8-byte broadcast load per entry)
    uint32_t* ent_s = reinterpret_cast<uint32_t*>(twr + N * 16);
    int32_t* offs_s = reinterpret_cast<int32_t*>(ent_s + (WEIGHTED ? 2 : 1) * n_ent);  // [K*N+1]

    const int q = blockIdx.x;
    const int tile = blockIdx.y;
    const int tid = threadIdx.x;
    const int w = tid >> 5, l = tid & 31;
    const int p = tile * 32 + l;
    const unsigned ky = (unsigned)(p / H), kz = (unsigned)(p - (p / H) * H);
    // entries staged as y << 16 | z (x and the term are the bin's): bits 16 and
    // up of u * (kz << 16 | ky) (mod 2^32) hold ky y + kz z (< 2^16 for N <=
    // 144; the z ky term stays below bit 16), one multiply per phase
    const uint32_t kyz = (kz << 16) | ky;

    for (int i = tid; i < N; i += blockDim.x) tws[i] = tw[i];
    for (int i = tid; i < N * 16; i += blockDim.x) twr[i] = tw[i >> 4];
    const int32_t* offs_g = offs + (size_t)q * (K * N + 1);
    for (int i = tid; i <= K * N; i += blockDim.x) offs_s[i] = offs_g[i];
    const uint32_t* ent_g = ent + (size_t)q * n_ent;
    const float* w_g = WEIGHTED ? ent_w + (size_t)q * n_ent : nullptr;
    for (int i = tid; i < n_ent; i += blockDim.x) {
        const uint32_t u = ent_g[i];
        const uint32_t yz = (((u >> 8) & 255u) << 16) | (u & 255u);
        if constexpr (WEIGHTED) {
            ent_s[2 * i] = yz;
            ent_s[2 * i + 1] = __float_as_uint(w_g[i]);
        } else {
            ent_s[i] = yz;
        }
    }
    __syncthreads();

    float2 S[R1];
#pragma unroll
    for (int i = 0; i < R1; ++i) S[i] = make_float2(0.f, 0.f);

    for (int t = 0; t < K; ++t) {
        float2 v[R1];
#pragma unroll
        for (int r = 0; r < R1; ++r) {
            const int x = w + G * r;
            const int b = offs_s[t * N + x], e = offs_s[t * N + x + 1];
            float2 acc = make_float2(0.f, 0.f);
            for (int j = b; j < e; ++j) {
                uint32_t ej;
                float wj = 1.f;
                if constexpr (WEIGHTED) {
                    const uint2 ew = reinterpret_cast<const uint2*>(ent_s)[j];
                    ej = ew.x;
                    wj = __uint_as_float(ew.y);
                } else {
                    ej = ent_s[j];
                }
                const uint32_t yz = (ej * kyz) >> 16;
                const unsigned ph = (N & (N - 1)) == 0 ? (yz & (unsigned)(N - 1)) : yz % (unsigned)N;
                const float2 z = twr[ph * 16 + (l & 15)];
                if constexpr (WEIGHTED) {
                    acc.x = fmaf(wj, z.x, acc.x);
                    acc.y = fmaf(wj, z.y, acc.y);
                } else {
                    acc.x += z.x;
                    acc.y += z.y;
                }
            }
            v[r] = acc;
        }
        dft<R1, -1>(v);
        float2* buf = xbuf + (BUFS == 2 ? (t & 1) * N * 32 : 0);
#pragma unroll
        for (int r = 0; r < R1; ++r) buf[(w * R1 + r) * 32 + l] = v[r];
        __syncthreads();
        float2 F[R1];
        line_pass2<P, -1, 1, 32>(buf, w, l, tws, F);
        if constexpr (BUFS == 1) __syncthreads();  // buf is rewritten by the next term
        const SpecT* sp = spec + (size_t)t * N * PP + p;
#pragma unroll
        for (int i = 0; i < P::NB; ++i)
#pragma unroll
            for (int r = 0; r < G; ++r) {
                const int kx = w + G * i + R1 * r;
                const float2 rv = spec_load(sp + (size_t)kx * PP);
                const float2 f = F[i * G + r];
                S[i * G + r].x += f.x * rv.x + f.y * rv.y;
                S[i * G + r].y += f.y * rv.x - f.x * rv.y;
            }
    }
    float2 v[R1];
    pass2_to_pass1_order<P>(S, v);
    dft<R1, +1>(v);
    float2* buf = xbuf + (BUFS == 2 ? (K & 1) * N * 32 : 0);
#pragma unroll
    for (int r = 0; r < R1; ++r) buf[(w * R1 + r) * 32 + l] = v[r];
    __syncthreads();
    float2 out[R1];
    line_pass2<P, +1, 1, 32>(buf, w, l, tws, out);
    float2* dst = g2 + (size_t)q * N * PP + p;
#pragma unroll
    for (int i = 0; i < P::NB; ++i)
#pragma unroll
        for (int r = 0; r < G; ++r) {
            const int x = w + G * i + R1 * r;
            dst[(size_t)x * PP] = out[i * G + r];
        }
}

// ---------------------------------------------------------------------------
// K3: plane kernel.  CTA = one (rotation, x) plane.  Inverse transform along
// ky (columns kz; the real DC and Nyquist columns share one complex column),
// then the half-spectrum rows along kz are turned into N reals through one
// N/2-point complex transform each; the plane's KC smallest (value, offset)
// cells are then selected exactly: the threads' own minima give an upper
// bound on the KC-th value (bitonic warp sorts and a merge) and only cells at
// or below it are sorted and merged into the plane's top KC.
// (FFTW c2r of FFTCorrelator::correlate + CorrelationProcessor::
// selectIntoQueue, docking_fft.hpp:452-468.)
// Input layouts: QUAD = false, the FFT pencil stage's [B][N][PP] (each plane
// contiguous); QUAD = true, the tensor pencil stage's x-quads
// [B][N/4][N*H][4] (four consecutive planes interleaved per pencil), read by
// clusters of 4 CTAs (planes 4c..4c+3) that each load a quarter of the
// pencils as whole 32-byte groups and store every plane's value into that
// plane's CTA through distributed shared memory.
// ---------------------------------------------------------------------------
template <int N, bool DBG, bool QUAD>
__global__ void __launch_bounds__(32 * SizeTraits<N>::G) plane_kernel(
    const float2* __restrict__ g2, const float2* __restrict__ tw, float* __restrict__ cand_v,
    int32_t* __restrict__ cand_i, float* __restrict__ dbg) {
    constexpr int PP = pencil_pitch(N);
    using PC = LinePlan<N, SizeTraits<N>::G>;
    using PR = LinePlan<N / 2, SizeTraits<N>::GR>;
    constexpr int G = PC::G, R1 = PC::R1;
    constexpr int GR = PR::G, R1R = PR::R1;
    constexpr int H = N / 2 + 1, NS = N / 2;
    constexpr int CC = (NS + 31) / 32;
    constexpr int NG = G / GR;
    constexpr int ROWS = 32 * NG;
    constexpr int ROUNDS = (N + ROWS - 1) / ROWS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* plane = reinterpret_cast<float2*>(smem_raw);  // [N][H]
    float2* tws = plane + N * H;                          // [N]
    float* lv_s = reinterpret_cast<float*>(tws + N);      // [G*KC]
    int* li_s = reinterpret_cast<int*>(lv_s + G * KC);    // [G*KC]
    constexpr int PCAND = 256;                            // candidate list capacity
    __shared__ float cand_sv[PCAND];
    __shared__ int cand_si[PCAND];
    __shared__ int n_cand;

    const int x = blockIdx.x;
    const int q = blockIdx.y;
    const int tid = threadIdx.x;
    const int w = tid >> 5, l = tid & 31;
    if constexpr (QUAD) asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
    for (int i = tid; i < N; i += blockDim.x) tws[i] = tw[i];
    // element (ky, kz) of plane x at src[ky * H + kz]: global memory (FFT
    // form) or this CTA's staged copy (x-quads)
    const float2* src = QUAD ? plane : g2 + ((size_t)q * N + x) * PP;
    if constexpr (QUAD) {
        constexpr int NH = N * H;
        static_assert(N % 4 == 0 && NH % 4 == 0, "x-quads need N % 4 == 0");
        uint32_t rank;
        asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
        const int xb = x - (int)rank;  // the cluster's first plane
        // this CTA's quarter of the pencils: NH / 2 16-byte halves (planes
        // xb, xb + 1 | xb + 2, xb + 3), one per thread and step, coalesced
        const float4* gs = reinterpret_cast<const float4*>(g2 + (size_t)q * NH * N + (size_t)(xb >> 2) * NH * 4) +
                           (size_t)rank * (NH / 2);
        const uint32_t loc = static_cast<uint32_t>(__cvta_generic_to_shared(plane)) + rank * (NH / 4) * 8u;
        uint32_t rb[4];
#pragma unroll
        for (int j = 0; j < 4; ++j)
            asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(rb[j]) : "r"(loc), "r"(j));
        asm volatile("barrier.cluster.wait.aligned;" ::: "memory");  // every CTA of the cluster runs
        // loads in batches ahead of their stores (a store's memory clobber
        // would otherwise hold each load until the previous store)
        constexpr int PER = (NH / 2 + 32 * G - 1) / (32 * G), BATCH = 9;
#pragma unroll
        for (int b0 = 0; b0 < PER; b0 += BATCH) {
            float4 a[BATCH];
#pragma unroll
            for (int k = 0; k < BATCH; ++k) {
                const int e = tid + (b0 + k) * 32 * G;
                if (b0 + k < PER && e < NH / 2) a[k] = gs[e];
            }
#pragma unroll
            for (int k = 0; k < BATCH; ++k) {
                const int e = tid + (b0 + k) * 32 * G;
                if (b0 + k < PER && e < NH / 2) {
                    const uint32_t off = (uint32_t)(e >> 1) * 8u;
                    const uint32_t d0 = (e & 1) ? rb[2] : rb[0], d1 = (e & 1) ? rb[3] : rb[1];
                    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(d0 + off), "f"(a[k].x), "f"(a[k].y)
                                 : "memory");
                    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(d1 + off), "f"(a[k].z), "f"(a[k].w)
                                 : "memory");
                }
            }
        }
        asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
    __syncthreads();

    // Warp-local passes at N = 128 (8 lanes share a column or a row, so
    // their exchanges need __syncwarp only).  A group's pass-1 outputs are
    // stored swizzled within the line: position 16a + b (columns) or 8a + b
    // (rows) at slot 16a + ((a + b) & 15) or 8a + ((a + b) & 7); with the
    // half-warp's two lines 8 apart (column kz or row y), every 8-byte access
    // of a half-warp hits distinct bank pairs.  Columns need the plane staged
    // in shared memory (x-quads); the FFT form's columns stay lane-per-column
    // for coalesced global loads.
    constexpr bool WLR = N == 128 && G == 8 && GR == 8 && R1R == 8;
    constexpr bool WLC = WLR && QUAD && R1 == 16;
    const int lg = l >> 3, lm = l & 7;  // group (line) within the warp, thread within the group

    // columns: inverse DFT along ky
    if constexpr (WLC) {
#pragma unroll 1
        for (int c = 0; c < CC; ++c) {
            const int s = 32 * c + w + 8 * lg;  // < NS
            float2 v[16];
#pragma unroll
            for (int r = 0; r < 16; ++r) {
                const int ky = lm + 8 * r;
                if (s == 0) {
                    const float2 d = plane[ky * H], ny = plane[ky * H + NS];
                    v[r] = make_float2(d.x - ny.y, d.y + ny.x);
                } else {
                    v[r] = plane[ky * H + s];
                }
            }
            dft<16, +1>(v);
            __syncwarp();  // the group's column is read: its slots take the outputs
#pragma unroll
            for (int r = 0; r < 16; ++r) plane[(16 * lm + ((r + lm) & 15)) * H + s] = v[r];
            __syncwarp();
            float2 out[16];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int j = lm + 8 * i;
                float2 u[8];
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    float2 a = plane[(16 * r + ((j + r) & 15)) * H + s];  // position j + 16 r
                    if (r != 0) a = ctwiddle<+1>(a, tws[j * r]);
                    u[r] = a;
                }
                dft<8, +1>(u);
#pragma unroll
                for (int r = 0; r < 8; ++r) out[i * 8 + r] = u[r];
            }
            __syncwarp();
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    const int y = lm + 8 * i + 16 * r;
                    const float2 o = out[i * 8 + r];
                    if (s == 0) {
                        plane[y * H] = make_float2(o.x, 0.f);
                        plane[y * H + NS] = make_float2(o.y, 0.f);
                    } else {
                        plane[y * H + s] = o;
                    }
                }
        }
    } else {
#pragma unroll 1
        for (int c = 0; c < CC; ++c) {
            const int s = 32 * c + l;
            const bool valid = s < NS;
            float2 v[R1];
#pragma unroll
            for (int r = 0; r < R1; ++r) {
                const int ky = w + G * r;
                float2 a = make_float2(0.f, 0.f);
                if (valid) {
                    if (s == 0) {
                        const float2 d = src[ky * H], ny = src[ky * H + NS];
                        a = make_float2(d.x - ny.y, d.y + ny.x);
                    } else {
                        a = src[ky * H + s];
                    }
                }
                v[r] = a;
            }
            dft<R1, +1>(v);
            if constexpr (QUAD) __syncthreads();  // the staged columns are read: their slots take the outputs
            if (valid) {
#pragma unroll
                for (int r = 0; r < R1; ++r) plane[(w * R1 + r) * H + s] = v[r];
            }
            __syncthreads();
            if (valid) {
                float2 out[R1];
                line_pass2<PC, +1, 1, H>(plane, w, s, tws, out);
#pragma unroll
                for (int i = 0; i < PC::NB; ++i)
#pragma unroll
                    for (int r = 0; r < G; ++r) {
                        const int y = w + G * i + R1 * r;
                        const float2 o = out[i * G + r];
                        if (s == 0) {
                            plane[y * H] = make_float2(o.x, 0.f);
                            plane[y * H + NS] = make_float2(o.y, 0.f);
                        } else {
                            plane[y * H + s] = o;
                        }
                    }
            }
        }
    }
    __syncthreads();

    // rows: C2R along kz via an N/2-point complex inverse DFT.  Each row's N
    // real outputs replace its spectrum in shared memory, and every thread
    // keeps the smallest (value, offset) it produced.
    const int gi = w / GR, m = WLR ? lm : w % GR;
    // the row a thread works on in round ro
    auto row_of = [&](int ro) { return WLR ? 32 * ro + w + 8 * lg : ro * ROWS + gi * 32 + l; };
    float bmin_v = INFINITY;
    int bmin_i = 0x7fffffff;
#pragma unroll 1
    for (int ro = 0; ro < ROUNDS; ++ro) {
        const int y = row_of(ro);
        const bool valid = y < N;
        float2* row = plane + (valid ? y : 0) * H;
        float2 v[R1R];
#pragma unroll
        for (int r = 0; r < R1R; ++r) {
            const int k = m + GR * r;
            float2 yk = make_float2(0.f, 0.f);
            if (valid) {
                const float2 X = row[k], Xm = row[NS - k];
                // A = X + conj(Xm), B = X - conj(Xm), Y = A + i * conj(w^k) * B
                const float2 A = make_float2(X.x + Xm.x, X.y - Xm.y);
                const float2 B = make_float2(X.x - Xm.x, X.y + Xm.y);
                const float2 cb = cmul_conj(B, tws[k]);
                yk = make_float2(A.x - cb.y, A.y + cb.x);
            }
            v[r] = yk;
        }
        float2 out[R1R];
        if constexpr (WLR) {
            __syncwarp();
            dft<8, +1>(v);
#pragma unroll
            for (int r = 0; r < 8; ++r) row[8 * m + ((r + m) & 7)] = v[r];
            __syncwarp();
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                float2 a = row[8 * r + ((m + r) & 7)];  // position m + 8 r
                if (r != 0) a = ctwiddle<+1>(a, tws[2 * m * r]);
                out[r] = a;
            }
            dft<8, +1>(out);
            __syncwarp();  // the row's spectrum is consumed: its slots take the real outputs
        } else {
            __syncthreads();
            dft<R1R, +1>(v);
            if (valid) {
#pragma unroll
                for (int r = 0; r < R1R; ++r) row[m * R1R + r] = v[r];
            }
            __syncthreads();
            if (valid) line_pass2<PR, +1, 2, 1>(row, m, 0, tws, out);
            __syncthreads();  // the row's spectrum is consumed: its slots take the real outputs
        }
        const int rowbase = (x * N + y) * N;
#pragma unroll
        for (int i = 0; i < PR::NB; ++i)
#pragma unroll
            for (int r = 0; r < GR; ++r) {
                const int mm = m + GR * i + R1R * r;
                const float2 o = out[i * GR + r];
                if (valid) {
                    row[mm] = o;
                    if constexpr (DBG) reinterpret_cast<float2*>(dbg + (size_t)q * N * N * N + rowbase)[mm] = o;
                    if (better(o.x, rowbase + 2 * mm, bmin_v, bmin_i)) { bmin_v = o.x; bmin_i = rowbase + 2 * mm; }
                    if (better(o.y, rowbase + 2 * mm + 1, bmin_v, bmin_i)) { bmin_v = o.y; bmin_i = rowbase + 2 * mm + 1; }
                }
            }
    }

    // Selection.  The KC-th best of the threads' minima bounds the plane's
    // KC-th best from above (at least KC cells lie at or below it), so only
    // cells at or below it can enter the plane's top KC.
    // Every warp sorts its threads' minima; warp 0 merges the warps' 16 best
    // (the KC best of all minima are among them).
    static_assert(KC == 16, "the bitonic selection keeps 16 of 32 lanes");
    // lists 0 .. nl-1 of KC (lv_s, li_s, ascending) merged pairwise over
    // log2(nl) levels into list 0 (warp w merges list w + step into list w);
    // every thread calls it
    auto tree_merge = [&](int nl) {
        for (int step = 1; step < nl; step <<= 1) {
            __syncthreads();
            if ((w & (2 * step - 1)) == 0 && w + step < nl) {
                float sv = l < KC ? lv_s[w * KC + l] : lv_s[(w + step) * KC + 31 - l];
                int si = l < KC ? li_s[w * KC + l] : li_s[(w + step) * KC + 31 - l];
                warp_merge32(sv, si, l);
                if (l < KC) {
                    lv_s[w * KC + l] = sv;
                    li_s[w * KC + l] = si;
                }
            }
        }
        __syncthreads();
    };
    {
        float sv = bmin_v;
        int si = bmin_i;
        warp_sort32(sv, si, l);
        if (l < KC) {
            lv_s[w * KC + l] = sv;
            li_s[w * KC + l] = si;
        }
    }
    if (tid == 0) n_cand = 0;
    tree_merge(G);
    const float tv = lv_s[KC - 1];
    const int ti = li_s[KC - 1];
    auto offer = [&](float v, int i) {
        if (!better(tv, ti, v, i)) {
            const int at = atomicAdd(&n_cand, 1);
            if (at < PCAND) { cand_sv[at] = v; cand_si[at] = i; }
        }
    };
    if constexpr (WLR) {
        // only a thread whose own minimum is at or below the bound holds
        // cells at or below it (usually a few per plane): the warp re-reads
        // each such lane's 64 cells together, two per lane (lane j: round
        // j / 8, radix position j % 8 of the row pass)
        unsigned qual = __ballot_sync(0xffffffffu, !better(tv, ti, bmin_v, bmin_i));
        while (qual) {
            const int L = __ffs(qual) - 1;
            qual &= qual - 1u;
            const int y = 32 * (l >> 3) + w + 8 * (L >> 3);
            const int mm = (L & 7) + 8 * (l & 7);
            const float2 o = plane[y * H + mm];
            const int rowbase = (x * N + y) * N;
            offer(o.x, rowbase + 2 * mm);
            offer(o.y, rowbase + 2 * mm + 1);
        }
    } else {
        // every thread re-reads its own cells (the positions the row pass gave it)
#pragma unroll 1
        for (int ro = 0; ro < ROUNDS; ++ro) {
            const int y = row_of(ro);
            if (y >= N) continue;
            const float2* row = plane + y * H;
            const int rowbase = (x * N + y) * N;
#pragma unroll
            for (int i = 0; i < PR::NB; ++i)
#pragma unroll
                for (int r = 0; r < GR; ++r) {
                    const int mm = m + GR * i + R1R * r;
                    const float2 o = row[mm];
                    offer(o.x, rowbase + 2 * mm);
                    offer(o.y, rowbase + 2 * mm + 1);
                }
        }
    }
    __syncthreads();
    const int nc = n_cand;
    if (nc <= PCAND) {
        // warp w sorts chunks w, w + G, .. of 32 candidates and keeps their
        // best KC in list w; the lists are then tree-merged
        const int nchunk = (nc + 31) >> 5;
        float sv = INFINITY;
        int si = 0x7fffffff;
        for (int c = w; c < nchunk; c += G) {
            const int e = 32 * c + l;
            float cv = e < nc ? cand_sv[e] : INFINITY;
            int ci = e < nc ? cand_si[e] : 0x7fffffff;
            warp_sort32(cv, ci, l);
            if (c == w) {
                sv = cv;
                si = ci;
            } else {
                const float rv = __shfl_sync(0xffffffffu, cv, 31 - l);
                const int ri = __shfl_sync(0xffffffffu, ci, 31 - l);
                if (l >= KC) {
                    sv = rv;
                    si = ri;
                }
                warp_merge32(sv, si, l);
            }
        }
        if (l < KC) {
            lv_s[w * KC + l] = sv;
            li_s[w * KC + l] = si;
        }
        tree_merge(nchunk < G ? nchunk : G);
        if (w == 0 && l < KC) {
            cand_v[((size_t)q * N + x) * KC + l] = lv_s[l];
            cand_i[((size_t)q * N + x) * KC + l] = li_s[l];
        }
        return;
    }
    // many cells tie at the bound (a flat plane): every warp offers its own
    // cells, then warp 0 merges the warps' lists
    WarpTopK tk;
    tk.init();
#pragma unroll 1
    for (int ro = 0; ro < ROUNDS; ++ro) {
        const int y = row_of(ro);
        const bool valid = y < N;
        const float2* row = plane + (valid ? y : 0) * H;
        const int rowbase = (x * N + y) * N;
#pragma unroll
        for (int i = 0; i < PR::NB; ++i)
#pragma unroll
            for (int r = 0; r < GR; ++r) {
                const int mm = m + GR * i + R1R * r;
                const float2 o = valid ? row[mm] : make_float2(INFINITY, INFINITY);
                tk.offer(o.x, valid ? rowbase + 2 * mm : 0x7fffffff, l);
                tk.offer(o.y, valid ? rowbase + 2 * mm + 1 : 0x7fffffff, l);
            }
    }
    if (l < KC) {
        lv_s[w * KC + l] = tk.lv;
        li_s[w * KC + l] = tk.li;
    }
    __syncthreads();
    if (w == 0) {
        merge_lists(lv_s, li_s, G * KC, tk, l);
        if (l < KC) {
            cand_v[((size_t)q * N + x) * KC + l] = tk.lv;
            cand_i[((size_t)q * N + x) * KC + l] = tk.li;
        }
    }
}

// ---------------------------------------------------------------------------
// K4: per-rotation merge of the plane pools, FP64 direct-space rescoring of
// the KC survivors, ascending order and the maxValCorr limit, translation by
// WrappedIndex::unwrap (docking_fft.hpp:316-389, Math/fft.hpp:199-206,
// Common/queue.hpp:221-251).
// ---------------------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(256) finalize_kernel(
    const float* __restrict__ cand_v, const int32_t* __restrict__ cand_i, const uint32_t* __restrict__ ent,
    const int32_t* __restrict__ status, const double* __restrict__ rgrid, int n_ent, int peak_stride, int k_out,
    double max_val, double h, int first_rot_id, fftdock_peak* __restrict__ peaks, int32_t* __restrict__ n_peaks,
    float* __restrict__ pool_v, int32_t* __restrict__ pool_i, const double* __restrict__ w64,
    const int32_t* __restrict__ ent_idx) {
    __shared__ float lv_s[8 * KC];
    __shared__ int li_s[8 * KC];
    __shared__ double score_s[KC];
    const int q = blockIdx.x;
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
    const long V = (long)N * N * N;
    WarpTopK tk;
    tk.init();
    const float* cv = cand_v + (size_t)q * N * KC;
    const int32_t* ci = cand_i + (size_t)q * N * KC;
    for (int base = w * 32; base < N * KC; base += 256) {
        const int e = base + l;
        const float v = e < N * KC ? cv[e] : INFINITY;
        const int i = e < N * KC ? ci[e] : 0x7fffffff;
        tk.offer(v, i, l);
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
            const int sx = off / (N * N), sy = (off / N) % N, sz = off % N;
            for (int j = l; j < n_ent; j += 32) {
                const uint32_t u = e_q[j];
                const int t = (int)(u >> 24);
                const int ax = (int)((u >> 16) & 255u), ay = (int)((u >> 8) & 255u), az = (int)(u & 255u);
                const int gx = ax - sx < 0 ? ax - sx + N : ax - sx;
                const int gy = ay - sy < 0 ? ay - sy + N : ay - sy;
                const int gz = az - sz < 0 ? az - sz + N : az - sz;
                const double rv = rgrid[(size_t)t * V + ((size_t)gx * N + gy) * N + gz];
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
        for (int c = 0; c < KC; ++c) { sc[c] = score_s[c]; of[c] = li_s[c]; }
        for (int a = 1; a < KC; ++a) {
            const double s = sc[a];
            const int o = of[a];
            int b = a - 1;
            while (b >= 0 && (sc[b] > s || (sc[b] == s && of[b] > o))) {
                sc[b + 1] = sc[b]; of[b + 1] = of[b]; --b;
            }
            sc[b + 1] = s; of[b + 1] = o;
        }
        int n = 0;
        if (status[q] == 0) {
            for (int c = 0; c < KC && n < k_out; ++c) {
                if (!(sc[c] < max_val) || of[c] < 0 || of[c] >= V) continue;
                const int sx = of[c] / (N * N), sy = (of[c] / N) % N, sz = of[c] % N;
                fftdock_peak pk;
                pk.rot_id = first_rot_id + q;
                pk.cell[0] = sx; pk.cell[1] = sy; pk.cell[2] = sz;
                const int s3[3] = {sx, sy, sz};
                for (int d = 0; d < 3; ++d) {
                    int yv = -s3[d];
                    if (yv < -(N / 2)) yv += N;
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

// generic batched line transform: line L -> base (L / inner_count) *
// outer_stride + (L % inner_count) * inner_stride, element e at base +
// e * elem_stride.  In place.  CTA = G warps x 32 lines.
template <typename T, int N, int SIGN>
__global__ void __launch_bounds__(32 * SizeTraits<N>::G) line_fft_kernel(
    cplx_t<T>* __restrict__ data, const cplx_t<T>* __restrict__ tw, long n_lines, long elem_stride, long inner_count,
    long inner_stride, long outer_stride) {
    using C = cplx_t<T>;
    using P = LinePlan<N, SizeTraits<N>::G>;
    constexpr int G = P::G, R1 = P::R1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* buf = reinterpret_cast<C*>(smem_raw);  // [N][32]
    C* tws = buf + N * 32;                    // [N]
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
    for (int i = tid; i < N; i += blockDim.x) tws[i] = tw[i];
    const long L = (long)blockIdx.x * 32 + l;
    const bool valid = L < n_lines;
    const long base = valid ? (L / inner_count) * outer_stride + (L % inner_count) * inner_stride : 0;
    C v[R1];
#pragma unroll
    for (int r = 0; r < R1; ++r) v[r] = valid ? data[base + (long)(w + G * r) * elem_stride] : cmake<C>(0, 0);
    dft<R1, SIGN>(v);
#pragma unroll
    for (int r = 0; r < R1; ++r) buf[(w * R1 + r) * 32 + l] = v[r];
    __syncthreads();
    C out[R1];
    line_pass2<P, SIGN, 1, 32>(buf, w, l, tws, out);
    if (valid) {
#pragma unroll
        for (int i = 0; i < P::NB; ++i)
#pragma unroll
            for (int r = 0; r < G; ++r) data[base + (long)(w + G * i + R1 * r) * elem_stride] = out[i * G + r];
    }
}

static __global__ void complexify_kernel(const double* __restrict__ re, double2* __restrict__ out, size_t V) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < V) out[i] = make_double2(re[i], 0.0);
}

// [N][N][N] complex -> [N][N][H] (kz < H)
static __global__ void half_extract_kernel(const double2* __restrict__ full, double2* __restrict__ half, int n, int h2) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t tot = (size_t)n * n * h2;
    if (i >= tot) return;
    const size_t row = i / h2;
    const int kz = (int)(i - row * h2);
    half[i] = full[row * n + kz];
}

__device__ __forceinline__ void spec_store(float2* p, float x, float y) { *p = make_float2(x, y); }
__device__ __forceinline__ void spec_store(__nv_bfloat162* p, float x, float y) { *p = __floats2bfloat162_rn(x, y); }

// [N][N*H] double -> [N][PP] FP32 or BF16 pairs scaled by 1/V
template <typename SpecT>
static __global__ void pack_spectrum_kernel(const double2* __restrict__ half, SpecT* __restrict__ spec, int n, int nh,
                                     int pp, double scale) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t tot = (size_t)n * pp;
    if (i >= tot) return;
    const size_t kx = i / pp;
    const int p = (int)(i - kx * pp);
    float ox = 0.f, oy = 0.f;
    if (p < nh) {
        const double2 v = half[kx * nh + p];
        ox = (float)(v.x * scale);
        oy = (float)(v.y * scale);
    }
    spec_store(spec + i, ox, oy);
}

}  // namespace fftdock
