// Queue + translational clustering stage of a batch (cfg.cluster_trans).
//
// Reference path per rotation: CorrelationProcessor::selectIntoQueue into a
// BoundPriorityQueue of maxNTransInp entries (include/PRODDL/docking_fft.hpp:
// 316-345,452-468, include/PRODDL/Common/queue.hpp:221-251), TranClust::process
// (docking_fft.hpp:57-113) over ClusterMatrix::cluster / getClusters
// (include/PRODDL/Geom/cluster.hpp:121-477), then getTranValuesFilled(maxNTrans)
// (docking_app.hpp:460, docking_fft.hpp:430-447).
//
// GPU form, per batch of rotations whose correlation grids the plane kernel
// has written to wide.corr ([B][N^3] float, cell offset order):
//   1. bound: the plane kernel's per-plane top-16 pools give an upper bound
//      on the queue's last value when m <= 16 N: the m-th smallest pooled
//      value, and the ceil(m/16)-th smallest of the planes' 16th values (at
//      least m cells lie at or below either);
//   2. gather: one streaming pass appends every cell below maxValCorr and at
//      or below the bound (64-bit keys: order-preserving float bits << 32 |
//      cell offset, unique, so ties resolve to the lower offset);
//   3. only if that set overflows kWideMax (or there was no bound): a radix
//      select, one 12-bit digit per pass (six passes at most), narrows the
//      set to the bin holding the m-th key, and a second gather collects it;
//   4. finish (one CTA per rotation): bitonic sort of the gathered keys in
//      shared memory, the first m are the queue; the leader walk of the
//      clustering; FP64 direct-space rescoring of the kept leaders; peaks.
// Predicates are evaluated in FP32 against maxValCorr rounded up to the next
// float, which selects exactly the floats whose double value is below it.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fftdock.h"
#include "internal.h"

namespace fftdock {
namespace {

typedef unsigned long long u64;

constexpr int kChunk = 16384;  // cells per CTA in the first gather pass
// cells per CTA in the radix passes and the final gather when a bound exists
// (only rotations whose gathered set overflowed take that path): a grid of a
// few CTAs per rotation keeps their mostly idle launches short.  Without a
// bound every rotation takes the radix path and they use kChunk.
constexpr int kRadixChunk = 16 * kChunk;
constexpr int kPassThreads = 256;
constexpr int kDigitBits = 12;
constexpr int kMaxPasses = 6;  // 5 x 12 + 4 = 64 key bits
constexpr int kFinishThreads = 1024;
constexpr int kMaxLeaders = FFTDOCK_MAX_PEAKS;
static_assert(kMaxLeaders <= kWidePool, "the leader arrays hold at most kWidePool entries");
constexpr int kPoolPerPlane = 16;  // KC of the plane kernel
constexpr int kPoolMax = 4096;     // >= 16 * largest grid edge, power of two

static_assert((1 << kDigitBits) == kWideBins, "digit width and bin count disagree");
static_assert(kChunk % (4 * kPassThreads) == 0, "chunks are read as float4 by every thread");

// order-preserving map of a float onto uint32 (-0 folded onto +0)
__device__ __forceinline__ uint32_t float_key(float v) {
    const uint32_t u = __float_as_uint(v == 0.0f ? 0.0f : v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float lane_elem(const float4& f, int j) {
    return j == 0 ? f.x : j == 1 ? f.y : j == 2 ? f.z : f.w;
}

// ascending bitonic sort of P (power of two) floats in shared memory
__device__ void block_sort_f(float* a, int P) {
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const float x = a[i], y = a[ixj];
                    if ((x > y) == ((i & k) == 0)) {
                        a[i] = y;
                        a[ixj] = x;
                    }
                }
            }
            __syncthreads();
        }
}

// per rotation: state, cleared histogram and counter, and the upper bound
// of the queue's last value from the plane pools ([B][N][16])
__global__ void __launch_bounds__(256) wide_bound_kernel(const float* __restrict__ pool, int N, int m,
                                                         WideState* __restrict__ st, uint32_t* __restrict__ hist,
                                                         int32_t* __restrict__ cnt) {
    __shared__ float pv[kPoolMax];
    __shared__ float tp[256];
    const int q = blockIdx.x;
    for (int i = threadIdx.x; i < kWideBins; i += blockDim.x) hist[(size_t)q * kWideBins + i] = 0;
    const int np = N * kPoolPerPlane;
    float thr = INFINITY;
    if (m <= np) {
        int P = 2;
        while (P < np) P <<= 1;
        const float* src = pool + (size_t)q * np;
        for (int i = threadIdx.x; i < P; i += blockDim.x) pv[i] = i < np ? src[i] : INFINITY;
        for (int p = threadIdx.x; p < 256; p += blockDim.x) {
            float mx = INFINITY;
            if (p < N) {
                mx = src[p * kPoolPerPlane];
                for (int c = 1; c < kPoolPerPlane; ++c) mx = fmaxf(mx, src[p * kPoolPerPlane + c]);
            }
            tp[p] = mx;
        }
        __syncthreads();
        block_sort_f(pv, P);
        block_sort_f(tp, 256);
        thr = fminf(pv[m - 1], tp[(m + kPoolPerPlane - 1) / kPoolPerPlane - 1]);
    }
    if (threadIdx.x == 0) {
        // without a bound the gathered set would be the whole grid: go
        // straight to the radix path
        const bool bounded = thr < INFINITY;
        WideState s;
        s.pfx = 0;
        s.nres = 0;
        s.need = m;
        s.below = 0;
        s.active = bounded ? 0 : 1;
        s.flags = bounded ? 0 : kWideRadix;
        s.thr = thr;
        st[q] = s;
        cnt[q] = 0;
    }
}

// after the bounded gather: rotations whose set overflowed take the radix path
__global__ void wide_check_kernel(WideState* __restrict__ st, int32_t* __restrict__ cnt, int nb) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nb) return;
    if (cnt[q] > kWideMax) {
        st[q].flags |= kWideRadix;
        st[q].active = 1;
        cnt[q] = 0;
    }
}

// histogram of the next digit of the keys inside each active rotation's bin
__global__ void __launch_bounds__(kPassThreads) wide_digit_kernel(const float* __restrict__ corr, long V,
                                                                  const WideState* __restrict__ st,
                                                                  uint32_t* __restrict__ hist, float mv,
                                                                  long chunk) {
    __shared__ uint32_t sh[kWideBins];
    const int q = blockIdx.y;
    const WideState s = st[q];
    if (!s.active) return;
    for (int i = threadIdx.x; i < kWideBins; i += blockDim.x) sh[i] = 0;
    __syncthreads();
    const int rem = 64 - s.nres;  // unresolved bits, > 0 while active
    const int bits = rem < kDigitBits ? rem : kDigitBits;
    const int shift = rem - bits;
    const u64 want = s.nres ? (s.pfx >> rem) : 0ull;
    const uint32_t dmask = (1u << bits) - 1u;
    const long c0 = (long)blockIdx.x * chunk;
    const long c1 = c0 + chunk < V ? c0 + chunk : V;
    const float4* src = reinterpret_cast<const float4*>(corr + (size_t)q * V);
    const int lane = threadIdx.x & 31;
    for (long e4 = c0 / 4 + threadIdx.x; e4 < c1 / 4; e4 += blockDim.x) {
        const float4 f = src[e4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float v = lane_elem(f, j);
            const u64 key = ((u64)float_key(v) << 32) | (u64)(4 * e4 + j);
            const bool in = v < mv && v <= s.thr && (s.nres == 0 || (key >> rem) == want);
            const uint32_t d = in ? (uint32_t)(key >> shift) & dmask : 0xffffffffu;
            const unsigned am = __activemask();
            const unsigned peers = __match_any_sync(am, d);
            if (in && lane == __ffs(peers) - 1) atomicAdd(&sh[d], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kWideBins; i += blockDim.x)
        if (sh[i]) atomicAdd(&hist[(size_t)q * kWideBins + i], sh[i]);
}

// fix the digit holding the need-th key of the bin; clear the histogram
__global__ void __launch_bounds__(256) wide_pick_kernel(WideState* __restrict__ st, uint32_t* __restrict__ hist) {
    constexpr int PER = kWideBins / 256;
    __shared__ uint32_t wsum[8];
    const int q = blockIdx.x;
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
    WideState s = st[q];
    if (!s.active) return;
    uint32_t* hq = hist + (size_t)q * kWideBins;
    uint32_t loc[PER];
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        loc[i] = hq[tid * PER + i];
        sum += loc[i];
    }
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (l >= o) incl += t;
    }
    if (l == 31) wsum[w] = incl;
    __syncthreads();
    uint32_t before = 0, total = 0;
    for (int k = 0; k < 8; ++k) {
        if (k < w) before += wsum[k];
        total += wsum[k];
    }
    const uint32_t excl = before + incl - sum;
#pragma unroll
    for (int i = 0; i < PER; ++i) hq[tid * PER + i] = 0;
    const uint32_t need = (uint32_t)s.need;
    if (s.nres == 0 && total < need) {
        // fewer cells than the queue bound pass maxValCorr: keep them all
        if (tid == 0) {
            s.flags |= kWideAll;
            s.active = 0;
            st[q] = s;
        }
        return;
    }
    if (excl < need && excl + sum >= need) {
        const int rem = 64 - s.nres;
        const int bits = rem < kDigitBits ? rem : kDigitBits;
        const int shift = rem - bits;
        uint32_t c = excl;
        int d = tid * PER + PER - 1;
        uint32_t inbin = 0;
        for (int i = 0; i < PER; ++i) {
            if (c + loc[i] >= need) {
                d = tid * PER + i;
                inbin = loc[i];
                break;
            }
            c += loc[i];
        }
        s.below += (int)c;
        s.need -= (int)c;
        s.pfx |= (u64)d << shift;
        s.nres += bits;
        if ((long)s.below + inbin <= kWideMax || s.nres >= 64) s.active = 0;
        st[q] = s;
    }
}

// append the cells of each rotation's set to its key list.  phase 0 (bounded
// rotations): every cell below maxValCorr and at or below the bound (the
// count may exceed kWideMax; only kWideMax keys are stored).  phase 1
// (radix-path rotations): every such cell whose key is at or below the final
// bin.
__global__ void __launch_bounds__(kPassThreads) wide_gather_kernel(const float* __restrict__ corr, long V,
                                                                   const WideState* __restrict__ st,
                                                                   u64* __restrict__ cand, int32_t* __restrict__ cnt,
                                                                   float mv, int phase, long chunk) {
    const int q = blockIdx.y;
    const WideState s = st[q];
    const bool radix = (s.flags & kWideRadix) != 0;
    if (radix != (phase == 1)) return;
    const bool all = phase == 0 || (s.flags & kWideAll) != 0 || s.nres == 0;
    const int rem = 64 - s.nres;
    const u64 bound = all ? 0ull : (s.pfx >> rem);
    const long c0 = (long)blockIdx.x * chunk;
    const long c1 = c0 + chunk < V ? c0 + chunk : V;
    const float4* src = reinterpret_cast<const float4*>(corr + (size_t)q * V);
    u64* out = cand + (size_t)q * kWideMax;
    const int lane = threadIdx.x & 31;
    for (long e4 = c0 / 4 + threadIdx.x; e4 < c1 / 4; e4 += blockDim.x) {
        const float4 f = src[e4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float v = lane_elem(f, j);
            bool ok = v < mv && v <= s.thr;
            u64 key = 0;
            if (ok) {
                key = ((u64)float_key(v) << 32) | (u64)(4 * e4 + j);
                ok = all || (key >> rem) <= bound;
            }
            const unsigned am = __activemask();
            const unsigned mask = __ballot_sync(am, ok);
            if (mask == 0u) continue;
            const int leader = __ffs(mask) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(&cnt[q], __popc(mask));
            base = __shfl_sync(am, base, leader);
            if (ok) {
                const int idx = base + __popc(mask & ((1u << lane) - 1u));
                if (idx < kWideMax) out[idx] = key;
            }
        }
    }
}

__device__ __forceinline__ void translation_of(int off, int N, double h, int* cell, double* t) {
    cell[0] = off / (N * N);
    cell[1] = (off / N) % N;
    cell[2] = off % N;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int y = -cell[d];
        if (y < -(N / 2)) y += N;
        t[d] = h * (double)y;
    }
}

// (dx^2 + dy^2) + dz^2 in FP64 without contraction (blitz sum order)
__device__ __forceinline__ double dist2(const double* a, double bx, double by, double bz) {
    const double dx = __dsub_rn(a[0], bx), dy = __dsub_rn(a[1], by), dz = __dsub_rn(a[2], bz);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__global__ void __launch_bounds__(kFinishThreads) wide_finish_kernel(
    const u64* __restrict__ cand, const int32_t* __restrict__ cnt, const uint32_t* __restrict__ ent,
    const int32_t* __restrict__ status, const double* __restrict__ rgrid, int n_ent, int N, int m, int order,
    double rad2, int max_out, int k_out, double max_val, int peak_stride, double h, int first_rot_id,
    fftdock_peak* __restrict__ peaks, int32_t* __restrict__ n_peaks, const double* __restrict__ w64,
    const int32_t* __restrict__ ent_idx) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    u64* keys = reinterpret_cast<u64*>(smem_raw);  // [kWideMax]
    __shared__ int lead_pos[kWidePool];
    __shared__ double lead_t[kMaxLeaders][3];
    __shared__ double score_s[kWidePool];
    __shared__ int off_s[kWidePool];
    __shared__ int n_lead_s;
    const int q = blockIdx.x;
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
    const long V = (long)N * N * N;
    int n = cnt[q];
    if (n > kWideMax) n = kWideMax;
    int P = 2;
    while (P < n) P <<= 1;
    const u64* src = cand + (size_t)q * kWideMax;
    for (int i = tid; i < P; i += blockDim.x) keys[i] = i < n ? src[i] : ~0ull;
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < P; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const u64 a = keys[i], b = keys[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        keys[i] = b;
                        keys[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    const int me = n < m ? n : m;  // the queue: the first me keys, ascending
    if (order == kWideNoClustering) {
        // no clustering: every queue entry is a candidate
        const int nq = me < kWidePool ? me : kWidePool;
        for (int c = tid; c < nq; c += blockDim.x) lead_pos[c] = c;
        if (tid == 0) n_lead_s = nq;
    } else if (w == 0) {
        int nl = 0;
        for (int base = 0; base < me && nl < max_out; base += 32) {
            const int k = base + l;
            const bool valid = k < me;
            const int pos = order == FFTDOCK_CLUSTER_ORDER_BEST_FIRST ? k : me - 1 - k;
            int cell[3];
            double t[3];
            translation_of(valid ? (int)(uint32_t)keys[pos] : 0, N, h, cell, t);
            bool covered = !valid;
            for (int j = 0; j < nl && !covered; ++j)
                covered = dist2(t, lead_t[j][0], lead_t[j][1], lead_t[j][2]) <= rad2;
            unsigned un = __ballot_sync(0xffffffffu, !covered);
            while (un != 0u && nl < max_out) {
                const int src_l = __ffs(un) - 1;
                const double lx = __shfl_sync(0xffffffffu, t[0], src_l);
                const double ly = __shfl_sync(0xffffffffu, t[1], src_l);
                const double lz = __shfl_sync(0xffffffffu, t[2], src_l);
                if (l == src_l) {
                    lead_pos[nl] = pos;
                    lead_t[nl][0] = t[0];
                    lead_t[nl][1] = t[1];
                    lead_t[nl][2] = t[2];
                    covered = true;
                }
                ++nl;
                if (l > src_l && !covered) covered = dist2(t, lx, ly, lz) <= rad2;
                un = __ballot_sync(0xffffffffu, !covered);
            }
            __syncwarp();
        }
        if (l == 0) n_lead_s = nl;
    }
    __syncthreads();
    const int nl = n_lead_s;
    // FP64 direct-space rescoring, one warp per leader (same summation as
    // the finalize kernel of the default path)
    for (int c = w; c < nl; c += kFinishThreads / 32) {
        const int off = (int)(uint32_t)keys[lead_pos[c]];
        const uint32_t* e_q = ent + (size_t)q * n_ent;
        const int sx = off / (N * N), sy = (off / N) % N, sz = off % N;
        double sum = 0.0;
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
        if (l == 0) score_s[c] = sum;
    }
    __syncthreads();
    if (order == kWideNoClustering) {
        // sort the rescored queue by (energy, offset), then the first k_out
        // below maxValCorr are the peaks, ascending
        int P2 = 1;
        while (P2 < nl) P2 <<= 1;
        for (int i = tid; i < P2; i += blockDim.x) {
            off_s[i] = i < nl ? (int)(uint32_t)keys[lead_pos[i]] : 0x7fffffff;
            if (i >= nl) score_s[i] = INFINITY;
        }
        __syncthreads();
        for (int kk = 2; kk <= P2; kk <<= 1)
            for (int j = kk >> 1; j > 0; j >>= 1) {
                for (int i = tid; i < P2; i += blockDim.x) {
                    const int ixj = i ^ j;
                    if (ixj > i) {
                        const double a = score_s[i], b = score_s[ixj];
                        const int oa = off_s[i], ob = off_s[ixj];
                        const bool a_after = a > b || (a == b && oa > ob);
                        if (a_after == ((i & kk) == 0)) {
                            score_s[i] = b;
                            score_s[ixj] = a;
                            off_s[i] = ob;
                            off_s[ixj] = oa;
                        }
                    }
                }
                __syncthreads();
            }
        if (tid == 0) {
            int np = 0;
            if (status[q] == 0) {
                for (int c = 0; c < nl && np < k_out; ++c) {
                    if (!(score_s[c] < max_val)) continue;
                    fftdock_peak pk;
                    pk.rot_id = first_rot_id + q;
                    translation_of(off_s[c], N, h, pk.cell, pk.t);
                    pk.score = score_s[c];
                    peaks[(size_t)q * peak_stride + np] = pk;
                    ++np;
                }
            }
            n_peaks[q] = np;
        }
        return;
    }
    if (tid == 0) {
        int np = 0;
        if (status[q] == 0) {
            for (int c = 0; c < nl; ++c) {
                fftdock_peak pk;
                pk.rot_id = first_rot_id + q;
                translation_of((int)(uint32_t)keys[lead_pos[c]], N, h, pk.cell, pk.t);
                pk.score = score_s[c];
                peaks[(size_t)q * peak_stride + np] = pk;
                ++np;
            }
        }
        n_peaks[q] = np;
    }
}

}  // namespace

cudaError_t wide_select_batch(const BatchArgs& a, int N, cudaStream_t s) {
    const int nb = a.n_rot;
    if (nb <= 0) return cudaSuccess;
    const WideArgs& w = a.wide;
    const long V = (long)N * N * N;
    if (N * kPoolPerPlane > kPoolMax || N > 256 || V % 4 != 0) return cudaErrorInvalidValue;
    // maxValCorr rounded up to a float: v < mv  <=>  (double)v < maxValCorr
    float mv = (float)a.max_val;
    if ((double)mv < a.max_val) mv = nextafterf(mv, INFINITY);
    wide_bound_kernel<<<nb, 256, 0, s>>>(a.cand_v, N, w.m, w.st, w.hist, w.cnt);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const dim3 grid((unsigned)((V + kChunk - 1) / kChunk), (unsigned)nb);
    const long rchunk = w.m > N * kPoolPerPlane ? (long)kChunk : (long)kRadixChunk;
    const dim3 grid_r((unsigned)((V + rchunk - 1) / rchunk), (unsigned)nb);
    wide_gather_kernel<<<grid, kPassThreads, 0, s>>>(w.corr, V, w.st, w.cand, w.cnt, mv, 0, (long)kChunk);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    wide_check_kernel<<<(nb + 127) / 128, 128, 0, s>>>(w.st, w.cnt, nb);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    for (int p = 0; p < kMaxPasses; ++p) {
        wide_digit_kernel<<<grid_r, kPassThreads, 0, s>>>(w.corr, V, w.st, w.hist, mv, rchunk);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        wide_pick_kernel<<<nb, 256, 0, s>>>(w.st, w.hist);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    wide_gather_kernel<<<grid_r, kPassThreads, 0, s>>>(w.corr, V, w.st, w.cand, w.cnt, mv, 1, rchunk);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const size_t sm = (size_t)kWideMax * sizeof(u64);
    e = cudaFuncSetAttribute((const void*)wide_finish_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    const int max_out = a.k_out < kMaxLeaders ? a.k_out : kMaxLeaders;
    wide_finish_kernel<<<nb, kFinishThreads, sm, s>>>(w.cand, w.cnt, a.ent, a.status, a.rgrid, a.n_ent, N, w.m,
                                                      w.order, w.rad2, max_out, a.k_out, a.max_val, a.peak_stride,
                                                      a.h, a.first_rot_id, a.peaks, a.n_peaks, a.lig_w64,
                                                      a.lig_w64 ? a.ent_idx : nullptr);
    return cudaGetLastError();
}

}  // namespace fftdock
