// Learned rotation proposal (no counterpart in the reference).
//
// A small network predicts, for one receptor/ligand pair and one rotation,
// the best (lowest) correlation score the FFT scan would find for that
// rotation, from a coarse occupancy grid of the rotated ligand and a
// receptor descriptor.  Rotations it ranks low are skipped before the scan;
// the exhaustive scan stays the fallback and the judge of its recall.
//
// Network (one sample):
//   x0  16^3 occupancy of the rotated ligand (atom count / 4 per cell; the
//       cube of half-width L = the ligand's largest atom distance from its
//       rotation centre, cell 2L/16)
//   a1 = relu(conv(x0;  1 -> 16, 3^3, stride 2, pad 1))   16 x 8^3
//   a2 = relu(conv(a1; 16 -> 32, 3^3, stride 2, pad 1))   32 x 4^3
//   a3 = relu(conv(a2; 32 -> 64, 3^3, stride 2, pad 1))   64 x 2^3 = 512
//   u  = [a3, receptor descriptor (128)]                  640
//   h1 = relu(W1 u + b1)                                  256
//   y  = w2 . h1 + b2
//
// Every contraction is a BF16 x BF16 -> FP32 GEMM on the tensor cores
// (mma.sync m16n8k16), batched over the samples: each convolution is an
// im2col matrix [samples x positions][taps x input channels] times the
// weights [taps x input channels][output channels] (activations stored
// channel-last), the fully connected layer [samples][640] x [640][256]; the
// backward pass multiplies the BF16 activation gradients by the transposed
// weights (input gradients, summed back over the taps by a gather: col2im)
// and by the im2col matrices (weight gradients, reduced over samples and
// positions with a deterministic split of K).
// Precision: BF16 copies of the FP32 master weights (the convolution weights
// also in [output channel][tap][input channel] order); activations x0, a1,
// a2, a3, u, h1 and activation gradients dzf, dz3, dz2, dz1 stored as BF16;
// every sum accumulated in FP32 in a fixed order; weight gradients FP32;
// Adam updates the FP32 masters.
//
// Training step (captured once in a CUDA graph, replayed per step): sample
// indices come from a hash of (seed, device step counter, slot), so a replay
// needs no host input.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "fftdock.h"
#include "internal.h"

namespace {

typedef __nv_bfloat16 bf16;

constexpr int G0 = 16;
constexpr int C1 = 16, C2 = 32, C3 = 64;
constexpr int D1 = 8, D2 = 4, D3 = 2;
constexpr int NX0 = G0 * G0 * G0;
constexpr int P1 = D1 * D1 * D1, P2 = D2 * D2 * D2, P3 = D3 * D3 * D3;  // output positions per layer
constexpr int K1 = 32, K2 = 27 * C1, K3 = 27 * C2;                      // im2col widths (conv1: 27 taps padded)
constexpr int NA3 = C3 * P3;
constexpr int DESC = FFTDOCK_PROPOSAL_DESC;
constexpr int NU = NA3 + DESC;
constexpr int HID = 256;

// parameter layout (FP32 masters and BF16 copies share it)
constexpr int OW1 = 0;
constexpr int OB1 = OW1 + C1 * 27;
constexpr int OW2 = OB1 + C1;
constexpr int OB2 = OW2 + C2 * C1 * 27;
constexpr int OW3 = OB2 + C2;
constexpr int OB3 = OW3 + C3 * C2 * 27;
constexpr int OF1 = OB3 + C3;  // [NU][HID], input-major
constexpr int OFB1 = OF1 + NU * HID;
constexpr int OF2 = OFB1 + HID;
constexpr int OFB2 = OF2 + HID;
constexpr int NPARAM = OFB2 + 1;
// permuted BF16 convolution weights: wp1[co][K1], wp2[co][tap * C1 + ci], wp3[co][tap * C2 + ci]
constexpr int OP1 = 0, OP2 = OP1 + C1 * K1, OP3 = OP2 + C2 * K2, NPERM = OP3 + C3 * K3;

constexpr int THREADS = 256;
constexpr int MAX_BATCH = 4096;
constexpr int PREDICT_CHUNK = 4096;
constexpr int WS_FLOATS = 1 << 19;  // split-K partial sums
constexpr int kColsumParts = 64;    // row blocks of a bias-gradient column sum

__device__ __forceinline__ float b2f(bf16 v) { return __bfloat162float(v); }
__device__ __forceinline__ bf16 f2b(float v) { return __float2bfloat16_rn(v); }

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    // splitmix64 finaliser
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// ---------------------------------------------------------------------------
// GEMM: C[M][N] = A[M][K] x B[K][N], BF16 operands, FP32 accumulation on the
// tensor cores.  A is row-major (AT = false: A[m * lda + k]) or stored
// transposed (AT = true: A[k * lda + m]); B likewise ("KN", BT = false:
// B[k * ldb + n]; "NK", BT = true: B[n * ldb + k]).  The contiguous extent of
// each operand and its leading dimension are multiples of 8 and its base is
// 16-byte aligned (checked by the host), so every global load is a uint4 of
// 8 elements.  CTA tile 64 x 64 x 32, four warps of 32 x 32; tiles staged in
// shared memory as [row][k] (pitch 40 elements: the fragment loads hit 32
// distinct banks).  gridDim.z > 1 splits K into equal multiples of 32; each
// split hands its partial sums to the epilogue with its index.
// ---------------------------------------------------------------------------
constexpr int GBM = 64, GBN = 64, GBK = 32, GPITCH = GBK + 8, GTHREADS = 128;

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// one 64 x 32 operand tile into smem[row][k]: rows r0.., k k0.. of a matrix
// whose element (row, k) is at p[row * ld + k] (T = false) or p[k * ld + row]
__device__ __forceinline__ void load_tile(bf16 (*s)[GPITCH], const bf16* __restrict__ p, int ld, bool T, int r0,
                                          int rows, int k0, int k1) {
    const int t = threadIdx.x;
    if (!T) {
        // 64 rows x 4 groups of 8 k
        for (int e = t; e < 64 * 4; e += GTHREADS) {
            const int rr = e >> 2, kk = (e & 3) * 8;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (r0 + rr < rows && k0 + kk < k1) v = *reinterpret_cast<const uint4*>(p + (size_t)(r0 + rr) * ld + k0 + kk);
            *reinterpret_cast<uint4*>(&s[rr][kk]) = v;
        }
    } else {
        // 32 k x 8 groups of 8 rows
        for (int e = t; e < 32 * 8; e += GTHREADS) {
            const int kk = e >> 3, rr = (e & 7) * 8;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (r0 + rr < rows && k0 + kk < k1) v = *reinterpret_cast<const uint4*>(p + (size_t)(k0 + kk) * ld + r0 + rr);
            const uint32_t q[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
                s[rr + i][kk] = __ushort_as_bfloat16((unsigned short)((q[i >> 1] >> (16 * (i & 1))) & 0xffffu));
        }
    }
}

template <bool AT, bool BT, class Epi>
__global__ void __launch_bounds__(GTHREADS) gemm_kernel(int M, int N, int K, const bf16* __restrict__ A, int lda,
                                                        const bf16* __restrict__ B, int ldb, int k_chunk, Epi epi) {
    __shared__ __align__(16) bf16 As[GBM][GPITCH];
    __shared__ __align__(16) bf16 Bs[GBN][GPITCH];
    const int m0 = blockIdx.y * GBM, n0 = blockIdx.x * GBN;
    const int kb = blockIdx.z * k_chunk, ke = min(K, kb + k_chunk);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int gid = lane >> 2, tig = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[i][j][c] = 0.f;
    for (int k0 = kb; k0 < ke; k0 += GBK) {
        load_tile(As, A, lda, AT, m0, M, k0, ke);
        load_tile(Bs, B, ldb, !BT, n0, N, k0, ke);
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < GBK; ks += 16) {
            uint32_t a[2][4], b[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + 16 * i + gid;
                a[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * tig]);
                a[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * tig]);
                a[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][ks + 2 * tig + 8]);
                a[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + 2 * tig + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int n = wn + 8 * j + gid;
                b[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[n][ks + 2 * tig]);
                b[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[n][ks + 2 * tig + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], a[i], b[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int r = m0 + wm + 16 * i + gid + (c >= 2 ? 8 : 0);
                const int n = n0 + wn + 8 * j + 2 * tig + (c & 1);
                if (r < M && n < N) epi(r, n, acc[i][j][c], blockIdx.z);
            }
}

// split-K partial sums ws[z][M][N] -> the epilogue, summed in split order
template <class Epi>
__global__ void splitk_reduce_kernel(const float* __restrict__ ws, int splits, int M, int N, Epi epi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M * N) return;
    float v = 0.f;
    for (int z = 0; z < splits; ++z) v += ws[(size_t)z * M * N + i];
    epi(i / N, i % N, v, 0);
}

struct EpiPartial {  // split-K: partial sums of split z
    float* ws;
    int M, N;
    __device__ void operator()(int r, int c, float v, int z) const { ws[((size_t)z * M + r) * N + c] = v; }
};
struct EpiF32 {
    float* out;
    int ld;
    __device__ void operator()(int r, int c, float v, int) const { out[(size_t)r * ld + c] = v; }
};
struct EpiBiasRelu {  // activations (channel-last rows)
    bf16* out;
    int ld;
    const bf16* bias;
    __device__ void operator()(int r, int c, float v, int) const {
        v += b2f(bias[c]);
        out[(size_t)r * ld + c] = f2b(v > 0.f ? v : 0.f);
    }
};
struct EpiConv3 {  // row s * P3 + pos, column co -> u[s][co * P3 + pos]
    bf16* u;
    const bf16* bias;
    __device__ void operator()(int r, int c, float v, int) const {
        v += b2f(bias[c]);
        u[(size_t)(r / P3) * NU + c * P3 + r % P3] = f2b(v > 0.f ? v : 0.f);
    }
};
struct EpiDz3 {  // dU[s][i], i = co * P3 + pos < NA3 -> dz3[s * P3 + pos][co], masked by u > 0
    bf16* dz3;
    const bf16* u;
    __device__ void operator()(int r, int c, float v, int) const {
        const bool on = b2f(u[(size_t)r * NU + c]) > 0.f;
        dz3[((size_t)r * P3 + c % P3) * C3 + c / P3] = f2b(on ? v : 0.f);
    }
};
struct EpiWgrad {  // column tap * cin + ci of output channel r -> g[(r * cin + ci) * 27 + tap]
    float* g;
    int cin;
    float* gbias;  // conv1: column 27 (the ones column of its im2col) is the bias gradient
    __device__ void operator()(int r, int c, float v, int) const {
        const int tap = c / cin, ci = c % cin;
        if (tap < 27) g[((size_t)r * cin + ci) * 27 + tap] = v;
        else if (gbias && tap == 27) gbias[r] = v;
    }
};

// ---------------------------------------------------------------------------
// samples, occupancy and the im2col / col2im gathers
// ---------------------------------------------------------------------------
struct Ligands {
    const double* xyz;    // all ligands' atoms, concatenated
    const int* start;     // first atom of each ligand
    const int* count;
    const double* half;   // L of each ligand
    const float* desc;    // [n_lig][DESC]
};

// where a batch's samples come from: hashed draws from the training set
// (mode 0), the set's samples base.. in order (mode 1), or rotations
// rot[base..] of one ligand (mode 2, prediction)
struct SampleSrc {
    int mode;
    const int* lig;        // [n] (modes 0, 1)
    const double* rot;     // [n][9]
    int n;
    int base;
    int fixed_lig;         // mode 2
    const uint32_t* step;  // mode 0
    uint64_t seed;         // mode 0
};

// occupancy counts of the rotated ligand; p' = R p with the scan's operation
// order (((r0 x0) + r1 x1) + r2 x2, no contraction), cell = floor((p' + L) /
// (2L/16)) clamped to the cube
__device__ void occupancy(const double* __restrict__ xyz, int n, double L, const double* __restrict__ rot,
                          float* __restrict__ occ) {
    for (int i = threadIdx.x; i < NX0; i += THREADS) occ[i] = 0.f;
    __syncthreads();
    const double cs = (2.0 * L) / (double)G0;
    for (int a = threadIdx.x; a < n; a += THREADS) {
        const double p0 = xyz[3 * a], p1 = xyz[3 * a + 1], p2 = xyz[3 * a + 2];
        int c[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double q = __dadd_rn(__dadd_rn(__dmul_rn(rot[3 * d], p0), __dmul_rn(rot[3 * d + 1], p1)),
                                       __dmul_rn(rot[3 * d + 2], p2));
            int k = (int)floor(__ddiv_rn(__dadd_rn(q, L), cs));
            c[d] = k < 0 ? 0 : (k > G0 - 1 ? G0 - 1 : k);
        }
        atomicAdd(&occ[(c[0] * G0 + c[1]) * G0 + c[2]], 1.0f);
    }
    __syncthreads();
}

// input position of output position (oz, oy, ox) under tap t of a stride-2,
// pad-1 3^3 convolution over a din^3 grid; -1 outside
__device__ __forceinline__ int tap_source(int din, int oz, int oy, int ox, int t) {
    const int z = 2 * oz - 1 + t / 9, y = 2 * oy - 1 + (t / 3) % 3, x = 2 * ox - 1 + t % 3;
    if (z < 0 || z >= din || y < 0 || y >= din || x < 0 || x >= din) return -1;
    return (z * din + y) * din + x;
}

// one CTA per sample: occupancy -> x0 (BF16) -> conv1's im2col rows
// x1c[s * P1 + pos][tap]: column 27 is 1 (its weight is zero, and the
// weight-gradient GEMM gets the bias gradient there), 28..31 zero; the
// descriptor -> u[s][NA3..]
__global__ void __launch_bounds__(THREADS) prep_kernel(Ligands lg, SampleSrc src, bf16* __restrict__ x1c,
                                                       bf16* __restrict__ u, int* __restrict__ sidx) {
    __shared__ float occ[NX0];
    __shared__ bf16 x0[NX0];
    const int b = blockIdx.x;
    int idx, lig;
    const double* rot;
    if (src.mode == 2) {
        idx = src.base + b;
        lig = src.fixed_lig;
        rot = src.rot + 9 * (size_t)idx;
    } else {
        if (src.mode == 1) {
            idx = src.base + b;
        } else {
            const uint64_t h = mix64(src.seed ^ mix64(((uint64_t)(*src.step) << 20) ^ (uint64_t)b));
            idx = (int)(h % (uint64_t)src.n);
        }
        lig = src.lig[idx];
        rot = src.rot + 9 * (size_t)idx;
    }
    if (threadIdx.x == 0 && sidx) sidx[b] = idx;
    occupancy(lg.xyz + 3 * (size_t)lg.start[lig], lg.count[lig], lg.half[lig], rot, occ);
    for (int i = threadIdx.x; i < NX0; i += THREADS) x0[i] = f2b(0.25f * occ[i]);
    for (int i = threadIdx.x; i < DESC; i += THREADS) u[(size_t)b * NU + NA3 + i] = f2b(lg.desc[(size_t)lig * DESC + i]);
    __syncthreads();
    // rows of 32 taps as 4 groups of 8
    for (int e = threadIdx.x; e < P1 * 4; e += THREADS) {
        const int pos = e >> 2, t0 = (e & 3) * 8;
        const int oz = pos / (D1 * D1), oy = (pos / D1) % D1, ox = pos % D1;
        uint32_t q[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int t = t0 + i;
            const int src_i = t < 27 ? tap_source(G0, oz, oy, ox, t) : -1;
            const uint32_t h = t == 27 ? (uint32_t)__bfloat16_as_ushort(f2b(1.f))
                                       : (src_i >= 0 ? (uint32_t)__bfloat16_as_ushort(x0[src_i]) : 0u);
            q[i >> 1] |= h << (16 * (i & 1));
        }
        *reinterpret_cast<uint4*>(x1c + ((size_t)b * P1 + pos) * K1 + t0) = make_uint4(q[0], q[1], q[2], q[3]);
    }
}

// im2col of a channel-last activation act[s * PIN + pos_in][CIN] into
// col[s * POUT + pos][tap * CIN + ci]; one thread per (row, tap)
template <int CIN, int DIN>
__global__ void im2col_kernel(const bf16* __restrict__ act, bf16* __restrict__ col, int n_samples) {
    constexpr int DOUT = DIN / 2, POUT = DOUT * DOUT * DOUT, PIN = DIN * DIN * DIN;
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n_samples * POUT * 27) return;
    const int t = (int)(e % 27);
    const size_t row = e / 27;
    const int s = (int)(row / POUT), pos = (int)(row % POUT);
    const int src_i = tap_source(DIN, pos / (DOUT * DOUT), (pos / DOUT) % DOUT, pos % DOUT, t);
    uint4* dst = reinterpret_cast<uint4*>(col + row * (27 * CIN) + t * CIN);
    const uint4* sp = reinterpret_cast<const uint4*>(act + ((size_t)s * PIN + (src_i < 0 ? 0 : src_i)) * CIN);
#pragma unroll
    for (int i = 0; i < CIN / 8; ++i) dst[i] = src_i >= 0 ? sp[i] : make_uint4(0u, 0u, 0u, 0u);
}

// col2im: the input gradient of a convolution from the gradient of its
// im2col matrix dcol[s * POUT + pos][tap * CIN + ci] (FP32), summed over the
// taps in order, masked by act > 0 (the ReLU of the layer below), BF16
template <int CIN, int DIN>
__global__ void col2im_kernel(const float* __restrict__ dcol, const bf16* __restrict__ act, bf16* __restrict__ dz,
                             int n_samples) {
    constexpr int DOUT = DIN / 2, POUT = DOUT * DOUT * DOUT, PIN = DIN * DIN * DIN;
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)n_samples * PIN * CIN) return;
    const int ci = (int)(e % CIN);
    const size_t row = e / CIN;
    const int s = (int)(row / PIN), p = (int)(row % PIN);
    const int z = p / (DIN * DIN), y = (p / DIN) % DIN, x = p % DIN;
    float acc = 0.f;
    if (b2f(act[e]) > 0.f) {
        for (int t = 0; t < 27; ++t) {
            const int tz = z + 1 - t / 9, ty = y + 1 - (t / 3) % 3, tx = x + 1 - t % 3;
            if (tz < 0 || ty < 0 || tx < 0 || (tz & 1) || (ty & 1) || (tx & 1)) continue;
            if ((tz >> 1) >= DOUT || (ty >> 1) >= DOUT || (tx >> 1) >= DOUT) continue;
            const int pos = ((tz >> 1) * DOUT + (ty >> 1)) * DOUT + (tx >> 1);
            acc += dcol[((size_t)s * POUT + pos) * (27 * CIN) + t * CIN + ci];
        }
    }
    dz[e] = f2b(acc);
}

// column sums out[c] = sum_r in[r * ld + c] (BF16 in, FP32 out) in a fixed
// order: block (x, y) sums rows [y * chunk, (y + 1) * chunk) of columns
// 32 x .. 32 x + 31 (lane = column, warps stride the rows) into
// part[y][c]; colsum_final_kernel adds the parts in order
__global__ void __launch_bounds__(THREADS) colsum_kernel(const bf16* __restrict__ in, int rows, int cols, int ld,
                                                         int chunk, float* __restrict__ part) {
    __shared__ float red[THREADS / 32][32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const int c = blockIdx.x * 32 + l;
    const int r0 = blockIdx.y * chunk, r1 = min(rows, r0 + chunk);
    float acc = 0.f;
    if (c < cols)
        for (int r = r0 + w; r < r1; r += THREADS / 32) acc += b2f(in[(size_t)r * ld + c]);
    red[w][l] = acc;
    __syncthreads();
    if (w == 0 && c < cols) {
        float v = 0.f;
        for (int k = 0; k < THREADS / 32; ++k) v += red[k][l];
        part[(size_t)blockIdx.y * cols + c] = v;
    }
}

__global__ void colsum_final_kernel(const float* __restrict__ part, int parts, int cols, float* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float v = 0.f;
    for (int k = 0; k < parts; ++k) v += part[(size_t)k * cols + c];
    out[c] = v;
}

// head: y = w2 . h1 + b2 (one warp per sample).  Training (target != null):
// loss, dy = 2 (y - t) / B and dzf = (h1 > 0) dy w2 (BF16)
__global__ void __launch_bounds__(THREADS) head_kernel(const bf16* __restrict__ wb, const bf16* __restrict__ h1, int n,
                                                       float* __restrict__ y_out, const float* __restrict__ target,
                                                       const int* __restrict__ sidx, int batch, float* __restrict__ dy,
                                                       bf16* __restrict__ dzf, double* __restrict__ loss_acc) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    const int s = blockIdx.x * (THREADS / 32) + w;
    if (s >= n) return;
    float acc = 0.f;
    for (int j = l; j < HID; j += 32) acc += b2f(wb[OF2 + j]) * b2f(h1[(size_t)s * HID + j]);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    const float y = b2f(wb[OFB2]) + acc;
    if (y_out && l == 0) y_out[s] = y;
    if (!target) return;
    const float t = target[sidx[s]];
    const float d = 2.f * (y - t) / (float)batch;
    if (l == 0) {
        dy[s] = d;
        atomicAdd(loss_acc, (double)((y - t) * (y - t)) / (double)batch);
    }
    for (int j = l; j < HID; j += 32)
        dzf[(size_t)s * HID + j] = f2b(b2f(h1[(size_t)s * HID + j]) > 0.f ? d * b2f(wb[OF2 + j]) : 0.f);
}

// dw2[j] = sum_s dy[s] h1[s][j], db2 = sum_s dy[s]
__global__ void __launch_bounds__(THREADS) fc2_wgrad_kernel(const bf16* __restrict__ h1, const float* __restrict__ dy,
                                                            int B, float* __restrict__ g) {
    const int j = threadIdx.x;
    float acc = 0.f;
    for (int s = 0; s < B; ++s) acc += b2f(h1[(size_t)s * HID + j]) * dy[s];
    g[OF2 + j] = acc;
    if (j == 0) {
        float d = 0.f;
        for (int s = 0; s < B; ++s) d += dy[s];
        g[OFB2] = d;
    }
}

// BF16 copies of master weight i: the master layout, and the permuted
// convolution weights
__device__ __forceinline__ void store_copies(int i, float w, bf16* __restrict__ wb, bf16* __restrict__ wp) {
    const bf16 v = f2b(w);
    wb[i] = v;
    if (i >= OW1 && i < OB1) {
        const int j = i - OW1;
        wp[OP1 + (j / 27) * K1 + j % 27] = v;
    } else if (i >= OW2 && i < OB2) {
        const int j = i - OW2, co = j / (C1 * 27), ci = (j / 27) % C1, t = j % 27;
        wp[OP2 + co * K2 + t * C1 + ci] = v;
    } else if (i >= OW3 && i < OB3) {
        const int j = i - OW3, co = j / (C2 * 27), ci = (j / 27) % C2, t = j % 27;
        wp[OP3 + co * K3 + t * C2 + ci] = v;
    }
}

// Adam on the FP32 masters (bias-corrected), BF16 copies refreshed
__global__ void adam_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, bf16* __restrict__ wb, bf16* __restrict__ wp,
                            const uint32_t* __restrict__ step_ctr, float lr, float b1, float b2, float eps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t t = *step_ctr + 1u;
    if (i < NPARAM) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float mh = mi / (1.f - powf(b1, (float)t));
        const float vh = vi / (1.f - powf(b2, (float)t));
        const float wi = w[i] - lr * mh / (sqrtf(vh) + eps);
        w[i] = wi;
        store_copies(i, wi, wb, wp);
    }
}

__global__ void step_advance_kernel(uint32_t* step_ctr) { *step_ctr += 1u; }

__global__ void to_bf16_kernel(const float* __restrict__ w, bf16* __restrict__ wb, bf16* __restrict__ wp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < NPARAM) store_copies(i, w[i], wb, wp);
}

template <typename T> cudaError_t dalloc(T** p, size_t n) {
    *p = nullptr;
    return cudaMalloc((void**)p, (n ? n : 1) * sizeof(T));
}
template <typename T> void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// work buffers of a batch of up to cap samples
struct Work {
    int cap = 0;
    bool grads = false;  // the backward buffers are allocated
    bf16* x1c = nullptr;  // [cap * P1][K1]
    bf16* a1 = nullptr;   // [cap * P1][C1]
    bf16* x2c = nullptr;  // [cap * P2][K2]
    bf16* a2 = nullptr;   // [cap * P2][C2]
    bf16* x3c = nullptr;  // [cap * P3][K3]
    bf16* u = nullptr;    // [cap][NU]
    bf16* h1 = nullptr;   // [cap][HID]
    int* sidx = nullptr;  // [cap] sample index of each slot
    float* y = nullptr;   // [cap]
    // backward
    float* dy = nullptr;    // [cap]
    bf16* dzf = nullptr;    // [cap][HID]
    bf16* dz3 = nullptr;    // [cap * P3][C3]
    float* dx3 = nullptr;   // [cap * P3][K3]
    bf16* dz2 = nullptr;    // [cap * P2][C2]
    float* dx2 = nullptr;   // [cap * P2][K2]
    bf16* dz1 = nullptr;    // [cap * P1][C1]
    float* ws = nullptr;    // [WS_FLOATS] split-K partial sums
    float* cs = nullptr;    // [kColsumParts][HID] column-sum parts
    void release() {
        dfree(x1c);
        dfree(a1);
        dfree(x2c);
        dfree(a2);
        dfree(x3c);
        dfree(u);
        dfree(h1);
        dfree(sidx);
        dfree(y);
        dfree(dy);
        dfree(dzf);
        dfree(dz3);
        dfree(dx3);
        dfree(dz2);
        dfree(dx2);
        dfree(dz1);
        dfree(ws);
        dfree(cs);
        cap = 0;
        grads = false;
    }
};

}  // namespace

struct fftdock_proposal {
    int device = 0;
    std::string err;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    // parameters
    float* w = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* g = nullptr;
    bf16* wb = nullptr;
    bf16* wp = nullptr;  // permuted convolution weights
    uint32_t* step = nullptr;
    double* loss = nullptr;
    // ligands (device copies grow by reallocation)
    std::vector<double> h_xyz;
    std::vector<int> h_start, h_count;
    std::vector<double> h_half;
    std::vector<float> h_desc;
    double* xyz = nullptr;
    int* start = nullptr;
    int* count = nullptr;
    double* half = nullptr;
    float* desc = nullptr;
    bool lig_dirty = false;
    // samples
    std::vector<int> h_lig;
    std::vector<double> h_rot;
    std::vector<float> h_target;
    int* s_lig = nullptr;
    double* s_rot = nullptr;
    float* s_target = nullptr;
    int n_dev_samples = 0;
    bool samples_dirty = false;
    // batch work
    Work wk;
    // captured training step
    cudaGraphExec_t graph = nullptr;
    int graph_batch = 0;
    float graph_lr = 0.f;
    uint64_t graph_seed = 0;
};

namespace {

int pfail(fftdock_proposal* p, int code, const std::string& msg) {
    if (p) p->err = msg;
    return code;
}

#define PK(expr)                                                                             \
    do {                                                                                     \
        cudaError_t e_ = (expr);                                                             \
        if (e_ != cudaSuccess) return pfail(p, FFTDOCK_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

Ligands ligands(const fftdock_proposal* p) { return Ligands{p->xyz, p->start, p->count, p->half, p->desc}; }

void drop_graph(fftdock_proposal* p) {
    if (p->graph) {
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
}

int sync_ligands(fftdock_proposal* p) {
    if (!p->lig_dirty) return FFTDOCK_OK;
    PK(cudaStreamSynchronize(p->stream));
    dfree(p->xyz);
    dfree(p->start);
    dfree(p->count);
    dfree(p->half);
    dfree(p->desc);
    PK(dalloc(&p->xyz, p->h_xyz.size()));
    PK(dalloc(&p->start, p->h_start.size()));
    PK(dalloc(&p->count, p->h_count.size()));
    PK(dalloc(&p->half, p->h_half.size()));
    PK(dalloc(&p->desc, p->h_desc.size()));
    PK(cudaMemcpy(p->xyz, p->h_xyz.data(), p->h_xyz.size() * sizeof(double), cudaMemcpyHostToDevice));
    PK(cudaMemcpy(p->start, p->h_start.data(), p->h_start.size() * sizeof(int), cudaMemcpyHostToDevice));
    PK(cudaMemcpy(p->count, p->h_count.data(), p->h_count.size() * sizeof(int), cudaMemcpyHostToDevice));
    PK(cudaMemcpy(p->half, p->h_half.data(), p->h_half.size() * sizeof(double), cudaMemcpyHostToDevice));
    PK(cudaMemcpy(p->desc, p->h_desc.data(), p->h_desc.size() * sizeof(float), cudaMemcpyHostToDevice));
    p->lig_dirty = false;
    drop_graph(p);
    return FFTDOCK_OK;
}

int sync_samples(fftdock_proposal* p) {
    if (!p->samples_dirty) return FFTDOCK_OK;
    PK(cudaStreamSynchronize(p->stream));
    dfree(p->s_lig);
    dfree(p->s_rot);
    dfree(p->s_target);
    PK(dalloc(&p->s_lig, p->h_lig.size()));
    PK(dalloc(&p->s_rot, p->h_rot.size()));
    PK(dalloc(&p->s_target, p->h_target.size()));
    PK(cudaMemcpy(p->s_lig, p->h_lig.data(), p->h_lig.size() * sizeof(int), cudaMemcpyHostToDevice));
    PK(cudaMemcpy(p->s_rot, p->h_rot.data(), p->h_rot.size() * sizeof(double), cudaMemcpyHostToDevice));
    PK(cudaMemcpy(p->s_target, p->h_target.data(), p->h_target.size() * sizeof(float), cudaMemcpyHostToDevice));
    p->n_dev_samples = (int)p->h_lig.size();
    p->samples_dirty = false;
    drop_graph(p);
    return FFTDOCK_OK;
}

// work buffers for cap samples (backward buffers when grads)
int grow_work(fftdock_proposal* p, int cap, bool grads) {
    Work& w = p->wk;
    if (cap <= w.cap && (!grads || w.grads)) return FFTDOCK_OK;
    PK(cudaStreamSynchronize(p->stream));
    const int c = std::max(cap, w.cap);
    const bool gr = grads || w.grads;
    w.release();
    drop_graph(p);
    PK(dalloc(&w.x1c, (size_t)c * P1 * K1));
    PK(dalloc(&w.a1, (size_t)c * P1 * C1));
    PK(dalloc(&w.x2c, (size_t)c * P2 * K2));
    PK(dalloc(&w.a2, (size_t)c * P2 * C2));
    PK(dalloc(&w.x3c, (size_t)c * P3 * K3));
    PK(dalloc(&w.u, (size_t)c * NU));
    PK(dalloc(&w.h1, (size_t)c * HID));
    PK(dalloc(&w.sidx, (size_t)c));
    PK(dalloc(&w.y, (size_t)c));
    if (gr) {
        PK(dalloc(&w.dy, (size_t)c));
        PK(dalloc(&w.dzf, (size_t)c * HID));
        PK(dalloc(&w.dz3, (size_t)c * P3 * C3));
        PK(dalloc(&w.dx3, (size_t)c * P3 * K3));
        PK(dalloc(&w.dz2, (size_t)c * P2 * C2));
        PK(dalloc(&w.dx2, (size_t)c * P2 * K2));
        PK(dalloc(&w.dz1, (size_t)c * P1 * C1));
        PK(dalloc(&w.ws, (size_t)WS_FLOATS));
        PK(dalloc(&w.cs, (size_t)kColsumParts * HID));
    }
    w.cap = c;
    w.grads = gr;
    return FFTDOCK_OK;
}

// C = A x B through gemm_kernel, K split into `splits` parts (partial sums
// reduced in split order into the epilogue)
template <bool AT, bool BT, class Epi>
cudaError_t gemm(int M, int N, int K, const bf16* A, int lda, const bf16* B, int ldb, Epi epi, int splits, float* ws,
                 cudaStream_t s) {
    // the partial sums fit the workspace
    splits = std::max(1, std::min(splits, (int)((size_t)WS_FLOATS / ((size_t)M * N))));
    const int kc = ((K + splits * GBK - 1) / (splits * GBK)) * GBK;
    splits = (K + kc - 1) / kc;
    dim3 grid((N + GBN - 1) / GBN, (M + GBM - 1) / GBM, splits);
    if (splits == 1) {
        gemm_kernel<AT, BT, Epi><<<grid, GTHREADS, 0, s>>>(M, N, K, A, lda, B, ldb, kc, epi);
        return cudaGetLastError();
    }
    gemm_kernel<AT, BT, EpiPartial><<<grid, GTHREADS, 0, s>>>(M, N, K, A, lda, B, ldb, kc, EpiPartial{ws, M, N});
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    splitk_reduce_kernel<Epi><<<(M * N + 255) / 256, 256, 0, s>>>(ws, splits, M, N, epi);
    return cudaGetLastError();
}

// forward of n samples (n <= work capacity): u, h1 and y in the work buffers
cudaError_t launch_forward(fftdock_proposal* p, int n, const SampleSrc& src, cudaStream_t s) {
    Work& w = p->wk;
    cudaError_t e;
    prep_kernel<<<n, THREADS, 0, s>>>(ligands(p), src, w.x1c, w.u, w.sidx);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = gemm<false, true>(n * P1, C1, K1, w.x1c, K1, p->wp + OP1, K1, EpiBiasRelu{w.a1, C1, p->wb + OB1}, 1,
                               nullptr, s)) != cudaSuccess)
        return e;
    const size_t c2 = (size_t)n * P2 * 27, c3 = (size_t)n * P3 * 27;
    im2col_kernel<C1, D1><<<(unsigned)((c2 + 255) / 256), 256, 0, s>>>(w.a1, w.x2c, n);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = gemm<false, true>(n * P2, C2, K2, w.x2c, K2, p->wp + OP2, K2, EpiBiasRelu{w.a2, C2, p->wb + OB2}, 1,
                               nullptr, s)) != cudaSuccess)
        return e;
    im2col_kernel<C2, D2><<<(unsigned)((c3 + 255) / 256), 256, 0, s>>>(w.a2, w.x3c, n);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = gemm<false, true>(n * P3, C3, K3, w.x3c, K3, p->wp + OP3, K3, EpiConv3{w.u, p->wb + OB3}, 1, nullptr,
                               s)) != cudaSuccess)
        return e;
    return gemm<false, false>(n, HID, NU, w.u, NU, p->wb + OF1, HID, EpiBiasRelu{w.h1, HID, p->wb + OFB1}, 1, nullptr,
                              s);
}

// K split of a weight gradient over rows samples x positions
int wgrad_splits(int rows) { return std::max(1, std::min(256, rows / 1024)); }

// bias gradient: column sums of a BF16 activation gradient [rows][cols]
cudaError_t colsum(const bf16* in, int rows, int cols, float* part, float* out, cudaStream_t s) {
    const int parts = std::max(1, std::min(kColsumParts, rows / 256));
    const int chunk = (rows + parts - 1) / parts;
    colsum_kernel<<<dim3((cols + 31) / 32, parts), THREADS, 0, s>>>(in, rows, cols, cols, chunk, part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    colsum_final_kernel<<<(cols + 255) / 256, 256, 0, s>>>(part, parts, cols, out);
    return cudaGetLastError();
}

// the batch's forward, loss, backward and weight gradients into p->g (no update)
cudaError_t launch_gradients(fftdock_proposal* p, int B, const SampleSrc& src, const float* target, cudaStream_t s) {
    Work& w = p->wk;
    cudaError_t e = launch_forward(p, B, src, s);
    if (e != cudaSuccess) return e;
    float* g = p->g;
    head_kernel<<<(B + 7) / 8, THREADS, 0, s>>>(p->wb, w.h1, B, w.y, target, w.sidx, B, w.dy, w.dzf, p->loss);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    fc2_wgrad_kernel<<<1, THREADS, 0, s>>>(w.h1, w.dy, B, g);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // fc1: dW1 = u^T dzf, db1 = column sums of dzf, du -> dz3 (masked by a3 > 0)
    if ((e = gemm<true, false>(NU, HID, B, w.u, NU, w.dzf, HID, EpiF32{g + OF1, HID}, 1, nullptr, s)) != cudaSuccess)
        return e;
    if ((e = colsum(w.dzf, B, HID, w.cs, g + OFB1, s)) != cudaSuccess) return e;
    if ((e = gemm<false, true>(B, NA3, HID, w.dzf, HID, p->wb + OF1, HID, EpiDz3{w.dz3, w.u}, 1, nullptr, s)) !=
        cudaSuccess)
        return e;
    // conv3
    const int r3 = B * P3, r2 = B * P2, r1 = B * P1;
    if ((e = gemm<true, false>(C3, K3, r3, w.dz3, C3, w.x3c, K3, EpiWgrad{g + OW3, C2, nullptr}, wgrad_splits(r3),
                               w.ws, s)) != cudaSuccess)
        return e;
    if ((e = colsum(w.dz3, r3, C3, w.cs, g + OB3, s)) != cudaSuccess) return e;
    if ((e = gemm<false, false>(r3, K3, C3, w.dz3, C3, p->wp + OP3, K3, EpiF32{w.dx3, K3}, 1, nullptr, s)) !=
        cudaSuccess)
        return e;
    const size_t e2 = (size_t)B * P2 * C2, e1 = (size_t)B * P1 * C1;
    col2im_kernel<C2, D2><<<(unsigned)((e2 + 255) / 256), 256, 0, s>>>(w.dx3, w.a2, w.dz2, B);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // conv2
    if ((e = gemm<true, false>(C2, K2, r2, w.dz2, C2, w.x2c, K2, EpiWgrad{g + OW2, C1, nullptr}, wgrad_splits(r2),
                               w.ws, s)) != cudaSuccess)
        return e;
    if ((e = colsum(w.dz2, r2, C2, w.cs, g + OB2, s)) != cudaSuccess) return e;
    if ((e = gemm<false, false>(r2, K2, C2, w.dz2, C2, p->wp + OP2, K2, EpiF32{w.dx2, K2}, 1, nullptr, s)) !=
        cudaSuccess)
        return e;
    col2im_kernel<C1, D1><<<(unsigned)((e1 + 255) / 256), 256, 0, s>>>(w.dx2, w.a1, w.dz1, B);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // conv1 (the input needs no gradient; the bias gradient is column 27)
    return gemm<true, false>(C1, K1, r1, w.dz1, C1, w.x1c, K1, EpiWgrad{g + OW1, 1, g + OB1}, wgrad_splits(r1), w.ws,
                             s);
}

}  // namespace

extern "C" {

int32_t fftdock_proposal_n_params(void) { return NPARAM; }

const char* fftdock_proposal_last_error(const fftdock_proposal* p) { return p ? p->err.c_str() : "null proposal"; }

int fftdock_proposal_create(int32_t device, uint64_t seed, fftdock_proposal** out) {
    if (!out) return FFTDOCK_EINVAL;
    *out = nullptr;
    fftdock_proposal* p = new (std::nothrow) fftdock_proposal();
    if (!p) return FFTDOCK_ENOMEM;
    *out = p;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return pfail(p, FFTDOCK_ECUDA, "no CUDA device");
    if (device < 0 || device >= ndev) return pfail(p, FFTDOCK_EINVAL, "device ordinal out of range");
    p->device = device;
    fftdock::DeviceScope dev_scope(device);
    PK(dev_scope.status());
    cudaDeviceProp prop;
    PK(cudaGetDeviceProperties(&prop, device));
    if (prop.major != 10 || prop.minor != 3)
        return pfail(p, FFTDOCK_EUNSUPPORTED, std::string("built for sm_103a only; device is ") + prop.name);
    PK(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    PK(cudaEventCreateWithFlags(&p->ev, cudaEventDisableTiming));
    PK(dalloc(&p->w, NPARAM));
    PK(dalloc(&p->m, NPARAM));
    PK(dalloc(&p->v, NPARAM));
    PK(dalloc(&p->g, NPARAM));
    PK(dalloc(&p->wb, NPARAM));
    PK(dalloc(&p->wp, NPERM));
    PK(cudaMemset(p->wp, 0, NPERM * sizeof(bf16)));  // conv1's padding taps stay zero
    PK(dalloc(&p->step, 1));
    PK(dalloc(&p->loss, 1));
    // He-normal initial weights, zero biases
    std::vector<float> w(NPARAM, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int n, int fan_in) {
        std::normal_distribution<double> nd(0.0, std::sqrt(2.0 / (double)fan_in));
        for (int i = 0; i < n; ++i) w[off + i] = (float)nd(rng);
    };
    fill(OW1, C1 * 27, 27);
    fill(OW2, C2 * C1 * 27, C1 * 27);
    fill(OW3, C3 * C2 * 27, C2 * 27);
    fill(OF1, NU * HID, NU);
    fill(OF2, HID, HID);
    PK(cudaMemcpy(p->w, w.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    PK(cudaMemset(p->m, 0, NPARAM * sizeof(float)));
    PK(cudaMemset(p->v, 0, NPARAM * sizeof(float)));
    PK(cudaMemset(p->step, 0, sizeof(uint32_t)));
    to_bf16_kernel<<<(NPARAM + 255) / 256, 256, 0, p->stream>>>(p->w, p->wb, p->wp);
    PK(cudaGetLastError());
    PK(cudaStreamSynchronize(p->stream));
    return FFTDOCK_OK;
}

void fftdock_proposal_destroy(fftdock_proposal* p) {
    if (!p) return;
    if (p->stream) cudaStreamSynchronize(p->stream);
    if (p->graph) cudaGraphExecDestroy(p->graph);
    dfree(p->w);
    dfree(p->m);
    dfree(p->v);
    dfree(p->g);
    dfree(p->wb);
    dfree(p->wp);
    dfree(p->step);
    dfree(p->loss);
    dfree(p->xyz);
    dfree(p->start);
    dfree(p->count);
    dfree(p->half);
    dfree(p->desc);
    dfree(p->s_lig);
    dfree(p->s_rot);
    dfree(p->s_target);
    p->wk.release();
    if (p->ev) cudaEventDestroy(p->ev);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

int fftdock_proposal_get_params(fftdock_proposal* p, float* out) {
    if (!p || !out) return FFTDOCK_EINVAL;
    fftdock::DeviceScope dev_scope(p->device);
    PK(dev_scope.status());
    PK(cudaStreamSynchronize(p->stream));
    PK(cudaMemcpy(out, p->w, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return FFTDOCK_OK;
}

int fftdock_proposal_set_params(fftdock_proposal* p, const float* in) {
    if (!p || !in) return FFTDOCK_EINVAL;
    for (int i = 0; i < NPARAM; ++i)
        if (!std::isfinite(in[i])) return pfail(p, FFTDOCK_EINVAL, "non-finite parameter");
    fftdock::DeviceScope dev_scope(p->device);
    PK(dev_scope.status());
    PK(cudaStreamSynchronize(p->stream));
    PK(cudaMemcpy(p->w, in, NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    PK(cudaMemset(p->m, 0, NPARAM * sizeof(float)));
    PK(cudaMemset(p->v, 0, NPARAM * sizeof(float)));
    PK(cudaMemset(p->step, 0, sizeof(uint32_t)));
    to_bf16_kernel<<<(NPARAM + 255) / 256, 256, 0, p->stream>>>(p->w, p->wb, p->wp);
    PK(cudaGetLastError());
    PK(cudaStreamSynchronize(p->stream));
    return FFTDOCK_OK;
}

int fftdock_proposal_add_ligand(fftdock_proposal* p, int32_t n, const double* xyz, const float* rec_desc,
                                int32_t* id) {
    if (!p || n < 1 || !xyz || !rec_desc || !id) return pfail(p, FFTDOCK_EINVAL, "bad arguments");
    double L = 0.0;
    for (int i = 0; i < n; ++i) {
        const double a = xyz[3 * i], b = xyz[3 * i + 1], c = xyz[3 * i + 2];
        if (!std::isfinite(a) || !std::isfinite(b) || !std::isfinite(c))
            return pfail(p, FFTDOCK_EINVAL, "non-finite ligand coordinate");
        L = std::max(L, std::sqrt(a * a + b * b + c * c));
    }
    for (int i = 0; i < DESC; ++i)
        if (!std::isfinite(rec_desc[i])) return pfail(p, FFTDOCK_EINVAL, "non-finite descriptor");
    if (!(L > 0.0)) L = 1.0;
    *id = (int32_t)p->h_start.size();
    p->h_start.push_back((int)(p->h_xyz.size() / 3));
    p->h_count.push_back(n);
    p->h_half.push_back(L);
    p->h_xyz.insert(p->h_xyz.end(), xyz, xyz + 3 * (size_t)n);
    p->h_desc.insert(p->h_desc.end(), rec_desc, rec_desc + DESC);
    p->lig_dirty = true;
    return FFTDOCK_OK;
}

int fftdock_proposal_add_samples(fftdock_proposal* p, int32_t lig, int32_t n, const double* rot, const float* target) {
    if (!p || n < 0 || (n > 0 && (!rot || !target))) return pfail(p, FFTDOCK_EINVAL, "bad arguments");
    if (lig < 0 || lig >= (int32_t)p->h_start.size()) return pfail(p, FFTDOCK_EINVAL, "unknown ligand id");
    for (int i = 0; i < n; ++i)
        if (!std::isfinite(target[i])) return pfail(p, FFTDOCK_EINVAL, "non-finite target");
    p->h_lig.insert(p->h_lig.end(), (size_t)n, lig);
    p->h_rot.insert(p->h_rot.end(), rot, rot + 9 * (size_t)n);
    p->h_target.insert(p->h_target.end(), target, target + n);
    p->samples_dirty = true;
    return FFTDOCK_OK;
}

int fftdock_proposal_clear_samples(fftdock_proposal* p) {
    if (!p) return FFTDOCK_EINVAL;
    p->h_lig.clear();
    p->h_rot.clear();
    p->h_target.clear();
    p->samples_dirty = true;
    return FFTDOCK_OK;
}

int fftdock_proposal_train(fftdock_proposal* p, int32_t steps, int32_t batch, float lr, uint64_t seed,
                           float* mean_loss) {
    if (!p || steps < 0 || batch < 1 || batch > MAX_BATCH || !(lr > 0.f))
        return pfail(p, FFTDOCK_EINVAL, "bad arguments");
    fftdock::DeviceScope dev_scope(p->device);
    PK(dev_scope.status());
    int rc;
    if ((rc = sync_ligands(p)) || (rc = sync_samples(p)) || (rc = grow_work(p, batch, true))) return rc;
    if (p->n_dev_samples < 1) return pfail(p, FFTDOCK_ESTATE, "no training samples");
    if (p->graph && (p->graph_batch != batch || p->graph_lr != lr || p->graph_seed != seed)) {
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
    cudaStream_t s = p->stream;
    if (!p->graph) {
        SampleSrc src{0, p->s_lig, p->s_rot, p->n_dev_samples, 0, 0, p->step, seed};
        cudaGraph_t g = nullptr;
        PK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = launch_gradients(p, batch, src, p->s_target, s);
        if (e == cudaSuccess) {
            adam_kernel<<<(NPARAM + 255) / 256, 256, 0, s>>>(p->w, p->m, p->v, p->g, p->wb, p->wp, p->step, lr, 0.9f,
                                                             0.999f, 1e-8f);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            step_advance_kernel<<<1, 1, 0, s>>>(p->step);
            e = cudaGetLastError();
        }
        cudaError_t e2 = cudaStreamEndCapture(s, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return pfail(p, FFTDOCK_ECUDA, std::string("capture of the training step: ") +
                                               cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        e = cudaGraphInstantiate(&p->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return pfail(p, FFTDOCK_ECUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        p->graph_batch = batch;
        p->graph_lr = lr;
        p->graph_seed = seed;
    }
    PK(cudaMemsetAsync(p->loss, 0, sizeof(double), s));
    for (int i = 0; i < steps; ++i) PK(cudaGraphLaunch(p->graph, s));
    double loss = 0.0;
    PK(cudaMemcpyAsync(&loss, p->loss, sizeof(double), cudaMemcpyDeviceToHost, s));
    PK(cudaStreamSynchronize(s));
    if (mean_loss) *mean_loss = steps > 0 ? (float)(loss / steps) : 0.f;
    return FFTDOCK_OK;
}

int fftdock_proposal_gradients(fftdock_proposal* p, int32_t n, const int32_t* lig, const double* rot,
                               const float* target, float* grads, float* loss) {
    if (!p || n < 1 || n > MAX_BATCH || !lig || !rot || !target || !grads)
        return pfail(p, FFTDOCK_EINVAL, "bad arguments");
    for (int i = 0; i < n; ++i)
        if (lig[i] < 0 || lig[i] >= (int32_t)p->h_start.size()) return pfail(p, FFTDOCK_EINVAL, "unknown ligand id");
    fftdock::DeviceScope dev_scope(p->device);
    PK(dev_scope.status());
    int rc;
    if ((rc = sync_ligands(p)) || (rc = grow_work(p, n, true))) return rc;
    cudaStream_t s = p->stream;
    int* d_lig = nullptr;
    double* d_rot = nullptr;
    float* d_t = nullptr;
    PK(dalloc(&d_lig, n));
    cudaError_t e = dalloc(&d_rot, 9 * (size_t)n);
    if (e == cudaSuccess) e = dalloc(&d_t, n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_lig, lig, n * sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rot, rot, 9 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_t, target, n * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->loss, 0, sizeof(double), s);
    if (e == cudaSuccess) e = launch_gradients(p, n, SampleSrc{1, d_lig, d_rot, n, 0, 0, nullptr, 0}, d_t, s);
    double l = 0.0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(grads, p->g, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&l, p->loss, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(d_lig);
    cudaFree(d_rot);
    cudaFree(d_t);
    if (e != cudaSuccess) return pfail(p, FFTDOCK_ECUDA, std::string("gradients: ") + cudaGetErrorString(e));
    if (e2 != cudaSuccess) return pfail(p, FFTDOCK_ECUDA, std::string("gradients: ") + cudaGetErrorString(e2));
    if (loss) *loss = (float)l;
    return FFTDOCK_OK;
}

int fftdock_proposal_predict_device(fftdock_proposal* p, int32_t lig, int32_t n, const double* d_rot, float* d_out,
                                    void* stream) {
    if (!p || n < 0 || (n > 0 && (!d_rot || !d_out))) return pfail(p, FFTDOCK_EINVAL, "bad arguments");
    if (lig < 0 || lig >= (int32_t)p->h_start.size()) return pfail(p, FFTDOCK_EINVAL, "unknown ligand id");
    if (n == 0) return FFTDOCK_OK;
    fftdock::DeviceScope dev_scope(p->device);
    PK(dev_scope.status());
    int rc;
    if ((rc = sync_ligands(p))) return rc;
    if ((rc = grow_work(p, std::min(n, PREDICT_CHUNK), false))) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : p->stream;
    if (stream) {
        // parameters and work buffers are ordered on the library's stream
        PK(cudaEventRecord(p->ev, p->stream));
        PK(cudaStreamWaitEvent(s, p->ev, 0));
    }
    for (int off = 0; off < n; off += PREDICT_CHUNK) {
        const int nc = std::min(PREDICT_CHUNK, n - off);
        PK(launch_forward(p, nc, SampleSrc{2, nullptr, d_rot, n, off, lig, nullptr, 0}, s));
        head_kernel<<<(nc + 7) / 8, THREADS, 0, s>>>(p->wb, p->wk.h1, nc, d_out + off, nullptr, nullptr, nc, nullptr,
                                                     nullptr, nullptr);
        PK(cudaGetLastError());
    }
    if (stream) {
        // later work on the library's stream reuses the buffers
        PK(cudaEventRecord(p->ev, s));
        PK(cudaStreamWaitEvent(p->stream, p->ev, 0));
    }
    return FFTDOCK_OK;
}

int fftdock_proposal_predict(fftdock_proposal* p, int32_t lig, int32_t n, const double* rot, float* out) {
    if (!p || n < 0 || (n > 0 && (!rot || !out))) return pfail(p, FFTDOCK_EINVAL, "bad arguments");
    if (n == 0) return FFTDOCK_OK;
    fftdock::DeviceScope dev_scope(p->device);
    PK(dev_scope.status());
    double* d_rot = nullptr;
    float* d_out = nullptr;
    PK(dalloc(&d_rot, 9 * (size_t)n));
    cudaError_t e = dalloc(&d_out, n);
    cudaStream_t s = p->stream;
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_rot, rot, 9 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s);
    int rc = FFTDOCK_OK;
    if (e == cudaSuccess) rc = fftdock_proposal_predict_device(p, lig, n, d_rot, d_out, nullptr);
    if (e == cudaSuccess && rc == FFTDOCK_OK) e = cudaMemcpyAsync(out, d_out, n * sizeof(float), cudaMemcpyDeviceToHost, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    cudaFree(d_rot);
    cudaFree(d_out);
    if (rc) return rc;
    if (e != cudaSuccess) return pfail(p, FFTDOCK_ECUDA, std::string("predict: ") + cudaGetErrorString(e));
    if (e2 != cudaSuccess) return pfail(p, FFTDOCK_ECUDA, std::string("predict: ") + cudaGetErrorString(e2));
    return FFTDOCK_OK;
}

// radial element histograms about the box centre: element e in 0..3, shell
// floor(r / 1.5 A) clamped to 31, divided by the atom count
int fftdock_receptor_descriptor(int32_t n, const double* xyz, const int32_t* element, float* out) {
    if (n < 0 || (n > 0 && (!xyz || !element)) || !out) return FFTDOCK_EINVAL;
    for (int i = 0; i < DESC; ++i) out[i] = 0.f;
    if (n == 0) return FFTDOCK_OK;
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) lo[d] = hi[d] = xyz[d];
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            const double v = xyz[3 * i + d];
            if (!std::isfinite(v)) return FFTDOCK_EINVAL;
            lo[d] = std::min(lo[d], v);
            hi[d] = std::max(hi[d], v);
        }
    std::vector<double> h(DESC, 0.0);
    for (int i = 0; i < n; ++i) {
        if (element[i] < 0 || element[i] > 3) return FFTDOCK_EINVAL;
        double r2 = 0.0;
        for (int d = 0; d < 3; ++d) {
            const double c = 0.5 * (lo[d] + hi[d]);
            const double t = xyz[3 * i + d] - c;
            r2 = r2 + t * t;
        }
        int shell = (int)std::floor(std::sqrt(r2) / 1.5);
        if (shell > 31) shell = 31;
        h[element[i] * 32 + shell] += 1.0;
    }
    for (int i = 0; i < DESC; ++i) out[i] = (float)(h[i] / (double)n);
    return FFTDOCK_OK;
}

// occupancy of the receptor in the scan frame: the cube of half-width L (the
// box's largest half-extent) about the box centre in 4 x 4 x 4 cells; values
// 0..63 the fraction of all atoms per cell, 64..127 the fraction of the outer
// atoms (distance from the centre above 0.7 of the largest) per cell
int fftdock_receptor_descriptor_oriented(int32_t n, const double* xyz, float* out) {
    if (n < 0 || (n > 0 && !xyz) || !out) return FFTDOCK_EINVAL;
    for (int i = 0; i < DESC; ++i) out[i] = 0.f;
    if (n == 0) return FFTDOCK_OK;
    double lo[3], hi[3], c[3];
    for (int d = 0; d < 3; ++d) lo[d] = hi[d] = xyz[d];
    for (int i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            const double v = xyz[3 * i + d];
            if (!std::isfinite(v)) return FFTDOCK_EINVAL;
            lo[d] = std::min(lo[d], v);
            hi[d] = std::max(hi[d], v);
        }
    double L = 0.0, rmax = 0.0;
    for (int d = 0; d < 3; ++d) {
        c[d] = 0.5 * (lo[d] + hi[d]);
        L = std::max(L, 0.5 * (hi[d] - lo[d]));
    }
    std::vector<double> r(n);
    for (int i = 0; i < n; ++i) {
        double r2 = 0.0;
        for (int d = 0; d < 3; ++d) r2 += (xyz[3 * i + d] - c[d]) * (xyz[3 * i + d] - c[d]);
        r[i] = std::sqrt(r2);
        rmax = std::max(rmax, r[i]);
    }
    if (!(L > 0.0)) L = 1.0;
    std::vector<double> h(DESC, 0.0);
    for (int i = 0; i < n; ++i) {
        int cell = 0;
        for (int d = 0; d < 3; ++d) {
            int k = (int)std::floor((xyz[3 * i + d] - (c[d] - L)) / (0.5 * L));
            k = std::min(std::max(k, 0), 3);
            cell = cell * 4 + k;
        }
        h[cell] += 1.0;
        if (r[i] > 0.7 * rmax) h[64 + cell] += 1.0;
    }
    for (int i = 0; i < DESC; ++i) out[i] = (float)(h[i] / (double)n);
    return FFTDOCK_OK;
}

}  // extern "C"
