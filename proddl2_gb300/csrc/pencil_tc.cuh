// Tensor-core form of the pencil stage (tcgen05, sm_103a).
//
// For one pencil (ky, kz) and a group of 128 rotations r, the pencil kernel's
// "forward x-FFT, conj(R^_t) product summed over terms, inverse x-FFT" is a
// circular correlation along x:
//   G2_r(x) = sum_t sum_{n < W} F_{r,t}(x0 + n) c_t((x0 + n - x) mod N)
// where F_{r,t}(x') = sum over ligand entries of bin (t, x') of w^(ky y + kz z)
// (the y and z stages as direct sums), [x0, x0 + W) is a window holding the
// ligand's cells for every rotation, and c_t(d) = conj(R2_t(d, ky, kz)) / N^2
// is the receptor transformed along y and z only.  That is a complex GEMM
//   D[x][r] = sum_k C[x][k] F[r][k],  k = (t, n, re/im)
// run on the tensor cores as real M = 128 (x) x N = 128 (r) x K = 16 MMAs,
// D_re and D_im in tensor memory.  FP32 accuracy comes from splitting each
// operand into FP16 hi + lo parts and accumulating hi*hi + hi*lo + lo*hi in
// FP32; per-pencil power-of-two scales keep both parts in the normal range.
//
// CTA: warps 0-3 produce (thread = rotation of the group) and run the
// epilogue, warp 4 issues the MMAs.  A ring of STAGES shared-memory stages,
// each one chunk = 8 window bins of one term, is handed over with mbarriers;
// every wait is bounded and a timeout is reported through *err.
#pragma once

#include <cuda_fp16.h>

#include "fft_core.cuh"
#include "tc05.cuh"

namespace fftdock {

constexpr int TC_STAGES = 4;
constexpr int TC_ROT = 128;                 // rotations per CTA (MMA N)
constexpr int TC_TILE = 128 * 16 * 2;       // bytes of one 128 x 16 FP16 operand tile
constexpr int TC_STAGE_BYTES = 6 * TC_TILE; // C_re hi/lo, C_im hi/lo, F hi/lo
constexpr uint32_t TC_LBO = 128, TC_SBO = 256;
constexpr uint64_t TC_WAIT_NS = 2000000000ull;  // 2 s per wait
constexpr float TC_F_SCALE = 16.0f;         // scale of the ligand sums before the FP16 split

struct TcPair {      // one receptor circulant sample d, as FP16 pairs
    __half2 re_h;    // (Re c, -Im c) hi: multiplies (F_re, F_im) into the real output
    __half2 im_h;    // (Im c,  Re c) hi: into the imaginary output
    __half2 re_l;
    __half2 im_l;
};

__device__ __forceinline__ void split_h2(float a, float b, __half2& hi, __half2& lo) {
    hi = __floats2half2_rn(a, b);
    const float2 back = __half22float2(hi);
    lo = __floats2half2_rn(a - back.x, b - back.y);
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d)
                 : "memory");
}
__device__ __forceinline__ uint32_t h2u(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }

template <int N>
__global__ void __launch_bounds__(160, 1) pencil_tc_kernel(
    const float2* __restrict__ circ, const int8_t* __restrict__ cscale, const uint32_t* __restrict__ ent,
    const int32_t* __restrict__ offs, const float2* __restrict__ tw, float2* __restrict__ g2, int K, int n_ent,
    int n_rot, int x0, int W, int* __restrict__ err) {
    static_assert(N <= 128, "the tensor pencil stage covers x in one 128-row tile");
    constexpr int H = N / 2 + 1;
    constexpr int NH = N * H;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* stages = smem_raw;                                               // [STAGES][6 tiles]
    TcPair* pairs = reinterpret_cast<TcPair*>(smem_raw + TC_STAGES * TC_STAGE_BYTES);  // [N]
    float2* tws = reinterpret_cast<float2*>(pairs + N);                             // [N]
    __shared__ __align__(8) uint64_t full_bar[TC_STAGES];
    __shared__ __align__(8) uint64_t empty_bar[TC_STAGES];
    __shared__ __align__(8) uint64_t done_bar;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;

    // a timeout elsewhere in this launch already failed the scan: do nothing
    if (*(volatile int*)err != 0) return;
    const int p = blockIdx.x;           // pencil
    const int g = blockIdx.y;           // rotation group
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const unsigned ky = (unsigned)(p / H), kz = (unsigned)(p - (p / H) * H);
    const int n_chunks = K * (W / 8);
    const float c_scale = ldexpf(1.0f, (int)cscale[p]);

    for (int i = tid; i < N; i += blockDim.x) tws[i] = tw[i];
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, 256);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            tc::mbar_init(&full_bar[s], 128);
            tc::mbar_init(&empty_bar[s], 1);
        }
        tc::mbar_init(&done_bar, 1);
        abort_flag = 0;
        tc::fence_barrier_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    const uint32_t sbase = tc::smem_u32(stages);

    if (warp == 4) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            const uint32_t idesc = tc::idesc_f16_f32(128, TC_ROT);
            for (int q = 0; q < n_chunks; ++q) {
                const int s = q % TC_STAGES;
                if (*(volatile int*)&abort_flag ||
                    !tc::mbar_wait(&full_bar[s], (uint32_t)((q / TC_STAGES) & 1), TC_WAIT_NS)) {
                    atomicOr(err, 1);
                    abort_flag = 1;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t st = sbase + s * TC_STAGE_BYTES;
                const uint64_t cre_h = tc::smem_desc(st + 0 * TC_TILE, TC_LBO, TC_SBO);
                const uint64_t cre_l = tc::smem_desc(st + 1 * TC_TILE, TC_LBO, TC_SBO);
                const uint64_t cim_h = tc::smem_desc(st + 2 * TC_TILE, TC_LBO, TC_SBO);
                const uint64_t cim_l = tc::smem_desc(st + 3 * TC_TILE, TC_LBO, TC_SBO);
                const uint64_t f_h = tc::smem_desc(st + 4 * TC_TILE, TC_LBO, TC_SBO);
                const uint64_t f_l = tc::smem_desc(st + 5 * TC_TILE, TC_LBO, TC_SBO);
                const uint32_t acc = q > 0 ? 1u : 0u;
                tc::mma_f16(tmem, cre_h, f_h, idesc, acc);
                tc::mma_f16(tmem, cre_h, f_l, idesc, 1u);
                tc::mma_f16(tmem, cre_l, f_h, idesc, 1u);
                tc::mma_f16(tmem + TC_ROT, cim_h, f_h, idesc, acc);
                tc::mma_f16(tmem + TC_ROT, cim_h, f_l, idesc, 1u);
                tc::mma_f16(tmem + TC_ROT, cim_l, f_h, idesc, 1u);
                tc::mma_commit(&empty_bar[s]);
            }
            tc::mma_commit(&done_bar);
        }
        __syncwarp();
    } else {
        // ---------------- producers: thread r = rotation of the group ----------------
        const int r = tid;
        const int rot = g * TC_ROT + r;
        const bool live = rot < n_rot;
        const uint32_t* ent_r = ent + (size_t)(live ? rot : 0) * n_ent;
        const int32_t* offs_r = offs + (size_t)(live ? rot : 0) * (K * N + 1);
        const int x = r;  // output row of the circulant tiles this thread expands
        for (int q = 0; q < n_chunks; ++q) {
            const int t = q / (W / 8);
            const int n0 = (q - t * (W / 8)) * 8;
            if (n0 == 0) {
                // receptor circulant samples of term t, scaled and split
                asm volatile("bar.sync 1, 128;" ::: "memory");
                for (int d = r; d < N; d += 128) {
                    const float2 c = circ[((size_t)t * NH + p) * N + d];
                    const float cr = c.x * c_scale, ci = c.y * c_scale;
                    TcPair pr;
                    split_h2(cr, -ci, pr.re_h, pr.re_l);
                    split_h2(ci, cr, pr.im_h, pr.im_l);
                    pairs[d] = pr;
                }
                asm volatile("bar.sync 1, 128;" ::: "memory");
            }
            // ligand sums of 8 window bins for this thread's rotation
            float2 f[8];
            if (live) {
                const int32_t* ob = offs_r + t * N;
                int xb = x0 + n0;
                int b = xb < N ? ob[xb] : 0;
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int xi = xb + i;
                    float2 acc = make_float2(0.f, 0.f);
                    if (xi < N) {
                        const int e = ob[xi + 1];
                        for (int j = b; j < e; ++j) {
                            const uint32_t u = __ldg(ent_r + j);
                            const unsigned ph = (ky * ((u >> 8) & 255u) + kz * (u & 255u)) % (unsigned)N;
                            const float2 z = tws[ph];
                            acc.x += z.x;
                            acc.y += z.y;
                        }
                        b = e;
                    }
                    f[i] = acc;
                }
            } else {
#pragma unroll
                for (int i = 0; i < 8; ++i) f[i] = make_float2(0.f, 0.f);
            }
            const int s = q % TC_STAGES;
            // after a timeout anywhere, keep iterating (the named barriers
            // above need every producer) but stop handing stages over
            if (*(volatile int*)&abort_flag) continue;
            if (!tc::mbar_wait(&empty_bar[s], (uint32_t)(((q / TC_STAGES) & 1) ^ 1), TC_WAIT_NS)) {
                atomicOr(err, 2);
                abort_flag = 1;
                continue;
            }
            const uint32_t st = sbase + s * TC_STAGE_BYTES;
            // F tile row r: k = 2i + {re, im}
            {
                __half2 hi[8], lo[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) split_h2(f[i].x * TC_F_SCALE, f[i].y * TC_F_SCALE, hi[i], lo[i]);
                const uint32_t o0 = tc::kmajor_offset(r, 0, TC_LBO, TC_SBO);
                const uint32_t o1 = tc::kmajor_offset(r, 8, TC_LBO, TC_SBO);
                st_shared_v4(st + 4 * TC_TILE + o0, h2u(hi[0]), h2u(hi[1]), h2u(hi[2]), h2u(hi[3]));
                st_shared_v4(st + 4 * TC_TILE + o1, h2u(hi[4]), h2u(hi[5]), h2u(hi[6]), h2u(hi[7]));
                st_shared_v4(st + 5 * TC_TILE + o0, h2u(lo[0]), h2u(lo[1]), h2u(lo[2]), h2u(lo[3]));
                st_shared_v4(st + 5 * TC_TILE + o1, h2u(lo[4]), h2u(lo[5]), h2u(lo[6]), h2u(lo[7]));
            }
            // circulant tile row x: k = 2i + {re, im} -> c((x0 + n0 + i - x) mod N)
            {
                TcPair v[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    if (x < N) {
                        int d = (x0 + n0 + i - x) % N;
                        if (d < 0) d += N;
                        v[i] = pairs[d];
                    } else {
                        const __half2 z = __floats2half2_rn(0.f, 0.f);
                        v[i] = TcPair{z, z, z, z};
                    }
                }
                const uint32_t o0 = tc::kmajor_offset(x, 0, TC_LBO, TC_SBO);
                const uint32_t o1 = tc::kmajor_offset(x, 8, TC_LBO, TC_SBO);
                st_shared_v4(st + 0 * TC_TILE + o0, h2u(v[0].re_h), h2u(v[1].re_h), h2u(v[2].re_h), h2u(v[3].re_h));
                st_shared_v4(st + 0 * TC_TILE + o1, h2u(v[4].re_h), h2u(v[5].re_h), h2u(v[6].re_h), h2u(v[7].re_h));
                st_shared_v4(st + 1 * TC_TILE + o0, h2u(v[0].re_l), h2u(v[1].re_l), h2u(v[2].re_l), h2u(v[3].re_l));
                st_shared_v4(st + 1 * TC_TILE + o1, h2u(v[4].re_l), h2u(v[5].re_l), h2u(v[6].re_l), h2u(v[7].re_l));
                st_shared_v4(st + 2 * TC_TILE + o0, h2u(v[0].im_h), h2u(v[1].im_h), h2u(v[2].im_h), h2u(v[3].im_h));
                st_shared_v4(st + 2 * TC_TILE + o1, h2u(v[4].im_h), h2u(v[5].im_h), h2u(v[6].im_h), h2u(v[7].im_h));
                st_shared_v4(st + 3 * TC_TILE + o0, h2u(v[0].im_l), h2u(v[1].im_l), h2u(v[2].im_l), h2u(v[3].im_l));
                st_shared_v4(st + 3 * TC_TILE + o1, h2u(v[4].im_l), h2u(v[5].im_l), h2u(v[6].im_l), h2u(v[7].im_l));
            }
            tc::fence_proxy_async_smem();
            tc::mbar_arrive(&full_bar[s]);
        }
        // ---------------- epilogue: TMEM -> g2[rot][p][x] ----------------
        if (!tc::mbar_wait(&done_bar, 0, TC_WAIT_NS)) atomicOr(err, 4);
        tc::fence_after_sync();
        const float inv = 1.0f / (c_scale * TC_F_SCALE);
        const int xo = 32 * warp + lane;  // TMEM lane = output row x
#pragma unroll 1
        for (int cb = 0; cb < TC_ROT / 32; ++cb) {
            uint32_t dre[32], dim[32];
            tc::tmem_ld_32x32b_x32(tmem + ((uint32_t)(32 * warp) << 16) + cb * 32, dre);
            tc::tmem_ld_32x32b_x32(tmem + ((uint32_t)(32 * warp) << 16) + TC_ROT + cb * 32, dim);
            tc::tmem_wait_ld();
            if (xo < N) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const int rr = g * TC_ROT + cb * 32 + j;
                    if (rr < n_rot)
                        g2[((size_t)rr * NH + p) * N + xo] =
                            make_float2(__uint_as_float(dre[j]) * inv, __uint_as_float(dim[j]) * inv);
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 256);
}

// per-pencil power-of-two exponent so that the largest circulant component
// of the pencil (over all terms) scales to about 2^13
template <int N>
__global__ void circ_scale_kernel(const float2* __restrict__ circ, int K, int8_t* __restrict__ cscale) {
    constexpr int NH = N * (N / 2 + 1);
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NH) return;
    float m = 0.f;
    for (int t = 0; t < K; ++t)
        for (int d = 0; d < N; ++d) {
            const float2 c = circ[((size_t)t * NH + p) * N + d];
            m = fmaxf(m, fmaxf(fabsf(c.x), fabsf(c.y)));
        }
    int e = 0;
    if (m > 0.f) {
        int ex;
        frexpf(m, &ex);  // m in [2^(ex-1), 2^ex)
        e = 13 - ex;
    }
    e = e < -100 ? -100 : (e > 100 ? 100 : e);
    cscale[p] = (int8_t)e;
}

// circ[t][p][d] = conj(R2_t(d, p)) / N^2 from the y/z-transformed half grid [N][N*H]
static __global__ void pack_circ_kernel(const double2* __restrict__ half, float2* __restrict__ circ_t, int n, int nh,
                                        double scale) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t tot = (size_t)n * nh;
    if (i >= tot) return;
    const size_t p = i / n;
    const int d = (int)(i - p * n);
    const double2 v = half[(size_t)d * nh + p];
    circ_t[i] = make_float2((float)(v.x * scale), (float)(-v.y * scale));
}

}  // namespace fftdock
