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
// operand into FP16 hi + lo parts and accumulating hi*hi + hi*lo + lo*hi;
// per-pencil power-of-two scales keep both parts in the normal range.  The
// tensor core's FP32 accumulation does not round to nearest, and its error
// grows with the length of the chain of MMAs into one accumulator (270 at
// 18 terms and a 40-cell window), so the terms are split into
// ceil(Ka / tg) groups of as equal a size as possible (at most tg terms), the
// accumulator restarts at each group, and the groups' sums are added in FP32
// (round to nearest).  The running sum between groups lives in a dense
// 128 KB slot buffer of the CTA's (SM, tensor-memory half), which stays in L2
// (one slot per CTA that can be resident: the two CTAs of an SM hold
// different tensor-memory columns), and the output is written once.
//
// Operands.  C is Toeplitz: the tile of window chunk n0 = 8c is
//   C_c[x][i] = c_t((x0 + 8c + i - x) mod N) = E[x + W - 8 - 8c][i],
//   E[e][i]   = c_t((x0 + W - 8 + i - e) mod N),  e < 120 + W,
// so one extended tile E of 120 + W rows per term serves every chunk: chunk
// c's descriptor starts (W/8 - 1 - c) 8-row groups into E.  F comes from the
// ligand entries of the term, which ligand prep writes transposed per group
// of 128 rotations ([entry / 4][rotation][entry % 4], sorted by (term, x) per
// rotation, each term's range padded to a multiple of 8, x relative to x0;
// padding and cells outside the window carry x' = W, a dummy staging row).
// A term's entries occupy the same index range in every rotation; two threads
// per rotation walk the two halves of the range with coalesced loads.  Each
// keeps the running sum of its current x bin and stores it after every entry
// into an FP32 staging row (the last store of a bin holds its sum: the
// entries are sorted by x), which needs no branch.  The second half's first
// bin may continue the first half's last one: its partial sum goes to a side
// slot and is added after both halves are done.  The staging rows, laid over
// the F tiles, are then converted in place into the hi/lo tiles.  The phase
// table (scaled by the F scale) is replicated per lane ([phase][lane]) so
// that the 32 lanes' lookups never share a bank.
//
// CTA (256 threads): eight producer warps (two threads per rotation); thread
// 0 also issues each term's MMAs after a barrier of all producers.  The
// producers fill the next term's tiles only after the tensor core has read
// the current ones, so two CTAs share an SM (shared memory and 2 x 256 TMEM
// columns permitting) and overlap each other's MMAs and production; 16 warps
// per SM leave 128 registers per thread.  All waits are bounded; a timeout is
// reported through *err.
#pragma once

#include <cuda_fp16.h>

#include "fft_core.cuh"
#include "internal.h"
#include "tc05.cuh"

namespace fftdock {

constexpr int TC_ROT = kTcRot;              // rotations per CTA (MMA N)
constexpr int TC_THREADS = 256;             // 8 producer warps; thread 0 also issues the MMAs
constexpr uint32_t TC_LBO = 128, TC_SBO = 256;
constexpr uint32_t TC_FTILE = 128 * 16 * 2;       // one 128 x 16 FP16 tile (hi or lo)
constexpr uint32_t TC_FCHUNK = 2 * TC_FTILE;      // hi + lo of one window chunk
constexpr uint64_t TC_WAIT_NS = 2000000000ull;    // 2 s per wait
constexpr float TC_F_SCALE = 16.0f;               // scale of the ligand sums before the FP16 split

// stored and loaded as one 128-bit shared-memory access (four 32-bit
// accesses 16 bytes apart would conflict four ways)
struct __align__(16) TcPair {      // one receptor circulant sample d, as FP16 pairs
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

// Shared-memory accesses to the operand tiles and staging rows.  Volatile:
// they keep their order among themselves and against the fences and barriers
// (volatile, with memory clobbers); without a clobber of their own, ordinary
// loads of other shared arrays may move across them.
__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d));
}
__device__ __forceinline__ void st_shared_f2(uint32_t addr, float a, float b) {
    asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(a), "f"(b));
}
__device__ __forceinline__ float2 ld_shared_f2(uint32_t addr) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}
// load from a table that no longer changes: not volatile, so the compiler
// may schedule it freely
__device__ __forceinline__ float2 ld_shared_f2_const(uint32_t addr) {
    float2 v;
    asm("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}
__device__ __forceinline__ uint32_t h2u(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }
__device__ __forceinline__ __half2 u2h(uint32_t u) { return *reinterpret_cast<__half2*>(&u); }
// one circulant sample (re_h, im_h, re_l, im_l) as one 128-bit load
__device__ __forceinline__ TcPair ld_pair(uint32_t addr) {
    uint32_t a, b, c, d;
    asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];" : "=r"(a), "=r"(b), "=r"(c), "=r"(d) : "r"(addr));
    TcPair v;
    v.re_h = u2h(a);
    v.im_h = u2h(b);
    v.re_l = u2h(c);
    v.im_l = u2h(d);
    return v;
}

// Running-sum slot accesses: relaxed at GPU scope, like the atomic adds
// between them, so that one thread's accesses to a cell stay in program
// order (coherence of morally strong operations on one location).
__device__ __forceinline__ void st_relaxed_f2(float2* p, float2 v) {
    asm volatile("st.relaxed.gpu.global.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ float2 ld_relaxed_f2(const float2* p) {
    float2 v;
    asm volatile("ld.relaxed.gpu.global.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p) : "memory");
    return v;
}

// 8-row groups of the extended circulant tile E for a window of 8 n_chunks
// cells and mt 128-row output tiles
__host__ __device__ constexpr int tc_ext_groups(int n_chunks, int mt = 1) { return 16 * mt - 1 + n_chunks; }
// output tiles of 128 x rows for an x extent of n cells (n <= 256)
__host__ __device__ constexpr int tc_tiles(int n) { return n > 128 ? 2 : 1; }

// Box grids (pencil_tc_kernel<0, MT>): sizes per axis, nx <= 128 MT, pencil
// p = ky hz + kz of nh = ny hz pencils, x-quads over nxp = nx rounded up to
// 4, and the FP32 twiddle tables of the y and z axes
// (e^{-2 pi i m / n}).  The phase of an entry is the product of its y and z
// phases, from two tables per CTA (its pencil's ky and kz).
struct TcBox {
    int nx, ny, nz, hz, nh, nxp;
    const float2* twy;
    const float2* twz;
};

// dynamic shared memory of pencil_tc_kernel: F tiles / staging rows
// [chunks][hi|lo], E tiles [4 parts][groups][256 B], phase table [N][32]
// float2, staged samples [N], side slots [128] float2, term table; at least
// 76 KB so that no more than two CTAs (2 x 256 TMEM columns) share an SM
__host__ __device__ inline size_t tc_smem_bytes(int N, int n_chunks, int n_terms) {
    const int mt = tc_tiles(N);
    size_t b = (size_t)n_chunks * TC_FCHUNK + 1024 + (size_t)4 * tc_ext_groups(n_chunks, mt) * 256 +
               (size_t)N * 32 * 8 + (size_t)N * sizeof(TcPair) + (size_t)TC_ROT * 8 + (size_t)(2 * n_terms + 1) * 4;
    b = (b + 15) & ~(size_t)15;
    return b < 76 * 1024 ? 76 * 1024 : b;
}
// box grids: the y and z phase tables per half-warp lane ([n][16] float2)
// in place of the [N][32] table
__host__ __device__ inline size_t tc_smem_bytes_box(int nx, int ny, int nz, int n_chunks, int n_terms) {
    size_t b = (size_t)n_chunks * TC_FCHUNK + 1024 + (size_t)4 * tc_ext_groups(n_chunks, tc_tiles(nx)) * 256 +
               (size_t)(ny + nz) * 16 * 8 + (size_t)nx * sizeof(TcPair) + (size_t)TC_ROT * 8 +
               (size_t)(2 * n_terms + 1) * 4;
    b = (b + 15) & ~(size_t)15;
    return b < 76 * 1024 ? 76 * 1024 : b;
}

// A rotation's sorted walk, eight entries at a time: first the eight phase
// lookups (so that none waits behind a staging store), then for each entry
// the running sum of its x bin (restarted when x changes), stored into the
// bin's staging row or, for SIDE and the walk's first bin, into the side slot.
// Entry e = x' << 24 | y << 16 | z and kyz = kz << 16 | ky: bits 16 and up
// of e * kyz (mod 2^32) hold ky y + kz z (< 2^15; the z ky term stays below
// bit 16 and x' ky starts at bit 24), so a power-of-two N needs one multiply
// and one field extract for the phase.
template <int N>
__device__ __forceinline__ unsigned tc_phase(uint32_t e, uint32_t kyz) {
    if constexpr ((N & (N - 1)) == 0) return ((e * kyz) >> 16) & (unsigned)(N - 1);
    else return (((e & 0xffffffu) * kyz) >> 16) % (unsigned)N;
}

// N = 0 (box grids): twl and tzl are this lane's columns of the y and z
// phase tables ([n][16] float2), and the phase is their complex product.
template <bool SIDE, int N>
__device__ __forceinline__ void tc_entries8(const uint32_t (&e)[8], uint32_t kyz, uint32_t twl, uint32_t tzl,
                                            uint32_t stg, uint32_t sd, unsigned first, unsigned& cur, float2& acc) {
    float2 z[8];
    unsigned xr[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        // x relative to the window start; padding and cells outside the
        // window carry x' = W, a dummy staging row
        xr[q] = e[q] >> 24;
        if constexpr (N == 0) {
            const float2 a = ld_shared_f2_const(twl + ((e[q] >> 16) & 255u) * 128u);
            const float2 b = ld_shared_f2_const(tzl + (e[q] & 255u) * 128u);
            z[q] = make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
        } else {
            z[q] = ld_shared_f2_const(twl + tc_phase<N>(e[q], kyz) * 256u);
        }
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float keep = xr[q] != cur ? 0.f : 1.f;
        acc.x = fmaf(acc.x, keep, z[q].x);
        acc.y = fmaf(acc.y, keep, z[q].y);
        cur = xr[q];
        uint32_t dst = stg + xr[q] * 1024u;
        if (SIDE) dst = xr[q] == first ? sd : dst;
        st_shared_f2(dst, acc.x, acc.y);
    }
}

// Walk nblk blocks of 8 rows from eq (this rotation's quads of rows: one
// uint4 per 4 rows, consecutive quads 128 uint4 apart), blocks 0 and 1
// already loaded into (a0, a1) and (b0, b1).  Two blocks are in flight while
// one is summed; the loads may run up to 16 rows past the range, which the
// entry buffer provides.
template <bool SIDE, int N>
__device__ __forceinline__ void tc_walk(const uint4* eq, int nblk, uint32_t kyz, uint32_t twl, uint32_t tzl,
                                        uint32_t stg, uint32_t sd, unsigned first, unsigned W, uint4 a0, uint4 a1,
                                        uint4 b0, uint4 b1) {
    (void)W;
    unsigned cur = 0xffffffffu;
    float2 acc = make_float2(0.f, 0.f);
    if (nblk <= 0) return;
    uint4 c0, c1;
    auto ld = [&](int blk, uint4& x0, uint4& x1) {
        x0 = __ldg(eq + (size_t)(2 * blk) * TC_ROT);
        x1 = __ldg(eq + (size_t)(2 * blk + 1) * TC_ROT);
    };
    auto sum = [&](const uint4& x0, const uint4& x1) {
        const uint32_t e[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
        tc_entries8<SIDE, N>(e, kyz, twl, tzl, stg, sd, first, cur, acc);
    };
    for (int blk = 0; blk < nblk; blk += 3) {
        ld(blk + 2, c0, c1);
        sum(a0, a1);
        if (blk + 1 >= nblk) break;
        ld(blk + 3, a0, a1);
        sum(b0, b1);
        if (blk + 2 >= nblk) break;
        ld(blk + 4, b0, b1);
        sum(c0, c1);
    }
}

// tinfo: [0, Ka] padded entry starts (multiples of 8) of the Ka non-empty
// terms, [Ka + 1, 2 Ka] their term ids; n_pad = entry rows per rotation group.
// N = 0: a box grid of the sizes in bx (every N-dependent length below is
// then bx's runtime value).  MT output tiles of 128 x rows: MT = 2 (x extent
// up to 256) doubles the MMAs of a chunk (the second tile's circulant rows
// start 16 8-row groups further into E) and takes 512 TMEM columns, one CTA
// per SM.
template <int N, int MT>
__global__ void __launch_bounds__(TC_THREADS, MT == 1 ? 2 : 1) pencil_tc_kernel(
    const float2* __restrict__ circ, const int8_t* __restrict__ cscale, const uint32_t* __restrict__ ent_t,
    const int32_t* __restrict__ tinfo, int Ka, const float2* __restrict__ tw, float2* __restrict__ g2t, int n_pad,
    int n_rot, int x0, int W, int tg, float2* __restrict__ slots, int n_slots, TcBox bx, int* __restrict__ err) {
    static_assert(N <= 128 * MT && (MT == 1 || MT == 2), "the tensor pencil stage covers x in MT 128-row tiles");
    constexpr bool BOX = N == 0;
    constexpr uint32_t TM_COLS = 256u * MT;
    const int nx = BOX ? bx.nx : N;                  // x extent (correlation length)
    const int H = BOX ? bx.hz : N / 2 + 1;           // kz per ky
    const int NH = BOX ? bx.nh : N * (N / 2 + 1);    // pencils
    const int NXP = BOX ? bx.nxp : N;                // x extent of the x-quads
    const int NC = W >> 3;
    const int RG = tc_ext_groups(NC, MT);
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* fbuf = smem_raw;                                            // [NC][hi | lo]
    unsigned char* abuf = fbuf + NC * TC_FCHUNK + 1024;                        // [4][RG][256] after the dummy row
    float2* twr = reinterpret_cast<float2*>(abuf + 4 * RG * 256);              // [N][32] (box: [ny][16], [nz][16])
    const int tw_len = BOX ? (bx.ny + bx.nz) * 16 : N * 32;
    TcPair* pr = reinterpret_cast<TcPair*>(twr + tw_len);                      // [nx]
    float2* side = reinterpret_cast<float2*>(pr + nx);                         // [128]
    int32_t* tinf = reinterpret_cast<int32_t*>(side + TC_ROT);                 // [2 Ka + 1]
    __shared__ __align__(8) uint64_t empty_bar;
    __shared__ __align__(8) uint64_t done_bar;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;

    const int p = blockIdx.x;           // pencil
    const int g = blockIdx.y;           // rotation group
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const unsigned ky = (unsigned)(p / H), kz = (unsigned)(p - (p / H) * H);
    const uint32_t kyz = (kz << 16) | ky;  // the phase multiplier of tc_phase
    const float c_scale = ldexpf(1.0f, (int)cscale[p]);

    if (tid == 0) abort_flag = *(volatile int*)err;
    __syncthreads();
    // a timeout elsewhere in this launch already failed the scan: do nothing
    if (abort_flag) return;

    if constexpr (BOX) {
        // this pencil's phases along y (scaled by the F scale) and z, per
        // half-warp lane: the lookups of a half-warp never share a bank
        for (int i = tid; i < bx.ny * 16; i += blockDim.x) {
            const float2 v = bx.twy[(int)(((unsigned)(i >> 4) * ky) % (unsigned)bx.ny)];
            twr[i] = make_float2(v.x * TC_F_SCALE, v.y * TC_F_SCALE);
        }
        for (int i = tid; i < bx.nz * 16; i += blockDim.x) twr[bx.ny * 16 + i] = bx.twz[(int)(((unsigned)(i >> 4) * kz) % (unsigned)bx.nz)];
    } else {
        for (int i = tid; i < N * 32; i += blockDim.x) {
            const float2 v = tw[i >> 5];
            twr[i] = make_float2(v.x * TC_F_SCALE, v.y * TC_F_SCALE);
        }
    }
    for (int i = tid; i <= 2 * Ka; i += blockDim.x) tinf[i] = tinfo[i];
    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, TM_COLS);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&empty_bar, 1);
        tc::mbar_init(&done_bar, 1);
        tc::fence_barrier_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_base;
    // group of processing step k: ng groups, sizes differing by at most one
    const int ng = (Ka + tg - 1) / tg;
    auto group_of = [&](int k) { return (k * ng) / Ka; };
    auto starts_group = [&](int k) { return k == 0 || group_of(k) != group_of(k - 1); };
    const uint32_t fb = tc::smem_u32(fbuf);
    const uint32_t ab = tc::smem_u32(abuf);
    const uint32_t prb = tc::smem_u32(pr);

    // MMA issue for term k (thread 0, after the producers' arrivals): 6 MMAs
    // per window chunk into the real and imaginary accumulators, then a
    // commit that arrives on empty_bar once they have read the tiles
    const uint32_t idesc = tc::idesc_f16_f32(128, TC_ROT);
    auto issue_term = [&](int k) {
        for (int c = 0; c < NC; ++c) {
            const uint64_t f_h = tc::smem_desc(fb + c * TC_FCHUNK, TC_LBO, TC_SBO);
            const uint64_t f_l = tc::smem_desc(fb + c * TC_FCHUNK + TC_FTILE, TC_LBO, TC_SBO);
            // each group of terms starts a fresh accumulator
            const uint32_t acc = (starts_group(k) && c == 0) ? 0u : 1u;
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                const uint32_t d_re = tmem + 256u * mt, d_im = d_re + TC_ROT;
                const uint32_t ao = (uint32_t)(NC - 1 - c + 16 * mt) * TC_SBO;
                const uint64_t cre_h = tc::smem_desc(ab + 0 * RG * 256 + ao, TC_LBO, TC_SBO);
                const uint64_t cre_l = tc::smem_desc(ab + 1 * RG * 256 + ao, TC_LBO, TC_SBO);
                const uint64_t cim_h = tc::smem_desc(ab + 2 * RG * 256 + ao, TC_LBO, TC_SBO);
                const uint64_t cim_l = tc::smem_desc(ab + 3 * RG * 256 + ao, TC_LBO, TC_SBO);
                tc::mma_f16(d_re, cre_h, f_h, idesc, acc);
                tc::mma_f16(d_re, cre_h, f_l, idesc, 1u);
                tc::mma_f16(d_re, cre_l, f_h, idesc, 1u);
                tc::mma_f16(d_im, cim_h, f_h, idesc, acc);
                tc::mma_f16(d_im, cim_h, f_l, idesc, 1u);
                tc::mma_f16(d_im, cim_l, f_h, idesc, 1u);
            }
        }
        tc::mma_commit(&empty_bar);
    };

    // Thread (warp, lane) holds output row x = 32 (warp % 4) + lane of the
    // rotations [64 half, 64 half + 64) (its TMEM lane and columns).
    // Running sum of the completed groups: this CTA's slot, [rotation][x]
    // raw accumulator values (a warp access covers 256 consecutive bytes).
    // The first group's sum is stored, later ones are added with FP32
    // atomic adds (round to nearest, performed in L2, no wait), and the last
    // group's sum is added by the output pass.  Every access to one element
    // comes from one thread in program order, so the order of the additions
    // is fixed ((S1 + S2) + S3 ...) and the result the same in every run.
    uint32_t smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    // 256-column allocations start at column 0 or 256 (two CTAs per SM);
    // with two tiles the CTA holds all 512 columns and both of the SM's slots
    const int slot = MT == 1 ? (int)smid * 2 + (int)((tmem >> 8) & 1u) : (int)smid * 2;
    const bool slot_ok = slot + MT - 1 < n_slots;
    if (ng > 1 && !slot_ok && tid == 0) {
        atomicOr(err, 32);
        abort_flag = 1;
    }
    const int xo = 32 * (warp & 3) + lane;  // TMEM lane = output row x
    const uint32_t trow = (uint32_t)(32 * (warp & 3)) << 16;
    const int half = tid >> 7;
    float2* const sb = slots + (size_t)(slot_ok ? slot : 0) * (TC_ROT * 128) + xo;
    auto drain_group = [&](bool first) {
        if (!slot_ok) return;
#pragma unroll 1
        for (int cb = 0; cb < 4 * MT; ++cb) {
            const int mt = cb >> 2;  // tile: its own slot and 256 TMEM columns
            const int c0 = half * 64 + (cb & 3) * 16;
            float2* const st = sb + (size_t)mt * (TC_ROT * 128);
            uint32_t dre[16], dim[16];
            tc::tmem_ld_32x32b_x16(tmem + 256u * mt + trow + c0, dre);
            tc::tmem_ld_32x32b_x16(tmem + 256u * mt + trow + TC_ROT + c0, dim);
            tc::tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float2 v = make_float2(__uint_as_float(dre[j]), __uint_as_float(dim[j]));
                if (first) st_relaxed_f2(st + (size_t)(c0 + j) * 128, v);
                else atomicAdd(st + (size_t)(c0 + j) * 128, v);
            }
        }
    };
    // TMEM (+ the running sum) -> x-quads g2t[rot][x/4][p][x%4] (a warp
    // access covers 8 whole sectors), in blocks of 8 rotations.  The running
    // sum of a block is loaded one block ahead; block 0's loads are issued
    // before the wait for the last MMAs.
    const float inv = 1.0f / (c_scale * TC_F_SCALE);
    const bool with_sum = ng > 1 && slot_ok;
    // block cb: tile cb / 8, rotations half * 64 + (cb % 8) * 8 ..
    auto load_run = [&](int cb, float2 (&run)[8]) {
        const int c0 = half * 64 + (cb & 7) * 8;
        const float2* st = sb + (size_t)(cb >> 3) * (TC_ROT * 128);
#pragma unroll
        for (int j = 0; j < 8; ++j) run[j] = ld_relaxed_f2(st + (size_t)(c0 + j) * 128);
    };
    auto out_block = [&](int cb, const float2 (&run)[8]) {
        const int mt = cb >> 3;
        const int c0 = half * 64 + (cb & 7) * 8;
        const int x = 128 * mt + xo;  // output row
        uint32_t dre[8], dim[8];
        tc::tmem_ld_32x32b_x8(tmem + 256u * mt + trow + c0, dre);
        tc::tmem_ld_32x32b_x8(tmem + 256u * mt + trow + TC_ROT + c0, dim);
        tc::tmem_wait_ld();
        if (x < nx) {
            float2* ob = g2t + (size_t)(g * TC_ROT + c0) * NH * NXP + (size_t)(x >> 2) * NH * 4 + (size_t)p * 4 +
                         (x & 3);
            const int nj = min(8, n_rot - (g * TC_ROT + c0));
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                float2 v = make_float2(__uint_as_float(dre[j]), __uint_as_float(dim[j]));
                if (with_sum) v = make_float2(run[j].x + v.x, run[j].y + v.y);
                if (j < nj) ob[(size_t)j * NH * NXP] = make_float2(v.x * inv, v.y * inv);
            }
        }
    };

    {
        // ---------------- producers: thread (r, half) ----------------
        const int r = tid & 127;
        const int half = tid >> 7;
        // this rotation's quads of rows of the group ([g][row / 4][rotation][4])
        const uint4* ent_g = reinterpret_cast<const uint4*>(ent_t) + (size_t)g * (n_pad / 4) * TC_ROT + r;
        // this lane's copy of the phase table (box: its half-warp column of
        // the y table, and of the z table)
        const uint32_t twl = tc::smem_u32(twr) + (uint32_t)(BOX ? (lane & 15) : lane) * 8u;
        const uint32_t tzl = BOX ? twl + (uint32_t)bx.ny * 128u : 0u;
        const uint32_t stg = fb + (uint32_t)r * 8u;                     // staging row x' at stg + 1024 x'
        const uint32_t sd = tc::smem_u32(side) + (uint32_t)r * 8u;
        const uint32_t r0 = tc::kmajor_offset((uint32_t)r, 0, TC_LBO, TC_SBO);
        const uint32_t r1 = tc::kmajor_offset((uint32_t)r, 8, TC_LBO, TC_SBO);
        // the loads a term starts with (its circulant sample, this thread's
        // first two entry blocks) are issued before the wait for the tensor
        // core, so that they land while it reads the previous term's tiles
        float2 cpre = make_float2(0.f, 0.f);
        uint4 pa0, pa1, pb0, pb1;
        auto preload = [&](int kk) {
            const int jt = tinf[kk], m8 = (tinf[kk + 1] - jt) >> 3;
            const int bb = half ? (m8 + 1) >> 1 : 0;
            const uint4* q = ent_g + (size_t)((jt >> 2) + 2 * bb) * TC_ROT;
            pa0 = __ldg(q);
            pa1 = __ldg(q + TC_ROT);
            pb0 = __ldg(q + 2 * TC_ROT);
            pb1 = __ldg(q + 3 * TC_ROT);
            if (tid < nx) cpre = circ[((size_t)tinf[Ka + 1 + kk] * NH + p) * nx + tid];
        };
        preload(0);
        for (int k = 0; k < Ka; ++k) {
            // the tensor core has read the previous term's tiles: one lane
            // per warp polls the barrier and the warp follows it, except
            // before a drain, whose tensor-memory loads every thread orders
            // after its own wait
            if (k >= 1) {
                if ((lane == 0 || starts_group(k)) && !*(volatile int*)&abort_flag &&
                    !tc::mbar_wait(&empty_bar, (uint32_t)((k - 1) & 1), TC_WAIT_NS)) {
                    atomicOr(err, 2);
                    abort_flag = 1;
                }
                __syncwarp();
            }
            // a group of terms is complete in TMEM: add it into the output
            // before term k restarts the accumulator (the loads have finished
            // when this thread reaches the barrier before the MMA issue)
            if (k >= 1 && starts_group(k) && !*(volatile int*)&abort_flag) {
                tc::fence_after_sync();
                drain_group(group_of(k - 1) == 0);
                tc::fence_before_sync();
            }
            // receptor circulant samples of the term, scaled and split
            if (tid < nx) {
                const float2 c = cpre;
                const float cr = c.x * c_scale, ci = c.y * c_scale;
                TcPair v;
                split_h2(cr, -ci, v.re_h, v.re_l);
                split_h2(ci, cr, v.im_h, v.im_l);
                st_shared_v4(prb + (uint32_t)tid * 16u, h2u(v.re_h), h2u(v.im_h), h2u(v.re_l), h2u(v.im_l));
            }
            // zero the staging rows (W x 128 float2, the F tile bytes)
            for (uint32_t off = (uint32_t)tid * 16u; off < (uint32_t)W * 1024u; off += 256u * 16u)
                st_shared_v4(fb + off, 0u, 0u, 0u, 0u);
            asm volatile("bar.sync 1, 256;" ::: "memory");
            // extended circulant tile E: row e, k = 2i + {re, im} -> c((x0 + W - 8 + i - e) mod N)
            for (int e = tid; e < 8 * RG; e += 256) {
                int d0 = (x0 + W - 8 - e) % nx;
                if (d0 < 0) d0 += nx;
                TcPair v[8];
#pragma unroll
                for (int i2 = 0; i2 < 8; ++i2) {
                    const int d = d0 + i2;
                    v[i2] = ld_pair(prb + (uint32_t)(d < nx ? d : d - nx) * 16u);
                }
                const uint32_t o0 = tc::kmajor_offset((uint32_t)e, 0, TC_LBO, TC_SBO);
                const uint32_t o1 = tc::kmajor_offset((uint32_t)e, 8, TC_LBO, TC_SBO);
                const uint32_t pre = ab, prl = ab + RG * 256, pie = ab + 2 * RG * 256, pil = ab + 3 * RG * 256;
                st_shared_v4(pre + o0, h2u(v[0].re_h), h2u(v[1].re_h), h2u(v[2].re_h), h2u(v[3].re_h));
                st_shared_v4(pre + o1, h2u(v[4].re_h), h2u(v[5].re_h), h2u(v[6].re_h), h2u(v[7].re_h));
                st_shared_v4(prl + o0, h2u(v[0].re_l), h2u(v[1].re_l), h2u(v[2].re_l), h2u(v[3].re_l));
                st_shared_v4(prl + o1, h2u(v[4].re_l), h2u(v[5].re_l), h2u(v[6].re_l), h2u(v[7].re_l));
                st_shared_v4(pie + o0, h2u(v[0].im_h), h2u(v[1].im_h), h2u(v[2].im_h), h2u(v[3].im_h));
                st_shared_v4(pie + o1, h2u(v[4].im_h), h2u(v[5].im_h), h2u(v[6].im_h), h2u(v[7].im_h));
                st_shared_v4(pil + o0, h2u(v[0].im_l), h2u(v[1].im_l), h2u(v[2].im_l), h2u(v[3].im_l));
                st_shared_v4(pil + o1, h2u(v[4].im_l), h2u(v[5].im_l), h2u(v[6].im_l), h2u(v[7].im_l));
            }
            // this thread's half of the term's rows, in blocks of 8
            const int jt0 = tinf[k], n8 = (tinf[k + 1] - jt0) >> 3;
            const int na = (n8 + 1) >> 1;
            const int b0 = half ? na : 0, nb8 = half ? n8 - na : na;
            const uint4* eq = ent_g + (size_t)((jt0 >> 2) + 2 * b0) * TC_ROT;
            // the second half's first bin goes to the side slot
            const unsigned first = half && nb8 > 0 ? (pa0.x >> 24) : 0xfffffffeu;
            if (half)
                tc_walk<true, N>(eq, nb8, kyz, twl, tzl, stg, sd, first, (unsigned)W, pa0, pa1, pb0, pb1);
            else
                tc_walk<false, N>(eq, nb8, kyz, twl, tzl, stg, sd, first, (unsigned)W, pa0, pa1, pb0, pb1);
            asm volatile("bar.sync 1, 256;" ::: "memory");
            // the second half's first bin: add its partial sum
            if (half && first < (unsigned)W) {
                const float2 a = ld_shared_f2(stg + first * 1024u), b = ld_shared_f2(sd);
                st_shared_f2(stg + first * 1024u, a.x + b.x, a.y + b.y);
            }
            asm volatile("bar.sync 1, 256;" ::: "memory");
            // staging rows -> F tiles (hi, lo): thread half h converts chunks
            // c = 2 s + h; chunk c's staging rows and tiles occupy the same
            // bytes, so every thread reads its chunk before any thread writes
            for (int s2 = 0; 2 * s2 < NC; ++s2) {
                const int c = 2 * s2 + half;
                float2 v[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) v[i] = c < NC ? ld_shared_f2(stg + (uint32_t)(8 * c + i) * 1024u)
                                                          : make_float2(0.f, 0.f);
                asm volatile("bar.sync 1, 256;" ::: "memory");
                if (c < NC) {
                    uint32_t hi[8], lo[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        __half2 a, b;
                        split_h2(v[i].x, v[i].y, a, b);
                        hi[i] = h2u(a);
                        lo[i] = h2u(b);
                    }
                    const uint32_t fc = fb + (uint32_t)c * TC_FCHUNK;
                    st_shared_v4(fc + r0, hi[0], hi[1], hi[2], hi[3]);
                    st_shared_v4(fc + r1, hi[4], hi[5], hi[6], hi[7]);
                    st_shared_v4(fc + TC_FTILE + r0, lo[0], lo[1], lo[2], lo[3]);
                    st_shared_v4(fc + TC_FTILE + r1, lo[4], lo[5], lo[6], lo[7]);
                }
            }
            // the next term's first loads, then the tiles are complete: a
            // CTA barrier (no polling), after which thread 0 issues the MMAs
            if (k + 1 < Ka) preload(k + 1);
            tc::fence_proxy_async_smem();
            asm volatile("bar.sync 1, 256;" ::: "memory");
            if (tid == 0 && !*(volatile int*)&abort_flag) {
                tc::fence_after_sync();
                issue_term(k);
            }
        }
        // arrives when every MMA issued above has completed
        if (tid == 0) tc::mma_commit(&done_bar);
        // ---- epilogue: TMEM (+ running sum) -> x-quads g2t[rot][x/4][p][x%4] ----
        float2 run_a[8], run_b[8];
        if (with_sum) load_run(0, run_a);
        if (!*(volatile int*)&abort_flag && !tc::mbar_wait(&done_bar, 0, TC_WAIT_NS)) {
            atomicOr(err, 4);
            abort_flag = 1;
        }
        tc::fence_after_sync();
#pragma unroll 1
        for (int cb = 0; cb < 8 * MT; cb += 2) {
            if (with_sum) load_run(cb + 1, run_b);
            out_block(cb, run_a);
            if (with_sum && cb + 2 < 8 * MT) load_run(cb + 2, run_a);
            out_block(cb + 1, run_b);
        }
    }
    // the MMA issuer's done barrier covers every MMA before TMEM is released
    if (tid == 0 && !tc::mbar_wait(&done_bar, 0, TC_WAIT_NS)) atomicOr(err, 16);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TM_COLS);
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

// box grids: the same per pencil p < nh over samples d < nx
static __global__ void circ_scale_box_kernel(const float2* __restrict__ circ, int K, int nh, int nx,
                                      int8_t* __restrict__ cscale) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nh) return;
    float m = 0.f;
    for (int t = 0; t < K; ++t)
        for (int d = 0; d < nx; ++d) {
            const float2 c = circ[((size_t)t * nh + p) * nx + d];
            m = fmaxf(m, fmaxf(fabsf(c.x), fabsf(c.y)));
        }
    int e = 0;
    if (m > 0.f) {
        int ex;
        frexpf(m, &ex);
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
