// Learned rotation proposal (no counterpart in the reference).
//
// A small network predicts, for one receptor/ligand pair and one rotation,
// the best (lowest) correlation score the FFT scan would find for that
// rotation, from a coarse occupancy grid of the rotated ligand and a
// rotation-invariant receptor descriptor.  Rotations it ranks low are skipped
// before the scan; the exhaustive scan stays the fallback and the judge of
// its recall.
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
// Precision: weights are used as BF16 copies of FP32 master weights;
// activations x0, a1, a2, a3, u, h1 are stored as BF16; every sum is
// accumulated in FP32; gradients are FP32; Adam updates the FP32 masters.
//
// Training step (captured once in a CUDA graph, replayed per step): sample
// indices come from a hash of (seed, device step counter, slot), so a replay
// needs no host input.  train_sample_kernel (forward + activation gradients,
// one CTA per sample) -> conv/fc weight-gradient reductions over the batch ->
// Adam (which advances the step counter).
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
constexpr int NA1 = C1 * D1 * D1 * D1;
constexpr int NA2 = C2 * D2 * D2 * D2;
constexpr int NA3 = C3 * D3 * D3 * D3;
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

constexpr int THREADS = 256;
constexpr int MAX_BATCH = 4096;

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
// per-sample building blocks (THREADS threads, operands in shared memory)
// ---------------------------------------------------------------------------

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

// out = relu(conv(in) + b), 3^3 taps, stride 2, pad 1; out stored as BF16
template <int CIN, int COUT, int DIN>
__device__ void conv_fwd(const bf16* __restrict__ in, const bf16* __restrict__ w, const bf16* __restrict__ b,
                         bf16* __restrict__ out) {
    constexpr int DOUT = DIN / 2, P = DOUT * DOUT * DOUT, NIN = DIN * DIN * DIN;
    for (int o = threadIdx.x; o < COUT * P; o += THREADS) {
        const int co = o / P, r = o % P;
        const int oz = r / (DOUT * DOUT), oy = (r / DOUT) % DOUT, ox = r % DOUT;
        float acc = b2f(b[co]);
        for (int ci = 0; ci < CIN; ++ci) {
            const bf16* wk = w + (co * CIN + ci) * 27;
            const bf16* ic = in + ci * NIN;
#pragma unroll
            for (int kz = 0; kz < 3; ++kz) {
                const int z = 2 * oz - 1 + kz;
                if (z < 0 || z >= DIN) continue;
#pragma unroll
                for (int ky = 0; ky < 3; ++ky) {
                    const int y = 2 * oy - 1 + ky;
                    if (y < 0 || y >= DIN) continue;
#pragma unroll
                    for (int kx = 0; kx < 3; ++kx) {
                        const int x = 2 * ox - 1 + kx;
                        if (x < 0 || x >= DIN) continue;
                        acc += b2f(wk[(kz * 3 + ky) * 3 + kx]) * b2f(ic[(z * DIN + y) * DIN + x]);
                    }
                }
            }
        }
        out[o] = f2b(acc > 0.f ? acc : 0.f);
    }
}

// dz_in = conv^T(dout) masked by act_in > 0 (the ReLU of the layer below)
template <int CIN, int COUT, int DIN>
__device__ void conv_bwd_data(const float* __restrict__ dout, const bf16* __restrict__ w,
                              const bf16* __restrict__ act_in, float* __restrict__ dz_in) {
    constexpr int DOUT = DIN / 2, P = DOUT * DOUT * DOUT, NIN = DIN * DIN * DIN;
    for (int e = threadIdx.x; e < CIN * NIN; e += THREADS) {
        const int ci = e / NIN, r = e % NIN;
        const int z = r / (DIN * DIN), y = (r / DIN) % DIN, x = r % DIN;
        float acc = 0.f;
        if (b2f(act_in[e]) > 0.f) {
            for (int kz = 0; kz < 3; ++kz) {
                const int tz = z + 1 - kz;
                if (tz < 0 || (tz & 1) || (tz >> 1) >= DOUT) continue;
                for (int ky = 0; ky < 3; ++ky) {
                    const int ty = y + 1 - ky;
                    if (ty < 0 || (ty & 1) || (ty >> 1) >= DOUT) continue;
                    for (int kx = 0; kx < 3; ++kx) {
                        const int tx = x + 1 - kx;
                        if (tx < 0 || (tx & 1) || (tx >> 1) >= DOUT) continue;
                        const int pos = ((tz >> 1) * DOUT + (ty >> 1)) * DOUT + (tx >> 1);
                        const int k = (kz * 3 + ky) * 3 + kx;
                        for (int co = 0; co < COUT; ++co) acc += b2f(w[(co * CIN + ci) * 27 + k]) * dout[co * P + pos];
                    }
                }
            }
        }
        dz_in[e] = acc;
    }
}

struct Ligands {
    const double* xyz;    // all ligands' atoms, concatenated
    const int* start;     // first atom of each ligand
    const int* count;
    const double* half;   // L of each ligand
    const float* desc;    // [n_lig][DESC]
};

// shared memory of one sample's forward pass
struct FwdSmem {
    float occ[NX0];
    bf16 x0[NX0];
    bf16 a1[NA1];
    bf16 a2[NA2];
    bf16 u[NU];
    bf16 h1[HID];
    float red[THREADS / 32];
};

// forward of one sample; returns y on every thread
__device__ float forward(const bf16* __restrict__ wb, const Ligands& lg, int lig, const double* rot, FwdSmem& s) {
    occupancy(lg.xyz + 3 * (size_t)lg.start[lig], lg.count[lig], lg.half[lig], rot, s.occ);
    for (int i = threadIdx.x; i < NX0; i += THREADS) s.x0[i] = f2b(0.25f * s.occ[i]);
    for (int i = threadIdx.x; i < DESC; i += THREADS) s.u[NA3 + i] = f2b(lg.desc[(size_t)lig * DESC + i]);
    __syncthreads();
    conv_fwd<1, C1, G0>(s.x0, wb + OW1, wb + OB1, s.a1);
    __syncthreads();
    conv_fwd<C1, C2, D1>(s.a1, wb + OW2, wb + OB2, s.a2);
    __syncthreads();
    conv_fwd<C2, C3, D2>(s.a2, wb + OW3, wb + OB3, s.u);
    __syncthreads();
    {
        const int j = threadIdx.x;  // THREADS == HID
        float acc = b2f(wb[OFB1 + j]);
        for (int i = 0; i < NU; ++i) acc += b2f(wb[OF1 + i * HID + j]) * b2f(s.u[i]);
        s.h1[j] = f2b(acc > 0.f ? acc : 0.f);
        float t = b2f(wb[OF2 + j]) * b2f(s.h1[j]);
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if ((j & 31) == 0) s.red[j >> 5] = t;
    }
    __syncthreads();
    float y = b2f(wb[OFB2]);
    for (int k = 0; k < THREADS / 32; ++k) y += s.red[k];
    return y;
}

static_assert(THREADS == HID, "one thread per hidden unit");

__global__ void __launch_bounds__(THREADS) predict_kernel(const bf16* __restrict__ wb, Ligands lg, int lig,
                                                          const double* __restrict__ rot, int n,
                                                          float* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FwdSmem& s = *reinterpret_cast<FwdSmem*>(smem_raw);
    const int b = blockIdx.x;
    if (b >= n) return;
    const float y = forward(wb, lg, lig, rot + 9 * (size_t)b, s);
    if (threadIdx.x == 0) out[b] = y;
}

// activations and activation gradients of a batch, kept for the weight
// gradients
struct Store {
    bf16* x0;     // [B][NX0]
    bf16* a1;     // [B][NA1]
    bf16* a2;     // [B][NA2]
    bf16* u;      // [B][NU]
    bf16* h1;     // [B][HID]
    float* dz1;   // [B][NA1]
    float* dz2;   // [B][NA2]
    float* dz3;   // [B][NA3]
    float* dzf;   // [B][HID]
    float* dy;    // [B]
};

struct Samples {
    const int* lig;        // [n]
    const double* rot;     // [n][9]
    const float* target;   // [n]
    int n;
};

struct TrainSmem {
    FwdSmem f;
    float dzf[HID];
    float dz3[NA3];
    float dz2[NA2];
};

// one sample of a training batch: forward, loss, activation gradients.
// explicit >= 0: sample b is explicit + b (no sampling)
__global__ void __launch_bounds__(THREADS) train_sample_kernel(const bf16* __restrict__ wb, Ligands lg, Samples sm,
                                                               const uint32_t* __restrict__ step_ctr, uint64_t seed,
                                                               int batch, int explicit_base, Store st,
                                                               double* __restrict__ loss_acc) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>(smem_raw);
    const int b = blockIdx.x;
    int idx;
    if (explicit_base >= 0) {
        idx = explicit_base + b;
    } else {
        const uint64_t h = mix64(seed ^ mix64(((uint64_t)(*step_ctr) << 20) ^ (uint64_t)b));
        idx = (int)(h % (uint64_t)sm.n);
    }
    const int lig = sm.lig[idx];
    const float y = forward(wb, lg, lig, sm.rot + 9 * (size_t)idx, s.f);
    const float t = sm.target[idx];
    const float dy = 2.f * (y - t) / (float)batch;
    const int tid = threadIdx.x;
    if (tid == 0) {
        st.dy[b] = dy;
        atomicAdd(loss_acc, (double)((y - t) * (y - t)) / (double)batch);
    }
    // dz of the hidden layer (ReLU mask from h1)
    {
        const int j = tid;
        const float g = b2f(s.f.h1[j]) > 0.f ? dy * b2f(wb[OF2 + j]) : 0.f;
        s.dzf[j] = g;
        st.dzf[(size_t)b * HID + j] = g;
    }
    __syncthreads();
    // du for the conv features, masked by a3 > 0: one warp per input row
    {
        const int w = tid >> 5, l = tid & 31;
        for (int i = w; i < NA3; i += THREADS / 32) {
            float acc = 0.f;
            for (int j = l; j < HID; j += 32) acc += b2f(wb[OF1 + i * HID + j]) * s.dzf[j];
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (l == 0) s.dz3[i] = b2f(s.f.u[i]) > 0.f ? acc : 0.f;
        }
    }
    __syncthreads();
    conv_bwd_data<C2, C3, D2>(s.dz3, wb + OW3, s.f.a2, s.dz2);
    __syncthreads();
    // dz1 goes straight to global memory
    conv_bwd_data<C1, C2, D1>(s.dz2, wb + OW2, s.f.a1, st.dz1 + (size_t)b * NA1);
    // stores for the weight gradients
    for (int i = tid; i < NX0; i += THREADS) st.x0[(size_t)b * NX0 + i] = s.f.x0[i];
    for (int i = tid; i < NA1; i += THREADS) st.a1[(size_t)b * NA1 + i] = s.f.a1[i];
    for (int i = tid; i < NA2; i += THREADS) {
        st.a2[(size_t)b * NA2 + i] = s.f.a2[i];
        st.dz2[(size_t)b * NA2 + i] = s.dz2[i];
    }
    for (int i = tid; i < NU; i += THREADS) st.u[(size_t)b * NU + i] = s.f.u[i];
    for (int i = tid; i < NA3; i += THREADS) st.dz3[(size_t)b * NA3 + i] = s.dz3[i];
    st.h1[(size_t)b * HID + tid] = s.f.h1[tid];
}

// dW[co][ci][27] and db[co] of a conv layer, reduced over the batch; one
// CTA per (co, ci)
template <int CIN, int COUT, int DIN>
__global__ void __launch_bounds__(THREADS) conv_wgrad_kernel(const bf16* __restrict__ act_in,
                                                             const float* __restrict__ dz, int B,
                                                             float* __restrict__ gw, float* __restrict__ gb) {
    constexpr int DOUT = DIN / 2, P = DOUT * DOUT * DOUT, NIN = DIN * DIN * DIN;
    __shared__ float red[28][THREADS / 32];
    const int co = blockIdx.x / CIN, ci = blockIdx.x % CIN;
    float acc[28];
#pragma unroll
    for (int k = 0; k < 28; ++k) acc[k] = 0.f;
    for (int idx = threadIdx.x; idx < B * P; idx += THREADS) {
        const int s = idx / P, pos = idx % P;
        const float g = dz[((size_t)s * COUT + co) * P + pos];
        if (g == 0.f) continue;
        const int oz = pos / (DOUT * DOUT), oy = (pos / DOUT) % DOUT, ox = pos % DOUT;
        const bf16* ic = act_in + ((size_t)s * CIN + ci) * NIN;
#pragma unroll
        for (int kz = 0; kz < 3; ++kz) {
            const int z = 2 * oz - 1 + kz;
#pragma unroll
            for (int ky = 0; ky < 3; ++ky) {
                const int y = 2 * oy - 1 + ky;
#pragma unroll
                for (int kx = 0; kx < 3; ++kx) {
                    const int x = 2 * ox - 1 + kx;
                    if (z >= 0 && z < DIN && y >= 0 && y < DIN && x >= 0 && x < DIN)
                        acc[(kz * 3 + ky) * 3 + kx] += g * b2f(ic[(z * DIN + y) * DIN + x]);
                }
            }
        }
        acc[27] += g;
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 28; ++k) {
        float v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (l == 0) red[k][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < 28) {
        float v = 0.f;
        for (int k = 0; k < THREADS / 32; ++k) v += red[threadIdx.x][k];
        if (threadIdx.x < 27) gw[(co * CIN + ci) * 27 + threadIdx.x] = v;
        else if (ci == 0) gb[co] = v;
    }
}

// fully connected gradients: blocks 0..NU-1 give dW1[i][*] (block 0 also
// db1), block NU gives dw2 and db2
__global__ void __launch_bounds__(THREADS) fc_wgrad_kernel(Store st, int B, float* __restrict__ g) {
    const int j = threadIdx.x;
    if (blockIdx.x < NU) {
        const int i = blockIdx.x;
        float acc = 0.f, accb = 0.f;
        for (int s = 0; s < B; ++s) {
            const float d = st.dzf[(size_t)s * HID + j];
            acc += b2f(st.u[(size_t)s * NU + i]) * d;
            accb += d;
        }
        g[OF1 + i * HID + j] = acc;
        if (i == 0) g[OFB1 + j] = accb;
    } else {
        float acc = 0.f;
        for (int s = 0; s < B; ++s) acc += b2f(st.h1[(size_t)s * HID + j]) * st.dy[s];
        g[OF2 + j] = acc;
        if (j == 0) {
            float d = 0.f;
            for (int s = 0; s < B; ++s) d += st.dy[s];
            g[OFB2] = d;
        }
    }
}

// Adam on the FP32 masters (bias-corrected), BF16 copies refreshed; the last
// thread of the grid advances the step counter
__global__ void adam_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, bf16* __restrict__ wb, uint32_t* __restrict__ step_ctr,
                            float lr, float b1, float b2, float eps) {
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
        wb[i] = f2b(wi);
    }
}

__global__ void step_advance_kernel(uint32_t* step_ctr) { *step_ctr += 1u; }

__global__ void to_bf16_kernel(const float* __restrict__ w, bf16* __restrict__ wb, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wb[i] = f2b(w[i]);
}

template <typename T> cudaError_t dalloc(T** p, size_t n) {
    *p = nullptr;
    return cudaMalloc((void**)p, (n ? n : 1) * sizeof(T));
}
template <typename T> void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

}  // namespace

struct fftdock_proposal {
    int device = 0;
    std::string err;
    cudaStream_t stream = nullptr;
    // parameters
    float* w = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* g = nullptr;
    bf16* wb = nullptr;
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
    int cap_batch = 0;
    Store st{};
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

int sync_ligands(fftdock_proposal* p) {
    if (!p->lig_dirty) return FFTDOCK_OK;
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
    if (p->graph) {
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
    return FFTDOCK_OK;
}

int sync_samples(fftdock_proposal* p) {
    if (!p->samples_dirty) return FFTDOCK_OK;
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
    if (p->graph) {
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
    return FFTDOCK_OK;
}

void free_store(Store& s) {
    dfree(s.x0);
    dfree(s.a1);
    dfree(s.a2);
    dfree(s.u);
    dfree(s.h1);
    dfree(s.dz1);
    dfree(s.dz2);
    dfree(s.dz3);
    dfree(s.dzf);
    dfree(s.dy);
}

int grow_store(fftdock_proposal* p, int B) {
    if (B <= p->cap_batch) return FFTDOCK_OK;
    free_store(p->st);
    p->cap_batch = 0;
    Store& s = p->st;
    PK(dalloc(&s.x0, (size_t)B * NX0));
    PK(dalloc(&s.a1, (size_t)B * NA1));
    PK(dalloc(&s.a2, (size_t)B * NA2));
    PK(dalloc(&s.u, (size_t)B * NU));
    PK(dalloc(&s.h1, (size_t)B * HID));
    PK(dalloc(&s.dz1, (size_t)B * NA1));
    PK(dalloc(&s.dz2, (size_t)B * NA2));
    PK(dalloc(&s.dz3, (size_t)B * NA3));
    PK(dalloc(&s.dzf, (size_t)B * HID));
    PK(dalloc(&s.dy, (size_t)B));
    p->cap_batch = B;
    if (p->graph) {
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
    return FFTDOCK_OK;
}

cudaError_t set_smem_attr() {
    static std::once_flag once;
    static cudaError_t res = cudaSuccess;
    std::call_once(once, [] {
        res = cudaFuncSetAttribute((const void*)predict_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)sizeof(FwdSmem));
        if (res == cudaSuccess)
            res = cudaFuncSetAttribute((const void*)train_sample_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TrainSmem));
    });
    return res;
}

// the batch's forward/backward and the weight gradients (no update)
cudaError_t launch_gradients(fftdock_proposal* p, int B, uint64_t seed, int explicit_base, Samples sm,
                             cudaStream_t s) {
    train_sample_kernel<<<B, THREADS, sizeof(TrainSmem), s>>>(p->wb, ligands(p), sm, p->step, seed, B, explicit_base,
                                                               p->st, p->loss);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    conv_wgrad_kernel<1, C1, G0><<<C1 * 1, THREADS, 0, s>>>(p->st.x0, p->st.dz1, B, p->g + OW1, p->g + OB1);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    conv_wgrad_kernel<C1, C2, D1><<<C2 * C1, THREADS, 0, s>>>(p->st.a1, p->st.dz2, B, p->g + OW2, p->g + OB2);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    conv_wgrad_kernel<C2, C3, D2><<<C3 * C2, THREADS, 0, s>>>(p->st.a2, p->st.dz3, B, p->g + OW3, p->g + OB3);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    fc_wgrad_kernel<<<NU + 1, THREADS, 0, s>>>(p->st, B, p->g);
    return cudaGetLastError();
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
    PK(set_smem_attr());
    PK(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    PK(dalloc(&p->w, NPARAM));
    PK(dalloc(&p->m, NPARAM));
    PK(dalloc(&p->v, NPARAM));
    PK(dalloc(&p->g, NPARAM));
    PK(dalloc(&p->wb, NPARAM));
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
    to_bf16_kernel<<<(NPARAM + 255) / 256, 256, 0, p->stream>>>(p->w, p->wb, NPARAM);
    PK(cudaGetLastError());
    PK(cudaStreamSynchronize(p->stream));
    return FFTDOCK_OK;
}

void fftdock_proposal_destroy(fftdock_proposal* p) {
    if (!p) return;
    if (p->graph) cudaGraphExecDestroy(p->graph);
    dfree(p->w);
    dfree(p->m);
    dfree(p->v);
    dfree(p->g);
    dfree(p->wb);
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
    free_store(p->st);
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
    to_bf16_kernel<<<(NPARAM + 255) / 256, 256, 0, p->stream>>>(p->w, p->wb, NPARAM);
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
    if ((rc = sync_ligands(p)) || (rc = sync_samples(p)) || (rc = grow_store(p, batch))) return rc;
    if (p->n_dev_samples < 1) return pfail(p, FFTDOCK_ESTATE, "no training samples");
    if (p->graph && (p->graph_batch != batch || p->graph_lr != lr || p->graph_seed != seed)) {
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
    cudaStream_t s = p->stream;
    if (!p->graph) {
        Samples sm{p->s_lig, p->s_rot, p->s_target, p->n_dev_samples};
        cudaGraph_t g = nullptr;
        PK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = launch_gradients(p, batch, seed, -1, sm, s);
        if (e == cudaSuccess) {
            adam_kernel<<<(NPARAM + 255) / 256, 256, 0, s>>>(p->w, p->m, p->v, p->g, p->wb, p->step, lr, 0.9f,
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
    if ((rc = sync_ligands(p)) || (rc = grow_store(p, n))) return rc;
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
    if (e == cudaSuccess) e = launch_gradients(p, n, 0, 0, Samples{d_lig, d_rot, d_t, n}, s);
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
    cudaStream_t s = stream ? (cudaStream_t)stream : p->stream;
    if (stream) {
        // parameters may still be in flight on the library's own stream
        PK(cudaStreamSynchronize(p->stream));
    }
    predict_kernel<<<n, THREADS, sizeof(FwdSmem), s>>>(p->wb, ligands(p), lig, d_rot, n, d_out);
    PK(cudaGetLastError());
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
