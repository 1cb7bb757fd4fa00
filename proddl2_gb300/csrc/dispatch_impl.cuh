// Per-size launchers.  Included by the kernels_nXX.cu translation units, each
// of which instantiates SizeOpsImpl<N> for its grid sizes.
#pragma once

#include "internal.h"
#include "scan_kernels.cuh"
#include "pencil_tc.cuh"

namespace fftdock {

template <int N> struct SizeOpsImpl {
    static constexpr int G = SizeTraits<N>::G;
    static constexpr int H = N / 2 + 1;

    static size_t pencil_smem_w(int K, int n_ent, bool weighted) {
        return pencil_smem(K, n_ent) + (weighted ? (size_t)n_ent * sizeof(float) : 0);
    }
    static size_t pencil_smem(int K, int n_ent) {
        return (size_t)PencilTraits<N>::BUFS * N * 32 * sizeof(float2) + (size_t)N * 17 * sizeof(float2) +
               ((size_t)K * N + 1) * sizeof(int32_t) +
               (size_t)n_ent * sizeof(uint32_t);
    }
    static size_t plane_smem() { return (size_t)N * H * sizeof(float2) + N * sizeof(float2) + (size_t)G * KC * 8; }
    template <typename T> static size_t line_smem() { return (size_t)(N * 32 + N) * sizeof(cplx_t<T>); }

    static cudaError_t set_smem(const void* fn, size_t bytes) {
        if (bytes <= 48 * 1024) return cudaSuccess;
        return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    }

    template <typename T, int SIGN>
    static cudaError_t line_fft(cplx_t<T>* data, const cplx_t<T>* tw, long n_lines, long elem_stride,
                                long inner_count, long inner_stride, long outer_stride, cudaStream_t s) {
        const size_t sm = line_smem<T>();
        cudaError_t e = set_smem((const void*)line_fft_kernel<T, N, SIGN>, sm);
        if (e != cudaSuccess) return e;
        const long blocks = (n_lines + 31) / 32;
        line_fft_kernel<T, N, SIGN><<<(unsigned)blocks, 32 * G, sm, s>>>(data, tw, n_lines, elem_stride,
                                                                        inner_count, inner_stride, outer_stride);
        return cudaGetLastError();
    }

    // the tensor pencil stage: one 128-row x tile up to 128, two up to 256
    static constexpr bool kHasTc = N <= 256;


    static cudaError_t circ_scales(const float2* circ, int K, int8_t* cscale, cudaStream_t s) {
        if constexpr (kHasTc) {
            const int nh = N * H;
            circ_scale_kernel<N><<<(nh + 127) / 128, 128, 0, s>>>(circ, K, cscale);
            return cudaGetLastError();
        } else {
            return cudaErrorNotSupported;
        }
    }

    static cudaError_t receptor_fft(const double* rgrid_t, double2* cbuf, double2* hbuf, const double2* tw64,
                                    void* spec_t, int spec_bf16, int PP, float2* circ_t, cudaStream_t s) {
        const size_t V = (size_t)N * N * N;
        complexify_kernel<<<(unsigned)((V + 255) / 256), 256, 0, s>>>(rgrid_t, cbuf, V);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        // z: lines (x, y), contiguous elements
        e = line_fft<double, -1>(cbuf, tw64, (long)N * N, 1, N, N, (long)N * N, s);
        if (e != cudaSuccess) return e;
        const size_t NHt = (size_t)N * N * H;
        half_extract_kernel<<<(unsigned)((NHt + 255) / 256), 256, 0, s>>>(cbuf, hbuf, N, H);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        // y: lines (x, kz) of [N][N][H]
        e = line_fft<double, -1>(hbuf, tw64, (long)N * H, H, H, 1, (long)N * H, s);
        if (e != cudaSuccess) return e;
        if (circ_t) {
            // receptor transformed along z and y only: circulant samples of the tensor path
            const size_t tot = (size_t)N * N * H;
            pack_circ_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(hbuf, circ_t, N, N * H,
                                                                         1.0 / ((double)N * N));
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        // x: lines p = (ky, kz)
        e = line_fft<double, -1>(hbuf, tw64, (long)N * H, (long)N * H, (long)N * H, 1, 0, s);
        if (e != cudaSuccess) return e;
        const size_t tot = (size_t)N * PP;
        if (spec_bf16)
            pack_spectrum_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(
                hbuf, static_cast<__nv_bfloat162*>(spec_t), N, N * H, PP, 1.0 / (double)V);
        else
            pack_spectrum_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(
                hbuf, static_cast<float2*>(spec_t), N, N * H, PP, 1.0 / (double)V);
        return cudaGetLastError();
    }

    template <typename SpecT, bool W> static cudaError_t launch_pencil(const BatchArgs& a, int nb, cudaStream_t s) {
        const size_t sm2 = pencil_smem_w(a.K, a.n_ent, W);
        cudaError_t e = set_smem((const void*)pencil_kernel<N, SpecT, W>, sm2);
        if (e != cudaSuccess) return e;
        dim3 grid2(nb, a.PP / 32);
        pencil_kernel<N, SpecT, W><<<grid2, 32 * G, sm2, s>>>(static_cast<const SpecT*>(a.spec), a.ent, a.offs,
                                                              a.tw32, a.g2, a.K, a.n_ent, a.ent_w);
        return cudaGetLastError();
    }

    template <bool DBG, bool QUAD>
    static cudaError_t launch_plane(dim3 grid, size_t sm, const float2* src, const BatchArgs& a, float* corr,
                                    cudaStream_t s) {
        cudaError_t e = set_smem((const void*)plane_kernel<N, DBG, QUAD>, sm);
        if (e != cudaSuccess) return e;
        if constexpr (QUAD) {
            // clusters of 4 CTAs along x (the planes of one x-quad)
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = grid;
            cfg.blockDim = dim3(32 * G);
            cfg.dynamicSmemBytes = sm;
            cfg.stream = s;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = 4;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            return cudaLaunchKernelEx(&cfg, plane_kernel<N, DBG, QUAD>, src, (const float2*)a.tw32, a.cand_v,
                                      a.cand_i, corr);
        } else {
            plane_kernel<N, DBG, QUAD><<<grid, 32 * G, sm, s>>>(src, a.tw32, a.cand_v, a.cand_i, corr);
            return cudaGetLastError();
        }
    }
    template <bool QUAD>
    static cudaError_t plane(dim3 grid, size_t sm, const float2* src, const BatchArgs& a, float* corr,
                             cudaStream_t s) {
        return corr ? launch_plane<true, QUAD>(grid, sm, src, a, corr, s)
                    : launch_plane<false, QUAD>(grid, sm, src, a, nullptr, s);
    }

    // K1 over a.n_rot rotations
    static cudaError_t prep(const BatchArgs& a, cudaStream_t s) {
        const int nb = a.n_rot;
        if (nb <= 0) return cudaSuccess;
        const Geo geo = make_geo(a.h, N, N, N);
        const size_t sm1 = ((size_t)a.K * N + 1) * sizeof(int32_t) + (size_t)a.n_ent * sizeof(uint32_t);
        cudaError_t e = set_smem((const void*)ligand_prep_kernel<N>, sm1);
        if (e != cudaSuccess) return e;
        ligand_prep_kernel<N><<<nb, 256, sm1, s>>>(a.rot, a.lig_xyz, a.lig_term, a.n_ent, a.K, geo, a.ent, a.offs,
                                                    a.status, a.lig_w32, a.lig_w32 ? a.ent_w : nullptr, a.ent_idx,
                                                    a.use_tc ? a.ent_t : nullptr, a.tpad, a.n_pad, a.x0,
                                                    a.W);
        return cudaGetLastError();
    }

    // K2 + K3 over a.n_rot rotations (and, on the queue + clustering path,
    // the selection that writes the peaks).  a.ev (optional): events recorded
    // before K2, between K2 and K3, after K3 and after the clustering stage.
    static cudaError_t middle(const BatchArgs& a, cudaStream_t s) {
        const int nb = a.n_rot;
        if (nb <= 0) return cudaSuccess;
        cudaError_t e;
        if (a.ev && (e = cudaEventRecord(a.ev[0], s)) != cudaSuccess) return e;
        bool tc = false;
        if constexpr (kHasTc) {
            if (a.use_tc) {
                tc = true;
                const size_t smt = tc_smem_bytes(N, a.W / 8, a.n_tc_terms);
                constexpr int MT = tc_tiles(N);
                if ((e = set_smem((const void*)pencil_tc_kernel<N, MT>, smt)) != cudaSuccess) return e;
                dim3 gridt(N * H, (nb + TC_ROT - 1) / TC_ROT);
                const int tg = a.tc_group > 0 ? a.tc_group : FFTDOCK_TC_TERMS_PER_SUM_DEFAULT;
                pencil_tc_kernel<N, MT><<<gridt, TC_THREADS, smt, s>>>(a.circ, a.cscale, a.ent_t, a.tinfo,
                                                                      a.n_tc_terms, a.tw32, a.g2t, a.n_pad, nb, a.x0,
                                                                      a.W, tg, a.tc_slots, a.tc_n_slots, TcBox{},
                                                                      a.err);
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
            }
        }
        if (!tc) {
            if (a.lig_w32) {
                if (a.spec_bf16) return cudaErrorNotSupported;  // weighted sets run with FP32 spectra
                e = launch_pencil<float2, true>(a, nb, s);
            } else {
                e = a.spec_bf16 ? launch_pencil<__nv_bfloat162, false>(a, nb, s) : launch_pencil<float2, false>(a, nb, s);
            }
            if (e != cudaSuccess) return e;
        }
        if (a.ev && (e = cudaEventRecord(a.ev[1], s)) != cudaSuccess) return e;
        // K3 (the queue + clustering path also writes every correlation grid)
        const size_t sm3 = plane_smem();
        dim3 grid3(N, nb);
        float* corr = a.dbg_corr ? a.dbg_corr : a.wide.corr;
        if constexpr (kHasTc) {
            if (tc) e = plane<true>(grid3, sm3, a.g2t, a, corr, s);  // the tensor stage's x-quads
        }
        if (!tc) e = plane<false>(grid3, sm3, a.g2, a, corr, s);
        if (e != cudaSuccess) return e;
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if (a.ev && (e = cudaEventRecord(a.ev[2], s)) != cudaSuccess) return e;
        if (a.wide.corr) {
            BatchArgs w = a;
            w.wide.corr = corr;
            if ((e = wide_select_batch(w, N, s)) != cudaSuccess) return e;
            if (a.ev && (e = cudaEventRecord(a.ev[3], s)) != cudaSuccess) return e;
        }
        return cudaSuccess;
    }

    // K4 over a.n_rot rotations (not on the queue + clustering path)
    static cudaError_t finish(const BatchArgs& a, cudaStream_t s) {
        const int nb = a.n_rot;
        if (nb <= 0 || a.wide.corr) return cudaSuccess;
        finalize_kernel<N><<<nb, 256, 0, s>>>(a.cand_v, a.cand_i, a.ent, a.status, a.rgrid, a.n_ent, a.peak_stride,
                                              a.k_out, a.max_val, a.h, a.first_rot_id, a.peaks, a.n_peaks,
                                              a.pool_v, a.pool_i, a.lig_w64, a.lig_w64 ? a.ent_idx : nullptr);
        return cudaGetLastError();
    }

    // the whole pipeline for one batch (work buffers sized for a.n_rot)
    static cudaError_t scan_batch(const BatchArgs& a, cudaStream_t s) {
        cudaError_t e = prep(a, s);
        if (e != cudaSuccess) return e;
        BatchArgs m = a;
        m.ev = nullptr;
        if ((e = middle(m, s)) != cudaSuccess) return e;
        return finish(a, s);
    }

    // cudaFuncGetAttributes loads a kernel's code under lazy module loading
    static cudaError_t load_fft_form(int spec_bf16) {
        cudaFuncAttributes fa;
        cudaError_t e = cudaFuncGetAttributes(&fa, (const void*)ligand_prep_kernel<N>);
        if (e == cudaSuccess)
            e = spec_bf16 ? cudaFuncGetAttributes(&fa, (const void*)pencil_kernel<N, __nv_bfloat162, false>)
                          : cudaFuncGetAttributes(&fa, (const void*)pencil_kernel<N, float2, false>);
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void*)plane_kernel<N, false, false>);
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void*)finalize_kernel<N>);
        return e;
    }

    static const SizeOps* ops() {
        static const SizeOps o{N, &receptor_fft, &circ_scales, kHasTc, &scan_batch, &pencil_smem, &prep, &middle,
                               &finish, &load_fft_form};
        return &o;
    }
};

}  // namespace fftdock
