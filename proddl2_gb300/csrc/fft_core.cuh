// Shared FFT building blocks for the correlation-scan kernels.
//
// Every 1-D transform of length N in this library is a two-pass Stockham
// decomposition N = R1 * G executed by G warps, one line per lane:
//   pass 1: warp w holds the line's elements x = w + G*r (r < R1) in
//           registers and does one radix-R1 DFT in registers;
//   exchange through shared memory (one element per (position, lane));
//   pass 2: warp w does R1/G radix-G butterflies j = w + G*i, twiddled by
//           w_N^(j*r), leaving X[j + R1*k2] in registers.
// Requires G*G | N so that R1 is a multiple of G.  The output distribution
// (thread w holds k = w mod G) is exactly the input distribution of the next
// transform's pass 1, which is what lets the scan kernels chain
// forward transform -> spectrum multiply -> inverse transform in registers.
//
// Sign convention: SIGN = -1 is the forward DFT X[k] = sum x[n] e^{-2 pi i nk/N},
// SIGN = +1 the unnormalised inverse.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

namespace fftdock {

// ---------------------------------------------------------------------------
// complex helpers (float2 / double2)
// ---------------------------------------------------------------------------
template <typename T> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };
template <typename T> using cplx_t = typename cplx<T>::type;

template <typename C> __host__ __device__ __forceinline__ C cmake(double re, double im) {
    C r; r.x = (decltype(r.x))re; r.y = (decltype(r.y))im; return r;
}
__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 operator-(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
// a * conj(b)
template <typename C> __device__ __forceinline__ C cmul_conj(C a, C b) {
    C r; r.x = a.x * b.x + a.y * b.y; r.y = a.y * b.x - a.x * b.y; return r;
}
// multiply by w or conj(w) depending on SIGN (tables hold e^{-2 pi i k/N})
template <int SIGN, typename C> __device__ __forceinline__ C ctwiddle(C a, C w) {
    if constexpr (SIGN < 0) return cmul(a, w); else return cmul_conj(a, w);
}
// multiply by i*SIGN
template <int SIGN, typename C> __device__ __forceinline__ C mul_isign(C a) {
    C r;
    if constexpr (SIGN < 0) { r.x = a.y; r.y = -a.x; }   // * (-i)
    else { r.x = -a.y; r.y = a.x; }                       // * (+i)
    return r;
}
template <typename C, typename S> __device__ __forceinline__ C cscale(C a, S s) {
    C r; r.x = a.x * s; r.y = a.y * s; return r;
}

// ---------------------------------------------------------------------------
// compile-time trigonometry: cos/sin(2 pi m / R) by exact quadrant reduction
// and a Taylor series on [0, pi/2] (converges to double precision).
// ---------------------------------------------------------------------------
constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double taylor_sin(double x) {
    double term = x, sum = x;
    for (int i = 1; i < 16; ++i) { term *= -x * x / ((2.0 * i) * (2.0 * i + 1.0)); sum += term; }
    return sum;
}
constexpr double taylor_cos(double x) {
    double term = 1.0, sum = 1.0;
    for (int i = 1; i < 16; ++i) { term *= -x * x / ((2.0 * i - 1.0) * (2.0 * i)); sum += term; }
    return sum;
}
constexpr double cos2pi(long m, long r) {
    m %= r; if (m < 0) m += r;
    const long q = (4 * m) / r;
    const long rem = 4 * m - q * r;
    const double phi = (kPi / 2.0) * ((double)rem / (double)r);
    const double c = taylor_cos(phi), s = taylor_sin(phi);
    return q == 0 ? c : q == 1 ? -s : q == 2 ? -c : s;
}
constexpr double sin2pi(long m, long r) {
    m %= r; if (m < 0) m += r;
    const long q = (4 * m) / r;
    const long rem = 4 * m - q * r;
    const double phi = (kPi / 2.0) * ((double)rem / (double)r);
    const double c = taylor_cos(phi), s = taylor_sin(phi);
    return q == 0 ? s : q == 1 ? c : q == 2 ? -s : -c;
}

constexpr int smallest_factor(int r) {
    return (r % 4 == 0 && r != 8) ? 4 : (r % 2 == 0) ? 2 : (r % 3 == 0) ? 3 : (r % 5 == 0) ? 5 : (r % 7 == 0) ? 7 : r;
}

// ---------------------------------------------------------------------------
// In-register DFT of length R on v[OFF + STRIDE*n], n < R (natural order in
// and out).  Small radices are written out; composite radices recurse by
// decimation in time R = A * B.
// ---------------------------------------------------------------------------
template <int R, int SIGN, int OFF = 0, int STRIDE = 1> struct Dft;

template <int SIGN, int OFF, int STRIDE> struct Dft<1, SIGN, OFF, STRIDE> {
    template <typename C> __device__ __forceinline__ static void run(C*) {}
};

template <int SIGN, int OFF, int STRIDE> struct Dft<2, SIGN, OFF, STRIDE> {
    template <typename C> __device__ __forceinline__ static void run(C* v) {
        C a = v[OFF], b = v[OFF + STRIDE];
        v[OFF] = a + b; v[OFF + STRIDE] = a - b;
    }
};

template <int SIGN, int OFF, int STRIDE> struct Dft<3, SIGN, OFF, STRIDE> {
    template <typename C> __device__ __forceinline__ static void run(C* v) {
        using T = decltype(v[0].x);
        constexpr double c = -0.5;
        constexpr double s = 0.86602540378443864676372317075293618;  // sin(2 pi / 3)
        C x0 = v[OFF], x1 = v[OFF + STRIDE], x2 = v[OFF + 2 * STRIDE];
        C t = x1 + x2, u = x1 - x2;
        C m = x0 + cscale(t, (T)c);
        C is = mul_isign<SIGN>(cscale(u, (T)s));
        v[OFF] = x0 + t;
        v[OFF + STRIDE] = m + is;
        v[OFF + 2 * STRIDE] = m - is;
    }
};

template <int SIGN, int OFF, int STRIDE> struct Dft<4, SIGN, OFF, STRIDE> {
    template <typename C> __device__ __forceinline__ static void run(C* v) {
        C x0 = v[OFF], x1 = v[OFF + STRIDE], x2 = v[OFF + 2 * STRIDE], x3 = v[OFF + 3 * STRIDE];
        C a = x0 + x2, b = x0 - x2, c = x1 + x3, d = mul_isign<SIGN>(x1 - x3);
        v[OFF] = a + c;
        v[OFF + 2 * STRIDE] = a - c;
        v[OFF + STRIDE] = b + d;
        v[OFF + 3 * STRIDE] = b - d;
    }
};

// cos/sin(2 pi M / R) as constants evaluated by the compiler
template <int M, int R> struct TwC {
    static constexpr double c = cos2pi(M, R);
    static constexpr double s = sin2pi(M, R);
};

// y * exp(SIGN 2 pi i M / R): quarter turns are swaps and sign flips, eighth
// turns cost two adds and two multiplies, the rest a full complex multiply
// (IEEE rules keep the compiler from dropping products with 0 and 1 itself)
template <int SIGN, int M0, int R, typename C> __device__ __forceinline__ C twiddle_const(C y) {
    using T = decltype(y.x);
    constexpr int M = ((M0 % R) + R) % R;
    if constexpr (M == 0) {
        return y;
    } else if constexpr ((4 * M) % R == 0) {
        constexpr int q = (4 * M) / R;  // 1, 2, 3 quarter turns
        if constexpr (q == 2) {
            C r; r.x = -y.x; r.y = -y.y; return r;
        } else if constexpr ((q == 1) == (SIGN > 0)) {
            return mul_isign<+1>(y);
        } else {
            return mul_isign<-1>(y);
        }
    } else if constexpr ((8 * M) % R == 0) {
        constexpr int e = (8 * M) / R;  // 1, 3, 5, 7 eighth turns
        constexpr double h = 0.70710678118654752440084436210484903;
        constexpr double cs = (e == 1 || e == 7) ? h : -h;
        constexpr double sn = SIGN * ((e == 1 || e == 3) ? h : -h);
        C r;
        if constexpr ((cs > 0) == (sn > 0)) {  // s = c
            r.x = (T)cs * (y.x - y.y);
            r.y = (T)cs * (y.y + y.x);
        } else {                               // s = -c
            r.x = (T)cs * (y.x + y.y);
            r.y = (T)cs * (y.y - y.x);
        }
        return r;
    } else {
        C w;
        w.x = (T)TwC<M, R>::c;
        w.y = (T)(SIGN * TwC<M, R>::s);
        return cmul(y, w);
    }
}

// odd prime radix by the symmetric direct formula
template <int R, int SIGN, int OFF, int STRIDE> struct DftPrime {
    static constexpr int H = (R - 1) / 2;
    template <typename C, int K, int... Ns>
    __device__ __forceinline__ static void out_k(const C* sp, const C* sm, C x0, C* out,
                                                 std::integer_sequence<int, Ns...>) {
        using T = decltype(x0.x);
        C re = x0, im;
        im.x = 0;
        im.y = 0;
        ((re = re + cscale(sp[Ns + 1], (T)TwC<((Ns + 1) * K) % R, R>::c)), ...);
        ((im = im + cscale(sm[Ns + 1], (T)TwC<((Ns + 1) * K) % R, R>::s)), ...);
        const C ji = mul_isign<SIGN>(im);
        out[K] = re + ji;
        out[R - K] = re - ji;
    }
    template <typename C, int... Ks>
    __device__ __forceinline__ static void outs(const C* sp, const C* sm, C x0, C* out,
                                                std::integer_sequence<int, Ks...>) {
        (out_k<C, Ks + 1>(sp, sm, x0, out, std::make_integer_sequence<int, H>{}), ...);
    }
    template <typename C> __device__ __forceinline__ static void run(C* v) {
        C sp[H + 1], sm[H + 1];
        const C x0 = v[OFF];
        C tot = x0;
#pragma unroll
        for (int n = 1; n <= H; ++n) {
            sp[n] = v[OFF + n * STRIDE] + v[OFF + (R - n) * STRIDE];
            sm[n] = v[OFF + n * STRIDE] - v[OFF + (R - n) * STRIDE];
            tot = tot + sp[n];
        }
        C out[R];
        outs<C>(sp, sm, x0, out, std::make_integer_sequence<int, H>{});
        v[OFF] = tot;
#pragma unroll
        for (int k = 1; k < R; ++k) v[OFF + k * STRIDE] = out[k];
    }
};
template <int SIGN, int OFF, int STRIDE> struct Dft<5, SIGN, OFF, STRIDE> : DftPrime<5, SIGN, OFF, STRIDE> {};
template <int SIGN, int OFF, int STRIDE> struct Dft<7, SIGN, OFF, STRIDE> : DftPrime<7, SIGN, OFF, STRIDE> {};

// composite radix: R = A * B, decimation in time.
//   sub-DFTs of length B over v[OFF + STRIDE*(A*n2 + n1)] for each n1 < A,
//   twiddle by w_R^(n1*k1), then DFT_A over n1 for each k1; result X[k1 + B*k2]
//   lands in a temporary and is written back in natural order.
template <int R, int SIGN, int OFF, int STRIDE> struct DftComposite {
    static constexpr int A = smallest_factor(R);
    static constexpr int B = R / A;
    static_assert(A < R, "radix must factor over 2, 3, 4, 5, 7");
    template <int N1> struct Sub {
        template <typename C> __device__ __forceinline__ static void run(C* v) {
            Dft<B, SIGN, OFF + STRIDE * N1, STRIDE * A>::run(v);
            if constexpr (N1 + 1 < A) Sub<N1 + 1>::run(v);
        }
    };
    // output column k1: twiddle Y_{n1}[k1] by w_R^(n1 k1), DFT_A over n1,
    // X[k1 + B k2] = Z[k2]
    template <typename C, int K1, int... N1s>
    __device__ __forceinline__ static void column(const C* v, C* tmp, std::integer_sequence<int, N1s...>) {
        C z[A] = {twiddle_const<SIGN, N1s * K1, R>(v[OFF + STRIDE * (A * K1 + N1s)])...};
        Dft<A, SIGN, 0, 1>::run(z);
        ((tmp[K1 + B * N1s] = z[N1s]), ...);
    }
    template <typename C, int... K1s>
    __device__ __forceinline__ static void columns(const C* v, C* tmp, std::integer_sequence<int, K1s...>) {
        (column<C, K1s>(v, tmp, std::make_integer_sequence<int, A>{}), ...);
    }
    template <typename C> __device__ __forceinline__ static void run(C* v) {
        Sub<0>::run(v);
        // after the sub-DFTs, Y_{n1}[k1] sits at v[OFF + STRIDE*(A*k1 + n1)]
        C tmp[R];
        columns<C>(v, tmp, std::make_integer_sequence<int, B>{});
#pragma unroll
        for (int k = 0; k < R; ++k) v[OFF + STRIDE * k] = tmp[k];
    }
};
template <int R, int SIGN, int OFF, int STRIDE> struct Dft : DftComposite<R, SIGN, OFF, STRIDE> {};

template <int R, int SIGN, typename C> __device__ __forceinline__ void dft(C* v) {
    Dft<R, SIGN, 0, 1>::run(v);
}

// ---------------------------------------------------------------------------
// Two-pass line plan
// ---------------------------------------------------------------------------
template <int N_, int G_> struct LinePlan {
    static constexpr int N = N_;
    static constexpr int G = G_;
    static constexpr int R1 = N / G;
    static constexpr int NB = R1 / G;  // pass-2 butterflies per warp
    static_assert(N % G == 0 && R1 % G == 0, "two-pass plan needs G*G | N");
};

// pass 2 of a line transform from a shared buffer laid out [position][LP]
// (lane-minor, LP lanes per position).  Thread of warp w, lane column `col`,
// reads butterflies j = w + G*i and returns out[i*G + r] = X[j + R1*r].
// `tw` holds e^{-2 pi i k / (N*TWS)} for k < N*TWS; the plan's twiddle
// w_N^(j*r) is tw[TWS*j*r].
template <class P, int SIGN, int TWS, int LP, typename C>
__device__ __forceinline__ void line_pass2(const C* buf, int w, int col, const C* tw, C* out) {
#pragma unroll
    for (int i = 0; i < P::NB; ++i) {
        const int j = w + P::G * i;
        C u[P::G];
#pragma unroll
        for (int r = 0; r < P::G; ++r) {
            C a = buf[(j + r * P::R1) * LP + col];
            if (r != 0) a = ctwiddle<SIGN>(a, tw[TWS * j * r]);
            u[r] = a;
        }
        dft<P::G, SIGN>(u);
#pragma unroll
        for (int r = 0; r < P::G; ++r) out[i * P::G + r] = u[r];
    }
}

// Reorder a pass-2 output distribution (out[i*G + k2] = X[w + G*i + R1*k2])
// into the pass-1 input order of the next transform of the same length
// (v[r] = X[w + G*r]).
template <class P, typename C>
__device__ __forceinline__ void pass2_to_pass1_order(const C* out, C* v) {
#pragma unroll
    for (int i = 0; i < P::NB; ++i)
#pragma unroll
        for (int k2 = 0; k2 < P::G; ++k2) v[i + P::NB * k2] = out[i * P::G + k2];
}

}  // namespace fftdock
