// Compile-time Stockham FFT of many lines held in shared memory.
//
// Same decimation-in-time Stockham stage as fft_core.cuh, but the line
// length N and its radix schedule are template parameters, so every index
// computation (butterfly position, twiddle index, output slot) folds to
// constant shifts and multiplies, and the stage loops unroll.
//
// Threads: TPL = N / R0 threads per line (R0 = first radix); a stage of
// radix r has N / r butterflies, i.e. ceil((N/r) / TPL) per thread.
//
// Shared-memory line buffers are line-major with an XOR swizzle inside each
// 128-byte group:  element j of line l sits at  l*NP + (j ^ (((j >> S) ^ l) & M))
// (S, M = 4, 15 for 8-byte complex; 3, 7 for 16-byte complex; NP = N rounded
// up to a multiple of M+1).  The XOR only permutes elements inside their own
// group, so every address stays inside [l*NP, (l+1)*NP).  It spreads the
// stride-r Stockham writes and the column-tile transposes over all banks.
#pragma once
#include "fft_core.cuh"

namespace gbct {

using gbfft::dft2;
using gbfft::dft3;
using gbfft::dft4;
using gbfft::dft5;
using gbfft::dft8;

template <typename T> struct Swz;
template <> struct Swz<float> { static constexpr int S = 4, M = 15; };
template <> struct Swz<double> { static constexpr int S = 3, M = 7; };

template <typename T, int N> struct Pad {
  static constexpr int G = Swz<T>::M + 1;
  static constexpr int NP = (N + G - 1) / G * G;
};

template <typename T, int NP>
__device__ __forceinline__ int sw(int l, int j) {
  return l * NP + (j ^ (((j >> Swz<T>::S) ^ l) & Swz<T>::M));
}

template <int... Rs> struct Sched {};

// radix schedules (first radix sets threads per line)
template <int N> struct Plan;
template <> struct Plan<32> { using S = Sched<8, 4>; static constexpr int R0 = 8; };
template <> struct Plan<64> { using S = Sched<8, 8>; static constexpr int R0 = 8; };
template <> struct Plan<96> { using S = Sched<8, 4, 3>; static constexpr int R0 = 8; };
#ifndef GB_CT_R16_128
#define GB_CT_R16_128 0
#endif
#if GB_CT_R16_128
template <> struct Plan<128> { using S = Sched<16, 8>; static constexpr int R0 = 16; };
#else
template <> struct Plan<128> { using S = Sched<8, 4, 4>; static constexpr int R0 = 8; };
#endif
template <> struct Plan<160> { using S = Sched<8, 4, 5>; static constexpr int R0 = 8; };
template <> struct Plan<256> { using S = Sched<8, 8, 4>; static constexpr int R0 = 8; };
template <> struct Plan<360> { using S = Sched<8, 5, 3, 3>; static constexpr int R0 = 8; };

template <int N> struct Tpl { static constexpr int value = N / Plan<N>::R0; };

// 16-point DFT as 4 x 4: four stride-4 DFT4s, twiddles W16^(m k1), then a
// DFT4 across them (X[k1 + 4 k2]); W16 = exp(DIR 2 pi i / 16).
template <int DIR, typename T>
__device__ __forceinline__ void dft16(cpx<T>* u) {
  const T c = (T)0.92387953251128675613;   // cos(pi / 8)
  const T s = (T)0.38268343236508977173;   // sin(pi / 8)
  const T h = (T)GB_R2;
  const T d = DIR < 0 ? (T)-1 : (T)1;
  const cpx<T> w1 = {c, d * s}, w2 = {h, d * h}, w3 = {s, d * c}, w6 = {-h, d * h}, w9 = {-c, -d * s};
  cpx<T> q[4][4];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
#pragma unroll
    for (int j = 0; j < 4; ++j) q[m][j] = u[m + 4 * j];
    dft4<DIR, T>(q[m]);
  }
  q[1][1] = c_mul(q[1][1], w1);
  q[1][2] = c_mul(q[1][2], w2);
  q[1][3] = c_mul(q[1][3], w3);
  q[2][1] = c_mul(q[2][1], w2);
  q[2][2] = c_rot<DIR>(q[2][2]);
  q[2][3] = c_mul(q[2][3], w6);
  q[3][1] = c_mul(q[3][1], w3);
  q[3][2] = c_mul(q[3][2], w6);
  q[3][3] = c_mul(q[3][3], w9);
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    cpx<T> e[4] = {q[0][k1], q[1][k1], q[2][k1], q[3][k1]};
    dft4<DIR, T>(e);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) u[k1 + 4 * k2] = e[k2];
  }
}

template <int DIR, typename T, int R>
__device__ __forceinline__ void dft(cpx<T>* u) {
  if constexpr (R == 2) dft2<DIR, T>(u);
  else if constexpr (R == 3) dft3<DIR, T>(u);
  else if constexpr (R == 4) dft4<DIR, T>(u);
  else if constexpr (R == 5) dft5<DIR, T>(u);
  else if constexpr (R == 8) dft8<DIR, T>(u);
  else if constexpr (R == 16) dft16<DIR, T>(u);
  else static_assert(R == 2, "radix not implemented");
}

template <int DIR, typename T, int N, int R, int P>
__device__ __forceinline__ void stage(const cpx<T>* __restrict__ in, cpx<T>* __restrict__ out,
                                      const cpx<T>* __restrict__ tw, int l, int lane) {
  constexpr int NB = N / R;
  constexpr int TPL = Tpl<N>::value;
  constexpr int TWS = N / (P * R);
  constexpr int ITERS = (NB + TPL - 1) / TPL;
  constexpr int NP = Pad<T, N>::NP;
#pragma unroll
  for (int it = 0; it < ITERS; ++it) {
    const int i = lane + it * TPL;
    if ((NB % TPL) != 0 && i >= NB) break;
    const int k = (P == 1) ? 0 : i % P;
    cpx<T> u[R];
#pragma unroll
    for (int t = 0; t < R; ++t) {
      cpx<T> v = in[sw<T, NP>(l, i + t * NB)];
      if (P > 1 && t > 0) {
        const cpx<T> w = tw[t * k * TWS];
        v = DIR < 0 ? c_mul(v, w) : c_mulc(v, w);
      }
      u[t] = v;
    }
    dft<DIR, T, R>(u);
    const int j0 = (i - k) * R + k;
#pragma unroll
    for (int t = 0; t < R; ++t) out[sw<T, NP>(l, j0 + t * P)] = u[t];
  }
}

template <int DIR, typename T, int N, int P, int R0, int... Rs>
__device__ __forceinline__ cpx<T>* run(cpx<T>* a, cpx<T>* b, const cpx<T>* tw, int l, int lane, bool active) {
  if (active) stage<DIR, T, N, R0, P>(a, b, tw, l, lane);
  __syncthreads();
  if constexpr (sizeof...(Rs) == 0) return b;
  else return run<DIR, T, N, P * R0, Rs...>(b, a, tw, l, lane, active);
}

template <int DIR, typename T, int N, int... Rs>
__device__ __forceinline__ cpx<T>* run_sched(Sched<Rs...>, cpx<T>* a, cpx<T>* b, const cpx<T>* tw, int l, int lane,
                                             bool active) {
  return run<DIR, T, N, 1, Rs...>(a, b, tw, l, lane, active);
}

// Transform lines of the CTA in place of buffer a (result returned: a or b).
// Every thread of the CTA must call it (it contains __syncthreads).
template <int DIR, typename T, int N>
__device__ __forceinline__ cpx<T>* fft(cpx<T>* a, cpx<T>* b, const cpx<T>* tw, int l, int lane, bool active) {
  return run_sched<DIR, T, N>(typename Plan<N>::S{}, a, b, tw, l, lane, active);
}

// ---------------------------------------------------------------------------
// FP64 elementary functions for the pointwise epilogue: a single-precision
// seed refined by Newton iterations in double (quadratic convergence: the
// ~1e-7 seed reaches full double precision after two steps).  Used for
// x > 0 finite arguments in the float range.
// ---------------------------------------------------------------------------
// x^(-1/3): Newton on f(z) = z^-3 - x:  z <- z (4 - x z^3) / 3
__device__ __forceinline__ double rcbrt_d(double x) {
  double z = (double)(1.0f / cbrtf((float)x));
  z = z * (4.0 - x * z * z * z) * (1.0 / 3.0);
  z = z * (4.0 - x * z * z * z) * (1.0 / 3.0);
  return z;
}
// x^(-1/2): Newton on f(z) = z^-2 - x:  z <- z (3 - x z^2) / 2
__device__ __forceinline__ double rsqrt_d(double x) {
  double z = (double)rsqrtf((float)x);
  z = z * (1.5 - 0.5 * x * z * z);
  z = z * (1.5 - 0.5 * x * z * z);
  return z;
}
__device__ __forceinline__ float rcbrt_d(float x) { return rcbrtf(x); }
__device__ __forceinline__ float rsqrt_d(float x) { return rsqrtf(x); }

}  // namespace gbct
