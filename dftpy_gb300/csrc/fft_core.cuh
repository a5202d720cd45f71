// Mixed-radix Stockham FFT of many short lines held in shared memory.
//
// A CTA holds L lines of length n in shared memory at buf[l*ls + j*es]
// (element j of line l).  One stage of radix r with p = product of the
// previous radices maps, for every butterfly index i in [0, n/r):
//     k = i % p
//     u_t = in[i + t*n/r] * w^(t*k),  w = exp(DIR*2*pi*i/(p*r))   t = 0..r-1
//     v   = DFT_r(u)
//     out[(i-k)*r + k + t*p] = v_t
// which leaves the transform in natural order after the last stage
// (decimation-in-time Stockham autosort).  Twiddles come from one table
// tw[m] = exp(-2 pi i m / n), m in [0, n): w^(t*k) = tw[t*k*(n/(p*r))]
// (conjugated for the inverse direction).
#pragma once
#include "common.cuh"

namespace gbfft {

// radix constants (exact decimal expansions of the trigonometric values)
#define GB_S3 0.86602540378443864676   // sin(2 pi / 3)
#define GB_C5A 0.30901699437494742410  // cos(2 pi / 5)
#define GB_C5B -0.80901699437494742410 // cos(4 pi / 5)
#define GB_S5A 0.95105651629515357212  // sin(2 pi / 5)
#define GB_S5B 0.58778525229247312917  // sin(4 pi / 5)
#define GB_R2 0.70710678118654752440   // sqrt(1/2)

template <int DIR, typename T>
__device__ __forceinline__ void dft2(cpx<T>* u) {
  cpx<T> a = u[0], b = u[1];
  u[0] = c_add(a, b);
  u[1] = c_sub(a, b);
}

template <int DIR, typename T>
__device__ __forceinline__ void dft3(cpx<T>* u) {
  const T s3 = (T)GB_S3;
  cpx<T> t1 = c_add(u[1], u[2]);
  cpx<T> t2 = c_sub(u[0], c_scale(t1, (T)0.5));
  cpx<T> t3 = c_scale(c_sub(u[1], u[2]), s3);
  u[0] = c_add(u[0], t1);
  cpx<T> r = c_rot<DIR>(t3);  // DIR*i*t3
  u[1] = c_add(t2, r);
  u[2] = c_sub(t2, r);
}

template <int DIR, typename T>
__device__ __forceinline__ void dft4(cpx<T>* u) {
  cpx<T> a = c_add(u[0], u[2]);
  cpx<T> b = c_sub(u[0], u[2]);
  cpx<T> c = c_add(u[1], u[3]);
  cpx<T> d = c_rot<DIR>(c_sub(u[1], u[3]));
  u[0] = c_add(a, c);
  u[2] = c_sub(a, c);
  u[1] = c_add(b, d);
  u[3] = c_sub(b, d);
}

template <int DIR, typename T>
__device__ __forceinline__ void dft5(cpx<T>* u) {
  const T c1 = (T)GB_C5A, c2 = (T)GB_C5B, s1 = (T)GB_S5A, s2 = (T)GB_S5B;
  cpx<T> t1 = c_add(u[1], u[4]);
  cpx<T> t2 = c_add(u[2], u[3]);
  cpx<T> t3 = c_sub(u[1], u[4]);
  cpx<T> t4 = c_sub(u[2], u[3]);
  cpx<T> a1 = {u[0].x + c1 * t1.x + c2 * t2.x, u[0].y + c1 * t1.y + c2 * t2.y};
  cpx<T> a2 = {u[0].x + c2 * t1.x + c1 * t2.x, u[0].y + c2 * t1.y + c1 * t2.y};
  cpx<T> b1 = {s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y};
  cpx<T> b2 = {s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y};
  u[0] = c_add(u[0], c_add(t1, t2));
  cpx<T> r1 = c_rot<DIR>(b1), r2 = c_rot<DIR>(b2);
  u[1] = c_add(a1, r1);
  u[4] = c_sub(a1, r1);
  u[2] = c_add(a2, r2);
  u[3] = c_sub(a2, r2);
}

template <int DIR, typename T>
__device__ __forceinline__ void dft8(cpx<T>* u) {
  const T h = (T)GB_R2;
  cpx<T> b[4], c[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    b[k] = c_add(u[k], u[k + 4]);
    c[k] = c_sub(u[k], u[k + 4]);
  }
  // c_k *= exp(DIR * i * pi * k / 4)
  c[1] = c_scale(c_add(c[1], c_rot<DIR>(c[1])), h);
  c[2] = c_rot<DIR>(c[2]);
  c[3] = c_scale(c_sub(c_rot<DIR>(c[3]), c[3]), h);
  dft4<DIR, T>(b);
  dft4<DIR, T>(c);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    u[2 * k] = b[k];
    u[2 * k + 1] = c[k];
  }
}

// One Stockham stage over all lines of the CTA.
//   in/out: shared buffers, element (line l, index j) at l*ls + j*es
//   LINE_FAST: consecutive threads walk the butterfly index (line-major
//   buffers); otherwise they walk the line index (column-tile buffers).
template <int DIR, typename T, bool LINE_FAST>
__device__ __forceinline__ void stage(const cpx<T>* __restrict__ in, cpx<T>* __restrict__ out,
                                      const cpx<T>* __restrict__ tw, int n, int r, int p,
                                      int nlines, int ls, int es, int tid, int nthr) {
  const int nb = n / r;
  const int tws = n / (p * r);
  const int total = nb * nlines;
  for (int idx = tid; idx < total; idx += nthr) {
    int i, l;
    if (LINE_FAST) { i = idx % nb; l = idx / nb; }
    else { l = idx % nlines; i = idx / nlines; }
    const int k = i % p;
    const cpx<T>* src = in + l * ls;
    cpx<T>* dst = out + l * ls;
    const int j0 = (i - k) * r + k;
    if (r == 2 || r == 3 || r == 4 || r == 5 || r == 8) {
      cpx<T> u[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        if (t < r) {
          cpx<T> v = src[(i + t * nb) * es];
          if (t > 0 && k > 0) {
            cpx<T> w = tw[t * k * tws];
            v = DIR < 0 ? c_mul(v, w) : c_mulc(v, w);
          }
          u[t] = v;
        }
      }
      switch (r) {
        case 2: dft2<DIR, T>(u); break;
        case 3: dft3<DIR, T>(u); break;
        case 4: dft4<DIR, T>(u); break;
        case 5: dft5<DIR, T>(u); break;
        default: dft8<DIR, T>(u); break;
      }
#pragma unroll
      for (int t = 0; t < 8; ++t)
        if (t < r) dst[(j0 + t * p) * es] = u[t];
    } else {
      // generic odd radix: direct DFT, O(r^2), twiddles from the table
      const int wr = n / r;
      for (int q = 0; q < r; ++q) {
        cpx<T> acc = {(T)0, (T)0};
        for (int t = 0; t < r; ++t) {
          cpx<T> v = src[(i + t * nb) * es];
          int m = (t * k * tws + ((t * q) % r) * wr) % n;
          cpx<T> w = tw[m];
          v = DIR < 0 ? c_mul(v, w) : c_mulc(v, w);
          acc = c_add(acc, v);
        }
        dst[(j0 + q * p) * es] = acc;
      }
    }
  }
}

// Full transform of all lines; returns the buffer holding the result.
template <int DIR, typename T, bool LINE_FAST>
__device__ cpx<T>* lines_fft(cpx<T>* a, cpx<T>* b, const cpx<T>* tw, const AxisPlan& ax,
                             int nlines, int ls, int es) {
  int p = 1;
  const int tid = threadIdx.x, nthr = blockDim.x;
  for (int s = 0; s < ax.nst; ++s) {
    const int r = ax.radix[s];
    stage<DIR, T, LINE_FAST>(a, b, tw, ax.n, r, p, nlines, ls, es, tid, nthr);
    __syncthreads();
    cpx<T>* t = a; a = b; b = t;
    p *= r;
  }
  return a;
}

}  // namespace gbfft
