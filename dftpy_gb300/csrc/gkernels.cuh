// Reciprocal-space kernels K(|G|) on the half spectrum, shared by the
// generic and the compile-time-size passes.
#pragma once
#include "plan.h"

namespace gbk {

constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ int ffreq(int i, int n) { return (i <= (n - 1) / 2) ? i : i - n; }

template <typename T>
__device__ __forceinline__ T gg_of(const GInfo& g, int m0, int m1, int m2) {
  const T gx = (T)m0 * (T)g.bg[0] + (T)m1 * (T)g.bg[3] + (T)m2 * (T)g.bg[6];
  const T gy = (T)m0 * (T)g.bg[1] + (T)m1 * (T)g.bg[4] + (T)m2 * (T)g.bg[7];
  const T gz = (T)m0 * (T)g.bg[2] + (T)m1 * (T)g.bg[5] + (T)m2 * (T)g.bg[8];
  return gx * gx + gy * gy + gz * gz;
}

// Evaluate a kernel K(|G|) at half-spectrum index (i0, i1, k2) in the
// reference's convention: with full grids every axis uses fftfreq, and where
// an index sits on a Nyquist plane the value is averaged with the one at
// the conjugate partner (-i0, -i1, -k2) -- the real part of the inverse
// transform sees exactly that average.  Half grids only average inside the
// k2 = 0 and k2 = n2/2 planes, which are the ones irfftn symmetrises.
template <typename T, typename F>
__device__ __forceinline__ T sym_kernel(const GInfo& g, int i0, int i1, int k2, F kv) {
  const int m0 = ffreq(i0, g.n0), m1 = ffreq(i1, g.n1);
  const int m2 = g.full ? ffreq(k2, g.n2) : k2;
  T k = kv(gg_of<T>(g, m0, m1, m2));
  const bool nyq = ((g.n0 & 1) == 0 && 2 * i0 == g.n0) || ((g.n1 & 1) == 0 && 2 * i1 == g.n1) ||
                   (g.full && (g.n2 & 1) == 0 && 2 * k2 == g.n2);
  const bool plane = g.full || k2 == 0 || ((g.n2 & 1) == 0 && 2 * k2 == g.n2);
  if (nyq && plane) {
    const int p0 = ffreq((g.n0 - i0) % g.n0, g.n0), p1 = ffreq((g.n1 - i1) % g.n1, g.n1);
    const int p2 = g.full ? ffreq((g.n2 - k2) % g.n2, g.n2) : k2;
    k = (k + kv(gg_of<T>(g, p0, p1, p2))) * (T)0.5;
  }
  return k;
}

template <typename T>
__device__ __forceinline__ T kernel_value(const GInfo& g, int type, const void* arr, int i0, int i1, int k2) {
  if (type == KER_HARTREE)
    return sym_kernel<T>(g, i0, i1, k2, [](T gg) { return gg > (T)0 ? (T)(4.0 * kPi) / gg : (T)0; });
  if (type == KER_G2) return sym_kernel<T>(g, i0, i1, k2, [](T gg) { return gg; });
  if (type == KER_ARRAY)
    return __ldg(reinterpret_cast<const T*>(arr) + ((int64_t)i0 * g.n1 + i1) * g.n2h + k2);
  return (T)1;
}


}  // namespace gbk
