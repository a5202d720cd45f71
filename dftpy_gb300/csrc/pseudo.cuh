// Device helpers shared by the set-up kernels (v_loc, Ewald) and the force
// kernels: reciprocal-space geometry, v(|G|) lines, PME B-spline spreading,
// separable structure-factor phases and the reference half-space mask.
#pragma once

#include "plan.h"

namespace {


__device__ __forceinline__ int ffreq(int i, int n) { return (i <= (n - 1) / 2) ? i : i - n; }

__device__ __forceinline__ double gg_at(const GInfo& g, int m0, int m1, int m2) {
  const double gx = m0 * g.bg[0] + m1 * g.bg[3] + m2 * g.bg[6];
  const double gy = m0 * g.bg[1] + m1 * g.bg[4] + m2 * g.bg[7];
  const double gz = m0 * g.bg[2] + m1 * g.bg[5] + m2 * g.bg[8];
  return gx * gx + gy * gy + gz * gz;
}

struct VTabs {
  gbofdft_vtable t[GBOFDFT_MAX_SPECIES];
  int n;
};

__device__ double vline_eval(const gbofdft_vtable& t, double q) {
  if (!(q < t.gmax)) return 0.0;
  if (q < t.gmin) {
    const double dx = q / t.dp;
    return t.q4[0] + dx * (t.q4[1] + dx * (t.q4[2] + dx * (t.q4[3] + dx * t.q4[4]))) / 24.0;
  }
  // the interval x[lo] <= q < x[lo + 1]: first the index a uniform grid
  // would give (the tables' usual case: two loads), else a bisection; both
  // find the same interval
  int lo;
  {
    int g = -1;
    if (t.m >= 2) {
      const double x0 = __ldg(t.x), xl = __ldg(t.x + t.m - 1);
      const double f = xl > x0 ? (q - x0) / (xl - x0) * (double)(t.m - 1) : 0.0;
      g = f < 0.0 ? 0 : (f > (double)(t.m - 2) ? t.m - 2 : (int)f);
      if (!(__ldg(t.x + g) <= q && q < __ldg(t.x + g + 1))) g = -1;
    }
    if (g >= 0) {
      lo = g;
    } else {
      lo = 0;
      int hi = t.m - 1;  // x[lo] <= q < x[hi]
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(t.x + mid) <= q) lo = mid; else hi = mid;
      }
    }
  }
  const double u = q - __ldg(t.x + lo);
  const double* cc = t.c + 4 * (size_t)lo;
  return __ldg(cc) + u * (__ldg(cc + 1) + u * (__ldg(cc + 2) + u * __ldg(cc + 3)));
}

// Nyquist-plane partner rule (same as the reciprocal kernels in passes.cu)
__device__ __forceinline__ bool needs_sym(const GInfo& g, int i0, int i1, int k2) {
  const bool nyq = ((g.n0 & 1) == 0 && 2 * i0 == g.n0) || ((g.n1 & 1) == 0 && 2 * i1 == g.n1) ||
                   (g.full && (g.n2 & 1) == 0 && 2 * k2 == g.n2);
  const bool plane = g.full || k2 == 0 || ((g.n2 & 1) == 0 && 2 * k2 == g.n2);
  return nyq && plane;
}

__device__ __forceinline__ int m2_of(const GInfo& g, int k2) { return g.full ? ffreq(k2, g.n2) : k2; }
__device__ __forceinline__ int m2_partner(const GInfo& g, int k2) {
  return g.full ? ffreq((g.n2 - k2) % g.n2, g.n2) : k2;
}

__device__ __forceinline__ void decode(const GInfo& g, int64_t id, int& i0, int& i1, int& k2) {
  k2 = (int)(id % g.n2h);
  const int64_t r = id / g.n2h;
  i1 = (int)(r % g.n1);
  i0 = (int)(r / g.n1);
}

// Cardinal B-spline weights of one axis (CBspline.calc_Mn, ewald.py:63-80):
// M[i] = M_order(x + i), i = 0 .. order-1, for the fractional offset x.
// With dM, also the derivative along the axis in grid units times n:
// dM[i] = n (M'_(order-1)[i+1] - M'_(order-1)[i]) with M' the order-1 spline
// on an array sized for order (its last entry stays 0), as the force
// routines of the reference build it (pseudo/__init__.py:501-511).
__device__ inline void bspline_weights(double x, int order, int n, double* M, double* dM) {
  double Mn[32], M2[32];
  for (int i = 0; i <= order; ++i) { Mn[i] = 0.0; M2[i] = 0.0; }
  Mn[1] = x; Mn[2] = 1.0 - x;
  M2[1] = x; M2[2] = 1.0 - x;
  for (int i = 3; i <= order; ++i)
    for (int j = 0; j < i; ++j) {
      const int nn = i - j;
      Mn[nn] = ((x + nn - 1) * Mn[nn] + (j + 1 - x) * Mn[nn - 1]) / (i - 1);
      if (i < order) M2[nn] = ((x + nn - 1) * M2[nn] + (j + 1 - x) * M2[nn - 1]) / (i - 1);
    }
  for (int i = 0; i < order; ++i) {
    M[i] = Mn[i + 1];
    if (dM) dM[i] = (double)n * (M2[i + 1] - M2[i]);
  }
}

// ---- PME charge spreading ---------------------------------------------------
// One CTA per atom (atoms of other species skip).  Q[(1 + floor(u_d) - i_d)
// mod n_d] += w_a M_(i0+1) M_(i1+1) M_(i2+1)  (CBspline.get_PME_Qarray).
template <typename T>
__global__ void k_pme_spread(GInfo g, const double* __restrict__ spos, const double* __restrict__ w,
                             const int* __restrict__ species, int want, int order, T* __restrict__ Q) {
  const int a = blockIdx.x;
  if (species && species[a] != want) return;
  __shared__ double M[3][32];
  __shared__ int fl[3];
  if (threadIdx.x < 3) {
    const int d = threadIdx.x;
    const int n = d == 0 ? g.n0 : (d == 1 ? g.n1 : g.n2);
    const double u = spos[3 * a + d] * n;
    const double f = floor(u);
    bspline_weights(u - f, order, n, M[d], nullptr);
    fl[d] = (int)f;
  }
  __syncthreads();
  const double wa = w ? w[a] : 1.0;
  const int o3 = order * order * order;
  for (int t = threadIdx.x; t < o3; t += blockDim.x) {
    const int i = t / (order * order), j = (t / order) % order, k = t % order;
    int l0 = (1 + fl[0] - i) % g.n0; if (l0 < 0) l0 += g.n0;
    int l1 = (1 + fl[1] - j) % g.n1; if (l1 < 0) l1 += g.n1;
    int l2 = (1 + fl[2] - k) % g.n2; if (l2 < 0) l2 += g.n2;
    atomicAdd(Q + ((int64_t)l0 * g.n1 + l1) * g.n2 + l2, (T)(wa * M[0][i] * M[1][j] * M[2][k]));
  }
}

__device__ __forceinline__ double2 bprod(const double2* bm0, const double2* bm1, const double2* bm2, int i0, int i1,
                                         int k2) {
  const double2 b0 = bm0[i0], b1 = bm1[i1], b2 = bm2[k2];
  double2 b = {b0.x * b1.x - b0.y * b1.y, b0.x * b1.y + b0.y * b1.x};
  return double2{b.x * b2.x - b.y * b2.y, b.x * b2.y + b.y * b2.x};
}

// Phase tables exp(-2 pi i m s_{a,d}) for every atom a.
//   mode 0: index i in [0, n) of axis d, m = fftfreq(i)
//   mode 1: axis 2 stored index k2 in [0, n2h), m = m2_of(k2)
//   mode 2: axis 2 stored index, m = m2_partner(k2)
__global__ void k_phase_table(GInfo g, const double* __restrict__ spos, int nat, int d, int mode,
                              double2* __restrict__ out) {
  const int n = mode == 0 ? (d == 0 ? g.n0 : (d == 1 ? g.n1 : g.n2)) : g.n2h;
  const int64_t total = (int64_t)nat * n;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(id / n), i = (int)(id % n);
    int m;
    if (mode == 0) m = ffreq(i, n);
    else if (mode == 1) m = m2_of(g, i);
    else m = m2_partner(g, i);
    double x = (double)m * spos[3 * a + d];
    x -= rint(x);
    double sn, cs;
    sincospi(-2.0 * x, &sn, &cs);
    out[id] = double2{cs, sn};
  }
}

__device__ __forceinline__ double2 phase(const double2* ph0, const double2* ph1, const double2* ph2, const GInfo& g,
                                         int a, int i0, int i1, int k2) {
  const double2 e0 = ph0[(int64_t)a * g.n0 + i0], e1 = ph1[(int64_t)a * g.n1 + i1];
  const double2 e2 = ph2[(int64_t)a * g.n2h + k2];
  double2 e = {e0.x * e1.x - e0.y * e1.y, e0.x * e1.y + e0.y * e1.x};
  return double2{e.x * e2.x - e.y * e2.y, e.x * e2.y + e.y * e2.x};
}

// reference half-space mask (grid.py:658-695) on the stored half spectrum
__device__ __forceinline__ bool gmask(const GInfo& g, int i0, int i1, int k2) {
  const int D0 = g.n0 / 2, D1 = g.n1 / 2, D2 = g.n2 / 2;
  const bool e0 = (g.n0 & 1) == 0, e1 = (g.n1 & 1) == 0, e2 = (g.n2 & 1) == 0;
  if (k2 == 0) {
    if (i0 == 0 && i1 > D1) return false;
    if (i0 > D0) return false;
    if (e0 && i0 == D0 && i1 > D1) return false;
    if (e0 && e1 && i0 == D0 && i1 == D1) return false;
    if (e1 && i0 == 0 && i1 == D1) return false;
  }
  if (e2 && k2 == D2) {
    if (i0 == 0 && i1 == 0) return false;
    if (i0 == 0 && i1 > D1) return false;
    if (i0 > D0) return false;
    if (e1 && i0 == 0 && i1 == D1) return false;
    if (e0 && i0 == D0 && i1 == 0) return false;
    if (e0 && i0 == D0 && i1 > D1) return false;
  }
  if (e0 && e1 && e2 && i0 == D0 && i1 == D1 && k2 == D2) return false;
  return true;
}


int grid_blocks(int64_t total) {
  int64_t b = (total + 255) / 256;
  return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
}

size_t round256(size_t x) { return (x + 255) / 256 * 256; }

size_t phase_bytes(const gbofdft_plan* p, int nat) {
  return round256(sizeof(double2) * (size_t)nat * (p->n[0] + p->n[1] + 2 * (size_t)p->n2h));
}

void phase_tables(gbofdft_plan* p, const double* spos, int nat, double2* base, cudaStream_t st, double2** ph0,
                  double2** ph1, double2** ph2, double2** ph2p) {
  *ph0 = base;
  *ph1 = *ph0 + (size_t)nat * p->n[0];
  *ph2 = *ph1 + (size_t)nat * p->n[1];
  *ph2p = *ph2 + (size_t)nat * p->n2h;
  k_phase_table<<<grid_blocks((int64_t)nat * p->n[0]), 256, 0, st>>>(p->gi, spos, nat, 0, 0, *ph0);
  k_phase_table<<<grid_blocks((int64_t)nat * p->n[1]), 256, 0, st>>>(p->gi, spos, nat, 1, 0, *ph1);
  k_phase_table<<<grid_blocks((int64_t)nat * p->n2h), 256, 0, st>>>(p->gi, spos, nat, 2, 1, *ph2);
  k_phase_table<<<grid_blocks((int64_t)nat * p->n2h), 256, 0, st>>>(p->gi, spos, nat, 2, 2, *ph2p);
}


}  // namespace
