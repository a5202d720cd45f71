// LWT / LMGP nonlocal kinetic functional on the device (dftpy
// functional/kedf/lwt.py:82-341 LWTPotentialEnergy, 36-79 guess_kf_bound,
// kernel.py:267-322 MGPKernelTable, 379-405 LWTKernelKf).
//
// The kernel depends on the local Fermi wavevector k_F(r) = 2 (3 pi^2 rho)^(1/3)
// through interpolation between knots k_i = k_min 1.15^i.  Per knot i:
//   p_i = ifft(K(q / k_i) rho^beta(G)),   m_i = ifft(K'(q / k_i) / k_i rho^beta(G))
// (one shared forward transform of rho^beta), then per point the interval
// [k_i, k_i+1] holding k_F(r) gives the interpolation weights.  The
// reference's second potential term sum_i K_i fft(rho^alpha w_i) (with masked
// interval weights) is regrouped by linearity into one forward transform per
// knot of the accumulated weight field.
#include <math.h>
#include <string.h>

#include <chrono>
#include <vector>

#include "gkernels.cuh"
#include "plan.h"

double kf_of_host(double rho);

namespace {

constexpr double kZero = 1e-30;

__device__ __forceinline__ int ffreq_l(int i, int n) { return (i <= (n - 1) / 2) ? i : i - n; }

// uniform-grid cubic spline table: coefficients c[j] (4 values) on
// [j deta, (j+1) deta]; eta >= etamax returns the end value.  A is the
// arithmetic type: double for FP64 plans, float (with an FP32 copy of the
// coefficients) for FP32 plans, so FP32 evaluations run no FP64 per element.
template <typename A>
struct UTable {
  const A* c;
  int neta;
  A deta, inv_deta, etamax, endval;
};

template <typename A>
__device__ __forceinline__ A utab_eval(const UTable<A>& t, A eta) {
  if (!(eta < t.etamax)) return t.endval;
  int j;
  if constexpr (sizeof(A) == 8) j = (int)(eta / t.deta);
  else j = (int)(eta * t.inv_deta);
  if (j > t.neta - 2) j = t.neta - 2;
  if (j < 0) j = 0;
  const A u = eta - j * t.deta;
  const A* cc = t.c + 4 * (size_t)j;
  return __ldg(cc) + u * (__ldg(cc + 1) + u * (__ldg(cc + 2) + u * __ldg(cc + 3)));
}

// reciprocal lattice rows in the arithmetic type
template <typename A>
struct BG {
  A b[9];
};

template <typename A>
__device__ __forceinline__ A gg_a(const BG<A>& bg, int m0, int m1, int m2) {
  const A f0 = (A)m0, f1 = (A)m1, f2 = (A)m2;
  const A gx = f0 * bg.b[0] + f1 * bg.b[3] + f2 * bg.b[6];
  const A gy = f0 * bg.b[1] + f1 * bg.b[4] + f2 * bg.b[7];
  const A gz = f0 * bg.b[2] + f1 * bg.b[5] + f2 * bg.b[8];
  return gx * gx + gy * gy + gz * gz;
}

// K(|G| / kf) in the Nyquist-partner-averaged form of gbk::sym_kernel, with
// the geometry in the arithmetic type A
template <typename A>
__device__ __forceinline__ A lwt_kval(const GInfo& g, const BG<A>& bg, const UTable<A>& t, A inv_kf, int i0, int i1,
                                      int k2) {
  if constexpr (sizeof(A) == 8) {
    return gbk::sym_kernel<double>(g, i0, i1, k2, [&](double gg) { return utab_eval(t, sqrt(gg) * inv_kf); });
  } else {
    const int m0 = ffreq_l(i0, g.n0), m1 = ffreq_l(i1, g.n1), m2 = g.full ? ffreq_l(k2, g.n2) : k2;
    A k = utab_eval(t, sqrt(gg_a(bg, m0, m1, m2)) * inv_kf);
    const bool nyq = ((g.n0 & 1) == 0 && 2 * i0 == g.n0) || ((g.n1 & 1) == 0 && 2 * i1 == g.n1) ||
                     (g.full && (g.n2 & 1) == 0 && 2 * k2 == g.n2);
    const bool plane = g.full || k2 == 0 || ((g.n2 & 1) == 0 && 2 * k2 == g.n2);
    if (nyq && plane) {
      const int p0 = ffreq_l((g.n0 - i0) % g.n0, g.n0), p1 = ffreq_l((g.n1 - i1) % g.n1, g.n1);
      const int p2 = g.full ? ffreq_l((g.n2 - k2) % g.n2, g.n2) : k2;
      k = (k + utab_eval(t, sqrt(gg_a(bg, p0, p1, p2)) * inv_kf)) * (A)0.5;
    }
    return k;
  }
}

// Spectral kernels walk the half spectrum row by row: one CTA per (i0, i1)
// row at a time, its threads over k2, so no per-element index division.
// dst[f] = coef_f * K_f(q / kf) * src   (f = 0: kernel table, f = 1: derivative table)
template <typename T>
__global__ void k_lwt_kmul(GInfo g, BG<T> bg, const cpx<T>* __restrict__ src, int64_t sld, cpx<T>* __restrict__ dst,
                           int64_t dfs, int nf, UTable<T> tk, UTable<T> td, double kf, double scale) {
  const int nrow = g.n0 * g.n1;
  const T inv_kf = (T)(1.0 / kf), kfT = (T)kf, scT = (T)scale;
  for (int row = blockIdx.x; row < nrow; row += gridDim.x) {
    const int i0 = row / g.n1, i1 = row - i0 * g.n1;
    for (int k2 = threadIdx.x; k2 < g.n2h; k2 += blockDim.x) {
      const cpx<T> s = src[(int64_t)row * sld + k2];
      for (int f = 0; f < nf; ++f) {
        const UTable<T>& t = f == 0 ? tk : td;
        T kv = (T)0;
        if (!(i0 == 0 && i1 == 0 && k2 == 0)) kv = lwt_kval<T>(g, bg, t, inv_kf, i0, i1, k2);
        if (f == 1) kv /= kfT;
        const T c = kv * scT;
        dst[f * dfs + (int64_t)row * g.ld2 + k2] = cpx<T>{s.x * c, s.y * c};
      }
    }
  }
}

// acc (+)= K(q/kf) U + [D(q/kf)/kf Ud]     (half spectra, layout ld2)
template <typename T>
__global__ void k_lwt_acc(GInfo g, BG<T> bg, const cpx<T>* __restrict__ U, int64_t ufs, int nf, UTable<T> tk,
                          UTable<T> td, double kf, double scale, cpx<T>* __restrict__ acc, int first) {
  const int nrow = g.n0 * g.n1;
  const T inv_kf = (T)(1.0 / kf), kfT = (T)kf, scT = (T)scale;
  for (int row = blockIdx.x; row < nrow; row += gridDim.x)
  for (int k2 = threadIdx.x; k2 < g.n2h; k2 += blockDim.x) {
    const int i0 = row / g.n1, i1 = row - i0 * g.n1;
    const int64_t o = (int64_t)row * g.ld2 + k2;
    T ax = (T)0, ay = (T)0;
    if (!(i0 == 0 && i1 == 0 && k2 == 0)) {
      for (int f = 0; f < nf; ++f) {
        const UTable<T>& t = f == 0 ? tk : td;
        T kv = lwt_kval<T>(g, bg, t, inv_kf, i0, i1, k2);
        if (f == 1) kv /= kfT;
        const cpx<T> u = U[f * ufs + o];
        ax += kv * scT * u.x;
        ay += kv * scT * u.y;
      }
    }
    if (first) acc[o] = cpx<T>{ax, ay};
    else acc[o] = cpx<T>{acc[o].x + ax, acc[o].y + ay};
  }
}

__device__ __forceinline__ double kf_of(double rho) { return 2.0 * cbrt(3.0 * 9.86960440108935861883 * rho); }
__device__ __forceinline__ float kf_of(float rho) { return 2.0f * cbrtf(29.6088132032680758f * rho); }

// once per evaluation: kf(r) = 2 (3 pi^2 rho)^(1/3) clamped at kfmax, and
// rho^alpha (rho clamped at 1e-30)
template <typename T>
__global__ void k_lwt_pre(int64_t n, const T* __restrict__ rho, double kfmax, double alpha, T* __restrict__ kfo,
                          T* __restrict__ rao) {
  const T kfm = (T)kfmax, al = (T)alpha;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T r = rho[i];
    T kf = kf_of(r);
    if (kf > kfm) kf = kfm;
    const T rc = r > (T)0 ? r : (T)kZero;
    kfo[i] = kf;
    rao[i] = pow(rc, al);
  }
}

struct IntervalArgs {
  const void* rho;
  const void *kf, *ra;      // k_lwt_pre fields
  const void *p0, *p1, *m0, *m1;
  void *pot1, *pot3;
  void *w0, *w1, *wd0, *wd1;   // weight fields of knots i and i+1 (wd: derivative kernels, hermite)
  double kl, kr, kfmax, alpha;
  int first, hermite, kdd, mcalc;
  int64_t n;
};

// Interval [kl, kr] of the knot list: pot1, pot3 at its points and the
// weights of its two knots (lwt.py:196-291).  first: also the region below
// the first knot.
template <typename T>
__global__ void k_lwt_interval(IntervalArgs a) {
  const T *kfp = reinterpret_cast<const T*>(a.kf), *rap = reinterpret_cast<const T*>(a.ra);
  const T *p0 = reinterpret_cast<const T*>(a.p0), *p1 = reinterpret_cast<const T*>(a.p1);
  const T *m0 = reinterpret_cast<const T*>(a.m0), *m1 = reinterpret_cast<const T*>(a.m1);
  T *pot1 = reinterpret_cast<T*>(a.pot1), *pot3 = reinterpret_cast<T*>(a.pot3);
  T *w0 = reinterpret_cast<T*>(a.w0), *w1 = reinterpret_cast<T*>(a.w1);
  T *wd0 = reinterpret_cast<T*>(a.wd0), *wd1 = reinterpret_cast<T*>(a.wd1);
  const T kl = (T)a.kl, kr_e = (T)(a.kr + 1e-18), kl_e = (T)(a.kl + 1e-18);
  const T dk = (T)(a.kr - a.kl), inv_kl = (T)(1.0 / a.kl);
  const T one = (T)1, two = (T)2, three = (T)3;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
    const T kf = kfp[i];
    const T rA = rap[i];
    if (a.first && kf < kl_e) {
      T t;
      if constexpr (sizeof(T) == 8) t = (kf - kl) / kl;
      else t = (kf - kl) * inv_kl;
      pot1[i] = p0[i] * t;
      if (a.kdd > 1) w0[i] += rA * t;
    }
    if (!(kf > kl && kf < kr_e)) continue;
    const T t = (kf - kl) / dk;
    if (!a.hermite) {
      const T t0 = one - t;
      pot1[i] = p0[i] * t0 + p1[i] * t;
      if (a.kdd > 1) {
        w0[i] += rA * t0;
        w1[i] += rA * t;
        if (a.kdd == 3) pot3[i] = m0[i] * t0 + m1[i] * t;
      }
    } else {
      const T t2 = t * t, t3 = t2 * t;
      const T h00 = two * t3 - three * t2 + one, h10 = t3 - two * t2 + t, h01 = one - h00, h11 = t3 - t2;
      pot1[i] = h00 * p0[i] + h01 * p1[i] + dk * (h10 * m0[i] + h11 * m1[i]);
      if (a.kdd > 1) {
        w0[i] += rA * h00;
        w1[i] += rA * h01;
        wd0[i] += rA * dk * h10;
        wd1[i] += rA * dk * h11;
        if (a.kdd == 3) {
          const T six = (T)6, four = (T)4;
          const T h00D = six * t2 - six * t, h10D = three * t2 - four * t + one, h01D = -h00D,
                  h11D = three * t2 - two * t;
          pot3[i] = (h00D * p0[i] + h01D * p1[i]) / dk + h10D * m0[i] + h11D * m1[i];
        }
      }
    }
  }
}

// final assembly (lwt.py:305-341): low-density weight, energy, potential
template <typename T>
__global__ void k_lwt_final(int64_t n, const T* __restrict__ rho, const T* __restrict__ kfp,
                            const T* __restrict__ rap, const T* __restrict__ pot1, const T* __restrict__ pot2,
                            const T* __restrict__ pot3, double alpha, double beta, double rhov, double ld, int vcalc,
                            int have_pot2, T* __restrict__ pot, double* __restrict__ partial) {
  const T al = (T)alpha, be = (T)beta, ldT = (T)ld, inv_rhov_ld = (T)(1.0 / pow(rhov, ld));
  const T third = (T)(1.0 / 3.0);
  T es = (T)0;   // per-thread energy sum in the field precision, FP64 above
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T r = rho[i];
    T fac = (T)1;
    if (r < (T)1e-6) {
      if constexpr (sizeof(T) == 8) fac = pow(fabs(r), ld) / pow(rhov, ld);
      else fac = pow(fabs(r), ldT) * inv_rhov_ld;
    }
    if (r < (T)0) fac = (T)0;
    const T rc = r > (T)0 ? r : (T)kZero;
    const T rA = rap[i];
    const T p1 = pot1[i] * fac;
    es += rA * p1;
    if (vcalc) {
      const T kf = kfp[i];
      const T p2 = (have_pot2 ? pot2[i] : pot1[i]) * fac;
      const T p3 = pot3[i] * fac;
      const T rB = alpha == beta ? rA : pow(rc, be);
      T v;
      if constexpr (sizeof(T) == 8) v = p1 * al * (rA / rc) + p2 * be * (rB / rc) + p3 * (kf / 3.0) * (rA / rc);
      else v = p1 * al * (rA / rc) + p2 * be * (rB / rc) + p3 * (kf * third) * (rA / rc);
      pot[i] = pot[i] + v;
    }
  }
  __shared__ double red[32];
  double v = warp_sum((double)es);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t.add(red[w]);
    partial[blockIdx.x] = t.value();
  }
}

// energies[NL] += dV * sum(partials); energies[TOTAL] likewise
__global__ void k_lwt_energy(const double* __restrict__ partial, int nb, double dV, double* __restrict__ e) {
  __shared__ double red[32];
  KSum s;
  s.init();
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s.add(partial[i]);
  double v = warp_sum(s.value());
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t.add(red[w]);
    const double en = t.value() * dV;
    e[GB_E_NL] += en;
    e[GB_E_TOTAL] += en;
  }
}

template <typename T>
__global__ void k_minmax(int64_t n, const T* __restrict__ x, double* __restrict__ part) {
  T mnT = x[0], mxT = x[0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T v = x[i];
    mnT = v < mnT ? v : mnT;
    mxT = v > mxT ? v : mxT;
  }
  double mn = (double)mnT, mx = (double)mxT;
  for (int o = 16; o > 0; o >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  __shared__ double smn[32], smx[32];
  if ((threadIdx.x & 31) == 0) { smn[threadIdx.x >> 5] = mn; smx[threadIdx.x >> 5] = mx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { mn = fmin(mn, smn[w]); mx = fmax(mx, smx[w]); }
    mn = fmin(mn, smn[0]);
    mx = fmax(mx, smx[0]);
    part[2 * blockIdx.x] = mn;
    part[2 * blockIdx.x + 1] = mx;
  }
}

// MGP kernel table: sum_{i=1..np} G(eta / t_i^(1/3)) / t_i^(1/6), t_i = i / np,
// G = cubic spline on the log-spaced knots gp (beyond [gp0, gpm] the end
// values).  The knot interval comes from a single-precision logarithm guess
// corrected against the double knots.
__global__ void k_mgp_table(const double* __restrict__ gp, const double* __restrict__ c, int m,
                            const double* __restrict__ eta, int neta, int np, double coe, double* __restrict__ out) {
  extern __shared__ double tsh[];  // [np] 1/cbrt(t), [np] t^(-1/6)
  for (int i = threadIdx.x; i < np; i += blockDim.x) {
    const double t = (double)(i + 1) / (double)np;
    tsh[i] = 1.0 / cbrt(t);
    tsh[np + i] = 1.0 / pow(t, 1.0 / 6.0);
  }
  __syncthreads();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= neta) return;
  const double e = eta[j];
  const double lo = gp[0], hi = gp[m - 1];
  const float inv_lr = (float)((m - 1) / log(hi / lo));
  KSum s;
  s.init();
  for (int i = 0; i < np; ++i) {
    double x = e * tsh[i];
    x = fmin(fmax(x, lo), hi);
    int a = (int)(logf((float)(x / lo)) * inv_lr);
    a = a < 0 ? 0 : (a > m - 2 ? m - 2 : a);
    while (a > 0 && __ldg(gp + a) > x) --a;
    while (a < m - 2 && __ldg(gp + a + 1) <= x) ++a;
    const double u = x - __ldg(gp + a);
    const double* cc = c + 4 * (size_t)a;
    const double gval = __ldg(cc) + u * (__ldg(cc + 1) + u * (__ldg(cc + 2) + u * __ldg(cc + 3)));
    s.add(gval * tsh[np + i]);
  }
  out[j] = s.value() * coe;
}

int blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
}

size_t r256(size_t x) { return (x + 255) / 256 * 256; }

// launch shape of the row-wise spectral kernels: threads cover one half
// row (k2 = 0 .. n2h-1) in whole warps, CTAs stride over the rows
struct RowLaunch {
  int blocks, threads;
};
RowLaunch row_launch(const gbofdft_plan* p) {
  const int nrow = p->gi.n0 * p->gi.n1;
  int th = (p->gi.n2h + 31) / 32 * 32;
  if (th > 256) th = 256;
  return RowLaunch{nrow < 4096 ? nrow : 4096, th};
}

constexpr int kMaxNetaF32 = 200001;   // FP32 table copies: coefficients of at most this many points

struct LwtBufs {
  void *p[2], *m[2], *w[2], *wd[2], *pot1, *pot2, *pot3, *kf, *ra;
  void *S, *T, *U, *G;   // spectra: rho^beta, knot work (2), weights (2), pot2 accumulator
  float *ktab_f, *dtab_f; // FP32 copies of the kernel tables (FP32 plans)
  double* part;
};

size_t lwt_field_bytes(const gbofdft_plan* p) { return r256(gb_elem(p) * (size_t)p->N); }
size_t lwt_spec_bytes(const gbofdft_plan* p) { return r256(2 * gb_elem(p) * (size_t)p->NGld); }

LwtBufs lwt_layout(const gbofdft_plan* p, void* work) {
  char* b = reinterpret_cast<char*>(work);
  const size_t fb = lwt_field_bytes(p), sb = lwt_spec_bytes(p);
  LwtBufs L;
  // p[c] and m[c] adjacent: the inverse transforms of a knot's two spectra
  // are one launch sequence with a field stride of one field
  void** fields[] = {&L.p[0], &L.m[0], &L.p[1], &L.m[1], &L.w[0], &L.w[1], &L.wd[0], &L.wd[1],
                     &L.pot1, &L.pot2, &L.pot3, &L.kf, &L.ra};
  for (int i = 0; i < 13; ++i) { *fields[i] = b; b += fb; }
  L.ktab_f = reinterpret_cast<float*>(b); b += r256(sizeof(float) * 4 * (size_t)kMaxNetaF32);
  L.dtab_f = reinterpret_cast<float*>(b); b += r256(sizeof(float) * 4 * (size_t)kMaxNetaF32);
  L.S = b; b += sb;
  L.T = b; b += 2 * sb;
  L.U = b; b += 2 * sb;
  L.G = b; b += sb;
  L.part = reinterpret_cast<double*>(b);
  return L;
}

template <typename T>
UTable<T> utab(const gbofdft_lwt* d, int deriv, const float* fcopy) {
  UTable<T> t;
  if constexpr (sizeof(T) == 8) t.c = deriv ? d->dtab_c : d->ktab_c;
  else t.c = fcopy;
  t.neta = d->neta;
  const double deta = d->etamax / (d->neta - 1);
  t.deta = (T)deta;
  t.inv_deta = (T)(1.0 / deta);
  t.etamax = (T)d->etamax;
  t.endval = (T)(deriv ? d->dtab_end : d->ktab_end);
  return t;
}

__global__ void k_to_float(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

template <typename T>
BG<T> bg_of(const gbofdft_plan* p) {
  BG<T> b;
  for (int i = 0; i < 9; ++i) b.b[i] = (T)p->bg[i];
  return b;
}

// forward 3D transform of a real field (scale 1) into spectrum layout ld2
int fwd3d(gbofdft_plan* p, const void* in, void* spec, int op, double beta, cudaStream_t st) {
  int rc = gb_rows_fwd(p, in, spec, 0, p->ld2, 1, &op, beta, 1.0, st);
  if (!rc) rc = gb_cols(p, spec, 0, p->ld2, 1, 1, -1, 1.0, st);
  if (!rc) rc = gb_cols(p, spec, 0, p->ld2, 1, 0, -1, 1.0, st);
  return rc;
}

// inverse 3D transform of nf spectra (consumed) into real fields out (stride ostride)
int inv3d(gbofdft_plan* p, void* spec, int64_t fstride, int nf, void* out, int64_t ostride, cudaStream_t st) {
  int rc = gb_cols(p, spec, fstride, p->ld2, nf, 0, 1, 1.0, st);
  if (!rc) rc = gb_cols(p, spec, fstride, p->ld2, nf, 1, 1, 1.0, st);
  if (!rc) rc = gb_rows_inv_store(p, spec, fstride, p->ld2, nf, out, ostride, 1.0, st);
  return rc;
}

template <typename T>
int lwt_run(gbofdft_plan* p, const void* rho, gbofdft_lwt* d, void* pot, double* energies, int calc_v, int calc_e,
            cudaStream_t st) {
  const int64_t N = p->N;
  LwtBufs L = lwt_layout(p, d->work);
  const int nb = blocks_for(N);
  const T* rhoT = reinterpret_cast<const T*>(rho);
  // rho extrema -> k_F bounds (guess_kf_bound, lwt.py:36-79)
  k_minmax<T><<<256, 256, 0, st>>>(N, rhoT, L.part);
  GB_CHECK_LAUNCH();
  std::vector<double> mm(512);
  GB_CUDA(cudaMemcpyAsync(mm.data(), L.part, sizeof(double) * 512, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  double rmin = 1e300, rmax = -1e300;
  for (int b = 0; b < 256; ++b) { rmin = fmin(rmin, mm[2 * b]); rmax = fmax(rmax, mm[2 * b + 1]); }
  const double kf_l = kf_of_host(rmin), kf_r = kf_of_host(rmax);
  d->nknots = 0;
  if (fabs(kf_r - kf_l) < 1e-8) return 0;  // homogeneous density: no contribution
  double kfmin, kfmax;
  if (d->kfmin_opt > 0 && d->kfmax_opt > 0) {
    kfmin = d->kfmin_opt;
    kfmax = d->kfmax_opt;
  } else {
    double kfmin_prev = d->kfmin_state, kfmax_prev = d->kfmax_state;
    kfmin = d->kfmin_opt > 0 ? d->kfmin_opt : -1.0;
    kfmax = d->kfmax_opt > 0 ? d->kfmax_opt : -1.0;
    if (!(kfmin_prev > 0)) { kfmin_prev = 10; if (!(kfmin > 0)) kfmin = kf_l; }
    if (!(kfmax_prev > 0)) { kfmax_prev = 1.0; if (!(kfmax > 0)) kfmax = kf_r; }
    if (!(kfmin > 0) || kfmin > kfmin_prev) kfmin = kfmin_prev;
    if (!(kfmax > 0) || kfmax < kfmax_prev) kfmax = kfmax_prev;
    if (kfmin > kf_l) {
      const double kfl[] = {1E-5, 1E-4, 5E-3, 1E-3, 5E-3, 1E-2, 5E-2, 0.1, 0.5, 1.0};
      const double ratio = kf_l / kfmin;
      for (int i = 9; i > 0; --i)
        if (ratio > kfl[i]) { kfmin *= kfl[i]; break; }
    }
    if (kfmin < 1e-3) kfmin = 1e-3;
    if (kfmax < kf_r) kfmax += (nearbyint((kf_r - kfmax) / 0.5) + 1) * 0.5;
    d->kfmin_state = kfmin;
    d->kfmax_state = kfmax;
  }
  const int nsp = (int)ceil(log(kfmax / kfmin) / log(d->ratio)) + 1;
  GB_REQUIRE(nsp >= 2 && nsp <= 4096, "lwt: %d knots from kf range [%g, %g]", nsp, kfmin, kfmax);
  std::vector<double> kfl(nsp);
  for (int i = 0; i < nsp; ++i) kfl[i] = kfmin * pow(d->ratio, (double)i);
  kfl[0] -= 1e-16;
  kfl[nsp - 1] += 1e-16;
  d->nknots = nsp;
  const int kdd = calc_v ? d->kdd : 1;
  const int hermite = d->interp == 1;
  const int mcalc = kdd > 1 || hermite;
  const int nkf = mcalc ? 2 : 1;
  if constexpr (sizeof(T) == 4) {
    GB_REQUIRE(d->neta <= kMaxNetaF32, "lwt: FP32 plans take at most %d table points (neta %d)", kMaxNetaF32,
               d->neta);
    const int64_t nc = 4 * (int64_t)(d->neta - 1);
    k_to_float<<<blocks_for(nc), 256, 0, st>>>(nc, d->ktab_c, L.ktab_f);
    k_to_float<<<blocks_for(nc), 256, 0, st>>>(nc, d->dtab_c, L.dtab_f);
    GB_CHECK_LAUNCH();
  }
  const UTable<T> tk = utab<T>(d, 0, L.ktab_f), td = utab<T>(d, 1, L.dtab_f);
  const BG<T> bg = bg_of<T>(p);
  k_lwt_pre<T><<<nb, 256, 0, st>>>(N, rhoT, kfmax, d->alpha, reinterpret_cast<T*>(L.kf), reinterpret_cast<T*>(L.ra));
  GB_CHECK_LAUNCH();
  const double invN = 1.0 / (double)N;
  const RowLaunch rl = row_launch(p);
  const size_t fb = lwt_field_bytes(p), sb = lwt_spec_bytes(p);
  const int64_t sfs = (int64_t)(sb / (2 * gb_elem(p)));  // complex elements per spectrum slot
  // shared forward transform of rho^beta (rho clamped to 1e-30 below)
  int rc = fwd3d(p, rho, L.S, OP_POWB, d->beta, st);
  if (rc) return rc;
  GB_CUDA(cudaMemsetAsync(L.pot1, 0, fb, st));
  GB_CUDA(cudaMemsetAsync(L.pot3, 0, fb, st));
  GB_CUDA(cudaMemsetAsync(L.w[0], 0, fb, st));
  GB_CUDA(cudaMemsetAsync(L.wd[0], 0, fb, st));
  const int nwf = hermite ? 2 : 1;
  int cur = 0;
  const int64_t ofs = (int64_t)(fb / gb_elem(p));   // p[c] -> m[c], in elements
  // weights of knot kk complete: G (+)= K_kk fft(w) (+ D_kk fft(wd))
  auto accumulate = [&](int kk, const void* w, const void* wd, int first) -> int {
    int r2 = fwd3d(p, w, L.U, OP_RHO, 1.0, st);
    if (!r2 && hermite) r2 = fwd3d(p, wd, (char*)L.U + sb, OP_RHO, 1.0, st);
    if (r2) return r2;
    k_lwt_acc<T><<<rl.blocks, rl.threads, 0, st>>>(p->gi, bg, (const cpx<T>*)L.U, sfs, nwf, tk, td, kfl[kk], invN,
                                                    (cpx<T>*)L.G, first);
    GB_CHECK_LAUNCH();
    return 0;
  };
  for (int k = 0; k < nsp; ++k) {
    // p[cur] (and m[cur], the next field): the knot's kernels times the shared
    // spectrum, inverse-transformed in one launch sequence
    k_lwt_kmul<T><<<rl.blocks, rl.threads, 0, st>>>(p->gi, bg, (const cpx<T>*)L.S, p->ld2, (cpx<T>*)L.T, sfs, nkf,
                                                     tk, td, kfl[k], invN);
    GB_CHECK_LAUNCH();
    if ((rc = inv3d(p, L.T, sfs, nkf, L.p[cur], ofs, st))) return rc;
    if (k >= 1) {
      const int prv = cur ^ 1;
      IntervalArgs a;
      a.rho = rho; a.kf = L.kf; a.ra = L.ra; a.p0 = L.p[prv]; a.p1 = L.p[cur]; a.m0 = L.m[prv]; a.m1 = L.m[cur];
      a.pot1 = L.pot1; a.pot3 = L.pot3;
      a.w0 = L.w[prv]; a.w1 = L.w[cur]; a.wd0 = L.wd[prv]; a.wd1 = L.wd[cur];
      a.kl = kfl[k - 1]; a.kr = kfl[k]; a.kfmax = kfmax; a.alpha = d->alpha;
      a.first = (k == 1); a.hermite = hermite; a.kdd = kdd; a.mcalc = mcalc; a.n = N;
      if (kdd > 1) {
        // weights of knot k start at zero before this interval adds to them
        GB_CUDA(cudaMemsetAsync(L.w[cur], 0, fb, st));
        if (hermite) GB_CUDA(cudaMemsetAsync(L.wd[cur], 0, fb, st));
      }
      k_lwt_interval<T><<<nb, 256, 0, st>>>(a);
      GB_CHECK_LAUNCH();
      // weights of knot k-1 are complete
      if (kdd > 1 && (rc = accumulate(k - 1, L.w[prv], L.wd[prv], k == 1))) return rc;
    }
    cur ^= 1;
  }
  const int last = cur ^ 1;
  if (kdd > 1) {
    if ((rc = accumulate(nsp - 1, L.w[last], L.wd[last], 0))) return rc;
    if (calc_v && (rc = inv3d(p, L.G, sfs, 1, L.pot2, 0, st))) return rc;
  }
  const double ld = fmax(0.1, d->ldw > 0 ? d->ldw : 1.0 / 6.0);
  k_lwt_final<T><<<nb, 256, 0, st>>>(N, rhoT, (const T*)L.kf, (const T*)L.ra, (const T*)L.pot1, (const T*)L.pot2,
                                      (const T*)L.pot3, d->alpha, d->beta, rmax, ld, calc_v, kdd > 1,
                                      reinterpret_cast<T*>(pot), L.part);
  GB_CHECK_LAUNCH();
  if (calc_e && energies) {
    k_lwt_energy<<<1, 256, 0, st>>>(L.part, nb, p->dV, energies);
    GB_CHECK_LAUNCH();
  }
  return 0;
}

}  // namespace

double kf_of_host(double rho) { return 2.0 * cbrt(3.0 * 9.86960440108935861883 * rho); }

int gb_lwt_eval(gbofdft_plan* p, const void* rho, gbofdft_lwt* d, void* pot, double* energies, int calc_v, int calc_e,
                cudaStream_t st) {
  GB_REQUIRE(d->work && d->ktab_c && d->dtab_c && d->neta >= 4, "lwt: tables or workspace missing");
  int64_t need = 0;
  gbofdft_lwt_workspace_bytes(p, &need);
  GB_REQUIRE(d->work_bytes >= need, "lwt: workspace %lld < %lld bytes", (long long)d->work_bytes, (long long)need);
  GB_REQUIRE(((uintptr_t)d->work & 255) == 0, "lwt: workspace must be 256-byte aligned");
  GB_REQUIRE(d->interp == 0 || d->interp == 1, "lwt: interp must be 0 (linear) or 1 (hermite)");
  GB_REQUIRE(d->kdd >= 1 && d->kdd <= 3 && d->ratio > 1.0, "lwt: bad kdd / ratio");
  return p->prec == GBOFDFT_F64 ? lwt_run<double>(p, rho, d, pot, energies, calc_v, calc_e, st)
                                : lwt_run<float>(p, rho, d, pot, energies, calc_v, calc_e, st);
}

extern "C" {

int gbofdft_lwt_workspace_bytes(const gbofdft_plan* p, int64_t* bytes) {
  GB_REQUIRE(p && bytes, "lwt_workspace_bytes: null argument");
  *bytes = (int64_t)(13 * lwt_field_bytes(p) + 6 * lwt_spec_bytes(p) + 2 * r256(sizeof(float) * 4 * kMaxNetaF32) +
                     r256(sizeof(double) * 8192));
  return GBOFDFT_OK;
}

int gbofdft_mgp_table(const double* gp, const double* coef, int m, const double* eta, int neta, int maxpoints,
                      double* table_out, void* stream) {
  GB_REQUIRE(gp && coef && eta && table_out && m >= 4 && neta >= 2 && maxpoints >= 1, "mgp_table: bad arguments");
  const double ctf = 0.3 * pow(3.0 * 9.86960440108935861883, 2.0 / 3.0);
  const double coe = 4.0 / 5.0 * ctf * 5.0 / 6.0 / (double)maxpoints;
  GB_REQUIRE(maxpoints <= 4096, "mgp_table: maxpoints %d > 4096", maxpoints);
  k_mgp_table<<<(neta + 127) / 128, 128, sizeof(double) * 2 * maxpoints, (cudaStream_t)stream>>>(
      gp, coef, m, eta, neta, maxpoints, coe, table_out);
  GB_CHECK_LAUNCH();
  return GBOFDFT_OK;
}

}  // extern "C"
