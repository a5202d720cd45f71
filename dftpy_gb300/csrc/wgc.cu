// WGC nonlocal kinetic term (density-dependent kernel, second-order
// expansion about the mean density rho*).  No reference counterpart: the
// method is Wang, Govind and Carter, Phys. Rev. B 60, 16350 (1999).
//
//   E_NL = int int rho^a(r) K(xi(r, r'); r - r') rho^b(r'),
//   xi = [ (k_F(r)^g + k_F(r')^g) / 2 ]^(1/g),
//   K(xi) = K0 + K1 (u + u')/6 + Kq (u^2 + u'^2) + Kx u u',  u = (rho - rho*)/rho*,
// K1 = k dK/dk, K2 = k^2 d^2K/dk^2, Kq = (g - 5)/72 K1 + K2/72,
// Kx = (1 - g)/36 K1 + K2/36, and the kernel's shape tabulated on the host so
// that the expanded functional keeps the Lindhard response at rho*.  With
//   X0 = K0*B + K1*(uB)/6 + Kq*(u^2 B), X1 = K1*B/6 + Kx*(uB), X2 = Kq*B
// (A = rho^a, B = rho^b; Y0..Y2 the same with A):
//   E = int A (X0 + u X1 + u^2 X2),
//   V = A'(X0 + u X1 + u^2 X2) + (A/rho*)(X1 + 2u X2) + B'(Y0 + u Y1 + u^2 Y2) + (B/rho*)(Y1 + 2u Y2).
// One evaluation: a pointwise pass (the 3 or 6 transformed fields), their
// forward transforms, one reciprocal-space pass forming X and Y, the
// inverse transforms and a pointwise pass adding V and reducing E.  With
// a == b, Y = X and half the transforms are skipped.
#include <math.h>

#include "gkernels.cuh"
#include "plan.h"

namespace {

constexpr double kZeroRho = 1e-30;

size_t r256(size_t x) { return (x + 255) & ~(size_t)255; }

struct WgcBufs {
  void* f[6];       // real fields: transform inputs, then X0..X2, Y0..Y2
  void* s[6];       // spectra (internal layout)
  double* part;     // per-CTA energy partials
  double* vref;     // FP64 plans: the NL potential of the last reference evaluation [N]
  double* eref;     // FP64 plans: its NL energy [1]
  double* pw[2];    // FP64 plans: rho^a and rho^b of the current evaluation [N] each
  void* o[6];       // FP32 plane-pipeline plans: the combinations' spectra (plane-major)
};

// FP32 plans whose grid has the plane pipeline run the WGC transforms there
bool wgc_plane(const gbofdft_plan* p) { return p->prec == GBOFDFT_F32 && p->plane_ok && gb_use_ct(); }

constexpr int kBlocks = 1216;
constexpr int kThreads = 256;

// per-CTA energy partials: the grid-stride passes use kBlocks, the fused
// inverse row pass of the plane pipeline one per pair of rows at most
int64_t wgc_part_count(const gbofdft_plan* p) {
  const int64_t rows = (int64_t)p->n[0] * p->n[1] / 2 + 1;
  return rows > kBlocks ? rows : kBlocks;
}

WgcBufs wgc_layout(const gbofdft_plan* p, void* work) {
  const size_t fb = r256(gb_elem(p) * (size_t)p->N), sb = r256(2 * gb_elem(p) * (size_t)p->NGld);
  char* b = reinterpret_cast<char*>(work);
  WgcBufs W;
  for (int i = 0; i < 6; ++i) { W.f[i] = b; b += fb; }
  for (int i = 0; i < 6; ++i) { W.s[i] = b; b += sb; }
  W.part = reinterpret_cast<double*>(b);
  b += r256(sizeof(double) * (size_t)wgc_part_count(p));
  W.vref = nullptr;
  W.eref = nullptr;
  W.pw[0] = W.pw[1] = nullptr;
  for (int i = 0; i < 6; ++i) W.o[i] = nullptr;
  if (p->prec == GBOFDFT_F64) {
    W.vref = reinterpret_cast<double*>(b);
    b += r256(sizeof(double) * (size_t)p->N);
    W.eref = reinterpret_cast<double*>(b);
    b += 256;
    for (int i = 0; i < 2; ++i) {
      W.pw[i] = reinterpret_cast<double*>(b);
      b += r256(sizeof(double) * (size_t)p->N);
    }
  } else if (wgc_plane(p)) {
    for (int i = 0; i < 6; ++i) { W.o[i] = b; b += sb; }
  }
  return W;
}

// FP64 workspaces keep a reference evaluation for the delta evaluations of
// the mixed-precision refinement: the X / Y fields of the last evaluation
// (in f[0..5]), its NL potential and energy
size_t wgc_bytes(const gbofdft_plan* p) {
  size_t b = 6 * r256(gb_elem(p) * (size_t)p->N) + 6 * r256(2 * gb_elem(p) * (size_t)p->NGld) +
             r256(sizeof(double) * (size_t)wgc_part_count(p));
  if (p->prec == GBOFDFT_F64) b += 3 * r256(sizeof(double) * (size_t)p->N) + 256;
  else if (wgc_plane(p)) b += 6 * r256(2 * gb_elem(p) * (size_t)p->NGld);
  return b;
}

// Column c of the kernel table at eta: cubic (Catmull-Rom) interpolation in
// t = ln(eta) on the uniform table grid; eta^2 scaling below the first point
// (the kernels go as eta^2 there), the last value beyond the table.
__device__ double table_at(const double* __restrict__ tab, int m, double t0, double h, int c, double eta) {
  const double* col = tab + (size_t)c * m;
  if (eta <= 0.0) return 0.0;
  const double t = log(eta);
  if (t <= t0) {
    const double r = eta / exp(t0);
    return col[0] * r * r;
  }
  const double x = (t - t0) / h;
  int i = (int)floor(x);
  if (i >= m - 1) return col[m - 1];
  const double u = x - i;
  const double y1 = col[i], y2 = col[i + 1];
  const double y0 = i > 0 ? col[i - 1] : 2.0 * y1 - y2;
  const double y3 = i + 2 < m ? col[i + 2] : 2.0 * y2 - y1;
  return y1 + 0.5 * u * ((y2 - y0) + u * ((2.0 * y0 - 5.0 * y1 + 4.0 * y2 - y3) + u * (3.0 * (y1 - y2) + y3 - y0)));
}

// K0, K1, Kq, Kx on the half spectrum (API layout, 4 consecutive arrays):
// C times the table columns at eta = |G| / 2k_F, partner-averaged on the
// symmetrised planes like the Wang-Teter kernel
template <typename T>
__global__ void k_wgc_kernels(GInfo g, double tkf, double C, const double* __restrict__ tab, int m, double t0,
                              double h, T* __restrict__ out) {
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int k2 = (int)(id % g.n2h);
    const int64_t r = id / g.n2h;
    const int i1 = (int)(r % g.n1), i0 = (int)(r / g.n1);
    for (int c = 0; c < 4; ++c) {
      const double v = gbk::sym_kernel<double>(
          g, i0, i1, k2, [&](double gg) { return C * table_at(tab, m, t0, h, c, sqrt(gg) / tkf); });
      out[c * total + id] = (T)v;
    }
  }
}

// plane-major copy of the four kernels: element (i0, i1, k2) of kernel c at
// pm[c NG + (k2 n0 + i0) n1 + i1]
__global__ void k_wgc_kernels_pm(GInfo g, const float* __restrict__ K, float* __restrict__ pm) {
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < 4 * total;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(id / total);
    const int64_t r = id - c * total;            // plane-major index within kernel c
    const int64_t plane = (int64_t)g.n0 * g.n1;
    const int k2 = (int)(r / plane);
    const int64_t rr = r - k2 * plane;           // i0 n1 + i1
    pm[id] = K[c * total + rr * g.n2h + k2];
  }
}

// pointwise arithmetic in the field precision (FP32 plans stay off the FP64 pipe)
__device__ __forceinline__ float wpow(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double wpow(double x, double y) { return pow(x, y); }

// A = rc^a and B = rc^b.  FP64: one logarithm and two exponentials instead
// of two pow calls (the FP64 pipe of this part is slow and these powers
// dominated the FP64 pointwise passes); exp(a ln rc) carries a relative error
// of about |a ln rc| ulp, below 1e-14 for rc >= 1e-30.
__device__ __forceinline__ void wpow2(float rc, float a, float b, int two, float& A, float& B) {
  B = powf(rc, b);
  A = two ? powf(rc, a) : B;
}
__device__ __forceinline__ void wpow2(double rc, double a, double b, int two, double& A, double& B) {
  const double L = log(rc);
  B = exp(b * L);
  A = two ? exp(a * L) : B;
}

// transform inputs: F0 = B, F1 = u B, F2 = u^2 B (and A, u A, u^2 A); pa / pb
// (optional) keep A and B for the final pass
template <typename T>
__global__ void k_wgc_prep(int64_t n, const T* __restrict__ rho, T rho0, T a, T b, int two, T* __restrict__ f0,
                           T* __restrict__ f1, T* __restrict__ f2, T* __restrict__ f3, T* __restrict__ f4,
                           T* __restrict__ f5, T* __restrict__ pa, T* __restrict__ pb) {
  const T inv0 = (T)1 / rho0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T rc = rho[i] > (T)kZeroRho ? rho[i] : (T)kZeroRho;
    const T u = (rc - rho0) * inv0;
    T A, B;
    wpow2(rc, a, b, two, A, B);
    if (pa) { pa[i] = A; pb[i] = B; }
    f0[i] = B;
    f1[i] = u * B;
    f2[i] = u * u * B;
    if (two) {
      f3[i] = A;
      f4[i] = u * A;
      f5[i] = u * u * A;
    }
  }
}

// X^ from the three spectra of one exponent (in place), scaled by 1/N
template <typename T>
__global__ void k_wgc_combine(GInfo g, int ld2, const T* __restrict__ K, T scale, cpx<T>* __restrict__ s0,
                              cpx<T>* __restrict__ s1, cpx<T>* __restrict__ s2) {
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int k2 = (int)(id % g.n2h);
    const int64_t r = id / g.n2h;
    const int64_t j = r * ld2 + k2;
    const T k0 = K[id], k1 = K[total + id] * (T)(1.0 / 6.0), kq = K[2 * total + id], kx = K[3 * total + id];
    const cpx<T> a = s0[j], bb = s1[j], c = s2[j];
    s0[j] = cpx<T>{(k0 * a.x + k1 * bb.x + kq * c.x) * scale, (k0 * a.y + k1 * bb.y + kq * c.y) * scale};
    s1[j] = cpx<T>{(k1 * a.x + kx * bb.x) * scale, (k1 * a.y + kx * bb.y) * scale};
    s2[j] = cpx<T>{kq * a.x * scale, kq * a.y * scale};
  }
}

// V added to pot and per-CTA partials of E = int A (X0 + u X1 + u^2 X2); the
// field arithmetic runs in T, the energy sum in FP64 (per-thread sums in T,
// combined in FP64 across threads and CTAs), and without CALC_E no FP64 at all
template <typename T, bool WANT_E>
__global__ void __launch_bounds__(kThreads) k_wgc_final(int64_t n, const T* __restrict__ rho, T rho0, T a, T b,
                                                         int two, const T* __restrict__ x0, const T* __restrict__ x1,
                                                         const T* __restrict__ x2, const T* __restrict__ y0,
                                                         const T* __restrict__ y1, const T* __restrict__ y2,
                                                         T* __restrict__ pot, int calc_v, double* __restrict__ part,
                                                         T* __restrict__ vstore, const T* __restrict__ pa,
                                                         const T* __restrict__ pb) {
  const T inv0 = (T)1 / rho0;
  T es = (T)0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T rc = rho[i] > (T)kZeroRho ? rho[i] : (T)kZeroRho;
    const T u = (rc - rho0) * inv0;
    const T A = pa ? pa[i] : wpow(rc, a);
    const T X0 = x0[i], X1 = x1[i], X2 = x2[i];
    const T sx = X0 + u * X1 + u * u * X2;
    if (WANT_E) es += A * sx;
    if (calc_v) {
      T v;
      if (two) {
        const T B = pb ? pb[i] : wpow(rc, b);
        const T Y0 = y0[i], Y1 = y1[i], Y2 = y2[i];
        v = a * A / rc * sx + A * inv0 * (X1 + (T)2 * u * X2) + b * B / rc * (Y0 + u * Y1 + u * u * Y2) +
            B * inv0 * (Y1 + (T)2 * u * Y2);
      } else {
        v = (T)2 * (a * A / rc * sx + A * inv0 * (X1 + (T)2 * u * X2));
      }
      pot[i] += v;
      if (vstore) vstore[i] = v;
    }
  }
  if constexpr (!WANT_E) return;
  __shared__ double red[kThreads / 32];
  const double v = warp_sum((double)es);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < kThreads / 32; ++w) t.add(red[w]);
    part[blockIdx.x] = t.value();
  }
}

// The FP32 potential-only final pass, four points per thread with 16-byte
// loads and stores (n % 4 == 0; the fields are 16-byte aligned): the
// per-point pass is latency-bound on its seven input streams otherwise.
__global__ void __launch_bounds__(kThreads) k_wgc_final_v4(int64_t n4, const float4* __restrict__ rho, float rho0,
                                                            float a, float b, int two, const float4* __restrict__ x0,
                                                            const float4* __restrict__ x1,
                                                            const float4* __restrict__ x2,
                                                            const float4* __restrict__ y0,
                                                            const float4* __restrict__ y1,
                                                            const float4* __restrict__ y2,
                                                            float4* __restrict__ pot) {
  const float inv0 = 1.0f / rho0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 r4 = rho[i], X04 = x0[i], X14 = x1[i], X24 = x2[i];
    float4 Y04 = X04, Y14 = X14, Y24 = X24;
    if (two) {
      Y04 = y0[i];
      Y14 = y1[i];
      Y24 = y2[i];
    }
    float4 p4 = pot[i];
    const float* rr = &r4.x;
    const float *X0 = &X04.x, *X1 = &X14.x, *X2 = &X24.x, *Y0 = &Y04.x, *Y1 = &Y14.x, *Y2 = &Y24.x;
    float* pp = &p4.x;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float rc = rr[k] > (float)kZeroRho ? rr[k] : (float)kZeroRho;
      const float u = (rc - rho0) * inv0;
      const float A = powf(rc, a);
      const float sx = X0[k] + u * X1[k] + u * u * X2[k];
      float v;
      if (two) {
        const float B = powf(rc, b);
        v = a * A / rc * sx + A * inv0 * (X1[k] + 2.0f * u * X2[k]) +
            b * B / rc * (Y0[k] + u * Y1[k] + u * u * Y2[k]) + B * inv0 * (Y1[k] + 2.0f * u * Y2[k]);
      } else {
        v = 2.0f * (a * A / rc * sx + A * inv0 * (X1[k] + 2.0f * u * X2[k]));
      }
      pp[k] += v;
    }
    pot[i] = p4;
  }
}

// energies[NL] and energies[TOTAL] += base + dV * sum(partials) (e may be
// null); eref (may be null) = dV * sum(partials)
__global__ void k_wgc_energy(const double* __restrict__ part, int nb, double dV, double* __restrict__ e,
                             double* __restrict__ eref, const double* __restrict__ base) {
  __shared__ double red[32];
  KSum s;
  s.init();
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s.add(part[i]);
  const double v = warp_sum(s.value());
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t.add(red[w]);
    const double en = t.value() * dV + (base ? *base : 0.0);
    if (e) {
      e[GB_E_NL] += en;
      e[GB_E_TOTAL] += en;
    }
    if (eref) *eref = en;
  }
}

// X0..X2 (and Y0..Y2) into W.f[0..5] on the plane pipeline (FP32): the
// transform inputs are made from rho in the forward row pass (rho given) or
// read from W.f[0..5] (rho null); K: the plane-major kernels.  pot given
// (potential-only evaluations): the inverse row pass adds the NL potential
// to pot directly instead of storing the fields.
int wgc_xfields_plane(gbofdft_plan* p, const WgcBufs& W, int two, const float* K, const float* rho,
                      const gbofdft_wgc* d, cudaStream_t st, float* pot = nullptr, double* part = nullptr,
                      int64_t* nblk = nullptr) {
  const int nfield = two ? 6 : 3;
  const int64_t fs = (int64_t)((char*)W.s[1] - (char*)W.s[0]) / (int64_t)sizeof(float2);
  const int64_t os = (int64_t)((char*)W.o[1] - (char*)W.o[0]) / (int64_t)sizeof(float2);
  const int64_t rs = (int64_t)((char*)W.f[1] - (char*)W.f[0]) / (int64_t)sizeof(float);
  int rc = 0;
  if (rho) {
    rc = gb_ct_rows_fwd_wgc_pm_f32(p, rho, W.s[0], fs, d->beta, d->rho0, st);
    if (!rc && two) rc = gb_ct_rows_fwd_wgc_pm_f32(p, rho, W.s[3], fs, d->alpha, d->rho0, st);
  } else {
    const int op = OP_RHO;
    for (int i = 0; i < nfield && !rc; ++i) rc = gb_ct_rows_fwd_pm_f32(p, W.f[i], W.s[i], fs, 1, &op, 1.0, st);
  }
  if (!rc) rc = gb_plane_fwd_f32(p, W.s[0], fs, nfield, st);
  if (!rc) rc = gb_plane_wgc_inv_f32(p, W.s[0], fs, W.o[0], os, two ? 2 : 1, K, 1.0 / (double)p->N, st);
  if (!rc && pot && rho) {
    rc = gb_ct_rows_inv_wgc_pm_f32(p, W.o[0], os, two, rho, d->rho0, d->alpha, d->beta, pot, part, nblk, st);
    if (rc == 1) return gb_set_error(GBOFDFT_ERR_STATE, "wgc: plane size without specialisation");
    return rc;
  }
  for (int h = 0; h < (two ? 2 : 1) && !rc; ++h) rc = gb_ct_rows_inv_store_pm_f32(p, W.o[3 * h], os, 3, W.f[3 * h], rs, st);
  if (rc == 1) return gb_set_error(GBOFDFT_ERR_STATE, "wgc: plane size without specialisation");
  return rc;
}

// X0..X2 (and Y0..Y2) into W.f[0..5] from the transform inputs in W.f[0..5]
template <typename T>
int wgc_xfields(gbofdft_plan* p, const WgcBufs& W, int two, const void* kernels, cudaStream_t st) {
  const int nfield = two ? 6 : 3;
  const int op = OP_RHO;
  for (int i = 0; i < nfield; ++i) {
    int rc = gb_rows_fwd(p, W.f[i], W.s[i], 0, p->ld2, 1, &op, 1.0, 1.0, st);
    if (!rc) rc = gb_cols(p, W.s[i], 0, p->ld2, 1, 1, -1, 1.0, st);
    if (!rc) rc = gb_cols(p, W.s[i], 0, p->ld2, 1, 0, -1, 1.0, st);
    if (rc) return rc;
  }
  const T* K = reinterpret_cast<const T*>(kernels);
  const T scale = (T)(1.0 / (double)p->N);
  for (int h = 0; h < (two ? 2 : 1); ++h) {
    k_wgc_combine<T><<<kBlocks, kThreads, 0, st>>>(p->gi, p->ld2, K, scale, (cpx<T>*)W.s[3 * h],
                                                    (cpx<T>*)W.s[3 * h + 1], (cpx<T>*)W.s[3 * h + 2]);
    GB_CHECK_LAUNCH();
    gb_count_launch();
  }
  const int64_t fstride = (int64_t)((char*)W.s[1] - (char*)W.s[0]) / (int64_t)(2 * gb_elem(p));
  const int64_t ostride = (int64_t)((char*)W.f[1] - (char*)W.f[0]) / (int64_t)gb_elem(p);
  for (int h = 0; h < (two ? 2 : 1); ++h) {
    int rc = gb_cols(p, W.s[3 * h], fstride, p->ld2, 3, 0, 1, 1.0, st);
    if (!rc) rc = gb_cols(p, W.s[3 * h], fstride, p->ld2, 3, 1, 1, 1.0, st);
    if (!rc) rc = gb_rows_inv_store(p, W.s[3 * h], fstride, p->ld2, 3, W.f[3 * h], ostride, 1.0, st);
    if (rc) return rc;
  }
  return 0;
}

// store_ref (FP64 plans): also keep the NL potential and energy as the
// reference of later delta evaluations (the X / Y fields stay in W.f)
template <typename T>
int wgc_run(gbofdft_plan* p, const void* rho, const gbofdft_wgc* d, void* pot, double* energies, int calc_v,
            int calc_e, int store_ref, cudaStream_t st) {
  WgcBufs W = wgc_layout(p, d->work);
  const int two = fabs(d->alpha - d->beta) > 1e-12;
  const T* r = reinterpret_cast<const T*>(rho);
  int rc;
  if (wgc_plane(p) && p->wgc_pm && p->wgc_pm_src == d->kernels) {
    if (calc_v && !store_ref) {
      // the inverse rows add the potential themselves (and sum the energy
      // integrand per CTA) instead of storing the six fields
      int64_t nblk = 0;
      rc = wgc_xfields_plane(p, W, two, p->wgc_pm, reinterpret_cast<const float*>(rho), d, st,
                             reinterpret_cast<float*>(pot), calc_e ? W.part : nullptr, &nblk);
      if (rc || !calc_e) return rc;
      if (nblk > wgc_part_count(p)) return gb_set_error(GBOFDFT_ERR_STATE, "wgc: partials buffer too small");
      k_wgc_energy<<<1, 256, 0, st>>>(W.part, (int)nblk, p->dV, energies, nullptr, nullptr);
      GB_CHECK_LAUNCH();
      gb_count_launch();
      return 0;
    }
    rc = wgc_xfields_plane(p, W, two, p->wgc_pm, reinterpret_cast<const float*>(rho), d, st);
  } else {
    k_wgc_prep<T><<<kBlocks, kThreads, 0, st>>>(p->N, r, (T)d->rho0, (T)d->alpha, (T)d->beta, two, (T*)W.f[0],
                                                (T*)W.f[1], (T*)W.f[2], (T*)W.f[3], (T*)W.f[4], (T*)W.f[5],
                                                (T*)W.pw[0], (T*)W.pw[1]);
    GB_CHECK_LAUNCH();
    gb_count_launch();
    rc = wgc_xfields<T>(p, W, two, d->kernels, st);
  }
  if (rc) return rc;
  T* vstore = nullptr;
  if (store_ref) {
    calc_v = 1;
    vstore = reinterpret_cast<T*>(W.vref);
  }
  const int want_e = calc_e || store_ref;
  const T* y = reinterpret_cast<const T*>(two ? W.f[3] : W.f[0]);
  auto a16 = [](const void* q) { return ((uintptr_t)q & 15) == 0; };
  if constexpr (sizeof(T) == 4) {
    if (!want_e && calc_v && p->N % 4 == 0 && a16(rho) && a16(pot) && a16(W.f[0]) && a16(W.f[1]) && a16(W.f[2]) &&
        a16(y) && (!two || (a16(W.f[4]) && a16(W.f[5])))) {
      const int64_t n4 = p->N / 4;
      const int nb = (int)((n4 + kThreads - 1) / kThreads < 4 * kBlocks ? (n4 + kThreads - 1) / kThreads : 4 * kBlocks);
      k_wgc_final_v4<<<nb, kThreads, 0, st>>>(
          n4, reinterpret_cast<const float4*>(rho), (float)d->rho0, (float)d->alpha, (float)d->beta, two,
          reinterpret_cast<const float4*>(W.f[0]), reinterpret_cast<const float4*>(W.f[1]),
          reinterpret_cast<const float4*>(W.f[2]), reinterpret_cast<const float4*>(y),
          two ? reinterpret_cast<const float4*>(W.f[4]) : nullptr,
          two ? reinterpret_cast<const float4*>(W.f[5]) : nullptr, reinterpret_cast<float4*>(pot));
      GB_CHECK_LAUNCH();
      gb_count_launch();
      return 0;
    }
  }
  if (want_e)
    k_wgc_final<T, true><<<kBlocks, kThreads, 0, st>>>(p->N, r, (T)d->rho0, (T)d->alpha, (T)d->beta, two,
                                                       (const T*)W.f[0], (const T*)W.f[1], (const T*)W.f[2], y,
                                                       two ? (const T*)W.f[4] : nullptr,
                                                       two ? (const T*)W.f[5] : nullptr, (T*)pot, calc_v, W.part,
                                                       vstore, (const T*)W.pw[0], (const T*)W.pw[1]);
  else
    k_wgc_final<T, false><<<kBlocks, kThreads, 0, st>>>(p->N, r, (T)d->rho0, (T)d->alpha, (T)d->beta, two,
                                                        (const T*)W.f[0], (const T*)W.f[1], (const T*)W.f[2], y,
                                                        two ? (const T*)W.f[4] : nullptr,
                                                        two ? (const T*)W.f[5] : nullptr, (T*)pot, calc_v, W.part,
                                                        vstore, (const T*)W.pw[0], (const T*)W.pw[1]);
  GB_CHECK_LAUNCH();
  gb_count_launch();
  if (want_e) {
    k_wgc_energy<<<1, 256, 0, st>>>(W.part, kBlocks, p->dV, calc_e ? energies : nullptr,
                                    store_ref ? W.eref : nullptr, nullptr);
    GB_CHECK_LAUNCH();
    gb_count_launch();
  }
  return 0;
}

// ---- delta evaluation (FP64 result from FP32 transforms of the change) -----
//
// For a density rho close to the reference rho_r of the last store_ref
// evaluation, the transform inputs F = {B, uB, u^2 B, A, uA, u^2 A} change by
// dF, and by linearity X(rho) = X(rho_r) + K * dF.  dF is formed from the
// two FP64 densities with relative FP32 accuracy in the change (power laws
// as b^p expm1(p log1p((a - b)/b)), products as d(fg) = df g + f_r dg),
// transformed by the FP32 plan, and the NL potential and energy are formed
// as FP32 changes on the stored FP64 reference: the error is ~1e-7 of the
// change, not of the value.

struct WgcDeltaPt {
  float dA, A, Ar, dAp, Apr, dB, B, Br, dBp, Bpr, du, u, ur;
};

// the power-law factors at rho and their changes from rho_r (both clamped at 1e-30)
__device__ __forceinline__ WgcDeltaPt wgc_delta_point(double rho, double rref, double rho0, float a, float b) {
  const double rc = rho > kZeroRho ? rho : kZeroRho;
  const double rr = rref > kZeroRho ? rref : kZeroRho;
  const float rf = (float)rr;
  const float d = (float)(rc - rr);
  const float L = log1pf(d / rf);
  WgcDeltaPt q;
  q.Ar = powf(rf, a);
  q.dA = q.Ar * expm1f(a * L);
  q.A = q.Ar + q.dA;
  q.Apr = a * q.Ar / rf;
  q.dAp = q.Apr * expm1f((a - 1.0f) * L);
  q.Br = powf(rf, b);
  q.dB = q.Br * expm1f(b * L);
  q.B = q.Br + q.dB;
  q.Bpr = b * q.Br / rf;
  q.dBp = q.Bpr * expm1f((b - 1.0f) * L);
  const float inv0 = (float)(1.0 / rho0);
  q.ur = (float)((rr - rho0) / rho0);
  q.du = d * inv0;
  q.u = q.ur + q.du;
  return q;
}

// dF (FP32) into f0..f5
__global__ void k_wgc_delta_prep(int64_t n, const double* __restrict__ rho, const double* __restrict__ rref,
                                 double rho0, float a, float b, int two, float* __restrict__ f0,
                                 float* __restrict__ f1, float* __restrict__ f2, float* __restrict__ f3,
                                 float* __restrict__ f4, float* __restrict__ f5) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const WgcDeltaPt q = wgc_delta_point(rho[i], rref[i], rho0, a, b);
    const float du2 = q.du * (q.u + q.ur);          // u^2 - u_r^2
    const float ur2 = q.ur * q.ur;
    f0[i] = q.dB;
    f1[i] = q.du * q.B + q.ur * q.dB;
    f2[i] = du2 * q.B + ur2 * q.dB;
    if (two) {
      f3[i] = q.dA;
      f4[i] = q.du * q.A + q.ur * q.dA;
      f5[i] = du2 * q.A + ur2 * q.dA;
    }
  }
}

// pot += V_r + dV and per-CTA partials of the energy change; xr: the FP64
// reference X / Y fields, dx: their FP32 changes
template <bool WANT_E>
__global__ void __launch_bounds__(kThreads) k_wgc_delta_final(
    int64_t n, const double* __restrict__ rho, const double* __restrict__ rref, double rho0, float a, float b,
    int two, const double* __restrict__ xr0, const double* __restrict__ xr1, const double* __restrict__ xr2,
    const double* __restrict__ yr0, const double* __restrict__ yr1, const double* __restrict__ yr2,
    const float* __restrict__ dx0, const float* __restrict__ dx1, const float* __restrict__ dx2,
    const float* __restrict__ dy0, const float* __restrict__ dy1, const float* __restrict__ dy2,
    const double* __restrict__ vref, double* __restrict__ pot, double* __restrict__ part) {
  const float inv0 = (float)(1.0 / rho0);
  float es = 0.0f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const WgcDeltaPt q = wgc_delta_point(rho[i], rref[i], rho0, a, b);
    const float du2 = q.du * (q.u + q.ur);
    // sx = X0 + u X1 + u^2 X2 and tx = X1 + 2 u X2 at rho, and their changes
    const float X0 = (float)xr0[i], X1 = (float)xr1[i], X2 = (float)xr2[i];
    const float d0 = dx0[i], d1 = dx1[i], d2 = dx2[i];
    const float dsx = d0 + q.u * d1 + q.du * X1 + q.u * q.u * d2 + du2 * X2;
    const float sx = X0 + q.ur * X1 + q.ur * q.ur * X2 + dsx;
    const float dtx = d1 + 2.0f * (q.u * d2 + q.du * X2);
    const float tx = X1 + 2.0f * q.ur * X2 + dtx;
    float dv = q.dAp * sx + q.Apr * dsx + (q.dA * tx + q.Ar * dtx) * inv0;
    if (two) {
      const float Y0 = (float)yr0[i], Y1 = (float)yr1[i], Y2 = (float)yr2[i];
      const float e0 = dy0[i], e1 = dy1[i], e2 = dy2[i];
      const float dsy = e0 + q.u * e1 + q.du * Y1 + q.u * q.u * e2 + du2 * Y2;
      const float sy = Y0 + q.ur * Y1 + q.ur * q.ur * Y2 + dsy;
      const float dty = e1 + 2.0f * (q.u * e2 + q.du * Y2);
      const float ty = Y1 + 2.0f * q.ur * Y2 + dty;
      dv += q.dBp * sy + q.Bpr * dsy + (q.dB * ty + q.Br * dty) * inv0;
    } else {
      dv *= 2.0f;
    }
    pot[i] += vref[i] + (double)dv;
    if (WANT_E) es += q.dA * sx + q.Ar * dsx;
  }
  if constexpr (!WANT_E) return;
  __shared__ double red[kThreads / 32];
  const double v = warp_sum((double)es);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < kThreads / 32; ++w) t.add(red[w]);
    part[blockIdx.x] = t.value();
  }
}

}  // namespace

static int wgc_check(const gbofdft_plan* p, const gbofdft_wgc* d) {
  GB_REQUIRE(d->kernels && d->work, "wgc: kernels or workspace missing");
  GB_REQUIRE(d->rho0 > 0.0, "wgc: rho0 must be positive (got %g)", d->rho0);
  GB_REQUIRE(d->work_bytes >= (int64_t)wgc_bytes(p), "wgc: workspace %lld < %lld bytes", (long long)d->work_bytes,
             (long long)wgc_bytes(p));
  GB_REQUIRE(((uintptr_t)d->work & 255) == 0, "wgc: workspace must be 256-byte aligned");
  return 0;
}

int gb_wgc_eval(gbofdft_plan* p, const void* rho, const gbofdft_wgc* d, void* pot, double* energies, int calc_v,
                int calc_e, int store_ref, cudaStream_t st) {
  int rc = wgc_check(p, d);
  if (rc) return rc;
  GB_REQUIRE(!store_ref || p->prec == GBOFDFT_F64, "wgc: a delta reference needs an FP64 plan");
  return p->prec == GBOFDFT_F64 ? wgc_run<double>(p, rho, d, pot, energies, calc_v, calc_e, store_ref, st)
                                : wgc_run<float>(p, rho, d, pot, energies, calc_v, calc_e, 0, st);
}

int gb_wgc_eval_delta(gbofdft_plan* p64, gbofdft_plan* p32, const double* rho, const double* rho_ref,
                      const gbofdft_wgc* d64, const gbofdft_wgc* d32, double* pot, double* energies, int calc_e,
                      cudaStream_t st) {
  int rc = wgc_check(p64, d64);
  if (!rc) rc = wgc_check(p32, d32);
  if (rc) return rc;
  GB_REQUIRE(p64->prec == GBOFDFT_F64 && p32->prec == GBOFDFT_F32, "wgc delta: needs an FP64 and an FP32 plan");
  GB_REQUIRE(fabs(d64->alpha - d32->alpha) < 1e-12 && fabs(d64->beta - d32->beta) < 1e-12,
             "wgc delta: the FP64 and FP32 terms have different exponents");
  GB_REQUIRE(fabs(d64->rho0 - d32->rho0) <= 1e-6 * d64->rho0,
             "wgc delta: the FP32 kernels were built at another mean density (%g vs %g)", d32->rho0, d64->rho0);
  WgcBufs W64 = wgc_layout(p64, d64->work);
  WgcBufs W32 = wgc_layout(p32, d32->work);
  const int two = fabs(d64->alpha - d64->beta) > 1e-12;
  const float a = (float)d64->alpha, b = (float)d64->beta;
  float* f[6];
  for (int i = 0; i < 6; ++i) f[i] = reinterpret_cast<float*>(W32.f[i]);
  k_wgc_delta_prep<<<kBlocks, kThreads, 0, st>>>(p64->N, rho, rho_ref, d64->rho0, a, b, two, f[0], f[1], f[2], f[3],
                                                 f[4], f[5]);
  GB_CHECK_LAUNCH();
  gb_count_launch();
  if (wgc_plane(p32) && p32->wgc_pm && p32->wgc_pm_src == d32->kernels)
    rc = wgc_xfields_plane(p32, W32, two, p32->wgc_pm, nullptr, d32, st);
  else
    rc = wgc_xfields<float>(p32, W32, two, d32->kernels, st);
  if (rc) return rc;
  const double* xr[6];
  for (int i = 0; i < 6; ++i) xr[i] = reinterpret_cast<const double*>(W64.f[two || i < 3 ? i : i - 3]);
  const float* dy[3] = {f[two ? 3 : 0], f[two ? 4 : 1], f[two ? 5 : 2]};
  if (calc_e)
    k_wgc_delta_final<true><<<kBlocks, kThreads, 0, st>>>(p64->N, rho, rho_ref, d64->rho0, a, b, two, xr[0], xr[1],
                                                          xr[2], xr[3], xr[4], xr[5], f[0], f[1], f[2], dy[0], dy[1],
                                                          dy[2], W64.vref, pot, W64.part);
  else
    k_wgc_delta_final<false><<<kBlocks, kThreads, 0, st>>>(p64->N, rho, rho_ref, d64->rho0, a, b, two, xr[0], xr[1],
                                                           xr[2], xr[3], xr[4], xr[5], f[0], f[1], f[2], dy[0], dy[1],
                                                           dy[2], W64.vref, pot, W64.part);
  GB_CHECK_LAUNCH();
  gb_count_launch();
  if (calc_e) {
    k_wgc_energy<<<1, 256, 0, st>>>(W64.part, kBlocks, p64->dV, energies, nullptr, W64.eref);
    GB_CHECK_LAUNCH();
    gb_count_launch();
  }
  return 0;
}

extern "C" {

int gbofdft_wgc_workspace_bytes(const gbofdft_plan* p, int64_t* bytes) {
  GB_REQUIRE(p && bytes, "wgc_workspace_bytes: null argument");
  *bytes = (int64_t)wgc_bytes(p);
  return GBOFDFT_OK;
}

int gbofdft_wgc_kernels(gbofdft_plan* p, double rho0, double alpha, double beta, const double* table, int m,
                        double t0, double h, void* out, void* stream) {
  GB_REQUIRE(p && out && table, "wgc_kernels: null argument");
  GB_REQUIRE(rho0 > 0.0, "wgc_kernels: rho0 must be positive (got %g)", rho0);
  GB_REQUIRE(m >= 4 && h > 0.0, "wgc_kernels: table needs >= 4 points and a positive step");
  GB_REQUIRE(alpha > 0.0 && beta > 0.0, "wgc_kernels: alpha, beta must be positive");
  const double kPi = 3.14159265358979323846;
  const double tkf = 2.0 * cbrt(3.0 * rho0 * kPi * kPi);
  const double ctf = 0.3 * pow(3.0 * kPi * kPi, 2.0 / 3.0);
  const double C = 5.0 / (9.0 * alpha * beta * pow(rho0, alpha + beta - 5.0 / 3.0)) * ctf;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t total = p->NG;
  const int nblk = (int)((total + 255) / 256 > 4096 ? 4096 : (total + 255) / 256);
  if (p->prec == GBOFDFT_F64)
    k_wgc_kernels<double><<<nblk, 256, 0, st>>>(p->gi, tkf, C, table, m, t0, h, (double*)out);
  else
    k_wgc_kernels<float><<<nblk, 256, 0, st>>>(p->gi, tkf, C, table, m, t0, h, (float*)out);
  GB_CHECK_LAUNCH();
  gb_count_launch();
  if (wgc_plane(p)) {
    // plans with the plane pipeline keep a plane-major copy (allocated with
    // the first kernels built on the plan)
    if (!p->wgc_pm) {
      cudaError_t e = cudaMalloc(&p->wgc_pm, sizeof(float) * 4 * (size_t)p->NG);
      if (e != cudaSuccess) {
        p->wgc_pm = nullptr;
        return gb_set_error(GBOFDFT_ERR_ALLOC, "wgc kernels: plane-major copy: %s", cudaGetErrorString(e));
      }
    }
    const int64_t n4 = 4 * total;
    k_wgc_kernels_pm<<<(int)((n4 + 255) / 256 > 4096 ? 4096 : (n4 + 255) / 256), 256, 0, st>>>(
        p->gi, reinterpret_cast<const float*>(out), p->wgc_pm);
    GB_CHECK_LAUNCH();
    gb_count_launch();
    p->wgc_pm_src = out;
  }
  return GBOFDFT_OK;
}

}  // extern "C"
