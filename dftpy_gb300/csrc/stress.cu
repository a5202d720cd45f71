// Stress tensors (3 x 3, Ha/Bohr^3) of the terms of TotalFunctional.get_stress
// (src/dftpy/functional/total_functional.py:176-209):
//
//   TF        kedf/tf.py:52-62        -(2/3) E_TF / Omega  (diagonal)
//   vW        kedf/vw.py:97-112       -(y/4) dV/Omega sum_r d_i rho d_j rho / rho,
//                                      d_i rho = ifft(i G_i rho(G))
//   WT        kedf/wt.py:75-105       F sum_mask (G_i G_j / G^2 - delta_ij / 3) L'(q / 2k_F)
//                                      Re(rho^a(G) conj(rho^b(G))) / Omega^2 - (2/3) E_NL / Omega
//   LDA       xc/semilocal_xc.py:308-322   (E_xc - int V_xc rho) / Omega  (diagonal)
//   Hartree   hartree.py:68-90        8 pi / Omega^2 sum_mask G_i G_j |rho(G)|^2 / G^4 - E_H / Omega
//   PP (PME)  pseudo/__init__.py:525-562, (exact) :431-455
//   Ewald     ewald.py:523-538, 609-662 (real), 719-760 (exact rec), 915-963 (PME rec)
//
// Every G-space term is one reduction over the reference's half-space mask
// of a per-G weight times G_i G_j (six sums) and a scalar sum; the real-space
// terms reduce to the same seven slots.  Per-CTA partials are summed in a
// fixed order (deterministic), and a small kernel assembles
//   out_ij (+)= A s_ij + delta_ij (B s_7 + C)
// with scalars the host derives from the energies.
#include <math.h>
#include <string.h>

#include "gkernels.cuh"
#include "passes_ct.cuh"
#include "pseudo.cuh"

namespace {

constexpr int kSB = 512;       // CTAs of the grid-sized reductions
constexpr int kST = 256;       // threads per CTA
constexpr int kNS = 7;         // xx xy xz yy yz zz, scalar

enum { SM_HARTREE = 0, SM_WT = 1, SM_PP_PME = 2, SM_PP_EXACT = 3, SM_EWALD = 4 };

// d v / dq of a species table: the derivative of its cubic spline on
// gp[1:] (the first piece extrapolated below gp[1]), 0 from gp[-1] on
// (LocalPseudo._PP_Derivative_One, pseudo/__init__.py:406-412).
__device__ double vline_deriv(const gbofdft_vtable& t, double q) {
  if (!(q < t.gmax)) return 0.0;
  int lo = 0;
  if (q >= __ldg(t.x)) {
    int hi = t.m - 1;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(t.x + mid) <= q) lo = mid; else hi = mid;
    }
  }
  const double u = q - __ldg(t.x + lo);
  const double* cc = t.c + 4 * (size_t)lo;
  return __ldg(cc + 1) + u * (2.0 * __ldg(cc + 2) + u * 3.0 * __ldg(cc + 3));
}

// derivative of the inverse Lindhard function times eta (kedf/kernel.py:197-211)
__device__ double lindhard_deriv(double eta, double mu) {
  const double atol = 1.0e-10;
  double d;
  if (eta < atol) {
    d = -2.0 * eta * (1.0 / 3.0 - 3.0 * mu);
  } else if (fabs(eta - 1.0) < atol) {
    d = -48.0;
  } else {
    const double t = log(fabs((1.0 + eta) / (1.0 - eta)));
    const double den = 0.5 + 0.25 * (1.0 - eta * eta) / eta * t;
    d = (0.5 / eta - 0.25 * (eta * eta + 1.0) / (eta * eta) * t) / (den * den) + 6.0 * eta * mu;
  }
  return d * eta;
}

struct GsArgs {
  GInfo g;
  int mode;
  const void* a;           // HARTREE, PP: rho(G); WT: rho^alpha(G); EWALD: S(G) (PME: FFT(Q), times B here)
  const void* b;           // WT: rho^beta(G); PP_PME: FFT(Q_s)
  const double2 *bm0, *bm1, *bm2;  // PME b(m) (PP_PME, EWALD with PME)
  gbofdft_vtable vt;       // PP_PME: this species' table
  VTabs vts;               // PP_EXACT: all tables
  const int* species;
  int nat;
  const double2 *ph0, *ph1, *ph2;  // PP_EXACT phase tables
  double tkf, eta;
  double* partial;         // [gridDim.x][kNS]
};

template <typename T>
__device__ __forceinline__ double2 ld2(const void* p, int64_t i) {
  const cpx<T> v = reinterpret_cast<const cpx<T>*>(p)[i];
  return double2{(double)v.x, (double)v.y};
}

__device__ __forceinline__ void block_store7(double (&s)[kNS], double* partial) {
  __shared__ double red[kST / 32][kNS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kNS; ++k) {
    const double v = warp_sum(s[k]);
    if (lane == 0) red[w][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < kNS) {
    KSum t;
    t.init();
    for (int ww = 0; ww < kST / 32; ++ww) t.add(red[ww][threadIdx.x]);
    partial[(int64_t)blockIdx.x * kNS + threadIdx.x] = t.value();
  }
}

template <typename T>
__global__ void __launch_bounds__(kST) k_gstress(GsArgs a) {
  const GInfo& g = a.g;
  double s[kNS] = {0, 0, 0, 0, 0, 0, 0};
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    int i0, i1, k2;
    decode(g, id, i0, i1, k2);
    if (!gmask(g, i0, i1, k2)) continue;
    const int m0 = ffreq(i0, g.n0), m1 = ffreq(i1, g.n1), m2 = m2_of(g, k2);
    const double gx = m0 * g.bg[0] + m1 * g.bg[3] + m2 * g.bg[6];
    const double gy = m0 * g.bg[1] + m1 * g.bg[4] + m2 * g.bg[7];
    const double gz = m0 * g.bg[2] + m1 * g.bg[5] + m2 * g.bg[8];
    const double gg = gx * gx + gy * gy + gz * gz;
    double w = 0.0, ws = 0.0;   // weight of G_i G_j, scalar contribution
    if (a.mode == SM_HARTREE) {
      if (!(gg > 0.0)) continue;
      const double2 r = ld2<T>(a.a, id);
      w = (r.x * r.x + r.y * r.y) / (gg * gg);
    } else if (a.mode == SM_WT) {
      const double2 A = ld2<T>(a.a, id), B = ld2<T>(a.b, id);
      const double dd = lindhard_deriv(sqrt(gg) / a.tkf, 1.0) * (A.x * B.x + A.y * B.y);
      w = gg > 0.0 ? dd / gg : 0.0;
      ws = dd;
    } else if (a.mode == SM_PP_PME) {
      if (!(gg > 0.0)) continue;
      const double q = sqrt(gg);
      const double2 r = ld2<T>(a.a, id), Q = ld2<T>(a.b, id);
      const double2 b = bprod(a.bm0, a.bm1, a.bm2, i0, i1, k2);
      // Re(conj(r) b Q) v'(q) / q
      const double bqx = b.x * Q.x - b.y * Q.y, bqy = b.x * Q.y + b.y * Q.x;
      w = (r.x * bqx + r.y * bqy) * vline_deriv(a.vt, q) / q;
    } else if (a.mode == SM_PP_EXACT) {
      if (!(gg > 0.0)) continue;
      const double q = sqrt(gg);
      double vx = 0.0, vy = 0.0;   // sum_a v'_s(a)(q) conj(exp(-i G.R_a))
      double dv[GBOFDFT_MAX_SPECIES];
      for (int sp = 0; sp < a.vts.n; ++sp) dv[sp] = vline_deriv(a.vts.t[sp], q);
      for (int at = 0; at < a.nat; ++at) {
        const double2 e = phase(a.ph0, a.ph1, a.ph2, g, at, i0, i1, k2);
        const double d = dv[a.species[at]];
        vx += d * e.x;
        vy -= d * e.y;
      }
      const double2 r = ld2<T>(a.a, id);
      w = (r.x * vx - r.y * vy) / q;
    } else {  // SM_EWALD
      if (!(gg > 0.0)) continue;
      double2 S = ld2<T>(a.a, id);
      if (a.bm0) {
        const double2 b = bprod(a.bm0, a.bm1, a.bm2, i0, i1, k2);
        S = double2{S.x * b.x - S.y * b.y, S.x * b.y + S.y * b.x};
      }
      const double e = (S.x * S.x + S.y * S.y) * exp(-gg / (4.0 * a.eta)) / gg;
      w = e * 2.0 * (1.0 + gg / (4.0 * a.eta)) / gg;
      ws = e;
    }
    s[0] += gx * gx * w; s[1] += gx * gy * w; s[2] += gx * gz * w;
    s[3] += gy * gy * w; s[4] += gy * gz * w; s[5] += gz * gz * w;
    s[6] += ws;
  }
  block_store7(s, a.partial);
}

// sums7 (+)= fixed-order sum of the per-CTA partials
__global__ void k_reduce7(const double* __restrict__ partial, int nblk, double* __restrict__ sums7, int accumulate) {
  const int k = threadIdx.x;
  if (k >= kNS) return;
  KSum t;
  t.init();
  for (int b = 0; b < nblk; ++b) t.add(partial[(int64_t)b * kNS + k]);
  sums7[k] = accumulate ? sums7[k] + t.value() : t.value();
}

// out_ij (+)= A s_ij + delta_ij (B s_7 + C)
__global__ void k_assemble(const double* __restrict__ s7, double A, double B, double C, double* __restrict__ out,
                           int accumulate) {
  const int k = threadIdx.x;
  if (k >= 9) return;
  const int i = k / 3, j = k % 3;
  const int lo = i < j ? i : j, hi = i < j ? j : i;
  const int idx = lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);   // xx xy xz yy yz zz
  double v = A * s7[idx];
  if (i == j) v += B * s7[6] + C;
  out[k] = accumulate ? out[k] + v : v;
}

// spectra of the density gradient: out_d = i G_d rho(G), d = 0,1,2.  On
// full grids the components along Nyquist axes are dropped: the real part of
// the inverse transform of the full array sees (G - G')/2 there, G' the
// vector of the conjugate partner index.
template <typename T>
__global__ void k_grad_spec(GInfo g, const cpx<T>* __restrict__ rhoG, cpx<T>* __restrict__ out, int64_t fs) {
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    int i0, i1, k2;
    decode(g, id, i0, i1, k2);
    double f0 = ffreq(i0, g.n0), f1 = ffreq(i1, g.n1), f2 = m2_of(g, k2);
    if (g.full) {
      if ((g.n0 & 1) == 0 && 2 * i0 == g.n0) f0 = 0.0;
      if ((g.n1 & 1) == 0 && 2 * i1 == g.n1) f1 = 0.0;
      if ((g.n2 & 1) == 0 && 2 * k2 == g.n2) f2 = 0.0;
    }
    const cpx<T> r = rhoG[id];
    for (int d = 0; d < 3; ++d) {
      const double gd = f0 * g.bg[d] + f1 * g.bg[3 + d] + f2 * g.bg[6 + d];
      out[d * fs + id] = cpx<T>{(T)(-gd * (double)r.y), (T)(gd * (double)r.x)};
    }
  }
}

// sum_r d_i d_j / rho (six sums)
template <typename T>
__global__ void __launch_bounds__(kST) k_vw_sum(int64_t n, const T* __restrict__ d0, const T* __restrict__ d1,
                                                 const T* __restrict__ d2, const T* __restrict__ rho,
                                                 double* __restrict__ partial) {
  double s[kNS] = {0, 0, 0, 0, 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double r = (double)rho[i];
    const double a = d0[i], b = d1[i], c = d2[i];
    s[0] += a * a / r; s[1] += a * b / r; s[2] += a * c / r;
    s[3] += b * b / r; s[4] += b * c / r; s[5] += c * c / r;
  }
  block_store7(s, partial);
}

// sum_r V_xc(rho) rho into the scalar slot (PZ81 potential in FP64)
template <typename T>
__global__ void __launch_bounds__(kST) k_lda_vrho(int64_t n, const T* __restrict__ rho, double* __restrict__ partial) {
  double s[kNS] = {0, 0, 0, 0, 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double r = (double)rho[i];
    double eps, v;
    gbct::pz_lda_ct<double>(r, eps, v, false);
    s[6] += v * r;
  }
  block_store7(s, partial);
}

template <typename T>
__global__ void k_pow(int64_t n, const T* __restrict__ rho, double p, T* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (T)pow((double)rho[i], p);
}

__global__ void k_sum(int64_t n, const double* __restrict__ x, double* __restrict__ partial) {
  KSum s;
  s.init();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s.add(x[i]);
  __shared__ double red[kST / 32];
  const double v = warp_sum(s.value());
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < kST / 32; ++w) t.add(red[w]);
    partial[blockIdx.x] = t.value();
  }
}

template <typename T>
__global__ void k_sumT(int64_t n, const T* __restrict__ x, double* __restrict__ partial) {
  double s[kNS] = {0, 0, 0, 0, 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s[6] += (double)x[i];
  block_store7(s, partial);
}

// Ewald real-space stress, one CTA per atom ia (ewald.py:609-662):
// q_ia sum_j q_j (2 sqrt(eta/pi) exp(-eta r^2) + erfc(sqrt(eta) r) / r) r_i r_j / r^2
__global__ void __launch_bounds__(kST) k_ewald_real_stress(const double* __restrict__ pos,
                                                            const double* __restrict__ q, int nat,
                                                            const double* __restrict__ img, int nimg, double rmax,
                                                            double eta, double* __restrict__ partial) {
  const int ia = blockIdx.x;
  const double se = sqrt(eta), c = 2.0 * se / sqrt(3.14159265358979323846);
  const double xi = pos[3 * ia], yi = pos[3 * ia + 1], zi = pos[3 * ia + 2];
  double s[kNS] = {0, 0, 0, 0, 0, 0, 0};
  const int64_t tot = (int64_t)nimg * nat;
  for (int64_t t = threadIdx.x; t < tot; t += blockDim.x) {
    const int im = (int)(t / nat), j = (int)(t % nat);
    const double dx = xi - (pos[3 * j] - img[3 * im]);
    const double dy = yi - (pos[3 * j + 1] - img[3 * im + 1]);
    const double dz = zi - (pos[3 * j + 2] - img[3 * im + 2]);
    const double d = sqrt(dx * dx + dy * dy + dz * dz);
    if (!(d < rmax && d > 0.001)) continue;
    const double wgt = q[ia] * q[j] * (c * exp(-eta * d * d) + erfc(se * d) / d) / (d * d);
    s[0] += wgt * dx * dx; s[1] += wgt * dx * dy; s[2] += wgt * dx * dz;
    s[3] += wgt * dy * dy; s[4] += wgt * dy * dz; s[5] += wgt * dz * dz;
  }
  block_store7(s, partial);
}

// S(G) = sum_a q_a exp(-i G.R_a)
__global__ void k_strf_q(GInfo g, const double* __restrict__ q, int nat, const double2* __restrict__ ph0,
                         const double2* __restrict__ ph1, const double2* __restrict__ ph2, double2* __restrict__ S) {
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    int i0, i1, k2;
    decode(g, id, i0, i1, k2);
    double sx = 0.0, sy = 0.0;
    for (int a = 0; a < nat; ++a) {
      const double2 e = phase(ph0, ph1, ph2, g, a, i0, i1, k2);
      sx += q[a] * e.x;
      sy += q[a] * e.y;
    }
    S[id] = double2{sx, sy};
  }
}

struct Bufs {
  char *spec[4];      // complex NG each (plan precision; spec[3] holds S in double2 for exact Ewald)
  char *field[4];     // real N each
  double2* phase;
  double* partial;    // max(kSB, nat) x kNS
  double* sums;       // 8
};

size_t spec_bytes(const gbofdft_plan* p) { return round256(2 * sizeof(double) * (size_t)p->NG); }
size_t field_bytes(const gbofdft_plan* p) { return round256(sizeof(double) * (size_t)p->N); }

Bufs layout(const gbofdft_plan* p, int nat, void* work) {
  char* b = reinterpret_cast<char*>(work);
  Bufs B;
  for (int i = 0; i < 4; ++i) { B.spec[i] = b; b += spec_bytes(p); }
  for (int i = 0; i < 4; ++i) { B.field[i] = b; b += field_bytes(p); }
  B.phase = reinterpret_cast<double2*>(b); b += phase_bytes(p, nat > 0 ? nat : 1);
  B.partial = reinterpret_cast<double*>(b); b += round256(sizeof(double) * kNS * (size_t)(nat > kSB ? nat : kSB));
  B.sums = reinterpret_cast<double*>(b);
  return B;
}

size_t work_bytes(const gbofdft_plan* p, int nat) {
  return 4 * spec_bytes(p) + 4 * field_bytes(p) + phase_bytes(p, nat > 0 ? nat : 1) +
         round256(sizeof(double) * kNS * (size_t)(nat > kSB ? nat : kSB)) + round256(sizeof(double) * 8);
}

template <typename T>
int gstress(gbofdft_plan* p, GsArgs& a, const Bufs& B, int accumulate, cudaStream_t st) {
  a.g = p->gi;
  a.partial = B.partial;
  k_gstress<T><<<kSB, kST, 0, st>>>(a);
  GB_CHECK_LAUNCH();
  k_reduce7<<<1, 32, 0, st>>>(B.partial, kSB, B.sums, accumulate);
  GB_CHECK_LAUNCH();
  return 0;
}

int assemble(const Bufs& B, double A, double Bd, double C, double* out, int accumulate, cudaStream_t st) {
  k_assemble<<<1, 32, 0, st>>>(B.sums, A, Bd, C, out, accumulate);
  GB_CHECK_LAUNCH();
  return 0;
}

double read_scalar(const double* dev, cudaStream_t st, int* rc) {
  double h = 0.0;
  cudaError_t e = cudaMemcpyAsync(&h, dev, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  *rc = e == cudaSuccess ? 0 : gb_set_error(GBOFDFT_ERR_CUDA, "stress: %s", cudaGetErrorString(e));
  return h;
}

template <typename T>
int functional_stress(gbofdft_plan* p, const void* rho, const gbofdft_functional* f, const double* en, void* work,
                      double* out, cudaStream_t st) {
  const Bufs B = layout(p, 1, work);
  const double Om = p->volume, dV = p->dV;
  const T* r = reinterpret_cast<const T*>(rho);
  int rc;
  GB_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * 45, st));
  GB_CUDA(cudaMemsetAsync(B.sums, 0, sizeof(double) * 8, st));
  // TF
  if (f->tf) {
    k_assemble<<<1, 32, 0, st>>>(B.sums, 0.0, 0.0, -2.0 / 3.0 * en[GBOFDFT_E_TF] / Om, out + 0, 0);
    GB_CHECK_LAUNCH();
  }
  // rho(G)
  if ((rc = gbofdft_fft_r2c(p, rho, B.spec[0], st))) return rc;
  // vW: gradient spectra -> real gradients -> sum d_i d_j / rho
  if (f->vw) {
    k_grad_spec<T><<<grid_blocks(p->NG), 256, 0, st>>>(p->gi, (const cpx<T>*)B.spec[0], (cpx<T>*)B.spec[1], p->NG);
    GB_CHECK_LAUNCH();
    for (int d = 0; d < 3; ++d) {
      char* sd = B.spec[1] + d * 2 * gb_elem(p) * p->NG;
      if ((rc = gbofdft_fft_c2r(p, sd, B.field[d], st))) return rc;
    }
    k_vw_sum<T><<<kSB, kST, 0, st>>>(p->N, (const T*)B.field[0], (const T*)B.field[1], (const T*)B.field[2], r,
                                      B.partial);
    GB_CHECK_LAUNCH();
    k_reduce7<<<1, 32, 0, st>>>(B.partial, kSB, B.sums, 0);
    GB_CHECK_LAUNCH();
    if ((rc = assemble(B, -0.25 * dV * f->vw_y / Om, 0.0, 0.0, out + 9, 0, st))) return rc;
  }
  // WT nonlocal term
  if (f->wt) {
    k_sumT<T><<<kSB, kST, 0, st>>>(p->N, r, B.partial);
    GB_CHECK_LAUNCH();
    k_reduce7<<<1, 32, 0, st>>>(B.partial, kSB, B.sums, 0);
    GB_CHECK_LAUNCH();
    const double rho0 = read_scalar(B.sums + 6, st, &rc) / (double)p->N;
    if (rc) return rc;
    const double al = f->wt_alpha, be = f->wt_beta;
    k_pow<T><<<grid_blocks(p->N), 256, 0, st>>>(p->N, r, al, (T*)B.field[0]);
    GB_CHECK_LAUNCH();
    if ((rc = gbofdft_fft_r2c(p, B.field[0], B.spec[1], st))) return rc;
    const char* specB = B.spec[1];
    if (fabs(al - be) > 0.0) {
      k_pow<T><<<grid_blocks(p->N), 256, 0, st>>>(p->N, r, be, (T*)B.field[1]);
      GB_CHECK_LAUNCH();
      if ((rc = gbofdft_fft_r2c(p, B.field[1], B.spec[2], st))) return rc;
      specB = B.spec[2];
    }
    const double tkf = 2.0 * cbrt(3.0 * rho0 * 9.86960440108935861883);
    GsArgs a;
    memset(&a, 0, sizeof(a));
    a.mode = SM_WT; a.a = B.spec[1]; a.b = specB; a.tkf = tkf;
    if ((rc = gstress<T>(p, a, B, 0, st))) return rc;
    const double F = 9.86960440108935861883 / (al * be * pow(rho0, al + be - 2.0) * tkf / 2.0);
    if ((rc = assemble(B, F / (Om * Om), -F / (3.0 * Om * Om), -2.0 / 3.0 * en[GBOFDFT_E_NL] / Om, out + 18, 0,
                       st)))
      return rc;
  }
  // LDA
  if (f->xc) {
    k_lda_vrho<T><<<kSB, kST, 0, st>>>(p->N, r, B.partial);
    GB_CHECK_LAUNCH();
    k_reduce7<<<1, 32, 0, st>>>(B.partial, kSB, B.sums, 0);
    GB_CHECK_LAUNCH();
    if ((rc = assemble(B, 0.0, -dV / Om, en[GBOFDFT_E_XC] / Om, out + 27, 0, st))) return rc;
  }
  // Hartree
  if (f->hartree) {
    GsArgs a;
    memset(&a, 0, sizeof(a));
    a.mode = SM_HARTREE; a.a = B.spec[0];
    if ((rc = gstress<T>(p, a, B, 0, st))) return rc;
    const double pi = 3.14159265358979323846;
    if ((rc = assemble(B, 8.0 * pi / (Om * Om), 0.0, -en[GBOFDFT_E_HARTREE] / Om, out + 36, 0, st))) return rc;
  }
  return 0;
}

template <typename T>
int pp_stress(gbofdft_plan* p, const void* rho, int nspec, const gbofdft_vtable* tabs, int nat,
              const double* spos, const int* species, int pme, int order, const double* bm_dev, double e_pp,
              void* work, double* out, cudaStream_t st) {
  const Bufs B = layout(p, nat, work);
  const double Om = p->volume;
  int rc;
  if ((rc = gbofdft_fft_r2c(p, rho, B.spec[0], st))) return rc;
  if (pme) {
    const double2* bm = reinterpret_cast<const double2*>(bm_dev);
    for (int s = 0; s < nspec; ++s) {
      GB_CUDA(cudaMemsetAsync(B.field[0], 0, gb_elem(p) * p->N, st));
      k_pme_spread<T><<<nat, 256, 0, st>>>(p->gi, spos, nullptr, species, s, order, (T*)B.field[0]);
      GB_CHECK_LAUNCH();
      if ((rc = gbofdft_fft_r2c(p, B.field[0], B.spec[1], st))) return rc;
      GsArgs a;
      memset(&a, 0, sizeof(a));
      a.mode = SM_PP_PME; a.a = B.spec[0]; a.b = B.spec[1]; a.vt = tabs[s];
      a.bm0 = bm; a.bm1 = bm + p->n[0]; a.bm2 = bm + p->n[0] + p->n[1];
      if ((rc = gstress<T>(p, a, B, s > 0, st))) return rc;
    }
    return assemble(B, -2.0 * (double)p->N / (Om * Om * Om), 0.0, -e_pp / Om, out, 0, st);
  }
  double2 *ph0, *ph1, *ph2, *ph2p;
  phase_tables(p, spos, nat, B.phase, st, &ph0, &ph1, &ph2, &ph2p);
  GB_CHECK_LAUNCH();
  GsArgs a;
  memset(&a, 0, sizeof(a));
  a.mode = SM_PP_EXACT; a.a = B.spec[0]; a.species = species; a.nat = nat;
  a.ph0 = ph0; a.ph1 = ph1; a.ph2 = ph2;
  a.vts.n = nspec;
  for (int s = 0; s < nspec; ++s) a.vts.t[s] = tabs[s];
  if ((rc = gstress<T>(p, a, B, 0, st))) return rc;
  return assemble(B, -2.0 / (Om * Om), 0.0, -e_pp / Om, out, 0, st);
}

template <typename T>
int ewald_stress(gbofdft_plan* p, int nat, const double* pos, const double* spos, const double* charges,
                 double eta, double rmax, const double* images, int nimg, int pme, int order, const double* bm_dev,
                 double qsum, void* work, double* out, cudaStream_t st) {
  const Bufs B = layout(p, nat, work);
  const double Om = p->volume, pi = 3.14159265358979323846;
  int rc;
  k_ewald_real_stress<<<nat, kST, 0, st>>>(pos, charges, nat, images, nimg, rmax, eta, B.partial);
  GB_CHECK_LAUNCH();
  k_reduce7<<<1, 32, 0, st>>>(B.partial, nat, B.sums, 0);
  GB_CHECK_LAUNCH();
  if ((rc = assemble(B, -0.5 / Om, 0.0, 0.0, out, 0, st))) return rc;
  GsArgs a;
  memset(&a, 0, sizeof(a));
  a.mode = SM_EWALD; a.eta = eta;
  double scale;
  if (pme) {
    GB_CUDA(cudaMemsetAsync(B.field[0], 0, gb_elem(p) * p->N, st));
    k_pme_spread<T><<<nat, 256, 0, st>>>(p->gi, spos, charges, nullptr, 0, order, (T*)B.field[0]);
    GB_CHECK_LAUNCH();
    if ((rc = gbofdft_fft_r2c(p, B.field[0], B.spec[0], st))) return rc;
    const double2* bm = reinterpret_cast<const double2*>(bm_dev);
    a.a = B.spec[0]; a.bm0 = bm; a.bm1 = bm + p->n[0]; a.bm2 = bm + p->n[0] + p->n[1];
    if ((rc = gstress<T>(p, a, B, 0, st))) return rc;
    scale = 2.0 * 2.0 * pi / (Om * Om) / (p->dV * p->dV);
  } else {
    double2 *ph0, *ph1, *ph2, *ph2p;
    phase_tables(p, spos, nat, B.phase, st, &ph0, &ph1, &ph2, &ph2p);
    GB_CHECK_LAUNCH();
    double2* S = reinterpret_cast<double2*>(B.spec[3]);
    k_strf_q<<<grid_blocks(p->NG), 256, 0, st>>>(p->gi, charges, nat, ph0, ph1, ph2, S);
    GB_CHECK_LAUNCH();
    a.a = S;
    if ((rc = gstress<double>(p, a, B, 0, st))) return rc;
    scale = 4.0 * pi / (Om * Om);
  }
  const double s_g0 = qsum * qsum * 4.0 * pi * (1.0 / (4.0 * eta * Om * Om) / 2.0);
  return assemble(B, scale, -scale, s_g0, out, 1, st);
}

}  // namespace

extern "C" {

int gbofdft_stress_workspace_bytes(const gbofdft_plan* p, int nat, int64_t* bytes) {
  GB_REQUIRE(p && bytes && nat >= 0, "stress_workspace_bytes: bad argument");
  *bytes = (int64_t)work_bytes(p, nat);
  return GBOFDFT_OK;
}

int gbofdft_stress_functional(gbofdft_plan* p, const void* rho, const gbofdft_functional* f,
                              const double energies[GBOFDFT_NE], void* work, int64_t work_bytes_, double* out_dev,
                              void* stream) {
  GB_REQUIRE(p && rho && f && energies && work && out_dev, "stress_functional: null argument");
  GB_REQUIRE(!f->lwt, "stress_functional: the LWT/LMGP stress is not part of this path");
  int64_t need = 0;
  gbofdft_stress_workspace_bytes(p, 1, &need);
  GB_REQUIRE(work_bytes_ >= need, "stress_functional: workspace %lld < %lld bytes", (long long)work_bytes_,
             (long long)need);
  GB_REQUIRE(((uintptr_t)work & 255) == 0, "stress_functional: workspace must be 256-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  return p->prec == GBOFDFT_F64 ? functional_stress<double>(p, rho, f, energies, work, out_dev, st)
                                : functional_stress<float>(p, rho, f, energies, work, out_dev, st);
}

int gbofdft_pp_stress(gbofdft_plan* p, const void* rho, int nspec, const gbofdft_vtable* tables, int nat,
                      const double* spos_dev, const int* species_dev, int pme, int order, const double* bm_dev,
                      double e_pp, void* work, int64_t work_bytes_, double* out_dev, void* stream) {
  GB_REQUIRE(p && rho && tables && spos_dev && species_dev && work && out_dev, "pp_stress: null argument");
  GB_REQUIRE(nspec >= 1 && nspec <= GBOFDFT_MAX_SPECIES && nat >= 1, "pp_stress: bad sizes");
  GB_REQUIRE(!pme || (bm_dev && order >= 2 && order <= 30), "pp_stress: PME needs the b(m) table");
  int64_t need = 0;
  gbofdft_stress_workspace_bytes(p, nat, &need);
  GB_REQUIRE(work_bytes_ >= need, "pp_stress: workspace %lld < %lld bytes", (long long)work_bytes_,
             (long long)need);
  GB_REQUIRE(((uintptr_t)work & 255) == 0, "pp_stress: workspace must be 256-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  return p->prec == GBOFDFT_F64
             ? pp_stress<double>(p, rho, nspec, tables, nat, spos_dev, species_dev, pme, order, bm_dev, e_pp, work,
                                 out_dev, st)
             : pp_stress<float>(p, rho, nspec, tables, nat, spos_dev, species_dev, pme, order, bm_dev, e_pp, work,
                                out_dev, st);
}

int gbofdft_ewald_stress(gbofdft_plan* p, int nat, const double* pos_dev, const double* spos_dev,
                         const double* charges_dev, double eta, double rmax, const double* images_dev, int nimg,
                         int pme, int order, const double* bm_dev, double charge_sum, void* work,
                         int64_t work_bytes_, double* out_dev, void* stream) {
  GB_REQUIRE(p && pos_dev && spos_dev && charges_dev && images_dev && work && out_dev, "ewald_stress: null argument");
  GB_REQUIRE(nat >= 1 && nimg >= 1 && eta > 0.0, "ewald_stress: bad arguments");
  GB_REQUIRE(!pme || (bm_dev && order >= 2 && order <= 30), "ewald_stress: PME needs the b(m) table");
  int64_t need = 0;
  gbofdft_stress_workspace_bytes(p, nat, &need);
  GB_REQUIRE(work_bytes_ >= need, "ewald_stress: workspace %lld < %lld bytes", (long long)work_bytes_,
             (long long)need);
  GB_REQUIRE(((uintptr_t)work & 255) == 0, "ewald_stress: workspace must be 256-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  return p->prec == GBOFDFT_F64
             ? ewald_stress<double>(p, nat, pos_dev, spos_dev, charges_dev, eta, rmax, images_dev, nimg, pme, order,
                                    bm_dev, charge_sum, work, out_dev, st)
             : ewald_stress<float>(p, nat, pos_dev, spos_dev, charges_dev, eta, rmax, images_dev, nimg, pme, order,
                                   bm_dev, charge_sum, work, out_dev, st);
}

}  // extern "C"
