// FFT passes over a 3D grid with the OF-DFT pointwise work fused in.
//
// Data layout (C order): real fields T[n0][n1][n2]; spectra are the half
// spectrum cpx<T>[n0][n1][ld2] (the first n2h = n2/2+1 columns are valid).
//
//   rows forward   real rows -> axis-2 R2C; two real rows ride in one complex
//                  line (z = a + i b), separated after the transform.  The
//                  prologue derives up to GB_MAX_FIELDS fields from one read
//                  of the input (rho, sqrt(rho), rho^beta).
//   cols           axis-1 or axis-0 C2C on tiles of tb adjacent columns
//                  (coalesced along the contiguous axis).
//   cols conv      axis-0 forward, multiply by a reciprocal-space kernel,
//                  axis-0 inverse, in one pass (no spectrum round trip).
//   rows inverse   axis-2 C2R (irfftn semantics: imaginary parts of the DC
//                  and Nyquist columns are ignored), two rows per line; the
//                  epilogue either stores or assembles the OF-DFT potential
//                  and the energy densities (compensated FP64 partial sums).
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "fft_core.cuh"
#include "gkernels.cuh"
#include "plan.h"
#include "lindhard.cuh"

using namespace gbfft;
using gbk::ffreq;
using gbk::gg_of;
using gbk::sym_kernel;
using gbk::kernel_value;

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kZero = 1e-30;                       // dftpy ZERO

template <typename T> __device__ __forceinline__ T ld(const T* p) { return __ldg(p); }

template <typename T>
__device__ __forceinline__ void load_twiddles(cpx<T>* dst, const cpx<T>* src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// rho^beta; beta == 5/6 uses sqrt(rho) * cbrt(rho)
template <typename T> __device__ __forceinline__ T pow_beta(T x, double beta) {
  if (fabs(beta - 5.0 / 6.0) < 1e-15) return sqrt(x) * cbrt(x);
  return pow(x, (T)beta);
}

template <typename T>
__device__ __forceinline__ T prologue(int op, T rho, double beta) {
  if (op == OP_SQRT) {
    T r = rho > (T)0 ? rho : (T)kZero;
    return sqrt(r);
  }
  if (op == OP_POWB) {
    T r = rho < (T)kZero ? (T)kZero : rho;
    return pow_beta<T>(r, beta);
  }
  return rho;
}

// ---------------------------------------------------------------------------
// rows forward (R2C along axis 2)
// ---------------------------------------------------------------------------
struct RowsFwdArgs {
  const void* in;
  void* out;
  int64_t fstride;
  int nrows, n2, n2h, ld2, nf, pairs;
  int op[GB_MAX_FIELDS];
  double beta, scale;
  AxisPlan ax;
  const void* tw;
};

template <typename T>
__global__ void __launch_bounds__(256) k_rows_fwd(RowsFwdArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n2 = a.n2, P = a.pairs, nf = a.nf;
  cpx<T>* tw = reinterpret_cast<cpx<T>*>(smem_raw);
  const int nl = nf * P;
  cpx<T>* A = tw + n2;
  cpx<T>* B = A + (size_t)nl * n2;
  load_twiddles<T>(tw, reinterpret_cast<const cpx<T>*>(a.tw), n2);
  const T* in = reinterpret_cast<const T*>(a.in);
  const int64_t base = (int64_t)blockIdx.x * 2 * P;
  T* Af = reinterpret_cast<T*>(A);
  for (int idx = threadIdx.x; idx < 2 * P * n2; idx += blockDim.x) {
    const int rr = idx / n2, j = idx - rr * n2;
    const int64_t R = base + rr;
    const bool ok = R < a.nrows;
    const T x = ok ? ld(in + R * n2 + j) : (T)0;
    for (int f = 0; f < nf; ++f) {
      const T v = ok ? prologue<T>(a.op[f], x, a.beta) : (T)0;
      Af[2 * ((size_t)(f * P + (rr >> 1)) * n2 + j) + (rr & 1)] = v;
    }
  }
  __syncthreads();
  cpx<T>* res = lines_fft<-1, T, true>(A, B, tw, a.ax, nl, n2, 1);
  const int n2h = a.n2h;
  const T half = (T)0.5 * (T)a.scale;
  cpx<T>* out = reinterpret_cast<cpx<T>*>(a.out);
  for (int idx = threadIdx.x; idx < nl * n2h; idx += blockDim.x) {
    const int line = idx / n2h, k = idx - line * n2h;
    const int f = line / P, pp = line - f * P;
    const cpx<T> Z = res[(size_t)line * n2 + k];
    const cpx<T> Zc = res[(size_t)line * n2 + (k == 0 ? 0 : n2 - k)];
    const int64_t ra = base + 2 * pp, rb = ra + 1;
    if (ra >= a.nrows) continue;
    cpx<T>* o = out + f * a.fstride;
    o[ra * a.ld2 + k] = cpx<T>{(Z.x + Zc.x) * half, (Z.y - Zc.y) * half};
    if (rb < a.nrows) o[rb * a.ld2 + k] = cpx<T>{(Z.y + Zc.y) * half, (Zc.x - Z.x) * half};
  }
}

// ---------------------------------------------------------------------------
// rows inverse (C2R along axis 2) with store or OF-DFT epilogue
// ---------------------------------------------------------------------------
struct RowsInvArgs {
  const void* in;
  int64_t fstride;
  int nrows, n2, n2h, ld2, nf, pairs;
  AxisPlan ax;
  const void* tw;
  // store epilogue
  void* out;
  int64_t ostride;
  double scale;
  // evaluation epilogue
  EvalDesc ev;
  const void* rho;
  const void* vloc;
  void* pot;
  double* partials;
  int calc_e;
};

template <typename T>
__device__ __forceinline__ cpx<T>* rows_inv_core(const RowsInvArgs& a, cpx<T>* tw, cpx<T>* A, cpx<T>* B,
                                                  int64_t base) {
  const int n2 = a.n2, n2h = a.n2h, P = a.pairs, nl = a.nf * P;
  load_twiddles<T>(tw, reinterpret_cast<const cpx<T>*>(a.tw), n2);
  const cpx<T>* in = reinterpret_cast<const cpx<T>*>(a.in);
  for (int idx = threadIdx.x; idx < nl * n2h; idx += blockDim.x) {
    const int line = idx / n2h, k = idx - line * n2h;
    const int f = line / P, pp = line - f * P;
    const int64_t ra = base + 2 * pp, rb = ra + 1;
    cpx<T> va = {(T)0, (T)0}, vb = {(T)0, (T)0};
    const cpx<T>* src = in + f * a.fstride;
    if (ra < a.nrows) va = src[ra * a.ld2 + k];
    if (rb < a.nrows) vb = src[rb * a.ld2 + k];
    const bool edge = (k == 0) || (2 * k == n2);
    if (edge) { va.y = (T)0; vb.y = (T)0; }
    cpx<T>* L = A + (size_t)line * n2;
    L[k] = cpx<T>{va.x - vb.y, va.y + vb.x};
    if (k > 0 && 2 * k < n2) L[n2 - k] = cpx<T>{va.x + vb.y, vb.x - va.y};
  }
  __syncthreads();
  return lines_fft<1, T, true>(A, B, tw, a.ax, nl, n2, 1);
}

template <typename T>
__global__ void __launch_bounds__(256) k_rows_inv_store(RowsInvArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n2 = a.n2, P = a.pairs, nl = a.nf * P;
  cpx<T>* tw = reinterpret_cast<cpx<T>*>(smem_raw);
  cpx<T>* A = tw + n2;
  cpx<T>* B = A + (size_t)nl * n2;
  const int64_t base = (int64_t)blockIdx.x * 2 * P;
  cpx<T>* res = rows_inv_core<T>(a, tw, A, B, base);
  T* out = reinterpret_cast<T*>(a.out);
  const T s = (T)a.scale;
  for (int idx = threadIdx.x; idx < 2 * P * n2; idx += blockDim.x) {
    const int rr = idx / n2, j = idx - rr * n2;
    const int64_t R = base + rr;
    if (R >= a.nrows) continue;
    for (int f = 0; f < a.nf; ++f) {
      const cpx<T> z = res[(size_t)(f * P + (rr >> 1)) * n2 + j];
      out[f * a.ostride + R * n2 + j] = ((rr & 1) ? z.y : z.x) * s;
    }
  }
}

// Perdew-Zunger 1981 LDA (unpolarised): energy density per particle and
// potential; rho^(1/3) clamped at 1e-30 as in the reference.
template <typename T>
__device__ __forceinline__ void pz_lda(T rho, T& eps, T& pot, bool want_e) {
  const T a = (T)0.0311, b = (T)-0.048, c = (T)0.0020, d = (T)-0.0116;
  const T g = (T)-0.1423, b1 = (T)1.0529, b2 = (T)0.3334;
  T rc = cbrt(rho);
  if (rc < (T)kZero) rc = (T)kZero;
  const T rs = (T)0.62035049089940001667 / rc;          // (3/(4 pi))^(1/3)
  const T cx = (T)0.98474502184269654115;                // (3/pi)^(1/3)
  pot = -cx * rc;
  eps = (T)(-0.75) * cx * rc;
  if (rs < (T)1) {
    const T lr = log(rs);
    pot += lr * (a + (T)(2.0 / 3.0) * c * rs) + b - (T)(1.0 / 3.0) * a + (T)(1.0 / 3.0) * ((T)2 * d - c) * rs;
    if (want_e) eps += a * lr + b + c * rs * lr + d * rs;
  } else {
    const T sq = sqrt(rs);
    const T den = (T)1 + b1 * sq + b2 * rs;
    pot += (g + ((T)(7.0 / 6.0) * g * b1) * sq + ((T)(4.0 / 3.0) * g * b2 * rs)) / (den * den);
    if (want_e) eps += g / den;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_rows_inv_eval(RowsInvArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n2 = a.n2, P = a.pairs, nl = a.nf * P;
  cpx<T>* tw = reinterpret_cast<cpx<T>*>(smem_raw);
  cpx<T>* A = tw + n2;
  cpx<T>* B = A + (size_t)nl * n2;
  const int64_t base = (int64_t)blockIdx.x * 2 * P;
  cpx<T>* res = rows_inv_core<T>(a, tw, A, B, base);
  const EvalDesc& ev = a.ev;
  const T* rhop = reinterpret_cast<const T*>(a.rho);
  const T* vlocp = reinterpret_cast<const T*>(a.vloc);
  T* potp = reinterpret_cast<T*>(a.pot);
  const bool want_e = a.calc_e != 0;
  const T ctf = (T)2.87123400018819181594;             // (3/10)(3 pi^2)^(2/3)
  const T alpha = (T)ev.wt_alpha;
  KSum es[6];
#pragma unroll
  for (int c = 0; c < 6; ++c) es[c].init();
  for (int idx = threadIdx.x; idx < 2 * P * n2; idx += blockDim.x) {
    const int rr = idx / n2, j = idx - rr * n2;
    const int64_t R = base + rr;
    if (R >= a.nrows) continue;
    const int pp = rr >> 1;
    const bool odd = rr & 1;
    const int64_t gidx = R * n2 + j;
    const T rho = ld(rhop + gidx);
    T pot = (T)0;
    if (ev.tf) {
      const T cr = cbrt(rho * rho);
      pot += (T)(5.0 / 3.0) * ctf * cr * (T)ev.tf_x;
      if (want_e) {
        T r5 = rho * rho;
        r5 = r5 * rho; r5 = r5 * rho; r5 = r5 * rho;
        es[0].add((double)(cbrt(r5) * ctf) * ev.tf_x);
      }
    }
    if (ev.vw) {
      const cpx<T> z = res[(size_t)(ev.slot_vw * P + pp) * n2 + j];
      const T w = odd ? z.y : z.x;
      T rm = rho > (T)0 ? rho : (T)kZero;
      T sq = sqrt(rm);
      if (fabs(sq) < (T)kZero) sq = (T)kZero;
      const T v = (T)0.5 * w / sq;
      pot += v * (T)ev.vw_y;
      if (want_e && rho > (T)0) es[1].add((double)(rho * v) * ev.vw_y);
    }
    if (ev.wt) {
      const cpx<T> z = res[(size_t)(ev.slot_wt * P + pp) * n2 + j];
      const T kc = odd ? z.y : z.x;
      const T rc = rho < (T)kZero ? (T)kZero : rho;
      const T rb = pow_beta<T>(rc, ev.wt_beta);
      const T v = (T)2 * alpha * (rb / rc) * kc;
      pot += v;
      if (want_e) es[2].add((double)(v * rho / ((T)2 * alpha)));
    }
    if (ev.xc) {
      T eps, vx;
      pz_lda<T>(rho, eps, vx, want_e);
      pot += vx;
      if (want_e) es[3].add((double)(eps * rho));
    }
    if (ev.hartree) {
      const cpx<T> z = res[(size_t)(ev.slot_h * P + pp) * n2 + j];
      const T vh = odd ? z.y : z.x;
      pot += vh;
      if (want_e) es[4].add(0.5 * (double)vh * (double)rho);
    }
    if (ev.pp) {
      const T vl = ld(vlocp + gidx);
      pot += vl;
      if (want_e) es[5].add((double)vl * (double)rho);
    }
    potp[gidx] = pot;
  }
  if (!want_e) return;
  __shared__ double red[8][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    double v = warp_sum(es[c].value());
    if (lane == 0) red[warp][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double s = 0.0;
    const int nw = blockDim.x >> 5;
    for (int w = 0; w < nw; ++w) s += red[w][threadIdx.x];
    a.partials[(int64_t)blockIdx.x * GB_NE + threadIdx.x] = s;
  }
}

// Sum per-CTA partials in a fixed order; slot GB_E_TOTAL gets the sum of
// the components (times dV) plus the constant ion-ion term.
// One CTA per energy component (the FP64 sums spread over 6 SMs); the last
// CTA to finish adds the components into the total.  counter: zero on entry,
// left zero.
__global__ void __launch_bounds__(256) k_energy_final(const double* __restrict__ partials, int64_t nblk,
                                                      double dV, double e_ion, double* __restrict__ e,
                                                      unsigned* counter) {
  __shared__ double red[8];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c = blockIdx.x;
  KSum s;
  s.init();
  for (int64_t b = threadIdx.x; b < nblk; b += blockDim.x) s.add(partials[b * GB_NE + c]);
  const double v = warp_sum(s.value());
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t.add(red[w]);
    e[c] = t.value() * dV;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0) {
    __threadfence();
    double tot = 0.0;
    for (int k = 0; k < 6; ++k) tot += __ldcg(e + k);
    e[GB_E_EXTRA] = 0.0;
    e[GB_E_TOTAL] = tot + e_ion;
    *counter = 0u;
  }
}

// ---------------------------------------------------------------------------
// column passes
// ---------------------------------------------------------------------------
struct ColsArgs {
  void* data;
  int64_t fstride;
  int n;           // transform length
  int64_t stride;  // complex elements between consecutive line elements
  int64_t ostride; // complex elements between outer groups (blockIdx.y)
  int ncols, tb;
  AxisPlan ax;
  const void* tw;
  double scale;
  // convolution (axis 0 only)
  GInfo gi;
  KerDesc kd;
};

template <typename T>
__device__ __forceinline__ void cols_load(const ColsArgs& a, cpx<T>* buf, const cpx<T>* base, int nc) {
  for (int idx = threadIdx.x; idx < a.n * nc; idx += blockDim.x) {
    const int j = idx / nc, c = idx - j * nc;
    buf[j * a.tb + c] = base[(int64_t)j * a.stride + c];
  }
}

template <typename T>
__device__ __forceinline__ void cols_store(const ColsArgs& a, const cpx<T>* buf, cpx<T>* base, int nc, T s) {
  for (int idx = threadIdx.x; idx < a.n * nc; idx += blockDim.x) {
    const int j = idx / nc, c = idx - j * nc;
    base[(int64_t)j * a.stride + c] = c_scale(buf[j * a.tb + c], s);
  }
}

template <typename T, int DIR>
__global__ void __launch_bounds__(256) k_cols(ColsArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cpx<T>* tw = reinterpret_cast<cpx<T>*>(smem_raw);
  cpx<T>* A = tw + a.n;
  cpx<T>* B = A + (size_t)a.n * a.tb;
  load_twiddles<T>(tw, reinterpret_cast<const cpx<T>*>(a.tw), a.n);
  const int c0 = blockIdx.x * a.tb;
  const int nc = min(a.tb, a.ncols - c0);
  cpx<T>* base = reinterpret_cast<cpx<T>*>(a.data) + blockIdx.z * a.fstride + blockIdx.y * a.ostride + c0;
  cols_load<T>(a, A, base, nc);
  __syncthreads();
  cpx<T>* res = lines_fft<DIR, T, false>(A, B, tw, a.ax, nc, 1, a.tb);
  cols_store<T>(a, res, base, nc, (T)a.scale);
}

template <typename T>
__global__ void __launch_bounds__(256) k_cols_conv(ColsArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cpx<T>* tw = reinterpret_cast<cpx<T>*>(smem_raw);
  cpx<T>* A = tw + a.n;
  cpx<T>* B = A + (size_t)a.n * a.tb;
  load_twiddles<T>(tw, reinterpret_cast<const cpx<T>*>(a.tw), a.n);
  const int c0 = blockIdx.x * a.tb;
  const int nc = min(a.tb, a.ncols - c0);
  const int f = blockIdx.z, i1 = blockIdx.y;
  cpx<T>* base = reinterpret_cast<cpx<T>*>(a.data) + f * a.fstride + i1 * a.ostride + c0;
  cols_load<T>(a, A, base, nc);
  __syncthreads();
  cpx<T>* res = lines_fft<-1, T, false>(A, B, tw, a.ax, nc, 1, a.tb);
  const int type = a.kd.type[f];
  const T coef = (T)a.kd.coef[f];
  const void* arr = a.kd.arr[f];
  for (int idx = threadIdx.x; idx < a.n * nc; idx += blockDim.x) {
    const int j = idx / nc, c = idx - j * nc;
    const T kval = kernel_value<T>(a.gi, type, arr, j, i1, c0 + c) * coef;
    res[j * a.tb + c] = c_scale(res[j * a.tb + c], kval);
  }
  __syncthreads();
  cpx<T>* other = (res == A) ? B : A;
  res = lines_fft<1, T, false>(res, other, tw, a.ax, nc, 1, a.tb);
  cols_store<T>(a, res, base, nc, (T)1);
}

// ---------------------------------------------------------------------------
// Wang-Teter kernel table on the half spectrum (inverse Lindhard function).
// ---------------------------------------------------------------------------
using gblind::lindhard_inv;

template <typename T>
// out: half-spectrum layout; out_pm (optional): the same values plane-major,
// (k2 * n0 + i0) * n1 + i1
__global__ void k_wt_kernel(GInfo g, double tkf, double factor, double x, T* __restrict__ out,
                            T* __restrict__ out_pm) {
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int k2 = (int)(id % g.n2h);
    const int64_t r = id / g.n2h;
    const int i1 = (int)(r % g.n1), i0 = (int)(r / g.n1);
    const double v = sym_kernel<double>(g, i0, i1, k2, [&](double gg) {
      return lindhard_inv(sqrt(gg) / tkf, x, 1.0) * factor;
    });
    out[id] = (T)v;
    if (out_pm) out_pm[(int64_t)k2 * g.n0 * g.n1 + r] = (T)v;
  }
}

// Truncated-Newton preconditioner for the phi-space Hessian of a near-uniform
// density rho0 (diagonal in G): 1 / ((2/3) k_F^2 / F_Lindhard(|G| / 2k_F) + 8 pi rho0 / G^2),
// the inverse of the kinetic (Lindhard) plus Hartree curvature of the
// uniform electron gas; 0 at G = 0.
template <typename T>
__global__ void k_precond(GInfo g, double rho0, T* __restrict__ out, float* __restrict__ out_pm) {
  const double kf = cbrt(3.0 * kPi * kPi * rho0);
  const double ckin = 2.0 / 3.0 * kf * kf, tkf = 2.0 * kf, ch = 8.0 * kPi * rho0;
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    const int k2 = (int)(id % g.n2h);
    const int64_t r = id / g.n2h;
    const int i1 = (int)(r % g.n1), i0 = (int)(r / g.n1);
    const double v = sym_kernel<double>(g, i0, i1, k2, [&](double gg) {
      return gg > 0.0 ? 1.0 / (ckin * lindhard_inv(sqrt(gg) / tkf, 0.0, 0.0) + ch / gg) : 0.0;
    });
    out[id] = (T)v;
    if (out_pm) out_pm[(int64_t)k2 * g.n0 * g.n1 + r] = (float)v;
  }
}

template <typename T> size_t rows_smem(int n2, int nl) { return sizeof(cpx<T>) * ((size_t)n2 + 2 * (size_t)nl * n2); }
template <typename T> size_t cols_smem(int n, int tb) { return sizeof(cpx<T>) * ((size_t)n + 2 * (size_t)n * tb); }

template <typename K> int set_smem(K kern, size_t bytes) {
  if (bytes > 48 * 1024) GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <typename T>
static int rows_fwd_t(gbofdft_plan* p, const void* in, void* spec, int64_t fstride, int ld2, int nf,
                      const int* ops, double beta, double scale, cudaStream_t st) {
  RowsFwdArgs a;
  a.in = in; a.out = spec; a.fstride = fstride;
  a.nrows = p->n[0] * p->n[1]; a.n2 = p->n[2]; a.n2h = p->n2h; a.ld2 = ld2; a.nf = nf;
  a.pairs = p->pairs;
  for (int f = 0; f < GB_MAX_FIELDS; ++f) a.op[f] = f < nf ? ops[f] : OP_RHO;
  a.beta = beta; a.scale = scale; a.ax = p->ax[2]; a.tw = p->tw[2];
  const size_t sm = rows_smem<T>(a.n2, nf * a.pairs);
  if (set_smem(k_rows_fwd<T>, sm)) return GBOFDFT_ERR_CUDA;
  const int nblk = (a.nrows + 2 * a.pairs - 1) / (2 * a.pairs);
  k_rows_fwd<T><<<nblk, 256, sm, st>>>(a);
  GB_CHECK_LAUNCH();
  return 0;
}

int gb_use_ct() {
  static int v = -1;
  if (v < 0) {
    const char* e = getenv("GBOFDFT_GENERIC_FFT");
    v = (e && e[0] == '1') ? 0 : 1;
  }
  return v;
}

int gb_rows_fwd(gbofdft_plan* p, const void* in, void* spec, int64_t fstride, int ld2, int nf, const int* ops,
                double beta, double scale, cudaStream_t st) {
  if (gb_use_ct()) {
    const int rc = p->prec == GBOFDFT_F64 ? gb_ct_rows_fwd_f64(p, in, spec, fstride, ld2, nf, ops, beta, scale, st)
                                          : gb_ct_rows_fwd_f32(p, in, spec, fstride, ld2, nf, ops, beta, scale, st);
    if (rc != 1) return rc;
  }
  return p->prec == GBOFDFT_F64 ? rows_fwd_t<double>(p, in, spec, fstride, ld2, nf, ops, beta, scale, st)
                                : rows_fwd_t<float>(p, in, spec, fstride, ld2, nf, ops, beta, scale, st);
}

template <typename T>
static RowsInvArgs rows_inv_args(gbofdft_plan* p, const void* spec, int64_t fstride, int ld2, int nf) {
  RowsInvArgs a;
  memset(&a, 0, sizeof(a));
  a.in = spec; a.fstride = fstride;
  a.nrows = p->n[0] * p->n[1]; a.n2 = p->n[2]; a.n2h = p->n2h; a.ld2 = ld2; a.nf = nf;
  a.pairs = p->pairs; a.ax = p->ax[2]; a.tw = p->tw[2];
  return a;
}

template <typename T>
static int rows_inv_store_t(gbofdft_plan* p, const void* spec, int64_t fstride, int ld2, int nf, void* out,
                            int64_t ostride, double scale, cudaStream_t st) {
  RowsInvArgs a = rows_inv_args<T>(p, spec, fstride, ld2, nf);
  a.out = out; a.ostride = ostride; a.scale = scale;
  const size_t sm = rows_smem<T>(a.n2, nf * a.pairs);
  if (set_smem(k_rows_inv_store<T>, sm)) return GBOFDFT_ERR_CUDA;
  const int nblk = (a.nrows + 2 * a.pairs - 1) / (2 * a.pairs);
  k_rows_inv_store<T><<<nblk, 256, sm, st>>>(a);
  GB_CHECK_LAUNCH();
  return 0;
}

int gb_rows_inv_store(gbofdft_plan* p, const void* spec, int64_t fstride, int ld2, int nf, void* out,
                      int64_t ostride, double scale, cudaStream_t st) {
  if (gb_use_ct()) {
    const int rc = p->prec == GBOFDFT_F64
                       ? gb_ct_rows_inv_f64(p, spec, fstride, ld2, nf, out, ostride, scale, nullptr, nullptr, nullptr,
                                            nullptr, 0, nullptr, nullptr, st)
                       : gb_ct_rows_inv_f32(p, spec, fstride, ld2, nf, out, ostride, scale, nullptr, nullptr, nullptr,
                                            nullptr, 0, nullptr, nullptr, st);
    if (rc != 1) return rc;
  }
  return p->prec == GBOFDFT_F64 ? rows_inv_store_t<double>(p, spec, fstride, ld2, nf, out, ostride, scale, st)
                                : rows_inv_store_t<float>(p, spec, fstride, ld2, nf, out, ostride, scale, st);
}

template <typename T>
static int rows_inv_eval_t(gbofdft_plan* p, const void* spec, int64_t fstride, int nf, const EvalDesc& ev,
                           const void* rho, const void* vloc, void* pot, int calc_e, double* energies,
                           cudaStream_t st) {
  RowsInvArgs a = rows_inv_args<T>(p, spec, fstride, p->ld2, nf);
  a.ev = ev; a.rho = rho; a.vloc = vloc; a.pot = pot; a.partials = p->partials; a.calc_e = calc_e;
  const int P = a.pairs;
  const size_t sm = rows_smem<T>(a.n2, (nf > 0 ? nf : 1) * P);
  if (nf == 0) a.nf = 0;
  if (set_smem(k_rows_inv_eval<T>, sm)) return GBOFDFT_ERR_CUDA;
  const int64_t nblk = (a.nrows + 2 * P - 1) / (2 * P);
  if (nblk > p->max_partials) return gb_set_error(GBOFDFT_ERR_STATE, "partials buffer too small");
  k_rows_inv_eval<T><<<(unsigned)nblk, 256, sm, st>>>(a);
  GB_CHECK_LAUNCH();
  if (calc_e) {
    k_energy_final<<<6, 256, 0, st>>>(p->partials, nblk, p->dV, ev.e_ion, energies, gb_plan_counter(p));
    GB_CHECK_LAUNCH();
  }
  return 0;
}

int gb_rows_inv_eval(gbofdft_plan* p, const void* spec, int64_t fstride, int nf, const EvalDesc& ev,
                     const void* rho, const void* vloc, void* pot, int calc_e, double* energies, cudaStream_t st) {
  if (gb_use_ct()) {
    int64_t nblk = 0;
    const int rc = p->prec == GBOFDFT_F64
                       ? gb_ct_rows_inv_f64(p, spec, fstride, p->ld2, nf, nullptr, 0, 1.0, &ev, rho, vloc, pot, calc_e,
                                            p->partials, &nblk, st)
                       : gb_ct_rows_inv_f32(p, spec, fstride, p->ld2, nf, nullptr, 0, 1.0, &ev, rho, vloc, pot, calc_e,
                                            p->partials, &nblk, st);
    if (rc == 0 && calc_e) {
      if (nblk > p->max_partials) return gb_set_error(GBOFDFT_ERR_STATE, "partials buffer too small");
      k_energy_final<<<6, 256, 0, st>>>(p->partials, nblk, p->dV, ev.e_ion, energies, gb_plan_counter(p));
      GB_CHECK_LAUNCH();
    }
    if (rc != 1) return rc;
  }
  return p->prec == GBOFDFT_F64
             ? rows_inv_eval_t<double>(p, spec, fstride, nf, ev, rho, vloc, pot, calc_e, energies, st)
             : rows_inv_eval_t<float>(p, spec, fstride, nf, ev, rho, vloc, pot, calc_e, energies, st);
}

template <typename T>
static ColsArgs cols_args(gbofdft_plan* p, void* spec, int64_t fstride, int ld2, int axis, double scale) {
  ColsArgs a;
  memset(&a, 0, sizeof(a));
  a.data = spec; a.fstride = fstride;
  a.n = p->n[axis];
  a.stride = axis == 1 ? ld2 : (int64_t)p->n[1] * ld2;
  a.ostride = axis == 1 ? (int64_t)p->n[1] * ld2 : ld2;
  a.ncols = p->n2h; a.tb = p->tb[axis];
  a.ax = p->ax[axis]; a.tw = p->tw[axis]; a.scale = scale;
  a.gi = p->gi;
  a.gi.ld2 = ld2;
  return a;
}

template <typename T>
static int cols_t(gbofdft_plan* p, void* spec, int64_t fstride, int ld2, int nf, int axis, int dir, double scale,
                  cudaStream_t st) {
  ColsArgs a = cols_args<T>(p, spec, fstride, ld2, axis, scale);
  const size_t sm = cols_smem<T>(a.n, a.tb);
  dim3 grid((a.ncols + a.tb - 1) / a.tb, p->n[axis == 1 ? 0 : 1], nf);
  if (dir < 0) {
    if (set_smem(k_cols<T, -1>, sm)) return GBOFDFT_ERR_CUDA;
    k_cols<T, -1><<<grid, 256, sm, st>>>(a);
  } else {
    if (set_smem(k_cols<T, 1>, sm)) return GBOFDFT_ERR_CUDA;
    k_cols<T, 1><<<grid, 256, sm, st>>>(a);
  }
  GB_CHECK_LAUNCH();
  return 0;
}

int gb_cols(gbofdft_plan* p, void* spec, int64_t fstride, int ld2, int nf, int axis, int dir, double scale,
            cudaStream_t st) {
  if (gb_use_ct()) {
    const int rc = p->prec == GBOFDFT_F64 ? gb_ct_cols_f64(p, spec, fstride, ld2, nf, axis, dir, scale, nullptr, st)
                                          : gb_ct_cols_f32(p, spec, fstride, ld2, nf, axis, dir, scale, nullptr, st);
    if (rc != 1) return rc;
  }
  return p->prec == GBOFDFT_F64 ? cols_t<double>(p, spec, fstride, ld2, nf, axis, dir, scale, st)
                                : cols_t<float>(p, spec, fstride, ld2, nf, axis, dir, scale, st);
}

template <typename T>
static int cols_conv_t(gbofdft_plan* p, void* spec, int64_t fstride, int ld2, int nf, const KerDesc& kd,
                       double scale, cudaStream_t st) {
  ColsArgs a = cols_args<T>(p, spec, fstride, ld2, 0, 1.0);
  a.kd = kd;
  for (int f = 0; f < nf; ++f) a.kd.coef[f] = kd.coef[f] * scale;
  const size_t sm = cols_smem<T>(a.n, a.tb);
  if (set_smem(k_cols_conv<T>, sm)) return GBOFDFT_ERR_CUDA;
  dim3 grid((a.ncols + a.tb - 1) / a.tb, p->n[1], nf);
  k_cols_conv<T><<<grid, 256, sm, st>>>(a);
  GB_CHECK_LAUNCH();
  return 0;
}

int gb_cols_conv(gbofdft_plan* p, void* spec, int64_t fstride, int ld2, int nf, const KerDesc& kd, double scale,
                 cudaStream_t st) {
  if (gb_use_ct()) {
    KerDesc k2 = kd;
    for (int f = 0; f < nf; ++f) k2.coef[f] = kd.coef[f] * scale;
    const int rc = p->prec == GBOFDFT_F64 ? gb_ct_cols_f64(p, spec, fstride, ld2, nf, 0, -1, 1.0, &k2, st)
                                          : gb_ct_cols_f32(p, spec, fstride, ld2, nf, 0, -1, 1.0, &k2, st);
    if (rc != 1) return rc;
  }
  return p->prec == GBOFDFT_F64 ? cols_conv_t<double>(p, spec, fstride, ld2, nf, kd, scale, st)
                                : cols_conv_t<float>(p, spec, fstride, ld2, nf, kd, scale, st);
}

int gb_eval_plane(gbofdft_plan* p, const void* rho, int nf, const int* ops, double beta, const KerDesc& kd,
                  const EvalDesc& ev, const void* vloc, void* pot, int calc_e, double* energies, cudaStream_t st) {
  if (!p->plane || p->prec != GBOFDFT_F32 || nf <= 0 || !gb_use_ct()) return 1;
  const float* pm_arr[GB_MAX_FIELDS] = {nullptr, nullptr, nullptr, nullptr};
  for (int f = 0; f < nf; ++f) {
    if (kd.type[f] != KER_ARRAY) continue;
    if (!p->wt_pm || kd.arr[f] != p->wt_pm_src) return 1;
    pm_arr[f] = p->wt_pm;
  }
  const int64_t fs = p->NG;
  int rc = gb_ct_rows_fwd_pm_f32(p, rho, p->spec, fs, nf, ops, beta, st);
  if (!rc) rc = gb_plane_conv_f32(p, p->spec, fs, nf, &kd, pm_arr, 1.0 / (double)p->N, st);
  if (rc) return rc == 1 ? gb_set_error(GBOFDFT_ERR_STATE, "plane pipeline: size without specialisation") : rc;
  int64_t nblk = 0;
  rc = gb_ct_rows_inv_eval_pm_f32(p, p->spec, fs, nf, &ev, rho, vloc, pot, calc_e, p->partials, &nblk, st);
  if (rc) return rc == 1 ? gb_set_error(GBOFDFT_ERR_STATE, "plane pipeline: size without specialisation") : rc;
  if (calc_e) {
    if (nblk > p->max_partials) return gb_set_error(GBOFDFT_ERR_STATE, "partials buffer too small");
    k_energy_final<<<6, 256, 0, st>>>(p->partials, nblk, p->dV, ev.e_ion, energies, gb_plan_counter(p));
    GB_CHECK_LAUNCH();
  }
  return 0;
}

// energies = reference energies + the changes k_energy_final wrote
__global__ void k_add_ref_energies(double* __restrict__ e, const double* __restrict__ eref) {
  if (threadIdx.x < GB_NE) e[threadIdx.x] += eref[threadIdx.x];
}

int gb_eval_delta_core(gbofdft_plan* p64, gbofdft_plan* p32, const double* rho, const double* rho_ref,
                       const double* pot_ref, const double* eref, const double* cref, int nf, const int* ops,
                       double beta, const KerDesc& kd, const EvalDesc& ev, const double* vloc, double* pot,
                       int calc_e, double* energies, cudaStream_t st) {
  GB_REQUIRE(p32->plane_ok && p32->prec == GBOFDFT_F32 && nf > 0 && gb_use_ct(),
             "delta evaluation: needs an FP32 plan with the plane pipeline");
  const float* pm_arr[GB_MAX_FIELDS] = {nullptr, nullptr, nullptr, nullptr};
  for (int f = 0; f < nf; ++f) {
    if (kd.type[f] != KER_ARRAY) continue;
    GB_REQUIRE(p32->wt_pm && kd.arr[f] == p32->wt_pm_src,
               "delta evaluation: the FP32 kernel table was not built on the FP32 plan");
    pm_arr[f] = p32->wt_pm;
  }
  const int64_t fs = p32->NG;
  int rc = gb_delta_rows_fwd(p32, rho, rho_ref, p32->spec, fs, nf, ops, beta, st);
  if (!rc) rc = gb_plane_conv_f32(p32, p32->spec, fs, nf, &kd, pm_arr, 1.0 / (double)p32->N, st);
  if (rc) return rc == 1 ? gb_set_error(GBOFDFT_ERR_STATE, "delta evaluation: plane size without specialisation") : rc;
  int64_t nblk = 0;
  rc = gb_delta_rows_inv_eval(p32, p32->spec, fs, nf, &ev, rho, rho_ref, pot_ref, vloc, cref, p64->N, pot, calc_e,
                              p64->partials, &nblk, st);
  if (rc) return rc;
  if (calc_e) {
    if (nblk > p64->max_partials) return gb_set_error(GBOFDFT_ERR_STATE, "partials buffer too small");
    // the partials are energy changes: sum them (no ion term), add the reference's
    k_energy_final<<<6, 256, 0, st>>>(p64->partials, nblk, p64->dV, 0.0, energies, gb_plan_counter(p64));
    GB_CHECK_LAUNCH();
    k_add_ref_energies<<<1, 32, 0, st>>>(energies, eref);
    GB_CHECK_LAUNCH();
  }
  return 0;
}

int gb_build_precond(gbofdft_plan* p, double rho0, void* out, cudaStream_t st) {
  GB_REQUIRE(rho0 > 0.0, "preconditioner: rho0 must be positive (got %g)", rho0);
  // the optimiser's workspace keeps it between solves of the same grid: the
  // table depends on the grid and the mean density only (stream order makes
  // the earlier build complete before any later reader on the plan's stream)
  for (int i = 0; i < 2; ++i)
    if (p->precond_buf[i] == out && p->precond_rho0[i] == rho0) return 0;
  const int64_t total = p->NG;
  const int nblk = (int)((total + 255) / 256 > 4096 ? 4096 : (total + 255) / 256);
  // plans that convolve with it on the plane pipeline keep a plane-major copy
  if (p->plane_precond && p->plane_ok && !p->precond_pm) {
    cudaError_t e = cudaMalloc(&p->precond_pm, sizeof(float) * (size_t)p->NG);
    if (e != cudaSuccess) {
      p->precond_pm = nullptr;
      return gb_set_error(GBOFDFT_ERR_ALLOC, "preconditioner: plane-major copy: %s", cudaGetErrorString(e));
    }
  }
  float* pm = p->plane_precond && p->plane_ok ? p->precond_pm : nullptr;
  if (p->prec == GBOFDFT_F64)
    k_precond<double><<<nblk, 256, 0, st>>>(p->gi, rho0, reinterpret_cast<double*>(out), nullptr);
  else k_precond<float><<<nblk, 256, 0, st>>>(p->gi, rho0, reinterpret_cast<float*>(out), pm);
  GB_CHECK_LAUNCH();
  const int slot = p->precond_next;
  p->precond_next ^= 1;
  p->precond_buf[slot] = out;
  p->precond_rho0[slot] = rho0;
  if (pm) p->precond_pm_src = out;
  return 0;
}

int gb_build_wt_kernel(gbofdft_plan* p, double rho0, double x, double alpha, double beta, void* out,
                       cudaStream_t st) {
  GB_REQUIRE(rho0 > 0.0, "wt kernel: rho0 must be positive (got %g)", rho0);
  const double tkf = 2.0 * cbrt(3.0 * rho0 * kPi * kPi);
  const double ctf = 0.3 * pow(3.0 * kPi * kPi, 2.0 / 3.0);
  const double factor = 5.0 / (9.0 * alpha * beta * pow(rho0, alpha + beta - 5.0 / 3.0)) * ctf;
  const int64_t total = p->NG;
  const int nblk = (int)((total + 255) / 256 > 4096 ? 4096 : (total + 255) / 256);
  if (p->prec == GBOFDFT_F64) {
    k_wt_kernel<double><<<nblk, 256, 0, st>>>(p->gi, tkf, factor, x, reinterpret_cast<double*>(out), nullptr);
  } else {
    // plans that can use the plane pipeline keep a plane-major copy of the table
    // (allocated with the first table built on the plan)
    if (p->plane_ok && !p->wt_pm) {
      cudaError_t e = cudaMalloc(&p->wt_pm, sizeof(float) * (size_t)p->NG);
      if (e != cudaSuccess) {
        p->wt_pm = nullptr;
        return gb_set_error(GBOFDFT_ERR_ALLOC, "wt kernel: plane-major table: %s", cudaGetErrorString(e));
      }
    }
    k_wt_kernel<float><<<nblk, 256, 0, st>>>(p->gi, tkf, factor, x, reinterpret_cast<float*>(out),
                                             p->plane_ok ? p->wt_pm : nullptr);
    p->wt_pm_src = p->plane_ok ? out : nullptr;
  }
  GB_CHECK_LAUNCH();
  return 0;
}
