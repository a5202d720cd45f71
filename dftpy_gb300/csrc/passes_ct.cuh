// Compile-time-size versions of the FFT passes of passes.cu (same data
// layout, same semantics), instantiated for the grid sizes of the workloads.
// Each launcher returns 1 when the size has no specialisation (the caller
// then uses the generic runtime-radix kernels), 0 on success, or an error.
#pragma once
#include <math.h>
#include <string.h>
#include <type_traits>

#include "fft_ct.cuh"
#include "gkernels.cuh"
#include "plan.h"

namespace gbct {

constexpr double kZero = 1e-30;

template <typename F>
__host__ inline bool ct_dispatch(int n, F&& f) {
  switch (n) {
    case 32: f(std::integral_constant<int, 32>{}); return true;
    case 64: f(std::integral_constant<int, 64>{}); return true;
    case 96: f(std::integral_constant<int, 96>{}); return true;
    case 128: f(std::integral_constant<int, 128>{}); return true;
    case 160: f(std::integral_constant<int, 160>{}); return true;
    case 256: f(std::integral_constant<int, 256>{}); return true;
    case 360: f(std::integral_constant<int, 360>{}); return true;
    default: return false;
  }
}

// Launch-shape parameters (overridable at build time for tuning sweeps)
#ifndef GB_CT_RP_F32
#define GB_CT_RP_F32 4
#endif
#ifndef GB_CT_TB_F32
#define GB_CT_TB_F32 16
#endif
#ifndef GB_CT_TB_F32_LARGE
#define GB_CT_TB_F32_LARGE 8   // FP32 column tiles of lines longer than 256
#endif
#ifndef GB_CT_ROWS_MINB
#define GB_CT_ROWS_MINB 1
#endif
#ifndef GB_CT_COLS_MINB
#define GB_CT_COLS_MINB 1
#endif
#ifndef GB_CT_PF_F32
#define GB_CT_PF_F32 4      // density / v_loc values prefetched per thread in the FP32 evaluation epilogue (measured best)
#endif
#ifndef GB_CT_CONV_MINB
#define GB_CT_CONV_MINB 5   // FP32 convolution pass, N <= 128: >= 5 CTAs/SM (measured best at 128^3; no spills)
#endif

template <typename T> struct RowsCfg;            // row pairs per CTA (per field)
template <> struct RowsCfg<float> { static constexpr int RP = GB_CT_RP_F32; };
template <> struct RowsCfg<double> { static constexpr int RP = 4; };
// threads of a row-pass CTA: TPL per line, one line per (field, row pair)
template <typename T, int N> constexpr int rows_threads_max() { return Tpl<N>::value * RowsCfg<T>::RP * GB_MAX_FIELDS; }
template <typename T, int N> struct ColsCfg {     // columns per tile
  static constexpr int TB = sizeof(T) == 4 ? (N <= 256 ? GB_CT_TB_F32 : GB_CT_TB_F32_LARGE) : 8;
};
// minimum resident CTAs per SM for the column passes (caps registers)
template <typename T, int N, bool CONV> constexpr int cols_minb() {
  if constexpr (CONV) return (sizeof(T) == 4 && N <= 128) ? GB_CT_CONV_MINB : 1;
  else return GB_CT_COLS_MINB;
}

// A scalar kernel parameter in both precisions, converted on the host: the
// FP32 kernels then run without double->float conversions, which execute on
// the FP64 pipe (a slow one on this part).
struct Sc {
  double d;
  float f;
  void set(double v) { d = v; f = (float)v; }
};
template <typename T> __device__ __forceinline__ T sc(const Sc& s) {
  if constexpr (sizeof(T) == 8) return s.d; else return s.f;
}

// ---- pointwise functions -----------------------------------------------------
// x^(1/2), x^(5/6) and friends for x >= 1e-30 (the reference's clamps)
template <typename T> __device__ __forceinline__ T sqrt_pos(T x) { return x * rsqrt_d(x); }

template <typename T> __device__ __forceinline__ T pow_beta_ct(T x, bool b56, T beta) {
  if (b56) {
    const T z3 = rcbrt_d(x), z2 = rsqrt_d(x);
    return (x * z2) * (x * z3 * z3);         // x^(1/2) x^(1/3)
  }
  return pow(x, beta);
}

template <typename T>
__device__ __forceinline__ T prologue_ct(int op, T rho, bool b56, T beta, T rho0 = (T)0, T inv0 = (T)0) {
  if (op == OP_SQRT) return sqrt_pos<T>(rho > (T)0 ? rho : (T)kZero);
  if (op == OP_POWB) return pow_beta_ct<T>(rho < (T)kZero ? (T)kZero : rho, b56, beta);
  if (op >= OP_WGC0) {
    // the WGC transform inputs rho^e u^k, rho clamped at 1e-30 (e = beta)
    const T rc = rho > (T)kZero ? rho : (T)kZero;
    const T B = pow_beta_ct<T>(rc, b56, beta);
    const T u = (rc - rho0) * inv0;
    return op == OP_WGC0 ? B : (op == OP_WGC1 ? u * B : u * u * B);
  }
  return rho;
}

// ---- rows forward ---------------------------------------------------------------
// One CTA: RP row pairs of the input, all nf derived fields transformed at
// once (line = field * RP + pair; TPL threads per line).
struct CtRowsFwd {
  const void* in;
  void* out;
  int64_t fstride;
  int nrows, ld2, nf;
  int op[GB_MAX_FIELDS];
  int b56;            // beta == 5/6
  Sc beta, half;      // half = scale / 2
  Sc rho0, inv0;      // WGC prologues: expansion density and its inverse
  const void* tw;
};

// PM: write plane-major spectra (k2 * nrows + row) for the plane pass;
// consecutive threads then take consecutive rows of one k2.
template <typename T, int N, bool PM>
__global__ void __launch_bounds__(rows_threads_max<T, N>(), GB_CT_ROWS_MINB) k_ct_rows_fwd(CtRowsFwd a) {
  constexpr int RP = RowsCfg<T>::RP, TPL = Tpl<N>::value, NP = Pad<T, N>::NP, NH = N / 2 + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nl = a.nf * RP;
  cpx<T>* tw = reinterpret_cast<cpx<T>*>(smem_raw);
  cpx<T>* A = tw + N;
  cpx<T>* B = A + nl * NP;
  T* R = reinterpret_cast<T*>(B + nl * NP);      // [2 RP][N] real input rows
  const int tid = threadIdx.x, l = tid / TPL, lane = tid % TPL;
  const int64_t base = (int64_t)blockIdx.x * 2 * RP;
  const cpx<T>* twg = reinterpret_cast<const cpx<T>*>(a.tw);
  for (int i = tid; i < N; i += blockDim.x) tw[i] = twg[i];
  const T* in = reinterpret_cast<const T*>(a.in);
  // input rows: batches of independent loads ahead of their stores
  constexpr int NE = 2 * RP * N, UNR = 4;
#pragma unroll 1
  for (int b0 = 0; b0 < NE; b0 += UNR * (int)blockDim.x) {
    T v[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const int idx = b0 + u * (int)blockDim.x + tid;
      const int64_t row = base + idx / N;
      v[u] = (idx < NE && row < a.nrows) ? __ldg(in + row * N + idx % N) : (T)0;
    }
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const int idx = b0 + u * (int)blockDim.x + tid;
      if (idx < NE) R[idx] = v[u];
    }
  }
  __syncthreads();
  const bool b56 = a.b56 != 0;
  const T beta = sc<T>(a.beta);
  const T rho0 = sc<T>(a.rho0), inv0 = sc<T>(a.inv0);
  // the three WGC inputs rho^e u^k (k = 0, 1, 2) of one exponent share the
  // power: computed once per point (the same arithmetic as prologue_ct)
  const bool wgc3 = a.nf == 3 && a.op[0] == OP_WGC0 && a.op[1] == OP_WGC1 && a.op[2] == OP_WGC2;
  if (wgc3) {
    for (int idx = tid; idx < RP * N; idx += blockDim.x) {
      const int l2 = idx / N, j = idx % N;
      const int64_t ra = base + 2 * l2;
      T B[2] = {(T)0, (T)0}, u[2] = {(T)0, (T)0};
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (ra + h < a.nrows) {
          const T rho = R[(2 * l2 + h) * N + j];
          const T rc = rho > (T)kZero ? rho : (T)kZero;
          B[h] = pow_beta_ct<T>(rc, b56, beta);
          u[h] = (rc - rho0) * inv0;
        }
      }
      A[sw<T, NP>(0 * RP + l2, j)] = cpx<T>{B[0], B[1]};
      A[sw<T, NP>(1 * RP + l2, j)] = cpx<T>{u[0] * B[0], u[1] * B[1]};
      A[sw<T, NP>(2 * RP + l2, j)] = cpx<T>{u[0] * u[0] * B[0], u[1] * u[1] * B[1]};
    }
  }
  // fields in an unrolled outer loop: the field's prologue op is a
  // compile-time parameter index, and every index split below is by a
  // compile-time constant
#pragma unroll
  for (int f = 0; f < GB_MAX_FIELDS; ++f) {
    if (wgc3 || f >= a.nf) break;
    const int op = a.op[f];
    for (int idx = tid; idx < RP * N; idx += blockDim.x) {
      const int l2 = idx / N, j = idx % N;
      const int64_t ra = base + 2 * l2;
      const T x0 = ra < a.nrows ? prologue_ct<T>(op, R[(2 * l2) * N + j], b56, beta, rho0, inv0) : (T)0;
      const T x1 = ra + 1 < a.nrows ? prologue_ct<T>(op, R[(2 * l2 + 1) * N + j], b56, beta, rho0, inv0) : (T)0;
      A[sw<T, NP>(f * RP + l2, j)] = cpx<T>{x0, x1};
    }
  }
  __syncthreads();
  cpx<T>* res = fft<-1, T, N>(A, B, tw, l, lane, true);
  cpx<T>* out = reinterpret_cast<cpx<T>*>(a.out);
  const T half = sc<T>(a.half);
#pragma unroll
  for (int f = 0; f < GB_MAX_FIELDS; ++f) {
    if (f >= a.nf) break;
    cpx<T>* o = out + f * a.fstride;
    for (int idx = tid; idx < RP * NH; idx += blockDim.x) {
      // plane-major: consecutive threads take consecutive row pairs of one k
      const int l2 = PM ? idx % RP : idx / NH, k = PM ? idx / RP : idx % NH;
      const int line = f * RP + l2;
      const int64_t ra = base + 2 * l2, rb = ra + 1;
      if (ra >= a.nrows) continue;
      const cpx<T> Z = res[sw<T, NP>(line, k)];
      const cpx<T> Zc = res[sw<T, NP>(line, k == 0 ? 0 : N - k)];
      const int64_t ia = PM ? (int64_t)k * a.nrows + ra : ra * a.ld2 + k;
      const int64_t ib = PM ? ia + 1 : ia + a.ld2;
      o[ia] = cpx<T>{(Z.x + Zc.x) * half, (Z.y - Zc.y) * half};
      if (rb < a.nrows) o[ib] = cpx<T>{(Z.y + Zc.y) * half, (Zc.x - Z.x) * half};
    }
  }
}

// ---- rows inverse ----------------------------------------------------------------
struct CtRowsInv {
  const void* in;
  int64_t fstride;
  int nrows, ld2, nf;
  const void* tw;
  void* out;
  int64_t ostride;
  Sc scale;
  EvalDesc ev;
  Sc tf_v, tf_e, vw_y, two_alpha, inv_two_alpha, wt_beta;  // evaluation constants
  int b56;
  const void* rho;
  const void* vloc;
  void* pot;
  double* partials;
  int calc_e;
};

// irfftn line build (all fields) + inverse FFT; result line (f * RP + pair)
// holds row 2 pair in .x and row 2 pair + 1 in .y.
template <typename T, int N, bool PM = false, int NFMAX = GB_MAX_FIELDS>
__device__ __forceinline__ cpx<T>* ct_rows_inv_lines(const CtRowsInv& a, int64_t base, cpx<T>* tw, cpx<T>* A,
                                                     cpx<T>* B) {
  constexpr int RP = RowsCfg<T>::RP, TPL = Tpl<N>::value, NP = Pad<T, N>::NP, NH = N / 2 + 1;
  const int tid = threadIdx.x, l = tid / TPL, lane = tid % TPL;
  const int nl = a.nf * RP;
  const cpx<T>* src0 = reinterpret_cast<const cpx<T>*>(a.in);
#pragma unroll
  for (int f = 0; f < NFMAX; ++f) {
    if (f >= a.nf) break;
    const cpx<T>* src = src0 + f * a.fstride;
    for (int idx = tid; idx < RP * NH; idx += blockDim.x) {
      const int l2 = PM ? idx % RP : idx / NH, k = PM ? idx / RP : idx % NH;
      const int line = f * RP + l2;
      const int64_t ra = base + 2 * l2, rb = ra + 1;
      const int64_t ia = PM ? (int64_t)k * a.nrows + ra : ra * a.ld2 + k;
      const int64_t ib = PM ? ia + 1 : ia + a.ld2;
      cpx<T> va = {(T)0, (T)0}, vb = {(T)0, (T)0};
      if (ra < a.nrows) va = src[ia];
      if (rb < a.nrows) vb = src[ib];
      if (k == 0 || 2 * k == N) { va.y = (T)0; vb.y = (T)0; }
      A[sw<T, NP>(line, k)] = cpx<T>{va.x - vb.y, va.y + vb.x};
      if (k > 0 && 2 * k < N) A[sw<T, NP>(line, N - k)] = cpx<T>{va.x + vb.y, vb.x - va.y};
    }
  }
  __syncthreads();
  return fft<1, T, N>(A, B, tw, l, lane, true);
}

template <typename T, int N, bool PM = false>
__global__ void __launch_bounds__(rows_threads_max<T, N>()) k_ct_rows_inv_store(CtRowsInv a) {
  constexpr int RP = RowsCfg<T>::RP, NP = Pad<T, N>::NP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nl = a.nf * RP;
  cpx<T>* tw = reinterpret_cast<cpx<T>*>(smem_raw);
  cpx<T>* A = tw + N;
  cpx<T>* B = A + nl * NP;
  const int tid = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * 2 * RP;
  const cpx<T>* twg = reinterpret_cast<const cpx<T>*>(a.tw);
  for (int i = tid; i < N; i += blockDim.x) tw[i] = twg[i];
  cpx<T>* res = ct_rows_inv_lines<T, N, PM>(a, base, tw, A, B);
  T* out = reinterpret_cast<T*>(a.out);
  const T s = sc<T>(a.scale);
  for (int idx = tid; idx < a.nf * 2 * RP * N; idx += blockDim.x) {
    const int f = idx / (2 * RP * N), r = idx % (2 * RP * N);
    const int rr = r / N, j = r % N;
    const int64_t row = base + rr;
    if (row >= a.nrows) continue;
    const cpx<T> z = res[sw<T, NP>(f * RP + (rr >> 1), j)];
    out[f * a.ostride + row * N + j] = ((rr & 1) ? z.y : z.x) * s;
  }
}

// WGC nonlocal potential from its six real-space fields (X0..X2 from rho^b,
// Y0..Y2 from rho^a): the inverse row pass of the combined spectra with the
// potential added to pot in the same kernel (FP32, potential only), instead
// of storing the six fields and reading them back.
struct CtRowsInvWgc {
  CtRowsInv r;          // spectra (plane-major), nf = 6 (3 when a == b), twiddles
  const float* rho;
  float rho0, inv0, ea, eb;
  int two;
  float* pot;
  double* part;         // non-null: per-CTA partial sums of int A (X0 + u X1 + u^2 X2)
};

template <int N>
__global__ void __launch_bounds__(Tpl<N>::value * RowsCfg<float>::RP * 6) k_ct_rows_inv_wgc(CtRowsInvWgc a) {
  constexpr int RP = RowsCfg<float>::RP, NP = Pad<float, N>::NP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nl = a.r.nf * RP;
  cpx<float>* tw = reinterpret_cast<cpx<float>*>(smem_raw);
  cpx<float>* A = tw + N;
  cpx<float>* B = A + nl * NP;
  const int tid = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * 2 * RP;
  const cpx<float>* twg = reinterpret_cast<const cpx<float>*>(a.r.tw);
  for (int i = tid; i < N; i += blockDim.x) tw[i] = twg[i];
  cpx<float>* res = ct_rows_inv_lines<float, N, true, 6>(a.r, base, tw, A, B);
  const int gy = a.two ? 3 : 0;
  float es = 0.0f;   // per-thread energy sum (a handful of points), FP64 above
  for (int idx = tid; idx < 2 * RP * N; idx += blockDim.x) {
    const int rr = idx / N, j = idx % N;
    const int64_t row = base + rr;
    if (row >= a.r.nrows) continue;
    const int64_t g = row * N + j;
    const int pr = rr >> 1;
    auto fld = [&](int f) {
      const cpx<float> z = res[sw<float, NP>(f * RP + pr, j)];
      return (rr & 1) ? z.y : z.x;
    };
    const float X0 = fld(0), X1 = fld(1), X2 = fld(2);
    const float Y0 = fld(gy), Y1 = fld(gy + 1), Y2 = fld(gy + 2);
    const float r = __ldg(a.rho + g);
    const float rc = r > (float)kZero ? r : (float)kZero;
    const float u = (rc - a.rho0) * a.inv0;
    const float Aa = powf(rc, a.ea);
    const float sx = X0 + u * X1 + u * u * X2;
    es += Aa * sx;
    float v;
    if (a.two) {
      const float Bb = powf(rc, a.eb);
      v = a.ea * Aa / rc * sx + Aa * a.inv0 * (X1 + 2.0f * u * X2) + a.eb * Bb / rc * (Y0 + u * Y1 + u * u * Y2) +
          Bb * a.inv0 * (Y1 + 2.0f * u * Y2);
    } else {
      v = 2.0f * (a.ea * Aa / rc * sx + Aa * a.inv0 * (X1 + 2.0f * u * X2));
    }
    a.pot[g] += v;
  }
  if (!a.part) return;
  __shared__ double red[32];
  const int lane32 = tid & 31, warp = tid >> 5;
  const double wsum = warp_sum((double)es);
  if (lane32 == 0) red[warp] = wsum;
  __syncthreads();
  if (tid == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) t.add(red[w]);
    a.part[blockIdx.x] = t.value();
  }
}

template <typename T>
__device__ __forceinline__ void pz_lda_ct(T rho, T& eps, T& pot, bool want_e) {
  const T a = (T)0.0311, b = (T)-0.048, c = (T)0.0020, d = (T)-0.0116;
  const T g = (T)-0.1423, b1 = (T)1.0529, b2 = (T)0.3334;
  const T cx = (T)0.98474502184269654115;                 // (3/pi)^(1/3)
  T rc, inv_rc;                                             // rho^(1/3), clamped at 1e-30
  if (rho > (T)kZero) {
    inv_rc = rcbrt_d(rho);
    rc = rho * inv_rc * inv_rc;
  } else {
    rc = cbrt(rho);
    if (rc < (T)kZero) rc = (T)kZero;
    inv_rc = (T)1 / rc;
  }
  const T rs = (T)0.62035049089940001667 * inv_rc;        // (3/(4 pi))^(1/3) / rho^(1/3)
  pot = -cx * rc;
  eps = (T)(-0.75) * cx * rc;
  if (rs < (T)1) {
    const T lr = log(rs);
    pot += lr * (a + (T)(2.0 / 3.0) * c * rs) + b - (T)(1.0 / 3.0) * a + (T)(1.0 / 3.0) * ((T)2 * d - c) * rs;
    if (want_e) eps += a * lr + b + c * rs * lr + d * rs;
  } else {
    const T sq = rs * rsqrt_d(rs);
    const T inv = (T)1 / ((T)1 + b1 * sq + b2 * rs);
    pot += (g + ((T)(7.0 / 6.0) * g * b1) * sq + ((T)(4.0 / 3.0) * g * b2 * rs)) * inv * inv;
    if (want_e) eps += g * inv;
  }
}

// WANT_E is a template parameter so the potential-only instantiation holds no
// FP64 accumulation at all (if-converted, never-taken FP64 code still
// occupies the FP64 pipe).
template <typename T, int N, bool WANT_E, bool PM = false>
__global__ void __launch_bounds__(rows_threads_max<T, N>(), GB_CT_ROWS_MINB) k_ct_rows_inv_eval(CtRowsInv a) {
  constexpr int RP = RowsCfg<T>::RP, NP = Pad<T, N>::NP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nl = (a.nf > 0 ? a.nf : 1) * RP;
  cpx<T>* tw = reinterpret_cast<cpx<T>*>(smem_raw);
  cpx<T>* A = tw + N;
  cpx<T>* B = A + nl * NP;
  const int tid = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * 2 * RP;
  const cpx<T>* twg = reinterpret_cast<const cpx<T>*>(a.tw);
  for (int i = tid; i < N; i += blockDim.x) tw[i] = twg[i];
  const EvalDesc& ev = a.ev;
  const T* rhop = reinterpret_cast<const T*>(a.rho);
  const T* vlocp = reinterpret_cast<const T*>(a.vloc);
  // the density and v_loc of this thread's first PF elements, loaded before
  // the transforms so their latency is hidden behind them
  constexpr int PF = sizeof(T) == 4 ? GB_CT_PF_F32 : 4;
  T pre_rho[PF], pre_vl[PF];
#pragma unroll
  for (int m = 0; m < PF; ++m) {
    const int idx = tid + m * (int)blockDim.x;
    const int64_t row = base + idx / N;
    const bool ok = idx < 2 * RP * N && row < a.nrows;
    const int64_t gidx = row * N + idx % N;
    pre_rho[m] = ok ? __ldg(rhop + gidx) : (T)0;
    pre_vl[m] = (ok && ev.pp) ? __ldg(vlocp + gidx) : (T)0;
  }
  cpx<T>* res = A;
  if (a.nf > 0) res = ct_rows_inv_lines<T, N, PM>(a, base, tw, A, B);
  T* potp = reinterpret_cast<T*>(a.pot);
  constexpr bool want_e = WANT_E;
  const T tf_v = sc<T>(a.tf_v);             // (5/3) C_TF x
  const T tf_e = sc<T>(a.tf_e);             // C_TF x
  const T vw_y = sc<T>(a.vw_y);
  const T two_alpha = sc<T>(a.two_alpha);
  const T inv_two_alpha = sc<T>(a.inv_two_alpha);
  const T wt_beta = sc<T>(a.wt_beta);
  const bool b56 = a.b56 != 0;
  // per-thread energy sums in the field precision (a handful of elements per
  // thread); combined in FP64 across threads and CTAs
  T es[6] = {0, 0, 0, 0, 0, 0};
  // FP64 only: optional copy of the convolution results (delta-evaluation reference)
  T* coutp = nullptr;
  if constexpr (sizeof(T) == 8) coutp = reinterpret_cast<T*>(ev.cout);
  auto point = [&](int idx, T rho, T vl_pre) {
    const int rr = idx / N, j = idx % N;
    const int64_t row = base + rr;
    if (row >= a.nrows) return;
    const int64_t gidx = row * N + j;
    const int pr = rr >> 1;
    const bool odd = rr & 1;
    const bool pos = rho > (T)kZero;
    // rho^(-1/3) and rho^(-1/2) for positive densities (shared by TF, vW, WT)
    T z3 = (T)0, z2 = (T)0;
    if (pos) { z3 = rcbrt_d(rho); z2 = rsqrt_d(rho); }
    T pot = (T)0;
    if (ev.tf) {
      T r23;                                              // cbrt(rho^2)
      if (pos) r23 = rho * z3;
      else r23 = cbrt(rho * rho);
      pot += tf_v * r23;
      if (want_e) {
        T r53;                                            // cbrt(rho^5)
        if (pos) r53 = rho * rho * z3;
        else { T r5 = rho * rho; r5 = r5 * rho; r5 = r5 * rho; r5 = r5 * rho; r53 = cbrt(r5); }
        es[0] += r53 * tf_e;
      }
    }
    if (ev.vw) {
      const cpx<T> zz = res[sw<T, NP>(ev.slot_vw * RP + pr, j)];
      const T w = odd ? zz.y : zz.x;
      if constexpr (sizeof(T) == 8) if (coutp) coutp[ev.slot_vw * ev.cstride + gidx] = w;
      // 1 / max(sqrt(rho_m), 1e-30), rho_m = rho if rho > 0 else 1e-30
      const T inv_sq = pos ? z2 : (rho > (T)0 ? (T)1 / fmax(sqrt(rho), (T)kZero) : (T)1e15);
      const T v = (T)0.5 * w * inv_sq;
      pot += v * vw_y;
      if (want_e && rho > (T)0) es[1] += rho * v * vw_y;
    }
    if (ev.wt) {
      const cpx<T> zz = res[sw<T, NP>(ev.slot_wt * RP + pr, j)];
      const T kc = odd ? zz.y : zz.x;
      if constexpr (sizeof(T) == 8) if (coutp) coutp[ev.slot_wt * ev.cstride + gidx] = kc;
      T rb_over_rc;                                       // rc^(beta - 1), rc = max(rho, 1e-30)
      if (b56) {
        if (pos) rb_over_rc = rho * z3 * z3 * z2;          // rho^(1/3) rho^(-1/2)
        else { const T rc = (T)kZero; rb_over_rc = sqrt(rc) * cbrt(rc) / rc; }
      } else {
        const T rc = rho < (T)kZero ? (T)kZero : rho;
        rb_over_rc = pow(rc, wt_beta) / rc;
      }
      const T v = two_alpha * rb_over_rc * kc;
      pot += v;
      if (want_e) es[2] += v * rho * inv_two_alpha;
    }
    if (ev.xc) {
      T eps, vx;
      pz_lda_ct<T>(rho, eps, vx, want_e);
      pot += vx;
      if (want_e) es[3] += eps * rho;
    }
    if (ev.hartree) {
      const cpx<T> zz = res[sw<T, NP>(ev.slot_h * RP + pr, j)];
      const T vh = odd ? zz.y : zz.x;
      if constexpr (sizeof(T) == 8) if (coutp) coutp[ev.slot_h * ev.cstride + gidx] = vh;
      pot += vh;
      if (want_e) es[4] += (T)0.5 * vh * rho;
    }
    if (ev.pp) {
      const T vl = vl_pre;
      pot += vl;
      if (want_e) es[5] += vl * rho;
    }
    potp[gidx] = pot;
  };
  // one element per iteration (not unrolled: an unrolled epilogue doubles the
  // registers and halves the occupancy); the first PF come from the
  // prefetch registers
#pragma unroll 1
  for (int m = 0, idx = tid; idx < 2 * RP * N; ++m, idx += blockDim.x) {
    T rho, vl;
    if (m < PF) {
#pragma unroll
      for (int q = 0; q < PF; ++q)
        if (q == m) { rho = pre_rho[q]; vl = pre_vl[q]; }
    } else {
      const int64_t row = base + idx / N;
      if (row >= a.nrows) continue;
      const int64_t gidx = row * N + idx % N;
      rho = __ldg(rhop + gidx);
      vl = ev.pp ? __ldg(vlocp + gidx) : (T)0;
    }
    point(idx, rho, vl);
  }
  if constexpr (!WANT_E) return;
  __shared__ double red[32][6];
  const int lane32 = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const double v = warp_sum((double)es[c]);
    if (lane32 == 0) red[warp][c] = v;
  }
  __syncthreads();
  if (tid < 6) {
    KSum s;
    s.init();
    const int nw = (blockDim.x + 31) >> 5;
    for (int w = 0; w < nw; ++w) s.add(red[w][tid]);
    a.partials[(int64_t)blockIdx.x * GB_NE + tid] = s.value();
  }
}

// ---- columns -------------------------------------------------------------------
struct CtCols {
  void* data;
  int64_t fstride, stride, ostride;
  int ncols;
  const void* tw;
  Sc scale;
  Sc coef[GB_MAX_FIELDS];
  float bgf[9];        // reciprocal lattice rows in FP32 (FP32 convolution)
  GInfo gi;
  KerDesc kd;
};

// General kernel value (Nyquist partner averaging; FP64 geometry), kept out
// of line so the FP32 fast loop is not if-converted into it.
template <typename T>
__device__ __noinline__ T kernel_value_slow(const GInfo& g, int type, const void* arr, int i0, int i1, int k2) {
  return gbk::kernel_value<T>(g, type, arr, i0, i1, k2);
}

// FP32 |G|^2 along an axis-0 column: gg(m0) = (qa m0 + qb) m0 + qd with
// qa = |b0|^2, qb = 2 b0.u, qd = |u|^2, u = m1 b1 + m2 b2 (one column).
__device__ __forceinline__ void col_quadratic(const float* bg, float m1, float m2, float& qa, float& qb, float& qd) {
  const float ux = m1 * bg[3] + m2 * bg[6], uy = m1 * bg[4] + m2 * bg[7], uz = m1 * bg[5] + m2 * bg[8];
  qa = bg[0] * bg[0] + bg[1] * bg[1] + bg[2] * bg[2];
  qb = 2.0f * (bg[0] * ux + bg[1] * uy + bg[2] * uz);
  qd = ux * ux + uy * uy + uz * uz;
}

template <typename T, int N, int DIR, bool CONV>
__global__ void __launch_bounds__(Tpl<N>::value * ColsCfg<T, N>::TB, (cols_minb<T, N, CONV>()))
k_ct_cols(CtCols a) {
  constexpr int TB = ColsCfg<T, N>::TB, TPL = Tpl<N>::value, NP = Pad<T, N>::NP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cpx<T>* tw = reinterpret_cast<cpx<T>*>(smem_raw);
  cpx<T>* A = tw + N;
  cpx<T>* B = A + TB * NP;
  const int tid = threadIdx.x, l = tid / TPL, lane = tid % TPL;
  const cpx<T>* twg = reinterpret_cast<const cpx<T>*>(a.tw);
  for (int i = tid; i < N; i += blockDim.x) tw[i] = twg[i];
  const int c0 = blockIdx.x * TB;
  const int nc = min(TB, a.ncols - c0);
  const int f = blockIdx.z, outer = blockIdx.y;
  cpx<T>* base = reinterpret_cast<cpx<T>*>(a.data) + f * a.fstride + outer * a.ostride + c0;
  for (int idx = tid; idx < N * TB; idx += blockDim.x) {
    const int c = idx % TB, j = idx / TB;
    A[sw<T, NP>(c, j)] = c < nc ? base[(int64_t)j * a.stride + c] : cpx<T>{(T)0, (T)0};
  }
  __syncthreads();
  cpx<T>* res;
  if constexpr (!CONV) {
    res = fft<DIR, T, N>(A, B, tw, l, lane, true);
  } else {
    res = fft<-1, T, N>(A, B, tw, l, lane, true);
    const int type = a.kd.type[f];
    const T coef = sc<T>(a.coef[f]);
    const void* arr = a.kd.arr[f];
    bool done = false;
    if constexpr (sizeof(T) == 4) {
      if (type == KER_HARTREE || type == KER_G2) {
        // axis-0 line: i0 = j varies, i1 = outer, k2 = c0 + c.  |G|^2 from a
        // per-column quadratic in m0 (no per-element conversions); points on
        // a Nyquist plane take the partner-averaged general path.
        __shared__ float s_m0[N];
        __shared__ float s_qa[TB], s_qb[TB], s_qd[TB];
        __shared__ int s_sym[TB];
        const GInfo& g = a.gi;
        for (int j = tid; j < N; j += blockDim.x) s_m0[j] = (float)gbk::ffreq(j, N);
        if (tid < TB) {
          const int k2 = c0 + tid;
          const float m1 = (float)gbk::ffreq(outer, g.n1);
          const float m2 = (float)(g.full ? gbk::ffreq(k2, g.n2) : k2);
          col_quadratic(a.bgf, m1, m2, s_qa[tid], s_qb[tid], s_qd[tid]);
          const bool plane = g.full || k2 == 0 || ((g.n2 & 1) == 0 && 2 * k2 == g.n2);
          const bool nyq = ((g.n1 & 1) == 0 && 2 * outer == g.n1) || (g.full && (g.n2 & 1) == 0 && 2 * k2 == g.n2);
          s_sym[tid] = plane ? (nyq ? 2 : 1) : 0;   // 2: every point, 1: only i0 = n0/2
        }
        __syncthreads();
        const bool hart = type == KER_HARTREE;
        const T fourpi_c = (T)(4.0f * 3.14159265358979323846f) * coef;
        for (int idx = tid; idx < N * TB; idx += blockDim.x) {
          const int c = idx % TB, j = idx / TB;
          if (c >= nc) continue;
          const int sy = s_sym[c];
          T kv;
          if (sy == 2 || (sy == 1 && (N & 1) == 0 && 2 * j == N)) {
            kv = kernel_value_slow<T>(g, type, arr, j, outer, c0 + c) * coef;
          } else {
            const float m0 = s_m0[j];
            const float gg = (s_qa[c] * m0 + s_qb[c]) * m0 + s_qd[c];
            kv = hart ? (gg > 0.0f ? fourpi_c / gg : 0.0f) : gg * coef;
          }
          const int p = sw<T, NP>(c, j);
          res[p] = c_scale(res[p], kv);
        }
        done = true;
      }
    }
    if (!done) {
      for (int idx = tid; idx < N * TB; idx += blockDim.x) {
        const int c = idx % TB, j = idx / TB;
        if (c >= nc) continue;
        const T kv = gbk::kernel_value<T>(a.gi, type, arr, j, outer, c0 + c) * coef;
        const int p = sw<T, NP>(c, j);
        res[p] = c_scale(res[p], kv);
      }
    }
    __syncthreads();
    cpx<T>* other = (res == A) ? B : A;
    res = fft<1, T, N>(res, other, tw, l, lane, true);
  }
  const T s = sc<T>(a.scale);
  for (int idx = tid; idx < N * TB; idx += blockDim.x) {
    const int c = idx % TB, j = idx / TB;
    if (c < nc) base[(int64_t)j * a.stride + c] = c_scale(res[sw<T, NP>(c, j)], s);
  }
}

// ---- launchers -------------------------------------------------------------------
// Raise a kernel's dynamic shared-memory limit once to the largest size it
// has been launched with (keyed by kernel address and device).
template <typename K> inline int ct_smem(K kern, size_t bytes) {
  if (bytes <= 48 * 1024) return 0;
  int dev = 0;
  cudaGetDevice(&dev);
  const void* key = reinterpret_cast<const void*>(kern);
  if (gb_smem_granted(key, dev) >= (int)bytes) return 0;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return gb_set_error(GBOFDFT_ERR_CUDA, "smem attribute: %s", cudaGetErrorString(e));
  gb_smem_grant(key, dev, (int)bytes);
  return 0;
}

template <typename T, bool PM = false>
int ct_rows_fwd(gbofdft_plan* p, const void* in, void* spec, int64_t fstride, int ld2, int nf, const int* ops,
                double beta, double scale, cudaStream_t st, double rho0 = 0.0) {
  int rc = 1;
  ct_dispatch(p->n[2], [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    constexpr int RP = RowsCfg<T>::RP, NP = Pad<T, N>::NP;
    CtRowsFwd a;
    a.in = in; a.out = spec; a.fstride = fstride;
    a.nrows = p->n[0] * p->n[1]; a.ld2 = ld2; a.nf = nf;
    for (int f = 0; f < GB_MAX_FIELDS; ++f) a.op[f] = f < nf ? ops[f] : OP_RHO;
    a.b56 = fabs(beta - 5.0 / 6.0) < 1e-15;
    a.beta.set(beta);
    a.half.set(0.5 * scale);
    a.rho0.set(rho0);
    a.inv0.set(rho0 > 0.0 ? 1.0 / rho0 : 0.0);
    a.tw = p->tw[2];
    const size_t sm = sizeof(cpx<T>) * (N + 2 * (size_t)nf * RP * NP) + sizeof(T) * 2 * RP * N;
    if ((rc = ct_smem(k_ct_rows_fwd<T, N, PM>, sm))) return;
    const int nblk = (a.nrows + 2 * RP - 1) / (2 * RP);
    k_ct_rows_fwd<T, N, PM><<<nblk, Tpl<N>::value * RP * nf, sm, st>>>(a);
    gb_count_launch();
    cudaError_t e = cudaGetLastError();
    rc = e == cudaSuccess ? 0 : gb_set_error(GBOFDFT_ERR_CUDA, "ct_rows_fwd: %s", cudaGetErrorString(e));
  });
  return rc;
}

template <typename T, bool PM = false>
int ct_rows_inv(gbofdft_plan* p, const void* spec, int64_t fstride, int ld2, int nf, void* out, int64_t ostride,
                double scale, const EvalDesc* ev, const void* rho, const void* vloc, void* pot, int calc_e,
                double* partials, int64_t* nblk_out, cudaStream_t st) {
  int rc = 1;
  ct_dispatch(p->n[2], [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    constexpr int RP = RowsCfg<T>::RP, NP = Pad<T, N>::NP;
    CtRowsInv a;
    memset(&a, 0, sizeof(a));
    a.in = spec; a.fstride = fstride; a.nrows = p->n[0] * p->n[1]; a.ld2 = ld2; a.nf = nf; a.tw = p->tw[2];
    a.out = out; a.ostride = ostride; a.scale.set(scale);
    const int nblk = (a.nrows + 2 * RP - 1) / (2 * RP);
    if (nblk_out) *nblk_out = nblk;
    if (ev) {
      a.ev = *ev; a.rho = rho; a.vloc = vloc; a.pot = pot; a.calc_e = calc_e; a.partials = partials;
      const double ctf = 2.87123400018819181594;    // (3/10)(3 pi^2)^(2/3)
      a.tf_v.set(5.0 / 3.0 * ctf * ev->tf_x);
      a.tf_e.set(ctf * ev->tf_x);
      a.vw_y.set(ev->vw_y);
      a.two_alpha.set(2.0 * ev->wt_alpha);
      a.inv_two_alpha.set(ev->wt_alpha != 0.0 ? 1.0 / (2.0 * ev->wt_alpha) : 0.0);
      a.wt_beta.set(ev->wt_beta);
      a.b56 = fabs(ev->wt_beta - 5.0 / 6.0) < 1e-15;
      const int nfl = nf > 0 ? nf : 1;
      const size_t sm = sizeof(cpx<T>) * (N + 2 * (size_t)nfl * RP * NP);
      if (calc_e) {
        if ((rc = ct_smem(k_ct_rows_inv_eval<T, N, true, PM>, sm))) return;
        k_ct_rows_inv_eval<T, N, true, PM><<<nblk, Tpl<N>::value * RP * nfl, sm, st>>>(a);
      } else {
        if ((rc = ct_smem(k_ct_rows_inv_eval<T, N, false, PM>, sm))) return;
        k_ct_rows_inv_eval<T, N, false, PM><<<nblk, Tpl<N>::value * RP * nfl, sm, st>>>(a);
      }
    } else if constexpr (PM) {
      const size_t sm = sizeof(cpx<T>) * (N + 2 * (size_t)nf * RP * NP);
      if ((rc = ct_smem(k_ct_rows_inv_store<T, N, true>, sm))) return;
      k_ct_rows_inv_store<T, N, true><<<nblk, Tpl<N>::value * RP * nf, sm, st>>>(a);
    } else {
      const size_t sm = sizeof(cpx<T>) * (N + 2 * (size_t)nf * RP * NP);
      if ((rc = ct_smem(k_ct_rows_inv_store<T, N>, sm))) return;
      k_ct_rows_inv_store<T, N><<<nblk, Tpl<N>::value * RP * nf, sm, st>>>(a);
    }
    gb_count_launch();
    cudaError_t e = cudaGetLastError();
    rc = e == cudaSuccess ? 0 : gb_set_error(GBOFDFT_ERR_CUDA, "ct_rows_inv: %s", cudaGetErrorString(e));
  });
  return rc;
}

inline int ct_rows_inv_wgc(gbofdft_plan* p, const void* spec, int64_t fstride, int two, const float* rho, double rho0,
                           double ea, double eb, float* pot, double* part, int64_t* nblk_out, cudaStream_t st) {
  int rc = 1;
  ct_dispatch(p->n[2], [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    constexpr int RP = RowsCfg<float>::RP, NP = Pad<float, N>::NP;
    CtRowsInvWgc a;
    memset(&a, 0, sizeof(a));
    a.r.in = spec; a.r.fstride = fstride; a.r.nrows = p->n[0] * p->n[1]; a.r.ld2 = 0; a.r.nf = two ? 6 : 3;
    a.r.tw = p->tw[2];
    a.rho = rho; a.rho0 = (float)rho0; a.inv0 = (float)(1.0 / rho0); a.ea = (float)ea; a.eb = (float)eb;
    a.two = two; a.pot = pot; a.part = part;
    const int nblk = (a.r.nrows + 2 * RP - 1) / (2 * RP);
    if (nblk_out) *nblk_out = nblk;
    const size_t sm = sizeof(cpx<float>) * (N + 2 * (size_t)a.r.nf * RP * NP);
    if ((rc = ct_smem(k_ct_rows_inv_wgc<N>, sm))) return;
    k_ct_rows_inv_wgc<N><<<nblk, Tpl<N>::value * RP * a.r.nf, sm, st>>>(a);
    gb_count_launch();
    cudaError_t e = cudaGetLastError();
    rc = e == cudaSuccess ? 0 : gb_set_error(GBOFDFT_ERR_CUDA, "ct_rows_inv_wgc: %s", cudaGetErrorString(e));
  });
  return rc;
}

template <typename T, int DIR, bool CONV>
int ct_cols_t(gbofdft_plan* p, void* spec, int64_t fstride, int ld2, int nf, int axis, double scale,
              const KerDesc* kd, cudaStream_t st) {
  int rc = 1;
  ct_dispatch(p->n[axis], [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    constexpr int TB = ColsCfg<T, N>::TB, NP = Pad<T, N>::NP;
    CtCols a;
    memset(&a, 0, sizeof(a));
    a.data = spec; a.fstride = fstride;
    a.stride = axis == 1 ? ld2 : (int64_t)p->n[1] * ld2;
    a.ostride = axis == 1 ? (int64_t)p->n[1] * ld2 : ld2;
    a.ncols = p->n2h; a.tw = p->tw[axis]; a.scale.set(scale);
    a.gi = p->gi;
    for (int i = 0; i < 9; ++i) a.bgf[i] = (float)p->bg[i];
    if (kd) {
      a.kd = *kd;
      for (int f = 0; f < GB_MAX_FIELDS; ++f) a.coef[f].set(kd->coef[f]);
    }
    const size_t sm = sizeof(cpx<T>) * (N + 2 * TB * NP);
    if ((rc = ct_smem(k_ct_cols<T, N, DIR, CONV>, sm))) return;
    dim3 grid((p->n2h + TB - 1) / TB, p->n[axis == 1 ? 0 : 1], nf);
    k_ct_cols<T, N, DIR, CONV><<<grid, Tpl<N>::value * TB, sm, st>>>(a);
    gb_count_launch();
    cudaError_t e = cudaGetLastError();
    rc = e == cudaSuccess ? 0 : gb_set_error(GBOFDFT_ERR_CUDA, "ct_cols: %s", cudaGetErrorString(e));
  });
  return rc;
}

}  // namespace gbct

#include "plane_ct.cuh"

namespace gbct {

// Plane convolution pass over plane-major spectra (FP32); returns 1 when the
// plane sizes have no specialisation or do not fit in shared memory.
inline int plane_conv_f32(gbofdft_plan* p, void* spec, int64_t fstride, int nf, const KerDesc& kd,
                          const float* const* pm_arr, double scale, cudaStream_t st) {
  int rc = 1;
  plane_dispatch(p->n[0], p->n[1], [&](auto a0, auto a1) {
    constexpr int N0 = decltype(a0)::value, N1 = decltype(a1)::value;
    PlaneArgs a;
    memset(&a, 0, sizeof(a));
    a.spec = reinterpret_cast<float2*>(spec);
    a.fstride = fstride;
    a.tw0 = p->tw[0];
    a.tw1 = p->tw[1];
    a.gi = p->gi;
    for (int i = 0; i < 9; ++i) a.bgf[i] = (float)p->bg[i];
    for (int f = 0; f < GB_MAX_FIELDS; ++f) {
      a.type[f] = f < nf ? kd.type[f] : KER_NONE;
      a.arr[f] = (f < nf && kd.type[f] == KER_ARRAY) ? pm_arr[f] : nullptr;
      a.coef[f] = (float)(kd.coef[f] * scale);
    }
    for (int f = 0; f < nf; ++f)
      if (a.type[f] == KER_ARRAY && !a.arr[f]) {
        rc = gb_set_error(GBOFDFT_ERR_ARG, "plane_conv: field %d has no plane-major kernel table", f);
        return;
      }
    const size_t sm = PlaneCfg<N0, N1>::kSmem;
    auto launch = [&](auto kern) {
      if ((rc = ct_smem(kern, sm))) return;
      kern<<<dim3(p->n2h, nf), PlaneCfg<N0, N1>::NT, sm, st>>>(a);
    };
    if constexpr (plane_variants<N0, N1>() > 1) {
      if (p->plane_variant == 1) launch(k_plane_conv<N0, N1, 1>);
      else launch(k_plane_conv<N0, N1, 0>);
    } else {
      launch(k_plane_conv<N0, N1, 0>);
    }
    if (rc) return;
    gb_count_launch();
    cudaError_t e = cudaGetLastError();
    rc = e == cudaSuccess ? 0 : gb_set_error(GBOFDFT_ERR_CUDA, "plane_conv: %s", cudaGetErrorString(e));
  });
  return rc;
}

template <typename K> inline void plane_args_common(gbofdft_plan* p, K& a) {
  a.tw0 = p->tw[0];
  a.tw1 = p->tw[1];
}

// forward plane transforms (axis 1 then axis 0) of nf plane-major fields, in place
inline int plane_fwd_f32(gbofdft_plan* p, void* spec, int64_t fstride, int nf, cudaStream_t st) {
  int rc = 1;
  plane_dispatch(p->n[0], p->n[1], [&](auto a0, auto a1) {
    constexpr int N0 = decltype(a0)::value, N1 = decltype(a1)::value;
    PlaneFwdArgs a;
    a.spec = reinterpret_cast<float2*>(spec);
    a.fstride = fstride;
    plane_args_common(p, a);
    const size_t sm = PlaneCfg<N0, N1>::kSmemXform;
    auto launch = [&](auto kern) {
      if ((rc = ct_smem(kern, sm))) return;
      kern<<<dim3(p->n2h, nf), PlaneCfg<N0, N1>::NT, sm, st>>>(a);
    };
    if constexpr (plane_variants<N0, N1>() > 1) {
      if (p->plane_variant == 1) launch(k_plane_fwd<N0, N1, 1>);
      else launch(k_plane_fwd<N0, N1, 0>);
    } else {
      launch(k_plane_fwd<N0, N1, 0>);
    }
    if (rc) return;
    gb_count_launch();
    cudaError_t e = cudaGetLastError();
    rc = e == cudaSuccess ? 0 : gb_set_error(GBOFDFT_ERR_CUDA, "plane_fwd: %s", cudaGetErrorString(e));
  });
  return rc;
}

// WGC kernel combination and inverse plane transforms (axis 0 then axis 1)
inline int plane_wgc_inv_f32(gbofdft_plan* p, const void* spec, int64_t fstride, void* out, int64_t ostride,
                             int ngroups, const float* K, double scale, cudaStream_t st) {
  int rc = 1;
  plane_dispatch(p->n[0], p->n[1], [&](auto a0, auto a1) {
    constexpr int N0 = decltype(a0)::value, N1 = decltype(a1)::value;
    PlaneWgcArgs a;
    a.in = reinterpret_cast<const float2*>(spec);
    a.fstride = fstride;
    a.out = reinterpret_cast<float2*>(out);
    a.ostride = ostride;
    a.K = K;
    a.kstride = p->NG;
    a.scale = (float)scale;
    plane_args_common(p, a);
    const size_t sm = PlaneCfg<N0, N1>::kSmemXform;
    auto launch = [&](auto kern) {
      if ((rc = ct_smem(kern, sm))) return;
      kern<<<dim3(p->n2h, 3, ngroups), PlaneCfg<N0, N1>::NT, sm, st>>>(a);
    };
    if constexpr (plane_variants<N0, N1>() > 1) {
      if (p->plane_variant == 1) launch(k_plane_wgc_inv<N0, N1, 1>);
      else launch(k_plane_wgc_inv<N0, N1, 0>);
    } else {
      launch(k_plane_wgc_inv<N0, N1, 0>);
    }
    if (rc) return;
    gb_count_launch();
    cudaError_t e = cudaGetLastError();
    rc = e == cudaSuccess ? 0 : gb_set_error(GBOFDFT_ERR_CUDA, "plane_wgc_inv: %s", cudaGetErrorString(e));
  });
  return rc;
}

}  // namespace gbct

// Plane-major evaluation pipeline (FP32 only).
#define GB_CT_DEFINE_PLANE()                                                                                   \
  int gb_ct_rows_fwd_pm_f32(gbofdft_plan* p, const void* in, void* spec, int64_t fstride, int nf,             \
                            const int* ops, double beta, cudaStream_t st) {                                   \
    return gbct::ct_rows_fwd<float, true>(p, in, spec, fstride, 0, nf, ops, beta, 1.0, st);                   \
  }                                                                                                            \
  int gb_ct_rows_inv_eval_pm_f32(gbofdft_plan* p, const void* spec, int64_t fstride, int nf,                  \
                                 const EvalDesc* ev, const void* rho, const void* vloc, void* pot, int calc_e,  \
                                 double* partials, int64_t* nblk, cudaStream_t st) {                           \
    return gbct::ct_rows_inv<float, true>(p, spec, fstride, 0, nf, nullptr, 0, 1.0, ev, rho, vloc, pot,       \
                                          calc_e, partials, nblk, st);                                         \
  }                                                                                                            \
  int gb_plane_conv_f32(gbofdft_plan* p, void* spec, int64_t fstride, int nf, const KerDesc* kd,               \
                        const float* const* pm_arr, double scale, cudaStream_t st) {                          \
    return gbct::plane_conv_f32(p, spec, fstride, nf, *kd, pm_arr, scale, st);                                \
  }                                                                                                            \
  int gb_ct_rows_fwd_wgc_pm_f32(gbofdft_plan* p, const void* rho, void* spec, int64_t fstride, double e,        \
                                double rho0, cudaStream_t st) {                                               \
    const int ops[3] = {OP_WGC0, OP_WGC1, OP_WGC2};                                                            \
    return gbct::ct_rows_fwd<float, true>(p, rho, spec, fstride, 0, 3, ops, e, 1.0, st, rho0);                \
  }                                                                                                            \
  int gb_ct_rows_inv_store_pm_f32(gbofdft_plan* p, const void* spec, int64_t fstride, int nf, void* out,       \
                                  int64_t ostride, cudaStream_t st) {                                          \
    return gbct::ct_rows_inv<float, true>(p, spec, fstride, 0, nf, out, ostride, 1.0, nullptr, nullptr,        \
                                          nullptr, nullptr, 0, nullptr, nullptr, st);                          \
  }                                                                                                            \
  int gb_ct_rows_inv_wgc_pm_f32(gbofdft_plan* p, const void* spec, int64_t fstride, int two, const float* rho,   \
                                double rho0, double ea, double eb, float* pot, double* part, int64_t* nblk,     \
                                cudaStream_t st) {                                                            \
    return gbct::ct_rows_inv_wgc(p, spec, fstride, two, rho, rho0, ea, eb, pot, part, nblk, st);              \
  }                                                                                                            \
  int gb_plane_fwd_f32(gbofdft_plan* p, void* spec, int64_t fstride, int nf, cudaStream_t st) {                \
    return gbct::plane_fwd_f32(p, spec, fstride, nf, st);                                                      \
  }                                                                                                            \
  int gb_plane_wgc_inv_f32(gbofdft_plan* p, const void* spec, int64_t fstride, void* out, int64_t ostride,     \
                           int ngroups, const float* K, double scale, cudaStream_t st) {                       \
    return gbct::plane_wgc_inv_f32(p, spec, fstride, out, ostride, ngroups, K, scale, st);                     \
  }                                                                                                            \
  int gb_plane_supported_f32(int n0, int n1, int n2) {                                                         \
    bool rows = gbct::ct_dispatch(n2, [](auto) {});                                                            \
    bool plane = gbct::plane_dispatch(n0, n1, [](auto, auto) {});                                              \
    return rows && plane;                                                                                      \
  }                                                                                                            \
  int gb_plane_variants_f32(int n0, int n1) {                                                                  \
    int nv = 0;                                                                                                \
    gbct::plane_dispatch(n0, n1, [&](auto a0, auto a1) {                                                       \
      nv = gbct::plane_variants<decltype(a0)::value, decltype(a1)::value>();                                   \
    });                                                                                                        \
    return nv;                                                                                                 \
  }

// Instantiate the launchers of one precision (one translation unit each).
#define GB_CT_DEFINE(T, SUF)                                                                                    \
  int gb_ct_rows_fwd_##SUF(gbofdft_plan* p, const void* in, void* spec, int64_t fstride, int ld2, int nf,      \
                           const int* ops, double beta, double scale, cudaStream_t st) {                      \
    return gbct::ct_rows_fwd<T>(p, in, spec, fstride, ld2, nf, ops, beta, scale, st);                          \
  }                                                                                                            \
  int gb_ct_rows_inv_##SUF(gbofdft_plan* p, const void* spec, int64_t fstride, int ld2, int nf, void* out,     \
                           int64_t ostride, double scale, const EvalDesc* ev, const void* rho, const void* vloc, \
                           void* pot, int calc_e, double* partials, int64_t* nblk, cudaStream_t st) {           \
    return gbct::ct_rows_inv<T>(p, spec, fstride, ld2, nf, out, ostride, scale, ev, rho, vloc, pot, calc_e,      \
                                partials, nblk, st);                                                            \
  }                                                                                                            \
  int gb_ct_cols_##SUF(gbofdft_plan* p, void* spec, int64_t fstride, int ld2, int nf, int axis, int dir,        \
                       double scale, const KerDesc* kd, cudaStream_t st) {                                      \
    if (kd) return gbct::ct_cols_t<T, -1, true>(p, spec, fstride, ld2, nf, axis, scale, kd, st);               \
    return dir < 0 ? gbct::ct_cols_t<T, -1, false>(p, spec, fstride, ld2, nf, axis, scale, nullptr, st)         \
                   : gbct::ct_cols_t<T, 1, false>(p, spec, fstride, ld2, nf, axis, scale, nullptr, st);         \
  }
