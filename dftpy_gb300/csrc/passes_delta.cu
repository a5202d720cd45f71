// Delta evaluation: the functional at a density rho close to a reference
// density rho_ref whose FP64 convolution results C_ref, potential and
// energies are known.  The convolutions are linear, so
//   C(rho) = C_ref + K * (g(rho) - g(rho_ref))
// for each derived field g (rho, sqrt(rho), rho^beta): the change of g is
// formed accurately (FP64 difference, power laws through log1p / expm1),
// rounded to FP32 and transformed by the FP32 plane pipeline.  FP32 rounding
// then perturbs C by ~1e-7 of the CHANGE instead of ~1e-16 of C, which for
// changes below ~1e-3 of the density is at the FP64 energy resolution of the
// functional.  The pointwise terms (TF, vW, WT, LDA, Hartree, local PP) are
// formed the same way, as FP32 changes added to the FP64 reference potential
// and energies (the FP64 pipe of this part is ~60x slower than FP32).
//
// Layouts are those of the FP32 plane pipeline: the row passes read and
// write plane-major spectra (passes_ct.cuh, plane_ct.cuh).
#include "passes_ct.cuh"

namespace gbct {

// g(a) - g(b) for the forward prologue op (OP_RHO, OP_SQRT, OP_POWB with
// exponent beta), both densities clamped at 1e-30 as the prologues clamp
// them (the square root clamps non-positive values only: values in
// (0, 1e-30) change it by < 1e-15).  Relative FP32 accuracy in the change:
//   sqrt(a) - sqrt(b) = (a - b) / (sqrt(a) + sqrt(b)),
//   a^p - b^p = b^p expm1(p log1p((a - b) / b)).
__device__ __forceinline__ float delta_op(int op, double a, double b, float beta) {
  if (op == OP_RHO) return (float)(a - b);
  const double ac = a < kZero ? kZero : a, bc = b < kZero ? kZero : b;
  const double d = ac - bc;
  const float bf = (float)bc;
  if (op == OP_SQRT) return (float)d / (sqrtf((float)ac) + sqrtf(bf));
  const float t = (float)d / bf;
  return powf(bf, beta) * expm1f(beta * log1pf(t));
}

struct DeltaRowsFwd {
  const double* rho;
  const double* ref;
  void* out;
  int64_t fstride;
  int nrows, nf;
  int op[GB_MAX_FIELDS];
  float beta;
  const void* tw;
};

// One CTA: RP row pairs, every field's change transformed along axis 2 (R2C)
// and written plane-major (as k_ct_rows_fwd<float, N, true>).
template <int N>
__global__ void __launch_bounds__(rows_threads_max<float, N>(), GB_CT_ROWS_MINB) k_delta_rows_fwd(DeltaRowsFwd a) {
  constexpr int RP = RowsCfg<float>::RP, TPL = Tpl<N>::value, NP = Pad<float, N>::NP, NH = N / 2 + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nl = a.nf * RP;
  cpx<float>* tw = reinterpret_cast<cpx<float>*>(smem_raw);
  cpx<float>* A = tw + N;
  cpx<float>* B = A + nl * NP;
  const int tid = threadIdx.x, l = tid / TPL, lane = tid % TPL;
  const int64_t base = (int64_t)blockIdx.x * 2 * RP;
  const cpx<float>* twg = reinterpret_cast<const cpx<float>*>(a.tw);
  for (int i = tid; i < N; i += blockDim.x) tw[i] = twg[i];
  for (int idx = tid; idx < 2 * RP * N; idx += blockDim.x) {
    const int rr = idx / N, j = idx % N;
    const int64_t row = base + rr;
    const bool ok = row < a.nrows;
    double x = 0.0, x0 = 0.0;
    if (ok) {
      x = __ldg(a.rho + row * N + j);
      x0 = __ldg(a.ref + row * N + j);
    }
#pragma unroll
    for (int f = 0; f < GB_MAX_FIELDS; ++f) {
      if (f >= a.nf) break;
      const float dv = ok ? delta_op(a.op[f], x, x0, a.beta) : 0.0f;
      // rows 2 pr and 2 pr + 1 share one complex line (real and imaginary part)
      reinterpret_cast<float*>(&A[sw<float, NP>(f * RP + (rr >> 1), j)])[rr & 1] = dv;
    }
  }
  __syncthreads();
  cpx<float>* res = fft<-1, float, N>(A, B, tw, l, lane, true);
  cpx<float>* out = reinterpret_cast<cpx<float>*>(a.out);
#pragma unroll
  for (int f = 0; f < GB_MAX_FIELDS; ++f) {
    if (f >= a.nf) break;
    cpx<float>* o = out + f * a.fstride;
    for (int idx = tid; idx < RP * NH; idx += blockDim.x) {
      const int l2 = idx % RP, k = idx / RP;
      const int line = f * RP + l2;
      const int64_t ra = base + 2 * l2, rb = ra + 1;
      if (ra >= a.nrows) continue;
      const cpx<float> Z = res[sw<float, NP>(line, k)];
      const cpx<float> Zc = res[sw<float, NP>(line, k == 0 ? 0 : N - k)];
      const int64_t ia = (int64_t)k * a.nrows + ra;
      o[ia] = cpx<float>{(Z.x + Zc.x) * 0.5f, (Z.y - Zc.y) * 0.5f};
      if (rb < a.nrows) o[ia + 1] = cpx<float>{(Z.y + Zc.y) * 0.5f, (Zc.x - Z.x) * 0.5f};
    }
  }
}

struct DeltaRowsInv {
  CtRowsInv c;          // spectra, geometry and twiddles of the FP32 inverse row pass
  EvalDesc ev;
  const double* rho;
  const double* rho_ref;
  const double* pot_ref;   // the reference evaluation's potential (fused terms)
  const double* vloc;
  const double* cref;   // field slot f at cref + f * cstride
  int64_t cstride;
  double* pot;
  double* partials;
  double tf_v, tf_e, vw_y, two_alpha, inv_two_alpha, wt_beta;
  int b56;
};

// The FP64 epilogue of one point (the same formulas and clamps as the FP64
// evaluation): potential and the six energy densities (before dV).
__device__ __forceinline__ void point64(const DeltaRowsInv& a, double rho, double w, double kc, double vh,
                                        double vl, double& pot, double (&e)[6]) {
  const EvalDesc& ev = a.ev;
  const bool pos = rho > kZero;
  double z3 = 0.0, z2 = 0.0;
  if (pos) { z3 = rcbrt_d(rho); z2 = rsqrt_d(rho); }
  pot = 0.0;
  for (int k = 0; k < 6; ++k) e[k] = 0.0;
  if (ev.tf) {
    pot += a.tf_v * (pos ? rho * z3 : cbrt(rho * rho));
    double r53;
    if (pos) r53 = rho * rho * z3;
    else { double r5 = rho * rho; r5 = r5 * rho; r5 = r5 * rho; r5 = r5 * rho; r53 = cbrt(r5); }
    e[0] = r53 * a.tf_e;
  }
  if (ev.vw) {
    const double inv_sq = pos ? z2 : (rho > 0.0 ? 1.0 / fmax(sqrt(rho), kZero) : 1e15);
    const double v = 0.5 * w * inv_sq;
    pot += v * a.vw_y;
    if (rho > 0.0) e[1] = rho * v * a.vw_y;
  }
  if (ev.wt) {
    double rb_over_rc;
    if (a.b56) {
      if (pos) rb_over_rc = rho * z3 * z3 * z2;
      else { const double rc = kZero; rb_over_rc = sqrt(rc) * cbrt(rc) / rc; }
    } else {
      const double rc = rho < kZero ? kZero : rho;
      rb_over_rc = pow(rc, a.wt_beta) / rc;
    }
    const double v = a.two_alpha * rb_over_rc * kc;
    pot += v;
    e[2] = v * rho * a.inv_two_alpha;
  }
  if (ev.xc) {
    double eps, vx;
    pz_lda_ct<double>(rho, eps, vx, true);
    pot += vx;
    e[3] = eps * rho;
  }
  if (ev.hartree) {
    pot += vh;
    e[4] = 0.5 * vh * rho;
  }
  if (ev.pp) {
    pot += vl;
    e[5] = vl * rho;
  }
}

// (b (1 + t))^p - b^p = bp expm1(p L) for bp = b^p, L = log1p(t): FP32 with
// the relative accuracy of FP32 in the change
__device__ __forceinline__ float pdelta(float bp, float L, float p) { return bp * expm1f(p * L); }

// Inverse row pass (C2R of the transformed changes) + the pointwise terms as
// changes against the reference evaluation: with L = log1p((rho - rho_ref)
// / rho_ref), every power law of rho changes by b^p expm1(p L); products
// change by d(uv) = du v + u0 dv; the PZ81 correlation (rs >= 1: N(s) /
// D(s)^2 and g / D(s), s = sqrt(rs)) by the exact rational-function
// differences in ds = s - s0, and (rs < 1) through d ln rs = -L / 3.  All of
// it in FP32, accurate to FP32 in the change, added to the reference
// potential in FP64; energies as FP32 per-thread sums of the changes.  Points
// with rho or rho_ref at the 1e-30 clamp, or with rs on different sides of 1
// (or within 1e-5 of it), take the FP64 epilogue at both densities.
template <int N, bool WANT_E>
__global__ void __launch_bounds__(rows_threads_max<float, N>(), GB_CT_ROWS_MINB) k_delta_rows_inv_eval(DeltaRowsInv a) {
  constexpr int RP = RowsCfg<float>::RP, NP = Pad<float, N>::NP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nl = a.c.nf * RP;
  cpx<float>* tw = reinterpret_cast<cpx<float>*>(smem_raw);
  cpx<float>* A = tw + N;
  cpx<float>* B = A + nl * NP;
  const int tid = threadIdx.x;
  const int64_t base = (int64_t)blockIdx.x * 2 * RP;
  const cpx<float>* twg = reinterpret_cast<const cpx<float>*>(a.c.tw);
  for (int i = tid; i < N; i += blockDim.x) tw[i] = twg[i];
  const cpx<float>* res = ct_rows_inv_lines<float, N, true>(a.c, base, tw, A, B);
  const EvalDesc& ev = a.ev;
  constexpr float cx = 0.98474502184269654115f;           // (3/pi)^(1/3)
  constexpr float RSC = 0.62035049089940001667f;          // (3/(4 pi))^(1/3)
  constexpr float la = 0.0311f, lb = -0.048f, lc = 0.0020f, ld = -0.0116f;
  constexpr float lg = -0.1423f, lb1 = 1.0529f, lb2 = 0.3334f;
  const float tf_v = (float)a.tf_v, tf_e = (float)a.tf_e, vw_y = (float)a.vw_y;
  const float two_alpha = (float)a.two_alpha, beta = (float)a.wt_beta;
  float es[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll 1
  for (int idx = tid; idx < 2 * RP * N; idx += blockDim.x) {
    const int rr = idx / N, j = idx % N;
    const int64_t row = base + rr;
    if (row >= a.c.nrows) continue;
    const int64_t gidx = row * N + j;
    const int pr = rr >> 1;
    const bool odd = rr & 1;
    const double rho = __ldg(a.rho + gidx), rho0 = __ldg(a.rho_ref + gidx);
    // transformed changes of the convolutions and their reference values
    float dw = 0.f, dkc = 0.f, dvh = 0.f;
    double w0 = 0.0, kc0 = 0.0, vh0 = 0.0;
    if (ev.vw) {
      const cpx<float> zz = res[sw<float, NP>(ev.slot_vw * RP + pr, j)];
      dw = odd ? zz.y : zz.x;
      w0 = __ldg(a.cref + ev.slot_vw * a.cstride + gidx);
    }
    if (ev.wt) {
      const cpx<float> zz = res[sw<float, NP>(ev.slot_wt * RP + pr, j)];
      dkc = odd ? zz.y : zz.x;
      kc0 = __ldg(a.cref + ev.slot_wt * a.cstride + gidx);
    }
    if (ev.hartree) {
      const cpx<float> zz = res[sw<float, NP>(ev.slot_h * RP + pr, j)];
      dvh = odd ? zz.y : zz.x;
      vh0 = __ldg(a.cref + ev.slot_h * a.cstride + gidx);
    }
    const double vl = ev.pp ? __ldg(a.vloc + gidx) : 0.0;
    // fast path: both densities above the clamp, LDA branch the same on both
    bool fast = rho > kZero && rho0 > kZero;
    const float r0 = (float)rho0, dr = (float)(rho - rho0);
    float L = 0.f, z3 = 0.f, z2 = 0.f, rs0 = 0.f, drs = 0.f;
    if (fast) {
      L = log1pf(dr / r0);
      z3 = rcbrtf(r0);
      z2 = rsqrtf(r0);
      rs0 = RSC * z3;
      drs = pdelta(rs0, L, -1.0f / 3.0f);
      if (ev.xc) {
        const float rs = rs0 + drs;
        if ((rs0 < 1.f) != (rs < 1.f) || fabsf(rs0 - 1.f) < 1e-5f || fabsf(rs - 1.f) < 1e-5f) fast = false;
      }
    }
    if (!fast) {
      double e1[6], e0[6], p1;
      point64(a, rho, w0 + (double)dw, kc0 + (double)dkc, vh0 + (double)dvh, vl, p1, e1);
      a.pot[gidx] = p1;
      if (WANT_E) {
        double p0;
        point64(a, rho0, w0, kc0, vh0, vl, p0, e0);
#pragma unroll
        for (int k = 0; k < 6; ++k) es[k] += (float)(e1[k] - e0[k]);
      }
      continue;
    }
    const float r = r0 + dr;                          // rho (FP32, for the small products)
    const float c13 = r0 * z3 * z3;                   // rho0^(1/3)
    float dpot = 0.f;
    if (ev.tf) {
      dpot += tf_v * pdelta(r0 * z3, L, 2.0f / 3.0f);               // rho^(2/3)
      if (WANT_E) es[0] += tf_e * pdelta(r0 * r0 * z3, L, 5.0f / 3.0f);
    }
    if (ev.vw) {
      // v = (1/2) w rho^(-1/2); e = (1/2) w rho^(1/2)
      const float wr = (float)w0;
      const float dzm = pdelta(z2, L, -0.5f);
      dpot += 0.5f * vw_y * (dw * (z2 + dzm) + wr * dzm);
      if (WANT_E) {
        const float q0 = r0 * z2, dq = pdelta(q0, L, 0.5f);
        es[1] += 0.5f * vw_y * (dw * (q0 + dq) + wr * dq);
      }
    }
    if (ev.wt) {
      // v = 2 alpha rho^(beta - 1) kc; e = rho^beta kc
      const float kr = (float)kc0;
      const float y0 = a.b56 ? z2 * c13 : powf(r0, beta - 1.0f);
      const float dy = pdelta(y0, L, beta - 1.0f);
      dpot += two_alpha * (dkc * (y0 + dy) + kr * dy);
      if (WANT_E) {
        const float q0 = r0 * y0, dq = pdelta(q0, L, beta);
        es[2] += dkc * (q0 + dq) + kr * dq;
      }
    }
    if (ev.xc) {
      // exchange: v = -cx rho^(1/3), e = -(3/4) cx rho^(4/3)
      dpot += -cx * pdelta(c13, L, 1.0f / 3.0f);
      float de = 0.f;
      if (WANT_E) de = -0.75f * cx * pdelta(r0 * c13, L, 4.0f / 3.0f);
      float dvc, dec, ec0;
      if (rs0 >= 1.f) {
        // vc = N / D^2, ec = g / D; N = g + a1 s + a2 s^2, D = 1 + b1 s + b2 s^2
        constexpr float a1 = 7.0f / 6.0f * lg * lb1, a2 = 4.0f / 3.0f * lg * lb2;
        const float s0 = sqrtf(rs0);
        const float ds = pdelta(s0, L, -1.0f / 6.0f);
        const float s = s0 + ds;
        const float N0 = lg + a1 * s0 + a2 * s0 * s0;
        const float D0 = 1.0f + lb1 * s0 + lb2 * s0 * s0;
        const float E = lb1 + lb2 * (s + s0);
        const float Ap = a1 + a2 * (s + s0);
        const float D = D0 + ds * E;
        dvc = ds * (Ap * D0 * D0 - N0 * E * (2.0f * D0 + ds * E)) / (D * D * D0 * D0);
        dec = -lg * ds * E / (D * D0);
        ec0 = lg / D0;
      } else {
        // vc = a ln rs + b - a/3 + (2/3) c rs ln rs + (2d - c)/3 rs
        const float dln = -L / 3.0f;
        const float ln0 = logf(rs0);
        const float drsln = (rs0 + drs) * dln + drs * ln0;
        dvc = la * dln + (2.0f / 3.0f) * lc * drsln + (2.0f * ld - lc) / 3.0f * drs;
        dec = la * dln + lc * drsln + ld * drs;
        ec0 = la * ln0 + lb + lc * rs0 * ln0 + ld * rs0;
      }
      dpot += dvc;
      if (WANT_E) es[3] += de + dec * r + ec0 * dr;
    }
    if (ev.hartree) {
      dpot += dvh;
      if (WANT_E) es[4] += 0.5f * (dvh * r + (float)vh0 * dr);
    }
    if (ev.pp && WANT_E) es[5] += (float)vl * dr;
    a.pot[gidx] = __ldg(a.pot_ref + gidx) + (double)dpot;
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

}  // namespace gbct

int gb_delta_supported(int n0, int n1, int n2) { return gb_plane_supported_f32(n0, n1, n2); }

int gb_delta_rows_fwd(gbofdft_plan* p, const double* rho, const double* rho_ref, void* spec, int64_t fstride, int nf,
                      const int* ops, double beta, cudaStream_t st) {
  using namespace gbct;
  int rc = 1;
  ct_dispatch(p->n[2], [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    constexpr int RP = RowsCfg<float>::RP, NP = Pad<float, N>::NP;
    DeltaRowsFwd a;
    memset(&a, 0, sizeof(a));
    a.rho = rho; a.ref = rho_ref; a.out = spec; a.fstride = fstride;
    a.nrows = p->n[0] * p->n[1]; a.nf = nf;
    for (int f = 0; f < GB_MAX_FIELDS; ++f) a.op[f] = f < nf ? ops[f] : OP_RHO;
    a.beta = (float)beta;
    a.tw = p->tw[2];
    const size_t sm = sizeof(cpx<float>) * (N + 2 * (size_t)nf * RP * NP);
    if ((rc = ct_smem(k_delta_rows_fwd<N>, sm))) return;
    const int nblk = (a.nrows + 2 * RP - 1) / (2 * RP);
    k_delta_rows_fwd<N><<<nblk, Tpl<N>::value * RP * nf, sm, st>>>(a);
    gb_count_launch();
    cudaError_t e = cudaGetLastError();
    rc = e == cudaSuccess ? 0 : gb_set_error(GBOFDFT_ERR_CUDA, "delta_rows_fwd: %s", cudaGetErrorString(e));
  });
  return rc == 1 ? gb_set_error(GBOFDFT_ERR_STATE, "delta evaluation: row length %d without specialisation", p->n[2])
                 : rc;
}

int gb_delta_rows_inv_eval(gbofdft_plan* p, const void* spec, int64_t fstride, int nf, const EvalDesc* ev,
                           const double* rho, const double* rho_ref, const double* pot_ref, const double* vloc,
                           const double* cref, int64_t cstride, double* pot, int calc_e, double* partials,
                           int64_t* nblk_out, cudaStream_t st) {
  using namespace gbct;
  int rc = 1;
  ct_dispatch(p->n[2], [&](auto nc) {
    constexpr int N = decltype(nc)::value;
    constexpr int RP = RowsCfg<float>::RP, NP = Pad<float, N>::NP;
    DeltaRowsInv a;
    memset(&a, 0, sizeof(a));
    a.c.in = spec; a.c.fstride = fstride; a.c.nrows = p->n[0] * p->n[1]; a.c.ld2 = 0; a.c.nf = nf;
    a.c.tw = p->tw[2];
    a.ev = *ev;
    a.rho = rho; a.rho_ref = rho_ref; a.pot_ref = pot_ref; a.vloc = vloc; a.cref = cref; a.cstride = cstride;
    a.pot = pot; a.partials = partials;
    const double ctf = 2.87123400018819181594;    // (3/10)(3 pi^2)^(2/3)
    a.tf_v = 5.0 / 3.0 * ctf * ev->tf_x;
    a.tf_e = ctf * ev->tf_x;
    a.vw_y = ev->vw_y;
    a.two_alpha = 2.0 * ev->wt_alpha;
    a.inv_two_alpha = ev->wt_alpha != 0.0 ? 1.0 / (2.0 * ev->wt_alpha) : 0.0;
    a.wt_beta = ev->wt_beta;
    a.b56 = fabs(ev->wt_beta - 5.0 / 6.0) < 1e-15;
    const int nblk = (a.c.nrows + 2 * RP - 1) / (2 * RP);
    if (nblk_out) *nblk_out = nblk;
    const size_t sm = sizeof(cpx<float>) * (N + 2 * (size_t)nf * RP * NP);
    if (calc_e) {
      if ((rc = ct_smem(k_delta_rows_inv_eval<N, true>, sm))) return;
      k_delta_rows_inv_eval<N, true><<<nblk, Tpl<N>::value * RP * nf, sm, st>>>(a);
    } else {
      if ((rc = ct_smem(k_delta_rows_inv_eval<N, false>, sm))) return;
      k_delta_rows_inv_eval<N, false><<<nblk, Tpl<N>::value * RP * nf, sm, st>>>(a);
    }
    gb_count_launch();
    cudaError_t e = cudaGetLastError();
    rc = e == cudaSuccess ? 0 : gb_set_error(GBOFDFT_ERR_CUDA, "delta_rows_inv_eval: %s", cudaGetErrorString(e));
  });
  return rc == 1 ? gb_set_error(GBOFDFT_ERR_STATE, "delta evaluation: row length %d without specialisation", p->n[2])
                 : rc;
}
