// Delta evaluation: the functional at a density rho close to a reference
// density rho_ref whose FP64 convolution results C_ref are known.  The
// convolutions are linear, so
//   C(rho) = C_ref + K * (g(rho) - g(rho_ref))
// for each derived field g (rho, sqrt(rho), rho^beta): the change of g is
// formed accurately (FP64 difference, power laws through log1p / expm1),
// rounded to FP32 and transformed by the FP32 plane pipeline.  FP32 rounding
// then perturbs C by ~1e-7 of the CHANGE instead of ~1e-16 of C, which for
// changes below ~1e-3 of the density is at the FP64 energy resolution of the
// functional.  The pointwise epilogue (TF, vW, WT, LDA, Hartree, local PP)
// runs in FP64 on C_ref + the transformed change, with the same formulas and
// clamps as the FP64 evaluation.
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
  const double* vloc;
  const double* cref;   // field slot f at cref + f * cstride
  int64_t cstride;
  double* pot;
  double* partials;
  double tf_v, tf_e, vw_y, two_alpha, inv_two_alpha, wt_beta;
  int b56;
};

// Inverse row pass (C2R of the transformed changes) + FP64 epilogue on
// C_ref + change; energies as per-CTA partial sums (GB_NE per CTA).
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
  double es[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll 1
  for (int idx = tid; idx < 2 * RP * N; idx += blockDim.x) {
    const int rr = idx / N, j = idx % N;
    const int64_t row = base + rr;
    if (row >= a.c.nrows) continue;
    const int64_t gidx = row * N + j;
    const int pr = rr >> 1;
    const bool odd = rr & 1;
    const double rho = __ldg(a.rho + gidx);
    auto conv = [&](int slot) {
      const cpx<float> zz = res[sw<float, NP>(slot * RP + pr, j)];
      return __ldg(a.cref + slot * a.cstride + gidx) + (double)(odd ? zz.y : zz.x);
    };
    const bool pos = rho > kZero;
    double z3 = 0.0, z2 = 0.0;
    if (pos) { z3 = rcbrt_d(rho); z2 = rsqrt_d(rho); }
    double pot = 0.0;
    if (ev.tf) {
      const double r23 = pos ? rho * z3 : cbrt(rho * rho);
      pot += a.tf_v * r23;
      if (WANT_E) {
        double r53;
        if (pos) r53 = rho * rho * z3;
        else { double r5 = rho * rho; r5 = r5 * rho; r5 = r5 * rho; r5 = r5 * rho; r53 = cbrt(r5); }
        es[0] += r53 * a.tf_e;
      }
    }
    if (ev.vw) {
      const double w = conv(ev.slot_vw);
      const double inv_sq = pos ? z2 : (rho > 0.0 ? 1.0 / fmax(sqrt(rho), kZero) : 1e15);
      const double v = 0.5 * w * inv_sq;
      pot += v * a.vw_y;
      if (WANT_E && rho > 0.0) es[1] += rho * v * a.vw_y;
    }
    if (ev.wt) {
      const double kc = conv(ev.slot_wt);
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
      if (WANT_E) es[2] += v * rho * a.inv_two_alpha;
    }
    if (ev.xc) {
      double eps, vx;
      pz_lda_ct<double>(rho, eps, vx, WANT_E);
      pot += vx;
      if (WANT_E) es[3] += eps * rho;
    }
    if (ev.hartree) {
      const double vh = conv(ev.slot_h);
      pot += vh;
      if (WANT_E) es[4] += 0.5 * vh * rho;
    }
    if (ev.pp) {
      const double vl = __ldg(a.vloc + gidx);
      pot += vl;
      if (WANT_E) es[5] += vl * rho;
    }
    a.pot[gidx] = pot;
  }
  if constexpr (!WANT_E) return;
  __shared__ double red[32][6];
  const int lane32 = tid & 31, warp = tid >> 5;
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const double v = warp_sum(es[c]);
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
                           const double* rho, const double* vloc, const double* cref, int64_t cstride, double* pot,
                           int calc_e, double* partials, int64_t* nblk_out, cudaStream_t st) {
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
    a.rho = rho; a.vloc = vloc; a.cref = cref; a.cstride = cstride; a.pot = pot; a.partials = partials;
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
