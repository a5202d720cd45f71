// Truncated-Newton direct density optimisation on the device.
//
// Host control flow mirrors dftpy's Optimization.optimize_rho with method
// "TN" (src/dftpy/optimization/optimization.py:91-147 get_direction_TN,
// :204-225 OrthogonalNormalization, :227-279 ValueAndDerivative,
// :281-520 optimize_rho, :522-535 check_converge) and the More-Thuente line
// search of LineSearchDcsrch2 (math_utils.py:76-106).  Every field-sized
// operation is a fused elementwise kernel whose dot products finish in the
// same launch (the last CTA to arrive sums the per-CTA partials in a fixed
// order with compensated FP64 arithmetic), so results are deterministic.
// Scalars cross to the host once per evaluation (one small D2H copy).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <mutex>
#include <vector>

#include "dcsrch.h"
#include "plan.h"

namespace {

constexpr int kRedBlocks = 1216;  // 8 x 152 SMs
constexpr int kRedThreads = 256;
constexpr int kMaxVals = 4;

// scalar slots in the workspace scalar array
enum {
  S_A = 0, S_B = 1, S_C = 2, S_D = 3,   // generic reduction outputs
  S_PAP = 4, S_R1 = 8,                  // TN inner loop
  S_ALPHA = 12,                         // CG step r0 / pAp in the loop precision (0 if pAp < 0)
  S_RZ = 14, S_RZN = 15,                // preconditioned CG: r.z (current, new)
  S_BETA = 24,                          // preconditioned CG: beta in the loop precision
  S_EN = 16,                            // energies (GB_NE)
  S_DR = 28,                            // delta evaluation: ||rho - rho_ref||^2, ||rho_ref||^2
  S_COUNT = 64
};

struct Ws {
  void* f[16];
  double* partials;  // kRedBlocks * kMaxVals
  double* sc;        // S_COUNT
  unsigned* counter;
};

enum { F_PHI = 0, F_RHO, F_POT, F_RES0, F_P, F_CGR, F_CGP, F_AP, F_DIR, F_BEST, F_PHI1, F_POT1, F_TMP,
       F_Z, F_PC, F_NF };   // F_Z, F_PC: preconditioned residual and preconditioner (half spectrum)

struct NoPost {
  __device__ void operator()() const {}
};

// Grid reduction epilogue: per-CTA partials, then the last CTA to arrive sums
// them in a fixed order into out[0..NV) and runs post() (scalars derived from
// the sums, computed once instead of per element).
template <typename ACC>
__device__ __forceinline__ ACC warp_sum_acc(ACC v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// acc: per-thread sums in the field precision ACC; the warp sums are formed in
// ACC (a few dozen elements each) and everything above them in FP64.
template <int NV, typename ACC, typename P = NoPost>
__device__ __forceinline__ void reduce_finalize(const ACC (&acc)[NV], double* partials, double* out,
                                                unsigned* counter, P post = P()) {
  __shared__ double red[kRedThreads / 32][NV];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const ACC v = warp_sum_acc(acc[k]);
    if (lane == 0) red[warp][k] = (double)v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int w = 0; w < kRedThreads / 32; ++w) s += red[w][k];
      partials[blockIdx.x * NV + k] = s;
    }
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    KSum s;
    s.init();
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s.add(__ldcg(partials + b * NV + k));
    double v = warp_sum(s.value());
    if (lane == 0) red[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      KSum s;
      s.init();
      for (int w = 0; w < kRedThreads / 32; ++w) s.add(red[w][k]);
      out[k] = s.value();
    }
    *counter = 0u;
    post();
  }
}

// f(i, ACC* contributions[NV]) for i in [0, n).  Each thread accumulates its
// elements in the field precision ACC (a handful per thread); the per-thread
// sums are combined in FP64 (compensated at the CTA and grid level).
template <int NV, typename ACC, typename F, typename P = NoPost>
__global__ void __launch_bounds__(kRedThreads) k_map_reduce(int64_t n, F f, double* partials, double* out,
                                                           unsigned* counter, P post = P()) {
  constexpr int NA = NV > 0 ? NV : 1;
  ACC acc[NA];
#pragma unroll
  for (int k = 0; k < NA; ++k) acc[k] = (ACC)0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    ACC c[NA];
    f(i, c);
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] += c[k];
  }
  if constexpr (NV > 0) reduce_finalize<NV, ACC>(acc, partials, out, counter, post);
}

template <int NV, typename ACC, typename F, typename P = NoPost>
int launch_mr(const Ws& w, int64_t n, F f, int slot, cudaStream_t st, P post = P()) {
  int nb = (int)((n + kRedThreads * 4 - 1) / (kRedThreads * 4));
  if (nb > kRedBlocks) nb = kRedBlocks;
  if (nb < 1) nb = 1;
  k_map_reduce<NV, ACC><<<nb, kRedThreads, 0, st>>>(n, f, w.partials, w.sc + slot, w.counter, post);
  GB_CHECK_LAUNCH();
  return 0;
}

}  // namespace

// Fields of the Hessian-precision inner loop (split mode only)
enum { H_PHI = 0, H_RB, H_POT, H_CGR, H_CGP, H_AP, H_DIR, H_BEST, H_PHI1, H_POT1, H_TMP, H_Z, H_PC, H_NF };

struct TnState {
  gbofdft_plan* p;
  const gbofdft_functional* fn;
  Ws w;
  cudaStream_t st;
  double host[S_COUNT];
  int n_ev, n_v, n_hv;
  int n_sync;
  double t_sync;  // host seconds blocked in stream synchronisation
  double t_start;
  // split mode: Hessian products in another precision (hp != nullptr)
  gbofdft_plan* hp;
  const gbofdft_functional* hfn;
  void* hf[H_NF];
  bool verbose;   // GBOFDFT_TN_VERBOSE=1: per-iteration trace on stderr
  bool time_evals;  // CUDA-event timing of the FP32 potential-only evaluations
  // delta evaluations of the FP64 functional (split mode): state, rebase
  // threshold, whether this solve has made a reference yet
  gbofdft_delta* delta;
  double delta_rtol;
  bool delta_ref;
  int n_delta;
};

// CUDA-event pairs around timed evaluations (per host thread, reused across
// solves); completed pairs are read at the next stream synchronisation.
struct EvTimer {
  static constexpr int K = 64;
  cudaEvent_t a[K], b[K];
  bool init = false;
  int n = 0;
  double ms = 0.0;
  int count = 0;
};
static thread_local EvTimer g_evt;

static void evt_drain() {
  for (int i = 0; i < g_evt.n; ++i) {
    float t = 0.0f;
    if (cudaEventSynchronize(g_evt.b[i]) == cudaSuccess && cudaEventElapsedTime(&t, g_evt.a[i], g_evt.b[i]) == cudaSuccess) {
      g_evt.ms += t;
      ++g_evt.count;
    }
  }
  g_evt.n = 0;
}

static int evt_begin(cudaStream_t st) {
  if (!g_evt.init) {
    for (int i = 0; i < EvTimer::K; ++i) {
      GB_CUDA(cudaEventCreate(&g_evt.a[i]));
      GB_CUDA(cudaEventCreate(&g_evt.b[i]));
    }
    g_evt.init = true;
  }
  if (g_evt.n == EvTimer::K) evt_drain();
  GB_CUDA(cudaEventRecord(g_evt.a[g_evt.n], st));
  return 0;
}

static int evt_end(cudaStream_t st) {
  GB_CUDA(cudaEventRecord(g_evt.b[g_evt.n], st));
  ++g_evt.n;
  return 0;
}

// gbofdft_eval, with the FP32 potential-only calls timed when requested
static int tn_eval(TnState& s, gbofdft_plan* plan, const gbofdft_functional* fn, const void* rho, void* pot,
                   double* en, int calc) {
  const bool t = s.time_evals && plan->prec == GBOFDFT_F32 && !(calc & GBOFDFT_CALC_E);
  int rc;
  if (t && (rc = evt_begin(s.st))) return rc;
  rc = gbofdft_eval(plan, rho, fn, pot, en, calc, s.st);
  if (!rc && t) rc = evt_end(s.st);
  return rc;
}

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Page-locked landing buffers of the scalar read-back, one per host thread
// while it lives (a copy into pageable memory is staged by the driver and
// costs more than the copy itself on every one of a solve's ~70
// synchronisations).  Buffers of exited threads go back to a pool, so
// short-lived worker threads do not allocate page-locked memory each time.
static std::mutex g_pin_mu;
static std::vector<double*> g_pin_free;

struct PinnedScalars {
  double* p = nullptr;
  ~PinnedScalars() {
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_pin_mu);
    g_pin_free.push_back(p);
  }
};
static thread_local PinnedScalars g_pinned;

static int pinned_scalars(double** out) {
  if (!g_pinned.p) {
    {
      std::lock_guard<std::mutex> lk(g_pin_mu);
      if (!g_pin_free.empty()) {
        g_pinned.p = g_pin_free.back();
        g_pin_free.pop_back();
      }
    }
    if (!g_pinned.p) {
      void* ptr = nullptr;
      GB_CUDA(cudaMallocHost(&ptr, sizeof(double) * S_COUNT));
      g_pinned.p = reinterpret_cast<double*>(ptr);
    }
  }
  *out = g_pinned.p;
  return 0;
}

static int ts_sync(TnState& s) {
  const double t0 = now_s();
  double* pin = nullptr;
  int rc = pinned_scalars(&pin);
  if (rc) return rc;
  GB_CUDA(cudaMemcpyAsync(pin, s.w.sc, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, s.st));
  GB_CUDA(cudaStreamSynchronize(s.st));
  memcpy(s.host, pin, sizeof(double) * S_COUNT);
  s.t_sync += now_s() - t0;
  ++s.n_sync;
  if (s.time_evals) evt_drain();
  return 0;
}

static int ts_eval(TnState& s, const void* rho, void* pot, bool want_e) {
  if (want_e) ++s.n_ev; else ++s.n_v;
  double* en = want_e ? s.w.sc + S_EN : nullptr;
  const int calc = GBOFDFT_CALC_V | (want_e ? GBOFDFT_CALC_E : 0);
  if (!s.delta) return tn_eval(s, s.p, s.fn, rho, pot, en, calc);
  // delta evaluation against the solve's reference density unless rho has
  // moved more than delta_rtol from it (then a full evaluation rebases)
  bool rebase = !s.delta_ref;
  if (!rebase) {
    const double* r = reinterpret_cast<const double*>(rho);
    const double* r0 = gb_delta_ref(s.delta);
    int rc = launch_mr<2, double>(s.w, s.p->N, [=] __device__(int64_t i, double* c) {
      const double d = r[i] - r0[i];
      c[0] = d * d;
      c[1] = r0[i] * r0[i];
    }, S_DR, s.st);
    if (rc || (rc = ts_sync(s))) return rc;
    rebase = !(s.host[S_DR] <= s.delta_rtol * s.delta_rtol * s.host[S_DR + 1]);
  }
  if (!rebase) ++s.n_delta;
  const int rc = gbofdft_eval_delta(s.delta, rho, s.fn, s.hfn, pot, en, calc, rebase ? 1 : 0, s.st);
  if (!rc) s.delta_ref = true;
  return rc;
}

template <typename T>
static T* F(TnState& s, int i) { return reinterpret_cast<T*>(s.w.f[i]); }

// Field pointers of the TN inner loop (get_direction_TN) in precision TH.
// rb is the finite-difference base (V(phi) - mu) phi evaluated in TH; the
// right-hand side is the outer residual.  In the single-precision-pair
// ("split") mode the inner loop runs on TH copies; otherwise its fields are
// the outer ones and rb is the outer residual itself.
template <typename TH>
struct DirFields {
  TH *phi, *rb, *cgr, *cgp, *ap, *dir, *best, *phi1, *rho1, *pot1;
  TH* z;          // preconditioned residual (PCG only)
  const TH* pc;   // preconditioner on the half spectrum; nullptr: plain CG (the reference's)
};

// TN direction (optimization.py:91-147) with Hessian products
//   A p = ((V(phi + eps p) - mu)(phi + eps p) - rb) / eps
// evaluated by `plan`/`fn` in precision TH; CG on A dir = -res0 (res0 in T).
// The direction is left in F_P (precision T).
template <typename T, typename TH>
static int tn_direction(TnState& s, gbofdft_plan* plan, const gbofdft_functional* fn, const DirFields<TH>& d,
                        double mu, double eps_fixed, double eps_rel, int maxfun, double cg_rtol) {
  const int64_t N = s.p->N;
  cudaStream_t st = s.st;
  const Ws& w = s.w;
  int rc;
  const T* res0 = F<T>(s, F_RES0);
  const bool split = (void*)d.phi != s.w.f[F_PHI];
  TH* cgr = d.cgr;
  TH* cgp = d.cgp;
  TH* dir = d.dir;
  TH* rb = d.rb;
  const TH muH = (TH)mu;
  if (split) {
    // TH copy of phi and the finite-difference base at it
    const T* phiT = F<T>(s, F_PHI);
    TH* ph = d.phi;
    TH* rho1 = d.rho1;
    rc = launch_mr<0, TH>(w, N, [=] __device__(int64_t i, TH* c) {
      const TH v = (TH)phiT[i];
      ph[i] = v;
      rho1[i] = v * v;
    }, S_A, st);
    if (rc) return rc;
    ++s.n_hv;
    if ((rc = tn_eval(s, plan, fn, rho1, d.pot1, nullptr, GBOFDFT_CALC_V))) return rc;
    TH* pot1 = d.pot1;
    rc = launch_mr<0, TH>(w, N, [=] __device__(int64_t i, TH* c) { rb[i] = (pot1[i] - muH) * ph[i]; }, S_A, st);
    if (rc) return rc;
  }
  {
    TH* phic = d.phi;
    rc = launch_mr<2, TH>(w, N, [=] __device__(int64_t i, TH* c) {
      const TH r = -(TH)res0[i];
      cgr[i] = r;
      cgp[i] = r;
      dir[i] = (TH)0;
      c[0] = r * r;
      c[1] = phic[i] * phic[i];
    }, S_A, st);
    if (rc) return rc;
  }
  const bool pcg = d.pc != nullptr;
  double* scw0 = w.sc;
  if (pcg) {
    // z = P r, p = z, rz = r.z
    if ((rc = gbofdft_convolve(plan, cgr, d.z, GBOFDFT_KER_ARRAY, d.pc, 1.0, st))) return rc;
    TH* zz = d.z;
    rc = launch_mr<1, TH>(w, N, [=] __device__(int64_t i, TH* c) {
      const TH zi = zz[i];
      cgp[i] = zi;
      c[0] = cgr[i] * zi;
    }, S_RZ, st);
    if (rc) return rc;
  }
  if ((rc = ts_sync(s))) return rc;
  const double rz0 = s.host[S_RZ];
  // stopping tests on r.r (the reference's), or on r.z with the preconditioner
  double r0Norm = pcg ? rz0 : s.host[S_A];
  const double r0_first = r0Norm;
  int jend = 0;
  const double rr0 = s.host[S_A];
  const double epsi = eps_rel > 0 && rr0 > 0 ? eps_rel * sqrt(s.host[S_B] / rr0) : eps_fixed;
  const double rConv = r0Norm * cg_rtol;
  double rmin = 1e10;          // min(rLists) with rLists = [1e10]
  double prev_min = 1e10;
  bool use_best = false;
  bool have_best = false;      // Best starts as the zero direction
  double beta = 0.0;
  for (int j = 0; j < maxfun; ++j) {
    jend = j + 1;
    TH* phi = d.phi;
    TH* phi1 = d.phi1;
    TH* rho1 = d.rho1;
    const TH eT = (TH)epsi, bT = (TH)beta;
    const bool first = (j == 0);
    if (!pcg) {
      rc = launch_mr<0, TH>(w, N, [=] __device__(int64_t i, TH* c) {
        TH pv = cgp[i];
        if (!first) { pv = cgr[i] + bT * pv; cgp[i] = pv; }
        const TH p1 = phi[i] + eT * pv;
        phi1[i] = p1;
        rho1[i] = p1 * p1;
      }, S_A, st);
    } else {
      const TH* zz = d.z;
      const TH* bd = reinterpret_cast<const TH*>(w.sc + S_BETA);
      rc = launch_mr<0, TH>(w, N, [=] __device__(int64_t i, TH* c) {
        TH pv = cgp[i];
        if (!first) { pv = zz[i] + *bd * pv; cgp[i] = pv; }
        const TH p1 = phi[i] + eT * pv;
        phi1[i] = p1;
        rho1[i] = p1 * p1;
      }, S_A, st);
    }
    if (rc) return rc;
    TH* pot1 = d.pot1;
    if (split) ++s.n_hv; else ++s.n_v;
    if ((rc = tn_eval(s, plan, fn, rho1, pot1, nullptr, GBOFDFT_CALC_V))) return rc;
    TH* ap = d.ap;
    const TH inv_e = (TH)(1.0 / epsi);
    double* scw = w.sc;
    const double r0c = r0Norm;
    // alpha = r0 / pAp, once, by the last CTA of the pAp reduction
    const bool pcgc = pcg;
    auto alpha_post = [=] __device__() {
      const double pap = scw[S_PAP];
      const double num = pcgc ? scw[S_RZ] : r0c;
      TH* al = reinterpret_cast<TH*>(scw + S_ALPHA);
      al[0] = pap < 0.0 ? (TH)0 : (TH)(num / pap);
      al[1] = pap < 0.0 ? (TH)1 : (TH)0;   // negative curvature: no update
    };
    rc = launch_mr<1, TH>(w, N, [=] __device__(int64_t i, TH* c) {
      const TH a = ((pot1[i] - muH) * phi1[i] - rb[i]) * inv_e;
      ap[i] = a;
      c[0] = cgp[i] * a;
    }, S_PAP, st, alpha_post);
    if (rc) return rc;
    const TH* alp = reinterpret_cast<const TH*>(w.sc + S_ALPHA);
    rc = launch_mr<1, TH>(w, N, [=] __device__(int64_t i, TH* c) {
      if (alp[1] != (TH)0) { c[0] = (TH)0; return; }
      const TH alpha = alp[0];
      dir[i] += alpha * cgp[i];
      const TH r = cgr[i] - alpha * ap[i];
      cgr[i] = r;
      c[0] = r * r;
    }, S_R1, st);
    if (rc) return rc;
    if (pcg) {
      // z = P r; beta = r.z / previous r.z (device scalars)
      if ((rc = gbofdft_convolve(plan, cgr, d.z, GBOFDFT_KER_ARRAY, d.pc, 1.0, st))) return rc;
      TH* zz = d.z;
      auto beta_post = [=] __device__() {
        const double rzn = scw0[S_RZN], rzo = scw0[S_RZ];
        *reinterpret_cast<TH*>(scw0 + S_BETA) = rzo != 0.0 ? (TH)(rzn / rzo) : (TH)0;
        scw0[S_RZ] = rzn;
      };
      rc = launch_mr<1, TH>(w, N, [=] __device__(int64_t i, TH* c) { c[0] = cgr[i] * zz[i]; }, S_RZN, st,
                            beta_post);
      if (rc) return rc;
    }
    if ((rc = ts_sync(s))) return rc;
    const double pAp = s.host[S_PAP];
    if (pAp < 0.0) {
      if (j == 0) {
        // direction = r0Norm / pAp * p  (r.z / pAp with the preconditioner)
        const TH sc = (TH)((pcg ? rz0 : r0Norm) / pAp);
        rc = launch_mr<0, TH>(w, N, [=] __device__(int64_t i, TH* c) { dir[i] = sc * cgp[i]; }, S_A, st);
        if (rc) return rc;
      }
      break;
    }
    const double r1Norm = pcg ? s.host[S_RZ] : s.host[S_R1];
    if (r1Norm < rmin) {
      GB_CUDA(cudaMemcpyAsync(d.best, dir, sizeof(TH) * N, cudaMemcpyDeviceToDevice, st));
      have_best = true;
    }
    prev_min = rmin;
    if (r1Norm < rmin) rmin = r1Norm;
    if (r1Norm < rConv) break;
    if (r1Norm > 1000.0 * prev_min) { use_best = true; break; }
    if (j > 10 && fabs(r0Norm - r1Norm) < 0.1 * r0Norm) { use_best = true; break; }
    beta = r1Norm / r0Norm;
    r0Norm = r1Norm;
  }
  if (s.verbose)
    fprintf(stderr, "[gbofdft tn]   cg %s steps %d r0 %.3e rmin %.3e eps %.3e best %d\n", split ? "split" : "same",
            jend, r0_first, rmin, epsi, (int)(use_best && have_best));
  // Best aliases the direction itself until the first improvement copies it
  const TH* src = (use_best && have_best) ? d.best : dir;
  T* p = F<T>(s, F_P);
  rc = launch_mr<0, T>(w, N, [=] __device__(int64_t i, T* c) { p[i] = (T)src[i]; }, S_A, st);
  return rc;
}

template <typename T>
static int tn_run(TnState& s, void* rho_io, const gbofdft_tn_options& o, gbofdft_tn_result* res) {
  const int64_t N = s.p->N;
  const double dV = s.p->dV;
  cudaStream_t st = s.st;
  const Ws& w = s.w;
  int rc;
  T* rio = reinterpret_cast<T*>(rho_io);
  // ---- initial phi (optimization.py:305-316) --------------------------------
  {
    T* phi = F<T>(s, F_PHI);
    rc = launch_mr<2, T>(w, N, [=] __device__(int64_t i, T* c) {
      const T r = rio[i];
      const T ph = r > (T)0 ? sqrt(r) : (sizeof(T) == 8 ? (T)1e-300 : (T)1e-30);
      phi[i] = ph;
      c[0] = r;
      c[1] = ph * ph;
    }, S_A, st);
    if (rc) return rc;
    if ((rc = ts_sync(s))) return rc;
    // a density with NaN/Inf values or without electrons has no solution:
    // report it instead of iterating on it (the sums are on the host already)
    if (!isfinite(s.host[S_A]) || !isfinite(s.host[S_B]) || !(s.host[S_A] > 0.0) || !(s.host[S_B] > 0.0))
      return gb_set_error(GBOFDFT_ERR_NUMERIC,
                          "optimize_tn: the initial density has non-finite values or no electrons "
                          "(sum rho = %g, sum phi^2 = %g)", s.host[S_A], s.host[S_B]);
    const T fac = (T)sqrt(s.host[S_A] / s.host[S_B]);
    if (o.precond) {
      // preconditioner of the uniform gas at the mean density
      const double rho0 = s.host[S_A] / (double)N;
      if ((rc = gb_build_precond(s.p, rho0, s.w.f[F_PC], st))) return rc;
      if (s.hp && (rc = gb_build_precond(s.hp, rho0, s.hf[H_PC], st))) return rc;
    }
    T* rho = F<T>(s, F_RHO);
    rc = launch_mr<0, T>(w, N, [=] __device__(int64_t i, T* c) {
      const T ph = phi[i] * fac;
      phi[i] = ph;
      rho[i] = ph * ph;
    }, S_A, st);
    if (rc) return rc;
  }
  if ((rc = ts_eval(s, F<T>(s, F_RHO), F<T>(s, F_POT), true))) return rc;
  // mu and residual
  auto mu_residual = [&](double& mu, double& energy, double& resN) -> int {
    T* phi = F<T>(s, F_PHI);
    T* pot = F<T>(s, F_POT);
    T* rho = F<T>(s, F_RHO);
    int r = launch_mr<2, T>(w, N, [=] __device__(int64_t i, T* c) {
      const T ph = phi[i];
      const T rr = ph * ph;
      rho[i] = rr;
      c[0] = pot[i] * rr;
      c[1] = rr;
    }, S_A, st);
    if (r) return r;
    if ((r = ts_sync(s))) return r;
    energy = s.host[S_EN + GB_E_TOTAL];
    mu = (s.host[S_A] * dV) / (s.host[S_B] * dV);
    if (!isfinite(energy) || !isfinite(mu))
      return gb_set_error(GBOFDFT_ERR_NUMERIC, "optimize_tn: non-finite energy (%g) or chemical potential (%g)",
                          energy, mu);
    const T muT = (T)mu;
    T* res0 = F<T>(s, F_RES0);
    r = launch_mr<1, T>(w, N, [=] __device__(int64_t i, T* c) {
      const T v = (pot[i] - muT) * phi[i];
      res0[i] = v;
      c[0] = v * v;
    }, S_C, st);
    resN = 0.0;
    return r;
  };
  double mu, energy, resN;
  if ((rc = mu_residual(mu, energy, resN))) return rc;
  if (o.res0_max > 0.0) {
    // the caller's check of its starting density: a residual above res0_max
    // returns at once (rho_io untouched), converged = 3
    if ((rc = ts_sync(s))) return rc;
    const double r0 = sqrt(s.host[S_C] * dV);
    if (!(r0 <= o.res0_max)) {
      res->energy = energy;
      res->mu = mu;
      res->converged = 3;
      res->n_iter = 0;
      res->n_eval_ev = s.n_ev;
      res->n_eval_v = s.n_v;
      res->n_eval_hess = s.n_hv;
      res->n_history = 0;
      res->n_sync = s.n_sync;
      res->t_sync = s.t_sync;
      res->t_total = now_s() - s.t_start;
      res->n_eval_delta = s.n_delta;
      for (int k = 0; k < GBOFDFT_NE; ++k) res->energies[k] = s.host[S_EN + k];
      return 0;
    }
  }
  const int hist_cap = res->history_cap;
  int nh = 0;
  double ehist_last[64];
  int nhist = 0;
  auto push_hist = [&](double e) {
    if (res->history && nh < hist_cap) res->history[nh++] = e;
    if (nhist < 64) ehist_last[nhist++] = e;
    else { memmove(ehist_last, ehist_last + 1, sizeof(double) * 63); ehist_last[63] = e; }
  };
  push_hist(energy);
  double theta = 0.1;
  int converged = 1;
  int it;
  // eps > 0: fixed step (the reference's 1e-9); eps < 0: |eps| relative to
  // ||phi|| / ||residual|| of each TN direction (single precision needs a step
  // the perturbation phi + eps p can resolve); eps == 0: 1e-9
  const double eps_fixed = o.eps > 0 ? o.eps : 1e-9;
  const double eps_rel = o.eps < 0 ? -o.eps : 0.0;
  for (it = 1; it < o.maxiter; ++it) {
    // ---- TN direction (optimization.py:91-147) -----------------------------
    bool done_dir = false;
    if constexpr (sizeof(T) == 8) {
      if (s.hp) {
        // split: FP64 residual, Hessian products in single precision
        DirFields<float> d;
        float** hf = reinterpret_cast<float**>(s.hf);
        d.phi = hf[H_PHI]; d.rb = hf[H_RB]; d.cgr = hf[H_CGR]; d.cgp = hf[H_CGP]; d.ap = hf[H_AP];
        d.dir = hf[H_DIR]; d.best = hf[H_BEST]; d.phi1 = hf[H_PHI1]; d.rho1 = hf[H_TMP]; d.pot1 = hf[H_POT1];
        d.z = hf[H_Z]; d.pc = o.precond ? hf[H_PC] : nullptr;
        if ((rc = tn_direction<T, float>(s, s.hp, s.hfn, d, mu, eps_fixed, eps_rel, o.maxfun, o.cg_rtol))) return rc;
        done_dir = true;
      }
    }
    if (!done_dir) {
      DirFields<T> d;
      d.phi = F<T>(s, F_PHI); d.rb = F<T>(s, F_RES0); d.cgr = F<T>(s, F_CGR); d.cgp = F<T>(s, F_CGP);
      d.ap = F<T>(s, F_AP); d.dir = F<T>(s, F_DIR); d.best = F<T>(s, F_BEST); d.phi1 = F<T>(s, F_PHI1);
      d.rho1 = F<T>(s, F_TMP); d.pot1 = F<T>(s, F_POT1);
      d.z = F<T>(s, F_Z); d.pc = o.precond ? F<T>(s, F_PC) : nullptr;
      if ((rc = tn_direction<T, T>(s, s.p, s.fn, d, mu, eps_fixed, eps_rel, o.maxfun, o.cg_rtol))) return rc;
    }
    // ---- OrthogonalNormalization (optimization.py:204-225) -----------------
    double theta0 = 0.0, d0 = 0.0;
    auto orthonormalize = [&]() -> int {
      T* phi = F<T>(s, F_PHI);
      T* p = F<T>(s, F_P);
      T* pot = F<T>(s, F_POT);
      int r = launch_mr<2, T>(w, N, [=] __device__(int64_t i, T* c) {
        c[0] = phi[i] * phi[i];
        c[1] = p[i] * phi[i];
      }, S_A, st);
      if (r) return r;
      if ((r = ts_sync(s))) return r;
      const double Ne = s.host[S_A] * dV;
      const T fac = (T)(s.host[S_B] * dV / Ne);
      r = launch_mr<1, T>(w, N, [=] __device__(int64_t i, T* c) {
        const T v = p[i] - fac * phi[i];
        p[i] = v;
        c[0] = v * v;
      }, S_C, st);
      if (r) return r;
      if ((r = ts_sync(s))) return r;
      const double pNorm = s.host[S_C] * dV;
      theta0 = sqrt(pNorm / Ne);
      const T sc = (T)sqrt(Ne / pNorm);
      r = launch_mr<1, T>(w, N, [=] __device__(int64_t i, T* c) {
        const T v = p[i] * sc;
        p[i] = v;
        c[0] = pot[i] * phi[i] * v;
      }, S_D, st);
      if (r) return r;
      if ((r = ts_sync(s))) return r;
      d0 = s.host[S_D];
      return 0;
    };
    if ((rc = orthonormalize())) return rc;
    if (d0 * 2.0 > 0.0) {  // "Change to steepest descent" (optimization.py:371-380)
      T* p = F<T>(s, F_P);
      T* res0 = F<T>(s, F_RES0);
      rc = launch_mr<0, T>(w, N, [=] __device__(int64_t i, T* c) { p[i] = -res0[i]; }, S_A, st);
      if (rc) return rc;
      if ((rc = orthonormalize())) return rc;
    }
    theta = fmin(theta0, theta);
    // quadratic-model decrease of a Newton step along p: |g| theta0 / 2 with
    // g = dE/dtheta at 0.  Below pred_stop the step cannot change the energy
    // by more than the requested resolution: stop converged.
    const double pred = fabs(d0 * dV) * theta0;
    if (o.pred_stop > 0.0 && pred < o.pred_stop) {
      converged = 0;
      break;
    }
    // Newton step whose model decrease is below the energy resolution: the
    // line search cannot judge it from energies; take it as it is.
    const bool newton_only = o.eres > 0.0 && pred < o.eres * fmax(1.0, fabs(energy));
    // ---- line search over the rotation angle (ValueAndDerivative) ----------
    Dcsrch ls;
    dcs_init(ls, o.c1, o.c2, o.xtol, 0.0, 3.14159265358979323846);
    int task = DCS_START;
    double stp = theta, fval = energy, gval = 2.0 * d0 * dV;
    bool accepted = false;
    int nls;
    if (newton_only) stp = theta0;
    for (nls = 0; nls < o.maxls; ++nls) {
      if (!newton_only) {
        task = dcs_step(ls, stp, fval, gval, task);
        if (task != DCS_FG) break;
      }
      T* phi = F<T>(s, F_PHI);
      T* p = F<T>(s, F_P);
      T* phi1 = F<T>(s, F_PHI1);
      T* rho1 = F<T>(s, F_TMP);
      const T ct = (T)cos(stp), sn = (T)sin(stp);
      rc = launch_mr<0, T>(w, N, [=] __device__(int64_t i, T* c) {
        const T v = phi[i] * ct + p[i] * sn;
        phi1[i] = v;
        rho1[i] = v * v;
      }, S_A, st);
      if (rc) return rc;
      T* pot1 = F<T>(s, F_POT1);
      if ((rc = ts_eval(s, rho1, pot1, true))) return rc;
      rc = launch_mr<1, T>(w, N, [=] __device__(int64_t i, T* c) {
        const T p2 = p[i] * ct - phi[i] * sn;
        c[0] = pot1[i] * phi1[i] * p2;
      }, S_A, st);
      if (rc) return rc;
      if ((rc = ts_sync(s))) return rc;
      fval = s.host[S_EN + GB_E_TOTAL];
      gval = 2.0 * s.host[S_A] * dV;
      accepted = true;
      if (newton_only) {
        task = DCS_CONV;
        if (s.verbose)
          fprintf(stderr, "[gbofdft tn] it %d Newton step %.6e below the energy resolution (pred %.3e, df %.3e)\n",
                  it, stp, pred, fval - energy);
        ++nls;
        break;
      }
      // energy change below the evaluation's resolution: the sufficient-
      // decrease test cannot be decided, the derivative (computed from the
      // potential, not from energy differences) still can -- accept a step
      // that has reduced |dE/dtheta| enough.
      if (o.eres > 0.0 && fabs(fval - energy) <= o.eres * fmax(1.0, fabs(energy)) &&
          fabs(gval) <= o.c2 * fabs(2.0 * d0 * dV)) {
        task = DCS_CONV;
        if (s.verbose)
          fprintf(stderr, "[gbofdft tn] it %d ls %d stp %.6e accepted at energy resolution (df %.3e g %.3e)\n", it,
                  nls, stp, fval - energy, gval);
        ++nls;
        break;
      }
      if (s.verbose)
        fprintf(stderr, "[gbofdft tn] it %d ls %d stp %.6e f %.12f df %.3e g %.6e task %d\n", it, nls, stp, fval,
                fval - energy, gval, task);
    }
    if (s.verbose)
      fprintf(stderr, "[gbofdft tn] it %d E %.12f d0*dV %.6e theta0 %.6e theta %.6e ls_end task %d nls %d\n", it,
              energy, d0 * dV, theta0, theta, task, nls);
    if (nls >= o.maxls || task == DCS_WARN || task == DCS_ERROR || !accepted) {
      converged = 1;  // line search failed (optimization.py:440-444)
      break;
    }
    theta = stp;
    // accept: phi <- newphi, pot <- newpot (swap buffers)
    void* t0 = s.w.f[F_PHI]; s.w.f[F_PHI] = s.w.f[F_PHI1]; s.w.f[F_PHI1] = t0;
    void* t1 = s.w.f[F_POT]; s.w.f[F_POT] = s.w.f[F_POT1]; s.w.f[F_POT1] = t1;
    if ((rc = mu_residual(mu, energy, resN))) return rc;
    push_hist(energy);
    // a Newton step whose inner CG reduced the residual to cg_rtol leaves a
    // model decrease of about cg_rtol x this step's for the next one: below
    // pred_stop, stop without computing that direction
    if (o.pred_stop > 0.0 && o.pred_next && pred * o.cg_rtol < o.pred_stop) {
      converged = 0;
      break;
    }
    // check_converge (optimization.py:522-535)
    if (nhist - 1 >= o.ncheck) {
      bool ok = true;
      for (int i = 0; i < o.ncheck; ++i)
        if (fabs(ehist_last[nhist - 2 - i] - ehist_last[nhist - 1]) > o.econv) { ok = false; break; }
      if (ok) { converged = 0; break; }
    }
  }
  if (it >= o.maxiter) converged = 2;
  // final density = phi^2
  {
    T* phi = F<T>(s, F_PHI);
    rc = launch_mr<0, T>(w, N, [=] __device__(int64_t i, T* c) { rio[i] = phi[i] * phi[i]; }, S_A, st);
    if (rc) return rc;
    if ((rc = ts_sync(s))) return rc;
  }
  res->energy = energy;
  res->mu = mu;
  res->converged = converged;
  res->n_iter = it;
  res->n_eval_ev = s.n_ev;
  res->n_eval_v = s.n_v;
  res->n_eval_hess = s.n_hv;
  res->n_history = nh;
  res->n_sync = s.n_sync;
  res->t_sync = s.t_sync;
  res->t_total = now_s() - s.t_start;
  if (s.time_evals) {
    evt_drain();
    res->t_eval_timed = g_evt.ms * 1e-3;
    res->n_eval_timed = g_evt.count;
  }
  res->n_eval_delta = s.n_delta;
  for (int k = 0; k < GBOFDFT_NE; ++k) res->energies[k] = s.host[S_EN + k];
  return 0;
}

extern "C" {

int gbofdft_tn_workspace_bytes(const gbofdft_plan* p, int64_t* bytes) {
  GB_REQUIRE(p && bytes, "tn_workspace_bytes: null argument");
  const size_t fb = ((gb_elem(p) * (size_t)p->N + 255) / 256) * 256;
  *bytes = (int64_t)(fb * F_NF + sizeof(double) * (kRedBlocks * kMaxVals + S_COUNT) + 256);
  return GBOFDFT_OK;
}

int gbofdft_tn_options_default(gbofdft_tn_options* o) {
  GB_REQUIRE(o, "tn_options_default: null argument");
  // defaults of Optimization (optimization.py:64-77)
  o->econv = 1.0e-5;
  o->maxfun = 50;
  o->maxiter = 200;
  o->maxls = 30;
  o->c1 = 1e-4;
  o->c2 = 0.2;
  o->xtol = 1e-12;
  o->ncheck = 2;
  o->eps = 0.0;
  o->pred_stop = 0.0;
  o->eres = 0.0;
  o->cg_rtol = 0.1;
  o->pred_next = 0;
  o->precond = 0;
  o->time_evals = 0;
  o->delta = nullptr;
  o->delta_rtol = 1e-3;
  o->res0_max = 0.0;
  return GBOFDFT_OK;
}

int gbofdft_tn_hess_workspace_bytes(const gbofdft_plan* hp, int64_t* bytes) {
  GB_REQUIRE(hp && bytes, "tn_hess_workspace_bytes: null argument");
  const size_t fb = ((gb_elem(hp) * (size_t)hp->N + 255) / 256) * 256;
  *bytes = (int64_t)(fb * H_NF + 256);
  return GBOFDFT_OK;
}

int gbofdft_optimize_tn(gbofdft_plan* p, const gbofdft_functional* f, void* rho_io, const gbofdft_tn_options* o,
                        void* workspace, int64_t workspace_bytes, gbofdft_tn_result* res, void* stream) {
  return gbofdft_optimize_tn_split(p, f, nullptr, nullptr, rho_io, o, workspace, workspace_bytes, nullptr, 0, res,
                                   stream);
}

int gbofdft_optimize_tn_split(gbofdft_plan* p, const gbofdft_functional* f, gbofdft_plan* hp,
                              const gbofdft_functional* hf, void* rho_io, const gbofdft_tn_options* o,
                              void* workspace, int64_t workspace_bytes, void* hworkspace, int64_t hworkspace_bytes,
                              gbofdft_tn_result* res, void* stream) {
  GB_REQUIRE(p && f && rho_io && o && workspace && res, "optimize_tn: null argument");
  if (hp) {
    GB_REQUIRE(hf && hworkspace, "optimize_tn_split: Hessian plan without functional or workspace");
    GB_REQUIRE(p->prec == GBOFDFT_F64 && hp->prec == GBOFDFT_F32,
               "optimize_tn_split: the outer plan must be FP64 and the Hessian plan FP32");
    GB_REQUIRE(hp->n[0] == p->n[0] && hp->n[1] == p->n[1] && hp->n[2] == p->n[2] &&
                   memcmp(hp->lattice, p->lattice, sizeof(p->lattice)) == 0 && hp->full == p->full,
               "optimize_tn_split: the Hessian plan describes another grid");
    int64_t hneed = 0;
    gbofdft_tn_hess_workspace_bytes(hp, &hneed);
    GB_REQUIRE(hworkspace_bytes >= hneed, "optimize_tn_split: Hessian workspace %lld bytes < %lld",
               (long long)hworkspace_bytes, (long long)hneed);
    GB_REQUIRE(((uintptr_t)hworkspace & 255) == 0, "optimize_tn_split: Hessian workspace must be 256-byte aligned");
  }
  GB_REQUIRE(!o->delta || hp, "optimize_tn: delta evaluation needs the split mode (an FP32 Hessian plan)");
  GB_REQUIRE(!o->delta || o->delta_rtol > 0.0, "optimize_tn: delta_rtol must be > 0");
  GB_REQUIRE(o->pred_stop >= 0.0, "optimize_tn: pred_stop must be >= 0");
  GB_REQUIRE(o->cg_rtol > 0.0 && o->cg_rtol < 1.0, "optimize_tn: cg_rtol must be in (0, 1)");
  int64_t need = 0;
  gbofdft_tn_workspace_bytes(p, &need);
  GB_REQUIRE(workspace_bytes >= need, "optimize_tn: workspace %lld bytes < %lld", (long long)workspace_bytes,
             (long long)need);
  GB_REQUIRE(o->maxiter >= 1 && o->maxfun >= 1 && o->maxls >= 1 && o->ncheck >= 1 && o->ncheck < 60,
             "optimize_tn: bad options");
  GB_REQUIRE(((uintptr_t)workspace & 255) == 0, "optimize_tn: workspace must be 256-byte aligned");
  TnState s;
  memset(&s, 0, sizeof(s));
  s.p = p;
  s.fn = f;
  s.st = (cudaStream_t)stream;
  s.t_start = now_s();
  {
    const char* v = getenv("GBOFDFT_TN_VERBOSE");
    s.verbose = v && v[0] == '1';
  }
  s.time_evals = o->time_evals != 0;
  res->t_eval_timed = 0.0;
  res->n_eval_timed = 0;
  res->n_eval_delta = 0;
  if (s.time_evals) {
    g_evt.n = 0;
    g_evt.ms = 0.0;
    g_evt.count = 0;
  }
  const size_t fb = ((gb_elem(p) * (size_t)p->N + 255) / 256) * 256;
  char* base = reinterpret_cast<char*>(workspace);
  for (int i = 0; i < F_NF; ++i) s.w.f[i] = base + fb * i;
  s.w.partials = reinterpret_cast<double*>(base + fb * F_NF);
  s.w.sc = s.w.partials + kRedBlocks * kMaxVals;
  s.w.counter = reinterpret_cast<unsigned*>(s.w.sc + S_COUNT);
  GB_CUDA(cudaMemsetAsync(s.w.sc, 0, sizeof(double) * S_COUNT + 256, s.st));
  memset(res->energies, 0, sizeof(res->energies));
  if (hp) {
    s.hp = hp;
    s.hfn = hf;
    const size_t hb = ((gb_elem(hp) * (size_t)hp->N + 255) / 256) * 256;
    char* hbase = reinterpret_cast<char*>(hworkspace);
    for (int i = 0; i < H_NF; ++i) s.hf[i] = hbase + hb * i;
    s.delta = o->delta;
    s.delta_rtol = o->delta_rtol;
  }
  return p->prec == GBOFDFT_F64 ? tn_run<double>(s, rho_io, *o, res) : tn_run<float>(s, rho_io, *o, res);
}

int gbofdft_dcsrch(double* state, int64_t state_len, double* stp, double f, double g, int task) {
  // Host-side line-search step, exposed for tests and for callers that run
  // their own loops.  state holds the Dcsrch struct (>= 24 doubles); on
  // DCS_START it is initialised from state[0..4] = ftol, gtol, xtol, stpmin,
  // stpmax.  Returns the new task code (DCS_* values).
  GB_REQUIRE(state && stp && state_len * (int64_t)sizeof(double) >= (int64_t)sizeof(Dcsrch),
             "dcsrch: state buffer too small");
  Dcsrch s;
  memcpy(&s, state, sizeof(Dcsrch));
  if (task == DCS_START) dcs_init(s, state[0], state[1], state[2], state[3], state[4]);
  const int t = dcs_step(s, *stp, f, g, task);
  memcpy(state, &s, sizeof(Dcsrch));
  return t;
}

}  // extern "C"
