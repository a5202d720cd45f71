// C ABI entry points: plans, FFTs, the fused functional evaluation.
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>

#include <new>
#include <vector>

#include "plan.h"

#include <atomic>
#include <map>
#include <mutex>

static thread_local char g_err[1024] = "";
static std::atomic<long long> g_launches(0);

void gb_count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// dynamic shared-memory grants already made with cudaFuncSetAttribute
static std::mutex g_smem_mu;
static std::map<std::pair<const void*, int>, int> g_smem;

int gb_smem_granted(const void* kern, int dev) {
  std::lock_guard<std::mutex> lk(g_smem_mu);
  auto it = g_smem.find({kern, dev});
  return it == g_smem.end() ? 0 : it->second;
}

void gb_smem_grant(const void* kern, int dev, int bytes) {
  std::lock_guard<std::mutex> lk(g_smem_mu);
  int& v = g_smem[{kern, dev}];
  if (bytes > v) v = bytes;
}

int gb_set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

size_t gb_elem(const gbofdft_plan* p) { return p->prec == GBOFDFT_F64 ? 8 : 4; }

static void factorize(int n, AxisPlan& ax) {
  ax.n = n;
  ax.nst = 0;
  int m = n;
  const int pref[] = {8, 4, 2, 3, 5};
  for (int r : pref)
    while (m % r == 0 && ax.nst < GB_MAX_STAGES) { ax.radix[ax.nst++] = r; m /= r; }
  for (int pr = 7; m > 1 && ax.nst < GB_MAX_STAGES; pr += 2)
    while (m % pr == 0) { ax.radix[ax.nst++] = pr; m /= pr; }
}

static void det_inv(const double* L, double* inv, double* det) {
  const double a = L[0], b = L[1], c = L[2], d = L[3], e = L[4], f = L[5], g = L[6], h = L[7], i = L[8];
  const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
  *det = a * A + b * B + c * C;
  const double id = 1.0 / *det;
  inv[0] = A * id; inv[1] = -(b * i - c * h) * id; inv[2] = (b * f - c * e) * id;
  inv[3] = B * id; inv[4] = (a * i - c * g) * id;  inv[5] = -(a * f - c * d) * id;
  inv[6] = C * id; inv[7] = -(a * h - b * g) * id; inv[8] = (a * e - b * d) * id;
}

extern "C" {

int gbofdft_version(void) { return GBOFDFT_ABI_VERSION; }

int gbofdft_launch_count(int64_t* count) {
  GB_REQUIRE(count, "launch_count: null argument");
  *count = (int64_t)g_launches.load(std::memory_order_relaxed);
  return GBOFDFT_OK;
}

int gbofdft_last_error(char* buf, size_t len) {
  size_t n = strlen(g_err);
  if (buf && len) {
    size_t m = n < len - 1 ? n : len - 1;
    memcpy(buf, g_err, m);
    buf[m] = 0;
  }
  return (int)n;
}

int gbofdft_plan_destroy(gbofdft_plan* p) {
  if (!p) return GBOFDFT_OK;
  for (int a = 0; a < 3; ++a)
    if (p->tw[a]) cudaFree(p->tw[a]);
  if (p->spec) cudaFree(p->spec);
  if (p->partials) cudaFree(p->partials);
  if (p->scratch) cudaFree(p->scratch);
  if (p->wt_pm) cudaFree(p->wt_pm);
  if (p->precond_pm) cudaFree(p->precond_pm);
  if (p->wgc_pm) cudaFree(p->wgc_pm);
  delete p;
  return GBOFDFT_OK;
}

int gbofdft_plan_create(const int nr[3], const double lattice[9], int precision, int full, gbofdft_plan** out) {
  GB_REQUIRE(nr && lattice && out, "plan_create: null argument");
  GB_REQUIRE(precision == GBOFDFT_F32 || precision == GBOFDFT_F64, "plan_create: bad precision %d", precision);
  for (int a = 0; a < 3; ++a)
    GB_REQUIRE(nr[a] >= 1 && nr[a] <= GB_MAX_N, "plan_create: nr[%d]=%d outside [1, %d]", a, nr[a], GB_MAX_N);
  *out = nullptr;
  gbofdft_plan* p = new (std::nothrow) gbofdft_plan;
  if (!p) return gb_set_error(GBOFDFT_ERR_ALLOC, "plan_create: host allocation failed");
  memset(p, 0, sizeof(*p));
  for (int a = 0; a < 3; ++a) p->n[a] = nr[a];
  p->n2h = nr[2] / 2 + 1;
  // internal spectrum rows padded to whole 128-byte lines
  {
    const int per_line = precision == GBOFDFT_F64 ? 8 : 16;
    p->ld2 = (p->n2h + per_line - 1) / per_line * per_line;
  }
  p->full = full ? 1 : 0;
  p->prec = precision;
  cudaGetDevice(&p->device);
  memcpy(p->lattice, lattice, sizeof(double) * 9);
  double inv[9], det;
  det_inv(lattice, inv, &det);
  if (!(fabs(det) > 0.0)) {
    delete p;
    return gb_set_error(GBOFDFT_ERR_ARG, "plan_create: singular lattice");
  }
  const double twopi = 6.283185307179586476925286766559;
  // bg = 2 pi inv(L)^T, rows are reciprocal vectors
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) p->bg[r * 3 + c] = twopi * inv[c * 3 + r];
  p->volume = fabs(det);
  p->N = (int64_t)nr[0] * nr[1] * nr[2];
  p->NG = (int64_t)nr[0] * nr[1] * p->n2h;
  p->NGld = (int64_t)nr[0] * nr[1] * p->ld2;
  p->dV = p->volume / (double)p->N;
  const size_t cs = 2 * gb_elem(p);
  // The plan's initial device contents (twiddles, the zeroed counter) are
  // written on a stream of its own and complete before plan_create returns:
  // cudaMemcpy from pageable memory and cudaMemset return before the device
  // has finished, on the legacy stream, which the callers' non-blocking
  // streams do not wait for -- a first transform on such a stream could read
  // a half-written table.
  cudaStream_t init_st = nullptr;
  {
    cudaError_t e = cudaStreamCreateWithFlags(&init_st, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete p; return gb_set_error(GBOFDFT_ERR_CUDA, "plan_create: %s", cudaGetErrorString(e)); }
  }
  auto fail = [&](int code, const char* what, cudaError_t e) {
    cudaStreamSynchronize(init_st);
    cudaStreamDestroy(init_st);
    gbofdft_plan_destroy(p);
    return gb_set_error(code, "plan_create: %s%s", what, cudaGetErrorString(e));
  };
  for (int a = 0; a < 3; ++a) {
    factorize(nr[a], p->ax[a]);
    std::vector<double> t(2 * (size_t)nr[a]);
    for (int m = 0; m < nr[a]; ++m) {
      // exp(-2 pi i m / n); reduce by symmetry to keep the angle small
      const long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double)m / (long double)nr[a];
      t[2 * m] = (double)cosl(ang);
      t[2 * m + 1] = (double)sinl(ang);
    }
    cudaError_t e = cudaMalloc(&p->tw[a], cs * nr[a]);
    if (e != cudaSuccess) return fail(GBOFDFT_ERR_ALLOC, "", e);
    // from pageable memory the copy returns once the host buffer is staged,
    // so t / tf may go out of scope before the stream has run it
    if (precision == GBOFDFT_F64) {
      e = cudaMemcpyAsync(p->tw[a], t.data(), cs * nr[a], cudaMemcpyHostToDevice, init_st);
    } else {
      std::vector<float> tf(t.begin(), t.end());
      e = cudaMemcpyAsync(p->tw[a], tf.data(), cs * nr[a], cudaMemcpyHostToDevice, init_st);
    }
    if (e != cudaSuccess) return fail(GBOFDFT_ERR_CUDA, "", e);
  }
  // column tile: keep (n + 2 n tb) complex elements within ~96 KB
  for (int a = 0; a < 3; ++a) {
    const int n = nr[a];
    int tb = (int)((96 * 1024 / cs - n) / (2 * (size_t)n));
    if (tb > 16) tb = 16;
    if (tb < 1) tb = 1;
    p->tb[a] = tb;
  }
  p->pairs = 2;
  const size_t rows_sm = cs * ((size_t)nr[2] + 2 * (size_t)GB_MAX_FIELDS * p->pairs * nr[2]);
  if (rows_sm > 200 * 1024 || cs * ((size_t)nr[0] * (1 + 2 * p->tb[0])) > 220 * 1024 ||
      cs * ((size_t)nr[1] * (1 + 2 * p->tb[1])) > 220 * 1024) {
    cudaStreamSynchronize(init_st);
    cudaStreamDestroy(init_st);
    gbofdft_plan_destroy(p);
    return gb_set_error(GBOFDFT_ERR_UNSUPPORTED, "plan_create: grid %dx%dx%d too large for the line passes",
                        nr[0], nr[1], nr[2]);
  }
  cudaError_t e = cudaMalloc(&p->spec, cs * (size_t)GB_MAX_FIELDS * p->NGld);
  const int64_t nrows = (int64_t)nr[0] * nr[1];
  p->max_partials = (nrows + 2 * p->pairs - 1) / (2 * p->pairs) + 1;
  if (e == cudaSuccess) e = cudaMalloc(&p->partials, sizeof(double) * GB_NE * p->max_partials);
  if (e == cudaSuccess) e = cudaMalloc(&p->scratch, sizeof(double) * 4096);
  // the counter slot starts at 0
  if (e == cudaSuccess) e = cudaMemsetAsync(p->scratch, 0, sizeof(double) * 4096, init_st);
  if (e != cudaSuccess) return fail(GBOFDFT_ERR_ALLOC, "workspace: ", e);
  e = cudaStreamSynchronize(init_st);
  cudaStreamDestroy(init_st);
  if (e != cudaSuccess) {
    gbofdft_plan_destroy(p);
    return gb_set_error(GBOFDFT_ERR_CUDA, "plan_create: initial copies: %s", cudaGetErrorString(e));
  }
  memcpy(p->gi.bg, p->bg, sizeof(p->bg));
  p->gi.n0 = nr[0]; p->gi.n1 = nr[1]; p->gi.n2 = nr[2]; p->gi.n2h = p->n2h; p->gi.ld2 = p->ld2;
  p->gi.full = p->full;
  // FP32 grids whose (n0, n1) plane fits in shared memory evaluate through
  // the plane pipeline (GBOFDFT_PLANE=0 selects the column passes instead)
  const char* pe = getenv("GBOFDFT_PLANE");
  p->plane_ok = precision == GBOFDFT_F32 && gb_plane_supported_f32(nr[0], nr[1], nr[2]);
  p->plane = p->plane_ok && !(pe && pe[0] == '0');
  p->plane_variant = 0;
  // GBOFDFT_PLANE_PRECOND=1: the TN preconditioner's convolutions through the
  // plane pipeline too (one field: fills fewer SMs than the column passes, so
  // it pays only when other streams run beside it)
  const char* pp = getenv("GBOFDFT_PLANE_PRECOND");
  p->plane_precond = p->plane && pp && pp[0] == '1';
  *out = p;
  return GBOFDFT_OK;
}

int gbofdft_plan_schedules(const gbofdft_plan* p, int* count) {
  GB_REQUIRE(p && count, "plan_schedules: null argument");
  *count = 1 + (p->plane_ok ? gb_plane_variants_f32(p->n[0], p->n[1]) : 0);
  return GBOFDFT_OK;
}

int gbofdft_plan_set_schedule(gbofdft_plan* p, int schedule) {
  GB_REQUIRE(p, "plan_set_schedule: null argument");
  int count = 0;
  gbofdft_plan_schedules(p, &count);
  GB_REQUIRE(schedule >= 0 && schedule < count, "plan_set_schedule: schedule %d outside [0, %d)", schedule, count);
  p->plane = schedule > 0;
  p->plane_variant = schedule > 0 ? schedule - 1 : 0;
  return GBOFDFT_OK;
}

int gbofdft_plan_get_schedule(const gbofdft_plan* p, int* schedule) {
  GB_REQUIRE(p && schedule, "plan_get_schedule: null argument");
  *schedule = p->plane ? 1 + p->plane_variant : 0;
  return GBOFDFT_OK;
}

int gbofdft_plan_sizes(const gbofdft_plan* p, int64_t out[4]) {
  GB_REQUIRE(p && out, "plan_sizes: null argument");
  out[0] = p->N;
  out[1] = p->NG;
  out[2] = p->n2h;
  out[3] = (int64_t)(2 * gb_elem(p) * (GB_MAX_FIELDS * p->NGld + p->n[0] + p->n[1] + p->n[2])) +
           (int64_t)sizeof(double) * (GB_NE * p->max_partials + 4096);
  return GBOFDFT_OK;
}

int gbofdft_fft_r2c(gbofdft_plan* p, const void* in, void* out, void* stream) {
  GB_REQUIRE(p && in && out, "fft_r2c: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int op = OP_RHO;
  int rc = gb_rows_fwd(p, in, out, 0, p->n2h, 1, &op, 1.0, p->dV, st);
  if (!rc) rc = gb_cols(p, out, 0, p->n2h, 1, 1, -1, 1.0, st);
  if (!rc) rc = gb_cols(p, out, 0, p->n2h, 1, 0, -1, 1.0, st);
  return rc;
}

int gbofdft_fft_c2r(gbofdft_plan* p, const void* in, void* out, void* stream) {
  GB_REQUIRE(p && in && out, "fft_c2r: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t cs = 2 * gb_elem(p);
  GB_CUDA(cudaMemcpy2DAsync(p->spec, cs * p->ld2, in, cs * p->n2h, cs * p->n2h, (size_t)p->n[0] * p->n[1],
                            cudaMemcpyDeviceToDevice, st));
  int rc = gb_cols(p, p->spec, 0, p->ld2, 1, 0, 1, 1.0, st);
  if (!rc) rc = gb_cols(p, p->spec, 0, p->ld2, 1, 1, 1, 1.0, st);
  if (!rc) rc = gb_rows_inv_store(p, p->spec, 0, p->ld2, 1, out, 0, 1.0 / ((double)p->N * p->dV), st);
  return rc;
}

int gbofdft_convolve(gbofdft_plan* p, const void* in, void* out, int kernel, const void* karr, double coef,
                     void* stream) {
  GB_REQUIRE(p && in && out, "convolve: null argument");
  GB_REQUIRE(kernel >= GBOFDFT_KER_NONE && kernel <= GBOFDFT_KER_ARRAY, "convolve: bad kernel %d", kernel);
  GB_REQUIRE(kernel != GBOFDFT_KER_ARRAY || karr, "convolve: kernel array missing");
  cudaStream_t st = (cudaStream_t)stream;
  const int op = OP_RHO;
  KerDesc kd;
  memset(&kd, 0, sizeof(kd));
  kd.type[0] = kernel;
  kd.arr[0] = karr;
  kd.coef[0] = coef;
  if (p->plane_precond && kernel == GBOFDFT_KER_ARRAY && karr == p->precond_pm_src && p->precond_pm && gb_use_ct()) {
    // the preconditioner: rows forward, one plane convolution, rows inverse
    const float* pm_arr[GB_MAX_FIELDS] = {p->precond_pm, nullptr, nullptr, nullptr};
    const int64_t fs = p->NG;
    int rc = gb_ct_rows_fwd_pm_f32(p, in, p->spec, fs, 1, &op, 1.0, st);
    if (!rc) rc = gb_plane_conv_f32(p, p->spec, fs, 1, &kd, pm_arr, 1.0 / (double)p->N, st);
    if (!rc) rc = gb_ct_rows_inv_store_pm_f32(p, p->spec, fs, 1, out, 0, st);
    if (rc != 1) return rc;
  }
  int rc = gb_rows_fwd(p, in, p->spec, 0, p->ld2, 1, &op, 1.0, 1.0, st);
  if (!rc) rc = gb_cols(p, p->spec, 0, p->ld2, 1, 1, -1, 1.0, st);
  if (!rc) rc = gb_cols_conv(p, p->spec, 0, p->ld2, 1, kd, 1.0 / (double)p->N, st);
  if (!rc) rc = gb_cols(p, p->spec, 0, p->ld2, 1, 1, 1, 1.0, st);
  if (!rc) rc = gb_rows_inv_store(p, p->spec, 0, p->ld2, 1, out, 0, 1.0, st);
  return rc;
}

}  // extern "C"

// Evaluation descriptors of a functional: the fused terms' epilogue flags and
// constants, the convolution fields (prologue op, kernel) in slot order.
static int eval_descs(const gbofdft_functional* f, EvalDesc& ev, KerDesc& kd, int* ops, int& nf) {
  GB_REQUIRE(!f->wt || f->wt_kernel, "eval: WT enabled without a kernel table");
  GB_REQUIRE(!f->wt || fabs(f->wt_alpha - f->wt_beta) < 1e-9,
             "eval: fused WT path requires alpha == beta (got %g, %g)", f->wt_alpha, f->wt_beta);
  GB_REQUIRE(f->xc == 0 || f->xc == 1, "eval: unsupported xc %d", f->xc);
  memset(&ev, 0, sizeof(ev));
  memset(&kd, 0, sizeof(kd));
  nf = 0;
  ev.tf = f->tf; ev.tf_x = f->tf_x;
  ev.vw = f->vw; ev.vw_y = f->vw_y;
  ev.wt = f->wt; ev.wt_alpha = f->wt_alpha; ev.wt_beta = f->wt_beta;
  ev.xc = f->xc; ev.hartree = f->hartree; ev.pp = f->vloc != nullptr; ev.e_ion = f->e_ion;
  if (f->hartree) { ev.slot_h = nf; ops[nf] = OP_RHO; kd.type[nf] = KER_HARTREE; kd.coef[nf] = 1.0; ++nf; }
  if (f->vw) { ev.slot_vw = nf; ops[nf] = OP_SQRT; kd.type[nf] = KER_G2; kd.coef[nf] = 1.0; ++nf; }
  if (f->wt) {
    ev.slot_wt = nf; ops[nf] = OP_POWB; kd.type[nf] = KER_ARRAY; kd.arr[nf] = f->wt_kernel; kd.coef[nf] = 1.0;
    ++nf;
  }
  return 0;
}

// the nonlocal terms evaluated outside the fused passes (added to pot /
// energies); wgc_ref: the WGC term also keeps this evaluation as the
// reference of later WGC delta evaluations
static int eval_extra(gbofdft_plan* p, const void* rho, const gbofdft_functional* f, void* pot, double* energies,
                      int calc, cudaStream_t st, int wgc_ref = 0) {
  int rc = 0;
  if (f->lwt)
    rc = gb_lwt_eval(p, rho, f->lwt, pot, energies, (calc & GBOFDFT_CALC_V) ? 1 : 0, (calc & GBOFDFT_CALC_E) ? 1 : 0,
                     st);
  if (!rc && f->wgc)
    rc = gb_wgc_eval(p, rho, f->wgc, pot, energies, (calc & GBOFDFT_CALC_V) ? 1 : 0, (calc & GBOFDFT_CALC_E) ? 1 : 0,
                     wgc_ref, st);
  return rc;
}

// gbofdft_eval; cout != nullptr (FP64 compile-time-size passes) also stores
// the convolution results, field slot f at cout + f * N; extras = 0 leaves
// out the LWT / WGC terms (the fused terms alone)
static int eval_impl(gbofdft_plan* p, const void* rho, const gbofdft_functional* f, void* pot, double* energies,
                     int calc, void* cout, cudaStream_t st, bool extras = true) {
  GB_REQUIRE(p && rho && f && pot, "eval: null argument");
  GB_REQUIRE(!(calc & GBOFDFT_CALC_E) || energies, "eval: energies buffer required with CALC_E");
  EvalDesc ev;
  KerDesc kd;
  int ops[GB_MAX_FIELDS];
  int nf = 0;
  int rc = eval_descs(f, ev, kd, ops, nf);
  if (rc) return rc;
  ev.cout = cout;
  ev.cstride = p->N;
  const int64_t fs = p->NGld;
  if (!cout) {
    rc = gb_eval_plane(p, rho, nf, ops, f->wt_beta, kd, ev, f->vloc, pot, (calc & GBOFDFT_CALC_E) ? 1 : 0, energies,
                       st);
    if (rc == 0) return extras ? eval_extra(p, rho, f, pot, energies, calc, st) : 0;
    if (rc != 1) return rc;
  } else {
    GB_REQUIRE(p->prec == GBOFDFT_F64 && gb_use_ct(), "eval: convolution output needs the FP64 specialised passes");
  }
  rc = 0;
  if (nf > 0) {
    rc = gb_rows_fwd(p, rho, p->spec, fs, p->ld2, nf, ops, f->wt_beta, 1.0, st);
    if (!rc) rc = gb_cols(p, p->spec, fs, p->ld2, nf, 1, -1, 1.0, st);
    if (!rc) rc = gb_cols_conv(p, p->spec, fs, p->ld2, nf, kd, 1.0 / (double)p->N, st);
    if (!rc) rc = gb_cols(p, p->spec, fs, p->ld2, nf, 1, 1, 1.0, st);
  }
  if (!rc)
    rc = gb_rows_inv_eval(p, p->spec, fs, nf, ev, rho, f->vloc, pot, (calc & GBOFDFT_CALC_E) ? 1 : 0, energies, st);
  if (!rc && extras) rc = eval_extra(p, rho, f, pot, energies, calc, st);
  return rc;
}

// Delta-evaluation state: the reference density, its FP64 convolution
// results, potential and energies of the fused terms, on the FP64 plan's grid.
struct gbofdft_delta {
  gbofdft_plan* p64;
  gbofdft_plan* p32;
  double* buf;      // rho_ref [N], pot_ref [N], C_ref [GB_MAX_FIELDS][N], E_ref [GB_NE]
  int valid;
  int wgc_ref;      // the FP64 WGC term's workspace holds the reference of rho_ref
  int nf;
  int ops[GB_MAX_FIELDS];
  int kind[GB_MAX_FIELDS];
};

const double* gb_delta_ref(const gbofdft_delta* d) { return d->buf; }

extern "C" {

int gbofdft_eval(gbofdft_plan* p, const void* rho, const gbofdft_functional* f, void* pot, double* energies,
                 int calc, void* stream) {
  return eval_impl(p, rho, f, pot, energies, calc, nullptr, (cudaStream_t)stream);
}

int gbofdft_delta_create(gbofdft_plan* plan, gbofdft_plan* hplan, gbofdft_delta** out) {
  GB_REQUIRE(plan && hplan && out, "delta_create: null argument");
  *out = nullptr;
  GB_REQUIRE(plan->prec == GBOFDFT_F64 && hplan->prec == GBOFDFT_F32,
             "delta_create: needs an FP64 plan and an FP32 plan");
  GB_REQUIRE(plan->n[0] == hplan->n[0] && plan->n[1] == hplan->n[1] && plan->n[2] == hplan->n[2] &&
                 plan->full == hplan->full,
             "delta_create: the plans are on different grids");
  GB_REQUIRE(hplan->plane_ok && gb_delta_supported(plan->n[0], plan->n[1], plan->n[2]),
             "delta_create: grid %d x %d x %d has no plane-pipeline specialisation", plan->n[0], plan->n[1],
             plan->n[2]);
  gbofdft_delta* d = new gbofdft_delta;
  memset(d, 0, sizeof(*d));
  d->p64 = plan;
  d->p32 = hplan;
  cudaError_t e = cudaMalloc(&d->buf, sizeof(double) * ((size_t)plan->N * (2 + GB_MAX_FIELDS) + GB_NE));
  if (e != cudaSuccess) {
    delete d;
    return gb_set_error(GBOFDFT_ERR_ALLOC, "delta_create: %s", cudaGetErrorString(e));
  }
  *out = d;
  return 0;
}

int gbofdft_delta_destroy(gbofdft_delta* d) {
  if (!d) return 0;
  if (d->buf) cudaFree(d->buf);
  delete d;
  return 0;
}

int gbofdft_eval_delta(gbofdft_delta* d, const void* rho, const gbofdft_functional* f,
                       const gbofdft_functional* hf, void* pot, double* energies, int calc, int rebase,
                       void* stream) {
  GB_REQUIRE(d && rho && f && pot, "eval_delta: null argument");
  GB_REQUIRE(!(calc & GBOFDFT_CALC_E) || energies, "eval_delta: energies buffer required with CALC_E");
  cudaStream_t st = (cudaStream_t)stream;
  EvalDesc ev;
  KerDesc kd;
  int ops[GB_MAX_FIELDS];
  int nf = 0;
  int rc = eval_descs(f, ev, kd, ops, nf);
  if (rc) return rc;
  const int64_t N = d->p64->N;
  double* rho_ref = d->buf;
  double* pot_ref = d->buf + N;
  double* cref = d->buf + 2 * N;
  double* eref = d->buf + (2 + GB_MAX_FIELDS) * N;
  if (nf == 0) return eval_impl(d->p64, rho, f, pot, energies, calc, nullptr, st);
  if (rebase) {
    // the fused terms in full FP64 (energies always, into the state), kept as
    // the reference; then the LWT / WGC terms on top of the caller's outputs
    rc = eval_impl(d->p64, rho, f, pot, eref, calc | GBOFDFT_CALC_E, cref, st, false);
    if (rc) return rc;
    GB_CUDA(cudaMemcpyAsync(rho_ref, rho, sizeof(double) * (size_t)N, cudaMemcpyDeviceToDevice, st));
    GB_CUDA(cudaMemcpyAsync(pot_ref, pot, sizeof(double) * (size_t)N, cudaMemcpyDeviceToDevice, st));
    if (calc & GBOFDFT_CALC_E)
      GB_CUDA(cudaMemcpyAsync(energies, eref, sizeof(double) * GB_NE, cudaMemcpyDeviceToDevice, st));
    d->valid = 1;
    d->nf = nf;
    for (int i = 0; i < GB_MAX_FIELDS; ++i) {
      d->ops[i] = i < nf ? ops[i] : -1;
      d->kind[i] = i < nf ? kd.type[i] : -1;
    }
    d->wgc_ref = 0;
    rc = eval_extra(d->p64, rho, f, pot, energies, calc, st, f->wgc ? 1 : 0);
    if (!rc && f->wgc) d->wgc_ref = 1;
    return rc;
  }
  GB_REQUIRE(d->valid, "eval_delta: no reference evaluation yet (call with rebase = 1 first)");
  GB_REQUIRE(d->nf == nf, "eval_delta: functional terms differ from the reference evaluation's");
  for (int i = 0; i < nf; ++i)
    GB_REQUIRE(d->ops[i] == ops[i] && d->kind[i] == kd.type[i],
               "eval_delta: functional terms differ from the reference evaluation's");
  if (f->wt) {
    GB_REQUIRE(hf && hf->wt && hf->wt_kernel, "eval_delta: WT needs the FP32 functional's kernel table");
    kd.arr[ev.slot_wt] = hf->wt_kernel;
  }
  rc = gb_eval_delta_core(d->p64, d->p32, reinterpret_cast<const double*>(rho), rho_ref, pot_ref, eref, cref, nf, ops,
                          f->wt_beta, kd, ev, reinterpret_cast<const double*>(f->vloc),
                          reinterpret_cast<double*>(pot), (calc & GBOFDFT_CALC_E) ? 1 : 0, energies, st);
  if (rc) return rc;
  // the WGC term as a change from its reference when the FP32 functional has
  // one; LWT (and WGC without an FP32 counterpart) in full FP64
  const bool wgc_delta = f->wgc && d->wgc_ref && hf && hf->wgc &&
                         fabs(f->wgc->rho0 - hf->wgc->rho0) <= 1e-6 * f->wgc->rho0;
  gbofdft_functional rest = *f;
  if (wgc_delta) rest.wgc = nullptr;
  else d->wgc_ref = 0;   // a full WGC evaluation overwrites the reference's fields
  rc = eval_extra(d->p64, rho, &rest, pot, energies, calc, st);
  if (!rc && wgc_delta)
    rc = gb_wgc_eval_delta(d->p64, d->p32, reinterpret_cast<const double*>(rho), rho_ref, f->wgc, hf->wgc,
                           reinterpret_cast<double*>(pot), energies, (calc & GBOFDFT_CALC_E) ? 1 : 0, st);
  return rc;
}

int gbofdft_wt_kernel(gbofdft_plan* p, double rho0, double x, double alpha, double beta, void* out, void* stream) {
  GB_REQUIRE(p && out, "wt_kernel: null argument");
  return gb_build_wt_kernel(p, rho0, x, alpha, beta, out, (cudaStream_t)stream);
}

}  // extern "C"

unsigned* gb_plan_counter(gbofdft_plan* p) { return reinterpret_cast<unsigned*>(p->scratch + 4095); }
