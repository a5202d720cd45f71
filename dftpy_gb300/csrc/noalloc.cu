// gbofdft_convolve_noalloc: the reciprocal-space convolution of
// gbofdft_convolve for callers that cannot allocate device memory.
//
// Some callers of this library run where cudaMalloc / cudaFree are not
// available to them: a plugin invoked inside another framework that owns
// every byte of device memory through its own allocator, or code that must
// not trigger the implicit device synchronisation cudaMalloc and cudaFree can
// cause.  They cannot create a gbofdft_plan (plan creation allocates the
// twiddle tables and workspaces), so this entry point takes the grid
// description directly and keeps all of its scratch -- the three twiddle
// tables and one spectrum -- in a fixed, file-scope device array.
//
// Limits and behaviour:
//  * scratch is GB_NOALLOC_BYTES (16 MiB); every GPU that loads the library
//    holds it until the process exits.  The twiddle tables plus one spectrum
//    (n0 * n1 * (n2/2+1 rounded up to a 128-byte row) complex elements) must
//    fit; larger grids are rejected with GBOFDFT_ERR_UNSUPPORTED.
//  * every call shares that array: calls whose work overlaps on the GPU (two
//    streams, or two devices' calls that somehow alias) race and corrupt each
//    other.  Serialise them.  Each call rewrites everything it reads from the
//    array (twiddles and the whole spectrum region), so nothing has to be
//    cleared between calls.
//  * a call that fails after it has started (a launch error in a later pass)
//    may already have rewritten the twiddles and part of the spectrum: the
//    array's contents are never valid across calls anyway.
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device, with that device current); make
//    that first call before any stream capture begins.  The address is kept
//    per device number for the life of the process: after cudaDeviceReset,
//    or from a different context on the same device (made through the
//    driver API), it no longer belongs to the current module -- neither is
//    supported.
//  * the twiddle factors are computed on the device (sincospi in double
//    precision), while gbofdft_plan_create tabulates them on the host in long
//    double, so the result equals gbofdft_convolve's to rounding, not bit
//    for bit.
#include <math.h>
#include <string.h>

#include <mutex>

#include "plan.h"

#define GB_NOALLOC_BYTES (16u << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[GB_NOALLOC_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[64];

// Device address of the scratch array for the current device (set-up on the
// first call per device).
static int noalloc_scratch(void** out) {
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_REQUIRE(dev >= 0 && dev < 64, "convolve_noalloc: device index %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return gb_set_error(GBOFDFT_ERR_CUDA, "convolve_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return GBOFDFT_OK;
}

// exp(-2 pi i m / n), m in [0, n), written as complex<prec>
__global__ void k_noalloc_twiddles(int n, int f64, void* out) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * (double)m / (double)n, &s, &c);
    if (f64) reinterpret_cast<double2*>(out)[m] = double2{c, s};
    else reinterpret_cast<float2*>(out)[m] = float2{(float)c, (float)s};
  }
}

static void na_factorize(int n, AxisPlan& ax) {
  ax.n = n;
  ax.nst = 0;
  int m = n;
  const int pref[] = {8, 4, 2, 3, 5};
  for (int r : pref)
    while (m % r == 0 && ax.nst < GB_MAX_STAGES) { ax.radix[ax.nst++] = r; m /= r; }
  for (int pr = 7; m > 1 && ax.nst < GB_MAX_STAGES; pr += 2)
    while (m % pr == 0) { ax.radix[ax.nst++] = pr; m /= pr; }
}

static size_t na_round(size_t x) { return (x + 255) / 256 * 256; }

extern "C" int gbofdft_convolve_noalloc(const int nr[3], const double lattice[9], int precision, int full,
                                        const void* in, void* out, int kernel, const void* kernel_array,
                                        double coef, void* stream) {
  GB_REQUIRE(nr && lattice && in && out, "convolve_noalloc: null argument");
  GB_REQUIRE(precision == GBOFDFT_F32 || precision == GBOFDFT_F64, "convolve_noalloc: bad precision %d", precision);
  GB_REQUIRE(kernel >= GBOFDFT_KER_NONE && kernel <= GBOFDFT_KER_ARRAY, "convolve_noalloc: bad kernel %d", kernel);
  GB_REQUIRE(kernel != GBOFDFT_KER_ARRAY || kernel_array, "convolve_noalloc: kernel array missing");
  for (int a = 0; a < 3; ++a)
    GB_REQUIRE(nr[a] >= 1 && nr[a] <= GB_MAX_N, "convolve_noalloc: nr[%d]=%d outside [1, %d]", a, nr[a], GB_MAX_N);
  // grid description (the geometry gbofdft_plan_create computes), on the stack
  gbofdft_plan p;
  memset(&p, 0, sizeof(p));
  for (int a = 0; a < 3; ++a) p.n[a] = nr[a];
  p.n2h = nr[2] / 2 + 1;
  const int per_line = precision == GBOFDFT_F64 ? 8 : 16;
  p.ld2 = (p.n2h + per_line - 1) / per_line * per_line;
  p.full = full ? 1 : 0;
  p.prec = precision;
  GB_CUDA(cudaGetDevice(&p.device));
  memcpy(p.lattice, lattice, sizeof(double) * 9);
  const double* L = lattice;
  const double A = L[4] * L[8] - L[5] * L[7], B = -(L[3] * L[8] - L[5] * L[6]), C = L[3] * L[7] - L[4] * L[6];
  const double det = L[0] * A + L[1] * B + L[2] * C;
  GB_REQUIRE(fabs(det) > 0.0, "convolve_noalloc: singular lattice");
  const double id = 1.0 / det;
  const double inv[9] = {A * id, -(L[1] * L[8] - L[2] * L[7]) * id, (L[1] * L[5] - L[2] * L[4]) * id,
                         B * id, (L[0] * L[8] - L[2] * L[6]) * id, -(L[0] * L[5] - L[2] * L[3]) * id,
                         C * id, -(L[0] * L[7] - L[1] * L[6]) * id, (L[0] * L[4] - L[1] * L[3]) * id};
  const double twopi = 6.283185307179586476925286766559;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) p.bg[r * 3 + c] = twopi * inv[c * 3 + r];
  p.volume = fabs(det);
  p.N = (int64_t)nr[0] * nr[1] * nr[2];
  p.NG = (int64_t)nr[0] * nr[1] * p.n2h;
  p.NGld = (int64_t)nr[0] * nr[1] * p.ld2;
  p.dV = p.volume / (double)p.N;
  const size_t cs = precision == GBOFDFT_F64 ? 16 : 8;
  for (int a = 0; a < 3; ++a) {
    na_factorize(nr[a], p.ax[a]);
    int tb = (int)((96 * 1024 / cs - nr[a]) / (2 * (size_t)nr[a]));
    p.tb[a] = tb > 16 ? 16 : (tb < 1 ? 1 : tb);
  }
  p.pairs = 2;
  memcpy(p.gi.bg, p.bg, sizeof(p.bg));
  p.gi.n0 = nr[0]; p.gi.n1 = nr[1]; p.gi.n2 = nr[2]; p.gi.n2h = p.n2h; p.gi.ld2 = p.ld2; p.gi.full = p.full;
  // scratch layout: three twiddle tables, then one spectrum
  size_t off[4];
  size_t need = 0;
  for (int a = 0; a < 3; ++a) { off[a] = need; need += na_round(cs * (size_t)nr[a]); }
  off[3] = need;
  need += na_round(cs * (size_t)p.NGld);
  if (need > GB_NOALLOC_BYTES)
    return gb_set_error(GBOFDFT_ERR_UNSUPPORTED,
                        "convolve_noalloc: grid %dx%dx%d (%s) needs %zu bytes of scratch, the fixed array holds %u",
                        nr[0], nr[1], nr[2], precision == GBOFDFT_F64 ? "f64" : "f32", need, GB_NOALLOC_BYTES);
  void* base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc) return rc;
  char* b = reinterpret_cast<char*>(base);
  cudaStream_t st = (cudaStream_t)stream;
  for (int a = 0; a < 3; ++a) {
    p.tw[a] = b + off[a];
    k_noalloc_twiddles<<<(nr[a] + 255) / 256, 256, 0, st>>>(nr[a], precision == GBOFDFT_F64, p.tw[a]);
    GB_CHECK_LAUNCH();
  }
  p.spec = b + off[3];
  // the gbofdft_convolve pipeline on the fixed scratch
  const int op = OP_RHO;
  KerDesc kd;
  memset(&kd, 0, sizeof(kd));
  kd.type[0] = kernel;
  kd.arr[0] = kernel_array;
  kd.coef[0] = coef;
  rc = gb_rows_fwd(&p, in, p.spec, 0, p.ld2, 1, &op, 1.0, 1.0, st);
  if (!rc) rc = gb_cols(&p, p.spec, 0, p.ld2, 1, 1, -1, 1.0, st);
  if (!rc) rc = gb_cols_conv(&p, p.spec, 0, p.ld2, 1, kd, 1.0 / (double)p.N, st);
  if (!rc) rc = gb_cols(&p, p.spec, 0, p.ld2, 1, 1, 1, 1.0, st);
  if (!rc) rc = gb_rows_inv_store(&p, p.spec, 0, p.ld2, 1, out, 0, 1.0, st);
  return rc;
}
