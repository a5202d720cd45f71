// Shared definitions for the gbofdft CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/gbofdft.h"

// ---------------------------------------------------------------------------
// Error reporting: every entry point returns a status and records a message.
// ---------------------------------------------------------------------------
int gb_set_error(int code, const char* fmt, ...);

#define GB_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t _e = (call);                                                       \
    if (_e != cudaSuccess)                                                         \
      return gb_set_error(GBOFDFT_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__,    \
                          #call, cudaGetErrorString(_e));                          \
  } while (0)

void gb_count_launch();

#define GB_CHECK_LAUNCH()                                                          \
  do {                                                                             \
    gb_count_launch();                                                             \
    cudaError_t _e = cudaGetLastError();                                           \
    if (_e != cudaSuccess)                                                         \
      return gb_set_error(GBOFDFT_ERR_CUDA, "%s:%d launch: %s", __FILE__, __LINE__, \
                          cudaGetErrorString(_e));                                 \
  } while (0)

#define GB_REQUIRE(cond, ...)                                                      \
  do {                                                                             \
    if (!(cond)) return gb_set_error(GBOFDFT_ERR_ARG, __VA_ARGS__);                \
  } while (0)

// ---------------------------------------------------------------------------
// Complex helpers on float2 / double2 (interleaved re, im).
// ---------------------------------------------------------------------------
template <typename T> struct CplxOf;
template <> struct CplxOf<float> { using type = float2; };
template <> struct CplxOf<double> { using type = double2; };
template <typename T> using cpx = typename CplxOf<T>::type;

template <typename V> __device__ __forceinline__ V c_add(V a, V b) { return V{a.x + b.x, a.y + b.y}; }
template <typename V> __device__ __forceinline__ V c_sub(V a, V b) { return V{a.x - b.x, a.y - b.y}; }
template <typename V> __device__ __forceinline__ V c_mul(V a, V b) {
  return V{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// a * conj(b)
template <typename V> __device__ __forceinline__ V c_mulc(V a, V b) {
  return V{a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
template <typename V, typename S> __device__ __forceinline__ V c_scale(V a, S s) { return V{a.x * s, a.y * s}; }
// multiply by -i (forward) or +i (inverse): DIR = -1 forward, +1 inverse
template <int DIR, typename V> __device__ __forceinline__ V c_rot(V a) {
  return DIR < 0 ? V{a.y, -a.x} : V{-a.y, a.x};
}

// ---------------------------------------------------------------------------
// FFT axis schedule (mixed radix Stockham).
// ---------------------------------------------------------------------------
#define GB_MAX_STAGES 16
#define GB_MAX_N 2048
#define GB_MAX_FIELDS 4

struct AxisPlan {
  int n;
  int nst;
  int radix[GB_MAX_STAGES];
};

// Energy slots (indices into the energies array)
enum {
  GB_E_TF = 0,
  GB_E_VW = 1,
  GB_E_NL = 2,
  GB_E_XC = 3,
  GB_E_HARTREE = 4,
  GB_E_PSEUDO = 5,
  GB_E_EXTRA = 6,
  GB_E_TOTAL = 7,
  GB_NE = 8
};

// ---------------------------------------------------------------------------
// Compensated (Neumaier) FP64 accumulation.
// ---------------------------------------------------------------------------
struct KSum {
  double s, c;
  __device__ __forceinline__ void init() { s = 0.0; c = 0.0; }
  __device__ __forceinline__ void add(double x) {
    double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x; else c += (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ double value() const { return s + c; }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
