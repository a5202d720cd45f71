// Density guesses and normalisation.
//
//   gbofdft_density_normalize: rho[rho < dtol] = dtol, nc = integral(rho),
//     rho *= ncharge / nc when ncharge > 1e-6 (the clamp-and-scale step of
//     DensityGenerator.guess_rho_atom / get_3d_value_recipe,
//     density/density.py:226-234, 288-297).
//   gbofdft_density_guess: superposed atomic densities from per-species
//     reciprocal-space tables rho_s(|G|) (get_3d_value_recipe,
//     density/density.py:252-300): the structure-factor machinery of the
//     local pseudopotential (PME or exact) with the density tables, an inverse
//     transform, then the clamp-and-scale step.
//
// Both run on the plan's stream without a host synchronisation: the integral
// is reduced per CTA into the plan's scratch and every CTA of the scaling
// pass re-adds those partials in the same fixed order.
#include <math.h>

#include "plan.h"

namespace {

constexpr int kNormBlocks = 1216;  // 8 CTAs per SM on 152 SMs; <= the 4096-double scratch
constexpr int kNormThreads = 256;

template <typename T>
__global__ void __launch_bounds__(kNormThreads) k_clamp_partial(T* __restrict__ rho, int64_t n, double dtol,
                                                                double* __restrict__ partial) {
  // per-thread sums in the field precision (a handful of elements each; no
  // FP64 instruction per element in the FP32 instantiation), FP64 above
  const T tol = (T)dtol;
  T acc = (T)0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T v = rho[i];
    if (v < tol) {
      v = tol;
      rho[i] = v;
    }
    acc += v;
  }
  __shared__ double red[kNormThreads / 32];
  const double v = warp_sum((double)acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < kNormThreads / 32; ++w) t.add(red[w]);
    partial[blockIdx.x] = t.value();
  }
}

// sum of the per-CTA partials by the whole CTA in a fixed order (thread t
// takes partials t, t + kNormThreads, ...; then warps, then warp results), so
// every CTA that computes it gets the same value
__device__ __forceinline__ double cta_sum_partials(const double* __restrict__ partial, int nblk) {
  __shared__ double red[kNormThreads / 32];
  KSum t;
  t.init();
  for (int b = threadIdx.x; b < nblk; b += kNormThreads) t.add(__ldcg(partial + b));
  const double v = warp_sum(t.value());
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  KSum u;
  u.init();
  for (int w = 0; w < kNormThreads / 32; ++w) u.add(red[w]);
  return u.value();
}

template <typename T>
__global__ void __launch_bounds__(kNormThreads) k_scale_to(T* __restrict__ rho, int64_t n,
                                                           const double* __restrict__ partial, int nblk, double dV,
                                                           double ncharge, double* __restrict__ nc_out) {
  const double nc = cta_sum_partials(partial, nblk) * dV;
  if (nc_out && blockIdx.x == 0 && threadIdx.x == 0) *nc_out = nc;
  const T f = (T)(ncharge > 1e-6 ? ncharge / nc : 1.0);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    rho[i] = rho[i] * f;
}

}  // namespace

extern "C" {

int gbofdft_density_normalize(gbofdft_plan* p, void* rho, double dtol, double ncharge, double* nc_dev,
                              void* stream) {
  GB_REQUIRE(p && rho, "density_normalize: null argument");
  GB_REQUIRE(!isnan(dtol) && !isnan(ncharge), "density_normalize: NaN argument");
  cudaStream_t st = (cudaStream_t)stream;
  double* part = p->scratch;
  if (p->prec == GBOFDFT_F64) {
    k_clamp_partial<double><<<kNormBlocks, kNormThreads, 0, st>>>((double*)rho, p->N, dtol, part);
    GB_CHECK_LAUNCH();
    k_scale_to<double><<<kNormBlocks, kNormThreads, 0, st>>>((double*)rho, p->N, part, kNormBlocks, p->dV, ncharge,
                                                            nc_dev);
  } else {
    k_clamp_partial<float><<<kNormBlocks, kNormThreads, 0, st>>>((float*)rho, p->N, dtol, part);
    GB_CHECK_LAUNCH();
    k_scale_to<float><<<kNormBlocks, kNormThreads, 0, st>>>((float*)rho, p->N, part, kNormBlocks, p->dV, ncharge,
                                                           nc_dev);
  }
  GB_CHECK_LAUNCH();
  return GBOFDFT_OK;
}

int gbofdft_density_guess(gbofdft_plan* p, int nspec, const gbofdft_vtable* tables, int nat, const double* spos_dev,
                          const int* species_dev, int pme, int order, const double* bm_dev, void* work,
                          int64_t work_bytes, void* rho_recip, void* rho, double dtol, double ncharge,
                          void* stream) {
  GB_REQUIRE(p && rho && rho_recip, "density_guess: null argument");
  int rc = gbofdft_vloc(p, nspec, tables, nat, spos_dev, species_dev, pme, order, bm_dev, work, work_bytes,
                        rho_recip, rho, stream);
  if (rc) return rc;
  return gbofdft_density_normalize(p, rho, dtol, ncharge, nullptr, stream);
}

}  // extern "C"
