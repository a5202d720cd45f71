// Forces on the ions from the local pseudopotential and the Ewald sum.
//
//   PME local PP (LocalPseudo._ForcePME, pseudo/__init__.py:475-523):
//     per species s: phi_s = ifft(rhoG conj(B) vline_s, G=0 -> 0); each atom
//     of s gathers phi_s over its order^3 B-spline support with the
//     derivative weights QD_d, F_a = -(QD^T phi) cell_inv.
//   exact local PP (LocalPseudo._Force, :457-473):
//     F_a = 2/Omega sum_{G in mask} G vline_s(|G|) Im(rhoG exp(+i G.R_a)).
//   Ewald real space (ewald.py:541-575): pair/image sum, one CTA per atom.
//   Ewald PME reciprocal (Forces_rec_PME, ewald.py:810-857):
//     phi = ifft(FFT(Q) |B|^2 exp(-G^2/4eta)/G^2); F_a -= q_a 4 pi/dV (QD^T phi) cell_inv.
//   Ewald exact reciprocal (Forces_rec, ewald.py:578-604):
//     F_a = 8 pi/Omega sum_{G in mask} G (Re(s_a) Im(S) - Im(s_a) Re(S)) exp(-G^2/4eta)/G^2,
//     s_a = q_a exp(-i G.R_a), S = sum_a s_a.
//
// Grid-sized work (field construction, FFTs) runs on the whole device; the
// per-atom gathers and sums are one CTA per atom with a fixed-order
// reduction, so the forces are bitwise reproducible run to run.
#include <math.h>
#include <string.h>

#include "gkernels.cuh"
#include "pseudo.cuh"

namespace {

// mode 0: out = rhoG conj(B) vline(|G|)              (G = 0 -> 0)
// mode 1: out = Q(G) |B|^2 exp(-G^2/(4 eta)) / G^2   (G = 0 -> 0)
// The G-dependent factor is evaluated in the Nyquist-partner-averaged form
// (gbk::sym_kernel), which is what the real part of the reference's inverse
// transform of the full array sees.
template <typename T>
__global__ void k_force_field(GInfo g, int mode, const cpx<T>* __restrict__ in, const double2* __restrict__ bm0,
                              const double2* __restrict__ bm1, const double2* __restrict__ bm2, gbofdft_vtable vt,
                              double eta, cpx<T>* __restrict__ out) {
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    int i0, i1, k2;
    decode(g, id, i0, i1, k2);
    if (id == 0) { out[0] = cpx<T>{(T)0, (T)0}; continue; }
    const double2 b = bprod(bm0, bm1, bm2, i0, i1, k2);
    const cpx<T> v = in[id];
    if (mode == 0) {
      const double kv = gbk::sym_kernel<double>(g, i0, i1, k2, [&](double gg) { return vline_eval(vt, sqrt(gg)); });
      out[id] = cpx<T>{(T)(((double)v.x * b.x + (double)v.y * b.y) * kv),
                       (T)(((double)v.y * b.x - (double)v.x * b.y) * kv)};
    } else {
      const double kv = gbk::sym_kernel<double>(
          g, i0, i1, k2, [&](double gg) { return gg > 0.0 ? exp(-gg / (4.0 * eta)) / gg : 0.0; });
      const double bb = (b.x * b.x + b.y * b.y) * kv;
      out[id] = cpx<T>{(T)((double)v.x * bb), (T)((double)v.y * bb)};
    }
  }
}

struct Mat3 {
  double m[9];  // row-major, cell_inv = inv(lattice)
};

__device__ __forceinline__ void block_sum3(double& a0, double& a1, double& a2, double s[3]) {
  __shared__ double red[3][32];
  a0 = warp_sum(a0);
  a1 = warp_sum(a1);
  a2 = warp_sum(a2);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][w] = a0; red[1][w] = a1; red[2][w] = a2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    s[0] = s[1] = s[2] = 0.0;
    for (int ww = 0; ww < (int)(blockDim.x >> 5); ++ww)
      for (int d = 0; d < 3; ++d) s[d] += red[d][ww];
  }
}

// One CTA per atom a of species `want` (all atoms if species is null):
//   acc_d = sum_support QD_d(i,j,k) phi(l(i,j,k)),  F_a (+)= scale w_a (acc^T cell_inv)
template <typename T>
__global__ void k_force_gather(GInfo g, const double* __restrict__ spos, const int* __restrict__ species, int want,
                               int order, const T* __restrict__ phi, const double* __restrict__ w, double scale,
                               Mat3 ci, double* __restrict__ F) {
  const int a = blockIdx.x;
  if (species && species[a] != want) return;
  __shared__ double M[3][32], dM[3][32];
  __shared__ int fl[3];
  if (threadIdx.x < 3) {
    const int d = threadIdx.x;
    const int n = d == 0 ? g.n0 : (d == 1 ? g.n1 : g.n2);
    const double u = spos[3 * a + d] * n;
    const double f = floor(u);
    bspline_weights(u - f, order, n, M[d], dM[d]);
    fl[d] = (int)f;
  }
  __syncthreads();
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  const int o3 = order * order * order;
  for (int t = threadIdx.x; t < o3; t += blockDim.x) {
    const int i = t / (order * order), j = (t / order) % order, k = t % order;
    int l0 = (1 + fl[0] - i) % g.n0; if (l0 < 0) l0 += g.n0;
    int l1 = (1 + fl[1] - j) % g.n1; if (l1 < 0) l1 += g.n1;
    int l2 = (1 + fl[2] - k) % g.n2; if (l2 < 0) l2 += g.n2;
    const double v = (double)phi[((int64_t)l0 * g.n1 + l1) * g.n2 + l2];
    a0 += dM[0][i] * M[1][j] * M[2][k] * v;
    a1 += M[0][i] * dM[1][j] * M[2][k] * v;
    a2 += M[0][i] * M[1][j] * dM[2][k] * v;
  }
  double s[3];
  block_sum3(a0, a1, a2, s);
  if (threadIdx.x == 0) {
    const double sc = scale * (w ? w[a] : 1.0);
    for (int c = 0; c < 3; ++c) F[3 * a + c] += sc * (s[0] * ci.m[c] + s[1] * ci.m[3 + c] + s[2] * ci.m[6 + c]);
  }
}

// Ewald real-space forces, one CTA per atom i (ewald.py:541-575)
__global__ void k_ewald_real_forces(const double* __restrict__ pos, const double* __restrict__ q, int nat,
                                    const double* __restrict__ img, int nimg, double rmax, double seta,
                                    double* __restrict__ F) {
  const int i = blockIdx.x;
  const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
  const double c2 = 2.0 / sqrt(3.14159265358979323846);
  double f0 = 0.0, f1 = 0.0, f2 = 0.0;
  const int64_t tot = (int64_t)nimg * nat;
  for (int64_t t = threadIdx.x; t < tot; t += blockDim.x) {
    const int im = (int)(t / nat), j = (int)(t % nat);
    const double dx = xi - (pos[3 * j] - img[3 * im]);
    const double dy = yi - (pos[3 * j + 1] - img[3 * im + 1]);
    const double dz = zi - (pos[3 * j + 2] - img[3 * im + 2]);
    const double d = sqrt(dx * dx + dy * dy + dz * dz);
    if (!(d < rmax && d > 0.001)) continue;
    const double x = d * seta;
    const double wgt = q[j] * (erfc(x) / (x * x * x) + c2 * exp(-x * x) / (x * x));
    f0 += dx * wgt;
    f1 += dy * wgt;
    f2 += dz * wgt;
  }
  double s[3];
  block_sum3(f0, f1, f2, s);
  if (threadIdx.x == 0) {
    const double sc = q[i] * seta * seta * seta;
    F[3 * i] = s[0] * sc;
    F[3 * i + 1] = s[1] * sc;
    F[3 * i + 2] = s[2] * sc;
  }
}

// S(G) = sum_a q_a exp(-i G.R_a) on the stored half spectrum
__global__ void k_strf(GInfo g, const double* __restrict__ q, int nat, const double2* __restrict__ ph0,
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

// Exact-structure-factor forces over the reference half-space mask.  Grid
// (nblk, nat): CTA (b, a) sums its stride of G for atom a into
// partial[a][b][3]; k_force_partials reduces the blocks in a fixed order.
//   mode 0: w = vline_{s(a)}(|G|) Im(rhoG conj(e_a))
//   mode 1: w = q_a (Re(e_a) Im(S) - Im(e_a) Re(S)) exp(-G^2/4eta)/G^2
template <typename T>
__global__ void k_exact_forces(GInfo g, int mode, const double2* __restrict__ ph0, const double2* __restrict__ ph1,
                               const double2* __restrict__ ph2, const cpx<T>* __restrict__ rhoG, VTabs vts,
                               const int* __restrict__ species, const double2* __restrict__ S,
                               const double* __restrict__ q, double eta, double* __restrict__ partial) {
  const int a = blockIdx.y;
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  const int sp = mode == 0 ? species[a] : 0;
  double f0 = 0.0, f1 = 0.0, f2 = 0.0;
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
    const double2 e = phase(ph0, ph1, ph2, g, a, i0, i1, k2);
    double w;
    if (mode == 0) {
      const cpx<T> r = rhoG[id];
      w = vline_eval(vts.t[sp], sqrt(gg)) * ((double)r.y * e.x - (double)r.x * e.y);
    } else {
      if (!(gg > 0.0)) continue;
      const double2 s = S[id];
      w = q[a] * (e.x * s.y - e.y * s.x) * exp(-gg / (4.0 * eta)) / gg;
    }
    f0 += gx * w;
    f1 += gy * w;
    f2 += gz * w;
  }
  double s[3];
  block_sum3(f0, f1, f2, s);
  if (threadIdx.x == 0) {
    double* o = partial + ((int64_t)a * gridDim.x + blockIdx.x) * 3;
    o[0] = s[0];
    o[1] = s[1];
    o[2] = s[2];
  }
}

__global__ void k_force_partials(const double* __restrict__ partial, int nblk, double scale, double* __restrict__ F) {
  const int a = blockIdx.x;
  if (threadIdx.x < 3) {
    KSum s;
    s.init();
    for (int b = 0; b < nblk; ++b) s.add(partial[((int64_t)a * nblk + b) * 3 + threadIdx.x]);
    F[3 * a + threadIdx.x] += s.value() * scale;
  }
}

constexpr int kExactBlocks = 128;  // G-blocks per atom in the exact sums

Mat3 cell_inverse(const gbofdft_plan* p) {
  // inv(lattice) = bg^T / (2 pi)
  Mat3 c;
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) c.m[r * 3 + k] = p->bg[k * 3 + r] / 6.283185307179586476925286766559;
  return c;
}

size_t exact_bytes(const gbofdft_plan* p, int nat) {
  return round256(2 * gb_elem(p) * (size_t)p->NG) + round256(sizeof(double2) * (size_t)p->NG) +
         phase_bytes(p, nat) + round256(sizeof(double) * 3 * (size_t)nat * kExactBlocks);
}

size_t pme_bytes(const gbofdft_plan* p) {
  return 2 * round256(2 * gb_elem(p) * (size_t)p->NG) + round256(gb_elem(p) * (size_t)p->N);
}

}  // namespace

extern "C" {

int gbofdft_forces_workspace_bytes(const gbofdft_plan* p, int nat, int64_t* bytes) {
  GB_REQUIRE(p && bytes && nat >= 1, "forces_workspace_bytes: bad argument");
  const size_t a = pme_bytes(p), b = exact_bytes(p, nat);
  *bytes = (int64_t)(a > b ? a : b);
  return GBOFDFT_OK;
}

int gbofdft_pp_forces(gbofdft_plan* p, const void* rho, int nspec, const gbofdft_vtable* tabs, int nat,
                      const double* spos_dev, const int* species_dev, int pme, int order, const double* bm_dev,
                      void* work, int64_t work_bytes, double* forces_dev, void* stream) {
  GB_REQUIRE(p && rho && tabs && spos_dev && species_dev && work && forces_dev, "pp_forces: null argument");
  GB_REQUIRE(nspec >= 1 && nspec <= GBOFDFT_MAX_SPECIES && nat >= 1 && nat <= 65535,
             "pp_forces: bad sizes (nspec %d, nat %d)", nspec, nat);
  int64_t need = 0;
  gbofdft_forces_workspace_bytes(p, nat, &need);
  GB_REQUIRE(work_bytes >= need, "pp_forces: workspace %lld < %lld bytes", (long long)work_bytes, (long long)need);
  GB_REQUIRE(((uintptr_t)work & 255) == 0, "pp_forces: workspace must be 256-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t es = gb_elem(p);
  const bool f64 = p->prec == GBOFDFT_F64;
  char* base = reinterpret_cast<char*>(work);
  char* rhoG = base;
  char* next = base + round256(2 * es * (size_t)p->NG);
  int rc = gbofdft_fft_r2c(p, rho, rhoG, stream);
  if (rc) return rc;
  GB_CUDA(cudaMemsetAsync(forces_dev, 0, sizeof(double) * 3 * nat, st));
  if (pme) {
    GB_REQUIRE(bm_dev && order >= 2 && order <= 30, "pp_forces: PME needs the b(m) table and 2 <= order <= 30");
    const double2* bm = reinterpret_cast<const double2*>(bm_dev);
    const double2 *bm0 = bm, *bm1 = bm + p->n[0], *bm2 = bm + p->n[0] + p->n[1];
    char* fg = next;
    char* phi = fg + round256(2 * es * (size_t)p->NG);
    const Mat3 ci = cell_inverse(p);
    const int nb = grid_blocks(p->NG);
    for (int s = 0; s < nspec; ++s) {
      if (f64)
        k_force_field<double><<<nb, 256, 0, st>>>(p->gi, 0, (const double2*)rhoG, bm0, bm1, bm2, tabs[s], 0.0,
                                                 (double2*)fg);
      else
        k_force_field<float><<<nb, 256, 0, st>>>(p->gi, 0, (const float2*)rhoG, bm0, bm1, bm2, tabs[s], 0.0,
                                                (float2*)fg);
      GB_CHECK_LAUNCH();
      if ((rc = gbofdft_fft_c2r(p, fg, phi, stream))) return rc;
      // fft() carries dV and ifft() divides by it: phi is the reference's rhoPB
      if (f64)
        k_force_gather<double><<<nat, 256, 0, st>>>(p->gi, spos_dev, species_dev, s, order, (const double*)phi,
                                                   nullptr, -1.0, ci, forces_dev);
      else
        k_force_gather<float><<<nat, 256, 0, st>>>(p->gi, spos_dev, species_dev, s, order, (const float*)phi,
                                                  nullptr, -1.0, ci, forces_dev);
      GB_CHECK_LAUNCH();
    }
  } else {
    double2* S = reinterpret_cast<double2*>(next);  // unused by the PP sum
    char* phb = next + round256(sizeof(double2) * (size_t)p->NG);
    double* partial = reinterpret_cast<double*>(phb + phase_bytes(p, nat));
    double2 *ph0, *ph1, *ph2, *ph2p;
    phase_tables(p, spos_dev, nat, reinterpret_cast<double2*>(phb), st, &ph0, &ph1, &ph2, &ph2p);
    GB_CHECK_LAUNCH();
    VTabs vt;
    memset(&vt, 0, sizeof(vt));
    vt.n = nspec;
    for (int s = 0; s < nspec; ++s) vt.t[s] = tabs[s];
    const dim3 grid(kExactBlocks, nat);
    if (f64)
      k_exact_forces<double><<<grid, 256, 0, st>>>(p->gi, 0, ph0, ph1, ph2, (const double2*)rhoG, vt, species_dev, S,
                                                  nullptr, 0.0, partial);
    else
      k_exact_forces<float><<<grid, 256, 0, st>>>(p->gi, 0, ph0, ph1, ph2, (const float2*)rhoG, vt, species_dev, S,
                                                 nullptr, 0.0, partial);
    GB_CHECK_LAUNCH();
    k_force_partials<<<nat, 32, 0, st>>>(partial, kExactBlocks, 2.0 / p->volume, forces_dev);
    GB_CHECK_LAUNCH();
  }
  return GBOFDFT_OK;
}

int gbofdft_ewald_forces(gbofdft_plan* p, int nat, const double* pos_dev, const double* spos_dev,
                         const double* charges_dev, double eta, double rmax, const double* images_dev, int nimg,
                         int pme, int order, const double* bm_dev, void* work, int64_t work_bytes, double* forces_dev,
                         void* stream) {
  GB_REQUIRE(p && pos_dev && spos_dev && charges_dev && images_dev && work && forces_dev,
             "ewald_forces: null argument");
  GB_REQUIRE(nat >= 1 && nat <= 65535 && nimg >= 1 && eta > 0.0, "ewald_forces: bad arguments");
  int64_t need = 0;
  gbofdft_forces_workspace_bytes(p, nat, &need);
  GB_REQUIRE(work_bytes >= need, "ewald_forces: workspace %lld < %lld bytes", (long long)work_bytes,
             (long long)need);
  GB_REQUIRE(((uintptr_t)work & 255) == 0, "ewald_forces: workspace must be 256-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t es = gb_elem(p);
  const bool f64 = p->prec == GBOFDFT_F64;
  char* base = reinterpret_cast<char*>(work);
  k_ewald_real_forces<<<nat, 256, 0, st>>>(pos_dev, charges_dev, nat, images_dev, nimg, rmax, sqrt(eta),
                                           forces_dev);
  GB_CHECK_LAUNCH();
  int rc;
  if (pme) {
    GB_REQUIRE(bm_dev && order >= 2 && order <= 30, "ewald_forces: PME needs the b(m) table and 2 <= order <= 30");
    const double2* bm = reinterpret_cast<const double2*>(bm_dev);
    const double2 *bm0 = bm, *bm1 = bm + p->n[0], *bm2 = bm + p->n[0] + p->n[1];
    char* qg = base;
    char* fg = qg + round256(2 * es * (size_t)p->NG);
    char* qr = fg + round256(2 * es * (size_t)p->NG);  // Q, then phi
    GB_CUDA(cudaMemsetAsync(qr, 0, es * p->N, st));
    if (f64) k_pme_spread<double><<<nat, 256, 0, st>>>(p->gi, spos_dev, charges_dev, nullptr, 0, order, (double*)qr);
    else k_pme_spread<float><<<nat, 256, 0, st>>>(p->gi, spos_dev, charges_dev, nullptr, 0, order, (float*)qr);
    GB_CHECK_LAUNCH();
    if ((rc = gbofdft_fft_r2c(p, qr, qg, stream))) return rc;
    gbofdft_vtable none;
    memset(&none, 0, sizeof(none));
    const int nb = grid_blocks(p->NG);
    if (f64)
      k_force_field<double><<<nb, 256, 0, st>>>(p->gi, 1, (const double2*)qg, bm0, bm1, bm2, none, eta, (double2*)fg);
    else
      k_force_field<float><<<nb, 256, 0, st>>>(p->gi, 1, (const float2*)qg, bm0, bm1, bm2, none, eta, (float2*)fg);
    GB_CHECK_LAUNCH();
    if ((rc = gbofdft_fft_c2r(p, fg, qr, stream))) return rc;
    const Mat3 ci = cell_inverse(p);
    const double scale = -4.0 * 3.14159265358979323846 / p->dV;
    if (f64)
      k_force_gather<double><<<nat, 256, 0, st>>>(p->gi, spos_dev, nullptr, 0, order, (const double*)qr, charges_dev,
                                                 scale, ci, forces_dev);
    else
      k_force_gather<float><<<nat, 256, 0, st>>>(p->gi, spos_dev, nullptr, 0, order, (const float*)qr, charges_dev,
                                                scale, ci, forces_dev);
    GB_CHECK_LAUNCH();
  } else {
    char* Sb = base + round256(2 * es * (size_t)p->NG);
    double2* S = reinterpret_cast<double2*>(Sb);
    char* phb = Sb + round256(sizeof(double2) * (size_t)p->NG);
    double* partial = reinterpret_cast<double*>(phb + phase_bytes(p, nat));
    double2 *ph0, *ph1, *ph2, *ph2p;
    phase_tables(p, spos_dev, nat, reinterpret_cast<double2*>(phb), st, &ph0, &ph1, &ph2, &ph2p);
    GB_CHECK_LAUNCH();
    k_strf<<<grid_blocks(p->NG), 256, 0, st>>>(p->gi, charges_dev, nat, ph0, ph1, ph2, S);
    GB_CHECK_LAUNCH();
    VTabs none;
    memset(&none, 0, sizeof(none));
    const dim3 grid(kExactBlocks, nat);
    k_exact_forces<double><<<grid, 256, 0, st>>>(p->gi, 1, ph0, ph1, ph2, nullptr, none, nullptr, S, charges_dev, eta,
                                                partial);
    GB_CHECK_LAUNCH();
    k_force_partials<<<nat, 32, 0, st>>>(partial, kExactBlocks, 8.0 * 3.14159265358979323846 / p->volume,
                                         forces_dev);
    GB_CHECK_LAUNCH();
  }
  return GBOFDFT_OK;
}

}  // extern "C"
