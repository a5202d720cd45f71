// Set-up kernels on the device: local pseudopotential v_loc(G) and the
// ion-ion (Ewald) energy.  Everything grid-sized runs here; the host only
// prepares 1-D tables (spline coefficients of v(|G|), PME b(m) factors,
// lattice images) and scalars.
//
//   vline(q): cubic spline of the species' v(|G|) table for gp[1] <= q <
//   gp[-1], a quartic through (v2, v1, v0, v1, v2) for q < gp[1], 0 beyond
//   (dftpy LocalPseudo.calc_vlines, functional/pseudo/__init__.py:350-375).
//   PME structure factor: order-p cardinal B-spline charge spreading, FFT,
//   times b0(m0) b1(m1) b2(m2) (ewald.py:11-195, pseudo/__init__.py:389-404).
//   Exact structure factor: sum_a exp(-i G.R_a) (pseudo/__init__.py:377-387)
//   from separable phases exp(-2 pi i m_d s_d).
#include <math.h>
#include <string.h>

#include "pseudo.cuh"

namespace {

// v(G) (+)= vline(|G|) * FFT(Q)(G) * B(G) * scale   (PME, one species)
template <typename T>
__global__ void k_pme_vloc_acc(GInfo g, gbofdft_vtable vt, const cpx<T>* __restrict__ fq,
                               const double2* __restrict__ bm0, const double2* __restrict__ bm1,
                               const double2* __restrict__ bm2, double scale, cpx<T>* __restrict__ v, int first) {
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    int i0, i1, k2;
    decode(g, id, i0, i1, k2);
    const int m0 = ffreq(i0, g.n0), m1 = ffreq(i1, g.n1);
    double vl = vline_eval(vt, sqrt(gg_at(g, m0, m1, m2_of(g, k2))));
    if (needs_sym(g, i0, i1, k2)) {
      const int p0 = ffreq((g.n0 - i0) % g.n0, g.n0), p1 = ffreq((g.n1 - i1) % g.n1, g.n1);
      vl = 0.5 * (vl + vline_eval(vt, sqrt(gg_at(g, p0, p1, m2_partner(g, k2)))));
    }
    const double2 b = bprod(bm0, bm1, bm2, i0, i1, k2);
    const cpx<T> q = fq[id];
    const double s = vl * scale;
    const double vx = ((double)q.x * b.x - (double)q.y * b.y) * s;
    const double vy = ((double)q.x * b.y + (double)q.y * b.x) * s;
    if (first) v[id] = cpx<T>{(T)vx, (T)vy};
    else v[id] = cpx<T>{(T)((double)v[id].x + vx), (T)((double)v[id].y + vy)};
  }
}

// exact structure factor: v(G) = sum_s vline_s(|G|) sum_{a in s} exp(-i G.R_a);
// on partner-averaged points 0.5 (vl S(G) + conj(vl' S(G')))
template <typename T>
__global__ void k_exact_vloc(GInfo g, VTabs vts, const int* __restrict__ species, int nat,
                             const double2* __restrict__ ph0, const double2* __restrict__ ph1,
                             const double2* __restrict__ ph2, const double2* __restrict__ ph2p,
                             cpx<T>* __restrict__ v) {
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    int i0, i1, k2;
    decode(g, id, i0, i1, k2);
    const int m0 = ffreq(i0, g.n0), m1 = ffreq(i1, g.n1);
    const double q = sqrt(gg_at(g, m0, m1, m2_of(g, k2)));
    const bool sym = needs_sym(g, i0, i1, k2);
    const int j0 = (g.n0 - i0) % g.n0, j1 = (g.n1 - i1) % g.n1;
    const double qp = sym ? sqrt(gg_at(g, ffreq(j0, g.n0), ffreq(j1, g.n1), m2_partner(g, k2))) : 0.0;
    double ax = 0.0, ay = 0.0;
    for (int s = 0; s < vts.n; ++s) {
      double sx = 0.0, sy = 0.0, px = 0.0, py = 0.0;
      for (int a = 0; a < nat; ++a) {
        if (species[a] != s) continue;
        const double2 e = phase(ph0, ph1, ph2, g, a, i0, i1, k2);
        sx += e.x; sy += e.y;
        if (sym) {
          const double2 f = phase(ph0, ph1, ph2p, g, a, j0, j1, k2);
          px += f.x; py += f.y;
        }
      }
      const double vl = vline_eval(vts.t[s], q);
      if (sym) {
        const double vlp = vline_eval(vts.t[s], qp);
        ax += 0.5 * (vl * sx + vlp * px);
        ay += 0.5 * (vl * sy - vlp * py);
      } else {
        ax += vl * sx;
        ay += vl * sy;
      }
    }
    v[id] = cpx<T>{(T)ax, (T)ay};
  }
}

// ---- Ewald ---------------------------------------------------------------------
// real-space sum, one CTA per atom i (ewald.py:281-317 / 372-447)
__global__ void k_ewald_real(const double* __restrict__ pos, const double* __restrict__ q, int nat,
                             const double* __restrict__ img, int nimg, double rmax, double seta,
                             double* __restrict__ partial) {
  const int i = blockIdx.x;
  KSum s;
  s.init();
  const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
  const int64_t tot = (int64_t)nimg * nat;
  for (int64_t t = threadIdx.x; t < tot; t += blockDim.x) {
    const int im = (int)(t / nat), j = (int)(t % nat);
    const double dx = xi - (pos[3 * j] - img[3 * im]);
    const double dy = yi - (pos[3 * j + 1] - img[3 * im + 1]);
    const double dz = zi - (pos[3 * j + 2] - img[3 * im + 2]);
    const double d = sqrt(dx * dx + dy * dy + dz * dz);
    if (d < rmax && d > 0.001) s.add(q[j] * erfc(seta * d) / d);
  }
  __shared__ double red[32];
  double v = warp_sum(s.value());
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t.add(red[w]);
    partial[i] = q[i] * t.value();
  }
}

template <int NB>
__device__ __forceinline__ void block_partial(KSum& s, double* partial) {
  __shared__ double red[NB / 32];
  double v = warp_sum(s.value());
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < NB / 32; ++w) t.add(red[w]);
    partial[blockIdx.x] = t.value();
  }
}

// sum over the mask of |S(G)|^2 exp(-G^2/(4 eta)) / G^2, S = FFT(Q) B (ewald.py:786-808)
template <typename T>
__global__ void __launch_bounds__(256) k_ewald_rec_pme(GInfo g, const cpx<T>* __restrict__ fq,
                                                       const double2* __restrict__ bm0, const double2* __restrict__ bm1,
                                                       const double2* __restrict__ bm2, double eta,
                                                       double* __restrict__ partial) {
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  KSum s;
  s.init();
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    int i0, i1, k2;
    decode(g, id, i0, i1, k2);
    if (!gmask(g, i0, i1, k2)) continue;
    const double gg = gg_at(g, ffreq(i0, g.n0), ffreq(i1, g.n1), m2_of(g, k2));
    if (!(gg > 0.0)) continue;
    const double2 b0 = bm0[i0], b1 = bm1[i1], b2 = bm2[k2];
    const double bb = (b0.x * b0.x + b0.y * b0.y) * (b1.x * b1.x + b1.y * b1.y) * (b2.x * b2.x + b2.y * b2.y);
    const cpx<T> q = fq[id];
    s.add(((double)q.x * q.x + (double)q.y * q.y) * bb * exp(-gg / (4.0 * eta)) / gg);
  }
  block_partial<256>(s, partial);
}

// exact reciprocal sum, S(G) = sum_a q_a exp(-i G.R_a) (ewald.py:449-466)
__global__ void __launch_bounds__(256) k_ewald_rec_exact(GInfo g, const double* __restrict__ q, int nat,
                                                         const double2* __restrict__ ph0,
                                                         const double2* __restrict__ ph1,
                                                         const double2* __restrict__ ph2, double eta,
                                                         double* __restrict__ partial) {
  const int64_t total = (int64_t)g.n0 * g.n1 * g.n2h;
  KSum s;
  s.init();
  for (int64_t id = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; id < total;
       id += (int64_t)gridDim.x * blockDim.x) {
    int i0, i1, k2;
    decode(g, id, i0, i1, k2);
    if (!gmask(g, i0, i1, k2)) continue;
    const double gg = gg_at(g, ffreq(i0, g.n0), ffreq(i1, g.n1), m2_of(g, k2));
    if (!(gg > 0.0)) continue;
    double sx = 0.0, sy = 0.0;
    for (int a = 0; a < nat; ++a) {
      const double2 e = phase(ph0, ph1, ph2, g, a, i0, i1, k2);
      sx += q[a] * e.x;
      sy += q[a] * e.y;
    }
    s.add((sx * sx + sy * sy) * exp(-gg / (4.0 * eta)) / gg);
  }
  block_partial<256>(s, partial);
}

__global__ void k_sum_partials(const double* __restrict__ p, int n, double scale, double* __restrict__ out) {
  KSum s;
  s.init();
  for (int i = threadIdx.x; i < n; i += blockDim.x) s.add(p[i]);
  __shared__ double red[8];
  double v = warp_sum(s.value());
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    KSum t;
    t.init();
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t.add(red[w]);
    *out = t.value() * scale;
  }
}

}  // namespace

extern "C" {

int gbofdft_setup_workspace_bytes(const gbofdft_plan* p, int nat, int64_t* bytes) {
  GB_REQUIRE(p && bytes && nat >= 1, "setup_workspace_bytes: bad argument");
  const size_t es = gb_elem(p);
  const size_t pme = round256(es * (size_t)p->N) + round256(2 * es * (size_t)p->NG) + round256(sizeof(double) * 8192);
  const size_t ex = phase_bytes(p, nat) + round256(sizeof(double) * 8192);
  *bytes = (int64_t)(pme > ex ? pme : ex);
  return GBOFDFT_OK;
}

int gbofdft_vloc(gbofdft_plan* p, int nspec, const gbofdft_vtable* tabs, int nat, const double* spos_dev,
                 const int* species_dev, int pme, int order, const double* bm_dev, void* work, int64_t work_bytes,
                 void* vloc_recip, void* vloc_real, void* stream) {
  GB_REQUIRE(p && tabs && spos_dev && species_dev && work && vloc_recip, "vloc: null argument");
  GB_REQUIRE(nspec >= 1 && nspec <= GBOFDFT_MAX_SPECIES && nat >= 1, "vloc: bad sizes (nspec %d, nat %d)", nspec,
             nat);
  int64_t need = 0;
  gbofdft_setup_workspace_bytes(p, nat, &need);
  GB_REQUIRE(work_bytes >= need, "vloc: workspace %lld < %lld bytes", (long long)work_bytes, (long long)need);
  GB_REQUIRE(((uintptr_t)work & 255) == 0, "vloc: workspace must be 256-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  const int nb = grid_blocks(p->NG);
  const bool f64 = p->prec == GBOFDFT_F64;
  if (pme) {
    GB_REQUIRE(bm_dev && order >= 2 && order <= 30, "vloc: PME needs the b(m) table and 2 <= order <= 30");
    const double2* bm = reinterpret_cast<const double2*>(bm_dev);
    const double2 *bm0 = bm, *bm1 = bm + p->n[0], *bm2 = bm + p->n[0] + p->n[1];
    const size_t es = gb_elem(p);
    char* qr = reinterpret_cast<char*>(work);
    char* qg = qr + round256(es * (size_t)p->N);
    const double scale = 1.0 / p->dV;  // fft() carries dV; times N / Omega
    for (int s = 0; s < nspec; ++s) {
      GB_CUDA(cudaMemsetAsync(qr, 0, es * p->N, st));
      if (f64) k_pme_spread<double><<<nat, 256, 0, st>>>(p->gi, spos_dev, nullptr, species_dev, s, order, (double*)qr);
      else k_pme_spread<float><<<nat, 256, 0, st>>>(p->gi, spos_dev, nullptr, species_dev, s, order, (float*)qr);
      GB_CHECK_LAUNCH();
      int rc = gbofdft_fft_r2c(p, qr, qg, stream);
      if (rc) return rc;
      if (f64)
        k_pme_vloc_acc<double><<<nb, 256, 0, st>>>(p->gi, tabs[s], (const double2*)qg, bm0, bm1, bm2, scale,
                                                  (double2*)vloc_recip, s == 0);
      else
        k_pme_vloc_acc<float><<<nb, 256, 0, st>>>(p->gi, tabs[s], (const float2*)qg, bm0, bm1, bm2, scale,
                                                 (float2*)vloc_recip, s == 0);
      GB_CHECK_LAUNCH();
    }
  } else {
    double2 *ph0, *ph1, *ph2, *ph2p;
    phase_tables(p, spos_dev, nat, reinterpret_cast<double2*>(work), st, &ph0, &ph1, &ph2, &ph2p);
    GB_CHECK_LAUNCH();
    VTabs vt;
    memset(&vt, 0, sizeof(vt));
    vt.n = nspec;
    for (int s = 0; s < nspec; ++s) vt.t[s] = tabs[s];
    if (f64)
      k_exact_vloc<double><<<nb, 256, 0, st>>>(p->gi, vt, species_dev, nat, ph0, ph1, ph2, ph2p, (double2*)vloc_recip);
    else
      k_exact_vloc<float><<<nb, 256, 0, st>>>(p->gi, vt, species_dev, nat, ph0, ph1, ph2, ph2p, (float2*)vloc_recip);
    GB_CHECK_LAUNCH();
  }
  if (vloc_real) return gbofdft_fft_c2r(p, vloc_recip, vloc_real, stream);
  return GBOFDFT_OK;
}

int gbofdft_ewald(gbofdft_plan* p, int nat, const double* pos_dev, const double* spos_dev, const double* charges_dev,
                  double eta, double rmax, const double* images_dev, int nimg, int pme, int order, const double* bm_dev,
                  void* work, int64_t work_bytes, double* out_dev, void* stream) {
  GB_REQUIRE(p && pos_dev && spos_dev && charges_dev && images_dev && work && out_dev, "ewald: null argument");
  GB_REQUIRE(nat >= 1 && nimg >= 1 && eta > 0.0, "ewald: bad arguments");
  int64_t need = 0;
  gbofdft_setup_workspace_bytes(p, nat, &need);
  GB_REQUIRE(work_bytes >= need, "ewald: workspace %lld < %lld bytes", (long long)work_bytes, (long long)need);
  GB_REQUIRE(((uintptr_t)work & 255) == 0, "ewald: workspace must be 256-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t es = gb_elem(p);
  char* base = reinterpret_cast<char*>(work);
  double* partial;
  // real space
  {
    size_t off = pme ? round256(es * (size_t)p->N) + round256(2 * es * (size_t)p->NG) : phase_bytes(p, nat);
    partial = reinterpret_cast<double*>(base + off);
    GB_REQUIRE(nat <= 8192, "ewald: at most 8192 atoms");
    k_ewald_real<<<nat, 256, 0, st>>>(pos_dev, charges_dev, nat, images_dev, nimg, rmax, sqrt(eta), partial);
    GB_CHECK_LAUNCH();
    k_sum_partials<<<1, 256, 0, st>>>(partial, nat, 0.5, out_dev + 0);
    GB_CHECK_LAUNCH();
  }
  const int nb = grid_blocks(p->NG) > 2048 ? 2048 : grid_blocks(p->NG);
  if (pme) {
    GB_REQUIRE(bm_dev && order >= 2 && order <= 30, "ewald: PME needs the b(m) table");
    char* qr = base;
    char* qg = qr + round256(es * (size_t)p->N);
    GB_CUDA(cudaMemsetAsync(qr, 0, es * p->N, st));
    if (p->prec == GBOFDFT_F64)
      k_pme_spread<double><<<nat, 256, 0, st>>>(p->gi, spos_dev, charges_dev, nullptr, 0, order, (double*)qr);
    else
      k_pme_spread<float><<<nat, 256, 0, st>>>(p->gi, spos_dev, charges_dev, nullptr, 0, order, (float*)qr);
    GB_CHECK_LAUNCH();
    int rc = gbofdft_fft_r2c(p, qr, qg, stream);
    if (rc) return rc;
    const double2* bm = reinterpret_cast<const double2*>(bm_dev);
    if (p->prec == GBOFDFT_F64)
      k_ewald_rec_pme<double><<<nb, 256, 0, st>>>(p->gi, (const double2*)qg, bm, bm + p->n[0], bm + p->n[0] + p->n[1],
                                                 eta, partial);
    else
      k_ewald_rec_pme<float><<<nb, 256, 0, st>>>(p->gi, (const float2*)qg, bm, bm + p->n[0], bm + p->n[0] + p->n[1],
                                                eta, partial);
    GB_CHECK_LAUNCH();
    // 4 pi / Omega / dV^2 (fft carries dV)
    k_sum_partials<<<1, 256, 0, st>>>(partial, nb, 4.0 * 3.14159265358979323846 / p->volume / (p->dV * p->dV),
                                      out_dev + 1);
  } else {
    double2 *ph0, *ph1, *ph2, *ph2p;
    phase_tables(p, spos_dev, nat, reinterpret_cast<double2*>(base), st, &ph0, &ph1, &ph2, &ph2p);
    GB_CHECK_LAUNCH();
    k_ewald_rec_exact<<<nb, 256, 0, st>>>(p->gi, charges_dev, nat, ph0, ph1, ph2, eta, partial);
    GB_CHECK_LAUNCH();
    k_sum_partials<<<1, 256, 0, st>>>(partial, nb, 4.0 * 3.14159265358979323846 / p->volume, out_dev + 1);
  }
  GB_CHECK_LAUNCH();
  return GBOFDFT_OK;
}

}  // extern "C"
