// Plane convolution pass: for one spectrum field and one k2, the whole
// (n0 x n1) plane is held in shared memory and transformed forward along
// axis 1 and axis 0, multiplied by the reciprocal-space kernel and
// transformed back -- the three column passes of the evaluation pipeline in
// one launch, with one read and one write of each spectrum.
//
// Spectra are plane-major here: element (i0, i1, k2) of field f sits at
//   spec[f * fstride + (k2 * n0 + i0) * n1 + i1]
// so a plane is one contiguous block; the row passes read and write that
// layout (PM instantiations of k_ct_rows_fwd / k_ct_rows_inv_eval).
//
// The FFT stages run in place in the plane buffer: every thread loads the
// inputs of its butterflies (and twiddles them) into registers, the CTA
// synchronises, and the outputs are written over the inputs.  A Stockham
// stage is a permutation of whole lines, so reading everything before
// writing anything makes in-place exactly the ping-pong result.  Lines are
// processed in chunks so that a thread holds at most GB_PLANE_REGS complex
// values (16: no register spills at 512 threads for every specialised size).
//
// The plane uses the XOR-swizzled line-major layout of fft_ct.cuh with lines
// = rows i0 (elements i1): axis-1 stages walk along a line, axis-0 stages
// map consecutive threads to consecutive columns i1, so both access
// patterns are free of bank conflicts.
#pragma once

namespace gbct {

#ifndef GB_PLANE_THREADS
#define GB_PLANE_THREADS 512       // threads per plane CTA
#endif
#ifndef GB_PLANE_THREADS_128
#define GB_PLANE_THREADS_128 1024  // ... for 128 x 128 planes (measured best; 64 registers)
#endif
#ifndef GB_PLANE_REGS
#define GB_PLANE_REGS 16
#endif
#ifndef GB_PLANE_R16
#define GB_PLANE_R16 1      // 128-point plane transforms as 16 x 8 (else 8 x 4 x 4)
#endif
constexpr int kPlaneRegs = GB_PLANE_REGS;   // complex values a thread holds in one stage

template <int N0, int N1> struct PlaneCfg {
  static constexpr int NT = (N0 == 128 && N1 == 128) ? GB_PLANE_THREADS_128 : GB_PLANE_THREADS;
  static constexpr int NP1 = Pad<float, N1>::NP;
  static constexpr size_t kPlaneBytes = sizeof(float2) * (size_t)N0 * NP1;
  static constexpr size_t kSmall = sizeof(float2) * (N0 + N1) + sizeof(float) * 3 * (N0 + N1);
  static constexpr size_t kTable = sizeof(float) * (size_t)N0 * N1;
  // the kernel table's plane is staged in shared memory (asynchronous copy
  // overlapped with the forward transforms) when it fits beside the plane
  static constexpr bool table_smem = kPlaneBytes + kTable + kSmall <= 227 * 1024 && (N0 * N1) % 4 == 0;
  static constexpr size_t kSmem = kPlaneBytes + (table_smem ? kTable : 0) + kSmall;
  static constexpr bool fits = kSmem <= 227 * 1024;
  // transform-only plane kernels (no kernel table, no G tables): plane + twiddles
  static constexpr size_t kSmemXform = kPlaneBytes + sizeof(float2) * (N0 + N1);
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// smallest number of line chunks (a divisor of NL) with at most kPlaneRegs
// complex values per thread in a radix-R stage
template <int NL, int NB, int R, int NT>
constexpr int plane_chunks() {
  for (int c = 1; c <= NL; ++c) {
    if (NL % c) continue;
    const int per = (NL / c) * NB;
    const int iters = (per + NT - 1) / NT;
    if (iters * R <= kPlaneRegs) return c;
  }
  return NL;
}

// radix schedules of the plane transforms (every stage is a full read and
// write of the plane, so fewer, larger stages are usually better).  V selects
// a variant where there is more than one: for 128, V = 0 is 16 x 8 and V = 1
// is the line passes' 8 x 4 x 4 (the autotuner times both).
template <int N, int V> struct PlaneSched { using S = typename Plan<N>::S; };
#if GB_PLANE_R16
template <> struct PlaneSched<128, 0> { using S = Sched<16, 8>; };
#endif
template <int N0, int N1> constexpr int plane_variants() { return (N0 == 128 || N1 == 128) ? 2 : 1; }

template <int N1>
__device__ __forceinline__ int paddr(int i0, int i1) {
  return sw<float, Pad<float, N1>::NP>(i0, i1);
}

// Stage modes: in place in shared memory, inputs read straight from the
// plane in global memory (the first stage of the first transform), or
// outputs written straight to global memory (the last stage of the last
// transform) -- each saves one pass over the shared plane.
enum { PS_SMEM = 0, PS_FROM_GLOBAL = 1, PS_TO_GLOBAL = 2 };

struct PsIdentity {
  __device__ __forceinline__ float2 operator()(int, int, float2 v) const { return v; }
};

// One in-place Stockham stage (radix R, stride P) of every line along axis
// AX (1: lines are rows i0, elements i1; 0: lines are columns i1, elements i0).
// outf(j, l, v) is applied to every output (element j of line l) before it
// is stored.
template <int DIR, int AX, int N0, int N1, int R, int P, int MODE, typename OUTF>
__device__ __forceinline__ void pstage(float2* __restrict__ pl, const float2* __restrict__ tw,
                                       const float2* __restrict__ gsrc, float2* __restrict__ gdst, OUTF outf) {
  constexpr int N = AX == 1 ? N1 : N0;
  constexpr int NL = AX == 1 ? N0 : N1;
  constexpr int NB = N / R;
  constexpr int TWS = N / (P * R);
  constexpr int NT = PlaneCfg<N0, N1>::NT;
  constexpr int CH = plane_chunks<NL, NB, R, NT>();
  constexpr int LC = NL / CH;
  constexpr int PER = LC * NB;
  constexpr int IT = (PER + NT - 1) / NT;
  static_assert(MODE == PS_SMEM || AX == 1, "global operands are rows of the plane");
  const int tid = threadIdx.x;
#pragma unroll 1
  for (int c0 = 0; c0 < NL; c0 += LC) {
    float2 u[IT][R];
    int lo[IT], jo[IT];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
      const int b = tid + it * NT;
      lo[it] = -1;
      if ((PER % NT) != 0 && b >= PER) continue;
      int l, i;
      if constexpr (AX == 1) { l = c0 + b / NB; i = b % NB; }
      else { l = c0 + b % LC; i = b / LC; }
      const int k = (P == 1) ? 0 : i % P;
#pragma unroll
      for (int t = 0; t < R; ++t) {
        const int j = i + t * NB;
        float2 v;
        if constexpr (MODE == PS_FROM_GLOBAL) v = gsrc[l * N1 + j];
        else v = AX == 1 ? pl[paddr<N1>(l, j)] : pl[paddr<N1>(j, l)];
        if (P > 1 && t > 0) {
          const float2 w = tw[t * k * TWS];
          v = DIR < 0 ? c_mul(v, w) : c_mulc(v, w);
        }
        u[it][t] = v;
      }
      dft<DIR, float, R>(u[it]);
      lo[it] = l;
      jo[it] = (i - k) * R + k;
    }
    if constexpr (MODE == PS_SMEM) __syncthreads();
#pragma unroll
    for (int it = 0; it < IT; ++it) {
      if (lo[it] < 0) continue;
#pragma unroll
      for (int t = 0; t < R; ++t) {
        const int j = jo[it] + t * P;
        const float2 v = outf(j, lo[it], u[it][t]);
        if constexpr (MODE == PS_TO_GLOBAL) gdst[lo[it] * N1 + j] = v;
        else if constexpr (AX == 1) pl[paddr<N1>(lo[it], j)] = v;
        else pl[paddr<N1>(j, lo[it])] = v;
      }
    }
  }
  if constexpr (MODE != PS_TO_GLOBAL) __syncthreads();
}

template <int DIR, int AX, int N0, int N1, int P, int FIRST, int LAST, typename OUTF, int R0, int... Rs>
__device__ __forceinline__ void prun(float2* pl, const float2* tw, const float2* gsrc, float2* gdst, OUTF outf) {
  constexpr bool last = sizeof...(Rs) == 0;
  constexpr int mode = (P == 1 && FIRST == PS_FROM_GLOBAL) ? PS_FROM_GLOBAL : (last ? LAST : PS_SMEM);
  static_assert(!(P == 1 && last && FIRST != PS_SMEM && LAST != PS_SMEM), "single-stage schedule");
  if constexpr (last) {
    pstage<DIR, AX, N0, N1, R0, P, mode>(pl, tw, gsrc, gdst, outf);
  } else {
    pstage<DIR, AX, N0, N1, R0, P, mode>(pl, tw, gsrc, gdst, PsIdentity{});
    prun<DIR, AX, N0, N1, P * R0, FIRST, LAST, OUTF, Rs...>(pl, tw, gsrc, gdst, outf);
  }
}

template <int DIR, int AX, int N0, int N1, int FIRST, int LAST, typename OUTF, int... Rs>
__device__ __forceinline__ void prun_sched(Sched<Rs...>, float2* pl, const float2* tw, const float2* gsrc,
                                           float2* gdst, OUTF outf) {
  prun<DIR, AX, N0, N1, 1, FIRST, LAST, OUTF, Rs...>(pl, tw, gsrc, gdst, outf);
}

// whole-plane 1-D transforms along one axis; FIRST / LAST select where the
// first stage reads and the last stage writes, outf post-processes the last
// stage's outputs
template <int DIR, int AX, int N0, int N1, int V, int FIRST = PS_SMEM, int LAST = PS_SMEM,
          typename OUTF = PsIdentity>
__device__ __forceinline__ void plane_fft(float2* pl, const float2* tw, const float2* gsrc = nullptr,
                                          float2* gdst = nullptr, OUTF outf = OUTF{}) {
  prun_sched<DIR, AX, N0, N1, FIRST, LAST>(typename PlaneSched<AX == 1 ? N1 : N0, V>::S{}, pl, tw, gsrc, gdst, outf);
}

struct PlaneArgs {
  float2* spec;
  int64_t fstride;
  const void* tw0;
  const void* tw1;
  GInfo gi;
  float bgf[9];         // reciprocal lattice rows in FP32
  int type[GB_MAX_FIELDS];
  const float* arr[GB_MAX_FIELDS];   // plane-major kernel tables (KER_ARRAY)
  float coef[GB_MAX_FIELDS];
};

template <int N0, int N1, int V>
__global__ void __launch_bounds__(PlaneCfg<N0, N1>::NT, 1) k_plane_conv(PlaneArgs a) {
  constexpr int kPlaneThreads = PlaneCfg<N0, N1>::NT;
  constexpr int NP1 = Pad<float, N1>::NP;
  using Cfg = PlaneCfg<N0, N1>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* pl = reinterpret_cast<float2*>(smem_raw);
  float* ktab = reinterpret_cast<float*>(smem_raw + Cfg::kPlaneBytes);      // [N0 * N1] when staged
  float2* tw0 = reinterpret_cast<float2*>(smem_raw + Cfg::kPlaneBytes + (Cfg::table_smem ? Cfg::kTable : 0));
  float2* tw1 = tw0 + N0;
  float* gA = reinterpret_cast<float*>(tw1 + N1);   // [3][N0]: m0 b0 + m2 b2
  float* gB = gA + 3 * N0;                          // [3][N1]: m1 b1
  const int tid = threadIdx.x;
  const int k2 = blockIdx.x, f = blockIdx.y;
  const GInfo& g = a.gi;
  float2* gp = a.spec + f * a.fstride + (int64_t)k2 * (N0 * N1);
  const int type = a.type[f];
  const float* karr = a.arr[f] ? a.arr[f] + (int64_t)k2 * (N0 * N1) : nullptr;
  if constexpr (Cfg::table_smem) {
    // start the table plane's copy; it completes behind the forward transforms
    if (type == KER_ARRAY) {
      for (int idx = tid; idx < N0 * N1 / 4; idx += kPlaneThreads) cp_async16(ktab + 4 * idx, karr + 4 * idx);
    }
    cp_async_commit();
  }
  const float2* t0 = reinterpret_cast<const float2*>(a.tw0);
  const float2* t1 = reinterpret_cast<const float2*>(a.tw1);
  for (int i = tid; i < N0; i += kPlaneThreads) tw0[i] = t0[i];
  for (int i = tid; i < N1; i += kPlaneThreads) tw1[i] = t1[i];
  const float m2 = (float)(g.full ? gbk::ffreq(k2, g.n2) : k2);
  for (int i = tid; i < N0; i += kPlaneThreads) {
    const float m0 = (float)gbk::ffreq(i, N0);
    gA[i] = m0 * a.bgf[0] + m2 * a.bgf[6];
    gA[N0 + i] = m0 * a.bgf[1] + m2 * a.bgf[7];
    gA[2 * N0 + i] = m0 * a.bgf[2] + m2 * a.bgf[8];
  }
  for (int i = tid; i < N1; i += kPlaneThreads) {
    const float m1 = (float)gbk::ffreq(i, N1);
    gB[i] = m1 * a.bgf[3];
    gB[N1 + i] = m1 * a.bgf[4];
    gB[2 * N1 + i] = m1 * a.bgf[5];
  }
  __syncthreads();
  // forward along axis 1, its first stage reading the plane from global memory
  plane_fft<-1, 1, N0, N1, V, PS_FROM_GLOBAL>(pl, tw1, gp);
  // forward along axis 0 with the kernel multiply fused into its last stage;
  // points on a Nyquist line of a symmetrised plane take the partner-averaged
  // general path (as the column passes do)
  const bool plane_sym = g.full || k2 == 0 || ((g.n2 & 1) == 0 && 2 * k2 == g.n2);
  const bool nyq2 = g.full && (g.n2 & 1) == 0 && 2 * k2 == g.n2;
  const float coef = a.coef[f];
  const float fourpi_c = 4.0f * 3.14159265358979323846f * coef;
  if constexpr (Cfg::table_smem) {
    cp_async_wait_all();
    __syncthreads();
  }
  auto kmul = [&](int i0, int i1, float2 v) {
    float kv;
    if (type == KER_ARRAY) {
      kv = (Cfg::table_smem ? ktab[i0 * N1 + i1] : __ldg(karr + i0 * N1 + i1)) * coef;
    } else {
      const bool special = plane_sym && (nyq2 || ((N0 & 1) == 0 && 2 * i0 == N0) || ((N1 & 1) == 0 && 2 * i1 == N1));
      if (special) {
        kv = kernel_value_slow<float>(g, type, nullptr, i0, i1, k2) * coef;
      } else {
        const float gx = gA[i0] + gB[i1], gy = gA[N0 + i0] + gB[N1 + i1], gz = gA[2 * N0 + i0] + gB[2 * N1 + i1];
        const float gg = gx * gx + gy * gy + gz * gz;
        kv = type == KER_HARTREE ? (gg > 0.0f ? fourpi_c / gg : 0.0f) : (type == KER_G2 ? gg * coef : coef);
      }
    }
    return c_scale(v, kv);
  };
  plane_fft<-1, 0, N0, N1, V, PS_SMEM, PS_SMEM>(pl, tw0, nullptr, nullptr, kmul);
  plane_fft<1, 0, N0, N1, V>(pl, tw0);
  // inverse along axis 1, its last stage writing the plane to global memory
  plane_fft<1, 1, N0, N1, V, PS_SMEM, PS_TO_GLOBAL>(pl, tw1, nullptr, gp);
}

// ---- plane transforms of the WGC term --------------------------------------------
// The WGC nonlocal term needs the forward transforms of its transform inputs
// (three fields per exponent), a pointwise combination ACROSS those fields
// with four kernels, and the inverse transforms of the three combinations:
//   X0 = K0 F0 + K1/6 F1 + Kq F2,  X1 = K1/6 F0 + Kx F1,  X2 = Kq F0.
// A plane of one field fills a CTA's shared memory, so the combination
// cannot sit between the forward and inverse stages of one CTA: the forward
// plane pass writes every field's spectrum plane back (in place), and the
// inverse pass reads the three input planes of its group from global memory
// (L2), combines them into its own output plane and transforms it back.

struct PlaneFwdArgs {
  float2* spec;
  int64_t fstride;
  const void* tw0;
  const void* tw1;
};

template <int N0, int N1, int V>
__global__ void __launch_bounds__(PlaneCfg<N0, N1>::NT, 1) k_plane_fwd(PlaneFwdArgs a) {
  constexpr int NT = PlaneCfg<N0, N1>::NT;
  using Cfg = PlaneCfg<N0, N1>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* pl = reinterpret_cast<float2*>(smem_raw);
  float2* tw0 = reinterpret_cast<float2*>(smem_raw + Cfg::kPlaneBytes);
  float2* tw1 = tw0 + N0;
  const int tid = threadIdx.x;
  const int k2 = blockIdx.x, f = blockIdx.y;
  float2* gp = a.spec + f * a.fstride + (int64_t)k2 * (N0 * N1);
  const float2* t0 = reinterpret_cast<const float2*>(a.tw0);
  const float2* t1 = reinterpret_cast<const float2*>(a.tw1);
  for (int i = tid; i < N0; i += NT) tw0[i] = t0[i];
  for (int i = tid; i < N1; i += NT) tw1[i] = t1[i];
  __syncthreads();
  plane_fft<-1, 1, N0, N1, V, PS_FROM_GLOBAL>(pl, tw1, gp);
  plane_fft<-1, 0, N0, N1, V>(pl, tw0);
  // the spectrum plane back to global memory, row by row (coalesced)
  for (int idx = tid; idx < N0 * N1; idx += NT) gp[idx] = pl[paddr<N1>(idx / N1, idx % N1)];
}

struct PlaneWgcArgs {
  const float2* in;     // forward spectra of the transform inputs, group h at in + 3 h fstride
  int64_t fstride;
  float2* out;          // the combinations' planes, transformed back (group h, output j at out + (3 h + j) ostride)
  int64_t ostride;
  const float* K;       // plane-major K0, K1, Kq, Kx at K + c kstride
  int64_t kstride;
  float scale;          // 1 / N of the inverse transform
  const void* tw0;
  const void* tw1;
};

template <int N0, int N1, int V>
__global__ void __launch_bounds__(PlaneCfg<N0, N1>::NT, 1) k_plane_wgc_inv(PlaneWgcArgs a) {
  constexpr int NT = PlaneCfg<N0, N1>::NT;
  using Cfg = PlaneCfg<N0, N1>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* pl = reinterpret_cast<float2*>(smem_raw);
  float2* tw0 = reinterpret_cast<float2*>(smem_raw + Cfg::kPlaneBytes);
  float2* tw1 = tw0 + N0;
  const int tid = threadIdx.x;
  const int k2 = blockIdx.x, j = blockIdx.y, h = blockIdx.z;
  const int64_t po = (int64_t)k2 * (N0 * N1);
  const float2* s0 = a.in + 3 * h * a.fstride + po;
  const float2* s1 = s0 + a.fstride;
  const float2* s2 = s1 + a.fstride;
  const float* K0 = a.K + po;
  const float* K1 = K0 + a.kstride;
  const float* Kq = K1 + a.kstride;
  const float* Kx = Kq + a.kstride;
  float2* gp = a.out + (3 * h + j) * a.ostride + po;
  const float2* t0 = reinterpret_cast<const float2*>(a.tw0);
  const float2* t1 = reinterpret_cast<const float2*>(a.tw1);
  for (int i = tid; i < N0; i += NT) tw0[i] = t0[i];
  for (int i = tid; i < N1; i += NT) tw1[i] = t1[i];
  const float sc = a.scale, sc6 = a.scale * (1.0f / 6.0f);
  for (int idx = tid; idx < N0 * N1; idx += NT) {
    const float2 f0 = s0[idx];
    float2 v;
    if (j == 0) {
      const float2 f1 = s1[idx], f2 = s2[idx];
      const float k0 = __ldg(K0 + idx) * sc, k1 = __ldg(K1 + idx) * sc6, kq = __ldg(Kq + idx) * sc;
      v = float2{k0 * f0.x + k1 * f1.x + kq * f2.x, k0 * f0.y + k1 * f1.y + kq * f2.y};
    } else if (j == 1) {
      const float2 f1 = s1[idx];
      const float k1 = __ldg(K1 + idx) * sc6, kx = __ldg(Kx + idx) * sc;
      v = float2{k1 * f0.x + kx * f1.x, k1 * f0.y + kx * f1.y};
    } else {
      const float kq = __ldg(Kq + idx) * sc;
      v = float2{kq * f0.x, kq * f0.y};
    }
    pl[paddr<N1>(idx / N1, idx % N1)] = v;
  }
  __syncthreads();
  plane_fft<1, 0, N0, N1, V>(pl, tw0);
  plane_fft<1, 1, N0, N1, V, PS_SMEM, PS_TO_GLOBAL>(pl, tw1, nullptr, gp);
}

// plane sizes with a specialisation (the workloads' grids)
template <typename F>
__host__ inline bool plane_size_dispatch(int n, F&& f) {
  switch (n) {
    case 64: f(std::integral_constant<int, 64>{}); return true;
    case 96: f(std::integral_constant<int, 96>{}); return true;
    case 128: f(std::integral_constant<int, 128>{}); return true;
    case 160: f(std::integral_constant<int, 160>{}); return true;
    default: return false;
  }
}

template <typename F>
__host__ inline bool plane_dispatch(int n0, int n1, F&& f) {
  bool ok = false;
  plane_size_dispatch(n0, [&](auto a) {
    plane_size_dispatch(n1, [&](auto b) {
      constexpr int N0 = decltype(a)::value, N1 = decltype(b)::value;
      if constexpr (PlaneCfg<N0, N1>::fits) {
        f(a, b);
        ok = true;
      }
    });
  });
  return ok;
}

}  // namespace gbct
