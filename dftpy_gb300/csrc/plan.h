// Host-side plan: grid geometry, FFT schedules, device tables and workspaces.
#pragma once
#include "common.cuh"

struct GInfo {           // reciprocal-space geometry passed to kernels by value
  double bg[9];          // reciprocal lattice vectors, rows (2 pi inv(L)^T)
  int n0, n1, n2, n2h, ld2;
  int full;              // 1: full-grid G convention (fftfreq on every axis)
};

struct gbofdft_plan {
  int n[3];
  int n2h;               // n2 / 2 + 1
  int ld2;               // row pitch of internal spectra (complex elements)
  int full;
  int prec;              // GBOFDFT_F32 / GBOFDFT_F64
  int device;
  double lattice[9];
  double bg[9];
  double volume, dV;
  int64_t N;             // n0 n1 n2
  int64_t NG;            // n0 n1 n2h (API spectrum size)
  int64_t NGld;          // n0 n1 ld2 (internal spectrum size)
  AxisPlan ax[3];
  void* tw[3];           // device twiddle tables, complex<prec>[n_axis]
  void* spec;            // GB_MAX_FIELDS internal spectra
  double* partials;      // per-CTA energy partial sums
  int64_t max_partials;  // rows of GB_NE doubles
  double* scratch;       // small device scratch (reductions), 4096 doubles
  int tb[3];             // column tile width per axis
  int pairs;             // row pairs per CTA in the row passes
  GInfo gi;
  // FP32 plane-major evaluation pipeline (rows -> plane convolution -> rows)
  int plane;             // 1: the grid has the plane pipeline (and uses it)
  int plane_ok;          // 1: the grid has a plane specialisation
  int plane_variant;     // radix-schedule variant of the plane pass (autotuned)
  float* wt_pm;          // plane-major copy of the last WT kernel table built on this plan
  const void* wt_pm_src; // the table that copy belongs to
  float* wgc_pm;         // plane-major copy of the last WGC kernels (4 x NG) built on this plan
  const void* wgc_pm_src; // the kernels that copy belongs to
  // the buffers the last two TN preconditioners were built into and their
  // mean densities (a rebuild is skipped when both match): the FP32 stage
  // and the refinement's Hessian products keep one each on the same plan
  const void* precond_buf[2];
  double precond_rho0[2];
  int precond_next;         // slot the next build replaces
  float* precond_pm;        // FP32 plane-pipeline plans: plane-major copy of one preconditioner ...
  const void* precond_pm_src;  // ... the one built into this buffer
  int plane_precond;        // 1: preconditioner convolutions through the plane pipeline
};

size_t gb_elem(const gbofdft_plan* p);  // bytes per real scalar
// zero-initialised grid-reduction ticket in the plan's scratch (last double;
// scratch[0..4094] are free for per-CTA partial sums)
unsigned* gb_plan_counter(gbofdft_plan* p);

// ---- pass launchers (passes.cu) -------------------------------------------
// forward prologues; OP_WGC0..2: rho^e u^k (k = 0, 1, 2) of the WGC term,
// u = (rho - rho0) / rho0, exponent e in the beta argument
enum { OP_RHO = 0, OP_SQRT = 1, OP_POWB = 2, OP_WGC0 = 3, OP_WGC1 = 4, OP_WGC2 = 5 };
enum { KER_NONE = 0, KER_HARTREE = 1, KER_G2 = 2, KER_ARRAY = 3 };

struct EvalDesc {
  int tf, vw, wt, xc, hartree, pp;
  int slot_h, slot_vw, slot_wt;   // field slot of each convolution output
  double tf_x, vw_y, wt_alpha, wt_beta;
  double e_ion;
  // optional (FP64 compile-time-size passes only): the convolution results
  // before the pointwise epilogue, field slot f at cout + f * cstride
  void* cout;
  int64_t cstride;
};

struct KerDesc {
  int type[GB_MAX_FIELDS];
  const void* arr[GB_MAX_FIELDS];
  double coef[GB_MAX_FIELDS];
};

int gb_rows_fwd(gbofdft_plan* p, const void* in, void* spec, int64_t fstride, int ld2, int nf,
                const int* ops, double beta, double scale, cudaStream_t st);
int gb_rows_inv_store(gbofdft_plan* p, const void* spec, int64_t fstride, int ld2, int nf,
                      void* out, int64_t ostride, double scale, cudaStream_t st);
int gb_rows_inv_eval(gbofdft_plan* p, const void* spec, int64_t fstride, int nf, const EvalDesc& ev,
                     const void* rho, const void* vloc, void* pot, int calc_e, double* energies,
                     cudaStream_t st);
int gb_cols(gbofdft_plan* p, void* spec, int64_t fstride, int ld2, int nf, int axis, int dir,
            double scale, cudaStream_t st);
int gb_cols_conv(gbofdft_plan* p, void* spec, int64_t fstride, int ld2, int nf, const KerDesc& kd,
                 double scale, cudaStream_t st);
// compile-time-size passes (passes_ct_*.cu): return 1 when the size has no
// specialisation, 0 on success, an error code otherwise
int gb_ct_rows_fwd_f32(gbofdft_plan*, const void*, void*, int64_t, int, int, const int*, double, double, cudaStream_t);
int gb_ct_rows_fwd_f64(gbofdft_plan*, const void*, void*, int64_t, int, int, const int*, double, double, cudaStream_t);
int gb_ct_rows_inv_f32(gbofdft_plan*, const void*, int64_t, int, int, void*, int64_t, double, const EvalDesc*,
                       const void*, const void*, void*, int, double*, int64_t*, cudaStream_t);
int gb_ct_rows_inv_f64(gbofdft_plan*, const void*, int64_t, int, int, void*, int64_t, double, const EvalDesc*,
                       const void*, const void*, void*, int, double*, int64_t*, cudaStream_t);
int gb_ct_cols_f32(gbofdft_plan*, void*, int64_t, int, int, int, int, double, const KerDesc*, cudaStream_t);
// plane-major FP32 pipeline (passes_ct_f32.cu)
int gb_ct_rows_fwd_pm_f32(gbofdft_plan*, const void*, void*, int64_t, int, const int*, double, cudaStream_t);
int gb_ct_rows_inv_eval_pm_f32(gbofdft_plan*, const void*, int64_t, int, const EvalDesc*, const void*, const void*,
                               void*, int, double*, int64_t*, cudaStream_t);
int gb_plane_conv_f32(gbofdft_plan*, void*, int64_t, int, const KerDesc*, const float* const*, double, cudaStream_t);
int gb_plane_supported_f32(int n0, int n1, int n2);
// WGC fields on the plane pipeline (FP32): the forward rows with the WGC
// prologues (3 fields rho^e u^k from rho), the forward plane transforms of
// nf fields (in place), the kernel combination and inverse plane transforms
// of ngroups groups of three fields (K: the plane-major kernels K0, K1, Kq,
// Kx), and the inverse rows storing real fields
int gb_ct_rows_fwd_wgc_pm_f32(gbofdft_plan*, const void* rho, void* spec, int64_t fstride, double e, double rho0,
                              cudaStream_t);
int gb_plane_fwd_f32(gbofdft_plan*, void* spec, int64_t fstride, int nf, cudaStream_t);
int gb_plane_wgc_inv_f32(gbofdft_plan*, const void* spec, int64_t fstride, void* out, int64_t ostride, int ngroups,
                         const float* K, double scale, cudaStream_t);
int gb_ct_rows_inv_store_pm_f32(gbofdft_plan*, const void* spec, int64_t fstride, int nf, void* out, int64_t ostride,
                                cudaStream_t);
// the inverse rows of the six (three when a == b) combined WGC spectra with
// the NL potential added to pot (FP32 evaluations); part non-null: per-CTA
// partial sums of the NL energy integrand, *nblk of them
int gb_ct_rows_inv_wgc_pm_f32(gbofdft_plan*, const void* spec, int64_t fstride, int two, const float* rho, double rho0,
                              double ea, double eb, float* pot, double* part, int64_t* nblk, cudaStream_t);
int gb_plane_variants_f32(int n0, int n1);
// the plane-major evaluation (returns 1 when the plan has no plane pipeline
// or a kernel table has no plane-major copy)
int gb_eval_plane(gbofdft_plan* p, const void* rho, int nf, const int* ops, double beta, const KerDesc& kd,
                  const EvalDesc& ev, const void* vloc, void* pot, int calc_e, double* energies, cudaStream_t st);
int gb_ct_cols_f64(gbofdft_plan*, void*, int64_t, int, int, int, int, double, const KerDesc*, cudaStream_t);
// delta evaluation (passes_delta.cu): FP32 transforms of the change of the
// derived fields against a reference density, FP64 pointwise work
int gb_delta_rows_fwd(gbofdft_plan* p32, const double* rho, const double* rho_ref, void* spec, int64_t fstride,
                      int nf, const int* ops, double beta, cudaStream_t st);
int gb_delta_rows_inv_eval(gbofdft_plan* p32, const void* spec, int64_t fstride, int nf, const EvalDesc* ev,
                           const double* rho, const double* rho_ref, const double* pot_ref, const double* vloc,
                           const double* cref, int64_t cstride, double* pot, int calc_e, double* partials,
                           int64_t* nblk, cudaStream_t st);
int gb_delta_supported(int n0, int n1, int n2);
// the whole delta evaluation of the fused terms (passes.cu): plane pipeline
// of p32 on the changes, FP64 epilogue into pot / energies (energies use p64's
// partials and dV)
int gb_eval_delta_core(gbofdft_plan* p64, gbofdft_plan* p32, const double* rho, const double* rho_ref,
                       const double* pot_ref, const double* eref, const double* cref, int nf, const int* ops,
                       double beta, const KerDesc& kd, const EvalDesc& ev, const double* vloc, double* pot,
                       int calc_e, double* energies, cudaStream_t st);
// the reference density of a delta-evaluation state (device, N doubles)
const double* gb_delta_ref(const gbofdft_delta* d);
void gb_count_launch();
int gb_smem_granted(const void* kern, int dev);
void gb_smem_grant(const void* kern, int dev, int bytes);
int gb_use_ct();  // 0 forces the generic passes (GBOFDFT_GENERIC_FFT=1)

int gb_lwt_eval(gbofdft_plan* p, const void* rho, gbofdft_lwt* d, void* pot, double* energies, int calc_v,
                int calc_e, cudaStream_t st);
// store_ref (FP64 plans): keep this evaluation as the reference of gb_wgc_eval_delta
int gb_wgc_eval(gbofdft_plan* p, const void* rho, const gbofdft_wgc* d, void* pot, double* energies, int calc_v,
                int calc_e, int store_ref, cudaStream_t st);
// the WGC term at rho from the reference kept by the last store_ref
// evaluation with d64 (at rho_ref): FP32 transforms of the change with p32 /
// d32, the NL potential added to pot, the energy to energies (with calc_e)
int gb_wgc_eval_delta(gbofdft_plan* p64, gbofdft_plan* p32, const double* rho, const double* rho_ref,
                      const gbofdft_wgc* d64, const gbofdft_wgc* d32, double* pot, double* energies, int calc_e,
                      cudaStream_t st);

// phi-space TN preconditioner of the uniform gas rho0 on the half spectrum (real, NG values)
int gb_build_precond(gbofdft_plan* p, double rho0, void* out, cudaStream_t st);
int gb_build_wt_kernel(gbofdft_plan* p, double rho0, double x, double alpha, double beta, void* out,
                       cudaStream_t st);
