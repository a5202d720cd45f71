/*
 * gbofdft: GB300-native orbital-free DFT energy/potential evaluation and
 * direct density optimisation -- the C ABI.
 *
 * Every entry point returns an int status (GBOFDFT_OK = 0, otherwise a
 * gbofdft_status code; gbofdft_last_error() gives the message).  All device
 * pointers are caller-owned; a plan owns only its tables and workspaces, so
 * entry points never allocate.  Work is ordered on the given CUDA stream
 * (``stream`` is a cudaStream_t, NULL = legacy default stream) and nothing
 * synchronises unless the entry point says so.  A plan holds per-plan
 * workspaces: do not use one plan on two streams at the same time.
 *
 * Precision: GBOFDFT_F64 plans take double / complex-double buffers,
 * GBOFDFT_F32 plans float / complex-float.  Energies are always double.
 *
 * Layouts (C order): real field [n0][n1][n2]; spectrum (half) complex
 * [n0][n1][n2/2+1], interleaved re/im.  Forward transforms carry the grid
 * volume element dV, inverse ones 1/dV (dftpy's field.py convention).
 */
#ifndef GBOFDFT_H
#define GBOFDFT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBOFDFT_ABI_VERSION 1

enum gbofdft_status {
  GBOFDFT_OK = 0,
  GBOFDFT_ERR_ARG = 1,         /* bad argument (python: ValueError / TypeError) */
  GBOFDFT_ERR_CUDA = 2,        /* CUDA runtime error */
  GBOFDFT_ERR_UNSUPPORTED = 3, /* size or option not supported */
  GBOFDFT_ERR_ALLOC = 4,       /* plan workspace allocation failed */
  GBOFDFT_ERR_NUMERIC = 5,     /* non-finite or invalid numerical state */
  GBOFDFT_ERR_STATE = 6        /* inconsistent plan / buffer state */
};

enum gbofdft_precision { GBOFDFT_F32 = 0, GBOFDFT_F64 = 1 };

enum gbofdft_calc { GBOFDFT_CALC_E = 1, GBOFDFT_CALC_V = 2 };

/* energies[] slots written by gbofdft_eval (Hartree atomic units) */
enum gbofdft_energy_slot {
  GBOFDFT_E_TF = 0,
  GBOFDFT_E_VW = 1,
  GBOFDFT_E_NL = 2,
  GBOFDFT_E_XC = 3,
  GBOFDFT_E_HARTREE = 4,
  GBOFDFT_E_PSEUDO = 5,
  GBOFDFT_E_EXTRA = 6,
  GBOFDFT_E_TOTAL = 7,
  GBOFDFT_NE = 8
};

typedef struct gbofdft_plan gbofdft_plan;

/* ABI version of the loaded library. */
int gbofdft_version(void);

/* Number of kernels this library has launched in this process (monotonic). */
int gbofdft_launch_count(int64_t* count);

/* Copy the last error message (thread-local) into buf; returns its length. */
int gbofdft_last_error(char* buf, size_t len);

/*
 * Grid plan.  Replaces dftpy DirectGrid / ReciprocalGrid set-up
 * (src/dftpy/grid.py:302-330 DirectGrid.__init__, :384-415 get_reciprocal).
 * lattice: 3x3 row-major, rows are lattice vectors (Bohr).  full = 1 selects
 * the reference's full-grid G convention (DirectGrid(full=True)).
 */
int gbofdft_plan_create(const int nr[3], const double lattice[9], int precision, int full,
                        gbofdft_plan** out);
int gbofdft_plan_destroy(gbofdft_plan* plan);

/* out[0] = N real points, out[1] = half-spectrum size, out[2] = n2/2+1,
 * out[3] = device workspace bytes held by the plan. */
int gbofdft_plan_sizes(const gbofdft_plan* plan, int64_t out[4]);

/* Forward 3D R2C, times dV.  Replaces DirectField.fft (src/dftpy/field.py:373-390). */
int gbofdft_fft_r2c(gbofdft_plan* plan, const void* in, void* out, void* stream);

/* Inverse 3D C2R, divided by dV, irfftn semantics; ``in`` is not modified.
 * Replaces ReciprocalField.ifft(force_real=True) (src/dftpy/field.py:739-764). */
int gbofdft_fft_c2r(gbofdft_plan* plan, const void* in, void* out, void* stream);

/* Reciprocal-space kernels for gbofdft_convolve */
enum gbofdft_kernel { GBOFDFT_KER_NONE = 0, GBOFDFT_KER_HARTREE = 1, GBOFDFT_KER_G2 = 2, GBOFDFT_KER_ARRAY = 3 };

/*
 * out = ifft(fft(in) * coef * K(G)) in one pipeline (real in, real out).
 * K = 4 pi / G^2 (G=0 -> 0), G^2, or a real half-spectrum array.
 * Replaces the fft -> multiply -> ifft pattern of hartree.py:34-38,
 * vw.py:45-49 and wt.py:21.
 */
int gbofdft_convolve(gbofdft_plan* plan, const void* in, void* out, int kernel, const void* kernel_array,
                     double coef, void* stream);

/*
 * Allocation-free variant of gbofdft_convolve, for callers that cannot
 * allocate device memory (code running under another framework's allocator,
 * or code that must avoid the implicit synchronisation of cudaMalloc /
 * cudaFree).  No counterpart in the reference: it exists for those callers.
 * Takes the grid directly (no plan: creating one allocates) and keeps its
 * scratch -- twiddle tables and one spectrum -- in a fixed 16 MiB device
 * array inside the library (held by every GPU that loads it, until exit).
 * Grids whose scratch does not fit are rejected (GBOFDFT_ERR_UNSUPPORTED),
 * e.g. 96^3 fits in FP64, 128^3 in FP32 only.  All calls share the array:
 * calls that overlap on the GPU race; serialise them (a call that fails part
 * way may also leave the array rewritten).  The first call on a device looks
 * the array up (cudaGetSymbolAddress) and keeps the address for the process:
 * make it before any stream capture; a device reset or another context on
 * the same device is not supported.  Same arguments as gbofdft_convolve; the
 * result equals its result to rounding (the twiddles are computed on the
 * device instead of on the host).
 */
int gbofdft_convolve_noalloc(const int nr[3], const double lattice[9], int precision, int full, const void* in,
                             void* out, int kernel, const void* kernel_array, double coef, void* stream);

/*
 * LWT / LMGP nonlocal kinetic term (kedf/lwt.py:82-341 LWTPotentialEnergy):
 * kernel K(q / k_F(r)) interpolated between k_F knots k_min ratio^i.  The
 * kernel tables are cubic splines on the uniform grid eta_j = j etamax /
 * (neta - 1): ktab_c (neta-1 pieces x 4 coefficients, device) of K(eta) and
 * dtab_c of K'(eta) (-eta) (lwt.py:553-561), with their values at etamax.
 * kfmin_state / kfmax_state carry the automatic k_F bounds across calls
 * (guess_kf_bound, lwt.py:36-79); set them <= 0 for a fresh start.
 */
typedef struct gbofdft_lwt {
  int interp;              /* 0 linear, 1 hermite */
  int kdd;                 /* 1..3 (the reference's default 3) */
  double alpha, beta, ratio, ldw;
  double etamax;
  int neta;
  const double* ktab_c;
  double ktab_end;
  const double* dtab_c;
  double dtab_end;
  double kfmin_opt, kfmax_opt;     /* fixed bounds (> 0) or automatic (<= 0) */
  double kfmin_state, kfmax_state; /* automatic bounds carried between calls */
  void* work;                      /* device workspace, 256-byte aligned */
  int64_t work_bytes;              /* >= gbofdft_lwt_workspace_bytes */
  int nknots;                      /* out: knots used by the last call */
} gbofdft_lwt;

int gbofdft_lwt_workspace_bytes(const gbofdft_plan* plan, int64_t* bytes);

/*
 * MGP kernel table (kedf/kernel.py:267-322 MGPKernelTable): table_out[j] =
 * (4/5) C_TF (5/6) / maxpoints * sum_{i=1..maxpoints} G(eta_j t_i^(-1/3)) t_i^(-1/6),
 * t_i = i / maxpoints, G the cubic spline (pieces coef, knots gp[0..m-1], end
 * values beyond) of the inverse Lindhard function.  All pointers device.
 */
int gbofdft_mgp_table(const double* gp, const double* coef, int m, const double* eta, int neta, int maxpoints,
                      double* table_out, void* stream);

/*
 * WGC nonlocal kinetic term (density-dependent kernel): no reference
 * counterpart (the reference's KEDF set, kedf/__init__.py:27-69, has none);
 * the published method of Wang, Govind and Carter, PRB 60, 16350 (1999), with
 * the two-body Fermi wavevector xi = [(k_F(r)^gamma + k_F(r')^gamma)/2]^(1/gamma)
 * and the kernel expanded to second order in (rho - rho0)/rho0 about rho0.
 * The kernel's shape w(eta) solves the linear-response equation (so that the
 * expanded functional keeps the Lindhard response at rho0); it is tabulated
 * on the host: table = 4 columns of m FP64 values (K0, K1, Kq, Kx per unit
 * prefactor, device) on t = ln(eta) = t0 + i h.  gbofdft_wgc_kernels scales
 * and interpolates them onto the half spectrum (API layout, plan precision)
 * for one rho0.  Order 0 tables are the Wang-Teter kernel (K1 = Kq = Kx = 0).
 * alpha == beta halves the work.  Its energy goes to the NL slot.
 */
typedef struct gbofdft_wgc {
  double alpha, beta, gamma;
  double rho0;                     /* expansion density (the mean density) */
  int order;                       /* 0, 1 or 2 */
  const void* kernels;             /* 4 x NG real values */
  void* work;                      /* device workspace, 256-byte aligned */
  int64_t work_bytes;              /* >= gbofdft_wgc_workspace_bytes */
} gbofdft_wgc;

/* Bytes of the term's workspace; FP64 plans also hold a delta-evaluation
 * reference (see gbofdft_eval_delta). */
int gbofdft_wgc_workspace_bytes(const gbofdft_plan* plan, int64_t* bytes);
int gbofdft_wgc_kernels(gbofdft_plan* plan, double rho0, double alpha, double beta, const double* table, int m,
                        double t0, double h, void* kernels_out, void* stream);

/* Functional composition for gbofdft_eval (TotalFunctional of
 * KEDF(TF/vW/WT/LWT) + XC(LDA) + HARTREE + PSEUDO). */
typedef struct gbofdft_functional {
  int tf;                /* Thomas-Fermi, kedf/tf.py:66-80 */
  double tf_x;
  int vw;                /* von Weizsaecker, kedf/vw.py:115-131 */
  double vw_y;
  int wt;                /* Wang-Teter nonlocal, kedf/wt.py:109-132 */
  double wt_alpha, wt_beta;
  const void* wt_kernel; /* real half spectrum from gbofdft_wt_kernel */
  int xc;                /* 1 = Perdew-Zunger LDA, xc/semilocal_xc.py:253-290 */
  int hartree;           /* hartree.py:24-45 */
  const void* vloc;      /* real field (local pseudopotential) or NULL, pseudo/__init__.py:219-234 */
  double e_ion;          /* constant ion-ion energy added to the total */
  gbofdft_lwt* lwt;      /* LWT/LMGP nonlocal term or NULL (its energy goes to the NL slot); the
                            call reads the density extrema back to the host to place the knots */
  gbofdft_wgc* wgc;      /* WGC nonlocal term or NULL (its energy goes to the NL slot) */
} gbofdft_functional;

/*
 * Energy and potential of the composed functional at rho.
 * Replaces TotalFunctional.compute (src/dftpy/functional/total_functional.py:107-146).
 * calc: GBOFDFT_CALC_E | GBOFDFT_CALC_V.  pot (real field) is always written;
 * with CALC_E, energies_dev (device, GBOFDFT_NE doubles) receives the
 * component energies and the total (ion-ion term included).
 */
int gbofdft_eval(gbofdft_plan* plan, const void* rho, const gbofdft_functional* f, void* pot,
                 double* energies_dev, int calc, void* stream);

/*
 * Delta evaluation (no reference counterpart; the FP64 evaluations of the
 * mixed-precision refinement).  The convolutions of the fused terms are
 * linear, so at a density rho near a reference density rho_ref
 *   C(rho) = C(rho_ref) + K * (g(rho) - g(rho_ref))
 * for each derived field g (rho, sqrt(rho), rho^beta).  A state holds rho_ref
 * and its FP64 C(rho_ref); a delta evaluation transforms the change of g in
 * FP32 (plane pipeline of hplan) and runs the pointwise terms in FP64, so its
 * error is ~1e-7 of the change rather than of C.  rebase = 1 runs the full
 * FP64 evaluation (gbofdft_eval) at rho and makes rho the reference.  The WGC
 * term, when f and hf both have one, is evaluated the same way: the rebase
 * keeps its X / Y fields, NL potential and energy in the FP64 term's
 * workspace, and a delta evaluation transforms the change of its transform
 * inputs (rho^b, u rho^b, u^2 rho^b and the same with a) in FP32 and forms
 * the potential and energy as FP32 changes on that reference (the FP64 WGC
 * workspace must not be used for other evaluations between a rebase and the
 * delta evaluations that follow it).  The LWT term is always evaluated in
 * full FP64.
 * plan: FP64, hplan: FP32 on the same grid (a plane-pipeline size); f: the
 * FP64 functional, hf: the same terms in FP32 (its WT kernel table built on
 * hplan).  Other arguments as gbofdft_eval.
 */
typedef struct gbofdft_delta gbofdft_delta;
int gbofdft_delta_create(gbofdft_plan* plan, gbofdft_plan* hplan, gbofdft_delta** out);
int gbofdft_delta_destroy(gbofdft_delta* d);
int gbofdft_eval_delta(gbofdft_delta* d, const void* rho, const gbofdft_functional* f,
                       const gbofdft_functional* hf, void* pot, double* energies_dev, int calc, int rebase,
                       void* stream);

/*
 * Wang-Teter kernel on the half spectrum for mean density rho0.
 * Replaces get_ke_kernel_wt / WTKernel (kedf/wt.py:58-73, kedf/kernel.py:325-334).
 */
int gbofdft_wt_kernel(gbofdft_plan* plan, double rho0, double x, double alpha, double beta, void* kernel_out,
                      void* stream);

/* ---- set-up: local pseudopotential and ion-ion energy --------------------- */

#define GBOFDFT_MAX_SPECIES 16

/* One species' v(|G|) table, evaluated as dftpy's LocalPseudo.calc_vlines
 * (functional/pseudo/__init__.py:350-375): cubic spline pieces on knots x[0..m-1]
 * (c: (m-1) x 4 coefficients of a + b u + c u^2 + d u^3, u = q - x[i]) for
 * gmin <= q < gmax, quartic q4[0..4] in q/dp (divided by 24 for the
 * non-constant part, math_utils.py:457-467) below gmin, 0 from gmax on.
 * x and c are device pointers. */
typedef struct gbofdft_vtable {
  const double* x;
  const double* c;
  int m;
  double q4[5];
  double dp, gmin, gmax;
} gbofdft_vtable;

/* Device workspace bytes for gbofdft_vloc / gbofdft_ewald with nat atoms. */
int gbofdft_setup_workspace_bytes(const gbofdft_plan* plan, int nat, int64_t* bytes);

/*
 * Local pseudopotential v_loc on the half spectrum (vloc_recip, complex) and,
 * if vloc_real != NULL, in real space.  spos_dev: fractional positions
 * (nat x 3, in [0,1)), species_dev: species index per atom.  pme != 0 uses
 * order-`order` cardinal B-spline structure factors with bm_dev = the b(m)
 * factors of the three axes concatenated (n0 + n1 + n2/2+1 complex doubles);
 * pme == 0 the exact structure factor.
 * Replaces LocalPseudo.local_PP / _PP_Reciprocal(_PME)
 * (src/dftpy/functional/pseudo/__init__.py:237-246, 377-404).
 */
int gbofdft_vloc(gbofdft_plan* plan, int nspec, const gbofdft_vtable* tables, int nat, const double* spos_dev,
                 const int* species_dev, int pme, int order, const double* bm_dev, void* work, int64_t work_bytes,
                 void* vloc_recip, void* vloc_real, void* stream);

/*
 * Ewald sums of the ions: out_dev[0] = real-space part, out_dev[1] =
 * reciprocal part (PME or exact).  The host adds the constant correction
 * and chooses eta, rmax and the lattice images (nimg x 3 Cartesian offsets).
 * Replaces ewald.Energy_real(_fast2), Energy_rec(_PME) (src/dftpy/ewald.py:281-466,
 * 786-808).
 */
int gbofdft_ewald(gbofdft_plan* plan, int nat, const double* pos_dev, const double* spos_dev,
                  const double* charges_dev, double eta, double rmax, const double* images_dev, int nimg, int pme,
                  int order, const double* bm_dev, void* work, int64_t work_bytes, double* out_dev, void* stream);

/* ---- density guesses -------------------------------------------------------- */

/*
 * In place on rho (plan precision, device): rho[rho < dtol] = dtol, then
 * nc = sum(rho) dV (FP64, fixed order) and, if ncharge > 1e-6,
 * rho *= ncharge / nc.  nc_dev (device double, may be NULL) receives nc.
 * Pass dtol = -HUGE_VAL to skip the clamp, ncharge = 0 to skip the scaling.
 * Replaces the clamp-and-scale step of DensityGenerator.guess_rho_atom and
 * get_3d_value_recipe (src/dftpy/density/density.py:226-234, 288-297).
 */
int gbofdft_density_normalize(gbofdft_plan* plan, void* rho, double dtol, double ncharge, double* nc_dev,
                              void* stream);

/*
 * Superposed atomic densities from per-species reciprocal-space tables
 * rho_s(|G|) (same table format and structure-factor options as
 * gbofdft_vloc; a table is 0 from gmax on and, with q4 = 0, below gmin),
 * written to rho_recip (half spectrum) and rho (real space), then clamped at
 * dtol and scaled to ncharge electrons as gbofdft_density_normalize.
 * Workspace: gbofdft_setup_workspace_bytes.
 * Replaces DensityGenerator.guess_rho -> get_3d_value_recipe
 * (src/dftpy/density/density.py:151-197, 252-300).
 */
int gbofdft_density_guess(gbofdft_plan* plan, int nspec, const gbofdft_vtable* tables, int nat,
                          const double* spos_dev, const int* species_dev, int pme, int order, const double* bm_dev,
                          void* work, int64_t work_bytes, void* rho_recip, void* rho, double dtol, double ncharge,
                          void* stream);

/* ---- forces on the ions -------------------------------------------------- */

/* Device workspace bytes for gbofdft_pp_forces / gbofdft_ewald_forces with nat atoms. */
int gbofdft_forces_workspace_bytes(const gbofdft_plan* plan, int nat, int64_t* bytes);

/*
 * Forces of the local pseudopotential on the ions for the density rho
 * (device, plan precision): forces_dev = nat x 3 doubles (Ha/Bohr),
 * overwritten.  Arguments as gbofdft_vloc; pme != 0 gathers the B-spline
 * derivative of ifft(rhoG conj(B) vline_s) per species, pme == 0 sums the
 * exact structure factor over the half-space G mask.  At most 65535 atoms.
 * Replaces LocalPseudo.force -> _ForcePME / _Force
 * (src/dftpy/functional/pseudo/__init__.py:457-523).
 */
int gbofdft_pp_forces(gbofdft_plan* plan, const void* rho, int nspec, const gbofdft_vtable* tables, int nat,
                      const double* spos_dev, const int* species_dev, int pme, int order, const double* bm_dev,
                      void* work, int64_t work_bytes, double* forces_dev, void* stream);

/*
 * Ewald forces on the ions, real-space part plus reciprocal part (PME or
 * exact), written to forces_dev (nat x 3 doubles, Ha/Bohr).  eta, rmax and
 * the images as for gbofdft_ewald.
 * Replaces ewald.forces, Forces_real, Forces_rec, Forces_rec_PME
 * (src/dftpy/ewald.py:510-604, 810-857).
 */
int gbofdft_ewald_forces(gbofdft_plan* plan, int nat, const double* pos_dev, const double* spos_dev,
                         const double* charges_dev, double eta, double rmax, const double* images_dev, int nimg,
                         int pme, int order, const double* bm_dev, void* work, int64_t work_bytes,
                         double* forces_dev, void* stream);

/* ---- stress --------------------------------------------------------------- */

/* Device workspace bytes for the stress entry points with nat atoms (0: functional terms only). */
int gbofdft_stress_workspace_bytes(const gbofdft_plan* plan, int nat, int64_t* bytes);

/*
 * Stress tensors (Ha/Bohr^3, row-major 3x3) of the density-functional terms
 * of f at rho: out_dev[0..44] = TF, vW, WT nonlocal, LDA, Hartree (9 doubles
 * each; zero for disabled terms).  energies: host copy of the energies
 * gbofdft_eval wrote for this rho (slots GBOFDFT_E_*).  Synchronises the
 * stream once when WT is enabled (the mean density).  Replaces
 * ThomasFermiStress, vonWeizsackerStress, WTStress, LDAStress and
 * HartreeFunctionalStress (src/dftpy/functional/kedf/tf.py:52-62,
 * kedf/vw.py:97-112, kedf/wt.py:75-105, xc/semilocal_xc.py:308-322,
 * hartree.py:68-90) as TotalFunctional.get_stress calls them
 * (total_functional.py:176-209).
 */
int gbofdft_stress_functional(gbofdft_plan* plan, const void* rho, const gbofdft_functional* f,
                              const double energies[GBOFDFT_NE], void* workspace, int64_t workspace_bytes,
                              double* out_dev, void* stream);

/*
 * Local-pseudopotential stress (out_dev: 9 doubles), PME or exact structure
 * factor; e_pp the local-PP energy at rho; other arguments as gbofdft_vloc.
 * Replaces LocalPseudo.stress -> _StressPME / _Stress
 * (src/dftpy/functional/pseudo/__init__.py:248-258, 431-455, 525-562).
 */
int gbofdft_pp_stress(gbofdft_plan* plan, const void* rho, int nspec, const gbofdft_vtable* tables, int nat,
                      const double* spos_dev, const int* species_dev, int pme, int order, const double* bm_dev,
                      double e_pp, void* workspace, int64_t workspace_bytes, double* out_dev, void* stream);

/*
 * Ewald stress (out_dev: 9 doubles): real-space part plus the PME or exact
 * reciprocal part and its G = 0 term (charge_sum = sum of the ionic charges);
 * eta, rmax and the images as for gbofdft_ewald.
 * Replaces ewald.stress, Stress_real, Stress_rec, Stress_rec_PME
 * (src/dftpy/ewald.py:523-538, 609-662, 719-760, 915-963).
 */
int gbofdft_ewald_stress(gbofdft_plan* plan, int nat, const double* pos_dev, const double* spos_dev,
                         const double* charges_dev, double eta, double rmax, const double* images_dev, int nimg,
                         int pme, int order, const double* bm_dev, double charge_sum, void* workspace,
                         int64_t workspace_bytes, double* out_dev, void* stream);

/* ---- direct density optimisation (truncated Newton) ---------------------- */

/* Options of Optimization(optimization_method="TN") (optimization.py:64-77). */
typedef struct gbofdft_tn_options {
  double econv;  /* stop when the last ncheck energy changes are <= econv (Ha) */
  int maxfun;    /* inner CG iterations per TN direction */
  int maxiter;   /* outer iterations */
  int maxls;     /* line-search evaluations per outer iteration */
  double c1, c2, xtol; /* More-Thuente parameters */
  int ncheck;
  double eps;    /* finite-difference step of the Hessian product: > 0 fixed
                    (the reference uses 1e-9), < 0 relative: |eps| ||phi|| / ||r0||
                    per TN direction (single precision), 0 -> 1e-9 */
  double pred_stop; /* > 0: stop converged when the quadratic-model energy
                       decrease of the next Newton step, |dE/dtheta| theta0 / 2,
                       is below it (no reference counterpart); 0: off */
  double eres;      /* > 0: relative energy resolution of the evaluation; a
                       line-search trial whose energy change is below
                       eres max(1, |E|) is accepted when |dE/dtheta| <= c2 |dE/dtheta(0)|
                       (no reference counterpart); 0: off (the reference's test) */
  double cg_rtol;   /* inner CG stops when r.r < cg_rtol r0.r0 (the reference: 0.1) */
  int pred_next;    /* with pred_stop > 0: also stop after a step whose model
                       decrease times cg_rtol is below pred_stop (no reference
                       counterpart); 0: off */
  int precond;      /* 1: preconditioned inner CG with the inverse phi-space
                       Hessian of the uniform electron gas at the mean density
                       (Lindhard kinetic + Hartree curvature, applied by FFT);
                       no reference counterpart.  0: the reference's plain CG */
  int time_evals;   /* 1: time the FP32 potential-only evaluations with CUDA
                       events (result t_eval_timed / n_eval_timed); 0: off */
  gbofdft_delta* delta; /* split mode only: evaluate the FP64 energies and
                           potentials by gbofdft_eval_delta against the last
                           full evaluation (NULL: every one in full FP64) */
  double delta_rtol;    /* rebase (full FP64 evaluation) when
                           ||rho - rho_ref|| > delta_rtol ||rho_ref|| */
  double res0_max;      /* > 0: check the start -- when the residual norm
                           sqrt(int ((V - mu) phi)^2) at the initial density
                           exceeds it (or is not finite), return at once with
                           converged = 3 and the density unchanged, so the
                           caller can start again from another one; 0: off
                           (no reference counterpart) */
} gbofdft_tn_options;

typedef struct gbofdft_tn_result {
  double energy;          /* total energy at the final density (Ha) */
  double mu;              /* chemical potential (Ha) */
  int converged;          /* 0 converged, 1 line search failed, 2 maxiter,
                             3 start rejected by res0_max */
  int n_iter;
  int n_eval_ev;          /* energy+potential evaluations */
  int n_eval_v;           /* potential-only evaluations */
  double energies[GBOFDFT_NE];
  double* history;        /* optional host array receiving the energy history */
  int history_cap;
  int n_history;
  int n_sync;             /* host synchronisations performed */
  double t_sync;          /* host seconds spent waiting in them (scalar read-backs) */
  double t_total;         /* host seconds in gbofdft_optimize_tn */
  int n_eval_hess;        /* potential evaluations in the Hessian plan (split mode) */
  double t_eval_timed;    /* with time_evals: device seconds of the timed evaluations */
  int n_eval_timed;       /* ... and their number */
  int n_eval_delta;       /* with opts.delta: evaluations done as delta evaluations */
} gbofdft_tn_result;

int gbofdft_tn_options_default(gbofdft_tn_options* opts);

/* Bytes of device workspace gbofdft_optimize_tn needs for this plan. */
int gbofdft_tn_workspace_bytes(const gbofdft_plan* plan, int64_t* bytes);

/*
 * Minimise the composed functional over rho (fixed electron number) by
 * truncated Newton in phi = sqrt(rho) with the orthogonal rotation line
 * search.  rho_io: initial density in, optimised density out.  workspace:
 * caller-owned device buffer (256-byte aligned) of gbofdft_tn_workspace_bytes.
 * Synchronises the stream (the control flow needs the scalars).  Returns
 * GBOFDFT_ERR_NUMERIC when the initial density holds NaN/Inf or no
 * electrons, or an evaluation gives a non-finite energy; GBOFDFT_ERR_ARG for
 * a workspace smaller than gbofdft_tn_workspace_bytes.
 * Replaces Optimization.optimize_rho with method "TN"
 * (src/dftpy/optimization/optimization.py:281-520).
 */
int gbofdft_optimize_tn(gbofdft_plan* plan, const gbofdft_functional* f, void* rho_io,
                        const gbofdft_tn_options* opts, void* workspace, int64_t workspace_bytes,
                        gbofdft_tn_result* result, void* stream);

/* Bytes of device workspace gbofdft_optimize_tn_split needs for its Hessian plan. */
int gbofdft_tn_hess_workspace_bytes(const gbofdft_plan* hplan, int64_t* bytes);

/*
 * gbofdft_optimize_tn with the Hessian-vector products of the inner CG loop
 * evaluated by a second, single-precision plan and functional on the same
 * grid (hplan FP32, plan FP64): residual, orthonormalisation, line search and
 * convergence test stay in FP64, each TN direction costs one FP32 base
 * evaluation plus one FP32 evaluation per CG step.  opts->eps applies to the
 * FP32 products (use a relative step, eps < 0).  hplan == NULL is
 * gbofdft_optimize_tn.  No reference counterpart: a precision split of
 * Optimization.optimize_rho's TN (optimization.py:91-147, 281-520).
 */
int gbofdft_optimize_tn_split(gbofdft_plan* plan, const gbofdft_functional* f, gbofdft_plan* hplan,
                              const gbofdft_functional* hf, void* rho_io, const gbofdft_tn_options* opts,
                              void* workspace, int64_t workspace_bytes, void* hworkspace, int64_t hworkspace_bytes,
                              gbofdft_tn_result* result, void* stream);

/*
 * One call of the More-Thuente line-search state machine (host only).
 * Replaces minpack2.dcsrch as driven by LineSearchDcsrch2
 * (src/dftpy/math_utils.py:76-106).  task codes: 0 START, 1 FG (evaluate f,g
 * at *stp), 2 CONVERGENCE, 3 WARNING, 4 ERROR.  On START, state[0..4] hold
 * ftol, gtol, xtol, stpmin, stpmax; state needs >= 24 doubles.
 */
int gbofdft_dcsrch(double* state, int64_t state_len, double* stp, double f, double g, int task);

/* ---- evaluation schedules (autotuning) ----------------------------------------
 * No reference counterpart (the reference's only FFT planning is pyFFTW's
 * FFTW_MEASURE, math_utils.py:181-222).  Schedule 0 is the column-pass
 * pipeline; schedules 1.. (FP32 plans whose (n0, n1) plane has a
 * specialisation) are the plane pipeline with radix-schedule variant
 * (schedule - 1).  All give the same result within FP32 rounding; an
 * autotuner times them and keeps the fastest.
 */
int gbofdft_plan_schedules(const gbofdft_plan* plan, int* count);
int gbofdft_plan_set_schedule(gbofdft_plan* plan, int schedule);
int gbofdft_plan_get_schedule(const gbofdft_plan* plan, int* schedule);

/* ---- learned initial guess: network kernels ----------------------------------
 * No reference counterpart (the reference's guesses are density/density.py:
 * 151-319: uniform or superposed atomic densities; the network maps those
 * and v_loc to a starting sqrt(rho)).  Activations [C][D][H][W] FP32 on a
 * periodic grid; weights [C_out][C_in][27] BF16 (tap = (dz+1)*9 + (dy+1)*3 +
 * (dx+1)); FP32 accumulation; all pointers device.
 */

/* out = conv(in) + bias; transposed != 0: the input gradient (weights
 * transposed in (C_out, C_in), taps reversed; in = output gradient with cin =
 * the layer's C_out, out with cout = its C_in; bias must be NULL). */
int gbofdft_nn_conv3d(const float* in, int cin, const void* w_bf16, const float* bias, float* out, int cout, int D,
                      int H, int W, int transposed, void* stream);
/* gw[co][ci][tap] = sum_v gout[co][v] in[ci][v + d_tap]; gb[co] = sum_v gout[co][v] (gb may be NULL). */
int gbofdft_nn_conv3d_wgrad(const float* in, int cin, const float* gout, int cout, int D, int H, int W, float* gw,
                            float* gb, void* stream);
/* op: 0 SiLU(a), 1 b * SiLU'(a), 2 a + b, 3 2x average pool, 4 its adjoint, 5 2x nearest upsample, 6 its
 * adjoint, 7 2x periodic trilinear upsample (cell-centred: fine point i at coarse i/2 - 1/4), 8 its
 * adjoint; (C, D, H, W) are the fine-grid extents for ops 3-8. */
int gbofdft_nn_pointwise(int op, const float* a, const float* b, float* out, int C, int D, int H, int W,
                         void* stream);
/* loss = sum (pred - target)^2 / sum target^2 (device double), grad = d loss / d pred (may be NULL). */
int gbofdft_nn_sqerr(const float* pred, const float* target, int64_t n, float* grad, double* loss_dev, void* work,
                     void* stream);
int gbofdft_nn_sqerr_work_bytes(int64_t* bytes);
/* Adam step on FP32 master weights w (moments m, v; step >= 1); refreshes the BF16 copy when w_bf16 != NULL. */
int gbofdft_nn_adam(float* w, const float* g, float* m, float* v, void* w_bf16, int64_t n, double lr, double b1,
                    double b2, double eps, int step, void* stream);
int gbofdft_nn_to_bf16(const float* a, void* b, int64_t n, void* stream);

/*
 * Tensor-core (tcgen05) forward convolution of the inner layers: the
 * activations are rounded to BF16, products accumulate in FP32 in tensor
 * memory.  Layer shapes: c_in, c_out in {16, 32, 48, 64} pairs of the
 * network, H a multiple of 16, W of 8 (..._supported returns 1 when a shape
 * has a kernel).  w_packed: the BF16 weights repacked by ..._pack from
 * [c_out][c_in][27] to [tap][c_in / 8][c_out][c_in % 8].  act = 1 applies
 * SiLU to conv + bias; skip (or NULL): a [c_out][D][H][W] tensor added after
 * that; up = 1: in is a (D/2, H/2, W/2) grid read as its nearest-neighbour
 * 2x upsampling.  nstore <= c_out: only output channels [0, nstore) are
 * written (bias, skip and out hold nstore channels; a narrower layer runs as a
 * c_out-wide one with zero weights).  err: device int, set non-zero if a wait
 * inside the kernel timed out (the output is then incomplete).
 */
int gbofdft_nn_conv3d_tc_supported(int cin, int cout, int D, int H, int W);
int gbofdft_nn_conv3d_tc_pack(const void* w_bf16, int cin, int cout, void* w_packed, void* stream);
int gbofdft_nn_conv3d_tc(const void* in, int cin, const void* w_packed, const void* bias, void* out, int cout,
                         int nstore, int D, int H, int W, int act, const void* skip, int up, int* err, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GBOFDFT_H */
