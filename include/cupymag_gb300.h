/*
 * cupymag_gb300 -- C-ABI of the GB300 (sm_103a) kernels for CuPyMag's
 * Gauss-Seidel-projection LLG time step.
 *
 * Every function takes plain device pointers, sizes and a cudaStream_t passed
 * as void*; launches are asynchronous on that stream.  Functions return a
 * status code (cpm_status); on CPM_CUDA_ERROR / CPM_BAD_ARG the message is
 * available from cpm_last_error_string() (per calling thread).  The library
 * never allocates user-visible memory: solvers take a caller-owned workspace
 * whose size is given by cpm_cg_workspace_bytes().
 *
 * Layouts (as in the reference): a 3-vector field (n,3) and a Voigt strain
 * (n,6) are row-major "AoS" arrays; the elastic displacement u is the block
 * vector [ux | uy | uz] of length 3n; the eigenstrain E0 is node-interleaved
 * (6n).  CSR matrices use int32 column indices and int32 or int64 row
 * pointers, FP64 values (plus an optional FP32 copy of the values for the
 * mixed-precision solver).
 */
#ifndef CUPYMAG_GB300_H
#define CUPYMAG_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  CPM_OK = 0,
  CPM_NOT_CONVERGED = 1,   /* maxiter reached (linear_solvers.py:64-74 raises) */
  CPM_BARRIER_TIMEOUT = 2, /* a bounded grid-barrier wait ran out */
  CPM_NONFINITE = 3,       /* NaN/Inf met in a CG scalar */
  CPM_BAD_ARG = 4,
  CPM_CUDA_ERROR = 5
} cpm_status;

/* Sparse matrix in CSR form (device pointers).  vals32 may be NULL. */
typedef struct {
  int64_t rows, cols, nnz;
  const void *indptr;      /* int32_t[rows+1] or int64_t[rows+1] */
  int32_t indptr_is64;
  const int32_t *indices;  /* int32_t[nnz], sorted per row */
  const double *vals;      /* double[nnz] */
  const float *vals32;     /* float[nnz] or NULL */
  int64_t max_row_nnz;     /* longest row (0: unknown; sets the rows-per-thread-group split) */
} cpm_csr;

/* Per-solve result written by the solvers (device memory). */
typedef struct {
  int32_t status;          /* cpm_status of the solve */
  int32_t iters[3];        /* CG iterations per right-hand side */
  int32_t outer;           /* reliable updates (mixed precision) */
  int32_t df_updates;      /* of those, updates on a double-float residual (cpm_cg_solve_stencil) */
  double resid[3];         /* final ||r|| per right-hand side */
  double bnorm[3];         /* ||b|| per right-hand side */
} cpm_cg_info;

/* Solver controls. */
typedef struct {
  double tol;              /* stop when ||r|| <= tol * ||b||  (cupyx cg semantics) */
  int32_t maxiter;
  int32_t use_init_host;   /* x holds the initial guess (if use_init_dev is NULL) */
  const int32_t *use_init_dev; /* device flag read at launch time, or NULL */
  int32_t precision;       /* 0 = FP64 CG, 1 = FP32 CG with reliable updates on FP64 (or proven double-float) residuals */
  double inner_tol;        /* reliable update when the FP32 residual fell by this factor (default 0.1) */
  int32_t max_outer;       /* unused (kept for layout) */
  int32_t form;            /* FP32 stencil solvers: CPM_CG_FORM_DEFAULT (= three grid barriers per
                              iteration), CPM_CG_FORM_THREE_BARRIER, CPM_CG_FORM_TWO_BARRIER;
                              FFT solves: CPM_CG_FORM_DEFAULT (direct refinement with an anchored
                              plan) or CPM_CG_FORM_FFT_PCG */
  double barrier_timeout_s;/* bound on every grid-barrier wait (seconds) */
  /* Residual carry of the FFT direct solve (cpm_cg_solve_stencil_fft with an anchored plan; all three
   * NULL: none).  carry_b and carry_t hold one vector each of the system's size, carry_valid one int,
   * all on the device.  Each FP64 residual pass stores t = b - A x in carry_t and the solve's b in
   * carry_b; at exit the solve sets *carry_valid to 1 when its final x is the x of its last residual
   * pass (converged, or stopped at maxiter) and to 0 otherwise.  A warm-started solve that finds
   * *carry_valid = 1 takes (b - carry_b) + carry_t as its first residual, three vector reads in place
   * of an FP64 product; if that residual already meets the stopping test an FP64 residual confirms it.
   * The caller zeroes *carry_valid whenever x changes other than by the solve that wrote the carry. */
  double *carry_b;
  double *carry_t;
  int32_t *carry_valid;
} cpm_cg_opts;

/* Iteration forms of the FP32 stencil CG (cpm_cg_opts.form).  Both run CG to
 * the same FP64 stopping test; the two-barrier form keeps s ~ A p beside p and
 * forms A r in its one product, so an iteration needs one reduction of four
 * sums instead of two reductions and a third barrier.  The two-barrier form is
 * opt-in: on GB300 it measured slower per iteration, and its FP32 recurrences
 * drift enough to stall the 128^3 elastic and demag solves. */
enum { CPM_CG_FORM_DEFAULT = 0, CPM_CG_FORM_THREE_BARRIER = 1, CPM_CG_FORM_TWO_BARRIER = 2, CPM_CG_FORM_FFT_PCG = 3 };

/* ---- library ---- */
const char *cpm_version(void);
const char *cpm_last_error_string(void);
int cpm_device_sm_count(int device);

/* ---- sparse matrix-vector products ----
 * Replaces the cupyx CSR `A @ x` used throughout the step
 * (cupymag/core/Micromagnetics.py:123,166,217-219,227,233,280-288).
 * y[:, k] = alpha * A x[:, k] for k < nvec (nvec 1 or 3, (n,nvec) layout). */
int cpm_spmv_csr(const cpm_csr *A, const double *x, double *y, double alpha, int nvec, void *stream);

/* Same-pattern triple product (Fx, Fy, Fz share indptr/indices).
 * mode 0 (cupymag/utils/compute_derivatives.py:36-58, compute_Hd_from_U):
 *      y[i, k] = alpha * (A_k x)_i,  x (n,), y (n,3).
 * mode 1 (cupymag/core/Micromagnetics.py:166-168, demag right-hand side):
 *      y[i] = alpha * sum_k (A_k (x[:,k] - shift[k]))_i,  y[pin] = 0 if pin >= 0,
 *      x (n,3), shift = device double[3] or NULL, y (n,). */
int cpm_spmv_csr_multi(const cpm_csr *A, const double *vals_y, const double *vals_z, const double *x,
                       double *y, double alpha, int mode, const double *shift, int64_t pin, void *stream);

/* ---- conjugate gradient ----
 * Replaces cupymag/solvers/linear_solvers.py:20-74 (cupyx cg): unpreconditioned
 * CG, x0 used only when use_init, ||b|| == 0 returns b, stop on
 * ||r|| <= tol ||b|| checked after each update, info != 0 at maxiter.
 * One persistent cooperative launch does SpMV, dot products and vector updates
 * for every iteration; nrhs 1 or 3 independent right-hand sides share A
 * ((n,nrhs) layout), each with its own scalars and stopping test. */
size_t cpm_cg_workspace_bytes(int64_t n, int nrhs, int precision);
int cpm_cg_solve(const cpm_csr *A, const double *b, double *x, int nrhs, const cpm_cg_opts *opts,
                 void *workspace, size_t workspace_bytes, cpm_cg_info *info_dev, void *stream);

/* Same solve as cpm_cg_solve, for callers that cannot allocate device memory:
 * code that runs while another component owns all allocation (a fixed memory
 * arena or pool handed out by a host application, an embedding that forbids
 * cudaMalloc after start-up), or that must not add allocation calls to a path
 * it has already sized.  It takes no workspace: its scratch is a fixed 32 MiB
 * array in device memory, built into this library, which every GPU that loads
 * the library holds until the process exits.  It calls no cudaMalloc,
 * cudaFree or allocating library routine.  The limit is about 1.03 million
 * values of n * nrhs in FP64 (1.65 million in the FP32-refinement form); larger
 * solves are rejected with CPM_BAD_ARG and a message.  The first call on each
 * device looks up the array's device address (cudaGetSymbolAddress) with that
 * device current and keeps it for the life of the process; make that first
 * call before any stream capture.  The kept address does not survive a reset
 * of the device's context (cudaDeviceReset, or a primary context released and
 * created again): do not call this entry point after one.  All calls
 * share the one array and it keeps the last call's contents (the solver clears
 * what must start at zero), so calls whose kernels overlap on the GPU -- on
 * different streams or different host threads -- race and give wrong results.
 * No counterpart in the reference. */
int cpm_cg_solve_noalloc(const cpm_csr *A, const double *b, double *x, int nrhs, const cpm_cg_opts *opts,
                         cpm_cg_info *info_dev, void *stream);

/* ---- matrix-free periodic hex operators ----
 * The structured hex grid's operators are 27-point periodic stencils; these
 * entry points apply them (and run the same CG on them) without streaming
 * CSR values.  coef[(a*ncomp + b)*27 + d], d = (dx+1)*9 + (dy+1)*3 + (dz+1),
 * is the coefficient between component a of DOF p and component b of DOF
 * p + (dx,dy,dz) (wrapped), DOF = (i*ny + j)*nz + k -- exactly the values of
 * the CSR rows built by structured assembly (assemble_demag.py:186-233,
 * assemble_Gauss_Seidel.py:163-214, assemble_elasticity.py:350-459).  The
 * coefficients are host values (this struct lives in host memory); the
 * kernels receive them as launch parameters.
 * flags (device uint8 per DOF, may be NULL): 1 = unit row (anchors, defect
 * DOFs of A1/A2), 2 = empty row (defect rows of the mass matrix), 4 = the
 * DOF's column is dropped from every other row (final_assembly.py:59-158),
 * 8 = some neighbour of this DOF carries flag 4 (its row takes the checked
 * path; all other rows skip the per-neighbour flag tests), 16 = some
 * neighbour carries flag 4 without flag 1 (the FP32 refinement solver keeps
 * its vectors zero at pinned DOFs, flags 1|4, and tests columns only in rows
 * with flag 16). */
typedef struct {
  int32_t nx, ny, nz;      /* cells per axis (>= 3), n = nx*ny*nz DOFs */
  int32_t ncomp;           /* 1: scalar operator; 3: elastic operator on [ux|uy|uz] */
  double coef[243];        /* 27*ncomp*ncomp FP64 coefficients (FP32 copies are rounded from these) */
  const uint8_t *flags;    /* per-DOF row/column flags, or NULL */
} cpm_stencil;

/* y = alpha * A x (FP64); nvec 1 or 3 ((n,nvec) layout) for ncomp = 1. */
int cpm_stencil_apply(const cpm_stencil *S, const double *x, double *y, double alpha, int nvec, void *stream);

/* y = A x in FP32 with FP32 coefficients: the product of the FP32 refinement
 * form's inner iterations (the A @ p of the cupyx CG that solve_cg calls,
 * cupymag/solvers/linear_solvers.py:60-62).
 * form 0: per DOF; 1: quads of 4 DOFs along z with aligned vector loads
 * (nz % 4 == 0, 4-byte aligned flags, 16-byte aligned x and y); 2: quads
 * with scalar loads (any nz; 4-byte aligned flags).  Every form gives the
 * same bits per output. */
int cpm_stencil_apply32(const cpm_stencil *S, const float *x, float *y, int nvec, int form, void *stream);

/* cpm_cg_solve on a stencil operator: same semantics, options and info;
 * workspace size cpm_cg_workspace_bytes(n * ncomp, nrhs, precision) at least.
 * With cpm_cg_stencil_workspace_bytes(n * ncomp, nrhs, precision) bytes (one
 * more float vector in the FP32 form), the FP32 form of a scalar operator may
 * compute its reliable updates' residuals in double-float arithmetic (x held
 * as two floats, about 48 significant bits) where their error provably stays
 * below a quarter of tol * ||b||: the stencil's symbol bounds the operator's
 * smallest eigenvalue, and the solve checks that every flagged row is pinned
 * (identity row, excluded column).  Such a residual decides convergence only
 * when it is below tol * ||b|| by more than its error bound; closer to the
 * threshold the solve takes FP64 residuals. */
int cpm_cg_solve_stencil(const cpm_stencil *S, const double *b, double *x, int nrhs, const cpm_cg_opts *opts,
                         void *workspace, size_t workspace_bytes, cpm_cg_info *info_dev, void *stream);
size_t cpm_cg_stencil_workspace_bytes(int64_t unknowns, int nrhs, int precision);
/* The bound behind that choice, as a multiple of ||b||: 2 g sum|c| / sigma_min with g = 128 * 2^-48 and
 * sigma_min a lower bound of the stencil's symbol (its part even along every axis is minimised over the 8
 * corners cos theta = +-1, the rest bounded by the sum of its magnitudes); -1 where sigma_min <= 0 or the
 * stencil is not scalar.  Host only (reads S->coef and S->ncomp). */
double cpm_stencil_df_error_bound(const cpm_stencil *S);

/* ---- block-diagonal CG over many stencil systems (the serving loop) ----
 * Replaces, for a batch of independent runs, one solve_cg call per run
 * (cupymag/solvers/linear_solvers.py:20-74, called from
 * cupymag/core/Micromagnetics.py:123,170,223,229,235,290) with one launch.
 * All systems of a batch have the same operator kind (ncomp, nrhs) and the
 * same coefficient table; grids, flags, tolerances, maxiter and warm-start
 * flags are per system.  Each system keeps cupyx cg semantics and gets its
 * own cpm_cg_info.  A system's result does not depend on the other systems
 * of the batch (bit-for-bit). */
typedef struct {
  int32_t nx, ny, nz;      /* cells per axis (>= 3) */
  int32_t maxiter;         /* >= 1 */
  double tol;              /* stop when ||r|| <= tol * ||b|| */
  const uint8_t *flags;    /* per-DOF flags as in cpm_stencil, or NULL */
  const double *b;         /* device right-hand side(s) */
  double *x;               /* device solution (initial guess when *use_init_dev != 0) */
  const int32_t *use_init_dev; /* device warm-start flag, or NULL (cold start) */
  cpm_cg_info *info;       /* device result record of this system */
  void *work;              /* device work vectors, cpm_batch_work_bytes() bytes, 256-byte aligned */
} cpm_batch_system;

/* Launch plan built by cpm_batch_plan_build (host struct; `dev` is device memory). */
typedef struct {
  void *dev;
  int64_t bytes;
  int32_t nsys, grid, ncomp, nrhs, precision, total_chunks;
  double coef[243];
} cpm_batch_plan;

/* Work-vector bytes of one system on an nx x ny x nz grid; 0 for invalid dimensions. */
int64_t cpm_batch_work_bytes(int32_t nx, int32_t ny, int32_t nz, int32_t ncomp, int32_t nrhs, int32_t precision);

/* Device bytes of the plan for these systems (CTA assignment, partial sums, tables). */
int cpm_batch_plan_bytes(const cpm_batch_system *sys, int32_t nsys, int32_t ncomp, int32_t nrhs,
                         int32_t precision, int64_t *bytes);

/* Build the plan into plan_dev (256-byte aligned, plan_bytes from
 * cpm_batch_plan_bytes): copies the system table to the device and waits for
 * the copy on `stream`, so it is called outside stream capture, once per
 * batch composition.  coef: host, 27*ncomp*ncomp FP64 coefficients. */
int cpm_batch_plan_build(const cpm_batch_system *sys, int32_t nsys, int32_t ncomp, int32_t nrhs,
                         int32_t precision, const double *coef, void *plan_dev, int64_t plan_bytes,
                         cpm_batch_plan *plan, void *stream);

/* Solve every system of the plan in one cooperative launch on `stream`
 * (a memset and a kernel: the call can be captured in a CUDA graph).  opts:
 * inner_tol and barrier_timeout_s are used; tolerances, maxiter and
 * warm-start flags come from the systems. */
int cpm_cg_solve_blockdiag(const cpm_batch_plan *plan, const cpm_cg_opts *opts, void *stream);

/* ---- device assembly (unstructured meshes) ----
 * Duplicate summation of the COO -> CSR conversion that the reference leaves
 * to cupyx (cupymag/utils/final_assembly.py:160-205, assemble_stiffness_matrix
 * and assemble_mass_matrix): vals_sorted holds the element entries ordered by
 * a stable sort on (row, col); seg_start[0..nseg] delimits the runs of equal
 * (row, col); out[s] is the in-order sum of run s (deterministic). */
int cpm_coo_segment_sum(const double *vals_sorted, const int64_t *seg_start, int64_t nseg, double *out,
                        void *stream);

/* ---- LLG step kernels (cupymag/core/Micromagnetics.py:110-307) ---- */
typedef struct {
  double K1, elasC1, elasC2, elasC3, lambda100;
  double Nd[3];            /* demagnetisation factors */
  double Hext[3];          /* applied field (normalised) */
  double R[9];             /* [100] -> [111] rotation, row-major; used when rot111 */
  int32_t rot111;
  int32_t has_E;           /* 0: strain is identically zero (ME off) */
  const double *hext_sched;/* device (steps, 3) field schedule, or NULL to use Hext */
  const int32_t *hext_step;/* device index of the current step into hext_sched */
} cpm_field_params;

/* Effective field of Micromagnetics.py:175-215 (rot111 variant :190-211) at
 * magnetisation mm (n,3): anisotropy + magnetoelastic terms from the strain E
 * (n,6, or NULL when has_E = 0), half of the demag field H~ (n,3) and of
 * H_bar = -Nd * avg_m (avg_m: device double[3]), plus Hext.  Writes the field
 * f (n,3) when f != NULL and t = f * dt + mm (n,3). */
int cpm_llg_field(const cpm_field_params *P, int64_t n, const double *mm, const double *E, const double *Ht,
                  const double *avg_m, double dt, double *f, double *t, void *stream);

/* End-of-step record for runs driven by a device step counter (a captured
 * step replayed along a field sweep): hist[4*s + 0..2] = avg_m,
 * hist[4*s + 3] = sumsq, then *step_dev = s + 1, for s = *step_dev < capacity.
 * The reference appends the same values to its hysteresis output
 * (Micromagnetics.py:303-317). */
int cpm_record_step(const double *avg_m, const double *sumsq, double *hist, int32_t *step_dev, int32_t capacity,
                    void *stream);

/* Gauss-Seidel star updates (Micromagnetics.py:225-237).  g (n,3) holds
 * (g1n, g2n, g3n), f (n,3) the field from cpm_llg_field, mstar (n,3) the star
 * magnetisation being built:
 *   stage 1: m1* = m1 + g2n m3 - g3n m2,   out = f1 dt + m1*  (n)
 *   stage 2: m2* = m2 + g3n m1* - g1* m3,  out = f2 dt + m2*  (n)
 *   stage 3: m3* = m3 + g1* m2* - g2* m1*. */
int cpm_gs_star(int stage, int64_t n, const double *m, const double *g, const double *g1star,
                const double *g2star, const double *f, double dt, double *mstar, double *out, void *stream);

/* Renormalisation step of Micromagnetics.py:292-307: m = mss / |mss| (0 where
 * |mss| < 1e-14), m = 0 where defect_mask[i] (uint8, may be NULL),
 * sumsq = sum (m - m_prev)^2, m_prev = m, *use_init_dev = sumsq < thresh (if
 * not NULL), avg_out[3] = <m> = (w . m) / volume.  scratch: device doubles,
 * cpm_volavg_scratch_doubles() of them, zero-initialised once. */
int cpm_renorm_sumsq(int64_t n, const double *mss, const uint8_t *defect_mask, double *m, double *m_prev,
                     const double *w, double volume, double thresh, double *sumsq_out, double *avg_out,
                     int32_t *use_init_dev, double *scratch, void *stream);

/* Volume average (cupymag/utils/volume_average.py:155-216) in per-DOF weight
 * form: out[c] = (sum_i w_i f[i,c]) / volume for ncomp in {1,3,6} interleaved
 * components; with R9 != NULL (ncomp = 3) the average of f R.  The weights fold
 * the reference's quadrature (N at Gauss points times |detJ| w) per DOF.
 * scratch as for cpm_renorm_sumsq. */
size_t cpm_volavg_scratch_doubles(int ncomp);
int cpm_volavg(int64_t n, int ncomp, const double *f, const double *w, double volume, const double *R9,
               double *out, double *scratch, void *stream);

/* ---- circulant (FFT) preconditioned FP32 CG inside FP64 refinement ----
 * The refinement form of the elastic and demag solves (the A @ p CG of
 * solve_cg, cupymag/solvers/linear_solvers.py:59-74, with the preconditioner
 * argument M that solve_cg passes to cupyx cg): on the periodic hex grid these
 * operators are block-circulant except for the anchor at DOF 0, so the inverse
 * of the circulant part, applied with 3D DFTs, leaves a perturbation of rank
 * <= 9 and preconditioned CG converges in tens of iterations where plain CG
 * needs thousands.  The plan holds the DFT twiddles and the inverse symbol
 * (per wave vector k: 1 float, or the 6 floats of a symmetric 3x3 block; the
 * singular k = 0 block is replaced by the operator's diagonal).  Every line
 * length works (any prime factors).  The host struct is filled by the build
 * call; `dev` is caller-owned device memory of cpm_fft_precond_bytes().
 *
 * Layouts of the spectrum: SLAB keeps the nz/2 + 1 non-negative z frequencies
 * of the real field and does the z and y DFTs of one x-plane in one pass
 * (three passes per apply; needs an x-plane's half spectrum, about
 * ny (nz/2 + 1) complex values twice, in the 227 KB of shared memory of an SM:
 * every grid up to 160^3); PASSES does five passes over the full complex field
 * (any grid).  AUTO picks SLAB where it fits. */
enum {
  CPM_FFT_LAYOUT_AUTO = 0,
  CPM_FFT_LAYOUT_SLAB = 1,
  CPM_FFT_LAYOUT_PASSES = 2
};

typedef struct {
  int32_t nx, ny, nz, ncomp;
  void *dev;               /* device memory of the plan (twiddles, inverse symbol) */
  int64_t bytes;
  int32_t npass[3];        /* radix passes per axis */
  int32_t radix[3][16];
  int32_t layout;          /* in: the requested CPM_FFT_LAYOUT_*; out: the plan's (SLAB or PASSES) */
  int32_t anchor;          /* in: the node whose rows and columns the operator pins (flags 1|4 there,
                              no flag but 8 elsewhere; the build checks), or -1 */
} cpm_fft_precond;

/* Device bytes of a plan for an nx x ny x nz grid (ncomp 1 or 3); 0 when unsupported. */
int64_t cpm_fft_precond_bytes(int32_t nx, int32_t ny, int32_t nz, int32_t ncomp);
/* Build the plan of stencil operator S into dev (256-byte aligned), in the layout P->layout asks
 * for (CPM_BAD_ARG for SLAB on a grid it does not fit). */
int cpm_fft_precond_build(const cpm_stencil *S, void *dev, int64_t bytes, cpm_fft_precond *P, void *stream);
/* z = M r alone (FP32; r, z of ncomp*n values, [x|y|z] blocks for ncomp 3); work: a complex
 * buffer of 8 * ncomp * n bytes, 16-byte aligned. */
int cpm_fft_precond_apply(const cpm_fft_precond *P, const float *r, float *z, void *work, int64_t work_bytes,
                          void *stream);
/* The solve: same contract as cpm_cg_solve_stencil (b, x FP64, tol, maxiter, warm-start flag,
 * stopping test ||b - A x|| <= tol ||b|| on the FP64 residual, zero b returns b, the
 * reference's status on maxiter), for nrhs 1.
 *
 * With an anchored plan (P->anchor >= 0) the solve is direct refinement: A = [[I, 0], [0, C_rr]]
 * (C the circulant, node a pinned) is inverted exactly by e = C+ t~ + 1 (t_a - (C+ t~)_a), where
 * t~ = t plus C_ra t_a on the free nodes and minus the sum of those at a (so t~ sums to zero,
 * orthogonal to the translations that span ker C), C+ t~ the FFT apply.  Each outer step is one
 * FP64 residual and one FP32 FFT solve; info->iters[0] and info->outer count the steps.
 * Otherwise (or with opts->form = CPM_CG_FORM_FFT_PCG) FP32 CG preconditioned by C'^-1 runs
 * inside the refinement: opts->inner_tol is the residual drop of each inner solve (default
 * 1e-4); info->iters[0] counts inner iterations and info->outer the FP64 residuals. */
size_t cpm_cg_fft_workspace_bytes(int32_t nx, int32_t ny, int32_t nz, int32_t ncomp);
int cpm_cg_solve_stencil_fft(const cpm_stencil *S, const cpm_fft_precond *P, const double *b, double *x,
                             const cpm_cg_opts *opts, void *workspace, size_t workspace_bytes,
                             cpm_cg_info *info_dev, void *stream);

/* ---- matrix-free derivative and coupling operators (structured hex grids) ----
 * On a grid of identical unit cells the derivative matrices F_i (F_i[p,q] =
 * integral of N_p dN_q/dx_i, cupymag/physics/assemble_demag.py:95-184) and the
 * magnetoelastic coupling F_el = B^T C S (assemble_elasticity.py:268-459) are
 * 27-point periodic stencils, d = (dx+1)*9 + (dy+1)*3 + (dz+1) as for
 * cpm_stencil.  These entry points apply them without the CSR matrices (FP64;
 * results equal the CSR products to rounding).  Host structs; coefficients
 * travel as launch parameters. */
typedef struct {
  int32_t nx, ny, nz;      /* cells per axis (>= 3) */
  int32_t pad;
  double fx[27], fy[27], fz[27];  /* stencils of Fx, Fy, Fz */
} cpm_deriv_stencil;

/* Matrix-free form of cpm_spmv_csr_multi: mode 0 (compute_Hd_from_U,
 * cupymag/utils/compute_derivatives.py:36-58): y[i,k] = alpha (F_k x)_i, x (n,),
 * y (n,3); mode 1 (demag right-hand side, cupymag/core/Micromagnetics.py:166-168):
 * y[i] = alpha sum_k (F_k (x[:,k] - shift[k]))_i, y[pin] = 0 if pin >= 0,
 * x (n,3), shift device double[3] or NULL. */
int cpm_stencil_deriv(const cpm_deriv_stencil *D, const double *x, double *y, double alpha, int mode,
                      const double *shift, int64_t pin, void *stream);

/* Matrix-free form of cpm_strain_from_u (compute_derivatives.py:60-125): E
 * (n,6) Voigt strain from u = [ux|uy|uz]; R9 (row-major 3x3, device) or NULL.
 * E 16-byte aligned. */
int cpm_stencil_strain(const cpm_deriv_stencil *D, const double *u, const double *R9, double *E, void *stream);

typedef struct {
  int32_t nx, ny, nz;      /* cells per axis (>= 3) */
  int32_t anchor;          /* 1: rows of DOF 0 (b_el[0], b_el[n], b_el[2n]) are empty, as the reference's
                              F_el anchors them (assemble_elasticity.py:461-527) */
  double coef[486];        /* coef[(a*6 + v)*27 + d]: displacement component a, Voigt column v */
} cpm_fel_stencil;

/* b_el (3n, [x|y|z]) = F_el E0 with E0 (6n, node-interleaved Voigt, 16-byte
 * aligned): the right-hand side of the elastic solve (Micromagnetics.py:123)
 * without the 162-non-zero-per-row CSR matrix. */
int cpm_stencil_fel(const cpm_fel_stencil *F, const double *E0, double *b_el, void *stream);

/* Magnetostrictive eigenstrain E0 (6n, node-interleaved Voigt with doubled
 * shears), cupymag/utils/final_assembly.py:208-266.  With R9/M36 (both or
 * neither) it is built from m100 = m R and rotated per node by M^T
 * (Micromagnetics.py:112-119). */
int cpm_build_E0(int64_t n, const double *m, double lam100, double lam111, const double *R9,
                 const double *M36, double *E0, void *stream);

/* Strain from displacement (cupymag/utils/compute_derivatives.py:60-125): E
 * (n,6) from the shared-pattern derivative matrices Fx (this CSR) and the
 * value arrays of Fy, Fz applied to u = [ux|uy|uz]; R9 (row-major 3x3) or NULL. */
int cpm_strain_from_u(const cpm_csr *Fx, const double *vals_y, const double *vals_z, const double *u,
                      const double *R9, double *E, void *stream);

/* Micromagnetics.py:132-162: E = (E - <E>) + E_bar, then E M^{-T} when rot111.
 * E_bar is formed on the device from <m100> (or <m> without rotation; device
 * double[3]), lam100, lam111 and S sigma (device double[6]), rotated by M when
 * rot111.  avgE: device double[6]; M36, MinvT36: device row-major 6x6. */
int cpm_strain_finalize(int64_t n, double *E, const double *avgE, const double *avg_m100, double lam100,
                        double lam111, const double *Ebar_sigma6, const double *M36, const double *MinvT36,
                        int rot111, void *stream);

#ifdef __cplusplus
}
#endif

#endif
