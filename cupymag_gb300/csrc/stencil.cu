// Matrix-free periodic hex operators and the conjugate gradient on them (sm_103a).
//
// Every cell of the structured hex grid is the same unit cube, so each
// assembled operator is a 27-point periodic stencil whose coefficients are
// exactly the values the CSR rows carry (physics/structured_hex.py builds
// both from one element matrix).  Applying the stencil instead of streaming
// the CSR removes the matrix traffic (12 bytes per non-zero; 6.1 GB per
// elastic product at 128^3), leaving the vectors, which the 126 MB L2 mostly
// holds.  The anchor and defect modifications are per-DOF flags:
//   kRowIdentity  row is the unit row (anchors, defect DOFs of A1/A2)
//   kRowZero      row is empty (defect rows of the mass matrix F1)
//   kColExcluded  the DOF's column is empty in every other row
// which reproduces the CSR operators' action exactly, up to summation order.
//
// Vector layouts: scalar operators (nc = 1) act on (n, nrhs) interleaved
// vectors; the elastic operator (nc = 3) acts on one block vector
// [ux | uy | uz] of length 3n with coefficient blocks c[(a*3 + b)*27 + d].
//
// The solver is the same cupyx-semantics CG as csrc/cg.cu (three phases per
// iteration, bounded grid barriers, fixed-order reductions), in FP64
// (precision 0) or in FP32 with FP64 reliable updates (precision 1): the
// residual is periodically replaced by b - A x computed with the FP64
// coefficients and the FP64 x, so the stopping test ||b - A x|| <= tol ||b||
// is the FP64 one, while the iterations run on FP32 vectors with FP32
// coefficients and FP64 dot accumulation.  GB300 issues FP32 FMAs at many
// times its FP64 rate, so the FP32 iterations are bound by vector traffic.
#include <algorithm>
#include <cmath>

#include "stencil_ops.cuh"

namespace cpm {

struct StencilCG {
  StencilOp S;
  const double *b;
  double *x;
  double tol;
  int maxiter;
  int use_init_host;
  const int *use_init_dev;
  double inner_tol;
  int max_outer;
  double *r, *p, *q;           // FP64 vectors (precision 0)
  float *r32, *p32, *q32, *d32;  // FP32 vectors (precision 1); the two-barrier form uses q32 as w = A r
  float *s32;                    // two-barrier form: s ~ A p
  double *part;
  GridBarrier *bar;
  cpm_cg_info *info;
  unsigned long long timeout_ns;
  int64_t dofs_per_cta;
  int quads;  // nz % 4 == 0, 4-byte aligned flags, 16-byte aligned x: the FP32 phases run on quads
  float *xh, *xl;     // x split into floats hi + lo for double-float residual passes (null: FP64 only)
  df::DF cdf[27];     // the scalar coefficients as double-float values
  double df_err;      // error bound of a double-float residual as a multiple of ||b|| (<= 0: off)
};

// Number of independent systems (each with its own CG scalars).
template <int NC, int NR>
__host__ __device__ constexpr int n_systems() { return NC == 1 ? NR : 1; }

template <int NC, int NR>
__device__ __forceinline__ int sys_of(int comp) { return NC == 1 ? comp : 0; }

// ---------------------------------------------------------------- FP64 stencil CG
template <int NC, int NR>
__global__ void __launch_bounds__(kCGThreads) cg_stencil_fp64_kernel(const __grid_constant__ StencilCG a) {
  constexpr int U = NC * NR;
  constexpr int NS = n_systems<NC, NR>();
  __shared__ double s_red[2 * 3][kCGWarps];
  const int64_t n = a.S.n;
  const int64_t d0 = min(n, (int64_t)blockIdx.x * a.dofs_per_cta);
  const int64_t d1 = min(n, d0 + a.dofs_per_cta);
  const bool use_init = a.use_init_dev ? (__ldcg(a.use_init_dev) != 0) : (a.use_init_host != 0);
  const unsigned long long tns = a.timeout_ns;
  int par = 0;

  double v[2 * NS];
#pragma unroll
  for (int j = 0; j < 2 * NS; ++j) v[j] = 0.0;
  for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
    double y[U];
    if (use_init) apply<double, NC, NR>(a.S, a.x, (int)dof, y);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = uidx<NC, NR>(n, dof, u);
      const double bi = a.b[i];
      const double ri = use_init ? bi - y[u] : bi;
      a.r[i] = ri;
      a.p[i] = ri;
      if (!use_init) a.x[i] = 0.0;
      v[sys_of<NC, NR>(u)] = fma(bi, bi, v[sys_of<NC, NR>(u)]);
      v[NS + sys_of<NC, NR>(u)] = fma(ri, ri, v[NS + sys_of<NC, NR>(u)]);
    }
  }
  if (!grid_sum<2 * NS>(v, a.part, par, a.bar, tns, s_red)) {
    set_status(a.info, CPM_BARRIER_TIMEOUT);
    return;
  }
  double atol[NS], rho[NS], resid[NS];
  int active[NS], iters[NS];
  bool any = false;
#pragma unroll
  for (int j = 0; j < NS; ++j) {
    const double bn = sqrt(v[j]);
    atol[j] = a.tol * bn;
    rho[j] = v[NS + j];
    resid[j] = sqrt(v[NS + j]);
    active[j] = bn != 0.0;
    iters[j] = 0;
    any |= active[j] != 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.info->bnorm[j] = bn;
  }
  if (use_init) {
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads)
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (!active[sys_of<NC, NR>(u)]) a.x[uidx<NC, NR>(n, dof, u)] = a.b[uidx<NC, NR>(n, dof, u)];
  }
  int status = CPM_OK;
  for (int k = 0; any && k < a.maxiter; ++k) {
    if (k > 0 && !grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
    double pq[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) pq[j] = 0.0;
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
      double y[U];
      apply<double, NC, NR>(a.S, a.p, (int)dof, y);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = uidx<NC, NR>(n, dof, u);
        a.q[i] = y[u];
        pq[sys_of<NC, NR>(u)] = fma(a.p[i], y[u], pq[sys_of<NC, NR>(u)]);
      }
    }
    if (!grid_sum<NS>(pq, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
    double alpha[NS];
    bool bad = false;
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      alpha[j] = active[j] ? rho[j] / pq[j] : 0.0;
      if (active[j] && !isfinite(alpha[j])) bad = true;
    }
    if (bad) { status = CPM_NONFINITE; break; }
    double rr[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) rr[j] = 0.0;
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int s = sys_of<NC, NR>(u);
        if (!active[s]) continue;
        const int64_t i = uidx<NC, NR>(n, dof, u);
        a.x[i] = __fma_rn(alpha[s], a.p[i], a.x[i]);
        const double rn = __fma_rn(-alpha[s], a.q[i], a.r[i]);
        a.r[i] = rn;
        rr[s] = fma(rn, rn, rr[s]);
      }
    }
    if (!grid_sum<NS>(rr, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
    any = false;
    double beta[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      beta[j] = 0.0;
      if (!active[j]) continue;
      if (!isfinite(rr[j])) bad = true;
      iters[j] += 1;
      beta[j] = rr[j] / rho[j];
      rho[j] = rr[j];
      resid[j] = sqrt(rr[j]);
      if (resid[j] <= atol[j]) active[j] = 0;
      any |= active[j] != 0;
    }
    if (bad) { status = CPM_NONFINITE; break; }
    if (!any || k + 1 >= a.maxiter) break;
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int s = sys_of<NC, NR>(u);
        if (!active[s]) continue;
        const int64_t i = uidx<NC, NR>(n, dof, u);
        a.p[i] = __fma_rn(beta[s], a.p[i], a.r[i]);
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int st = status;
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      if (st == CPM_OK && active[j]) st = CPM_NOT_CONVERGED;
      a.info->iters[j] = iters[j];
      a.info->resid[j] = resid[j];
    }
    a.info->outer = 0;
    set_status(a.info, st);
  } else if (status != CPM_OK && threadIdx.x == 0) {
    set_status(a.info, status);
  }
}

// ---------------------------------------------------------------- FP32 CG with reliable updates
// Mixed-precision CG with reliable updates (Sleijpen & van der Vorst, 1996):
// the iteration runs on FP32 vectors (p, q, the correction d and the
// recursive residual r) with FP32 stencil coefficients and FP64 dot
// accumulation across threads.  When the recursive residual has fallen by a
// factor delta (inner_tol) below the last true residual -- or below the
// stopping threshold, or at maxiter -- the next iteration's first phase also
// computes the true residual t = b - A64 x with the FP64 coefficients and the
// FP64 x (the direction phase before it folded d into x, own unknowns only):
// t replaces r and rho and decides convergence (the stopping test
// ||b - A x|| <= tol ||b|| is only ever decided on t).  For scalar stencils
// whose symbol bounds the error (df_error_bound) t may be computed in
// double-float arithmetic from x split into two floats (xh, xl, written where x
// changes): 15 FP32 operations per term in place of an FP64 FMA issued at 1/64
// of the FP32 rate.  Such a t decides convergence only when it is below the
// threshold by more than its proven error; within that band of the threshold
// the solve takes FP64 residuals from then on (IRState.exact), and one pass
// serves every pending system, in double-float only when all of them allow it.
// Measured on GB300, 128^3 A1 with three right-hand sides, cold: 3.85 ms per
// solve against 4.19 ms with FP64 residuals, at the same 36 iterations.  The
// 3-RHS double-float pass takes one right-hand side at a time: all three at
// once needed 2 KB of spills at this kernel's 64 registers.  That iteration's direction p was formed from
// the recursive residual, so its step length is the exact line search
// alpha = (t.p) / (p.A p).  The update costs no extra grid barrier.
// info->outer counts the reliable updates.  With nz % 4 == 0 the FP32
// product runs on quads of 4 DOFs along z (apply4_c).  Pinned DOFs (identity
// row, excluded column: the defects of A1/A2, the anchors) decouple: their
// solution is x = b, written when the solve ends; until then x, r, p and q
// stay zero there and their rows' residual is zero, so neither the FP32
// product nor the FP64 residual needs per-neighbour column tests: flagged
// quads keep the register-blocked form (measured on GB300, 128^3 A1 with a
// 16^3 defect: the CTAs holding the defect's quads had made every other CTA
// wait 14 us of a 47 us iteration).  The CG state lives in
// shared memory (IRState), updated by thread 0 after each reduction, so the
// DOF loops keep only alpha/beta and bitmasks in registers.
// 256-thread CTAs, four per SM (measured faster than one 1024-thread CTA per
// SM: the CTA-wide reductions and barriers of 32 warps cost more than the
// extra grid-barrier arrivals of 4x as many CTAs).
constexpr int kIRThreads = 256;

template <int NC, int NR>
__global__ void __launch_bounds__(kIRThreads, 4) cg_stencil_ir_kernel(const __grid_constant__ StencilCG a) {
  constexpr int U = NC * NR;
  constexpr int NS = n_systems<NC, NR>();
  constexpr int TH = kIRThreads;
  __shared__ double s_red[9][TH / kWarp];
  __shared__ IRState st[NS];
  __shared__ float s_ab[NS];
  __shared__ int s_mask[4];  // active, need, error status, double-float pass
  const int64_t n = a.S.n;
  const int64_t d0 = min(n, (int64_t)blockIdx.x * a.dofs_per_cta);
  const int64_t d1 = min(n, d0 + a.dofs_per_cta);
  const bool quads = a.quads != 0;
  const bool use_init = a.use_init_dev ? (__ldcg(a.use_init_dev) != 0) : (a.use_init_host != 0);
  const unsigned long long tns = a.timeout_ns;
  const double *__restrict__ b = a.b;
  double *x = a.x;
  float *r32 = a.r32, *p32 = a.p32, *q32 = a.q32, *d32 = a.d32;
  float *xh = NC == 1 ? a.xh : nullptr, *xl = a.xl;
  int par = 0;

  // ---- prologue: r = b - A64 x (FP64), r32 = p32 = r, d = 0; ||b||, ||r||; with the split form of x,
  // also the split x and a count of the flagged rows that are not pinned
  double v[2 * NS + 1];
#pragma unroll
  for (int j = 0; j < 2 * NS + 1; ++j) v[j] = 0.0;
  for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH) {
    double y[U];
    // a pinned DOF (identity row, excluded column) is solved by x = b, written when the solve ends;
    // until then x, its residual and every FP32 vector stay zero there, so the products need no
    // column tests
    const bool pin = is_pinned(a.S, dof);
    if (xh && a.S.flags) {
      const int fr = a.S.flags[dof] & (kRowIdentity | kRowZero | kColExcluded);
      if (fr && !pin) v[2 * NS] += 1.0;
    }
    if (use_init && !pin) apply<double, NC, NR>(a.S, x, (int)dof, y);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = uidx<NC, NR>(n, dof, u);
      const double bi = b[i];
      const double ri = pin ? 0.0 : use_init ? bi - y[u] : bi;
      if (pin || !use_init) x[i] = 0.0;
      if (xh) split_store((pin || !use_init) ? 0.0 : x[i], xh, xl, i);
      const float rf = (float)ri;
      r32[i] = rf;
      p32[i] = rf;
      d32[i] = 0.0f;
      const int s = sys_of<NC, NR>(u);
      v[s] = fma(bi, bi, v[s]);
      v[NS + s] = fma(ri, ri, v[NS + s]);
    }
  }
  if (!grid_sum<2 * NS + 1>(v, a.part, par, a.bar, tns, s_red, xh ? 2 * NS + 1 : 2 * NS)) {
    set_status(a.info, CPM_BARRIER_TIMEOUT);
    return;
  }
  if (threadIdx.x == 0) {
    int am = 0;
    for (int j = 0; j < NS; ++j) {
      ir_init(st[j], sqrt(v[j]), v[NS + j], a.tol);
      // the error bound holds where every flagged row is pinned (the operator on the free DOFs is a
      // principal submatrix of the circulant one)
      if (xh && v[2 * NS] == 0.0 && a.df_err > 0.0) st[j].dfe = a.df_err * sqrt(v[j]);
      am |= st[j].active << j;
      if (blockIdx.x == 0) a.info->bnorm[j] = sqrt(v[j]);
    }
    s_mask[0] = am;
    s_mask[1] = 0;
    s_mask[2] = CPM_OK;
    s_mask[3] = 0;
  }
  __syncthreads();
  int activem = s_mask[0], needm = 0, dfpass = 0;
  if (use_init) {
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH)
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (!((activem >> sys_of<NC, NR>(u)) & 1)) x[uidx<NC, NR>(n, dof, u)] = b[uidx<NC, NR>(n, dof, u)];
  }
  int status = CPM_OK;
  for (int k = 0; activem && k <= a.maxiter; ++k) {
    if (k > 0 && !grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
    // ---- phase 1: q = A32 p, p.q (FP32 per thread); pending: t = b - A64 x, r32 = t, t.t, t.p
    float pqf[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) pqf[j] = 0.0f;
    if (quads) {
      for (int64_t qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * TH) {
        float y[4][U];
        apply4_c<float, NC, NR, true, true>(a.S, a.S.c32, p32, (int)qd, y);
        quad_store<float, NC, NR>(q32, n, qd, y);
        quad_dot<NC, NR>(p32, n, qd, y, pqf);
      }
    } else {
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH) {
        float y[U];
        apply<float, NC, NR>(a.S, p32, (int)dof, y);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t i = uidx<NC, NR>(n, dof, u);
          q32[i] = y[u];
          pqf[sys_of<NC, NR>(u)] = fmaf(p32[i], y[u], pqf[sys_of<NC, NR>(u)]);
        }
      }
    }
    double pt[3 * NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      pt[j] = (double)pqf[j];
      pt[NS + j] = 0.0;
      pt[2 * NS + j] = 0.0;
    }
    if (needm && dfpass) {
      if constexpr (NC == 1) {
        // double-float residual: x from its split form, the coefficients as hi + lo floats; one
        // right-hand side per pass (four outputs and six values per column in registers)
        const int step = quads ? 4 : 1;
        for (int64_t dof = d0 + step * threadIdx.x; dof < d1; dof += step * TH) {
#pragma unroll 1
          for (int s = 0; s < NR; ++s) {
            if (!((needm >> s) & 1)) continue;
            df::DF yt[4][1];
            if constexpr (NR == 1) {
              const XSplit xs{xh, xl};
              if (quads) apply4_c<df::DF, 1, 1, true, true>(a.S, a.cdf, xs, (int)dof, yt);
              else apply_c<df::DF, 1, 1>(a.S, a.cdf, xs, (int)dof, yt[0]);
            } else {
              const XSplitR xs{xh, xl, NR, s};
              if (quads) apply4_c<df::DF, 1, 1, true, true>(a.S, a.cdf, xs, (int)dof, yt);
              else apply_c<df::DF, 1, 1>(a.S, a.cdf, xs, (int)dof, yt[0]);
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              if (kk > 0 && !quads) break;
              const int64_t i = uidx<NC, NR>(n, dof + kk, s);
              const double t =
                  is_pinned(a.S, dof + kk) ? 0.0 : (b[i] - (double)yt[kk][0].hi) - (double)yt[kk][0].lo;
              r32[i] = (float)t;
              pt[NS + s] = fma(t, t, pt[NS + s]);
              pt[2 * NS + s] = fma(t, (double)p32[i], pt[2 * NS + s]);
            }
          }
        }
      }
    } else if (needm) {
      // d was folded into x by the previous direction phase; pinned rows keep t = 0
      if (quads) {
        for (int64_t qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * TH) {
          double yt[4][U];
          apply4_c<double, NC, NR, true, true>(a.S, a.S.c64, x, (int)qd, yt);
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            const bool pin = is_pinned(a.S, qd + kk);
#pragma unroll
            for (int u = 0; u < U; ++u) {
              const int s = sys_of<NC, NR>(u);
              if (!((needm >> s) & 1)) continue;
              const int64_t i = uidx<NC, NR>(n, qd + kk, u);
              const double t = pin ? 0.0 : b[i] - yt[kk][u];
              r32[i] = (float)t;
              pt[NS + s] = fma(t, t, pt[NS + s]);
              pt[2 * NS + s] = fma(t, (double)p32[i], pt[2 * NS + s]);
            }
          }
        }
      } else {
        for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH) {
          double yt[U];
          apply<double, NC, NR>(a.S, x, (int)dof, yt);
          const bool pin = is_pinned(a.S, dof);
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int s = sys_of<NC, NR>(u);
            if (!((needm >> s) & 1)) continue;
            const int64_t i = uidx<NC, NR>(n, dof, u);
            const double t = pin ? 0.0 : b[i] - yt[u];
            r32[i] = (float)t;
            pt[NS + s] = fma(t, t, pt[NS + s]);
            pt[2 * NS + s] = fma(t, (double)p32[i], pt[2 * NS + s]);
          }
        }
      }
    }
    // t.t and t.p only on an iteration with a pending update (FP64 adds are slow on GB300)
    if (!grid_sum<3 * NS>(pt, a.part, par, a.bar, tns, s_red, needm ? 3 * NS : NS)) {
      status = CPM_BARRIER_TIMEOUT;
      break;
    }
    if (threadIdx.x == 0) {
      int am = 0, bad = 0;
      for (int j = 0; j < NS; ++j) {
        double al;
        bad |= ir_after_pq(st[j], pt[j], pt[NS + j], pt[2 * NS + j], a.maxiter, al, dfpass != 0);
        s_ab[j] = (float)al;
        am |= st[j].active << j;
      }
      if (needm) st[0].updates += 1;
      if (needm && dfpass) st[0].dfupd += 1;
      s_mask[0] = am;
      s_mask[2] = bad ? CPM_NONFINITE : CPM_OK;
    }
    __syncthreads();
    if (s_mask[2] != CPM_OK) { status = s_mask[2]; break; }
    float af[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) af[j] = s_ab[j];
    activem = s_mask[0];
    // ---- phase 2: active: d += alpha p, r32 -= alpha q, r32.r32
    float rrf[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) rrf[j] = 0.0f;
    if (quads) {
      for (int64_t qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * TH)
        quad_update<NC, NR, NS>(n, qd, activem, af, d32, p32, q32, r32, rrf);
    } else {
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int s = sys_of<NC, NR>(u);
          if (!((activem >> s) & 1)) continue;
          const int64_t i = uidx<NC, NR>(n, dof, u);
          d32[i] = fmaf(af[s], p32[i], d32[i]);
          const float rn = fmaf(-af[s], q32[i], r32[i]);
          r32[i] = rn;
          rrf[s] = fmaf(rn, rn, rrf[s]);
        }
      }
    }
    double rr[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) rr[j] = (double)rrf[j];
    if (!grid_sum<NS>(rr, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
    if (threadIdx.x == 0) {
      int nm = 0, bad = 0, dfall = 1;
      for (int j = 0; j < NS; ++j) {
        float be;
        bad |= ir_after_rr(st[j], rr[j], a.inner_tol, a.maxiter, be);
        s_ab[j] = be;
        nm |= st[j].need << j;
        if (st[j].need && !st[j].dfok) dfall = 0;
      }
      s_mask[1] = nm;
      s_mask[2] = bad ? CPM_NONFINITE : CPM_OK;
      // one pass serves every pending system: double-float only when all of them allow it
      s_mask[3] = (nm && dfall) ? 1 : 0;
    }
    __syncthreads();
    if (s_mask[2] != CPM_OK) { status = s_mask[2]; break; }
    needm = s_mask[1];
    dfpass = s_mask[3];
    if (!activem) break;
    float beta[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) beta[j] = s_ab[j];
    // ---- phase 3: p = r32 + beta p; pending updates: x += d, d = 0
    if (quads) {
      for (int64_t qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * TH)
        quad_direction<NC, NR, NS>(n, qd, activem, needm, beta, p32, r32, x, d32, xh, xl);
    } else {
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int s = sys_of<NC, NR>(u);
          const int64_t i = uidx<NC, NR>(n, dof, u);
          if ((activem >> s) & 1) p32[i] = fmaf(beta[s], p32[i], r32[i]);
          if ((needm >> s) & 1) {
            const double xn = x[i] + (double)d32[i];
            x[i] = xn;
            d32[i] = 0.0f;
            if (xh) split_store(xn, xh, xl, i);
          }
        }
      }
    }
  }
  // the pinned DOFs' solution
  if (a.S.flags)
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH)
      if (is_pinned(a.S, dof))
#pragma unroll
        for (int u = 0; u < U; ++u) x[uidx<NC, NR>(n, dof, u)] = b[uidx<NC, NR>(n, dof, u)];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int stt = status;
    for (int j = 0; j < NS; ++j) {
      if (stt == CPM_OK && (st[j].unconv || st[j].active)) stt = CPM_NOT_CONVERGED;
      a.info->iters[j] = st[j].iters;
      a.info->resid[j] = st[j].resid;
    }
    a.info->outer = st[0].updates;
    a.info->df_updates = st[0].dfupd;
    set_status(a.info, stt);
  } else if (status != CPM_OK && threadIdx.x == 0) {
    set_status(a.info, status);
  }
}


// ---------------------------------------------------------------- FP32 CG with two grid barriers per iteration
// The refinement form of cg_stencil_ir_kernel rearranged so that an iteration
// passes two grid barriers instead of three (IR2State in cg_common.cuh has
// the recurrences).  Per iteration:
//   phase B: w = A32 r (the only product), partial r.w; a system in its
//            replacement pass also folds x += d, d = 0 here;
//            -> reduction barrier: g, dl, e, f of every system;
//   phase A: p = r + beta p, s = w + beta s, d += alpha p, r -= alpha s, and the
//            next reduction's partials r.r, r.s, r.p of the new r (own unknowns
//            only); a system due for a reliable update instead computes
//            t = b - A64 (x + d) in FP64, r = t, and the partials of t;
//            -> barrier (the next product reads r at neighbouring DOFs).
// The vector traffic is that of the three-barrier form (44 B per unknown and
// iteration: r gathered and w written in B; r, p, w, s, d read and r, p, s, d
// written in A).  A replacement pass costs one extra pass of both phases with
// an FP64 product; the stopping test is decided on t only, as in the
// three-barrier form.
// Opt-in (CPM_CG_FORM_TWO_BARRIER).  Measured on GB300 it is not faster: cold
// elastic solves took 42.4 us per iteration at 64^3 (three-barrier 35.4) and
// 100.6 us at 128^3 (77.6), where the five FP32 vectors no longer fit the L2;
// and at 128^3 the elastic and demag solves stalled (20000 iterations), as the
// FP32 recurrences for s ~ A p and p.s drift over thousands of iterations.
template <int NC, int NR>
__global__ void __launch_bounds__(kIRThreads, 4) cg_stencil_ir2_kernel(const __grid_constant__ StencilCG a) {
  constexpr int U = NC * NR;
  constexpr int NS = n_systems<NC, NR>();
  constexpr int NV = 4 * NS;  // per system: g, dl, e, f (record slots g: [0,NS), dl: [NS,2NS), e, f after)
  constexpr int TH = kIRThreads;
  __shared__ double s_tot[NV];
  __shared__ double s_w[8][kCGThreads];  // staging of the block sums
  __shared__ IR2State st[NS];
  __shared__ float s_al[NS], s_be[NS];
  __shared__ int s_mask[4];  // update mask, replacement mask, active mask, status
  const int64_t n = a.S.n;
  const int64_t d0 = min(n, (int64_t)blockIdx.x * a.dofs_per_cta);
  const int64_t d1 = min(n, d0 + a.dofs_per_cta);
  const bool quads = a.quads != 0;
  const bool use_init = a.use_init_dev ? (__ldcg(a.use_init_dev) != 0) : (a.use_init_host != 0);
  const unsigned long long tns = a.timeout_ns;
  const int G = gridDim.x;
  const double *__restrict__ b = a.b;
  double *x = a.x;
  float *r32 = a.r32, *p32 = a.p32, *w32 = a.q32, *s32 = a.s32, *d32 = a.d32;
  double *half0 = a.part, *half1 = a.part + kPartHalf;

  // ---- prologue: r = b - A64 x (FP64), r32 = r, p = s = d = 0; ||b||^2, ||r||^2
  double v[2 * NS];
#pragma unroll
  for (int j = 0; j < 2 * NS; ++j) v[j] = 0.0;
  for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH) {
    double y[U];
    if (use_init) apply<double, NC, NR>(a.S, x, (int)dof, y);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = uidx<NC, NR>(n, dof, u);
      const double bi = b[i];
      const double ri = use_init ? bi - y[u] : bi;
      if (!use_init) x[i] = 0.0;
      r32[i] = (float)ri;
      p32[i] = 0.0f;
      s32[i] = 0.0f;
      d32[i] = 0.0f;
      const int sy = sys_of<NC, NR>(u);
      v[sy] = fma(bi, bi, v[sy]);
      v[NS + sy] = fma(ri, ri, v[NS + sy]);
    }
  }
  block_sum_wide<2 * NS>(v, s_tot, s_w);
  // this CTA's record of the prologue reduction (half 0) and the g slots of the
  // first product's reduction (half 1: g = r.r, e = f = 0 since p = s = 0)
  if (threadIdx.x < 2 * NS) half0[(size_t)blockIdx.x * 2 * NS + threadIdx.x] = s_tot[threadIdx.x];
  if (threadIdx.x < NV) {
    const int j = threadIdx.x;
    half1[(size_t)blockIdx.x * NV + j] = j < NS ? s_tot[NS + j] : 0.0;
  }
  if (!grid_sync(a.bar, G, tns)) {
    set_status(a.info, CPM_BARRIER_TIMEOUT);
    return;
  }
  sum_records<2 * NS>(half0, G, v, s_tot, s_w);
  if (threadIdx.x == 0) {
    int am = 0;
    for (int j = 0; j < NS; ++j) {
      ir2_init(st[j], sqrt(v[j]), v[NS + j], a.tol);
      am |= st[j].active << j;
      if (blockIdx.x == 0) a.info->bnorm[j] = sqrt(v[j]);
    }
    s_mask[2] = am;
  }
  __syncthreads();
  int activem = s_mask[2], repm = 0;
  if (use_init) {
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH)
#pragma unroll
      for (int u = 0; u < U; ++u)
        if (!((activem >> sys_of<NC, NR>(u)) & 1)) x[uidx<NC, NR>(n, dof, u)] = b[uidx<NC, NR>(n, dof, u)];
  }
  int status = CPM_OK;
  const int max_pass = 2 * a.maxiter + 8;
  for (int pass = 0; activem && pass < max_pass; ++pass) {
    // ---- phase B: w = A32 r, r.w; replacement passes fold x += d, d = 0
    float dlf[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) dlf[j] = 0.0f;
    if (quads) {
      for (int64_t qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * TH) {
        float y[4][U];
        apply4_c<float, NC, NR>(a.S, a.S.c32, r32, (int)qd, y);
        quad_store<float, NC, NR>(w32, n, qd, y);
        quad_dot<NC, NR>(r32, n, qd, y, dlf);
      }
    } else {
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH) {
        float y[U];
        apply<float, NC, NR>(a.S, r32, (int)dof, y);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t i = uidx<NC, NR>(n, dof, u);
          w32[i] = y[u];
          dlf[sys_of<NC, NR>(u)] = fmaf(r32[i], y[u], dlf[sys_of<NC, NR>(u)]);
        }
      }
    }
    if (repm) {
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH)
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (!((repm >> sys_of<NC, NR>(u)) & 1)) continue;
          const int64_t i = uidx<NC, NR>(n, dof, u);
          x[i] += (double)d32[i];
          d32[i] = 0.0f;
        }
    }
    double dl[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) dl[j] = (double)dlf[j];
    block_sum_wide<NS>(dl, s_tot, s_w);
    double *half = a.part + (size_t)(1 - (pass & 1)) * kPartHalf;  // pass 0 uses half 1
    if (threadIdx.x < NS) half[(size_t)blockIdx.x * NV + NS + threadIdx.x] = s_tot[threadIdx.x];
    if (!grid_sync(a.bar, G, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
    double t[NV];
    sum_records<NV>(half, G, t, s_tot, s_w);
    if (threadIdx.x == 0) {
      int um = 0, rm = 0, am = 0, bad = 0;
      for (int j = 0; j < NS; ++j) {
        float al, be;
        int mode;
        bad |= ir2_after(st[j], t[j], t[NS + j], t[2 * NS + j], t[3 * NS + j], a.inner_tol, a.maxiter, al, be, mode)
                   ? 1 : 0;
        s_al[j] = al;
        s_be[j] = be;
        um |= (mode == 1) << j;
        rm |= (mode == 2) << j;
        am |= st[j].active << j;
      }
      s_mask[0] = um;
      s_mask[1] = rm;
      s_mask[2] = am;
      s_mask[3] = bad ? CPM_NONFINITE : CPM_OK;
    }
    __syncthreads();
    if (s_mask[3] != CPM_OK) { status = s_mask[3]; break; }
    const int updm = s_mask[0];
    repm = s_mask[1];
    activem = s_mask[2];
    if (!activem) break;
    float af[NS], bf[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      af[j] = s_al[j];
      bf[j] = s_be[j];
    }
    // ---- phase A: updates, or the true residual for a replacement pass; partials of the new r
    float gf[NS], ef[NS], ff[NS];
    double gr[3 * NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) gf[j] = ef[j] = ff[j] = 0.0f;
#pragma unroll
    for (int j = 0; j < 3 * NS; ++j) gr[j] = 0.0;
    if (updm) {
      if (quads) {
        for (int64_t qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * TH)
          quad_update2<NC, NR, NS>(n, qd, updm, af, bf, r32, p32, w32, s32, d32, gf, ef, ff);
      } else {
        for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH)
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int sy = sys_of<NC, NR>(u);
            if (!((updm >> sy) & 1)) continue;
            update2_one(uidx<NC, NR>(n, dof, u), af[sy], bf[sy], r32, p32, w32, s32, d32, gf[sy], ef[sy], ff[sy]);
          }
      }
    }
    if (repm) {
      const XPlusD xd{x, d32};
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += TH) {
        double yt[U];
        apply_c<double, NC, NR>(a.S, a.S.c64, xd, (int)dof, yt);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int sy = sys_of<NC, NR>(u);
          if (!((repm >> sy) & 1)) continue;
          const int64_t i = uidx<NC, NR>(n, dof, u);
          const double tv = b[i] - yt[u];
          r32[i] = (float)tv;
          gr[sy] = fma(tv, tv, gr[sy]);
          gr[NS + sy] = fma(tv, (double)s32[i], gr[NS + sy]);
          gr[2 * NS + sy] = fma(tv, (double)p32[i], gr[2 * NS + sy]);
        }
      }
    }
    double gef[3 * NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      gef[j] = (double)gf[j] + gr[j];
      gef[NS + j] = (double)ef[j] + gr[NS + j];
      gef[2 * NS + j] = (double)ff[j] + gr[2 * NS + j];
    }
    block_sum_wide<3 * NS>(gef, s_tot, s_w);
    double *next = a.part + (size_t)(pass & 1) * kPartHalf;  // the half of the next pass's reduction
    if (threadIdx.x < 3 * NS) {
      const int j = threadIdx.x;  // g -> slot j, e -> 2NS + .., f -> 3NS + ..
      const int slot = j < NS ? j : NS + j;
      next[(size_t)blockIdx.x * NV + slot] = s_tot[j];
    }
    if (!grid_sync(a.bar, G, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int stt = status;
    int upd = 0;
    for (int j = 0; j < NS; ++j) {
      if (stt == CPM_OK && (st[j].unconv || st[j].active)) stt = CPM_NOT_CONVERGED;
      a.info->iters[j] = st[j].iters;
      a.info->resid[j] = st[j].resid;
      upd += st[j].updates;
    }
    a.info->outer = upd;
    set_status(a.info, stt);
  } else if (status != CPM_OK && threadIdx.x == 0) {
    set_status(a.info, status);
  }
}

// ---------------------------------------------------------------- y = alpha A x (FP64)
// Same product on quads of 4 DOFs along z (nz % 4 == 0, 16-byte aligned x and y).
template <int NC, int NR>
__global__ void __launch_bounds__(256) stencil_apply4_kernel(const __grid_constant__ StencilOp S, const double *x,
                                                             double *y, double alpha) {
  const int64_t nq = S.n / 4;
  for (int64_t qd = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; qd < nq; qd += (int64_t)gridDim.x * blockDim.x) {
    double t[4][NC * NR];
    apply4_c<double, NC, NR>(S, S.c64, x, (int)(4 * qd), t);
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
#pragma unroll
      for (int u = 0; u < NC * NR; ++u) t[kk][u] = alpha * t[kk][u];
    quad_store<double, NC, NR>(y, S.n, 4 * qd, t);
  }
}

template <int NC, int NR>
__global__ void __launch_bounds__(256) stencil_apply_kernel(const __grid_constant__ StencilOp S, const double *x, double *y, double alpha) {
  for (int64_t dof = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; dof < S.n;
       dof += (int64_t)gridDim.x * blockDim.x) {
    double t[NC * NR];
    apply<double, NC, NR>(S, x, (int)dof, t);
#pragma unroll
    for (int u = 0; u < NC * NR; ++u) y[uidx<NC, NR>(S.n, dof, u)] = alpha * t[u];
  }
}

// ---------------------------------------------------------------- y = A x (FP32, the refinement form's product)
// FORM 0: per DOF (apply_c); 1: quads with aligned vector loads (nz % 4 == 0);
// 2: quads with scalar loads (any nz).  The same products the FP32 CG phases run.
template <int NC, int NR, int FORM>
__global__ void __launch_bounds__(256) stencil_apply32_kernel(const __grid_constant__ StencilOp S, const float *x,
                                                              float *y) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (FORM == 0) {
    for (int64_t dof = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; dof < S.n; dof += stride) {
      float t[NC * NR];
      apply_c<float, NC, NR>(S, S.c32, x, (int)dof, t);
#pragma unroll
      for (int u = 0; u < NC * NR; ++u) y[uidx<NC, NR>(S.n, dof, u)] = t[u];
    }
  } else {
    const int64_t nq = (S.n + 3) / 4;
    for (int64_t qd = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; qd < nq; qd += stride) {
      float t[4][NC * NR];
      apply4_c<float, NC, NR, FORM == 1>(S, S.c32, x, (int)(4 * qd), t);
      quad_store<float, NC, NR, FORM == 1>(y, S.n, 4 * qd, t);
    }
  }
}

static StencilOp to_op(const cpm_stencil *s) {
  StencilOp S;
  S.nx = s->nx;
  S.ny = s->ny;
  S.nz = s->nz;
  S.n = s->nx * s->ny * s->nz;
  S.flags = s->flags;
  const int nc = 27 * s->ncomp * s->ncomp;
  for (int i = 0; i < 243; ++i) {
    S.c64[i] = i < nc ? s->coef[i] : 0.0;
    S.c32[i] = (float)S.c64[i];
  }
  return S;
}

// The quad form needs whole quads in every z-line and 4-byte aligned flags
// (the solver's own vectors are 256-byte aligned).
static bool quads_ok(const cpm_stencil *s) {
  return (s->nz & 3) == 0 && ((uintptr_t)s->flags & 3) == 0;
}

static int check_stencil(const cpm_stencil *s, const char *who) {
  if (!s || s->nx < 3 || s->ny < 3 || s->nz < 3 || (s->ncomp != 1 && s->ncomp != 3) ||
      (int64_t)s->nx * s->ny * s->nz * s->ncomp >= (int64_t)1 << 31) {
    set_error("%s: bad stencil (at least 3 cells per axis, ncomp 1 or 3, fewer than 2^31 unknowns)", who);
    return CPM_BAD_ARG;
  }
  return CPM_OK;
}

// Error bound of the double-float residual t = b - A x of a scalar stencil, as a multiple of ||b||
// (-1: none).  Each row's double-float sum of 27 terms is within 94 * 2^-48 of the sum of their
// magnitudes (csrc/stencil_ops.cuh, df::fma), and the final FP64 subtractions add less than 2^-50, so
// |t_df - t| <= g |A| |x| elementwise with g = 128 * 2^-48, and ||t_df - t|| <= g sum|c| ||x||.  On the
// free DOFs (every flagged row pinned, checked on the device) A is a principal submatrix of the
// circulant operator, so its eigenvalues are at least the minimum of the symbol
// sigma(theta) = sum_d c_d cos(theta . d), and ||x|| <= (||b|| + ||t||) / sigma_min.  The part of c that
// is even along every axis has a symbol multilinear in (cos theta_x, cos theta_y, cos theta_z), whose
// minimum is at one of the 8 corners cos = +-1; the rest of c moves sigma by at most the sum of its
// magnitudes.  With e = g sum|c| / sigma_min, a residual with ||t_df|| <= tol ||b|| - 2 e ||b|| has
// ||t|| <= (tol ||b|| - e ||b||) / (1 - e) <= tol ||b||: the bound returned is 2 e.
static double df_error_bound(const cpm_stencil *s) {
  if (s->ncomp != 1) return -1.0;
  const double *c = s->coef;
  double even[27], s1 = 0.0, odd = 0.0;
  for (int d = 0; d < 27; ++d) {
    const int ia = d / 9, ib = (d / 3) % 3, ic = d % 3;
    double acc = 0.0;
    for (int m = 0; m < 8; ++m) {
      const int ja = (m & 1) ? 2 - ia : ia, jb = (m & 2) ? 2 - ib : ib, jc = (m & 4) ? 2 - ic : ic;
      acc += c[(ja * 3 + jb) * 3 + jc];
    }
    even[d] = acc / 8.0;
    s1 += std::fabs(c[d]);
    odd += std::fabs(c[d] - even[d]);
  }
  double smin = INFINITY;
  for (int m = 0; m < 8; ++m) {
    const double u[3] = {(m & 1) ? -1.0 : 1.0, (m & 2) ? -1.0 : 1.0, (m & 4) ? -1.0 : 1.0};
    double sig = 0.0;
    for (int d = 0; d < 27; ++d) {
      const int o[3] = {d / 9 - 1, (d / 3) % 3 - 1, d % 3 - 1};
      double w = even[d];
      for (int ax = 0; ax < 3; ++ax) w *= o[ax] ? u[ax] : 1.0;
      sig += w;
    }
    smin = std::min(smin, sig);
  }
  smin -= odd;
  if (!(smin > 0.0) || !(s1 > 0.0)) return -1.0;
  const double g = 128.0 * std::ldexp(1.0, -48);
  return 2.0 * g * s1 / smin;
}

template <int NC, int NR>
static int launch_stencil_cg(const cpm_stencil *s, const double *b, double *x, const cpm_cg_opts *o, Workspace &w,
                             float *xlo, cpm_cg_info *info, cudaStream_t st) {
  StencilCG a{};
  a.S = to_op(s);
  a.b = b;
  a.x = x;
  a.tol = o->tol;
  a.maxiter = o->maxiter;
  a.use_init_host = o->use_init_host;
  a.use_init_dev = o->use_init_dev;
  a.inner_tol = o->inner_tol > 0 ? o->inner_tol : 0.1;
  a.max_outer = o->max_outer > 0 ? o->max_outer : 60;
  a.r = w.r;
  a.p = w.p0;
  a.q = w.q;
  a.r32 = w.r32;
  a.p32 = w.pa32;
  a.q32 = w.q32;
  a.d32 = w.d32;
  a.s32 = w.pb32;
  a.part = w.part;
  a.bar = w.bar;
  a.info = info;
  const double tmo = o->barrier_timeout_s > 0 ? o->barrier_timeout_s : 2.0;
  a.timeout_ns = (unsigned long long)(tmo * 1e9);
  const bool fp64 = o->precision == 0;
  // FP32 form: three grid barriers per iteration unless the caller asks for the two-barrier form
  const bool two = !fp64 && o->form == CPM_CG_FORM_TWO_BARRIER;
  // double-float residual passes: scalar operators in the three-barrier form, with room for the split
  // x (the free pb32 vector and xlo) and an error bound at most a quarter of the tolerance, so that
  // most convergence decisions can be taken on them
  a.df_err = -1.0;
  if (!fp64 && !two && NC == 1 && xlo) {
    const double e = df_error_bound(s);
    if (e > 0.0 && e <= 0.25 * o->tol) {
      a.df_err = e;
      a.xh = w.pb32;
      a.xl = xlo;
      for (int d = 0; d < 27; ++d) {
        const float h = (float)s->coef[d];
        a.cdf[d] = df::DF(h, (float)(s->coef[d] - (double)h));
      }
    }
  }
  const void *fn = fp64 ? (const void *)cg_stencil_fp64_kernel<NC, NR>
                        : two ? (const void *)cg_stencil_ir2_kernel<NC, NR> : (const void *)cg_stencil_ir_kernel<NC, NR>;
  const int threads = fp64 ? kCGThreads : kIRThreads;
  int occ = 0;
  CPM_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, 0));
  if (occ < 1) {
    set_error("stencil cg: kernel cannot be resident on an SM");
    return CPM_CUDA_ERROR;
  }
  const int64_t n = a.S.n;
  // vector quads need whole quads per z-line, aligned flags and an aligned x
  a.quads = quads_ok(s) && ((uintptr_t)x & 15) == 0 ? 1 : 0;
  // The FP32 quad product (4 outputs and 27 independent loads per thread) runs best on few, full
  // CTAs.  The elastic per-DOF product (grids with nz % 4 != 0) needs every resident CTA to hide its
  // gather latency; the scalar ones do not.  Measured on GB300: elastic 81^3 per DOF 80 us per
  // iteration on one CTA per SM, 64.6 us on all of them (80^3 in quads: 45.7 us); demag 81^3 and the
  // 3-RHS A1 81^3 per DOF slower on all CTAs (53 and 178 us).
  int64_t gmax = (int64_t)occ * sm_count();
  if (!fp64 && (a.quads || NC == 1))
    gmax = (int64_t)ir_ctas_per_sm(s->nx * (int64_t)s->ny * s->nz, NC * NR, occ) * sm_count();
  if (gmax > kMaxGrid) gmax = kMaxGrid;
  int64_t G = (n + threads - 1) / threads;
  if (G > gmax) G = gmax;
  if (G < 1) G = 1;
  int64_t per = (n + G - 1) / G;
  per = (per + 31) / 32 * 32;
  G = (n + per - 1) / per;
  a.dofs_per_cta = per;
  if (two && G * 4 * n_systems<NC, NR>() > (int64_t)kPartHalf) {
    set_error("stencil cg: %lld CTAs exceed the partial-sum records of the two-barrier form", (long long)G);
    return CPM_BAD_ARG;
  }
  CPM_TRY(cudaMemsetAsync(w.bar, 0, sizeof(GridBarrier), st));
  CPM_TRY(cudaMemsetAsync(info, 0, sizeof(cpm_cg_info), st));
  void *args[] = {&a};
  CPM_TRY(cudaLaunchCooperativeKernel(fn, dim3((unsigned)G), dim3(threads), args, 0, st));
  return CPM_OK;
}

}  // namespace cpm

extern "C" int cpm_cg_solve_stencil(const cpm_stencil *S, const double *b, double *x, int nrhs,
                                    const cpm_cg_opts *opts, void *workspace, size_t workspace_bytes,
                                    cpm_cg_info *info_dev, void *stream) {
  using namespace cpm;
  if (int e = check_stencil(S, "cpm_cg_solve_stencil")) return e;
  if (!b || !x || !opts || !workspace || !info_dev || (nrhs != 1 && nrhs != 3) || (S->ncomp == 3 && nrhs != 1)) {
    set_error("cpm_cg_solve_stencil: bad arguments (nrhs 1 or 3; the elastic operator takes one block vector)");
    return CPM_BAD_ARG;
  }
  const int prec = opts->precision ? 1 : 0;
  const int64_t n = (int64_t)S->nx * S->ny * S->nz;
  const int64_t unknowns = n * S->ncomp;
  const size_t need = layout(unknowns, nrhs, prec, nullptr, nullptr);
  if (workspace_bytes < need) {
    set_error("cpm_cg_solve_stencil: workspace too small (%zu < %zu bytes)", workspace_bytes, need);
    return CPM_BAD_ARG;
  }
  Workspace w;
  layout(unknowns, nrhs, prec, (char *)workspace, &w);
  // the low half of the split x, where the caller sized the workspace for it
  float *xlo = nullptr;
  if (prec && workspace_bytes >= cpm_cg_stencil_workspace_bytes(unknowns, nrhs, prec))
    xlo = (float *)((char *)workspace + need);
  cudaStream_t st = (cudaStream_t)stream;
  if (S->ncomp == 3) return launch_stencil_cg<3, 1>(S, b, x, opts, w, xlo, info_dev, st);
  return nrhs == 1 ? launch_stencil_cg<1, 1>(S, b, x, opts, w, xlo, info_dev, st)
                   : launch_stencil_cg<1, 3>(S, b, x, opts, w, xlo, info_dev, st);
}

extern "C" double cpm_stencil_df_error_bound(const cpm_stencil *S) {
  if (!S) return -1.0;
  return cpm::df_error_bound(S);
}

extern "C" size_t cpm_cg_stencil_workspace_bytes(int64_t unknowns, int nrhs, int precision) {
  using namespace cpm;
  const size_t base = layout(unknowns, nrhs, precision ? 1 : 0, nullptr, nullptr);
  return precision ? base + align256(sizeof(float) * (size_t)unknowns * nrhs) : base;
}

extern "C" int cpm_stencil_apply(const cpm_stencil *S, const double *x, double *y, double alpha, int nvec,
                                 void *stream) {
  using namespace cpm;
  if (int e = check_stencil(S, "cpm_stencil_apply")) return e;
  if (!x || !y || (nvec != 1 && nvec != 3) || (S->ncomp == 3 && nvec != 1)) {
    set_error("cpm_stencil_apply: bad vectors");
    return CPM_BAD_ARG;
  }
  const StencilOp op = to_op(S);
  int64_t g = (op.n + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (g > cap) g = cap;
  cudaStream_t st = (cudaStream_t)stream;
  if (quads_ok(S) && (((uintptr_t)x | (uintptr_t)y) & 15) == 0) {
    const int64_t gq = std::max<int64_t>(1, std::min<int64_t>(g, (op.n / 4 + 255) / 256));
    if (S->ncomp == 3)
      stencil_apply4_kernel<3, 1><<<(int)gq, 256, 0, st>>>(op, x, y, alpha);
    else if (nvec == 1)
      stencil_apply4_kernel<1, 1><<<(int)gq, 256, 0, st>>>(op, x, y, alpha);
    else
      stencil_apply4_kernel<1, 3><<<(int)gq, 256, 0, st>>>(op, x, y, alpha);
    return check_launch("cpm_stencil_apply");
  }
  if (S->ncomp == 3)
    stencil_apply_kernel<3, 1><<<(int)g, 256, 0, st>>>(op, x, y, alpha);
  else if (nvec == 1)
    stencil_apply_kernel<1, 1><<<(int)g, 256, 0, st>>>(op, x, y, alpha);
  else
    stencil_apply_kernel<1, 3><<<(int)g, 256, 0, st>>>(op, x, y, alpha);
  return check_launch("cpm_stencil_apply");
}

extern "C" int cpm_stencil_apply32(const cpm_stencil *S, const float *x, float *y, int nvec, int form, void *stream) {
  using namespace cpm;
  if (int e = check_stencil(S, "cpm_stencil_apply32")) return e;
  if (!x || !y || (nvec != 1 && nvec != 3) || (S->ncomp == 3 && nvec != 1) || form < 0 || form > 2) {
    set_error("cpm_stencil_apply32: bad vectors or form (0 per DOF, 1 aligned quads, 2 scalar-load quads)");
    return CPM_BAD_ARG;
  }
  if ((form == 1 && !(quads_ok(S) && (((uintptr_t)x | (uintptr_t)y) & 15) == 0)) ||
      (form == 2 && ((uintptr_t)S->flags & 3) != 0)) {
    set_error("cpm_stencil_apply32: form %d needs %s", form,
              form == 1 ? "nz % 4 == 0, 4-byte aligned flags and 16-byte aligned x and y" : "4-byte aligned flags");
    return CPM_BAD_ARG;
  }
  const StencilOp op = to_op(S);
  const int64_t units = form == 0 ? op.n : (op.n + 3) / 4;
  const int64_t g = std::max<int64_t>(1, std::min<int64_t>((units + 255) / 256, (int64_t)sm_count() * 8));
  cudaStream_t st = (cudaStream_t)stream;
#define CPM_APPLY32(F)                                                                    \
  do {                                                                                    \
    if (S->ncomp == 3)                                                                    \
      stencil_apply32_kernel<3, 1, F><<<(int)g, 256, 0, st>>>(op, x, y);                  \
    else if (nvec == 1)                                                                   \
      stencil_apply32_kernel<1, 1, F><<<(int)g, 256, 0, st>>>(op, x, y);                  \
    else                                                                                  \
      stencil_apply32_kernel<1, 3, F><<<(int)g, 256, 0, st>>>(op, x, y);                  \
  } while (0)
  if (form == 0) CPM_APPLY32(0);
  else if (form == 1) CPM_APPLY32(1);
  else CPM_APPLY32(2);
#undef CPM_APPLY32
  return check_launch("cpm_stencil_apply32");
}
