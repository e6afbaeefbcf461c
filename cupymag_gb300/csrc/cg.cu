// Persistent fused conjugate gradient for the GSPM LLG step (sm_103a).
//
// Replaces cupymag/solvers/linear_solvers.py:20-74, i.e. cupyx's cg, whose
// algorithm is restated here:
//   x = x0 if use_init else 0;  if ||b|| == 0 return b;  atol = tol ||b||;
//   r = b - A x;  repeat: rho = r.r; p = r (first) or r + (rho/rho_old) p;
//   q = A p; alpha = rho / (p.q); x += alpha p; r -= alpha q; iters++;
//   stop when ||r|| <= atol (after the update) or iters == maxiter.
//
// One cooperative launch runs every iteration.  Each CTA owns a contiguous
// block of rows; one iteration is two phases separated by a grid barrier:
//   phase 1 (warp per row): p_new = r + beta p_old is formed on the fly while
//     gathering, q = A p_new, and the CTA's partial of p.q;
//   phase 2 (thread per row): x += alpha p, r -= alpha q, partial of r.r.
// p is double-buffered so rows can gather neighbours' p_old while the owner
// writes p_new.  Dot products are reduced in a fixed order (warp shuffle
// tree, warps in order, CTAs in order) so results are deterministic, and every
// CTA reduces the per-CTA partials itself, so all CTAs agree on alpha, beta
// and on the stopping test without a third barrier.
//
// nrhs = 3 solves three systems with the same matrix (the g1n/g2n/g3n and
// m1ss/m2ss/m3ss triples of Micromagnetics.py:221-223,280-290) in one sweep of
// the matrix; each right-hand side keeps its own scalars, iteration count and
// stopping test, so each result equals the single-system solve.
//
// precision = 1: FP32 CG (FP32 values and vectors, FP64 dot accumulation)
// with FP64 reliable updates of x and of the residual b - A64 x.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "cg_common.cuh"
#include "csr_tile.cuh"

namespace cpm {

template <int NR, typename IT>
struct CGArgs {
  int64_t n;
  const IT *rp;
  const int *ci;
  const double *av;
  const float *av32;
  const double *b;
  double *x;
  double tol;
  int maxiter;
  int use_init_host;
  const int *use_init_dev;
  double inner_tol;
  int max_outer;
  // workspace
  double *r, *p0, *p1, *q;                 // FP64 vectors (n*NR each)
  float *r32, *pa32, *pb32, *q32, *d32;    // FP32 vectors (mixed precision)
  double *part;                            // [G][2*NR]
  GridBarrier *bar;
  cpm_cg_info *info;
  unsigned long long timeout_ns;
  int64_t rows_per_cta;
  int group;                               // threads per row in the staged SpMV
};

// Lanes per row of the FP32 product of the refinement form (group_row in csr_tile.cuh).
constexpr int kCsrGroup = 4;

template <typename IT>
__device__ __forceinline__ void row_range(const IT *rp, int64_t row, int64_t &s, int64_t &e) {
  s = (int64_t)__ldg(rp + row);
  e = (int64_t)__ldg(rp + row + 1);
}

// ------------------------------------------------------------------ FP64 CG
// Three phases per iteration, each ended by a grid barrier:
//   1. q = A p over staged tiles (one FP64 FMA per non-zero), partial p.q;
//   2. x += alpha p, r -= alpha q, partial r.r;
//   3. p = r + beta p for the CTA's own rows.
// Forming p in its own pass (instead of r + beta p_old inside the gather)
// keeps the FP64 work of the SpMV at one FMA per non-zero, which is what the
// FP64 pipes of GB300 can sustain at HBM speed.
template <int NR, typename IT>
__global__ void __launch_bounds__(kCGThreads) cg_fp64_kernel(CGArgs<NR, IT> a) {
  __shared__ double s_red[2 * NR][kCGWarps];
  extern __shared__ __align__(16) unsigned char s_tile[];
  const TileSmem tile = tile_smem(s_tile);
  const int G = a.group;
  const int R = kCGThreads / G;
  const bool lead = (threadIdx.x % G) == 0;
  const int64_t r0 = min(a.n, (int64_t)blockIdx.x * a.rows_per_cta);
  const int64_t r1 = min(a.n, r0 + a.rows_per_cta);
  const bool use_init = a.use_init_dev ? (__ldcg(a.use_init_dev) != 0) : (a.use_init_host != 0);
  const unsigned long long tns = a.timeout_ns;
  int par = 0;
  double *p = a.p0;

  // ---- prologue: r = b - A x (or r = b, x = 0), p = r, ||b||^2, ||r||^2
  double v[2 * NR];
#pragma unroll
  for (int j = 0; j < 2 * NR; ++j) v[j] = 0.0;
  if (use_init) {
    for (int64_t t0 = r0; t0 < r1; t0 += R) {
      double acc[NR];
      const int64_t row = tile_rows<NR, IT>(a.rp, a.ci, a.av, a.x, t0, min(r1, t0 + R), G, tile, acc);
      if (row >= 0 && lead) {
#pragma unroll
        for (int j = 0; j < NR; ++j) {
          const double bj = a.b[row * NR + j];
          const double rj = bj - acc[j];
          a.r[row * NR + j] = rj;
          p[row * NR + j] = rj;
          v[j] = fma(bj, bj, v[j]);
          v[NR + j] = fma(rj, rj, v[NR + j]);
        }
      }
    }
  } else {
    for (int64_t row = r0 + threadIdx.x; row < r1; row += kCGThreads) {
#pragma unroll
      for (int j = 0; j < NR; ++j) {
        const double bj = a.b[row * NR + j];
        a.r[row * NR + j] = bj;
        p[row * NR + j] = bj;
        a.x[row * NR + j] = 0.0;
        v[j] = fma(bj, bj, v[j]);
        v[NR + j] = fma(bj, bj, v[NR + j]);
      }
    }
  }
  if (!grid_sum<2 * NR>(v, a.part, par, a.bar, tns, s_red)) {
    set_status(a.info, CPM_BARRIER_TIMEOUT);
    return;
  }
  double atol[NR], rho[NR], resid[NR];
  int active[NR], iters[NR];
  bool any = false;
#pragma unroll
  for (int j = 0; j < NR; ++j) {
    const double bn = sqrt(v[j]);
    atol[j] = a.tol * bn;
    rho[j] = v[NR + j];
    resid[j] = sqrt(v[NR + j]);
    active[j] = bn != 0.0;
    iters[j] = 0;
    any |= active[j] != 0;
    if (bn == 0.0 && use_init) {
      // cupyx returns b itself when ||b|| == 0
      for (int64_t row = r0 + threadIdx.x; row < r1; row += kCGThreads) a.x[row * NR + j] = a.b[row * NR + j];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.info->bnorm[j] = bn;
  }

  int status = CPM_OK;
  for (int k = 0; any && k < a.maxiter; ++k) {
    // ---- phase 1: q = A p, partial p.q
    double pq[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) pq[j] = 0.0;
    for (int64_t t0 = r0; t0 < r1; t0 += R) {
      double acc[NR];
      const int64_t row = tile_rows<NR, IT>(a.rp, a.ci, a.av, p, t0, min(r1, t0 + R), G, tile, acc);
      if (row >= 0 && lead) {
#pragma unroll
        for (int j = 0; j < NR; ++j) {
          a.q[row * NR + j] = acc[j];
          pq[j] = fma(p[row * NR + j], acc[j], pq[j]);
        }
      }
    }
    if (!grid_sum<NR>(pq, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
    double alpha[NR];
    bool bad = false;
#pragma unroll
    for (int j = 0; j < NR; ++j) {
      alpha[j] = active[j] ? rho[j] / pq[j] : 0.0;
      if (active[j] && !isfinite(alpha[j])) bad = true;
    }
    if (bad) { status = CPM_NONFINITE; break; }

    // ---- phase 2: x += alpha p, r -= alpha q, partial r.r
    double rr[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) rr[j] = 0.0;
    for (int64_t row = r0 + threadIdx.x; row < r1; row += kCGThreads) {
#pragma unroll
      for (int j = 0; j < NR; ++j) {
        if (!active[j]) continue;
        const int64_t i = row * NR + j;
        a.x[i] = __fma_rn(alpha[j], p[i], a.x[i]);
        const double rn = __fma_rn(-alpha[j], a.q[i], a.r[i]);
        a.r[i] = rn;
        rr[j] = fma(rn, rn, rr[j]);
      }
    }
    if (!grid_sum<NR>(rr, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
    any = false;
    double beta[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) {
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

    // ---- phase 3: p = r + beta p (own rows)
    for (int64_t row = r0 + threadIdx.x; row < r1; row += kCGThreads) {
#pragma unroll
      for (int j = 0; j < NR; ++j) {
        if (!active[j]) continue;
        const int64_t i = row * NR + j;
        p[i] = __fma_rn(beta[j], p[i], a.r[i]);
      }
    }
    if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int st = status;
#pragma unroll
    for (int j = 0; j < NR; ++j) {
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

// ---------------------------------------------------------------------------
// FP32 CG with FP64 reliable updates on CSR matrices: the algorithm of the
// stencil solver (csrc/stencil.cu): FP32 values (A->vals32) and FP32 vectors
// (p, q, the correction d, the recursive residual r) with FP32 per-thread dot
// partials summed in FP64 across threads; when the recursive residual has
// fallen by inner_tol (or below the threshold, or at maxiter) the next
// iteration's first phase also computes the true residual t = b - A64 x with
// the FP64 values (staged tiles; the direction phase before it folded d into
// x), t replaces r and rho and decides convergence, and that iteration's step
// is the exact line search (t.p) / (p.A p).  Three grid barriers per iteration.
// Every product reads its rows in place by 4-lane groups (group_row): no
// shared-memory tiles, so more CTAs per SM hide the gathers.  Measured on GB300
// (FP32 product, 3 RHS scalar / elastic / tet rows): tet96 elasticity 373 -> 289
// us per iteration, demag 66 -> 53, hex 64^3 elasticity 179 -> 129, against the
// staged tiles, which the FP64 solver keeps (faster there: tet96 elasticity 520
// against 668 us in place).  The CG state lives in shared memory (IRState).
template <int NR, typename IT>
__global__ void __launch_bounds__(kCGThreads) cg_ir_kernel(CGArgs<NR, IT> a) {
  __shared__ double s_red[9][kCGWarps];
  __shared__ IRState st[NR];
  __shared__ float s_ab[NR];
  __shared__ int s_mask[3];  // active, need, status
  const bool lead = (threadIdx.x % kCsrGroup) == 0;
  const int64_t r0 = min(a.n, (int64_t)blockIdx.x * a.rows_per_cta);
  const int64_t r1 = min(a.n, r0 + a.rows_per_cta);
  const bool use_init = a.use_init_dev ? (__ldcg(a.use_init_dev) != 0) : (a.use_init_host != 0);
  const unsigned long long tns = a.timeout_ns;
  double *x = a.x;
  float *r32 = a.r32, *p32 = a.pa32, *q32 = a.q32, *d32 = a.d32;
  int par = 0;

  // ---- prologue: r = b - A64 x (or b), r32 = p32 = r, d = 0
  double v[2 * NR];
#pragma unroll
  for (int j = 0; j < 2 * NR; ++j) v[j] = 0.0;
  if (use_init) {
    for (int64_t t0 = r0; t0 < r1; t0 += kCGThreads / kCsrGroup) {
      double acc[NR];
      const int64_t row = t0 + threadIdx.x / kCsrGroup;
      group_row<NR, kCsrGroup, IT>(a.rp, a.ci, a.av, x, row, r1, acc);
      if (row < r1 && lead) {
#pragma unroll
        for (int j = 0; j < NR; ++j) {
          const double bj = a.b[row * NR + j];
          const double rj = bj - acc[j];
          const float rf = (float)rj;
          r32[row * NR + j] = rf;
          p32[row * NR + j] = rf;
          d32[row * NR + j] = 0.0f;
          v[j] = fma(bj, bj, v[j]);
          v[NR + j] = fma(rj, rj, v[NR + j]);
        }
      }
    }
  } else {
    for (int64_t row = r0 + threadIdx.x; row < r1; row += kCGThreads) {
#pragma unroll
      for (int j = 0; j < NR; ++j) {
        const double bj = a.b[row * NR + j];
        const float rf = (float)bj;
        x[row * NR + j] = 0.0;
        r32[row * NR + j] = rf;
        p32[row * NR + j] = rf;
        d32[row * NR + j] = 0.0f;
        v[j] = fma(bj, bj, v[j]);
        v[NR + j] = fma(bj, bj, v[NR + j]);
      }
    }
  }
  if (!grid_sum<2 * NR>(v, a.part, par, a.bar, tns, s_red)) {
    set_status(a.info, CPM_BARRIER_TIMEOUT);
    return;
  }
  if (threadIdx.x == 0) {
    int am = 0;
    for (int j = 0; j < NR; ++j) {
      ir_init(st[j], sqrt(v[j]), v[NR + j], a.tol);
      am |= st[j].active << j;
      if (blockIdx.x == 0) a.info->bnorm[j] = sqrt(v[j]);
    }
    s_mask[0] = am;
    s_mask[1] = 0;
    s_mask[2] = CPM_OK;
  }
  __syncthreads();
  int activem = s_mask[0], needm = 0;
  if (use_init) {
    for (int j = 0; j < NR; ++j)
      if (!((activem >> j) & 1))
        for (int64_t row = r0 + threadIdx.x; row < r1; row += kCGThreads) x[row * NR + j] = a.b[row * NR + j];
  }
  int status = CPM_OK;
  for (int k = 0; activem && k <= a.maxiter; ++k) {
    if (k > 0 && !grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
    // ---- phase 1: q = A32 p, p.q; pending: t = b - A64 x, r32 = t, t.t, t.p
    float pqf[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) pqf[j] = 0.0f;
    for (int64_t t0 = r0; t0 < r1; t0 += kCGThreads / kCsrGroup) {
      float acc[NR];
      const int64_t row = t0 + threadIdx.x / kCsrGroup;
      group_row<NR, kCsrGroup, IT, float>(a.rp, a.ci, a.av32, p32, row, r1, acc);
      if (row < r1 && lead) {
#pragma unroll
        for (int j = 0; j < NR; ++j) {
          q32[row * NR + j] = acc[j];
          pqf[j] = fmaf(p32[row * NR + j], acc[j], pqf[j]);
        }
      }
    }
    double pt[3 * NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) {
      pt[j] = (double)pqf[j];
      pt[NR + j] = 0.0;
      pt[2 * NR + j] = 0.0;
    }
    if (needm) {
      // d was folded into x by the previous direction phase
      for (int64_t t0 = r0; t0 < r1; t0 += kCGThreads / kCsrGroup) {
        double acc[NR];
        const int64_t row = t0 + threadIdx.x / kCsrGroup;
        group_row<NR, kCsrGroup, IT>(a.rp, a.ci, a.av, x, row, r1, acc);
        if (row < r1 && lead) {
#pragma unroll
          for (int j = 0; j < NR; ++j) {
            if (!((needm >> j) & 1)) continue;
            const double t = a.b[row * NR + j] - acc[j];
            r32[row * NR + j] = (float)t;
            pt[NR + j] = fma(t, t, pt[NR + j]);
            pt[2 * NR + j] = fma(t, (double)p32[row * NR + j], pt[2 * NR + j]);
          }
        }
      }
    }
    // t.t and t.p only on an iteration with a pending update (FP64 adds are slow on GB300)
    if (!grid_sum<3 * NR>(pt, a.part, par, a.bar, tns, s_red, needm ? 3 * NR : NR)) {
      status = CPM_BARRIER_TIMEOUT;
      break;
    }
    if (threadIdx.x == 0) {
      int am = 0, bad = 0;
      for (int j = 0; j < NR; ++j) {
        double al;
        bad |= ir_after_pq(st[j], pt[j], pt[NR + j], pt[2 * NR + j], a.maxiter, al);
        s_ab[j] = (float)al;
        am |= st[j].active << j;
      }
      if (needm) st[0].updates += 1;
      s_mask[0] = am;
      s_mask[2] = bad ? CPM_NONFINITE : CPM_OK;
    }
    __syncthreads();
    if (s_mask[2] != CPM_OK) { status = s_mask[2]; break; }
    float af[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) af[j] = s_ab[j];
    activem = s_mask[0];
    // ---- phase 2: active: d += alpha p, r32 -= alpha q, r32.r32
    float rrf[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) rrf[j] = 0.0f;
    for (int64_t row = r0 + threadIdx.x; row < r1; row += kCGThreads) {
#pragma unroll
      for (int j = 0; j < NR; ++j) {
        if (!((activem >> j) & 1)) continue;
        const int64_t i = row * NR + j;
        d32[i] = fmaf(af[j], p32[i], d32[i]);
        const float rn = fmaf(-af[j], q32[i], r32[i]);
        r32[i] = rn;
        rrf[j] = fmaf(rn, rn, rrf[j]);
      }
    }
    double rr[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) rr[j] = (double)rrf[j];
    if (!grid_sum<NR>(rr, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
    if (threadIdx.x == 0) {
      int nm = 0, bad = 0;
      for (int j = 0; j < NR; ++j) {
        float be;
        bad |= ir_after_rr(st[j], rr[j], a.inner_tol, a.maxiter, be);
        s_ab[j] = be;
        nm |= st[j].need << j;
      }
      s_mask[1] = nm;
      s_mask[2] = bad ? CPM_NONFINITE : CPM_OK;
    }
    __syncthreads();
    if (s_mask[2] != CPM_OK) { status = s_mask[2]; break; }
    needm = s_mask[1];
    if (!activem) break;
    float beta[NR];
#pragma unroll
    for (int j = 0; j < NR; ++j) beta[j] = s_ab[j];
    // ---- phase 3: p = r32 + beta p; pending updates: x += d, d = 0
    for (int64_t row = r0 + threadIdx.x; row < r1; row += kCGThreads)
#pragma unroll
      for (int j = 0; j < NR; ++j) {
        const int64_t i = row * NR + j;
        if ((activem >> j) & 1) p32[i] = fmaf(beta[j], p32[i], r32[i]);
        if ((needm >> j) & 1) {
          x[i] += (double)d32[i];
          d32[i] = 0.0f;
        }
      }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int stt = status;
    for (int j = 0; j < NR; ++j) {
      if (stt == CPM_OK && (st[j].unconv || st[j].active)) stt = CPM_NOT_CONVERGED;
      a.info->iters[j] = st[j].iters;
      a.info->resid[j] = st[j].resid;
    }
    a.info->outer = st[0].updates;
    set_status(a.info, stt);
  } else if (status != CPM_OK && threadIdx.x == 0) {
    set_status(a.info, status);
  }
}

constexpr int kOccDevices = 64;
static std::mutex g_occ_mu;
static int g_occ[kOccDevices][2][2][2] = {};

template <int NR, typename IT>
static int launch_cg(const cpm_csr *A, const double *b, double *x, const cpm_cg_opts *o, Workspace &w,
                     cpm_cg_info *info, cudaStream_t st) {
  CGArgs<NR, IT> a{};
  a.n = A->rows;
  a.rp = (const IT *)A->indptr;
  a.ci = A->indices;
  a.av = A->vals;
  a.av32 = A->vals32;
  a.b = b;
  a.x = x;
  a.tol = o->tol;
  a.maxiter = o->maxiter;
  a.use_init_host = o->use_init_host;
  a.use_init_dev = o->use_init_dev;
  a.inner_tol = o->inner_tol > 0 ? o->inner_tol : 0.1;
  a.max_outer = o->max_outer > 0 ? o->max_outer : 50;
  a.r = w.r;
  a.p0 = w.p0;
  a.p1 = w.p1;
  a.q = w.q;
  a.r32 = w.r32;
  a.pa32 = w.pa32;
  a.pb32 = w.pb32;
  a.q32 = w.q32;
  a.d32 = w.d32;
  a.part = w.part;
  a.bar = w.bar;
  a.info = info;
  const double tmo = o->barrier_timeout_s > 0 ? o->barrier_timeout_s : 2.0;
  a.timeout_ns = (unsigned long long)(tmo * 1e9);

  const bool fp64 = o->precision == 0;
  const void *fn = fp64 ? (const void *)cg_fp64_kernel<NR, IT> : (const void *)cg_ir_kernel<NR, IT>;
  const int smem = fp64 ? kTileSmemBytes : 0;  // staged tiles (FP64 solver) or none (refinement form)
  // occupancy (and the shared-memory attribute, a per-device setting) resolved once per device and
  // kernel variant, under a lock: host threads may launch on different devices at once
  const int dev = device_id();
  if (dev < 0 || dev >= kOccDevices) {
    set_error("cg: device ordinal %d out of range", dev);
    return CPM_BAD_ARG;
  }
  const int pi = o->precision ? 1 : 0, ri = NR == 3, ii = sizeof(IT) == 8;
  int occ = 0;
  {
    std::lock_guard<std::mutex> lock(g_occ_mu);
    int &cached = g_occ[dev][pi][ri][ii];  // occupancy + 1, 0 = not resolved
    if (cached == 0) {
      if (smem) CPM_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
      int blocks = 0;
      CPM_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, kCGThreads, smem));
      cached = blocks + 1;
    }
    occ = cached - 1;
  }
  if (occ < 1) {
    set_error("cg: kernel cannot be resident on an SM");
    return CPM_CUDA_ERROR;
  }
  int64_t maxrow = A->max_row_nnz > 0 ? A->max_row_nnz : (A->nnz + A->rows - 1) / (A->rows > 0 ? A->rows : 1);
  a.group = group_size(maxrow, kCGThreads);
  int64_t gmax = (int64_t)occ * sm_count();
  if (gmax > kMaxGrid) gmax = kMaxGrid;
  // at least ~64 rows per CTA so small systems do not pay for idle CTAs at barriers
  int64_t G = (a.n + 63) / 64;
  if (G > gmax) G = gmax;
  if (G < 1) G = 1;
  int64_t rpc = (a.n + G - 1) / G;
  rpc = (rpc + 31) / 32 * 32;
  G = (a.n + rpc - 1) / rpc;
  if (G < 1) G = 1;
  a.rows_per_cta = rpc;

  CPM_TRY(cudaMemsetAsync(w.bar, 0, sizeof(GridBarrier), st));
  CPM_TRY(cudaMemsetAsync(info, 0, sizeof(cpm_cg_info), st));
  void *args[] = {&a};
  CPM_TRY(cudaLaunchCooperativeKernel(fn, dim3((unsigned)G), dim3(kCGThreads), args, smem, st));
  return CPM_OK;
}

}  // namespace cpm

extern "C" size_t cpm_cg_workspace_bytes(int64_t n, int nrhs, int precision) {
  return cpm::layout(n, nrhs, precision ? 1 : 0, nullptr, nullptr);
}

namespace cpm {

static int solve_impl(const cpm_csr *A, const double *b, double *x, int nrhs, const cpm_cg_opts *opts,
                      void *workspace, size_t workspace_bytes, cpm_cg_info *info_dev, void *stream, const char *who) {
  if (!A || !b || !x || !opts || !workspace || !info_dev) {
    set_error("%s: null argument", who);
    return CPM_BAD_ARG;
  }
  if (nrhs != 1 && nrhs != 3) {
    set_error("%s: nrhs must be 1 or 3 (got %d)", who, nrhs);
    return CPM_BAD_ARG;
  }
  if (A->rows != A->cols) {
    set_error("%s: matrix must be square (%lld x %lld)", who, (long long)A->rows, (long long)A->cols);
    return CPM_BAD_ARG;
  }
  const int prec = opts->precision ? 1 : 0;
  if (prec == 1 && !A->vals32) {
    set_error("%s: mixed precision needs the FP32 copy of the values (vals32)", who);
    return CPM_BAD_ARG;
  }
  if (opts->maxiter < 0) {
    set_error("%s: maxiter must be >= 0", who);
    return CPM_BAD_ARG;
  }
  const size_t need = layout(A->rows, nrhs, prec, nullptr, nullptr);
  if (workspace_bytes < need) {
    set_error("%s: workspace too small (%zu < %zu bytes)", who, workspace_bytes, need);
    return CPM_BAD_ARG;
  }
  if (A->rows == 0) return CPM_OK;
  Workspace w;
  layout(A->rows, nrhs, prec, (char *)workspace, &w);
  cudaStream_t st = (cudaStream_t)stream;
  if (A->indptr_is64) {
    return nrhs == 1 ? launch_cg<1, int64_t>(A, b, x, opts, w, info_dev, st)
                     : launch_cg<3, int64_t>(A, b, x, opts, w, info_dev, st);
  }
  return nrhs == 1 ? launch_cg<1, int32_t>(A, b, x, opts, w, info_dev, st)
                   : launch_cg<3, int32_t>(A, b, x, opts, w, info_dev, st);
}

// ---------------------------------------------------------------- no-allocation variant
// Scratch of cpm_cg_solve_noalloc: a fixed array in device memory that exists
// in every context that loads this library, for the life of the process.
// 32 MiB holds the FP64 solver's four vectors for n * nrhs up to about 1.03
// million (FP32-refinement form: five float vectors, about 1.65 million).
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_cg_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  The first call
// on a device resolves it with cudaGetSymbolAddress (with that device current)
// and caches it; later calls only read the cache.
static int noalloc_scratch(void **out) {
  int dev = 0;
  CPM_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("cpm_cg_solve_noalloc: device ordinal %d out of range", dev);
    return CPM_BAD_ARG;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (g_noalloc_ptr[dev] == nullptr) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_cg_noalloc_scratch);
    if (e != cudaSuccess || ptr == nullptr) {
      set_error("cpm_cg_solve_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return CPM_CUDA_ERROR;
    }
    g_noalloc_ptr[dev] = ptr;
  }
  *out = g_noalloc_ptr[dev];
  return CPM_OK;
}

}  // namespace cpm

extern "C" int cpm_cg_solve(const cpm_csr *A, const double *b, double *x, int nrhs, const cpm_cg_opts *opts,
                            void *workspace, size_t workspace_bytes, cpm_cg_info *info_dev, void *stream) {
  return cpm::solve_impl(A, b, x, nrhs, opts, workspace, workspace_bytes, info_dev, stream, "cpm_cg_solve");
}

extern "C" int cpm_cg_solve_noalloc(const cpm_csr *A, const double *b, double *x, int nrhs, const cpm_cg_opts *opts,
                                    cpm_cg_info *info_dev, void *stream) {
  using namespace cpm;
  if (!A || !opts) {
    set_error("cpm_cg_solve_noalloc: null argument");
    return CPM_BAD_ARG;
  }
  const size_t need = layout(A->rows, nrhs == 3 ? 3 : 1, opts->precision ? 1 : 0, nullptr, nullptr);
  if (need > kNoAllocScratchBytes) {
    set_error("cpm_cg_solve_noalloc: this solve needs %zu bytes of scratch but the built-in array holds %zu "
              "(n * nrhs up to about 1.03 million in FP64); use cpm_cg_solve with a workspace instead",
              need, kNoAllocScratchBytes);
    return CPM_BAD_ARG;
  }
  void *ws = nullptr;
  if (int s = noalloc_scratch(&ws)) return s;
  return solve_impl(A, b, x, nrhs, opts, ws, kNoAllocScratchBytes, info_dev, stream, "cpm_cg_solve_noalloc");
}
