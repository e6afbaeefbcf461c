// Pieces shared by the CSR and stencil conjugate-gradient kernels.
#pragma once

#include "cpm_common.cuh"

namespace cpm {

constexpr int kCGThreads = 256;
constexpr int kCGWarps = kCGThreads / kWarp;
constexpr int kMaxGrid = 4096;                 // CTAs of one cooperative launch (upper bound)
constexpr size_t kPartHalf = (size_t)9 * kMaxGrid;  // doubles per half of the partials buffer (<= 9 sums per CTA)

// Block-wide sum of the first nv of NV values per thread, deterministic;
// result broadcast (values nv.. are left as they are; s[j][0] holds total j).
// A GB300 SM issues FP64 adds at about 1/64 of its FP32 rate (one warp
// instruction holds the FP64 pipe for ~64 cycles), so the reductions count
// FP64 instructions: they skip values not in use, and one warp adds a
// block's values (13 FP64 warp instructions per value, where shuffles in
// every warp and a per-thread sum of the warp sums took 48).
// The staging array of block_sum: one per block size, shared by every instantiation.
template <int NT>
__device__ __forceinline__ double *block_sum_scratch() {
  __shared__ double s_all[NT];
  return s_all;
}

// NT: the block's thread count.
template <int NV, int NW, int NT = kCGThreads>
__device__ __forceinline__ void block_sum(double (&v)[NV], double (*s)[NW], int nv = NV) {
  // per value: every thread stores its value, one warp adds NT/32 per lane (threads l, l + 32,
  // l + 64, ..., in order: consecutive lanes read consecutive words, no bank conflicts) and then the
  // 32 lane sums with a fixed shuffle tree
  double *s_all = block_sum_scratch<NT>();
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    if (j >= nv) break;
    s_all[threadIdx.x] = v[j];
    __syncthreads();
    if (threadIdx.x < kWarp) {
      double t = 0.0;
#pragma unroll
      for (int k = 0; k < NT / kWarp; ++k) t += s_all[k * kWarp + lane];
      t = warp_sum(t);
      if (lane == 0) s[j][0] = t;
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    if (j >= nv) break;
    v[j] = s[j][0];
  }
  __syncthreads();
}

// Write this CTA's partials of the first nv of NV values, barrier, and reduce
// all CTAs' partials.  The partials buffer alternates between two halves: a
// CTA may start writing the next reduction's partials while slower CTAs still
// read this one's, and the barrier of the next reduction orders the reuse of
// a half.
template <int NV, int NW, int NT = kCGThreads>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double *part, int &parity, GridBarrier *bar,
                                         unsigned long long tns, double (*s)[NW], int nv = NV) {
  block_sum<NV, NW, NT>(v, s, nv);
  const int G = gridDim.x;
  part += (size_t)parity * kPartHalf;
  parity ^= 1;
#pragma unroll
  for (int j = 0; j < NV; ++j)
    if (threadIdx.x == j && j < nv) part[(size_t)blockIdx.x * NV + j] = v[j];
  if (!grid_sync(bar, G, tns)) return false;
  double acc[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) acc[j] = 0.0;
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
#pragma unroll
    for (int j = 0; j < NV; ++j)
      if (j < nv) acc[j] += __ldcg(&part[(size_t)g * NV + j]);
  }
  block_sum<NV, NW, NT>(acc, s, nv);
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j] = j < nv ? acc[j] : 0.0;
  return true;
}

// ---------------------------------------------------------------- reliable-update CG state
// State of one system of the FP32 CG with lagged FP64 reliable updates
// (csrc/cg.cu, csrc/stencil.cu, csrc/batched.cu).  The transitions below are the whole
// scalar logic of that solver; the kernels call them once per reduction.
// dfe > 0: the pending update may be a double-float residual whose error is at most dfe (csrc/stencil.cu);
// dfok marks an update scheduled that way, exact forces FP64 updates from then on, dfupd counts the
// double-float updates.
struct IRState {
  double atol, resid, rho, r0, dfe;
  int active, need, iters, unconv, updates, dfok, exact, dfupd;
};

__device__ __forceinline__ void ir_init(IRState &s, double bnorm, double rr0, double tol) {
  s.atol = tol * bnorm;
  s.rho = rr0;
  s.resid = sqrt(rr0);
  s.r0 = s.resid;
  s.dfe = 0.0;
  s.active = bnorm != 0.0;
  s.need = 0;
  s.iters = 0;
  s.unconv = 0;
  s.updates = 0;
  s.dfok = 0;
  s.exact = 0;
  s.dfupd = 0;
}

// After the p.q reduction (pq) with, for a pending update, the true residual
// norm tt = t.t and tp = t.p: decide convergence on t and return alpha
// (exact line search along p when t replaced the residual).  Returns true on
// a non-finite value.
// With dfpass the residual was double-float: it decides convergence only outside its error bound
// (resid <= atol - dfe); within dfe of atol every later update is FP64.
__device__ __forceinline__ bool ir_after_pq(IRState &s, double pq, double tt, double tp, int maxiter, double &alpha,
                                            bool dfpass = false) {
  bool bad = false;
  alpha = 0.0;
  if (s.need) {
    s.resid = sqrt(tt);
    s.r0 = s.resid;
    s.rho = tt;
    if (!isfinite(s.resid)) bad = true;
    if (dfpass) {
      if (s.resid <= s.atol - s.dfe) s.active = 0;
      else if (s.resid <= s.atol + s.dfe) s.exact = 1;
    } else if (s.resid <= s.atol) s.active = 0;
    else if (s.iters >= maxiter) {
      s.active = 0;
      s.unconv = 1;
    }
  }
  if (s.active) {
    alpha = (s.need ? tp : s.rho) / pq;
    if (!isfinite(alpha)) bad = true;
  }
  return bad;
}

// After the r.r reduction: count the iteration, schedule a reliable update
// (residual fell by delta since the last true residual, reached the
// threshold, or maxiter) and return beta.  Returns true on a non-finite value.
__device__ __forceinline__ bool ir_after_rr(IRState &s, double rr, double delta, int maxiter, float &beta) {
  s.need = 0;
  beta = 0.0f;
  if (!s.active) return false;
  const bool bad = !isfinite(rr);
  s.iters += 1;
  const double rn = sqrt(rr);
  s.need = (rn < delta * s.r0) || (rn <= s.atol) || (s.iters >= maxiter);
  s.dfok = s.need && s.dfe > 0.0 && !s.exact && s.iters < maxiter;
  beta = (float)(rr / s.rho);
  s.rho = rr;
  return bad;
}

// ---------------------------------------------------------------- two-barrier reliable-update CG state
// One system of the FP32 CG with two grid barriers per iteration
// (csrc/stencil.cu, cg_stencil_ir2_kernel).  The iteration keeps s ~ A p
// beside p and forms w = A r in its only product, so each iteration needs one
// reduction of four sums of the current residual r:
//   g = r.r, dl = r.w, e = r.s_prev, f = r.p_prev
// from which (A symmetric, so p_prev.w = s_prev.r)
//   beta = g / g_prev,  p.s = dl + 2 beta e + beta^2 (p.s)_prev,  r.p = g + beta f,
//   alpha = (r.p) / (p.s)
// (alpha as an exact line search along p, which keeps the iteration sound after
// r is replaced).  A reliable update is a replacement pass: the true residual
// t = b - A64 (x + d) replaces r, the next product forms w = A t, and the
// convergence test ||b - A x|| <= tol ||b|| is decided on t alone.
struct IR2State {
  double atol, resid, r0, gprev, psprev;
  int active, rep, first, iters, unconv, updates;
};

__device__ __forceinline__ void ir2_init(IR2State &s, double bnorm, double rr0, double tol) {
  s.atol = tol * bnorm;
  s.resid = sqrt(rr0);
  s.r0 = s.resid;
  s.gprev = 0.0;
  s.psprev = 0.0;
  s.active = bnorm != 0.0;
  s.rep = 0;
  s.first = 1;
  s.iters = 0;
  s.unconv = 0;
  s.updates = 0;
}

// After the reduction of (g, dl, e, f): mode 0 = idle (converged or stopped),
// 1 = update with alpha and beta, 2 = replacement pass (the product of this
// pass is discarded).  Returns true on a non-finite value.
__device__ __forceinline__ bool ir2_after(IR2State &s, double g, double dl, double e, double f, double delta,
                                          int maxiter, float &alpha, float &beta, int &mode) {
  mode = 0;
  alpha = beta = 0.0f;
  if (!s.active) return false;
  if (!isfinite(g)) return true;
  if (s.rep) {
    // g = t.t of the true residual: decide convergence on it
    s.rep = 0;
    s.resid = sqrt(g);
    s.r0 = s.resid;
    if (s.resid <= s.atol) {
      s.active = 0;
      return false;
    }
    if (s.iters >= maxiter) {
      s.active = 0;
      s.unconv = 1;
      return false;
    }
  } else if (!s.first) {
    // g = r.r of the recursive residual left by the last update
    s.iters += 1;
    const double rn = sqrt(g);
    if (rn < delta * s.r0 || rn <= s.atol || s.iters >= maxiter) {
      s.rep = 1;
      s.updates += 1;
      mode = 2;
      return false;
    }
  }
  const double b = s.first ? 0.0 : g / s.gprev;
  const double ps = s.first ? dl : dl + 2.0 * b * e + b * b * s.psprev;
  const double rp = s.first ? g : g + b * f;
  const double a = rp / ps;
  if (!isfinite(a) || !isfinite(b)) return true;
  s.first = 0;
  s.gprev = g;
  s.psprev = ps;
  alpha = (float)a;
  beta = (float)b;
  mode = 1;
  return false;
}

// Block-wide sums of the first nv of NV values per thread, up to eight values
// at a time (warp w adds value w): per value the order of block_sum (lane l
// adds threads 8l..8l+7 in order, then the fixed shuffle tree), with two block
// barriers per eight values.  The totals land in tot[0..nv) (shared) and in v.
// s_w: the kernel's one shared staging array of 8 x kCGThreads doubles.
template <int NV>
__device__ __forceinline__ void block_sum_wide(double (&v)[NV], double *tot, double (*s_w)[kCGThreads],
                                               int nv = NV) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j0 = 0; j0 < NV; j0 += 8) {
    if (j0 >= nv) break;
#pragma unroll
    for (int jj = 0; jj < 8; ++jj)
      if (j0 + jj < NV && j0 + jj < nv) s_w[jj][threadIdx.x] = v[j0 + jj];
    __syncthreads();
    if (j0 + warp < nv && j0 + warp < NV) {
      double t = 0.0;
#pragma unroll
      for (int k = 0; k < kCGThreads / kWarp; ++k) t += s_w[warp][k * kWarp + lane];
      t = warp_sum(t);
      if (lane == 0) tot[j0 + warp] = t;
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < NV; ++j)
    if (j < nv) v[j] = tot[j];
}

// Totals over all CTAs of records of NV values (record of CTA g at half + g*NV),
// added in CTA order by every CTA after a grid barrier.
template <int NV>
__device__ __forceinline__ void sum_records(const double *half, int G, double (&v)[NV], double *tot,
                                            double (*s_w)[kCGThreads]) {
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j] = 0.0;
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] += __ldcg(&half[(size_t)g * NV + j]);
  }
  block_sum_wide<NV>(v, tot, s_w);
}

__device__ __forceinline__ void set_status(cpm_cg_info *info, int st) {
  atomicMax(&info->status, st);
}

// ------------------------------------------------------------------ launch
struct Workspace {
  GridBarrier *bar;
  double *part;
  double *r, *p0, *p1, *q;
  float *r32, *pa32, *pb32, *q32, *d32;
};

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// CTAs per SM of the FP32 solvers: fewer, fuller CTAs while the work is small
// (fewer grid-barrier arrivals and partial sums, more independent loads per
// thread), up to the resident limit.  Measured on GB300 (elastic 48^3..128^3,
// scalar 64^3..128^3): the best shapes hold about 4500 DOFs per CTA for
// operators with 3 unknowns per DOF and about 6500 for scalar ones.
inline int ir_ctas_per_sm(int64_t dofs, int unknowns_per_dof, int occ) {
  const int64_t per_sm = dofs / (sm_count() > 0 ? sm_count() : 1);
  const int64_t target = unknowns_per_dof >= 3 ? 4500 : 6500;
  int64_t c = per_sm / target;
  if (c < 1) c = 1;
  if (c > occ) c = occ;
  return (int)c;
}




inline size_t layout(int64_t n, int nrhs, int precision, char *base, Workspace *w) {
  size_t off = 0;
  auto take = [&](size_t bytes) -> char * {
    char *p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  Workspace t{};
  t.bar = (GridBarrier *)take(sizeof(GridBarrier));
  t.part = (double *)take(sizeof(double) * 2 * kPartHalf);
  const size_t nv = (size_t)n * nrhs;
  if (precision == 0) {
    t.r = (double *)take(8 * nv);
    t.p0 = (double *)take(8 * nv);
    t.p1 = (double *)take(8 * nv);
    t.q = (double *)take(8 * nv);
  } else {
    t.r32 = (float *)take(4 * nv);
    t.pa32 = (float *)take(4 * nv);
    t.pb32 = (float *)take(4 * nv);
    t.q32 = (float *)take(4 * nv);
    t.d32 = (float *)take(4 * nv);
  }
  if (w) *w = t;
  return off;
}


}  // namespace cpm
