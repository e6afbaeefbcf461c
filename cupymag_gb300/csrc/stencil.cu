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
// (precision 0) or as FP32 CG inside FP64 iterative refinement (precision 1):
// the refinement residual b - A x applies the FP64 coefficients to the FP64
// x, so the stopping test ||b - A x|| <= tol ||b|| is the FP64 one, while the
// inner iterations run on FP32 vectors with FP32 coefficients and FP64 dot
// accumulation.  GB300 issues FP32 FMAs at many times its FP64 rate, so the
// FP32 inner iterations are bound by the vectors' L2/HBM traffic alone.
#include <cmath>

#include "cg_common.cuh"

namespace cpm {

enum : uint8_t { kRowIdentity = 1, kRowZero = 2, kColExcluded = 4 };

struct StencilOp {
  int nx, ny, nz;
  int64_t n;
  const double *c64;
  const float *c32;
  const uint8_t *flags;
};

// Wrapped neighbour offsets of a DOF along each axis (index 0: -1, 1: 0, 2: +1).
struct Nbr {
  int64_t xi[3];
  int yj[3];
  int zk[3];
};

__device__ __forceinline__ Nbr neighbours(const StencilOp &S, int64_t dof) {
  const int64_t nyz = (int64_t)S.ny * S.nz;
  const int i = (int)(dof / nyz);
  const int64_t rem = dof - (int64_t)i * nyz;
  const int j = (int)(rem / S.nz);
  const int k = (int)(rem - (int64_t)j * S.nz);
  Nbr b;
  b.xi[0] = (int64_t)(i == 0 ? S.nx - 1 : i - 1) * nyz;
  b.xi[1] = (int64_t)i * nyz;
  b.xi[2] = (int64_t)(i == S.nx - 1 ? 0 : i + 1) * nyz;
  b.yj[0] = (j == 0 ? S.ny - 1 : j - 1) * S.nz;
  b.yj[1] = j * S.nz;
  b.yj[2] = (j == S.ny - 1 ? 0 : j + 1) * S.nz;
  b.zk[0] = k == 0 ? S.nz - 1 : k - 1;
  b.zk[1] = k;
  b.zk[2] = k == S.nz - 1 ? 0 : k + 1;
  return b;
}

// y = A x at one DOF for a scalar operator (nc = 1), nr interleaved vectors.
// Accumulates in T (FP64 for the FP64 products, FP32 for the inner solve).
template <typename T, int NR>
__device__ __forceinline__ void apply_scalar(const StencilOp &S, const T *c, const T *x, int64_t dof, T (&y)[NR]) {
#pragma unroll
  for (int r = 0; r < NR; ++r) y[r] = T(0);
  const uint8_t f = S.flags ? S.flags[dof] : 0;
  if (f & kRowIdentity) {
#pragma unroll
    for (int r = 0; r < NR; ++r) y[r] = x[dof * NR + r];
    return;
  }
  if (f & kRowZero) return;
  const Nbr b = neighbours(S, dof);
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int bb = 0; bb < 3; ++bb)
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        const int64_t q = b.xi[a] + b.yj[bb] + b.zk[cc];
        if (S.flags && (S.flags[q] & kColExcluded)) continue;
        const T w = c[(a * 3 + bb) * 3 + cc];
#pragma unroll
        for (int r = 0; r < NR; ++r) y[r] = fma(w, x[q * NR + r], y[r]);
      }
}

// y = A x at one DOF for the elastic operator (nc = 3, block vectors).
template <typename T>
__device__ __forceinline__ void apply_elastic(const StencilOp &S, const T *c, const T *x, int64_t dof, T (&y)[3]) {
  const int64_t n = S.n;
  y[0] = y[1] = y[2] = T(0);
  const uint8_t f = S.flags ? S.flags[dof] : 0;
  if (f & kRowIdentity) {
    y[0] = x[dof];
    y[1] = x[n + dof];
    y[2] = x[2 * n + dof];
    return;
  }
  if (f & kRowZero) return;
  const Nbr b = neighbours(S, dof);
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int bb = 0; bb < 3; ++bb)
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        const int64_t q = b.xi[a] + b.yj[bb] + b.zk[cc];
        if (S.flags && (S.flags[q] & kColExcluded)) continue;
        const int d = (a * 3 + bb) * 3 + cc;
        const T u0 = x[q], u1 = x[n + q], u2 = x[2 * n + q];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          T acc = y[r];
          acc = fma(c[(r * 3 + 0) * 27 + d], u0, acc);
          acc = fma(c[(r * 3 + 1) * 27 + d], u1, acc);
          acc = fma(c[(r * 3 + 2) * 27 + d], u2, acc);
          y[r] = acc;
        }
      }
}

// Unknown index of (dof, component) for the NC/NR layouts.
template <int NC, int NR>
__device__ __forceinline__ int64_t uidx(int64_t n, int64_t dof, int comp) {
  return NC == 1 ? dof * NR + comp : (int64_t)comp * n + dof;
}

// y at one DOF (all NC*NR components) in T.
template <typename T, int NC, int NR>
__device__ __forceinline__ void apply(const StencilOp &S, const T *c, const T *x, int64_t dof, T (&y)[NC * NR]) {
  if (NC == 1) {
    T t[NR];
    apply_scalar<T, NR>(S, c, x, dof, t);
#pragma unroll
    for (int r = 0; r < NR; ++r) y[r] = t[r];
  } else {
    T t[3];
    apply_elastic<T>(S, c, x, dof, t);
#pragma unroll
    for (int r = 0; r < 3; ++r) y[r] = t[r];
  }
}

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
  float *r32, *p32, *q32, *d32;  // FP32 vectors (precision 1)
  double *part;
  GridBarrier *bar;
  cpm_cg_info *info;
  unsigned long long timeout_ns;
  int64_t dofs_per_cta;
};

// Number of independent systems (each with its own CG scalars).
template <int NC, int NR>
__host__ __device__ constexpr int n_systems() { return NC == 1 ? NR : 1; }

template <int NC, int NR>
__device__ __forceinline__ int sys_of(int comp) { return NC == 1 ? comp : 0; }

// Coefficients staged in shared memory (27 * NC * NC values).
template <typename T, int NC>
__device__ __forceinline__ const T *stage_coef(const T *c, T *smem) {
  for (int i = threadIdx.x; i < 27 * NC * NC; i += blockDim.x) smem[i] = c[i];
  __syncthreads();
  return smem;
}

// ---------------------------------------------------------------- FP64 stencil CG
template <int NC, int NR>
__global__ void __launch_bounds__(kCGThreads) cg_stencil_fp64_kernel(StencilCG a) {
  constexpr int U = NC * NR;
  constexpr int NS = n_systems<NC, NR>();
  __shared__ double s_red[2 * 3][kCGWarps];
  __shared__ double s_c[27 * NC * NC];
  const double *c = stage_coef<double, NC>(a.S.c64, s_c);
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
    if (use_init) apply<double, NC, NR>(a.S, c, a.x, dof, y);
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
      apply<double, NC, NR>(a.S, c, a.p, dof, y);
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

// ---------------------------------------------------------------- FP32 CG in FP64 refinement
template <int NC, int NR>
__global__ void __launch_bounds__(kCGThreads) cg_stencil_ir_kernel(StencilCG a) {
  constexpr int U = NC * NR;
  constexpr int NS = n_systems<NC, NR>();
  __shared__ double s_red[2 * 3][kCGWarps];
  __shared__ double s_c[27 * NC * NC];
  __shared__ float s_c32[27 * NC * NC];
  const double *c = stage_coef<double, NC>(a.S.c64, s_c);
  const float *c32 = stage_coef<float, NC>(a.S.c32, s_c32);
  const int64_t n = a.S.n;
  const int64_t d0 = min(n, (int64_t)blockIdx.x * a.dofs_per_cta);
  const int64_t d1 = min(n, d0 + a.dofs_per_cta);
  const bool use_init = a.use_init_dev ? (__ldcg(a.use_init_dev) != 0) : (a.use_init_host != 0);
  const unsigned long long tns = a.timeout_ns;
  int par = 0;

  double bb[NS];
#pragma unroll
  for (int j = 0; j < NS; ++j) bb[j] = 0.0;
  for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads)
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t i = uidx<NC, NR>(n, dof, u);
      const double bi = a.b[i];
      if (!use_init) a.x[i] = 0.0;
      bb[sys_of<NC, NR>(u)] = fma(bi, bi, bb[sys_of<NC, NR>(u)]);
    }
  if (!grid_sum<NS>(bb, a.part, par, a.bar, tns, s_red)) {
    set_status(a.info, CPM_BARRIER_TIMEOUT);
    return;
  }
  double atol[NS], resid[NS];
  int active[NS], iters[NS];
  bool any = false;
#pragma unroll
  for (int j = 0; j < NS; ++j) {
    const double bn = sqrt(bb[j]);
    atol[j] = a.tol * bn;
    resid[j] = bn;
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
  int outer = 0, total = 0;
  while (any) {
    // ---- refinement residual in FP64: r = b - A x; FP32 copies; d = 0
    if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
    double red[2 * NS];
#pragma unroll
    for (int j = 0; j < 2 * NS; ++j) red[j] = 0.0;
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
      double y[U];
      apply<double, NC, NR>(a.S, c, a.x, dof, y);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = uidx<NC, NR>(n, dof, u);
        const double ri = a.b[i] - y[u];
        const float rf = (float)ri;
        a.r32[i] = rf;
        a.p32[i] = rf;
        a.d32[i] = 0.0f;
        const int s = sys_of<NC, NR>(u);
        red[s] = fma(ri, ri, red[s]);
        red[NS + s] = fma((double)rf, (double)rf, red[NS + s]);
      }
    }
    if (!grid_sum<2 * NS>(red, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
    any = false;
    double rho[NS], iatol[NS];
    int iact[NS];
    bool iany = false;
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      if (active[j]) {
        resid[j] = sqrt(red[j]);
        if (!(resid[j] > atol[j])) active[j] = 0;
      }
      any |= active[j] != 0;
      rho[j] = red[NS + j];
      iact[j] = active[j];
      iatol[j] = a.inner_tol * sqrt(red[NS + j]);
      iany |= iact[j] != 0;
    }
    if (!any || outer >= a.max_outer || total >= a.maxiter) break;
    ++outer;
    // ---- inner FP32 CG on A d = r
    for (int kin = 0; iany && total < a.maxiter; ++kin, ++total) {
      if (kin > 0 && !grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
      double pq[NS];
#pragma unroll
      for (int j = 0; j < NS; ++j) pq[j] = 0.0;
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
        float y[U];
        apply<float, NC, NR>(a.S, c32, a.p32, dof, y);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t i = uidx<NC, NR>(n, dof, u);
          a.q32[i] = y[u];
          const int s = sys_of<NC, NR>(u);
          pq[s] = fma((double)a.p32[i], (double)y[u], pq[s]);
        }
      }
      if (!grid_sum<NS>(pq, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
      double alpha[NS];
      bool bad = false;
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        alpha[j] = iact[j] ? rho[j] / pq[j] : 0.0;
        if (iact[j] && !isfinite(alpha[j])) bad = true;
      }
      if (bad) { status = CPM_NONFINITE; break; }
      double rr[NS];
#pragma unroll
      for (int j = 0; j < NS; ++j) rr[j] = 0.0;
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int s = sys_of<NC, NR>(u);
          if (!iact[s]) continue;
          const int64_t i = uidx<NC, NR>(n, dof, u);
          const float af = (float)alpha[s];
          a.d32[i] = fmaf(af, a.p32[i], a.d32[i]);
          const float rn = fmaf(-af, a.q32[i], a.r32[i]);
          a.r32[i] = rn;
          rr[s] = fma((double)rn, (double)rn, rr[s]);
        }
      }
      if (!grid_sum<NS>(rr, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
      iany = false;
      float beta[NS];
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        beta[j] = 0.0f;
        if (!iact[j]) continue;
        if (!isfinite(rr[j])) bad = true;
        iters[j] += 1;
        beta[j] = (float)(rr[j] / rho[j]);
        rho[j] = rr[j];
        if (sqrt(rr[j]) <= iatol[j]) iact[j] = 0;
        iany |= iact[j] != 0;
      }
      if (bad) { status = CPM_NONFINITE; break; }
      if (!iany) break;
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int s = sys_of<NC, NR>(u);
          if (!iact[s]) continue;
          const int64_t i = uidx<NC, NR>(n, dof, u);
          a.p32[i] = fmaf(beta[s], a.p32[i], a.r32[i]);
        }
      }
    }
    if (status != CPM_OK) break;
    // ---- x += d (own DOFs only; the next residual pass starts with a barrier)
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads)
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = uidx<NC, NR>(n, dof, u);
        if (active[sys_of<NC, NR>(u)]) a.x[i] += (double)a.d32[i];
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
    a.info->outer = outer;
    set_status(a.info, st);
  } else if (status != CPM_OK && threadIdx.x == 0) {
    set_status(a.info, status);
  }
}

// ---------------------------------------------------------------- y = alpha A x (FP64)
template <int NC, int NR>
__global__ void __launch_bounds__(256) stencil_apply_kernel(StencilOp S, const double *x, double *y, double alpha) {
  __shared__ double s_c[27 * NC * NC];
  const double *c = stage_coef<double, NC>(S.c64, s_c);
  for (int64_t dof = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; dof < S.n;
       dof += (int64_t)gridDim.x * blockDim.x) {
    double t[NC * NR];
    apply<double, NC, NR>(S, c, x, dof, t);
#pragma unroll
    for (int u = 0; u < NC * NR; ++u) y[uidx<NC, NR>(S.n, dof, u)] = alpha * t[u];
  }
}

static StencilOp to_op(const cpm_stencil *s) {
  StencilOp S;
  S.nx = s->nx;
  S.ny = s->ny;
  S.nz = s->nz;
  S.n = (int64_t)s->nx * s->ny * s->nz;
  S.c64 = s->coef;
  S.c32 = s->coef32;
  S.flags = s->flags;
  return S;
}

static int check_stencil(const cpm_stencil *s, const char *who) {
  if (!s || !s->coef || s->nx < 3 || s->ny < 3 || s->nz < 3 || (s->ncomp != 1 && s->ncomp != 3)) {
    set_error("%s: bad stencil (needs coefficients, at least 3 cells per axis, ncomp 1 or 3)", who);
    return CPM_BAD_ARG;
  }
  return CPM_OK;
}

template <int NC, int NR>
static int launch_stencil_cg(const cpm_stencil *s, const double *b, double *x, const cpm_cg_opts *o, Workspace &w,
                             cpm_cg_info *info, cudaStream_t st) {
  StencilCG a{};
  a.S = to_op(s);
  a.b = b;
  a.x = x;
  a.tol = o->tol;
  a.maxiter = o->maxiter;
  a.use_init_host = o->use_init_host;
  a.use_init_dev = o->use_init_dev;
  a.inner_tol = o->inner_tol > 0 ? o->inner_tol : 1e-4;
  a.max_outer = o->max_outer > 0 ? o->max_outer : 60;
  a.r = w.r;
  a.p = w.p0;
  a.q = w.q;
  a.r32 = w.r32;
  a.p32 = w.pa32;
  a.q32 = w.q32;
  a.d32 = w.d32;
  a.part = w.part;
  a.bar = w.bar;
  a.info = info;
  const double tmo = o->barrier_timeout_s > 0 ? o->barrier_timeout_s : 2.0;
  a.timeout_ns = (unsigned long long)(tmo * 1e9);
  const bool fp64 = o->precision == 0;
  const void *fn = fp64 ? (const void *)cg_stencil_fp64_kernel<NC, NR> : (const void *)cg_stencil_ir_kernel<NC, NR>;
  int occ = 0;
  CPM_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kCGThreads, 0));
  if (occ < 1) {
    set_error("stencil cg: kernel cannot be resident on an SM");
    return CPM_CUDA_ERROR;
  }
  const int64_t n = a.S.n;
  int64_t gmax = (int64_t)occ * sm_count();
  if (gmax > kMaxGrid) gmax = kMaxGrid;
  int64_t G = (n + 255) / 256;
  if (G > gmax) G = gmax;
  if (G < 1) G = 1;
  int64_t per = (n + G - 1) / G;
  per = (per + 31) / 32 * 32;
  G = (n + per - 1) / per;
  a.dofs_per_cta = per;
  CPM_TRY(cudaMemsetAsync(w.bar, 0, sizeof(GridBarrier), st));
  CPM_TRY(cudaMemsetAsync(info, 0, sizeof(cpm_cg_info), st));
  void *args[] = {&a};
  CPM_TRY(cudaLaunchCooperativeKernel(fn, dim3((unsigned)G), dim3(kCGThreads), args, 0, st));
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
  if (prec && !S->coef32) {
    set_error("cpm_cg_solve_stencil: mixed precision needs the FP32 coefficients");
    return CPM_BAD_ARG;
  }
  const int64_t n = (int64_t)S->nx * S->ny * S->nz;
  const int64_t unknowns = n * S->ncomp;
  const size_t need = layout(unknowns, nrhs, prec, nullptr, nullptr);
  if (workspace_bytes < need) {
    set_error("cpm_cg_solve_stencil: workspace too small (%zu < %zu bytes)", workspace_bytes, need);
    return CPM_BAD_ARG;
  }
  Workspace w;
  layout(unknowns, nrhs, prec, (char *)workspace, &w);
  cudaStream_t st = (cudaStream_t)stream;
  if (S->ncomp == 3) return launch_stencil_cg<3, 1>(S, b, x, opts, w, info_dev, st);
  return nrhs == 1 ? launch_stencil_cg<1, 1>(S, b, x, opts, w, info_dev, st)
                   : launch_stencil_cg<1, 3>(S, b, x, opts, w, info_dev, st);
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
  if (S->ncomp == 3)
    stencil_apply_kernel<3, 1><<<(int)g, 256, 0, st>>>(op, x, y, alpha);
  else if (nvec == 1)
    stencil_apply_kernel<1, 1><<<(int)g, 256, 0, st>>>(op, x, y, alpha);
  else
    stencil_apply_kernel<1, 3><<<(int)g, 256, 0, st>>>(op, x, y, alpha);
  return check_launch("cpm_stencil_apply");
}
