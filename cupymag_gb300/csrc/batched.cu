// Block-diagonal conjugate gradient: many stencil systems in one persistent
// cooperative launch (sm_103a).  This is the solver of the serving loop.
//
// A batch holds S independent systems A_s x_s = b_s of one operator kind
// (scalar with 1 or 3 right-hand sides, or elastic) on periodic hex grids of
// different sizes that share one coefficient table (requests with the same
// material and time step).  Each system's DOFs are cut into chunks whose size
// depends only on the operator kind and the system's own size; a chunk's
// partial dot products are reduced in a fixed order, and a system's totals add
// its own chunks' partials in a fixed order.  A system's iterates are
// therefore bit-for-bit the same whether it is solved alone or together with
// any other systems: the batch only changes which CTA works on which chunk.
//
// CTAs are given to systems in proportion to their chunks (equal load per
// CTA; CTA l of a system takes its chunks l, l + ncta, ...).  All CTAs pass
// the same grid barriers; a system that has converged idles, and the launch
// ends when a device counter of systems that are still iterating drops to
// zero.  Every wait is bounded (GridBarrier).
//
// Precision 0 is the three-phase FP64 CG of csrc/stencil.cu.  Precision 1 is
// FP32 CG with FP64 reliable updates in a form that needs no extra barrier:
// when the FP32 recursive residual has fallen by inner_tol (or below the
// stopping threshold, or at maxiter), the next iteration's first phase also
// computes the true residual t = b - A64 x in FP64 beside q = A32 p (the
// direction phase before it folded d into x); t replaces the FP32 residual
// and rho and decides convergence.  The direction p of that iteration was formed from
// the recursive residual, so its step length is the exact line search
// alpha = (t.p) / (p.A p) rather than (t.t) / (p.A p).  The stopping test is
// only ever decided on the FP64 true residual.
#include <algorithm>
#include <cmath>
#include <vector>

#include "stencil_ops.cuh"

namespace cpm {

constexpr int kSlot = 12;        // doubles per chunk partial (>= 3 values x 3 systems)
constexpr int kMaxChunks = 1024;  // chunks of one system (a multiple of kCGThreads)

// Grid geometry of one system in registers.
struct Geo {
  int nx, ny, nz, n;
  const uint8_t *flags;
};

struct BSeg {
  int nx, ny, nz, n;
  const uint8_t *flags;
  const double *b;
  double *x;
  const int *use_init_dev;
  cpm_cg_info *info;
  double tol;
  int maxiter;
  int chunk0, nchunks, cta0, ncta, chunk_dofs;
  int quads;                     // FP32 product on quads of 4 DOFs along z
  double *r, *p, *q;             // precision 0
  float *r32, *p32, *q32, *d32;  // precision 1 (the two-barrier form uses q32 as w = A r)
  float *s32;                    // two-barrier form: s ~ A p
};

struct BatchArgs {
  double c64[243];
  float c32[243];
  const BSeg *segs;
  const int *cta_seg;
  double *part;          // two halves of total_chunks * kSlot doubles
  long long half;
  GridBarrier *bar;
  int *live;             // systems (segments) still iterating
  unsigned long long timeout_ns;
  double inner_tol;
};

template <int NC, int NR>
__host__ __device__ constexpr int b_systems() { return NC == 1 ? NR : 1; }

template <int NC, int NR>
__device__ __forceinline__ int b_sys(int comp) { return NC == 1 ? comp : 0; }

// Chunks whose warp sums a CTA stages in shared memory before one flush.
constexpr int kStage = 8;
constexpr int kStageDoubles = kStage * 9 * kCGWarps;

// Partials of this CTA's chunks: body(d0, d1, v) accumulates the calling
// thread's DOFs of [d0, d1) (stride kCGThreads) into v.  A chunk's partial is
// the sum, in warp order, of its warps' shuffle sums: the same value whichever
// CTA computes the chunk.  The warp sums of up to kStage chunks wait in
// `stage` and are added and written together, so a chunk costs shuffles but
// no block barrier.
struct SlotIdentity {
  __device__ __forceinline__ int operator()(int j) const { return j; }
};

template <int NV, typename Body, typename Slot = SlotIdentity>
__device__ __forceinline__ void chunk_partials(const BSeg &S, int l, double *half, double *stage, int nv,
                                               Body body, Slot slot = Slot()) {
  static_assert(NV <= 9, "stage holds at most 9 sums per chunk");
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int held = 0, first = l;
  for (int c = l; c < S.nchunks; c += S.ncta) {
    double v[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = 0.0;
    const int d0 = c * S.chunk_dofs;
    const int d1 = min(S.n, d0 + S.chunk_dofs);
    body(d0, d1, v);
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      if (j >= nv) break;
      const double t = warp_sum(v[j]);
      if (lane == 0) stage[(held * NV + j) * kCGWarps + w] = t;
    }
    if (++held == kStage || c + S.ncta >= S.nchunks) {
      __syncthreads();
      for (int t = threadIdx.x; t < held * NV; t += kCGThreads) {
        const int cl = t / NV, j = t - cl * NV;
        if (j >= nv) continue;
        const double *src = stage + t * kCGWarps;
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < kCGWarps; ++k) s += src[k];
        half[(size_t)(S.chunk0 + first + cl * S.ncta) * kSlot + slot(j)] = s;
      }
      __syncthreads();
      held = 0;
      first = c + S.ncta;
    }
  }
}

// One reduction of the first nv of NV values: this CTA's chunk partials (when
// `work`), a grid barrier, the segment's totals in chunk order (values nv..
// come back zero).  Every CTA calls it equally often; the partial buffer
// alternates halves as in grid_sum.
template <int NV, typename Body>
__device__ __forceinline__ bool seg_reduce(const BatchArgs &a, const BSeg &S, int l, bool work, int &par,
                                           double (*sred)[kCGWarps], double *stage, double (&v)[NV], Body body,
                                           int nv = NV) {
  double *half = a.part + (size_t)par * (size_t)a.half;
  par ^= 1;
  if (work) chunk_partials<NV>(S, l, half, stage, nv, body);
  if (!grid_sync(a.bar, gridDim.x, a.timeout_ns)) return false;
  if (work) {
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = 0.0;
    // at most kMaxChunks / kCGThreads = 4 chunk partials per thread, in chunk order
    for (int c = threadIdx.x; c < S.nchunks; c += kCGThreads) {
      const double *src = half + (size_t)(S.chunk0 + c) * kSlot;
#pragma unroll
      for (int j = 0; j < NV; ++j)
        if (j < nv) v[j] += __ldcg(src + j);
    }
    block_sum<NV>(v, sred, nv);
  }
  return true;
}

__device__ __forceinline__ void write_info(cpm_cg_info *info, int status, const int *iters, const double *resid,
                                           int ns, int outer, const GridBarrier *bar) {
  int st = status;
  if (*(volatile const int *)&bar->error && st == CPM_OK) st = CPM_BARRIER_TIMEOUT;
  for (int j = 0; j < 3; ++j) {
    info->iters[j] = j < ns ? iters[j] : 0;
    info->resid[j] = j < ns ? resid[j] : 0.0;
  }
  info->outer = outer;
  info->df_updates = 0;
  info->status = st;
}

// ---------------------------------------------------------------- FP64
template <int NC, int NR>
__global__ void __launch_bounds__(kCGThreads, 2) cg_batched_fp64_kernel(const __grid_constant__ BatchArgs a) {
  constexpr int U = NC * NR;
  constexpr int NS = b_systems<NC, NR>();
  __shared__ double s_red[9][kCGWarps];
  __shared__ double s_stage[kStageDoubles];
  // the CTA's system record, read once into shared memory (its fields are re-read cheaply there)
  __shared__ BSeg s_seg;
  if (threadIdx.x == 0) s_seg = a.segs[a.cta_seg[blockIdx.x]];
  __syncthreads();
  const BSeg &S = s_seg;
  const int l = blockIdx.x - S.cta0;
  const bool lead = l == 0 && threadIdx.x == 0;
  const Geo g{S.nx, S.ny, S.nz, S.n, S.flags};
  const int64_t n = g.n;
  const double *__restrict__ b = S.b;
  double *x = S.x, *r = S.r, *p = S.p, *q = S.q;
  const double tol = S.tol;
  const int maxiter = S.maxiter;
  const bool use_init = S.use_init_dev && __ldcg(S.use_init_dev) != 0;
  const double *c = a.c64;
  int par = 0;

  double v[2 * NS];
  bool ok = seg_reduce<2 * NS>(a, S, l, true, par, s_red, s_stage, v, [&](int d0, int d1, double (&w)[2 * NS]) {
    for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
      double y[U];
      if (use_init) apply_c<double, NC, NR>(g, c, x, dof, y);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = uidx<NC, NR>(n, dof, u);
        const double bi = b[i];
        const double ri = use_init ? bi - y[u] : bi;
        r[i] = ri;
        p[i] = ri;
        if (!use_init) x[i] = 0.0;
        const int s = b_sys<NC, NR>(u);
        w[s] = fma(bi, bi, w[s]);
        w[NS + s] = fma(ri, ri, w[NS + s]);
      }
    }
  });
  double atol[NS], rho[NS], resid[NS];
  int active[NS], iters[NS], unconv[NS];
  bool any = false;
  int status = ok ? CPM_OK : CPM_BARRIER_TIMEOUT;
#pragma unroll
  for (int j = 0; j < NS; ++j) {
    const double bn = ok ? sqrt(v[j]) : 0.0;
    atol[j] = tol * bn;
    rho[j] = ok ? v[NS + j] : 0.0;
    resid[j] = sqrt(rho[j]);
    active[j] = bn != 0.0;
    iters[j] = 0;
    unconv[j] = 0;
    any |= active[j] != 0;
  }
  if (lead) {
    for (int j = 0; j < 3; ++j) S.info->bnorm[j] = j < NS ? sqrt(ok ? v[j] : 0.0) : 0.0;
    if (any) atomicAdd(a.live, 1);
  }
  if (ok && use_init) {
    for (int cc = l; cc < S.nchunks; cc += S.ncta) {
      const int d1 = min(g.n, (cc + 1) * S.chunk_dofs);
      for (int dof = cc * S.chunk_dofs + threadIdx.x; dof < d1; dof += kCGThreads)
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (!active[b_sys<NC, NR>(u)]) x[uidx<NC, NR>(n, dof, u)] = b[uidx<NC, NR>(n, dof, u)];
    }
  }
  for (int k = 0; ok; ++k) {
    if (k > 0) {
      if (!grid_sync(a.bar, gridDim.x, a.timeout_ns)) { status = CPM_BARRIER_TIMEOUT; break; }
      // every change of the counter happened before this barrier and none
      // happens before the next one: all CTAs read the same value
      if (__ldcg(a.live) == 0) break;
    }
    // ---- q = A p, p.q
    double pq[NS];
    if (!seg_reduce<NS>(a, S, l, any, par, s_red, s_stage, pq, [&](int d0, int d1, double (&w)[NS]) {
          for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
            double y[U];
            apply_c<double, NC, NR>(g, c, p, dof, y);
#pragma unroll
            for (int u = 0; u < U; ++u) {
              const int64_t i = uidx<NC, NR>(n, dof, u);
              q[i] = y[u];
              w[b_sys<NC, NR>(u)] = fma(p[i], y[u], w[b_sys<NC, NR>(u)]);
            }
          }
        })) {
      status = CPM_BARRIER_TIMEOUT;
      break;
    }
    double alpha[NS];
    bool bad = false;
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      alpha[j] = (any && active[j]) ? rho[j] / pq[j] : 0.0;
      if (any && active[j] && !isfinite(alpha[j])) bad = true;
    }
    if (bad) {
      status = CPM_NONFINITE;
#pragma unroll
      for (int j = 0; j < NS; ++j) active[j] = 0;
      if (lead) atomicSub(a.live, 1);
      any = false;
    }
    // ---- x += alpha p, r -= alpha q, r.r
    double rr[NS];
    if (!seg_reduce<NS>(a, S, l, any, par, s_red, s_stage, rr, [&](int d0, int d1, double (&w)[NS]) {
          for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
#pragma unroll
            for (int u = 0; u < U; ++u) {
              const int s = b_sys<NC, NR>(u);
              if (!active[s]) continue;
              const int64_t i = uidx<NC, NR>(n, dof, u);
              x[i] = __fma_rn(alpha[s], p[i], x[i]);
              const double rn = __fma_rn(-alpha[s], q[i], r[i]);
              r[i] = rn;
              w[s] = fma(rn, rn, w[s]);
            }
          }
        })) {
      status = CPM_BARRIER_TIMEOUT;
      break;
    }
    if (!any) continue;
    double beta[NS];
    bool still = false;
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
      else if (iters[j] >= maxiter) { active[j] = 0; unconv[j] = 1; }
      still |= active[j] != 0;
    }
    if (bad) {
      status = CPM_NONFINITE;
      still = false;
    }
    if (!still) {
      if (lead) atomicSub(a.live, 1);
      any = false;
      continue;
    }
    // ---- p = r + beta p
    for (int cc = l; cc < S.nchunks; cc += S.ncta) {
      const int d1 = min(g.n, (cc + 1) * S.chunk_dofs);
      for (int dof = cc * S.chunk_dofs + threadIdx.x; dof < d1; dof += kCGThreads)
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int s = b_sys<NC, NR>(u);
          if (!active[s]) continue;
          const int64_t i = uidx<NC, NR>(n, dof, u);
          p[i] = __fma_rn(beta[s], p[i], r[i]);
        }
    }
  }
  if (lead) {
    int st = status;
#pragma unroll
    for (int j = 0; j < NS; ++j)
      if (st == CPM_OK && (unconv[j] || active[j])) st = CPM_NOT_CONVERGED;
    write_info(S.info, st, iters, resid, NS, 0, a.bar);
  }
}

// ---------------------------------------------------------------- FP32 + FP64 reliable updates
// The single-system FP32 solver of csrc/stencil.cu per segment (three grid
// barriers per iteration, lagged reliable updates with the exact line search,
// quads when nz % 4 == 0).  The CG state of the CTA's system lives in shared
// memory (IRState, updated by thread 0 after each reduction with the
// transitions of stencil_ops.cuh), so the DOF loops keep only alpha/beta and
// two bitmasks in registers.
template <int NC, int NR>
__global__ void __launch_bounds__(kCGThreads, (NC == 1 && NR == 3) ? 3 : 4) cg_batched_ir_kernel(
    const __grid_constant__ BatchArgs a) {
  constexpr int U = NC * NR;
  constexpr int NS = b_systems<NC, NR>();
  __shared__ double s_red[9][kCGWarps];
  __shared__ double s_stage[kStageDoubles];
  __shared__ IRState st[NS];
  __shared__ float s_ab[NS];
  __shared__ int s_mask[3];  // active, need, status
  // the CTA's system record, read once into shared memory (its fields are re-read cheaply there)
  __shared__ BSeg s_seg;
  if (threadIdx.x == 0) s_seg = a.segs[a.cta_seg[blockIdx.x]];
  __syncthreads();
  const BSeg &S = s_seg;
  const int l = blockIdx.x - S.cta0;
  const bool lead = l == 0;
  const Geo g{S.nx, S.ny, S.nz, S.n, S.flags};
  const int64_t n = g.n;
  const double *__restrict__ b = S.b;
  double *x = S.x;
  float *r32 = S.r32, *p32 = S.p32, *q32 = S.q32, *d32 = S.d32;
  const bool use_init = S.use_init_dev && __ldcg(S.use_init_dev) != 0;
  const bool quads = S.quads != 0;  // chunks are multiples of 4 DOFs
  int par = 0;

  // ---- r = b - A64 x, r32 = p32 = r, d = 0; ||b||, ||r||
  double v[2 * NS];
  bool ok = seg_reduce<2 * NS>(a, S, l, true, par, s_red, s_stage, v, [&](int d0, int d1, double (&w)[2 * NS]) {
    for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
      double y[U];
      if (use_init) apply_c<double, NC, NR>(g, a.c64, x, dof, y);
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t i = uidx<NC, NR>(n, dof, u);
        const double bi = b[i];
        const double ri = use_init ? bi - y[u] : bi;
        if (!use_init) x[i] = 0.0;
        r32[i] = (float)ri;
        p32[i] = (float)ri;
        d32[i] = 0.0f;
        const int s = b_sys<NC, NR>(u);
        w[s] = fma(bi, bi, w[s]);
        w[NS + s] = fma(ri, ri, w[NS + s]);
      }
    }
  });
  if (threadIdx.x == 0) {
    int am = 0;
    for (int j = 0; j < NS; ++j) {
      const double bn = ok ? sqrt(v[j]) : 0.0;
      ir_init(st[j], bn, ok ? v[NS + j] : 0.0, S.tol);
      am |= st[j].active << j;
      if (lead) S.info->bnorm[j] = bn;
    }
    if (lead) {
      for (int j = NS; j < 3; ++j) S.info->bnorm[j] = 0.0;
      if (am) atomicAdd(a.live, 1);
    }
    s_mask[0] = am;
    s_mask[1] = 0;
    s_mask[2] = CPM_OK;
  }
  __syncthreads();
  int activem = s_mask[0], needm = 0;
  int status = ok ? CPM_OK : CPM_BARRIER_TIMEOUT;
  if (ok && use_init) {
    for (int cc = l; cc < S.nchunks; cc += S.ncta) {
      const int d1 = min(g.n, (cc + 1) * S.chunk_dofs);
      for (int dof = cc * S.chunk_dofs + threadIdx.x; dof < d1; dof += kCGThreads)
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (!((activem >> b_sys<NC, NR>(u)) & 1)) x[uidx<NC, NR>(n, dof, u)] = b[uidx<NC, NR>(n, dof, u)];
    }
  }
  for (int k = 0; ok; ++k) {
    if (k > 0) {
      if (!grid_sync(a.bar, gridDim.x, a.timeout_ns)) { status = CPM_BARRIER_TIMEOUT; break; }
      // every change of the counter happened before this barrier and none
      // happens before the next one: all CTAs read the same value
      if (__ldcg(a.live) == 0) break;
    }
    const bool busy = activem != 0;  // pending updates belong to active systems
    // ---- q = A32 p, p.q (FP32 per thread); pending updates: t = b - A64 x, r32 = t, t.t, t.p
    double pt[3 * NS];
    if (!seg_reduce<3 * NS>(a, S, l, busy, par, s_red, s_stage, pt, [&](int d0, int d1, double (&w)[3 * NS]) {
          float pqf[NS];
#pragma unroll
          for (int j = 0; j < NS; ++j) pqf[j] = 0.0f;
          if (quads) {
            for (int qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * kCGThreads) {
              float y[4][U];
              apply4_c<float, NC, NR>(g, a.c32, p32, qd, y);
              quad_store<float, NC, NR>(q32, n, qd, y);
              quad_dot<NC, NR>(p32, n, qd, y, pqf);
            }
          } else {
            for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
              float y[U];
              apply_c<float, NC, NR>(g, a.c32, p32, dof, y);
#pragma unroll
              for (int u = 0; u < U; ++u) {
                const int64_t i = uidx<NC, NR>(n, dof, u);
                q32[i] = y[u];
                pqf[b_sys<NC, NR>(u)] = fmaf(p32[i], y[u], pqf[b_sys<NC, NR>(u)]);
              }
            }
          }
#pragma unroll
          for (int j = 0; j < NS; ++j) w[j] += (double)pqf[j];
          if (needm) {
            // d was folded into x by the previous direction phase
            for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
              double yt[U];
              apply_c<double, NC, NR>(g, a.c64, x, dof, yt);
#pragma unroll
              for (int u = 0; u < U; ++u) {
                const int s = b_sys<NC, NR>(u);
                if (!((needm >> s) & 1)) continue;
                const int64_t i = uidx<NC, NR>(n, dof, u);
                const double t = b[i] - yt[u];
                r32[i] = (float)t;
                w[NS + s] = fma(t, t, w[NS + s]);
                w[2 * NS + s] = fma(t, (double)p32[i], w[2 * NS + s]);
              }
            }
          }
        }, needm ? 3 * NS : NS)) {  // t.t and t.p only on an iteration with a pending update
      status = CPM_BARRIER_TIMEOUT;
      break;
    }
    float af[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) af[j] = 0.0f;
    if (busy) {
      if (threadIdx.x == 0) {
        int am = 0, bad = 0;
        for (int j = 0; j < NS; ++j) {
          double al;
          bad |= ir_after_pq(st[j], pt[j], pt[NS + j], pt[2 * NS + j], S.maxiter, al) ? 1 : 0;
          s_ab[j] = (float)al;
          am |= st[j].active << j;
        }
        if (needm) st[0].updates += 1;
        if (bad) {
          for (int j = 0; j < NS; ++j) st[j].active = 0;
          am = 0;
        }
        if (lead && am == 0) atomicSub(a.live, 1);
        s_mask[0] = am;
        s_mask[2] = bad ? CPM_NONFINITE : CPM_OK;
      }
      __syncthreads();
      activem = s_mask[0];
      if (s_mask[2] != CPM_OK) {
        status = s_mask[2];
        needm = 0;
      }
#pragma unroll
      for (int j = 0; j < NS; ++j) af[j] = s_ab[j];
    }
    // ---- active: d += alpha p, r32 -= alpha q, r32.r32
    double rr[NS];
    if (!seg_reduce<NS>(a, S, l, activem != 0, par, s_red, s_stage, rr, [&](int d0, int d1, double (&w)[NS]) {
          float rrf[NS];
#pragma unroll
          for (int j = 0; j < NS; ++j) rrf[j] = 0.0f;
          if (quads) {
            for (int qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * kCGThreads)
              quad_update<NC, NR, NS>(n, qd, activem, af, d32, p32, q32, r32, rrf);
          } else {
            for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
#pragma unroll
              for (int u = 0; u < U; ++u) {
                const int s = b_sys<NC, NR>(u);
                if (!((activem >> s) & 1)) continue;
                const int64_t i = uidx<NC, NR>(n, dof, u);
                d32[i] = fmaf(af[s], p32[i], d32[i]);
                const float rn = fmaf(-af[s], q32[i], r32[i]);
                r32[i] = rn;
                rrf[s] = fmaf(rn, rn, rrf[s]);
              }
            }
          }
#pragma unroll
          for (int j = 0; j < NS; ++j) w[j] = (double)rrf[j];
        })) {
      status = CPM_BARRIER_TIMEOUT;
      break;
    }
    needm = 0;
    if (!activem) continue;
    if (threadIdx.x == 0) {
      int nm = 0, bad = 0;
      for (int j = 0; j < NS; ++j) {
        float be;
        bad |= ir_after_rr(st[j], rr[j], a.inner_tol, S.maxiter, be) ? 1 : 0;
        s_ab[j] = be;
        nm |= st[j].need << j;
      }
      if (bad) {
        for (int j = 0; j < NS; ++j) st[j].active = st[j].need = 0;
        nm = 0;
        if (lead) atomicSub(a.live, 1);
      }
      s_mask[0] = bad ? 0 : activem;
      s_mask[1] = nm;
      s_mask[2] = bad ? CPM_NONFINITE : CPM_OK;
    }
    __syncthreads();
    if (s_mask[2] != CPM_OK) {
      status = s_mask[2];
      activem = 0;
      continue;
    }
    needm = s_mask[1];
    float beta[NS];
#pragma unroll
    for (int j = 0; j < NS; ++j) beta[j] = s_ab[j];
    // ---- p = r32 + beta p; pending updates: x += d, d = 0
    for (int cc = l; cc < S.nchunks; cc += S.ncta) {
      const int d1 = min(g.n, (cc + 1) * S.chunk_dofs);
      if (quads) {
        for (int qd = cc * S.chunk_dofs + 4 * threadIdx.x; qd < d1; qd += 4 * kCGThreads)
          quad_direction<NC, NR, NS>(n, qd, activem, needm, beta, p32, r32, x, d32);
      } else {
        for (int dof = cc * S.chunk_dofs + threadIdx.x; dof < d1; dof += kCGThreads)
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int s = b_sys<NC, NR>(u);
            const int64_t i = uidx<NC, NR>(n, dof, u);
            if ((activem >> s) & 1) p32[i] = fmaf(beta[s], p32[i], r32[i]);
            if ((needm >> s) & 1) {
              x[i] += (double)d32[i];
              d32[i] = 0.0f;
            }
          }
      }
    }
  }
  if (lead && threadIdx.x == 0) {
    int sta = status;
    if (*(volatile const int *)&a.bar->error && sta == CPM_OK) sta = CPM_BARRIER_TIMEOUT;
    for (int j = 0; j < 3; ++j) {
      if (j < NS && sta == CPM_OK && (st[j].unconv || st[j].active)) sta = CPM_NOT_CONVERGED;
      S.info->iters[j] = j < NS ? st[j].iters : 0;
      S.info->resid[j] = j < NS ? st[j].resid : 0.0;
    }
    S.info->outer = st[0].updates;
    S.info->df_updates = 0;
    S.info->status = sta;
  }
}


// ---------------------------------------------------------------- FP32, two grid barriers per iteration
// Opt-in (CPM_CG_FORM_TWO_BARRIER; the single-system form measured slower and,
// at 128^3, stalling on the elastic and demag solves).  The two-barrier
// iteration of csrc/stencil.cu (cg_stencil_ir2_kernel, state transitions in
// IR2State) per segment: phase B forms w = A32 r and the chunk
// partials of r.w (a system in its replacement pass also folds x += d, d = 0),
// then the reduction barrier; phase A updates p, s, d, r (or computes the true
// residual t = b - A64 (x + d) for a replacement pass) and stores the chunk
// partials r.r, r.s, r.p of the new r in the next reduction's records, then the
// barrier before the next product.  A chunk's record holds its 4 NS sums
// (slots: g, r.w, e, f per system), written by the two phases in turn; a
// system's totals add its own chunks in a fixed order, so its iterates do not
// depend on the rest of the batch.
template <int NC, int NR>
__global__ void __launch_bounds__(kCGThreads, (NC == 1 && NR == 3) ? 3 : 4) cg_batched_ir2_kernel(const __grid_constant__ BatchArgs a) {
  constexpr int U = NC * NR;
  constexpr int NS = b_systems<NC, NR>();
  constexpr int NV = 4 * NS;
  __shared__ double s_tot[NV];
  __shared__ double s_w[8][kCGThreads];
  __shared__ double s_stage[kStageDoubles];
  __shared__ IR2State st[NS];
  __shared__ float s_al[NS], s_be[NS];
  __shared__ int s_mask[4];  // update, replacement, active, status
  __shared__ BSeg s_seg;
  if (threadIdx.x == 0) s_seg = a.segs[a.cta_seg[blockIdx.x]];
  __syncthreads();
  const BSeg &S = s_seg;
  const int l = blockIdx.x - S.cta0;
  const bool lead = l == 0;
  const Geo g{S.nx, S.ny, S.nz, S.n, S.flags};
  const int64_t n = g.n;
  const double *__restrict__ b = S.b;
  double *x = S.x;
  float *r32 = S.r32, *p32 = S.p32, *w32 = S.q32, *s32 = S.s32, *d32 = S.d32;
  const bool use_init = S.use_init_dev && __ldcg(S.use_init_dev) != 0;
  const bool quads = S.quads != 0;
  int par = 0;

  // ---- prologue: r = b - A64 x, r32 = r, p = s = d = 0; ||b||^2, ||r||^2 (half 0),
  // and the g slots of the first product's reduction (half 1: g = r.r; e = f = 0)
  double *h0 = a.part, *h1 = a.part + (size_t)a.half;
  chunk_partials<2 * NS>(S, l, h0, s_stage, 2 * NS, [&](int d0, int d1, double (&w)[2 * NS]) {
    for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
      double y[U];
      if (use_init) apply_c<double, NC, NR>(g, a.c64, x, dof, y);
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
        const int sy = b_sys<NC, NR>(u);
        w[sy] = fma(bi, bi, w[sy]);
        w[NS + sy] = fma(ri, ri, w[NS + sy]);
      }
    }
  });
  // the g slots of half 1 repeat the r.r partials (slots NS..2NS of half 0); e and f start at zero
  __syncthreads();
  for (int c = l; c < S.nchunks; c += S.ncta)
    for (int j = threadIdx.x; j < NV; j += kCGThreads) {
      const size_t rec = (size_t)(S.chunk0 + c) * kSlot;
      h1[rec + j] = j < NS ? h0[rec + NS + j] : 0.0;
    }
  bool ok = grid_sync(a.bar, gridDim.x, a.timeout_ns);
  double v[2 * NS];
  if (ok) {
#pragma unroll
    for (int j = 0; j < 2 * NS; ++j) v[j] = 0.0;
    for (int c = threadIdx.x; c < S.nchunks; c += kCGThreads) {
      const double *src = h0 + (size_t)(S.chunk0 + c) * kSlot;
#pragma unroll
      for (int j = 0; j < 2 * NS; ++j) v[j] += __ldcg(src + j);
    }
    block_sum_wide<2 * NS>(v, s_tot, s_w);
  }
  if (threadIdx.x == 0) {
    int am = 0;
    for (int j = 0; j < NS; ++j) {
      const double bn = ok ? sqrt(v[j]) : 0.0;
      ir2_init(st[j], bn, ok ? v[NS + j] : 0.0, S.tol);
      am |= st[j].active << j;
      if (lead) S.info->bnorm[j] = bn;
    }
    if (lead) {
      for (int j = NS; j < 3; ++j) S.info->bnorm[j] = 0.0;
      if (am) atomicAdd(a.live, 1);
    }
    s_mask[2] = am;
  }
  __syncthreads();
  int activem = s_mask[2], repm = 0;
  int status = ok ? CPM_OK : CPM_BARRIER_TIMEOUT;
  if (ok && use_init) {
    for (int cc = l; cc < S.nchunks; cc += S.ncta) {
      const int d1 = min(g.n, (cc + 1) * S.chunk_dofs);
      for (int dof = cc * S.chunk_dofs + threadIdx.x; dof < d1; dof += kCGThreads)
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (!((activem >> b_sys<NC, NR>(u)) & 1)) x[uidx<NC, NR>(n, dof, u)] = b[uidx<NC, NR>(n, dof, u)];
    }
  }
  par = 1;  // the first product's reduction uses half 1
  const int max_pass = 2 * S.maxiter + 8;
  for (int pass = 0; ok; ++pass) {
    // ---- phase B: w = A32 r, r.w; replacement passes fold x += d, d = 0
    double *half = a.part + (size_t)par * (size_t)a.half;
    const bool busy = activem != 0;
    if (busy) {
      chunk_partials<NS>(S, l, half, s_stage, NS, [&](int d0, int d1, double (&w)[NS]) {
        float dlf[NS];
#pragma unroll
        for (int j = 0; j < NS; ++j) dlf[j] = 0.0f;
        if (quads) {
          for (int qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * kCGThreads) {
            float y[4][U];
            apply4_c<float, NC, NR>(g, a.c32, r32, qd, y);
            quad_store<float, NC, NR>(w32, n, qd, y);
            quad_dot<NC, NR>(r32, n, qd, y, dlf);
          }
        } else {
          for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
            float y[U];
            apply_c<float, NC, NR>(g, a.c32, r32, dof, y);
#pragma unroll
            for (int u = 0; u < U; ++u) {
              const int64_t i = uidx<NC, NR>(n, dof, u);
              w32[i] = y[u];
              dlf[b_sys<NC, NR>(u)] = fmaf(r32[i], y[u], dlf[b_sys<NC, NR>(u)]);
            }
          }
        }
        if (repm) {
          for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads)
#pragma unroll
            for (int u = 0; u < U; ++u) {
              if (!((repm >> b_sys<NC, NR>(u)) & 1)) continue;
              const int64_t i = uidx<NC, NR>(n, dof, u);
              x[i] += (double)d32[i];
              d32[i] = 0.0f;
            }
        }
#pragma unroll
        for (int j = 0; j < NS; ++j) w[j] = (double)dlf[j];
      }, [](int j) { return NS + j; });
    }
    if (!grid_sync(a.bar, gridDim.x, a.timeout_ns)) { status = CPM_BARRIER_TIMEOUT; break; }
    int updm = 0;
    if (busy) {
      double t[NV];
#pragma unroll
      for (int j = 0; j < NV; ++j) t[j] = 0.0;
      for (int c = threadIdx.x; c < S.nchunks; c += kCGThreads) {
        const double *src = half + (size_t)(S.chunk0 + c) * kSlot;
#pragma unroll
        for (int j = 0; j < NV; ++j) t[j] += __ldcg(src + j);
      }
      block_sum_wide<NV>(t, s_tot, s_w);
      if (threadIdx.x == 0) {
        int um = 0, rm = 0, am = 0, bad = 0;
        for (int j = 0; j < NS; ++j) {
          float al, be;
          int mode;
          bad |= ir2_after(st[j], t[j], t[NS + j], t[2 * NS + j], t[3 * NS + j], a.inner_tol, S.maxiter, al, be,
                           mode) ? 1 : 0;
          if (!bad && pass + 1 >= max_pass && st[j].active) {
            st[j].active = 0;
            st[j].unconv = 1;
            mode = 0;
          }
          s_al[j] = al;
          s_be[j] = be;
          um |= (mode == 1) << j;
          rm |= (mode == 2) << j;
          am |= st[j].active << j;
        }
        if (bad) {
          for (int j = 0; j < NS; ++j) st[j].active = 0;
          um = rm = am = 0;
        }
        if (lead && am == 0) atomicSub(a.live, 1);
        s_mask[0] = um;
        s_mask[1] = rm;
        s_mask[2] = am;
        s_mask[3] = bad ? CPM_NONFINITE : CPM_OK;
      }
      __syncthreads();
      if (s_mask[3] != CPM_OK) status = s_mask[3];
      updm = s_mask[0];
      repm = s_mask[1];
      activem = s_mask[2];
    }
    par ^= 1;
    // ---- phase A: updates, or the true residual for a replacement pass; partials of the new r
    if (activem) {
      float af[NS], bf[NS];
#pragma unroll
      for (int j = 0; j < NS; ++j) {
        af[j] = s_al[j];
        bf[j] = s_be[j];
      }
      double *next = a.part + (size_t)par * (size_t)a.half;
      chunk_partials<3 * NS>(S, l, next, s_stage, 3 * NS, [&](int d0, int d1, double (&w)[3 * NS]) {
        float gf[NS], ef[NS], ff[NS];
#pragma unroll
        for (int j = 0; j < NS; ++j) gf[j] = ef[j] = ff[j] = 0.0f;
        if (updm) {
          if (quads) {
            for (int qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * kCGThreads)
              quad_update2<NC, NR, NS>(n, qd, updm, af, bf, r32, p32, w32, s32, d32, gf, ef, ff);
          } else {
            for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads)
#pragma unroll
              for (int u = 0; u < U; ++u) {
                const int sy = b_sys<NC, NR>(u);
                if (!((updm >> sy) & 1)) continue;
                update2_one(uidx<NC, NR>(n, dof, u), af[sy], bf[sy], r32, p32, w32, s32, d32, gf[sy], ef[sy],
                            ff[sy]);
              }
          }
        }
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          w[j] = (double)gf[j];
          w[NS + j] = (double)ef[j];
          w[2 * NS + j] = (double)ff[j];
        }
        if (repm) {
          const XPlusD xd{x, d32};
          for (int dof = d0 + threadIdx.x; dof < d1; dof += kCGThreads) {
            double yt[U];
            apply_c<double, NC, NR>(g, a.c64, xd, dof, yt);
#pragma unroll
            for (int u = 0; u < U; ++u) {
              const int sy = b_sys<NC, NR>(u);
              if (!((repm >> sy) & 1)) continue;
              const int64_t i = uidx<NC, NR>(n, dof, u);
              const double tv = b[i] - yt[u];
              r32[i] = (float)tv;
              w[sy] = fma(tv, tv, w[sy]);
              w[NS + sy] = fma(tv, (double)s32[i], w[NS + sy]);
              w[2 * NS + sy] = fma(tv, (double)p32[i], w[2 * NS + sy]);
            }
          }
        }
      }, [](int j) { return j < NS ? j : NS + j; });
    }
    if (!grid_sync(a.bar, gridDim.x, a.timeout_ns)) { status = CPM_BARRIER_TIMEOUT; break; }
    // every change of the counter happened before this barrier and none happens
    // before the next one: all CTAs read the same value
    if (__ldcg(a.live) == 0) break;
  }
  if (lead && threadIdx.x == 0) {
    int sta = status;
    if (*(volatile const int *)&a.bar->error && sta == CPM_OK) sta = CPM_BARRIER_TIMEOUT;
    int upd = 0;
    for (int j = 0; j < 3; ++j) {
      if (j < NS && sta == CPM_OK && (st[j].unconv || st[j].active)) sta = CPM_NOT_CONVERGED;
      S.info->iters[j] = j < NS ? st[j].iters : 0;
      S.info->resid[j] = j < NS ? st[j].resid : 0.0;
      if (j < NS) upd += st[j].updates;
    }
    S.info->outer = upd;
    S.info->df_updates = 0;
    S.info->status = sta;
  }
}

// ---------------------------------------------------------------- host side
// DOFs per chunk of one system: a base size per operator kind, doubled until
// the system has at most kMaxChunks chunks.  It depends on the system alone,
// never on the rest of the batch, so the chunk partials (and every iterate)
// are the same alone and in any mix.
static int chunk_dofs_for(int ncomp, int nrhs, int64_t n) {
  int64_t cd = ncomp == 3 ? 1024 : (nrhs == 3 ? 2048 : 4096);
  while ((n + cd - 1) / cd > kMaxChunks) cd *= 2;
  return (int)cd;
}

// form: CPM_CG_FORM_* of the FP32 solver (the three-barrier form unless the two-barrier one is asked for)
static const void *batched_kernel(int ncomp, int nrhs, int precision, int form) {
  if (precision == 0) {
    if (ncomp == 3) return (const void *)cg_batched_fp64_kernel<3, 1>;
    return nrhs == 3 ? (const void *)cg_batched_fp64_kernel<1, 3> : (const void *)cg_batched_fp64_kernel<1, 1>;
  }
  if (form != CPM_CG_FORM_TWO_BARRIER) {
    if (ncomp == 3) return (const void *)cg_batched_ir_kernel<3, 1>;
    return nrhs == 3 ? (const void *)cg_batched_ir_kernel<1, 3> : (const void *)cg_batched_ir_kernel<1, 1>;
  }
  if (ncomp == 3) return (const void *)cg_batched_ir2_kernel<3, 1>;
  return nrhs == 3 ? (const void *)cg_batched_ir2_kernel<1, 3> : (const void *)cg_batched_ir2_kernel<1, 1>;
}

// FP64 work vectors r, p, q; FP32 r, p, q (w), d and s (the two-barrier form's A p)
constexpr int kWorkVecs64 = 3, kWorkVecs32 = 5;

static size_t vec_bytes(int64_t n, int ncomp, int nrhs, int precision) {
  return align256((size_t)n * ncomp * nrhs * (precision ? 4 : 8));
}

struct PlanLayout {
  size_t bar, part, segs, ctamap, total;
};

static PlanLayout plan_layout(int64_t total_chunks, int nsys, int grid) {
  PlanLayout L;
  L.bar = 0;                       // GridBarrier (16 bytes) then the live counter at +16
  L.part = 256;
  L.segs = L.part + align256(sizeof(double) * 2 * (size_t)total_chunks * kSlot);
  L.ctamap = L.segs + align256(sizeof(BSeg) * (size_t)nsys);
  L.total = L.ctamap + align256(sizeof(int) * (size_t)grid);
  return L;
}

struct Assignment {
  std::vector<int> nchunks, ncta;
  int64_t total_chunks = 0;
  int grid = 0;
};

static int assign(const cpm_batch_system *sys, int nsys, int ncomp, int nrhs, int precision, Assignment &A,
                  const char *who) {
  if (!sys || nsys < 1 || (ncomp != 1 && ncomp != 3) || (nrhs != 1 && nrhs != 3) || (ncomp == 3 && nrhs != 1) ||
      precision < 0 || precision > 1) {
    set_error("%s: bad batch (nsys >= 1, ncomp 1 or 3, nrhs 1 or 3 with ncomp 1, precision 0 or 1)", who);
    return CPM_BAD_ARG;
  }
  A.nchunks.assign(nsys, 0);
  A.total_chunks = 0;
  for (int s = 0; s < nsys; ++s) {
    const cpm_batch_system &y = sys[s];
    const int64_t n = (int64_t)y.nx * y.ny * y.nz;
    if (y.nx < 3 || y.ny < 3 || y.nz < 3 || n * ncomp * nrhs >= ((int64_t)1 << 31) || !y.b || !y.x || !y.info ||
        !y.work || ((uintptr_t)y.work & 255) || y.maxiter < 1 || !(y.tol >= 0.0)) {
      set_error("%s: bad system %d (at least 3 cells per axis, fewer than 2^31 unknowns, b, x, info and a "
                "256-byte aligned work buffer set, maxiter >= 1, tol >= 0)", who, s);
      return CPM_BAD_ARG;
    }
    const int cd = chunk_dofs_for(ncomp, nrhs, n);
    A.nchunks[s] = (int)((n + cd - 1) / cd);
    A.total_chunks += A.nchunks[s];
  }
  // the plan's grid must be resident for every kernel form that may launch it
  int occ = 0;
  CPM_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batched_kernel(ncomp, nrhs, precision, 0), kCGThreads,
                                                        0));
  if (precision) {
    int occ2 = 0;
    CPM_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &occ2, batched_kernel(ncomp, nrhs, precision, CPM_CG_FORM_TWO_BARRIER), kCGThreads, 0));
    occ = std::min(occ, occ2);
  }
  if (occ < 1) {
    set_error("%s: kernel cannot be resident on an SM", who);
    return CPM_CUDA_ERROR;
  }
  // all resident CTAs: a batch's chunk reductions spread over more CTAs (fewer CTAs, as the
  // single-system solver uses for small grids, measured slower for batches)
  int64_t gmax = (int64_t)occ * sm_count();
  if (gmax > kMaxGrid) gmax = kMaxGrid;
  if (nsys > gmax) {
    set_error("%s: %d systems exceed the %lld CTAs that can be resident; split the batch", who, nsys,
              (long long)gmax);
    return CPM_BAD_ARG;
  }
  // equal chunks per CTA: the smallest load whose CTA count fits
  int64_t load = std::max<int64_t>(1, (A.total_chunks + gmax - 1) / gmax);
  for (;; ++load) {
    int64_t g = 0;
    for (int s = 0; s < nsys; ++s) g += (A.nchunks[s] + load - 1) / load;
    if (g <= gmax) break;
  }
  A.ncta.assign(nsys, 0);
  A.grid = 0;
  for (int s = 0; s < nsys; ++s) {
    A.ncta[s] = (int)((A.nchunks[s] + load - 1) / load);
    A.grid += A.ncta[s];
  }
  return CPM_OK;
}

}  // namespace cpm

extern "C" int64_t cpm_batch_work_bytes(int32_t nx, int32_t ny, int32_t nz, int32_t ncomp, int32_t nrhs,
                                        int32_t precision) {
  using namespace cpm;
  if (nx < 1 || ny < 1 || nz < 1 || (ncomp != 1 && ncomp != 3) || (nrhs != 1 && nrhs != 3)) return 0;
  const int64_t n = (int64_t)nx * ny * nz;
  return (int64_t)((precision ? kWorkVecs32 : kWorkVecs64) * vec_bytes(n, ncomp, nrhs, precision));
}

extern "C" int cpm_batch_plan_bytes(const cpm_batch_system *sys, int32_t nsys, int32_t ncomp, int32_t nrhs,
                                    int32_t precision, int64_t *bytes) {
  using namespace cpm;
  Assignment A;
  if (int e = assign(sys, nsys, ncomp, nrhs, precision, A, "cpm_batch_plan_bytes")) return e;
  if (!bytes) {
    set_error("cpm_batch_plan_bytes: bytes is NULL");
    return CPM_BAD_ARG;
  }
  *bytes = (int64_t)plan_layout(A.total_chunks, nsys, A.grid).total;
  return CPM_OK;
}

extern "C" int cpm_batch_plan_build(const cpm_batch_system *sys, int32_t nsys, int32_t ncomp, int32_t nrhs,
                                    int32_t precision, const double *coef, void *plan_dev, int64_t plan_bytes,
                                    cpm_batch_plan *plan, void *stream) {
  using namespace cpm;
  Assignment A;
  if (int e = assign(sys, nsys, ncomp, nrhs, precision, A, "cpm_batch_plan_build")) return e;
  const PlanLayout L = plan_layout(A.total_chunks, nsys, A.grid);
  if (!coef || !plan || !plan_dev || plan_bytes < (int64_t)L.total || ((uintptr_t)plan_dev & 255)) {
    set_error("cpm_batch_plan_build: bad arguments (coef, plan and a 256-byte aligned device buffer of at least "
              "%zu bytes)", L.total);
    return CPM_BAD_ARG;
  }
  std::vector<BSeg> segs(nsys);
  std::vector<int> cmap(A.grid);
  int chunk0 = 0, cta0 = 0;
  for (int s = 0; s < nsys; ++s) {
    const cpm_batch_system &y = sys[s];
    BSeg &S = segs[s];
    S = BSeg{};
    S.nx = y.nx;
    S.ny = y.ny;
    S.nz = y.nz;
    S.n = y.nx * y.ny * y.nz;
    S.flags = y.flags;
    S.b = y.b;
    S.x = y.x;
    S.use_init_dev = y.use_init_dev;
    S.info = y.info;
    S.tol = y.tol;
    S.maxiter = y.maxiter;
    S.chunk0 = chunk0;
    S.nchunks = A.nchunks[s];
    S.cta0 = cta0;
    S.ncta = A.ncta[s];
    S.chunk_dofs = chunk_dofs_for(ncomp, nrhs, S.n);
    // quads need whole quads per z-line, 4-byte aligned flags and an aligned x; other grids take the
    // per-DOF product (scalar-load quads and quads on a padded copy of p measured slower in this kernel)
    S.quads = (y.nz & 3) == 0 && ((uintptr_t)y.flags & 3) == 0 && ((uintptr_t)y.x & 15) == 0;
    const size_t vb = vec_bytes(S.n, ncomp, nrhs, precision);
    char *w = (char *)y.work;
    if (precision == 0) {
      S.r = (double *)w;
      S.p = (double *)(w + vb);
      S.q = (double *)(w + 2 * vb);
    } else {
      S.r32 = (float *)w;
      S.p32 = (float *)(w + vb);
      S.q32 = (float *)(w + 2 * vb);
      S.d32 = (float *)(w + 3 * vb);
      S.s32 = (float *)(w + 4 * vb);
    }
    for (int t = 0; t < S.ncta; ++t) cmap[cta0 + t] = s;
    chunk0 += S.nchunks;
    cta0 += S.ncta;
  }
  cudaStream_t st = (cudaStream_t)stream;
  char *base = (char *)plan_dev;
  CPM_TRY(cudaMemcpyAsync(base + L.segs, segs.data(), sizeof(BSeg) * nsys, cudaMemcpyHostToDevice, st));
  CPM_TRY(cudaMemcpyAsync(base + L.ctamap, cmap.data(), sizeof(int) * A.grid, cudaMemcpyHostToDevice, st));
  CPM_TRY(cudaStreamSynchronize(st));  // the staging vectors go out of scope
  plan->dev = plan_dev;
  plan->bytes = (int64_t)L.total;
  plan->nsys = nsys;
  plan->grid = A.grid;
  plan->ncomp = ncomp;
  plan->nrhs = nrhs;
  plan->precision = precision;
  plan->total_chunks = (int32_t)A.total_chunks;
  const int nc = 27 * ncomp * ncomp;
  for (int i = 0; i < 243; ++i) plan->coef[i] = i < nc ? coef[i] : 0.0;
  return CPM_OK;
}

extern "C" int cpm_cg_solve_blockdiag(const cpm_batch_plan *plan, const cpm_cg_opts *opts, void *stream) {
  using namespace cpm;
  if (!plan || !plan->dev || plan->nsys < 1 || plan->grid < 1 || !opts) {
    set_error("cpm_cg_solve_blockdiag: bad arguments (a built plan and options)");
    return CPM_BAD_ARG;
  }
  const PlanLayout L = plan_layout(plan->total_chunks, plan->nsys, plan->grid);
  char *base = (char *)plan->dev;
  BatchArgs a{};
  for (int i = 0; i < 243; ++i) {
    a.c64[i] = plan->coef[i];
    a.c32[i] = (float)plan->coef[i];
  }
  a.segs = (const BSeg *)(base + L.segs);
  a.cta_seg = (const int *)(base + L.ctamap);
  a.part = (double *)(base + L.part);
  a.half = (long long)plan->total_chunks * kSlot;
  a.bar = (GridBarrier *)(base + L.bar);
  a.live = (int *)(base + L.bar + sizeof(GridBarrier));
  const double tmo = opts->barrier_timeout_s > 0 ? opts->barrier_timeout_s : 2.0;
  a.timeout_ns = (unsigned long long)(tmo * 1e9);
  a.inner_tol = opts->inner_tol > 0 ? opts->inner_tol : 0.1;
  cudaStream_t st = (cudaStream_t)stream;
  CPM_TRY(cudaMemsetAsync(base + L.bar, 0, 32, st));
  void *args[] = {&a};
  CPM_TRY(cudaLaunchCooperativeKernel(batched_kernel(plan->ncomp, plan->nrhs, plan->precision, opts->form),
                                      dim3(plan->grid),
                                      dim3(kCGThreads), args, 0, st));
  return CPM_OK;
}
