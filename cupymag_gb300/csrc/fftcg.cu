// FP32 conjugate gradient preconditioned by the circulant inverse, inside FP64 refinement (sm_103a).
//
// On the periodic hex grid the elastic operator A_el and the demag operator
// A_demag are block-circulant stencils except for the anchor at DOF 0, whose
// rows and columns the reference replaces by the identity
// (cupymag/physics/assemble_demag.py:307-341, assemble_elasticity.py:461-527).
// The 3D DFT diagonalises the circulant part C: per wave vector k a 3x3 (or
// 1x1) real symmetric symbol C^(k) = sum_d c_d cos(theta_k . d).  M = C'^-1,
// with C' = C except C'^(0) = sigma I (sigma the operator's diagonal), is an
// SPD preconditioner with M A = I + (rank <= 9), so preconditioned CG needs a
// few tens of iterations where plain CG needs thousands (2700 for 128^3
// elasticity).
//
// The solve is the refinement form of the cupyx-semantics solve_cg
// (cupymag/solvers/linear_solvers.py:59-74) with the same stopping test on the
// FP64 residual: an outer loop computes t = b - A64 x in FP64, stops when
// ||t|| <= tol ||b||, else runs FP32 preconditioned CG on A e = t from e = 0 until
// its residual has dropped by inner_tol (default 1e-4) and adds e to x.  The
// whole solve is one persistent cooperative launch; every grid barrier is
// bounded (GridBarrier).  Per inner iteration:
//   z = M r: DFT along z, y, then along x with the symbol solve and the
//            inverse DFT along x in the same shared-memory tile, inverse along
//            y and z (five passes over the complex field, with r.z);
//   p = z + beta p; q = A32 p with p.q; d += alpha p, r -= alpha q with r.r.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fft.cuh"
#include "stencil_ops.cuh"

namespace cpm {

constexpr int kFftThreads = 256;
constexpr int kFftTile = 4096;  // complex values per shared-memory tile buffer (two buffers per CTA)

struct FftGrid {
  int nx, ny, nz, n, nc;
  FftAxis ax, ay, az;
  const float *sym;  // inverse symbol per wave vector: nc == 1: 1 float; nc == 3: xx yy zz xy yz xz
  float2 *C;         // complex field, nc * n
  int lz, kty, ktx;  // lines per tile of the z, y and x passes
};

// ---------------------------------------------------------------- the five passes
// z lines of the real input (per component): forward DFT along z into C.
__device__ void pass_z_fwd(const FftGrid &g, const float *r, float2 *s0, float2 *s1) {
  const int nlines = g.nx * g.ny;
  const int per = (nlines + g.lz - 1) / g.lz;
  const int ntiles = g.nc * per;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int c = tile / per, l0 = (tile - c * per) * g.lz;
    const int L = min(g.lz, nlines - l0);
    const float *src = r + (int64_t)c * g.n + (int64_t)l0 * g.nz;
    const int ld = line_stride(g.nz);
    for (int e = threadIdx.x; e < L * g.nz; e += blockDim.x) {
      const int l = e / g.nz, k = e - l * g.nz;
      s0[l * ld + k] = make_float2(src[e], 0.0f);
    }
    __syncthreads();
    const float2 *out = dft_lines(s0, s1, g.az, L, false);
    float2 *dst = g.C + (int64_t)c * g.n + (int64_t)l0 * g.nz;
    for (int e = threadIdx.x; e < L * g.nz; e += blockDim.x) {
      const int l = e / g.nz, k = e - l * g.nz;
      dst[e] = out[l * ld + k];
    }
    __syncthreads();
  }
}

// y lines (tiles of kty consecutive z at fixed x), forward or inverse, in place in C.
__device__ void pass_y(const FftGrid &g, bool inverse, float2 *s0, float2 *s1) {
  const int kb = (g.nz + g.kty - 1) / g.kty;
  const int ntiles = g.nc * g.nx * kb;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int c = tile / (g.nx * kb);
    const int rem = tile - c * g.nx * kb;
    const int i = rem / kb, k0 = (rem - i * kb) * g.kty;
    const int kv = min(g.kty, g.nz - k0);
    float2 *base = g.C + (int64_t)c * g.n + (int64_t)i * g.ny * g.nz + k0;
    const int ld = line_stride(g.ny);
    for (int e = threadIdx.x; e < kv * g.ny; e += blockDim.x) {
      const int j = e / kv, kk = e - j * kv;
      s0[kk * ld + j] = base[(int64_t)j * g.nz + kk];
    }
    __syncthreads();
    const float2 *out = dft_lines(s0, s1, g.ay, kv, inverse);
    for (int e = threadIdx.x; e < kv * g.ny; e += blockDim.x) {
      const int j = e / kv, kk = e - j * kv;
      base[(int64_t)j * g.nz + kk] = out[kk * ld + j];
    }
    __syncthreads();
  }
}

// x lines of every component (tiles of ktx consecutive z at fixed y): forward DFT,
// u^(k) = S^-1(k) r^(k), inverse DFT, all in the tile.
__device__ void pass_x_solve(const FftGrid &g, float2 *s0, float2 *s1) {
  const int kb = (g.nz + g.ktx - 1) / g.ktx;
  const int ntiles = g.ny * kb;
  const int nc = g.nc;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int j = tile / kb, k0 = (tile - j * kb) * g.ktx;
    const int kv = min(g.ktx, g.nz - k0);
    const int lines = nc * kv;
    const int ld = line_stride(g.nx);
    for (int e = threadIdx.x; e < lines * g.nx; e += blockDim.x) {
      const int i = e / lines, lr = e - i * lines;  // lr = c * kv + kk
      const int c = lr / kv, kk = lr - c * kv;
      s0[lr * ld + i] = g.C[(int64_t)c * g.n + ((int64_t)i * g.ny + j) * g.nz + k0 + kk];
    }
    __syncthreads();
    float2 *spec = dft_lines(s0, s1, g.ax, lines, false);
    for (int e = threadIdx.x; e < kv * g.nx; e += blockDim.x) {
      const int i = e / kv, kk = e - i * kv;
      const int64_t kidx = ((int64_t)i * g.ny + j) * g.nz + k0 + kk;
      if (nc == 1) {
        const float w = __ldg(g.sym + kidx);
        float2 &v = spec[kk * ld + i];
        v.x *= w;
        v.y *= w;
      } else {
        const float *m = g.sym + 6 * kidx;
        const float mxx = __ldg(m), myy = __ldg(m + 1), mzz = __ldg(m + 2);
        const float mxy = __ldg(m + 3), myz = __ldg(m + 4), mxz = __ldg(m + 5);
        float2 &a = spec[(0 * kv + kk) * ld + i];
        float2 &b = spec[(1 * kv + kk) * ld + i];
        float2 &d = spec[(2 * kv + kk) * ld + i];
        const float2 va = a, vb = b, vd = d;
        a = make_float2(mxx * va.x + mxy * vb.x + mxz * vd.x, mxx * va.y + mxy * vb.y + mxz * vd.y);
        b = make_float2(mxy * va.x + myy * vb.x + myz * vd.x, mxy * va.y + myy * vb.y + myz * vd.y);
        d = make_float2(mxz * va.x + myz * vb.x + mzz * vd.x, mxz * va.y + myz * vb.y + mzz * vd.y);
      }
    }
    __syncthreads();
    float2 *other = spec == s0 ? s1 : s0;
    const float2 *out = dft_lines(spec, other, g.ax, lines, true);
    for (int e = threadIdx.x; e < lines * g.nx; e += blockDim.x) {
      const int i = e / lines, lr = e - i * lines;
      const int c = lr / kv, kk = lr - c * kv;
      g.C[(int64_t)c * g.n + ((int64_t)i * g.ny + j) * g.nz + k0 + kk] = out[lr * ld + i];
    }
    __syncthreads();
  }
}

// Inverse DFT along z, z_out = Re / n; returns this thread's FP32 partial of r . z_out
// (r may be NULL: no partial).
__device__ float pass_z_inv(const FftGrid &g, float *zout, const float *r, float2 *s0, float2 *s1) {
  const int nlines = g.nx * g.ny;
  const int per = (nlines + g.lz - 1) / g.lz;
  const int ntiles = g.nc * per;
  const float scale = 1.0f / (float)g.n;
  float acc = 0.0f;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int c = tile / per, l0 = (tile - c * per) * g.lz;
    const int L = min(g.lz, nlines - l0);
    const float2 *src = g.C + (int64_t)c * g.n + (int64_t)l0 * g.nz;
    const int ld = line_stride(g.nz);
    for (int e = threadIdx.x; e < L * g.nz; e += blockDim.x) {
      const int l = e / g.nz, k = e - l * g.nz;
      s0[l * ld + k] = src[e];
    }
    __syncthreads();
    const float2 *out = dft_lines(s0, s1, g.az, L, true);
    const int64_t off = (int64_t)c * g.n + (int64_t)l0 * g.nz;
    for (int e = threadIdx.x; e < L * g.nz; e += blockDim.x) {
      const int l = e / g.nz, k = e - l * g.nz;
      const float v = out[l * ld + k].x * scale;
      zout[off + e] = v;
      if (r) acc = fmaf(r[off + e], v, acc);
    }
    __syncthreads();
  }
  return acc;
}

// ---------------------------------------------------------------- the inverse symbol (setup)
struct SymArgs {
  int nx, ny, nz, nc;
  double c[243];
  double sigma;
  const double *cx, *sx, *cy, *sy, *cz, *sz;  // cos / sin of 2 pi i / n per axis (device tables)
  float *sym;
};

__global__ void __launch_bounds__(256) fft_symbol_kernel(const __grid_constant__ SymArgs a) {
  const int64_t n = (int64_t)a.nx * a.ny * a.nz;
  for (int64_t kidx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; kidx < n;
       kidx += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(kidx / ((int64_t)a.ny * a.nz));
    const int rem = (int)(kidx - (int64_t)ix * a.ny * a.nz);
    const int iy = rem / a.nz, iz = rem - iy * a.nz;
    // e^{i theta_a d} for d = -1, 0, 1 per axis
    double ex[3][2], ey[3][2], ez[3][2];
    ex[0][0] = a.cx[ix]; ex[0][1] = -a.sx[ix]; ex[1][0] = 1.0; ex[1][1] = 0.0; ex[2][0] = a.cx[ix]; ex[2][1] = a.sx[ix];
    ey[0][0] = a.cy[iy]; ey[0][1] = -a.sy[iy]; ey[1][0] = 1.0; ey[1][1] = 0.0; ey[2][0] = a.cy[iy]; ey[2][1] = a.sy[iy];
    ez[0][0] = a.cz[iz]; ez[0][1] = -a.sz[iz]; ez[1][0] = 1.0; ez[1][1] = 0.0; ez[2][0] = a.cz[iz]; ez[2][1] = a.sz[iz];
    double S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int dx = 0; dx < 3; ++dx)
      for (int dy = 0; dy < 3; ++dy) {
        const double pr = ex[dx][0] * ey[dy][0] - ex[dx][1] * ey[dy][1];
        const double pi = ex[dx][0] * ey[dy][1] + ex[dx][1] * ey[dy][0];
        for (int dz = 0; dz < 3; ++dz) {
          const double re = pr * ez[dz][0] - pi * ez[dz][1];  // Re e^{i theta . d}
          const int d = (dx * 3 + dy) * 3 + dz;
          for (int p = 0; p < a.nc; ++p)
            for (int q = 0; q < a.nc; ++q) S[p][q] += a.c[(p * a.nc + q) * 27 + d] * re;
        }
      }
    if (kidx == 0) {
      for (int p = 0; p < 3; ++p)
        for (int q = 0; q < 3; ++q) S[p][q] = p == q ? a.sigma : 0.0;
    }
    if (a.nc == 1) {
      a.sym[kidx] = (float)(1.0 / S[0][0]);
    } else {
      // symmetric 3x3 inverse by cofactors (S is symmetric: average the off-diagonal pairs)
      const double xx = S[0][0], yy = S[1][1], zz = S[2][2];
      const double xy = 0.5 * (S[0][1] + S[1][0]), yz = 0.5 * (S[1][2] + S[2][1]), xz = 0.5 * (S[0][2] + S[2][0]);
      const double cxx = yy * zz - yz * yz, cyy = xx * zz - xz * xz, czz = xx * yy - xy * xy;
      const double cxy = xz * yz - xy * zz, cyz = xy * xz - xx * yz, cxz = xy * yz - xz * yy;
      const double det = xx * cxx + xy * cxy + xz * cxz;
      const double id = 1.0 / det;
      float *o = a.sym + 6 * kidx;
      o[0] = (float)(cxx * id);
      o[1] = (float)(cyy * id);
      o[2] = (float)(czz * id);
      o[3] = (float)(cxy * id);
      o[4] = (float)(cyz * id);
      o[5] = (float)(cxz * id);
    }
  }
}

// ---------------------------------------------------------------- plan layout
struct PrecondLayout {
  size_t tw[3], trig[3], sym, total;
};

static PrecondLayout precond_layout(int nx, int ny, int nz, int nc) {
  PrecondLayout L{};
  const int dims[3] = {nx, ny, nz};
  size_t off = 0;
  for (int a = 0; a < 3; ++a) {
    L.tw[a] = off;
    off += align256(sizeof(float2) * dims[a]);
    L.trig[a] = off;
    off += align256(sizeof(double) * 2 * dims[a]);
  }
  L.sym = off;
  off += align256(sizeof(float) * (size_t)nx * ny * nz * (nc == 3 ? 6 : 1));
  L.total = off;
  return L;
}

// Radices of n: 4s, a 2, then 3, 5, 7 and larger primes.
static int radices(int n, int *out) {
  int k = 0, m = n;
  while (m % 4 == 0 && k < kFftMaxPass) { out[k++] = 4; m /= 4; }
  while (m % 2 == 0 && k < kFftMaxPass) { out[k++] = 2; m /= 2; }
  for (int p = 3; m > 1 && k < kFftMaxPass; p += 2)
    while (m % p == 0 && k < kFftMaxPass) { out[k++] = p; m /= p; }
  return m == 1 ? k : -1;
}

static FftAxis axis_of(const cpm_fft_precond *P, int a) {
  FftAxis ax{};
  ax.n = a == 0 ? P->nx : a == 1 ? P->ny : P->nz;
  ax.npass = P->npass[a];
  for (int s = 0; s < kFftMaxPass; ++s) ax.radix[s] = P->radix[a][s];
  const PrecondLayout L = precond_layout(P->nx, P->ny, P->nz, P->ncomp);
  ax.tw = (const float2 *)((const char *)P->dev + L.tw[a]);
  return ax;
}

static FftGrid grid_of(const cpm_fft_precond *P, float2 *C) {
  FftGrid g{};
  g.nx = P->nx;
  g.ny = P->ny;
  g.nz = P->nz;
  g.n = P->nx * P->ny * P->nz;
  g.nc = P->ncomp;
  g.ax = axis_of(P, 0);
  g.ay = axis_of(P, 1);
  g.az = axis_of(P, 2);
  const PrecondLayout L = precond_layout(P->nx, P->ny, P->nz, P->ncomp);
  g.sym = (const float *)((const char *)P->dev + L.sym);
  g.C = C;
  g.lz = std::max(1, kFftTile / line_stride(g.nz));
  g.kty = std::max(1, std::min(g.nz, kFftTile / line_stride(g.ny)));
  g.ktx = std::max(1, std::min(g.nz, kFftTile / (g.nc * line_stride(g.nx))));
  return g;
}

static bool precond_dims_ok(int nx, int ny, int nz, int nc) {
  int r[kFftMaxPass];
  return nx >= 3 && ny >= 3 && nz >= 3 && (nc == 1 || nc == 3) && line_stride(nx) * nc <= kFftTile &&
         line_stride(ny) <= kFftTile && line_stride(nz) <= kFftTile &&
         (int64_t)nx * ny * nz * nc < ((int64_t)1 << 31) && radices(nx, r) >= 0 &&
         radices(ny, r) >= 0 && radices(nz, r) >= 0;
}

// ---------------------------------------------------------------- the preconditioned solve
struct FftCGArgs {
  StencilOp S;
  FftGrid F;
  const double *b;
  double *x;
  double tol;
  int maxiter;
  int use_init_host;
  const int *use_init_dev;
  double inner_tol;
  float *r, *z, *p, *q, *d;
  double *part;
  GridBarrier *bar;
  cpm_cg_info *info;
  unsigned long long timeout_ns;
  int64_t dofs_per_cta;
  int quads;
};

constexpr int kInnerMax = 200;  // iterations of one inner preconditioned solve (a safety bound)

template <int NC>
__global__ void __launch_bounds__(kFftThreads, 2) cg_stencil_fft_kernel(const __grid_constant__ FftCGArgs a) {
  extern __shared__ float2 fsm[];
  float2 *s0 = fsm, *s1 = fsm + kFftTile;
  __shared__ double s_red[3][kCGWarps];
  const int64_t n = a.S.n;
  const int64_t d0 = min(n, (int64_t)blockIdx.x * a.dofs_per_cta);
  const int64_t d1 = min(n, d0 + a.dofs_per_cta);
  const bool use_init = a.use_init_dev ? (__ldcg(a.use_init_dev) != 0) : (a.use_init_host != 0);
  const unsigned long long tns = a.timeout_ns;
  const double *__restrict__ b = a.b;
  double *x = a.x;
  float *r = a.r, *z = a.z, *p = a.p, *q = a.q, *d = a.d;
  int par = 0;

  // ---- ||b||; x = 0 for a cold start
  double v[1] = {0.0};
  for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kFftThreads)
#pragma unroll
    for (int u = 0; u < NC; ++u) {
      const int64_t i = uidx<NC, 1>(n, dof, u);
      const double bi = b[i];
      v[0] = fma(bi, bi, v[0]);
      if (!use_init) x[i] = 0.0;
    }
  if (!grid_sum<1>(v, a.part, par, a.bar, tns, s_red)) {
    set_status(a.info, CPM_BARRIER_TIMEOUT);
    return;
  }
  const double bnorm = sqrt(v[0]);
  const double atol = a.tol * bnorm;
  int status = CPM_OK, iters = 0, outer = 0, conv = 0;
  double resid = 0.0;
  if (bnorm == 0.0) {
    // cupyx cg returns b itself for a zero right-hand side
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kFftThreads)
#pragma unroll
      for (int u = 0; u < NC; ++u) x[uidx<NC, 1>(n, dof, u)] = b[uidx<NC, 1>(n, dof, u)];
    conv = 1;
  }
  while (!conv) {
    // ---- true residual t = b - A64 x (x complete after the last barrier): r = t, d = 0
    double tt[1] = {0.0};
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kFftThreads) {
      double y[NC];
      apply<double, NC, 1>(a.S, x, (int)dof, y);
#pragma unroll
      for (int u = 0; u < NC; ++u) {
        const int64_t i = uidx<NC, 1>(n, dof, u);
        const double t = b[i] - y[u];
        r[i] = (float)t;
        d[i] = 0.0f;
        tt[0] = fma(t, t, tt[0]);
      }
    }
    if (!grid_sum<1>(tt, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
    resid = sqrt(tt[0]);
    if (!isfinite(resid)) { status = CPM_NONFINITE; break; }
    if (resid <= atol) { conv = 1; break; }
    if (iters >= a.maxiter) break;
    outer += 1;
    const double target = fmax(a.inner_tol * resid, 0.5 * atol);
    double rho_old = 0.0;
    for (int it = 0; it < kInnerMax && iters < a.maxiter; ++it) {
      // ---- z = M r
      pass_z_fwd(a.F, r, s0, s1);
      if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
      pass_y(a.F, false, s0, s1);
      if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
      pass_x_solve(a.F, s0, s1);
      if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
      pass_y(a.F, true, s0, s1);
      if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
      double rz[1] = {(double)pass_z_inv(a.F, z, r, s0, s1)};
      if (!grid_sum<1>(rz, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
      const double rho = rz[0];
      const float beta = it == 0 ? 0.0f : (float)(rho / rho_old);
      if (!isfinite(rho) || !isfinite((double)beta)) { status = CPM_NONFINITE; break; }
      rho_old = rho;
      // ---- p = z + beta p
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kFftThreads)
#pragma unroll
        for (int u = 0; u < NC; ++u) {
          const int64_t i = uidx<NC, 1>(n, dof, u);
          p[i] = it == 0 ? z[i] : fmaf(beta, p[i], z[i]);
        }
      if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
      // ---- q = A32 p, p.q
      float pqf[1] = {0.0f};
      if (a.quads) {
        for (int64_t qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * kFftThreads) {
          float y[4][NC];
          apply4_c<float, NC, 1>(a.S, a.S.c32, p, (int)qd, y);
          quad_store<float, NC, 1>(q, n, qd, y);
          quad_dot<NC, 1>(p, n, qd, y, pqf);
        }
      } else {
        for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kFftThreads) {
          float y[NC];
          apply<float, NC, 1>(a.S, p, (int)dof, y);
#pragma unroll
          for (int u = 0; u < NC; ++u) {
            const int64_t i = uidx<NC, 1>(n, dof, u);
            q[i] = y[u];
            pqf[0] = fmaf(p[i], y[u], pqf[0]);
          }
        }
      }
      double pq[1] = {(double)pqf[0]};
      if (!grid_sum<1>(pq, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
      const float alpha = (float)(rho / pq[0]);
      if (!isfinite((double)alpha)) { status = CPM_NONFINITE; break; }
      // ---- d += alpha p, r -= alpha q, r.r
      float rrf = 0.0f;
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kFftThreads)
#pragma unroll
        for (int u = 0; u < NC; ++u) {
          const int64_t i = uidx<NC, 1>(n, dof, u);
          d[i] = fmaf(alpha, p[i], d[i]);
          const float rn = fmaf(-alpha, q[i], r[i]);
          r[i] = rn;
          rrf = fmaf(rn, rn, rrf);
        }
      double rr[1] = {(double)rrf};
      if (!grid_sum<1>(rr, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
      iters += 1;
      if (!isfinite(rr[0])) { status = CPM_NONFINITE; break; }
      if (sqrt(rr[0]) <= target) break;
    }
    if (status != CPM_OK) break;
    // ---- x += d (own unknowns), then a barrier before the next true residual gathers x
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += kFftThreads)
#pragma unroll
      for (int u = 0; u < NC; ++u) {
        const int64_t i = uidx<NC, 1>(n, dof, u);
        x[i] += (double)d[i];
      }
    if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int st = status;
    if (st == CPM_OK && !conv) st = CPM_NOT_CONVERGED;
    a.info->iters[0] = iters;
    a.info->iters[1] = a.info->iters[2] = 0;
    a.info->resid[0] = resid;
    a.info->bnorm[0] = bnorm;
    a.info->outer = outer;
    set_status(a.info, st);
  } else if (status != CPM_OK && threadIdx.x == 0) {
    set_status(a.info, status);
  }
}

// ---------------------------------------------------------------- M r alone (tests)
__global__ void __launch_bounds__(kFftThreads) fft_pass_kernel(const __grid_constant__ FftGrid g, int which,
                                                               const float *r, float *zout) {
  extern __shared__ float2 fsm[];
  float2 *s0 = fsm, *s1 = fsm + kFftTile;
  if (which == 0) pass_z_fwd(g, r, s0, s1);
  else if (which == 1) pass_y(g, false, s0, s1);
  else if (which == 2) pass_x_solve(g, s0, s1);
  else if (which == 3) pass_y(g, true, s0, s1);
  else pass_z_inv(g, zout, nullptr, s0, s1);
}

static int precond_check(const cpm_fft_precond *P, const char *who) {
  if (!P || !P->dev || !precond_dims_ok(P->nx, P->ny, P->nz, P->ncomp)) {
    set_error("%s: bad preconditioner plan", who);
    return CPM_BAD_ARG;
  }
  return CPM_OK;
}

static size_t fft_cg_layout(int64_t n, int nc, char *base, Workspace *w, float2 **C, float **z) {
  size_t off = 0;
  auto take = [&](size_t bytes) -> char * {
    char *ptr = base ? base + off : nullptr;
    off += align256(bytes);
    return ptr;
  };
  Workspace t{};
  t.bar = (GridBarrier *)take(sizeof(GridBarrier));
  t.part = (double *)take(sizeof(double) * 2 * kPartHalf);
  const size_t nv = (size_t)n * nc;
  t.r32 = (float *)take(4 * nv);
  t.pa32 = (float *)take(4 * nv);
  t.q32 = (float *)take(4 * nv);
  t.d32 = (float *)take(4 * nv);
  float *zz = (float *)take(4 * nv);
  float2 *cc = (float2 *)take(8 * nv);
  if (w) *w = t;
  if (C) *C = cc;
  if (z) *z = zz;
  return off;
}

}  // namespace cpm

extern "C" int64_t cpm_fft_precond_bytes(int32_t nx, int32_t ny, int32_t nz, int32_t ncomp) {
  using namespace cpm;
  if (!precond_dims_ok(nx, ny, nz, ncomp)) return 0;
  return (int64_t)precond_layout(nx, ny, nz, ncomp).total;
}

extern "C" int cpm_fft_precond_build(const cpm_stencil *S, void *dev, int64_t bytes, cpm_fft_precond *P,
                                     void *stream) {
  using namespace cpm;
  if (!S || !P || !dev || ((uintptr_t)dev & 255) || !precond_dims_ok(S->nx, S->ny, S->nz, S->ncomp)) {
    set_error("cpm_fft_precond_build: bad arguments (a stencil with at least 3 cells per axis and a 256-byte "
              "aligned device buffer)");
    return CPM_BAD_ARG;
  }
  const PrecondLayout L = precond_layout(S->nx, S->ny, S->nz, S->ncomp);
  if (bytes < (int64_t)L.total) {
    set_error("cpm_fft_precond_build: buffer too small (%lld < %zu bytes)", (long long)bytes, L.total);
    return CPM_BAD_ARG;
  }
  P->nx = S->nx;
  P->ny = S->ny;
  P->nz = S->nz;
  P->ncomp = S->ncomp;
  P->dev = dev;
  P->bytes = (int64_t)L.total;
  cudaStream_t st = (cudaStream_t)stream;
  char *base = (char *)dev;
  const int dims[3] = {S->nx, S->ny, S->nz};
  for (int a = 0; a < 3; ++a) {
    for (int s = 0; s < kFftMaxPass; ++s) P->radix[a][s] = 0;
    P->npass[a] = radices(dims[a], P->radix[a]);
    const int nn = dims[a];
    std::vector<float2> tw(nn);
    std::vector<double> trig(2 * nn);
    for (int t = 0; t < nn; ++t) {
      const double ang = 2.0 * M_PI * (double)t / (double)nn;
      tw[t] = make_float2((float)std::cos(ang), (float)-std::sin(ang));
      trig[t] = std::cos(ang);
      trig[nn + t] = std::sin(ang);
    }
    CPM_TRY(cudaMemcpyAsync(base + L.tw[a], tw.data(), sizeof(float2) * nn, cudaMemcpyHostToDevice, st));
    CPM_TRY(cudaMemcpyAsync(base + L.trig[a], trig.data(), sizeof(double) * 2 * nn, cudaMemcpyHostToDevice, st));
    CPM_TRY(cudaStreamSynchronize(st));  // the host tables go out of scope
  }
  SymArgs s{};
  s.nx = S->nx;
  s.ny = S->ny;
  s.nz = S->nz;
  s.nc = S->ncomp;
  const int nc2 = 27 * S->ncomp * S->ncomp;
  for (int i = 0; i < 243; ++i) s.c[i] = i < nc2 ? S->coef[i] : 0.0;
  // the zero wave vector (the translations, singular in the circulant part) gets the operator's diagonal
  double diag = 0.0;
  for (int c = 0; c < S->ncomp; ++c) diag += S->coef[(c * S->ncomp + c) * 27 + 13];
  s.sigma = diag / S->ncomp;
  const double *trig[3] = {(const double *)(base + L.trig[0]), (const double *)(base + L.trig[1]),
                           (const double *)(base + L.trig[2])};
  s.cx = trig[0];
  s.sx = trig[0] + S->nx;
  s.cy = trig[1];
  s.sy = trig[1] + S->ny;
  s.cz = trig[2];
  s.sz = trig[2] + S->nz;
  s.sym = (float *)(base + L.sym);
  const int64_t n = (int64_t)S->nx * S->ny * S->nz;
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 16));
  fft_symbol_kernel<<<g, 256, 0, st>>>(s);
  return check_launch("cpm_fft_precond_build");
}

extern "C" int cpm_fft_precond_apply(const cpm_fft_precond *P, const float *r, float *z, void *work,
                                     int64_t work_bytes, void *stream) {
  using namespace cpm;
  if (int e = precond_check(P, "cpm_fft_precond_apply")) return e;
  const int64_t n = (int64_t)P->nx * P->ny * P->nz;
  if (!r || !z || !work || work_bytes < (int64_t)(8 * n * P->ncomp) || ((uintptr_t)work & 15)) {
    set_error("cpm_fft_precond_apply: bad vectors or a complex work buffer under %lld bytes",
              (long long)(8 * n * P->ncomp));
    return CPM_BAD_ARG;
  }
  const FftGrid g = grid_of(P, (float2 *)work);
  const size_t smem = 2 * kFftTile * sizeof(float2);
  CPM_TRY(cudaFuncSetAttribute((const void *)fft_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  cudaStream_t st = (cudaStream_t)stream;
  for (int w = 0; w < 5; ++w) {
    fft_pass_kernel<<<sm_count() * 2, kFftThreads, smem, st>>>(g, w, r, z);
    if (int e = check_launch("cpm_fft_precond_apply")) return e;
  }
  return CPM_OK;
}

extern "C" size_t cpm_cg_fft_workspace_bytes(int32_t nx, int32_t ny, int32_t nz, int32_t ncomp) {
  return cpm::fft_cg_layout((int64_t)nx * ny * nz, ncomp, nullptr, nullptr, nullptr, nullptr);
}

extern "C" int cpm_cg_solve_stencil_fft(const cpm_stencil *S, const cpm_fft_precond *P, const double *b, double *x,
                                        const cpm_cg_opts *o, void *workspace, size_t workspace_bytes,
                                        cpm_cg_info *info, void *stream) {
  using namespace cpm;
  if (int e = precond_check(P, "cpm_cg_solve_stencil_fft")) return e;
  if (!S || !b || !x || !o || !workspace || !info || S->nx != P->nx || S->ny != P->ny || S->nz != P->nz ||
      S->ncomp != P->ncomp || ((uintptr_t)workspace & 255)) {
    set_error("cpm_cg_solve_stencil_fft: bad arguments (stencil, plan of the same grid, vectors, options, "
              "256-byte aligned workspace, info)");
    return CPM_BAD_ARG;
  }
  const int nc = S->ncomp;
  const int64_t n = (int64_t)S->nx * S->ny * S->nz;
  const size_t need = fft_cg_layout(n, nc, nullptr, nullptr, nullptr, nullptr);
  if (workspace_bytes < need) {
    set_error("cpm_cg_solve_stencil_fft: workspace too small (%zu < %zu bytes)", workspace_bytes, need);
    return CPM_BAD_ARG;
  }
  Workspace w;
  float2 *C;
  float *zz;
  fft_cg_layout(n, nc, (char *)workspace, &w, &C, &zz);
  FftCGArgs a{};
  a.S.nx = S->nx;
  a.S.ny = S->ny;
  a.S.nz = S->nz;
  a.S.n = (int)n;
  a.S.flags = S->flags;
  const int ncoef = 27 * nc * nc;
  for (int i = 0; i < 243; ++i) {
    a.S.c64[i] = i < ncoef ? S->coef[i] : 0.0;
    a.S.c32[i] = (float)a.S.c64[i];
  }
  a.F = grid_of(P, C);
  a.b = b;
  a.x = x;
  a.tol = o->tol;
  a.maxiter = o->maxiter;
  a.use_init_host = o->use_init_host;
  a.use_init_dev = o->use_init_dev;
  a.inner_tol = o->inner_tol > 0 ? o->inner_tol : 1e-4;
  a.r = w.r32;
  a.p = w.pa32;
  a.q = w.q32;
  a.d = w.d32;
  a.z = zz;
  a.part = w.part;
  a.bar = w.bar;
  a.info = info;
  const double tmo = o->barrier_timeout_s > 0 ? o->barrier_timeout_s : 2.0;
  a.timeout_ns = (unsigned long long)(tmo * 1e9);
  a.quads = (S->nz & 3) == 0 && ((uintptr_t)S->flags & 3) == 0;
  const void *fn = nc == 3 ? (const void *)cg_stencil_fft_kernel<3> : (const void *)cg_stencil_fft_kernel<1>;
  const size_t smem = 2 * kFftTile * sizeof(float2);
  CPM_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  CPM_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kFftThreads, smem));
  if (occ < 1) {
    set_error("cpm_cg_solve_stencil_fft: kernel cannot be resident on an SM");
    return CPM_CUDA_ERROR;
  }
  int64_t G = std::min<int64_t>((int64_t)occ * sm_count(), kMaxGrid);
  int64_t per = (n + G - 1) / G;
  per = (per + 31) / 32 * 32;
  G = std::max<int64_t>(1, (n + per - 1) / per);
  a.dofs_per_cta = per;
  CPM_TRY(cudaMemsetAsync(w.bar, 0, sizeof(GridBarrier), (cudaStream_t)stream));
  CPM_TRY(cudaMemsetAsync(info, 0, sizeof(cpm_cg_info), (cudaStream_t)stream));
  void *args[] = {&a};
  CPM_TRY(cudaLaunchCooperativeKernel(fn, dim3((unsigned)G), dim3(kFftThreads), args, smem, (cudaStream_t)stream));
  return CPM_OK;
}
