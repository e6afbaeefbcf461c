// Element-wise and reduction kernels of the GSPM LLG step (sm_103a).
//
// Restates, per DOF, the array expressions of cupymag/core/Micromagnetics.py
// and the helpers it calls.  This file is compiled with FMA contraction off
// (-fmad=false): the reference evaluates each `a * b + c` as two separately
// rounded array operations, and keeping the same association order and the
// same roundings makes these kernels agree with it to the last bit wherever
// the inputs agree.
//
// Reductions (volume averages, sumsq) are deterministic: a fixed grid for a
// given n and GPU, fixed-order block trees, and the last CTA to finish sums the
// per-CTA partials in CTA order.
#include "cpm_common.cuh"
#include "csr_tile.cuh"

namespace cpm {

constexpr int kEwThreads = 256;
constexpr int kRedMaxGrid = 1024;
constexpr int kRedSlots = 8;  // values per CTA in the partials area

static int ew_grid(int64_t n) {
  int64_t g = (n + kEwThreads - 1) / kEwThreads;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

static int red_grid(int64_t n) {
  int64_t g = (n + 4 * kEwThreads - 1) / (4 * kEwThreads);
  int64_t cap = (int64_t)sm_count() * 2;
  if (cap > kRedMaxGrid) cap = kRedMaxGrid;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

// Sum NV values over the CTA; result valid in every thread.
template <int NV>
__device__ __forceinline__ void cta_sum(double (&v)[NV]) {
  __shared__ double s[NV][kEwThreads / kWarp];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    const double t = warp_sum(v[j]);
    if (lane == 0) s[j][w] = t;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < kEwThreads / kWarp; ++k) t += s[j][k];
    v[j] = t;
  }
  __syncthreads();
}

// Publish this CTA's partials; returns true in the CTA that finishes last,
// with the grid totals in v.  scratch[0] is the ticket counter (reset by the
// last CTA), partials start at scratch + 8.
template <int NV>
__device__ __forceinline__ bool grid_total(double (&v)[NV], double *scratch) {
  __shared__ int s_last;
  cta_sum<NV>(v);
  double *part = scratch + 8;
  if (threadIdx.x < NV) part[(size_t)blockIdx.x * kRedSlots + threadIdx.x] = v[threadIdx.x];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int *ctr = reinterpret_cast<unsigned int *>(scratch);
    const unsigned int t = atomicAdd(ctr, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  double acc[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) acc[j] = 0.0;
  for (int g = threadIdx.x; g < (int)gridDim.x; g += blockDim.x) {
#pragma unroll
    for (int j = 0; j < NV; ++j) acc[j] += __ldcg(&part[(size_t)g * kRedSlots + j]);
  }
  cta_sum<NV>(acc);
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j] = acc[j];
  if (threadIdx.x == 0) *reinterpret_cast<unsigned int *>(scratch) = 0u;
  return true;
}

// ------------------------------------------------------------ volume average
// <f>_c = (sum_i w_i f_ic) / V, optionally of f R (3 components, row-major R),
// volume_average.py:155-216 with the per-element quadrature folded into w.
template <int NC, bool ROT>
__global__ void __launch_bounds__(kEwThreads) volavg_kernel(int64_t n, const double *__restrict__ f,
                                                            const double *__restrict__ w, const double *R9,
                                                            double volume, double *out, double *scratch) {
  double acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = 0.0;
  double R[9];
  if (ROT) {
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = R9[k];
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double wi = w[i];
    if (ROT) {
      const double m0 = f[3 * i], m1 = f[3 * i + 1], m2 = f[3 * i + 2];
#pragma unroll
      for (int c = 0; c < 3; ++c) acc[c] += wi * (m0 * R[c] + m1 * R[3 + c] + m2 * R[6 + c]);
    } else {
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[c] += wi * f[i * NC + c];
    }
  }
  if (grid_total<NC>(acc, scratch) && threadIdx.x < NC) out[threadIdx.x] = acc[threadIdx.x] / volume;
}

// ------------------------------------------------------------ effective field
struct FieldP {
  double K1, C1, C2, C3, lam;
  double Nd[3], Hext[3], R[9];
  int rot, hasE;
  const double *hsched;  // device field schedule (steps x 3) or NULL
  const int *hstep;      // device index into hsched
};

__global__ void __launch_bounds__(kEwThreads) field_kernel(FieldP P, int64_t n, const double *__restrict__ mm,
                                                           const double *__restrict__ E,
                                                           const double *__restrict__ Ht,
                                                           const double *__restrict__ avg_m, double dt,
                                                           double *__restrict__ fout, double *__restrict__ t) {
  const double hb0 = 0.5 * (-P.Nd[0] * avg_m[0]);
  const double hb1 = 0.5 * (-P.Nd[1] * avg_m[1]);
  const double hb2 = 0.5 * (-P.Nd[2] * avg_m[2]);
  const double k2 = -2.0 * P.K1, c1 = 2.0 * P.C1, c2 = 2.0 * P.C2, c3 = P.C3;
  double H0 = P.Hext[0], H1 = P.Hext[1], H2 = P.Hext[2];
  if (P.hsched) {
    const int64_t s = *P.hstep;
    H0 = P.hsched[3 * s];
    H1 = P.hsched[3 * s + 1];
    H2 = P.hsched[3 * s + 2];
  }
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x0 = mm[3 * i], x1 = mm[3 * i + 1], x2 = mm[3 * i + 2];
    double e0 = 0, e1 = 0, e2 = 0, e3 = 0, e4 = 0, e5 = 0;
    if (P.hasE) {
      e0 = E[6 * i];
      e1 = E[6 * i + 1];
      e2 = E[6 * i + 2];
      e3 = E[6 * i + 3];
      e4 = E[6 * i + 4];
      e5 = E[6 * i + 5];
    }
    const double h0 = 0.5 * Ht[3 * i], h1 = 0.5 * Ht[3 * i + 1], h2 = 0.5 * Ht[3 * i + 2];
    double f0, f1, f2;
    if (!P.rot) {
      const double s0 = x0 * x0, s1 = x1 * x1, s2 = x2 * x2;
      const double o0 = s1 + s2, o1 = s2 + s0, o2 = s0 + s1;
      f0 = (((k2 * x0) * o0 + hb0) + h0) + H0;
      f1 = (((k2 * x1) * o1 + hb1) + h1) + H1;
      f2 = (((k2 * x2) * o2 + hb2) + h2) + H2;
      if (P.hasE) {
        f0 = ((f0 - (c1 * x0) * o0) - (c2 * (e0 - P.lam)) * x0) - c3 * (e3 * x1 + e5 * x2);
        f1 = ((f1 - (c1 * x1) * o1) - (c2 * (e1 - P.lam)) * x1) - c3 * (e4 * x2 + e3 * x0);
        f2 = ((f2 - (c1 * x2) * o2) - (c2 * (e2 - P.lam)) * x2) - c3 * (e5 * x0 + e4 * x1);
      }
    } else {
      const double *R = P.R;
      // m100 = m R
      const double y0 = (x0 * R[0] + x1 * R[3]) + x2 * R[6];
      const double y1 = (x0 * R[1] + x1 * R[4]) + x2 * R[7];
      const double y2 = (x0 * R[2] + x1 * R[5]) + x2 * R[8];
      const double s0 = y0 * y0, s1 = y1 * y1, s2 = y2 * y2;
      const double o0 = s1 + s2, o1 = s2 + s0, o2 = s0 + s1;
      double v0 = (k2 * y0) * o0, v1 = (k2 * y1) * o1, v2 = (k2 * y2) * o2;
      if (P.hasE) {
        v0 = ((v0 - (c1 * y0) * o0) - (c2 * (e0 - P.lam)) * y0) - c3 * (e3 * y1 + e5 * y2);
        v1 = ((v1 - (c1 * y1) * o1) - (c2 * (e1 - P.lam)) * y1) - c3 * (e4 * y2 + e3 * y0);
        v2 = ((v2 - (c1 * y2) * o2) - (c2 * (e2 - P.lam)) * y2) - c3 * (e5 * y0 + e4 * y1);
      }
      // v R^T
      const double w0 = (v0 * R[0] + v1 * R[1]) + v2 * R[2];
      const double w1 = (v0 * R[3] + v1 * R[4]) + v2 * R[5];
      const double w2 = (v0 * R[6] + v1 * R[7]) + v2 * R[8];
      f0 = ((w0 + hb0) + h0) + H0;
      f1 = ((w1 + hb1) + h1) + H1;
      f2 = ((w2 + hb2) + h2) + H2;
    }
    if (fout) {
      fout[3 * i] = f0;
      fout[3 * i + 1] = f1;
      fout[3 * i + 2] = f2;
    }
    t[3 * i] = f0 * dt + x0;
    t[3 * i + 1] = f1 * dt + x1;
    t[3 * i + 2] = f2 * dt + x2;
  }
}

// ------------------------------------------------------------ GS star chain
__global__ void __launch_bounds__(kEwThreads) gs_star_kernel(int stage, int64_t n, const double *__restrict__ m,
                                                             const double *__restrict__ g,
                                                             const double *__restrict__ g1s,
                                                             const double *__restrict__ g2s,
                                                             const double *__restrict__ f, double dt,
                                                             double *__restrict__ mstar, double *__restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (stage == 1) {
      // m1* = m1 + g2n m3 - g3n m2   (Micromagnetics.py:225-226)
      const double ms = (m[3 * i] + g[3 * i + 1] * m[3 * i + 2]) - g[3 * i + 2] * m[3 * i + 1];
      mstar[3 * i] = ms;
      out[i] = f[3 * i] * dt + ms;
    } else if (stage == 2) {
      // m2* = m2 + g3n m1* - g1* m3   (:231-232)
      const double ms = (m[3 * i + 1] + g[3 * i + 2] * mstar[3 * i]) - g1s[i] * m[3 * i + 2];
      mstar[3 * i + 1] = ms;
      out[i] = f[3 * i + 1] * dt + ms;
    } else {
      // m3* = m3 + g1* m2* - g2* m1*  (:237)
      mstar[3 * i + 2] = (m[3 * i + 2] + g1s[i] * mstar[3 * i + 1]) - g2s[i] * mstar[3 * i];
    }
  }
}

// ------------------------------------------------------------ renormalise
// Micromagnetics.py:292-307: m = mss/|mss| (0 below 1e-14), defect rows 0,
// sumsq = sum (m - m_prev)^2, m_prev = m, use_init = sumsq < thresh, <m>.
__global__ void __launch_bounds__(kEwThreads) renorm_kernel(int64_t n, const double *__restrict__ mss,
                                                            const uint8_t *__restrict__ defect,
                                                            double *__restrict__ m, double *__restrict__ m_prev,
                                                            const double *__restrict__ w, double volume,
                                                            double thresh, double *sumsq_out, double *avg_out,
                                                            int *use_init, double *scratch) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double a0 = mss[3 * i], a1 = mss[3 * i + 1], a2 = mss[3 * i + 2];
    const double mag = sqrt((a0 * a0 + a1 * a1) + a2 * a2);
    double n0 = 0.0, n1 = 0.0, n2 = 0.0;
    if (!(fabs(mag) < 1e-14) && !(defect && defect[i])) {
      n0 = a0 / mag;
      n1 = a1 / mag;
      n2 = a2 / mag;
    }
    const double d0 = n0 - m_prev[3 * i], d1 = n1 - m_prev[3 * i + 1], d2 = n2 - m_prev[3 * i + 2];
    acc[0] += (d0 * d0 + d1 * d1) + d2 * d2;
    m[3 * i] = n0;
    m[3 * i + 1] = n1;
    m[3 * i + 2] = n2;
    m_prev[3 * i] = n0;
    m_prev[3 * i + 1] = n1;
    m_prev[3 * i + 2] = n2;
    const double wi = w[i];
    acc[1] += wi * n0;
    acc[2] += wi * n1;
    acc[3] += wi * n2;
  }
  if (grid_total<4>(acc, scratch) && threadIdx.x == 0) {
    *sumsq_out = acc[0];
    avg_out[0] = acc[1] / volume;
    avg_out[1] = acc[2] / volume;
    avg_out[2] = acc[3] / volume;
    if (use_init) *use_init = acc[0] < thresh ? 1 : 0;
  }
}

// ------------------------------------------------------------ eigenstrain
// final_assembly.py:208-266; with rotation, E0 is built from m100 = m R and
// then rotated per node by M^T (Micromagnetics.py:112-119).
__global__ void __launch_bounds__(kEwThreads) e0_kernel(int64_t n, const double *__restrict__ m, double l100,
                                                        double l111, const double *R9, const double *M36,
                                                        double *__restrict__ E0) {
  const double a = 1.5 * l100, b = 1.5 * l111, third = 1.0 / 3.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double x = m[3 * i], y = m[3 * i + 1], z = m[3 * i + 2];
    if (R9) {
      const double y0 = (x * R9[0] + y * R9[3]) + z * R9[6];
      const double y1 = (x * R9[1] + y * R9[4]) + z * R9[7];
      const double y2 = (x * R9[2] + y * R9[5]) + z * R9[8];
      x = y0;
      y = y1;
      z = y2;
    }
    double e[6];
    e[0] = a * (x * x - third);
    e[1] = a * (y * y - third);
    e[2] = a * (z * z - third);
    e[3] = 2.0 * (b * (x * y));
    e[4] = 2.0 * (b * (y * z));
    e[5] = 2.0 * (b * (x * z));
    if (M36) {
#pragma unroll
      for (int r = 0; r < 6; ++r) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) s += e[k] * M36[6 * r + k];
        E0[6 * i + r] = s;
      }
    } else {
#pragma unroll
      for (int r = 0; r < 6; ++r) E0[6 * i + r] = e[r];
    }
  }
}

// ------------------------------------------------------------ strain from u
// compute_derivatives.py:60-125: nine products D_a u_b from the shared-pattern
// matrices (Fx, Fy, Fz), combined into Voigt strain (optionally rotated by R).
// Staged tiles, G threads per row, nine FP64 FMAs per non-zero.
constexpr int kStrainThreads = 256;

template <typename IT>
__global__ void __launch_bounds__(kStrainThreads) strain_kernel(int64_t n, const IT *__restrict__ rp,
                                                                const int *__restrict__ ci,
                                                                const double *__restrict__ ax,
                                                                const double *__restrict__ ay,
                                                                const double *__restrict__ az,
                                                                const double *__restrict__ u, const double *R9,
                                                                double *__restrict__ E, int G) {
  extern __shared__ __align__(16) unsigned char smem[];
  const MultiTile<3> t = multi_tile_smem<3>(smem);
  const int R = kStrainThreads / G;
  const double *vals[3] = {ax, ay, az};
  const int64_t ntiles = (n + R - 1) / R;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t t0 = tile * R, t1 = min(n, t0 + R);
    double d[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // d[a][b] = (D_a u_b)_row
    const int64_t row = visit_tile<3, IT>(rp, ci, vals, t0, t1, G, t, [&](const double (&v)[3], int64_t c) {
      const double uu[3] = {__ldg(u + c), __ldg(u + n + c), __ldg(u + 2 * n + c)};
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) d[a][b] = __fma_rn(v[a], uu[b], d[a][b]);
    });
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) d[a][b] = group_sum(d[a][b], G);
    if (row >= 0 && (threadIdx.x % G) == 0) {
      double out[6];
      if (!R9) {
        out[0] = d[0][0];
        out[1] = d[1][1];
        out[2] = d[2][2];
        out[3] = d[1][0] + d[0][1];
        out[4] = d[2][1] + d[1][2];
        out[5] = d[2][0] + d[0][2];
      } else {
        const double *R = R9;  // R[r][c] = R9[3r+c]
        const double dxx = d[0][0], dyx = d[1][0], dzx = d[2][0];
        const double dxy = d[0][1], dyy = d[1][1], dzy = d[2][1];
        const double dxz = d[0][2], dyz = d[1][2], dzz = d[2][2];
        out[0] = (R[0] * dxx + R[3] * dyx) + R[6] * dzx;
        out[1] = (R[1] * dxy + R[4] * dyy) + R[7] * dzy;
        out[2] = (R[2] * dxz + R[5] * dyz) + R[8] * dzz;
        out[3] = ((R[1] * dxx + R[4] * dyx) + R[7] * dzx) + ((R[0] * dxy + R[3] * dyy) + R[6] * dzy);
        out[4] = ((R[2] * dxy + R[5] * dyy) + R[8] * dzy) + ((R[1] * dxz + R[4] * dyz) + R[7] * dzz);
        out[5] = ((R[2] * dxx + R[5] * dyx) + R[8] * dzx) + ((R[0] * dxz + R[3] * dyz) + R[6] * dzz);
      }
#pragma unroll
      for (int c = 0; c < 6; ++c) E[6 * row + c] = out[c];
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ strain finalize
// Micromagnetics.py:132-162: E -= <E>; E += E_bar; E = E M^{-T} (rot111).
__global__ void __launch_bounds__(kEwThreads) strain_fin_kernel(int64_t n, double *__restrict__ E,
                                                                const double *avgE, const double *am,
                                                                double l100, double l111, const double *Es,
                                                                const double *M36, const double *MinvT36,
                                                                int rot) {
  __shared__ double sEb[6], sAvg[6], sMi[36];
  if (threadIdx.x == 0) {
    const double a0 = am[0], a1 = am[1], a2 = am[2];
    double eb[6];
    eb[0] = (1.5 * l100) * (a0 * a0 - 1.0 / 3.0) + Es[0];
    eb[1] = (1.5 * l100) * (a1 * a1 - 1.0 / 3.0) + Es[1];
    eb[2] = (1.5 * l100) * (a2 * a2 - 1.0 / 3.0) + Es[2];
    eb[3] = ((3.0 * l111) * a0) * a1 + Es[3];
    eb[4] = ((3.0 * l111) * a1) * a2 + Es[4];
    eb[5] = ((3.0 * l111) * a0) * a2 + Es[5];
    for (int r = 0; r < 6; ++r) {
      if (rot) {
        double s = 0.0;
        for (int k = 0; k < 6; ++k) s += M36[6 * r + k] * eb[k];
        sEb[r] = s;
      } else {
        sEb[r] = eb[r];
      }
      sAvg[r] = avgE[r];
    }
  }
  if (rot && threadIdx.x < 36) sMi[threadIdx.x] = MinvT36[threadIdx.x];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double e[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) e[c] = (E[6 * i + c] - sAvg[c]) + sEb[c];
    if (rot) {
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) s += e[k] * sMi[6 * k + c];
        E[6 * i + c] = s;
      }
    } else {
#pragma unroll
      for (int c = 0; c < 6; ++c) E[6 * i + c] = e[c];
    }
  }
}

}  // namespace cpm

// ============================================================== C-ABI
using namespace cpm;

extern "C" size_t cpm_volavg_scratch_doubles(int ncomp) {
  (void)ncomp;
  return 8 + (size_t)kRedMaxGrid * kRedSlots;
}

extern "C" int cpm_volavg(int64_t n, int ncomp, const double *f, const double *w, double volume, const double *R9,
                          double *out, double *scratch, void *stream) {
  if (!f || !w || !out || !scratch || n <= 0 || !(ncomp == 1 || ncomp == 3 || ncomp == 6) ||
      (R9 && ncomp != 3)) {
    set_error("cpm_volavg: bad arguments");
    return CPM_BAD_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int g = red_grid(n);
  if (R9)
    volavg_kernel<3, true><<<g, kEwThreads, 0, st>>>(n, f, w, R9, volume, out, scratch);
  else if (ncomp == 1)
    volavg_kernel<1, false><<<g, kEwThreads, 0, st>>>(n, f, w, nullptr, volume, out, scratch);
  else if (ncomp == 3)
    volavg_kernel<3, false><<<g, kEwThreads, 0, st>>>(n, f, w, nullptr, volume, out, scratch);
  else
    volavg_kernel<6, false><<<g, kEwThreads, 0, st>>>(n, f, w, nullptr, volume, out, scratch);
  return check_launch("cpm_volavg");
}

extern "C" int cpm_llg_field(const cpm_field_params *P, int64_t n, const double *mm, const double *E,
                             const double *Ht, const double *avg_m, double dt, double *f, double *t, void *stream) {
  if (!P || !mm || !Ht || !avg_m || !t || (P->has_E && !E)) {
    set_error("cpm_llg_field: bad arguments");
    return CPM_BAD_ARG;
  }
  if (n <= 0) return CPM_OK;
  FieldP q;
  q.K1 = P->K1;
  q.C1 = P->elasC1;
  q.C2 = P->elasC2;
  q.C3 = P->elasC3;
  q.lam = P->lambda100;
  for (int k = 0; k < 3; ++k) {
    q.Nd[k] = P->Nd[k];
    q.Hext[k] = P->Hext[k];
  }
  for (int k = 0; k < 9; ++k) q.R[k] = P->R[k];
  q.rot = P->rot111;
  q.hasE = P->has_E;
  q.hsched = P->hext_sched;
  q.hstep = P->hext_step;
  if (q.hsched && !q.hstep) {
    set_error("cpm_llg_field: hext_sched without hext_step");
    return CPM_BAD_ARG;
  }
  field_kernel<<<ew_grid(n), kEwThreads, 0, (cudaStream_t)stream>>>(q, n, mm, E, Ht, avg_m, dt, f, t);
  return check_launch("cpm_llg_field");
}

// ------------------------------------------------------------ per-step record
__global__ void record_step_kernel(const double *avg_m, const double *sumsq, double *hist, int *step, int cap) {
  const int s = *step;
  if (s < cap) {
    hist[4 * s] = avg_m[0];
    hist[4 * s + 1] = avg_m[1];
    hist[4 * s + 2] = avg_m[2];
    hist[4 * s + 3] = *sumsq;
    *step = s + 1;
  }
}

extern "C" int cpm_record_step(const double *avg_m, const double *sumsq, double *hist, int32_t *step_dev,
                               int32_t capacity, void *stream) {
  if (!avg_m || !sumsq || !hist || !step_dev || capacity < 1) {
    set_error("cpm_record_step: bad arguments");
    return CPM_BAD_ARG;
  }
  record_step_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(avg_m, sumsq, hist, step_dev, capacity);
  return check_launch("cpm_record_step");
}

extern "C" int cpm_gs_star(int stage, int64_t n, const double *m, const double *g, const double *g1s,
                           const double *g2s, const double *f, double dt, double *mstar, double *out,
                           void *stream) {
  if (stage < 1 || stage > 3 || !m || !mstar || (stage < 3 && (!f || !out)) || (stage >= 1 && !g) ||
      (stage >= 2 && !g1s) || (stage == 3 && !g2s)) {
    set_error("cpm_gs_star: bad arguments");
    return CPM_BAD_ARG;
  }
  if (n <= 0) return CPM_OK;
  gs_star_kernel<<<ew_grid(n), kEwThreads, 0, (cudaStream_t)stream>>>(stage, n, m, g, g1s, g2s, f, dt, mstar, out);
  return check_launch("cpm_gs_star");
}

extern "C" int cpm_renorm_sumsq(int64_t n, const double *mss, const uint8_t *defect_mask, double *m,
                                double *m_prev, const double *w, double volume, double thresh, double *sumsq_out,
                                double *avg_out, int32_t *use_init_dev, double *scratch, void *stream) {
  if (!mss || !m || !m_prev || !w || !sumsq_out || !avg_out || !scratch || n <= 0) {
    set_error("cpm_renorm_sumsq: bad arguments");
    return CPM_BAD_ARG;
  }
  renorm_kernel<<<red_grid(n), kEwThreads, 0, (cudaStream_t)stream>>>(n, mss, defect_mask, m, m_prev, w, volume,
                                                                      thresh, sumsq_out, avg_out, use_init_dev,
                                                                      scratch);
  return check_launch("cpm_renorm_sumsq");
}

extern "C" int cpm_build_E0(int64_t n, const double *m, double lam100, double lam111, const double *R9,
                            const double *M36, double *E0, void *stream) {
  if (!m || !E0 || (R9 == nullptr) != (M36 == nullptr)) {
    set_error("cpm_build_E0: bad arguments (R and M go together)");
    return CPM_BAD_ARG;
  }
  if (n <= 0) return CPM_OK;
  e0_kernel<<<ew_grid(n), kEwThreads, 0, (cudaStream_t)stream>>>(n, m, lam100, lam111, R9, M36, E0);
  return check_launch("cpm_build_E0");
}

extern "C" int cpm_strain_from_u(const cpm_csr *Fx, const double *vals_y, const double *vals_z, const double *u,
                                 const double *R9, double *E, void *stream) {
  if (!Fx || !Fx->indptr || !Fx->indices || !Fx->vals || !vals_y || !vals_z || !u || !E || Fx->rows != Fx->cols) {
    set_error("cpm_strain_from_u: bad arguments");
    return CPM_BAD_ARG;
  }
  const int64_t n = Fx->rows;
  if (n <= 0) return CPM_OK;
  const int64_t mr = Fx->max_row_nnz > 0 ? Fx->max_row_nnz : (Fx->nnz + n - 1) / n;
  const int G = group_size_cap(mr, kStrainThreads, multi_cap<3>());
  const int64_t tiles = (n + kStrainThreads / G - 1) / (kStrainThreads / G);
  cudaStream_t st = (cudaStream_t)stream;
  const void *fn = Fx->indptr_is64 ? (const void *)strain_kernel<int64_t> : (const void *)strain_kernel<int32_t>;
  // the shared-memory attribute is per device: set it (cheaply) on every call, then query the occupancy
  int occ = 0;
  CPM_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, multi_smem<3>()));
  CPM_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kStrainThreads, multi_smem<3>()));
  if (occ < 1) occ = 1;
  int64_t g = (int64_t)occ * sm_count();
  if (g > tiles) g = tiles;
  if (Fx->indptr_is64)
    strain_kernel<int64_t><<<(int)g, kStrainThreads, multi_smem<3>(), st>>>(
        n, (const int64_t *)Fx->indptr, Fx->indices, Fx->vals, vals_y, vals_z, u, R9, E, G);
  else
    strain_kernel<int32_t><<<(int)g, kStrainThreads, multi_smem<3>(), st>>>(
        n, (const int32_t *)Fx->indptr, Fx->indices, Fx->vals, vals_y, vals_z, u, R9, E, G);
  return check_launch("cpm_strain_from_u");
}

extern "C" int cpm_strain_finalize(int64_t n, double *E, const double *avgE, const double *avg_m100,
                                   double lam100, double lam111, const double *Ebar_sigma6, const double *M36,
                                   const double *MinvT36, int rot111, void *stream) {
  if (!E || !avgE || !avg_m100 || !Ebar_sigma6 || (rot111 && (!M36 || !MinvT36))) {
    set_error("cpm_strain_finalize: bad arguments");
    return CPM_BAD_ARG;
  }
  if (n <= 0) return CPM_OK;
  strain_fin_kernel<<<ew_grid(n), kEwThreads, 0, (cudaStream_t)stream>>>(n, E, avgE, avg_m100, lam100, lam111,
                                                                         Ebar_sigma6, M36, MinvT36, rot111);
  return check_launch("cpm_strain_finalize");
}
