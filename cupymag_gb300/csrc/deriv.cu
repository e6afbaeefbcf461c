// Matrix-free derivative and coupling operators of the periodic hex grid (sm_103a).
//
// The three derivative matrices F_i (F_i[p, q] = integral of N_p dN_q/dx_i,
// cupymag/physics/assemble_demag.py:95-184) and the magnetoelastic coupling
// F_el = B^T C S (cupymag/physics/assemble_elasticity.py:268-459) are, on a
// grid of identical unit cells, 27-point periodic stencils: the coefficient
// between DOF p and DOF p + d is the same for every p.  These kernels apply
// them without the CSR matrices, which at 128^3 hold 1.6 GB (Fx, Fy, Fz) and
// 12.2 GB (F_el):
//
// * cpm_stencil_deriv  mode 0: Hd = alpha (Fx U, Fy U, Fz U)  (compute_derivatives.py:36-58)
//                      mode 1: b = alpha sum_i F_i (m_i - <m>_i), b[pin] = 0  (Micromagnetics.py:166-168)
// * cpm_stencil_strain  E (n,6) from u = [ux|uy|uz], optionally rotated by R
//                       (compute_derivatives.py:60-125)
// * cpm_stencil_fel     b_el = F_el E0, E0 node-interleaved (6n), b_el [x|y|z] (Micromagnetics.py:123),
//                       with the reference's empty anchor rows 0, n, 2n
//                       (assemble_elasticity.py:461-527)
//
// Every product is FP64 with the coefficients in the launch parameters
// (constant bank operands of the FMAs), so all three are bound by GB300's FP64
// pipe (about 2 FP64 operations per clock per SM); a few warps per SM keep it
// busy, so the kernels use the registers they need (no occupancy cap).
//
// The stencils are odd in the offset, c(-d) = -c(d) with c(0) = 0: on the
// periodic grid F_i[p, q] = integral of N_p dN_q/dx_i integrates by parts into
// -F_i[q, p], and F_el = B^T C S is a first-derivative operator the same way
// (the assembled coefficients are odd to 1e-16 of their size).  Each pair of
// opposite neighbours then enters once, as the difference of the two gathered
// values times the odd part (c(d) - c(-d)) / 2, and the difference serves every
// output: FP64 operations per DOF 81 -> 52 (Hd), 162 -> 78 (demag right-hand
// side: the mean shift cancels in the difference), 243 -> 156 (strain) and
// 486 -> 312 (F_el).  The host checks the oddness of the caller's stencil
// (|c(d) + c(-d)| <= 1e-12 max |c|, |c(0)| as small) and otherwise sums all 27
// neighbours in lexicographic offset order.  Results agree with the CSR
// products to rounding.
#include <algorithm>
#include <cmath>

#include "stencil_ops.cuh"

namespace cpm {

constexpr int kDerivThreads = 256;

struct DerivArgs {
  int nx, ny, nz, n;
  const uint8_t *flags;  // unused (neighbours() takes any record with these fields)
  double f[3][27];
  double h[3][13];       // odd part (f[d] - f[26 - d]) / 2 of offsets d < 13 (the pair d, 26 - d)
};

struct FelArgs {
  int nx, ny, nz, n;
  const uint8_t *flags;
  int anchor;
  double c[3 * 6 * 27];
  double h[3 * 6 * 13];  // odd part, as DerivArgs::h, per (output, input)
};

// The neighbours d and 26 - d (opposite offsets) of a DOF with wrapped offsets b, d < 13.
__device__ __forceinline__ void pair_nodes(const Nbr &b, int d, int &qp, int &qm) {
  const int ia = d / 9, ib = (d / 3) % 3, ic = d % 3;
  qp = b.xi[ia] + b.yj[ib] + b.zk[ic];
  qm = b.xi[2 - ia] + b.yj[2 - ib] + b.zk[2 - ic];
}

static inline int64_t deriv_grid(int64_t n) {
  const int64_t cap = (int64_t)sm_count() * 8;
  return std::max<int64_t>(1, std::min<int64_t>((n + kDerivThreads - 1) / kDerivThreads, cap));
}

// ---------------------------------------------------------------- Hd and the demag right-hand side
template <int MODE, bool ODD>
__global__ void __launch_bounds__(kDerivThreads) deriv_kernel(const __grid_constant__ DerivArgs a,
                                                              const double *__restrict__ x, double *__restrict__ y,
                                                              double alpha, const double *shift, int64_t pin) {
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  if (MODE == 1 && shift) {
    s0 = shift[0];
    s1 = shift[1];
    s2 = shift[2];
  }
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < a.n; p += stride) {
    const Nbr b = neighbours(a, (int)p);
    double acc0 = 0.0, acc1 = 0.0, acc2 = 0.0;
    if (ODD) {
#pragma unroll
      for (int d = 0; d < 13; ++d) {
        int qp, qm;
        pair_nodes(b, d, qp, qm);
        if (MODE == 0) {
          const double v = __ldg(x + qp) - __ldg(x + qm);
          acc0 = fma(a.h[0][d], v, acc0);
          acc1 = fma(a.h[1][d], v, acc1);
          acc2 = fma(a.h[2][d], v, acc2);
        } else {
          acc0 = fma(a.h[0][d], __ldg(x + 3 * (int64_t)qp + 0) - __ldg(x + 3 * (int64_t)qm + 0), acc0);
          acc1 = fma(a.h[1][d], __ldg(x + 3 * (int64_t)qp + 1) - __ldg(x + 3 * (int64_t)qm + 1), acc1);
          acc2 = fma(a.h[2][d], __ldg(x + 3 * (int64_t)qp + 2) - __ldg(x + 3 * (int64_t)qm + 2), acc2);
        }
      }
    }
#pragma unroll
    for (int ia = 0; ia < 3; ++ia)
#pragma unroll
      for (int ib = 0; ib < 3; ++ib)
#pragma unroll
        for (int ic = 0; ic < 3; ++ic) {
          if (ODD) continue;
          const int q = b.xi[ia] + b.yj[ib] + b.zk[ic];
          const int d = (ia * 3 + ib) * 3 + ic;
          if (MODE == 0) {
            const double v = __ldg(x + q);
            acc0 = fma(a.f[0][d], v, acc0);
            acc1 = fma(a.f[1][d], v, acc1);
            acc2 = fma(a.f[2][d], v, acc2);
          } else {
            acc0 = fma(a.f[0][d], __ldg(x + 3 * (int64_t)q + 0) - s0, acc0);
            acc1 = fma(a.f[1][d], __ldg(x + 3 * (int64_t)q + 1) - s1, acc1);
            acc2 = fma(a.f[2][d], __ldg(x + 3 * (int64_t)q + 2) - s2, acc2);
          }
        }
    if (MODE == 0) {
      y[3 * p + 0] = alpha * acc0;
      y[3 * p + 1] = alpha * acc1;
      y[3 * p + 2] = alpha * acc2;
    } else {
      y[p] = p == pin ? 0.0 : alpha * ((acc0 + acc1) + acc2);
    }
  }
}

// ---------------------------------------------------------------- strain from u
template <bool ODD>
__global__ void __launch_bounds__(kDerivThreads) strain_stencil_kernel(const __grid_constant__ DerivArgs a,
                                                                       const double *__restrict__ u,
                                                                       const double *R9, double *__restrict__ E) {
  const int64_t n = a.n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  double R[9];
  if (R9) {
#pragma unroll
    for (int k = 0; k < 9; ++k) R[k] = R9[k];
  }
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
    const Nbr b = neighbours(a, (int)p);
    double d[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // d[a][b] = (F_a u_b)_p
    if (ODD) {
#pragma unroll
      for (int s = 0; s < 13; ++s) {
        int qp, qm;
        pair_nodes(b, s, qp, qm);
        const double uu[3] = {__ldg(u + qp) - __ldg(u + qm), __ldg(u + n + qp) - __ldg(u + n + qm),
                              __ldg(u + 2 * n + qp) - __ldg(u + 2 * n + qm)};
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int c = 0; c < 3; ++c) d[k][c] = fma(a.h[k][s], uu[c], d[k][c]);
      }
    }
#pragma unroll
    for (int ia = 0; ia < 3 && !ODD; ++ia)
#pragma unroll
      for (int ib = 0; ib < 3; ++ib)
#pragma unroll
        for (int ic = 0; ic < 3; ++ic) {
          const int q = b.xi[ia] + b.yj[ib] + b.zk[ic];
          const int s = (ia * 3 + ib) * 3 + ic;
          const double uu[3] = {__ldg(u + q), __ldg(u + n + q), __ldg(u + 2 * n + q)};
#pragma unroll
          for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int c = 0; c < 3; ++c) d[k][c] = fma(a.f[k][s], uu[c], d[k][c]);
        }
    double out[6];
    if (!R9) {
      out[0] = d[0][0];
      out[1] = d[1][1];
      out[2] = d[2][2];
      out[3] = d[1][0] + d[0][1];
      out[4] = d[2][1] + d[1][2];
      out[5] = d[2][0] + d[0][2];
    } else {
      // R[r][c] = R9[3r+c]; the association of the reference's rotated strain (compute_derivatives.py:94-123)
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
    double2 *e2 = reinterpret_cast<double2 *>(E + 6 * p);
    e2[0] = make_double2(out[0], out[1]);
    e2[1] = make_double2(out[2], out[3]);
    e2[2] = make_double2(out[4], out[5]);
  }
}

// ---------------------------------------------------------------- b_el = F_el E0
template <bool ODD>
__global__ void __launch_bounds__(kDerivThreads, 3) fel_stencil_kernel(const __grid_constant__ FelArgs a,
                                                                    const double *__restrict__ E0,
                                                                    double *__restrict__ y) {
  const int64_t n = a.n;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += stride) {
    double acc[3] = {0.0, 0.0, 0.0};
    if (ODD && !(a.anchor && p == 0)) {
      const Nbr b = neighbours(a, (int)p);
#pragma unroll
      for (int d = 0; d < 13; ++d) {
        int qp, qm;
        pair_nodes(b, d, qp, qm);
        const double2 *ep = reinterpret_cast<const double2 *>(E0 + 6 * (int64_t)qp);
        const double2 *em = reinterpret_cast<const double2 *>(E0 + 6 * (int64_t)qm);
        const double2 p01 = __ldg(ep), p23 = __ldg(ep + 1), p45 = __ldg(ep + 2);
        const double2 m01 = __ldg(em), m23 = __ldg(em + 1), m45 = __ldg(em + 2);
        const double v[6] = {p01.x - m01.x, p01.y - m01.y, p23.x - m23.x, p23.y - m23.y, p45.x - m45.x, p45.y - m45.y};
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int k = 0; k < 6; ++k) acc[r] = fma(a.h[(r * 6 + k) * 13 + d], v[k], acc[r]);
      }
    } else if (!(a.anchor && p == 0)) {
      const Nbr b = neighbours(a, (int)p);
#pragma unroll
      for (int ia = 0; ia < 3; ++ia)
#pragma unroll
        for (int ib = 0; ib < 3; ++ib)
#pragma unroll
          for (int ic = 0; ic < 3; ++ic) {
            const int q = b.xi[ia] + b.yj[ib] + b.zk[ic];
            const int d = (ia * 3 + ib) * 3 + ic;
            const double2 *e = reinterpret_cast<const double2 *>(E0 + 6 * (int64_t)q);
            const double2 v01 = __ldg(e), v23 = __ldg(e + 1), v45 = __ldg(e + 2);
            const double v[6] = {v01.x, v01.y, v23.x, v23.y, v45.x, v45.y};
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
              for (int k = 0; k < 6; ++k) acc[r] = fma(a.c[(r * 6 + k) * 27 + d], v[k], acc[r]);
          }
    }
    y[p] = acc[0];
    y[n + p] = acc[1];
    y[2 * n + p] = acc[2];
  }
}

static bool grid_ok(int nx, int ny, int nz, int64_t parts) {
  return nx >= 3 && ny >= 3 && nz >= 3 && (int64_t)nx * ny * nz * parts < ((int64_t)1 << 31);
}

static DerivArgs deriv_args(const cpm_deriv_stencil *D) {
  DerivArgs a{};
  a.nx = D->nx;
  a.ny = D->ny;
  a.nz = D->nz;
  a.n = D->nx * D->ny * D->nz;
  a.flags = nullptr;
  for (int d = 0; d < 27; ++d) {
    a.f[0][d] = D->fx[d];
    a.f[1][d] = D->fy[d];
    a.f[2][d] = D->fz[d];
  }
  for (int k = 0; k < 3; ++k)
    for (int d = 0; d < 13; ++d) a.h[k][d] = 0.5 * (a.f[k][d] - a.f[k][26 - d]);
  return a;
}

// Whether each run of 27 coefficients is odd in the offset (to 1e-12 of its largest magnitude).
static bool stencils_odd(const double *c, int count) {
  for (int s = 0; s < count; ++s) {
    const double *v = c + 27 * s;
    double big = 0.0;
    for (int d = 0; d < 27; ++d) big = std::max(big, std::fabs(v[d]));
    const double tol = 1e-12 * big;
    if (std::fabs(v[13]) > tol) return false;
    for (int d = 0; d < 13; ++d)
      if (std::fabs(v[d] + v[26 - d]) > tol) return false;
  }
  return true;
}

}  // namespace cpm

extern "C" int cpm_stencil_deriv(const cpm_deriv_stencil *D, const double *x, double *y, double alpha, int mode,
                                 const double *shift, int64_t pin, void *stream) {
  using namespace cpm;
  if (!D || !x || !y || (mode != 0 && mode != 1) || !grid_ok(D->nx, D->ny, D->nz, 6)) {
    set_error("cpm_stencil_deriv: bad arguments (at least 3 cells per axis, mode 0 or 1)");
    return CPM_BAD_ARG;
  }
  const DerivArgs a = deriv_args(D);
  cudaStream_t st = (cudaStream_t)stream;
  const int g = (int)deriv_grid(a.n);
  const bool odd = stencils_odd(&a.f[0][0], 3);
  if (mode == 0) {
    if (odd) deriv_kernel<0, true><<<g, kDerivThreads, 0, st>>>(a, x, y, alpha, nullptr, -1);
    else deriv_kernel<0, false><<<g, kDerivThreads, 0, st>>>(a, x, y, alpha, nullptr, -1);
  } else {
    if (odd) deriv_kernel<1, true><<<g, kDerivThreads, 0, st>>>(a, x, y, alpha, shift, pin);
    else deriv_kernel<1, false><<<g, kDerivThreads, 0, st>>>(a, x, y, alpha, shift, pin);
  }
  return check_launch("cpm_stencil_deriv");
}

extern "C" int cpm_stencil_strain(const cpm_deriv_stencil *D, const double *u, const double *R9, double *E,
                                  void *stream) {
  using namespace cpm;
  if (!D || !u || !E || ((uintptr_t)E & 15) || !grid_ok(D->nx, D->ny, D->nz, 6)) {
    set_error("cpm_stencil_strain: bad arguments (at least 3 cells per axis, 16-byte aligned E)");
    return CPM_BAD_ARG;
  }
  const DerivArgs a = deriv_args(D);
  const int g = (int)deriv_grid(a.n);
  if (stencils_odd(&a.f[0][0], 3))
    strain_stencil_kernel<true><<<g, kDerivThreads, 0, (cudaStream_t)stream>>>(a, u, R9, E);
  else
    strain_stencil_kernel<false><<<g, kDerivThreads, 0, (cudaStream_t)stream>>>(a, u, R9, E);
  return check_launch("cpm_stencil_strain");
}

extern "C" int cpm_stencil_fel(const cpm_fel_stencil *F, const double *E0, double *b_el, void *stream) {
  using namespace cpm;
  if (!F || !E0 || !b_el || ((uintptr_t)E0 & 15) || !grid_ok(F->nx, F->ny, F->nz, 6)) {
    set_error("cpm_stencil_fel: bad arguments (at least 3 cells per axis, 16-byte aligned E0)");
    return CPM_BAD_ARG;
  }
  FelArgs a{};
  a.nx = F->nx;
  a.ny = F->ny;
  a.nz = F->nz;
  a.n = F->nx * F->ny * F->nz;
  a.flags = nullptr;
  a.anchor = F->anchor ? 1 : 0;
  for (int i = 0; i < 3 * 6 * 27; ++i) a.c[i] = F->coef[i];
  for (int s = 0; s < 18; ++s)
    for (int d = 0; d < 13; ++d) a.h[s * 13 + d] = 0.5 * (a.c[s * 27 + d] - a.c[s * 27 + 26 - d]);
  const int g = (int)deriv_grid(a.n);
  if (stencils_odd(a.c, 18))
    fel_stencil_kernel<true><<<g, kDerivThreads, 0, (cudaStream_t)stream>>>(a, E0, b_el);
  else
    fel_stencil_kernel<false><<<g, kDerivThreads, 0, (cudaStream_t)stream>>>(a, E0, b_el);
  return check_launch("cpm_stencil_fel");
}
