// Matrix-free periodic hex operators: per-DOF application (shared by the
// single-system solver in stencil.cu and the batched solver in batched.cu).
#pragma once

#include "cg_common.cuh"

namespace cpm {

enum : uint8_t { kRowIdentity = 1, kRowZero = 2, kColExcluded = 4, kNearExcluded = 8 };

// Operator description carried in the kernel's launch parameters: the
// coefficients are read from the parameter (constant) bank with compile-time
// offsets inside the unrolled loops, so no load instruction precedes an FMA.
struct StencilOp {
  int nx, ny, nz, n;
  const uint8_t *flags;
  double c64[243];
  float c32[243];
};

// Wrapped neighbour offsets of a DOF along each axis (index 0: -1, 1: 0, 2: +1).
struct Nbr {
  int xi[3];
  int yj[3];
  int zk[3];
};

// Geo is any record with int nx, ny, nz, n and const uint8_t *flags.
template <typename Geo>
__device__ __forceinline__ Nbr neighbours(const Geo &S, int dof) {
  const unsigned nyz = (unsigned)S.ny * (unsigned)S.nz;
  const unsigned i = (unsigned)dof / nyz;
  const unsigned rem = (unsigned)dof - i * nyz;
  const unsigned j = rem / (unsigned)S.nz;
  const unsigned k = rem - j * (unsigned)S.nz;
  Nbr b;
  b.xi[0] = (int)((i == 0 ? S.nx - 1 : i - 1) * nyz);
  b.xi[1] = (int)(i * nyz);
  b.xi[2] = (int)((i == (unsigned)S.nx - 1 ? 0 : i + 1) * nyz);
  b.yj[0] = (int)((j == 0 ? S.ny - 1 : j - 1) * S.nz);
  b.yj[1] = (int)(j * S.nz);
  b.yj[2] = (int)((j == (unsigned)S.ny - 1 ? 0 : j + 1) * S.nz);
  b.zk[0] = (int)(k == 0 ? S.nz - 1 : k - 1);
  b.zk[1] = (int)k;
  b.zk[2] = (int)(k == (unsigned)S.nz - 1 ? 0 : k + 1);
  return b;
}

template <typename T>
__device__ __forceinline__ const T *coefs(const StencilOp &S);
template <>
__device__ __forceinline__ const double *coefs<double>(const StencilOp &S) { return S.c64; }
template <>
__device__ __forceinline__ const float *coefs<float>(const StencilOp &S) { return S.c32; }

// y = A x at one DOF for a scalar operator (nc = 1), NR interleaved vectors.
// CHECK selects the path that tests every neighbour's column flag.
template <typename T, int NR, bool CHECK, typename Geo, typename TX>
__device__ __forceinline__ void scalar_rows(const Geo &S, const T *c, const TX *__restrict__ x, int dof,
                                            T (&y)[NR]) {
  const Nbr b = neighbours(S, dof);
#pragma unroll
  for (int r = 0; r < NR; ++r) y[r] = T(0);
#pragma unroll
  for (int ia = 0; ia < 3; ++ia)
#pragma unroll
    for (int ib = 0; ib < 3; ++ib)
#pragma unroll
      for (int ic = 0; ic < 3; ++ic) {
        const int q = b.xi[ia] + b.yj[ib] + b.zk[ic];
        if (CHECK && (S.flags[q] & kColExcluded)) continue;
        const T w = c[(ia * 3 + ib) * 3 + ic];
#pragma unroll
        for (int r = 0; r < NR; ++r) y[r] = fma(w, (T)x[q * NR + r], y[r]);
      }
}

template <typename T, bool CHECK, typename Geo, typename TX>
__device__ __forceinline__ void elastic_rows(const Geo &S, const T *c, const TX *__restrict__ x, int dof,
                                             T (&y)[3]) {
  const int n = S.n;
  const Nbr b = neighbours(S, dof);
  y[0] = y[1] = y[2] = T(0);
#pragma unroll
  for (int ia = 0; ia < 3; ++ia)
#pragma unroll
    for (int ib = 0; ib < 3; ++ib)
#pragma unroll
      for (int ic = 0; ic < 3; ++ic) {
        const int q = b.xi[ia] + b.yj[ib] + b.zk[ic];
        if (CHECK && (S.flags[q] & kColExcluded)) continue;
        const int d = (ia * 3 + ib) * 3 + ic;
        const T u0 = (T)x[q], u1 = (T)x[n + q], u2 = (T)x[2 * n + q];
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

// y at one DOF (all NC*NR components) in T, for x stored as TX.  Rows
// flagged as unit / empty are handled first; only rows next to an excluded
// column test neighbour flags.
template <typename T, int NC, int NR, typename Geo, typename TX>
__device__ __forceinline__ void apply_c(const Geo &S, const T *c, const TX *__restrict__ x, int dof,
                                        T (&y)[NC * NR]) {
  const uint8_t f = S.flags ? S.flags[dof] : 0;
  if (f & (kRowIdentity | kRowZero)) {
#pragma unroll
    for (int u = 0; u < NC * NR; ++u)
      y[u] = (f & kRowIdentity) ? (T)x[NC == 1 ? dof * NR + u : u * S.n + dof] : T(0);
    return;
  }
  if (NC == 1) {
    T t[NR];
    if (f & kNearExcluded) scalar_rows<T, NR, true>(S, c, x, dof, t);
    else scalar_rows<T, NR, false>(S, c, x, dof, t);
#pragma unroll
    for (int r = 0; r < NR; ++r) y[r] = t[r];
  } else {
    T t[3];
    if (f & kNearExcluded) elastic_rows<T, true>(S, c, x, dof, t);
    else elastic_rows<T, false>(S, c, x, dof, t);
#pragma unroll
    for (int r = 0; r < 3; ++r) y[r] = t[r];
  }
}

// y at one DOF with the operator's own (launch-parameter) coefficients.
template <typename T, int NC, int NR>
__device__ __forceinline__ void apply(const StencilOp &S, const T *__restrict__ x, int dof, T (&y)[NC * NR]) {
  apply_c<T, NC, NR>(S, coefs<T>(S), x, dof, y);
}

// Unknown index of (dof, component) for the NC/NR layouts.
template <int NC, int NR>
__device__ __forceinline__ int64_t uidx(int64_t n, int64_t dof, int comp) {
  return NC == 1 ? dof * NR + comp : (int64_t)comp * n + dof;
}

}  // namespace cpm
