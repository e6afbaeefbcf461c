// Matrix-free periodic hex operators: per-DOF application (shared by the
// single-system solver in stencil.cu and the batched solver in batched.cu).
#pragma once

#include "cg_common.cuh"

namespace cpm {

enum : uint8_t { kRowIdentity = 1, kRowZero = 2, kColExcluded = 4, kNearExcluded = 8, kNearUnpinned = 16 };

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

// ---------------------------------------------------------------- double-float operands
// A double-float value: the unevaluated sum hi + lo of two floats, about 48 significant bits (Dekker
// 1971).  The residual passes of the FP32 refinement CG use it where its error bound allows
// (csrc/stencil.cu): GB300 issues FP32 instructions at about 64 times its FP64 rate.
namespace df {
struct DF {
  float hi, lo;
  __device__ __forceinline__ DF(float h = 0.0f, float l = 0.0f) : hi(h), lo(l) {}
};
// acc + w x, renormalised (|lo| at most half an ulp of hi).  The product's high part w.hi x.hi splits
// exactly into p + e by an FMA; the cross terms w.hi x.lo and w.lo x.hi join e in FP32 (w.lo x.lo, below
// 2^-48 of the product, is dropped); acc.hi + p is added exactly by Knuth's TwoSum, the low parts in
// FP32, and Fast2Sum renormalises.  Per term the error is at most 2^-48 (13 |w x| + 3 S) with S a bound
// of |acc| and of the sum, so a sum of 27 terms is within 94 * 2^-48 of sum |terms|.  The _rn
// intrinsics keep the compiler from contracting the TwoSum's additions with the product.
__device__ __forceinline__ DF fma(const DF &w, const DF &x, const DF &acc) {
  const float p = __fmul_rn(w.hi, x.hi);
  float e = fmaf(w.hi, x.hi, -p);
  e = fmaf(w.hi, x.lo, e);
  e = fmaf(w.lo, x.hi, e);
  const float s = __fadd_rn(acc.hi, p);
  const float bv = __fsub_rn(s, acc.hi);
  const float err = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bv)), __fsub_rn(p, bv));
  const float l = __fadd_rn(acc.lo, __fadd_rn(err, e));
  const float h = __fadd_rn(s, l);
  return DF(h, __fsub_rn(l, __fsub_rn(h, s)));
}
}  // namespace df

// An FP64 vector held as two float vectors hi + lo (hi = x rounded to float, lo = x - hi rounded).
struct XSplit {
  const float *hi, *lo;
};
template <typename T>
__device__ __forceinline__ T ld(const XSplit &s, int64_t i, int) { return T(s.hi[i], s.lo[i]); }
template <typename T, bool VEC>
__device__ __forceinline__ void ldq(const XSplit &s, int64_t i, int c, T *v) {
  if (VEC) {
    float h[4], l[4];
    Vec4<float>::load(s.hi + i, h);
    Vec4<float>::load(s.lo + i, l);
#pragma unroll
    for (int e = 0; e < 4; ++e) v[e] = T(h[e], l[e]);
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) v[e] = ld<T>(s, i + e, c);
  }
}
// Right-hand side r of an interleaved split vector of nr right-hand sides (element i at i * nr + r),
// read one value at a time: the double-float residual of nr > 1 vectors takes one vector per pass.
struct XSplitR {
  const float *hi, *lo;
  int nr, r;
};
template <typename T>
__device__ __forceinline__ T ld(const XSplitR &s, int64_t i, int) {
  const int64_t k = i * s.nr + s.r;
  return T(s.hi[k], s.lo[k]);
}
template <typename T, bool VEC>
__device__ __forceinline__ void ldq(const XSplitR &s, int64_t i, int c, T *v) {
#pragma unroll
  for (int e = 0; e < 4; ++e) v[e] = ld<T>(s, i + e, c);
}
// x into its split form at element i.
__device__ __forceinline__ void split_store(double v, float *hi, float *lo, int64_t i) {
  const float h = __double2float_rn(v);
  hi[i] = h;
  lo[i] = __double2float_rn(v - (double)h);
}

template <typename T>
__device__ __forceinline__ const T *coefs(const StencilOp &S);
template <>
__device__ __forceinline__ const double *coefs<double>(const StencilOp &S) { return S.c64; }
template <>
__device__ __forceinline__ const float *coefs<float>(const StencilOp &S) { return S.c32; }

// y = A x at one DOF for a scalar operator (nc = 1), NR interleaved vectors.
// CHECK selects the path that tests every neighbour's column flag.
template <typename T, int NR, bool CHECK, typename Geo, typename XS>
__device__ __forceinline__ void scalar_rows(const Geo &S, const T *c, const XS &x, int dof,
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
        for (int r = 0; r < NR; ++r) y[r] = fma(w, ld<T>(x, (int64_t)q * NR + r, r), y[r]);
      }
}

template <typename T, bool CHECK, typename Geo, typename XS>
__device__ __forceinline__ void elastic_rows(const Geo &S, const T *c, const XS &x, int dof,
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
        const T u0 = ld<T>(x, q, 0), u1 = ld<T>(x, (int64_t)n + q, 1), u2 = ld<T>(x, 2 * (int64_t)n + q, 2);
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
template <typename T, int NC, int NR, typename Geo, typename XS>
__device__ __forceinline__ void apply_c(const Geo &S, const T *c, const XS &x, int dof,
                                        T (&y)[NC * NR]) {
  const uint8_t f = S.flags ? S.flags[dof] : 0;
  if (f & (kRowIdentity | kRowZero)) {
#pragma unroll
    for (int u = 0; u < NC * NR; ++u)
      y[u] = (f & kRowIdentity) ? ld<T>(x, NC == 1 ? (int64_t)dof * NR + u : (int64_t)u * S.n + dof, u) : T(0);
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

// A pinned DOF: identity row and excluded column (the system decouples there: x = b).
template <typename Geo>
__device__ __forceinline__ bool is_pinned(const Geo &S, int64_t dof) {
  return S.flags && (S.flags[dof] & (kRowIdentity | kColExcluded)) == (kRowIdentity | kColExcluded);
}

// ---------------------------------------------------------------- four DOFs along z
// The quad DOF by DOF (flagged quads; for the scalar form of apply4_c also
// quads that leave their z-line); outputs past the end of the grid are zero.
template <typename T, int NC, int NR, bool VEC, typename Geo, typename XS>
__device__ __forceinline__ void apply4_per_dof(const Geo &S, const T *c, const XS &x, int d0,
                                               T (&y)[4][NC * NR]) {
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    T t[NC * NR];
    if (VEC || d0 + kk < S.n) {
      apply_c<T, NC, NR>(S, c, x, d0 + kk, t);
    } else {
#pragma unroll
      for (int u = 0; u < NC * NR; ++u) t[u] = T(0);
    }
#pragma unroll
    for (int u = 0; u < NC * NR; ++u) y[kk][u] = t[u];
  }
}

// The FMAs of the quad at z = k0..k0+3 of the z-lines whose first elements
// are xo[ia] + yo[ib] (the 9 (x, y) neighbour columns) in vector x, with the
// wrapped edge positions km (k0 - 1) and kp (k0 + 4); cs is the component
// stride of the elastic layout.
template <typename T, int NC, int NR, bool VEC, typename XS>
__device__ __forceinline__ void quad_columns(const T *c, const XS &x, const int (&xo)[3], const int (&yo)[3], int k0,
                                             int km, int kp, int64_t cs, T (&y)[4][NC * NR]) {
#pragma unroll
  for (int kk = 0; kk < 4; ++kk)
#pragma unroll
    for (int u = 0; u < NC * NR; ++u) y[kk][u] = T(0);
#pragma unroll
  for (int ia = 0; ia < 3; ++ia)
#pragma unroll
    for (int ib = 0; ib < 3; ++ib) {
      const int col = xo[ia] + yo[ib];
      if (NC == 1) {
        // w[z][r]: z = 0 is k0 - 1, 1..4 the quad, 5 is k0 + 4
        T w[6][NR];
        if (NR == 1) {
          T v[4];
          ldq<T, VEC>(x, (int64_t)col + k0, 0, v);
          w[0][0] = ld<T>(x, (int64_t)col + km, 0);
#pragma unroll
          for (int e = 0; e < 4; ++e) w[1 + e][0] = v[e];
          w[5][0] = ld<T>(x, (int64_t)col + kp, 0);
        } else {
#pragma unroll
          for (int h = 0; h < NR; ++h) {
            T v[4];
            ldq<T, VEC>(x, (int64_t)(col + k0) * NR + 4 * h, (4 * h) % NR, v);
#pragma unroll
            for (int e = 0; e < 4; ++e) w[1 + (4 * h + e) / NR][(4 * h + e) % NR] = v[e];
          }
#pragma unroll
          for (int r = 0; r < NR; ++r) {
            w[0][r] = ld<T>(x, (int64_t)(col + km) * NR + r, r);
            w[5][r] = ld<T>(x, (int64_t)(col + kp) * NR + r, r);
          }
        }
#pragma unroll
        for (int ic = 0; ic < 3; ++ic) {
          const T cw = c[(ia * 3 + ib) * 3 + ic];
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
#pragma unroll
            for (int r = 0; r < NR; ++r) y[kk][r] = fma(cw, w[kk + ic][r], y[kk][r]);
        }
      } else {
        T w[3][6];
#pragma unroll
        for (int cm = 0; cm < 3; ++cm) {
          const int64_t xc = (int64_t)cm * cs + col;
          T v[4];
          ldq<T, VEC>(x, xc + k0, cm, v);
          w[cm][0] = ld<T>(x, xc + km, cm);
#pragma unroll
          for (int e = 0; e < 4; ++e) w[cm][1 + e] = v[e];
          w[cm][5] = ld<T>(x, xc + kp, cm);
        }
#pragma unroll
        for (int ic = 0; ic < 3; ++ic) {
          const int d = (ia * 3 + ib) * 3 + ic;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
#pragma unroll
            for (int r = 0; r < 3; ++r) {
              T acc = y[kk][r];
              acc = fma(c[(r * 3 + 0) * 27 + d], w[0][kk + ic], acc);
              acc = fma(c[(r * 3 + 1) * 27 + d], w[1][kk + ic], acc);
              acc = fma(c[(r * 3 + 2) * 27 + d], w[2][kk + ic], acc);
              y[kk][r] = acc;
            }
        }
      }
    }
}

// Register-blocked application to the quad of DOFs d0..d0+3 (d0 % 4 == 0).
// When the quad lies in one z-line (at k0..k0+3), each of the 9 (x, y)
// neighbour columns is read once per component as 4 consecutive values plus
// the two wrapped edge values k0-1 and k0+4, and serves all three z offsets
// of all four DOFs: 6 loads where the per-DOF form makes 12.  The FMAs run in
// the per-DOF order (neighbour d = (dx, dy, dz) lexicographic, then
// components), so every y is bit-identical to apply_c's.  A quad with a
// flagged DOF (unit / empty row or a neighbour of an excluded column) takes
// apply_c per DOF.
//
// VEC: nz % 4 == 0 and 16-byte aligned operands, so every quad lies in one
// z-line and each group of 4 is one aligned vector load; the solvers use this
// form.  Otherwise (any nz) the groups of 4 are scalar loads and a quad that
// crosses the end of its z-line takes apply_c per DOF.  On GB300 the scalar
// form is slower than the per-DOF product (each lane's loads are 16 bytes
// apart, so every load instruction moves four cache lines through L1); only
// the FP32 product entry point offers it.
//
// PINS: the operand is zero at every pinned DOF (identity row and excluded
// column: flags 1|4), as the FP32 CG keeps it, so an excluded pinned column
// adds nothing and needs no test.  A flagged quad then takes the register-
// blocked product too and only its unit / empty rows are overwritten; only a
// quad next to an excluded column whose row is not an identity row (flag 16)
// takes the per-DOF checked product.
template <typename T, int NC, int NR, bool VEC = true, bool PINS = false, typename Geo, typename XS>
__device__ __forceinline__ void apply4_c(const Geo &S, const T *c, const XS &x, int d0,
                                         T (&y)[4][NC * NR]) {
  if (PINS && VEC && S.flags) {
    const uint32_t w = *reinterpret_cast<const uint32_t *>(S.flags + d0);
    if (w & 0x10101010u) {
      apply4_per_dof<T, NC, NR, VEC>(S, c, x, d0, y);
      return;
    }
    const Nbr b = neighbours(S, d0);
    const int k0 = b.zk[1];
    const int km = b.zk[0];
    const int kp = (k0 + 4 == S.nz) ? 0 : k0 + 4;
    quad_columns<T, NC, NR, VEC>(c, x, b.xi, b.yj, k0, km, kp, (int64_t)S.n, y);
    if (w & 0x03030303u) {
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const uint32_t f = (w >> (8 * kk)) & 3u;
        if (!f) continue;
#pragma unroll
        for (int u = 0; u < NC * NR; ++u)
          y[kk][u] = (f & kRowIdentity)
                         ? ld<T>(x, NC == 1 ? (int64_t)(d0 + kk) * NR + u : (int64_t)u * S.n + d0 + kk, u)
                         : T(0);
      }
    }
    return;
  }
  if (VEC && S.flags && *reinterpret_cast<const uint32_t *>(S.flags + d0) != 0u) {
    apply4_per_dof<T, NC, NR, VEC>(S, c, x, d0, y);
    return;
  }
  const Nbr b = neighbours(S, d0);
  const int k0 = b.zk[1];
  if (!VEC && (k0 + 4 > S.nz || (S.flags && *reinterpret_cast<const uint32_t *>(S.flags + d0) != 0u))) {
    apply4_per_dof<T, NC, NR, VEC>(S, c, x, d0, y);
    return;
  }
  const int km = b.zk[0];                                  // k0 - 1 (wrapped)
  const int kp = (k0 + 4 == S.nz) ? 0 : k0 + 4;            // k0 + 4 (wrapped)
  quad_columns<T, NC, NR, VEC>(c, x, b.xi, b.yj, k0, km, kp, (int64_t)S.n, y);
}

// The NC*NR unknowns o[kk][u] of the quad d0..d0+3 into a vector (aligned vector stores, or scalar
// stores of the DOFs inside the grid).
template <typename T, int NC, int NR, bool VEC = true>
__device__ __forceinline__ void quad_store(T *v, int64_t n, int64_t d0, const T (&o)[4][NC * NR]) {
  if (!VEC) {
    // scalar stores of the DOFs of the quad inside the grid (any alignment)
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
      if (d0 + kk < n) {
#pragma unroll
        for (int u = 0; u < NC * NR; ++u) v[NC == 3 ? (int64_t)u * n + d0 + kk : (d0 + kk) * NR + u] = o[kk][u];
      }
    return;
  }
  if (NC == 3) {
#pragma unroll
    for (int cm = 0; cm < 3; ++cm) {
      T t[4];
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) t[kk] = o[kk][cm];
      Vec4<T>::store(v + cm * n + d0, t);
    }
  } else {
#pragma unroll
    for (int h = 0; h < NR; ++h) {
      T t[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) t[e] = o[(4 * h + e) / NR][(4 * h + e) % NR];
      Vec4<T>::store(v + d0 * NR + 4 * h, t);
    }
  }
}

// acc[sys(u)] += v[quad, u] * y[kk][u] over the quad, reading v in aligned groups
// of 4 (VEC) or element by element for the DOFs inside the grid.
template <int NC, int NR, bool VEC = true>
__device__ __forceinline__ void quad_dot(const float *v, int64_t n, int64_t d0, const float (&y)[4][NC * NR],
                                         float (&acc)[NC == 1 ? NR : 1]) {
  if (!VEC) {
    if (NC == 3) {
#pragma unroll
      for (int cm = 0; cm < 3; ++cm)
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
          if (d0 + kk < n) acc[0] = fmaf(v[(int64_t)cm * n + d0 + kk], y[kk][cm], acc[0]);
    } else {
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        if (d0 + kk < n) {
#pragma unroll
          for (int r = 0; r < NR; ++r) acc[r] = fmaf(v[(d0 + kk) * NR + r], y[kk][r], acc[r]);
        }
    }
    return;
  }
  if (NC == 3) {
#pragma unroll
    for (int cm = 0; cm < 3; ++cm) {
      float t[4];
      Vec4<float>::load(v + cm * n + d0, t);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) acc[0] = fmaf(t[kk], y[kk][cm], acc[0]);
    }
  } else {
#pragma unroll
    for (int h = 0; h < NR; ++h) {
      float t[4];
      Vec4<float>::load(v + d0 * NR + 4 * h, t);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int kk = (4 * h + e) / NR, r = (4 * h + e) % NR;
        acc[r] = fmaf(t[e], y[kk][r], acc[r]);
      }
    }
  }
}

// ---------------------------------------------------------------- vectorised update phases on quads
// The unknowns of quad d0..d0+3 in aligned groups of 4: group h starts at
// (NC == 3: h * n + d0; else d0 * NR + 4 h) and element e belongs to system
// (NC == 1 && NR == 3 ? (4h + e) % 3 : 0).
template <int NC, int NR>
__device__ __forceinline__ int64_t quad_base(int64_t n, int64_t d0, int h) {
  return NC == 3 ? h * n + d0 : d0 * NR + 4 * h;
}
template <int NC, int NR>
__device__ __forceinline__ int quad_sys(int h, int e) {
  return (NC == 1 && NR == 3) ? (4 * h + e) % 3 : 0;
}

// Active systems: d += alpha p, r -= alpha q, rr += r^2 (FP32 per thread).
template <int NC, int NR, int NS>
__device__ __forceinline__ void quad_update(int64_t n, int64_t d0, int activem, const float (&af)[NS], float *d32,
                                            const float *p32, const float *q32, float *r32, float (&rrf)[NS]) {
  constexpr int H = NC == 3 ? 3 : NR;
#pragma unroll
  for (int h = 0; h < H; ++h) {
    bool upd = false;
#pragma unroll
    for (int e = 0; e < 4; ++e) upd |= (activem >> quad_sys<NC, NR>(h, e)) & 1;
    if (!upd) continue;
    const int64_t i0 = quad_base<NC, NR>(n, d0, h);
    float dd[4], pp[4], qq[4], rr[4];
    Vec4<float>::load(d32 + i0, dd);
    Vec4<float>::load(p32 + i0, pp);
    Vec4<float>::load(q32 + i0, qq);
    Vec4<float>::load(r32 + i0, rr);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int s = quad_sys<NC, NR>(h, e);
      if (!((activem >> s) & 1)) continue;
      dd[e] = fmaf(af[s], pp[e], dd[e]);
      rr[e] = fmaf(-af[s], qq[e], rr[e]);
      rrf[s] = fmaf(rr[e], rr[e], rrf[s]);
    }
    Vec4<float>::store(r32 + i0, rr);
    Vec4<float>::store(d32 + i0, dd);
  }
}

// p = r + beta p for the active systems; for systems with a pending reliable
// update also x += d, d = 0 (own unknowns only, so the next phase's true
// residual is a plain product on x), and the split form of x where xh is set.
template <int NC, int NR, int NS>
__device__ __forceinline__ void quad_direction(int64_t n, int64_t d0, int activem, int needm,
                                               const float (&beta)[NS], float *p32, const float *r32, double *x,
                                               float *d32, float *xh = nullptr, float *xl = nullptr) {
  constexpr int H = NC == 3 ? 3 : NR;
#pragma unroll
  for (int h = 0; h < H; ++h) {
    const int64_t i0 = quad_base<NC, NR>(n, d0, h);
    float pp[4], rr[4];
    Vec4<float>::load(p32 + i0, pp);
    Vec4<float>::load(r32 + i0, rr);
    bool fold = false;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int s = quad_sys<NC, NR>(h, e);
      if ((activem >> s) & 1) pp[e] = fmaf(beta[s], pp[e], rr[e]);
      fold |= (needm >> s) & 1;
    }
    Vec4<float>::store(p32 + i0, pp);
    if (fold) {
      float dd[4];
      double xv[4];
      Vec4<float>::load(d32 + i0, dd);
      Vec4<double>::load(x + i0, xv);
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if ((needm >> quad_sys<NC, NR>(h, e)) & 1) {
          xv[e] += (double)dd[e];
          dd[e] = 0.0f;
        }
      Vec4<double>::store(x + i0, xv);
      Vec4<float>::store(d32 + i0, dd);
      if (xh) {
        float h[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          h[e] = __double2float_rn(xv[e]);
          l[e] = __double2float_rn(xv[e] - (double)h[e]);
        }
        Vec4<float>::store(xh + i0, h);
        Vec4<float>::store(xl + i0, l);
      }
    }
  }
}

// ---------------------------------------------------------------- two-barrier FP32 CG: update phase
// Phase A of the two-barrier FP32 CG (csrc/stencil.cu, cg_stencil_ir2_kernel) on
// the quad d0..d0+3, for the systems in `upd`:
//   p = r + beta p,  s = w + beta s   (s tracks A p, w = A r from the product phase)
//   d += alpha p,    r -= alpha s
// and the next reduction's partials of the new r: g += r.r, e += r.s, f += r.p
// (FP32 per thread).  Every vector is read and written at the thread's own
// unknowns, so this phase needs no neighbour data.
template <int NC, int NR, int NS>
__device__ __forceinline__ void quad_update2(int64_t n, int64_t d0, int upd, const float (&af)[NS],
                                             const float (&bf)[NS], float *r32, float *p32, const float *w32,
                                             float *s32, float *d32, float (&g)[NS], float (&e)[NS],
                                             float (&f)[NS]) {
  constexpr int H = NC == 3 ? 3 : NR;
#pragma unroll
  for (int h = 0; h < H; ++h) {
    bool any = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) any |= (upd >> quad_sys<NC, NR>(h, k)) & 1;
    if (!any) continue;
    const int64_t i0 = quad_base<NC, NR>(n, d0, h);
    float rr[4], pp[4], ww[4], ss[4], dd[4];
    Vec4<float>::load(r32 + i0, rr);
    Vec4<float>::load(p32 + i0, pp);
    Vec4<float>::load(w32 + i0, ww);
    Vec4<float>::load(s32 + i0, ss);
    Vec4<float>::load(d32 + i0, dd);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int sy = quad_sys<NC, NR>(h, k);
      if (!((upd >> sy) & 1)) continue;
      pp[k] = fmaf(bf[sy], pp[k], rr[k]);
      ss[k] = fmaf(bf[sy], ss[k], ww[k]);
      dd[k] = fmaf(af[sy], pp[k], dd[k]);
      rr[k] = fmaf(-af[sy], ss[k], rr[k]);
      g[sy] = fmaf(rr[k], rr[k], g[sy]);
      e[sy] = fmaf(rr[k], ss[k], e[sy]);
      f[sy] = fmaf(rr[k], pp[k], f[sy]);
    }
    Vec4<float>::store(r32 + i0, rr);
    Vec4<float>::store(p32 + i0, pp);
    Vec4<float>::store(s32 + i0, ss);
    Vec4<float>::store(d32 + i0, dd);
  }
}

// The same update for one unknown i of system sy (per-DOF path).
__device__ __forceinline__ void update2_one(int64_t i, float a, float b, float *r32, float *p32, const float *w32,
                                            float *s32, float *d32, float &g, float &e, float &f) {
  const float p = fmaf(b, p32[i], r32[i]);
  const float s = fmaf(b, s32[i], w32[i]);
  const float r = fmaf(-a, s, r32[i]);
  d32[i] = fmaf(a, p, d32[i]);
  p32[i] = p;
  s32[i] = s;
  r32[i] = r;
  g = fmaf(r, r, g);
  e = fmaf(r, s, e);
  f = fmaf(r, p, f);
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
