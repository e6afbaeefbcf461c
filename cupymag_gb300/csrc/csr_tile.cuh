// Shared-memory staged CSR row products for FP64 on sm_103a.
//
// GB300 has little FP64 throughput (about 2 FP64 lanes per clock per SM), so
// an FP64 SpMV is limited by FP64 instructions as much as by HBM.  The
// warp-per-row scheme spends 5 FP64 shuffle-adds per row on the reduction,
// more than the 27 products of a scalar row can afford.  Here each row is
// summed by a small group of G threads (G = 1 for the 27-entry scalar rows,
// 4 for the 81-entry elastic rows, 8 for the 162-entry coupling rows) with one
// fused multiply-add per non-zero and log2(G) adds per row.
//
// Coalescing comes from staging: the CTA copies a tile's contiguous
// value/index stream into shared memory with 16-byte cp.async.cg copies
// (L2 only, so the stream does not evict the gathered vector from L1), then
// the thread groups read their rows from shared memory.  For the structured
// hex operators consecutive threads own consecutive rows, whose columns are
// shifted by one, so the gathers of x are coalesced too.
#pragma once

#include "cpm_common.cuh"

namespace cpm {

// Single-value tiles are sized so four 256-thread CTAs fit on an SM (43 KB each):
// while one CTA waits for its copies the others compute.
constexpr int kTileCap = 3584;                          // non-zeros per staged tile
constexpr int kTileSmemBytes = kTileCap * 8 + 16 + (kTileCap + 4) * 4 + 16;
// Tiles of three value arrays (Fx, Fy, Fz) are larger so 27-entry rows keep
// small thread groups.
constexpr int kMultiSmemBytes = 86064;

struct TileSmem {
  double *v;  // kTileCap + 2 values (offset so 16-byte copies land aligned)
  int *c;     // kTileCap + 4 indices
};

__device__ __forceinline__ TileSmem tile_smem(unsigned char *base) {
  TileSmem t;
  t.v = reinterpret_cast<double *>(base);
  t.c = reinterpret_cast<int *>(base + (size_t)(kTileCap + 2) * 8);
  return t;
}

__device__ __forceinline__ void cp16(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Copy values/indices [s, e) into shared memory.  Element s + i lands at
// v[i + (s & 1)] and c[i + (s & 3)], so global and shared 16-byte boundaries
// coincide.  Caller guarantees e - s <= kTileCap.  Ends with __syncthreads().
__device__ __forceinline__ void stage(const TileSmem &t, const double *av, const int *ci, int64_t s, int64_t e) {
  const int ov = (int)(s & 1), oc = (int)(s & 3);
  const int tid = threadIdx.x;
  // values: 16-byte pairs [pa, pb); head element s when s is odd, tail e-1 when e is odd
  const int64_t pa = (s + 1) & ~int64_t(1), pb = e & ~int64_t(1);
  for (int64_t g = pa + 2 * (int64_t)tid; g < pb; g += 2 * (int64_t)blockDim.x) cp16(t.v + (g - s) + ov, av + g);
  if (tid == 0 && (s & 1) && s < e) t.v[ov] = __ldcs(av + s);
  if (tid == 1 && (e & 1) && e - 1 >= pa) t.v[(e - 1 - s) + ov] = __ldcs(av + e - 1);
  // indices: 16-byte quads [qa, qb); head [s, min(qa, e)), tail [max(qb, qa), e)
  const int64_t qa = (s + 3) & ~int64_t(3), qb = e & ~int64_t(3);
  for (int64_t g = qa + 4 * (int64_t)tid; g < qb; g += 4 * (int64_t)blockDim.x) cp16(t.c + (g - s) + oc, ci + g);
  const int64_t hend = qa < e ? qa : e;
  const int64_t tbeg = qb > qa ? qb : qa;
  if (tid >= 32 && tid < 35 && s + (tid - 32) < hend) t.c[(tid - 32) + oc] = __ldcs(ci + s + (tid - 32));
  if (tid >= 64 && tid < 67 && tbeg + (tid - 64) < e) t.c[(tbeg + (tid - 64) - s) + oc] = __ldcs(ci + tbeg + (tid - 64));
  cp_wait_all();
  __syncthreads();
}

// Row sums y_row = sum_k a_k x[c_k] for rows [t0, t1) of a tile, G threads per
// row (threadIdx.x / G = local row).  Returns, in every thread, its row (or -1)
// and the group's complete sum in acc (valid in the group's first lane).
// NR right-hand sides are interleaved in x ((cols, NR) layout).
template <int NR, typename IT, typename XS = const double *>
__device__ __forceinline__ int64_t tile_rows(const IT *__restrict__ rp, const int *__restrict__ ci,
                                             const double *__restrict__ av, const XS &x, int64_t t0, int64_t t1,
                                             int G, const TileSmem &t, double (&acc)[NR]) {
  const int64_t s = (int64_t)__ldg(rp + t0), e = (int64_t)__ldg(rp + t1);
  const bool staged = (e - s) <= kTileCap;
  if (staged) stage(t, av, ci, s, e);
  const int lr = threadIdx.x / G, sub = threadIdx.x % G;
  const int64_t row = t0 + lr;
#pragma unroll
  for (int j = 0; j < NR; ++j) acc[j] = 0.0;
  if (row < t1) {
    const int64_t rs = (int64_t)__ldg(rp + row), re = (int64_t)__ldg(rp + row + 1);
    if (staged) {
      const int ov = (int)(s & 1), oc = (int)(s & 3);
      const double *vv = t.v + ov - s;
      const int *cc = t.c + oc - s;
#pragma unroll 4
      for (int64_t k = rs + sub; k < re; k += G) {
        const double a = vv[k];
        const int64_t c = cc[k];
#pragma unroll
        for (int j = 0; j < NR; ++j) acc[j] = fma(a, ld<double>(x, c * NR + j, j), acc[j]);
      }
    } else {
      for (int64_t k = rs + sub; k < re; k += G) {
        const double a = __ldcs(av + k);
        const int64_t c = __ldcs(ci + k);
#pragma unroll
        for (int j = 0; j < NR; ++j) acc[j] = fma(a, ld<double>(x, c * NR + j, j), acc[j]);
      }
    }
  }
  for (int o = 1; o < G; o <<= 1) {
#pragma unroll
    for (int j = 0; j < NR; ++j) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
  }
  __syncthreads();  // shared tile may be overwritten by the next call
  return (row < t1) ? row : -1;
}

// FP32 form for the mixed-precision solver: FP32 values and indices staged in
// the same 16-byte quads (element s + i lands at v[i + (s & 3)], c[i + (s & 3)]),
// FP32 products and FP32 group sums.
struct TileSmem32 {
  float *v;  // kTileCap + 4 values
  int *c;    // kTileCap + 4 indices
};

__device__ __forceinline__ TileSmem32 tile_smem32(unsigned char *base) {
  TileSmem32 t;
  t.v = reinterpret_cast<float *>(base);
  t.c = reinterpret_cast<int *>(base + (size_t)(kTileCap + 4) * 4);
  return t;
}

__device__ __forceinline__ void stage32(const TileSmem32 &t, const float *av, const int *ci, int64_t s, int64_t e) {
  const int oc = (int)(s & 3);
  const int tid = threadIdx.x;
  const int64_t qa = (s + 3) & ~int64_t(3), qb = e & ~int64_t(3);
  for (int64_t g = qa + 4 * (int64_t)tid; g < qb; g += 4 * (int64_t)blockDim.x) {
    cp16(t.v + (g - s) + oc, av + g);
    cp16(t.c + (g - s) + oc, ci + g);
  }
  const int64_t hend = qa < e ? qa : e;
  const int64_t tbeg = qb > qa ? qb : qa;
  if (tid >= 32 && tid < 35 && s + (tid - 32) < hend) {
    t.v[(tid - 32) + oc] = __ldcs(av + s + (tid - 32));
    t.c[(tid - 32) + oc] = __ldcs(ci + s + (tid - 32));
  }
  if (tid >= 64 && tid < 67 && tbeg + (tid - 64) < e) {
    t.v[(tbeg + (tid - 64) - s) + oc] = __ldcs(av + tbeg + (tid - 64));
    t.c[(tbeg + (tid - 64) - s) + oc] = __ldcs(ci + tbeg + (tid - 64));
  }
  cp_wait_all();
  __syncthreads();
}

template <int NR, typename IT>
__device__ __forceinline__ int64_t tile_rows32(const IT *__restrict__ rp, const int *__restrict__ ci,
                                               const float *__restrict__ av, const float *x, int64_t t0, int64_t t1,
                                               int G, const TileSmem32 &t, float (&acc)[NR]) {
  const int64_t s = (int64_t)__ldg(rp + t0), e = (int64_t)__ldg(rp + t1);
  const bool staged = (e - s) <= kTileCap;
  if (staged) stage32(t, av, ci, s, e);
  const int lr = threadIdx.x / G, sub = threadIdx.x % G;
  const int64_t row = t0 + lr;
#pragma unroll
  for (int j = 0; j < NR; ++j) acc[j] = 0.0f;
  if (row < t1) {
    const int64_t rs = (int64_t)__ldg(rp + row), re = (int64_t)__ldg(rp + row + 1);
    if (staged) {
      const int oc = (int)(s & 3);
      const float *vv = t.v + oc - s;
      const int *cc = t.c + oc - s;
#pragma unroll 4
      for (int64_t k = rs + sub; k < re; k += G) {
        const float a = vv[k];
        const int64_t c = cc[k];
#pragma unroll
        for (int j = 0; j < NR; ++j) acc[j] = fmaf(a, x[c * NR + j], acc[j]);
      }
    } else {
      for (int64_t k = rs + sub; k < re; k += G) {
        const float a = __ldcs(av + k);
        const int64_t c = __ldcs(ci + k);
#pragma unroll
        for (int j = 0; j < NR; ++j) acc[j] = fmaf(a, x[c * NR + j], acc[j]);
      }
    }
  }
  for (int o = 1; o < G; o <<= 1) {
#pragma unroll
    for (int j = 0; j < NR; ++j) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
  }
  __syncthreads();  // shared tile may be overwritten by the next call
  return (row < t1) ? row : -1;
}

// Threads per row for a matrix whose longest row has `maxlen` entries and a
// CTA of `threads`: the smallest power of two G with (threads / G) * maxlen
// fitting one staged tile.
inline int group_size(int64_t maxlen, int threads) {
  int G = 1;
  while (G < 32 && (int64_t)(threads / G) * maxlen > kTileCap) G <<= 1;
  return G;
}

}  // namespace cpm

namespace cpm {

// ---------------------------------------------------------------------------
// Several value arrays sharing one pattern (Fx, Fy, Fz): stage the indices
// once and NV value streams.  Capacity in non-zeros for NV value arrays.
template <int NV>
__host__ __device__ constexpr int multi_cap() {
  return NV == 1 ? kTileCap : ((kMultiSmemBytes - 64) / (8 * NV + 4)) / 4 * 4 - 4;
}

template <int NV>
__host__ __device__ constexpr int multi_smem() {
  return NV == 1 ? kTileSmemBytes : kMultiSmemBytes;
}

template <int NV>
struct MultiTile {
  double *v[NV];
  int *c;
};

template <int NV>
__device__ __forceinline__ MultiTile<NV> multi_tile_smem(unsigned char *base) {
  MultiTile<NV> t;
  size_t off = 0;
  for (int q = 0; q < NV; ++q) {
    t.v[q] = reinterpret_cast<double *>(base + off);
    off += ((size_t)(multi_cap<NV>() + 2) * 8 + 15) / 16 * 16;
  }
  t.c = reinterpret_cast<int *>(base + off);
  return t;
}

template <int NV>
__device__ __forceinline__ void stage_multi(const MultiTile<NV> &t, const double *const *av, const int *ci, int64_t s,
                                            int64_t e) {
  const int ov = (int)(s & 1), oc = (int)(s & 3);
  const int tid = threadIdx.x;
  const int64_t pa = (s + 1) & ~int64_t(1), pb = e & ~int64_t(1);
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    for (int64_t g = pa + 2 * (int64_t)tid; g < pb; g += 2 * (int64_t)blockDim.x) cp16(t.v[q] + (g - s) + ov, av[q] + g);
    if (tid == 0 && (s & 1) && s < e) t.v[q][ov] = __ldcs(av[q] + s);
    if (tid == 1 && (e & 1) && e - 1 >= pa) t.v[q][(e - 1 - s) + ov] = __ldcs(av[q] + e - 1);
  }
  const int64_t qa = (s + 3) & ~int64_t(3), qb = e & ~int64_t(3);
  for (int64_t g = qa + 4 * (int64_t)tid; g < qb; g += 4 * (int64_t)blockDim.x) cp16(t.c + (g - s) + oc, ci + g);
  const int64_t hend = qa < e ? qa : e;
  const int64_t tbeg = qb > qa ? qb : qa;
  if (tid >= 32 && tid < 35 && s + (tid - 32) < hend) t.c[(tid - 32) + oc] = __ldcs(ci + s + (tid - 32));
  if (tid >= 64 && tid < 67 && tbeg + (tid - 64) < e) t.c[(tbeg + (tid - 64) - s) + oc] = __ldcs(ci + tbeg + (tid - 64));
  cp_wait_all();
  __syncthreads();
}

// Visit the non-zeros of this thread's share of its row in a tile of rows
// [t0, t1): f(a[NV], col) for k = row_start + sub, step G.  Returns the row or
// -1.  The caller combines the G partial results and must __syncthreads()
// before the next tile reuses shared memory.
template <int NV, typename IT, class F>
__device__ __forceinline__ int64_t visit_tile(const IT *__restrict__ rp, const int *__restrict__ ci,
                                              const double *const *av, int64_t t0, int64_t t1, int G,
                                              const MultiTile<NV> &t, F &&f) {
  const int64_t s = (int64_t)__ldg(rp + t0), e = (int64_t)__ldg(rp + t1);
  const bool staged = (e - s) <= multi_cap<NV>();
  if (staged) stage_multi<NV>(t, av, ci, s, e);
  const int lr = threadIdx.x / G, sub = threadIdx.x % G;
  const int64_t row = t0 + lr;
  if (row < t1) {
    const int64_t rs = (int64_t)__ldg(rp + row), re = (int64_t)__ldg(rp + row + 1);
    double a[NV];
    if (staged) {
      const int ov = (int)(s & 1), oc = (int)(s & 3);
#pragma unroll 4
      for (int64_t k = rs + sub; k < re; k += G) {
#pragma unroll
        for (int q = 0; q < NV; ++q) a[q] = t.v[q][k - s + ov];
        f(a, (int64_t)t.c[k - s + oc]);
      }
    } else {
      for (int64_t k = rs + sub; k < re; k += G) {
#pragma unroll
        for (int q = 0; q < NV; ++q) a[q] = __ldcs(av[q] + k);
        f(a, (int64_t)__ldcs(ci + k));
      }
    }
  }
  return row < t1 ? row : -1;
}

// Row `row` (< rows) summed by the G lanes of its group (lane sub = threadIdx.x % G takes entries
// start + sub, start + sub + G, ...), entries read in place: each load instruction of a warp fills whole
// 32-byte sectors of its 32 / G rows.  The sum of the group's lanes ends in every lane (log2(G) shuffle-
// adds); every lane of the warp must call it (a row past the end sums zero).  NR right-hand sides are
// interleaved in x; TA is the arithmetic type (FP64, or FP32 for the refinement form's products).
template <int NR, int G, typename IT, typename TA = double, typename TV = double, typename TX = double>
__device__ __forceinline__ void group_row(const IT *__restrict__ rp, const int *__restrict__ ci,
                                          const TV *__restrict__ av, const TX *x, int64_t row, int64_t rows,
                                          TA (&acc)[NR]) {
#pragma unroll
  for (int j = 0; j < NR; ++j) acc[j] = TA(0);
  if (row < rows) {
    const int sub = threadIdx.x % G;
    const int64_t rs = (int64_t)__ldg(rp + row), re = (int64_t)__ldg(rp + row + 1);
#pragma unroll 4
    for (int64_t k = rs + sub; k < re; k += G) {
      const TA a = (TA)__ldcs(av + k);
      const int64_t c = __ldcs(ci + k);
#pragma unroll
      for (int j = 0; j < NR; ++j) acc[j] = fma(a, (TA)x[c * NR + j], acc[j]);
    }
  }
#pragma unroll
  for (int o = 1; o < G; o <<= 1)
#pragma unroll
    for (int j = 0; j < NR; ++j) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
}

__device__ __forceinline__ double group_sum(double v, int G) {
  for (int o = 1; o < G; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

inline int group_size_cap(int64_t maxlen, int threads, int cap) {
  int G = 1;
  while (G < 32 && (int64_t)(threads / G) * maxlen > cap) G <<= 1;
  return G;
}

}  // namespace cpm
