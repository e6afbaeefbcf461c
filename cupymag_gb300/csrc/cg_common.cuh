// Pieces shared by the CSR and stencil conjugate-gradient kernels.
#pragma once

#include "cpm_common.cuh"

namespace cpm {

constexpr int kCGThreads = 256;
constexpr int kCGWarps = kCGThreads / kWarp;
constexpr int kMaxGrid = 4096;                 // CTAs of one cooperative launch (upper bound)
constexpr size_t kPartHalf = (size_t)9 * kMaxGrid;  // doubles per half of the partials buffer (<= 9 sums per CTA)

// Block-wide sum of NV values per thread over NW warps, deterministic; result broadcast.
template <int NV, int NW>
__device__ __forceinline__ void block_sum(double (&v)[NV], double (*s)[NW]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double t = warp_sum(v[j]);
    if (lane == 0) s[j][w] = t;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < NW; ++k) t += s[j][k];
    v[j] = t;
  }
  __syncthreads();
}

// Write this CTA's NV partials, barrier, and reduce all CTAs' partials.
// The partials buffer alternates between two halves: a CTA may start writing
// the next reduction's partials while slower CTAs still read this one's, and
// the barrier of the next reduction orders the reuse of a half.
template <int NV, int NW>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double *part, int &parity, GridBarrier *bar,
                                         unsigned long long tns, double (*s)[NW]) {
  block_sum<NV>(v, s);
  const int G = gridDim.x;
  part += (size_t)parity * kPartHalf;
  parity ^= 1;
#pragma unroll
  for (int j = 0; j < NV; ++j)
    if (threadIdx.x == j) part[(size_t)blockIdx.x * NV + j] = v[j];
  if (!grid_sync(bar, G, tns)) return false;
  double acc[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) acc[j] = 0.0;
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
#pragma unroll
    for (int j = 0; j < NV; ++j) acc[j] += __ldcg(&part[(size_t)g * NV + j]);
  }
  block_sum<NV>(acc, s);
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j] = acc[j];
  return true;
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
