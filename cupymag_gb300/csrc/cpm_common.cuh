// Shared device helpers for the cupymag_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/cupymag_gb300.h"

namespace cpm {

constexpr int kWarp = 32;

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);
int check_launch(const char *what);

#define CPM_TRY(call)                                                         \
  do {                                                                        \
    cudaError_t _e = (call);                                                  \
    if (_e != cudaSuccess) {                                                  \
      ::cpm::set_error("%s: %s", #call, cudaGetErrorString(_e));              \
      return CPM_CUDA_ERROR;                                                  \
    }                                                                         \
  } while (0)

int sm_count();
int device_id();

// ---------------------------------------------------------------- timing
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---------------------------------------------------------------- loads
// Read-only (matrix) loads go through the non-coherent path; vectors that
// the same launch rewrites use plain loads.
template <typename T>
__device__ __forceinline__ T ldg(const T *p) { return __ldg(p); }

// Streaming load for matrix data read once per sweep (ld.global.cs: evict-first
// in L1 and L2), so the solve's vectors stay resident in the 126 MB L2.
__device__ __forceinline__ double ld_stream(const double *p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float *p) { return __ldcs(p); }
__device__ __forceinline__ int ld_stream(const int *p) { return __ldcs(p); }

// ---------------------------------------------------------------- vector access
template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
  static __device__ __forceinline__ void load(const float *p, float *v) {
    const float4 t = *reinterpret_cast<const float4 *>(p);
    v[0] = t.x;
    v[1] = t.y;
    v[2] = t.z;
    v[3] = t.w;
  }
  static __device__ __forceinline__ void store(float *p, const float *v) {
    *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
};
template <>
struct Vec4<double> {
  static __device__ __forceinline__ void load(const double *p, double *v) {
    const double2 a = *reinterpret_cast<const double2 *>(p);
    const double2 b = *reinterpret_cast<const double2 *>(p + 2);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
  }
  static __device__ __forceinline__ void store(double *p, const double *v) {
    *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
    *reinterpret_cast<double2 *>(p + 2) = make_double2(v[2], v[3]);
  }
};

// ---------------------------------------------------------------- operand loaders
// The products read their operand through ld / ld4: element i (component c:
// the right-hand side of an interleaved scalar vector, or the displacement
// component) of a vector of any storage type, converted to T.
template <typename T, typename TX>
__device__ __forceinline__ T ld(const TX *x, int64_t i, int) { return (T)x[i]; }

template <typename T, typename TX>
__device__ __forceinline__ void ld4(const TX *x, int64_t i, int, T *v) {
  TX t[4];
  Vec4<TX>::load(x + i, t);
#pragma unroll
  for (int e = 0; e < 4; ++e) v[e] = (T)t[e];
}

// The operand x + d of an FP64 product: the FP64 iterate x plus the FP32
// correction d of the refinement form (element i, converted to double).
struct XPlusD {
  const double *x;
  const float *d;
};
template <typename T>
__device__ __forceinline__ T ld(const XPlusD &s, int64_t i, int) { return (T)(s.x[i] + (double)s.d[i]); }

// Elements i..i+3: one aligned vector load (VEC) or four scalar loads.
template <typename T, bool VEC, typename TX>
__device__ __forceinline__ void ldq(const TX *x, int64_t i, int c, T *v) {
  if (VEC) {
    ld4<T>(x, i, c, v);
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) v[e] = ld<T>(x, i + e, c);
  }
}

// ---------------------------------------------------------------- reductions
// Fixed shuffle pattern: the result is a deterministic function of the inputs.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------- grid barrier
// Generation-free barrier over all CTAs of a cooperative launch: a 64-bit
// arrival counter that only grows.  Thread 0 of each CTA arrives with one
// atomic add (its CTA's writes, ordered before it by the block barrier, are
// published with it) and reads the round from the value it got back: the
// round ends when the counter reaches the next multiple of the CTA count
// (every CTA arrives once per round and none can arrive twice before all
// arrived once).  The add is a release; the waiters poll with relaxed loads
// and every CTA, the last to arrive included, takes one acquire fence after
// its wait (acquire loads in the polling loop slowed the CTAs still working on
// the same SM).  Every wait
// is bounded by `timeout_ns` of GPU global time; on expiry the CTA sets `error`
// and returns false, and every other waiter leaves when it sees the error
// word, so no CTA can spin forever.  The counter starts at zero (the launcher
// clears the struct).  Measured on GB300: 1.8 us per barrier for 456 CTAs,
// where a counter reset plus a generation flip by the last arriver took 3.3 us.
struct GridBarrier {
  unsigned long long count;
  int error;
  int pad;
};

__device__ __forceinline__ unsigned long long barrier_arrive(unsigned long long *count) {
  unsigned long long old;
  asm volatile("atom.add.release.gpu.global.u64 %0, [%1], 1;" : "=l"(old) : "l"(count) : "memory");
  return old;
}

__device__ __forceinline__ unsigned long long barrier_load(const unsigned long long *count) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(count) : "memory");
  return v;
}

__device__ __forceinline__ void barrier_acquire() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

__device__ __forceinline__ bool grid_sync(GridBarrier *bar, unsigned int nblocks,
                                          unsigned long long timeout_ns) {
  __shared__ int s_fail;
  __syncthreads();
  if (threadIdx.x == 0) {
    int fail = 0;
    const unsigned long long old = barrier_arrive(&bar->count);
    const unsigned long long target = (old / nblocks + 1ull) * nblocks;
    if (old + 1ull < target) {
      const unsigned long long t0 = global_ns();
      unsigned int spins = 0;
      while (barrier_load(&bar->count) < target) {
        // the error word and the clock are read on polls 1, 2, 4, ..., 32 and then every 64th
        ++spins;
        if ((spins & 63u) == 0 || (spins < 64u && (spins & (spins - 1u)) == 0)) {
          if (*(volatile int *)&bar->error) { fail = 1; break; }
          if (global_ns() - t0 > timeout_ns) {
            atomicExch(&bar->error, 1);
            fail = 1;
            break;
          }
        }
      }
    }
    // acquire the other CTAs' writes (released by their arrivals) once, after the wait
    barrier_acquire();
    if (*(volatile int *)&bar->error) fail = 1;
    s_fail = fail;
  }
  __syncthreads();
  return s_fail == 0;
}

}  // namespace cpm
