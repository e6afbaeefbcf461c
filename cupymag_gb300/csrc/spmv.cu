// CSR sparse matrix-vector products used by the LLG step (sm_103a).
//
// The reference applies every operator with cupyx's CSR `A @ x`
// (cuSPARSE).  Here the products are warp-per-row kernels: the 32 lanes of a
// warp stride over one row's non-zeros with coalesced loads of the values and
// column indices (streamed past L1 with an L2 evict-first hint so the vectors
// stay cached), gather x, and reduce with a fixed shuffle tree (deterministic).
// Matrices of the hex grid have 27 (scalar), 81 (elastic stiffness) or 162
// (elastic coupling) non-zeros per row.
#include "cpm_common.cuh"

namespace cpm {

constexpr int kSpThreads = 256;
constexpr int kSpWarps = kSpThreads / kWarp;

static int sp_grid(int64_t rows) {
  int64_t g = (rows + kSpWarps - 1) / kSpWarps;
  const int64_t cap = (int64_t)sm_count() * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

template <typename IT, int NV>
__global__ void __launch_bounds__(kSpThreads) spmv_kernel(int64_t rows, const IT *__restrict__ rp,
                                                          const int *__restrict__ ci, const double *__restrict__ av,
                                                          const double *__restrict__ x, double *__restrict__ y,
                                                          double alpha) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (int64_t)blockIdx.x * kSpWarps + (threadIdx.x >> 5);
  const int64_t ws = (int64_t)gridDim.x * kSpWarps;
  for (int64_t row = w0; row < rows; row += ws) {
    const int64_t s = (int64_t)__ldg(rp + row), e = (int64_t)__ldg(rp + row + 1);
    double acc[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) acc[j] = 0.0;
    for (int64_t k = s + lane; k < e; k += kWarp) {
      const double v = ld_stream(av + k);
      const int64_t c = ld_stream(ci + k);
#pragma unroll
      for (int j = 0; j < NV; ++j) acc[j] = fma(v, __ldg(x + c * NV + j), acc[j]);
    }
#pragma unroll
    for (int j = 0; j < NV; ++j) acc[j] = warp_sum(acc[j]);
    if (lane == 0) {
#pragma unroll
      for (int j = 0; j < NV; ++j) y[row * NV + j] = alpha * acc[j];
    }
  }
}

// mode 0: y[i,k] = alpha (A_k x)_i           (three matrices, one vector)
// mode 1: y[i]   = alpha sum_k (A_k (x_k - shift_k))_i, y[pin] = 0
template <typename IT, int MODE>
__global__ void __launch_bounds__(kSpThreads) spmv3_kernel(int64_t rows, const IT *__restrict__ rp,
                                                           const int *__restrict__ ci, const double *__restrict__ ax,
                                                           const double *__restrict__ ay,
                                                           const double *__restrict__ az,
                                                           const double *__restrict__ x, double *__restrict__ y,
                                                           double alpha, const double *__restrict__ shift,
                                                           int64_t pin) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (int64_t)blockIdx.x * kSpWarps + (threadIdx.x >> 5);
  const int64_t ws = (int64_t)gridDim.x * kSpWarps;
  double sh0 = 0.0, sh1 = 0.0, sh2 = 0.0;
  if (MODE == 1 && shift) {
    sh0 = shift[0];
    sh1 = shift[1];
    sh2 = shift[2];
  }
  for (int64_t row = w0; row < rows; row += ws) {
    const int64_t s = (int64_t)__ldg(rp + row), e = (int64_t)__ldg(rp + row + 1);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int64_t k = s + lane; k < e; k += kWarp) {
      const int64_t c = ld_stream(ci + k);
      const double vx = ld_stream(ax + k), vy = ld_stream(ay + k), vz = ld_stream(az + k);
      if (MODE == 0) {
        const double xv = __ldg(x + c);
        a0 = fma(vx, xv, a0);
        a1 = fma(vy, xv, a1);
        a2 = fma(vz, xv, a2);
      } else {
        a0 = fma(vx, __ldg(x + 3 * c + 0) - sh0, a0);
        a1 = fma(vy, __ldg(x + 3 * c + 1) - sh1, a1);
        a2 = fma(vz, __ldg(x + 3 * c + 2) - sh2, a2);
      }
    }
    a0 = warp_sum(a0);
    a1 = warp_sum(a1);
    a2 = warp_sum(a2);
    if (lane == 0) {
      if (MODE == 0) {
        y[3 * row + 0] = alpha * a0;
        y[3 * row + 1] = alpha * a1;
        y[3 * row + 2] = alpha * a2;
      } else {
        // (Fx m~x + Fy m~y) + Fz m~z, then the sign (Micromagnetics.py:166)
        y[row] = (row == pin) ? 0.0 : alpha * ((a0 + a1) + a2);
      }
    }
  }
}

static int check_csr(const cpm_csr *A, const char *who) {
  if (!A || !A->indptr || !A->indices || !A->vals) {
    set_error("%s: incomplete CSR matrix", who);
    return CPM_BAD_ARG;
  }
  if (A->rows < 0 || A->cols < 0 || A->nnz < 0) {
    set_error("%s: negative matrix dimension", who);
    return CPM_BAD_ARG;
  }
  if (!A->indptr_is64 && A->nnz > INT32_MAX) {
    set_error("%s: nnz %lld needs int64 row pointers", who, (long long)A->nnz);
    return CPM_BAD_ARG;
  }
  return CPM_OK;
}

}  // namespace cpm

extern "C" int cpm_spmv_csr(const cpm_csr *A, const double *x, double *y, double alpha, int nvec, void *stream) {
  using namespace cpm;
  if (int s = check_csr(A, "cpm_spmv_csr")) return s;
  if (!x || !y || (nvec != 1 && nvec != 3)) {
    set_error("cpm_spmv_csr: bad vectors (nvec must be 1 or 3)");
    return CPM_BAD_ARG;
  }
  if (A->rows == 0) return CPM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int g = sp_grid(A->rows);
  if (A->indptr_is64) {
    if (nvec == 1)
      spmv_kernel<int64_t, 1><<<g, kSpThreads, 0, st>>>(A->rows, (const int64_t *)A->indptr, A->indices, A->vals, x, y, alpha);
    else
      spmv_kernel<int64_t, 3><<<g, kSpThreads, 0, st>>>(A->rows, (const int64_t *)A->indptr, A->indices, A->vals, x, y, alpha);
  } else {
    if (nvec == 1)
      spmv_kernel<int32_t, 1><<<g, kSpThreads, 0, st>>>(A->rows, (const int32_t *)A->indptr, A->indices, A->vals, x, y, alpha);
    else
      spmv_kernel<int32_t, 3><<<g, kSpThreads, 0, st>>>(A->rows, (const int32_t *)A->indptr, A->indices, A->vals, x, y, alpha);
  }
  return check_launch("cpm_spmv_csr");
}

extern "C" int cpm_spmv_csr_multi(const cpm_csr *A, const double *vals_y, const double *vals_z, const double *x,
                                  double *y, double alpha, int mode, const double *shift, int64_t pin,
                                  void *stream) {
  using namespace cpm;
  if (int s = check_csr(A, "cpm_spmv_csr_multi")) return s;
  if (!vals_y || !vals_z || !x || !y || (mode != 0 && mode != 1) || A->rows != A->cols) {
    set_error("cpm_spmv_csr_multi: bad arguments");
    return CPM_BAD_ARG;
  }
  if (A->rows == 0) return CPM_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int g = sp_grid(A->rows);
#define CPM_SP3(IT, M)                                                                                     \
  spmv3_kernel<IT, M><<<g, kSpThreads, 0, st>>>(A->rows, (const IT *)A->indptr, A->indices, A->vals, vals_y, \
                                                 vals_z, x, y, alpha, shift, pin)
  if (A->indptr_is64) {
    if (mode == 0) CPM_SP3(int64_t, 0); else CPM_SP3(int64_t, 1);
  } else {
    if (mode == 0) CPM_SP3(int32_t, 0); else CPM_SP3(int32_t, 1);
  }
#undef CPM_SP3
  return check_launch("cpm_spmv_csr_multi");
}
