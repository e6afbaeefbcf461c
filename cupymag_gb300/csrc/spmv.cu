// CSR sparse matrix-vector products used by the LLG step (sm_103a).
//
// The reference applies every operator with cupyx's CSR `A @ x`
// (cuSPARSE).  Here tiles of rows are staged into shared memory and summed by
// small thread groups with one FP64 FMA per non-zero (csr_tile.cuh); the sum
// order is fixed, so results are deterministic.  Matrices of the hex grid have
// 27 (scalar), 81 (elastic stiffness) or 162 (elastic coupling) non-zeros per
// row.
#include "cpm_common.cuh"
#include "csr_tile.cuh"

namespace cpm {

constexpr int kSpThreads = 256;

// Staged thread-group-per-row kernels (see csr_tile.cuh): one FP64 FMA per
// non-zero and value, tiles of rows handed out grid-stride.
static int tile_grid(int64_t tiles, const void *fn, int smem) {
  static int occ_cache[8] = {};
  static const void *fn_cache[8] = {};
  int occ = 0;
  for (int i = 0; i < 8; ++i)
    if (fn_cache[i] == fn) occ = occ_cache[i];
  if (occ == 0) {
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kSpThreads, smem);
    if (occ < 1) occ = 1;
    for (int i = 0; i < 8; ++i)
      if (fn_cache[i] == nullptr) {
        fn_cache[i] = fn;
        occ_cache[i] = occ;
        break;
      }
  }
  int64_t g = (int64_t)occ * sm_count();
  if (g > tiles) g = tiles;
  return (int)(g < 1 ? 1 : g);
}

template <typename IT, int NV>
__global__ void __launch_bounds__(kSpThreads) spmv_kernel(int64_t rows, const IT *__restrict__ rp,
                                                          const int *__restrict__ ci, const double *__restrict__ av,
                                                          const double *__restrict__ x, double *__restrict__ y,
                                                          double alpha, int G) {
  extern __shared__ __align__(16) unsigned char smem[];
  const MultiTile<1> t = multi_tile_smem<1>(smem);
  const int R = kSpThreads / G;
  const double *vals[1] = {av};
  const int64_t ntiles = (rows + R - 1) / R;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t t0 = tile * R, t1 = min(rows, t0 + R);
    double acc[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) acc[j] = 0.0;
    const int64_t row = visit_tile<1, IT>(rp, ci, vals, t0, t1, G, t, [&](const double (&a)[1], int64_t c) {
#pragma unroll
      for (int j = 0; j < NV; ++j) acc[j] = fma(a[0], __ldg(x + c * NV + j), acc[j]);
    });
#pragma unroll
    for (int j = 0; j < NV; ++j) acc[j] = group_sum(acc[j], G);
    if (row >= 0 && (threadIdx.x % G) == 0) {
#pragma unroll
      for (int j = 0; j < NV; ++j) y[row * NV + j] = alpha * acc[j];
    }
    __syncthreads();
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
                                                           int64_t pin, int G) {
  extern __shared__ __align__(16) unsigned char smem[];
  const MultiTile<3> t = multi_tile_smem<3>(smem);
  const int R = kSpThreads / G;
  const double *vals[3] = {ax, ay, az};
  double sh0 = 0.0, sh1 = 0.0, sh2 = 0.0;
  if (MODE == 1 && shift) {
    sh0 = shift[0];
    sh1 = shift[1];
    sh2 = shift[2];
  }
  const int64_t ntiles = (rows + R - 1) / R;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t t0 = tile * R, t1 = min(rows, t0 + R);
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    const int64_t row = visit_tile<3, IT>(rp, ci, vals, t0, t1, G, t, [&](const double (&a)[3], int64_t c) {
      if (MODE == 0) {
        const double xv = __ldg(x + c);
        a0 = fma(a[0], xv, a0);
        a1 = fma(a[1], xv, a1);
        a2 = fma(a[2], xv, a2);
      } else {
        a0 = fma(a[0], __ldg(x + 3 * c + 0) - sh0, a0);
        a1 = fma(a[1], __ldg(x + 3 * c + 1) - sh1, a1);
        a2 = fma(a[2], __ldg(x + 3 * c + 2) - sh2, a2);
      }
    });
    a0 = group_sum(a0, G);
    a1 = group_sum(a1, G);
    a2 = group_sum(a2, G);
    if (row >= 0 && (threadIdx.x % G) == 0) {
      if (MODE == 0) {
        y[3 * row + 0] = alpha * a0;
        y[3 * row + 1] = alpha * a1;
        y[3 * row + 2] = alpha * a2;
      } else {
        // (Fx m~x + Fy m~y) + Fz m~z, then the sign (Micromagnetics.py:166)
        y[row] = (row == pin) ? 0.0 : alpha * ((a0 + a1) + a2);
      }
    }
    __syncthreads();
  }
}

static int64_t max_row(const cpm_csr *A) {
  return A->max_row_nnz > 0 ? A->max_row_nnz : (A->nnz + A->rows - 1) / (A->rows > 0 ? A->rows : 1);
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
  const int G = group_size_cap(max_row(A), kSpThreads, multi_cap<1>());
  const int64_t tiles = (A->rows + kSpThreads / G - 1) / (kSpThreads / G);
#define CPM_SP1(IT, NV)                                                                                          \
  do {                                                                                                           \
    const void *fn = (const void *)spmv_kernel<IT, NV>;                                                          \
    spmv_kernel<IT, NV><<<tile_grid(tiles, fn, multi_smem<1>()), kSpThreads, multi_smem<1>(), st>>>(           \
        A->rows, (const IT *)A->indptr, A->indices, A->vals, x, y, alpha, G);                                    \
  } while (0)
  if (A->indptr_is64) {
    if (nvec == 1) CPM_SP1(int64_t, 1); else CPM_SP1(int64_t, 3);
  } else {
    if (nvec == 1) CPM_SP1(int32_t, 1); else CPM_SP1(int32_t, 3);
  }
#undef CPM_SP1
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
  const int G = group_size_cap(max_row(A), kSpThreads, multi_cap<3>());
  const int64_t tiles = (A->rows + kSpThreads / G - 1) / (kSpThreads / G);
#define CPM_SP3(IT, M)                                                                                         \
  do {                                                                                                         \
    const void *fn = (const void *)spmv3_kernel<IT, M>;                                                        \
    spmv3_kernel<IT, M><<<tile_grid(tiles, fn, multi_smem<3>()), kSpThreads, multi_smem<3>(), st>>>(         \
        A->rows, (const IT *)A->indptr, A->indices, A->vals, vals_y, vals_z, x, y, alpha, shift, pin, G);      \
  } while (0)
  if (A->indptr_is64) {
    if (mode == 0) CPM_SP3(int64_t, 0); else CPM_SP3(int64_t, 1);
  } else {
    if (mode == 0) CPM_SP3(int32_t, 0); else CPM_SP3(int32_t, 1);
  }
#undef CPM_SP3
  return check_launch("cpm_spmv_csr_multi");
}
