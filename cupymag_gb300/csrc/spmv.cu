// CSR sparse matrix-vector products used by the LLG step (sm_103a).
//
// The reference applies every operator with cupyx's CSR `A @ x`
// (cuSPARSE).  Here tiles of rows are staged into shared memory and summed by
// small thread groups with one FP64 FMA per non-zero (csr_tile.cuh); the sum
// order is fixed, so results are deterministic.  Matrices of the hex grid have
// 27 (scalar), 81 (elastic stiffness) or 162 (elastic coupling) non-zeros per
// row.
#include <algorithm>

#include "cpm_common.cuh"
#include "csr_tile.cuh"

namespace cpm {

constexpr int kSpThreads = 256;

// Staged thread-group-per-row kernel of the three-matrix product (see csr_tile.cuh): one FP64 FMA per
// non-zero and value, tiles of rows handed out grid-stride.
// The shared-memory attribute is a per-device setting, so it is set on every call (cheap) and the
// occupancy is queried with it.
static int tile_grid(int64_t tiles, const void *fn, int smem) {
  int occ = 0;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kSpThreads, smem);
  if (occ < 1) occ = 1;
  int64_t g = (int64_t)occ * sm_count();
  if (g > tiles) g = tiles;
  return (int)(g < 1 ? 1 : g);
}

// Rows read in place by groups of G lanes (G = 4 for rows of 16 or more entries, else 2): the group's
// lanes take entries k = start + sub, start + sub + G, ..., so each load instruction of a warp fills
// whole 32-byte sectors of 32 / G rows (no staging, no shared memory, full occupancy), and the row sum
// costs log2(G) FP64 shuffle-adds per lane.  On GB300 the FP64 pipe, not HBM, bounds a CSR SpMV (one
// FMA per 12-byte non-zero at about 2 FP64 operations per clock per SM); the 16-lane groups of the
// staged kernel spent 64 lane-slots of FP64 adds per 162-entry row (28 % of the FP64 work), these 8.
template <typename IT, int NV, int G>
__global__ void __launch_bounds__(kSpThreads) spmv_rows_kernel(int64_t rows, const IT *__restrict__ rp,
                                                               const int *__restrict__ ci,
                                                               const double *__restrict__ av,
                                                               const double *__restrict__ x, double *__restrict__ y,
                                                               double alpha) {
  // the row loop is uniform over the CTA, so every lane reaches the shuffles (rows past the end sum zero)
  const int64_t per_cta = blockDim.x / G;
  for (int64_t base = (int64_t)blockIdx.x * per_cta; base < rows; base += (int64_t)gridDim.x * per_cta) {
    const int64_t row = base + threadIdx.x / G;
    double acc[NV];
    group_row<NV, G, IT>(rp, ci, av, x, row, rows, acc);
    if (row < rows && threadIdx.x % G == 0)
#pragma unroll
      for (int j = 0; j < NV; ++j) y[row * NV + j] = alpha * acc[j];
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
  // rows of 16 or more entries: groups of 4 lanes; shorter rows: pairs.  Five CTAs per SM: the rows in
  // flight then span a few tens of MB of the matrix; measured on GB300 (128^3 F_el, A_el, A_demag; 64^3
  // F_el, A_el) 0.63 / 0.60 / 0.64 / 0.75 / 0.69 of HBM, against 0.54 / 0.51 / 0.63 / 0.71 / 0.68 with
  // sixteen (more rows in flight, less reuse of the gathered vector) and 0.42 / 0.39 with two
  const int G = max_row(A) >= 16 ? 4 : 2;
  const int64_t want = (A->rows * G + kSpThreads - 1) / kSpThreads;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count() * 5));
#define CPM_SP1(IT, NV)                                                                                          \
  do {                                                                                                           \
    if (G == 4)                                                                                                  \
      spmv_rows_kernel<IT, NV, 4><<<grid, kSpThreads, 0, st>>>(A->rows, (const IT *)A->indptr, A->indices,       \
                                                               A->vals, x, y, alpha);                            \
    else                                                                                                         \
      spmv_rows_kernel<IT, NV, 2><<<grid, kSpThreads, 0, st>>>(A->rows, (const IT *)A->indptr, A->indices,       \
                                                               A->vals, x, y, alpha);                            \
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
