// Device-side COO -> CSR summation for unstructured meshes (sm_103a).
//
// The reference builds every operator as COO triplets (one per element
// entry) and lets cupyx sum the duplicates when it converts to CSR
// (cupymag/utils/final_assembly.py:160-205).  Here the host side sorts the
// keys row * ncols + col with a stable sort (so duplicates keep their element
// order) and this kernel adds each run of equal keys in that order: the
// result is a deterministic function of the element order, whatever the
// launch configuration.
#include "cpm_common.cuh"

namespace cpm {

__global__ void segment_sum_kernel(const double *__restrict__ vals, const int64_t *__restrict__ start,
                                   int64_t nseg, double *__restrict__ out) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nseg;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = start[s + 1];
    double acc = 0.0;
    for (int64_t i = start[s]; i < e; ++i) acc += vals[i];
    out[s] = acc;
  }
}

}  // namespace cpm

extern "C" int cpm_coo_segment_sum(const double *vals_sorted, const int64_t *seg_start, int64_t nseg, double *out,
                                   void *stream) {
  using namespace cpm;
  if (nseg < 0 || (nseg > 0 && (!vals_sorted || !seg_start || !out))) {
    set_error("cpm_coo_segment_sum: bad arguments");
    return CPM_BAD_ARG;
  }
  if (nseg == 0) return CPM_OK;
  int64_t g = (nseg + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 16;
  if (g > cap) g = cap;
  segment_sum_kernel<<<(unsigned)g, 256, 0, (cudaStream_t)stream>>>(vals_sorted, seg_start, nseg, out);
  return check_launch("cpm_coo_segment_sum");
}
