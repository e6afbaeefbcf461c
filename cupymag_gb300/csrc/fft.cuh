// Mixed-radix discrete Fourier transforms of short lines held in shared memory (sm_103a).
//
// The circulant preconditioner of csrc/fftcg.cu diagonalises a periodic
// stencil operator with 3D DFTs of the grid, done as one pass of 1D DFTs per
// axis.  Each pass loads a tile of lines (a line is at most a few hundred
// points) into shared memory, transforms them there and writes them back.
//
// A line of length n = R_1 R_2 ... R_m is transformed by Stockham auto-sort
// passes (one per radix R, alternating between two shared buffers; Govindaraju
// et al., "High performance discrete Fourier transforms on graphics
// processors", SC 2008).  With Ns the product of the radices done so far, the
// pass computes for every output index
//     out[(j / Ns) Ns R + (j % Ns) + q Ns] = sum_r in[j + r n / R] W^(r ((j % Ns) n / (Ns R) + q n / R))
// with W = exp(-2 pi i / n) (its conjugate for the inverse transform), j <
// n / R, q < R.  Every output is one work item of R complex multiply-adds with
// twiddles from a table of W^t, t < n, computed in double precision on the
// host; a radix is any factor of n (powers of two go as radix 4, a left-over 2
// as radix 2, then 3, 5, 7 and any larger prime), so every line length works.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cpm {

constexpr int kFftMaxPass = 16;

// One axis: its length, radices and twiddle table (device, n float2).
struct FftAxis {
  int n, npass;
  int radix[kFftMaxPass];
  const float2 *tw;
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// 1D DFTs of `lines` lines of length ax.n stored at buf[line * ax.n + i] (shared
// memory), with scratch of the same size; returns the buffer holding the
// result.  inverse: conjugate twiddles, no scaling.  All threads of the block
// take part; ends with a block barrier.
__device__ __forceinline__ float2 *dft_lines(float2 *buf, float2 *scratch, const FftAxis &ax, int lines,
                                             bool inverse) {
  const int n = ax.n;
  float2 *src = buf, *dst = scratch;
  int Ns = 1;
  for (int s = 0; s < ax.npass; ++s) {
    const int R = ax.radix[s];
    const int m = n / R;
    const int span = n / (Ns * R);
    const int total = lines * n;
    for (int w = threadIdx.x; w < total; w += blockDim.x) {
      const int line = w / n;
      const int o = w - line * n;  // work item: (j, q) with j = o % m, q = o / m
      const int q = o / m;
      const int j = o - q * m;
      const int k = j % Ns;
      const int bt = k * span + q * m;  // twiddle exponent of input r is r * bt (mod n)
      const float2 *in = src + line * n + j;
      float2 acc = make_float2(0.0f, 0.0f);
      int t = 0;
      for (int r = 0; r < R; ++r) {
        float2 wv = __ldg(ax.tw + t);
        if (inverse) wv.y = -wv.y;
        const float2 v = in[r * m];
        acc.x = fmaf(v.x, wv.x, fmaf(-v.y, wv.y, acc.x));
        acc.y = fmaf(v.x, wv.y, fmaf(v.y, wv.x, acc.y));
        t += bt;  // bt < n, so one subtraction keeps t < n
        if (t >= n) t -= n;
      }
      dst[line * n + (j / Ns) * Ns * R + k + q * Ns] = acc;
    }
    __syncthreads();
    float2 *tmp = src;
    src = dst;
    dst = tmp;
    Ns *= R;
  }
  return src;
}

}  // namespace cpm
