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
// n / R, q < R, with twiddles from a table of W^t, t < n, computed in double
// precision on the host.  Radices 2, 3 and 4 run as butterflies (one work item
// per j: the pre-twiddles, then the R-point DFT with constant factors); any
// other radix (5, 7 and larger primes) as one work item per output with R
// complex multiply-adds.  Powers of two go as radix 4 and a left-over 2, so
// every line length works.
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

// In-place R-point DFT of v (forward: exp(-2 pi i qr / R); inverse: conjugate).
template <int R>
__device__ __forceinline__ void butterfly(float2 (&v)[R], bool inverse);

template <>
__device__ __forceinline__ void butterfly<2>(float2 (&v)[2], bool) {
  const float2 a = v[0], b = v[1];
  v[0] = make_float2(a.x + b.x, a.y + b.y);
  v[1] = make_float2(a.x - b.x, a.y - b.y);
}

template <>
__device__ __forceinline__ void butterfly<4>(float2 (&v)[4], bool inverse) {
  const float2 a0 = make_float2(v[0].x + v[2].x, v[0].y + v[2].y);
  const float2 a1 = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
  const float2 a2 = make_float2(v[1].x + v[3].x, v[1].y + v[3].y);
  const float2 d = make_float2(v[1].x - v[3].x, v[1].y - v[3].y);
  // (v1 - v3) times -i (forward) or +i (inverse)
  const float2 a3 = inverse ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
  v[0] = make_float2(a0.x + a2.x, a0.y + a2.y);
  v[2] = make_float2(a0.x - a2.x, a0.y - a2.y);
  v[1] = make_float2(a1.x + a3.x, a1.y + a3.y);
  v[3] = make_float2(a1.x - a3.x, a1.y - a3.y);
}

template <>
__device__ __forceinline__ void butterfly<3>(float2 (&v)[3], bool inverse) {
  // W = exp(-2 pi i / 3) = c - i s with c = -1/2, s = sqrt(3)/2 (inverse: s -> -s)
  const float s = inverse ? -0.8660254037844386f : 0.8660254037844386f;
  const float2 sum = make_float2(v[1].x + v[2].x, v[1].y + v[2].y);
  const float2 dif = make_float2(v[1].x - v[2].x, v[1].y - v[2].y);
  const float2 t = make_float2(v[0].x - 0.5f * sum.x, v[0].y - 0.5f * sum.y);
  // -i s (v1 - v2) = (s dif.y, -s dif.x)
  v[0] = make_float2(v[0].x + sum.x, v[0].y + sum.y);
  v[1] = make_float2(t.x + s * dif.y, t.y - s * dif.x);
  v[2] = make_float2(t.x - s * dif.y, t.y + s * dif.x);
}

// One Stockham pass of radix R (2, 3 or 4): every work item is one butterfly j of a
// line, with the pre-twiddles W^(r (j % Ns) n / (Ns R)) (exponents below n, no wrap).
template <int R>
__device__ __forceinline__ void stockham_pass(const float2 *src, float2 *dst, int n, int ld, int lines, int Ns,
                                              const float2 *tw, bool inverse) {
  const int m = n / R;
  const int span = n / (Ns * R);
  const int total = lines * m;
  for (int b = threadIdx.x; b < total; b += blockDim.x) {
    const int line = b / m;
    const int j = b - line * m;
    const int jd = j / Ns;
    const int k = j - jd * Ns;
    const float2 *in = src + line * ld + j;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[r * m];
    if (k != 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 w = __ldg(tw + r * k * span);
        if (inverse) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    butterfly<R>(v, inverse);
    float2 *out = dst + line * ld + jd * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) out[r * Ns] = v[r];
  }
}

// Any radix R: every work item is one output (j, q), R complex multiply-adds.
__device__ __forceinline__ void stockham_pass_any(const float2 *src, float2 *dst, int n, int ld, int lines, int Ns,
                                                  int R, const float2 *tw, bool inverse) {
  const int m = n / R;
  const int span = n / (Ns * R);
  const int total = lines * n;
  for (int w = threadIdx.x; w < total; w += blockDim.x) {
    const int line = w / n;
    const int o = w - line * n;
    const int q = o / m;
    const int j = o - q * m;
    const int k = j % Ns;
    const int bt = k * span + q * m;  // twiddle exponent of input r is r * bt (mod n); bt < n
    const float2 *in = src + line * ld + j;
    float2 acc = make_float2(0.0f, 0.0f);
    int t = 0;
    for (int r = 0; r < R; ++r) {
      float2 wv = __ldg(tw + t);
      if (inverse) wv.y = -wv.y;
      const float2 v = in[r * m];
      acc.x = fmaf(v.x, wv.x, fmaf(-v.y, wv.y, acc.x));
      acc.y = fmaf(v.x, wv.y, fmaf(v.y, wv.x, acc.y));
      t += bt;
      if (t >= n) t -= n;
    }
    dst[line * ld + (j / Ns) * Ns * R + k + q * Ns] = acc;
  }
}

// Shared-memory stride of a line of length n: odd, so that threads walking
// across lines (the tile loads of the y and x passes) hit different banks.
__host__ __device__ __forceinline__ int line_stride(int n) { return n | 1; }

// 1D DFTs of `lines` lines of length ax.n stored at buf[line * line_stride(n) + i]
// (shared memory), with scratch of the same size; returns the buffer holding
// the result.  inverse: conjugate twiddles, no scaling.  All threads of the
// block take part; ends with a block barrier.
__device__ __forceinline__ float2 *dft_lines(float2 *buf, float2 *scratch, const FftAxis &ax, int lines,
                                             bool inverse) {
  const int n = ax.n;
  const int ld = line_stride(n);
  float2 *src = buf, *dst = scratch;
  int Ns = 1;
  for (int s = 0; s < ax.npass; ++s) {
    const int R = ax.radix[s];
    if (R == 4) stockham_pass<4>(src, dst, n, ld, lines, Ns, ax.tw, inverse);
    else if (R == 2) stockham_pass<2>(src, dst, n, ld, lines, Ns, ax.tw, inverse);
    else if (R == 3) stockham_pass<3>(src, dst, n, ld, lines, Ns, ax.tw, inverse);
    else stockham_pass_any(src, dst, n, ld, lines, Ns, R, ax.tw, inverse);
    __syncthreads();
    float2 *tmp = src;
    src = dst;
    dst = tmp;
    Ns *= R;
  }
  return src;
}

}  // namespace cpm
