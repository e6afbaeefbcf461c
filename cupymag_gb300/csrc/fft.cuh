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
// precision on the host (the kernels keep a copy in shared memory).  Radices
// 2, 3, 4 and 8 run as butterflies (one work item per j: the pre-twiddles,
// then the R-point DFT with constant factors); any other radix (5, 7 and
// larger primes) as one work item per output with R complex multiply-adds.
// Powers of two go as radix 8, then 4 and 2, so every line length works.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cpm {

constexpr int kFftMaxPass = 16;

// One axis: its length, radices and twiddle table (device memory, n float2; the kernels copy it to
// shared memory).
struct FftAxis {
  int n, npass;
  int radix[kFftMaxPass];
  const float2 *tw;
};

// floor(e / d) for 0 <= e < 2^22 and inv = the correctly rounded 1/d: (e + 1/2) / d lies at
// least 1/(2d) from every integer, and the float product's relative error (below 2^-23) stays
// under that margin for these e, so the truncation is exact.  A handful of instructions where an
// integer division by a runtime value takes a few dozen.
__device__ __forceinline__ int qdiv(int e, float inv) { return __float2int_rz(((float)e + 0.5f) * inv); }

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
__device__ __forceinline__ void butterfly<8>(float2 (&v)[8], bool inverse) {
  // radix-2 split: E = DFT4(v0, v2, v4, v6), O = DFT4(v1, v3, v5, v7),
  // X[q] = E[q] + W8^q O[q], X[q + 4] = E[q] - W8^q O[q], W8 = exp(-i pi / 4) (inverse: conjugate)
  float2 e[4] = {v[0], v[2], v[4], v[6]};
  float2 o[4] = {v[1], v[3], v[5], v[7]};
  butterfly<4>(e, inverse);
  butterfly<4>(o, inverse);
  constexpr float h = 0.70710678118654752f;  // sqrt(2) / 2
  const float sg = inverse ? 1.0f : -1.0f;    // sign of the imaginary part of W8
  // W8^1 = h (1 + sg i), W8^2 = sg i, W8^3 = h (-1 + sg i)
  const float2 o1 = make_float2(h * (o[1].x - sg * o[1].y), h * (o[1].y + sg * o[1].x));
  const float2 o2 = make_float2(-sg * o[2].y, sg * o[2].x);
  const float2 o3 = make_float2(h * (-o[3].x - sg * o[3].y), h * (-o[3].y + sg * o[3].x));
  v[0] = make_float2(e[0].x + o[0].x, e[0].y + o[0].y);
  v[4] = make_float2(e[0].x - o[0].x, e[0].y - o[0].y);
  v[1] = make_float2(e[1].x + o1.x, e[1].y + o1.y);
  v[5] = make_float2(e[1].x - o1.x, e[1].y - o1.y);
  v[2] = make_float2(e[2].x + o2.x, e[2].y + o2.y);
  v[6] = make_float2(e[2].x - o2.x, e[2].y - o2.y);
  v[3] = make_float2(e[3].x + o3.x, e[3].y + o3.y);
  v[7] = make_float2(e[3].x - o3.x, e[3].y - o3.y);
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

// Walks the work items e = tid, tid + blockDim, ... of a rows x cols grid (cols varying fastest)
// as (row, col) pairs, stepping without a division per item: one block-wide step advances
// row by blockDim / cols and col by blockDim % cols (with one carry).
struct Walk2 {
  int row, col, drow, dcol, cols;
  __device__ __forceinline__ Walk2(int cols_, float inv_cols) : cols(cols_) {
    row = qdiv(threadIdx.x, inv_cols);
    col = threadIdx.x - row * cols;
    drow = qdiv(blockDim.x, inv_cols);
    dcol = blockDim.x - drow * cols;
  }
  __device__ __forceinline__ void next() {
    col += dcol;
    row += drow;
    if (col >= cols) {
      col -= cols;
      ++row;
    }
  }
};

// One Stockham pass of radix R (2, 3, 4 or 8) over `lines` lines: every work item is one
// butterfly j of one line, with the pre-twiddles W^(r (j % Ns) n / (Ns R)) (exponents below n,
// no wrap).  The items go line-fastest: the lanes of a warp take consecutive lines at the same j,
// so their shared-memory loads and stores stride by the odd line stride (no bank conflicts) and
// their twiddles are one broadcast address.
template <int R, bool INV>
__device__ __forceinline__ void stockham_pass(const float2 *__restrict__ src, float2 *__restrict__ dst, int n,
                                              int ld, int lines, int Ns, const float2 *__restrict__ tw) {
  const int m = n / R;
  const int span = n / (Ns * R);
  const float inv_ns = __frcp_rn((float)Ns);
  for (Walk2 w(lines, __frcp_rn((float)lines)); w.row < m; w.next()) {
    const int j = w.row, line = w.col;
    const int jd = qdiv(j, inv_ns);
    const int k = j - jd * Ns;
    const float2 *in = src + line * ld + j;
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[r * m];
    if (k != 0) {
      const int step = k * span;
      int t = step;
#pragma unroll
      for (int r = 1; r < R; ++r, t += step) {
        float2 wv = tw[t];
        if (INV) wv.y = -wv.y;
        v[r] = cmul(v[r], wv);
      }
    }
    butterfly<R>(v, INV);
    float2 *out = dst + line * ld + jd * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) out[r * Ns] = v[r];
  }
}

// Any radix R: every work item is one output (j, q) of one line, R complex multiply-adds
// (line-fastest as above).
template <bool INV>
__device__ __forceinline__ void stockham_pass_any(const float2 *__restrict__ src, float2 *__restrict__ dst, int n,
                                                  int ld, int lines, int Ns, int R, const float2 *__restrict__ tw) {
  const int m = n / R;
  const int span = n / (Ns * R);
  const float inv_m = __frcp_rn((float)m), inv_ns = __frcp_rn((float)Ns);
  for (Walk2 w(lines, __frcp_rn((float)lines)); w.row < n; w.next()) {
    const int o = w.row, line = w.col;
    const int q = qdiv(o, inv_m);
    const int j = o - q * m;
    const int jd = qdiv(j, inv_ns);
    const int k = j - jd * Ns;
    const int bt = k * span + q * m;  // twiddle exponent of input r is r * bt (mod n); bt < n
    const float2 *in = src + line * ld + j;
    float2 acc = make_float2(0.0f, 0.0f);
    int t = 0;
    for (int r = 0; r < R; ++r) {
      float2 wv = tw[t];
      if (INV) wv.y = -wv.y;
      const float2 v = in[r * m];
      acc.x = fmaf(v.x, wv.x, fmaf(-v.y, wv.y, acc.x));
      acc.y = fmaf(v.x, wv.y, fmaf(v.y, wv.x, acc.y));
      t += bt;
      if (t >= n) t -= n;
    }
    dst[line * ld + jd * Ns * R + k + q * Ns] = acc;
  }
}

// Shared-memory stride of a line of length n: odd, so that threads walking
// across lines (the tile loads of the y and x passes) hit different banks.
__host__ __device__ __forceinline__ int line_stride(int n) { return n | 1; }

// 1D DFTs of `lines` lines of length ax.n stored at buf[line * line_stride(n) + i]
// (shared memory), with scratch of the same size; returns the buffer holding
// the result.  tw: the axis' twiddle table (shared memory).  INV: conjugate
// twiddles, no scaling.  All threads of the block take part; ends with a block
// barrier.
template <bool INV>
__device__ __forceinline__ float2 *dft_lines(float2 *buf, float2 *scratch, const FftAxis &ax, const float2 *tw,
                                             int lines) {
  const int n = ax.n;
  const int ld = line_stride(n);
  float2 *src = buf, *dst = scratch;
  int Ns = 1;
  for (int s = 0; s < ax.npass; ++s) {
    const int R = ax.radix[s];
    if (R == 8) stockham_pass<8, INV>(src, dst, n, ld, lines, Ns, tw);
    else if (R == 4) stockham_pass<4, INV>(src, dst, n, ld, lines, Ns, tw);
    else if (R == 2) stockham_pass<2, INV>(src, dst, n, ld, lines, Ns, tw);
    else if (R == 3) stockham_pass<3, INV>(src, dst, n, ld, lines, Ns, tw);
    else stockham_pass_any<INV>(src, dst, n, ld, lines, Ns, R, tw);
    __syncthreads();
    float2 *tmp = src;
    src = dst;
    dst = tmp;
    Ns *= R;
  }
  return src;
}

}  // namespace cpm
