// FFT solves of the elastic and demag operators inside FP64 refinement (sm_103a).
//
// On the periodic hex grid the elastic operator A_el and the demag operator
// A_demag are block-circulant stencils except for the anchor at DOF 0, whose
// rows and columns the reference replaces by the identity
// (cupymag/physics/assemble_demag.py:307-341, assemble_elasticity.py:461-527).
// The 3D DFT diagonalises the circulant part C: per wave vector k a 3x3 (or
// 1x1) real symmetric symbol C^(k) = sum_d c_d cos(theta_k . d).
//
// Both forms are the refinement form of the cupyx-semantics solve_cg
// (cupymag/solvers/linear_solvers.py:59-74) with the same stopping test on the
// FP64 residual: an outer loop computes t = b - A64 x in FP64 and stops when
// ||t|| <= tol ||b||.  The whole solve is one persistent cooperative launch;
// every grid barrier is bounded (GridBarrier).
//  * Direct refinement (the default where the plan has an anchor): A e = t is
//    solved exactly by one FFT apply of C's pseudo-inverse on t plus the
//    anchor's column at its 26 neighbours (every component summed to zero),
//    and a translation that sets the anchored values (anchor_rhs); x += e.
//    FP32 gives about 5 digits per step: two steps per 128^3 solve.  A cold
//    start's first residual is b itself (x = 0, no product); a warm start from
//    the x of a valid residual carry takes (b - b_carry) + t_carry instead of a
//    product (cpm_cg_opts.carry_*).
//  * Preconditioned CG (CPM_CG_FORM_FFT_PCG, and plans without an anchor):
//    M = C'^-1, with C' = C except C'^(0) = sigma I (sigma the operator's
//    diagonal), is an SPD preconditioner with M A = I + (rank <= 9); FP32
//    preconditioned CG on A e = t from e = 0 runs until its residual has
//    dropped by inner_tol (default 1e-4), then x += e.  Per inner iteration:
//    z = M r with r.z; p = z + beta p; q = A32 p with p.q; d += alpha p,
//    r -= alpha q with r.r.
//
// z = M r has two layouts of the spectrum:
//  * slab (the default where it fits in shared memory): r is real, so along z
//    only the nz/2 + 1 non-negative frequencies are kept (the others are the
//    conjugates).  Pass 1 takes one x-plane of one component per CTA step:
//    the real z lines two at a time as one complex DFT (lines 2p + i 2p+1),
//    split into the two half spectra, then the DFT along y of every kz column,
//    all in shared memory, one read of r and one write of the half spectrum.
//    Pass 2 takes tiles of (kz, y) columns of all components: DFT along x,
//    the 3x3 (1x1) symbol solve, inverse DFT along x.  Pass 3 undoes pass 1
//    (inverse y, the two half spectra joined into one complex line, inverse
//    z) and writes z with the partial of r.z.  Three passes, two grid
//    barriers plus the r.z sum, half the complex traffic.
//  * five passes over the full complex field (grids whose x-plane does not fit
//    in shared memory): DFT along z, y, x with the symbol solve and the
//    inverse along x in one tile, inverse along y, inverse along z.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fft.cuh"
#include "stencil_ops.cuh"

namespace cpm {

constexpr int kFftTile = 4096;  // five-pass layout: complex values per tile buffer (two buffers per CTA)
// slab layout: the largest dynamic shared memory of a CTA (two regions and the twiddle tables),
// under the 227 KB of an SM with the kernel's static reductions beside it
constexpr size_t kSlabSmemMax = 220 * 1024;

// Threads per CTA and resident CTAs per SM of the solve kernel, per layout.
template <int LAYOUT>
struct FftShape;
template <>
struct FftShape<CPM_FFT_LAYOUT_SLAB> {
  static constexpr int threads = 512, blocks = 1;
};
template <>
struct FftShape<CPM_FFT_LAYOUT_PASSES> {
  static constexpr int threads = 256, blocks = 2;
};

struct FftGrid {
  int nx, ny, nz, n, nc;
  int layout;
  FftAxis ax, ay, az;
  // inverse symbol per wave vector: nc == 1: 1 float; nc == 3: xx yy zz xy yz xz.
  // five passes: wave vector (i, j, k) at ((i ny + j) nz + k), the 6 values together;
  // slab: (i, kz, j) at (i h + kz) ny + j, one plane of nx h ny values per entry.
  const float *sym;
  float2 *C;         // complex field: nc * n (five passes) or nc * nx * h * ny (slab, [c][i][kz][j])
  int lz, kty, ktx;  // five passes: lines per tile of the z, y and x passes
  int h, pc, reg;    // slab: nz / 2 + 1, (kz, y) columns per x tile, complex values per shared region
};

// Complex values of one shared-memory region.
__host__ __device__ __forceinline__ int fft_region(const FftGrid &g) {
  return g.layout == CPM_FFT_LAYOUT_SLAB ? g.reg : kFftTile;
}

// Dynamic shared memory of a pass or solve CTA: two regions and the twiddle tables of the three axes.
static size_t fft_smem_bytes(const FftGrid &g) {
  return sizeof(float2) * (2 * (size_t)fft_region(g) + g.nx + g.ny + g.nz);
}

// Copy the three twiddle tables into shared memory (behind the two regions); ends with a block barrier.
__device__ __forceinline__ void load_twiddles(const FftGrid &g, float2 *fsm, const float2 *&twx,
                                              const float2 *&twy, const float2 *&twz) {
  float2 *t = fsm + 2 * fft_region(g);
  for (int e = threadIdx.x; e < g.nx; e += blockDim.x) t[e] = g.ax.tw[e];
  for (int e = threadIdx.x; e < g.ny; e += blockDim.x) t[g.nx + e] = g.ay.tw[e];
  for (int e = threadIdx.x; e < g.nz; e += blockDim.x) t[g.nx + g.ny + e] = g.az.tw[e];
  twx = t;
  twy = t + g.nx;
  twz = t + g.nx + g.ny;
  __syncthreads();
}

// Symbol solve of one wave vector: the nc values v[c] (shared memory, stride cs) times the
// inverse symbol at index kidx (plane stride ps between the 6 entries; 1 for the interleaved form
// with kidx already scaled by 6).
__device__ __forceinline__ void symbol_solve(const float *sym, int64_t kidx, int64_t ps, int nc, float2 *v,
                                             int cs) {
  if (nc == 1) {
    const float w = __ldg(sym + kidx);
    v->x *= w;
    v->y *= w;
    return;
  }
  const float mxx = __ldg(sym + kidx), myy = __ldg(sym + kidx + ps), mzz = __ldg(sym + kidx + 2 * ps);
  const float mxy = __ldg(sym + kidx + 3 * ps), myz = __ldg(sym + kidx + 4 * ps), mxz = __ldg(sym + kidx + 5 * ps);
  float2 &a = v[0];
  float2 &b = v[cs];
  float2 &d = v[2 * cs];
  const float2 va = a, vb = b, vd = d;
  a = make_float2(mxx * va.x + mxy * vb.x + mxz * vd.x, mxx * va.y + mxy * vb.y + mxz * vd.y);
  b = make_float2(mxy * va.x + myy * vb.x + myz * vd.x, mxy * va.y + myy * vb.y + myz * vd.y);
  d = make_float2(mxz * va.x + myz * vb.x + mzz * vd.x, mxz * va.y + myz * vb.y + mzz * vd.y);
}

// ---------------------------------------------------------------- slab layout
// Pass 1, per (component c, x-plane i): real z lines -> half spectra along z -> DFT along y -> C.
__device__ void slab_fwd(const FftGrid &g, const float *__restrict__ r, float2 *R0, float2 *R1,
                         const float2 *twy, const float2 *twz) {
  const int ny = g.ny, nz = g.nz, h = g.h, P = (ny + 1) >> 1;
  const int ldz = line_stride(nz), ldy = line_stride(ny), Hc = h * ny;
  const float inv_nz = __frcp_rn((float)nz), inv_h = __frcp_rn((float)h), inv_ny = __frcp_rn((float)ny);
  const float inv_nx = __frcp_rn((float)g.nx);
  for (int s = blockIdx.x; s < g.nc * g.nx; s += gridDim.x) {
    const int c = qdiv(s, inv_nx), i = s - c * g.nx;
    const float *src = r + (int64_t)c * g.n + (int64_t)i * ny * nz;
    // lines 2p and 2p+1 (zero past the last line) as the real and imaginary parts of line p
    for (Walk2 w(nz, inv_nz); w.row < P; w.next()) {
      const int p = w.row, k = w.col;
      const int j = 2 * p;
      const float re = src[j * nz + k];
      const float im = j + 1 < ny ? src[(j + 1) * nz + k] : 0.0f;
      R0[p * ldz + k] = make_float2(re, im);
    }
    __syncthreads();
    float2 *Z = dft_lines<false>(R0, R1, g.az, twz, P);
    float2 *B = Z == R0 ? R1 : R0;
    // Z = A + i B' with A, B' the spectra of the two real lines: A[k] = (Z[k] + conj Z[-k]) / 2,
    // B'[k] = (Z[k] - conj Z[-k]) / 2i; kept for k < h, stored as columns B[kz][j]
    for (Walk2 w(h, inv_h); w.row < P; w.next()) {
      const int p = w.row, k = w.col;
      const float2 a = Z[p * ldz + k];
      const float2 m = Z[p * ldz + (k == 0 ? 0 : nz - k)];
      B[k * ldy + 2 * p] = make_float2(0.5f * (a.x + m.x), 0.5f * (a.y - m.y));
      if (2 * p + 1 < ny) B[k * ldy + 2 * p + 1] = make_float2(0.5f * (a.y + m.y), 0.5f * (m.x - a.x));
    }
    __syncthreads();
    const float2 *Y = dft_lines<false>(B, Z, g.ay, twy, h);
    float2 *dst = g.C + (int64_t)s * Hc;
    for (Walk2 w(ny, inv_ny); w.row < h; w.next()) dst[w.row * ny + w.col] = Y[w.row * ldy + w.col];
    __syncthreads();
  }
}

// Pass 2, per tile of pc consecutive (kz, y) columns: DFT along x of every component, the symbol
// solve per wave vector, inverse DFT along x, in place in C.
__device__ void slab_x_solve(const FftGrid &g, float2 *R0, float2 *R1, const float2 *twx) {
  const int nx = g.nx, nc = g.nc, Hc = g.h * g.ny, pc = g.pc;
  const int ldx = line_stride(nx);
  const int ntiles = (Hc + pc - 1) / pc;
  const int64_t plane = (int64_t)nx * Hc;
  const float inv_nx = __frcp_rn((float)nx);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int c0 = t * pc, pv = min(pc, Hc - c0);
    const float inv_pv = __frcp_rn((float)pv);
    const int lines = nc * pv;  // line c pv + l: component c, column c0 + l
    for (Walk2 w(pv, inv_pv); w.row < nc * nx; w.next()) {
      const int ci = w.row, l = w.col;  // ci = c nx + i
      const int c = qdiv(ci, inv_nx), i = ci - c * nx;
      R0[(c * pv + l) * ldx + i] = g.C[(int64_t)ci * Hc + c0 + l];
    }
    __syncthreads();
    float2 *spec = dft_lines<false>(R0, R1, g.ax, twx, lines);
    for (Walk2 w(pv, inv_pv); w.row < nx; w.next())
      symbol_solve(g.sym, (int64_t)w.row * Hc + c0 + w.col, plane, nc, spec + w.col * ldx + w.row, pv * ldx);
    __syncthreads();
    float2 *other = spec == R0 ? R1 : R0;
    const float2 *out = dft_lines<true>(spec, other, g.ax, twx, lines);
    for (Walk2 w(pv, inv_pv); w.row < nc * nx; w.next()) {
      const int ci = w.row, l = w.col;
      const int c = qdiv(ci, inv_nx), i = ci - c * nx;
      g.C[(int64_t)ci * Hc + c0 + l] = out[(c * pv + l) * ldx + i];
    }
    __syncthreads();
  }
}

// Pass 3, per (c, i): inverse DFT along y, the half spectra of lines 2p and 2p+1 joined as
// Z = A + i B' (A[-k] = conj A[k]), inverse DFT along z, zout = (Re, Im) / n.  Returns this
// thread's FP32 partial of r . zout (r may be NULL: no partial).
__device__ float slab_inv(const FftGrid &g, float *__restrict__ zout, const float *__restrict__ r, float2 *R0,
                          float2 *R1, const float2 *twy, const float2 *twz) {
  const int ny = g.ny, nz = g.nz, h = g.h, P = (ny + 1) >> 1;
  const int ldz = line_stride(nz), ldy = line_stride(ny), Hc = h * ny;
  const float inv_nz = __frcp_rn((float)nz), inv_ny = __frcp_rn((float)ny), inv_nx = __frcp_rn((float)g.nx);
  const float scale = 1.0f / (float)g.n;
  float acc = 0.0f;
  for (int s = blockIdx.x; s < g.nc * g.nx; s += gridDim.x) {
    const int c = qdiv(s, inv_nx), i = s - c * g.nx;
    const float2 *src = g.C + (int64_t)s * Hc;
    for (Walk2 w(ny, inv_ny); w.row < h; w.next()) R0[w.row * ldy + w.col] = src[w.row * ny + w.col];
    __syncthreads();
    float2 *Y = dft_lines<true>(R0, R1, g.ay, twy, h);
    float2 *Z = Y == R0 ? R1 : R0;
    for (Walk2 w(nz, inv_nz); w.row < P; w.next()) {
      const int p = w.row, k = w.col;
      const bool lo = k < h;
      const int kk = lo ? k : nz - k;
      const int j = 2 * p;
      float2 a = Y[kk * ldy + j];
      float2 b = j + 1 < ny ? Y[kk * ldy + j + 1] : make_float2(0.0f, 0.0f);
      if (!lo) {
        a.y = -a.y;
        b.y = -b.y;
      }
      Z[p * ldz + k] = make_float2(a.x - b.y, a.y + b.x);
    }
    __syncthreads();
    const float2 *out = dft_lines<true>(Z, Y, g.az, twz, P);
    const int64_t off = (int64_t)c * g.n + (int64_t)i * ny * nz;
    for (Walk2 w(nz, inv_nz); w.row < ny; w.next()) {
      const int j = w.row, e = j * nz + w.col;
      const float2 u = out[(j >> 1) * ldz + w.col];
      const float v = ((j & 1) ? u.y : u.x) * scale;
      zout[off + e] = v;
      if (r) acc = fmaf(r[off + e], v, acc);
    }
    __syncthreads();
  }
  return acc;
}

// ---------------------------------------------------------------- five-pass layout
// z lines of the real input (per component): forward DFT along z into C.
__device__ void pass_z_fwd(const FftGrid &g, const float *r, float2 *s0, float2 *s1, const float2 *twz) {
  const int nlines = g.nx * g.ny;
  const int per = (nlines + g.lz - 1) / g.lz;
  const int ntiles = g.nc * per;
  const int ld = line_stride(g.nz);
  const float inv_nz = __frcp_rn((float)g.nz);
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int c = tile / per, l0 = (tile - c * per) * g.lz;
    const int L = min(g.lz, nlines - l0);
    const float *src = r + (int64_t)c * g.n + (int64_t)l0 * g.nz;
    for (int e = threadIdx.x; e < L * g.nz; e += blockDim.x) {
      const int l = qdiv(e, inv_nz), k = e - l * g.nz;
      s0[l * ld + k] = make_float2(src[e], 0.0f);
    }
    __syncthreads();
    const float2 *out = dft_lines<false>(s0, s1, g.az, twz, L);
    float2 *dst = g.C + (int64_t)c * g.n + (int64_t)l0 * g.nz;
    for (int e = threadIdx.x; e < L * g.nz; e += blockDim.x) {
      const int l = qdiv(e, inv_nz), k = e - l * g.nz;
      dst[e] = out[l * ld + k];
    }
    __syncthreads();
  }
}

// y lines (tiles of kty consecutive z at fixed x), forward or inverse, in place in C.
__device__ void pass_y(const FftGrid &g, bool inverse, float2 *s0, float2 *s1, const float2 *twy) {
  const int kb = (g.nz + g.kty - 1) / g.kty;
  const int ntiles = g.nc * g.nx * kb;
  const int ld = line_stride(g.ny);
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int c = tile / (g.nx * kb);
    const int rem = tile - c * g.nx * kb;
    const int i = rem / kb, k0 = (rem - i * kb) * g.kty;
    const int kv = min(g.kty, g.nz - k0);
    float2 *base = g.C + (int64_t)c * g.n + (int64_t)i * g.ny * g.nz + k0;
    const float inv_kv = __frcp_rn((float)kv);
    for (int e = threadIdx.x; e < kv * g.ny; e += blockDim.x) {
      const int j = qdiv(e, inv_kv), kk = e - j * kv;
      s0[kk * ld + j] = base[(int64_t)j * g.nz + kk];
    }
    __syncthreads();
    const float2 *out = inverse ? dft_lines<true>(s0, s1, g.ay, twy, kv) : dft_lines<false>(s0, s1, g.ay, twy, kv);
    for (int e = threadIdx.x; e < kv * g.ny; e += blockDim.x) {
      const int j = qdiv(e, inv_kv), kk = e - j * kv;
      base[(int64_t)j * g.nz + kk] = out[kk * ld + j];
    }
    __syncthreads();
  }
}

// x lines of every component (tiles of ktx consecutive z at fixed y): forward DFT,
// u^(k) = S^-1(k) r^(k), inverse DFT, all in the tile.
__device__ void pass_x_solve(const FftGrid &g, float2 *s0, float2 *s1, const float2 *twx) {
  const int kb = (g.nz + g.ktx - 1) / g.ktx;
  const int ntiles = g.ny * kb;
  const int nc = g.nc;
  const int ld = line_stride(g.nx);
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int j = tile / kb, k0 = (tile - j * kb) * g.ktx;
    const int kv = min(g.ktx, g.nz - k0);
    const int lines = nc * kv;
    const float inv_lines = __frcp_rn((float)lines), inv_kv = __frcp_rn((float)kv);
    for (int e = threadIdx.x; e < lines * g.nx; e += blockDim.x) {
      const int i = qdiv(e, inv_lines), lr = e - i * lines;  // lr = c * kv + kk
      const int c = qdiv(lr, inv_kv), kk = lr - c * kv;
      s0[lr * ld + i] = g.C[(int64_t)c * g.n + ((int64_t)i * g.ny + j) * g.nz + k0 + kk];
    }
    __syncthreads();
    float2 *spec = dft_lines<false>(s0, s1, g.ax, twx, lines);
    for (int e = threadIdx.x; e < kv * g.nx; e += blockDim.x) {
      const int i = qdiv(e, inv_kv), kk = e - i * kv;
      const int64_t kidx = ((int64_t)i * g.ny + j) * g.nz + k0 + kk;
      symbol_solve(g.sym, nc == 1 ? kidx : 6 * kidx, 1, nc, spec + kk * ld + i, kv * ld);
    }
    __syncthreads();
    float2 *other = spec == s0 ? s1 : s0;
    const float2 *out = dft_lines<true>(spec, other, g.ax, twx, lines);
    for (int e = threadIdx.x; e < lines * g.nx; e += blockDim.x) {
      const int i = qdiv(e, inv_lines), lr = e - i * lines;
      const int c = qdiv(lr, inv_kv), kk = lr - c * kv;
      g.C[(int64_t)c * g.n + ((int64_t)i * g.ny + j) * g.nz + k0 + kk] = out[lr * ld + i];
    }
    __syncthreads();
  }
}

// Inverse DFT along z, z_out = Re / n; returns this thread's FP32 partial of r . z_out
// (r may be NULL: no partial).
__device__ float pass_z_inv(const FftGrid &g, float *zout, const float *r, float2 *s0, float2 *s1,
                            const float2 *twz) {
  const int nlines = g.nx * g.ny;
  const int per = (nlines + g.lz - 1) / g.lz;
  const int ntiles = g.nc * per;
  const float scale = 1.0f / (float)g.n;
  const int ld = line_stride(g.nz);
  const float inv_nz = __frcp_rn((float)g.nz);
  float acc = 0.0f;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int c = tile / per, l0 = (tile - c * per) * g.lz;
    const int L = min(g.lz, nlines - l0);
    const float2 *src = g.C + (int64_t)c * g.n + (int64_t)l0 * g.nz;
    for (int e = threadIdx.x; e < L * g.nz; e += blockDim.x) {
      const int l = qdiv(e, inv_nz), k = e - l * g.nz;
      s0[l * ld + k] = src[e];
    }
    __syncthreads();
    const float2 *out = dft_lines<true>(s0, s1, g.az, twz, L);
    const int64_t off = (int64_t)c * g.n + (int64_t)l0 * g.nz;
    for (int e = threadIdx.x; e < L * g.nz; e += blockDim.x) {
      const int l = qdiv(e, inv_nz), k = e - l * g.nz;
      const float v = out[l * ld + k].x * scale;
      zout[off + e] = v;
      if (r) acc = fmaf(r[off + e], v, acc);
    }
    __syncthreads();
  }
  return acc;
}

// z = M r of either layout with the grid barriers between its passes; returns this thread's
// partial of r . z (the caller's grid sum is the last barrier).  false: a barrier timed out.
template <int LAYOUT>
__device__ __forceinline__ bool precondition(const FftGrid &g, const float *r, float *z, float2 *s0, float2 *s1,
                                             const float2 *twx, const float2 *twy, const float2 *twz,
                                             GridBarrier *bar, unsigned long long tns, float &rz) {
  if (LAYOUT == CPM_FFT_LAYOUT_SLAB) {
    slab_fwd(g, r, s0, s1, twy, twz);
    if (!grid_sync(bar, gridDim.x, tns)) return false;
    slab_x_solve(g, s0, s1, twx);
    if (!grid_sync(bar, gridDim.x, tns)) return false;
    rz = slab_inv(g, z, r, s0, s1, twy, twz);
  } else {
    pass_z_fwd(g, r, s0, s1, twz);
    if (!grid_sync(bar, gridDim.x, tns)) return false;
    pass_y(g, false, s0, s1, twy);
    if (!grid_sync(bar, gridDim.x, tns)) return false;
    pass_x_solve(g, s0, s1, twx);
    if (!grid_sync(bar, gridDim.x, tns)) return false;
    pass_y(g, true, s0, s1, twy);
    if (!grid_sync(bar, gridDim.x, tns)) return false;
    rz = pass_z_inv(g, z, r, s0, s1, twz);
  }
  return true;
}

// ---------------------------------------------------------------- the inverse symbol (setup)
struct SymArgs {
  int nx, ny, nz, nc;
  int slab, h;  // slab layout: wave vectors (i, kz < h, j), one plane per symbol entry
  double c[243];
  double sigma;
  const double *cx, *sx, *cy, *sy, *cz, *sz;  // cos / sin of 2 pi i / n per axis (device tables)
  float *sym;
};

__global__ void __launch_bounds__(256) fft_symbol_kernel(const __grid_constant__ SymArgs a) {
  const int64_t n = a.slab ? (int64_t)a.nx * a.h * a.ny : (int64_t)a.nx * a.ny * a.nz;
  for (int64_t kidx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; kidx < n;
       kidx += (int64_t)gridDim.x * blockDim.x) {
    int ix, iy, iz;
    if (a.slab) {
      ix = (int)(kidx / ((int64_t)a.h * a.ny));
      const int rem = (int)(kidx - (int64_t)ix * a.h * a.ny);
      iz = rem / a.ny;
      iy = rem - iz * a.ny;
    } else {
      ix = (int)(kidx / ((int64_t)a.ny * a.nz));
      const int rem = (int)(kidx - (int64_t)ix * a.ny * a.nz);
      iy = rem / a.nz;
      iz = rem - iy * a.nz;
    }
    // e^{i theta_a d} for d = -1, 0, 1 per axis
    double ex[3][2], ey[3][2], ez[3][2];
    ex[0][0] = a.cx[ix]; ex[0][1] = -a.sx[ix]; ex[1][0] = 1.0; ex[1][1] = 0.0; ex[2][0] = a.cx[ix]; ex[2][1] = a.sx[ix];
    ey[0][0] = a.cy[iy]; ey[0][1] = -a.sy[iy]; ey[1][0] = 1.0; ey[1][1] = 0.0; ey[2][0] = a.cy[iy]; ey[2][1] = a.sy[iy];
    ez[0][0] = a.cz[iz]; ez[0][1] = -a.sz[iz]; ez[1][0] = 1.0; ez[1][1] = 0.0; ez[2][0] = a.cz[iz]; ez[2][1] = a.sz[iz];
    double S[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int dx = 0; dx < 3; ++dx)
      for (int dy = 0; dy < 3; ++dy) {
        const double pr = ex[dx][0] * ey[dy][0] - ex[dx][1] * ey[dy][1];
        const double pi = ex[dx][0] * ey[dy][1] + ex[dx][1] * ey[dy][0];
        for (int dz = 0; dz < 3; ++dz) {
          const double re = pr * ez[dz][0] - pi * ez[dz][1];  // Re e^{i theta . d}
          const int d = (dx * 3 + dy) * 3 + dz;
          for (int p = 0; p < a.nc; ++p)
            for (int q = 0; q < a.nc; ++q) S[p][q] += a.c[(p * a.nc + q) * 27 + d] * re;
        }
      }
    if (kidx == 0) {
      for (int p = 0; p < 3; ++p)
        for (int q = 0; q < 3; ++q) S[p][q] = p == q ? a.sigma : 0.0;
    }
    if (a.nc == 1) {
      a.sym[kidx] = (float)(1.0 / S[0][0]);
    } else {
      // symmetric 3x3 inverse by cofactors (S is symmetric: average the off-diagonal pairs)
      const double xx = S[0][0], yy = S[1][1], zz = S[2][2];
      const double xy = 0.5 * (S[0][1] + S[1][0]), yz = 0.5 * (S[1][2] + S[2][1]), xz = 0.5 * (S[0][2] + S[2][0]);
      const double cxx = yy * zz - yz * yz, cyy = xx * zz - xz * xz, czz = xx * yy - xy * xy;
      const double cxy = xz * yz - xy * zz, cyz = xy * xz - xx * yz, cxz = xy * yz - xz * yy;
      const double det = xx * cxx + xy * cxy + xz * cxz;
      const double id = 1.0 / det;
      const int64_t base = a.slab ? kidx : 6 * kidx, st = a.slab ? n : 1;
      const double v[6] = {cxx * id, cyy * id, czz * id, cxy * id, cyz * id, cxz * id};
      for (int m = 0; m < 6; ++m) a.sym[base + m * st] = (float)v[m];
    }
  }
}

// Counts the nodes whose row/column flags (bits 1, 2, 4) differ from a single pinned node `anchor`
// (flags 1|4 there, none elsewhere; bit 8 marks rows that take the checked path and is ignored).
__global__ void __launch_bounds__(256) anchor_check_kernel(const uint8_t *flags, int64_t n, int anchor, int *bad) {
  int cnt = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int f = flags[i] & 7;
    cnt += (i == anchor) ? (f != 5) : (f != 0);
  }
  if (cnt) atomicAdd(bad, cnt);
}

// ---------------------------------------------------------------- plan layout
struct PrecondLayout {
  size_t tw[3], trig[3], sym, check, total;
};

static PrecondLayout precond_layout(int nx, int ny, int nz, int nc) {
  PrecondLayout L{};
  const int dims[3] = {nx, ny, nz};
  size_t off = 0;
  for (int a = 0; a < 3; ++a) {
    L.tw[a] = off;
    off += align256(sizeof(float2) * dims[a]);
    L.trig[a] = off;
    off += align256(sizeof(double) * 2 * dims[a]);
  }
  // sized for the full spectrum (the slab layout's half spectrum takes less)
  L.sym = off;
  off += align256(sizeof(float) * (size_t)nx * ny * nz * (nc == 3 ? 6 : 1));
  L.check = off;  // one int: the anchor check of the build
  off += 256;
  L.total = off;
  return L;
}

// Radices of n: 8s, a 4 and a 2, then 3, 5, 7 and larger primes.
static int radices(int n, int *out) {
  int k = 0, m = n;
  while (m % 8 == 0 && k < kFftMaxPass) { out[k++] = 8; m /= 8; }
  while (m % 4 == 0 && k < kFftMaxPass) { out[k++] = 4; m /= 4; }
  while (m % 2 == 0 && k < kFftMaxPass) { out[k++] = 2; m /= 2; }
  for (int p = 3; m > 1 && k < kFftMaxPass; p += 2)
    while (m % p == 0 && k < kFftMaxPass) { out[k++] = p; m /= p; }
  return m == 1 ? k : -1;
}

// Complex values per shared region of the slab layout: the paired z lines, the kz columns along
// y, and at least one x line of every component.
static int slab_region(int nx, int ny, int nz, int nc) {
  const int P = (ny + 1) / 2, h = nz / 2 + 1;
  return std::max({P * line_stride(nz), h * line_stride(ny), nc * line_stride(nx)});
}

static bool slab_fits(int nx, int ny, int nz, int nc) {
  return sizeof(float2) * (2 * (size_t)slab_region(nx, ny, nz, nc) + nx + ny + nz) <= kSlabSmemMax;
}

static int auto_layout(int nx, int ny, int nz, int nc) {
  return slab_fits(nx, ny, nz, nc) ? CPM_FFT_LAYOUT_SLAB : CPM_FFT_LAYOUT_PASSES;
}

static bool precond_dims_ok(int nx, int ny, int nz, int nc) {
  int r[kFftMaxPass];
  return nx >= 3 && ny >= 3 && nz >= 3 && (nc == 1 || nc == 3) && line_stride(nx) * nc <= kFftTile &&
         line_stride(ny) <= kFftTile && line_stride(nz) <= kFftTile &&
         (int64_t)nx * ny * nz * nc < ((int64_t)1 << 31) && radices(nx, r) >= 0 &&
         radices(ny, r) >= 0 && radices(nz, r) >= 0;
}

static FftAxis axis_of(const cpm_fft_precond *P, int a) {
  FftAxis ax{};
  ax.n = a == 0 ? P->nx : a == 1 ? P->ny : P->nz;
  ax.npass = P->npass[a];
  for (int s = 0; s < kFftMaxPass; ++s) ax.radix[s] = P->radix[a][s];
  const PrecondLayout L = precond_layout(P->nx, P->ny, P->nz, P->ncomp);
  ax.tw = (const float2 *)((const char *)P->dev + L.tw[a]);
  return ax;
}

// Lines per tile: as many as a tile buffer holds, but no more than spreads the pass over all G CTAs.
static int tile_lines(int cap, int64_t units, int64_t G) {
  const int64_t even = (units + G - 1) / G;
  return (int)std::max<int64_t>(1, std::min<int64_t>(cap, even));
}

static FftGrid grid_of(const cpm_fft_precond *P, float2 *C, int64_t G) {
  FftGrid g{};
  g.nx = P->nx;
  g.ny = P->ny;
  g.nz = P->nz;
  g.n = P->nx * P->ny * P->nz;
  g.nc = P->ncomp;
  g.layout = P->layout;
  g.ax = axis_of(P, 0);
  g.ay = axis_of(P, 1);
  g.az = axis_of(P, 2);
  const PrecondLayout L = precond_layout(P->nx, P->ny, P->nz, P->ncomp);
  g.sym = (const float *)((const char *)P->dev + L.sym);
  g.C = C;
  if (g.layout == CPM_FFT_LAYOUT_SLAB) {
    g.h = g.nz / 2 + 1;
    g.reg = slab_region(g.nx, g.ny, g.nz, g.nc);
    // x tiles: as many columns as a region holds, spread evenly over the waves of G CTAs, a
    // multiple of 4 columns (32-byte segments of the complex rows) where that still fits
    const int64_t Hc = (int64_t)g.h * g.ny;
    const int cap = std::max(1, g.reg / (g.nc * line_stride(g.nx)));
    const int64_t waves = std::max<int64_t>(1, ((Hc + cap - 1) / cap + G - 1) / G);
    int pc = (int)std::min<int64_t>(cap, (Hc + waves * G - 1) / (waves * G));
    if ((pc + 3) / 4 * 4 <= cap) pc = (pc + 3) / 4 * 4;
    g.pc = std::max(1, pc);
  } else {
    g.lz = tile_lines(std::max(1, kFftTile / line_stride(g.nz)), (int64_t)g.nc * g.nx * g.ny, G);
    g.kty = tile_lines(std::max(1, std::min(g.nz, kFftTile / line_stride(g.ny))), (int64_t)g.nc * g.nx * g.nz, G);
    g.ktx = tile_lines(std::max(1, std::min(g.nz, kFftTile / (g.nc * line_stride(g.nx)))), (int64_t)g.ny * g.nz, G);
  }
  return g;
}

// ---------------------------------------------------------------- the preconditioned solve
struct FftCGArgs {
  StencilOp S;
  FftGrid F;
  const double *b;
  double *x;
  double tol;
  int maxiter;
  int use_init_host;
  const int *use_init_dev;
  double inner_tol;
  float *r, *z, *p, *q, *d;
  double *part;
  GridBarrier *bar;
  cpm_cg_info *info;
  unsigned long long timeout_ns;
  int64_t dofs_per_cta;
  int quads;
  int anchor;  // >= 0: direct refinement with this pinned node; -1: preconditioned CG
  int even;    // elastic stencil even in the offset: the FP64 residual sums opposite neighbours first
  double *cb, *ct;  // residual carry of the direct solve: b and t = b - A64 x of the last residual pass
  int *carry_valid;  // device flag: cb, ct belong to the current x (read at entry, written at exit)
  double e64[9 * 14];  // even part (c(d) + c(26 - d)) / 2 per block (p, q) for d < 13, then c(13)
};

constexpr int kInnerMax = 200;  // iterations of one inner preconditioned solve (a safety bound)

// q = A32 p on this CTA's DOFs [d0, d1); returns the thread's FP32 partial of p . q.
template <int NC, int NT>
__device__ __forceinline__ float product32(const FftCGArgs &a, int64_t d0, int64_t d1) {
  const int64_t n = a.S.n;
  const float *p = a.p;
  float *q = a.q;
  float pqf[1] = {0.0f};
  if (a.quads) {
    for (int64_t qd = d0 + 4 * threadIdx.x; qd < d1; qd += 4 * NT) {
      float y[4][NC];
      apply4_c<float, NC, 1>(a.S, a.S.c32, p, (int)qd, y);
      quad_store<float, NC, 1>(q, n, qd, y);
      quad_dot<NC, 1>(p, n, qd, y, pqf);
    }
  } else {
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += NT) {
      float y[NC];
      apply<float, NC, 1>(a.S, p, (int)dof, y);
#pragma unroll
      for (int u = 0; u < NC; ++u) {
        const int64_t i = uidx<NC, 1>(n, dof, u);
        q[i] = y[u];
        pqf[0] = fmaf(p[i], y[u], pqf[0]);
      }
    }
  }
  return pqf[0];
}

// y = A64 x at one unflagged DOF of the elastic operator whose blocks are even in the offset
// (c(-d) = c(d), to 1e-16 of their size: the symmetric element stiffness on identical cells):
// each pair of opposite neighbours is summed once per component and serves the three rows, 165
// FP64 operations where the 27-point form takes 243.
__device__ __forceinline__ void apply_even3(const FftCGArgs &a, const double *x, int dof, double (&y)[3]) {
  const int64_t n = a.S.n;
  const Nbr b = neighbours(a.S, dof);
  const double x0 = x[dof], x1 = x[n + dof], x2 = x[2 * n + dof];
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const double *e = a.e64 + (p * 3) * 14;
    y[p] = fma(e[13], x0, fma(e[14 + 13], x1, e[28 + 13] * x2));
  }
#pragma unroll
  for (int d = 0; d < 13; ++d) {
    const int ia = d / 9, ib = (d / 3) % 3, ic = d % 3;
    const int qp = b.xi[ia] + b.yj[ib] + b.zk[ic];
    const int qm = b.xi[2 - ia] + b.yj[2 - ib] + b.zk[2 - ic];
    const double s0 = x[qp] + x[qm], s1 = x[n + qp] + x[n + qm], s2 = x[2 * n + qp] + x[2 * n + qm];
#pragma unroll
    for (int p = 0; p < 3; ++p) {
      const double *e = a.e64 + (p * 3) * 14;
      y[p] = fma(e[d], s0, fma(e[14 + d], s1, fma(e[28 + d], s2, y[p])));
    }
  }
}

// t = b - A64 x on this CTA's DOFs: r = t (FP32), d = 0; v[0] = the thread's FP64 partial of t . t
// and, with SUMS, v[1 + c] = its partial of the sum of component c of t.  With SUMS and a carry,
// t goes to the carry too (and b, on the solve's first pass: wb).  x0: x = 0 (a cold start's first
// pass), so t = b exactly and the product is skipped.
template <int NC, int NT, bool SUMS, int NV>
__device__ __forceinline__ void true_residual64(const FftCGArgs &a, int64_t d0, int64_t d1, double (&v)[NV],
                                                bool wb, bool x0) {
  const int64_t n = a.S.n;
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j] = 0.0;
  for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += NT) {
    double y[NC];
    if (x0) {
#pragma unroll
      for (int u = 0; u < NC; ++u) y[u] = 0.0;
    } else if constexpr (NC == 3) {
      if (a.even && !(a.S.flags && a.S.flags[dof])) apply_even3(a, a.x, (int)dof, y);
      else apply<double, NC, 1>(a.S, a.x, (int)dof, y);
    } else {
      apply<double, NC, 1>(a.S, a.x, (int)dof, y);
    }
#pragma unroll
    for (int u = 0; u < NC; ++u) {
      const int64_t i = uidx<NC, 1>(n, dof, u);
      const double bi = a.b[i], t = bi - y[u];
      a.r[i] = (float)t;
      if (!SUMS) a.d[i] = 0.0f;
      v[0] = fma(t, t, v[0]);
      if (SUMS) {
        v[1 + u] += t;
        if (a.ct) {
          a.ct[i] = t;
          if (wb) a.cb[i] = bi;
        }
      }
    }
  }
}

// The first residual of a warm start from the x of the carry: t = (b - b_c) + t_c, no product
// (b - A x = (b - b_c) + (b_c - A x)).  Same outputs as true_residual64 with SUMS; the carry takes b and t.
template <int NC, int NT>
__device__ __forceinline__ void carried_residual(const FftCGArgs &a, int64_t d0, int64_t d1, double (&v)[1 + NC]) {
  const int64_t n = a.S.n;
#pragma unroll
  for (int j = 0; j < 1 + NC; ++j) v[j] = 0.0;
  for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += NT)
#pragma unroll
    for (int u = 0; u < NC; ++u) {
      const int64_t i = uidx<NC, 1>(n, dof, u);
      const double bi = a.b[i], t = (bi - a.cb[i]) + a.ct[i];
      a.r[i] = (float)t;
      a.cb[i] = bi;
      a.ct[i] = t;
      v[0] = fma(t, t, v[0]);
      v[1 + u] += t;
    }
}

// The right-hand side t~ of the direct step (CTA 0, after the residual's grid sum): the free
// nodes r next to the anchor a take (C_ra t_a)_r = sum_q c_pq(a - r) t_a,q, and the anchor takes
// minus the sum over the free nodes, so that every component of t~ sums to zero.  ta: t at the
// anchor (FP64); v[1 + c]: the sum of component c of t over all nodes.
template <int NC>
__device__ __forceinline__ void anchor_rhs(const FftCGArgs &a, const double (&ta)[NC], const double *v, float *r) {
  const int an = a.anchor, nx = a.S.nx, ny = a.S.ny, nz = a.S.nz;
  const int64_t n = a.S.n;
  const int ia = an / (ny * nz), ja = (an / nz) % ny, ka = an % nz;
  const int t = threadIdx.x;
  if (t < 27 * NC && t % 27 != 13) {
    const int d = t % 27, p = t / 27;
    const int dx = d / 9 - 1, dy = (d / 3) % 3 - 1, dz = d % 3 - 1;
    // the row r with r + d = a (periodic): its column a carries c(d)
    const int node = (((ia - dx + nx) % nx) * ny + (ja - dy + ny) % ny) * nz + (ka - dz + nz) % nz;
    double corr = 0.0;
#pragma unroll
    for (int q = 0; q < NC; ++q) corr = fma(a.S.c64[(p * NC + q) * 27 + d], ta[q], corr);
    r[(int64_t)p * n + node] += (float)corr;
  }
  if (t < NC) {
    double s = v[1 + t] - ta[t];
    for (int d = 0; d < 27; ++d) {
      if (d == 13) continue;
#pragma unroll
      for (int q = 0; q < NC; ++q) s = fma(a.S.c64[(t * NC + q) * 27 + d], ta[q], s);
    }
    r[(int64_t)t * n + an] = (float)(-s);
  }
}

template <int NC, int LAYOUT>
__global__ void __launch_bounds__(FftShape<LAYOUT>::threads, FftShape<LAYOUT>::blocks)
    cg_stencil_fft_kernel(const __grid_constant__ FftCGArgs a) {
  constexpr int NT = FftShape<LAYOUT>::threads, NW = NT / kWarp;
  extern __shared__ float2 fsm[];
  float2 *s0 = fsm, *s1 = fsm + fft_region(a.F);
  const float2 *twx, *twy, *twz;
  load_twiddles(a.F, fsm, twx, twy, twz);
  __shared__ double s_red[3][NW];
  const int64_t n = a.S.n;
  const int64_t d0 = min(n, (int64_t)blockIdx.x * a.dofs_per_cta);
  const int64_t d1 = min(n, d0 + a.dofs_per_cta);
  const bool use_init = a.use_init_dev ? (__ldcg(a.use_init_dev) != 0) : (a.use_init_host != 0);
  const unsigned long long tns = a.timeout_ns;
  const double *__restrict__ b = a.b;
  double *x = a.x;
  float *r = a.r, *z = a.z, *p = a.p, *q = a.q, *d = a.d;
  int par = 0;

  // ---- ||b||; x = 0 for a cold start
  double v[1] = {0.0};
  for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += NT)
#pragma unroll
    for (int u = 0; u < NC; ++u) {
      const int64_t i = uidx<NC, 1>(n, dof, u);
      const double bi = b[i];
      v[0] = fma(bi, bi, v[0]);
      if (!use_init) x[i] = 0.0;
    }
  if (!grid_sum<1, NW, NT>(v, a.part, par, a.bar, tns, s_red)) {
    set_status(a.info, CPM_BARRIER_TIMEOUT);
    if (a.carry_valid && blockIdx.x == 0 && threadIdx.x == 0) *a.carry_valid = 0;
    return;
  }
  const double bnorm = sqrt(v[0]);
  const double atol = a.tol * bnorm;
  int status = CPM_OK, iters = 0, outer = 0, conv = 0;
  double resid = 0.0;
  if (bnorm == 0.0) {
    // cupyx cg returns b itself for a zero right-hand side
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += NT)
#pragma unroll
      for (int u = 0; u < NC; ++u) x[uidx<NC, 1>(n, dof, u)] = b[uidx<NC, 1>(n, dof, u)];
    conv = 1;
  }
  // ---- direct refinement: x += A^-1 t with the anchored exact inverse, one FFT solve per step.
  // A warm start from the x of a valid carry takes its first residual from the carry; a carried
  // residual that already meets the test is confirmed by an FP64 residual before the solve stops.
  // `settled`: the loop left right after a residual pass of the final x (the carry then stays valid).
  bool carry = a.ct && use_init && !conv && __ldcg(a.carry_valid) == 1;
  bool first = true, settled = false;
  while (!conv && a.anchor >= 0) {
    const int an = a.anchor;
    double v[1 + NC];
    const bool carried = carry;
    if (carried) carried_residual<NC, NT>(a, d0, d1, v);
    else true_residual64<NC, NT, true>(a, d0, d1, v, first, first && !use_init);
    carry = first = false;
    if (!grid_sum<1 + NC, NW, NT>(v, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
    resid = sqrt(v[0]);
    if (!isfinite(resid)) { status = CPM_NONFINITE; break; }
    if (resid <= atol) {
      if (carried) continue;
      conv = 1;
      settled = true;
      break;
    }
    if (iters >= a.maxiter) { settled = true; break; }
    outer += 1;
    iters += 1;
    // the anchored rows are identity rows: t_a = b_a - x_a
    double ta[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) ta[c] = b[(int64_t)c * n + an] - x[(int64_t)c * n + an];
    if (blockIdx.x == 0) anchor_rhs<NC>(a, ta, v, r);
    if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
    float rzf = 0.0f;
    if (!precondition<LAYOUT>(a.F, r, z, s0, s1, twx, twy, twz, a.bar, tns, rzf) ||
        !grid_sync(a.bar, gridDim.x, tns)) {
      status = CPM_BARRIER_TIMEOUT;
      break;
    }
    // e = z + 1 (t_a - z_a): x += e (own unknowns), then a barrier before the next residual
    double gam[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) gam[c] = ta[c] - (double)z[(int64_t)c * n + an];
    if (!isfinite(gam[0])) { status = CPM_NONFINITE; break; }
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += NT)
#pragma unroll
      for (int u = 0; u < NC; ++u) {
        const int64_t i = uidx<NC, 1>(n, dof, u);
        x[i] += (double)z[i] + gam[u];
      }
    if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
  }
  while (!conv && a.anchor < 0 && status == CPM_OK) {
    // ---- true residual t = b - A64 x (x complete after the last barrier): r = t, d = 0
    double tt[1];
    true_residual64<NC, NT, false>(a, d0, d1, tt, false, outer == 0 && !use_init);
    if (!grid_sum<1, NW, NT>(tt, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
    resid = sqrt(tt[0]);
    if (!isfinite(resid)) { status = CPM_NONFINITE; break; }
    if (resid <= atol) { conv = 1; break; }
    if (iters >= a.maxiter) break;
    outer += 1;
    const double target = fmax(a.inner_tol * resid, 0.5 * atol);
    double rho_old = 0.0;
    for (int it = 0; it < kInnerMax && iters < a.maxiter; ++it) {
      // ---- z = M r, r.z
      float rzf = 0.0f;
      if (!precondition<LAYOUT>(a.F, r, z, s0, s1, twx, twy, twz, a.bar, tns, rzf)) {
        status = CPM_BARRIER_TIMEOUT;
        break;
      }
      double rz[1] = {(double)rzf};
      if (!grid_sum<1, NW, NT>(rz, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
      const double rho = rz[0];
      const float beta = it == 0 ? 0.0f : (float)(rho / rho_old);
      if (!isfinite(rho) || !isfinite((double)beta)) { status = CPM_NONFINITE; break; }
      rho_old = rho;
      // ---- p = z + beta p
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += NT)
#pragma unroll
        for (int u = 0; u < NC; ++u) {
          const int64_t i = uidx<NC, 1>(n, dof, u);
          p[i] = it == 0 ? z[i] : fmaf(beta, p[i], z[i]);
        }
      if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
      // ---- q = A32 p, p.q
      double pq[1] = {(double)product32<NC, NT>(a, d0, d1)};
      if (!grid_sum<1, NW, NT>(pq, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
      const float alpha = (float)(rho / pq[0]);
      if (!isfinite((double)alpha)) { status = CPM_NONFINITE; break; }
      // ---- d += alpha p, r -= alpha q, r.r
      float rrf = 0.0f;
      for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += NT)
#pragma unroll
        for (int u = 0; u < NC; ++u) {
          const int64_t i = uidx<NC, 1>(n, dof, u);
          d[i] = fmaf(alpha, p[i], d[i]);
          const float rn = fmaf(-alpha, q[i], r[i]);
          r[i] = rn;
          rrf = fmaf(rn, rn, rrf);
        }
      double rr[1] = {(double)rrf};
      if (!grid_sum<1, NW, NT>(rr, a.part, par, a.bar, tns, s_red)) { status = CPM_BARRIER_TIMEOUT; break; }
      iters += 1;
      if (!isfinite(rr[0])) { status = CPM_NONFINITE; break; }
      if (sqrt(rr[0]) <= target) break;
    }
    if (status != CPM_OK) break;
    // ---- x += d (own unknowns), then a barrier before the next true residual gathers x
    for (int64_t dof = d0 + threadIdx.x; dof < d1; dof += NT)
#pragma unroll
      for (int u = 0; u < NC; ++u) {
        const int64_t i = uidx<NC, 1>(n, dof, u);
        x[i] += (double)d[i];
      }
    if (!grid_sync(a.bar, gridDim.x, tns)) { status = CPM_BARRIER_TIMEOUT; break; }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int st = status;
    if (st == CPM_OK && !conv) st = CPM_NOT_CONVERGED;
    a.info->iters[0] = iters;
    a.info->iters[1] = a.info->iters[2] = 0;
    a.info->resid[0] = resid;
    a.info->bnorm[0] = bnorm;
    a.info->outer = outer;
    set_status(a.info, st);
    if (a.carry_valid) *a.carry_valid = (settled && status == CPM_OK) ? 1 : 0;
  } else if (status != CPM_OK && threadIdx.x == 0) {
    set_status(a.info, status);
  }
}

// ---------------------------------------------------------------- M r alone (tests)
// One pass of z = M r per launch (the launches order the passes): slab passes 0..2, five-pass 0..4.
__global__ void __launch_bounds__(512) fft_pass_kernel(const __grid_constant__ FftGrid g, int which,
                                                       const float *r, float *zout) {
  extern __shared__ float2 fsm[];
  float2 *s0 = fsm, *s1 = fsm + fft_region(g);
  const float2 *twx, *twy, *twz;
  load_twiddles(g, fsm, twx, twy, twz);
  if (g.layout == CPM_FFT_LAYOUT_SLAB) {
    if (which == 0) slab_fwd(g, r, s0, s1, twy, twz);
    else if (which == 1) slab_x_solve(g, s0, s1, twx);
    else slab_inv(g, zout, nullptr, s0, s1, twy, twz);
  } else {
    if (which == 0) pass_z_fwd(g, r, s0, s1, twz);
    else if (which == 1) pass_y(g, false, s0, s1, twy);
    else if (which == 2) pass_x_solve(g, s0, s1, twx);
    else if (which == 3) pass_y(g, true, s0, s1, twy);
    else pass_z_inv(g, zout, nullptr, s0, s1, twz);
  }
}

static int precond_check(const cpm_fft_precond *P, const char *who) {
  if (!P || !P->dev || !precond_dims_ok(P->nx, P->ny, P->nz, P->ncomp) ||
      (P->layout != CPM_FFT_LAYOUT_SLAB && P->layout != CPM_FFT_LAYOUT_PASSES) ||
      (P->layout == CPM_FFT_LAYOUT_SLAB && !slab_fits(P->nx, P->ny, P->nz, P->ncomp)) || P->anchor < -1 ||
      (int64_t)P->anchor >= (int64_t)P->nx * P->ny * P->nz) {
    set_error("%s: bad preconditioner plan", who);
    return CPM_BAD_ARG;
  }
  return CPM_OK;
}

static size_t fft_cg_layout(int64_t n, int nc, char *base, Workspace *w, float2 **C, float **z) {
  size_t off = 0;
  auto take = [&](size_t bytes) -> char * {
    char *ptr = base ? base + off : nullptr;
    off += align256(bytes);
    return ptr;
  };
  Workspace t{};
  t.bar = (GridBarrier *)take(sizeof(GridBarrier));
  t.part = (double *)take(sizeof(double) * 2 * kPartHalf);
  const size_t nv = (size_t)n * nc;
  t.r32 = (float *)take(4 * nv);
  t.pa32 = (float *)take(4 * nv);
  t.q32 = (float *)take(4 * nv);
  t.d32 = (float *)take(4 * nv);
  float *zz = (float *)take(4 * nv);
  float2 *cc = (float2 *)take(8 * nv);  // the full spectrum (the slab layout uses about half)
  if (w) *w = t;
  if (C) *C = cc;
  if (z) *z = zz;
  return off;
}

}  // namespace cpm

extern "C" int64_t cpm_fft_precond_bytes(int32_t nx, int32_t ny, int32_t nz, int32_t ncomp) {
  using namespace cpm;
  if (!precond_dims_ok(nx, ny, nz, ncomp)) return 0;
  return (int64_t)precond_layout(nx, ny, nz, ncomp).total;
}

extern "C" int cpm_fft_precond_build(const cpm_stencil *S, void *dev, int64_t bytes, cpm_fft_precond *P,
                                     void *stream) {
  using namespace cpm;
  if (!S || !P || !dev || ((uintptr_t)dev & 255) || !precond_dims_ok(S->nx, S->ny, S->nz, S->ncomp)) {
    set_error("cpm_fft_precond_build: bad arguments (a stencil with at least 3 cells per axis and a 256-byte "
              "aligned device buffer)");
    return CPM_BAD_ARG;
  }
  const int want = P->layout;
  if (want != CPM_FFT_LAYOUT_AUTO && want != CPM_FFT_LAYOUT_SLAB && want != CPM_FFT_LAYOUT_PASSES) {
    set_error("cpm_fft_precond_build: unknown layout %d", want);
    return CPM_BAD_ARG;
  }
  if (want == CPM_FFT_LAYOUT_SLAB && !slab_fits(S->nx, S->ny, S->nz, S->ncomp)) {
    set_error("cpm_fft_precond_build: an x-plane of the %dx%dx%d grid does not fit the slab layout's shared "
              "memory", S->nx, S->ny, S->nz);
    return CPM_BAD_ARG;
  }
  const PrecondLayout L = precond_layout(S->nx, S->ny, S->nz, S->ncomp);
  if (bytes < (int64_t)L.total) {
    set_error("cpm_fft_precond_build: buffer too small (%lld < %zu bytes)", (long long)bytes, L.total);
    return CPM_BAD_ARG;
  }
  P->nx = S->nx;
  P->ny = S->ny;
  P->nz = S->nz;
  P->ncomp = S->ncomp;
  const int64_t nodes = (int64_t)S->nx * S->ny * S->nz;
  if (P->anchor < -1 || P->anchor >= nodes || (P->anchor >= 0 && !S->flags)) {
    set_error("cpm_fft_precond_build: anchor %d is not a node of the grid, or the stencil has no flags", P->anchor);
    return CPM_BAD_ARG;
  }
  P->layout = want == CPM_FFT_LAYOUT_AUTO ? auto_layout(S->nx, S->ny, S->nz, S->ncomp) : want;
  P->dev = dev;
  P->bytes = (int64_t)L.total;
  cudaStream_t st = (cudaStream_t)stream;
  char *base = (char *)dev;
  const int dims[3] = {S->nx, S->ny, S->nz};
  for (int a = 0; a < 3; ++a) {
    for (int s = 0; s < kFftMaxPass; ++s) P->radix[a][s] = 0;
    P->npass[a] = radices(dims[a], P->radix[a]);
    const int nn = dims[a];
    std::vector<float2> tw(nn);
    std::vector<double> trig(2 * nn);
    for (int t = 0; t < nn; ++t) {
      const double ang = 2.0 * M_PI * (double)t / (double)nn;
      tw[t] = make_float2((float)std::cos(ang), (float)-std::sin(ang));
      trig[t] = std::cos(ang);
      trig[nn + t] = std::sin(ang);
    }
    CPM_TRY(cudaMemcpyAsync(base + L.tw[a], tw.data(), sizeof(float2) * nn, cudaMemcpyHostToDevice, st));
    CPM_TRY(cudaMemcpyAsync(base + L.trig[a], trig.data(), sizeof(double) * 2 * nn, cudaMemcpyHostToDevice, st));
    CPM_TRY(cudaStreamSynchronize(st));  // the host tables go out of scope
  }
  SymArgs s{};
  s.nx = S->nx;
  s.ny = S->ny;
  s.nz = S->nz;
  s.nc = S->ncomp;
  s.slab = P->layout == CPM_FFT_LAYOUT_SLAB;
  s.h = S->nz / 2 + 1;
  const int nc2 = 27 * S->ncomp * S->ncomp;
  for (int i = 0; i < 243; ++i) s.c[i] = i < nc2 ? S->coef[i] : 0.0;
  // the zero wave vector (the translations, singular in the circulant part) gets the operator's diagonal
  double diag = 0.0;
  for (int c = 0; c < S->ncomp; ++c) diag += S->coef[(c * S->ncomp + c) * 27 + 13];
  s.sigma = diag / S->ncomp;
  const double *trig[3] = {(const double *)(base + L.trig[0]), (const double *)(base + L.trig[1]),
                           (const double *)(base + L.trig[2])};
  s.cx = trig[0];
  s.sx = trig[0] + S->nx;
  s.cy = trig[1];
  s.sy = trig[1] + S->ny;
  s.cz = trig[2];
  s.sz = trig[2] + S->nz;
  s.sym = (float *)(base + L.sym);
  const int64_t n = (int64_t)S->nx * S->ny * S->nz;
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 16));
  fft_symbol_kernel<<<g, 256, 0, st>>>(s);
  if (int e = check_launch("cpm_fft_precond_build")) return e;
  if (P->anchor >= 0) {
    // the direct solve inverts exactly the circulant with one pinned node: check the flags say so
    int *bad = (int *)(base + L.check);
    CPM_TRY(cudaMemsetAsync(bad, 0, sizeof(int), st));
    anchor_check_kernel<<<g, 256, 0, st>>>(S->flags, n, P->anchor, bad);
    if (int e = check_launch("cpm_fft_precond_build")) return e;
    int h_bad = 0;
    CPM_TRY(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    CPM_TRY(cudaStreamSynchronize(st));
    if (h_bad) {
      set_error("cpm_fft_precond_build: the stencil's flags are not one pinned node at %d (%d nodes differ)",
                P->anchor, h_bad);
      return CPM_BAD_ARG;
    }
  }
  return CPM_OK;
}

extern "C" int cpm_fft_precond_apply(const cpm_fft_precond *P, const float *r, float *z, void *work,
                                     int64_t work_bytes, void *stream) {
  using namespace cpm;
  if (int e = precond_check(P, "cpm_fft_precond_apply")) return e;
  const int64_t n = (int64_t)P->nx * P->ny * P->nz;
  if (!r || !z || !work || work_bytes < (int64_t)(8 * n * P->ncomp) || ((uintptr_t)work & 15)) {
    set_error("cpm_fft_precond_apply: bad vectors or a complex work buffer under %lld bytes",
              (long long)(8 * n * P->ncomp));
    return CPM_BAD_ARG;
  }
  const bool slab = P->layout == CPM_FFT_LAYOUT_SLAB;
  const int G = sm_count() * 2;
  const FftGrid g = grid_of(P, (float2 *)work, G);
  const size_t smem = fft_smem_bytes(g);
  CPM_TRY(cudaFuncSetAttribute((const void *)fft_pass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  cudaStream_t st = (cudaStream_t)stream;
  for (int w = 0; w < (slab ? 3 : 5); ++w) {
    fft_pass_kernel<<<G, slab ? 512 : 256, smem, st>>>(g, w, r, z);
    if (int e = check_launch("cpm_fft_precond_apply")) return e;
  }
  return CPM_OK;
}

extern "C" size_t cpm_cg_fft_workspace_bytes(int32_t nx, int32_t ny, int32_t nz, int32_t ncomp) {
  return cpm::fft_cg_layout((int64_t)nx * ny * nz, ncomp, nullptr, nullptr, nullptr, nullptr);
}

extern "C" int cpm_cg_solve_stencil_fft(const cpm_stencil *S, const cpm_fft_precond *P, const double *b, double *x,
                                        const cpm_cg_opts *o, void *workspace, size_t workspace_bytes,
                                        cpm_cg_info *info, void *stream) {
  using namespace cpm;
  if (int e = precond_check(P, "cpm_cg_solve_stencil_fft")) return e;
  if (!S || !b || !x || !o || !workspace || !info || S->nx != P->nx || S->ny != P->ny || S->nz != P->nz ||
      S->ncomp != P->ncomp || ((uintptr_t)workspace & 255)) {
    set_error("cpm_cg_solve_stencil_fft: bad arguments (stencil, plan of the same grid, vectors, options, "
              "256-byte aligned workspace, info)");
    return CPM_BAD_ARG;
  }
  const int nc = S->ncomp;
  const int64_t n = (int64_t)S->nx * S->ny * S->nz;
  const size_t need = fft_cg_layout(n, nc, nullptr, nullptr, nullptr, nullptr);
  if (workspace_bytes < need) {
    set_error("cpm_cg_solve_stencil_fft: workspace too small (%zu < %zu bytes)", workspace_bytes, need);
    return CPM_BAD_ARG;
  }
  Workspace w;
  float2 *C;
  float *zz;
  fft_cg_layout(n, nc, (char *)workspace, &w, &C, &zz);
  FftCGArgs a{};
  a.S.nx = S->nx;
  a.S.ny = S->ny;
  a.S.nz = S->nz;
  a.S.n = (int)n;
  a.S.flags = S->flags;
  const int ncoef = 27 * nc * nc;
  for (int i = 0; i < 243; ++i) {
    a.S.c64[i] = i < ncoef ? S->coef[i] : 0.0;
    a.S.c32[i] = (float)a.S.c64[i];
  }
  a.b = b;
  a.x = x;
  a.tol = o->tol;
  a.maxiter = o->maxiter;
  a.use_init_host = o->use_init_host;
  a.use_init_dev = o->use_init_dev;
  a.inner_tol = o->inner_tol > 0 ? o->inner_tol : 1e-4;
  a.r = w.r32;
  a.p = w.pa32;
  a.q = w.q32;
  a.d = w.d32;
  a.z = zz;
  a.part = w.part;
  a.bar = w.bar;
  a.info = info;
  const double tmo = o->barrier_timeout_s > 0 ? o->barrier_timeout_s : 2.0;
  a.timeout_ns = (unsigned long long)(tmo * 1e9);
  a.quads = (S->nz & 3) == 0 && ((uintptr_t)S->flags & 3) == 0;
  a.anchor = (P->anchor >= 0 && o->form != CPM_CG_FORM_FFT_PCG) ? P->anchor : -1;
  const int ncarry = !!o->carry_b + !!o->carry_t + !!o->carry_valid;
  if (ncarry != 0 && ncarry != 3) {
    set_error("cpm_cg_solve_stencil_fft: carry_b, carry_t and carry_valid are given together or not at all");
    return CPM_BAD_ARG;
  }
  if (ncarry == 3 && (o->carry_b == b || o->carry_t == b || o->carry_b == x || o->carry_t == x ||
                      o->carry_b == o->carry_t)) {
    set_error("cpm_cg_solve_stencil_fft: the carry vectors must not alias b, x or each other");
    return CPM_BAD_ARG;
  }
  a.cb = o->carry_b;
  a.ct = o->carry_t;
  a.carry_valid = o->carry_valid;
  if (nc == 3) {
    // even blocks (to 1e-12 of their largest coefficient): the pair-summed FP64 residual
    a.even = 1;
    for (int blk = 0; blk < 9; ++blk) {
      const double *c = S->coef + 27 * blk;
      double big = 0.0;
      for (int d = 0; d < 27; ++d) big = std::max(big, std::fabs(c[d]));
      for (int d = 0; d < 13; ++d) {
        if (std::fabs(c[d] - c[26 - d]) > 1e-12 * big) a.even = 0;
        a.e64[blk * 14 + d] = 0.5 * (c[d] + c[26 - d]);
      }
      a.e64[blk * 14 + 13] = c[13];
    }
  }
  const bool slab = P->layout == CPM_FFT_LAYOUT_SLAB;
  const void *fn = slab ? (nc == 3 ? (const void *)cg_stencil_fft_kernel<3, CPM_FFT_LAYOUT_SLAB>
                                   : (const void *)cg_stencil_fft_kernel<1, CPM_FFT_LAYOUT_SLAB>)
                        : (nc == 3 ? (const void *)cg_stencil_fft_kernel<3, CPM_FFT_LAYOUT_PASSES>
                                   : (const void *)cg_stencil_fft_kernel<1, CPM_FFT_LAYOUT_PASSES>);
  const int threads = slab ? FftShape<CPM_FFT_LAYOUT_SLAB>::threads : FftShape<CPM_FFT_LAYOUT_PASSES>::threads;
  // the tiles depend on the grid size and the shared memory on the layout; the grid size on the
  // occupancy of that shared memory (the region size does not depend on G)
  FftGrid g0 = grid_of(P, C, 1);
  const size_t smem = fft_smem_bytes(g0);
  CPM_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int occ = 0;
  CPM_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, smem));
  if (occ < 1) {
    set_error("cpm_cg_solve_stencil_fft: kernel cannot be resident on an SM");
    return CPM_CUDA_ERROR;
  }
  int64_t G = std::min<int64_t>((int64_t)occ * sm_count(), kMaxGrid);
  int64_t per = (n + G - 1) / G;
  per = (per + 31) / 32 * 32;
  G = std::max<int64_t>(1, (n + per - 1) / per);
  a.dofs_per_cta = per;
  a.F = grid_of(P, C, G);
  CPM_TRY(cudaMemsetAsync(w.bar, 0, sizeof(GridBarrier), (cudaStream_t)stream));
  CPM_TRY(cudaMemsetAsync(info, 0, sizeof(cpm_cg_info), (cudaStream_t)stream));
  void *args[] = {&a};
  CPM_TRY(cudaLaunchCooperativeKernel(fn, dim3((unsigned)G), dim3(threads), args, smem, (cudaStream_t)stream));
  return CPM_OK;
}
