// step_lanes.cu -- FP64 passes of the batched mixed-precision step, one thread
// per lane.
//
// A batch holds thousands of independent lanes (rows or columns of many
// cases).  Here one thread runs each lane's banded recurrences sequentially,
// so every lane of every warp issues useful FP64 work and no scan, shuffle or
// barrier is needed (the single-case kernels of step_fp64.cu use 16-thread
// scans instead, because one case has too few lanes to fill the GPU).
// The banded operators couple indices of equal parity only (offsets 0, +-2,
// +-4), the Chebyshev derivative maps one parity onto the other, and the
// fields are independent, so most passes split each lane into independent
// (field, parity) sub-lanes (blockIdx.y): up to 6 threads per lane instead
// of one, for latency hiding, with every recurrence still sequential.
// Column lanes (x direction) are read and written coalesced across a warp;
// row lanes (y direction) stream through L1, each thread along its own row.
// Multi-pass kernels re-read their own earlier results from L1/L2.
//
// Operations and their reference lines are those of the FP64 kernels:
// to_ortho / from_ortho (composite_stencil.rs:117-276, linalg.rs:14-57),
// differentiate (ortho.rs:107-125), MatVecFdma (matvec.rs:142-248), Fdma
// (fdma.rs:179-227), the RBC step (navier.rs:622-721).
//
// Work item: (case, first lane, lane count <= blockDim.x, 0).
#include "lane_ops.cuh"
#include "step_fp64.h"

namespace rbc {
namespace dev {

// Chebyshev derivative d = D a of a lane whose coefficients arrive in
// descending index order: d_{n-1} = 0, d_i = 2(i+1) a_{i+1} + d_{i+2}
// (1 <= i <= n-2), d_0 = a_1 + d_2 / 2.  step(i, a_i) returns d_i.
template <class T>
struct DescDiff {
  T a_next, d1, d2;
  int n;
  __device__ __forceinline__ explicit DescDiff(int n_) : a_next(zero_v<T>()), d1(zero_v<T>()), d2(zero_v<T>()), n(n_) {}
  __device__ __forceinline__ T step(int i, T a_i) {
    T d;
    if (i == n - 1) d = zero_v<T>();
    else if (i >= 1) d = fmas(d2, a_next, exact_double(2 * i + 2));
    else d = fmas(a_next, d2, 0.5);
    d2 = d1;
    d1 = d;
    a_next = a_i;
    return d;
  }
};

// composite stencil p_i = diag_i c_i + low2_{i-2} c_{i-2} of a strided lane
// (c has b.m entries; Chebyshev / Fourier bases are the identity)
template <class T>
__device__ __forceinline__ T stencil_lane(const BasisDev& b, const T* c, long long s, int i) {
  if (b.kind == 0 || b.kind == 5) return c[(long long)i * s];
  const int m = b.m;
  T v = zero_v<T>();
  if (i < m) v = b.unit_diag ? c[(long long)i * s] : scal(c[(long long)i * s], b.diag[i]);
  if (i >= 2 && i - 2 < m) {
    const T t = c[(long long)(i - 2) * s];
    v = (i < m) ? fmas(v, t, b.low2[i - 2]) : scal(t, b.low2[i - 2]);
  }
  return v;
}

// per-row factor pointers of a banded solver
struct FdmaRow {
  const double *low, *dinv, *up1, *up2;
  int m;
};
__device__ __forceinline__ FdmaRow fdma_row(const FdmaDev& f, int row) {
  const size_t o = (f.rows > 1) ? (size_t)row * f.stride : 0;
  return FdmaRow{f.low + o, f.dinv + o, f.up1 + o, f.up2 + o, f.m};
}

// Fdma forward elimination x_i += low_{i-2} x_{i-2} of a strided lane, in place
template <class T>
__device__ __forceinline__ void fdma_fwd_lane(const FdmaRow& f, T* x, long long s) {
  T xm1 = zero_v<T>(), xm2 = zero_v<T>();
#pragma unroll 4
  for (int i = 0; i < f.m; i++) {
    T v = x[(long long)i * s];
    if (i >= 2) v = fmas(v, xm2, f.low[i - 2]);
    x[(long long)i * s] = v;
    xm2 = xm1;
    xm1 = v;
  }
}
// Fdma back substitution x_j = x_j / dia_j - up1_j x_{j+2} - up2_j x_{j+4}
// (factors stored as 1/dia and -up/dia), in place
template <class T>
__device__ __forceinline__ void fdma_bwd_lane(const FdmaRow& f, T* x, long long s) {
  T p1 = zero_v<T>(), p2 = zero_v<T>(), p3 = zero_v<T>(), p4 = zero_v<T>();
#pragma unroll 4
  for (int j = f.m - 1; j >= 0; j--) {
    T v = scal(x[(long long)j * s], f.dinv[j]);
    if (j + 2 < f.m) v = fmas(v, p2, f.up1[j]);
    if (j + 4 < f.m) v = fmas(v, p4, f.up2[j]);
    x[(long long)j * s] = v;
    p4 = p3;
    p3 = p2;
    p2 = p1;
    p1 = v;
  }
}

// pinv row r (entries at r, r+2, r+4) of a strided lane of length n
template <class T>
__device__ __forceinline__ T pinv_lane(const PinvDev& p, const T* a, long long s, int r) {
  const int m = p.n - 2;
  T v = scal(a[(long long)r * s], p.dia[r]);
  if (r < m - 2) v = fmas(v, a[(long long)(r + 2) * s], p.up1[r]);
  if (r < m - 4) v = fmas(v, a[(long long)(r + 4) * s], p.up2[r]);
  return v;
}

// least-squares from_ortho of a strided lane (composite basis), in two passes:
// rhs and forward sweep into `out`, then back substitution in place.
template <class T>
__device__ __forceinline__ void from_ortho_lane(const BasisDev& b, const T* p, long long ps, T* out, long long os) {
  const int m = b.m;
  T g1 = zero_v<T>(), g2 = zero_v<T>();
#pragma unroll 4
  for (int i = 0; i < m; i++) {
    const T d = fmas(b.unit_diag ? p[(long long)i * ps] : scal(p[(long long)i * ps], b.diag[i]), p[(long long)(i + 2) * ps], b.low2[i]);
    const double q = b.fo_dinv[i];
    T g = scal(d, q);
    if (i >= 2) g = fmas(g, g2, -b.fo_off[i - 2] * q);
    out[(long long)i * os] = g;
    g2 = g1;
    g1 = g;
  }
  T x1 = zero_v<T>(), x2 = zero_v<T>();
#pragma unroll 4
  for (int j = m - 1; j >= 0; j--) {
    T x = out[(long long)j * os];
    if (j + 2 < m) x = fmas(x, x2, -b.fo_w[j]);
    out[(long long)j * os] = x;
    x2 = x1;
    x1 = x;
  }
}

// ---- parity chains: index q, q+2, q+4, ... of a lane --------------------------
// largest index < n of parity q (or -1)
__device__ __forceinline__ int top_par(int n, int q) { return ((n - 1 - q) & 1) ? n - 2 : n - 1; }

// Each chain below loads kPB elements (and their coefficients) into registers
// before running their recurrence steps: the chains are latency-bound, and
// loads issued one step at a time behind the previous step's store (which
// the compiler cannot reorder) left about 15 stall cycles per instruction.
// The arithmetic and its order are those of the one-element-at-a-time form.
constexpr int kPB = 8;
// box y3 and y5 (row chains, 40 registers) measured best with 2 and 1 elements
// ahead: y3 0.23 / 0.26 / 0.35 ms per ensemble step with 2 / 1 / 4, y5 0.29 /
// 0.30 with 1 / 4
constexpr int kPBY3 = 2;
constexpr int kPBY5 = 1;
// complex (periodic Y2) chains, elements of two doubles each: Y2A 4 (8 took
// 196 registers, five 64-thread blocks per SM), Y2B 6, Y2C 8, each the
// fastest measured
constexpr int kPBC = 4;
constexpr int kPBCB = 6;
constexpr int kPBCC = 8;

// Chebyshev derivative d = D a on the indices of parity q, descending:
// d_{n-1} = 0, d_i = 2(i+1) a_{i+1} + d_{i+2}, d_0 = a_1 + d_2 / 2; a(i)
// supplies a_i (parity 1-q), store(i, d_i) receives the result
template <class T, int PB = kPB, class A, class S>
__device__ __forceinline__ void diff_par(int n, int q, A a, S store) {
  T d2 = zero_v<T>();
  for (int i0 = top_par(n, q); i0 >= 0; i0 -= 2 * PB) {
    T av[PB];
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int i = i0 - 2 * e;
      av[e] = (i >= 0 && i < n - 1) ? a(i + 1) : zero_v<T>();
    }
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int i = i0 - 2 * e;
      if (i < 0) break;
      T d;
      if (i == n - 1) d = zero_v<T>();
      else if (i >= 1) d = fmas(d2, av[e], exact_double(2 * i + 2));
      else d = fmas(av[e], d2, 0.5);
      store(i, d);
      d2 = d;
    }
  }
}

// Fdma forward elimination on the parity-q indices of a strided lane, in place
template <class T, int PB = kPB>
__device__ __forceinline__ void fdma_fwd_par(const FdmaRow& f, T* x, long long s, int q) {
  T xm2 = zero_v<T>();
  for (int i0 = q; i0 < f.m; i0 += 2 * PB) {
    T xv[PB];
    double lv[PB];
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int i = i0 + 2 * e;
      xv[e] = i < f.m ? x[(long long)i * s] : zero_v<T>();
      lv[e] = (i < f.m && i >= 2) ? __ldg(f.low + i - 2) : 0.0;
    }
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int i = i0 + 2 * e;
      if (i >= f.m) break;
      T v = xv[e];
      if (i >= 2) v = fmas(v, xm2, lv[e]);
      x[(long long)i * s] = v;
      xm2 = v;
    }
  }
}

// Fdma back substitution on the parity-q indices of a strided lane, in place
template <class T, int PB = kPB>
__device__ __forceinline__ void fdma_bwd_par(const FdmaRow& f, T* x, long long s, int q) {
  T p2 = zero_v<T>(), p4 = zero_v<T>();
  for (int j0 = top_par(f.m, q); j0 >= 0; j0 -= 2 * PB) {
    T xv[PB];
    double dv[PB], u1[PB], u2[PB];
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int j = j0 - 2 * e;
      const bool in = j >= 0;
      xv[e] = in ? x[(long long)j * s] : zero_v<T>();
      dv[e] = in ? __ldg(f.dinv + j) : 0.0;
      u1[e] = (in && j + 2 < f.m) ? __ldg(f.up1 + j) : 0.0;
      u2[e] = (in && j + 4 < f.m) ? __ldg(f.up2 + j) : 0.0;
    }
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int j = j0 - 2 * e;
      if (j < 0) break;
      T v = scal(xv[e], dv[e]);
      if (j + 2 < f.m) v = fmas(v, p2, u1[e]);
      if (j + 4 < f.m) v = fmas(v, p4, u2[e]);
      x[(long long)j * s] = v;
      p4 = p2;
      p2 = v;
    }
  }
}

// pinv rows fused with the Fdma forward elimination on the parity-q indices:
// out_i = pinv_i(in) + low_{i-2} out_{i-2}, i < f.m (in and out are different lanes)
template <class T, int PB = kPB>
__device__ __forceinline__ void pinv_fwd_par(const PinvDev& p, const FdmaRow& f, const T* in, long long is, T* out,
                                             long long os, int q) {
  T xm2 = zero_v<T>();
  for (int i0 = q; i0 < f.m; i0 += 2 * PB) {
    T pv[PB];
    double lv[PB];
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int i = i0 + 2 * e;
      pv[e] = i < f.m ? pinv_lane<T>(p, in, is, i) : zero_v<T>();
      lv[e] = (i < f.m && i >= 2) ? __ldg(f.low + i - 2) : 0.0;
    }
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int i = i0 + 2 * e;
      if (i >= f.m) break;
      T v = pv[e];
      if (i >= 2) v = fmas(v, xm2, lv[e]);
      out[(long long)i * os] = v;
      xm2 = v;
    }
  }
}

// from_ortho (least squares, stride-2 tridiagonal) on the parity-q chain, the
// forward sweep with its factors multiplied out at set-up (BasisDev::fo_a..c);
// `in` and `out` may be the same lane (a batch reads its inputs, including
// p_{i+2} of its last element, before writing)
template <class T, int PB = kPB>
__device__ __forceinline__ void from_ortho_par(const BasisDev& b, const T* p, long long ps, T* out, long long os, int q) {
  const int m = b.m;
  T g2 = zero_v<T>();
  for (int i0 = q; i0 < m; i0 += 2 * PB) {
    T dv[PB];
    double cv[PB];
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int i = i0 + 2 * e;
      if (i < m) {
        dv[e] = fmas(scal(p[(long long)i * ps], __ldg(b.fo_a + i)), p[(long long)(i + 2) * ps], __ldg(b.fo_b + i));
        cv[e] = __ldg(b.fo_c + i);
      } else {
        dv[e] = zero_v<T>();
        cv[e] = 0.0;
      }
    }
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int i = i0 + 2 * e;
      if (i >= m) break;
      const T g = fmas(dv[e], g2, cv[e]);  // fo_c is 0 for i < 2
      out[(long long)i * os] = g;
      g2 = g;
    }
  }
  T x2 = zero_v<T>();
  for (int j0 = top_par(m, q); j0 >= 0; j0 -= 2 * PB) {
    T xv[PB];
    double wv[PB];
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int j = j0 - 2 * e;
      xv[e] = j >= 0 ? out[(long long)j * os] : zero_v<T>();
      wv[e] = (j >= 0 && j + 2 < m) ? __ldg(b.fo_w + j) : 0.0;
    }
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int j = j0 - 2 * e;
      if (j < 0) break;
      T x = xv[e];
      if (j + 2 < m) x = fmas(x, x2, -wv[e]);
      out[(long long)j * os] = x;
      x2 = x;
    }
  }
}

#define LANE_PROLOGUE                                                        \
  const int4 w = work[blockIdx.x];                                           \
  if ((int)threadIdx.x >= w.z) return;                                       \
  const CaseDev& c = cases[w.x];                                             \
  if (c.gate != nullptr && c.gate[1] == 0) return;                           \
  const int lane = w.y + (int)threadIdx.x;                                   \
  const int sub = (int)blockIdx.y;                                           \
  (void)sub;

// row kernels: the two parity chains of a row run on adjacent threads of a
// warp (q = threadIdx.x & 1), so a warp's loads of elements k and k + 1 share
// sectors; blockIdx.y selects the field or part
#define ROW_PROLOGUE                                                         \
  const int4 w = work[blockIdx.x];                                           \
  if ((int)(threadIdx.x >> 1) >= w.z) return;                                \
  const CaseDev& c = cases[w.x];                                             \
  if (c.gate != nullptr && c.gate[1] == 0) return;                           \
  const int lane = w.y + (int)(threadIdx.x >> 1);                            \
  const int q = (int)(threadIdx.x & 1);                                      \
  const int sub = (int)blockIdx.y;                                           \
  (void)sub;

// d/dx p0 / aspect -> s[0] (nx x ny), columns j < ny; sub = parity of the output rows
__global__ void __launch_bounds__(128) k_lp_box_gpx(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  LANE_PROLOGUE
  const int j = lane, nx = c.nx, ny = c.ny;
  const double inv_asp = 1.0 / c.aspect;
  const double* p0 = static_cast<const double*>(c.p0) + j;
  double* gp = static_cast<double*>(c.s[0]) + j;
  diff_par<double>(nx, sub, [&](int i) { return p0[(long long)i * ny]; },
                   [&](int i, double d) { gp[(long long)i * ny] = d * inv_asp; });
}

// pinv_x and the ADI x solve of the three fields: s[1..3] -> s[4..6], columns
// j < myc; sub = 2 * field + parity
__global__ void __launch_bounds__(128) k_lp_box_x2(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  LANE_PROLOGUE
  const int j = lane, myc = c.myc, f = sub >> 1, q = sub & 1;
  const double* in = static_cast<const double*>(c.s[1 + f]) + j;
  double* out = static_cast<double*>(c.s[4 + f]) + j;
  const FdmaRow F = fdma_row(f < 2 ? c.hu_x : c.ht_x, 0);
  pinv_fwd_par<double>(c.pinv_x, F, in, myc, out, myc, q);
  fdma_bwd_par<double>(F, out, myc, q);
}

// divergence and pinv_x: A = s[1], B = s[2] (mxc x ny) -> div s[3] (nx x ny),
// pinv_x div -> m_z (mxc x ny), columns j < ny; sub = parity of the rows
// (Dx A on parity q from Sx A on parity 1 - q)
__global__ void __launch_bounds__(128) k_lp_box_x3(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  LANE_PROLOGUE
  const int j = lane, nx = c.nx, ny = c.ny, mxc = c.mxc, q = sub;
  const double inv_asp = 1.0 / c.aspect;
  const double* A = static_cast<const double*>(c.s[1]) + j;
  const double* B = static_cast<const double*>(c.s[2]) + j;
  double* dv = static_cast<double*>(c.s[3]) + j;
  diff_par<double>(nx, q, [&](int i) { return stencil_lane<double>(c.xu, A, ny, i); },
                   [&](int i, double da) { dv[(long long)i * ny] = fma(da, inv_asp, stencil_lane<double>(c.xu, B, ny, i)); });
  float* z = static_cast<float*>(c.m_z) + j;  // FP32: the input of the eigenbasis GEMM
#pragma unroll 4
  for (int r = q; r < mxc; r += 2) z[(long long)r * ny] = (float)pinv_lane<double>(c.pinv_x, dv, ny, r);
}

// projection along x from p1 (computed by the eigenbasis GEMM): p1[0][0] = 0;
// Gp = Sx^N p1 -> s[0], E = Sx+ (Dx Sx^N p1 / s) -> s[1], Fv = Sx+ Sx^N p1 -> s[2]
// (s arrays as mxc/nx x myc), columns j < myc.  sub = 2 * part + parity q:
// part 0: Gp and Fv on the rows of parity q; part 1: E on the rows of parity
// 1 - q, from Gp of parity q formed again from p1 (the two parts share no
// intermediate, so they run on different threads)
__global__ void __launch_bounds__(128) k_lp_box_x4(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  LANE_PROLOGUE
  const int j = lane, nx = c.nx, myc = c.myc, q = sub & 1, part = sub >> 1;
  double* p1 = static_cast<double*>(c.p1) + j;
  // p1[0][0] = 0 is stored for the later passes; within this pass it is read
  // as zero, so no thread reads the element while it is written
  if (j == 0 && q == 0 && part == 0) p1[0] = 0.0;
  const bool z0 = j == 0;
  auto gp_at = [&](int i) {  // (Sx^N p1)_i
    const BasisDev& b = c.xp;
    auto pv = [&](int r) { return (z0 && r == 0) ? 0.0 : p1[(long long)r * myc]; };
    if (b.kind == 0 || b.kind == 5) return pv(i);
    double v = 0.0;
    if (i < b.m) v = b.unit_diag ? pv(i) : pv(i) * b.diag[i];
    if (i >= 2 && i - 2 < b.m) v = (i < b.m) ? fma(pv(i - 2), b.low2[i - 2], v) : pv(i - 2) * b.low2[i - 2];
    return v;
  };
  if (part == 0) {
    double* gp = static_cast<double*>(c.s[0]) + j;
    double* fv = static_cast<double*>(c.s[2]) + j;
#pragma unroll 4
    for (int i = q; i < nx; i += 2) gp[(long long)i * myc] = gp_at(i);
    from_ortho_par<double>(c.xu, gp, myc, fv, myc, q);
  } else {
    const double inv_asp = 1.0 / c.aspect;
    double* e = static_cast<double*>(c.s[1]) + j;
    diff_par<double>(nx, 1 - q, [&](int i) { return gp_at(i); },
                     [&](int i, double d) { e[(long long)i * myc] = d * inv_asp; });
    from_ortho_par<double>(c.xu, e, myc, e, myc, 1 - q);
  }
}

// rows i < nx: convection (m_cv), x stencils of the state, right-hand sides,
// pinv_y -> s[1..3].  sub = 2 * field + parity q: the field's right-hand side
// and pinv rows on the columns of parity q (dP/dy on parity q comes from p0 on
// parity 1 - q)
__global__ void __launch_bounds__(256) k_lp_box_y2(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  ROW_PROLOGUE
  const int i = lane, ny = c.ny, myc = c.myc, mxc = c.mxc, kx = c.kx, ky = c.ky, f = sub;
  const double dt = c.dt;
  const void* f3[3] = {c.ux, c.uy, c.temp};
  const BasisDev* xb[3] = {&c.xu, &c.xu, &c.xt};
  const double* cv = static_cast<const double*>(c.m_cv);
  const double* P = static_cast<const double*>(c.p0) + (size_t)i * ny;
  const double* gpx = static_cast<const double*>(c.s[0]) + (size_t)i * ny;
  const double* bco = static_cast<const double*>(c.bc_ortho) + (size_t)i * ny;
  const double* bcd = static_cast<const double*>(c.bc_diff) + (size_t)i * ny;
  // x stencil of field ff at row i, column k (the composite x basis of each field)
  auto sx = [&](int ff, int k) -> double {
    if (k < 0 || k >= myc) return 0.0;
    const double* a = static_cast<const double*>(f3[ff]);
    const BasisDev& b = *xb[ff];
    double v = 0.0;
    bool has = false;
    if (i < mxc) { v = b.unit_diag ? a[(size_t)i * myc + k] : a[(size_t)i * myc + k] * b.diag[i]; has = true; }
    if (i >= 2 && i - 2 < mxc) {
      const double t = a[(size_t)(i - 2) * myc + k];
      v = has ? fma(t, b.low2[i - 2], v) : t * b.low2[i - 2];
    }
    return v;
  };
  // y stencil O_k = diag_k SX_k + low2_{k-2} SX_{k-2} (CD basis)
  auto oy = [&](int ff, int k) -> double {
    double v = 0.0;
    if (k < myc) v = c.ycd.unit_diag ? sx(ff, k) : sx(ff, k) * c.ycd.diag[k];
    if (k >= 2 && k - 2 < myc) v = (k < myc) ? fma(sx(ff, k - 2), c.ycd.low2[k - 2], v) : sx(ff, k - 2) * c.ycd.low2[k - 2];
    return v;
  };
  double* out = static_cast<double*>(c.s[1 + f]) + (size_t)i * myc;
  const PinvDev& pv = c.pinv_y;
  double r2 = 0.0, r4 = 0.0, g2 = 0.0;
  for (int k0 = top_par(ny, q); k0 >= 0; k0 -= 2 * kPB) {
    // the batch's loads first: stencils of the state, convection, pressure, boundary terms
    double ov[kPB], cvv[kPB], pk[kPB], xv[kPB];
#pragma unroll
    for (int e = 0; e < kPB; e++) {
      const int k = k0 - 2 * e;
      ov[e] = cvv[e] = pk[e] = xv[e] = 0.0;
      if (k < 0) continue;
      ov[e] = oy(f, k);
      if (i < kx && k < ky) cvv[e] = cv[((size_t)f * kx + i) * ky + k];
      if (f == 0) pk[e] = gpx[k];
      else if (f == 1) {
        if (k < ny - 1) pk[e] = P[k + 1];
        xv[e] = oy(2, k) + bco[k];
      } else {
        xv[e] = bcd[k];
        if (c.m_bclin && i < kx && k < ky) cvv[e] = add_bclin(cvv[e], oy(1, k), c.m_bcg, i);
      }
    }
#pragma unroll
    for (int e = 0; e < kPB; e++) {
      const int k = k0 - 2 * e;
      if (k < 0) break;
      double r;
      if (f == 0) {
        r = fnms(fnms(ov[e], pk[e], dt), cvv[e], dt);
      } else if (f == 1) {  // dP/dy at k (descending derivative recurrence), buoyancy
        double g;
        if (k == ny - 1) g = 0.0;
        else if (k >= 1) g = fmas(g2, pk[e], exact_double(2 * k + 2));
        else g = fmas(pk[e], g2, 0.5);
        g2 = g;
        r = fnms(fmas(fnms(ov[e], g, dt), xv[e], dt), cvv[e], dt);
      } else {
        r = fnms(ov[e] + xv[e], cvv[e], dt);
      }
      if (k < myc) {
        double v = r * pv.dia[k];
        if (k < myc - 2) v = fma(r2, pv.up1[k], v);
        if (k < myc - 4) v = fma(r4, pv.up2[k], v);
        out[k] = v;
      }
      r4 = r2;
      r2 = r;
    }
  }
}

// rows i < mxc: ADI y solves; ux*, uy* in place (s[4], s[5]), temperature ->
// state; A = Sy ux* -> s[1], B = Dy Sy uy* -> s[2] (mxc x ny).  sub = 2 *
// field + parity q: the field's chain of parity q, then A on parity q (ux) or
// B on parity 1 - q (uy)
__global__ void __launch_bounds__(256) k_lp_box_y3(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  ROW_PROLOGUE
  const int i = lane, ny = c.ny, myc = c.myc, f = sub;
  double* F = static_cast<double*>(c.s[4 + f]) + (size_t)i * myc;
  const FdmaRow R = fdma_row(f < 2 ? c.hu_y : c.ht_y, 0);
  {
    double xm2 = 0.0;
#pragma unroll 4
    for (int k = q; k < R.m; k += 2) {
      double v = F[k];
      if (k >= 2) v = fma(xm2, R.low[k - 2], v);
      F[k] = v;
      xm2 = v;
    }
  }
  fdma_bwd_par<double, kPBY3>(R, F, 1, q);
  bool bad = false;
  if (f == 2) {
    double* tt = static_cast<double*>(c.temp) + (size_t)i * myc;
    for (int k = q; k < myc; k += 2) {
      tt[k] = F[k];
      bad |= !finite_v(F[k]);
    }
  } else {
    for (int k = q; k < myc; k += 2) bad |= !finite_v(F[k]);
  }
  if (f == 0) {
    double* A = static_cast<double*>(c.s[1]) + (size_t)i * ny;
#pragma unroll 4
    for (int k = q; k < ny; k += 2) A[k] = stencil_lane<double>(c.ycd, F, 1, k);
  } else if (f == 1) {
    double* B = static_cast<double*>(c.s[2]) + (size_t)i * ny;
    diff_par<double, kPBY3>(ny, 1 - q, [&](int k) { return stencil_lane<double>(c.ycd, F, 1, k); },
                     [&](int k, double d) { B[k] = d; });
  }
  if (bad) atomicOr(c.status, 1u);
}

// rows i < mxc: pinv_y of the eigenbasis-transformed divergence and the
// Poisson row solve: s[6] (zf, mxc x ny) -> s[7] (mxc x myc); sub = parity
__global__ void __launch_bounds__(256) k_lp_box_y4(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  ROW_PROLOGUE
  const int i = lane, ny = c.ny, myc = c.myc;
  const double* zf = static_cast<const double*>(c.s[6]) + (size_t)i * ny;
  double* wv = static_cast<double*>(c.s[7]) + (size_t)i * myc;
  const FdmaRow R = fdma_row(c.pois_y, i);
  pinv_fwd_par<double>(c.pinv_y, R, zf, 1, wv, 1, q);
  // back substitution (FP64 in place), each result also rounded into m_z:
  // the FP32 input of the eigenbasis GEMM
  float* wf = static_cast<float*>(c.m_z) + (size_t)i * myc;
  double p2 = 0.0, p4 = 0.0;
#pragma unroll 4
  for (int j = top_par(R.m, q); j >= 0; j -= 2) {
    double v = wv[j] * R.dinv[j];
    if (j + 2 < R.m) v = fma(p2, R.up1[j], v);
    if (j + 4 < R.m) v = fma(p4, R.up2[j], v);
    wf[j] = (float)v;
    p4 = p2;
    p2 = v;
  }
}

// rows i < nx: ux = ux* - Sy+ Sy^N E ; uy = uy* - Sy+ Dy Sy^N Fv ;
// p0 = (p0 - nu div) + Sy^N Gp / dt  (scratch rows: s[6], s[7]).
// sub = 2 * part + parity q: part 0 ux, part 1 uy, part 2 p0, on parity q
__global__ void __launch_bounds__(256) k_lp_box_y5(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  ROW_PROLOGUE
  const int i = lane, ny = c.ny, myc = c.myc, mxc = c.mxc, part = sub;
  if (part == 2) {
    const double* Gp = static_cast<const double*>(c.s[0]) + (size_t)i * myc;
    double* p0 = static_cast<double*>(c.p0) + (size_t)i * ny;
    const double* dv = static_cast<const double*>(c.s[3]) + (size_t)i * ny;
#pragma unroll 4
    for (int k = q; k < ny; k += 2) {
      const double v = fnms(p0[k], dv[k], c.nu);
      p0[k] = fmas(v, stencil_lane<double>(c.ycn, Gp, 1, k), c.inv_dt);
    }
    return;
  }
  if (i >= mxc) return;
  double* d = static_cast<double*>(c.s[6 + part]) + (size_t)i * ny;
  if (part == 0) {  // Sy^N E on parity q
    const double* E = static_cast<const double*>(c.s[1]) + (size_t)i * myc;
#pragma unroll 4
    for (int k = q; k < ny; k += 2) d[k] = stencil_lane<double>(c.ycn, E, 1, k);
  } else {  // Dy Sy^N Fv on parity q (from Sy^N Fv on parity 1 - q)
    const double* Fv = static_cast<const double*>(c.s[2]) + (size_t)i * myc;
    diff_par<double, kPBY5>(ny, q, [&](int k) { return stencil_lane<double>(c.ycn, Fv, 1, k); },
                     [&](int k, double v) { d[k] = v; });
  }
  from_ortho_par<double, kPBY5>(c.ycd, d, 1, d, 1, q);
  double* u = static_cast<double*>(part == 0 ? c.ux : c.uy) + (size_t)i * myc;
  const double* us = static_cast<const double*>(c.s[4 + part]) + (size_t)i * myc;
  bool bad = false;
  for (int k = q; k < myc; k += 2) {
    const double a = us[k] - d[k];
    u[k] = a;
    bad |= !finite_v(a);
  }
  if (bad) atomicOr(c.status, 1u);
}

// ============================================================================
// Periodic Y2 (rows i < mx, complex): right-hand sides, pinv_y, per-row
// Helmholtz solves, divergence, Poisson row solve (p1[0,0] = 0), projection
// and the pres[0] update, from the convection term m_cv (navier.rs:622-721).
// Scratch rows (ny): yw[0] div, yw[1] dp/dx, yw[2] dp/dy.
// ============================================================================
__global__ void __launch_bounds__(128) k_lp_per_y2(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  LANE_PROLOGUE
  const int i = lane, ny = c.ny, myc = c.myc, kx = c.kx, ky = c.ky;
  const double dt = c.dt, inv_asp = 1.0 / c.aspect, ki = (double)i;
  double2* F[3] = {static_cast<double2*>(c.ux) + (size_t)i * myc, static_cast<double2*>(c.uy) + (size_t)i * myc,
                   static_cast<double2*>(c.temp) + (size_t)i * myc};
  double2* P = static_cast<double2*>(c.p0) + (size_t)i * ny;
  const double2* cv = static_cast<const double2*>(c.m_cv);
  const double2* bco = static_cast<const double2*>(c.bc_ortho) + (size_t)i * ny;
  const double2* bcd = static_cast<const double2*>(c.bc_diff) + (size_t)i * ny;
  double2* dvr = static_cast<double2*>(c.yw[0]) + (size_t)i * ny;
  double2* dpx = static_cast<double2*>(c.yw[1]) + (size_t)i * ny;
  double2* dpy = static_cast<double2*>(c.yw[2]) + (size_t)i * ny;
  double2* p1 = static_cast<double2*>(c.p1) + (size_t)i * myc;
  const PinvDev& pv = c.pinv_y;

  // 1. descending k: O_f = Sy F_f, dP/dy, right-hand sides, pinv rows (in place
  //    over the state rows: F_k is last read at step k)
  {
    DescDiff<double2> G(ny);
    double2 R[3][5];
    for (int f = 0; f < 3; f++)
      for (int q = 0; q < 5; q++) R[f][q] = c2(0.0, 0.0);
    for (int k = ny - 1; k >= 0; k--) {
      double2 O[3];
      for (int f = 0; f < 3; f++) O[f] = stencil_lane<double2>(c.ycd, F[f], 1, k);
      const double2 pk = P[k];
      const double2 g = G.step(k, pk);
      const bool incv = i < kx && k < ky;
      const double2 c0 = incv ? cv[((size_t)0 * kx + i) * ky + k] : c2(0.0, 0.0);
      const double2 c1 = incv ? cv[((size_t)1 * kx + i) * ky + k] : c2(0.0, 0.0);
      double2 cc2 = incv ? cv[((size_t)2 * kx + i) * ky + k] : c2(0.0, 0.0);
      if (incv && c.m_bclin) cc2 = add_bclin(cc2, O[1], c.m_bcg, i);
      for (int f = 0; f < 3; f++)
        for (int q = 4; q > 0; q--) R[f][q] = R[f][q - 1];
      const double2 gx = mul_ik(pk, ki) * inv_asp;
      R[0][0] = fnms(fnms(O[0], gx, dt), c0, dt);
      const double2 that = O[2] + bco[k];
      R[1][0] = fnms(fmas(fnms(O[1], g, dt), that, dt), c1, dt);
      R[2][0] = fnms(O[2] + bcd[k], cc2, dt);
      if (k < myc)
        for (int f = 0; f < 3; f++) {
          double2 v = scal(R[f][0], pv.dia[k]);
          if (k < myc - 2) v = fmas(v, R[f][2], pv.up1[k]);
          if (k < myc - 4) v = fmas(v, R[f][4], pv.up2[k]);
          F[f][k] = v;
        }
    }
  }
  // 2./3. the rows' banded Helmholtz solves: ux*, uy* (hu_y), temperature (ht_y)
  for (int f = 0; f < 3; f++) {
    const FdmaRow R = fdma_row(f < 2 ? c.hu_y : c.ht_y, i);
    fdma_fwd_lane<double2>(R, F[f], 1);
    fdma_bwd_lane<double2>(R, F[f], 1);
  }
  // 4. divergence = ik/s Sy ux* + Dy Sy uy* (descending), pinv rows -> p1
  {
    DescDiff<double2> G(ny);
    double2 W[5];
    for (int q = 0; q < 5; q++) W[q] = c2(0.0, 0.0);
    for (int k = ny - 1; k >= 0; k--) {
      const double2 o0 = stencil_lane<double2>(c.ycd, F[0], 1, k);
      const double2 g = G.step(k, stencil_lane<double2>(c.ycd, F[1], 1, k));
      const double2 d = mul_ik(o0, ki) * inv_asp + g;
      dvr[k] = d;
      for (int q = 4; q > 0; q--) W[q] = W[q - 1];
      W[0] = d;
      if (k < myc) {
        double2 v = scal(W[0], pv.dia[k]);
        if (k < myc - 2) v = fmas(v, W[2], pv.up1[k]);
        if (k < myc - 4) v = fmas(v, W[4], pv.up2[k]);
        p1[k] = v;
      }
    }
  }
  // 5./6. Poisson row solve -> pseudo pressure row (p1[0,0] = 0)
  {
    const FdmaRow R = fdma_row(c.pois_y, i);
    fdma_fwd_lane<double2>(R, p1, 1);
    fdma_bwd_lane<double2>(R, p1, 1);
    if (i == 0) p1[0] = c2(0.0, 0.0);
  }
  // 7. projection gradients (descending): O1 = Sy^N p1, dp/dy = Dy O1, dp/dx = ik/s O1;
  //    pres[0] = (pres[0] - nu div) + O1 / dt
  {
    DescDiff<double2> G(ny);
    for (int k = ny - 1; k >= 0; k--) {
      const double2 o1 = stencil_lane<double2>(c.ycn, p1, 1, k);
      dpy[k] = G.step(k, o1);
      dpx[k] = mul_ik(o1, ki) * inv_asp;
      const double2 v = fnms(P[k], dvr[k], c.nu);
      P[k] = fmas(v, o1, c.inv_dt);
    }
  }
  // 8./9. from_ortho of the gradients and the velocity update
  from_ortho_lane<double2>(c.ycd, dpx, 1, dpx, 1);
  from_ortho_lane<double2>(c.ycd, dpy, 1, dpy, 1);
  bool bad = false;
  for (int k = 0; k < myc; k++) {
    const double2 a = F[0][k] - dpx[k];
    const double2 b = F[1][k] - dpy[k];
    F[0][k] = a;
    F[1][k] = b;
    bad |= !(finite_v(a) && finite_v(b) && finite_v(F[2][k]));
  }
  if (bad) atomicOr(c.status, 1u);
}

// ============================================================================
// Periodic Y2 as three launches of one thread per sub-lane (rows i < mx,
// complex).  Y2A writes the Helmholtz solutions to scratch (yw[3..5]) because
// the uy right-hand side reads the old temperature; Y2C moves them into the
// state.  Same operations as k_lp_per_y2 (navier.rs:622-721).
// ============================================================================
// Y2A, field f, parity q: right-hand side, pinv rows and the row's banded
// Helmholtz solve of one field on the columns of parity q
template <int PB = kPBC>
__device__ __forceinline__ void per_y2a_row(const CaseDev& c, const int i, const int q, const int f) {
  const int ny = c.ny, myc = c.myc, kx = c.kx, ky = c.ky;
  const double dt = c.dt, inv_asp = 1.0 / c.aspect, kis = (double)i * inv_asp;  // ik/s
  const void* st3[3] = {c.ux, c.uy, c.temp};
  const double2* Fo = static_cast<const double2*>(st3[f]) + (size_t)i * myc;
  const double2* To = static_cast<const double2*>(c.temp) + (size_t)i * myc;
  const double2* Uo = static_cast<const double2*>(c.uy) + (size_t)i * myc;
  const double2* P = static_cast<const double2*>(c.p0) + (size_t)i * ny;
  const double2* cv = static_cast<const double2*>(c.m_cv);
  const double2* bco = static_cast<const double2*>(c.bc_ortho) + (size_t)i * ny;
  const double2* bcd = static_cast<const double2*>(c.bc_diff) + (size_t)i * ny;
  double2* out = static_cast<double2*>(c.yw[3 + f]) + (size_t)i * ny;
  const PinvDev& pv = c.pinv_y;
  double2 r2 = c2(0.0, 0.0), r4 = c2(0.0, 0.0), g2 = c2(0.0, 0.0);
  for (int k0 = top_par(ny, q); k0 >= 0; k0 -= 2 * PB) {
    // the batch's loads first (stencil, convection, pressure, boundary terms)
    double2 ov[PB], cvv[PB], pk[PB], xv[PB];
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int k = k0 - 2 * e;
      ov[e] = cvv[e] = pk[e] = xv[e] = c2(0.0, 0.0);
      if (k < 0) continue;
      ov[e] = stencil_lane<double2>(c.ycd, Fo, 1, k);
      if (i < kx && k < ky) cvv[e] = cv[((size_t)f * kx + i) * ky + k];
      if (f == 0) pk[e] = P[k];
      else if (f == 1) {
        if (k < ny - 1) pk[e] = P[k + 1];
        xv[e] = stencil_lane<double2>(c.ycd, To, 1, k) + bco[k];
      } else {
        xv[e] = bcd[k];
        if (c.m_bclin && i < kx && k < ky) cvv[e] = add_bclin(cvv[e], stencil_lane<double2>(c.ycd, Uo, 1, k), c.m_bcg, i);
      }
    }
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int k = k0 - 2 * e;
      if (k < 0) break;
      const double2 o = ov[e], cvk = cvv[e];
      double2 r;
      if (f == 0) {
        const double2 gx = mul_ik(pk[e], kis);
        r = fnms(fnms(o, gx, dt), cvk, dt);
      } else if (f == 1) {  // dP/dy at k (descending derivative recurrence), buoyancy
        double2 g;
        if (k == ny - 1) g = c2(0.0, 0.0);
        else if (k >= 1) g = fmas(g2, pk[e], exact_double(2 * k + 2));
        else g = fmas(pk[e], g2, 0.5);
        g2 = g;
        r = fnms(fmas(fnms(o, g, dt), xv[e], dt), cvk, dt);
      } else {
        r = fnms(o + xv[e], cvk, dt);
      }
      if (k < myc) {
        double2 v = scal(r, pv.dia[k]);
        if (k < myc - 2) v = fmas(v, r2, pv.up1[k]);
        if (k < myc - 4) v = fmas(v, r4, pv.up2[k]);
        out[k] = v;
      }
      r4 = r2;
      r2 = r;
    }
  }
  const FdmaRow R = fdma_row(f < 2 ? c.hu_y : c.ht_y, i);
  fdma_fwd_par<double2, PB>(R, out, 1, q);
  fdma_bwd_par<double2, PB>(R, out, 1, q);
}
__global__ void __launch_bounds__(256) k_lp_per_y2a(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  ROW_PROLOGUE
  per_y2a_row(c, lane, q, sub);
}

// Y2B, parity q: divergence ik/s Sy ux* + Dy Sy uy* on parity q (from uy* on
// parity 1 - q), pinv rows and the Poisson row solve -> p1 (p1[0,0] = 0)
template <int PB = kPBCB>
__device__ __forceinline__ void per_y2b_row(const CaseDev& c, const int i, const int q) {
  const int ny = c.ny, myc = c.myc;
  const double inv_asp = 1.0 / c.aspect, kis = (double)i * inv_asp;  // ik/s
  const double2* U = static_cast<const double2*>(c.yw[3]) + (size_t)i * ny;
  const double2* V = static_cast<const double2*>(c.yw[4]) + (size_t)i * ny;
  double2* dvr = static_cast<double2*>(c.yw[0]) + (size_t)i * ny;
  double2* p1 = static_cast<double2*>(c.p1) + (size_t)i * myc;
  const PinvDev& pv = c.pinv_y;
  double2 g2 = c2(0.0, 0.0), w2 = c2(0.0, 0.0), w4 = c2(0.0, 0.0);
  for (int k0 = top_par(ny, q); k0 >= 0; k0 -= 2 * PB) {
    double2 ov[PB], vv[PB];  // Sy ux* at k, Sy uy* at k + 1
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int k = k0 - 2 * e;
      ov[e] = vv[e] = c2(0.0, 0.0);
      if (k < 0) continue;
      ov[e] = stencil_lane<double2>(c.ycd, U, 1, k);
      if (k < ny - 1) vv[e] = stencil_lane<double2>(c.ycd, V, 1, k + 1);
    }
#pragma unroll
    for (int e = 0; e < PB; e++) {
      const int k = k0 - 2 * e;
      if (k < 0) break;
      double2 g;
      if (k == ny - 1) g = c2(0.0, 0.0);
      else if (k >= 1) g = fmas(g2, vv[e], exact_double(2 * k + 2));
      else g = fmas(vv[e], g2, 0.5);
      g2 = g;
      const double2 d = c2(fma(-ov[e].y, kis, g.x), fma(ov[e].x, kis, g.y));  // ik/s Sy ux* + g
      dvr[k] = d;
      if (k < myc) {
        double2 v = scal(d, pv.dia[k]);
        if (k < myc - 2) v = fmas(v, w2, pv.up1[k]);
        if (k < myc - 4) v = fmas(v, w4, pv.up2[k]);
        p1[k] = v;
      }
      w4 = w2;
      w2 = d;
    }
  }
  const FdmaRow R = fdma_row(c.pois_y, i);
  fdma_fwd_par<double2, PB>(R, p1, 1, q);
  fdma_bwd_par<double2, PB>(R, p1, 1, q);
  if (i == 0 && q == 0) p1[0] = c2(0.0, 0.0);
}
__global__ void __launch_bounds__(256) k_lp_per_y2b(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  ROW_PROLOGUE
  per_y2b_row(c, lane, q);
}

// Y2C, parity q and part: part 0: O1 = Sy^N p1, dp/dx, pres[0] and ux,
// temperature on parity q; part 1: dp/dy on parity 1 - q and uy there
template <int PB = kPBCC>
__device__ __forceinline__ void per_y2c_row(const CaseDev& c, const int i, const int q, const int part) {
  const int ny = c.ny, myc = c.myc;
  const double inv_asp = 1.0 / c.aspect, kis = (double)i * inv_asp;  // ik/s
  const double2* p1 = static_cast<const double2*>(c.p1) + (size_t)i * myc;
  bool bad = false;
  if (part == 0) {
    double2* dpx = static_cast<double2*>(c.yw[1]) + (size_t)i * ny;
    double2* P = static_cast<double2*>(c.p0) + (size_t)i * ny;
    const double2* dvr = static_cast<const double2*>(c.yw[0]) + (size_t)i * ny;
    for (int k0 = q; k0 < ny; k0 += 2 * PB) {
      double2 ov[PB], pv0[PB], dv[PB];
#pragma unroll
      for (int e = 0; e < PB; e++) {
        const int k = k0 + 2 * e;
        ov[e] = pv0[e] = dv[e] = c2(0.0, 0.0);
        if (k >= ny) continue;
        ov[e] = stencil_lane<double2>(c.ycn, p1, 1, k);
        pv0[e] = P[k];
        dv[e] = dvr[k];
      }
#pragma unroll
      for (int e = 0; e < PB; e++) {
        const int k = k0 + 2 * e;
        if (k >= ny) break;
        dpx[k] = mul_ik(ov[e], kis);
        const double2 v = fnms(pv0[e], dv[e], c.nu);
        P[k] = fmas(v, ov[e], c.inv_dt);
      }
    }
    from_ortho_par<double2, PB>(c.ycd, dpx, 1, dpx, 1, q);
    const double2* U = static_cast<const double2*>(c.yw[3]) + (size_t)i * ny;
    const double2* T = static_cast<const double2*>(c.yw[5]) + (size_t)i * ny;
    double2* ux = static_cast<double2*>(c.ux) + (size_t)i * myc;
    double2* tt = static_cast<double2*>(c.temp) + (size_t)i * myc;
    for (int k = q; k < myc; k += 2) {
      const double2 a = U[k] - dpx[k];
      const double2 t = T[k];
      ux[k] = a;
      tt[k] = t;
      bad |= !(finite_v(a) && finite_v(t));
    }
  } else {
    double2* dpy = static_cast<double2*>(c.yw[2]) + (size_t)i * ny;
    diff_par<double2, PB>(ny, 1 - q, [&](int k) { return stencil_lane<double2>(c.ycn, p1, 1, k); },
                      [&](int k, double2 d) { dpy[k] = d; });
    from_ortho_par<double2, PB>(c.ycd, dpy, 1, dpy, 1, 1 - q);
    const double2* V = static_cast<const double2*>(c.yw[4]) + (size_t)i * ny;
    double2* uy = static_cast<double2*>(c.uy) + (size_t)i * myc;
    for (int k = 1 - q; k < myc; k += 2) {
      const double2 b = V[k] - dpy[k];
      uy[k] = b;
      bad |= !finite_v(b);
    }
  }
  if (bad) atomicOr(c.status, 1u);
}
__global__ void __launch_bounds__(256) k_lp_per_y2c(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  ROW_PROLOGUE
  per_y2c_row(c, lane, q, sub);
}

// The three phases in one launch: a CTA of three 64-thread groups per work
// item of up to 32 rows runs Y2A (group = field), then Y2B (group 0), then
// Y2C (groups 0 and 1 = part), with a CTA barrier between the phases.  Every
// array a phase reads is a row of this item's, written by the CTA's own
// threads before the barrier, which makes those writes visible to it; each
// thread does the arithmetic of the three launches (the elements loaded ahead
// change only the order of the loads), so the results are the same.  The
// rows' intermediates are re-read while they are still in L1/L2, and two
// launch tails go.  Four elements ahead in every phase (128 registers) was
// the fastest of (2..4, 2..6, 2..8) on the 256-case ensemble: 1.07 ms against
// 1.13 ms for the three launches.
__global__ void __launch_bounds__(3 * kLaneBlock) k_lp_per_y2f(const CaseDev* __restrict__ cases,
                                                               const int4* __restrict__ work) {
  const int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // the whole CTA: no barrier is left waiting
  const int t = (int)(threadIdx.x % kLaneBlock), grp = (int)(threadIdx.x / kLaneBlock);
  const bool active = (t >> 1) < w.z;
  const int lane = w.y + (t >> 1), q = t & 1;
  if (active) per_y2a_row<4>(c, lane, q, grp);
  __syncthreads();
  if (active && grp == 0) per_y2b_row<4>(c, lane, q);
  __syncthreads();
  if (active && grp < 2) per_y2c_row<4>(c, lane, q, grp);
}

#undef LANE_PROLOGUE

}  // namespace dev

// grid.y of each one-thread-per-lane kernel: column kernels put (field,
// parity) sub-lanes there; row kernels put the field or part there and the
// parity on adjacent threads (256 threads for 128 lanes)
int lane_kernel_subs(int kernel) {
  switch (kernel) {
    case K_LP_BOX_X2: return 6;
    case K_LP_BOX_GPX: case K_LP_BOX_X3: return 2;
    case K_LP_BOX_X4: return 4;
    case K_LP_BOX_Y2: case K_LP_BOX_Y3: case K_LP_BOX_Y5: case K_LP_PER_Y2A: return 3;
    case K_LP_PER_Y2C: return 2;
    default: return 1;
  }
}
bool lane_kernel_rows(int kernel) {
  switch (kernel) {
    case K_LP_BOX_Y2: case K_LP_BOX_Y3: case K_LP_BOX_Y4: case K_LP_BOX_Y5:
    case K_LP_PER_Y2A: case K_LP_PER_Y2B: case K_LP_PER_Y2C: case K_LP_PER_Y2F: return true;
    default: return false;
  }
}

cudaError_t launch_lane_kernel(int kernel, int nblocks, cudaStream_t s, const CaseDev* cases, const int4* work) {
  dim3 g(nblocks, lane_kernel_subs(kernel)), b(kernel == K_LP_PER_Y2F ? 3 * kLaneBlock : kLaneBlock);
  switch (kernel) {
    case K_LP_BOX_GPX: dev::k_lp_box_gpx<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_BOX_X2: dev::k_lp_box_x2<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_BOX_X3: dev::k_lp_box_x3<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_BOX_X4: dev::k_lp_box_x4<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_BOX_Y2: dev::k_lp_box_y2<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_BOX_Y3: dev::k_lp_box_y3<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_BOX_Y4: dev::k_lp_box_y4<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_BOX_Y5: dev::k_lp_box_y5<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_PER_Y2: dev::k_lp_per_y2<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_PER_Y2A: dev::k_lp_per_y2a<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_PER_Y2B: dev::k_lp_per_y2b<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_PER_Y2C: dev::k_lp_per_y2c<<<g, b, 0, s>>>(cases, work); break;
    case K_LP_PER_Y2F: dev::k_lp_per_y2f<<<g, b, 0, s>>>(cases, work); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace rbc
