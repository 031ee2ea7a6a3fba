// lane_ops.cuh -- CTA-cooperative 1-D operations on lanes held in shared memory.
//
// A "lane" is one 1-D line of a 2-D field along the axis being processed
// (a row for y passes, a column for x passes).  Each function is executed by
// all threads of the CTA (tid, nth) and ends with __syncthreads().  Lanes of
// the same call are stored at base + l*ld.  T is double (real data) or
// double2 (complex data, interleaved re/im).
//
// Operations and the reference code they restate:
//   to_ortho / from_ortho   funspace/src/chebyshev/composite_stencil.rs:207-276, linalg.rs:14-57
//   cheb_diff               funspace/src/chebyshev/ortho.rs:107-125
//   matvec_pinv             src/solver/matvec.rs:172-193
//   fdma_solve              src/solver/fdma.rs:101-118 (factors swept at set-up)
//   dct1 (fwd/bwd)          funspace/src/chebyshev/ortho.rs:235-312 (DCT-I = REDFT00)
//   c2r / r2c               funspace/src/fourier/r2c.rs:160-226 (1/n on the inverse)
#pragma once
#include <cuda_runtime.h>

#include "chain_scan.cuh"
#include "rbc_dev.h"

namespace rbc {
namespace dev {


// quotient of non-negative idx < 2^31/n by n through a multiply-high
struct FastDiv {
  unsigned c;
  __device__ __forceinline__ explicit FastDiv(int n) : c(0xFFFFFFFFu / (unsigned)n + 1u) {}
  __device__ __forceinline__ int operator()(int idx) const { return (int)__umulhi((unsigned)idx, c); }
};

// ------------------------------------------------------------------ scalars
__device__ __forceinline__ double2 c2(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ double2 operator+(double2 a, double2 b) { return c2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 operator-(double2 a, double2 b) { return c2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 operator*(double2 a, double s) { return c2(a.x * s, a.y * s); }
__device__ __forceinline__ double2 cmul(double2 a, double2 w) {
  return c2(fma(a.x, w.x, -a.y * w.y), fma(a.x, w.y, a.y * w.x));
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 w) {  // a * conj(w)
  return c2(fma(a.x, w.x, a.y * w.y), fma(a.y, w.x, -a.x * w.y));
}
__device__ __forceinline__ double2 conj2(double2 a) { return c2(a.x, -a.y); }

template <class T> __device__ __forceinline__ T zero_v();
template <> __device__ __forceinline__ double zero_v<double>() { return 0.0; }
template <> __device__ __forceinline__ double2 zero_v<double2>() { return c2(0.0, 0.0); }

__device__ __forceinline__ double scal(double a, double s) { return a * s; }
__device__ __forceinline__ double2 scal(double2 a, double s) { return c2(a.x * s, a.y * s); }
// a - b*s, a + b*s (fused)
__device__ __forceinline__ double fnms(double a, double b, double s) { return fma(-b, s, a); }
__device__ __forceinline__ double2 fnms(double2 a, double2 b, double s) { return c2(fma(-b.x, s, a.x), fma(-b.y, s, a.y)); }
__device__ __forceinline__ double fmas(double a, double b, double s) { return fma(b, s, a); }
__device__ __forceinline__ double2 fmas(double2 a, double2 b, double s) { return c2(fma(b.x, s, a.x), fma(b.y, s, a.y)); }
// Temperature convection term plus the boundary-field term of a boundary
// field linear in y (CaseDev::m_bclin): ct + g * o with o = to_ortho(uy) at
// the same (dealiased) index.  On a Fourier axis, row 0 takes the real part of
// o only, as the c2r -> r2c round trip of the product does.
__device__ __forceinline__ double add_bclin(double ct, double o, double g, int) { return fma(o, g, ct); }
__device__ __forceinline__ double2 add_bclin(double2 ct, double2 o, double g, int row) {
  return row == 0 ? c2(fma(o.x, g, ct.x), ct.y) : c2(fma(o.x, g, ct.x), fma(o.y, g, ct.y));
}
// finiteness from the exponent bits (integer operations: comparisons and
// conversions of doubles run at the FP64 rate on this GPU)
__device__ __forceinline__ bool finite_v(double a) {
  return ((unsigned long long)__double_as_longlong(a) & 0x7FF0000000000000ull) != 0x7FF0000000000000ull;
}
__device__ __forceinline__ bool finite_v(double2 a) { return finite_v(a.x) && finite_v(a.y); }
// n (1 <= n < 2^31) as a double, assembled from its bits with integer
// operations; equal to (double)n
__device__ __forceinline__ double exact_double(int n) {
  const int e = 31 - __clz(n);  // 2^e <= n < 2^(e+1)
  const unsigned long long mant = ((unsigned long long)(unsigned)n << (52 - e)) & ((1ull << 52) - 1ull);
  return __longlong_as_double((long long)(((unsigned long long)(1023 + e) << 52) | mant));
}

// multiply by i*k / s  (Fourier derivative of order 1, then division by the scale)
__device__ __forceinline__ double2 mul_ik(double2 a, double k) { return c2(-a.y * k, a.x * k); }

// ------------------------------------------------------------------ stencils
// composite -> ortho along a lane: p_i = diag_i c_i + low2_{i-2} c_{i-2}
template <class T>
__device__ __forceinline__ T stencil_at(const BasisDev& b, const T* c, int i) {
  int n = b.n, m = b.m;
  if (b.kind == 0 || b.kind == 5) return c[i];  // Chebyshev / Fourier: identity
  if (b.kind == 3 || b.kind == 4) {             // boundary basis
    if (i == 0) return fmas(scal(c[0], b.t0[0]), c[1], b.t0[1]);
    if (i == 1) return fmas(scal(c[0], b.t1[0]), c[1], b.t1[1]);
    return zero_v<T>();
  }
  T v = zero_v<T>();
  if (i < m) v = b.unit_diag ? c[i] : scal(c[i], b.diag[i]);
  if (i >= 2 && i - 2 < m) v = (i < m) ? fmas(v, c[i - 2], b.low2[i - 2]) : scal(c[i - 2], b.low2[i - 2]);
  (void)n;
  return v;
}

template <class T>
static __device__ void to_ortho(const BasisDev& b, const T* in, int in_ld, T* out, int out_ld, int nl, int tid, int nth) {
  int n = (b.kind == 5) ? b.m : b.n;
  const FastDiv dn(n);
  for (int idx = tid; idx < nl * n; idx += nth) {
    int l = dn(idx), i = idx - l * n;
    out[l * out_ld + i] = stencil_at(b, in + l * in_ld, i);
  }
  __syncthreads();
}

// ortho -> composite (least squares, stride-2 tridiagonal).  in and out may not alias.
template <class T>
static __device__ void from_ortho(const BasisDev& b, const T* in, int in_ld, T* out, int out_ld, int nl, int tid, int nth) {
  int m = b.m;
  if (b.kind == 0 || b.kind == 5) {
    for (int idx = tid; idx < nl * m; idx += nth) {
      int l = idx / m, i = idx - l * m;
      out[l * out_ld + i] = in[l * in_ld + i];
    }
    __syncthreads();
    return;
  }
  if (b.kind == 3 || b.kind == 4) {
    for (int l = tid; l < nl; l += nth) {
      const T* p = in + l * in_ld;
      T c0 = fmas(scal(p[0], b.t0[0]), p[1], b.t1[0]);
      T c1 = fmas(scal(p[0], b.t0[1]), p[1], b.t1[1]);
      out[l * out_ld + 0] = fmas(scal(c0, b.bc_inv[0]), c1, b.bc_inv[1]);
      out[l * out_ld + 1] = fmas(scal(c0, b.bc_inv[2]), c1, b.bc_inv[3]);
    }
    __syncthreads();
    return;
  }
  const FastDiv dm(m);
  for (int idx = tid; idx < nl * m; idx += nth) {
    int l = dm(idx), i = idx - l * m;
    const T* p = in + l * in_ld;
    out[l * out_ld + i] = fmas(b.unit_diag ? p[i] : scal(p[i], b.diag[i]), p[i + 2], b.low2[i]);
  }
  __syncthreads();
  // forward g_i = (d_i - a_{i-2} g_{i-2}) / den_i, then x_j = g_j - w_j x_{j+2},
  // one group of threads per (lane, parity) chain
  const double* __restrict__ off = b.fo_off;
  const double* __restrict__ dinv = b.fo_dinv;
  const double* __restrict__ w = b.fo_w;
  auto len_of = [&](int c) { return (m - (c & 1) + 1) >> 1; };
  chains1<16, T>(
      2 * nl, len_of,
      [&](int c, int t, double& a, T& v) {
        int i = (c & 1) + 2 * t;
        T d = out[(c >> 1) * out_ld + i];
        double q = dinv[i];
        a = t ? -off[i - 2] * q : 0.0;
        v = scal(d, q);
      },
      [&](int c, int t, T x) { out[(c >> 1) * out_ld + (c & 1) + 2 * t] = x; }, tid, nth);
  __syncthreads();
  auto top_of = [&](int c) { int par = c & 1; return ((m - 1 - par) & 1) ? m - 2 : m - 1; };
  chains1<16, T>(
      2 * nl, len_of,
      [&](int c, int t, double& a, T& v) {
        int j = top_of(c) - 2 * t;
        v = out[(c >> 1) * out_ld + j];
        a = t ? -w[j] : 0.0;
      },
      [&](int c, int t, T x) { out[(c >> 1) * out_ld + top_of(c) - 2 * t] = x; }, tid, nth);
  __syncthreads();
}

// ------------------------------------------------------------------ derivatives
// Chebyshev derivative of order `times` (1 or 2) of ortho lanes: out = D^times in
// (in and out may alias only if times == 0).
template <class T>
static __device__ void cheb_diff(const T* in, int in_ld, T* out, int out_ld, int n, int nl, int times, T* tmp, int tmp_ld,
                          int tid, int nth) {
  if (times == 0) {
    if (in != out)
      for (int idx = tid; idx < nl * n; idx += nth) {
        int l = idx / n, i = idx - l * n;
        out[l * out_ld + i] = in[l * in_ld + i];
      }
    __syncthreads();
    return;
  }
  const T* src = in;
  int src_ld = in_ld;
  for (int t = 0; t < times; t++) {
    T* dst = (t == times - 1) ? out : tmp;
    int dst_ld = (t == times - 1) ? out_ld : tmp_ld;
    // d_0 = a_1; d_i = 2(i+1) a_{i+1} (1 <= i <= n-2); d_{n-1} = 0
    const FastDiv dn(n);
    for (int idx = tid; idx < nl * n; idx += nth) {
      int l = dn(idx), i = idx - l * n;
      const T* a = src + l * src_ld;
      T v;
      if (i == 0) v = a[1];
      else if (i < n - 1) v = scal(a[i + 1], exact_double(2 * i + 2));
      else v = zero_v<T>();
      dst[l * dst_ld + i] = v;
    }
    __syncthreads();
    // suffix sums d_i += d_{i+2} for i = n-3 .. 1 (per parity), then d_0 += d_2 / 2
    {
      T* dd = dst;
      const int dl = dst_ld;
      auto top2 = [&](int c) { int par = c & 1; return ((n - 3 - par) & 1) ? n - 2 : n - 1; };  // start element
      auto len_of = [&](int c) {
        int par = c & 1, st = top2(c), lo = par ? 1 : 2;
        return st >= lo ? (st - lo) / 2 + 1 : 1;
      };
      chains1<16, T>(
          2 * nl, len_of,
          [&](int c, int t, double& a, T& v) {
            v = dd[(c >> 1) * dl + top2(c) - 2 * t];
            a = t ? 1.0 : 0.0;
          },
          [&](int c, int t, T x) { dd[(c >> 1) * dl + top2(c) - 2 * t] = x; }, tid, nth);
      __syncthreads();
      for (int l = tid; l < nl; l += nth) dd[l * dl] = fmas(dd[l * dl], dd[l * dl + 2], 0.5);
      __syncthreads();
    }
    src = dst;
    src_ld = dst_ld;
  }
}

// ------------------------------------------------------------------ banded solvers
// out (n-2 per lane) = pinv(n) * in (n per lane)
template <class T>
static __device__ void matvec_pinv(const PinvDev& p, const T* in, int in_ld, T* out, int out_ld, int nl, int tid, int nth) {
  int m = p.n - 2;
  const FastDiv dm(m);
  for (int idx = tid; idx < nl * m; idx += nth) {
    int l = dm(idx), i = idx - l * m;
    const T* a = in + l * in_ld;
    T v = scal(a[i], p.dia[i]);
    if (i < m - 2) v = fmas(v, a[i + 2], p.up1[i]);
    if (i < m - 4) v = fmas(v, a[i + 4], p.up2[i]);
    out[l * out_ld + i] = v;
  }
  __syncthreads();
}

// In-place banded solve with swept factors (offsets -2, 0, 2, 4; fdma.rs:101-118).
// FdmaDev stores low = -low_swept, dinv = 1/dia, up1 = -up1/dia, up2 = -up2/dia.
// Lanes l < split use factor set f0, the others f1; a factor set with rows > 1
// gives lane l the row (row0 + l*lane_step).
template <class T>
__device__ void fdma_solve2(const FdmaDev& f0, const FdmaDev& f1, int split, T* x, int ld, int nl, int row0,
                            int lane_step, int tid, int nth) {
  const int m = f0.m;
  auto fac = [&](int l) -> const FdmaDev& { return l < split ? f0 : f1; };
  auto offs = [&](int l) -> size_t {
    const FdmaDev& f = fac(l);
    return (f.rows > 1) ? (size_t)(row0 + l * lane_step) * f.stride : 0;
  };
  auto len_of = [&](int c) { return (m - (c & 1) + 1) >> 1; };
  // forward elimination x_i -= low_{i-2} x_{i-2}
  chains1<16, T>(
      2 * nl, len_of,
      [&](int c, int t, double& a, T& v) {
        int l = c >> 1, i = (c & 1) + 2 * t;
        v = x[l * ld + i];
        a = t ? fac(l).low[offs(l) + i - 2] : 0.0;
      },
      [&](int c, int t, T v) { x[(c >> 1) * ld + (c & 1) + 2 * t] = v; }, tid, nth);
  __syncthreads();
  // back substitution x_j = (x_j - up1_j x_{j+2} - up2_j x_{j+4}) / dia_j
  auto top_of = [&](int c) { int par = c & 1; return ((m - 1 - par) & 1) ? m - 2 : m - 1; };
  chains2<16, T>(
      2 * nl, len_of,
      [&](int c, int t, double& a, double& cc, T& v) {
        int l = c >> 1, j = top_of(c) - 2 * t;
        const FdmaDev& f = fac(l);
        size_t o = offs(l);
        v = scal(x[l * ld + j], f.dinv[o + j]);
        a = t ? f.up1[o + j] : 0.0;
        cc = t >= 2 ? f.up2[o + j] : 0.0;
      },
      [&](int c, int t, T v) { x[(c >> 1) * ld + top_of(c) - 2 * t] = v; }, tid, nth);
  __syncthreads();
}

template <class T>
__device__ void fdma_solve(const FdmaDev& f, T* x, int ld, int nl, int row0, int lane_step, int tid, int nth) {
  fdma_solve2<T>(f, f, nl, x, ld, nl, row0, lane_step, tid, nth);
}

// ------------------------------------------------------------------ FFT
// Radix-4 (+ one radix-2) Stockham complex FFT of nl lanes of length L = 2^log2L
// held in a (lane stride ld).  tw has length twL (multiple of L), tw[t] =
// exp(-2 pi i t / twL).  Forward uses exp(-...), inverse exp(+...), both
// unnormalised.  Returns the buffer (a or b) holding the result.
__device__ __forceinline__ double2* fft_pow2(double2* a, double2* b, int L, int log2L, int nl, int ld,
                                              const double2* __restrict__ tw, int twL, bool inv, int tid, int nth) {
  int Ns = 1;
  if (log2L & 1) {
    int half = L >> 1;
    for (int idx = tid; idx < nl * half; idx += nth) {
      int l = idx >> (log2L - 1), j = idx & (half - 1);
      double2 v0 = a[l * ld + j], v1 = a[l * ld + j + half];
      b[l * ld + 2 * j] = v0 + v1;
      b[l * ld + 2 * j + 1] = v0 - v1;
    }
    __syncthreads();
    double2* t = a; a = b; b = t;
    Ns = 2;
  }
  int quarter = L >> 2;
  int lq = log2L - 2;
  while (Ns < L) {
    int tstep = twL / (Ns * 4);
    for (int idx = tid; idx < nl * quarter; idx += nth) {
      int l = idx >> lq, j = idx & (quarter - 1);
      const double2* src = a + l * ld;
      double2 v0 = src[j], v1 = src[j + quarter], v2 = src[j + 2 * quarter], v3 = src[j + 3 * quarter];
      int jm = j & (Ns - 1);
      if (jm) {
        int e = jm * tstep;
        double2 w1 = tw[e], w2 = tw[2 * e], w3 = tw[3 * e];
        if (inv) { v1 = cmulc(v1, w1); v2 = cmulc(v2, w2); v3 = cmulc(v3, w3); }
        else { v1 = cmul(v1, w1); v2 = cmul(v2, w2); v3 = cmul(v3, w3); }
      }
      double2 s0 = v0 + v2, d0 = v0 - v2, s1 = v1 + v3, d1 = v1 - v3;
      // forward: d1 * (-i) ; inverse: d1 * (+i)
      double2 r = inv ? c2(-d1.y, d1.x) : c2(d1.y, -d1.x);
      double2* dst = b + l * ld + (j - jm) * 4 + jm;
      dst[0] = s0 + s1;
      dst[Ns] = d0 + r;
      dst[2 * Ns] = s0 - s1;
      dst[3 * Ns] = d0 - r;
    }
    __syncthreads();
    double2* t = a; a = b; b = t;
    Ns <<= 2;
  }
  return a;
}

// ------------------------------------------------------------------ FFT of any length
// Complex arithmetic for the two lane types (the FP64 form and the FP32
// mixed form share the mixed-radix FFT below).
__device__ __forceinline__ double2 cx_add(double2 a, double2 b) { return c2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cx_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cx_sub(double2 a, double2 b) { return c2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cx_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// a * w (forward) or a * conj(w) (inverse)
__device__ __forceinline__ double2 cx_tw(double2 a, double2 w, bool inv) { return inv ? cmulc(a, w) : cmul(a, w); }
__device__ __forceinline__ float2 cx_tw(float2 a, float2 w, bool inv) {
  return inv ? make_float2(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y)
             : make_float2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
}
// a * (-i) (forward) or a * (+i) (inverse)
__device__ __forceinline__ double2 cx_rot(double2 a, bool inv) { return inv ? c2(-a.y, a.x) : c2(a.y, -a.x); }
__device__ __forceinline__ float2 cx_rot(float2 a, bool inv) {
  return inv ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// Stockham autosort FFT of nl lanes of length L = rad[0] * ... * rad[nrad-1]
// (lane stride ld), unnormalised, exp(-+2 pi i jk / L).  tw[t] =
// exp(-2 pi i t / twL) with L dividing twL.  Stage s of radix p, after
// sub-transforms of length Ns: input j + r L/p (r < p) is twiddled by
// w^(r (j mod Ns)), w = exp(-2 pi i / (Ns p)), and the p-point DFT's output q
// goes to (j - j mod Ns) p + (j mod Ns) + q Ns.  Radix 4 and 2 use the
// butterflies; other radices the direct p-point DFT through the same table.
// Returns the buffer that holds the result (a or b).
template <class C>
__device__ C* fft_mixed(C* a, C* b, int L, const int* rad, int nrad, int nl, int ld, const C* __restrict__ tw,
                        int twL, bool inv, int tid, int nth) {
  int Ns = 1;
  for (int st = 0; st < nrad; st++) {
    const int p = rad[st];
    const int Lp = L / p;
    const int tstep = twL / (Ns * p);  // w = tw[tstep]
    const int pstep = twL / p;         // exp(-2 pi i / p) = tw[pstep]
    for (int idx = tid; idx < nl * Lp; idx += nth) {
      const int l = idx / Lp, j = idx - l * Lp;
      const int jm = j % Ns;
      const C* src = a + (size_t)l * ld + j;
      C* dst = b + (size_t)l * ld + (j - jm) * p + jm;
      if (p == 4) {
        C v0 = src[0], v1 = src[Lp], v2 = src[2 * Lp], v3 = src[3 * Lp];
        if (jm) {
          const int e = jm * tstep;
          v1 = cx_tw(v1, tw[e], inv);
          v2 = cx_tw(v2, tw[2 * e], inv);
          v3 = cx_tw(v3, tw[3 * e], inv);
        }
        const C s0 = cx_add(v0, v2), d0 = cx_sub(v0, v2), s1 = cx_add(v1, v3);
        const C r = cx_rot(cx_sub(v1, v3), inv);
        dst[0] = cx_add(s0, s1);
        dst[Ns] = cx_add(d0, r);
        dst[2 * Ns] = cx_sub(s0, s1);
        dst[3 * Ns] = cx_sub(d0, r);
      } else if (p == 2) {
        C v0 = src[0], v1 = src[Lp];
        if (jm) v1 = cx_tw(v1, tw[jm * tstep], inv);
        dst[0] = cx_add(v0, v1);
        dst[Ns] = cx_sub(v0, v1);
      } else if (p <= 8) {
        C v[8];
        for (int r = 0; r < p; r++) {
          v[r] = src[(size_t)r * Lp];
          if (jm && r) v[r] = cx_tw(v[r], tw[r * jm * tstep], inv);
        }
        for (int q = 0; q < p; q++) {
          C acc = v[0];
          for (int r = 1; r < p; r++) {
            const int e = (r * q) % p;
            acc = cx_add(acc, e ? cx_tw(v[r], tw[e * pstep], inv) : v[r]);
          }
          dst[q * Ns] = acc;
        }
      } else {  // a large prime factor: the inputs are twiddled again for every output
        for (int q = 0; q < p; q++) {
          C acc = src[0];
          for (int r = 1; r < p; r++) {
            C vr = src[(size_t)r * Lp];
            if (jm) vr = cx_tw(vr, tw[r * jm * tstep], inv);
            const int e = (r * q) % p;
            acc = cx_add(acc, e ? cx_tw(vr, tw[e * pstep], inv) : vr);
          }
          dst[q * Ns] = acc;
        }
      }
    }
    __syncthreads();
    C* t = a;
    a = b;
    b = t;
    Ns *= p;
  }
  return a;
}

// ------------------------------------------------------------------ Chebyshev transforms
// pre/post factors of ortho.rs:235-312 for index k of length n (N = n-1)
__device__ __forceinline__ double cheb_fwd_post(int k, int n, double inv_nm1) {
  double s = (k & 1) ? -inv_nm1 : inv_nm1;
  return (k == 0 || k == n - 1) ? s * 0.5 : s;
}
__device__ __forceinline__ double cheb_bwd_pre(int k, int n) {
  double s = (k & 1) ? -0.5 : 0.5;
  return (k == 0 || k == n - 1) ? s * 2.0 : s;
}

// Complex lanes, FFT variant (length 2N, kept for reference): out = DCT-I(pre .* in) .* post
// wa, wb: work lanes of length >= L with stride wld.
static __device__ void dct1_fft2_c(const ChebXformDev& cx, bool forward, const double2* in, int in_ld, double2* out,
                           int out_ld, int nl, double2* wa, double2* wb, int wld, int tid, int nth) {
  int n = cx.n, N = n - 1, L = cx.L;
  for (int idx = tid; idx < nl * L; idx += nth) {
    int l = idx >> cx.log2L, j = idx & (L - 1);
    int src = j <= N ? j : L - j;
    double2 v = in[l * in_ld + src];
    if (!forward) v = v * cheb_bwd_pre(src, n);
    wa[l * wld + j] = v;
  }
  __syncthreads();
  double2* r = fft_pow2(wa, wb, L, cx.log2L, nl, wld, cx.tw, L, false, tid, nth);
  for (int idx = tid; idx < nl * n; idx += nth) {
    int l = idx / n, k = idx - l * n;
    double2 v = r[l * wld + k];
    out[l * out_ld + k] = forward ? v * cheb_fwd_post(k, n, cx.inv_nm1) : v;
  }
  __syncthreads();
}

// Real lanes, FFT variant (length 2N): two real lanes per complex FFT.
static __device__ void dct1_fft2_r(const ChebXformDev& cx, bool forward, const double* in, int in_ld, double* out, int out_ld,
                           int nl, double2* wa, double2* wb, int wld, int tid, int nth) {
  int n = cx.n, N = n - 1, L = cx.L;
  int np = (nl + 1) >> 1;
  for (int idx = tid; idx < np * L; idx += nth) {
    int q = idx >> cx.log2L, j = idx & (L - 1);
    int src = j <= N ? j : L - j;
    double pre = forward ? 1.0 : cheb_bwd_pre(src, n);
    double re = in[(2 * q) * in_ld + src] * pre;
    double im = (2 * q + 1 < nl) ? in[(2 * q + 1) * in_ld + src] * pre : 0.0;
    wa[q * wld + j] = c2(re, im);
  }
  __syncthreads();
  double2* r = fft_pow2(wa, wb, L, cx.log2L, np, wld, cx.tw, L, false, tid, nth);
  for (int idx = tid; idx < nl * n; idx += nth) {
    int l = idx / n, k = idx - l * n;
    double2 v = r[(l >> 1) * wld + k];
    double s = (l & 1) ? v.y : v.x;
    out[l * out_ld + k] = forward ? s * cheb_fwd_post(k, n, cx.inv_nm1) : s;
  }
  __syncthreads();
}

// ---- DCT-I through a complex FFT of length N = n-1 (N a power of two).
// For lanes z_0..z_N (complex, or two real lanes packed as re/im):
//   Z_j = (z_j + z_{N-j}) - 2 sin(pi j/N) (z_j - z_{N-j}),   W = FFT_N(Z)
//   C_{2k}   = (W_k + W_{N-k}) / 2                     k = 0 .. N/2
//   C_{2k+1} = C_{2k-1} + (i/2) (W_k - W_{N-k})        k = 1 .. N/2-1
//   C_1      = z_0 - z_N + 2 sum_{j=1}^{N-1} z_j cos(pi j/N)
// (the pre-twiddled real-FFT route to REDFT00; the odd outputs are a prefix
// sum computed with a warp scan).  cx.tw holds exp(-i pi t / N), t < 2N.
struct DctLanesC {  // complex lanes
  const double2* in;
  int in_ld;
  double2* out;
  int out_ld;
  __device__ double2 load(int l, int j) const { return in[l * in_ld + j]; }
  __device__ void store(int l, int k, double2 v) const { out[l * out_ld + k] = v; }
};
struct DctLanesR {  // pairs of real lanes (2q, 2q+1) -> (re, im)
  const double* in;
  int in_ld;
  double* out;
  int out_ld;
  int nl;  // real lanes
  __device__ double2 load(int q, int j) const {
    double a = in[(2 * q) * in_ld + j];
    double b = (2 * q + 1 < nl) ? in[(2 * q + 1) * in_ld + j] : 0.0;
    return c2(a, b);
  }
  __device__ void store(int q, int k, double2 v) const {
    out[(2 * q) * out_ld + k] = v.x;
    if (2 * q + 1 < nl) out[(2 * q + 1) * out_ld + k] = v.y;
  }
};

template <class Lanes>
static __device__ void dct1_half(const ChebXformDev& cx, bool forward, const Lanes& io, int nl, double2* wa,
                                 double2* wb, int wld, int tid, int nth) {
  const int n = cx.n, N = n - 1, lN = cx.log2L - 1, half = N >> 1;
  const double2* __restrict__ tw = cx.tw;
  const int lane_id = tid & 31, warp = tid >> 5, nwarp = nth >> 5;
  // C_1 per lane (warp reduction), kept at wa[l*wld + N]
  for (int l = warp; l < nl; l += nwarp) {
    double2 acc = c2(0.0, 0.0);
    for (int j = 1 + lane_id; j < N; j += 32) {
      double2 v = io.load(l, j);
      if (!forward) v = v * cheb_bwd_pre(j, n);
      acc = fmas(acc, v, tw[j].x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    if (lane_id == 0) {
      double2 z0 = io.load(l, 0), zN = io.load(l, N);
      if (!forward) { z0 = z0 * cheb_bwd_pre(0, n); zN = zN * cheb_bwd_pre(N, n); }
      wa[l * wld + N] = (z0 - zN) + acc * 2.0;
    }
  }
  for (int idx = tid; idx < nl * N; idx += nth) {
    int l = idx >> lN, j = idx & (N - 1);
    double2 a = io.load(l, j), b = io.load(l, N - j);
    if (!forward) { a = a * cheb_bwd_pre(j, n); b = b * cheb_bwd_pre(N - j, n); }
    double s2 = -2.0 * tw[j].y;  // 2 sin(pi j / N)
    wa[l * wld + j] = fnms(a + b, a - b, s2);
  }
  __syncthreads();
  double2* r = fft_pow2(wa, wb, N, lN, nl, wld, tw, 2 * N, false, tid, nth);
  // even outputs
  const FastDiv dh(half + 1);
  for (int idx = tid; idx < nl * (half + 1); idx += nth) {
    int l = dh(idx), k = idx - l * (half + 1);
    double2 v = (r[l * wld + (k & (N - 1))] + r[l * wld + ((N - k) & (N - 1))]) * 0.5;
    if (forward) v = v * cheb_fwd_post(2 * k, n, cx.inv_nm1);
    io.store(l, 2 * k, v);
  }
  // odd outputs: prefix sum, one warp per lane
  const int K = half - 1;
  const int per = (K + 31) >> 5;
  for (int l = warp; l < nl; l += nwarp) {
    const double2* rl = r + l * wld;
    int k0 = 1 + lane_id * per;
    double2 loc = c2(0.0, 0.0);
    for (int t = 0; t < per; t++) {
      int k = k0 + t;
      if (k <= K) {
        double2 d = rl[k] - rl[N - k];
        loc = loc + c2(-0.5 * d.y, 0.5 * d.x);
      }
    }
    // exclusive warp scan of the chunk sums
    double2 inc = loc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      double ux = __shfl_up_sync(0xffffffffu, inc.x, o);
      double uy = __shfl_up_sync(0xffffffffu, inc.y, o);
      if (lane_id >= o) { inc.x += ux; inc.y += uy; }
    }
    double2 run = wa[l * wld + N] + (inc - loc);  // C_1 + sum of the previous chunks
    if (lane_id == 0) {
      double2 c1 = wa[l * wld + N];
      io.store(l, 1, forward ? c1 * cheb_fwd_post(1, n, cx.inv_nm1) : c1);
    }
    for (int t = 0; t < per; t++) {
      int k = k0 + t;
      if (k <= K) {
        double2 d = rl[k] - rl[N - k];
        run = run + c2(-0.5 * d.y, 0.5 * d.x);
        io.store(l, 2 * k + 1, forward ? run * cheb_fwd_post(2 * k + 1, n, cx.inv_nm1) : run);
      }
    }
  }
  __syncthreads();
}

// Dense variant (any n): out[k] = sum_j M[k][j] in[j]
template <class T>
static __device__ void dct1_dense(const ChebXformDev& cx, bool forward, const T* in, int in_ld, T* out, int out_ld, int nl,
                           int tid, int nth) {
  int n = cx.n;
  const double* __restrict__ M = forward ? cx.fwd : cx.bwd;
  for (int idx = tid; idx < nl * n; idx += nth) {
    int l = idx / n, k = idx - l * n;
    const T* a = in + l * in_ld;
    const double* row = M + (size_t)k * n;
    T acc = zero_v<T>();
    for (int j = 0; j < n; j++) acc = fmas(acc, a[j], __ldg(row + j));
    out[l * out_ld + k] = acc;
  }
  __syncthreads();
}

// ------------------------------------------------------------------ Fourier (x)
// length-M complex FFT of the Fourier descriptor (radix-4/2 or mixed radix)
__device__ __forceinline__ double2* fourier_fft(const FourierXformDev& fx, double2* wa, double2* wb, int nl, int wld,
                                                bool inv, int tid, int nth) {
  if (fx.log2M >= 0) return fft_pow2(wa, wb, fx.M, fx.log2M, nl, wld, fx.tw, fx.n, inv, tid, nth);
  return fft_mixed<double2>(wa, wb, fx.M, fx.rad, fx.nrad, nl, wld, fx.tw, fx.n, inv, tid, nth);
}
// lane and element of a flat index over nl lanes of M
__device__ __forceinline__ void fourier_split(const FourierXformDev& fx, int idx, int& l, int& k) {
  if (fx.log2M >= 0) {
    l = idx >> fx.log2M;
    k = idx & (fx.M - 1);
  } else {
    l = idx / fx.M;
    k = idx - l * fx.M;
  }
}

// Odd n: c2r and r2c through a full-length complex FFT (M = n).
static __device__ void c2r_odd(const FourierXformDev& fx, const double2* in, int in_ld, int in_stride, double* out,
                               int out_ld, int nl, double2* wa, double2* wb, int wld, int tid, int nth) {
  const int n = fx.n, h = n / 2;
  for (int idx = tid; idx < nl * n; idx += nth) {
    int l, k;
    fourier_split(fx, idx, l, k);
    const double2* X = in + l * in_ld;
    double2 v = k <= h ? X[k * in_stride] : conj2(X[(n - k) * in_stride]);
    if (k == 0) v.y = 0.0;
    wa[l * wld + k] = v;
  }
  __syncthreads();
  double2* r = fourier_fft(fx, wa, wb, nl, wld, true, tid, nth);
  const double s = 1.0 / (double)n;
  for (int idx = tid; idx < nl * n; idx += nth) {
    int l, k;
    fourier_split(fx, idx, l, k);
    out[l * out_ld + k] = r[l * wld + k].x * s;
  }
  __syncthreads();
}
static __device__ void r2c_odd(const FourierXformDev& fx, const double* in, int in_ld, double2* out, int out_ld,
                               int out_stride, int keep, int nl, double2* wa, double2* wb, int wld, int tid, int nth) {
  const int n = fx.n;
  for (int idx = tid; idx < nl * n; idx += nth) {
    int l, k;
    fourier_split(fx, idx, l, k);
    wa[l * wld + k] = c2(in[l * in_ld + k], 0.0);
  }
  __syncthreads();
  double2* r = fourier_fft(fx, wa, wb, nl, wld, false, tid, nth);
  for (int idx = tid; idx < nl * keep; idx += nth) {
    const int l = idx / keep, k = idx - l * keep;
    out[l * out_ld + k * out_stride] = r[l * wld + k];
  }
  __syncthreads();
}

// c2r: in = n/2+1 complex per lane (DC imag and Nyquist imag ignored), out = n reals.
// Lane l reads in[l*in_ld + k*in_stride].
static __device__ void c2r(const FourierXformDev& fx, const double2* in, int in_ld, int in_stride, double* out, int out_ld,
                    int nl, double2* wa, double2* wb, int wld, int tid, int nth) {
  if (fx.n & 1) {
    c2r_odd(fx, in, in_ld, in_stride, out, out_ld, nl, wa, wb, wld, tid, nth);
    return;
  }
  int M = fx.M;
  for (int idx = tid; idx < nl * M; idx += nth) {
    int l, k;
    fourier_split(fx, idx, l, k);
    const double2* X = in + l * in_ld;
    double2 xk = X[k * in_stride];
    double2 xm = X[(M - k) * in_stride];
    if (k == 0) { xk.y = 0.0; xm.y = 0.0; }
    double2 xc = conj2(xm);
    double2 d = xk - xc;
    double2 t = cmulc(d, fx.tw[k]);  // e^{+2 pi i k / n} (xk - xc)
    wa[l * wld + k] = c2(xk.x + xc.x - t.y, xk.y + xc.y + t.x);
  }
  __syncthreads();
  double2* r = fourier_fft(fx, wa, wb, nl, wld, true, tid, nth);
  double s = 1.0 / (double)fx.n;
  for (int idx = tid; idx < nl * M; idx += nth) {
    int l, k;
    fourier_split(fx, idx, l, k);
    double2 v = r[l * wld + k];
    out[l * out_ld + 2 * k] = v.x * s;
    out[l * out_ld + 2 * k + 1] = v.y * s;
  }
  __syncthreads();
}

// r2c: in = n reals per lane, out = first `keep` (<= n/2+1) complex values;
// lane l writes out[l*out_ld + k*out_stride].
static __device__ void r2c(const FourierXformDev& fx, const double* in, int in_ld, double2* out, int out_ld, int out_stride,
                    int keep, int nl, double2* wa, double2* wb, int wld, int tid, int nth) {
  if (fx.n & 1) {
    r2c_odd(fx, in, in_ld, out, out_ld, out_stride, keep, nl, wa, wb, wld, tid, nth);
    return;
  }
  int M = fx.M;
  for (int idx = tid; idx < nl * M; idx += nth) {
    int l, k;
    fourier_split(fx, idx, l, k);
    wa[l * wld + k] = c2(in[l * in_ld + 2 * k], in[l * in_ld + 2 * k + 1]);
  }
  __syncthreads();
  double2* r = fourier_fft(fx, wa, wb, nl, wld, false, tid, nth);
  for (int idx = tid; idx < nl * keep; idx += nth) {
    int l = idx / keep, k = idx - l * keep;
    double2 zk = r[l * wld + (k == M ? 0 : k)];
    double2 zc = conj2(r[l * wld + (k == 0 ? 0 : M - k)]);
    double2 e = (zk + zc) * 0.5;
    double2 dd = zk - zc;
    double2 o = c2(dd.y * 0.5, -dd.x * 0.5);  // (zk - zc) / (2i)
    out[l * out_ld + k * out_stride] = e + cmul(o, fx.tw[k]);
  }
  __syncthreads();
}

}  // namespace dev
}  // namespace rbc

namespace rbc {
namespace dev {
// DCT-I of complex / real lanes through the half-length FFT (n = 2^p + 1).
// `in` and `out` may alias.  wa, wb: work lanes of length >= n with stride wld.
static __device__ void dct1_fft_c(const ChebXformDev& cx, bool forward, const double2* in, int in_ld, double2* out,
                                  int out_ld, int nl, double2* wa, double2* wb, int wld, int tid, int nth) {
  // the outputs are written after every input has been read (C_1 and Z use a barrier)
  DctLanesC io{in, in_ld, out, out_ld};
  dct1_half(cx, forward, io, nl, wa, wb, wld, tid, nth);
}
static __device__ void dct1_fft_r(const ChebXformDev& cx, bool forward, const double* in, int in_ld, double* out,
                                  int out_ld, int nl, double2* wa, double2* wb, int wld, int tid, int nth) {
  DctLanesR io{in, in_ld, out, out_ld, nl};
  dct1_half(cx, forward, io, (nl + 1) >> 1, wa, wb, wld, tid, nth);
}
}  // namespace dev
}  // namespace rbc
