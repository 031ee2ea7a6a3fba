// chain_scan.cuh -- warp-parallel linear recurrences along lane chains.
//
// The banded operators of the spectral step (Chebyshev derivative suffix sums,
// the stride-2 tridiagonal of from_ortho, the forward elimination and back
// substitution of the swept banded solve) are linear recurrences along each
// parity chain of a lane.  On this GPU an FP64 warp instruction occupies the
// FP64 pipe for the whole warp however few threads are active, so a chain run
// by one thread wastes 31/32 of the pipe.  Here each chain is run by a group
// of T threads as a scan of affine maps:
//   first order   x_t = a_t x_{t-1} + b_t
//   second order  (x_t, x_{t-1}) = [[a_t, c_t], [1, 0]] (x_{t-1}, x_{t-2}) + (b_t, 0)
// phase 1 composes each thread's block of E = ceil(len / T) maps, phase 2 scans
// the T block maps with shuffles, phase 3 replays the block from the exclusive
// prefix.  Coefficients are real; values are double or double2.  Warps with
// no chain left skip the rounds (the CTA-wide calls often have 2 chains).
#pragma once
#include <cuda_runtime.h>

namespace rbc {
namespace dev {

__device__ __forceinline__ double shfl_up_v(double v, int o, int w) { return __shfl_up_sync(0xffffffffu, v, o, w); }
__device__ __forceinline__ double2 shfl_up_v(double2 v, int o, int w) {
  return make_double2(__shfl_up_sync(0xffffffffu, v.x, o, w), __shfl_up_sync(0xffffffffu, v.y, o, w));
}
__device__ __forceinline__ double axpy_v(double a, double x, double b) { return fma(a, x, b); }
__device__ __forceinline__ double2 axpy_v(double a, double2 x, double2 b) {
  return make_double2(fma(a, x.x, b.x), fma(a, x.y, b.y));
}
template <class V> __device__ __forceinline__ V zero_val();
template <> __device__ __forceinline__ double zero_val<double>() { return 0.0; }
template <> __device__ __forceinline__ double2 zero_val<double2>() { return make_double2(0.0, 0.0); }

// First-order chains.  coef(c, t, a, b) gives the map of element t of chain c
// (t = 0 must give a = 0), store(c, t, x) receives x_t.  All threads of the
// CTA call this (uniformly); it contains no barrier.
template <int T, class V, class LenF, class CoefF, class StoreF>
__device__ __forceinline__ void chains1(int nch, LenF len_of, CoefF coef, StoreF store, int tid, int nth) {
  static_assert(T <= 32 && (32 % T) == 0, "a group lies within one warp");
  const int g = tid / T, gl = tid % T, ng = nth / T;
  for (int base = 0; base < nch; base += ng) {
    // a warp whose groups all lie past the last chain has no work here or in
    // later rounds (its shuffles involve only itself)
    if (base + (tid & ~31) / T >= nch) break;
    const int c = base + g;
    const bool on = c < nch;
    const int len = on ? len_of(c) : 0;
    const int E = (len + T - 1) / T;
    const int t0 = gl * E, t1 = min(t0 + E, len);
    double A = 1.0;
    V B = zero_val<V>();
    for (int t = t0; t < t1; t++) {
      double a;
      V b;
      coef(c, t, a, b);
      B = axpy_v(a, B, b);
      A = a * A;
    }
#pragma unroll
    for (int o = 1; o < T; o <<= 1) {
      double Ap = shfl_up_v(A, o, T);
      V Bp = shfl_up_v(B, o, T);
      if (gl >= o) {
        B = axpy_v(A, Bp, B);
        A = A * Ap;
      }
    }
    V x = shfl_up_v(B, 1, T);  // value before this thread's block (map 0 has a = 0)
    if (gl == 0) x = zero_val<V>();
    for (int t = t0; t < t1; t++) {
      double a;
      V b;
      coef(c, t, a, b);
      x = axpy_v(a, x, b);
      store(c, t, x);
    }
  }
}

// Second-order chains: x_t = a_t x_{t-1} + c_t x_{t-2} + b_t.  coef(c, t, a, cc, b).
template <int T, class V, class LenF, class CoefF, class StoreF>
__device__ __forceinline__ void chains2(int nch, LenF len_of, CoefF coef, StoreF store, int tid, int nth) {
  static_assert(T <= 32 && (32 % T) == 0, "a group lies within one warp");
  const int g = tid / T, gl = tid % T, ng = nth / T;
  for (int base = 0; base < nch; base += ng) {
    if (base + (tid & ~31) / T >= nch) break;  // as in chains1
    const int c = base + g;
    const bool on = c < nch;
    const int len = on ? len_of(c) : 0;
    const int E = (len + T - 1) / T;
    const int t0 = gl * E, t1 = min(t0 + E, len);
    // block map: (x, x') -> (m00 x + m01 x' + B0, m10 x + m11 x' + B1)
    double m00 = 1.0, m01 = 0.0, m10 = 0.0, m11 = 1.0;
    V B0 = zero_val<V>(), B1 = zero_val<V>();
    for (int t = t0; t < t1; t++) {
      double a, cc;
      V b;
      coef(c, t, a, cc, b);
      // new = [[a, cc], [1, 0]] * old + (b, 0)
      double n00 = fma(a, m00, cc * m10), n01 = fma(a, m01, cc * m11);
      V nb0 = axpy_v(a, B0, axpy_v(cc, B1, b));
      m10 = m00; m11 = m01; B1 = B0;
      m00 = n00; m01 = n01; B0 = nb0;
    }
#pragma unroll
    for (int o = 1; o < T; o <<= 1) {
      double p00 = shfl_up_v(m00, o, T), p01 = shfl_up_v(m01, o, T);
      double p10 = shfl_up_v(m10, o, T), p11 = shfl_up_v(m11, o, T);
      V q0 = shfl_up_v(B0, o, T), q1 = shfl_up_v(B1, o, T);
      if (gl >= o) {
        // self o prev: M = M_self M_prev, B = M_self B_prev + B_self
        double n00 = fma(m00, p00, m01 * p10), n01 = fma(m00, p01, m01 * p11);
        double n10 = fma(m10, p00, m11 * p10), n11 = fma(m10, p01, m11 * p11);
        V nb0 = axpy_v(m00, q0, axpy_v(m01, q1, B0));
        V nb1 = axpy_v(m10, q0, axpy_v(m11, q1, B1));
        m00 = n00; m01 = n01; m10 = n10; m11 = n11; B0 = nb0; B1 = nb1;
      }
    }
    // state before the block: (x_{t0-1}, x_{t0-2}) = inclusive result of the previous thread
    V x1 = shfl_up_v(B0, 1, T), x2 = shfl_up_v(B1, 1, T);
    if (gl == 0) { x1 = zero_val<V>(); x2 = zero_val<V>(); }
    for (int t = t0; t < t1; t++) {
      double a, cc;
      V b;
      coef(c, t, a, cc, b);
      V x = axpy_v(a, x1, axpy_v(cc, x2, b));
      store(c, t, x);
      x2 = x1;
      x1 = x;
    }
  }
}

}  // namespace dev
}  // namespace rbc
