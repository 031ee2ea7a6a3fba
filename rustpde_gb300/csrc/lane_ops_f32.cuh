// lane_ops_f32.cuh -- FP32 lane operations of the mixed-precision form: the
// Fourier transforms and products of the convection term, which the reference
// computes in FP64 (funspace/src/fourier/r2c.rs:160-226, conv_term.rs:22-42)
// and the mixed form evaluates in FP32.  Same algorithms as the FP64 lane
// operations (Stockham FFTs, r2c/c2r through half-length complex FFTs for even
// n), on float2 data with an FP32 twiddle table.
#pragma once
#include <cuda_runtime.h>

#include "lane_ops.cuh"

namespace rbc {
namespace dev {

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 operator+(float2 a, float2 b) { return f2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 operator-(float2 a, float2 b) { return f2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 operator*(float2 a, float s) { return f2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 fcmul(float2 a, float2 w) { return f2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x); }
__device__ __forceinline__ float2 fcmulc(float2 a, float2 w) { return f2(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y); }
__device__ __forceinline__ float2 fconj(float2 a) { return f2(a.x, -a.y); }

// Stockham FFT of nl lanes of length L = 2^log2L (lane stride ld); tw[t] =
// exp(-2 pi i t / twL).  Returns the buffer holding the result.
__device__ __forceinline__ float2* fft_pow2_f(float2* a, float2* b, int L, int log2L, int nl, int ld,
                                              const float2* __restrict__ tw, int twL, bool inv, int tid, int nth) {
  int Ns = 1;
  if (log2L & 1) {
    const int half = L >> 1;
    for (int idx = tid; idx < nl * half; idx += nth) {
      const int l = idx >> (log2L - 1), j = idx & (half - 1);
      const float2 v0 = a[l * ld + j], v1 = a[l * ld + j + half];
      b[l * ld + 2 * j] = v0 + v1;
      b[l * ld + 2 * j + 1] = v0 - v1;
    }
    __syncthreads();
    float2* t = a; a = b; b = t;
    Ns = 2;
  }
  const int quarter = L >> 2, lq = log2L - 2;
  while (Ns < L) {
    const int tstep = twL / (Ns * 4);
    for (int idx = tid; idx < nl * quarter; idx += nth) {
      const int l = idx >> lq, j = idx & (quarter - 1);
      const float2* src = a + l * ld;
      float2 v0 = src[j], v1 = src[j + quarter], v2 = src[j + 2 * quarter], v3 = src[j + 3 * quarter];
      const int jm = j & (Ns - 1);
      if (jm) {
        const int e = jm * tstep;
        const float2 w1 = tw[e], w2 = tw[2 * e], w3 = tw[3 * e];
        if (inv) { v1 = fcmulc(v1, w1); v2 = fcmulc(v2, w2); v3 = fcmulc(v3, w3); }
        else { v1 = fcmul(v1, w1); v2 = fcmul(v2, w2); v3 = fcmul(v3, w3); }
      }
      const float2 s0 = v0 + v2, d0 = v0 - v2, s1 = v1 + v3, d1 = v1 - v3;
      const float2 r = inv ? f2(-d1.y, d1.x) : f2(d1.y, -d1.x);
      float2* dst = b + l * ld + (j - jm) * 4 + jm;
      dst[0] = s0 + s1;
      dst[Ns] = d0 + r;
      dst[2 * Ns] = s0 - s1;
      dst[3 * Ns] = d0 - r;
    }
    __syncthreads();
    float2* t = a; a = b; b = t;
    Ns <<= 2;
  }
  return a;
}

__device__ __forceinline__ float2* fourier_fft_f(const FourierXformDev& fx, float2* wa, float2* wb, int nl, int wld,
                                                 bool inv, int tid, int nth) {
  if (fx.log2M >= 0) return fft_pow2_f(wa, wb, fx.M, fx.log2M, nl, wld, fx.twf, fx.n, inv, tid, nth);
  return fft_mixed<float2>(wa, wb, fx.M, fx.rad, fx.nrad, nl, wld, fx.twf, fx.n, inv, tid, nth);
}

// c2r: lanes of n/2+1 complex values (imaginary parts of DC and Nyquist
// ignored) -> n reals, scaled by 1/n.  Lane l reads in[l*in_ld + k*in_stride].
__device__ __forceinline__ void c2r_f(const FourierXformDev& fx, const float2* in, int in_ld, int in_stride, float* out,
                                      int out_ld, int nl, float2* wa, float2* wb, int wld, int tid, int nth) {
  const int M = fx.M;
  const float s = 1.0f / (float)fx.n;
  if (fx.n & 1) {  // full-length complex FFT
    const int n = fx.n, h = n / 2;
    for (int idx = tid; idx < nl * n; idx += nth) {
      int l, k;
      fourier_split(fx, idx, l, k);
      const float2* X = in + l * in_ld;
      float2 v = k <= h ? X[k * in_stride] : fconj(X[(n - k) * in_stride]);
      if (k == 0) v.y = 0.f;
      wa[l * wld + k] = v;
    }
    __syncthreads();
    float2* r = fourier_fft_f(fx, wa, wb, nl, wld, true, tid, nth);
    for (int idx = tid; idx < nl * n; idx += nth) {
      int l, k;
      fourier_split(fx, idx, l, k);
      out[l * out_ld + k] = r[l * wld + k].x * s;
    }
    __syncthreads();
    return;
  }
  for (int idx = tid; idx < nl * M; idx += nth) {
    int l, k;
    fourier_split(fx, idx, l, k);
    const float2* X = in + l * in_ld;
    float2 xk = X[k * in_stride];
    float2 xm = X[(M - k) * in_stride];
    if (k == 0) { xk.y = 0.f; xm.y = 0.f; }
    const float2 xc = fconj(xm);
    const float2 t = fcmulc(xk - xc, fx.twf[k]);
    wa[l * wld + k] = f2(xk.x + xc.x - t.y, xk.y + xc.y + t.x);
  }
  __syncthreads();
  float2* r = fourier_fft_f(fx, wa, wb, nl, wld, true, tid, nth);
  for (int idx = tid; idx < nl * M; idx += nth) {
    int l, k;
    fourier_split(fx, idx, l, k);
    const float2 v = r[l * wld + k];
    out[l * out_ld + 2 * k] = v.x * s;
    out[l * out_ld + 2 * k + 1] = v.y * s;
  }
  __syncthreads();
}

// r2c: lanes of n reals -> first `keep` (<= n/2+1) complex values; lane l
// writes out[l*out_ld + k*out_stride].
__device__ __forceinline__ void r2c_f(const FourierXformDev& fx, const float* in, int in_ld, float2* out, int out_ld,
                                      int out_stride, int keep, int nl, float2* wa, float2* wb, int wld, int tid,
                                      int nth) {
  const int M = fx.M;
  if (fx.n & 1) {
    const int n = fx.n;
    for (int idx = tid; idx < nl * n; idx += nth) {
      int l, k;
      fourier_split(fx, idx, l, k);
      wa[l * wld + k] = f2(in[l * in_ld + k], 0.f);
    }
    __syncthreads();
    float2* r = fourier_fft_f(fx, wa, wb, nl, wld, false, tid, nth);
    for (int idx = tid; idx < nl * keep; idx += nth) {
      const int l = idx / keep, k = idx - l * keep;
      out[l * out_ld + k * out_stride] = r[l * wld + k];
    }
    __syncthreads();
    return;
  }
  for (int idx = tid; idx < nl * M; idx += nth) {
    int l, k;
    fourier_split(fx, idx, l, k);
    wa[l * wld + k] = f2(in[l * in_ld + 2 * k], in[l * in_ld + 2 * k + 1]);
  }
  __syncthreads();
  float2* r = fourier_fft_f(fx, wa, wb, nl, wld, false, tid, nth);
  for (int idx = tid; idx < nl * keep; idx += nth) {
    const int l = idx / keep, k = idx - l * keep;
    const float2 zk = r[l * wld + (k == M ? 0 : k)];
    const float2 zc = fconj(r[l * wld + (k == 0 ? 0 : M - k)]);
    const float2 e = (zk + zc) * 0.5f;
    const float2 dd = zk - zc;
    const float2 o = f2(dd.y * 0.5f, -dd.x * 0.5f);
    out[l * out_ld + k * out_stride] = e + fcmul(o, fx.twf[k]);
  }
  __syncthreads();
}

}  // namespace dev
}  // namespace rbc
