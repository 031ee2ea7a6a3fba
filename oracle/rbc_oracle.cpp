// rbc_oracle.cpp -- CPU FP64 restatement of rustpde's pseudo-spectral
// Rayleigh-Benard time step (TEST INFRASTRUCTURE ONLY).
//
// This file is the parity oracle and the timed CPU baseline.  It is never
// linked into, called by, or shipped with the GPU library: only tests/,
// __graft_entry__.smoke() and bench.py's CPU legs load it.
//
// It restates, operation by operation and in the reference's operation order,
// the following reference files (paths relative to the rustpde repository):
//   funspace/src/chebyshev/ortho.rs        Chebyshev nodes/transforms/derivative/pinv
//   funspace/src/chebyshev/composite.rs    composite bases (to/from_ortho, fwd/bwd, diff)
//   funspace/src/chebyshev/composite_stencil.rs + linalg.rs   stencils, stride-2 TDMA
//   funspace/src/chebyshev/dmsuite.rs      spectral second-derivative matrix
//   funspace/src/fourier/r2c.rs, c2c.rs    FourierR2c transforms, derivative, nodes
//   funspace/src/space2.rs                 axis order of the 2-D space operations
//   src/field.rs, src/field/average.rs     Field2, grid deltas, averages, solver ingredients
//   src/solver/{fdma,matvec,fdma_tensor,hholtz,hholtz_adi,poisson}.rs
//   src/navier/navier.rs, conv_term.rs, functions.rs   Navier2D setup/update/diagnostics
//
// Third-party arithmetic that the reference takes from crates (rustdct DCT-I,
// realfft r2c/c2r, ndarray-linalg eig/inv) is restated from the published
// definitions: DCT-I = REDFT00 (unnormalised), r2c unnormalised forward,
// c2r with 1/n and the imaginary parts of the DC and Nyquist bins ignored.
// The dense eigen-decomposition used by FdmaTensor (utils.rs:66-98) is NOT
// done here: the Python side of the oracle supplies it from numpy.linalg.eig
// (LAPACK geev, the same routine ndarray-linalg calls), see or_*_tensor_* below.
//
// Build: -O3 -ffp-contract=off (the reference does not contract a*b+c into FMA).
#include <atomic>
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

using cplx = std::complex<double>;
static const double PI = 3.14159265358979323846264338327950288;

// ---------------------------------------------------------------------------
// Scalar helpers mirroring num_complex / f64 arithmetic used by the reference.
// ---------------------------------------------------------------------------
inline double rmul(double a, double b) { return a * b; }
inline cplx rmul(cplx a, double b) { return cplx(a.real() * b, a.imag() * b); }
inline double rdiv(double a, double b) { return a / b; }
inline cplx rdiv(cplx a, double b) { return cplx(a.real() / b, a.imag() / b); }
// num_complex Complex / Complex with a purely real divisor (s, 0):
// re = (a*s + b*0)/(s*s), im = (b*s - a*0)/(s*s)   (space2.rs gradient scaling)
inline double div_scale(double a, double s) { return a / s; }
inline cplx div_scale(cplx a, double s) {
  double ns = s * s;
  double re = a.real() * s + a.imag() * 0.0;
  double im = a.imag() * s - a.real() * 0.0;
  return cplx(re / ns, im / ns);
}
inline cplx cmul(cplx a, cplx b) {  // num_complex multiplication
  return cplx(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
}
template <class T> inline T zero() { return T(0); }

// ---------------------------------------------------------------------------
// 2-D row-major array
// ---------------------------------------------------------------------------
template <class T> struct Arr2 {
  int n0 = 0, n1 = 0;
  std::vector<T> v;
  Arr2() = default;
  Arr2(int a, int b) : n0(a), n1(b), v((size_t)a * b, T(0)) {}
  T& operator()(int i, int j) { return v[(size_t)i * n1 + j]; }
  const T& operator()(int i, int j) const { return v[(size_t)i * n1 + j]; }
  size_t size() const { return v.size(); }
  T* data() { return v.data(); }
  const T* data() const { return v.data(); }
};
using Mat = Arr2<double>;

static Mat matmul(const Mat& a, const Mat& b) {
  if (a.n1 != b.n0) throw std::runtime_error("matmul shape");
  Mat c(a.n0, b.n1);
  for (int i = 0; i < a.n0; i++)
    for (int k = 0; k < a.n1; k++) {
      double aik = a(i, k);
      if (aik == 0.0) continue;
      for (int j = 0; j < b.n1; j++) c(i, j) += aik * b(k, j);
    }
  return c;
}

// ---------------------------------------------------------------------------
// Complex FFT of any length: self-sorting (Stockham) mixed-radix stages of
// radix 4, 2, 3 and any other prime up to 64, and Bluestein's chirp-z
// algorithm through a power-of-two FFT when the length has a prime factor
// above 64 (rustfft, behind the reference's DCT-I and r2c, is O(n log n) for
// every length too: its Rader and Bluestein algorithms).
//
// A stage of radix p on sub-length L with stride s (L = n, s = 1 first): for
// j < L/p and t < s, the p inputs x[t + s (j + r L/p)], r < p, go through a
// p-point DFT; output u is multiplied by exp(-2 pi i j u / L) and written to
// y[t + s (p j + u)].  That splits a length-L DFT into p DFTs of length L/p
// (X[u + p k] = DFT_{L/p}(y^u)[k]); the next stage takes L/p and stride s p,
// and after the last one the outputs are in natural order.
// ---------------------------------------------------------------------------
struct FFT {
  int n = 0;
  struct Stage {
    int p = 0, L = 0;
    std::vector<cplx> tw;     // tw[j (p - 1) + u - 1] = exp(-2 pi i j u / L), j < L/p, 0 < u < p
    std::vector<cplx> roots;  // exp(-2 pi i k / p), k < p (radices other than 2, 3, 4)
  };
  std::vector<Stage> stages;
  // Bluestein: chirp[k] = exp(-pi i k^2 / n), and the length-m FFT (m a power
  // of two >= 2n - 1) of the conjugate chirp wrapped around
  bool blue = false;
  int m = 0;
  std::vector<cplx> chirp, bfft;
  std::unique_ptr<FFT> sub;

  static cplx expi(long e, long d) {  // exp(-2 pi i e / d), the angle reduced exactly
    e %= d;
    if (e < 0) e += d;
    const double ang = 2.0 * PI * (double)e / (double)d;
    return cplx(std::cos(ang), -std::sin(ang));
  }

  explicit FFT(int n_) : n(n_) {
    std::vector<int> fac;
    int r = n;
    while (r % 4 == 0) { fac.push_back(4); r /= 4; }
    if (r % 2 == 0) { fac.push_back(2); r /= 2; }
    for (int p = 3; p * p <= r; p += 2)
      while (r % p == 0) { fac.push_back(p); r /= p; }
    if (r > 1) fac.push_back(r);
    int maxp = 1;
    for (int p : fac) maxp = std::max(maxp, p);
    if (maxp > 64) {
      blue = true;
      m = 1;
      while (m < 2 * n - 1) m *= 2;
      sub.reset(new FFT(m));
      chirp.resize(n);
      for (int k = 0; k < n; k++) chirp[k] = expi((long)k * k, 2L * n);  // exp(-pi i k^2 / n)
      std::vector<cplx> b(m, cplx(0.0, 0.0));
      b[0] = std::conj(chirp[0]);
      for (int k = 1; k < n; k++) b[k] = b[m - k] = std::conj(chirp[k]);
      bfft.resize(m);
      sub->exec(b.data(), bfft.data(), false);
      return;
    }
    int L = n;
    for (int p : fac) {
      Stage st;
      st.p = p;
      st.L = L;
      const int q = L / p;
      st.tw.resize((size_t)q * (p - 1));
      for (int j = 0; j < q; j++)
        for (int u = 1; u < p; u++) st.tw[(size_t)j * (p - 1) + u - 1] = expi((long)j * u, L);
      if (p != 2 && p != 3 && p != 4) {
        st.roots.resize(p);
        for (int k = 0; k < p; k++) st.roots[k] = expi(k, p);
      }
      stages.push_back(std::move(st));
      L = q;
    }
  }

  static inline cplx mul(cplx a, cplx b) {
    return cplx(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
  }

  // one stage: x (sub-length L, stride s) -> y
  static void stage(const Stage& st, int s, const cplx* x, cplx* y) {
    const int p = st.p, q = st.L / p;
    const cplx* tw = st.tw.data();
    if (p == 2) {
      for (int j = 0; j < q; j++) {
        const cplx w = tw[j];
        for (int t = 0; t < s; t++) {
          const cplx a0 = x[t + (size_t)s * j], a1 = x[t + (size_t)s * (j + q)];
          y[t + (size_t)s * (2 * j)] = a0 + a1;
          y[t + (size_t)s * (2 * j + 1)] = mul(a0 - a1, w);
        }
      }
    } else if (p == 4) {
      for (int j = 0; j < q; j++) {
        const cplx w1 = tw[3 * j], w2 = tw[3 * j + 1], w3 = tw[3 * j + 2];
        for (int t = 0; t < s; t++) {
          const cplx a0 = x[t + (size_t)s * j], a1 = x[t + (size_t)s * (j + q)];
          const cplx a2 = x[t + (size_t)s * (j + 2 * q)], a3 = x[t + (size_t)s * (j + 3 * q)];
          const cplx t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, t3 = a1 - a3;
          const cplx mit3(t3.imag(), -t3.real());  // -i t3
          cplx* o = y + t + (size_t)s * (4 * j);
          o[0] = t0 + t2;
          o[s] = mul(t1 + mit3, w1);
          o[2 * (size_t)s] = mul(t0 - t2, w2);
          o[3 * (size_t)s] = mul(t1 - mit3, w3);
        }
      }
    } else if (p == 3) {
      const double h = 0.86602540378443864676372317075293618;  // sin(2 pi / 3)
      for (int j = 0; j < q; j++) {
        const cplx w1 = tw[2 * j], w2 = tw[2 * j + 1];
        for (int t = 0; t < s; t++) {
          const cplx a0 = x[t + (size_t)s * j], a1 = x[t + (size_t)s * (j + q)];
          const cplx a2 = x[t + (size_t)s * (j + 2 * q)];
          const cplx sm = a1 + a2, df = a1 - a2;
          const cplx mid = a0 - 0.5 * sm;
          const cplx rot(h * df.imag(), -h * df.real());  // -i sin(2 pi / 3) (a1 - a2)
          cplx* o = y + t + (size_t)s * (3 * j);
          o[0] = a0 + sm;
          o[s] = mul(mid + rot, w1);
          o[2 * (size_t)s] = mul(mid - rot, w2);
        }
      }
    } else {
      // odd prime p: inputs r and p - r pair up, sum s_r and difference d_r;
      // outputs u and p - u share c = a_0 + sum s_r cos(2 pi r u / p) and
      // v = sum d_r sin(2 pi r u / p): b_u = c - i v, b_{p-u} = c + i v
      const cplx* rt = st.roots.data();  // cos + i(-sin) of 2 pi k / p
      const int hp = (p - 1) / 2;
      thread_local std::vector<cplx> sm, df;
      sm.resize(hp + 1);
      df.resize(hp + 1);
      for (int j = 0; j < q; j++) {
        for (int t = 0; t < s; t++) {
          const cplx a0 = x[t + (size_t)s * j];
          cplx b0 = a0;
          for (int r = 1; r <= hp; r++) {
            const cplx ar = x[t + (size_t)s * (j + (size_t)r * q)], ap = x[t + (size_t)s * (j + (size_t)(p - r) * q)];
            sm[r] = ar + ap;
            df[r] = ar - ap;
            b0 += sm[r];
          }
          cplx* o = y + t + (size_t)s * ((size_t)p * j);
          o[0] = b0;
          for (int u = 1; u <= hp; u++) {
            double cr = a0.real(), ci = a0.imag(), vr = 0.0, vi = 0.0;
            int e = 0;
            for (int r = 1; r <= hp; r++) {
              e += u;
              if (e >= p) e -= p;
              const double cs = rt[e].real(), sn = -rt[e].imag();
              cr += sm[r].real() * cs;
              ci += sm[r].imag() * cs;
              vr += df[r].real() * sn;
              vi += df[r].imag() * sn;
            }
            // -i v = (vi, -vr), +i v = (-vi, vr)
            o[(size_t)s * u] = mul(cplx(cr + vi, ci - vr), tw[(size_t)j * (p - 1) + u - 1]);
            o[(size_t)s * (p - u)] = mul(cplx(cr - vi, ci + vr), tw[(size_t)j * (p - 1) + p - u - 1]);
          }
        }
      }
    }
  }

  // out = sum_j in_j exp(-+ 2 pi i jk/n); unnormalised both ways (the inverse
  // is conj(forward(conj(x)))); in and out may be the same array
  void exec(const cplx* in, cplx* out, bool inv) const {
    if (blue) {
      // X_k = chirp_k sum_j (x_j chirp_j) conj(chirp_{k-j})
      thread_local std::vector<cplx> a, A;
      a.assign(m, cplx(0.0, 0.0));
      A.resize(m);
      for (int j = 0; j < n; j++) a[j] = mul(inv ? std::conj(in[j]) : in[j], chirp[j]);
      sub->exec(a.data(), A.data(), false);
      for (int k = 0; k < m; k++) A[k] = mul(A[k], bfft[k]);
      sub->exec(A.data(), a.data(), true);
      const double s = 1.0 / (double)m;
      for (int k = 0; k < n; k++) {
        const cplx v = mul(a[k] * s, chirp[k]);
        out[k] = inv ? std::conj(v) : v;
      }
      return;
    }
    thread_local std::vector<cplx> b0, b1;
    if ((int)b0.size() < n) { b0.resize(n); b1.resize(n); }
    cplx* x = b0.data();
    cplx* y = b1.data();
    for (int j = 0; j < n; j++) x[j] = inv ? std::conj(in[j]) : in[j];
    int s = 1;
    for (const Stage& st : stages) {
      stage(st, s, x, y);
      std::swap(x, y);
      s *= st.p;
    }
    for (int k = 0; k < n; k++) out[k] = inv ? std::conj(x[k]) : x[k];
  }
};

static std::shared_ptr<FFT> get_fft(int n) {
  thread_local std::vector<std::shared_ptr<FFT>> cache;
  for (auto& f : cache)
    if (f->n == n) return f;
  cache.push_back(std::make_shared<FFT>(n));
  return cache.back();
}

// Length whose DCT-I runs as its defining sum instead of through the FFT
// (or_set_dense_dct; -1: none).  Both are exact restatements of the same
// transform; tests use the pair to measure how much a case's results move
// with the transform's rounding alone.
static std::atomic<int> g_dense_dct_n{-1};

// Even-length real transforms: the n/2-point complex FFT and the factors
// exp(-2 pi i k / n), k < n/2, of the split into even and odd samples
struct RealFFT {
  int n = 0;
  std::shared_ptr<FFT> half;
  std::vector<cplx> w;
};
static const RealFFT& get_real_fft(int n) {
  thread_local std::vector<std::unique_ptr<RealFFT>> cache;
  for (auto& r : cache)
    if (r->n == n) return *r;
  auto r = std::make_unique<RealFFT>();
  r->n = n;
  r->half = get_fft(n / 2);
  r->w.resize(n / 2);
  for (int k = 0; k < n / 2; k++) r->w[k] = FFT::expi(k, n);
  cache.push_back(std::move(r));
  return *cache.back();
}

// real -> complex, unnormalised, m = n/2+1 outputs (ndfft_r2c).  Even n: the
// n/2-point complex FFT of z_j = x_2j + i x_2j+1 gives the DFTs E and O of
// the even and odd samples, and X_k = E_k + exp(-2 pi i k/n) O_k.
static void rfft(const double* x, cplx* X, int n) {
  if (n % 2 != 0 || n < 4) {
    auto f = get_fft(n);
    thread_local std::vector<cplx> a;
    a.resize(n);
    for (int j = 0; j < n; j++) a[j] = cplx(x[j], 0.0);
    f->exec(a.data(), a.data(), false);
    for (int k = 0; k <= n / 2; k++) X[k] = a[k];
    return;
  }
  const int h = n / 2;
  const RealFFT& rf = get_real_fft(n);
  thread_local std::vector<cplx> z;
  z.resize(h);
  for (int j = 0; j < h; j++) z[j] = cplx(x[2 * j], x[2 * j + 1]);
  rf.half->exec(z.data(), z.data(), false);
  X[0] = cplx(z[0].real() + z[0].imag(), 0.0);
  X[h] = cplx(z[0].real() - z[0].imag(), 0.0);
  for (int k = 1; k < h; k++) {
    const cplx zk = z[k], zc = std::conj(z[h - k]);
    const cplx e = 0.5 * (zk + zc);
    const cplx d = 0.5 * (zk - zc);
    const cplx o(d.imag(), -d.real());  // (zk - zc) / (2 i)
    X[k] = e + FFT::mul(rf.w[k], o);
  }
}

// complex -> real with 1/n (ndifft_r2c); imaginary parts of DC (and Nyquist
// for even n) are ignored, Hermitian symmetry assumed.  Even n: one n/2-point
// inverse FFT of Z_k = (a_k + conj a_{h-k}) + i (a_k - conj a_{h-k}) exp(2 pi i k/n)
// gives x_2j + i x_2j+1 (h = n/2).
static void irfft(const cplx* X, double* x, int n) {
  const double s = 1.0 / (double)n;
  if (n % 2 != 0 || n < 4) {
    auto f = get_fft(n);
    thread_local std::vector<cplx> a;
    a.resize(n);
    const int m = n / 2 + 1;
    a[0] = cplx(X[0].real(), 0.0);
    for (int k = 1; k < m; k++) a[k] = X[k];
    if (n % 2 == 0) a[n / 2] = cplx(X[n / 2].real(), 0.0);
    for (int k = 1; k < m; k++)
      if (n - k != k) a[n - k] = std::conj(X[k]);
    f->exec(a.data(), a.data(), true);
    for (int j = 0; j < n; j++) x[j] = a[j].real() * s;
    return;
  }
  const int h = n / 2;
  const RealFFT& rf = get_real_fft(n);
  thread_local std::vector<cplx> z;
  z.resize(h);
  for (int k = 0; k < h; k++) {
    const cplx ak = k == 0 ? cplx(X[0].real(), 0.0) : X[k];
    const cplx ah = k == 0 ? cplx(X[h].real(), 0.0) : X[h - k];  // a_{h-k}; k = 0: the Nyquist bin
    const cplx ac = std::conj(ah);
    const cplx d = FFT::mul(ak - ac, std::conj(rf.w[k]));  // (a_k - conj a_{h-k}) exp(2 pi i k/n)
    z[k] = (ak + ac) + cplx(-d.imag(), d.real());
  }
  rf.half->exec(z.data(), z.data(), true);
  for (int j = 0; j < h; j++) {
    x[2 * j] = z[j].real() * s;
    x[2 * j + 1] = z[j].imag() * s;
  }
}

// DCT-I (REDFT00, unnormalised): X_k = x_0 + (-1)^k x_N + 2 sum_{j=1}^{N-1} x_j cos(pi j k / N),
// the real parts of the 2N-point DFT of the even extension
static void dct1(const double* x, double* X, int n) {
  int N = n - 1;
  if (N < 1) { X[0] = x[0]; return; }
  if (n == g_dense_dct_n.load(std::memory_order_relaxed)) {
    for (int k = 0; k <= N; k++) {
      double acc = 0.0;
      for (int j = 0; j <= N; j++) {
        const long r = ((long)j * k) % (2L * N);  // the angle pi j k / N reduced exactly
        acc += ((j == 0 || j == N) ? 1.0 : 2.0) * x[j] * std::cos(M_PI * (double)r / (double)N);
      }
      X[k] = acc;
    }
    return;
  }
  thread_local std::vector<double> a;
  thread_local std::vector<cplx> b;
  a.resize(2 * N);
  b.resize(N + 1);
  for (int j = 0; j <= N; j++) a[j] = x[j];
  for (int j = 1; j < N; j++) a[2 * N - j] = x[j];
  rfft(a.data(), b.data(), 2 * N);
  for (int k = 0; k <= N; k++) X[k] = b[k].real();
}

// ---------------------------------------------------------------------------
// One-dimensional bases (funspace)
// ---------------------------------------------------------------------------
enum BaseKind { CHEB = 0, CD = 1, CN = 2, CDBC = 3, CNBC = 4, FOURIER = 5 };

struct Base {
  int kind = CHEB;
  int n = 0;  // physical size
  int m = 0;  // spectral size
  std::vector<double> x;
  std::vector<double> corr_fwd, corr_bwd;  // ortho.rs:56-63
  std::vector<double> diag, low2, main_, off;  // composite_stencil.rs:117-171
  double t0[2] = {0, 0}, t1[2] = {0, 0};         // composite_stencil.rs:300-330
  std::vector<double> kk;                        // Fourier wavenumbers 0..m-1

  bool fourier() const { return kind == FOURIER; }
  bool composite() const { return kind == CD || kind == CN || kind == CDBC || kind == CNBC; }
  bool bc() const { return kind == CDBC || kind == CNBC; }

  Base() = default;
  Base(int kind_, int n_) : kind(kind_), n(n_) {
    if (kind == FOURIER) {
      m = n / 2 + 1;
      // c2c.rs:63-66: Array1::range(0, 2pi, 2pi/n)
      x.resize(n);
      double step = 2.0 * PI / (double)n;
      for (int i = 0; i < n; i++) x[i] = 0.0 + step * (double)i;
      kk.resize(m);
      for (int i = 0; i < m; i++) kk[i] = (double)i;
      return;
    }
    // ortho.rs:71-80 Gauss-Lobatto nodes
    x.resize(n);
    double mm = (double)(n - 1);
    for (int k = 0; k < n; k++) {
      double arg = PI * (mm - 2.0 * (double)k) / (2.0 * mm);
      x[k] = -std::sin(arg);
    }
    corr_fwd.resize(n);
    corr_bwd.resize(n);
    for (int i = 0; i < n; i++) {
      double c = std::pow(-1.0, (double)i);
      corr_fwd[i] = c * (1.0 / (double)(n - 1));
      corr_bwd[i] = c / 2.0;
    }
    if (kind == CHEB) { m = n; return; }
    if (kind == CD || kind == CN) {
      m = n - 2;
      diag.assign(m, 1.0);
      low2.assign(m, 0.0);
      for (int k = 0; k < m; k++) {
        if (kind == CD) low2[k] = -1.0;
        else {
          double k_ = (double)(k * k), k2 = (double)((k + 2) * (k + 2));
          low2[k] = -1.0 * k_ / k2;
        }
      }
      main_.assign(m, 0.0);
      off.assign(m - 2, 0.0);
      for (int i = 0; i < m; i++) main_[i] = diag[i] * diag[i] + low2[i] * low2[i];
      for (int i = 0; i < m - 2; i++) off[i] = diag[i + 2] * low2[i];
      return;
    }
    m = 2;  // boundary bases
    if (kind == CDBC) {
      t0[0] = 0.5; t0[1] = 0.5; t1[0] = -0.5; t1[1] = 0.5;
    } else {
      t0[0] = 0.5; t0[1] = 0.5; t1[0] = -(1.0 / 8.0); t1[1] = 1.0 / 8.0;
    }
  }
  int len_phys() const { return n; }
  int len_spec() const { return m; }
  int len_ortho() const { return fourier() ? m : n; }

  // ----- Chebyshev transforms on real lanes (ortho.rs:235-312)
  void cheb_forward(const double* in, double* out) const {
    dct1(in, out, n);
    for (int i = 0; i < n; i++) out[i] = out[i] * corr_fwd[i];
    out[0] = out[0] * 0.5;
    out[n - 1] = out[n - 1] * 0.5;
  }
  void cheb_backward(const double* in, double* out) const {
    thread_local std::vector<double> buf;
    buf.resize(n);
    for (int i = 0; i < n; i++) buf[i] = in[i] * corr_bwd[i];
    buf[0] = buf[0] * 2.0;
    buf[n - 1] = buf[n - 1] * 2.0;
    dct1(buf.data(), out, n);
  }
  // ----- stencils (composite_stencil.rs:207-229, 250-276, 339-406)
  template <class T> void to_ortho(const T* c, T* p) const {
    if (!composite()) { for (int i = 0; i < len_ortho(); i++) p[i] = c[i]; return; }
    for (int i = 0; i < n; i++) p[i] = T(0);
    if (bc()) {
      p[0] = rmul(c[0], t0[0]) + rmul(c[1], t0[1]);
      p[1] = rmul(c[0], t1[0]) + rmul(c[1], t1[1]);
      return;
    }
    p[0] = rmul(c[0], diag[0]);
    p[1] = rmul(c[1], diag[1]);
    for (int i = 2; i < n - 2; i++) p[i] = rmul(c[i], diag[i]) + rmul(c[i - 2], low2[i - 2]);
    p[n - 2] = rmul(c[n - 4], low2[n - 4]);
    p[n - 1] = rmul(c[n - 3], low2[n - 3]);
  }
  template <class T> void from_ortho(const T* p, T* c) const {
    if (!composite()) { for (int i = 0; i < len_ortho(); i++) c[i] = p[i]; return; }
    if (bc()) {
      T c0 = rmul(p[0], t0[0]) + rmul(p[1], t1[0]);
      T c1 = rmul(p[0], t0[1]) + rmul(p[1], t1[1]);
      double a = t0[0] * t0[0] + t1[0] * t1[0];
      double b = t0[0] * t0[1] + t1[0] * t1[1];
      double cc = t0[1] * t0[0] + t1[1] * t1[0];
      double d = t0[1] * t0[1] + t1[1] * t1[1];
      double det = 1.0 / (a * d - b * cc);
      c[0] = rmul(rmul(c0, d) - rmul(c1, b), det);
      c[1] = rmul(rmul(c1, a) - rmul(c0, cc), det);
      return;
    }
    for (int i = 0; i < m; i++) c[i] = rmul(p[i], diag[i]) + rmul(p[i + 2], low2[i]);
    tdma(off.data(), main_.data(), off.data(), c, m, (int)off.size());
  }
  // linalg.rs:14-57 (stride-2 tridiagonal solve, a/c at offsets -2/+2)
  template <class T>
  static void tdma(const double* a, const double* b, const double* c, T* d, int n, int clen) {
    thread_local std::vector<T> xs, gs;
    thread_local std::vector<double> ws;
    xs.assign(n, T(0)); gs.assign(n, T(0)); ws.assign(std::max(n - 2, 1), 0.0);
    T* x = xs.data(); T* g = gs.data(); double* w = ws.data();
    w[0] = c[0] / b[0];
    g[0] = rdiv(d[0], b[0]);
    if (clen > 1) w[1] = c[1] / b[1];
    g[1] = rdiv(d[1], b[1]);
    for (int i = 2; i < n - 2; i++) w[i] = c[i] / (b[i] - a[i - 2] * w[i - 2]);
    for (int i = 2; i < n; i++) g[i] = rdiv(d[i] - rmul(g[i - 2], a[i - 2]), b[i] - a[i - 2] * w[i - 2]);
    x[n - 1] = g[n - 1];
    x[n - 2] = g[n - 2];
    for (int i = n - 2; i >= 1; i--) x[i - 1] = g[i - 1] - rmul(x[i + 1], w[i - 1]);
    for (int i = 0; i < n; i++) d[i] = x[i];
  }
  // ----- derivatives (ortho.rs:107-125, r2c.rs:88-99) on ortho coefficients
  template <class T> void diff_ortho(T* d, int times) const {
    if (fourier()) {
      for (int t = 0; t < times; t++)
        for (int i = 0; i < m; i++) d[i] = cmul_ik(d[i], kk[i]);
      return;
    }
    int len = n;
    for (int t = 0; t < times; t++) {
      d[0] = d[1];
      for (int i = 1; i < len - 1; i++) d[i] = rmul(d[i + 1], 2.0 * (double)(i + 1));
      d[n - 1] = T(0);
      for (int i = n - 3; i >= 1; i--) d[i] = d[i] + d[i + 2];
      d[0] = d[0] + rdiv(d[2], 2.0);
    }
  }
  static double cmul_ik(double, double) { throw std::runtime_error("fourier derivative on real data"); }
  static cplx cmul_ik(cplx d, double k) { return cmul(d, cplx(0.0, k)); }

  // ----- spectral operator matrices (ortho.rs:147-180, dmsuite.rs:24-49, r2c.rs:372-394)
  Mat mass() const {
    if (fourier() || kind == CHEB) {
      int s = fourier() ? m : n;
      Mat e(s, s);
      for (int i = 0; i < s; i++) e(i, i) = 1.0;
      return e;
    }
    Mat s(n, m);
    if (bc()) {
      s(0, 0) = t0[0]; s(0, 1) = t0[1]; s(1, 0) = t1[0]; s(1, 1) = t1[1];
      return s;
    }
    for (int i = 0; i < m; i++) { s(i, i) = diag[i]; s(i + 2, i) = low2[i]; }
    return s;
  }
  Mat laplace() const {
    if (fourier()) {
      Mat l(m, m);
      for (int i = 0; i < m; i++) l(i, i) = -kk[i] * kk[i];
      return l;
    }
    Mat d(n, n);
    for (int p = 0; p < n; p++)
      for (int q = p + 2; q < n; q++)
        if ((p + q) % 2 == 0) d(p, q) = (double)((long)q * ((long)q * q - (long)p * p));
    for (int q = 0; q < n; q++) d(0, q) *= 0.5;
    return d;
  }
  Mat laplace_inv() const {
    if (fourier()) {
      Mat l = laplace();
      for (int i = 1; i < m; i++) l(i, i) = 1.0 / l(i, i);
      return l;
    }
    Mat p(n, n);
    p(2, 0) = 0.25;
    for (int i = 3; i < n; i++) p(i, i - 2) = 1.0 / (double)(4 * i * (i - 1));
    for (int i = 2; i < n - 2; i++) p(i, i) = -1.0 / (double)(2 * (i * i - 1));
    for (int i = 2; i < n - 4; i++) p(i, i + 2) = 1.0 / (double)(4 * i * (i + 1));
    return p;
  }
  Mat laplace_inv_eye() const {
    int s = fourier() ? m : n;
    Mat e(s - (fourier() ? 1 : 2), s);
    int off_ = fourier() ? 1 : 2;
    for (int i = 0; i < e.n0; i++) e(i, i + off_) = 1.0;
    return e;
  }
  // field.rs:194-225  ingredients_for_hholtz
  void ingredients(Mat& a, Mat& b, Mat& pre, bool& has_pre) const {
    Mat mss = mass();
    if (fourier()) { a = mss; b = laplace(); has_pre = false; return; }
    Mat lap = laplace();
    Mat peye = laplace_inv_eye();
    Mat pinv = matmul(peye, laplace_inv());
    if (kind == CHEB) {
      Mat ms(mss.n0, mss.n1 - 2);
      for (int i = 0; i < ms.n0; i++)
        for (int j = 0; j < ms.n1; j++) ms(i, j) = mss(i, j + 2);
      a = matmul(pinv, ms);
      b = matmul(peye, ms);
    } else {
      a = matmul(pinv, mss);
      b = matmul(peye, mss);
    }
    pre = pinv;
    has_pre = true;
  }
};

// ---------------------------------------------------------------------------
// Apply a lane function along an axis of a 2-D row-major array.
// ---------------------------------------------------------------------------
template <class Tin, class Tout, class F>
static void along(const Arr2<Tin>& in, Arr2<Tout>& out, int axis, F f) {
  int lanes = axis == 0 ? in.n1 : in.n0;
  int lin = axis == 0 ? in.n0 : in.n1;
  int lout = axis == 0 ? out.n0 : out.n1;
  if ((axis == 0 ? out.n1 : out.n0) != lanes) throw std::runtime_error("along: lane mismatch");
  long work = (long)lanes * (lin + lout);
#pragma omp parallel if (work > 8192)
  {
    std::vector<Tin> a(lin);
    std::vector<Tout> b(lout);
#pragma omp for schedule(static)
    for (int l = 0; l < lanes; l++) {
      if (axis == 0) for (int i = 0; i < lin; i++) a[i] = in(i, l);
      else for (int i = 0; i < lin; i++) a[i] = in(l, i);
      f(a.data(), b.data());
      if (axis == 0) for (int i = 0; i < lout; i++) out(i, l) = b[i];
      else for (int i = 0; i < lout; i++) out(l, i) = b[i];
    }
  }
}

// ---------------------------------------------------------------------------
// Space2 (space2.rs) -- T = double for R2r x R2r, cplx for R2c x R2r.
// ---------------------------------------------------------------------------
template <class T> struct Space2 {
  Base b0, b1;
  Space2() = default;
  Space2(const Base& a, const Base& b) : b0(a), b1(b) {}
  int phys0() const { return b0.n; }
  int phys1() const { return b1.n; }
  int spec0() const { return b0.m; }
  int spec1() const { return b1.m; }

  // forward: base1 along axis 1, then base0 along axis 0 (space2.rs:323-333)
  Arr2<T> forward(const Arr2<double>& v) const {
    Arr2<double> buf(v.n0, b1.m);
    const Base& B1 = b1;
    along(v, buf, 1, [&](const double* in, double* out) {
      thread_local std::vector<double> o;
      o.resize(B1.n);
      B1.cheb_forward(in, o.data());
      B1.from_ortho(o.data(), out);
    });
    return forward0(buf);
  }
  Arr2<T> forward0(const Arr2<double>& buf) const;
  // backward: base0 along axis 0, then base1 along axis 1 (space2.rs:346-356)
  Arr2<double> backward(const Arr2<T>& vhat) const {
    Arr2<double> buf = backward0(vhat);
    Arr2<double> out(buf.n0, b1.n);
    const Base& B1 = b1;
    along(buf, out, 1, [&](const double* in, double* o) {
      thread_local std::vector<double> p;
      p.resize(B1.n);
      B1.to_ortho(in, p.data());
      B1.cheb_backward(p.data(), o);
    });
    return out;
  }
  Arr2<double> backward0(const Arr2<T>& vhat) const;
  Arr2<T> to_ortho(const Arr2<T>& in) const {
    Arr2<T> buf(b0.len_ortho(), in.n1);
    const Base& B0 = b0; const Base& B1 = b1;
    along(in, buf, 0, [&](const T* a, T* o) { B0.to_ortho(a, o); });
    Arr2<T> out(buf.n0, b1.len_ortho());
    along(buf, out, 1, [&](const T* a, T* o) { B1.to_ortho(a, o); });
    return out;
  }
  Arr2<T> from_ortho(const Arr2<T>& in) const {
    Arr2<T> buf(b0.m, in.n1);
    const Base& B0 = b0; const Base& B1 = b1;
    along(in, buf, 0, [&](const T* a, T* o) { B0.from_ortho(a, o); });
    Arr2<T> out(buf.n0, b1.m);
    along(buf, out, 1, [&](const T* a, T* o) { B1.from_ortho(a, o); });
    return out;
  }
  // gradient (space2.rs:246-264): differentiate axis 0, then axis 1, then / scale
  Arr2<T> gradient(const Arr2<T>& in, int d0, int d1, const double* scale) const {
    Arr2<T> buf(b0.len_ortho(), in.n1);
    const Base& B0 = b0; const Base& B1 = b1;
    along(in, buf, 0, [&](const T* a, T* o) { B0.to_ortho(a, o); B0.diff_ortho(o, d0); });
    Arr2<T> out(buf.n0, b1.len_ortho());
    along(buf, out, 1, [&](const T* a, T* o) { B1.to_ortho(a, o); B1.diff_ortho(o, d1); });
    if (scale) {
      // f64::powi: repeated multiplication
      double s0 = 1.0, s1 = 1.0;
      for (int i = 0; i < d0; i++) s0 *= scale[0];
      for (int i = 0; i < d1; i++) s1 *= scale[1];
      double sc = s0 * s1;
      for (auto& e : out.v) e = div_scale(e, sc);
    }
    return out;
  }
};

template <> Arr2<double> Space2<double>::forward0(const Arr2<double>& buf) const {
  Arr2<double> out(b0.m, buf.n1);
  const Base& B0 = b0;
  along(buf, out, 0, [&](const double* in, double* o) {
    thread_local std::vector<double> p;
    p.resize(B0.n);
    B0.cheb_forward(in, p.data());
    B0.from_ortho(p.data(), o);
  });
  return out;
}
template <> Arr2<cplx> Space2<cplx>::forward0(const Arr2<double>& buf) const {
  Arr2<cplx> out(b0.m, buf.n1);
  int n = b0.n;
  along(buf, out, 0, [&](const double* in, cplx* o) { rfft(in, o, n); });
  return out;
}
template <> Arr2<double> Space2<double>::backward0(const Arr2<double>& vhat) const {
  Arr2<double> out(b0.n, vhat.n1);
  const Base& B0 = b0;
  along(vhat, out, 0, [&](const double* in, double* o) {
    thread_local std::vector<double> p;
    p.resize(B0.n);
    B0.to_ortho(in, p.data());
    B0.cheb_backward(p.data(), o);
  });
  return out;
}
template <> Arr2<double> Space2<cplx>::backward0(const Arr2<cplx>& vhat) const {
  Arr2<double> out(b0.n, vhat.n1);
  int n = b0.n;
  along(vhat, out, 0, [&](const cplx* in, double* o) { irfft(in, o, n); });
  return out;
}

// ---------------------------------------------------------------------------
// Field2 (field.rs:67-163, average.rs:25-57)
// ---------------------------------------------------------------------------
template <class T> struct Field2 {
  Space2<T> space;
  Arr2<double> v;
  Arr2<T> vhat;
  std::vector<double> x[2], dx[2];
  Field2() = default;
  explicit Field2(const Space2<T>& s) : space(s) {
    v = Arr2<double>(s.phys0(), s.phys1());
    vhat = Arr2<T>(s.spec0(), s.spec1());
    x[0] = s.b0.x; x[1] = s.b1.x;
    for (int a = 0; a < 2; a++) {
      bool periodic = (a == 0 ? s.b0 : s.b1).fourier();
      dx[a] = get_dx(x[a], periodic);
    }
  }
  static std::vector<double> get_dx(const std::vector<double>& x, bool periodic) {
    size_t n = x.size();
    std::vector<double> dx(n);
    if (periodic) {
      for (size_t i = 0; i < n; i++) dx[i] = x[2] - x[1];
      return dx;
    }
    for (size_t i = 0; i < n; i++) {
      double l = i == 0 ? x[0] : (x[i] + x[i - 1]) / 2.0;
      double r = i == n - 1 ? x[n - 1] : (x[i + 1] + x[i]) / 2.0;
      dx[i] = r - l;
    }
    return dx;
  }
  void forward() { vhat = space.forward(v); }
  void backward() { v = space.backward(vhat); }
  Arr2<T> to_ortho() const { return space.to_ortho(vhat); }
  void from_ortho(const Arr2<T>& in) { vhat = space.from_ortho(in); }
  Arr2<T> gradient(int d0, int d1, const double* scale) const { return space.gradient(vhat, d0, d1, scale); }
  std::vector<double> average_axis(int axis) const {
    // average.rs:25-35: weighted = v * dx[axis] / length, summed over axis
    double length = std::fabs(x[axis].back() - x[axis][0]);
    int n0 = v.n0, n1 = v.n1;
    if (axis == 0) {
      std::vector<double> s(n1, 0.0);
      for (int i = 0; i < n0; i++)
        for (int j = 0; j < n1; j++) s[j] += v(i, j) * dx[0][i] / length;
      return s;
    }
    std::vector<double> s(n0, 0.0);
    for (int i = 0; i < n0; i++)
      for (int j = 0; j < n1; j++) s[i] += v(i, j) * dx[1][j] / length;
    return s;
  }
  double average() const {
    std::vector<double> ax = average_axis(0);
    double length = std::fabs(x[1].back() - x[1][0]);
    double s = 0.0;
    for (size_t j = 0; j < ax.size(); j++) s += ax[j] * dx[1][j] / length;
    return s;
  }
};

// ---------------------------------------------------------------------------
// Banded solvers (fdma.rs, matvec.rs)
// ---------------------------------------------------------------------------
static std::vector<double> diagonal(const Mat& a, int offset) {
  int n = a.n0;
  int m = std::abs(offset);
  std::vector<double> d(n - m);
  for (int i = 0; i < n - m; i++) d[i] = offset >= 0 ? a(i, i + m) : a(i + m, i);
  return d;
}

struct Fdma {
  int n = 0;
  std::vector<double> low, dia, up1, up2;
  bool swept = false;
  static Fdma raw(const Mat& a) {
    Fdma f;
    f.n = a.n0;
    f.low = diagonal(a, -2); f.dia = diagonal(a, 0); f.up1 = diagonal(a, 2); f.up2 = diagonal(a, 4);
    return f;
  }
  static Fdma from_matrix(const Mat& a) { Fdma f = raw(a); f.sweep(); return f; }
  void sweep() {  // fdma.rs:73-82
    for (int i = 2; i < n; i++) {
      low[i - 2] /= dia[i - 2];
      dia[i] -= low[i - 2] * up1[i - 2];
      if (i < n - 2) up1[i] -= low[i - 2] * up2[i - 2];
    }
    swept = true;
  }
  Fdma plus_scaled(const Fdma& o, double l) const {  // &fdma0 + &(&fdma1 * l)
    Fdma f;
    f.n = n;
    f.low.resize(low.size()); f.dia.resize(dia.size()); f.up1.resize(up1.size()); f.up2.resize(up2.size());
    for (size_t i = 0; i < low.size(); i++) f.low[i] = low[i] + o.low[i] * l;
    for (size_t i = 0; i < dia.size(); i++) f.dia[i] = dia[i] + o.dia[i] * l;
    for (size_t i = 0; i < up1.size(); i++) f.up1[i] = up1[i] + o.up1[i] * l;
    for (size_t i = 0; i < up2.size(); i++) f.up2[i] = up2[i] + o.up2[i] * l;
    return f;
  }
  template <class T> void solve_lane(T* x) const {  // fdma.rs:101-118
    for (int i = 2; i < n; i++) x[i] = x[i] - rmul(x[i - 2], low[i - 2]);
    x[n - 1] = rdiv(x[n - 1], dia[n - 1]);
    x[n - 2] = rdiv(x[n - 2], dia[n - 2]);
    x[n - 3] = rdiv(x[n - 3] - rmul(x[n - 1], up1[n - 3]), dia[n - 3]);
    x[n - 4] = rdiv(x[n - 4] - rmul(x[n - 2], up1[n - 4]), dia[n - 4]);
    for (int i = n - 5; i >= 0; i--)
      x[i] = rdiv(x[i] - rmul(x[i + 2], up1[i]) - rmul(x[i + 4], up2[i]), dia[i]);
  }
  template <class T> Arr2<T> solve(const Arr2<T>& in, int axis) const {
    if (!swept) throw std::runtime_error("Fdma: Forward sweep must be performed for solve! Abort.");
    Arr2<T> out(in.n0, in.n1);
    along(in, out, axis, [&](const T* a, T* o) {
      for (int i = 0; i < n; i++) o[i] = a[i];
      solve_lane(o);
    });
    return out;
  }
};

struct MatVecFdma {
  int m = 0, n = 0;
  std::vector<double> low, dia, up1, up2;
  MatVecFdma() = default;
  explicit MatVecFdma(const Mat& a) {  // matvec.rs:142-170
    m = a.n0; n = a.n1;
    low.assign(m, 0.0); dia.assign(m, 0.0); up1.assign(m, 0.0); up2.assign(m, 0.0);
    for (int i = 0; i < m; i++) {
      dia[i] = a(i, i);
      if (i > 1) low[i] = a(i, i - 2);
      if (i < m - 2) up1[i] = a(i, i + 2);
      if (i < m - 4) up2[i] = a(i, i + 4);
    }
  }
  template <class T> void lane(const T* in, T* out) const {  // matvec.rs:172-193
    int nn = m;
    for (int i = 0; i < nn; i++) {
      out[i] = rmul(in[i], dia[i]);
      if (i > 1) out[i] = out[i] + rmul(in[i - 2], low[i]);
      if (i < nn - 2) out[i] = out[i] + rmul(in[i + 2], up1[i]);
      if (i < nn - 4) out[i] = out[i] + rmul(in[i + 4], up2[i]);
    }
  }
  template <class T> Arr2<T> solve(const Arr2<T>& in, int axis) const {
    Arr2<T> out(axis == 0 ? m : in.n0, axis == 0 ? in.n1 : m);
    along(in, out, axis, [&](const T* a, T* o) { lane(a, o); });
    return out;
  }
};

// ---------------------------------------------------------------------------
// FdmaTensor (fdma_tensor.rs:105-235), 2-D only (1-D uses a swept Fdma)
// ---------------------------------------------------------------------------
struct FdmaTensor2 {
  int n = 0;
  Fdma fdma[2];
  bool diag0 = true;
  std::vector<double> lam;
  Mat fwd, bwd;  // when !diag0
  Mat a0, c0;    // kept for the external eigen-decomposition
  double alpha = 0.0;
  bool pending = false;
  void init(const Mat& a0_, const Mat& a1, const Mat& c0_, const Mat& c1, bool is_diag0, double alpha_) {
    alpha = alpha_;
    diag0 = is_diag0;
    if (is_diag0) lam = diagonal(a0_, 0);
    else { a0 = a0_; c0 = c0_; pending = true; }
    n = a1.n0;
    fdma[0] = Fdma::raw(a1);
    fdma[1] = Fdma::raw(c1);
  }
  template <class T> Arr2<T> solve(const Arr2<T>& in) const {
    if (pending) throw std::runtime_error("FdmaTensor: eigen-decomposition not supplied");
    if (in.n0 != (int)lam.size() || in.n1 != n) throw std::runtime_error("Dimension mismatch in Tensor!");
    Arr2<T> out(in.n0, in.n1);
    if (!diag0) out = dense0(fwd, in);
    else out = in;
    int rows = out.n0;
#pragma omp parallel for schedule(static) if (rows * n > 8192)
    for (int i = 0; i < rows; i++) {
      double l = lam[i] + alpha;
      Fdma f = fdma[0].plus_scaled(fdma[1], l);
      f.sweep();
      f.solve_lane(&out(i, 0));
    }
    if (!diag0) out = dense0(bwd, out);
    return out;
  }
  template <class T> static Arr2<T> dense0(const Mat& p, const Arr2<T>& x) {
    Arr2<T> y(p.n0, x.n1);
#pragma omp parallel for schedule(static) if (p.n0 * x.n1 > 8192)
    for (int i = 0; i < p.n0; i++)
      for (int k = 0; k < p.n1; k++) {
        double pik = p(i, k);
        if (pik == 0.0) continue;
        for (int j = 0; j < x.n1; j++) y(i, j) += rmul(x(k, j), pik);
      }
    return y;
  }
};

// Solver wrappers (hholtz.rs, hholtz_adi.rs, poisson.rs) -- 2-D and 1-D
enum SolverKind { S_HHOLTZ = 0, S_HHOLTZ_ADI = 1, S_POISSON = 2 };

struct Solver2 {
  int kind = S_HHOLTZ_ADI;
  bool has_mv[2] = {false, false};
  MatVecFdma mv[2];
  Fdma adi[2];         // HholtzAdi
  FdmaTensor2 tensor;  // Hholtz / Poisson
  template <class T> void build(const Space2<T>& sp, int kind_, const double c[2]) {
    kind = kind_;
    const Base* b[2] = {&sp.b0, &sp.b1};
    Mat A[2], B[2], P[2];
    for (int ax = 0; ax < 2; ax++) {
      bool hp;
      b[ax]->ingredients(A[ax], B[ax], P[ax], hp);
      has_mv[ax] = hp;
      if (hp) mv[ax] = MatVecFdma(P[ax]);
    }
    if (kind == S_HHOLTZ_ADI) {
      for (int ax = 0; ax < 2; ax++) {
        Mat mat(A[ax].n0, A[ax].n1);
        for (size_t i = 0; i < mat.v.size(); i++) mat.v[i] = A[ax].v[i] - B[ax].v[i] * c[ax];
        adi[ax] = Fdma::from_matrix(mat);
      }
      return;
    }
    Mat lap[2], mss[2];
    for (int ax = 0; ax < 2; ax++) {
      lap[ax] = Mat(B[ax].n0, B[ax].n1);
      for (size_t i = 0; i < lap[ax].v.size(); i++)
        lap[ax].v[i] = kind == S_HHOLTZ ? (-1.0 * B[ax].v[i]) * c[ax] : B[ax].v[i] * c[ax];
      mss[ax] = A[ax];
    }
    tensor.init(lap[0], lap[1], mss[0], mss[1], b[0]->fourier(), kind == S_HHOLTZ ? 1.0 : 0.0);
    if (kind == S_POISSON && !tensor.pending) singular_shift();
  }
  void singular_shift() {  // poisson.rs:80-83
    if (std::fabs(tensor.lam[0]) < 1e-10)
      for (auto& l : tensor.lam) l -= 1e-10;
  }
  void set_eig(const double* lam, const double* fwd, const double* bwd) {
    int m = tensor.a0.n0;
    tensor.lam.assign(lam, lam + m);
    tensor.fwd = Mat(m, m);
    tensor.bwd = Mat(m, m);
    std::memcpy(tensor.fwd.data(), fwd, sizeof(double) * m * m);
    std::memcpy(tensor.bwd.data(), bwd, sizeof(double) * m * m);
    tensor.pending = false;
    if (kind == S_POISSON) singular_shift();
  }
  template <class T> Arr2<T> solve(const Arr2<T>& in) const {
    Arr2<T> rhs = has_mv[0] ? mv[0].solve(in, 0) : in;
    if (has_mv[1]) rhs = mv[1].solve(rhs, 1);
    if (kind == S_HHOLTZ_ADI) {
      Arr2<T> o = adi[0].solve(rhs, 0);
      return adi[1].solve(o, 1);
    }
    return tensor.solve(rhs);
  }
};

// 1-D solvers for the reference's 1-D known-answer tests
struct Solver1 {
  bool has_mv = false;
  MatVecFdma mv;
  Fdma f;
  void build(const Base& b, int kind, double c) {
    Mat A, B, P;
    bool hp;
    b.ingredients(A, B, P, hp);
    has_mv = hp;
    if (hp) mv = MatVecFdma(P);
    Mat mat(A.n0, A.n1);
    if (kind == S_HHOLTZ_ADI) {
      for (size_t i = 0; i < mat.v.size(); i++) mat.v[i] = A.v[i] - B.v[i] * c;
    } else if (kind == S_HHOLTZ) {  // FdmaTensor<1>: only a = laplacian is used
      for (size_t i = 0; i < mat.v.size(); i++) mat.v[i] = (-1.0 * B.v[i]) * c;
    } else {
      for (size_t i = 0; i < mat.v.size(); i++) mat.v[i] = B.v[i] * c;
    }
    f = Fdma::from_matrix(mat);
  }
  void solve(const double* in, double* out) const {
    std::vector<double> rhs(f.n);
    if (has_mv) mv.lane(in, rhs.data());
    else for (int i = 0; i < f.n; i++) rhs[i] = in[i];
    for (int i = 0; i < f.n; i++) out[i] = rhs[i];
    f.solve_lane(out);
  }
};

// ---------------------------------------------------------------------------
// Navier2D (navier.rs)
// ---------------------------------------------------------------------------
inline double get_nu(double ra, double pr, double h) { double f = pr / (ra / std::pow(h, 3.0)); return std::sqrt(f); }
inline double get_ka(double ra, double pr, double h) { double f = 1.0 / ((ra / std::pow(h, 3.0)) * pr); return std::sqrt(f); }

inline uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

template <class T> struct Navier2D {
  Field2<T> field, temp, ux, uy, pres[2], fieldbc;
  Solver2 solver[4];
  double nu, ka, ra, pr, time = 0.0, dt;
  double scale[2];
  bool dealias_on = true;
  bool periodic = false;
  // solid-mask penalisation (navier.rs:189-190, 551-560, 579-584, 603-608):
  // solid[0] = mask, solid[1] = target temperature, both physical (nx x ny)
  bool has_solid = false;
  Arr2<double> solid[2];
  static constexpr double solid_eta = 1e-2;

  void scale_coords() {  // navier.rs:500-512
    Field2<T>* fs[4] = {&temp, &ux, &uy, &pres[0]};
    for (auto f : fs) {
      for (auto& e : f->x[0]) e *= scale[0];
      for (auto& e : f->x[1]) e *= scale[1];
      for (auto& e : f->dx[0]) e *= scale[0];
      for (auto& e : f->dx[1]) e *= scale[1];
    }
  }
  void build(int nx, int ny, double ra_, double pr_, double dt_, double aspect, int kind);

  // conv_term.rs:22-42  u * backward(gradient(field))
  Arr2<double> conv_term(const Field2<T>& f, const Arr2<double>& u, int d0, int d1) {
    field.vhat = f.gradient(d0, d1, scale);
    field.backward();
    Arr2<double> r(u.n0, u.n1);
    for (size_t i = 0; i < r.v.size(); i++) r.v[i] = u.v[i] * field.v.v[i];
    return r;
  }
  void dealias(Arr2<T>& vh) {  // navier.rs:1022-1032
    int nxk = vh.n0 * 2 / 3, nyk = vh.n1 * 2 / 3;
    for (int i = 0; i < vh.n0; i++)
      for (int j = 0; j < vh.n1; j++)
        if (i >= nxk || j >= nyk) vh(i, j) = T(0);
  }
  static void add(Arr2<double>& a, const Arr2<double>& b) { for (size_t i = 0; i < a.v.size(); i++) a.v[i] += b.v[i]; }
  Arr2<T> conv_finish(const Arr2<double>& conv) {
    field.v = conv;
    field.forward();
    if (dealias_on) dealias(field.vhat);
    return field.vhat;
  }
  // conv -= damp with damp = (-1/eta) * mask * w  (navier.rs:579-584)
  void solid_damp(Arr2<double>& c, const Arr2<double>& w) const {
    for (size_t i = 0; i < c.v.size(); i++) c.v[i] -= ((-1.0 / solid_eta) * solid[0].v[i]) * w.v[i];
  }
  Arr2<T> conv_ux(const Arr2<double>& u, const Arr2<double>& v) {
    Arr2<double> c = conv_term(ux, u, 1, 0);
    add(c, conv_term(ux, v, 0, 1));
    if (has_solid) solid_damp(c, u);
    return conv_finish(c);
  }
  Arr2<T> conv_uy(const Arr2<double>& u, const Arr2<double>& v) {
    Arr2<double> c = conv_term(uy, u, 1, 0);
    add(c, conv_term(uy, v, 0, 1));
    if (has_solid) solid_damp(c, v);
    return conv_finish(c);
  }
  Arr2<T> conv_temp(const Arr2<double>& u, const Arr2<double>& v) {
    Arr2<double> c = conv_term(temp, u, 1, 0);
    add(c, conv_term(temp, v, 0, 1));
    add(c, conv_term(fieldbc, u, 1, 0));
    add(c, conv_term(fieldbc, v, 0, 1));
    if (has_solid) {  // navier.rs:551-560: damp = (-1/eta) * mask * (T + T_bc - value)
      temp.backward();
      Arr2<double> w(c.n0, c.n1);
      for (size_t i = 0; i < w.v.size(); i++) w.v[i] = (temp.v.v[i] + fieldbc.v.v[i]) - solid[1].v[i];
      solid_damp(c, w);
    }
    return conv_finish(c);
  }
  static void axpy(Arr2<T>& r, const Arr2<T>& x, double a) {  // r += x * a (or r -= via a<0 handled by caller)
    for (size_t i = 0; i < r.v.size(); i++) r.v[i] += rmul(x.v[i], a);
  }
  static void sub_scaled(Arr2<T>& r, const Arr2<T>& x, double a) {
    for (size_t i = 0; i < r.v.size(); i++) r.v[i] -= rmul(x.v[i], a);
  }
  void solve_ux(const Arr2<double>& u, const Arr2<double>& v) {  // navier.rs:622-633
    Arr2<T> rhs = ux.to_ortho();
    sub_scaled(rhs, pres[0].gradient(1, 0, scale), dt);
    Arr2<T> conv = conv_ux(u, v);
    sub_scaled(rhs, conv, dt);
    ux.vhat = solver[0].solve(rhs);
  }
  void solve_uy(const Arr2<double>& u, const Arr2<double>& v, const Arr2<T>& buoy) {  // :636-654
    Arr2<T> rhs = uy.to_ortho();
    sub_scaled(rhs, pres[0].gradient(0, 1, scale), dt);
    axpy(rhs, buoy, dt);
    Arr2<T> conv = conv_uy(u, v);
    sub_scaled(rhs, conv, dt);
    uy.vhat = solver[1].solve(rhs);
  }
  void solve_temp(const Arr2<double>& u, const Arr2<double>& v) {  // :660-674
    Arr2<T> rhs = temp.to_ortho();
    Arr2<T> g = fieldbc.gradient(2, 0, scale);
    for (size_t i = 0; i < rhs.v.size(); i++) rhs.v[i] += rmul(rmul(g.v[i], dt), ka);
    g = fieldbc.gradient(0, 2, scale);
    for (size_t i = 0; i < rhs.v.size(); i++) rhs.v[i] += rmul(rmul(g.v[i], dt), ka);
    Arr2<T> conv = conv_temp(u, v);
    sub_scaled(rhs, conv, dt);
    temp.vhat = solver[2].solve(rhs);
  }
  Arr2<T> divergence() {  // :698-703
    Arr2<T> r = ux.gradient(1, 0, scale);
    Arr2<T> b = uy.gradient(0, 1, scale);
    for (size_t i = 0; i < r.v.size(); i++) r.v[i] += b.v[i];
    return r;
  }
  void project_velocity(double c) {  // :683-695
    Arr2<T> dpdx = pres[1].gradient(1, 0, scale);
    Arr2<T> dpdy = pres[1].gradient(0, 1, scale);
    Arr2<T> ux_old = ux.vhat, uy_old = uy.vhat;
    ux.from_ortho(dpdx);
    uy.from_ortho(dpdy);
    T cinto = T(-c);
    for (size_t i = 0; i < ux.vhat.v.size(); i++) ux.vhat.v[i] = mulT(ux.vhat.v[i], cinto) + ux_old.v[i];
    for (size_t i = 0; i < uy.vhat.v.size(); i++) uy.vhat.v[i] = mulT(uy.vhat.v[i], cinto) + uy_old.v[i];
  }
  static double mulT(double a, double b) { return a * b; }
  static cplx mulT(cplx a, cplx b) { return cmul(a, b); }
  static cplx divT(cplx a, cplx b) {  // num_complex division
    double ns = b.real() * b.real() + b.imag() * b.imag();
    double re = a.real() * b.real() + a.imag() * b.imag();
    double im = a.imag() * b.real() - a.real() * b.imag();
    return cplx(re / ns, im / ns);
  }
  void solve_pres(const Arr2<T>& f) {  // :710-715
    pres[1].vhat = solver[3].solve(f);
    pres[1].vhat(0, 0) = T(0);
  }
  void update_pres(const Arr2<T>& div) {  // :717-721
    Arr2<T>& p0 = pres[0].vhat;
    for (size_t i = 0; i < p0.v.size(); i++) p0.v[i] = p0.v[i] - rmul(div.v[i], nu);
    T inv_dt = T(1.0 / dt);
    Arr2<T> p1o = pres[1].to_ortho();
    for (size_t i = 0; i < p0.v.size(); i++) p0.v[i] = p0.v[i] + mulT(p1o.v[i], inv_dt);
  }
  void update() {  // navier.rs:737-765
    Arr2<T> that = temp.to_ortho();
    Arr2<T> bo = fieldbc.to_ortho();
    for (size_t i = 0; i < that.v.size(); i++) that.v[i] = that.v[i] + bo.v[i];
    ux.backward();
    uy.backward();
    Arr2<double> u = ux.v, v = uy.v;
    solve_ux(u, v);
    solve_uy(u, v, that);
    Arr2<T> div = divergence();
    solve_pres(div);
    project_velocity(1.0);
    update_pres(div);
    solve_temp(u, v);
    time += dt;
  }
  // functions.rs:12-101
  double eval_nu() {
    field.vhat = temp.to_ortho();
    Arr2<T> bo = fieldbc.to_ortho();
    for (size_t i = 0; i < field.vhat.v.size(); i++) field.vhat.v[i] = field.vhat.v[i] + bo.v[i];
    Arr2<T> dtdz = field.gradient(0, 1, nullptr);
    for (auto& e : dtdz.v) e = rmul(e, -1.0);
    for (auto& e : dtdz.v) e = rmul(e, 1.0 / (scale[1] / 2.0));
    field.vhat = dtdz;
    field.backward();
    std::vector<double> xa = field.average_axis(0);
    return (xa.back() + xa[0]) / 2.0;
  }
  double eval_nuvol() {
    field.vhat = temp.to_ortho();
    Arr2<T> bo = fieldbc.to_ortho();
    for (size_t i = 0; i < field.vhat.v.size(); i++) field.vhat.v[i] = field.vhat.v[i] + bo.v[i];
    field.backward();
    uy.backward();
    Arr2<double> uyt(field.v.n0, field.v.n1);
    for (size_t i = 0; i < uyt.v.size(); i++) uyt.v[i] = field.v.v[i] * uy.v.v[i];
    Arr2<T> dtdz = field.gradient(0, 1, nullptr);
    for (auto& e : dtdz.v) e = rdiv(e, scale[1] * -1.0);
    field.vhat = dtdz;
    field.backward();
    for (size_t i = 0; i < uyt.v.size(); i++) field.v.v[i] = (field.v.v[i] + uyt.v[i] / ka) * 2.0 * scale[1];
    return field.average();
  }
  double eval_re() {
    ux.backward();
    uy.backward();
    for (size_t i = 0; i < field.v.v.size(); i++) {
      double e = ux.v.v[i] * ux.v.v[i] + uy.v.v[i] * uy.v.v[i];
      field.v.v[i] = std::sqrt(e);
    }
    for (auto& e : field.v.v) e *= 2.0 * scale[1] / nu;
    return field.average();
  }
  // kinetic energy <(ux^2+uy^2)/2> with the same volume weights as eval_re
  double eval_ke() {
    ux.backward();
    uy.backward();
    for (size_t i = 0; i < field.v.v.size(); i++)
      field.v.v[i] = 0.5 * (ux.v.v[i] * ux.v.v[i] + uy.v.v[i] * uy.v.v[i]);
    return field.average();
  }
  double div_norm() {
    Arr2<T> d = divergence();
    double s = 0.0;
    for (auto& e : d.v) s += sq(e);
    return std::sqrt(s);
  }
  static double sq(double a) { return a * a; }
  static double sq(cplx a) { return a.real() * a.real() + a.imag() * a.imag(); }
  // navier.rs:1035-1076 apply_sin_cos / apply_cos_sin
  static void apply_mode(Field2<T>& f, double amp, double m, double n, bool sin_cos) {
    const auto& x = f.x[0];
    const auto& y = f.x[1];
    std::vector<double> xs(x.size()), ys(y.size());
    for (size_t i = 0; i < x.size(); i++) xs[i] = (x[i] - x[0]) / (x.back() - x[0]);
    for (size_t j = 0; j < y.size(); j++) ys[j] = (y[j] - y[0]) / (y.back() - y[0]);
    double ax = PI * m, ay = PI * n;
    for (int i = 0; i < f.v.n0; i++)
      for (int j = 0; j < f.v.n1; j++)
        f.v(i, j) = sin_cos ? amp * std::sin(ax * xs[i]) * std::cos(ay * ys[j])
                            : amp * std::cos(ax * xs[i]) * std::sin(ay * ys[j]);
    f.forward();
  }
  void set_velocity(double amp, double m, double n) {
    apply_mode(ux, amp, m, n, true);
    apply_mode(uy, -amp, m, n, false);
  }
  void set_temperature(double amp, double m, double n) { apply_mode(temp, -amp, m, n, false); }
  // seeded interior noise: u = (splitmix64 >> 11) * 2^-53 drawn in row-major
  // order over every grid point; value amp*(2u-1) at interior points, 0 on walls.
  void set_temperature_noise(double amp, uint64_t seed) {
    uint64_t s = seed;
    int n0 = temp.v.n0, n1 = temp.v.n1;
    for (int i = 0; i < n0; i++)
      for (int j = 0; j < n1; j++) {
        double u = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
        bool wall = (j == 0 || j == n1 - 1) || (!periodic && (i == 0 || i == n0 - 1));
        temp.v(i, j) = wall ? 0.0 : amp * (2.0 * u - 1.0);
      }
    temp.forward();
  }
  void zero_pressure() {
    for (auto& e : pres[0].vhat.v) e = T(0);
    for (auto& e : pres[1].vhat.v) e = T(0);
  }
};

template <> void Navier2D<double>::build(int nx, int ny, double ra_, double pr_, double dt_, double aspect, int kind) {
  // navier.rs:219-307 (kind 0: adiabatic sidewalls, 1: conducting)
  periodic = false;
  ra = ra_; pr = pr_; dt = dt_;
  scale[0] = aspect; scale[1] = 1.0;
  nu = get_nu(ra, pr, scale[1] * 2.0);
  ka = get_ka(ra, pr, scale[1] * 2.0);
  ux = Field2<double>(Space2<double>(Base(CD, nx), Base(CD, ny)));
  uy = Field2<double>(Space2<double>(Base(CD, nx), Base(CD, ny)));
  temp = Field2<double>(Space2<double>(Base(kind == 0 ? CN : CD, nx), Base(CD, ny)));
  pres[0] = Field2<double>(Space2<double>(Base(CHEB, nx), Base(CHEB, ny)));
  pres[1] = Field2<double>(Space2<double>(Base(CN, nx), Base(CN, ny)));
  field = Field2<double>(Space2<double>(Base(CHEB, nx), Base(CHEB, ny)));
  double cu[2] = {dt * nu / std::pow(scale[0], 2.0), dt * nu / std::pow(scale[1], 2.0)};
  double ct[2] = {dt * ka / std::pow(scale[0], 2.0), dt * ka / std::pow(scale[1], 2.0)};
  double cp[2] = {1.0 / std::pow(scale[0], 2.0), 1.0 / std::pow(scale[1], 2.0)};
  solver[0].build(ux.space, S_HHOLTZ_ADI, cu);
  solver[1].build(uy.space, S_HHOLTZ_ADI, cu);
  solver[2].build(temp.space, S_HHOLTZ_ADI, ct);
  solver[3].build(pres[1].space, S_POISSON, cp);
  scale_coords();
  // bc_rbc (navier.rs:314-332)
  Base xb(CHEB, nx), yb(CDBC, ny);
  fieldbc = Field2<double>(Space2<double>(xb, yb));
  Arr2<double> bc(nx, 2);
  for (int i = 0; i < nx; i++) { bc(i, 0) = 0.5; bc(i, 1) = -0.5; }
  along(bc, fieldbc.vhat, 0, [&](const double* in, double* o) { xb.cheb_forward(in, o); });
  fieldbc.backward();
  fieldbc.forward();
}

template <> void Navier2D<cplx>::build(int nx, int ny, double ra_, double pr_, double dt_, double aspect, int) {
  // navier.rs:384-467
  periodic = true;
  ra = ra_; pr = pr_; dt = dt_;
  scale[0] = aspect; scale[1] = 1.0;
  nu = get_nu(ra, pr, scale[1] * 2.0);
  ka = get_ka(ra, pr, scale[1] * 2.0);
  ux = Field2<cplx>(Space2<cplx>(Base(FOURIER, nx), Base(CD, ny)));
  uy = Field2<cplx>(Space2<cplx>(Base(FOURIER, nx), Base(CD, ny)));
  temp = Field2<cplx>(Space2<cplx>(Base(FOURIER, nx), Base(CD, ny)));
  pres[0] = Field2<cplx>(Space2<cplx>(Base(FOURIER, nx), Base(CHEB, ny)));
  pres[1] = Field2<cplx>(Space2<cplx>(Base(FOURIER, nx), Base(CN, ny)));
  field = Field2<cplx>(Space2<cplx>(Base(FOURIER, nx), Base(CHEB, ny)));
  double cu[2] = {dt * nu / std::pow(scale[0], 2.0), dt * nu / std::pow(scale[1], 2.0)};
  double ct[2] = {dt * ka / std::pow(scale[0], 2.0), dt * ka / std::pow(scale[1], 2.0)};
  double cp[2] = {1.0 / std::pow(scale[0], 2.0), 1.0 / std::pow(scale[1], 2.0)};
  solver[0].build(ux.space, S_HHOLTZ, cu);
  solver[1].build(uy.space, S_HHOLTZ, cu);
  solver[2].build(temp.space, S_HHOLTZ, ct);
  solver[3].build(pres[1].space, S_POISSON, cp);
  scale_coords();
  // bc_rbc_periodic (navier.rs:474-492)
  Base xb(FOURIER, nx), yb(CDBC, ny);
  fieldbc = Field2<cplx>(Space2<cplx>(xb, yb));
  Arr2<double> bc(nx, 2);
  for (int i = 0; i < nx; i++) { bc(i, 0) = 0.5; bc(i, 1) = -0.5; }
  along(bc, fieldbc.vhat, 0, [&](const double* in, cplx* o) { rfft(in, o, nx); });
  fieldbc.backward();
  fieldbc.forward();
}

// ---------------------------------------------------------------------------
// Navier2DAdjoint (navier_adjoint.rs): adjoint descent towards steady states
// (Farazmand 2016).  Each update runs one Navier2D step (dt_navier = 1e-2) to
// form the residual, smooths it with (1 - D2) Hholtz solves, and advances the
// state with the adjoint convection, explicit diffusion and a projection.
// ---------------------------------------------------------------------------
template <class T> struct Navier2DAdjoint {
  Navier2D<T> navier;
  Field2<T> field, temp[2], ux[2], uy[2], pres[2], fieldbc;
  Solver2 solver;        // Poisson on pres[1]
  Solver2 smoother[3];   // Hholtz (1 - D2) for ux, uy, temp
  Arr2<T> unsmoothed[3];
  double nu, ka, ra, pr, time = 0.0, dt, dt_navier = 1e-2;
  double scale[2];
  bool periodic = false;
  bool dealias_on = true;
  double res_tol = 1e-8;  // navier_adjoint.rs:120

  void build(int nx, int ny, double ra_, double pr_, double dt_, double aspect, int kind) {
    // navier_adjoint.rs:151-283 (box) and :287-409 (periodic)
    periodic = kind == 2;
    ra = ra_; pr = pr_; dt = dt_;
    scale[0] = aspect; scale[1] = 1.0;
    nu = get_nu(ra, pr, scale[1] * 2.0);
    ka = get_ka(ra, pr, scale[1] * 2.0);
    navier.build(nx, ny, ra, pr, dt_navier, aspect, kind);
    int xu = periodic ? FOURIER : CD, xt = periodic ? FOURIER : (kind == 0 ? CN : CD);
    int xo = periodic ? FOURIER : CHEB, xp = periodic ? FOURIER : CN;
    for (int k = 0; k < 2; k++) {
      ux[k] = Field2<T>(Space2<T>(Base(xu, nx), Base(CD, ny)));
      uy[k] = Field2<T>(Space2<T>(Base(xu, nx), Base(CD, ny)));
      temp[k] = Field2<T>(Space2<T>(Base(xt, nx), Base(CD, ny)));
    }
    pres[0] = Field2<T>(Space2<T>(Base(xo, nx), Base(CHEB, ny)));
    pres[1] = Field2<T>(Space2<T>(Base(xp, nx), Base(CN, ny)));
    field = Field2<T>(Space2<T>(Base(xo, nx), Base(CHEB, ny)));
    double cp[2] = {1.0 / std::pow(scale[0], 2.0), 1.0 / std::pow(scale[1], 2.0)};
    solver.build(pres[1].space, S_POISSON, cp);
    const double w = 1e0;  // weight_laplacian
    double cs[2] = {w / std::pow(scale[0], 2.0), w / std::pow(scale[1], 2.0)};
    smoother[0].build(ux[1].space, S_HHOLTZ, cs);
    smoother[1].build(uy[1].space, S_HHOLTZ, cs);
    smoother[2].build(temp[1].space, S_HHOLTZ, cs);
    // _scale (navier_adjoint.rs:419-438)
    Field2<T>* fs[7] = {&temp[0], &ux[0], &uy[0], &pres[0], &temp[1], &ux[1], &uy[1]};
    for (auto f : fs) {
      for (auto& e : f->x[0]) e *= scale[0];
      for (auto& e : f->x[1]) e *= scale[1];
      for (auto& e : f->dx[0]) e *= scale[0];
      for (auto& e : f->dx[1]) e *= scale[1];
    }
    fieldbc = navier.fieldbc;  // set_temp_bc(Navier2D::bc_rbc(nx, ny)), the same construction
  }
  Solver2* tensor_solver(int k) {
    switch (k) {
      case 0: return &navier.solver[3];
      case 1: return &solver;
      default: return &smoother[k - 2];
    }
  }
  static void add(Arr2<double>& a, const Arr2<double>& b) { for (size_t i = 0; i < a.v.size(); i++) a.v[i] += b.v[i]; }
  static T mulT(T a, T b) { return Navier2D<T>::mulT(a, b); }
  // conv_term.rs:22-42 on this solver's `field`
  Arr2<double> conv_term(const Field2<T>& f, const Arr2<double>& u, int d0, int d1) {
    field.vhat = f.gradient(d0, d1, scale);
    field.backward();
    Arr2<double> r(u.n0, u.n1);
    for (size_t i = 0; i < r.v.size(); i++) r.v[i] = u.v[i] * field.v.v[i];
    return r;
  }
  Arr2<T> conv_finish(const Arr2<double>& conv) {
    field.v = conv;
    field.forward();
    if (dealias_on) {  // navier.rs:1022-1032
      Arr2<T>& vh = field.vhat;
      int nxk = vh.n0 * 2 / 3, nyk = vh.n1 * 2 / 3;
      for (int i = 0; i < vh.n0; i++)
        for (int j = 0; j < vh.n1; j++)
          if (i >= nxk || j >= nyk) vh(i, j) = T(0);
    }
    return field.vhat;
  }
  // navier_adjoint.rs:541-577
  Arr2<T> conv_ux(const Arr2<double>& u, const Arr2<double>& v, const Arr2<double>& t) {
    Arr2<double> c = conv_term(ux[1], u, 1, 0);
    add(c, conv_term(ux[1], v, 0, 1));
    add(c, conv_term(ux[1], u, 1, 0));
    add(c, conv_term(uy[1], v, 1, 0));
    add(c, conv_term(temp[1], t, 1, 0));
    add(c, conv_term(temp[1], fieldbc.v, 1, 0));
    return conv_finish(c);
  }
  // navier_adjoint.rs:579-611
  Arr2<T> conv_uy(const Arr2<double>& u, const Arr2<double>& v, const Arr2<double>& t) {
    Arr2<double> c = conv_term(uy[1], u, 1, 0);
    add(c, conv_term(uy[1], v, 0, 1));
    add(c, conv_term(ux[1], u, 0, 1));
    add(c, conv_term(uy[1], v, 0, 1));
    add(c, conv_term(temp[1], t, 0, 1));
    add(c, conv_term(temp[1], fieldbc.v, 0, 1));
    return conv_finish(c);
  }
  // navier_adjoint.rs:613-628
  Arr2<T> conv_temp(const Arr2<double>& u, const Arr2<double>& v) {
    Arr2<double> c = conv_term(temp[1], u, 1, 0);
    add(c, conv_term(temp[1], v, 0, 1));
    return conv_finish(c);
  }
  static void add_scaled(Arr2<T>& r, const Arr2<T>& x, double a) { for (size_t i = 0; i < r.v.size(); i++) r.v[i] += rmul(x.v[i], a); }
  static void sub_scaled(Arr2<T>& r, const Arr2<T>& x, double a) { for (size_t i = 0; i < r.v.size(); i++) r.v[i] -= rmul(x.v[i], a); }
  static void add_scaled2(Arr2<T>& r, const Arr2<T>& x, double a, double b) {
    for (size_t i = 0; i < r.v.size(); i++) r.v[i] += rmul(rmul(x.v[i], a), b);
  }
  // navier_adjoint.rs:630-653 / 655-678: explicit update of the velocity
  void solve_u(int which, const Arr2<double>& u, const Arr2<double>& v, const Arr2<double>& t) {
    Field2<T>& f0 = which == 0 ? ux[0] : uy[0];
    Field2<T>& f1 = which == 0 ? ux[1] : uy[1];
    Arr2<T> rhs = f0.to_ortho();
    sub_scaled(rhs, which == 0 ? pres[0].gradient(1, 0, scale) : pres[0].gradient(0, 1, scale), dt);
    Arr2<T> conv = which == 0 ? conv_ux(u, v, t) : conv_uy(u, v, t);
    add_scaled(rhs, conv, dt);
    add_scaled2(rhs, f1.gradient(2, 0, scale), dt, nu);
    add_scaled2(rhs, f1.gradient(0, 2, scale), dt, nu);
    f0.from_ortho(rhs);
  }
  // navier_adjoint.rs:680-695
  void solve_temp(const Arr2<double>& u, const Arr2<double>& v) {
    Arr2<T> rhs = temp[0].to_ortho();
    Arr2<T> conv = conv_temp(u, v);
    add_scaled(rhs, conv, dt);
    add_scaled(rhs, uy[1].to_ortho(), dt);
    add_scaled2(rhs, temp[1].gradient(2, 0, scale), dt, ka);
    add_scaled2(rhs, temp[1].gradient(0, 2, scale), dt, ka);
    temp[0].from_ortho(rhs);
  }
  void project_velocity(double c) {  // navier_adjoint.rs:697-710
    Arr2<T> dpdx = pres[1].gradient(1, 0, scale);
    Arr2<T> dpdy = pres[1].gradient(0, 1, scale);
    Arr2<T> ox = ux[0].vhat, oy = uy[0].vhat;
    ux[0].from_ortho(dpdx);
    uy[0].from_ortho(dpdy);
    T cinto = T(-c);
    for (size_t i = 0; i < ux[0].vhat.v.size(); i++) ux[0].vhat.v[i] = mulT(ux[0].vhat.v[i], cinto) + ox.v[i];
    for (size_t i = 0; i < uy[0].vhat.v.size(); i++) uy[0].vhat.v[i] = mulT(uy[0].vhat.v[i], cinto) + oy.v[i];
  }
  Arr2<T> divergence() {  // navier_adjoint.rs:712-717
    Arr2<T> r = ux[0].gradient(1, 0, scale);
    Arr2<T> b = uy[0].gradient(0, 1, scale);
    for (size_t i = 0; i < r.v.size(); i++) r.v[i] += b.v[i];
    return r;
  }
  void solve_pres(const Arr2<T>& f) {  // navier_adjoint.rs:719-723
    pres[1].vhat = solver.solve(f);
    pres[1].vhat(0, 0) = T(0);
  }
  void update_pres() {  // navier_adjoint.rs:725-729
    T inv_dt = T(1.0 / dt);
    Arr2<T> p1o = pres[1].to_ortho();
    for (size_t i = 0; i < p1o.v.size(); i++) pres[0].vhat.v[i] += mulT(p1o.v[i], inv_dt);
  }
  void update_residual() {  // navier_adjoint.rs:731-754
    navier.ux.vhat = ux[0].vhat;
    navier.uy.vhat = uy[0].vhat;
    navier.temp.vhat = temp[0].vhat;
    navier.update();
    Field2<T>* nf[3] = {&navier.ux, &navier.uy, &navier.temp};
    Field2<T>* sf[3] = {&ux[0], &uy[0], &temp[0]};
    Field2<T>* rf[3] = {&ux[1], &uy[1], &temp[1]};
    for (int k = 0; k < 3; k++) {
      Arr2<T>& a = nf[k]->vhat;
      for (size_t i = 0; i < a.v.size(); i++) a.v[i] = rdiv(a.v[i] - sf[k]->vhat.v[i], navier.dt);
      unsmoothed[k] = nf[k]->to_ortho();
      rf[k]->vhat = smoother[k].solve(unsmoothed[k]);
      T rescale = T(-1.0);
      for (auto& e : rf[k]->vhat.v) e = mulT(e, rescale);
    }
  }
  void update() {  // navier_adjoint.rs:767-800
    ux[0].backward();
    uy[0].backward();
    temp[0].backward();
    Arr2<double> u = ux[0].v, v = uy[0].v, t = temp[0].v;
    update_residual();
    solve_u(0, u, v, t);
    solve_u(1, u, v, t);
    Arr2<T> div = divergence();
    solve_pres(div);
    project_velocity(1.0);
    update_pres();
    solve_temp(u, v);
    time += dt;
  }
  static double norm_l2(const Arr2<T>& a) {  // navier_adjoint.rs:915-925
    double s = 0.0;
    for (const auto& e : a.v) s += Navier2D<T>::sq(e);
    return std::sqrt(s);
  }
  bool exit() {  // navier_adjoint.rs:889-906
    if (std::isnan(norm_l2(divergence()))) return true;
    return norm_l2(ux[1].vhat) + norm_l2(uy[1].vhat) + norm_l2(temp[1].vhat) < res_tol;
  }
  // Nu, Nuvol, Re of the adjoint state (navier_adjoint.rs:932-963): the same
  // functions on fields of the same spaces, evaluated through `navier`
  double eval(int what) {
    navier.ux.vhat = ux[0].vhat;
    navier.uy.vhat = uy[0].vhat;
    navier.temp.vhat = temp[0].vhat;
    switch (what) {
      case 0: return navier.eval_nu();
      case 1: return navier.eval_nuvol();
      case 2: return navier.eval_re();
      case 3: return navier.eval_ke();
      default: return norm_l2(divergence());
    }
  }
};

}  // namespace oracle

// ===========================================================================
// C interface for the Python side of the oracle (ctypes).
// ===========================================================================
using namespace oracle;

struct OrNavier {
  bool periodic;
  Navier2D<double> box;
  Navier2D<cplx> per;
};

static thread_local std::string g_err;

// field ids: 0 temp, 1 ux, 2 uy, 3 pres0, 4 pres1, 5 fieldbc
template <class T> static Field2<T>* pick(Navier2D<T>& n, int id) {
  switch (id) {
    case 0: return &n.temp;
    case 1: return &n.ux;
    case 2: return &n.uy;
    case 3: return &n.pres[0];
    case 4: return &n.pres[1];
    case 5: return &n.fieldbc;
    case 6: return &n.field;
  }
  return nullptr;
}
template <class T> static Arr2<T> mk(const double* d, int n0, int n1) {
  Arr2<T> a(n0, n1);
  std::memcpy(a.data(), d, sizeof(T) * a.size());
  return a;
}
template <class T> static void put(const Arr2<T>& a, double* out) { std::memcpy(out, a.data(), sizeof(T) * a.size()); }

extern "C" {

const char* or_last_error() { return g_err.c_str(); }

int or_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
void or_set_dense_dct(int n) { g_dense_dct_n.store(n); }

// ---- Navier2D ------------------------------------------------------------
// kind: 0 box adiabatic (Navier2D::new, adiabatic=true), 1 box conducting,
//       2 periodic (Navier2D::new_periodic)
void* or_navier_new(int nx, int ny, double ra, double pr, double dt, double aspect, int kind) {
  try {
    auto* h = new OrNavier();
    h->periodic = kind == 2;
    if (h->periodic) h->per.build(nx, ny, ra, pr, dt, aspect, kind);
    else h->box.build(nx, ny, ra, pr, dt, aspect, kind);
    return h;
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void or_navier_free(void* p) { delete (OrNavier*)p; }

// Box Poisson needs the dense eigen-decomposition from the Python side.
int or_navier_tensor_pending(void* p, int* m) {
  auto* h = (OrNavier*)p;
  if (h->periodic) return 0;
  auto& t = h->box.solver[3].tensor;
  if (!t.pending) return 0;
  *m = t.a0.n0;
  return 1;
}
void or_navier_tensor_get(void* p, double* a0, double* c0) {
  auto& t = ((OrNavier*)p)->box.solver[3].tensor;
  std::memcpy(a0, t.a0.data(), sizeof(double) * t.a0.size());
  std::memcpy(c0, t.c0.data(), sizeof(double) * t.c0.size());
}
void or_navier_tensor_set(void* p, const double* lam, const double* fwd, const double* bwd) {
  ((OrNavier*)p)->box.solver[3].set_eig(lam, fwd, bwd);
}

// shape of the spectral array; returns 1 if complex
int or_navier_shape(void* p, int id, int* n0, int* n1, int* p0, int* p1) {
  auto* h = (OrNavier*)p;
  if (h->periodic) {
    auto* f = pick(h->per, id);
    *n0 = f->vhat.n0; *n1 = f->vhat.n1; *p0 = f->v.n0; *p1 = f->v.n1;
    return 1;
  }
  auto* f = pick(h->box, id);
  *n0 = f->vhat.n0; *n1 = f->vhat.n1; *p0 = f->v.n0; *p1 = f->v.n1;
  return 0;
}
void or_navier_get(void* p, int id, double* out) {
  auto* h = (OrNavier*)p;
  if (h->periodic) {
    auto* f = pick(h->per, id);
    std::memcpy(out, f->vhat.data(), sizeof(cplx) * f->vhat.size());
  } else {
    auto* f = pick(h->box, id);
    std::memcpy(out, f->vhat.data(), sizeof(double) * f->vhat.size());
  }
}
void or_navier_set(void* p, int id, const double* in) {
  auto* h = (OrNavier*)p;
  if (h->periodic) {
    auto* f = pick(h->per, id);
    std::memcpy(f->vhat.data(), in, sizeof(cplx) * f->vhat.size());
  } else {
    auto* f = pick(h->box, id);
    std::memcpy(f->vhat.data(), in, sizeof(double) * f->vhat.size());
  }
}
// physical values: backward() of the field (modifies the field's v only)
void or_navier_get_phys(void* p, int id, double* out) {
  auto* h = (OrNavier*)p;
  if (h->periodic) {
    auto* f = pick(h->per, id);
    f->backward();
    std::memcpy(out, f->v.data(), sizeof(double) * f->v.size());
  } else {
    auto* f = pick(h->box, id);
    f->backward();
    std::memcpy(out, f->v.data(), sizeof(double) * f->v.size());
  }
}
void or_navier_coords(void* p, int id, double* x, double* y) {
  auto* h = (OrNavier*)p;
  if (h->periodic) {
    auto* f = pick(h->per, id);
    std::memcpy(x, f->x[0].data(), sizeof(double) * f->x[0].size());
    std::memcpy(y, f->x[1].data(), sizeof(double) * f->x[1].size());
  } else {
    auto* f = pick(h->box, id);
    std::memcpy(x, f->x[0].data(), sizeof(double) * f->x[0].size());
    std::memcpy(y, f->x[1].data(), sizeof(double) * f->x[1].size());
  }
}
void or_navier_set_velocity(void* p, double amp, double m, double n) {
  auto* h = (OrNavier*)p;
  if (h->periodic) h->per.set_velocity(amp, m, n); else h->box.set_velocity(amp, m, n);
}
void or_navier_set_temperature(void* p, double amp, double m, double n) {
  auto* h = (OrNavier*)p;
  if (h->periodic) h->per.set_temperature(amp, m, n); else h->box.set_temperature(amp, m, n);
}
void or_navier_set_temperature_noise(void* p, double amp, uint64_t seed) {
  auto* h = (OrNavier*)p;
  if (h->periodic) h->per.set_temperature_noise(amp, seed); else h->box.set_temperature_noise(amp, seed);
}
void or_navier_zero_pressure(void* p) {
  auto* h = (OrNavier*)p;
  if (h->periodic) h->per.zero_pressure(); else h->box.zero_pressure();
}
int or_navier_update(void* p, int nsteps) {
  try {
    auto* h = (OrNavier*)p;
    for (int s = 0; s < nsteps; s++) {
      if (h->periodic) h->per.update(); else h->box.update();
    }
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}
// Independent cases advanced together: one case per thread at a time (the
// order given, dynamically scheduled), each case's own loops on that thread
// alone.  The way an ensemble of independent solves fills a many-core host.
int or_navier_update_many(void** hs, int n, int nsteps) {
  int bad = 0;
  std::string err;
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < n; i++) {
    try {
      auto* h = (OrNavier*)hs[i];
      for (int s = 0; s < nsteps; s++) {
        if (h->periodic) h->per.update(); else h->box.update();
      }
    } catch (std::exception& e) {
#pragma omp critical(or_update_many_err)
      {
        bad = 1;
        err = e.what();
      }
    }
  }
  if (bad) {
    g_err = err;
    return -1;
  }
  return 0;
}
// Navier2D::solid = Some([mask, value]) (navier.rs:189-190); mask == NULL clears it.
// mask, value: physical nx x ny arrays (value NULL = zeros)
void or_navier_set_solid(void* p, const double* mask, const double* value) {
  auto* h = (OrNavier*)p;
  auto set = [&](auto& n) {
    if (!mask) { n.has_solid = false; return; }
    int n0 = n.temp.v.n0, n1 = n.temp.v.n1;
    n.solid[0] = mk<double>(mask, n0, n1);
    n.solid[1] = Arr2<double>(n0, n1);
    if (value) n.solid[1] = mk<double>(value, n0, n1);
    n.has_solid = true;
  };
  if (h->periodic) set(h->per); else set(h->box);
}
double or_navier_time(void* p) {
  auto* h = (OrNavier*)p;
  return h->periodic ? h->per.time : h->box.time;
}
void or_navier_set_time(void* p, double t) {
  auto* h = (OrNavier*)p;
  if (h->periodic) h->per.time = t; else h->box.time = t;
}
// what: 0 Nu, 1 Nuvol, 2 Re, 3 KE, 4 |div|_2
double or_navier_eval(void* p, int what) {
  auto* h = (OrNavier*)p;
  if (h->periodic) {
    auto& n = h->per;
    switch (what) { case 0: return n.eval_nu(); case 1: return n.eval_nuvol(); case 2: return n.eval_re(); case 3: return n.eval_ke(); case 4: return n.div_norm(); }
  } else {
    auto& n = h->box;
    switch (what) { case 0: return n.eval_nu(); case 1: return n.eval_nuvol(); case 2: return n.eval_re(); case 3: return n.eval_ke(); case 4: return n.div_norm(); }
  }
  return NAN;
}
void or_navier_params(void* p, double* out) {  // nu, ka, ra, pr, dt, scale0, scale1
  auto* h = (OrNavier*)p;
  if (h->periodic) { auto& n = h->per; double v[7] = {n.nu, n.ka, n.ra, n.pr, n.dt, n.scale[0], n.scale[1]}; std::memcpy(out, v, sizeof v); }
  else { auto& n = h->box; double v[7] = {n.nu, n.ka, n.ra, n.pr, n.dt, n.scale[0], n.scale[1]}; std::memcpy(out, v, sizeof v); }
}

// ---- Navier2DAdjoint ----------------------------------------------------------
struct OrAdjoint {
  bool periodic;
  Navier2DAdjoint<double> box;
  Navier2DAdjoint<cplx> per;
};
void* or_adjoint_new(int nx, int ny, double ra, double pr, double dt, double aspect, int kind) {
  try {
    auto* h = new OrAdjoint();
    h->periodic = kind == 2;
    if (h->periodic) h->per.build(nx, ny, ra, pr, dt, aspect, kind);
    else h->box.build(nx, ny, ra, pr, dt, aspect, kind);
    return h;
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void or_adjoint_free(void* p) { delete (OrAdjoint*)p; }
// dense eigen-decompositions: k = 0 the inner Navier2D's Poisson, 1 the
// adjoint's Poisson, 2..4 the smoothers of ux, uy, temp
int or_adjoint_tensor_pending(void* p, int k, int* m) {
  auto* h = (OrAdjoint*)p;
  Solver2* s = h->periodic ? h->per.tensor_solver(k) : h->box.tensor_solver(k);
  if (!s->tensor.pending) return 0;
  *m = s->tensor.a0.n0;
  return 1;
}
void or_adjoint_tensor_get(void* p, int k, double* a0, double* c0) {
  auto* h = (OrAdjoint*)p;
  Solver2* s = h->periodic ? h->per.tensor_solver(k) : h->box.tensor_solver(k);
  std::memcpy(a0, s->tensor.a0.data(), 8 * s->tensor.a0.size());
  std::memcpy(c0, s->tensor.c0.data(), 8 * s->tensor.c0.size());
}
void or_adjoint_tensor_set(void* p, int k, const double* lam, const double* fwd, const double* bwd) {
  auto* h = (OrAdjoint*)p;
  Solver2* s = h->periodic ? h->per.tensor_solver(k) : h->box.tensor_solver(k);
  s->set_eig(lam, fwd, bwd);
}
}  // extern "C"
// field ids: 0 temp, 1 ux, 2 uy, 3 pres[0], 4 pres[1], 10 temp[1], 11 ux[1], 12 uy[1]
template <class T> static Field2<T>* adj_pick(Navier2DAdjoint<T>& a, int id) {
  switch (id) {
    case 0: return &a.temp[0];
    case 1: return &a.ux[0];
    case 2: return &a.uy[0];
    case 3: return &a.pres[0];
    case 4: return &a.pres[1];
    case 10: return &a.temp[1];
    case 11: return &a.ux[1];
    case 12: return &a.uy[1];
  }
  return nullptr;
}
extern "C" {
int or_adjoint_shape(void* p, int id, int* n0, int* n1) {
  auto* h = (OrAdjoint*)p;
  if (h->periodic) { auto* f = adj_pick(h->per, id); *n0 = f->vhat.n0; *n1 = f->vhat.n1; return 1; }
  auto* f = adj_pick(h->box, id); *n0 = f->vhat.n0; *n1 = f->vhat.n1; return 0;
}
void or_adjoint_get(void* p, int id, double* out) {
  auto* h = (OrAdjoint*)p;
  if (h->periodic) put(adj_pick(h->per, id)->vhat, out); else put(adj_pick(h->box, id)->vhat, out);
}
void or_adjoint_set(void* p, int id, const double* in) {
  auto* h = (OrAdjoint*)p;
  if (h->periodic) { auto* f = adj_pick(h->per, id); f->vhat = mk<cplx>(in, f->vhat.n0, f->vhat.n1); }
  else { auto* f = adj_pick(h->box, id); f->vhat = mk<double>(in, f->vhat.n0, f->vhat.n1); }
}
void or_adjoint_set_velocity(void* p, double amp, double m, double n) {  // navier_adjoint.rs:965-968
  auto* h = (OrAdjoint*)p;
  if (h->periodic) { Navier2D<cplx>::apply_mode(h->per.ux[0], amp, m, n, true); Navier2D<cplx>::apply_mode(h->per.uy[0], -amp, m, n, false); }
  else { Navier2D<double>::apply_mode(h->box.ux[0], amp, m, n, true); Navier2D<double>::apply_mode(h->box.uy[0], -amp, m, n, false); }
}
void or_adjoint_set_temperature(void* p, double amp, double m, double n) {  // :969-971
  auto* h = (OrAdjoint*)p;
  if (h->periodic) Navier2D<cplx>::apply_mode(h->per.temp[0], -amp, m, n, false);
  else Navier2D<double>::apply_mode(h->box.temp[0], -amp, m, n, false);
}
int or_adjoint_update(void* p, int nsteps) {
  try {
    auto* h = (OrAdjoint*)p;
    for (int s = 0; s < nsteps; s++) {
      if (h->periodic) h->per.update(); else h->box.update();
    }
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}
double or_adjoint_time(void* p) { auto* h = (OrAdjoint*)p; return h->periodic ? h->per.time : h->box.time; }
double or_adjoint_eval(void* p, int what) { auto* h = (OrAdjoint*)p; return h->periodic ? h->per.eval(what) : h->box.eval(what); }
int or_adjoint_exit(void* p) { auto* h = (OrAdjoint*)p; return h->periodic ? h->per.exit() : h->box.exit(); }
// |unsmoothed residual| (u, v, T) and |smoothed residual| (u, v, T) (navier_adjoint.rs:866-874)
void or_adjoint_residual(void* p, double* out) {
  auto* h = (OrAdjoint*)p;
  auto fill = [&](auto& a) {
    for (int k = 0; k < 3; k++) out[k] = a.unsmoothed[k].v.empty() ? 0.0 : a.norm_l2(a.unsmoothed[k]);
    out[3] = a.norm_l2(a.ux[1].vhat); out[4] = a.norm_l2(a.uy[1].vhat); out[5] = a.norm_l2(a.temp[1].vhat);
  };
  if (h->periodic) fill(h->per); else fill(h->box);
}

// ---- Space2 / Field2 primitives (funspace) ----------------------------------
struct OrSpace {
  bool cpx;
  Space2<double> r;
  Space2<cplx> c;
};
void* or_space_new(int k0, int n0, int k1, int n1) {
  auto* s = new OrSpace();
  s->cpx = k0 == FOURIER;
  if (s->cpx) s->c = Space2<cplx>(Base(k0, n0), Base(k1, n1));
  else s->r = Space2<double>(Base(k0, n0), Base(k1, n1));
  return s;
}
void or_space_free(void* p) { delete (OrSpace*)p; }
// sizes: [phys0, phys1, spec0, spec1, ortho0, ortho1]
int or_space_sizes(void* p, int* out) {
  auto* s = (OrSpace*)p;
  const Base& a = s->cpx ? s->c.b0 : s->r.b0;
  const Base& b = s->cpx ? s->c.b1 : s->r.b1;
  out[0] = a.n; out[1] = b.n; out[2] = a.m; out[3] = b.m; out[4] = a.len_ortho(); out[5] = b.len_ortho();
  return s->cpx ? 1 : 0;
}
void or_space_forward(void* p, const double* in, double* out) {
  auto* s = (OrSpace*)p;
  if (s->cpx) put(s->c.forward(mk<double>(in, s->c.phys0(), s->c.phys1())), out);
  else put(s->r.forward(mk<double>(in, s->r.phys0(), s->r.phys1())), out);
}
void or_space_backward(void* p, const double* in, double* out) {
  auto* s = (OrSpace*)p;
  if (s->cpx) put(s->c.backward(mk<cplx>(in, s->c.spec0(), s->c.spec1())), out);
  else put(s->r.backward(mk<double>(in, s->r.spec0(), s->r.spec1())), out);
}
void or_space_to_ortho(void* p, const double* in, double* out) {
  auto* s = (OrSpace*)p;
  if (s->cpx) put(s->c.to_ortho(mk<cplx>(in, s->c.spec0(), s->c.spec1())), out);
  else put(s->r.to_ortho(mk<double>(in, s->r.spec0(), s->r.spec1())), out);
}
void or_space_from_ortho(void* p, const double* in, double* out) {
  auto* s = (OrSpace*)p;
  if (s->cpx) put(s->c.from_ortho(mk<cplx>(in, s->c.b0.len_ortho(), s->c.b1.len_ortho())), out);
  else put(s->r.from_ortho(mk<double>(in, s->r.b0.len_ortho(), s->r.b1.len_ortho())), out);
}
// scale may be NULL (None)
void or_space_gradient(void* p, const double* in, double* out, int d0, int d1, const double* scale) {
  auto* s = (OrSpace*)p;
  if (s->cpx) put(s->c.gradient(mk<cplx>(in, s->c.spec0(), s->c.spec1()), d0, d1, scale), out);
  else put(s->r.gradient(mk<double>(in, s->r.spec0(), s->r.spec1()), d0, d1, scale), out);
}
// grid coordinates and deltas of a Field2 on this space
void or_space_coords(void* p, double* x0, double* x1, double* dx0, double* dx1) {
  auto* s = (OrSpace*)p;
  if (s->cpx) {
    Field2<cplx> f(s->c);
    std::memcpy(x0, f.x[0].data(), 8 * f.x[0].size()); std::memcpy(x1, f.x[1].data(), 8 * f.x[1].size());
    std::memcpy(dx0, f.dx[0].data(), 8 * f.dx[0].size()); std::memcpy(dx1, f.dx[1].data(), 8 * f.dx[1].size());
  } else {
    Field2<double> f(s->r);
    std::memcpy(x0, f.x[0].data(), 8 * f.x[0].size()); std::memcpy(x1, f.x[1].data(), 8 * f.x[1].size());
    std::memcpy(dx0, f.dx[0].data(), 8 * f.dx[0].size()); std::memcpy(dx1, f.dx[1].data(), 8 * f.dx[1].size());
  }
}
// Field2::average_axis / average on physical values v
void or_space_average_axis(void* p, const double* v, int axis, double* out) {
  auto* s = (OrSpace*)p;
  if (s->cpx) { Field2<cplx> f(s->c); f.v = mk<double>(v, f.v.n0, f.v.n1); auto r = f.average_axis(axis); std::memcpy(out, r.data(), 8 * r.size()); }
  else { Field2<double> f(s->r); f.v = mk<double>(v, f.v.n0, f.v.n1); auto r = f.average_axis(axis); std::memcpy(out, r.data(), 8 * r.size()); }
}
double or_space_average(void* p, const double* v) {
  auto* s = (OrSpace*)p;
  if (s->cpx) { Field2<cplx> f(s->c); f.v = mk<double>(v, f.v.n0, f.v.n1); return f.average(); }
  Field2<double> f(s->r); f.v = mk<double>(v, f.v.n0, f.v.n1); return f.average();
}

// ---- 1-D lane primitives (for the reference's 1-D known-answer tests) -------
void or_base_forward(int kind, int n, const double* in, double* out) {
  Base b(kind, n);
  if (b.fourier()) { rfft(in, (cplx*)out, n); return; }
  std::vector<double> o(n);
  b.cheb_forward(in, o.data());
  b.from_ortho(o.data(), out);
}
void or_base_backward(int kind, int n, const double* in, double* out) {
  Base b(kind, n);
  if (b.fourier()) { irfft((const cplx*)in, out, n); return; }
  std::vector<double> o(n);
  b.to_ortho(in, o.data());
  b.cheb_backward(o.data(), out);
}
void or_base_to_ortho(int kind, int n, const double* in, double* out) { Base b(kind, n); b.to_ortho(in, out); }
void or_base_from_ortho(int kind, int n, const double* in, double* out) { Base b(kind, n); b.from_ortho(in, out); }
// composite differentiate: to_ortho then ortho recurrence (output ortho-sized)
void or_base_differentiate(int kind, int n, const double* in, double* out, int times) {
  Base b(kind, n);
  if (b.fourier()) {
    const cplx* ci = (const cplx*)in;
    cplx* co = (cplx*)out;
    for (int i = 0; i < b.m; i++) co[i] = ci[i];
    b.diff_ortho(co, times);
    return;
  }
  b.to_ortho(in, out);
  b.diff_ortho(out, times);
}
void or_base_coords(int kind, int n, double* x) { Base b(kind, n); std::memcpy(x, b.x.data(), 8 * b.x.size()); }
// dense matrices: which 0 mass, 1 laplace, 2 laplace_inv, 3 laplace_inv_eye; returns rows/cols
void or_base_matrix(int kind, int n, int which, double* out, int* rows, int* cols) {
  Base b(kind, n);
  Mat m = which == 0 ? b.mass() : which == 1 ? b.laplace() : which == 2 ? b.laplace_inv() : b.laplace_inv_eye();
  *rows = m.n0; *cols = m.n1;
  if (out) std::memcpy(out, m.data(), 8 * m.size());
}

// ---- banded solvers ----------------------------------------------------------
// Fdma::from_matrix + solve on one lane (fdma.rs)
void or_fdma_solve(const double* mat, int n, const double* b, double* x) {
  Mat a(n, n);
  std::memcpy(a.data(), mat, 8 * (size_t)n * n);
  Fdma f = Fdma::from_matrix(a);
  for (int i = 0; i < n; i++) x[i] = b[i];
  f.solve_lane(x);
}
void or_fdma_solve_c(const double* mat, int n, const double* b, double* x) {
  Mat a(n, n);
  std::memcpy(a.data(), mat, 8 * (size_t)n * n);
  Fdma f = Fdma::from_matrix(a);
  cplx* xc = (cplx*)x;
  for (int i = 0; i < n; i++) xc[i] = ((const cplx*)b)[i];
  f.solve_lane(xc);
}
// MatVecFdma::new(mat (m x n)).solve(data (rows x cols), axis)
void or_matvec_fdma(const double* mat, int m, int n, const double* in, int r, int c, int axis, double* out) {
  Mat a(m, n);
  std::memcpy(a.data(), mat, 8 * (size_t)m * n);
  MatVecFdma mv(a);
  Arr2<double> x = mk<double>(in, r, c);
  put(mv.solve(x, axis), out);
}

// 1-D solver known-answer tests: kind = S_HHOLTZ / S_HHOLTZ_ADI / S_POISSON
void or_solver1d(int basekind, int n, int kind, double c, const double* in, double* out) {
  Base b(basekind, n);
  Solver1 s;
  s.build(b, kind, c);
  s.solve(in, out);
}

// Many lanes of one Chebyshev-family basis (row-major lanes x length), the
// 1-D axis operations of Space2 (ortho.rs:235-312, composite.rs:156-238) and
// HholtzAdi::solve along one axis (hholtz_adi.rs:92-131): op 0 forward
// (n -> m), 1 backward (m -> n), 2 to_ortho (m -> n), 3 from_ortho (n -> m),
// 4 Helmholtz solve with coefficient c (n -> m).  One basis and one solver
// serve every lane; lanes run in parallel (OpenMP), as the reference's rayon
// par_for_each over lanes.
int or_lanes_apply(int kind, int n, int op, int lanes, double c, const double* in, double* out) {
  try {
    Base b(kind, n);
    if (b.fourier()) throw std::runtime_error("or_lanes_apply: Chebyshev-family bases only");
    const int m = b.m;
    const int il = (op == 0 || op == 3 || op == 4) ? n : m;
    const int ol = (op == 0 || op == 3 || op == 4) ? m : n;
    Solver1 s;
    if (op == 4) s.build(b, S_HHOLTZ_ADI, c);
#pragma omp parallel for schedule(static)
    for (int l = 0; l < lanes; l++) {
      const double* x = in + (size_t)l * il;
      double* y = out + (size_t)l * ol;
      std::vector<double> o(n);
      switch (op) {
        case 0: b.cheb_forward(x, o.data()); b.from_ortho(o.data(), y); break;
        case 1: b.to_ortho(x, o.data()); b.cheb_backward(o.data(), y); break;
        case 2: b.to_ortho(x, y); break;
        case 3: b.from_ortho(x, y); break;
        default: s.solve(x, y); break;
      }
    }
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// 2-D field solvers (Hholtz / HholtzAdi / Poisson) on a space
struct OrSolver {
  OrSpace* sp;
  Solver2 s;
};
void* or_solver_new(void* space, int kind, double c0, double c1) {
  try {
    auto* sp = (OrSpace*)space;
    auto* o = new OrSolver();
    o->sp = sp;
    double c[2] = {c0, c1};
    if (sp->cpx) o->s.build(sp->c, kind, c);
    else o->s.build(sp->r, kind, c);
    return o;
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void or_solver_free(void* p) { delete (OrSolver*)p; }
int or_solver_tensor_pending(void* p, int* m) {
  auto& t = ((OrSolver*)p)->s.tensor;
  if (!t.pending) return 0;
  *m = t.a0.n0;
  return 1;
}
void or_solver_tensor_get(void* p, double* a0, double* c0) {
  auto& t = ((OrSolver*)p)->s.tensor;
  std::memcpy(a0, t.a0.data(), 8 * t.a0.size());
  std::memcpy(c0, t.c0.data(), 8 * t.c0.size());
}
void or_solver_tensor_set(void* p, const double* lam, const double* fwd, const double* bwd) {
  ((OrSolver*)p)->s.set_eig(lam, fwd, bwd);
}
// solve: input is ortho-sized (rows x cols), output spectral-sized
int or_solver_solve(void* p, const double* in, int r, int c, double* out) {
  try {
    auto* o = (OrSolver*)p;
    if (o->sp->cpx) put(o->s.solve(mk<cplx>(in, r, c)), out);
    else put(o->s.solve(mk<double>(in, r, c)), out);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}
// FdmaTensor with user matrices (fdma_tensor.rs test_tensor2d): a, c are n x n,
// the same pair is used on both axes; eigen-decomposition supplied externally.
struct OrTensor { FdmaTensor2 t; };
void* or_tensor_new(const double* a, const double* c, int n, double alpha) {
  Mat A(n, n), C(n, n);
  std::memcpy(A.data(), a, 8 * (size_t)n * n);
  std::memcpy(C.data(), c, 8 * (size_t)n * n);
  auto* o = new OrTensor();
  o->t.init(A, A, C, C, false, alpha);
  return o;
}
void or_tensor_set(void* p, const double* lam, const double* fwd, const double* bwd) {
  auto& t = ((OrTensor*)p)->t;
  int m = t.a0.n0;
  t.lam.assign(lam, lam + m);
  t.fwd = Mat(m, m); t.bwd = Mat(m, m);
  std::memcpy(t.fwd.data(), fwd, 8 * (size_t)m * m);
  std::memcpy(t.bwd.data(), bwd, 8 * (size_t)m * m);
  t.pending = false;
}
void or_tensor_solve(void* p, const double* in, double* out) {
  auto& t = ((OrTensor*)p)->t;
  put(t.solve(mk<double>(in, (int)t.lam.size(), t.n)), out);
}
void or_tensor_free(void* p) { delete (OrTensor*)p; }

}  // extern "C"
