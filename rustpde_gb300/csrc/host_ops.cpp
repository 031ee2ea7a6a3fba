// host_ops.cpp -- set-up arithmetic (see host_ops.h).  Compiled with
// -ffp-contract=off so that operator coefficients are formed with the same
// roundings as the reference's (non-fused) products.
#include "host_ops.h"

#include <map>
#include <mutex>

#include <algorithm>
#include <cmath>
#include <numeric>

namespace rbc {

static const long double PI_L = 3.141592653589793238462643383279502884L;

uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

HostBasis make_basis(int kind, int n) {
  HostBasis b;
  b.kind = kind;
  b.n = n;
  if (kind == FOURIER) {
    // r2c.rs:45-70, c2c.rs:63-66 (nodes 0, 2pi/n, ...)
    b.m = n / 2 + 1;
    b.x.resize(n);
    double step = 2.0 * 3.14159265358979323846 / (double)n;
    for (int i = 0; i < n; i++) b.x[i] = 0.0 + step * (double)i;
    return b;
  }
  // ortho.rs:71-80 Gauss-Lobatto nodes
  b.x.resize(n);
  double mm = (double)(n - 1);
  for (int k = 0; k < n; k++) b.x[k] = -std::sin(3.14159265358979323846 * (mm - 2.0 * (double)k) / (2.0 * mm));
  if (kind == CHEB) {
    b.m = n;
    return b;
  }
  if (kind == CD || kind == CN) {
    // composite_stencil.rs:117-171
    int m = n - 2;
    b.m = m;
    b.diag.assign(m, 1.0);
    b.low2.assign(m, 0.0);
    for (int k = 0; k < m; k++) {
      if (kind == CD) b.low2[k] = -1.0;
      else b.low2[k] = -1.0 * (double)(k * k) / (double)((k + 2) * (k + 2));
    }
    std::vector<double> main_(m);
    b.fo_off.assign(std::max(m - 2, 0), 0.0);
    for (int i = 0; i < m; i++) main_[i] = b.diag[i] * b.diag[i] + b.low2[i] * b.low2[i];
    for (int i = 0; i < m - 2; i++) b.fo_off[i] = b.diag[i + 2] * b.low2[i];
    // linalg.rs:14-57: the sweep ratios and denominators depend on the basis only
    const std::vector<double>& a = b.fo_off;
    const std::vector<double>& c = b.fo_off;
    b.fo_w.assign(std::max(m - 2, 0), 0.0);
    b.fo_dinv.assign(m, 0.0);
    std::vector<double>& w = b.fo_w;
    w[0] = c[0] / main_[0];
    if (c.size() > 1) w[1] = c[1] / main_[1];
    for (int i = 2; i < m - 2; i++) w[i] = c[i] / (main_[i] - a[i - 2] * w[i - 2]);
    b.fo_dinv[0] = 1.0 / main_[0];
    b.fo_dinv[1] = 1.0 / main_[1];
    for (int i = 2; i < m; i++) b.fo_dinv[i] = 1.0 / (main_[i] - a[i - 2] * w[i - 2]);
    return b;
  }
  // boundary bases composite_stencil.rs:300-330, solve_vec at :382-406
  b.m = 2;
  if (kind == CDBC) {
    b.t0[0] = 0.5; b.t0[1] = 0.5; b.t1[0] = -0.5; b.t1[1] = 0.5;
  } else {
    b.t0[0] = 0.5; b.t0[1] = 0.5; b.t1[0] = -(1.0 / 8.0); b.t1[1] = 1.0 / 8.0;
  }
  double a = b.t0[0] * b.t0[0] + b.t1[0] * b.t1[0];
  double bb = b.t0[0] * b.t0[1] + b.t1[0] * b.t1[1];
  double c = b.t0[1] * b.t0[0] + b.t1[1] * b.t1[0];
  double d = b.t0[1] * b.t0[1] + b.t1[1] * b.t1[1];
  double det = 1.0 / (a * d - bb * c);
  // comp0 = (c0 d - c1 b) det ; comp1 = (c1 a - c0 c) det
  b.bc_inv[0] = d * det; b.bc_inv[1] = -bb * det;
  b.bc_inv[2] = -c * det; b.bc_inv[3] = a * det;
  return b;
}

Band4 band_combine(const Band4& a, const Band4& b, double l) {
  Band4 f;
  f.n = a.n;
  f.low.resize(a.low.size()); f.dia.resize(a.dia.size()); f.up1.resize(a.up1.size()); f.up2.resize(a.up2.size());
  for (size_t i = 0; i < a.low.size(); i++) f.low[i] = a.low[i] + b.low[i] * l;
  for (size_t i = 0; i < a.dia.size(); i++) f.dia[i] = a.dia[i] + b.dia[i] * l;
  for (size_t i = 0; i < a.up1.size(); i++) f.up1[i] = a.up1[i] + b.up1[i] * l;
  for (size_t i = 0; i < a.up2.size(); i++) f.up2[i] = a.up2[i] + b.up2[i] * l;
  return f;
}

void band_sweep(Band4& f) {
  int n = f.n;
  for (int i = 2; i < n; i++) {
    f.low[i - 2] /= f.dia[i - 2];
    f.dia[i] -= f.low[i - 2] * f.up1[i - 2];
    if (i < n - 2) f.up1[i] -= f.low[i - 2] * f.up2[i - 2];
  }
}

std::vector<double> band_dense(const Band4& b) {
  int n = b.n;
  std::vector<double> d((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) d[(size_t)i * n + i] = b.dia[i];
  for (int i = 0; i + 2 < n; i++) d[(size_t)(i + 2) * n + i] = b.low[i];
  for (int i = 0; i + 2 < n; i++) d[(size_t)i * n + i + 2] = b.up1[i];
  for (int i = 0; i + 4 < n; i++) d[(size_t)i * n + i + 4] = b.up2[i];
  return d;
}

// Entries of peye*laplace_inv for ortho length n (ortho.rs:147-180): row r of
// the result is row r+2 of _pinv(n, 2).
static double pinv_entry(int n, int r, int col) {
  int i = r + 2;
  if (i == 2 && col == 0) return 0.25;
  if (col == i - 2 && i >= 3 && i < n) return 1.0 / (double)(4 * i * (i - 1));
  if (col == i && i >= 2 && i < n - 2) return -1.0 / (double)(2 * (i * i - 1));
  if (col == i + 2 && i >= 2 && i < n - 4) return 1.0 / (double)(4 * i * (i + 1));
  return 0.0;
}

Pinv make_pinv(int n) {
  Pinv p;
  p.n = n;
  int m = n - 2;
  p.dia.assign(m, 0.0); p.up1.assign(m, 0.0); p.up2.assign(m, 0.0);
  for (int i = 0; i < m; i++) {
    p.dia[i] = pinv_entry(n, i, i);
    if (i < m - 2) p.up1[i] = pinv_entry(n, i, i + 2);
    if (i < m - 4) p.up2[i] = pinv_entry(n, i, i + 4);
  }
  return p;
}

void hholtz_ingredients(const HostBasis& b, Band4& A, Band4& B) {
  // A = pinv*S, B = peye*S for a composite (Dirichlet/Neumann) basis; the
  // products sum k = j then k = j+2, the order of a dense row-by-column product.
  int n = b.n, m = b.m;
  auto S = [&](int k, int j) -> double {
    if (k == j) return b.diag[j];
    if (k == j + 2) return b.low2[j];
    return 0.0;
  };
  auto Aent = [&](int i, int j) -> double {
    double s = 0.0;
    bool first = true;
    for (int k : {j, j + 2}) {
      if (k < 0 || k >= n) continue;
      double p = pinv_entry(n, i, k);
      if (p == 0.0) continue;
      double t = p * S(k, j);
      s = first ? t : s + t;
      first = false;
    }
    return s;
  };
  auto Bent = [&](int i, int j) -> double { return S(i + 2, j); };
  A.n = B.n = m;
  A.low.assign(m - 2, 0.0); A.dia.assign(m, 0.0); A.up1.assign(m - 2, 0.0); A.up2.assign(std::max(m - 4, 0), 0.0);
  B.low.assign(m - 2, 0.0); B.dia.assign(m, 0.0); B.up1.assign(m - 2, 0.0); B.up2.assign(std::max(m - 4, 0), 0.0);
  for (int i = 0; i < m; i++) {
    A.dia[i] = Aent(i, i);
    B.dia[i] = Bent(i, i);
  }
  for (int i = 0; i + 2 < m; i++) {
    A.low[i] = Aent(i + 2, i); A.up1[i] = Aent(i, i + 2);
    B.low[i] = Bent(i + 2, i); B.up1[i] = Bent(i, i + 2);
  }
  for (int i = 0; i + 4 < m; i++) {
    A.up2[i] = Aent(i, i + 4);
    B.up2[i] = Bent(i, i + 4);
  }
}

std::vector<double> matmul(int n, int k, int m, const std::vector<double>& A, const std::vector<double>& B) {
  std::vector<double> C((size_t)n * m, 0.0);
  for (int i = 0; i < n; i++)
    for (int l = 0; l < k; l++) {
      double a = A[(size_t)i * k + l];
      if (a == 0.0) continue;
      const double* br = &B[(size_t)l * m];
      double* cr = &C[(size_t)i * m];
      for (int j = 0; j < m; j++) cr[j] += a * br[j];
    }
  return C;
}

bool invert(int n, const std::vector<double>& A, std::vector<double>& Ainv) {
  // Gauss-Jordan with partial pivoting
  std::vector<double> a(A);
  Ainv.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) Ainv[(size_t)i * n + i] = 1.0;
  for (int c = 0; c < n; c++) {
    int p = c;
    double best = std::fabs(a[(size_t)c * n + c]);
    for (int r = c + 1; r < n; r++) {
      double v = std::fabs(a[(size_t)r * n + c]);
      if (v > best) { best = v; p = r; }
    }
    if (best == 0.0) return false;
    if (p != c) {
      for (int j = 0; j < n; j++) {
        std::swap(a[(size_t)p * n + j], a[(size_t)c * n + j]);
        std::swap(Ainv[(size_t)p * n + j], Ainv[(size_t)c * n + j]);
      }
    }
    double inv = 1.0 / a[(size_t)c * n + c];
    for (int j = 0; j < n; j++) { a[(size_t)c * n + j] *= inv; Ainv[(size_t)c * n + j] *= inv; }
    for (int r = 0; r < n; r++) {
      if (r == c) continue;
      double f = a[(size_t)r * n + c];
      if (f == 0.0) continue;
      for (int j = 0; j < n; j++) {
        a[(size_t)r * n + j] -= f * a[(size_t)c * n + j];
        Ainv[(size_t)r * n + j] -= f * Ainv[(size_t)c * n + j];
      }
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// Real eigen-decomposition: Householder Hessenberg reduction, Francis
// double-shift QR to real Schur form (Golub & Van Loan, Alg. 7.4.2, 7.5.1-2),
// eigenvectors by back-substitution on the triangular factor.
// ---------------------------------------------------------------------------
namespace {
struct MatRM {
  int n;
  std::vector<double> a;
  double& operator()(int i, int j) { return a[(size_t)i * n + j]; }
};

// Householder vector: v[0] = 1, (I - beta v v^T) x = mu e_1
void house(const double* x, int len, double* v, double& beta) {
  double sigma = 0.0;
  for (int i = 1; i < len; i++) sigma += x[i] * x[i];
  v[0] = 1.0;
  for (int i = 1; i < len; i++) v[i] = x[i];
  if (sigma == 0.0) { beta = 0.0; return; }
  double mu = std::sqrt(x[0] * x[0] + sigma);
  double v0 = x[0] <= 0.0 ? x[0] - mu : -sigma / (x[0] + mu);
  beta = 2.0 * v0 * v0 / (sigma + v0 * v0);
  for (int i = 1; i < len; i++) v[i] /= v0;
}

void apply_left(MatRM& H, int r0, int len, const double* v, double beta, int c0, int c1) {
  if (beta == 0.0) return;
  for (int j = c0; j <= c1; j++) {
    double s = 0.0;
    for (int k = 0; k < len; k++) s += v[k] * H(r0 + k, j);
    s *= beta;
    for (int k = 0; k < len; k++) H(r0 + k, j) -= s * v[k];
  }
}
void apply_right(MatRM& H, int c0, int len, const double* v, double beta, int r0, int r1) {
  if (beta == 0.0) return;
  for (int i = r0; i <= r1; i++) {
    double s = 0.0;
    for (int k = 0; k < len; k++) s += H(i, c0 + k) * v[k];
    s *= beta;
    for (int k = 0; k < len; k++) H(i, c0 + k) -= s * v[k];
  }
}
}  // namespace

bool eig_real(int n, const std::vector<double>& A, std::vector<double>& lam, std::vector<double>& V,
              std::string* err) {
  MatRM H{n, A};
  MatRM Z{n, std::vector<double>((size_t)n * n, 0.0)};
  for (int i = 0; i < n; i++) Z(i, i) = 1.0;
  std::vector<double> x(n), v(n);
  // Hessenberg reduction
  for (int k = 0; k < n - 2; k++) {
    int len = n - k - 1;
    for (int i = 0; i < len; i++) x[i] = H(k + 1 + i, k);
    double beta;
    house(x.data(), len, v.data(), beta);
    apply_left(H, k + 1, len, v.data(), beta, 0, n - 1);
    apply_right(H, k + 1, len, v.data(), beta, 0, n - 1);
    apply_right(Z, k + 1, len, v.data(), beta, 0, n - 1);
    for (int i = k + 2; i < n; i++) H(i, k) = 0.0;
  }
  double anorm = 0.0;
  for (double e : H.a) anorm = std::max(anorm, std::fabs(e));
  const double eps = 2.220446049250313e-16;
  int hi = n - 1;
  int iter = 0, total = 0;
  while (hi >= 0) {
    int l = hi;
    while (l > 0) {
      double s = std::fabs(H(l - 1, l - 1)) + std::fabs(H(l, l));
      if (s == 0.0) s = anorm;
      if (std::fabs(H(l, l - 1)) <= eps * s) break;
      l--;
    }
    if (l > 0) H(l, l - 1) = 0.0;
    if (l == hi) { hi--; iter = 0; continue; }
    if (l == hi - 1) {
      // 2x2 block: reduce to upper triangular when the eigenvalues are real
      double a = H(hi - 1, hi - 1), b = H(hi - 1, hi), c = H(hi, hi - 1), d = H(hi, hi);
      double p = 0.5 * (a - d);
      double disc = p * p + b * c;
      if (disc < 0.0) {
        if (err) *err = "eig_real: complex eigenvalue pair";
        return false;
      }
      double sq = std::sqrt(disc);
      double l1 = d + (p >= 0 ? p + sq : p - sq);  // eigenvalue placed at (hi-1, hi-1)
      // eigenvector of [[a,b],[c,d]] for l1
      double e0, e1;
      if (std::fabs(b) + std::fabs(l1 - a) >= std::fabs(l1 - d) + std::fabs(c)) { e0 = b; e1 = l1 - a; }
      else { e0 = l1 - d; e1 = c; }
      double nr = std::hypot(e0, e1);
      double cs = e0 / nr, sn = e1 / nr;
      // G = [[cs, -sn], [sn, cs]]: H <- G^T H G on rows/cols (hi-1, hi)
      for (int j = hi - 1; j < n; j++) {
        double h0 = H(hi - 1, j), h1 = H(hi, j);
        H(hi - 1, j) = cs * h0 + sn * h1;
        H(hi, j) = -sn * h0 + cs * h1;
      }
      for (int i = 0; i <= hi; i++) {
        double h0 = H(i, hi - 1), h1 = H(i, hi);
        H(i, hi - 1) = cs * h0 + sn * h1;
        H(i, hi) = -sn * h0 + cs * h1;
      }
      for (int i = 0; i < n; i++) {
        double z0 = Z(i, hi - 1), z1 = Z(i, hi);
        Z(i, hi - 1) = cs * z0 + sn * z1;
        Z(i, hi) = -sn * z0 + cs * z1;
      }
      H(hi, hi - 1) = 0.0;
      hi -= 2;
      iter = 0;
      continue;
    }
    if (++iter > 60 || ++total > 60 * n) {
      if (err) *err = "eig_real: QR iteration did not converge";
      return false;
    }
    // Francis double shift on the active block l..hi
    double s, t;
    if (iter == 10 || iter == 20) {  // exceptional shift
      double w = std::fabs(H(hi, hi - 1)) + std::fabs(H(hi - 1, hi - 2));
      s = 1.5 * w + H(hi, hi);
      t = w * w;
    } else {
      s = H(hi - 1, hi - 1) + H(hi, hi);
      t = H(hi - 1, hi - 1) * H(hi, hi) - H(hi - 1, hi) * H(hi, hi - 1);
    }
    double xx = H(l, l) * H(l, l) + H(l, l + 1) * H(l + 1, l) - s * H(l, l) + t;
    double yy = H(l + 1, l) * (H(l, l) + H(l + 1, l + 1) - s);
    double zz = H(l + 1, l) * H(l + 2, l + 1);
    double vv[3], beta;
    for (int p = l; p <= hi - 2; p++) {
      double xv[3] = {xx, yy, zz};
      house(xv, 3, vv, beta);
      int q = std::max(l, p - 1);
      apply_left(H, p, 3, vv, beta, q, n - 1);
      int r = std::min(p + 3, hi);
      apply_right(H, p, 3, vv, beta, 0, r);
      apply_right(Z, p, 3, vv, beta, 0, n - 1);
      xx = H(p + 1, p);
      yy = H(p + 2, p);
      if (p < hi - 2) zz = H(p + 3, p);
    }
    double xv[2] = {xx, yy};
    house(xv, 2, vv, beta);
    apply_left(H, hi - 1, 2, vv, beta, hi - 2, n - 1);
    apply_right(H, hi - 1, 2, vv, beta, 0, hi);
    apply_right(Z, hi - 1, 2, vv, beta, 0, n - 1);
  }
  // eigenvectors of the upper triangular T = H
  std::vector<double> Y((size_t)n * n, 0.0);
  double small = eps * anorm;
  for (int k = 0; k < n; k++) {
    double lk = H(k, k);
    Y[(size_t)k * n + k] = 1.0;
    for (int i = k - 1; i >= 0; i--) {
      double s2 = 0.0;
      for (int j = i + 1; j <= k; j++) s2 += H(i, j) * Y[(size_t)j * n + k];
      double den = H(i, i) - lk;
      if (std::fabs(den) < small) den = den >= 0 ? small : -small;
      Y[(size_t)i * n + k] = -s2 / den;
    }
  }
  std::vector<double> Vu = matmul(n, n, n, Z.a, Y);
  // normalise columns, sort descending (stable argsort, reversed)
  std::vector<double> ev(n);
  for (int k = 0; k < n; k++) ev[k] = H(k, k);
  std::vector<int> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return ev[a] < ev[b]; });
  std::reverse(perm.begin(), perm.end());
  lam.resize(n);
  V.assign((size_t)n * n, 0.0);
  for (int c = 0; c < n; c++) {
    int k = perm[c];
    lam[c] = ev[k];
    double nrm = 0.0;
    for (int i = 0; i < n; i++) nrm += Vu[(size_t)i * n + k] * Vu[(size_t)i * n + k];
    nrm = std::sqrt(nrm);
    for (int i = 0; i < n; i++) V[(size_t)i * n + c] = Vu[(size_t)i * n + k] / nrm;
  }
  return true;
}

std::vector<double> twiddles(int L) {
  std::vector<double> t(2 * (size_t)L);
  for (int k = 0; k < L; k++) {
    long double ang = 2.0L * PI_L * (long double)k / (long double)L;
    t[2 * k] = (double)cosl(ang);
    t[2 * k + 1] = (double)(-sinl(ang));
  }
  return t;
}

// cos(pi * j * k / N) evaluated from the reduced integer angle
static double cospi_frac(long jk, int N) {
  long t = jk % (2L * N);
  return (double)cosl(PI_L * (long double)t / (long double)N);
}

static std::vector<double> cheb_dense_forward_impl(int n);
static std::vector<double> cheb_dense_backward_impl(int n);

// The dense transform matrices depend on n only: computed once per size.
static std::vector<double> cheb_dense_cached(int n, bool fwd) {
  static std::mutex mu;
  static std::map<std::pair<int, bool>, std::vector<double>> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(n, fwd);
  auto it = cache.find(key);
  if (it == cache.end()) it = cache.emplace(key, fwd ? cheb_dense_forward_impl(n) : cheb_dense_backward_impl(n)).first;
  return it->second;
}
std::vector<double> cheb_dense_forward(int n) { return cheb_dense_cached(n, true); }
std::vector<double> cheb_dense_backward(int n) { return cheb_dense_cached(n, false); }

static std::vector<double> cheb_dense_forward_impl(int n) {
  int N = n - 1;
  std::vector<double> M((size_t)n * n);
  for (int k = 0; k < n; k++) {
    double sk = ((k % 2) ? -1.0 : 1.0) * (1.0 / (double)(n - 1));
    if (k == 0 || k == N) sk *= 0.5;
    for (int j = 0; j < n; j++) {
      double wj = (j == 0 || j == N) ? 1.0 : 2.0;
      M[(size_t)k * n + j] = sk * wj * cospi_frac((long)j * k, N);
    }
  }
  return M;
}

static std::vector<double> cheb_dense_backward_impl(int n) {
  int N = n - 1;
  std::vector<double> M((size_t)n * n);
  for (int j = 0; j < n; j++)
    for (int k = 0; k < n; k++) {
      double s = ((k % 2) ? -1.0 : 1.0) / 2.0;
      if (k == 0 || k == N) s *= 2.0;
      double wk = (k == 0 || k == N) ? 1.0 : 2.0;
      M[(size_t)j * n + k] = wk * s * cospi_frac((long)j * k, N);
    }
  return M;
}

}  // namespace rbc
