// dense_ops.cpp -- see dense_ops.h.
#include "dense_ops.h"

#include <cmath>
#include <stdexcept>

namespace rbc {

static const long double kPiL = 3.141592653589793238462643383279502884L;

LMat lm_identity(int n) {
  LMat I(n, n);
  for (int i = 0; i < n; i++) I.at(i, i) = 1.0L;
  return I;
}

LMat lm_mul(const LMat& A, const LMat& B) {
  if (A.cols != B.rows) throw std::runtime_error("lm_mul: shape mismatch");
  LMat C(A.rows, B.cols);
  for (int i = 0; i < A.rows; i++)
    for (int k = 0; k < A.cols; k++) {
      const long double a = A.at(i, k);
      if (a == 0.0L) continue;
      const long double* b = &B.a[(size_t)k * B.cols];
      long double* c = &C.a[(size_t)i * C.cols];
      for (int j = 0; j < B.cols; j++) c[j] += a * b[j];
    }
  return C;
}

LMat lm_scale(const LMat& A, long double s) {
  LMat C = A;
  for (auto& v : C.a) v *= s;
  return C;
}

LMat lm_rows(const LMat& A, int r0, int r1) {
  LMat C(r1 - r0, A.cols);
  for (int i = r0; i < r1; i++)
    for (int j = 0; j < A.cols; j++) C.at(i - r0, j) = A.at(i, j);
  return C;
}

LMat lm_vstack(const LMat& A, const LMat& B) {
  if (A.cols != B.cols) throw std::runtime_error("lm_vstack: shape mismatch");
  LMat C(A.rows + B.rows, A.cols);
  for (size_t i = 0; i < A.a.size(); i++) C.a[i] = A.a[i];
  for (size_t i = 0; i < B.a.size(); i++) C.a[A.a.size() + i] = B.a[i];
  return C;
}

std::vector<double> lm_to_double(const LMat& A) {
  std::vector<double> d(A.a.size());
  for (size_t i = 0; i < d.size(); i++) d[i] = (double)A.a[i];
  return d;
}

static long double cospi_l(long jk, int N) {
  const long t = jk % (2L * N);
  return cosl(kPiL * (long double)t / (long double)N);
}

LMat lm_cheb_forward(int n) {
  const int N = n - 1;
  LMat F(n, n);
  for (int k = 0; k < n; k++) {
    long double sk = ((k & 1) ? -1.0L : 1.0L) / (long double)N;
    if (k == 0 || k == N) sk *= 0.5L;
    for (int j = 0; j < n; j++) {
      const long double wj = (j == 0 || j == N) ? 1.0L : 2.0L;
      F.at(k, j) = sk * wj * cospi_l((long)j * k, N);
    }
  }
  return F;
}

LMat lm_cheb_backward(int n) {
  const int N = n - 1;
  LMat B(n, n);
  for (int j = 0; j < n; j++)
    for (int k = 0; k < n; k++) {
      long double s = ((k & 1) ? -0.5L : 0.5L);
      if (k == 0 || k == N) s *= 2.0L;
      const long double wk = (k == 0 || k == N) ? 1.0L : 2.0L;
      B.at(j, k) = wk * s * cospi_l((long)j * k, N);
    }
  return B;
}

LMat lm_cheb_diff(int n) {
  // d_0 = sum_{j odd} j a_j ;  d_k = sum_{j > k, j - k odd} 2 j a_j
  LMat D(n, n);
  for (int k = 0; k < n; k++)
    for (int j = k + 1; j < n; j += 2) D.at(k, j) = (k == 0 ? 1.0L : 2.0L) * (long double)j;
  return D;
}

LMat lm_stencil(const HostBasis& b) {
  const int no = b.ortho_len(), m = b.m;
  if (!b.composite()) return lm_identity(no);
  LMat S(no, m);
  if (b.bc()) {
    S.at(0, 0) = b.t0[0]; S.at(0, 1) = b.t0[1];
    S.at(1, 0) = b.t1[0]; S.at(1, 1) = b.t1[1];
    return S;
  }
  for (int j = 0; j < m; j++) {
    S.at(j, j) = b.diag[j];
    S.at(j + 2, j) = b.low2[j];
  }
  return S;
}

LMat lm_from_ortho(const HostBasis& b) {
  const int no = b.ortho_len(), m = b.m;
  if (!b.composite()) return lm_identity(no);
  LMat P(m, no);
  if (b.bc()) {
    // c = bc_inv * (S^T p)
    for (int j = 0; j < 2; j++) {
      const long double s0 = j == 0 ? b.t0[0] : b.t1[0];  // (S^T e_j)_0
      const long double s1 = j == 0 ? b.t0[1] : b.t1[1];  // (S^T e_j)_1
      P.at(0, j) = b.bc_inv[0] * s0 + b.bc_inv[1] * s1;
      P.at(1, j) = b.bc_inv[2] * s0 + b.bc_inv[3] * s1;
    }
    return P;
  }
  // columns: the reference's stride-2 tridiagonal least-squares solve applied to e_j
  std::vector<long double> d(m), x(m);
  for (int j = 0; j < no; j++) {
    for (int i = 0; i < m; i++) {
      long double v = 0.0L;
      if (i == j) v += b.diag[i];
      if (i + 2 == j) v += b.low2[i];
      d[i] = v;
    }
    for (int i = 0; i < m; i++) {
      long double g = d[i];
      if (i >= 2) g -= (long double)b.fo_off[i - 2] * x[i - 2];
      x[i] = g * (long double)b.fo_dinv[i];
    }
    for (int i = m - 3; i >= 0; i--) x[i] -= (long double)b.fo_w[i] * x[i + 2];
    for (int i = 0; i < m; i++) P.at(i, j) = x[i];
  }
  return P;
}

LMat lm_pinv(int n) {
  Pinv p = make_pinv(n);
  LMat M(n - 2, n);
  for (int r = 0; r < n - 2; r++) {
    M.at(r, r) = p.dia[r];
    if (r + 2 < n) M.at(r, r + 2) = p.up1[r];
    if (r + 4 < n) M.at(r, r + 4) = p.up2[r];
  }
  return M;
}

}  // namespace rbc
