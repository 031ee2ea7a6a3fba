// dense_ops.h -- dense matrices of the 1-D spectral operators (host, set-up).
//
// The mixed-precision form applies compositions of stencils, derivatives and
// Chebyshev transforms along a lane as one dense matrix on the tensor cores.
// The compositions are formed here once, in long double, and rounded to
// double before the TF32 split.
#pragma once
#include <vector>

#include "host_ops.h"

namespace rbc {

struct LMat {
  int rows = 0, cols = 0;
  std::vector<long double> a;  // row-major
  LMat() = default;
  LMat(int r, int c) : rows(r), cols(c), a((size_t)r * c, 0.0L) {}
  long double& at(int i, int j) { return a[(size_t)i * cols + j]; }
  long double at(int i, int j) const { return a[(size_t)i * cols + j]; }
};

LMat lm_identity(int n);
LMat lm_mul(const LMat& A, const LMat& B);
LMat lm_scale(const LMat& A, long double s);
LMat lm_rows(const LMat& A, int r0, int r1);   // rows [r0, r1)
LMat lm_vstack(const LMat& A, const LMat& B);
std::vector<double> lm_to_double(const LMat& A);

// Chebyshev transforms of length n with the reference's normalisation
// (funspace/src/chebyshev/ortho.rs:235-312): ortho = F phys, phys = B ortho.
LMat lm_cheb_forward(int n);
LMat lm_cheb_backward(int n);
// First derivative on ortho coefficients (ortho.rs:107-125), n x n.
LMat lm_cheb_diff(int n);
// Stencil of a basis: ortho = S spec (ortho_len x m); identity for Chebyshev.
LMat lm_stencil(const HostBasis& b);
// Least-squares inverse of the stencil (composite_stencil.rs:240-276): spec = P ortho.
LMat lm_from_ortho(const HostBasis& b);
// peye * laplace_inv rows (ortho.rs:147-180), (n-2) x n.
LMat lm_pinv(int n);

}  // namespace rbc
