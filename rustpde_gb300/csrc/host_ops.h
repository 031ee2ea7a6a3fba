// host_ops.h -- set-up arithmetic of the spectral RBC library (host side).
//
// Everything here runs once per case (or per funspace space / solver) at
// creation time: basis stencils, the banded operators that the Helmholtz and
// Poisson solvers factorise, the eigen-decomposition of the box Poisson
// operator, and the transform tables.  Time stepping never runs on the host.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace rbc {

enum BaseKind { CHEB = 0, CD = 1, CN = 2, CDBC = 3, CNBC = 4, FOURIER = 5 };

// One-dimensional basis (funspace/src/chebyshev/{ortho,composite,composite_stencil}.rs,
// funspace/src/fourier/r2c.rs).
struct HostBasis {
  int kind = CHEB;
  int n = 0;  // physical length
  int m = 0;  // spectral length
  std::vector<double> x;           // grid coordinates (unscaled)
  std::vector<double> diag, low2;  // composite stencil p_i = diag_i c_i + low2_{i-2} c_{i-2}
  double t0[2] = {0, 0}, t1[2] = {0, 0};  // boundary stencil (2 modes)
  // from_ortho (stride-2 tridiagonal least squares, linalg.rs:14-57), data-independent part
  std::vector<double> fo_off;   // off-diagonal a = c (m-2)
  std::vector<double> fo_w;     // forward-sweep ratios w (m-2)
  std::vector<double> fo_dinv;  // 1/denominator (m)
  double bc_inv[4] = {0, 0, 0, 0};  // boundary basis: c = bc_inv * (S^T p), row-major 2x2

  bool fourier() const { return kind == FOURIER; }
  bool composite() const { return kind == CD || kind == CN || kind == CDBC || kind == CNBC; }
  bool bc() const { return kind == CDBC || kind == CNBC; }
  int ortho_len() const { return fourier() ? m : n; }
};

HostBasis make_basis(int kind, int n);

// Raw or swept diagonals (offsets -2, 0, +2, +4) of an n x n banded matrix (fdma.rs).
struct Band4 {
  int n = 0;
  std::vector<double> low, dia, up1, up2;  // n-2, n, n-2, n-4
};
Band4 band_combine(const Band4& a, const Band4& b, double l);  // a + b*l  (fdma.rs Add/Mul)
void band_sweep(Band4& f);                                      // fdma.rs:73-82
std::vector<double> band_dense(const Band4& b);

// Rows of the pseudo-inverse pinv = peye * laplace_inv (ortho.rs:147-180) as
// MatVecFdma stores them (matvec.rs:142-170): (n-2) rows, entries at i, i+2, i+4.
struct Pinv {
  int n = 0;  // ortho length; rows = n-2
  std::vector<double> dia, up1, up2;  // n-2 each (zero where the matrix is zero)
};
Pinv make_pinv(int n);

// field.rs:194-225 ingredients for a composite basis: A = pinv*S, B = peye*S.
void hholtz_ingredients(const HostBasis& b, Band4& A, Band4& B);

// Dense real eigen-decomposition with real eigenvalues: A V = V diag(lam),
// sorted by descending eigenvalue (utils.rs:66-98).  Row-major n x n.
bool eig_real(int n, const std::vector<double>& A, std::vector<double>& lam, std::vector<double>& V,
              std::string* err);
bool invert(int n, const std::vector<double>& A, std::vector<double>& Ainv);
std::vector<double> matmul(int n, int k, int m, const std::vector<double>& A, const std::vector<double>& B);

// Tables
std::vector<double> twiddles(int L);  // interleaved (re, im) of exp(-2 pi i t / L), t < L
// Dense Chebyshev transform matrices including the correction factors of
// ortho.rs:235-312.  fwd: ortho = M phys; bwd: phys = M ortho.  Row-major n x n.
std::vector<double> cheb_dense_forward(int n);
std::vector<double> cheb_dense_backward(int n);

inline bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

uint64_t splitmix64(uint64_t& s);

}  // namespace rbc
