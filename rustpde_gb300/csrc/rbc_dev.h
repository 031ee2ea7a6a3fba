// rbc_dev.h -- device-resident descriptors of one RBC case (shared by host and
// device code).  All pointers are device pointers into the case's arena.
//
// Layout in HBM: row-major (x, y) arrays with y contiguous, as the reference's
// ndarray default; complex spectral data interleaved (re, im) = double2.
#pragma once
#include <cstdint>

namespace rbc {

// One basis along one axis (tables built by host_ops.cpp make_basis).
struct BasisDev {
  int kind;   // BaseKind
  int n;      // physical / ortho length (Fourier: physical length)
  int m;      // spectral length
  int unit_diag;          // 1 when every diag_i is 1 (the composite bases here): the
                          // stencils skip the product, which is exact either way
  const double* diag;     // composite stencil diag (m)
  const double* low2;     // composite stencil low2 (m)
  const double* fo_off;   // from_ortho tdma off-diagonal (m-2)
  const double* fo_w;     // from_ortho tdma ratios (m-2)
  const double* fo_dinv;  // from_ortho tdma 1/denominators (m)
  // forward sweep of from_ortho with its factors multiplied out:
  // g_i = fo_a_i p_i + fo_b_i p_{i+2} + fo_c_i g_{i-2}
  const double* fo_a;     // diag_i / den_i (m)
  const double* fo_b;     // low2_i / den_i (m)
  const double* fo_c;     // -off_{i-2} / den_i, 0 for i < 2 (m)
  double t0[2], t1[2];    // boundary stencil
  double bc_inv[4];       // boundary least-squares inverse
};

// Rows of peye*laplace_inv for ortho length n (n-2 rows, entries at i, i+2, i+4).
struct PinvDev {
  int n;
  int pad_;
  const double* dia;
  const double* up1;
  const double* up2;
};

// Swept banded factors (offsets -2,0,2,4) of length m; `rows` > 1 means one
// factorisation per lane (row i at offset i*stride).
struct FdmaDev {
  int m;
  int rows;
  int stride;
  int pad_;
  const double* low;   // -low of the swept factors (m-2)
  const double* dinv;  // 1/dia (m)
  const double* up1;   // -up1/dia (m-2)
  const double* up2;   // -up2/dia (m-4)
};

// Chebyshev transform along an axis of length n: FFT (n = 2^p + 1) or dense.
struct ChebXformDev {
  int n;
  int use_fft;        // 1: DCT-I via complex FFT of length L = 2(n-1)
  int L;              // FFT length
  int log2L;
  const double2* tw;  // exp(-2 pi i t / L), t < L
  double inv_nm1;     // 1 / (n - 1)
  const double* fwd;  // dense n x n forward matrix (row = output)
  const double* bwd;  // dense n x n backward matrix
};

// Fourier r2c/c2r along x of physical length n (any n >= 4).  Even n runs
// through a complex FFT of half length M = n/2, odd n through one of length
// M = n.  A power-of-two M uses radix-4/2 Stockham stages (log2M >= 0);
// any other M the mixed-radix stages rad[0..nrad) (product M).
struct FourierXformDev {
  int n;        // physical length
  int M;        // complex FFT length: n/2 (even n) or n (odd n)
  int log2M;    // log2(M) when M is a power of two, else -1
  int nrad;     // mixed-radix stages (log2M < 0)
  int rad[16];  // their radices: 4s, then 2, 3, 5, 7 and any larger prime factors
  const double2* tw;  // exp(-2 pi i t / n), t < n
  const float2* twf;  // the same table rounded to FP32 (mixed-precision form)
};

enum CaseKind { KIND_BOX_ADIABATIC = 0, KIND_BOX_CONDUCTING = 1, KIND_PERIODIC = 2 };

// Everything the FP64 step kernels need for one case.
struct CaseDev {
  int kind;
  int nx, ny;      // physical grid
  int mx;          // spectral rows of ortho x arrays: box nx, periodic nx/2+1
  int mxc;         // spectral rows of composite-x arrays: box nx-2, periodic nx/2+1
  int myc;         // composite y length ny-2
  int kx, ky;      // dealias: rows kept (ortho x), columns kept (ortho y)
  double dt, nu, ka, aspect;
  double inv_dt;

  // bases: y (CD velocity/temp, CN pseudo pressure, CHEB pressure) and x
  BasisDev ycd, ycn;
  BasisDev xu;   // x basis of ux/uy (CD) or Fourier
  BasisDev xt;   // x basis of temperature (CN adiabatic / CD conducting) or Fourier
  BasisDev xp;   // x basis of pseudo pressure (CN) or Fourier
  PinvDev pinv_y;   // length ny
  PinvDev pinv_x;   // length nx (box)
  ChebXformDev cy;  // Chebyshev along y (length ny)
  ChebXformDev cx;  // Chebyshev along x (box)
  FourierXformDev fx;  // Fourier along x (periodic)

  // solvers
  FdmaDev hu_y, hu_x;    // box ADI velocity (y, x); periodic: hu_y per row
  FdmaDev ht_y, ht_x;    // box ADI temperature; periodic: per row
  FdmaDev pois_y;        // per-row factors of the pressure Poisson solve
  const double* pois_fwd;  // box: (mxc x mxc) eigenbasis forward, row-major
  const double* pois_bwd;  // box: eigenbasis backward

  // state (spectral): real (box) or double2 (periodic) elements
  void* ux;   // mxc x myc
  void* uy;   // mxc x myc
  void* temp; // mxc x myc
  void* p0;   // mx x ny
  void* p1;   // mxc x myc (Neumann)

  // constants derived from the temperature boundary field
  const void* bc_ortho;   // mx x ny: to_ortho(fieldbc)
  const void* bc_diff;    // mx x ny: dt*ka*(d2/dx2 + d2/dy2) fieldbc
  const double* bc_dx;    // nx x ny physical d/dx fieldbc
  const double* bc_dy;    // nx x ny physical d/dy fieldbc
  const double* bc_v;     // nx x ny physical fieldbc

  // solid-mask penalisation (navier.rs:551-560, 579-584, 603-608); null when
  // the case has no solid.  The x pass then also transforms the temperature.
  const double* solid_cm;   // nx x ny: (-1/eta) * mask, eta = 1e-2
  const double* solid_val;  // nx x ny: temperature imposed inside the solid

  // scratch (per case)
  void* yw[6];   // y-pass outputs (Y0, Y1 for ux, uy, temp): mxc x ny
  void* q[3];    // x-pass outputs (dealiased products, x transformed): kx x ny
  void* s[8];    // further scratch for the box pass sequence
  unsigned int* status;  // bit 0: non-finite value seen
  double* accum;         // reductions
  // serving: gate[0] = steps left, gate[1] = 1 when the case advances in the
  // current step (set by the gate kernel at the start of each step); null
  // outside the serving loop (always advance)
  int* gate;
  int pad_g;

  // mixed-precision form (precision RBC_PREC_MIXED): the dense transforms run
  // as tensor-core lane GEMMs, the convection products in FP32
  int mixed;
  // Mixed form: the boundary convection term's part m_bcg * uy, with m_bcg the
  // mean of d(fieldbc)/dy, is added in FP64 by the pass that forms the
  // temperature right-hand side, as m_bcg times the dealiased to_ortho(uy)
  // (the exact forward transform of m_bcg * uy).  It is linear in the state
  // and drives the convective instability; carried through the FP32 products
  // and two tensor-core transforms, their truncation bias shifted the growth
  // rate of near-critical cases.  m_bcy holds d(fieldbc)/dy - m_bcg.
  int m_bclin;
  double m_bcg;
  void* m_y[3];   // FP32 y-pass outputs [Y0 | Y1] per field, stored transposed: (2 ny) x mx
  void* m_q;      // FP32 x-transformed products, transposed: 3 x (ny x kx)
  void* m_cv;     // FP64 convection term, spectral: 3 x (kx x ky)
  void* m_ph[8];  // box: FP32 physical fields (nx x ny)
  void* m_p[3];   // box: FP32 products, then their x transforms
  void* m_z;      // box: FP32 pinv_x of the divergence (mxc x ny), then the FP32 Poisson row solutions (mxc x myc)
  void* m_s32;    // FP32 copy of ux, uy, temp, the y GEMM's input: 3 x mxc rows of s32_row_floats(), a
                  // real row padded to a multiple of 4 floats, a complex row as [re | im] parts of that length
  const float* m_bcx;  // FP32 d(fieldbc)/dx, transposed: ny x nx
  const float* m_bcy;  // FP32 d(fieldbc)/dy - m_bcg, transposed: ny x nx
};

// Row length (floats) of the mixed form's FP32 state copy m_s32 and of the
// box y GEMM's output rows m_y (mxc values): padded to a multiple of 4 floats
// so that the lane GEMM reads them with aligned 16-byte loads.
__host__ __device__ inline int pad4(int n) { return (n + 3) & ~3; }
__host__ __device__ inline int s32_row_floats(const CaseDev& c) {
  return c.kind == KIND_PERIODIC ? 2 * pad4(c.myc) : pad4(c.myc);
}

}  // namespace rbc
