// step_fp64.cu -- the plain FP64 Rayleigh-Benard time step as fused lane passes.
//
// One call of Integrate::update (src/navier/navier.rs:737-765) is decomposed
// into passes along y (lanes = rows, contiguous) and along x (lanes = columns).
// Linear operators acting on different axes commute, so each pass applies all
// the work that is local to its lanes; the reference's results are reproduced
// up to floating-point reassociation.
//
//  periodic (FourierR2c x Chebyshev):  Y1 -> X -> Y2            (3 launches)
//  box (Chebyshev x Chebyshev):        Y1 -> X1 -> Y2 -> X2 -> Y3 -> X3 -> Y4 -> X4 -> Y5
//
// Each launch takes a table of work items (case, first lane, lane count); a
// batch of cases is the same launch with a longer table.
#include "lane_ops.cuh"
#include "per_device.h"
#include "prims.h"
#include "step_fp64.h"

#include <algorithm>

namespace rbc {
namespace dev {

static __device__ __forceinline__ void flag_nonfinite(unsigned int* status) { atomicOr(status, 1u); }

// load a lane set: lane l (0 <= l < 3*nr) = field (l / nr), row (r0 + l % nr)
template <class T>
__device__ void load_rows3(void* const f[3], int row_len, int r0, int nr, T* dst, int ld, int tid, int nth) {
  for (int idx = tid; idx < 3 * nr * row_len; idx += nth) {
    int l = idx / row_len, j = idx - l * row_len;
    int fi = l / nr, r = l - fi * nr;
    dst[l * ld + j] = static_cast<const T*>(f[fi])[(size_t)(r0 + r) * row_len + j];
  }
  __syncthreads();
}

// ============================================================================
// Y1: Y0_f = Ty^-1 Sy f,  Y1_f = Ty^-1 Dy Sy f   for f in (ux, uy, temp)
// ============================================================================
template <class T>
__global__ void __launch_bounds__(256) k_y1(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int r0 = w.y, nr = w.z;
  const int ny = c.ny, myc = c.myc, ld = c.ny + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  extern __shared__ double2 smem[];
  T* IN = reinterpret_cast<T*>(smem);
  T* O = IN + 3 * nr * ld;   // 3nr ortho lanes, followed by
  T* D = O + 3 * nr * ld;    // 3nr derivative lanes
  T* TMP = D + 3 * nr * ld;
  double2* WA = reinterpret_cast<double2*>(TMP + 3 * nr * ld + 2);
  WA = reinterpret_cast<double2*>((reinterpret_cast<size_t>(WA) + 15) & ~size_t(15));
  const int wld = c.cy.use_fft ? c.cy.L : 1;
  double2* WB = WA + (size_t)3 * nr * wld;
  void* f3[3] = {c.ux, c.uy, c.temp};
  load_rows3<T>(f3, myc, r0, nr, IN, ld, tid, nth);
  to_ortho<T>(c.ycd, IN, ld, O, ld, 3 * nr, tid, nth);
  cheb_diff<T>(O, ld, D, ld, ny, 3 * nr, 1, TMP, ld, tid, nth);
  // inverse Chebyshev transform of O and D (6nr lanes, O and D contiguous)
  if (c.cy.use_fft) {
    if constexpr (sizeof(T) == 16) {
      dct1_fft_c(c.cy, false, (const double2*)O, ld, (double2*)O, ld, 3 * nr, WA, WB, wld, tid, nth);
      dct1_fft_c(c.cy, false, (const double2*)D, ld, (double2*)D, ld, 3 * nr, WA, WB, wld, tid, nth);
    } else {
      dct1_fft_r(c.cy, false, (const double*)O, ld, (double*)O, ld, 6 * nr, WA, WB, wld, tid, nth);
    }
  } else {
    dct1_dense<T>(c.cy, false, O, ld, TMP, ld, 3 * nr, tid, nth);
    for (int idx = tid; idx < 3 * nr * ny; idx += nth) {
      int l = idx / ny, k = idx - l * ny;
      O[l * ld + k] = TMP[l * ld + k];
    }
    __syncthreads();
    dct1_dense<T>(c.cy, false, D, ld, TMP, ld, 3 * nr, tid, nth);
    for (int idx = tid; idx < 3 * nr * ny; idx += nth) {
      int l = idx / ny, k = idx - l * ny;
      D[l * ld + k] = TMP[l * ld + k];
    }
    __syncthreads();
  }
  // store: yw[2f] = O lanes, yw[2f+1] = D lanes; row stride ny
  for (int idx = tid; idx < 6 * nr * ny; idx += nth) {
    int l = idx / ny, k = idx - l * ny;
    int which = l / (3 * nr), ll = l - which * 3 * nr;
    int fi = ll / nr, r = ll - fi * nr;
    const T* src = which ? D : O;
    static_cast<T*>(c.yw[2 * fi + which])[(size_t)(r0 + r) * ny + k] = src[ll * ld + k];
  }
}

size_t smem_y1(const CaseDev& c, int nr, bool cplx) {
  size_t es = cplx ? 16 : 8;
  size_t ld = c.ny + 1;
  size_t base = 4 * 3 * nr * ld * es + 2 * 8 + 16;
  size_t wld = c.cy.use_fft ? c.cy.L : 1;
  return base + 2 * (size_t)3 * nr * wld * 16 + 64;
}

// solid-mask damping of the convection products at physical point g
// (navier.rs:551-560, 579-584, 603-608): conv -= (-1/eta) mask w with
// w = ux, uy, and T + T_bc - value for the temperature (f = 2)
__device__ __forceinline__ double solid_damp(const CaseDev& c, int f, size_t g, double p, double u, double v, double t) {
  const double cm = c.solid_cm[g];
  const double w = f == 0 ? u : f == 1 ? v : (t + c.bc_v[g]) - c.solid_val[g];
  return p - cm * w;
}

// ============================================================================
// Periodic X pass: one column j of the Y arrays.
//  u = F^-1 Y0_ux, v = F^-1 Y0_uy;  for f: a = F^-1 (ik/s Y0_f), b = F^-1 Y1_f
//  P_f = u a + v b (+ u dbc/dx + v dbc/dy for temp);  Q_f = F P_f, rows < kx
//  With a solid mask a ninth lane carries T = F^-1 Y0_t for the damping term.
// ============================================================================
__global__ void __launch_bounds__(256) k_per_x(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int j = w.y;
  const int mx = c.mx, nx = c.nx, ny = c.ny, M = c.fx.M;
  const int tid = threadIdx.x, nth = blockDim.x;
  const double inv_asp = 1.0 / c.aspect;
  const bool solid = c.solid_cm != nullptr;
  const int NL = solid ? 9 : 8;
  extern __shared__ double2 smem[];
  const int ild = mx + 1;         // input lanes (complex)
  double2* IN = smem;             // NL lanes
  double2* WA = IN + NL * ild;    // NL lanes of M
  double2* WB = WA + NL * M;
  double* PH = reinterpret_cast<double*>(IN);  // physical lanes alias the inputs (NL x nx reals)
  // lane order: Y0u, Y0v, ikY0u, Y1u, ikY0v, Y1v, ikY0t, Y1t (, Y0t)
  for (int idx = tid; idx < NL * mx; idx += nth) {
    int l = idx / mx, k = idx - l * mx;
    int src = (l == 8) ? 4 : (l < 2) ? 2 * l : (l & 1 ? 2 * ((l - 2) >> 1) + 1 : 2 * ((l - 2) >> 1));
    double2 v = static_cast<const double2*>(c.yw[src])[(size_t)k * ny + j];
    if (l >= 2 && l < 8 && !(l & 1)) v = mul_ik(v, (double)k) * inv_asp;
    IN[l * ild + k] = v;
  }
  __syncthreads();
  c2r(c.fx, IN, ild, 1, PH, nx, NL, WA, WB, M, tid, nth);
  // products into lanes 2, 4, 6
  const double* bx = c.bc_dx;
  const double* by = c.bc_dy;
  for (int idx = tid; idx < 3 * nx; idx += nth) {
    int f = idx / nx, x = idx - f * nx;
    double u = PH[x], v = PH[nx + x];
    double a = PH[(2 + 2 * f) * nx + x], b = PH[(3 + 2 * f) * nx + x];
    double p = u * a + v * b;
    if (f == 2) {
      p = p + u * bx[(size_t)x * ny + j];
      p = p + v * by[(size_t)x * ny + j];
    }
    if (solid) p = solid_damp(c, f, (size_t)x * ny + j, p, u, v, PH[8 * nx + x]);
    PH[(2 + 2 * f) * nx + x] = p;
  }
  __syncthreads();
  double2* q = static_cast<double2*>(c.q[0]);
  r2c(c.fx, PH + 2 * nx, 2 * nx, q + j, c.kx * ny, ny, c.kx, 3, WA, WB, M, tid, nth);
}

size_t smem_per_x(const CaseDev& c) {
  const size_t nl = c.solid_cm ? 9 : 8;
  size_t ild = c.mx + 1;
  size_t in_bytes = std::max(nl * ild * 16, nl * c.nx * 8);
  return in_bytes + 2 * nl * (size_t)c.fx.M * 16 + 64;
}

// ============================================================================
// Periodic Y2 pass: one row i.  Convection DCT, right-hand sides, Helmholtz
// solves (Hholtz per row), divergence, Poisson row solve, projection and the
// pressure update (navier.rs:622-721).
// ============================================================================
// stage the factors of row `row` of a per-row banded solver into shared memory
__device__ FdmaDev stage_fdma_row(const FdmaDev& f, int row, double* dst, int tid, int nth) {
  const int m = f.m;
  const size_t off = (f.rows > 1) ? (size_t)row * f.stride : 0;
  for (int k = tid; k < m; k += nth) {
    dst[k] = f.low[off + k];
    dst[m + k] = f.dinv[off + k];
    dst[2 * m + k] = f.up1[off + k];
    dst[3 * m + k] = f.up2[off + k];
  }
  FdmaDev r = f;
  r.rows = 1;
  r.stride = 0;
  r.low = dst;
  r.dinv = dst + m;
  r.up1 = dst + 2 * m;
  r.up2 = dst + 3 * m;
  return r;
}

// PRE: the convection term arrives already transformed along y (m_cv, FP64,
// from the mixed-precision form's tensor-core GEMM) instead of q.
template <bool PRE>
__global__ void __launch_bounds__(256) k_per_y2(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int i = w.y;
  const int ny = c.ny, myc = c.myc, kx = c.kx, ky = c.ky;
  const int ld = ny + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  const double dt = c.dt, nu = c.nu, inv_asp = 1.0 / c.aspect, ki = (double)i;
  extern __shared__ double2 smem[];
  double2* CV = smem;        // 3 lanes conv
  double2* REG = CV + 3 * ld;
  // during the convection transform REG holds the FFT work lanes; afterwards:
  double2* F = REG;          // 3 lanes composite state (old, then new)
  double2* O = F + 3 * ld;   // 3 lanes
  // rhs lanes (lane 0 later: divergence); with the convection term given (PRE)
  // they overwrite the convection lanes, which are dead once the rhs is formed
  double2* R = PRE ? CV : O + 3 * ld;
  double2* P = PRE ? O + 3 * ld : R + 3 * ld;  // p0 row
  double2* G = P + ld;       // d/dy
  double2* X1 = G + ld;      // 3 lanes
  const int wld = c.cy.use_fft ? c.cy.L : 1;
  double2* WA = REG;
  double2* WB = WA + 3 * wld;
  const size_t reg_elems = PRE ? (size_t)11 * ld : max((size_t)14 * ld, (size_t)6 * wld);
  double* FAC = reinterpret_cast<double*>(REG + reg_elems);
  // per-row factors of the three banded solves
  const FdmaDev fu = stage_fdma_row(c.hu_y, i, FAC, tid, nth);
  const FdmaDev ft = stage_fdma_row(c.ht_y, i, FAC + 4 * myc, tid, nth);
  const FdmaDev fp = stage_fdma_row(c.pois_y, i, FAC + 8 * myc, tid, nth);

  // 1. convection: forward Chebyshev transform of Q_f[i], dealiased
  if (PRE) {
    const double2* cv = static_cast<const double2*>(c.m_cv);
    for (int idx = tid; idx < 3 * ny; idx += nth) {
      int f = idx / ny, k = idx - f * ny;
      CV[f * ld + k] = (i < kx && k < ky) ? cv[((size_t)f * kx + i) * ky + k] : c2(0.0, 0.0);
    }
  } else if (i < kx) {
    const double2* q = static_cast<const double2*>(c.q[0]);
    for (int idx = tid; idx < 3 * ny; idx += nth) {
      int f = idx / ny, k = idx - f * ny;
      CV[f * ld + k] = q[(size_t)f * kx * ny + (size_t)i * ny + k];
    }
    __syncthreads();
    if (c.cy.use_fft) dct1_fft_c(c.cy, true, CV, ld, CV, ld, 3, WA, WB, wld, tid, nth);
    else {
      dct1_dense<double2>(c.cy, true, CV, ld, REG, ld, 3, tid, nth);
      for (int idx = tid; idx < 3 * ny; idx += nth) {
        int f = idx / ny, k = idx - f * ny;
        CV[f * ld + k] = REG[f * ld + k];
      }
      __syncthreads();
    }
    for (int idx = tid; idx < 3 * ny; idx += nth) {
      int f = idx / ny, k = idx - f * ny;
      if (k >= ky) CV[f * ld + k] = c2(0.0, 0.0);
    }
  } else {
    for (int idx = tid; idx < 3 * ny; idx += nth) CV[(idx / ny) * ld + idx % ny] = c2(0.0, 0.0);
  }
  __syncthreads();
  // 2. right-hand sides
  void* f3[3] = {c.ux, c.uy, c.temp};
  for (int idx = tid; idx < 3 * myc; idx += nth) {
    int f = idx / myc, k = idx - f * myc;
    F[f * ld + k] = static_cast<const double2*>(f3[f])[(size_t)i * myc + k];
  }
  const double2* p0 = static_cast<const double2*>(c.p0);
  for (int k = tid; k < ny; k += nth) P[k] = p0[(size_t)i * ny + k];
  __syncthreads();
  to_ortho<double2>(c.ycd, F, ld, O, ld, 3, tid, nth);
  cheb_diff<double2>(P, ld, G, ld, ny, 1, 1, nullptr, ld, tid, nth);
  const double2* bco = static_cast<const double2*>(c.bc_ortho);
  const double2* bcd = static_cast<const double2*>(c.bc_diff);
  for (int k = tid; k < ny; k += nth) {
    double2 gx = mul_ik(P[k], ki) * inv_asp;
    double2 cu = CV[k], cvv = CV[ld + k], ct = CV[2 * ld + k];
    if (PRE && c.m_bclin && i < kx && k < ky) ct = add_bclin(ct, O[ld + k], c.m_bcg, i);
    R[k] = fnms(fnms(O[k], gx, dt), cu, dt);
    double2 that = O[2 * ld + k] + bco[(size_t)i * ny + k];
    R[ld + k] = fnms(fmas(fnms(O[ld + k], G[k], dt), that, dt), cvv, dt);
    R[2 * ld + k] = fnms(O[2 * ld + k] + bcd[(size_t)i * ny + k], ct, dt);
  }
  __syncthreads();
  // 3. Helmholtz: pinv_y then the row's banded solve
  matvec_pinv<double2>(c.pinv_y, R, ld, F, ld, 3, tid, nth);
  // ux*, uy* (factors fu) and temp (factors ft): 6 chains in one phase
  fdma_solve2<double2>(fu, ft, 2, F, ld, 3, 0, 0, tid, nth);
  // 4. divergence = ik/s Sy ux* + Dy Sy uy*
  to_ortho<double2>(c.ycd, F, ld, O, ld, 2, tid, nth);
  cheb_diff<double2>(O + ld, ld, G, ld, ny, 1, 1, nullptr, ld, tid, nth);
  for (int k = tid; k < ny; k += nth) R[k] = mul_ik(O[k], ki) * inv_asp + G[k];  // R lane 0 = div
  __syncthreads();
  // 5. Poisson row solve -> pseudo pressure row
  matvec_pinv<double2>(c.pinv_y, R, ld, X1, ld, 1, tid, nth);
  fdma_solve<double2>(fp, X1, ld, 1, 0, 0, tid, nth);
  if (i == 0 && tid == 0) X1[0] = c2(0.0, 0.0);
  __syncthreads();
  double2* p1 = static_cast<double2*>(c.p1);
  for (int k = tid; k < myc; k += nth) p1[(size_t)i * myc + k] = X1[k];
  // 6. projection: O1 = Sy^N p1; dpdx = ik/s O1; dpdy = Dy O1
  to_ortho<double2>(c.ycn, X1, ld, O, ld, 1, tid, nth);  // O lane 0 = O1
  cheb_diff<double2>(O, ld, G, ld, ny, 1, 1, nullptr, ld, tid, nth);  // G = dpdy
  for (int k = tid; k < ny; k += nth) {
    O[ld + k] = mul_ik(O[k], ki) * inv_asp;  // O lane 1 = dpdx
    O[2 * ld + k] = G[k];                     // O lane 2 = dpdy
  }
  __syncthreads();
  from_ortho<double2>(c.ycd, O + ld, ld, X1 + ld, ld, 2, tid, nth);  // X1 lanes 1, 2
  // 7. pressure update and stores
  double2* pw = static_cast<double2*>(c.p0);
  for (int k = tid; k < ny; k += nth) {
    double2 v = fnms(P[k], R[k], nu);
    pw[(size_t)i * ny + k] = fmas(v, O[k], c.inv_dt);
  }
  double2* ux = static_cast<double2*>(c.ux);
  double2* uy = static_cast<double2*>(c.uy);
  double2* tt = static_cast<double2*>(c.temp);
  bool bad = false;
  for (int k = tid; k < myc; k += nth) {
    double2 a = F[k] - X1[ld + k];
    double2 b = F[ld + k] - X1[2 * ld + k];
    double2 t = F[2 * ld + k];
    ux[(size_t)i * myc + k] = a;
    uy[(size_t)i * myc + k] = b;
    tt[(size_t)i * myc + k] = t;
    bad |= !(finite_v(a) && finite_v(b) && finite_v(t));
  }
  if (bad) flag_nonfinite(c.status);
}

// ============================================================================
// Periodic Y2 split in two launches for more CTAs per SM:
//  Y2a (row i, field f): convection transform, right-hand side, pinv_y and the
//       row's banded Helmholtz solve; writes ux*, uy* (into the state arrays,
//       overwritten by Y2b) and the new temperature.
//  Y2b (row i): divergence, Poisson row solve, projection, pressure update.
// ============================================================================
__global__ void __launch_bounds__(256) k_per_y2a(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int i = w.y, f = w.w;
  const int ny = c.ny, myc = c.myc, kx = c.kx, ky = c.ky;
  const int ld = ny + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  const double dt = c.dt, inv_asp = 1.0 / c.aspect, ki = (double)i;
  extern __shared__ double2 smem[];
  double2* CV = smem;   // conv lane
  double2* REG = CV + ld;
  double2* F = REG;      // composite row of field f
  double2* T2 = F + ld;  // composite temperature row (buoyancy of uy)
  double2* O = T2 + ld;  // ortho of F
  double2* OT = O + ld;  // ortho of T2
  double2* R = OT + ld;  // rhs
  double2* P = R + ld;   // p0 row
  double2* G = P + ld;   // d/dy p0
  const int wld = c.cy.use_fft ? c.cy.L : 1;
  double2* WA = REG;
  double2* WB = WA + wld;
  const size_t reg_elems = max((size_t)7 * ld, (size_t)2 * wld);
  double* FAC = reinterpret_cast<double*>(REG + reg_elems);
  const FdmaDev fr = stage_fdma_row(f == 2 ? c.ht_y : c.hu_y, i, FAC, tid, nth);
  void* f3[3] = {c.ux, c.uy, c.temp};
  // convection
  if (i < kx) {
    const double2* q = static_cast<const double2*>(c.q[0]) + (size_t)f * kx * ny + (size_t)i * ny;
    for (int k = tid; k < ny; k += nth) CV[k] = q[k];
    __syncthreads();
    if (c.cy.use_fft) dct1_fft_c(c.cy, true, CV, ld, CV, ld, 1, WA, WB, wld, tid, nth);
    else {
      dct1_dense<double2>(c.cy, true, CV, ld, REG, ld, 1, tid, nth);
      for (int k = tid; k < ny; k += nth) CV[k] = REG[k];
      __syncthreads();
    }
    for (int k = tid; k < ny; k += nth)
      if (k >= ky) CV[k] = c2(0.0, 0.0);
  } else {
    for (int k = tid; k < ny; k += nth) CV[k] = c2(0.0, 0.0);
  }
  __syncthreads();
  // right-hand side
  const double2* st = static_cast<const double2*>(f3[f]) + (size_t)i * myc;
  for (int k = tid; k < myc; k += nth) F[k] = st[k];
  const double2* p0 = static_cast<const double2*>(c.p0) + (size_t)i * ny;
  if (f < 2)
    for (int k = tid; k < ny; k += nth) P[k] = p0[k];
  if (f == 1) {
    const double2* tt = static_cast<const double2*>(c.temp) + (size_t)i * myc;
    for (int k = tid; k < myc; k += nth) T2[k] = tt[k];
  }
  __syncthreads();
  to_ortho<double2>(c.ycd, F, ld, O, ld, f == 1 ? 2 : 1, tid, nth);  // O (and OT for uy)
  if (f == 1) cheb_diff<double2>(P, ld, G, ld, ny, 1, 1, nullptr, ld, tid, nth);
  const double2* bco = static_cast<const double2*>(c.bc_ortho) + (size_t)i * ny;
  const double2* bcd = static_cast<const double2*>(c.bc_diff) + (size_t)i * ny;
  for (int k = tid; k < ny; k += nth) {
    double2 r;
    if (f == 0) {
      double2 gx = mul_ik(P[k], ki) * inv_asp;
      r = fnms(fnms(O[k], gx, dt), CV[k], dt);
    } else if (f == 1) {
      double2 that = OT[k] + bco[k];
      r = fnms(fmas(fnms(O[k], G[k], dt), that, dt), CV[k], dt);
    } else {
      r = fnms(O[k] + bcd[k], CV[k], dt);
    }
    R[k] = r;
  }
  __syncthreads();
  matvec_pinv<double2>(c.pinv_y, R, ld, F, ld, 1, tid, nth);
  fdma_solve<double2>(fr, F, ld, 1, 0, 0, tid, nth);
  // ux*, uy* go to the state arrays (Y2b overwrites them with the projected
  // fields); the new temperature goes to scratch yw[0] because the uy work of
  // the same row still reads the old temperature for the buoyancy.
  double2* out = (f == 2 ? static_cast<double2*>(c.yw[0]) : static_cast<double2*>(f3[f])) + (size_t)i * myc;
  bool bad = false;
  for (int k = tid; k < myc; k += nth) {
    double2 v = F[k];
    out[k] = v;
    bad |= !finite_v(v);
  }
  if (bad) flag_nonfinite(c.status);
}

size_t smem_per_y2a(const CaseDev& c) {
  size_t ld = c.ny + 1;
  size_t wld = c.cy.use_fft ? c.cy.L : 1;
  size_t reg = std::max((size_t)7 * ld, (size_t)2 * wld);
  return (ld + reg) * 16 + (size_t)4 * c.myc * 8 + 64;
}

__global__ void __launch_bounds__(256) k_per_y2b(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int i = w.y;
  const int ny = c.ny, myc = c.myc;
  const int ld = ny + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  const double nu = c.nu, inv_asp = 1.0 / c.aspect, ki = (double)i;
  extern __shared__ double2 smem[];
  double2* F = smem;       // 2 lanes: ux*, uy*
  double2* O = F + 2 * ld; // 3 lanes
  double2* R = O + 3 * ld; // divergence
  double2* G = R + ld;
  double2* X1 = G + ld;    // 3 lanes
  double* FAC = reinterpret_cast<double*>(X1 + 3 * ld);
  const FdmaDev fp = stage_fdma_row(c.pois_y, i, FAC, tid, nth);
  double2* ux = static_cast<double2*>(c.ux) + (size_t)i * myc;
  double2* uy = static_cast<double2*>(c.uy) + (size_t)i * myc;
  for (int k = tid; k < myc; k += nth) {
    F[k] = ux[k];
    F[ld + k] = uy[k];
  }
  __syncthreads();
  to_ortho<double2>(c.ycd, F, ld, O, ld, 2, tid, nth);
  cheb_diff<double2>(O + ld, ld, G, ld, ny, 1, 1, nullptr, ld, tid, nth);
  for (int k = tid; k < ny; k += nth) R[k] = mul_ik(O[k], ki) * inv_asp + G[k];
  __syncthreads();
  matvec_pinv<double2>(c.pinv_y, R, ld, X1, ld, 1, tid, nth);
  fdma_solve<double2>(fp, X1, ld, 1, 0, 0, tid, nth);
  if (i == 0 && tid == 0) X1[0] = c2(0.0, 0.0);
  __syncthreads();
  double2* p1 = static_cast<double2*>(c.p1) + (size_t)i * myc;
  for (int k = tid; k < myc; k += nth) p1[k] = X1[k];
  to_ortho<double2>(c.ycn, X1, ld, O, ld, 1, tid, nth);
  cheb_diff<double2>(O, ld, G, ld, ny, 1, 1, nullptr, ld, tid, nth);
  for (int k = tid; k < ny; k += nth) {
    O[ld + k] = mul_ik(O[k], ki) * inv_asp;
    O[2 * ld + k] = G[k];
  }
  __syncthreads();
  from_ortho<double2>(c.ycd, O + ld, ld, X1 + ld, ld, 2, tid, nth);
  double2* pw = static_cast<double2*>(c.p0) + (size_t)i * ny;
  for (int k = tid; k < ny; k += nth) {
    double2 v = fnms(pw[k], R[k], nu);
    pw[k] = fmas(v, O[k], c.inv_dt);
  }
  const double2* tn = static_cast<const double2*>(c.yw[0]) + (size_t)i * myc;
  double2* tt = static_cast<double2*>(c.temp) + (size_t)i * myc;
  bool bad = false;
  for (int k = tid; k < myc; k += nth) {
    double2 a = F[k] - X1[ld + k];
    double2 b = F[ld + k] - X1[2 * ld + k];
    ux[k] = a;
    uy[k] = b;
    tt[k] = tn[k];
    bad |= !(finite_v(a) && finite_v(b));
  }
  if (bad) flag_nonfinite(c.status);
}

size_t smem_per_y2b(const CaseDev& c) {
  size_t ld = c.ny + 1;
  return (size_t)10 * ld * 16 + (size_t)4 * c.myc * 8 + 64;
}

size_t smem_per_y2(const CaseDev& c) {
  size_t ld = c.ny + 1;
  size_t wld = c.cy.use_fft ? c.cy.L : 1;
  size_t reg = std::max((size_t)14 * ld, (size_t)6 * wld);
  return (3 * ld + reg) * 16 + (size_t)12 * c.myc * 8 + 64;
}
// k_per_y2<true>: the rhs lanes reuse the convection lanes
size_t smem_per_y2_pre(const CaseDev& c) {
  size_t ld = c.ny + 1;
  return (3 * ld + 11 * ld) * 16 + (size_t)12 * c.myc * 8 + 64;
}

// ============================================================================
// Box passes (Chebyshev in x).  Real data.
// ============================================================================
// X1: columns j < ny.  x-backward of the y-transformed state, products,
// x-forward of the products (rows < kx), and d/dx p0.
__global__ void __launch_bounds__(256) k_box_x1(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int j = w.y;
  const int nx = c.nx, ny = c.ny, mxc = c.mxc, kx = c.kx;
  const int ld = nx + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  const double inv_asp = 1.0 / c.aspect;
  const bool solid = c.solid_cm != nullptr;
  const int NL = solid ? 9 : 8;
  extern __shared__ double2 smem[];
  double* IN = reinterpret_cast<double*>(smem);  // NL lanes composite-x (mxc)
  double* OR = IN + NL * ld;                     // NL ortho lanes (nx)
  double* PH = OR + NL * ld;                     // NL physical lanes
  double* TMP = PH + NL * ld;                    // NL lanes
  double2* WA = reinterpret_cast<double2*>(TMP + NL * ld + 2);
  WA = reinterpret_cast<double2*>((reinterpret_cast<size_t>(WA) + 15) & ~size_t(15));
  const int wld = c.cx.use_fft ? c.cx.L : 1;
  double2* WB = WA + ((NL + 1) >> 1) * wld;
  // lanes: 0 Y0u, 1 Y0v, 2 Y0u(dx), 3 Y1u, 4 Y0v(dx), 5 Y1v, 6 Y0t(dx), 7 Y1t (, 8 Y0t)
  for (int idx = tid; idx < NL * mxc; idx += nth) {
    int l = idx / mxc, k = idx - l * mxc;
    int src = (l == 8) ? 4 : (l < 2) ? 2 * l : (l & 1 ? 2 * ((l - 2) >> 1) + 1 : 2 * ((l - 2) >> 1));
    IN[l * ld + k] = static_cast<const double*>(c.yw[src])[(size_t)k * ny + j];
  }
  __syncthreads();
  // x stencils: lanes 0-5 use the velocity basis, 6-8 the temperature basis
  to_ortho<double>(c.xu, IN, ld, OR, ld, 6, tid, nth);
  to_ortho<double>(c.xt, IN + 6 * ld, ld, OR + 6 * ld, ld, NL - 6, tid, nth);
  // d/dx for lanes 2, 4, 6 (in place through TMP)
  for (int f = 0; f < 3; f++) {
    double* lane = OR + (2 + 2 * f) * ld;
    cheb_diff<double>(lane, ld, TMP, ld, nx, 1, 1, TMP + ld, ld, tid, nth);
    for (int k = tid; k < nx; k += nth) lane[k] = TMP[k] * inv_asp;
    __syncthreads();
  }
  if (c.cx.use_fft) dct1_fft_r(c.cx, false, OR, ld, PH, ld, NL, WA, WB, wld, tid, nth);
  else dct1_dense<double>(c.cx, false, OR, ld, PH, ld, NL, tid, nth);
  // products (lanes 2, 4, 6)
  for (int idx = tid; idx < 3 * nx; idx += nth) {
    int f = idx / nx, x = idx - f * nx;
    double u = PH[x], v = PH[ld + x];
    double p = u * PH[(2 + 2 * f) * ld + x] + v * PH[(3 + 2 * f) * ld + x];
    if (f == 2) {
      p = p + u * c.bc_dx[(size_t)x * ny + j];
      p = p + v * c.bc_dy[(size_t)x * ny + j];
    }
    if (solid) p = solid_damp(c, f, (size_t)x * ny + j, p, u, v, PH[8 * ld + x]);
    TMP[f * ld + x] = p;
  }
  __syncthreads();
  // forward x transform of the 3 products -> OR lanes 0..2
  if (c.cx.use_fft) dct1_fft_r(c.cx, true, TMP, ld, OR, ld, 3, WA, WB, wld, tid, nth);
  else dct1_dense<double>(c.cx, true, TMP, ld, OR, ld, 3, tid, nth);
  double* q = static_cast<double*>(c.q[0]);
  for (int idx = tid; idx < 3 * kx; idx += nth) {
    int f = idx / kx, k = idx - f * kx;
    q[(size_t)f * kx * ny + (size_t)k * ny + j] = OR[f * ld + k];
  }
  // d/dx p0 column / aspect -> s[0] (nx x ny)
  const double* p0 = static_cast<const double*>(c.p0);
  for (int k = tid; k < nx; k += nth) IN[k] = p0[(size_t)k * ny + j];
  __syncthreads();
  cheb_diff<double>(IN, ld, TMP, ld, nx, 1, 1, TMP + ld, ld, tid, nth);
  double* gp = static_cast<double*>(c.s[0]);
  for (int k = tid; k < nx; k += nth) gp[(size_t)k * ny + j] = TMP[k] * inv_asp;
}

// d/dx p0 / aspect for column j -> s[0] (nx x ny): the pressure-gradient part
// of X1, run on its own in the mixed-precision step (FP64)
__global__ void __launch_bounds__(256) k_box_gpx(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int j = w.y;
  const int nx = c.nx, ny = c.ny;
  const int ld = nx + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  const double inv_asp = 1.0 / c.aspect;
  extern __shared__ double2 smem[];
  double* IN = reinterpret_cast<double*>(smem);
  double* TMP = IN + ld;
  const double* p0 = static_cast<const double*>(c.p0);
  for (int k = tid; k < nx; k += nth) IN[k] = p0[(size_t)k * ny + j];
  __syncthreads();
  cheb_diff<double>(IN, ld, TMP, ld, nx, 1, 1, TMP + ld, ld, tid, nth);
  double* gp = static_cast<double*>(c.s[0]);
  for (int k = tid; k < nx; k += nth) gp[(size_t)k * ny + j] = TMP[k] * inv_asp;
}

size_t smem_box_gpx(const CaseDev& c) { return 3 * (size_t)(c.nx + 1) * 8 + 64; }

size_t smem_box_x1(const CaseDev& c) {
  const size_t nl = c.solid_cm ? 9 : 8;
  size_t ld = c.nx + 1;
  size_t wld = c.cx.use_fft ? c.cx.L : 1;
  return 4 * nl * ld * 8 + 2 * ((nl + 1) / 2) * wld * 16 + 64;
}

// Y2: rows i < nx (ortho x).  conv (y forward, dealiased), rhs, pinv_y -> s[1..3]
// PRE: the convection term arrives transformed (m_cv, from the tensor-core GEMMs).
template <bool PRE>
__global__ void __launch_bounds__(256) k_box_y2(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int i = w.y;
  const int nx = c.nx, ny = c.ny, myc = c.myc, kx = c.kx, ky = c.ky, mxc = c.mxc;
  const int ld = ny + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  const double dt = c.dt;
  extern __shared__ double2 smem[];
  double* CV = reinterpret_cast<double*>(smem);  // 3 lanes
  double* SX = CV + 3 * ld;   // 3 lanes: Sx f (composite y)
  double* O = SX + 3 * ld;    // 3 lanes
  double* R = O + 3 * ld;     // 3 lanes
  double* P = R + 3 * ld;
  double* G = P + ld;
  double* TMP = G + ld;       // 3 lanes
  double2* WA = reinterpret_cast<double2*>(TMP + 3 * ld + 2);
  WA = reinterpret_cast<double2*>((reinterpret_cast<size_t>(WA) + 15) & ~size_t(15));
  const int wld = c.cy.use_fft ? c.cy.L : 1;
  double2* WB = WA + 2 * wld;
  (void)nx;
  if (PRE) {
    const double* cv = static_cast<const double*>(c.m_cv);
    for (int idx = tid; idx < 3 * ny; idx += nth) {
      int f = idx / ny, k = idx - f * ny;
      CV[f * ld + k] = (i < kx && k < ky) ? cv[((size_t)f * kx + i) * ky + k] : 0.0;
    }
  } else if (i < kx) {
    const double* q = static_cast<const double*>(c.q[0]);
    for (int idx = tid; idx < 3 * ny; idx += nth) {
      int f = idx / ny, k = idx - f * ny;
      TMP[f * ld + k] = q[(size_t)f * kx * ny + (size_t)i * ny + k];
    }
    __syncthreads();
    if (c.cy.use_fft) dct1_fft_r(c.cy, true, TMP, ld, CV, ld, 3, WA, WB, wld, tid, nth);
    else dct1_dense<double>(c.cy, true, TMP, ld, CV, ld, 3, tid, nth);
    for (int idx = tid; idx < 3 * ny; idx += nth) {
      int f = idx / ny, k = idx - f * ny;
      if (k >= ky) CV[f * ld + k] = 0.0;
    }
  } else {
    for (int idx = tid; idx < 3 * ny; idx += nth) CV[(idx / ny) * ld + idx % ny] = 0.0;
  }
  // (Sx f)[i] = diag_i f[i] + low2_{i-2} f[i-2] for composite rows
  void* f3[3] = {c.ux, c.uy, c.temp};
  const BasisDev* xb[3] = {&c.xu, &c.xu, &c.xt};
  for (int idx = tid; idx < 3 * myc; idx += nth) {
    int f = idx / myc, k = idx - f * myc;
    const double* a = static_cast<const double*>(f3[f]);
    const BasisDev& b = *xb[f];
    double v = 0.0;
    bool has = false;
    if (i < mxc) { v = b.unit_diag ? a[(size_t)i * myc + k] : a[(size_t)i * myc + k] * b.diag[i]; has = true; }
    if (i >= 2 && i - 2 < mxc) {
      double t = a[(size_t)(i - 2) * myc + k];
      v = has ? fma(t, b.low2[i - 2], v) : t * b.low2[i - 2];
    }
    SX[f * ld + k] = v;
  }
  const double* p0 = static_cast<const double*>(c.p0);
  for (int k = tid; k < ny; k += nth) P[k] = p0[(size_t)i * ny + k];
  __syncthreads();
  to_ortho<double>(c.ycd, SX, ld, O, ld, 3, tid, nth);
  cheb_diff<double>(P, ld, G, ld, ny, 1, 1, TMP, ld, tid, nth);
  const double* gpx = static_cast<const double*>(c.s[0]);
  const double* bco = static_cast<const double*>(c.bc_ortho);
  const double* bcd = static_cast<const double*>(c.bc_diff);
  for (int k = tid; k < ny; k += nth) {
    R[k] = fnms(fnms(O[k], gpx[(size_t)i * ny + k], dt), CV[k], dt);
    double that = O[2 * ld + k] + bco[(size_t)i * ny + k];
    R[ld + k] = fnms(fmas(fnms(O[ld + k], G[k], dt), that, dt), CV[ld + k], dt);
    double ct = CV[2 * ld + k];
    if (PRE && c.m_bclin && i < kx && k < ky) ct = add_bclin(ct, O[ld + k], c.m_bcg, i);
    R[2 * ld + k] = fnms(O[2 * ld + k] + bcd[(size_t)i * ny + k], ct, dt);
  }
  __syncthreads();
  matvec_pinv<double>(c.pinv_y, R, ld, O, ld, 3, tid, nth);
  for (int idx = tid; idx < 3 * myc; idx += nth) {
    int f = idx / myc, k = idx - f * myc;
    static_cast<double*>(c.s[1 + f])[(size_t)i * myc + k] = O[f * ld + k];
  }
}

size_t smem_box_y2(const CaseDev& c) {
  size_t ld = c.ny + 1;
  size_t wld = c.cy.use_fft ? c.cy.L : 1;
  return 17 * ld * 8 + 2 * 2 * wld * 16 + 64;
}

// X2: columns j < myc.  pinv_x then the ADI x solve.  s[1..3] -> s[4..6] (mxc x myc)
__global__ void __launch_bounds__(256) k_box_x2(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int j = w.y;
  const int nx = c.nx, myc = c.myc, mxc = c.mxc;
  const int ld = nx + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  extern __shared__ double2 smem[];
  double* IN = reinterpret_cast<double*>(smem);
  double* OUT = IN + 3 * ld;
  for (int idx = tid; idx < 3 * nx; idx += nth) {
    int f = idx / nx, k = idx - f * nx;
    IN[f * ld + k] = static_cast<const double*>(c.s[1 + f])[(size_t)k * myc + j];
  }
  __syncthreads();
  matvec_pinv<double>(c.pinv_x, IN, ld, OUT, ld, 3, tid, nth);
  fdma_solve<double>(c.hu_x, OUT, ld, 2, 0, 0, tid, nth);
  fdma_solve<double>(c.ht_x, OUT + 2 * ld, ld, 1, 0, 0, tid, nth);
  for (int idx = tid; idx < 3 * mxc; idx += nth) {
    int f = idx / mxc, k = idx - f * mxc;
    static_cast<double*>(c.s[4 + f])[(size_t)k * myc + j] = OUT[f * ld + k];
  }
}

size_t smem_box_x2(const CaseDev& c) { return 6 * (size_t)(c.nx + 1) * 8 + 64; }

// Y3: rows i < mxc.  ADI y solve -> ux*, uy*, temp(new); A = Sy ux*, B = Dy Sy uy*
__global__ void __launch_bounds__(256) k_box_y3(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int i = w.y;
  const int ny = c.ny, myc = c.myc;
  const int ld = ny + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  extern __shared__ double2 smem[];
  double* F = reinterpret_cast<double*>(smem);
  double* O = F + 3 * ld;
  double* B = O + 2 * ld;
  double* TMP = B + ld;
  for (int idx = tid; idx < 3 * myc; idx += nth) {
    int f = idx / myc, k = idx - f * myc;
    F[f * ld + k] = static_cast<const double*>(c.s[4 + f])[(size_t)i * myc + k];
  }
  __syncthreads();
  fdma_solve<double>(c.hu_y, F, ld, 2, 0, 0, tid, nth);
  fdma_solve<double>(c.ht_y, F + 2 * ld, ld, 1, 0, 0, tid, nth);
  to_ortho<double>(c.ycd, F, ld, O, ld, 2, tid, nth);
  cheb_diff<double>(O + ld, ld, B, ld, ny, 1, 1, TMP, ld, tid, nth);
  // ux*, uy* -> s[4], s[5] (in place);  temp -> state
  bool bad = false;
  double* tt = static_cast<double*>(c.temp);
  for (int idx = tid; idx < 3 * myc; idx += nth) {
    int f = idx / myc, k = idx - f * myc;
    double v = F[f * ld + k];
    if (f < 2) static_cast<double*>(c.s[4 + f])[(size_t)i * myc + k] = v;
    else tt[(size_t)i * myc + k] = v;
    bad |= !isfinite(v);
  }
  double* A = static_cast<double*>(c.s[1]);   // mxc x ny
  double* Bs = static_cast<double*>(c.s[2]);  // mxc x ny
  for (int k = tid; k < ny; k += nth) {
    A[(size_t)i * ny + k] = O[k];
    Bs[(size_t)i * ny + k] = B[k];
  }
  if (bad) flag_nonfinite(c.status);
}

size_t smem_box_y3(const CaseDev& c) { return 8 * (size_t)(c.ny + 1) * 8 + 64; }

// X3: columns j < ny.  div = Dx Sx A / s + Sx B  (-> s[3], nx x ny);
// Zf = fwd * pinv_x div  (-> s[1] reused? no: s[6], mxc x ny)
// MIX: stop after pinv_x and store it (m_z); the eigenbasis product runs as a GEMM.
template <bool MIX>
__global__ void __launch_bounds__(256) k_box_x3(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int j = w.y;
  const int nx = c.nx, ny = c.ny, mxc = c.mxc;
  const int ld = nx + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  const double inv_asp = 1.0 / c.aspect;
  extern __shared__ double2 smem[];
  double* IN = reinterpret_cast<double*>(smem);  // 2 lanes (mxc)
  double* OR = IN + 2 * ld;                      // 2 lanes (nx)
  double* DV = OR + 2 * ld;                      // div lane
  double* Z = DV + ld;                           // pinv lane
  double* TMP = Z + ld;                          // 2 lanes
  const double* A = static_cast<const double*>(c.s[1]);
  const double* B = static_cast<const double*>(c.s[2]);
  for (int k = tid; k < mxc; k += nth) {
    IN[k] = A[(size_t)k * ny + j];
    IN[ld + k] = B[(size_t)k * ny + j];
  }
  __syncthreads();
  to_ortho<double>(c.xu, IN, ld, OR, ld, 2, tid, nth);
  cheb_diff<double>(OR, ld, TMP, ld, nx, 1, 1, TMP + ld, ld, tid, nth);
  double* dv = static_cast<double*>(c.s[3]);
  for (int k = tid; k < nx; k += nth) {
    double v = TMP[k] * inv_asp + OR[ld + k];
    DV[k] = v;
    dv[(size_t)k * ny + j] = v;
  }
  __syncthreads();
  matvec_pinv<double>(c.pinv_x, DV, ld, Z, ld, 1, tid, nth);
  if (MIX) {  // FP32: the input of the eigenbasis GEMM
    float* mz = static_cast<float*>(c.m_z);
    for (int r = tid; r < mxc; r += nth) mz[(size_t)r * ny + j] = (float)Z[r];
    return;
  }
  // dense eigenbasis forward along x
  double* zf = static_cast<double*>(c.s[6]);
  for (int r = tid; r < mxc; r += nth) {
    const double* row = c.pois_fwd + (size_t)r * mxc;
    double acc = 0.0;
    for (int k = 0; k < mxc; k++) acc = fma(__ldg(row + k), Z[k], acc);
    zf[(size_t)r * ny + j] = acc;
  }
}

size_t smem_box_x3(const CaseDev& c) { return 8 * (size_t)(c.nx + 1) * 8 + 64; }

// Y4: rows i < mxc.  pinv_y then the Poisson row solve (eigen row i) -> s[7] (mxc x myc)
// MIX: in FP32 into m_z instead, the input of the eigenbasis GEMM
template <bool MIX>
__global__ void __launch_bounds__(256) k_box_y4(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int i = w.y;
  const int ny = c.ny, myc = c.myc;
  const int ld = ny + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  extern __shared__ double2 smem[];
  double* IN = reinterpret_cast<double*>(smem);
  double* OUT = IN + ld;
  const double* zf = static_cast<const double*>(c.s[6]);
  for (int k = tid; k < ny; k += nth) IN[k] = zf[(size_t)i * ny + k];
  __syncthreads();
  matvec_pinv<double>(c.pinv_y, IN, ld, OUT, ld, 1, tid, nth);
  fdma_solve<double>(c.pois_y, OUT, ld, 1, i, 0, tid, nth);
  if (MIX) {  // FP32 into m_z: the input of the eigenbasis GEMM
    float* wf = static_cast<float*>(c.m_z);
    for (int k = tid; k < myc; k += nth) wf[(size_t)i * myc + k] = (float)OUT[k];
    return;
  }
  double* wv = static_cast<double*>(c.s[7]);
  for (int k = tid; k < myc; k += nth) wv[(size_t)i * myc + k] = OUT[k];
}

size_t smem_box_y4(const CaseDev& c) { return 2 * (size_t)(c.ny + 1) * 8 + 64; }

// X4: columns j < myc.  p1 = bwd * W (p1[0][0] = 0).  E = Sx+ Dx Sx^N p1 / s,
// Fv = Sx+ Sx^N p1 (-> s[1], s[2] as mxc x myc), Gp = Sx^N p1 (-> s[0], nx x myc)
// MIX: p1 = bwd * W was computed by a GEMM; read it (and set p1[0][0] = 0).
template <bool MIX>
__global__ void __launch_bounds__(256) k_box_x4(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int j = w.y;
  const int nx = c.nx, myc = c.myc, mxc = c.mxc;
  const int ld = nx + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  const double inv_asp = 1.0 / c.aspect;
  extern __shared__ double2 smem[];
  double* W = reinterpret_cast<double*>(smem);
  double* PV = W + ld;
  double* OR = PV + ld;       // Sx^N p1 (nx)
  double* D = OR + ld;        // 2 lanes: Dx OR / s, OR copy
  double* FO = D + 2 * ld;    // 2 lanes from_ortho
  double* TMP = FO + 2 * ld;  // 2 lanes
  double* p1 = static_cast<double*>(c.p1);
  if (MIX) {
    for (int r = tid; r < mxc; r += nth) {
      double v = p1[(size_t)r * myc + j];
      if (j == 0 && r == 0) {
        v = 0.0;
        p1[0] = 0.0;
      }
      PV[r] = v;
    }
  } else {
    const double* wv = static_cast<const double*>(c.s[7]);
    for (int k = tid; k < mxc; k += nth) W[k] = wv[(size_t)k * myc + j];
    __syncthreads();
    for (int r = tid; r < mxc; r += nth) {
      const double* row = c.pois_bwd + (size_t)r * mxc;
      double acc = 0.0;
      for (int k = 0; k < mxc; k++) acc = fma(__ldg(row + k), W[k], acc);
      if (j == 0 && r == 0) acc = 0.0;
      PV[r] = acc;
      p1[(size_t)r * myc + j] = acc;
    }
  }
  __syncthreads();
  to_ortho<double>(c.xp, PV, ld, OR, ld, 1, tid, nth);
  cheb_diff<double>(OR, ld, TMP, ld, nx, 1, 1, TMP + ld, ld, tid, nth);
  double* gp = static_cast<double*>(c.s[0]);
  for (int k = tid; k < nx; k += nth) {
    D[k] = TMP[k] * inv_asp;
    D[ld + k] = OR[k];
    gp[(size_t)k * myc + j] = OR[k];
  }
  __syncthreads();
  from_ortho<double>(c.xu, D, ld, FO, ld, 2, tid, nth);
  double* e = static_cast<double*>(c.s[1]);
  double* fv = static_cast<double*>(c.s[2]);
  for (int k = tid; k < mxc; k += nth) {
    e[(size_t)k * myc + j] = FO[k];
    fv[(size_t)k * myc + j] = FO[ld + k];
  }
}

size_t smem_box_x4(const CaseDev& c) { return 9 * (size_t)(c.nx + 1) * 8 + 64; }

// Y5: rows i < nx.  ux = ux* - Sy+ Sy^N E ; uy = uy* - Sy+ Dy Sy^N Fv ;
// p0 = (p0 - nu div) + Sy^N Gp / dt
__global__ void __launch_bounds__(256) k_box_y5(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int i = w.y;
  const int ny = c.ny, myc = c.myc, mxc = c.mxc;
  const int ld = ny + 1;
  const int tid = threadIdx.x, nth = blockDim.x;
  extern __shared__ double2 smem[];
  double* IN = reinterpret_cast<double*>(smem);  // 3 lanes (myc): E, Fv, Gp
  double* OR = IN + 3 * ld;                      // 3 lanes
  double* D = OR + 3 * ld;                       // 2 lanes: dpdx, dpdy
  double* FO = D + 2 * ld;                       // 2 lanes
  double* TMP = FO + 2 * ld;
  const double* e = static_cast<const double*>(c.s[1]);
  const double* fv = static_cast<const double*>(c.s[2]);
  const double* gp = static_cast<const double*>(c.s[0]);
  for (int k = tid; k < myc; k += nth) {
    if (i < mxc) {
      IN[k] = e[(size_t)i * myc + k];
      IN[ld + k] = fv[(size_t)i * myc + k];
    }
    IN[2 * ld + k] = gp[(size_t)i * myc + k];
  }
  __syncthreads();
  if (i < mxc) {
    to_ortho<double>(c.ycn, IN, ld, OR, ld, 2, tid, nth);
    cheb_diff<double>(OR + ld, ld, D + ld, ld, ny, 1, 1, TMP, ld, tid, nth);
    for (int k = tid; k < ny; k += nth) D[k] = OR[k];
    __syncthreads();
    from_ortho<double>(c.ycd, D, ld, FO, ld, 2, tid, nth);
    double* ux = static_cast<double*>(c.ux);
    double* uy = static_cast<double*>(c.uy);
    const double* us = static_cast<const double*>(c.s[4]);
    const double* vs = static_cast<const double*>(c.s[5]);
    bool bad = false;
    for (int k = tid; k < myc; k += nth) {
      double a = us[(size_t)i * myc + k] - FO[k];
      double b = vs[(size_t)i * myc + k] - FO[ld + k];
      ux[(size_t)i * myc + k] = a;
      uy[(size_t)i * myc + k] = b;
      bad |= !(isfinite(a) && isfinite(b));
    }
    if (bad) flag_nonfinite(c.status);
  }
  to_ortho<double>(c.ycn, IN + 2 * ld, ld, OR + 2 * ld, ld, 1, tid, nth);
  double* p0 = static_cast<double*>(c.p0);
  const double* dv = static_cast<const double*>(c.s[3]);
  for (int k = tid; k < ny; k += nth) {
    double v = fnms(p0[(size_t)i * ny + k], dv[(size_t)i * ny + k], c.nu);
    p0[(size_t)i * ny + k] = fmas(v, OR[2 * ld + k], c.inv_dt);
  }
}

size_t smem_box_y5(const CaseDev& c) { return 12 * (size_t)(c.ny + 1) * 8 + 64; }

}  // namespace dev

// ---------------------------------------------------------------------------
// host-side launch helpers
// ---------------------------------------------------------------------------
static inline size_t clamp_smem(size_t s) { return (s + 127) & ~size_t(127); }

cudaError_t configure_step_kernels() {
  static PerDeviceFlag done;
  if (done.test()) return cudaSuccess;
  const int big = (int)smem_limit();
  cudaError_t e;
#define SET_ATTR(k)                                                                          \
  e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, big);             \
  if (e != cudaSuccess) return e;
  SET_ATTR(dev::k_y1<double>);
  SET_ATTR(dev::k_y1<double2>);
  SET_ATTR(dev::k_per_x);
  SET_ATTR(dev::k_per_y2<false>);
  SET_ATTR(dev::k_per_y2<true>);
  SET_ATTR(dev::k_per_y2a);
  SET_ATTR(dev::k_per_y2b);
  SET_ATTR(dev::k_box_x1);
  SET_ATTR(dev::k_box_y2<false>);
  SET_ATTR(dev::k_box_y2<true>);
  SET_ATTR(dev::k_box_x2);
  SET_ATTR(dev::k_box_gpx);
  SET_ATTR(dev::k_box_y3);
  SET_ATTR(dev::k_box_x3<false>);
  SET_ATTR(dev::k_box_x3<true>);
  SET_ATTR(dev::k_box_y4<false>);
  SET_ATTR(dev::k_box_y4<true>);
  SET_ATTR(dev::k_box_x4<false>);
  SET_ATTR(dev::k_box_x4<true>);
  SET_ATTR(dev::k_box_y5);
#undef SET_ATTR
  done.set();
  return cudaSuccess;
}

StepPlan build_step_plan(const CaseDev& c) {
  StepPlan p;
  bool per = c.kind == KIND_PERIODIC;
  auto add = [&](int kernel, int lanes, size_t smem) {
    StepLaunch L;
    L.kernel = kernel;
    L.smem = clamp_smem(smem);
    for (int i = 0; i < lanes; i++) L.items.push_back(make_int4(0, i, 1, 0));
    p.launches.push_back(L);
  };
  if (per) {
    add(K_Y1_C, c.mxc, dev::smem_y1(c, 1, true));
    add(K_PER_X, c.ny, dev::smem_per_x(c));
    // fused Y2 (one CTA per row): faster than the split Y2a/Y2b pair on this
    // GPU because each FP64 warp instruction costs its warp ~64 cycles and the
    // split leaves single-lane CTAs with long per-warp FP64 chains
    add(K_PER_Y2, c.mx, dev::smem_per_y2(c));
  } else {
    add(K_Y1_R, c.mxc, dev::smem_y1(c, 1, false));
    add(K_BOX_X1, c.ny, dev::smem_box_x1(c));
    add(K_BOX_Y2, c.nx, dev::smem_box_y2(c));
    add(K_BOX_X2, c.myc, dev::smem_box_x2(c));
    add(K_BOX_Y3, c.mxc, dev::smem_box_y3(c));
    add(K_BOX_X3, c.ny, dev::smem_box_x3(c));
    add(K_BOX_Y4, c.mxc, dev::smem_box_y4(c));
    add(K_BOX_X4, c.myc, dev::smem_box_x4(c));
    add(K_BOX_Y5, c.nx, dev::smem_box_y5(c));
  }
  return p;
}

cudaError_t launch_step_kernel(int kernel, int nblocks, size_t smem, cudaStream_t s, const CaseDev* cases,
                               const int4* work) {
  dim3 g(nblocks), b(256);
  switch (kernel) {
    case K_Y1_C: dev::k_y1<double2><<<g, b, smem, s>>>(cases, work); break;
    case K_Y1_R: dev::k_y1<double><<<g, b, smem, s>>>(cases, work); break;
    case K_PER_X: dev::k_per_x<<<g, b, smem, s>>>(cases, work); break;
    case K_PER_Y2: dev::k_per_y2<false><<<g, b, smem, s>>>(cases, work); break;
    case K_PER_Y2_PRE: dev::k_per_y2<true><<<g, b, smem, s>>>(cases, work); break;
    case K_PER_Y2A: dev::k_per_y2a<<<g, b, smem, s>>>(cases, work); break;
    case K_PER_Y2B: dev::k_per_y2b<<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_X1: dev::k_box_x1<<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_Y2: dev::k_box_y2<false><<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_Y2_PRE: dev::k_box_y2<true><<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_X2: dev::k_box_x2<<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_GPX: dev::k_box_gpx<<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_Y3: dev::k_box_y3<<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_X3: dev::k_box_x3<false><<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_X3_MIX: dev::k_box_x3<true><<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_Y4: dev::k_box_y4<false><<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_Y4_MIX: dev::k_box_y4<true><<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_X4: dev::k_box_x4<false><<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_X4_MIX: dev::k_box_x4<true><<<g, b, smem, s>>>(cases, work); break;
    case K_BOX_Y5: dev::k_box_y5<<<g, b, smem, s>>>(cases, work); break;
    case K_PER_Y2_PRE_T128: dev::k_per_y2<true><<<g, dim3(128), smem, s>>>(cases, work); break;
    case K_BOX_Y2_PRE_T128: dev::k_box_y2<true><<<g, dim3(128), smem, s>>>(cases, work); break;
    case K_BOX_X3_MIX_T128: dev::k_box_x3<true><<<g, dim3(128), smem, s>>>(cases, work); break;
    case K_BOX_Y5_T128: dev::k_box_y5<<<g, dim3(128), smem, s>>>(cases, work); break;
    default: return launch_mixed_kernel(kernel, nblocks, smem, s, cases, work);
  }
  return cudaGetLastError();
}

}  // namespace rbc
