// step_mixed.cu -- the mixed-precision Rayleigh-Benard step.
//
// Same pass structure as the FP64 step (step_fp64.cu), with the work split by
// the arithmetic each part needs:
//   * dense operators along a lane (stencil + derivative + Chebyshev
//     transform compositions) run on the tensor cores as 3xTF32 lane GEMMs
//     (lane_gemm.cu);
//   * the convection products and the Fourier transforms around them run in
//     FP32 (lane_ops_f32.cuh);
//   * the banded Helmholtz / Poisson sweeps, the pressure projection, the
//     divergence correction and the update of the spectral state stay FP64
//     (the FP64 lane kernels, fed the convection term already transformed).
//
//  periodic:  G1 (y, GEMM) -> X (FP32) -> G2 (y, GEMM) -> Y2 (FP64)
#include "lane_ops.cuh"
#include "lane_ops_f32.cuh"
#include "per_device.h"
#include "prims.h"
#include "step_fp64.h"

#include <algorithm>
#include <cstring>

namespace rbc {
namespace dev {

// ============================================================================
// Periodic X pass in FP32: column j of the transposed y-pass outputs.
//  u = F^-1 Y0_ux, v = F^-1 Y0_uy;  for f: a = F^-1 (ik/s Y0_f), b = F^-1 Y1_f
//  P_f = u a + v b (+ u dbc/dx + v (dbc/dy - g0) for temp; the Y2 pass adds the
//  g0 v part in FP64);  Q_f = F P_f, rows < kx
// (navier.rs:538-616, conv_term.rs:22-42)
// ============================================================================
__global__ void __launch_bounds__(256) k_per_x_mixed(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  const int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int j = w.y;
  const int mx = c.mx, nx = c.nx, ny = c.ny, M = c.fx.M, kx = c.kx;
  const int tid = threadIdx.x, nth = blockDim.x;
  const float inv_asp = (float)(1.0 / c.aspect);
  extern __shared__ float2 smf[];
  const int ild = mx + 1;
  float2* IN = smf;          // 8 input lanes
  float2* WA = IN + 8 * ild;  // 8 FFT work lanes of M
  float2* WB = WA + 8 * M;
  float* PH = reinterpret_cast<float*>(IN);  // 8 physical lanes of nx (alias the inputs)
  // lane order: Y0u, Y0v, ikY0u, Y1u, ikY0v, Y1v, ikY0t, Y1t
  for (int idx = tid; idx < 8 * mx; idx += nth) {
    const int l = idx / mx, k = idx - l * mx;
    int f, y1, ik;
    if (l < 2) { f = l; y1 = 0; ik = 0; }
    else { f = (l - 2) >> 1; y1 = l & 1; ik = !(l & 1); }
    const float2* src = static_cast<const float2*>(c.m_y[f]);
    float2 v = src[(size_t)(y1 ? ny + j : j) * mx + k];
    if (ik) {
      const float kk = (float)k * inv_asp;
      v = f2(-v.y * kk, v.x * kk);
    }
    IN[l * ild + k] = v;
  }
  __syncthreads();
  c2r_f(c.fx, IN, ild, 1, PH, nx, 8, WA, WB, M, tid, nth);
  const float* bx = c.m_bcx + (size_t)j * nx;
  const float* by = c.m_bcy + (size_t)j * nx;
  for (int idx = tid; idx < 3 * nx; idx += nth) {
    const int f = idx / nx, x = idx - f * nx;
    const float u = PH[x], v = PH[nx + x];
    float p = u * PH[(2 + 2 * f) * nx + x] + v * PH[(3 + 2 * f) * nx + x];
    if (f == 2) p += u * bx[x] + v * by[x];
    PH[(2 + 2 * f) * nx + x] = p;
  }
  __syncthreads();
  float2* q = static_cast<float2*>(c.m_q);
  r2c_f(c.fx, PH + 2 * nx, 2 * nx, q + (size_t)j * kx, ny * kx, 1, kx, 3, WA, WB, M, tid, nth);
}

// ============================================================================
// Box products in FP32 (one y index n per CTA, transposed physical arrays):
//   P_u = u du/dx + v du/dy,  P_v = u dv/dx + v dv/dy,
//   P_t = u dT/dx + v dT/dy + u dbc/dx + v (dbc/dy - g0)   (navier.rs:538-616;
//   the y2 pass adds the g0 v part in FP64)
// m_ph: 0 [u | du/dx], 1 [v | dv/dx] (ny x 2nx), 2 du/dy, 3 dv/dy, 4 dT/dx,
// 5 dT/dy (ny x nx).  m_p[f]: ny x nx.
// ============================================================================
__global__ void __launch_bounds__(256) k_box_prod_mixed(const CaseDev* __restrict__ cases,
                                                        const int4* __restrict__ work) {
  const int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;  // case idle this step (serving)
  const int n = w.y, nx = c.nx;
  const float* pu = static_cast<const float*>(c.m_ph[0]) + (size_t)n * 2 * nx;
  const float* pv = static_cast<const float*>(c.m_ph[1]) + (size_t)n * 2 * nx;
  const size_t o = (size_t)n * nx;
  const float* dyu = static_cast<const float*>(c.m_ph[2]) + o;
  const float* dyv = static_cast<const float*>(c.m_ph[3]) + o;
  const float* dxt = static_cast<const float*>(c.m_ph[4]) + o;
  const float* dyt = static_cast<const float*>(c.m_ph[5]) + o;
  const float* bx = c.m_bcx + o;
  const float* by = c.m_bcy + o;
  float* p0 = static_cast<float*>(c.m_p[0]) + o;
  float* p1 = static_cast<float*>(c.m_p[1]) + o;
  float* p2 = static_cast<float*>(c.m_p[2]) + o;
  for (int x = threadIdx.x; x < nx; x += blockDim.x) {
    const float u = pu[x], dxu = pu[nx + x], v = pv[x], dxv = pv[nx + x];
    p0[x] = u * dxu + v * dyu[x];
    p1[x] = u * dxv + v * dyv[x];
    p2[x] = u * dxt[x] + v * dyt[x] + u * bx[x] + v * by[x];
  }
}

// Serving gate: for each member case decide whether it advances in this step
// (steps left > 0) and count the step down.
__global__ void k_gate(const CaseDev* __restrict__ cases, const int* __restrict__ members, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int* g = cases[members[i]].gate;
  if (g == nullptr) return;
  const int run = g[0] > 0 ? 1 : 0;
  g[1] = run;
  g[0] -= run;
}

// FP32 copy of row i of ux, uy, temp (the y GEMM's input, rounded once here
// instead of once per output tile inside the GEMM; the GEMM rounds FP64 input
// to FP32 the same way)
__global__ void __launch_bounds__(128) k_state_f32(const CaseDev* __restrict__ cases, const int4* __restrict__ work) {
  const int4 w = work[blockIdx.x];
  const CaseDev& c = cases[w.x];
  if (c.gate != nullptr && c.gate[1] == 0) return;
  const int i = w.y;
  const int myc = c.myc, mp = pad4(myc);
  const bool per = c.kind == KIND_PERIODIC;
  const size_t rl = (size_t)myc * (per ? 2 : 1);  // doubles per state row
  const size_t ld = (size_t)s32_row_floats(c);    // floats per FP32 row
  const size_t fs = (size_t)c.mxc * ld;
  const double* src[3] = {static_cast<const double*>(c.ux), static_cast<const double*>(c.uy),
                          static_cast<const double*>(c.temp)};
  float* dst = static_cast<float*>(c.m_s32);
  // a complex row (re, im interleaved) is split into its [re | im] parts
  for (int f = 0; f < 3; f++)
    for (size_t k = threadIdx.x; k < rl; k += blockDim.x) {
      const size_t o = per ? (k & 1) * mp + (k >> 1) : k;
      dst[f * fs + i * ld + o] = (float)src[f][i * rl + k];
    }
}

size_t smem_per_x_mixed(const CaseDev& c) {
  return ((size_t)8 * (c.mx + 1) + (size_t)16 * c.fx.M) * 8 + 64;
}

}  // namespace dev

// ---------------------------------------------------------------------------
// plan of the mixed-precision step
// ---------------------------------------------------------------------------
static inline size_t clamp_smem_m(size_t s) { return (s + 127) & ~size_t(127); }

StepPlan build_mixed_plan(const CaseDev& c, const MixedOps& ops, int variant) {
  const bool lane_parallel = variant != 0;  // 128-thread or one-thread-per-lane forms
  const bool lp = variant >= 2;             // one-thread-per-lane forms wherever they exist
  const bool fused = variant == 3;          // ... with the periodic Y2 launches fused into one
  StepPlan p;
  // pass ids: one per pass, the same in every variant; `group` >= 0 gives the
  // following launches one shared id (a pass made of several launches)
  int npass = 0, group = -1;
  auto push = [&](StepLaunch& L) {
    L.pass = group >= 0 ? group : npass++;
    p.launches.push_back(L);
  };
  auto add = [&](int kernel, int lanes, size_t smem) {
    StepLaunch L;
    L.kernel = kernel;
    L.smem = clamp_smem_m(smem);
    for (int i = 0; i < lanes; i++) L.items.push_back(make_int4(0, i, 1, 0));
    push(L);
  };
  // one-thread-per-lane kernel: items of lane_item_lanes() consecutive lanes
  // of length `len` (item.w = the item's cost, lanes x len)
  auto add_lp = [&](int kernel, int lanes, int len) {
    StepLaunch L;
    L.kernel = kernel;
    L.smem = 0;
    const int per = lane_item_lanes(kernel);
    for (int i = 0; i < lanes; i += per) {
      const int n = std::min(per, lanes - i);
      L.items.push_back(make_int4(0, i, n, n * len));
    }
    push(L);
  };
  auto add_gemm = [&](const GemmJobDev& j) {
    StepLaunch L;
    L.kernel = K_GEMM;
    L.gemm_ws = ops.ws;
    L.smem = ops.ws ? gemm_ws_smem_bytes(j.NT) : gemm_smem_bytes(j.NT);
    L.jobs.push_back(j);
    push(L);
  };
  const int mx = c.mx, ny = c.ny, myc = c.myc, kx = c.kx, ky = c.ky;
  // FP32 copy of the state rows, read by G1 (rows of s32_row_floats floats)
  const int s32ld = s32_row_floats(c);
  void* s32[3];
  for (int f = 0; f < 3; f++) s32[f] = static_cast<float*>(c.m_s32) + (size_t)f * c.mxc * s32ld;
  add(K_STATE_F32, c.mxc, 0);
  if (c.kind == KIND_PERIODIC) {
    // G1: rows of ux, uy, temp (complex, [re | im] parts) -> [Y0 | Y1] (FP32), stored transposed
    LaneSideDev in = lane_rows(s32, 3, mx, myc, s32ld / 2, LT_F32, true);
    in.elem_stride = 1;
    in.part_stride = s32ld / 2;
    LaneSideDev out;
    std::memset(&out, 0, sizeof out);
    for (int f = 0; f < 3; f++) out.ptr[f] = c.m_y[f];
    out.nf = 3; out.rows = mx; out.parts = 2; out.type = LT_F32;
    out.lane_stride = 2; out.part_stride = 1; out.elem_stride = 2LL * mx; out.len = 2 * ny; out.lane_fast = 1;
    add_gemm(make_gemm_job(in, out, ops.y1, myc, 2 * ny, 1.0, c.status, ops.ntmax));
    // X: FP32 convection, one CTA per column (256 threads, or 128 in the batch forms)
    add(lane_parallel ? K_PER_X_MIXED_T128 : K_PER_X_MIXED, ny, dev::smem_per_x_mixed(c));
    // G2: y transform of the x-transformed products (FP32, transposed) -> m_cv (FP64)
    LaneSideDev qi;
    std::memset(&qi, 0, sizeof qi);
    for (int f = 0; f < 3; f++) qi.ptr[f] = static_cast<float2*>(c.m_q) + (size_t)f * ny * kx;
    qi.nf = 3; qi.rows = kx; qi.parts = 2; qi.type = LT_F32;
    qi.lane_stride = 2; qi.part_stride = 1; qi.elem_stride = 2LL * kx; qi.len = ny; qi.lane_fast = 1;
    void* cvp[3];
    for (int f = 0; f < 3; f++) cvp[f] = static_cast<double2*>(c.m_cv) + (size_t)f * kx * ky;
    LaneSideDev co = lane_rows(cvp, 3, kx, ky, ky, LT_F64, true);
    add_gemm(make_gemm_job(qi, co, ops.y2, ny, ky, 1.0, c.status, ops.ntmax));
    // Y2: FP64 right-hand sides, banded solves, projection, pressure update:
    // one CTA per row (256 or 128 threads), or three launches of one thread
    // per (field, parity) sub-lane, or those three phases in one launch
    if (lp) {
      group = npass++;
      if (fused) {
        add_lp(K_LP_PER_Y2F, mx, ny);
      } else {
        add_lp(K_LP_PER_Y2A, mx, ny);
        add_lp(K_LP_PER_Y2B, mx, ny);
        add_lp(K_LP_PER_Y2C, mx, ny);
      }
      group = -1;
    } else {
      add(lane_parallel ? K_PER_Y2_PRE_T128 : K_PER_Y2_PRE, mx, dev::smem_per_y2_pre(c));
    }
    return p;
  }
  // ---- box
  const int nx = c.nx, mxc = c.mxc;
  auto side = [](void* const* ptrs, int nf, int rows, int len, long long lane_stride, long long elem_stride,
                 int type, int lane_fast) {
    LaneSideDev sd;
    std::memset(&sd, 0, sizeof sd);
    for (int f = 0; f < nf; f++) sd.ptr[f] = ptrs[f];
    sd.nf = nf; sd.rows = rows; sd.parts = 1; sd.type = type; sd.len = len;
    sd.lane_stride = lane_stride; sd.elem_stride = elem_stride; sd.lane_fast = lane_fast;
    return sd;
  };
  auto fptr = [](void* base, size_t off_floats) { return static_cast<void*>(static_cast<float*>(base) + off_floats); };
  // G1: rows of ux, uy, temp (FP32 copy, mxc rows of myc) -> [Y0 | Y1] transposed (2 ny rows of
  // mxc values, row stride pad4(mxc), FP32)
  const int myld = pad4(mxc);
  {
    void* yo[3] = {c.m_y[0], c.m_y[1], c.m_y[2]};
    add_gemm(make_gemm_job(lane_rows(s32, 3, mxc, myc, s32ld, LT_F32, false),
                           side(yo, 3, mxc, 2 * ny, 1, myld, LT_F32, 1), ops.y1, myc, 2 * ny, 1.0, c.status, ops.ntmax));
  }
  // GX: x stencils, derivatives and backward transforms -> physical (transposed), one launch of 4 jobs
  {
    StepLaunch L;
    L.kernel = K_GEMM;
    L.pass = npass++;
    void* a_in[2] = {c.m_y[0], c.m_y[1]};
    void* a_out[2] = {c.m_ph[0], c.m_ph[1]};
    L.jobs.push_back(make_gemm_job(lane_rows(a_in, 2, ny, mxc, myld, LT_F32, false),
                                   lane_rows(a_out, 2, ny, 2 * nx, 2 * nx, LT_F32, false), ops.xa, mxc, 2 * nx, 1.0,
                                   c.status, ops.ntmax));
    void* b_in[2] = {fptr(c.m_y[0], (size_t)ny * myld), fptr(c.m_y[1], (size_t)ny * myld)};
    void* b_out[2] = {c.m_ph[2], c.m_ph[3]};
    L.jobs.push_back(make_gemm_job(lane_rows(b_in, 2, ny, mxc, myld, LT_F32, false),
                                   lane_rows(b_out, 2, ny, nx, nx, LT_F32, false), ops.xb, mxc, nx, 1.0, c.status, ops.ntmax));
    void* c_in[1] = {c.m_y[2]};
    void* c_out[1] = {c.m_ph[4]};
    L.jobs.push_back(make_gemm_job(lane_rows(c_in, 1, ny, mxc, myld, LT_F32, false),
                                   lane_rows(c_out, 1, ny, nx, nx, LT_F32, false), ops.xc, mxc, nx, 1.0, c.status, ops.ntmax));
    void* d_in[1] = {fptr(c.m_y[2], (size_t)ny * myld)};
    void* d_out[1] = {c.m_ph[5]};
    L.jobs.push_back(make_gemm_job(lane_rows(d_in, 1, ny, mxc, myld, LT_F32, false),
                                   lane_rows(d_out, 1, ny, nx, nx, LT_F32, false), ops.xd, mxc, nx, 1.0, c.status, ops.ntmax));
    size_t sm = 0;
    for (const GemmJobDev& j : L.jobs) sm = std::max(sm, ops.ws ? gemm_ws_smem_bytes(j.NT) : gemm_smem_bytes(j.NT));
    L.smem = sm;
    L.gemm_ws = ops.ws;
    p.launches.push_back(L);
  }
  // products (FP32)
  add(K_BOX_PROD_MIXED, ny, 0);
  // GX2: forward x transform of the products, rows < kx -> G (kx x ny per field, FP32)
  {
    void* pin[3] = {c.m_p[0], c.m_p[1], c.m_p[2]};
    void* gout[3];
    for (int f = 0; f < 3; f++) gout[f] = fptr(c.m_q, (size_t)f * kx * ny);
    add_gemm(make_gemm_job(lane_rows(pin, 3, ny, nx, nx, LT_F32, false), side(gout, 3, ny, kx, 1, ny, LT_F32, 1),
                           ops.x2, nx, kx, 1.0, c.status, ops.ntmax));
  }
  // GY2: forward y transform, columns < ky -> m_cv (FP64, kx x ky per field)
  {
    void* gin[3];
    void* cvp[3];
    for (int f = 0; f < 3; f++) {
      gin[f] = fptr(c.m_q, (size_t)f * kx * ny);
      cvp[f] = static_cast<double*>(c.m_cv) + (size_t)f * kx * ky;
    }
    add_gemm(make_gemm_job(lane_rows(gin, 3, kx, ny, ny, LT_F32, false), lane_rows(cvp, 3, kx, ky, ky, LT_F64, false),
                           ops.y2, ny, ky, 1.0, c.status, ops.ntmax));
  }
  // FP64: pressure gradient, Helmholtz (ADI), divergence, Poisson, projection.
  // Each pass has up to three forms: a CTA per lane (variant 0), the same
  // kernel with 128 threads (variant 1, where it exists; otherwise the lane
  // form) and one thread per (field, parity) sub-lane (variant 2, where it
  // exists; variant 3 differs from it in the periodic Y2 pass alone);
  // rbc_batch_create times the forms of every pass on the batch and keeps the
  // fastest.
  if (lane_parallel) add_lp(K_LP_BOX_GPX, ny, nx);
  else add(K_BOX_GPX, ny, dev::smem_box_gpx(c));
  if (lp) add_lp(K_LP_BOX_Y2, nx, ny);
  else add(lane_parallel ? K_BOX_Y2_PRE_T128 : K_BOX_Y2_PRE, nx, dev::smem_box_y2(c));
  if (lane_parallel) {
    add_lp(K_LP_BOX_X2, myc, mxc);
    add_lp(K_LP_BOX_Y3, mxc, ny);
  } else {
    add(K_BOX_X2, myc, dev::smem_box_x2(c));
    add(K_BOX_Y3, mxc, dev::smem_box_y3(c));
  }
  if (lp) add_lp(K_LP_BOX_X3, ny, nx);
  else add(lane_parallel ? K_BOX_X3_MIX_T128 : K_BOX_X3_MIX, ny, dev::smem_box_x3(c));
  {  // eigenbasis forward along x: s[6] = fwd * m_z (columns j < ny)
    void* zi[1] = {c.m_z};
    void* zo[1] = {c.s[6]};
    add_gemm(make_gemm_job(lane_cols(zi, 1, ny, mxc, ny, LT_F32, 0), lane_cols(zo, 1, ny, mxc, ny, LT_F64, 0), ops.pf,
                           mxc, mxc, 1.0, c.status, ops.ntmax));
  }
  if (lane_parallel) add_lp(K_LP_BOX_Y4, mxc, ny);
  else add(K_BOX_Y4_MIX, mxc, dev::smem_box_y4(c));
  {  // eigenbasis backward along x: p1 = bwd * W (FP32 Poisson row solutions in m_z, columns j < myc)
    void* wi[1] = {c.m_z};
    void* po[1] = {c.p1};
    add_gemm(make_gemm_job(lane_cols(wi, 1, myc, mxc, myc, LT_F32, 0), lane_cols(po, 1, myc, mxc, myc, LT_F64, 0),
                           ops.pb, mxc, mxc, 1.0, c.status, ops.ntmax));
  }
  if (lane_parallel) add_lp(K_LP_BOX_X4, myc, nx);
  else add(K_BOX_X4_MIX, myc, dev::smem_box_x4(c));
  if (lp) add_lp(K_LP_BOX_Y5, nx, ny);
  else add(lane_parallel ? K_BOX_Y5_T128 : K_BOX_Y5, nx, dev::smem_box_y5(c));
  return p;
}

// Largest dynamic shared memory of the CTA passes of build_mixed_plan(c, ops,
// 0) (its other variants use less), from the sizes and transform forms alone;
// *kernel receives that pass.  The lane kernels and the GEMMs use none or a
// fixed amount.
size_t mixed_plan_smem(const CaseDev& c, int* kernel) {
  std::vector<std::pair<int, size_t>> k;
  if (c.kind == KIND_PERIODIC) {
    k = {{K_PER_X_MIXED, dev::smem_per_x_mixed(c)}, {K_PER_Y2_PRE, dev::smem_per_y2_pre(c)}};
  } else {
    k = {{K_BOX_GPX, dev::smem_box_gpx(c)}, {K_BOX_Y2_PRE, dev::smem_box_y2(c)}, {K_BOX_X2, dev::smem_box_x2(c)},
         {K_BOX_Y3, dev::smem_box_y3(c)},  {K_BOX_X3_MIX, dev::smem_box_x3(c)}, {K_BOX_Y4_MIX, dev::smem_box_y4(c)},
         {K_BOX_X4_MIX, dev::smem_box_x4(c)}, {K_BOX_Y5, dev::smem_box_y5(c)}};
  }
  size_t m = 0;
  for (const auto& e : k)
    if (clamp_smem_m(e.second) > m) { m = clamp_smem_m(e.second); *kernel = e.first; }
  return m;
}

cudaError_t configure_mixed_kernels() {
  static PerDeviceFlag done;
  if (done.test()) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(dev::k_per_x_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem_limit());
  if (e != cudaSuccess) return e;
  e = configure_gemm_kernels();
  if (e == cudaSuccess) done.set();
  return e;
}

cudaError_t launch_mixed_kernel(int kernel, int nblocks, size_t smem, cudaStream_t s, const CaseDev* cases,
                                const int4* work) {
  switch (kernel) {
    case K_PER_X_MIXED: dev::k_per_x_mixed<<<nblocks, 256, smem, s>>>(cases, work); break;
    case K_STATE_F32: dev::k_state_f32<<<nblocks, 128, 0, s>>>(cases, work); break;
    case K_PER_X_MIXED_T128: dev::k_per_x_mixed<<<nblocks, 128, smem, s>>>(cases, work); break;
    case K_BOX_PROD_MIXED: dev::k_box_prod_mixed<<<nblocks, 256, 0, s>>>(cases, work); break;
    default: return launch_lane_kernel(kernel, nblocks, s, cases, work);
  }
  return cudaGetLastError();
}

// Algorithmic HBM bytes of one launch: every array the launch must read or
// write, counted once (operator tables and the boundary-field constants
// included; re-reads from L2 and shared memory are not).
double launch_algorithmic_bytes(const StepLaunch& L, const CaseDev* cases) {
  if (L.kernel == K_GEMM) {
    double b = 0;
    for (const GemmJobDev& j : L.jobs) {
      const double ie = j.in.type == LT_F64 ? 8 : 4, oe = j.out.type == LT_F64 ? 8 : 4;
      b += (double)j.lanes * ((double)j.K * ie + (double)j.N * oe);
      b += (double)j.ntiles * j.kchunks * 2.0 * j.NT * kGemmKC * 4;  // split operator
    }
    return b;
  }
  double b = 0;
  for (const int4& it : L.items) {
    const CaseDev& c = cases[it.x];
    const double nx = c.nx, ny = c.ny, mx = c.mx, mxc = c.mxc, myc = c.myc, kx = c.kx, ky = c.ky;
    const double z = c.kind == KIND_PERIODIC ? 16 : 8;  // spectral element
    const double lanes = it.z > 0 ? it.z : 1;
    double v = 0;
    int kernel = L.kernel;
    // box y4 of the mixed form also writes the solution's FP32 copy (the
    // eigenbasis GEMM's input)
    if (kernel == K_LP_BOX_Y4 || kernel == K_BOX_Y4_MIX) v += myc * 4;
    switch (kernel) {  // the one-thread-per-lane kernels move the same arrays
      case K_LP_BOX_GPX: kernel = K_BOX_GPX; break;
      case K_LP_BOX_X2: kernel = K_BOX_X2; break;
      case K_LP_BOX_X3: kernel = K_BOX_X3_MIX; break;
      case K_LP_BOX_X4: kernel = K_BOX_X4_MIX; break;
      case K_LP_BOX_Y2: kernel = K_BOX_Y2_PRE; break;
      case K_LP_BOX_Y3: kernel = K_BOX_Y3; break;
      case K_LP_BOX_Y4: case K_BOX_Y4_MIX: kernel = K_BOX_Y4; break;
      case K_LP_BOX_Y5: kernel = K_BOX_Y5; break;
      case K_LP_PER_Y2: kernel = K_PER_Y2_PRE; break;
      case K_PER_Y2_PRE_T128: kernel = K_PER_Y2_PRE; break;
      case K_LP_PER_Y2B: case K_LP_PER_Y2C: kernel = -1; break;  // counted with Y2A
      case K_PER_X_MIXED_T128: kernel = K_PER_X_MIXED; break;
      case K_BOX_Y2_PRE_T128: kernel = K_BOX_Y2_PRE; break;
      case K_BOX_X3_MIX_T128: kernel = K_BOX_X3_MIX; break;
      case K_BOX_Y5_T128: kernel = K_BOX_Y5; break;
      default: break;
    }
    switch (kernel) {
      case K_Y1_C: case K_Y1_R: v = 3 * myc * z + 6 * ny * z; break;
      case K_PER_X: v = 6 * mx * z + 2 * nx * 8 + 3 * kx * z; break;
      case K_LP_PER_Y2A:  // the three launches of the periodic Y2 pass move the Y2 arrays once
      case K_LP_PER_Y2F:
      case K_PER_Y2: case K_PER_Y2_PRE:
        v = (kernel == K_PER_Y2 ? 3 * ny : 3 * ky) * z + 2 * 3 * myc * z + 2 * ny * z + 2 * ny * z + 12 * myc * 8 +
            myc * z;
        break;
      case K_PER_X_MIXED: v = 6 * mx * 8 + 2 * nx * 4 + 3 * kx * 8; break;
      case K_STATE_F32: v = 3 * myc * (z + z / 2); break;
      case K_BOX_X1: v = 6 * mxc * 8 + 3 * nx * 8 + 3 * kx * 8 + nx * 8; break;
      case K_BOX_Y2: case K_BOX_Y2_PRE:
        v = (kernel == K_BOX_Y2 ? 3 * ny : 3 * ky) * 8 + 6 * myc * 8 + 4 * ny * 8 + 3 * myc * 8;
        break;
      case K_BOX_X2: v = 3 * nx * 8 + 3 * mxc * 8; break;
      case K_BOX_Y3: v = 6 * myc * 8 + 2 * ny * 8; break;
      case K_BOX_X3: case K_BOX_X3_MIX: v = 2 * mxc * 8 + nx * 8 + mxc * 8; break;
      // the row's own Poisson factors (four arrays of myc: the y operator
      // depends on the row's x eigenvalue), its right-hand side in, its solution out
      case K_BOX_Y4: v += ny * 8 + myc * 8 + 4 * myc * 8; break;
      case K_BOX_X4: case K_BOX_X4_MIX: v = mxc * 8 + nx * 8 + 3 * mxc * 8; break;
      case K_BOX_Y5: v = 7 * myc * 8 + 3 * ny * 8; break;
      case K_BOX_PROD_MIXED: v = 13 * nx * 4; break;
      case K_BOX_GPX: v = 2 * nx * 8; break;
      default: v = 0;
    }
    b += v * lanes;
  }
  return b;
}

cudaError_t launch_gate(const CaseDev* cases, const int* members, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  dev::k_gate<<<(n + 127) / 128, 128, 0, s>>>(cases, members, n);
  return cudaGetLastError();
}

const char* step_kernel_name(int kernel) {
  static const char* names[] = {"y1_complex", "y1_real", "periodic_x", "periodic_y2", "box_x1", "box_y2",
                                "box_x2", "box_y3", "box_x3", "box_y4", "box_x4", "box_y5", "periodic_y2a",
                                "periodic_y2b", "periodic_y2_pre", "periodic_x_mixed", "box_prod_mixed",
                                "box_y2_pre", "box_x3_mix", "box_x4_mix", "box_gpx", "lanes_box_gpx",
                                "lanes_box_x2", "lanes_box_x3", "lanes_box_x4", "lanes_box_y2", "lanes_box_y3",
                                "lanes_box_y4", "lanes_box_y5", "lanes_periodic_y2", "periodic_y2_pre_t128",
                                "box_y2_pre_t128", "box_x3_mix_t128", "box_y5_t128", "lanes_periodic_y2a",
                                "lanes_periodic_y2b", "lanes_periodic_y2c", "state_f32", "periodic_x_mixed_t128",
                                "lanes_periodic_y2_fused", "box_y4_mix"};
  if (kernel == K_GEMM) return "lane_gemm";
  if (kernel >= 0 && kernel < K_NUM_STEP_KERNELS) return names[kernel];
  return "";
}

}  // namespace rbc
