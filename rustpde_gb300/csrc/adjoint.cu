// adjoint.cu -- Navier2DAdjoint (src/navier/navier_adjoint.rs) on the GPU.
//
// The adjoint descent (Farazmand 2016) looks for steady states: each update
// runs one Navier2D step with dt = 1e-2 from the current state, takes the
// residual (new - old) / 1e-2, smooths it with the Hholtz operator (1 - D2)
// (navier_adjoint.rs:731-754), then advances the state explicitly with the
// adjoint convection, the diffusion of the smoothed residual and a pressure
// projection (navier_adjoint.rs:767-800).
//
// Device form: the inner Navier2D is a library case (its fused step kernels,
// enqueued directly); everything else is lane passes of the funspace
// primitives and elementwise kernels.  One update (about 150 launches) is
// captured once as a CUDA graph and replayed on the inner case's stream.
#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "case_access.h"
#include "host_ops.h"
#include "prims.h"
#include "spectral_rbc.h"

using namespace rbc;

namespace {

struct AdjError : std::runtime_error {
  int code;
  AdjError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define ADJ_BEGIN try {
#define ADJ_END                                                              \
  }                                                                          \
  catch (AdjError & e) { return set_last_error(e.code, e.what()); }          \
  catch (std::bad_alloc&) { return set_last_error(RBC_ERR_NOMEM, "host allocation failed"); } \
  catch (std::exception & e) {                                               \
    std::string w = e.what();                                                \
    return set_last_error(w.find("cudaMalloc") != std::string::npos ? RBC_ERR_NOMEM : RBC_ERR_CUDA, w); \
  }                                                                          \
  return RBC_OK;

void need(bool ok, const std::string& msg) {
  if (!ok) throw AdjError(RBC_ERR_INVALID, msg);
}

// Elementwise updates over n doubles (complex arrays interleaved: every
// scalar below is real, so complex arithmetic is componentwise).  Products
// and sums are rounded separately, as the reference evaluates them.
enum AdjOp {
  EW_RESIDUAL = 0,  // y = (y - a) / s0
  EW_SCALE,         // y = y * s0
  EW_SUB_SCALED,    // y = y - a * s0
  EW_ADD_SCALED,    // y = y + a * s0
  EW_ADD_SCALED2,   // y = y + (a * s0) * s1
  EW_AXPY_FIRST,    // y = a * s0 + y
  EW_PRODUCT,       // y = a * b
  EW_ADD_PRODUCT    // y = y + a * b
};

__global__ void k_adj_ew(int op, double* __restrict__ y, const double* __restrict__ a, const double* __restrict__ b,
                         double s0, double s1, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double r;
    switch (op) {
      case EW_RESIDUAL: r = __ddiv_rn(__dsub_rn(y[i], a[i]), s0); break;
      case EW_SCALE: r = __dmul_rn(y[i], s0); break;
      case EW_SUB_SCALED: r = __dsub_rn(y[i], __dmul_rn(a[i], s0)); break;
      case EW_ADD_SCALED: r = __dadd_rn(y[i], __dmul_rn(a[i], s0)); break;
      case EW_ADD_SCALED2: r = __dadd_rn(y[i], __dmul_rn(__dmul_rn(a[i], s0), s1)); break;
      case EW_AXPY_FIRST: r = __dadd_rn(__dmul_rn(a[i], s0), y[i]); break;
      case EW_PRODUCT: r = __dmul_rn(a[i], b[i]); break;
      default: r = __dadd_rn(y[i], __dmul_rn(a[i], b[i])); break;
    }
    y[i] = r;
  }
}

// navier.rs:1022-1032: zero rows >= 2 n0 / 3 and columns >= 2 n1 / 3
__global__ void k_adj_dealias(double* a, int n0, int n1, int kx, int ky, int w) {
  size_t n = (size_t)n0 * n1;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(idx / n1), j = (int)(idx - (size_t)i * n1);
    if (i >= kx || j >= ky)
      for (int c = 0; c < w; c++) a[idx * w + c] = 0.0;
  }
}

void ew(int op, void* y, const void* a, const void* b, double s0, double s1, size_t n, cudaStream_t st) {
  int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
  if (blocks < 1) blocks = 1;
  k_adj_ew<<<blocks, 256, 0, st>>>(op, static_cast<double*>(y), static_cast<const double*>(a),
                                   static_cast<const double*>(b), s0, s1, n);
  cuda_check(cudaGetLastError(), "elementwise kernel launch");
}

}  // namespace

struct RbcAdjoint {
  RbcParams p{};
  RbcCase* nav = nullptr;  // Navier2D with dt_navier = 1e-2 (navier_adjoint.rs:176)
  CaseAccess na{};
  Arena arena;
  SpaceDev sp_u, sp_t, sp_p0, sp_p1, sp_field;
  SolverDev pois, smooth_u, smooth_t;
  bool cplx = false;
  int nx = 0, ny = 0;
  double nu = 0, ka = 0, scale[2] = {1, 1}, dt = 0, dt_nav = 1e-2, time = 0;
  // state [0] and smoothed residuals [1]
  void *ux0 = nullptr, *uy0 = nullptr, *t0 = nullptr, *p0 = nullptr, *p1 = nullptr;
  void *ux1 = nullptr, *uy1 = nullptr, *t1 = nullptr;
  void* uns[3] = {nullptr, nullptr, nullptr};  // unsmoothed residuals (ortho)
  double *U = nullptr, *V = nullptr, *T = nullptr, *G = nullptr, *C = nullptr;  // physical
  void *rhs = nullptr, *og = nullptr, *ch = nullptr, *fx = nullptr;
  void* tmp = nullptr;
  double* d_red = nullptr;
  size_t n_spec_u = 0, n_spec_t = 0, n_p0 = 0, n_p1 = 0, n_ortho = 0, n_phys = 0;  // doubles
  cudaStream_t st = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  ~RbcAdjoint() {
    if (st) cudaStreamSynchronize(st);
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    if (nav) rbc_destroy(nav);
  }
  void sync() { cuda_check(cudaStreamSynchronize(st), "stream synchronize"); }
};

namespace {

void dealias(RbcAdjoint* a, void* spec) {
  const SpaceDev& s = a->sp_field;
  const int n0 = s.spec0, n1 = s.spec1;
  size_t n = (size_t)n0 * n1;
  int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
  k_adj_dealias<<<blocks, 256, 0, a->st>>>(static_cast<double*>(spec), n0, n1, n0 * 2 / 3, n1 * 2 / 3,
                                          a->cplx ? 2 : 1);
  cuda_check(cudaGetLastError(), "dealias kernel launch");
}

// conv accumulator C (physical) += w * backward(gradient(f, d)); first = assign
void conv_term(RbcAdjoint* a, const SpaceDev& s, const void* f, const double* w, int d0, int d1, bool first) {
  space_gradient_physical(s, f, a->G, d0, d1, a->scale, a->tmp, a->st);
  ew(first ? EW_PRODUCT : EW_ADD_PRODUCT, a->C, w, a->G, 0, 0, a->n_phys, a->st);
}

// C -> field forward transform, dealiased, into a->ch (ortho-shaped)
void conv_finish(RbcAdjoint* a) {
  space_forward(a->sp_field, a->C, a->ch, a->tmp, a->st);
  dealias(a, a->ch);
}

// one adjoint update (navier_adjoint.rs:767-800), enqueued on a->st
void enqueue_update(RbcAdjoint* a) {
  cudaStream_t st = a->st;
  const double dt = a->dt;
  // convection fields: physical ux, uy, temp of the state
  space_backward(a->sp_u, a->ux0, a->U, a->tmp, st);
  space_backward(a->sp_u, a->uy0, a->V, a->tmp, st);
  space_backward(a->sp_t, a->t0, a->T, a->tmp, st);

  // ---- update_residual (navier_adjoint.rs:731-754)
  cuda_check(cudaMemcpyAsync(a->na.ux, a->ux0, a->n_spec_u * 8, cudaMemcpyDeviceToDevice, st), "copy state");
  cuda_check(cudaMemcpyAsync(a->na.uy, a->uy0, a->n_spec_u * 8, cudaMemcpyDeviceToDevice, st), "copy state");
  cuda_check(cudaMemcpyAsync(a->na.temp, a->t0, a->n_spec_t * 8, cudaMemcpyDeviceToDevice, st), "copy state");
  case_enqueue_step(a->nav, st);
  void* nf[3] = {a->na.ux, a->na.uy, a->na.temp};
  void* sf[3] = {a->ux0, a->uy0, a->t0};
  void* rf[3] = {a->ux1, a->uy1, a->t1};
  const SpaceDev* sp[3] = {&a->sp_u, &a->sp_u, &a->sp_t};
  const SolverDev* sm[3] = {&a->smooth_u, &a->smooth_u, &a->smooth_t};
  const size_t ns[3] = {a->n_spec_u, a->n_spec_u, a->n_spec_t};
  for (int k = 0; k < 3; k++) {
    ew(EW_RESIDUAL, nf[k], sf[k], nullptr, a->dt_nav, 0, ns[k], st);
    space_to_ortho(*sp[k], nf[k], a->uns[k], a->tmp, st);
    solver_solve(*sm[k], *sp[k], a->uns[k], rf[k], a->tmp, st);
    ew(EW_SCALE, rf[k], nullptr, nullptr, -1.0, 0, ns[k], st);
  }

  // ---- solve_ux / solve_uy (navier_adjoint.rs:630-678), explicit
  for (int which = 0; which < 2; which++) {
    void* f0 = which == 0 ? a->ux0 : a->uy0;
    const void* f1 = which == 0 ? a->ux1 : a->uy1;
    space_to_ortho(a->sp_u, f0, a->rhs, a->tmp, st);
    space_gradient(a->sp_p0, a->p0, a->og, which == 0 ? 1 : 0, which == 0 ? 0 : 1, a->scale, a->tmp, st);
    ew(EW_SUB_SCALED, a->rhs, a->og, nullptr, dt, 0, a->n_ortho, st);
    if (which == 0) {  // conv_ux (navier_adjoint.rs:541-577)
      conv_term(a, a->sp_u, a->ux1, a->U, 1, 0, true);
      conv_term(a, a->sp_u, a->ux1, a->V, 0, 1, false);
      conv_term(a, a->sp_u, a->ux1, a->U, 1, 0, false);
      conv_term(a, a->sp_u, a->uy1, a->V, 1, 0, false);
      conv_term(a, a->sp_t, a->t1, a->T, 1, 0, false);
      conv_term(a, a->sp_t, a->t1, a->na.bc_phys, 1, 0, false);
    } else {  // conv_uy (navier_adjoint.rs:579-611)
      conv_term(a, a->sp_u, a->uy1, a->U, 1, 0, true);
      conv_term(a, a->sp_u, a->uy1, a->V, 0, 1, false);
      conv_term(a, a->sp_u, a->ux1, a->U, 0, 1, false);
      conv_term(a, a->sp_u, a->uy1, a->V, 0, 1, false);
      conv_term(a, a->sp_t, a->t1, a->T, 0, 1, false);
      conv_term(a, a->sp_t, a->t1, a->na.bc_phys, 0, 1, false);
    }
    conv_finish(a);
    ew(EW_ADD_SCALED, a->rhs, a->ch, nullptr, dt, 0, a->n_ortho, st);
    space_gradient(a->sp_u, f1, a->og, 2, 0, a->scale, a->tmp, st);
    ew(EW_ADD_SCALED2, a->rhs, a->og, nullptr, dt, a->nu, a->n_ortho, st);
    space_gradient(a->sp_u, f1, a->og, 0, 2, a->scale, a->tmp, st);
    ew(EW_ADD_SCALED2, a->rhs, a->og, nullptr, dt, a->nu, a->n_ortho, st);
    space_from_ortho(a->sp_u, a->rhs, f0, a->tmp, st);
  }

  // ---- projection (navier_adjoint.rs:697-729)
  space_gradient(a->sp_u, a->ux0, a->rhs, 1, 0, a->scale, a->tmp, st);
  space_gradient(a->sp_u, a->uy0, a->og, 0, 1, a->scale, a->tmp, st);
  ew(EW_ADD_SCALED, a->rhs, a->og, nullptr, 1.0, 0, a->n_ortho, st);  // div = d/dx ux + d/dy uy
  solver_solve(a->pois, a->sp_p1, a->rhs, a->p1, a->tmp, st);
  cuda_check(cudaMemsetAsync(a->p1, 0, a->cplx ? 16 : 8, st), "p1[0,0] = 0");
  for (int which = 0; which < 2; which++) {
    void* f0 = which == 0 ? a->ux0 : a->uy0;
    space_gradient(a->sp_p1, a->p1, a->og, which == 0 ? 1 : 0, which == 0 ? 0 : 1, a->scale, a->tmp, st);
    space_from_ortho(a->sp_u, a->og, a->fx, a->tmp, st);
    ew(EW_AXPY_FIRST, f0, a->fx, nullptr, -1.0, 0, a->n_spec_u, st);
  }
  space_to_ortho(a->sp_p1, a->p1, a->og, a->tmp, st);
  ew(EW_ADD_SCALED, a->p0, a->og, nullptr, 1.0 / dt, 0, a->n_p0, st);

  // ---- solve_temp (navier_adjoint.rs:680-695)
  space_to_ortho(a->sp_t, a->t0, a->rhs, a->tmp, st);
  conv_term(a, a->sp_t, a->t1, a->U, 1, 0, true);  // conv_temp (navier_adjoint.rs:613-628)
  conv_term(a, a->sp_t, a->t1, a->V, 0, 1, false);
  conv_finish(a);
  ew(EW_ADD_SCALED, a->rhs, a->ch, nullptr, dt, 0, a->n_ortho, st);
  space_to_ortho(a->sp_u, a->uy1, a->og, a->tmp, st);  // adjoint buoyancy
  ew(EW_ADD_SCALED, a->rhs, a->og, nullptr, dt, 0, a->n_ortho, st);
  space_gradient(a->sp_t, a->t1, a->og, 2, 0, a->scale, a->tmp, st);
  ew(EW_ADD_SCALED2, a->rhs, a->og, nullptr, dt, a->ka, a->n_ortho, st);
  space_gradient(a->sp_t, a->t1, a->og, 0, 2, a->scale, a->tmp, st);
  ew(EW_ADD_SCALED2, a->rhs, a->og, nullptr, dt, a->ka, a->n_ortho, st);
  space_from_ortho(a->sp_t, a->rhs, a->t0, a->tmp, st);
}

void* state_ptr(RbcAdjoint* a, int field, size_t* n) {
  switch (field) {
    case RBC_TEMP: *n = a->n_spec_t; return a->t0;
    case RBC_UX: *n = a->n_spec_u; return a->ux0;
    case RBC_UY: *n = a->n_spec_u; return a->uy0;
    case RBC_PRES: *n = a->n_p0; return a->p0;
    case RBC_PSEUDO_PRES: *n = a->n_p1; return a->p1;
    case RBC_ADJ_TEMP_RES: *n = a->n_spec_t; return a->t1;
    case RBC_ADJ_UX_RES: *n = a->n_spec_u; return a->ux1;
    case RBC_ADJ_UY_RES: *n = a->n_spec_u; return a->uy1;
  }
  throw AdjError(RBC_ERR_INVALID, "unknown adjoint field id");
}

const SpaceDev& state_space(const RbcAdjoint* a, int field) {
  switch (field) {
    case RBC_TEMP:
    case RBC_ADJ_TEMP_RES: return a->sp_t;
    case RBC_UX:
    case RBC_UY:
    case RBC_ADJ_UX_RES:
    case RBC_ADJ_UY_RES: return a->sp_u;
    case RBC_PRES: return a->sp_p0;
    case RBC_PSEUDO_PRES: return a->sp_p1;
  }
  throw AdjError(RBC_ERR_INVALID, "unknown adjoint field id");
}

double norm_l2(RbcAdjoint* a, const void* v, size_t n) {
  sum_squares(static_cast<const double*>(v), n, a->d_red, a->st);
  double h = 0;
  cuda_check(cudaMemcpyAsync(&h, a->d_red, 8, cudaMemcpyDeviceToHost, a->st), "d2h");
  a->sync();
  return std::sqrt(h);
}

// copy the adjoint state into the inner case (for its diagnostics and ICs)
void state_to_nav(RbcAdjoint* a) {
  cuda_check(cudaMemcpyAsync(a->na.ux, a->ux0, a->n_spec_u * 8, cudaMemcpyDeviceToDevice, a->st), "copy state");
  cuda_check(cudaMemcpyAsync(a->na.uy, a->uy0, a->n_spec_u * 8, cudaMemcpyDeviceToDevice, a->st), "copy state");
  cuda_check(cudaMemcpyAsync(a->na.temp, a->t0, a->n_spec_t * 8, cudaMemcpyDeviceToDevice, a->st), "copy state");
}

}  // namespace

extern "C" {

int rbc_adjoint_create(const RbcParams* params, RbcAdjoint** out) {
  ADJ_BEGIN
  need(params != nullptr && out != nullptr, "rbc_adjoint_create: null argument");
  *out = nullptr;
  need(params->precision == RBC_PREC_FP64, "rbc_adjoint_create: the adjoint solver runs in FP64");
  std::unique_ptr<RbcAdjoint> a(new RbcAdjoint());
  a->p = *params;
  RbcParams np = *params;
  np.dt = a->dt_nav;
  int rc = rbc_create(&np, &a->nav);
  if (rc != RBC_OK) throw AdjError(rc, std::string("rbc_adjoint_create: ") + rbc_last_error());
  a->na = case_access(a->nav);
  a->st = a->na.stream;
  a->nu = a->na.nu;
  a->ka = a->na.ka;
  a->scale[0] = a->na.scale[0];
  a->scale[1] = a->na.scale[1];
  a->dt = params->dt;
  const int nx = params->nx, ny = params->ny;
  a->nx = nx;
  a->ny = ny;
  const bool per = params->kind == RBC_PERIODIC;
  a->cplx = per;
  Arena& A = a->arena;
  const int xu = per ? FOURIER : CD, xt = per ? FOURIER : (params->kind == RBC_BOX_ADIABATIC ? CN : CD);
  const int xo = per ? FOURIER : CHEB, xp = per ? FOURIER : CN;
  build_space(A, a->sp_u, xu, nx, CD, ny);
  build_space(A, a->sp_t, xt, nx, CD, ny);
  build_space(A, a->sp_p0, xo, nx, CHEB, ny);
  build_space(A, a->sp_p1, xp, nx, CN, ny);
  build_space(A, a->sp_field, xo, nx, CHEB, ny);
  const double s0 = std::pow(a->scale[0], 2.0), s1 = std::pow(a->scale[1], 2.0);
  const double cp[2] = {1.0 / s0, 1.0 / s1};
  const double w = 1e0;  // weight_laplacian (navier_adjoint.rs:203)
  const double cs[2] = {w / s0, w / s1};
  std::string err;
  if (!build_solver(A, a->sp_p1, SV_KIND_POISSON, cp, a->pois, &err) ||
      !build_solver(A, a->sp_u, SV_KIND_HHOLTZ, cs, a->smooth_u, &err) ||
      !build_solver(A, a->sp_t, SV_KIND_HHOLTZ, cs, a->smooth_t, &err))
    throw AdjError(RBC_ERR_UNSUPPORTED, "rbc_adjoint_create: " + err);
  const size_t cw = per ? 2 : 1;
  a->n_spec_u = (size_t)a->sp_u.spec0 * a->sp_u.spec1 * cw;
  a->n_spec_t = (size_t)a->sp_t.spec0 * a->sp_t.spec1 * cw;
  a->n_p0 = (size_t)a->sp_p0.spec0 * a->sp_p0.spec1 * cw;
  a->n_p1 = (size_t)a->sp_p1.spec0 * a->sp_p1.spec1 * cw;
  a->n_ortho = (size_t)a->sp_field.spec0 * a->sp_field.spec1 * cw;
  a->n_phys = (size_t)nx * ny;
  auto al = [&](size_t nd) { return A.alloc(nd * 8); };
  a->ux0 = al(a->n_spec_u); a->uy0 = al(a->n_spec_u); a->t0 = al(a->n_spec_t);
  a->p0 = al(a->n_p0); a->p1 = al(a->n_p1);
  a->ux1 = al(a->n_spec_u); a->uy1 = al(a->n_spec_u); a->t1 = al(a->n_spec_t);
  for (int k = 0; k < 3; k++) a->uns[k] = al(a->n_ortho);
  a->U = static_cast<double*>(al(a->n_phys));
  a->V = static_cast<double*>(al(a->n_phys));
  a->T = static_cast<double*>(al(a->n_phys));
  a->G = static_cast<double*>(al(a->n_phys));
  a->C = static_cast<double*>(al(a->n_phys));
  a->rhs = al(a->n_ortho); a->og = al(a->n_ortho); a->ch = al(a->n_ortho);
  a->fx = al(std::max(a->n_spec_u, a->n_spec_t));
  size_t te = 0;
  for (const SpaceDev* s : {&a->sp_u, &a->sp_t, &a->sp_p0, &a->sp_p1, &a->sp_field}) te = std::max(te, tmp_elems(*s));
  a->tmp = A.alloc(te * 16);
  a->d_red = static_cast<double*>(A.alloc(64));
  cuda_check(cudaStreamSynchronize(cudaStreamLegacy), "allocation");
  // one update as a CUDA graph
  cuda_check(cudaStreamBeginCapture(a->st, cudaStreamCaptureModeThreadLocal), "begin capture");
  try {
    enqueue_update(a.get());
  } catch (...) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(a->st, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  cuda_check(cudaStreamEndCapture(a->st, &a->graph), "end capture");
  cuda_check(cudaGraphInstantiate(&a->gexec, a->graph, 0), "graph instantiate");
  *out = a.release();
  ADJ_END
}

int rbc_adjoint_destroy(RbcAdjoint* a) {
  ADJ_BEGIN
  delete a;
  ADJ_END
}

int rbc_adjoint_set_velocity(RbcAdjoint* a, double amp, double m, double n) {
  ADJ_BEGIN
  need(a != nullptr, "rbc_adjoint_set_velocity: null argument");
  int rc = rbc_set_velocity(a->nav, amp, m, n);
  if (rc != RBC_OK) throw AdjError(rc, rbc_last_error());
  cuda_check(cudaMemcpyAsync(a->ux0, a->na.ux, a->n_spec_u * 8, cudaMemcpyDeviceToDevice, a->st), "copy state");
  cuda_check(cudaMemcpyAsync(a->uy0, a->na.uy, a->n_spec_u * 8, cudaMemcpyDeviceToDevice, a->st), "copy state");
  a->sync();
  ADJ_END
}

int rbc_adjoint_set_temperature(RbcAdjoint* a, double amp, double m, double n) {
  ADJ_BEGIN
  need(a != nullptr, "rbc_adjoint_set_temperature: null argument");
  int rc = rbc_set_temperature(a->nav, amp, m, n);
  if (rc != RBC_OK) throw AdjError(rc, rbc_last_error());
  cuda_check(cudaMemcpyAsync(a->t0, a->na.temp, a->n_spec_t * 8, cudaMemcpyDeviceToDevice, a->st), "copy state");
  a->sync();
  ADJ_END
}

int rbc_adjoint_step(RbcAdjoint* a, int nsteps) {
  ADJ_BEGIN
  need(a != nullptr && nsteps >= 0, "rbc_adjoint_step: invalid argument");
  for (int i = 0; i < nsteps; i++) {
    cuda_check(cudaGraphLaunch(a->gexec, a->st), "graph launch");
    a->time += a->dt;
  }
  ADJ_END
}

int rbc_adjoint_synchronize(RbcAdjoint* a) {
  ADJ_BEGIN
  need(a != nullptr, "rbc_adjoint_synchronize: null argument");
  a->sync();
  ADJ_END
}

int rbc_adjoint_get_time(const RbcAdjoint* a, double* t) {
  ADJ_BEGIN
  need(a && t, "rbc_adjoint_get_time: null argument");
  *t = a->time;
  ADJ_END
}

int rbc_adjoint_set_time(RbcAdjoint* a, double t) {
  ADJ_BEGIN
  need(a != nullptr, "rbc_adjoint_set_time: null argument");
  a->time = t;
  rbc_set_time(a->nav, t);
  ADJ_END
}

int rbc_adjoint_field_shape(const RbcAdjoint* a, int field, int* n0, int* n1, int* is_complex) {
  ADJ_BEGIN
  need(a && n0 && n1 && is_complex, "rbc_adjoint_field_shape: null argument");
  const SpaceDev& s = state_space(a, field);
  *n0 = s.spec0;
  *n1 = s.spec1;
  *is_complex = s.cplx;
  ADJ_END
}

int rbc_adjoint_get_state(RbcAdjoint* a, int field, double* host, size_t n_doubles) {
  ADJ_BEGIN
  need(a && host, "rbc_adjoint_get_state: null argument");
  size_t n = 0;
  void* d = state_ptr(a, field, &n);
  need(n == n_doubles, "rbc_adjoint_get_state: size mismatch");
  cuda_check(cudaMemcpyAsync(host, d, n * 8, cudaMemcpyDeviceToHost, a->st), "d2h");
  a->sync();
  ADJ_END
}

int rbc_adjoint_set_state(RbcAdjoint* a, int field, const double* host, size_t n_doubles) {
  ADJ_BEGIN
  need(a && host, "rbc_adjoint_set_state: null argument");
  size_t n = 0;
  void* d = state_ptr(a, field, &n);
  need(n == n_doubles, "rbc_adjoint_set_state: size mismatch");
  cuda_check(cudaMemcpyAsync(d, host, n * 8, cudaMemcpyHostToDevice, a->st), "h2d");
  a->sync();
  ADJ_END
}

// Nu, Nuvol, Re, KE, |div| of the adjoint state (navier_adjoint.rs:932-963):
// the inner case's functions on a copy of the state (same spaces)
int rbc_adjoint_eval(RbcAdjoint* a, int what, double* out) {
  ADJ_BEGIN
  need(a && out, "rbc_adjoint_eval: null argument");
  state_to_nav(a);
  int rc = rbc_eval(a->nav, what, out);
  if (rc != RBC_OK) throw AdjError(rc, rbc_last_error());
  ADJ_END
}

// |unsmoothed residual| of ux, uy, temp and |smoothed residual| (navier_adjoint.rs:866-874)
int rbc_adjoint_residual(RbcAdjoint* a, double out[6]) {
  ADJ_BEGIN
  need(a && out, "rbc_adjoint_residual: null argument");
  for (int k = 0; k < 3; k++) out[k] = norm_l2(a, a->uns[k], a->n_ortho);
  out[3] = norm_l2(a, a->ux1, a->n_spec_u);
  out[4] = norm_l2(a, a->uy1, a->n_spec_u);
  out[5] = norm_l2(a, a->t1, a->n_spec_t);
  ADJ_END
}

// navier_adjoint.rs:889-906: stop on a NaN divergence or when the smoothed
// residual is below 1e-8
int rbc_adjoint_exit(RbcAdjoint* a, int* stop) {
  ADJ_BEGIN
  need(a && stop, "rbc_adjoint_exit: null argument");
  double div = 0;
  state_to_nav(a);
  int rc = rbc_eval(a->nav, RBC_DIV_NORM, &div);
  if (rc != RBC_OK) throw AdjError(rc, rbc_last_error());
  double r = norm_l2(a, a->ux1, a->n_spec_u) + norm_l2(a, a->uy1, a->n_spec_u) + norm_l2(a, a->t1, a->n_spec_t);
  *stop = (std::isnan(div) || r < 1e-8) ? 1 : 0;
  ADJ_END
}

// Navier2DAdjoint::write (navier_adjoint.rs:1005-1040): temp (plus the boundary
// field), ux, uy, pres and the scalars, through the inner case's snapshot
// writer on a copy of the adjoint state (the header's dt is the inner step's)
int rbc_adjoint_write_snapshot(RbcAdjoint* a, const char* path) {
  ADJ_BEGIN
  need(a && path, "rbc_adjoint_write_snapshot: null argument");
  state_to_nav(a);
  cuda_check(cudaMemcpyAsync(a->na.p0, a->p0, a->n_p0 * 8, cudaMemcpyDeviceToDevice, a->st), "copy state");
  a->sync();
  double t_nav = 0.0;
  rbc_get_time(a->nav, &t_nav);
  rbc_set_time(a->nav, a->time);
  int rc = rbc_write_snapshot(a->nav, path);
  rbc_set_time(a->nav, t_nav);
  if (rc != RBC_OK) throw AdjError(rc, rbc_last_error());
  ADJ_END
}

// Navier2DAdjoint::read (navier_adjoint.rs:991-999): temp, ux, uy and time
int rbc_adjoint_read_snapshot(RbcAdjoint* a, const char* path) {
  ADJ_BEGIN
  need(a && path, "rbc_adjoint_read_snapshot: null argument");
  double t_nav = 0.0;
  rbc_get_time(a->nav, &t_nav);
  int rc = rbc_read_snapshot(a->nav, path);
  if (rc != RBC_OK) throw AdjError(rc, rbc_last_error());
  double t = 0.0;
  rbc_get_time(a->nav, &t);
  rbc_set_time(a->nav, t_nav);
  a->time = t;
  cuda_check(cudaMemcpyAsync(a->ux0, a->na.ux, a->n_spec_u * 8, cudaMemcpyDeviceToDevice, a->st), "copy state");
  cuda_check(cudaMemcpyAsync(a->uy0, a->na.uy, a->n_spec_u * 8, cudaMemcpyDeviceToDevice, a->st), "copy state");
  cuda_check(cudaMemcpyAsync(a->t0, a->na.temp, a->n_spec_t * 8, cudaMemcpyDeviceToDevice, a->st), "copy state");
  a->sync();
  ADJ_END
}

int rbc_adjoint_get_stream(RbcAdjoint* a, void** stream) {
  ADJ_BEGIN
  need(a && stream, "rbc_adjoint_get_stream: null argument");
  *stream = a->st;
  ADJ_END
}

}  // extern "C"
