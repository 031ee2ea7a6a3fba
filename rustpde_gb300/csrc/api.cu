// api.cu -- C ABI of the spectral RBC library (include/spectral_rbc.h).
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "host_ops.h"
#include "prims.h"
#include "spectral_rbc.h"
#include "step_fp64.h"

namespace rbc {

static thread_local std::string g_err;

struct ApiError : std::runtime_error {
  int code;
  ApiError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

static int fail(int code, const std::string& m) {
  g_err = m;
  return code;
}

#define API_BEGIN try {
#define API_END                                              \
  }                                                          \
  catch (ApiError & e) { return fail(e.code, e.what()); }    \
  catch (std::bad_alloc&) { return fail(RBC_ERR_NOMEM, "host allocation failed"); } \
  catch (std::exception & e) {                               \
    std::string w = e.what();                                \
    int code = (w.find("cudaMalloc") != std::string::npos) ? RBC_ERR_NOMEM : RBC_ERR_CUDA; \
    return fail(code, w);                                    \
  }                                                          \
  return RBC_OK;

static void require(bool ok, const std::string& msg) {
  if (!ok) throw ApiError(RBC_ERR_INVALID, msg);
}

static double get_nu(double ra, double pr, double h) { return std::sqrt(pr / (ra / std::pow(h, 3.0))); }
static double get_ka(double ra, double pr, double h) { return std::sqrt(1.0 / ((ra / std::pow(h, 3.0)) * pr)); }

}  // namespace rbc

using namespace rbc;

struct RbcCase {
  RbcParams p{};
  bool periodic = false;
  Arena arena;
  CaseDev hd{};
  CaseDev* d_case = nullptr;
  SpaceDev sp_u, sp_t, sp_p0, sp_p1, sp_field, sp_bc;
  double nu = 0, ka = 0, scale[2] = {1, 1};
  void* tmp = nullptr;
  double* phys[4] = {nullptr, nullptr, nullptr, nullptr};
  void* spec_tmp[3] = {nullptr, nullptr, nullptr};
  void* bc_vhat = nullptr;
  double* bc_phys = nullptr;
  double* d_wx = nullptr;
  double* d_wy = nullptr;
  double* d_red = nullptr;
  cudaStream_t stream = nullptr;
  StepPlan plan;
  std::vector<int4*> d_work;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  double time = 0.0;
  bool own_stream = true;
  bool in_batch = false;
  ~RbcCase() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    if (stream) {
      cudaStreamSynchronize(stream);
      if (own_stream) cudaStreamDestroy(stream);
    }
  }
  size_t spec_elem() const { return periodic ? 16 : 8; }
  void sync() { cuda_check(cudaStreamSynchronize(stream), "stream synchronize"); }
};

struct FsSpace {
  Arena arena;
  SpaceDev s;
  void* tmp = nullptr;
};

struct SvSolver {
  FsSpace* space = nullptr;
  Arena arena;
  SolverDev sv;
};

namespace {

const SpaceDev& field_space(const RbcCase* c, int field) {
  switch (field) {
    case RBC_TEMP: return c->sp_t;
    case RBC_UX:
    case RBC_UY: return c->sp_u;
    case RBC_PRES: return c->sp_p0;
    case RBC_PSEUDO_PRES: return c->sp_p1;
    case RBC_FIELDBC: return c->sp_bc;
  }
  throw ApiError(RBC_ERR_INVALID, "unknown field id");
}

void* field_ptr(RbcCase* c, int field) {
  switch (field) {
    case RBC_TEMP: return c->hd.temp;
    case RBC_UX: return c->hd.ux;
    case RBC_UY: return c->hd.uy;
    case RBC_PRES: return c->hd.p0;
    case RBC_PSEUDO_PRES: return c->hd.p1;
    case RBC_FIELDBC: return c->bc_vhat;
  }
  throw ApiError(RBC_ERR_INVALID, "unknown field id");
}

size_t spec_doubles(const RbcCase* c, int field) {
  const SpaceDev& s = field_space(c, field);
  return (size_t)s.spec0 * s.spec1 * (s.cplx ? 2 : 1);
}

// grid coordinates of Navier2D fields, scaled like Navier2D::_scale (navier.rs:500-512)
void coords(const RbcCase* c, int field, std::vector<double>& x, std::vector<double>& y) {
  const SpaceDev& s = field_space(c, field);
  x = s.hb0.x;
  y = s.hb1.x;
  if (field == RBC_TEMP || field == RBC_UX || field == RBC_UY || field == RBC_PRES) {
    for (double& e : x) e *= c->scale[0];
    for (double& e : y) e *= c->scale[1];
  }
}

std::vector<double> get_dx(const std::vector<double>& x, bool periodic) {  // field.rs:135-163
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

void build_case(RbcCase* c, bool with_graph = true) {
  const RbcParams& p = c->p;
  Arena& A = c->arena;
  const int nx = p.nx, ny = p.ny;
  const bool per = c->periodic;
  c->scale[0] = p.aspect;
  c->scale[1] = 1.0;
  c->nu = get_nu(p.ra, p.pr, c->scale[1] * 2.0);
  c->ka = get_ka(p.ra, p.pr, c->scale[1] * 2.0);
  const int xk_u = per ? FOURIER : CD;
  const int xk_t = per ? FOURIER : (p.kind == RBC_BOX_ADIABATIC ? CN : CD);
  const int xk_o = per ? FOURIER : CHEB;
  const int xk_p = per ? FOURIER : CN;
  build_space(A, c->sp_u, xk_u, nx, CD, ny);
  build_space(A, c->sp_t, xk_t, nx, CD, ny);
  build_space(A, c->sp_p0, xk_o, nx, CHEB, ny);
  build_space(A, c->sp_p1, xk_p, nx, CN, ny);
  build_space(A, c->sp_field, xk_o, nx, CHEB, ny);
  build_space(A, c->sp_bc, xk_o, nx, CDBC, ny);

  CaseDev& h = c->hd;
  std::memset(&h, 0, sizeof h);
  h.kind = p.kind;
  h.nx = nx;
  h.ny = ny;
  h.mx = c->sp_p0.spec0;
  h.mxc = c->sp_u.spec0;
  h.myc = ny - 2;
  h.kx = h.mx * 2 / 3;  // navier.rs:1022-1032 on the (mx, ny) field array
  h.ky = ny * 2 / 3;
  h.dt = p.dt;
  h.nu = c->nu;
  h.ka = c->ka;
  h.aspect = p.aspect;
  h.inv_dt = 1.0 / p.dt;
  h.ycd = c->sp_u.b1;
  h.ycn = c->sp_p1.b1;
  h.xu = c->sp_u.b0;
  h.xt = c->sp_t.b0;
  h.xp = c->sp_p1.b0;
  h.pinv_y = upload_pinv(A, ny);
  h.cy = c->sp_u.c1;
  if (per) h.fx = c->sp_u.f0;
  else {
    h.pinv_x = upload_pinv(A, nx);
    h.cx = c->sp_u.c0;
  }
  const double s0 = std::pow(c->scale[0], 2.0), s1 = std::pow(c->scale[1], 2.0);
  const double cu[2] = {p.dt * c->nu / s0, p.dt * c->nu / s1};
  const double ct[2] = {p.dt * c->ka / s0, p.dt * c->ka / s1};
  const double cp[2] = {1.0 / s0, 1.0 / s1};
  std::string err;
  if (per) {
    // Hholtz (FdmaTensor, Fourier-diagonal x) for ux, uy, temp; Poisson for pres[1]
    h.hu_y = upload_fdma(A, hholtz_rows(c->sp_u.hb0, c->sp_u.hb1, cu[0], cu[1], 1.0, false, nullptr, nullptr, nullptr, &err));
    h.ht_y = upload_fdma(A, hholtz_rows(c->sp_t.hb0, c->sp_t.hb1, ct[0], ct[1], 1.0, false, nullptr, nullptr, nullptr, &err));
    h.pois_y = upload_fdma(A, hholtz_rows(c->sp_p1.hb0, c->sp_p1.hb1, cp[0], cp[1], 0.0, true, nullptr, nullptr, nullptr, &err));
  } else {
    // HholtzAdi for ux, uy, temp; Poisson (eigen-decomposed x) for pres[1]
    h.hu_y = upload_fdma(A, {adi_factor(c->sp_u.hb1, cu[1])});
    h.hu_x = upload_fdma(A, {adi_factor(c->sp_u.hb0, cu[0])});
    h.ht_y = upload_fdma(A, {adi_factor(c->sp_t.hb1, ct[1])});
    h.ht_x = upload_fdma(A, {adi_factor(c->sp_t.hb0, ct[0])});
    std::vector<double> fwd, bwd;
    h.pois_y = upload_fdma(A, hholtz_rows(c->sp_p1.hb0, c->sp_p1.hb1, cp[0], cp[1], 0.0, true, nullptr, &fwd, &bwd, &err));
    h.pois_fwd = A.upload(fwd);
    h.pois_bwd = A.upload(bwd);
  }
  const size_t es = c->spec_elem();
  const size_t nstate = (size_t)h.mxc * h.myc;
  h.ux = A.alloc(nstate * es);
  h.uy = A.alloc(nstate * es);
  h.temp = A.alloc(nstate * es);
  h.p0 = A.alloc((size_t)h.mx * ny * es);
  h.p1 = A.alloc(nstate * es);
  for (int k = 0; k < 6; k++) h.yw[k] = A.alloc((size_t)h.mxc * ny * es);
  h.q[0] = A.alloc((size_t)3 * std::max(h.kx, 1) * ny * es);
  if (!per)
    for (int k = 0; k < 8; k++) h.s[k] = A.alloc((size_t)nx * ny * 8);
  void* bco = A.alloc((size_t)h.mx * ny * es);
  void* bcd = A.alloc((size_t)h.mx * ny * es);
  double* bdx = static_cast<double*>(A.alloc((size_t)nx * ny * 8));
  double* bdy = static_cast<double*>(A.alloc((size_t)nx * ny * 8));
  h.bc_ortho = bco;
  h.bc_diff = bcd;
  h.bc_dx = bdx;
  h.bc_dy = bdy;
  h.status = static_cast<unsigned int*>(A.alloc(16));
  h.accum = static_cast<double*>(A.alloc(64));
  // generic scratch
  size_t te = 0;
  for (const SpaceDev* s : {&c->sp_u, &c->sp_t, &c->sp_p0, &c->sp_p1, &c->sp_field, &c->sp_bc})
    te = std::max(te, tmp_elems(*s));
  c->tmp = A.alloc(te * 16);
  for (int k = 0; k < 4; k++) c->phys[k] = static_cast<double*>(A.alloc((size_t)nx * ny * 8));
  for (int k = 0; k < 3; k++) c->spec_tmp[k] = A.alloc((size_t)std::max(h.mx, nx) * ny * 16);
  c->bc_vhat = A.alloc((size_t)h.mx * 2 * es);
  c->bc_phys = static_cast<double*>(A.alloc((size_t)nx * ny * 8));
  c->d_red = static_cast<double*>(A.alloc(64));
  // averaging weights on the unscaled coordinates of `field` (average.rs)
  {
    std::vector<double> x = c->sp_field.hb0.x, y = c->sp_field.hb1.x;
    std::vector<double> dx = get_dx(x, per), dy = get_dx(y, false);
    double lx = std::fabs(x.back() - x[0]), ly = std::fabs(y.back() - y[0]);
    std::vector<double> wx(nx), wy(ny);
    for (int i = 0; i < nx; i++) wx[i] = dx[i] / lx;
    for (int j = 0; j < ny; j++) wy[j] = dy[j] / ly;
    c->d_wx = A.upload(wx);
    c->d_wy = A.upload(wy);
  }
  cuda_check(cudaDeviceSynchronize(), "allocation");
  c->d_case = static_cast<CaseDev*>(A.alloc(sizeof(CaseDev)));
  cuda_check(cudaMemcpy(c->d_case, &h, sizeof(CaseDev), cudaMemcpyHostToDevice), "copy case descriptor");

  // ---- temperature boundary field: bc_rbc / bc_rbc_periodic (navier.rs:314-332, 474-492)
  cudaStream_t st = c->stream;
  {
    std::vector<double> bc((size_t)nx * 2);
    for (int i = 0; i < nx; i++) { bc[2 * i] = 0.5; bc[2 * i + 1] = -0.5; }
    double* d_bc = c->phys[0];
    cuda_check(cudaMemcpyAsync(d_bc, bc.data(), bc.size() * 8, cudaMemcpyHostToDevice, st), "upload bc");
    axis0_forward(c->sp_bc, d_bc, c->bc_vhat, 2, st);
    space_backward(c->sp_bc, c->bc_vhat, c->bc_phys, c->tmp, st);
    space_forward(c->sp_bc, c->bc_phys, c->bc_vhat, c->tmp, st);
    // derived constants of the step
    space_to_ortho(c->sp_bc, c->bc_vhat, bco, c->tmp, st);
    void* gxx = c->spec_tmp[0];
    void* gyy = c->spec_tmp[1];
    space_gradient(c->sp_bc, c->bc_vhat, gxx, 2, 0, c->scale, c->tmp, st);
    space_gradient(c->sp_bc, c->bc_vhat, gyy, 0, 2, c->scale, c->tmp, st);
    size_t nd = (size_t)h.mx * ny * (per ? 2 : 1);
    phys_combine(5, (const double*)gxx, (const double*)gyy, nullptr, p.dt, c->ka, (double*)bcd, nd, st);
    space_gradient(c->sp_bc, c->bc_vhat, gxx, 1, 0, c->scale, c->tmp, st);
    space_backward(c->sp_field, gxx, bdx, c->tmp, st);
    space_gradient(c->sp_bc, c->bc_vhat, gxx, 0, 1, c->scale, c->tmp, st);
    space_backward(c->sp_field, gxx, bdy, c->tmp, st);
    c->sync();
  }
  // ---- step plan, work tables and the CUDA graph of one update()
  cuda_check(configure_step_kernels(), "configure step kernels");
  c->plan = build_step_plan(h);
  if (!with_graph) return;
  for (auto& L : c->plan.launches) {
    int4* w = static_cast<int4*>(A.alloc(L.items.size() * sizeof(int4)));
    cuda_check(cudaMemcpy(w, L.items.data(), L.items.size() * sizeof(int4), cudaMemcpyHostToDevice), "work table");
    c->d_work.push_back(w);
  }
  cuda_check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
  cudaError_t le = cudaSuccess;
  for (size_t k = 0; k < c->plan.launches.size(); k++) {
    auto& L = c->plan.launches[k];
    cudaError_t e = launch_step_kernel(L.kernel, (int)L.items.size(), L.smem, st, c->d_case, c->d_work[k]);
    if (e != cudaSuccess && le == cudaSuccess) le = e;
  }
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamEndCapture(st, &g);
  cuda_check(le, "step kernel launch");
  cuda_check(ce, "end capture");
  c->graph = g;
  cuda_check(cudaGraphInstantiate(&c->gexec, g, 0), "graph instantiate");
}

// physical initial condition -> spectral state (Field2::forward)
void set_phys(RbcCase* c, int field, const std::vector<double>& v) {
  double* d = c->phys[0];
  cuda_check(cudaMemcpyAsync(d, v.data(), v.size() * 8, cudaMemcpyHostToDevice, c->stream), "upload");
  space_forward(field_space(c, field), d, field_ptr(c, field), c->tmp, c->stream);
  c->sync();
}

void apply_mode(RbcCase* c, int field, double amp, double m, double n, bool sin_cos) {
  // navier.rs:1035-1076 on normalised (scaled) coordinates
  std::vector<double> x, y;
  coords(c, field, x, y);
  std::vector<double> xs(x.size()), ys(y.size());
  for (size_t i = 0; i < x.size(); i++) xs[i] = (x[i] - x[0]) / (x.back() - x[0]);
  for (size_t j = 0; j < y.size(); j++) ys[j] = (y[j] - y[0]) / (y.back() - y[0]);
  const double PI = 3.14159265358979323846;
  double ax = PI * m, ay = PI * n;
  std::vector<double> v(x.size() * y.size());
  for (size_t i = 0; i < x.size(); i++)
    for (size_t j = 0; j < y.size(); j++)
      v[i * y.size() + j] = sin_cos ? amp * std::sin(ax * xs[i]) * std::cos(ay * ys[j])
                                    : amp * std::cos(ax * xs[i]) * std::sin(ay * ys[j]);
  set_phys(c, field, v);
}

double eval_case(RbcCase* c, int what) {
  cudaStream_t st = c->stream;
  const int nx = c->p.nx, ny = c->p.ny;
  const size_t nphys = (size_t)nx * ny;
  const CaseDev& h = c->hd;
  double out = 0.0;
  switch (what) {
    case RBC_NU: {
      // field.vhat = to_ortho(temp) + to_ortho(fieldbc); -dT/dz / (scale_y / 2); x-average at the plates
      void* tv = c->spec_tmp[0];
      void* g = c->spec_tmp[1];
      space_to_ortho(c->sp_t, h.temp, tv, c->tmp, st);
      size_t nd = (size_t)h.mx * ny * (c->periodic ? 2 : 1);
      phys_combine(3, (const double*)tv, (const double*)h.bc_ortho, nullptr, 0, 0, (double*)tv, nd, st);
      space_gradient(c->sp_field, tv, g, 0, 1, nullptr, c->tmp, st);
      phys_combine(4, (const double*)g, nullptr, nullptr, -(1.0 / (c->scale[1] / 2.0)), 0, (double*)g, nd, st);
      space_backward(c->sp_field, g, c->phys[0], c->tmp, st);
      weighted_col_sums(c->phys[0], nx, ny, c->d_wx, 0, c->d_red, st);
      weighted_col_sums(c->phys[0], nx, ny, c->d_wx, ny - 1, c->d_red + 1, st);
      double r[2];
      cuda_check(cudaMemcpyAsync(r, c->d_red, 16, cudaMemcpyDeviceToHost, st), "d2h");
      c->sync();
      out = (r[1] + r[0]) / 2.0;
      break;
    }
    case RBC_NUVOL: {
      void* tv = c->spec_tmp[0];
      void* g = c->spec_tmp[1];
      space_to_ortho(c->sp_t, h.temp, tv, c->tmp, st);
      size_t nd = (size_t)h.mx * ny * (c->periodic ? 2 : 1);
      phys_combine(3, (const double*)tv, (const double*)h.bc_ortho, nullptr, 0, 0, (double*)tv, nd, st);
      space_backward(c->sp_field, tv, c->phys[0], c->tmp, st);  // T
      space_backward(c->sp_u, h.uy, c->phys[1], c->tmp, st);    // uy
      space_gradient(c->sp_field, tv, g, 0, 1, nullptr, c->tmp, st);
      phys_combine(6, (const double*)g, nullptr, nullptr, c->scale[1] * -1.0, 0, (double*)g, nd, st);
      space_backward(c->sp_field, g, c->phys[2], c->tmp, st);   // dT/dz
      phys_combine(0, c->phys[2], c->phys[0], c->phys[1], c->ka, c->scale[1], c->phys[3], nphys, st);
      weighted_sum(c->phys[3], nx, ny, c->d_wx, c->d_wy, c->d_red, st);
      cuda_check(cudaMemcpyAsync(&out, c->d_red, 8, cudaMemcpyDeviceToHost, st), "d2h");
      c->sync();
      break;
    }
    case RBC_RE:
    case RBC_KE: {
      space_backward(c->sp_u, h.ux, c->phys[0], c->tmp, st);
      space_backward(c->sp_u, h.uy, c->phys[1], c->tmp, st);
      if (what == RBC_RE)
        phys_combine(1, c->phys[0], c->phys[1], nullptr, 2.0 * c->scale[1] / c->nu, 0, c->phys[2], nphys, st);
      else phys_combine(2, c->phys[0], c->phys[1], nullptr, 0, 0, c->phys[2], nphys, st);
      weighted_sum(c->phys[2], nx, ny, c->d_wx, c->d_wy, c->d_red, st);
      cuda_check(cudaMemcpyAsync(&out, c->d_red, 8, cudaMemcpyDeviceToHost, st), "d2h");
      c->sync();
      break;
    }
    case RBC_DIV_NORM: {
      void* a = c->spec_tmp[0];
      void* b = c->spec_tmp[1];
      space_gradient(c->sp_u, h.ux, a, 1, 0, c->scale, c->tmp, st);
      space_gradient(c->sp_u, h.uy, b, 0, 1, c->scale, c->tmp, st);
      size_t nd = (size_t)h.mx * ny * (c->periodic ? 2 : 1);
      phys_combine(3, (const double*)a, (const double*)b, nullptr, 0, 0, (double*)a, nd, st);
      sum_squares((const double*)a, nd, c->d_red, st);
      cuda_check(cudaMemcpyAsync(&out, c->d_red, 8, cudaMemcpyDeviceToHost, st), "d2h");
      c->sync();
      out = std::sqrt(out);
      break;
    }
    default:
      throw ApiError(RBC_ERR_INVALID, "unknown diagnostic id");
  }
  return out;
}

}  // namespace

extern "C" {

const char* rbc_last_error(void) { return g_err.c_str(); }
const char* rbc_version(void) { return "spectral_rbc 0.1 (sm_103a, FP64 step)"; }

static void validate_params(const RbcParams& p) {
  require(p.kind >= 0 && p.kind <= 2, "rbc_create: unknown kind");
  require(p.ra > 0 && p.pr > 0 && p.dt > 0 && p.aspect > 0, "rbc_create: ra, pr, dt, aspect must be positive");
  require(p.ny >= 8 && p.ny <= 4097, "rbc_create: ny must be in [8, 4097]");
  if (p.kind == RBC_PERIODIC)
    require(p.nx >= 8 && p.nx <= 8192 && is_pow2(p.nx), "rbc_create: periodic nx must be a power of two in [8, 8192]");
  else require(p.nx >= 8 && p.nx <= 4097, "rbc_create: nx must be in [8, 4097]");
  if (p.precision != RBC_PREC_FP64)
    throw ApiError(RBC_ERR_UNSUPPORTED, "rbc_create: single cases run in FP64; mixed precision is a batch form");
}

int rbc_create(const RbcParams* params, RbcCase** out) {
  API_BEGIN
  require(params != nullptr && out != nullptr, "rbc_create: null argument");
  *out = nullptr;
  const RbcParams& p = *params;
  validate_params(p);
  cuda_check(configure_prim_kernels(), "configure kernels");
  std::unique_ptr<RbcCase> c(new RbcCase());
  c->p = p;
  c->periodic = p.kind == RBC_PERIODIC;
  cuda_check(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream create");
  build_case(c.get());
  *out = c.release();
  API_END
}

int rbc_destroy(RbcCase* c) {
  API_BEGIN
  require(c == nullptr || !c->in_batch, "rbc_destroy: the case belongs to a batch (destroy the batch)");
  delete c;
  API_END
}

int rbc_get_params(const RbcCase* c, double out[7]) {
  API_BEGIN
  require(c && out, "rbc_get_params: null argument");
  double v[7] = {c->nu, c->ka, c->p.ra, c->p.pr, c->p.dt, c->scale[0], c->scale[1]};
  std::memcpy(out, v, sizeof v);
  API_END
}

int rbc_set_velocity(RbcCase* c, double amp, double m, double n) {
  API_BEGIN
  require(c != nullptr, "null case");
  apply_mode(c, RBC_UX, amp, m, n, true);
  apply_mode(c, RBC_UY, -amp, m, n, false);
  API_END
}

int rbc_set_temperature(RbcCase* c, double amp, double m, double n) {
  API_BEGIN
  require(c != nullptr, "null case");
  apply_mode(c, RBC_TEMP, -amp, m, n, false);
  API_END
}

int rbc_set_temperature_noise(RbcCase* c, double amp, uint64_t seed) {
  API_BEGIN
  require(c != nullptr, "null case");
  int nx = c->p.nx, ny = c->p.ny;
  std::vector<double> v((size_t)nx * ny);
  uint64_t s = seed;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) {
      double u = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
      bool wall = (j == 0 || j == ny - 1) || (!c->periodic && (i == 0 || i == nx - 1));
      v[(size_t)i * ny + j] = wall ? 0.0 : amp * (2.0 * u - 1.0);
    }
  set_phys(c, RBC_TEMP, v);
  API_END
}

int rbc_random_disturbance(RbcCase* c, double amp, uint64_t seed) {
  // navier.rs:939-948 / 1079-1090 with a seeded uniform(-amp, amp)
  API_BEGIN
  require(c != nullptr, "null case");
  int nx = c->p.nx, ny = c->p.ny;
  uint64_t s = seed;
  std::vector<double> v((size_t)nx * ny);
  std::vector<double> t;
  for (int f : {RBC_TEMP, RBC_UX, RBC_UY}) {
    for (auto& e : v) {
      double u = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
      e = amp * (2.0 * u - 1.0);
    }
    set_phys(c, f, v);
    if (f == RBC_TEMP) t = v;
  }
  // temp.v = temp.v - fieldbc.v; temp.forward()
  std::vector<double> bc((size_t)nx * ny);
  cuda_check(cudaMemcpy(bc.data(), c->bc_phys, bc.size() * 8, cudaMemcpyDeviceToHost), "d2h");
  for (size_t i = 0; i < t.size(); i++) t[i] = t[i] - bc[i];
  set_phys(c, RBC_TEMP, t);
  API_END
}

int rbc_step(RbcCase* c, int nsteps) {
  API_BEGIN
  require(c != nullptr && nsteps >= 0, "rbc_step: invalid argument");
  require(c->gexec != nullptr, "rbc_step: the case belongs to a batch (use rbc_batch_step)");
  for (int s = 0; s < nsteps; s++) {
    cuda_check(cudaGraphLaunch(c->gexec, c->stream), "graph launch");
    c->time += c->p.dt;
  }
  API_END
}

int rbc_synchronize(RbcCase* c) {
  API_BEGIN
  require(c != nullptr, "null case");
  c->sync();
  API_END
}

int rbc_get_time(const RbcCase* c, double* t) {
  API_BEGIN
  require(c && t, "null argument");
  *t = c->time;
  API_END
}
int rbc_set_time(RbcCase* c, double t) {
  API_BEGIN
  require(c != nullptr, "null case");
  c->time = t;
  API_END
}
int rbc_get_dt(const RbcCase* c, double* dt) {
  API_BEGIN
  require(c && dt, "null argument");
  *dt = c->p.dt;
  API_END
}

int rbc_status(RbcCase* c, int* status) {
  API_BEGIN
  require(c && status, "null argument");
  unsigned int s = 0;
  cuda_check(cudaMemcpyAsync(&s, c->hd.status, 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
  c->sync();
  *status = (int)s;
  API_END
}

int rbc_exit(RbcCase* c, int* stop) {
  API_BEGIN
  require(c && stop, "null argument");
  double d = eval_case(c, RBC_DIV_NORM);
  *stop = std::isnan(d) ? 1 : 0;
  API_END
}

int rbc_integrate(RbcCase* c, double max_time, double save_intervall, rbc_callback cb, void* user,
                  long* steps_done) {
  // lib.rs:155-187
  API_BEGIN
  require(c != nullptr, "null case");
  const long MAX_TIMESTEP = 10000000;
  long timestep = 0;
  require(c->gexec != nullptr, "rbc_integrate: the case belongs to a batch (use rbc_batch_step)");
  double dt = c->p.dt;
  double eps_dt = dt * 1e-4;
  while (true) {
    cuda_check(cudaGraphLaunch(c->gexec, c->stream), "graph launch");
    c->time += dt;
    timestep++;
    if (save_intervall > 0 && cb) {
      double r = std::fmod(c->time, save_intervall);
      if (r < dt / 2.0 || r > save_intervall - dt / 2.0) {
        c->sync();
        if (cb(c, c->time, user) != 0) break;
      }
    }
    if (c->time + eps_dt >= max_time) break;
    if (timestep >= MAX_TIMESTEP) break;
    unsigned int s = 0;
    cuda_check(cudaMemcpyAsync(&s, c->hd.status, 4, cudaMemcpyDeviceToHost, c->stream), "d2h");
    c->sync();
    if (s & 1u) {
      int stop = 0;
      double d = eval_case(c, RBC_DIV_NORM);
      stop = std::isnan(d);
      if (stop) break;
    }
  }
  c->sync();
  if (steps_done) *steps_done = timestep;
  API_END
}

int rbc_field_shape(const RbcCase* c, int field, int* n0, int* n1, int* is_complex) {
  API_BEGIN
  require(c && n0 && n1 && is_complex, "null argument");
  const SpaceDev& s = field_space(c, field);
  *n0 = s.spec0;
  *n1 = s.spec1;
  *is_complex = s.cplx ? 1 : 0;
  API_END
}

int rbc_get_state(RbcCase* c, int field, double* host, size_t n_doubles) {
  API_BEGIN
  require(c && host, "null argument");
  size_t n = spec_doubles(c, field);
  require(n_doubles == n, "rbc_get_state: size mismatch, expected " + std::to_string(n));
  cuda_check(cudaMemcpyAsync(host, field_ptr(c, field), n * 8, cudaMemcpyDeviceToHost, c->stream), "d2h");
  c->sync();
  API_END
}

int rbc_set_state(RbcCase* c, int field, const double* host, size_t n_doubles) {
  API_BEGIN
  require(c && host, "null argument");
  require(field != RBC_FIELDBC, "rbc_set_state: fieldbc is read only");
  size_t n = spec_doubles(c, field);
  require(n_doubles == n, "rbc_set_state: size mismatch, expected " + std::to_string(n));
  cuda_check(cudaMemcpyAsync(field_ptr(c, field), host, n * 8, cudaMemcpyHostToDevice, c->stream), "h2d");
  c->sync();
  API_END
}

int rbc_get_physical(RbcCase* c, int field, double* host, size_t n_doubles) {
  API_BEGIN
  require(c && host, "null argument");
  size_t n = (size_t)c->p.nx * c->p.ny;
  require(n_doubles == n, "rbc_get_physical: size mismatch, expected " + std::to_string(n));
  space_backward(field_space(c, field), field_ptr(c, field), c->phys[0], c->tmp, c->stream);
  cuda_check(cudaMemcpyAsync(host, c->phys[0], n * 8, cudaMemcpyDeviceToHost, c->stream), "d2h");
  c->sync();
  API_END
}

int rbc_get_coords(const RbcCase* c, int field, double* x, double* y) {
  API_BEGIN
  require(c && x && y, "null argument");
  std::vector<double> xs, ys;
  coords(c, field, xs, ys);
  std::memcpy(x, xs.data(), xs.size() * 8);
  std::memcpy(y, ys.data(), ys.size() * 8);
  API_END
}

int rbc_eval(RbcCase* c, int what, double* out) {
  API_BEGIN
  require(c && out, "null argument");
  *out = eval_case(c, what);
  API_END
}

int rbc_get_stream(RbcCase* c, void** stream) {
  API_BEGIN
  require(c && stream, "null argument");
  *stream = (void*)c->stream;
  API_END
}

int rbc_device_bytes(const RbcCase* c, size_t* bytes) {
  API_BEGIN
  require(c && bytes, "null argument");
  *bytes = c->arena.bytes();
  API_END
}

// ---------------------------------------------------------------- batches
}  // extern "C"

struct RbcBatch {
  std::vector<RbcCase*> cases;
  cudaStream_t stream = nullptr;
  std::vector<cudaStream_t> branch;
  std::vector<cudaEvent_t> events;
  Arena arena;
  CaseDev* d_cases = nullptr;
  struct Bucket {
    int kind, nx, ny;
    std::vector<int> members;
    StepPlan plan;
    std::vector<int4*> d_work;
  };
  std::vector<Bucket> buckets;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int launches = 0;
  ~RbcBatch() {
    if (stream) cudaStreamSynchronize(stream);
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    for (RbcCase* c : cases) delete c;
    for (auto e : events) cudaEventDestroy(e);
    for (auto s : branch) cudaStreamDestroy(s);
    if (stream) cudaStreamDestroy(stream);
  }
};

extern "C" {

int rbc_batch_create(const RbcParams* params, int ncases, RbcBatch** out) {
  API_BEGIN
  require(params != nullptr && out != nullptr && ncases > 0, "rbc_batch_create: invalid argument");
  *out = nullptr;
  for (int i = 0; i < ncases; i++) validate_params(params[i]);
  cuda_check(configure_prim_kernels(), "configure kernels");
  std::unique_ptr<RbcBatch> b(new RbcBatch());
  cuda_check(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream create");
  for (int i = 0; i < ncases; i++) {
    std::unique_ptr<RbcCase> c(new RbcCase());
    c->p = params[i];
    c->periodic = params[i].kind == RBC_PERIODIC;
    c->stream = b->stream;
    c->own_stream = false;
    c->in_batch = true;
    build_case(c.get(), false);
    b->cases.push_back(c.release());
  }
  // device table of all case descriptors
  std::vector<CaseDev> hd;
  for (RbcCase* c : b->cases) hd.push_back(c->hd);
  b->d_cases = b->arena.upload(hd);
  // buckets of equal (kind, nx, ny)
  for (int i = 0; i < ncases; i++) {
    const RbcParams& p = params[i];
    int kind = p.kind == RBC_PERIODIC ? 2 : 0;  // both box kinds share kernels
    int found = -1;
    for (size_t k = 0; k < b->buckets.size(); k++)
      if (b->buckets[k].kind == kind && b->buckets[k].nx == p.nx && b->buckets[k].ny == p.ny) found = (int)k;
    if (found < 0) {
      RbcBatch::Bucket bk;
      bk.kind = kind;
      bk.nx = p.nx;
      bk.ny = p.ny;
      b->buckets.push_back(bk);
      found = (int)b->buckets.size() - 1;
    }
    b->buckets[found].members.push_back(i);
  }
  for (auto& bk : b->buckets) {
    const RbcCase* first = b->cases[bk.members[0]];
    bk.plan = first->plan;
    for (auto& L : bk.plan.launches) {
      std::vector<int4> items;
      size_t lanes = L.items.size();
      items.reserve(lanes * bk.members.size());
      for (size_t li = 0; li < lanes; li++)
        for (int m : bk.members) items.push_back(make_int4(m, L.items[li].y, L.items[li].z, L.items[li].w));
      L.items = items;
      bk.d_work.push_back(b->arena.upload(items));
    }
  }
  cuda_check(cudaDeviceSynchronize(), "batch set-up");
  // graph: one branch per bucket
  size_t nb = b->buckets.size();
  b->branch.resize(nb);
  b->events.resize(nb + 1);
  for (size_t k = 0; k < nb; k++) cuda_check(cudaStreamCreateWithFlags(&b->branch[k], cudaStreamNonBlocking), "stream");
  for (auto& e : b->events) cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
  cuda_check(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  cudaError_t le = cudaEventRecord(b->events[nb], b->stream);
  for (size_t k = 0; k < nb && le == cudaSuccess; k++) {
    auto& bk = b->buckets[k];
    cudaStream_t s = b->branch[k];
    le = cudaStreamWaitEvent(s, b->events[nb], 0);
    for (size_t li = 0; li < bk.plan.launches.size() && le == cudaSuccess; li++) {
      auto& L = bk.plan.launches[li];
      le = launch_step_kernel(L.kernel, (int)L.items.size(), L.smem, s, b->d_cases, bk.d_work[li]);
      b->launches++;
    }
    if (le == cudaSuccess) le = cudaEventRecord(b->events[k], s);
    if (le == cudaSuccess) le = cudaStreamWaitEvent(b->stream, b->events[k], 0);
  }
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
  cuda_check(le, "batch capture");
  cuda_check(ce, "end capture");
  b->graph = g;
  cuda_check(cudaGraphInstantiate(&b->gexec, g, 0), "graph instantiate");
  *out = b.release();
  API_END
}

int rbc_batch_destroy(RbcBatch* b) {
  API_BEGIN
  delete b;
  API_END
}
int rbc_batch_size(const RbcBatch* b, int* n) {
  API_BEGIN
  require(b && n, "null argument");
  *n = (int)b->cases.size();
  API_END
}
int rbc_batch_case(RbcBatch* b, int i, RbcCase** c) {
  API_BEGIN
  require(b && c && i >= 0 && i < (int)b->cases.size(), "rbc_batch_case: invalid argument");
  *c = b->cases[i];
  API_END
}
int rbc_batch_step(RbcBatch* b, int nsteps) {
  API_BEGIN
  require(b && nsteps >= 0, "rbc_batch_step: invalid argument");
  for (int s = 0; s < nsteps; s++) {
    cuda_check(cudaGraphLaunch(b->gexec, b->stream), "graph launch");
    for (RbcCase* c : b->cases) c->time += c->p.dt;
  }
  API_END
}
int rbc_batch_synchronize(RbcBatch* b) {
  API_BEGIN
  require(b != nullptr, "null batch");
  cuda_check(cudaStreamSynchronize(b->stream), "stream synchronize");
  API_END
}
int rbc_batch_layout(const RbcBatch* b, int* nbuckets, int* launches) {
  API_BEGIN
  require(b && nbuckets && launches, "null argument");
  *nbuckets = (int)b->buckets.size();
  *launches = b->launches;
  API_END
}
int rbc_batch_get_stream(RbcBatch* b, void** stream) {
  API_BEGIN
  require(b && stream, "null argument");
  *stream = (void*)b->stream;
  API_END
}

int rbc_profile_step(RbcCase* c, int nsteps, double* stage_ms, int max_stages, int* nstages) {
  API_BEGIN
  require(c && stage_ms && nstages && nsteps > 0, "rbc_profile_step: invalid argument");
  require(!c->in_batch, "rbc_profile_step: the case belongs to a batch");
  int ns = (int)c->plan.launches.size();
  *nstages = ns;
  std::vector<cudaEvent_t> ev(ns + 1);
  for (auto& e : ev) cuda_check(cudaEventCreate(&e), "event create");
  std::vector<double> acc(ns, 0.0);
  for (int s = 0; s < nsteps; s++) {
    cuda_check(cudaEventRecord(ev[0], c->stream), "event record");
    for (int k = 0; k < ns; k++) {
      auto& L = c->plan.launches[k];
      cuda_check(launch_step_kernel(L.kernel, (int)L.items.size(), L.smem, c->stream, c->d_case, c->d_work[k]),
                 "stage launch");
      cuda_check(cudaEventRecord(ev[k + 1], c->stream), "event record");
    }
    c->time += c->p.dt;
    c->sync();
    for (int k = 0; k < ns; k++) {
      float ms = 0.f;
      cuda_check(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]), "elapsed");
      acc[k] += ms;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  for (int k = 0; k < ns && k < max_stages; k++) stage_ms[k] = acc[k] / nsteps;
  API_END
}

const char* rbc_stage_name(const RbcCase* c, int k) {
  static const char* names[] = {"y1_complex", "y1_real", "periodic_x", "periodic_y2", "box_x1", "box_y2",
                                "box_x2", "box_y3", "box_x3", "box_y4", "box_x4", "box_y5", "periodic_y2a",
                                "periodic_y2b"};
  if (!c || k < 0 || k >= (int)c->plan.launches.size()) return "";
  int id = c->plan.launches[k].kernel;
  return (id >= 0 && id < 14) ? names[id] : "";
}

// ---- device memory helpers
int rbc_host_alloc_pinned(void** ptr, size_t bytes) {
  API_BEGIN
  require(ptr != nullptr, "null argument");
  cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) throw ApiError(RBC_ERR_NOMEM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
  API_END
}
int rbc_host_free_pinned(void* ptr) {
  API_BEGIN
  cuda_check(cudaFreeHost(ptr), "cudaFreeHost");
  API_END
}
int rbc_dev_alloc(void** ptr, size_t bytes) {
  API_BEGIN
  require(ptr != nullptr, "null argument");
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) throw ApiError(RBC_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  API_END
}
int rbc_dev_free(void* ptr) {
  API_BEGIN
  cuda_check(cudaFree(ptr), "cudaFree");
  API_END
}
int rbc_memcpy_h2d(void* dst, const void* src, size_t bytes) {
  API_BEGIN
  cuda_check(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "cudaMemcpy h2d");
  API_END
}
int rbc_memcpy_d2h(void* dst, const void* src, size_t bytes) {
  API_BEGIN
  cuda_check(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost), "cudaMemcpy d2h");
  API_END
}
int rbc_device_synchronize(void) {
  API_BEGIN
  cuda_check(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
  API_END
}

// ---- funspace primitives
int fs_space_create(int base0, int n0, int base1, int n1, FsSpace** out) {
  API_BEGIN
  require(out != nullptr, "null argument");
  *out = nullptr;
  require(base0 >= 0 && base0 <= 5 && base1 >= 0 && base1 <= 4, "fs_space_create: unknown base (Fourier along axis 0 only)");
  require(n0 >= 4 && n1 >= 4 && n0 <= 8192 && n1 <= 8192, "fs_space_create: sizes must be in [4, 8192]");
  if (base0 == FS_FOURIER_R2C) require(is_pow2(n0), "fs_space_create: Fourier length must be a power of two");
  cuda_check(configure_prim_kernels(), "configure kernels");
  std::unique_ptr<FsSpace> s(new FsSpace());
  build_space(s->arena, s->s, base0, n0, base1, n1);
  s->tmp = s->arena.alloc(tmp_elems(s->s) * 16);
  *out = s.release();
  API_END
}
int fs_space_destroy(FsSpace* s) {
  API_BEGIN
  delete s;
  API_END
}
int fs_space_shape(const FsSpace* s, int which, int* n0, int* n1, int* is_complex) {
  API_BEGIN
  require(s && n0 && n1 && is_complex, "null argument");
  const SpaceDev& d = s->s;
  if (which == FS_PHYSICAL) { *n0 = d.phys0; *n1 = d.phys1; *is_complex = 0; }
  else if (which == FS_SPECTRAL) { *n0 = d.spec0; *n1 = d.spec1; *is_complex = d.cplx; }
  else if (which == FS_ORTHO) { *n0 = d.ortho0; *n1 = d.ortho1; *is_complex = d.cplx; }
  else throw ApiError(RBC_ERR_INVALID, "fs_space_shape: unknown selector");
  API_END
}
#define FS_CHECK(p) require((p) != nullptr, "null argument")
int fs_forward(FsSpace* s, const double* d_phys, double* d_spec, void* stream) {
  API_BEGIN
  FS_CHECK(s); FS_CHECK(d_phys); FS_CHECK(d_spec);
  space_forward(s->s, d_phys, d_spec, s->tmp, (cudaStream_t)stream);
  API_END
}
int fs_backward(FsSpace* s, const double* d_spec, double* d_phys, void* stream) {
  API_BEGIN
  FS_CHECK(s); FS_CHECK(d_phys); FS_CHECK(d_spec);
  space_backward(s->s, d_spec, d_phys, s->tmp, (cudaStream_t)stream);
  API_END
}
int fs_to_ortho(FsSpace* s, const double* d_spec, double* d_ortho, void* stream) {
  API_BEGIN
  FS_CHECK(s); FS_CHECK(d_spec); FS_CHECK(d_ortho);
  space_to_ortho(s->s, d_spec, d_ortho, s->tmp, (cudaStream_t)stream);
  API_END
}
int fs_from_ortho(FsSpace* s, const double* d_ortho, double* d_spec, void* stream) {
  API_BEGIN
  FS_CHECK(s); FS_CHECK(d_spec); FS_CHECK(d_ortho);
  space_from_ortho(s->s, d_ortho, d_spec, s->tmp, (cudaStream_t)stream);
  API_END
}
int fs_gradient(FsSpace* s, const double* d_spec, double* d_ortho, int deriv0, int deriv1, const double* scale,
                void* stream) {
  API_BEGIN
  FS_CHECK(s); FS_CHECK(d_spec); FS_CHECK(d_ortho);
  require(deriv0 >= 0 && deriv0 <= 2 && deriv1 >= 0 && deriv1 <= 2, "fs_gradient: derivative order must be 0..2");
  space_gradient(s->s, d_spec, d_ortho, deriv0, deriv1, scale, s->tmp, (cudaStream_t)stream);
  API_END
}

}  // extern "C"

// ---- fs_forward_noalloc: fixed device scratch instead of the space's own.
// The buffer is a file-scope device array, so it exists as soon as the
// library's device code is loaded on a device; its address is looked up once
// per device and cached.
namespace {
static __device__ __align__(256) double g_noalloc_scratch[FS_NOALLOC_SCRATCH_BYTES / sizeof(double)];
constexpr int kNoallocMaxDevices = 64;
std::atomic<void*> g_noalloc_addr[kNoallocMaxDevices];

void* noalloc_scratch_for_current_device() {
  int dev = -1;
  cuda_check(cudaGetDevice(&dev), "fs_forward_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kNoallocMaxDevices)
    throw ApiError(RBC_ERR_UNSUPPORTED, "fs_forward_noalloc: device ordinal beyond 63");
  void* p = g_noalloc_addr[dev].load(std::memory_order_acquire);
  if (p) return p;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr)
    throw ApiError(RBC_ERR_CUDA, std::string("fs_forward_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  g_noalloc_addr[dev].store(p, std::memory_order_release);
  return p;
}
}  // namespace

extern "C" {

int fs_forward_noalloc(FsSpace* s, const double* d_phys, double* d_spec, void* stream) {
  API_BEGIN
  FS_CHECK(s); FS_CHECK(d_phys); FS_CHECK(d_spec);
  // intermediate of space_forward: phys0 x spec1 real values after the axis-1 pass
  const size_t need = (size_t)s->s.phys0 * (size_t)s->s.spec1 * sizeof(double);
  if (need > (size_t)FS_NOALLOC_SCRATCH_BYTES)
    throw ApiError(RBC_ERR_INVALID, "fs_forward_noalloc: the space needs " + std::to_string(need) +
                                        " bytes of scratch, more than the fixed " +
                                        std::to_string((size_t)FS_NOALLOC_SCRATCH_BYTES));
  void* scratch = noalloc_scratch_for_current_device();
  space_forward(s->s, d_phys, d_spec, scratch, (cudaStream_t)stream);
  API_END
}

int sv_create(FsSpace* s, int kind, const double c[2], SvSolver** out) {
  API_BEGIN
  require(s && c && out, "null argument");
  *out = nullptr;
  require(kind >= 0 && kind <= 2, "sv_create: unknown solver kind");
  std::unique_ptr<SvSolver> v(new SvSolver());
  v->space = s;
  std::string err;
  if (!build_solver(v->arena, s->s, kind, c, v->sv, &err)) throw ApiError(RBC_ERR_UNSUPPORTED, "sv_create: " + err);
  *out = v.release();
  API_END
}
int sv_destroy(SvSolver* sv) {
  API_BEGIN
  delete sv;
  API_END
}
int sv_solve(SvSolver* sv, const double* d_in, double* d_out, void* stream) {
  API_BEGIN
  require(sv && d_in && d_out, "null argument");
  solver_solve(sv->sv, sv->space->s, d_in, d_out, sv->space->tmp, (cudaStream_t)stream);
  API_END
}

}  // extern "C"
