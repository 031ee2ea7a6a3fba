// api.cu -- C ABI of the spectral RBC library (include/spectral_rbc.h).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "case_access.h"
#include "dense_ops.h"
#include "host_ops.h"
#include "lane_gemm.h"
#include "prims.h"
#include "trace.h"
#include "solid_masks.h"
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
int set_last_error(int code, const std::string& m) { return fail(code, m); }

#define API_BEGIN try {
#define API_END                                              \
  }                                                          \
  catch (ApiError & e) { return fail(e.code, e.what()); }    \
  catch (SizeError & e) { return fail(RBC_ERR_INVALID, e.what()); } \
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

// Device copies of a step plan: work tables of the lane kernels, job and tile
// tables of the tensor-core GEMM launches.  own: the tables' memory when the
// plan holds it itself (plans rebuilt during a case's life, on a solid mask
// change); replacing such a plan frees the old tables.
struct DevPlan {
  std::vector<int4*> work;
  std::vector<GemmJobDev*> jobs;
  std::vector<int4*> tiles;
  std::vector<int> ntiles, max_nt;
  std::shared_ptr<Arena> own;
};

static void upload_plan(Arena& A, const StepPlan& plan, DevPlan& dp) {
  dp = DevPlan();
  for (const StepLaunch& L : plan.launches) {
    int4* w = nullptr;
    GemmJobDev* j = nullptr;
    int4* t = nullptr;
    int nt = 0, mnt = 0;
    if (L.kernel == K_GEMM) {
      std::vector<int4> tiles;
      gemm_tiles(L.jobs, tiles);
      j = A.upload(L.jobs);
      t = A.upload(tiles);
      nt = (int)tiles.size();
      for (const GemmJobDev& g : L.jobs) mnt = std::max(mnt, g.NT);
    } else {
      w = A.upload(L.items);
    }
    dp.work.push_back(w);
    dp.jobs.push_back(j);
    dp.tiles.push_back(t);
    dp.ntiles.push_back(nt);
    dp.max_nt.push_back(mnt);
  }
}

// Upload a plan into memory of its own, replacing dp (and freeing the tables
// dp held itself).  No launch may still use dp's tables: the caller has
// synchronised the streams that ran them, and replaces the graphs that name
// them before the next step.
static void upload_plan_owned(const StepPlan& plan, DevPlan& dp) {
  auto mem = std::make_shared<Arena>();
  DevPlan fresh;
  upload_plan(*mem, plan, fresh);
  fresh.own = std::move(mem);
  dp = std::move(fresh);
}

static cudaError_t launch_entry(const StepLaunch& L, const DevPlan& dp, size_t k, cudaStream_t st,
                                const CaseDev* cases) {
  if (L.kernel == K_GEMM)
    return launch_lane_gemm(dp.jobs[k], dp.tiles[k], dp.ntiles[k], dp.max_nt[k], st, L.gemm_ws != 0);
  return launch_step_kernel(L.kernel, (int)L.items.size(), L.smem, st, cases, dp.work[k]);
}

// One plan for a group of cases of the same kind and precision (any sizes):
// each launch carries every member's work items (case index = the member's
// position in the case table) or GEMM jobs; its shared memory is the largest
// any member needs.  gates (optional): per member, the device flag that
// idles the member's GEMM jobs.
static StepPlan merge_plans(const std::vector<const StepPlan*>& plans, const std::vector<int>& case_index,
                            const std::vector<const int*>& gates) {
  StepPlan P = *plans[0];
  for (size_t li = 0; li < P.launches.size(); li++) {
    StepLaunch& L = P.launches[li];
    L.items.clear();
    L.jobs.clear();
    for (size_t m = 0; m < plans.size(); m++) {
      const StepLaunch& S = plans[m]->launches.at(li);
      if (S.kernel != L.kernel) throw std::runtime_error("merge_plans: plans of different structure");
      L.smem = std::max(L.smem, S.smem);
      for (const int4& it : S.items) L.items.push_back(make_int4(case_index[m], it.y, it.z, it.w));
      for (GemmJobDev j : S.jobs) {
        if (!gates.empty()) j.active = gates[m];
        L.jobs.push_back(j);
      }
    }
    // items that carry a cost (one-thread-per-lane kernels): most expensive
    // first, so the last CTAs to start are the cheapest
    if (!L.items.empty() && L.items[0].w > 0)
      std::stable_sort(L.items.begin(), L.items.end(), [](const int4& a, const int4& b) { return a.w > b.w; });
  }
  return P;
}

// Dense operator compositions of the mixed step (long double, before the
// split), shared by every case of a size.
enum MixedOpKind {
  MOP_BS_CD = 0,   // B S (Dirichlet composite -> physical)
  MOP_BDS_CD = 1,  // B D S (first derivative, physical)
  MOP_BS_CN = 2,   // the same for the Neumann composite basis
  MOP_BDS_CN = 3,
  MOP_FWD_23 = 4   // forward Chebyshev, rows < 2n/3 (one axis of the 2/3 truncation)
};
static std::mutex g_ops_mu;
static std::map<std::pair<int, int>, LMat> g_ops_cache;

static const LMat& mixed_operator(int which, int n) {
  std::lock_guard<std::mutex> lk(g_ops_mu);
  auto key = std::make_pair(which, n);
  auto it = g_ops_cache.find(key);
  if (it != g_ops_cache.end()) return it->second;
  LMat M;
  if (which == MOP_FWD_23) {
    M = lm_rows(lm_cheb_forward(n), 0, n * 2 / 3);
  } else {
    HostBasis b = make_basis(which <= MOP_BDS_CD ? CD : CN, n);
    LMat S = lm_stencil(b), Bk = lm_cheb_backward(n);
    if (which == MOP_BS_CD || which == MOP_BS_CN) M = lm_mul(Bk, S);
    else M = lm_mul(Bk, lm_mul(lm_cheb_diff(n), S));
  }
  return g_ops_cache.emplace(key, std::move(M)).first->second;
}

// Pack rows blocks [A0 * s0 ; A1 * s1 ; ...] (long double) as one split operand.
static const float* upload_op(Arena& a, std::initializer_list<std::pair<const LMat*, long double>> blocks,
                              int ntmax = 64) {
  int rows = 0, cols = -1;
  for (auto& b : blocks) {
    rows += b.first->rows;
    if (cols < 0) cols = b.first->cols;
    if (cols != b.first->cols) throw std::runtime_error("upload_op: column mismatch");
  }
  std::vector<double> W((size_t)rows * cols);
  size_t o = 0;
  for (auto& b : blocks)
    for (long double v : b.first->a) W[o++] = (double)(v * b.second);
  return a.upload(pack_gemm_w(W, rows, cols, gemm_tile_n(rows, ntmax)));
}

// Packed operators that depend on the size alone (the y transforms, the box's
// x forward transform and stencil-transform products, the Poisson eigenbases)
// are uploaded once per device and read by every case of that size: a batch of
// many cases of a few sizes then keeps one copy of each in L2 instead of one
// per case (every lane block of a GEMM re-reads its operator chunk by chunk).
// They stay allocated until the process exits, a few MB per distinct size, and
// are not counted against a serving budget.
static std::mutex g_shared_ops_mu;
static std::map<std::pair<int, std::string>, const float*> g_shared_ops;

template <class Make>
static const float* shared_op(const std::string& key, Make make) {
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "get device");
  std::lock_guard<std::mutex> lk(g_shared_ops_mu);
  auto it = g_shared_ops.find({dev, key});
  if (it != g_shared_ops.end()) return it->second;
  const std::vector<float> pk = make();
  void* d = nullptr;
  cuda_check(cudaMalloc(&d, pk.size() * sizeof(float)), "cudaMalloc shared operator");
  cuda_check(cudaMemcpy(d, pk.data(), pk.size() * sizeof(float), cudaMemcpyHostToDevice), "shared operator");
  const float* p = static_cast<const float*>(d);
  g_shared_ops.emplace(std::make_pair(dev, key), p);
  return p;
}
static std::vector<float> pack_blocks(std::initializer_list<std::pair<const LMat*, long double>> blocks,
                                      int ntmax = 64) {
  int rows = 0, cols = -1;
  for (auto& b : blocks) {
    rows += b.first->rows;
    if (cols < 0) cols = b.first->cols;
    if (cols != b.first->cols) throw std::runtime_error("pack_blocks: column mismatch");
  }
  std::vector<double> W((size_t)rows * cols);
  size_t o = 0;
  for (auto& b : blocks)
    for (long double v : b.first->a) W[o++] = (double)(v * b.second);
  return pack_gemm_w(W, rows, cols, gemm_tile_n(rows, ntmax));
}
// shared-operator key of a packing for tiles of at most ntmax outputs
static std::string op_key(const std::string& k, int ntmax) {
  return ntmax == 64 ? k : k + ":nt" + std::to_string(ntmax);
}

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
  std::vector<StepPlan> plan_alts;  // mixed form in batches: the other forms of the passes (autotuned)
  DevPlan dp;
  MixedOps mops;
  MixedOps mops_w;  // mixed form in batches: the operators packed for 128-output GEMM tiles (a tuned form)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  double time = 0.0;
  bool own_stream = true;
  bool in_batch = false;
  int* gate_mem = nullptr;  // device int[2] used by the serving loop (CaseDev::gate)
  // Statistics (statistics.rs): averages in the `field` space, allocated on first use
  void* st_field[4] = {nullptr, nullptr, nullptr, nullptr};  // temp, ux, uy, nusselt (spectral)
  double st_tot_time = 0.0, st_avg_time = 0.0;
  long st_num_save = 0;
  // diagnostics series recorded by rbc_diag_record (navier.rs:826-838)
  std::vector<double> dg_time, dg_nu, dg_nuvol, dg_re;
  // solid mask (navier.rs:189-190): host copies of [mask, value] and the
  // device arrays [(-1/eta) mask | value] the x pass reads
  std::vector<double> solid_host[2];
  double* solid_mem = nullptr;
  struct RbcBatch* batch = nullptr;  // the batch a batch case belongs to (its descriptor is batch->d_cases[batch_index])
  int batch_index = -1;
  ~RbcCase() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    if (stream) {
      cudaStreamSynchronize(stream);
      if (own_stream) cudaStreamDestroy(stream);
    }
    if (solid_mem) cudaFree(solid_mem);
  }
  size_t spec_elem() const { return periodic ? 16 : 8; }
  void sync() { cuda_check(cudaStreamSynchronize(stream), "stream synchronize"); }
};

struct FsSpace {
  Arena arena;
  SpaceDev s;
  void* tmp = nullptr;
};

struct FsLanes {
  Arena arena;
  LanesDev L;
  int precision = RBC_PREC_FP64;
  // mixed form: packed split operators per FS_OP_* (device)
  const float* w[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  unsigned int* d_status = nullptr;
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

// Spectral state of a case: temp, ux, uy, pres[0], pres[1] (each rounded up
// to 256 bytes).  sizes[k] receives the unpadded bytes of array k.
static size_t state_layout(const RbcParams& p, size_t sizes[5]) {
  const bool per = p.kind == RBC_PERIODIC;
  const size_t es = per ? 16 : 8;
  const size_t mx = per ? (size_t)p.nx / 2 + 1 : (size_t)p.nx;
  const size_t mxc = per ? mx : (size_t)p.nx - 2;
  const size_t nstate = mxc * (size_t)(p.ny - 2);
  sizes[0] = sizes[1] = sizes[2] = sizes[4] = nstate * es;
  sizes[3] = mx * (size_t)p.ny * es;
  size_t t = 0;
  for (int k = 0; k < 5; k++) t += (sizes[k] + 255) & ~size_t(255);
  return t;
}

void capture_graph(RbcCase* c);

// state_region: optional device region of state_layout() bytes that holds the
// case's spectral state (a batch keeps all its cases' state contiguous).
// with_graph: a case stepped on its own (rbc_create): its plan and CUDA graph
// are built here; batches and the serving loop (with_graph = false) merge the
// plans of many cases and use the one-thread-per-lane FP64 kernels.
void build_case(RbcCase* c, bool with_graph = true, char* state_region = nullptr) {
  const RbcParams& p = c->p;
  Arena& A = c->arena;
  const int nx = p.nx, ny = p.ny;
  const bool per = c->periodic;
  c->scale[0] = p.aspect;
  c->scale[1] = 1.0;
  // the packed operators of the mixed form: tiles of at most 64 outputs, and
  // in batches also 128 (the autotuner times both)
  c->mops_w.ntmax = 128;
  std::vector<MixedOps*> mixed_sets{&c->mops};
  if (!with_graph) mixed_sets.push_back(&c->mops_w);
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
  // Shared memory of the step's CTA passes, before the set-up work (a size
  // the kernels cannot run is refused at once).  A Chebyshev transform through
  // an FFT keeps 2(n-1) complex work elements per lane there; where a pass
  // then exceeds the device's limit, that axis uses the dense transform (an
  // n x n product per lane), x first (the box x pass holds the most lanes).
  // Only sizes and transform forms enter those amounts.
  {
    CaseDev hs = h;
    hs.mixed = p.precision == RBC_PREC_MIXED;
    auto need_of = [&](int* kernel) {
      if (hs.mixed) return mixed_plan_smem(hs, kernel);
      size_t m = 0;
      for (const StepLaunch& L : build_step_plan(hs).launches)
        if (L.smem > m) { m = L.smem; *kernel = L.kernel; }
      return m;
    };
    int kern = -1;
    for (int axis = per ? 1 : 0; axis < 2 && need_of(&kern) > smem_limit(); axis++) {
      ChebXformDev& cx = axis == 0 ? h.cx : h.cy;
      if (!cx.use_fft) continue;
      cx = upload_cheb(A, axis == 0 ? nx : ny, false);
      (axis == 0 ? hs.cx : hs.cy) = cx;
    }
    const size_t need = need_of(&kern);
    if (need > smem_limit())
      throw SizeError("rbc_create: a " + std::to_string(nx) + " x " + std::to_string(ny) + " case needs " +
                      std::to_string(need) + " bytes of shared memory per block in its " + step_kernel_name(kern) +
                      " pass; this device allows " + std::to_string(smem_limit()));
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
    if (p.precision == RBC_PREC_MIXED) {
      const int mxc = nx - 2;
      // the eigenbasis depends on the basis and the size only
      const std::string k = "pois" + std::to_string(c->sp_p1.hb0.kind) + ":" + std::to_string(mxc);
      for (MixedOps* o : mixed_sets) {
        const int nt = o->ntmax;
        o->pf = shared_op(op_key(k + ":fwd", nt), [&] { return pack_gemm_w(fwd, mxc, mxc, gemm_tile_n(mxc, nt)); });
        o->pb = shared_op(op_key(k + ":bwd", nt), [&] { return pack_gemm_w(bwd, mxc, mxc, gemm_tile_n(mxc, nt)); });
      }
    }
  }
  const size_t es = c->spec_elem();
  const size_t nstate = (size_t)h.mxc * h.myc;
  if (state_region) {
    size_t sz[5];
    state_layout(p, sz);
    void* arr[5];
    char* q = state_region;
    for (int k = 0; k < 5; k++) {
      arr[k] = q;
      q += (sz[k] + 255) & ~size_t(255);
    }
    h.temp = arr[0]; h.ux = arr[1]; h.uy = arr[2]; h.p0 = arr[3]; h.p1 = arr[4];
    cuda_check(cudaMemset(state_region, 0, (size_t)(q - state_region)), "clear state");
  } else {
    h.ux = A.alloc(nstate * es);
    h.uy = A.alloc(nstate * es);
    h.temp = A.alloc(nstate * es);
    h.p0 = A.alloc((size_t)h.mx * ny * es);
    h.p1 = A.alloc(nstate * es);
  }
  for (int k = 0; k < 6; k++) h.yw[k] = A.alloc((size_t)h.mxc * ny * es);
  h.q[0] = A.alloc((size_t)3 * std::max(h.kx, 1) * ny * es);
  if (!per)
    for (int k = 0; k < 8; k++) h.s[k] = A.alloc((size_t)nx * ny * 8);
  h.mixed = p.precision == RBC_PREC_MIXED;
  if (h.mixed) {
    for (int f = 0; f < 3; f++) h.m_y[f] = A.alloc((size_t)2 * ny * h.mx * 8);
    h.m_q = A.alloc((size_t)3 * ny * std::max(h.kx, 1) * 8);
    h.m_cv = A.alloc((size_t)3 * std::max(h.kx, 1) * h.ky * 16);
    // FP32 state copy: rows padded to 16 bytes, complex rows as [re | im] (rbc_dev.h)
    h.m_s32 = A.alloc((size_t)3 * h.mxc * s32_row_floats(h) * 4);
    h.m_bcx = static_cast<const float*>(A.alloc((size_t)nx * ny * 4));
    h.m_bcy = static_cast<const float*>(A.alloc((size_t)nx * ny * 4));
    for (MixedOps* o : mixed_sets) {
      const int nt = o->ntmax;
      o->y1 = shared_op(op_key("bs_bds_cd:" + std::to_string(ny), nt), [&] {
        return pack_blocks({{&mixed_operator(MOP_BS_CD, ny), 1.0L}, {&mixed_operator(MOP_BDS_CD, ny), 1.0L}}, nt);
      });
      o->y2 = shared_op(op_key("fwd23:" + std::to_string(ny), nt),
                        [&] { return pack_blocks({{&mixed_operator(MOP_FWD_23, ny), 1.0L}}, nt); });
    }
    if (!per) {
      for (int k = 0; k < 6; k++) h.m_ph[k] = A.alloc((size_t)2 * nx * ny * 4);
      for (int k = 0; k < 3; k++) h.m_p[k] = A.alloc((size_t)nx * ny * 4);
      h.m_z = A.alloc((size_t)nx * ny * 8);
      const long double inv_asp = 1.0L / (long double)p.aspect;
      const bool tn = p.kind == RBC_BOX_ADIABATIC;  // temperature: Neumann in x
      const LMat& bsu = mixed_operator(MOP_BS_CD, nx);
      const LMat& bdsu = mixed_operator(MOP_BDS_CD, nx);
      const LMat& bst = mixed_operator(tn ? MOP_BS_CN : MOP_BS_CD, nx);
      const LMat& bdst = mixed_operator(tn ? MOP_BDS_CN : MOP_BDS_CD, nx);
      // the derivative rows carry the aspect ratio (per case); the rest depends on the size only
      for (MixedOps* o : mixed_sets) {
        const int nt = o->ntmax;
        o->xa = upload_op(A, {{&bsu, 1.0L}, {&bdsu, inv_asp}}, nt);
        o->xb = shared_op(op_key("bs_cd:" + std::to_string(nx), nt), [&] { return pack_blocks({{&bsu, 1.0L}}, nt); });
        o->xc = upload_op(A, {{&bdst, inv_asp}}, nt);
        o->xd = shared_op(op_key(std::string(tn ? "bs_cn:" : "bs_cd:") + std::to_string(nx), nt),
                          [&] { return pack_blocks({{&bst, 1.0L}}, nt); });
        o->x2 = shared_op(op_key("fwd23:" + std::to_string(nx), nt),
                          [&] { return pack_blocks({{&mixed_operator(MOP_FWD_23, nx), 1.0L}}, nt); });
      }
    }
  }
  void* bco = A.alloc((size_t)h.mx * ny * es);
  void* bcd = A.alloc((size_t)h.mx * ny * es);
  double* bdx = static_cast<double*>(A.alloc((size_t)nx * ny * 8));
  double* bdy = static_cast<double*>(A.alloc((size_t)nx * ny * 8));
  h.bc_ortho = bco;
  h.bc_diff = bcd;
  h.bc_dx = bdx;
  h.bc_dy = bdy;
  h.status = static_cast<unsigned int*>(A.alloc(16));
  c->gate_mem = static_cast<int*>(A.alloc(16));
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
  h.bc_v = c->bc_phys;
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
  // the arena's zero fills ran on the legacy stream (or were synchronised by a
  // stream-ordered arena); wait for them without waiting for other streams
  cuda_check(cudaStreamSynchronize(cudaStreamLegacy), "allocation");
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
    if (h.mixed) {
      // FP32 copies of the boundary-field derivatives, transposed (ny x nx)
      std::vector<double> hx((size_t)nx * ny), hy((size_t)nx * ny);
      cuda_check(cudaMemcpy(hx.data(), bdx, hx.size() * 8, cudaMemcpyDeviceToHost), "copy bc dx");
      cuda_check(cudaMemcpy(hy.data(), bdy, hy.size() * 8, cudaMemcpyDeviceToHost), "copy bc dy");
      // The boundary convection term u dbc/dx + v dbc/dy splits into g0 v,
      // with g0 the mean of dbc/dy, and the remainder u dbc/dx + v (dbc/dy - g0).
      // The FP32 products carry only the remainder (rounding-level for the
      // conduction profile, which is linear in y); the FP64 pass that forms the
      // temperature right-hand side adds g0 * dealias(to_ortho(uy)), the exact
      // forward transform of g0 v (rbc_dev.h m_bclin).
      double g0 = 0.0;
      for (double v : hy) g0 += v;
      g0 /= (double)hy.size();
      std::vector<float> tx((size_t)nx * ny), ty((size_t)nx * ny);
      for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
          tx[(size_t)j * nx + i] = (float)hx[(size_t)i * ny + j];
          ty[(size_t)j * nx + i] = (float)(hy[(size_t)i * ny + j] - g0);
        }
      cuda_check(cudaMemcpy(const_cast<float*>(h.m_bcx), tx.data(), tx.size() * 4, cudaMemcpyHostToDevice), "bc dx");
      cuda_check(cudaMemcpy(const_cast<float*>(h.m_bcy), ty.data(), ty.size() * 4, cudaMemcpyHostToDevice), "bc dy");
      h.m_bclin = 1;
      h.m_bcg = g0;
      cuda_check(cudaMemcpy(c->d_case, &h, sizeof(CaseDev), cudaMemcpyHostToDevice), "copy case descriptor");
    }
  }
  // ---- step plan, work tables and the CUDA graph of one update()
  cuda_check(configure_step_kernels(), "configure step kernels");
  if (h.mixed) cuda_check(configure_mixed_kernels(), "configure mixed kernels");
  auto make_plans = [&]() {
    if (h.mixed) {
      c->plan = build_mixed_plan(h, c->mops, 0);
      if (!with_graph) {  // forms 1-3 of the FP64 passes; GEMM forms 4 (128-output tiles), 5 (warp-specialised)
        MixedOps ws = c->mops;
        ws.ws = 1;
        c->plan_alts = {build_mixed_plan(h, c->mops, 1), build_mixed_plan(h, c->mops, 2),
                        build_mixed_plan(h, c->mops, 3), build_mixed_plan(h, c->mops_w, 0),
                        build_mixed_plan(h, ws, 0)};
      }
    } else {
      c->plan = build_step_plan(h);
    }
  };
  // the largest shared-memory working set of a launch (and its kernel)
  auto plan_smem = [&](int* kernel) {
    size_t m = 0;
    auto scan = [&](const StepPlan& P) {
      for (const StepLaunch& L : P.launches)
        if (L.smem > m) { m = L.smem; *kernel = L.kernel; }
    };
    scan(c->plan);
    for (const StepPlan& P : c->plan_alts) scan(P);
    return m;
  };
  make_plans();
  int kern = -1;
  const size_t need = plan_smem(&kern);  // checked before the set-up (above); the plans are the same
  if (need > smem_limit())
    throw SizeError("rbc_create: a " + std::to_string(nx) + " x " + std::to_string(ny) + " case needs " +
                    std::to_string(need) + " bytes of shared memory per block in its " + step_kernel_name(kern) +
                    " pass; this device allows " + std::to_string(smem_limit()));
  if (!with_graph) return;
  capture_graph(c);
}

// Upload the case's plan and capture one update() as a CUDA graph (replacing
// a previous graph).
void capture_graph(RbcCase* c) {
  cudaStream_t st = c->stream;
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->gexec = nullptr;
  c->graph = nullptr;
  upload_plan_owned(c->plan, c->dp);
  cuda_check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
  cudaError_t le = cudaSuccess;
  for (size_t k = 0; k < c->plan.launches.size(); k++) {
    cudaError_t e = launch_entry(c->plan.launches[k], c->dp, k, st, c->d_case);
    if (e != cudaSuccess && le == cudaSuccess) le = e;
  }
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamEndCapture(st, &g);
  cuda_check(le, "step kernel launch");
  cuda_check(ce, "end capture");
  c->graph = g;
  cuda_check(cudaGraphInstantiate(&c->gexec, g, 0), "graph instantiate");
}

}  // namespace

namespace rbc {
CaseAccess case_access(RbcCase* c) {
  CaseAccess a;
  a.temp = c->hd.temp;
  a.ux = c->hd.ux;
  a.uy = c->hd.uy;
  a.p0 = c->hd.p0;
  a.p1 = c->hd.p1;
  a.bc_vhat = c->bc_vhat;
  a.bc_phys = c->bc_phys;
  a.stream = c->stream;
  a.nu = c->nu;
  a.ka = c->ka;
  a.scale[0] = c->scale[0];
  a.scale[1] = c->scale[1];
  return a;
}
void case_enqueue_step(RbcCase* c, cudaStream_t st) {
  if (!c->gexec) throw std::runtime_error("case_enqueue_step: the case belongs to a batch");
  for (size_t k = 0; k < c->plan.launches.size(); k++)
    cuda_check(launch_entry(c->plan.launches[k], c->dp, k, st, c->d_case), "step kernel launch");
}
}  // namespace rbc

namespace {
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

// temperature = amp*(2u-1) at interior collocation points, 0 on the walls,
// u from splitmix64(seed) drawn in row-major order
void set_temperature_noise(RbcCase* c, double amp, uint64_t seed) {
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
    require(p.nx >= 8 && p.nx <= 8192, "rbc_create: periodic nx must be in [8, 8192]");
  else require(p.nx >= 8 && p.nx <= 4097, "rbc_create: nx must be in [8, 4097]");
  require(p.precision == RBC_PREC_FP64 || p.precision == RBC_PREC_MIXED, "rbc_create: unknown precision");

}

int rbc_create(const RbcParams* params, RbcCase** out) {
  API_BEGIN
  TraceRange tr("rbc_create");
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
  set_temperature_noise(c, amp, seed);
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
  TraceRange tr("rbc_step");
  require(c != nullptr && nsteps >= 0, "rbc_step: invalid argument");
  require(c->gexec != nullptr, "rbc_step: the case belongs to a batch (use rbc_batch_step)");
  for (int s = 0; s < nsteps; s++) {
    cuda_check(cudaGraphLaunch(c->gexec, c->stream), "graph launch");
    c->time += c->p.dt;
  }
  API_END
}

// a batch case's solid mask changed (defined with the batch)
static void batch_solid_changed(RbcCase* c);

// navier.rs:189-190 (`navier.solid = Some([mask, value])`) with the damping of
// conv_ux / conv_uy / conv_temp (navier.rs:551-560, 579-584, 603-608).
int rbc_set_solid(RbcCase* c, const double* mask, const double* value, size_t n_doubles) {
  API_BEGIN
  require(c != nullptr, "rbc_set_solid: null case");
  if (c->hd.mixed) throw ApiError(RBC_ERR_UNSUPPORTED, "rbc_set_solid: solid masks need RBC_PREC_FP64");
  if (c->in_batch && c->batch == nullptr)
    throw ApiError(RBC_ERR_UNSUPPORTED, "rbc_set_solid: the case belongs to a serving loop");
  const size_t np = (size_t)c->p.nx * c->p.ny;
  c->sync();
  if (mask == nullptr) {
    c->hd.solid_cm = nullptr;
    c->hd.solid_val = nullptr;
    c->solid_host[0].clear();
    c->solid_host[1].clear();
  } else {
    require(n_doubles == np, "rbc_set_solid: mask and value hold nx*ny doubles");
    const double eta = 1e-2;  // navier.rs:553, 581, 605
    std::vector<double> dev(2 * np);
    c->solid_host[0].assign(mask, mask + np);
    c->solid_host[1].assign(np, 0.0);
    if (value) c->solid_host[1].assign(value, value + np);
    for (size_t i = 0; i < np; i++) {
      dev[i] = (-1.0 / eta) * mask[i];
      dev[np + i] = c->solid_host[1][i];
    }
    if (!c->solid_mem) cuda_check(cudaMalloc(&c->solid_mem, 2 * np * 8), "cudaMalloc solid mask");
    cuda_check(cudaMemcpy(c->solid_mem, dev.data(), 2 * np * 8, cudaMemcpyHostToDevice), "upload solid mask");
    c->hd.solid_cm = c->solid_mem;
    c->hd.solid_val = c->solid_mem + np;
  }
  cuda_check(cudaMemcpy(c->d_case, &c->hd, sizeof(CaseDev), cudaMemcpyHostToDevice), "copy case descriptor");
  // the x pass's lane count (and shared memory) depends on the solid
  c->plan = build_step_plan(c->hd);
  if (c->batch != nullptr) batch_solid_changed(c);
  else capture_graph(c);
  API_END
}

int rbc_get_solid(const RbcCase* c, int* present, double* mask, double* value, size_t n_doubles) {
  API_BEGIN
  require(c != nullptr && present != nullptr, "rbc_get_solid: null argument");
  *present = c->solid_host[0].empty() ? 0 : 1;
  if (*present && (mask || value)) {
    const size_t np = c->solid_host[0].size();
    require(n_doubles == np, "rbc_get_solid: mask and value hold nx*ny doubles");
    if (mask) std::memcpy(mask, c->solid_host[0].data(), np * 8);
    if (value) std::memcpy(value, c->solid_host[1].data(), np * 8);
  }
  API_END
}

// ---- solid mask generators (src/navier/solid_masks.rs) ----------------------
int rbc_solid_cylinder_inner(const double* x, int nx, const double* y, int ny, double x0, double y0, double radius,
                             double* mask, double* value) {
  API_BEGIN
  require(x && y && mask && value && nx > 0 && ny > 0, "rbc_solid_cylinder_inner: invalid argument");
  require(radius > 0, "rbc_solid_cylinder_inner: radius must be positive");
  solid_cylinder_inner(x, nx, y, ny, x0, y0, radius, mask, value);
  API_END
}

int rbc_solid_roughness_sinusoid(const double* x, int nx, const double* y, int ny, double height, double wavenumber,
                                 double* mask, double* value) {
  API_BEGIN
  require(x && y && mask && value && nx > 0 && ny > 1, "rbc_solid_roughness_sinusoid: invalid argument");
  require(height > 0, "rbc_solid_roughness_sinusoid: height must be positive");
  solid_roughness_sinusoid(x, nx, y, ny, height, wavenumber, mask, value);
  API_END
}

int rbc_solid_porosity(const double* x, int nx, const double* y, int ny, double diameter, double porosity,
                       double* mask, double* value) {
  API_BEGIN
  require(x && y && mask && value && nx > 1 && ny > 1, "rbc_solid_porosity: invalid argument");
  require(diameter > 0 && porosity >= 0 && porosity <= 1, "rbc_solid_porosity: diameter > 0, porosity in [0, 1]");
  solid_porosity(x, nx, y, ny, diameter, porosity, mask, value);
  API_END
}

// solid_masks.rs:144-174: the porosity mask on a 513 x 513 Chebyshev grid,
// forward transform, the first (nx, ny) coefficients (broadcast_2d), backward
// transform on the (nx, ny) Chebyshev grid.  The transforms run on the GPU.
int rbc_solid_porosity_interpolate(int nx, int ny, double diameter, double porosity, double* mask, double* value) {
  API_BEGIN
  require(mask && value && nx >= 4 && ny >= 4 && nx <= 8192 && ny <= 8192,
          "rbc_solid_porosity_interpolate: invalid argument");
  require(diameter > 0 && porosity >= 0 && porosity <= 1, "rbc_solid_porosity_interpolate: diameter > 0, porosity in [0, 1]");
  cuda_check(configure_prim_kernels(), "configure kernels");
  const int nf = 513;
  Arena A;
  SpaceDev fine, coarse;
  build_space(A, fine, CHEB, nf, CHEB, nf);
  build_space(A, coarse, CHEB, nx, CHEB, ny);
  const size_t nff = (size_t)nf * nf, nc = (size_t)nx * ny;
  std::vector<double> hm(nff), hv(nff);
  solid_porosity(fine.hb0.x.data(), nf, fine.hb1.x.data(), nf, diameter, porosity, hm.data(), hv.data());
  double* d_phys = static_cast<double*>(A.alloc(nff * 8));
  double* d_spec = static_cast<double*>(A.alloc(nff * 8));
  double* d_cs = static_cast<double*>(A.alloc(nc * 8));
  double* d_out = static_cast<double*>(A.alloc(nc * 8));
  void* tmp = A.alloc(std::max(tmp_elems(fine), tmp_elems(coarse)) * 16);
  cuda_check(cudaDeviceSynchronize(), "allocation");
  const int r = std::min(nx, nf), q = std::min(ny, nf);
  double* outs[2] = {mask, value};
  const std::vector<double>* ins[2] = {&hm, &hv};
  for (int k = 0; k < 2; k++) {
    cuda_check(cudaMemcpy(d_phys, ins[k]->data(), nff * 8, cudaMemcpyHostToDevice), "upload mask");
    space_forward(fine, d_phys, d_spec, tmp, nullptr);
    cuda_check(cudaMemset(d_cs, 0, nc * 8), "clear");
    cuda_check(cudaMemcpy2D(d_cs, (size_t)ny * 8, d_spec, (size_t)nf * 8, (size_t)q * 8, r, cudaMemcpyDeviceToDevice),
               "truncate coefficients");
    space_backward(coarse, d_cs, d_out, tmp, nullptr);
    cuda_check(cudaMemcpy(outs[k], d_out, nc * 8, cudaMemcpyDeviceToHost), "download mask");
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
    if (s & kStatusGemmTimeout) {
      if (steps_done) *steps_done = timestep;
      throw ApiError(RBC_ERR_CUDA, "rbc_integrate: a tensor-core completion wait timed out (the step's results are "
                                   "incomplete)");
    }
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
  size_t n = c->arena.bytes();
  if (c->dp.own) n += c->dp.own->bytes();
  if (c->solid_mem) n += 2 * (size_t)c->p.nx * c->p.ny * sizeof(double);
  *bytes = n;
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
    DevPlan dp;
    size_t state_begin = 0, state_end = 0;  // the members' states: one contiguous range of d_state
    cudaGraph_t graph = nullptr;             // one step of this group alone (rbc_batch_step_io)
    cudaGraphExec_t gexec = nullptr;
  };
  std::vector<Bucket> buckets;
  bool use_priority = false;      // the critical group's branch captured at high priority
  std::vector<size_t> io_order;  // groups in the order their inputs are copied in: shortest step first
  std::vector<cudaEvent_t> io_events;  // a group's input copy done (rbc_batch_step_io)
  struct Tuned {
    int kernel_cta, kernel_lanes;
    float ms_cta, ms_lanes;
    int form;  // form kept: 0 CTA per lane, 1 to 4 the other plan variants
    bool gemm;  // a GEMM pass (its forms are tile widths)
  };
  std::vector<Tuned> tuning;          // autotuner decisions (rbc_batch_tuning)
  struct TransformChoice {
    int bucket;
    float ms_gemm, ms_butterfly;  // the group's step, launches timed alone
    bool butterfly;               // kept the butterfly (plain FP64) plan
  };
  std::vector<TransformChoice> transforms;  // groups of butterfly sizes (rbc_batch_tuning_forms, third part)
  char* d_state = nullptr;            // every case's spectral state, contiguous
  size_t state_bytes = 0;
  std::vector<size_t> state_offset;   // byte offset of case i in d_state
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int launches = 0;
  ~RbcBatch() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto& s : branch) cudaStreamSynchronize(s);
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& bk : buckets) {
      if (bk.gexec) cudaGraphExecDestroy(bk.gexec);
      if (bk.graph) cudaGraphDestroy(bk.graph);
    }
    for (RbcCase* c : cases) delete c;
    for (auto e : events) cudaEventDestroy(e);
    for (auto e : io_events) cudaEventDestroy(e);
    for (auto s : branch) cudaStreamDestroy(s);
    if (stream) cudaStreamDestroy(stream);
  }
};

// The batch step as CUDA graphs: one graph with a branch per group (the
// critical group's branch at high priority), and one graph per group for
// rbc_batch_step_io.  Earlier graphs are replaced.
static void batch_capture_graphs(RbcBatch* b) {
  const size_t nb = b->buckets.size();
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->gexec = nullptr;
  b->graph = nullptr;
  for (auto& bk : b->buckets) {
    if (bk.gexec) cudaGraphExecDestroy(bk.gexec);
    if (bk.graph) cudaGraphDestroy(bk.graph);
    bk.gexec = nullptr;
    bk.graph = nullptr;
  }
  b->launches = 0;
  cuda_check(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  cudaError_t le = cudaEventRecord(b->events[nb], b->stream);
  for (size_t k = 0; k < nb && le == cudaSuccess; k++) {
    auto& bk = b->buckets[k];
    cudaStream_t s = b->branch[k];
    le = cudaStreamWaitEvent(s, b->events[nb], 0);
    for (size_t li = 0; li < bk.plan.launches.size() && le == cudaSuccess; li++) {
      le = launch_entry(bk.plan.launches[li], bk.dp, li, s, b->d_cases);
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
  cuda_check(cudaGraphInstantiate(&b->gexec, g, b->use_priority ? cudaGraphInstantiateFlagUseNodePriority : 0),
             "graph instantiate");
  // rbc_batch_step_io: one graph per group, captured on the group's branch
  // stream (its priority), and the groups' inputs copied in shortest step
  // first: that group computes while the longer group's input arrives, and
  // its results go back while the longer group still runs (256-case ensemble:
  // 4.32 ms per step against 4.78 ms longest first, 5.3 ms with the copies
  // and the step in sequence)
  for (size_t k = 0; k < nb; k++) {
    auto& bk = b->buckets[k];
    cudaStream_t s = b->branch[k];
    cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaError_t e = cudaSuccess;
    for (size_t li = 0; li < bk.plan.launches.size() && e == cudaSuccess; li++)
      e = launch_entry(bk.plan.launches[li], bk.dp, li, s, b->d_cases);
    cudaGraph_t bg = nullptr;
    const cudaError_t be = cudaStreamEndCapture(s, &bg);
    bk.graph = bg;  // freed by the destructor whatever follows
    cuda_check(e, "group capture");
    cuda_check(be, "end capture");
    cuda_check(cudaGraphInstantiate(&bk.gexec, bg, b->use_priority ? cudaGraphInstantiateFlagUseNodePriority : 0),
               "graph instantiate");
  }
}

// A batch case's solid mask changed: its descriptor in the batch's table, its
// group's plan (the x pass's lanes and shared memory follow the mask) and the
// batch's graphs are rebuilt (FP64 groups; the mixed form has no solid lane).
static void batch_solid_changed(RbcCase* c) {
  RbcBatch* b = c->batch;
  cuda_check(cudaStreamSynchronize(b->stream), "stream synchronize");
  for (auto s : b->branch) cuda_check(cudaStreamSynchronize(s), "stream synchronize");
  cuda_check(cudaMemcpy(b->d_cases + c->batch_index, &c->hd, sizeof(CaseDev), cudaMemcpyHostToDevice),
             "copy case descriptor");
  for (auto& bk : b->buckets) {
    if (std::find(bk.members.begin(), bk.members.end(), c->batch_index) == bk.members.end()) continue;
    std::vector<const StepPlan*> plans;
    for (int m : bk.members) {
      b->cases[m]->plan = build_step_plan(b->cases[m]->hd);
      plans.push_back(&b->cases[m]->plan);
    }
    bk.plan = merge_plans(plans, bk.members, {});
    upload_plan_owned(bk.plan, bk.dp);
  }
  batch_capture_graphs(b);
}

extern "C" {

int rbc_batch_create(const RbcParams* params, int ncases, RbcBatch** out) {
  API_BEGIN
  TraceRange tr("rbc_batch_create");
  require(params != nullptr && out != nullptr && ncases > 0, "rbc_batch_create: invalid argument");
  *out = nullptr;
  for (int i = 0; i < ncases; i++) validate_params(params[i]);
  cuda_check(configure_prim_kernels(), "configure kernels");
  std::unique_ptr<RbcBatch> b(new RbcBatch());
  cuda_check(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream create");
  // groups of equal kind (box / periodic) and precision, any size: one launch
  // per pass covers every case of the group.  Mixed-precision cases whose
  // Chebyshev lengths are all 2^p + 1 (ny, and nx of a box) form groups of
  // their own (+8): there the transforms also have a butterfly form, and the
  // autotuner picks between that and the tensor-core GEMMs per group
  for (int i = 0; i < ncases; i++) {
    const RbcParams& p = params[i];
    const bool bfly = p.precision == RBC_PREC_MIXED && is_pow2(p.ny - 1) &&
                      (p.kind == RBC_PERIODIC || is_pow2(p.nx - 1));
    int kind = (p.kind == RBC_PERIODIC ? 2 : 0) + 4 * p.precision + (bfly ? 8 : 0);
    int found = -1;
    for (size_t k = 0; k < b->buckets.size(); k++)
      if (b->buckets[k].kind == kind) found = (int)k;
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
  // the state of each group's cases is one contiguous range (group by group,
  // cases in index order within a group), so that rbc_batch_step_io moves a
  // group's state with one copy each way
  size_t sz[5];
  b->state_offset.assign(ncases, 0);
  for (auto& bk : b->buckets) {
    bk.state_begin = b->state_bytes;
    for (int i : bk.members) {
      b->state_offset[i] = b->state_bytes;
      b->state_bytes += state_layout(params[i], sz);
    }
    bk.state_end = b->state_bytes;
  }
  b->d_state = static_cast<char*>(b->arena.alloc(b->state_bytes));
  for (int i = 0; i < ncases; i++) {
    std::unique_ptr<RbcCase> c(new RbcCase());
    c->p = params[i];
    c->periodic = params[i].kind == RBC_PERIODIC;
    c->stream = b->stream;
    c->own_stream = false;
    c->in_batch = true;
    c->batch = b.get();
    c->batch_index = i;
    build_case(c.get(), false, b->d_state + b->state_offset[i]);
    b->cases.push_back(c.release());
  }
  // device table of all case descriptors
  std::vector<CaseDev> hd;
  for (RbcCase* c : b->cases) hd.push_back(c->hd);
  b->d_cases = b->arena.upload(hd);
  for (auto& bk : b->buckets) {
    std::vector<const StepPlan*> plans;
    for (int m : bk.members) plans.push_back(&b->cases[m]->plan);
    bk.plan = merge_plans(plans, bk.members, {});
    upload_plan(b->arena, bk.plan, bk.dp);
    // autotune: where a pass has other forms (128-thread CTAs, one thread per
    // sub-lane; a form may take several launches), time every form on this
    // batch and keep the fastest (the state is still zero; the choice is made
    // once, so the batch's numbers do not depend on later timings)
    const size_t nalt = b->cases[bk.members[0]]->plan_alts.size();
    std::vector<StepPlan> alts(nalt);
    std::vector<DevPlan> adps(nalt);
    for (size_t a = 0; a < nalt; a++) {
      std::vector<const StepPlan*> ap;
      for (int m : bk.members) ap.push_back(&b->cases[m]->plan_alts[a]);
      alts[a] = merge_plans(ap, bk.members, {});
      upload_plan(b->arena, alts[a], adps[a]);
    }
    cuda_check(cudaDeviceSynchronize(), "batch set-up");
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "event");
    cuda_check(cudaEventCreate(&e1), "event");
    auto time_launch = [&](const StepLaunch& L, const DevPlan& dp, size_t li) {
      cuda_check(launch_entry(L, dp, li, b->stream, b->d_cases), "autotune launch");  // warm-up
      float best = 1e30f;
      for (int r = 0; r < 3; r++) {
        cuda_check(cudaEventRecord(e0, b->stream), "event");
        cuda_check(launch_entry(L, dp, li, b->stream, b->d_cases), "autotune launch");
        cuda_check(cudaEventRecord(e1, b->stream), "event");
        cuda_check(cudaEventSynchronize(e1), "event");
        float ms = 0.f;
        cuda_check(cudaEventElapsedTime(&ms, e0, e1), "event");
        best = std::min(best, ms);
      }
      return best;
    };
    // launch indices of each pass, in order
    auto passes = [](const StepPlan& P) {
      std::vector<std::vector<size_t>> g;
      for (size_t li = 0; li < P.launches.size(); li++) {
        if (g.empty() || P.launches[g.back()[0]].pass != P.launches[li].pass) g.emplace_back();
        g.back().push_back(li);
      }
      return g;
    };
    // a launch's identity for the comparison of forms: its kernel, and for a
    // GEMM launch the widest tile of its jobs and its form (forms 0, 4 and 5
    // differ there only)
    auto kernels_of = [](const StepPlan& P, const std::vector<size_t>& g) {
      std::vector<int> k;
      for (size_t li : g) {
        const StepLaunch& L = P.launches[li];
        int id = L.kernel;
        if (L.kernel == K_GEMM) {
          int nt = 0;
          for (const GemmJobDev& j : L.jobs) nt = std::max(nt, j.NT);
          id = K_GEMM * 1000 + nt + (L.gemm_ws ? 500 : 0);
        }
        k.push_back(id);
      }
      return k;
    };
    const auto gb = passes(bk.plan);
    std::vector<std::vector<std::vector<size_t>>> ga(nalt);
    for (size_t a = 0; a < nalt; a++) {
      ga[a] = passes(alts[a]);
      if (ga[a].size() != gb.size()) throw std::runtime_error("autotune: plan forms of different pass structure");
    }
    // RBC_BATCH_FORM pins the forms instead (profiling runs: a profiler's
    // per-launch overhead distorts the timings): "<passes>[;<gemms>]".  The
    // first part is one digit 0..3 for every FP64 pass that has forms, or a
    // comma-separated list with one digit per such pass, in the order of those
    // passes in rbc_batch_tuning; the second is the same for the GEMM passes
    // (0: 64-output tiles, 4: 128), all 0 when it is absent
    const char* fenv = std::getenv("RBC_BATCH_FORM");
    std::vector<int> forced_fp64, forced_gemm, forced_transform;
    if (fenv) {
      int part = 0;
      for (const char* q = fenv; *q; q++) {
        if (*q == ';') part++;
        else if (*q >= '0' && *q <= '5')
          (part == 0 ? forced_fp64 : part == 1 ? forced_gemm : forced_transform).push_back(*q - '0');
      }
      if (part < 1) forced_gemm = {0};
      if (part < 2) forced_transform = {0};
    }
    StepPlan tuned;
    for (size_t pi = 0; pi < gb.size(); pi++) {
      auto group_time = [&](const StepPlan& P, const DevPlan& dp, const std::vector<size_t>& g) {
        float t = 0.f;
        for (size_t li : g) t += time_launch(P.launches[li], dp, li);
        return t;
      };
      std::vector<std::vector<int>> seen{kernels_of(bk.plan, gb[pi])};
      float t_base = -1.f, t_best_alt = 1e30f;
      int best = -1, best_alt_kernel = bk.plan.launches[gb[pi][0]].kernel;
      for (size_t a = 0; a < nalt; a++) {
        // the fused periodic Y2 form (variant 3) holds its registers through
        // three phases; beside another group it slowed the whole step (256-case
        // ensemble: 3.34 ms against 3.09 ms) although the pass alone was 5 %
        // faster, and passes are timed alone here: it is timed for batches of
        // one group only (RBC_BATCH_FORM still selects it)
        if (a == 2 && b->buckets.size() > 1) continue;
        const auto ks = kernels_of(alts[a], ga[a][pi]);
        if (std::find(seen.begin(), seen.end(), ks) != seen.end()) continue;
        seen.push_back(ks);
        if (t_base < 0) t_base = group_time(bk.plan, bk.dp, gb[pi]);
        const float t = group_time(alts[a], adps[a], ga[a][pi]);
        if (t < t_best_alt) {
          t_best_alt = t;
          best_alt_kernel = ks[0];
          if (t < t_base) best = (int)a;
        }
      }
      if (t_base >= 0) {
        const bool gemm = bk.plan.launches[gb[pi][0]].kernel == K_GEMM;
        const std::vector<int>& fl = gemm ? forced_gemm : forced_fp64;
        size_t pos = 0;  // this decision's place among the batch's decisions of its kind
        for (const auto& t : b->tuning) pos += t.gemm == gemm;
        int forced = -1;
        if (fl.size() == 1) forced = fl[0];
        else if (pos < fl.size()) forced = fl[pos];
        if (forced == 0) best = -1;
        else if (forced > 0 && (size_t)forced <= nalt) best = forced - 1;
        b->tuning.push_back({bk.plan.launches[gb[pi][0]].kernel, best_alt_kernel, t_base, t_best_alt, best + 1, gemm});
      }
      const StepPlan& src = best >= 0 ? alts[best] : bk.plan;
      for (size_t li : (best >= 0 ? ga[best][pi] : gb[pi])) tuned.launches.push_back(src.launches[li]);
    }
    bk.plan = std::move(tuned);
    bk.dp = DevPlan();
    upload_plan(b->arena, bk.plan, bk.dp);
    // transform-as-GEMM against the butterfly (groups of butterfly sizes, kind
    // +8): the group's plain plan runs every transform as an FFT butterfly in
    // FP64 (so at least as accurate), the products in FP64 too.  The whole step
    // of each plan is timed (its launches alone, as above) and the faster kept;
    // the third part of RBC_BATCH_FORM pins the choice (0 GEMM, 1 butterfly)
    if (bk.kind & 8) {
      std::vector<StepPlan> fp(bk.members.size());
      std::vector<const StepPlan*> fpp;
      bool fits = true;
      for (size_t m = 0; m < bk.members.size(); m++) {
        fp[m] = build_step_plan(b->cases[bk.members[m]]->hd);
        for (const StepLaunch& L : fp[m].launches) fits = fits && L.smem <= smem_limit();
        fpp.push_back(&fp[m]);
      }
      if (fits) {
        StepPlan bp = merge_plans(fpp, bk.members, {});
        DevPlan bdp;
        upload_plan(b->arena, bp, bdp);
        auto whole = [&](const StepPlan& P, const DevPlan& dp) {
          float t = 0.f;
          for (size_t li = 0; li < P.launches.size(); li++) t += time_launch(P.launches[li], dp, li);
          return t;
        };
        const float t_gemm = whole(bk.plan, bk.dp), t_bfly = whole(bp, bdp);
        const size_t pos = b->transforms.size();
        int forced = -1;
        if (forced_transform.size() == 1) forced = forced_transform[0];
        else if (pos < forced_transform.size()) forced = forced_transform[pos];
        const bool use_bfly = forced >= 0 ? forced == 1 : t_bfly < t_gemm;
        b->transforms.push_back({(int)(&bk - b->buckets.data()), t_gemm, t_bfly, use_bfly});
        if (use_bfly) {
          bk.plan = std::move(bp);
          bk.dp = bdp;
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  // the timing runs wrote into the state and scratch: the batch starts from zero
  cuda_check(cudaMemsetAsync(b->d_state, 0, b->state_bytes, b->stream), "clear state");
  for (RbcCase* c : b->cases) cuda_check(cudaMemsetAsync(c->hd.status, 0, 16, b->stream), "clear status");
  cuda_check(cudaDeviceSynchronize(), "batch set-up");
  // graph: one branch per bucket.  The branches run side by side; the one
  // with the longest step (timed here, launches in sequence) is the critical
  // path and is captured on a high-priority stream, so its thread blocks are
  // dispatched first and the other branches fill the SMs it leaves idle
  // (kernel nodes take the capturing stream's priority)
  size_t nb = b->buckets.size();
  std::vector<float> bucket_ms(nb, 0.f);
  {
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "event");
    cuda_check(cudaEventCreate(&e1), "event");
    for (size_t k = 0; k < nb; k++) {
      const auto& bk = b->buckets[k];
      float best = 1e30f;
      for (int r = 0; r < 2; r++) {
        cuda_check(cudaEventRecord(e0, b->stream), "event");
        for (size_t li = 0; li < bk.plan.launches.size(); li++)
          cuda_check(launch_entry(bk.plan.launches[li], bk.dp, li, b->stream, b->d_cases), "bucket timing launch");
        cuda_check(cudaEventRecord(e1, b->stream), "event");
        cuda_check(cudaEventSynchronize(e1), "event");
        float ms = 0.f;
        cuda_check(cudaEventElapsedTime(&ms, e0, e1), "event");
        best = std::min(best, ms);
      }
      bucket_ms[k] = best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cuda_check(cudaMemsetAsync(b->d_state, 0, b->state_bytes, b->stream), "clear state");
    for (RbcCase* c : b->cases) cuda_check(cudaMemsetAsync(c->hd.status, 0, 16, b->stream), "clear status");
    cuda_check(cudaStreamSynchronize(b->stream), "batch set-up");
  }
  const size_t critical = (size_t)(std::max_element(bucket_ms.begin(), bucket_ms.end()) - bucket_ms.begin());
  bool use_priority = nb > 1;
  if (const char* f = std::getenv("RBC_BATCH_PRIORITY"))
    if (f[0] == '0' && f[1] == '\0') use_priority = false;
  int prio_low = 0, prio_high = 0;
  cuda_check(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high), "stream priority range");
  b->branch.resize(nb);
  b->events.resize(nb + 1);
  for (size_t k = 0; k < nb; k++) {
    const int prio = !use_priority ? 0 : (k == critical ? prio_high : prio_low);
    cuda_check(cudaStreamCreateWithPriority(&b->branch[k], cudaStreamNonBlocking, prio), "stream");
  }
  for (auto& e : b->events) cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
  b->use_priority = use_priority;
  batch_capture_graphs(b.get());
  b->io_order.resize(nb);
  for (size_t k = 0; k < nb; k++) b->io_order[k] = k;
  std::stable_sort(b->io_order.begin(), b->io_order.end(),
                   [&](size_t x, size_t y) { return bucket_ms[x] < bucket_ms[y]; });
  b->io_events.resize(nb);
  for (auto& e : b->io_events) cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
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
  TraceRange tr("rbc_batch_step");
  require(b && nsteps >= 0, "rbc_batch_step: invalid argument");
  for (int s = 0; s < nsteps; s++) {
    cuda_check(cudaGraphLaunch(b->gexec, b->stream), "graph launch");
    for (RbcCase* c : b->cases) c->time += c->p.dt;
  }
  API_END
}
int rbc_batch_step_io(RbcBatch* b, const void* host_in, void* host_out, size_t bytes, int nsteps) {
  API_BEGIN
  TraceRange tr("rbc_batch_step_io");
  require(b && host_in && host_out && nsteps >= 0, "rbc_batch_step_io: invalid argument");
  require(bytes == b->state_bytes, "rbc_batch_step_io: size mismatch (see rbc_batch_state_bytes)");
  const size_t nb = b->buckets.size();
  // after the work already queued on the batch stream; each group: its input
  // range in (after the previous group's: shortest step first), its steps,
  // its output range back, on its own branch, so that one group's copies
  // overlap the other groups' steps
  cuda_check(cudaEventRecord(b->events[nb], b->stream), "event");
  cudaEvent_t prev = nullptr;
  for (size_t k : b->io_order) {
    const auto& bk = b->buckets[k];
    cudaStream_t s = b->branch[k];
    const size_t o = bk.state_begin, n = bk.state_end - bk.state_begin;
    cuda_check(cudaStreamWaitEvent(s, b->events[nb], 0), "stream wait");
    if (prev != nullptr) cuda_check(cudaStreamWaitEvent(s, prev, 0), "stream wait");
    TraceRange tg("group: copy in, steps, copy out");
    cuda_check(cudaMemcpyAsync(b->d_state + o, static_cast<const char*>(host_in) + o, n, cudaMemcpyHostToDevice, s),
               "state copy h2d");
    cuda_check(cudaEventRecord(b->io_events[k], s), "event");
    prev = b->io_events[k];
    for (int t = 0; t < nsteps; t++) cuda_check(cudaGraphLaunch(bk.gexec, s), "graph launch");
    cuda_check(cudaMemcpyAsync(static_cast<char*>(host_out) + o, b->d_state + o, n, cudaMemcpyDeviceToHost, s),
               "state copy d2h");
    cuda_check(cudaEventRecord(b->events[k], s), "event");
    cuda_check(cudaStreamWaitEvent(b->stream, b->events[k], 0), "stream wait");
  }
  for (int t = 0; t < nsteps; t++)
    for (RbcCase* c : b->cases) c->time += c->p.dt;
  cuda_check(cudaStreamSynchronize(b->stream), "stream synchronize");
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
int rbc_batch_tuning(const RbcBatch* b, int k, int* kernel_cta, int* kernel_lanes, double* ms_cta, double* ms_lanes,
                     int* n) {
  API_BEGIN
  require(b && n, "null argument");
  *n = (int)b->tuning.size();
  if (k >= 0 && k < *n) {
    const auto& t = b->tuning[k];
    if (kernel_cta) *kernel_cta = t.kernel_cta;
    if (kernel_lanes) *kernel_lanes = t.kernel_lanes;
    if (ms_cta) *ms_cta = t.ms_cta;
    if (ms_lanes) *ms_lanes = t.ms_lanes;
  }
  API_END
}

int rbc_batch_tuning_forms(const RbcBatch* b, char* buf, size_t len) {
  API_BEGIN
  require(b && buf && len > 0, "rbc_batch_tuning_forms: invalid argument");
  std::string s, g;
  for (const auto& t : b->tuning) {
    std::string& d = t.gemm ? g : s;
    if (!d.empty()) d += ',';
    d += (char)('0' + t.form);
  }
  std::string t;
  for (const auto& x : b->transforms) {
    if (!t.empty()) t += ',';
    t += x.butterfly ? '1' : '0';
  }
  if (!g.empty() || !t.empty()) s += ";" + g;
  if (!t.empty()) s += ";" + t;
  require(s.size() < len, "rbc_batch_tuning_forms: buffer too small");
  std::memcpy(buf, s.c_str(), s.size() + 1);
  API_END
}

int rbc_batch_state_bytes(const RbcBatch* b, size_t* bytes) {
  API_BEGIN
  require(b && bytes, "null argument");
  *bytes = b->state_bytes;
  API_END
}
int rbc_batch_get_state_all(RbcBatch* b, void* host, size_t bytes) {
  API_BEGIN
  require(b && host, "null argument");
  require(bytes == b->state_bytes, "rbc_batch_get_state_all: size mismatch (see rbc_batch_state_bytes)");
  cuda_check(cudaMemcpyAsync(host, b->d_state, bytes, cudaMemcpyDeviceToHost, b->stream), "state copy d2h");
  cuda_check(cudaStreamSynchronize(b->stream), "stream synchronize");
  API_END
}
int rbc_batch_set_state_all(RbcBatch* b, const void* host, size_t bytes) {
  API_BEGIN
  require(b && host, "null argument");
  require(bytes == b->state_bytes, "rbc_batch_set_state_all: size mismatch (see rbc_batch_state_bytes)");
  cuda_check(cudaMemcpyAsync(b->d_state, host, bytes, cudaMemcpyHostToDevice, b->stream), "state copy h2d");
  cuda_check(cudaStreamSynchronize(b->stream), "stream synchronize");
  API_END
}
int rbc_batch_state_offset(const RbcBatch* b, int i, size_t* offset) {
  API_BEGIN
  require(b && offset && i >= 0 && i < (int)b->cases.size(), "rbc_batch_state_offset: invalid argument");
  *offset = b->state_offset[i];
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
      TraceRange ts(step_kernel_name(c->plan.launches[k].kernel));
      cuda_check(launch_entry(c->plan.launches[k], c->dp, k, c->stream, c->d_case),
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

int rbc_stage_bytes(const RbcCase* c, int k, double* bytes) {
  API_BEGIN
  require(c && bytes && k >= 0 && k < (int)c->plan.launches.size(), "rbc_stage_bytes: invalid argument");
  *bytes = launch_algorithmic_bytes(c->plan.launches[k], &c->hd);
  API_END
}

int rbc_batch_profile_step(RbcBatch* b, int nsteps, double* stage_ms, double* stage_bytes, int* stage_kernel,
                           int max_stages, int* nstages) {
  API_BEGIN
  require(b && stage_ms && nstages && nsteps > 0, "rbc_batch_profile_step: invalid argument");
  // stages = distinct kernels of the batch step, in order of first appearance;
  // each launch of every bucket runs alone between two events
  std::vector<int> kid;
  std::vector<double> ms_acc, bytes;
  std::vector<CaseDev> hd;
  for (RbcCase* c : b->cases) hd.push_back(c->hd);
  auto slot = [&](int kernel) {
    for (size_t i = 0; i < kid.size(); i++)
      if (kid[i] == kernel) return (int)i;
    kid.push_back(kernel);
    ms_acc.push_back(0.0);
    bytes.push_back(0.0);
    return (int)kid.size() - 1;
  };
  for (auto& bk : b->buckets)
    for (auto& L : bk.plan.launches) bytes[slot(L.kernel)] += launch_algorithmic_bytes(L, hd.data());
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "event create");
  cuda_check(cudaEventCreate(&e1), "event create");
  for (int s = 0; s < nsteps; s++) {
    for (auto& bk : b->buckets)
      for (size_t li = 0; li < bk.plan.launches.size(); li++) {
        TraceRange ts(step_kernel_name(bk.plan.launches[li].kernel));
        cuda_check(cudaEventRecord(e0, b->stream), "event record");
        cuda_check(launch_entry(bk.plan.launches[li], bk.dp, li, b->stream, b->d_cases), "stage launch");
        cuda_check(cudaEventRecord(e1, b->stream), "event record");
        cuda_check(cudaEventSynchronize(e1), "event sync");
        float ms = 0.f;
        cuda_check(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
        ms_acc[slot(bk.plan.launches[li].kernel)] += ms;
      }
    for (RbcCase* c : b->cases) c->time += c->p.dt;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *nstages = (int)kid.size();
  for (int k = 0; k < (int)kid.size() && k < max_stages; k++) {
    stage_ms[k] = ms_acc[k] / nsteps;
    if (stage_bytes) stage_bytes[k] = bytes[k];
    if (stage_kernel) stage_kernel[k] = kid[k];
  }
  API_END
}

// every launch of the batch step timed alone, in step order (bucket by
// bucket): kernel id, bucket, pass id, mean ms and algorithmic bytes
int rbc_batch_profile_launches(RbcBatch* b, int nsteps, int* kernel, int* bucket, int* pass, double* ms_out,
                               double* bytes_out, int max_launches, int* nlaunches) {
  API_BEGIN
  require(b && kernel && bucket && pass && ms_out && nlaunches && nsteps > 0, "rbc_batch_profile_launches: invalid argument");
  std::vector<CaseDev> hd;
  for (RbcCase* c : b->cases) hd.push_back(c->hd);
  std::vector<double> acc;
  int n = 0;
  for (size_t k = 0; k < b->buckets.size(); k++)
    for (auto& L : b->buckets[k].plan.launches) {
      if (n < max_launches) {
        kernel[n] = L.kernel;
        bucket[n] = (int)k;
        pass[n] = L.pass;
        if (bytes_out) bytes_out[n] = launch_algorithmic_bytes(L, hd.data());
      }
      n++;
    }
  acc.assign(n, 0.0);
  cudaEvent_t e0, e1;
  cuda_check(cudaEventCreate(&e0), "event create");
  cuda_check(cudaEventCreate(&e1), "event create");
  for (int s = 0; s < nsteps; s++) {
    int idx = 0;
    for (auto& bk : b->buckets)
      for (size_t li = 0; li < bk.plan.launches.size(); li++, idx++) {
        TraceRange ts(step_kernel_name(bk.plan.launches[li].kernel));
        cuda_check(cudaEventRecord(e0, b->stream), "event record");
        cuda_check(launch_entry(bk.plan.launches[li], bk.dp, li, b->stream, b->d_cases), "stage launch");
        cuda_check(cudaEventRecord(e1, b->stream), "event record");
        cuda_check(cudaEventSynchronize(e1), "event sync");
        float ms = 0.f;
        cuda_check(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
        acc[idx] += ms;
      }
    for (RbcCase* c : b->cases) c->time += c->p.dt;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (int k = 0; k < n && k < max_launches; k++) ms_out[k] = acc[k] / nsteps;
  *nlaunches = n;
  API_END
}

const char* rbc_kernel_name(int kernel) { return step_kernel_name(kernel); }

const char* rbc_stage_name(const RbcCase* c, int k) {
  if (!c || k < 0 || k >= (int)c->plan.launches.size()) return "";
  return step_kernel_name(c->plan.launches[k].kernel);
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
int rbc_set_device(int ordinal) {
  API_BEGIN
  int n = 0;
  cuda_check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
  require(ordinal >= 0 && ordinal < n, "rbc_set_device: ordinal out of range (" + std::to_string(n) + " devices)");
  cuda_check(cudaSetDevice(ordinal), "cudaSetDevice");
  API_END
}
int rbc_get_device(int* ordinal) {
  API_BEGIN
  require(ordinal != nullptr, "null argument");
  cuda_check(cudaGetDevice(ordinal), "cudaGetDevice");
  API_END
}

// ---- funspace primitives
int fs_space_create(int base0, int n0, int base1, int n1, FsSpace** out) {
  API_BEGIN
  require(out != nullptr, "null argument");
  *out = nullptr;
  require(base0 >= 0 && base0 <= 5 && base1 >= 0 && base1 <= 4, "fs_space_create: unknown base (Fourier along axis 0 only)");
  require(n0 >= 4 && n1 >= 4 && n0 <= 8192 && n1 <= 8192, "fs_space_create: sizes must be in [4, 8192]");
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
  if (e != cudaSuccess || p == nullptr) {
    // clear the runtime's last error: the launch check of the next call would
    // otherwise report this failure as its own
    (void)cudaGetLastError();
    throw ApiError(RBC_ERR_CUDA, std::string("fs_forward_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  }
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

// ---- batched 1-D lanes
static const float* upload_split(Arena& a, const LMat& M) {
  std::vector<float> pk = pack_gemm_w(lm_to_double(M), M.rows, M.cols, gemm_tile_n(M.rows));
  return a.upload(pk);
}

int fs_lanes_create(int base, int n, int precision, FsLanes** out) {
  API_BEGIN
  require(out != nullptr, "null argument");
  *out = nullptr;
  require(base == FS_CHEBYSHEV || base == FS_CHEB_DIRICHLET || base == FS_CHEB_NEUMANN,
          "fs_lanes_create: Chebyshev-family bases only");
  require(n >= 8 && n <= 2048, "fs_lanes_create: n must be in [8, 2048]");
  require(precision == RBC_PREC_FP64 || precision == RBC_PREC_MIXED, "fs_lanes_create: unknown precision");
  cuda_check(configure_prim_kernels(), "configure kernels");
  cuda_check(configure_gemm_kernels(), "configure gemm kernels");
  std::unique_ptr<FsLanes> p(new FsLanes());
  p->precision = precision;
  build_lanes(p->arena, p->L, base, n);
  p->d_status = static_cast<unsigned int*>(p->arena.alloc(16));
  if (precision == RBC_PREC_MIXED) {
    const HostBasis& hb = p->L.hb;
    LMat S = lm_stencil(hb), P = lm_from_ortho(hb);
    p->w[FS_OP_FORWARD] = upload_split(p->arena, lm_mul(P, lm_cheb_forward(n)));
    p->w[FS_OP_BACKWARD] = upload_split(p->arena, lm_mul(lm_cheb_backward(n), S));
    p->w[FS_OP_TO_ORTHO] = upload_split(p->arena, S);
    p->w[FS_OP_FROM_ORTHO] = upload_split(p->arena, P);
    if (hb.composite()) p->w[FS_OP_HHOLTZ] = upload_split(p->arena, lm_pinv(n));
  }
  *out = p.release();
  API_END
}
int fs_lanes_destroy(FsLanes* p) {
  API_BEGIN
  delete p;
  API_END
}
int fs_lanes_shape(const FsLanes* p, int* n, int* m) {
  API_BEGIN
  require(p && n && m, "null argument");
  *n = p->L.hb.n;
  *m = p->L.hb.m;
  API_END
}
int fs_lanes_set_hholtz(FsLanes* p, double c) {
  API_BEGIN
  require(p != nullptr, "null argument");
  require(std::isfinite(c), "fs_lanes_set_hholtz: coefficient must be finite");
  lanes_set_hholtz(p->arena, p->L, c);
  API_END
}
int fs_lanes_status(FsLanes* p, void* stream, unsigned int* status) {
  API_BEGIN
  require(p && status, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  unsigned int v = 0;
  cuda_check(cudaMemcpyAsync(&v, p->d_status, 4, cudaMemcpyDeviceToHost, st), "d2h");
  cuda_check(cudaMemsetAsync(p->d_status, 0, 4, st), "clear status");
  cuda_check(cudaStreamSynchronize(st), "synchronize");
  *status = v;
  API_END
}
int rbc_set_gemm_wait_limit(long long polls) {
  API_BEGIN
  cuda_check(set_gemm_wait_limit(polls), "set the lane GEMM wait limit");
  API_END
}
int fs_lanes_apply(FsLanes* p, int op, const double* d_in, double* d_out, int lanes, void* stream) {
  API_BEGIN
  require(p && d_in && d_out, "null argument");
  require(op >= FS_OP_FORWARD && op <= FS_OP_HHOLTZ, "fs_lanes_apply: unknown operation");
  require(lanes >= 0, "fs_lanes_apply: negative lane count");
  if (lanes == 0) return RBC_OK;
  if (op == FS_OP_HHOLTZ) require(p->L.has_solver, "fs_lanes_apply: call fs_lanes_set_hholtz first");
  cudaStream_t st = (cudaStream_t)stream;
  if (p->precision == RBC_PREC_FP64) {
    lanes_apply(p->L, op, d_in, d_out, lanes, st);
  } else {
    int il, ol;
    lane_op_lengths(p->L, op, &il, &ol);
    void* ip[1] = {const_cast<double*>(d_in)};
    void* opp[1] = {d_out};
    GemmJobDev j = make_gemm_job(lane_rows(ip, 1, lanes, il, il, LT_F64, false),
                                 lane_rows(opp, 1, lanes, ol, ol, LT_F64, false), p->w[op], il, ol, 1.0, p->d_status);
    cuda_check(launch_lane_gemm_one(j, st), "lane gemm launch");
    if (op == FS_OP_HHOLTZ) lanes_fdma(p->L, d_out, lanes, st);
  }
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

// ---- Diffusion2D (src/navier/diffusion.rs:113-238) -------------------------
}  // extern "C"

struct DfCase {
  Arena arena;
  SpaceDev s;
  SpaceDev sbc;  // space of the boundary field (add_fieldbc)
  SolverDev sv;
  double kappa = 0.0, dt = 0.0, time = 0.0;
  void* vhat = nullptr;   // composite state (spec0 x spec1)
  void* k = nullptr;      // F pinv_x pinv_y C (spec0 x spec1)
  void* c_ortho = nullptr;
  void* bc_vhat = nullptr;
  double* bc_v = nullptr;  // physical boundary field
  double* phys = nullptr;
  void* tmp = nullptr;
  void* tmp2 = nullptr;
  std::vector<double> force;  // dt-free force (ortho0 x ortho1, real spaces)
  bool has_bc = false;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  ~DfCase() {
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    if (stream) {
      cudaStreamSynchronize(stream);
      cudaStreamDestroy(stream);
    }
  }
  size_t es() const { return s.cplx ? 16 : 8; }
  size_t spec_doubles() const { return (size_t)s.spec0 * s.spec1 * (s.cplx ? 2 : 1); }
  size_t ortho_doubles() const { return (size_t)s.ortho0 * s.ortho1 * (s.cplx ? 2 : 1); }
  void sync() { cuda_check(cudaStreamSynchronize(stream), "stream synchronize"); }
};

namespace {
// C = dt force + (dt kappa) d2/dx2 fieldbc + (dt kappa) d2/dy2 fieldbc in ortho
// space (diffusion.rs:192-201), then K = F pinv_x pinv_y C on the device.
void df_refresh_constant(DfCase* d) {
  const size_t n = d->ortho_doubles();
  std::vector<double> c(n, 0.0);
  if (!d->force.empty())
    for (size_t i = 0; i < n; i++) c[i] = d->dt * d->force[i];
  if (d->has_bc) {
    std::vector<double> gxx(n), gyy(n);
    space_gradient(d->sbc, d->bc_vhat, d->c_ortho, 2, 0, nullptr, d->tmp, d->stream);
    cuda_check(cudaMemcpyAsync(gxx.data(), d->c_ortho, n * 8, cudaMemcpyDeviceToHost, d->stream), "d2h");
    d->sync();
    space_gradient(d->sbc, d->bc_vhat, d->c_ortho, 0, 2, nullptr, d->tmp, d->stream);
    cuda_check(cudaMemcpyAsync(gyy.data(), d->c_ortho, n * 8, cudaMemcpyDeviceToHost, d->stream), "d2h");
    d->sync();
    const double dk = d->dt * d->kappa;
    for (size_t i = 0; i < n; i++) c[i] = (c[i] + dk * gxx[i]) + dk * gyy[i];
  }
  cuda_check(cudaMemcpyAsync(d->c_ortho, c.data(), n * 8, cudaMemcpyHostToDevice, d->stream), "h2d");
  diffusion_constant(d->sv, d->s, d->c_ortho, d->k, d->tmp, d->stream);
  d->sync();
}
}  // namespace

extern "C" {

int df_create(int base0, int n0, int base1, int n1, double kappa, double dt, DfCase** out) {
  API_BEGIN
  require(out != nullptr, "df_create: null argument");
  *out = nullptr;
  require(base0 >= 0 && base0 <= 5 && base1 >= 0 && base1 <= 4, "df_create: unknown base (Fourier along axis 0 only)");
  require(n0 >= 6 && n1 >= 6 && n0 <= 8192 && n1 <= 8192, "df_create: sizes must be in [6, 8192]");
  require(kappa > 0 && dt > 0, "df_create: kappa and dt must be positive");
  cuda_check(configure_prim_kernels(), "configure kernels");
  std::unique_ptr<DfCase> d(new DfCase());
  d->kappa = kappa;
  d->dt = dt;
  build_space(d->arena, d->s, base0, n0, base1, n1);
  // Hholtz::new(&field, [dt * kappa, dt * kappa]) (diffusion.rs:142)
  const double c[2] = {dt * kappa, dt * kappa};
  std::string err;
  if (!build_solver(d->arena, d->s, SV_KIND_HHOLTZ, c, d->sv, &err))
    throw ApiError(RBC_ERR_UNSUPPORTED, "df_create: " + err);
  const size_t es = d->es();
  d->vhat = d->arena.alloc((size_t)d->s.spec0 * d->s.spec1 * es);
  d->k = d->arena.alloc((size_t)d->s.spec0 * d->s.spec1 * es);
  d->c_ortho = d->arena.alloc((size_t)d->s.ortho0 * d->s.ortho1 * es);
  d->tmp = d->arena.alloc(tmp_elems(d->s) * 16);
  d->tmp2 = d->arena.alloc(tmp_elems(d->s) * 16);
  d->phys = static_cast<double*>(d->arena.alloc((size_t)n0 * n1 * 8));
  cuda_check(cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking), "stream create");
  cuda_check(cudaStreamSynchronize(cudaStreamLegacy), "allocation");
  // one update as a CUDA graph (the constant K stays at its address)
  cuda_check(cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  try {
    diffusion_step(d->sv, d->s, d->vhat, d->k, d->tmp2, d->stream);
  } catch (...) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(d->stream, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  cuda_check(cudaStreamEndCapture(d->stream, &d->graph), "end capture");
  cuda_check(cudaGraphInstantiate(&d->gexec, d->graph, 0), "graph instantiate");
  *out = d.release();
  API_END
}

int df_destroy(DfCase* d) {
  API_BEGIN
  delete d;
  API_END
}

int df_shape(const DfCase* d, int which, int* n0, int* n1, int* is_complex) {
  API_BEGIN
  require(d && n0 && n1 && is_complex, "df_shape: null argument");
  switch (which) {
    case FS_PHYSICAL: *n0 = d->s.phys0; *n1 = d->s.phys1; *is_complex = 0; break;
    case FS_SPECTRAL: *n0 = d->s.spec0; *n1 = d->s.spec1; *is_complex = d->s.cplx; break;
    case FS_ORTHO: *n0 = d->s.ortho0; *n1 = d->s.ortho1; *is_complex = d->s.cplx; break;
    default: throw ApiError(RBC_ERR_INVALID, "df_shape: unknown array kind");
  }
  API_END
}

int df_get_state(DfCase* d, double* host, size_t n_doubles) {
  API_BEGIN
  require(d && host && n_doubles == d->spec_doubles(), "df_get_state: invalid argument");
  cuda_check(cudaMemcpyAsync(host, d->vhat, n_doubles * 8, cudaMemcpyDeviceToHost, d->stream), "d2h");
  d->sync();
  API_END
}

int df_set_state(DfCase* d, const double* host, size_t n_doubles) {
  API_BEGIN
  require(d && host && n_doubles == d->spec_doubles(), "df_set_state: invalid argument");
  cuda_check(cudaMemcpyAsync(d->vhat, host, n_doubles * 8, cudaMemcpyHostToDevice, d->stream), "h2d");
  d->sync();
  API_END
}

// diffusion.rs:156-163: v = 0 except v[n/2, m/2] = 1, then forward
int df_impulse(DfCase* d) {
  API_BEGIN
  require(d != nullptr, "df_impulse: null argument");
  const int n0 = d->s.phys0, n1 = d->s.phys1;
  std::vector<double> v((size_t)n0 * n1, 0.0);
  v[(size_t)(n0 / 2) * n1 + n1 / 2] = 1.0;
  cuda_check(cudaMemcpyAsync(d->phys, v.data(), v.size() * 8, cudaMemcpyHostToDevice, d->stream), "h2d");
  space_forward(d->s, d->phys, d->vhat, d->tmp, d->stream);
  d->sync();
  API_END
}

// diffusion.rs:168-171: the force has the shape of field.v and is added to the
// ortho-space right-hand side, so real (Chebyshev x Chebyshev) spaces only
int df_add_force(DfCase* d, const double* force, size_t n_doubles) {
  API_BEGIN
  require(d && force, "df_add_force: null argument");
  require(!d->s.cplx && d->s.ortho0 == d->s.phys0 && d->s.ortho1 == d->s.phys1,
          "df_add_force: shape mismatch (the force has the physical shape, the right-hand side the ortho shape)");
  require(n_doubles == (size_t)d->s.phys0 * d->s.phys1, "df_add_force: the force holds n0*n1 doubles");
  d->force.assign(force, force + n_doubles);
  df_refresh_constant(d);
  API_END
}

// diffusion.rs:176-179: boundary field on the space (base0, base1) of the same
// sizes; its Laplacian enters the right-hand side (diffusion.rs:197-201)
int df_add_fieldbc(DfCase* d, int base0, int base1, const double* vhat, size_t n_doubles) {
  API_BEGIN
  require(d && vhat, "df_add_fieldbc: null argument");
  require(base0 >= 0 && base0 <= 5 && base1 >= 0 && base1 <= 4, "df_add_fieldbc: unknown base");
  require((base0 == FS_FOURIER_R2C) == (d->s.cplx != 0), "df_add_fieldbc: the boundary field's space type differs");
  SpaceDev sb;
  build_space(d->arena, sb, base0, d->s.phys0, base1, d->s.phys1);
  require(sb.ortho0 == d->s.ortho0 && sb.ortho1 == d->s.ortho1, "df_add_fieldbc: shape mismatch");
  require(n_doubles == (size_t)sb.spec0 * sb.spec1 * (sb.cplx ? 2 : 1), "df_add_fieldbc: vhat size mismatch");
  d->sbc = sb;
  d->bc_vhat = d->arena.alloc(n_doubles * 8);
  d->bc_v = static_cast<double*>(d->arena.alloc((size_t)d->s.phys0 * d->s.phys1 * 8));
  cuda_check(cudaStreamSynchronize(cudaStreamLegacy), "allocation");
  cuda_check(cudaMemcpyAsync(d->bc_vhat, vhat, n_doubles * 8, cudaMemcpyHostToDevice, d->stream), "h2d");
  space_backward(d->sbc, d->bc_vhat, d->bc_v, d->tmp, d->stream);
  d->has_bc = true;
  df_refresh_constant(d);
  API_END
}

int df_step(DfCase* d, int nsteps) {
  API_BEGIN
  require(d != nullptr && nsteps >= 0, "df_step: invalid argument");
  for (int i = 0; i < nsteps; i++) {
    cuda_check(cudaGraphLaunch(d->gexec, d->stream), "graph launch");
    d->time += d->dt;
  }
  API_END
}

int df_synchronize(DfCase* d) {
  API_BEGIN
  require(d != nullptr, "df_synchronize: null argument");
  d->sync();
  API_END
}

int df_get_time(const DfCase* d, double* t) {
  API_BEGIN
  require(d && t, "df_get_time: null argument");
  *t = d->time;
  API_END
}

int df_get_dt(const DfCase* d, double* dt) {
  API_BEGIN
  require(d && dt, "df_get_dt: null argument");
  *dt = d->dt;
  API_END
}

// field.backward() (diffusion.rs:217), plus fieldbc.v when with_bc (diffusion.rs:219-221)
int df_get_physical(DfCase* d, int with_bc, double* host, size_t n_doubles) {
  API_BEGIN
  require(d && host && n_doubles == (size_t)d->s.phys0 * d->s.phys1, "df_get_physical: invalid argument");
  space_backward(d->s, d->vhat, d->phys, d->tmp, d->stream);
  cuda_check(cudaMemcpyAsync(host, d->phys, n_doubles * 8, cudaMemcpyDeviceToHost, d->stream), "d2h");
  d->sync();
  if (with_bc && d->has_bc) {
    std::vector<double> bc(n_doubles);
    cuda_check(cudaMemcpy(bc.data(), d->bc_v, n_doubles * 8, cudaMemcpyDeviceToHost), "d2h");
    for (size_t i = 0; i < n_doubles; i++) host[i] = host[i] + bc[i];
  }
  API_END
}

int df_get_stream(DfCase* d, void** stream) {
  API_BEGIN
  require(d && stream, "df_get_stream: null argument");
  *stream = d->stream;
  API_END
}

}  // extern "C"

// ============================================================================
// Serving loop (rbc_server_*): continuous batching of RBC solve requests.
//
// A scheduler thread owns the GPU work.  Each round it (1) admits pending
// requests whose case fits the HBM budget (host set-up on a separate stream,
// so it overlaps the steps in flight), (2) when the set of active cases has
// changed, rebuilds the batched step -- groups of equal kind and precision,
// a gate kernel per group, the group's launches, all captured into one CUDA
// graph -- and (3) launches `chunk_steps` graph steps.  The gate
// kernel counts each case's remaining steps down on the device and idles the
// case once it has reached its horizon, so cases of different horizons share
// a chunk and every case stops exactly at its own step count.  Finished cases
// are evaluated (Nu, KE), their memory returned to the pool and their results
// queued for rbc_server_poll.  A case computes the same numbers alone or in
// any mix: no kernel or tile combines data of two cases.
// ============================================================================
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_set>

struct RbcServer {
  RbcServerConfig cfg{};
  int device = 0;
  cudaStream_t stream = nullptr;  // steps
  std::vector<cudaStream_t> branch;  // low-priority graph branches (one per group)
  cudaStream_t branch_hi = nullptr;  // the branch of the group with the most work
  std::vector<cudaEvent_t> bev;
  cudaEvent_t fork = nullptr, chunk_done = nullptr;
  std::thread th;
  std::vector<std::thread> workers;
  std::mutex mu;
  std::condition_variable cv;
  bool stop = false;
  bool failed = false;
  std::string error;
  struct Req {
    long long id;
    RbcParams p;
    double horizon;
    uint64_t seed;
    double t_submit;
    long steps;
  };
  struct Slot {
    Req r;
    RbcCase* c;
    long left;
    double t_admit;
    size_t bytes;
    bool cancelled;
  };
  std::deque<Req> pending;      // submitted, not yet taken by a set-up worker
  std::deque<Slot> ready;       // built, initial fields set, waiting for a slot
  std::vector<Slot> active;     // advancing
  std::deque<RbcRequestResult> done;
  // ids being built by a set-up worker, and ids cancelled while building,
  // ready or active (the thread that holds the case retires it)
  std::unordered_set<long long> building_ids, cancelled;
  int building = 0;
  long long next_id = 0;
  size_t bytes_in_use = 0;      // building (reserved), ready and active cases
  size_t peak_bytes = 0;        // largest bytes_in_use so far
  double gp_steps = 0;
  long long steps_launched = 0, rebuilds = 0, completed = 0;
  std::chrono::steady_clock::time_point t0;
  // batched step of the current active set
  std::unique_ptr<Arena> plan_arena;
  struct Bucket {
    std::vector<int> members;
    StepPlan plan;
    DevPlan dp;
    int* d_members = nullptr;
  };
  std::vector<Bucket> buckets;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  bool dirty = true;
  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

// Upper bound of a case's device bytes (reserved against the budget while the
// case is built; the actual arena size replaces it afterwards).
static size_t case_bytes_bound(const RbcParams& p) {
  const size_t n = (size_t)(p.nx + 2) * (size_t)(p.ny + 2);
  size_t b = n * 8 * 160;                       // fields, scratch and tables
  if (p.kind != RBC_PERIODIC) b += (size_t)p.nx * p.nx * 8 * 16;  // eigenbases and dense x operators
  if (p.precision == RBC_PREC_MIXED) b += ((size_t)p.nx * p.nx + (size_t)p.ny * p.ny) * 4 * 24;
  return b + (4u << 20);
}

static void server_free_graph(RbcServer* S) {
  if (S->gexec) cudaGraphExecDestroy(S->gexec);
  if (S->graph) cudaGraphDestroy(S->graph);
  S->gexec = nullptr;
  S->graph = nullptr;
}

// Set-up worker: builds the case of the next pending request on its own
// stream (host arithmetic, allocations from the stream-ordered pool, boundary
// field, initial fields) while the scheduler keeps stepping.
static void server_worker(RbcServer* S) {
  cudaStream_t st = nullptr;
  try {
    cuda_check(cudaSetDevice(S->device), "set device");
    cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
    for (;;) {
      RbcServer::Req r;
      size_t reserve = 0;
      {
        std::unique_lock<std::mutex> lk(S->mu);
        for (;;) {
          if (S->stop || S->failed) {
            cudaStreamDestroy(st);
            return;
          }
          if (!S->pending.empty()) {
            reserve = case_bytes_bound(S->pending.front().p);
            const bool alone = S->bytes_in_use == 0;
            if (alone || S->bytes_in_use + reserve <= S->cfg.hbm_budget_bytes) break;
          }
          S->cv.wait_for(lk, std::chrono::milliseconds(2));
        }
        r = S->pending.front();
        S->pending.pop_front();
        S->bytes_in_use += reserve;
        S->peak_bytes = std::max(S->peak_bytes, S->bytes_in_use);
        S->building++;
        S->building_ids.insert(r.id);
      }
      std::unique_ptr<RbcCase> c(new RbcCase());
      c->p = r.p;
      c->periodic = r.p.kind == RBC_PERIODIC;
      c->stream = st;
      c->own_stream = false;
      c->in_batch = true;  // stepped by the server only
      c->arena.set_stream_ordered(true);
      bool fits = true;
      try {
        build_case(c.get(), false);
        fits = c->arena.bytes() <= S->cfg.hbm_budget_bytes;
        if (fits) {
          // initial fields: set_velocity(0.2, 1, 1) and seeded temperature noise 1e-3
          apply_mode(c.get(), RBC_UX, 0.2, 1.0, 1.0, true);
          apply_mode(c.get(), RBC_UY, -0.2, 1.0, 1.0, false);
          set_temperature_noise(c.get(), 1e-3, r.seed);
          const int g[2] = {(int)r.steps, 0};
          cuda_check(cudaMemcpyAsync(c->gate_mem, g, sizeof g, cudaMemcpyHostToDevice, st), "gate");
          cuda_check(cudaStreamSynchronize(st), "setup synchronize");
        }
      } catch (std::exception& e) {
        // an allocation that fails is an answer for this request, not for the loop
        if (std::string(e.what()).find("cudaMalloc") == std::string::npos) throw;
        fits = false;
      }
      const size_t bytes = c->arena.bytes();
      std::lock_guard<std::mutex> lk(S->mu);
      S->building--;
      S->building_ids.erase(r.id);
      S->bytes_in_use -= reserve;
      const bool cancelled = S->cancelled.erase(r.id) > 0;
      if (!fits || cancelled) {
        RbcRequestResult res{};
        res.id = r.id;
        res.status = cancelled ? RBC_ERR_CANCELLED : RBC_ERR_NOMEM;
        res.t_submit = r.t_submit;
        res.t_admit = res.t_done = S->now();
        res.grid_points = (long long)r.p.nx * r.p.ny;
        S->done.push_back(res);
        S->completed++;
        c.reset();
      } else {
        S->bytes_in_use += bytes;
        S->peak_bytes = std::max(S->peak_bytes, S->bytes_in_use);
        c->stream = S->stream;
        S->ready.push_back(RbcServer::Slot{r, c.release(), r.steps, 0.0, bytes, false});
      }
      S->cv.notify_all();
    }
  } catch (std::exception& e) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->failed = true;
    S->error = e.what();
    S->cv.notify_all();
  }
  if (st) cudaStreamDestroy(st);
}

// Move built cases into free slots.
static void server_admit(RbcServer* S) {
  std::lock_guard<std::mutex> lk(S->mu);
  // cases cancelled while they waited for a slot: retired without a step
  for (size_t i = 0; i < S->ready.size();) {
    RbcServer::Slot& sl = S->ready[i];
    if (!S->cancelled.erase(sl.r.id)) {
      i++;
      continue;
    }
    RbcRequestResult res{};
    res.id = sl.r.id;
    res.status = RBC_ERR_CANCELLED;
    res.t_submit = sl.r.t_submit;
    res.t_admit = res.t_done = S->now();
    res.grid_points = (long long)sl.r.p.nx * sl.r.p.ny;
    delete sl.c;
    S->bytes_in_use -= sl.bytes;
    S->done.push_back(res);
    S->completed++;
    S->ready.erase(S->ready.begin() + i);
  }
  while (!S->ready.empty() && (int)S->active.size() < S->cfg.max_active) {
    RbcServer::Slot sl = S->ready.front();
    S->ready.pop_front();
    sl.t_admit = S->now();
    S->active.push_back(sl);
    S->dirty = true;
  }
}

// Batched step of the active set: buckets, gate kernels, one CUDA graph.
static void server_rebuild(RbcServer* S) {
  server_free_graph(S);
  S->buckets.clear();
  S->plan_arena.reset(new Arena());
  S->plan_arena->set_stream_ordered(true);
  Arena& A = *S->plan_arena;
  std::vector<CaseDev> hd;
  for (auto& sl : S->active) {
    CaseDev d = sl.c->hd;
    d.gate = sl.c->gate_mem;
    hd.push_back(d);
  }
  CaseDev* d_cases = A.upload(hd);
  for (int i = 0; i < (int)S->active.size(); i++) {
    const RbcParams& p = S->active[i].r.p;
    int found = -1;
    for (size_t k = 0; k < S->buckets.size(); k++) {
      const RbcParams& q = S->active[S->buckets[k].members[0]].r.p;
      if ((q.kind == RBC_PERIODIC) == (p.kind == RBC_PERIODIC) && q.precision == p.precision) found = (int)k;
    }
    if (found < 0) {
      S->buckets.emplace_back();
      found = (int)S->buckets.size() - 1;
    }
    S->buckets[found].members.push_back(i);
  }
  // the forms of the passes: a CTA per lane by default; RBC_SERVER_FORM=1, 2,
  // 3 or 4 selects the 128-thread, the one-thread-per-sub-lane, that form with
  // the periodic Y2 launches fused, or 128-output GEMM tiles, for every case (a
  // case's arithmetic never depends on the other cases in any form, so results
  // stay the same alone and in a mix)
  int form = 0;
  if (const char* f = std::getenv("RBC_SERVER_FORM"))
    if (f[0] >= '1' && f[0] <= '5' && f[1] == '\0') form = f[0] - '0';
  for (auto& bk : S->buckets) {
    std::vector<const StepPlan*> plans;
    std::vector<const int*> gates;
    for (int m : bk.members) {
      RbcCase* mc = S->active[m].c;
      plans.push_back(form > 0 && (int)mc->plan_alts.size() >= form ? &mc->plan_alts[form - 1] : &mc->plan);
      gates.push_back(S->active[m].c->gate_mem + 1);
    }
    bk.plan = merge_plans(plans, bk.members, gates);
    upload_plan(A, bk.plan, bk.dp);
    bk.d_members = A.upload(bk.members);
  }
  const size_t nb = S->buckets.size();
  int prio_low = 0, prio_high = 0;
  cuda_check(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high), "stream priority range");
  while (S->branch.size() < nb) {
    cudaStream_t s;
    cudaEvent_t e;
    cuda_check(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio_low), "stream");
    cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
    S->branch.push_back(s);
    S->bev.push_back(e);
  }
  if (S->branch_hi == nullptr)
    cuda_check(cudaStreamCreateWithPriority(&S->branch_hi, cudaStreamNonBlocking, prio_high), "stream");
  // As in a batch, the group with the most work is the step's critical path
  // and runs on a high-priority branch, so the other groups fill the SMs it
  // leaves idle.  The set changes too often to time the groups, so the work
  // is estimated: grid points times the per-point cost of the kind measured
  // on the 256-case ensemble (box 0.77 ns, periodic 0.56 ns per grid point in
  // the mixed form), times 3 for the FP64 form.  Only the schedule depends on
  // it, not the numbers.
  size_t critical = 0;
  double best = -1.0;
  for (size_t k = 0; k < nb; k++) {
    double w = 0.0;
    for (int m : S->buckets[k].members) {
      const RbcParams& p = S->active[m].r.p;
      w += (double)p.nx * p.ny * (p.kind == RBC_PERIODIC ? 0.56 : 0.77) * (p.precision == RBC_PREC_FP64 ? 3.0 : 1.0);
    }
    if (w > best) {
      best = w;
      critical = k;
    }
  }
  const bool use_priority = nb > 1;
  cuda_check(cudaStreamBeginCapture(S->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  cudaError_t le = cudaEventRecord(S->fork, S->stream);
  for (size_t k = 0; k < nb && le == cudaSuccess; k++) {
    auto& bk = S->buckets[k];
    cudaStream_t s = (use_priority && k == critical) ? S->branch_hi : S->branch[k];
    le = cudaStreamWaitEvent(s, S->fork, 0);
    if (le == cudaSuccess) le = launch_gate(d_cases, bk.d_members, (int)bk.members.size(), s);
    for (size_t li = 0; li < bk.plan.launches.size() && le == cudaSuccess; li++)
      le = launch_entry(bk.plan.launches[li], bk.dp, li, s, d_cases);
    if (le == cudaSuccess) le = cudaEventRecord(S->bev[k], s);
    if (le == cudaSuccess) le = cudaStreamWaitEvent(S->stream, S->bev[k], 0);
  }
  cudaGraph_t g = nullptr;
  cudaError_t ce = cudaStreamEndCapture(S->stream, &g);
  cuda_check(le, "server capture");
  cuda_check(ce, "end capture");
  S->graph = g;
  cuda_check(cudaGraphInstantiate(&S->gexec, g, use_priority ? cudaGraphInstantiateFlagUseNodePriority : 0),
             "graph instantiate");
  S->rebuilds++;
  S->dirty = false;
}

static void server_finish(RbcServer* S) {
  {
    // active cases cancelled during the chunk stop here, between chunks
    std::lock_guard<std::mutex> lk(S->mu);
    for (auto& sl : S->active)
      if (S->cancelled.erase(sl.r.id)) sl.cancelled = true;
  }
  for (int i = (int)S->active.size() - 1; i >= 0; i--) {
    RbcServer::Slot& sl = S->active[i];
    if (sl.left > 0 && !sl.cancelled) continue;
    RbcRequestResult res{};
    res.id = sl.r.id;
    res.steps = (int)(sl.r.steps - sl.left);
    res.sim_time = sl.c->time;
    res.t_submit = sl.r.t_submit;
    res.t_admit = sl.t_admit;
    unsigned int st = 0;
    cuda_check(cudaMemcpy(&st, sl.c->hd.status, sizeof st, cudaMemcpyDeviceToHost), "status");
    res.status = st == 0 ? RBC_OK : ((st & 1u) ? RBC_ERR_NUMERIC : RBC_ERR_CUDA);
    if (sl.cancelled) res.status = RBC_ERR_CANCELLED;
    res.nu = eval_case(sl.c, RBC_NU);
    res.ke = eval_case(sl.c, RBC_KE);
    res.t_done = S->now();
    res.grid_points = sl.r.p.nx * sl.r.p.ny;
    delete sl.c;
    std::lock_guard<std::mutex> lk(S->mu);
    S->bytes_in_use -= sl.bytes;
    S->active.erase(S->active.begin() + i);
    S->dirty = true;
    S->done.push_back(res);
    S->completed++;
  }
  S->cv.notify_all();
}

static void server_main(RbcServer* S) {
  try {
    cuda_check(cudaSetDevice(S->device), "set device");
    for (;;) {
      server_admit(S);
      {
        std::unique_lock<std::mutex> lk(S->mu);
        if (S->stop || S->failed) break;
        if (S->active.empty()) {
          S->cv.notify_all();
          S->cv.wait_for(lk, std::chrono::milliseconds(1), [&] { return S->stop || !S->ready.empty(); });
          continue;
        }
      }
      if (S->dirty) {
        TraceRange tr("server: rebuild the batched step");
        server_rebuild(S);
      }
      const int n = S->cfg.chunk_steps;
      TraceRange tc("server: chunk");
      for (int k = 0; k < n; k++) cuda_check(cudaGraphLaunch(S->gexec, S->stream), "graph launch");
      cuda_check(cudaEventRecord(S->chunk_done, S->stream), "event record");
      {
        std::lock_guard<std::mutex> lk(S->mu);
        for (auto& sl : S->active) {
          const long applied = std::min<long>(n, sl.left);
          sl.left -= applied;
          sl.c->time += applied * sl.r.p.dt;
          S->gp_steps += (double)applied * sl.r.p.nx * sl.r.p.ny;
        }
        S->steps_launched += n;
      }
      cuda_check(cudaEventSynchronize(S->chunk_done), "chunk");
      server_finish(S);
    }
  } catch (std::exception& e) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->failed = true;
    S->error = e.what();
  }
  S->cv.notify_all();
}

extern "C" {

int rbc_server_create(const RbcServerConfig* cfg, RbcServer** out) {
  API_BEGIN
  require(cfg && out, "null argument");
  *out = nullptr;
  require(cfg->max_active > 0 && cfg->chunk_steps > 0 && cfg->hbm_budget_bytes > 0,
          "rbc_server_create: max_active, chunk_steps and hbm_budget_bytes must be positive");
  require(cfg->setup_threads > 0 && cfg->setup_threads <= 64, "rbc_server_create: setup_threads must be in [1, 64]");
  cuda_check(configure_prim_kernels(), "configure kernels");
  cuda_check(configure_step_kernels(), "configure step kernels");
  cuda_check(configure_mixed_kernels(), "configure mixed kernels");
  std::unique_ptr<RbcServer> S(new RbcServer());
  S->cfg = *cfg;
  cuda_check(cudaGetDevice(&S->device), "get device");
  cuda_check(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking), "stream");
  cuda_check(cudaEventCreateWithFlags(&S->fork, cudaEventDisableTiming), "event");
  cuda_check(cudaEventCreateWithFlags(&S->chunk_done, cudaEventDisableTiming), "event");
  S->t0 = std::chrono::steady_clock::now();
  RbcServer* raw = S.get();
  S->th = std::thread([raw] { server_main(raw); });
  for (int k = 0; k < cfg->setup_threads; k++) S->workers.emplace_back([raw] { server_worker(raw); });
  *out = S.release();
  API_END
}

int rbc_server_submit(RbcServer* S, const RbcParams* p, double horizon, uint64_t seed, long long* id) {
  API_BEGIN
  require(S && p && id, "null argument");
  validate_params(*p);
  require(std::isfinite(horizon) && horizon > 0, "rbc_server_submit: horizon must be positive");
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->failed) throw ApiError(RBC_ERR_CUDA, "server stopped: " + S->error);
  RbcServer::Req r;
  r.id = S->next_id++;
  r.p = *p;
  r.horizon = horizon;
  r.seed = seed;
  r.t_submit = S->now();
  r.steps = std::max<long>(1, std::lround(horizon / p->dt));
  S->pending.push_back(r);
  *id = r.id;
  S->cv.notify_all();
  API_END
}

int rbc_server_cancel(RbcServer* S, long long id, int* found) {
  API_BEGIN
  require(S && found, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  *found = 0;
  for (auto it = S->pending.begin(); it != S->pending.end(); ++it) {
    if (it->id != id) continue;
    RbcRequestResult res{};
    res.id = id;
    res.status = RBC_ERR_CANCELLED;
    res.t_submit = it->t_submit;
    res.t_admit = res.t_done = S->now();
    res.grid_points = (long long)it->p.nx * it->p.ny;
    S->pending.erase(it);
    S->done.push_back(res);
    S->completed++;
    *found = 1;
    S->cv.notify_all();
    return RBC_OK;
  }
  bool live = S->building_ids.count(id) > 0;
  for (auto& sl : S->ready) live = live || sl.r.id == id;
  for (auto& sl : S->active) live = live || sl.r.id == id;
  if (live) {
    S->cancelled.insert(id);
    *found = 1;
  }
  S->cv.notify_all();
  API_END
}

int rbc_server_poll(RbcServer* S, RbcRequestResult* out, int max_results, int* n) {
  API_BEGIN
  require(S && n && (out || max_results == 0), "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  int k = 0;
  while (k < max_results && !S->done.empty()) {
    out[k++] = S->done.front();
    S->done.pop_front();
  }
  *n = k;
  if (S->failed && k == 0) throw ApiError(RBC_ERR_CUDA, "server stopped: " + S->error);
  API_END
}

int rbc_server_wait_idle(RbcServer* S, double timeout_s, int* idle) {
  API_BEGIN
  require(S && idle, "null argument");
  std::unique_lock<std::mutex> lk(S->mu);
  auto quiet = [&] { return S->pending.empty() && S->ready.empty() && S->active.empty() && S->building == 0; };
  S->cv.wait_for(lk, std::chrono::duration<double>(std::max(0.0, timeout_s)), [&] { return S->failed || quiet(); });
  if (S->failed) throw ApiError(RBC_ERR_CUDA, "server stopped: " + S->error);
  *idle = quiet() ? 1 : 0;
  API_END
}

int rbc_server_stats(RbcServer* S, RbcServerStats* st) {
  API_BEGIN
  require(S && st, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  st->now = S->now();
  st->pending = (int)(S->pending.size() + S->ready.size()) + S->building;
  st->active = (int)S->active.size();
  st->completed = S->completed;
  st->bytes_in_use = S->bytes_in_use;
  st->grid_point_steps = S->gp_steps;
  st->steps_launched = S->steps_launched;
  st->rebuilds = S->rebuilds;
  st->peak_bytes_in_use = S->peak_bytes;
  API_END
}

int rbc_server_destroy(RbcServer* S) {
  API_BEGIN
  if (!S) return RBC_OK;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv.notify_all();
  if (S->th.joinable()) S->th.join();
  for (auto& w : S->workers)
    if (w.joinable()) w.join();
  cudaStreamSynchronize(S->stream);
  server_free_graph(S);
  for (auto& sl : S->active) delete sl.c;
  for (auto& sl : S->ready) delete sl.c;
  S->active.clear();
  S->ready.clear();
  S->plan_arena.reset();
  for (auto s : S->branch) cudaStreamDestroy(s);
  if (S->branch_hi) cudaStreamDestroy(S->branch_hi);
  for (auto e : S->bev) cudaEventDestroy(e);
  cudaEventDestroy(S->fork);
  cudaEventDestroy(S->chunk_done);
  cudaStreamDestroy(S->stream);
  delete S;
  API_END
}

}  // extern "C"

// ============================================================================
// Snapshots: Navier2D::write / Navier2D::read (navier.rs:961-1013) in a
// self-describing binary file (no HDF5 library here) with a JSON sidecar.
// Datasets follow the reference's HDF5 layout: groups temp, ux, uy, pres with
// "v" (physical; temp includes the boundary field) and "vhat" (spectral;
// complex arrays as "vhat_re" / "vhat_im"), the grid "x", "dx", "y", "dy" at
// the root, and the scalars time, ra, pr, nu, kappa.  Reading restores vhat
// of each group, broadcasting (copying the overlapping low modes, read.rs:
// 116-125) when the resolution differs, and the time.
//
// File layout (little-endian):
//   "RBCSNAP1" | u32 version | u32 ndatasets | i32 nx, ny, kind, precision |
//   f64 dt, aspect | f64 time, ra, pr, nu, kappa |
//   ndatasets x { char name[32] | i64 rows, cols | u64 offset, bytes } | data
// ============================================================================
#include <cstdio>
#include <fstream>

namespace {

struct SnapEntry {
  char name[32];
  int64_t rows, cols;
  uint64_t offset, bytes;
};

constexpr char kSnapMagic[8] = {'R', 'B', 'C', 'S', 'N', 'A', 'P', '1'};

void put_dataset(std::vector<SnapEntry>& table, std::vector<std::vector<double>>& blobs, const std::string& name,
                 int64_t rows, int64_t cols, std::vector<double> data) {
  SnapEntry e{};
  std::snprintf(e.name, sizeof e.name, "%s", name.c_str());
  e.rows = rows;
  e.cols = cols;
  e.bytes = data.size() * 8;
  table.push_back(e);
  blobs.push_back(std::move(data));
}

}  // namespace

extern "C" {

int rbc_write_snapshot(RbcCase* c, const char* path) {
  API_BEGIN
  require(c && path, "null argument");
  c->sync();
  const int nx = c->p.nx, ny = c->p.ny;
  std::vector<SnapEntry> table;
  std::vector<std::vector<double>> blobs;
  const struct { const char* group; int field; } groups[4] = {
      {"temp", RBC_TEMP}, {"ux", RBC_UX}, {"uy", RBC_UY}, {"pres", RBC_PRES}};
  std::vector<double> bc((size_t)nx * ny);
  cuda_check(cudaMemcpy(bc.data(), c->bc_phys, bc.size() * 8, cudaMemcpyDeviceToHost), "d2h");
  for (const auto& g : groups) {
    const SpaceDev& s = field_space(c, g.field);
    // physical values (Field2::backward; the temperature with the boundary field added)
    space_backward(s, field_ptr(c, g.field), c->phys[0], c->tmp, c->stream);
    std::vector<double> v((size_t)nx * ny);
    cuda_check(cudaMemcpyAsync(v.data(), c->phys[0], v.size() * 8, cudaMemcpyDeviceToHost, c->stream), "d2h");
    c->sync();
    if (g.field == RBC_TEMP)
      for (size_t k = 0; k < v.size(); k++) v[k] += bc[k];
    put_dataset(table, blobs, std::string(g.group) + "/v", nx, ny, std::move(v));
    const size_t n = spec_doubles(c, g.field);
    std::vector<double> vh(n);
    cuda_check(cudaMemcpy(vh.data(), field_ptr(c, g.field), n * 8, cudaMemcpyDeviceToHost), "d2h");
    if (s.cplx) {
      std::vector<double> re(n / 2), im(n / 2);
      for (size_t k = 0; k < n / 2; k++) {
        re[k] = vh[2 * k];
        im[k] = vh[2 * k + 1];
      }
      put_dataset(table, blobs, std::string(g.group) + "/vhat_re", s.spec0, s.spec1, std::move(re));
      put_dataset(table, blobs, std::string(g.group) + "/vhat_im", s.spec0, s.spec1, std::move(im));
    } else {
      put_dataset(table, blobs, std::string(g.group) + "/vhat", s.spec0, s.spec1, std::move(vh));
    }
  }
  // solid mask (navier.rs:998-1001)
  if (!c->solid_host[0].empty()) put_dataset(table, blobs, "solid/mask", nx, ny, c->solid_host[0]);
  std::vector<double> x, y;
  coords(c, RBC_TEMP, x, y);
  put_dataset(table, blobs, "x", (int64_t)x.size(), 1, x);
  put_dataset(table, blobs, "dx", (int64_t)x.size(), 1, get_dx(x, c->periodic));
  put_dataset(table, blobs, "y", (int64_t)y.size(), 1, y);
  put_dataset(table, blobs, "dy", (int64_t)y.size(), 1, get_dx(y, false));
  // offsets
  const uint64_t head = 8 + 4 + 4 + 4 * 4 + 8 * 2 + 8 * 5 + table.size() * sizeof(SnapEntry);
  uint64_t off = head;
  for (auto& e : table) {
    e.offset = off;
    off += e.bytes;
  }
  const std::string tmp_path = std::string(path) + ".partial";
  {
    std::ofstream f(tmp_path, std::ios::binary | std::ios::trunc);
    if (!f) throw ApiError(RBC_ERR_INVALID, std::string("rbc_write_snapshot: cannot open ") + tmp_path);
    const uint32_t version = 1, nd = (uint32_t)table.size();
    const int32_t ip[4] = {c->p.nx, c->p.ny, c->p.kind, c->p.precision};
    const double dp[2] = {c->p.dt, c->p.aspect};
    const double sc[5] = {c->time, c->p.ra, c->p.pr, c->nu, c->ka};
    f.write(kSnapMagic, 8);
    f.write(reinterpret_cast<const char*>(&version), 4);
    f.write(reinterpret_cast<const char*>(&nd), 4);
    f.write(reinterpret_cast<const char*>(ip), sizeof ip);
    f.write(reinterpret_cast<const char*>(dp), sizeof dp);
    f.write(reinterpret_cast<const char*>(sc), sizeof sc);
    f.write(reinterpret_cast<const char*>(table.data()), table.size() * sizeof(SnapEntry));
    for (const auto& b : blobs) f.write(reinterpret_cast<const char*>(b.data()), b.size() * 8);
    if (!f) throw ApiError(RBC_ERR_INVALID, "rbc_write_snapshot: write failed");
  }
  if (std::rename(tmp_path.c_str(), path) != 0)
    throw ApiError(RBC_ERR_INVALID, std::string("rbc_write_snapshot: cannot create ") + path);
  // human-readable sidecar
  std::ofstream js(std::string(path) + ".json", std::ios::trunc);
  js.precision(17);
  js << "{\"format\": \"RBCSNAP1\", \"version\": 1, \"binary\": \"" << path << "\",\n"
     << " \"params\": {\"nx\": " << c->p.nx << ", \"ny\": " << c->p.ny << ", \"kind\": " << c->p.kind
     << ", \"precision\": " << c->p.precision << ", \"ra\": " << c->p.ra << ", \"pr\": " << c->p.pr
     << ", \"dt\": " << c->p.dt << ", \"aspect\": " << c->p.aspect << "},\n"
     << " \"scalars\": {\"time\": " << c->time << ", \"ra\": " << c->p.ra << ", \"pr\": " << c->p.pr
     << ", \"nu\": " << c->nu << ", \"kappa\": " << c->ka << "},\n \"datasets\": [";
  for (size_t k = 0; k < table.size(); k++)
    js << (k ? ",\n  " : "\n  ") << "{\"name\": \"" << table[k].name << "\", \"shape\": [" << table[k].rows << ", "
       << table[k].cols << "], \"dtype\": \"<f8\", \"offset\": " << table[k].offset << "}";
  js << "\n ]}\n";
  API_END
}

int rbc_read_snapshot(RbcCase* c, const char* path) {
  API_BEGIN
  require(c && path, "null argument");
  std::ifstream f(path, std::ios::binary);
  if (!f) throw ApiError(RBC_ERR_INVALID, std::string("rbc_read_snapshot: cannot open ") + path);
  char magic[8];
  uint32_t version = 0, nd = 0;
  int32_t ip[4];
  double dp[2], sc[5];
  f.read(magic, 8);
  f.read(reinterpret_cast<char*>(&version), 4);
  f.read(reinterpret_cast<char*>(&nd), 4);
  f.read(reinterpret_cast<char*>(ip), sizeof ip);
  f.read(reinterpret_cast<char*>(dp), sizeof dp);
  f.read(reinterpret_cast<char*>(sc), sizeof sc);
  if (!f || std::memcmp(magic, kSnapMagic, 8) != 0 || version != 1 || nd > 4096)
    throw ApiError(RBC_ERR_INVALID, "rbc_read_snapshot: not a snapshot file of this library");
  std::vector<SnapEntry> table(nd);
  f.read(reinterpret_cast<char*>(table.data()), nd * sizeof(SnapEntry));
  if (!f) throw ApiError(RBC_ERR_INVALID, "rbc_read_snapshot: truncated header");
  auto find = [&](const std::string& name) -> const SnapEntry* {
    for (const auto& e : table)
      if (name == std::string(e.name, strnlen(e.name, sizeof e.name))) return &e;
    return nullptr;
  };
  auto load = [&](const SnapEntry& e) {
    if (e.rows < 0 || e.cols < 0 || e.bytes != (uint64_t)(e.rows * e.cols) * 8)
      throw ApiError(RBC_ERR_INVALID, "rbc_read_snapshot: inconsistent dataset entry");
    std::vector<double> v((size_t)(e.rows * e.cols));
    f.seekg((std::streamoff)e.offset);
    f.read(reinterpret_cast<char*>(v.data()), e.bytes);
    if (!f) throw ApiError(RBC_ERR_INVALID, "rbc_read_snapshot: truncated data");
    return v;
  };
  const struct { const char* group; int field; } groups[4] = {
      {"temp", RBC_TEMP}, {"ux", RBC_UX}, {"uy", RBC_UY}, {"pres", RBC_PRES}};
  for (const auto& g : groups) {
    const SpaceDev& s = field_space(c, g.field);
    const std::string base = std::string(g.group) + "/vhat";
    std::vector<double> cur(spec_doubles(c, g.field), 0.0);
    if (s.cplx) {
      const SnapEntry* re = find(base + "_re");
      const SnapEntry* im = find(base + "_im");
      if (!re || !im) throw ApiError(RBC_ERR_INVALID, "rbc_read_snapshot: missing complex dataset " + base);
      std::vector<double> vr = load(*re), vi = load(*im);
      const int64_t r = std::min<int64_t>(re->rows, s.spec0), q = std::min<int64_t>(re->cols, s.spec1);
      for (int64_t i = 0; i < r; i++)
        for (int64_t j = 0; j < q; j++) {
          cur[2 * ((size_t)i * s.spec1 + j)] = vr[(size_t)i * re->cols + j];
          cur[2 * ((size_t)i * s.spec1 + j) + 1] = vi[(size_t)i * re->cols + j];
        }
    } else {
      const SnapEntry* e = find(base);
      if (!e) throw ApiError(RBC_ERR_INVALID, "rbc_read_snapshot: missing dataset " + base);
      std::vector<double> v = load(*e);
      const int64_t r = std::min<int64_t>(e->rows, s.spec0), q = std::min<int64_t>(e->cols, s.spec1);
      for (int64_t i = 0; i < r; i++)
        for (int64_t j = 0; j < q; j++) cur[(size_t)i * s.spec1 + j] = v[(size_t)i * e->cols + j];
    }
    c->sync();
    cuda_check(cudaMemcpy(field_ptr(c, g.field), cur.data(), cur.size() * 8, cudaMemcpyHostToDevice), "h2d");
  }
  c->time = sc[0];
  API_END
}

}  // extern "C"

// ============================================================================
// Statistics (src/navier/statistics.rs) and the diagnostics series of
// Navier2D::callback (navier.rs:826-838), computed on the device.
// ============================================================================
namespace {

void stats_alloc(RbcCase* c) {
  if (c->st_field[0]) return;
  const size_t bytes = (size_t)c->sp_field.spec0 * c->sp_field.spec1 * (c->periodic ? 16 : 8);
  for (auto& f : c->st_field) f = c->arena.alloc(bytes);
}

size_t field_doubles(const RbcCase* c) {
  return (size_t)c->sp_field.spec0 * c->sp_field.spec1 * (c->periodic ? 2 : 1);
}

}  // namespace

extern "C" {

int rbc_stats_reset(RbcCase* c) {
  // Statistics::new (statistics.rs:55-87)
  API_BEGIN
  require(c != nullptr, "null case");
  stats_alloc(c);
  c->sync();
  for (auto f : c->st_field) cuda_check(cudaMemset(f, 0, field_doubles(c) * 8), "clear statistics");
  c->st_tot_time = c->time;
  c->st_avg_time = 0.0;
  c->st_num_save = 0;
  API_END
}

int rbc_stats_update(RbcCase* c) {
  // Statistics::update (statistics.rs:127-153) with that = to_ortho(temp) +
  // to_ortho(fieldbc), uxhat / uyhat = to_ortho of the velocities
  // (navier.rs:795-800); the Nusselt field as statistics.rs:206-234
  API_BEGIN
  require(c != nullptr, "null case");
  stats_alloc(c);
  if (c->time < c->st_tot_time) throw ApiError(RBC_ERR_INVALID, "rbc_stats_update: time precedes the statistics");
  cudaStream_t st = c->stream;
  const int nx = c->p.nx, ny = c->p.ny;
  const size_t nd = field_doubles(c), nphys = (size_t)nx * ny;
  const CaseDev& h = c->hd;
  void* that = c->spec_tmp[0];
  space_to_ortho(c->sp_t, h.temp, that, c->tmp, st);
  phys_combine(3, (const double*)that, (const double*)h.bc_ortho, nullptr, 0, 0, (double*)that, nd, st);
  const double w = (double)c->st_num_save;
  phys_combine(7, (const double*)c->st_field[0], (const double*)that, nullptr, w, w + 1.0,
               (double*)c->st_field[0], nd, st);
  space_to_ortho(c->sp_u, h.ux, c->st_field[1], c->tmp, st);
  space_to_ortho(c->sp_u, h.uy, c->st_field[2], c->tmp, st);
  // nusselt: ((dT/dz / -s_y) + uy T / kappa) * 2 s_y, forward
  space_backward(c->sp_field, c->st_field[2], c->phys[1], c->tmp, st);  // uy
  space_backward(c->sp_field, that, c->phys[0], c->tmp, st);            // T
  void* g = c->spec_tmp[1];
  space_gradient(c->sp_field, that, g, 0, 1, nullptr, c->tmp, st);
  phys_combine(6, (const double*)g, nullptr, nullptr, c->scale[1] * -1.0, 0, (double*)g, nd, st);
  space_backward(c->sp_field, g, c->phys[2], c->tmp, st);  // dT/dz
  phys_combine(0, c->phys[2], c->phys[0], c->phys[1], c->ka, c->scale[1], c->phys[3], nphys, st);
  space_forward(c->sp_field, c->phys[3], c->st_field[3], c->tmp, st);
  c->sync();
  c->st_num_save += 1;
  c->st_avg_time += c->time - c->st_tot_time;
  c->st_tot_time = c->time;
  API_END
}

int rbc_stats_info(const RbcCase* c, double* tot_time, double* avg_time, long* num_save) {
  API_BEGIN
  require(c && tot_time && avg_time && num_save, "null argument");
  *tot_time = c->st_tot_time;
  *avg_time = c->st_avg_time;
  *num_save = c->st_num_save;
  API_END
}

// which: 0 temperature average, 1 ux, 2 uy, 3 Nusselt field (spectral, `field` space)
int rbc_stats_get(RbcCase* c, int which, double* host, size_t n_doubles) {
  API_BEGIN
  require(c && host && which >= 0 && which < 4, "rbc_stats_get: invalid argument");
  stats_alloc(c);
  require(n_doubles == field_doubles(c), "rbc_stats_get: size mismatch, expected " + std::to_string(field_doubles(c)));
  c->sync();
  cuda_check(cudaMemcpy(host, c->st_field[which], n_doubles * 8, cudaMemcpyDeviceToHost), "d2h");
  API_END
}

int rbc_stats_write(RbcCase* c, const char* path) {
  // Statistics::write (statistics.rs:165-191): groups temp, ux, uy, nusselt
  // (v and vhat) and the scalars, in the snapshot file format
  API_BEGIN
  require(c && path, "null argument");
  stats_alloc(c);
  c->sync();
  const int nx = c->p.nx, ny = c->p.ny;
  const SpaceDev& s = c->sp_field;
  std::vector<SnapEntry> table;
  std::vector<std::vector<double>> blobs;
  const char* groups[4] = {"temp", "ux", "uy", "nusselt"};
  for (int k = 0; k < 4; k++) {
    space_backward(s, c->st_field[k], c->phys[0], c->tmp, c->stream);
    std::vector<double> v((size_t)nx * ny);
    cuda_check(cudaMemcpyAsync(v.data(), c->phys[0], v.size() * 8, cudaMemcpyDeviceToHost, c->stream), "d2h");
    c->sync();
    put_dataset(table, blobs, std::string(groups[k]) + "/v", nx, ny, std::move(v));
    std::vector<double> vh(field_doubles(c));
    cuda_check(cudaMemcpy(vh.data(), c->st_field[k], vh.size() * 8, cudaMemcpyDeviceToHost), "d2h");
    if (s.cplx) {
      std::vector<double> re(vh.size() / 2), im(vh.size() / 2);
      for (size_t q = 0; q < re.size(); q++) { re[q] = vh[2 * q]; im[q] = vh[2 * q + 1]; }
      put_dataset(table, blobs, std::string(groups[k]) + "/vhat_re", s.spec0, s.spec1, std::move(re));
      put_dataset(table, blobs, std::string(groups[k]) + "/vhat_im", s.spec0, s.spec1, std::move(im));
    } else {
      put_dataset(table, blobs, std::string(groups[k]) + "/vhat", s.spec0, s.spec1, std::move(vh));
    }
  }
  put_dataset(table, blobs, "tot_time", 1, 1, {c->st_tot_time});
  put_dataset(table, blobs, "avg_time", 1, 1, {c->st_avg_time});
  put_dataset(table, blobs, "num_save", 1, 1, {(double)c->st_num_save});
  put_dataset(table, blobs, "ka", 1, 1, {c->ka});
  std::vector<double> x, y;
  coords(c, RBC_TEMP, x, y);
  put_dataset(table, blobs, "x", (int64_t)x.size(), 1, x);
  put_dataset(table, blobs, "dx", (int64_t)x.size(), 1, get_dx(x, c->periodic));
  put_dataset(table, blobs, "y", (int64_t)y.size(), 1, y);
  put_dataset(table, blobs, "dy", (int64_t)y.size(), 1, get_dx(y, false));
  const uint64_t head = 8 + 4 + 4 + 4 * 4 + 8 * 2 + 8 * 5 + table.size() * sizeof(SnapEntry);
  uint64_t off = head;
  for (auto& e : table) { e.offset = off; off += e.bytes; }
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) throw ApiError(RBC_ERR_INVALID, std::string("rbc_stats_write: cannot open ") + path);
  const uint32_t version = 1, nd = (uint32_t)table.size();
  const int32_t ip[4] = {c->p.nx, c->p.ny, c->p.kind, c->p.precision};
  const double dp[2] = {c->p.dt, c->p.aspect};
  const double sc[5] = {c->st_tot_time, c->p.ra, c->p.pr, c->nu, c->ka};
  f.write(kSnapMagic, 8);
  f.write(reinterpret_cast<const char*>(&version), 4);
  f.write(reinterpret_cast<const char*>(&nd), 4);
  f.write(reinterpret_cast<const char*>(ip), sizeof ip);
  f.write(reinterpret_cast<const char*>(dp), sizeof dp);
  f.write(reinterpret_cast<const char*>(sc), sizeof sc);
  f.write(reinterpret_cast<const char*>(table.data()), table.size() * sizeof(SnapEntry));
  for (const auto& b : blobs) f.write(reinterpret_cast<const char*>(b.data()), b.size() * 8);
  if (!f) throw ApiError(RBC_ERR_INVALID, "rbc_stats_write: write failed");
  API_END
}

int rbc_diag_record(RbcCase* c) {
  // Navier2D::callback diagnostics (navier.rs:819-838): time, Nu, Nuvol, Re
  API_BEGIN
  require(c != nullptr, "null case");
  const double nu = eval_case(c, RBC_NU), nuv = eval_case(c, RBC_NUVOL), re = eval_case(c, RBC_RE);
  c->dg_time.push_back(c->time);
  c->dg_nu.push_back(nu);
  c->dg_nuvol.push_back(nuv);
  c->dg_re.push_back(re);
  API_END
}

int rbc_diag_series(const RbcCase* c, double* time, double* nu, double* nuvol, double* re, int max_entries, int* n) {
  API_BEGIN
  require(c && n, "null argument");
  *n = (int)c->dg_time.size();
  const int k = std::min(*n, std::max(max_entries, 0));
  for (int i = 0; i < k; i++) {
    if (time) time[i] = c->dg_time[i];
    if (nu) nu[i] = c->dg_nu[i];
    if (nuvol) nuvol[i] = c->dg_nuvol[i];
    if (re) re[i] = c->dg_re[i];
  }
  API_END
}

}  // extern "C"
