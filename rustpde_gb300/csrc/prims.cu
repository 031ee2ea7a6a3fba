// prims.cu -- generic 2-D funspace / solver operations (see prims.h).
#include <cmath>
#include <algorithm>
#include <cstring>
#include <stdexcept>

#include "lane_ops.cuh"
#include "per_device.h"
#include "prims.h"

#include <map>
#include <mutex>
#include <tuple>

namespace rbc {

// ---------------------------------------------------------------- arena
// library-owned stream of the stream-ordered arenas, one per device
static cudaStream_t pool_stream() {
  static std::mutex mu;
  static std::map<int, cudaStream_t> streams;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = streams.find(dev);
  if (it != streams.end()) return it->second;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    throw std::runtime_error("cudaStreamCreate failed");
  // keep freed blocks in the pool for the next cases instead of returning them
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  streams[dev] = s;
  return s;
}

Arena::~Arena() {
  if (ordered_) {
    cudaStream_t s = pool_stream();
    for (void* p : ptrs_) cudaFreeAsync(p, s);
  } else {
    for (void* p : ptrs_) cudaFree(p);
  }
}
void* Arena::alloc(size_t bytes) {
  if (bytes == 0) bytes = 16;
  void* p = nullptr;
  if (ordered_) {
    cudaStream_t s = pool_stream();
    cudaError_t e = cudaMallocAsync(&p, bytes, s);
    if (e != cudaSuccess) throw std::runtime_error(std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    e = cudaMemsetAsync(p, 0, bytes, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // usable from any stream once this returns
    if (e != cudaSuccess) {
      cudaFreeAsync(p, s);
      throw std::runtime_error(std::string("cudaMemset failed: ") + cudaGetErrorString(e));
    }
  } else {
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) throw std::runtime_error(std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
    e = cudaMemset(p, 0, bytes);
    if (e != cudaSuccess) {
      cudaFree(p);
      throw std::runtime_error(std::string("cudaMemset failed: ") + cudaGetErrorString(e));
    }
  }
  ptrs_.push_back(p);
  bytes_ += bytes;
  return p;
}
void Arena::copy_h2d(void* d, const void* h, size_t n) {
  cudaError_t e = cudaMemcpy(d, h, n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) throw std::runtime_error(std::string("cudaMemcpy failed: ") + cudaGetErrorString(e));
}

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------- uploads
BasisDev upload_basis(Arena& a, const HostBasis& b) {
  BasisDev d;
  std::memset(&d, 0, sizeof d);
  d.kind = b.kind;
  d.n = b.n;
  d.m = b.m;
  d.diag = a.upload(b.diag);
  d.unit_diag = !b.diag.empty() && std::all_of(b.diag.begin(), b.diag.end(), [](double v) { return v == 1.0; });
  d.low2 = a.upload(b.low2);
  d.fo_off = a.upload(b.fo_off);
  d.fo_w = a.upload(b.fo_w);
  d.fo_dinv = a.upload(b.fo_dinv);
  if (!b.fo_dinv.empty()) {
    const int m = b.m;
    std::vector<double> fa(m), fb(m), fc(m, 0.0);
    for (int i = 0; i < m; i++) {
      fa[i] = b.diag[i] * b.fo_dinv[i];
      fb[i] = b.low2[i] * b.fo_dinv[i];
      if (i >= 2) fc[i] = -b.fo_off[i - 2] * b.fo_dinv[i];
    }
    d.fo_a = a.upload(fa);
    d.fo_b = a.upload(fb);
    d.fo_c = a.upload(fc);
  }
  for (int i = 0; i < 2; i++) { d.t0[i] = b.t0[i]; d.t1[i] = b.t1[i]; }
  for (int i = 0; i < 4; i++) d.bc_inv[i] = b.bc_inv[i];
  return d;
}

static int ilog2(int v) {
  int r = 0;
  while ((1 << r) < v) r++;
  return r;
}

ChebXformDev upload_cheb(Arena& a, int n, bool allow_fft) {
  ChebXformDev d;
  std::memset(&d, 0, sizeof d);
  d.n = n;
  int N = n - 1;
  d.inv_nm1 = 1.0 / (double)(n - 1);
  d.use_fft = (allow_fft && N >= 2 && is_pow2(N)) ? 1 : 0;
  if (d.use_fft) {
    d.L = 2 * N;
    d.log2L = ilog2(d.L);
    d.tw = reinterpret_cast<const double2*>(a.upload(twiddles(d.L)));
  } else {
    d.L = 0;
    d.fwd = a.upload(cheb_dense_forward(n));
    d.bwd = a.upload(cheb_dense_backward(n));
  }
  return d;
}

FourierXformDev upload_fourier(Arena& a, int n) {
  FourierXformDev d;
  std::memset(&d, 0, sizeof d);
  if (n < 4) throw std::runtime_error("FourierR2c length must be >= 4");
  d.n = n;
  d.M = (n & 1) ? n : n / 2;
  if (is_pow2(d.M)) {
    d.log2M = ilog2(d.M);
  } else {
    // mixed-radix stages: radix 4 while it divides, then 2, 3, 5, 7 and the
    // remaining prime factors
    d.log2M = -1;
    int r = d.M;
    auto push = [&](int p) {
      if (d.nrad >= 16) throw std::runtime_error("FourierR2c: too many FFT stages");
      d.rad[d.nrad++] = p;
      r /= p;
    };
    while (r % 4 == 0) push(4);
    while (r % 2 == 0) push(2);
    for (int p = 3; p * p <= r; p += 2)
      while (r % p == 0) push(p);
    if (r > 1) push(r);
  }
  std::vector<double> tw = twiddles(n);
  d.tw = reinterpret_cast<const double2*>(a.upload(tw));
  std::vector<float> twf(tw.size());
  for (size_t i = 0; i < tw.size(); i++) twf[i] = (float)tw[i];
  d.twf = reinterpret_cast<const float2*>(a.upload(twf));
  return d;
}

PinvDev upload_pinv(Arena& a, int n) {
  Pinv p = make_pinv(n);
  PinvDev d;
  std::memset(&d, 0, sizeof d);
  d.n = n;
  d.dia = a.upload(p.dia);
  d.up1 = a.upload(p.up1);
  d.up2 = a.upload(p.up2);
  return d;
}

FdmaDev upload_fdma(Arena& a, const std::vector<Band4>& rows) {
  FdmaDev d;
  std::memset(&d, 0, sizeof d);
  int m = rows[0].n;
  int R = (int)rows.size();
  d.m = m;
  d.rows = R;
  d.stride = m;
  std::vector<double> low((size_t)R * m, 0.0), dinv((size_t)R * m, 0.0), up1((size_t)R * m, 0.0),
      up2((size_t)R * m, 0.0);
  // device form of the swept factors: low negated, 1/dia, and the upper
  // diagonals divided by dia and negated (x_j = x_j/dia_j + up1' x_{j+2} + up2' x_{j+4})
  for (int r = 0; r < R; r++) {
    const Band4& f = rows[r];
    for (size_t i = 0; i < f.low.size(); i++) low[(size_t)r * m + i] = -f.low[i];
    for (int i = 0; i < m; i++) dinv[(size_t)r * m + i] = 1.0 / f.dia[i];
    for (size_t i = 0; i < f.up1.size(); i++) up1[(size_t)r * m + i] = -f.up1[i] / f.dia[i];
    for (size_t i = 0; i < f.up2.size(); i++) up2[(size_t)r * m + i] = -f.up2[i] / f.dia[i];
  }
  d.low = a.upload(low);
  d.dinv = a.upload(dinv);
  d.up1 = a.upload(up1);
  d.up2 = a.upload(up2);
  return d;
}

static size_t space_pass_smem(const SpaceDev& s);

void build_space(Arena& a, SpaceDev& s, int kind0, int n0, int kind1, int n1) {
  if (kind1 == FOURIER) throw std::runtime_error("FourierR2c is supported along axis 0 only");
  s.hb0 = make_basis(kind0, n0);
  s.hb1 = make_basis(kind1, n1);
  s.b0 = upload_basis(a, s.hb0);
  s.b1 = upload_basis(a, s.hb1);
  s.cplx = kind0 == FOURIER;
  if (s.cplx) s.f0 = upload_fourier(a, n0);
  else s.c0 = upload_cheb(a, n0);
  s.c1 = upload_cheb(a, n1);
  s.phys0 = n0; s.phys1 = n1;
  s.spec0 = s.hb0.m; s.spec1 = s.hb1.m;
  s.ortho0 = s.hb0.ortho_len(); s.ortho1 = s.hb1.ortho_len();
  // a DCT-I through an FFT needs 2(n-1) complex work elements per lane in
  // shared memory; where a pass would then exceed the device's limit, the
  // dense form of the transform (an n x n product per lane) is used instead
  if (space_pass_smem(s) > smem_limit()) {
    if (!s.cplx && s.c0.use_fft) s.c0 = upload_cheb(a, n0, false);
    if (s.c1.use_fft) s.c1 = upload_cheb(a, n1, false);
  }
  const size_t need = space_pass_smem(s);
  if (need > smem_limit())
    throw SizeError("space of lengths " + std::to_string(n0) + " x " + std::to_string(n1) + " needs " +
                    std::to_string(need) + " bytes of shared memory per block for its lanes; this device allows " +
                    std::to_string(smem_limit()));
}

Band4 adi_factor(const HostBasis& b, double c) {
  // hholtz_adi.rs:44-63: Fdma::from_matrix(mat_a - mat_b * c)
  Band4 A, B;
  if (b.fourier()) {
    int m = b.m;
    Band4 f;
    f.n = m;
    f.low.assign(m - 2, 0.0); f.dia.assign(m, 0.0); f.up1.assign(m - 2, 0.0); f.up2.assign(std::max(m - 4, 0), 0.0);
    for (int i = 0; i < m; i++) {
      double lap = -(double)i * (double)i;
      f.dia[i] = 1.0 - lap * c;
    }
    band_sweep(f);
    return f;
  }
  hholtz_ingredients(b, A, B);
  Band4 f = A;
  for (size_t i = 0; i < f.low.size(); i++) f.low[i] = A.low[i] - B.low[i] * c;
  for (size_t i = 0; i < f.dia.size(); i++) f.dia[i] = A.dia[i] - B.dia[i] * c;
  for (size_t i = 0; i < f.up1.size(); i++) f.up1[i] = A.up1[i] - B.up1[i] * c;
  for (size_t i = 0; i < f.up2.size(); i++) f.up2[i] = A.up2[i] - B.up2[i] * c;
  band_sweep(f);
  return f;
}

std::vector<Band4> hholtz_rows(const HostBasis& bx, const HostBasis& by, double cx, double cy, double alpha,
                               bool poisson, std::vector<double>* lam_out, std::vector<double>* fwd,
                               std::vector<double>* bwd, std::string* err) {
  // FdmaTensor::from_matrix (fdma_tensor.rs:105-153) with
  //  Hholtz  (hholtz.rs:42-76):  laplacian = -mat_b * c, mass = mat_a, alpha = 1
  //  Poisson (poisson.rs:50-90): laplacian =  mat_b * c, mass = mat_a, alpha = 0
  if (by.fourier() || !by.composite() || by.bc()) throw std::runtime_error("tensor solver: axis 1 must be composite");
  Band4 Ay, By;
  hholtz_ingredients(by, Ay, By);
  Band4 a1 = By;  // laplacian along y
  for (auto* v : {&a1.low, &a1.dia, &a1.up1, &a1.up2}) {
    size_t k = 0;
    const std::vector<double>& src = (v == &a1.low) ? By.low : (v == &a1.dia) ? By.dia : (v == &a1.up1) ? By.up1 : By.up2;
    for (double& e : *v) { e = poisson ? src[k] * cy : (-1.0 * src[k]) * cy; k++; }
  }
  const Band4& c1 = Ay;
  std::vector<double> lam;
  if (bx.fourier()) {
    // diagonal laplacian diag(-k^2)
    lam.resize(bx.m);
    for (int i = 0; i < bx.m; i++) {
      double lap = -((double)i * (double)i);
      lam[i] = poisson ? lap * cx : (-1.0 * lap) * cx;
    }
  } else {
    if (!bx.composite() || bx.bc()) throw std::runtime_error("tensor solver: axis 0 must be composite or Fourier");
    // The eigen-decomposition of inv(C) (s B) with s = +1 (Poisson) or -1
    // (Hholtz) depends on the basis and size only; the scale cx > 0 of the
    // reference's matrix multiplies the eigenvalues and leaves the
    // eigenvectors unchanged, so it is applied afterwards and the O(n^3)
    // decomposition is computed once per (basis, size, sign) and shared.
    struct Eig {
      std::vector<double> lam, fwd, bwd;
    };
    static std::mutex mu;
    static std::map<std::tuple<int, int, bool>, Eig> cache;
    const auto key = std::make_tuple(bx.kind, bx.n, poisson);
    const Eig* E = nullptr;
    {
      std::lock_guard<std::mutex> lk(mu);
      auto it = cache.find(key);
      if (it != cache.end()) E = &it->second;
    }
    if (E == nullptr) {
      Band4 Ax, Bx;
      hholtz_ingredients(bx, Ax, Bx);
      int m = bx.m;
      std::vector<double> a0 = band_dense(Bx), c0 = band_dense(Ax);
      for (double& e : a0) e = poisson ? e : (-1.0 * e);
      std::vector<double> cinv;
      if (!invert(m, c0, cinv)) throw std::runtime_error("tensor solver: singular mass matrix");
      std::vector<double> xmat = matmul(m, m, m, cinv, a0);
      Eig ne;
      std::string e2;
      if (!eig_real(m, xmat, ne.lam, ne.bwd, &e2)) {
        if (err) *err = e2;
        throw std::runtime_error(e2);
      }
      std::vector<double> P;
      if (!invert(m, ne.bwd, P)) throw std::runtime_error("tensor solver: eigenvector matrix is singular");
      ne.fwd = matmul(m, m, m, P, cinv);
      std::lock_guard<std::mutex> lk(mu);
      E = &cache.emplace(key, std::move(ne)).first->second;
    }
    lam = E->lam;
    for (double& l : lam) l *= cx;
    if (fwd) *fwd = E->fwd;
    if (bwd) *bwd = E->bwd;
  }
  if (poisson && std::fabs(lam[0]) < 1e-10) {  // poisson.rs:80-83
    for (double& l : lam) l -= 1e-10;
  }
  std::vector<Band4> rows;
  rows.reserve(lam.size());
  for (double l0 : lam) {
    double l = l0 + alpha;
    Band4 f = band_combine(a1, c1, l);
    band_sweep(f);
    rows.push_back(f);
  }
  if (lam_out) *lam_out = lam;
  return rows;
}

bool build_solver(Arena& a, const SpaceDev& s, int kind, const double c[2], SolverDev& out, std::string* err) {
  try {
    out = SolverDev();
    out.kind = kind;
    out.m0 = s.spec0;
    out.m1 = s.spec1;
    const HostBasis* hb[2] = {&s.hb0, &s.hb1};
    for (int ax = 0; ax < 2; ax++) {
      const HostBasis& b = *hb[ax];
      if (b.bc() || b.kind == CHEB) throw std::runtime_error("solver spaces need composite or Fourier bases");
      out.has_pinv[ax] = !b.fourier();
      if (out.has_pinv[ax]) out.pinv[ax] = upload_pinv(a, b.n);
    }
    if (kind == SV_KIND_HHOLTZ_ADI) {
      for (int ax = 0; ax < 2; ax++) out.adi[ax] = upload_fdma(a, {adi_factor(*hb[ax], c[ax])});
      return true;
    }
    std::vector<double> fwd, bwd;
    std::vector<Band4> rows = hholtz_rows(s.hb0, s.hb1, c[0], c[1], kind == SV_KIND_HHOLTZ ? 1.0 : 0.0,
                                          kind == SV_KIND_POISSON, nullptr, &fwd, &bwd, err);
    out.rows = upload_fdma(a, rows);
    out.dense = !s.hb0.fourier();
    if (out.dense) {
      out.fwd = a.upload(fwd);
      out.bwd = a.upload(bwd);
    }
    return true;
  } catch (std::exception& e) {
    if (err) *err = e.what();
    return false;
  }
}

// ---------------------------------------------------------------- generic pass
enum PassOpCode {
  P_TO_ORTHO = 1, P_FROM_ORTHO, P_DIFF, P_FDIFF, P_DCT_FWD, P_DCT_BWD, P_R2C, P_C2R, P_SCALE, P_MATVEC, P_FDMA,
  P_DENSE, P_ADD
};
struct PassOp {
  int code;
  int arg;
};
struct PassDesc {
  const void* in;
  void* out;
  int in_cplx, out_cplx;
  int lanes, in_len;
  long long in_ls, in_es, out_ls, out_es;
  int nops;
  PassOp ops[6];
  BasisDev basis;
  ChebXformDev cx;
  FourierXformDev fx;
  PinvDev pinv;
  FdmaDev fdma;
  const double* dense;
  int dense_rows, dense_cols;
  double scale;
  int lmax, wl;
  const void* add;  // P_ADD: A[k] += add[lane*add_ls + k] (complex when in_cplx)
  long long add_ls;
};

namespace dev {
__global__ void __launch_bounds__(128) k_pass(const __grid_constant__ PassDesc d) {
  const int lane = blockIdx.x;
  const int tid = threadIdx.x, nth = blockDim.x;
  extern __shared__ double2 sm[];
  double2* A = sm;
  double2* B = A + d.lmax;
  double2* T = B + d.lmax;
  double2* WA = T + d.lmax;
  double2* WB = WA + d.wl;
  double* R = reinterpret_cast<double*>(WB + d.wl);
  int len = d.in_len;
  for (int k = tid; k < len; k += nth) {
    long long off = lane * d.in_ls + k * d.in_es;
    A[k] = d.in_cplx ? static_cast<const double2*>(d.in)[off] : c2(static_cast<const double*>(d.in)[off], 0.0);
  }
  __syncthreads();
  for (int o = 0; o < d.nops; o++) {
    const PassOp op = d.ops[o];
    switch (op.code) {
      case P_TO_ORTHO:
        to_ortho<double2>(d.basis, A, 0, B, 0, 1, tid, nth);
        len = d.basis.kind == 5 ? d.basis.m : d.basis.n;
        { double2* t = A; A = B; B = t; }
        break;
      case P_FROM_ORTHO:
        from_ortho<double2>(d.basis, A, 0, B, 0, 1, tid, nth);
        len = d.basis.m;
        { double2* t = A; A = B; B = t; }
        break;
      case P_DIFF:
        if (op.arg > 0) {
          cheb_diff<double2>(A, 0, B, 0, len, 1, op.arg, T, 0, tid, nth);
          double2* t = A; A = B; B = t;
        }
        break;
      case P_FDIFF:
        for (int k = tid; k < len; k += nth) {
          double2 v = A[k];
          for (int t = 0; t < op.arg; t++) v = mul_ik(v, (double)k);
          A[k] = v;
        }
        __syncthreads();
        break;
      case P_DCT_FWD:
      case P_DCT_BWD: {
        bool fwd = op.code == P_DCT_FWD;
        if (d.cx.use_fft) dct1_fft_c(d.cx, fwd, A, 0, B, 0, 1, WA, WB, d.wl, tid, nth);
        else dct1_dense<double2>(d.cx, fwd, A, 0, B, 0, 1, tid, nth);
        double2* t = A; A = B; B = t;
        break;
      }
      case P_R2C:
        for (int k = tid; k < len; k += nth) R[k] = A[k].x;
        __syncthreads();
        r2c(d.fx, R, 0, B, 0, 1, d.fx.n / 2 + 1, 1, WA, WB, d.wl, tid, nth);
        len = d.fx.n / 2 + 1;
        { double2* t = A; A = B; B = t; }
        break;
      case P_C2R:
        c2r(d.fx, A, 0, 1, R, 0, 1, WA, WB, d.wl, tid, nth);
        len = d.fx.n;
        for (int k = tid; k < len; k += nth) B[k] = c2(R[k], 0.0);
        __syncthreads();
        { double2* t = A; A = B; B = t; }
        break;
      case P_SCALE:
        for (int k = tid; k < len; k += nth) A[k] = A[k] * d.scale;
        __syncthreads();
        break;
      case P_MATVEC:
        matvec_pinv<double2>(d.pinv, A, 0, B, 0, 1, tid, nth);
        len = d.pinv.n - 2;
        { double2* t = A; A = B; B = t; }
        break;
      case P_FDMA:
        fdma_solve<double2>(d.fdma, A, 0, 1, lane, 0, tid, nth);
        break;
      case P_ADD:
        for (int k = tid; k < len; k += nth) {
          long long off = lane * d.add_ls + k;
          A[k] = A[k] + (d.in_cplx ? static_cast<const double2*>(d.add)[off] : c2(static_cast<const double*>(d.add)[off], 0.0));
        }
        __syncthreads();
        break;
      case P_DENSE:
        for (int r = tid; r < d.dense_rows; r += nth) {
          const double* row = d.dense + (size_t)r * d.dense_cols;
          double2 acc = c2(0.0, 0.0);
          for (int k = 0; k < d.dense_cols; k++) acc = fmas(acc, A[k], __ldg(row + k));
          B[r] = acc;
        }
        __syncthreads();
        len = d.dense_rows;
        { double2* t = A; A = B; B = t; }
        break;
      default:
        break;
    }
  }
  for (int k = tid; k < len; k += nth) {
    long long off = lane * d.out_ls + k * d.out_es;
    if (d.out_cplx) static_cast<double2*>(d.out)[off] = A[k];
    else static_cast<double*>(d.out)[off] = A[k].x;
  }
}

__global__ void k_axpby(double* y, const double* x, double a, double b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = a * y[i] + b * x[i];
}
__global__ void k_set(double* y, double v, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) y[i] = v;
}
__global__ void k_combine(int op, const double* a, const double* b, const double* c, double s0, double s1,
                          double* out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double r;
    switch (op) {
      case 0: r = ((a[i] + (b[i] * c[i]) / s0) * 2.0) * s1; break;  // Nuvol integrand
      case 1: r = sqrt(a[i] * a[i] + b[i] * b[i]) * s0; break;     // Re integrand
      case 2: r = 0.5 * (a[i] * a[i] + b[i] * b[i]); break;        // kinetic energy
      case 3: r = a[i] + b[i]; break;
      case 5: r = (a[i] * s0) * s1 + (b[i] * s0) * s1; break;     // (g_xx dt) ka + (g_yy dt) ka
      case 6: r = a[i] / s0; break;
      case 7: r = (a[i] * s0 + b[i]) / s1; break;                  // running mean (statistics.rs:142-144)
      default: r = a[i] * s0; break;
    }
    out[i] = r;
  }
}
// single-block deterministic reductions
__global__ void k_wsum(const double* v, int n0, int n1, const double* wx, const double* wy, double* out) {
  __shared__ double red[1024];
  double acc = 0.0;
  for (int j = threadIdx.x; j < n1; j += blockDim.x) {
    double cs = 0.0;
    for (int i = 0; i < n0; i++) cs += v[(size_t)i * n1 + j] * wx[i];
    acc += cs * wy[j];
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}
__global__ void k_colsum(const double* v, int n0, int n1, const double* wx, int j, double* out) {
  __shared__ double red[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n0; i += blockDim.x) acc += v[(size_t)i * n1 + j] * wx[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}
__global__ void k_sumsq(const double* v, size_t n, double* out) {
  __shared__ double red[1024];
  double acc = 0.0;
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) acc += v[i] * v[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}
}  // namespace dev

static size_t pass_smem(const PassDesc& d) {
  return (size_t)(3 * d.lmax + 2 * d.wl) * 16 + (size_t)d.lmax * 2 * 8 + 64;
}

static void run_pass(PassDesc& d, cudaStream_t st) {
  size_t sm = pass_smem(d);
  dev::k_pass<<<d.lanes, 128, sm, st>>>(d);
  cuda_check(cudaGetLastError(), "pass kernel launch");
}

static PassDesc base_desc(const SpaceDev& s);
static size_t space_pass_smem(const SpaceDev& s) { return pass_smem(base_desc(s)); }

static PassDesc base_desc(const SpaceDev& s) {
  PassDesc d;
  std::memset(&d, 0, sizeof d);
  int m0 = std::max(std::max(s.phys0, s.spec0), s.ortho0);
  int m1 = std::max(std::max(s.phys1, s.spec1), s.ortho1);
  d.lmax = std::max(m0, m1) + 2;
  int wl = 2;
  if (s.c1.use_fft) wl = std::max(wl, s.c1.L);
  if (!s.cplx && s.c0.use_fft) wl = std::max(wl, s.c0.L);
  if (s.cplx) wl = std::max(wl, s.f0.M);
  d.wl = wl;
  return d;
}

size_t tmp_elems(const SpaceDev& s) {
  size_t m0 = std::max(std::max(s.phys0, s.spec0), s.ortho0);
  size_t m1 = std::max(std::max(s.phys1, s.spec1), s.ortho1);
  return 2 * m0 * m1;
}

// axis-0 pass setup: lanes are columns (count `cols`), element stride `cols`
static void set_axis0(PassDesc& d, const void* in, int in_cplx, void* out, int out_cplx, int cols, int len) {
  d.in = in; d.out = out; d.in_cplx = in_cplx; d.out_cplx = out_cplx;
  d.lanes = cols; d.in_len = len;
  d.in_ls = 1; d.in_es = cols; d.out_ls = 1; d.out_es = cols;
}
static void set_axis1(PassDesc& d, const void* in, int in_cplx, void* out, int out_cplx, int rows, int in_cols,
                      int out_cols) {
  d.in = in; d.out = out; d.in_cplx = in_cplx; d.out_cplx = out_cplx;
  d.lanes = rows; d.in_len = in_cols;
  d.in_ls = in_cols; d.in_es = 1; d.out_ls = out_cols; d.out_es = 1;
}
static void add_op(PassDesc& d, int code, int arg = 0) { d.ops[d.nops++] = PassOp{code, arg}; }

void space_forward(const SpaceDev& s, const double* phys, void* spec, void* tmp, cudaStream_t st) {
  PassDesc d = base_desc(s);
  set_axis1(d, phys, 0, tmp, 0, s.phys0, s.phys1, s.spec1);
  d.cx = s.c1; d.basis = s.b1;
  add_op(d, P_DCT_FWD);
  if (s.hb1.composite()) add_op(d, P_FROM_ORTHO);
  run_pass(d, st);
  PassDesc e = base_desc(s);
  set_axis0(e, tmp, 0, spec, s.cplx, s.spec1, s.phys0);
  if (s.cplx) { e.fx = s.f0; add_op(e, P_R2C); }
  else {
    e.cx = s.c0; e.basis = s.b0;
    add_op(e, P_DCT_FWD);
    if (s.hb0.composite()) add_op(e, P_FROM_ORTHO);
  }
  run_pass(e, st);
}

void axis0_forward(const SpaceDev& s, const double* in, void* out, int cols, cudaStream_t st) {
  PassDesc e = base_desc(s);
  set_axis0(e, in, 0, out, s.cplx, cols, s.phys0);
  if (s.cplx) { e.fx = s.f0; add_op(e, P_R2C); }
  else {
    e.cx = s.c0; e.basis = s.b0;
    add_op(e, P_DCT_FWD);
    if (s.hb0.composite()) add_op(e, P_FROM_ORTHO);
  }
  run_pass(e, st);
}

void space_backward(const SpaceDev& s, const void* spec, double* phys, void* tmp, cudaStream_t st) {
  PassDesc d = base_desc(s);
  set_axis0(d, spec, s.cplx, tmp, 0, s.spec1, s.spec0);
  if (s.cplx) { d.fx = s.f0; add_op(d, P_C2R); }
  else {
    d.cx = s.c0; d.basis = s.b0;
    if (s.hb0.composite()) add_op(d, P_TO_ORTHO);
    add_op(d, P_DCT_BWD);
  }
  run_pass(d, st);
  PassDesc e = base_desc(s);
  set_axis1(e, tmp, 0, phys, 0, s.phys0, s.spec1, s.phys1);
  e.cx = s.c1; e.basis = s.b1;
  if (s.hb1.composite()) add_op(e, P_TO_ORTHO);
  add_op(e, P_DCT_BWD);
  run_pass(e, st);
}

// backward(gradient(f)) on the physical grid in two passes, the field read
// once per axis: x pass to_ortho, derivative, backward transform; y pass the
// same with the 1/scale^deriv factor (conv_term.rs:22-42 does the gradient,
// then Field2::backward of the ortho result).
void space_gradient_physical(const SpaceDev& s, const void* spec, double* phys, int d0, int d1, const double* scale,
                             void* tmp, cudaStream_t st) {
  PassDesc d = base_desc(s);
  set_axis0(d, spec, s.cplx, tmp, 0, s.spec1, s.spec0);
  if (s.cplx) {
    d.fx = s.f0;
    if (d0 > 0) add_op(d, P_FDIFF, d0);
    add_op(d, P_C2R);
  } else {
    d.cx = s.c0; d.basis = s.b0;
    if (s.hb0.composite()) add_op(d, P_TO_ORTHO);
    add_op(d, P_DIFF, d0);
    add_op(d, P_DCT_BWD);
  }
  run_pass(d, st);
  PassDesc e = base_desc(s);
  set_axis1(e, tmp, 0, phys, 0, s.phys0, s.spec1, s.phys1);
  e.cx = s.c1; e.basis = s.b1;
  if (s.hb1.composite()) add_op(e, P_TO_ORTHO);
  add_op(e, P_DIFF, d1);
  if (scale) {
    double s0 = 1.0, s1 = 1.0;
    for (int i = 0; i < d0; i++) s0 *= scale[0];
    for (int i = 0; i < d1; i++) s1 *= scale[1];
    e.scale = 1.0 / (s0 * s1);
    add_op(e, P_SCALE);
  }
  add_op(e, P_DCT_BWD);
  run_pass(e, st);
}

void space_backward_ortho(const SpaceDev& s, const void* ortho, double* phys, void* tmp, cudaStream_t st) {
  PassDesc d = base_desc(s);
  set_axis0(d, ortho, s.cplx, tmp, 0, s.ortho1, s.ortho0);
  if (s.cplx) { d.fx = s.f0; add_op(d, P_C2R); }
  else { d.cx = s.c0; add_op(d, P_DCT_BWD); }
  run_pass(d, st);
  PassDesc e = base_desc(s);
  set_axis1(e, tmp, 0, phys, 0, s.phys0, s.ortho1, s.phys1);
  e.cx = s.c1;
  add_op(e, P_DCT_BWD);
  run_pass(e, st);
}

void space_to_ortho(const SpaceDev& s, const void* spec, void* ortho, void* tmp, cudaStream_t st) {
  PassDesc d = base_desc(s);
  set_axis0(d, spec, s.cplx, tmp, s.cplx, s.spec1, s.spec0);
  d.basis = s.b0;
  add_op(d, P_TO_ORTHO);
  run_pass(d, st);
  PassDesc e = base_desc(s);
  set_axis1(e, tmp, s.cplx, ortho, s.cplx, s.ortho0, s.spec1, s.ortho1);
  e.basis = s.b1;
  add_op(e, P_TO_ORTHO);
  run_pass(e, st);
}

void space_from_ortho(const SpaceDev& s, const void* ortho, void* spec, void* tmp, cudaStream_t st) {
  PassDesc d = base_desc(s);
  set_axis0(d, ortho, s.cplx, tmp, s.cplx, s.ortho1, s.ortho0);
  d.basis = s.b0;
  add_op(d, P_FROM_ORTHO);
  run_pass(d, st);
  PassDesc e = base_desc(s);
  set_axis1(e, tmp, s.cplx, spec, s.cplx, s.spec0, s.ortho1, s.spec1);
  e.basis = s.b1;
  add_op(e, P_FROM_ORTHO);
  run_pass(e, st);
}

void space_gradient(const SpaceDev& s, const void* spec, void* ortho, int d0, int d1, const double* scale,
                    void* tmp, cudaStream_t st) {
  PassDesc d = base_desc(s);
  set_axis0(d, spec, s.cplx, tmp, s.cplx, s.spec1, s.spec0);
  d.basis = s.b0;
  add_op(d, P_TO_ORTHO);
  add_op(d, s.cplx ? P_FDIFF : P_DIFF, d0);
  run_pass(d, st);
  PassDesc e = base_desc(s);
  set_axis1(e, tmp, s.cplx, ortho, s.cplx, s.ortho0, s.spec1, s.ortho1);
  e.basis = s.b1;
  add_op(e, P_TO_ORTHO);
  add_op(e, P_DIFF, d1);
  if (scale) {
    double s0 = 1.0, s1 = 1.0;
    for (int i = 0; i < d0; i++) s0 *= scale[0];
    for (int i = 0; i < d1; i++) s1 *= scale[1];
    e.scale = 1.0 / (s0 * s1);
    add_op(e, P_SCALE);
  }
  run_pass(e, st);
}

void solver_solve(const SolverDev& sv, const SpaceDev& s, const void* in_ortho, void* out_spec, void* tmp,
                  cudaStream_t st) {
  int cx = s.cplx;
  size_t half = tmp_elems(s) / 2;
  void* t0 = tmp;
  void* t1 = static_cast<char*>(tmp) + half * 16;
  if (sv.kind == SV_KIND_HHOLTZ_ADI) {
    PassDesc d = base_desc(s);
    set_axis0(d, in_ortho, cx, t0, cx, s.ortho1, s.ortho0);
    if (sv.has_pinv[0]) { d.pinv = sv.pinv[0]; add_op(d, P_MATVEC); }
    d.fdma = sv.adi[0];
    add_op(d, P_FDMA);
    run_pass(d, st);
    PassDesc e = base_desc(s);
    set_axis1(e, t0, cx, out_spec, cx, s.spec0, s.ortho1, s.spec1);
    if (sv.has_pinv[1]) { e.pinv = sv.pinv[1]; add_op(e, P_MATVEC); }
    e.fdma = sv.adi[1];
    add_op(e, P_FDMA);
    run_pass(e, st);
    return;
  }
  // tensor solver: pinv_x and eigenbasis forward along x, pinv_y and the
  // per-row banded solve along y, eigenbasis backward along x
  PassDesc d = base_desc(s);
  set_axis0(d, in_ortho, cx, t0, cx, s.ortho1, s.ortho0);
  if (sv.has_pinv[0]) { d.pinv = sv.pinv[0]; add_op(d, P_MATVEC); }
  if (sv.dense) { d.dense = sv.fwd; d.dense_rows = sv.m0; d.dense_cols = sv.m0; add_op(d, P_DENSE); }
  run_pass(d, st);
  PassDesc e = base_desc(s);
  set_axis1(e, t0, cx, sv.dense ? t1 : out_spec, cx, s.spec0, s.ortho1, s.spec1);
  if (sv.has_pinv[1]) { e.pinv = sv.pinv[1]; add_op(e, P_MATVEC); }
  e.fdma = sv.rows;
  add_op(e, P_FDMA);
  run_pass(e, st);
  if (sv.dense) {
    PassDesc f = base_desc(s);
    set_axis0(f, t1, cx, out_spec, cx, s.spec1, s.spec0);
    f.dense = sv.bwd; f.dense_rows = sv.m0; f.dense_cols = sv.m0;
    add_op(f, P_DENSE);
    run_pass(f, st);
  }
}

// ---------------------------------------------------------------- Diffusion2D
// Diffusion2D::update (src/navier/diffusion.rs:186-207): rhs = to_ortho(vhat) + C,
// vhat = Hholtz.solve(rhs).  Operators acting on different axes commute, so
// the update runs as lane passes over the composite state:
//   X1 (columns): Sx, pinv_x, eigenbasis forward           vhat -> t0
//   Y  (rows):    Sy, pinv_y, + K (row i), row i banded solve  t0 -> t1
//   X2 (columns): eigenbasis backward                       t1 -> vhat
// with K = F pinv_x pinv_y C.  With a Fourier axis 0 (no x operator) only the
// Y pass runs, in place on vhat.
void diffusion_constant(const SolverDev& sv, const SpaceDev& s, const void* c_ortho, void* k_out, void* tmp,
                        cudaStream_t st) {
  const int cx = s.cplx;
  const bool xpass = sv.has_pinv[0] || sv.dense;
  if (xpass) {
    PassDesc d = base_desc(s);
    set_axis0(d, c_ortho, cx, tmp, cx, s.ortho1, s.ortho0);
    if (sv.has_pinv[0]) { d.pinv = sv.pinv[0]; add_op(d, P_MATVEC); }
    if (sv.dense) { d.dense = sv.fwd; d.dense_rows = sv.m0; d.dense_cols = sv.m0; add_op(d, P_DENSE); }
    run_pass(d, st);
  }
  PassDesc e = base_desc(s);
  set_axis1(e, xpass ? tmp : c_ortho, cx, k_out, cx, s.spec0, s.ortho1, s.spec1);
  if (sv.has_pinv[1]) { e.pinv = sv.pinv[1]; add_op(e, P_MATVEC); }
  run_pass(e, st);
}

void diffusion_step(const SolverDev& sv, const SpaceDev& s, void* vhat, const void* k, void* tmp, cudaStream_t st) {
  const int cx = s.cplx;
  const bool xpass = s.hb0.composite() || sv.has_pinv[0] || sv.dense;
  size_t half = tmp_elems(s) / 2;
  void* t0 = tmp;
  void* t1 = static_cast<char*>(tmp) + half * 16;
  if (xpass) {
    PassDesc d = base_desc(s);
    set_axis0(d, vhat, cx, t0, cx, s.spec1, s.spec0);
    d.basis = s.b0;
    if (s.hb0.composite()) add_op(d, P_TO_ORTHO);
    if (sv.has_pinv[0]) { d.pinv = sv.pinv[0]; add_op(d, P_MATVEC); }
    if (sv.dense) { d.dense = sv.fwd; d.dense_rows = sv.m0; d.dense_cols = sv.m0; add_op(d, P_DENSE); }
    run_pass(d, st);
  }
  PassDesc e = base_desc(s);
  set_axis1(e, xpass ? t0 : vhat, cx, sv.dense ? t1 : vhat, cx, s.spec0, s.spec1, s.spec1);
  e.basis = s.b1;
  if (s.hb1.composite()) add_op(e, P_TO_ORTHO);
  if (sv.has_pinv[1]) { e.pinv = sv.pinv[1]; add_op(e, P_MATVEC); }
  if (k) { e.add = k; e.add_ls = s.spec1; add_op(e, P_ADD); }
  e.fdma = sv.rows;
  add_op(e, P_FDMA);
  run_pass(e, st);
  if (sv.dense) {
    PassDesc f = base_desc(s);
    set_axis0(f, t1, cx, vhat, cx, s.spec1, s.spec0);
    f.dense = sv.bwd; f.dense_rows = sv.m0; f.dense_cols = sv.m0;
    add_op(f, P_DENSE);
    run_pass(f, st);
  }
}

static PassDesc lanes_desc(const LanesDev& L);

void build_lanes(Arena& a, LanesDev& L, int kind, int n) {
  if (kind != CHEB && kind != CD && kind != CN) throw std::runtime_error("lanes: Chebyshev-family bases only");
  L.hb = make_basis(kind, n);
  L.b = upload_basis(a, L.hb);
  L.cx = upload_cheb(a, n);
  L.has_solver = false;
  // the dense transform where the FFT form's work lanes do not fit (as for spaces)
  if (pass_smem(lanes_desc(L)) > smem_limit() && L.cx.use_fft) L.cx = upload_cheb(a, n, false);
  const size_t need = pass_smem(lanes_desc(L));
  if (need > smem_limit())
    throw SizeError("lanes of length " + std::to_string(n) + " need " + std::to_string(need) +
                    " bytes of shared memory per block; this device allows " + std::to_string(smem_limit()));
}

void lanes_set_hholtz(Arena& a, LanesDev& L, double c) {
  if (!L.hb.composite()) throw std::runtime_error("lanes: the Helmholtz solve needs a composite basis");
  L.pinv = upload_pinv(a, L.hb.n);
  L.adi = upload_fdma(a, {adi_factor(L.hb, c)});
  L.has_solver = true;
}

void lane_op_lengths(const LanesDev& L, int op, int* in_len, int* out_len) {
  const int n = L.hb.n, m = L.hb.m;
  switch (op) {
    case LOP_FORWARD: *in_len = n; *out_len = m; break;
    case LOP_BACKWARD: *in_len = m; *out_len = n; break;
    case LOP_TO_ORTHO: *in_len = m; *out_len = n; break;
    case LOP_FROM_ORTHO: *in_len = n; *out_len = m; break;
    case LOP_HHOLTZ: *in_len = n; *out_len = m; break;
    default: throw std::runtime_error("lanes: unknown operation");
  }
}

static PassDesc lanes_desc(const LanesDev& L) {
  PassDesc d;
  std::memset(&d, 0, sizeof d);
  d.lmax = L.hb.n + 2;
  d.wl = L.cx.use_fft ? std::max(2, L.cx.L) : 2;
  d.basis = L.b;
  d.cx = L.cx;
  return d;
}

void lanes_apply(const LanesDev& L, int op, const double* in, double* out, int lanes, cudaStream_t st) {
  int il, ol;
  lane_op_lengths(L, op, &il, &ol);
  PassDesc d = lanes_desc(L);
  set_axis1(d, in, 0, out, 0, lanes, il, ol);
  const bool comp = L.hb.composite();
  switch (op) {
    case LOP_FORWARD: add_op(d, P_DCT_FWD); if (comp) add_op(d, P_FROM_ORTHO); break;
    case LOP_BACKWARD: if (comp) add_op(d, P_TO_ORTHO); add_op(d, P_DCT_BWD); break;
    case LOP_TO_ORTHO: add_op(d, P_TO_ORTHO); break;
    case LOP_FROM_ORTHO: add_op(d, P_FROM_ORTHO); break;
    case LOP_HHOLTZ:
      if (!L.has_solver) throw std::runtime_error("lanes: Helmholtz coefficient not set");
      d.pinv = L.pinv; add_op(d, P_MATVEC);
      d.fdma = L.adi; add_op(d, P_FDMA);
      break;
  }
  run_pass(d, st);
}

void lanes_fdma(const LanesDev& L, double* x, int lanes, cudaStream_t st) {
  if (!L.has_solver) throw std::runtime_error("lanes: Helmholtz coefficient not set");
  PassDesc d = lanes_desc(L);
  set_axis1(d, x, 0, x, 0, lanes, L.hb.m, L.hb.m);
  d.fdma = L.adi;
  add_op(d, P_FDMA);
  run_pass(d, st);
}

void axpby(double* y, const double* x, double a, double b, size_t n, cudaStream_t st) {
  dev::k_axpby<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, st>>>(y, x, a, b, n);
  cuda_check(cudaGetLastError(), "axpby");
}
void set_value(double* y, double v, size_t n, cudaStream_t st) {
  dev::k_set<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, st>>>(y, v, n);
  cuda_check(cudaGetLastError(), "set_value");
}
void phys_combine(int op, const double* a, const double* b, const double* c, double s0, double s1, double* out,
                  size_t n, cudaStream_t st) {
  dev::k_combine<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, st>>>(op, a, b, c, s0, s1, out, n);
  cuda_check(cudaGetLastError(), "combine");
}
void weighted_sum(const double* v, int n0, int n1, const double* wx, const double* wy, double* out,
                  cudaStream_t st) {
  dev::k_wsum<<<1, 1024, 0, st>>>(v, n0, n1, wx, wy, out);
  cuda_check(cudaGetLastError(), "weighted_sum");
}
void weighted_col_sums(const double* v, int n0, int n1, const double* wx, int j, double* out, cudaStream_t st) {
  dev::k_colsum<<<1, 256, 0, st>>>(v, n0, n1, wx, j, out);
  cuda_check(cudaGetLastError(), "weighted_col_sums");
}
void sum_squares(const double* v, size_t n, double* out, cudaStream_t st) {
  dev::k_sumsq<<<1, 1024, 0, st>>>(v, n, out);
  cuda_check(cudaGetLastError(), "sum_squares");
}

size_t smem_limit() {
  static std::atomic<size_t> lim[64];
  const int d = current_device();
  size_t v = d < 64 ? lim[d].load() : 0;
  if (v == 0) {
    int a = 0;
    if (cudaDeviceGetAttribute(&a, cudaDevAttrMaxSharedMemoryPerBlockOptin, d) == cudaSuccess && a > 0) {
      v = (size_t)a;
    } else {
      cudaGetLastError();  // leave no error behind for the next launch check
      v = 200 * 1024;
    }
    if (d < 64) lim[d].store(v);
  }
  return v;
}

cudaError_t configure_prim_kernels() {
  static PerDeviceFlag done;
  if (done.test()) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(dev::k_pass, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_limit());
  if (e == cudaSuccess) done.set();
  return e;
}

}  // namespace rbc
