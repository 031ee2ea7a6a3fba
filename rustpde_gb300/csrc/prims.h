// prims.h -- generic 2-D funspace / solver operations on device buffers.
//
// These serve the drop-in primitives (Field2 forward/backward/to_ortho/
// from_ortho/gradient, Hholtz/HholtzAdi/Poisson solves), the set-up of each
// case (boundary field, initial conditions) and the diagnostics.  Each 2-D
// operation is a sequence of single-axis "passes"; a pass applies a short
// chain of lane operations to every lane (one CTA per lane).
#pragma once
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "host_ops.h"
#include "rbc_dev.h"

namespace rbc {

// Owner of device allocations (freed on destruction).  By default blocks come
// from cudaMalloc (whose free waits for the device).  A stream-ordered arena
// takes them from the device's memory pool (cudaMallocAsync / cudaFreeAsync on
// a library-owned stream): allocating and freeing never waits for other
// streams, so a serving loop can build and retire cases while steps run.  Its
// owner must make sure no work still uses the memory when it is destroyed.
class Arena {
 public:
  Arena() = default;
  Arena(const Arena&) = delete;
  Arena& operator=(const Arena&) = delete;
  ~Arena();
  void set_stream_ordered(bool on) { ordered_ = on; }
  void* alloc(size_t bytes);  // zero-initialised; throws std::runtime_error on failure
  template <class T> T* upload(const std::vector<T>& v) {
    if (v.empty()) return nullptr;
    T* p = static_cast<T*>(alloc(v.size() * sizeof(T)));
    copy_h2d(p, v.data(), v.size() * sizeof(T));
    return p;
  }
  size_t bytes() const { return bytes_; }

 private:
  void copy_h2d(void* d, const void* h, size_t n);
  std::vector<void*> ptrs_;
  size_t bytes_ = 0;
  bool ordered_ = false;
};

void cuda_check(cudaError_t e, const char* what);  // throws std::runtime_error

// A size the kernels cannot run: a lane or a case whose shared-memory working
// set per block exceeds what the device allows (the C ABI reports it as
// RBC_ERR_INVALID).
struct SizeError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
// Dynamic shared memory a block may use on this device (the opt-in maximum,
// which the library's kernels are configured for), bytes.
size_t smem_limit();

// Device tables of one basis along one axis.
BasisDev upload_basis(Arena& a, const HostBasis& b);
// allow_fft = false: the dense form even where n - 1 is a power of two
ChebXformDev upload_cheb(Arena& a, int n, bool allow_fft = true);
FourierXformDev upload_fourier(Arena& a, int n);
PinvDev upload_pinv(Arena& a, int n);
FdmaDev upload_fdma(Arena& a, const std::vector<Band4>& rows);  // swept factors, one per row

// A 2-D space of two bases (funspace/src/space2.rs).
struct SpaceDev {
  HostBasis hb0, hb1;
  BasisDev b0, b1;
  ChebXformDev c0, c1;
  FourierXformDev f0;
  bool cplx = false;  // spectral data complex (Fourier along axis 0)
  int phys0 = 0, phys1 = 0, spec0 = 0, spec1 = 0, ortho0 = 0, ortho1 = 0;
};
void build_space(Arena& a, SpaceDev& s, int kind0, int n0, int kind1, int n1);

// Solvers (src/solver/{hholtz,hholtz_adi,poisson}.rs) on a space.
enum SolverKindDev { SV_KIND_HHOLTZ = 0, SV_KIND_HHOLTZ_ADI = 1, SV_KIND_POISSON = 2 };
struct SolverDev {
  int kind = SV_KIND_HHOLTZ_ADI;
  bool has_pinv[2] = {false, false};
  PinvDev pinv[2];
  FdmaDev adi[2];      // HholtzAdi
  FdmaDev rows;        // tensor solvers: factors per row of axis 0
  bool dense = false;  // eigenbasis products along axis 0
  const double* fwd = nullptr;
  const double* bwd = nullptr;
  int m0 = 0, m1 = 0;  // spectral sizes
};
// c: the two coefficients of the reference constructors.  Returns false with
// a message for unsupported combinations.
bool build_solver(Arena& a, const SpaceDev& s, int kind, const double c[2], SolverDev& out, std::string* err);

// Host-side factor computation shared by the case set-up (navier fields).
std::vector<Band4> hholtz_rows(const HostBasis& bx, const HostBasis& by, double cx, double cy, double alpha,
                               bool poisson, std::vector<double>* lam_out, std::vector<double>* fwd,
                               std::vector<double>* bwd, std::string* err);
Band4 adi_factor(const HostBasis& b, double c);

// 2-D operations (enqueued on `st`; `tmp` must hold max(phys0,spec0,ortho0) x
// max(phys1,spec1,ortho1) complex values).
void space_forward(const SpaceDev& s, const double* phys, void* spec, void* tmp, cudaStream_t st);
void space_backward(const SpaceDev& s, const void* spec, double* phys, void* tmp, cudaStream_t st);
// forward transform along axis 0 only of a (phys0 x cols) real array (Transform::forward_inplace, axis 0)
void axis0_forward(const SpaceDev& s, const double* in, void* out, int cols, cudaStream_t st);
void space_to_ortho(const SpaceDev& s, const void* spec, void* ortho, void* tmp, cudaStream_t st);
void space_from_ortho(const SpaceDev& s, const void* ortho, void* spec, void* tmp, cudaStream_t st);
void space_gradient(const SpaceDev& s, const void* spec, void* ortho, int d0, int d1, const double* scale,
                    void* tmp, cudaStream_t st);
// backward(gradient(spec)) onto the physical grid (two passes)
void space_gradient_physical(const SpaceDev& s, const void* spec, double* phys, int d0, int d1, const double* scale,
                             void* tmp, cudaStream_t st);
// backward transform of an ortho-sized array (the `field` space of Navier2D)
void space_backward_ortho(const SpaceDev& s, const void* ortho, double* phys, void* tmp, cudaStream_t st);
void solver_solve(const SolverDev& sv, const SpaceDev& s, const void* in_ortho, void* out_spec, void* tmp,
                  cudaStream_t st);
size_t tmp_elems(const SpaceDev& s);
// Diffusion2D (src/navier/diffusion.rs): K = F pinv_x pinv_y C for the constant
// ortho-space term C of the right-hand side (spec0 x spec1), and one update of
// the composite state vhat in place (k may be null: C = 0).  Tensor (Hholtz)
// solvers only.
void diffusion_constant(const SolverDev& sv, const SpaceDev& s, const void* c_ortho, void* k_out, void* tmp,
                        cudaStream_t st);
void diffusion_step(const SolverDev& sv, const SpaceDev& s, void* vhat, const void* k, void* tmp, cudaStream_t st);

// Batched 1-D operations (FP64) on `lanes` contiguous lanes of one
// Chebyshev-family basis: forward, backward, to_ortho, from_ortho and the 1-D
// HholtzAdi solve (hholtz_adi.rs:92-131 along one axis).
enum LaneOp { LOP_FORWARD = 0, LOP_BACKWARD = 1, LOP_TO_ORTHO = 2, LOP_FROM_ORTHO = 3, LOP_HHOLTZ = 4 };
struct LanesDev {
  HostBasis hb;
  BasisDev b;
  ChebXformDev cx;
  PinvDev pinv;
  FdmaDev adi;
  bool has_solver = false;
};
void build_lanes(Arena& a, LanesDev& L, int kind, int n);
void lanes_set_hholtz(Arena& a, LanesDev& L, double c);
// input / output lengths of an operation
void lane_op_lengths(const LanesDev& L, int op, int* in_len, int* out_len);
void lanes_apply(const LanesDev& L, int op, const double* in, double* out, int lanes, cudaStream_t st);
// the banded part of the HholtzAdi solve alone: x (m per lane) solved in place
void lanes_fdma(const LanesDev& L, double* x, int lanes, cudaStream_t st);

// Elementwise helpers on device arrays of n doubles
void axpby(double* y, const double* x, double a, double b, size_t n, cudaStream_t st);  // y = a*y + b*x
void set_value(double* y, double v, size_t n, cudaStream_t st);
// weights for volume averages (average.rs): result = sum_ij v_ij wx_i wy_j
void weighted_sum(const double* v, int n0, int n1, const double* wx, const double* wy, double* out,
                  cudaStream_t st);
void weighted_col_sums(const double* v, int n0, int n1, const double* wx, int j, double* out, cudaStream_t st);
void sum_squares(const double* v, size_t n, double* out, cudaStream_t st);
void phys_combine(int op, const double* a, const double* b, const double* c, double s0, double s1, double* out,
                  size_t n, cudaStream_t st);

cudaError_t configure_prim_kernels();

}  // namespace rbc
