// step_fp64.h -- launch plan of the FP64 time step (see step_fp64.cu).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "lane_gemm.h"
#include "rbc_dev.h"

namespace rbc {

enum StepKernel {
  K_Y1_C = 0, K_Y1_R, K_PER_X, K_PER_Y2,
  K_BOX_X1, K_BOX_Y2, K_BOX_X2, K_BOX_Y3, K_BOX_X3, K_BOX_Y4, K_BOX_X4, K_BOX_Y5,
  K_PER_Y2A, K_PER_Y2B,
  // mixed-precision form
  K_PER_Y2_PRE, K_PER_X_MIXED, K_BOX_PROD_MIXED, K_BOX_Y2_PRE, K_BOX_X3_MIX, K_BOX_X4_MIX, K_BOX_GPX,
  // one thread per lane (batched mixed-precision form, step_lanes.cu)
  K_LP_BOX_GPX, K_LP_BOX_X2, K_LP_BOX_X3, K_LP_BOX_X4, K_LP_BOX_Y2, K_LP_BOX_Y3, K_LP_BOX_Y4, K_LP_BOX_Y5,
  K_LP_PER_Y2,
  // the same CTA-per-lane kernels launched with 128 threads (more CTAs per SM)
  K_PER_Y2_PRE_T128, K_BOX_Y2_PRE_T128, K_BOX_X3_MIX_T128, K_BOX_Y5_T128,
  // periodic Y2 as three one-thread-per-sub-lane launches (right-hand sides and
  // Helmholtz solves; divergence and Poisson; projection and updates)
  K_LP_PER_Y2A, K_LP_PER_Y2B, K_LP_PER_Y2C,
  // FP32 copy of the state rows for the y GEMM (mixed form)
  K_STATE_F32,
  // the periodic FP32 x pass launched with 128 threads
  K_PER_X_MIXED_T128,
  // the three periodic Y2 launches as one (a CTA barrier between the phases)
  K_LP_PER_Y2F,
  // box Y4 of the mixed form (FP32 output for the eigenbasis GEMM)
  K_BOX_Y4_MIX,
  K_NUM_STEP_KERNELS,
  K_GEMM = 100  // tensor-core lane GEMM (jobs instead of work items)
};

struct StepLaunch {
  int kernel;
  int gemm_ws = 0;  // K_GEMM: 1 for the warp-specialised form
  int pass = -1;  // launches of one pass share the id (the autotuner swaps whole passes)
  size_t smem;
  std::vector<int4> items;       // (case index, first lane, lane count, 0)
  std::vector<GemmJobDev> jobs;  // K_GEMM only
};

struct StepPlan {
  std::vector<StepLaunch> launches;
};

cudaError_t configure_step_kernels();
StepPlan build_step_plan(const CaseDev& c);
// largest dynamic shared memory of a launch of the mixed-precision plan (and its kernel)
size_t mixed_plan_smem(const CaseDev& c, int* kernel);

// Operators of the mixed-precision step (packed tensor-core operands, device).
struct MixedOps {
  const float* y1 = nullptr;  // [B S ; B D S] along y: (2 ny) x (ny - 2)
  const float* y2 = nullptr;  // forward Chebyshev along y, rows < ky: ky x ny
  // box only, along x (aspect ratio folded into the derivative rows)
  const float* xa = nullptr;  // [B S_u ; B D S_u / s] : (2 nx) x (nx - 2)
  const float* xb = nullptr;  // B S_u : nx x (nx - 2)
  const float* xc = nullptr;  // B D S_t / s : nx x (nx - 2)
  const float* xd = nullptr;  // B S_t : nx x (nx - 2)
  const float* x2 = nullptr;  // forward Chebyshev along x, rows < kx: kx x nx
  const float* pf = nullptr;  // Poisson eigenbasis forward: (nx - 2) x (nx - 2)
  const float* pb = nullptr;  // Poisson eigenbasis backward: (nx - 2) x (nx - 2)
  int ntmax = 64;  // the widest GEMM output tile these operators are packed for (64 or 128)
  int ws = 0;      // 1: the GEMMs in the warp-specialised form (ntmax 64)
};
// variant 0: a CTA per lane; 1: 128-thread CTAs where that form exists, else
// one thread per lane; 2: one thread per (field, parity) sub-lane where that
// form exists, else 128-thread CTAs; 3: as 2 with the periodic Y2 launches
// fused.  The GEMM tiles follow ops.ntmax.
StepPlan build_mixed_plan(const CaseDev& c, const MixedOps& ops, int variant);
int lane_kernel_subs(int kernel);
bool lane_kernel_rows(int kernel);
cudaError_t launch_lane_kernel(int kernel, int nblocks, cudaStream_t s, const CaseDev* cases, const int4* work);
// one-thread-per-lane kernels: 64 threads per CTA, i.e. 64 column lanes or 32
// row lanes (two parity threads each) per work item; small items, sorted by
// cost (item.w = lanes x lane length) in merged plans, keep the SMs evenly busy
constexpr int kLaneBlock = 64;
inline int lane_item_lanes(int kernel) { return lane_kernel_rows(kernel) ? kLaneBlock / 2 : kLaneBlock; }
const char* step_kernel_name(int kernel);
// serving gate of the cases members[0..n) of `cases` (see CaseDev::gate)
cudaError_t launch_gate(const CaseDev* cases, const int* members, int n, cudaStream_t s);
// algorithmic HBM bytes of one launch (cases: host copies indexed by item case)
double launch_algorithmic_bytes(const StepLaunch& L, const CaseDev* cases);
cudaError_t configure_mixed_kernels();
cudaError_t launch_mixed_kernel(int kernel, int nblocks, size_t smem, cudaStream_t s, const CaseDev* cases,
                                const int4* work);
cudaError_t launch_step_kernel(int kernel, int nblocks, size_t smem, cudaStream_t s, const CaseDev* cases,
                               const int4* work);

namespace dev {
size_t smem_y1(const CaseDev& c, int nr, bool cplx);
size_t smem_per_x(const CaseDev& c);
size_t smem_per_y2(const CaseDev& c);
size_t smem_per_y2_pre(const CaseDev& c);
size_t smem_per_y2a(const CaseDev& c);
size_t smem_per_y2b(const CaseDev& c);
size_t smem_per_x_mixed(const CaseDev& c);
size_t smem_box_x1(const CaseDev& c);
size_t smem_box_gpx(const CaseDev& c);
size_t smem_box_y2(const CaseDev& c);
size_t smem_box_x2(const CaseDev& c);
size_t smem_box_y3(const CaseDev& c);
size_t smem_box_x3(const CaseDev& c);
size_t smem_box_y4(const CaseDev& c);
size_t smem_box_x4(const CaseDev& c);
size_t smem_box_y5(const CaseDev& c);
}  // namespace dev

}  // namespace rbc
