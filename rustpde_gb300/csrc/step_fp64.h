// step_fp64.h -- launch plan of the FP64 time step (see step_fp64.cu).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "rbc_dev.h"

namespace rbc {

enum StepKernel {
  K_Y1_C = 0, K_Y1_R, K_PER_X, K_PER_Y2,
  K_BOX_X1, K_BOX_Y2, K_BOX_X2, K_BOX_Y3, K_BOX_X3, K_BOX_Y4, K_BOX_X4, K_BOX_Y5,
  K_PER_Y2A, K_PER_Y2B,
  K_NUM_STEP_KERNELS
};

struct StepLaunch {
  int kernel;
  size_t smem;
  std::vector<int4> items;  // (case index, first lane, lane count, 0)
};

struct StepPlan {
  std::vector<StepLaunch> launches;
};

cudaError_t configure_step_kernels();
StepPlan build_step_plan(const CaseDev& c);
cudaError_t launch_step_kernel(int kernel, int nblocks, size_t smem, cudaStream_t s, const CaseDev* cases,
                               const int4* work);

namespace dev {
size_t smem_y1(const CaseDev& c, int nr, bool cplx);
size_t smem_per_x(const CaseDev& c);
size_t smem_per_y2(const CaseDev& c);
size_t smem_per_y2a(const CaseDev& c);
size_t smem_per_y2b(const CaseDev& c);
size_t smem_box_x1(const CaseDev& c);
size_t smem_box_y2(const CaseDev& c);
size_t smem_box_x2(const CaseDev& c);
size_t smem_box_y3(const CaseDev& c);
size_t smem_box_x3(const CaseDev& c);
size_t smem_box_y4(const CaseDev& c);
size_t smem_box_x4(const CaseDev& c);
size_t smem_box_y5(const CaseDev& c);
}  // namespace dev

}  // namespace rbc
