// case_access.h -- library-internal access to an RbcCase's device state, for
// solvers built on top of a Navier2D case (the adjoint solver).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "spectral_rbc.h"

namespace rbc {

struct CaseAccess {
  void* temp;   // spectral state (device)
  void* ux;
  void* uy;
  void* p0;
  void* p1;
  const void* bc_vhat;    // fieldbc spectral coefficients
  const double* bc_phys;  // fieldbc physical values (nx x ny)
  cudaStream_t stream;    // the case stream
  double nu, ka, scale[2];
};
CaseAccess case_access(RbcCase* c);
// Record `msg` for rbc_last_error and return `code`.
int set_last_error(int code, const std::string& msg);
// Enqueue the launches of one update() of a case stepped on its own on `st`
// (valid inside a stream capture).  The case time is not advanced.
void case_enqueue_step(RbcCase* c, cudaStream_t st);

}  // namespace rbc
