// per_device.h -- state kept once per CUDA device (kernel attributes, device
// limits): cudaFuncSetAttribute applies to the current device's copy of a
// kernel, so a process that drives several devices configures each.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

namespace rbc {

inline int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess) {
    cudaGetLastError();  // leave no error behind for the next launch check
    d = 0;
  }
  return d;
}

// A flag per device ordinal (ordinals >= 64 are never marked: configured again each time).
struct PerDeviceFlag {
  std::atomic<unsigned long long> bits{0};
  bool test() const {
    const int d = current_device();
    return d < 64 && ((bits.load() >> d) & 1ull) != 0;
  }
  void set() {
    const int d = current_device();
    if (d < 64) bits.fetch_or(1ull << d);
  }
};

}  // namespace rbc
