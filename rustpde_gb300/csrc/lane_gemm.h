// lane_gemm.h -- dense operators applied along lanes on the tensor cores.
//
// A "lane" is one 1-D line of a field along the axis being transformed: a row
// (contiguous) or a column (strided), real or one part (re / im) of a complex
// row.  A lane GEMM applies one dense real matrix W (N x K) to many lanes:
//     out[lane][n] = scale * sum_k W[n][k] * in[lane][k]
// which is the batched N x N matrix product form of the Chebyshev transforms,
// of stencil / derivative / transform compositions and of the box Poisson
// eigenbasis products.  The product runs on tcgen05 as 3xTF32
// (a_hi b_hi + a_hi b_lo + a_lo b_hi, FP32 accumulation in tensor memory).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace rbc {

enum LaneType { LT_F64 = 0, LT_F32 = 1 };

// How the lanes of one side (input or output) of a job map to memory.  Lane l
// of the job is (field f, row r, part p) with l = (f * rows + r) * parts + p;
// element k of that lane lives at
//     ptr[f] + r * lane_stride + p * part_stride + k * elem_stride   (scalars)
struct LaneSideDev {
  void* ptr[6];
  long long lane_stride;
  long long elem_stride;
  int nf, rows, parts, type;
  int part_stride;
  int len;        // valid elements: K for the input side, N for the output side
  int lane_fast;  // 1 when consecutive lanes are closer in memory than consecutive elements
  int pad_;
};

struct GemmJobDev {
  LaneSideDev in, out;
  const float* w;  // split operand packed by pack_gemm_w
  unsigned int* status;  // receives kStatusGemmTimeout
  const int* active;     // when set and 0, the job's tiles do nothing (serving gate)
  double scale;
  int K, N;
  int NT;       // output columns per tile (multiple of 16, <= 128)
  int kchunks;  // ceil(K / 32)
  int lanes;    // nf * rows * parts
  int ntiles;   // ceil(N / NT)
};

constexpr int kGemmLanes = 128;    // lanes per tile (tcgen05 M)
constexpr int kGemmThreads = 256;  // threads per CTA (warps 0-3 also read the accumulators)
constexpr int kGemmKC = 32;      // K elements per staged chunk

// Output tile width for N outputs, tiles of at most ntmax (64 or 128) outputs.
int gemm_tile_n(int N, int ntmax = 64);
// Split W (N x K row-major, FP64) into TF32 hi / lo parts laid out as the
// kernel stages them: for tile t and chunk c a block of 2 * NT * 32 floats
// (hi then lo), each in the K-major core-matrix order of the tcgen05 operand.
std::vector<float> pack_gemm_w(const std::vector<double>& W, int N, int K, int NT);
// Tiles (job, first lane, output tile, 0) of a job list.
void gemm_tiles(const std::vector<GemmJobDev>& jobs, std::vector<int4>& tiles);
size_t gemm_smem_bytes(int NT);
// the warp-specialised form's (NT <= 64): two input and two operator chunk buffers
size_t gemm_ws_smem_bytes(int NT);
cudaError_t configure_gemm_kernels();
// jobs and tiles are device arrays; max_nt = largest NT among the jobs.  ws:
// the warp-specialised form (producer, MMA and flush warps; max_nt <= 64).
cudaError_t launch_lane_gemm(const GemmJobDev* jobs, const int4* tiles, int ntiles_total, int max_nt,
                             cudaStream_t st, bool ws = false);

// Poll limit of the kernel's bounded completion waits on the current device
// (negative: the default, 2^22 polls).  A small limit makes the waits run out
// so that the time-out path (status bit, no stores, tensor memory freed) can
// be tested; it affects every lane GEMM launched on the device afterwards.
cudaError_t set_gemm_wait_limit(long long polls);

// One job passed by value (no tables): lanes tiled in order.
cudaError_t launch_lane_gemm_one(const GemmJobDev& job, cudaStream_t st);
// ntmax: the widest output tile (the operator w must be packed for gemm_tile_n(N, ntmax))
GemmJobDev make_gemm_job(const LaneSideDev& in, const LaneSideDev& out, const float* w, int K, int N, double scale,
                         unsigned int* status, int ntmax = 64);
// Lanes that are rows of row-major (rows x row_len) arrays, real or complex
// interleaved (each complex row is two lanes, re then im).
LaneSideDev lane_rows(void* const* ptrs, int nf, int rows, int len, int row_len, int type, bool complex_);
// Lanes that are columns col0 .. col0+cols-1 of real row-major (. x row_len) arrays.
LaneSideDev lane_cols(void* const* ptrs, int nf, int cols, int len, int row_len, int type, int col0);

// Status bit set by the kernel when a tensor-core completion wait ran out.
constexpr unsigned int kStatusGemmTimeout = 2u;

}  // namespace rbc
