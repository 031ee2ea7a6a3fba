// lane_gemm.cu -- tcgen05 3xTF32 lane GEMM (see lane_gemm.h).
//
// One CTA (8 warps) computes a tile of 128 lanes x NT outputs of one job:
//   * the threads stage a 128 x 32 chunk of the input lanes into shared memory,
//     converting each value v to TF32 hi = rna(v) and lo = rna(v - hi), written
//     straight into the K-major core-matrix layout the tensor core reads
//     (8 rows x 16 bytes per core matrix, no swizzle);
//   * the matching chunk of the pre-split operator W is copied as-is;
//   * one thread issues 4 k-steps x 3 tcgen05.mma (lo*hi, hi*lo, hi*hi) and
//     commits to an mbarrier.  The hi*hi products of each chunk go to a fresh
//     partial accumulator in tensor memory (two, used alternately); while the
//     next chunk's MMAs run, the threads add the finished partial into an FP32
//     running total with round-to-nearest.  The tensor core's accumulation
//     truncates, so summing the whole K range in one accumulator biased every
//     output by about (K/8) ulp; per-chunk partials keep that to 4 ulp of a
//     partial.  The small lo*hi + hi*lo corrections accumulate over all of K
//     in a third accumulator;
//   * after the last chunk each warp reads its 32 lanes of total + corrections
//     back with tcgen05.ld, stages them through shared memory and stores them
//     coalesced.
// Every wait is bounded: on time-out the kernel sets kStatusGemmTimeout, skips
// the stores, drains its MMA in flight (again bounded), frees its tensor memory
// and returns.
#include "lane_gemm.h"
#include "per_device.h"

#include <algorithm>
#include <cstring>
#include <type_traits>

namespace rbc {
namespace dev {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor, no swizzle: start address, leading
// (K-direction) and stride (M/N-direction) byte offsets between core matrices.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of this architecture
  return d;
}

// byte offset of element (row r, k) of an R-row, 32-wide K-major chunk
__device__ __forceinline__ int cm_off(int r, int k, int R) {
  return ((k >> 2) * (R >> 3) + (r >> 3)) * 128 + (r & 7) * 16 + (k & 3) * 4;
}

// Round to TF32 (10 mantissa bits), to nearest with ties away from zero:
// add half a TF32 ulp to the magnitude bits and clear the 13 low bits.  A
// carry into the exponent is the correct rounding up to the next binade (or
// to infinity).  For finite values this is the rounding of cvt.rna.tf32.f32,
// in two integer operations.
__device__ __forceinline__ float tf32_rna(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ const char* lane_addr(const LaneSideDev& s, int l) {
  const int per_f = s.rows * s.parts;
  const int f = l / per_f;
  const int rem = l - f * per_f;
  const int r = rem / s.parts;
  const int p = rem - r * s.parts;
  const long long es = s.type == LT_F64 ? 8 : 4;
  return static_cast<const char*>(s.ptr[f]) + ((long long)r * s.lane_stride + (long long)p * s.part_stride) * es;
}

__device__ __forceinline__ void mbar_init(uint64_t* m, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count));
}
__device__ __forceinline__ bool mbar_try(uint64_t* m, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(m)), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

// 32 columns of a warp's 32 tensor-memory lanes; the caller waits (tcgen05.wait::ld)
__device__ __forceinline__ void tmem_ld32_nowait(uint32_t addr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(addr));
}

// tensor-memory columns of a tile: a power of two holding the two chunk
// partials, the corrections and the running total (NT each), with the last
// region padded to whole 32-column epilogue loads
__host__ __device__ inline uint32_t gemm_tmem_cols(int NT) {
  const uint32_t need = 3u * (uint32_t)NT + (((uint32_t)NT + 31u) & ~31u);
  uint32_t c = 32;
  while (c < need) c <<= 1;
  return c;
}

__device__ __forceinline__ void tmem_st8(uint32_t addr, const float (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(addr),
               "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
               "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
               "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
               : "memory");
}

__device__ __forceinline__ void tmem_ld8_nowait(uint32_t addr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(addr));
}

// running total += chunk partial (or = partial for the first chunk), all 8
// warps: warp w covers tensor-memory lanes 32 (w % 4) .. + 31 and every other
// 8-column block (from block w / 4), up to 8 blocks (NT <= 128), in rounds of
// two blocks: each round issues its loads before one wait (all blocks at once
// needed registers that spilled).
__device__ __forceinline__ void tmem_accumulate(uint32_t tmem, uint32_t part, uint32_t total, int NT, bool first,
                                                int warp) {
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
  const int cb0 = (warp >> 2) * 8;
#pragma unroll
  for (int h = 0; h < 4; h++) {
    if (32 * h >= NT) break;  // uniform across the CTA
    uint32_t p[2][8], t[2][8];
#pragma unroll
    for (int b = 0; b < 2; b++) {
      const int cb = cb0 + 16 * (2 * h + b);
      if (cb < NT) {
        tmem_ld8_nowait(tmem + lane_base + part + (uint32_t)cb, p[b]);
        if (!first) tmem_ld8_nowait(tmem + lane_base + total + (uint32_t)cb, t[b]);
      }
    }
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int b = 0; b < 2; b++) {
      const int cb = cb0 + 16 * (2 * h + b);
      if (cb < NT) {
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; j++)
          v[j] = first ? __uint_as_float(p[b][j]) : __fadd_rn(__uint_as_float(t[b][j]), __uint_as_float(p[b][j]));
        tmem_st8(tmem + lane_base + total + (uint32_t)cb, v);
      }
    }
  }
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

constexpr long long kWaitLimit = 1LL << 22;  // try_wait polls before a completion wait is declared lost
// The poll limit of the completion waits on this device (kWaitLimit unless a
// test lowers it through set_gemm_wait_limit to make the time-out path run).
// After a time-out the kernel still drains its MMA in flight with kWaitLimit
// polls before it frees tensor memory.
__device__ long long g_gemm_wait_limit = kWaitLimit;

__device__ __forceinline__ void cp_async16(uint32_t saddr, const void* g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// bounded wait for completion phase `parity` of the MMA barrier; true when it
// completed.  Warp 0 polls the barrier and the other warps wait at
// __syncthreads (256 polling threads took the issue slots of the SM's other
// CTA); the callers' tcgen05.fence::after_thread_sync orders every thread's
// later tensor-memory and shared-memory accesses after the completion.
__device__ __forceinline__ bool mma_wait(uint64_t* mbar, uint32_t parity, long long limit) {
  int done = 1;
  if (threadIdx.x < 32) {
    bool d = false;
    for (long long i = 0; i < limit && !d; i++) d = mbar_try(mbar, parity);
    done = d ? 1 : 0;
  }
  return __syncthreads_and(done) != 0;
}

// Input chunk of a tile held in registers between its global loads and its
// conversion: item (lane l, quad kq) -> 4 consecutive k of one lane.  NTHR
// threads stage a chunk (the whole CTA, or the producer warps of the
// warp-specialised form), 1024 / NTHR (lane, 4-k quad) items each.
template <class T, int NTHR = kGemmThreads>
struct AChunk {
  T v[1024 / NTHR][4];
};

// A thread's items are the same in every chunk of a tile: item it of thread
// tid is q = tid + NTHR it, lane l and quad kq as below.  With lanes fast in
// memory (columns) a thread keeps one lane and steps kq by NTHR / 128; with
// rows it keeps kq and steps the lane by NTHR / 8.  The lane addresses
// (element 4 kq of each item's lane) are formed once per tile.
template <class T, int NTHR = kGemmThreads>
struct ATile {
  const T* src[1024 / NTHR];  // nullptr: lane past the job's end (zeros)
  int es;               // element stride of the lanes (a row length at most)
  int soff0, sstep;     // shared-memory byte offset of item 0, step per item
  bool vec;             // unit element stride and every item 16-byte aligned: vector loads
};

__device__ __forceinline__ void item_lane_quad(int q, bool lane_fast, int& l, int& kq) {
  const int llo = q & 7, r = q >> 3;
  l = lane_fast ? (r & 15) * 8 + llo : (r >> 3) * 8 + llo;
  kq = lane_fast ? r >> 4 : r & 7;
}

template <class T, int NTHR = kGemmThreads>
__device__ __forceinline__ void a_setup(ATile<T, NTHR>& t, const GemmJobDev& J, const char* const* ib, int tid) {
  constexpr int kItems = 1024 / NTHR;
  const bool lf = J.in.lane_fast != 0;
  t.es = (int)J.in.elem_stride;
#pragma unroll
  for (int it = 0; it < kItems; it++) {
    int l, kq;
    item_lane_quad(tid + NTHR * it, lf, l, kq);
    const T* b = reinterpret_cast<const T*>(ib[l]);
    t.src[it] = b != nullptr ? b + (long long)(kq * 4) * t.es : nullptr;
    if (it == 0) t.soff0 = cm_off(l, kq * 4, kGemmLanes);
  }
  // item it+1 is NTHR / 128 quads further (lanes fast) or NTHR / 8 lanes further (rows)
  t.sstep = lf ? (NTHR / 128) * (kGemmLanes / 8) * 128 : (NTHR / 64) * 128;
  // chunk starts are 32 elements apart, so an aligned item stays aligned
  t.vec = t.es == 1;
#pragma unroll
  for (int it = 0; it < kItems; it++)
    if (t.src[it] != nullptr && (reinterpret_cast<uintptr_t>(t.src[it]) & 15u) != 0) t.vec = false;
}

// 4 consecutive elements from a 16-byte aligned address
__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
  const float4 x = __ldg(reinterpret_cast<const float4*>(p));
  v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&v)[4]) {
  const double2 x = __ldg(reinterpret_cast<const double2*>(p));
  const double2 y = __ldg(reinterpret_cast<const double2*>(p) + 1);
  v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
}

// loads of chunk k0 .. k0+31; only the job's last chunk checks k < K
template <class T, int NTHR = kGemmThreads>
__device__ __forceinline__ void a_load(AChunk<T, NTHR>& a, const ATile<T, NTHR>& t, int k0, int K, bool lane_fast,
                                       int tid) {
  constexpr int kItems = 1024 / NTHR;
  const int o = k0 * t.es;
  if (k0 + kGemmKC <= K) {
    if (t.vec) {
#pragma unroll
      for (int it = 0; it < kItems; it++) {
        const T* p = t.src[it];
        if (p != nullptr) {
          ld4(p + o, a.v[it]);
        } else {
#pragma unroll
          for (int e = 0; e < 4; e++) a.v[it][e] = T(0);
        }
      }
    } else if (t.es == 1) {
#pragma unroll
      for (int it = 0; it < kItems; it++) {
        const T* p = t.src[it] != nullptr ? t.src[it] + o : nullptr;
#pragma unroll
        for (int e = 0; e < 4; e++) a.v[it][e] = p != nullptr ? __ldg(p + e) : T(0);
      }
    } else {
#pragma unroll
      for (int it = 0; it < kItems; it++) {
        const T* p = t.src[it];
#pragma unroll
        for (int e = 0; e < 4; e++) a.v[it][e] = p != nullptr ? __ldg(p + o + e * t.es) : T(0);
      }
    }
  } else {
#pragma unroll
    for (int it = 0; it < kItems; it++) {
      int l, kq;
      item_lane_quad(tid + NTHR * it, lane_fast, l, kq);
      const T* p = t.src[it];
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int k = k0 + kq * 4 + e;
        a.v[it][e] = (p != nullptr && k < K) ? __ldg(p + o + e * t.es) : T(0);
      }
    }
  }
}

template <class T, int NTHR = kGemmThreads>
__device__ __forceinline__ void a_store(const AChunk<T, NTHR>& a, const ATile<T, NTHR>& t, unsigned char* Ahi,
                                        unsigned char* Alo) {
  constexpr int kItems = 1024 / NTHR;
#pragma unroll
  for (int it = 0; it < kItems; it++) {
    float4 hi, lo;
    float x;
    // lo is rounded to TF32 here: left to the tensor core it would be
    // truncated, a bias that accumulates along K
    x = (float)a.v[it][0]; hi.x = tf32_rna(x); lo.x = tf32_rna(x - hi.x);
    x = (float)a.v[it][1]; hi.y = tf32_rna(x); lo.y = tf32_rna(x - hi.y);
    x = (float)a.v[it][2]; hi.z = tf32_rna(x); lo.z = tf32_rna(x - hi.z);
    x = (float)a.v[it][3]; hi.w = tf32_rna(x); lo.w = tf32_rna(x - hi.w);
    const int off = t.soff0 + it * t.sstep;
    *reinterpret_cast<float4*>(Ahi + off) = hi;
    *reinterpret_cast<float4*>(Alo + off) = lo;
  }
}

// issue the asynchronous copy of operator chunk c (hi block then lo block),
// nthr threads
__device__ __forceinline__ void w_issue(const float* wsrc, int c, int NT, unsigned char* wbuf, int tid,
                                        int nthr = kGemmThreads) {
  const char* g = reinterpret_cast<const char*>(wsrc + (size_t)c * 2 * NT * kGemmKC);
  const uint32_t sb = smem_u32(wbuf);
  for (int i = tid; i < NT * 16; i += nthr) cp_async16(sb + i * 16, g + (size_t)i * 16);
}

// Output of a tile: total + corrections read back from tensor memory (warps
// 0-3, 32 columns at a time), staged through shared memory, stored coalesced.
// Every thread of the CTA takes part (two CTA barriers per 32 columns).
__device__ __forceinline__ void gemm_epilogue(const GemmJobDev& J, uint32_t tmem, uint32_t total, uint32_t corr,
                                              int NT, int tile_n, char* const* ob, float* stage, int tid, int warp,
                                              int wl) {
  // output mapping of staged element q = tid + 256 it -> (lane l, column n):
  // 0: lanes fast in memory (columns); 1: real rows; 2: complex rows (re, im
  // lanes of one row interleaved)
  const int omode = J.out.lane_fast ? 0 : (J.out.parts == 2 ? 2 : 1);
  const long long oes = J.out.elem_stride;
  const int otype = J.out.type;
  const double scale = J.scale;
  const int nbase = tile_n * NT;
  const int nvalid = min(NT, J.N - nbase);  // valid columns of this tile
  for (int cc = 0; cc < NT; cc += 32) {
    if (warp < 4) {  // warp w reads accumulator lanes 32w .. 32w+31
      uint32_t r[32], q[32];
      tmem_ld32_nowait(tmem + ((uint32_t)(warp * 32) << 16) + total + (uint32_t)cc, r);
      tmem_ld32_nowait(tmem + ((uint32_t)(warp * 32) << 16) + corr + (uint32_t)cc, q);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 32; j++)
        stage[(warp * 32 + wl) * 33 + j] = __fadd_rn(__uint_as_float(r[j]), __uint_as_float(q[j]));
    }
    __syncthreads();
    // FP32 outputs of scale 1 are stored as they are (a round trip through
    // FP64 would run at the FP64 rate on this GPU)
    // A thread's lane (lanes fast) or column (rows) is the same in all 16
    // iterations, so its addresses advance by a constant: staged element
    // q = tid + 256 it is (lane l, column n) with
    //   0: l = tid & 127, n = (tid >> 7) + 2 it
    //   1: l = (tid >> 5) + 8 it, n = tid & 31
    //   2: l = 2 (tid >> 6) + (tid & 1) + 8 it, n = (tid >> 1) & 31
    const long long esz = otype == LT_F64 ? 8 : 4;
    auto store_all = [&](auto store, auto mode) {
      constexpr int M = decltype(mode)::value;
      if constexpr (M == 0) {
        const int l = tid & 127, n0 = tid >> 7;
        char* base = ob[l];
        if (base != nullptr) {
          char* pp = base + (long long)(nbase + cc + n0) * oes * esz;
          const long long step = 2 * oes * esz;
          const float* sv = stage + l * 33 + n0;
#pragma unroll 4
          for (int it = 0; it < 4096 / kGemmThreads; it++, pp += step)
            if (cc + n0 + 2 * it < nvalid) store(pp, sv[2 * it]);
        }
      } else {
        const int n = M == 1 ? (tid & 31) : ((tid >> 1) & 31);
        const int l0 = M == 1 ? (tid >> 5) : 2 * (tid >> 6) + (tid & 1);
        if (cc + n < nvalid) {
          const long long off = (long long)(nbase + cc + n) * oes * esz;
#pragma unroll 4
          for (int it = 0; it < 4096 / kGemmThreads; it++) {
            const int l = l0 + 8 * it;
            char* base = ob[l];
            if (base != nullptr) store(base + off, stage[l * 33 + n]);
          }
        }
      }
    };
    auto store_typed = [&](auto mode) {
      if (otype == LT_F64 && scale == 1.0)  // no FP64 product (the conversion alone runs at the FP64 rate)
        store_all([&](char* p, float f) { *reinterpret_cast<double*>(p) = (double)f; }, mode);
      else if (otype == LT_F64)
        store_all([&](char* p, float f) { *reinterpret_cast<double*>(p) = (double)f * scale; }, mode);
      else if (scale == 1.0)
        store_all([&](char* p, float f) { *reinterpret_cast<float*>(p) = f; }, mode);
      else
        store_all([&](char* p, float f) { *reinterpret_cast<float*>(p) = (float)((double)f * scale); }, mode);
    };
    if (omode == 0) store_typed(std::integral_constant<int, 0>());
    else if (omode == 1) store_typed(std::integral_constant<int, 1>());
    else store_typed(std::integral_constant<int, 2>());
    __syncthreads();
  }
}

template <class T>
__device__ __forceinline__ void gemm_tile_t(const GemmJobDev& J, const int lane0, const int tile_n) {
  const int NT = J.NT;
  const int tid = threadIdx.x, warp = tid >> 5, wl = tid & 31;
  extern __shared__ __align__(128) unsigned char sm[];
  // A chunk (hi, lo) | operator chunk buffers 0 and 1 (hi, lo each) | tail
  unsigned char* Ahi = sm;
  unsigned char* Alo = sm + 16384;
  unsigned char* Wb[2] = {sm + 32768, sm + 32768 + 2 * NT * 128};
  unsigned char* tail = sm + 32768 + 4 * NT * 128;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(tail);
  uint32_t* slot = reinterpret_cast<uint32_t*>(tail + 8);
  const char** ib = reinterpret_cast<const char**>(tail + 16);
  char** ob = reinterpret_cast<char**>(tail + 16 + kGemmLanes * 8);
  float* stage = reinterpret_cast<float*>(sm);  // [128][33], reuses the A chunk after the last MMA

  if (tid < kGemmLanes) {
    const int l = lane0 + tid;
    const char* ip = nullptr;
    char* op = nullptr;
    if (l < J.lanes) {
      ip = lane_addr(J.in, l);
      op = const_cast<char*>(lane_addr(J.out, l));
    }
    ib[tid] = ip;
    ob[tid] = op;
  }
  const float* wsrc = J.w + (size_t)tile_n * J.kchunks * 2 * NT * kGemmKC;
  w_issue(wsrc, 0, NT, Wb[0], tid);  // operator chunk 0 in flight during the set-up
  cp_async_commit();
  // tensor-memory columns: chunk partials of the hi*hi products at 0 and NT
  // (alternate chunks), the lo*hi + hi*lo corrections at 2 NT, the running
  // total at 3 NT; corrections and total are added with round-to-nearest at
  // the end (accumulated into the hi*hi sum the corrections would lose bits
  // to the tensor core's truncating accumulation)
  const uint32_t ncols = gemm_tmem_cols(NT);
  const uint32_t corr = 2u * (uint32_t)NT, total = 3u * (uint32_t)NT;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) mbar_init(mbar, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  // instruction descriptor: D f32, A/B tf32, K-major both, N = NT, M = 128
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NT >> 3) << 17) | ((128u >> 4) << 24);
  const uint32_t a_lbo = (kGemmLanes / 8) * 128, w_lbo = (uint32_t)(NT / 8) * 128;
  bool ok = true;
  const long long wait_limit = g_gemm_wait_limit;
  uint32_t pending = 0;  // phase parity of the commit a failed wait left in flight
  const int K = J.K, kchunks = J.kchunks;
  const bool in_lf = J.in.lane_fast != 0;
  ATile<T> at;
  a_setup<T>(at, J, ib, tid);
  AChunk<T> a;
  a_load<T>(a, at, 0, K, in_lf, tid);

  for (int c = 0; c < kchunks; c++) {
    // the A buffer and operator buffer (c+1)&1 were read by MMA c-1
    if (c > 0) {
      pending = (uint32_t)((c - 1) & 1);
      ok = mma_wait(mbar, pending, wait_limit);
      tc_fence_after();
      if (!ok) break;
    }
    a_store<T>(a, at, Ahi, Alo);
    // next input chunk in flight through the barrier, the MMAs and the flush
    if (c + 1 < kchunks) a_load<T>(a, at, (c + 1) * kGemmKC, K, in_lf, tid);
    if (c + 1 < kchunks) w_issue(wsrc, c + 1, NT, Wb[(c + 1) & 1], tid);
    cp_async_commit();
    cp_async_wait1();  // operator chunk c has landed (this thread's copies)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
      unsigned char* Whi = Wb[c & 1];
      unsigned char* Wlo = Whi + NT * 128;
      const uint32_t part = (uint32_t)((c & 1) * NT);
#pragma unroll
      for (int s = 0; s < kGemmKC / 8; s++) {
        const uint64_t ah = umma_desc(smem_u32(Ahi) + s * 2 * a_lbo, a_lbo, 128);
        const uint64_t al = umma_desc(smem_u32(Alo) + s * 2 * a_lbo, a_lbo, 128);
        const uint64_t wh = umma_desc(smem_u32(Whi) + s * 2 * w_lbo, w_lbo, 128);
        const uint64_t wlo = umma_desc(smem_u32(Wlo) + s * 2 * w_lbo, w_lbo, 128);
        const uint32_t acc = (c > 0 || s > 0) ? 1u : 0u;
        mma_tf32(tmem + corr, al, wh, idesc, acc);
        mma_tf32(tmem + corr, ah, wlo, idesc, 1u);
        mma_tf32(tmem + part, ah, wh, idesc, s > 0 ? 1u : 0u);  // fresh partial per chunk
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(mbar))
                   : "memory");
    }
    // the previous chunk's partial into the running total, while chunk c multiplies
    if (c > 0) tmem_accumulate(tmem, (uint32_t)(((c - 1) & 1) * NT), total, NT, c == 1, warp);
  }
  if (ok) {
    pending = (uint32_t)((kchunks - 1) & 1);
    ok = mma_wait(mbar, pending, wait_limit);
    tc_fence_after();
    if (ok) {
      tmem_accumulate(tmem, (uint32_t)(((kchunks - 1) & 1) * NT), total, NT, kchunks == 1, warp);
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
    }
  }
  asm volatile("cp.async.wait_all;" ::: "memory");

  if (ok) {
    gemm_epilogue(J, tmem, total, corr, NT, tile_n, ob, stage, tid, warp, wl);
  } else {
    if (tid == 0 && J.status != nullptr) atomicOr(J.status, kStatusGemmTimeout);
    // the MMAs of the commit that was not seen to complete may still read
    // shared memory and write tensor memory: wait for them (bounded) before
    // the shared memory and the columns are given back
    mma_wait(mbar, pending, kWaitLimit);
    tc_fence_after();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// ---------------------------------------------------------------------------
// Warp-specialised form (a tuned GEMM form): the same products, partials,
// corrections and epilogue, with the per-chunk sequence split over roles that
// hand chunks on through mbarriers instead of CTA barriers:
//   * warps 0-3 (producers) stage chunk c (input converted to hi/lo TF32; the
//     operator chunk as one bulk copy whose bytes the same barrier counts)
//     into buffer c % 2 and arrive on full;
//   * warp 4, lane 0 waits for full (and for the flush of the chunk that last
//     used the same partial columns), issues the chunk's 12 MMAs and commits
//     to mdone;
//   * warps 4-7 (one tensor-memory lane quadrant each) wait for mdone and add
//     the chunk's partial into the running total, then arrive on flushed.
// So staging chunk c+1, the MMAs of chunk c and the flush of chunk c-1 overlap.
// Buffers and partials are double-buffered; each barrier's phases alternate
// per use, and no role gets more than one phase ahead of another.  Every wait
// is bounded: a warp that gives up sets the tile's abort flag, the others give
// up at their next check, and the tile then drains its committed MMAs, sets
// kStatusGemmTimeout and frees its tensor memory.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mbar_arrive(uint64_t* m) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(m)) : "memory");
}
// one arrival that also announces `bytes` of asynchronous transfer to come
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* m, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                   smem_u32(m)),
               "r"(bytes)
               : "memory");
}
// bulk copy global -> shared (16-byte aligned, size a multiple of 16), its
// completion counted on the mbarrier's transaction count
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* m) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(m))
               : "memory");
}

// bounded wait of one warp for phase `parity` of an mbarrier: lane 0 polls
// (giving up early once the tile is aborted), the outcome goes to all lanes
__device__ __forceinline__ bool warp_mbar_wait(uint64_t* m, uint32_t parity, long long limit,
                                               volatile int* abort_flag) {
  int ok = 0;
  if ((threadIdx.x & 31) == 0) {
    for (long long i = 0; i < limit; i++) {
      if (mbar_try(m, parity)) {
        ok = 1;
        break;
      }
      if ((i & 1023) == 1023 && *abort_flag) break;
    }
    if (!ok) *abort_flag = 1;
  }
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// running total += chunk partial (or = partial for the first chunk) for one
// warp's 32 tensor-memory lanes (quadrant q) and all NT <= 64 columns, in
// rounds of two 8-column blocks
__device__ __forceinline__ void tmem_accumulate_warp(uint32_t tmem, uint32_t part, uint32_t total, int NT,
                                                     bool first, int q) {
  const uint32_t lane_base = (uint32_t)(q * 32) << 16;
#pragma unroll
  for (int h = 0; h < 4; h++) {
    const int cb = 16 * h;
    if (cb >= NT) break;  // NT is a multiple of 16: both blocks of a round are valid
    uint32_t p[2][8], t[2][8];
#pragma unroll
    for (int b = 0; b < 2; b++) {
      tmem_ld8_nowait(tmem + lane_base + part + (uint32_t)(cb + 8 * b), p[b]);
      if (!first) tmem_ld8_nowait(tmem + lane_base + total + (uint32_t)(cb + 8 * b), t[b]);
    }
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int b = 0; b < 2; b++) {
      float v[8];
#pragma unroll
      for (int j = 0; j < 8; j++)
        v[j] = first ? __uint_as_float(p[b][j]) : __fadd_rn(__uint_as_float(t[b][j]), __uint_as_float(p[b][j]));
      tmem_st8(tmem + lane_base + total + (uint32_t)(cb + 8 * b), v);
    }
  }
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// shared memory of the warp-specialised form: two input chunks (hi, lo), two
// operator chunks, six barriers and three words, the lane bases
__host__ __device__ inline size_t gemm_ws_smem_base(int NT) {
  return 65536 + (size_t)4 * NT * 128 + 64 + 2 * kGemmLanes * 8;
}

template <class T>
__device__ __forceinline__ void gemm_tile_ws_t(const GemmJobDev& J, const int lane0, const int tile_n) {
  const int NT = J.NT;  // <= 64
  const int tid = threadIdx.x, warp = tid >> 5, wl = tid & 31;
  extern __shared__ __align__(128) unsigned char sm[];
  unsigned char* Ab[2] = {sm, sm + 32768};
  unsigned char* Wb[2] = {sm + 65536, sm + 65536 + 2 * NT * 128};
  unsigned char* tail = sm + 65536 + 4 * NT * 128;
  uint64_t* full = reinterpret_cast<uint64_t*>(tail);  // [2]
  uint64_t* mdone = full + 2;                          // [2]
  uint64_t* flushed = full + 4;                        // [2]
  uint32_t* slot = reinterpret_cast<uint32_t*>(tail + 48);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tail + 52);
  volatile int* issued = reinterpret_cast<volatile int*>(tail + 56);   // chunks whose MMAs were committed
  volatile int* wissued = reinterpret_cast<volatile int*>(tail + 60);  // chunks whose operator copy was issued
  const char** ib = reinterpret_cast<const char**>(tail + 64);
  char** ob = reinterpret_cast<char**>(tail + 64 + kGemmLanes * 8);
  float* stage = reinterpret_cast<float*>(sm);  // epilogue staging, after the last MMA

  if (tid < kGemmLanes) {
    const int l = lane0 + tid;
    const char* ip = nullptr;
    char* op = nullptr;
    if (l < J.lanes) {
      ip = lane_addr(J.in, l);
      op = const_cast<char*>(lane_addr(J.out, l));
    }
    ib[tid] = ip;
    ob[tid] = op;
  }
  const float* wsrc = J.w + (size_t)tile_n * J.kchunks * 2 * NT * kGemmKC;
  const uint32_t ncols = gemm_tmem_cols(NT);
  const uint32_t corr = 2u * (uint32_t)NT, total = 3u * (uint32_t)NT;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < 2; s++) {
      mbar_init(&full[s], 129);  // the producers, and the arrival that announces the operator chunk's bytes
      mbar_init(&mdone[s], 1);
      mbar_init(&flushed[s], 128);
    }
    *abort_flag = 0;
    *issued = 0;
    *wissued = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NT >> 3) << 17) | ((128u >> 4) << 24);
  const uint32_t a_lbo = (kGemmLanes / 8) * 128, w_lbo = (uint32_t)(NT / 8) * 128;
  const long long wait_limit = g_gemm_wait_limit;
  const int K = J.K, kchunks = J.kchunks;

  if (warp < 4) {
    // producers: stage chunk c into buffer c % 2 once the MMAs of chunk c-2 are done with it
    const bool in_lf = J.in.lane_fast != 0;
    ATile<T, 128> at;
    a_setup<T, 128>(at, J, ib, tid);
    AChunk<T, 128> a;
    a_load<T, 128>(a, at, 0, K, in_lf, tid);
    for (int c = 0; c < kchunks; c++) {
      const int s = c & 1;
      if (c >= 2 && !warp_mbar_wait(&mdone[s], (uint32_t)(((c >> 1) - 1) & 1), wait_limit, abort_flag)) break;
      if (tid == 0) {
        const uint32_t wbytes = (uint32_t)(2 * NT * kGemmKC * 4);
        mbar_arrive_expect_tx(&full[s], wbytes);
        bulk_g2s(Wb[s], wsrc + (size_t)c * 2 * NT * kGemmKC, wbytes, &full[s]);
        *wissued = c + 1;
      }
      // no exit between the copy's issue and this chunk's arrival: every issued
      // copy completes its phase of full, which an aborted tile waits for
      a_store<T, 128>(a, at, Ab[s], Ab[s] + 16384);
      if (c + 1 < kchunks) a_load<T, 128>(a, at, (c + 1) * kGemmKC, K, in_lf, tid);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(&full[s]);
    }
  } else {
    // MMA issue (warp 4, lane 0) and the flush of the previous chunk (warps 4-7)
    const int quad = warp - 4;
    for (int c = 0; c <= kchunks; c++) {
      if (c < kchunks && warp == 4) {
        int ok = 1;
        if (wl == 0) {
          const int s = c & 1;
          ok = 0;
          for (long long i = 0; i < wait_limit && !ok; i++) {
            ok = mbar_try(&full[s], (uint32_t)((c >> 1) & 1)) ? 1 : 0;
            if (!ok && (i & 1023) == 1023 && *abort_flag) break;
          }
          if (ok && c >= 2) {
            ok = 0;
            for (long long i = 0; i < wait_limit && !ok; i++) {
              ok = mbar_try(&flushed[s], (uint32_t)(((c >> 1) - 1) & 1)) ? 1 : 0;
              if (!ok && (i & 1023) == 1023 && *abort_flag) break;
            }
          }
          if (ok) {
            tc_fence_after();
            unsigned char* Ahi = Ab[s];
            unsigned char* Alo = Ab[s] + 16384;
            unsigned char* Whi = Wb[s];
            unsigned char* Wlo = Whi + NT * 128;
            const uint32_t part = (uint32_t)(s * NT);
#pragma unroll
            for (int ks = 0; ks < kGemmKC / 8; ks++) {
              const uint64_t ah = umma_desc(smem_u32(Ahi) + ks * 2 * a_lbo, a_lbo, 128);
              const uint64_t al = umma_desc(smem_u32(Alo) + ks * 2 * a_lbo, a_lbo, 128);
              const uint64_t wh = umma_desc(smem_u32(Whi) + ks * 2 * w_lbo, w_lbo, 128);
              const uint64_t wlo = umma_desc(smem_u32(Wlo) + ks * 2 * w_lbo, w_lbo, 128);
              const uint32_t acc = (c > 0 || ks > 0) ? 1u : 0u;
              mma_tf32(tmem + corr, al, wh, idesc, acc);
              mma_tf32(tmem + corr, ah, wlo, idesc, 1u);
              mma_tf32(tmem + part, ah, wh, idesc, ks > 0 ? 1u : 0u);  // fresh partial per chunk
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mdone[s]))
                         : "memory");
            *issued = c + 1;
          } else {
            *abort_flag = 1;
          }
        }
        if (__shfl_sync(0xffffffffu, ok, 0) == 0) break;
      }
      if (c >= 1) {
        const int c1 = c - 1, s1 = c1 & 1;
        if (!warp_mbar_wait(&mdone[s1], (uint32_t)((c1 >> 1) & 1), wait_limit, abort_flag)) break;
        tc_fence_after();
        tmem_accumulate_warp(tmem, (uint32_t)(s1 * NT), total, NT, c1 == 0, quad);
        tc_fence_before();
        mbar_arrive(&flushed[s1]);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const bool ok = *abort_flag == 0;
  if (ok) {
    gemm_epilogue(J, tmem, total, corr, NT, tile_n, ob, stage, tid, warp, wl);
  } else {
    if (tid == 0) {
      if (J.status != nullptr) atomicOr(J.status, kStatusGemmTimeout);
      // operator copies not consumed by an MMA, and the last commit on each
      // buffer, may still be in flight: wait for them (bounded) before the
      // shared memory and the columns are given back
      const int n = *issued, nw = *wissued;
      for (int c = n; c < nw; c++)
        for (long long i = 0; i < kWaitLimit; i++)
          if (mbar_try(&full[c & 1], (uint32_t)((c >> 1) & 1))) break;
      for (int c = n - 2 < 0 ? 0 : n - 2; c < n; c++)
        for (long long i = 0; i < kWaitLimit; i++)
          if (mbar_try(&mdone[c & 1], (uint32_t)((c >> 1) & 1))) break;
    }
    tc_fence_after();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

__device__ __forceinline__ void gemm_tile(const GemmJobDev& J, const int lane0, const int tile_n) {
  if (J.active != nullptr && *J.active == 0) return;
  if (J.in.type == LT_F64) gemm_tile_t<double>(J, lane0, tile_n);
  else gemm_tile_t<float>(J, lane0, tile_n);
}

// grouped form: tile table entries (job, first lane, output tile, 0)
__global__ void __launch_bounds__(kGemmThreads, 2) k_lane_gemm(const GemmJobDev* __restrict__ jobs,
                                                                const int4* __restrict__ tiles) {
  const int4 tl = tiles[blockIdx.x];
  gemm_tile(jobs[tl.x], tl.y, tl.z);
}

// the same tiles in the warp-specialised form (output tiles of at most 64 columns)
__global__ void __launch_bounds__(kGemmThreads, 2) k_lane_gemm_ws(const GemmJobDev* __restrict__ jobs,
                                                                   const int4* __restrict__ tiles) {
  const int4 tl = tiles[blockIdx.x];
  const GemmJobDev& J = jobs[tl.x];
  if (J.active != nullptr && *J.active == 0) return;
  if (J.in.type == LT_F64) gemm_tile_ws_t<double>(J, tl.y, tl.z);
  else gemm_tile_ws_t<float>(J, tl.y, tl.z);
}

// single job passed by value: block b -> lanes (b / ntiles) * 128, output tile b % ntiles
__global__ void __launch_bounds__(kGemmThreads, 2) k_lane_gemm_one(const __grid_constant__ GemmJobDev J) {
  const int b = blockIdx.x;
  gemm_tile(J, (b / J.ntiles) * kGemmLanes, b % J.ntiles);
}

}  // namespace dev

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int gemm_tile_n(int N, int ntmax) {
  // at most ntmax outputs per tile, wider outputs split into equal tiles.
  // 64: 4 NT tensor-memory columns per CTA (two chunk partials, corrections,
  // total) leave room for two CTAs per SM; 128: one CTA holds all 512 columns
  auto r16 = [](int v) { return (v + 15) & ~15; };
  if (N <= ntmax) return r16(N);
  int t = (N + ntmax - 1) / ntmax;
  return r16((N + t - 1) / t);
}

static float tf32_rna_host(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u = (u + 0x1000u) & 0xFFFFE000u;  // round to nearest (ties away) at the 10-bit mantissa
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

static int cm_off_host(int r, int k, int R) {
  return ((k >> 2) * (R >> 3) + (r >> 3)) * 128 + (r & 7) * 16 + (k & 3) * 4;
}

std::vector<float> pack_gemm_w(const std::vector<double>& W, int N, int K, int NT) {
  const int ntiles = (N + NT - 1) / NT, kch = (K + kGemmKC - 1) / kGemmKC;
  const size_t blk = (size_t)2 * NT * kGemmKC;
  std::vector<float> out((size_t)ntiles * kch * blk, 0.0f);
  for (int t = 0; t < ntiles; t++)
    for (int c = 0; c < kch; c++) {
      float* b = out.data() + ((size_t)t * kch + c) * blk;
      for (int nl = 0; nl < NT; nl++) {
        const int n = t * NT + nl;
        if (n >= N) break;
        for (int kl = 0; kl < kGemmKC; kl++) {
          const int k = c * kGemmKC + kl;
          if (k >= K) break;
          const double w = W[(size_t)n * K + k];
          const float hi = tf32_rna_host((float)w);
          const float lo = tf32_rna_host((float)(w - (double)hi));
          const int off = cm_off_host(nl, kl, NT) / 4;
          b[off] = hi;
          b[(size_t)NT * kGemmKC + off] = lo;
        }
      }
    }
  return out;
}

void gemm_tiles(const std::vector<GemmJobDev>& jobs, std::vector<int4>& tiles) {
  tiles.clear();
  for (size_t j = 0; j < jobs.size(); j++)
    for (int l0 = 0; l0 < jobs[j].lanes; l0 += kGemmLanes)
      for (int t = 0; t < jobs[j].ntiles; t++) tiles.push_back(make_int4((int)j, l0, t, 0));
  // longest tiles (most K chunks) first, so the last wave holds short ones;
  // the sort is stable, so the output tiles of one lane block stay adjacent
  // and share its input in L2
  std::stable_sort(tiles.begin(), tiles.end(),
                   [&](const int4& a, const int4& b) { return jobs[a.x].kchunks > jobs[b.x].kchunks; });
}

size_t gemm_smem_bytes(int NT) {
  // A chunk (hi, lo) + two operator chunks (hi, lo) + barrier, tmem slot, lane bases
  const size_t base = 32768 + (size_t)4 * NT * 128 + 16 + 2 * kGemmLanes * 8;
  const size_t ncols = dev::gemm_tmem_cols(NT);
  // keep (resident CTAs per SM) x (tensor-memory columns) within the 512
  // columns: at most 512 / ncols CTAs fit, so ask for enough shared memory
  // (of the 228 KB per SM, 1 KB reserved per CTA) that no more become resident.
  // A CTA holding all 512 columns asks for more than what is left beside the
  // smallest GEMM CTA, so that no CTA of another GEMM launch (its tcgen05.alloc
  // would wait for columns) shares its SM
  const size_t sm_total = 228 * 1024;
  if (ncols >= 512) return std::max(base, sm_total - 2 * 1024 - gemm_smem_bytes(16) + 1);
  const size_t max_ctas = 512 / ncols;
  const size_t floor_b = sm_total / (max_ctas + 1) - 1024 + 1;
  return std::max(base, floor_b);
}

size_t gemm_ws_smem_bytes(int NT) {
  // as gemm_smem_bytes: no more CTAs per SM than the tensor-memory columns allow
  return std::max(dev::gemm_ws_smem_base(NT), gemm_smem_bytes(NT));
}

cudaError_t configure_gemm_kernels() {
  static PerDeviceFlag done;
  if (done.test()) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(dev::k_lane_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)gemm_smem_bytes(128));  // tiles hold at most 128 outputs
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(dev::k_lane_gemm_one, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)gemm_smem_bytes(128));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(dev::k_lane_gemm_ws, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)gemm_ws_smem_bytes(64));
  if (e == cudaSuccess) done.set();
  return e;
}

cudaError_t set_gemm_wait_limit(long long polls) {
  const long long v = polls < 0 ? dev::kWaitLimit : polls;
  return cudaMemcpyToSymbol(dev::g_gemm_wait_limit, &v, sizeof v);
}

cudaError_t launch_lane_gemm_one(const GemmJobDev& job, cudaStream_t st) {
  const int blocks = ((job.lanes + kGemmLanes - 1) / kGemmLanes) * job.ntiles;
  if (blocks <= 0) return cudaSuccess;
  dev::k_lane_gemm_one<<<blocks, kGemmThreads, gemm_smem_bytes(job.NT), st>>>(job);
  return cudaGetLastError();
}

GemmJobDev make_gemm_job(const LaneSideDev& in, const LaneSideDev& out, const float* w, int K, int N, double scale,
                         unsigned int* status, int ntmax) {
  GemmJobDev j;
  std::memset(&j, 0, sizeof j);
  j.in = in;
  j.out = out;
  j.w = w;
  j.K = K;
  j.N = N;
  j.NT = gemm_tile_n(N, ntmax);
  j.kchunks = (K + kGemmKC - 1) / kGemmKC;
  j.ntiles = (N + j.NT - 1) / j.NT;
  j.lanes = in.nf * in.rows * in.parts;
  j.scale = scale;
  j.status = status;
  return j;
}

LaneSideDev lane_rows(void* const* ptrs, int nf, int rows, int len, int row_len, int type, bool complex_) {
  LaneSideDev s;
  std::memset(&s, 0, sizeof s);
  for (int f = 0; f < nf; f++) s.ptr[f] = ptrs[f];
  s.nf = nf;
  s.rows = rows;
  s.parts = complex_ ? 2 : 1;
  s.type = type;
  s.lane_stride = (long long)row_len * s.parts;
  s.elem_stride = s.parts;
  s.part_stride = complex_ ? 1 : 0;
  s.len = len;
  s.lane_fast = 0;
  return s;
}

LaneSideDev lane_cols(void* const* ptrs, int nf, int cols, int len, int row_len, int type, int col0) {
  LaneSideDev s;
  std::memset(&s, 0, sizeof s);
  const size_t es = type == LT_F64 ? 8 : 4;
  for (int f = 0; f < nf; f++) s.ptr[f] = static_cast<char*>(ptrs[f]) + (size_t)col0 * es;
  s.nf = nf;
  s.rows = cols;
  s.parts = 1;
  s.type = type;
  s.lane_stride = 1;
  s.elem_stride = row_len;
  s.part_stride = 0;
  s.len = len;
  s.lane_fast = 1;
  return s;
}

cudaError_t launch_lane_gemm(const GemmJobDev* jobs, const int4* tiles, int ntiles_total, int max_nt,
                             cudaStream_t st, bool ws) {
  if (ntiles_total <= 0) return cudaSuccess;
  if (ws) {
    if (max_nt > 64) return cudaErrorInvalidValue;
    dev::k_lane_gemm_ws<<<ntiles_total, kGemmThreads, gemm_ws_smem_bytes(max_nt), st>>>(jobs, tiles);
  } else {
    dev::k_lane_gemm<<<ntiles_total, kGemmThreads, gemm_smem_bytes(max_nt), st>>>(jobs, tiles);
  }
  return cudaGetLastError();
}

}  // namespace rbc
