// lvg_common.cuh — shared types, error handling and device helpers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>

#include "louvain_gb300.h"

namespace lvg {

// ------------------------------------------------------------------ errors

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define LVG_CUDA(call)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess) {                                                                    \
      throw ::lvg::Error(e_ == cudaErrorMemoryAllocation ? LVG_ENOMEM : LVG_ECUDA,              \
                         std::string(#call) + ": " + cudaGetErrorString(e_) + " (" __FILE__ ":" + \
                             std::to_string(__LINE__) + ")");                                   \
    }                                                                                           \
  } while (0)

// Kernels launched by the calling thread (for the launch count of a call).
inline unsigned long long &launch_counter() {
  static thread_local unsigned long long c = 0;
  return c;
}

#define LVG_CHECK_LAUNCH()            \
  do {                                \
    ++::lvg::launch_counter();        \
    LVG_CUDA(cudaGetLastError());     \
  } while (0)

// ------------------------------------------------------------------ constants

constexpr uint32_t EMPTY = 0xFFFFFFFFu;  // empty hash slot
constexpr int WARP = 32;
constexpr int NUM_SMS_HINT = 152;

// Fixed-point scale of the per-iteration gain sum (exact, order free).
constexpr double GAIN_FIX = 65536.0;

// Device error flags (bit set in Engine::d_err).
constexpr uint32_t ERR_TABLE_FULL = 1u;
constexpr uint32_t ERR_BAD_ID = 2u;  // an input id was >= span
constexpr uint32_t ERR_WORKLIST = 4u;  // a worklist append fell outside its degree bin's slice

// Degree bins of the per-vertex (and per-community) reduce kernels.
//   bin 0: degree 0 (nothing to scan)
//   bins 1-4: sub-warp tiles of 4/8/16/32 lanes, degree <= tile
//   bins 5-8: one warp, shared table of 128..1024 slots, degree <= 64..512
//   bins 9-10: one block, shared table of 4096 / 16384 slots, degree <= 2048 / 8192
//   bin 11: one block, global-memory table, degree > 8192
constexpr int NUM_BINS = 12;
__host__ __device__ inline int degree_bin(uint64_t d) {
  if (d == 0) return 0;
  if (d <= 4) return 1;
  if (d <= 8) return 2;
  if (d <= 16) return 3;
  if (d <= 32) return 4;
  if (d <= 64) return 5;
  if (d <= 128) return 6;
  if (d <= 256) return 7;
  if (d <= 512) return 8;
  if (d <= 2048) return 9;
  if (d <= 8192) return 10;
  return 11;
}
constexpr uint64_t BIN_MAX_DEGREE[NUM_BINS] = {0, 4, 8, 16, 32, 64, 128, 256, 512, 2048, 8192, ~0ull};

// Degree bins of the local-moving kernels at run time: bin b (1..10) takes
// the degrees (hi[b-1], hi[b]], with hi[b] <= BIN_MAX_DEGREE[b] so that every
// vertex fits its bin's kernel (tile width, table capacity); hi[10] stays
// 8192 (the hubs above it have their own plan and tables). Lowering hi[b]
// hands the bin's upper degrees to the next bin's wider tile and larger
// table; hi[b] == hi[b-1] empties bin b. The defaults are BIN_MAX_DEGREE.
struct BinLimits {
  uint32_t hi[NUM_BINS];
};
__host__ __device__ inline BinLimits default_bin_limits() {
  // BIN_MAX_DEGREE, with the last bin's unbounded reach as 2^32-1
  return BinLimits{{0, 4, 8, 16, 32, 64, 128, 256, 512, 2048, 8192, 0xffffffffu}};
}
__host__ __device__ inline bool operator==(const BinLimits &a, const BinLimits &b) {
  for (int i = 0; i < NUM_BINS; ++i)
    if (a.hi[i] != b.hi[i]) return false;
  return true;
}
__host__ __device__ __forceinline__ int degree_bin(uint64_t d, const BinLimits &L) {
  if (d == 0) return 0;
  int b = NUM_BINS - 1;
#pragma unroll
  for (int i = NUM_BINS - 2; i >= 1; --i)
    if (d <= L.hi[i]) b = i;
  return b;
}

// Colour classes of the local-moving sweeps. Each iteration visits the
// classes one after another, so a vertex sees the moves its neighbours in
// earlier classes made in the same iteration (as in the reference's
// sequential sweep). The class of a vertex is a hash of its id.
constexpr int MAX_COLORS = 64;
constexpr int DEFAULT_COLORS_ASYNC = 8;
constexpr int DEFAULT_COLORS_SYNC = 16;
// Static Louvain in asynchronous mode with the default class count: the
// first iteration of the first pass, where every vertex is a singleton and
// nearly all of them move, sweeps FIRST_COLORS_STATIC classes; the later
// iterations STATIC_COLORS_ASYNC. Measured with the oracle's replay of the
// class rule against 3 asynchronous runs of its OpenMP port (R-MAT scale 16
// edge factor 48, R-MAT scale 18, the 131072-vertex planted partition): 8
// classes throughout came out 0.0037 / 0.0003 / 0.0002 below the port's
// modularity, 64 then 16 within 0.0001 of it on all three.
constexpr int FIRST_COLORS_STATIC = 64;
constexpr int STATIC_COLORS_ASYNC = 16;
constexpr int MAX_BUCKETS = MAX_COLORS * NUM_BINS;
__host__ __device__ inline uint32_t vertex_color(uint32_t u, uint32_t k) {
  uint32_t h = u * 0x9E3779B1u;
  h ^= h >> 16;
  return h % k;
}

// ------------------------------------------------------------------ device helpers

__device__ __forceinline__ uint32_t hash_slot(uint32_t k, uint32_t mask) {
  return (k * 0x9E3779B1u) & mask;
}

// Multiplicative hash using the high bits, for power-of-two capacities >= 2.
__device__ __forceinline__ uint32_t hash_hi(uint32_t k, int log2cap) {
  return (k * 0x9E3779B1u) >> (32 - log2cap);
}

// Vertex weights and community totals are FP64 on the device, as the
// reference's LOUVAIN_WEIGHT_TYPE (inc/louvain.hxx:67): a community total
// moves by atomic additions of vertex weights, and sums of integer weights
// below 2^53 are exact in any order, so the totals are order-free (and
// deterministic mode reproducible) at any graph size.
using tot_t = double;

// Gain of moving a vertex (weight wu, wuf = its FP32 rounding; links kc to c
// and kd to its own community d) into community c: M times the reference's
// deltaModularity (inc/properties.hxx:253-256),
//   g = (kc - kd) - wuf * f32((wu + tc) - td) * kr,
// the totals' part in FP64 and rounded once, the rest in FP32. Written with
// explicit round-to-nearest intrinsics so no FMA contraction changes the
// result; the oracle's orc_louvain_sync evaluates the same operations in the
// same order.
__device__ __forceinline__ float gain_of(float kc, float kd, double wu, float wuf, double tc, double td,
                                         float kr) {
  const float a = __fsub_rn(kc, kd);
  const float c = __double2float_rn(__dsub_rn(__dadd_rn(wu, tc), td));
  const float d = __fmul_rn(wuf, c);
  const float e = __fmul_rn(d, kr);
  return __fsub_rn(a, e);
}

// Candidate order: larger gain first, then lower community id.
__device__ __forceinline__ bool better(float g, uint32_t c, float bg, uint32_t bc) {
  return g > bg || (g == bg && c < bc);
}

// g * 2^16 is exact in FP32, so rounding it to an integer equals the oracle's
// llrint((double)g * 65536.0).
__device__ __forceinline__ unsigned long long gain_to_fix(float g) {
  return (unsigned long long)__float2ll_rn(g * 65536.0f);
}

// Smallest l with 2^l >= x (x >= 1).
__device__ __forceinline__ int ceil_log2(uint64_t x) { return x <= 1 ? 0 : 64 - __clzll(x - 1); }

template <class T>
__device__ __forceinline__ T ld_relaxed(const T *p) {
  return *((const volatile T *)p);
}

}  // namespace lvg
