// lvg_noalloc.cu — modularity of a membership without any device allocation.
//
// lvg_modularity() needs per-community FP64 totals and takes them from the
// graph handle's workspace, which the library allocates with cudaMalloc.
// Some callers cannot allocate device memory at call time: a host framework
// that has reserved the GPU's memory for its own pool, a latency-critical
// loop that must not pay cudaMalloc's cost and implicit synchronisation, or
// a deployment that forbids allocation after start-up. For them,
// lvg_modularity_noalloc() works on caller-owned device buffers and keeps its
// scratch in a fixed file-scope device array instead.
#include <mutex>

#include "lvg_internal.cuh"

namespace lvg {
namespace {

// Per-community FP64 totals for up to LVG_NOALLOC_MAX_SPAN slots, then four
// accumulators: intra-community weight, sum of squared totals, total edge
// weight, out-of-range id flag. 8 MiB + 32 B, held by every GPU that loads
// the library until the process exits.
constexpr size_t ACC = LVG_NOALLOC_MAX_SPAN;
static __device__ __align__(256) double g_noalloc_scratch[LVG_NOALLOC_MAX_SPAN + 4];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
double *g_addr[MAX_DEVICES] = {};

// The device address of the scratch array on the current device, looked up
// once per device (the host-side symbol is only a stand-in, not a device
// address).
double *scratch_address() {
  int dev = 0;
  LVG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) throw Error(LVG_EINVAL, "device index out of range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    LVG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_addr[dev] = static_cast<double *>(p);
  }
  return g_addr[dev];
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One warp per vertex: intra-community weight, the community's total, and
// the total edge weight (modularityBy, inc/properties.hxx:178-191). Ids that
// fall outside the span are skipped and flagged.
__global__ void noalloc_terms_kernel(const uint64_t *off, const uint32_t *key, const float *w, const uint8_t *ex,
                                     size_t n, const uint32_t *memb, double *scratch) {
  const size_t warps = size_t(gridDim.x) * blockDim.x / 32;
  const int lane = threadIdx.x & 31;
  double in = 0, all = 0;
  bool bad = false;
  for (size_t u = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; u < n; u += warps) {
    if (ex && !ex[u]) continue;
    const uint32_t c = memb[u];
    if (c >= n) { bad = true; continue; }
    double tot = 0;
    for (uint64_t j = off[u] + lane; j < off[u + 1]; j += 32) {
      const uint32_t v = key[j];
      const double x = w[j];
      tot += x;
      if (v >= n) { bad = true; continue; }
      if (memb[v] == c) in += x;
    }
    tot = warp_sum(tot);
    if (lane == 0 && tot != 0.0) atomicAdd(&scratch[c], tot);
    all += lane == 0 ? tot : 0.0;
  }
  in = warp_sum(in);
  all = warp_sum(all);
  bad = __any_sync(0xffffffffu, bad);
  if (lane == 0) {
    if (in != 0.0) atomicAdd(&scratch[ACC + 0], in);
    if (all != 0.0) atomicAdd(&scratch[ACC + 2], all);
    if (bad) scratch[ACC + 3] = 1.0;
  }
}

__global__ void noalloc_squares_kernel(size_t n, double *scratch) {
  double s = 0;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    s += scratch[i] * scratch[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(&scratch[ACC + 1], s);
}

__global__ void noalloc_final_kernel(const double *scratch, double M, double R, double *out) {
  if (scratch[ACC + 3] != 0.0) {
    *out = __longlong_as_double(0x7ff8000000000000ll);  // NaN: an id was out of range
    return;
  }
  if (M <= 0) M = scratch[ACC + 2] / 2;
  *out = scratch[ACC + 0] / (2 * M) - R * scratch[ACC + 1] / (4 * M * M);
}

}  // namespace
}  // namespace lvg

extern "C" int lvg_modularity_noalloc(size_t span, const uint64_t *offsets, const uint32_t *keys,
                                      const float *weights, const uint8_t *exists, const uint32_t *membership,
                                      double M, double R, double *out, void *stream) {
  // keys and weights are read for every vertex with edges: a null one would be
  // a device fault, not an error code, so it is refused here (a caller with an
  // edgeless graph passes any valid device pointer).
  if (!offsets || !keys || !weights || !membership || !out || span == 0)
    return lvg::fail_noalloc(LVG_EINVAL, "lvg_modularity_noalloc: null argument or empty span");
  if (span > LVG_NOALLOC_MAX_SPAN)
    return lvg::fail_noalloc(LVG_EINVAL, "lvg_modularity_noalloc: span exceeds LVG_NOALLOC_MAX_SPAN (1048576)");
  try {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double *scratch = lvg::scratch_address();
    // Every call shares the array and it keeps the last call's contents: clear
    // the totals this call uses and the accumulators.
    LVG_CUDA(cudaMemsetAsync(scratch, 0, span * sizeof(double), s));
    LVG_CUDA(cudaMemsetAsync(scratch + lvg::ACC, 0, 4 * sizeof(double), s));
    lvg::noalloc_terms_kernel<<<lvg::grid_for(span * 32, 256), 256, 0, s>>>(offsets, keys, weights, exists, span,
                                                                             membership, scratch);
    LVG_CHECK_LAUNCH();
    lvg::noalloc_squares_kernel<<<lvg::grid_for(span, 256), 256, 0, s>>>(span, scratch);
    LVG_CHECK_LAUNCH();
    lvg::noalloc_final_kernel<<<1, 1, 0, s>>>(scratch, M, R, out);
    LVG_CHECK_LAUNCH();
    return LVG_OK;
  } catch (const lvg::Error &e) {
    return lvg::fail_noalloc(e.code, e.what());
  }
}
