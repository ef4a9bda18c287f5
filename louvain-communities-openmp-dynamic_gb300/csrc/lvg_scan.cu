// lvg_scan.cu — device-wide exclusive scans and the stable degree-bin split.
//
// The scan replaces the reference's two-level per-thread exclusiveScanOmpW
// (inc/_vector.hxx:1496-1524) used for renumbering (inc/louvain.hxx:941-945)
// and for the community and super-vertex CSR offsets (inc/louvain.hxx:804, 990).
// It is a reduce-then-scan over 4096-element tiles (no inter-block waiting).
#include "lvg_internal.cuh"

namespace lvg {
namespace {

constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

template <class T>
__device__ __forceinline__ T warp_incl_scan(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Exclusive block scan of one value per thread; returns the block total via *tot.
template <class T>
__device__ __forceinline__ T block_excl_scan(T v, T *tot) {
  __shared__ T wsum[SCAN_BLOCK / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T inc = warp_incl_scan(v);
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    T x = lane < SCAN_BLOCK / 32 ? wsum[lane] : T(0);
    x = warp_incl_scan(x);
    if (lane < SCAN_BLOCK / 32) wsum[lane] = x;
  }
  __syncthreads();
  T before = wid ? wsum[wid - 1] : T(0);
  *tot = wsum[SCAN_BLOCK / 32 - 1];
  __syncthreads();
  return before + inc - v;
}

template <class T>
__global__ void __launch_bounds__(SCAN_BLOCK) scan_reduce_kernel(const T *in, size_t n, T *partial) {
  size_t base = size_t(blockIdx.x) * SCAN_TILE;
  T s = 0;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    size_t j = base + size_t(i) * SCAN_BLOCK + threadIdx.x;
    if (j < n) s += in[j];
  }
  T tot;
  block_excl_scan(s, &tot);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

template <class T>
__global__ void __launch_bounds__(SCAN_BLOCK) scan_tile_kernel(const T *in, T *out, size_t n, const T *prefix,
                                                               T *total) {
  __shared__ T tile[SCAN_TILE + SCAN_TILE / 32];
  auto idx = [](int i) { return i + (i >> 5); };  // pad to break bank conflicts
  size_t base = size_t(blockIdx.x) * SCAN_TILE;
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    int k = i * SCAN_BLOCK + threadIdx.x;
    size_t j = base + k;
    tile[idx(k)] = j < n ? in[j] : T(0);
  }
  __syncthreads();
  T acc = 0;
  T loc[SCAN_ITEMS];
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    loc[i] = acc;
    acc += tile[idx(threadIdx.x * SCAN_ITEMS + i)];
  }
  T tot;
  T before = block_excl_scan(acc, &tot);
  T pre = prefix ? prefix[blockIdx.x] : T(0);
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) tile[idx(threadIdx.x * SCAN_ITEMS + i)] = pre + before + loc[i];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    int k = i * SCAN_BLOCK + threadIdx.x;
    size_t j = base + k;
    if (j < n) out[j] = tile[idx(k)];
  }
  if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *total = pre + tot;
}

template <class T>
void exclusive_scan_impl(const T *in, T *out, size_t n, T *total, T *scratch, cudaStream_t s) {
  if (n == 0) {
    if (total) LVG_CUDA(cudaMemsetAsync(total, 0, sizeof(T), s));
    return;
  }
  size_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb == 1) {
    scan_tile_kernel<T><<<1, SCAN_BLOCK, 0, s>>>(in, out, n, nullptr, total);
    LVG_CHECK_LAUNCH();
    return;
  }
  scan_reduce_kernel<T><<<unsigned(nb), SCAN_BLOCK, 0, s>>>(in, n, scratch);
  LVG_CHECK_LAUNCH();
  exclusive_scan_impl<T>(scratch, scratch, nb, nullptr, scratch + nb, s);
  scan_tile_kernel<T><<<unsigned(nb), SCAN_BLOCK, 0, s>>>(in, out, n, scratch, total);
  LVG_CHECK_LAUNCH();
}

// ------------------------------------------------------------------ binning

constexpr int BIN_THREADS = 256;

// Items of a graph union (gid != nullptr) take the class of their id within
// their own graph (gbase[g] = the graph's first item), so that each graph's
// classes are those it has alone.
__device__ __forceinline__ int bucket_of(size_t j, unsigned long long d, int colors, const uint32_t *gid,
                                         const uint32_t *gbase, const BinLimits &lim) {
  const uint32_t id = gid ? uint32_t(j) - gbase[gid[j]] : uint32_t(j);
  return int(vertex_color(id, uint32_t(colors))) * NUM_BINS + degree_bin(d, lim);
}

template <class D>
__global__ void __launch_bounds__(BIN_THREADS) bin_count_kernel(const D *deg, const uint8_t *ex, size_t n, int colors,
                                                                const uint32_t *gid, const uint32_t *gbase,
                                                                uint32_t *counts, unsigned long long *maxdeg,
                                                                unsigned nb, BinLimits lim) {
  __shared__ uint32_t cnt[MAX_BUCKETS];
  __shared__ unsigned long long mx[NUM_BINS];
  const int nbk = colors * NUM_BINS;
  for (int k = threadIdx.x; k < nbk; k += BIN_THREADS) cnt[k] = 0;
  if (threadIdx.x < NUM_BINS) mx[threadIdx.x] = 0;
  __syncthreads();
  size_t base = size_t(blockIdx.x) * BIN_CHUNK;
  for (int k = threadIdx.x; k < BIN_CHUNK; k += BIN_THREADS) {
    size_t j = base + k;
    if (j >= n || (ex && !ex[j])) continue;
    unsigned long long d = deg[j];
    atomicAdd(&cnt[bucket_of(j, d, colors, gid, gbase, lim)], 1u);
    atomicMax(&mx[degree_bin(d, lim)], d);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nbk; k += BIN_THREADS) counts[size_t(k) * nb + blockIdx.x] = cnt[k];
  if (threadIdx.x < NUM_BINS && mx[threadIdx.x]) atomicMax(&maxdeg[threadIdx.x], mx[threadIdx.x]);
}

template <class D>
__global__ void __launch_bounds__(BIN_THREADS) bin_scatter_kernel(const D *deg, const uint8_t *ex, size_t n,
                                                                  int colors, const uint32_t *gid,
                                                                  const uint32_t *gbase, const uint32_t *offs,
                                                                  unsigned nb, uint32_t *list, BinLimits lim) {
  constexpr int NW = BIN_THREADS / 32;
  __shared__ uint32_t wcnt[NW][MAX_BUCKETS];
  __shared__ uint32_t run[MAX_BUCKETS];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nbk = colors * NUM_BINS;
  for (int k = threadIdx.x; k < nbk; k += BIN_THREADS) run[k] = offs[size_t(k) * nb + blockIdx.x];
  size_t base = size_t(blockIdx.x) * BIN_CHUNK;
  for (int r = 0; r < BIN_CHUNK; r += BIN_THREADS) {
    for (int k = threadIdx.x; k < NW * nbk; k += BIN_THREADS) wcnt[k / nbk][k % nbk] = 0;
    __syncthreads();
    size_t j = base + r + threadIdx.x;
    int b = -1;
    if (j < n && (!ex || ex[j])) b = bucket_of(j, (unsigned long long)deg[j], colors, gid, gbase, lim);
    unsigned m = __match_any_sync(0xffffffffu, b);
    unsigned rank = __popc(m & ((1u << lane) - 1));
    if (b >= 0 && rank == 0) wcnt[wid][b] = __popc(m);
    __syncthreads();
    if (b >= 0) {
      uint32_t pos = run[b] + rank;
      for (int w2 = 0; w2 < wid; ++w2) pos += wcnt[w2][b];
      list[pos] = uint32_t(j);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nbk; k += BIN_THREADS) {
      uint32_t add = 0;
      for (int w2 = 0; w2 < NW; ++w2) add += wcnt[w2][k];
      run[k] += add;
    }
    __syncthreads();
  }
}

// Gather group starts (offs[k*nb]) and the total into out[0..nbk].
__global__ void bin_starts_kernel(const uint32_t *offs, unsigned nb, int nbk, const uint32_t *total, uint32_t *out) {
  for (int k = threadIdx.x; k <= nbk; k += blockDim.x) out[k] = k < nbk ? offs[size_t(k) * nb] : *total;
}

template <class D>
void bin_items_impl(const D *deg, const uint8_t *ex, size_t n, int colors, const uint32_t *gid,
                    const uint32_t *gbase, uint32_t *list, size_t *bin_start, uint64_t *bin_maxdeg, uint32_t *scratch,
                    uint32_t *host, cudaStream_t s, const BinLimits &lim) {
  const int nbk = colors * NUM_BINS;
  if (n == 0) {
    for (int b = 0; b <= nbk; ++b) bin_start[b] = 0;
    for (int b = 0; b < NUM_BINS; ++b) bin_maxdeg[b] = 0;
    return;
  }
  unsigned nb = unsigned((n + BIN_CHUNK - 1) / BIN_CHUNK);
  size_t nc = size_t(nbk) * nb;
  // scratch layout: maxdeg u64[NUM_BINS] | starts u32[nbk+1] | total u32 | counts u32[nc] | scan scratch
  unsigned long long *maxdeg = reinterpret_cast<unsigned long long *>(scratch);
  uint32_t *starts = scratch + 2 * NUM_BINS;
  uint32_t *total = starts + nbk + 1;
  uint32_t *counts = total + 1;
  uint32_t *sscratch = counts + nc;
  LVG_CUDA(cudaMemsetAsync(maxdeg, 0, NUM_BINS * sizeof(unsigned long long), s));
  bin_count_kernel<D><<<nb, BIN_THREADS, 0, s>>>(deg, ex, n, colors, gid, gbase, counts, maxdeg, nb, lim);
  LVG_CHECK_LAUNCH();
  exclusive_scan_impl<uint32_t>(counts, counts, nc, total, sscratch, s);
  bin_scatter_kernel<D><<<nb, BIN_THREADS, 0, s>>>(deg, ex, n, colors, gid, gbase, counts, nb, list, lim);
  LVG_CHECK_LAUNCH();
  bin_starts_kernel<<<1, 256, 0, s>>>(counts, nb, nbk, total, starts);
  LVG_CHECK_LAUNCH();
  // host mirror: maxdeg (2*NUM_BINS u32) then starts (nbk+1)
  LVG_CUDA(cudaMemcpyAsync(host, scratch, (2 * NUM_BINS + nbk + 1) * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  LVG_CUDA(cudaStreamSynchronize(s));
  const unsigned long long *hm = reinterpret_cast<const unsigned long long *>(host);
  const uint32_t *hs = host + 2 * NUM_BINS;
  for (int b = 0; b <= nbk; ++b) bin_start[b] = hs[b];
  for (int b = 0; b < NUM_BINS; ++b) bin_maxdeg[b] = hm[b];
}

}  // namespace

size_t scan_scratch_elems(size_t n) {
  size_t tot = 64;
  while (n > size_t(SCAN_TILE)) {
    n = (n + SCAN_TILE - 1) / SCAN_TILE;
    tot += n;
  }
  return tot + 64;
}

void exclusive_scan_u32(const uint32_t *in, uint32_t *out, size_t n, uint32_t *total, uint32_t *scratch,
                        cudaStream_t s) {
  exclusive_scan_impl<uint32_t>(in, out, n, total, scratch, s);
}

void exclusive_scan_u64(const uint64_t *in, uint64_t *out, size_t n, uint64_t *total, uint64_t *scratch,
                        cudaStream_t s) {
  exclusive_scan_impl<unsigned long long>(reinterpret_cast<const unsigned long long *>(in),
                                          reinterpret_cast<unsigned long long *>(out), n,
                                          reinterpret_cast<unsigned long long *>(total),
                                          reinterpret_cast<unsigned long long *>(scratch), s);
}

size_t bin_scratch_elems(size_t n, int colors) {
  size_t nb = (n + BIN_CHUNK - 1) / BIN_CHUNK;
  size_t nc = size_t(colors) * NUM_BINS * nb;
  return 2 * NUM_BINS + size_t(colors) * NUM_BINS + 2 + nc + scan_scratch_elems(nc) + 16;
}

size_t bin_host_elems(int colors) { return 2 * NUM_BINS + size_t(colors) * NUM_BINS + 8; }

void bin_items_u32(const uint32_t *deg, const uint8_t *ex, size_t n, int colors, uint32_t *list, size_t *bin_start,
                   uint64_t *bin_maxdeg, uint32_t *scratch, uint32_t *host_pinned, cudaStream_t s,
                   const uint32_t *gid, const uint32_t *gbase, const BinLimits &lim) {
  bin_items_impl<uint32_t>(deg, ex, n, colors, gid, gbase, list, bin_start, bin_maxdeg, scratch, host_pinned, s,
                           lim);
}

void bin_items_u64(const uint64_t *deg, const uint8_t *ex, size_t n, int colors, uint32_t *list, size_t *bin_start,
                   uint64_t *bin_maxdeg, uint32_t *scratch, uint32_t *host_pinned, cudaStream_t s) {
  bin_items_impl<unsigned long long>(reinterpret_cast<const unsigned long long *>(deg), ex, n, colors, nullptr,
                                     nullptr, list,
                                     bin_start, bin_maxdeg, scratch, host_pinned, s, default_bin_limits());
}

}  // namespace lvg
