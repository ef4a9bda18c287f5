// lvg_aggregate.cu — aggregation phase (replaces louvainAggregateEdgesOmpW
// and louvainAggregateOmpW, inc/louvain.hxx:897-912, 987-992).
//
// Input: a level, its renumbered membership, the community -> member CSR and
// the row capacity offsets yoff (exclusive scan of each community's total
// degree, as louvainCommunityTotalDegreeOmpW + scan do, inc/louvain.hxx:989-990).
// Each community merges the neighbour communities of all its members'
// edges, self-loops included (louvainScanCommunitiesW<true>), into a hash
// table sized by the community's total degree, then writes the distinct
// (community, summed weight) pairs to its row at yoff[c] and the row's degree
// to ydeg[c] (the reference's gapped DiGraphCsr). The super-vertex's weight
// (louvainVertexWeightsOmpW on the new level, :1209: the row sum, self-loop
// included) equals the community's total and is taken from the FP64 totals
// by the driver (launch_next_vertex_weights), not re-summed here.
//
// Communities are binned by total degree like vertices in the move kernels:
// sub-warp tiles / warps with shared tables for small communities, blocks
// with shared tables (and a global-memory fallback when a community has too
// many distinct neighbours) for large ones. Inside a tile, the members' edge
// lists are flattened with a tile prefix scan over member degrees, so lanes
// stay busy whatever the member degrees are. Internal edges (into the
// community itself, the hottest key) are summed privately per lane and added
// once.
#include "lvg_internal.cuh"

namespace lvg {
namespace {

__host__ __device__ constexpr int ilog2c(int x) { return x <= 1 ? 0 : 1 + ilog2c(x >> 1); }

template <int T>
__device__ __forceinline__ unsigned tile_mask() {
  if (T == 32) return 0xffffffffu;
  const int lane = threadIdx.x & 31;
  return ((1u << T) - 1u) << (lane & ~(T - 1));
}

template <class KP, class VP>
__device__ __forceinline__ bool table_add(KP keys, VP vals, int log2cap, uint32_t c, float w) {
  const uint32_t mask = (1u << log2cap) - 1u;
  uint32_t s = hash_hi(c, log2cap);
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    uint32_t k = keys[s];
    if (k == c) { atomicAdd(&vals[s], w); return true; }
    if (k == EMPTY) {
      uint32_t prev = atomicCAS(&keys[s], EMPTY, c);
      if (prev == EMPTY || prev == c) { atomicAdd(&vals[s], w); return true; }
    }
    s = (s + 1u) & mask;
  }
  return false;
}

// Warp-aggregated insert (the lanes holding the same key sum their weights
// in lane order; the lowest of them calls ins).
template <class Ins>
__device__ __forceinline__ bool agg_warp_insert(uint32_t c, float w, Ins ins) {
  const unsigned grp = __match_any_sync(0xffffffffu, c);
  const int lane = threadIdx.x & 31;
  const unsigned cnt = c == EMPTY ? 0u : unsigned(__popc(grp));
  const unsigned most = __reduce_max_sync(0xffffffffu, cnt);
  float sum = 0.f;
  unsigned rem = grp;
  for (unsigned it = 0; it < most; ++it) {
    const int src = rem ? __ffs(rem) - 1 : lane;
    rem &= rem - 1u;
    const float x = __shfl_sync(0xffffffffu, w, src);
    if (it < cnt) sum += x;
  }
  if (c != EMPTY && (grp & ((1u << lane) - 1u)) == 0u) return ins(c, sum);
  return true;
}

// Visit all edges of members cmem[m0..m1), T lanes cooperating (tile mask
// m). Edges into the community itself (`self`, the hottest key: every
// internal edge) are summed in the lane-private `self_w`; the others go to
// `add(key, weight)`, which returns false to stop early. Returns edges read.
template <int T, class Add>
__device__ __forceinline__ uint64_t visit_members(const AggArgs &a, uint32_t m0, uint32_t m1, int tl, unsigned m,
                                                  uint32_t self, float &self_w, Add add) {
  uint64_t nread = 0;
  bool go = true;
  for (uint32_t base = m0; base < m1; base += T) {
    const uint32_t mm = base + tl;
    uint32_t dg = 0;
    uint64_t o = 0;
    if (mm < m1) {
      const uint32_t u = a.cmem[mm];
      dg = a.deg[u];
      o = a.off[u];
    }
    uint32_t incl = dg;
#pragma unroll
    for (int sh = 1; sh < T; sh <<= 1) {
      uint32_t t = __shfl_up_sync(m, incl, sh, T);
      if (tl >= sh) incl += t;
    }
    const uint32_t total = __shfl_sync(m, incl, T - 1, T);
    nread += total;
    for (uint32_t k0 = 0; k0 < total; k0 += T) {
      const uint32_t k = k0 + tl;
      // owner lane: first lane whose inclusive prefix exceeds k
      int lo = 0, hi = T - 1;
#pragma unroll
      for (int step = 0; step < ilog2c(T); ++step) {
        const int mid = (lo + hi) >> 1;
        const uint32_t x = __shfl_sync(m, incl, mid, T);
        if (x <= k) lo = mid + 1; else hi = mid;
      }
      const uint32_t oincl = __shfl_sync(m, incl, lo, T);
      const uint32_t odeg = __shfl_sync(m, dg, lo, T);
      const uint64_t oo = __shfl_sync(m, o, lo, T);
      uint32_t c = EMPTY;
      float w = 0.f;
      if (go && k < total) {
        const uint64_t e = oo + (k - (oincl - odeg));
        c = a.vcom[a.key[e]];
        w = a.w[e];
        if (c == self) { self_w += w; c = EMPTY; }
      }
      if constexpr (T == 32) {
        // a whole warp: lanes holding the same community add once
        go = __all_sync(0xffffffffu, agg_warp_insert(c, w, add)) && go;
      } else {
        if (c != EMPTY) go = add(c, w);
      }
    }
  }
  return nread;
}

constexpr int TILE_BLOCK = 256;

template <int T, int C>
__global__ void __launch_bounds__(TILE_BLOCK) agg_tile_kernel(AggArgs a) {
  constexpr int LOGC = ilog2c(C);
  constexpr int TPB = TILE_BLOCK / T;
  extern __shared__ __align__(16) uint8_t smem[];
  const int tib = threadIdx.x / T;
  const int tl = threadIdx.x & (T - 1);
  const int lane = threadIdx.x & 31;
  uint32_t *keys = reinterpret_cast<uint32_t *>(smem) + tib * C;
  float *vals = reinterpret_cast<float *>(smem + size_t(TPB) * C * sizeof(uint32_t)) + tib * C;
  const unsigned m = tile_mask<T>();
  const uint32_t ntiles = gridDim.x * TPB;
  unsigned long long nread = 0;
  bool ok = true;
  for (uint32_t i = blockIdx.x * TPB + tib; i < a.count; i += ntiles) {
    const uint32_t c = a.list[i];
    const uint32_t m0 = a.coff[c], m1 = a.coff[c + 1];
#pragma unroll
    for (int s = tl; s < C; s += T) { keys[s] = EMPTY; vals[s] = 0.f; }
    __syncwarp(m);
    float self_w = 0.f;
    nread += visit_members<T>(a, m0, m1, tl, m, c, self_w, [&](uint32_t k, float w) {
      ok &= table_add(keys, vals, LOGC, k, w);
      return true;
    });
#pragma unroll
    for (int sh = T / 2; sh > 0; sh >>= 1) self_w += __shfl_xor_sync(m, self_w, sh, T);
    __syncwarp(m);
    if (tl == 0 && self_w != 0.f) ok &= table_add(keys, vals, LOGC, c, self_w);
    __syncwarp(m);
    const uint64_t y0 = a.yoff[c];
    uint32_t cnt = 0;
#pragma unroll
    for (int s0 = 0; s0 < C; s0 += T) {
      const int s = s0 + tl;
      const uint32_t k = keys[s];
      const bool has = k != EMPTY;
      const unsigned bal = (__ballot_sync(m, has) >> (lane & ~(T - 1))) & (T == 32 ? 0xffffffffu : ((1u << T) - 1u));
      if (has) {
        const uint32_t r = __popc(bal & ((1u << tl) - 1u));
        const float v = vals[s];
        a.ykey[y0 + cnt + r] = k;
        a.yw[y0 + cnt + r] = v;
      }
      cnt += __popc(bal);
    }
    if (tl == 0) a.ydeg[c] = cnt;
    __syncwarp(m);
  }
  if (tl != 0) nread = 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nread += __shfl_xor_sync(0xffffffffu, nread, o);
  const bool bad = __any_sync(0xffffffffu, !ok);
  if (lane == 0) {
    if (nread) atomicAdd(&a.ctr->agg_edges, nread);
    if (bad) atomicOr(&a.ctr->err, ERR_TABLE_FULL);
  }
}

__device__ __forceinline__ bool smem_add_budget(uint32_t *keys, float *vals, int log2cap, uint32_t c, float w,
                                                unsigned *used, unsigned limit) {
  const uint32_t mask = (1u << log2cap) - 1u;
  uint32_t s = hash_hi(c, log2cap);
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    uint32_t k = keys[s];
    if (k == c) { atomicAdd(&vals[s], w); return true; }
    if (k == EMPTY) {
      if (atomicAdd(used, 1u) >= limit) return false;
      uint32_t prev = atomicCAS(&keys[s], EMPTY, c);
      if (prev == EMPTY || prev == c) { atomicAdd(&vals[s], w); return true; }
    }
    s = (s + 1u) & mask;
  }
  return false;
}

// One block per community (total degree > 512); each warp flattens a
// 32-member chunk at a time. The community is merged in a shared table of
// 2^LOGS slots with a claim budget (half the slots); a community with more
// distinct neighbour communities is redone with a table in its block's
// region of global memory (2^a.glog2 slots). The table holds
// min(total degree, community count) * 2 slots rounded up to a power of two.
template <int B, int LOGS>
__global__ void __launch_bounds__(B) agg_block_kernel(AggArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ uint32_t s_cnt;
  __shared__ unsigned s_used;
  __shared__ int s_over;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t *skeys = reinterpret_cast<uint32_t *>(smem);
  float *svals = reinterpret_cast<float *>(smem + (size_t(1) << LOGS) * sizeof(uint32_t));
  uint32_t *gkeys = a.gkeys ? a.gkeys + (size_t(blockIdx.x) << a.glog2) : nullptr;
  float *gvals = a.gvals ? a.gvals + (size_t(blockIdx.x) << a.glog2) : nullptr;
  unsigned long long nread = 0;
  bool ok = true;
  for (uint32_t i = blockIdx.x; i < a.count; i += gridDim.x) {
    const uint32_t c = a.list[i];
    const uint32_t m0 = a.coff[c], m1 = a.coff[c + 1];
    const uint64_t y0 = a.yoff[c], tdeg = a.yoff[c + 1] - y0;
    const uint64_t want = 2ull * (tdeg < a.cn ? tdeg : a.cn);
    int lg = min(LOGS, max(1, ceil_log2(want)));
    uint32_t ccap = 1u << lg;
    for (uint32_t s = threadIdx.x; s < ccap; s += B) { skeys[s] = EMPTY; svals[s] = 0.f; }
    if (threadIdx.x == 0) { s_cnt = 0; s_used = 0; s_over = 0; }
    __syncthreads();
    const unsigned limit = ccap >> 1;
    float self_w = 0.f;
    uint64_t nr = 0;
    for (uint32_t b0 = m0 + uint32_t(wid) * 32; b0 < m1; b0 += B) {
      const uint32_t b1 = b0 + 32 < m1 ? b0 + 32 : m1;
      nr += visit_members<32>(a, b0, b1, lane, 0xffffffffu, c, self_w, [&](uint32_t k, float w) {
        if (smem_add_budget(skeys, svals, lg, k, w, &s_used, limit)) return true;
        s_over = 1;
        return false;
      });
    }
    __syncthreads();
    uint32_t *keys = skeys;
    float *vals = svals;
    if (s_over) {
      lg = min(a.glog2, max(1, ceil_log2(want)));
      ccap = 1u << lg;
      keys = gkeys;
      vals = gvals;
      if (!keys) { ok = false; ccap = 0; }
      for (uint32_t s = threadIdx.x; s < ccap; s += B) { keys[s] = EMPTY; vals[s] = 0.f; }
      __syncthreads();
      self_w = 0.f;
      nr = 0;
      if (keys)
        for (uint32_t b0 = m0 + uint32_t(wid) * 32; b0 < m1; b0 += B) {
          const uint32_t b1 = b0 + 32 < m1 ? b0 + 32 : m1;
          nr += visit_members<32>(a, b0, b1, lane, 0xffffffffu, c, self_w, [&](uint32_t k, float w) {
            ok &= table_add(keys, vals, lg, k, w);
            return true;
          });
        }
    }
    nread += nr;
    // internal weight: one insertion per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) self_w += __shfl_xor_sync(0xffffffffu, self_w, o);
    if (lane == 0 && self_w != 0.f && ccap) ok &= table_add(keys, vals, lg, c, self_w);
    __syncthreads();
    for (uint32_t s0 = 0; s0 < ccap; s0 += B) {
      const uint32_t s = s0 + threadIdx.x;
      const uint32_t k = s < ccap ? keys[s] : EMPTY;
      const bool has = k != EMPTY;
      const unsigned bal = __ballot_sync(0xffffffffu, has);
      uint32_t base = 0;
      if (lane == 0 && bal) base = atomicAdd(&s_cnt, uint32_t(__popc(bal)));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (has) {
        const uint32_t r = __popc(bal & ((1u << lane) - 1u));
        const float v = vals[s];
        a.ykey[y0 + base + r] = k;
        a.yw[y0 + base + r] = v;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) a.ydeg[c] = s_cnt;
    __syncthreads();
  }
  if (lane != 0) nread = 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nread += __shfl_xor_sync(0xffffffffu, nread, o);
  const bool bad = __any_sync(0xffffffffu, !ok);
  if (lane == 0) {
    if (nread) atomicAdd(&a.ctr->agg_edges, nread);
    if (bad) atomicOr(&a.ctr->err, ERR_TABLE_FULL);
  }
}

// ------------------------------------------------------------ communities above total degree 8192
//
// A community's members' edges, flattened in member order, are the range
// [mpre[m0], mpre[m1]) of the member-degree prefix mpre. The largest
// communities (after the first pass of a power-law graph, a handful hold
// most of the edges) are cut into AGG_CHUNK-edge chunks, one block each; a
// block merges its chunk in a listed shared table with warp-aggregated
// inserts and adds the distinct (community, weight) pairs to the community's
// table in global memory, which agg_gfinish_kernel then writes out as the
// community's row. Each block finds the member of every edge of a batch by a
// binary search over the batch's window of member prefixes in shared memory.

template <int B, int LOGS>
__global__ void __launch_bounds__(B) agg_chunk_kernel(AggArgs a, AggChunks ch) {
  extern __shared__ __align__(16) uint8_t smem[];
  constexpr uint32_t CS = 1u << LOGS;
  __shared__ uint64_t win[B + 1];
  __shared__ unsigned s_used;
  __shared__ uint32_t s_mi;
  uint32_t *skeys = reinterpret_cast<uint32_t *>(smem);
  float *svals = reinterpret_cast<float *>(smem + size_t(CS) * 4);
  uint32_t *slist = reinterpret_cast<uint32_t *>(smem + size_t(CS) * 8);
  for (uint32_t s2 = threadIdx.x; s2 < CS; s2 += B) { skeys[s2] = EMPTY; svals[s2] = 0.f; }
  const uint2 cj = ch.chunk[blockIdx.x];  // (community slot, chunk index)
  const uint32_t j = cj.x;
  const uint32_t c = ch.comm[j];
  const uint32_t m0 = a.coff[c], m1 = a.coff[c + 1];
  const uint64_t ebeg = ch.mpre[m0], eend = ch.mpre[m1];
  const uint64_t e0 = ebeg + uint64_t(cj.y) * AGG_CHUNK;
  const uint64_t e1 = min(eend, e0 + AGG_CHUNK);
  uint32_t *gk = ch.gkeys + ch.toff[j];
  float *gv = ch.gvals + ch.toff[j];
  const int glg = ch.tlog[j];
  const unsigned limit = CS >> 1;
  if (threadIdx.x == 0) {
    s_used = 0;
    // the member holding edge e0: the last m in [m0, m1) with mpre[m] <= e0
    uint32_t lo = m0, hi = m1 - 1;
    while (lo < hi) {
      const uint32_t mid = lo + (hi - lo + 1) / 2;
      if (ch.mpre[mid] <= e0) lo = mid; else hi = mid - 1;
    }
    s_mi = lo;
  }
  __syncthreads();
  unsigned long long nread = 0;
  bool ok = true;
  uint64_t base = e0;
  while (base < e1) {  // block-uniform
    const uint32_t mi = s_mi;
    const uint32_t nw = min(uint32_t(B), m1 - mi);  // members staged: mi .. mi+nw-1
    for (uint32_t t = threadIdx.x; t <= nw; t += B) win[t] = ch.mpre[mi + t];
    __syncthreads();
    // this pass of the loop: edges [base, stop), all inside the staged members
    const uint64_t stop = min(e1, min(base + B, win[nw]));
    const uint64_t e = base + threadIdx.x;
    uint32_t key = EMPTY;
    float w = 0.f;
    if (e < stop) {
      uint32_t lo = 0, hi = nw - 1;  // last window entry <= e
      while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (win[mid] <= e) lo = mid; else hi = mid - 1;
      }
      const uint32_t u = a.cmem[mi + lo];
      const uint64_t x = a.off[u] + (e - win[lo]);
      key = a.vcom[__ldcs(a.key + x)];
      w = __ldcs(a.w + x);
      ++nread;
    }
    agg_warp_insert(key, w, [&](uint32_t k, float v) {
      // the shared table while its claim budget lasts, then the global one
      const uint32_t mask = CS - 1u;
      uint32_t sl = hash_hi(k, LOGS);
      for (uint32_t probe = 0; probe <= mask; ++probe) {
        const uint32_t kk = skeys[sl];
        if (kk == k) { atomicAdd(&svals[sl], v); return true; }
        if (kk == EMPTY) {
          const unsigned r = atomicAdd(&s_used, 1u);
          if (r >= limit) break;
          const uint32_t prev = atomicCAS(&skeys[sl], EMPTY, k);
          if (prev == EMPTY) { slist[r] = sl; atomicAdd(&svals[sl], v); return true; }
          slist[r] = EMPTY;
          if (prev == k) { atomicAdd(&svals[sl], v); return true; }
        }
        sl = (sl + 1u) & mask;
      }
      ok &= table_add(gk, gv, glg, k, v);
      return true;
    });
    __syncthreads();  // every thread has read win[] and s_mi
    // the next round starts at the member holding edge `stop`
    if (threadIdx.x == 0) {
      if (stop < win[nw]) {
        uint32_t lo = 0, hi = nw - 1;
        while (lo < hi) {
          const uint32_t mid = (lo + hi + 1) >> 1;
          if (win[mid] <= stop) lo = mid; else hi = mid - 1;
        }
        s_mi = mi + lo;
      } else {
        s_mi = mi + nw;  // past the staged members (also when they had no edges left)
      }
    }
    base = stop;
    __syncthreads();
  }
  // the shared table into the community's global table
  const unsigned nl = min(s_used, limit);
  for (unsigned i = threadIdx.x; i < nl; i += B) {
    const uint32_t sl = slist[i];
    if (sl != EMPTY) ok &= table_add(gk, gv, glg, skeys[sl], svals[sl]);
  }
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) nread += __shfl_xor_sync(0xffffffffu, nread, o);
  const bool bad = __any_sync(0xffffffffu, !ok);
  if (lane == 0) {
    if (nread) atomicAdd(&a.ctr->agg_edges, nread);
    if (bad) atomicOr(&a.ctr->err, ERR_TABLE_FULL);
  }
}

// The global tables of the chunked communities into their rows: a thread
// per slot, output positions by a warp-aggregated cursor per community
// (ydeg).
__global__ void agg_gfinish_kernel(AggArgs a, AggChunks ch, uint64_t slots) {
  const int lane = threadIdx.x & 31;
  for (uint64_t base = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32 * 32; base < slots;
       base += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t t = base + lane;
    uint32_t jj = EMPTY, k = EMPTY;
    float v = 0.f;
    if (t < slots) {
      uint32_t lo = 0, hi = ch.n - 1;  // the community whose region holds slot t
      while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (ch.toff[mid] <= t) lo = mid; else hi = mid - 1;
      }
      k = ch.gkeys[t];
      if (k != EMPTY) { jj = lo; v = ch.gvals[t]; }
    }
    const unsigned grp = __match_any_sync(0xffffffffu, jj);
    const int leader = __ffs(grp) - 1;
    uint32_t at = 0;
    const uint32_t c = jj != EMPTY ? ch.comm[jj] : 0u;
    if (jj != EMPTY && lane == leader) at = atomicAdd(&a.ydeg[c], uint32_t(__popc(grp)));
    at = __shfl_sync(grp, at, leader);
    if (jj != EMPTY) {
      const uint64_t y = a.yoff[c] + at + __popc(grp & ((1u << lane) - 1u));
      a.ykey[y] = k;
      a.yw[y] = v;
    }
  }
}

__global__ void comm_tdeg_kernel(const uint32_t *list, size_t n, const uint64_t *yoff, uint64_t *out) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    out[i] = yoff[list[i] + 1] - yoff[list[i]];
}

__global__ void member_degrees_kernel(const uint32_t *cmem, const uint32_t *deg, size_t n, uint64_t *dst) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    dst[i] = deg[cmem[i]];
}

int sms() {  // SM count of the device, queried once (thread-safe static init)
  static const int n = [] {
    int dev = 0, c = 0;
    LVG_CUDA(cudaGetDevice(&dev));
    LVG_CUDA(cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev));
    return c;
  }();
  return n;
}

template <class K>
void set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) LVG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
}

template <int T, int C>
void launch_tile(const AggArgs &a, cudaStream_t s) {
  constexpr int TPB = TILE_BLOCK / T;
  const size_t smem = size_t(TPB) * C * 8;
  auto k = agg_tile_kernel<T, C>;
  static bool configured = false;
  if (!configured) { set_smem(k, smem); configured = true; }
  size_t want = (a.count + TPB - 1) / TPB;
  size_t cap = size_t(sms()) * (smem > 32 * 1024 ? 3 : 8);
  unsigned grid = unsigned(want < cap ? want : cap);
  if (!grid) return;
  k<<<grid, TILE_BLOCK, smem, s>>>(a);
  LVG_CHECK_LAUNCH();
}

template <int B, int LOGS>
void launch_big(const AggArgs &a, cudaStream_t s) {
  const size_t smem = (size_t(1) << LOGS) * 8;
  auto k = agg_block_kernel<B, LOGS>;
  static bool configured = false;
  if (!configured) { set_smem(k, smem); configured = true; }
  unsigned grid = unsigned(global_table_blocks(a.count));
  if (!grid) return;
  k<<<grid, B, smem, s>>>(a);
  LVG_CHECK_LAUNCH();
}

}  // namespace

void launch_comm_tdeg(const uint32_t *list, size_t n, const uint64_t *yoff, uint64_t *out, cudaStream_t s) {
  if (!n) return;
  comm_tdeg_kernel<<<grid_for(n, 256), 256, 0, s>>>(list, n, yoff, out);
  LVG_CHECK_LAUNCH();
}

void launch_member_degrees(const uint32_t *cmem, const uint32_t *deg, size_t n, uint64_t *dst, cudaStream_t s) {
  if (!n) return;
  member_degrees_kernel<<<grid_for(n, 256), 256, 0, s>>>(cmem, deg, n, dst);
  LVG_CHECK_LAUNCH();
}

constexpr int AGG_CHUNK_B = 256, AGG_CHUNK_LOGS = 11;

void launch_aggregate_chunks(const AggArgs &a, const AggChunks &ch, size_t chunks, uint64_t slots, cudaStream_t s) {
  if (!chunks) return;
  const size_t smem = (size_t(1) << AGG_CHUNK_LOGS) * 10;  // keys, values, claimed list
  agg_chunk_kernel<AGG_CHUNK_B, AGG_CHUNK_LOGS><<<unsigned(chunks), AGG_CHUNK_B, smem, s>>>(a, ch);
  LVG_CHECK_LAUNCH();
  agg_gfinish_kernel<<<grid_for(slots, 256), 256, 0, s>>>(a, ch, slots);
  LVG_CHECK_LAUNCH();
}

void launch_aggregate_bin(int b, const AggArgs &a, cudaStream_t s) {
  switch (b) {
    case 1: launch_tile<4, 8>(a, s); break;
    case 2: launch_tile<8, 16>(a, s); break;
    case 3: launch_tile<16, 32>(a, s); break;
    case 4: launch_tile<32, 64>(a, s); break;
    case 5: launch_tile<32, 128>(a, s); break;
    case 6: launch_tile<32, 256>(a, s); break;
    case 7: launch_tile<32, 512>(a, s); break;
    case 8: launch_tile<32, 1024>(a, s); break;
    case 9: launch_big<256, 12>(a, s); break;
    case 10: launch_big<512, 13>(a, s); break;
    case 11: launch_big<512, 13>(a, s); break;
    default: break;
  }
}

}  // namespace lvg
