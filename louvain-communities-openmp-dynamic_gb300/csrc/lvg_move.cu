// lvg_move.cu — local-moving phase (replaces louvainMoveOmpW,
// inc/louvain.hxx:588-609, with louvainScanCommunitiesW :423,
// louvainChooseCommunity :455 and louvainChangeCommunityOmpW :496).
//
// The reference gives each OpenMP thread a dense span-sized table and walks
// all vertices. Here vertices are grouped by degree and each group gets the
// cheapest table that fits:
//   bins 1-4  (degree <= 4/8/16/32): a tile of 4/8/16/32 lanes per vertex, a
//             shared-memory open-addressing table of 2x the tile size;
//   bins 5-8  (degree <= 64..512):   one warp per vertex, shared table of
//             128..1024 slots;
//   bins 9-10 (degree <= 2048/8192): one block per vertex, shared table of
//             4096 / 16384 slots;
//   bin 11    (larger hubs):         one block per vertex, table in global
//             memory (a per-block region of HBM, L2 resident when it fits).
// Per vertex: clear the table, insert (community of each neighbour, weight)
// for neighbours outside the vertex's own community (the own community's
// weight is a lane-private sum), compute the FP32 gain of each candidate,
// take the tile/block argmax (largest gain, then lowest id), and move with two
// atomic updates of the community totals. A moved vertex marks its neighbours
// affected; every processed vertex clears its own flag.
//
// Asynchronous mode (the reference's semantics) reads and writes membership,
// totals and flags in place. Deterministic mode only records each vertex's
// decision (dec[u]) and its neighbour marks (mark[]); the caller applies the
// decisions of a colour class after all of them were taken.
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

// Insert (c, w) into an open-addressing table of 2^log2cap slots (linear
// probing). The probe count is bounded by the capacity; false = table full,
// which cannot happen while capacity >= 2 x degree (checked by the caller's
// bin choice) and is reported as an error flag if it ever does.
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

__device__ __forceinline__ void take_better(float &bg, uint32_t &bc, float og, uint32_t oc) {
  if (better(og, oc, bg, bc)) { bg = og; bc = oc; }
}

__device__ __forceinline__ void flush_counters(Counters *ctr, int bin, unsigned long long fix, unsigned long long nv,
                                               unsigned long long ne, unsigned long long nm, bool bad) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    fix += __shfl_xor_sync(0xffffffffu, fix, o);
    nv += __shfl_xor_sync(0xffffffffu, nv, o);
    ne += __shfl_xor_sync(0xffffffffu, ne, o);
    nm += __shfl_xor_sync(0xffffffffu, nm, o);
  }
  bool anybad = __any_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0) {
    if (fix) atomicAdd(&ctr->el_fix, fix);
    if (nv) { atomicAdd(&ctr->vertices, nv); atomicAdd(&ctr->bin_vertices[bin], nv); }
    if (ne) { atomicAdd(&ctr->edges, ne); atomicAdd(&ctr->bin_edges[bin], ne); }
    if (nm) atomicAdd(&ctr->moves, nm);
    if (anybad) atomicOr(&ctr->err, ERR_TABLE_FULL);
  }
}

// ------------------------------------------------------------ tile / warp kernel

constexpr int TILE_BLOCK = 256;

template <int T, int C, bool SYNC>
__global__ void __launch_bounds__(TILE_BLOCK) move_tile_kernel(MoveArgs a) {
  constexpr int LOGC = ilog2c(C);
  constexpr int TPB = TILE_BLOCK / T;
  extern __shared__ __align__(16) uint8_t smem[];
  const int tib = threadIdx.x / T;
  const int tl = threadIdx.x & (T - 1);
  uint32_t *keys = reinterpret_cast<uint32_t *>(smem) + tib * C;
  float *vals = reinterpret_cast<float *>(smem + size_t(TPB) * C * sizeof(uint32_t)) + tib * C;
  const unsigned m = tile_mask<T>();
  const uint32_t ntiles = gridDim.x * TPB;
  unsigned long long fix = 0, nv = 0, ne = 0, nm = 0;
  bool bad = false;
  for (uint32_t i = blockIdx.x * TPB + tib; i < a.count; i += ntiles) {
    const uint32_t u = a.list[i];
    int act = 0;
    if (tl == 0) act = a.vaff[u] && (!a.fa || a.fa[u]);
    act = __shfl_sync(m, act, 0, T);
    if (!act) continue;
    const uint64_t o = a.off[u];
    const uint32_t dg = a.deg[u];
    const uint32_t d = a.vcom[u];
#pragma unroll
    for (int s = tl; s < C; s += T) { keys[s] = EMPTY; vals[s] = 0.f; }
    __syncwarp(m);
    float kd = 0.f;
    bool ok = true;
    for (uint32_t j = tl; j < dg; j += T) {
      const uint32_t v = a.key[o + j];
      if (v == u) continue;
      const float ww = a.w[o + j];
      const uint32_t c = a.vcom[v];
      if (c == d) kd += ww;
      else ok &= table_add(keys, vals, LOGC, c, ww);
    }
#pragma unroll
    for (int sh = T / 2; sh > 0; sh >>= 1) kd += __shfl_xor_sync(m, kd, sh, T);
    __syncwarp(m);
    float wu = 0.f, td = 0.f;
    if (tl == 0) { wu = a.vtot[u]; td = a.ctot[d]; }
    wu = __shfl_sync(m, wu, 0, T);
    td = __shfl_sync(m, td, 0, T);
    float bg = 0.f;
    uint32_t bc = EMPTY;
#pragma unroll
    for (int s = tl; s < C; s += T) {
      const uint32_t c = keys[s];
      if (c == EMPTY) continue;
      const float g = gain_f32(vals[s], kd, wu, a.ctot[c], td, a.kr);
      if (g > 0.f) take_better(bg, bc, g, c);
    }
#pragma unroll
    for (int sh = T / 2; sh > 0; sh >>= 1) {
      const float og = __shfl_xor_sync(m, bg, sh, T);
      const uint32_t oc = __shfl_xor_sync(m, bc, sh, T);
      take_better(bg, bc, og, oc);
    }
    const bool moved = bc != EMPTY && bc != 0;
    if (tl == 0) {
      if (bc != EMPTY) fix += gain_to_fix(bg);
      if (moved) {
        if (SYNC) {
          a.dec[u] = bc;
        } else {
          atomicAdd(&a.ctot[d], -wu);
          atomicAdd(&a.ctot[bc], wu);
          a.vcom[u] = bc;
        }
      }
    }
    if (moved) {
      uint8_t *mk = SYNC ? a.mark : a.vaff;
      for (uint32_t j = tl; j < dg; j += T) {
        const uint32_t v = a.key[o + j];
        if (v != u) mk[v] = 1;
      }
    }
    if (tl == 0) {
      a.vaff[u] = 0;
      ++nv;
      ne += dg;
      nm += moved;
    }
    bad |= !ok;
    __syncwarp(m);
  }
  flush_counters(a.ctr, a.bin, fix, nv, ne, nm, bad);
}

// ------------------------------------------------------------ block kernel

template <int B>
__device__ __forceinline__ float block_sum(float v, float *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  float t = 0.f;
  for (int k = 0; k < B / 32; ++k) t += red[k];
  __syncthreads();
  return t;
}

template <int B>
__device__ __forceinline__ void block_argmax(float &bg, uint32_t &bc, float *rg, uint32_t *rc) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float og = __shfl_xor_sync(0xffffffffu, bg, o);
    const uint32_t oc = __shfl_xor_sync(0xffffffffu, bc, o);
    take_better(bg, bc, og, oc);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { rg[wid] = bg; rc[wid] = bc; }
  __syncthreads();
  bg = 0.f;
  bc = EMPTY;
  for (int k = 0; k < B / 32; ++k) take_better(bg, bc, rg[k], rc[k]);
  __syncthreads();
}

// One block per vertex. GLOBAL = table in global memory (bin 11), else in
// dynamic shared memory; the block's region holds 2^log2cap slots and each
// vertex uses the smallest power of two >= 2x its degree.
template <int B, bool GLOBAL, bool SYNC>
__global__ void __launch_bounds__(B) move_block_kernel(MoveArgs a, int log2cap) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ float red_g[B / 32];
  __shared__ uint32_t red_c[B / 32];
  __shared__ int s_act;
  const uint32_t cap = 1u << log2cap;
  uint32_t *keys;
  float *vals;
  if (GLOBAL) {
    keys = a.gkeys + size_t(blockIdx.x) * cap;
    vals = a.gvals + size_t(blockIdx.x) * cap;
  } else {
    keys = reinterpret_cast<uint32_t *>(smem);
    vals = reinterpret_cast<float *>(smem + size_t(cap) * sizeof(uint32_t));
  }
  unsigned long long fix = 0, nv = 0, ne = 0, nm = 0;
  bool bad = false;
  for (uint32_t i = blockIdx.x; i < a.count; i += gridDim.x) {
    const uint32_t u = a.list[i];
    if (threadIdx.x == 0) s_act = a.vaff[u] && (!a.fa || a.fa[u]);
    __syncthreads();
    const int act = s_act;
    __syncthreads();
    if (!act) continue;
    const uint64_t o = a.off[u];
    const uint32_t dg = a.deg[u];
    const uint32_t d = a.vcom[u];
    const int lg = min(log2cap, max(1, ceil_log2(2ull * dg)));
    const uint32_t vcap = 1u << lg;
    for (uint32_t s = threadIdx.x; s < vcap; s += B) { keys[s] = EMPTY; vals[s] = 0.f; }
    __syncthreads();
    float kd = 0.f;
    bool ok = true;
    for (uint32_t j = threadIdx.x; j < dg; j += B) {
      const uint32_t v = a.key[o + j];
      if (v == u) continue;
      const float ww = a.w[o + j];
      const uint32_t c = a.vcom[v];
      if (c == d) kd += ww;
      else ok &= table_add(keys, vals, lg, c, ww);
    }
    kd = block_sum<B>(kd, red_g);  // includes a barrier: table complete
    const float wu = a.vtot[u];
    const float td = a.ctot[d];
    float bg = 0.f;
    uint32_t bc = EMPTY;
    for (uint32_t s = threadIdx.x; s < vcap; s += B) {
      const uint32_t c = keys[s];
      if (c == EMPTY) continue;
      const float g = gain_f32(vals[s], kd, wu, a.ctot[c], td, a.kr);
      if (g > 0.f) take_better(bg, bc, g, c);
    }
    block_argmax<B>(bg, bc, red_g, red_c);
    const bool moved = bc != EMPTY && bc != 0;
    if (threadIdx.x == 0) {
      if (bc != EMPTY) fix += gain_to_fix(bg);
      if (moved) {
        if (SYNC) {
          a.dec[u] = bc;
        } else {
          atomicAdd(&a.ctot[d], -wu);
          atomicAdd(&a.ctot[bc], wu);
          a.vcom[u] = bc;
        }
      }
    }
    if (moved) {
      uint8_t *mk = SYNC ? a.mark : a.vaff;
      for (uint32_t j = threadIdx.x; j < dg; j += B) {
        const uint32_t v = a.key[o + j];
        if (v != u) mk[v] = 1;
      }
    }
    if (threadIdx.x == 0) {
      a.vaff[u] = 0;
      ++nv;
      ne += dg;
      nm += moved;
    }
    bad |= !ok;
    __syncthreads();
  }
  flush_counters(a.ctr, a.bin, fix, nv, ne, nm, bad);
}

int g_num_sms = 0;
int num_sms() {
  if (!g_num_sms) {
    int dev = 0;
    LVG_CUDA(cudaGetDevice(&dev));
    LVG_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
  }
  return g_num_sms;
}

template <class K>
void set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) LVG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
}

template <int T, int C, bool SYNC>
void launch_tile(const MoveArgs &a, cudaStream_t s) {
  constexpr int TPB = TILE_BLOCK / T;
  const size_t smem = size_t(TPB) * C * 8;
  auto k = move_tile_kernel<T, C, SYNC>;
  static bool configured = false;
  if (!configured) { set_smem(k, smem); configured = true; }
  size_t want = (a.count + TPB - 1) / TPB;
  size_t cap = size_t(num_sms()) * (smem > 32 * 1024 ? 3 : 8);
  unsigned grid = unsigned(want < cap ? want : cap);
  if (!grid) return;
  k<<<grid, TILE_BLOCK, smem, s>>>(a);
  LVG_CHECK_LAUNCH();
}

template <int B, int LOGC, bool SYNC>
void launch_block_smem(const MoveArgs &a, cudaStream_t s) {
  const size_t smem = (size_t(1) << LOGC) * 8;
  auto k = move_block_kernel<B, false, SYNC>;
  static bool configured = false;
  if (!configured) { set_smem(k, smem); configured = true; }
  size_t cap = size_t(num_sms()) * (smem > 64 * 1024 ? 1 : 2);
  unsigned grid = unsigned(a.count < cap ? a.count : cap);
  if (!grid) return;
  k<<<grid, B, smem, s>>>(a, LOGC);
  LVG_CHECK_LAUNCH();
}

template <bool SYNC>
void launch_bin(int b, const MoveArgs &a, cudaStream_t s) {
  switch (b) {
    case 1: launch_tile<4, 8, SYNC>(a, s); break;
    case 2: launch_tile<8, 16, SYNC>(a, s); break;
    case 3: launch_tile<16, 32, SYNC>(a, s); break;
    case 4: launch_tile<32, 64, SYNC>(a, s); break;
    case 5: launch_tile<32, 128, SYNC>(a, s); break;
    case 6: launch_tile<32, 256, SYNC>(a, s); break;
    case 7: launch_tile<32, 512, SYNC>(a, s); break;
    case 8: launch_tile<32, 1024, SYNC>(a, s); break;
    case 9: launch_block_smem<256, 12, SYNC>(a, s); break;
    case 10: launch_block_smem<512, 14, SYNC>(a, s); break;
    case 11: {
      unsigned grid = unsigned(global_table_blocks(a.count));
      if (!grid) return;
      move_block_kernel<512, true, SYNC><<<grid, 512, 0, s>>>(a, a.glog2);
      LVG_CHECK_LAUNCH();
      break;
    }
    default: break;
  }
}

}  // namespace

int global_table_blocks(size_t count) {
  size_t cap = size_t(num_sms()) * 2;
  return int(count < cap ? count : cap);
}

void launch_move_bin(int b, bool sync, const MoveArgs &a, cudaStream_t s) {
  if (sync) launch_bin<true>(b, a, s);
  else launch_bin<false>(b, a, s);
}

}  // namespace lvg
