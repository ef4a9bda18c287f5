// lvg_hubtab.cu — resident hub tables: building them from a membership, and
// the updates that are not made by the local-moving kernels themselves
// (deterministic mode's decided moves, a batch's edges).
//
// A hub (a vertex above degree 8192) costs the local-moving phase a scan of
// all of its edges every time it is evaluated, to count its neighbours per
// community (louvainScanCommunitiesW, inc/louvain.hxx:423). On a unit-weight
// graph those counts are exact integers, so they can be kept instead: built
// once from a membership, then changed by one per move of a neighbour. A hub
// is then evaluated from its table (a few dozen to a few thousand slots)
// instead of its edges (up to millions), with the same gains as a fresh scan.
#include <algorithm>

#include "lvg_internal.cuh"

#define GRID_STRIDE(i, n) for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < (n); i += size_t(gridDim.x) * blockDim.x)

namespace lvg {
namespace {

constexpr int HTB_B = 256;    // build: threads per chunk block
constexpr int HTB_LOG = 12;   // build: shared slots per chunk block
constexpr uint32_t HTB_PROBES = 32;  // a longer probe in shared memory goes to HBM

// Add k to community c's count in a table of 2^lg slots (linear probing).
// False when every slot holds another key.
__device__ __forceinline__ bool cnt_add(uint32_t *keys, uint32_t *cnts, int lg, uint32_t c, uint32_t k) {
  const uint32_t mask = (1u << lg) - 1u;
  uint32_t s = hash_hi(c, lg);
  for (uint32_t p = 0; p <= mask; ++p) {
    uint32_t x = ld_relaxed(keys + s);
    if (x == EMPTY) {
      x = atomicCAS(keys + s, EMPTY, c);
      if (x == EMPTY) x = c;
    }
    if (x == c) {
      atomicAdd(cnts + s, k);
      return true;
    }
    s = (s + 1u) & mask;
  }
  return false;
}

__global__ void ht_slots_kernel(const uint32_t *hubs, size_t n, uint32_t *slot) {
  GRID_STRIDE(i, n) slot[hubs[i]] = uint32_t(i);
}

// Build step 1: a block per chunk of a hub's edges (the hub plan's chunks, all
// colour classes). The chunk's neighbours' communities are counted in shared
// memory first (a hub's neighbours fall into few communities), then added to
// the hub's scratch table in HBM, which has at least twice the hub's degree in
// slots and so always has room. A key that finds no slot within HTB_PROBES
// shared probes goes straight to the scratch table.
__global__ void __launch_bounds__(HTB_B) ht_scratch_kernel(const uint64_t *off, const uint32_t *key, const uint4 *chunk,
                                                          size_t nchunks, const uint32_t *q, const uint32_t *slot,
                                                          const uint64_t *soff, const uint8_t *slg, uint32_t *skey,
                                                          uint32_t *scnt, Counters *ctr) {
  constexpr uint32_t CS = 1u << HTB_LOG;
  __shared__ uint32_t tk[CS];
  __shared__ uint32_t tc[CS];
  bool bad = false;
  for (size_t ci = blockIdx.x; ci < nchunks; ci += gridDim.x) {
    const uint4 ch = chunk[ci];
    const uint32_t u = ch.w;
    const uint32_t h = slot[u];
    for (uint32_t s = threadIdx.x; s < CS; s += HTB_B) { tk[s] = EMPTY; tc[s] = 0; }
    __syncthreads();
    uint32_t *gk = skey + soff[h], *gc = scnt + soff[h];
    const int glg = slg[h];
    const uint64_t o = off[u] + ch.y;
    const uint32_t n = ch.z - ch.y;
    for (uint32_t j = threadIdx.x; j < n; j += HTB_B) {
      const uint32_t v = __ldcs(key + o + j);
      if (v == u) continue;
      const uint32_t c = q[v];
      uint32_t s = hash_hi(c, HTB_LOG);
      bool done = false;
      for (uint32_t p = 0; p < HTB_PROBES; ++p) {
        uint32_t x = tk[s];
        if (x == EMPTY) {
          x = atomicCAS(&tk[s], EMPTY, c);
          if (x == EMPTY) x = c;
        }
        if (x == c) {
          atomicAdd(&tc[s], 1u);
          done = true;
          break;
        }
        s = (s + 1u) & (CS - 1u);
      }
      if (!done) bad |= !cnt_add(gk, gc, glg, c, 1u);
    }
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < CS; s += HTB_B)
      if (tk[s] != EMPTY) bad |= !cnt_add(gk, gc, glg, tk[s], tc[s]);
    __syncthreads();
  }
  if (bad) atomicOr(&ctr->err, ERR_TABLE_FULL);
}

// Build step 2: distinct communities of each hub (a block per hub).
__global__ void ht_count_kernel(size_t hubs, const uint64_t *soff, const uint8_t *slg, const uint32_t *skey,
                                uint32_t *n) {
  __shared__ uint32_t total;
  for (size_t h = blockIdx.x; h < hubs; h += gridDim.x) {
    if (threadIdx.x == 0) total = 0;
    __syncthreads();
    const uint64_t o = soff[h];
    const uint32_t cap = 1u << slg[h];
    uint32_t c = 0;
    for (uint32_t s = threadIdx.x; s < cap; s += blockDim.x) c += skey[o + s] != EMPTY;
#pragma unroll
    for (int x = 16; x > 0; x >>= 1) c += __shfl_xor_sync(0xffffffffu, c, x);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&total, c);
    __syncthreads();
    if (threadIdx.x == 0) n[h] = total;
    __syncthreads();
  }
}

// Build step 3: each hub's scratch entries into its table (a block per hub;
// the table has at least four times the entries in slots). Hubs marked bad
// (too many communities for the largest table) are skipped.
__global__ void ht_fill_kernel(size_t hubs, const uint64_t *soff, const uint8_t *slg, const uint32_t *skey,
                               const uint32_t *scnt, HubTabView t) {
  for (size_t h = blockIdx.x; h < hubs; h += gridDim.x) {
    if (t.bad[h]) continue;
    const uint64_t o = soff[h];
    const uint32_t cap = 1u << slg[h];
    uint32_t *k = t.key + t.off[h], *c = t.cnt + t.off[h];
    for (uint32_t s = threadIdx.x; s < cap; s += blockDim.x) {
      const uint32_t x = skey[o + s];
      if (x != EMPTY && !cnt_add(k, c, t.lg[h], x, scnt[o + s])) ht_mark_bad(t, uint32_t(h));
    }
  }
}

// Deterministic mode: the table updates of a class's decided moves, a warp
// per listed vertex (vertices that stay exit at once).
__global__ void ht_sync_moves_kernel(const uint64_t *off, const uint32_t *deg, const uint32_t *key,
                                     const uint32_t *list, size_t n, const uint32_t *dec, const uint32_t *vcom,
                                     HubTabView t, Counters *ctr) {
  const int lane = threadIdx.x & 31;
  const size_t warps = (size_t(gridDim.x) * blockDim.x) / 32;
  for (size_t i = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; i < n; i += warps) {
    const uint32_t u = list[i];
    const uint32_t c = dec[u];
    if (c == EMPTY) continue;
    const uint32_t d = vcom[u];
    const uint64_t o = off[u];
    const uint32_t dg = deg[u];
    for (uint32_t j = lane; j < dg; j += 32) {
      const uint32_t v = __ldcs(key + o + j);
      if (v != u) ht_move(t, v, d, c, ctr);
    }
  }
}

// A batch's edges (u, v) of hubs u: v's community loses (deletions, sign -1)
// or gains (insertions) one neighbour of u.
__global__ void ht_batch_kernel(const uint32_t *src, const uint32_t *dst, size_t n, bool insert, const uint32_t *q,
                                HubTabView t, Counters *ctr) {
  GRID_STRIDE(i, n) {
    const uint32_t u = src[i], v = dst[i];
    if (u == v) continue;
    const uint32_t h = t.slot[u];
    if (h == NO_HUB || t.bad[h]) continue;
    const uint32_t c = q[v];
    uint32_t *k = t.key + t.off[h], *cn = t.cnt + t.off[h];
    const int lg = t.lg[h];
    const uint32_t mask = (1u << lg) - 1u;
    if (insert) {
      if (!cnt_add(k, cn, lg, c, 1u)) {
        ht_mark_bad(t, h);
        atomicAdd(&ctr->ht_over, 1ull);
      }
    } else {
      bool found = false;
      uint32_t s = hash_hi(c, lg);
      for (uint32_t p = 0; p <= mask; ++p) {
        const uint32_t x = ld_relaxed(k + s);
        if (x == c) { atomicSub(cn + s, 1u); found = true; break; }
        if (x == EMPTY) break;
        s = (s + 1u) & mask;
      }
      if (!found) {
        ht_mark_bad(t, h);
        atomicAdd(&ctr->ht_over, 1ull);
      }
    }
  }
}

unsigned blocks_for(size_t n, size_t cap) { return unsigned(std::max<size_t>(1, std::min(n, cap))); }

}  // namespace

void launch_ht_slots(const uint32_t *hubs, size_t n, uint32_t *slot, cudaStream_t s) {
  if (!n) return;
  ht_slots_kernel<<<grid_for(n, 256), 256, 0, s>>>(hubs, n, slot);
  LVG_CHECK_LAUNCH();
}

void launch_ht_scratch(const Level &lv, const uint32_t *q, const uint32_t *slot, const uint64_t *soff,
                       const uint8_t *slg, uint32_t *skey, uint32_t *scnt, Counters *ctr, cudaStream_t s) {
  const size_t n = lv.hub.chunks;
  if (!n) return;
  ht_scratch_kernel<<<blocks_for(n, size_t(1) << 16), HTB_B, 0, s>>>(lv.off, lv.key, lv.hub.chunk, n, q, slot, soff,
                                                                    slg, skey, scnt, ctr);
  LVG_CHECK_LAUNCH();
}

void launch_ht_count(size_t hubs, const uint64_t *soff, const uint8_t *slg, const uint32_t *skey, uint32_t *n,
                     cudaStream_t s) {
  if (!hubs) return;
  ht_count_kernel<<<blocks_for(hubs, size_t(1) << 16), 256, 0, s>>>(hubs, soff, slg, skey, n);
  LVG_CHECK_LAUNCH();
}

void launch_ht_fill(size_t hubs, const uint64_t *soff, const uint8_t *slg, const uint32_t *skey,
                    const uint32_t *scnt, const HubTabView &t, cudaStream_t s) {
  if (!hubs) return;
  ht_fill_kernel<<<blocks_for(hubs, size_t(1) << 16), 256, 0, s>>>(hubs, soff, slg, skey, scnt, t);
  LVG_CHECK_LAUNCH();
}

void launch_ht_sync_moves(const Level &lv, const uint32_t *list, size_t n, const uint32_t *dec, const uint32_t *vcom,
                          const HubTabView &t, Counters *ctr, cudaStream_t s) {
  if (!n) return;
  ht_sync_moves_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(lv.off, lv.deg, lv.key, list, n, dec, vcom, t, ctr);
  LVG_CHECK_LAUNCH();
}

void launch_ht_batch(const uint32_t *src, const uint32_t *dst, size_t n, bool insert, const uint32_t *q,
                     const HubTabView &t, Counters *ctr, cudaStream_t s) {
  if (!n) return;
  ht_batch_kernel<<<grid_for(n, 256), 256, 0, s>>>(src, dst, n, insert, q, t, ctr);
  LVG_CHECK_LAUNCH();
}

}  // namespace lvg
