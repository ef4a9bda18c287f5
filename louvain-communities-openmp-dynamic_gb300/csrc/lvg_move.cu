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
//   bins 9-11 (degree > 512):        one block per vertex, shared table of
//             4096 / 8192 slots with a claim budget; a vertex with more
//             distinct neighbour communities than the budget is redone with
//             a table in its block's region of global memory.
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
#include <algorithm>

#include "lvg_internal.cuh"

namespace lvg {
namespace {

__host__ __device__ constexpr int ilog2c(int x) { return x <= 1 ? 0 : 1 + ilog2c(x >> 1); }

template <int T>
__device__ __forceinline__ unsigned tile_mask() {
  if constexpr (T == 32) {
    return 0xffffffffu;
  } else {
    const int lane = threadIdx.x & 31;
    return ((1u << T) - 1u) << (lane & ~(T - 1));
  }
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

// The graph-dependent constants of vertex u: R/(2M) and the community that is
// never a move target (the reference's `if (c)`, inc/louvain.hxx:602). For a
// graph union they are those of u's own graph (MoveArgs::gid), so each graph
// moves exactly as it would alone.
struct GraphOf {
  float kr;
  uint32_t zero, g;
  __device__ __forceinline__ GraphOf(const MoveArgs &a, uint32_t u) : kr(a.kr), zero(0), g(0) {
    if (a.gid) {
      g = a.gid[u];
      kr = a.gkr[g];
      zero = a.gzero[g];
    }
  }
};

// Adds a vertex's best gain to the iteration's sum: per thread (flushed per
// block) for one graph, per graph for a union.
__device__ __forceinline__ void add_gain(const MoveArgs &a, const GraphOf &G, unsigned long long &fix, float bg) {
  if (a.gfix) atomicAdd(&a.gfix[G.g], gain_to_fix(bg));
  else fix += gain_to_fix(bg);
}

__device__ __forceinline__ void flush_counters(Counters *ctr, int bin, unsigned long long fix, unsigned long long nv,
                                               unsigned long long ne, unsigned long long nm, bool bad,
                                               unsigned long long no = 0) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    fix += __shfl_xor_sync(0xffffffffu, fix, o);
    nv += __shfl_xor_sync(0xffffffffu, nv, o);
    ne += __shfl_xor_sync(0xffffffffu, ne, o);
    nm += __shfl_xor_sync(0xffffffffu, nm, o);
    no += __shfl_xor_sync(0xffffffffu, no, o);
  }
  bool anybad = __any_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0) {
    if (fix) atomicAdd(&ctr->el_fix, fix);
    if (nv) { atomicAdd(&ctr->vertices, nv); atomicAdd(&ctr->bin_vertices[bin], nv); }
    if (ne) { atomicAdd(&ctr->edges, ne); atomicAdd(&ctr->bin_edges[bin], ne); }
    if (nm) atomicAdd(&ctr->moves, nm);
    if (no) atomicAdd(&ctr->bin_over[bin], no);
    if (anybad) atomicOr(&ctr->err, ERR_TABLE_FULL);
  }
}

// Warp-aggregated insertion: the 32 lanes of a converged warp each hold a
// (c, w) pair (c == EMPTY: nothing). Lanes holding the same key are combined
// (weights summed in lane order) and only the lowest such lane calls
// ins(c, sum). Hot keys then cost one table atomic per warp instead of one
// per lane. With UNIT (every weight 1) the sum is the group's size. Returns
// false on the lanes whose ins() failed.
template <bool UNIT, class Ins>
__device__ __forceinline__ bool warp_insert(uint32_t c, float w, Ins ins) {
  const unsigned grp = __match_any_sync(0xffffffffu, c);
  const int lane = threadIdx.x & 31;
  const bool leader = (grp & ((1u << lane) - 1u)) == 0u;
  if constexpr (UNIT) {
    return !(leader && c != EMPTY) || ins(c, float(__popc(grp)));
  } else {
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
    return !(leader && c != EMPTY) || ins(c, sum);
  }
}

// Edge weight i of the level, or 1 for a unit-weight level (not read).
template <bool UNIT>
__device__ __forceinline__ float edge_weight(const MoveArgs &a, uint64_t i) {
  if constexpr (UNIT) return 1.f;
  else return __ldcs(a.w + i);
}

// ------------------------------------------------------------ tile / warp kernel

constexpr int TILE_BLOCK = 256;

// The tiles of one block work through list[0..count): tile t of the block
// takes items first + t, first + t + ntiles, ... (ntiles = tiles of all the
// blocks sharing the list). Counters are flushed for degree bin `bin`.
template <int T, int C, bool SYNC, bool UNIT>
__device__ __forceinline__ void tile_loop(const MoveArgs &a, const uint32_t *list, uint32_t count, uint32_t first,
                                          uint32_t ntiles, uint8_t *smem, int bin) {
  constexpr int LOGC = ilog2c(C);
  constexpr int TPB = TILE_BLOCK / T;
  const int tib = threadIdx.x / T;
  const int tl = threadIdx.x & (T - 1);
  uint32_t *keys = reinterpret_cast<uint32_t *>(smem) + tib * C;
  float *vals = reinterpret_cast<float *>(smem + size_t(TPB) * C * sizeof(uint32_t)) + tib * C;
  const unsigned m = tile_mask<T>();
  unsigned long long fix = 0, nv = 0, ne = 0, nm = 0, no = 0;
  bool bad = false;
  for (uint32_t i = first + tib; i < count; i += ntiles) {
    const uint32_t u = list[i];  // active (compacted worklist)
    const GraphOf G(a, u);
    const uint64_t o = a.off[u];
    const uint32_t dg = a.deg[u];
    const uint32_t d = a.vcom[u];
    // the vertex's weight and its community's total, loaded while the edges
    // are scanned (a racy snapshot in asynchronous mode, as any read of them
    // is; fixed within a class in deterministic mode)
    double wu = 0.0, td = 0.0;
    if (tl == 0) { wu = a.vtot[u]; td = a.ctot[d]; }
    // (the table loops unrolled by at most 8: the 512- and 1024-slot tables'
    // fully unrolled loops stalled the fused degree 129-512 launch on
    // instruction fetch)
#pragma unroll 8
    for (int s = tl; s < C; s += T) { keys[s] = EMPTY; vals[s] = 0.f; }
    __syncwarp(m);
    float kd = 0.f;
    bool ok = true;
    // U independent edge loads per lane in flight (degree <= C/2, so a lane
    // has at most C/(2T) edges).
    constexpr int U = (C / (2 * T)) < 1 ? 1 : ((C / (2 * T)) > 4 ? 4 : (C / (2 * T)));
    if (T == 32) {
      // one warp per vertex: warp-uniform batches, hot keys combined per warp;
      // the next batch's ids and weights load while this one's communities do
      uint32_t nv[U];
      float nw[U];
#pragma unroll
      for (int k = 0; k < U; ++k) {
        const uint32_t j = k * 32 + tl;
        nv[k] = j < dg ? __ldcs(a.key + o + j) : u;
        nw[k] = j < dg ? edge_weight<UNIT>(a, o + j) : 0.f;
      }
      for (uint32_t base = 0; base < dg; base += U * 32) {
        uint32_t v[U];
        float w[U];
#pragma unroll
        for (int k = 0; k < U; ++k) { v[k] = nv[k]; w[k] = nw[k]; }
        if (base + U * 32 < dg) {
#pragma unroll
          for (int k = 0; k < U; ++k) {
            const uint32_t j = base + U * 32 + k * 32 + tl;
            nv[k] = j < dg ? __ldcs(a.key + o + j) : u;
            nw[k] = j < dg ? edge_weight<UNIT>(a, o + j) : 0.f;
          }
        }
        uint32_t c[U];
#pragma unroll
        for (int k = 0; k < U; ++k) {
          c[k] = v[k] != u ? a.vcom[v[k]] : EMPTY;
          if (c[k] == d) { kd += w[k]; c[k] = EMPTY; }
        }
#pragma unroll
        for (int k = 0; k < U; ++k)
          ok &= warp_insert<UNIT>(c[k], w[k],
                                  [&](uint32_t cc, float ww) { return table_add(keys, vals, LOGC, cc, ww); });
      }
    } else
    for (uint32_t j0 = tl; j0 < dg; j0 += U * T) {
      uint32_t v[U];
      float w[U];
#pragma unroll
      for (int k = 0; k < U; ++k) {
        const uint32_t j = j0 + k * T;
        v[k] = j < dg ? __ldcs(a.key + o + j) : u;
        w[k] = j < dg ? edge_weight<UNIT>(a, o + j) : 0.f;
      }
      uint32_t c[U];
#pragma unroll
      for (int k = 0; k < U; ++k) c[k] = v[k] != u ? a.vcom[v[k]] : EMPTY;
#pragma unroll
      for (int k = 0; k < U; ++k) {
        if (c[k] == EMPTY) continue;
        if (c[k] == d) kd += w[k];
        else ok &= table_add(keys, vals, LOGC, c[k], w[k]);
      }
    }
#pragma unroll
    for (int sh = T / 2; sh > 0; sh >>= 1) kd += __shfl_xor_sync(m, kd, sh, T);
    __syncwarp(m);
    wu = __shfl_sync(m, wu, 0, T);
    td = __shfl_sync(m, td, 0, T);
    const float wuf = __double2float_rn(wu);
    float bg = 0.f;
    uint32_t bc = EMPTY;
#pragma unroll 8
    for (int s = tl; s < C; s += T) {
      const uint32_t c = keys[s];
      if (c == EMPTY) continue;
      const float g = gain_of(vals[s], kd, wu, wuf, a.ctot[c], td, G.kr);
      if (g > 0.f) take_better(bg, bc, g, c);
    }
#pragma unroll
    for (int sh = T / 2; sh > 0; sh >>= 1) {
      const float og = __shfl_xor_sync(m, bg, sh, T);
      const uint32_t oc = __shfl_xor_sync(m, bc, sh, T);
      take_better(bg, bc, og, oc);
    }
    const bool moved = bc != EMPTY && bc != G.zero;
    if (tl == 0) {
      if (bc != EMPTY) add_gain(a, G, fix, bg);
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
        const uint32_t v = __ldcs(a.key + o + j);
        if (v != u) {
          mk[v] = 1;
          if (!SYNC && a.ht.key) ht_move(a.ht, v, d, bc, a.ctr);
        }
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
  flush_counters(a.ctr, bin, fix, nv, ne, nm, bad, no);
}

// Tiles with tables of up to 256 slots: registers capped for 8 resident
// blocks per SM (these kernels wait on gathers; more warps hide more of it —
// measured on graph unions: the degree 17-64 kernels ran 26 % faster).
template <int T, int C, bool SYNC, bool UNIT>
__global__ void __launch_bounds__(TILE_BLOCK, (C <= 256 ? 8 : 1)) move_tile_kernel(MoveArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  constexpr int TPB = TILE_BLOCK / T;
  const uint32_t count = a.count_ptr ? *a.count_ptr : a.count;
  tile_loop<T, C, SYNC, UNIT>(a, a.list, count, blockIdx.x * TPB, gridDim.x * TPB, smem, a.bin);
}

// Several degree bins of one colour class in one launch (bins lo..hi of
// 1..8): the blocks [sb.block_begin[b-lo], sb.block_begin[b-lo+1]) serve bin
// b with its own tile size and table, as move_tile_kernel would. Used when the
// classes' worklists are short (dynamic-frontier and delta-screening passes
// over the uploaded graph), where a launch per bin would cost more than its
// work.
// MINB: resident blocks per SM the kernel is compiled for. Bins 1-6 come in
// two variants (lvg_tuning.small_regs): 8 blocks (32 registers a thread,
// some values spilled to local memory) or 4 (64 registers, none spilled).
template <int LO, int HI, bool SYNC, bool UNIT, int MINB>
__global__ void __launch_bounds__(TILE_BLOCK, MINB) move_small_kernel(MoveArgs a, SmallBins sb) {
  extern __shared__ __align__(16) uint8_t smem[];
  int k = 0;
  while (k < HI - LO && blockIdx.x >= sb.block_begin[k + 1]) ++k;
  // constant indices into sb (a dynamic index would copy it to local memory)
  switch (LO + k) {
#define LVG_SMALL_CASE(B, T, C)                                                                          \
  case B:                                                                                                \
    if (B >= LO && B <= HI) {                                                                            \
      constexpr int J = (B >= LO && B <= HI) ? B - LO : 0;                                              \
      const uint32_t b0 = sb.block_begin[J], nb = sb.block_begin[J + 1] - b0;                           \
      tile_loop<T, C, SYNC, UNIT>(a, sb.list[J], *sb.count_ptr[J], (blockIdx.x - b0) * (TILE_BLOCK / T),\
                            nb * (TILE_BLOCK / T), smem, B);                                             \
    }                                                                                                    \
    break;
    LVG_SMALL_CASE(1, 4, 8)
    LVG_SMALL_CASE(2, 8, 16)
    LVG_SMALL_CASE(3, 16, 32)
    LVG_SMALL_CASE(4, 32, 64)
    LVG_SMALL_CASE(5, 32, 128)
    LVG_SMALL_CASE(6, 32, 256)
    LVG_SMALL_CASE(7, 32, 512)
    LVG_SMALL_CASE(8, 32, 1024)
#undef LVG_SMALL_CASE
    default: break;
  }
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

// Insert into a shared table with a claim budget: a new key may take a slot
// only while fewer than `limit` slots were claimed (load <= 50 %). Returns
// false when the budget is exhausted; the caller then redoes the vertex with
// a table in global memory, so no key is ever split between two tables.
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

// A shared-memory table that also lists its claimed slots, so that the
// argmax and the reset after a vertex touch only those slots. Claims are
// limited to `limit` (half the table); a reservation whose slot was taken by
// another key is listed as EMPTY.
struct ListedTable {
  uint32_t *keys;
  float *vals;
  uint32_t *list;
  unsigned *used;
};

__device__ __forceinline__ bool lt_add(const ListedTable &t, int log2cap, uint32_t c, float w, unsigned limit) {
  const uint32_t mask = (1u << log2cap) - 1u;
  uint32_t s = hash_hi(c, log2cap);
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    const uint32_t k = t.keys[s];
    if (k == c) { atomicAdd(&t.vals[s], w); return true; }
    if (k == EMPTY) {
      const unsigned r = atomicAdd(t.used, 1u);
      if (r >= limit) return false;
      const uint32_t prev = atomicCAS(&t.keys[s], EMPTY, c);
      if (prev == EMPTY) {
        t.list[r] = s;
        atomicAdd(&t.vals[s], w);
        return true;
      }
      t.list[r] = EMPTY;
      if (prev == c) { atomicAdd(&t.vals[s], w); return true; }
    }
    s = (s + 1u) & mask;
  }
  return false;
}

// Reset the listed slots (call with the whole block; ends with a barrier).
template <int B>
__device__ __forceinline__ void lt_reset(const ListedTable &t, unsigned n) {
  for (unsigned i = threadIdx.x; i < n; i += B) {
    const uint32_t s = t.list[i];
    if (s != EMPTY) { t.keys[s] = EMPTY; t.vals[s] = 0.f; }
  }
  __syncthreads();
}

// Scan edges [o, o+n) of u with the whole block (warp-uniform trip counts, 4
// independent loads in flight per lane) into a table via add(c, w), called
// once per distinct key per warp batch. Edges into the own community d are
// summed in the lane-private return value. Stops (block-uniformly per warp)
// as soon as an add() fails. Edge ids and weights are read with the
// streaming hint (evict first): each is read once per scan, while the
// membership array that every edge gathers from should stay in L2.
template <int B, bool UNIT, class Add>
__device__ __forceinline__ float scan_edges(const MoveArgs &a, uint32_t u, uint64_t o, uint32_t n, uint32_t d,
                                            Add add) {
  constexpr int U = 4;
  const uint32_t lane = threadIdx.x & 31u;
  float kd = 0.f;
  // the next batch's ids and weights are loaded while this batch's
  // communities are gathered (two loads in flight instead of one after the
  // other)
  uint32_t nv[U];
  float nw[U];
  const uint32_t base0 = threadIdx.x & ~31u;
#pragma unroll
  for (int k = 0; k < U; ++k) {
    const uint32_t j = base0 + k * B + lane;
    nv[k] = j < n ? __ldcs(a.key + o + j) : u;
    nw[k] = j < n ? edge_weight<UNIT>(a, o + j) : 0.f;
  }
  for (uint32_t base = base0; base < n; base += U * B) {
    uint32_t v[U];
    float w[U];
#pragma unroll
    for (int k = 0; k < U; ++k) { v[k] = nv[k]; w[k] = nw[k]; }
    const uint32_t next = base + U * B;
    if (next < n) {
#pragma unroll
      for (int k = 0; k < U; ++k) {
        const uint32_t j = next + k * B + lane;
        nv[k] = j < n ? __ldcs(a.key + o + j) : u;
        nw[k] = j < n ? edge_weight<UNIT>(a, o + j) : 0.f;
      }
    }
    uint32_t c[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      c[k] = v[k] != u ? a.vcom[v[k]] : EMPTY;
      if (c[k] == d) { kd += w[k]; c[k] = EMPTY; }
    }
    bool fail = false;
#pragma unroll
    for (int k = 0; k < U; ++k) fail |= !warp_insert<UNIT>(c[k], w[k], add);
    if (__any_sync(0xffffffffu, fail)) break;
  }
  return kd;
}

// The hot keys of a hub chunk (hub_chunk_kernel): up to HOT_KEYS of the
// communities its first edges fell into most, held in registers by every
// thread. Unused entries hold NO_KEY, which matches no community and not EMPTY.
constexpr int HOT_KEYS = 8;
constexpr uint32_t NO_KEY = 0xFFFFFFFEu;

// scan_edges with a hot set: an edge into the own community or one of the
// hot communities adds to a lane-private sum (kd / hc[h]); only the others go
// through the warp-aggregated table insert, and a batch of 32 edges with none
// left skips it. After static Louvain a hub's neighbours fall into few
// communities (on R-MAT, the 8 most frequent of a chunk's first 1024 edges
// take 99 % of the rest), so nearly every edge stays out of shared memory.
template <int B, bool UNIT, class Add>
__device__ __forceinline__ float scan_edges_hot(const MoveArgs &a, uint32_t u, uint64_t o, uint32_t n, uint32_t d,
                                                const uint32_t (&hot)[HOT_KEYS], float (&hc)[HOT_KEYS], Add add) {
  constexpr int U = 4;
  const uint32_t lane = threadIdx.x & 31u;
  float kd = 0.f;
  uint32_t nv[U];
  float nw[U];
  const uint32_t base0 = threadIdx.x & ~31u;
#pragma unroll
  for (int k = 0; k < U; ++k) {
    const uint32_t j = base0 + k * B + lane;
    nv[k] = j < n ? __ldcs(a.key + o + j) : u;
    nw[k] = j < n ? edge_weight<UNIT>(a, o + j) : 0.f;
  }
  for (uint32_t base = base0; base < n; base += U * B) {
    uint32_t v[U];
    float w[U];
#pragma unroll
    for (int k = 0; k < U; ++k) { v[k] = nv[k]; w[k] = nw[k]; }
    const uint32_t next = base + U * B;
    if (next < n) {
#pragma unroll
      for (int k = 0; k < U; ++k) {
        const uint32_t j = next + k * B + lane;
        nv[k] = j < n ? __ldcs(a.key + o + j) : u;
        nw[k] = j < n ? edge_weight<UNIT>(a, o + j) : 0.f;
      }
    }
    uint32_t c[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      c[k] = v[k] != u ? a.vcom[v[k]] : EMPTY;
      if (c[k] == d) { kd += w[k]; c[k] = EMPTY; }
#pragma unroll
      for (int h = 0; h < HOT_KEYS; ++h)
        if (c[k] == hot[h]) { hc[h] += w[k]; c[k] = EMPTY; }
    }
    bool fail = false;
#pragma unroll
    for (int k = 0; k < U; ++k)
      if (__any_sync(0xffffffffu, c[k] != EMPTY)) fail |= !warp_insert<UNIT>(c[k], w[k], add);
    if (__any_sync(0xffffffffu, fail)) break;
  }
  return kd;
}

// One block per vertex (degree 513..8192). The vertex is first aggregated in
// a listed shared table of 2^LOGS slots (cleared once per block, then reset
// slot by slot); if it has more distinct neighbour communities than the
// budget (half the slots), it is redone with a table in this block's region
// of global memory (2^a.glog2 slots). After the first local-moving
// iterations a high-degree vertex's neighbours fall into few communities, so
// the shared table almost always suffices and the argmax visits only the
// claimed slots.
template <int B, int LOGS, bool SYNC, bool UNIT>
__global__ void __launch_bounds__(B) move_big_kernel(MoveArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ float red_g[B / 32];
  __shared__ uint32_t red_c[B / 32];
  __shared__ unsigned s_used;
  __shared__ int s_over;
  constexpr uint32_t CS = 1u << LOGS;
  ListedTable t;
  t.keys = reinterpret_cast<uint32_t *>(smem);
  t.vals = reinterpret_cast<float *>(smem + size_t(CS) * 4);
  t.list = reinterpret_cast<uint32_t *>(smem + size_t(CS) * 8);
  t.used = &s_used;
  for (uint32_t s2 = threadIdx.x; s2 < CS; s2 += B) { t.keys[s2] = EMPTY; t.vals[s2] = 0.f; }
  uint32_t *gkeys = a.gkeys ? a.gkeys + (size_t(blockIdx.x) << a.glog2) : nullptr;
  float *gvals = a.gvals ? a.gvals + (size_t(blockIdx.x) << a.glog2) : nullptr;
  unsigned long long fix = 0, nv = 0, ne = 0, nm = 0, no = 0;
  bool bad = false;
  const uint32_t count = a.count_ptr ? *a.count_ptr : a.count;
  __syncthreads();
  for (uint32_t i = blockIdx.x; i < count; i += gridDim.x) {
    // the worklist holds only active vertices (compact_active_kernel), and
    // only the vertex itself clears its flag
    const uint32_t u = a.list[i];
    const GraphOf G(a, u);
    if (threadIdx.x == 0) {
      s_used = 0;
      s_over = 0;
    }
    __syncthreads();
    const uint64_t o = a.off[u];
    const uint32_t dg = a.deg[u];
    const uint32_t d = a.vcom[u];
    int lg = min(LOGS, max(1, ceil_log2(2ull * dg)));
    const unsigned limit = (1u << lg) >> 1;
    // static Louvain's first iteration (a.big_direct): the neighbours are
    // still singletons, so a vertex of more edges than the claim budget would
    // overflow the shared table: straight to the table in global memory
    float kd = 0.f;
    if (a.big_direct && dg > limit) {
      if (threadIdx.x == 0) s_over = 1;
    } else {
      kd = scan_edges<B, UNIT>(a, u, o, dg, d, [&](uint32_t c, float w) {
        if (lt_add(t, lg, c, w, limit)) return true;
        s_over = 1;
        return false;
      });
    }
    __syncthreads();
    const unsigned nlist = min(s_used, limit);
    const bool over = s_over;
    bool ok = true;
    uint32_t gcap = 0;
    if (over) {
      // attempt 2: global table sized for the degree
      lt_reset<B>(t, nlist);
      lg = min(a.glog2, max(1, ceil_log2(2ull * dg)));
      gcap = gkeys ? (1u << lg) : 0;
      if (!gkeys) ok = false;
      for (uint32_t s2 = threadIdx.x; s2 < gcap; s2 += B) { gkeys[s2] = EMPTY; gvals[s2] = 0.f; }
      __syncthreads();
      if (gkeys) kd = scan_edges<B, UNIT>(a, u, o, dg, d, [&](uint32_t c, float w) {
        ok &= table_add(gkeys, gvals, lg, c, w);
        return true;
      });
    }
    kd = block_sum<B>(kd, red_g);  // barrier: table complete
    const double wu = a.vtot[u];
    const float wuf = __double2float_rn(wu);
    const double td = a.ctot[d];
    float bg = 0.f;
    uint32_t bc = EMPTY;
    if (!over) {
      for (unsigned j = threadIdx.x; j < nlist; j += B) {
        const uint32_t s2 = t.list[j];
        if (s2 == EMPTY) continue;
        const uint32_t c = t.keys[s2];
        const float g = gain_of(t.vals[s2], kd, wu, wuf, a.ctot[c], td, G.kr);
        if (g > 0.f) take_better(bg, bc, g, c);
      }
    } else {
      for (uint32_t s2 = threadIdx.x; s2 < gcap; s2 += B) {
        const uint32_t c = gkeys[s2];
        if (c == EMPTY) continue;
        const float g = gain_of(gvals[s2], kd, wu, wuf, a.ctot[c], td, G.kr);
        if (g > 0.f) take_better(bg, bc, g, c);
      }
    }
    block_argmax<B>(bg, bc, red_g, red_c);
    if (!over) lt_reset<B>(t, nlist);
    const bool moved = bc != EMPTY && bc != G.zero;
    if (threadIdx.x == 0) {
      if (bc != EMPTY) add_gain(a, G, fix, bg);
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
        const uint32_t v = __ldcs(a.key + o + j);
        if (v != u) {
          mk[v] = 1;
          if (!SYNC && a.ht.key) ht_move(a.ht, v, d, bc, a.ctr);
        }
      }
    }
    if (threadIdx.x == 0) {
      a.vaff[u] = 0;
      ++nv;
      ne += dg;
      nm += moved;
      no += over;
    }
    bad |= !ok;
    __syncthreads();
  }
  flush_counters(a.ctr, a.bin, fix, nv, ne, nm, bad, no);
}

// ------------------------------------------------------------ chunked hubs

// Hub path, step 1: one block per chunk (lvg_tuning::hub_chunk edges) of one hub of the
// colour class. The chunk is merged in a listed shared table with a claim
// budget and its distinct (community, weight) pairs are written to the
// chunk's partial region; a chunk with more distinct communities than the
// budget writes its raw pairs instead. Edges into the hub's own community are
// summed separately into hub_kd[u].
template <int B, int LOGS, bool UNIT>
__global__ void __launch_bounds__(B) hub_chunk_kernel(MoveArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ float red_g[B / 32];
  __shared__ float red_h[B / 32][HOT_KEYS];
  __shared__ uint32_t s_hot[HOT_KEYS];
  __shared__ int s_act;
  __shared__ unsigned s_used, s_cnt, s_nhot;
  __shared__ int s_over;
  constexpr uint32_t CS = 1u << LOGS;
  ListedTable t;
  t.keys = reinterpret_cast<uint32_t *>(smem);
  t.vals = reinterpret_cast<float *>(smem + size_t(CS) * 4);
  t.list = reinterpret_cast<uint32_t *>(smem + size_t(CS) * 8);
  t.used = &s_used;
  __shared__ int s_skip;
  // a block per chunk, or (resident hub tables: most blocks have nothing to
  // do) fewer blocks looping over the chunks
  const size_t c0 = a.hub.chunk_begin[a.color], nch = a.hub.chunk_begin[a.color + 1] - c0;
  for (size_t k = blockIdx.x; k < nch; k += gridDim.x) {
    const size_t ci = c0 + k;
    __syncthreads();  // the previous chunk's readers of the shared state are done
    if (threadIdx.x == 0) s_skip = a.ht.key && ld_relaxed(a.ht.nbad) == 0;
    __syncthreads();  // (one decision for the block: nbad may change meanwhile)
    if (s_skip) {  // every hub is done by hub_table_kernel
      if (threadIdx.x == 0) a.chunk_cnt[ci] = EMPTY;  // (the merge may still find a table gone bad)
      continue;
    }
    const uint4 ch = a.hub.chunk[ci];
    const uint32_t u = ch.w;  // the hub vertex
    if (threadIdx.x == 0) {
      s_act = a.vaff[u] && (!a.fa || a.fa[u]) && (!a.gact || a.gact[a.gid[u]]) &&
              !(a.ht.key && !a.ht.bad[a.ht.slot[u]]);  // a hub with a good table is done by hub_table_kernel
      s_used = 0;
      s_over = 0;
      s_cnt = 0;
      s_nhot = 0;
    }
    __syncthreads();
    if (!s_act) {
      if (threadIdx.x == 0) a.chunk_cnt[ci] = EMPTY;  // tells step 2 the hub was inactive
      continue;
    }
    const uint64_t o = a.off[u] + ch.y;
    const uint32_t n = ch.z - ch.y;
    const uint32_t d = a.vcom[u];
    const int lg = min(LOGS, max(1, ceil_log2(2ull * n)));
    const uint32_t vcap = 1u << lg;
    for (uint32_t s2 = threadIdx.x; s2 < vcap; s2 += B) { t.keys[s2] = EMPTY; t.vals[s2] = 0.f; }
    __syncthreads();
    const unsigned limit = vcap >> 1;
    auto add = [&](uint32_t c, float w) {
      if (lt_add(t, lg, c, w, limit)) return true;
      s_over = 1;
      return false;
    };
    // the first edges (one batch per thread) through the table, then the hot
    // set: the keys that took at least 1/64 of their weight
    const uint32_t nA = min(n, uint32_t(4 * B));
    float kd = scan_edges<B, UNIT>(a, u, o, nA, d, add);
    __syncthreads();
    if (n > nA && !s_over) {
      const unsigned nl = min(s_used, limit);
      float part = 0.f;
      for (unsigned j = threadIdx.x; j < nl; j += B) {
        const uint32_t s2 = t.list[j];
        if (s2 != EMPTY) part += t.vals[s2];
      }
      const float thr = block_sum<B>(part, red_g) * (1.f / 64.f);
      for (unsigned j = threadIdx.x; j < nl; j += B) {
        const uint32_t s2 = t.list[j];
        if (s2 != EMPTY && t.vals[s2] >= thr) {
          const unsigned h = atomicAdd(&s_nhot, 1u);
          if (h < HOT_KEYS) s_hot[h] = t.keys[s2];
        }
      }
      __syncthreads();
      uint32_t hot[HOT_KEYS];
      float hc[HOT_KEYS];
      const unsigned nh = min(s_nhot, unsigned(HOT_KEYS));
  #pragma unroll
      for (int h = 0; h < HOT_KEYS; ++h) { hot[h] = unsigned(h) < nh ? s_hot[h] : NO_KEY; hc[h] = 0.f; }
      kd += scan_edges_hot<B, UNIT>(a, u, o + nA, n - nA, d, hot, hc, add);
      // the hot keys' sums into the table, where the keys are already
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  #pragma unroll
      for (int h = 0; h < HOT_KEYS; ++h) {
        float x = hc[h];
  #pragma unroll
        for (int of = 16; of > 0; of >>= 1) x += __shfl_xor_sync(0xffffffffu, x, of);
        if (lane == 0) red_h[wid][h] = x;
      }
      __syncthreads();
      if (threadIdx.x < nh) {
        float x = 0.f;
        for (int k = 0; k < B / 32; ++k) x += red_h[k][threadIdx.x];
        if (x != 0.f) add(s_hot[threadIdx.x], x);
      }
    }
    __syncthreads();
    uint32_t *pk = a.part_key + a.hub.chunk_part[ci];
    float *pv = a.part_val + a.hub.chunk_part[ci];
    if (!s_over) {
      const unsigned nl = min(s_used, limit);
      for (unsigned j = threadIdx.x; j < nl; j += B) {
        const uint32_t s2 = t.list[j];
        if (s2 == EMPTY) continue;
        const uint32_t pos = atomicAdd(&s_cnt, 1u);
        pk[pos] = t.keys[s2];
        pv[pos] = t.vals[s2];
      }
    } else {
      // too many distinct communities in this chunk: hand its raw pairs on
      kd = 0.f;
      for (uint32_t j = threadIdx.x; j < n; j += B) {
        const uint32_t v = __ldcs(a.key + o + j);
        const uint32_t c = v != u ? a.vcom[v] : EMPTY;
        const float w = edge_weight<UNIT>(a, o + j);
        if (c == d) kd += w;
        if (c != EMPTY && c != d) {
          const uint32_t pos = atomicAdd(&s_cnt, 1u);
          pk[pos] = c;
          pv[pos] = w;
        }
      }
    }
    kd = block_sum<B>(kd, red_g);
    if (threadIdx.x == 0) {
      if (kd != 0.f) atomicAdd(&a.hub_kd[u], kd);
      a.chunk_cnt[ci] = s_cnt;
      if (s_over) {
        atomicAdd(&a.ctr->hub_chunk_over, 1ull);
        a.hub_over[ch.x] = 1;
      }
    }
  }
}

// Hub path, step 1b (launched when a.spill_keys is set: static Louvain's
// first sweep, where every neighbour community starts as a singleton and a
// hub's chunks hand on about as many raw pairs as the hub has edges): one
// block per chunk of a hub that a chunk marked, inserting the chunk's partial
// entries into the hub's spill table, so that a large hub is merged by as many
// blocks as it has chunks instead of by one. The table holds at least twice
// the hub's degree and its distinct keys are at most the degree, so the
// probes stay bounded.
template <int B>
__global__ void __launch_bounds__(B) hub_spill_kernel(MoveArgs a) {
  const size_t ci = a.hub.chunk_begin[a.color] + blockIdx.x;
  const uint4 ch = a.hub.chunk[ci];
  if (!a.hub_over[ch.x]) return;
  const uint32_t cnt = a.chunk_cnt[ci];
  if (cnt == EMPTY) return;
  const uint64_t p = a.hub.chunk_part[ci];
  const int lg = a.hub.hub_tlog[ch.x];
  uint32_t *keys = a.spill_keys + a.hub.hub_toff[ch.x];
  float *vals = a.spill_vals + a.hub.hub_toff[ch.x];
  bool ok = true;
  for (uint32_t q = threadIdx.x; q < cnt; q += B) ok &= table_add(keys, vals, lg, a.part_key[p + q], a.part_val[p + q]);
  if (!ok) atomicOr(&a.ctr->err, ERR_TABLE_FULL);
}

// Hub path, step 1c (with step 1b): the best community of every spilled hub
// of the class, over all of its spill table at once — a thread per slot, so a
// hub of a million edges is searched by thousands of threads, not one block.
// Each candidate's gain is packed with its id (gain bits above, ~id below: the
// larger gain, then the lower id, as `better`; only positive gains, whose bits
// order as the floats do) and the hub's best taken with a 64-bit atomicMax.
// The slots are cleared behind the search for the next class.
__global__ void hub_argmax_kernel(MoveArgs a) {
  const size_t slots = a.hub.class_slots[a.color];
  const uint32_t *pages = a.hub.page_hub + a.hub.page_begin[a.color];
  const int lane = threadIdx.x & 31;
  for (size_t base = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32 * 32; base < slots;
       base += size_t(gridDim.x) * blockDim.x) {
    const uint32_t g = pages[base >> SPILL_PAGE_LOG];  // one hub per warp (pages are whole warps)
    if (!a.hub_over[g]) continue;
    const size_t s = base + lane;
    const uint32_t c = a.spill_keys[s];
    unsigned long long best = 0;
    if (c != EMPTY) {
      const uint32_t u = a.hub.hub_vertex[g];
      const GraphOf G(a, u);
      const uint32_t d = a.vcom[u];
      const double wu = a.vtot[u];
      const float g2 = gain_of(a.spill_vals[s], a.hub_kd[u], wu, __double2float_rn(wu), a.ctot[c], a.ctot[d], G.kr);
      if (g2 > 0.f) best = (static_cast<unsigned long long>(__float_as_uint(g2)) << 32) | (0xFFFFFFFFu - c);
      a.spill_keys[s] = EMPTY;
      a.spill_vals[s] = 0.f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, best, o);
      best = x > best ? x : best;
    }
    if (lane == 0 && best) atomicMax(&a.hub_best[g], best);
  }
}

// The move of a hub once its best community is known (either merge path):
// the gain into the iteration's sum, the move (or, deterministic, the
// decision), the neighbours marked, the hub's own flag cleared.
template <int B, bool SYNC>
__device__ __forceinline__ void hub_decide(const MoveArgs &a, const GraphOf &G, uint32_t u, uint32_t d, uint32_t dg,
                                           uint32_t scanned, double wu, float bg, uint32_t bc, bool over,
                                           unsigned long long &fix, unsigned long long &nv, unsigned long long &ne,
                                           unsigned long long &nm, unsigned long long &no) {
  const bool moved = bc != EMPTY && bc != G.zero;
  if (threadIdx.x == 0) {
    a.hub_kd[u] = 0.f;
    if (bc != EMPTY) add_gain(a, G, fix, bg);
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
    const uint64_t o = a.off[u];
    for (uint32_t j = threadIdx.x; j < dg; j += B) {
      const uint32_t v = __ldcs(a.key + o + j);
      if (v != u) {
        mk[v] = 1;
        if (!SYNC && a.ht.key) ht_move(a.ht, v, d, bc, a.ctr);
      }
    }
  }
  if (threadIdx.x == 0) {
    a.vaff[u] = 0;
    ++nv;
    ne += scanned;
    nm += moved;
    no += over;
  }
}

// Hub path, step 2: one block per hub of the colour class (grid-stride).
// Merges the partial entries of the hub's chunks (listed shared table with a
// claim budget; global fallback region otherwise), then chooses and applies
// the move like the other local-moving kernels.
template <int B, int LOGS, bool SYNC>
__global__ void __launch_bounds__(B) hub_merge_kernel(MoveArgs a) {
  extern __shared__ __align__(16) uint8_t smem[];
  __shared__ float red_g[B / 32];
  __shared__ uint32_t red_c[B / 32];
  __shared__ unsigned s_used;
  __shared__ int s_over;
  __shared__ float s_kd;
  constexpr uint32_t CS = 1u << LOGS;
  ListedTable t;
  t.keys = reinterpret_cast<uint32_t *>(smem);
  t.vals = reinterpret_cast<float *>(smem + size_t(CS) * 4);
  t.list = reinterpret_cast<uint32_t *>(smem + size_t(CS) * 8);
  t.used = &s_used;
  if (a.ht.key) {  // resident hub tables: nothing to merge while none is bad
    if (threadIdx.x == 0) s_over = ld_relaxed(a.ht.nbad) != 0;
    __syncthreads();
    if (!s_over) return;
    __syncthreads();
  }
  for (uint32_t s2 = threadIdx.x; s2 < CS; s2 += B) { t.keys[s2] = EMPTY; t.vals[s2] = 0.f; }
  uint32_t *gkeys = a.gkeys ? a.gkeys + (size_t(blockIdx.x) << a.glog2) : nullptr;
  float *gvals = a.gvals ? a.gvals + (size_t(blockIdx.x) << a.glog2) : nullptr;
  const size_t h0 = a.hub.hub_begin[a.color], h1 = a.hub.hub_begin[a.color + 1];
  unsigned long long fix = 0, nv = 0, ne = 0, nm = 0, no = 0;
  bool bad = false;
  __syncthreads();
  for (size_t g = h0 + blockIdx.x; g < h1; g += gridDim.x) {
    const uint32_t u = a.hub.hub_vertex[g];
    const GraphOf G(a, u);
    const uint32_t c0 = a.hub.hub_first[g], c1 = a.hub.hub_first[g + 1];
    if (threadIdx.x == 0) {
      s_used = 0;
      s_over = 0;
      s_kd = a.hub_kd[u];
    }
    // Merged only if every chunk aggregated it. The chunks read the hub's
    // flag when they start, and a hub can be marked meanwhile (by a move of
    // its own class, in a kernel running beside the chunks): then some
    // chunks skipped it (count EMPTY) and its partials are incomplete, so it
    // waits for the next iteration and its partial own-community sum is
    // dropped.
    bool stale = false;
    for (uint32_t c = c0 + threadIdx.x; c < c1; c += B) stale |= a.chunk_cnt[c] == EMPTY;
    // spilled: the hub's partials went to its spill table (hub_spill_kernel)
    // and its best community was found there (hub_argmax_kernel)
    const bool spilled = a.spill_keys && a.hub_over[g];
    if (__syncthreads_or(stale)) {
      if (threadIdx.x == 0) { a.hub_kd[u] = 0.f; a.hub_over[g] = 0; a.hub_best[g] = 0; }
      __syncthreads();
      continue;
    }
    const uint32_t dg = a.deg[u];
    const uint32_t d = a.vcom[u];
    if (spilled) {
      const unsigned long long best = a.hub_best[g];
      const float bg = best ? __uint_as_float(uint32_t(best >> 32)) : 0.f;
      const uint32_t bc = best ? 0xFFFFFFFFu - uint32_t(best) : EMPTY;
      __syncthreads();  // every thread has read the best before it is reset
      hub_decide<B, SYNC>(a, G, u, d, dg, dg, a.vtot[u], bg, bc, false, fix, nv, ne, nm, no);
      if (threadIdx.x == 0) { a.hub_over[g] = 0; a.hub_best[g] = 0; }
      __syncthreads();
      continue;
    }
    int lg = min(LOGS, max(1, ceil_log2(2ull * dg)));
    const unsigned limit = (1u << lg) >> 1;
    // a warp per chunk: the chunks' partial lists merge in parallel (a hub of
    // a million edges has ~60 chunks)
    {
      const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
      bool stop = false;
      for (uint32_t c = c0 + warp; c < c1 && !stop; c += B / 32) {
        const uint64_t p = a.hub.chunk_part[c];
        const uint32_t cnt = a.chunk_cnt[c];
        for (uint32_t q = lane; q < cnt; q += 32)
          if (!lt_add(t, lg, a.part_key[p + q], a.part_val[p + q], limit)) {
            s_over = 1;
            stop = true;
            break;
          }
      }
    }
    __syncthreads();
    const unsigned nlist = min(s_used, limit);
    const bool over = s_over;
    bool ok = true;
    uint32_t gcap = 0;
    if (over) {
      lt_reset<B>(t, nlist);
      lg = min(a.glog2, max(1, ceil_log2(2ull * dg)));
      gcap = gkeys ? (1u << lg) : 0;
      if (!gkeys) ok = false;
      for (uint32_t s2 = threadIdx.x; s2 < gcap; s2 += B) { gkeys[s2] = EMPTY; gvals[s2] = 0.f; }
      __syncthreads();
      if (gkeys)
        for (uint32_t c = c0 + (threadIdx.x >> 5); c < c1; c += B / 32) {
          const uint64_t p = a.hub.chunk_part[c];
          const uint32_t cnt = a.chunk_cnt[c];
          for (uint32_t q = threadIdx.x & 31u; q < cnt; q += 32)
            ok &= table_add(gkeys, gvals, lg, a.part_key[p + q], a.part_val[p + q]);
        }
      __syncthreads();
    }
    const float kd = s_kd;
    const double wu = a.vtot[u];
    const float wuf = __double2float_rn(wu);
    const double td = a.ctot[d];
    float bg = 0.f;
    uint32_t bc = EMPTY;
    if (!over) {
      for (unsigned j = threadIdx.x; j < nlist; j += B) {
        const uint32_t s2 = t.list[j];
        if (s2 == EMPTY) continue;
        const uint32_t c = t.keys[s2];
        const float g2 = gain_of(t.vals[s2], kd, wu, wuf, a.ctot[c], td, G.kr);
        if (g2 > 0.f) take_better(bg, bc, g2, c);
      }
    } else {
      for (uint32_t s2 = threadIdx.x; s2 < gcap; s2 += B) {
        const uint32_t c = gkeys[s2];
        if (c == EMPTY) continue;
        const float g2 = gain_of(gvals[s2], kd, wu, wuf, a.ctot[c], td, G.kr);
        if (g2 > 0.f) take_better(bg, bc, g2, c);
      }
    }
    block_argmax<B>(bg, bc, red_g, red_c);
    if (!over) lt_reset<B>(t, nlist);
    hub_decide<B, SYNC>(a, G, u, d, dg, dg, wu, bg, bc, over, fix, nv, ne, nm, no);
    if (threadIdx.x == 0) a.hub_over[g] = 0;
    bad |= !ok;
    __syncthreads();
  }
  flush_counters(a.ctr, a.bin, fix, nv, ne, nm, bad, no);
}

// Hub path with resident tables (MoveArgs::ht): one block per hub of the
// colour class (grid-stride) whose table is good. The candidates are the
// table's communities with a nonzero count, k_d is the own community's count,
// and the move is taken as on the chunked path (hub_decide), which also
// brings the tables of the hub's neighbours that are hubs up to date. No edge
// of the hub is read unless it moves. A hub whose table is bad is left to the
// chunked path, launched after this kernel.
template <int B, bool SYNC>
__global__ void __launch_bounds__(B) hub_table_kernel(MoveArgs a) {
  __shared__ float red_g[B / 32];
  __shared__ uint32_t red_c[B / 32];
  __shared__ int s_go;
  __shared__ float s_kd;
  const size_t h0 = a.hub.hub_begin[a.color], h1 = a.hub.hub_begin[a.color + 1];
  unsigned long long fix = 0, nv = 0, ne = 0, nm = 0, no = 0, slots = 0;
  for (size_t g = h0 + blockIdx.x; g < h1; g += gridDim.x) {
    const uint32_t u = a.hub.hub_vertex[g];
    if (threadIdx.x == 0) {
      const uint32_t h = a.ht.slot[u];
      s_go = a.vaff[u] && (!a.fa || a.fa[u]) && h != NO_HUB && !a.ht.bad[h];
      s_kd = 0.f;
    }
    __syncthreads();
    const bool go = s_go;
    if (go) {
      const GraphOf G(a, u);
      const uint32_t h = a.ht.slot[u];
      const uint32_t d = a.vcom[u];
      const uint64_t o = a.ht.off[h];
      const uint32_t n = 1u << a.ht.lg[h];
      for (uint32_t s2 = threadIdx.x; s2 < n; s2 += B)
        if (a.ht.key[o + s2] == d) s_kd = float(a.ht.cnt[o + s2]);
      __syncthreads();
      const float kd = s_kd;
      const double wu = a.vtot[u], td = a.ctot[d];
      const float wuf = __double2float_rn(wu);
      float bg = 0.f;
      uint32_t bc = EMPTY;
      for (uint32_t s2 = threadIdx.x; s2 < n; s2 += B) {
        const uint32_t c = a.ht.key[o + s2];
        if (c == EMPTY || c == d) continue;
        const uint32_t k = a.ht.cnt[o + s2];
        if (!k) continue;
        const float g2 = gain_of(float(k), kd, wu, wuf, a.ctot[c], td, G.kr);
        if (g2 > 0.f) take_better(bg, bc, g2, c);
      }
      block_argmax<B>(bg, bc, red_g, red_c);
      hub_decide<B, SYNC>(a, G, u, d, a.deg[u], 0, wu, bg, bc, false, fix, nv, ne, nm, no);
      if (threadIdx.x == 0) slots += n;
    }
    __syncthreads();
  }
  flush_counters(a.ctr, NUM_BINS - 1, fix, nv, ne, nm, false, no);
  if (threadIdx.x == 0 && slots) atomicAdd(&a.ctr->ht_slots, slots);
}

int num_sms() {  // SM count of the device, queried once (thread-safe static init)
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

template <int LO, int HI, bool SYNC, bool UNIT, int MINB>
void launch_small(const MoveArgs &a, SmallBins sb, cudaStream_t s) {
  // shared memory of the largest table among the bins (tiles x C x 8 bytes)
  constexpr size_t CMAX = size_t(TILE_BLOCK / (HI <= 1 ? 4 : HI == 2 ? 8 : HI == 3 ? 16 : 32)) *
                          (size_t(4) << HI) * 8;
  auto k = move_small_kernel<LO, HI, SYNC, UNIT, MINB>;
  static bool configured = false;
  if (!configured) { set_smem(k, CMAX); configured = true; }
  const unsigned grid = sb.block_begin[HI - LO + 1];
  if (!grid) return;
  k<<<grid, TILE_BLOCK, CMAX, s>>>(a, sb);
  LVG_CHECK_LAUNCH();
}

template <int T, int C, bool SYNC, bool UNIT>
void launch_tile(const MoveArgs &a, cudaStream_t s) {
  constexpr int TPB = TILE_BLOCK / T;
  const size_t smem = size_t(TPB) * C * 8;
  auto k = move_tile_kernel<T, C, SYNC, UNIT>;
  static bool configured = false;
  if (!configured) { set_smem(k, smem); configured = true; }
  size_t want = (a.count + TPB - 1) / TPB;
  size_t cap = size_t(num_sms()) * (smem > 32 * 1024 ? 3 : 8);
  unsigned grid = unsigned(want < cap ? want : cap);
  if (!grid) return;
  k<<<grid, TILE_BLOCK, smem, s>>>(a);
  LVG_CHECK_LAUNCH();
}

// Block size and shared-table size (log2 slots) of the large-degree kernels.
// Tables of 2^11 slots (a 1024-community claim budget before the global
// fallback) keep several blocks resident per SM; after the first iterations
// a high-degree vertex's neighbours fall into few communities.
constexpr int BIG9_B = 256, BIG9_LOGS = 11;     // degree 513-2048
constexpr int BIG10_B = 256, BIG10_LOGS = 11;   // degree 2049-8192
constexpr int HUBC_B = 256, HUBC_LOGS = 11;     // hub chunks (lvg_tuning::hub_chunk edges each)
constexpr int HUBM_B = 512, HUBM_LOGS = 13;     // hub merge
constexpr int HUBS_B = 256;                     // hub spill
constexpr int HUBT_B = 128;                     // resident hub tables

// Resident blocks of a large-degree kernel on the whole device, queried once.
template <class K>
unsigned resident_blocks(K kernel, int block, size_t smem) {
  int per_sm = 0;
  LVG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem));
  return unsigned(std::max(1, per_sm)) * unsigned(num_sms());
}

template <int B, int LOGS, bool SYNC, bool UNIT>
unsigned big_grid(size_t count, int cap_per_sm) {
  const size_t smem = (size_t(1) << LOGS) * 10;  // keys, values, claimed list
  static const unsigned resident = [&] {
    set_smem(move_big_kernel<B, LOGS, SYNC, UNIT>, smem);
    return resident_blocks(move_big_kernel<B, LOGS, SYNC, UNIT>, B, smem);
  }();
  size_t r = resident;
  if (cap_per_sm > 0) r = std::min(r, size_t(cap_per_sm) * size_t(num_sms()));
  return unsigned(std::min<size_t>(count, r));
}

template <int B, int LOGS, bool SYNC, bool UNIT>
void launch_big(const MoveArgs &a, cudaStream_t s) {
  const size_t smem = (size_t(1) << LOGS) * 10;
  const unsigned grid = big_grid<B, LOGS, SYNC, UNIT>(a.count, a.big_cap);
  if (!grid) return;
  move_big_kernel<B, LOGS, SYNC, UNIT><<<grid, B, smem, s>>>(a);
  LVG_CHECK_LAUNCH();
}

template <bool SYNC, bool UNIT>
void launch_hubs(const MoveArgs &a, cudaStream_t s, cudaStream_t s_tab) {
  const size_t smem1 = (size_t(1) << HUBC_LOGS) * 10, smem2 = (size_t(1) << HUBM_LOGS) * 10;
  const size_t nch = a.hub.chunk_begin[a.color + 1] - a.hub.chunk_begin[a.color];
  const size_t nh = a.hub.hub_begin[a.color + 1] - a.hub.hub_begin[a.color];
  if (!nh) return;
  auto k1 = hub_chunk_kernel<HUBC_B, HUBC_LOGS, UNIT>;
  auto k2 = hub_merge_kernel<HUBM_B, HUBM_LOGS, SYNC>;
  static bool configured = false;
  if (!configured) { set_smem(k1, smem1); set_smem(k2, smem2); configured = true; }
  if (a.ht.key) {
    hub_table_kernel<HUBT_B, SYNC><<<unsigned(std::min<size_t>(nh, size_t(num_sms()) * 8)), HUBT_B, 0,
                                     s_tab ? s_tab : s>>>(a);
    LVG_CHECK_LAUNCH();
  }
  // with resident tables the chunks only mark themselves empty (unless a
  // table went bad): a few blocks per SM loop over them
  const size_t g1 = a.ht.key ? std::min<size_t>(nch, size_t(num_sms()) * 2) : nch;
  k1<<<unsigned(g1), HUBC_B, smem1, s>>>(a);
  LVG_CHECK_LAUNCH();
  if (a.spill_keys) {
    hub_spill_kernel<HUBS_B><<<unsigned(nch), HUBS_B, 0, s>>>(a);
    LVG_CHECK_LAUNCH();
    const size_t slots = a.hub.class_slots[a.color];
    const unsigned grid = unsigned(std::min<size_t>((slots + 255) / 256, size_t(num_sms()) * 8));
    if (grid) {
      hub_argmax_kernel<<<grid, 256, 0, s>>>(a);
      LVG_CHECK_LAUNCH();
    }
  }
  // (with resident tables the merge has only the hubs of bad tables to do:
  // a block per SM, looping over the hubs)
  const size_t g2 = a.ht.key ? std::min<size_t>(size_t(global_table_blocks(nh)), size_t(num_sms()))
                             : size_t(global_table_blocks(nh));
  k2<<<unsigned(g2), HUBM_B, smem2, s>>>(a);
  LVG_CHECK_LAUNCH();
}

template <bool SYNC, bool UNIT>
void launch_bin(int b, const MoveArgs &a, cudaStream_t s) {
  switch (b) {
    case 1: launch_tile<4, 8, SYNC, UNIT>(a, s); break;
    case 2: launch_tile<8, 16, SYNC, UNIT>(a, s); break;
    case 3: launch_tile<16, 32, SYNC, UNIT>(a, s); break;
    case 4: launch_tile<32, 64, SYNC, UNIT>(a, s); break;
    case 5: launch_tile<32, 128, SYNC, UNIT>(a, s); break;
    case 6: launch_tile<32, 256, SYNC, UNIT>(a, s); break;
    case 7: launch_tile<32, 512, SYNC, UNIT>(a, s); break;
    case 8: launch_tile<32, 1024, SYNC, UNIT>(a, s); break;
    case 9: launch_big<BIG9_B, BIG9_LOGS, SYNC, UNIT>(a, s); break;
    case 10: launch_big<BIG10_B, BIG10_LOGS, SYNC, UNIT>(a, s); break;
    default: break;
  }
}

}  // namespace

// Blocks of a large-degree launch (the count of its global table regions).
int move_grid_blocks(int bin, bool sync, bool unit, size_t count, int big_cap) {
  if (bin == 9) {
    if (sync) return int(unit ? big_grid<BIG9_B, BIG9_LOGS, true, true>(count, big_cap)
                              : big_grid<BIG9_B, BIG9_LOGS, true, false>(count, big_cap));
    return int(unit ? big_grid<BIG9_B, BIG9_LOGS, false, true>(count, big_cap)
                    : big_grid<BIG9_B, BIG9_LOGS, false, false>(count, big_cap));
  }
  if (bin == 10) {
    if (sync) return int(unit ? big_grid<BIG10_B, BIG10_LOGS, true, true>(count, big_cap)
                              : big_grid<BIG10_B, BIG10_LOGS, true, false>(count, big_cap));
    return int(unit ? big_grid<BIG10_B, BIG10_LOGS, false, true>(count, big_cap)
                    : big_grid<BIG10_B, BIG10_LOGS, false, false>(count, big_cap));
  }
  return global_table_blocks(count);  // the hub merge
}

int global_table_blocks(size_t count) {
  size_t cap = size_t(num_sms()) * 3;
  return int(count < cap ? count : cap);
}

// The kernel variants: deterministic or not, unit weights (no weight
// reads) or not.
void launch_move_hubs(bool sync, const MoveArgs &a, cudaStream_t s, cudaStream_t s_tab) {
  if (sync) { if (a.unit) launch_hubs<true, true>(a, s, s_tab); else launch_hubs<true, false>(a, s, s_tab); }
  else if (a.unit) launch_hubs<false, true>(a, s, s_tab);
  else launch_hubs<false, false>(a, s, s_tab);
}

int device_sms() { return num_sms(); }

template <int MINB>
void launch_small_1_6(bool sync, const MoveArgs &a, const SmallBins &sb, cudaStream_t s) {
  if (sync) {
    if (a.unit) launch_small<1, 6, true, true, MINB>(a, sb, s);
    else launch_small<1, 6, true, false, MINB>(a, sb, s);
  } else if (a.unit) {
    launch_small<1, 6, false, true, MINB>(a, sb, s);
  } else {
    launch_small<1, 6, false, false, MINB>(a, sb, s);
  }
}

void launch_move_small(int lo, int hi, bool sync, const MoveArgs &a, const SmallBins &sb, cudaStream_t s,
                       int small_regs) {
  if (lo == 1 && hi == 6) {
    if (small_regs == 64) launch_small_1_6<4>(sync, a, sb, s);
    else launch_small_1_6<8>(sync, a, sb, s);
  } else if (lo == 7 && hi == 8) {
    if (sync) {
      if (a.unit) launch_small<7, 8, true, true, 1>(a, sb, s);
      else launch_small<7, 8, true, false, 1>(a, sb, s);
    } else if (a.unit) {
      launch_small<7, 8, false, true, 1>(a, sb, s);
    } else {
      launch_small<7, 8, false, false, 1>(a, sb, s);
    }
  } else {
    throw Error(LVG_EINVAL, "launch_move_small: unsupported bin range");
  }
}

void launch_move_bin(int b, bool sync, const MoveArgs &a, cudaStream_t s) {
  if (sync) { if (a.unit) launch_bin<true, true>(b, a, s); else launch_bin<true, false>(b, a, s); }
  else if (a.unit) launch_bin<false, true>(b, a, s);
  else launch_bin<false, false>(b, a, s);
}

}  // namespace lvg
