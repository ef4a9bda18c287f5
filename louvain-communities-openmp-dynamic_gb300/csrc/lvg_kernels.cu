// lvg_kernels.cu — initialisation, batch-update, marking, renumbering,
// community-CSR and modularity kernels.
#include <algorithm>

#include "lvg_internal.cuh"

namespace lvg {
namespace {

int sms() {  // SM count of the device, queried once (thread-safe static init)
  static const int n = [] {
    int dev = 0, c = 0;
    LVG_CUDA(cudaGetDevice(&dev));
    LVG_CUDA(cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev));
    return c;
  }();
  return n;
}

#define GRID_STRIDE(i, n) for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < (n); i += size_t(gridDim.x) * blockDim.x)

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void block_add_double(double v, double *dst) {
  __shared__ double red[32];
  v = warp_sum_d(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double t = lane < int(blockDim.x >> 5) ? red[lane] : 0.0;
    t = warp_sum_d(t);
    if (lane == 0 && t != 0.0) atomicAdd(dst, t);
  }
}

__global__ void degrees_kernel(const uint64_t *off, uint32_t *deg, size_t n) {
  GRID_STRIDE(u, n) deg[u] = uint32_t(off[u + 1] - off[u]);
}

// louvainVertexWeightsOmpW (inc/louvain.hxx:210) + louvainInitializeOmpW
// (:285) for level 0: one warp per vertex (lane-strided rows).
__global__ void init_static_kernel(const uint64_t *off, const uint32_t *deg, const float *w, const uint8_t *ex,
                                   size_t n, const uint32_t *gid, const uint32_t *gbase, uint32_t *ucom, tot_t *utot,
                                   tot_t *ctot) {
  const size_t warps = size_t(gridDim.x) * blockDim.x / 32;
  const int lane = threadIdx.x & 31;
  for (size_t u = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; u < n; u += warps) {
    const bool has = !ex || ex[u];
    double s = 0.0;  // FP64, as the reference's vector<W> (exact for integer weights)
    if (has) {
      const uint64_t o = off[u];
      const uint32_t d = deg[u];
      for (uint32_t j = lane; j < d; j += 32) s += double(w[o + j]);
#pragma unroll
      for (int k = 16; k > 0; k >>= 1) s += __shfl_xor_sync(0xffffffffu, s, k);
    }
    if (lane == 0) {
      // an absent vertex starts in community 0 (of its own graph in a union)
      ucom[u] = has ? uint32_t(u) : (gid ? gbase[gid[u]] : 0u);
      utot[u] = s;
      ctot[u] = s;
    }
  }
}

__global__ void count_nonunit_kernel(const float *w, size_t m, unsigned long long *dst) {
  unsigned long long c = 0;
  GRID_STRIDE(i, m) c += w[i] != 1.0f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(dst, c);
}

__global__ void total_weight_kernel(const float *w, size_t m, double *dst) {
  double s = 0;
  GRID_STRIDE(i, m) s += (double)w[i];
  block_add_double(s, dst);
}

// louvainVertexWeightsOmpW in FP64: a warp per row.
__global__ void vertex_weights_f64_kernel(const uint64_t *off, const uint32_t *deg, const float *w, const uint8_t *ex,
                                          size_t n, double *vtot) {
  const size_t warps = size_t(gridDim.x) * blockDim.x / 32;
  const int lane = threadIdx.x & 31;
  for (size_t u = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; u < n; u += warps) {
    double s = 0;
    if (!ex || ex[u]) {
      const uint64_t o = off[u];
      for (uint32_t j = lane; j < deg[u]; j += 32) s += double(w[o + j]);
      s = warp_sum_d(s);
    }
    if (lane == 0) vtot[u] = s;
  }
}

// louvainCommunityWeightsOmpW in FP64: ctot[q[u]] += vtot[u].
__global__ void community_weights_f64_kernel(const uint32_t *q, const double *vtot, size_t n, double *ctot) {
  GRID_STRIDE(u, n) if (vtot[u] != 0.0) atomicAdd(&ctot[q[u]], vtot[u]);
}

__global__ void fill_f32_kernel(float *p, size_t n, float v) {
  GRID_STRIDE(i, n) p[i] = v;
}

// louvainUpdateWeightsFromOmpU (inc/louvain.hxx:374-388): per directed batch
// edge, the source's weight and its community's total move by the weight.
// Lanes of a warp with the same source (the batch is source-sorted) or the
// same community add their weights first and the lowest of them adds the sum:
// a large community would otherwise take thousands of atomics on one word.
__device__ __forceinline__ void group_add(tot_t *p, uint32_t key, double x, int lane) {
  const unsigned grp = __match_any_sync(0xffffffffu, key);
  double sum = 0.0;
  for (unsigned r = grp; r; r &= r - 1u) sum += __shfl_sync(grp, x, __ffs(r) - 1);
  if (key != EMPTY && (grp & ((1u << lane) - 1u)) == 0u) atomicAdd(p + key, sum);
}

__global__ void batch_weights_kernel(const uint32_t *src, const float *w, size_t n, float sign,
                                     const uint32_t *vcom, tot_t *vtot, tot_t *ctot) {
  const int lane = threadIdx.x & 31;
  for (size_t base = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32 * 32; base < n;
       base += size_t(gridDim.x) * blockDim.x) {
    const size_t i = base + lane;
    uint32_t u = EMPTY, c = EMPTY;
    double x = 0.0;
    if (i < n) {
      u = src[i];
      x = double(sign) * double(w[i]);
      if (ctot) c = vcom[u];
    }
    if (vtot) group_add(vtot, u, x, lane);  // either side may be left out
    if (ctot) group_add(ctot, c, x, lane);
  }
}

// louvainAffectedVerticesFrontierOmpW (inc/louvain.hxx:1606-1624).
__global__ void df_mark_kernel(const uint32_t *ds, const uint32_t *dd, size_t nd, const uint32_t *is,
                               const uint32_t *id, size_t ni, const uint32_t *vcom, uint8_t *vaff) {
  GRID_STRIDE(i, nd + ni) {
    if (i < nd) {
      if (vcom[ds[i]] == vcom[dd[i]]) vaff[ds[i]] = 1;
    } else {
      const size_t j = i - nd;
      if (vcom[is[j]] != vcom[id[j]]) vaff[is[j]] = 1;
    }
  }
}

// Dynamic-frontier Louvain's start: louvainUpdateWeightsFromOmpU
// (inc/louvain.hxx:374-388, deletions subtracted, insertions added, summed
// per warp by vertex and by community as batch_weights_kernel does) and
// louvainAffectedVerticesFrontierOmpW (:1606-1624) in one pass over the
// batch, entry i < nd a deletion, else insertion i - nd. Both read only the
// prior membership. A source that exists with degree 0 is left unmarked: the
// local-moving sweep would clear its flag without moving it, and no move marks
// it again (it has no neighbours), so the residual flags are the same.
// With wl (one colour class), a vertex's first marker (an atomic OR on the
// flag's word, so the vertex is listed once) appends it to the worklist of its
// degree bin, at the class's bin offsets, bounded by the bin's slice like the
// compaction's appends; pre_flag then tells the first compaction to take
// these lists.
__global__ void df_start_kernel(const uint32_t *ds, const uint32_t *dd, const float *dw, size_t nd,
                                const uint32_t *is, const uint32_t *id, const float *iw, size_t ni,
                                const uint32_t *vcom, tot_t *vtot, tot_t *ctot, const uint32_t *deg,
                                const uint8_t *ex, BinLimits lim, uint8_t *vaff, BinBounds bb, uint32_t *wl,
                                Counters *ctr) {
  const int lane = threadIdx.x & 31;
  const size_t n = nd + ni;
  if (wl && blockIdx.x == 0 && threadIdx.x == 0) ctr->pre_flag = 1u;
  for (size_t base = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32 * 32; base < n;
       base += size_t(gridDim.x) * blockDim.x) {
    const size_t i = base + lane;
    uint32_t u = EMPTY, c = EMPTY;
    double x = 0.0;
    bool mark = false;
    if (i < n) {
      const bool del = i < nd;
      const size_t j = del ? i : i - nd;
      u = del ? ds[j] : is[j];
      const uint32_t v = del ? dd[j] : id[j];
      x = del ? -double(dw[j]) : double(iw[j]);
      c = vcom[u];
      mark = del ? c == vcom[v] : c != vcom[v];
    }
    if (vtot) group_add(vtot, u, x, lane);  // (nullptr: updated before the run)
    group_add(ctot, c, x, lane);
    int b = -1;
    if (mark) {
      const uint32_t d = deg[u];
      if (d == 0 && (!ex || ex[u])) {
        mark = false;
      } else if (!wl) {
        vaff[u] = 1;
      } else {
        const unsigned sh = 8u * (u & 3u);
        const unsigned old = atomicOr(reinterpret_cast<unsigned int *>(vaff) + (u >> 2), 1u << sh);
        if (!((old >> sh) & 0xffu)) {  // the first to mark u lists it
          const int x2 = degree_bin(d, lim);
          if (x2 >= 1 && x2 <= NUM_BINS - 2) b = x2;
        }
      }
    }
    if (wl) {
      const unsigned grp = __match_any_sync(0xffffffffu, b);
      const int leader = __ffs(grp) - 1;
      uint32_t at = 0;
      if (b >= 0 && lane == leader) at = atomicAdd(&ctr->pre_count[b], uint32_t(__popc(grp)));
      at = __shfl_sync(0xffffffffu, at, leader);
      if (b >= 0) {
        const uint32_t slot = at + __popc(grp & ((1u << lane) - 1u));
        if (slot < bb.start[b + 1] - bb.start[b]) wl[bb.start[b] + slot] = u;
        else atomicOr(&ctr->err, ERR_WORKLIST);
      }
    }
  }
}

// Delta-screening, deletions (inc/louvain.hxx:1448-1456).
__global__ void ds_del_kernel(const uint32_t *ds, const uint32_t *dd, size_t nd, const uint32_t *vcom,
                              uint8_t *vertices, uint8_t *neighbors, uint8_t *communities) {
  GRID_STRIDE(i, nd) {
    const uint32_t u = ds[i], v = dd[i];
    if (vcom[u] != vcom[v]) continue;
    vertices[u] = 1;
    neighbors[u] = 1;
    communities[vcom[v]] = 1;
  }
}

__device__ __forceinline__ double delta_modularity(double vcout, double vdout, double vtot, double ctot,
                                                   double dtot, double M, double R) {
  return (vcout - vdout) / M - R * vtot * (vtot + ctot - dtot) / (2 * M * M);
}

// Delta-screening, insertions (inc/louvain.hxx:1457-1479): one block per
// source; the inserted cross-community edges are merged per community, the
// best community is chosen by the reference's FP64 ΔQ with its tie rule
// (first community in batch order wins), and if the gain is positive the
// source, its neighbours and that community are flagged. The FP64 here is
// batch sized; it makes the flags match the reference bit for bit.
constexpr int DS_BLOCK = 128;
constexpr int DS_LOG = 11;  // shared table: 2048 slots, sources with <= 1024 insertions
// The sources with more than 32 insertions come listed by ds_ins_warp_kernel
// after the segment heads (seg[ns + k] = first insertion of long source k).
__global__ void __launch_bounds__(DS_BLOCK) ds_ins_kernel(const uint32_t *is, const uint32_t *id, const float *iw,
                                                          size_t ni, const uint32_t *seg, const unsigned int *nseg,
                                                          const unsigned int *nlong, const uint32_t *vcom,
                                                          const tot_t *vtot, const tot_t *ctot, double M, double R,
                                                          uint8_t *vertices, uint8_t *neighbors,
                                                          uint8_t *communities, uint32_t *gkeys, float *gvals,
                                                          uint32_t *gfirst, int glog2, Counters *ctr) {
  __shared__ uint32_t skeys[1 << DS_LOG];
  __shared__ float svals[1 << DS_LOG];
  __shared__ uint32_t sfirst[1 << DS_LOG];
  __shared__ double rb[DS_BLOCK / 32];
  __shared__ uint32_t rf[DS_BLOCK / 32], rc[DS_BLOCK / 32];
  const unsigned ns = *nseg, nl = *nlong;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (unsigned k = blockIdx.x; k < nl; k += gridDim.x) {
    const size_t s0 = seg[ns + k];
    const uint32_t u = is[s0];
    // segment end: first index with a larger source (the batch is sorted)
    size_t lo = s0 + 33, hi = ni;
    while (lo < hi) {
      size_t mid = (lo + hi) >> 1;
      if (is[mid] <= u) lo = mid + 1; else hi = mid;
    }
    const size_t s1 = lo, len = s1 - s0;
    const bool global = len * 2 > (size_t(1) << DS_LOG);
    // a table sized for the segment: clearing and scanning all 2048 slots
    // would cost more than the insertions of a source with a few dozen
    const int lg = global ? glog2 : max(1, ceil_log2(2 * len));
    const uint32_t cap = 1u << lg, mask = cap - 1u;
    uint32_t *keys = global ? gkeys + size_t(blockIdx.x) * cap : skeys;
    float *vals = global ? gvals + size_t(blockIdx.x) * cap : svals;
    uint32_t *first = global ? gfirst + size_t(blockIdx.x) * cap : sfirst;
    for (uint32_t s = threadIdx.x; s < cap; s += DS_BLOCK) { keys[s] = EMPTY; vals[s] = 0.f; first[s] = 0xffffffffu; }
    __syncthreads();
    const uint32_t d = vcom[u];
    bool ok = true;
    for (size_t j = s0 + threadIdx.x; j < s1; j += DS_BLOCK) {
      const uint32_t c = vcom[id[j]];
      if (c == d) continue;
      uint32_t sl = hash_hi(c, lg);
      bool done = false;
      for (uint32_t probe = 0; probe <= mask && !done; ++probe) {
        uint32_t k = keys[sl];
        if (k == EMPTY) {
          uint32_t prev = atomicCAS(&keys[sl], EMPTY, c);
          k = prev == EMPTY ? c : prev;
        }
        if (k == c) {
          atomicAdd(&vals[sl], iw[j]);
          atomicMin(&first[sl], uint32_t(j - s0));
          done = true;
        }
        sl = (sl + 1u) & mask;
      }
      ok &= done;
    }
    __syncthreads();
    const double vu = vtot[u], td = ctot[d];
    double be = 0;
    uint32_t bf = 0xffffffffu, bc = 0;
    for (uint32_t s = threadIdx.x; s < cap; s += DS_BLOCK) {
      const uint32_t c = keys[s];
      if (c == EMPTY) continue;
      const double e = delta_modularity((double)vals[s], 0.0, vu, (double)ctot[c], td, M, R);
      if (e > be || (e == be && e > 0 && first[s] < bf)) { be = e; bf = first[s]; bc = c; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double oe = __shfl_xor_sync(0xffffffffu, be, o);
      const uint32_t of = __shfl_xor_sync(0xffffffffu, bf, o);
      const uint32_t oc = __shfl_xor_sync(0xffffffffu, bc, o);
      if (oe > be || (oe == be && oe > 0 && of < bf)) { be = oe; bf = of; bc = oc; }
    }
    if (lane == 0) { rb[wid] = be; rf[wid] = bf; rc[wid] = bc; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double e = 0;
      uint32_t f = 0xffffffffu, c = 0;
      for (int k = 0; k < DS_BLOCK / 32; ++k)
        if (rb[k] > e || (rb[k] == e && rb[k] > 0 && rf[k] < f)) { e = rb[k]; f = rf[k]; c = rc[k]; }
      if (e > 0) {
        vertices[u] = 1;
        neighbors[u] = 1;
        communities[c] = 1;
      }
      if (!ok) atomicOr(&ctr->err, ERR_TABLE_FULL);
    }
    __syncthreads();
  }
}

// Constants of the FP32 screen of ds_ins_warp_kernel. In range (ok), every
// intermediate stays a normal float: M in [1e-15, 1e15], R in (0, 1e6], and
// |vtot|, |ctot| <= 2M. The screened gain x - y, x = vcout/M, y =
// R vtot (vtot + ctot_c - ctot_d) / (2M^2), takes about ten roundings of
// 2^-24 relative to |x| and to yb = R |vtot| (|vtot| + |ctot_c| + |ctot_d|) /
// (2M^2) (the constants' conversions and the FP32 roundings of the FP64
// totals included; the cancellation in vtot + ctot_c - ctot_d is bounded by
// yb's terms), and the reference's FP64
// value differs from the exact one by about 2^-50 of the same; 2^-20 covers
// both with room. DS_SCREEN_ABS covers results below the normal range.
struct DsScreen {
  float invM, inv2MM, R;
  bool ok;
};
constexpr float DS_SCREEN_REL = 9.5367431640625e-07f;  // 2^-20
constexpr float DS_SCREEN_ABS = 1e-36f;

// The same for sources with at most 32 insertions (nearly all of them): a
// warp per source, lane k holding insertion k; lanes of the same community
// sum their weights in batch order and the lowest of them (the community's
// first insertion) carries it into the argmax.
__global__ void ds_ins_warp_kernel(const uint32_t *is, const uint32_t *id, const float *iw, size_t ni,
                                   uint32_t *seg, const unsigned int *nseg, unsigned int *nlong, const uint32_t *vcom,
                                   const tot_t *vtot, const tot_t *ctot, double M, double R, DsScreen sc,
                                   uint8_t *vertices, uint8_t *neighbors, uint8_t *communities) {
  const unsigned ns = *nseg;
  const int lane = threadIdx.x & 31;
  const size_t warps = size_t(gridDim.x) * blockDim.x / 32;
  for (size_t sidx = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; sidx < ns; sidx += warps) {
    const size_t s0 = seg[sidx];
    const uint32_t u = is[s0];
    const size_t j = s0 + 1 + lane;
    const unsigned past = __ballot_sync(0xffffffffu, j >= ni || is[j] != u);
    if (!past) {  // more than 32 insertions: listed for ds_ins_kernel (warp-uniform)
      // ns segments of which L have 33 or more insertions: ns + L <= ni, the
      // capacity of seg
      if (lane == 0) seg[ns + atomicAdd(nlong, 1u)] = uint32_t(s0);
      continue;
    }
    const uint32_t len = uint32_t(__ffs(past));  // 1 + the lanes still in the segment
    const uint32_t d = vcom[u];
    uint32_t c = EMPTY;
    float w = 0.f;
    if (uint32_t(lane) < len) {
      c = vcom[id[s0 + lane]];
      w = iw[s0 + lane];
      if (c == d) c = EMPTY;
    }
    const unsigned grp = __match_any_sync(0xffffffffu, c);
    float sum = 0.f;
    for (unsigned r = grp; r; r &= r - 1u) sum += __shfl_sync(grp, w, __ffs(r) - 1);
    const bool leader = c != EMPTY && (grp & ((1u << lane) - 1u)) == 0u;
    // FP32 screen: e32 is the gain within er of the exact value, and of the
    // reference's FP64 value too; when every sign and the winner are clear by
    // more than the bound, FP64 (slow on this part) is skipped
    const double vu64 = vtot[u], td64 = ctot[d];
    const float vu = float(vu64), td = float(td64);
    float e32 = 0.f, er = 0.f;
    if (leader) {
      const float tc = float(ctot[c]);
      const float x = sum * sc.invM;
      const float y = sc.R * vu * (vu + tc - td) * sc.inv2MM;
      const float yb = sc.R * fabsf(vu) * (fabsf(vu) + fabsf(tc) + fabsf(td)) * sc.inv2MM;
      e32 = x - y;
      er = DS_SCREEN_REL * (fabsf(x) + yb) + DS_SCREEN_ABS;
    }
    const unsigned cand = __ballot_sync(0xffffffffu, leader);
    const unsigned pos = __ballot_sync(0xffffffffu, leader && e32 > er);
    const unsigned neg = __ballot_sync(0xffffffffu, leader && e32 < -er);
    bool slow = !sc.ok || (pos | neg) != cand;
    bool flag = false;
    uint32_t bc = 0;
    if (!slow && pos) {
      const bool mine = (pos >> lane) & 1u;
      float bv = mine ? e32 : -INFINITY;
      int bl = lane;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int ol = __shfl_xor_sync(0xffffffffu, bl, o);
        if (ov > bv || (ov == bv && ol < bl)) { bv = ov; bl = ol; }
      }
      const float lo = __shfl_sync(0xffffffffu, e32 - er, bl);
      const unsigned amb = __ballot_sync(0xffffffffu, mine && lane != bl && e32 + er >= lo);
      slow = amb != 0u;
      flag = !slow;
      bc = __shfl_sync(0xffffffffu, c, bl);
    }
    if (slow) {  // the reference's FP64 rule (warp-uniform branch)
      double be = 0;
      uint32_t bf = 0xffffffffu;
      bc = 0;
      if (leader) {
        const double e = delta_modularity(double(sum), 0.0, vu64, ctot[c], td64, M, R);
        if (e > 0) { be = e; bf = uint32_t(lane); bc = c; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double oe = __shfl_xor_sync(0xffffffffu, be, o);
        const uint32_t of = __shfl_xor_sync(0xffffffffu, bf, o);
        const uint32_t oc = __shfl_xor_sync(0xffffffffu, bc, o);
        if (oe > be || (oe == be && oe > 0 && of < bf)) { be = oe; bf = of; bc = oc; }
      }
      flag = be > 0;
    }
    if (lane == 0 && flag) {
      vertices[u] = 1;
      neighbors[u] = 1;
      communities[bc] = 1;
    }
  }
}

// The insertions, a warp per 32 consecutive entries (the first pass): a
// source whose insertions all lie in the warp's window and whose screen is
// clear (no gain within the bound of zero, the best clear of the others) is
// settled here; the others' first insertions are listed in seg (count nseg)
// for ds_ins_warp_kernel. Lanes of the same source and community sum their
// weights in batch order (the reference's vcout); the lowest of them stands
// for the community, so lane order is the reference's scan order.
__global__ void ds_ins_lane_kernel(const uint32_t *is, const uint32_t *id, const float *iw, size_t ni,
                                   uint32_t *seg, unsigned int *nseg, const uint32_t *vcom, const tot_t *vtot,
                                   const tot_t *ctot, DsScreen sc, uint8_t *vertices, uint8_t *neighbors,
                                   uint8_t *communities) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  for (size_t base = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32 * 32; base < ni;
       base += size_t(gridDim.x) * blockDim.x) {
    const size_t j = base + lane;
    const bool in = j < ni;
    const uint32_t u = in ? is[j] : EMPTY;
    // the source before the window (lane 0) and after it (lane 31)
    uint32_t edge = EMPTY;
    if (lane == 0 && base > 0) edge = is[base - 1];
    if (lane == 31 && j + 1 < ni) edge = is[j + 1];
    const uint32_t before = __shfl_sync(0xffffffffu, edge, 0), after = __shfl_sync(0xffffffffu, edge, 31);
    const uint32_t u0 = __shfl_sync(0xffffffffu, u, 0), u31 = __shfl_sync(0xffffffffu, u, 31);
    const bool foreign = in && u == u0 && before == u0;  // its head is in an earlier window
    const bool crossing = in && u == u31 && after == u31;  // it goes on past the window
    const bool local = in && !foreign && !crossing;
    const unsigned segm = __match_any_sync(0xffffffffu, u);  // the source's lanes (contiguous)
    const int h = __ffs(segm) - 1, t = 31 - __clz(segm);
    uint32_t c = EMPTY, d = 0;
    float w = 0.f;
    if (local) {
      d = vcom[u];
      c = vcom[id[j]];
      w = iw[j];
      if (c == d) c = EMPTY;
    }
    const unsigned grp = __match_any_sync(0xffffffffu, (uint64_t(u) << 32) | c);
    float sum = 0.f;
    for (unsigned r = grp; r; r &= r - 1u) sum += __shfl_sync(grp, w, __ffs(r) - 1);
    const bool leader = c != EMPTY && (grp & below) == 0u;
    float e32 = 0.f, er = 0.f;
    if (leader) {
      const float vu = float(vtot[u]), td = float(ctot[d]), tc = float(ctot[c]);
      const float x = sum * sc.invM;
      const float y = sc.R * vu * (vu + tc - td) * sc.inv2MM;
      const float yb = sc.R * fabsf(vu) * (fabsf(vu) + fabsf(tc) + fabsf(td)) * sc.inv2MM;
      e32 = x - y;
      er = DS_SCREEN_REL * (fabsf(x) + yb) + DS_SCREEN_ABS;
    }
    const bool pos = leader && e32 > er;
    const unsigned cand = __ballot_sync(0xffffffffu, leader);
    const unsigned unc = __ballot_sync(0xffffffffu, leader && !pos && !(e32 < -er));
    const unsigned posm = __ballot_sync(0xffffffffu, pos);
    // the largest screened gain of each source (lowest lane on ties): a scan
    // over the source's lanes, read at its last lane
    float bv = pos ? e32 : -INFINITY;
    int bl = lane;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float ov = __shfl_up_sync(0xffffffffu, bv, o);
      const int ol = __shfl_up_sync(0xffffffffu, bl, o);
      if (lane - o >= h && (ov > bv || (ov == bv && ol < bl))) { bv = ov; bl = ol; }
    }
    const int best = __shfl_sync(0xffffffffu, bl, t);
    const float lo = __shfl_sync(0xffffffffu, e32 - er, best);
    const uint32_t bc = __shfl_sync(0xffffffffu, c, best);
    const unsigned amb = __ballot_sync(0xffffffffu, pos && lane != best && e32 + er >= lo);
    const bool slow = ((unc | amb) & segm) != 0u || (!sc.ok && (cand & segm) != 0u);
    // heads of the sources left to the per-source pass
    const bool head = lane == h && in && !foreign;
    const bool list = head && (crossing || slow);
    const unsigned lm = __ballot_sync(0xffffffffu, list);
    unsigned at = 0;
    if (lm && lane == __ffs(lm) - 1) at = atomicAdd(nseg, unsigned(__popc(lm)));
    at = __shfl_sync(0xffffffffu, at, __ffs(lm ? lm : 1u) - 1);
    if (list) seg[at + __popc(lm & below)] = uint32_t(j);
    if (head && local && !slow && (posm & segm)) {
      vertices[u] = 1;
      neighbors[u] = 1;
      communities[bc] = 1;
    }
  }
}

// Delta-screening expansion (inc/louvain.hxx:1480-1485): members of flagged
// communities (a thread per vertex), and the vertices flagged for their
// neighbours, listed for ds_neighbors_kernel: those of degree up to
// DS_WARP_DEG from the front of the list (count[0]), the others from its back
// (count[1]); the list holds n entries.
constexpr uint32_t DS_WARP_DEG = 256;
__global__ void ds_expand_kernel(const uint8_t *ex, size_t n, const uint32_t *vcom, const uint32_t *deg,
                                 const uint8_t *neighbors, const uint8_t *communities, uint8_t *vertices,
                                 uint32_t *list, uint32_t *count) {
  const int lane = threadIdx.x & 31;
  for (size_t base = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32 * 32; base < n;
       base += size_t(gridDim.x) * blockDim.x) {
    const size_t u = base + lane;
    const bool has = u < n && (!ex || ex[u]);
    if (has && communities[vcom[u]]) vertices[u] = 1;
    const bool nb = has && neighbors[u];
    const bool big = nb && deg[u] > DS_WARP_DEG;
    const unsigned m = __ballot_sync(0xffffffffu, nb && !big), mb = __ballot_sync(0xffffffffu, big);
    uint32_t at = 0, atb = 0;
    if (m && lane == __ffs(m) - 1) at = atomicAdd(&count[0], uint32_t(__popc(m)));
    if (mb && lane == __ffs(mb) - 1) atb = atomicAdd(&count[1], uint32_t(__popc(mb)));
    at = __shfl_sync(0xffffffffu, at, __ffs(m ? m : 1u) - 1);
    atb = __shfl_sync(0xffffffffu, atb, __ffs(mb ? mb : 1u) - 1);
    const unsigned below = (1u << lane) - 1u;
    if (nb && !big) list[at + __popc(m & below)] = uint32_t(u);
    if (big) list[n - 1 - (atb + __popc(mb & below))] = uint32_t(u);
  }
}

// Set a flag that is most often set already (the neighbours of hubs repeat):
// the read usually hits L1, where the plain store would go to L2 every time.
// A stale 0 only costs a redundant store; a flag is never cleared here.
__device__ __forceinline__ void mark_once(uint8_t *flags, uint32_t v) {
  if (!flags[v]) flags[v] = 1;
}

// The neighbours of the listed vertices: a warp per vertex up to degree
// DS_WARP_DEG (ds_neighbors_kernel); above it, chunks of DS_WARP_DEG edges
// balanced over the blocks (ds_neighbors_big_kernel).
__global__ void ds_neighbors_kernel(const uint64_t *off, const uint32_t *deg, const uint32_t *key,
                                    const uint32_t *list, const uint32_t *count, uint8_t *vertices) {
  const uint32_t nw = count[0];
  const int lane = threadIdx.x & 31;
  const size_t warps = size_t(gridDim.x) * blockDim.x / 32;
  for (size_t i = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; i < nw; i += warps) {
    const uint32_t u = list[i];
    const uint64_t o = off[u];
    const uint32_t d = deg[u];
    for (uint32_t j = lane; j < d; j += 32) mark_once(vertices, key[o + j]);
  }
}

// Per listed vertex above DS_WARP_DEG (list[n - 1 - i], i < count[1]), its
// 256-edge chunks; zero past the list (the whole array is scanned).
__global__ void ds_big_chunks_kernel(const uint32_t *deg, const uint32_t *list, const uint32_t *count, size_t n,
                                     uint32_t *chunks) {
  const uint32_t nb = count[1];
  GRID_STRIDE(i, n) chunks[i] = i < nb ? (deg[list[n - 1 - i]] + DS_WARP_DEG - 1) / DS_WARP_DEG : 0u;
}

// The adjacencies of those vertices with each block taking an equal range of
// the chunks (chunks = their exclusive prefix, total = the chunk count): a hub
// is spread over many blocks, and no block waits on one.
__global__ void ds_neighbors_big_kernel(const uint64_t *off, const uint32_t *deg, const uint32_t *key,
                                        const uint32_t *list, const uint32_t *count, size_t n,
                                        const uint32_t *chunks, const uint32_t *total, uint8_t *vertices) {
  __shared__ uint32_t first;
  const uint32_t nb = count[1], T = *total;
  const uint32_t t0 = uint32_t(uint64_t(T) * blockIdx.x / gridDim.x);
  const uint32_t t1 = uint32_t(uint64_t(T) * (blockIdx.x + 1) / gridDim.x);
  if (t0 >= t1) return;  // block-uniform
  if (threadIdx.x == 0) {  // the vertex holding chunk t0: the last i with chunks[i] <= t0
    uint32_t lo = 0, hi = nb;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (chunks[mid] <= t0) lo = mid; else hi = mid;
    }
    first = lo;
  }
  __syncthreads();
  for (uint32_t i = first, t = t0; t < t1; ++i) {
    const uint32_t u = list[n - 1 - i];
    const uint64_t o = off[u];
    const uint32_t d = deg[u];
    const uint32_t cb = chunks[i], ce = i + 1 < nb ? chunks[i + 1] : T;
    const uint32_t stop = min(ce, t1);
    const uint32_t e1 = min(d, (stop - cb) * DS_WARP_DEG);
    for (uint32_t j = (t - cb) * DS_WARP_DEG + threadIdx.x; j < e1; j += blockDim.x) mark_once(vertices, key[o + j]);
    t = stop;
  }
}

__global__ void clear_isolated_kernel(const uint32_t *list, size_t n, uint8_t *vaff, const uint8_t *fa) {
  GRID_STRIDE(i, n) {
    const uint32_t u = list[i];
    if (vaff[u] && (!fa || fa[u])) vaff[u] = 0;
  }
}

// The same over several lists (the degree-0 buckets of every colour class):
// block b serves list b % k.
__global__ void clear_isolated_multi_kernel(IsolatedLists L, uint8_t *vaff, const uint8_t *fa) {
  const int j = blockIdx.x % L.k;
  const size_t nb = gridDim.x / L.k + (size_t(j) < gridDim.x % L.k ? 1 : 0);
  const size_t blk = blockIdx.x / L.k;
  for (size_t i = blk * blockDim.x + threadIdx.x; i < L.n[j]; i += nb * blockDim.x) {
    const uint32_t u = L.list[j][i];
    if (vaff[u] && (!fa || fa[u])) vaff[u] = 0;
  }
}

// The dynamic-frontier first pass: its only affected vertices of degree 0
// are batch endpoints (the marking touches nothing else, and moves mark
// neighbours only), so the clearing of isolated vertices needs only those.
__global__ void clear_isolated_endpoints_kernel(const uint32_t *a, size_t na, const uint32_t *b, size_t nb,
                                                const uint32_t *deg, const uint8_t *ex, uint8_t *vaff) {
  GRID_STRIDE(i, na + nb) {
    const uint32_t u = i < na ? a[i] : b[i - na];
    if (deg[u] == 0 && (!ex || ex[u])) vaff[u] = 0;
  }
}

__global__ void merge_marks_kernel(uint8_t *vaff, uint8_t *mark, size_t n) {
  GRID_STRIDE(i, n) {
    if (mark[i]) { vaff[i] = 1; mark[i] = 0; }
  }
}

// Deterministic mode: commit the decisions of one colour class (the moves of
// louvainChangeCommunityOmpW, inc/louvain.hxx:496-503, applied after every
// vertex of the class has decided from the same state).
__global__ void apply_moves_kernel(const uint32_t *list, size_t n, uint32_t *dec, uint32_t *vcom, tot_t *ctot,
                                   const tot_t *vtot) {
  GRID_STRIDE(i, n) {
    const uint32_t u = list[i];
    const uint32_t c = dec[u];
    if (c == EMPTY) continue;
    const uint32_t d = vcom[u];
    atomicAdd(&ctot[d], -vtot[u]);
    atomicAdd(&ctot[c], vtot[u]);
    vcom[u] = c;
    dec[u] = EMPTY;
  }
}

// louvainCommunityExistsOmpW (inc/louvain.hxx:668-682): flags only; the
// count comes from the scan total.
__global__ void community_flags_kernel(const uint8_t *ex, size_t n, const uint32_t *vcom, uint32_t *cext) {
  GRID_STRIDE(u, n) {
    if (ex && !ex[u]) continue;
    cext[vcom[u]] = 1;
  }
}

// louvainLookupCommunitiesOmpU (inc/louvain.hxx:839-844).
__global__ void lookup_kernel(uint32_t *a, const uint32_t *map, size_t n) {
  GRID_STRIDE(u, n) a[u] = map[a[u]];
}

// Member counts (louvainCountCommunityVerticesOmpW :752) and total degrees
// (louvainCommunityTotalDegreeOmpW :712), with warp-aggregated atomics.
__global__ void community_sizes_kernel(const uint32_t *deg, const uint8_t *ex, size_t n, const uint32_t *vcom,
                                       uint32_t *csize, unsigned long long *ctdeg) {
  const int lane = threadIdx.x & 31;
  for (size_t base = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32 * 32; base < n;
       base += size_t(gridDim.x) * blockDim.x) {
    const size_t u = base + lane;
    const bool has = u < n && (!ex || ex[u]);
    const uint32_t c = has ? vcom[u] : EMPTY;
    const unsigned long long d = has ? deg[u] : 0;
    const unsigned grp = __match_any_sync(0xffffffffu, c);
    // sum of degrees over the lanes that share this community (full-warp shuffles)
    unsigned long long dsum = 0;
#pragma unroll 8
    for (int l = 0; l < 32; ++l) {
      const uint32_t cl = __shfl_sync(0xffffffffu, c, l);
      const unsigned long long dl = __shfl_sync(0xffffffffu, d, l);
      if (cl == c) dsum += dl;
    }
    if (has && lane == __ffs(grp) - 1) {
      atomicAdd(&csize[c], uint32_t(__popc(grp)));
      atomicAdd(&ctdeg[c], dsum);
    }
  }
}

// Member scatter (louvainCommunityVerticesOmpW :800-812): atomic cursors,
// warp-aggregated; member order within a community is unspecified, as in
// the reference.
__global__ void community_scatter_kernel(const uint8_t *ex, size_t n, const uint32_t *vcom, const uint32_t *coff,
                                         uint32_t *ccur, uint32_t *cmem) {
  const int lane = threadIdx.x & 31;
  for (size_t base = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32 * 32; base < n;
       base += size_t(gridDim.x) * blockDim.x) {
    const size_t u = base + lane;
    const bool has = u < n && (!ex || ex[u]);
    const uint32_t c = has ? vcom[u] : EMPTY;
    const unsigned grp = __match_any_sync(0xffffffffu, c);
    const int leader = __ffs(grp) - 1;
    uint32_t b = 0;
    if (has && lane == leader) b = atomicAdd(&ccur[c], uint32_t(__popc(grp)));
    b = __shfl_sync(0xffffffffu, b, leader);
    if (has) cmem[coff[c] + b + __popc(grp & ((1u << lane) - 1u))] = uint32_t(u);
  }
}

// louvainInitializeOmpW on an aggregated level + the driver's vaff fill
// (inc/louvain.hxx:1207-1210).
// The next level's vertex weights from this level's community totals (see
// launch_next_vertex_weights).
__global__ void next_vertex_weights_kernel(const uint32_t *cext, size_t span, const uint32_t *total,
                                           const tot_t *ctot, tot_t *vnext) {
  GRID_STRIDE(c, span) {
    const uint32_t id = cext[c];
    const uint32_t next = c + 1 < span ? cext[c + 1] : *total;
    if (next > id) vnext[id] = ctot[c];
  }
}

__global__ void level_init_kernel(size_t n, const tot_t *vtot, uint32_t *vcom, tot_t *ctot, uint8_t *vaff) {
  GRID_STRIDE(u, n) {
    vcom[u] = uint32_t(u);
    ctot[u] = vtot[u];
    vaff[u] = 1;
  }
}

// Active vertices of one colour class into per-bin worklists (warp-aggregated
// appends; the order within a worklist is unspecified).
__global__ void compact_active_kernel(const uint32_t *bins, BinBounds bb, const uint8_t *vaff, const uint8_t *fa,
                                      const uint32_t *gid, const uint8_t *gact, uint32_t *wl, uint32_t *wl_count) {
  const uint64_t begin = bb.start[1], end = bb.start[NUM_BINS - 1];
  const int lane = threadIdx.x & 31;
  for (uint64_t base = begin + (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32 * 32; base < end;
       base += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t pos = base + lane;
    int b = -1;
    uint32_t u = 0;
    if (pos < end) {
      u = bins[pos];
      if (vaff[u] && (!fa || fa[u]) && (!gact || gact[gid[u]])) {
        b = 1;
        while (pos >= bb.start[b + 1]) ++b;
      }
    }
    const unsigned grp = __match_any_sync(0xffffffffu, b);
    const int leader = __ffs(grp) - 1;
    uint32_t at = 0;
    if (b >= 0 && lane == leader) at = atomicAdd(&wl_count[b], uint32_t(__popc(grp)));
    at = __shfl_sync(0xffffffffu, at, leader);
    if (b >= 0) wl[bb.start[b] + at + __popc(grp & ((1u << lane) - 1u))] = u;
  }
}

// The same for a level with one colour class (no graph union): a sequential
// pass over the flags (and existence bytes), sixteen per lane and load, in
// place of a gather of every listed vertex's flag; the degree is read only
// for the active vertices, which a warp appends in rounds (one active vertex
// per lane and round, warp-aggregated per bin). The worklists get the same
// vertices: existing ones of bins 1..NUM_BINS-2.
// The bin is recomputed from deg[u], so the append is bounded by the bin's
// slice [bb.start[b], bb.start[b+1]) as well: should deg ever change without
// the bins being recomputed, an append past the slice is dropped and flagged
// (ERR_WORKLIST) instead of writing into the next bin's slice.
__global__ void compact_active_scan_kernel(const uint32_t *deg, const uint8_t *ex, size_t span, BinBounds bb,
                                           BinLimits lim, const uint8_t *vaff, const uint8_t *fa, uint32_t *wl,
                                           uint32_t *wl_count, Counters *ctr) {
  // the first iteration of a dynamic-frontier run: its worklists were filled
  // while the batch was marked (df_start_kernel); take their counts (the
  // flag is cleared after the iteration, in stream order)
  if (ctr->pre_flag) {
    if (blockIdx.x == 0 && threadIdx.x < NUM_BINS) {
      wl_count[threadIdx.x] = ctr->pre_count[threadIdx.x];
      ctr->pre_count[threadIdx.x] = 0;
    }
    return;
  }
  unsigned int *err = &ctr->err;
  const int lane = threadIdx.x & 31;
  const size_t words = (span + 15) / 16;
  // a warp takes WPL * 32 consecutive words, their flag loads issued
  // together; bit 16 k + j of a lane's mask: vertex 16 (wbase + 32 k + lane) + j
  constexpr int WPL = 4;
  for (size_t wbase = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32 * 32 * WPL; wbase < words;
       wbase += size_t(gridDim.x) * blockDim.x * WPL) {
    uint4 pre[WPL];
#pragma unroll
    for (int k = 0; k < WPL; ++k) {
      const size_t w = wbase + size_t(k) * 32 + lane;
      pre[k] = w < words && w * 16 + 16 <= span ? reinterpret_cast<const uint4 *>(vaff)[w] : make_uint4(0, 0, 0, 0);
    }
    unsigned long long act = 0;
#pragma unroll
    for (int k = 0; k < WPL; ++k) {
      const size_t w = wbase + size_t(k) * 32 + lane;
      if (w >= words) continue;
      unsigned a16 = 0;
      const size_t u0 = w * 16;
      if (u0 + 16 <= span) {
        const uint32_t fw[4] = {pre[k].x, pre[k].y, pre[k].z, pre[k].w};
        uint32_t ew[4] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu};
        uint32_t aw[4] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu};
        if ((fw[0] | fw[1] | fw[2] | fw[3]) && ex) {
          const uint4 e = reinterpret_cast<const uint4 *>(ex)[w];
          ew[0] = e.x; ew[1] = e.y; ew[2] = e.z; ew[3] = e.w;
        }
        if ((fw[0] | fw[1] | fw[2] | fw[3]) && fa) {
          const uint4 e = reinterpret_cast<const uint4 *>(fa)[w];
          aw[0] = e.x; aw[1] = e.y; aw[2] = e.z; aw[3] = e.w;
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const uint32_t sh = 8u * (j & 3);
          if (((fw[j >> 2] >> sh) & 0xffu) && ((ew[j >> 2] >> sh) & 0xffu) && ((aw[j >> 2] >> sh) & 0xffu))
            a16 |= 1u << j;
        }
      } else {
        for (size_t u = u0; u < span; ++u)
          if (vaff[u] && (!ex || ex[u]) && (!fa || fa[u])) a16 |= 1u << (u - u0);
      }
      act |= static_cast<unsigned long long>(a16) << (16 * k);
    }
    while (__any_sync(0xffffffffu, act != 0ull)) {
      int b = -1;
      uint32_t u = 0;
      if (act) {
        const int j = __ffsll(static_cast<long long>(act)) - 1;
        act &= act - 1ull;
        u = uint32_t((wbase + size_t(j >> 4) * 32 + lane) * 16 + (j & 15));
        const int x = degree_bin(deg[u], lim);
        if (x >= 1 && x <= NUM_BINS - 2) b = x;
      }
      const unsigned grp = __match_any_sync(0xffffffffu, b);
      const int leader = __ffs(grp) - 1;
      uint32_t at = 0;
      if (b >= 0 && lane == leader) at = atomicAdd(&wl_count[b], uint32_t(__popc(grp)));
      at = __shfl_sync(0xffffffffu, at, leader);
      if (b >= 0) {
        const uint32_t slot = at + __popc(grp & ((1u << lane) - 1u));
        if (slot < bb.start[b + 1] - bb.start[b]) wl[bb.start[b] + slot] = u;
        else atomicOr(err, ERR_WORKLIST);
      }
    }
  }
}

__global__ void gather_u32_kernel(const uint32_t *idx, size_t n, const uint32_t *src, uint32_t *dst) {
  GRID_STRIDE(i, n) dst[i] = src[idx[i]];
}

__global__ void check_ids_kernel(const uint32_t *a, size_t n, uint32_t limit, unsigned int *err) {
  bool bad = false;
  GRID_STRIDE(i, n) bad |= a[i] >= limit;
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(err, ERR_BAD_ID);
}

// check_ids_kernel, and whether q equals the cached memberships c0 / c1
// (nullptr: not compared): diff[k] is set if any entry differs.
__global__ void check_prior_kernel(const uint32_t *q, size_t n, uint32_t limit, const uint32_t *c0,
                                   const uint32_t *c1, unsigned int *err, unsigned int *diff) {
  bool bad = false, d0 = false, d1 = false;
  GRID_STRIDE(i, n) {
    const uint32_t x = q[i];
    bad |= x >= limit;
    if (c0) d0 |= __ldcs(c0 + i) != x;
    if (c1) d1 |= __ldcs(c1 + i) != x;
  }
  const bool lead = (threadIdx.x & 31) == 0;
  if (__any_sync(0xffffffffu, bad) && lead) atomicOr(err, ERR_BAD_ID);
  if (__any_sync(0xffffffffu, d0) && lead) atomicOr(&diff[0], 1u);
  if (__any_sync(0xffffffffu, d1) && lead) atomicOr(&diff[1], 1u);
}

// Flags equal to 1, sixteen bytes per load (bytewise compares); the tail
// past the last whole 16-byte word bytewise.
__global__ void count_flags_kernel(const uint8_t *f, size_t n, unsigned long long *dst) {
  unsigned long long c = 0;
  const size_t n16 = n / 16;
  const uint4 *f16 = reinterpret_cast<const uint4 *>(f);
  auto ones = [](const uint4 &v) {
    return __popc(__vcmpeq4(v.x, 0x01010101u)) / 8 + __popc(__vcmpeq4(v.y, 0x01010101u)) / 8 +
           __popc(__vcmpeq4(v.z, 0x01010101u)) / 8 + __popc(__vcmpeq4(v.w, 0x01010101u)) / 8;
  };
  // four loads in flight per thread
  const size_t stride = size_t(gridDim.x) * blockDim.x;
  size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n16; i += 4 * stride) {
    const uint4 v0 = f16[i], v1 = f16[i + stride], v2 = f16[i + 2 * stride], v3 = f16[i + 3 * stride];
    c += ones(v0) + ones(v1) + ones(v2) + ones(v3);
  }
  for (; i < n16; i += stride) c += ones(f16[i]);
  GRID_STRIDE(i, n - n16 * 16) c += f[n16 * 16 + i] == 1;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(dst, c);
}

// modularityBy (inc/properties.hxx:178-191) in FP64: intra-community weight
// and per-community totals. One warp per vertex.
__global__ void modularity_kernel(const uint64_t *off, const uint32_t *deg, const uint32_t *key, const float *w,
                                  const uint8_t *ex, size_t n, const uint32_t *memb, double *ctot64,
                                  double *intra) {
  const size_t warps = size_t(gridDim.x) * blockDim.x / 32;
  const int lane = threadIdx.x & 31;
  double in = 0;
  for (size_t u = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; u < n; u += warps) {
    if (ex && !ex[u]) continue;
    const uint32_t c = memb[u];
    const uint64_t o = off[u];
    const uint32_t d = deg[u];
    double tot = 0;
    for (uint32_t j = lane; j < d; j += 32) {
      const double x = w[o + j];
      tot += x;
      if (memb[key[o + j]] == c) in += x;
    }
    tot = warp_sum_d(tot);
    if (lane == 0 && tot != 0.0) atomicAdd(&ctot64[c], tot);
  }
  block_add_double(in, intra);
}

__global__ void sq_sum_kernel(const double *x, size_t n, double *dst) {
  double s = 0;
  GRID_STRIDE(i, n) s += x[i] * x[i];
  block_add_double(s, dst);
}

}  // namespace

int grid_for(size_t n, int block, int max_blocks_per_sm) {
  size_t want = (n + block - 1) / block;
  size_t cap = size_t(sms()) * max_blocks_per_sm;
  size_t g = want < cap ? want : cap;
  return int(g ? g : 1);
}

void launch_degrees(const uint64_t *off, uint32_t *deg, size_t span, cudaStream_t s) {
  if (!span) return;
  degrees_kernel<<<grid_for(span, 256), 256, 0, s>>>(off, deg, span);
  LVG_CHECK_LAUNCH();
}

void launch_fill_u8(uint8_t *p, uint8_t v, size_t n, cudaStream_t s) {
  if (n) LVG_CUDA(cudaMemsetAsync(p, v, n, s));
}

// Byte fill by the SMs: 16-byte stores over the aligned middle, bytes at
// the ends; stream-ordered stores that do not depend on the copy engines,
// which carry the host transfers of the drop-in calls.
__global__ void fill_bytes_kernel(uint8_t *p, size_t n, uint8_t v) {
  const size_t head = (16 - (reinterpret_cast<uintptr_t>(p) & 15)) & 15;
  const size_t h = head < n ? head : n;
  const size_t words = (n - h) / 16;
  const size_t tail = h + words * 16;
  const uint32_t b4 = 0x01010101u * v;
  const uint4 w = make_uint4(b4, b4, b4, b4);
  uint4 *q = reinterpret_cast<uint4 *>(p + h);
  const size_t t0 = size_t(blockIdx.x) * blockDim.x + threadIdx.x, st = size_t(gridDim.x) * blockDim.x;
  for (size_t i = t0; i < words; i += st) q[i] = w;
  for (size_t i = t0; i < h; i += st) p[i] = v;
  for (size_t i = tail + t0; i < n; i += st) p[i] = v;
}

// The start of a local-moving iteration: the gain sum and the classes'
// worklist counts to zero (one launch for both).
__global__ void iter_begin_kernel(unsigned long long *el_fix, uint32_t *wl_count, int n) {
  if (threadIdx.x == 0) *el_fix = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) wl_count[i] = 0;
}

void launch_iter_begin(unsigned long long *el_fix, uint32_t *wl_count, int n, cudaStream_t s) {
  iter_begin_kernel<<<1, 256, 0, s>>>(el_fix, wl_count, n);
  LVG_CHECK_LAUNCH();
}

void launch_fill_bytes(void *p, uint8_t v, size_t n, cudaStream_t s) {
  if (!n) return;
  fill_bytes_kernel<<<grid_for((n + 15) / 16, 256), 256, 0, s>>>(static_cast<uint8_t *>(p), n, v);
  LVG_CHECK_LAUNCH();
}

void launch_fill_f32(float *p, size_t n, float v, cudaStream_t s) {
  if (!n) return;
  fill_f32_kernel<<<grid_for(n, 256), 256, 0, s>>>(p, n, v);
  LVG_CHECK_LAUNCH();
}

void launch_init_static(const Level &g, uint32_t *ucom, tot_t *utot, tot_t *ctot, cudaStream_t s) {
  if (!g.span) return;
  init_static_kernel<<<grid_for(g.span * 32, 256), 256, 0, s>>>(g.off, g.deg, g.w, g.ex, g.span, g.gid, g.gbase,
                                                                 ucom, utot, ctot);
  LVG_CHECK_LAUNCH();
}

void launch_vertex_weights_f64(const Level &g, double *vtot, cudaStream_t s) {
  if (!g.span) return;
  vertex_weights_f64_kernel<<<grid_for(g.span * 32, 256), 256, 0, s>>>(g.off, g.deg, g.w, g.ex, g.span, vtot);
  LVG_CHECK_LAUNCH();
}

void launch_community_weights_f64(const uint32_t *q, const double *vtot, size_t n, double *ctot, cudaStream_t s) {
  LVG_CUDA(cudaMemsetAsync(ctot, 0, n * sizeof(double), s));
  if (!n) return;
  community_weights_f64_kernel<<<grid_for(n, 256), 256, 0, s>>>(q, vtot, n, ctot);
  LVG_CHECK_LAUNCH();
}

void launch_count_nonunit(const float *w, size_t n, Counters *ctr, cudaStream_t s) {
  if (!n) return;
  count_nonunit_kernel<<<grid_for(n, 256), 256, 0, s>>>(w, n, &ctr->nonunit);
  LVG_CHECK_LAUNCH();
}

void launch_total_weight(const float *w, size_t n, Counters *ctr, cudaStream_t s) {
  LVG_CUDA(cudaMemsetAsync(&ctr->fp64[0], 0, sizeof(double), s));
  if (!n) return;
  total_weight_kernel<<<grid_for(n, 256), 256, 0, s>>>(w, n, &ctr->fp64[0]);
  LVG_CHECK_LAUNCH();
}

void launch_batch_weights(const uint32_t *src, const float *w, size_t n, float sign, const uint32_t *vcom,
                          tot_t *vtot, tot_t *ctot, cudaStream_t s) {
  if (!n) return;
  batch_weights_kernel<<<grid_for(n, 256), 256, 0, s>>>(src, w, n, sign, vcom, vtot, ctot);
  LVG_CHECK_LAUNCH();
}

void launch_df_start(const uint32_t *ds, const uint32_t *dd, const float *dw, size_t nd, const uint32_t *is,
                     const uint32_t *id, const float *iw, size_t ni, const uint32_t *vcom, tot_t *vtot, tot_t *ctot,
                     const Level &g, uint8_t *vaff, const BinBounds *bb, uint32_t *wl, Counters *ctr,
                     cudaStream_t s) {
  // with lists, the first compaction takes them even for an empty batch
  const size_t n = nd + ni;
  if (!n && !bb) return;
  df_start_kernel<<<n ? grid_for(n, 256) : 1, 256, 0, s>>>(ds, dd, dw, nd, is, id, iw, ni, vcom, vtot, ctot, g.deg,
                                                          g.ex, g.lim, vaff, bb ? *bb : BinBounds{},
                                                          bb ? wl : nullptr, ctr);
  LVG_CHECK_LAUNCH();
}

void launch_df_mark(const uint32_t *ds, const uint32_t *dd, size_t nd, const uint32_t *is, const uint32_t *id,
                    size_t ni, const uint32_t *vcom, uint8_t *vaff, cudaStream_t s) {
  if (!(nd + ni)) return;
  df_mark_kernel<<<grid_for(nd + ni, 256), 256, 0, s>>>(ds, dd, nd, is, id, ni, vcom, vaff);
  LVG_CHECK_LAUNCH();
}

void launch_ds_mark(const Level &g, const uint32_t *ds, const uint32_t *dd, size_t nd, const uint32_t *is,
                    const uint32_t *id, const float *iw, size_t ni, const uint32_t *seg, size_t nseg_cap,
                    const uint32_t *vcom, const tot_t *vtot, const tot_t *ctot, double M, double R,
                    uint8_t *vertices, uint8_t *neighbors, uint8_t *communities, uint32_t *gkeys, float *gvals,
                    uint32_t *gfirst, int glog2, Counters *ctr, uint32_t *list, uint32_t *count, uint32_t *chunks,
                    uint32_t *scan_scratch, cudaStream_t s) {
  (void)nseg_cap;
  if (nd) {
    ds_del_kernel<<<grid_for(nd, 256), 256, 0, s>>>(ds, dd, nd, vcom, vertices, neighbors, communities);
    LVG_CHECK_LAUNCH();
  }
  if (ni) {
    DsScreen sc;
    sc.ok = M >= 1e-15 && M <= 1e15 && R > 0 && R <= 1e6;
    sc.invM = sc.ok ? float(1.0 / M) : 0.f;
    sc.inv2MM = sc.ok ? float(1.0 / (2 * M * M)) : 0.f;
    sc.R = float(R);
    unsigned int *nseg = &ctr->cn, *nlong = &ctr->ds_long;  // scratch counters
    LVG_CUDA(cudaMemsetAsync(nseg, 0, sizeof(unsigned int), s));
    LVG_CUDA(cudaMemsetAsync(nlong, 0, sizeof(unsigned int), s));
    ds_ins_lane_kernel<<<grid_for(ni, 256), 256, 0, s>>>(is, id, iw, ni, const_cast<uint32_t *>(seg), nseg, vcom,
                                                          vtot, ctot, sc, vertices, neighbors, communities);
    LVG_CHECK_LAUNCH();
    ds_ins_warp_kernel<<<grid_for(ni * 32, 256), 256, 0, s>>>(is, id, iw, ni, const_cast<uint32_t *>(seg), nseg,
                                                                nlong, vcom, vtot, ctot, M, R, sc, vertices,
                                                                neighbors, communities);
    LVG_CHECK_LAUNCH();
    ds_ins_kernel<<<global_table_blocks(ni / 33 + 1), DS_BLOCK, 0, s>>>(is, id, iw, ni, seg, nseg, nlong, vcom,
                                                                       vtot, ctot, M, R, vertices, neighbors,
                                                                       communities, gkeys, gvals, gfirst, glog2,
                                                                       ctr);
    LVG_CHECK_LAUNCH();
  }
  if (g.span) {
    LVG_CUDA(cudaMemsetAsync(count, 0, 2 * sizeof(uint32_t), s));
    ds_expand_kernel<<<grid_for(g.span, 256), 256, 0, s>>>(g.ex, g.span, vcom, g.deg, neighbors, communities,
                                                            vertices, list, count);
    LVG_CHECK_LAUNCH();
    ds_neighbors_kernel<<<unsigned(sms()) * 8, 256, 0, s>>>(g.off, g.deg, g.key, list, count, vertices);
    LVG_CHECK_LAUNCH();
    ds_big_chunks_kernel<<<grid_for(g.span, 256), 256, 0, s>>>(g.deg, list, count, g.span, chunks);
    LVG_CHECK_LAUNCH();
    exclusive_scan_u32(chunks, chunks, g.span, &ctr->ds_chunks, scan_scratch, s);
    ds_neighbors_big_kernel<<<unsigned(sms()) * 8, 256, 0, s>>>(g.off, g.deg, g.key, list, count, g.span, chunks,
                                                               &ctr->ds_chunks, vertices);
    LVG_CHECK_LAUNCH();
  }
}

void launch_clear_isolated(const uint32_t *list, size_t n, uint8_t *vaff, const uint8_t *fa, cudaStream_t s) {
  if (!n) return;
  clear_isolated_kernel<<<grid_for(n, 256), 256, 0, s>>>(list, n, vaff, fa);
  LVG_CHECK_LAUNCH();
}

void launch_clear_isolated_multi(const IsolatedLists &L, uint8_t *vaff, const uint8_t *fa, cudaStream_t s) {
  size_t most = 0, total = 0;
  for (int j = 0; j < L.k; ++j) { most = std::max(most, L.n[j]); total += L.n[j]; }
  if (!total) return;
  const unsigned grid = unsigned(std::min<size_t>(size_t(L.k) * ((most + 255) / 256), size_t(sms()) * 8 * L.k));
  clear_isolated_multi_kernel<<<grid, 256, 0, s>>>(L, vaff, fa);
  LVG_CHECK_LAUNCH();
}

void launch_merge_marks(uint8_t *vaff, uint8_t *mark, size_t n, cudaStream_t s) {
  if (!n) return;
  merge_marks_kernel<<<grid_for(n, 256), 256, 0, s>>>(vaff, mark, n);
  LVG_CHECK_LAUNCH();
}

void launch_apply_moves(const uint32_t *list, size_t n, uint32_t *dec, uint32_t *vcom, tot_t *ctot,
                        const tot_t *vtot, cudaStream_t s) {
  if (!n) return;
  apply_moves_kernel<<<grid_for(n, 256), 256, 0, s>>>(list, n, dec, vcom, ctot, vtot);
  LVG_CHECK_LAUNCH();
}

void launch_community_flags(const Level &g, const uint32_t *vcom, uint32_t *cext, cudaStream_t s) {
  if (!g.span) return;
  community_flags_kernel<<<grid_for(g.span, 256), 256, 0, s>>>(g.ex, g.span, vcom, cext);
  LVG_CHECK_LAUNCH();
}

void launch_lookup(uint32_t *a, const uint32_t *map, size_t n, cudaStream_t s) {
  if (!n) return;
  lookup_kernel<<<grid_for(n, 256), 256, 0, s>>>(a, map, n);
  LVG_CHECK_LAUNCH();
}

void launch_community_sizes(const Level &g, const uint32_t *vcom, uint32_t *csize, uint64_t *ctdeg,
                            cudaStream_t s) {
  if (!g.span) return;
  community_sizes_kernel<<<grid_for(g.span, 256), 256, 0, s>>>(g.deg, g.ex, g.span, vcom, csize,
                                                                reinterpret_cast<unsigned long long *>(ctdeg));
  LVG_CHECK_LAUNCH();
}

void launch_community_scatter(const Level &g, const uint32_t *vcom, const uint32_t *coff, uint32_t *ccur,
                              uint32_t *cmem, cudaStream_t s) {
  if (!g.span) return;
  community_scatter_kernel<<<grid_for(g.span, 256), 256, 0, s>>>(g.ex, g.span, vcom, coff, ccur, cmem);
  LVG_CHECK_LAUNCH();
}

void launch_next_vertex_weights(const uint32_t *cext, size_t span, const uint32_t *total, const tot_t *ctot,
                                tot_t *vtot_next, cudaStream_t s) {
  if (!span) return;
  next_vertex_weights_kernel<<<grid_for(span, 256), 256, 0, s>>>(cext, span, total, ctot, vtot_next);
  LVG_CHECK_LAUNCH();
}

void launch_level_init(size_t n, const tot_t *vtot, uint32_t *vcom, tot_t *ctot, uint8_t *vaff, cudaStream_t s) {
  if (!n) return;
  level_init_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, vtot, vcom, ctot, vaff);
  LVG_CHECK_LAUNCH();
}

void launch_compact_active(const uint32_t *bins, const BinBounds &bb, const uint8_t *vaff, const uint8_t *fa,
                           uint32_t *wl, uint32_t *wl_count, cudaStream_t s, const uint32_t *gid,
                           const uint8_t *gact) {
  const uint64_t n = bb.start[NUM_BINS - 1] - bb.start[1];
  if (!n) return;
  compact_active_kernel<<<grid_for(n, 256), 256, 0, s>>>(bins, bb, vaff, fa, gid, gact, wl, wl_count);
  LVG_CHECK_LAUNCH();
}

void launch_compact_active_scan(const Level &g, const BinBounds &bb, const uint8_t *vaff, const uint8_t *fa,
                                uint32_t *wl, uint32_t *wl_count, Counters *ctr, cudaStream_t s) {
  if (!g.span) return;
  compact_active_scan_kernel<<<grid_for((g.span + 15) / 16, 256, 4), 256, 0, s>>>(g.deg, g.ex, g.span, bb, g.lim, vaff,
                                                                                  fa, wl, wl_count, ctr);
  LVG_CHECK_LAUNCH();
}

void launch_gather_u32(const uint32_t *idx, size_t n, const uint32_t *src, uint32_t *dst, cudaStream_t s) {
  if (!n) return;
  gather_u32_kernel<<<grid_for(n, 256), 256, 0, s>>>(idx, n, src, dst);
  LVG_CHECK_LAUNCH();
}

void launch_check_ids(const uint32_t *a, size_t n, uint32_t limit, Counters *ctr, cudaStream_t s) {
  if (!n) return;
  check_ids_kernel<<<grid_for(n, 256), 256, 0, s>>>(a, n, limit, &ctr->err);
  LVG_CHECK_LAUNCH();
}

void launch_check_prior(const uint32_t *q, size_t n, uint32_t limit, const uint32_t *c0, const uint32_t *c1,
                        Counters *ctr, cudaStream_t s) {
  LVG_CUDA(cudaMemsetAsync(ctr->qdiff, 0, sizeof(ctr->qdiff), s));
  if (!n) return;
  check_prior_kernel<<<grid_for(n, 256), 256, 0, s>>>(q, n, limit, c0, c1, &ctr->err, ctr->qdiff);
  LVG_CHECK_LAUNCH();
}

void launch_clear_isolated_endpoints(const uint32_t *a, size_t na, const uint32_t *b, size_t nb,
                                     const uint32_t *deg, const uint8_t *ex, uint8_t *vaff, cudaStream_t s) {
  if (!na && !nb) return;
  clear_isolated_endpoints_kernel<<<grid_for(na + nb, 256), 256, 0, s>>>(a, na, b, nb, deg, ex, vaff);
  LVG_CHECK_LAUNCH();
}

__global__ void iter_end_kernel(Counters *ctr, double M, double E, int L, bool by_graph,
                                cudaGraphConditionalHandle h) {
  const unsigned l = ++ctr->dev_iters;
  bool more;
  if (by_graph) {  // graph unions: iter_control_kernel ran each graph's test
    ctr->dev_el = 0;
    more = ctr->gactive != 0;
  } else {
    const double el = double(ctr->el_fix) / GAIN_FIX / M;
    ctr->dev_el = el;
    more = el > E;
  }
  ctr->pre_flag = 0;  // the first iteration's listed worklists are used up
  cudaGraphSetConditional(h, (more && l < unsigned(L) && !ctr->err) ? 1u : 0u);
}

void launch_iter_end(Counters *ctr, double M, double E, int L, bool by_graph, cudaGraphConditionalHandle h,
                     cudaStream_t s) {
  iter_end_kernel<<<1, 1, 0, s>>>(ctr, M, E, L, by_graph, h);
  LVG_CHECK_LAUNCH();
}

void launch_count_flags(const uint8_t *f, size_t n, Counters *ctr, cudaStream_t s) {
  launch_fill_bytes(&ctr->affected, 0, sizeof(unsigned long long), s);
  if (!n) return;
  count_flags_kernel<<<grid_for(n, 256), 256, 0, s>>>(f, n, &ctr->affected);
  LVG_CHECK_LAUNCH();
}

void launch_modularity(const Level &g, const uint32_t *memb, double *ctot64, Counters *ctr, cudaStream_t s) {
  LVG_CUDA(cudaMemsetAsync(&ctr->fp64[1], 0, sizeof(double), s));
  LVG_CUDA(cudaMemsetAsync(ctot64, 0, g.span * sizeof(double), s));
  if (!g.span) return;
  modularity_kernel<<<grid_for(g.span * 32, 256), 256, 0, s>>>(g.off, g.deg, g.key, g.w, g.ex, g.span, memb, ctot64,
                                                               &ctr->fp64[1]);
  LVG_CHECK_LAUNCH();
}

void launch_sq_sum(const double *x, size_t n, Counters *ctr, cudaStream_t s) {
  LVG_CUDA(cudaMemsetAsync(&ctr->fp64[2], 0, sizeof(double), s));
  if (!n) return;
  sq_sum_kernel<<<grid_for(n, 256), 256, 0, s>>>(x, n, &ctr->fp64[2]);
  LVG_CHECK_LAUNCH();
}

}  // namespace lvg
