// lvg_update.cu — applying a batch update to a graph resident in HBM.
//
// The reference prepares each batch on the host, outside its timed section:
// tidyBatchUpdateU (inc/batch.hxx:202-209) keeps the deletions whose edge is
// present and the insertions whose edge is absent, sorted by (source,
// target) without duplicates; applyBatchUpdateOmpU (inc/batch.hxx:241-248)
// then removes and adds them on LazyBitset rows that stay sorted
// (inc/_bitset.hxx:227-261), and an added edge makes both endpoints present
// (DiGraph::addEdge, inc/Graph.hxx:318-334). main.cxx:108-109 runs the two
// back to back, and hands the tidied batch to the dynamic methods.
//
// Here the uploaded graph is a gapped CSR: row u holds deg[u] sorted entries
// at off[u] with room for cap[u]; gaps and unused pool entries hold (0, 0.0).
// Only the rows the batch touches are rewritten, one warp per row:
//   merge:  the warp tests every deletion and insertion of its row against
//           the row (the tidy filter), keeping running counts of the kept
//           ones; every surviving entry and every kept insertion then finds
//           its output position with binary searches, so the row is
//           rewritten into scratch without a sequential merge;
//   commit: the row is copied back in place when it fits its capacity, or to
//           a fresh stretch of the overflow pool (bump allocation) when it
//           outgrows it; what the row no longer uses is zeroed.
// The host hands the batch over sorted by (source, target) with duplicates
// removed, and one UpdRow per touched source vertex. The kept flags are left
// in keep[] (deletions, then insertions) for the tidied batch.
#include "lvg_internal.cuh"

namespace lvg {
namespace {

// Number of entries of sorted a[0..n) that are < x.
__device__ __forceinline__ uint32_t count_less(const uint32_t *a, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ double warp_sum_f64(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Step 1, one warp per touched row: the tidy filter and the row's plan.
//   ikeep/dkeep: the insertion is absent / the deletion is present in the row;
//   ipre[j] / dpre[j]: kept insertions / deletions before j in the row;
//   P.n1: new degree; P.f0: first old index whose position changes (0 when
//   the row moves to the pool); P.len: entries to rewrite (n1 - f0);
//   P.src: source items (old entries from f0, then every insertion);
//   P.grow: pool entries the row takes (0 unless it outgrows its capacity).
// Also the change of the edge count and of the total weight (FP64), and the
// endpoints of kept insertions marked present in ex (when given).
__global__ void row_plan_kernel(const uint64_t *off, const uint32_t *deg, const uint32_t *cap, const uint32_t *key,
                                const float *w, const UpdRow *rows, size_t nrows, const uint32_t *dd,
                                const uint32_t *id, const float *iw, size_t nd_all, uint32_t *pre, uint32_t *keep,
                                RowPlan *plan, uint64_t *len, uint64_t *src, uint64_t *grow, uint8_t *ex,
                                unsigned long long *upd, double *wdelta) {
  const size_t warps = size_t(gridDim.x) * blockDim.x / 32;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1;
  long long edges = 0;
  double dw = 0;
  for (size_t r = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; r < nrows; r += warps) {
    const UpdRow R = rows[r];
    const uint64_t o = off[R.u];
    const uint32_t n = deg[R.u];
    const uint32_t *row = key + o;
    const uint32_t *dl = dd + R.d0, nd = R.d1 - R.d0;
    const uint32_t *il = id + R.i0, ni = R.i1 - R.i0;
    uint32_t *dpre = pre + R.d0, *ipre = pre + nd_all + R.i0;
    uint32_t *dkeep = keep + R.d0, *ikeep = keep + nd_all + R.i0;
    uint32_t icarry = 0, dcarry = 0, first = n;
    for (uint32_t b = 0; b < ni; b += 32) {  // warp-uniform bound
      const uint32_t j = b + lane;
      bool k = false;
      if (j < ni) {
        const uint32_t p = count_less(row, n, il[j]);
        k = !(p < n && row[p] == il[j]);
        if (k) {
          first = min(first, p);
          dw += double(iw[R.i0 + j]);
          if (ex) ex[il[j]] = 1;
        }
      }
      const uint32_t m = __ballot_sync(0xffffffffu, k);
      if (j < ni) {
        ipre[j] = icarry + __popc(m & lt);
        ikeep[j] = k;
      }
      icarry += __popc(m);
    }
    for (uint32_t b = 0; b < nd; b += 32) {
      const uint32_t j = b + lane;
      bool k = false;
      if (j < nd) {
        const uint32_t p = count_less(row, n, dl[j]);
        k = p < n && row[p] == dl[j];
        if (k) {
          first = min(first, p);
          dw -= double(w[o + p]);
        }
      }
      const uint32_t m = __ballot_sync(0xffffffffu, k);
      if (j < nd) {
        dpre[j] = dcarry + __popc(m & lt);
        dkeep[j] = k;
      }
      dcarry += __popc(m);
    }
    first = __reduce_min_sync(0xffffffffu, first);
    if (lane == 0) {
      const uint32_t n1 = n - dcarry + icarry;
      const bool moved = n1 > cap[R.u];
      const uint32_t f0 = moved ? 0 : first;
      RowPlan P;
      P.n1 = n1;
      P.f0 = f0;
      P.dcarry = dcarry;
      P.icarry = icarry;
      plan[r] = P;
      len[r] = n1 - f0;
      src[r] = uint64_t(n - f0) + ni;
      grow[r] = moved ? row_capacity(n1) : 0;
      edges += (long long)n1 - (long long)n;
      if (icarry && ex) ex[R.u] = 1;
    }
  }
  dw = warp_sum_f64(dw);
  if (lane == 0) {
    if (edges) atomicAdd(&upd[UPD_EDGES], (unsigned long long)edges);
    if (dw != 0.0) atomicAdd(wdelta, dw);
  }
}

// The row an item of a flat range belongs to: the last r with start[r] <= x.
__device__ __forceinline__ uint32_t row_of(const uint64_t *start, uint32_t nrows, uint64_t x) {
  uint32_t lo = 0, hi = nrows;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (start[mid] <= x) lo = mid; else hi = mid;
  }
  return lo;
}

// Step 2, one thread per source item (old entries from f0, then insertions)
// of all touched rows: the item's place in the rewritten row, into scratch.
// An old entry at i goes to i - (kept deletions before it) + (kept
// insertions before it); a kept insertion j to j's kept rank + (old entries
// before it) - (kept deletions before it).
__global__ void merge_items_kernel(const uint64_t *off, const uint32_t *deg, const uint32_t *key, const float *w,
                                   const UpdRow *rows, uint32_t nrows, const uint32_t *dd, const uint32_t *id,
                                   const float *iw, size_t nd_all, const uint32_t *pre, const uint32_t *keep,
                                   const RowPlan *plan, const uint64_t *src, uint64_t total, const uint64_t *spos,
                                   uint32_t *skey, float *sw) {
  for (uint64_t x = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; x < total;
       x += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t r = row_of(src, nrows, x);
    const UpdRow R = rows[r];
    const RowPlan P = plan[r];
    const uint64_t o = off[R.u];
    const uint32_t n = deg[R.u];
    const uint32_t *row = key + o;
    const uint32_t *dl = dd + R.d0, nd = R.d1 - R.d0;
    const uint32_t *il = id + R.i0, ni = R.i1 - R.i0;
    const uint32_t *dpre = pre + R.d0, *ipre = pre + nd_all + R.i0;
    const uint32_t j = uint32_t(x - src[r]);
    const uint64_t base = spos[r];
    if (j < n - P.f0) {
      const uint32_t i = P.f0 + j;
      const uint32_t k = row[i];
      const uint32_t a = count_less(dl, nd, k);
      if (a < nd && dl[a] == k) continue;  // deleted (present, so kept)
      const uint32_t b = count_less(il, ni, k);
      const uint32_t at = i - (a < nd ? dpre[a] : P.dcarry) + (b < ni ? ipre[b] : P.icarry) - P.f0;
      skey[base + at] = k;
      sw[base + at] = w[o + i];
    } else {
      const uint32_t jj = j - (n - P.f0);
      if (!keep[nd_all + R.i0 + jj]) continue;  // already present: tidied away
      const uint32_t k = il[jj];
      const uint32_t a = count_less(dl, nd, k);
      const uint32_t at = ipre[jj] + count_less(row, n, k) - (a < nd ? dpre[a] : P.dcarry) - P.f0;
      skey[base + at] = k;
      sw[base + at] = iw[R.i0 + jj];
    }
  }
}

// Step 3, one thread per rewritten entry: scratch -> the row's place (in
// place from f0, or the row's new stretch in the pool at pool + gpos[r]).
__global__ void copy_items_kernel(const uint64_t *off, const UpdRow *rows, uint32_t nrows, const RowPlan *plan,
                                  const uint64_t *spos, uint64_t total, const uint64_t *grow, const uint64_t *gpos,
                                  uint64_t pool, const uint32_t *skey, const float *sw, uint32_t *key, float *w) {
  for (uint64_t x = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; x < total;
       x += uint64_t(gridDim.x) * blockDim.x) {
    const uint32_t r = row_of(spos, nrows, x);
    const uint64_t dst = (grow[r] ? pool + gpos[r] : off[rows[r].u]) + plan[r].f0 + (x - spos[r]);
    key[dst] = skey[x];
    w[dst] = sw[x];
  }
}

// Step 4, one warp per touched row: zero what the row no longer uses (the
// tail in place; the old stretch and the new stretch's slack when it moved)
// and set its offset, capacity and degree.
__global__ void finish_rows_kernel(uint64_t *off, uint32_t *deg, uint32_t *cap, uint32_t *key, float *w,
                                   const UpdRow *rows, size_t nrows, const RowPlan *plan, const uint64_t *grow,
                                   const uint64_t *gpos, uint64_t pool) {
  const size_t warps = size_t(gridDim.x) * blockDim.x / 32;
  const uint32_t lane = threadIdx.x & 31;
  for (size_t r = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; r < nrows; r += warps) {
    const uint32_t u = rows[r].u;
    const uint32_t n0 = deg[u], n1 = plan[r].n1;
    const uint64_t o = off[u];
    if (grow[r]) {
      const uint64_t no = pool + gpos[r];
      const uint32_t nc = uint32_t(grow[r]);
      for (uint32_t i = lane; i < n0; i += 32) { key[o + i] = 0; w[o + i] = 0.f; }
      for (uint32_t i = n1 + lane; i < nc; i += 32) { key[no + i] = 0; w[no + i] = 0.f; }
      __syncwarp();  // every lane has read the row's old extent
      if (lane == 0) { off[u] = no; cap[u] = nc; deg[u] = n1; }
    } else {
      for (uint32_t i = n1 + lane; i < n0; i += 32) { key[o + i] = 0; w[o + i] = 0.f; }
      __syncwarp();
      if (lane == 0) deg[u] = n1;
    }
  }
}

// Present vertices, counted into *dst.
__global__ void count_present_kernel(const uint8_t *ex, size_t n, unsigned long long *dst) {
  unsigned long long c = 0;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    c += ex[i] != 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(dst, c);
}

// Spread a compact CSR into the gapped layout (one warp per row; gaps zero).
__global__ void spread_rows_kernel(const uint64_t *coff, const uint32_t *ckey, const float *cw, size_t n,
                                   const uint64_t *off, const uint32_t *cap, uint32_t *key, float *w) {
  const size_t warps = size_t(gridDim.x) * blockDim.x / 32;
  const uint32_t lane = threadIdx.x & 31;
  for (size_t u = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; u < n; u += warps) {
    const uint64_t s = coff[u], d = coff[u + 1] - coff[u], o = off[u];
    for (uint32_t i = lane; i < cap[u]; i += 32) {
      key[o + i] = i < d ? ckey[s + i] : 0;
      w[o + i] = i < d ? cw[s + i] : 0.f;
    }
  }
}

// Degrees and capacities of a compact CSR.
__global__ void row_caps_kernel(const uint64_t *coff, size_t n, uint32_t *deg, uint32_t *cap, uint64_t *cap64) {
  for (size_t u = size_t(blockIdx.x) * blockDim.x + threadIdx.x; u < n; u += size_t(gridDim.x) * blockDim.x) {
    const uint32_t d = uint32_t(coff[u + 1] - coff[u]);
    const uint32_t c = row_capacity(d);
    deg[u] = d;
    cap[u] = c;
    cap64[u] = c;
  }
}

// Fresh capacities from the current degrees.
__global__ void fresh_caps_kernel(const uint32_t *deg, size_t n, uint32_t *cap, uint64_t *cap64) {
  for (size_t u = size_t(blockIdx.x) * blockDim.x + threadIdx.x; u < n; u += size_t(gridDim.x) * blockDim.x) {
    const uint32_t c = row_capacity(deg[u]);
    cap[u] = c;
    cap64[u] = c;
  }
}

// ---------------------------------------------------------------- plan

// Batch entry i as a packed (src << b | dst) key, with its index.
__global__ void pack_keys_kernel(const uint32_t *src, const uint32_t *dst, size_t n, int b, uint64_t *key,
                                 uint32_t *val) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    key[i] = uint64_t(src[i]) << b | dst[i];
    val[i] = uint32_t(i);
  }
}

// First of each run of equal keys; the sort is stable, so that is the first
// occurrence in batch order.
__global__ void first_flags_kernel(const uint64_t *key, size_t n, uint32_t *flag) {
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    flag[i] = i == 0 || key[i] != key[i - 1];
}

__global__ void unpack_keys_kernel(const uint64_t *key, const uint32_t *val, const uint32_t *flag,
                                   const uint32_t *pos, size_t n, int b, const float *w, uint32_t *os, uint32_t *od,
                                   float *ow) {
  const uint64_t mask = (uint64_t(1) << b) - 1;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    if (!flag[i]) continue;
    const uint32_t o = pos[i];
    os[o] = uint32_t(key[i] >> b);
    od[o] = uint32_t(key[i] & mask);
    ow[o] = w[val[i]];
  }
}

// touched[u] = 1 for every source of the (deduplicated) lists; their lengths
// are read from the device (*nd, *ni).
__global__ void touch_kernel(const uint32_t *ds, const uint32_t *nd, const uint32_t *is, const uint32_t *ni,
                             size_t cap, uint32_t *touched) {
  const uint32_t a = *nd, c = *ni;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < cap; i += size_t(gridDim.x) * blockDim.x) {
    if (i < a) touched[ds[i]] = 1;
    if (i < c) touched[is[i]] = 1;
  }
}

__device__ __forceinline__ uint32_t lower_bound_u32(const uint32_t *a, uint32_t n, uint32_t x) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// One UpdRow per touched vertex, in id order; the longest insertion run into
// upd[UPD_MAXG].
__global__ void plan_rows_kernel(const uint32_t *touched, const uint32_t *tpos, size_t span, const uint32_t *ds,
                                 const uint32_t *nd, const uint32_t *is, const uint32_t *ni, UpdRow *rows,
                                 unsigned long long *upd) {
  const uint32_t a = *nd, c = *ni;
  for (size_t u = size_t(blockIdx.x) * blockDim.x + threadIdx.x; u < span; u += size_t(gridDim.x) * blockDim.x) {
    if (!touched[u]) continue;
    UpdRow R;
    R.u = uint32_t(u);
    R.d0 = lower_bound_u32(ds, a, R.u);
    R.d1 = lower_bound_u32(ds, a, R.u + 1);
    R.i0 = lower_bound_u32(is, c, R.u);
    R.i1 = lower_bound_u32(is, c, R.u + 1);
    rows[tpos[u]] = R;
    if (R.i1 > R.i0) atomicMax(&upd[UPD_MAXG], (unsigned long long)(R.i1 - R.i0));
  }
}

// Compaction of a sorted batch list by its kept flags (the tidied batch):
// entry i goes to pos[i] - *pos_base when keep[i].
__global__ void tidy_compact_kernel(const uint32_t *src, const uint32_t *dst, const float *w, size_t n,
                                    const uint32_t *keep, const uint32_t *pos, const uint32_t *pos_base,
                                    uint32_t *osrc, uint32_t *odst, float *ow) {
  const uint32_t b = pos_base ? *pos_base : 0;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    if (!keep[i]) continue;
    const uint32_t o = pos[i] - b;
    osrc[o] = src[i];
    odst[o] = dst[i];
    ow[o] = w[i];
  }
}

// Copy every row into a new gapped layout (one warp per row; gaps zero).
__global__ void relayout_kernel(const uint64_t *old_off, const uint32_t *deg, const uint32_t *old_key,
                                const float *old_w, size_t n, const uint64_t *off, const uint32_t *cap,
                                uint32_t *key, float *w) {
  const size_t warps = size_t(gridDim.x) * blockDim.x / 32;
  const uint32_t lane = threadIdx.x & 31;
  for (size_t u = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; u < n; u += warps) {
    const uint64_t s = old_off[u], o = off[u];
    const uint32_t d = deg[u];
    for (uint32_t i = lane; i < cap[u]; i += 32) {
      key[o + i] = i < d ? old_key[s + i] : 0;
      w[o + i] = i < d ? old_w[s + i] : 0.f;
    }
  }
}

}  // namespace

void launch_row_caps(const uint64_t *coff, size_t n, uint32_t *deg, uint32_t *cap, uint64_t *cap64, cudaStream_t s) {
  if (!n) return;
  row_caps_kernel<<<grid_for(n, 256), 256, 0, s>>>(coff, n, deg, cap, cap64);
  LVG_CHECK_LAUNCH();
}

void launch_spread_rows(const uint64_t *coff, const uint32_t *ckey, const float *cw, size_t n, const uint64_t *off,
                        const uint32_t *cap, uint32_t *key, float *w, cudaStream_t s) {
  if (!n) return;
  spread_rows_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(coff, ckey, cw, n, off, cap, key, w);
  LVG_CHECK_LAUNCH();
}

void launch_row_plan(const uint64_t *off, const uint32_t *deg, const uint32_t *cap, const uint32_t *key,
                     const float *w, const UpdRow *rows, size_t nrows, const uint32_t *dd, const uint32_t *id,
                     const float *iw, size_t nd_all, uint32_t *pre, uint32_t *keep, RowPlan *plan, uint64_t *len,
                     uint64_t *src, uint64_t *grow, uint8_t *ex, unsigned long long *upd, double *wdelta,
                     cudaStream_t s) {
  if (!nrows) return;
  row_plan_kernel<<<grid_for(nrows * 32, 256), 256, 0, s>>>(off, deg, cap, key, w, rows, nrows, dd, id, iw, nd_all,
                                                              pre, keep, plan, len, src, grow, ex, upd, wdelta);
  LVG_CHECK_LAUNCH();
}

void launch_merge_items(const uint64_t *off, const uint32_t *deg, const uint32_t *key, const float *w,
                        const UpdRow *rows, size_t nrows, const uint32_t *dd, const uint32_t *id, const float *iw,
                        size_t nd_all, const uint32_t *pre, const uint32_t *keep, const RowPlan *plan,
                        const uint64_t *src, uint64_t total, const uint64_t *spos, uint32_t *skey, float *sw,
                        cudaStream_t s) {
  if (!total) return;
  merge_items_kernel<<<grid_for(total, 256), 256, 0, s>>>(off, deg, key, w, rows, uint32_t(nrows), dd, id, iw, nd_all,
                                                          pre, keep, plan, src, total, spos, skey, sw);
  LVG_CHECK_LAUNCH();
}

void launch_copy_items(const uint64_t *off, const UpdRow *rows, size_t nrows, const RowPlan *plan,
                       const uint64_t *spos, uint64_t total, const uint64_t *grow, const uint64_t *gpos,
                       uint64_t pool, const uint32_t *skey, const float *sw, uint32_t *key, float *w,
                       cudaStream_t s) {
  if (!total) return;
  copy_items_kernel<<<grid_for(total, 256), 256, 0, s>>>(off, rows, uint32_t(nrows), plan, spos, total, grow, gpos,
                                                         pool, skey, sw, key, w);
  LVG_CHECK_LAUNCH();
}

void launch_finish_rows(uint64_t *off, uint32_t *deg, uint32_t *cap, uint32_t *key, float *w, const UpdRow *rows,
                        size_t nrows, const RowPlan *plan, const uint64_t *grow, const uint64_t *gpos,
                        uint64_t pool, cudaStream_t s) {
  if (!nrows) return;
  finish_rows_kernel<<<grid_for(nrows * 32, 256), 256, 0, s>>>(off, deg, cap, key, w, rows, nrows, plan, grow, gpos,
                                                                 pool);
  LVG_CHECK_LAUNCH();
}

void launch_count_present(const uint8_t *ex, size_t span, unsigned long long *upd, cudaStream_t s) {
  if (!span) return;
  count_present_kernel<<<grid_for(span, 256), 256, 0, s>>>(ex, span, &upd[UPD_ORDER]);
  LVG_CHECK_LAUNCH();
}

void launch_tidy_compact(const uint32_t *src, const uint32_t *dst, const float *w, size_t n, const uint32_t *keep,
                         const uint32_t *pos, const uint32_t *pos_base, uint32_t *osrc, uint32_t *odst, float *ow,
                         cudaStream_t s) {
  if (!n) return;
  tidy_compact_kernel<<<grid_for(n, 256), 256, 0, s>>>(src, dst, w, n, keep, pos, pos_base, osrc, odst, ow);
  LVG_CHECK_LAUNCH();
}

void launch_pack_keys(const uint32_t *src, const uint32_t *dst, size_t n, int b, uint64_t *key, uint32_t *val,
                      cudaStream_t s) {
  if (!n) return;
  pack_keys_kernel<<<grid_for(n, 256), 256, 0, s>>>(src, dst, n, b, key, val);
  LVG_CHECK_LAUNCH();
}

void launch_first_flags(const uint64_t *key, size_t n, uint32_t *flag, cudaStream_t s) {
  if (!n) return;
  first_flags_kernel<<<grid_for(n, 256), 256, 0, s>>>(key, n, flag);
  LVG_CHECK_LAUNCH();
}

void launch_unpack_keys(const uint64_t *key, const uint32_t *val, const uint32_t *flag, const uint32_t *pos,
                        size_t n, int b, const float *w, uint32_t *os, uint32_t *od, float *ow, cudaStream_t s) {
  if (!n) return;
  unpack_keys_kernel<<<grid_for(n, 256), 256, 0, s>>>(key, val, flag, pos, n, b, w, os, od, ow);
  LVG_CHECK_LAUNCH();
}

void launch_plan_rows(const uint32_t *ds, const uint32_t *nd, const uint32_t *is, const uint32_t *ni, size_t cap,
                      uint32_t *touched, uint32_t *tpos, uint32_t *scan, size_t span, UpdRow *rows,
                      unsigned long long *upd, uint32_t *nrows, cudaStream_t s) {
  LVG_CUDA(cudaMemsetAsync(touched, 0, span * sizeof(uint32_t), s));
  if (cap) {
    touch_kernel<<<grid_for(cap, 256), 256, 0, s>>>(ds, nd, is, ni, cap, touched);
    LVG_CHECK_LAUNCH();
  }
  exclusive_scan_u32(touched, tpos, span, nrows, scan, s);
  plan_rows_kernel<<<grid_for(span, 256), 256, 0, s>>>(touched, tpos, span, ds, nd, is, ni, rows, upd);
  LVG_CHECK_LAUNCH();
}

void launch_fresh_caps(const uint32_t *deg, size_t n, uint32_t *cap, uint64_t *cap64, cudaStream_t s) {
  if (!n) return;
  fresh_caps_kernel<<<grid_for(n, 256), 256, 0, s>>>(deg, n, cap, cap64);
  LVG_CHECK_LAUNCH();
}

void launch_relayout_rows(const uint64_t *old_off, const uint32_t *deg, const uint32_t *old_key, const float *old_w,
                          size_t n, const uint64_t *off, const uint32_t *cap, uint32_t *key, float *w,
                          cudaStream_t s) {
  if (!n) return;
  relayout_kernel<<<grid_for(n * 32, 256), 256, 0, s>>>(old_off, deg, old_key, old_w, n, off, cap, key, w);
  LVG_CHECK_LAUNCH();
}

}  // namespace lvg
