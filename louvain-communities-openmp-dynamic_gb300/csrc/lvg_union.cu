// lvg_union.cu — kernels of graph unions: many independent graphs laid out
// back to back and clustered by one static Louvain run (lvg_static_union),
// each graph keeping the pass driver of inc/louvain.hxx:1180-1215 for itself.
//
// Graph i owns the vertices [gbase[i], gbase[i+1]) of each level; its
// communities are ids in the same range, since no edge leaves a graph. The
// per-graph control (GraphCtl) decides, for each graph alone, what the
// reference's driver decides for the whole graph: when an iteration loop
// stops, whether a pass aggregates, and when the graph is done.
#include "lvg_internal.cuh"

namespace lvg {
namespace {

#define GRID_STRIDE(i, n) for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < (n); i += size_t(gridDim.x) * blockDim.x)

int grid(size_t n, int block) { return grid_for(n, block); }

// One block per graph: gid[x] = i over the graph's range.
__global__ void fill_gid_kernel(const uint32_t *vb, size_t n, uint32_t *gid) {
  for (size_t i = blockIdx.x; i < n; i += gridDim.x)
    for (uint32_t x = vb[i] + threadIdx.x; x < vb[i + 1]; x += blockDim.x) gid[x] = uint32_t(i);
}

__global__ void union_degrees_kernel(const uint32_t *deg, size_t span, uint64_t *dst) {
  GRID_STRIDE(u, span) dst[u] = deg[u];
}

// A warp per row: the row's entries, ids shifted by the graph's first vertex.
__global__ void union_rows_kernel(const uint64_t *off, const uint32_t *deg, const uint32_t *key, const float *w,
                                  size_t span, uint32_t vbase, const uint64_t *coff, uint32_t *ckey, float *cw) {
  const size_t warps = size_t(gridDim.x) * blockDim.x / 32;
  const int lane = threadIdx.x & 31;
  for (size_t u = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32; u < span; u += warps) {
    const uint64_t o = off[u], t = coff[vbase + u];
    const uint32_t d = deg[u];
    for (uint32_t j = lane; j < d; j += 32) {
      ckey[t + j] = key[o + j] + vbase;
      cw[t + j] = w[o + j];
    }
  }
}

// The iteration loop of louvainMoveOmpW (inc/louvain.hxx:588-609) per graph:
// el = Σ gains / M; stop when el <= E or after L iterations.
__global__ void iter_control_kernel(size_t n, GraphCtl *ctl, uint8_t *gact, unsigned long long *fix, const double *M,
                                    double E, int L, unsigned int *active) {
  GRID_STRIDE(i, n) {
    if (!gact[i]) continue;
    const double el = double(fix[i]) / GAIN_FIX / M[i];
    fix[i] = 0;
    GraphCtl &c = ctl[i];
    c.el = el;
    c.it += 1;
    if (el <= E || c.it >= uint32_t(L)) gact[i] = 0;
    else atomicAdd(active, 1u);
  }
}

__global__ void pass_begin_kernel(size_t n, GraphCtl *ctl, uint8_t *gact) {
  GRID_STRIDE(i, n) {
    ctl[i].it = 0;
    ctl[i].el = 0;
    gact[i] = !ctl[i].done;
  }
}

// After local moving: m = iterations (0 if the first found nothing),
// l += max(m, 1), ++p; done when m <= 1 or p >= P (inc/louvain.hxx:1190-1193).
__global__ void pass_end_kernel(size_t n, GraphCtl *ctl, int P) {
  GRID_STRIDE(i, n) {
    GraphCtl &c = ctl[i];
    if (c.done) continue;
    const uint32_t m = (c.it > 1 || c.el != 0) ? c.it : 0;
    c.l += m > 1 ? m : 1;
    c.p += 1;
    c.fin = m <= 1 || c.p >= uint32_t(P);
  }
}

// The driver's loop condition `M > 0 && P > 0`: such graphs never start.
__global__ void pass_skip_kernel(size_t n, GraphCtl *ctl, const double *M, int P) {
  GRID_STRIDE(i, n) ctl[i].fin = !(M[i] > 0 && P > 0);
}

__global__ void union_flags_kernel(const uint8_t *ex, size_t span, const uint32_t *vcom, const uint32_t *gid,
                                   const GraphCtl *ctl, uint32_t *cext) {
  GRID_STRIDE(u, span) {
    if (ex && !ex[u]) continue;
    const GraphCtl &c = ctl[gid[u]];
    if (c.fin || c.done) continue;
    cext[vcom[u]] = 1;
  }
}

// One block per graph: count its communities; at CN/GN >= tol the graph
// finishes here (inc/louvain.hxx:1195-1196) and its flags are cleared so
// that it takes no ids on the next level.
__global__ void union_tolerance_kernel(size_t n, const uint32_t *gbase, uint32_t *cext, GraphCtl *ctl,
                                       const uint64_t *order, bool first, double tol) {
  __shared__ unsigned long long part[32];
  __shared__ int s_fin;
  for (size_t i = blockIdx.x; i < n; i += gridDim.x) {
    GraphCtl &c = ctl[i];
    if (c.fin || c.done) continue;  // block-uniform
    const uint32_t b0 = gbase[i], b1 = gbase[i + 1];
    unsigned long long k = 0;
    for (uint32_t x = b0 + threadIdx.x; x < b1; x += blockDim.x) k += cext[x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = k;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long cn = 0;
      for (int w = 0; w < int(blockDim.x >> 5); ++w) cn += part[w];
      const double gn = first ? double(order[i]) : double(b1 - b0);
      c.cn = uint32_t(cn);
      s_fin = double(cn) / gn >= tol;
      if (s_fin) c.fin = 1;
    }
    __syncthreads();
    if (s_fin)
      for (uint32_t x = b0 + threadIdx.x; x < b1; x += blockDim.x) cext[x] = 0;
    __syncthreads();
  }
}

__global__ void union_snapshot_kernel(size_t span, const uint32_t *gid, const uint32_t *gbase, const uint32_t *vb0,
                                      const GraphCtl *ctl, const tot_t *ctot, const uint8_t *vaff, tot_t *ct_res,
                                      uint8_t *aff_res) {
  GRID_STRIDE(x, span) {
    const uint32_t i = gid[x];
    if (ctl[i].done) continue;
    const size_t r = size_t(vb0[i]) + (x - gbase[i]);
    ct_res[r] = ctot[x];
    aff_res[r] = vaff[x];
  }
}

__global__ void union_finalize_kernel(size_t S, const uint32_t *gid0, const uint32_t *ucom, const uint32_t *vcom,
                                      const uint32_t *gbase, const GraphCtl *ctl, uint32_t *q) {
  GRID_STRIDE(v, S) {
    const uint32_t i = gid0[v];
    const GraphCtl &c = ctl[i];
    if (!c.fin || c.done) continue;
    const uint32_t x = ucom[v];
    q[v] = (vcom ? vcom[x] : x) - gbase[i];
  }
}

__global__ void union_mark_done_kernel(size_t n, GraphCtl *ctl) {
  GRID_STRIDE(i, n) {
    if (ctl[i].fin) {
      ctl[i].done = 1;
      ctl[i].fin = 0;
    }
  }
}

__global__ void union_lookup_kernel(uint32_t *ucom, const uint32_t *map, size_t S, const uint32_t *gid0,
                                    const GraphCtl *ctl) {
  GRID_STRIDE(v, S) {
    if (ctl[gid0[v]].done) continue;
    ucom[v] = map[ucom[v]];
  }
}

__global__ void union_bases_kernel(size_t n, const uint32_t *gbase, size_t span, const uint32_t *cext,
                                   const uint32_t *total, uint32_t *gbase_new) {
  GRID_STRIDE(i, n + 1) {
    const uint32_t b = gbase[i];
    gbase_new[i] = b < span ? cext[b] : *total;
  }
}

__global__ void union_aggex_kernel(const uint8_t *ex, size_t span, const uint32_t *gid, const GraphCtl *ctl,
                                   uint8_t *aggex) {
  GRID_STRIDE(u, span) {
    const GraphCtl &c = ctl[gid[u]];
    aggex[u] = (!ex || ex[u]) && !c.fin && !c.done;
  }
}

// One block per graph: residual flags equal to 1 (as count_flags_kernel).
__global__ void union_affected_kernel(size_t n, const uint32_t *vb0, const uint8_t *aff, GraphCtl *ctl) {
  __shared__ unsigned long long part[32];
  for (size_t i = blockIdx.x; i < n; i += gridDim.x) {
    unsigned long long k = 0;
    for (uint32_t x = vb0[i] + threadIdx.x; x < vb0[i + 1]; x += blockDim.x) k += aff[x] == 1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) k += __shfl_xor_sync(0xffffffffu, k, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = k;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long t = 0;
      for (int w = 0; w < int(blockDim.x >> 5); ++w) t += part[w];
      ctl[i].aff = t;
    }
    __syncthreads();
  }
}

unsigned blocks_per_graph(size_t n) { return unsigned(std::min<size_t>(n, size_t(1) << 20)); }

}  // namespace

void launch_fill_gid(const uint32_t *vb, size_t n, uint32_t *gid, cudaStream_t s) {
  if (!n) return;
  fill_gid_kernel<<<blocks_per_graph(n), 256, 0, s>>>(vb, n, gid);
  LVG_CHECK_LAUNCH();
}

void launch_union_degrees(const uint32_t *deg, size_t span, uint64_t *dst, cudaStream_t s) {
  if (!span) return;
  union_degrees_kernel<<<grid(span, 256), 256, 0, s>>>(deg, span, dst);
  LVG_CHECK_LAUNCH();
}

void launch_union_rows(const uint64_t *off, const uint32_t *deg, const uint32_t *key, const float *w, size_t span,
                       uint32_t vbase, const uint64_t *coff, uint32_t *ckey, float *cw, cudaStream_t s) {
  if (!span) return;
  union_rows_kernel<<<grid(span * 32, 256), 256, 0, s>>>(off, deg, key, w, span, vbase, coff, ckey, cw);
  LVG_CHECK_LAUNCH();
}

void launch_iter_control(size_t n, GraphCtl *ctl, uint8_t *gact, unsigned long long *fix, const double *M, double E,
                         int L, Counters *ctr, cudaStream_t s) {
  LVG_CUDA(cudaMemsetAsync(&ctr->gactive, 0, sizeof(unsigned int), s));
  iter_control_kernel<<<grid(n, 256), 256, 0, s>>>(n, ctl, gact, fix, M, E, L, &ctr->gactive);
  LVG_CHECK_LAUNCH();
}

void launch_pass_begin(size_t n, GraphCtl *ctl, uint8_t *gact, cudaStream_t s) {
  pass_begin_kernel<<<grid(n, 256), 256, 0, s>>>(n, ctl, gact);
  LVG_CHECK_LAUNCH();
}

void launch_pass_end(size_t n, GraphCtl *ctl, int P, cudaStream_t s) {
  pass_end_kernel<<<grid(n, 256), 256, 0, s>>>(n, ctl, P);
  LVG_CHECK_LAUNCH();
}

void launch_pass_skip(size_t n, GraphCtl *ctl, const double *M, int P, cudaStream_t s) {
  pass_skip_kernel<<<grid(n, 256), 256, 0, s>>>(n, ctl, M, P);
  LVG_CHECK_LAUNCH();
}

void launch_union_flags(const uint8_t *ex, size_t span, const uint32_t *vcom, const uint32_t *gid,
                        const GraphCtl *ctl, uint32_t *cext, cudaStream_t s) {
  if (!span) return;
  union_flags_kernel<<<grid(span, 256), 256, 0, s>>>(ex, span, vcom, gid, ctl, cext);
  LVG_CHECK_LAUNCH();
}

void launch_union_tolerance(size_t n, const uint32_t *gbase, uint32_t *cext, GraphCtl *ctl, const uint64_t *order,
                            bool first, double tol, cudaStream_t s) {
  union_tolerance_kernel<<<blocks_per_graph(n), 256, 0, s>>>(n, gbase, cext, ctl, order, first, tol);
  LVG_CHECK_LAUNCH();
}

void launch_union_snapshot(size_t span, const uint32_t *gid, const uint32_t *gbase, const uint32_t *vb0,
                           const GraphCtl *ctl, const tot_t *ctot, const uint8_t *vaff, tot_t *ct_res,
                           uint8_t *aff_res, cudaStream_t s) {
  if (!span) return;
  union_snapshot_kernel<<<grid(span, 256), 256, 0, s>>>(span, gid, gbase, vb0, ctl, ctot, vaff, ct_res, aff_res);
  LVG_CHECK_LAUNCH();
}

void launch_union_finalize(size_t S, const uint32_t *gid0, const uint32_t *ucom, const uint32_t *vcom,
                           const uint32_t *gbase, GraphCtl *ctl, uint32_t *q, cudaStream_t s) {
  if (!S) return;
  union_finalize_kernel<<<grid(S, 256), 256, 0, s>>>(S, gid0, ucom, vcom, gbase, ctl, q);
  LVG_CHECK_LAUNCH();
}

void launch_union_mark_done(size_t n, GraphCtl *ctl, cudaStream_t s) {
  union_mark_done_kernel<<<grid(n, 256), 256, 0, s>>>(n, ctl);
  LVG_CHECK_LAUNCH();
}

void launch_union_lookup(uint32_t *ucom, const uint32_t *map, size_t S, const uint32_t *gid0, const GraphCtl *ctl,
                         cudaStream_t s) {
  if (!S) return;
  union_lookup_kernel<<<grid(S, 256), 256, 0, s>>>(ucom, map, S, gid0, ctl);
  LVG_CHECK_LAUNCH();
}

void launch_union_bases(size_t n, const uint32_t *gbase, size_t span, const uint32_t *cext, const uint32_t *total,
                        uint32_t *gbase_new, cudaStream_t s) {
  union_bases_kernel<<<grid(n + 1, 256), 256, 0, s>>>(n, gbase, span, cext, total, gbase_new);
  LVG_CHECK_LAUNCH();
}

void launch_union_aggex(const uint8_t *ex, size_t span, const uint32_t *gid, const GraphCtl *ctl, uint8_t *aggex,
                        cudaStream_t s) {
  if (!span) return;
  union_aggex_kernel<<<grid(span, 256), 256, 0, s>>>(ex, span, gid, ctl, aggex);
  LVG_CHECK_LAUNCH();
}

void launch_union_affected(size_t n, const uint32_t *vb0, const uint8_t *aff_res, GraphCtl *ctl, cudaStream_t s) {
  union_affected_kernel<<<blocks_per_graph(n), 256, 0, s>>>(n, vb0, aff_res, ctl);
  LVG_CHECK_LAUNCH();
}

}  // namespace lvg
