// lvg_server.cu — a serving loop over many graphs resident in HBM.
//
// The reference processes one graph and one batch at a time on the host
// (main.cxx:101-135: tidy + apply the batch, then each dynamic method). A
// server keeps many graphs and their community state in HBM and answers a
// stream of batch updates: each request is a host batch for one graph; a
// worker uploads it, tidies and applies it to the graph in HBM, and runs the
// configured dynamic method from the graph's current state, which the result
// replaces. Requests for one graph run in arrival order, one at a time;
// requests for different graphs run concurrently on the graphs' own streams
// (one host worker thread per request in flight). With `coalesce` set, a
// worker that picks a graph takes the requests queued for it (up to
// `coalesce` batch entries) and serves them as one batch — their union, tidied
// and applied at once — so that fixed per-request costs are paid once under
// load; every one of them then completes with that run's result (the info's
// `group` and `coalesced` fields say which requests ran together). The tidy
// applies every deletion of a batch before every insertion and drops an
// insertion of an edge already present, so a group closes at the first request
// that touches an edge an earlier request of the group inserts or deletes
// (insert-then-delete, delete-then-insert, or a second insertion of one edge):
// the graph after a group is then the graph after its requests one by one.
// Admission control keeps
// the device bytes of the resident graphs under a budget: a graph is admitted
// on its measured bytes after its first run (graph, workspace, state) plus
// the per-request scratch, and only while the device has that much free.
//
// Host code only: it calls the library's own C-ABI.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "lvg_internal.cuh"

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  uint64_t ticket = 0;
  int graph = 0;
  std::vector<uint32_t> ds, dd, is, id;
  std::vector<float> dw, iw;
  double t_submit = 0;
};

struct Slot {
  lvg_graph *g = nullptr;
  lvg_state *st = nullptr;
  lvg_device_batch *db = nullptr;  // reused by every request of the graph
  bool owns_graph = false;
  std::deque<Request> q;
  bool busy = false;
  size_t bytes = 0;
  uint64_t served = 0;
};

}  // namespace

struct lvg_server {
  lvg_server_options opt{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::vector<std::unique_ptr<Slot>> slots;
  std::unordered_map<uint64_t, lvg_request_info> done;
  std::vector<std::thread> workers;
  bool stop = false;
  uint64_t next_ticket = 1;
  size_t bytes_used = 0, rr = 0, pending = 0;
  int device = 0;
  // statistics since the last reset
  std::vector<double> lat;
  double sum_queue = 0, sum_apply = 0, sum_run = 0;
  uint64_t completed = 0, updates = 0, failed = 0;
  double t_first = 0, t_last = 0;
};

namespace {

// The next graph with work and no request in flight (round robin), or -1.
int pick(lvg_server *sv) {
  const size_t n = sv->slots.size();
  for (size_t k = 0; k < n; ++k) {
    const size_t i = (sv->rr + k) % n;
    Slot &s = *sv->slots[i];
    if (!s.busy && !s.q.empty()) {
      sv->rr = i + 1;
      return int(i);
    }
  }
  return -1;
}

// Directed edges a coalesced group inserts and deletes so far.
struct GroupEdges {
  std::unordered_set<uint64_t> ins, del;
  static uint64_t key(uint32_t u, uint32_t v) { return uint64_t(u) << 32 | v; }
  // Whether r touches an edge the group already inserts or deletes in a way
  // the union's tidy would resolve differently from r applied after it.
  bool conflicts(const Request &r) const {
    for (size_t i = 0; i < r.ds.size(); ++i)
      if (ins.count(key(r.ds[i], r.dd[i]))) return true;
    for (size_t i = 0; i < r.is.size(); ++i) {
      const uint64_t k = key(r.is[i], r.id[i]);
      if (ins.count(k) || del.count(k)) return true;
    }
    return false;
  }
  void add(const Request &r) {
    for (size_t i = 0; i < r.ds.size(); ++i) del.insert(key(r.ds[i], r.dd[i]));
    for (size_t i = 0; i < r.is.size(); ++i) ins.insert(key(r.is[i], r.id[i]));
  }
};

// The union of several requests' batches (deletions, then insertions, in
// arrival order).
Request merge(std::vector<Request> &rs) {
  if (rs.size() == 1) return std::move(rs[0]);
  Request m;
  m.graph = rs[0].graph;
  m.t_submit = rs[0].t_submit;
  for (auto &r : rs) {
    m.ds.insert(m.ds.end(), r.ds.begin(), r.ds.end());
    m.dd.insert(m.dd.end(), r.dd.begin(), r.dd.end());
    m.dw.insert(m.dw.end(), r.dw.begin(), r.dw.end());
    m.is.insert(m.is.end(), r.is.begin(), r.is.end());
    m.id.insert(m.id.end(), r.id.begin(), r.id.end());
    m.iw.insert(m.iw.end(), r.iw.begin(), r.iw.end());
  }
  return m;
}

void serve(lvg_server *sv, Slot &s, const Request &r, lvg_request_info &info) {
  const double t0 = now_ms();
  info.queue_ms = t0 - r.t_submit;
  lvg_batch b{r.ds.size(), r.ds.data(), r.dd.data(), r.dw.data(), r.is.size(), r.is.data(), r.id.data(),
              r.iw.data()};
  int rc = s.db ? lvg_device_batch_set(s.db, &b) : lvg_device_batch_create(s.g, &b, &s.db);
  lvg_device_batch *db = s.db;
  if (rc == LVG_OK) rc = lvg_graph_apply_device_batch(s.g, db);
  const double t1 = now_ms();
  info.apply_ms = t1 - t0;
  if (rc == LVG_OK) {
    size_t nd = 0, ni = 0;
    lvg_device_batch_size(db, &nd, &ni);
    info.tidy_deletions = nd;
    info.tidy_insertions = ni;
    lvg_result res{};
    rc = lvg_run_resident(s.g, sv->opt.method, db, s.st, s.st, &sv->opt.louvain, &res);
    info.iterations = res.iterations;
    info.passes = res.passes;
    info.affected = res.affectedVertices;
  }
  info.run_ms = now_ms() - t1;
  info.status = rc;
}

void worker(lvg_server *sv) {
  cudaSetDevice(sv->device);
  std::unique_lock<std::mutex> lk(sv->mu);
  for (;;) {
    int i = -1;
    sv->cv_work.wait(lk, [&] { return sv->stop || (i = pick(sv)) >= 0; });
    if (i < 0) return;  // stopping and nothing runnable
    Slot &s = *sv->slots[size_t(i)];
    std::vector<Request> rs;
    size_t entries = 0;
    GroupEdges seen;
    // one request, or (coalescing) the queued ones up to the entry cap and the
    // first conflicting request
    for (;;) {
      const Request &r = s.q.front();
      const size_t n = r.ds.size() + r.is.size();
      if (!rs.empty() && (entries + n > sv->opt.coalesce || seen.conflicts(r))) break;
      if (sv->opt.coalesce) seen.add(r);
      entries += n;
      rs.push_back(std::move(s.q.front()));
      s.q.pop_front();
      if (!sv->opt.coalesce || s.q.empty()) break;
    }
    s.busy = true;
    lk.unlock();
    std::vector<uint64_t> tickets;
    std::vector<double> submitted;
    for (auto &r : rs) { tickets.push_back(r.ticket); submitted.push_back(r.t_submit); }
    const Request r = merge(rs);
    lvg_request_info info{};
    info.graph = r.graph;
    serve(sv, s, r, info);
    const double t = now_ms();
    lk.lock();
    s.busy = false;
    ++s.served;
    for (size_t k = 0; k < tickets.size(); ++k) {
      lvg_request_info ik = info;
      ik.ticket = tickets[k];
      ik.group = tickets[0];
      ik.coalesced = int(tickets.size());
      ik.latency_ms = t - submitted[k];
      ik.queue_ms = info.queue_ms + (submitted[0] - submitted[k]);
      --sv->pending;
      if (ik.status == LVG_OK) {
        ++sv->completed;
        sv->lat.push_back(ik.latency_ms);
        sv->sum_queue += ik.queue_ms;
        sv->sum_apply += ik.apply_ms;
        sv->sum_run += ik.run_ms;
      } else {
        ++sv->failed;
      }
      if (sv->t_first == 0 || submitted[k] < sv->t_first) sv->t_first = submitted[k];
      sv->done[tickets[k]] = ik;
    }
    if (info.status == LVG_OK) sv->updates += entries;
    sv->t_last = std::max(sv->t_last, t);
    sv->cv_done.notify_all();
    sv->cv_work.notify_all();
  }
}

}  // namespace

extern "C" {

void lvg_server_options_default(lvg_server_options *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->workers = 8;
  o->hbm_budget = size_t(120) << 30;
  o->method = LVG_METHOD_FRONTIER;
  lvg_options_default(&o->louvain);
}

size_t lvg_graph_footprint(size_t span, size_t edges) {
  // gapped rows + pool (~1.3 x 8 B per edge), two aggregation levels (2 x 8 B
  // per edge), per-vertex arrays of the graph, workspace and one state
  return edges * 27 + span * 200 + (size_t(4) << 20);
}

int lvg_server_create(const lvg_server_options *o, lvg_server **out) {
  if (!out) return lvg::fail_noalloc(LVG_EINVAL, "null argument");
  *out = nullptr;
  std::unique_ptr<lvg_server> sv(new lvg_server());
  if (o) sv->opt = *o; else lvg_server_options_default(&sv->opt);
  if (sv->opt.workers < 1 || sv->opt.workers > 256 || sv->opt.method < LVG_METHOD_NAIVE ||
      sv->opt.method > LVG_METHOD_FRONTIER)
    return lvg::fail_noalloc(LVG_EINVAL, "lvg_server_create: bad options");
  if (cudaGetDevice(&sv->device) != cudaSuccess) return lvg::fail_noalloc(LVG_ECUDA, "no CUDA device");
  for (int i = 0; i < sv->opt.workers; ++i) sv->workers.emplace_back(worker, sv.get());
  *out = sv.release();
  return LVG_OK;
}

int lvg_server_add_graph(lvg_server *sv, lvg_graph *g, int take_ownership, const uint32_t *q, const double *qvtot,
                         const double *qctot, int *graph_id) {
  if (!sv || !g || !graph_id) return lvg::fail_noalloc(LVG_EINVAL, "null argument");
  if (q && (!qvtot || !qctot)) return lvg::fail_noalloc(LVG_EINVAL, "lvg_server_add_graph: q without weights");
  {  // a first check on the a-priori estimate, before any work
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->bytes_used + lvg_graph_footprint(lvg_graph_span(g), lvg_graph_size(g)) / 2 > sv->opt.hbm_budget)
      return lvg::fail_noalloc(LVG_ENOMEM, "lvg_server_add_graph: the HBM budget is used up (admission denied)");
  }
  lvg_state *st = nullptr;
  int rc = lvg_state_create(g, &st);
  if (rc != LVG_OK) return rc;
  if (q) {
    rc = lvg_state_set(st, q, qvtot, qctot);
  } else {  // no prior: the static communities
    lvg_result res{};
    rc = lvg_run_resident(g, LVG_METHOD_STATIC, nullptr, nullptr, st, &sv->opt.louvain, &res);
  }
  if (rc == LVG_OK) rc = lvg_graph_trim(g, 1);  // the static pass's hash tables are not needed again
  if (rc != LVG_OK) {
    lvg_state_destroy(st);
    return rc;
  }
  // measured: graph + workspace + state, plus per-request scratch (span-sized
  // plan arrays, batch-sized buffers, the dynamic pass's hash tables)
  const size_t span = lvg_graph_span(g);
  const size_t bytes = lvg_graph_device_bytes(g) + lvg_state_device_bytes(st) + 24 * span + (size_t(64) << 20);
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
  std::lock_guard<std::mutex> lk(sv->mu);
  const size_t now = lvg_graph_device_bytes(g) + lvg_state_device_bytes(st);
  if (sv->bytes_used + bytes > sv->opt.hbm_budget || free_b < bytes - now + (size_t(1) << 30)) {
    lvg_state_destroy(st);
    return lvg::fail_noalloc(LVG_ENOMEM, "lvg_server_add_graph: the HBM budget is used up (admission denied)");
  }
  sv->bytes_used += bytes;
  std::unique_ptr<Slot> s(new Slot());
  s->g = g;
  s->st = st;
  s->owns_graph = take_ownership != 0;
  s->bytes = bytes;
  sv->slots.push_back(std::move(s));
  *graph_id = int(sv->slots.size() - 1);
  return LVG_OK;
}

int lvg_server_set_coalesce(lvg_server *sv, size_t coalesce) {
  if (!sv) return lvg::fail_noalloc(LVG_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(sv->mu);
  sv->opt.coalesce = coalesce;
  return LVG_OK;
}

int lvg_server_submit(lvg_server *sv, int graph_id, const lvg_batch *b, uint64_t *ticket) {
  if (!sv || !b || !ticket) return lvg::fail_noalloc(LVG_EINVAL, "null argument");
  Request r;
  r.graph = graph_id;
  r.ds.assign(b->del_src, b->del_src + b->num_deletions);
  r.dd.assign(b->del_dst, b->del_dst + b->num_deletions);
  r.dw.assign(b->del_w, b->del_w + b->num_deletions);
  r.is.assign(b->ins_src, b->ins_src + b->num_insertions);
  r.id.assign(b->ins_dst, b->ins_dst + b->num_insertions);
  r.iw.assign(b->ins_w, b->ins_w + b->num_insertions);
  std::lock_guard<std::mutex> lk(sv->mu);
  if (graph_id < 0 || size_t(graph_id) >= sv->slots.size())
    return lvg::fail_noalloc(LVG_EINVAL, "lvg_server_submit: unknown graph");
  r.t_submit = now_ms();
  r.ticket = sv->next_ticket++;
  *ticket = r.ticket;
  sv->slots[size_t(graph_id)]->q.push_back(std::move(r));
  ++sv->pending;
  sv->cv_work.notify_one();
  return LVG_OK;
}

int lvg_server_wait(lvg_server *sv, uint64_t ticket, lvg_request_info *info) {
  if (!sv) return lvg::fail_noalloc(LVG_EINVAL, "null argument");
  std::unique_lock<std::mutex> lk(sv->mu);
  if (ticket == 0 || ticket >= sv->next_ticket) return lvg::fail_noalloc(LVG_EINVAL, "lvg_server_wait: unknown ticket");
  sv->cv_done.wait(lk, [&] { return sv->done.count(ticket) > 0; });
  const lvg_request_info r = sv->done[ticket];
  sv->done.erase(ticket);
  if (info) *info = r;
  return r.status;
}

int lvg_server_drain(lvg_server *sv) {
  if (!sv) return lvg::fail_noalloc(LVG_EINVAL, "null argument");
  std::unique_lock<std::mutex> lk(sv->mu);
  sv->cv_done.wait(lk, [&] { return sv->pending == 0; });
  return sv->failed ? LVG_ECUDA : LVG_OK;
}

int lvg_server_stats(lvg_server *sv, int reset, lvg_server_stats_t *out) {
  if (!sv || !out) return lvg::fail_noalloc(LVG_EINVAL, "null argument");
  std::lock_guard<std::mutex> lk(sv->mu);
  std::memset(out, 0, sizeof(*out));
  out->completed = sv->completed;
  out->failed = sv->failed;
  out->updates = sv->updates;
  out->graphs = sv->slots.size();
  out->hbm_reserved = sv->bytes_used;
  std::vector<double> l = sv->lat;
  if (!l.empty()) {
    std::sort(l.begin(), l.end());
    auto pct = [&](double p) { return l[std::min(l.size() - 1, size_t(p * double(l.size() - 1) + 0.5))]; };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    out->max_ms = l.back();
    double sum = 0;
    for (double x : l) sum += x;
    out->mean_ms = sum / double(l.size());
    out->mean_queue_ms = sv->sum_queue / double(l.size());
    out->mean_apply_ms = sv->sum_apply / double(l.size());
    out->mean_run_ms = sv->sum_run / double(l.size());
  }
  out->wall_s = sv->t_last > sv->t_first ? (sv->t_last - sv->t_first) / 1e3 : 0;
  out->updates_per_s = out->wall_s > 0 ? double(sv->updates) / out->wall_s : 0;
  out->requests_per_s = out->wall_s > 0 ? double(sv->completed) / out->wall_s : 0;
  if (reset) {
    sv->lat.clear();
    sv->sum_queue = sv->sum_apply = sv->sum_run = 0;
    sv->completed = sv->updates = sv->failed = 0;
    sv->t_first = sv->t_last = 0;
  }
  return LVG_OK;
}

int lvg_server_membership(lvg_server *sv, int graph_id, uint32_t *membership, double *vtot, double *ctot) {
  if (!sv) return lvg::fail_noalloc(LVG_EINVAL, "null argument");
  std::unique_lock<std::mutex> lk(sv->mu);
  if (graph_id < 0 || size_t(graph_id) >= sv->slots.size())
    return lvg::fail_noalloc(LVG_EINVAL, "lvg_server_membership: unknown graph");
  Slot &s = *sv->slots[size_t(graph_id)];
  sv->cv_done.wait(lk, [&] { return !s.busy && s.q.empty(); });
  return lvg_state_get(s.st, membership, vtot, ctot);
}

lvg_graph *lvg_server_graph(lvg_server *sv, int graph_id) {
  if (!sv) return nullptr;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (graph_id < 0 || size_t(graph_id) >= sv->slots.size()) return nullptr;
  return sv->slots[size_t(graph_id)]->g;
}

int lvg_static_many(lvg_graph *const *graphs, size_t n, const lvg_options *o, int workers, int trim,
                    lvg_result *results) {
  if ((n && (!graphs || !results)) || workers < 1 || workers > 256)
    return lvg::fail_noalloc(LVG_EINVAL, "lvg_static_many: bad argument");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return lvg::fail_noalloc(LVG_ECUDA, "no CUDA device");
  std::atomic<size_t> next{0};
  std::atomic<int> first_err{LVG_OK};
  auto work = [&] {
    cudaSetDevice(dev);
    for (size_t i; (i = next.fetch_add(1)) < n;) {
      int rc = lvg_static(graphs[i], o, &results[i]);
      if (rc == LVG_OK && trim) rc = lvg_graph_trim(graphs[i], trim);
      int ok = LVG_OK;
      if (rc != LVG_OK) first_err.compare_exchange_strong(ok, rc);
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < std::min<int>(workers, int(n)); ++t) pool.emplace_back(work);
  work();
  for (auto &t : pool) t.join();
  return first_err.load();
}

int lvg_server_destroy(lvg_server *sv) {
  if (!sv) return LVG_OK;
  {
    std::unique_lock<std::mutex> lk(sv->mu);
    sv->cv_done.wait(lk, [&] { return sv->pending == 0; });
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  for (auto &t : sv->workers) t.join();
  for (auto &s : sv->slots) {
    lvg_device_batch_destroy(s->db);
    lvg_state_destroy(s->st);
    if (s->owns_graph) lvg_graph_destroy(s->g);
  }
  delete sv;
  return LVG_OK;
}

}  // extern "C"
