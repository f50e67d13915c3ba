// lx_server.cpp -- continuous batching of submitted simulations (lx_server_*).
//
// The reference runs one simulation per process (main.cc:53-72).  The server is the engine's
// serving loop: a worker thread owns one lx_batch and steps every running request together,
// chunk by chunk; between chunks finished requests leave, cancelled ones are dropped and
// queued ones join, so no request waits for the others to finish.
//
//   worker:  admit (create handles for the queue head while they fit the device budget)
//            -> enqueue a chunk (lx_batch_step_async) -> prepare the next handles while the
//            GPU runs -> lx_batch_wait -> retire finished / failed / cancelled requests
//
// The chunk is the server's chunk, shortened so that no running request passes its step
// count.  Built only on the public C ABI (luxum.h) plus the CUDA runtime for the default
// budget and the device: a server runs on the device current at its creation (one server
// per GPU for several GPUs).
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "luxum.h"

namespace lx {
lx_status set_thread_error(const char* msg, lx_status st);
}

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  long long id = 0;
  lx_params params;
  int steps = 0;
  std::vector<double> material[3];
  double material_scale = 1.0;
  std::vector<int> boxes;
  std::vector<double> box_eps;
  int dft_axis = 0, dft_index = 0, dft_every = 1;
  std::vector<double> omega;
  double bytes = 0.0;  // admission estimate
  double cells = 0.0;
  int state = LX_REQ_QUEUED;
  bool cancel = false;
  int done = 0;  // steps taken
  int readers = 0;  // client calls reading a finished request's handle outside the lock
  lx_sim* sim = nullptr;
  int dft_id = -1;
  double t_submit = -1, t_start = -1, t_end = -1;
  std::string err;
};

}  // namespace

struct lx_server {
  lx_server_config cfg;
  Clock::time_point t0;
  std::mutex mu;
  std::condition_variable work_cv;  // queue or stop changed
  std::condition_variable done_cv;  // a request reached a final state
  std::map<long long, std::shared_ptr<Request>> reqs;
  std::deque<std::shared_ptr<Request>> queue;
  std::vector<std::shared_ptr<Request>> running;   // members of the batch
  std::vector<std::shared_ptr<Request>> prepared;  // handles created, not yet in the batch
  long long next_id = 1;
  int device = 0;  // CUDA device current at lx_server_create; the worker runs on it
  bool stop = false;
  lx_batch* batch = nullptr;
  lx_server_stats stats;
  std::set<std::array<int, 4>> tried;    // classes tuned (or found to have no tile shape); worker only
  std::vector<lx_tune_entry> table;      // copy of the batch's tile-shape table for clients (under mu)
  std::thread worker;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

lx_status sfail(lx_status st, const std::string& m) { return lx::set_thread_error(m.c_str(), st); }

bool final_state(int s) { return s == LX_REQ_DONE || s == LX_REQ_FAILED || s == LX_REQ_CANCELLED; }

void count_state(lx_server_stats& st, int s, int d) {
  switch (s) {
    case LX_REQ_QUEUED: st.queued += d; break;
    case LX_REQ_RUNNING: st.running += d; break;
    case LX_REQ_DONE: st.done += d; break;
    case LX_REQ_FAILED: st.failed += d; break;
    default: st.cancelled += d; break;
  }
}

// state change under srv->mu
void set_state(lx_server* srv, Request& r, int s) {
  count_state(srv->stats, r.state, -1);
  r.state = s;
  count_state(srv->stats, s, +1);
  if (final_state(s)) {
    r.t_end = srv->now();
    srv->done_cv.notify_all();
  }
}

// Creates and configures a request's handle (no lock held: device allocation and uploads).
lx_status make_sim(Request& r) {
  lx_sim* s = nullptr;
  lx_status st = lx_sim_create(&r.params, &s);
  if (st) {
    r.err = lx_last_error(nullptr);
    return st;
  }
  for (int c = 0; c < 3 && !st; c++)
    if (!r.material[c].empty())
      st = lx_sim_set_material(s, c, r.material[c].data(), r.material[c].size(), r.material_scale);
  for (size_t b = 0; b < r.box_eps.size() && !st; b++)
    st = lx_sim_set_eps_box(s, &r.boxes[6 * b], &r.boxes[6 * b + 3], r.box_eps[b]);
  if (!st && !r.omega.empty())
    st = lx_sim_add_dft_plane(s, r.dft_axis, r.dft_index, (int)r.omega.size(), r.omega.data(), r.dft_every, &r.dft_id);
  if (!st) st = lx_sim_sync(s);
  if (st) {
    r.err = lx_last_error(s);
    lx_sim_destroy(s);
    return st;
  }
  r.sim = s;
  return LX_OK;
}

// Takes queue heads that fit the budget and creates their handles into `prepared`.
void prepare(lx_server* srv) {
  std::unique_lock<std::mutex> lk(srv->mu);
  for (;;) {
    if (srv->stop || srv->queue.empty()) return;
    std::shared_ptr<Request> r = srv->queue.front();
    if (r->cancel) {
      srv->queue.pop_front();
      set_state(srv, *r, LX_REQ_CANCELLED);
      continue;
    }
    const size_t live = srv->running.size() + srv->prepared.size();
    if (live > 0) {
      if (srv->stats.bytes_running + r->bytes > srv->cfg.budget_bytes) return;
      if (srv->cfg.max_running > 0 && (int)live >= srv->cfg.max_running) return;
    }
    srv->queue.pop_front();
    srv->stats.bytes_running += r->bytes;
    lk.unlock();
    const lx_status st = make_sim(*r);
    lk.lock();
    if (st) {
      srv->stats.bytes_running -= r->bytes;
      set_state(srv, *r, LX_REQ_FAILED);
      continue;
    }
    srv->prepared.push_back(r);
  }
}

// Moves prepared handles into the batch (lock held by the caller for the bookkeeping; the
// batch itself is touched only by the worker).
void join(lx_server* srv) {
  for (auto& r : srv->prepared) {
    if (r->cancel) {
      lx_sim_destroy(r->sim);
      r->sim = nullptr;
      srv->stats.bytes_running -= r->bytes;
      set_state(srv, *r, LX_REQ_CANCELLED);
      continue;
    }
    const lx_status st = lx_batch_add(srv->batch, r->sim);
    if (st) {
      r->err = lx_last_error(nullptr);
      lx_sim_destroy(r->sim);
      r->sim = nullptr;
      srv->stats.bytes_running -= r->bytes;
      set_state(srv, *r, LX_REQ_FAILED);
      continue;
    }
    r->t_start = srv->now();
    set_state(srv, *r, LX_REQ_RUNNING);
    srv->running.push_back(r);
  }
  srv->prepared.clear();
  srv->stats.peak_running = std::max(srv->stats.peak_running, (int)srv->running.size());
  srv->stats.peak_bytes_running = std::max(srv->stats.peak_bytes_running, srv->stats.bytes_running);
}

// Tunes the tile shape of each prepared handle's class that has not been tried yet, on twins
// of the handle (lx_batch_tune_member), before it joins.  Worker only, with the batch idle; the
// twins are created and freed inside, outside the memory budget.  A failed tuning leaves the
// default shape.
void tune_prepared(lx_server* srv) {
  if (srv->cfg.tune_steps <= 0) return;
  std::vector<lx_sim*> sims;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    for (auto& r : srv->prepared)
      if (!r->cancel && r->sim) sims.push_back(r->sim);
  }
  for (lx_sim* s : sims) {
    lx_tune_entry k;
    if (lx_sim_tune_class(s, &k)) continue;
    if (!srv->tried.insert({k.planar, k.size_class, k.precision, k.slab_class}).second) continue;
    const auto t0 = Clock::now();
    int m = 0;
    lx_batch_tune_member(srv->batch, s, srv->cfg.tune_steps, &m);
    int n = 0;
    std::vector<lx_tune_entry> table;
    if (!lx_batch_get_tune_table(srv->batch, nullptr, 0, &n) && n > 0) {
      table.resize(n);
      lx_batch_get_tune_table(srv->batch, table.data(), n, &n);
    }
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stats.tune_seconds += std::chrono::duration<double>(Clock::now() - t0).count();
    if (m) srv->stats.tuned_classes += 1;
    srv->table.swap(table);
  }
}

// Retires running requests that finished, blew up or were cancelled (lock held).
void retire(lx_server* srv) {
  std::vector<std::shared_ptr<Request>> keep;
  for (auto& r : srv->running) {
    double m = 0.0;
    lx_sim_max_e2(r->sim, &m);
    int to = -1;
    if (!std::isfinite(m)) {
      r->err = "max|E|^2 is not finite after step " + std::to_string(r->done);
      to = LX_REQ_FAILED;
    } else if (r->cancel) {
      to = LX_REQ_CANCELLED;
    } else if (r->done >= r->steps) {
      to = LX_REQ_DONE;
    }
    if (to < 0) {
      keep.push_back(r);
      continue;
    }
    lx_batch_remove(srv->batch, r->sim);
    srv->stats.bytes_running -= r->bytes;
    if (to != LX_REQ_DONE) {
      lx_sim_destroy(r->sim);
      r->sim = nullptr;
    }
    set_state(srv, *r, to);
  }
  srv->running.swap(keep);
}

void worker_main(lx_server* srv) {
  cudaSetDevice(srv->device);
  auto since = [](Clock::time_point t) { return std::chrono::duration<double>(Clock::now() - t).count(); };
  for (;;) {
    auto t0 = Clock::now();
    prepare(srv);
    const double dp = since(t0);
    tune_prepared(srv);
    int n = 0;
    {
      std::unique_lock<std::mutex> lk(srv->mu);
      srv->stats.prepare_seconds += dp;
      t0 = Clock::now();
      join(srv);
      srv->stats.join_seconds += since(t0);
      if (srv->stop) break;
      if (srv->running.empty()) {
        if (srv->queue.empty()) srv->work_cv.wait(lk, [&] { return srv->stop || !srv->queue.empty(); });
        continue;
      }
      n = srv->cfg.chunk;
      for (auto& r : srv->running) n = std::min(n, r->steps - r->done);
    }
    const auto c0 = Clock::now();
    lx_status st = n > 0 ? lx_batch_step_async(srv->batch, n) : LX_OK;
    const double ds = since(c0);
    t0 = Clock::now();
    if (!st) prepare(srv);  // next handles are created while the chunk runs
    const double dp2 = since(t0);
    t0 = Clock::now();
    const lx_status wst = lx_batch_wait(srv->batch);
    const double dw = since(t0);
    if (!st) st = wst;
    std::unique_lock<std::mutex> lk(srv->mu);
    srv->stats.busy_seconds += since(c0);
    srv->stats.enqueue_seconds += ds;
    srv->stats.prepare_seconds += dp2;
    srv->stats.wait_seconds += dw;
    srv->stats.chunks += 1;
    if (st && st != LX_ERR_BLOWUP) {
      // a CUDA failure of the shared chunk fails every request in it
      const std::string why = lx_last_error(nullptr);
      for (auto& r : srv->running) {
        lx_batch_remove(srv->batch, r->sim);
        lx_sim_destroy(r->sim);
        r->sim = nullptr;
        r->err = why;
        srv->stats.bytes_running -= r->bytes;
        set_state(srv, *r, LX_REQ_FAILED);
      }
      srv->running.clear();
      continue;
    }
    for (auto& r : srv->running) {
      r->done += n;
      srv->stats.cell_updates += r->cells * n;
    }
    t0 = Clock::now();
    retire(srv);
    srv->stats.retire_seconds += since(t0);
  }
  // stopping: cancel what is left
  std::unique_lock<std::mutex> lk(srv->mu);
  for (auto& r : srv->running) {
    lx_batch_remove(srv->batch, r->sim);
    lx_sim_destroy(r->sim);
    r->sim = nullptr;
    set_state(srv, *r, LX_REQ_CANCELLED);
  }
  srv->running.clear();
  for (auto& r : srv->prepared) {
    lx_sim_destroy(r->sim);
    r->sim = nullptr;
    set_state(srv, *r, LX_REQ_CANCELLED);
  }
  srv->prepared.clear();
  for (auto& r : srv->queue) set_state(srv, *r, LX_REQ_CANCELLED);
  srv->queue.clear();
}

std::shared_ptr<Request> find(lx_server* srv, long long id) {
  auto it = srv->reqs.find(id);
  return it == srv->reqs.end() ? nullptr : it->second;
}

}  // namespace

extern "C" LX_API void lx_server_config_init(lx_server_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof *cfg);
  cfg->precision = LX_PREC_FP32;
  cfg->chunk = 100;
}

extern "C" LX_API void lx_request_init(lx_request* r) {
  if (!r) return;
  std::memset(r, 0, sizeof *r);
  lx_params_init(&r->params);
  r->material_scale = 1.0;
  r->dft_every = 1;
}

extern "C" LX_API lx_status lx_server_create(const lx_server_config* cfg, lx_server** out) {
  if (!out) return sfail(LX_ERR_INVALID, "null argument");
  lx_server_config c;
  lx_server_config_init(&c);
  if (cfg) c = *cfg;
  if (c.precision < LX_PREC_FP64 || c.precision > LX_PREC_FP16S) return sfail(LX_ERR_INVALID, "bad precision");
  if (c.chunk < 1) return sfail(LX_ERR_INVALID, "chunk must be >= 1");
  if (c.max_running < 0 || c.budget_bytes < 0 || c.tune_steps < 0 || c.tune_entries < 0)
    return sfail(LX_ERR_INVALID, "negative limit");
  if (c.tune_entries > 0 && !c.tune_table) return sfail(LX_ERR_INVALID, "tune_entries without tune_table");
  if (c.budget_bytes == 0) {
    size_t fr = 0, tot = 0;
    const cudaError_t e = cudaMemGetInfo(&fr, &tot);
    if (e != cudaSuccess) return sfail(LX_ERR_CUDA, std::string("cudaMemGetInfo: ") + cudaGetErrorString(e));
    c.budget_bytes = 0.9 * (double)fr;
  }
  lx_server* srv = new (std::nothrow) lx_server();
  if (!srv) return sfail(LX_ERR_OOM, "host allocation failed");
  srv->cfg = c;
  srv->t0 = Clock::now();
  cudaGetDevice(&srv->device);
  std::memset(&srv->stats, 0, sizeof srv->stats);
  lx_status st = lx_batch_create(&srv->batch);
  if (!st) st = lx_batch_set_chunk(srv->batch, c.chunk);
  if (!st && c.tune_entries > 0) {
    st = lx_batch_set_tune_table(srv->batch, c.tune_table, c.tune_entries);
    int n = 0;
    if (!st) st = lx_batch_get_tune_table(srv->batch, nullptr, 0, &n);  // the batch's copy: one entry per class
    if (!st) {
      srv->table.resize(n);
      st = lx_batch_get_tune_table(srv->batch, srv->table.data(), n, &n);
    }
    if (!st)
      for (const auto& e : srv->table) srv->tried.insert({e.planar, e.size_class, e.precision, e.slab_class});
  }
  srv->cfg.tune_table = nullptr;  // copied: the caller's array need not outlive the call
  srv->cfg.tune_entries = 0;
  if (st) {
    if (srv->batch) lx_batch_destroy(srv->batch);
    delete srv;
    return st;
  }
  srv->worker = std::thread(worker_main, srv);
  *out = srv;
  return LX_OK;
}

extern "C" LX_API void lx_server_destroy(lx_server* srv) {
  if (!srv) return;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->stop = true;
  }
  srv->work_cv.notify_all();
  if (srv->worker.joinable()) srv->worker.join();
  for (auto& kv : srv->reqs)
    if (kv.second->sim) lx_sim_destroy(kv.second->sim);
  lx_batch_destroy(srv->batch);
  delete srv;
}

extern "C" LX_API lx_status lx_server_submit(lx_server* srv, const lx_request* req, long long* id) {
  if (!srv || !req || !id) return sfail(LX_ERR_INVALID, "null argument");
  if (req->params.precision != srv->cfg.precision) return sfail(LX_ERR_INVALID, "request precision differs from the server's");
  if (req->steps < 0) return sfail(LX_ERR_INVALID, "steps must be >= 0");
  if (req->n_boxes < 0 || (req->n_boxes > 0 && (!req->boxes || !req->box_eps)))
    return sfail(LX_ERR_INVALID, "n_boxes boxes and permittivities are required");
  if (req->nfreq < 0 || (req->nfreq > 0 && !req->omega)) return sfail(LX_ERR_INVALID, "nfreq frequencies are required");
  size_t bytes = 0;
  lx_status st = lx_params_device_bytes(&req->params, &bytes);  // validates the parameters
  if (st) return st;
  auto r = std::make_shared<Request>();
  r->params = req->params;
  r->steps = req->steps;
  for (int c = 0; c < 3; c++) {
    if (!req->material[c]) continue;
    int shp[3];
    if ((st = lx_params_field_shape(&req->params, c, shp))) return st;
    const size_t n = (size_t)shp[0] * shp[1] * shp[2];
    if (n == 0) return sfail(LX_ERR_INVALID, "material given for a component this grid does not have");
    r->material[c].assign(req->material[c], req->material[c] + n);
  }
  r->material_scale = req->material_scale;
  r->boxes.assign(req->boxes, req->boxes + 6 * (size_t)req->n_boxes);
  r->box_eps.assign(req->box_eps, req->box_eps + req->n_boxes);
  r->dft_axis = req->dft_axis;
  r->dft_index = req->dft_index;
  r->dft_every = req->dft_every;
  if (req->nfreq > 0) r->omega.assign(req->omega, req->omega + req->nfreq);
  const double Nx = req->params.Nx, Ny = req->params.isPlanar ? 1 : req->params.Ny, Nz = req->params.Nz;
  r->cells = Nx * Ny * Nz;
  // DFT accumulators: nfreq x 4 components x plane x (re, im)
  const double plane = req->dft_axis == 0 ? Ny * Nz : (req->dft_axis == 1 ? Nx * Nz : Nx * Ny);
  r->bytes = (double)bytes + 64.0 * req->nfreq * plane;
  for (int c = 0; c < 3; c++) r->bytes += 8.0 * r->material[c].size();  // transfer staging
  std::lock_guard<std::mutex> lk(srv->mu);
  r->id = srv->next_id++;
  r->t_submit = srv->now();
  srv->reqs[r->id] = r;
  srv->queue.push_back(r);
  srv->stats.submitted += 1;
  srv->stats.queued += 1;
  *id = r->id;
  srv->work_cv.notify_all();
  return LX_OK;
}

extern "C" LX_API lx_status lx_server_poll(lx_server* srv, long long id, int* state) {
  if (!srv || !state) return sfail(LX_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  auto r = find(srv, id);
  if (!r) return sfail(LX_ERR_INVALID, "no such request");
  *state = r->state;
  return LX_OK;
}

extern "C" LX_API lx_status lx_server_wait(lx_server* srv, long long id, double timeout_s, int* state) {
  if (!srv) return sfail(LX_ERR_INVALID, "null argument");
  std::unique_lock<std::mutex> lk(srv->mu);
  auto r = find(srv, id);
  if (!r) return sfail(LX_ERR_INVALID, "no such request");
  auto pred = [&] { return final_state(r->state); };
  if (timeout_s < 0) srv->done_cv.wait(lk, pred);
  else srv->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
  if (state) *state = r->state;
  return LX_OK;
}

extern "C" LX_API lx_status lx_server_cancel(lx_server* srv, long long id) {
  if (!srv) return sfail(LX_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  auto r = find(srv, id);
  if (!r) return sfail(LX_ERR_INVALID, "no such request");
  if (final_state(r->state)) return LX_OK;
  r->cancel = true;
  if (r->state == LX_REQ_QUEUED) {
    auto it = std::find(srv->queue.begin(), srv->queue.end(), r);
    if (it != srv->queue.end()) {
      srv->queue.erase(it);
      set_state(srv, *r, LX_REQ_CANCELLED);
    }
  }
  return LX_OK;
}

static lx_status done_request(lx_server* srv, long long id, std::shared_ptr<Request>& r) {
  r = find(srv, id);
  if (!r) return sfail(LX_ERR_INVALID, "no such request");
  if (r->state != LX_REQ_DONE || !r->sim) return sfail(LX_ERR_STATE, "request has not finished");
  return LX_OK;
}

// Runs `read` on a finished request's handle without holding the server lock (the call may
// wait on the GPU); take/release refuse the request meanwhile.
template <class F>
static lx_status read_done(lx_server* srv, long long id, F read) {
  std::shared_ptr<Request> r;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    lx_status st = done_request(srv, id, r);
    if (st) return st;
    r->readers++;
  }
  const lx_status st = read(*r);
  std::lock_guard<std::mutex> lk(srv->mu);
  r->readers--;
  return st;
}

extern "C" LX_API lx_status lx_server_flux(lx_server* srv, long long id, double* flux, int nfreq) {
  if (!srv || !flux) return sfail(LX_ERR_INVALID, "null argument");
  return read_done(srv, id, [&](Request& r) {
    if (r.dft_id < 0) return sfail(LX_ERR_STATE, "request has no DFT plane");
    return lx_sim_dft_flux(r.sim, r.dft_id, flux, nfreq);
  });
}

extern "C" LX_API lx_status lx_server_max_e2(lx_server* srv, long long id, double* out) {
  if (!srv || !out) return sfail(LX_ERR_INVALID, "null argument");
  return read_done(srv, id, [&](Request& r) { return lx_sim_max_e2(r.sim, out); });
}

extern "C" LX_API lx_status lx_server_times(lx_server* srv, long long id, double t[3]) {
  if (!srv || !t) return sfail(LX_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  auto r = find(srv, id);
  if (!r) return sfail(LX_ERR_INVALID, "no such request");
  t[0] = r->t_submit;
  t[1] = r->t_start;
  t[2] = r->t_end;
  return LX_OK;
}

extern "C" LX_API lx_status lx_server_take(lx_server* srv, long long id, lx_sim** sim) {
  if (!srv || !sim) return sfail(LX_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  std::shared_ptr<Request> r;
  lx_status st = done_request(srv, id, r);
  if (st) return st;
  if (r->readers) return sfail(LX_ERR_STATE, "request is being read by another call");
  *sim = r->sim;
  r->sim = nullptr;
  srv->reqs.erase(id);
  return LX_OK;
}

extern "C" LX_API lx_status lx_server_release(lx_server* srv, long long id) {
  if (!srv) return sfail(LX_ERR_INVALID, "null argument");
  lx_sim* s = nullptr;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto r = find(srv, id);
    if (!r) return sfail(LX_ERR_INVALID, "no such request");
    if (!final_state(r->state)) return sfail(LX_ERR_STATE, "request is still queued or running");
    if (r->readers) return sfail(LX_ERR_STATE, "request is being read by another call");
    s = r->sim;
    r->sim = nullptr;
    srv->reqs.erase(id);
  }
  if (s) lx_sim_destroy(s);
  return LX_OK;
}

extern "C" LX_API const char* lx_server_error(lx_server* srv, long long id) {
  if (!srv) return "";
  std::lock_guard<std::mutex> lk(srv->mu);
  auto r = find(srv, id);
  return r ? r->err.c_str() : "";
}

extern "C" LX_API lx_status lx_server_stats_get(lx_server* srv, lx_server_stats* st) {
  if (!srv || !st) return sfail(LX_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  *st = srv->stats;
  return LX_OK;
}

extern "C" LX_API lx_status lx_server_tune_table(lx_server* srv, lx_tune_entry* e, int cap, int* n) {
  if (!srv || !n || cap < 0 || (cap > 0 && !e)) return sfail(LX_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lk(srv->mu);
  for (int q = 0; q < cap && q < (int)srv->table.size(); q++) e[q] = srv->table[q];
  *n = (int)srv->table.size();
  return LX_OK;
}
