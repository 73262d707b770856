// gf_server.cpp -- a request loop with HBM-budget admission and continuous
// batching on one device.
//
// Requests (reconstructions and bare projections, of any geometry) wait in
// arrival order.  A loader thread admits the head of the queue when its
// device bytes (gf_recon_bytes) fit the remaining budget and fewer than
// max_active requests run, builds its context (own stream) and
// reconstruction, and loads its data; a projection is answered right there.
// A worker thread keeps one iteration in flight for every loaded
// reconstruction: when its completion event fires the next iteration is
// queued, so requests of different sizes advance independently, their
// kernels overlap on the device, and loading a new request does not stall
// the running ones.  A finished request's image is read back, its memory
// returned (stream-ordered, to the device's pool), and the loader
// re-examines the queue.  Results do not depend on what else runs: each
// request owns its buffers and the kernels are deterministic.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gf_internal.h"

using namespace gf;

namespace {

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Latencies of completed requests in logarithmic bins 1 % wide (1 us to
// about 3 h), so a server that runs for days holds a fixed 2 K counters and
// reads its percentiles in constant time.  A percentile is reported as the
// geometric centre of its bin, clamped to the smallest and largest latency
// seen: within 0.5 % of the exact order statistic.
struct LatencyHist {
  static constexpr double kLo = 1e-3;  // ms
  static constexpr double kStep = 1.01;
  static constexpr int kBins = 2048;
  std::vector<int64_t> bins = std::vector<int64_t>(kBins, 0);
  int64_t n = 0;
  double sum = 0, lo = 0, hi = 0;
  static int bin_of(double ms) {
    if (!(ms > kLo)) return 0;
    const double k = std::log(ms / kLo) / std::log(kStep);
    return std::min(kBins - 1, 1 + (int)k);
  }
  void add(double ms) {
    bins[bin_of(ms)]++;
    lo = n ? std::min(lo, ms) : ms;
    hi = n ? std::max(hi, ms) : ms;
    n++;
    sum += ms;
  }
  // smallest bin whose cumulative count reaches the rank of fraction f
  double quantile(double f) const {
    const int64_t rank = std::min<int64_t>(n - 1, (int64_t)(f * (double)(n - 1) + 0.5));
    int64_t c = 0;
    for (int k = 0; k < kBins; k++) {
      c += bins[k];
      if (c > rank) {
        const double mid = k == 0 ? kLo : kLo * std::pow(kStep, (double)k - 0.5);
        return std::min(hi, std::max(lo, mid));
      }
    }
    return hi;
  }
};

struct Job {
  int64_t id = 0;
  gf_request req{};
  int64_t bytes = 0;
  double t_submit = 0, t_admit = 0, t_loaded = 0, t_done = 0;
  gf_ctx* ctx = nullptr;
  gf_recon* rec = nullptr;
  cudaEvent_t ev = nullptr;
  bool in_flight = false;
  int iters = 0;
  int state = 0;  // 0 queued, 1 active, 2 done
  bool claimed = false;  // a gf_server_wait is waiting for it
  gf_status status = GF_OK;
  std::string err;
};

}  // namespace

struct gf_server {
  int device = 0;
  int64_t budget = 0;
  int max_active = 1;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job*> queue;
  std::vector<Job*> active;  // loaded reconstructions
  int loading = 0;           // admitted, being set up
  std::unordered_map<int64_t, Job*> jobs;
  int64_t next_id = 1, bytes_in_use = 0, peak_bytes = 0, submitted = 0, completed = 0, failed = 0;
  int peak_active = 0;
  double t_first = -1;
  LatencyHist lat;  // latencies of completed requests (bounded)
  double sum_queue = 0, sum_load = 0, sum_run = 0, last_done = 0;
  bool stop = false;
  std::thread worker;
  std::vector<std::thread> loaders;

  void run();   // advances loaded reconstructions
  void load();  // admits and sets up queued requests
  void finish(Job* j, gf_status st);
  gf_status start(Job* j);
};

static void release(Job* j) {
  if (j->ev) cudaEventDestroy(j->ev);
  if (j->rec) gf_recon_destroy(j->rec);
  if (j->ctx) gf_destroy(j->ctx);
  j->ev = nullptr;
  j->rec = nullptr;
  j->ctx = nullptr;
}

void gf_server::finish(Job* j, gf_status st) {
  // the failing call's message, before the clean-up calls below run
  const std::string err = st != GF_OK ? std::string(gf_last_error()) : std::string();
  release(j);
  std::lock_guard<std::mutex> lk(mu);
  j->status = st;
  if (st != GF_OK) j->err = err;
  j->t_done = now_ms();
  j->state = 2;
  bytes_in_use -= j->bytes;
  if (st == GF_OK) {
    completed++;
    lat.add(j->t_done - j->t_submit);
    sum_queue += j->t_admit - j->t_submit;
    sum_load += j->t_loaded - j->t_admit;
    sum_run += j->t_done - j->t_loaded;
    last_done = std::max(last_done, j->t_done);
  } else {
    failed++;
  }
  active.erase(std::remove(active.begin(), active.end(), j), active.end());
  cv_done.notify_all();
  cv_work.notify_all();  // memory and a slot came free
}

gf_status gf_server::start(Job* j) {
  const gf_request& q = j->req;
  GF_TRY(gf_create(&q.geometry, q.nsubsets, device, &j->ctx));
  gf_recon_params p;
  gf_recon_defaults(q.kind == GF_REQ_PROJECT ? 0 : 1, &p);
  p.niter = q.niter;
  p.storage = q.storage;
  GF_TRY(gf_recon_create(j->ctx, &p, &j->rec));
  GF_TRY(gf_recon_load(j->rec, q.h_image, q.h_dsino, nullptr, q.h_norm, nullptr, 0));
  GF_CK(cudaEventCreateWithFlags(&j->ev, cudaEventDisableTiming));
  return GF_OK;
}

void gf_server::load() {
  cudaSetDevice(device);
  for (;;) {
    Job* j = nullptr;
    {
      std::unique_lock<std::mutex> lk(mu);
      for (;;) {
        while (!queue.empty() && queue.front()->bytes > budget) {  // can never fit
          Job* x = queue.front();
          queue.pop_front();
          x->state = 2;
          x->status = GF_ERR_NOMEM;
          x->err = "request needs more device memory than the server's budget";
          x->t_done = now_ms();
          failed++;
          cv_done.notify_all();
        }
        // the head waits for memory or a slot; arrival order is kept
        if (!queue.empty() && (int)active.size() + loading < max_active && bytes_in_use + queue.front()->bytes <= budget)
          break;
        if (stop && queue.empty()) {
          cv_work.notify_all();
          return;
        }
        cv_work.wait(lk);
      }
      j = queue.front();
      queue.pop_front();
      bytes_in_use += j->bytes;
      peak_bytes = std::max(peak_bytes, bytes_in_use);
      j->state = 1;
      j->t_admit = now_ms();
      loading++;
      peak_active = std::max(peak_active, (int)active.size() + loading);
    }
    gf_status st = start(j);
    j->t_loaded = now_ms();
    const bool project = j->req.kind == GF_REQ_PROJECT;
    if (st == GF_OK && project) st = gf_recon_get_proj_ref(j->rec, j->req.h_out);
    {
      std::lock_guard<std::mutex> lk(mu);
      loading--;
      if (st == GF_OK && !project) active.push_back(j);
    }
    if (st != GF_OK || project) finish(j, st);
    cv_work.notify_all();
  }
}

void gf_server::run() {
  cudaSetDevice(device);
  for (;;) {
    std::vector<Job*> act;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&] { return !active.empty() || (stop && queue.empty() && loading == 0); });
      if (active.empty()) return;
      act = active;
    }
    // one iteration in flight per loaded reconstruction
    bool progressed = false;
    for (Job* j : act) {
      if (j->in_flight) {
        cudaError_t e = cudaEventQuery(j->ev);
        if (e == cudaErrorNotReady) continue;
        j->in_flight = false;
        progressed = true;
        if (e != cudaSuccess) {
          finish(j, cuda_error(e, "request iteration"));
          continue;
        }
        j->iters++;
      }
      if (j->iters >= j->req.niter) {
        finish(j, gf_recon_get_image(j->rec, 0, 0, j->req.h_out));
        progressed = true;
        continue;
      }
      gf_status st = gf_recon_iterate(j->rec, 1);
      if (st == GF_OK && cudaEventRecord(j->ev, j->ctx->stream) != cudaSuccess) st = cuda_error(cudaGetLastError(), "event");
      if (st != GF_OK) {
        finish(j, st);
        continue;
      }
      j->in_flight = true;
      progressed = true;
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

extern "C" {

gf_status gf_recon_bytes(const gf_geometry* gg, int32_t nsub, const gf_recon_params* p, int64_t nev, int64_t* bytes) {
  if (!gg || !p || !bytes) return set_error(GF_ERR_ARG, "null argument");
  Geom geo{gg->res, gg->nzs, gg->nrad, gg->nang, gg->span, gg->nseg, gg->pitch_mm, gg->diam_det_mm, gg->fov_mm};
  Plan pl;
  std::string err;
  if (!make_plan(geo, nsub, &pl, &err)) return set_error(GF_ERR_GEOMETRY, err);
  const int64_t v = pl.nvoxp * 4, d = pl.ndata * 4, all = pl.all_elems();
  int64_t b = v + d + 64 * 1024;  // image, proj_ref, context tables
  if (p->image_storage != GF_STORE_F32) b -= pl.nvoxp * 2;  // 16-bit doubles image
  if (p->mode == 0) {
    b += pl.nvox * 4;  // staging
  } else {
    b += 3 * v;                                                                   // second image, psf, ratio
    b += (int64_t)pl.amax * pl.g.nrad * pl.PS * (p->storage == GF_STORE_F32 ? 8 : 4);  // ratio sinogram
    b += all * 8 + all * 4;                                                       // data/background, mask
    b += 3 * d;                                                                   // staging
  }
  if (p->mode >= 2) b += all * 8 + v;
  if (p->mode == 3) b += 3 * d + nev * (8 + 16 + 8);  // events, their sorted ends, their shares
  *bytes = b;
  return GF_OK;
}

gf_status gf_server_create(int32_t device, int64_t budget, int32_t max_active, gf_server** out) {
  if (!out || budget <= 0 || max_active < 1) return set_error(GF_ERR_ARG, "bad argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return set_error(GF_ERR_NODEV, "no such CUDA device");
  }
  gf_server* s = new gf_server();
  s->device = device;
  s->budget = budget;
  s->max_active = max_active;
  s->worker = std::thread([s] { s->run(); });
  // one loader: concurrent pageable host->device copies from several threads
  // held up the worker's launches and made every request slower
  s->loaders.emplace_back([s] { s->load(); });
  *out = s;
  return GF_OK;
}

void gf_server_destroy(gf_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& t : s->loaders)
    if (t.joinable()) t.join();
  if (s->worker.joinable()) s->worker.join();
  for (auto& kv : s->jobs) {
    release(kv.second);
    delete kv.second;
  }
  delete s;
}

gf_status gf_server_submit(gf_server* s, const gf_request* q, int64_t* id) {
  if (!s || !q || !id || !q->h_out) return set_error(GF_ERR_ARG, "bad argument");
  if (q->kind == GF_REQ_RECON && (!q->h_dsino || !q->h_norm || q->niter < 0))
    return set_error(GF_ERR_ARG, "a reconstruction needs a sinogram, a normalization and niter >= 0");
  if (q->kind == GF_REQ_PROJECT && !q->h_image) return set_error(GF_ERR_ARG, "a projection needs an image");
  if (q->kind != GF_REQ_RECON && q->kind != GF_REQ_PROJECT) return set_error(GF_ERR_ARG, "unknown request kind");
  gf_recon_params p;
  gf_recon_defaults(q->kind == GF_REQ_PROJECT ? 0 : 1, &p);
  p.storage = q->storage;
  Job* j = new Job();
  j->req = *q;
  gf_status st = gf_recon_bytes(&q->geometry, q->nsubsets, &p, 0, &j->bytes);
  if (st != GF_OK) {
    delete j;
    return st;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    j->id = s->next_id++;
    j->t_submit = now_ms();
    if (s->t_first < 0) s->t_first = j->t_submit;
    s->jobs[j->id] = j;
    s->queue.push_back(j);
    s->submitted++;
    *id = j->id;
  }
  s->cv_work.notify_all();
  return GF_OK;
}

gf_status gf_server_wait(gf_server* s, int64_t id, double* latency_ms) {
  if (!s) return set_error(GF_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) return set_error(GF_ERR_ARG, "unknown request id");
  Job* j = it->second;
  // one waiter per request: the waiter that returns deletes it
  if (j->claimed) return set_error(GF_ERR_ARG, "request is already being waited for");
  j->claimed = true;
  s->cv_done.wait(lk, [&] { return j->state == 2; });
  // the request is finished and nothing else refers to it: forget it here, so
  // a long-running server holds only requests that are queued, running or
  // not yet waited for
  const double lat = j->t_done - j->t_submit;
  const gf_status st = j->status;
  const std::string err = j->err;
  s->jobs.erase(it);
  delete j;
  if (latency_ms) *latency_ms = lat;
  if (st != GF_OK) return set_error(st, err);
  return GF_OK;
}

gf_status gf_server_get_stats(gf_server* s, gf_server_stats* o) {
  if (!s || !o) return set_error(GF_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  *o = gf_server_stats{};
  o->submitted = s->submitted;
  o->completed = s->completed;
  o->failed = s->failed;
  o->queued = (int64_t)s->queue.size();
  o->active = (int64_t)s->active.size() + s->loading;
  o->bytes_in_use = s->bytes_in_use;
  o->peak_bytes = s->peak_bytes;
  o->budget_bytes = s->budget;
  o->peak_active = s->peak_active;
  if (s->lat.n > 0) {
    o->p50_ms = s->lat.quantile(0.50);
    o->p99_ms = s->lat.quantile(0.99);
    o->max_ms = s->lat.hi;
    o->mean_ms = s->lat.sum / (double)s->lat.n;
    o->queue_ms = s->sum_queue / (double)s->completed;
    o->load_ms = s->sum_load / (double)s->completed;
    o->run_ms = s->sum_run / (double)s->completed;
    if (s->last_done > s->t_first)
      o->throughput_per_s = (double)s->completed / ((s->last_done - s->t_first) / 1000.0);
  }
  return GF_OK;
}

}  // extern "C"
