// gf_batch.cpp -- frames that advance together, replayed from a CUDA graph.
//
// Each frame is a loaded gf_recon with its own resident data, subset count
// and stream.  One iteration of every frame is captured once: a fork event on
// the batch's origin stream, each frame's sub-iteration kernels on its own
// stream (a parallel branch of the graph, so frames overlap on the device),
// a join event per frame back to the origin.  The graph is then launched once
// per iteration.  Replay is exact because a sub-iteration's launches depend
// only on the frame's (type, subset) cursor, which returns to the start
// after a full iteration, and every buffer is updated in place.  The graph
// holds each frame's launch parameters as captured (tile shapes, the mode-3
// event count and buffers); a frame whose context was retuned or whose load
// changed them since (gf_ctx::gen, gf_recon::gen) makes the next iterate
// capture the graph again.
#include <utility>
#include <vector>

#include "gf_internal.h"

using namespace gf;

struct gf_batch {
  std::vector<gf_recon*> frames;
  int device = 0;
  cudaStream_t origin = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  std::vector<std::pair<int64_t, int64_t>> cap_gen;  // (context, reconstruction) generations at capture
};

static bool stale(const gf_batch* b) {
  for (size_t i = 0; i < b->frames.size(); i++) {
    const gf_recon* r = b->frames[i];
    if (b->cap_gen[i] != std::make_pair(r->ctx->gen, r->gen)) return true;
  }
  return false;
}

static void drop_graph(gf_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

extern "C" {

gf_status gf_batch_create(int32_t n, gf_recon* const* frames, gf_batch** out) {
  if (!out || n <= 0 || !frames) return set_error(GF_ERR_ARG, "bad argument");
  *out = nullptr;
  for (int i = 0; i < n; i++) {
    if (!frames[i]) return set_error(GF_ERR_ARG, "null frame");
    if (!frames[i]->loaded) return set_error(GF_ERR_STATE, "every frame must be loaded");
    if (frames[i]->ntypes == 0) return set_error(GF_ERR_STATE, "mode-0 frames have no iterations");
    if (frames[i]->ctx->device != frames[0]->ctx->device) return set_error(GF_ERR_ARG, "frames on different devices");
  }
  gf_batch* b = new gf_batch();
  b->frames.assign(frames, frames + n);
  b->device = frames[0]->ctx->device;
  cudaSetDevice(b->device);
  cudaError_t e = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  b->joins.assign(n, nullptr);
  for (int i = 0; i < n && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&b->joins[i], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    gf_batch_destroy(b);
    return cuda_error(e, "batch set-up");
  }
  *out = b;
  return GF_OK;
}

void gf_batch_destroy(gf_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->origin) cudaStreamSynchronize(b->origin);
  drop_graph(b);
  for (auto ev : b->joins)
    if (ev) cudaEventDestroy(ev);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->origin) cudaStreamDestroy(b->origin);
  delete b;
}

static gf_status capture(gf_batch* b) {
  for (gf_recon* r : b->frames)
    if (r->cur_type != 0 || r->cur_sub != 0) return set_error(GF_ERR_STATE, "frames must stand at an iteration boundary");
  // the frames' streams must be idle before they join the capture
  for (gf_recon* r : b->frames) GF_CK(cudaStreamSynchronize(r->ctx->stream));
  std::vector<bool> prof(b->frames.size());
  for (size_t i = 0; i < b->frames.size(); i++) {
    prof[i] = b->frames[i]->prof;
    b->frames[i]->prof = false;  // no timing events inside the graph
  }
  GF_CK(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed));
  gf_status st = GF_OK;
  cudaError_t e = cudaEventRecord(b->fork, b->origin);
  for (size_t i = 0; i < b->frames.size() && e == cudaSuccess && st == GF_OK; i++) {
    gf_recon* r = b->frames[i];
    e = cudaStreamWaitEvent(r->ctx->stream, b->fork, 0);
    if (e != cudaSuccess) break;
    const int per = r->ntypes * r->ctx->plan.nsub;
    const int64_t l0 = r->ctx->launches;
    for (int k = 0; k < per && st == GF_OK; k++) st = gf_recon_subiteration(r);
    r->launches_per_iteration = r->ctx->launches - l0;
    r->ctx->launches = l0;  // captured, not yet run
    if (st == GF_OK) e = cudaEventRecord(b->joins[i], r->ctx->stream);
    if (e == cudaSuccess && st == GF_OK) e = cudaStreamWaitEvent(b->origin, b->joins[i], 0);
  }
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(b->origin, &g);
  for (size_t i = 0; i < b->frames.size(); i++) b->frames[i]->prof = prof[i];
  if (st != GF_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_error(e, "capture");
  }
  if (e2 != cudaSuccess) return cuda_error(e2, "cudaStreamEndCapture");
  b->graph = g;
  GF_CK(cudaGraphInstantiate(&b->exec, g, 0));
  b->cap_gen.clear();
  for (gf_recon* r : b->frames) b->cap_gen.emplace_back(r->ctx->gen, r->gen);
  // capturing advanced every frame's host cursor by one iteration, but the
  // captured work has not run: the first replay below is that iteration
  for (gf_recon* r : b->frames) {
    r->iters_done -= 1;
    r->subs_done -= (int64_t)r->ntypes * r->ctx->plan.nsub;
  }
  return GF_OK;
}

gf_status gf_batch_iterate(gf_batch* b, int32_t n, int32_t use_graph) {
  if (!b || n < 0) return set_error(GF_ERR_ARG, "bad argument");
  GF_CK(cudaSetDevice(b->device));
  if (!use_graph) {
    for (int it = 0; it < n; it++)
      for (gf_recon* r : b->frames) GF_TRY(gf_recon_iterate(r, 1));
    return GF_OK;
  }
  if (b->exec && stale(b)) {
    // a replay still queued on the origin stream may use the old graph
    GF_CK(cudaStreamSynchronize(b->origin));
    drop_graph(b);
  }
  if (!b->exec) GF_TRY(capture(b));
  // the frames' own streams may hold work queued outside the graph
  for (gf_recon* r : b->frames) {
    GF_CK(cudaEventRecord(b->fork, r->ctx->stream));
    GF_CK(cudaStreamWaitEvent(b->origin, b->fork, 0));
  }
  for (int it = 0; it < n; it++) {
    GF_CK(cudaGraphLaunch(b->exec, b->origin));
    for (gf_recon* r : b->frames) {
      r->iters_done += 1;
      r->subs_done += (int64_t)r->ntypes * r->ctx->plan.nsub;
      r->ctx->launches += r->launches_per_iteration;
    }
  }
  // later work on a frame's own stream runs after the replays
  for (size_t i = 0; i < b->frames.size(); i++) {
    GF_CK(cudaEventRecord(b->joins[i], b->origin));
    GF_CK(cudaStreamWaitEvent(b->frames[i]->ctx->stream, b->joins[i], 0));
  }
  return GF_OK;
}

gf_status gf_batch_synchronize(gf_batch* b) {
  if (!b) return set_error(GF_ERR_ARG, "null batch");
  GF_CK(cudaStreamSynchronize(b->origin));
  for (gf_recon* r : b->frames) GF_CK(cudaStreamSynchronize(r->ctx->stream));
  return GF_OK;
}

}  // extern "C"
