// gf_batch.cpp -- frames that advance together, replayed from a CUDA graph.
//
// Each frame is a loaded gf_recon with its own resident data, subset count
// and stream.  The frames are split into units: with fusing on
// (gf_batch_set_fused), mode-1 frames that share geometry, storage, filters
// and tile shapes form fused groups of up to kMaxFrames, whatever their
// subset counts, whose sub-iterations run every stage as one launch over the
// frames that have that subset (fused_subiteration); every other frame is a
// unit of its own.  Frames of a group with the same subset count and equal
// normalization masks (the frames of one scanner and normalization)
// back-project two per warp, sharing the per-view geometry and the mask rows.
//
// One iteration of every unit is captured once: a fork event on the batch's
// origin stream, each unit's kernels on the stream of its first frame (a
// parallel branch of the graph, so units overlap on the device), a join event
// per unit back to the origin.  The graph is then launched once per
// iteration.  Replay is exact because a sub-iteration's launches depend only
// on the frames' (type, subset) cursors, which return to the start after a
// full iteration, and every buffer is updated in place.  The graph holds the
// launch parameters as captured (tile shapes, the mode-3 event count and
// buffers, the grouping); a frame whose context was retuned or whose load
// changed them since (gf_ctx::gen, gf_recon::gen), or a change of fusing,
// makes the next iterate capture the graph again.
#include <algorithm>
#include <utility>
#include <vector>

#include "gf_internal.h"

using namespace gf;

struct gf_batch {
  std::vector<gf_recon*> frames;
  int device = 0;
  int fused = 0;  // gf_batch_set_fused: 0 off, 1 groups (paired back projection where masks match), 2 groups
  std::vector<std::vector<int>> units;  // frame indices: a fused group, or one frame
  // per unit and member: its pairing class (the first member with the same
  // subset count and an equal normalization mask), or -1 (back-projected alone)
  std::vector<std::vector<int>> cls;
  int* d_flag = nullptr;                // device flag of the mask comparison
  cudaStream_t origin = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> joins;  // one per frame (a unit uses its first frame's)
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

// Units in frame order: with fusing, each frame joins the first open group
// it can fuse with (fewer than kMaxFrames members), else opens a new one.
static void make_units(gf_batch* b) {
  b->units.clear();
  for (int i = 0; i < (int)b->frames.size(); i++) {
    bool placed = false;
    if (b->fused && b->frames[i]->p.mode == 1) {
      for (auto& u : b->units) {
        if ((int)u.size() < kMaxFrames && fusable(b->frames[u[0]], b->frames[i])) {
          u.push_back(i);
          placed = true;
          break;
        }
      }
    }
    if (!placed) b->units.push_back({i});
  }
}

// Which frames of a fused group may back-project two per warp: those with
// the same subset count whose static normalization masks (every subset, in
// that count's layout) are equal bit for bit, compared on the device after
// the frames' queued work (their loads) has finished.
static gf_status check_masks(gf_batch* b) {
  b->cls.assign(b->units.size(), {});
  for (size_t k = 0; k < b->units.size(); k++) {
    const auto& u = b->units[k];
    b->cls[k].assign(u.size(), -1);
    if (b->fused != 1 || u.size() < 2) continue;
    if (b->frames[u[0]]->ctx->bp_form != GF_BP_PER_VIEW) continue;
    for (size_t j = 0; j < u.size(); j++) {
      const gf_recon* r = b->frames[u[j]];
      b->cls[k][j] = (int)j;  // a class of its own unless an earlier leader matches
      for (size_t i = 0; i < j; i++) {
        if (b->cls[k][i] != (int)i) continue;  // not a class leader
        const gf_recon* l = b->frames[u[i]];
        if (l->ctx->plan.nsub != r->ctx->plan.nsub) continue;
        bool same = l->cal == r->cal;
        if (!same) {
          GF_CK(cudaStreamSynchronize(l->ctx->stream));
          GF_CK(cudaStreamSynchronize(r->ctx->stream));
          GF_CK(launch_differs(l->cal, r->cal, (size_t)l->ctx->plan.all_elems(), b->d_flag, b->origin));
          int flag = 1;
          GF_CK(cudaMemcpyAsync(&flag, b->d_flag, sizeof(int), cudaMemcpyDeviceToHost, b->origin));
          GF_CK(cudaStreamSynchronize(b->origin));
          same = flag == 0;
        }
        if (same) {
          b->cls[k][j] = (int)i;
          break;
        }
      }
    }
  }
  return GF_OK;
}

// One iteration of one unit on its first frame's stream.  A fused group's
// frames may differ in subset count: step s runs the frames that have a
// subset s, each at its own subset s, so every frame visits its subsets in
// order as it would alone.
static gf_status unit_iteration(gf_batch* b, size_t k) {
  const std::vector<int>& u = b->units[k];
  if (u.size() == 1) return gf_recon_iterate(b->frames[u[0]], 1);
  // the group's work stays on its first member's stream in every step
  cudaStream_t st = b->frames[u[0]]->ctx->stream;
  int smax = 0;
  for (int i : u) smax = std::max(smax, b->frames[i]->ctx->plan.nsub);
  for (int s = 0; s < smax; s++) {
    std::vector<gf_recon*> G;
    std::vector<int> C;
    for (size_t j = 0; j < u.size(); j++) {
      gf_recon* r = b->frames[u[j]];
      if (r->ctx->plan.nsub <= s) continue;
      G.push_back(r);
      C.push_back(b->cls[k][j]);
    }
    GF_TRY(fused_subiteration(G.data(), (int)G.size(), C.data(), st));
  }
  return GF_OK;
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
    for (int j = 0; j < i; j++)
      if (frames[j] == frames[i]) return set_error(GF_ERR_ARG, "a frame appears twice");
  }
  gf_batch* b = new gf_batch();
  b->frames.assign(frames, frames + n);
  b->device = frames[0]->ctx->device;
  make_units(b);
  cudaSetDevice(b->device);
  cudaError_t e = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  b->joins.assign(n, nullptr);
  for (int i = 0; i < n && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&b->joins[i], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_flag, sizeof(int));
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
  if (b->d_flag) cudaFree(b->d_flag);
  delete b;
}

gf_status gf_batch_set_fused(gf_batch* b, int32_t fused) {
  if (!b) return set_error(GF_ERR_ARG, "null batch");
  if (fused < 0 || fused > 2) return set_error(GF_ERR_ARG, "fused must be 0, 1 or 2");
  if (fused == b->fused) return GF_OK;
  GF_CK(cudaSetDevice(b->device));
  GF_CK(cudaStreamSynchronize(b->origin));  // a queued replay may still use the graph
  drop_graph(b);
  b->fused = fused;
  make_units(b);
  return GF_OK;
}

gf_status gf_batch_groups(gf_batch* b, int32_t* ngroups, int32_t* largest, int32_t* paired) {
  if (!b) return set_error(GF_ERR_ARG, "null batch");
  GF_CK(cudaSetDevice(b->device));
  GF_TRY(check_masks(b));
  int n = 0, big = 0, pairs = 0;
  for (size_t k = 0; k < b->units.size(); k++) {
    n++;
    big = std::max(big, (int)b->units[k].size());
    // pairs of the first step, where every member takes part
    const std::vector<int>& c = b->cls[k];
    for (size_t j = 0; j < c.size(); j++)
      if (c[j] == (int)j) pairs += (int)std::count(c.begin(), c.end(), (int)j) / 2;
  }
  if (ngroups) *ngroups = n;
  if (largest) *largest = big;
  if (paired) *paired = pairs;
  return GF_OK;
}

}  // extern "C"

static gf_status capture(gf_batch* b) {
  for (gf_recon* r : b->frames)
    if (r->cur_type != 0 || r->cur_sub != 0) return set_error(GF_ERR_STATE, "frames must stand at an iteration boundary");
  // fusing may have been switched on before the frames matched (a retune):
  // group them as they stand now
  make_units(b);
  // the frames' streams must be idle before they join the capture
  for (gf_recon* r : b->frames) GF_CK(cudaStreamSynchronize(r->ctx->stream));
  GF_TRY(check_masks(b));
  std::vector<bool> prof(b->frames.size());
  std::vector<gf_ctx*> ctxs;  // each context once: frames may share one
  std::vector<int64_t> l0;
  for (size_t i = 0; i < b->frames.size(); i++) {
    prof[i] = b->frames[i]->prof;
    b->frames[i]->prof = false;  // no timing events inside the graph
    b->frames[i]->marking = false;
    gf_ctx* c = b->frames[i]->ctx;
    if (std::find(ctxs.begin(), ctxs.end(), c) == ctxs.end()) {
      ctxs.push_back(c);
      l0.push_back(c->launches);
    }
  }
  GF_CK(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed));
  gf_status st = GF_OK;
  cudaError_t e = cudaEventRecord(b->fork, b->origin);
  for (size_t k = 0; k < b->units.size() && e == cudaSuccess && st == GF_OK; k++) {
    const int first = b->units[k][0];
    cudaStream_t s = b->frames[first]->ctx->stream;
    e = cudaStreamWaitEvent(s, b->fork, 0);
    if (e != cudaSuccess) break;
    st = unit_iteration(b, k);
    if (st == GF_OK) e = cudaEventRecord(b->joins[first], s);
    if (e == cudaSuccess && st == GF_OK) e = cudaStreamWaitEvent(b->origin, b->joins[first], 0);
  }
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(b->origin, &g);
  // a replay counts each context's captured launches once, through the
  // first of its frames
  for (size_t i = 0; i < b->frames.size(); i++) {
    b->frames[i]->prof = prof[i];
    b->frames[i]->marking = true;
    b->frames[i]->launches_per_iteration = 0;
  }
  for (size_t k = 0; k < ctxs.size(); k++) {
    for (gf_recon* r : b->frames) {
      if (r->ctx == ctxs[k]) {
        r->launches_per_iteration = ctxs[k]->launches - l0[k];
        break;
      }
    }
    ctxs[k]->launches = l0[k];  // captured, not yet run
  }
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

extern "C" {

gf_status gf_batch_iterate(gf_batch* b, int32_t n, int32_t use_graph) {
  if (!b || n < 0) return set_error(GF_ERR_ARG, "bad argument");
  GF_CK(cudaSetDevice(b->device));
  if (!use_graph) {
    make_units(b);
    GF_TRY(check_masks(b));
    for (int it = 0; it < n; it++) {
      for (size_t ku = 0; ku < b->units.size(); ku++) {
        const std::vector<int>& u = b->units[ku];
        // a fused group runs on its first frame's stream: it waits for the
        // other frames' queued work, and their later work waits for it
        cudaStream_t s0 = b->frames[u[0]]->ctx->stream;
        for (size_t k = 1; k < u.size(); k++) {
          GF_CK(cudaEventRecord(b->joins[u[k]], b->frames[u[k]]->ctx->stream));
          GF_CK(cudaStreamWaitEvent(s0, b->joins[u[k]], 0));
        }
        GF_TRY(unit_iteration(b, ku));
        if (u.size() > 1) {
          GF_CK(cudaEventRecord(b->joins[u[0]], s0));
          b->frames[u[0]]->mark();
          for (size_t k = 1; k < u.size(); k++) {
            GF_CK(cudaStreamWaitEvent(b->frames[u[k]]->ctx->stream, b->joins[u[0]], 0));
            b->frames[u[k]]->mark();  // the group's work, seen from this frame's stream
          }
        }
      }
    }
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
    b->frames[i]->mark();
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
