// gf_tune.cpp -- picks the projectors' tile shapes for a context by timing.
//
// Forward projector: R (planes per thread run; odd, so a warp's shared loads
// fall in distinct banks) and the number of ray steps staged per shared-memory
// chunk.  Back projector: warps (image columns) per block.  Each candidate
// runs once to warm up and three times under CUDA events on subset 0 of the
// context's geometry with a unit-cylinder image; the fastest is kept.
#include <vector>

#include "gf_internal.h"

using namespace gf;

namespace {

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  Timer() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~Timer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

gf_status upload_runs(gf_ctx* c, const FpSchedule& f) {
  std::vector<int4> runs(f.runs.size());
  for (size_t i = 0; i < runs.size(); i++) runs[i] = make_int4(f.runs[i].seg, f.runs[i].p0, f.runs[i].n, f.runs[i].pad);
  GF_CK(cudaMemcpyAsync(c->d_runs, runs.data(), runs.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream));
  GF_CK(cudaStreamSynchronize(c->stream));
  return GF_OK;
}

}  // namespace

extern "C" gf_status gf_set_tile_shapes(gf_ctx* c, int32_t fp_run, int32_t fp_chunk, int32_t bp_warps) {
  if (!c) return set_error(GF_ERR_ARG, "null context");
  if (bp_warps != 4 && bp_warps != 8) return set_error(GF_ERR_ARG, "back-projector warps per block must be 4 or 8");
  if (fp_run != 9 && fp_run != 17 && fp_run != 25 && fp_run != 33)
    return set_error(GF_ERR_ARG, "forward-projector run length must be 9, 17, 25 or 33");
  FpSchedule f;
  if (!make_fp_schedule(c->plan, fp_run, fp_chunk, &f))
    return set_error(GF_ERR_GEOMETRY, "no forward-projector schedule with these shapes fits this geometry");
  GF_CK(cudaSetDevice(c->device));
  GF_TRY(upload_runs(c, f));
  c->fps = std::move(f);
  c->bp_warps = bp_warps;
  c->gen++;  // graphs captured with the old shapes are stale
  return GF_OK;
}

extern "C" gf_status gf_tune(gf_ctx* c, int32_t* fp_run, int32_t* fp_chunk, int32_t* bp_warps) {
  if (!c) return set_error(GF_ERR_ARG, "null context");
  GF_CK(cudaSetDevice(c->device));
  GF_TRY(c->ensure_scratch());
  const Plan& p = c->plan;
  const size_t nsub0 = (size_t)p.sub_nang[0] * p.g.nrad * p.PS;
  float2* dbg = nullptr;
  float* cal = nullptr;
  GF_CK(cudaMallocAsync(&dbg, nsub0 * sizeof(float2), c->stream));
  if (cudaMallocAsync(&cal, nsub0 * sizeof(float), c->stream) != cudaSuccess) {
    cudaFreeAsync(dbg, c->stream);
    return cuda_error(cudaGetLastError(), "cudaMallocAsync (tune)");
  }
  auto done = [&](gf_status s) {
    cudaFreeAsync(dbg, c->stream);
    cudaFreeAsync(cal, c->stream);
    cudaStreamSynchronize(c->stream);
    return s;
  };
  cudaStream_t st = c->stream;
  cudaError_t e = cudaMemsetAsync(dbg, 0, nsub0 * sizeof(float2), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(cal, 0, nsub0 * sizeof(float), st);
  if (e == cudaSuccess) e = launch_cylinder(c->dg, 1.0f, c->s_img, st);
  if (e != cudaSuccess) return done(cuda_error(e, "tune set-up"));
  Timer tm;
  auto time_it = [&](auto&& launch, float* ms) -> gf_status {
    cudaError_t x = launch();
    if (x != cudaSuccess) return cuda_error(x, "tune launch");
    cudaEventRecord(tm.a, st);
    for (int k = 0; k < 3; k++)
      if ((x = launch()) != cudaSuccess) return cuda_error(x, "tune launch");
    cudaEventRecord(tm.b, st);
    if ((x = cudaEventSynchronize(tm.b)) != cudaSuccess) return cuda_error(x, "tune sync");
    cudaEventElapsedTime(ms, tm.a, tm.b);
    *ms /= 3.f;
    return GF_OK;
  };
  // forward projector
  FpSchedule best = c->fps;
  float best_ms = 3.0e38f;
  for (int R : {9, 17, 25, 33}) {
    for (int lc : {16, 32, 64}) {
      FpSchedule f;
      if (!make_fp_schedule(p, R, lc, &f)) continue;
      gf_status s = upload_runs(c, f);
      if (s != GF_OK) return done(s);
      FpArgs a = c->fp_args(0, c->s_img);
      a.nruns = (int)f.runs.size();
      a.padl = f.padl;
      a.cw = f.cw;
      a.lc = f.lc;
      a.fr[0].dbg = dbg;
      a.fr[0].cal = cal;
      a.fr[0].corrcal = c->s_cc;
      float ms = 0.f;
      s = time_it([&] { return launch_fp(a, f, st); }, &ms);
      if (s != GF_OK) return done(s);
      c->launches += 4;
      if (ms < best_ms) {
        best_ms = ms;
        best = f;
      }
    }
  }
  c->fps = best;
  gf_status s = upload_runs(c, best);
  if (s != GF_OK) return done(s);
  // back projector
  int best_w = c->bp_warps;
  float best_bp = 3.0e38f;
  for (int w : {4, 8}) {
    BpArgs b = c->bp_args(0, c->s_cc, c->s_numer, c->s_denom, 0);
    float ms = 0.f;
    s = time_it([&] { return launch_bp(b, w, st); }, &ms);
    if (s != GF_OK) return done(s);
    c->launches += 4;
    if (ms < best_bp) {
      best_bp = ms;
      best_w = w;
    }
  }
  c->bp_warps = best_w;
  c->gen++;  // graphs captured with the old shapes are stale
  if (fp_run) *fp_run = c->fps.R;
  if (fp_chunk) *fp_chunk = c->fps.lc;
  if (bp_warps) *bp_warps = c->bp_warps;
  return done(GF_OK);
}
