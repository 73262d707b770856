// gf_recon.cpp -- one reconstruction of a CLI mode, resident on the device.
//
// Replaces osem3d() (GFIRST.cu:44-575).  The reference keeps its images on
// the host and crosses to the device once per view; here every array stays
// in HBM for the whole reconstruction and a sub-iteration is a fixed chain
// of kernels on one stream:
//   psf    = XY PSF of the current image                      (GFIRST.cu:324-340)
//   FP     = forward projection + ratio -> (corr, calib)       (GFIRST.cu:346-430)
//            [VLOR triples: FP -> split -> ratio, GFIRST.cu:373-430]
//   BP     = back projection -> NUMER, DENOM                   (GFIRST.cu:436-469)
//   update = ratio, XY PSF, axial filter, multiply, edges      (GFIRST.cu:482-502)
//   [triples, once per iteration: joint bilateral filter + blend, GFIRST.cu:510-526]
// Subset s holds the angles t with t % nsub == s; sub-iterations run
// iteration -> type (doubles, triples) -> subset.  With nsub = 1 this is the
// reference's loop.  The joint filter runs after the triples type's last
// subset, i.e. once per iteration as in the reference.
#include <algorithm>
#include <cstring>

#include "gf_internal.h"

using namespace gf;

gf_status gf_recon::alloc(size_t bytes, void** q) {
  *q = nullptr;
  cudaError_t e = cudaMallocAsync(q, bytes ? bytes : 16, ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_error(e, "cudaMallocAsync (reconstruction)");
  }
  owned.push_back(DevBuf{*q, bytes});
  return GF_OK;
}

void gf_recon::release(void* q) {
  if (!q) return;
  for (size_t i = 0; i < owned.size(); i++) {
    if (owned[i].p == q) {
      cudaFreeAsync(q, ctx->stream);
      owned.erase(owned.begin() + (long)i);
      return;
    }
  }
}

void gf_recon::stage_begin(int stage) {
  if (!prof) return;
  if (ev_used == evs.size()) {
    StageEv e{stage, nullptr, nullptr};
    cudaEventCreate(&e.a);
    cudaEventCreate(&e.b);
    evs.push_back(e);
  }
  evs[ev_used].stage = stage;
  cudaEventRecord(evs[ev_used].a, ctx->stream);
}

void gf_recon::stage_end() {
  if (!prof) return;
  cudaEventRecord(evs[ev_used].b, ctx->stream);
  ev_used++;
}

gf_status gf_recon::project_all(const float* img_zfast, float* proj_full) {
  for (int s = 0; s < ctx->plan.nsub; s++) {
    FpArgs a = ctx->fp_args(s, img_zfast);
    a.fr[0].proj_full = proj_full;
    GF_LAUNCH(ctx, launch_fp(a, ctx->fps, ctx->stream));
  }
  return GF_OK;
}

// STEP 3, initial images (GFIRST.cu:282-288), and the mode-3 triples
// projection that weights the VLOR split (refreshed subset by subset later).
gf_status gf_recon::init_images() {
  gf_ctx* c = ctx;
  cudaStream_t st = c->stream;
  GF_LAUNCH(c, launch_cylinder(c->dg, 1.0f, img[0], st, store(0)));
  GF_LAUNCH(c, launch_cylinder(c->dg, p.mode == 1 ? 0.0f : 1.0f, img[1], st, store(1)));
  if (p.mode == 3) {
    GF_LAUNCH(c, launch_conv_xy(c->dg, img[1], g_fw, psf, st, store(1)));
    GF_TRY(project_all(psf, proj_t));
    GF_CK(cudaMemsetAsync(datos_v, 0, c->plan.ndata * sizeof(float), st));
  }
  iters_done = 0;
  subs_done = 0;
  cur_type = cur_sub = 0;
  return GF_OK;
}

gf_status gf_recon::subiteration(int t, int s) {
  gf_ctx* c = ctx;
  const Plan& pl = c->plan;
  cudaStream_t st = c->stream;
  const int na = pl.sub_nang[s];
  const int64_t off = pl.sub_off[s];
  stage_begin(GF_STAGE_PSF);
  GF_LAUNCH(c, launch_conv_xy(c->dg, img[t], g_fw, psf, st, store(t)));
  stage_end();
  FpArgs a = c->fp_args(s, psf);
  if (p.mode == 3 && t == 1) {
    a.fr[0].proj_full = proj_t;
    stage_begin(GF_STAGE_FP);
    GF_LAUNCH(c, launch_fp(a, c->fps, st));
    stage_end();
    stage_begin(GF_STAGE_VLOR);
    GF_CK(cudaMemsetAsync(datos_v, 0, (size_t)pl.ndata * sizeof(float), st));
    GF_LAUNCH(c, launch_vlor_split_sorted(c->dg, vlor_keys, nev, events, proj_t, blankt, vlor_share, datos_v, st));
    GF_LAUNCH(c, launch_ratio_gather(c->dg, c->d_rowmap, s, na, proj_t, datos_v, dbg[1] + off, cal + off, corrcal,
                                     p.storage, st));
    stage_end();
  } else {
    a.fr[0].dbg = dbg[t] + off;
    a.fr[0].cal = cal + off;
    a.fr[0].corrcal = corrcal;
    a.storage = p.storage;
    stage_begin(GF_STAGE_FP);
    GF_LAUNCH(c, launch_fp(a, c->fps, st));
    stage_end();
  }
  BpArgs b = c->bp_args(s, corrcal, ratio, nullptr, p.storage);
  b.ratio = 1;
  // Triples data are mostly zero, and where a ratio of exactly 0 meets a
  // sentinel row the gap rule (GFIRST_GPU_Kernels.cu:157) turns on whether an
  // interpolation weight rounds to 0: the triples image follows the
  // reference's per-voxel rounding, or it drifts by ~1e-3 from it.
  if (t == 1) b.fast = 0;
  stage_begin(GF_STAGE_BP);
  GF_LAUNCH(c, launch_bp(b, c->bp_warps, st));
  stage_end();
  stage_begin(GF_STAGE_UPDATE);
  GF_LAUNCH(c, launch_update(c->dg, ratio, g_bw, g5, img[t], st, store(t)));
  stage_end();
  if (t == 1 && s == pl.nsub - 1) {
    // GFIRST.cu:512-524: r=4, sigma3D=0.75, sigmaI=0.025, max_ref over the doubles image
    stage_begin(GF_STAGE_BILATERAL);
    GF_LAUNCH(c, launch_max_nonneg(c->dg, img[0], d_max, st, store(0)));
    GF_LAUNCH(c, launch_bilateral(c->dg, img[1], img[0], d_max, 0.f, 4, 0.025f, c->d_gtab, filt, st, store(0)));
    GF_LAUNCH(c, launch_blend(c->dg, img[1], filt, st, store(1)));
    stage_end();
  }
  return GF_OK;
}

void gf_recon::advance() {
  subs_done++;
  if (++cur_sub == ctx->plan.nsub) {
    cur_sub = 0;
    if (++cur_type == ntypes) {
      cur_type = 0;
      iters_done++;
    }
  }
}

namespace gf {

bool fusable(const gf_recon* a, const gf_recon* b) {
  const gf_ctx* x = a->ctx;
  const gf_ctx* y = b->ctx;
  const Geom& g = x->plan.g;
  const Geom& h = y->plan.g;
  const bool same_geom = g.res == h.res && g.nzs == h.nzs && g.nrad == h.nrad && g.nang == h.nang &&
                         g.span == h.span && g.nseg == h.nseg && g.pitch == h.pitch && g.diam == h.diam &&
                         g.fov == h.fov;
  // the subset counts may differ: each frame's launch entry names its subset
  return a->p.mode == 1 && b->p.mode == 1 && a->loaded && b->loaded && x->device == y->device && same_geom &&
         a->p.storage == b->p.storage && a->p.image_storage == b->p.image_storage && a->p.psf_fw == b->p.psf_fw &&
         a->p.psf_bw == b->p.psf_bw && x->bp_form == y->bp_form && x->bp_warps == y->bp_warps &&
         x->fps.R == y->fps.R && x->fps.lc == y->fps.lc;
}

gf_status fused_subiteration(gf_recon* const* G, int nfr, const int* cls, cudaStream_t st) {
  if (nfr < 1 || nfr > kMaxFrames) return set_error(GF_ERR_ARG, "fused group size out of range");
  gf_recon* r0 = G[0];
  gf_ctx* c = r0->ctx;
  const int s = r0->cur_sub;
  for (int k = 1; k < nfr; k++)
    if (G[k]->cur_sub != s || G[k]->cur_type != 0 || !fusable(r0, G[k]))
      return set_error(GF_ERR_STATE, "frames of a fused group must match and stand at the same subset");
  ImgFrames f{};
  for (int k = 0; k < nfr; k++) {
    f.fr[k].in = G[k]->img[0];
    f.fr[k].out = G[k]->psf;
  }
  GF_LAUNCH(c, launch_conv_xy_frames(c->dg, f, nfr, r0->g_fw, st, r0->store(0)));
  // every frame at subset s of its own subset count: its own angles and its
  // own offset into the subset-ordered data
  FpArgs a = c->fp_args(s, nullptr);
  a.nfr = nfr;
  a.storage = r0->p.storage;
  for (int k = 0; k < nfr; k++) {
    const Plan& pk = G[k]->ctx->plan;
    const int64_t off = pk.sub_off[s];
    a.fr[k] = FpFrame{G[k]->psf, G[k]->dbg[0] + off, G[k]->cal + off, G[k]->corrcal, nullptr, s, pk.nsub,
                      pk.sub_nang[s]};
  }
  GF_LAUNCH(c, launch_fp(a, c->fps, st));
  // the back projector keeps the subset a launch constant: one launch per
  // subset count among the frames; within it, frames of one class (same
  // normalization mask) share a warp per column two by two
  std::vector<bool> done(nfr, false);
  for (int k0 = 0; k0 < nfr; k0++) {
    if (done[k0]) continue;
    const Plan& pl = G[k0]->ctx->plan;
    BpArgs b = c->bp_args(s, nullptr, nullptr, nullptr, r0->p.storage);
    b.g.nsub = pl.nsub;
    b.na = pl.sub_nang[s];
    b.ratio = 1;
    std::vector<int> pairs, singles;
    for (int k = k0; k < nfr; k++) {
      if (done[k] || G[k]->ctx->plan.nsub != pl.nsub) continue;
      done[k] = true;
      int j = -1;
      if (b.fast && cls && cls[k] >= 0)
        for (int m = k + 1; m < nfr && j < 0; m++)
          if (!done[m] && cls[m] == cls[k]) j = m;
      if (j >= 0) {
        done[j] = true;
        pairs.push_back(k);
        pairs.push_back(j);
      } else {
        singles.push_back(k);
      }
    }
    if (!pairs.empty()) {
      b.nfr = (int)pairs.size();
      for (size_t i = 0; i < pairs.size(); i++) b.fr[i] = BpFrame{G[pairs[i]]->corrcal, G[pairs[i]]->ratio, nullptr};
      GF_LAUNCH(c, launch_bp_pairs(b, c->bp_warps, st));
    }
    if (!singles.empty()) {
      b.nfr = (int)singles.size();
      for (size_t i = 0; i < singles.size(); i++)
        b.fr[i] = BpFrame{G[singles[i]]->corrcal, G[singles[i]]->ratio, nullptr};
      GF_LAUNCH(c, launch_bp(b, c->bp_warps, st));
    }
  }
  ImgFrames u{};
  for (int k = 0; k < nfr; k++) u.fr[k] = ImgFrame{G[k]->ratio, nullptr, G[k]->img[0]};
  GF_LAUNCH(c, launch_update_frames(c->dg, u, nfr, r0->g_bw, r0->g5, st, r0->store(0)));
  for (int k = 0; k < nfr; k++) G[k]->advance();
  return GF_OK;
}

}  // namespace gf

extern "C" {

gf_status gf_recon_defaults(int32_t mode, gf_recon_params* out) {
  if (!out) return set_error(GF_ERR_ARG, "null output");
  if (mode < 0 || mode > 3) return set_error(GF_ERR_ARG, "mode must be 0..3");
  // GFIRST.h:21-30
  out->mode = mode;
  out->niter = 60;
  out->psf_fw = 1.5f;
  out->psf_bw = 1.5f;
  out->scale_d = (float)(3.70e-4 * 162.0);
  out->scale_t = (float)(3.70e-4 * 162.0);
  out->storage = GF_STORE_F32;
  out->image_storage = GF_STORE_F32;
  return GF_OK;
}

gf_status gf_recon_create(gf_ctx* c, const gf_recon_params* prm, gf_recon** out) {
  if (!c || !prm || !out) return set_error(GF_ERR_ARG, "null argument");
  *out = nullptr;
  if (prm->mode < 0 || prm->mode > 3) return set_error(GF_ERR_ARG, "mode must be 0..3");
  if (prm->niter < 0) return set_error(GF_ERR_ARG, "niter must be >= 0");
  if (prm->storage < GF_STORE_F32 || prm->storage > GF_STORE_BF16) return set_error(GF_ERR_ARG, "unknown storage");
  if (prm->image_storage < GF_STORE_F32 || prm->image_storage > GF_STORE_BF16)
    return set_error(GF_ERR_ARG, "unknown image storage");
  if (prm->image_storage != GF_STORE_F32 && prm->mode == 0)
    return set_error(GF_ERR_ARG, "mode 0 has no reconstructed image");
  GF_CK(cudaSetDevice(c->device));
  gf_recon* r = new gf_recon();
  r->ctx = c;
  c->recons.push_back(r);
  r->p = *prm;
  GF_CK(cudaEventCreateWithFlags(&r->ev_last, cudaEventDisableTiming));
  r->ntypes = prm->mode == 0 ? 0 : (prm->mode == 1 ? 1 : 2);
  const Plan& pl = c->plan;
  auto fail = [&](gf_status st) {
    gf_recon_destroy(r);
    return st;
  };
  gf_status st;
#define ALLOC(ptr, n) \
  if ((st = r->alloc_t((size_t)(n), &(ptr))) != GF_OK) return fail(st)
  // the images: FP32, or 16-bit elements (image_storage; the triples image of
  // modes 2-3 too, mode 1's unused triples image stays FP32)
  if ((st = r->alloc((size_t)pl.nvoxp * (r->store(0) == GF_STORE_F32 ? 4 : 2), (void**)&r->img[0])) != GF_OK)
    return fail(st);
  ALLOC(r->proj_ref, pl.ndata);
  if (prm->mode >= 1) {
    if ((st = r->alloc((size_t)pl.nvoxp * (r->store(1) == GF_STORE_F32 ? 4 : 2), (void**)&r->img[1])) != GF_OK)
      return fail(st);
    ALLOC(r->psf, pl.nvoxp);
    ALLOC(r->ratio, pl.nvoxp);
    if ((st = r->alloc((size_t)pl.amax * pl.g.nrad * pl.PS * (prm->storage == GF_STORE_F32 ? 8 : 4), &r->corrcal)) != GF_OK)
      return fail(st);
    ALLOC(r->dbg[0], pl.all_elems());
    ALLOC(r->cal, pl.all_elems());
  }
  if (prm->mode >= 2) {
    ALLOC(r->dbg[1], pl.all_elems());
    ALLOC(r->filt, pl.nvoxp);
    ALLOC(r->d_max, 1);
    if ((st = c->ensure_gtab(0.75f)) != GF_OK) return fail(st);
  }
  if (prm->mode == 3) {
    ALLOC(r->proj_t, pl.ndata);
    ALLOC(r->blankt, pl.ndata);
    ALLOC(r->datos_v, pl.ndata);
  }
#undef ALLOC
  r->g_fw = gauss9(prm->psf_fw);
  r->g_bw = gauss9(prm->psf_bw);
  r->g5 = gauss5();
  *out = r;
  return GF_OK;
}

void gf_recon_destroy(gf_recon* r) {
  if (!r) return;
  auto& rs = r->ctx->recons;
  rs.erase(std::remove(rs.begin(), rs.end(), r), rs.end());
  for (auto& b : r->owned) cudaFreeAsync(b.p, r->ctx->stream);
  cudaStreamSynchronize(r->ctx->stream);
  for (auto& e : r->evs) {
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  if (r->ev_last) cudaEventDestroy(r->ev_last);
  if (r->ev_staged) cudaEventDestroy(r->ev_staged);
  if (r->ev_stage_free) cudaEventDestroy(r->ev_stage_free);
  delete r;
}

static gf_status load_impl(gf_recon* r, const float* h_image, const float* h_dsino, const float* h_tsino,
                           const float* h_norm, const int32_t* h_events, int64_t nevents, bool wait) {
  if (!r) return set_error(GF_ERR_ARG, "null reconstruction");
  gf_ctx* c = r->ctx;
  const Plan& pl = c->plan;
  cudaStream_t st = c->stream;
  const int mode = r->p.mode;
  if (mode == 0 && !h_image) return set_error(GF_ERR_ARG, "mode 0 needs an image");
  if (mode >= 1 && (!h_dsino || !h_norm)) return set_error(GF_ERR_ARG, "modes 1-3 need a sinogram and a normalization");
  if (mode >= 2 && !h_tsino) return set_error(GF_ERR_ARG, "modes 2-3 need a triples sinogram");
  if (mode == 3 && (nevents < 0 || (nevents > 0 && !h_events))) return set_error(GF_ERR_ARG, "mode 3 needs VLOR events");
  GF_CK(cudaSetDevice(c->device));
  // device staging of the host inputs, kept for later loads
  size_t stage_n = (size_t)2 * pl.ndata + (size_t)pl.ndata;
  if (mode == 0) stage_n = pl.nvox;
  if (!r->stage) GF_TRY(r->alloc_t(stage_n, &r->stage));
  float* stage = r->stage;
  auto done = [&](gf_status s) {
    if (wait || s != GF_OK) cudaStreamSynchronize(st);
    return s;
  };
  auto ck = [&](cudaError_t e, const char* w) { return e == cudaSuccess ? GF_OK : cuda_error(e, w); };
  gf_status s;
  if (mode == 0) {
    if ((s = ck(cudaMemcpyAsync(stage, h_image, pl.nvox * sizeof(float), cudaMemcpyHostToDevice, st), "upload image")) != GF_OK) return done(s);
    // mode 0: an FP32 image (image_storage is refused for it)
    float* img0 = static_cast<float*>(r->img[0]);
    if ((s = ck(launch_file_to_zfast(c->dg, stage, img0, st), "layout")) != GF_OK) return done(s);
    if ((s = r->project_all(img0, r->proj_ref)) != GF_OK) return done(s);
    r->loaded = true;
    r->mark();
    return done(GF_OK);
  }
  // STEP 1: projection of a unit cylinder -> proj_ref (GFIRST.cu:151-184).  It
  // depends on the geometry alone, so later loads of this reconstruction keep it.
  if (!r->cyl_proj_ready) {
    // the unit cylinder in the FP32 PSF buffer (the doubles image may be 16-bit)
    if ((s = ck(launch_cylinder(c->dg, 1.0f, r->psf, st), "cylinder")) != GF_OK) return done(s);
    if ((s = r->project_all(r->psf, r->proj_ref)) != GF_OK) return done(s);
    r->cyl_proj_ready = true;
  }
  // STEP 2: data (GFIRST.cu:207-260)
  // The sinogram and normalization go to the device staging on the
  // context's copy stream, so they can stream in while the context's
  // compute stream still runs earlier work (another reconstruction's
  // iterations); the layout kernels wait for them on the compute stream, and
  // the next load's copies wait until those kernels have read the staging.
  float* s2 = stage;                      // 2*NDATA
  float* sn = stage + 2 * pl.ndata;       // NDATA
  if (!r->ev_staged) {
    if ((s = ck(cudaEventCreateWithFlags(&r->ev_staged, cudaEventDisableTiming), "event")) != GF_OK) return done(s);
    if ((s = ck(cudaEventCreateWithFlags(&r->ev_stage_free, cudaEventDisableTiming), "event")) != GF_OK) return done(s);
  }
  cudaStream_t cs = c->copy_stream;
  // first load: the staging was just allocated in the compute stream's order,
  // so the copies wait for that point of it
  if (!r->stage_used && (s = ck(cudaEventRecord(r->ev_stage_free, st), "record staging")) != GF_OK) return done(s);
  if ((s = ck(cudaStreamWaitEvent(cs, r->ev_stage_free, 0), "wait staging")) != GF_OK) return done(s);
  if ((s = ck(cudaMemcpyAsync(s2, h_dsino, 2 * pl.ndata * sizeof(float), cudaMemcpyHostToDevice, cs), "upload sinogram")) != GF_OK) return done(s);
  if ((s = ck(cudaMemcpyAsync(sn, h_norm, pl.ndata * sizeof(float), cudaMemcpyHostToDevice, cs), "upload norm")) != GF_OK) return done(s);
  if ((s = ck(cudaEventRecord(r->ev_staged, cs), "record staging")) != GF_OK) return done(s);
  if ((s = ck(cudaStreamWaitEvent(st, r->ev_staged, 0), "wait upload")) != GF_OK) return done(s);
  if ((s = ck(launch_build_dbg(c->dg, c->d_rowmap, s2, r->dbg[0], st), "build data")) != GF_OK) return done(s);
  if ((s = ck(launch_build_cal(c->dg, c->d_rowmap, r->proj_ref, sn, r->cal, st), "build mask")) != GF_OK) return done(s);
  if (mode >= 2) {
    if ((s = ck(cudaMemcpyAsync(s2, h_tsino, 2 * pl.ndata * sizeof(float), cudaMemcpyHostToDevice, st), "upload triples")) != GF_OK) return done(s);
    if ((s = ck(launch_build_dbg(c->dg, c->d_rowmap, s2, r->dbg[1], st), "build triples")) != GF_OK) return done(s);
  }
  if (mode == 3) {
    if (nevents != r->nev) r->gen++;  // the split's launch holds the count
    r->nev = nevents;
    if (nevents > 0) {
      if (nevents > r->ev_cap) {
        // the smaller buffers go back to the pool before the larger ones are taken
        r->release(r->events);
        r->release(r->vlor_keys);
        r->release(r->vlor_share);
        r->events = nullptr;
        r->vlor_keys = nullptr;
        r->vlor_share = nullptr;
        r->ev_cap = 0;
        r->gen++;
        if ((s = r->alloc_t((size_t)nevents * 2, &r->events)) != GF_OK) return done(s);
        if ((s = r->alloc_t((size_t)nevents * 2, &r->vlor_keys)) != GF_OK) return done(s);
        if ((s = r->alloc_t((size_t)nevents * 2, &r->vlor_share)) != GF_OK) return done(s);
        r->ev_cap = nevents;
      }
      if ((s = ck(cudaMemcpyAsync(r->events, h_events, (size_t)nevents * 2 * sizeof(int32_t), cudaMemcpyHostToDevice, st), "upload events")) != GF_OK) return done(s);
      // the event ends in the order the VLOR split adds them (temporaries stream-ordered)
      unsigned long long* keys_tmp = nullptr;
      void* temp = nullptr;
      const size_t tb = vlor_sort_temp_bytes(nevents);
      cudaError_t e = cudaMallocAsync(&keys_tmp, (size_t)nevents * 2 * sizeof(unsigned long long), st);
      if (e == cudaSuccess) e = cudaMallocAsync(&temp, tb ? tb : 16, st);
      if (e == cudaSuccess) e = launch_vlor_sort(c->dg, r->events, nevents, keys_tmp, r->vlor_keys, temp, tb, st);
      if (keys_tmp) cudaFreeAsync(keys_tmp, st);
      if (temp) cudaFreeAsync(temp, st);
      if ((s = ck(e, "sort VLOR events")) != GF_OK) return done(s);
    }
    // counts in datos_v (scratch for now), then BLANKT (GFIRST.cu:229-247)
    if ((s = ck(cudaMemsetAsync(r->datos_v, 0, pl.ndata * sizeof(float), st), "memset")) != GF_OK) return done(s);
    if ((s = ck(launch_vlor_count(c->dg, r->events, nevents, r->datos_v, st), "vlor count")) != GF_OK) return done(s);
    if ((s = ck(launch_blankt(c->dg, r->datos_v, s2, r->blankt, st), "blankt")) != GF_OK) return done(s);
  }
  // the staging is free again once the compute stream has passed the layout kernels
  if ((s = ck(cudaEventRecord(r->ev_stage_free, st), "record staging free")) != GF_OK) return done(s);
  r->stage_used = true;
  if ((s = r->init_images()) != GF_OK) return done(s);
  r->loaded = true;
  r->mark();
  return done(GF_OK);
}

gf_status gf_recon_load(gf_recon* r, const float* h_image, const float* h_dsino, const float* h_tsino,
                        const float* h_norm, const int32_t* h_events, int64_t nevents) {
  return load_impl(r, h_image, h_dsino, h_tsino, h_norm, h_events, nevents, true);
}

gf_status gf_recon_load_async(gf_recon* r, const float* h_image, const float* h_dsino, const float* h_tsino,
                              const float* h_norm, const int32_t* h_events, int64_t nevents) {
  return load_impl(r, h_image, h_dsino, h_tsino, h_norm, h_events, nevents, false);
}

gf_status gf_recon_restart(gf_recon* r) {
  if (!r) return set_error(GF_ERR_ARG, "null reconstruction");
  if (!r->loaded) return set_error(GF_ERR_STATE, "gf_recon_load has not run");
  if (r->ntypes == 0) return GF_OK;
  GF_TRY(r->init_images());
  r->mark();
  return GF_OK;
}

gf_status gf_recon_subiteration(gf_recon* r) {
  if (!r) return set_error(GF_ERR_ARG, "null reconstruction");
  if (!r->loaded) return set_error(GF_ERR_STATE, "gf_recon_load has not run");
  if (r->ntypes == 0) return set_error(GF_ERR_STATE, "mode 0 has no iterations");
  GF_TRY(r->subiteration(r->cur_type, r->cur_sub));
  r->advance();
  r->mark();
  return GF_OK;
}

gf_status gf_recon_iterate(gf_recon* r, int32_t n) {
  if (!r) return set_error(GF_ERR_ARG, "null reconstruction");
  if (n < 0) return set_error(GF_ERR_ARG, "n must be >= 0");
  if (r->ntypes == 0) return n == 0 ? GF_OK : set_error(GF_ERR_STATE, "mode 0 has no iterations");
  const int64_t per = (int64_t)r->ntypes * r->ctx->plan.nsub;
  for (int64_t k = 0; k < per * n; k++) GF_TRY(gf_recon_subiteration(r));
  return GF_OK;
}

gf_status gf_recon_profile(gf_recon* r, int32_t enable) {
  if (!r) return set_error(GF_ERR_ARG, "null reconstruction");
  GF_CK(cudaStreamSynchronize(r->ctx->stream));
  r->prof = enable != 0;
  r->ev_used = 0;
  return GF_OK;
}

gf_status gf_recon_profile_read(gf_recon* r, int32_t stage, double* total_ms, int64_t* count) {
  if (!r || !total_ms || !count) return set_error(GF_ERR_ARG, "null argument");
  if (stage < 0 || stage >= GF_NUM_STAGES) return set_error(GF_ERR_ARG, "no such stage");
  GF_CK(cudaStreamSynchronize(r->ctx->stream));
  double tot = 0;
  int64_t n = 0;
  for (size_t i = 0; i < r->ev_used; i++) {
    if (r->evs[i].stage != stage) continue;
    float ms = 0.f;
    GF_CK(cudaEventElapsedTime(&ms, r->evs[i].a, r->evs[i].b));
    tot += ms;
    n++;
  }
  *total_ms = tot;
  *count = n;
  return GF_OK;
}

gf_status gf_recon_progress(const gf_recon* r, int32_t* it, int64_t* sub) {
  if (!r) return set_error(GF_ERR_ARG, "null reconstruction");
  if (it) *it = r->iters_done;
  if (sub) *sub = r->subs_done;
  return GF_OK;
}

gf_status gf_recon_get_image(gf_recon* r, int32_t type, int32_t scaled, float* h_out) {
  if (!r || !h_out) return set_error(GF_ERR_ARG, "null argument");
  if (type < 0 || type > 1 || !r->img[type]) return set_error(GF_ERR_ARG, "no such image");
  gf_ctx* c = r->ctx;
  const Plan& pl = c->plan;
  // on the context's copy stream, after this reconstruction's own queued
  // work only: work queued later for other reconstructions of the context
  // (the next data set's iterations) is not waited for
  cudaStream_t cs = c->copy_stream;
  GF_CK(cudaStreamWaitEvent(cs, r->ev_last, 0));
  float* tmp = nullptr;
  GF_CK(cudaMallocAsync(&tmp, pl.nvox * sizeof(float), cs));
  const float scale = type == 0 ? r->p.scale_d : r->p.scale_t;
  cudaError_t e = launch_zfast_to_file(c->dg, r->img[type], scale, scaled ? 1 : 0, tmp, cs, r->store(type));
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_out, tmp, pl.nvox * sizeof(float), cudaMemcpyDeviceToHost, cs);
  cudaFreeAsync(tmp, cs);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
  if (e != cudaSuccess) return cuda_error(e, "get image");
  return GF_OK;
}

gf_status gf_recon_get_proj_ref(gf_recon* r, float* h_out) {
  if (!r || !h_out) return set_error(GF_ERR_ARG, "null argument");
  if (!r->loaded) return set_error(GF_ERR_STATE, "gf_recon_load has not run");
  GF_CK(cudaMemcpyAsync(h_out, r->proj_ref, r->ctx->plan.ndata * sizeof(float), cudaMemcpyDeviceToHost, r->ctx->stream));
  GF_CK(cudaStreamSynchronize(r->ctx->stream));
  return GF_OK;
}

gf_status gf_recon_get_sinog_vlor(gf_recon* r, float* h_out) {
  if (!r || !h_out) return set_error(GF_ERR_ARG, "null argument");
  if (r->p.mode != 3) return set_error(GF_ERR_STATE, "only mode 3 splits VLOR events");
  GF_CK(cudaMemcpyAsync(h_out, r->datos_v, r->ctx->plan.ndata * sizeof(float), cudaMemcpyDeviceToHost, r->ctx->stream));
  GF_CK(cudaStreamSynchronize(r->ctx->stream));
  return GF_OK;
}

}  // extern "C"
