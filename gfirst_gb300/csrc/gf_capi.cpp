// gf_capi.cpp -- the C-ABI of include/gfirst.h: geometry, context, operator
// entry points on device buffers in the reference's file layouts.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "gf_internal.h"

namespace gf {

static thread_local std::string g_err;

gf_status set_error(gf_status st, const std::string& msg) {
  g_err = msg;
  return st;
}

gf_status cuda_error(cudaError_t e, const char* what) {
  gf_status st = (e == cudaErrorMemoryAllocation) ? GF_ERR_NOMEM : GF_ERR_CUDA;
  return set_error(st, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

Taps9 gauss9(float psf) {
  // calcGaussianCoefficients, GFIRST_GPU_Kernels.cu:322-330
  Taps9 t{};
  float total = 0.f;
  for (int z = -4; z <= 4; ++z) {
    float a = (float)z * 1.662f / (psf + 0.1f);
    total += expf(-(a * a));
  }
  for (int k = 0, z = -4; z <= 4; ++z, ++k) {
    float a = (float)z * 1.662f / (psf + 0.1f);
    t.c[k] = expf(-(a * a)) / total;
  }
  return t;
}

Taps5 gauss5() {
  // gaussian_filterZ, GFIRST_CPU_Kernels.cpp:169-173
  Taps5 t{};
  float total = 0.f;
  for (int z = -2; z <= 2; ++z) total += expf(-(((float)z * 1.0f) * ((float)z * 1.0f)));
  for (int k = 0, z = -2; z <= 2; ++z, ++k) t.c[k] = expf(-(((float)z * 1.0f) * ((float)z * 1.0f))) / total;
  return t;
}

std::vector<float> bilateral_table(float sigma3d) {
  // float G = exp(-dist_spatial2/((2.0*sigma3D)*(2.0*sigma3D))), GFIRST_GPU_Kernels.cu:526-528
  std::vector<float> t(729);
  const double cs = (2.0 * (double)sigma3d) * (2.0 * (double)sigma3d);
  for (int dz = -4; dz <= 4; dz++)
    for (int dy = -4; dy <= 4; dy++)
      for (int dx = -4; dx <= 4; dx++) {
        float d2 = (float)(dx * dx + dy * dy + dz * dz);
        t[((dz + 4) * 9 + (dy + 4)) * 9 + (dx + 4)] = (float)exp((double)(-d2) / cs);
      }
  return t;
}

static bool to_geom(const gf_geometry* g, Geom* out) {
  if (!g) return false;
  *out = Geom{g->res, g->nzs, g->nrad, g->nang, g->span, g->nseg, g->pitch_mm, g->diam_det_mm, g->fov_mm};
  return true;
}

}  // namespace gf

using namespace gf;

// ---------------------------------------------------------------- context
gf_status gf_ctx::alloc(size_t bytes, void** p) {
  // stream-ordered: no device-wide synchronisation when contexts come and go
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMallocAsync(p, bytes, stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_error(e, "cudaMallocAsync");
  }
  owned.push_back(DevBuf{*p, bytes});
  return GF_OK;
}

gf_status gf_ctx::ensure_scratch() {
  if (s_img) return GF_OK;
  const Plan& p = plan;
  GF_TRY(alloc_t(p.nvoxp, &s_img));
  GF_TRY(alloc_t(p.nvoxp, &s_img2));
  GF_TRY(alloc_t(p.nvoxp, &s_numer));
  GF_TRY(alloc_t(p.nvoxp, &s_denom));
  GF_TRY(alloc_t((size_t)p.amax * p.g.nrad * p.PS, &s_cc));
  return GF_OK;
}

gf_status gf_ctx::ensure_gtab(float sigma3d) {
  if (!d_gtab) GF_TRY(alloc_t(729, &d_gtab));
  if (gtab_sigma != sigma3d) {
    std::vector<float> t = bilateral_table(sigma3d);
    GF_CK(cudaMemcpyAsync(d_gtab, t.data(), 729 * sizeof(float), cudaMemcpyHostToDevice, stream));
    GF_CK(cudaStreamSynchronize(stream));
    gtab_sigma = sigma3d;
  }
  return GF_OK;
}

FpArgs gf_ctx::fp_args(int subset, const float* img_zfast) const {
  FpArgs a{};
  a.g = dg;
  a.nfr = 1;
  a.fr[0].img = img_zfast;
  a.fr[0].subset = subset;
  a.fr[0].nsub = plan.nsub;
  a.fr[0].na = plan.sub_nang[subset];
  a.runs = d_runs;
  a.nruns = (int)fps.runs.size();
  a.padl = fps.padl;
  a.cw = fps.cw;
  a.lc = fps.lc;
  return a;
}

BpArgs gf_ctx::bp_args(int subset, const void* cc, float* numer, float* denom, int storage) const {
  BpArgs b{};
  b.g = dg;
  b.subset = subset;
  b.na = plan.sub_nang[subset];
  b.nfr = 1;
  b.fr[0].corrcal = cc;
  b.fr[0].numer = numer;
  b.fr[0].denom = denom;
  b.storage = storage;
  b.fast = bp_form == GF_BP_PER_VIEW ? 1 : 0;
  b.pad_lo = bpp.pad_lo;
  b.rbuf = bpp.rbuf;
  return b;
}

extern "C" {

gf_status gf_set_bp_form(gf_ctx* c, int32_t form) {
  if (!c) return set_error(GF_ERR_ARG, "null context");
  if (form != GF_BP_PER_VOXEL && form != GF_BP_PER_VIEW) return set_error(GF_ERR_ARG, "unknown back-projector form");
  if (form != c->bp_form) c->gen++;  // captured graphs hold the form
  c->bp_form = form;
  return GF_OK;
}

gf_status gf_bp_staged_rows(const gf_geometry* g, int32_t* pad_lo, int32_t* pad_hi, int32_t* rbuf) {
  Geom geo;
  if (!to_geom(g, &geo)) return set_error(GF_ERR_ARG, "null geometry");
  Plan p;
  std::string err;
  if (!make_plan(geo, 1, &p, &err)) return set_error(GF_ERR_GEOMETRY, err);
  const BpPads b = bp_fast_pads(p);
  if (pad_lo) *pad_lo = b.pad_lo;
  if (pad_hi) *pad_hi = b.pad_hi;
  if (rbuf) *rbuf = b.rbuf;
  return GF_OK;
}

gf_status gf_kernel_launches(const gf_ctx* c, int64_t* n) {
  if (!c || !n) return set_error(GF_ERR_ARG, "null argument");
  *n = c->launches;
  return GF_OK;
}

int32_t gf_abi_version(void) { return GF_ABI_VERSION; }

const char* gf_last_error(void) { return g_err.c_str(); }

gf_status gf_geometry_reference(gf_geometry* out) {
  if (!out) return set_error(GF_ERR_ARG, "null output");
  // GFIRST.h:5-15, 33-35
  *out = gf_geometry{128, 159, 147, 168, 11, 15, 1.63f, 165.7758f, 100.0f};
  return GF_OK;
}

gf_status gf_geometry_sizes(const gf_geometry* g, int64_t* planes, int64_t* ndata, int64_t* nvox) {
  Geom geo;
  if (!to_geom(g, &geo)) return set_error(GF_ERR_ARG, "null geometry");
  Plan p;
  std::string err;
  if (!make_plan(geo, 1, &p, &err)) return set_error(GF_ERR_GEOMETRY, err);
  if (planes) *planes = p.P;
  if (ndata) *ndata = p.ndata;
  if (nvox) *nvox = p.nvox;
  return GF_OK;
}

gf_status gf_segment_table(const gf_geometry* g, int32_t* idz, int32_t* zmin, int32_t* nz_acum) {
  Geom geo;
  if (!to_geom(g, &geo)) return set_error(GF_ERR_ARG, "null geometry");
  Plan p;
  std::string err;
  if (!make_plan(geo, 1, &p, &err)) return set_error(GF_ERR_GEOMETRY, err);
  for (int s = 0; s < geo.nseg; s++) {
    if (idz) idz[s] = p.seg[s].idz;
    if (zmin) zmin[s] = p.seg[s].zmin;
    if (nz_acum) nz_acum[s] = p.seg[s].acc;
  }
  if (nz_acum) nz_acum[geo.nseg] = p.P;
  return GF_OK;
}

gf_status gf_lor_index(const gf_geometry* g, int32_t seg_ind, int32_t iz0, int32_t itheta, int32_t ird,
                       int64_t* lor) {
  Geom geo;
  if (!to_geom(g, &geo) || !lor) return set_error(GF_ERR_ARG, "null argument");
  Plan p;
  std::string err;
  if (!make_plan(geo, 1, &p, &err)) return set_error(GF_ERR_GEOMETRY, err);
  if (seg_ind < 0 || seg_ind >= geo.nseg || itheta < 0 || itheta >= geo.nang || ird < 0 || ird >= geo.nrad)
    return set_error(GF_ERR_ARG, "index out of range");
  const Seg& s = p.seg[seg_ind];
  if (iz0 < s.zmin || iz0 >= geo.nzs - s.zmin) return set_error(GF_ERR_ARG, "plane outside the segment");
  *lor = lor_index(p, seg_ind, iz0, itheta, ird);
  return GF_OK;
}

gf_status gf_create(const gf_geometry* g, int32_t nsubsets, int32_t device, gf_ctx** out) {
  if (!out) return set_error(GF_ERR_ARG, "null output");
  *out = nullptr;
  Geom geo;
  if (!to_geom(g, &geo)) return set_error(GF_ERR_ARG, "null geometry");
  Plan plan;
  std::string err;
  if (!make_plan(geo, nsubsets, &plan, &err)) return set_error(GF_ERR_GEOMETRY, err);
  if (plan.NZP > 256) return set_error(GF_ERR_GEOMETRY, "nzs above 256 is not supported");
  if (plan.amax > 1024) return set_error(GF_ERR_GEOMETRY, "more than 1024 angles in one subset");
  if (plan.all_elems() >= ((int64_t)1 << 31)) return set_error(GF_ERR_GEOMETRY, "sinogram too large for int32 offsets");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(GF_ERR_NODEV, "no CUDA device");
  }
  if (device < 0 || device >= ndev) return set_error(GF_ERR_NODEV, "device index out of range");
  GF_CK(cudaSetDevice(device));
  cudaDeviceProp prop;
  GF_CK(cudaGetDeviceProperties(&prop, device));
  if (!(prop.major == 10 && prop.minor == 3))
    return set_error(GF_ERR_NODEV, std::string("this library is built for sm_103a; device is ") + prop.name);
  FpSchedule fps;
  // default tile shapes; gf_tune picks them by timing
  if (!make_fp_schedule(plan, fp_default_R(plan), 32, &fps))
    return set_error(GF_ERR_GEOMETRY, "no forward-projector schedule fits");

  {
    // keep memory returned by cudaFreeAsync cached in the device's pool, so
    // reconstructions created after others finish reuse it without a round
    // trip to the driver (process-local setting)
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  }
  gf_ctx* c = new gf_ctx();
  c->bpp = bp_fast_pads(plan);
  c->plan = std::move(plan);
  c->fps = std::move(fps);
  c->device = device;
  auto fail = [&](gf_status st) {
    gf_destroy(c);
    return st;
  };
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(cuda_error(cudaGetLastError(), "cudaStreamCreate"));
  c->own_stream = true;
  if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(cuda_error(cudaGetLastError(), "cudaStreamCreate (copies)"));
  const Plan& p = c->plan;
  std::vector<DevSeg> segs(p.g.nseg);
  for (int s = 0; s < p.g.nseg; s++)
    segs[s] = DevSeg{p.seg[s].zmin, p.seg[s].nplanes, p.seg[s].acc, p.seg[s].blk, p.seg[s].dz, p.seg[s].fz, 0, 0};
  std::vector<float2> trig(p.g.nang);
  for (int t = 0; t < p.g.nang; t++) trig[t] = make_float2(p.sinv[t], p.cosv[t]);
  std::vector<int2> rowmap(p.PS, make_int2(-1, -1));
  for (int s = 0; s < p.g.nseg; s++) {
    const Seg& sg = p.seg[s];
    rowmap[sg.blk] = make_int2(s, -1);
    for (int k = 0; k < sg.nplanes; k++) rowmap[sg.blk + 1 + k] = make_int2(s, sg.zmin + k);
    rowmap[sg.blk + sg.nplanes + 1] = make_int2(s, -2);
  }
  std::vector<int4> runs(c->fps.runs.size());
  for (size_t i = 0; i < runs.size(); i++) {
    const Run& r = c->fps.runs[i];
    runs[i] = make_int4(r.seg, r.p0, r.n, r.pad);
  }
  gf_status st;
  if ((st = c->alloc_t(segs.size(), &c->d_seg)) != GF_OK) return fail(st);
  if ((st = c->alloc_t(trig.size(), &c->d_trig)) != GF_OK) return fail(st);
  if ((st = c->alloc_t(rowmap.size(), &c->d_rowmap)) != GF_OK) return fail(st);
  if ((st = c->alloc_t(512, &c->d_runs)) != GF_OK) return fail(st);  // room for any schedule (<= 512 threads)
  cudaMemcpyAsync(c->d_seg, segs.data(), segs.size() * sizeof(DevSeg), cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->d_trig, trig.data(), trig.size() * sizeof(float2), cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->d_rowmap, rowmap.data(), rowmap.size() * sizeof(int2), cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->d_runs, runs.data(), runs.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream);
  if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return fail(cuda_error(e, "table upload"));
  DevGeom& d = c->dg;
  d.res = p.g.res; d.nzs = p.g.nzs; d.nrad = p.g.nrad; d.nang = p.g.nang; d.nseg = p.g.nseg; d.nzp = p.NZP;
  d.P = p.P; d.PP = p.PP; d.PS = p.PS; d.nsub = p.nsub;
  d.radm = p.radm; d.resm = p.resm; d.fx_fp = p.fx_fp; d.fx_bp = p.fx_bp;
  d.lam0 = p.lam0; d.lam1 = p.lam1;
  d.seg = c->d_seg;
  d.trig = c->d_trig;
  *out = c;
  return GF_OK;
}

void gf_destroy(gf_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  // reconstructions still open on this context go first: they free on its stream
  while (!c->recons.empty()) gf_recon_destroy(c->recons.back());
  // wait for the context's work, then return its memory on a stream of the
  // library's own, so a caller's stream set by gf_set_stream is not needed
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  cudaGetLastError();
  cudaStream_t fs = nullptr;
  if (cudaStreamCreateWithFlags(&fs, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    fs = nullptr;
  }
  for (auto& b : c->owned) cudaFreeAsync(b.p, fs);
  cudaStreamSynchronize(fs);
  if (fs) cudaStreamDestroy(fs);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  delete c;
}

gf_status gf_set_stream(gf_ctx* c, void* s) {
  if (!c) return set_error(GF_ERR_ARG, "null context");
  GF_CK(cudaStreamSynchronize(c->stream));
  if (c->own_stream) cudaStreamDestroy(c->stream);
  c->own_stream = false;
  c->stream = static_cast<cudaStream_t>(s);
  if (!s) {
    GF_CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  return GF_OK;
}

gf_status gf_synchronize(gf_ctx* c) {
  if (!c) return set_error(GF_ERR_ARG, "null context");
  GF_CK(cudaStreamSynchronize(c->stream));
  return GF_OK;
}

gf_status gf_device_alloc(gf_ctx* c, size_t bytes, void** d) {
  if (!c || !d) return set_error(GF_ERR_ARG, "null argument");
  GF_CK(cudaSetDevice(c->device));
  cudaError_t e = cudaMalloc(d, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_error(e, "cudaMalloc");
  }
  return GF_OK;
}

gf_status gf_device_free(gf_ctx* c, void* d) {
  if (!c) return set_error(GF_ERR_ARG, "null context");
  GF_CK(cudaFree(d));
  return GF_OK;
}

gf_status gf_host_alloc(size_t bytes, void** h) {
  if (!h) return set_error(GF_ERR_ARG, "null argument");
  cudaError_t e = cudaMallocHost(h, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_error(e, "cudaMallocHost");
  }
  return GF_OK;
}

gf_status gf_host_free(void* h) {
  GF_CK(cudaFreeHost(h));
  return GF_OK;
}

gf_status gf_copy_to_device(gf_ctx* c, void* d, const void* h, size_t bytes) {
  if (!c || (!d && bytes) || (!h && bytes)) return set_error(GF_ERR_ARG, "null argument");
  GF_CK(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, c->stream));
  GF_CK(cudaStreamSynchronize(c->stream));
  return GF_OK;
}

gf_status gf_copy_to_host(gf_ctx* c, void* h, const void* d, size_t bytes) {
  if (!c || (!d && bytes) || (!h && bytes)) return set_error(GF_ERR_ARG, "null argument");
  GF_CK(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, c->stream));
  GF_CK(cudaStreamSynchronize(c->stream));
  return GF_OK;
}

// ---------------------------------------------------------------- VLOR endpoints
static gf_status endpoints_of(const Plan& p, int64_t bin, float* out6) {
  const Geom& geo = p.g;
  if (bin < 0 || bin >= p.ndata) return set_error(GF_ERR_ARG, "bin out of range");
  const int64_t row = bin / ((int64_t)geo.nrad * geo.nang);
  const int t = (int)((bin / geo.nrad) % geo.nang), ird = (int)(bin % geo.nrad);
  int s = 0;
  while (s + 1 < geo.nseg && p.seg[s + 1].acc <= row) s++;
  const Seg& sg = p.seg[s];
  const int iz0 = (int)(row - sg.acc) + sg.zmin;
  // the forward projector's ray of this bin (GFIRST_GPU_Kernels.cu:75-96), in mm
  const double vx = (double)(geo.fov / (float)geo.res), hs = 0.5 * (double)geo.pitch;
  const double sn = p.sinv[t], cs = p.cosv[t];
  const double x0 = (double)p.fx_fp * ((double)ird - (double)p.radm) * vx;
  const double cx = x0 * cs, cy = x0 * sn;
  const double R = 0.5 * (double)geo.diam;
  const double h2 = R * R - x0 * x0;
  if (h2 <= 0.0) return set_error(GF_ERR_ARG, "bin's line of response misses the detector ring");
  const double lam = std::sqrt(h2) / vx;  // voxel steps from the closest point to the ring
  for (int k = 0; k < 2; k++) {
    const double l = k == 0 ? -lam : lam;
    const double zt = (double)iz0 + 0.5 + l * (double)sg.dz;
    out6[3 * k + 0] = (float)(cx + l * vx * sn);
    out6[3 * k + 1] = (float)(cy - l * vx * cs);
    out6[3 * k + 2] = (float)((zt - 0.5 * geo.nzs) * hs);
  }
  return GF_OK;
}

gf_status gf_bin_endpoints(const gf_geometry* gg, int64_t bin, float* out6) {
  return gf_bins_endpoints(gg, 1, &bin, out6);
}

gf_status gf_bins_endpoints(const gf_geometry* gg, int64_t n, const int64_t* bins, float* out) {
  Geom geo;
  if (!to_geom(gg, &geo) || (n > 0 && (!bins || !out)) || n < 0) return set_error(GF_ERR_ARG, "bad argument");
  Plan p;
  std::string err;
  if (!make_plan(geo, 1, &p, &err)) return set_error(GF_ERR_GEOMETRY, err);
  for (int64_t i = 0; i < n; i++) GF_TRY(endpoints_of(p, bins[i], out + 6 * i));
  return GF_OK;
}

gf_status gf_vlor_from_endpoints(gf_ctx* c, const float* d_lors, int64_t n, int32_t* d_events) {
  if (!c || (!d_lors && n) || (!d_events && n) || n < 0) return set_error(GF_ERR_ARG, "bad argument");
  const float vx = c->plan.g.fov / (float)c->plan.g.res, hs = 0.5f * c->plan.g.pitch;
  GF_LAUNCH(c, launch_vlor_endpoints(c->dg, d_lors, n, vx, hs, d_events, c->stream));
  return GF_OK;
}

// ---------------------------------------------------------------- operators
static gf_status check_subset(const gf_ctx* c, int32_t subset) {
  if (!c) return set_error(GF_ERR_ARG, "null context");
  if (subset < 0 || subset >= c->plan.nsub) return set_error(GF_ERR_ARG, "subset out of range");
  return GF_OK;
}

gf_status gf_forward_project(gf_ctx* c, const float* d_image, int32_t subset, float* d_proj) {
  GF_TRY(check_subset(c, subset));
  if (!d_image || !d_proj) return set_error(GF_ERR_ARG, "null buffer");
  GF_TRY(c->ensure_scratch());
  GF_LAUNCH(c, launch_file_to_zfast(c->dg, d_image, c->s_img, c->stream));
  FpArgs a = c->fp_args(subset, c->s_img);
  a.fr[0].proj_full = d_proj;
  GF_LAUNCH(c, launch_fp(a, c->fps, c->stream));
  return GF_OK;
}

gf_status gf_ratio(gf_ctx* c, const float* d_proj, const float* d_data, const float* d_bg, int32_t subset,
                   float* d_corr) {
  GF_TRY(check_subset(c, subset));
  if (!d_proj || !d_data || !d_bg || !d_corr) return set_error(GF_ERR_ARG, "null buffer");
  GF_LAUNCH(c, launch_ratio_file(c->dg, subset, d_proj, d_data, d_bg, d_corr, c->stream));
  return GF_OK;
}

gf_status gf_norm_mask(gf_ctx* c, const float* d_pb, const float* d_b, float* d_calib) {
  if (!c || !d_pb || !d_b || !d_calib) return set_error(GF_ERR_ARG, "null argument");
  GF_LAUNCH(c, launch_norm_mask(c->dg, d_pb, d_b, d_calib, c->stream));
  return GF_OK;
}

gf_status gf_back_project(gf_ctx* c, const float* d_corr, const float* d_calib, int32_t subset, float* d_numer,
                          float* d_denom) {
  GF_TRY(check_subset(c, subset));
  if (!d_corr || !d_calib || !d_numer || !d_denom) return set_error(GF_ERR_ARG, "null buffer");
  GF_TRY(c->ensure_scratch());
  const int na = c->plan.sub_nang[subset];
  GF_LAUNCH(c, launch_corrcal_from_file(c->dg, c->d_rowmap, subset, na, d_corr, d_calib, c->s_cc, c->stream));
  BpArgs b = c->bp_args(subset, c->s_cc, c->s_numer, c->s_denom, 0);
  GF_LAUNCH(c, launch_bp(b, c->bp_warps, c->stream));
  GF_LAUNCH(c, launch_zfast_to_file(c->dg, c->s_numer, 1.f, 0, d_numer, c->stream));
  GF_LAUNCH(c, launch_zfast_to_file(c->dg, c->s_denom, 1.f, 0, d_denom, c->stream));
  return GF_OK;
}

gf_status gf_psf_xy(gf_ctx* c, const float* d_in, float psf, float* d_out) {
  if (!c || !d_in || !d_out) return set_error(GF_ERR_ARG, "null argument");
  GF_TRY(c->ensure_scratch());
  GF_LAUNCH(c, launch_file_to_zfast(c->dg, d_in, c->s_img, c->stream));
  GF_LAUNCH(c, launch_conv_xy(c->dg, c->s_img, gauss9(psf), c->s_img2, c->stream));
  GF_LAUNCH(c, launch_zfast_to_file(c->dg, c->s_img2, 1.f, 0, d_out, c->stream));
  return GF_OK;
}

gf_status gf_image_update(gf_ctx* c, float* d_image, const float* d_numer, const float* d_denom, float psf_bw) {
  if (!c || !d_image || !d_numer || !d_denom) return set_error(GF_ERR_ARG, "null argument");
  GF_TRY(c->ensure_scratch());
  GF_LAUNCH(c, launch_file_to_zfast(c->dg, d_numer, c->s_numer, c->stream));
  GF_LAUNCH(c, launch_file_to_zfast(c->dg, d_denom, c->s_denom, c->stream));
  GF_LAUNCH(c, launch_file_to_zfast(c->dg, d_image, c->s_img, c->stream));
  GF_LAUNCH(c, launch_voxel_ratio(c->dg, c->s_numer, c->s_denom, c->s_img2, c->stream));
  GF_LAUNCH(c, launch_update(c->dg, c->s_img2, gauss9(psf_bw), gauss5(), c->s_img, c->stream));
  GF_LAUNCH(c, launch_zfast_to_file(c->dg, c->s_img, 1.f, 0, d_image, c->stream));
  return GF_OK;
}

gf_status gf_bilateral(gf_ctx* c, const float* d_in, const float* d_ref, float max_ref, int32_t r, float sigma3d,
                       float sigmai, float* d_out) {
  if (!c || !d_in || !d_ref || !d_out) return set_error(GF_ERR_ARG, "null argument");
  if (r < 0 || r > 4) return set_error(GF_ERR_ARG, "window radius must be in [0, 4]");
  GF_TRY(c->ensure_scratch());
  GF_TRY(c->ensure_gtab(sigma3d));
  GF_LAUNCH(c, launch_file_to_zfast(c->dg, d_in, c->s_img, c->stream));
  GF_LAUNCH(c, launch_file_to_zfast(c->dg, d_ref, c->s_img2, c->stream));
  GF_LAUNCH(c, launch_bilateral(c->dg, c->s_img, c->s_img2, nullptr, max_ref, r, sigmai, c->d_gtab, c->s_numer, c->stream));
  GF_LAUNCH(c, launch_zfast_to_file(c->dg, c->s_numer, 1.f, 0, d_out, c->stream));
  return GF_OK;
}

gf_status gf_vlor_count(gf_ctx* c, const int32_t* d_ev, int64_t n, float* d_count) {
  if (!c || (!d_ev && n) || !d_count || n < 0) return set_error(GF_ERR_ARG, "bad argument");
  GF_LAUNCH(c, launch_vlor_count(c->dg, d_ev, n, d_count, c->stream));
  return GF_OK;
}

gf_status gf_vlor_split(gf_ctx* c, const int32_t* d_ev, int64_t n, const float* d_proj, const float* d_blankt,
                        float* d_out) {
  if (!c || (!d_ev && n) || !d_proj || !d_blankt || !d_out || n < 0) return set_error(GF_ERR_ARG, "bad argument");
  if (n == 0) return GF_OK;
  if (n >= (1ll << 30)) return set_error(GF_ERR_ARG, "more than 2^30 events");
  // event ends sorted by (bin, event) in temporaries, then every bin's shares
  // added in event order: the reference's sums, no atomics
  cudaStream_t st = c->stream;
  unsigned long long *keys_tmp = nullptr, *keys = nullptr;
  float* share = nullptr;
  void* temp = nullptr;
  const size_t tb = vlor_sort_temp_bytes(n);
  cudaError_t e = cudaMallocAsync(&keys_tmp, (size_t)n * 2 * sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = cudaMallocAsync(&keys, (size_t)n * 2 * sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = cudaMallocAsync(&share, (size_t)n * 2 * sizeof(float), st);
  if (e == cudaSuccess) e = cudaMallocAsync(&temp, tb ? tb : 16, st);
  if (e == cudaSuccess) e = launch_vlor_sort(c->dg, d_ev, n, keys_tmp, keys, temp, tb, st);
  if (e == cudaSuccess) e = launch_vlor_split_sorted(c->dg, keys, n, d_ev, d_proj, d_blankt, share, d_out, st);
  if (e == cudaSuccess) c->launches += 4;
  if (keys_tmp) cudaFreeAsync(keys_tmp, st);
  if (keys) cudaFreeAsync(keys, st);
  if (share) cudaFreeAsync(share, st);
  if (temp) cudaFreeAsync(temp, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_error(e, "VLOR split");
  }
  return GF_OK;
}

}  // extern "C"
