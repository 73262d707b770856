// gf_noalloc.cu -- forward projection for callers that cannot allocate device
// memory.
//
// Some callers of this library cannot call cudaMalloc: a host that owns all
// device memory itself (a real-time acquisition system with a fixed memory
// map, an embedding framework with its own pool), or code running where a new
// allocation would stall or be refused.  gf_create allocates tables and
// gf_forward_project stages a transposed image in context scratch, so neither
// suits them.  gf_forward_project_noalloc takes the geometry by value and
// keeps everything it needs beyond the caller's input and output -- the
// z-fastest copy of the image, the segment and angle tables and the thread
// schedule -- in one file-scope __device__ array of GF_NOALLOC_SCRATCH_BYTES.
// Every GPU that loads the library holds that array until the process exits.
//
// The array's name in host code is a host-side stand-in, not a device
// address, so its device address is taken with cudaGetSymbolAddress once per
// device, with that device current, on the first call on that device.  All
// calls share the one array and it keeps the last call's contents; every call
// rewrites what it reads before reading it.  Calls whose work overlaps on the
// GPU (different streams, or another host thread) race on the array.
#include <cstring>
#include <mutex>
#include <vector>

#include "gf_internal.h"

namespace gf {

static __device__ __align__(256) unsigned char g_noalloc_scratch[GF_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[256] = {nullptr};

static size_t align256(size_t n) { return (n + 255) / 256 * 256; }

}  // namespace gf

using namespace gf;

extern "C" gf_status gf_forward_project_noalloc(const gf_geometry* gg, int32_t nsubsets, int32_t subset,
                                                const float* d_image, float* d_proj, void* cuda_stream) {
  if (!gg || !d_image || !d_proj) return set_error(GF_ERR_ARG, "null argument");
  Geom geo{gg->res, gg->nzs, gg->nrad, gg->nang, gg->span, gg->nseg, gg->pitch_mm, gg->diam_det_mm, gg->fov_mm};
  Plan plan;
  std::string err;
  if (!make_plan(geo, nsubsets, &plan, &err)) return set_error(GF_ERR_GEOMETRY, err);
  if (subset < 0 || subset >= plan.nsub) return set_error(GF_ERR_ARG, "subset out of range");
  FpSchedule fps;
  if (!make_fp_schedule(plan, fp_default_R(plan), 32, &fps))
    return set_error(GF_ERR_GEOMETRY, "no forward-projector schedule fits");
  // scratch layout: image (z-fastest) | segments | angles | thread runs
  const size_t b_img = align256((size_t)plan.nvoxp * sizeof(float));
  const size_t b_seg = align256((size_t)geo.nseg * sizeof(DevSeg));
  const size_t b_trig = align256((size_t)geo.nang * sizeof(float2));
  const size_t b_runs = align256(fps.runs.size() * sizeof(int4));
  const size_t need = b_img + b_seg + b_trig + b_runs;
  if (need > (size_t)GF_NOALLOC_SCRATCH_BYTES)
    return set_error(GF_ERR_ARG, "gf_forward_project_noalloc: geometry needs " + std::to_string(need) +
                                     " bytes of scratch, more than its fixed " +
                                     std::to_string((size_t)GF_NOALLOC_SCRATCH_BYTES) + " bytes");
  int dev = 0;
  GF_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) return set_error(GF_ERR_NODEV, "device index out of range");
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
      g_noalloc_addr[dev] = p;
    }
    base = static_cast<unsigned char*>(g_noalloc_addr[dev]);
  }
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  float* img = reinterpret_cast<float*>(base);
  DevSeg* dseg = reinterpret_cast<DevSeg*>(base + b_img);
  float2* dtrig = reinterpret_cast<float2*>(base + b_img + b_seg);
  int4* druns = reinterpret_cast<int4*>(base + b_img + b_seg + b_trig);
  std::vector<DevSeg> segs(geo.nseg);
  for (int s = 0; s < geo.nseg; s++) {
    const Seg& sg = plan.seg[s];
    segs[s] = DevSeg{sg.zmin, sg.nplanes, sg.acc, sg.blk, sg.dz, sg.fz, 0, 0};
  }
  std::vector<float2> trig(geo.nang);
  for (int t = 0; t < geo.nang; t++) trig[t] = make_float2(plan.sinv[t], plan.cosv[t]);
  std::vector<int4> runs(fps.runs.size());
  for (size_t i = 0; i < runs.size(); i++) runs[i] = make_int4(fps.runs[i].seg, fps.runs[i].p0, fps.runs[i].n, fps.runs[i].pad);
  // pageable sources: each copy has read its source when the call returns
  GF_CK(cudaMemcpyAsync(dseg, segs.data(), segs.size() * sizeof(DevSeg), cudaMemcpyHostToDevice, st));
  GF_CK(cudaMemcpyAsync(dtrig, trig.data(), trig.size() * sizeof(float2), cudaMemcpyHostToDevice, st));
  GF_CK(cudaMemcpyAsync(druns, runs.data(), runs.size() * sizeof(int4), cudaMemcpyHostToDevice, st));
  DevGeom dg{};
  dg.res = geo.res; dg.nzs = geo.nzs; dg.nrad = geo.nrad; dg.nang = geo.nang; dg.nseg = geo.nseg;
  dg.nzp = plan.NZP; dg.P = plan.P; dg.PP = plan.PP; dg.PS = plan.PS; dg.nsub = plan.nsub;
  dg.radm = plan.radm; dg.resm = plan.resm; dg.fx_fp = plan.fx_fp; dg.fx_bp = plan.fx_bp;
  dg.lam0 = plan.lam0; dg.lam1 = plan.lam1;
  dg.seg = dseg;
  dg.trig = dtrig;
  GF_CK(launch_file_to_zfast(dg, d_image, img, st));
  FpArgs a{};
  a.g = dg;
  a.nfr = 1;
  a.fr[0].img = img;
  a.fr[0].subset = subset;
  a.fr[0].nsub = plan.nsub;
  a.fr[0].na = plan.sub_nang[subset];
  a.runs = druns;
  a.nruns = (int)fps.runs.size();
  a.padl = fps.padl;
  a.cw = fps.cw;
  a.lc = fps.lc;
  a.fr[0].proj_full = d_proj;
  GF_CK(launch_fp(a, fps, st));
  return GF_OK;
}
