// gf_internal.h -- host-side context and reconstruction objects behind the C-ABI.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/gfirst.h"
#include "gf_kernels.h"
#include "gf_plan.h"

namespace gf {

gf_status set_error(gf_status st, const std::string& msg);
gf_status cuda_error(cudaError_t e, const char* what);

#define GF_CK(x)                                                \
  do {                                                          \
    cudaError_t e__ = (x);                                      \
    if (e__ != cudaSuccess) return ::gf::cuda_error(e__, #x);   \
  } while (0)

// Launch one of this library's kernels: count it and check the launch.
#define GF_LAUNCH(ctx, x)                                       \
  do {                                                          \
    (ctx)->launches++;                                          \
    cudaError_t e__ = (x);                                      \
    if (e__ != cudaSuccess) return ::gf::cuda_error(e__, #x);   \
  } while (0)

#define GF_TRY(x)                         \
  do {                                    \
    gf_status s__ = (x);                  \
    if (s__ != GF_OK) return s__;         \
  } while (0)

Taps9 gauss9(float psf);   // calcGaussianCoefficients, GFIRST_GPU_Kernels.cu:322-330
Taps5 gauss5();            // gaussian_filterZ's taps, GFIRST_CPU_Kernels.cpp:169-173
std::vector<float> bilateral_table(float sigma3d);  // 9x9x9 spatial weights

// Device buffer owned by a context or reconstruction.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  template <class T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace gf

struct gf_ctx {
  gf::Plan plan;
  gf::FpSchedule fps;
  gf::DevGeom dg{};
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaStream_t copy_stream = nullptr;  // host-to-device uploads of loads (overlap the compute stream)
  std::vector<gf::DevBuf> owned;  // freed on destroy
  std::vector<gf_recon*> recons;  // reconstructions still open on this context (destroyed with it)
  gf::DevSeg* d_seg = nullptr;
  float2* d_trig = nullptr;
  int2* d_rowmap = nullptr;
  int4* d_runs = nullptr;
  float* d_gtab = nullptr;
  float gtab_sigma = -1.f;
  // scratch of the operator entry points, allocated on first use
  int64_t launches = 0;  // kernels launched by this context
  // Bumped whenever a launch parameter that a captured graph holds changes
  // (the projectors' tile shapes, gf_tune); gf_batch recaptures on a change.
  int64_t gen = 0;
  int bp_warps = 4;      // back-projector warps (columns) per block (eight blocks per SM fit the register cap)
  // back projector's axial interpolation for doubles images and the operator
  // entry point (gf_set_bp_form); triples images always use GF_BP_PER_VOXEL
  int bp_form = GF_BP_PER_VIEW;
  gf::BpPads bpp;        // staged-row buffer of the per-view form
  float* s_img = nullptr;
  float* s_img2 = nullptr;
  float* s_numer = nullptr;
  float* s_denom = nullptr;
  float2* s_cc = nullptr;

  gf_status alloc(size_t bytes, void** p);
  template <class T> gf_status alloc_t(size_t n, T** p) {
    return alloc(n * sizeof(T), reinterpret_cast<void**>(p));
  }
  gf_status ensure_scratch();
  gf_status ensure_gtab(float sigma3d);
  gf::FpArgs fp_args(int subset, const float* img_zfast) const;
  gf::BpArgs bp_args(int subset, const void* corrcal, float* numer, float* denom, int storage) const;
};

struct gf_recon {
  gf_ctx* ctx = nullptr;
  gf_recon_params p{};
  int ntypes = 1;
  bool loaded = false;
  std::vector<gf::DevBuf> owned;
  void* img[2] = {nullptr, nullptr};  // z-fast images (doubles, triples), updated in place
  // element type of image t: image_storage, except mode 1's unused triples image (FP32)
  int store(int t) const { return (t == 0 || p.mode >= 2) ? p.image_storage : GF_STORE_F32; }
  float* psf = nullptr;
  float* ratio = nullptr;  // the back projector's update ratio NUMER/DENOM, z-fast
  float* filt = nullptr;
  void* corrcal = nullptr;  // (ratio, mask) pairs of the current subset, gf_recon_params::storage
  float2* dbg[2] = {nullptr, nullptr};
  float* cal = nullptr;
  float* proj_ref = nullptr;
  bool cyl_proj_ready = false;  // proj_ref holds the unit-cylinder projection (modes 1-3)
  float* proj_t = nullptr;  // triples projection, file layout (VLOR split weights)
  int32_t* events = nullptr;
  unsigned long long* vlor_keys = nullptr;  // event ends sorted by (bin, event), 2*nev
  float* vlor_share = nullptr;              // each event end's share of one split, 2*nev
  int64_t nev = 0, ev_cap = 0;
  float* blankt = nullptr;
  float* datos_v = nullptr;
  float* d_max = nullptr;
  float* stage = nullptr;  // device staging of host inputs (3*NDATA floats)
  cudaEvent_t ev_last = nullptr;        // the last work queued for this reconstruction (compute stream)
  bool marking = true;                  // off while a batch captures this reconstruction's work
  void mark() {
    if (ev_last && marking) cudaEventRecord(ev_last, ctx->stream);
  }
  cudaEvent_t ev_staged = nullptr;      // the uploads into `stage` are done (copy stream)
  cudaEvent_t ev_stage_free = nullptr;  // the layout kernels have read `stage` (compute stream)
  bool stage_used = false;
  gf::Taps9 g_fw{}, g_bw{};
  gf::Taps5 g5{};
  int iters_done = 0;
  int64_t subs_done = 0;
  int cur_type = 0, cur_sub = 0;
  int64_t launches_per_iteration = 0;  // kernels in one captured iteration
  // Bumped when a load changes what an iteration's launches capture (the
  // mode-3 event count or event buffers); gf_batch recaptures on a change.
  int64_t gen = 0;

  // stage profiling
  struct StageEv {
    int stage;
    cudaEvent_t a, b;
  };
  bool prof = false;
  std::vector<StageEv> evs;
  size_t ev_used = 0;
  void stage_begin(int stage);
  void stage_end();

  gf_status alloc(size_t bytes, void** p);
  // Returns an owned buffer to the device pool (stream-ordered) and forgets it.
  void release(void* p);
  template <class T> gf_status alloc_t(size_t n, T** q) {
    return alloc(n * sizeof(T), reinterpret_cast<void**>(q));
  }
  gf_status subiteration(int type, int subset);
  gf_status init_images();
  gf_status project_all(const float* img_zfast, float* proj_full);
  void advance();  // moves the (type, subset) cursor past one sub-iteration
};

namespace gf {
// Whether two loaded frames can share a fused launch: mode 1, one device and
// geometry, the same storage, filters, back-projector form and tile shapes
// (the subset counts may differ), so one launch per stage serves them all.
bool fusable(const gf_recon* a, const gf_recon* b);
// One sub-iteration of every frame of a fused group, all at the same subset
// index s, each at subset s of its own subset count: the forward PSF,
// projection + ratio and update are one launch each over the nfr <=
// kMaxFrames frames, the back projection one launch per subset count among
// them, on stream st (the group's: its first member's, which need not take
// part in every step) with the first frame's tables.  Advances every frame's
// cursor.  cls: frames with the same class >= 0 (same subset count and
// normalization mask; per-view back projector) back-project two per warp.
gf_status fused_subiteration(gf_recon* const* G, int nfr, const int* cls, cudaStream_t st);
}  // namespace gf
