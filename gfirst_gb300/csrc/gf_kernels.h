// gf_kernels.h -- host-callable launchers of the sm_103a kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "gf_device.cuh"
#include "gf_plan.h"

namespace gf {

// (ratio, mask) pair storage of the per-subset sinogram.
template <int S> struct PairT;
template <> struct PairT<0> { using type = float2; };
template <> struct PairT<1> { using type = __half2; };
template <> struct PairT<2> { using type = __nv_bfloat162; };

struct Taps9 { float c[9]; };
struct Taps5 { float c[5]; };

// One launch may serve several frames of one geometry (a fused group of a
// batch): every per-frame buffer sits in a table of kMaxFrames entries passed
// by value, the launch has one grid slice per frame, and a block takes its
// frame's entry.  In the forward projector the frames may differ in subset
// count (each entry names its frame's subset); the back projector's frames
// share one.  A single-frame launch fills entry 0.
constexpr int kMaxFrames = 16;

// ---- forward projector (gf_fp.cu) ----
struct FpFrame {
  const float* img;        // z-fast image (after the forward PSF)
  const float2* dbg;       // subset layout (data*RES, max(bg*RES,0)); with corrcal
  const float* cal;        // subset layout normalization mask; with corrcal
  void* corrcal;           // subset layout (corr, calib) pairs output, or null
  float* proj_full;        // file-layout projection output, or null
  int subset, nsub, na;    // the frame's subset, its subset count and the subset's angles
};
struct FpArgs {
  DevGeom g;               // g.nsub unused: each frame names its own
  const int4* runs;        // FpSchedule::runs as (seg, p0, n, pad)
  int nruns, padl, cw, lc;
  int storage;             // corrcal pair type: 0 float2, 1 __half2, 2 __nv_bfloat162
  int nfr;                 // frames in this launch (grid z); 0 is taken as 1
  FpFrame fr[kMaxFrames];
};
cudaError_t launch_fp(const FpArgs& a, const FpSchedule& s, cudaStream_t st);

// ---- back projector (gf_bp.cu) ----
struct BpFrame {
  const void* corrcal;     // subset layout (corr, calib) pairs
  float* numer;            // z-fast
  float* denom;            // z-fast
};
// The back projector's launches serve one subset (of g.nsub) for all frames.
struct BpArgs {
  DevGeom g;
  int subset, na;          // na: angles in this subset
  int nfr;                 // frames in this launch (grid y); 0 is taken as 1
  BpFrame fr[kMaxFrames];
  int storage;             // corrcal pair type, as FpArgs::storage
  // Axial interpolation: 0 per voxel with the reference's rounding (the
  // oracle's sums bit for bit), 1 per view (BpPads; within 1e-5 of it).
  int fast;
  int pad_lo, rbuf;        // fast form: staged-row buffer per warp (BpPads)
  // 0: write the column sums to BpFrame::numer and ::denom; 1: write the
  // update ratio NUMER/DENOM (divVxVGPU) to ::numer alone (::denom unused).
  int ratio;
};
cudaError_t launch_bp(const BpArgs& a, int warps, cudaStream_t st);
// Per-view form over a.nfr = 2n frames as n pairs (frames 2p, 2p + 1) that
// share their normalization mask: one warp per column and pair.
cudaError_t launch_bp_pairs(const BpArgs& a, int warps, cudaStream_t st);
// Lets kernel k use up to the device's opt-in shared memory per block.  Every
// call sets the same value, so host threads that launch one kernel with
// different shared-memory sizes at the same time cannot undo each other's
// setting between the attribute call and the launch.
template <class K>
inline cudaError_t allow_max_smem(K k) {
  static const int maxsm = [] {
    int dev = 0, v = 48 * 1024;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
  }();
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, maxsm);
}


// ---- image kernels (gf_image.cu) ----
// Image elements: in_store/img_store/out_store 0 FP32, 1 FP16, 2 BF16 (16-bit image storage).
// out = XY PSF of the image `in`.
cudaError_t launch_conv_xy(const DevGeom& g, const void* in, const Taps9& t, float* out, cudaStream_t st,
                           int in_store = 0);
// out = the update ratio NUMER/DENOM (1 where DENOM < 0.001), z-fast.
cudaError_t launch_voxel_ratio(const DevGeom& g, const float* numer, const float* denom, float* out,
                               cudaStream_t st);
// img *= axial_filter(XY PSF of the update ratio), then the edge-slice copy;
// in place, one launch.
cudaError_t launch_update(const DevGeom& g, const float* ratio, const Taps9& t9, const Taps5& t5, void* img,
                          cudaStream_t st, int img_store = 0);
// The same two over nfr frames of one geometry in one launch each.
struct ImgFrame {
  const void* in;  // conv_xy: the image; update: the ratio (FP32)
  float* out;      // conv_xy output
  void* img;       // update: the image updated in place
};
struct ImgFrames {
  ImgFrame fr[kMaxFrames];
};
cudaError_t launch_conv_xy_frames(const DevGeom& g, const ImgFrames& f, int nfr, const Taps9& t, cudaStream_t st,
                                  int in_store = 0);
cudaError_t launch_update_frames(const DevGeom& g, const ImgFrames& f, int nfr, const Taps9& t9, const Taps5& t5,
                                 cudaStream_t st, int img_store = 0);
// Output slices per CTA of the update kernel.
int update_chunk(const DevGeom& g);
cudaError_t launch_file_to_zfast(const DevGeom& g, const float* in, float* out, cudaStream_t st);
cudaError_t launch_zfast_to_file(const DevGeom& g, const void* in, float scale, int mask, float* out,
                                 cudaStream_t st, int in_store = 0);
cudaError_t launch_cylinder(const DevGeom& g, float val, void* out, cudaStream_t st, int out_store = 0);
// store: element type of the image arguments (0 FP32, 1 FP16, 2 BF16)
cudaError_t launch_max_nonneg(const DevGeom& g, const void* img, float* d_max, cudaStream_t st, int store = 0);
cudaError_t launch_bilateral(const DevGeom& g, const void* in, const void* ref, const float* d_max_ref,
                             float max_ref, int r, float sigmai, const float* gtab, float* out, cudaStream_t st,
                             int store = 0);
cudaError_t launch_blend(const DevGeom& g, void* img2, const float* filt, cudaStream_t st, int store = 0);

// ---- sinogram kernels (gf_sino.cu) ----
// rowmap[row'] = (segment, plane) of a padded row, (-1,-1) for a pad row.
cudaError_t launch_build_dbg(const DevGeom& g, const int2* rowmap, const float* sino2, float2* dbg,
                             cudaStream_t st);
cudaError_t launch_build_cal(const DevGeom& g, const int2* rowmap, const float* proj_ref, const float* norm,
                             float* cal, cudaStream_t st);
cudaError_t launch_corrcal_from_file(const DevGeom& g, const int2* rowmap, int subset, int na, const float* corr,
                                     const float* calib, float2* corrcal, cudaStream_t st);
cudaError_t launch_ratio_gather(const DevGeom& g, const int2* rowmap, int subset, int na, const float* proj_full,
                                const float* datos_v, const float2* dbg_t, const float* cal, void* corrcal,
                                int storage, cudaStream_t st);
cudaError_t launch_ratio_file(const DevGeom& g, int subset, const float* proj, const float* data, const float* bg,
                              float* corr, cudaStream_t st);
cudaError_t launch_norm_mask(const DevGeom& g, const float* proj_blank, const float* blank, float* calib,
                             cudaStream_t st);
// *flag = 1 (device int) when the n floats of a and b differ anywhere.
cudaError_t launch_differs(const float* a, const float* b, size_t n, int* flag, cudaStream_t st);
cudaError_t launch_vlor_count(const DevGeom& g, const int32_t* ev, long long nev, float* cnt, cudaStream_t st);
cudaError_t launch_blankt(const DevGeom& g, const float* cnt, const float* tsino_raw, float* blankt,
                          cudaStream_t st);

// The split in the reference's order: keys of the event ends sorted by (bin,
// event) once (launch_vlor_sort; keys_tmp and keys hold 2*nev entries, temp
// vlor_sort_temp_bytes(nev) bytes), then each event's two shares computed into
// share (2*nev floats) and each bin's shares summed in event order.
size_t vlor_sort_temp_bytes(long long nev);
cudaError_t launch_vlor_sort(const DevGeom& g, const int32_t* ev, long long nev, unsigned long long* keys_tmp,
                             unsigned long long* keys, void* temp, size_t temp_bytes, cudaStream_t st);
cudaError_t launch_vlor_split_sorted(const DevGeom& g, const unsigned long long* keys, long long nev,
                                     const int32_t* ev, const float* proj, const float* blankt, float* share,
                                     float* out, cudaStream_t st);

cudaError_t launch_vlor_endpoints(const DevGeom& g, const float* lors, long long n, float vx, float hs, int32_t* ev,
                                  cudaStream_t st);

}  // namespace gf
