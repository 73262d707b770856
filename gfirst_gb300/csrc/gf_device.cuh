// gf_device.cuh -- device-side geometry and helpers shared by the kernels.
//
// Rounding: where a kernel must agree bit for bit with the reference's
// expression (coordinates, the image-update chain) it uses the explicit
// round-to-nearest intrinsics, so nvcc cannot fuse a multiply and an add the
// source writes as two operations.  Interpolation is lerp(a,b,w) =
// fma(w, b-a, a), the rule the CPU oracle uses for the texture unit.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gf {

struct DevSeg {
  int zmin, nplanes, acc, blk;
  float dz, fz;
  int pad0, pad1;
};

// Geometry passed by value to every kernel.
struct DevGeom {
  int res, nzs, nrad, nang, nseg, nzp;
  int P, PP, PS, nsub;
  float radm, resm, fx_fp, fx_bp;
  int lam0, lam1;
  const DevSeg* seg;    // nseg entries
  const float2* trig;   // per angle (sin, cos)
};

#ifdef __CUDACC__
__device__ __forceinline__ float2 pair_f(float2 v) { return v; }
__device__ __forceinline__ float2 pair_f(__half2 v) { return __half22float2(v); }
__device__ __forceinline__ float2 pair_f(__nv_bfloat162 v) { return __bfloat1622float2(v); }
template <class P> __device__ __forceinline__ P pair_from(float2 v);
template <> __device__ __forceinline__ float2 pair_from<float2>(float2 v) { return v; }
template <> __device__ __forceinline__ __half2 pair_from<__half2>(float2 v) { return __float22half2_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat162 pair_from<__nv_bfloat162>(float2 v) { return __float22bfloat162_rn(v); }

__device__ __forceinline__ float lerp_rn(float a, float b, float w) { return __fmaf_rn(w, __fsub_rn(b, a), a); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }
// The update ratio of divVxVGPU (GFIRST_GPU_Kernels.cu:173-182): NUMER/DENOM,
// 1 where DENOM < 0.001.
__device__ __forceinline__ float update_ratio(float n, float d) { return d < 0.001f ? 1.0f : __fdiv_rn(n, d); }

// Angle index of the l-th angle of subset s of nsub.
__device__ __forceinline__ int subset_angle(int s, int nsub, int l) { return s + l * nsub; }
__device__ __forceinline__ int subset_angle(const DevGeom& g, int s, int l) { return subset_angle(s, g.nsub, l); }
#endif

}  // namespace gf
