// gf_image.cu -- image-domain kernels on z-fast volumes [RES][RES][NZP].
//
// The update chain of GFIRST.cu:482-502 (divVxVGPU, convolutionXY,
// gaussian_filterZ, multiply, edge-slice copy; the back projector writes the
// ratio, the rest is one kernel), the forward PSF
// (GFIRST.cu:324-340), the joint bilateral filter (GFIRST_GPU_Kernels.cu:
// 508-539) and layout conversions.  All of these are HBM-bound except the
// bilateral filter; they keep the reference's operation order with explicit
// round-to-nearest arithmetic so their results equal the reference's.
#include "gf_kernels.h"

namespace gf {

// Image elements: FP32, or FP16/BF16 storage of the reconstructed images
// (every operation in FP32; a store rounds to nearest even).
__device__ __forceinline__ float img_ld(const float* p) { return *p; }
__device__ __forceinline__ float img_ld(const __half* p) { return __half2float(*p); }
__device__ __forceinline__ float img_ld(const __nv_bfloat16* p) { return __bfloat162float(*p); }
__device__ __forceinline__ void img_st(float* p, float v) { *p = v; }
__device__ __forceinline__ void img_st(__half* p, float v) { *p = __float2half_rn(v); }
__device__ __forceinline__ void img_st(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }

// ---- separable XY Gaussian, GFIRST_GPU_Kernels.cu:332-358 -----------------
// Stages the 16x16-column tile around output columns [x0, x0+8) x [y0, y0+8)
// at this lane's slice z into S, 0 outside the image (or everywhere when
// !zok): warp ty loads halo columns ty and ty + 8 of every halo row, so the
// two columns' bounds and offsets are computed once and each row is one
// stride further.
template <class T>
__device__ __forceinline__ void stage_halo(float (&S)[16][16][32], const T* __restrict__ in, bool zok, int z, int x0,
                                           int y0, int ty, int lane, int RES, int NZP) {
  const int xa = x0 - 4 + ty, xb = x0 + 4 + ty;  // xb >= 4
  const bool oka = zok && xa >= 0 && xa < RES, okb = zok && xb < RES;
  const long long rs = (long long)RES * NZP;
  const long long ra = ((long long)(y0 - 4) * RES + xa) * NZP + z;  // element offset at halo row 0, column xa
  const long long rb = ra + 8LL * NZP;                               // column xb
#pragma unroll
  for (int yy = 0; yy < 16; yy++) {
    const int y = y0 - 4 + yy;
    const bool oky = y >= 0 && y < RES;
    S[yy][ty][lane] = (oky && oka) ? img_ld(in + (ra + yy * rs)) : 0.f;
    S[yy][ty + 8][lane] = (oky && okb) ? img_ld(in + (rb + yy * rs)) : 0.f;
  }
}

// conv_xy9 runs it on an 8x8-column, 32-slice tile staged with a 4-column
// halo in S: the y pass is zero-padded; the x pass runs only for
// 3 < x < RES-4 and border columns output the raw input.  Thread (row ty,
// lane) leaves the 8 outputs of its row at its slice in v[].
__device__ __forceinline__ void conv_xy9(float (&S)[16][16][32], int ty, int lane, int x0, int RES, const Taps9& G,
                                         float (&v)[8]) {
  // the y pass of row ty over the 16 halo columns stays in this thread's
  // registers: the x pass below reads only its own row and slice
  float yv[16];
#pragma unroll
  for (int xx = 0; xx < 16; xx++) {
    float acc = __fmul_rn(S[ty][xx][lane], G.c[0]);
#pragma unroll
    for (int k = 1; k < 9; k++) acc = __fadd_rn(acc, __fmul_rn(S[ty + k][xx][lane], G.c[k]));
    yv[xx] = acc;
  }
#pragma unroll
  for (int xo = 0; xo < 8; xo++) {
    const int x = x0 + xo;
    if (x > 3 && x < RES - 4) {
      float a = __fmul_rn(yv[xo], G.c[0]);
#pragma unroll
      for (int k = 1; k < 9; k++) a = __fadd_rn(a, __fmul_rn(yv[xo + k], G.c[k]));
      v[xo] = a;
    } else {
      v[xo] = S[ty + 4][xo + 4][lane];
    }
  }
}

// The forward PSF (GFIRST.cu:324-340) of an image.  CTA: 8x8 columns x 32
// slices; grid z runs over (frame, 32-slice chunk): frame f's buffers are
// fr.fr[f].
template <class T>
__global__ void __launch_bounds__(256) conv_xy_kernel(const DevGeom g, const ImgFrames fr, const Taps9 G) {
  __shared__ float S[16][16][32];
  const int nzc = g.nzp / 32;
  const int f = blockIdx.z / nzc;
  const T* __restrict__ in = static_cast<const T*>(fr.fr[f].in);
  float* __restrict__ out = fr.fr[f].out;
  const int lane = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int x0 = blockIdx.x * 8, y0 = blockIdx.y * 8, z = (blockIdx.z - f * nzc) * 32 + lane;
  const int RES = g.res, NZP = g.nzp;
  stage_halo(S, in, true, z, x0, y0, ty, lane, RES, NZP);
  __syncthreads();
  float v[8];
  conv_xy9(S, ty, lane, x0, RES, G, v);
  const int y = y0 + ty;
  if (y >= RES) return;
#pragma unroll
  for (int xo = 0; xo < 8; xo++) {
    const int x = x0 + xo;
    if (x >= RES) break;
    out[((size_t)y * RES + x) * NZP + z] = (z < g.nzs) ? v[xo] : 0.f;
  }
}

cudaError_t launch_conv_xy_frames(const DevGeom& g, const ImgFrames& f, int nfr, const Taps9& t, cudaStream_t st,
                                  int in_store) {
  if (nfr < 1 || nfr > kMaxFrames) return cudaErrorInvalidValue;
  for (int k = 0; k < nfr; k++)
    if (!f.fr[k].in || !f.fr[k].out) return cudaErrorInvalidValue;
  dim3 grid((g.res + 7) / 8, (g.res + 7) / 8, (g.nzp / 32) * nfr);
  if (in_store == 1) {
    conv_xy_kernel<__half><<<grid, 256, 0, st>>>(g, f, t);
  } else if (in_store == 2) {
    conv_xy_kernel<__nv_bfloat16><<<grid, 256, 0, st>>>(g, f, t);
  } else {
    conv_xy_kernel<float><<<grid, 256, 0, st>>>(g, f, t);
  }
  return cudaGetLastError();
}

cudaError_t launch_conv_xy(const DevGeom& g, const void* in, const Taps9& t, float* out, cudaStream_t st,
                           int in_store) {
  ImgFrames f{};
  f.fr[0].in = in;
  f.fr[0].out = out;
  return launch_conv_xy_frames(g, f, 1, t, st, in_store);
}

// ---- the update ratio, divVxVGPU (GFIRST_GPU_Kernels.cu:173-182) ------------
__global__ void __launch_bounds__(256) voxel_ratio_kernel(size_t n, const float* __restrict__ numer,
                                                          const float* __restrict__ denom, float* __restrict__ out) {
  const size_t i = (size_t)blockIdx.x * 256 + threadIdx.x;
  if (i < n) out[i] = update_ratio(numer[i], denom[i]);
}

cudaError_t launch_voxel_ratio(const DevGeom& g, const float* numer, const float* denom, float* out,
                               cudaStream_t st) {
  const size_t n = (size_t)g.res * g.res * g.nzp;
  voxel_ratio_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, numer, denom, out);
  return cudaGetLastError();
}

// ---- axial filter, gaussian_filterZ (GFIRST_CPU_Kernels.cpp:165-187) -------
// Its loop counter is incremented before use, so loop position (K, y, x)
// writes voxel (K, y, x)+1: voxel (z, y, x) takes the rule of slice z, except
// column (y=0, x=0), which takes the rule of slice z-1; reads past the last
// slice are 0.  The rule is applied centred on the voxel itself; m2..p2 are
// the inputs at slices z-2..z+2, already 0 outside [0, NZS).
// Which rule slice K takes, in the reference's order of tests: 0 the first
// slice's 2 taps, 1 the last slice's 2 taps, 2 the 3 taps of the second and
// second-to-last slices, 3 the 5-tap Gaussian.
__device__ __forceinline__ int zrule_of(int K, int NZS) {
  return K == 0 ? 0 : (K == NZS - 1 ? 1 : ((K == 1 || K == NZS - 2) ? 2 : 3));
}
__device__ __forceinline__ float zrule(float m2, float m1, float c0, float p1, float p2, int rule, const Taps5& g) {
  if (rule == 0) return __fadd_rn(__fmul_rn(0.5f, c0), __fmul_rn(0.5f, p1));
  if (rule == 1) return __fadd_rn(__fmul_rn(0.5f, m1), __fmul_rn(0.5f, c0));
  if (rule == 2)
    return __fadd_rn(__fadd_rn(__fmul_rn(0.333f, m1), __fmul_rn(0.333f, c0)), __fmul_rn(0.333f, p1));
  float v = __fmul_rn(g.c[0], m2);
  v = __fadd_rn(v, __fmul_rn(g.c[1], m1));
  v = __fadd_rn(v, __fmul_rn(g.c[2], c0));
  v = __fadd_rn(v, __fmul_rn(g.c[3], p1));
  v = __fadd_rn(v, __fmul_rn(g.c[4], p2));
  return v;
}

// ---- the image update of GFIRST.cu:482-496 in one pass ----------------------
// C = convolutionXY(ratio), img = img * gaussian_filterZ(C), then slice 0 <-
// slice 1 and slice NZS-1 <- slice NZS-2, in place.  CTA: 8x8 columns x `cs`
// output slices from z0; lane l holds slice z0 - 2 + l, so C is computed on
// the chunk and two slices either side (lanes 2..cs+1 are the outputs) and
// the axial taps are register shuffles of C.  The edge copies take the
// neighbour slice's old image value and rule, i.e. the neighbour's updated
// value: a shuffle of the products.  Slice 1 always sits in slice 0's chunk,
// and `cs` is chosen so that slice NZS-1 is never a chunk's first output, so
// a CTA reads image values of its own outputs only and the in-place update
// needs no ordering between CTAs.  Grid z runs over (frame, chunk).
template <class T>
__global__ void __launch_bounds__(256, 6) update_kernel(const DevGeom g, const ImgFrames fr, const Taps9 G,
                                                     const Taps5 t5, int cs) {
  __shared__ float S[16][16][32];
  const int nzc = (g.nzp + cs - 1) / cs;
  const int f = blockIdx.z / nzc;
  const float* __restrict__ ratio = static_cast<const float*>(fr.fr[f].in);
  T* img = static_cast<T*>(fr.fr[f].img);
  const int lane = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int x0 = blockIdx.x * 8, y0 = blockIdx.y * 8;
  const int z = (blockIdx.z - f * nzc) * cs - 2 + lane;
  const int RES = g.res, NZP = g.nzp, NZS = g.nzs;
  stage_halo(S, ratio, z >= 0 && z < NZP, z, x0, y0, ty, lane, RES, NZP);
  __syncthreads();
  float v[8];
  conv_xy9(S, ty, lane, x0, RES, G, v);
  const int y = y0 + ty;
  if (y >= RES) return;  // whole warp
  const bool out_lane = lane >= 2 && lane < cs + 2 && z < NZP;
  const bool zin = z >= 0 && z < NZS;
  const int rule = zrule_of(z, NZS);
#pragma unroll
  for (int xo = 0; xo < 8; xo++) {
    const int x = x0 + xo;
    if (x >= RES) break;  // whole warp
    const size_t o = ((size_t)y * RES + x) * NZP + z;
    const float iv = out_lane ? img_ld(img + o) : 0.f;
    const float c0 = zin ? v[xo] : 0.f;
    const float m1 = __shfl_up_sync(0xffffffffu, c0, 1), m2 = __shfl_up_sync(0xffffffffu, c0, 2);
    const float p1 = __shfl_down_sync(0xffffffffu, c0, 1), p2 = __shfl_down_sync(0xffffffffu, c0, 2);
    // column (0, 0) takes slice z-1's rule
    const float prod = __fmul_rn(iv, zrule(m2, m1, c0, p1, p2, (x == 0 && y == 0) ? zrule_of(z - 1, NZS) : rule, t5));
    const float up = __shfl_down_sync(0xffffffffu, prod, 1);  // slice z + 1
    const float dn = __shfl_up_sync(0xffffffffu, prod, 1);    // slice z - 1
    if (out_lane) img_st(img + o, z >= NZS ? 0.f : (z == 0 ? up : (z == NZS - 1 ? dn : prod)));
  }
}

int update_chunk(const DevGeom& g) { return (g.nzs > 1 && (g.nzs - 1) % 28 == 0) ? 27 : 28; }

cudaError_t launch_update_frames(const DevGeom& g, const ImgFrames& f, int nfr, const Taps9& t9, const Taps5& t5,
                                 cudaStream_t st, int img_store) {
  if (nfr < 1 || nfr > kMaxFrames) return cudaErrorInvalidValue;
  for (int k = 0; k < nfr; k++)
    if (!f.fr[k].in || !f.fr[k].img) return cudaErrorInvalidValue;
  const int cs = update_chunk(g);
  dim3 grid((g.res + 7) / 8, (g.res + 7) / 8, ((g.nzp + cs - 1) / cs) * nfr);
  switch (img_store) {
    case 0: update_kernel<float><<<grid, 256, 0, st>>>(g, f, t9, t5, cs); break;
    case 1: update_kernel<__half><<<grid, 256, 0, st>>>(g, f, t9, t5, cs); break;
    case 2: update_kernel<__nv_bfloat16><<<grid, 256, 0, st>>>(g, f, t9, t5, cs); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_update(const DevGeom& g, const float* ratio, const Taps9& t9, const Taps5& t5, void* img,
                          cudaStream_t st, int img_store) {
  ImgFrames f{};
  f.fr[0].in = ratio;
  f.fr[0].img = img;
  return launch_update_frames(g, f, 1, t9, t5, st, img_store);
}

// ---- layout conversion ------------------------------------------------------
// file [NZS][RES][RES] -> z-fast [RES][RES][NZP], padding slices set to 0.
__global__ void __launch_bounds__(256) file_to_zfast_kernel(const DevGeom g, const float* __restrict__ in,
                                                            float* __restrict__ out) {
  __shared__ float T[32][33];
  const int x0 = blockIdx.x * 32, y = blockIdx.y, z0 = blockIdx.z * 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int RES = g.res;
  for (int j = w; j < 32; j += 8) {
    const int z = z0 + j, x = x0 + lane;
    T[j][lane] = (z < g.nzs && x < RES) ? in[((size_t)z * RES + y) * RES + x] : 0.f;
  }
  __syncthreads();
  for (int i = w; i < 32; i += 8) {
    const int x = x0 + i;
    if (x < RES) out[((size_t)y * RES + x) * g.nzp + z0 + lane] = T[lane][i];
  }
}

cudaError_t launch_file_to_zfast(const DevGeom& g, const float* in, float* out, cudaStream_t st) {
  dim3 grid((g.res + 31) / 32, g.res, g.nzp / 32);
  file_to_zfast_kernel<<<grid, 256, 0, st>>>(g, in, out);
  return cudaGetLastError();
}

// z-fast -> file layout; with mask, the output scaling and the radius mask of
// GFIRST.cu:532-549.
template <class T>
__global__ void __launch_bounds__(256) zfast_to_file_kernel(const DevGeom g, const T* __restrict__ in,
                                                            float scale, int mask, float* __restrict__ out) {
  __shared__ float Tt[32][33];
  const int x0 = blockIdx.x * 32, y = blockIdx.y, z0 = blockIdx.z * 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int RES = g.res;
  for (int i = w; i < 32; i += 8) {
    const int x = x0 + i;
    Tt[i][lane] = (x < RES) ? img_ld(in + ((size_t)y * RES + x) * g.nzp + z0 + lane) : 0.f;
  }
  __syncthreads();
  const int RESM = RES / 2;
  for (int j = w; j < 32; j += 8) {
    const int z = z0 + j, x = x0 + lane;
    if (z >= g.nzs || x >= RES) continue;
    float v = Tt[lane][j];
    if (mask) {
      const float dist = (float)((x - RESM) * (x - RESM) + (y - RESM) * (y - RESM) - (RESM - 1) * (RESM - 1));
      v = (dist > 0.f) ? 0.f : __fmul_rn(v, scale);
    }
    out[((size_t)z * RES + y) * RES + x] = v;
  }
}

cudaError_t launch_zfast_to_file(const DevGeom& g, const void* in, float scale, int mask, float* out,
                                 cudaStream_t st, int in_store) {
  dim3 grid((g.res + 31) / 32, g.res, g.nzp / 32);
  switch (in_store) {
    case 0: zfast_to_file_kernel<<<grid, 256, 0, st>>>(g, static_cast<const float*>(in), scale, mask, out); break;
    case 1: zfast_to_file_kernel<<<grid, 256, 0, st>>>(g, static_cast<const __half*>(in), scale, mask, out); break;
    case 2:
      zfast_to_file_kernel<<<grid, 256, 0, st>>>(g, static_cast<const __nv_bfloat16*>(in), scale, mask, out);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// CreateInitialCylinder, GFIRST_CPU_Kernels.cpp:35-56, z-fast.
template <class T>
__global__ void cylinder_kernel(const DevGeom g, float val, T* out) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t n = (size_t)g.res * g.res * g.nzp;
  if (i >= n) return;
  const int z = (int)(i % g.nzp);
  const int colidx = (int)(i / g.nzp);
  const int y = colidx / g.res, x = colidx - y * g.res;
  const int h = g.res / 2;
  const long long r2 = (long long)(x - h) * (x - h) + (long long)(y - h) * (y - h);
  img_st(out + i, (z < g.nzs && r2 <= (long long)h * h) ? val : 0.f);
}

cudaError_t launch_cylinder(const DevGeom& g, float val, void* out, cudaStream_t st, int out_store) {
  const size_t n = (size_t)g.res * g.res * g.nzp;
  const unsigned nb = (unsigned)((n + 255) / 256);
  switch (out_store) {
    case 0: cylinder_kernel<<<nb, 256, 0, st>>>(g, val, static_cast<float*>(out)); break;
    case 1: cylinder_kernel<<<nb, 256, 0, st>>>(g, val, static_cast<__half*>(out)); break;
    case 2: cylinder_kernel<<<nb, 256, 0, st>>>(g, val, static_cast<__nv_bfloat16*>(out)); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// max(0, max over the image), GFIRST.cu:515, 521.  d_max must hold 0 before.
// A maximum is exact in any precision: the reference's host loop and this
// reduction give the same float.
template <class T>
__global__ void max_nonneg_kernel(const DevGeom g, const T* __restrict__ img, float* d_max) {
  const size_t n = (size_t)g.res * g.res * g.nzp;
  float m = 0.f;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float v = img_ld(img + i);
    if (v > m) m = v;
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(reinterpret_cast<int*>(d_max), __float_as_int(m));
}

cudaError_t launch_max_nonneg(const DevGeom& g, const void* img, float* d_max, cudaStream_t st, int store) {
  cudaError_t e = cudaMemsetAsync(d_max, 0, sizeof(float), st);
  if (e != cudaSuccess) return e;
  switch (store) {
    case 0: max_nonneg_kernel<<<304, 256, 0, st>>>(g, static_cast<const float*>(img), d_max); break;
    case 1: max_nonneg_kernel<<<304, 256, 0, st>>>(g, static_cast<const __half*>(img), d_max); break;
    case 2: max_nonneg_kernel<<<304, 256, 0, st>>>(g, static_cast<const __nv_bfloat16*>(img), d_max); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---- joint bilateral filter, GFIRST_GPU_Kernels.cu:508-539 ---------------
// CTA: 4x4 columns x 32 slices, reference and input staged with a halo of 4.
// Voxels with a coordinate below r give 0 (the reference's unsigned window
// start wraps and its loops run zero times).  Spatial weights come from a
// table computed on the host exactly as the reference computes them
// (double exp, stored as float); the intensity weight uses __expf in FP32
// (the reference evaluates it in double) and the intensity difference is
// scaled by 1/max_ref.
constexpr int BL_T = 4, BL_H = 4;
template <class T>
__global__ void __launch_bounds__(512) bilateral_kernel(const DevGeom g, const T* __restrict__ in,
                                                        const T* __restrict__ ref,
                                                        const float* __restrict__ d_max_ref, float max_ref_host,
                                                        int r, float neg_inv_ci, const float* __restrict__ gtab,
                                                        float* __restrict__ out) {
  constexpr int W = BL_T + 2 * BL_H;  // 12 columns
  constexpr int ZW = 32 + 2 * BL_H;   // 40 slices
  __shared__ float Sr[W][W][ZW + 1];
  __shared__ float Si[W][W][ZW + 1];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int x0 = blockIdx.x * BL_T, y0 = blockIdx.y * BL_T, z0 = blockIdx.z * 32;
  const int RES = g.res, NZS = g.nzs, NZP = g.nzp;
  for (int idx = threadIdx.x; idx < W * W * ZW; idx += blockDim.x) {
    const int zz = idx % ZW, c = idx / ZW;
    const int yy = c / W, xx = c % W;
    const int y = y0 - BL_H + yy, x = x0 - BL_H + xx, z = z0 - BL_H + zz;
    float vr = 0.f, vi = 0.f;
    if (y >= 0 && y < RES && x >= 0 && x < RES && z >= 0 && z < NZS) {
      const size_t o = ((size_t)y * RES + x) * NZP + z;
      vr = img_ld(ref + o);
      vi = img_ld(in + o);
    }
    Sr[yy][xx][zz] = vr;
    Si[yy][xx][zz] = vi;
  }
  __syncthreads();
  const int ty = wid >> 2, tx = wid & 3;
  const int y = y0 + ty, x = x0 + tx, z = z0 + lane;
  if (y >= RES || x >= RES) return;
  const float max_ref = d_max_ref ? *d_max_ref : max_ref_host;
  const float rinv = 1.0f / max_ref;
  float res = 0.f;
  if (z < NZS && x >= r && y >= r && z >= r) {
    const float ref0 = Sr[ty + BL_H][tx + BL_H][lane + BL_H];
    float norm = 0.f, sum = 0.f;
    for (int dz = -r; dz <= r; dz++) {
      if (z + dz >= NZS) break;
      for (int dy = -r; dy <= r; dy++) {
        if (y + dy >= RES) break;
        const float* rr = &Sr[ty + BL_H + dy][tx + BL_H][lane + BL_H + dz];
        const float* ii = &Si[ty + BL_H + dy][tx + BL_H][lane + BL_H + dz];
        const float* gw = gtab + ((dz + 4) * 9 + (dy + 4)) * 9 + 4;
        for (int dx = -r; dx <= r; dx++) {
          if (x + dx >= RES) break;
          const float d = __fmul_rn(__fsub_rn(rr[dx * (ZW + 1)], ref0), rinv);
          const float h = __expf(__fmul_rn(__fmul_rn(d, d), neg_inv_ci));
          const float w = __fmul_rn(h, __ldg(gw + dx));
          norm = __fadd_rn(norm, w);
          sum = __fadd_rn(sum, __fmul_rn(w, ii[dx * (ZW + 1)]));
        }
      }
    }
    res = ((double)norm > 1e-8) ? __fdiv_rn(sum, norm) : 0.f;
  }
  out[((size_t)y * RES + x) * NZP + z] = (z < NZS) ? res : 0.f;
}

cudaError_t launch_bilateral(const DevGeom& g, const void* in, const void* ref, const float* d_max_ref,
                             float max_ref, int r, float sigmai, const float* gtab, float* out, cudaStream_t st,
                             int store) {
  if (r < 0 || r > BL_H) return cudaErrorInvalidValue;
  const double ci = (2.0 * (double)sigmai) * (2.0 * (double)sigmai);
  const float neg_inv_ci = (float)(-1.0 / ci);
  dim3 grid((g.res + BL_T - 1) / BL_T, (g.res + BL_T - 1) / BL_T, g.nzp / 32);
  switch (store) {
#define GF_BL(S, T)                                                                                        \
  case S:                                                                                                  \
    bilateral_kernel<<<grid, 512, 0, st>>>(g, static_cast<const T*>(in), static_cast<const T*>(ref),     \
                                           d_max_ref, max_ref, r, neg_inv_ci, gtab, out);                 \
    break;
    GF_BL(0, float) GF_BL(1, __half) GF_BL(2, __nv_bfloat16)
#undef GF_BL
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// img2 = (1.0 - 0.1f)*img2 + 0.1f*filtered, GFIRST.cu:524 (double, as there).
template <class T>
__global__ void blend_kernel(size_t n, T* img2, const float* __restrict__ filt) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float fc = 0.1f;
  img_st(img2 + i,
         (float)(__dadd_rn(__dmul_rn(1.0 - (double)fc, (double)img_ld(img2 + i)), (double)__fmul_rn(fc, filt[i]))));
}

cudaError_t launch_blend(const DevGeom& g, void* img2, const float* filt, cudaStream_t st, int store) {
  const size_t n = (size_t)g.res * g.res * g.nzp;
  const unsigned nb = (unsigned)((n + 255) / 256);
  switch (store) {
    case 0: blend_kernel<<<nb, 256, 0, st>>>(n, static_cast<float*>(img2), filt); break;
    case 1: blend_kernel<<<nb, 256, 0, st>>>(n, static_cast<__half*>(img2), filt); break;
    case 2: blend_kernel<<<nb, 256, 0, st>>>(n, static_cast<__nv_bfloat16*>(img2), filt); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace gf
