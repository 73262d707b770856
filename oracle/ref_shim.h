// ref_shim.h -- host emulation of the CUDA pieces GFIRST's sources use, so
// that the reference program (its kernels and its osem3d()/main() driver,
// extracted verbatim by oracle/build_ref.py) can be compiled with g++ and
// run on the CPU to produce golden outputs.
//
// TEST INFRASTRUCTURE ONLY; outputs go to oracle/_ref/ (git-ignored).
//
// What this file supplies (everything else comes from the reference):
//  - the compile-time geometry of GFIRST.h, from -DGFR_* macros;
//  - CUDA keywords, dim3, threadIdx/blockIdx (thread-local), __syncthreads
//    (a std::barrier when a kernel launch needs one);
//  - texture<float,3> + tex3D: unnormalized coordinates, clamp addressing,
//    linear filtering with exact FP32 weights, each 1-D interpolation as
//    fma(w, b-a, a) -- the same rule as oracle/gf_oracle.c.  With
//    -DGFR_TEX8 the weights are rounded to 8 fractional bits instead, as the
//    CUDA Programming Guide's texture-fetch appendix describes the hardware.
//  - the runtime calls (cudaMalloc/cudaMemcpy/... on host memory) and the
//    host launch wrappers, with the launch shapes of
//    GFIRST_GPU_Kernels.cu:105-107, 166-171, 184-188, 214-219, 360-364,
//    540-543 and the array set-up of :221-281.
#pragma once
#include <barrier>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <thread>
#include <vector>

// ---- geometry (GFIRST.h:1-36) ----
static const float PI = 3.1415926f;
static const int NTBINS = 1;
static const int NRAD = GFR_NRAD;
static const int NANG = GFR_NANG;
static const int SPAN = GFR_SPAN;
static const int NSINOGS = GFR_NSINOGS;
static const int NSEGMENTS = GFR_NSEG;
static const int NDATA = NSINOGS * NANG * NRAD;
static const int RES = GFR_RES;
static const int NZS = GFR_NZS;
static const int NVOXELS = RES * RES * NZS;
static const int NPT = RES;
static const int NZSM = NZS / 2 - 1;
const int NITER = GFR_NITER;
const int NSUBSETS = 1;
const int Nav = 1;
const int NDATA_PART = NZS * NRAD;
float PSF_FW = 1.5;
float PSF_BW = 1.5;
float scale_D = 3.70e-4 * 162.0;
float scale_T = 3.70e-4 * 162.0;
static const float pitch = GFR_PITCH;
static const float DIAM_DET = GFR_DIAM;
static const float FOV = GFR_FOV;
static const float TOF_FOV = GFR_FOV;

// ---- allocation: zero-filled, with slack so that the reference's reads and
// writes one element past an array (gaussian_filterZ) land in zeros ----
static void* gfref_malloc(size_t n) { return calloc(n + 4096, 1); }
#define malloc(n) gfref_malloc(n)

// ---- CUDA keywords and thread indices ----
#define __global__
#define __device__
#define __constant__
#define __host__
#define __shared__ static
struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
static thread_local dim3 threadIdx, blockIdx, blockDim, gridDim;
static thread_local std::barrier<>* gfref_bar = nullptr;
static inline void __syncthreads() {
  if (gfref_bar) gfref_bar->arrive_and_wait();
}

// ---- runtime ----
typedef int cudaError;
typedef int cudaError_t;
static const int cudaSuccess = 0;
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
static inline cudaError cudaGetLastError() { return cudaSuccess; }
static inline cudaError cudaThreadSynchronize() { return cudaSuccess; }
static inline const char* cudaGetErrorString(cudaError) { return "no error"; }
static inline cudaError cudaMalloc(void** p, size_t n) { *p = gfref_malloc(n); return cudaSuccess; }
static inline cudaError cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { memcpy(d, s, n); return cudaSuccess; }
#define cudaMemcpyToSymbol(sym, src, n) memcpy(&(sym), (src), (n))

// ---- textures ----
enum cudaTextureAddressMode { cudaAddressModeWrap, cudaAddressModeClamp };
enum cudaTextureFilterMode { cudaFilterModePoint, cudaFilterModeLinear };
template <class T, int D>
struct texture {
  int normalized = 0;
  cudaTextureFilterMode filterMode = cudaFilterModePoint;
  cudaTextureAddressMode addressMode[3] = {cudaAddressModeClamp, cudaAddressModeClamp, cudaAddressModeClamp};
  std::vector<float> data;
  int w = 0, h = 0, d = 0;
};
static inline int gfref_clamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline float gfref_w(float w) {
#ifdef GFR_TEX8
  return floorf(w * 256.0f + 0.5f) / 256.0f;
#else
  return w;
#endif
}
static inline float gfref_lerp(float a, float b, float w) { return fmaf(gfref_w(w), b - a, a); }
static float tex3D(const texture<float, 3>& t, float x, float y, float z) {
  float xb = x - 0.5f, yb = y - 0.5f, zb = z - 0.5f;
  float fx = floorf(xb), fy = floorf(yb), fz = floorf(zb);
  float a = xb - fx, b = yb - fy, c = zb - fz;
  int i = (int)fx, j = (int)fy, k = (int)fz;
  int i0 = gfref_clamp(i, 0, t.w - 1), i1 = gfref_clamp(i + 1, 0, t.w - 1);
  int j0 = gfref_clamp(j, 0, t.h - 1), j1 = gfref_clamp(j + 1, 0, t.h - 1);
  int k0 = gfref_clamp(k, 0, t.d - 1), k1 = gfref_clamp(k + 1, 0, t.d - 1);
  auto T = [&](int ii, int jj, int kk) { return t.data[((size_t)kk * t.h + jj) * t.w + ii]; };
  float v0 = gfref_lerp(gfref_lerp(T(i0, j0, k0), T(i1, j0, k0), a), gfref_lerp(T(i0, j1, k0), T(i1, j1, k0), a), b);
  float v1 = gfref_lerp(gfref_lerp(T(i0, j0, k1), T(i1, j0, k1), a), gfref_lerp(T(i0, j1, k1), T(i1, j1, k1), a), b);
  return gfref_lerp(v0, v1, c);
}

// File-scope objects of GFIRST_GPU_Kernels.cu:28-38.
const int BSX = 256;
float d_G1D[9];
texture<float, 3> imgEstTex;
texture<float, 3> CorrTex;
texture<float, 3> CalibTex;

// ---- kernel launch emulation ----
template <class F>
static void gfref_launch(dim3 grid, dim3 block, F body) {
  int nb = (int)(grid.x * grid.y * grid.z);
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < nb; b++) {
    gridDim = grid;
    blockDim = block;
    blockIdx = dim3(b % grid.x, (b / grid.x) % grid.y, b / (grid.x * grid.y));
    for (unsigned tz = 0; tz < block.z; tz++)
      for (unsigned ty = 0; ty < block.y; ty++)
        for (unsigned tx = 0; tx < block.x; tx++) {
          threadIdx = dim3(tx, ty, tz);
          body();
        }
  }
}
// For kernels that synchronize inside a block: one OS thread per CUDA thread.
template <class F>
static void gfref_launch_sync(dim3 grid, dim3 block, F body) {
  int nb = (int)(grid.x * grid.y * grid.z);
  int nt = (int)(block.x * block.y * block.z);
  for (int b = 0; b < nb; b++) {
    std::barrier<> bar(nt);
    dim3 bi(b % grid.x, (b / grid.x) % grid.y, b / (grid.x * grid.y));
    std::vector<std::thread> th;
    th.reserve(nt);
    for (int t = 0; t < nt; t++)
      th.emplace_back([&, t] {
        gridDim = grid;
        blockDim = block;
        blockIdx = bi;
        threadIdx = dim3(t % block.x, (t / block.x) % block.y, t / (block.x * block.y));
        gfref_bar = &bar;
        body();
        gfref_bar = nullptr;
      });
    for (auto& x : th) x.join();
  }
}
