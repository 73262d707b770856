// ref_gpu_shim.cuh -- builds the reference program's own GPU path with the
// CUDA 13 toolkit for sm_103a: its kernels, its host launch wrappers and
// texture set-up (GFIRST_GPU_Kernels.cu), its osem3d()/main() driver
// (GFIRST.cu) and the CPU routines they call (GFIRST_CPU_Kernels.cpp), all
// extracted verbatim by oracle/build_ref.py into oracle/_ref/ (git-ignored,
// never committed).  The result is a baseline of the reference's GPU design
// -- one launch per (segment, angle) view, the host scatter/gather and the
// texture uploads between them -- on the same GPU as this library.
//
// TEST INFRASTRUCTURE ONLY: timed by `bench.py --impl reference-shim`,
// never part of the library.
//
// What this file supplies (everything else is the reference's code):
//  - the compile-time geometry of GFIRST.h, from -DGFR_* macros;
//  - the file-scope objects of GFIRST_GPU_Kernels.cu:24-38;
//  - the legacy texture-reference API the reference is written against
//    (removed in CUDA 12): texture<T, D> is a host struct holding the fields
//    the reference sets (normalized, filterMode, addressMode);
//    cudaBindTextureToArray(tex, array, desc) creates a texture object over
//    the cudaArray with those fields and stores it in the __constant__
//    variable tex_dev; tex3D(tex, x, y, z) in device code reads through
//    tex_dev.  Later cudaMemcpy3D uploads into the array are seen through the
//    same object, as they were through the bound reference.
//  - cudaThreadSynchronize (removed) as cudaDeviceSynchronize.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>

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
__device__ __constant__ float pitch = GFR_PITCH;
__device__ __constant__ float DIAM_DET = GFR_DIAM;
__device__ __constant__ float FOV = GFR_FOV;
__device__ __constant__ float TOF_FOV = GFR_FOV;

// ---- legacy texture references on texture objects ----
template <class T, int D>
struct texture {
  int normalized = 0;
  cudaTextureFilterMode filterMode = cudaFilterModePoint;
  cudaTextureAddressMode addressMode[3] = {cudaAddressModeClamp, cudaAddressModeClamp, cudaAddressModeClamp};
};

template <class T, int D, class Store>
static cudaError_t gfrg_bind(const texture<T, D>& t, cudaArray_t a, Store store) {
  cudaResourceDesc rd;
  memset(&rd, 0, sizeof(rd));
  rd.resType = cudaResourceTypeArray;
  rd.res.array.array = a;
  cudaTextureDesc td;
  memset(&td, 0, sizeof(td));
  td.normalizedCoords = t.normalized;
  td.filterMode = t.filterMode;
  td.readMode = cudaReadModeElementType;
  for (int i = 0; i < 3; i++) td.addressMode[i] = t.addressMode[i];
  cudaTextureObject_t o = 0;
  cudaError_t e = cudaCreateTextureObject(&o, &rd, &td, nullptr);
  if (e != cudaSuccess) {
    fprintf(stderr, "texture object: %s\n", cudaGetErrorString(e));
    exit(1);
  }
  return store(o);
}

#define cudaBindTextureToArray(t, a, desc) \
  gfrg_bind(t, a, [&](cudaTextureObject_t o_) { return cudaMemcpyToSymbol(t##_dev, &o_, sizeof(o_)); })
#define tex3D(t, x, y, z) ::tex3D<float>(t##_dev, x, y, z)
#define cudaThreadSynchronize cudaDeviceSynchronize

// ---- file-scope objects of GFIRST_GPU_Kernels.cu:24-38 ----
#define BLOCK_W 8
#define BLOCK_H 8
const int BSX = 256;
__constant__ float d_G1D[9];
texture<float, 3> imgEstTex;
__constant__ cudaTextureObject_t imgEstTex_dev;
cudaArray* array3dImg = 0;
texture<float, 3> CorrTex;
__constant__ cudaTextureObject_t CorrTex_dev;
cudaArray* array3dCorr = 0;
texture<float, 3> CalibTex;
__constant__ cudaTextureObject_t CalibTex_dev;
cudaArray* array3dCalib = 0;
