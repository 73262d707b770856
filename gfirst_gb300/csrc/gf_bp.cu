// gf_bp.cu -- voxel-driven back projector.
//
// Reference: BACKWPROJ_K (GFIRST_GPU_Kernels.cu:109-164), one launch per
// (segment, angle) view, each reading-modifying-writing the whole NUMER and
// DENOM volumes, after two host->device texture uploads and followed by a
// device synchronisation (GFIRST.cu:436-469).
//
// GB300 design.  One warp owns one image column (x, y); lane l holds voxels
// z = l, l+32, ... in registers for the whole subset, so NUMER/DENOM are
// written once per sub-iteration instead of read and written per view.  For a
// column and angle the radial bilinear coordinate is fixed; it is computed
// once per angle into shared memory.  The views are visited in the
// reference's order (segments outer, angles inner) and every coordinate is
// computed with the reference's rounding, so each voxel's sums are the
// reference's sums bit for bit.  The (corr, calib) pairs of a view sit in
// radial-major rows, so the 32 lanes of a warp (consecutive z, hence
// consecutive rows) read contiguous 8-byte pairs; the padded rows around each
// segment stand in for the clamp / -1000 texels at the plane-range edges.
#include "gf_kernels.h"

namespace gf {

template <int Q>
__global__ void __launch_bounds__(256) bp_kernel(const BpArgs a) {
  extern __shared__ int4 bcache[];  // [warps per block][na]
  const DevGeom& g = a.g;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int colidx = blockIdx.x * (blockDim.x >> 5) + wib;
  if (colidx >= g.res * g.res) return;  // whole warp
  const int iy = colidx / g.res, ix = colidx - iy * g.res;
  int4* my = bcache + wib * a.na;

  // GFIRST_GPU_Kernels.cu:136-147
  const float xv = __fsub_rn((float)ix, g.resm), yv = __fsub_rn((float)iy, g.resm);
  for (int tl = lane; tl < a.na; tl += 32) {
    const float2 sc = g.trig[subset_angle(g, a.subset, tl)];
    const float xrot = __fadd_rn(__fmul_rn(xv, sc.y), __fmul_rn(yv, sc.x));
    const float yrot = __fadd_rn(__fmul_rn(-xv, sc.x), __fmul_rn(yv, sc.y));
    const float x = __fadd_rn(__fadd_rn(g.radm, __fmul_rn(xrot, g.fx_bp)), 0.5f);
    const float xb = __fsub_rn(x, 0.5f);
    const float fl = floorf(xb);
    const int i = (int)fl;
    const int i0 = clampi(i, 0, g.nrad - 1), i1 = clampi(i + 1, 0, g.nrad - 1);
    const int rb = tl * g.nrad;
    my[tl] = make_int4((rb + i0) * g.PS, (rb + i1) * g.PS, __float_as_int(__fsub_rn(xb, fl)), __float_as_int(yrot));
  }
  __syncwarp();

  float na[Q], da[Q];
#pragma unroll
  for (int q = 0; q < Q; q++) na[q] = da[q] = 0.f;

  for (int s = 0; s < g.nseg; s++) {
    const DevSeg sg = g.seg[s];
    const float zlo = (float)sg.zmin, zhi = (float)(g.nzs - sg.zmin);
    const int roff = sg.blk + 1 - sg.zmin;
    for (int tl = 0; tl < a.na; tl++) {
      const int4 e = my[tl];
      const float al = __int_as_float(e.z);
      const float t = __fmul_rn(__int_as_float(e.w), sg.fz);  // yrot*fz
      const float2* p0 = a.corrcal + e.x + roff;
      const float2* p1 = a.corrcal + e.y + roff;
#pragma unroll
      for (int q = 0; q < Q; q++) {
        const int iz = lane + 32 * q;
        // z = float(iz) + yrot*fz + 0.5f, GFIRST_GPU_Kernels.cu:148
        const float z = __fadd_rn(__fadd_rn((float)iz, t), 0.5f);
        if (iz < g.nzs && z >= zlo && z < zhi) {
          const float zb = __fsub_rn(z, 0.5f);
          const float fz = floorf(zb);
          const int j = (int)fz;
          const float be = __fsub_rn(zb, fz);
          const float2 t00 = __ldg(p0 + j), t10 = __ldg(p1 + j);
          const float2 t01 = __ldg(p0 + j + 1), t11 = __ldg(p1 + j + 1);
          const float c = lerp_rn(lerp_rn(t00.x, t10.x, al), lerp_rn(t01.x, t11.x, al), be);
          const float k = lerp_rn(lerp_rn(t00.y, t10.y, al), lerp_rn(t01.y, t11.y, al), be);
          // GFIRST_GPU_Kernels.cu:157: a negative interpolated value (a gap) zeroes both
          if (!(k < 0.f || c < 0.f)) {
            na[q] = __fadd_rn(na[q], c);
            da[q] = __fadd_rn(da[q], k);
          }
        }
      }
    }
  }
  float* no = a.numer + (size_t)colidx * g.nzp;
  float* dO = a.denom + (size_t)colidx * g.nzp;
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int iz = lane + 32 * q;
    no[iz] = iz < g.nzs ? na[q] : 0.f;
    dO[iz] = iz < g.nzs ? da[q] : 0.f;
  }
}

cudaError_t launch_bp(const BpArgs& a, cudaStream_t st) {
  const int warps = 8;
  const int Q = a.g.nzp / 32;
  size_t smem = (size_t)warps * a.na * sizeof(int4);
  dim3 grid((a.g.res * a.g.res + warps - 1) / warps);
  void (*k)(BpArgs) = nullptr;
  switch (Q) {
    case 1: k = bp_kernel<1>; break;
    case 2: k = bp_kernel<2>; break;
    case 3: k = bp_kernel<3>; break;
    case 4: k = bp_kernel<4>; break;
    case 5: k = bp_kernel<5>; break;
    case 6: k = bp_kernel<6>; break;
    case 7: k = bp_kernel<7>; break;
    case 8: k = bp_kernel<8>; break;
    default: return cudaErrorInvalidValue;
  }
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k<<<grid, warps * 32, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace gf
