// gf_fp.cu -- forward projector with the fused data/projection ratio.
//
// Reference: FORWPROJ_K (GFIRST_GPU_Kernels.cu:40-102), one launch per
// (segment, angle) view with a blocking copy and a host scatter per launch
// (GFIRST.cu:346-365), then the ratio loop of GFIRST.cu:413-430.
//
// GB300 design.  One CTA owns one (angle, radial bin) pair: every ray of that
// pair, across all segments and planes, is parallel and shares the in-plane
// sample positions (x, y) of each step lambda; only z differs.  So the CTA
//  (1) resamples the image once per step onto a z column, B[lambda][z] =
//      bilinear_xy(image[z], x(lambda), y(lambda)), reading the four z-fast
//      image columns around (x, y) with coalesced loads (image in L2);
//  (2) sums every ray of the pair from shared memory: ray (segment, plane
//      iz0) at step lambda needs B[lambda] at z = iz0 + lambda*dz, a 1-D
//      interpolation whose integer offset and fraction are the same for all
//      planes of a segment, so a thread walks a run of R consecutive planes
//      with R+1 shared loads and R interpolations per step;
//  (3) applies the ratio in the epilogue and writes (corr, calib) pairs
//      contiguously in the radial-major layout the back projector reads.
// Work per ray-sample is one shared load and one 1-D interpolation instead of
// eight texel reads; the image and data stream from HBM once.
#include "gf_kernels.h"

namespace gf {

template <int R, bool RATIO, bool FULL, int STORE>
__global__ void __launch_bounds__(512) fp_kernel(const FpArgs a) {
  using Pair = typename PairT<STORE>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int lc = a.lc, cw = a.cw;
  int4* offs = reinterpret_cast<int4*>(smraw);              // [lc]
  float2* wts = reinterpret_cast<float2*>(offs + lc);        // [lc]
  float* col = reinterpret_cast<float*>(wts + lc);           // [lc][cw]

  const DevGeom& g = a.g;
  const FpFrame& F = a.fr[blockIdx.z];
  const int ird = blockIdx.x, tl = blockIdx.y;
  // a frame with fewer angles in its subset than the launch's largest: its
  // surplus blocks march no rays and write nothing (an early return here
  // costs the kernel 13 registers)
  const bool active = tl < F.na;
  const int lam_end = active ? g.lam1 : g.lam0 - 1;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int theta = subset_angle(F.subset, F.nsub, active ? tl : 0);
  const float2 sc = g.trig[theta];
  const float sn = sc.x, cs = sc.y;
  // GFIRST_GPU_Kernels.cu:79-87 (fac = RES/NPT = 1 makes dx = sin, dy = -cos exactly)
  const float x0 = __fmul_rn(g.fx_fp, __fsub_rn((float)ird, g.radm));
  const float xc = __fadd_rn(__fadd_rn(g.resm, __fmul_rn(x0, cs)), 0.5f);
  const float yc = __fadd_rn(__fadd_rn(g.resm, __fmul_rn(x0, sn)), 0.5f);
  const float dx = sn, dy = -cs;
  const int RES = g.res, NZS = g.nzs, NZP = g.nzp;

  int4 run = make_int4(-1, 0, 0, 0);
  if (tid < a.nruns) run = a.runs[tid];
  float dz = 0.f;
  int zbase = 0;
  if (run.x >= 0) {
    dz = g.seg[run.x].dz;
    zbase = a.padl + run.y;
  }
  float acc[R];
#pragma unroll
  for (int j = 0; j < R; j++) acc[j] = 0.f;

  const int npad = cw - NZS;
  for (int lb = g.lam0; lb <= lam_end; lb += lc) {
    const int nl = min(lc, g.lam1 - lb + 1);
    for (int l = tid; l < nl; l += nt) {
      const float fl = (float)(lb + l);
      const float x = __fadd_rn(xc, __fmul_rn(fl, dx));
      const float y = __fadd_rn(yc, __fmul_rn(fl, dy));
      const float xb = __fsub_rn(x, 0.5f), yb = __fsub_rn(y, 0.5f);
      const float fx = floorf(xb), fy = floorf(yb);
      const int i = (int)fx, j = (int)fy;
      const int i0 = clampi(i, 0, RES - 1), i1 = clampi(i + 1, 0, RES - 1);
      const int j0 = clampi(j, 0, RES - 1), j1 = clampi(j + 1, 0, RES - 1);
      offs[l] = make_int4((j0 * RES + i0) * NZP, (j0 * RES + i1) * NZP, (j1 * RES + i0) * NZP, (j1 * RES + i1) * NZP);
      wts[l] = make_float2(__fsub_rn(xb, fx), __fsub_rn(yb, fy));
    }
    __syncthreads();
    for (int idx = tid; idx < nl * NZP; idx += nt) {
      const int l = idx / NZP, z = idx - l * NZP;
      if (z < NZS) {
        const int4 o = offs[l];
        const float2 w = wts[l];
        const float v00 = __ldg(F.img + o.x + z), v10 = __ldg(F.img + o.y + z);
        const float v01 = __ldg(F.img + o.z + z), v11 = __ldg(F.img + o.w + z);
        col[l * cw + a.padl + z] = lerp_rn(lerp_rn(v00, v10, w.x), lerp_rn(v01, v11, w.x), w.y);
      }
    }
    __syncthreads();
    if (npad > 0) {
      for (int idx = tid; idx < nl * npad; idx += nt) {
        const int l = idx / npad, p = idx - l * npad;
        float* c = col + l * cw;
        if (p < a.padl) c[p] = c[a.padl];
        else c[a.padl + NZS + (p - a.padl)] = c[a.padl + NZS - 1];
      }
      __syncthreads();
    }
    if (run.x >= 0) {
      for (int l = 0; l < nl; l++) {
        const float t = __fmul_rn((float)(lb + l), dz);
        const float mf = floorf(t);
        const float f = __fsub_rn(t, mf);
        const float* c = col + l * cw + zbase + (int)mf;
        float va = c[0];
#pragma unroll
        for (int j = 0; j < R; j++) {
          const float vb = c[j + 1];
          acc[j] += lerp_rn(va, vb, f);
          va = vb;
        }
      }
    }
    __syncthreads();
  }

  if (run.x < 0 || !active) return;
  const DevSeg sg = g.seg[run.x];
  const size_t base = ((size_t)tl * g.nrad + ird) * g.PS;
  const float2 sentinel = make_float2(-1000.f, -1000.f);
#pragma unroll
  for (int j = 0; j < R; j++) {
    if (j < run.z) {
      const int iz0 = run.y + j;
      const float proj = acc[j];
      if (FULL) {
        const size_t lor = ((size_t)(iz0 - sg.zmin) + sg.acc) * ((size_t)g.nrad * g.nang) + (size_t)theta * g.nrad + ird;
        F.proj_full[lor] = proj;
      }
      if (RATIO) {
        const size_t o = base + sg.blk + 1 + (iz0 - sg.zmin);
        const float2 db = F.dbg[o];
        const float s = __fadd_rn(proj, db.y);
        const float corr = (s >= 0.01f) ? __fdiv_rn(db.x, s) : -1000.f;
        Pair* cc_out = static_cast<Pair*>(F.corrcal);
        const Pair cc = pair_from<Pair>(make_float2(corr, F.cal[o]));
        cc_out[o] = cc;
        if (j == 0 && (run.w & 1)) cc_out[o - 1] = (run.x == 0) ? cc : pair_from<Pair>(sentinel);
        if (j == run.z - 1 && (run.w & 2)) cc_out[o + 1] = (run.x == 0) ? cc : pair_from<Pair>(sentinel);
      }
    }
  }
}

template <int R, bool RATIO, bool FULL, int STORE>
static cudaError_t launch_fp_t(const FpArgs& a, const FpSchedule& s, cudaStream_t st) {
  auto k = fp_kernel<R, RATIO, FULL, STORE>;
  size_t smem = s.smem_bytes();
  cudaError_t e = allow_max_smem(k);
  if (e != cudaSuccess) return e;
  int na = 0;
  for (int f = 0; f < (a.nfr > 1 ? a.nfr : 1); f++) na = a.fr[f].na > na ? a.fr[f].na : na;
  dim3 grid(a.g.nrad, na, a.nfr > 1 ? a.nfr : 1);
  k<<<grid, s.nthreads, smem, st>>>(a);
  return cudaGetLastError();
}

template <int R>
static cudaError_t launch_fp_r(const FpArgs& a, const FpSchedule& s, cudaStream_t st) {
  if (!a.fr[0].corrcal) return launch_fp_t<R, false, true, 0>(a, s, st);
  switch (a.storage) {
    case 0:
      return a.fr[0].proj_full ? launch_fp_t<R, true, true, 0>(a, s, st) : launch_fp_t<R, true, false, 0>(a, s, st);
    case 1: return launch_fp_t<R, true, false, 1>(a, s, st);
    case 2: return launch_fp_t<R, true, false, 2>(a, s, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_fp(const FpArgs& a, const FpSchedule& s, cudaStream_t st) {
  if (a.nfr < 0 || a.nfr > kMaxFrames) return cudaErrorInvalidValue;
  // every frame of a launch has the outputs of frame 0 (one kernel variant)
  for (int f = 0; f < (a.nfr > 1 ? a.nfr : 1); f++) {
    const FpFrame& F = a.fr[f];
    if (!F.img || (!F.corrcal && !F.proj_full)) return cudaErrorInvalidValue;
    if (!F.corrcal != !a.fr[0].corrcal || !F.proj_full != !a.fr[0].proj_full) return cudaErrorInvalidValue;
    if (F.corrcal && (!F.dbg || !F.cal)) return cudaErrorInvalidValue;
    // the subset's angles: subset + l*nsub for l < na, all inside [0, nang)
    if (F.nsub < 1 || F.subset < 0 || F.subset >= F.nsub || F.na < 1 ||
        F.na != (a.g.nang - F.subset + F.nsub - 1) / F.nsub)
      return cudaErrorInvalidValue;
  }
  if (a.fr[0].corrcal && a.fr[0].proj_full && a.storage != 0) return cudaErrorInvalidValue;
  switch (s.R) {
    case 9: return launch_fp_r<9>(a, s, st);
    case 17: return launch_fp_r<17>(a, s, st);
    case 25: return launch_fp_r<25>(a, s, st);
    case 33: return launch_fp_r<33>(a, s, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace gf
