// gf_bp.cu -- voxel-driven back projector.
//
// Reference: BACKWPROJ_K (GFIRST_GPU_Kernels.cu:109-164), one launch per
// (segment, angle) view, each reading-modifying-writing the whole NUMER and
// DENOM volumes, after two host->device texture uploads and followed by a
// device synchronisation (GFIRST.cu:436-469).
//
// GB300 design.  One warp owns one image column (x, y); lane l holds voxels
// z = l, l+32, ... and their (NUMER, DENOM) pairs in registers for the whole
// subset, so the volumes (or, in a reconstruction, their update ratio) are
// written once per sub-iteration.  For a column
// and an angle the radial coordinate is fixed, so per (segment, angle) view:
//  (1) the warp interpolates every plane row of the view radially once
//      (lanes along rows: coalesced 8-byte (corr, calib) loads from the
//      radial-major layout) into warp-private shared memory;
//  (2) each voxel interpolates between two of those rows along z.
// That is one radial interpolation per row instead of two per voxel; lanes
// whose voxel lies outside the segment's plane range do no work.
// (corr, calib) are processed as packed FP32 pairs (sm_100+ f32x2 FMA/add/sub),
// each element rounded as the scalar operation would be.  Views are visited
// in the reference's order (segments outer, angles inner) with the
// reference's coordinate rounding, so every voxel's sums are the reference's
// sums bit for bit.
//
// Issue and latency: the per-chunk voxel work has no branch on other lanes
// (no vote), so the chunks' dependency chains interleave; lanes whose voxel
// lies outside the segment's range are predicated off.  The floor of the axial
// coordinate is taken with a round-down add of 1.5*2^23 instead of the
// conversion pipe.  The views of a segment run with the segment's row chunk
// count fixed at compile time (one switch per segment), so staging issues no
// instructions for chunks beyond the segment's rows; for a segment narrower
// than the column, a view's voxel work issues only the lane chunks that can
// hold its in-range voxels (voxel_window).  What keeps issue below peak is
// dependency latency, which resident warps hide, so up to 160 slices the
// kernel is held to 64 registers (eight 4-warp blocks per SM): the next view's
// rows are prefetched into registers during the current view's voxels, all
// of them for 16-bit pairs and the first three row chunks for FP32 pairs.
#include "gf_kernels.h"

namespace gf {

// A column's results: its (NUMER, DENOM) sums, padding slices 0; or, with
// `ratio`, the update ratio of the two alone in NUMER's buffer (padding
// slices 1, the ratio of zero sums).
template <int Q>
__device__ __forceinline__ void store_column(const BpFrame& F, int ratio, size_t cb, int lane, int nzs,
                                             const float2 (&acc)[Q]) {
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int iz = lane + 32 * q;
    if (ratio) {
      F.numer[cb + iz] = iz < nzs ? update_ratio(acc[q].x, acc[q].y) : 1.f;
    } else {
      F.numer[cb + iz] = iz < nzs ? acc[q].x : 0.f;
      F.denom[cb + iz] = iz < nzs ? acc[q].y : 0.f;
    }
  }
}

// a - b on packed pairs, each element rounded as the scalar subtraction
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  float2 c;
  asm("{\n\t.reg .b64 ra, rb, rc;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rc, ra, rb;\n\tmov.b64 {%0, %1}, rc;\n\t}"
      : "=f"(c.x), "=f"(c.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return c;
}

// a + w*(b - a), the reference texture unit's linear filter in exact FP32
__device__ __forceinline__ float2 lerp2(float2 a, float2 b, float2 w) { return __ffma2_rn(w, sub2(b, a), a); }

// The voxels of one view: each lane's voxels interpolate between two staged
// rows along z and add to their (NUMER, DENOM) sums.
template <int Q, int LO, int HI>
__device__ __forceinline__ void voxel_views(float2 (&acc)[Q], const float (&fiz)[Q], const float2* rows, float t,
                                            float zlo, float zhi, int zm1, int nzs, int lane) {
#pragma unroll
  for (int q = LO; q <= HI; q++) {
    // z = float(iz) + yrot*fz + 0.5f, GFIRST_GPU_Kernels.cu:148
    const float z = __fadd_rn(__fadd_rn(fiz[q], t), 0.5f);
    // every lane of chunks 0..Q-2 holds a voxel (NZP = NZS rounded up to 32)
    const bool in = (q < Q - 1 || lane + 32 * q < nzs) && z >= zlo && z < zhi;
    if (in) {
      const float zb = __fsub_rn(z, 0.5f);
      // floor(zb): zb + 1.5*2^23 rounded down holds it in the low mantissa
      // bits (|zb| < 2^22), so both the float and the integer come without
      // a conversion instruction
      const float y = __fadd_rd(zb, 12582912.0f);
      const float fz = __fsub_rn(y, 12582912.0f);
      const int j = (__float_as_int(y) - 0x4B400000) - zm1;
      const float be = __fsub_rn(zb, fz);
      const float2 v = lerp2(rows[j], rows[j + 1], make_float2(be, be));
      // GFIRST_GPU_Kernels.cu:157: a negative interpolated value (a gap) zeroes both
      if (!(v.y < 0.f || v.x < 0.f)) acc[q] = __fadd2_rn(acc[q], v);
    }
  }
}

// The voxels of one view for a segment whose rows fill NCH lane chunks.  Its
// in-range voxels (z = iz + t + 0.5 rounded, in [zlo, zhi), nzs - 2*zmin =
// nrow - 2 <= 32*NCH - 2 of them at most, consecutive in iz since the rounded
// z is monotone) lie in the NCH + 1 chunks from the chunk of
// izlo = floor(zlo - t - 1): izlo is at most two below the first in-range
// voxel, so the last one is at most 32*(izlo/32) + 31 + 2 + 32*NCH - 2.  When
// that window is narrower than the column, only its chunks issue (one
// compile-time instance per window start); the per-voxel range test stays.
template <int Q, int NCH>
__device__ __forceinline__ void voxel_window(float2 (&acc)[Q], const float (&fiz)[Q], const float2* rows, float t,
                                             float zlo, float zhi, int zm1, int nzs, int lane) {
  constexpr int W = NCH + 1;
  if constexpr (W >= Q) {
    voxel_views<Q, 0, Q - 1>(acc, fiz, rows, t, zlo, zhi, zm1, nzs, lane);
  } else {
    const int izlo = max(__float2int_rd(__fsub_rn(__fsub_rn(zlo, t), 1.0f)), 0);
    switch (min(izlo >> 5, Q - W)) {
#define GF_VW(L) \
  case L:        \
    if constexpr (L <= Q - W) voxel_views<Q, L, L + W - 1>(acc, fiz, rows, t, zlo, zhi, zm1, nzs, lane); \
    break;
      GF_VW(0) GF_VW(1) GF_VW(2) GF_VW(3) GF_VW(4) GF_VW(5) GF_VW(6)
#undef GF_VW
    }
  }
}

// The voxels of one view, per-view form: the axial fraction and the row
// offset of the view are shared by every voxel of the column (z = iz + t +
// 0.5 is taken without the per-voxel rounding, which moves a weight by at
// most one unit in the last place of iz + t), so lane chunk q reads staged
// rows rv[32q] and rv[32q + 1] at fixed offsets from one per-view pointer.
// Voxels outside the segment's plane range read sentinel rows (or a
// sentinel pad row with weight >= 1/2): their interpolated mask is negative
// and the gap rule skips them, as the reference's range test does.
template <int Q, int LO, int HI>
__device__ __forceinline__ void voxel_views_fast(float2 (&acc)[Q], const float2* rv, float2 be2) {
#pragma unroll
  for (int q = LO; q <= HI; q++) {
    const float2 v = lerp2(rv[32 * q], rv[32 * q + 1], be2);
    if (!(v.y < 0.f || v.x < 0.f)) acc[q] = __fadd2_rn(acc[q], v);
  }
}

// voxel_window for the per-view form (same lane-chunk window).
template <int Q, int NCH>
__device__ __forceinline__ void voxel_window_fast(float2 (&acc)[Q], const float2* rv, float2 be2, float t,
                                                  float zlo) {
  constexpr int W = NCH + 1;  // bp_fast_pads (gf_plan.cpp) sizes the sentinel rows for this window
  if constexpr (W >= Q) {
    voxel_views_fast<Q, 0, Q - 1>(acc, rv, be2);
  } else {
    const int izlo = max(__float2int_rd(__fsub_rn(__fsub_rn(zlo, t), 1.0f)), 0);
    switch (min(izlo >> 5, Q - W)) {
#define GF_VWF(L) \
  case L:         \
    if constexpr (L <= Q - W) voxel_views_fast<Q, L, L + W - 1>(acc, rv, be2); \
    break;
      GF_VWF(0) GF_VWF(1) GF_VWF(2) GF_VWF(3) GF_VWF(4) GF_VWF(5) GF_VWF(6)
#undef GF_VWF
    }
  }
}

// Row chunks of FP32 pairs loaded during the previous view (the rest load
// while staging), per back-projector form.
#ifndef GF_BP_VIEW_PF32
#define GF_BP_VIEW_PF32 4
#endif
template <bool FAST>
constexpr int bp_pf32 = FAST ? GF_BP_VIEW_PF32 : 3;

// One segment's views with its row chunk count NCH fixed at compile time, so
// the staging issues exactly the chunks the segment's rows occupy.
template <int Q, int NCH, bool FAST, class Pair>
__device__ __forceinline__ void segment_views(float2 (&acc)[Q], const float (&fiz)[Q], const Pair* cc,
                                              const int4* my, float2* rows, const DevSeg& sg, int na, int nzs,
                                              int lane) {
  const float zlo = (float)sg.zmin, zhi = (float)(nzs - sg.zmin);
  const int zm1 = sg.zmin - 1;
  const int nrow = sg.nplanes + 2;
  // The rows of view tl + 1 are loaded into the registers that view tl's rows
  // have just left, before view tl's voxels, so their latency overlaps that
  // work.  16-bit pairs prefetch every chunk within 64 registers.  FP32 pairs
  // prefetch their first three chunks and load the others while staging: that
  // fits 64 registers too, and the eighth resident block per SM hides more
  // than the exposed loads cost (1.294 ms; all chunks prefetched at 72
  // registers, seven blocks: 1.336 ms; at 80 registers, six blocks: 1.343 ms).
  {
    constexpr int PF = (sizeof(Pair) == 8 && NCH > bp_pf32<FAST>) ? bp_pf32<FAST> : NCH;
    Pair c0[PF], c1[PF];
    auto load = [&](const int4& e) {
      const Pair* p0 = cc + e.x + sg.blk;
      const Pair* p1 = cc + e.y + sg.blk;
#pragma unroll
      for (int k = 0; k < PF; k++) {
        const int r = lane + 32 * k;
        if (k < NCH - 1 || r < nrow) {
          c0[k] = __ldg(p0 + r);
          c1[k] = __ldg(p1 + r);
        }
      }
    };
    int4 e = my[0];
    load(e);
    for (int tl = 0; tl < na; tl++) {
      const float2 al2 = make_float2(__int_as_float(e.z), __int_as_float(e.z));
      const float t = __fmul_rn(__int_as_float(e.w), sg.fz);  // yrot*fz
      __syncwarp();  // every lane is done reading the previous view's rows
      const Pair* q0 = cc + e.x + sg.blk;
      const Pair* q1 = cc + e.y + sg.blk;
#pragma unroll
      for (int k = 0; k < NCH; k++) {
        const int r = lane + 32 * k;
        if (k < NCH - 1 || r < nrow) {
          if (k < PF) rows[r] = lerp2(pair_f(c0[k < PF ? k : 0]), pair_f(c1[k < PF ? k : 0]), al2);
          else rows[r] = lerp2(pair_f(__ldg(q0 + r)), pair_f(__ldg(q1 + r)), al2);
        }
      }
      __syncwarp();
      if (tl + 1 < na) {
        e = my[tl + 1];
        load(e);
      }
      if constexpr (FAST) {
        // z = iz + t + 0.5 lies between rows floor(t) + iz - zm1 and the next
        const float ft = floorf(t);
        const float be = __fsub_rn(t, ft);
        const float2* rv = rows + ((int)ft - zm1) + lane;
        voxel_window_fast<Q, NCH>(acc, rv, make_float2(be, be), t, zlo);
      } else {
        voxel_window<Q, NCH>(acc, fiz, rows, t, zlo, zhi, zm1, nzs, lane);
      }
    }
  }
}

template <int Q, int STORE, bool FAST>
__device__ __forceinline__ void bp_column(const BpArgs& a, int rmax) {
  using Pair = typename PairT<STORE>::type;
  const BpFrame& F = a.fr[blockIdx.y];
  const Pair* cc = static_cast<const Pair*>(F.corrcal);
  extern __shared__ __align__(16) unsigned char smraw[];
  const DevGeom& g = a.g;
  const int nwarps = blockDim.x >> 5;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int colidx = blockIdx.x * nwarps + wib;
  if (colidx >= g.res * g.res) return;  // whole warp
  const int iy = colidx / g.res, ix = colidx - iy * g.res;
  int4* my = reinterpret_cast<int4*>(smraw) + wib * a.na;
  float2* rows = reinterpret_cast<float2*>(reinterpret_cast<int4*>(smraw) + nwarps * a.na) + wib * rmax;
  const float2 sentinel = make_float2(-1000.f, -1000.f);
  if constexpr (FAST) {
    // rmax = rbuf here: every row starts at the gap sentinel; views stage
    // theirs from offset pad_lo
    for (int r = lane; r < rmax; r += 32) rows[r] = sentinel;
    rows += a.pad_lo;
  }
  // per angle: radial texels, weight and yrot (GFIRST_GPU_Kernels.cu:136-147)
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

  float fiz[Q];
  float2 acc[Q];
#pragma unroll
  for (int q = 0; q < Q; q++) {
    fiz[q] = (float)(lane + 32 * q);
    acc[q] = make_float2(0.f, 0.f);
  }
  for (int s = 0; s < g.nseg; s++) {
    const DevSeg sg = g.seg[s];
    if constexpr (FAST) {
      // rows past this segment's back to the sentinel (a wider segment left
      // its rows there); the first view's warp barrier orders these stores
      __syncwarp();
      const int nrow = sg.nplanes + 2;
      for (int r = nrow + lane; r < rmax - a.pad_lo; r += 32) rows[r] = sentinel;
    }
    switch ((sg.nplanes + 2 + 31) >> 5) {
#define GF_SEG(N) \
  case N:         \
    if constexpr (N <= Q + 1) segment_views<Q, N, FAST>(acc, fiz, cc, my, rows, sg, a.na, g.nzs, lane); \
    break;
      GF_SEG(1) GF_SEG(2) GF_SEG(3) GF_SEG(4) GF_SEG(5) GF_SEG(6) GF_SEG(7) GF_SEG(8) GF_SEG(9)
#undef GF_SEG
    }
  }
  store_column<Q>(F, a.ratio, (size_t)colidx * g.nzp, lane, g.nzs, acc);
}

// ---- two frames per warp ------------------------------------------------
// Two frames of a fused group whose normalization masks are equal share one
// warp per column: the per-(column, angle) table, the per-view fraction, row
// offset and lane-chunk window, and the staged mask rows with their
// interpolation; only the ratios and the (NUMER, DENOM) sums are per frame.
// A staged row holds (ratio A, ratio B) and the mask, 12 bytes instead of
// two frames' 16, and each frame's row loads fetch only its ratio beside
// frame A's (ratio, mask) pair.  Every operation on a frame's values is the
// per-view form's (the packed f32x2 operations round each element as the
// scalar one), so each frame's sums equal the per-view form's for that frame
// alone, bit for bit.

__device__ __forceinline__ float ratio_of(const float2* p) { return *reinterpret_cast<const float*>(p); }
__device__ __forceinline__ float ratio_of(const __half2* p) { return __half2float(*reinterpret_cast<const __half*>(p)); }
__device__ __forceinline__ float ratio_of(const __nv_bfloat162* p) {
  return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(p));
}

template <int Q, int LO, int HI>
__device__ __forceinline__ void voxel_views_pair(float2 (&accA)[Q], float2 (&accB)[Q], const float2* rr,
                                                 const float* rc, float be) {
  const float2 be2 = make_float2(be, be);
#pragma unroll
  for (int q = LO; q <= HI; q++) {
    const float2 vr = lerp2(rr[32 * q], rr[32 * q + 1], be2);  // (ratio A, ratio B)
    const float vc = lerp_rn(rc[32 * q], rc[32 * q + 1], be);    // mask
    if (!(vc < 0.f || vr.x < 0.f)) accA[q] = __fadd2_rn(accA[q], make_float2(vr.x, vc));
    if (!(vc < 0.f || vr.y < 0.f)) accB[q] = __fadd2_rn(accB[q], make_float2(vr.y, vc));
  }
}

template <int Q, int NCH>
__device__ __forceinline__ void voxel_window_pair(float2 (&accA)[Q], float2 (&accB)[Q], const float2* rr,
                                                  const float* rc, float be, float t, float zlo) {
  constexpr int W = NCH + 1;  // the per-view form's window (bp_fast_pads sizes the sentinel rows for it)
  if constexpr (W >= Q) {
    voxel_views_pair<Q, 0, Q - 1>(accA, accB, rr, rc, be);
  } else {
    const int izlo = max(__float2int_rd(__fsub_rn(__fsub_rn(zlo, t), 1.0f)), 0);
    switch (min(izlo >> 5, Q - W)) {
#define GF_VWP(L) \
  case L:         \
    if constexpr (L <= Q - W) voxel_views_pair<Q, L, L + W - 1>(accA, accB, rr, rc, be); \
    break;
      GF_VWP(0) GF_VWP(1) GF_VWP(2) GF_VWP(3) GF_VWP(4) GF_VWP(5) GF_VWP(6)
#undef GF_VWP
    }
  }
}

#ifndef GF_BP_PAIR_PF32
#define GF_BP_PAIR_PF32 1
#endif
#ifndef GF_BP_PAIR_PF16
#define GF_BP_PAIR_PF16 3
#endif

template <int Q, int NCH, class Pair>
__device__ __forceinline__ void segment_views_pair(float2 (&accA)[Q], float2 (&accB)[Q], const Pair* ccA,
                                                   const Pair* ccB, const int4* my, float2* rr, float* rc,
                                                   const DevSeg& sg, int na, int lane) {
  const float zlo = (float)sg.zmin;
  const int zm1 = sg.zmin - 1;
  const int nrow = sg.nplanes + 2;
  // next view's rows loaded during the current view's voxels (the first
  // GF_BP_PAIR_PF32 / GF_BP_PAIR_PF16 chunks; the rest at staging)
  constexpr int PFC = sizeof(Pair) == 8 ? GF_BP_PAIR_PF32 : GF_BP_PAIR_PF16;
  constexpr int PF = NCH > PFC ? PFC : NCH;
  Pair a0[PF], a1[PF];
  float b0[PF], b1[PF];
  auto load = [&](const int4& e) {
    const Pair* pa0 = ccA + e.x + sg.blk;
    const Pair* pa1 = ccA + e.y + sg.blk;
    const Pair* pb0 = ccB + e.x + sg.blk;
    const Pair* pb1 = ccB + e.y + sg.blk;
#pragma unroll
    for (int k = 0; k < PF; k++) {
      const int r = lane + 32 * k;
      if (k < NCH - 1 || r < nrow) {
        a0[k] = __ldg(pa0 + r);
        a1[k] = __ldg(pa1 + r);
        b0[k] = ratio_of(pb0 + r);
        b1[k] = ratio_of(pb1 + r);
      }
    }
  };
  int4 e = my[0];
  load(e);
  for (int tl = 0; tl < na; tl++) {
    const float al = __int_as_float(e.z);
    const float2 al2 = make_float2(al, al);
    const float t = __fmul_rn(__int_as_float(e.w), sg.fz);  // yrot*fz
    __syncwarp();  // every lane is done reading the previous view's rows
    const Pair* qa0 = ccA + e.x + sg.blk;
    const Pair* qa1 = ccA + e.y + sg.blk;
    const Pair* qb0 = ccB + e.x + sg.blk;
    const Pair* qb1 = ccB + e.y + sg.blk;
#pragma unroll
    for (int k = 0; k < NCH; k++) {
      const int r = lane + 32 * k;
      if (k < NCH - 1 || r < nrow) {
        float2 va;
        float vb;
        if (k < PF) {
          va = lerp2(pair_f(a0[k < PF ? k : 0]), pair_f(a1[k < PF ? k : 0]), al2);
          vb = lerp_rn(b0[k < PF ? k : 0], b1[k < PF ? k : 0], al);
        } else {
          va = lerp2(pair_f(__ldg(qa0 + r)), pair_f(__ldg(qa1 + r)), al2);
          vb = lerp_rn(ratio_of(qb0 + r), ratio_of(qb1 + r), al);
        }
        rr[r] = make_float2(va.x, vb);
        rc[r] = va.y;
      }
    }
    __syncwarp();
    if (tl + 1 < na) {
      e = my[tl + 1];
      load(e);
    }
    const float ft = floorf(t);
    const float be = __fsub_rn(t, ft);
    const int off = ((int)ft - zm1) + lane;
    voxel_window_pair<Q, NCH>(accA, accB, rr + off, rc + off, be, t, zlo);
  }
}

// a.fr[2p] and a.fr[2p + 1] form pair p = blockIdx.y; staged rows per warp:
// rmax = rbuf float2 (ratios) + rbuf floats (mask).
template <int Q, int STORE>
__device__ __forceinline__ void bp_column_pair(const BpArgs& a, int rmax) {
  using Pair = typename PairT<STORE>::type;
  const BpFrame& FA = a.fr[2 * blockIdx.y];
  const BpFrame& FB = a.fr[2 * blockIdx.y + 1];
  const Pair* ccA = static_cast<const Pair*>(FA.corrcal);
  const Pair* ccB = static_cast<const Pair*>(FB.corrcal);
  extern __shared__ __align__(16) unsigned char smraw[];
  const DevGeom& g = a.g;
  const int nwarps = blockDim.x >> 5;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int colidx = blockIdx.x * nwarps + wib;
  if (colidx >= g.res * g.res) return;  // whole warp
  const int iy = colidx / g.res, ix = colidx - iy * g.res;
  int4* my = reinterpret_cast<int4*>(smraw) + wib * a.na;
  float2* rr = reinterpret_cast<float2*>(reinterpret_cast<int4*>(smraw) + nwarps * a.na) + wib * rmax;
  float* rc = reinterpret_cast<float*>(reinterpret_cast<float2*>(reinterpret_cast<int4*>(smraw) + nwarps * a.na) +
                                       nwarps * rmax) + wib * rmax;
  for (int r = lane; r < rmax; r += 32) {
    rr[r] = make_float2(-1000.f, -1000.f);
    rc[r] = -1000.f;
  }
  rr += a.pad_lo;
  rc += a.pad_lo;
  // per angle: radial texels, weight and yrot (GFIRST_GPU_Kernels.cu:136-147)
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
  float2 accA[Q], accB[Q];
#pragma unroll
  for (int q = 0; q < Q; q++) {
    accA[q] = make_float2(0.f, 0.f);
    accB[q] = make_float2(0.f, 0.f);
  }
  for (int s = 0; s < g.nseg; s++) {
    const DevSeg sg = g.seg[s];
    __syncwarp();
    const int nrow = sg.nplanes + 2;
    for (int r = nrow + lane; r < rmax - a.pad_lo; r += 32) {
      rr[r] = make_float2(-1000.f, -1000.f);
      rc[r] = -1000.f;
    }
    switch ((sg.nplanes + 2 + 31) >> 5) {
#define GF_SEGP(N) \
  case N:          \
    if constexpr (N <= Q + 1) segment_views_pair<Q, N>(accA, accB, ccA, ccB, my, rr, rc, sg, a.na, lane); \
    break;
      GF_SEGP(1) GF_SEGP(2) GF_SEGP(3) GF_SEGP(4) GF_SEGP(5) GF_SEGP(6) GF_SEGP(7) GF_SEGP(8) GF_SEGP(9)
#undef GF_SEGP
    }
  }
  const size_t cb = (size_t)colidx * g.nzp;
  store_column<Q>(FA, a.ratio, cb, lane, g.nzs, accA);
  store_column<Q>(FB, a.ratio, cb, lane, g.nzs, accB);
}

#ifndef GF_BP_PAIR_REGS
#define GF_BP_PAIR_REGS 80
#endif

template <int STORE>
constexpr int bp_pair_regs = GF_BP_PAIR_REGS;

template <int Q, int STORE>
__global__ void __launch_bounds__(256) __maxnreg__(bp_pair_regs<STORE>) bp_pair_kernel(const BpArgs a, int rmax) {
  bp_column_pair<Q, STORE>(a, rmax);
}

// One launch serves one subset: every frame takes angles subset + l*g.nsub,
// l < na (the frames of a fused group with another subset count get a launch
// of their own), which keeps the subset a launch constant in the kernels.
static bool subset_ok(const BpArgs& a) {
  return a.g.nsub >= 1 && a.subset >= 0 && a.subset < a.g.nsub && a.na >= 1 &&
         a.na == (a.g.nang - a.subset + a.g.nsub - 1) / a.g.nsub;
}

cudaError_t launch_bp_pairs(const BpArgs& a, int warps, cudaStream_t st) {
  if (!subset_ok(a)) return cudaErrorInvalidValue;
  if (warps < 1 || warps > 8) return cudaErrorInvalidValue;
  if (!a.fast || a.pad_lo < 0 || a.rbuf < a.pad_lo + a.g.nzs + 2) return cudaErrorInvalidValue;
  const int npairs = a.nfr / 2;
  if (npairs < 1 || 2 * npairs != a.nfr || a.nfr > kMaxFrames) return cudaErrorInvalidValue;
  for (int f = 0; f < a.nfr; f++)
    if (!a.fr[f].corrcal || !a.fr[f].numer || (!a.ratio && !a.fr[f].denom)) return cudaErrorInvalidValue;
  const int Q = a.g.nzp / 32;
  const int rmax = a.rbuf;
  dim3 grid((a.g.res * a.g.res + warps - 1) / warps, npairs);
  size_t smem = (size_t)warps * (a.na * sizeof(int4) + rmax * (sizeof(float2) + sizeof(float)));
  void (*k)(BpArgs, int) = nullptr;
  switch (a.storage * 16 + Q) {
#define GF_BPP_CASE(S, QQ) \
  case S * 16 + QQ: k = bp_pair_kernel<QQ, S>; break;
    GF_BPP_CASE(0, 1) GF_BPP_CASE(0, 2) GF_BPP_CASE(0, 3) GF_BPP_CASE(0, 4)
    GF_BPP_CASE(0, 5) GF_BPP_CASE(0, 6) GF_BPP_CASE(0, 7) GF_BPP_CASE(0, 8)
    GF_BPP_CASE(1, 1) GF_BPP_CASE(1, 2) GF_BPP_CASE(1, 3) GF_BPP_CASE(1, 4)
    GF_BPP_CASE(1, 5) GF_BPP_CASE(1, 6) GF_BPP_CASE(1, 7) GF_BPP_CASE(1, 8)
    GF_BPP_CASE(2, 1) GF_BPP_CASE(2, 2) GF_BPP_CASE(2, 3) GF_BPP_CASE(2, 4)
    GF_BPP_CASE(2, 5) GF_BPP_CASE(2, 6) GF_BPP_CASE(2, 7) GF_BPP_CASE(2, 8)
#undef GF_BPP_CASE
    default: return cudaErrorInvalidValue;
  }
  if (smem > 48 * 1024) {
    cudaError_t e = allow_max_smem(k);
    if (e != cudaSuccess) return e;
  }
  k<<<grid, warps * 32, smem, st>>>(a, rmax);
  return cudaGetLastError();
}

// Register budgets.  The kernel hides its latencies with resident warps: up
// to 160 slices both pair types are capped at 64 registers (eight 4-warp
// blocks per SM, no spill; FP32 with the shallower prefetch above) -- 1.296
// and 1.245 ms against 1.343 and 1.264 ms under the launch bounds of
// bp_kernel_deep (six and eight blocks).  The cap is a constant that depends
// on the template argument, so it stands beside the 256-thread bound (both
// reach the compiled kernel); the cap alone, or a (128, 8) launch bound,
// schedules worse: 1.340 and 1.266 ms.  Deeper columns keep the launch
// bounds below, which spill less there.
template <int STORE>
constexpr int bp_reg_cap = 64;

template <int Q, int STORE>
__global__ void __launch_bounds__(256) __maxnreg__(bp_reg_cap<STORE>) bp_kernel(const BpArgs a, int rmax) {
  bp_column<Q, STORE, false>(a, rmax);
}

template <int Q, int STORE>
__global__ void __launch_bounds__(256, STORE == 0 ? 3 : 4) bp_kernel_deep(const BpArgs a, int rmax) {
  bp_column<Q, STORE, false>(a, rmax);
}

// The per-view form needs no per-voxel z registers; the same caps apply.
template <int Q, int STORE>
__global__ void __launch_bounds__(256) __maxnreg__(bp_reg_cap<STORE>) bp_fast_kernel(const BpArgs a, int rmax) {
  bp_column<Q, STORE, true>(a, rmax);
}

template <int Q, int STORE>
__global__ void __launch_bounds__(256, STORE == 0 ? 3 : 4) bp_fast_kernel_deep(const BpArgs a, int rmax) {
  bp_column<Q, STORE, true>(a, rmax);
}

template <int Q, int STORE>
static void (*bp_entry(bool fast))(BpArgs, int) {
  if constexpr (Q <= 5) return fast ? bp_fast_kernel<Q, STORE> : bp_kernel<Q, STORE>;
  else return fast ? bp_fast_kernel_deep<Q, STORE> : bp_kernel_deep<Q, STORE>;
}

cudaError_t launch_bp(const BpArgs& a, int warps, cudaStream_t st) {
  if (warps < 1 || warps > 8) return cudaErrorInvalidValue;
  if (!subset_ok(a)) return cudaErrorInvalidValue;
  const int Q = a.g.nzp / 32;
  if (a.fast && (a.pad_lo < 0 || a.rbuf < a.pad_lo + a.g.nzs + 2)) return cudaErrorInvalidValue;
  const int rmax = a.fast ? a.rbuf : a.g.nzs + 2;
  if (a.nfr < 0 || a.nfr > kMaxFrames) return cudaErrorInvalidValue;
  for (int f = 0; f < (a.nfr > 1 ? a.nfr : 1); f++)
    if (!a.fr[f].corrcal || !a.fr[f].numer || (!a.ratio && !a.fr[f].denom)) return cudaErrorInvalidValue;
  dim3 grid((a.g.res * a.g.res + warps - 1) / warps, a.nfr > 1 ? a.nfr : 1);
  size_t smem = (size_t)warps * (a.na * sizeof(int4) + rmax * sizeof(float2));
  void (*k)(BpArgs, int) = nullptr;
  switch (a.storage * 16 + Q) {
#define GF_BP_CASE(S, QQ) \
  case S * 16 + QQ: k = bp_entry<QQ, S>(a.fast != 0); break;
    GF_BP_CASE(0, 1) GF_BP_CASE(0, 2) GF_BP_CASE(0, 3) GF_BP_CASE(0, 4)
    GF_BP_CASE(0, 5) GF_BP_CASE(0, 6) GF_BP_CASE(0, 7) GF_BP_CASE(0, 8)
    GF_BP_CASE(1, 1) GF_BP_CASE(1, 2) GF_BP_CASE(1, 3) GF_BP_CASE(1, 4)
    GF_BP_CASE(1, 5) GF_BP_CASE(1, 6) GF_BP_CASE(1, 7) GF_BP_CASE(1, 8)
    GF_BP_CASE(2, 1) GF_BP_CASE(2, 2) GF_BP_CASE(2, 3) GF_BP_CASE(2, 4)
    GF_BP_CASE(2, 5) GF_BP_CASE(2, 6) GF_BP_CASE(2, 7) GF_BP_CASE(2, 8)
#undef GF_BP_CASE
    default: return cudaErrorInvalidValue;
  }
  if (smem > 48 * 1024) {
    cudaError_t e = allow_max_smem(k);
    if (e != cudaSuccess) return e;
  }
  k<<<grid, warps * 32, smem, st>>>(a, rmax);
  return cudaGetLastError();
}

}  // namespace gf
