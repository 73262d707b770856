// gf_plan.h -- host-side geometry tables and device data layouts.
//
// Layouts on the device (all 128-byte aligned rows):
//  - image volumes are z-fastest: [RES][RES][NZP] (y, x, z), NZP = NZS
//    rounded up to 32, padding slices held at 0;
//  - sinogram data for the projectors is subset-local and radial-major:
//    [angle-in-subset][radial bin][row], one "row" per sinogram plane.  Each
//    segment's block of planes carries one extra row before and after
//    (PP = P + 2*NSEG rows, row stride PS = PP rounded up to 32): for
//    segment 0 they repeat its first/last plane (texture clamp), for oblique
//    segments they hold the -1000 gap sentinel that GFIRST.cu:447 writes
//    around a view's planes.  A back-projection sample then reads two
//    neighbouring rows with no branch.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gf {

struct Geom {
  int res, nzs, nrad, nang, span, nseg;
  float pitch, diam, fov;
};

// Per segment, in the reference's order idz = 0,-1,+1,-2,+2,... (GFIRST.cu:163-168).
struct Seg {
  int idz, zmin, nplanes;
  int acc;    // nz_acum[s] (GFIRST.cu:133-140)
  int blk;    // first padded row of this segment: acc + 2*s
  float dz;   // forward-projector z step per sample (GFIRST_GPU_Kernels.cu:83)
  float fz;   // back-projector z slope (GFIRST_GPU_Kernels.cu:134)
};

// One forward-projector thread's run of consecutive planes in one segment.
struct Run {
  int seg, p0, n, pad;  // pad: bit0 = writes the row before, bit1 = after
};

struct Plan {
  Geom g{};
  int P = 0, PP = 0, PS = 0, NZP = 0;
  int64_t ndata = 0, nvox = 0, nvoxp = 0;
  std::vector<Seg> seg;
  std::vector<float> sinv, cosv;  // per angle, sinf/cosf of GFIRST_GPU_Kernels.cu:75
  float radm = 0, resm = 0, fx_fp = 0, fx_bp = 0;
  int lam0 = 0, lam1 = 0;  // sample range of GFIRST_GPU_Kernels.cu:90-93
  int nsub = 1;
  std::vector<int> sub_nang;     // angles per subset
  std::vector<int64_t> sub_off;  // element offset of subset s in an all-subset array
  int amax = 0;                  // most angles in one subset
  int64_t sub_elems(int s) const { return (int64_t)sub_nang[s] * g.nrad * PS; }
  int64_t all_elems() const { return (int64_t)g.nang * g.nrad * PS; }
};

// Validates the geometry and fills every table; false with a message on error.
bool make_plan(const Geom& g, int nsub, Plan* out, std::string* err);

// Forward-projector schedule: runs of at most R planes, R odd so that the
// threads of a warp read shared memory without bank conflicts.
struct FpSchedule {
  int R = 0, nthreads = 0, lc = 0, padl = 0, padr = 0, cw = 0;
  std::vector<Run> runs;
  size_t smem_bytes() const;
};
bool make_fp_schedule(const Plan& p, int R, int lc, FpSchedule* out);
int fp_default_R(const Plan& p);

// Staged-row buffer of the back projector's per-view form: each warp stages a
// view's rows at offset pad_lo of a buffer of rbuf (corr, calib) pairs, the
// rest held at the -1000 gap sentinel.  A lane chunk reads its two rows at
// an offset fixed per view, so voxels outside the segment's plane range read
// sentinels there (or the segment's own sentinel pad rows with weight >=
// 1/2), which the gap rule skips as the range test would.  pad_lo and the
// rows past the widest segment cover every row any issued lane chunk reads,
// for every axial shift |t| <= |yrot| * |fz| the geometry allows.
struct BpPads {
  int pad_lo = 0, pad_hi = 0, rbuf = 0;
};
BpPads bp_fast_pads(const Plan& p);

// Sinogram bin of (segment, plane, angle, radial), GFIRST.cu:175-176.
inline int64_t lor_index(const Plan& p, int s, int iz0, int t, int r) {
  return ((int64_t)(iz0 - p.seg[s].zmin) + p.seg[s].acc) * ((int64_t)p.g.nrad * p.g.nang) + (int64_t)t * p.g.nrad + r;
}

}  // namespace gf
