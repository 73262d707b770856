// gf_plan.cpp -- geometry tables.  Every float constant is computed with the
// expression (and the float/double promotions) of the reference kernel it
// comes from, so the device code sees the reference's values.
#include "gf_plan.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>

namespace gf {

static const float PI_REF = 3.1415926f;  // GFIRST.h:1

static int seg_idz(int s) { return ((s + 1) / 2) * (1 - (s % 2) * 2); }
static int seg_zmin(const Geom& g, int idz) {
  return idz == 0 ? 0 : (std::abs(idz) - 1) * g.span + (g.span / 2 + 1);
}

bool make_plan(const Geom& g, int nsub, Plan* out, std::string* err) {
  auto fail = [&](const char* m) {
    if (err) *err = m;
    return false;
  };
  if (g.res < 8 || g.res > 1024) return fail("res must be in [8, 1024]");
  if (g.nzs < 5 || g.nzs > 1024) return fail("nzs must be in [5, 1024]");
  if (g.nrad < 2 || g.nrad > 4096) return fail("nrad must be in [2, 4096]");
  if (g.nang < 1 || g.nang > 4096) return fail("nang must be in [1, 4096]");
  if (g.span < 1 || g.nseg < 1 || g.nseg > 1023) return fail("span and nseg must be positive (nseg < 1024)");
  if (!(g.pitch > 0.f) || !(g.diam > 0.f) || !(g.fov > 0.f)) return fail("pitch, diam and fov must be positive");
  if (nsub < 1 || nsub > g.nang) return fail("nsubsets must be in [1, nang]");
  Plan p;
  p.g = g;
  p.nsub = nsub;
  p.NZP = (g.nzs + 31) / 32 * 32;
  int acc = 0;
  const float vx = g.fov / (float)g.res;
  for (int s = 0; s < g.nseg; s++) {
    Seg sg{};
    sg.idz = seg_idz(s);
    sg.zmin = seg_zmin(g, sg.idz);
    sg.nplanes = g.nzs - 2 * sg.zmin;
    if (sg.nplanes <= 0) return fail("a segment has no planes (nzs - 2*zmin <= 0)");
    sg.acc = acc;
    sg.blk = acc + 2 * s;
    int sgn = sg.idz == 0 ? 0 : sg.idz / std::abs(sg.idz);
    // dz = (FOV/NPT)*float(idz_signo*zmin)/(0.5f*DIAM_DET)    (float)
    sg.dz = ((g.fov / (float)g.res) * (float)(sgn * sg.zmin)) / (0.5f * g.diam);
    // fz = (dx)*float(idz_signo*zmin)/(DIAM_DET/2.0)          (float product, double division)
    sg.fz = (float)((double)(vx * (float)(sgn * sg.zmin)) / ((double)g.diam / 2.0));
    acc += sg.nplanes;
    p.seg.push_back(sg);
  }
  p.P = acc;
  p.PP = acc + 2 * g.nseg;
  p.PS = (p.PP + 31) / 32 * 32;
  p.ndata = (int64_t)p.P * g.nang * g.nrad;
  p.nvox = (int64_t)g.res * g.res * g.nzs;
  p.nvoxp = (int64_t)g.res * g.res * p.NZP;
  if (p.ndata >= ((int64_t)1 << 31)) return fail("NDATA must fit in int32 (the reference's VLOR bins are int32)");
  p.sinv.resize(g.nang);
  p.cosv.resize(g.nang);
  for (int t = 0; t < g.nang; t++) {
    float ang = -(float)t / (float)g.nang * PI_REF + PI_REF;
    p.sinv[t] = sinf(ang);
    p.cosv[t] = cosf(ang);
  }
  p.radm = (float)(g.nrad - 1) * 0.5f;
  p.resm = (float)(g.res - 1) * 0.5f;
  p.fx_fp = (0.5f * g.pitch) / vx;
  p.fx_bp = vx / (float)((double)g.pitch / 2.0);
  const float tof_size = (float)g.res / (float)1;
  p.lam0 = (int)floorf((0.0f - 0.5f) * tof_size);
  p.lam1 = (int)floorf((0.0f + 0.5f) * tof_size);
  p.sub_nang.assign(nsub, 0);
  for (int t = 0; t < g.nang; t++) p.sub_nang[t % nsub]++;
  p.sub_off.assign(nsub + 1, 0);
  for (int s = 0; s < nsub; s++) p.sub_off[s + 1] = p.sub_off[s] + p.sub_elems(s);
  p.amax = *std::max_element(p.sub_nang.begin(), p.sub_nang.end());
  *out = std::move(p);
  return true;
}

size_t FpSchedule::smem_bytes() const {
  return (size_t)lc * cw * sizeof(float) + (size_t)lc * (4 * sizeof(int) + 2 * sizeof(float));
}

bool make_fp_schedule(const Plan& p, int R, int lc, FpSchedule* out) {
  if (lc < 1 || lc > 256 || R < 1) return false;
  FpSchedule f;
  f.R = R;
  f.lc = lc;
  int kmin = 0, kmax = p.g.nzs - 1;
  for (int s = 0; s < p.g.nseg; s++) {
    const Seg& sg = p.seg[s];
    int end = p.g.nzs - sg.zmin;
    for (int p0 = sg.zmin; p0 < end; p0 += R) {
      Run r{s, p0, std::min(R, end - p0), 0};
      if (p0 == sg.zmin) r.pad |= 1;
      if (p0 + r.n == end) r.pad |= 2;
      f.runs.push_back(r);
      for (int lam : {p.lam0, p.lam1}) {
        float t = (float)lam * sg.dz;
        int m = (int)floorf(t);
        kmin = std::min(kmin, p0 + m);
        kmax = std::max(kmax, p0 + m + R);
      }
    }
  }
  f.nthreads = ((int)f.runs.size() + 31) / 32 * 32;
  if (f.nthreads > 512) return false;
  f.padl = -kmin;
  f.padr = kmax - (p.g.nzs - 1);
  f.cw = f.padl + p.g.nzs + f.padr;
  if (f.smem_bytes() > 200 * 1024) return false;
  *out = std::move(f);
  return true;
}

BpPads bp_fast_pads(const Plan& p) {
  // Mirrors the kernel's choice of lane chunks (all Q of them, or the NCH + 1
  // from the chunk of floor(zmin - t - 1)) and its row index j = iz +
  // floor(t) - (zmin - 1), and takes the extremes of j and j + 1 over every
  // piece of t: the functions change only where t or zmin - t crosses an
  // integer, so each integer is sampled on both sides (a float evaluation in
  // the kernel can fall only into an adjacent piece) and at its midpoint.
  const int Q = p.NZP / 32;
  const double ymax = std::sqrt(2.0) * (double)p.resm + 1.0;
  int lo = 0, hi = 0;
  for (const Seg& sg : p.seg) {
    const int nrow = sg.nplanes + 2;
    const int W = (nrow + 31) / 32 + 1;
    const double tmax = ymax * std::fabs((double)sg.fz) + 1.0;
    for (int m = (int)std::floor(-tmax) - 1; m <= (int)std::ceil(tmax) + 1; m++) {
      for (double t : {m - 1e-3, (double)m, m + 1e-3, m + 0.5}) {
        const int k = (int)std::floor(t) - (sg.zmin - 1);
        int c0 = 0, c1 = Q - 1;
        if (W < Q) {
          const int izlo = std::max((int)std::floor((double)sg.zmin - t - 1.0), 0);
          c0 = std::min(izlo >> 5, Q - W);
          c1 = c0 + W - 1;
        }
        lo = std::max(lo, -(32 * c0 + k));
        hi = std::max(hi, (32 * c1 + 31 + k + 1) - (nrow - 1));
      }
    }
  }
  BpPads b;
  b.pad_lo = lo + 2;
  b.pad_hi = hi + 2;
  b.rbuf = b.pad_lo + (p.g.nzs + 2) + b.pad_hi;
  return b;
}

int fp_default_R(const Plan& p) {
  for (int R : {9, 17, 25, 33}) {
    FpSchedule f;
    if (make_fp_schedule(p, R, 32, &f) && f.nthreads <= 512) return R;
  }
  return 33;
}

}  // namespace gf
