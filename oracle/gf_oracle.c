/*
 * gf_oracle.c -- CPU restatement of GFIRST's OSEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the parity oracle and the timed CPU baseline).
 * Nothing in the product library links, loads or calls this file.
 *
 * Every function follows the reference source literally; each cites the
 * file:line it restates (paths inside the GFIRST project).  Arithmetic rules:
 *  - every +,-,*,/ is rounded on its own (build with -ffp-contract=off), in
 *    the order the reference source writes it;
 *  - where the reference promotes to double (literals like 2.0, 1.0/s,
 *    1e-8, exp() of a double) this code promotes too;
 *  - texture fetches (tex3D with cudaFilterModeLinear, cudaAddressModeClamp,
 *    unnormalized coordinates, GFIRST_GPU_Kernels.cu:254-281) are emulated
 *    with exact FP32 weights: x-0.5, floor/frac, clamped texel indices, and
 *    each 1-D interpolation evaluated as fma(w, b-a, a).  The hardware's
 *    8-bit fixed-point weights are not emulated.
 *  - the reference build uses -use_fast_math (compile.sh:1); this code uses
 *    IEEE sinf/cosf and IEEE division instead.
 *
 * Parity pin: oracle/build_ref.py compiles the reference's own kernels and
 * osem3d() driver on the host (with a CUDA emulation shim) and
 * tests/golden/make_golden.py records their outputs; tests/test_oracle.py
 * checks this file against those fixtures.
 */
#include "gf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef gfo_real real;

#define GFO_IS_DOUBLE (sizeof(real) == sizeof(double))
#define RL(x) ((real)(x))

static inline real r_floor(real v) { return GFO_IS_DOUBLE ? (real)floor((double)v) : (real)floorf((float)v); }
static inline real r_fma(real a, real b, real c) {
  return GFO_IS_DOUBLE ? (real)fma((double)a, (double)b, (double)c) : (real)fmaf((float)a, (float)b, (float)c);
}
static inline real r_sin(real v) { return GFO_IS_DOUBLE ? (real)sin((double)v) : (real)sinf((float)v); }
static inline real r_cos(real v) { return GFO_IS_DOUBLE ? (real)cos((double)v) : (real)cosf((float)v); }
static inline real lerp(real a, real b, real w) { return r_fma(w, b - a, a); }
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* PI as the reference defines it (GFIRST.h:1). */
static const float PI_REF = 3.1415926f;

int gfo_real_bytes(void) { return (int)sizeof(real); }
int gfo_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* Segments and plane bookkeeping: GFIRST.cu:133-140 (nz_acum),       */
/* GFIRST.cu:163-168 (segment order 0,-1,+1,-2,+2,...),               */
/* GFIRST_GPU_Kernels.cu:54 (zmin).                                    */
/* ------------------------------------------------------------------ */
static int seg_idz(int idz_ind) {
  int isigno = 1 - (idz_ind % 2) * 2;
  return ((idz_ind + 1) / 2) * isigno;
}
static int seg_zmin(const gfo_geom* g, int idz) {
  if (idz == 0) return 0;
  return (abs(idz) - 1) * g->span + (g->span / 2 + 1);
}

void gfo_segments(const gfo_geom* g, int32_t* idz, int32_t* zmin, int32_t* nz_acum) {
  nz_acum[0] = 0;
  for (int s = 0; s < g->nseg; s++) {
    int k = seg_idz(s);
    if (idz) idz[s] = k;
    if (zmin) zmin[s] = seg_zmin(g, k);
    /* GFIRST.cu:137-139 uses the unsigned magnitude (idz_ind+1)/2; zmin is the same. */
    nz_acum[s + 1] = nz_acum[s] + (g->nzs - 2 * seg_zmin(g, k));
  }
}

int64_t gfo_planes(const gfo_geom* g) {
  if (g->nseg < 1 || g->res < 1 || g->nzs < 5 || g->nrad < 2 || g->nang < 1) return -1;
  int64_t p = 0;
  for (int s = 0; s < g->nseg; s++) {
    int n = g->nzs - 2 * seg_zmin(g, seg_idz(s));
    if (n <= 0) return -1;
    p += n;
  }
  return p;
}

/* GFIRST.cu:175-176 / 359-360 / 450-451 */
int64_t gfo_lor(const gfo_geom* g, int32_t seg_ind, int32_t iz0, int32_t itheta, int32_t ird) {
  int32_t* acc = (int32_t*)malloc(sizeof(int32_t) * (size_t)(g->nseg + 1));
  gfo_segments(g, NULL, NULL, acc);
  int zmin = seg_zmin(g, seg_idz(seg_ind));
  int64_t lor = ((int64_t)(iz0 - zmin) + acc[seg_ind]) * ((int64_t)g->nrad * g->nang) +
                (int64_t)itheta * g->nrad + ird;
  free(acc);
  return lor;
}

static int64_t ndata_of(const gfo_geom* g) { return gfo_planes(g) * g->nang * g->nrad; }
static int64_t nvox_of(const gfo_geom* g) { return (int64_t)g->res * g->res * g->nzs; }

/* CreateInitialCylinder, GFIRST_CPU_Kernels.cpp:35-56 */
void gfo_cylinder(const gfo_geom* g, real val, real* img) {
  const int RES = g->res;
  int64_t iV = 0;
  for (int z = 0; z < g->nzs; z++)
    for (int y = 0; y < RES; y++)
      for (int x = 0; x < RES; x++) {
        double dx = (double)(float)(x - RES / 2), dy = (double)(float)(y - RES / 2);
        img[iV++] = (pow(dx, 2) + pow(dy, 2) <= (double)((RES / 2) * (RES / 2))) ? val : RL(0.0f);
      }
}

/* ------------------------------------------------------------------ */
/* Texture emulation                                                  */
/* ------------------------------------------------------------------ */

/* tex3D(imgEstTex, x, y, z): image [NZS][RES][RES], clamp on all axes. */
static real tex3_img(const gfo_geom* g, const real* img, real x, real y, real z) {
  const int RES = g->res, NZS = g->nzs;
  real xb = x - RL(0.5f), yb = y - RL(0.5f), zb = z - RL(0.5f);
  real fx = r_floor(xb), fy = r_floor(yb), fz = r_floor(zb);
  real a = xb - fx, b = yb - fy, c = zb - fz;
  int i = (int)fx, j = (int)fy, k = (int)fz;
  int i0 = clampi(i, 0, RES - 1), i1 = clampi(i + 1, 0, RES - 1);
  int j0 = clampi(j, 0, RES - 1), j1 = clampi(j + 1, 0, RES - 1);
  int k0 = clampi(k, 0, NZS - 1), k1 = clampi(k + 1, 0, NZS - 1);
  const int64_t R2 = (int64_t)RES * RES;
  const real* s0 = img + k0 * R2;
  const real* s1 = img + k1 * R2;
  real v0 = lerp(lerp(s0[j0 * RES + i0], s0[j0 * RES + i1], a), lerp(s0[j1 * RES + i0], s0[j1 * RES + i1], a), b);
  real v1 = lerp(lerp(s1[j0 * RES + i0], s1[j0 * RES + i1], a), lerp(s1[j1 * RES + i0], s1[j1 * RES + i1], a), b);
  return lerp(v0, v1, c);
}

/* One (segment, angle) view buffer texel, GFIRST.cu:447-458: planes outside
 * [zmin, NZS-zmin) hold -1000. */
static inline real view_texel(const gfo_geom* g, const real* arr, int64_t seg_base, int zmin, int itheta,
                              int j, int i) {
  if (j < zmin || j >= g->nzs - zmin) return RL(-1000.0f);
  return arr[(seg_base + (j - zmin)) * ((int64_t)g->nrad * g->nang) + (int64_t)itheta * g->nrad + i];
}

/* tex3D(CorrTex, x, z, 0.5f) over an (NRAD, NZS, 1) array: bilinear in
 * (radial, plane) with clamp; the third coordinate lands on texel 0 with
 * weight 0, which leaves the value unchanged. */
static real tex2_view(const gfo_geom* g, const real* arr, int64_t seg_base, int zmin, int itheta, real x, real z) {
  real xb = x - RL(0.5f), zb = z - RL(0.5f);
  real fx = r_floor(xb), fz = r_floor(zb);
  real a = xb - fx, b = zb - fz;
  int i = (int)fx, j = (int)fz;
  int i0 = clampi(i, 0, g->nrad - 1), i1 = clampi(i + 1, 0, g->nrad - 1);
  int j0 = clampi(j, 0, g->nzs - 1), j1 = clampi(j + 1, 0, g->nzs - 1);
  real t00 = view_texel(g, arr, seg_base, zmin, itheta, j0, i0);
  real t10 = view_texel(g, arr, seg_base, zmin, itheta, j0, i1);
  real t01 = view_texel(g, arr, seg_base, zmin, itheta, j1, i0);
  real t11 = view_texel(g, arr, seg_base, zmin, itheta, j1, i1);
  return lerp(lerp(t00, t10, a), lerp(t01, t11, a), b);
}

/* ------------------------------------------------------------------ */
/* Forward projector: FORWPROJ_K, GFIRST_GPU_Kernels.cu:40-102,       */
/* scattered into the sinogram as GFIRST.cu:346-365 does.             */
/* ------------------------------------------------------------------ */
void gfo_fp(const gfo_geom* g, const real* img, int32_t nsub, int32_t subset, real* proj) {
  const int NRAD = g->nrad, NANG = g->nang, NZS = g->nzs, RES = g->res;
  const int NPT = RES, NTBINS = 1;
  int32_t* acc = (int32_t*)malloc(sizeof(int32_t) * (size_t)(g->nseg + 1));
  gfo_segments(g, NULL, NULL, acc);
  const real FOV = RL(g->fov), PITCH = RL(g->pitch), DIAM = RL(g->diam), PI = RL(PI_REF);
  const int nviews = g->nseg * NANG;
#pragma omp parallel for schedule(dynamic, 1)
  for (int v = 0; v < nviews; v++) {
    int idz_ind = v / NANG, itheta = v % NANG;
    if (itheta % nsub != subset) continue;
    int idz = seg_idz(idz_ind);
    int zmin = 0, idz_signo = 0;
    if (idz == 0) zmin = 0; else { zmin = (abs(idz) - 1) * g->span + (g->span / 2 + 1); idz_signo = idz / abs(idz); }
    real vx = FOV / RL(RES);
    real px = RL(0.5f) * PITCH;
    real fx = px / vx;
    real fac = RL((float)RES) / RL((float)NPT);
    real TOF_size = RL((float)NPT) / RL((float)NTBINS);
    real RADM = RL(NRAD - 1) * RL(0.5f);
    real RESM = RL(RES - 1) * RL(0.5f);
    real ang_th = -RL(itheta) / RL(NANG) * PI + PI;
    real sin_th = r_sin(ang_th), cos_th = r_cos(ang_th);
    real dx = fac * sin_th, dy = -fac * cos_th;
    real dz = (FOV / RL(NPT)) * RL(idz_signo * zmin) / (RL(0.5f) * DIAM);
    int iTOF = 0;
    int init_point = (int)r_floor((RL(iTOF) - RL(0.5f)) * TOF_size);
    int end_point = (int)r_floor((RL(iTOF) + RL(0.5f)) * TOF_size);
    for (int iz0 = zmin; iz0 < NZS - zmin; iz0++) {
      for (int ix0 = 0; ix0 < NRAD; ix0++) {
        real x0 = fx * (RL(ix0) - RADM);
        real xc = RESM + (x0 * cos_th) + RL(0.5f);
        real yc = RESM + (x0 * sin_th) + RL(0.5f);
        real zc = RL(iz0) + RL(0.5f);
        real p = RL(0.0f);
        for (int lambda = init_point; lambda <= end_point; lambda++) {
          real x = xc + RL(lambda) * dx;
          real y = yc + RL(lambda) * dy;
          real z = zc + RL(lambda) * dz;
          p += tex3_img(g, img, x, y, z);
        }
        int64_t lor = ((int64_t)(iz0 - zmin) + acc[idz_ind]) * ((int64_t)NRAD * NANG) + (int64_t)itheta * NRAD + ix0;
        proj[lor] = p;
      }
    }
  }
  free(acc);
}

/* Ratio with gap sentinel, GFIRST.cu:413-430, over the bins of one subset. */
void gfo_ratio(const gfo_geom* g, const real* proj, const real* data, const real* bg, int32_t nsub,
               int32_t subset, real* corr) {
  const int64_t n = ndata_of(g);
  const int NRAD = g->nrad, NANG = g->nang;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    int itheta = (int)((i / NRAD) % NANG);
    if (itheta % nsub != subset) continue;
    real val_proy = proj[i], val_dato = data[i], val_bg = bg[i];
    if ((double)val_bg < 0.) val_bg = RL(0.0f);
    if (val_proy + val_bg >= RL(0.01f)) corr[i] = val_dato / (val_proy + val_bg);
    else corr[i] = RL(-1000.0f);
  }
}

/* Normalization gap mask, GFIRST.cu:453-458. */
void gfo_calib(const gfo_geom* g, const real* proj_blank, const real* blank, real* calib) {
  const int64_t n = ndata_of(g);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++)
    calib[i] = ((double)proj_blank[i] > 0.01 && (double)blank[i] > 0.01) ? RL(1.0f) : RL(-1000.0f);
}

/* ------------------------------------------------------------------ */
/* Back projector: BACKWPROJ_K, GFIRST_GPU_Kernels.cu:109-164, run    */
/* per view in the order of GFIRST.cu:436-469 (segments outer, angles */
/* inner), NUMER/DENOM cleared first (GFIRST.cu:436-437).             */
/* ------------------------------------------------------------------ */
void gfo_bp(const gfo_geom* g, const real* corr, const real* calib, int32_t nsub, int32_t subset, real* numer,
            real* denom) {
  const int RES = g->res, NZS = g->nzs, NRAD = g->nrad, NANG = g->nang;
  int32_t* acc = (int32_t*)malloc(sizeof(int32_t) * (size_t)(g->nseg + 1));
  gfo_segments(g, NULL, NULL, acc);
  const real FOV = RL(g->fov), PITCH = RL(g->pitch), DIAM = RL(g->diam), PI = RL(PI_REF);
  /* per-view constants */
  const int nviews = g->nseg * NANG;
  real* vsin = (real*)malloc(sizeof(real) * (size_t)nviews);
  real* vcos = (real*)malloc(sizeof(real) * (size_t)nviews);
  real* vfz = (real*)malloc(sizeof(real) * (size_t)nviews);
  int* vzmin = (int*)malloc(sizeof(int) * (size_t)nviews);
  real dxv = FOV / RL(RES);
  real px = (real)((double)PITCH / 2.0);
  real fx = dxv / px;
  real RADM = RL(NRAD - 1) * RL(0.5f);
  real RESM = RL(RES - 1) * RL(0.5f);
  for (int v = 0; v < nviews; v++) {
    int idz_ind = v / NANG, itheta = v % NANG;
    int idz = seg_idz(idz_ind), zmin, idz_signo = 0;
    if (idz == 0) zmin = 0; else { zmin = (abs(idz) - 1) * g->span + (g->span / 2 + 1); idz_signo = idz / abs(idz); }
    vzmin[v] = zmin;
    /* fz = (dx)*float(idz_signo*zmin)/(DIAM_DET/2.0): float product, double division */
    vfz[v] = (real)((double)(dxv * RL(idz_signo * zmin)) / ((double)DIAM / 2.0));
    real ang_th = -RL(itheta) / RL(NANG) * PI + PI;
    vsin[v] = r_sin(ang_th);
    vcos[v] = r_cos(ang_th);
  }
  const int64_t R2 = (int64_t)RES * RES;
#pragma omp parallel for schedule(static)
  for (int64_t iV = 0; iV < R2 * NZS; iV++) {
    int iz = (int)(iV / R2), iy = (int)((iV / RES) % RES), ix = (int)(iV % RES);
    real xv = RL(ix) - RESM;
    real yv = RL(iy) - RESM;
    real nsum = RL(0.0f), dsum = RL(0.0f);
    for (int idz_ind = 0; idz_ind < g->nseg; idz_ind++) {
      for (int itheta = subset; itheta < NANG; itheta += nsub) {
        int v = idz_ind * NANG + itheta;
        int zmin = vzmin[v];
        real sin_th = vsin[v], cos_th = vcos[v], fz = vfz[v];
        real xrot = xv * cos_th + yv * sin_th;
        real yrot = -xv * sin_th + yv * cos_th;
        real x = RADM + xrot * fx + RL(0.5f);
        real z = RL(iz) + yrot * fz + RL(0.5f);
        real c = RL(0.0f), cal = RL(0.0f);
        if (z >= RL(zmin) && z < RL(NZS - zmin)) {
          c = tex2_view(g, corr, acc[idz_ind], zmin, itheta, x, z);
          cal = tex2_view(g, calib, acc[idz_ind], zmin, itheta, x, z);
        }
        if (cal < RL(0.0f) || c < RL(0.0f)) { c = RL(0.0f); cal = RL(0.0f); }
        nsum += c;
        dsum += cal;
      }
    }
    numer[iV] = nsum;
    denom[iV] = dsum;
  }
  free(vsin); free(vcos); free(vfz); free(vzmin); free(acc);
}

/* ------------------------------------------------------------------ */
/* Image update chain                                                 */
/* ------------------------------------------------------------------ */

/* calcGaussianCoefficients, GFIRST_GPU_Kernels.cu:322-330 */
void gfo_gauss9(float psf, float* g9) {
  float total = 0.f;
  for (int z = -4; z <= 4; ++z) {
    float t = (float)z * 1.662f / (psf + 0.1f);
    total += expf(-(t * t));
  }
  int k = 0;
  for (int z = -4; z <= 4; ++z) {
    float t = (float)z * 1.662f / (psf + 0.1f);
    g9[k++] = expf(-(t * t)) / total;
  }
}

/* divVxVGPU, GFIRST_GPU_Kernels.cu:173-182 */
void gfo_div(const real* a, const real* b, int64_t n, real* r) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) r[i] = (b[i] < RL(0.001f)) ? RL(1.0f) : a[i] / b[i];
}

/* convolutionXY_GPU, GFIRST_GPU_Kernels.cu:332-358: y pass zero-padded,
 * x pass only for 3 < col < RES-4; border columns output the raw input. */
void gfo_conv_xy(const gfo_geom* g, const real* in, const float* g9, real* out) {
  const int RES = g->res, NZS = g->nzs;
  const int64_t R2 = (int64_t)RES * RES;
  real G[9];
  for (int k = 0; k < 9; k++) G[k] = RL(g9[k]);
#pragma omp parallel for schedule(static)
  for (int plane = 0; plane < NZS; plane++) {
    const real* src = in + plane * R2;
    real* dst = out + plane * R2;
    real* yconv = (real*)malloc(sizeof(real) * (size_t)RES);
    for (int c = 0; c < RES; c++) {
      for (int col = 0; col < RES; col++) {
        real acc = RL(0.0f);
        for (int k = 0; k < 9; k++) {
          int row = c - 4 + k;
          real v = (row >= 0 && row < RES) ? src[row * RES + col] : RL(0.0f);
          acc = (k == 0) ? v * G[0] : acc + v * G[k];
        }
        yconv[col] = acc;
      }
      for (int col = 0; col < RES; col++) {
        real xc = src[c * RES + col];
        if (col > 3 && col < RES - 4) {
          real acc = RL(0.0f);
          for (int k = 0; k < 9; k++) acc = (k == 0) ? yconv[col - 4] * G[0] : acc + yconv[col - 4 + k] * G[k];
          xc = acc;
        }
        dst[c * RES + col] = xc;
      }
    }
    free(yconv);
  }
}

/* gaussian_filterZ, GFIRST_CPU_Kernels.cpp:165-187, with its index shift:
 * the loop counter is incremented before use, so loop position (K,J,I)
 * writes voxel K*RES*RES+J*RES+I+1 with the rule of slice K.  Voxel 0 is
 * never written; the read and the write one past the end are taken as 0
 * and dropped. */
static inline real zin(const real* in, int64_t idx, int64_t n) { return (idx >= 0 && idx < n) ? in[idx] : RL(0.0f); }

void gfo_filter_z(const gfo_geom* g, const real* in, real* out) {
  const int RES = g->res, NZS = g->nzs;
  const int64_t R2 = (int64_t)RES * RES, n = R2 * NZS;
  float g1f[5];
  float total = 0.f;
  for (int z = -2; z <= 2; ++z) total += expf(-(((float)z * 1.0f) * ((float)z * 1.0f)));
  for (int k = 0, z = -2; z <= 2; ++z, ++k) g1f[k] = expf(-(((float)z * 1.0f) * ((float)z * 1.0f))) / total;
  real g1[5];
  for (int k = 0; k < 5; k++) g1[k] = RL(g1f[k]);
#pragma omp parallel for schedule(static)
  for (int64_t pos = 0; pos < n; pos++) {
    int K = (int)(pos / R2);
    int64_t iV = pos + 1;
    real v = RL(0.0f);
    int wrote = 0;
    if (K == 0) { v = RL(0.5f) * zin(in, iV, n) + RL(0.5f) * zin(in, iV + R2, n); wrote = 1; }
    if (K == NZS - 1) { v = RL(0.5f) * zin(in, iV - R2, n) + RL(0.5f) * zin(in, iV, n); wrote = 1; }
    if (K == 1 || K == NZS - 2) {
      v = RL(0.333f) * zin(in, iV - R2, n) + RL(0.333f) * zin(in, iV, n) + RL(0.333f) * zin(in, iV + R2, n);
      wrote = 1;
    }
    if (K > 1 && K < NZS - 2) {
      v = g1[0] * zin(in, iV - 2 * R2, n) + g1[1] * zin(in, iV - R2, n) + g1[2] * zin(in, iV, n) +
          g1[3] * zin(in, iV + R2, n) + g1[4] * zin(in, iV + 2 * R2, n);
      wrote = 1;
    }
    if (wrote && iV < n) out[iV] = v;
  }
}

/* Image update, GFIRST.cu:482-502: ratio, XY PSF, axial filter (its output
 * buffer holds DENOM beforehand, GFIRST.cu:471-472, so voxel 0 keeps
 * DENOM[0]), multiply, edge slices copied inwards. */
void gfo_update(const gfo_geom* g, real* img, const real* numer, const real* denom, const float* g9_bw) {
  const int64_t n = nvox_of(g), R2 = (int64_t)g->res * g->res;
  real* r = (real*)malloc(sizeof(real) * (size_t)n);
  real* c = (real*)malloc(sizeof(real) * (size_t)n);
  real* f = (real*)malloc(sizeof(real) * (size_t)n);
  gfo_div(numer, denom, n, r);
  gfo_conv_xy(g, r, g9_bw, c);
  memcpy(f, denom, sizeof(real) * (size_t)n);
  gfo_filter_z(g, c, f);
  for (int64_t i = 0; i < n; i++) img[i] *= f[i];
  for (int64_t i = 0; i < R2; i++) {
    img[i] = img[i + R2];
    img[i + (g->nzs - 1) * R2] = img[i + (g->nzs - 2) * R2];
  }
  free(r); free(c); free(f);
}

/* jointbilateralfilter3D_K, GFIRST_GPU_Kernels.cu:508-539.  The loop
 * counters are unsigned, so a window start below 0 wraps and the loop runs
 * zero times: voxels with any coordinate < r get norm 0 and output 0. */
void gfo_bilateral(const gfo_geom* g, const real* in, const real* ref, real max_ref, int32_t r, float sigma3d,
                   float sigmai, real* out) {
  const int RES = g->res, NZS = g->nzs;
  const int64_t R2 = (int64_t)RES * RES;
  const double ci = (2.0 * (double)sigmai) * (2.0 * (double)sigmai);
  const double cs = (2.0 * (double)sigma3d) * (2.0 * (double)sigma3d);
#pragma omp parallel for schedule(dynamic, 1)
  for (int iz = 0; iz < NZS; iz++) {
    for (int iy = 0; iy < RES; iy++) {
      for (int ix = 0; ix < RES; ix++) {
        int64_t iV = iz * R2 + (int64_t)iy * RES + ix;
        real ref_value = ref[iV];
        real norm = RL(0.0f), sum = RL(0.0f);
        if (ix >= r && iy >= r && iz >= r) {
          for (int izz = iz - r; izz <= iz + r; izz++)
            for (int iyy = iy - r; iyy <= iy + r; iyy++)
              for (int ixx = ix - r; ixx <= ix + r; ixx++) {
                if (ixx < RES && iyy < RES && izz < NZS) {
                  int64_t iW = izz * R2 + (int64_t)iyy * RES + ixx;
                  real di = (ref[iW] - ref_value) / max_ref;
                  real dist_intensity2 = di * di;
                  real dist_spatial2 = RL((float)((ixx - ix) * (ixx - ix) + (iyy - iy) * (iyy - iy) + (izz - iz) * (izz - iz)));
                  /* float H = exp(double expression); float G likewise */
                  real H = (real)exp((double)(-dist_intensity2) / ci);
                  real G = (real)exp((double)(-dist_spatial2) / cs);
                  norm += H * G;
                  sum += H * G * in[iW];
                }
              }
        }
        out[iV] = ((double)norm > 1e-8) ? sum / norm : RL(0.0f);
      }
    }
  }
}

/* GFIRST.cu:524: img2 = (1.0-filt_coef)*img2 + filt_coef*filtered */
void gfo_blend(int64_t n, real* img2, const real* filtered) {
  const float filt_coef = 0.1f;
  for (int64_t i = 0; i < n; i++)
    img2[i] = (real)((1.0 - (double)filt_coef) * (double)img2[i] + (double)(RL(filt_coef) * filtered[i]));
}

/* GFIRST.cu:515, 521 */
real gfo_max_ref(int64_t n, const real* img) {
  real m = RL(0.0f);
  for (int64_t i = 0; i < n; i++) if (img[i] > m) m = img[i];
  return m;
}

/* VLOR count pass, GFIRST.cu:229-240 (cnt must be zeroed by the caller) */
void gfo_vlor_count(const gfo_geom* g, const int32_t* ev, int64_t nev, real* cnt) {
  const int64_t NDATA = ndata_of(g);
  for (int64_t e = 0; e < nev; e++) {
    int64_t i1 = (int64_t)ev[2 * e] - 1, i2 = (int64_t)ev[2 * e + 1] - 1;
    if (i1 <= 0 || i2 <= 0 || i1 >= NDATA || i2 >= NDATA) continue;
    cnt[i1] += RL(1.0f);
    cnt[i2] += RL(1.0f);
  }
}

/* BLANKT, GFIRST.cu:244-247 (datos_t already scaled by RES) */
void gfo_blankt(const gfo_geom* g, const real* cnt, const real* datos_t, real* blankt) {
  const int64_t NDATA = ndata_of(g);
  for (int64_t i = 0; i < NDATA; i++) {
    real val = cnt[i];
    blankt[i] = ((double)val > 0.01) ? datos_t[i] / (RL(g->res) * val) : RL(0.0f);
  }
}

/* VLOR split, GFIRST.cu:373-389 (out must be zeroed by the caller) */
void gfo_vlor_split(const gfo_geom* g, const int32_t* ev, int64_t nev, const real* proj, const real* blankt,
                    real* out) {
  const int64_t NDATA = ndata_of(g);
  for (int64_t e = 0; e < nev; e++) {
    int64_t i1 = (int64_t)ev[2 * e] - 1, i2 = (int64_t)ev[2 * e + 1] - 1;
    if (i1 <= 0 || i2 <= 0 || i1 >= NDATA || i2 >= NDATA) continue;
    real valor = blankt[i1] + blankt[i2];
    real s1 = proj[i1], s2 = proj[i2];
    real s = s1 + s2;
    real s_inv = (s > RL(0.01f)) ? (real)(1.0 / (double)s) : RL(0.0f);
    out[i1] += s1 * s_inv * valor;
    out[i2] += s2 * s_inv * valor;
  }
}

/* Output image, GFIRST.cu:532-549: scale, then zero outside radius RESM-1. */
void gfo_output_image(const gfo_geom* g, const real* img, float scale, real* out) {
  const int RES = g->res;
  const int RESM = RES / 2;
  int64_t iV = 0;
  for (int z = 0; z < g->nzs; z++)
    for (int y = 0; y < RES; y++)
      for (int x = 0; x < RES; x++, iV++) {
        float dist = (float)((x - RESM) * (x - RESM) + (y - RESM) * (y - RESM) - (RESM - 1) * (RESM - 1));
        out[iV] = (dist > 0.f) ? RL(0.0f) : img[iV] * RL(scale);
      }
}

/* ------------------------------------------------------------------ */
/* Whole reconstruction: osem3d, GFIRST.cu:44-575, with subsets        */
/* (angle t in subset t % nsub, subsets visited in order inside each   */
/* type; nsub = 1 is the reference loop).                              */
/* ------------------------------------------------------------------ */
int gfo_recon(const gfo_geom* g, const gfo_params* p, const real* image, const real* dsino, const real* tsino,
              const real* norm, const int32_t* ev, int64_t nev, real* proj_ref, real* img_d, real* img_t,
              real* sinog_vlor) {
  if (gfo_planes(g) < 0 || p->nsub < 1 || p->nsub > g->nang) return -1;
  const int64_t NDATA = ndata_of(g), NVOX = nvox_of(g);
  const int mode = p->mode, S = p->nsub;
  const real RES_F = RL(g->res);
  real* pref = (real*)calloc((size_t)NDATA, sizeof(real));
  real* img = (real*)malloc(sizeof(real) * (size_t)NVOX);

  /* STEP 1: projection of the input image (mode 0) or of a unit cylinder */
  if (mode == 0) memcpy(img, image, sizeof(real) * (size_t)NVOX);
  else gfo_cylinder(g, RL(1.0f), img);
  gfo_fp(g, img, 1, 0, pref);
  if (proj_ref) memcpy(proj_ref, pref, sizeof(real) * (size_t)NDATA);
  if (mode == 0) { free(pref); free(img); return 0; }

  /* STEP 2: data */
  real* calib = (real*)malloc(sizeof(real) * (size_t)NDATA);
  gfo_calib(g, pref, norm, calib);
  real* dd = (real*)malloc(sizeof(real) * (size_t)(2 * NDATA));
  for (int64_t i = 0; i < 2 * NDATA; i++) dd[i] = RES_F * dsino[i];
  real* dt = NULL;
  real *blankt = NULL, *datos_v = NULL;
  if (mode >= 2) {
    dt = (real*)malloc(sizeof(real) * (size_t)(2 * NDATA));
    for (int64_t i = 0; i < 2 * NDATA; i++) dt[i] = RES_F * tsino[i];
  }
  if (mode == 3) {
    real* cnt = (real*)calloc((size_t)NDATA, sizeof(real));
    gfo_vlor_count(g, ev, nev, cnt);
    blankt = (real*)malloc(sizeof(real) * (size_t)NDATA);
    gfo_blankt(g, cnt, dt, blankt);
    free(cnt);
    datos_v = (real*)malloc(sizeof(real) * (size_t)NDATA);
  }
  int ntypes = (mode == 1) ? 1 : 2;

  /* STEP 3: initial images */
  real* im[2];
  im[0] = img;
  gfo_cylinder(g, RL(1.0f), im[0]);
  im[1] = (real*)malloc(sizeof(real) * (size_t)NVOX);
  gfo_cylinder(g, (mode == 1) ? RL(0.0f) : RL(1.0f), im[1]);

  float gfw[9], gbw[9];
  gfo_gauss9(p->psf_fw, gfw);
  gfo_gauss9(p->psf_bw, gbw);
  real* psf = (real*)malloc(sizeof(real) * (size_t)NVOX);
  real* proj = (real*)calloc((size_t)NDATA, sizeof(real));
  real* corr = (real*)calloc((size_t)NDATA, sizeof(real));
  real* numer = (real*)malloc(sizeof(real) * (size_t)NVOX);
  real* denom = (real*)malloc(sizeof(real) * (size_t)NVOX);
  real* filt = (real*)malloc(sizeof(real) * (size_t)NVOX);
  real* tproj = NULL; /* triples projection cache for the VLOR split */
  if (mode == 3) {
    tproj = (real*)calloc((size_t)NDATA, sizeof(real));
    gfo_conv_xy(g, im[1], gfw, psf);
    gfo_fp(g, psf, 1, 0, tproj);
  }

  /* STEP 4: iterations */
  for (int iter = 1; iter <= p->niter; iter++) {
    for (int itype = 0; itype < ntypes; itype++) {
      for (int s = 0; s < S; s++) {
        gfo_conv_xy(g, im[itype], gfw, psf);
        real* pr = (mode == 3 && itype == 1) ? tproj : proj;
        gfo_fp(g, psf, S, s, pr);
        const real *dat, *bgp;
        if (itype == 0) { dat = dd; bgp = dd + NDATA; }
        else if (mode == 2) { dat = dt; bgp = dt + NDATA; }
        else {
          memset(datos_v, 0, sizeof(real) * (size_t)NDATA);
          gfo_vlor_split(g, ev, nev, tproj, blankt, datos_v);
          if (sinog_vlor) memcpy(sinog_vlor, datos_v, sizeof(real) * (size_t)NDATA);
          for (int64_t i = 0; i < NDATA; i++) datos_v[i] *= RES_F;
          dat = datos_v; bgp = dt + NDATA;
        }
        gfo_ratio(g, pr, dat, bgp, S, s, corr);
        gfo_bp(g, corr, calib, S, s, numer, denom);
        gfo_update(g, im[itype], numer, denom, gbw);
        /* joint filter once per iteration, after the triples type's last subset */
        if (itype == 1 && s == S - 1) {
          real max_ref = gfo_max_ref(NVOX, im[0]);
          gfo_bilateral(g, im[1], im[0], max_ref, 4, 0.75f, 0.025f, filt);
          gfo_blend(NVOX, im[1], filt);
        }
      }
    }
  }
  if (img_d) memcpy(img_d, im[0], sizeof(real) * (size_t)NVOX);
  if (img_t) memcpy(img_t, im[1], sizeof(real) * (size_t)NVOX);
  free(pref); free(calib); free(dd); free(dt); free(blankt); free(datos_v); free(im[0]); free(im[1]);
  free(psf); free(proj); free(corr); free(numer); free(denom); free(filt); free(tproj);
  return 0;
}
