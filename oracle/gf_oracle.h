/*
 * gf_oracle.h -- CPU restatement of GFIRST's OSEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle the GPU library is
 * checked against; only tests/, __graft_entry__.smoke() and the CPU-baseline
 * leg of bench.py load it.  The product never links or calls it.
 *
 * One source, two builds: liboracle_f32.so (GFO_REAL=float, the parity
 * oracle, follows the reference's FP32 expressions literally) and
 * liboracle_f64.so (GFO_REAL=double, the accuracy oracle: the same formulas
 * and the same float geometry constants, evaluated in double).
 *
 * All arrays use the reference's file layouts:
 *   image    [NZS][RES][RES]     x fastest       (GFIRST_CPU_Kernels.cpp:58-66)
 *   sinogram [P][NANG][NRAD]     radial fastest  (GFIRST.cu:175-176)
 * where P = nz_acum[NSEG] is the number of sinogram planes.
 */
#ifndef GF_ORACLE_H
#define GF_ORACLE_H
#include <stdint.h>

#ifndef GFO_REAL
#define GFO_REAL float
#endif
typedef GFO_REAL gfo_real;

#ifdef __cplusplus
extern "C" {
#endif

/* Scanner + image geometry; the reference holds these as compile-time
 * constants (GFIRST.h:4-36).  Lengths are in mm and kept as float, like the
 * reference's __constant__ floats. */
typedef struct gfo_geom {
  int32_t res, nzs, nrad, nang, span, nseg;
  float pitch, diam, fov;
} gfo_geom;

/* Reconstruction parameters (GFIRST.h:21-30 plus the subset count, which the
 * reference declares but never uses: NSUBSETS=1, GFIRST.h:22). */
typedef struct gfo_params {
  int32_t mode;      /* 0 projection, 1 doubles, 2 doubles+triples, 3 doubles + triples VLOR */
  int32_t nsub;      /* subsets; angle t belongs to subset t % nsub */
  int32_t niter;
  float psf_fw, psf_bw;
} gfo_params;

int64_t gfo_planes(const gfo_geom* g);            /* P, or -1 when a segment has no planes */
void gfo_segments(const gfo_geom* g, int32_t* idz, int32_t* zmin, int32_t* nz_acum);
int64_t gfo_lor(const gfo_geom* g, int32_t seg_ind, int32_t iz0, int32_t itheta, int32_t ird);

void gfo_cylinder(const gfo_geom* g, gfo_real val, gfo_real* img);
void gfo_fp(const gfo_geom* g, const gfo_real* img, int32_t nsub, int32_t subset, gfo_real* proj);
void gfo_ratio(const gfo_geom* g, const gfo_real* proj, const gfo_real* data, const gfo_real* bg,
               int32_t nsub, int32_t subset, gfo_real* corr);
void gfo_calib(const gfo_geom* g, const gfo_real* proj_blank, const gfo_real* blank, gfo_real* calib);
void gfo_bp(const gfo_geom* g, const gfo_real* corr, const gfo_real* calib, int32_t nsub,
            int32_t subset, gfo_real* numer, gfo_real* denom);
void gfo_gauss9(float psf, float* g9);
void gfo_div(const gfo_real* a, const gfo_real* b, int64_t n, gfo_real* r);
void gfo_conv_xy(const gfo_geom* g, const gfo_real* in, const float* g9, gfo_real* out);
void gfo_filter_z(const gfo_geom* g, const gfo_real* in, gfo_real* out);
void gfo_update(const gfo_geom* g, gfo_real* img, const gfo_real* numer, const gfo_real* denom,
                const float* g9_bw);
void gfo_bilateral(const gfo_geom* g, const gfo_real* in, const gfo_real* ref, gfo_real max_ref,
                   int32_t r, float sigma3d, float sigmai, gfo_real* out);
void gfo_blend(int64_t n, gfo_real* img2, const gfo_real* filtered);
gfo_real gfo_max_ref(int64_t n, const gfo_real* img);
void gfo_vlor_count(const gfo_geom* g, const int32_t* ev, int64_t nev, gfo_real* cnt);
void gfo_blankt(const gfo_geom* g, const gfo_real* cnt, const gfo_real* datos_t, gfo_real* blankt);
void gfo_vlor_split(const gfo_geom* g, const int32_t* ev, int64_t nev, const gfo_real* proj,
                    const gfo_real* blankt, gfo_real* out);
void gfo_output_image(const gfo_geom* g, const gfo_real* img, float scale, gfo_real* out);

/* Whole reconstruction of one CLI mode.  Inputs are the already-parsed files:
 * image (mode 0, NVOX), dsino/tsino (2*NDATA each: prompts then background,
 * not yet scaled by RES), norm (NDATA), ev (nev int32 pairs, 1-based bins,
 * end-of-file duplicate already applied).  Outputs (any may be NULL):
 * proj_ref (NDATA), img_d/img_t (NVOX, raw images after niter iterations),
 * sinog_vlor (NDATA, last VLOR split before the RES scaling).
 * Returns 0, or -1 for an invalid geometry. */
int gfo_recon(const gfo_geom* g, const gfo_params* p, const gfo_real* image,
              const gfo_real* dsino, const gfo_real* tsino, const gfo_real* norm,
              const int32_t* ev, int64_t nev, gfo_real* proj_ref, gfo_real* img_d,
              gfo_real* img_t, gfo_real* sinog_vlor);

int gfo_real_bytes(void);
int gfo_threads(void);

#ifdef __cplusplus
}
#endif
#endif
