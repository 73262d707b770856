/*
 * gfirst.h -- C-ABI of the GB300 (sm_103a) GFIRST OSEM hot path.
 *
 * The reference (jlherraiz/GFIRST) is one program with no library API: its
 * hot path is reached through the command line (GFIRST.cu:577-621), its raw
 * file formats (GFIRST_CPU_Kernels.cpp:25-142), and, inside the program, the
 * per-view host wrappers FORWPROJ/BACKWPROJ/... of GFIRST_GPU_Kernels.cu that
 * osem3d() (GFIRST.cu:44-575) calls.  Each entry point below names the
 * reference interface it replaces.  Conventions:
 *  - plain pointers and sizes only; every call returns gf_status, never exits;
 *  - `d_` pointers are device memory, `h_` pointers host memory;
 *  - device arrays use the reference's layouts: images [NZS][RES][RES]
 *    (x fastest), sinograms [P][NANG][NRAD] (radial fastest), P = planes;
 *  - work is queued on the context's stream (gf_set_stream); a
 *    reconstruction's host-to-device loads and image read-backs run on the
 *    context's own copy stream, ordered against that stream by events; calls
 *    that take host buffers return after their results are in host memory;
 *  - a context is used by one host thread at a time.
 */
#ifndef GFIRST_H
#define GFIRST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GF_ABI_VERSION 3

typedef enum gf_status {
  GF_OK = 0,
  GF_ERR_ARG = 1,      /* null pointer, size or mode out of range */
  GF_ERR_GEOMETRY = 2, /* a segment has no planes, or sizes out of range */
  GF_ERR_CUDA = 3,     /* a CUDA call failed (text in gf_last_error) */
  GF_ERR_NOMEM = 4,    /* device allocation failed or over the memory budget */
  GF_ERR_IO = 5,       /* file missing, unreadable or unwritable */
  GF_ERR_STATE = 6,    /* call out of order */
  GF_ERR_NODEV = 7,    /* no usable CUDA device */
  GF_ERR_TIMEOUT = 8   /* a bounded device wait gave up */
} gf_status;

/* Scanner and image geometry: the compile-time constants of GFIRST.h:4-36
 * (RES, NZS, NRAD, NANG, SPAN, NSEGMENTS, pitch, DIAM_DET, FOV), here chosen
 * at run time.  NPT = RES and one TOF bin, as in the reference. */
typedef struct gf_geometry {
  int32_t res, nzs, nrad, nang, span, nseg;
  float pitch_mm, diam_det_mm, fov_mm;
} gf_geometry;

typedef struct gf_ctx gf_ctx;
typedef struct gf_recon gf_recon;

/* ---- version, errors ---------------------------------------------------- */
int32_t gf_abi_version(void);
/* Text of the last error on this host thread (empty when none). */
const char* gf_last_error(void);

/* ---- geometry (GFIRST.h:4-36; GFIRST.cu:133-140, 163-176) ---------------- */
/* The constants compiled into the reference (GFIRST.h:4-36). */
gf_status gf_geometry_reference(gf_geometry* out);
/* planes P = nz_acum[NSEG] (GFIRST.h:9 NSINOGS), NDATA = P*NANG*NRAD
 * (GFIRST.h:11), NVOX = RES*RES*NZS (GFIRST.h:16). */
gf_status gf_geometry_sizes(const gf_geometry* g, int64_t* planes, int64_t* ndata, int64_t* nvox);
/* Segment order 0,-1,+1,-2,+2,... (GFIRST.cu:163-168), zmin
 * (GFIRST_GPU_Kernels.cu:54) and nz_acum (GFIRST.cu:133-140, nseg+1 entries). */
gf_status gf_segment_table(const gf_geometry* g, int32_t* idz, int32_t* zmin, int32_t* nz_acum);
/* Sinogram bin of a line of response, GFIRST.cu:175-176. */
gf_status gf_lor_index(const gf_geometry* g, int32_t seg_ind, int32_t iz0, int32_t itheta, int32_t ird,
                       int64_t* lor);

/* ---- context -------------------------------------------------------------- */
/* Replaces the global set-up of osem3d() (textures and cudaMallocs,
 * GFIRST.cu:57-83; crearTexturas, GFIRST_GPU_Kernels.cu:254-281).  Angles
 * t with t % nsubsets == s form subset s; nsubsets = 1 is the reference's
 * loop over all angles (NSUBSETS = 1, GFIRST.h:22). */
gf_status gf_create(const gf_geometry* g, int32_t nsubsets, int32_t device, gf_ctx** out);
/* Also destroys the reconstructions still open on the context. */
void gf_destroy(gf_ctx* ctx);
/* Queue later work on this cudaStream_t (NULL: the context's own stream).  The
 * stream must stay valid while the context queues work on it. */
gf_status gf_set_stream(gf_ctx* ctx, void* cuda_stream);
gf_status gf_synchronize(gf_ctx* ctx);

/* Axial interpolation of the back projector (BACKWPROJ_K,
 * GFIRST_GPU_Kernels.cu:148-152: z = float(iz) + yrot*fz + 0.5f per voxel).
 * GF_BP_PER_VOXEL takes z with that rounding for every voxel, so NUMER and
 * DENOM are the FP32 oracle's sums bit for bit.  GF_BP_PER_VIEW takes the
 * axial fraction of yrot*fz once per (column, view) for all voxels of the
 * column -- an interpolation weight moves by at most one unit in the last
 * place of iz + yrot*fz (about 1e-5 relative in the sums) -- and lets voxels
 * outside the segment's planes fall to the gap rule through sentinel rows
 * instead of a range test.  The reference's own hardware interpolation
 * quantises these weights to 1/256.  Default GF_BP_PER_VIEW.  The form
 * applies to gf_back_project and to the doubles image of reconstructions;
 * triples images (modes 2-3) always take GF_BP_PER_VOXEL: their data are
 * mostly zero, and where a ratio of 0 meets a gap sentinel the reference's
 * gap rule turns on whether a weight rounds to exactly 0. */
enum { GF_BP_PER_VOXEL = 0, GF_BP_PER_VIEW = 1 };
gf_status gf_set_bp_form(gf_ctx* ctx, int32_t form);
/* The per-view form's staged-row buffer for a geometry (no device work): a
 * view's rows sit at offset pad_lo of rbuf (corr, calib) pairs per warp, the
 * rest hold the gap sentinel; pad_hi rows past a segment's last row are
 * read.  Shared memory per 4-warp block: 4 * (16 * angles per subset + 8 *
 * rbuf) bytes. */
gf_status gf_bp_staged_rows(const gf_geometry* g, int32_t* pad_lo, int32_t* pad_hi, int32_t* rbuf);

/* Device memory helpers for callers without a CUDA runtime of their own. */
gf_status gf_device_alloc(gf_ctx* ctx, size_t bytes, void** d_ptr);
gf_status gf_device_free(gf_ctx* ctx, void* d_ptr);
/* Page-locked host memory (fast host<->device copies). */
gf_status gf_host_alloc(size_t bytes, void** h_ptr);
gf_status gf_host_free(void* h_ptr);
/* Synchronous copies on the context's stream. */
gf_status gf_copy_to_device(gf_ctx* ctx, void* d_dst, const void* h_src, size_t bytes);
gf_status gf_copy_to_host(gf_ctx* ctx, void* h_dst, const void* d_src, size_t bytes);

/* ---- operators on device buffers (file layouts) -------------------------- */
/* Forward projection of every (segment, angle) view of one subset into the
 * sinogram; bins of other subsets are left untouched.  Replaces FORWPROJ
 * (GFIRST_GPU_Kernels.cu:105-107, kernel :40-102) looped with its scatter
 * (GFIRST.cu:346-365).  No PSF is applied. */
gf_status gf_forward_project(gf_ctx* ctx, const float* d_image, int32_t subset, float* d_proj);
/* Data/projection ratio with the gap sentinel over one subset's bins:
 * corr = data/(proj+max(bg,0)) when proj+bg >= 0.01, else -1000.
 * Replaces the host loop of GFIRST.cu:413-430. */
gf_status gf_ratio(gf_ctx* ctx, const float* d_proj, const float* d_data, const float* d_bg, int32_t subset,
                   float* d_corr);
/* Normalization mask calib = 1 where proj_blank > 0.01 and blank > 0.01, else
 * -1000 (GFIRST.cu:453-458). */
gf_status gf_norm_mask(gf_ctx* ctx, const float* d_proj_blank, const float* d_blank, float* d_calib);
/* Back projection of one subset: clears numer/denom, then accumulates every
 * (segment, angle) view of the subset in the reference's order.  Replaces
 * BACKWPROJ (GFIRST_GPU_Kernels.cu:166-171, kernel :109-164) looped with its
 * gather (GFIRST.cu:436-469). */
gf_status gf_back_project(gf_ctx* ctx, const float* d_corr, const float* d_calib, int32_t subset,
                          float* d_numer, float* d_denom);
/* XY Gaussian PSF (9 taps, border columns passed through).  Replaces
 * calcGaussianCoefficients + convolutionXY (GFIRST_GPU_Kernels.cu:322-364). */
gf_status gf_psf_xy(gf_ctx* ctx, const float* d_in, float psf, float* d_out);
/* Multiplicative update, in place: ratio numer/denom (1 where denom<0.001),
 * XY PSF, axial filter, multiply, edge slices copied inwards.  Replaces
 * GFIRST.cu:482-502 (dividirVxVGPU, convolutionXY, gaussian_filterZ of
 * GFIRST_CPU_Kernels.cpp:165-187). */
gf_status gf_image_update(gf_ctx* ctx, float* d_image, const float* d_numer, const float* d_denom, float psf_bw);
/* Joint bilateral filter of `in` guided by `ref`.  Replaces
 * jointbilateralfilter3D (GFIRST_GPU_Kernels.cu:508-543). */
gf_status gf_bilateral(gf_ctx* ctx, const float* d_in, const float* d_ref, float max_ref, int32_t r,
                       float sigma3d, float sigmai, float* d_out);
/* VLOR end counts (d_count must be zeroed by the caller), GFIRST.cu:229-240.
 * Events are int32 pairs of 1-based bins. */
gf_status gf_vlor_count(gf_ctx* ctx, const int32_t* d_events, int64_t nevents, float* d_count);
/* VLOR split of each event between its two bins in proportion to d_proj,
 * added to d_out (zeroed by the caller for the reference's SINOG_VLOR),
 * GFIRST.cu:373-389.  Each bin's shares are added in event order, as the
 * reference's loop adds them, so the result is the reference's bit for bit;
 * the ordering uses device temporaries of 40 bytes per event. */
gf_status gf_vlor_split(gf_ctx* ctx, const int32_t* d_events, int64_t nevents, const float* d_proj,
                        const float* d_blankt, float* d_out);

/* ---- forward projection without device allocation ------------------------ */
/* Size of the fixed device scratch behind gf_forward_project_noalloc. */
#define GF_NOALLOC_SCRATCH_BYTES (16u << 20)
/* Forward projection of one subset, as gf_forward_project, for callers that
 * cannot allocate device memory (a host that owns the whole device memory
 * map, an embedding framework with its own pool, code where an allocation
 * would stall or be refused).  No counterpart in the reference.  Needs no
 * context and calls no cudaMalloc/cudaFree: its scratch (the image
 * transposed to z-fastest order plus the geometry tables) lives in one
 * file-scope device array of GF_NOALLOC_SCRATCH_BYTES bytes, held by every
 * GPU that loads the library until the process exits.  Geometries whose
 * scratch exceeds it (image RES*RES*NZS padded to 32 slices, about 4.1 M
 * voxels) are rejected with GF_ERR_ARG.  Runs on the current device and on
 * `cuda_stream` (NULL: the legacy default stream).  The first call on a
 * device looks up the array's device address and keeps it for the life of
 * the process, so a cudaDeviceReset of that device ends this entry point's
 * use there.  All calls share the array: calls whose work overlaps on the
 * GPU race. */
gf_status gf_forward_project_noalloc(const gf_geometry* g, int32_t nsubsets, int32_t subset, const float* d_image,
                                     float* d_proj, void* cuda_stream);

/* ---- VLOR events as LOR endpoints (no counterpart in the reference, whose
 * VLOR file holds int32 pairs of 1-based bins, GFIRST.cu:213-240) ---------- */
/* Endpoints in mm of the line of response of sinogram bin `bin` (0-based):
 * out6 = (x1,y1,z1,x2,y2,z2), both ends on the detector ring (radius
 * DIAM_DET/2), x/y about the scanner axis, z about the centre of the axial
 * field of view.  The line is the one the forward projector samples for that
 * bin (GFIRST_GPU_Kernels.cu:75-96). */
gf_status gf_bin_endpoints(const gf_geometry* g, int64_t bin, float* out6);
/* The same for n bins: out holds 6 floats per bin. */
gf_status gf_bins_endpoints(const gf_geometry* g, int64_t n, const int64_t* bins, float* out);
/* Converts n VLOR events given as two LORs each (12 float32 per event:
 * endpoints of the first candidate LOR, then of the second) to the
 * reference's event format (int32 pairs of 1-based bins; 0 where a LOR falls
 * outside the sinogram).  Inverse of gf_bin_endpoints at bin centres: angle
 * from the in-plane direction, radial bin from the distance to the axis,
 * segment from the axial slope, plane from the axial position at the point
 * closest to the axis. */
gf_status gf_vlor_from_endpoints(gf_ctx* ctx, const float* d_lors, int64_t nevents, int32_t* d_events);

/* ---- whole reconstruction -------------------------------------------------- */
/* The four CLI modes of GFIRST.cu:588-617: 0 projection of an image,
 * 1 doubles sinogram + normalization, 2 doubles + triples sinograms,
 * 3 doubles sinogram + triples VLOR list. */
typedef struct gf_recon_params {
  int32_t mode;
  int32_t niter;   /* NITER, GFIRST.h:21 */
  float psf_fw;    /* PSF_FW, GFIRST.h:26 */
  float psf_bw;    /* PSF_BW, GFIRST.h:27 */
  float scale_d;   /* scale_D, GFIRST.h:29 */
  float scale_t;   /* scale_T, GFIRST.h:30 */
  int32_t storage; /* per-subset (ratio, mask) sinogram storage: GF_STORE_F32
                      (the reference's precision), GF_STORE_F16 or
                      GF_STORE_BF16; arithmetic stays FP32 */
  int32_t image_storage; /* storage of the reconstructed images (doubles,
                            and triples in modes 2-3) between
                            sub-iterations: GF_STORE_F32 (the reference),
                            GF_STORE_F16 or GF_STORE_BF16 (every update and
                            the joint filter's blend round the image to 16
                            bits; arithmetic stays FP32); not for mode 0 */
} gf_recon_params;

enum { GF_STORE_F32 = 0, GF_STORE_F16 = 1, GF_STORE_BF16 = 2 };

/* Reference defaults (GFIRST.h:21-30). */
gf_status gf_recon_defaults(int32_t mode, gf_recon_params* out);
/* Allocates every device buffer of one reconstruction and keeps it resident. */
gf_status gf_recon_create(gf_ctx* ctx, const gf_recon_params* p, gf_recon** out);
void gf_recon_destroy(gf_recon* r);
/* Inputs are the parsed files (gf_read_* below): h_dsino/h_tsino 2*NDATA
 * floats (prompts then background, before the RES scaling), h_norm NDATA
 * floats, h_events nevents int32 pairs; unused inputs may be NULL.  Runs the
 * normalization projection (GFIRST.cu:151-184) and the data set-up
 * (GFIRST.cu:207-288).  Mode 0 takes h_image (NVOX floats) instead. */
gf_status gf_recon_load(gf_recon* r, const float* h_image, const float* h_dsino, const float* h_tsino,
                        const float* h_norm, const int32_t* h_events, int64_t nevents);
/* The same work queued without waiting for it (no counterpart in the
 * reference): the host-to-device copies go on the context's copy stream, the
 * data set-up that follows them on the context's stream.  The host buffers
 * must stay untouched until the load has run (gf_synchronize, or a call that
 * returns host results such as gf_recon_get_image).  With two
 * reconstructions of one context, the next data set's copies overlap the
 * current one's iterations. */
gf_status gf_recon_load_async(gf_recon* r, const float* h_image, const float* h_dsino, const float* h_tsino,
                              const float* h_norm, const int32_t* h_events, int64_t nevents);
/* Back to the initial images of GFIRST.cu:282-288 (and the initial triples
 * projection of mode 3) without reloading the data; progress restarts at 0. */
gf_status gf_recon_restart(gf_recon* r);
/* Queue n full iterations (every type, every subset), GFIRST.cu:303-564. */
gf_status gf_recon_iterate(gf_recon* r, int32_t n);
/* Queue one sub-iteration (one type, one subset) and advance the cursor. */
gf_status gf_recon_subiteration(gf_recon* r);
/* Completed iterations and sub-iterations so far. */
gf_status gf_recon_progress(const gf_recon* r, int32_t* iterations, int64_t* subiterations);
/* Image of type 0 (doubles) or 1 (triples), file layout, NVOX floats.
 * scaled != 0 applies the output scaling and mask of GFIRST.cu:532-549.
 * Waits for this reconstruction's queued work only: the read runs on the
 * context's copy stream, so work queued since for other reconstructions of
 * the context keeps running. */
gf_status gf_recon_get_image(gf_recon* r, int32_t type, int32_t scaled, float* h_out);
/* proj_ref.raw contents (GFIRST.cu:183-184), NDATA floats. */
gf_status gf_recon_get_proj_ref(gf_recon* r, float* h_out);
/* SINOG_VLOR.raw contents of the last triples sub-iteration (GFIRST.cu:391-394). */
gf_status gf_recon_get_sinog_vlor(gf_recon* r, float* h_out);

/* ---- batches of frames (no counterpart in the reference, which
 * reconstructs one acquisition per run) ------------------------------------ */
typedef struct gf_batch gf_batch;
/* Groups loaded reconstructions (frames) that advance together; frames may
 * have different subset counts and modes, each keeps its own resident data.
 * The recons must outlive the batch. */
gf_status gf_batch_create(int32_t nframes, gf_recon* const* frames, gf_batch** out);
void gf_batch_destroy(gf_batch* b);
/* Advances every frame by n full iterations.  With use_graph != 0 one
 * iteration of all frames is captured once into a CUDA graph -- each frame's
 * kernels on its own branch, so frames overlap on the device -- and replayed
 * n times; frames must stand at an iteration boundary.  With use_graph = 0
 * the kernels are launched directly, frame by frame.  Asynchronous. */
gf_status gf_batch_iterate(gf_batch* b, int32_t n, int32_t use_graph);
gf_status gf_batch_synchronize(gf_batch* b);
/* With fused = 1 or 2, mode-1 frames that share geometry, storage, filters,
 * back-projector form and tile shapes advance as fused groups of up to 16,
 * whatever their subset counts: step s of a group's iteration runs the
 * frames that have a subset s, each at its own subset s; the forward PSF,
 * projection + ratio and update are one kernel launch over those frames and
 * the back projection one launch per subset count among them, each frame
 * keeping its own data and results (the same as alone, bit for bit).  With fused = 1, frames of a group with the
 * same subset count and equal normalization masks (checked on the device),
 * back projector in the per-view form, back-project two per warp, sharing
 * the per-view geometry and the staged mask rows; fused = 2 keeps one frame
 * per warp.  Other frames run on their own.  0 turns fusing off.  Takes
 * effect at the next iterate. */
gf_status gf_batch_set_fused(gf_batch* b, int32_t fused);
/* Units the batch runs (fused groups and single frames), the size of the
 * largest group and the frame pairs back-projected together, as they stand
 * now (waits for the frames' queued work to compare their masks). */
gf_status gf_batch_groups(gf_batch* b, int32_t* units, int32_t* largest, int32_t* paired);

/* ---- serving (no counterpart in the reference) ---------------------------- */
/* Device bytes a reconstruction of these parameters holds (admission control). */
gf_status gf_recon_bytes(const gf_geometry* g, int32_t nsubsets, const gf_recon_params* p, int64_t nevents,
                         int64_t* bytes);

typedef struct gf_server gf_server;
enum { GF_REQ_RECON = 0, GF_REQ_PROJECT = 1 };
/* One request.  RECON: a mode-1 reconstruction of h_dsino (2*NDATA) and
 * h_norm (NDATA), niter iterations, result = the raw doubles image (NVOX) in
 * h_out.  PROJECT: the projection of h_image (NVOX), result = NDATA floats in
 * h_out.  Host buffers must stay valid until the request completes. */
typedef struct gf_request {
  int32_t kind;
  gf_geometry geometry;
  int32_t nsubsets;
  int32_t niter;
  int32_t storage;  /* GF_STORE_* */
  const float* h_image;
  const float* h_dsino;
  const float* h_norm;
  float* h_out;
} gf_request;
typedef struct gf_server_stats {
  int64_t submitted, completed, failed, queued, active;
  double p50_ms, p99_ms, mean_ms, max_ms;  /* submit-to-result latency of completed requests;
                                              p50/p99 from 1 %-wide log bins (within 0.5 %),
                                              mean and max exact */
  double throughput_per_s;                 /* completed requests / seconds since the first submit */
  int64_t bytes_in_use, peak_bytes, budget_bytes;
  int32_t peak_active;
  /* means over completed requests: waiting in the queue, set-up and loading
   * (context, buffers, host->device copies), iterations and read-back */
  double queue_ms, load_ms, run_ms;
} gf_server_stats;
/* A request loop on one device: requests are admitted in arrival order while
 * their device bytes fit the budget and fewer than max_active run, and are
 * set up and loaded on a loader thread; every loaded request keeps one
 * iteration in flight on its own stream, so work of different requests
 * overlaps on the device, and finished requests free their memory for the
 * queue (continuous batching). */
gf_status gf_server_create(int32_t device, int64_t budget_bytes, int32_t max_active, gf_server** out);
/* Stops after the queued and active requests finish. */
void gf_server_destroy(gf_server* s);
gf_status gf_server_submit(gf_server* s, const gf_request* req, int64_t* id);
/* Blocks until request id completes; its status (GF_OK or the failure).  The
 * server then forgets the request: each id is waited for once, by one thread
 * (a second concurrent wait for the same id returns GF_ERR_ARG). */
gf_status gf_server_wait(gf_server* s, int64_t id, double* latency_ms);
gf_status gf_server_get_stats(gf_server* s, gf_server_stats* out);

/* ---- autotuning (no counterpart in the reference) ------------------------ */
/* Times the forward projector's thread schedules (run length R of planes per
 * thread, samples per shared-memory chunk) and the back projector's warps per
 * block on this context's geometry with synthetic data, keeps the fastest,
 * and reports them.  Subsequent launches of the context use them. */
gf_status gf_tune(gf_ctx* ctx, int32_t* fp_run, int32_t* fp_chunk, int32_t* bp_warps);
/* Sets the tile shapes gf_tune picks (fp_run 9, 17, 25 or 33; fp_chunk 1..256
 * ray steps per shared-memory chunk; bp_warps 4 or 8), e.g. one context's
 * tuned shapes on others of the same geometry; GF_ERR_GEOMETRY when the
 * schedule does not fit the geometry. */
gf_status gf_set_tile_shapes(gf_ctx* ctx, int32_t fp_run, int32_t fp_chunk, int32_t bp_warps);

/* ---- measurement (no counterpart in the reference, which only prints a
 * one-second wall clock, GFIRST.cu:51-52, 572-573) ------------------------- */
typedef enum gf_stage {
  GF_STAGE_PSF = 0,       /* forward XY PSF of the current image */
  GF_STAGE_FP = 1,        /* forward projection (+ fused ratio) */
  GF_STAGE_VLOR = 2,      /* VLOR split + ratio (mode 3 triples) */
  GF_STAGE_BP = 3,        /* back projection */
  GF_STAGE_UPDATE = 4,    /* ratio, XY PSF, axial filter, multiply */
  GF_STAGE_BILATERAL = 5, /* joint bilateral filter + blend */
  GF_NUM_STAGES = 6
} gf_stage;
/* Record CUDA events around every stage of later sub-iterations (on the
 * context's stream); enabling clears what was recorded. */
gf_status gf_recon_profile(gf_recon* r, int32_t enable);
/* Synchronizes, then returns the summed device time (ms) and the number of
 * recorded instances of one stage. */
gf_status gf_recon_profile_read(gf_recon* r, int32_t stage, double* total_ms, int64_t* count);
/* Kernels this context has launched so far. */
gf_status gf_kernel_launches(const gf_ctx* ctx, int64_t* n);

/* ---- raw files (GFIRST_CPU_Kernels.cpp:25-142, GFIRST.cu:229-240) --------- */
/* ReadSinogram_Type (GFIRST_CPU_Kernels.cpp:104-142): int32 file, re-read as
 * float32 when the largest int exceeds 1e6; h_out gets 2*ndata floats (zeros
 * past the end of the file; a missing file gives GF_ERR_IO and zeros). */
gf_status gf_read_sinogram(const char* path, int64_t ndata, float* h_out);
/* ReadImage (GFIRST_CPU_Kernels.cpp:58-66): nvox floats. */
gf_status gf_read_image(const char* path, int64_t nvox, float* h_out);
/* VLOR list as GFIRST.cu:232-240 consumes it, including the extra pass of its
 * while(!feof) loop over the last record.  With h_events NULL only the count
 * is returned; otherwise up to *nevents pairs are written. */
gf_status gf_read_vlor(const char* path, int32_t* h_events, int64_t* nevents);
/* VLOR events as LOR endpoints: 48-byte records of 12 float32 (see
 * gf_vlor_from_endpoints); trailing bytes of a partial record are ignored.
 * With h_lors NULL only the count is returned. */
gf_status gf_read_vlor_endpoints(const char* path, float* h_lors, int64_t* nevents);
/* WriteImage (GFIRST_CPU_Kernels.cpp:25-33). */
gf_status gf_write_raw(const char* path, const float* h_data, int64_t n);

#ifdef __cplusplus
}
#endif
#endif /* GFIRST_H */
