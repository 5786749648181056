/*
 * tp.h -- C ABI of the GB300 tile processor (libtp.so).
 *
 * Drop-in boundary for the imagej-elphel tile-processor path.  The reference
 * has no C ABI: its GPU boundary is the Java class
 * com.elphel.imagej.gpu.GPUTileProcessor (JCuda + NVRTC), and its CPU twin is
 * ImageDtt.clt_aberrations_quad_corr.  Each entry point below names the
 * reference method it replaces (paths relative to src/main/java/com/elphel/imagej/).
 *
 * Conventions
 *  - every function returns tp_status (0 = TP_OK) and never aborts;
 *    tp_last_error() returns the message of the last failure on a handle;
 *  - host pointers are borrowed for the duration of the call (copied);
 *  - device memory is owned by the handle and released by tp_destroy
 *    (the reference never frees its buffers);
 *  - one handle per host thread / stream; a handle is not thread-safe;
 *  - `stream` arguments are cudaStream_t passed as void* (NULL = the handle's
 *    own stream);  every call that enqueues work records the end of that work;
 *    the tp_get_* calls copy on the handle's own stream after it (wherever it
 *    was enqueued) and synchronise that stream only, never the device; the
 *    *_async getters enqueue the copy on the caller's stream and return.
 *
 * Array layouts (row-major, C order):
 *  image       [height][pitch]           f32 or u16 (Bayer mosaic or mono)
 *  kernels     [kernels_vert][kernels_hor][num_colors][4][64]  f32
 *  kernel_offs [kernels_vert][kernels_hor][num_colors][8]      f32 (CltExtra)
 *  clt         [tilesY*tilesX][num_sensors][num_colors][4][64] f32
 *              (CLT index = horizontal_freq*8 + vertical_freq, the
 *               ImageDtt.extract_correct_tile orientation)
 *  corr        [tilesY*tilesX][num_pairs][15*15]                f32
 *  disparity   [tilesY*tilesX][TP_DISP_N]                       f32
 *  rbg         [num_colors][height+8][width+8]                  f32 per sensor
 */
#ifndef TP_H
#define TP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TP_MAX_SENSORS 16
#define TP_MAX_PAIRS 120
/* Task-input limits, checked on the host before anything is uploaded or launched
 * (the reference trusts its Java host instead, GPUTileProcessor.java:363-371, 686-778):
 *  - tp_set_tasks: every port must be finite and lie within TP_PORT_MARGIN pixels
 *    of the image, -TP_PORT_MARGIN <= x <= width + TP_PORT_MARGIN (y likewise);
 *  - tp_set_tile_ops: the target disparity of every tile with tile_op != 0 must be
 *    finite with |disparity| <= TP_MAX_DISPARITY pixels.
 * A violation returns TP_ERR_ARG and leaves the handle unchanged.  Ports computed on
 * the device from the geometry are not limited: a window corner further than the
 * margin outside the image is moved to the margin keeping its parity, which leaves
 * the (edge-mirrored) window content and the residual shift unchanged. */
#define TP_PORT_MARGIN 1024
#define TP_MAX_DISPARITY 4096.0f

typedef struct tp_handle tp_handle;

typedef enum {
  TP_OK = 0,
  TP_ERR_ARG = 1,      /* invalid argument / size */
  TP_ERR_CUDA = 2,     /* CUDA runtime error */
  TP_ERR_STATE = 3,    /* call order (e.g. no tasks set) */
  TP_ERR_NOMEM = 4,    /* device allocation failed */
  TP_ERR_TIMEOUT = 5,  /* a bounded device wait expired */
  TP_ERR_NOT_BUILT = 6, /* the CUDA kernels are not available */
  TP_ERR_SCRATCH_LIMIT = 7 /* request larger than the fixed scratch of a no-allocation entry point */
} tp_status;

typedef enum { TP_F32 = 0, TP_U16 = 1 } tp_dtype;

typedef enum {
  TP_KERNELS_GPU = 0,  /* GPUTileProcessor.setConvolutionKernel layout: 64 coefficients transposed */
  TP_KERNELS_CPU = 1   /* ImageDtt clt_kernels coefficient order (not transposed) */
} tp_kernel_layout;

/* per-tile disparity record (subset of ImageDtt.java:64-76 disparity_map) */
enum {
  TP_DISP_INT = 0, TP_DISP_CM = 1, TP_DISP_STRENGTH = 2, TP_DISP_HOR = 3, TP_DISP_HOR_STRENGTH = 4,
  TP_DISP_VERT = 5, TP_DISP_VERT_STRENGTH = 6, TP_DISP_CM_S0 = 7, TP_DISP_IXY = 8, TP_DISP_N = 9
};

/* Compile-time #defines of GPUTileProcessor (GPUTileProcessor.java:79-98, 262-276),
 * runtime values here. */
typedef struct {
  int num_sensors;     /* NUM_CAMS, 1..16 */
  int num_colors;      /* NUM_COLORS: 1 (mono) or 3 (Bayer: R, B, G planes) */
  int width, height;   /* IMG_WIDTH, IMG_HEIGHT (multiples of 8) */
  int kernels_hor;     /* KERNELS_HOR (0 = identity kernels, no aberration correction) */
  int kernels_vert;    /* KERNELS_VERT */
  int kernel_step;     /* KERNELS_STEP (16) */
  int bayer_red_row;   /* BAYER_RED_ROW (reference 0) */
  int bayer_red_col;   /* BAYER_RED_COL (reference 1) */
  int device;          /* CUDA device ordinal */
} tp_config;

/* GeometryCorrection lens/extrinsic model (GeometryCorrection.java:36-90, 1004-1076),
 * generalised to free per-sensor azimuth/tilt/roll/zoom. */
typedef struct {
  int pixel_width, pixel_height;  /* pixelCorrectionWidth/Height */
  double focal_length;            /* mm */
  double pixel_size;              /* um */
  double distortion_radius;       /* mm */
  double distortion[7];           /* distortionC, B, A, A5, A6, A7, A8 */
  double rXY[TP_MAX_SENSORS][2];  /* lens offsets in disparity units */
  double pXY0[TP_MAX_SENSORS][2]; /* sensor centres, pixels */
  double azimuth[TP_MAX_SENSORS]; /* radians */
  double tilt[TP_MAX_SENSORS];
  double roll[TP_MAX_SENSORS];    /* full roll (CorrVector roll + factory roll), radians */
  double zoom[TP_MAX_SENSORS];    /* zoom - 1 */
} tp_geometry;

/* correlation pair: Correlation2d.PAIRS entry (Correlation2d.java:52-71) */
typedef struct {
  int cam1, cam2;
  int kind;          /* 0 horizontal, 1 vertical, 2 main diagonal, 3 other diagonal, 4 general */
  int in_combo;      /* contributes to the combined strip (dbg_pair_mask bit) */
  float bx, by;      /* strip direction (disparity-axis step), used by kind 4 */
} tp_pair;

/* ImageDttParameters subset (ImageDttParameters.java:30-112) + per-call values */
typedef struct {
  float fat_zero;        /* corr_fat_zero */
  float corr_sigma;      /* LPF sigma (as in ImageDtt.java:1669: not squared) */
  float corr_red, corr_blue;
  float corr_offset;
  float min_corr;
  int corr_strip_hight;  /* rows of the combined strip (<= 16) */
  int twice_diagonal;
  float enhortho_width, enhortho_scale;
  int corr_wndy_size; float corr_wndy_hwidth, corr_wndy_blur;
  int corr_wndx_size; float corr_wndx_hwidth, corr_wndx_blur;
} tp_corr_params;

/* texture tiles (CLTParameters fields read by ImageDtt.java:2662-2812) */
typedef struct {
  float min_shot;          /* 10.0: shot-noise correction below this is linear */
  float scale_shot;        /* 3.0: scale after sqrt; <= 0 disables the correction */
  float diff_sigma;        /* 5.0: pixel value difference sigma of the port weights */
  float corr_magic_scale;  /* 0.85: extra shift = disparity x port offset / this */
  int dust_remove;         /* 1 */
  int keep_weights;        /* 1: 12 rows per tile (RGBA, 4 port weights, 4 rms), 0: 4 rows */
  int corr_mode;           /* 2: disparity used for the extra shift: 0 INT, 1 CM, 2 POLY (the LMA
                              disparity of tp_lma_refine after the current forward; none without
                              it), 3 HOR, 4 VERT; -1 gives no extra shift */
  int aux;                 /* 1: also keep per tile max_diff[4] and ports_rgb[12] */
} tp_texture_params;

/* lifecycle: GPUTileProcessor() (GPUTileProcessor.java:243-360) */
tp_status tp_create(const tp_config *cfg, tp_handle **out);
tp_status tp_destroy(tp_handle *h);
/* copies the last error message (NUL-terminated) */
tp_status tp_last_error(const tp_handle *h, char *buf, int buf_len);
/* Process-wide cap on the device bytes one handle may hold (0 = no cap, the default), for a GPU
 * shared with other work: an allocation that would exceed it fails like a failed cudaMalloc --
 * tp_create returns TP_ERR_NOMEM and frees what it had allocated; a lazily allocated buffer
 * (correlation surfaces, frames, textures, LMA, adjoint) fails its call with TP_ERR_NOMEM and
 * leaves the handle usable.  No reference counterpart (GPUTileProcessor allocates fixed sizes in
 * its constructor and never frees). */
tp_status tp_set_memory_limit(size_t max_bytes_per_handle);
/* device bytes the handle holds now */
tp_status tp_get_memory_usage(const tp_handle *h, size_t *bytes);
/* fills the reference defaults (ImageDttParameters.java:30-112, fat_zero 0.05, corr_sigma 0.8) */
tp_status tp_default_corr_params(tp_corr_params *p);
/* CLTParameters defaults of the texture path (min_shot 10, scale_shot 3, diff_sigma 5,
 * corr_magic_scale 0.85, dust_remove, keep_weights, corr_mode 2) */
tp_status tp_default_texture_params(tp_texture_params *p);
/* the 6 quad pairs Correlation2d.PAIRS[0..5]; returns the count in *n */
tp_status tp_quad_pairs(tp_pair *pairs, int *n);

/* inputs
 * A setter that overwrites a device buffer is ordered after the handle's work already enqueued,
 * on whichever stream: the asynchronous ones (tp_set_image_async, tp_calc_kernels,
 * tp_set_tile_ops) wait for it on their stream, the synchronous ones (tp_set_geometry,
 * tp_set_kernels, tp_set_image, tp_set_lpf, tp_set_corr) on the host before they copy. */
/* GeometryCorrection set-up used by stage 1 (getPortsCoordinatesAndDerivatives) */
tp_status tp_set_geometry(tp_handle *h, const tp_geometry *g);

/* The auxiliary camera of a rig (GeometryCorrection.RigOffset, GeometryCorrection.java:256-975). */
typedef struct {
  double main_disparity_radius;  /* mm: GeometryCorrection.disparityRadius of the main camera */
  double aux_disparity_radius;   /* mm: of the auxiliary camera */
  double baseline;               /* mm: auxiliary centre from the main one */
  double aux_angle;              /* rad: direction of the baseline */
  double aux_azimuth, aux_tilt, aux_roll; /* rad: the auxiliary camera's rotation */
  double aux_zoom;               /* zoom - 1 */
} tp_rig_offset;
/* Makes h a rig's auxiliary camera, with ports as ImageDtt.clt_bi_quad computes them
 * (ImageDtt.java:8972-8996, getPortsCoordinatesAndDerivatives(gc_main, use_rig_offsets = true)):
 * aux is this camera's own model, main_camera the main camera's.  Task disparities are then the
 * main camera's, scaled by aux / main disparity radius; the tile centre is undistorted with the
 * main camera's model; the lens offsets are RigOffset.rXY_aux (recalcRXY 728-747: the baseline
 * offset plus the lens offsets rotated by aux_roll); each sensor's rotation is followed by the rig
 * rotation (CorrVector.getRotMatrices(rigMatrix) 1016-1025, RigOffset.getRotMatrix 770-800).
 * main_camera or rig NULL: as tp_set_geometry(h, aux).  tp_backward refuses such a handle. */
tp_status tp_set_rig_geometry(tp_handle *h, const tp_geometry *aux, const tp_geometry *main_camera,
                              const tp_rig_offset *rig);
/* setConvolutionKernel (GPUTileProcessor.java:373-379) / setConvolutionKernels (381-435) */
tp_status tp_set_kernels(tp_handle *h, int cam, const float *kernels, const float *kernel_offsets, int layout);
/* setBayerImage (GPUTileProcessor.java:437-450); pitch in elements (0 = width) */
tp_status tp_set_image(tp_handle *h, int cam, const void *image, int dtype, size_t pitch);
/* as tp_set_image, but only enqueued on `stream` (NULL = the handle's stream): the host buffer
 * (best page-locked) must stay valid and unchanged until the stream has passed the copy, and
 * work on other streams that reads this sensor's image must be ordered after it by the caller
 * (no reference counterpart: setBayerImage copies synchronously) */
tp_status tp_set_image_async(tp_handle *h, int cam, const void *image, int dtype, size_t pitch, void *stream);
/* per-colour gain applied while reading the mosaic (QuadCLT.java:181-185 scales green by 0.5
 * before the GPU mosaic is formed); default {1, 1, 1} for R, B, G */
tp_status tp_set_color_scales(tp_handle *h, const float *scales);
/* setTasks (GPUTileProcessor.java:363-371): TpTask.asFloatArray layout,
 * per task {task (int bits), tx | ty << 16 (int bits), xy[num_sensors][2]} */
tp_status tp_set_tasks(tp_handle *h, const float *packed_tasks, int num_tasks);
/* setFullFrameImages(float[] target_disparities) + getTileSubcamOffsets
 * (GPUTileProcessor.java:472-527, 686-778) computed on the device in FP64:
 * tiles with tile_op != 0 (ImageDtt tile_op[ty][tx]) become tasks in row-major order.
 * Returns without waiting for the device: the arrays are copied (the caller's buffers are free
 * on return) and uploaded after the handle's last work, and the handle's next work runs after
 * the upload; tp_get_num_tasks is known at once. */
tp_status tp_set_tile_ops(tp_handle *h, const int *tile_op, const float *target_disparity);
/* The aberration-kernel chain of QuadCLT.calculateCLTKernel (QuadCLT.java:433-667,
 * ImageDtt.java:4625-4734) on the device: psf [kernels_vert][kernels_hor][num_colors][64][64]
 * double-resolution PSFs (float, host memory, or device memory when psf_on_device) ->
 * this sensor's kernel table in the TP_KERNELS_CPU layout and its CltExtra records
 * (data_x, data_y, center_x, center_y); normalize: kernel x window sums to 16
 * (clt_normalize_kernel); coord_corr: the 3x3 least-squares centre slopes dxc_dx ..
 * dyc_dy (ImageDtt.clt_fill_coord_corr 4792-4851), else those four are 0. */
tp_status tp_calc_kernels(tp_handle *h, int cam, const float *psf, int psf_on_device, int normalize,
                          int coord_corr, void *stream);
/* copies a sensor's kernel table (TP_KERNELS_CPU layout) and CltExtra records to the host */
tp_status tp_get_kernels(tp_handle *h, int cam, float *kernels, float *kernel_offsets);
/* setLpfRbg (GPUTileProcessor.java:780-812): lpf[num_colors][64] applied by tp_imclt; NULL = off */
tp_status tp_set_lpf(tp_handle *h, const float *lpf);
/* execConverCorrectTiles stores a low-pass filtered CLT: it passes lpf_mask = 7
 * (GPUTileProcessor.java:547) and convertCorrectTile multiplies the CLT of every colour whose bit
 * is set by that colour's LPF (TileProcessor.cuh:1037-1061).  With a mask set here, the CLT stored
 * by tp_process / tp_convert_correct (tp_get_clt, and what tp_imclt reads) carries the filter of
 * tp_set_lpf for those colours the same way, and tp_imclt does not apply it again, so the RBG
 * frames are unchanged.  The correlation of tp_process still uses the unfiltered CLT (the CPU
 * path's semantics); tp_correlate, tp_textures, tp_rig_correlate and tp_backward (unless it
 * recomputes the CLT) read the stored CLT and return TP_ERR_STATE while a mask is in effect.
 * One bit per colour (0..2^num_colors - 1); default 0 (the CPU path's unfiltered CLT); it takes
 * effect only while tp_set_lpf has a filter set. */
tp_status tp_set_clt_lpf_mask(tp_handle *h, int lpf_mask);
/* GPU_DTT24_DRV (dtt8x8.cuh:100-158, the reference's kernel for testing and profiling the
 * transforms alone): every 8x8 block of a float image in device memory through one 2D transform,
 * rows first (horizontal: DST if bit 0 of dtt_mode is set, else DCT), then columns (vertical:
 * bit 1); modes 0-3 DCT-IV / DST-IV, 4-7 DCT-II / DST-II, all orthonormal as DttRad2.dct_iv /
 * dst_iv / dct_ii.  dst and src (device pointers, dst may equal src) share src_stride (floats);
 * width and height are multiples of 8.  Enqueued on stream (NULL: the default stream); the first
 * call on a device uploads the transform tables (a synchronous copy). */
tp_status tp_dtt8x8(float *dst, const float *src, int src_stride, int width, int height, int dtt_mode,
                    void *stream);
/* correlation set-up (ImageDtt.clt_aberrations_quad_corr_new arguments, ImageDtt.java:1491-1546) */
tp_status tp_set_corr(tp_handle *h, const tp_corr_params *p, const tp_pair *pairs, int num_pairs);
/* texture set-up; the LPF and colour weights are those of tp_set_corr */
tp_status tp_set_texture_params(tp_handle *h, const tp_texture_params *p);

/* execution */
/* stage 1 on the device when tile ops are set (getTileSubcamOffsets, GPUTileProcessor.java:686-778) */
tp_status tp_ports(tp_handle *h, void *stream);
/* execConverCorrectTiles (GPUTileProcessor.java:530-558): stage 2 */
tp_status tp_convert_correct(tp_handle *h, void *stream);
/* ImageDtt.java:2101-2245 on the device: pair correlation (stage 3a) */
tp_status tp_correlate(tp_handle *h, void *stream);
/* ImageDtt.java:2114-2245: strips, combination, argmax, centroid, ortho (stage 3b) */
tp_status tp_extract(tp_handle *h, void *stream);
/* execImcltRbg (GPUTileProcessor.java:560-597): stage 4a */
tp_status tp_imclt(tp_handle *h, void *stream);
/* texture tiles of the current CLT and disparity (ImageDtt.java:2662-2812, tile_combine_rgba
 * 2830-3000): 4 sensors x 3 colours only (TP_ERR_ARG otherwise) */
tp_status tp_textures(tp_handle *h, void *stream);
/* ports + convert_correct + correlate + extract in one call (ImageDtt.clt_aberrations_quad_corr) */
tp_status tp_process(tp_handle *h, void *stream);
/* schedule of the fused forward kernel: tiles per CTA and warps per CTA (0 = defaults): warp per
 * tile with 1, 2 or 4 tiles per CTA (tiles_per_block == warps_per_block), or one tile per CTA of 2,
 * 3 or 4 warps splitting its colour items and pairs (3 warps: 80 registers, 8 CTAs per SM);
 * chosen by tileproc.autotune (no reference counterpart: the reference hard-codes
 * TILES_PER_BLOCK, GPUTileProcessor.java:92) */
tp_status tp_set_schedule(tp_handle *h, int tiles_per_block, int warps_per_block);
tp_status tp_synchronize(tp_handle *h);

/* outputs (host copies) */
tp_status tp_get_num_tasks(const tp_handle *h, int *n);
tp_status tp_get_ports(tp_handle *h, double *ports);            /* [num_tasks][S][2] */
tp_status tp_get_task_tiles(tp_handle *h, int *txy);            /* [num_tasks] tx | ty << 16 */
tp_status tp_get_subtiles(tp_handle *h, int *int_tl, float *residual); /* [num_tasks][S][C][2] each */
tp_status tp_get_clt(tp_handle *h, float *clt);
tp_status tp_get_corr(tp_handle *h, float *corr);
tp_status tp_get_disparity(tp_handle *h, float *disparity);
/* getRBG (GPUTileProcessor.java:599-626): [num_colors][height+8][width+8] */
tp_status tp_get_rbg(tp_handle *h, int cam, float *rbg);
/* as tp_get_rbg / tp_get_disparity, but only enqueued on `stream` (NULL = the handle's stream)
 * after the handle's last enqueued work; the host buffer (best page-locked) holds the result once
 * the stream has passed the copy.  No reference counterpart: getRBG copies synchronously.  A
 * frame loop reads frame k's colour frames this way while frame k+1 is processed; work that
 * rewrites the frames (the next tp_imclt) must be ordered after the copy by the caller. */
tp_status tp_get_rbg_async(tp_handle *h, int cam, float *rbg, void *stream);
tp_status tp_get_disparity_async(tp_handle *h, float *disparity, void *stream);
/* texture_tiles[ty][tx]: [tilesY*tilesX][4 or 12][256] (R, B, G, alpha, weights, rms) */
tp_status tp_get_textures(tp_handle *h, float *tex);
/* [tilesY*tilesX][16]: max_diff[4] (IMG_DIFF0_INDEX), ports_rgb[12] (IMG_TONE_RGB, colour * 4 + port) */
tp_status tp_get_texture_aux(tp_handle *h, float *aux);

/* ---- LMA disparity ("POLY"): Correlation2d.corrLMA (Correlation2d.java:1754-1877)
 * with Correlations2dLMA (Correlations2dLMA.java:211-640), run by ImageDtt at
 * ImageDtt.java:2254-2288.  After tp_process on a quad pair layout, every tile
 * whose CM disparity exists and whose integer-max strength exceeds
 * min_poly_strength is refitted: the ortho pairs (horizontal, vertical
 * transposed) and the diagonal pairs (main, other flipped) are averaged into
 * two groups, cells reached from the CM centre through bi-convex cells are
 * sampled, and a per-group parabola with a common centre and widths is fitted
 * by Levenberg-Marquardt.  Output per tile {disparity, strength, half-width
 * WM, WXY} (getDisparityStrengthWidth; NaN where not run or not converged).
 * With mix_corr_poly the result also replaces TP_DISP_CM and TP_DISP_STRENGTH
 * of the disparity record, and with fo_correct the far/foreground correction
 * may replace TP_DISP_CM, as the reference does; the pass then needs a new
 * tp_process before it can run again.  Pair kinds 4 (general) do not take
 * part; cnvx_hwnd_size is at most 4.  Defaults: ImageDttParameters.java:32-109. */
typedef struct {
  float min_poly_strength;  /* 0.2 */
  int mix_corr_poly;        /* 1 */
  float ortho_vasw_pwr;     /* 2.0: sample weight x |value|^pwr */
  int cnvx_hwnd_size;       /* 4 */
  float cnvx_weight;        /* 0.5: weight of selected non-convex cells */
  int cnvx_add3x3;          /* 1: the 3x3 cells around the centre are always sampled */
  int adjust_wm, adjust_wy, adjust_wxy, adjust_ag; /* 1, 0, 1, 1 */
  float half_width, cost_wy, cost_wxy;             /* 2.0, 0.1, 0.1 */
  float lambda_initial, lambda_scale_good, lambda_scale_bad, lambda_max, rms_diff; /* 0.1, 0.5, 8, 100, 0.001 */
  int num_iter;             /* 20 */
  int pair_mask;            /* bit i: pair i takes part (dbg_pair_mask 0x3f) */
  /* far / foreground correction (corr4dirsLMA + foregroundCorrect, ImageDtt.java:2294-2335):
   * one more fit per pair orientation; where they disagree by at least fo_min_diff the
   * largest (fo_far: smallest) disparity replaces TP_DISP_CM */
  int fo_correct;           /* 1 */
  int fo_far;               /* 0 */
  int fo_ortho;             /* 1: the extreme orientations must be orthogonal for the overcorrection */
  float fo_min_strength;    /* 0.1 */
  float fo_min_eff;         /* 0.25: strength x (WM - WXY) / (WM + WXY) */
  float fo_min_eff_ratio;   /* 0.65 */
  float fo_max_hwidth;      /* 3.0 */
  float fo_min_diff;        /* 0.2 */
  float fo_overcorrection;  /* 0.0 */
  float fo_lim_overcorr;    /* 2.0 */
  /* lazy-eye mismatch (clt_mismatch, ImageDtt.java:2340-2418; off by default as there): the
   * orientation fits always run, the foreground correction is not applied to TP_DISP_CM, and
   * where the fits agree to mismatch_max_diff every pair's peak centre of mass within
   * max_corr_radius of the disparity (Correlation2d.mismatchPairsCM) goes to tp_get_lma_mismatch */
  int mismatch;             /* 0 */
  float max_corr_radius;    /* 3.9 (EyesisCorrectionParameters) */
  float mismatch_max_diff;  /* 1.0 */
  /* the polynomial measure instead (ImageDttParameters.java:50-52; ImageDtt.java:2349-2405): each
   * pair sampled alone like the LMA (weights x |value|^max_corr_radius, as there) and fitted by a
   * weighted quadric A x^2 + B y^2 + C xy + D x + E y + F, whose maximum gives the pair's offsets
   * and strength (Correlation2d.mismatchPairs 1434-1503, Correlations2dLMA.getMaxXYPoly 641-704);
   * an offset beyond ly_crazy_poly zeroes the pair's strength, and with ly_poly_backup any failed
   * or implausible pair sends all pairs of the tile to the centre-of-mass measure */
  int ly_poly;              /* 0 */
  float ly_crazy_poly;      /* 1.0 */
  int ly_poly_backup;       /* 1 */
} tp_lma_params;
tp_status tp_default_lma_params(tp_lma_params *p);
tp_status tp_lma_refine(tp_handle *h, const tp_lma_params *p, void *stream);
/* out [tilesY*tilesX][4] */
tp_status tp_get_lma(tp_handle *h, float *out);
/* The 2D maximum of every pair's correlation surface of the last tp_process: out
 * [tilesY*tilesX][num_pairs][3] = {dx, dy, strength}, px from the surface centre (x right,
 * y down): the first cell of the largest value in index order (NaN cells skipped), refined by a
 * parabola through it and its two neighbours on each axis (the fraction clamped to +-0.5); {NaN,
 * NaN, 0} where the maximum is on the surface's border or no cell is finite, all NaN for tiles
 * outside the task list.  A pair's maximum lies at (port error of cam1) - (port error of cam2):
 * the per-pair offsets of any pair layout that the extrinsic refinement's coarse stage fits, as
 * the reference's extrinsic fitting consumes its lazy-eye pair offsets (clt_mismatch,
 * ImageDtt.java:2340-2418; AlignmentCorrection).  No reference counterpart as an entry point.
 * Computed on the device (a warp per surface) after the handle's work, then copied like the
 * other getters. */
tp_status tp_get_pair_maxima(tp_handle *h, float *out);
/* out [tilesY*tilesX][num_pairs][3] = {dx, dy, strength} per pair (NaN, NaN, 0 where not measured),
 * after tp_lma_refine with mismatch set */
tp_status tp_get_lma_mismatch(tp_handle *h, float *out);

/* ---- rig: main and auxiliary quad cameras (ImageDtt.clt_bi_quad, ImageDtt.java:8731-) ----
 * Inter-camera correlation of the sensor-averaged CLT of each camera
 * (Correlation2d.correlateInterCamerasFD / cltMixCameras, Correlation2d.java:401-448)
 * with the main camera's correlation set-up, and its disparity along the rig
 * baseline (ImageDtt.tileInterCamCorrs 7370-7496; the LMA branch is tp_rig_lma):
 * rec = {BI_DISP_CROSS, BI_STR_CROSS (mass / (sigma x cm_max_normalization)^2),
 * BI_DISP_CROSS_DX, BI_DISP_CROSS_DY (NaN until tp_rig_lma)}.  Both cameras share the
 * tile grid and colours and have run tp_process (each with its own geometry and
 * target disparities); tiles the auxiliary camera has no task for get
 * {NaN, 0, NaN, NaN}.  Results are kept by the main handle. */
tp_status tp_rig_correlate(tp_handle *main_camera, tp_handle *aux_camera, float cm_max_normalization, int no_int_x0,
                           void *stream);
/* corr [tilesY*tilesX][15*15], rec [tilesY*tilesX][4]; either may be NULL */
tp_status tp_get_rig(tp_handle *main_camera, float *corr, float *rec);
/* The LMA branch of tileInterCamCorrs (ImageDtt.java:7497-7560) on the last tp_rig_correlate:
 * where the record's strength exceeds p->min_poly_strength, the LMA of tp_lma_refine runs on the
 * inter-camera surface (one horizontal pair, centred at -disparity; fo_correct, mismatch and
 * mix_corr_poly do not apply), and where it converges use_poly (rig.use_poly) replaces
 * BI_DISP_CROSS / BI_STR_CROSS by its disparity / strength, and the peak's offset around x = 0
 * fills BI_DISP_CROSS_DX / DY: with use_xy_poly (rig.use_xy_poly) the maximum of the quadric fit
 * to the convex-region samples weighted x |value|^ortho_vasw_pwr (Correlation2d.single2dPoly
 * 1509-1536; NaN where the fit has no maximum), else the centre of mass of the positive cells
 * within max_corr_radius (single2dCM 1538-1585).  Runs once per tp_rig_correlate (TP_ERR_STATE
 * otherwise); p NULL: tp_default_lma_params. */
tp_status tp_rig_lma(tp_handle *main_camera, const tp_lma_params *p, int use_poly, int use_xy_poly, void *stream);

/* ---- batches (no reference counterpart: the reference processes one scene per
 * GPUTileProcessor instance and launch) ----
 * A batch runs the forward of many scenes -- handles of any sensor count,
 * colours, size and pair set, all on one device, each with its tasks and
 * correlation set up -- as one launch of the plans of all scenes and one
 * persistent forward kernel per schedule class (colour warp-per-tile, mono
 * warp-per-tile, mono with more than 8 pairs: 4 warps per tile) over a queue
 * of tiles in scene order, the classes running concurrently.  Warp-per-tile
 * scenes with at least 8 waves of tiles (8 x 16 x SM count) keep their own
 * forward launch inside the same step (they have no tail to share).  Colour
 * scenes need sensors x colours <= 16 and at most 8 pairs.  The handles stay owned by the caller and must
 * outlive the batch; results are read through each handle's getters. */
typedef struct tp_batch tp_batch;
tp_status tp_batch_create(tp_handle *const *scenes, int num_scenes, tp_batch **out);
tp_status tp_batch_destroy(tp_batch *b);
tp_status tp_batch_last_error(const tp_batch *b, char *buf, int buf_len);
/* plans every scene (always when replan != 0, else only where missing), then the one forward launch */
tp_status tp_batch_process(tp_batch *b, int replan, void *stream);
/* the same step (with replanning) captured once into a CUDA graph and replayed; the graph is
 * rebuilt when anything the capture holds by value changed for a scene -- its task count, a
 * device buffer reallocated (e.g. tp_set_corr with more pairs), the image dtype, colour scales,
 * pair count, strip rows, correlation parameters or schedule; inputs updated in place in the same
 * buffers (tp_set_image with the same dtype, tp_set_tile_ops, tp_set_geometry, tp_set_kernels)
 * are picked up by the replay */
tp_status tp_batch_run_graph(tp_batch *b, void *stream);
tp_status tp_batch_synchronize(tp_batch *b);

/* ---- adjoint (no reference counterpart: the reference has no derivative of
 * the correlation chain; its geometric part is GeometryCorrection
 * .getPortsCoordinatesAndDerivatives, GeometryCorrection.java:2159-2314) ----
 * For every tile with a centroid disparity d (TP_DISP_CM of the last
 * tp_process), tp_backward computes dd/d(port x, y) of every sensor by a
 * hand-written adjoint of centroid -> strip combination -> correlation ->
 * CLT -> residual window shift, contracts it with the FP64 port derivatives
 * into the Jacobian rows dd/d(azimuth, tilt, roll, zoom of each sensor) and
 * dd/d(tile target disparity), and returns the gradient of
 * L = sum over tiles of l(d) with dl/dd given per tile in dl_ddisp
 * ([tilesY*tilesX], host; NULL means l = d^2, i.e. 2 d).  Integer window
 * corners and the integer argmax are held fixed (piecewise constant).
 * Mono sensors, or Bayer colour sensors (the three colour planes of a sensor
 * share its port: their sensitivities add, and the pair chain runs back through
 * the colour mix of the correlation); ports from the geometry (tp_set_tile_ops);
 * run after tp_process.
 * dl_dextr [num_sensors][4] and dl_dtile_disp [tilesY*tilesX] are host
 * outputs (either may be NULL).  From the first tp_backward (or
 * tp_set_adjoint_mode) on, tp_process also records every pair's strip samples
 * ([tiles][pairs][strip entries] floats on the device) for the adjoint to read. */
tp_status tp_backward(tp_handle *h, const float *dl_ddisp, float *dl_dextr, float *dl_dtile_disp, void *stream);
/* 1: the adjoint recomputes each tile's CLT from the images instead of reading
 * the stored CLT back (for when the CLT buffer is not kept; a Bayer colour as the
 * dense fold of its sparse plane, which equals the forward's CLT to rounding);
 * default 0.  Also starts the strip-sample recording described at tp_backward. */
tp_status tp_set_adjoint_mode(tp_handle *h, int recompute_clt);
/* Jacobian of the last tp_backward: jac_extr [tiles][num_sensors][4] (dd per
 * azimuth, tilt, roll, zoom), jac_disp [tiles] (dd per target disparity),
 * disparity [tiles] (d, NaN where none); any pointer may be NULL */
tp_status tp_get_disparity_jacobian(tp_handle *h, float *jac_extr, float *jac_disp, float *disparity);
/* dd/d(port x, port y) per tile and sensor: [tiles][num_sensors][2] */
tp_status tp_get_port_sensitivities(tp_handle *h, float *sens);
/* FP64 port derivatives of the last tp_backward's plan, per task:
 * [num_tasks][num_sensors][2 (x, y)][5 (azimuth, tilt, roll, zoom, disparity)] */
tp_status tp_get_port_derivatives(tp_handle *h, double *deriv);

/* ---- no-allocation entry point ----
 * Row-major compaction of tile_op[num_tiles] into the task list, the same
 * result as tp_set_tile_ops (task_txy = tx | ty << 16, task_op, task_disp,
 * *num_tasks), on caller-owned DEVICE buffers: tile_op, disparity (may be
 * NULL: task_disp = 0), task_txy/task_op/task_disp (num_tiles entries each)
 * and num_tasks (one int).  No reference counterpart: the reference packs its
 * task list on the host (GPUTileProcessor.setTasks, GPUTileProcessor.java:
 * 686-778).  It allocates nothing -- no cudaMalloc/cudaFree and no allocating
 * library; its per-block counts live in a fixed device array of
 * TP_COMPACT_MAX_TILES / 1024 ints inside libtp.  num_tiles above
 * TP_COMPACT_MAX_TILES returns TP_ERR_SCRATCH_LIMIT.  A call outside a stream
 * capture looks the array's address up (cudaGetSymbolAddress) on the current
 * device and keeps it; a call on a capturing stream uses the address kept by
 * the last call outside one, so make the first call on each device before any
 * stream capture (else TP_ERR_STATE).  Calls on one device share
 * the array: calls that overlap in time (different streams or threads) race;
 * serialise them.  Runs on the current device and `stream` (NULL = the default
 * stream), asynchronously. */
#define TP_COMPACT_MAX_TILES (1024 * 1024)
#define TP_NOALLOC_MAX_DEVICES 64
tp_status tp_compact_tile_ops_noalloc(const int *tile_op, const float *disparity, int tilesX, int num_tiles,
                                      int *task_txy, int *task_op, float *task_disp, int *num_tasks,
                                      void *stream);

#ifdef __cplusplus
}
#endif
#endif
