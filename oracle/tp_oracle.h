/*
 * tp_oracle.h -- FP64 CPU restatement of the imagej-elphel tile-processor path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle for the
 * GB300 kernels and the timed CPU baseline ("port" of the reference CPU path).
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may
 * load it.  The product (libtp) never links or calls anything here.
 *
 * Reference: Elphel imagej-elphel (Java), files cited per function as
 *   J/ = src/main/java/com/elphel/imagej/
 *   DttRad2            J/tileprocessor/DttRad2.java
 *   ImageDtt           J/tileprocessor/ImageDtt.java
 *   Correlation2d      J/tileprocessor/Correlation2d.java
 *   GeometryCorrection J/tileprocessor/GeometryCorrection.java
 *   QuadCLT            J/tileprocessor/QuadCLT.java
 *
 * Parity status: the reference ships no tests, golden vectors or fixtures for
 * this path and its CPU path is Java (no JVM on this machine), so the CPU
 * stages are pinned by the restated source.  Stage 2 (convert/correct) and
 * IMCLT are additionally pinned against the reference's own CUDA kernels
 * (compiled from its sources by oracle/build_ref_gpu.py) through golden
 * fixtures under tests/golden/.  The texture-tile stage (or_texture_tile) has
 * no reference kernel to run and no fixture: parity unpinned for that stage,
 * which rests on the restated source alone.
 *
 * All arithmetic is double; compiled with -ffp-contract=off so that results
 * are identical on x86_64 and aarch64.
 */
#ifndef TP_ORACLE_H
#define TP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define OR_DTT 8          /* transform_size */
#define OR_DTT2 16
#define OR_CORR 15        /* 2*transform_size-1 */
#define OR_MAX_SENSORS 16
#define OR_MAX_PAIRS 120

/* disparity_map layout per tile (subset of ImageDtt.java:64-76 indices) */
enum {
  OR_DISP_INT = 0,          /* DISPARITY_INDEX_INT   */
  OR_DISP_CM = 1,           /* DISPARITY_INDEX_CM    */
  OR_DISP_STRENGTH = 2,     /* DISPARITY_STRENGTH_INDEX */
  OR_DISP_HOR = 3,          /* DISPARITY_INDEX_HOR   */
  OR_DISP_HOR_STRENGTH = 4, /* DISPARITY_INDEX_HOR_STRENGTH */
  OR_DISP_VERT = 5,         /* DISPARITY_INDEX_VERT  */
  OR_DISP_VERT_STRENGTH = 6,/* DISPARITY_INDEX_VERT_STRENGTH */
  OR_DISP_CM_S0 = 7,        /* getMaxXCm weight  (diagnostic) */
  OR_DISP_IXY = 8,          /* integer argmax column (diagnostic, NaN if none) */
  OR_DISP_N = 9
};

/* ---- DttRad2 ---- */
void or_dct_iv8(const double *x, double *y);           /* DttRad2.dct_iv   (80-85)  */
void or_dst_iv8(const double *x, double *y);           /* DttRad2.dst_iv   (87-98)  */
void or_dct_ii8(const double *x, double *y);           /* DttRad2.dct_ii   (68-78)  */
void or_dst_ii8(const double *x, double *y);           /* dtt8x8.cuh dttii_shared_mem, DST (296-378) */
/* GPU_DTT24_DRV (dtt8x8.cuh:100-158) on one row-major 8x8 block: rows (bit 0 of mode: DST), then
 * columns (bit 1); modes 0-3 DCT-IV / DST-IV, 4-7 DCT-II / DST-II */
void or_dtt24(const double *x, double *y, int mode);
/* mode bit0: horizontal sine, bit1: vertical sine; output transposed */
void or_dttt_iv(const double *x, double *y, int mode);   /* DttRad2.dttt_iv   (503-519) */
void or_dttt_iie(const double *x, double *y, int mode);  /* DttRad2.dttt_iie  (595-614) */
void or_dttt_iiie(const double *x, double *y, int mode); /* DttRad2.dttt_iiie (648-666) */
void or_dctiv_direct(const double *x, double *y);        /* DttRad2.dctiv_direct (848-862) */
void or_hwindow(double *hw8);                            /* set_window(1) (674-694) */
void or_shifted_fold(double shift_hor, double shift_vert,
                     double fold_k[4][64][4]);           /* get_shifted_fold_2d (263-314) */
void or_fold_index(int fold_index[64][4]);               /* set_fold_2d (146-203) */
void or_fold_tile(const double *tile256, int mode,
                  const double fold_k[4][64][4], double *y64); /* fold_tile (724-738) */
void or_unfold_tile(const double *x64, int mode, double *y256);  /* unfold_tile (770-780) */
void or_corr_unfold_tile(const double q[4][64], double *rslt225); /* corr_unfold_tile (443-489) */
void or_win2d(double *w256);                             /* getWin2d (697-713) */

/* ---- ImageDtt stage 2 ---- */
/*
 * extract_correct_tile (ImageDtt.java:4867-5426, non-debug branch).
 * image: one colour plane, row-major [height][width] (double).
 * kern/kext: kernel table for this colour, or NULL for identity (use_kernels=false):
 *   kern layout [kv][kh][4][64] CPU orientation, kext [kv][kh][8] (CltExtra order).
 * Writes clt[4][64], residual[2], and optionally int_tl[2] / ktile[2].
 */
void or_extract_correct_tile(const double *image, int width, int height,
                             const double *kern, const double *kext,
                             int kernels_hor, int kernels_vert, int kernel_step,
                             double centerX, double centerY,
                             double clt[4][64], double residual[2],
                             int int_tl[2], int ktile[2]);
void or_convolve_tile(double data[4][64], const double *kernel4x64); /* 5429-5488 */
void or_fract_shift(double clt[4][64], double shiftX, double shiftY); /* 5490-5584 */

/* correlation LPF (ImageDtt.java:1662-1690) -> filter[64] */
void or_corr_lpf(double corr_sigma, double *filter64);
/* setCltLpf + dttt_iiie * 2n (GPUTileProcessor.java:780-848) */
void or_clt_lpf(double sigma, double *lpf64);

/* ---- GeometryCorrection ---- */
typedef struct {
  int num_sensors;
  int pixel_width, pixel_height;   /* pixelCorrectionWidth/Height */
  double focal_length;             /* mm */
  double pixel_size;               /* um */
  double distortion_radius;        /* mm */
  double distortion[7];            /* C, B, A, A5, A6, A7, A8 */
  double rXY[OR_MAX_SENSORS][2];   /* disparity-normalised lens offsets */
  double pXY0[OR_MAX_SENSORS][2];  /* sensor centres, pixels */
  double azimuth[OR_MAX_SENSORS];  /* radians */
  double tilt[OR_MAX_SENSORS];
  double roll[OR_MAX_SENSORS];     /* full roll (vector roll + factory roll), radians */
  double zoom[OR_MAX_SENSORS];     /* zoom - 1 */
} or_geometry;

/* CorrVector.getRotMatrices (GeometryCorrection.java:1043-1076) */
void or_rot_matrices(const or_geometry *g, double rots[][3][3]);
/* CorrVector.getRotDeriveMatrices (1083-1147): [sensor][az,tilt,roll,zoom] */
void or_rot_deriv_matrices(const or_geometry *g, double drots[][4][3][3]);
/* calcReverseDistortionTable (2707-2757); returns table length, fills tbl (>= 2002) */
int or_reverse_distortion_table(const or_geometry *g, double *tbl, int tbl_cap);
/* getRByRDist (2802-2827) */
double or_r_by_rdist(const double *tbl, int tbl_len, double rDist);
/*
 * getPortsCoordinatesAndDerivatives (2159-2314), generalised to S sensors with
 * free per-sensor parameters.  deriv (nullable) receives [S][2][4] derivatives
 * of (x,y) w.r.t. (azimuth, tilt, roll, zoom) of that sensor (the reference
 * writes the same values into its 13-parameter layout).
 */
void or_ports(const or_geometry *g, const double rots[][3][3],
              const double drots[][4][3][3], const double *tbl, int tbl_len,
              double px, double py, double disparity,
              double pXY[][2], double deriv[][2][4]);

/* GeometryCorrection.RigOffset (256-975): the auxiliary camera's place in a rig */
typedef struct {
  double main_disparity_radius, aux_disparity_radius; /* mm, each camera's disparityRadius */
  double baseline, aux_angle;                         /* mm, rad: aux centre from the main one */
  double aux_azimuth, aux_tilt, aux_roll, aux_zoom;   /* rad, rad, rad, zoom - 1 */
} or_rig_offset;
/* RigOffset.getRotMatrix (770-800) */
void or_rig_matrix(const or_rig_offset *rig, double m[3][3]);
/* RigOffset.recalcRXY (728-747): rXY_aux [S][2] */
void or_rig_rxy(const or_geometry *aux, const or_rig_offset *rig, double rxy[][2]);
/* the auxiliary camera's ports as ImageDtt.clt_bi_quad computes them (8972-8996): the main
 * camera's disparity scaled by aux / main disparity radius, the centre undistorted with the main
 * camera's model, rXY_aux, each sensor's rotation times the rig matrix
 * (CorrVector.getRotMatrices(rigMatrix) 1016-1025) */
void or_rig_aux_ports(const or_geometry *aux, const or_geometry *main_g, const or_rig_offset *rig, double px,
                      double py, double disparity_main, double pXY[][2]);

/* ---- Correlation2d ---- */
typedef struct {
  int num_pairs;
  int cam1[OR_MAX_PAIRS], cam2[OR_MAX_PAIRS];
  /* strip direction b (disparity units per strip column) and flags */
  double bx[OR_MAX_PAIRS], by[OR_MAX_PAIRS];
  int kind[OR_MAX_PAIRS];     /* 0 hor, 1 vert, 2 diag main, 3 diag other, 4 general */
  int combo_mask_lo, combo_mask_hi;  /* pairs combined into strip_combo (bits 0..63, 64..119) */
} or_pairs;

typedef struct {
  double fat_zero;
  double corr_sigma;
  double corr_red, corr_blue;
  double corr_offset;
  double min_corr;
  int corr_strip_hight;
  int twice_diagonal;
  int enhortho_width;
  double enhortho_scale;
  int corr_wndy_size; double corr_wndy_hwidth, corr_wndy_blur;
  int corr_wndx_size; double corr_wndx_hwidth, corr_wndx_blur;
} or_corr_params;

void or_default_corr_params(or_corr_params *p);
/* the 6 quad pairs PAIRS[0..5] (Correlation2d.java:52-58) */
void or_quad_pairs(or_pairs *pp);

/* correlateCompositeFD for one pair (Correlation2d.java:275-389); clt1/clt2: [C][4][64] */
void or_correlate_pair(const double *clt1, const double *clt2, int num_colors,
                       const double *col_weights, const double *lpf64,
                       double fat_zero, double *corr225);
/* scaleRotateInterpoateSingleCorrelation generalised (610-718) */
void or_strip(const double *corr225, double bx, double by, int kind, int hwidth, double *strip);
/* combineInterpolatedCorrelations (730-790) */
void or_combine_strips(const double *strips, const int *use, int num_pairs, const int *is_diag,
                       int hwidth, double offset, int twice_diagonal, double *combo);
/* getMaxXYInt axis_only (802-843): returns 1 and ix, or 0 */
int or_max_xy_int_axis(const double *combo, int hwidth, double minMax, int *ix);
/* halfFlatTopWindow (1047-1081) */
void or_half_flat_top_window(int ihwidth, double hwidth, double blur, int normalize,
                             int notch, double scale, double *wnd);
/* getMaxXCm (936-1032): returns 1 and rslt[3] or 0 (null) */
int or_max_x_cm(const double *combo, int hwidth, int ixcenter,
                const double *wy, int wy_len, const double *wx, int wx_len, double rslt[3]);
/* createOrtoNotch (2654-2675) */
void or_ortho_notch(double enhortho_width, double enhortho_scale, double *notch15);
/* getMaxXSOrtho (2502-2651) with the 3-point parabola in closed form */
int or_max_xs_ortho(const double *corrs, const int *use, int num_pairs, double offset,
                    int is_vert, const double *notch15, double rslt[2]);
/* its two halves: the 15-entry profile (0 when no pair is used), and the sub-pixel maximum
 * {xcenter - 7, strength} around a given integer maximum of a profile */
int or_max_xs_ortho_profile(const double *corrs, const int *use, int num_pairs, double offset,
                            int is_vert, const double *notch15, double c1d[15]);
void or_ortho_at(const double *c1d, int icenter, double rslt[2]);
/* getMaxXCm of a combined strip at the integer maximum ix with the windows of cp (1 / 0 as or_max_x_cm) */
int or_cm_at(const or_corr_params *cp, const double *combo, int hwidth, int ix, double rslt[3]);

/* ---- IMCLT / textures ---- */
/* iclt_2d (ImageDtt.java:3559-3666) into the padded frame (W+8)x(H+8) (no edge
 * trimming); clt: [tilesY][tilesX][4][64]; accumulated into out (caller zeroes). */
void or_iclt_tile_add(const double clt[4][64], double scale, int tx, int ty,
                      double *frame, int frame_width);
/* all tiles of clt [tiles][S][C][256] accumulated into frames [S][C][H+8][W+8]
 * (zeroed first when zero_frames), optional per-colour lpf [C][64];
 * present[tile] == 0 skips a tile */
int or_imclt_frames(const double *clt, const int *present, int tilesX, int tilesY, int S, int C, double scale,
                    const double *lpf, double *frames, int num_threads, int zero_frames);

/* ---- rig (two quad cameras) inter-camera correlation, one tile ----
 * clt_main [s_main][nc][4][64], clt_aux [s_aux][nc][4][64] -> corr225 and
 * rec {disparity, strength, dx (NaN), dy (NaN)} (ImageDtt.tileInterCamCorrs) */
void or_rig_tile(const double *clt_main, int s_main, const double *clt_aux, int s_aux, int nc,
                 const or_corr_params *cp, double cm_max_normalization, int no_int_x0, double *corr225,
                 double rec[4]);

/* ---- LMA disparity ("POLY"): Correlation2d.corrLMA (Correlation2d.java:1754-1877) ----
 * Defaults from ImageDttParameters.java:32-109. */
typedef struct {
  double min_poly_strength;  /* 0.2: LMA only where the integer-max strength exceeds it */
  int mix_corr_poly;         /* 1: the LMA result replaces the CM disparity and strength */
  double ortho_vasw_pwr;     /* 2.0: sample weight x |value|^pwr */
  int cnvx_hwnd_size;        /* 4 */
  double cnvx_weight;        /* 0.5: weight of selected non-convex cells */
  int cnvx_add3x3;           /* 1 */
  int adjust_wm, adjust_wy, adjust_wxy, adjust_ag; /* 1, 0, 1, 1 */
  double half_width, cost_wy, cost_wxy;            /* 2.0, 0.1, 0.1 */
  double lambda_initial, lambda_scale_good, lambda_scale_bad, lambda_max, rms_diff; /* 0.1, 0.5, 8, 100, 0.001 */
  int num_iter;              /* 20 */
  int pair_mask;             /* bit i: pair i takes part (dbg_pair_mask 0x3f) */
} or_lma_params;
void or_default_lma_params(or_lma_params *p);
/* filterConvex (Correlation2d.java:2029-2208): weights [225] of the cells
 * grown from (x0c, y0c) (offsets from the centre) through bi-convex cells */
void or_filter_convex(const double *corr225, int hwin, int x0c, int y0c, int add3x3, double nc_cost,
                      double *weights225);
/*
 * One tile: corrs [np][225] with quad pair kinds (0 horizontal, 1 vertical,
 * 2 main diagonal, 3 other diagonal; others ignored), xcenter = the CM x of
 * the combined strip (= -CM disparity).  Groups ortho / diagonal are combined
 * (combineCompatiblePairs 462-490), sampled (addSamples 2230-2386) and fitted
 * (Correlations2dLMA initVector / runLma, 211-640).  Returns 1 when the LMA
 * succeeded, with out = {disparity, strength, half-width WM, WXY}
 * (getDisparityStrengthWidth); 0 otherwise (out NaN).  n_samples (optional)
 * receives the sample count.
 */
int or_corr_lma(const double *corrs, const int *kind, int np, double xcenter, const or_lma_params *p,
                double out[4], int *n_samples);

/* far/foreground correction (ImageDttParameters.java:54-63 defaults) */
typedef struct {
  int fo_correct, fo_far, fo_ortho;            /* 1, 0, 1 */
  double fo_min_strength, fo_min_eff, fo_min_eff_ratio, fo_max_hwidth, fo_min_diff; /* 0.1, 0.25, 0.65, 3.0, 0.2 */
  double fo_overcorrection, fo_lim_overcorr;   /* 0.0, 2.0 */
} or_fo_params;
void or_default_fo_params(or_fo_params *f);
/* Correlation2d.foregroundCorrect (1663-1749): dir [4][4] rows {disparity, strength, WM, WXY}
 * (valid[dir] = 0 for a missing direction) -> {disparity, eff strength, max - min, ortho} */
void or_foreground_correct(int bg, int ortho, const double dir[4][4], const int valid[4], double full_disp,
                           const or_fo_params *f, double rslt[4]);
/*
 * The disparity-record update of ImageDtt.java:2254-2335 for one tile: from the
 * record's CM disparity and strength, the main LMA (corrLMA over pair_mask),
 * the mix into CM / strength (mix_corr_poly), then with fo_correct the four
 * single-direction LMAs (corr4dirsLMA 1591-1645: horizontal, vertical, main
 * and other diagonal pairs) and foregroundCorrect.  rec [3] = {CM, strength,
 * POLY} in/out (POLY NaN unless the LMA ran); lma [4] = the main LMA's
 * {disparity, strength, WM, WXY} (NaN if none).  Returns 1 if the LMA ran.
 */
int or_lma_tile(const double *corrs, const int *kind, int np, const or_lma_params *p, const or_fo_params *f,
                double rec[3], double lma[4]);
/* the same with the lazy-eye mismatch (clt_mismatch, ImageDtt.java:2340-2418): when mism is not
 * NULL the orientation fits always run, CM is not foreground-corrected, and where their spread is
 * at most mismatch_max_diff mism [np][3] receives mismatchPairsCM (Correlation2d.java:1336-1431)
 * around the disparity with max_corr_radius (3.9); elsewhere {NaN, NaN, 0} */
int or_lma_tile_mismatch(const double *corrs, const int *kind, int np, const or_lma_params *p,
                         const or_fo_params *f, double max_corr_radius, double mismatch_max_diff, double rec[3],
                         double lma[4], double *mism);
/* the polynomial mismatch (ImageDttParameters.java:50-52 defaults) */
typedef struct {
  int ly_poly;           /* 0: mismatchPairs (quadric maxima) instead of mismatchPairsCM */
  double ly_crazy_poly;  /* 1.0: a larger quadric offset zeroes the pair's strength */
  int ly_poly_backup;    /* 1: any failed / implausible pair sends all pairs to mismatchPairsCM */
} or_ly_params;
/* or_lma_tile_mismatch with the choice of mismatch measure (ImageDtt.java:2349-2405); with
 * ly_poly each pair is sampled alone like corrLMA (|value|^max_corr_radius weights, as there)
 * and measured by or_quadratic_max (Correlation2d.mismatchPairs 1434-1503) */
int or_lma_tile_mismatch_ly(const double *corrs, const int *kind, int np, const or_lma_params *p,
                            const or_fo_params *f, double max_corr_radius, double mismatch_max_diff,
                            const or_ly_params *ly, double rec[3], double lma[4], double *mism);
/* Correlations2dLMA.getMaxXYPoly (641-704): weighted quadric fit of n samples (weight > 0 taken)
 * and its maximum -> xyv {x, y, value}; 0 when the fit or the maximum does not exist */
int or_quadratic_max(const double *x, const double *y, const double *v, const double *w, int n, double xyv[3]);
/* the LMA branch of the rig's inter-camera correlation (ImageDtt.java:7497-7560) on one tile:
 * rec {disparity, strength, dx, dy} updated in place; 1 when the LMA ran and converged */
int or_rig_lma(const double *corr225, const or_lma_params *p, int use_poly, int use_xy_poly, double max_corr_radius,
               double rec[4]);

/* ---- texture tiles (ImageDtt.java:2662-2812) ---- */
typedef struct {
  double min_shot, scale_shot;        /* CLTParameters 10.0, 3.0 */
  double diff_sigma, diff_threshold;  /* 5.0, 1.5 */
  double min_agree;                   /* 3.0 (not used by tile_combine_rgba) */
  int dust_remove, keep_weights;      /* true, true */
  double corr_magic_scale;            /* 0.85 */
} or_tex_params;

/*
 * One tile of 4 quad sensors x 3 colours (R, B, G): clt [4][3][4][64], shifted
 * by extra_disparity x port offset / corr_magic_scale first when non-zero;
 * filter = correlation LPF [64].  out [12][256]: R, B, G, alpha, 4 port
 * weights, 3 colour rms + weighted rms (the keep_weights layout of
 * tile_combine_rgba, colour order RBG).  aux (optional) [16]: max_diff[4],
 * ports_rgb[12] (chn * 4 + port).
 */
void or_texture_tile(const double *clt, const double *filter, int img_mask, const double *col_weights,
                     double extra_disparity, const or_tex_params *tp, double *out, double *aux);
/* or_texture_tile with test diagnostics diag[3]: the smallest relative margin over the pixels
 * between the second port of the best pair and the next port, of dust_remove's weakest-port
 * choice, and the smallest distance of a pixel's weight exponents from the double underflow of
 * exp (745.13); INFINITY where a choice is not made.  out_alt (may be NULL) [12][256]: the tile
 * with every choice whose margin is above 0 and below near_tie taken the other way (the outputs'
 * sensitivity to the near ties an FP32 evaluation may resolve differently; an exact tie comes
 * from identical inputs and is resolved the same way). */
void or_texture_tile_diag(const double *clt, const double *filter, int img_mask, const double *col_weights,
                          double extra_disparity, const or_tex_params *tp, double *out, double *aux,
                          double *diag, double *out_alt, double near_tie);
/* or_texture_tile over tiles[n] of clt [tiles][4][3][256] on num_threads threads;
 * out [n][12][256], aux [n][16] (or NULL), extra [n] (or NULL) */
int or_texture_tiles(const double *clt, const int *tiles, const int *img_mask, const double *extra, int n,
                     const double *filter, const double *col_weights, const or_tex_params *tp, double *out,
                     double *aux, int num_threads);

/* ---- kernel preparation (QuadCLT.java:433-667, ImageDtt.java:4625-4851) ---- */
/* one 64x64 double-resolution kernel -> 4x64 CLT (CPU orientation) + 8 extras */
void or_calc_clt_kernel(const double *src64x64, int normalize, double clt[4][64], double extra[8]);
/* clt_fill_coord_corr on one colour plane of [kv][kh][8] extras */
void or_fill_coord_corr(double *ext, int kh, int kv, int kern_step);

/* ---- full tile loop (clt_aberrations_quad_corr_new, ImageDtt.java:1491-2824) ---- */
typedef struct {
  int width, height;
  int num_sensors, num_colors;
  int kernels_hor, kernels_vert, kernel_step; /* kernels_hor==0 -> identity */
  int num_threads;
  int use_ports_in;   /* 1: take ports from ports_in instead of geometry */
  int corr;           /* run stage 3 */
} or_run_cfg;

/*
 * images: [S][C][H*W] planes (sparse colour planes for Bayer).
 * kern: [S] -> [C][kv][kh][4][64]; kext: [S] -> [C][kv][kh][8] (NULL when identity).
 * tile_op: [T] (0 = skip); disparity: [T].
 * outputs (nullable): ports [T][S][2], clt [T][S][C][4][64], corr [T][P][225],
 * disp [T][OR_DISP_N], int_tl [T][S][C][2], residual [T][S][C][2].
 * Returns 0 on success.
 */
int or_run(const or_run_cfg *cfg, const or_geometry *g, const double *ports_in,
           const double *const *images, const double *const *kern, const double *const *kext,
           const int *tile_op, const double *disparity,
           const or_pairs *pairs, const or_corr_params *cp,
           double *ports, double *clt, double *corr, double *disp,
           int *int_tl, double *residual);
/* or_run with per-tile diagnostics for the parity tests: diag [T][OR_DIAG_N] (NaN where absent) =
 * the combined strip rows [16][15] (the first min(corr_strip_hight, 16) rows filled), then the
 * horizontal and the vertical ortho profile [15] each (getMaxXSOrtho c1d) */
#define OR_DIAG_ROWS 16
#define OR_DIAG_N (OR_DIAG_ROWS * 15 + 30)
int or_run_diag(const or_run_cfg *cfg, const or_geometry *g, const double *ports_in,
                const double *const *images, const double *const *kern, const double *const *kext,
                const int *tile_op, const double *disparity,
                const or_pairs *pairs, const or_corr_params *cp,
                double *ports, double *clt, double *corr, double *disp,
                int *int_tl, double *residual, double *diag);

#ifdef __cplusplus
}
#endif
#endif
