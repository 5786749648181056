// tp_internal.h -- device-side data layout of the GB300 tile processor.
//
// One "scene" = the per-camera image set, kernel tables, geometry and task
// list that GPUTileProcessor keeps in its device buffers
// (GPUTileProcessor.java:296-358).  All kernels take a SceneDev by value so a
// batch of scenes is an array of these.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define TP_DTT 8
#define TP_CLT 256          // 4 quadrants x 64 coefficients
#define TP_CORR 225         // 15 x 15 correlation surface
#define TP_MAXS 16
#define TP_MAXP 120
#define TP_MAX_STRIP 16     // rows of the combined strip
#define TP_NDISP 9

// one (task, sensor, colour) sub-tile: integer window corner, residual shift
// and kernel-table index, computed in FP64 by the plan kernel
struct SubtilePlan {
  int tlx, tly;   // ctile_left, ctile_top (ImageDtt.java:4940-4941)
  int kidx;       // (ktileY * KH + ktileX) * C + colour, -1 for identity kernels
  float rx, ry;   // residual_shift (ImageDtt.java:4942-4943)
};

struct GeomDev {
  int num_sensors;
  int pixel_width, pixel_height;
  int tbl_len;
  double focal_length, pixel_size, distortion_radius;
  double fl_pix, ri_scale;  // focal_length / (0.001 pixel_size), 0.001 pixel_size / distortion_radius
  // the model that undistorts the tile centre (the reference's gc_main): this camera's own, or
  // the main camera's for a rig's auxiliary camera, whose reverse distortion table is then loaded
  int c_pixel_width, c_pixel_height;
  double c_pixel_size, c_distortion_radius;
  int rig;                     // 1: task disparities are main-camera ones, scaled by disp_num / disp_den
  double disp_num, disp_den;   // aux / main disparity radius
  double rad_coeff[7];
  double rad_dcoeff[7];  // rad_coeff[j] * (j + 1), the derivative's coefficients (the same products)
  double rXY[TP_MAXS][2];
  double pXY0[TP_MAXS][2];
  double rots[TP_MAXS][3][3];
  double drots[TP_MAXS][4][3][3];
};

struct PairDev {
  int cam1, cam2, kind, in_combo;
  float bx, by;
};

// correlation set-up read uniformly by every warp: passed to the fused kernel by value
// (__grid_constant__), so its fields are constant-bank operands
struct CorrConst {
  int num_pairs;
  int strip_rows;
  int twice_diagonal;
  int wndy_size, wndx_size;
  int num_hor, num_vert;  // pairs of kind 0 / 1 used for ortho extraction
  int num_combo;          // pairs contributing to the combined strip
  int log_combine;        // 1: geometric mean in log domain (generalised pair sets)
  float fat_zero;
  float corr_offset;
  float min_corr;
  float col_weights[3];
  float lpf[64];          // correlation LPF (ImageDtt.java:1662-1690)
  float wndy[TP_MAX_STRIP];
  float wndx[32];
  float notch[15];
  int hor_pairs[8], vert_pairs[8];  // pair indices of kind 0 / 1 (ortho maxima)
  int adj_rounds;                   // rounds of the adjoint's pair schedule (CorrDev::adj_round)
  PairDev pairs[TP_MAXP];
};

struct CorrDev : CorrConst {
  // strip sample codes of the quad kinds 0..3 per (row*15+col, down): source index
  // iy0*15+ix0 in bits 0-7, interpolation case in bits 8-9, -1 outside the surface
  // (lane-divergent reads: kept in global memory, L1-cached)
  short strip_code[4][TP_MAX_STRIP * 15][2];
  // the adjoint's pair schedule: per round up to 4 pairs of the combined strip (-1: none) whose
  // sensors are all distinct, so the four warps of a tile add their pairs' CLT gradients into
  // disjoint sensors, and every sensor's gradient is summed in the same pair order in every run
  short adj_round[TP_MAXP][4];
};

struct SceneDev {
  int num_sensors, num_colors;
  int width, height, tilesX, tilesY;
  int kh, kv, kernel_step;
  int bayer_red_row, bayer_red_col;
  int img_dtype[TP_MAXS];   // per camera: 0 f32, 1 u16
  int64_t img_pitch;        // elements
  float color_scale[3];
  const void *images[TP_MAXS];
  const float *kernels[TP_MAXS];   // [kv][kh][C][4][64] CPU orientation
  const float *kext[TP_MAXS];      // [kv][kh][C][8]
  // task list
  int num_tasks;
  const int *task_txy;       // [n] tx | ty << 16
  const int *task_op;        // [n]
  const float *task_disp;    // [n] target disparity (tile-op mode)
  const float *task_xy;      // [n][S][2] ports as given by tp_set_tasks (float mode)
  int ports_from_geometry;   // 1: compute ports in FP64 from GeomDev
  const GeomDev *geom;
  const double *rdist_tbl;   // reverse distortion table
  // products
  double *ports;             // [n][S][2]
  double *port_deriv;        // [n][S][2][5] d(x, y)/d(azimuth, tilt, roll, zoom, disparity) or null
  SubtilePlan *plan;         // [n][S][C]
  int *tile_task;            // [tilesY*tilesX] -> task index or -1
  float *clt;                // [tiles][S][C][256]
  float *corr;               // [tiles][P][225]
  float *disp;               // [tiles][TP_NDISP]
  float *rbg;                // [S][C][H+8][W+8]
  const float *lpf_rbg;      // [C][64] or null
  int clt_lpf_mask;          // colours whose stored CLT is multiplied by lpf_rbg (the reference GPU's lpf_mask)
  const CorrDev *corr_cfg;
  float *combo;              // [tiles][RE] combined strip rows the extraction reads, or null
  float *osum;               // [tiles][32][8] per-lane ortho profile products for the separate extraction pass, or null
  float *strips;             // [tiles][pairs][RE] per-pair strip samples (adjoint input), or null
  float *tex;                // [tiles][rows][256] texture tiles (R, B, G, alpha[, 4 weights, 4 rms])
  float *tex_aux;            // [tiles][16] max_diff[4], ports_rgb[12] or null
  int num_pairs;             // host copy of corr_cfg->num_pairs (launch sizing)
  int strip_rows;            // host copy of corr_cfg->strip_rows
  int wndy_size;             // host copy of corr_cfg->wndy_size
};

// texture-tile settings (CLTParameters defaults in tp_host.cu), read uniformly
struct TexConst {
  float lpf[64];            // correlation LPF (ImageDtt.java:1662-1690)
  float col_weights[3];     // R, B, G
  float min_shot, scale_shot, rsqrt_min_shot;
  float diff_sigma;
  float corr_magic_scale;
  int dust_remove;
  int rows;                 // 4 (RGBA) or 12 (keep_weights)
  const float *extra_src;   // [tiles][extra_stride] disparities for the extra shift
  int extra_stride;
  int extra_index;          // slot in extra_src, -1: no extra shift
};

// launchers (tp_plan.cu / tp_kernels.cu)
cudaError_t launch_plan(const SceneDev &sc, cudaStream_t st);
cudaError_t launch_tile_task_map(const SceneDev &sc, cudaStream_t st);
cudaError_t launch_convert_correct(const SceneDev &sc, cudaStream_t st);
cudaError_t launch_correlate(const SceneDev &sc, cudaStream_t st);
cudaError_t launch_extract(const SceneDev &sc, cudaStream_t st);
cudaError_t launch_imclt(const SceneDev &sc, cudaStream_t st);
cudaError_t launch_imclt_fast(const SceneDev &sc, cudaStream_t st);
cudaError_t launch_compact_tasks(const int *tile_op, const float *disparity, int tilesX, int num_tiles,
                                 int *task_txy, int *task_op, float *task_disp, int *num_tasks_dev,
                                 cudaStream_t st);
cudaError_t upload_kernel_constants();
// fused forward (tp_fused.cu): convert+correct, correlation, extraction in one kernel;
// tpb/nw = tiles and warps per CTA (<= 0: defaults for the sensor/colour layout)
cudaError_t launch_fused_forward(const SceneDev &sc, const CorrConst &cc, int tpb, int nw, cudaStream_t st);
cudaError_t upload_fused_constants();
// GPU_DTT24_DRV counterpart (tp_fused.cu): 2D DTT of one mode on every 8x8 block
cudaError_t launch_dtt8x8(float *dst, const float *src, int stride, int width, int height, int mode,
                          cudaStream_t st);
// batched plans (tp_plan.cu) and persistent forward over many scenes (tp_fused.cu):
// scene classes 0 = colour warp-per-tile, 1 = mono warp-per-tile, 2 = mono pair-per-warp
cudaError_t launch_plan_batch(const SceneDev *scenes_dev, const int *task_off_dev, int n, int total_tasks,
                              cudaStream_t st);
int batch_class(const SceneDev &sc);
int batch_units(const SceneDev &sc);
cudaError_t launch_fused_batch(int cls, const SceneDev *scenes_host, const SceneDev *scenes_dev,
                               const int *unit_off_dev, int n, int total_units, cudaStream_t st);
// rig inter-camera correlation (tp_fused.cu): rig_corr [tiles][225], rig_rec [tiles][4]
cudaError_t launch_rig(const SceneDev &mn, const SceneDev &ax, const CorrConst &cc, float *rig_corr, float *rig_rec,
                       float cm_norm, int no_int_x0, cudaStream_t st);
// task compaction into a fixed device scratch array (tp_plan.cu), no allocation
int compact_scratch_max_tiles();
cudaError_t compact_scratch_address(int **ptr);
cudaError_t launch_compact_tasks_scratch(const int *tile_op, const float *disparity, int tilesX, int num_tiles,
                                         int *task_txy, int *task_op, float *task_disp, int *num_tasks_dev,
                                         int *scratch, cudaStream_t st);
// adjoint (tp_adjoint.cu): per-tile dd/dport, Jacobian rows, loss gradient
cudaError_t upload_adjoint_constants();
int adjoint_smem_bytes(int S, int C);
cudaError_t launch_adjoint(const SceneDev &sc, const CorrConst &cc, int recompute, int use_strips, float *sens, float *dval,
                           const float *dl_dd, float *jac_e, float *jac_d, float *grad_d, float *partial,
                           float *grad_e, cudaStream_t st);
// kernel preparation from PSFs (tp_kernprep.cu)
cudaError_t upload_kernprep_constants();
// LMA disparity (tp_lma.cu): the fields of tp_lma_params
struct TpLmaConst {
  float min_poly_strength;
  int mix_corr_poly;
  float ortho_vasw_pwr;
  int cnvx_hwnd_size;
  float cnvx_weight;
  int cnvx_add3x3;
  int adjust_wm, adjust_wy, adjust_wxy, adjust_ag;
  float half_width, cost_wy, cost_wxy;
  float lambda_initial, lambda_scale_good, lambda_scale_bad, lambda_max, rms_diff;
  int num_iter, pair_mask;
  int fo_correct, fo_far, fo_ortho;
  float fo_min_strength, fo_min_eff, fo_min_eff_ratio, fo_max_hwidth, fo_min_diff, fo_overcorrection,
      fo_lim_overcorr;
  int mismatch;
  float max_corr_radius, mismatch_max_diff;
  int ly_poly, ly_poly_backup;
  float ly_crazy_poly;
};
cudaError_t upload_lma_constants();
cudaError_t launch_pair_maxima(const SceneDev &sc, int P, float *out, cudaStream_t st);
cudaError_t launch_lma(const SceneDev &sc, const CorrConst &cc, const TpLmaConst &c, float *lma_out,
                       float *mismatch_out, cudaStream_t st);
// the LMA branch of the rig's inter-camera correlation (tp_lma.cu); cc1: the one-pair set-up
cudaError_t launch_rig_lma(const SceneDev &mn, const CorrConst &cc1, const TpLmaConst &c, const float *rig_corr,
                           float *rig_rec, float *tmp_disp, float *tmp_lma, int use_poly, int use_xy_poly,
                           cudaStream_t st);
cudaError_t launch_kernel_prep(const float *psf_dev, int nk, int normalize, float *clt_out, float *ext_out,
                               cudaStream_t st);
cudaError_t launch_fill_coord_corr(float *ext, int kh, int kv, int C, int kern_step, cudaStream_t st);
// texture tiles (tp_texture.cu)
cudaError_t launch_textures(const SceneDev &sc, const TexConst &tc, cudaStream_t st);
cudaError_t upload_texture_constants();
