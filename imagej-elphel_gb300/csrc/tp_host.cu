// tp_host.cu -- C ABI of the GB300 tile processor (include/tp.h).
//
// Host-side equivalent of com.elphel.imagej.gpu.GPUTileProcessor: it owns the
// device buffers of one scene geometry, converts the reference's host data
// formats on upload, and launches the stage kernels on one CUDA stream.
// Errors never abort: every entry point returns a tp_status and records a
// message retrievable with tp_last_error().
#include "../../include/tp.h"
#include "tp_internal.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <mutex>
#include <unordered_map>
#include <string>
#include <vector>

struct tp_handle {
  tp_config cfg;
  int tilesX = 0, tilesY = 0, ntiles = 0;
  cudaStream_t stream = nullptr;
  // recorded on the stream of every call that enqueues work; the getters' copies wait for it
  cudaEvent_t ev_work = nullptr;
  std::string err;
  // device buffers
  void *d_images[TP_MAXS] = {};
  int img_dtype[TP_MAXS] = {};
  float *d_kern[TP_MAXS] = {};
  float *d_kext[TP_MAXS] = {};
  int *d_task_txy = nullptr, *d_task_op = nullptr;
  float *d_task_disp = nullptr, *d_task_xy = nullptr;
  int *d_tile_op = nullptr;
  float *d_tile_disp = nullptr;
  int *d_num_tasks = nullptr;
  double *d_ports = nullptr;
  double *d_port_deriv = nullptr;
  SubtilePlan *d_plan = nullptr;
  int *d_tile_task = nullptr;
  float *d_clt = nullptr, *d_corr = nullptr, *d_disp = nullptr, *d_rbg = nullptr;
  float *d_lpf_rbg = nullptr;
  GeomDev *d_geom = nullptr;
  double *d_rdist = nullptr;
  CorrDev *d_corr_cfg = nullptr;
  float *d_tex = nullptr, *d_tex_aux = nullptr;
  float *d_combo = nullptr;  // [tiles][RE] combined strip rows of the last forward (adjoint input)
  float *d_osum = nullptr;   // [tiles][32][8] ortho profile products handed to the extraction pass
  // Once the adjoint is in use (adj_record) the forward keeps what it needs: per-pair strip
  // samples [tiles][pairs][RE] and the plan's FP64 port derivatives
  float *d_strips = nullptr;
  size_t strips_cap = 0;
  int adj_record = 0, strips_valid = 0, deriv_valid = 0;
  float *d_psf_stage = nullptr;  // staging of host PSF tables for tp_calc_kernels
  float *d_rig_corr = nullptr, *d_rig_rec = nullptr;  // inter-camera correlation with an auxiliary camera
  float *d_rig_tmp = nullptr;  // rig LMA: disparity record [tiles][TP_NDISP], then the fit [tiles][4]
  int rig_lma_done = 0;        // the rig record already holds the LMA branch's values
  // page-locked copies of the last tile ops / disparities (tp_set_tile_ops returns before its
  // upload runs), reused once the event after their upload has passed
  int *h_stage_op = nullptr;
  float *h_stage_disp = nullptr;
  cudaEvent_t ev_stage = nullptr;
  float *d_lma = nullptr;    // [tiles][4] LMA disparity, strength, WM, WXY
  float *d_mismatch = nullptr;  // [tiles][pairs][3] lazy-eye mismatch of the last LMA pass that measured it
  size_t mismatch_cap = 0;
  float *d_pairmax = nullptr;   // [tiles][pairs][3] 2D maxima of the pair surfaces (tp_get_pair_maxima)
  size_t pairmax_cap = 0;
  int mismatch_pairs = -1;
  int disp_mixed = 0;        // the LMA replaced CM / strength since the last forward
  int lma_valid = 0;         // d_lma holds the LMA of the current forward (POLY for the textures)
  int rig_aux = 0;           // the geometry is a rig's auxiliary camera (tp_set_rig_geometry)
  size_t psf_stage_kernels = 0;
  // adjoint buffers (allocated by the first tp_backward)
  float *d_sens = nullptr, *d_dval = nullptr, *d_jac_e = nullptr, *d_jac_d = nullptr, *d_grad_d = nullptr;
  float *d_partial = nullptr, *d_grad_e = nullptr, *d_dldd = nullptr;
  int adj_recompute = 0, fwd_valid = 0, have_jac = 0;
  int images_since_fwd = 0;  // an image was set after the last forward (the adjoint's CLT recompute reads them)
  int tex_rows_alloc = 0, tex_rows = 0;  // allocated rows, rows of the last run
  // host state
  int num_tasks = 0;
  int ports_from_geometry = 0;
  int have_geometry = 0, have_tasks = 0, have_corr = 0, lpf_on = 0, planned = 0;
  int num_pairs = 0, corr_capacity = 0;
  int sched_tpb = 0, sched_nw = 0;  // fused-kernel schedule (0 = defaults)
  int clt_lpf_mask = 0;             // colours whose stored CLT carries the tp_set_lpf filter
  float color_scale[3] = {1.f, 1.f, 1.f};
  GeomDev geom_host;
  CorrDev corr_host;
  tp_texture_params tex_params;
  size_t dev_bytes = 0;                          // device bytes allocated through dalloc
  std::unordered_map<void *, size_t> dev_sizes;  // their sizes, for dfree
};

static tp_status fail(tp_handle *h, tp_status st, const std::string &msg) {
  if (h) h->err = msg;
  return st;
}
static tp_status cuda_fail(tp_handle *h, cudaError_t e, const char *where) {
  return fail(h, TP_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define CK(call, where)                                    \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, where); \
  } while (0)

extern "C" {
static tp_status d2h(tp_handle *h, void *dst, const void *src, size_t bytes, const char *where);
}

static cudaStream_t pick_stream(tp_handle *h, void *s) { return s ? (cudaStream_t)s : h->stream; }

// marks the end of the work just enqueued on st: the getters order their copies after it
static tp_status mark_work(tp_handle *h, cudaStream_t st) {
  const cudaError_t e = cudaEventRecord(h->ev_work, st);
  if (e != cudaSuccess) {
    h->err = std::string("event record: ") + cudaGetErrorString(e);
    return TP_ERR_CUDA;
  }
  return TP_OK;
}

// A setter that overwrites a device buffer first waits for the handle's work in flight, which may
// still read it on another stream: on the stream of its copy (after_work), or on the host before a
// synchronous copy or a free (work_done).
static tp_status after_work(tp_handle *h, cudaStream_t st, const char *where) {
  CK(cudaStreamWaitEvent(st, h->ev_work, 0), where);
  return TP_OK;
}
static tp_status work_done(tp_handle *h, const char *where) {
  CK(cudaEventSynchronize(h->ev_work), where);
  return TP_OK;
}

// Device allocations of a handle are counted against the process-wide cap of
// tp_set_memory_limit (0 = none): an allocation beyond it fails as a failed cudaMalloc does.
static std::atomic<size_t> g_mem_limit{0};

template <typename T>
static cudaError_t dalloc(tp_handle *h, T **p, size_t n) {
  const size_t bytes = n * sizeof(T) > 0 ? n * sizeof(T) : 1;
  const size_t lim = g_mem_limit.load();
  if (lim && h->dev_bytes + bytes > lim) return cudaErrorMemoryAllocation;
  const cudaError_t e = cudaMalloc((void **)p, bytes);
  if (e == cudaSuccess) {
    h->dev_bytes += bytes;
    h->dev_sizes[(void *)*p] = bytes;
  }
  return e;
}

static void dfree(tp_handle *h, void *p) {
  if (!p) return;
  auto it = h->dev_sizes.find(p);
  if (it != h->dev_sizes.end()) {
    h->dev_bytes -= it->second;
    h->dev_sizes.erase(it);
  }
  cudaFree(p);
}

// batch tables (not counted against a handle)
template <typename T>
static cudaError_t dalloc_batch(T **p, size_t n) {
  return cudaMalloc((void **)p, n * sizeof(T) > 0 ? n * sizeof(T) : 1);
}

// floats of the per-pair strip-sample buffer for the current correlation set-up
static size_t strips_need(const tp_handle *h) {
  const int RE = (h->corr_host.strip_rows < h->corr_host.wndy_size ? h->corr_host.strip_rows : h->corr_host.wndy_size) * 15;
  return (size_t)h->ntiles * (h->num_pairs > 0 ? h->num_pairs : 1) * RE;
}

static SceneDev scene_of(tp_handle *h) {
  SceneDev sc;
  memset(&sc, 0, sizeof(sc));
  const tp_config &c = h->cfg;
  sc.num_sensors = c.num_sensors;
  sc.num_colors = c.num_colors;
  sc.width = c.width;
  sc.height = c.height;
  sc.tilesX = h->tilesX;
  sc.tilesY = h->tilesY;
  sc.kh = c.kernels_hor;
  sc.kv = c.kernels_vert;
  sc.kernel_step = c.kernel_step;
  sc.bayer_red_row = c.bayer_red_row;
  sc.bayer_red_col = c.bayer_red_col;
  sc.img_pitch = c.width;
  for (int i = 0; i < 3; i++) sc.color_scale[i] = h->color_scale[i];
  for (int s = 0; s < c.num_sensors; s++) {
    sc.images[s] = h->d_images[s];
    sc.img_dtype[s] = h->img_dtype[s];
    sc.kernels[s] = h->d_kern[s];
    sc.kext[s] = h->d_kext[s];
  }
  sc.num_tasks = h->num_tasks;
  sc.task_txy = h->d_task_txy;
  sc.task_op = h->d_task_op;
  sc.task_disp = h->d_task_disp;
  sc.task_xy = h->d_task_xy;
  sc.ports_from_geometry = h->ports_from_geometry;
  sc.geom = h->d_geom;
  sc.rdist_tbl = h->d_rdist;
  sc.ports = h->d_ports;
  sc.port_deriv = nullptr;
  sc.plan = h->d_plan;
  sc.tile_task = h->d_tile_task;
  sc.clt = h->d_clt;
  sc.corr = h->d_corr;
  sc.disp = h->d_disp;
  sc.rbg = h->d_rbg;
  sc.lpf_rbg = h->lpf_on ? h->d_lpf_rbg : nullptr;
  sc.clt_lpf_mask = h->lpf_on ? h->clt_lpf_mask : 0;
  sc.corr_cfg = h->d_corr_cfg;
  sc.combo = h->d_combo;
  sc.osum = h->d_osum;
  sc.strips = (h->adj_record && h->d_strips && strips_need(h) <= h->strips_cap) ? h->d_strips : nullptr;
  sc.tex = h->d_tex;
  sc.tex_aux = h->tex_params.aux ? h->d_tex_aux : nullptr;
  sc.num_pairs = h->num_pairs;
  sc.strip_rows = h->corr_host.strip_rows;
  sc.wndy_size = h->corr_host.wndy_size;
  return sc;
}

// ---------------------------------------------------------------------------
// Geometry set-up on the host (GeometryCorrection.java), FP64.  Operation order
// follows the reference so the device ports are those of the FP64 CPU path.
// ---------------------------------------------------------------------------
static void m3mul(const double a[3][3], const double b[3][3], double c[3][3]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0;
      for (int k = 0; k < 3; k++) s += a[i][k] * b[k][j];
      c[i][j] = s;
    }
}

// CorrVector.getRotMatrices (1043-1076) and getRotDeriveMatrices (1083-1147)
static void host_rotations(const tp_geometry *g, int S, GeomDev *gd) {
  for (int chn = 0; chn < S; chn++) {
    double ca = cos(g->azimuth[chn]), sa = sin(g->azimuth[chn]);
    double ct = cos(g->tilt[chn]), st = sin(g->tilt[chn]);
    double zoom = (1.0 + g->zoom[chn]);
    double cr0 = cos(g->roll[chn]), sr0 = sin(g->roll[chn]);
    double cr = cr0 * zoom, sr = sr0 * zoom;
    const double AZ = -1.0, TL = 1.0, RL = 1.0;  // ROT_AZ_SGN, ROT_TL_SGN, ROT_RL_SGN
    double a_az[3][3] = {{ca, 0.0, sa * AZ}, {0.0, 1.0, 0.0}, {-sa * AZ, 0.0, ca}};
    double a_t[3][3] = {{1.0, 0.0, 0.0}, {0.0, ct, st * TL}, {0.0, -st * TL, ct}};
    double a_r[3][3] = {{cr, sr * RL, 0.0}, {-sr * RL, cr, 0.0}, {0.0, 0.0, 1.0}};
    double tmp[3][3];
    m3mul(a_t, a_az, tmp);
    m3mul(a_r, tmp, gd->rots[chn]);
    double a_rz[3][3] = {{cr0 * zoom, sr0 * zoom * RL, 0.0}, {-sr0 * zoom * RL, cr0 * zoom, 0.0}, {0.0, 0.0, 1.0}};
    double a_daz[3][3] = {{-sa, 0.0, ca * AZ}, {0.0, 0.0, 0.0}, {-ca * AZ, 0.0, -sa}};
    double a_dt[3][3] = {{0.0, 0.0, 0.0}, {0.0, -st, ct * TL}, {0.0, -ct * TL, -st}};
    double a_dr[3][3] = {{-sr0 * zoom, cr0 * zoom * RL, 0.0}, {-cr0 * zoom * RL, -sr0 * zoom, 0.0}, {0.0, 0.0, 0.0}};
    double a_dz[3][3] = {{cr0, sr0 * RL, 0.0}, {-sr0 * RL, cr0, 0.0}, {0.0, 0.0, 0.0}};
    m3mul(a_t, a_daz, tmp); m3mul(a_rz, tmp, gd->drots[chn][0]);
    m3mul(a_dt, a_az, tmp); m3mul(a_rz, tmp, gd->drots[chn][1]);
    m3mul(a_t, a_az, tmp); m3mul(a_dr, tmp, gd->drots[chn][2]);
    m3mul(a_t, a_az, tmp); m3mul(a_dz, tmp, gd->drots[chn][3]);
  }
}

// calcReverseDistortionTable (2707-2757)
static int host_rdist_table(const tp_geometry *g, std::vector<double> &tbl) {
  const double delta = 1E-8, minDerivative = 0.1, stepR = 0.001, maxR = 2.0;
  const int numIterations = 1000;
  double drDistDr = 1.0;
  double A8 = g->distortion[6], A7 = g->distortion[5], A6 = g->distortion[4], A5 = g->distortion[3];
  double A = g->distortion[2], B = g->distortion[1], C = g->distortion[0];
  bool use8 = (A8 != 0.0) || (A7 != 0.0) || (A6 != 0.0);
  double d = 1.0 - A8 - A7 - A6 - A5 - A - B - C;
  double rPrev = 0.0;
  int len = (int)ceil(maxR / stepR) + 1;
  tbl.assign(len, NAN);
  tbl[0] = 1.0 / d;
  for (int i = 1; i < len; i++) {
    double rDist = stepR * i;
    double r = rPrev + stepR / drDistDr;
    for (int it = 0; it < numIterations; it++) {
      double k;
      if (use8) {
        k = (((((((A8)*r + A7) * r + A6) * r + A5) * r + A) * r + B) * r + C) * r + d;
        drDistDr = (((((((8 * A8) * r + 7 * A7) * r + 6 * A6) * r + 5 * A5) * r + 4 * A) * r + 3 * B) * r + 2 * C) * r + d;
      } else {
        k = (((A5 * r + A) * r + B) * r + C) * r + d;
        drDistDr = (((5 * A5 * r + 4 * A) * r + 3 * B) * r + 2 * C) * r + d;
      }
      double rD = r * k;
      if (drDistDr < minDerivative) return len;  // too much distortion: rest stays NaN
      if (fabs(rD - rDist) < delta) break;
      r += (rDist - rD) / drDistDr;
    }
    rPrev = r;
    tbl[i] = r / rDist;
  }
  return len;
}

// ImageDtt.java:1662-1690 (sigma used unsquared, as there)
static void host_corr_lpf(double corr_sigma, float *out) {
  const int ts = 8;
  double fd[64];
  if (corr_sigma == 0) {
    fd[0] = 1.0;
    for (int i = 1; i < 64; i++) fd[i] = 0;
  } else {
    for (int i = 0; i < ts; i++)
      for (int j = 0; j < ts; j++) fd[i * ts + j] = exp(-(i * i + j * j) / (2 * corr_sigma));
  }
  double sum = 0;
  for (int i = 0; i < ts; i++)
    for (int j = 0; j < ts; j++) {
      double d = fd[i * ts + j];
      d *= cos(M_PI * i / (2 * ts)) * cos(M_PI * j / (2 * ts));
      if (i > 0) d *= 2.0;
      if (j > 0) d *= 2.0;
      sum += d;
    }
  for (int i = 0; i < 64; i++) fd[i] /= sum;
  // DttRad2.dttt_iiie (mode 0): DCT-IIIe along rows (transposed store), then along rows again
  double c3[8][8];
  double scale = sqrt(2.0 / 8);
  for (int j = 0; j < 8; j++) {
    double ej = ((j == 0) || (j == 7)) ? 0.5 : 1.0;
    for (int k = 0; k < 8; k++) c3[k][j] = scale * ej * cos(j * (2 * k + 1) * M_PI / 16);
  }
  double tmp[64], y[64];
  for (int i = 0; i < 8; i++)
    for (int k = 0; k < 8; k++) {
      double s = 0;
      for (int j = 0; j < 8; j++) s += c3[k][j] * fd[i * 8 + j];
      tmp[k * 8 + i] = s;
    }
  for (int i = 0; i < 8; i++)
    for (int k = 0; k < 8; k++) {
      double s = 0;
      for (int j = 0; j < 8; j++) s += c3[k][j] * tmp[i * 8 + j];
      y[i * 8 + k] = s;
    }
  for (int i = 0; i < 64; i++) out[i] = (float)(y[i] * 2 * ts);
}

// Correlation2d.halfFlatTopWindow (1047-1081)
static void host_half_flat_top(int n, double hwidth, double blur, bool notch, double scale, float *out) {
  std::vector<double> w(n);
  for (int i = 0; i < n; i++) {
    if (blur <= 0.0) w[i] = (i < hwidth) ? 1.0 : 0.0;
    else if (i < hwidth - blur / 2) w[i] = 1.0;
    else if (i > hwidth + blur / 2) w[i] = 0.0;
    else w[i] = 0.5 * (1.0 - sin(M_PI * (i - hwidth) / blur));
    if (notch) w[i] = 1.0 - w[i];
  }
  double s = 0.0;
  for (int i = 0; i < n; i++) s += ((i == 0) ? 1.0 : 2.0) * w[i];
  s = 1 / s;
  for (int i = 0; i < n; i++) out[i] = (float)(w[i] * s * scale);
}

// ---------------------------------------------------------------------------
extern "C" {

tp_status tp_default_corr_params(tp_corr_params *p) {
  if (!p) return TP_ERR_ARG;
  p->fat_zero = 0.05f;
  p->corr_sigma = 0.8f;
  p->corr_red = 0.5f;
  p->corr_blue = 0.2f;
  p->corr_offset = 0.1f;
  p->min_corr = 0.02f;
  p->corr_strip_hight = 9;
  p->twice_diagonal = 1;
  p->enhortho_width = 2;
  p->enhortho_scale = 0.0f;
  p->corr_wndy_size = 2; p->corr_wndy_hwidth = 1.0f; p->corr_wndy_blur = 1.0f;
  p->corr_wndx_size = 9; p->corr_wndx_hwidth = 6.0f; p->corr_wndx_blur = 5.0f;
  return TP_OK;
}

tp_status tp_default_texture_params(tp_texture_params *p) {
  if (!p) return TP_ERR_ARG;
  p->min_shot = 10.0f;         // CLTParameters.min_shot
  p->scale_shot = 3.0f;        // CLTParameters.scale_shot
  p->diff_sigma = 5.0f;        // CLTParameters.diff_sigma
  p->corr_magic_scale = 0.85f; // CLTParameters.corr_magic_scale
  p->dust_remove = 1;
  p->keep_weights = 1;
  p->corr_mode = 2;
  p->aux = 1;
  return TP_OK;
}

tp_status tp_quad_pairs(tp_pair *pairs, int *n) {
  static const int c1[6] = {0, 2, 0, 1, 0, 2}, c2[6] = {1, 3, 2, 3, 3, 1}, kind[6] = {0, 0, 1, 1, 2, 3};
  static const float bx[6] = {1, 1, 0, 0, 1, 1}, by[6] = {0, 0, 1, 1, 1, -1};
  if (!pairs || !n) return TP_ERR_ARG;
  for (int i = 0; i < 6; i++) {
    pairs[i].cam1 = c1[i]; pairs[i].cam2 = c2[i]; pairs[i].kind = kind[i]; pairs[i].in_combo = 1;
    pairs[i].bx = bx[i]; pairs[i].by = by[i];
  }
  *n = 6;
  return TP_OK;
}

tp_status tp_create(const tp_config *cfg, tp_handle **out) {
  if (!cfg || !out) return TP_ERR_ARG;
  *out = nullptr;
  if (cfg->num_sensors < 1 || cfg->num_sensors > TP_MAX_SENSORS) return TP_ERR_ARG;
  if (cfg->num_colors != 1 && cfg->num_colors != 3) return TP_ERR_ARG;
  if (cfg->width < 16 || cfg->height < 16 || (cfg->width % 8) || (cfg->height % 8) || (cfg->width & 1) ||
      cfg->width > 65535 * 8 || cfg->height > 32767 * 8)
    return TP_ERR_ARG;
  if (cfg->kernels_hor < 0 || cfg->kernels_vert < 0 || ((cfg->kernels_hor > 0) != (cfg->kernels_vert > 0)))
    return TP_ERR_ARG;
  if (cfg->kernels_hor > 0 && cfg->kernel_step <= 0) return TP_ERR_ARG;
  tp_handle *h = new tp_handle();
  h->cfg = *cfg;
  h->tilesX = cfg->width / 8;
  h->tilesY = cfg->height / 8;
  h->ntiles = h->tilesX * h->tilesY;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= cfg->device || cfg->device < 0) {
    delete h;
    return TP_ERR_NOT_BUILT;
  }
  const int S = cfg->num_sensors, C = cfg->num_colors;
  const size_t nt = h->ntiles, npix = (size_t)cfg->width * cfg->height;
  bool ok = cudaSetDevice(cfg->device) == cudaSuccess;
  ok = ok && cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && cudaEventCreateWithFlags(&h->ev_work, cudaEventDisableTiming) == cudaSuccess;
  ok = ok && upload_kernel_constants() == cudaSuccess;
  ok = ok && upload_fused_constants() == cudaSuccess;
  ok = ok && upload_texture_constants() == cudaSuccess;
  ok = ok && upload_adjoint_constants() == cudaSuccess;
  ok = ok && upload_kernprep_constants() == cudaSuccess;
  ok = ok && upload_lma_constants() == cudaSuccess;
  tp_default_texture_params(&h->tex_params);
  for (int s = 0; ok && s < S; s++) {
    ok = dalloc(h, (float **)&h->d_images[s], npix) == cudaSuccess;
    if (ok && cfg->kernels_hor > 0) {
      size_t nk = (size_t)cfg->kernels_hor * cfg->kernels_vert * C;
      ok = dalloc(h, &h->d_kern[s], nk * TP_CLT) == cudaSuccess && dalloc(h, &h->d_kext[s], nk * 8) == cudaSuccess;
    }
  }
  ok = ok && dalloc(h, &h->d_task_txy, nt) == cudaSuccess && dalloc(h, &h->d_task_op, nt) == cudaSuccess;
  ok = ok && dalloc(h, &h->d_task_disp, nt) == cudaSuccess && dalloc(h, &h->d_task_xy, nt * S * 2) == cudaSuccess;
  ok = ok && dalloc(h, &h->d_tile_op, nt) == cudaSuccess && dalloc(h, &h->d_tile_disp, nt) == cudaSuccess;
  ok = ok && dalloc(h, &h->d_num_tasks, 2 + nt / 1024 + 1) == cudaSuccess;  // count + per-block counts
  ok = ok && dalloc(h, &h->d_ports, nt * S * 2) == cudaSuccess;
  ok = ok && dalloc(h, &h->d_plan, nt * S * C) == cudaSuccess && dalloc(h, &h->d_tile_task, nt) == cudaSuccess;
  ok = ok && dalloc(h, &h->d_clt, nt * S * C * TP_CLT) == cudaSuccess;
  ok = ok && dalloc(h, &h->d_disp, nt * TP_NDISP) == cudaSuccess;
  ok = ok && dalloc(h, &h->d_lpf_rbg, 3 * 64) == cudaSuccess;
  ok = ok && dalloc(h, &h->d_geom, 1) == cudaSuccess && dalloc(h, &h->d_rdist, 2048 + 64) == cudaSuccess;
  ok = ok && dalloc(h, &h->d_corr_cfg, 1) == cudaSuccess;
  if (ok) ok = cudaMemsetAsync(h->d_clt, 0, nt * S * C * TP_CLT * sizeof(float), h->stream) == cudaSuccess;
  if (ok) ok = cudaStreamSynchronize(h->stream) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    tp_destroy(h);
    return TP_ERR_NOMEM;
  }
  // default correlation set-up: quad pairs for 4 sensors, none otherwise
  tp_corr_params cp;
  tp_default_corr_params(&cp);
  if (S == 4) {
    tp_pair pr[6];
    int n = 0;
    tp_quad_pairs(pr, &n);
    tp_set_corr(h, &cp, pr, n);
  }
  *out = h;
  return TP_OK;
}

tp_status tp_destroy(tp_handle *h) {
  if (!h) return TP_ERR_ARG;
  for (int s = 0; s < TP_MAXS; s++) {
    dfree(h, h->d_images[s]);
    dfree(h, h->d_kern[s]);
    dfree(h, h->d_kext[s]);
  }
  void *bufs[] = {h->d_task_txy, h->d_task_op, h->d_task_disp, h->d_task_xy, h->d_tile_op, h->d_tile_disp,
                  h->d_num_tasks, h->d_ports, h->d_port_deriv, h->d_plan, h->d_tile_task, h->d_clt, h->d_corr,
                  h->d_disp, h->d_rbg, h->d_lpf_rbg, h->d_geom, h->d_rdist, h->d_corr_cfg,
                  h->d_tex, h->d_tex_aux, h->d_sens, h->d_dval, h->d_jac_e, h->d_jac_d, h->d_grad_d,
                  h->d_partial, h->d_grad_e, h->d_dldd, h->d_combo, h->d_psf_stage, h->d_rig_corr, h->d_strips, h->d_lma, h->d_mismatch,
                  h->d_pairmax,
                  h->d_rig_rec, h->d_rig_tmp, h->d_osum};
  for (void *b : bufs) dfree(h, b);
  if (h->ev_stage) {
    cudaEventSynchronize(h->ev_stage);
    cudaEventDestroy(h->ev_stage);
  }
  if (h->h_stage_op) cudaFreeHost(h->h_stage_op);
  if (h->h_stage_disp) cudaFreeHost(h->h_stage_disp);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->ev_work) cudaEventDestroy(h->ev_work);
  delete h;
  return TP_OK;
}

tp_status tp_set_memory_limit(size_t max_bytes_per_handle) {
  g_mem_limit.store(max_bytes_per_handle);
  return TP_OK;
}

tp_status tp_get_memory_usage(const tp_handle *h, size_t *bytes) {
  if (!h || !bytes) return TP_ERR_ARG;
  *bytes = h->dev_bytes;
  return TP_OK;
}

tp_status tp_last_error(const tp_handle *h, char *buf, int n) {
  if (!h || !buf || n <= 0) return TP_ERR_ARG;
  snprintf(buf, (size_t)n, "%s", h->err.c_str());
  return TP_OK;
}

// RigOffset.getRotMatrix (GeometryCorrection.java:770-800): aux roll (with zoom) x tilt x azimuth
static void host_rig_matrix(const tp_rig_offset *r, double m[3][3]) {
  const double ca = cos(r->aux_azimuth), sa = sin(r->aux_azimuth);
  const double ct = cos(r->aux_tilt), st = sin(r->aux_tilt);
  const double zoom = 1.0 + r->aux_zoom;
  const double cr = cos(r->aux_roll) * zoom, sr = sin(r->aux_roll) * zoom;
  const double AZ = -1.0, TL = 1.0, RL = 1.0;
  const double a_az[3][3] = {{ca, 0.0, sa * AZ}, {0.0, 1.0, 0.0}, {-sa * AZ, 0.0, ca}};
  const double a_t[3][3] = {{1.0, 0.0, 0.0}, {0.0, ct, st * TL}, {0.0, -st * TL, ct}};
  const double a_r[3][3] = {{cr, sr * RL, 0.0}, {-sr * RL, cr, 0.0}, {0.0, 0.0, 1.0}};
  double t[3][3];
  m3mul(a_t, a_az, t);
  m3mul(a_r, t, m);
}

// the device geometry of camera g; the tile centre is undistorted with gc (g itself, or a rig's
// main camera), whose reverse distortion table is uploaded
static tp_status upload_geometry(tp_handle *h, const tp_geometry *g, const tp_geometry *gc, const tp_rig_offset *rig) {
  const int S = h->cfg.num_sensors;
  GeomDev &gd = h->geom_host;
  memset(&gd, 0, sizeof(gd));
  gd.num_sensors = S;
  gd.pixel_width = g->pixel_width;
  gd.pixel_height = g->pixel_height;
  gd.focal_length = g->focal_length;
  gd.pixel_size = g->pixel_size;
  gd.distortion_radius = g->distortion_radius;
  // per-camera constants of getPortsCoordinatesAndDerivatives, divided once here (IEEE division:
  // the same double as the device's correctly rounded one; host code is built without contraction)
  gd.fl_pix = g->focal_length / (0.001 * g->pixel_size);
  gd.ri_scale = (0.001 * g->pixel_size) / g->distortion_radius;
  gd.c_pixel_width = gc->pixel_width;
  gd.c_pixel_height = gc->pixel_height;
  gd.c_pixel_size = gc->pixel_size;
  gd.c_distortion_radius = gc->distortion_radius;
  for (int i = 0; i < 7; i++) {
    gd.rad_coeff[i] = g->distortion[i];
    gd.rad_dcoeff[i] = g->distortion[i] * (double)(i + 1);
  }
  for (int s = 0; s < S; s++)
    for (int k = 0; k < 2; k++) {
      gd.rXY[s][k] = g->rXY[s][k];
      gd.pXY0[s][k] = g->pXY0[s][k];
    }
  host_rotations(g, S, &gd);
  if (rig) {
    // RigOffset.recalcRXY (728-747): baseline offset plus the aux-roll-rotated lens offsets
    const double xc_pix = rig->baseline * cos(rig->aux_angle) / rig->aux_disparity_radius;
    const double yc_pix = rig->baseline * sin(rig->aux_angle) / rig->aux_disparity_radius;
    const double ssr = 1.0;
    for (int s = 0; s < S; s++) {
      gd.rXY[s][0] = xc_pix + cos(rig->aux_roll) * g->rXY[s][0] + ssr * sin(rig->aux_roll) * g->rXY[s][1];
      gd.rXY[s][1] = yc_pix - ssr * sin(rig->aux_roll) * g->rXY[s][0] + cos(rig->aux_roll) * g->rXY[s][1];
    }
    // CorrVector.getRotMatrices(rigMatrix) (1016-1025): each sensor's rotation, then the rig's
    double rm[3][3], t[3][3];
    host_rig_matrix(rig, rm);
    for (int s = 0; s < S; s++) {
      m3mul(gd.rots[s], rm, t);
      memcpy(gd.rots[s], t, sizeof(t));
      for (int k = 0; k < 4; k++) {
        m3mul(gd.drots[s][k], rm, t);
        memcpy(gd.drots[s][k], t, sizeof(t));
      }
    }
    gd.rig = 1;
    gd.disp_num = rig->aux_disparity_radius;
    gd.disp_den = rig->main_disparity_radius;
  }
  std::vector<double> tbl;
  gd.tbl_len = host_rdist_table(gc, tbl);
  if (gd.tbl_len > 2048 + 64) return fail(h, TP_ERR_ARG, "distortion table too long");
  if (after_work(h, h->stream, "tp_set_geometry") != TP_OK) return TP_ERR_CUDA;
  CK(cudaMemcpyAsync(h->d_geom, &gd, sizeof(gd), cudaMemcpyHostToDevice, h->stream), "tp_set_geometry");
  CK(cudaMemcpyAsync(h->d_rdist, tbl.data(), sizeof(double) * gd.tbl_len, cudaMemcpyHostToDevice, h->stream),
     "tp_set_geometry");
  CK(cudaStreamSynchronize(h->stream), "tp_set_geometry");
  h->have_geometry = 1;
  h->rig_aux = rig != nullptr;
  h->planned = 0;
  h->deriv_valid = 0;
  h->fwd_valid = 0;
  return TP_OK;
}

tp_status tp_set_geometry(tp_handle *h, const tp_geometry *g) {
  if (!h || !g) return TP_ERR_ARG;
  return upload_geometry(h, g, g, nullptr);
}

tp_status tp_set_rig_geometry(tp_handle *h, const tp_geometry *aux, const tp_geometry *main_camera,
                              const tp_rig_offset *rig) {
  if (!h || !aux) return TP_ERR_ARG;
  if (!main_camera || !rig) return upload_geometry(h, aux, aux, nullptr);
  if (!(rig->main_disparity_radius > 0.0) || !(rig->aux_disparity_radius > 0.0))
    return fail(h, TP_ERR_ARG, "tp_set_rig_geometry: disparity radii must be positive");
  return upload_geometry(h, aux, main_camera, rig);
}

tp_status tp_set_kernels(tp_handle *h, int cam, const float *kernels, const float *offs, int layout) {
  if (!h || !kernels || !offs) return TP_ERR_ARG;
  if (cam < 0 || cam >= h->cfg.num_sensors) return fail(h, TP_ERR_ARG, "tp_set_kernels: bad camera");
  if (h->cfg.kernels_hor <= 0) return fail(h, TP_ERR_STATE, "tp_set_kernels: handle created without kernels");
  size_t nk = (size_t)h->cfg.kernels_hor * h->cfg.kernels_vert * h->cfg.num_colors;
  if (layout != TP_KERNELS_GPU && layout != TP_KERNELS_CPU) return fail(h, TP_ERR_ARG, "tp_set_kernels: bad layout");
  if (work_done(h, "tp_set_kernels") != TP_OK) return TP_ERR_CUDA;
  if (layout == TP_KERNELS_GPU) {
    // undo the 8x8 transpose of GPUTileProcessor.setConvolutionKernels (406-410)
    std::vector<float> t(nk * TP_CLT);
    for (size_t k = 0; k < nk * 4; k++)
      for (int i0 = 0; i0 < 64; i0++) t[k * 64 + (((i0 & 7) << 3) | (i0 >> 3))] = kernels[k * 64 + i0];
    CK(cudaMemcpy(h->d_kern[cam], t.data(), nk * TP_CLT * sizeof(float), cudaMemcpyHostToDevice), "tp_set_kernels");
  } else {
    CK(cudaMemcpy(h->d_kern[cam], kernels, nk * TP_CLT * sizeof(float), cudaMemcpyHostToDevice), "tp_set_kernels");
  }
  CK(cudaMemcpy(h->d_kext[cam], offs, nk * 8 * sizeof(float), cudaMemcpyHostToDevice), "tp_set_kernels");
  h->planned = 0;
  h->deriv_valid = 0;
  h->fwd_valid = 0;
  return TP_OK;
}

tp_status tp_calc_kernels(tp_handle *h, int cam, const float *psf, int psf_on_device, int normalize, int coord_corr,
                          void *stream) {
  if (!h || !psf) return TP_ERR_ARG;
  if (cam < 0 || cam >= h->cfg.num_sensors) return fail(h, TP_ERR_ARG, "tp_calc_kernels: bad camera");
  if (h->cfg.kernels_hor <= 0) return fail(h, TP_ERR_STATE, "tp_calc_kernels: handle created without kernels");
  cudaStream_t st = pick_stream(h, stream);
  if (after_work(h, st, "tp_calc_kernels") != TP_OK) return TP_ERR_CUDA;
  const size_t nk = (size_t)h->cfg.kernels_hor * h->cfg.kernels_vert * h->cfg.num_colors;
  if (psf_on_device) {
    CK(launch_kernel_prep(psf, (int)nk, normalize, h->d_kern[cam], h->d_kext[cam], st), "tp_calc_kernels");
  } else {
    const size_t chunk = nk < 8192 ? nk : 8192;  // kernel tiles per staged upload (128 MB)
    if (h->psf_stage_kernels < chunk) {
      dfree(h, h->d_psf_stage);
      h->d_psf_stage = nullptr;
      h->psf_stage_kernels = 0;
      if (dalloc(h, &h->d_psf_stage, chunk * 4096) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, TP_ERR_NOMEM, "tp_calc_kernels: PSF staging buffer");
      }
      h->psf_stage_kernels = chunk;
    }
    for (size_t k0 = 0; k0 < nk; k0 += chunk) {
      const size_t n = (nk - k0) < chunk ? (nk - k0) : chunk;
      CK(cudaMemcpyAsync(h->d_psf_stage, psf + k0 * 4096, n * 4096 * sizeof(float), cudaMemcpyHostToDevice, st),
         "tp_calc_kernels");
      CK(launch_kernel_prep(h->d_psf_stage, (int)n, normalize, h->d_kern[cam] + k0 * TP_CLT, h->d_kext[cam] + k0 * 8,
                            st),
         "tp_calc_kernels");
      CK(cudaStreamSynchronize(st), "tp_calc_kernels");  // the staging buffer is reused
    }
  }
  if (coord_corr)
    CK(launch_fill_coord_corr(h->d_kext[cam], h->cfg.kernels_hor, h->cfg.kernels_vert, h->cfg.num_colors,
                              h->cfg.kernel_step, st),
       "tp_calc_kernels");
  h->planned = 0;
  h->deriv_valid = 0;
  h->fwd_valid = 0;
  return mark_work(h, st);
}

tp_status tp_get_kernels(tp_handle *h, int cam, float *kernels, float *kernel_offsets) {
  if (!h) return TP_ERR_ARG;
  if (cam < 0 || cam >= h->cfg.num_sensors || h->cfg.kernels_hor <= 0) return fail(h, TP_ERR_ARG, "tp_get_kernels");
  const size_t nk = (size_t)h->cfg.kernels_hor * h->cfg.kernels_vert * h->cfg.num_colors;
  tp_status r = TP_OK;
  if (kernels) r = d2h(h, kernels, h->d_kern[cam], nk * TP_CLT * sizeof(float), "tp_get_kernels");
  if (r == TP_OK && kernel_offsets) r = d2h(h, kernel_offsets, h->d_kext[cam], nk * 8 * sizeof(float), "tp_get_kernels");
  return r;
}

// Images and colour scales are read only by the forward (and by the adjoint when it recomputes
// the CLT): the last forward's products stay valid for the passes that read them (LMA, rig,
// IMCLT, textures), as in a frame loop that uploads the next frame during those passes.
tp_status tp_set_color_scales(tp_handle *h, const float *scales) {
  if (h) h->images_since_fwd = 1;
  if (!h || !scales) return TP_ERR_ARG;
  for (int i = 0; i < 3; i++) h->color_scale[i] = scales[i];
  return TP_OK;
}

tp_status tp_set_image(tp_handle *h, int cam, const void *image, int dtype, size_t pitch) {
  if (h) h->images_since_fwd = 1;
  if (!h || !image) return TP_ERR_ARG;
  if (cam < 0 || cam >= h->cfg.num_sensors) return fail(h, TP_ERR_ARG, "tp_set_image: bad camera");
  if (dtype != TP_F32 && dtype != TP_U16) return fail(h, TP_ERR_ARG, "tp_set_image: bad dtype");
  size_t es = dtype == TP_U16 ? 2 : 4;
  if (pitch == 0) pitch = h->cfg.width;
  if (pitch < (size_t)h->cfg.width) return fail(h, TP_ERR_ARG, "tp_set_image: pitch < width");
  if (after_work(h, h->stream, "tp_set_image") != TP_OK) return TP_ERR_CUDA;
  CK(cudaMemcpy2DAsync(h->d_images[cam], h->cfg.width * es, image, pitch * es, h->cfg.width * es, h->cfg.height,
                       cudaMemcpyHostToDevice, h->stream),
     "tp_set_image");
  CK(cudaStreamSynchronize(h->stream), "tp_set_image");
  h->img_dtype[cam] = dtype;
  return TP_OK;
}

tp_status tp_set_image_async(tp_handle *h, int cam, const void *image, int dtype, size_t pitch, void *stream) {
  if (h) h->images_since_fwd = 1;
  if (!h || !image) return TP_ERR_ARG;
  if (cam < 0 || cam >= h->cfg.num_sensors) return fail(h, TP_ERR_ARG, "tp_set_image_async: bad camera");
  if (dtype != TP_F32 && dtype != TP_U16) return fail(h, TP_ERR_ARG, "tp_set_image_async: bad dtype");
  size_t es = dtype == TP_U16 ? 2 : 4;
  if (pitch == 0) pitch = h->cfg.width;
  if (pitch < (size_t)h->cfg.width) return fail(h, TP_ERR_ARG, "tp_set_image_async: pitch < width");
  if (after_work(h, pick_stream(h, stream), "tp_set_image_async") != TP_OK) return TP_ERR_CUDA;
  CK(cudaMemcpy2DAsync(h->d_images[cam], h->cfg.width * es, image, pitch * es, h->cfg.width * es, h->cfg.height,
                       cudaMemcpyHostToDevice, pick_stream(h, stream)),
     "tp_set_image_async");
  h->img_dtype[cam] = dtype;
  return TP_OK;
}

tp_status tp_set_tasks(tp_handle *h, const float *packed, int n) {
  if (!h || (!packed && n > 0)) return TP_ERR_ARG;
  if (n < 0 || n > h->ntiles) return fail(h, TP_ERR_ARG, "tp_set_tasks: bad task count");
  const int S = h->cfg.num_sensors, rec = 2 + 2 * S;
  std::vector<int> txy(n), op(n);
  std::vector<float> xy((size_t)n * S * 2);
  const float lim[2][2] = {{-(float)TP_PORT_MARGIN, (float)(h->cfg.width + TP_PORT_MARGIN)},
                           {-(float)TP_PORT_MARGIN, (float)(h->cfg.height + TP_PORT_MARGIN)}};
  for (int i = 0; i < n; i++) {
    memcpy(&op[i], packed + (size_t)i * rec, 4);
    memcpy(&txy[i], packed + (size_t)i * rec + 1, 4);
    int tx = txy[i] & 0xffff, ty = txy[i] >> 16;
    if (tx >= h->tilesX || ty >= h->tilesY || ty < 0) return fail(h, TP_ERR_ARG, "tp_set_tasks: tile out of range");
    for (int k = 0; k < 2 * S; k++) {
      const float v = packed[(size_t)i * rec + 2 + k];
      // NaN fails both comparisons
      if (!(v >= lim[k & 1][0] && v <= lim[k & 1][1])) {
        char msg[160];
        snprintf(msg, sizeof(msg), "tp_set_tasks: task %d sensor %d port %c = %g is not finite or more than %d px "
                 "outside the image", i, k >> 1, (k & 1) ? 'y' : 'x', (double)v, TP_PORT_MARGIN);
        return fail(h, TP_ERR_ARG, msg);
      }
      xy[(size_t)i * 2 * S + k] = v;
    }
  }
  CK(cudaStreamWaitEvent(h->stream, h->ev_work, 0), "tp_set_tasks");  // in-flight work reads the old list
  if (n > 0) {
    CK(cudaMemcpyAsync(h->d_task_txy, txy.data(), n * sizeof(int), cudaMemcpyHostToDevice, h->stream), "tp_set_tasks");
    CK(cudaMemcpyAsync(h->d_task_op, op.data(), n * sizeof(int), cudaMemcpyHostToDevice, h->stream), "tp_set_tasks");
    CK(cudaMemcpyAsync(h->d_task_xy, xy.data(), xy.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream),
       "tp_set_tasks");
  }
  CK(cudaStreamSynchronize(h->stream), "tp_set_tasks");
  h->num_tasks = n;
  h->ports_from_geometry = 0;
  h->have_tasks = 1;
  h->planned = 0;
  h->deriv_valid = 0;
  h->fwd_valid = 0;
  return TP_OK;
}

// The tile ops go up without a host round trip: the task count is counted here (the compaction on
// the device selects the same tiles, tile_op != 0), the arrays are copied into page-locked staging
// (so the caller's buffers are free on return) and uploaded and compacted on the handle's stream
// after the handle's last work, which still reads the task list it replaces.
tp_status tp_set_tile_ops(tp_handle *h, const int *tile_op, const float *disp) {
  if (!h || !tile_op || !disp) return TP_ERR_ARG;
  if (!h->have_geometry) return fail(h, TP_ERR_STATE, "tp_set_tile_ops: geometry not set");
  int n = 0;
  for (int i = 0; i < h->ntiles; i++) {
    // NaN fails the comparison
    if (tile_op[i] != 0 && !(fabsf(disp[i]) <= TP_MAX_DISPARITY)) {
      char msg[160];
      snprintf(msg, sizeof(msg), "tp_set_tile_ops: tile %d disparity %g is not finite or beyond +-%g px", i,
               (double)disp[i], (double)TP_MAX_DISPARITY);
      return fail(h, TP_ERR_ARG, msg);
    }
    n += tile_op[i] != 0;
  }
  if (!h->h_stage_op) {
    if (cudaEventCreateWithFlags(&h->ev_stage, cudaEventDisableTiming) != cudaSuccess ||
        cudaMallocHost((void **)&h->h_stage_op, h->ntiles * sizeof(int)) != cudaSuccess ||
        cudaMallocHost((void **)&h->h_stage_disp, h->ntiles * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      return fail(h, TP_ERR_NOMEM, "tp_set_tile_ops: staging buffers");
    }
  } else {
    CK(cudaEventSynchronize(h->ev_stage), "tp_set_tile_ops");  // the previous upload has read them
  }
  memcpy(h->h_stage_op, tile_op, h->ntiles * sizeof(int));
  memcpy(h->h_stage_disp, disp, h->ntiles * sizeof(float));
  CK(cudaStreamWaitEvent(h->stream, h->ev_work, 0), "tp_set_tile_ops");
  CK(cudaMemcpyAsync(h->d_tile_op, h->h_stage_op, h->ntiles * sizeof(int), cudaMemcpyHostToDevice, h->stream),
     "tp_set_tile_ops");
  CK(cudaMemcpyAsync(h->d_tile_disp, h->h_stage_disp, h->ntiles * sizeof(float), cudaMemcpyHostToDevice,
                     h->stream),
     "tp_set_tile_ops");
  CK(cudaEventRecord(h->ev_stage, h->stream), "tp_set_tile_ops");
  CK(launch_compact_tasks(h->d_tile_op, h->d_tile_disp, h->tilesX, h->ntiles, h->d_task_txy, h->d_task_op,
                          h->d_task_disp, h->d_num_tasks, h->stream),
     "tp_set_tile_ops");
  h->num_tasks = n;
  h->ports_from_geometry = 1;
  h->have_tasks = 1;
  h->planned = 0;
  h->deriv_valid = 0;
  h->fwd_valid = 0;
  return mark_work(h, h->stream);
}

tp_status tp_set_lpf(tp_handle *h, const float *lpf) {
  if (!h) return TP_ERR_ARG;
  if (!lpf) {
    h->lpf_on = 0;
    return TP_OK;
  }
  if (work_done(h, "tp_set_lpf") != TP_OK) return TP_ERR_CUDA;
  CK(cudaMemcpy(h->d_lpf_rbg, lpf, h->cfg.num_colors * 64 * sizeof(float), cudaMemcpyHostToDevice), "tp_set_lpf");
  h->lpf_on = 1;
  return TP_OK;
}

tp_status tp_set_clt_lpf_mask(tp_handle *h, int lpf_mask) {
  if (!h) return TP_ERR_ARG;
  if (lpf_mask < 0 || (lpf_mask >> h->cfg.num_colors) != 0)
    return fail(h, TP_ERR_ARG, "tp_set_clt_lpf_mask: one bit per colour");
  h->clt_lpf_mask = lpf_mask;
  h->fwd_valid = 0;
  return TP_OK;
}

// the passes that read the stored CLT expect it unfiltered
static bool clt_filtered(const tp_handle *h) { return h->lpf_on && h->clt_lpf_mask; }

tp_status tp_set_corr(tp_handle *h, const tp_corr_params *p, const tp_pair *pairs, int np) {
  if (h) h->fwd_valid = 0;
  if (!h || !p || (!pairs && np > 0)) return TP_ERR_ARG;
  if (np < 0 || np > TP_MAX_PAIRS) return fail(h, TP_ERR_ARG, "tp_set_corr: too many pairs");
  if (p->corr_strip_hight < 1 || p->corr_strip_hight > TP_MAX_STRIP || p->corr_wndy_size < 1 ||
      p->corr_wndy_size > TP_MAX_STRIP || p->corr_wndx_size < 1 || p->corr_wndx_size > 32)
    return fail(h, TP_ERR_ARG, "tp_set_corr: window sizes out of range");
  CorrDev &cd = h->corr_host;
  memset(&cd, 0, sizeof(cd));
  cd.num_pairs = np;
  cd.strip_rows = p->corr_strip_hight;
  cd.twice_diagonal = p->twice_diagonal;
  cd.wndy_size = p->corr_wndy_size;
  cd.wndx_size = p->corr_wndx_size;
  cd.fat_zero = p->fat_zero;
  cd.corr_offset = p->corr_offset;
  cd.min_corr = p->min_corr;
  double g = 1.0 / (1.0 + p->corr_red + p->corr_blue);  // ImageDtt.java:1571-1581
  cd.col_weights[2] = (float)g;
  cd.col_weights[0] = (float)(p->corr_red * g);
  cd.col_weights[1] = (float)(p->corr_blue * g);
  host_corr_lpf(p->corr_sigma, cd.lpf);
  host_half_flat_top(p->corr_wndy_size, p->corr_wndy_hwidth, p->corr_wndy_blur, false, 1.0, cd.wndy);
  host_half_flat_top(p->corr_wndx_size, p->corr_wndx_hwidth, p->corr_wndx_blur, false, 2.0, cd.wndx);
  for (int i = 0; i < 15; i++) {  // Correlation2d.createOrtoNotch (2654-2675)
    double v = ((i < (8 - p->enhortho_width)) || (i > (8 - 2 + p->enhortho_width))) ? 1.0 : p->enhortho_scale;
    if (i == 7) v = 0.0;
    cd.notch[i] = (float)(v * sin(M_PI * (i + 1.0) / 16));
  }
  bool general = np > 6;
  for (int i = 0; i < np; i++) {
    if (pairs[i].cam1 < 0 || pairs[i].cam1 >= h->cfg.num_sensors || pairs[i].cam2 < 0 ||
        pairs[i].cam2 >= h->cfg.num_sensors || pairs[i].kind < 0 || pairs[i].kind > 4)
      return fail(h, TP_ERR_ARG, "tp_set_corr: bad pair");
    cd.pairs[i].cam1 = pairs[i].cam1;
    cd.pairs[i].cam2 = pairs[i].cam2;
    cd.pairs[i].kind = pairs[i].kind;
    cd.pairs[i].in_combo = pairs[i].in_combo;
    cd.pairs[i].bx = pairs[i].bx;
    cd.pairs[i].by = pairs[i].by;
    if (pairs[i].in_combo) cd.num_combo++;
    if (pairs[i].kind == 0) cd.num_hor++;
    if (pairs[i].kind == 1) cd.num_vert++;
    if (pairs[i].kind == 4) general = true;
  }
  cd.log_combine = general ? 1 : 0;
  if (general) cd.num_hor = cd.num_vert = 0;  // ortho maxima are defined for the quad layout only
  if (cd.num_hor > 8 || cd.num_vert > 8) return fail(h, TP_ERR_ARG, "tp_set_corr: more than 8 hor/vert pairs");
  for (int i = 0, nh = 0, nv = 0; i < np && !general; i++) {
    if (pairs[i].kind == 0) cd.hor_pairs[nh++] = i;
    if (pairs[i].kind == 1) cd.vert_pairs[nv++] = i;
  }
  // sample points of Correlation2d.scaleRotateInterpoateSingleCorrelation (610-718) for the quad kinds
  for (int kind = 0; kind < 4; kind++)
    for (int e = 0; e < TP_MAX_STRIP * 15; e++)
      for (int dn = 0; dn < 2; dn++) {
        const int row = e / 15, scol = e % 15 - 7, down = dn ? 1 : -1;
        const int sh = (kind > 1) ? 0 : 1, ilimit = 7 << sh;
        int xn, yn;
        if (kind == 0) { xn = 2 * scol + (row & 1); yn = down * row; }
        else if (kind == 1) { xn = down * row; yn = 2 * scol + (row & 1); }
        else if (kind == 2) { xn = scol - ((down * row) >> 1); yn = scol + ((down * row + 1) >> 1); }
        else { xn = scol - ((down * row) >> 1); yn = -scol - ((down * row + 1) >> 1); }
        short code = -1;
        if (!(xn > ilimit || xn < -ilimit || yn > ilimit || yn < -ilimit)) {
          const int ix0 = (xn + ilimit) >> sh, iy0 = (yn + ilimit) >> sh;
          const bool ix = (xn & ((1 << sh) - 1)) == 0, iy = (yn & ((1 << sh) - 1)) == 0;
          const int cs = (ix && iy) ? 0 : (iy ? 1 : (ix ? 2 : 3));
          code = (short)((iy0 * 15 + ix0) | (cs << 8));
        }
        cd.strip_code[kind][e][dn] = code;
      }
  // the adjoint's rounds: greedily, in pair order, up to 4 combined-strip pairs on distinct sensors
  {
    std::vector<int> left;
    for (int i = 0; i < np; i++)
      if (pairs[i].in_combo) left.push_back(i);
    int nr = 0;
    while (!left.empty()) {
      std::vector<int> rest;
      unsigned long long used = 0;
      int k = 0;
      for (int i : left) {
        const unsigned long long m = (1ull << pairs[i].cam1) | (1ull << pairs[i].cam2);
        if (k < 4 && !(used & m)) {
          cd.adj_round[nr][k++] = (short)i;
          used |= m;
        } else {
          rest.push_back(i);
        }
      }
      for (; k < 4; k++) cd.adj_round[nr][k] = -1;
      nr++;
      left.swap(rest);
    }
    cd.adj_rounds = nr;
  }
  if (work_done(h, "tp_set_corr") != TP_OK) return TP_ERR_CUDA;  // before the free and the table copy
  if (np > h->corr_capacity) {
    dfree(h, h->d_corr);
    h->d_corr = nullptr;
    h->corr_capacity = 0;
    if (dalloc(h, &h->d_corr, (size_t)h->ntiles * np * TP_CORR) != cudaSuccess) {
      cudaGetLastError();
      return fail(h, TP_ERR_NOMEM, "tp_set_corr: correlation buffer");
    }
    h->corr_capacity = np;
  }
  if (!h->d_combo && dalloc(h, &h->d_combo, (size_t)h->ntiles * TP_MAX_STRIP * 15) != cudaSuccess) {
    cudaGetLastError();
    return fail(h, TP_ERR_NOMEM, "tp_set_corr: combined strip buffer");
  }
  if (!h->d_osum && dalloc(h, &h->d_osum, (size_t)h->ntiles * 256) != cudaSuccess) {
    cudaGetLastError();
    return fail(h, TP_ERR_NOMEM, "tp_set_corr: ortho profile buffer");
  }
  CK(cudaMemcpy(h->d_corr_cfg, &cd, sizeof(cd), cudaMemcpyHostToDevice), "tp_set_corr");
  h->num_pairs = np;
  h->have_corr = 1;
  return TP_OK;
}

static tp_status ensure_plan(tp_handle *h, cudaStream_t st) {
  if (!h->have_tasks) return fail(h, TP_ERR_STATE, "no tasks set (tp_set_tasks / tp_set_tile_ops)");
  if (h->ports_from_geometry && !h->have_geometry) return fail(h, TP_ERR_STATE, "geometry not set");
  if (h->planned) return TP_OK;
  CK(cudaStreamWaitEvent(st, h->ev_work, 0), "plan");  // the task list, uploaded on the handle's stream
  SceneDev sc = scene_of(h);
  const bool with_deriv = h->adj_record && h->d_port_deriv && h->ports_from_geometry;
  if (with_deriv) sc.port_deriv = h->d_port_deriv;  // the adjoint's port derivatives, same ports
  CK(launch_plan(sc, st), "plan");
  CK(launch_tile_task_map(sc, st), "tile map");
  h->planned = 1;
  h->deriv_valid = with_deriv ? 1 : 0;
  return TP_OK;
}

tp_status tp_ports(tp_handle *h, void *stream) {
  if (!h) return TP_ERR_ARG;
  h->planned = 0;
  h->deriv_valid = 0;
  h->fwd_valid = 0;
  cudaStream_t st = pick_stream(h, stream);
  tp_status r = ensure_plan(h, st);
  return r != TP_OK ? r : mark_work(h, st);
}

tp_status tp_convert_correct(tp_handle *h, void *stream) {
  if (!h) return TP_ERR_ARG;
  cudaStream_t st = pick_stream(h, stream);
  tp_status r = ensure_plan(h, st);
  if (r != TP_OK) return r;
  CK(launch_convert_correct(scene_of(h), st), "convert_correct");
  h->lma_valid = 0;
  return mark_work(h, st);
}

tp_status tp_correlate(tp_handle *h, void *stream) {
  if (!h) return TP_ERR_ARG;
  if (!h->have_corr || h->num_pairs == 0) return fail(h, TP_ERR_STATE, "tp_correlate: no pairs set");
  if (clt_filtered(h)) return fail(h, TP_ERR_STATE, "tp_correlate: the stored CLT is low-pass filtered (tp_set_clt_lpf_mask)");
  cudaStream_t st = pick_stream(h, stream);
  tp_status r = ensure_plan(h, st);
  if (r != TP_OK) return r;
  CK(launch_correlate(scene_of(h), st), "correlate");
  return mark_work(h, st);
}

tp_status tp_extract(tp_handle *h, void *stream) {
  if (!h) return TP_ERR_ARG;
  if (!h->have_corr || h->num_pairs == 0) return fail(h, TP_ERR_STATE, "tp_extract: no pairs set");
  cudaStream_t st = pick_stream(h, stream);
  tp_status r = ensure_plan(h, st);
  if (r != TP_OK) return r;
  CK(launch_extract(scene_of(h), st), "extract");
  return mark_work(h, st);
}

tp_status tp_imclt(tp_handle *h, void *stream) {
  if (!h) return TP_ERR_ARG;
  cudaStream_t st = pick_stream(h, stream);
  tp_status r = ensure_plan(h, st);
  if (r != TP_OK) return r;
  if (!h->d_rbg) {
    size_t n = (size_t)h->cfg.num_sensors * h->cfg.num_colors * (h->cfg.width + 8) * (h->cfg.height + 8);
    if (dalloc(h, &h->d_rbg, n) != cudaSuccess) {
      cudaGetLastError();
      return fail(h, TP_ERR_NOMEM, "tp_imclt: frame buffer");
    }
  }
  CK(launch_imclt_fast(scene_of(h), st), "imclt");
  return mark_work(h, st);
}

tp_status tp_set_texture_params(tp_handle *h, const tp_texture_params *p) {
  if (!h || !p) return TP_ERR_ARG;
  if (!(p->diff_sigma > 0.f) || !(p->corr_magic_scale > 0.f) || (p->scale_shot > 0.f && !(p->min_shot > 0.f)))
    return fail(h, TP_ERR_ARG, "tp_set_texture_params: diff_sigma, corr_magic_scale and min_shot must be > 0");
  if (p->corr_mode < -1 || p->corr_mode > 4)
    return fail(h, TP_ERR_ARG, "tp_set_texture_params: corr_mode out of range");
  h->tex_params = *p;
  return TP_OK;
}

tp_status tp_textures(tp_handle *h, void *stream) {
  if (!h) return TP_ERR_ARG;
  if (h->cfg.num_sensors != 4 || h->cfg.num_colors != 3)
    return fail(h, TP_ERR_ARG, "tp_textures: texture tiles need 4 sensors x 3 colours");
  if (!h->have_corr) return fail(h, TP_ERR_STATE, "tp_textures: correlation set-up (LPF, colour weights) missing");
  if (clt_filtered(h)) return fail(h, TP_ERR_STATE, "tp_textures: the stored CLT is low-pass filtered (tp_set_clt_lpf_mask)");
  cudaStream_t st = pick_stream(h, stream);
  tp_status r = ensure_plan(h, st);
  if (r != TP_OK) return r;
  const tp_texture_params &p = h->tex_params;
  const int rows = p.keep_weights ? 12 : 4;
  if (rows > h->tex_rows_alloc) {
    dfree(h, h->d_tex);
    h->d_tex = nullptr;
    h->tex_rows_alloc = 0;
    if (dalloc(h, &h->d_tex, (size_t)h->ntiles * rows * 256) != cudaSuccess) {
      cudaGetLastError();
      return fail(h, TP_ERR_NOMEM, "tp_textures: texture buffer");
    }
    h->tex_rows_alloc = rows;
  }
  if (p.aux && !h->d_tex_aux && dalloc(h, &h->d_tex_aux, (size_t)h->ntiles * 16) != cudaSuccess) {
    cudaGetLastError();
    return fail(h, TP_ERR_NOMEM, "tp_textures: aux buffer");
  }
  TexConst tc;
  memset(&tc, 0, sizeof(tc));
  for (int i = 0; i < 64; i++) tc.lpf[i] = h->corr_host.lpf[i];
  for (int i = 0; i < 3; i++) tc.col_weights[i] = h->corr_host.col_weights[i];
  tc.min_shot = p.min_shot;
  tc.scale_shot = p.scale_shot;
  tc.rsqrt_min_shot = p.min_shot > 0.f ? (float)(1.0 / std::sqrt((double)p.min_shot)) : 0.f;
  tc.diff_sigma = p.diff_sigma;
  tc.corr_magic_scale = p.corr_magic_scale;
  tc.dust_remove = p.dust_remove;
  tc.rows = rows;
  // corr_mode -> disparity slot (ImageDtt.java:2422-2426): INT, CM, HOR, VERT from the disparity
  // record; POLY is the LMA disparity of tp_lma_refine on the current forward (none without it,
  // as a NaN POLY gives no shift in the reference)
  static const int slot[5] = {0, 1, -1, 3, 5};
  tc.extra_src = h->d_disp;
  tc.extra_stride = TP_NDISP;
  tc.extra_index = (p.corr_mode >= 0) ? slot[p.corr_mode] : -1;
  if (p.corr_mode == 2 && h->lma_valid && h->d_lma) {
    tc.extra_src = h->d_lma;
    tc.extra_stride = 4;
    tc.extra_index = 0;
  }
  if (tc.extra_index >= 0 && h->num_pairs == 0) tc.extra_index = -1;
  CK(launch_textures(scene_of(h), tc, st), "textures");
  h->tex_rows = rows;
  return mark_work(h, st);
}

tp_status tp_process(tp_handle *h, void *stream) {
  if (!h) return TP_ERR_ARG;
  // the plan (ports, window corners) is recomputed only when geometry, kernels or tasks changed
  cudaStream_t st = pick_stream(h, stream);
  tp_status r = ensure_plan(h, st);
  if (r != TP_OK) return r;
  if (h->num_pairs == 0) return tp_convert_correct(h, stream);
  const SceneDev sc = scene_of(h);
  CK(launch_fused_forward(sc, h->corr_host, h->sched_tpb, h->sched_nw, st), "fused forward");
  h->fwd_valid = 1;
  h->images_since_fwd = 0;
  h->strips_valid = sc.strips ? 1 : 0;
  h->disp_mixed = 0;
  h->lma_valid = 0;
  return mark_work(h, st);
}

tp_status tp_set_schedule(tp_handle *h, int tiles_per_block, int warps_per_block) {
  if (!h) return TP_ERR_ARG;
  // warp per tile: tiles per CTA == warps per CTA (<= 4); pair per warp: 1 tile per CTA of 2, 3 or 4 warps
  if (warps_per_block < 0 || warps_per_block > 4 || tiles_per_block < 0 || tiles_per_block > 4)
    return fail(h, TP_ERR_ARG, "tp_set_schedule: out of range");
  if (warps_per_block == 0) warps_per_block = tiles_per_block;
  if (tiles_per_block > 1 && tiles_per_block != warps_per_block)
    return fail(h, TP_ERR_ARG, "tp_set_schedule: several tiles per CTA need one warp per tile");

  h->sched_tpb = tiles_per_block;
  h->sched_nw = warps_per_block;
  return TP_OK;
}

tp_status tp_synchronize(tp_handle *h) {
  if (!h) return TP_ERR_ARG;
  CK(cudaEventSynchronize(h->ev_work), "tp_synchronize");
  CK(cudaStreamSynchronize(h->stream), "tp_synchronize");
  return TP_OK;
}

tp_status tp_get_num_tasks(const tp_handle *h, int *n) {
  if (!h || !n) return TP_ERR_ARG;
  *n = h->num_tasks;
  return TP_OK;
}

// Host copy of a device result: on the handle's own stream, after the last work enqueued through
// the handle (on whatever stream that went), then that stream alone is synchronised.
static tp_status d2h(tp_handle *h, void *dst, const void *src, size_t bytes, const char *where) {
  if (!dst) return fail(h, TP_ERR_ARG, where);
  if (!src) return fail(h, TP_ERR_STATE, std::string(where) + ": not computed");
  CK(cudaStreamWaitEvent(h->stream, h->ev_work, 0), where);
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream), where);
  CK(cudaStreamSynchronize(h->stream), where);
  return TP_OK;
}

// as d2h, enqueued on st after the handle's last work, without waiting
static tp_status d2h_async(tp_handle *h, void *dst, const void *src, size_t bytes, cudaStream_t st, const char *where) {
  if (!dst) return fail(h, TP_ERR_ARG, where);
  if (!src) return fail(h, TP_ERR_STATE, std::string(where) + ": not computed");
  CK(cudaStreamWaitEvent(st, h->ev_work, 0), where);
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st), where);
  return TP_OK;
}

tp_status tp_get_ports(tp_handle *h, double *ports) {
  if (!h) return TP_ERR_ARG;
  return d2h(h, ports, h->d_ports, (size_t)h->num_tasks * h->cfg.num_sensors * 2 * sizeof(double), "tp_get_ports");
}

tp_status tp_get_task_tiles(tp_handle *h, int *txy) {
  if (!h) return TP_ERR_ARG;
  return d2h(h, txy, h->d_task_txy, (size_t)h->num_tasks * sizeof(int), "tp_get_task_tiles");
}

tp_status tp_get_subtiles(tp_handle *h, int *int_tl, float *residual) {
  if (!h || !int_tl || !residual) return TP_ERR_ARG;
  size_t n = (size_t)h->num_tasks * h->cfg.num_sensors * h->cfg.num_colors;
  std::vector<SubtilePlan> p(n);
  tp_status r = d2h(h, p.data(), h->d_plan, n * sizeof(SubtilePlan), "tp_get_subtiles");
  if (r != TP_OK) return r;
  for (size_t i = 0; i < n; i++) {
    int_tl[2 * i] = p[i].tlx;
    int_tl[2 * i + 1] = p[i].tly;
    residual[2 * i] = p[i].rx;
    residual[2 * i + 1] = p[i].ry;
  }
  return TP_OK;
}

tp_status tp_get_clt(tp_handle *h, float *clt) {
  if (!h) return TP_ERR_ARG;
  return d2h(h, clt, h->d_clt, (size_t)h->ntiles * h->cfg.num_sensors * h->cfg.num_colors * TP_CLT * sizeof(float),
             "tp_get_clt");
}

tp_status tp_get_corr(tp_handle *h, float *corr) {
  if (!h) return TP_ERR_ARG;
  return d2h(h, corr, h->d_corr, (size_t)h->ntiles * h->num_pairs * TP_CORR * sizeof(float), "tp_get_corr");
}

tp_status tp_get_disparity(tp_handle *h, float *disp) {
  if (!h) return TP_ERR_ARG;
  return d2h(h, disp, h->d_disp, (size_t)h->ntiles * TP_NDISP * sizeof(float), "tp_get_disparity");
}

tp_status tp_get_rbg(tp_handle *h, int cam, float *rbg) {
  if (!h) return TP_ERR_ARG;
  if (cam < 0 || cam >= h->cfg.num_sensors) return fail(h, TP_ERR_ARG, "tp_get_rbg: bad camera");
  size_t plane = (size_t)(h->cfg.width + 8) * (h->cfg.height + 8) * h->cfg.num_colors;
  return d2h(h, rbg, h->d_rbg ? h->d_rbg + plane * cam : nullptr, plane * sizeof(float), "tp_get_rbg");
}

tp_status tp_get_rbg_async(tp_handle *h, int cam, float *rbg, void *stream) {
  if (!h) return TP_ERR_ARG;
  if (cam < 0 || cam >= h->cfg.num_sensors) return fail(h, TP_ERR_ARG, "tp_get_rbg_async: bad camera");
  size_t plane = (size_t)(h->cfg.width + 8) * (h->cfg.height + 8) * h->cfg.num_colors;
  return d2h_async(h, rbg, h->d_rbg ? h->d_rbg + plane * cam : nullptr, plane * sizeof(float),
                   pick_stream(h, stream), "tp_get_rbg_async");
}

tp_status tp_get_disparity_async(tp_handle *h, float *disp, void *stream) {
  if (!h) return TP_ERR_ARG;
  return d2h_async(h, disp, h->d_disp, (size_t)h->ntiles * TP_NDISP * sizeof(float), pick_stream(h, stream),
                   "tp_get_disparity_async");
}

tp_status tp_get_textures(tp_handle *h, float *tex) {
  if (!h) return TP_ERR_ARG;
  const int rows = h->tex_rows;
  return d2h(h, tex, rows ? h->d_tex : nullptr, (size_t)h->ntiles * rows * 256 * sizeof(float), "tp_get_textures");
}

tp_status tp_get_texture_aux(tp_handle *h, float *aux) {
  if (!h) return TP_ERR_ARG;
  return d2h(h, aux, h->d_tex_aux, (size_t)h->ntiles * 16 * sizeof(float), "tp_get_texture_aux");
}

// ---------------------------------------------------------------------------
// batches: many scenes (handles) through one persistent forward launch
// ---------------------------------------------------------------------------
struct tp_batch {
  std::vector<tp_handle *> scenes;
  std::vector<SceneDev> h_scenes;           // all scenes, for the batched plan
  std::vector<int> h_task_off;
  std::vector<SceneDev> h_cls[3];           // per schedule class: scenes sharing the persistent queue
  std::vector<int> h_cls_off[3];
  std::vector<tp_handle *> solo[3];         // scenes large enough to keep their own launch
  int cls_units[3] = {0, 0, 0};
  SceneDev *d_scenes = nullptr, *d_cls[3] = {nullptr, nullptr, nullptr};
  int *d_task_off = nullptr, *d_cls_off[3] = {nullptr, nullptr, nullptr};
  int device = 0, total_tasks = 0;
  cudaStream_t stream = nullptr, cls_stream[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev_fork = nullptr, ev_join[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev_done = nullptr;  // after the last enqueued step: the scene tables it reads may then be rewritten
  std::vector<unsigned char> up_tables;  // bytes of the scene tables on the device
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<std::vector<unsigned char>> graph_keys;  // scene_key of every scene when the graph was captured
  std::string err;
};

// Everything about a scene that a captured batch step holds by value: the SceneDev (device
// pointers, task count, dtypes, colour scales, pair count, strip rows), the correlation set-up the
// solo launches take as a kernel parameter, and the schedule.  Both structs are zero-filled
// before their fields are set (scene_of, tp_set_corr), so their bytes compare exactly.
static std::vector<unsigned char> scene_key(tp_handle *h) {
  SceneDev sc = scene_of(h);
  sc.strips = nullptr;  // batched forwards do not record strip samples
  const int sched[2] = {h->sched_tpb, h->sched_nw};
  std::vector<unsigned char> k(sizeof(SceneDev) + sizeof(CorrConst) + sizeof(sched));
  memcpy(k.data(), &sc, sizeof(SceneDev));
  memcpy(k.data() + sizeof(SceneDev), static_cast<const CorrConst *>(&h->corr_host), sizeof(CorrConst));
  memcpy(k.data() + sizeof(SceneDev) + sizeof(CorrConst), sched, sizeof(sched));
  return k;
}

static tp_status bfail(tp_batch *b, tp_status st, const std::string &msg) {
  if (b) b->err = msg;
  return st;
}

// refresh the device scene tables (buffers or task counts may have changed)
static tp_status batch_tables(tp_batch *b) {
  const int n = (int)b->scenes.size();
  b->h_scenes.resize(n);
  b->h_task_off.resize(n + 1);
  for (int c = 0; c < 3; c++) {
    b->h_cls[c].clear();
    b->h_cls_off[c].assign(1, 0);
  }
  for (int c = 0; c < 3; c++) b->solo[c].clear();
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  int t = 0;
  for (int i = 0; i < n; i++) {
    SceneDev sc = scene_of(b->scenes[i]);
    sc.strips = nullptr;  // batched forwards do not record strip samples
    b->h_scenes[i] = sc;
    b->h_task_off[i] = t;
    t += sc.num_tasks;
    const int c = batch_class(sc);
    // a warp-per-tile scene with at least 8 waves of tiles (16 warps per SM) has no tail
    // worth sharing: it keeps its own launch, captured in the same graph
    if (c != 2 && sc.num_tasks >= 8 * 16 * sms) {
      b->solo[c].push_back(b->scenes[i]);
      continue;
    }
    b->h_cls[c].push_back(sc);
    b->h_cls_off[c].push_back(b->h_cls_off[c].back() + batch_units(sc));
  }
  b->h_task_off[n] = t;
  b->total_tasks = t;
  for (int c = 0; c < 3; c++) b->cls_units[c] = b->h_cls_off[c].back();
  // upload only when a table changed, after the last step that read the old ones has finished
  std::vector<unsigned char> tb;
  auto put = [&tb](const void *p, size_t n) { tb.insert(tb.end(), (const unsigned char *)p, (const unsigned char *)p + n); };
  put(b->h_scenes.data(), n * sizeof(SceneDev));
  put(b->h_task_off.data(), (n + 1) * sizeof(int));
  for (int c = 0; c < 3; c++) {
    const int m = (int)b->h_cls[c].size();
    put(&m, sizeof(m));
    put(b->h_cls[c].data(), m * sizeof(SceneDev));
    put(b->h_cls_off[c].data(), (m + 1) * sizeof(int));
  }
  if (tb == b->up_tables) return TP_OK;
  if (cudaEventSynchronize(b->ev_done) != cudaSuccess) {
    cudaGetLastError();
    return bfail(b, TP_ERR_CUDA, "batch: waiting for the previous step");
  }
  bool ok = cudaMemcpy(b->d_scenes, b->h_scenes.data(), n * sizeof(SceneDev), cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(b->d_task_off, b->h_task_off.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice) ==
                cudaSuccess;
  for (int c = 0; ok && c < 3; c++) {
    const int m = (int)b->h_cls[c].size();
    if (m == 0) continue;
    ok = cudaMemcpy(b->d_cls[c], b->h_cls[c].data(), m * sizeof(SceneDev), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(b->d_cls_off[c], b->h_cls_off[c].data(), (m + 1) * sizeof(int), cudaMemcpyHostToDevice) ==
             cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    b->up_tables.clear();
    return bfail(b, TP_ERR_CUDA, "batch: scene table upload");
  }
  b->up_tables.swap(tb);
  return TP_OK;
}

// the plans (all scenes in one launch) and one persistent forward per class on its own
// stream, forked from and joined back into st
static tp_status batch_enqueue(tp_batch *b, int replan, cudaStream_t st) {
  bool need = replan != 0;
  for (tp_handle *h : b->scenes) need = need || !h->planned;
  if (need) {
    for (size_t i = 0; i < b->scenes.size(); i++) {
      const SceneDev &sc = b->h_scenes[i];
      if (cudaMemsetAsync(sc.tile_task, 0xff, sizeof(int) * sc.tilesX * sc.tilesY, st) != cudaSuccess) {
        cudaGetLastError();
        return bfail(b, TP_ERR_CUDA, "batch: tile map");
      }
    }
    if (launch_plan_batch(b->d_scenes, b->d_task_off, (int)b->scenes.size(), b->total_tasks, st) != cudaSuccess) {
      cudaGetLastError();
      return bfail(b, TP_ERR_CUDA, "batch: plan");
    }
    for (tp_handle *h : b->scenes) h->planned = 1;
  }
  if (cudaEventRecord(b->ev_fork, st) != cudaSuccess) return bfail(b, TP_ERR_CUDA, "batch: fork");
  for (int c = 0; c < 3; c++) {
    const int m = (int)b->h_cls[c].size();
    if (m == 0 && b->solo[c].empty()) continue;
    cudaStream_t cs = b->cls_stream[c];
    bool ok = cudaStreamWaitEvent(cs, b->ev_fork, 0) == cudaSuccess;
    for (tp_handle *h : b->solo[c]) {
      SceneDev ss = scene_of(h);
      ss.strips = nullptr;
      ok = ok && launch_fused_forward(ss, h->corr_host, h->sched_tpb, h->sched_nw, cs) == cudaSuccess;
    }
    if (m > 0)
      ok = ok && launch_fused_batch(c, b->h_cls[c].data(), b->d_cls[c], b->d_cls_off[c], m, b->cls_units[c], cs) ==
                     cudaSuccess;
    ok = ok && cudaEventRecord(b->ev_join[c], cs) == cudaSuccess && cudaStreamWaitEvent(st, b->ev_join[c], 0) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      return bfail(b, TP_ERR_CUDA, "batch: forward");
    }
  }
  for (tp_handle *h : b->scenes) {
    h->fwd_valid = 1;
    h->images_since_fwd = 0;
    h->strips_valid = 0;
    h->disp_mixed = 0;
    h->lma_valid = 0;
  }
  return TP_OK;
}

#define CK_B(call)                                                                       \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return bfail(b, TP_ERR_CUDA, std::string("batch: ") + cudaGetErrorString(e_)); \
  } while (0)

static void batch_drop_graph(tp_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

// the DTT tables this translation unit's kernels read are uploaded once per device
static std::mutex g_dtt_mu;
static bool g_dtt_ready[64];

tp_status tp_dtt8x8(float *dst, const float *src, int src_stride, int width, int height, int dtt_mode,
                    void *stream) {
  if (!dst || !src || width <= 0 || height <= 0 || (width & 7) || (height & 7) || src_stride < width ||
      dtt_mode < 0 || dtt_mode > 7)
    return TP_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return TP_ERR_CUDA;
  }
  if (dev < 0 || dev >= 64) return TP_ERR_ARG;
  {
    std::lock_guard<std::mutex> lock(g_dtt_mu);
    if (!g_dtt_ready[dev]) {
      if (upload_fused_constants() != cudaSuccess) {
        cudaGetLastError();
        return TP_ERR_CUDA;
      }
      g_dtt_ready[dev] = true;
    }
  }
  if (launch_dtt8x8(dst, src, src_stride, width, height, dtt_mode, (cudaStream_t)stream) != cudaSuccess) {
    cudaGetLastError();
    return TP_ERR_CUDA;
  }
  return TP_OK;
}

// Device address of the compaction scratch array per device (cudaGetSymbolAddress with that
// device current).  A call outside a stream capture looks it up again, so a device reset that
// reloaded the module is followed; a call inside a capture uses the address of the last call
// outside one.
static std::mutex g_scratch_mu;
static int *g_scratch_ptr[TP_NOALLOC_MAX_DEVICES];

tp_status tp_compact_tile_ops_noalloc(const int *tile_op, const float *disparity, int tilesX, int num_tiles,
                                      int *task_txy, int *task_op, float *task_disp, int *num_tasks,
                                      void *stream) {
  if (!tile_op || !task_txy || !task_op || !task_disp || !num_tasks || tilesX <= 0 || tilesX > 65535 ||
      num_tiles < 0 || num_tiles / tilesX > 32767)
    return TP_ERR_ARG;
  if (num_tiles > compact_scratch_max_tiles()) return TP_ERR_SCRATCH_LIMIT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TP_ERR_CUDA;
  if (dev < 0 || dev >= TP_NOALLOC_MAX_DEVICES) return TP_ERR_ARG;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing((cudaStream_t)stream, &cap) != cudaSuccess) {
    cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;  // unknown: do not call the symbol lookup
  }
  int *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (cap == cudaStreamCaptureStatusNone || !g_scratch_ptr[dev]) {
      if (cap != cudaStreamCaptureStatusNone) return TP_ERR_STATE;  // first call on a device inside a capture
      int *p = nullptr;
      if (compact_scratch_address(&p) != cudaSuccess || !p) {
        cudaGetLastError();
        return TP_ERR_CUDA;
      }
      g_scratch_ptr[dev] = p;
    }
    scratch = g_scratch_ptr[dev];
  }
  if (launch_compact_tasks_scratch(tile_op, disparity, tilesX, num_tiles, task_txy, task_op, task_disp, num_tasks,
                                   scratch, (cudaStream_t)stream) != cudaSuccess) {
    cudaGetLastError();
    return TP_ERR_CUDA;
  }
  return TP_OK;
}

tp_status tp_default_lma_params(tp_lma_params *p) {
  if (!p) return TP_ERR_ARG;
  // ImageDttParameters.java:32-109
  p->min_poly_strength = 0.2f;
  p->mix_corr_poly = 1;
  p->ortho_vasw_pwr = 2.0f;
  p->cnvx_hwnd_size = 4;
  p->cnvx_weight = 0.5f;
  p->cnvx_add3x3 = 1;
  p->adjust_wm = 1;
  p->adjust_wy = 0;
  p->adjust_wxy = 1;
  p->adjust_ag = 1;
  p->half_width = 2.0f;
  p->cost_wy = 0.1f;
  p->cost_wxy = 0.1f;
  p->lambda_initial = 0.1f;
  p->lambda_scale_good = 0.5f;
  p->lambda_scale_bad = 8.0f;
  p->lambda_max = 100.0f;
  p->rms_diff = 0.001f;
  p->num_iter = 20;
  p->pair_mask = 0x3f;
  p->fo_correct = 1;
  p->fo_far = 0;
  p->fo_ortho = 1;
  p->fo_min_strength = 0.1f;
  p->fo_min_eff = 0.25f;
  p->fo_min_eff_ratio = 0.65f;
  p->fo_max_hwidth = 3.0f;
  p->fo_min_diff = 0.2f;
  p->fo_overcorrection = 0.0f;
  p->fo_lim_overcorr = 2.0f;
  p->mismatch = 0;
  p->max_corr_radius = 3.9f;
  p->mismatch_max_diff = 1.0f;
  p->ly_poly = 0;
  p->ly_crazy_poly = 1.0f;
  p->ly_poly_backup = 1;
  return TP_OK;
}

// the device copy of the LMA settings
static TpLmaConst lma_const_of(const tp_lma_params &prm) {
  TpLmaConst c;
  c.min_poly_strength = prm.min_poly_strength;
  c.mix_corr_poly = prm.mix_corr_poly;
  c.ortho_vasw_pwr = prm.ortho_vasw_pwr;
  c.cnvx_hwnd_size = prm.cnvx_hwnd_size;
  c.cnvx_weight = prm.cnvx_weight;
  c.cnvx_add3x3 = prm.cnvx_add3x3;
  c.adjust_wm = prm.adjust_wm;
  c.adjust_wy = prm.adjust_wy;
  c.adjust_wxy = prm.adjust_wxy;
  c.adjust_ag = prm.adjust_ag;
  c.half_width = prm.half_width;
  c.cost_wy = prm.cost_wy;
  c.cost_wxy = prm.cost_wxy;
  c.lambda_initial = prm.lambda_initial;
  c.lambda_scale_good = prm.lambda_scale_good;
  c.lambda_scale_bad = prm.lambda_scale_bad;
  c.lambda_max = prm.lambda_max;
  c.rms_diff = prm.rms_diff;
  c.num_iter = prm.num_iter;
  c.pair_mask = prm.pair_mask;
  c.fo_correct = prm.fo_correct;
  c.fo_far = prm.fo_far;
  c.fo_ortho = prm.fo_ortho;
  c.fo_min_strength = prm.fo_min_strength;
  c.fo_min_eff = prm.fo_min_eff;
  c.fo_min_eff_ratio = prm.fo_min_eff_ratio;
  c.fo_max_hwidth = prm.fo_max_hwidth;
  c.fo_min_diff = prm.fo_min_diff;
  c.fo_overcorrection = prm.fo_overcorrection;
  c.fo_lim_overcorr = prm.fo_lim_overcorr;
  c.mismatch = prm.mismatch;
  c.max_corr_radius = prm.max_corr_radius;
  c.mismatch_max_diff = prm.mismatch_max_diff;
  c.ly_poly = prm.ly_poly;
  c.ly_poly_backup = prm.ly_poly_backup;
  c.ly_crazy_poly = prm.ly_crazy_poly;
  return c;
}

tp_status tp_lma_refine(tp_handle *h, const tp_lma_params *p, void *stream) {
  if (!h) return TP_ERR_ARG;
  tp_lma_params prm;
  if (p) prm = *p;
  else tp_default_lma_params(&prm);
  if (prm.cnvx_hwnd_size < 0 || prm.cnvx_hwnd_size > 4 || prm.num_iter < 0)
    return fail(h, TP_ERR_ARG, "tp_lma_refine: cnvx_hwnd_size must be 0..4");
  if (!h->have_corr || h->num_pairs == 0) return fail(h, TP_ERR_STATE, "tp_lma_refine: no correlation pairs");
  if (!h->fwd_valid) return fail(h, TP_ERR_STATE, "tp_lma_refine: run tp_process first");
  if (h->disp_mixed)
    return fail(h, TP_ERR_STATE, "tp_lma_refine: the disparity record already holds the LMA result; run tp_process");
  bool quad = false;
  for (int i = 0; i < h->num_pairs; i++) {
    const int k = h->corr_host.pairs[i].kind;
    if (k >= 0 && k <= 3 && i < 32 && ((prm.pair_mask >> i) & 1)) quad = true;
  }
  if (!quad) return fail(h, TP_ERR_ARG, "tp_lma_refine: needs pairs of the quad kinds 0..3");
  cudaStream_t st = pick_stream(h, stream);
  if (!h->d_lma) {
    if (dalloc(h, &h->d_lma, (size_t)h->ntiles * 4) != cudaSuccess) {
      cudaGetLastError();
      return fail(h, TP_ERR_NOMEM, "tp_lma_refine: buffer");
    }
  }
  CK(cudaMemsetAsync(h->d_lma, 0xff, (size_t)h->ntiles * 4 * sizeof(float), st), "tp_lma_refine");  // NaN
  const TpLmaConst c = lma_const_of(prm);
  if (prm.mismatch) {
    const size_t need = (size_t)h->ntiles * h->num_pairs * 3;
    if (need > h->mismatch_cap) {
      dfree(h, h->d_mismatch);
      h->d_mismatch = nullptr;
      h->mismatch_cap = 0;
      if (dalloc(h, &h->d_mismatch, need) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, TP_ERR_NOMEM, "tp_lma_refine: mismatch buffer");
      }
      h->mismatch_cap = need;
    }
    h->mismatch_pairs = h->num_pairs;
  }
  CK(launch_lma(scene_of(h), h->corr_host, c, h->d_lma, prm.mismatch ? h->d_mismatch : nullptr, st),
     "tp_lma_refine");
  if (prm.mix_corr_poly || prm.fo_correct) h->disp_mixed = 1;
  h->lma_valid = 1;
  return mark_work(h, st);
}

tp_status tp_get_lma_mismatch(tp_handle *h, float *out) {
  if (!h || !out) return TP_ERR_ARG;
  if (!h->d_mismatch || h->mismatch_pairs != h->num_pairs)
    return fail(h, TP_ERR_STATE, "tp_get_lma_mismatch: run tp_lma_refine with mismatch set first");
  return d2h(h, out, h->d_mismatch, (size_t)h->ntiles * h->num_pairs * 3 * sizeof(float), "tp_get_lma_mismatch");
}

tp_status tp_get_pair_maxima(tp_handle *h, float *out) {
  if (!h || !out) return TP_ERR_ARG;
  if (!h->have_corr || h->num_pairs == 0 || !h->d_corr || !h->fwd_valid)
    return fail(h, TP_ERR_STATE, "tp_get_pair_maxima: run tp_process first");
  const size_t need = (size_t)h->ntiles * h->num_pairs * 3;
  if (need > h->pairmax_cap) {
    if (work_done(h, "tp_get_pair_maxima") != TP_OK) return TP_ERR_CUDA;  // before the free
    dfree(h, h->d_pairmax);
    h->d_pairmax = nullptr;
    h->pairmax_cap = 0;
    if (dalloc(h, &h->d_pairmax, need) != cudaSuccess) {
      cudaGetLastError();
      return fail(h, TP_ERR_NOMEM, "tp_get_pair_maxima: buffer");
    }
    h->pairmax_cap = need;
  }
  CK(cudaStreamWaitEvent(h->stream, h->ev_work, 0), "tp_get_pair_maxima");
  CK(launch_pair_maxima(scene_of(h), h->num_pairs, h->d_pairmax, h->stream), "tp_get_pair_maxima");
  if (mark_work(h, h->stream) != TP_OK) return TP_ERR_CUDA;
  return d2h(h, out, h->d_pairmax, need * sizeof(float), "tp_get_pair_maxima");
}

tp_status tp_get_lma(tp_handle *h, float *out) {
  if (!h || !out) return TP_ERR_ARG;
  if (!h->d_lma) return fail(h, TP_ERR_STATE, "tp_get_lma: run tp_lma_refine first");
  return d2h(h, out, h->d_lma, (size_t)h->ntiles * 4 * sizeof(float), "tp_get_lma");
}

// the main camera's correlation set-up with one horizontal pair: camera 0 = main, 1 = auxiliary
static CorrConst rig_corr_const(const tp_handle *h) {
  CorrConst cc = h->corr_host;
  cc.num_pairs = 1;
  cc.num_combo = 1;
  cc.log_combine = 0;
  cc.num_hor = cc.num_vert = 0;
  cc.pairs[0].cam1 = 0;
  cc.pairs[0].cam2 = 1;
  cc.pairs[0].kind = 0;
  cc.pairs[0].in_combo = 1;
  cc.pairs[0].bx = 1.f;
  cc.pairs[0].by = 0.f;
  return cc;
}

tp_status tp_rig_correlate(tp_handle *main_h, tp_handle *aux, float cm_max_normalization, int no_int_x0,
                           void *stream) {
  tp_handle *h = main_h;
  if (!h || !aux) return TP_ERR_ARG;
  if (aux->tilesX != h->tilesX || aux->tilesY != h->tilesY || aux->cfg.num_colors != h->cfg.num_colors ||
      aux->cfg.device != h->cfg.device)
    return fail(h, TP_ERR_ARG, "tp_rig_correlate: the cameras differ in tile grid, colours or device");
  if (!h->have_corr) return fail(h, TP_ERR_STATE, "tp_rig_correlate: main camera has no correlation set-up");
  if (!h->fwd_valid || !aux->fwd_valid)
    return fail(h, TP_ERR_STATE, "tp_rig_correlate: run tp_process on both cameras first");
  if (clt_filtered(h) || clt_filtered(aux))
    return fail(h, TP_ERR_STATE, "tp_rig_correlate: a stored CLT is low-pass filtered (tp_set_clt_lpf_mask)");
  cudaStream_t st = pick_stream(h, stream);
  if (!h->d_rig_corr) {
    if (dalloc(h, &h->d_rig_corr, (size_t)h->ntiles * TP_CORR) != cudaSuccess ||
        dalloc(h, &h->d_rig_rec, (size_t)h->ntiles * 4) != cudaSuccess) {
      cudaGetLastError();
      return fail(h, TP_ERR_NOMEM, "tp_rig_correlate: buffers");
    }
    CK(cudaMemsetAsync(h->d_rig_corr, 0, (size_t)h->ntiles * TP_CORR * sizeof(float), st), "tp_rig_correlate");
  }
  CK(cudaStreamWaitEvent(st, aux->ev_work, 0), "tp_rig_correlate");  // both cameras' forwards
  CK(cudaStreamWaitEvent(st, h->ev_work, 0), "tp_rig_correlate");
  const CorrConst cc = rig_corr_const(h);
  CK(launch_rig(scene_of(h), scene_of(aux), cc, h->d_rig_corr, h->d_rig_rec, cm_max_normalization, no_int_x0, st),
     "tp_rig_correlate");
  h->rig_lma_done = 0;
  return mark_work(h, st);
}

tp_status tp_rig_lma(tp_handle *main_h, const tp_lma_params *p, int use_poly, int use_xy_poly, void *stream) {
  tp_handle *h = main_h;
  if (!h) return TP_ERR_ARG;
  tp_lma_params prm;
  if (p) prm = *p;
  else tp_default_lma_params(&prm);
  if (prm.cnvx_hwnd_size < 0 || prm.cnvx_hwnd_size > 4 || prm.num_iter < 0)
    return fail(h, TP_ERR_ARG, "tp_rig_lma: cnvx_hwnd_size must be 0..4");
  if (!h->d_rig_corr) return fail(h, TP_ERR_STATE, "tp_rig_lma: run tp_rig_correlate first");
  if (h->rig_lma_done)
    return fail(h, TP_ERR_STATE, "tp_rig_lma: the rig record already holds the LMA result; run tp_rig_correlate");
  cudaStream_t st = pick_stream(h, stream);
  if (!h->d_rig_tmp && dalloc(h, &h->d_rig_tmp, (size_t)h->ntiles * (TP_NDISP + 4)) != cudaSuccess) {
    cudaGetLastError();
    return fail(h, TP_ERR_NOMEM, "tp_rig_lma: buffer");
  }
  CK(cudaStreamWaitEvent(st, h->ev_work, 0), "tp_rig_lma");
  CK(launch_rig_lma(scene_of(h), rig_corr_const(h), lma_const_of(prm), h->d_rig_corr, h->d_rig_rec, h->d_rig_tmp,
                    h->d_rig_tmp + (size_t)h->ntiles * TP_NDISP, use_poly, use_xy_poly, st),
     "tp_rig_lma");
  h->rig_lma_done = 1;
  return mark_work(h, st);
}

tp_status tp_get_rig(tp_handle *h, float *corr, float *rec) {
  if (!h) return TP_ERR_ARG;
  if (!h->d_rig_corr) return fail(h, TP_ERR_STATE, "tp_get_rig: run tp_rig_correlate first");
  tp_status r = TP_OK;
  if (corr) r = d2h(h, corr, h->d_rig_corr, (size_t)h->ntiles * TP_CORR * sizeof(float), "tp_get_rig");
  if (r == TP_OK && rec) r = d2h(h, rec, h->d_rig_rec, (size_t)h->ntiles * 4 * sizeof(float), "tp_get_rig");
  return r;
}

// From the first adjoint on, the forward records every pair's strip samples [tiles][pairs][RE]
// so the adjoint reads them instead of re-interpolating the correlation surfaces.
static tp_status enable_strip_recording(tp_handle *h) {
  const size_t need = strips_need(h);
  if (need > h->strips_cap) {
    dfree(h, h->d_strips);
    h->d_strips = nullptr;
    h->strips_cap = 0;
    h->strips_valid = 0;
    if (dalloc(h, &h->d_strips, need) != cudaSuccess) {
      cudaGetLastError();
      h->adj_record = 0;
      return fail(h, TP_ERR_NOMEM, "adjoint: strip-sample buffer");
    }
    h->strips_cap = need;
  }
  h->adj_record = 1;
  return TP_OK;
}

tp_status tp_set_adjoint_mode(tp_handle *h, int recompute_clt) {
  if (!h) return TP_ERR_ARG;
  h->adj_recompute = recompute_clt ? 1 : 0;
  return enable_strip_recording(h);
}

tp_status tp_backward(tp_handle *h, const float *dl_ddisp, float *dl_dextr, float *dl_dtile_disp, void *stream) {
  if (!h) return TP_ERR_ARG;
  if (!h->ports_from_geometry || !h->have_geometry)
    return fail(h, TP_ERR_STATE, "tp_backward: needs tile ops with ports from the geometry (tp_set_tile_ops)");
  if (h->rig_aux)
    return fail(h, TP_ERR_STATE, "tp_backward: not for a rig's auxiliary camera (its disparities are the main camera's)");
  if (!h->fwd_valid || h->num_pairs == 0)
    return fail(h, TP_ERR_STATE, "tp_backward: run tp_process (with correlation pairs) first");
  if (clt_filtered(h) && !h->adj_recompute)
    return fail(h, TP_ERR_STATE, "tp_backward: the stored CLT is low-pass filtered (tp_set_clt_lpf_mask)");
  if (h->adj_recompute && h->images_since_fwd)
    return fail(h, TP_ERR_STATE, "tp_backward: the CLT recompute reads the images, which changed since tp_process");
  cudaStream_t st = pick_stream(h, stream);
  const size_t nt = h->ntiles, S = h->cfg.num_sensors;
  const int nb = (int)((nt + 256 / S - 1) / (256 / S));  // blocks of the contraction kernel (256 / S tasks each)
  if (!h->d_sens) {
    bool ok = dalloc(h, &h->d_port_deriv, nt * S * 10) == cudaSuccess && dalloc(h, &h->d_sens, nt * S * 2) == cudaSuccess &&
              dalloc(h, &h->d_dval, nt) == cudaSuccess && dalloc(h, &h->d_jac_e, nt * S * 4) == cudaSuccess &&
              dalloc(h, &h->d_jac_d, nt) == cudaSuccess && dalloc(h, &h->d_grad_d, nt) == cudaSuccess &&
              dalloc(h, &h->d_partial, (size_t)nb * S * 4) == cudaSuccess && dalloc(h, &h->d_grad_e, S * 4) == cudaSuccess &&
              dalloc(h, &h->d_dldd, nt) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      return fail(h, TP_ERR_NOMEM, "tp_backward: adjoint buffers");
    }
    CK(cudaMemsetAsync(h->d_grad_d, 0, nt * sizeof(float), st), "tp_backward");
    CK(cudaMemsetAsync(h->d_jac_d, 0, nt * sizeof(float), st), "tp_backward");
  }
  // the FP64 port derivatives of the current plan (same ports, corners and residuals): computed
  // here unless the forward's plan already produced them
  SceneDev sc = scene_of(h);
  sc.port_deriv = h->d_port_deriv;
  const int use_strips = h->strips_valid && sc.strips;
  tp_status rs = enable_strip_recording(h);  // later forwards keep their strip samples and derivatives
  if (rs != TP_OK) return rs;
  if (!h->deriv_valid) CK(launch_plan(sc, st), "tp_backward plan");
  h->deriv_valid = 1;
  if (dl_ddisp) CK(cudaMemcpyAsync(h->d_dldd, dl_ddisp, nt * sizeof(float), cudaMemcpyHostToDevice, st), "tp_backward");
  CK(launch_adjoint(sc, h->corr_host, h->adj_recompute, use_strips, h->d_sens, h->d_dval, dl_ddisp ? h->d_dldd : nullptr,
                    h->d_jac_e, h->d_jac_d, h->d_grad_d, h->d_partial, h->d_grad_e, st),
     "tp_backward adjoint");
  h->have_jac = 1;
  tp_status rm = mark_work(h, st);
  if (rm != TP_OK) return rm;
  if (dl_dextr) CK(cudaMemcpyAsync(dl_dextr, h->d_grad_e, S * 4 * sizeof(float), cudaMemcpyDeviceToHost, st), "tp_backward");
  if (dl_dtile_disp)
    CK(cudaMemcpyAsync(dl_dtile_disp, h->d_grad_d, nt * sizeof(float), cudaMemcpyDeviceToHost, st), "tp_backward");
  if (dl_dextr || dl_dtile_disp) CK(cudaStreamSynchronize(st), "tp_backward");
  return TP_OK;
}

tp_status tp_get_disparity_jacobian(tp_handle *h, float *jac_extr, float *jac_disp, float *disparity) {
  if (!h) return TP_ERR_ARG;
  if (!h->have_jac) return fail(h, TP_ERR_STATE, "tp_get_disparity_jacobian: run tp_backward first");
  const size_t nt = h->ntiles, S = h->cfg.num_sensors;
  tp_status r = TP_OK;
  if (jac_extr) r = d2h(h, jac_extr, h->d_jac_e, nt * S * 4 * sizeof(float), "tp_get_disparity_jacobian");
  if (r == TP_OK && jac_disp) r = d2h(h, jac_disp, h->d_jac_d, nt * sizeof(float), "tp_get_disparity_jacobian");
  if (r == TP_OK && disparity) r = d2h(h, disparity, h->d_dval, nt * sizeof(float), "tp_get_disparity_jacobian");
  return r;
}

tp_status tp_get_port_sensitivities(tp_handle *h, float *sens) {
  if (!h) return TP_ERR_ARG;
  if (!h->have_jac) return fail(h, TP_ERR_STATE, "tp_get_port_sensitivities: run tp_backward first");
  return d2h(h, sens, h->d_sens, (size_t)h->ntiles * h->cfg.num_sensors * 2 * sizeof(float),
             "tp_get_port_sensitivities");
}

tp_status tp_get_port_derivatives(tp_handle *h, double *deriv) {
  if (!h) return TP_ERR_ARG;
  if (!h->have_jac) return fail(h, TP_ERR_STATE, "tp_get_port_derivatives: run tp_backward first");
  return d2h(h, deriv, h->d_port_deriv, (size_t)h->num_tasks * h->cfg.num_sensors * 10 * sizeof(double),
             "tp_get_port_derivatives");
}

tp_status tp_batch_create(tp_handle *const *scenes, int n, tp_batch **out) {
  if (!scenes || !out || n <= 0 || n > 256) return TP_ERR_ARG;
  *out = nullptr;
  const int dev = scenes[0] ? scenes[0]->cfg.device : 0;
  for (int i = 0; i < n; i++) {
    tp_handle *h = scenes[i];
    if (!h || h->cfg.device != dev) return TP_ERR_ARG;
    if (!h->have_tasks || !h->have_corr || h->num_pairs == 0) return TP_ERR_STATE;
    const bool split = h->cfg.num_colors == 1 && h->num_pairs > 8;
    if (!split && h->cfg.num_sensors * h->cfg.num_colors > 16) return TP_ERR_ARG;  // warp-per-tile smem
    if (h->cfg.num_colors == 3 && h->num_pairs > 8) return TP_ERR_ARG;
  }
  tp_batch *b = new tp_batch();
  b->scenes.assign(scenes, scenes + n);
  b->device = dev;
  bool ok = cudaSetDevice(dev) == cudaSuccess &&
            cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming) == cudaSuccess &&
            dalloc_batch(&b->d_scenes, n) == cudaSuccess && dalloc_batch(&b->d_task_off, n + 1) == cudaSuccess;
  for (int c = 0; ok && c < 3; c++)
    ok = cudaStreamCreateWithFlags(&b->cls_stream[c], cudaStreamNonBlocking) == cudaSuccess &&
         cudaEventCreateWithFlags(&b->ev_join[c], cudaEventDisableTiming) == cudaSuccess &&
         dalloc_batch(&b->d_cls[c], n) == cudaSuccess && dalloc_batch(&b->d_cls_off[c], n + 1) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    tp_batch_destroy(b);
    return TP_ERR_NOMEM;
  }
  *out = b;
  return TP_OK;
}

tp_status tp_batch_destroy(tp_batch *b) {
  if (!b) return TP_ERR_ARG;
  batch_drop_graph(b);
  cudaFree(b->d_scenes);
  cudaFree(b->d_task_off);
  for (int c = 0; c < 3; c++) {
    cudaFree(b->d_cls[c]);
    cudaFree(b->d_cls_off[c]);
    if (b->cls_stream[c]) cudaStreamDestroy(b->cls_stream[c]);
    if (b->ev_join[c]) cudaEventDestroy(b->ev_join[c]);
  }
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev_done) cudaEventDestroy(b->ev_done);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return TP_OK;
}

tp_status tp_batch_last_error(const tp_batch *b, char *buf, int n) {
  if (!b || !buf || n <= 0) return TP_ERR_ARG;
  snprintf(buf, (size_t)n, "%s", b->err.c_str());
  return TP_OK;
}

tp_status tp_batch_process(tp_batch *b, int replan, void *stream) {
  if (!b) return TP_ERR_ARG;
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  for (tp_handle *h : b->scenes) {
    CK_B(cudaStreamSynchronize(h->stream));       // set-up copies on the handles' own streams
    CK_B(cudaStreamWaitEvent(st, h->ev_work, 0));  // each scene's earlier work, on any stream
  }
  tp_status r = batch_tables(b);
  if (r != TP_OK) return r;
  r = batch_enqueue(b, replan, st);
  if (r == TP_OK) CK_B(cudaEventRecord(b->ev_done, st));
  for (tp_handle *h : b->scenes)
    if (r == TP_OK && mark_work(h, st) != TP_OK) r = bfail(b, TP_ERR_CUDA, "batch: " + h->err);
  return r;
}

tp_status tp_batch_run_graph(tp_batch *b, void *stream) {
  if (!b) return TP_ERR_ARG;
  cudaStream_t st = stream ? (cudaStream_t)stream : b->stream;
  bool stale = !b->exec || b->graph_keys.size() != b->scenes.size();
  for (size_t i = 0; !stale && i < b->scenes.size(); i++) stale = b->graph_keys[i] != scene_key(b->scenes[i]);
  if (stale) {
    batch_drop_graph(b);
    for (tp_handle *h : b->scenes) {
      CK_B(cudaStreamSynchronize(h->stream));
      CK_B(cudaEventSynchronize(h->ev_work));
    }
    tp_status r = batch_tables(b);
    if (r != TP_OK) return r;
    CK_B(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed));
    r = batch_enqueue(b, 1, b->stream);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
    if (r != TP_OK) {
      if (g) cudaGraphDestroy(g);
      return r;
    }
    if (ec != cudaSuccess) return bfail(b, TP_ERR_CUDA, std::string("batch: capture: ") + cudaGetErrorString(ec));
    b->graph = g;
    CK_B(cudaGraphInstantiate(&b->exec, b->graph, 0));
    b->graph_keys.clear();
    for (tp_handle *h : b->scenes) b->graph_keys.push_back(scene_key(h));
  }
  for (tp_handle *h : b->scenes) CK_B(cudaStreamWaitEvent(st, h->ev_work, 0));
  CK_B(cudaGraphLaunch(b->exec, st));
  CK_B(cudaEventRecord(b->ev_done, st));
  for (tp_handle *h : b->scenes)
    if (mark_work(h, st) != TP_OK) return bfail(b, TP_ERR_CUDA, "batch: " + h->err);
  for (tp_handle *h : b->scenes) {
    h->fwd_valid = 1;
    h->images_since_fwd = 0;
    h->strips_valid = 0;
    h->disp_mixed = 0;
    h->lma_valid = 0;
  }
  return TP_OK;
}

tp_status tp_batch_synchronize(tp_batch *b) {
  if (!b) return TP_ERR_ARG;
  CK_B(cudaStreamSynchronize(b->stream));
  return TP_OK;
}

}  // extern "C"
