// tp_plan.cu -- stage 1 (port coordinates) and per-sub-tile window planning, FP64.
//
// Tile selection (integer window corner, kernel tile) must match the FP64
// reference bit for bit, so this translation unit evaluates the geometry in
// double precision with explicitly rounded operations (__dadd_rn etc. are never
// contracted into FMAs) in the operation order of
// GeometryCorrection.getPortsCoordinatesAndDerivatives and
// ImageDtt.extract_correct_tile.  GB300 FP64 throughput is low, so this runs
// as its own kernel with one thread per (task, sensor): ~100 FP64 operations
// per port instead of the FP32 pipeline paying for them per coefficient.
#include "tp.h"
#include "tp_internal.h"
#include <math_constants.h>

#define DADD(a, b) __dadd_rn((a), (b))
#define DSUB(a, b) __dsub_rn((a), (b))
#define DMUL(a, b) __dmul_rn((a), (b))
#define DDIV(a, b) __ddiv_rn((a), (b))
#define DSQRT(a) __dsqrt_rn(a)

// java.lang.Math.round(double), exact round-half-up
__device__ __forceinline__ double java_round(double x) {
  double f = floor(x);
  return (DSUB(x, f) >= 0.5) ? DADD(f, 1.0) : f;
}

// Window corner (an integral double) -> int.  A corner further than TP_PORT_MARGIN outside the
// image is moved to the margin keeping its parity: every pixel of such a window is outside the
// image, and the mirrored edge pixels it reads (Win::at, mirror) depend only on the corner's
// parity, so the window content is unchanged and the int arithmetic of the kernels that read it
// cannot overflow.  NaN (a port beyond the reverse distortion table) goes to the lower bound.
__device__ __forceinline__ int clamp_corner(double t, int n) {
  const double lo = -(double)(TP_PORT_MARGIN + 16), hi = (double)(n + TP_PORT_MARGIN);
  if (t >= lo && t <= hi) return (int)t;
  const int par = (t == t) ? (int)fabs(fmod(t, 2.0)) : 0;
  return (t > hi) ? (int)hi - (((int)hi & 1) ^ par) : (int)lo + (((int)lo & 1) ^ par);
}

// GeometryCorrection.getRByRDist (GeometryCorrection.java:2802-2827)
__device__ double r_by_rdist(const double *tbl, int len, double rDist) {
  if (rDist < 0) return CUDART_NAN;
  double q = DDIV(rDist, 0.001);
  int index = (int)floor(q);
  if (index >= len - 1) return CUDART_NAN;
  return DADD(tbl[index], DMUL(DSUB(tbl[index + 1], tbl[index]), DSUB(q, (double)index)));
}

__device__ __forceinline__ void mat3_vec(const double m[3][3], const double v[3], double r[3]) {
#pragma unroll
  for (int i = 0; i < 3; i++) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++) s = DADD(s, DMUL(m[i][k], v[k]));
    r[i] = s;
  }
}

// undistorted tile centre, the sensor-independent head of getPortsCoordinatesAndDerivatives, with
// the centre model (gc_main, 2179-2185)
__device__ __forceinline__ void center_undistort(const GeomDev &g, const double *tbl, double px, double py,
                                                 double &pXc, double &pYc) {
  const double pXcd = DSUB(px, DMUL(0.5, (double)g.c_pixel_width));
  const double pYcd = DSUB(py, DMUL(0.5, (double)g.c_pixel_height));
  const double rD = DMUL(DMUL(DSQRT(DADD(DMUL(pXcd, pXcd), DMUL(pYcd, pYcd))), 0.001), g.c_pixel_size);
  const double rND2R = r_by_rdist(tbl, g.tbl_len, DDIV(rD, g.c_distortion_radius));
  pXc = DMUL(pXcd, rND2R);
  pYc = DMUL(pYcd, rND2R);
}

// getPortsCoordinatesAndDerivatives (GeometryCorrection.java:2159-2314) for one sensor
// (pXc, pYc): the task's undistorted centre (center_undistort), the same for every sensor
__device__ void port_xy(const GeomDev &g, double pXc, double pYc, double disparity, int i, double &ox, double &oy,
                        double *deriv /* [2][5] or null */) {
  const double fl_pix = g.fl_pix, ri_scale = g.ri_scale;
  double vi[3] = {DSUB(pXc, DMUL(disparity, g.rXY[i][0])), DSUB(pYc, DMUL(disparity, g.rXY[i][1])), fl_pix};
  double rvi[3];
  mat3_vec(g.rots[i], vi, rvi);
  double norm_z = DDIV(fl_pix, rvi[2]);
  double pXci = DMUL(rvi[0], norm_z);
  double pYci = DMUL(rvi[1], norm_z);
  double rNDi = DSQRT(DADD(DMUL(pXci, pXci), DMUL(pYci, pYci)));
  double ri = DMUL(rNDi, ri_scale);
  double rD2rND = 1.0, rri = 1.0;
#pragma unroll
  for (int j = 0; j < 7; j++) {
    rri = DMUL(rri, ri);
    rD2rND = DADD(rD2rND, DMUL(g.rad_coeff[j], DSUB(rri, 1.0)));
  }
  ox = DADD(DMUL(pXci, rD2rND), g.pXY0[i][0]);
  oy = DADD(DMUL(pYci, rD2rND), g.pXY0[i][1]);
  if (deriv) {
    // quotients shared by the five parameters (a product with a reciprocal where the reference
    // divides: the derivatives differ from its by an ulp, the ports are not touched)
    const double ri_rnd = DDIV(ri_scale, rNDi);
    const double inv_rz = DDIV(1.0, rvi[2]);
    const double pXr = DMUL(pXci, inv_rz), pYr = DMUL(pYci, inv_rz);
    double drD2rND_dri = 0.0;
    rri = 1.0;
#pragma unroll
    for (int j = 0; j < 7; j++) {
      drD2rND_dri = DADD(drD2rND_dri, DMUL(g.rad_dcoeff[j], rri));
      rri = DMUL(rri, ri);
    }
#pragma unroll
    for (int k = 0; k < 5; k++) {  // azimuth, tilt, roll, zoom; then the tile disparity
      double dr[3];
      if (k < 4) {
        mat3_vec(g.drots[i][k], vi, dr);
      } else {  // d vi / d disparity = (-rX, -rY, 0)
        const double dvi[3] = {-g.rXY[i][0], -g.rXY[i][1], 0.0};
        mat3_vec(g.rots[i], dvi, dr);
      }
      double dpX = DSUB(DMUL(dr[0], norm_z), DMUL(pXr, dr[2]));
      double dpY = DSUB(DMUL(dr[1], norm_z), DMUL(pYr, dr[2]));
      if (k == 2) {  // roll: the reference keeps only the rotation term
        deriv[k] = DMUL(dpX, rD2rND);
        deriv[5 + k] = DMUL(dpY, rD2rND);
      } else {
        double dri = DMUL(ri_rnd, DADD(DMUL(pXci, dpX), DMUL(pYci, dpY)));
        double drD = DMUL(drD2rND_dri, dri);
        deriv[k] = DADD(DMUL(dpX, rD2rND), DMUL(pXci, drD));
        deriv[5 + k] = DADD(DMUL(dpY, rD2rND), DMUL(pYci, drD));
      }
    }
  }
}

// sensor part of getPortsCoordinatesAndDerivatives (GeometryCorrection.java:2190-2217)
__device__ __forceinline__ void sensor_port(const GeomDev &g, double pXc, double pYc, double disparity, int i,
                                            double &ox, double &oy) {
  const double fl_pix = g.fl_pix, ri_scale = g.ri_scale;
  const double vi[3] = {DSUB(pXc, DMUL(disparity, g.rXY[i][0])), DSUB(pYc, DMUL(disparity, g.rXY[i][1])), fl_pix};
  double rvi[3];
  mat3_vec(g.rots[i], vi, rvi);
  const double norm_z = DDIV(fl_pix, rvi[2]);
  const double pXci = DMUL(rvi[0], norm_z), pYci = DMUL(rvi[1], norm_z);
  const double ri = DMUL(DSQRT(DADD(DMUL(pXci, pXci), DMUL(pYci, pYci))), ri_scale);
  double rD2rND = 1.0, rri = 1.0;
#pragma unroll
  for (int j = 0; j < 7; j++) {
    rri = DMUL(rri, ri);
    rD2rND = DADD(rD2rND, DMUL(g.rad_coeff[j], DSUB(rri, 1.0)));
  }
  ox = DADD(DMUL(pXci, rD2rND), g.pXY0[i][0]);
  oy = DADD(DMUL(pYci, rD2rND), g.pXY0[i][1]);
}

// One thread per task: the centre is undistorted once, the kernel tile is found
// once per sensor (it depends on the port only), then each colour's window
// corner and residual shift (ImageDtt.java:4904-4943).  A division by a
// power-of-two kernel step is replaced by the multiplication with its exact
// reciprocal, which IEEE rounding makes bit-identical.
// sensors [s0, s1) of one task
__device__ __forceinline__ void plan_task(const SceneDev &sc, int task, int s0, int s1) {
  const int S = sc.num_sensors, C = sc.num_colors;
  const int txy = sc.task_txy[task];
  const int tx = txy & 0xffff, ty = txy >> 16;
  const double ctx = (double)(tx * TP_DTT + TP_DTT / 2), cty = (double)(ty * TP_DTT + TP_DTT / 2);
  double pXc = 0.0, pYc = 0.0, disparity = 0.0;
  if (sc.ports_from_geometry) {
    center_undistort(*sc.geom, sc.rdist_tbl, ctx, cty, pXc, pYc);
    disparity = (double)sc.task_disp[task];
    // a rig's auxiliary camera: disparity_main * aux radius / main radius (ImageDtt.java:8973)
    if (sc.geom->rig) disparity = DDIV(DMUL(disparity, sc.geom->disp_num), sc.geom->disp_den);
  }
  const int ks = sc.kernel_step;
  const bool pow2 = ks > 0 && (ks & (ks - 1)) == 0;
  const double inv_ks = pow2 ? 1.0 / (double)ks : 0.0;
  for (int s = s0; s < s1; s++) {
    double cx, cy;
    if (sc.ports_from_geometry) {
      if (sc.port_deriv) {
        double dv[10];
        port_xy(*sc.geom, pXc, pYc, disparity, s, cx, cy, dv);
        double *o = sc.port_deriv + ((size_t)task * S + s) * 10;
#pragma unroll
        for (int k = 0; k < 10; k++) o[k] = dv[k];
      } else {
        sensor_port(*sc.geom, pXc, pYc, disparity, s, cx, cy);
      }
    } else {
      cx = (double)sc.task_xy[((size_t)task * S + s) * 2];
      cy = (double)sc.task_xy[((size_t)task * S + s) * 2 + 1];
    }
    sc.ports[((size_t)task * S + s) * 2] = cx;
    sc.ports[((size_t)task * S + s) * 2 + 1] = cy;
    int ktx = 0, kty = 0;
    double kdx = 0.0, kdy = 0.0;
    if (sc.kh > 0) {
      const double qx = pow2 ? DMUL(cx, inv_ks) : DDIV(cx, (double)ks);
      const double qy = pow2 ? DMUL(cy, inv_ks) : DDIV(cy, (double)ks);
      ktx = (int)java_round(qx) + 1;
      kty = (int)java_round(qy) + 1;
      kty = kty < 0 ? 0 : (kty >= sc.kv ? sc.kv - 1 : kty);
      ktx = ktx < 0 ? 0 : (ktx >= sc.kh ? sc.kh - 1 : ktx);
      kdx = DSUB(cx, DMUL(DADD((double)(ktx - 1), 0.5), (double)ks));
      kdy = DSUB(cy, DMUL(DADD((double)(kty - 1), 0.5), (double)ks));
    }
    for (int c = 0; c < C; c++) {
      double px = DSUB(cx, (double)TP_DTT), py = DSUB(cy, (double)TP_DTT);
      int kidx = -1;
      if (sc.kh > 0) {
        kidx = (kty * sc.kh + ktx) * C + c;
        const float4 *ce4 = (const float4 *)(sc.kext[s] + (size_t)kidx * 8);
        const float4 e0 = __ldg(ce4), e1 = __ldg(ce4 + 1);  // data_x, data_y, -, -, dxc_dx, dxc_dy, dyc_dx, dyc_dy
        px = DSUB(DSUB(cx, (double)TP_DTT), DADD(DADD((double)e0.x, DMUL((double)e1.x, kdx)), DMUL((double)e1.y, kdy)));
        py = DSUB(DSUB(cy, (double)TP_DTT), DADD(DADD((double)e0.y, DMUL((double)e1.z, kdx)), DMUL((double)e1.w, kdy)));
      }
      const double tl = -java_round(-px), tt = -java_round(-py);
      SubtilePlan p;
      p.tlx = clamp_corner(tl, sc.width);
      p.tly = clamp_corner(tt, sc.height);
      p.kidx = kidx;
      p.rx = (float)(-(DSUB(px, tl)));
      p.ry = (float)(-(DSUB(py, tt)));
      sc.plan[((size_t)task * S + s) * C + c] = p;
    }
  }
}

// thread per (task, group of up to 4 sensors): 16-sensor scenes get 4x the threads
__global__ void plan_kernel(SceneDev sc) {
  const int groups = (sc.num_sensors + 3) >> 2;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sc.num_tasks * groups) return;
  const int task = i / groups, g = i - task * groups;
  const int s0 = g * 4, s1 = (s0 + 4 < sc.num_sensors) ? s0 + 4 : sc.num_sensors;
  plan_task(sc, task, s0, s1);
}

// the plans of a batch of scenes in one launch: thread per task of the
// concatenated task lists, scene found by binary search over the task offsets
__global__ void plan_batch_kernel(const SceneDev *__restrict__ scenes, const int *__restrict__ task_off, int n) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= task_off[n]) return;
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (task_off[mid] <= g) lo = mid;
    else hi = mid - 1;
  }
  const SceneDev &sc = scenes[lo];
  const int task = g - task_off[lo];
  plan_task(sc, task, 0, sc.num_sensors);
  const int txy = sc.task_txy[task];
  sc.tile_task[(txy >> 16) * sc.tilesX + (txy & 0xffff)] = task;
}

__global__ void tile_task_map_kernel(SceneDev sc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < sc.num_tasks) {
    int txy = sc.task_txy[i];
    int tile = (txy >> 16) * sc.tilesX + (txy & 0xffff);
    if (tile >= 0 && tile < sc.tilesX * sc.tilesY) sc.tile_task[tile] = i;
  }
}

// Row-major compaction of tiles with tile_op != 0 into the task list
// (GPUTileProcessor.setFullFrameImages order).  One block; deterministic.
__global__ void compact_tasks_kernel(const int *tile_op, const float *disparity, int tilesX, int num_tiles,
                                     int *task_txy, int *task_op, float *task_disp, int *num_tasks) {
  __shared__ int warp_sums[32];
  __shared__ int base;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int start = 0; start < num_tiles; start += blockDim.x) {
    int i = start + threadIdx.x;
    int op = (i < num_tiles) ? tile_op[i] : 0;
    int flag = op != 0;
    unsigned m = __ballot_sync(0xffffffffu, flag);
    int pre = __popc(m & ((1u << lane) - 1u));
    if (lane == 31) warp_sums[warp] = pre + flag;
    __syncthreads();
    if (warp == 0) {
      int v = (lane < nwarps) ? warp_sums[lane] : 0;
      int incl = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      if (lane < nwarps) warp_sums[lane] = incl - v;
    }
    __syncthreads();
    int pos = base + warp_sums[warp] + pre;
    if (flag) {
      int ty = i / tilesX, tx = i - ty * tilesX;
      task_txy[pos] = tx | (ty << 16);
      task_op[pos] = op;
      task_disp[pos] = disparity ? disparity[i] : 0.0f;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) base = pos + flag;
    __syncthreads();
  }
  if (threadIdx.x == 0) *num_tasks = base;
}

cudaError_t launch_plan(const SceneDev &sc, cudaStream_t st) {
  const int n = sc.num_tasks * ((sc.num_sensors + 3) / 4);
  if (n <= 0) return cudaSuccess;
  plan_kernel<<<(n + 63) / 64, 64, 0, st>>>(sc);
  return cudaGetLastError();
}

// tile maps are cleared by the caller (cudaMemsetAsync per scene) before this launch
cudaError_t launch_plan_batch(const SceneDev *scenes_dev, const int *task_off_dev, int n, int total_tasks,
                              cudaStream_t st) {
  if (total_tasks <= 0) return cudaSuccess;
  plan_batch_kernel<<<(total_tasks + 63) / 64, 64, 0, st>>>(scenes_dev, task_off_dev, n);
  return cudaGetLastError();
}

cudaError_t launch_tile_task_map(const SceneDev &sc, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(sc.tile_task, 0xff, sizeof(int) * sc.tilesX * sc.tilesY, st);
  if (e != cudaSuccess) return e;
  if (sc.num_tasks <= 0) return cudaSuccess;
  tile_task_map_kernel<<<(sc.num_tasks + 255) / 256, 256, 0, st>>>(sc);
  return cudaGetLastError();
}

// multi-block compaction: per-block counts, then each block adds the counts of
// the blocks before it and scatters its tiles in row-major order
constexpr int CB = 1024;
__global__ void compact_count_kernel(const int *tile_op, int num_tiles, int *block_counts) {
  const int i = blockIdx.x * CB + threadIdx.x;
  const int n = __syncthreads_count(i < num_tiles && tile_op[i] != 0);
  if (threadIdx.x == 0) block_counts[blockIdx.x] = n;
}

__global__ void compact_scatter_kernel(const int *tile_op, const float *disparity, int tilesX, int num_tiles,
                                       const int *block_counts, int *task_txy, int *task_op, float *task_disp,
                                       int *num_tasks) {
  __shared__ int warp_sums[32];
  __shared__ int base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp == 0) {
    int b = 0;
    for (int k = lane; k < blockIdx.x; k += 32) b += block_counts[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) b += __shfl_xor_sync(0xffffffffu, b, o);
    if (lane == 0) {
      base = b;
      if (blockIdx.x == gridDim.x - 1) *num_tasks = b + block_counts[blockIdx.x];
    }
  }
  const int i = blockIdx.x * CB + threadIdx.x;
  const int op = (i < num_tiles) ? tile_op[i] : 0;
  const int flag = op != 0;
  const unsigned m = __ballot_sync(0xffffffffu, flag);
  const int pre = __popc(m & ((1u << lane) - 1u));
  if (lane == 31) warp_sums[warp] = pre + flag;
  __syncthreads();
  if (warp == 0) {
    const int v = warp_sums[lane];
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    warp_sums[lane] = incl - v;
  }
  __syncthreads();
  if (flag) {
    const int pos = base + warp_sums[warp] + pre;
    const int ty = i / tilesX, tx = i - ty * tilesX;
    task_txy[pos] = tx | (ty << 16);
    task_op[pos] = op;
    task_disp[pos] = disparity ? disparity[i] : 0.0f;
  }
}

cudaError_t launch_compact_tasks(const int *tile_op, const float *disparity, int tilesX, int num_tiles,
                                 int *task_txy, int *task_op, float *task_disp, int *num_tasks_dev,
                                 cudaStream_t st) {
  const int nb = (num_tiles + CB - 1) / CB;
  if (nb <= 1) {
    compact_tasks_kernel<<<1, 1024, 0, st>>>(tile_op, disparity, tilesX, num_tiles, task_txy, task_op, task_disp,
                                             num_tasks_dev);
    return cudaGetLastError();
  }
  int *counts = num_tasks_dev + 1;  // the caller sizes num_tasks_dev for 1 + nb ints
  compact_count_kernel<<<nb, CB, 0, st>>>(tile_op, num_tiles, counts);
  compact_scatter_kernel<<<nb, CB, 0, st>>>(tile_op, disparity, tilesX, num_tiles, counts, task_txy, task_op,
                                            task_disp, num_tasks_dev);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Task compaction that allocates nothing: the per-block counts go to a fixed
// file-scope device array instead of a handle's buffer.  Every count slot the
// scatter reads is written earlier in the same call by compact_count_kernel,
// so nothing has to start at zero; concurrent calls on one device share the
// array and race.
// ---------------------------------------------------------------------------
constexpr int COMPACT_SCRATCH_BLOCKS = 1024;  // x CB tiles per block = 1,048,576 tiles
static __device__ __align__(256) int g_compact_scratch[COMPACT_SCRATCH_BLOCKS];

int compact_scratch_max_tiles() { return COMPACT_SCRATCH_BLOCKS * CB; }

cudaError_t compact_scratch_address(int **ptr) {
  return cudaGetSymbolAddress((void **)ptr, g_compact_scratch);
}

cudaError_t launch_compact_tasks_scratch(const int *tile_op, const float *disparity, int tilesX, int num_tiles,
                                         int *task_txy, int *task_op, float *task_disp, int *num_tasks_dev,
                                         int *scratch, cudaStream_t st) {
  const int nb = (num_tiles + CB - 1) / CB;
  if (nb > COMPACT_SCRATCH_BLOCKS) return cudaErrorInvalidValue;
  if (nb <= 1) {
    compact_tasks_kernel<<<1, 1024, 0, st>>>(tile_op, disparity, tilesX, num_tiles, task_txy, task_op, task_disp,
                                             num_tasks_dev);
    return cudaGetLastError();
  }
  compact_count_kernel<<<nb, CB, 0, st>>>(tile_op, num_tiles, scratch);
  compact_scatter_kernel<<<nb, CB, 0, st>>>(tile_op, disparity, tilesX, num_tiles, scratch, task_txy, task_op,
                                            task_disp, num_tasks_dev);
  return cudaGetLastError();
}
