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

// getPortsCoordinatesAndDerivatives (GeometryCorrection.java:2159-2314) for one sensor
__device__ void port_xy(const GeomDev &g, const double *tbl, double px, double py, double disparity, int i,
                        double &ox, double &oy, double *deriv /* [2][4] or null */) {
  double pXcd = DSUB(px, DMUL(0.5, (double)g.pixel_width));
  double pYcd = DSUB(py, DMUL(0.5, (double)g.pixel_height));
  double rD = DMUL(DMUL(DSQRT(DADD(DMUL(pXcd, pXcd), DMUL(pYcd, pYcd))), 0.001), g.pixel_size);
  double rND2R = r_by_rdist(tbl, g.tbl_len, DDIV(rD, g.distortion_radius));
  double pXc = DMUL(pXcd, rND2R);
  double pYc = DMUL(pYcd, rND2R);
  double fl_pix = DDIV(g.focal_length, DMUL(0.001, g.pixel_size));
  double ri_scale = DDIV(DMUL(0.001, g.pixel_size), g.distortion_radius);
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
    double drD2rND_dri = 0.0;
    rri = 1.0;
#pragma unroll
    for (int j = 0; j < 7; j++) {
      drD2rND_dri = DADD(drD2rND_dri, DMUL(DMUL(g.rad_coeff[j], (double)(j + 1)), rri));
      rri = DMUL(rri, ri);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {  // azimuth, tilt, roll, zoom
      double dr[3];
      mat3_vec(g.drots[i][k], vi, dr);
      double dpX = DSUB(DMUL(dr[0], norm_z), DDIV(DMUL(pXci, dr[2]), rvi[2]));
      double dpY = DSUB(DMUL(dr[1], norm_z), DDIV(DMUL(pYci, dr[2]), rvi[2]));
      if (k == 2) {  // roll: the reference keeps only the rotation term
        deriv[k] = DMUL(dpX, rD2rND);
        deriv[4 + k] = DMUL(dpY, rD2rND);
      } else {
        double dri = DMUL(DDIV(ri_scale, rNDi), DADD(DMUL(pXci, dpX), DMUL(pYci, dpY)));
        double drD = DMUL(drD2rND_dri, dri);
        deriv[k] = DADD(DMUL(dpX, rD2rND), DMUL(pXci, drD));
        deriv[4 + k] = DADD(DMUL(dpY, rD2rND), DMUL(pYci, drD));
      }
    }
  }
}

// one thread per (task, sensor): ports, then the window plan of each colour
__global__ void plan_kernel(SceneDev sc) {
  int gid = blockIdx.x * blockDim.x + threadIdx.x;
  int S = sc.num_sensors, C = sc.num_colors;
  int task = gid / S, s = gid - task * S;
  if (task >= sc.num_tasks) return;
  int txy = sc.task_txy[task];
  int tx = txy & 0xffff, ty = txy >> 16;
  double cx, cy;
  if (sc.ports_from_geometry) {
    double dv[8];
    port_xy(*sc.geom, sc.rdist_tbl, (double)(tx * TP_DTT + TP_DTT / 2), (double)(ty * TP_DTT + TP_DTT / 2),
            (double)sc.task_disp[task], s, cx, cy, sc.port_deriv ? dv : nullptr);
    if (sc.port_deriv) {
      double *o = sc.port_deriv + ((size_t)task * S + s) * 8;
#pragma unroll
      for (int k = 0; k < 8; k++) o[k] = dv[k];
    }
  } else {
    cx = (double)sc.task_xy[((size_t)task * S + s) * 2];
    cy = (double)sc.task_xy[((size_t)task * S + s) * 2 + 1];
  }
  sc.ports[((size_t)task * S + s) * 2] = cx;
  sc.ports[((size_t)task * S + s) * 2 + 1] = cy;
  for (int c = 0; c < C; c++) {
    double px = DSUB(cx, (double)TP_DTT), py = DSUB(cy, (double)TP_DTT);
    int kidx = -1;
    if (sc.kh > 0) {  // ImageDtt.java:4904-4932
      int ktx = (int)java_round(DDIV(cx, (double)sc.kernel_step)) + 1;
      int kty = (int)java_round(DDIV(cy, (double)sc.kernel_step)) + 1;
      kty = kty < 0 ? 0 : (kty >= sc.kv ? sc.kv - 1 : kty);
      ktx = ktx < 0 ? 0 : (ktx >= sc.kh ? sc.kh - 1 : ktx);
      kidx = (kty * sc.kh + ktx) * C + c;
      const float *ce = sc.kext[s] + (size_t)kidx * 8;
      double kdx = DSUB(cx, DMUL(DADD((double)(ktx - 1), 0.5), (double)sc.kernel_step));
      double kdy = DSUB(cy, DMUL(DADD((double)(kty - 1), 0.5), (double)sc.kernel_step));
      px = DSUB(DSUB(cx, (double)TP_DTT), DADD(DADD((double)ce[0], DMUL((double)ce[4], kdx)), DMUL((double)ce[5], kdy)));
      py = DSUB(DSUB(cy, (double)TP_DTT), DADD(DADD((double)ce[1], DMUL((double)ce[6], kdx)), DMUL((double)ce[7], kdy)));
    }
    double tl = -java_round(-px), tt = -java_round(-py);
    SubtilePlan p;
    p.tlx = (int)tl;
    p.tly = (int)tt;
    p.kidx = kidx;
    p.rx = (float)(-(DSUB(px, tl)));
    p.ry = (float)(-(DSUB(py, tt)));
    sc.plan[((size_t)task * S + s) * C + c] = p;
  }
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
  int n = sc.num_tasks * sc.num_sensors;
  if (n <= 0) return cudaSuccess;
  plan_kernel<<<(n + 127) / 128, 128, 0, st>>>(sc);
  return cudaGetLastError();
}

cudaError_t launch_tile_task_map(const SceneDev &sc, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(sc.tile_task, 0xff, sizeof(int) * sc.tilesX * sc.tilesY, st);
  if (e != cudaSuccess) return e;
  if (sc.num_tasks <= 0) return cudaSuccess;
  tile_task_map_kernel<<<(sc.num_tasks + 255) / 256, 256, 0, st>>>(sc);
  return cudaGetLastError();
}

cudaError_t launch_compact_tasks(const int *tile_op, const float *disparity, int tilesX, int num_tiles,
                                 int *task_txy, int *task_op, float *task_disp, int *num_tasks_dev,
                                 cudaStream_t st) {
  compact_tasks_kernel<<<1, 1024, 0, st>>>(tile_op, disparity, tilesX, num_tiles, task_txy, task_op, task_disp,
                                           num_tasks_dev);
  return cudaGetLastError();
}
