// tp_kernels.cu -- FP32 stages of the GB300 tile processor.
//
//   convert_correct : image window -> shifted-window fold -> 2D DCT-IV/DST-IV
//                     -> CLT-domain aberration convolution -> phase-rotation shift
//                     (ImageDtt.extract_correct_tile / convolve_tile / fract_shift,
//                      the reference GPU convert_correct_tiles)
//   correlate       : fat-zero-normalised pair correlation, colour mix, LPF,
//                     DCT-IIe/DST-IIe to the pixel domain, 15x15 unfold
//                     (Correlation2d.correlateCompositeFD)
//   extract         : disparity-axis strips, combination, integer argmax,
//                     windowed centroid, hor/vert ortho maxima (Correlation2d)
//   imclt           : inverse CLT with overlap-add into padded colour frames
//                     (ImageDtt.iclt_2d, the reference GPU imclt_rbg)
//
// Thread mapping: one warp owns one (tile, sensor, colour) sub-tile or one
// (tile, pair).  Lane l works on quadrant m = l>>3 and row r = l&7 for the
// separable 8-point transforms (the 8 values of a row stay in registers); the
// row<->column transpose goes through a per-warp shared-memory buffer padded to
// 9 floats per row so both access patterns are bank-conflict free.  Element-wise
// stages (convolution, shift, correlation products) use lane l on CLT indices
// l and l+32 so that global loads/stores of 4x64 floats are full 128-byte lines.
#include "tp_internal.h"
#include <math_constants.h>
#include <cmath>
#include <cstdint>

__constant__ float c_dct4[64];   // orthonormal DCT-IV, [k*8+n]
__constant__ float c_dct2e[64];  // DttRad2 CIIe, [j*8+k]
__constant__ float c_hwin[8];    // sine half-window (DttRad2.set_window(1))

cudaError_t upload_kernel_constants() {
  float d4[64], d2[64], hw[8];
  const double pi = 3.14159265358979323846;
  for (int k = 0; k < 8; k++)
    for (int n = 0; n < 8; n++) {
      d4[k * 8 + n] = (float)(std::sqrt(2.0 / 8) * std::cos(pi * (2 * n + 1) * (2 * k + 1) / 32.0));
      d2[k * 8 + n] = (float)(std::sqrt(2.0 / 8) * std::cos(pi * k * (2 * n + 1) / 16.0));
    }
  for (int i = 0; i < 8; i++) hw[i] = (float)std::sin(pi / 16.0 * (i + 0.5));
  cudaError_t e = cudaMemcpyToSymbol(c_dct4, d4, sizeof(d4));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_dct2e, d2, sizeof(d2));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_hwin, hw, sizeof(hw));
  return e;
}

// ---------------------------------------------------------------------------
// 8-point transforms on one lane's registers
// ---------------------------------------------------------------------------
__device__ __forceinline__ void dct4_mat(const float x[8], float y[8]) {
#pragma unroll
  for (int k = 0; k < 8; k++) {
    float s = 0.f;
#pragma unroll
    for (int n = 0; n < 8; n++) s = fmaf(c_dct4[k * 8 + n], x[n], s);
    y[k] = s;
  }
}
// DCT-IV, or DST-IV when `sine`: DST-IV(x)[k] = (-1)^k DCT-IV(reverse(x))[k]
// (the identity DttRad2.dst_iv is built on, DttRad2.java:87-98)
__device__ __forceinline__ void dtt4(const float x[8], float y[8], bool sine) {
  float xr[8];
#pragma unroll
  for (int n = 0; n < 8; n++) xr[n] = sine ? x[7 - n] : x[n];
  dct4_mat(xr, y);
#pragma unroll
  for (int k = 1; k < 8; k += 2) y[k] = sine ? -y[k] : y[k];
}
// DCT-IIe, or DST-IIe when `sine`: SIIe[j][k] = (-1)^k CIIe[7-j][k]
__device__ __forceinline__ void dtt2e(const float x[8], float y[8], bool sine) {
  float xs[8], t[8];
#pragma unroll
  for (int n = 0; n < 8; n++) xs[n] = (sine && (n & 1)) ? -x[n] : x[n];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    float s = 0.f;
#pragma unroll
    for (int n = 0; n < 8; n++) s = fmaf(c_dct2e[k * 8 + n], xs[n], s);
    t[k] = s;
  }
#pragma unroll
  for (int j = 0; j < 8; j++) y[j] = sine ? t[7 - j] : t[j];
}

// fold-index record of DttRad2.get_fold_indices (DttRad2.java:109-144) for n = 8
struct FoldIdx {
  int src0, win0, dwin0, src1, win1, dwin1;
  float sc0, ss0, ds0, sc1, ss1, ds1;
};
__device__ __forceinline__ FoldIdx fold_idx(int x) {
  FoldIdx f;
  if (x < 4) {
    f.src0 = 11 - x; f.win0 = 4 + x; f.sc0 = -1.f; f.ss0 = 1.f; f.dwin0 = 3 - x; f.ds0 = -1.f;
    f.src1 = 12 + x; f.win1 = 3 - x; f.sc1 = -1.f; f.ss1 = -1.f; f.dwin1 = 4 + x; f.ds1 = -1.f;
  } else {
    x -= 4;
    f.src0 = x; f.win0 = x; f.sc0 = 1.f; f.ss0 = 1.f; f.dwin0 = 7 - x; f.ds0 = 1.f;
    f.src1 = 7 - x; f.win1 = 7 - x; f.sc1 = -1.f; f.ss1 = 1.f; f.dwin1 = x; f.ds1 = 1.f;
  }
  return f;
}

__device__ __forceinline__ int bayer_color(int x, int y, int rr, int rc) {
  int xo = (x & 1) == rc, yo = (y & 1) == rr;
  return (xo && yo) ? 0 : ((!xo && !yo) ? 1 : 2);
}

__device__ __forceinline__ int mirror(int p, int n) {  // ImageDtt.java:4958-4969
  if (p < 0) return p & 1;
  if (p >= n) return n - 2 + (p & 1);
  return p;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Stage 2: convert + correct, one warp per (task, sensor, colour)
// ---------------------------------------------------------------------------
#define CC_WARPS 4
#define WIN_STRIDE 17
#define QBUF 288  // 4 quadrants x 8 rows x 9

__device__ __forceinline__ void convert_correct_subtile(const SceneDev &sc, int task, int s, int c,
                                                        float *wb, float *tb, int lane, float out_regs[4][2]) {
  const int S = sc.num_sensors, C = sc.num_colors;
  const SubtilePlan p = sc.plan[((size_t)task * S + s) * C + c];
  // 1. 16x16 window (mirrored at the image border), one colour of the mosaic
  {
    const int W = sc.width, H = sc.height;
    int col = lane & 15, r0 = lane >> 4;
    int x = mirror(p.tlx + col, W);
    const float scale = sc.color_scale[c];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      int row = 2 * k + r0;
      int y = mirror(p.tly + row, H);
      size_t o = (size_t)y * sc.img_pitch + x;
      float v = (sc.img_dtype[s] == 1) ? (float)__ldg((const uint16_t *)sc.images[s] + o)
                                    : __ldg((const float *)sc.images[s] + o);
      if (C == 3) v = (bayer_color(x, y, sc.bayer_red_row, sc.bayer_red_col) == c) ? v * scale : 0.f;
      else v *= scale;
      wb[row * WIN_STRIDE + col] = v;
    }
  }
  __syncwarp();
  const int m = lane >> 3, r = lane & 7;
  // 2. shifted-window fold (DttRad2.get_shifted_fold_2d + fold_tile), row r of quadrant m
  float ahs, ahc, avs, avc;
  sincospif(p.rx * 0.0625f, &ahs, &ahc);
  sincospif(p.ry * 0.0625f, &avs, &avc);
  float y[8];
  {
    FoldIdx fv = fold_idx(r);
    float vw0 = avc * c_hwin[fv.win0] + avs * c_hwin[fv.dwin0] * fv.ds0;
    float vw1 = avc * c_hwin[fv.win1] + avs * c_hwin[fv.dwin1] * fv.ds1;
    bool vb = (m >> 1) & 1, hb = m & 1;
    float vk0 = (vb ? fv.ss0 : fv.sc0) * vw0;
    float vk1 = (vb ? fv.ss1 : fv.sc1) * vw1;
    const float *row0 = wb + fv.src0 * WIN_STRIDE, *row1 = wb + fv.src1 * WIN_STRIDE;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      FoldIdx fh = fold_idx(j);  // compile-time after unrolling
      float hw0 = ahc * c_hwin[fh.win0] + ahs * c_hwin[fh.dwin0] * fh.ds0;
      float hw1 = ahc * c_hwin[fh.win1] + ahs * c_hwin[fh.dwin1] * fh.ds1;
      float hk0 = (hb ? fh.ss0 : fh.sc0) * hw0;
      float hk1 = (hb ? fh.ss1 : fh.sc1) * hw1;
      float a = fmaf(row0[fh.src1], hk1, row0[fh.src0] * hk0);
      float b = fmaf(row1[fh.src1], hk1, row1[fh.src0] * hk0);
      y[j] = fmaf(vk1, b, vk0 * a);
    }
  }
  // 3. horizontal DCT-IV / DST-IV, transposed store (DttRad2.dttt_iv first pass)
  float z[8];
  dtt4(y, z, m & 1);
#pragma unroll
  for (int j = 0; j < 8; j++) tb[m * 72 + j * 9 + r] = z[j];
  __syncwarp();
#pragma unroll
  for (int i = 0; i < 8; i++) y[i] = tb[m * 72 + r * 9 + i];
  // 4. vertical DCT-IV / DST-IV: lane (m, r) now holds clt[m][r*8 + k], r = horizontal frequency
  dtt4(y, z, (m >> 1) & 1);
  __syncwarp();  // everyone done reading the window before it is reused
#pragma unroll
  for (int k = 0; k < 8; k++) wb[m * 72 + r * 9 + k] = z[k];
  // shift coefficients: lanes 0-7 horizontal frequency i, lanes 8-15 vertical frequency k
  float cs_s, cs_c;
  {
    int f = lane & 7;
    float sh = (lane < 8) ? p.rx : p.ry;
    sincospif((f + 0.5f) * sh * 0.125f, &cs_s, &cs_c);
  }
  __syncwarp();
  // 5. CLT-domain convolution (ImageDtt.convolve_tile) and phase-rotation shift (fract_shift)
  const float *kp = (p.kidx >= 0) ? sc.kernels[s] + (size_t)p.kidx * TP_CLT : nullptr;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    int idx = lane + 32 * h;
    int off = (idx >> 3) * 9 + (idx & 7);
    float d0 = wb[off], d1 = wb[72 + off], d2 = wb[144 + off], d3 = wb[216 + off];
    float r0v = d0, r1v = d1, r2v = d2, r3v = d3;
    if (kp) {
      float k0 = __ldg(kp + idx), k1 = __ldg(kp + 64 + idx), k2 = __ldg(kp + 128 + idx), k3 = __ldg(kp + 192 + idx);
      // zi = {{0,-1,-2,3},{1,0,-3,-2},{2,-3,0,-1},{3,2,1,0}} (ImageDtt.java:5458-5462)
      r0v = d0 * k0 - d1 * k1 - d2 * k2 + d3 * k3;
      r1v = d1 * k0 + d0 * k1 - d3 * k2 - d2 * k3;
      r2v = d2 * k0 - d3 * k1 + d0 * k2 - d1 * k3;
      r3v = d3 * k0 + d2 * k1 + d1 * k2 + d0 * k3;
    }
    int fi = idx >> 3, fk = idx & 7;
    float ch = __shfl_sync(0xffffffffu, cs_c, fi), sh = __shfl_sync(0xffffffffu, cs_s, fi);
    float cv = __shfl_sync(0xffffffffu, cs_c, 8 + fk), sv = __shfl_sync(0xffffffffu, cs_s, 8 + fk);
    float t0 = r0v * ch - r1v * sh, t1 = r1v * ch + r0v * sh;
    float t2 = r2v * ch - r3v * sh, t3 = r3v * ch + r2v * sh;
    out_regs[0][h] = t0 * cv - t2 * sv;
    out_regs[2][h] = t2 * cv + t0 * sv;
    out_regs[1][h] = t1 * cv - t3 * sv;
    out_regs[3][h] = t3 * cv + t1 * sv;
  }
  __syncwarp();
}

__global__ void __launch_bounds__(CC_WARPS * 32) convert_correct_kernel(SceneDev sc) {
  __shared__ float smem[CC_WARPS][2 * QBUF];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *wb = smem[warp];
  float *tb = wb + QBUF;  // window (16x17) and the CLT buffer (4x8x9) share the first QBUF floats
  const int S = sc.num_sensors, C = sc.num_colors;
  const int total = sc.num_tasks * S * C;
  for (int st = blockIdx.x * CC_WARPS + warp; st < total; st += gridDim.x * CC_WARPS) {
    int task = st / (S * C), rem = st - task * S * C;
    int s = rem / C, c = rem - s * C;
    float o[4][2];
    convert_correct_subtile(sc, task, s, c, wb, tb, lane, o);
    int txy = sc.task_txy[task];
    size_t tile = (size_t)(txy >> 16) * sc.tilesX + (txy & 0xffff);
    float *dst = sc.clt + ((tile * S + s) * C + c) * TP_CLT;
    // the reference GPU's lpf_mask (TileProcessor.cuh:1037-1061): the stored CLT times the LPF
    const bool lp = sc.lpf_rbg && ((sc.clt_lpf_mask >> c) & 1);
    const float l0 = lp ? sc.lpf_rbg[c * 64 + lane] : 1.f, l1 = lp ? sc.lpf_rbg[c * 64 + lane + 32] : 1.f;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      dst[q * 64 + lane] = o[q][0] * l0;
      dst[q * 64 + lane + 32] = o[q][1] * l1;
    }
  }
}

// ---------------------------------------------------------------------------
// Stage 3a: pair correlation, one warp per (task, pair)
// ---------------------------------------------------------------------------
__device__ void correlate_pair_warp(const SceneDev &sc, const CorrDev &cfg, size_t tile, int pi, float *qb,
                                    float *tb, int lane, float *corr_out) {
  const int S = sc.num_sensors, C = sc.num_colors;
  const PairDev pd = cfg.pairs[pi];
  const float *c1 = sc.clt + (tile * S + pd.cam1) * C * TP_CLT;
  const float *c2 = sc.clt + (tile * S + pd.cam2) * C * TP_CLT;
  float acc[4][2];
  for (int c = 0; c < C; c++) {
    float d1[4][2], d2[4][2], a2[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      float s1 = 0.f, s2 = 0.f;
#pragma unroll
      for (int n = 0; n < 4; n++) {
        d1[n][h] = c1[c * TP_CLT + n * 64 + lane + 32 * h];
        d2[n][h] = c2[c * TP_CLT + n * 64 + lane + 32 * h];
        s1 = fmaf(d1[n][h], d1[n][h], s1);
        s2 = fmaf(d2[n][h], d2[n][h], s2);
      }
      a2[h] = sqrtf(s1 * s2);
    }
    float sa2 = warp_sum(a2[0] + a2[1]);
    float fz2 = sa2 * (1.0f / 64) * cfg.fat_zero * cfg.fat_zero;  // Correlation2d.java:214
    float w = (C == 1) ? 1.0f : cfg.col_weights[c];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      float scale = 1.0f / (a2[h] + fz2);
      // ZI = {{0,1,2,3},{-1,0,-3,2},{-2,-3,0,1},{3,-2,-1,0}} (Correlation2d.java:86-90)
      float t0 = d1[0][h] * d2[0][h] + d1[1][h] * d2[1][h] + d1[2][h] * d2[2][h] + d1[3][h] * d2[3][h];
      float t1 = -d1[1][h] * d2[0][h] + d1[0][h] * d2[1][h] - d1[3][h] * d2[2][h] + d1[2][h] * d2[3][h];
      float t2 = -d1[2][h] * d2[0][h] - d1[3][h] * d2[1][h] + d1[0][h] * d2[2][h] + d1[1][h] * d2[3][h];
      float t3 = d1[3][h] * d2[0][h] - d1[2][h] * d2[1][h] - d1[1][h] * d2[2][h] + d1[0][h] * d2[3][h];
      float sw = scale * w;
      if (c == 0) {
        acc[0][h] = t0 * sw; acc[1][h] = t1 * sw; acc[2][h] = t2 * sw; acc[3][h] = t3 * sw;
      } else {
        acc[0][h] = fmaf(t0, sw, acc[0][h]); acc[1][h] = fmaf(t1, sw, acc[1][h]);
        acc[2][h] = fmaf(t2, sw, acc[2][h]); acc[3][h] = fmaf(t3, sw, acc[3][h]);
      }
    }
  }
#pragma unroll
  for (int h = 0; h < 2; h++) {
    int idx = lane + 32 * h;
    float l = cfg.lpf[idx];
    int off = (idx >> 3) * 9 + (idx & 7);
#pragma unroll
    for (int q = 0; q < 4; q++) qb[q * 72 + off] = acc[q][h] * l;
  }
  __syncwarp();
  // DttRad2.dttt_iie per quadrant, mode = ((q<<1)&2)|((q>>1)&1) (Correlation2d.java:316-319)
  const int q = lane >> 3, r = lane & 7;
  float x[8], y[8];
#pragma unroll
  for (int e = 0; e < 8; e++) x[e] = qb[q * 72 + r * 9 + e];
  dtt2e(x, y, (q >> 1) & 1);
#pragma unroll
  for (int j = 0; j < 8; j++) tb[q * 72 + j * 9 + r] = y[j];
  __syncwarp();
#pragma unroll
  for (int e = 0; e < 8; e++) x[e] = tb[q * 72 + r * 9 + e];
  dtt2e(x, y, q & 1);
#pragma unroll
  for (int e = 0; e < 8; e++) qb[q * 72 + r * 9 + e] = y[e];  // qd[q][vertical r][horizontal e]
  __syncwarp();
  // DttRad2.corr_unfold_tile (443-489): 15x15 centred surface
  for (int o = lane; o < TP_CORR; o += 32) {
    int ri = o / 15, ci = o - ri * 15;
    int i = ri - 7, j = ci - 7;
    int a = i < 0 ? -i : i, b = j < 0 ? -j : j;
    float si = i < 0 ? -1.f : 1.f, sj = j < 0 ? -1.f : 1.f;
    float v = qb[a * 9 + b];
    if (b > 0) v += sj * qb[72 + a * 9 + b - 1];
    if (a > 0) v += si * qb[144 + (a - 1) * 9 + b];
    if (a > 0 && b > 0) v += si * sj * qb[216 + (a - 1) * 9 + b - 1];
    corr_out[o] = 0.25f * v;
  }
  __syncwarp();
}

#define CO_WARPS 4
__global__ void __launch_bounds__(CO_WARPS * 32) correlate_kernel(SceneDev sc) {
  __shared__ float smem[CO_WARPS][2 * QBUF];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const CorrDev &cfg = *sc.corr_cfg;
  const int P = cfg.num_pairs;
  const int total = sc.num_tasks * P;
  for (int w = blockIdx.x * CO_WARPS + warp; w < total; w += gridDim.x * CO_WARPS) {
    int task = w / P, pi = w - task * P;
    int txy = sc.task_txy[task];
    size_t tile = (size_t)(txy >> 16) * sc.tilesX + (txy & 0xffff);
    correlate_pair_warp(sc, cfg, tile, pi, smem[warp], smem[warp] + QBUF, lane,
                        sc.corr + (tile * P + pi) * TP_CORR);
  }
}

// ---------------------------------------------------------------------------
// Stage 3b: disparity extraction, one warp per tile
// ---------------------------------------------------------------------------
// one strip sample of scaleRotateInterpoateSingleCorrelation (Correlation2d.java:610-718)
__device__ __forceinline__ float strip_sample(const float *c, int kind, float bx, float by, int row, int scol,
                                              int down) {
  if (kind <= 3) {
    const int denom = (kind > 1) ? 1 : 2, ilimit = 7 * denom;
    int xnum, ynum;
    if (kind == 0) { xnum = 2 * scol + (row & 1); ynum = down * row; }
    else if (kind == 1) { xnum = down * row; ynum = 2 * scol + (row & 1); }
    else if (kind == 2) { xnum = scol - ((down * row) >> 1); ynum = scol + ((down * row + 1) >> 1); }
    else { xnum = scol - ((down * row) >> 1); ynum = -scol - ((down * row + 1) >> 1); }
    if (xnum > ilimit || xnum < -ilimit || ynum > ilimit || ynum < -ilimit) return CUDART_NAN_F;
    int ix0 = (xnum + ilimit) / denom, iy0 = (ynum + ilimit) / denom;
    bool int_x = (xnum % denom) == 0, int_y = (ynum % denom) == 0;
    if (int_x && int_y) return c[iy0 * 15 + ix0];
    float dx = (xnum + ilimit) / (float)denom - ix0, dy = (ynum + ilimit) / (float)denom - iy0;
    if (int_y) return (1.0f - dx) * c[iy0 * 15 + ix0] + dx * c[iy0 * 15 + ix0 + 1];
    if (int_x) return (1.0f - dy) * c[iy0 * 15 + ix0] + dy * c[(iy0 + 1) * 15 + ix0];
    return ((1.0f - dx) * (1.0f - dy) * c[iy0 * 15 + ix0]) + (dx * (1.0f - dy) * c[iy0 * 15 + ix0 + 1]) +
           ((1.0f - dx) * dy * c[(iy0 + 1) * 15 + ix0]) + (dx * dy * c[(iy0 + 1) * 15 + ix0 + 1]);
  }
  float a = scol + 0.5f * (row & 1), pp = 0.5f * down * row;
  float x = a * bx - pp * by, y = a * by + pp * bx;
  if (x > 7.f || x < -7.f || y > 7.f || y < -7.f) return CUDART_NAN_F;
  float fx = x + 7.f, fy = y + 7.f;
  int ix0 = min((int)floorf(fx), 13), iy0 = min((int)floorf(fy), 13);
  float dx = fx - ix0, dy = fy - iy0;
  return ((1.0f - dx) * (1.0f - dy) * c[iy0 * 15 + ix0]) + (dx * (1.0f - dy) * c[iy0 * 15 + ix0 + 1]) +
         ((1.0f - dx) * dy * c[(iy0 + 1) * 15 + ix0]) + (dx * dy * c[(iy0 + 1) * 15 + ix0 + 1]);
}

#define EX_WARPS 4
__global__ void __launch_bounds__(EX_WARPS * 32) extract_kernel(SceneDev sc) {
  __shared__ float smem[EX_WARPS][TP_CORR + TP_MAX_STRIP * 15 + 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const CorrDev &cfg = *sc.corr_cfg;
  const int P = cfg.num_pairs, rows = cfg.strip_rows, nent = rows * 15;
  const int ntiles = sc.tilesX * sc.tilesY;
  float *cb = smem[warp], *combo = cb + TP_CORR;
  for (int tile = blockIdx.x * EX_WARPS + warp; tile < ntiles; tile += gridDim.x * EX_WARPS) {
    float *dm = sc.disp + (size_t)tile * TP_NDISP;
    if (lane < TP_NDISP)
      dm[lane] = (lane == 2 || lane == 4 || lane == 6) ? 0.0f : CUDART_NAN_F;
    int task = sc.tile_task[tile];
    if (task < 0) continue;
    const float *corr = sc.corr + (size_t)tile * P * TP_CORR;
    // combined strip: product of clipped offset strips (combineInterpolatedCorrelations)
    float prod[8], lsum[8];
    int nanf_[8], zero[8];
#pragma unroll
    for (int t = 0; t < 8; t++) { prod[t] = 1.f; lsum[t] = 0.f; nanf_[t] = 0; zero[t] = 0; }
    for (int pi = 0; pi < P; pi++) {
      const PairDev pd = cfg.pairs[pi];
      if (!pd.in_combo) continue;
      __syncwarp();
      for (int o = lane; o < TP_CORR; o += 32) cb[o] = corr[(size_t)pi * TP_CORR + o];
      __syncwarp();
#pragma unroll
      for (int t = 0; t < 8; t++) {
        int e = lane + 32 * t;
        if (e < nent) {
          int row = e / 15, scol = e - row * 15 - 7;
          float d = strip_sample(cb, pd.kind, pd.bx, pd.by, row, scol, -1);
          if (row > 0) {
            float d2 = strip_sample(cb, pd.kind, pd.bx, pd.by, row, scol, 1);
            d = (isnan(d) || isnan(d2)) ? CUDART_NAN_F : (0.5f * d + 0.5f * d2);
          }
          float v = d + cfg.corr_offset;
          if (v < 0.0f) v = 0.0f;  // NaN passes through as in the reference
          if (isnan(v)) nanf_[t] = 1;
          else if (v == 0.0f) zero[t] = 1;
          else lsum[t] += logf(v);
          prod[t] *= cfg.twice_diagonal ? v * v : v;
        }
      }
    }
    const int ncomb = cfg.twice_diagonal ? 2 * cfg.num_combo : cfg.num_combo;
#pragma unroll
    for (int t = 0; t < 8; t++) {
      int e = lane + 32 * t;
      if (e < nent) {
        float v;
        if (cfg.log_combine) {
          v = nanf_[t] ? CUDART_NAN_F : (zero[t] ? 0.0f : expf(lsum[t] / cfg.num_combo) - cfg.corr_offset);
        } else {
          v = prod[t];
          if (v > 0.0f) v = powf(v, 1.0f / ncomb) - cfg.corr_offset;
        }
        combo[e] = v;
      }
    }
    __syncwarp();
    if (lane == 0) {
      // getMaxXYInt, axis only (Correlation2d.java:802-843)
      int imx = 0;
      for (int i = 1; i < 15; i++)
        if (isnan(combo[imx]) || combo[i] > combo[imx]) imx = i;
      if (combo[imx] >= cfg.min_corr) {
        int ix = imx - 7;
        dm[0] = (float)(-ix);
        dm[2] = combo[imx];
        dm[8] = (float)ix;
        // getMaxXCm (Correlation2d.java:936-1032)
        int dh = rows;
        float wys = 1.0f;
        if (dh > cfg.wndy_size) dh = cfg.wndy_size;
        else if (dh < cfg.wndy_size) {
          float swy = cfg.wndy[0];
          for (int i = 1; i < dh; i++) swy += cfg.wndy[i];
          wys = 1.0f / swy;
        }
        float s0 = 0.f, sx = 0.f, sx2 = 0.f;
        int x0 = 7 + ix;
        for (int dy = 0; dy < dh; dy++) {
          int odd = dy & 1;
          float wy = ((dy == 0) ? wys : 2.0f * wys) * cfg.wndy[dy];
          for (int adx = odd; adx < cfg.wndx_size; adx += 2)
            for (int dir = (adx == 0) ? 1 : -1; dir <= 1; dir += 2) {
              int idx = (adx * dir) >> 1;
              int xx = 2 * idx + odd, x1 = x0 + idx;
              if (x1 >= 0 && x1 < 15) {
                float d = combo[dy * 15 + x1];
                if (!isnan(d) && d > 0.0f) {
                  d *= wy * cfg.wndx[adx];
                  s0 += d;
                  sx += d * xx;
                  sx2 += d * xx * xx;
                }
              }
            }
        }
        if (s0 != 0.0f) {
          dm[1] = -(ix + sx / s0 / 2);
          dm[7] = s0;
        }
      }
    }
    __syncwarp();
    // ortho maxima (getMaxXSOrtho, Correlation2d.java:2502-2651): pass 0 horizontal, 1 vertical
    for (int pass = 0; pass < 2; pass++) {
      int npairs = pass ? cfg.num_vert : cfg.num_hor;
      if (npairs == 0) continue;
      float pr[15];
#pragma unroll
      for (int i = 0; i < 15; i++) pr[i] = 1.f;
      for (int pi = 0; pi < P; pi++) {
        const PairDev pd = cfg.pairs[pi];
        if (pd.kind != pass) continue;
        __syncwarp();
        for (int o = lane; o < TP_CORR; o += 32) cb[o] = corr[(size_t)pi * TP_CORR + o];
        __syncwarp();
        if (lane < 15) {
          int j = lane;
#pragma unroll
          for (int i = 0; i < 15; i++) {
            float d = pass ? 0.5f * (cb[j * 15 + i] + cb[j * 15 + 14 - i]) : 0.5f * (cb[i * 15 + j] + cb[(14 - i) * 15 + j]);
            pr[i] *= d + cfg.corr_offset;
          }
        }
      }
      __syncwarp();
      if (lane < 15) {
        float s = 0.f;
        float w = 1.0f / npairs;
#pragma unroll
        for (int i = 0; i < 15; i++) {
          float v = pr[i];
          v = (v > 0.0f) ? ((npairs == 2) ? sqrtf(v) : ((npairs == 1) ? v : powf(v, w))) - cfg.corr_offset
                         : -cfg.corr_offset;
          s += v * cfg.notch[i];
        }
        combo[TP_MAX_STRIP * 15 + lane] = s;
      }
      __syncwarp();
      if (lane == 0) {
        const float *c1d = combo + TP_MAX_STRIP * 15;
        int ic = 0;
        for (int i = 1; i < 15; i++) if (c1d[i] > c1d[ic]) ic = i;
        float xc = (float)ic;
        if (ic > 0 && ic < 14) {
          float f0 = c1d[ic - 1], f1 = c1d[ic], f2 = c1d[ic + 1];
          float den = f0 - 2.0f * f1 + f2;
          if (den != 0.0f) xc = ic + 0.5f * (f0 - f2) / den;
        }
        int ir = (int)floorf(xc + 0.5f);
        ir = ir < 0 ? 0 : (ir > 14 ? 14 : ir);
        dm[pass ? 5 : 3] = -(xc - 7.0f);
        dm[pass ? 6 : 4] = c1d[ir] / 8.0f;
      }
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------------------
// Stage 4a: IMCLT with overlap-add into the padded frame
// ---------------------------------------------------------------------------
#define IM_WARPS 8
#define IM_REG 8          // output region = 8x8 blocks of 8x8 pixels
#define IM_PX (IM_REG * 8)
#define IM_STRIDE (IM_PX + 1)

// DttRad2.get_unfold_index_signs (392-404): source index and the two signs
__device__ __forceinline__ void unfold_is(int x, int &idx, float &s1, float &s2) {
  int segm = x >> 2, xx = x & 3;
  if (segm == 0) { idx = xx + 4; s1 = 1.f; s2 = 1.f; }
  else if (segm == 1) { idx = 7 - xx; s1 = -1.f; s2 = 1.f; }
  else if (segm == 2) { idx = 3 - xx; s1 = -1.f; s2 = 1.f; }
  else { idx = xx; s1 = -1.f; s2 = -1.f; }
}

__global__ void __launch_bounds__(IM_WARPS * 32) imclt_kernel(SceneDev sc) {
  __shared__ float acc[IM_PX * IM_STRIDE];
  __shared__ float wbuf[IM_WARPS][2 * QBUF];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = sc.num_sensors, C = sc.num_colors;
  const int plane = blockIdx.z, s = plane / C, c = plane - s * C;
  const int bx0 = blockIdx.x * IM_REG, by0 = blockIdx.y * IM_REG;
  const int fw = sc.width + 8, fh = sc.height + 8;
  for (int i = threadIdx.x; i < IM_PX * IM_STRIDE; i += blockDim.x) acc[i] = 0.f;
  __syncthreads();
  float *b1 = wbuf[warp], *b2 = b1 + QBUF;
  const float *lpf = (sc.lpf_rbg && !((sc.clt_lpf_mask >> c) & 1)) ? sc.lpf_rbg + c * 64 : nullptr;
  // tiles touching the region: tx in [bx0-1, bx0+IM_REG-1]
  for (int ph = 0; ph < 4; ph++) {
    const int px_ = ph & 1, py_ = ph >> 1;
    int tx_first = bx0 - 1, ty_first = by0 - 1;
    if ((tx_first & 1) != px_) tx_first++;
    if ((ty_first & 1) != py_) ty_first++;
    const int ntx = (bx0 + IM_REG - 1 - tx_first) / 2 + 1, nty = (by0 + IM_REG - 1 - ty_first) / 2 + 1;
    for (int k = warp; k < ntx * nty; k += IM_WARPS) {
      int tx = tx_first + 2 * (k % ntx), ty = ty_first + 2 * (k / ntx);
      if (tx < 0 || ty < 0 || tx >= sc.tilesX || ty >= sc.tilesY) continue;
      size_t tile = (size_t)ty * sc.tilesX + tx;
      if (sc.tile_task[tile] < 0) continue;
      const float *src = sc.clt + (tile * S + s) * C * TP_CLT + c * TP_CLT;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        int idx = lane + 32 * h;
        float l = 0.25f * (lpf ? lpf[idx] : 1.0f);
        int off = (idx >> 3) * 9 + (idx & 7);
#pragma unroll
        for (int q = 0; q < 4; q++) b1[q * 72 + off] = src[q * 64 + idx] * l;
      }
      __syncwarp();
      // inverse DTT-IV with swapped mode (ImageDtt.java:3628): rows first
      const int m = lane >> 3, r = lane & 7;
      float x[8], y[8];
#pragma unroll
      for (int e = 0; e < 8; e++) x[e] = b1[m * 72 + r * 9 + e];
      dtt4(x, y, (m >> 1) & 1);
#pragma unroll
      for (int j = 0; j < 8; j++) b2[m * 72 + j * 9 + r] = y[j];
      __syncwarp();
#pragma unroll
      for (int e = 0; e < 8; e++) x[e] = b2[m * 72 + r * 9 + e];
      dtt4(x, y, m & 1);
      __syncwarp();
#pragma unroll
      for (int e = 0; e < 8; e++) b1[m * 72 + r * 9 + e] = y[e];  // tile_dct[m][vertical r][horizontal e]
      __syncwarp();
      // unfold (DttRad2.unfold_tile) and accumulate
      const int j = lane & 15;
      int ih;
      float hs1, hs2;
      unfold_is(j, ih, hs1, hs2);
      float hwj = c_hwin[(j < 8) ? j : 15 - j];
      float kh0 = hs1 * hwj, kh1 = hs2 * hwj;
      const int gx = tx * 8 + j - bx0 * 8;
#pragma unroll
      for (int t = 0; t < 8; t++) {
        int i = (lane >> 4) + 2 * t;
        int iv;
        float vs1, vs2;
        unfold_is(i, iv, vs1, vs2);
        float hwi = c_hwin[(i < 8) ? i : 15 - i];
        float kv0 = vs1 * hwi, kv1 = vs2 * hwi;
        int o = iv * 9 + ih;
        float v = (kv0 * kh0) * b1[o] + (kv0 * kh1) * b1[72 + o] + (kv1 * kh0) * b1[144 + o] + (kv1 * kh1) * b1[216 + o];
        int gy = ty * 8 + i - by0 * 8;
        if (gx >= 0 && gx < IM_PX && gy >= 0 && gy < IM_PX) acc[gy * IM_STRIDE + gx] += v;
      }
      __syncwarp();
    }
    __syncthreads();
  }
  float *dst = sc.rbg + (size_t)plane * fw * fh;
  for (int i = threadIdx.x; i < IM_PX * IM_PX; i += blockDim.x) {
    int ly = i / IM_PX, lx = i - ly * IM_PX;
    int gx = bx0 * 8 + lx, gy = by0 * 8 + ly;
    if (gx < fw && gy < fh) dst[(size_t)gy * fw + gx] = acc[ly * IM_STRIDE + lx];
  }
}

// ---------------------------------------------------------------------------
static int grid_for(int items, int per_block) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int need = (items + per_block - 1) / per_block;
  int cap = sms * 16;
  return need < cap ? (need > 0 ? need : 1) : cap;
}

cudaError_t launch_convert_correct(const SceneDev &sc, cudaStream_t st) {
  int n = sc.num_tasks * sc.num_sensors * sc.num_colors;
  if (n <= 0) return cudaSuccess;
  convert_correct_kernel<<<grid_for(n, CC_WARPS), CC_WARPS * 32, 0, st>>>(sc);
  return cudaGetLastError();
}

cudaError_t launch_correlate(const SceneDev &sc, cudaStream_t st) {
  int n = sc.num_tasks * sc.num_pairs;
  if (n <= 0) return cudaSuccess;
  correlate_kernel<<<grid_for(n, CO_WARPS), CO_WARPS * 32, 0, st>>>(sc);
  return cudaGetLastError();
}

cudaError_t launch_extract(const SceneDev &sc, cudaStream_t st) {
  int n = sc.tilesX * sc.tilesY;
  extract_kernel<<<grid_for(n, EX_WARPS), EX_WARPS * 32, 0, st>>>(sc);
  return cudaGetLastError();
}

cudaError_t launch_imclt(const SceneDev &sc, cudaStream_t st) {
  dim3 grid((sc.tilesX + 1 + IM_REG - 1) / IM_REG, (sc.tilesY + 1 + IM_REG - 1) / IM_REG,
            sc.num_sensors * sc.num_colors);
  imclt_kernel<<<grid, IM_WARPS * 32, 0, st>>>(sc);
  return cudaGetLastError();
}
