// tp_dtt.cuh -- 8-point DTT butterflies and window helpers shared by the tile kernels.
//
// Each translation unit that includes this header owns its own copy of the
// __constant__ tables and must call upload_dtt_constants() once (the launchers'
// constant upload does).  Transforms follow DttRad2 (DttRad2.java:80-98,
// 503-519, 595-666, 1107-1146); windows follow set_window mode 1 (674-694).
#pragma once
#include <math_constants.h>

#include <cmath>
#include <cstdint>

#include "tp_internal.h"

namespace {

__constant__ float k_hwin[8];      // sine half-window
__constant__ float k_dct2e[64];    // CIIe (used for the odd half of DCT-IIe)
__constant__ float k_d4c[4], k_d4s[4];  // scaled DCT-IV stage-1 rotations

// ---------------------------------------------------------------------------
// 8-point transforms
// ---------------------------------------------------------------------------
// orthonormal DCT-IV (Plonka-Tasche recursion as in DttRad2._dctiv_recurs)
__device__ __forceinline__ void dct4_fast(const float x[8], float y[8]) {
  const float C18 = 1.3065629648763766f, C38 = 0.5411961001461970f, SQ2 = 1.4142135623730951f;
  float u0[4], u1[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    u0[j] = fmaf(k_d4c[j], x[j], k_d4s[j] * x[7 - j]);
    float t = fmaf(k_d4c[3 - j], x[4 + j], -k_d4s[3 - j] * x[3 - j]);
    u1[j] = (j & 1) ? -t : t;
  }
  float v0[4], v1[4];
  {
    float a0 = u0[0] + u0[3], a1 = u0[1] + u0[2], b0 = u0[0] - u0[3], b1 = u0[1] - u0[2];
    v0[0] = a0 + a1; v0[2] = a0 - a1;
    v0[1] = fmaf(C18, b0, C38 * b1); v0[3] = fmaf(C38, b0, -C18 * b1);
  }
  {
    float a0 = u1[0] + u1[3], a1 = u1[1] + u1[2], b0 = u1[0] - u1[3], b1 = u1[1] - u1[2];
    v1[0] = a0 + a1; v1[2] = a0 - a1;
    v1[1] = fmaf(C18, b0, C38 * b1); v1[3] = fmaf(C38, b0, -C18 * b1);
  }
  y[0] = SQ2 * v0[0];
  y[7] = SQ2 * v1[0];
  y[2] = v0[1] + v1[3];  // w0[1] = v0[1] - (-1) v1[3]
  y[4] = v0[2] - v1[2];  // w0[2]
  y[6] = v0[3] + v1[1];  // w0[3]
  y[1] = v0[1] - v1[3];  // w1[0]
  y[3] = v0[2] + v1[2];  // w1[1]
  y[5] = v0[3] - v1[1];  // w1[2]
}
__device__ __forceinline__ void dtt4_fast(const float x[8], float y[8], bool sine) {
  float xr[8];
#pragma unroll
  for (int n = 0; n < 8; n++) xr[n] = sine ? x[7 - n] : x[n];
  dct4_fast(xr, y);
#pragma unroll
  for (int k = 1; k < 8; k += 2) y[k] = sine ? -y[k] : y[k];
}
// DCT-IIe (CIIe rows); DST-IIe via SIIe[j][k] = (-1)^k CIIe[7-j][k]
__device__ __forceinline__ void dtt2e_fast(const float x[8], float y[8], bool sine) {
  const float S = 0.5f;  // sqrt(2/8)
  const float C4 = 0.7071067811865476f, C8 = 0.9238795325112867f, C38 = 0.3826834323650898f;
  float xs[8];
#pragma unroll
  for (int n = 0; n < 8; n++) xs[n] = (sine && (n & 1)) ? -x[n] : x[n];
  float u0[4], u1[4];
#pragma unroll
  for (int j = 0; j < 4; j++) { u0[j] = xs[j] + xs[7 - j]; u1[j] = xs[j] - xs[7 - j]; }
  float a0 = u0[0] + u0[3], a1 = u0[1] + u0[2], b0 = u0[0] - u0[3], b1 = u0[1] - u0[2];
  float t[8];
  t[0] = S * (a0 + a1);
  t[4] = (S * C4) * (a0 - a1);
  t[2] = S * fmaf(C8, b0, C38 * b1);
  t[6] = S * fmaf(C38, b0, -C8 * b1);
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int k = 2 * j + 1;  // rows of CIIe for odd outputs, columns 0..3 (x[k]-x[7-k] symmetric)
    t[k] = fmaf(k_dct2e[k * 8 + 0], u1[0], fmaf(k_dct2e[k * 8 + 1], u1[1], fmaf(k_dct2e[k * 8 + 2], u1[2],
                k_dct2e[k * 8 + 3] * u1[3])));
  }
#pragma unroll
  for (int j = 0; j < 8; j++) y[j] = sine ? t[7 - j] : t[j];
}

struct FoldIdx {
  int src0, win0, dwin0, src1, win1, dwin1;
  float sc0, ss0, ds0, sc1, ss1, ds1;
};
// DttRad2.get_fold_indices (DttRad2.java:109-144), n = 8
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

__device__ __forceinline__ int mirror(int p, int n) {
  if (p < 0) return p & 1;
  if (p >= n) return n - 2 + (p & 1);
  return p;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// one pixel of the window: (row, col) relative to the window corner
struct Win {
  const void *img;
  int64_t pitch;
  int tlx, tly, W, H, u16, inside;
  float scale;
  __device__ __forceinline__ float at(int row, int col) const {
    int y = tly + row, x = tlx + col;
    if (!inside) { y = mirror(y, H); x = mirror(x, W); }
    size_t o = (size_t)y * pitch + x;
    float v = u16 ? (float)__ldg((const uint16_t *)img + o) : __ldg((const float *)img + o);
    return v * scale;
  }
};

// transpose of an 8x8 block held as one row per lane of an 8-lane group
__device__ __forceinline__ void group_transpose(float v[8], float *buf, int r) {
#pragma unroll
  for (int j = 0; j < 8; j++) buf[j * 9 + r] = v[j];
  __syncwarp();
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = buf[r * 9 + i];
  __syncwarp();
}

// fold weights of the shifted sine window (DttRad2.get_shifted_fold_2d, 263-314):
// (hc, hs) / (vc, vs) are the cosine / sine of pi/16 x the horizontal / vertical
// shift, or their derivatives (the weights are linear in them)
__device__ __forceinline__ void fold_weights(float hc, float hs, float vc, float vs, const FoldIdx &fv,
                                             float &vw0, float &vw1, float hw0[8], float hw1[8]) {
  vw0 = vc * k_hwin[fv.win0] + vs * k_hwin[fv.dwin0] * fv.ds0;
  vw1 = vc * k_hwin[fv.win1] + vs * k_hwin[fv.dwin1] * fv.ds1;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const FoldIdx fh = fold_idx(j);
    hw0[j] = hc * k_hwin[fh.win0] + hs * k_hwin[fh.dwin0] * fh.ds0;
    hw1[j] = hc * k_hwin[fh.win1] + hs * k_hwin[fh.dwin1] * fh.ds1;
  }
}

// fold of a dense 16x16 window and the four 2D DCT-IV/DST-IV (fold_tile, dttt_iv):
// lane r of the 8-lane group holds horizontal frequency r of each quadrant, o[m][v];
// PIX: the pixel source, at(row, col)
template <typename PIX = Win>
__device__ __forceinline__ void fold_dtt_dense(const PIX &w, const FoldIdx &fv, float vw0, float vw1,
                                               const float hw0[8], const float hw1[8], int r, float *tbuf,
                                               float o[4][8]) {
  // the lane's two source rows, read once for both vertical variants
  float p0[16], p1[16];
#pragma unroll
  for (int cix = 0; cix < 16; cix++) {
    p0[cix] = w.at(fv.src0, cix);
    p1[cix] = w.at(fv.src1, cix);
  }
  // vertical 2-tap combine once, then the two horizontal variants
#pragma unroll
  for (int vb = 0; vb < 2; vb++) {
    const float k0 = (vb ? fv.ss0 : fv.sc0) * vw0, k1 = (vb ? fv.ss1 : fv.sc1) * vw1;
    float vc[16];
#pragma unroll
    for (int cix = 0; cix < 16; cix++) vc[cix] = fmaf(k1, p1[cix], k0 * p0[cix]);
#pragma unroll
    for (int hb = 0; hb < 2; hb++) {
      float y[8];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const FoldIdx fh = fold_idx(j);
        const float h0 = (hb ? fh.ss0 : fh.sc0) * hw0[j], h1 = (hb ? fh.ss1 : fh.sc1) * hw1[j];
        y[j] = fmaf(h1, vc[fh.src1], h0 * vc[fh.src0]);
      }
      float z[8];
      dtt4_fast(y, z, hb);
      group_transpose(z, tbuf, r);
      dtt4_fast(z, o[vb * 2 + hb], vb);
    }
  }
}

// ---------------------------------------------------------------------------
// strip samples of a 15x15 correlation surface (Correlation2d.java:610-718)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float strip_sample(const float *c, int kind, float bx, float by, int row, int scol, int down) {
  if (kind <= 3) {
    const int sh = (kind > 1) ? 0 : 1, ilimit = 7 << sh;  // denom = 1 << sh
    int xnum, ynum;
    if (kind == 0) { xnum = 2 * scol + (row & 1); ynum = down * row; }
    else if (kind == 1) { xnum = down * row; ynum = 2 * scol + (row & 1); }
    else if (kind == 2) { xnum = scol - ((down * row) >> 1); ynum = scol + ((down * row + 1) >> 1); }
    else { xnum = scol - ((down * row) >> 1); ynum = -scol - ((down * row + 1) >> 1); }
    if (xnum > ilimit || xnum < -ilimit || ynum > ilimit || ynum < -ilimit) return CUDART_NAN_F;
    const int ix0 = (xnum + ilimit) >> sh, iy0 = (ynum + ilimit) >> sh;
    const bool int_x = (xnum & ((1 << sh) - 1)) == 0, int_y = (ynum & ((1 << sh) - 1)) == 0;
    if (int_x && int_y) return c[iy0 * 15 + ix0];
    const float dx = int_x ? 0.f : 0.5f, dy = int_y ? 0.f : 0.5f;
    if (int_y) return (1.0f - dx) * c[iy0 * 15 + ix0] + dx * c[iy0 * 15 + ix0 + 1];
    if (int_x) return (1.0f - dy) * c[iy0 * 15 + ix0] + dy * c[(iy0 + 1) * 15 + ix0];
    return ((1.0f - dx) * (1.0f - dy) * c[iy0 * 15 + ix0]) + (dx * (1.0f - dy) * c[iy0 * 15 + ix0 + 1]) +
           ((1.0f - dx) * dy * c[(iy0 + 1) * 15 + ix0]) + (dx * dy * c[(iy0 + 1) * 15 + ix0 + 1]);
  }
  const float a = scol + 0.5f * (row & 1), pp = 0.5f * down * row;
  const float x = a * bx - pp * by, y = a * by + pp * bx;
  if (x > 7.f || x < -7.f || y > 7.f || y < -7.f) return CUDART_NAN_F;
  const float fx = x + 7.f, fy = y + 7.f;
  const int ix0 = min((int)floorf(fx), 13), iy0 = min((int)floorf(fy), 13);
  const float dx = fx - ix0, dy = fy - iy0;
  return ((1.0f - dx) * (1.0f - dy) * c[iy0 * 15 + ix0]) + (dx * (1.0f - dy) * c[iy0 * 15 + ix0 + 1]) +
         ((1.0f - dx) * dy * c[(iy0 + 1) * 15 + ix0]) + (dx * dy * c[(iy0 + 1) * 15 + ix0 + 1]);
}

// one strip sample from a precomputed code (quad kinds): same arithmetic as
// Correlation2d.java:664-690 with dx, dy in {0, 0.5}
__device__ __forceinline__ float sample_code(const float *c, int code) {
  if (code < 0) return CUDART_NAN_F;
  const int idx = code & 255, cs = code >> 8;
  const float v = c[idx];
  if (cs == 0) return v;
  if (cs == 1) return 0.5f * v + 0.5f * c[idx + 1];
  if (cs == 2) return 0.5f * v + 0.5f * c[idx + 15];
  return ((0.25f * v + 0.25f * c[idx + 1]) + 0.25f * c[idx + 15]) + 0.25f * c[idx + 16];
}

cudaError_t upload_dtt_constants() {
  float hw[8], d2[64], c4[4], s4[4];
  const double pi = 3.14159265358979323846, sc = 1.0 / std::sqrt(8.0);
  for (int i = 0; i < 8; i++) hw[i] = (float)std::sin(pi / 16.0 * (i + 0.5));
  for (int k = 0; k < 8; k++)
    for (int n = 0; n < 8; n++) d2[k * 8 + n] = (float)(std::sqrt(2.0 / 8) * std::cos(pi * k * (2 * n + 1) / 16.0));
  for (int k = 0; k < 4; k++) {
    c4[k] = (float)(sc * std::cos((2 * k + 1) * pi / 32));
    s4[k] = (float)(sc * std::sin((2 * k + 1) * pi / 32));
  }
  cudaError_t e = cudaMemcpyToSymbol(k_hwin, hw, sizeof(hw));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(k_dct2e, d2, sizeof(d2));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(k_d4c, c4, sizeof(c4));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(k_d4s, s4, sizeof(s4));
  return e;
}

}  // namespace
