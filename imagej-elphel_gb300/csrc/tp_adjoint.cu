// tp_adjoint.cu -- hand-written adjoint of the forward chain (mono and Bayer colour sensors).
//
// For every tile the centroid disparity d (getMaxXCm over the combined strip,
// Correlation2d.java:936-1032) is a function of the residual shifts (rx, ry)
// of each sensor's window (ImageDtt.java:4940-4943), which follow the port
// coordinates, which follow the per-sensor extrinsics and the tile's target
// disparity (GeometryCorrection.getPortsCoordinatesAndDerivatives,
// GeometryCorrection.java:2159-2314).  The adjoint kernel computes, per tile,
// d and dd/d(port x, port y) of every sensor by reverse mode through
//   centroid -> strip combination (geometric mean) -> strip sampling ->
//   15x15 unfold -> 2D DCT-IIe/DST-IIe -> LPF -> fat-zero normalised product
// (Correlation2d.java:197-231, 556-790; DttRad2.java:443-489, 595-614) down to
// dd/dCLT of each sensor, then by forward mode through the CLT's dependence
// on the residual shift: the phase rotation (fract_shift, ImageDtt.java:
// 5490-5584) differentiated analytically, and the shifted fold window
// (DttRad2.get_shifted_fold_2d, 263-314) differentiated through its cos/sin
// mix.  The integer window corners and the integer argmax are piecewise
// constant and are held fixed.
//
// A second kernel contracts those port sensitivities with the FP64 port
// derivatives of the plan (azimuth, tilt, roll, zoom, disparity) into the
// per-tile Jacobian rows and the gradient of a per-tile loss.
//
// GB300 layout: one CTA of four warps per tile.  The tile's CLT [S][256]
// (read back from HBM or recomputed from the image) and its gradient [S][256]
// live in shared memory; warp 0 takes the centroid of the combined strip the
// forward kernel kept; then the warps split the pairs, each running a pair's
// reverse chain in registers and per-warp buffers (the transposed DCT-IIe is
// the transposed butterfly of the forward one) and adding into the gradient;
// the pairs go in rounds of four on distinct sensors (scheduled on the host),
// a barrier between rounds, so the gradient sums over the pairs are taken in a
// fixed order without atomics (a pair's strip taps go into its own 15x15
// gradient with one warp's shared-memory atomics); finally the warps split the
// sensors for the forward-mode shift derivatives.
#include "tp_dtt.cuh"

namespace {

constexpr float K16 = 0.19634954084936207f;  // pi / 16

struct AdjShape {
  int S, C, P, RE;
  int per_warp;   // floats of shared memory per warp
  int recompute;  // 1: recompute the CLT from the image instead of reading it back
  int use_strips; // 1: the forward recorded its per-pair strip samples in sc.strips
};

__device__ __forceinline__ void convolve(float o[4][8], const float *kp, int r) {
  if (!kp) return;
  float k[4][8];
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const float4 *p = (const float4 *)(kp + m * 64 + r * 8);
    const float4 a = __ldg(p), b = __ldg(p + 1);
    k[m][0] = a.x; k[m][1] = a.y; k[m][2] = a.z; k[m][3] = a.w;
    k[m][4] = b.x; k[m][5] = b.y; k[m][6] = b.z; k[m][7] = b.w;
  }
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const float d0 = o[0][v], d1 = o[1][v], d2 = o[2][v], d3 = o[3][v];
    const float k0 = k[0][v], k1 = k[1][v], k2 = k[2][v], k3 = k[3][v];
    o[0][v] = d0 * k0 - d1 * k1 - d2 * k2 + d3 * k3;
    o[1][v] = d1 * k0 + d0 * k1 - d3 * k2 - d2 * k3;
    o[2][v] = d2 * k0 - d3 * k1 + d0 * k2 - d1 * k3;
    o[3][v] = d3 * k0 + d2 * k1 + d1 * k2 + d0 * k3;
  }
}

// the phase rotation of fract_shift (same angles as the forward kernel)
__device__ __forceinline__ void rotate(float o[4][8], float rx, float ry, int r) {
  float ch, shh, cvr, svr;
  __sincosf(CUDART_PI_F * 0.0625f * (2 * r + 1) * rx, &shh, &ch);
  __sincosf(CUDART_PI_F * 0.0625f * (2 * r + 1) * ry, &svr, &cvr);
  const int base = threadIdx.x & 24;
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const float cv = __shfl_sync(0xffffffffu, cvr, base + v), sv = __shfl_sync(0xffffffffu, svr, base + v);
    const float t0 = o[0][v] * ch - o[1][v] * shh, t1 = o[1][v] * ch + o[0][v] * shh;
    const float t2 = o[2][v] * ch - o[3][v] * shh, t3 = o[3][v] * ch + o[2][v] * shh;
    o[0][v] = t0 * cv - t2 * sv;
    o[2][v] = t2 * cv + t0 * sv;
    o[1][v] = t1 * cv - t3 * sv;
    o[3][v] = t3 * cv + t1 * sv;
  }
}

// transpose of rotate (both turns are orthogonal: undone in reverse order)
__device__ __forceinline__ void rotate_t(float o[4][8], float rx, float ry, int r) {
  float ch, shh, cvr, svr;
  __sincosf(CUDART_PI_F * 0.0625f * (2 * r + 1) * rx, &shh, &ch);
  __sincosf(CUDART_PI_F * 0.0625f * (2 * r + 1) * ry, &svr, &cvr);
  const int base = threadIdx.x & 24;
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const float cv = __shfl_sync(0xffffffffu, cvr, base + v), sv = __shfl_sync(0xffffffffu, svr, base + v);
    const float t0 = o[0][v] * cv + o[2][v] * sv, t2 = o[2][v] * cv - o[0][v] * sv;
    const float t1 = o[1][v] * cv + o[3][v] * sv, t3 = o[3][v] * cv - o[1][v] * sv;
    o[0][v] = t0 * ch + t1 * shh;
    o[1][v] = t1 * ch - t0 * shh;
    o[2][v] = t2 * ch + t3 * shh;
    o[3][v] = t3 * ch - t2 * shh;
  }
}

// transpose of convolve (the per-frequency 4x4 sign matrix of the kernel, transposed)
__device__ __forceinline__ void convolve_t(float o[4][8], const float *kp, int r) {
  if (!kp) return;
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const float k0 = __ldg(kp + r * 8 + v), k1 = __ldg(kp + 64 + r * 8 + v), k2 = __ldg(kp + 128 + r * 8 + v),
                k3 = __ldg(kp + 192 + r * 8 + v);
    const float g0 = o[0][v], g1 = o[1][v], g2 = o[2][v], g3 = o[3][v];
    o[0][v] = k0 * g0 + k1 * g1 + k2 * g2 + k3 * g3;
    o[1][v] = -k1 * g0 + k0 * g1 - k3 * g2 + k2 * g3;
    o[2][v] = -k2 * g0 - k3 * g1 + k0 * g2 + k1 * g3;
    o[3][v] = k3 * g0 - k2 * g1 - k1 * g2 + k0 * g3;
  }
}

__device__ __forceinline__ Win make_win(const SceneDev &sc, const SubtilePlan &p, int s, int c = 0) {
  Win w;
  w.img = sc.images[s];
  w.pitch = sc.img_pitch;
  w.tlx = p.tlx; w.tly = p.tly; w.W = sc.width; w.H = sc.height;
  w.u16 = sc.img_dtype[s];
  w.inside = (p.tlx >= 0) && (p.tly >= 0) && (p.tlx <= sc.width - 16) && (p.tly <= sc.height - 16);
  w.scale = sc.color_scale[c];
  return w;
}

// one colour plane of a Bayer mosaic seen through a window: the mosaic's pixels of colour c
// (0 red, 1 blue, 2 green, on the Bayer phase (red row, red column)), zero elsewhere -- the
// sparse plane the forward transforms (the mirrored border keeps the pixel parity)
struct BayerWin {
  Win w;
  int c, rr, rc;
  __device__ __forceinline__ float at(int row, int col) const {
    const bool ry = ((w.tly + row) & 1) == rr, rx = ((w.tlx + col) & 1) == rc;
    const bool keep = (c == 0) ? (ry && rx) : ((c == 1) ? (!ry && !rx) : (ry != rx));
    return keep ? w.at(row, col) : 0.f;
  }
};

// taps of one strip sample (sample_code / strip_sample): returns the tap count
__device__ __forceinline__ int code_taps(int code, int idx[4], float wt[4]) {
  if (code < 0) return 0;
  const int i = code & 255, cs = code >> 8;
  idx[0] = i;
  if (cs == 0) { wt[0] = 1.f; return 1; }
  if (cs == 1) { wt[0] = 0.5f; idx[1] = i + 1; wt[1] = 0.5f; return 2; }
  if (cs == 2) { wt[0] = 0.5f; idx[1] = i + 15; wt[1] = 0.5f; return 2; }
  idx[1] = i + 1; idx[2] = i + 15; idx[3] = i + 16;
  wt[0] = wt[1] = wt[2] = wt[3] = 0.25f;
  return 4;
}
__device__ __forceinline__ int general_taps(float bx, float by, int row, int scol, int down, int idx[4],
                                            float wt[4]) {
  const float a = scol + 0.5f * (row & 1), pp = 0.5f * down * row;
  const float x = a * bx - pp * by, y = a * by + pp * bx;
  if (x > 7.f || x < -7.f || y > 7.f || y < -7.f) return 0;
  const float fx = x + 7.f, fy = y + 7.f;
  const int ix0 = min((int)floorf(fx), 13), iy0 = min((int)floorf(fy), 13);
  const float dx = fx - ix0, dy = fy - iy0;
  idx[0] = iy0 * 15 + ix0; wt[0] = (1.0f - dx) * (1.0f - dy);
  idx[1] = idx[0] + 1;     wt[1] = dx * (1.0f - dy);
  idx[2] = idx[0] + 15;    wt[2] = (1.0f - dx) * dy;
  idx[3] = idx[0] + 16;    wt[3] = dx * dy;
  return 4;
}

// one strip entry of a pair exactly as the forward kernel computes it
__device__ __forceinline__ float strip_entry(const float *c, const short *strip_code, const PairDev &pd, int e) {
  const int row = e / 15;
  float d;
  if (pd.kind <= 3) {
    const short2 code = *(const short2 *)&strip_code[(pd.kind * TP_MAX_STRIP * 15 + e) * 2];
    d = sample_code(c, code.x);
    if (row > 0) {
      const float d2 = sample_code(c, code.y);
      d = (isnan(d) || isnan(d2)) ? CUDART_NAN_F : (0.5f * d + 0.5f * d2);
    }
  } else {
    const int scol = e - row * 15 - 7;
    d = strip_sample(c, 4, pd.bx, pd.by, row, scol, -1);
    if (row > 0) {
      const float d2 = strip_sample(c, 4, pd.bx, pd.by, row, scol, 1);
      d = (isnan(d) || isnan(d2)) ? CUDART_NAN_F : (0.5f * d + 0.5f * d2);
    }
  }
  return d;
}

}  // namespace

constexpr int AD_NW = 4;  // warps per tile

// dd/d(port x, port y) of one (sensor, colour) sub-tile, 8-lane group (lane r holds row r):
// the dd/dCLT gl of the sub-tile is taken back once through the phase rotation, the kernel
// convolution and the 2D DCT-IV/DST-IV (symmetric transforms: the transpose runs through the same
// butterflies) to the folded tile, which is dotted with the fold of the pixels under the
// derivative window, one fold per direction, plus the rotation's own derivative.  gl is
// overwritten (with the folded gradient) where `own` is set.  Result in out[] of every lane.
template <typename PIX>
__device__ __forceinline__ void shift_sens(const SceneDev &sc, const PIX &w, const SubtilePlan &p, int s,
                                           const float *clt, float *gl_all, float *tbq, int r, bool own,
                                           float out[2]) {
  const float *kp = (p.kidx >= 0) ? sc.kernels[s] + (size_t)p.kidx * TP_CLT : nullptr;
  float ahs, ahc, avs, avc;
  __sincosf(CUDART_PI_F * 0.0625f * p.rx, &ahs, &ahc);
  __sincosf(CUDART_PI_F * 0.0625f * p.ry, &avs, &avc);
  const FoldIdx fv = fold_idx(r);
  const float *cl = clt + r * 8, *gl = gl_all + r * 8;
  // the rotation's own derivative (pi/16 (2k+1) x the CLT turned by 90 degrees) dotted with dd/dCLT
  float gdir[2] = {0.f, 0.f};
#pragma unroll
  for (int v = 0; v < 8; v++) {
    const float c0 = cl[v], c1 = cl[64 + v], c2 = cl[128 + v], c3 = cl[192 + v];
    const float g0 = gl[v], g1 = gl[64 + v], g2 = gl[128 + v], g3 = gl[192 + v];
    const float fx = K16 * (2 * r + 1), fy = K16 * (2 * v + 1);
    gdir[0] = fmaf(fx, (g1 * c0 - g0 * c1) + (g3 * c2 - g2 * c3), gdir[0]);
    gdir[1] = fmaf(fy, (g2 * c0 - g0 * c2) + (g3 * c1 - g1 * c3), gdir[1]);
  }
  float *gfs = gl_all + r * 8;  // gfs[m * 64 + j] for folded row r
  {
    float gf[4][8];
#pragma unroll
    for (int m = 0; m < 4; m++)
#pragma unroll
      for (int v = 0; v < 8; v++) gf[m][v] = gl[m * 64 + v];
    rotate_t(gf, p.rx, p.ry, r);
    convolve_t(gf, kp, r);
#pragma unroll
    for (int m = 0; m < 4; m++) {
      float u[8];
      dtt4_fast(gf[m], u, (m >> 1) & 1);
      group_transpose(u, tbq, r);
      dtt4_fast(u, gf[m], m & 1);
    }
    if (own) {
#pragma unroll
      for (int m = 0; m < 4; m++)
#pragma unroll
        for (int j2 = 0; j2 < 8; j2++) gfs[m * 64 + j2] = gf[m][j2];
    }
  }
  __syncwarp();
  // the lane's two source rows of the window, read once for both directions and both vertical
  // variants
  float p0[16], p1[16];
#pragma unroll
  for (int cix = 0; cix < 16; cix++) {
    p0[cix] = w.at(fv.src0, cix);
    p1[cix] = w.at(fv.src1, cix);
  }
  // per direction: the fold with the derivative window dotted with the folded gradient
#pragma unroll
  for (int dir = 0; dir < 2; dir++) {
    float vw0, vw1, hw0[8], hw1[8];
    if (dir == 0) fold_weights(-K16 * ahs, K16 * ahc, avc, avs, fv, vw0, vw1, hw0, hw1);
    else fold_weights(ahc, ahs, -K16 * avs, K16 * avc, fv, vw0, vw1, hw0, hw1);
    float acc = 0.f;
#pragma unroll
    for (int vb = 0; vb < 2; vb++) {
      const float k0 = (vb ? fv.ss0 : fv.sc0) * vw0, k1 = (vb ? fv.ss1 : fv.sc1) * vw1;
      float vc[16];
#pragma unroll
      for (int cix = 0; cix < 16; cix++) vc[cix] = fmaf(k1, p1[cix], k0 * p0[cix]);
#pragma unroll
      for (int hb = 0; hb < 2; hb++)
#pragma unroll
        for (int j2 = 0; j2 < 8; j2++) {
          const FoldIdx fh = fold_idx(j2);
          const float h0 = (hb ? fh.ss0 : fh.sc0) * hw0[j2], h1 = (hb ? fh.ss1 : fh.sc1) * hw1[j2];
          acc = fmaf(fmaf(h1, vc[fh.src1], h0 * vc[fh.src0]), gfs[(vb * 2 + hb) * 64 + j2], acc);
        }
    }
    gdir[dir] += acc;
  }
#pragma unroll
  for (int dir = 0; dir < 2; dir++) {
    gdir[dir] += __shfl_xor_sync(0xffffffffu, gdir[dir], 1);
    gdir[dir] += __shfl_xor_sync(0xffffffffu, gdir[dir], 2);
    gdir[dir] += __shfl_xor_sync(0xffffffffu, gdir[dir], 4);
  }
  // residual = TL - px: dd/dpx = -dd/drx; the kernel-centre offsets add the dependence of px, py
  // on the port through kdx, kdy (ImageDtt.java:4930-4939)
  const float gpx = -gdir[0], gpy = -gdir[1];
  out[0] = gpx;
  out[1] = gpy;
  if (p.kidx >= 0) {
    const float4 e1 = __ldg((const float4 *)(sc.kext[s] + (size_t)p.kidx * 8) + 1);
    out[0] = gpx * (1.0f - e1.x) - gpy * e1.z;
    out[1] = -gpx * e1.y + gpy * (1.0f - e1.w);
  }
}

// x = T^T y for the DCT-IIe / DST-IIe of dtt2e_fast (its transposed data flow)
__device__ __forceinline__ void dtt2e_transposed(const float y[8], float x[8], bool sine) {
  const float S = 0.5f;
  const float C4 = 0.7071067811865476f, C8 = 0.9238795325112867f, C38 = 0.3826834323650898f;
  float t[8];
#pragma unroll
  for (int k = 0; k < 8; k++) t[k] = sine ? y[7 - k] : y[k];
  float u1[4];
#pragma unroll
  for (int j = 0; j < 4; j++)
    u1[j] = fmaf(k_dct2e[8 + j], t[1], fmaf(k_dct2e[24 + j], t[3], fmaf(k_dct2e[40 + j], t[5], k_dct2e[56 + j] * t[7])));
  const float a0 = S * t[0] + (S * C4) * t[4], a1 = S * t[0] - (S * C4) * t[4];
  const float b0 = S * fmaf(C8, t[2], C38 * t[6]), b1 = S * fmaf(C38, t[2], -C8 * t[6]);
  const float u0[4] = {a0 + b0, a1 + b1, a1 - b1, a0 - b0};
#pragma unroll
  for (int j = 0; j < 4; j++) {
    x[j] = u0[j] + u1[j];
    x[7 - j] = u0[j] - u1[j];
  }
  if (sine) {
#pragma unroll
    for (int n = 1; n < 8; n += 2) x[n] = -x[n];
  }
}

__global__ void __launch_bounds__(32 * AD_NW, 4) adjoint_kernel(const __grid_constant__ SceneDev sc,
                                                             const __grid_constant__ AdjShape as,
                                                             const __grid_constant__ CorrConst cfg, float *sens,
                                                             float *dval) {
  extern __shared__ float sm[];
  __shared__ float s_d;
  __shared__ float s_sens[2 * TP_MAXS * 3];  // dd/d(port x, y) of every (sensor, colour)
  __shared__ float s_lpf[64];                // the correlation LPF, read per lane
  for (int i = threadIdx.x; i < 64; i += blockDim.x) s_lpf[i] = cfg.lpf[i];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, q = lane >> 3, r = lane & 7;
  const int S = as.S, C = as.C, P = as.P, RE = as.RE;
  float *s_clt = sm;                      // [S][C][256]
  float *s_g = s_clt + S * C * TP_CLT;    // [S][C][256] dd/dCLT
  float *gcmb = s_g + S * C * TP_CLT;     // [240] dd/dcombo
  float *gG = gcmb + 240;             // [240] combo + offset
  float *gs = gG + 240 + warp * 816;  // per warp: [240] dd/dsurface of the current pair
  float *qb = gs + 240;               // [4][72] quadrant buffer
  float *tb = qb + 288;               // [4][72] transpose buffer
  const short *strip_code = &sc.corr_cfg->strip_code[0][0][0];
  const float inv_n = 1.0f / cfg.num_combo;

  for (int task = blockIdx.x; task < sc.num_tasks; task += gridDim.x) {
    const int txy = sc.task_txy[task];
    const size_t tile = (size_t)(txy >> 16) * sc.tilesX + (txy & 0xffff);
    // ---------------- the tile's CLT ----------------
    if (as.recompute) {
      // every (sensor, colour) item, four per 8-lane group: a Bayer colour as the sparse plane of
      // its pixels (the dense fold of the masked window is the forward's CLT of that plane)
      const int items = S * C;
      for (int g = warp; g < (items + 3) / 4; g += AD_NW) {
        const int it = g * 4 + q;
        const int itc = it < items ? it : items - 1;
        const int s = itc / C, c = itc - s * C;
        const SubtilePlan p = sc.plan[(size_t)task * items + itc];
        float ahs, ahc, avs, avc;
        __sincosf(CUDART_PI_F * 0.0625f * p.rx, &ahs, &ahc);
        __sincosf(CUDART_PI_F * 0.0625f * p.ry, &avs, &avc);
        const FoldIdx fv = fold_idx(r);
        float vw0, vw1, hw0[8], hw1[8], o[4][8];
        fold_weights(ahc, ahs, avc, avs, fv, vw0, vw1, hw0, hw1);
        if (C == 1) {
          fold_dtt_dense(make_win(sc, p, s), fv, vw0, vw1, hw0, hw1, r, tb + q * 72, o);
        } else {
          BayerWin bw;
          bw.w = make_win(sc, p, s, c);
          bw.c = c;
          bw.rr = sc.bayer_red_row;
          bw.rc = sc.bayer_red_col;
          fold_dtt_dense(bw, fv, vw0, vw1, hw0, hw1, r, tb + q * 72, o);
        }
        convolve(o, (p.kidx >= 0) ? sc.kernels[s] + (size_t)p.kidx * TP_CLT : nullptr, r);
        rotate(o, p.rx, p.ry, r);
        if (it < items) {
#pragma unroll
          for (int m = 0; m < 4; m++)
#pragma unroll
            for (int v = 0; v < 8; v++) s_clt[it * TP_CLT + m * 64 + r * 8 + v] = o[m][v];
        }
      }
    } else {
      const float4 *src = (const float4 *)(sc.clt + tile * S * C * TP_CLT);
      for (int i = tid; i < S * C * 64; i += 32 * AD_NW) ((float4 *)s_clt)[i] = __ldg(src + i);
    }
    for (int i = tid; i < S * C * TP_CLT; i += 32 * AD_NW) s_g[i] = 0.f;

    // ---------------- centroid of the forward's combined strip, and dd/dcombo ----------------
    if (warp == 0) {
      for (int e = lane; e < 240; e += 32) {
        gG[e] = (e < RE) ? sc.combo[tile * RE + e] : 0.f;
        gcmb[e] = 0.f;
      }
      __syncwarp();
      float dres = CUDART_NAN_F;
      const float v = (lane < 15) ? gG[lane] : CUDART_NAN_F;
      float best = isnan(v) ? -CUDART_INF_F : v;
      int bi = lane < 15 ? lane : 99;
#pragma unroll
      for (int o2 = 16; o2 > 0; o2 >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o2);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o2);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      const unsigned finite = __ballot_sync(0xffffffffu, lane < 15 && !isnan(v));
      const int imx = finite ? bi : 14;
      const float vmax = gG[imx];
      if (vmax >= cfg.min_corr) {
        const int ix = imx - 7;
        int dh = cfg.strip_rows;
        float wys = 1.0f;
        if (dh > cfg.wndy_size) dh = cfg.wndy_size;
        else if (dh < cfg.wndy_size) {
          float swy = cfg.wndy[0];
          for (int i = 1; i < dh; i++) swy += cfg.wndy[i];
          wys = 1.0f / swy;
        }
        const int x0 = 7 + ix, nk = dh * 2 * cfg.wndx_size;
        float s0 = 0.f, sx = 0.f;
        for (int pass = 0; pass < 2; pass++) {
          const float xm = (pass == 1) ? sx / s0 : 0.f;
          for (int k = lane; k < nk; k += 32) {
            const int dy = k / (2 * cfg.wndx_size), rest = k - dy * 2 * cfg.wndx_size;
            const int adx = rest >> 1, dir = (rest & 1) ? 1 : -1, odd = dy & 1;
            if (((adx - odd) & 1) || (adx == 0 && dir < 0)) continue;
            const int idx = (adx * dir) >> 1, xx = 2 * idx + odd, x1 = x0 + idx;
            if (x1 < 0 || x1 >= 15) continue;
            const float d = gG[dy * 15 + x1];
            if (isnan(d) || !(d > 0.0f)) continue;
            const float wk = (((dy == 0) ? wys : 2.0f * wys) * cfg.wndy[dy]) * cfg.wndx[adx];
            if (pass == 0) {
              s0 += d * wk;
              sx += d * wk * xx;
            } else {
              // d(-(ix + sx/s0/2)) / d(combo): -(wk / (2 s0)) (xx - sx/s0)
              gcmb[dy * 15 + x1] = -(wk / (2.0f * s0)) * (xx - xm);
            }
          }
          if (pass == 0) {
            s0 = warp_sum(s0);
            sx = warp_sum(sx);
            if (s0 == 0.0f) break;
            dres = -(ix + sx / s0 / 2);
          }
        }
      }
      __syncwarp();
      // G = combo + offset, the geometric mean the strip entries enter
      for (int e = lane; e < RE; e += 32) gG[e] = gG[e] + cfg.corr_offset;
      if (lane == 0) s_d = dres;
    }
    __syncthreads();
    const float dres = s_d;
    if (isnan(dres)) {
      if (tid == 0) dval[tile] = CUDART_NAN_F;
      for (int i = tid; i < 2 * S; i += 32 * AD_NW) sens[tile * 2 * S + i] = 0.f;
      __syncthreads();
      continue;
    }

    // ---------------- reverse pass over the pairs, one round of AD_NW pairs at a time ----------------
    // A round's pairs are on distinct sensors (the host's schedule), so the warps add their CLT
    // gradients into disjoint parts of s_g; the barrier after each round orders the rounds, so
    // every gradient entry is summed in the same order in every run.  With the forward's strip
    // samples recorded and one entry per lane, the next round's sample is loaded one round ahead
    // so its latency overlaps this pair.
    const bool pre = as.use_strips && RE <= 32;
    const short *sched = &sc.corr_cfg->adj_round[0][0];
    int pnext = cfg.adj_rounds > 0 ? sched[warp] : -1;
    float vnext = 0.f;
    if (pre && pnext >= 0 && lane < RE) vnext = sc.strips[(tile * P + pnext) * RE + lane];
    for (int rd = 0; rd < cfg.adj_rounds; rd++) {
      const int pi = pnext;
      const float vcur = vnext;
      pnext = rd + 1 < cfg.adj_rounds ? sched[(rd + 1) * AD_NW + warp] : -1;
      if (pre && pnext >= 0 && lane < RE) vnext = sc.strips[(tile * P + pnext) * RE + lane];
      do {  // this warp's pair of the round (break: nothing to add)
        if (pi < 0) break;
        const PairDev pd = cfg.pairs[pi];
        if (!pd.in_combo) break;
        const float *c = sc.corr + (tile * P + pi) * TP_CORR;
        for (int i = lane; i < 240; i += 32) gs[i] = 0.f;
        for (int i = lane; i < 288; i += 32) qb[i] = 0.f;
        __syncwarp();
        // strip entries: d combo / d v_p = G / (n v_p) for the geometric mean of n pairs
        bool any = false;
        for (int e = lane; e < RE; e += 32) {
          if (gcmb[e] == 0.f) continue;
          const float d = pre ? vcur
                              : (as.use_strips ? sc.strips[(tile * P + pi) * RE + e]
                                               : strip_entry(c, strip_code, pd, e));
          const float v = d + cfg.corr_offset;
          if (!(v > 0.0f)) continue;
          const float f = __fdividef(gcmb[e] * gG[e] * inv_n, v);
          const int row = e / 15;
          const float half = row > 0 ? 0.5f : 1.0f;
          for (int side = 0; side < (row > 0 ? 2 : 1); side++) {
            int idx[4];
            float wt[4];
            int n;
            if (pd.kind <= 3) {
              const short2 code = *(const short2 *)&strip_code[(pd.kind * TP_MAX_STRIP * 15 + e) * 2];
              n = code_taps(side ? code.y : code.x, idx, wt);
            } else {
              n = general_taps(pd.bx, pd.by, row, e - row * 15 - 7, side ? 1 : -1, idx, wt);
            }
            for (int k = 0; k < n; k++) atomicAdd(&gs[idx[k]], f * half * wt[k]);
          }
          any = true;
        }
        if (!__any_sync(0xffffffffu, any)) break;
        __syncwarp();
        // 15x15 unfold (DttRad2.corr_unfold_tile) transposed into the four quadrants
#pragma unroll
        for (int k = 0; k < 2; k++) {
          const int a = (lane >> 3) + 4 * k, b = lane & 7;
          const float g1 = gs[(7 + a) * 15 + 7 + b];
          const float g2 = b ? gs[(7 + a) * 15 + 7 - b] : 0.f;
          const float g3 = a ? gs[(7 - a) * 15 + 7 + b] : 0.f;
          const float g4 = (a && b) ? gs[(7 - a) * 15 + 7 - b] : 0.f;
          qb[a * 9 + b] = 0.25f * (((g1 + g2) + g3) + g4);
          if (b) qb[72 + a * 9 + b - 1] = 0.25f * (((g1 - g2) + g3) - g4);
          if (a) qb[144 + (a - 1) * 9 + b] = 0.25f * (((g1 + g2) - g3) - g4);
          if (a && b) qb[216 + (a - 1) * 9 + b - 1] = 0.25f * (((g1 - g2) - g3) + g4);
        }
        __syncwarp();
        // 2D DCT-IIe/DST-IIe transposed: forward Z = Ta X^T Tb^T, so Xbar = Tb^T Zbar^T Ta
        {
          float z[8], v[8];
#pragma unroll
          for (int k = 0; k < 8; k++) z[k] = qb[q * 72 + k * 9 + r];  // column r of Zbar
          dtt2e_transposed(z, v, (q >> 1) & 1);                        // row r of V = Zbar^T Ta
#pragma unroll
          for (int n = 0; n < 8; n++) tb[q * 72 + r * 9 + n] = v[n];
          __syncwarp();
#pragma unroll
          for (int k = 0; k < 8; k++) z[k] = tb[q * 72 + k * 9 + r];  // column r of V
          dtt2e_transposed(z, v, q & 1);                               // column r of Xbar
#pragma unroll
          for (int k = 0; k < 8; k++) qb[q * 72 + k * 9 + r] = v[k];
          __syncwarp();
        }
        // LPF, colour mix and the fat-zero normalised product of each colour
        // (correlateSingleColorFD / correlateCompositeFD): acc = sum_c w_c t_c / (a2_c + fz2_c)
        float gq[4][2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int idx = lane + 32 * h;
          const float l = s_lpf[idx];
          const int off = (idx >> 3) * 9 + (idx & 7);
#pragma unroll
          for (int qq = 0; qq < 4; qq++) gq[qq][h] = qb[qq * 72 + off] * l;
        }
        const float fzz = cfg.fat_zero * cfg.fat_zero;
        for (int c = 0; c < C; c++) {
          const float wgt = (C == 1) ? 1.0f : cfg.col_weights[c];
          const float *c1 = s_clt + ((size_t)pd.cam1 * C + c) * TP_CLT;
          const float *c2 = s_clt + ((size_t)pd.cam2 * C + c) * TP_CLT;
          float d1[4][2], d2[4][2], a2[2], ia2[2], s1v[2], s2v[2];
#pragma unroll
          for (int h = 0; h < 2; h++) {
            float s1 = 0.f, s2 = 0.f;
#pragma unroll
            for (int m = 0; m < 4; m++) {
              d1[m][h] = c1[m * 64 + lane + 32 * h];
              d2[m][h] = c2[m * 64 + lane + 32 * h];
              s1 = fmaf(d1[m][h], d1[m][h], s1);
              s2 = fmaf(d2[m][h], d2[m][h], s2);
            }
            // |d1| |d2| with the forward's approximate square root; ia2 = 1 / a2 (0 where a2 = 0)
            const float pr = s1 * s2;
            ia2[h] = (pr > 0.0f) ? rsqrtf(pr) : 0.0f;
            a2[h] = pr * ia2[h];
            s1v[h] = s1;
            s2v[h] = s2;
          }
          const float fz2 = warp_sum(a2[0] + a2[1]) * (1.0f / 64) * fzz;
          float tg[4][2], dbar[2];
#pragma unroll
          for (int h = 0; h < 2; h++) {
            const float u = __fdividef(1.0f, a2[h] + fz2);
            const float t0 = d1[0][h] * d2[0][h] + d1[1][h] * d2[1][h] + d1[2][h] * d2[2][h] + d1[3][h] * d2[3][h];
            const float t1 = -d1[1][h] * d2[0][h] + d1[0][h] * d2[1][h] - d1[3][h] * d2[2][h] + d1[2][h] * d2[3][h];
            const float t2 = -d1[2][h] * d2[0][h] - d1[3][h] * d2[1][h] + d1[0][h] * d2[2][h] + d1[1][h] * d2[3][h];
            const float t3 = d1[3][h] * d2[0][h] - d1[2][h] * d2[1][h] - d1[1][h] * d2[2][h] + d1[0][h] * d2[3][h];
            const float swbar = gq[0][h] * t0 + gq[1][h] * t1 + gq[2][h] * t2 + gq[3][h] * t3;
            dbar[h] = -wgt * swbar * u * u;
            const float sw = wgt * u;
#pragma unroll
            for (int qq = 0; qq < 4; qq++) tg[qq][h] = gq[qq][h] * sw;
          }
          const float dsum = warp_sum(dbar[0] + dbar[1]) * (1.0f / 64) * fzz;
          float *g1p = s_g + ((size_t)pd.cam1 * C + c) * TP_CLT, *g2p = s_g + ((size_t)pd.cam2 * C + c) * TP_CLT;
#pragma unroll
          for (int h = 0; h < 2; h++) {
            const int idx = lane + 32 * h;
            const float a2bar = dbar[h] + dsum;
            const float T0 = tg[0][h], T1 = tg[1][h], T2 = tg[2][h], T3 = tg[3][h];
            float g1[4], g2[4];
            g1[0] = T0 * d2[0][h] + T1 * d2[1][h] + T2 * d2[2][h] + T3 * d2[3][h];
            g1[1] = T0 * d2[1][h] - T1 * d2[0][h] + T2 * d2[3][h] - T3 * d2[2][h];
            g1[2] = T0 * d2[2][h] + T1 * d2[3][h] - T2 * d2[0][h] - T3 * d2[1][h];
            g1[3] = T0 * d2[3][h] - T1 * d2[2][h] - T2 * d2[1][h] + T3 * d2[0][h];
            g2[0] = T0 * d1[0][h] - T1 * d1[1][h] - T2 * d1[2][h] + T3 * d1[3][h];
            g2[1] = T0 * d1[1][h] + T1 * d1[0][h] - T2 * d1[3][h] - T3 * d1[2][h];
            g2[2] = T0 * d1[2][h] - T1 * d1[3][h] + T2 * d1[0][h] - T3 * d1[1][h];
            g2[3] = T0 * d1[3][h] + T1 * d1[2][h] + T2 * d1[1][h] + T3 * d1[0][h];
            // a2 = sqrt(s1 s2): d a2 / d d1[m] = d1[m] s2 / a2
            const float k1 = a2bar * s2v[h] * ia2[h];
            const float k2 = a2bar * s1v[h] * ia2[h];
#pragma unroll
            for (int m = 0; m < 4; m++) {  // no other warp adds to these sensors in this round
              g1p[m * 64 + idx] += fmaf(k1, d1[m][h], g1[m]);
              g2p[m * 64 + idx] += fmaf(k2, d2[m][h], g2[m]);
            }
          }
        }
        __syncwarp();
      } while (0);
      __syncthreads();
    }

    // ---------------- dd/drx, dd/dry per sensor and colour (forward mode on the CLT) ----------------
    const int items = S * C;
    for (int g = warp; g < (items + 3) / 4; g += AD_NW) {
      const int it = g * 4 + q;
      const int itc = it < items ? it : items - 1;
      const int s = itc / C, c = itc - s * C;
      const SubtilePlan p = sc.plan[(size_t)task * S * C + itc];
      float gxy[2];
      if (C == 1) {
        shift_sens(sc, make_win(sc, p, s), p, s, s_clt + (size_t)itc * TP_CLT, s_g + (size_t)itc * TP_CLT,
                   tb + q * 72, r, it < items, gxy);
      } else {
        BayerWin bw;
        bw.w = make_win(sc, p, s, c);
        bw.c = c;
        bw.rr = sc.bayer_red_row;
        bw.rc = sc.bayer_red_col;
        shift_sens(sc, bw, p, s, s_clt + (size_t)itc * TP_CLT, s_g + (size_t)itc * TP_CLT, tb + q * 72, r,
                   it < items, gxy);
      }
      if (r == 0 && it < items) {
        s_sens[it * 2] = gxy[0];
        s_sens[it * 2 + 1] = gxy[1];
      }
    }
    __syncthreads();
    // a sensor's colours share its port: their sensitivities add, in colour order
    for (int i = tid; i < 2 * S; i += 32 * AD_NW) {
      const int s = i >> 1, k = i & 1;
      float v = 0.f;
      for (int c = 0; c < C; c++) v += s_sens[(s * C + c) * 2 + k];
      sens[(tile * S + s) * 2 + k] = v;
    }
    if (tid == 0) dval[tile] = dres;
    __syncthreads();
  }
}

// Per tile: Jacobian rows of d w.r.t. the sensors' (azimuth, tilt, roll, zoom)
// and the tile disparity, and the loss gradient with dL/dd = dl_dd (or 2 d).
// One thread per (task, sensor); a block holds 256 / S tasks.  The per-task sum
// over sensors and the block's partial sums of the extrinsic gradient (to
// `partial`) are taken in a fixed order, so the result is deterministic.
__global__ void __launch_bounds__(256) adjoint_contract_kernel(const __grid_constant__ SceneDev sc,
                                                              const float *sens, const float *dval,
                                                              const float *dl_dd, float *jac_e, float *jac_d,
                                                              float *grad_d, float *partial) {
  __shared__ float s_jd[256];
  __shared__ float s_ge[256][4];
  const int S = sc.num_sensors, tpb = 256 / S;
  const int lt = threadIdx.x / S, s = threadIdx.x - lt * S;
  const int task = blockIdx.x * tpb + lt;
  const bool act = lt < tpb && task < sc.num_tasks;
  float jd = 0.f, ge[4] = {0.f, 0.f, 0.f, 0.f};
  size_t tile = 0;
  float gbar = 0.f;
  if (act) {
    const int txy = sc.task_txy[task];
    tile = (size_t)(txy >> 16) * sc.tilesX + (txy & 0xffff);
    const float d = dval[tile];
    gbar = isnan(d) ? 0.f : (dl_dd ? dl_dd[tile] : 2.0f * d);
    const double *pd = sc.port_deriv + ((size_t)task * S + s) * 10;
    const float jx = sens[(tile * S + s) * 2], jy = sens[(tile * S + s) * 2 + 1];
    float j4[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      j4[k] = jx * (float)pd[k] + jy * (float)pd[5 + k];
      ge[k] = gbar * j4[k];
    }
    *(float4 *)(jac_e + (tile * S + s) * 4) = make_float4(j4[0], j4[1], j4[2], j4[3]);
    jd = jx * (float)pd[4] + jy * (float)pd[9];
  }
  s_jd[threadIdx.x] = jd;
#pragma unroll
  for (int k = 0; k < 4; k++) s_ge[threadIdx.x][k] = ge[k];
  __syncthreads();
  if (act && s == 0) {  // sensors in order
    float t = 0.f;
    for (int q = 0; q < S; q++) t += s_jd[lt * S + q];
    jac_d[tile] = t;
    grad_d[tile] = gbar * t;
  }
  if (threadIdx.x < S * 4) {  // the block's tasks in order
    const int ss = threadIdx.x >> 2, k = threadIdx.x & 3;
    float v = 0.f;
    for (int q = 0; q < tpb; q++) v += s_ge[q * S + ss][k];
    partial[(size_t)blockIdx.x * S * 4 + threadIdx.x] = v;
  }
}

// One block per extrinsic coordinate i: thread t sums the partials of blocks t, t + 256, ... in
// order, then a fixed tree over the 256 threads (deterministic; a single thread walking all
// partials waited on one dependent load per block)
__global__ void __launch_bounds__(256) adjoint_final_kernel(const float *partial, int nblocks, int n,
                                                            float *grad_e) {
  __shared__ float s[256];
  const int i = blockIdx.x, t = threadIdx.x;
  float v = 0.f;
  for (int b = t; b < nblocks; b += 256) v += partial[(size_t)b * n + i];
  s[t] = v;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (t < h) s[t] += s[t + h];
    __syncthreads();
  }
  if (t == 0) grad_e[i] = s[0];
}

cudaError_t upload_adjoint_constants() {
  cudaError_t e = upload_dtt_constants();
  if (e != cudaSuccess) return e;
  return cudaSuccess;
}

int adjoint_smem_bytes(int S, int C) { return (S * C * 2 * TP_CLT + 240 + 240 + AD_NW * 816) * 4; }

cudaError_t launch_adjoint(const SceneDev &sc, const CorrConst &cc, int recompute, int use_strips, float *sens,
                           float *dval,
                           const float *dl_dd, float *jac_e, float *jac_d, float *grad_d, float *partial,
                           float *grad_e, cudaStream_t st) {
  if (sc.num_tasks <= 0) return cudaSuccess;
  if ((sc.num_colors != 1 && sc.num_colors != 3) || !sc.port_deriv || !sc.combo) return cudaErrorInvalidValue;
  AdjShape as;
  as.S = sc.num_sensors;
  as.C = sc.num_colors;
  as.P = sc.num_pairs;
  as.RE = (sc.strip_rows < sc.wndy_size ? sc.strip_rows : sc.wndy_size) * 15;
  as.per_warp = adjoint_smem_bytes(as.S, as.C) / 4;
  as.recompute = recompute;
  as.use_strips = (use_strips && sc.strips) ? 1 : 0;
  const int bytes = adjoint_smem_bytes(as.S, as.C);
  cudaError_t e = cudaFuncSetAttribute(adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 152, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adjoint_kernel, 32 * AD_NW, bytes);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int grid = sc.num_tasks < sms * per_sm ? sc.num_tasks : sms * per_sm;
  adjoint_kernel<<<grid, 32 * AD_NW, bytes, st>>>(sc, as, cc, sens, dval);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int nb = (sc.num_tasks + 256 / sc.num_sensors - 1) / (256 / sc.num_sensors);
  adjoint_contract_kernel<<<nb, 256, 0, st>>>(sc, sens, dval, dl_dd, jac_e, jac_d, grad_d, partial);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  adjoint_final_kernel<<<sc.num_sensors * 4, 256, 0, st>>>(partial, nb, sc.num_sensors * 4, grad_e);
  return cudaGetLastError();
}
