// tp_fused.cu -- fused forward tile kernel: convert+correct -> pair correlation
// -> strip combination -> disparity extraction, one CTA per group of tiles.
//
// Same arithmetic as the stage kernels (ImageDtt.extract_correct_tile,
// convolve_tile, fract_shift; Correlation2d.correlateCompositeFD,
// scaleRotateInterpoateSingleCorrelation, combineInterpolatedCorrelations,
// getMaxXYInt, getMaxXCm, getMaxXSOrtho) but organised for GB300:
//
//  phase A  one warp = one colour of 4 sensors of a tile; lanes 8q..8q+7 own
//           sensor q, lane r owns folded row r.  The fold reads each needed
//           pixel once (L1-cached __ldg); 8-point DCT-IV/DST-IV run in
//           registers (Plonka-Tasche recursion, DttRad2.java:1107-1146, scale
//           folded into the first stage); the 8x8 transpose goes through a
//           9-padded shared buffer.  For Bayer planes only the transforms that
//           are not symmetric images of another are computed: a red/blue
//           window is sparse on a 2x2 lattice, so SC/CS/SS are index reversals
//           of CC with window-phase signs; a green window is a checkerboard, so
//           CS and SS are reversals of SC and CC.  That is 4 instead of 12 2D
//           transforms per sensor.  CLT goes to shared memory (for phase B) and
//           to HBM (a declared output); per-frequency amplitudes are cached.
//  phase B  one warp = one (tile, pair): the correlation product, fat-zero
//           normalisation, colour mix and LPF on 2 CLT indices per lane, the
//           four 2D DCT-IIe/DST-IIe in registers, the 15x15 unfold, the surface
//           to HBM, and that pair's strip folded into a per-warp running product.
//  phase C  one warp = one tile: combine the per-warp strip products, integer
//           argmax on the disparity axis, windowed centroid, hor/vert maxima.
#include "tp_dtt.cuh"

#include <cstddef>

namespace {

constexpr int SCR = 288;           // per-warp scratch floats: [4][8][9] transpose / surface buffer

// ---------------------------------------------------------------------------
// phase A: CLT of one sub-tile, lane r of the 8-lane group holds row r
// (= horizontal frequency r) of each quadrant on return: o[m][v].
// ---------------------------------------------------------------------------
template <int KIND, typename PIX = Win>  // 0 mono, 1 Bayer red/blue, 2 Bayer green; PIX: at(row, col)
__device__ __forceinline__ void subtile_clt(const PIX &w, float rx, float ry, int pc, int pr, int pg, int r,
                                            float *tbuf, float o[4][8]) {
  float ahs, ahc, avs, avc;
  __sincosf(CUDART_PI_F * 0.0625f * rx, &ahs, &ahc);
  __sincosf(CUDART_PI_F * 0.0625f * ry, &avs, &avc);
  const FoldIdx fv = fold_idx(r);
  float vw0, vw1, hw0[8], hw1[8];
  fold_weights(ahc, ahs, avc, avs, fv, vw0, vw1, hw0, hw1);
  if constexpr (KIND == 1) {
    // one nonzero pixel per folded value: the term whose source row/column has the colour's parity
    const bool a1 = (fv.src0 & 1) != pr;
    const int srow = a1 ? fv.src1 : fv.src0;
    const float vk = a1 ? fv.sc1 * vw1 : fv.sc0 * vw0;
    float y[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const FoldIdx fh = fold_idx(j);
      const bool b1 = (fh.src0 & 1) != pc;
      const int scol = b1 ? fh.src1 : fh.src0;
      const float hk = b1 ? fh.sc1 * hw1[j] : fh.sc0 * hw0[j];
      y[j] = (vk * hk) * w.at(srow, scol);
    }
    float z[8];
    dct4_fast(y, z);
    group_transpose(z, tbuf, r);
    dct4_fast(z, o[0]);
    // SC[h][v] = sh CC[7-h][v], CS[h][v] = sv CC[h][7-v], SS = sh sv CC[7-h][7-v]
    const float sh = pc ? -1.f : 1.f, sv = pr ? -1.f : 1.f;
#pragma unroll
    for (int v = 0; v < 8; v++) o[1][v] = sh * __shfl_xor_sync(0xffffffffu, o[0][v], 7);
#pragma unroll
    for (int v = 0; v < 8; v++) {
      o[2][v] = sv * o[0][7 - v];
      o[3][v] = sv * o[1][7 - v];
    }
  } else if constexpr (KIND == 2) {
    // two nonzero pixels per folded value (checkerboard): CC and SC folds
    float ycc[8], ysc[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const FoldIdx fh = fold_idx(j);
      float cc = 0.f, sc = 0.f;
#pragma unroll
      for (int a = 0; a < 2; a++) {
        const int srow = a ? fv.src1 : fv.src0;
        const float vk = a ? fv.sc1 * vw1 : fv.sc0 * vw0;
        const bool b1 = ((fh.src0 + srow) & 1) != pg;  // column term with (row + col) parity pg
        const int scol = b1 ? fh.src1 : fh.src0;
        const float x = vk * w.at(srow, scol);
        cc = fmaf(b1 ? fh.sc1 * hw1[j] : fh.sc0 * hw0[j], x, cc);
        sc = fmaf(b1 ? fh.ss1 * hw1[j] : fh.ss0 * hw0[j], x, sc);
      }
      ycc[j] = cc;
      ysc[j] = sc;
    }
    float z[8];
    dct4_fast(ycc, z);
    group_transpose(z, tbuf, r);
    dct4_fast(z, o[0]);
    dtt4_fast(ysc, z, true);
    group_transpose(z, tbuf, r);
    dct4_fast(z, o[1]);
    // CS[h][v] = sg SC[7-h][7-v], SS[h][v] = sg CC[7-h][7-v]
    const float sg = pg ? -1.f : 1.f;
#pragma unroll
    for (int v = 0; v < 8; v++) {
      o[2][7 - v] = sg * __shfl_xor_sync(0xffffffffu, o[1][v], 7);
      o[3][7 - v] = sg * __shfl_xor_sync(0xffffffffu, o[0][v], 7);
    }
  } else {
    fold_dtt_dense(w, fv, vw0, vw1, hw0, hw1, r, tbuf, o);
  }
}

// convolution with the kernel tile and the phase-rotation shift, in place on o[m][v]
__device__ __forceinline__ void conv_shift(float o[4][8], const float *kp, float rx, float ry, int r) {
  if (kp) {
    float k[4][8];
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const float4 *p = (const float4 *)(kp + m * 64 + r * 8);
      float4 a = __ldg(p), b = __ldg(p + 1);
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
  float ch, shh, cvr, svr;
  __sincosf(CUDART_PI_F * 0.0625f * (2 * r + 1) * rx, &shh, &ch);
  __sincosf(CUDART_PI_F * 0.0625f * (2 * r + 1) * ry, &svr, &cvr);
  const int base = threadIdx.x & 24;  // first lane of this 8-lane group
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

// the stored CLT of row r (horizontal frequency r) of the four quadrants; with the colour's bit
// in clt_lpf_mask multiplied by the LPF, as the reference GPU stores it (lpf_mask,
// TileProcessor.cuh:1037-1061, GPUTileProcessor.java:547); the correlation keeps the unfiltered copy
__device__ __forceinline__ void store_clt(const SceneDev &sc, int c, int r, float *gdst, const float o[4][8]) {
  if (sc.lpf_rbg && ((sc.clt_lpf_mask >> c) & 1)) {
    const float4 *lp = (const float4 *)(sc.lpf_rbg + c * 64 + r * 8);
    const float4 la = __ldg(lp), lb = __ldg(lp + 1);
#pragma unroll
    for (int m = 0; m < 4; m++) {
      *(float4 *)(gdst + m * 64) = make_float4(o[m][0] * la.x, o[m][1] * la.y, o[m][2] * la.z, o[m][3] * la.w);
      *(float4 *)(gdst + m * 64 + 4) = make_float4(o[m][4] * lb.x, o[m][5] * lb.y, o[m][6] * lb.z, o[m][7] * lb.w);
    }
    return;
  }
#pragma unroll
  for (int m = 0; m < 4; m++) {
    *(float4 *)(gdst + m * 64) = make_float4(o[m][0], o[m][1], o[m][2], o[m][3]);
    *(float4 *)(gdst + m * 64 + 4) = make_float4(o[m][4], o[m][5], o[m][6], o[m][7]);
  }
}

struct FwdShape {
  int nw;                 // warps per CTA (each warp owns whole tiles)
  int S, C, P, RE, quad;  // sensors, colours, pairs, strip entries, quad layout
  int clt_floats, per_warp;
};

}  // namespace

// ---------------------------------------------------------------------------
// the three phases of the forward for one tile, shared by the schedules
// ---------------------------------------------------------------------------
// phase A item gt = (colour, group of 4 sensors): lanes 8q..8q+7 own sensor 4g+q
template <int C>
__device__ __forceinline__ void fwd_clt_item(const SceneDev &sc, int S, int task, size_t tile, int gt, int groups,
                                             float *s_clt, float *scr, int lane) {
  const int q = lane >> 3, r = lane & 7;
  const int rr = sc.bayer_red_row, rc = sc.bayer_red_col;
  const int c = gt / groups, g = gt - c * groups;
  const int s = g * 4 + q;
  const bool act = s < S;
  const int sidx = act ? s : S - 1;
  const SubtilePlan p = sc.plan[((size_t)task * S + sidx) * C + c];
  Win w;
  w.img = sc.images[sidx];
  w.pitch = sc.img_pitch;
  w.tlx = p.tlx; w.tly = p.tly; w.W = sc.width; w.H = sc.height;
  w.u16 = sc.img_dtype[sidx];
  w.inside = (p.tlx >= 0) && (p.tly >= 0) && (p.tlx <= sc.width - 16) && (p.tly <= sc.height - 16);
  w.scale = sc.color_scale[c];
  float o[4][8];
  float *tbuf = scr + q * 72;
  if (C == 1) {
    subtile_clt<0>(w, p.rx, p.ry, 0, 0, 0, r, tbuf, o);
  } else if (c < 2) {
    const int pc = ((c == 0 ? rc : 1 - rc) - p.tlx) & 1, pr = ((c == 0 ? rr : 1 - rr) - p.tly) & 1;
    subtile_clt<1>(w, p.rx, p.ry, pc, pr, 0, r, tbuf, o);
  } else {
    const int pg = (p.tlx + p.tly + rc + rr + 1) & 1;
    subtile_clt<2>(w, p.rx, p.ry, 0, 0, pg, r, tbuf, o);
  }
  const float *kp = (p.kidx >= 0) ? sc.kernels[sidx] + (size_t)p.kidx * TP_CLT : nullptr;
  conv_shift(o, kp, p.rx, p.ry, r);
  if (act) {
    store_clt(sc, c, r, sc.clt + ((tile * S + s) * C + c) * TP_CLT + r * 8, o);
    // all four quadrants: after the convolution and the shift the Bayer symmetries no longer hold
    float *sdst = s_clt + ((size_t)s * C + c) * TP_CLT + r * 8;
#pragma unroll
    for (int m = 0; m < 4; m++) {
      *(float4 *)(sdst + m * 64) = make_float4(o[m][0], o[m][1], o[m][2], o[m][3]);
      *(float4 *)(sdst + m * 64 + 4) = make_float4(o[m][4], o[m][5], o[m][6], o[m][7]);
    }
  }
}

// phase B for pair pi: correlation surface to HBM, strip entries folded into cmb
// (NT = strip entries per lane / 32 rounded up: 1 when the extraction reads <= 32 entries)
// lpf: the correlation LPF (64 floats) in shared memory: each lane reads its own two entries,
// which from the kernel's parameter space would take one constant-cache access per lane
template <int C, int NT, bool OACC = false>
__device__ __forceinline__ void fwd_pair(const SceneDev &sc, const CorrConst &cfg, const float *lpf, size_t tile,
                                         int P, int pi, int RE, bool log_mode, const short *strip_code,
                                         const float *s_clt, float *scr, int lane, float cmb[8],
                                         float *corr_out = nullptr, float *oprod = nullptr) {
  const int q = lane >> 3, r = lane & 7;
  float *qb = scr;
  const PairDev pd = cfg.pairs[pi];
  const float *c1 = s_clt + (size_t)pd.cam1 * C * TP_CLT, *c2 = s_clt + (size_t)pd.cam2 * C * TP_CLT;
  // with one strip entry per lane its sample code is read ahead of the correlation arithmetic
  short2 code1 = make_short2(-1, -1);
  if (NT == 1 && pd.in_combo && pd.kind <= 3 && lane < RE)
    code1 = *(const short2 *)&strip_code[(pd.kind * TP_MAX_STRIP * 15 + lane) * 2];
  float acc[4][2];
#pragma unroll
  for (int c = 0; c < C; c++) {
    float d1[4][2], d2[4][2], a2[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      float s1 = 0.f, s2 = 0.f;
#pragma unroll
      for (int m = 0; m < 4; m++) {
        d1[m][h] = c1[c * TP_CLT + m * 64 + lane + 32 * h];
        d2[m][h] = c2[c * TP_CLT + m * 64 + lane + 32 * h];
        s1 = fmaf(d1[m][h], d1[m][h], s1);
        s2 = fmaf(d2[m][h], d2[m][h], s2);
      }
      const float pr = s1 * s2;
      a2[h] = (pr > 0.0f) ? pr * rsqrtf(pr) : 0.0f;  // |d1| |d2|; approximate square root (~2 ulp)
    }
    const float fz2 = warp_sum(a2[0] + a2[1]) * (1.0f / 64) * cfg.fat_zero * cfg.fat_zero;
    const float wgt = (C == 1) ? 1.0f : cfg.col_weights[c];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const float sw = __fdividef(wgt, a2[h] + fz2);
      const float t0 = d1[0][h] * d2[0][h] + d1[1][h] * d2[1][h] + d1[2][h] * d2[2][h] + d1[3][h] * d2[3][h];
      const float t1 = -d1[1][h] * d2[0][h] + d1[0][h] * d2[1][h] - d1[3][h] * d2[2][h] + d1[2][h] * d2[3][h];
      const float t2 = -d1[2][h] * d2[0][h] - d1[3][h] * d2[1][h] + d1[0][h] * d2[2][h] + d1[1][h] * d2[3][h];
      const float t3 = d1[3][h] * d2[0][h] - d1[2][h] * d2[1][h] - d1[1][h] * d2[2][h] + d1[0][h] * d2[3][h];
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
    const int idx = lane + 32 * h;
    const float l = lpf[idx];
    const int off = (idx >> 3) * 9 + (idx & 7);
#pragma unroll
    for (int qq = 0; qq < 4; qq++) qb[qq * 72 + off] = acc[qq][h] * l;
  }
  __syncwarp();
  {
    // both passes transpose in place: every row is read into registers before any is overwritten
    float x[8], y[8];
#pragma unroll
    for (int e = 0; e < 8; e++) x[e] = qb[q * 72 + r * 9 + e];
    dtt2e_fast(x, y, (q >> 1) & 1);
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 8; j++) qb[q * 72 + j * 9 + r] = y[j];
    __syncwarp();
#pragma unroll
    for (int e = 0; e < 8; e++) x[e] = qb[q * 72 + r * 9 + e];
    dtt2e_fast(x, y, q & 1);
    __syncwarp();
#pragma unroll
    for (int e = 0; e < 8; e++) qb[q * 72 + r * 9 + e] = y[e];
  }
  __syncwarp();
  // 15x15 unfold (DttRad2.corr_unfold_tile): each lane owns 2 cells (a, b) and writes their mirror
  // images; the quadrants are read into registers first, the surface then overwrites them
  float uA[2], uB[2], uC[2], uD[2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int a = (lane >> 3) + 4 * k, b = lane & 7;
    uA[k] = qb[a * 9 + b];
    uB[k] = b ? qb[72 + a * 9 + b - 1] : 0.f;
    uC[k] = a ? qb[144 + (a - 1) * 9 + b] : 0.f;
    uD[k] = (a && b) ? qb[216 + (a - 1) * 9 + b - 1] : 0.f;
  }
  __syncwarp();
  float *cs = qb;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int a = (lane >> 3) + 4 * k, b = lane & 7;
    const float A = uA[k], B = uB[k], Cc = uC[k], D = uD[k];
    cs[(7 + a) * 15 + 7 + b] = 0.25f * (((A + B) + Cc) + D);
    if (b) cs[(7 + a) * 15 + 7 - b] = 0.25f * (((A - B) + Cc) - D);
    if (a) cs[(7 - a) * 15 + 7 + b] = 0.25f * (((A + B) - Cc) - D);
    if (a && b) cs[(7 - a) * 15 + 7 - b] = 0.25f * (((A - B) - Cc) + D);
  }
  __syncwarp();
  if (OACC && (pd.kind == 0 || pd.kind == 1) && !cfg.log_combine) {
    // getMaxXSOrtho profile of a horizontal (lanes 0-14, columns) or vertical (lanes 16-30, rows)
    // pair, symmetrised (even in i, so rows 0..7 carry it) and multiplied into this lane's oprod
    const int half = lane >> 4, j = lane & 15;
    if (half == pd.kind && j < 15) {
      const int stride = half ? 1 : 15, base = half ? j * 15 : j;
#pragma unroll
      for (int i = 0; i < 8; i++)
        oprod[i] *= 0.5f * (cs[base + i * stride] + cs[base + (14 - i) * stride]) + cfg.corr_offset;
    }
  }
  float *gc = corr_out ? corr_out : sc.corr + (tile * P + pi) * TP_CORR;
  for (int o2 = lane; o2 < TP_CORR; o2 += 32) gc[o2] = cs[o2];
  if (pd.in_combo) {
#pragma unroll
    for (int t = 0; t < NT; t++) {
      const int e = lane + 32 * t;
      if (e < RE) {
        const int row = e / 15;
        float d;
        if (pd.kind <= 3) {
          const short2 code = (NT == 1) ? code1 : *(const short2 *)&strip_code[(pd.kind * TP_MAX_STRIP * 15 + e) * 2];
          d = sample_code(cs, code.x);
          if (row > 0) {
            const float d2 = sample_code(cs, code.y);
            d = (isnan(d) || isnan(d2)) ? CUDART_NAN_F : (0.5f * d + 0.5f * d2);
          }
        } else {
          const int scol = e - row * 15 - 7;
          d = strip_sample(cs, 4, pd.bx, pd.by, row, scol, -1);
          if (row > 0) {
            const float d2 = strip_sample(cs, 4, pd.bx, pd.by, row, scol, 1);
            d = (isnan(d) || isnan(d2)) ? CUDART_NAN_F : (0.5f * d + 0.5f * d2);
          }
        }
        if (sc.strips && !corr_out) sc.strips[(tile * P + pi) * RE + e] = d;  // kept for the adjoint
        float v = d + cfg.corr_offset;
        if (v < 0.0f) v = 0.0f;
        if (log_mode) cmb[t] += logf(v);
        else cmb[t] *= cfg.twice_diagonal ? v * v : v;
      }
    }
  }
  __syncwarp();
}

// phase C, lane-parallel half: the combined strip (geometric mean of the pairs' strips) into
// combo (shared) and sc.combo, and this lane's getMaxXSOrtho profile value (lanes 0-14 the
// horizontal pairs' column j, lanes 16-30 the vertical pairs' row j; -inf elsewhere)
template <int NT, bool OACC = false>
__device__ __forceinline__ float fwd_extract_values(const SceneDev &sc, const CorrConst &cfg, int quad, int P, int RE,
                                                    bool log_mode, int ncomb, size_t tile, float *combo, int lane,
                                                    const float cmb[8], const float *oprod) {
#pragma unroll
  for (int t = 0; t < NT; t++) {
    const int e = lane + 32 * t;
    if (e < RE) {
      float v = cmb[t];
      if (log_mode) v = isnan(v) ? CUDART_NAN_F : (isinf(v) ? 0.0f : expf(v / cfg.num_combo) - cfg.corr_offset);
      else if (v > 0.0f) v = powf(v, 1.0f / ncomb) - cfg.corr_offset;
      combo[e] = v;
      if (sc.combo) sc.combo[tile * RE + e] = v;  // kept for the adjoint (and the split extraction)
    }
  }
  float sum = -CUDART_INF_F;
  if (quad && (cfg.num_hor > 0 || cfg.num_vert > 0)) {
    // the surfaces of this tile were just written by this warp (L1/L2 resident)
    const int half = lane >> 4, j = lane & 15;
    const int np = half ? cfg.num_vert : cfg.num_hor;
    if (j < 15 && np > 0) {
      // the symmetrised profile is even in i (d[i] == d[14 - i]), so rows 0..7 carry it; all
      // loads of one pair are issued before their use
      float prod[8];
#pragma unroll
      for (int i = 0; i < 8; i++) prod[i] = OACC ? oprod[i] : 1.f;
      for (int k = 0; k < (OACC ? 0 : np); k++) {
        const float *cc = sc.corr + (tile * P + (half ? cfg.vert_pairs[k] : cfg.hor_pairs[k])) * TP_CORR;
        const int stride = half ? 1 : 15, base = half ? j * 15 : j;
        float a[8], b[8];
#pragma unroll
        for (int i = 0; i < 8; i++) {
          a[i] = cc[base + i * stride];
          b[i] = cc[base + (14 - i) * stride];
        }
#pragma unroll
        for (int i = 0; i < 8; i++) prod[i] *= 0.5f * (a[i] + b[i]) + cfg.corr_offset;
      }
      sum = 0.f;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const float p = prod[i];
        const float v = (p > 0.0f) ? ((np == 2) ? sqrtf(p) : ((np == 1) ? p : powf(p, 1.0f / np))) - cfg.corr_offset
                                   : -cfg.corr_offset;
        sum += v * ((i < 7) ? cfg.notch[i] + cfg.notch[14 - i] : cfg.notch[7]);
      }
    }
  }
  __syncwarp();
  return sum;
}

// phase C, serial half: integer argmax and windowed centroid of the combined strip (getMaxXYInt,
// getMaxXCm), the maxima of the ortho profiles (getMaxXSOrtho), the disparity record
__device__ __forceinline__ void fwd_extract_finish(const SceneDev &sc, const CorrConst &cfg, int quad, size_t tile,
                                                   const float *combo, float sum, int lane) {
  float res[TP_NDISP];
#pragma unroll
  for (int k = 0; k < TP_NDISP; k++) res[k] = (k == 2 || k == 4 || k == 6) ? 0.f : CUDART_NAN_F;
  {
    // integer argmax on row 0 (getMaxXYInt): first maximum over the non-NaN entries
    const float v = (lane < 15) ? combo[lane] : CUDART_NAN_F;
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
    const float vmax = combo[imx];
    if (vmax >= cfg.min_corr) {
      const int ix = imx - 7;
      res[0] = (float)(-ix);
      res[2] = vmax;
      res[8] = (float)ix;
      int dh = cfg.strip_rows;
      float wys = 1.0f;
      if (dh > cfg.wndy_size) dh = cfg.wndy_size;
      else if (dh < cfg.wndy_size) {
        float swy = cfg.wndy[0];
        for (int i = 1; i < dh; i++) swy += cfg.wndy[i];
        wys = 1.0f / swy;
      }
      float s0 = 0.f, sx = 0.f;
      const int x0 = 7 + ix, nk = dh * 2 * cfg.wndx_size;
      for (int k = lane; k < nk; k += 32) {  // windowed centroid (getMaxXCm), one sample per lane
        const int dy = k / (2 * cfg.wndx_size), rest = k - dy * 2 * cfg.wndx_size;
        const int adx = rest >> 1, dir = (rest & 1) ? 1 : -1, odd = dy & 1;
        if (((adx - odd) & 1) || (adx == 0 && dir < 0)) continue;
        const int idx = (adx * dir) >> 1, xx = 2 * idx + odd, x1 = x0 + idx;
        if (x1 < 0 || x1 >= 15) continue;
        float d = combo[dy * 15 + x1];
        if (isnan(d) || !(d > 0.0f)) continue;
        d *= (((dy == 0) ? wys : 2.0f * wys) * cfg.wndy[dy]) * cfg.wndx[adx];
        s0 += d;
        sx += d * xx;
      }
      s0 = warp_sum(s0);
      sx = warp_sum(sx);
      if (s0 != 0.0f) {
        res[1] = -(ix + sx / s0 / 2);
        res[7] = s0;
      }
    }
  }
  if (quad && (cfg.num_hor > 0 || cfg.num_vert > 0)) {
    // getMaxXSOrtho: lanes 0-14 horizontal pairs, lanes 16-30 vertical pairs
    const int half = lane >> 4, j = lane & 15;
    float best = sum;
    int bi = (j < 15) ? j : 99;
#pragma unroll
    for (int o2 = 8; o2 > 0; o2 >>= 1) {  // within each 16-lane half
      const float ob = __shfl_xor_sync(0xffffffffu, best, o2);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o2);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    const int ic = bi, base = half << 4;
    const float f0 = __shfl_sync(0xffffffffu, sum, base + (ic > 0 ? ic - 1 : 0));
    const float f1 = __shfl_sync(0xffffffffu, sum, base + ic);
    const float f2 = __shfl_sync(0xffffffffu, sum, base + (ic < 14 ? ic + 1 : 14));
    float xc = (float)ic;
    if (ic > 0 && ic < 14) {
      const float den = f0 - 2.0f * f1 + f2;
      if (den != 0.0f) xc = ic + 0.5f * (f0 - f2) / den;
    }
    int ir = (int)floorf(xc + 0.5f);
    ir = ir < 0 ? 0 : (ir > 14 ? 14 : ir);
    const float fr = __shfl_sync(0xffffffffu, sum, base + ir);
    const float hx = __shfl_sync(0xffffffffu, xc, 0), hs = __shfl_sync(0xffffffffu, fr, 0);
    const float vx = __shfl_sync(0xffffffffu, xc, 16), vs = __shfl_sync(0xffffffffu, fr, 16);
    if (cfg.num_hor > 0) { res[3] = -(hx - 7.0f); res[4] = hs / 8.0f; }
    if (cfg.num_vert > 0) { res[5] = -(vx - 7.0f); res[6] = vs / 8.0f; }
  }
  float *dm = sc.disp + tile * TP_NDISP;
  if (lane < TP_NDISP) {
    float v = res[0];
#pragma unroll
    for (int k = 1; k < TP_NDISP; k++) if (lane == k) v = res[k];
    dm[lane] = v;
  }
  __syncwarp();
}

// phase C: combined strip, integer argmax, centroid, ortho maxima, disparity record
template <int NT, bool OACC = false>
__device__ __forceinline__ void fwd_extract(const SceneDev &sc, const CorrConst &cfg, int quad, int P, int RE,
                                            bool log_mode, int ncomb, size_t tile, float *scr, int lane,
                                            const float cmb[8], const float *oprod = nullptr) {
  const float sum = fwd_extract_values<NT, OACC>(sc, cfg, quad, P, RE, log_mode, ncomb, tile, scr, lane, cmb, oprod);
  fwd_extract_finish(sc, cfg, quad, tile, scr, sum, lane);
}

// ---------------------------------------------------------------------------
// warp-per-tile schedule: one warp carries a tile through all stages, no CTA barriers
// ---------------------------------------------------------------------------
template <int C, int NT>  // colours: 1 (mono) or 3 (Bayer R, B, G); strip entries per lane / 32
__global__ void __launch_bounds__(128, 4) fused_forward_kernel(const __grid_constant__ SceneDev sc,
                                                               const __grid_constant__ FwdShape fs,
                                                               const __grid_constant__ CorrConst cfg) {
  extern __shared__ float sm[];
  __shared__ float s_lpf[64];  // the correlation LPF, read per lane by fwd_pair
  for (int i = threadIdx.x; i < 64; i += blockDim.x) s_lpf[i] = cfg.lpf[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = fs.S, P = fs.P, RE = fs.RE, NW = fs.nw;
  // per-warp shared memory: CLT of the tile [S][C][4][64] and a 288-float scratch buffer
  float *s_clt = sm + warp * fs.per_warp;
  float *scr = s_clt + fs.clt_floats;
  const short *strip_code = &sc.corr_cfg->strip_code[0][0][0];
  const int groups = (S + 3) >> 2;
  const bool log_mode = cfg.log_combine;
  const int ncomb = cfg.twice_diagonal ? 2 * cfg.num_combo : cfg.num_combo;
  for (int task = blockIdx.x * NW + warp; task < sc.num_tasks; task += gridDim.x * NW) {
    const int txy = sc.task_txy[task];
    const size_t tile = (size_t)(txy >> 16) * sc.tilesX + (txy & 0xffff);
    for (int gt = 0; gt < C * groups; gt++) fwd_clt_item<C>(sc, S, task, tile, gt, groups, s_clt, scr, lane);
    __syncwarp();
    float cmb[8];
#pragma unroll
    for (int t = 0; t < NT; t++) cmb[t] = log_mode ? 0.f : 1.f;
    float oprod[8];  // hor / vert profile products of this lane's column (row), filled by phase B
#pragma unroll
    for (int i = 0; i < 8; i++) oprod[i] = 1.f;
    for (int pi = 0; pi < P; pi++)
      fwd_pair<C, NT, true>(sc, cfg, s_lpf, tile, P, pi, RE, log_mode, strip_code, s_clt, scr, lane, cmb, nullptr,
                            oprod);
    fwd_extract<NT, true>(sc, cfg, fs.quad, P, RE, log_mode, ncomb, tile, scr, lane, cmb, oprod);
  }
}

// ---------------------------------------------------------------------------
// Warp per tile with staged image windows: scenes of 4 (or fewer) u16 Bayer sensors.
// The image reads of phase A are its main cost (the warp waits on them once per
// colour item), so each item's four 16x16 sensor windows are copied into shared
// memory one item ahead, while the warp computes the previous item: 16 rows x 24
// u16 from the 16-byte boundary below the window corner, three 16-byte cp.async
// chunks per row, into the CLT slot of (sensor, colour) -- that slot holds nothing
// until the item writes its CLT there, after its last window read.  The next
// tile's first windows go in after its correlation phase has read the CLT slots.
// Windows that cross the image border are gathered with the edge mirroring.
// ---------------------------------------------------------------------------
constexpr int WROW = 24;  // staged window row: 24 u16 (48 bytes)

__device__ __forceinline__ void cp_async16(void *dst_smem, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// pixel source of subtile_clt: a staged window, column sx of the 16-byte aligned copy
struct SWin {
  const uint16_t *base;
  int sx;
  float scale;
  __device__ __forceinline__ float at(int row, int col) const { return (float)base[row * WROW + sx + col] * scale; }
};

// lanes 8q..8q+7 (r = lane & 7) copy sensor q's window at corner (tlx, tly) into dst: 48 chunks,
// 6 per lane; chunk 2 of a row is left out where it would pass the row's end (then tlx is
// 16-byte aligned and the window lies in chunks 0 and 1)
__device__ __forceinline__ void stage_window(const SceneDev &sc, const uint16_t *img, int tlx, int tly,
                                             uint16_t *dst, int r) {
  const int x0 = tlx & ~7, W = sc.width, H = sc.height;
  const int64_t pitch = sc.img_pitch;
  if (tlx >= 0 && tly >= 0 && tlx <= W - 16 && tly <= H - 16) {
    const bool third = x0 + WROW <= W;
#pragma unroll
    for (int j = 0; j < 6; j++) {
      const int k = r + 8 * j, row = k / 3, part = k - row * 3;
      if (part < 2 || third) cp_async16(dst + row * WROW + part * 8, img + (size_t)(tly + row) * pitch + x0 + part * 8);
    }
  } else {
#pragma unroll 1
    for (int j = 0; j < 6; j++) {
      const int k = r + 8 * j, row = k / 3, part = k - row * 3;
      const size_t yo = (size_t)mirror(tly + row, H) * pitch;
#pragma unroll
      for (int e = 0; e < 8; e++) dst[row * WROW + part * 8 + e] = __ldg(img + yo + mirror(x0 + part * 8 + e, W));
    }
  }
}

__device__ __forceinline__ SubtilePlan load_plan(const SceneDev &sc, int task, int s, int c) {
  return sc.plan[((size_t)task * sc.num_sensors + s) * 3 + c];
}

// phase A item c (colour) of a staged tile: the window of (sensor q, c) is in its CLT slot; pn is
// the plan of item c + 1, whose windows are staged once this item's are read
__device__ __forceinline__ void fwd_clt_item_win(const SceneDev &sc, const uint16_t *img, int S, size_t tile, int c,
                                                 const SubtilePlan &p, const SubtilePlan &pn, float *s_clt,
                                                 float *scr, int lane) {
  const int q = lane >> 3, r = lane & 7;
  const int rr = sc.bayer_red_row, rc = sc.bayer_red_col;
  const bool act = q < S;
  const int sidx = act ? q : S - 1;
  SWin w;
  w.base = (const uint16_t *)(s_clt + ((size_t)sidx * 3 + c) * TP_CLT);
  w.sx = p.tlx - (p.tlx & ~7);
  w.scale = sc.color_scale[c];
  float o[4][8];
  float *tbuf = scr + q * 72;
  if (c < 2) {
    const int pc = ((c == 0 ? rc : 1 - rc) - p.tlx) & 1, pr = ((c == 0 ? rr : 1 - rr) - p.tly) & 1;
    subtile_clt<1>(w, p.rx, p.ry, pc, pr, 0, r, tbuf, o);
  } else {
    const int pg = (p.tlx + p.tly + rc + rr + 1) & 1;
    subtile_clt<2>(w, p.rx, p.ry, 0, 0, pg, r, tbuf, o);
  }
  // every lane has read this item's windows (the transposes in subtile_clt synchronise the warp)
  if (c < 2) {
    if (act) stage_window(sc, img, pn.tlx, pn.tly, (uint16_t *)(s_clt + ((size_t)q * 3 + c + 1) * TP_CLT), r);
    cp_async_commit();
  }
  const float *kp = (p.kidx >= 0) ? sc.kernels[sidx] + (size_t)p.kidx * TP_CLT : nullptr;
  conv_shift(o, kp, p.rx, p.ry, r);
  if (act) {
    store_clt(sc, c, r, sc.clt + ((tile * S + q) * 3 + c) * TP_CLT + r * 8, o);
    float *sdst = s_clt + ((size_t)q * 3 + c) * TP_CLT + r * 8;
#pragma unroll
    for (int m = 0; m < 4; m++) {
      *(float4 *)(sdst + m * 64) = make_float4(o[m][0], o[m][1], o[m][2], o[m][3]);
      *(float4 *)(sdst + m * 64 + 4) = make_float4(o[m][4], o[m][5], o[m][6], o[m][7]);
    }
  }
}

template <int NT, bool SPLIT_X>
__global__ void __launch_bounds__(128, 4) fused_forward_win_kernel(const __grid_constant__ SceneDev sc,
                                                                   const __grid_constant__ FwdShape fs,
                                                                   const __grid_constant__ CorrConst cfg) {
  extern __shared__ float sm[];
  __shared__ float s_lpf[64];  // the correlation LPF, read per lane by fwd_pair
  for (int i = threadIdx.x; i < 64; i += blockDim.x) s_lpf[i] = cfg.lpf[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, q = lane >> 3, r = lane & 7;
  const int S = fs.S, P = fs.P, RE = fs.RE, NW = fs.nw;
  float *s_clt = sm + warp * fs.per_warp;
  float *scr = s_clt + fs.clt_floats;
  const short *strip_code = &sc.corr_cfg->strip_code[0][0][0];
  const bool log_mode = cfg.log_combine;
  const int ncomb = cfg.twice_diagonal ? 2 * cfg.num_combo : cfg.num_combo;
  const bool act = q < S;
  const int sidx = act ? q : S - 1;
  const uint16_t *img = (const uint16_t *)sc.images[sidx];
  const int stride = gridDim.x * NW;
  SubtilePlan pc;
  int task = blockIdx.x * NW + warp;
  if (task < sc.num_tasks) {
    pc = load_plan(sc, task, sidx, 0);
    if (act) stage_window(sc, img, pc.tlx, pc.tly, (uint16_t *)(s_clt + (size_t)q * 3 * TP_CLT), r);
    cp_async_commit();
  }
  for (; task < sc.num_tasks; task += stride) {
    const int txy = sc.task_txy[task];
    const size_t tile = (size_t)(txy >> 16) * sc.tilesX + (txy & 0xffff);
#pragma unroll 1
    for (int c = 0; c < 3; c++) {
      const SubtilePlan pn = load_plan(sc, task, sidx, c < 2 ? c + 1 : c);
      cp_async_wait_all();  // this item's windows, copied by every lane
      __syncwarp();
      fwd_clt_item_win(sc, img, S, tile, c, pc, pn, s_clt, scr, lane);
      pc = pn;
    }
    __syncwarp();
    const int next = task + stride;
    if (next < sc.num_tasks) pc = load_plan(sc, next, sidx, 0);
    float cmb[8];
#pragma unroll
    for (int t = 0; t < NT; t++) cmb[t] = log_mode ? 0.f : 1.f;
    float oprod[8];
#pragma unroll
    for (int i = 0; i < 8; i++) oprod[i] = 1.f;
    for (int pi = 0; pi < P; pi++)
      fwd_pair<3, NT, true>(sc, cfg, s_lpf, tile, P, pi, RE, log_mode, strip_code, s_clt, scr, lane, cmb, nullptr,
                            oprod);
    if (next < sc.num_tasks) {  // the CLT slots are read (fwd_pair ends with __syncwarp): next tile's windows
      if (act) stage_window(sc, img, pc.tlx, pc.tly, (uint16_t *)(s_clt + (size_t)q * 3 * TP_CLT), r);
      cp_async_commit();
    }
    if (SPLIT_X) {
      // phase C in extract_kernel: the strip products and ortho profile products go out as they are
#pragma unroll
      for (int t = 0; t < NT; t++) {
        const int e = lane + 32 * t;
        if (e < RE) sc.combo[tile * RE + e] = cmb[t];
      }
      float4 *ob = (float4 *)(sc.osum + (tile * 32 + lane) * 8);
      ob[0] = make_float4(oprod[0], oprod[1], oprod[2], oprod[3]);
      ob[1] = make_float4(oprod[4], oprod[5], oprod[6], oprod[7]);
    } else {
      fwd_extract<NT, true>(sc, cfg, fs.quad, P, RE, log_mode, ncomb, tile, scr, lane, cmb, oprod);
    }
  }
  cp_async_wait_all();
}

// Phase C for the tiles of a fused forward that left it out: warp per task, from the strip
// products (in sc.combo, replaced by the combined strip) and the ortho profile products (sc.osum)
// the forward wrote.  Phase C is short chains of dependent shuffles, divides and powers; the
// fused kernel's 16 warps per SM cannot hide their latency, while this kernel's few registers
// and no CLT buffer let 64 warps share an SM.
template <int NT>
__global__ void __launch_bounds__(128) extract_kernel(const __grid_constant__ SceneDev sc,
                                                      const __grid_constant__ CorrConst cfg, int quad, int RE) {
  __shared__ float s_combo[4][TP_MAX_STRIP * 15];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int task = blockIdx.x * 4 + warp;
  if (task >= sc.num_tasks) return;  // whole warps
  const int txy = sc.task_txy[task];
  const size_t tile = (size_t)(txy >> 16) * sc.tilesX + (txy & 0xffff);
  float cmb[8], oprod[8];
#pragma unroll
  for (int t = 0; t < NT; t++) {
    const int e = lane + 32 * t;
    cmb[t] = (e < RE) ? sc.combo[tile * RE + e] : 0.f;
  }
  const float4 *ob = (const float4 *)(sc.osum + (tile * 32 + lane) * 8);
  const float4 o0 = ob[0], o1 = ob[1];
  oprod[0] = o0.x; oprod[1] = o0.y; oprod[2] = o0.z; oprod[3] = o0.w;
  oprod[4] = o1.x; oprod[5] = o1.y; oprod[6] = o1.z; oprod[7] = o1.w;
  const int ncomb = cfg.twice_diagonal ? 2 * cfg.num_combo : cfg.num_combo;
  float *combo = s_combo[warp];
  const float sum = fwd_extract_values<NT, true>(sc, cfg, quad, sc.num_pairs, RE, cfg.log_combine, ncomb, tile, combo,
                                                 lane, cmb, oprod);
  fwd_extract_finish(sc, cfg, quad, tile, combo, sum, lane);
}

// ---------------------------------------------------------------------------
// pair-per-warp schedule: a CTA of nw warps per tile shares the tile's CLT; the
// warps split the (colour, sensor-group) items, then the pairs, and warp 0
// combines their partial strip products for the extraction.  For many pairs
// (16 sensors, 120 pairs) this holds one CLT per CTA instead of one per warp.
// MAXT / MINB: the launch bounds.  With 3 warps for a quad colour scene (one colour
// item, then two pairs per warp) and 8 CTAs per SM the register budget is 85 per
// thread, for 24 resident warps sharing 8 tile CLTs.
// ---------------------------------------------------------------------------
template <int C, int NT, int MAXT = 128, int MINB = 4>
__global__ void __launch_bounds__(MAXT, MINB) fused_split_kernel(const __grid_constant__ SceneDev sc,
                                                          const __grid_constant__ FwdShape fs,
                                                          const __grid_constant__ CorrConst cfg) {
  extern __shared__ float sm[];
  __shared__ float s_lpf[64];  // the correlation LPF, read per lane by fwd_pair
  for (int i = threadIdx.x; i < 64; i += blockDim.x) s_lpf[i] = cfg.lpf[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = fs.S, P = fs.P, RE = fs.RE, NW = fs.nw;
  float *s_clt = sm;
  float *scr = sm + fs.clt_floats + warp * SCR;
  float *part = sm + fs.clt_floats + NW * SCR;  // [NW][240] partial strip combinations
  const short *strip_code = &sc.corr_cfg->strip_code[0][0][0];
  const int groups = (S + 3) >> 2;
  const bool log_mode = cfg.log_combine;
  const int ncomb = cfg.twice_diagonal ? 2 * cfg.num_combo : cfg.num_combo;
  for (int task = blockIdx.x; task < sc.num_tasks; task += gridDim.x) {
    const int txy = sc.task_txy[task];
    const size_t tile = (size_t)(txy >> 16) * sc.tilesX + (txy & 0xffff);
    for (int gt = warp; gt < C * groups; gt += NW) fwd_clt_item<C>(sc, S, task, tile, gt, groups, s_clt, scr, lane);
    __syncthreads();
    float cmb[8];
#pragma unroll
    for (int t = 0; t < NT; t++) cmb[t] = log_mode ? 0.f : 1.f;
    for (int pi = warp; pi < P; pi += NW)
      fwd_pair<C, NT>(sc, cfg, s_lpf, tile, P, pi, RE, log_mode, strip_code, s_clt, scr, lane, cmb);
#pragma unroll
    for (int t = 0; t < NT; t++) {
      const int e = lane + 32 * t;
      if (e < RE) part[warp * 240 + e] = cmb[t];
    }
    __syncthreads();  // also makes the surfaces every warp wrote visible to warp 0
    if (warp == 0) {
#pragma unroll
      for (int t = 0; t < NT; t++) {
        const int e = lane + 32 * t;
        if (e < RE) {
          float v = part[e];
          for (int w2 = 1; w2 < NW; w2++) v = log_mode ? v + part[w2 * 240 + e] : v * part[w2 * 240 + e];
          cmb[t] = v;
        }
      }
      fwd_extract<NT>(sc, cfg, fs.quad, P, RE, log_mode, ncomb, tile, scr, lane, cmb);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Batched persistent forward over many scenes of different sensor counts,
// colours, pair sets and sizes.  Scenes are grouped in three classes by the
// schedule their tiles take (colour warp-per-tile, mono warp-per-tile, mono
// pair-per-warp); each class is one persistent launch over a queue of units in
// scene order (NW tiles per unit for warp-per-tile, 1 tile per unit for
// pair-per-warp).  CTAs take units grid-stride, find the unit's scene by
// binary search over the unit offsets and keep the current scene's SceneDev in
// shared memory (reloaded only when the scene changes); the scene's
// correlation set-up is read through its device pointer.
// ---------------------------------------------------------------------------
constexpr int BATCH_MAX = 256;

__global__ void disp_init_kernel(float *disp, int n);

int batch_class(const SceneDev &sc) {
  if (sc.num_colors == 3) return 0;
  return sc.num_pairs > 8 ? 2 : 1;
}

static int class_warps(int cls) { return cls == 0 ? 1 : 4; }

int batch_units(const SceneDev &sc) {
  const int nw = batch_class(sc) == 2 ? 1 : class_warps(batch_class(sc));
  return (sc.num_tasks + nw - 1) / nw;
}

template <int C, bool SPLIT, int NW, int NT>
__global__ void __launch_bounds__(NW * 32, (NW == 1) ? 16 : 4)
    fused_batch_kernel(const SceneDev *__restrict__ scenes, const int *__restrict__ unit_off, int nscenes,
                       int total_units, int warp_floats, int cfg_floats) {
  extern __shared__ float smem[];
  __shared__ int s_off[BATCH_MAX + 1];
  __shared__ SceneDev s_sc;
  // the current scene's correlation set-up (header and its pairs) leads the dynamic shared memory
  CorrConst *s_cfg = (CorrConst *)smem;
  float *sm = smem + cfg_floats;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i <= nscenes; i += blockDim.x) s_off[i] = unit_off[i];
  int cur = -1;
  __syncthreads();
  for (int u = blockIdx.x; u < total_units; u += gridDim.x) {
    int lo = 0, hi = nscenes - 1;  // last scene whose first unit is <= u
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_off[mid] <= u) lo = mid;
      else hi = mid - 1;
    }
    if (lo != cur) {
      __syncthreads();
      const int *src = (const int *)(scenes + lo);
      int *dst = (int *)&s_sc;
      for (int i = threadIdx.x; i < (int)(sizeof(SceneDev) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
      const int cfg_words = (int)((offsetof(CorrConst, pairs) + scenes[lo].num_pairs * sizeof(PairDev)) / sizeof(int));
      const int *csrc = (const int *)scenes[lo].corr_cfg;
      for (int i = threadIdx.x; i < cfg_words; i += blockDim.x) ((int *)s_cfg)[i] = csrc[i];
      cur = lo;
      __syncthreads();
    }
    const SceneDev &sc = s_sc;
    const CorrConst &cfg = *s_cfg;
    const int S = sc.num_sensors, P = sc.num_pairs;
    const int RE = (sc.strip_rows < sc.wndy_size ? sc.strip_rows : sc.wndy_size) * 15;
    const short *strip_code = &sc.corr_cfg->strip_code[0][0][0];
    const int groups = (S + 3) >> 2;
    const bool log_mode = cfg.log_combine;
    const int ncomb = cfg.twice_diagonal ? 2 * cfg.num_combo : cfg.num_combo;
    const int lu = u - s_off[lo];
    if (SPLIT) {
      float *s_clt = sm;
      float *scr = sm + S * TP_CLT + warp * SCR;
      float *part = sm + S * TP_CLT + NW * SCR;
      const int task = lu;
      const int txy = sc.task_txy[task];
      const size_t tile = (size_t)(txy >> 16) * sc.tilesX + (txy & 0xffff);
      for (int gt = warp; gt < groups; gt += NW) fwd_clt_item<C>(sc, S, task, tile, gt, groups, s_clt, scr, lane);
      __syncthreads();
      float cmb[8];
#pragma unroll
      for (int t = 0; t < NT; t++) cmb[t] = log_mode ? 0.f : 1.f;
      for (int pi = warp; pi < P; pi += NW)
        fwd_pair<C, NT>(sc, cfg, cfg.lpf, tile, P, pi, RE, log_mode, strip_code, s_clt, scr, lane, cmb);
#pragma unroll
      for (int t = 0; t < NT; t++) {
        const int e = lane + 32 * t;
        if (e < RE) part[warp * 240 + e] = cmb[t];
      }
      __syncthreads();
      if (warp == 0) {
#pragma unroll
        for (int t = 0; t < NT; t++) {
          const int e = lane + 32 * t;
          if (e < RE) {
            float v = part[e];
            for (int w2 = 1; w2 < NW; w2++) v = log_mode ? v + part[w2 * 240 + e] : v * part[w2 * 240 + e];
            cmb[t] = v;
          }
        }
        fwd_extract<NT>(sc, cfg, P <= 8, P, RE, log_mode, ncomb, tile, scr, lane, cmb);
      }
      __syncthreads();
    } else {
      const int task = lu * NW + warp;
      if (task < sc.num_tasks) {
        float *s_clt = sm + warp * warp_floats;
        float *scr = s_clt + S * C * TP_CLT;
        const int txy = sc.task_txy[task];
        const size_t tile = (size_t)(txy >> 16) * sc.tilesX + (txy & 0xffff);
        for (int gt = 0; gt < C * groups; gt++) fwd_clt_item<C>(sc, S, task, tile, gt, groups, s_clt, scr, lane);
        __syncwarp();
        float cmb[8];
#pragma unroll
        for (int t = 0; t < NT; t++) cmb[t] = log_mode ? 0.f : 1.f;
        for (int pi = 0; pi < P; pi++)
          fwd_pair<C, NT>(sc, cfg, cfg.lpf, tile, P, pi, RE, log_mode, strip_code, s_clt, scr, lane, cmb);
        fwd_extract<NT>(sc, cfg, P <= 8, P, RE, log_mode, ncomb, tile, scr, lane, cmb);
      }
    }
  }
}

template <typename K>
static cudaError_t launch_batch_k(K kernel, int threads, int bytes, int total_units, const SceneDev *scenes_dev,
                                  const int *unit_off_dev, int n, int warp_floats, int cfg_floats, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 152, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, bytes);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int grid = total_units < sms * per_sm ? total_units : sms * per_sm;
  kernel<<<grid, threads, bytes, st>>>(scenes_dev, unit_off_dev, n, total_units, warp_floats, cfg_floats);
  return cudaGetLastError();
}

// one class: scenes_host / scenes_dev hold only that class's scenes, unit_off_dev their unit offsets
cudaError_t launch_fused_batch(int cls, const SceneDev *scenes_host, const SceneDev *scenes_dev,
                               const int *unit_off_dev, int n, int total_units, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (n > BATCH_MAX) return cudaErrorInvalidValue;
  int wf = 0, sp = 0, maxp = 0, maxre = 0;
  for (int i = 0; i < n; i++) {
    maxp = scenes_host[i].num_pairs > maxp ? scenes_host[i].num_pairs : maxp;
    const int re = (scenes_host[i].strip_rows < scenes_host[i].wndy_size ? scenes_host[i].strip_rows
                                                                         : scenes_host[i].wndy_size) * 15;
    maxre = re > maxre ? re : maxre;
    const SceneDev &sc = scenes_host[i];
    if (batch_class(sc) != cls || sc.strip_rows * 15 > 8 * 32) return cudaErrorInvalidValue;
    const int ntiles = sc.tilesX * sc.tilesY;
    disp_init_kernel<<<(ntiles * TP_NDISP + 255) / 256, 256, 0, st>>>(sc.disp, ntiles);
    const int f = ((sc.num_sensors * sc.num_colors * TP_CLT + SCR) + 3) & ~3;
    wf = f > wf ? f : wf;
    const int g = sc.num_sensors * TP_CLT + 4 * SCR + 4 * 240;
    sp = g > sp ? g : sp;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || total_units <= 0) return e;
  const int cf = (int)(((offsetof(CorrConst, pairs) + maxp * sizeof(PairDev)) + 15) / 16 * 4);
  if (maxre <= 32) {
    if (cls == 0) return launch_batch_k(fused_batch_kernel<3, false, 1, 1>, 32, (cf + wf) * 4, total_units,
                                        scenes_dev, unit_off_dev, n, wf, cf, st);
    if (cls == 1) return launch_batch_k(fused_batch_kernel<1, false, 4, 1>, 128, (cf + 4 * wf) * 4, total_units,
                                        scenes_dev, unit_off_dev, n, wf, cf, st);
    return launch_batch_k(fused_batch_kernel<1, true, 4, 1>, 128, (cf + sp) * 4, total_units, scenes_dev,
                          unit_off_dev, n, 0, cf, st);
  }
  if (cls == 0) return launch_batch_k(fused_batch_kernel<3, false, 1, 8>, 32, (cf + wf) * 4, total_units, scenes_dev,
                                      unit_off_dev, n, wf, cf, st);
  if (cls == 1) return launch_batch_k(fused_batch_kernel<1, false, 4, 8>, 128, (cf + 4 * wf) * 4, total_units,
                                      scenes_dev, unit_off_dev, n, wf, cf, st);
  return launch_batch_k(fused_batch_kernel<1, true, 4, 8>, 128, (cf + sp) * 4, total_units, scenes_dev, unit_off_dev,
                        n, 0, cf, st);
}

// ---------------------------------------------------------------------------
// Rig (two quad cameras): inter-camera correlation of the sensor-averaged CLT
// of each camera (Correlation2d.correlateInterCamerasFD / cltMixCameras,
// Correlation2d.java:401-448) and its disparity along the horizontal rig
// baseline (ImageDtt.tileInterCamCorrs, ImageDtt.java:7370-7560, without the
// LMA branch).  Warp per tile of the main camera's task list; the correlation
// is the forward kernel's pair phase run on the two averaged CLTs.
// ---------------------------------------------------------------------------
template <int C, int NT>
__global__ void __launch_bounds__(128, 4) rig_kernel(const __grid_constant__ SceneDev mn,
                                                     const __grid_constant__ SceneDev ax,
                                                     const __grid_constant__ CorrConst cfg, float *rig_corr,
                                                     float *rig_rec, float cm_norm, int no_int_x0, int per_warp) {
  extern __shared__ float sm[];
  __shared__ float s_lpf[64];  // the correlation LPF, read per lane by fwd_pair
  for (int i = threadIdx.x; i < 64; i += blockDim.x) s_lpf[i] = cfg.lpf[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, NW = blockDim.x >> 5;
  float *mix = sm + warp * per_warp;  // [2][C][256]
  float *scr = mix + 2 * C * TP_CLT;
  const int RE = (cfg.strip_rows < cfg.wndy_size ? cfg.strip_rows : cfg.wndy_size) * 15;
  const short *strip_code = &mn.corr_cfg->strip_code[0][0][0];
  const int ncomb = cfg.twice_diagonal ? 2 : 1;
  for (int task = blockIdx.x * NW + warp; task < mn.num_tasks; task += gridDim.x * NW) {
    const int txy = mn.task_txy[task];
    const size_t tile = (size_t)(txy >> 16) * mn.tilesX + (txy & 0xffff);
    float *rec = rig_rec + tile * 4;
    if (ax.tile_task[tile] < 0) {
      if (lane < 4) rec[lane] = (lane == 1) ? 0.f : CUDART_NAN_F;
      continue;
    }
    for (int i = lane; i < C * TP_CLT; i += 32) {
      float a = 0.f, b = 0.f;
      for (int s = 0; s < mn.num_sensors; s++) a += mn.clt[(tile * mn.num_sensors + s) * C * TP_CLT + i];
      for (int s = 0; s < ax.num_sensors; s++) b += ax.clt[(tile * ax.num_sensors + s) * C * TP_CLT + i];
      mix[i] = a * (1.0f / mn.num_sensors);
      mix[C * TP_CLT + i] = b * (1.0f / ax.num_sensors);
    }
    __syncwarp();
    float cmb[8];
#pragma unroll
    for (int t = 0; t < NT; t++) cmb[t] = 1.f;
    fwd_pair<C, NT>(mn, cfg, s_lpf, tile, 1, 0, RE, false, strip_code, mix, scr, lane, cmb, rig_corr + tile * TP_CORR);
    float *combo = scr;
#pragma unroll
    for (int t = 0; t < NT; t++) {
      const int e = lane + 32 * t;
      if (e < RE) {
        float v = cmb[t];
        if (v > 0.0f) v = powf(v, 1.0f / ncomb) - cfg.corr_offset;
        combo[e] = v;
      }
    }
    __syncwarp();
    float r0 = CUDART_NAN_F, r1 = 0.f;
    const float v = (lane < 15) ? combo[lane] : CUDART_NAN_F;
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
    const float vmax = combo[imx];
    if (vmax >= (no_int_x0 ? 0.5f : 1.0f) * cfg.min_corr) {
      const int ix = imx - 7;
      r0 = (float)(-ix);
      r1 = vmax;
      int dh = cfg.strip_rows;
      float wys = 1.0f;
      if (dh > cfg.wndy_size) dh = cfg.wndy_size;
      else if (dh < cfg.wndy_size) {
        float swy = cfg.wndy[0];
        for (int i = 1; i < dh; i++) swy += cfg.wndy[i];
        wys = 1.0f / swy;
      }
      const int ixc = no_int_x0 ? 0 : ix;
      const int x0 = 7 + ixc, nk = dh * 2 * cfg.wndx_size;
      float s0 = 0.f, sx = 0.f, sx2 = 0.f;
      for (int k = lane; k < nk; k += 32) {  // getMaxXCm with the second moment
        const int dy = k / (2 * cfg.wndx_size), rest = k - dy * 2 * cfg.wndx_size;
        const int adx = rest >> 1, dir = (rest & 1) ? 1 : -1, odd = dy & 1;
        if (((adx - odd) & 1) || (adx == 0 && dir < 0)) continue;
        const int idx = (adx * dir) >> 1, xx = 2 * idx + odd, x1 = x0 + idx;
        if (x1 < 0 || x1 >= 15) continue;
        float d = combo[dy * 15 + x1];
        if (isnan(d) || !(d > 0.0f)) continue;
        d *= (((dy == 0) ? wys : 2.0f * wys) * cfg.wndy[dy]) * cfg.wndx[adx];
        s0 += d;
        sx += d * xx;
        sx2 += d * xx * xx;
      }
      s0 = warp_sum(s0);
      sx = warp_sum(sx);
      sx2 = warp_sum(sx2);
      if (s0 != 0.0f) {
        r0 = -(ixc + sx / s0 / 2);
        const float sigma = sqrtf(s0 * sx2 - sx * sx) / s0 / 2, eff = sigma * cm_norm;
        r1 = s0 / (eff * eff);
      }
    }
    if (lane < 4) rec[lane] = (lane == 0) ? r0 : ((lane == 1) ? r1 : CUDART_NAN_F);
    __syncwarp();
  }
}

// tiles without a main-camera task keep {NaN, 0, NaN, NaN}
__global__ void rig_init_kernel(float *rig_rec, int ntiles) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ntiles * 4) rig_rec[i] = ((i & 3) == 1) ? 0.f : CUDART_NAN_F;
}

cudaError_t launch_rig(const SceneDev &mn, const SceneDev &ax, const CorrConst &cc, float *rig_corr, float *rig_rec,
                       float cm_norm, int no_int_x0, cudaStream_t st) {
  const int ntiles = mn.tilesX * mn.tilesY;
  rig_init_kernel<<<(ntiles * 4 + 255) / 256, 256, 0, st>>>(rig_rec, ntiles);
  if (mn.num_tasks <= 0) return cudaGetLastError();
  const int C = mn.num_colors;
  const int RE = (cc.strip_rows < cc.wndy_size ? cc.strip_rows : cc.wndy_size) * 15;
  const int per_warp = ((2 * C * TP_CLT + SCR) + 3) & ~3, nw = 4, bytes = per_warp * nw * 4;
  const int units = (mn.num_tasks + nw - 1) / nw;
  auto go = [&](auto kernel) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 152, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, nw * 32, bytes);
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const int grid = units < sms * per_sm ? units : sms * per_sm;
    kernel<<<grid, nw * 32, bytes, st>>>(mn, ax, cc, rig_corr, rig_rec, cm_norm, no_int_x0, per_warp);
    return cudaGetLastError();
  };
  if (RE <= 32) return C == 3 ? go(rig_kernel<3, 1>) : go(rig_kernel<1, 1>);
  return C == 3 ? go(rig_kernel<3, 8>) : go(rig_kernel<1, 8>);
}

// ---------------------------------------------------------------------------
// IMCLT (ImageDtt.iclt_2d, the reference GPU imclt_rbg) with overlap-add into the
// padded colour frames.  CTA = one 64x64-pixel region of one (sensor, colour)
// plane; the 9x9 tiles touching it are processed in the four tile-parity phases
// (tiles of one phase never overlap), so the region accumulates in shared memory
// without atomics and in a fixed order.  A warp carries 4 tiles at once, one per
// 8-lane group, lane r owning row r of each quadrant.
// ---------------------------------------------------------------------------
constexpr int IMCLT_IR = 14;     // region = IR x IR blocks of 8x8 pixels (14: 0.41 ms, 16: 0.43, 12: 0.44 on 4x2592x1936)
constexpr int IMCLT_WARPS = 9;   // 36 8-lane groups: the four parity phases (49, 56, 56, 64 tiles) in 2 rounds each

template <int IR>
__global__ void __launch_bounds__(32 * IMCLT_WARPS) imclt_fast_kernel(const __grid_constant__ SceneDev sc) {
  constexpr int IPX = IR * 8, ISTR = IPX + 1;
  extern __shared__ float acc[];  // [IPX][ISTR]
  __shared__ float tbuf_all[IMCLT_WARPS][4 * 72];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, q = lane >> 3, r = lane & 7;
  const int S = sc.num_sensors, C = sc.num_colors;
  const int plane = blockIdx.z, s = plane / C, c = plane - s * C;
  const int bx0 = blockIdx.x * IR, by0 = blockIdx.y * IR;
  const int fw = sc.width + 8, fh = sc.height + 8;
  for (int i = threadIdx.x; i < IPX * ISTR; i += blockDim.x) acc[i] = 0.f;
  __syncthreads();
  float *tbuf = tbuf_all[warp] + q * 72;
  // (a stored CLT that already carries the LPF, clt_lpf_mask, is not filtered again)
  const float *lpf = (sc.lpf_rbg && !((sc.clt_lpf_mask >> c) & 1)) ? sc.lpf_rbg + c * 64 : nullptr;
  // unfold rows fed by source row r (DttRad2.get_unfold_index_signs, 392-404)
  const int i1 = (r >= 4) ? r - 4 : 11 - r, i2 = (r >= 4) ? 11 - r : r + 12;
  const float sa1 = (r >= 4) ? 1.f : -1.f, sb1 = 1.f;    // signs (cos, sin branch) of row i1
  const float sa2 = -1.f, sb2 = (r >= 4) ? 1.f : -1.f;   // signs of row i2
  const float w1 = k_hwin[i1 < 8 ? i1 : 15 - i1], w2 = k_hwin[i2 < 8 ? i2 : 15 - i2];
  const float kc1 = sa1 * w1, ks1 = sb1 * w1, kc2 = sa2 * w2, ks2 = sb2 * w2;
  float lk[8];  // 0.25 x the colour's LPF for row r (the iclt_2d scale)
#pragma unroll
  for (int v = 0; v < 8; v++) lk[v] = 0.25f * (lpf ? lpf[r * 8 + v] : 1.0f);
  for (int ph = 0; ph < 4; ph++) {
    const int pxp = ph & 1, pyp = ph >> 1;
    int tx0 = bx0 - 1, ty0 = by0 - 1;
    if ((tx0 & 1) != pxp) tx0++;
    if ((ty0 & 1) != pyp) ty0++;
    const int ntx = (bx0 + IR - 1 - tx0) / 2 + 1, nty = (by0 + IR - 1 - ty0) / 2 + 1;
    for (int k0 = warp * 4; k0 < ntx * nty; k0 += 4 * IMCLT_WARPS) {
      const int k = k0 + q;
      const int tx = tx0 + 2 * (k % ntx), ty = ty0 + 2 * (k / ntx);
      bool act = k < ntx * nty && tx >= 0 && ty >= 0 && tx < sc.tilesX && ty < sc.tilesY;
      size_t tile = act ? (size_t)ty * sc.tilesX + tx : 0;
      if (act && sc.tile_task[tile] < 0) act = false;
      float o[4][8];
      const float *src = sc.clt + ((tile * S + s) * C + c) * TP_CLT + r * 8;
#pragma unroll
      for (int m = 0; m < 4; m++) {
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
        if (act) {
          a = __ldg((const float4 *)(src + m * 64));
          b = __ldg((const float4 *)(src + m * 64 + 4));
        }
        o[m][0] = a.x; o[m][1] = a.y; o[m][2] = a.z; o[m][3] = a.w;
        o[m][4] = b.x; o[m][5] = b.y; o[m][6] = b.z; o[m][7] = b.w;
      }
#pragma unroll
      for (int v = 0; v < 8; v++)
#pragma unroll
        for (int m = 0; m < 4; m++) o[m][v] *= lk[v];
      // inverse 2D DCT-IV/DST-IV with the swapped mode (ImageDtt.java:3628):
      // rows (vertical frequency) first, then columns
      float t[4][8];
#pragma unroll
      for (int m = 0; m < 4; m++) {
        float z[8];
        dtt4_fast(o[m], z, (m >> 1) & 1);
        group_transpose(z, tbuf, r);
        dtt4_fast(z, t[m], m & 1);  // lane r: vertical position r, t[m][x] horizontal position x
      }
      // unfold (DttRad2.unfold_tile) into rows i1, i2 and accumulate
      const int gy1 = ty * 8 + i1 - by0 * 8, gy2 = ty * 8 + i2 - by0 * 8;
#pragma unroll
      for (int jj = 0; jj < 16; jj++) {
        const int seg = jj >> 2, xx = jj & 3;
        const int ih = (seg == 0) ? xx + 4 : ((seg == 1) ? 7 - xx : ((seg == 2) ? 3 - xx : xx));
        const float hs1 = (seg == 0) ? 1.f : -1.f, hs2 = (seg == 3) ? -1.f : 1.f;
        const float wh = k_hwin[jj < 8 ? jj : 15 - jj];
        const float khc = hs1 * wh, khs = hs2 * wh;
        const float A = fmaf(khs, t[1][ih], khc * t[0][ih]);
        const float B = fmaf(khs, t[3][ih], khc * t[2][ih]);
        const int gx = tx * 8 + jj - bx0 * 8;
        if (act && gx >= 0 && gx < IPX) {
          if (gy1 >= 0 && gy1 < IPX) acc[gy1 * ISTR + gx] += fmaf(ks1, B, kc1 * A);
          if (gy2 >= 0 && gy2 < IPX) acc[gy2 * ISTR + gx] += fmaf(ks2, B, kc2 * A);
        }
      }
    }
    __syncthreads();
  }
  float *dst = sc.rbg + (size_t)plane * fw * fh;
  for (int i = threadIdx.x; i < IPX * IPX; i += blockDim.x) {
    const int ly = i / IPX, lx = i - ly * IPX;
    const int gx = bx0 * 8 + lx, gy = by0 * 8 + ly;
    if (gx < fw && gy < fh) dst[(size_t)gy * fw + gx] = acc[ly * ISTR + lx];
  }
}

cudaError_t launch_imclt_fast(const SceneDev &sc, cudaStream_t st) {
  constexpr int IR = IMCLT_IR;
  const int bytes = IR * 8 * (IR * 8 + 1) * 4;
  cudaError_t e = cudaFuncSetAttribute(imclt_fast_kernel<IR>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  dim3 grid((sc.tilesX + 1 + IR - 1) / IR, (sc.tilesY + 1 + IR - 1) / IR, sc.num_sensors * sc.num_colors);
  imclt_fast_kernel<IR><<<grid, 32 * IMCLT_WARPS, bytes, st>>>(sc);
  return cudaGetLastError();
}

__global__ void disp_init_kernel(float *disp, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n * TP_NDISP) {
    int k = i % TP_NDISP;
    disp[i] = (k == 2 || k == 4 || k == 6) ? 0.0f : CUDART_NAN_F;
  }
}

cudaError_t upload_fused_constants() { return upload_dtt_constants(); }

// GPU_DTT24_DRV (dtt8x8.cuh:100-158): every 8x8 block of a float image through the 2D transform of
// one mode, rows first (bit 0: DST), then columns (bit 1); modes 0-3 DCT-IV / DST-IV, 4-7 the
// orthonormal DCT-II / DST-II (the DCT-IIe butterflies with the constant term scaled by 1/sqrt 2).
// An 8-lane group per block, lane r holding row r, then column r after the transpose.
__device__ __forceinline__ void dtt8_mode(const float x[8], float y[8], int mode, bool sine) {
  if (mode < 4) {
    dtt4_fast(x, y, sine);
  } else {
    dtt2e_fast(x, y, sine);
    if (sine) y[7] *= 0.70710678118654752f;
    else y[0] *= 0.70710678118654752f;
  }
}

__global__ void __launch_bounds__(128) dtt8x8_kernel(float *dst, const float *src, int stride, int bw, int nblocks,
                                                     int mode) {
  __shared__ float tb[16][72];
  const int g = threadIdx.x >> 3, r = threadIdx.x & 7;
  const int blk = blockIdx.x * 16 + g;
  const bool act = blk < nblocks;
  const int b = act ? blk : nblocks - 1;  // every group takes part in the warp's transposes
  const int by = b / bw, bx = b - by * bw;
  const float *s = src + (size_t)(by * 8 + r) * stride + bx * 8;
  float x[8], y[8];
#pragma unroll
  for (int c = 0; c < 8; c++) x[c] = s[c];
  dtt8_mode(x, y, mode, mode & 1);
  group_transpose(y, tb[g], r);
  dtt8_mode(y, x, mode, (mode >> 1) & 1);
  group_transpose(x, tb[g], r);
  if (act) {
    float *d = dst + (size_t)(by * 8 + r) * stride + bx * 8;
#pragma unroll
    for (int c = 0; c < 8; c++) d[c] = x[c];
  }
}

cudaError_t launch_dtt8x8(float *dst, const float *src, int stride, int width, int height, int mode,
                          cudaStream_t st) {
  const int bw = width / 8, nblocks = bw * (height / 8);
  if (nblocks <= 0) return cudaSuccess;
  dtt8x8_kernel<<<(nblocks + 15) / 16, 128, 0, st>>>(dst, src, stride, bw, nblocks, mode);
  return cudaGetLastError();
}

static FwdShape make_shape(const SceneDev &sc, int nw) {
  FwdShape f;
  f.S = sc.num_sensors;
  f.C = sc.num_colors;
  f.P = sc.num_pairs;
  // only the strip rows the extraction reads are built: getMaxXYInt uses row 0 and
  // getMaxXCm clips the strip to the y-window (Correlation2d.java:944-951)
  f.RE = (sc.strip_rows < sc.wndy_size ? sc.strip_rows : sc.wndy_size) * 15;
  f.quad = (sc.num_pairs <= 8) ? 1 : 0;
  f.nw = nw > 0 ? nw : 4;  // the autotuner's pick on 4x2592x1936 Bayer and 4x512x384 mono
  f.clt_floats = f.S * f.C * TP_CLT;
  f.per_warp = f.clt_floats + SCR;
  f.per_warp = (f.per_warp + 3) & ~3;
  return f;
}

static int split_smem_floats(const FwdShape &f) { return f.clt_floats + f.nw * SCR + f.nw * 240; }

template <typename K>
static cudaError_t launch_persistent(K kernel, int threads, int bytes, int units, const SceneDev &sc,
                                     const FwdShape &f, const CorrConst &cc, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 152, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, bytes);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int grid = units < sms * per_sm ? units : sms * per_sm;
  kernel<<<grid, threads, bytes, st>>>(sc, f, cc);
  return cudaGetLastError();
}

// Schedules: tiles_per_block == warps_per_block (<= 4): warp per tile;
// tiles_per_block == 1 with warps_per_block 2, 3 or 4: pair per warp (CTA per tile).
cudaError_t launch_fused_forward(const SceneDev &sc, const CorrConst &cc, int tpb, int nw, cudaStream_t st) {
  const int ntiles = sc.tilesX * sc.tilesY;
  disp_init_kernel<<<(ntiles * TP_NDISP + 255) / 256, 256, 0, st>>>(sc.disp, ntiles);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || sc.num_tasks <= 0) return e;
  if (sc.strip_rows * 15 > 8 * 32) return cudaErrorInvalidConfiguration;
  if (tpb <= 0 && nw <= 0 && sc.num_pairs > 8) {  // default for many pairs: four warps share a tile
    tpb = 1;
    nw = 4;
  }
  FwdShape f = make_shape(sc, nw);
  if (f.nw > 4) return cudaErrorInvalidConfiguration;
  if (tpb == 1 && f.nw > 1) {
    const int bytes = split_smem_floats(f) * 4;
    if (f.nw == 3) {  // quad colour scenes: one colour item per warp, 8 CTAs per SM
      if (f.RE <= 32)
        return sc.num_colors == 3
                   ? launch_persistent(fused_split_kernel<3, 1, 96, 8>, 96, bytes, sc.num_tasks, sc, f, cc, st)
                   : launch_persistent(fused_split_kernel<1, 1, 96, 8>, 96, bytes, sc.num_tasks, sc, f, cc, st);
      return sc.num_colors == 3
                 ? launch_persistent(fused_split_kernel<3, 8, 96, 8>, 96, bytes, sc.num_tasks, sc, f, cc, st)
                 : launch_persistent(fused_split_kernel<1, 8, 96, 8>, 96, bytes, sc.num_tasks, sc, f, cc, st);
    }
    if (f.RE <= 32)
      return sc.num_colors == 3
                 ? launch_persistent(fused_split_kernel<3, 1>, f.nw * 32, bytes, sc.num_tasks, sc, f, cc, st)
                 : launch_persistent(fused_split_kernel<1, 1>, f.nw * 32, bytes, sc.num_tasks, sc, f, cc, st);
    return sc.num_colors == 3
               ? launch_persistent(fused_split_kernel<3, 8>, f.nw * 32, bytes, sc.num_tasks, sc, f, cc, st)
               : launch_persistent(fused_split_kernel<1, 8>, f.nw * 32, bytes, sc.num_tasks, sc, f, cc, st);
  }
  const int bytes = f.per_warp * f.nw * 4;
  const int units = (sc.num_tasks + f.nw - 1) / f.nw;
  bool all16 = true;
  for (int i = 0; i < sc.num_sensors; i++) all16 = all16 && sc.img_dtype[i] == 1;
  if (sc.num_colors == 3 && sc.num_sensors <= 4 && all16) {  // staged windows
    if (sc.combo && sc.osum) {  // the extraction's serial half in its own pass
      e = (f.RE <= 32) ? launch_persistent(fused_forward_win_kernel<1, true>, f.nw * 32, bytes, units, sc, f, cc, st)
                       : launch_persistent(fused_forward_win_kernel<8, true>, f.nw * 32, bytes, units, sc, f, cc, st);
      if (e != cudaSuccess) return e;
      if (f.RE <= 32) extract_kernel<1><<<(sc.num_tasks + 3) / 4, 128, 0, st>>>(sc, cc, f.quad, f.RE);
      else extract_kernel<8><<<(sc.num_tasks + 3) / 4, 128, 0, st>>>(sc, cc, f.quad, f.RE);
      return cudaGetLastError();
    }
    if (f.RE <= 32) return launch_persistent(fused_forward_win_kernel<1, false>, f.nw * 32, bytes, units, sc, f, cc, st);
    return launch_persistent(fused_forward_win_kernel<8, false>, f.nw * 32, bytes, units, sc, f, cc, st);
  }
  if (f.RE <= 32)
    return sc.num_colors == 3 ? launch_persistent(fused_forward_kernel<3, 1>, f.nw * 32, bytes, units, sc, f, cc, st)
                              : launch_persistent(fused_forward_kernel<1, 1>, f.nw * 32, bytes, units, sc, f, cc, st);
  return sc.num_colors == 3 ? launch_persistent(fused_forward_kernel<3, 8>, f.nw * 32, bytes, units, sc, f, cc, st)
                            : launch_persistent(fused_forward_kernel<1, 8>, f.nw * 32, bytes, units, sc, f, cc, st);
}
