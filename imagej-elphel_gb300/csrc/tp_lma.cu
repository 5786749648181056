// tp_lma.cu -- LMA disparity of the quad layout ("POLY", the reference's default
// disparity when mix_corr_poly is set): Correlation2d.corrLMA
// (Correlation2d.java:1754-1877) on the correlation surfaces of the last forward.
//
//  * the pairs are combined into an ortho group (horizontal as-is, vertical
//    transposed) and a diagonal group (main as-is, other flipped vertically),
//    each the mean of its pairs (combineCompatiblePairs 462-490);
//  * around the CM centre each group keeps the cells reached from it through
//    bi-convex cells in at most cnvx_hwnd_size steps (filterConvex 2029-2208)
//    and turns them into samples weighted by weight x pairs x |value|^vasw_pwr
//    (addSamples 2230-2386);
//  * the samples are fitted by Ag (1 - ((x - x0) s / Wx)^2 - (y s / Wy)^2) per
//    group (s = sqrt 2 for the diagonal group) with Levenberg-Marquardt and
//    the reference's lambda schedule (Correlations2dLMA.java:211-640).
//
// One warp per tile: cells and samples are spread over the lanes, the region
// growth runs one step per warp-synchronous pass, and the normal equations are
// reduced across the warp and solved redundantly by every lane (FP32).
#include "tp_dtt.cuh"

#include <cmath>

namespace {

constexpr int LMA_NW = 4;             // warps (tiles) per CTA
constexpr int LMA_ORTHO_ENTRIES = 81;  // addSamples enumeration, ortho group
constexpr int LMA_DIAG_ENTRIES = 145;  // addSamples enumeration, diagonal group
constexpr int LMA_MAX_SAMPLES = 162;   // 9x9 window cells per group
constexpr int LMA_NP = 6;              // X0, WM, WYD, WXY, AG0, AG1
constexpr int LMA_STAGE_PAIRS = 6;     // pair surfaces staged in shared memory (the quad layout's six)
constexpr int LMA_POLY_CHUNK = 6;      // pairs per polynomial-mismatch pass (one solving lane each)
constexpr int LMA_POLY_SCRATCH = 48;   // doubles of solver scratch per lane

// sample cell offsets from the (integer) centre, in the reference's enumeration order (global
// memory: consecutive lanes read consecutive entries)
__device__ signed char g_lma_cx[LMA_ORTHO_ENTRIES + LMA_DIAG_ENTRIES];
__device__ signed char g_lma_cy[LMA_ORTHO_ENTRIES + LMA_DIAG_ENTRIES];

__device__ __forceinline__ void cp_async4(float *dst_smem, const float *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(float *dst_smem, const float *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}

// per-warp shared memory (floats): group surfaces [2][225], samples x/y/v/w [4][162] + group bytes,
// the reduction buffer [28][33], accepted / trial normal equations, and the staged pair surfaces,
// which start on a 16-byte boundary for the 8-byte asynchronous copies
constexpr int LMA_OFF_RED = 450 + 4 * LMA_MAX_SAMPLES + LMA_MAX_SAMPLES / 4 + 1;
constexpr int LMA_OFF_STAGE = ((LMA_OFF_RED + 28 * 33 + 64) + 3) & ~3;
constexpr int LMA_OFF_RES = LMA_OFF_STAGE + LMA_STAGE_PAIRS * 225;  // [4][4] orientation fits
constexpr int LMA_PER_WARP = ((LMA_OFF_RES + 16) + 3) & ~3;
static_assert(LMA_OFF_STAGE % 4 == 0 && LMA_PER_WARP % 4 == 0, "staged surfaces must be 16-byte aligned");
// polynomial mismatch scratch: moments over the reduction buffer, solver rows over the group
// surfaces and samples, both 8-byte aligned and clear of the staged surfaces
static_assert(((LMA_OFF_RED + 1) & ~1) + 2 * 21 * LMA_POLY_CHUNK <= LMA_OFF_STAGE, "moments overlap the stage");
static_assert(2 * LMA_POLY_SCRATCH * LMA_POLY_CHUNK <= LMA_OFF_RED, "solver scratch overlaps the moments");
static_assert(LMA_POLY_CHUNK <= 32, "one solving lane per pair");

struct LmaDev {
  const float *corr;   // [tiles][P][225]
  float *disp;         // [tiles][TP_NDISP]
  float *lma;          // [tiles][4]
  float *mismatch;     // [tiles][P][3] lazy-eye mismatch, or null
  const int *task_txy;
  int num_tasks, tilesX, P;
  int kinds[TP_MAXP];  // pair kind or -1 when the pair does not take part
  int kind_count[4];   // taking part per kind
};

// Correlation2d.foregroundCorrect (Correlation2d.java:1663-1749) on the four orientation fits
// (rows {disparity, strength, WM, WXY}); returns the corrected disparity (full_disp if none)
__device__ __forceinline__ float foreground_correct(const TpLmaConst &c, const float dir[4][4], const bool valid[4],
                                                   float full_disp, float &spread) {
  float mn = CUDART_NAN_F, mx = CUDART_NAN_F, eff[4], width_d[4];
  int imn = -1, imx = -1;
  bool strong[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    strong[i] = false;
    width_d[i] = 0.f;
    eff[i] = CUDART_NAN_F;
    if (valid[i]) {
      if (isnan(mn) || dir[i][0] < mn) { mn = dir[i][0]; imn = i; }
      if (isnan(mx) || dir[i][0] > mx) { mx = dir[i][0]; imx = i; }
      eff[i] = dir[i][1] * (dir[i][2] - dir[i][3]) / (dir[i][2] + dir[i][3]);
      width_d[i] = dir[i][2] + dir[i][3];
      strong[i] = (dir[i][1] >= c.fo_min_strength) && (eff[i] >= c.fo_min_eff);
    }
  }
  const bool are_ortho = (imn ^ imx) == 1;
  float corr = c.fo_overcorrection * (mx - mn);
  const int isel = c.fo_far ? imn : imx, iother = c.fo_far ? imx : imn, iortho = isel ^ 1;
  // the indexed reads as selects, so the small arrays stay in registers
  float e_sel = 0.f, w_sel = 0.f, e_ortho = 0.f;
  bool s_sel = false, s_other = false;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    if (i == isel) { e_sel = eff[i]; w_sel = width_d[i]; s_sel = strong[i]; }
    if (i == iortho) e_ortho = eff[i];
    if (i == iother) s_other = strong[i];
  }
  if (isel < 0 || !s_sel) corr = CUDART_NAN_F;
  else if (w_sel > c.fo_max_hwidth) corr = CUDART_NAN_F;
  else if (e_sel / e_ortho < c.fo_min_eff_ratio) corr = CUDART_NAN_F;
  else {
    if (c.fo_ortho && !are_ortho) corr = 0.0f;
    else if (!s_other) corr = 0.0f;
    if (!(mx >= (mn + c.fo_min_diff))) corr = CUDART_NAN_F;
  }
  float disp = full_disp;
  if (!isnan(corr)) {
    if (c.fo_far) disp = fmaxf(mn - corr, full_disp - (full_disp - mn) * c.fo_lim_overcorr);
    else disp = fminf(mx + corr, full_disp + (mx - full_disp) * c.fo_lim_overcorr);
  }
  spread = mx - mn;
  return disp;
}

// Correlation2d.mismatchPairsCM (Correlation2d.java:1336-1431) for one pair of quad kind k:
// centre of mass of the positive cells within the radius around the pair's expected peak
__device__ __forceinline__ void mismatch_cm(const float *cs, int k, float xcenter, float radius, float out[3]) {
  const int ixc = (int)floorf(xcenter + 0.5f);
  const int icx = (k == 1) ? 0 : ixc, icy = (k == 0) ? 0 : ((k == 3) ? -ixc : ixc);
  const int iradius = (int)fabsf(radius), ir2 = (int)(radius * radius);
  const bool square = radius < 0.f;
  float s0 = 0.f, sx = 0.f, sy = 0.f;
  for (int y = -iradius; y <= iradius; y++) {
    const int dy = icy + y;
    if (dy < -7 || dy > 7) continue;
    for (int x = -iradius; x <= iradius; x++) {
      const int dx = icx + x;
      if (dx >= -7 && dx <= 7 && (square || y * y + x * x <= ir2)) {
        const float d = cs[112 + dy * 15 + dx];
        if (d > 0.0f) {
          s0 += d;
          sx += d * dx;
          sy += d * dy;
        }
      }
    }
  }
  const float xm = sx / s0, ym = sy / s0;
  const int ixm = isnan(xm) ? 0 : (int)floorf(xm + 0.5f), iym = isnan(ym) ? 0 : (int)floorf(ym + 0.5f);
  const float sv = cs[112 + iym * 15 + ixm];
  out[0] = (k == 1) ? -xm : xcenter - xm;
  out[1] = (k == 0) ? -ym : ((k == 3) ? -xcenter - ym : xcenter - ym);
  out[2] = sv;
}

// bits a..b (inclusive) of a row mask, none when b < a
__device__ __forceinline__ unsigned bit_range(int a, int b) {
  return (b < a) ? 0u : (((2u << b) - 1u) & ~((1u << a) - 1u));
}

constexpr int LMA_NEQ = 28;  // packed normal equations: A (upper 6x6, 21), b (6), weighted rms^2
// floats from the sample arrays to the end of the reduction buffer, free before the samples exist

// Weighted normal equations of the samples at parameters av (getFxJt, getWJtJlambda, getWYmFxRms),
// written to out[LMA_NEQ] for every lane: per-lane partial sums are transposed through red
// [LMA_NEQ][33] and lane k sums row k in a fixed order.
__device__ __forceinline__ void lma_eval(const float *sx, const float *sy, const float *sv, const float *sw,
                                         const unsigned char *sg, int gdiag_bits, int ns, const float av[LMA_NP],
                                         float w_wm, float w_wxy, float half_width, float *red, float *out,
                                         int lane) {
  float A[21], b[LMA_NP], r2 = 0.f;
#pragma unroll
  for (int k = 0; k < 21; k++) A[k] = 0.f;
#pragma unroll
  for (int k = 0; k < LMA_NP; k++) b[k] = 0.f;
  const float Wy = av[1] + av[2], Wx = Wy + av[3];
  const float iWx = 1.0f / Wx, iWy = 1.0f / Wy;
  for (int n = lane; n < ns; n += 32) {
    const int g = sg[n];
    const float ws = ((gdiag_bits >> g) & 1) ? 1.41421356237f : 1.0f;
    const float Ag = g ? av[5] : av[4];
    const float dxw = ws * (sx[n] - av[0]) * iWx, dyw = ws * sy[n] * iWy;
    const float d = 1.0f - dxw * dxw - dyw * dyw;
    const float e = sv[n] - d * Ag, w = sw[n], wr = w * e;
    const float dfdWx = 2.0f * Ag * dxw * dxw * iWx, dfdWy = 2.0f * Ag * dyw * dyw * iWy;
    const float j[LMA_NP] = {2.0f * ws * Ag * dxw * iWx, dfdWx + dfdWy, dfdWx + dfdWy, dfdWx,
                             (g == 0) ? d : 0.0f, (g == 1) ? d : 0.0f};
    r2 = fmaf(wr, e, r2);
    int k = 0;
#pragma unroll
    for (int a = 0; a < LMA_NP; a++) {
      b[a] = fmaf(j[a], wr, b[a]);
      const float wj = w * j[a];
#pragma unroll
      for (int c = a; c < LMA_NP; c++) {
        A[k] = fmaf(wj, j[c], A[k]);
        k++;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 21; k++) red[k * 33 + lane] = A[k];
#pragma unroll
  for (int k = 0; k < LMA_NP; k++) red[(21 + k) * 33 + lane] = b[k];
  red[27 * 33 + lane] = r2;
  __syncwarp();
  if (lane < LMA_NEQ) {
    float t = 0.f;
    for (int i = 0; i < 32; i++) t += red[lane * 33 + i];
    // the two regularisation samples: WM towards half_width, WXY towards 0
    const float e1 = half_width - av[1], e2 = -av[3];
    if (lane == 6) t += w_wm;                 // A (1, 1)
    if (lane == 15) t += w_wxy;               // A (3, 3)
    if (lane == 22) t += w_wm * e1;           // b 1
    if (lane == 24) t += w_wxy * e2;          // b 3
    if (lane == 27) t += w_wm * e1 * e1 + w_wxy * e2 * e2;
    out[lane] = t;
  }
  __syncwarp();
}

}  // namespace

// One Correlation2d.corrLMA fit of a tile from the staged pair surfaces `src` ([P][225]) of the
// pair kinds in kmask (bit k: kind k), centred at xcenter: res = {disparity, strength, WM, WXY}
// (getDisparityStrengthWidth); false when there are no samples or the fit did not converge.
// Samples of the selected pairs (BY_PAIR: bit = pair index, else bit = pair kind; pairs of kind -1
// never): the group surfaces (combineCompatiblePairs), filterConvex around the integer centre and
// addSamples with weights x |value|^vasw_pwr, compacted into sx/sy/sv/sw/sg in the reference's
// order.  Returns the sample count; ngroups / gdiag_bits (bit g: group g is the diagonal one)
// describe the groups.
template <bool BY_PAIR>
__device__ __forceinline__ int lma_samples(const LmaDev &ld, const TpLmaConst &c, unsigned sel_mask, float xcenter,
                                           float vasw_pwr, const float *src, float *gsurf, float *sx, float *sy,
                                           float *sv, float *sw, unsigned char *sg, int lane, int &ngroups_out,
                                           int &gdiag_bits_out) {
  const int hw = c.cnvx_hwnd_size;
  const int ixc = (int)floorf(xcenter + 0.5f);
  // ---- group surfaces (combineCompatiblePairs) ----
  int np_ortho = 0, np_diag = 0;
  for (int pi = 0; pi < ld.P; pi++) {
    const int k = ld.kinds[pi];
    if (k < 0 || !((sel_mask >> (BY_PAIR ? pi : k)) & 1)) continue;
    np_ortho += (k <= 1);
    np_diag += (k >= 2);
  }
  // group sums, pairs in index order (combineCompatiblePairs), 8 cells per lane in registers
  float go[8], gdg[8];
#pragma unroll
  for (int t = 0; t < 8; t++) go[t] = gdg[t] = 0.f;
  for (int pi = 0; pi < ld.P; pi++) {
    const int k = ld.kinds[pi];
    if (k < 0 || !((sel_mask >> (BY_PAIR ? pi : k)) & 1)) continue;
    const float *cs = src + pi * TP_CORR;
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const int i = lane + 32 * t;
      if (i < 225) {
        const int r = i / 15, q = i - r * 15;
        const float v = (k == 1) ? cs[q * 15 + r] : ((k == 3) ? cs[(14 - r) * 15 + q] : cs[i]);
        if (k >= 2) gdg[t] += v;
        else go[t] += v;
      }
    }
  }
#pragma unroll
  for (int t = 0; t < 8; t++) {
    const int i = lane + 32 * t;
    if (i < 225) {
      gsurf[i] = (np_ortho > 1) ? go[t] / np_ortho : go[t];
      gsurf[225 + i] = (np_diag > 1) ? gdg[t] / np_diag : gdg[t];
    }
  }
  __syncwarp();
  // ---- filterConvex, both groups at once: lanes 0-14 hold the ortho rows, lanes 16-30 the
  // diagonal rows, as 15-bit masks (bit = column) of the convex and the selected cells ----
  const int half = lane >> 4, r = lane & 15, hbase = half << 4;
  const bool rowlane = r < 15 && (half ? np_diag : np_ortho) > 0;
  const int x0 = ixc + 7, y0 = (half ? ixc : 0) + 7;
  const int min_row = max(y0 - hw, 0), max_row = min(y0 + hw, 14);
  const int min_col = max(x0 - hw, 0), max_col = min(x0 + hw, 14);
  unsigned conv = 0, sel = 0;
  if (rowlane) {
    const float *d = gsurf + 225 * half;
    if (r > min_row && r < max_row)
      for (int col = min_col + 1; col < max_col; col++) {
        const int i = r * 15 + col;
        if ((2 * d[i] > (d[i - 1] + d[i + 1])) && (2 * d[i] > (d[i - 15] + d[i + 15]))) conv |= 1u << col;
      }
    if (r == y0 && x0 >= min_col && x0 <= max_col) sel = 1u << x0;
  }
  {
    const unsigned lmask = bit_range(min_col + 1, x0), rmask = bit_range(x0, max_col - 1);
    const unsigned hmask = 0xffffu << hbase;
    bool active = rowlane;
    for (int istep = 0; istep < hw; istep++) {
      const bool first = istep == 0;
      const int smin_row = max(y0 - istep, 0), smax_row = min(y0 + istep, 14);
      const unsigned cols = bit_range(max(x0 - istep, 0), min(x0 + istep, 14));
      unsigned seln = sel;
      // up / down: the source row's selected cells (convex, or the start) grow into the next row
      const unsigned src = sel & cols & (first ? 0x7fffu : conv);
      const bool up_ok = istep < y0, down_ok = (y0 + istep) < max_row;
      const unsigned s_up = __shfl_sync(0xffffffffu, src, hbase + max(y0 - istep, 0));
      const unsigned s_dn = __shfl_sync(0xffffffffu, src, hbase + min(y0 + istep, 14));
      if (up_ok && r == y0 - istep - 1) {
        const unsigned c1 = s_up & conv;
        seln |= s_up | ((c1 & lmask) >> 1) | ((c1 & rmask) << 1);
      }
      if (down_ok && r == y0 + istep + 1) {
        const unsigned c1 = s_dn & conv;
        seln |= s_dn | ((c1 & lmask) >> 1) | ((c1 & rmask) << 1);
      }
      // left / right: the source column's cells grow sideways, and from a convex target up or
      // down towards the centre row's side
      unsigned push_up = 0, push_dn = 0;
      const bool in_rows = r >= smin_row && r <= smax_row;
#pragma unroll
      for (int side = 0; side < 2; side++) {
        const int col = side ? x0 + istep : x0 - istep;
        const bool ok = side ? ((x0 + istep) < max_col) : (istep < x0);
        if (!ok || !in_rows || col < 0 || col > 14) continue;
        const unsigned cb = 1u << col, tb = side ? (cb << 1) : (cb >> 1);
        if ((sel & cb) && (first || (conv & cb))) {
          seln |= tb;
          if (conv & tb) {
            if (r <= y0 && r > min_row) push_up |= tb;
            if (r >= y0 && r < max_row) push_dn |= tb;
          }
        }
      }
      seln |= __shfl_down_sync(0xffffffffu, push_up, 1) | __shfl_up_sync(0xffffffffu, push_dn, 1);
      if (!rowlane) seln = 0;
      const unsigned changed = __ballot_sync(0xffffffffu, active && seln != sel) & hmask;
      if (!changed) active = false;
      if (active) sel = seln;
      if (!__any_sync(0xffffffffu, active)) break;
    }
  }
  // ---- samples (addSamples), compacted in the enumeration order ----
  int ns = 0, ngroups = 0, gdiag_bits = 0;
  for (int gd = 0; gd < 2; gd++) {
    const int npg = gd ? np_diag : np_ortho;
    if (npg == 0) continue;
    const int base = gd ? LMA_ORTHO_ENTRIES : 0, cnt = gd ? LMA_DIAG_ENTRIES : LMA_ORTHO_ENTRIES;
    const float *d = gsurf + 225 * gd;
    int gnum = -1;  // groups are numbered in the order their first sample arrives
    for (int e0 = 0; e0 < cnt; e0 += 32) {
      const int e = e0 + lane;
      float w = 0.f, v = 0.f, x = 0.f, y = 0.f;
      int cxo = 99, cyo = 99;
      if (e < cnt) {
        cxo = __ldg(&g_lma_cx[base + e]);
        cyo = __ldg(&g_lma_cy[base + e]);
      }
      const int cx = cxo + ixc, cy = cyo + (gd ? ixc : 0);
      const bool inside = e < cnt && cx >= -7 && cx <= 7 && cy >= -7 && cy <= 7;
      const int srow = inside ? cy + 7 : 0;
      const unsigned rsel = __shfl_sync(0xffffffffu, sel, (gd << 4) + srow);
      const unsigned rconv = __shfl_sync(0xffffffffu, conv, (gd << 4) + srow);
      if (inside) {
        {
          const int idx = 112 + 15 * cy + cx, ccol = cx + 7, gy0 = (gd ? ixc : 0) + 7;
          float wc = 0.f;
          if ((rsel >> ccol) & 1) wc = ((rconv >> ccol) & 1) ? 1.0f : c.cnvx_weight;
          else if (c.cnvx_add3x3 && srow >= gy0 - 1 && srow <= gy0 + 1 && ccol >= ixc + 6 && ccol <= ixc + 8)
            wc = c.cnvx_weight;
          w = wc * npg;
          if (w > 0.f) {
            v = d[idx];
            if (vasw_pwr == 2.0f) w *= v * v;
            else if (vasw_pwr != 0.0f) w *= powf(fabsf(v), vasw_pwr);
            x = (gd ? 0.5f * (cxo + cyo) : (float)cxo) + (float)ixc;
            y = gd ? 0.5f * (cyo - cxo) : (float)cyo;
          }
        }
      }
      const unsigned take = __ballot_sync(0xffffffffu, w > 0.f);
      if (take && gnum < 0) {
        gnum = ngroups++;
        gdiag_bits |= gd << gnum;
      }
      if (w > 0.f) {
        const int o = ns + __popc(take & ((1u << lane) - 1u));
        if (o < LMA_MAX_SAMPLES) {
          sx[o] = x; sy[o] = y; sv[o] = v; sw[o] = w;
          sg[o] = (unsigned char)gnum;
        }
      }
      ns = min(ns + __popc(take), LMA_MAX_SAMPLES);
    }
  }
  __syncwarp();
  ngroups_out = ngroups;
  gdiag_bits_out = gdiag_bits;
  return ns;
}

// Correlation2d.corrLMA (1754-1877) on the pairs of the kinds in kmask: samples, then the
// Levenberg-Marquardt fit; res = {disparity, strength, WM, WXY}
__device__ __forceinline__ bool lma_fit(const LmaDev &ld, const TpLmaConst &c, int kmask, float xcenter,
                                        const float *src, float *gsurf, float *sx, float *sy, float *sv, float *sw,
                                        unsigned char *sg, float *red, float *acc, float *trial, int lane,
                                        float res[4]) {
  int ngroups, gdiag_bits;
  const int ns = lma_samples<false>(ld, c, (unsigned)kmask, xcenter, c.ortho_vasw_pwr, src, gsurf, sx, sy, sv, sw, sg,
                                    lane, ngroups, gdiag_bits);
  if (ns == 0) return false;
  // ---- initVector / setWeightsValues ----
  float wsum = 0.f, gw0 = 0.f, gw1 = 0.f, vmax = -CUDART_INF_F, smax = 0.f;
  int imx = 1 << 30;
  for (int n = lane; n < ns; n += 32) {
    float w = sw[n], v = sv[n];
    if (sg[n] == 0) gw0 += w; else gw1 += w;
    if (v > smax) smax = v;
    if (isnan(v) || isnan(w)) { w = 0.f; v = 0.f; sw[n] = 0.f; sv[n] = 0.f; }
    wsum += w;
    if (v > vmax) { vmax = v; imx = n; }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {  // first maximum of the sample values
    const float ov = __shfl_xor_sync(0xffffffffu, vmax, o);
    const int oi = __shfl_xor_sync(0xffffffffu, imx, o);
    if (ov > vmax || (ov == vmax && oi < imx)) { vmax = ov; imx = oi; }
  }
  wsum = warp_sum(wsum);
  gw0 = warp_sum(gw0);
  gw1 = warp_sum(gw1);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) smax = fmaxf(smax, __shfl_xor_sync(0xffffffffu, smax, o));
  const float pure = wsum;
  const float tot = wsum + c.cost_wy + c.cost_wxy;
  const float inv = (tot != 0.f) ? 1.0f / tot : 1.0f;
  for (int n = lane; n < ns; n += 32) sw[n] *= inv;
  __syncwarp();
  const float w_wm = c.cost_wy * inv, w_wxy = c.cost_wxy * inv;
  const float gwt[2] = {pure > 0.f ? gw0 / pure : gw0, pure > 0.f ? gw1 / pure : gw1};
  const bool mask[LMA_NP] = {true, c.adjust_wm != 0, c.adjust_wy != 0, c.adjust_wxy != 0,
                             c.adjust_ag != 0 && ngroups > 0, c.adjust_ag != 0 && ngroups > 1};
  float av[LMA_NP] = {xcenter, c.half_width, 0.f, 0.f, vmax, vmax};
  if (ngroups < 2) av[5] = 0.f;
  // ---- runLma / lmaStep ----
  // acc: normal equations at the accepted parameters; trial: at the proposed ones
  // iteration -1 evaluates the start (into acc); one inlined evaluation serves all
  float last = 0.f, initial = 0.f;
  float lambda = c.lambda_initial;
  bool success = false;
  for (int iter = -1; iter < c.num_iter; iter++) {
    float nav[LMA_NP];
    if (iter < 0) {
#pragma unroll
      for (int a = 0; a < LMA_NP; a++) nav[a] = av[a];
    } else {
      // (JtJ + lambda diag JtJ) delta = Jt W (y - f), masked parameters held (identity rows).
      // The matrix is symmetric positive (semi)definite: LDL^T without pivoting; a pivot that is
      // not positive marks it singular, as the zero pivot of the reference's LU inverse does.
      float M[LMA_NP][LMA_NP], rhs[LMA_NP];
      {
        int k = 0;
#pragma unroll
        for (int a = 0; a < LMA_NP; a++)
#pragma unroll
          for (int cc = a; cc < LMA_NP; cc++) {
            const bool keep = mask[a] && mask[cc];
            const float v = keep ? acc[k] : ((a == cc) ? 1.0f : 0.0f);
            M[a][cc] = v;
            M[cc][a] = v;
            k++;
          }
      }
#pragma unroll
      for (int a = 0; a < LMA_NP; a++) {
        if (mask[a]) M[a][a] += M[a][a] * lambda;
        rhs[a] = mask[a] ? acc[21 + a] : 0.0f;
      }
      float Lm[LMA_NP][LMA_NP], Dd[LMA_NP], Dinv[LMA_NP];
      bool singular = false;
#pragma unroll
      for (int r = 0; r < LMA_NP; r++) {
#pragma unroll
        for (int cc = 0; cc < r; cc++) {
          float t = M[r][cc];
#pragma unroll
          for (int k = 0; k < cc; k++) t -= Lm[r][k] * Lm[cc][k] * Dd[k];
          Lm[r][cc] = t * Dinv[cc];
        }
        float dd = M[r][r];
#pragma unroll
        for (int k = 0; k < r; k++) dd -= Lm[r][k] * Lm[r][k] * Dd[k];
        if (!(dd > 0.0f)) singular = true;
        Dd[r] = dd;
        Dinv[r] = (dd > 0.0f) ? 1.0f / dd : 0.0f;
      }
      if (singular) break;
      float delta[LMA_NP];
#pragma unroll
      for (int r = 0; r < LMA_NP; r++) {
        float t = rhs[r];
#pragma unroll
        for (int k = 0; k < r; k++) t -= Lm[r][k] * delta[k];
        delta[r] = t;
      }
#pragma unroll
      for (int r = LMA_NP - 1; r >= 0; r--) {
        float t = delta[r] * Dinv[r];
#pragma unroll
        for (int k = r + 1; k < LMA_NP; k++) t -= Lm[k][r] * delta[k];
        delta[r] = t;
      }
#pragma unroll
      for (int a = 0; a < LMA_NP; a++) nav[a] = av[a] + (mask[a] ? delta[a] : 0.0f);
    }
    lma_eval(sx, sy, sv, sw, sg, gdiag_bits, ns, nav, w_wm, w_wxy, c.half_width, red, iter < 0 ? acc : trial, lane);
    if (iter < 0) {
      last = initial = sqrtf(acc[27]);
      continue;
    }
    const float rms = sqrtf(trial[27]);
    bool done = false;
    if (rms < last) {
      success = true;
      done = rms >= last * (1.0f - c.rms_diff);
      last = rms;
#pragma unroll
      for (int a = 0; a < LMA_NP; a++) av[a] = nav[a];
      if (lane < LMA_NEQ) acc[lane] = trial[lane];
      __syncwarp();
    } else {
      success = false;
    }
    if (done) break;
    if (success) lambda *= c.lambda_scale_good;
    else {
      lambda *= c.lambda_scale_bad;
      if (lambda > c.lambda_max) break;
    }
  }
  if (!success && last < initial) success = true;
  if (!success) return false;
  // ---- getDisparityStrength(Width) ----
  float sum_amp = gwt[0] * av[4] + (ngroups > 1 ? gwt[1] * av[5] : 0.0f);
  if (sum_amp > 1.25f * smax) sum_amp = smax;
  res[0] = -av[0];
  res[1] = sum_amp;
  res[2] = av[1];
  res[3] = av[3];
  return true;
}

// Gaussian elimination with partial pivoting (the LU factorisation Jama's Matrix.det / solve use)
// of a [n][n+1] (matrix | right-hand side, row stride n + 1) in place, by one thread: returns the
// determinant and leaves the solution in column n.  Multipliers and back substitution use the
// pivot's reciprocal (FP64 division is a long sequence on this part; the results differ from
// dividing in the last bits only).
__device__ double gauss_det_solve(double *a, int n) {
  const int st = n + 1;
  double det = 1.0;
  for (int k = 0; k < n; k++) {
    int p = k;
    for (int i = k + 1; i < n; i++)
      if (fabs(a[i * st + k]) > fabs(a[p * st + k])) p = i;
    if (p != k) {
      for (int j = k; j < st; j++) {
        const double t = a[p * st + j];
        a[p * st + j] = a[k * st + j];
        a[k * st + j] = t;
      }
      det = -det;
    }
    const double piv = a[k * st + k];
    det *= piv;
    const double rp = 1.0 / piv;
    a[k * st + k] = rp;  // the reciprocal, for the back substitution
    if (piv != 0.0)
      for (int i = k + 1; i < n; i++) {
        const double m = a[i * st + k] * rp;
        for (int j = k + 1; j < st; j++) a[i * st + j] = fma(-m, a[k * st + j], a[i * st + j]);
      }
  }
  for (int k = n - 1; k >= 0; k--) {
    double x = a[k * st + n];
    for (int j = k + 1; j < n; j++) x = fma(-a[k * st + j], a[j * st + n], x);
    a[k * st + n] = x * a[k * st + k];
  }
  return det;
}

// squared product of the row norms of a [n][n] with row stride st (PolynomialApproximation.normMatix
// squared: the determinant tests |det| / norm < t are taken as det^2 < t^2 norm^2)
__device__ double row_norm_product_sq(const double *a, int n, int st) {
  double norm = 1.0;
  for (int i = 0; i < n; i++) {
    double d = 0.0;
    for (int j = 0; j < n; j++) d = fma(a[i * st + j], a[i * st + j], d);
    norm *= d;
  }
  return norm;
}

// |det| / sqrt(nsq) >= t, with nsq == 0 failing (quadraticApproximation's well-posedness test)
__device__ __forceinline__ bool det_ok(double det, double nsq, double t) {
  return nsq != 0.0 && det * det >= t * t * nsq;
}

// one level of a reduce-scatter: lanes with bit o keep the upper half of v (after their partner's
// values are added), the others the lower half
template <int HALF>
__device__ __forceinline__ void scatter_level(double *v, int lane, int o) {
  const bool hi = (lane & o) != 0;
#pragma unroll
  for (int k = 0; k < HALF; k++) {
    const double give = hi ? v[k] : v[k + HALF], keep = hi ? v[k + HALF] : v[k];
    v[k] = keep + __shfl_xor_sync(0xffffffffu, give, o);
  }
}

// Weighted moments of the samples for the quadric fit of quadraticApproximation (350-585): S00 S10
// S01 S20 S11 S02 S30 S21 S12 S03 S40 S31 S22 S13 S04 of the weights, then Z00 Z10 Z01 Z20 Z11
// Z02 of weight x value; samples with weight <= 0 are skipped.  Per-lane sums in FP64, then a
// reduce-scatter across the warp (21 values padded to 22 -> 11 -> 12 -> 6 -> 3 -> 4 -> 2 -> 1,
// 23 additions per lane instead of 105 for a full butterfly): lane 11 b4 + 6 b3 + 3 b2 + 2 b1 + b0
// (bits of the lane index) ends with that moment, except the lanes that hold a pad; each writes
// its moment to dst[21].
__device__ __forceinline__ void quadric_moments(const float *sx, const float *sy, const float *sv, const float *sw,
                                                int ns, int lane, double *dst) {
  double m[22];
#pragma unroll
  for (int i = 0; i < 22; i++) m[i] = 0.0;
  for (int n = lane; n < ns; n += 32) {
    const double w = sw[n];
    if (!(w > 0.0)) continue;
    const double x = sx[n], y = sy[n], x2 = x * x, y2 = y * y, wz = w * (double)sv[n];
    const double x3 = x2 * x, y3 = y2 * y;
    m[0] += w; m[1] += w * x; m[2] += w * y; m[3] += w * x2; m[4] += w * x * y; m[5] += w * y2;
    m[6] += w * x3; m[7] += w * x2 * y; m[8] += w * x * y2; m[9] += w * y3;
    m[10] += w * x3 * x; m[11] += w * x3 * y; m[12] += w * x2 * y2; m[13] += w * x * y3; m[14] += w * y3 * y;
    m[15] += wz; m[16] += wz * x; m[17] += wz * y; m[18] += wz * x2; m[19] += wz * x * y; m[20] += wz * y2;
  }
  m[21] = 0.0;
  scatter_level<11>(m, lane, 16);
  m[11] = 0.0;
  scatter_level<6>(m, lane, 8);
  scatter_level<3>(m, lane, 4);
  m[3] = 0.0;
  scatter_level<2>(m, lane, 2);
  scatter_level<1>(m, lane, 1);
  const int b0 = lane & 1, b1 = (lane >> 1) & 1, b2 = (lane >> 2) & 1, b3 = (lane >> 3) & 1, b4 = (lane >> 4) & 1;
  const int l4 = 2 * b1 + b0, l2 = 6 * b3 + 3 * b2 + l4, idx = 11 * b4 + l2;
  if (l4 != 3 && l2 != 11 && idx != 21) dst[idx] = m[0];
}

// Correlations2dLMA.getMaxXYPoly (641-704) from the moments, by one thread in FP64: the quadric
// A x^2 + B y^2 + C xy + D x + E y + F (quadraticApproximation, with the linear / quadratic
// determinant-to-norm thresholds 1e-20 / 1e-30 of quadraticMaxV2dX2Y2XY 201-221) and its
// maximum.  dm: >= 48 doubles of scratch.  Returns false when a test fails or the stationary
// point is not a maximum with a non-negative value.
__device__ bool quadric_max(const double *m, int ns, double *dm, double xyv[3]) {
  if (ns <= 0) return false;
  const double S00 = m[0], S10 = m[1], S01 = m[2], S20 = m[3], S11 = m[4], S02 = m[5], S30 = m[6], S21 = m[7],
               S12 = m[8], S03 = m[9], S40 = m[10], S31 = m[11], S22 = m[12], S13 = m[13], S04 = m[14];
  const double lin[12] = {S20, S11, S10, 0.0, S11, S02, S01, 0.0, S10, S01, S00, 0.0};
  for (int i = 0; i < 12; i++) dm[i] = lin[i];
  double nsq = row_norm_product_sq(dm, 3, 4);
  if (!det_ok(gauss_det_solve(dm, 3), nsq, 1.0e-20)) return false;  // linear fit only: no maximum
  const double q[42] = {S40, S22, S31, S30, S21, S20, m[18], S22, S04, S13, S12, S03, S02, m[20],
                        S31, S13, S22, S21, S12, S11, m[19], S30, S12, S21, S20, S11, S10, m[16],
                        S21, S03, S12, S11, S02, S01, m[17], S20, S02, S11, S10, S01, S00, m[15]};
  for (int i = 0; i < 42; i++) dm[i] = q[i];
  nsq = row_norm_product_sq(dm, 6, 7);
  if (!det_ok(gauss_det_solve(dm, 6), nsq, 1.0e-30)) return false;  // linear fit only
  const double A = dm[6], B = dm[13], Cq = dm[20], D = dm[27], E = dm[34], F = dm[41];
  double *t = dm + 42;
  t[0] = 2.0 * A; t[1] = Cq; t[2] = -D; t[3] = Cq; t[4] = 2.0 * B; t[5] = -E;
  nsq = row_norm_product_sq(t, 2, 3);
  if (!det_ok(gauss_det_solve(t, 2), nsq, 1.0e-30)) return false;
  const double x = t[2], y = t[5];
  const double v = A * x * x + B * y * y + Cq * x * y + D * x + E * y + F;
  if (v < 0.0 || A >= 0.0 || B >= 0.0) return false;  // negative strength, or not a maximum
  xyv[0] = x;
  xyv[1] = y;
  xyv[2] = v;
  return true;
}

// LY_POLY: the instantiation with the polynomial mismatch measure (the other never carries it)
template <bool LY_POLY>
__global__ void __launch_bounds__(32 * LMA_NW) lma_kernel(const __grid_constant__ LmaDev ld,
                                                         const __grid_constant__ TpLmaConst c) {
  extern __shared__ float sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *gsurf = sm + warp * LMA_PER_WARP;                      // [2][225]
  float *sx = gsurf + 450;                                      // samples
  float *sy = sx + LMA_MAX_SAMPLES, *sv = sy + LMA_MAX_SAMPLES, *sw = sv + LMA_MAX_SAMPLES;
  unsigned char *sg = (unsigned char *)(sw + LMA_MAX_SAMPLES);
  float *red = gsurf + LMA_OFF_RED;                             // [LMA_NEQ][33] transposed partial sums
  float *acc = red + LMA_NEQ * 33, *trial = acc + 32;
  float *stage = gsurf + LMA_OFF_STAGE;                         // [P][225] the tile's pair surfaces
  float *dres = gsurf + LMA_OFF_RES;                            // [4][4] the orientation fits
  // quadric moments [LMA_POLY_CHUNK][21] over the reduction buffer and the per-lane solver scratch
  // [LMA_POLY_CHUNK][LMA_POLY_SCRATCH] over the group surfaces (both free once the fits are done)
  double *dmom = (double *)(gsurf + ((LMA_OFF_RED + 1) & ~1));
  double *dsolve = (double *)gsurf;
  for (int task = blockIdx.x * LMA_NW + warp; task < ld.num_tasks; task += gridDim.x * LMA_NW) {
    const int txy = ld.task_txy[task];
    const size_t tile = (size_t)(txy >> 16) * ld.tilesX + (txy & 0xffff);
    float *rec = ld.lma + tile * 4;
    float *dm = ld.disp + tile * TP_NDISP;
    const float cm = dm[1], strength0 = dm[2];  // the record's CM disparity and strength
    if (lane < 4) rec[lane] = CUDART_NAN_F;
    if (ld.mismatch)  // {NaN, NaN, 0} unless measured below
      for (int i = lane; i < 3 * ld.P; i += 32) ld.mismatch[tile * 3 * ld.P + i] = (i % 3 == 2) ? 0.f : CUDART_NAN_F;
    if (isnan(cm) || !(strength0 > c.min_poly_strength)) continue;
    // The tile's surfaces are contiguous (P x 900 bytes): copied asynchronously, all in flight at
    // once, in 8-byte pieces when P is even (the tile's offset is then a multiple of 8 bytes).
    const float *src = ld.corr + tile * ld.P * TP_CORR;
    if (ld.P <= LMA_STAGE_PAIRS) {
      if ((ld.P & 1) == 0) {
        for (int k = lane; k < ld.P * TP_CORR / 2; k += 32) cp_async8(stage + 2 * k, src + 2 * k);
      } else {
        for (int k = lane; k < ld.P * TP_CORR; k += 32) cp_async4(stage + k, src + k);
      }
      asm volatile("cp.async.commit_group;\n" ::: "memory");
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      __syncwarp();
      src = stage;
    }
    // fit 0: all pairs (corrLMA); fits 1-4 with fo_correct: one pair orientation each
    // (corr4dirsLMA), centred at the (mixed) disparity.  One inlined copy of the fit serves all.
    float main_res[4] = {0.f, 0.f, 0.f, 0.f};
    float disparity = cm, strength = strength0, cm_out = cm, str_out = strength0;
    unsigned valid = 0;
    bool main_ok = false;
    const bool mism = ld.mismatch != nullptr;
    for (int f = 0; f < 5; f++) {
      if (f > 0 && !((c.fo_correct && strength > 0.0f) || mism)) break;
      if (f > 0 && ld.kind_count[f - 1] == 0) continue;
      float res[4];
      const bool ok = lma_fit(ld, c, f ? 1 << (f - 1) : 0xf, f ? -disparity : -cm, src, gsurf, sx, sy, sv, sw, sg,
                              red, acc, trial, lane, res);
      if (f == 0) {
        if (!ok) break;
        main_ok = true;
#pragma unroll
        for (int k = 0; k < 4; k++) main_res[k] = res[k];
        if (c.mix_corr_poly) {
          disparity = cm_out = res[0];
          strength = str_out = res[1];
        }
      } else if (ok) {
        valid |= 1u << (f - 1);
        if (lane < 4) dres[(f - 1) * 4 + lane] = (lane == 0) ? res[0] : ((lane == 1) ? res[1] : ((lane == 2) ? res[2] : res[3]));
      }
    }
    if (!main_ok) continue;
    __syncwarp();
    if ((c.fo_correct && strength > 0.0f) || mism) {  // foregroundCorrect (ImageDtt.java:2294-2418)
      float dd[4][4];
      bool vb[4];
#pragma unroll
      for (int d = 0; d < 4; d++) {
        vb[d] = (valid >> d) & 1;
#pragma unroll
        for (int k = 0; k < 4; k++) dd[d][k] = dres[d * 4 + k];
      }
      float spread;
      const float mod = foreground_correct(c, dd, vb, disparity, spread);
      // the corrected distance is not used while the mismatch is measured
      if (!mism && c.fo_correct && mod != disparity && strength > c.fo_min_strength) cm_out = mod;
      if (mism && spread <= c.mismatch_max_diff) {
        bool need_cm = true;
        if (LY_POLY) {
          // ImageDtt.java:2349-2383: each pair alone (mismatchPairs 1434-1503), the quadric's
          // maximum; an implausible offset zeroes the pair's strength, and with the backup any
          // failed or implausible pair sends the tile to the centre-of-mass measure
          // Pairs go in chunks: the warp samples each pair and reduces its moments, then lane j
          // solves the chunk's j-th pair (the solves are serial FP64 work, so one per lane).
          bool has_nan = false;
          const double xc = -(double)disparity;
          for (int c0 = 0; c0 < ld.P; c0 += LMA_POLY_CHUNK) {
            const int c1 = min(c0 + LMA_POLY_CHUNK, ld.P);
            int my_ns = 0;
            for (int pi = c0; pi < c1; pi++) {
              if (ld.kinds[pi] < 0) continue;
              int ng, gdb;
              const int ns = lma_samples<true>(ld, c, 1u << pi, -disparity, c.max_corr_radius, src, gsurf, sx, sy, sv,
                                               sw, sg, lane, ng, gdb);
              quadric_moments(sx, sy, sv, sw, ns, lane, dmom + (pi - c0) * 21);
              if (lane == pi - c0) my_ns = ns;
              __syncwarp();  // the next pair's samples overwrite these; the moments are written
            }
            const int pi = c0 + lane;
            bool bad = false;
            if (pi < c1 && ld.kinds[pi] >= 0) {
              const int k = ld.kinds[pi];
              double q[3], o0 = CUDART_NAN, o1 = CUDART_NAN, o2 = 0.0;
              if (quadric_max(dmom + lane * 21, my_ns, dsolve + lane * LMA_POLY_SCRATCH, q)) {
                if (k == 0) { o0 = xc - q[0]; o1 = -q[1]; }
                else if (k == 1) { o0 = -q[1]; o1 = xc - q[0]; }
                else if (k == 2) { o0 = xc - q[0] + q[1]; o1 = xc - q[0] - q[1]; }
                else { o0 = xc - q[0] + q[1]; o1 = -xc + q[0] + q[1]; }
                o2 = isnan(q[2]) ? 0.0 : q[2];
              }
              if (isnan(o0) || isnan(o1)) bad = true;
              else if (o2 != 0.0 && (fabs(o0) > c.ly_crazy_poly || fabs(o1) > c.ly_crazy_poly)) {
                o2 = 0.0;
                bad = true;
              }
              float *mo = ld.mismatch + (tile * ld.P + pi) * 3;
              mo[0] = (float)o0;
              mo[1] = (float)o1;
              mo[2] = (float)o2;
            }
            has_nan |= __any_sync(0xffffffffu, bad);
            __syncwarp();  // the scratch lies over the next chunk's group surfaces
          }
          need_cm = c.ly_poly_backup && has_nan;
          __syncwarp();
        }
        if (need_cm && lane < ld.P && ld.kinds[lane] >= 0) {
          float m3[3];
          mismatch_cm(src + lane * TP_CORR, ld.kinds[lane], -disparity, c.max_corr_radius, m3);
          float *mo = ld.mismatch + (tile * ld.P + lane) * 3;
          mo[0] = m3[0];
          mo[1] = m3[1];
          mo[2] = m3[2];
        }
      }
    }
    if (lane == 0) {
      rec[0] = main_res[0];
      rec[1] = main_res[1];
      rec[2] = main_res[2];
      rec[3] = main_res[3];
      dm[1] = cm_out;
      dm[2] = str_out;
    }
  }
}

cudaError_t upload_lma_constants() {
  // addSamples enumeration (Correlation2d.java:2314-2382): quadrant signs {-1,-1},{1,-1},{-1,1},{1,1}
  signed char cx[LMA_ORTHO_ENTRIES + LMA_DIAG_ENTRIES], cy[LMA_ORTHO_ENTRIES + LMA_DIAG_ENTRIES];
  static const int qs[4][2] = {{-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
  int n = 0;
  for (int diag = 0; diag < 2; diag++) {
    const int start = n;
    for (int arow = 0; arow < 9; arow += diag ? 1 : 2)
      for (int acol = diag ? (arow & 1) : 0; acol < 9; acol += 2)
        for (int q = 0; q < 4; q++) {
          if (!(((arow > 0) || (q & 2)) && ((acol > 0) || (q & 1)))) continue;
          if (diag) {
            cx[n] = (signed char)((qs[q][0] * acol - qs[q][1] * arow) / 2);
            cy[n] = (signed char)((qs[q][0] * acol + qs[q][1] * arow) / 2);
          } else {
            cx[n] = (signed char)((qs[q][0] * acol) / 2);
            cy[n] = (signed char)((qs[q][1] * arow) / 2);
          }
          n++;
        }
    if (n - start != (diag ? LMA_DIAG_ENTRIES : LMA_ORTHO_ENTRIES)) return cudaErrorInvalidValue;
  }
  cudaError_t e = cudaMemcpyToSymbol(g_lma_cx, cx, sizeof(cx));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_lma_cy, cy, sizeof(cy));
  return e;
}

int lma_smem_bytes() { return LMA_NW * LMA_PER_WARP * 4; }

// ---------------------------------------------------------------------------
// The LMA branch of ImageDtt.tileInterCamCorrs (ImageDtt.java:7497-7560) for a rig: the LMA pass
// above runs on the inter-camera surfaces ([tiles][1][225], one horizontal pair) from a record
// whose CM / strength are the rig's centre-of-mass values; then, where it converged, its
// disparity / strength replace the rig record's (use_poly), and the peak's 2D offset around x = 0
// fills dx, dy: single2dPoly (Correlation2d.java:1509-1536: the quadric of the convex-region
// samples, values as weights to ortho_vasw_pwr) with use_xy_poly, else single2dCM within
// max_corr_radius (1538-1585).  Warp per task.
// ---------------------------------------------------------------------------
__global__ void rig_disp_kernel(const float *rig_rec, float *disp, int ntiles) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntiles * TP_NDISP) return;
  const int t = i / TP_NDISP, k = i - t * TP_NDISP;
  disp[i] = (k == 1) ? rig_rec[t * 4] : ((k == 2) ? rig_rec[t * 4 + 1] : CUDART_NAN_F);
}

__global__ void __launch_bounds__(32 * LMA_NW) rig_xy_kernel(const __grid_constant__ LmaDev ld,
                                                            const __grid_constant__ TpLmaConst c, float *rig_rec,
                                                            int use_poly, int use_xy_poly) {
  extern __shared__ float sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *gsurf = sm + warp * LMA_PER_WARP;
  float *sx = gsurf + 450;
  float *sy = sx + LMA_MAX_SAMPLES, *sv = sy + LMA_MAX_SAMPLES, *sw = sv + LMA_MAX_SAMPLES;
  unsigned char *sg = (unsigned char *)(sw + LMA_MAX_SAMPLES);
  double *dmom = (double *)(gsurf + ((LMA_OFF_RED + 1) & ~1));
  double *dsolve = (double *)gsurf;  // the group surfaces are no longer needed when the solver runs
  for (int task = blockIdx.x * LMA_NW + warp; task < ld.num_tasks; task += gridDim.x * LMA_NW) {
    const int txy = ld.task_txy[task];
    const size_t tile = (size_t)(txy >> 16) * ld.tilesX + (txy & 0xffff);
    const float *lr = ld.lma + tile * 4;
    if (isnan(lr[0])) continue;  // the LMA did not run or did not converge
    const float *src = ld.corr + tile * TP_CORR;
    float dx = CUDART_NAN_F, dy = CUDART_NAN_F;
    if (use_xy_poly) {
      int ng, gdb;
      const int ns = lma_samples<true>(ld, c, 1u, 0.0f, c.ortho_vasw_pwr, src, gsurf, sx, sy, sv, sw, sg, lane, ng,
                                       gdb);
      quadric_moments(sx, sy, sv, sw, ns, lane, dmom);
      __syncwarp();
      if (lane == 0) {
        double q[3];
        if (quadric_max(dmom, ns, dsolve, q)) {
          dx = (float)(0.0 - q[0]);
          dy = (float)(-q[1]);
        }
      }
      __syncwarp();
    } else if (lane == 0) {
      float m3[3];
      mismatch_cm(src, 0, 0.0f, c.max_corr_radius, m3);
      dx = m3[0];
      dy = m3[1];
    }
    if (lane == 0) {
      float *rr = rig_rec + tile * 4;
      if (use_poly) {
        rr[0] = lr[0];
        rr[1] = lr[1];
      }
      rr[2] = dx;
      rr[3] = dy;
    }
  }
}

cudaError_t launch_rig_lma(const SceneDev &mn, const CorrConst &cc1, const TpLmaConst &c, const float *rig_corr,
                           float *rig_rec, float *tmp_disp, float *tmp_lma, int use_poly, int use_xy_poly,
                           cudaStream_t st) {
  const int ntiles = mn.tilesX * mn.tilesY;
  rig_disp_kernel<<<(ntiles * TP_NDISP + 255) / 256, 256, 0, st>>>(rig_rec, tmp_disp, ntiles);
  cudaError_t e = cudaMemsetAsync(tmp_lma, 0xff, (size_t)ntiles * 4 * sizeof(float), st);  // NaN
  if (e != cudaSuccess) return e;
  SceneDev sc = mn;
  sc.corr = const_cast<float *>(rig_corr);
  sc.disp = tmp_disp;
  TpLmaConst cl = c;
  cl.fo_correct = 0;
  cl.mismatch = 0;
  cl.mix_corr_poly = 0;
  cl.pair_mask = 1;
  e = launch_lma(sc, cc1, cl, tmp_lma, nullptr, st);
  if (e != cudaSuccess || mn.num_tasks <= 0) return e;
  LmaDev ld;
  ld.corr = rig_corr;
  ld.disp = tmp_disp;
  ld.lma = tmp_lma;
  ld.mismatch = nullptr;
  ld.task_txy = mn.task_txy;
  ld.num_tasks = mn.num_tasks;
  ld.tilesX = mn.tilesX;
  ld.P = 1;
  for (int k = 0; k < 4; k++) ld.kind_count[k] = 0;
  for (int i = 0; i < TP_MAXP; i++) ld.kinds[i] = -1;
  ld.kinds[0] = 0;
  ld.kind_count[0] = 1;
  const int bytes = lma_smem_bytes();
  e = cudaFuncSetAttribute(rig_xy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 152, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rig_xy_kernel, 32 * LMA_NW, bytes);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int units = (mn.num_tasks + LMA_NW - 1) / LMA_NW;
  const int grid = units < sms * per_sm ? units : sms * per_sm;
  rig_xy_kernel<<<grid, 32 * LMA_NW, bytes, st>>>(ld, cl, rig_rec, use_poly, use_xy_poly);
  return cudaGetLastError();
}

__global__ void mismatch_init_kernel(float *m, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) m[i] = (i % 3 == 2) ? 0.f : CUDART_NAN_F;
}

cudaError_t launch_lma(const SceneDev &sc, const CorrConst &cc, const TpLmaConst &c, float *lma_out,
                       float *mismatch_out, cudaStream_t st) {
  if (mismatch_out) {  // tiles without a task keep {NaN, NaN, 0}
    const int n = sc.tilesX * sc.tilesY * cc.num_pairs * 3;
    mismatch_init_kernel<<<(n + 255) / 256, 256, 0, st>>>(mismatch_out, n);
  }
  if (sc.num_tasks <= 0) return cudaSuccess;
  if (c.cnvx_hwnd_size < 0 || c.cnvx_hwnd_size > 4) return cudaErrorInvalidValue;  // 9x9 sample window
  LmaDev ld;
  ld.corr = sc.corr;
  ld.disp = sc.disp;
  ld.lma = lma_out;
  ld.mismatch = mismatch_out;
  ld.task_txy = sc.task_txy;
  ld.num_tasks = sc.num_tasks;
  ld.tilesX = sc.tilesX;
  ld.P = cc.num_pairs;
  for (int k = 0; k < 4; k++) ld.kind_count[k] = 0;
  for (int i = 0; i < TP_MAXP; i++) {
    const int k = (i < cc.num_pairs) ? cc.pairs[i].kind : -1;
    ld.kinds[i] = (k >= 0 && k <= 3 && i < 32 && ((c.pair_mask >> i) & 1)) ? k : -1;  // the mask holds 32 pairs
    if (ld.kinds[i] >= 0) ld.kind_count[ld.kinds[i]]++;
  }
  const int bytes = lma_smem_bytes();
  const auto kern = (mismatch_out && c.ly_poly) ? lma_kernel<true> : lma_kernel<false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 152, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * LMA_NW, bytes);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int units = (sc.num_tasks + LMA_NW - 1) / LMA_NW;
  const int grid = units < sms * per_sm ? units : sms * per_sm;
  kern<<<grid, 32 * LMA_NW, bytes, st>>>(ld, c);
  return cudaGetLastError();
}

// The 2D maximum of every task tile's pair surfaces, one warp per surface: the first cell of the
// largest value in index order (NaN cells count as -inf), then a parabola through it and its two
// neighbours on each axis (FP32: an FP64 division costs this part's FP64 pipe 1/64 of the FP32
// rate per warp; the fraction clamped to +-0.5 and taken as 0 where a neighbour is not finite).  out [tiles][P][3] = {dx, dy, strength}, px from the centre (x right, y down);
// {NaN, NaN, 0} where the maximum is on the border or not finite, all NaN outside the task list.
__global__ void __launch_bounds__(128) pair_max_kernel(const float *__restrict__ corr,
                                                       const int *__restrict__ task_txy, int num_tasks,
                                                       int tilesX, int P, float *out) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= (long long)num_tasks * P) return;  // whole warps
  const int task = (int)(w / P), pi = (int)(w - (long long)task * P);
  const int txy = task_txy[task];
  const size_t s = ((size_t)(txy >> 16) * tilesX + (txy & 0xffff)) * P + pi;
  const float *c = corr + s * TP_CORR;
  float best = -CUDART_INF_F;
  int bi = lane;
  for (int i = lane; i < TP_CORR; i += 32) {
    const float v = c[i];
    if (v > best) {  // false for NaN
      best = v;
      bi = i;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ob > best || (ob == best && oi < bi)) {
      best = ob;
      bi = oi;
    }
  }
  if (lane != 0) return;
  const int iy = bi / 15, ix = bi - 15 * iy;
  float *o = out + s * 3;
  if (ix < 1 || ix > 13 || iy < 1 || iy > 13 || !isfinite(best)) {
    o[0] = CUDART_NAN_F;
    o[1] = CUDART_NAN_F;
    o[2] = 0.f;
    return;
  }
  float f[2];
  for (int a = 0; a < 2; a++) {
    const int st = a ? 15 : 1;
    const float m = c[bi - st], p = c[bi + st];
    float fr = 0.f;
    if (isfinite(m) && isfinite(p)) {
      const float den = (m - 2.f * best) + p;
      if (den < 0.f) fr = fminf(0.5f, fmaxf(-0.5f, 0.5f * (m - p) / den));
    }
    f[a] = (float)((a ? iy : ix) - 7) + fr;
  }
  o[0] = f[0];
  o[1] = f[1];
  o[2] = best;
}

cudaError_t launch_pair_maxima(const SceneDev &sc, int P, float *out, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0xff, (size_t)sc.tilesX * sc.tilesY * P * 3 * sizeof(float), st);  // NaN
  if (e != cudaSuccess || sc.num_tasks <= 0 || P <= 0) return e;
  const long long warps = (long long)sc.num_tasks * P;
  pair_max_kernel<<<(unsigned)((warps + 3) / 4), 128, 0, st>>>(sc.corr, sc.task_txy, sc.num_tasks, sc.tilesX, P, out);
  return cudaGetLastError();
}
