// tp_texture.cu -- per-tile RGBA textures of a quad colour camera (stage 4b).
//
// Follows the texture branch of ImageDtt.clt_aberrations_quad_corr
// (ImageDtt.java:2662-2812): optional extra shift of every port by the
// measured disparity (2663-2678), per-port IMCLT of the CLT x 0.25 x
// correlation LPF into a full 16x16 tile (2680-2725), debayer with shot-noise
// correction (tile_debayer_shot_corr / tile_debayer, 3022-3147), port
// weighting by pairwise agreement (tile_combine_rgba, 2830-3000) with
// dust_remove (3002-3019), and the final RGB mix of the un-debayered tiles
// with the port weights (2788-2801).
//
// GB300 layout: one CTA of 128 threads per tile (grid-stride over the task
// list).  The 12 (port, colour) inverse transforms run on 12 of the CTA's 16
// 8-lane groups, lane r owning row r of each quadrant (the same register
// butterflies as the forward kernel).  Their unfold writes the tiles already
// divided by window^2 (the debayer's input) into zero-bordered 18x18 shared
// tiles, so the 3x3 stencil needs no edge tests.  Each thread then carries two
// pixels through debayer, shot-noise correction, port weighting and the RGB
// mix in registers; max_diff / ports_rgb take one block reduction.  Per tile
// the kernel reads the 12 KB CLT once and writes the 4 or 12 texture rows.
#include "tp_dtt.cuh"

namespace {

constexpr int TX_THREADS = 128;
constexpr int TX_P = 18;  // padded tile side
// exp(-x) of a double is 0 for x above this (below the smallest subnormal, 4.9e-324)
constexpr float TX_EXP_UNDERFLOW = 745.13f;

__device__ float d_tex_win2[256];   // lt_window2 = getWin2d()^2 (ImageDtt.java:2702, 697-713)
__device__ float d_tex_rwin2[256];  // 1 / lt_window2
__constant__ float k_rhwin[8];      // 1 / sine half-window

// the four quad ports' offsets used to scale the extra shift and the pair
// distances (ImageDtt.java:1564-1569)
__constant__ float k_port_off[4][2] = {{-0.5f, -0.5f}, {0.5f, -0.5f}, {-0.5f, 0.5f}, {0.5f, 0.5f}};

}  // namespace

// square root from the reciprocal square root (about 2 ulp; 0 at 0): for the rms rows, whose
// tolerance is far wider than the IEEE root's accuracy
__device__ __forceinline__ float sqrt_approx(float x) { return x > 0.f ? x * rsqrtf(x) : 0.f; }

// tile_debayer (ImageDtt.java:3047-3147) of two vertically adjacent pixels (y0, x), (y0 + 1, x):
// 3x3 stencil over the un-windowed tile (zero outside), the taps outside the tile dropped and the
// sum renormalised (k_corn / k_side edge factors); kern_rb = (1 2 1)^T (1 2 1) / 16 is separable,
// so the row sums of rows y0 - 1 .. y0 + 2 serve both pixels; then the shot-noise correction
// (tile_debayer_shot_corr, 3022-3045) and the window
__device__ __forceinline__ void debayer2(const TexConst &tc, float (*s_ic)[TX_P * TX_P], const float *s_win2, int x,
                                         int y0, float d[2][4][3], float part[16]) {
  const int p = (y0 + 1) * TX_P + x + 1;
  const bool ex = (x == 0) || (x == 15);
  float f_rb[2], f_g[2], lw[2];
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const int y = y0 + k;
    const bool ey = (y == 0) || (y == 15);
    f_rb[k] = (ey && ex) ? (16.0f / 9.0f) : ((ey || ex) ? (4.0f / 3.0f) : 1.0f);
    f_g[k] = (ey && ex) ? (4.0f / 3.0f) : ((ey || ex) ? (8.0f / 7.0f) : 1.0f);
    lw[k] = s_win2[y * 16 + x];
  }
#pragma unroll
  for (int ip = 0; ip < 4; ip++)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float *u = s_ic[ip * 3 + c] + p;  // pixel (y0, x)
      float acc[2];
      if (c != 2) {  // kern_rb
        float h[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const float *row = u + (k - 1) * TX_P;
          h[k] = fmaf(2.0f, row[0], row[-1] + row[1]);
        }
        acc[0] = 0.0625f * fmaf(2.0f, h[1], h[0] + h[2]);
        acc[1] = 0.0625f * fmaf(2.0f, h[2], h[1] + h[3]);
      } else {       // kern_g: sides 1/8, centre 1/2
        const float v0 = u[-TX_P], v1 = u[0], v2 = u[TX_P], v3 = u[2 * TX_P];
        acc[0] = fmaf(0.125f, (v0 + u[-1]) + (u[1] + v2), 0.5f * v1);
        acc[1] = fmaf(0.125f, (v1 + u[TX_P - 1]) + (u[TX_P + 1] + v3), 0.5f * v2);
      }
#pragma unroll
      for (int k = 0; k < 2; k++) {
        float a = acc[k] * ((c != 2) ? f_rb[k] : f_g[k]);
        if (tc.scale_shot > 0.f)
          a = tc.scale_shot * ((a > tc.min_shot) ? a * rsqrtf(a) : (tc.rsqrt_min_shot * a));
        d[k][ip][c] = a * lw[k];
        part[4 + c * 4 + ip] += d[k][ip][c];
      }
    }
}

// Per-pixel stage of a tile (debayer, shot noise, port weights, dust removal, alpha, RGB mix);
// FULL: all four ports used (the usual tile mask 0xF), so every mask test folds away.  Thread
// pr covers column pr & 15 of rows y0, y0 + 1: y0 = 2 (pr >> 5) for the first 16 lanes of a warp,
// 8 rows further down for the other 16, whose 18-float rows then start 144 floats (16 banks) on,
// so a warp's shared-memory reads of the stencils fall on 32 distinct banks.
template <bool FULL>
__device__ __forceinline__ void tex_pixels(const TexConst &tc, float (*s_ic)[TX_P * TX_P], const float *s_win2,
                                           const float *s_rwin2, float *out, int mask_rt, int used_rt,
                                           float inv_used, float ksigma, int tid, float part[16]) {
  const int mask = FULL ? 0xF : mask_rt;
  const int used = FULL ? 4 : used_rt;
  for (int pr = tid; pr < 128; pr += TX_THREADS) {
  const int x = pr & 15, y0 = ((pr >> 5) << 1) + (((pr >> 4) & 1) << 3);
  float dd[2][4][3];
  debayer2(tc, s_ic, s_win2, x, y0, dd, part);
#pragma unroll 1
  for (int k = 0; k < 2; k++) {
    const int y = y0 + k, i = y * 16 + x, p = (y + 1) * TX_P + x + 1;
    const float lw = s_win2[i], rlw = s_rwin2[p], rlw2 = rlw * rlw;
    float d[4][3];
#pragma unroll
    for (int ip = 0; ip < 4; ip++)
#pragma unroll
      for (int c = 0; c < 3; c++) d[ip][c] = k ? dd[1][ip][c] : dd[0][ip][c];
    if (tc.rows > 4) {  // per-colour rms across the used ports and their weighted norm
      float sw = 0.f;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int ip = 0; ip < 4; ip++)
          if (mask & (1 << ip)) { s0 += 1.f; s1 += d[ip][c]; }
        // sqrt(s0*s2 - s1^2)/s0 evaluated as the centred sum (no cancellation)
        const float m = __fdividef(s1, s0);
        float v = 0.f;
#pragma unroll
        for (int ip = 0; ip < 4; ip++)
          if (mask & (1 << ip)) v = fmaf(d[ip][c] - m, d[ip][c] - m, v);
        const float rms = __fdividef(sqrt_approx(v * s0), s0);
        out[(8 + c) * 256 + i] = rms;
        sw = fmaf(tc.col_weights[c] * rms, rms, sw);
      }
      out[11 * 256 + i] = sqrt_approx(sw);
    }
    // Weights are kept relative to the largest one (scale sc_w): every use of them below is
    // a ratio or homogeneous of degree 1 (dust_remove), so FP32 exp() cannot underflow to
    // 0/0 where the FP64 reference stays finite.  Where the reference's own weights
    // underflow in double (exponent below -745.13), its 0/0 results are reproduced.
    float pw[4] = {0.f, 0.f, 0.f, 0.f}, avg[3] = {0.f, 0.f, 0.f}, sc_w = 1.f;
    if (used > 1) {
      // pair weights: Gaussian of the weighted colour difference, scaled by the pair distance
      const float ks = ksigma * rlw2, ksd = 0.5f * ks;
      float ea[6];
      float amin = CUDART_INF_F;
#pragma unroll
      for (int a = 0, k = 0; a < 4; a++)
#pragma unroll
        for (int b = a + 1; b < 4; b++, k++) {
          ea[k] = CUDART_INF_F;
          if ((mask >> a) & (mask >> b) & 1) {
            // squared port distance: 1 for side pairs, 2 for the diagonals (0,3) and (1,2)
            float dd = 0.f;
#pragma unroll
            for (int c = 0; c < 3; c++) {
              const float dc = d[a][c] - d[b][c];
              dd = fmaf(tc.col_weights[c] * dc, dc, dd);
            }
            ea[k] = ((a + b == 3) ? ksd : ks) * dd;
            amin = fminf(amin, ea[k]);
          }
        }
      if (amin > TX_EXP_UNDERFLOW) {  // all pair weights 0 in double: 0/0 downstream
#pragma unroll
        for (int ip = 0; ip < 4; ip++) pw[ip] = (mask & (1 << ip)) ? CUDART_NAN_F : 0.f;
        avg[0] = avg[1] = avg[2] = CUDART_NAN_F;
      } else {
#pragma unroll
        for (int a = 0, k = 0; a < 4; a++)
#pragma unroll
          for (int b = a + 1; b < 4; b++, k++)
            if ((mask >> a) & (mask >> b) & 1) {
              const float e = __expf(amin - ea[k]);
              pw[a] += e;
              pw[b] += e;
            }
        int b1 = 0;
#pragma unroll
        for (int ip = 1; ip < 4; ip++) if (pw[ip] > pw[b1]) b1 = ip;
        int b2 = (b1 == 0) ? 1 : 0;
#pragma unroll
        for (int ip = b2 + 1; ip < 4; ip++) if (ip != b1 && pw[ip] > pw[b2]) b2 = ip;
        float p1 = 0.f, p2 = 0.f;  // register-resident selection of the two best ports
#pragma unroll
        for (int ip = 0; ip < 4; ip++) { if (ip == b1) p1 = pw[ip]; if (ip == b2) p2 = pw[ip]; }
        const float wa = __fdividef(p1, p1 + p2), wb = 1.0f - wa;
        float wv[4];  // the best pair's weights as a vector over the ports (the others 0)
#pragma unroll
        for (int ip = 0; ip < 4; ip++) wv[ip] = (ip == b1) ? wa : ((ip == b2) ? wb : 0.f);
#pragma unroll
        for (int c = 0; c < 3; c++) avg[c] = fmaf(wv[3], d[3][c], fmaf(wv[2], d[2][c], fmaf(wv[1], d[1][c], wv[0] * d[0][c])));
        // re-weight every used port by its distance from the best-pair average
        float eb[4], bmin = CUDART_INF_F;
#pragma unroll
        for (int ip = 0; ip < 4; ip++) {
          float d2 = 0.f;
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const float dc = d[ip][c] - avg[c];
            d2 = fmaf(tc.col_weights[c] * dc, dc, d2);
          }
          eb[ip] = ks * d2;
          if (mask & (1 << ip)) bmin = fminf(bmin, eb[ip]);
        }
        const bool zero = bmin > TX_EXP_UNDERFLOW;  // all weights 0 in double
#pragma unroll
        for (int ip = 0; ip < 4; ip++)
          if (mask & (1 << ip)) pw[ip] = zero ? 0.f : __expf(bmin - eb[ip]);
        sc_w = zero ? 1.f : expf(-bmin);
        const float kk = __fdividef(1.0f, ((pw[0] + pw[1]) + pw[2]) + pw[3]);
#pragma unroll
        for (int c = 0; c < 3; c++) {
          float v = 0.f;
#pragma unroll
          for (int ip = 0; ip < 4; ip++) v += kk * pw[ip] * d[ip][c];
          avg[c] = v;
        }
      }
    } else if (used > 0) {
#pragma unroll
      for (int ip = 0; ip < 4; ip++)
        if (mask & (1 << ip)) {
#pragma unroll
          for (int c = 0; c < 3; c++) avg[c] = d[ip][c];
          pw[ip] = 1.f;
        }
    }
    if (tc.dust_remove && used == 4) {  // dust_remove (ImageDtt.java:3002-3019), from port 1 as there
      int wi = 0;
#pragma unroll
      for (int ip = 1; ip < 4; ip++) if (pw[ip] < pw[wi]) wi = ip;
      float a = 0.f, pwi = 0.f;
#pragma unroll
      for (int ip = 0; ip < 4; ip++) { if (ip >= 1 && ip != wi) a += pw[ip]; if (ip == wi) pwi = pw[ip]; }
      a *= (1.0f / 3.0f);
      const float scl = 1.0f + __fdividef(a - pwi, a * 3.f);
#pragma unroll
      for (int ip = 1; ip < 4; ip++) if (ip != wi) pw[ip] *= scl;
#pragma unroll
      for (int ip = 0; ip < 4; ip++) if (ip == wi) pw[ip] *= __fdividef(pwi, a);
    }
    float alpha = 0.f;
#pragma unroll
    for (int ip = 0; ip < 4; ip++) if (mask & (1 << ip)) alpha += pw[ip];
    out[3 * 256 + i] = (alpha * sc_w) * (lw * inv_used);
    if (tc.rows > 4) {
#pragma unroll
      for (int ip = 0; ip < 4; ip++) out[(4 + ip) * 256 + i] = pw[ip] * sc_w;
    }
    // max_diff partial (ImageDtt.java:2964-2981); a NaN average is skipped as there
#pragma unroll
    for (int ip = 0; ip < 4; ip++)
      if (mask & (1 << ip)) {
        float d2 = 0.f;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const float dc = d[ip][c] - avg[c];
          d2 = fmaf(dc * dc, tc.col_weights[c], d2);
        }
        part[ip] = fmaxf(part[ip], d2 * lw);
      }
    // RGB mix of the un-debayered tiles (ImageDtt.java:2788-2801)
    float sw = ((pw[0] + pw[1]) + pw[2]) + pw[3];
    if (sw != 0.f) sw = __fdividef(1.0f, sw);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      float v = 0.f;
#pragma unroll
      for (int ip = 0; ip < 4; ip++) v += sw * pw[ip] * s_ic[ip * 3 + c][p];
      v *= lw;  // the tiles are kept un-windowed
      out[c * 256 + i] = v;
    }
  }
  }
}

__global__ void __launch_bounds__(TX_THREADS, 5) texture_kernel(const __grid_constant__ SceneDev sc,
                                                             const __grid_constant__ TexConst tc) {
  // per-port IMCLT tiles [port * 3 + colour][18 x 18]: the 16x16 tile inside a zero border,
  // so the debayer stencil needs no edge tests (the border is never written)
  __shared__ float s_ic[12][TX_P * TX_P];
  __shared__ float s_tbuf[16][72];   // transpose buffers, one per 8-lane group
  __shared__ float s_win2[256], s_rwin2[TX_P * TX_P], s_lpf[64];
  __shared__ float s_red[4][16];     // per-warp aux partials
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, q = lane >> 3, r = lane & 7;
  const int S = sc.num_sensors, C = sc.num_colors;
  for (int i = tid; i < 256; i += TX_THREADS) s_win2[i] = d_tex_win2[i];
  for (int i = tid; i < TX_P * TX_P; i += TX_THREADS) {
    const int y = i / TX_P - 1, x = i % TX_P - 1;
    const bool in = y >= 0 && y < 16 && x >= 0 && x < 16;
    s_rwin2[i] = in ? d_tex_rwin2[y * 16 + x] : 0.f;
    for (int pc = 0; pc < 12; pc++) s_ic[pc][i] = 0.f;
  }
  if (tid < 64) s_lpf[tid] = 0.25f * tc.lpf[tid];
  // unfold rows fed by source row r (DttRad2.get_unfold_index_signs, 392-404)
  const int i1 = (r >= 4) ? r - 4 : 11 - r, i2 = (r >= 4) ? 11 - r : r + 12;
  const float sa1 = (r >= 4) ? 1.f : -1.f, sb1 = 1.f;
  const float sa2 = -1.f, sb2 = (r >= 4) ? 1.f : -1.f;
  // the unfold writes the un-windowed tile (IMCLT / window^2, the debayer's input): the
  // window factors of DttRad2.unfold_tile become their reciprocals
  const float w1 = k_rhwin[i1 < 8 ? i1 : 15 - i1], w2 = k_rhwin[i2 < 8 ? i2 : 15 - i2];
  const float kc1 = sa1 * w1, ks1 = sb1 * w1, kc2 = sa2 * w2, ks2 = sb2 * w2;
  const float ksigma = 1.0f / (2.0f * tc.diff_sigma * tc.diff_sigma);
  __syncthreads();

  for (int task = blockIdx.x; task < sc.num_tasks; task += gridDim.x) {
    const int txy = sc.task_txy[task], op = sc.task_op[task];
    const size_t tile = (size_t)(txy >> 16) * sc.tilesX + (txy & 0xffff);
    const int mask = op & 0xf;  // ImageDtt.getImgMask (204)
    // extra disparity (ImageDtt.java:2422-2427, 2663): not for forced-disparity tiles
    float extra = 0.f;
    if (tc.extra_index >= 0 && !(op & 0x100)) {
      extra = tc.extra_src[tile * tc.extra_stride + tc.extra_index];
      if (isnan(extra)) extra = 0.f;
    }
    // ---------------- per-port IMCLT ----------------
    const int g = warp * 4 + q;  // warps 0-2 carry the 12 (port, colour) tiles
    if (g < 12) {
      const int port = g / 3, chn = g - 3 * port;
      const float *src = sc.clt + ((tile * S + port) * C + chn) * TP_CLT + r * 8;
      float o[4][8];
#pragma unroll
      for (int m = 0; m < 4; m++) {
        const float4 a = __ldg((const float4 *)(src + m * 64)), b = __ldg((const float4 *)(src + m * 64 + 4));
        o[m][0] = a.x; o[m][1] = a.y; o[m][2] = a.z; o[m][3] = a.w;
        o[m][4] = b.x; o[m][5] = b.y; o[m][6] = b.z; o[m][7] = b.w;
      }
      if (extra != 0.f) {  // fract_shift (ImageDtt.java:5490-5584) by the extra port shift
        const float sx = extra * k_port_off[port][0] / tc.corr_magic_scale;
        const float sy = extra * k_port_off[port][1] / tc.corr_magic_scale;
        float ch, shh, cvr, svr;
        sincospif(0.0625f * (2 * r + 1) * sx, &shh, &ch);
        sincospif(0.0625f * (2 * r + 1) * sy, &svr, &cvr);
        const int base = lane & 24;
#pragma unroll
        for (int v = 0; v < 8; v++) {
          const float cv = __shfl_sync(0xffffffffu, cvr, base + v);
          const float sv = __shfl_sync(0xffffffffu, svr, base + v);
          const float t0 = o[0][v] * ch - o[1][v] * shh, t1 = o[1][v] * ch + o[0][v] * shh;
          const float t2 = o[2][v] * ch - o[3][v] * shh, t3 = o[3][v] * ch + o[2][v] * shh;
          o[0][v] = t0 * cv - t2 * sv;
          o[2][v] = t2 * cv + t0 * sv;
          o[1][v] = t1 * cv - t3 * sv;
          o[3][v] = t3 * cv + t1 * sv;
        }
      }
#pragma unroll
      for (int v = 0; v < 8; v++) {
        const float l = s_lpf[r * 8 + v];
#pragma unroll
        for (int m = 0; m < 4; m++) o[m][v] *= l;
      }
      // inverse DCT-IV/DST-IV with the swapped mode (ImageDtt.java:2693)
      float t[4][8];
#pragma unroll
      for (int m = 0; m < 4; m++) {
        float z[8];
        dtt4_fast(o[m], z, (m >> 1) & 1);
        group_transpose(z, s_tbuf[g], r);
        dtt4_fast(z, t[m], m & 1);
      }
      float *dst = s_ic[g];
#pragma unroll
      for (int jj = 0; jj < 16; jj++) {
        const int seg = jj >> 2, xx = jj & 3;
        const int ih = (seg == 0) ? xx + 4 : ((seg == 1) ? 7 - xx : ((seg == 2) ? 3 - xx : xx));
        const float hs1 = (seg == 0) ? 1.f : -1.f, hs2 = (seg == 3) ? -1.f : 1.f;
        const float wh = k_rhwin[jj < 8 ? jj : 15 - jj];
        const float khc = hs1 * wh, khs = hs2 * wh;
        const float A = fmaf(khs, t[1][ih], khc * t[0][ih]);
        const float B = fmaf(khs, t[3][ih], khc * t[2][ih]);
        dst[(i1 + 1) * TX_P + jj + 1] = fmaf(ks1, B, kc1 * A);
        dst[(i2 + 1) * TX_P + jj + 1] = fmaf(ks2, B, kc2 * A);
      }
    }
    __syncthreads();
    // ---------------- per pixel: debayer + shot noise, port weights, alpha, RGB ----------------
    float *out = sc.tex + tile * (size_t)tc.rows * 256;
    const int used = (mask & 1) + ((mask >> 1) & 1) + ((mask >> 2) & 1) + ((mask >> 3) & 1);
    const float inv_used = 1.0f / used;  // inf for an empty mask: alpha is then 0 * inf = NaN as in double
    float part[16];  // this thread's max_diff[4] and ports_rgb[12] partials
#pragma unroll
    for (int k = 0; k < 16; k++) part[k] = 0.f;
    if (mask == 0xF) tex_pixels<true>(tc, s_ic, s_win2, s_rwin2, out, mask, used, inv_used, ksigma, tid, part);
    else tex_pixels<false>(tc, s_ic, s_win2, s_rwin2, out, mask, used, inv_used, ksigma, tid, part);
    if (sc.tex_aux) {
      // one block reduction for max_diff (max, entries 0-3) and ports_rgb (sum): a reduce-scatter
      // over the warp (each exchange halves the entries a lane keeps: 15 shuffles instead of 80),
      // after which lanes 2k and 2k + 1 hold entry k, then across the four warps
#pragma unroll
      for (int half = 8, m = 16; half > 0; half >>= 1, m >>= 1) {
        const bool up = (lane & m) != 0;
#pragma unroll
        for (int i = 0; i < half; i++) {
          const float keep = up ? part[half + i] : part[i];
          const float v = __shfl_xor_sync(0xffffffffu, up ? part[i] : part[half + i], m);
          // the entry kept here: index (lane >> 1) at the end, (lane >> 1) & ~(half - 1) + i now
          const int k = ((lane >> 1) & ~(half - 1) & 15) + i;
          part[i] = (k < 4) ? fmaxf(keep, v) : keep + v;
        }
      }
      {
        const int k = lane >> 1;
        const float v = __shfl_xor_sync(0xffffffffu, part[0], 1);
        part[0] = (k < 4) ? fmaxf(part[0], v) : part[0] + v;
        if (!(lane & 1)) s_red[warp][k] = part[0];
      }
      __syncthreads();
      if (tid < 16) {
        float* aux = sc.tex_aux + tile * 16;
        if (tid < 4) {
          const float m = fmaxf(fmaxf(s_red[0][tid], s_red[1][tid]), fmaxf(s_red[2][tid], s_red[3][tid]));
          aux[tid] = sqrtf(m);
        } else {
          aux[tid] = ((s_red[0][tid] + s_red[1][tid]) + (s_red[2][tid] + s_red[3][tid])) * (1.0f / 256.0f);
        }
      }
    }
    __syncthreads();
  }
}

cudaError_t upload_texture_constants() {
  cudaError_t e = upload_dtt_constants();
  if (e != cudaSuccess) return e;
  float w2[256], rw2[256];
  for (int i = 0; i < 16; i++)
    for (int j = 0; j < 16; j++) {
      const double wi = std::sin(3.14159265358979323846 / 16.0 * ((i < 8 ? i : 15 - i) + 0.5));
      const double wj = std::sin(3.14159265358979323846 / 16.0 * ((j < 8 ? j : 15 - j) + 0.5));
      const double w = wi * wj;
      w2[i * 16 + j] = (float)(w * w);
      rw2[i * 16 + j] = (float)(1.0 / (w * w));
    }
  float rh[8];
  for (int i = 0; i < 8; i++) rh[i] = (float)(1.0 / std::sin(3.14159265358979323846 / 16.0 * (i + 0.5)));
  e = cudaMemcpyToSymbol(k_rhwin, rh, sizeof(rh));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(d_tex_win2, w2, sizeof(w2));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(d_tex_rwin2, rw2, sizeof(rw2));
  return e;
}

cudaError_t launch_textures(const SceneDev &sc, const TexConst &tc, cudaStream_t st) {
  if (sc.num_tasks <= 0) return cudaSuccess;
  if (sc.num_sensors != 4 || sc.num_colors != 3) return cudaErrorInvalidValue;
  int dev = 0, sms = 152, per_sm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, texture_kernel, TX_THREADS, 0);
  if (per_sm < 1) per_sm = 1;
  const int grid = sc.num_tasks < sms * per_sm ? sc.num_tasks : sms * per_sm;
  texture_kernel<<<grid, TX_THREADS, 0, st>>>(sc, tc);
  return cudaGetLastError();
}
