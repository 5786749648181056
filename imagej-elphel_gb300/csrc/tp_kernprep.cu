// tp_kernprep.cu -- aberration-kernel preparation on the device.
//
// The chain of QuadCLT.calculateCLTKernel (QuadCLT.java:433-667) for every
// kernel tile of a sensor: a 64x64 double-resolution PSF is centred on its
// centroid and downscaled to 15x15 (clt_convert_double_kernel,
// ImageDtt.java:4625-4672), normalised so that kernel x window sums to 16
// (clt_normalize_kernel 4674-4696), split into its four symmetric quadrants
// (clt_symmetrize_kernel 4698-4723) and taken to the CLT domain with the 2D
// DCT-IIIe / DST-IIIe (clt_dtt3_kernel 4725-4734, DttRad2.java:648-666).  The
// kernel centre offsets get their per-grid derivatives from a 3x3
// least-squares fit over the neighbouring kernel tiles
// (clt_fill_coord_corr 4792-4851).
//
// One warp per kernel tile.  The centroid sums are accumulated in FP64 so
// the integer window centre (java round of the centroid) is the reference's;
// the rest is FP32.
#include "tp_internal.h"

#include <math_constants.h>

#include <cmath>

namespace {

__constant__ float k_c3[64], k_s3[64];  // CIIIe, SIIIe as y[k] = sum_j M[k * 8 + j] x[j]
__constant__ float k_nwin[64];          // cos(pi i / 16) cos(pi j / 16), the normalisation window

__device__ __forceinline__ double java_round_d(double x) {
  const double f = floor(x);
  return (x - f >= 0.5) ? f + 1.0 : f;
}

}  // namespace

__global__ void __launch_bounds__(128) kernel_prep_kernel(const float *__restrict__ psf, int nk, int normalize,
                                                          float *__restrict__ clt_out, float *__restrict__ ext_out) {
  __shared__ float s_dst[4][240];
  __shared__ float s_sym[4][4][64];
  __shared__ float s_tmp[4][4][64];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *dst = s_dst[warp];
  float(*sym)[64] = s_sym[warp];
  float(*tmp)[64] = s_tmp[warp];
  for (int k = blockIdx.x * 4 + warp; k < nk; k += gridDim.x * 4) {
    const float *src = psf + (size_t)k * 4096;
    // centroid (FP64 sums)
    double sx = 0.0, sy = 0.0, s = 0.0;
    for (int idx = lane; idx < 4096; idx += 32) {
      const double d = (double)__ldg(src + idx);
      const int i = (idx >> 6) - 32, j = (idx & 63) - 32;
      sx += j * d;
      sy += i * d;
      s += d;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
      s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    int src_x = (int)java_round_d(sx / s) + 32, src_y = (int)java_round_d(sy / s) + 32;
    if (src_x < 16) src_x = 15;
    else if (src_x > 48) src_x = 48;
    if (src_y < 16) src_y = 15;
    else if (src_y > 48) src_y = 48;
    // downscale to 15 x 15 with the 3x3 (1, 1/2, 1/4) weights around every second pixel
    const int ofs[9] = {0, -64, -1, 1, 64, -65, -63, 63, 65};
    const float wts[9] = {1.0f, 0.5f, 0.5f, 0.5f, 0.5f, 0.25f, 0.25f, 0.25f, 0.25f};
    float sn = 0.f;
    for (int o = lane; o < 225; o += 32) {
      const int i = o / 15 - 7, j = o - (o / 15) * 15 - 7;
      const int si = (src_y + 2 * i) * 64 + src_x + 2 * j;
      float d = 0.f;
#pragma unroll
      for (int t = 0; t < 9; t++) d = fmaf(wts[t], __ldg(src + si + ofs[t]), d);
      dst[o] = d;
      sn = fmaf(d, k_nwin[(i < 0 ? -i : i) * 8 + (j < 0 ? -j : j)], sn);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sn += __shfl_xor_sync(0xffffffffu, sn, o);
    __syncwarp();
    if (normalize) {
      const float scale = 16.0f / sn;
      for (int o = lane; o < 225; o += 32) dst[o] *= scale;
      __syncwarp();
    }
    // four symmetric quadrants (the AA quadrant takes the same signs as AS, as the reference does)
    for (int e = lane; e < 64; e += 32) {
      const int i = e >> 3, j = e & 7;
      const int c = 7 * 15 + 7;
      const float d0 = dst[c - i * 15 - j], d1 = dst[c - i * 15 + j], d2 = dst[c + i * 15 - j], d3 = dst[c + i * 15 + j];
      sym[0][i * 8 + j] = 0.25f * (((d0 + d1) + d2) + d3);
      if (j > 0) sym[1][i * 8 + j - 1] = 0.25f * (((-d0 + d1) - d2) + d3);
      if (i > 0) sym[2][(i - 1) * 8 + j] = 0.25f * (((-d0 - d1) + d2) + d3);
      if (i > 0 && j > 0) sym[3][(i - 1) * 8 + j - 1] = 0.25f * (((-d0 + d1) - d2) + d3);
      if (j == 7) {
        sym[1][i * 8 + 7] = 0.f;
        sym[3][i * 8 + 7] = 0.f;
      }
      if (i == 7) {
        sym[2][7 * 8 + j] = 0.f;
        sym[3][7 * 8 + j] = 0.f;
      }
    }
    __syncwarp();
    // 2D DCT-IIIe / DST-IIIe per quadrant q (rows with bit 0 of q, then columns with bit 1)
    for (int e = lane; e < 256; e += 32) {
      const int q = e >> 6, r = (e >> 3) & 7, kk = e & 7;
      const float *M = (q & 1) ? k_s3 : k_c3;
      float v = 0.f;
#pragma unroll
      for (int j = 0; j < 8; j++) v = fmaf(M[kk * 8 + j], sym[q][r * 8 + j], v);
      tmp[q][kk * 8 + r] = v;
    }
    __syncwarp();
    float *co = clt_out + (size_t)k * 256;
    for (int e = lane; e < 256; e += 32) {
      const int q = e >> 6, r = (e >> 3) & 7, kk = e & 7;
      const float *M = (q & 2) ? k_s3 : k_c3;
      float v = 0.f;
#pragma unroll
      for (int j = 0; j < 8; j++) v = fmaf(M[kk * 8 + j], tmp[q][r * 8 + j], v);
      co[q * 64 + r * 8 + kk] = v;
    }
    if (lane < 8) {
      float v = 0.f;
      if (lane == 0) v = 0.5f * (float)(src_x - 32);
      else if (lane == 1) v = 0.5f * (float)(src_y - 32);
      else if (lane == 2) v = (float)(0.5 * (sx / s));
      else if (lane == 3) v = (float)(0.5 * (sy / s));
      ext_out[(size_t)k * 8 + lane] = v;
    }
    __syncwarp();
  }
}

// 3x3 least-squares slopes of the kernel centre offsets over the kernel grid
// (clt_fill_coord_corr): ext [kv][kh][C][8], entries 4..7 written
__global__ void fill_coord_corr_kernel(float *ext, int kh, int kv, int C, int kern_step) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= kh * kv * C) return;
  const int c = g % C, t = g / C, tx = t % kh, ty = t / kh;
  double s0 = 0, sx = 0, sx2 = 0, sy = 0, sy2 = 0, sz = 0, sxz = 0, syz = 0, sw = 0, sxw = 0, syw = 0;
  for (int dty = -1; dty < 2; dty++) {
    const int y = ty + dty;
    if (y < 0 || y >= kv) continue;
    for (int dtx = -1; dtx < 2; dtx++) {
      const int x = tx + dtx;
      if (x < 0 || x >= kh) continue;
      const float *ce = ext + (((size_t)y * kh + x) * C + c) * 8;
      const double z = ce[2], w = ce[3];
      s0 += 1; sx += dtx; sx2 += dtx * dtx; sy += dty; sy2 += dty * dty;
      sz += z; sxz += dtx * z; syz += dty * z;
      sw += w; sxw += dtx * w; syw += dty * w;
    }
  }
  float *ce = ext + (((size_t)ty * kh + tx) * C + c) * 8;
  const double denom_x = (sx2 * s0 - sx * sx) * kern_step, denom_y = (sy2 * s0 - sy * sy) * kern_step;
  ce[4] = (float)((sxz * s0 - sz * sx) / denom_x);
  ce[5] = (float)((syz * s0 - sz * sy) / denom_y);
  ce[6] = (float)((sxw * s0 - sw * sx) / denom_x);
  ce[7] = (float)((syw * s0 - sw * sy) / denom_y);
}

cudaError_t upload_kernprep_constants() {
  float c3[64], s3[64], nw[64];
  const double pi = 3.14159265358979323846, scale = std::sqrt(2.0 / 8);
  for (int j = 0; j < 8; j++) {
    const double ej3 = (j == 0 || j == 7) ? 0.5 : 1.0, ejs = (j == 7) ? 0.5 : 1.0;
    for (int k = 0; k < 8; k++) {
      c3[k * 8 + j] = (float)(scale * ej3 * std::cos(j * (2 * k + 1) * pi / 16));
      s3[k * 8 + j] = (float)(scale * ejs * std::sin((j + 1) * (2 * k + 1) * pi / 16));
    }
  }
  for (int i = 0; i < 8; i++)
    for (int j = 0; j < 8; j++) nw[i * 8 + j] = (float)(std::cos(pi * i / 16) * std::cos(pi * j / 16));
  cudaError_t e = cudaMemcpyToSymbol(k_c3, c3, sizeof(c3));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(k_s3, s3, sizeof(s3));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(k_nwin, nw, sizeof(nw));
  return e;
}

cudaError_t launch_kernel_prep(const float *psf_dev, int nk, int normalize, float *clt_out, float *ext_out,
                               cudaStream_t st) {
  if (nk <= 0) return cudaSuccess;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int need = (nk + 3) / 4;
  const int grid = need < sms * 16 ? need : sms * 16;
  kernel_prep_kernel<<<grid, 128, 0, st>>>(psf_dev, nk, normalize, clt_out, ext_out);
  return cudaGetLastError();
}

cudaError_t launch_fill_coord_corr(float *ext, int kh, int kv, int C, int kern_step, cudaStream_t st) {
  const int n = kh * kv * C;
  if (n <= 0) return cudaSuccess;
  fill_coord_corr_kernel<<<(n + 127) / 128, 128, 0, st>>>(ext, kh, kv, C, kern_step);
  return cudaGetLastError();
}
