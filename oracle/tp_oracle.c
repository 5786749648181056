/*
 * tp_oracle.c -- FP64 CPU restatement of the imagej-elphel tile-processor path.
 *
 * TEST INFRASTRUCTURE ONLY (correctness oracle and timed CPU baseline).  The
 * product library never links this file.  Every function names the reference
 * method and line range it restates; J/ = src/main/java/com/elphel/imagej/.
 * Loop orders and operation orders follow the reference so that the FP64
 * results are those the Java code computes (up to libm last-ulp differences).
 */
#include "tp_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* DttRad2 (J/tileprocessor/DttRad2.java)                                     */
/* ------------------------------------------------------------------------- */

static double CN1[2][4], SN1[2][4];           /* setup_arrays (1043-1058) */
static double COSPI_1_8_SQRT2, COSPI_3_8_SQRT2, SQRT2;
static double CIIe[8][8], CIIIe[8][8], SIIe[8][8], SIIIe[8][8], CIV[8][8], CII[8][8];
static double HWINDOW[8];
static int FOLD_INDEX[64][4];
static int UNFOLD_INDEX[256];
static double UNFOLD_K[4][256];
static pthread_once_t tables_once = PTHREAD_ONCE_INIT;

/* DttRad2.get_fold_indices (109-144) */
static void fold_indices(int x, int n, int ind[2][6]) {
  int n1 = n >> 1;
  if (x < n1) {
    ind[0][0] = n + n1 - x - 1; ind[0][1] = n1 + x;     ind[0][2] = -1; ind[0][3] = 1;
    ind[0][4] = n1 - x - 1;     ind[0][5] = -1;
    ind[1][0] = n + n1 + x;     ind[1][1] = n1 - x - 1; ind[1][2] = -1; ind[1][3] = -1;
    ind[1][4] = n1 + x;         ind[1][5] = -1;
  } else {
    x -= n1;
    ind[0][0] = x;              ind[0][1] = x;          ind[0][2] = 1;  ind[0][3] = 1;
    ind[0][4] = n - x - 1;      ind[0][5] = 1;
    ind[1][0] = n - x - 1;      ind[1][1] = n - x - 1;  ind[1][2] = -1; ind[1][3] = 1;
    ind[1][4] = x;              ind[1][5] = 1;
  }
}

/* DttRad2.get_unfold_index_signs (392-404) */
static void unfold_index_signs(int x, int n, int is2[3]) {
  int n1 = n >> 1;
  int segm = x / n1;
  x = x % n1;
  switch (segm) {
    case 0: is2[0] = x + n1;     is2[1] = 1;  is2[2] = 1;  break;
    case 1: is2[0] = n - x - 1;  is2[1] = -1; is2[2] = 1;  break;
    case 2: is2[0] = n1 - x - 1; is2[1] = -1; is2[2] = 1;  break;
    default: is2[0] = x;         is2[1] = -1; is2[2] = -1; break;
  }
}

static void init_tables(void) {
  const int n = 8;
  COSPI_1_8_SQRT2 = cos(M_PI / 8) * sqrt(2.0);
  COSPI_3_8_SQRT2 = cos(3 * M_PI / 8) * sqrt(2.0);
  SQRT2 = sqrt(2.0);
  for (int t = 0; t < 2; t++) {                 /* setup_arrays (1043-1058) */
    int n1 = 2 << t;
    double pi_4n = M_PI / (8 * n1);
    for (int k = 0; k < n1; k++) {
      CN1[t][k] = cos((2 * k + 1) * pi_4n);
      SN1[t][k] = sin((2 * k + 1) * pi_4n);
    }
  }
  double scale = sqrt(2.0 / n);
  double pi_2n = M_PI / (2 * n);
  double pi_4n = M_PI / (4 * n);
  for (int j = 0; j < n; j++) {
    double ejc = (j == 0) ? sqrt(0.5) : 1.0;
    double ej3 = ((j == 0) || (j == (n - 1))) ? 0.5 : 1.0;
    double ejs = (j == (n - 1)) ? 0.5 : 1.0;
    for (int k = 0; k < n; k++) {
      CII[j][k] = scale * ejc * cos(j * (2 * k + 1) * pi_2n);          /* setup_CII  (1074-1093) */
      CIIe[j][k] = scale * cos(j * (2 * k + 1) * pi_2n);               /* setup_CIIe (1095-1111) */
      CIIIe[k][j] = scale * ej3 * cos(j * (2 * k + 1) * pi_2n);        /* setup_CIIIe (1113-1133) */
      SIIe[j][k] = scale * sin((j + 1) * (2 * k + 1) * pi_2n);         /* setup_SIIe (1154-1170) */
      SIIIe[k][j] = scale * ejs * sin((j + 1) * (2 * k + 1) * pi_2n);  /* setup_SIIIe (1172-1192) */
    }
  }
  for (int j = 0; j < n; j++)                                          /* setup_CIV (1136-1152) */
    for (int k = j; k < n; k++) {
      CIV[j][k] = scale * cos((2 * j + 1) * (2 * k + 1) * pi_4n);
      CIV[k][j] = CIV[j][k];
    }
  double f = M_PI / (2.0 * n);                                         /* set_window(1) (674-694) */
  for (int i = 0; i < n; i++) HWINDOW[i] = sin(f * (i + 0.5));
  /* set_fold_2d index part (146-170) */
  for (int i = 0; i < n; i++) {
    int fi[2][6], fj[2][6];
    fold_indices(i, n, fi);
    for (int j = 0; j < n; j++) {
      fold_indices(j, n, fj);
      int vert_ind[2] = {fi[0][0], fi[1][0]};
      int hor_ind[2] = {fj[0][0], fj[1][0]};
      for (int k = 0; k < 4; k++) FOLD_INDEX[n * i + j][k] = 2 * n * vert_ind[(k >> 1) & 1] + hor_ind[k & 1];
    }
  }
  /* set_unfold_2d (405-434) */
  int n2 = 2 * n;
  for (int i = 0; i < n2; i++) {
    int iv[3];
    unfold_index_signs(i, n, iv);
    double wv = HWINDOW[(i < n) ? i : n2 - i - 1];
    double k_vert[2] = {iv[1] * wv, iv[2] * wv};
    int index_vert = iv[0] * n;
    for (int j = 0; j < n2; j++) {
      int ih[3];
      unfold_index_signs(j, n, ih);
      double wh = HWINDOW[(j < n) ? j : n2 - j - 1];
      double k_hor[2] = {ih[1] * wh, ih[2] * wh};
      UNFOLD_INDEX[n2 * i + j] = index_vert + ih[0];
      for (int mode = 0; mode < 4; mode++) UNFOLD_K[mode][n2 * i + j] = k_vert[(mode >> 1) & 1] * k_hor[mode & 1];
    }
  }
}
static void tables(void) { pthread_once(&tables_once, init_tables); }

static int ilog2(int n) { int i = 0; for (; n > 1; n >>= 1) i++; return i; }

static void dctiv_recurs(const double *x, int n, double *y);

/* DttRad2._dctii_recurs (1083-1105) */
static void dctii_recurs(const double *x, int n, double *y) {
  if (n == 2) { y[0] = x[0] + x[1]; y[1] = x[0] - x[1]; return; }
  int n1 = n >> 1;
  double u0[4] = {0}, u1[4] = {0}, v0[4], v1[4];
  for (int j = 0; j < n1; j++) {
    u0[j] = (x[j] + x[n - j - 1]);
    u1[j] = (x[j] - x[n - j - 1]);
  }
  dctii_recurs(u0, n1, v0);
  dctiv_recurs(u1, n1, v1);
  for (int j = 0; j < n1; j++) { y[2 * j] = v0[j]; y[2 * j + 1] = v1[j]; }
}

/* DttRad2._dctiv_recurs (1107-1146) */
static void dctiv_recurs(const double *x, int n, double *y) {
  if (n == 2) {
    y[0] = COSPI_1_8_SQRT2 * x[0] + COSPI_3_8_SQRT2 * x[1];
    y[1] = COSPI_3_8_SQRT2 * x[0] - COSPI_1_8_SQRT2 * x[1];
    return;
  }
  int n1 = n >> 1;
  int t = ilog2(n1) - 1;
  double u0[4] = {0}, u1[4] = {0}, v0[4], v1[4], w0[4] = {0}, w1[4] = {0};
  for (int j = 0; j < n1; j++) {
    u0[j] = (CN1[t][j] * x[j] + SN1[t][j] * x[n - j - 1]);
    u1[j] = (double)(1 - 2 * (j & 1)) * (-SN1[t][n1 - j - 1] * x[n1 - j - 1] + CN1[t][n1 - j - 1] * x[n1 + j]);
  }
  dctii_recurs(u0, n1, v0);
  dctii_recurs(u1, n1, v1);
  w0[0] = SQRT2 * v0[0];
  w1[n1 - 1] = SQRT2 * v1[0];
  for (int j = 0; j < n1; j++) {
    int sgn = (1 - 2 * (j & 1));
    if (j > 0) w0[j] = v0[j] - sgn * v1[n1 - j];
    if (j < (n1 - 1)) w1[j] = v0[j + 1] - sgn * v1[n1 - j - 1];
  }
  for (int j = 0; j < n1; j++) { y[2 * j] = w0[j]; y[2 * j + 1] = w1[j]; }
}

void or_dct_iv8(const double *x, double *y) {  /* dct_iv (80-85) */
  tables();
  dctiv_recurs(x, 8, y);
  double scale = 1.0 / sqrt(8);
  for (int i = 0; i < 8; i++) y[i] *= scale;
}

void or_dst_iv8(const double *x, double *y) {  /* dst_iv (87-98) */
  tables();
  double xr[8];
  for (int i = 0, j = 7; i < 8; i++) xr[i] = x[j--];
  dctiv_recurs(xr, 8, y);
  double scale = 1.0 / sqrt(8);
  for (int i = 0; i < 8; i++) { y[i] *= scale; scale = -scale; }
}

void or_dct_ii8(const double *x, double *y) {  /* dct_ii (68-78) */
  tables();
  dctii_recurs(x, 8, y);
  double scale = 1.0 / sqrt(8);
  for (int i = 0; i < 8; i++) y[i] *= scale;
}

/* DST-II as the reference GPU computes it (dttii_shared_mem with dst_not_dct, dtt8x8.cuh:296-378):
 * the DCT-II of the input with its odd samples negated, output in reverse order */
void or_dst_ii8(const double *x, double *y) {
  double xs[8], t[8];
  for (int i = 0; i < 8; i++) xs[i] = (i & 1) ? -x[i] : x[i];
  or_dct_ii8(xs, t);
  for (int i = 0; i < 8; i++) y[i] = t[7 - i];
}

/* GPU_DTT24_DRV (dtt8x8.cuh:100-158) on one 8x8 block, row-major in and out: every row
 * transformed (horizontal pass: DCT if bit 0 of mode is clear, else DST), then every column
 * (vertical pass: bit 1); modes 0-3 DCT-IV / DST-IV (DttRad2.dct_iv / dst_iv), 4-7 DCT-II /
 * DST-II (DttRad2.dct_ii and its DST counterpart above) */
void or_dtt24(const double *x, double *y, int mode) {
  void (*fc)(const double *, double *) = (mode > 3) ? or_dct_ii8 : or_dct_iv8;
  void (*fs)(const double *, double *) = (mode > 3) ? or_dst_ii8 : or_dst_iv8;
  double tmp[64], line[8], out[8];
  for (int r = 0; r < 8; r++) {
    ((mode & 1) ? fs : fc)(x + 8 * r, out);
    memcpy(tmp + 8 * r, out, sizeof(out));
  }
  for (int c = 0; c < 8; c++) {
    for (int r = 0; r < 8; r++) line[r] = tmp[8 * r + c];
    ((mode & 2) ? fs : fc)(line, out);
    for (int r = 0; r < 8; r++) y[8 * r + c] = out[r];
  }
}

static void mat8(const double m[8][8], const double *x, double *y) {
  for (int i = 0; i < 8; i++) {
    y[i] = 0.0;
    for (int j = 0; j < 8; j++) y[i] += m[i][j] * x[j];
  }
}

void or_dctiv_direct(const double *x, double *y) { tables(); mat8(CIV, x, y); }

/* generic two-pass separable transform with transposed store (dttt_* pattern) */
static void dttt_generic(const double *x, double *y, int mode,
                         void (*fc)(const double *, double *), void (*fs)(const double *, double *)) {
  double line[8], out[8], tmp[64];
  for (int i = 0; i < 8; i++) {
    memcpy(line, x + 8 * i, sizeof(line));
    ((mode & 1) ? fs : fc)(line, out);
    for (int j = 0; j < 8; j++) tmp[j * 8 + i] = out[j];
  }
  for (int i = 0; i < 8; i++) {
    memcpy(line, tmp + 8 * i, sizeof(line));
    ((mode & 2) ? fs : fc)(line, out);
    memcpy(y + 8 * i, out, sizeof(out));
  }
}
static void dctiie_direct(const double *x, double *y) { mat8(CIIe, x, y); }
static void dstiie_direct(const double *x, double *y) { mat8(SIIe, x, y); }
static void dctiiie_direct(const double *x, double *y) { mat8(CIIIe, x, y); }
static void dstiiie_direct(const double *x, double *y) { mat8(SIIIe, x, y); }

void or_dttt_iv(const double *x, double *y, int mode) { tables(); dttt_generic(x, y, mode, or_dct_iv8, or_dst_iv8); }
void or_dttt_iie(const double *x, double *y, int mode) { tables(); dttt_generic(x, y, mode, dctiie_direct, dstiie_direct); }
void or_dttt_iiie(const double *x, double *y, int mode) { tables(); dttt_generic(x, y, mode, dctiiie_direct, dstiiie_direct); }

void or_hwindow(double *hw8) { tables(); memcpy(hw8, HWINDOW, sizeof(HWINDOW)); }
void or_fold_index(int fi[64][4]) { tables(); memcpy(fi, FOLD_INDEX, sizeof(FOLD_INDEX)); }

/* DttRad2.get_shifted_fold_2d (263-314) */
void or_shifted_fold(double shift_hor, double shift_vert, double fold_sk[4][64][4]) {
  tables();
  const int n = 8, n2 = 16;
  double ahc = cos(M_PI / n2 * shift_hor);
  double ahs = sin(M_PI / n2 * shift_hor);
  double avc = cos(M_PI / n2 * shift_vert);
  double avs = sin(M_PI / n2 * shift_vert);
  for (int i = 0; i < n; i++) {
    int fi[2][6];
    fold_indices(i, n, fi);
    double vw0 = avc * HWINDOW[fi[0][1]] + avs * HWINDOW[fi[0][4]] * fi[0][5];
    double vw1 = avc * HWINDOW[fi[1][1]] + avs * HWINDOW[fi[1][4]] * fi[1][5];
    double vert_k[2][2] = {{fi[0][2] * vw0, fi[1][2] * vw1}, {fi[0][3] * vw0, fi[1][3] * vw1}};
    for (int j = 0; j < n; j++) {
      int fj[2][6];
      fold_indices(j, n, fj);
      double hw0 = ahc * HWINDOW[fj[0][1]] + ahs * HWINDOW[fj[0][4]] * fj[0][5];
      double hw1 = ahc * HWINDOW[fj[1][1]] + ahs * HWINDOW[fj[1][4]] * fj[1][5];
      double hor_k[2][2] = {{fj[0][2] * hw0, fj[1][2] * hw1}, {fj[0][3] * hw0, fj[1][3] * hw1}};
      int indx = n * i + j;
      for (int mode = 0; mode < 4; mode++)
        for (int k = 0; k < 4; k++)
          fold_sk[mode][indx][k] = vert_k[(mode >> 1) & 1][(k >> 1) & 1] * hor_k[mode & 1][k & 1];
    }
  }
}

/* DttRad2.fold_tile (724-738) */
void or_fold_tile(const double *x, int mode, const double fold_k[4][64][4], double *y) {
  tables();
  for (int i = 0; i < 64; i++) {
    y[i] = 0;
    for (int k = 0; k < 4; k++) y[i] += x[FOLD_INDEX[i][k]] * fold_k[mode][i][k];
  }
}

/* DttRad2.unfold_tile (770-780) */
void or_unfold_tile(const double *x, int mode, double *y) {
  tables();
  for (int i = 0; i < 256; i++) y[i] = UNFOLD_K[mode][i] * x[UNFOLD_INDEX[i]];
}

/* DttRad2.corr_unfold_tile (443-489) */
void or_corr_unfold_tile(const double q[4][64], double *rslt) {
  const int ts = 8, cs = 15;
  const double sc = 0.25;
  rslt[cs * ts - ts] = sc * q[0][0];
  for (int j = 1; j < ts; j++) {
    rslt[cs * ts - ts + j] = sc * (q[0][j] + q[1][j - 1]);
    rslt[cs * ts - ts - j] = sc * (q[0][j] - q[1][j - 1]);
  }
  for (int i = 1; i < ts; i++) {
    rslt[cs * (ts + i) - ts] = sc * (q[0][i * ts] + q[2][(i - 1) * ts]);
    rslt[cs * (ts - i) - ts] = sc * (q[0][i * ts] - q[2][(i - 1) * ts]);
    for (int j = 1; j < ts; j++) {
      double a = q[0][i * ts + j], b = q[1][i * ts + j - 1], c = q[2][(i - 1) * ts + j], d = q[3][(i - 1) * ts + j - 1];
      rslt[cs * (ts + i) - ts + j] = sc * (a + b + c + d);
      rslt[cs * (ts + i) - ts - j] = sc * (a + -b + c + -d);
      rslt[cs * (ts - i) - ts + j] = sc * (a + b + -c + -d);
      rslt[cs * (ts - i) - ts - j] = sc * (a + -b + -c + d);
    }
  }
}

/* DttRad2.getWin2d (697-713) */
void or_win2d(double *rslt) {
  tables();
  const int size = 8, size2 = 16;
  for (int i = 0; i < size; i++) {
    int ia0 = i * size2, ia1 = (size2 - i - 1) * size2;
    for (int j = 0; j < size; j++) {
      double d = HWINDOW[i] * HWINDOW[j];
      rslt[ia0 + j] = d; rslt[ia1 + j] = d;
      rslt[ia0 + size2 - j - 1] = d; rslt[ia1 + size2 - j - 1] = d;
    }
  }
}

/* ------------------------------------------------------------------------- */
/* ImageDtt stage 2 (J/tileprocessor/ImageDtt.java)                           */
/* ------------------------------------------------------------------------- */

/* java.lang.Math.round(double): round half up, exact */
static long java_round(double x) {
  double f = floor(x);
  return (long)((x - f >= 0.5) ? f + 1.0 : f);
}

/* ImageDtt.convolve_tile (5429-5488) */
void or_convolve_tile(double data[4][64], const double *kernel) {
  static const int zi[4][4] = {{0, -1, -2, 3}, {1, 0, -3, -2}, {2, -3, 0, -1}, {3, 2, 1, 0}};
  double rslt[4][64];
  for (int i = 0; i < 64; i++)
    for (int n = 0; n < 4; n++) {
      rslt[n][i] = 0;
      for (int k = 0; k < 4; k++) {
        if (zi[n][k] < 0) rslt[n][i] -= data[-zi[n][k]][i] * kernel[k * 64 + i];
        else rslt[n][i] += data[zi[n][k]][i] * kernel[k * 64 + i];
      }
    }
  memcpy(data, rslt, sizeof(rslt));
}

/* ImageDtt.fract_shift (5490-5584) */
void or_fract_shift(double clt[4][64], double shiftX, double shiftY) {
  const int ts = 8;
  double cos_hor[64], sin_hor[64], cos_vert[64], sin_vert[64];
  for (int i = 0; i < ts; i++) {
    double ch = cos((i + 0.5) * M_PI * shiftX / ts);
    double sh = sin((i + 0.5) * M_PI * shiftX / ts);
    double cv = cos((i + 0.5) * M_PI * shiftY / ts);
    double sv = sin((i + 0.5) * M_PI * shiftY / ts);
    for (int j = 0; j < ts; j++) {
      int iv = ts * j + i, ih = ts * i + j;
      cos_hor[ih] = ch; sin_hor[ih] = sh;
      cos_vert[iv] = cv; sin_vert[iv] = sv;
    }
  }
  double t[4][64];
  for (int i = 0; i < 64; i++) {
    t[0][i] = clt[0][i] * cos_hor[i] - clt[1][i] * sin_hor[i];
    t[1][i] = clt[1][i] * cos_hor[i] + clt[0][i] * sin_hor[i];
    t[2][i] = clt[2][i] * cos_hor[i] - clt[3][i] * sin_hor[i];
    t[3][i] = clt[3][i] * cos_hor[i] + clt[2][i] * sin_hor[i];
  }
  for (int i = 0; i < 64; i++) {
    clt[0][i] = t[0][i] * cos_vert[i] - t[2][i] * sin_vert[i];
    clt[2][i] = t[2][i] * cos_vert[i] + t[0][i] * sin_vert[i];
    clt[1][i] = t[1][i] * cos_vert[i] - t[3][i] * sin_vert[i];
    clt[3][i] = t[3][i] * cos_vert[i] + t[1][i] * sin_vert[i];
  }
}

/* ImageDtt.extract_correct_tile (4867-5426), non-debug branch */
void or_extract_correct_tile(const double *image, int width, int height,
                             const double *kern, const double *kext,
                             int kh, int kv, int kernel_step,
                             double centerX, double centerY,
                             double clt[4][64], double residual[2], int int_tl[2], int ktile[2]) {
  tables();
  const int ts = 8, ts2 = 16;
  int use_kernels = (kern != NULL);
  double px = centerX - ts, py = centerY - ts;
  int ktileX = 0, ktileY = 0;
  if (use_kernels) {
    ktileX = (int)java_round(centerX / kernel_step) + 1;
    ktileY = (int)java_round(centerY / kernel_step) + 1;
    if (ktileY < 0) ktileY = 0; else if (ktileY >= kv) ktileY = kv - 1;
    if (ktileX < 0) ktileX = 0; else if (ktileX >= kh) ktileX = kh - 1;
    const double *ce = kext + ((size_t)ktileY * kh + ktileX) * 8;
    double kdx = centerX - (ktileX - 1 + 0.5) * kernel_step;
    double kdy = centerY - (ktileY - 1 + 0.5) * kernel_step;
    px = centerX - ts - (ce[0] + ce[4] * kdx + ce[5] * kdy);
    py = centerY - ts - (ce[1] + ce[6] * kdx + ce[7] * kdy);
  }
  int ctile_left = (int)-java_round(-px);
  int ctile_top = (int)-java_round(-py);
  residual[0] = -(px - ctile_left);
  residual[1] = -(py - ctile_top);
  if (int_tl) { int_tl[0] = ctile_left; int_tl[1] = ctile_top; }
  if (ktile) { ktile[0] = ktileX; ktile[1] = ktileY; }
  double tile_in[256];
  for (int i = 0; i < ts2; i++) {
    int pi = ctile_top + i;
    if (pi < 0) pi &= 1;
    else if (pi >= height) pi = height - 2 + (pi & 1);
    for (int j = 0; j < ts2; j++) {
      int pj = ctile_left + j;
      if (pj < 0) pj &= 1;
      else if (pj >= width) pj = width - 2 + (pj & 1);
      tile_in[ts2 * i + j] = image[(size_t)pi * width + pj];
    }
  }
  double fold_coeff[4][64][4];
  or_shifted_fold(residual[0], residual[1], fold_coeff);
  for (int mode = 0; mode < 4; mode++) {
    double folded[64];
    or_fold_tile(tile_in, mode, fold_coeff, folded);
    or_dttt_iv(folded, clt[mode], mode);
  }
  if (use_kernels) or_convolve_tile(clt, kern + ((size_t)ktileY * kh + ktileX) * 256);
}

/* correlation LPF filter, ImageDtt.clt_aberrations_quad_corr_new (1662-1690) */
void or_corr_lpf(double corr_sigma, double *filter) {
  tables();
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
  or_dttt_iiie(fd, filter, 0);
  for (int i = 0; i < 64; i++) filter[i] *= 2 * ts;
}

/* GPUTileProcessor.setCltLpf (814-848) + setLpfRbg scaling (780-812) */
void or_clt_lpf(double sigma, double *lpf) {
  tables();
  const int ts = 8;
  double l[64];
  if (sigma == 0.0) {
    l[0] = 1.0;
    for (int i = 1; i < 64; i++) l[i] = 0.0;
  } else {
    for (int i = 0; i < ts; i++)
      for (int j = 0; j < ts; j++) l[i * ts + j] = (double)(float)exp(-(i * i + j * j) / (2 * sigma));
    double sum = 0;
    for (int i = 0; i < ts; i++)
      for (int j = 0; j < ts; j++) {
        double d = l[i * ts + j];
        d *= cos(M_PI * i / (2 * ts)) * cos(M_PI * j / (2 * ts));
        if (i > 0) d *= 2.0;
        if (j > 0) d *= 2.0;
        sum += d;
      }
    for (int i = 0; i < 64; i++) l[i] /= sum;
  }
  or_dttt_iiie(l, lpf, 0);
  for (int i = 0; i < 64; i++) lpf[i] = lpf[i] * 2 * ts;
}

/* ------------------------------------------------------------------------- */
/* GeometryCorrection (J/tileprocessor/GeometryCorrection.java)               */
/* ------------------------------------------------------------------------- */

static void mat3_mul(const double a[3][3], const double b[3][3], double c[3][3]) {
  /* Jama Matrix.times: c[i][j] = sum_k a[i][k]*b[k][j] accumulated in k order */
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0;
      for (int k = 0; k < 3; k++) s += a[i][k] * b[k][j];
      c[i][j] = s;
    }
}

/* CorrVector.getRotMatrices (1043-1076) with ROT_AZ_SGN=-1, ROT_TL_SGN=1, ROT_RL_SGN=1 */
void or_rot_matrices(const or_geometry *g, double rots[][3][3]) {
  for (int chn = 0; chn < g->num_sensors; chn++) {
    double ca = cos(g->azimuth[chn]), sa = sin(g->azimuth[chn]);
    double ct = cos(g->tilt[chn]), st = sin(g->tilt[chn]);
    double zoom = (1.0 + g->zoom[chn]);
    double cr = cos(g->roll[chn]) * zoom, sr = sin(g->roll[chn]) * zoom;
    double a_az[3][3] = {{ca, 0.0, sa * -1.0}, {0.0, 1.0, 0.0}, {-sa * -1.0, 0.0, ca}};
    double a_t[3][3] = {{1.0, 0.0, 0.0}, {0.0, ct, st * 1.0}, {0.0, -st * 1.0, ct}};
    double a_r[3][3] = {{cr, sr * 1.0, 0.0}, {-sr * 1.0, cr, 0.0}, {0.0, 0.0, 1.0}};
    double tmp[3][3];
    mat3_mul(a_t, a_az, tmp);
    mat3_mul(a_r, tmp, rots[chn]);
  }
}

/* CorrVector.getRotDeriveMatrices (1083-1147): [chn][0 az, 1 tilt, 2 roll, 3 zoom] */
void or_rot_deriv_matrices(const or_geometry *g, double d[][4][3][3]) {
  for (int chn = 0; chn < g->num_sensors; chn++) {
    double ca = cos(g->azimuth[chn]), sa = sin(g->azimuth[chn]);
    double ct = cos(g->tilt[chn]), st = sin(g->tilt[chn]);
    double zoom = (1.0 + g->zoom[chn]);
    double cr = cos(g->roll[chn]), sr = sin(g->roll[chn]);
    double a_az[3][3] = {{ca, 0.0, sa * -1.0}, {0.0, 1.0, 0.0}, {-sa * -1.0, 0.0, ca}};
    double a_t[3][3] = {{1.0, 0.0, 0.0}, {0.0, ct, st * 1.0}, {0.0, -st * 1.0, ct}};
    double a_r[3][3] = {{cr * zoom, sr * zoom * 1.0, 0.0}, {-sr * zoom * 1.0, cr * zoom, 0.0}, {0.0, 0.0, 1.0}};
    double a_daz[3][3] = {{-sa, 0.0, ca * -1.0}, {0.0, 0.0, 0.0}, {-ca * -1.0, 0.0, -sa}};
    double a_dt[3][3] = {{0.0, 0.0, 0.0}, {0.0, -st, ct * 1.0}, {0.0, -ct * 1.0, -st}};
    double a_dr[3][3] = {{-sr * zoom, cr * zoom * 1.0, 0.0}, {-cr * zoom * 1.0, -sr * zoom, 0.0}, {0.0, 0.0, 0.0}};
    double a_dzoom[3][3] = {{cr, sr * 1.0, 0.0}, {-sr * 1.0, cr, 0.0}, {0.0, 0.0, 0.0}};
    double tmp[3][3];
    mat3_mul(a_t, a_daz, tmp); mat3_mul(a_r, tmp, d[chn][0]);
    mat3_mul(a_dt, a_az, tmp); mat3_mul(a_r, tmp, d[chn][1]);
    mat3_mul(a_t, a_az, tmp); mat3_mul(a_dr, tmp, d[chn][2]);
    mat3_mul(a_t, a_az, tmp); mat3_mul(a_dzoom, tmp, d[chn][3]);
  }
}

/* calcReverseDistortionTable (2707-2757): stepR=0.001, maxR=2.0 */
int or_reverse_distortion_table(const or_geometry *g, double *tbl, int cap) {
  const double delta = 1E-8, minDerivative = 0.1, stepR = 0.001, maxR = 2.0;
  const int numIterations = 1000;
  double drDistDr = 1.0;
  double A8 = g->distortion[6], A7 = g->distortion[5], A6 = g->distortion[4], A5 = g->distortion[3];
  double A = g->distortion[2], B = g->distortion[1], C = g->distortion[0];
  int use8 = (A8 != 0.0) || (A7 != 0.0) || (A6 != 0.0);
  double d = 1.0 - A8 - A7 - A6 - A5 - A - B - C;
  double rPrev = 0.0;
  int len = (int)ceil(maxR / stepR) + 1;
  if (len > cap) return -1;
  for (int j = 1; j < len; j++) tbl[j] = NAN;
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
      if (drDistDr < minDerivative) return len; /* bail out: rest stays NaN */
      if (fabs(rD - rDist) < delta) break;
      r += (rDist - rD) / drDistDr;
    }
    rPrev = r;
    tbl[i] = r / rDist;
  }
  return len;
}

/* getRByRDist (2802-2827) */
double or_r_by_rdist(const double *tbl, int len, double rDist) {
  const double stepR = 0.001;
  if (rDist < 0) return NAN;
  int index = (int)floor(rDist / stepR);
  if (index >= (len - 1)) return NAN;
  return tbl[index] + (tbl[index + 1] - tbl[index]) * (rDist / stepR - index);
}

static void mat3_vec(const double m[3][3], const double v[3], double r[3]) {
  for (int i = 0; i < 3; i++) {
    double s = 0;
    for (int k = 0; k < 3; k++) s += m[i][k] * v[k];
    r[i] = s;
  }
}

/* getPortsCoordinatesAndDerivatives (2159-2314), main camera (gc_main == this, no rig) */
/* getPortsCoordinatesAndDerivatives with the tile centre undistorted by the model gc (the
 * reference's gc_main argument, 2179-2185) and everything after by g */
static void ports_core(const or_geometry *gc, const double *tblc, int tblc_len, const or_geometry *g,
                       const double rots[][3][3], const double drots[][4][3][3], double px, double py,
                       double disparity, double pXY[][2], double deriv[][2][4]) {
  double pXcd = px - 0.5 * gc->pixel_width;
  double pYcd = py - 0.5 * gc->pixel_height;
  double rD = sqrt(pXcd * pXcd + pYcd * pYcd) * 0.001 * gc->pixel_size;
  double rND2R = or_r_by_rdist(tblc, tblc_len, rD / gc->distortion_radius);
  double pXc = pXcd * rND2R;
  double pYc = pYcd * rND2R;
  const double *rad_coeff = g->distortion; /* C, B, A, A5, A6, A7, A8 */
  double fl_pix = g->focal_length / (0.001 * g->pixel_size);
  double ri_scale = 0.001 * g->pixel_size / g->distortion_radius;
  for (int i = 0; i < g->num_sensors; i++) {
    double pXci0 = pXc - disparity * g->rXY[i][0];
    double pYci0 = pYc - disparity * g->rXY[i][1];
    double vi[3] = {pXci0, pYci0, fl_pix};
    double rvi[3];
    mat3_vec(rots[i], vi, rvi);
    double norm_z = fl_pix / rvi[2];
    double pXci = rvi[0] * norm_z;
    double pYci = rvi[1] * norm_z;
    double rNDi = sqrt(pXci * pXci + pYci * pYci);
    double ri = rNDi * ri_scale;
    double rD2rND = 1.0, rri = 1.0;
    for (int j = 0; j < 7; j++) {
      rri *= ri;
      rD2rND += rad_coeff[j] * (rri - 1.0);
    }
    double pXid = pXci * rD2rND;
    double pYid = pYci * rD2rND;
    pXY[i][0] = pXid + g->pXY0[i][0];
    pXY[i][1] = pYid + g->pXY0[i][1];
    if (deriv) {
      double dr[4][3];
      for (int k = 0; k < 4; k++) mat3_vec(drots[i][k], vi, dr[k]);
      double dpX[4], dpY[4];
      for (int k = 0; k < 4; k++) { /* az, tilt, roll, zoom */
        dpX[k] = dr[k][0] * norm_z - pXci * dr[k][2] / rvi[2];
        dpY[k] = dr[k][1] * norm_z - pYci * dr[k][2] / rvi[2];
      }
      double drD2rND_dri = 0.0;
      rri = 1.0;
      for (int j = 0; j < 7; j++) {
        drD2rND_dri += rad_coeff[j] * (j + 1) * rri;
        rri *= ri;
      }
      for (int k = 0; k < 4; k++) {
        if (k == 2) { /* roll: reference drops the radial term (2279-2280) */
          deriv[i][0][k] = dpX[k] * rD2rND;
          deriv[i][1][k] = dpY[k] * rD2rND;
        } else {
          double dri = ri_scale / rNDi * (pXci * dpX[k] + pYci * dpY[k]);
          double drD = drD2rND_dri * dri;
          deriv[i][0][k] = dpX[k] * rD2rND + pXci * drD;
          deriv[i][1][k] = dpY[k] * rD2rND + pYci * drD;
        }
      }
    }
  }
}

void or_ports(const or_geometry *g, const double rots[][3][3], const double drots[][4][3][3],
              const double *tbl, int tbl_len, double px, double py, double disparity,
              double pXY[][2], double deriv[][2][4]) {
  ports_core(g, tbl, tbl_len, g, rots, drots, px, py, disparity, pXY, deriv);
}

/* RigOffset.getRotMatrix (GeometryCorrection.java:770-800): aux roll (with zoom) x tilt x azimuth */
void or_rig_matrix(const or_rig_offset *rig, double m[3][3]) {
  const double ca = cos(rig->aux_azimuth), sa = sin(rig->aux_azimuth);
  const double ct = cos(rig->aux_tilt), st = sin(rig->aux_tilt);
  const double zoom = 1.0 + rig->aux_zoom;
  const double cr = cos(rig->aux_roll) * zoom, sr = sin(rig->aux_roll) * zoom;
  const double AZ = -1.0, TL = 1.0, RL = 1.0; /* ROT_AZ_SGN, ROT_TL_SGN, ROT_RL_SGN */
  const double a_az[3][3] = {{ca, 0.0, sa * AZ}, {0.0, 1.0, 0.0}, {-sa * AZ, 0.0, ca}};
  const double a_t[3][3] = {{1.0, 0.0, 0.0}, {0.0, ct, st * TL}, {0.0, -st * TL, ct}};
  const double a_r[3][3] = {{cr, sr * RL, 0.0}, {-sr * RL, cr, 0.0}, {0.0, 0.0, 1.0}};
  double t[3][3];
  mat3_mul(a_t, a_az, t);
  mat3_mul(a_r, t, m);
}

/* RigOffset.recalcRXY (728-747): per-sensor lens offsets of the auxiliary camera in its own
 * disparity units: the baseline offset plus the rXY rotated by the aux roll */
void or_rig_rxy(const or_geometry *aux, const or_rig_offset *rig, double rxy[][2]) {
  const double xc_pix = rig->baseline * cos(rig->aux_angle) / rig->aux_disparity_radius;
  const double yc_pix = rig->baseline * sin(rig->aux_angle) / rig->aux_disparity_radius;
  const double ssr = 1.0;
  for (int i = 0; i < aux->num_sensors; i++) {
    rxy[i][0] = xc_pix + cos(rig->aux_roll) * aux->rXY[i][0] + ssr * sin(rig->aux_roll) * aux->rXY[i][1];
    rxy[i][1] = yc_pix - ssr * sin(rig->aux_roll) * aux->rXY[i][0] + cos(rig->aux_roll) * aux->rXY[i][1];
  }
}

void or_rig_aux_ports(const or_geometry *aux, const or_geometry *main_g, const or_rig_offset *rig, double px,
                      double py, double disparity_main, double pXY[][2]) {
  or_geometry g = *aux;
  or_rig_rxy(aux, rig, g.rXY);
  double rots[OR_MAX_SENSORS][3][3], rm[3][3];
  or_rot_matrices(aux, rots);
  or_rig_matrix(rig, rm);
  for (int i = 0; i < aux->num_sensors; i++) { /* CorrVector.getRotMatrices(rigMatrix) 1016-1025 */
    double t[3][3];
    mat3_mul(rots[i], rm, t);
    memcpy(rots[i], t, sizeof(t));
  }
  static double tbl[2100];
  const int tbl_len = or_reverse_distortion_table(main_g, tbl, 2100);
  const double disparity = disparity_main * rig->aux_disparity_radius / rig->main_disparity_radius;
  ports_core(main_g, tbl, tbl_len, &g, (const double(*)[3][3])rots, NULL, px, py, disparity, pXY, NULL);
}

/* ------------------------------------------------------------------------- */
/* Correlation2d (J/tileprocessor/Correlation2d.java)                         */
/* ------------------------------------------------------------------------- */

void or_default_corr_params(or_corr_params *p) {
  /* ImageDttParameters.java:30-112 defaults, fat_zero/corr_sigma per config */
  p->fat_zero = 0.05;
  p->corr_sigma = 0.8;       /* CLTParameters.corr_sigma default */
  p->corr_red = 0.5;
  p->corr_blue = 0.2;
  p->corr_offset = 0.1;
  p->min_corr = 0.02;
  p->corr_strip_hight = 9;
  p->twice_diagonal = 1;
  p->enhortho_width = 2;
  p->enhortho_scale = 0.0;
  p->corr_wndy_size = 2; p->corr_wndy_hwidth = 1.0; p->corr_wndy_blur = 1.0;
  p->corr_wndx_size = 9; p->corr_wndx_hwidth = 6.0; p->corr_wndx_blur = 5.0;
}

void or_quad_pairs(or_pairs *pp) {
  /* PAIRS[0..5] (Correlation2d.java:52-58) */
  static const int c1[6] = {0, 2, 0, 1, 0, 2}, c2[6] = {1, 3, 2, 3, 3, 1}, kind[6] = {0, 0, 1, 1, 2, 3};
  static const double bx[6] = {1, 1, 0, 0, 1, 1}, by[6] = {0, 0, 1, 1, 1, -1};
  memset(pp, 0, sizeof(*pp));
  pp->num_pairs = 6;
  for (int i = 0; i < 6; i++) {
    pp->cam1[i] = c1[i]; pp->cam2[i] = c2[i]; pp->kind[i] = kind[i];
    pp->bx[i] = bx[i]; pp->by[i] = by[i];
  }
  pp->combo_mask_lo = 0x3f;
  pp->combo_mask_hi = 0;
}

/* correlateSingleColorFD (197-231) */
static void correlate_single(const double *d1, const double *d2, double fat_zero, double t[4][64]) {
  static const int ZI[4][4] = {{0, 1, 2, 3}, {-1, 0, -3, 2}, {-2, -3, 0, 1}, {3, -2, -1, 0}};
  double a2[64], sa2 = 0.0;
  for (int i = 0; i < 64; i++) {
    double s1 = 0.0, s2 = 0.0;
    for (int n = 0; n < 4; n++) {
      s1 += d1[n * 64 + i] * d1[n * 64 + i];
      s2 += d2[n * 64 + i] * d2[n * 64 + i];
    }
    a2[i] = sqrt(s1 * s2);
    sa2 += a2[i];
  }
  double fz2 = sa2 / 64 * fat_zero * fat_zero;
  for (int i = 0; i < 64; i++) {
    double scale = 1.0 / (a2[i] + fz2);
    for (int n = 0; n < 4; n++) {
      t[n][i] = 0;
      for (int k = 0; k < 4; k++) {
        if (ZI[n][k] < 0) t[n][i] -= d1[(-ZI[n][k]) * 64 + i] * d2[k * 64 + i];
        else t[n][i] += d1[ZI[n][k] * 64 + i] * d2[k * 64 + i];
      }
      t[n][i] *= scale;
    }
  }
}

/* correlateCompositeFD (275-328) */
void or_correlate_pair(const double *clt1, const double *clt2, int nc, const double *col_weights,
                       const double *lpf, double fat_zero, double *corr) {
  double one = 1.0;
  if (nc == 1) col_weights = &one;
  double acc[4][64], t[4][64];
  for (int col = 0; col < nc; col++) {
    correlate_single(clt1 + col * 256, clt2 + col * 256, fat_zero, t);
    for (int n = 0; n < 4; n++)
      for (int i = 0; i < 64; i++) {
        if (col == 0) acc[n][i] = t[n][i] * col_weights[col];
        else acc[n][i] += t[n][i] * col_weights[col];
      }
  }
  if (lpf)
    for (int n = 0; n < 4; n++)
      for (int i = 0; i < 64; i++) acc[n][i] *= lpf[i];
  double q[4][64];
  for (int quadrant = 0; quadrant < 4; quadrant++) {
    int mode = ((quadrant << 1) & 2) | ((quadrant >> 1) & 1);
    or_dttt_iie(acc[quadrant], q[quadrant], mode);
  }
  or_corr_unfold_tile(q, corr);
}

static double corr_at(const double *c, int iy, int ix) { return c[iy * 15 + ix]; }

/*
 * scaleRotateInterpoateSingleCorrelation (610-718) for kinds 0..3 with ss=1
 * (exact restatement); kind 4 is the documented generalisation to an
 * arbitrary baseline b: strip(row,col) samples the correlation at
 * (col + (row&1)/2) * b +/- (row/2) * b_perp (b_perp = b rotated 90 deg),
 * bilinearly interpolated, NaN outside the 15x15 support.  For b along the
 * four quad directions the kind-4 sampler visits the same points.
 */
void or_strip(const double *corr, double bx, double by, int kind, int hwidth, double *strip) {
  const int center = 7, width = 15;
  for (int i = 0; i < hwidth * width; i++) strip[i] = 0.0;
  if (kind <= 3) {
    int dir = kind, ss = 1;
    int denom = ss * ((dir > 1) ? 1 : 2);
    double rdenom = denom;
    int ilimit = center * denom;
    int xnum = 0, ynum = 0;
    for (int row = 0; row < hwidth; row++)
      for (int scol = -center; scol <= center; scol++) {
        int indx = row * width + scol + center;
        for (int down = -1; down < ((row == 0) ? 0 : 2); down += 2) {
          switch (dir) {
            case 0: xnum = 2 * scol + (row & 1); ynum = down * row; break;
            case 1: xnum = down * row; ynum = 2 * scol + (row & 1); break;
            case 2: xnum = scol - ((down * row) >> 1); ynum = scol + ((down * row + 1) >> 1); break;
            default: xnum = scol - ((down * row) >> 1); ynum = -scol - ((down * row + 1) >> 1); break;
          }
          if ((xnum > ilimit) || (xnum < -ilimit) || (ynum > ilimit) || (ynum < -ilimit)) {
            strip[indx] = NAN;
          } else {
            int ix0 = (xnum + ilimit) / denom, iy0 = (ynum + ilimit) / denom;
            int int_x = (xnum % denom) == 0, int_y = (ynum % denom) == 0;
            double d;
            if (int_x && int_y) {
              d = corr_at(corr, iy0, ix0);
            } else {
              double dx = (xnum + ilimit) / rdenom - ix0;
              double dy = (ynum + ilimit) / rdenom - iy0;
              if (int_y) d = (1.0 - dx) * corr_at(corr, iy0, ix0) + dx * corr_at(corr, iy0, ix0 + 1);
              else if (int_x) d = (1.0 - dy) * corr_at(corr, iy0, ix0) + dy * corr_at(corr, iy0 + 1, ix0);
              else
                d = ((1.0 - dx) * (1.0 - dy) * corr_at(corr, iy0, ix0)) + (dx * (1.0 - dy) * corr_at(corr, iy0, ix0 + 1)) +
                    ((1.0 - dx) * dy * corr_at(corr, iy0 + 1, ix0)) + (dx * dy * corr_at(corr, iy0 + 1, ix0 + 1));
            }
            if (row == 0) strip[indx] = d;
            else strip[indx] += 0.5 * d;
          }
        }
      }
    return;
  }
  /* kind 4: general baseline */
  for (int row = 0; row < hwidth; row++)
    for (int scol = -center; scol <= center; scol++) {
      int indx = row * width + scol + center;
      for (int down = -1; down < ((row == 0) ? 0 : 2); down += 2) {
        double a = scol + 0.5 * (row & 1), p = 0.5 * down * row;
        double x = a * bx - p * by, y = a * by + p * bx;
        if ((x > center) || (x < -center) || (y > center) || (y < -center)) {
          strip[indx] = NAN;
          continue;
        }
        double fx = x + center, fy = y + center;
        int ix0 = (int)floor(fx), iy0 = (int)floor(fy);
        if (ix0 > 2 * center - 1) ix0 = 2 * center - 1;
        if (iy0 > 2 * center - 1) iy0 = 2 * center - 1;
        double dx = fx - ix0, dy = fy - iy0;
        double d = ((1.0 - dx) * (1.0 - dy) * corr_at(corr, iy0, ix0)) + (dx * (1.0 - dy) * corr_at(corr, iy0, ix0 + 1)) +
                   ((1.0 - dx) * dy * corr_at(corr, iy0 + 1, ix0)) + (dx * dy * corr_at(corr, iy0 + 1, ix0 + 1));
        if (row == 0) strip[indx] = d;
        else strip[indx] += 0.5 * d;
      }
    }
}

/* combineInterpolatedCorrelations (730-790) */
void or_combine_strips(const double *strips, const int *use, int np, const int *is_diag, int hwidth,
                       double offset, int twice_diagonal, double *combo) {
  int len = hwidth * 15, ncombined = 0, have = 0;
  if (offset >= 0) {
    for (int p = 0; p < np; p++) {
      if (!use[p]) continue;
      const double *s = strips + (size_t)p * len;
      if (!have) { for (int i = 0; i < len; i++) combo[i] = 1.0; have = 1; }
      /* the reference squares every selected pair when twice_diagonal is set (759-765) */
      if (twice_diagonal) {
        for (int i = 0; i < len; i++) { double d = s[i] + offset; if (d < 0.0) d = 0.0; combo[i] *= d * d; }
        ncombined++;
      } else {
        for (int i = 0; i < len; i++) { double d = s[i] + offset; if (d < 0.0) d = 0.0; combo[i] *= d; }
      }
      ncombined++;
    }
    double pwr = 1.0 / ncombined;
    if (have)
      for (int i = 0; i < len; i++) if (combo[i] > 0.0) combo[i] = pow(combo[i], pwr) - offset;
  } else {
    for (int p = 0; p < np; p++) {
      if (!use[p]) continue;
      const double *s = strips + (size_t)p * len;
      if (!have) { for (int i = 0; i < len; i++) combo[i] = 0.0; have = 1; }
      if (twice_diagonal) { for (int i = 0; i < len; i++) combo[i] += 2 * s[i]; ncombined++; }
      else { for (int i = 0; i < len; i++) combo[i] += s[i]; }
      ncombined++;
    }
    double scale = 1.0 / ncombined;
    for (int i = 0; i < len; i++) combo[i] *= scale;
  }
}

/* getMaxXYInt (802-843), strip form => axis_only on row 0 */
int or_max_xy_int_axis(const double *data, int hwidth, double minMax, int *ix) {
  (void)hwidth;
  int imx = 0;
  for (int i = 1; i < 15; i++)
    if (isnan(data[imx]) || (data[i] > data[imx])) imx = i;
  if (!(data[imx] >= minMax)) return 0;
  *ix = imx % 15 - 7;
  return 1;
}

/* halfFlatTopWindow (1047-1081) */
void or_half_flat_top_window(int ihwidth, double hwidth, double blur, int normalize, int notch,
                             double scale, double *wnd) {
  for (int i = 0; i < ihwidth; i++) {
    if (blur <= 0.0) wnd[i] = (i < hwidth) ? 1.0 : 0.0;
    else {
      if (i < hwidth - blur / 2) wnd[i] = 1.0;
      else if (i > hwidth + blur / 2) wnd[i] = 0.0;
      else wnd[i] = 0.5 * (1.0 - sin(M_PI * (i - hwidth) / blur));
    }
    if (notch) wnd[i] = 1.0 - wnd[i];
  }
  if (normalize) {
    double s = 0.0;
    for (int i = 0; i < ihwidth; i++) s += ((i == 0) ? 1.0 : 2.0) * wnd[i];
    s = 1 / s;
    for (int i = 0; i < ihwidth; i++) wnd[i] *= s;
  }
  for (int i = 0; i < ihwidth; i++) wnd[i] *= scale;
}

/* getMaxXCm (936-1032) */
int or_max_x_cm(const double *data, int hwidth, int ixcenter, const double *window_y, int wy_len,
                const double *window_x, int wx_len, double rslt[3]) {
  const int center = 7, data_width = 15;
  int data_height = hwidth;
  double wy_scale = 1.0;
  if (data_height > wy_len) data_height = wy_len;
  else if (data_height < wy_len) {
    double swy = window_y[0];
    for (int i = 1; i < data_height; i++) swy += window_y[i];
    wy_scale = 1.0 / swy;
  }
  double s0 = 0.0, sx = 0.0, sx2 = 0.0;
  int x0 = center + ixcenter;
  for (int dy = 0; dy < data_height; dy++) {
    int odd = dy & 1;
    double wy = ((dy == 0) ? wy_scale : (2.0 * wy_scale)) * window_y[dy];
    int indx0 = data_width * dy;
    for (int adx = odd; adx < wx_len; adx += 2)
      for (int dir = (adx == 0) ? 1 : -1; dir <= 1; dir += 2) {
        int idx = (adx * dir) >> 1;
        int x = 2 * idx + odd;
        int x1 = x0 + idx;
        if ((x1 >= 0) && (x1 < data_width)) {
          double d = data[indx0 + x1];
          if (!isnan(d) && (d > 0.0)) {
            d *= wy * window_x[adx];
            s0 += d;
            sx += d * x;
            sx2 += d * x * x;
          }
        }
      }
  }
  if (s0 == 0.0) return 0;
  rslt[0] = ixcenter + sx / s0 / 2;
  rslt[1] = s0;
  rslt[2] = sqrt(s0 * sx2 - sx * sx) / s0 / 2;
  return 1;
}

/* createOrtoNotch (2654-2675) */
void or_ortho_notch(double enhortho_width, double enhortho_scale, double *notch) {
  const int ts = 8;
  for (int i = 0; i < 15; i++) {
    if ((i < (ts - enhortho_width)) || (i > (ts - 2 + enhortho_width))) notch[i] = 1.0;
    else notch[i] = enhortho_scale;
    if (i == (ts - 1)) notch[i] = 0.0;
    notch[i] *= sin(M_PI * (i + 1.0) / (2 * ts));
  }
}

/*
 * getMaxXSOrtho (2502-2651), symmetric=true, offset>=0 branch.  The 3-point
 * quadratic fit (PolynomialApproximation.polynomialApproximation1d, exact
 * interpolation through 3 points) is evaluated in closed form.
 */
/* the 15-entry profile c1d of getMaxXSOrtho (2502-2651): returns 0 when no pair is used */
int or_max_xs_ortho_profile(const double *corrs, const int *use, int np, double offset, int is_vert,
                            const double *notch, double c1d[15]) {
  const int cs = 15;
  int pairs[OR_MAX_PAIRS], n = 0;
  for (int p = 0; p < np; p++) if (use[p]) pairs[n++] = p;
  if (n == 0) return 0;
  double w = 1.0 / n;
  for (int j = 0; j < cs; j++) {
    c1d[j] = 0;
    for (int i = 0; i < cs; i++) {
      double combo = 1.0;
      for (int ip = 0; ip < n; ip++) {
        const double *c = corrs + (size_t)pairs[ip] * 225;
        double d;
        if (is_vert) d = (0.5 * (c[j * cs + i] + c[j * cs + (cs - i - 1)])) + offset;
        else d = (0.5 * (c[i * cs + j] + c[(cs - i - 1) * cs + j])) + offset;
        combo *= d;
      }
      if (combo > 0.0) combo = pow(combo, w) - offset;
      else combo = -offset;
      c1d[j] += combo * notch[i];
    }
  }
  return 1;
}

/* the sub-pixel maximum of a profile around the integer maximum icenter: {xcenter - 7, strength} */
void or_ortho_at(const double *c1d, int icenter, double rslt[2]) {
  const int cs = 15;
  double xcenter = icenter;
  if ((icenter > 0) && (icenter < (cs - 1))) {
    double f0 = c1d[icenter - 1], f1 = c1d[icenter], f2 = c1d[icenter + 1];
    double den = f0 - 2.0 * f1 + f2;
    if (den != 0.0) xcenter = icenter + 0.5 * (f0 - f2) / den;
  }
  icenter = (int)java_round(xcenter);
  if (icenter < 0) icenter = 0;
  if (icenter > cs - 1) icenter = cs - 1;
  rslt[0] = xcenter - 7;
  rslt[1] = c1d[icenter] / ((cs + 1) / 2);
}

int or_max_xs_ortho(const double *corrs, const int *use, int np, double offset, int is_vert,
                    const double *notch, double rslt[2]) {
  double c1d[15];
  if (!or_max_xs_ortho_profile(corrs, use, np, offset, is_vert, notch, c1d)) return 0;
  int icenter = 0;
  for (int i = 1; i < 15; i++) if (c1d[i] > c1d[icenter]) icenter = i;
  or_ortho_at(c1d, icenter, rslt);
  return 1;
}

/* getMaxXCm (936-1032) of a combined strip at the integer maximum ix, with the y / x windows of cp */
int or_cm_at(const or_corr_params *cp, const double *combo, int hw, int ix, double rslt[3]) {
  double wndy[32], wndx[32];
  or_half_flat_top_window(cp->corr_wndy_size, cp->corr_wndy_hwidth, cp->corr_wndy_blur, 1, 0, 1.0, wndy);
  or_half_flat_top_window(cp->corr_wndx_size, cp->corr_wndx_hwidth, cp->corr_wndx_blur, 1, 0, 2.0, wndx);
  return or_max_x_cm(combo, hw, ix, wndy, cp->corr_wndy_size, wndx, cp->corr_wndx_size, rslt);
}

/* ------------------------------------------------------------------------- */
/* IMCLT (ImageDtt.iclt_2d, 3559-3666) into the padded frame                  */
/* ------------------------------------------------------------------------- */
void or_iclt_tile_add(const double clt[4][64], double scale, int tx, int ty, double *frame, int fw) {
  for (int dct_mode = 0; dct_mode < 4; dct_mode++) {
    int idct_mode = ((dct_mode << 1) & 2) | ((dct_mode >> 1) & 1);
    double tile_dct[64], mdct[256];
    or_dttt_iv(clt[dct_mode], tile_dct, idct_mode);
    or_unfold_tile(tile_dct, dct_mode, mdct);
    for (int i = 0; i < 16; i++) {
      double *row = frame + (size_t)(ty * 8 + i) * fw + tx * 8;
      for (int j = 0; j < 16; j++) row[j] += scale * mdct[16 * i + j];
    }
  }
}

/* ------------------------------------------------------------------------- */
/* Texture tiles (ImageDtt.java:2662-2812, 2830-3147)                          */
/* ------------------------------------------------------------------------- */
static const double KERN_G[9] = {0.0, 0.125, 0.0, 0.125, 0.5, 0.125, 0.0, 0.125, 0.0};        /* ImageDtt.java:43-46 */
static const double KERN_RB[9] = {0.0625, 0.125, 0.0625, 0.125, 0.25, 0.125, 0.0625, 0.125, 0.0625}; /* 47-50 */
static const int CORN_SIDE_N[9] = {4, 6, 4, 6, 9, 6, 4, 6, 4};
static const int CORN_SIDE[9][9] = {                                                          /* 52-61 */
    {4, 5, 7, 8}, {3, 4, 5, 6, 7, 8}, {3, 4, 6, 7}, {1, 2, 4, 5, 7, 8}, {0, 1, 2, 3, 4, 5, 6, 7, 8},
    {0, 1, 3, 4, 6, 7}, {1, 2, 4, 5}, {0, 1, 2, 3, 4, 5}, {0, 1, 3, 4}};

/* tile_debayer (3047-3147) for a 16x16 tile */
static void tile_debayer(int rb, const double *tile, double *rslt) {
  const int ts = 16, tsm1 = 15;
  const int nb[9] = {-ts - 1, -ts, -ts + 1, -1, 0, 1, ts - 1, ts, ts + 1};
  const double *kern = rb ? KERN_RB : KERN_G;
  const double k_corn = rb ? (16.0 / 9.0) : (4.0 / 3.0), k_side = rb ? (4.0 / 3.0) : (8.0 / 7.0);
  for (int i = 0; i < 256; i++) rslt[i] = 0.0;
  for (int i = 0; i < ts; i++)
    for (int j = 0; j < ts; j++) {
      int rowt = (i == 0) ? 0 : ((i == tsm1) ? 2 : 1), colt = (j == 0) ? 0 : ((j == tsm1) ? 2 : 1);
      int type = rowt * 3 + colt, indx = i * ts + j;
      for (int k = 0; k < CORN_SIDE_N[type]; k++) {
        int dr = CORN_SIDE[type][k];
        rslt[indx] += tile[indx + nb[dr]] * kern[dr];
      }
      if (type != 4) rslt[indx] *= ((rowt != 1) && (colt != 1)) ? k_corn : k_side;
    }
}

/* tile_debayer_shot_corr (3022-3045) */
static void tile_debayer_shot_corr(int rb, const double *tile, const double *window2, double min_shot,
                                   double scale_shot, double *out) {
  double nw[256];
  for (int i = 0; i < 256; i++) nw[i] = tile[i] / window2[i];
  tile_debayer(rb, nw, out);
  if (scale_shot > 0) {
    double k = 1.0 / sqrt(min_shot);
    for (int i = 0; i < 256; i++) out[i] = scale_shot * ((out[i] > min_shot) ? sqrt(out[i]) : (k * out[i]));
  }
  for (int i = 0; i < 256; i++) out[i] = out[i] * window2[i];
}

/* relative margin below which a discrete choice of the texture stage counts as a near tie (the
 * test diagnostics flip such choices to measure their effect); set by or_texture_tile_diag */
static __thread double or_tex_near_tie = 1e-6;

/* dust_remove (3002-3019), port weights [4][256]; diag: the smallest relative margin of the
 * weakest-port choice (test diagnostics, may be NULL); flip: take the second weakest port where
 * the margin is a near tie (0 < margin < or_tex_near_tie) */
static void dust_remove(double pw[4][256], double *diag, int flip) {
  const int np = 4;
  for (int i = 0; i < 256; i++) {
    int wi = 0;
    for (int ip = 1; ip < np; ip++) if (pw[ip][i] < pw[wi][i]) wi = ip;
    if (diag || flip) {
      double mx = 0, next = INFINITY;
      int wn = -1;
      for (int ip = 0; ip < np; ip++) {
        if (pw[ip][i] > mx) mx = pw[ip][i];
        if (ip != wi && pw[ip][i] < next) { next = pw[ip][i]; wn = ip; }
      }
      const double m = mx > 0 ? (next - pw[wi][i]) / mx : INFINITY;
      if (diag && m < diag[1]) diag[1] = m;
      /* an exact tie comes from identical inputs, which FP32 resolves the same way */
      if (flip && m > 0 && m < or_tex_near_tie && wn >= 0) wi = wn;
    }
    double avg = 0;
    for (int ip = 1; ip < np; ip++) if (ip != wi) avg += pw[ip][i];
    avg /= (np - 1);
    double scale = 1.0 + (avg - pw[wi][i]) / (avg * (np - 1));
    for (int ip = 1; ip < np; ip++) if (ip != wi) pw[ip][i] *= scale;
    pw[wi][i] *= pw[wi][i] / avg;
  }
}

static const double PORT_OFFSETS[4][2] = {{-0.5, -0.5}, {0.5, -0.5}, {-0.5, 0.5}, {0.5, 0.5}};

/* tile_combine_rgba (2830-3000), keep_weights layout; iclt [4][3][256], window = lt_window2 */
/* diag (test diagnostics, may be NULL): [0] smallest relative margin over the pixels between the
 * second port of the best pair and the next one, [1] of dust_remove's weakest-port choice, [2]
 * smallest distance of a pixel's weight exponents from the double underflow of exp (745.13);
 * flip: where a margin is a near tie (0 < margin < or_tex_near_tie), take the other port (the
 * sensitivity of the output) */
static void tile_combine_rgba(double iclt[4][3][256], const double *lt_window, int port_mask, double diff_sigma,
                              const double *chn_weights, int dust, double *rgba /* [12][256] */, double *diag,
                              int flip) {
  const int ports = 4, numcol = 3;
  int usedPorts = ((port_mask >> 0) & 1) + ((port_mask >> 1) & 1) + ((port_mask >> 2) & 1) + ((port_mask >> 3) & 1);
  double pw[4][256], color_avg[3][256];
  memset(pw, 0, sizeof(pw));
  memset(color_avg, 0, sizeof(color_avg));
  const int rms_start = numcol + 1 + ports;
  for (int i = 0; i < 256; i++) {
    double sw = 0.0;
    for (int chn = 0; chn < numcol; chn++) {
      double s0 = 0, s1 = 0, s2 = 0;
      for (int ip = 0; ip < ports; ip++)
        if (port_mask & (1 << ip)) {
          s0 += 1;
          s1 += iclt[ip][chn][i];
          s2 += iclt[ip][chn][i] * iclt[ip][chn][i];
        }
      rgba[(rms_start + chn) * 256 + i] = sqrt(s0 * s2 - s1 * s1) / s0;
      sw += chn_weights[chn] * rgba[(rms_start + chn) * 256 + i] * rgba[(rms_start + chn) * 256 + i];
    }
    rgba[(rms_start + numcol) * 256 + i] = sqrt(sw);
  }
  if (usedPorts > 1) {
    double pair_dist2r[6];
    int pp[6][2], np = 0;
    double ksigma = 1.0 / (2.0 * diff_sigma * diff_sigma);
    for (int i = 0; i < ports; i++)
      if (port_mask & (1 << i))
        for (int j = i + 1; j < ports; j++)
          if (port_mask & (1 << j)) {
            double dx = PORT_OFFSETS[j][0] - PORT_OFFSETS[i][0], dy = PORT_OFFSETS[j][1] - PORT_OFFSETS[i][1];
            pp[np][0] = i; pp[np][1] = j;
            pair_dist2r[np++] = ksigma / (dx * dx + dy * dy);
          }
    for (int i = 0; i < 256; i++) {
      for (int ip = 0; ip < ports; ip++) pw[ip][i] = 0.0;
      double amin = INFINITY;
      for (int ip = 0; ip < np; ip++) {
        double d = 0;
        for (int chn = 0; chn < numcol; chn++) {
          double dc = iclt[pp[ip][0]][chn][i] - iclt[pp[ip][1]][chn][i];
          dc /= lt_window[i];
          d += chn_weights[chn] * dc * dc;
        }
        if (pair_dist2r[ip] * d < amin) amin = pair_dist2r[ip] * d;
        d = exp(-pair_dist2r[ip] * d);
        pw[pp[ip][0]][i] += d;
        pw[pp[ip][1]][i] += d;
      }
      int b1 = 0;
      for (int ip = b1 + 1; ip < ports; ip++) if (pw[ip][i] > pw[b1][i]) b1 = ip;
      int b2 = (b1 == 0) ? 1 : 0;
      for (int ip = b2 + 1; ip < ports; ip++) if ((ip != b1) && (pw[ip][i] > pw[b2][i])) b2 = ip;
      if (diag || flip) {
        /* the pair {b1, b2} is a set (its average does not depend on their order): what can flip
         * is the second port against the best of the others */
        double r2 = 0;
        int b3 = -1;
        for (int ip = 0; ip < ports; ip++)
          if ((port_mask & (1 << ip)) && ip != b1 && ip != b2 && pw[ip][i] > r2) { r2 = pw[ip][i]; b3 = ip; }
        const double m = (pw[b1][i] > 0 && b3 >= 0) ? (pw[b2][i] - r2) / pw[b1][i] : INFINITY;
        if (diag && m < diag[0]) diag[0] = m;
        if (diag && fabs(amin - 745.13) < diag[2]) diag[2] = fabs(amin - 745.13);
        if (flip && m > 0 && m < or_tex_near_tie) b2 = b3;
      }
      double w1 = pw[b1][i] / (pw[b1][i] + pw[b2][i]), w2 = 1.0 - w1;
      for (int chn = 0; chn < numcol; chn++) color_avg[chn][i] = w1 * iclt[b1][chn][i] + w2 * iclt[b2][chn][i];
      double d2[4];
      for (int ip = 0; ip < ports; ip++)
        if (port_mask & (1 << ip)) {
          d2[ip] = 0;
          for (int chn = 0; chn < numcol; chn++) {
            double dc = iclt[ip][chn][i] - color_avg[chn][i];
            dc /= lt_window[i];
            d2[ip] += chn_weights[chn] * dc * dc;
          }
          pw[ip][i] = exp(-ksigma * d2[ip]);
        }
      if (diag && !flip) {
        double bmin = INFINITY;
        for (int ip = 0; ip < ports; ip++)
          if ((port_mask & (1 << ip)) && ksigma * d2[ip] < bmin) bmin = ksigma * d2[ip];
        if (fabs(bmin - 745.13) < diag[2]) diag[2] = fabs(bmin - 745.13);
      }
      double k = 0.0;
      for (int ip = 0; ip < ports; ip++) k += pw[ip][i];
      k = 1.0 / k;
      for (int chn = 0; chn < numcol; chn++) {
        color_avg[chn][i] = 0;
        for (int ip = 0; ip < ports; ip++) color_avg[chn][i] += k * pw[ip][i] * iclt[ip][chn][i];
      }
    }
  } else if (usedPorts > 0) {
    for (int ip = 0; ip < ports; ip++)
      if (port_mask & (1 << ip))
        for (int i = 0; i < 256; i++) {
          for (int chn = 0; chn < numcol; chn++) color_avg[chn][i] = iclt[ip][chn][i];
          pw[ip][i] = 1.0;
        }
  }
  if (dust && (usedPorts == 4)) dust_remove(pw, diag, flip);
  for (int i = 0; i < 256; i++) {
    double alpha = 0.0;
    for (int ip = 0; ip < ports; ip++) if (port_mask & (1 << ip)) alpha += pw[ip][i];
    alpha *= lt_window[i] / usedPorts;
    rgba[3 * 256 + i] = alpha;
  }
  for (int chn = 0; chn < numcol; chn++) memcpy(rgba + chn * 256, color_avg[chn], sizeof(color_avg[chn]));
  for (int ip = 0; ip < ports; ip++) memcpy(rgba + (numcol + 1 + ip) * 256, pw[ip], sizeof(pw[ip]));
}

/* port weighting, aux values and the RGB mix of a tile's per-port tiles (ic: IMCLT, db: debayered) */
static void texture_tail(double ic[4][3][256], double db[4][3][256], const double *lt_window2, int img_mask,
                         const double *col_weights, const or_tex_params *tp, double *out, double *aux, double *diag,
                         int flip) {
  tile_combine_rgba(db, lt_window2, img_mask, tp->diff_sigma, col_weights, tp->dust_remove, out, diag, flip);
  if (aux) { /* max_diff (2964-2981) from the combined average, ports_rgb (2982-2994) */
    for (int ip = 0; ip < 4; ip++) {
      double md = 0;
      if (img_mask & (1 << ip))
        for (int i = 0; i < 256; i++) {
          double d2 = 0.0;
          for (int chn = 0; chn < 3; chn++) {
            double dc = db[ip][chn][i] - out[chn * 256 + i];
            d2 += dc * dc * col_weights[chn];
          }
          d2 *= lt_window2[i];
          if (d2 > md) md = d2;
        }
      aux[ip] = sqrt(md);
    }
    for (int ip = 0; ip < 4; ip++)
      for (int chn = 0; chn < 3; chn++) {
        double s = 0;
        for (int i = 0; i < 256; i++) s += db[ip][chn][i];
        aux[4 + chn * 4 + ip] = s / 256;
      }
  }
  /* RGB from the un-debayered tiles weighted by the port weights (ImageDtt.java:2788-2801) */
  for (int i = 0; i < 256; i++) {
    double sw = 0.0;
    for (int ip = 0; ip < 4; ip++) sw += out[(3 + 1 + ip) * 256 + i];
    if (sw != 0) sw = 1.0 / sw;
    for (int chn = 0; chn < 3; chn++) {
      double v = 0.0;
      for (int ip = 0; ip < 4; ip++) v += sw * out[(3 + 1 + ip) * 256 + i] * ic[ip][chn][i];
      out[chn * 256 + i] = v;
    }
  }
}

void or_texture_tile(const double *clt_in, const double *filter, int img_mask, const double *col_weights,
                     double extra_disparity, const or_tex_params *tp, double *out, double *aux) {
  or_texture_tile_diag(clt_in, filter, img_mask, col_weights, extra_disparity, tp, out, aux, NULL, NULL, 0.0);
}

void or_texture_tile_diag(const double *clt_in, const double *filter, int img_mask, const double *col_weights,
                          double extra_disparity, const or_tex_params *tp, double *out, double *aux, double *diag,
                          double *out_alt, double near_tie) {
  tables();
  or_tex_near_tie = near_tie;
  if (diag) diag[0] = diag[1] = diag[2] = INFINITY;
  double lt_window[256], lt_window2[256];
  or_win2d(lt_window);
  for (int i = 0; i < 256; i++) lt_window2[i] = lt_window[i] * lt_window[i];
  double(*ic)[3][256] = (double(*)[3][256])malloc(sizeof(double) * 4 * 3 * 256);
  double(*db)[3][256] = (double(*)[3][256])malloc(sizeof(double) * 4 * 3 * 256);
  double *clt = (double *)malloc(sizeof(double) * 4 * 3 * 256);
  memcpy(clt, clt_in, sizeof(double) * 4 * 3 * 256);
  if (extra_disparity != 0.0) /* 2663-2678 */
    for (int chn = 0; chn < 3; chn++)
      for (int i = 0; i < 4; i++)
        or_fract_shift((double(*)[64])(clt + (i * 3 + chn) * 256),
                       extra_disparity * PORT_OFFSETS[i][0] / tp->corr_magic_scale,
                       extra_disparity * PORT_OFFSETS[i][1] / tp->corr_magic_scale);
  const double scale = 0.25;
  for (int i = 0; i < 4; i++)
    for (int chn = 0; chn < 3; chn++) {
      for (int dct_mode = 0; dct_mode < 4; dct_mode++) {
        double t[64], tdct[64], mdct[256];
        const double *src = clt + ((i * 3 + chn) * 4 + dct_mode) * 64;
        for (int j = 0; j < 64; j++) t[j] = src[j] * (scale * filter[j]);
        int idct_mode = ((dct_mode << 1) & 2) | ((dct_mode >> 1) & 1);
        or_dttt_iv(t, tdct, idct_mode);
        or_unfold_tile(tdct, dct_mode, mdct);
        for (int j = 0; j < 256; j++) {
          if (dct_mode == 0) ic[i][chn][j] = mdct[j];
          else ic[i][chn][j] += mdct[j];
        }
      }
      tile_debayer_shot_corr(chn != 2, ic[i][chn], lt_window2, tp->min_shot, tp->scale_shot, db[i][chn]);
    }
  texture_tail(ic, db, lt_window2, img_mask, col_weights, tp, out, aux, diag, 0);
  if (out_alt) texture_tail(ic, db, lt_window2, img_mask, col_weights, tp, out_alt, NULL, NULL, 1);
  free(ic);
  free(db);
  free(clt);
}

/* ------------------------------------------------------------------------- */
/* Kernel preparation (QuadCLT.calculateCLTKernel 433-667, ImageDtt 4625-4851) */
/* ------------------------------------------------------------------------- */
void or_calc_clt_kernel(const double *src, int normalize, double clt[4][64], double extra[8]) {
  tables();
  const int src_size = 64, dtt_size = 8;
  double dst[225 + 8];
  memset(dst, 0, sizeof(dst));
  /* clt_convert_double_kernel (4625-4672) */
  static const int indices[9] = {0, -64, -1, 1, 64, -65, -63, 63, 65};
  static const double weights[9] = {1.0, 0.5, 0.5, 0.5, 0.5, 0.25, 0.25, 0.25, 0.25};
  int src_center = src_size / 2;
  double sx = 0.0, sy = 0.0, s = 0.0;
  int indx = 0;
  for (int i = -src_center; i < src_center; i++)
    for (int j = -src_center; j < src_center; j++) {
      double d = src[indx++];
      sx += j * d; sy += i * d; s += d;
    }
  int src_x = (int)java_round(sx / s) + src_center;
  int src_y = (int)java_round(sy / s) + src_center;
  if (src_x < 2 * dtt_size) src_x = 2 * dtt_size - 1;
  else if (src_x > (src_size - 2 * dtt_size)) src_x = src_size - 2 * dtt_size;
  if (src_y < 2 * dtt_size) src_y = 2 * dtt_size - 1;
  else if (src_y > (src_size - 2 * dtt_size)) src_y = src_size - 2 * dtt_size;
  indx = 0;
  for (int i = -dtt_size + 1; i < dtt_size; i++) {
    int src_i = (src_y + 2 * i) * src_size + src_x;
    for (int j = -dtt_size + 1; j < dtt_size; j++) {
      double d = 0.0;
      for (int k = 0; k < 9; k++) d += weights[k] * src[src_i + 2 * j + indices[k]];
      dst[indx++] = d;
    }
  }
  dst[indx++] = 0.5 * (src_x - src_center);
  dst[indx++] = 0.5 * (src_y - src_center);
  dst[indx++] = 0.5 * (sx / s);
  dst[indx++] = 0.5 * (sy / s);
  /* clt_normalize_kernel (4674-4696) with norm_sym_weights (QuadCLT.java:465-472) */
  if (normalize) {
    double window[64];
    for (int i = 0; i < dtt_size; i++)
      for (int j = 0; j < dtt_size; j++)
        window[i * dtt_size + j] = cos(M_PI * i / (2 * dtt_size)) * cos(M_PI * j / (2 * dtt_size));
    double sn = 0.0;
    indx = 0;
    for (int i = -dtt_size + 1; i < dtt_size; i++) {
      int ai = (i < 0) ? -i : i;
      for (int j = -dtt_size + 1; j < dtt_size; j++) {
        int aj = (j < 0) ? -j : j;
        sn += dst[indx++] * window[ai * dtt_size + aj];
      }
    }
    sn = 1.0 / sn;
    for (int i = 0; i < 225; i++) dst[i] *= 16 * sn;
  }
  /* clt_symmetrize_kernel (4698-4723) */
  double sym[4][64];
  memset(sym, 0, sizeof(sym));
  int in_size = 15, m1 = 7, center = m1 * in_size + m1;
  for (int i = 0; i < dtt_size; i++) {
    for (int j = 0; j < dtt_size; j++) {
      int i0 = center - i * in_size - j, i1 = center - i * in_size + j;
      int i2 = center + i * in_size - j, i3 = center + i * in_size + j;
      sym[0][i * 8 + j] = 0.25 * (dst[i0] + dst[i1] + dst[i2] + dst[i3]);
      if (j > 0) sym[1][i * 8 + j - 1] = 0.25 * (-dst[i0] + dst[i1] - dst[i2] + dst[i3]);
      if (i > 0) sym[2][(i - 1) * 8 + j] = 0.25 * (-dst[i0] - dst[i1] + dst[i2] + dst[i3]);
      if ((i > 0) && (j > 0)) sym[3][(i - 1) * 8 + (j - 1)] = 0.25 * (-dst[i0] + dst[i1] - dst[i2] + dst[i3]);
    }
    sym[1][i * 8 + m1] = 0.0;
    sym[2][m1 * 8 + i] = 0.0;
    sym[3][i * 8 + m1] = 0.0;
    sym[3][m1 * 8 + i] = 0.0;
  }
  /* clt_dtt3_kernel (4725-4734) */
  for (int q = 0; q < 4; q++) or_dttt_iiie(sym[q], clt[q], q);
  for (int i = 0; i < 8; i++) extra[i] = dst[225 + i];
}

/* ImageDtt.clt_fill_coord_corr (4792-4851) for one colour plane ext[kv][kh][8] */
void or_fill_coord_corr(double *ext, int kh, int kv, int kern_step) {
  for (int ty = 0; ty < kv; ty++)
    for (int tx = 0; tx < kh; tx++) {
      double s0 = 0, sx = 0, sx2 = 0, sy = 0, sy2 = 0, sz = 0, sxz = 0, syz = 0, sw = 0, sxw = 0, syw = 0;
      for (int dty = -1; dty < 2; dty++) {
        int y = ty + dty;
        if ((y < 0) || (y >= kv)) continue;
        for (int dtx = -1; dtx < 2; dtx++) {
          int x = tx + dtx;
          if ((x < 0) || (x >= kh)) continue;
          const double *ce = ext + ((size_t)y * kh + x) * 8;
          s0 += 1; sx += dtx; sx2 += dtx * dtx; sy += dty; sy2 += dty * dty;
          sz += ce[2]; sxz += dtx * ce[2]; syz += dty * ce[2];
          sw += ce[3]; sxw += dtx * ce[3]; syw += dty * ce[3];
        }
      }
      double *ce = ext + ((size_t)ty * kh + tx) * 8;
      double denom_x = (sx2 * s0 - sx * sx) * kern_step;
      double denom_y = (sy2 * s0 - sy * sy) * kern_step;
      ce[4] = (sxz * s0 - sz * sx) / denom_x;
      ce[5] = (syz * s0 - sz * sy) / denom_y;
      ce[6] = (sxw * s0 - sw * sx) / denom_x;
      ce[7] = (syw * s0 - sw * sy) / denom_y;
    }
}

/* ------------------------------------------------------------------------- */
/* Driver: clt_aberrations_quad_corr_new tile loop (ImageDtt.java:1491-2824)   */
/* ------------------------------------------------------------------------- */
typedef struct {
  const or_run_cfg *cfg;
  const or_geometry *g;
  const double *ports_in;
  const double *const *images, *const *kern, *const *kext;
  const int *tile_op;
  const double *disparity;
  const or_pairs *pairs;
  const or_corr_params *cp;
  double *ports, *clt, *corr, *disp;
  int *int_tl;
  double *residual;
  double *diag;  /* [T][OR_DIAG_N] or NULL: combined strip rows, hor / vert ortho profiles */
  double (*rots)[3][3];
  double *tbl;
  int tbl_len;
  double filter[64];
  double col_weights[3];
  double wndx[32], wndy[32], notch[15];
  int num_tiles;
  volatile int next;
} run_ctx;

static void run_tile(run_ctx *c, int nTile, double *wk_clt, double *wk_corr, double *wk_strips) {
  const or_run_cfg *cfg = c->cfg;
  const int S = cfg->num_sensors, C = cfg->num_colors;
  const int tilesX = cfg->width / 8;
  int tileY = nTile / tilesX, tileX = nTile % tilesX;
  const int P = c->pairs->num_pairs;
  const int hw = c->cp->corr_strip_hight;
  if (c->disp)
    for (int i = 0; i < OR_DISP_N; i++)
      c->disp[(size_t)nTile * OR_DISP_N + i] =
          ((i == OR_DISP_STRENGTH) || (i == OR_DISP_HOR_STRENGTH) || (i == OR_DISP_VERT_STRENGTH)) ? 0.0 : NAN;
  if (c->tile_op[nTile] == 0) return;
  double centerX = tileX * 8 + 8 / 2;
  double centerY = tileY * 8 + 8 / 2;
  double pxy[OR_MAX_SENSORS][2];
  if (cfg->use_ports_in) {
    for (int i = 0; i < S; i++) {
      pxy[i][0] = c->ports_in[((size_t)nTile * S + i) * 2];
      pxy[i][1] = c->ports_in[((size_t)nTile * S + i) * 2 + 1];
    }
  } else {
    or_ports(c->g, (const double(*)[3][3])c->rots, NULL, c->tbl, c->tbl_len, centerX, centerY,
             c->disparity[nTile], pxy, NULL);
  }
  if (c->ports)
    for (int i = 0; i < S; i++) {
      c->ports[((size_t)nTile * S + i) * 2] = pxy[i][0];
      c->ports[((size_t)nTile * S + i) * 2 + 1] = pxy[i][1];
    }
  /* stage 2: per colour, per sensor extract + fract_shift (1904-2061) */
  for (int chn = 0; chn < C; chn++) {
    for (int i = 0; i < S; i++) {
      double(*t)[64] = (double(*)[64])(wk_clt + ((size_t)i * C + chn) * 256);
      const double *kern = NULL, *kext = NULL;
      if (cfg->kernels_hor > 0) {
        size_t kplane = (size_t)cfg->kernels_hor * cfg->kernels_vert;
        kern = c->kern[i] + kplane * 256 * chn;
        kext = c->kext[i] + kplane * 8 * chn;
      }
      double res[2];
      int tl[2];
      or_extract_correct_tile(c->images[i * C + chn], cfg->width, cfg->height, kern, kext,
                              cfg->kernels_hor, cfg->kernels_vert, cfg->kernel_step, pxy[i][0], pxy[i][1],
                              t, res, tl, NULL);
      or_fract_shift(t, res[0], res[1]);
      size_t o = (((size_t)nTile * S + i) * C + chn) * 2;
      if (c->int_tl) { c->int_tl[o] = tl[0]; c->int_tl[o + 1] = tl[1]; }
      if (c->residual) { c->residual[o] = res[0]; c->residual[o + 1] = res[1]; }
    }
  }
  if (c->clt) memcpy(c->clt + (size_t)nTile * S * C * 256, wk_clt, sizeof(double) * S * C * 256);
  if (!cfg->corr) return;
  /* stage 3 (2101-2245) */
  for (int p = 0; p < P; p++)
    or_correlate_pair(wk_clt + (size_t)c->pairs->cam1[p] * C * 256, wk_clt + (size_t)c->pairs->cam2[p] * C * 256, C,
                      c->col_weights, c->filter, c->cp->fat_zero, wk_corr + (size_t)p * 225);
  if (c->corr) memcpy(c->corr + (size_t)nTile * P * 225, wk_corr, sizeof(double) * P * 225);
  if (!c->disp) return;
  int use[OR_MAX_PAIRS], is_diag[OR_MAX_PAIRS];
  for (int p = 0; p < P; p++) {
    use[p] = (p < 64) ? ((c->pairs->combo_mask_lo >> p) & 1) : ((c->pairs->combo_mask_hi >> (p - 64)) & 1);
    if (P > 6) use[p] = 1;
    is_diag[p] = (c->pairs->kind[p] == 2) || (c->pairs->kind[p] == 3);
    if (use[p]) or_strip(wk_corr + (size_t)p * 225, c->pairs->bx[p], c->pairs->by[p], c->pairs->kind[p], hw,
                         wk_strips + (size_t)p * hw * 15);
  }
  double combo[15 * 32];
  int general = P > 6;
  for (int p = 0; p < P; p++) general |= (c->pairs->kind[p] == 4);
  if (general) {
    /* Generalised pair sets (not in the reference): the same geometric mean of
     * the clipped offset strips, evaluated in the log domain so that products of
     * up to 120 factors neither overflow nor underflow. */
    int len = hw * 15, n = 0;
    for (int p = 0; p < P; p++) n += use[p];
    for (int i = 0; i < len; i++) {
      double ls = 0.0;
      int nan_ = 0, zero = 0;
      for (int p = 0; p < P; p++) {
        if (!use[p]) continue;
        double d = wk_strips[(size_t)p * len + i] + c->cp->corr_offset;
        if (d < 0.0) d = 0.0;
        if (isnan(d)) nan_ = 1;
        else if (d == 0.0) zero = 1;
        else ls += log(d);
      }
      combo[i] = nan_ ? NAN : (zero ? 0.0 : exp(ls / n) - c->cp->corr_offset);
    }
  } else {
    or_combine_strips(wk_strips, use, P, is_diag, hw, c->cp->corr_offset, c->cp->twice_diagonal, combo);
  }
  double *dm = c->disp + (size_t)nTile * OR_DISP_N;
  double *dg = c->diag ? c->diag + (size_t)nTile * OR_DIAG_N : NULL;
  if (dg) {
    for (int i = 0; i < OR_DIAG_N; i++) dg[i] = NAN;
    memcpy(dg, combo, sizeof(double) * (hw < OR_DIAG_ROWS ? hw : OR_DIAG_ROWS) * 15);
  }
  int ix;
  if (or_max_xy_int_axis(combo, hw, c->cp->min_corr, &ix)) {
    double strength = combo[ix + 8 - 1];
    dm[OR_DISP_INT] = -ix;
    dm[OR_DISP_STRENGTH] = strength;
    dm[OR_DISP_IXY] = ix;
    double cs[3];
    if (or_max_x_cm(combo, hw, ix, c->wndy, c->cp->corr_wndy_size, c->wndx, c->cp->corr_wndx_size, cs)) {
      dm[OR_DISP_CM] = -cs[0];
      dm[OR_DISP_CM_S0] = cs[1];
    }
  }
  int useo[OR_MAX_PAIRS];
  double r[2];
  for (int p = 0; p < P; p++) useo[p] = (c->pairs->kind[p] == 0);
  if (or_max_xs_ortho(wk_corr, useo, P, c->cp->corr_offset, 0, c->notch, r)) {
    dm[OR_DISP_HOR] = -r[0];
    dm[OR_DISP_HOR_STRENGTH] = r[1];
    if (dg) or_max_xs_ortho_profile(wk_corr, useo, P, c->cp->corr_offset, 0, c->notch, dg + OR_DIAG_ROWS * 15);
  }
  for (int p = 0; p < P; p++) useo[p] = (c->pairs->kind[p] == 1);
  if (or_max_xs_ortho(wk_corr, useo, P, c->cp->corr_offset, 1, c->notch, r)) {
    dm[OR_DISP_VERT] = -r[0];
    dm[OR_DISP_VERT_STRENGTH] = r[1];
    if (dg) or_max_xs_ortho_profile(wk_corr, useo, P, c->cp->corr_offset, 1, c->notch, dg + OR_DIAG_ROWS * 15 + 15);
  }
}

static void *run_worker(void *arg) {
  run_ctx *c = (run_ctx *)arg;
  const int S = c->cfg->num_sensors, C = c->cfg->num_colors, P = c->pairs->num_pairs;
  double *wk_clt = (double *)malloc(sizeof(double) * S * C * 256);
  double *wk_corr = (double *)malloc(sizeof(double) * (P + 1) * 225);
  double *wk_strips = (double *)malloc(sizeof(double) * (P + 1) * 15 * 32);
  for (int nTile = __atomic_fetch_add(&c->next, 1, __ATOMIC_RELAXED); nTile < c->num_tiles;
       nTile = __atomic_fetch_add(&c->next, 1, __ATOMIC_RELAXED))
    run_tile(c, nTile, wk_clt, wk_corr, wk_strips);
  free(wk_clt); free(wk_corr); free(wk_strips);
  return NULL;
}

int or_run(const or_run_cfg *cfg, const or_geometry *g, const double *ports_in,
           const double *const *images, const double *const *kern, const double *const *kext,
           const int *tile_op, const double *disparity, const or_pairs *pairs, const or_corr_params *cp,
           double *ports, double *clt, double *corr, double *disp, int *int_tl, double *residual) {
  return or_run_diag(cfg, g, ports_in, images, kern, kext, tile_op, disparity, pairs, cp, ports, clt, corr, disp,
                     int_tl, residual, NULL);
}

int or_run_diag(const or_run_cfg *cfg, const or_geometry *g, const double *ports_in,
                const double *const *images, const double *const *kern, const double *const *kext,
                const int *tile_op, const double *disparity, const or_pairs *pairs, const or_corr_params *cp,
                double *ports, double *clt, double *corr, double *disp, int *int_tl, double *residual,
                double *diag) {
  tables();
  if (cfg->num_sensors < 1 || cfg->num_sensors > OR_MAX_SENSORS) return -1;
  if (cfg->num_colors != 1 && cfg->num_colors != 3) return -2;
  if (cp->corr_strip_hight > 32 || cp->corr_wndx_size > 32 || cp->corr_wndy_size > 32) return -3;
  run_ctx c;
  memset(&c, 0, sizeof(c));
  c.cfg = cfg; c.g = g; c.ports_in = ports_in; c.images = images; c.kern = kern; c.kext = kext;
  c.tile_op = tile_op; c.disparity = disparity; c.pairs = pairs; c.cp = cp;
  c.ports = ports; c.clt = clt; c.corr = corr; c.disp = disp; c.int_tl = int_tl; c.residual = residual;
  c.diag = diag;
  c.num_tiles = (cfg->width / 8) * (cfg->height / 8);
  double rots[OR_MAX_SENSORS][3][3];
  double tbl[2100];
  if (!cfg->use_ports_in) {
    or_rot_matrices(g, rots);
    c.tbl_len = or_reverse_distortion_table(g, tbl, 2100);
    if (c.tbl_len < 0) return -4;
  }
  c.rots = rots;
  c.tbl = tbl;
  or_corr_lpf(cp->corr_sigma, c.filter);
  c.col_weights[2] = 1.0 / (1.0 + cp->corr_red + cp->corr_blue);  /* ImageDtt.java:1571-1581 */
  c.col_weights[0] = cp->corr_red * c.col_weights[2];
  c.col_weights[1] = cp->corr_blue * c.col_weights[2];
  or_half_flat_top_window(cp->corr_wndy_size, cp->corr_wndy_hwidth, cp->corr_wndy_blur, 1, 0, 1.0, c.wndy);
  or_half_flat_top_window(cp->corr_wndx_size, cp->corr_wndx_hwidth, cp->corr_wndx_blur, 1, 0, 2.0, c.wndx);
  or_ortho_notch(cp->enhortho_width, cp->enhortho_scale, c.notch);
  int nt = cfg->num_threads > 0 ? cfg->num_threads : 1;
  pthread_t th[256];
  if (nt > 256) nt = 256;
  for (int i = 0; i < nt; i++) pthread_create(&th[i], NULL, run_worker, &c);
  for (int i = 0; i < nt; i++) pthread_join(th[i], NULL);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* IMCLT of whole frames, threaded like ImageDtt.iclt_2d (3559-3666): four     */
/* passes over the tile parities, tiles of one pass never overlap.            */
/* ------------------------------------------------------------------------- */
typedef struct {
  const double *clt;
  const int *present;
  const double *lpf;
  double *frames;
  int tilesX, tilesY, S, C, pass;
  double scale;
  volatile int next;
} iclt_ctx;

static void *iclt_worker(void *arg) {
  iclt_ctx *c = (iclt_ctx *)arg;
  const int nx = (c->tilesX + 1 - (c->pass & 1)) / 2, ny = (c->tilesY + 1 - ((c->pass >> 1) & 1)) / 2;
  const int fw = c->tilesX * 8 + 8, fh = c->tilesY * 8 + 8;
  for (int n = __atomic_fetch_add(&c->next, 1, __ATOMIC_RELAXED); n < nx * ny;
       n = __atomic_fetch_add(&c->next, 1, __ATOMIC_RELAXED)) {
    int tx = 2 * (n % nx) + (c->pass & 1), ty = 2 * (n / nx) + ((c->pass >> 1) & 1);
    int tile = ty * c->tilesX + tx;
    if (c->present && !c->present[tile]) continue;
    for (int s = 0; s < c->S; s++)
      for (int col = 0; col < c->C; col++) {
        const double *src = c->clt + (((size_t)tile * c->S + s) * c->C + col) * 256;
        double q[4][64];
        for (int m = 0; m < 4; m++)
          for (int i = 0; i < 64; i++) q[m][i] = src[m * 64 + i] * (c->lpf ? c->lpf[col * 64 + i] : 1.0);
        or_iclt_tile_add((const double(*)[64])q, c->scale, tx, ty,
                         c->frames + ((size_t)s * c->C + col) * fw * fh, fw);
      }
  }
  return NULL;
}

int or_imclt_frames(const double *clt, const int *present, int tilesX, int tilesY, int S, int C, double scale,
                    const double *lpf, double *frames, int num_threads, int zero_frames) {
  tables();
  iclt_ctx c;
  memset(&c, 0, sizeof(c));
  c.clt = clt; c.present = present; c.lpf = lpf; c.frames = frames;
  c.tilesX = tilesX; c.tilesY = tilesY; c.S = S; c.C = C; c.scale = scale;
  size_t n = (size_t)S * C * (tilesX * 8 + 8) * (tilesY * 8 + 8);
  if (zero_frames) memset(frames, 0, n * sizeof(double));
  int nt = num_threads > 0 ? (num_threads > 256 ? 256 : num_threads) : 1;
  pthread_t th[256];
  for (int pass = 0; pass < 4; pass++) {
    c.pass = pass;
    c.next = 0;
    for (int i = 0; i < nt; i++) pthread_create(&th[i], NULL, iclt_worker, &c);
    for (int i = 0; i < nt; i++) pthread_join(th[i], NULL);
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Texture tiles of many tiles on a thread pool (the reference's per-tile     */
/* worker threads, ImageDtt.java:1750-2812)                                   */
/* ------------------------------------------------------------------------- */
typedef struct {
  const double *clt, *filter, *col_weights, *extra;
  const int *tiles, *img_mask;
  int n;
  const or_tex_params *tp;
  double *out, *aux;
  int next;
} tex_ctx;

static void *tex_worker(void *arg) {
  tex_ctx *c = (tex_ctx *)arg;
  for (int k = __atomic_fetch_add(&c->next, 1, __ATOMIC_RELAXED); k < c->n;
       k = __atomic_fetch_add(&c->next, 1, __ATOMIC_RELAXED)) {
    const int t = c->tiles[k];
    or_texture_tile(c->clt + (size_t)t * 4 * 3 * 256, c->filter, c->img_mask[k], c->col_weights,
                    c->extra ? c->extra[k] : 0.0, c->tp, c->out + (size_t)k * 12 * 256,
                    c->aux ? c->aux + (size_t)k * 16 : NULL);
  }
  return NULL;
}

int or_texture_tiles(const double *clt, const int *tiles, const int *img_mask, const double *extra, int n,
                     const double *filter, const double *col_weights, const or_tex_params *tp, double *out,
                     double *aux, int num_threads) {
  tables();
  tex_ctx c;
  memset(&c, 0, sizeof(c));
  c.clt = clt; c.filter = filter; c.col_weights = col_weights; c.extra = extra;
  c.tiles = tiles; c.img_mask = img_mask; c.n = n; c.tp = tp; c.out = out; c.aux = aux;
  int nt = num_threads > 0 ? (num_threads > 256 ? 256 : num_threads) : 1;
  pthread_t th[256];
  for (int i = 0; i < nt; i++) pthread_create(&th[i], NULL, tex_worker, &c);
  for (int i = 0; i < nt; i++) pthread_join(th[i], NULL);
  return 0;
}

/* ------------------------------------------------------------------------- */
/* Inter-camera (rig) correlation of two quad cameras for one tile:          */
/* Correlation2d.correlateInterCamerasFD (401-414) with cltMixCameras        */
/* (424-448), then ImageDtt.tileInterCamCorrs (7370-7560) without the LMA     */
/* branch (min_poly_strength above any strength) and with notch mode off.    */
/* ------------------------------------------------------------------------- */
void or_rig_tile(const double *clt_main, int s_main, const double *clt_aux, int s_aux, int nc,
                 const or_corr_params *cp, double cm_max_normalization, int no_int_x0, double *corr225,
                 double rec[4]) {
  tables();
  double mix[2][3 * 256];
  const double *src[2] = {clt_main, clt_aux};
  const int ns[2] = {s_main, s_aux};
  for (int k = 0; k < 2; k++) {
    for (int i = 0; i < nc * 256; i++) mix[k][i] = 0.0;
    for (int s = 0; s < ns[k]; s++)
      for (int i = 0; i < nc * 256; i++) mix[k][i] += src[k][(size_t)s * nc * 256 + i];
    const double kk = 1.0 / ns[k];
    for (int i = 0; i < nc * 256; i++) mix[k][i] *= kk;
  }
  double lpf[64], cw[3];
  or_corr_lpf(cp->corr_sigma, lpf);
  const double g = 1.0 / (1.0 + cp->corr_red + cp->corr_blue);
  cw[0] = cp->corr_red * g;
  cw[1] = cp->corr_blue * g;
  cw[2] = g;
  or_correlate_pair(mix[0], mix[1], nc, cw, lpf, cp->fat_zero, corr225);
  const int hw = cp->corr_strip_hight;
  double strip[16 * 15], combo[16 * 15];
  or_strip(corr225, 1.0, 0.0, 0, hw, strip);  /* PAIRS[0]: the horizontal pair grid */
  int use = 1, diag = 0;
  or_combine_strips(strip, &use, 1, &diag, hw, cp->corr_offset, cp->twice_diagonal, combo);
  rec[0] = NAN;
  rec[1] = 0.0;
  rec[2] = NAN;
  rec[3] = NAN;
  int ix;
  if (!or_max_xy_int_axis(combo, hw, (no_int_x0 ? 0.5 : 1.0) * cp->min_corr, &ix)) return;
  rec[0] = -ix;
  rec[1] = combo[ix + 7];
  double wndy[32], wndx[32], cs[3];
  or_half_flat_top_window(cp->corr_wndy_size, cp->corr_wndy_hwidth, cp->corr_wndy_blur, 1, 0, 1.0, wndy);
  or_half_flat_top_window(cp->corr_wndx_size, cp->corr_wndx_hwidth, cp->corr_wndx_blur, 1, 0, 2.0, wndx);
  if (or_max_x_cm(combo, hw, no_int_x0 ? 0 : ix, wndy, cp->corr_wndy_size, wndx, cp->corr_wndx_size, cs)) {
    rec[0] = -cs[0];
    const double eff = cs[2] * cm_max_normalization;
    rec[1] = cs[1] / (eff * eff);
  }
}

/* ===================== LMA disparity (Correlation2d.corrLMA) ===================== */

void or_default_lma_params(or_lma_params *p) {
  /* ImageDttParameters.java:32-109 */
  p->min_poly_strength = 0.2;
  p->mix_corr_poly = 1;
  p->ortho_vasw_pwr = 2.0;
  p->cnvx_hwnd_size = 4;
  p->cnvx_weight = 0.5;
  p->cnvx_add3x3 = 1;
  p->adjust_wm = 1; p->adjust_wy = 0; p->adjust_wxy = 1; p->adjust_ag = 1;
  p->half_width = 2.0; p->cost_wy = 0.1; p->cost_wxy = 0.1;
  p->lambda_initial = 0.1; p->lambda_scale_good = 0.5; p->lambda_scale_bad = 8.0; p->lambda_max = 100.0;
  p->rms_diff = 0.001;
  p->num_iter = 20;
  p->pair_mask = 0x3f;
}

/* Correlation2d.filterConvex (2029-2208) */
void or_filter_convex(const double *d, int hwin, int x0c, int y0c, int add3x3, double nc_cost, double *weights) {
  const int W = OR_CORR, center = OR_DTT - 1;
  const int x0 = x0c + center, y0 = y0c + center;
  unsigned char convex[OR_CORR * OR_CORR], sel[OR_CORR * OR_CORR], seln[OR_CORR * OR_CORR];
  memset(convex, 0, sizeof(convex));
  memset(sel, 0, sizeof(sel));
  for (int i = 0; i < W * W; i++) weights[i] = 0.0;
  int min_row = y0 - hwin, max_row = y0 + hwin, min_col = x0 - hwin, max_col = x0 + hwin;
  if (min_row < 0) min_row = 0;
  if (max_row >= W) max_row = W - 1;
  if (min_col < 0) min_col = 0;
  if (max_col >= W) max_col = W - 1;
  for (int row = min_row + 1; row < max_row; row++)
    for (int col = min_col + 1; col < max_col; col++) {
      const int i = row * W + col;
      convex[i] = (2 * d[i] > (d[i - 1] + d[i + 1])) && (2 * d[i] > (d[i - W] + d[i + W]));
    }
  if ((y0 >= min_row) && (y0 <= max_row) && (x0 >= min_col) && (x0 <= max_col)) sel[y0 * W + x0] = 1;
  for (int istep = 0; istep < hwin; istep++) {
    memcpy(seln, sel, sizeof(sel));
    const int first = (istep == 0);
    int num_new = 0;
    int smin_row = y0 - istep, smax_row = y0 + istep, smin_col = x0 - istep, smax_col = x0 + istep;
    if (smin_row < 0) smin_row = 0;
    if (smax_row >= W) smax_row = W - 1;
    if (smin_col < 0) smin_col = 0;
    if (smax_col >= W) smax_col = W - 1;
    if (istep < y0) { /* up */
      const int row = y0 - istep;
      for (int col = smin_col; col <= smax_col; col++) {
        const int i = row * W + col;
        if (sel[i] && (convex[i] || first)) {
          if (!seln[i - W]) { seln[i - W] = 1; num_new++; }
          const int j = i - W;
          if (convex[j]) {
            if ((col <= x0) && (col > min_col) && !seln[j - 1]) { seln[j - 1] = 1; num_new++; }
            if ((col >= x0) && (col < max_col) && !seln[j + 1]) { seln[j + 1] = 1; num_new++; }
          }
        }
      }
    }
    if ((y0 + istep) < max_row) { /* down */
      const int row = y0 + istep;
      for (int col = smin_col; col <= smax_col; col++) {
        const int i = row * W + col;
        if (sel[i] && (convex[i] || first)) {
          if (!seln[i + W]) { seln[i + W] = 1; num_new++; }
          const int j = i + W;
          if (convex[j]) {
            if ((col <= x0) && (col > min_col) && !seln[j - 1]) { seln[j - 1] = 1; num_new++; }
            if ((col >= x0) && (col < max_col) && !seln[j + 1]) { seln[j + 1] = 1; num_new++; }
          }
        }
      }
    }
    if (istep < x0) { /* left */
      const int col = x0 - istep;
      for (int row = smin_row; row <= smax_row; row++) {
        const int i = row * W + col;
        if (sel[i] && (convex[i] || first)) {
          if (!seln[i - 1]) { seln[i - 1] = 1; num_new++; }
          const int j = i - 1;
          if (convex[j]) {
            if ((row <= y0) && (row > min_row) && !seln[j - W]) { seln[j - W] = 1; num_new++; }
            if ((row >= y0) && (row < max_row) && !seln[j + W]) { seln[j + W] = 1; num_new++; }
          }
        }
      }
    }
    if ((x0 + istep) < max_col) { /* right */
      const int col = x0 + istep;
      for (int row = smin_row; row <= smax_row; row++) {
        const int i = row * W + col;
        if (sel[i] && (convex[i] || first)) {
          if (!seln[i + 1]) { seln[i + 1] = 1; num_new++; }
          const int j = i + 1;
          if (convex[j]) {
            if ((row <= y0) && (row > min_row) && !seln[j - W]) { seln[j - W] = 1; num_new++; }
            if ((row >= y0) && (row < max_row) && !seln[j + W]) { seln[j + W] = 1; num_new++; }
          }
        }
      }
    }
    if (num_new == 0) break;
    memcpy(sel, seln, sizeof(sel));
  }
  for (int i = 0; i < W * W; i++)
    if (sel[i]) weights[i] = convex[i] ? 1.0 : nc_cost;
  if (add3x3) {
    for (int row = y0 - 1; row <= y0 + 1; row++)
      if ((row >= 0) && (row < W))
        for (int col = x0 - 1; col <= x0 + 1; col++)
          if ((col >= 0) && (col < W)) {
            const int i = row * W + col;
            if (weights[i] == 0.0) weights[i] = nc_cost;
          }
  }
}

#define LMA_MAX_SAMPLES 512
#define LMA_NPAR 6 /* X0, WM, WYD, WXY, AG0, AG1 */
typedef struct {
  int ns;
  double x[LMA_MAX_SAMPLES], y[LMA_MAX_SAMPLES], v[LMA_MAX_SAMPLES], w[LMA_MAX_SAMPLES];
  int grp[LMA_MAX_SAMPLES];
  int ngroups, gdiag[2];
  /* setWeightsValues */
  double weights[LMA_MAX_SAMPLES + 2], values[LMA_MAX_SAMPLES + 2], group_weights[2], pure_weight;
  double all_pars[LMA_NPAR];
  int par_idx[LMA_NPAR], nv; /* vector -> all_pars index */
} or_lma;

/* Correlations2dLMA.getFxJt (334-384): fx [ns + 2], jt [nv][ns + 2] (or NULL) */
static void lma_fx_jt(const or_lma *L, const double *vec, double *fx, double *jt) {
  double av[LMA_NPAR];
  memcpy(av, L->all_pars, sizeof(av));
  for (int k = 0; k < L->nv; k++) av[L->par_idx[k]] = vec[k];
  const int np = L->ns + 2;
  const double sqrt2 = sqrt(2.0);
  for (int n = 0; n < L->ns; n++) {
    const int g = L->grp[n];
    const double wScale = L->gdiag[g] ? sqrt2 : 1.0;
    const double Wy = av[1] * 1.0 + av[2]; /* scales[si] = 1 for the quad layout */
    const double Wx = Wy + av[3];
    const double dx = L->x[n] - av[0];
    const double Ag = av[4 + g];
    const double dxw = wScale * dx / Wx, dyw = wScale * L->y[n] / Wy;
    const double d = (1.0 - dxw * dxw - dyw * dyw);
    fx[n] = d * Ag;
    if (jt) {
      const double dfdWx = Ag * 2 * dxw * dxw / Wx, dfdWy = Ag * 2 * dyw * dyw / Wy;
      for (int k = 0; k < L->nv; k++) {
        const int pi = L->par_idx[k];
        double j = 0.0;
        if (pi == 0) j = wScale * Ag * 2 * dxw / Wx;
        else if (pi == 1) j = 1.0 * (dfdWx + dfdWy);
        else if (pi == 2) j = dfdWx + dfdWy;
        else if (pi == 3) j = dfdWx;
        else j = (pi - 4 == g) ? d : 0.0;
        jt[k * np + n] = j;
      }
    }
  }
  fx[L->ns] = av[1];
  fx[L->ns + 1] = av[3];
  if (jt)
    for (int k = 0; k < L->nv; k++) {
      jt[k * np + L->ns] = (L->par_idx[k] == 1) ? 1.0 : 0.0;
      jt[k * np + L->ns + 1] = (L->par_idx[k] == 3) ? 1.0 : 0.0;
    }
}

/* getWYmFxRms (432-452): fx becomes weights (y - fx); returns rms (rms_pure optional) */
static double lma_rms(const or_lma *L, double *fx, double *rms_pure) {
  double rms = 0.0;
  for (int i = 0; i < L->ns; i++) {
    const double d = L->values[i] - fx[i];
    fx[i] = L->weights[i] * d;
    rms += fx[i] * d;
  }
  if (rms_pure) *rms_pure = sqrt(rms) / L->pure_weight;
  for (int i = L->ns; i < L->ns + 2; i++) {
    const double d = L->values[i] - fx[i];
    fx[i] = L->weights[i] * d;
    rms += fx[i] * d;
  }
  return sqrt(rms);
}

/* solve A x = b (n x n, row-major) by LU with partial pivoting; 0 if singular (a zero pivot) */
static int lma_solve(double *A, double *b, int n) {
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int r = c + 1; r < n; r++)
      if (fabs(A[r * n + c]) > fabs(A[p * n + c])) p = r;
    if (A[p * n + c] == 0.0) return 0;
    if (p != c) {
      for (int k = 0; k < n; k++) { const double t = A[c * n + k]; A[c * n + k] = A[p * n + k]; A[p * n + k] = t; }
      const double t = b[c]; b[c] = b[p]; b[p] = t;
    }
    for (int r = c + 1; r < n; r++) {
      const double f = A[r * n + c] / A[c * n + c];
      for (int k = c; k < n; k++) A[r * n + k] -= f * A[c * n + k];
      b[r] -= f * b[c];
    }
  }
  for (int r = n - 1; r >= 0; r--) {
    double s = b[r];
    for (int k = r + 1; k < n; k++) s -= A[r * n + k] * b[k];
    b[r] = s / A[r * n + r];
  }
  return 1;
}

static void lma_add_group(or_lma *L, const double *g, int diag, int npairs, double xcenter, const or_lma_params *p) {
  /* addSamples (2230-2386) for one group, scale 1 */
  static const int qs[4][2] = {{-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
  const int hw = p->cnvx_hwnd_size, hw2 = 2 * hw + 1, center = OR_DTT - 1, W = OR_CORR;
  const int center_index = (W + 1) * center;
  const int ixc = (int)floor(xcenter + 0.5); /* Math.round */
  const double xcs = ixc * 1.0, scale05 = 0.5;
  double fw[OR_CORR * OR_CORR];
  or_filter_convex(g, hw, ixc, diag ? ixc : 0, p->cnvx_add3x3, p->cnvx_weight, fw);
  int gnum = -1;
  for (int arow = 0; arow < hw2; arow += diag ? 1 : 2) {
    const int odd = diag ? (arow & 1) : 0;
    for (int acol = odd; acol < hw2; acol += 2)
      for (int q = 0; q < 4; q++) {
        if (!(((arow > 0) || (q & 2)) && ((acol > 0) || (q & 1)))) continue;
        int cx, cy;
        if (diag) {
          cx = (qs[q][0] * acol - qs[q][1] * arow) / 2 + ixc;
          cy = (qs[q][0] * acol + qs[q][1] * arow) / 2 + ixc;
        } else {
          cx = (qs[q][0] * acol) / 2 + ixc;
          cy = (qs[q][1] * arow) / 2;
        }
        if (cx < -center || cx > center || cy < -center || cy > center) continue;
        double w = fw[center_index + W * cy + cx] * npairs;
        if (!(w > 0.0)) continue;
        const double v = g[center_index + W * cy + cx];
        if (p->ortho_vasw_pwr != 0) w *= pow(fabs(v), p->ortho_vasw_pwr);
        if (L->ns >= LMA_MAX_SAMPLES) continue;
        if (gnum < 0) { /* groups are numbered in the order their first sample arrives */
          gnum = L->ngroups++;
          L->gdiag[gnum] = diag;
        }
        L->x[L->ns] = qs[q][0] * acol * scale05 + xcs;
        L->y[L->ns] = qs[q][1] * arow * scale05;
        L->v[L->ns] = v;
        L->w[L->ns] = w;
        L->grp[L->ns] = gnum;
        L->ns++;
      }
  }
}

int or_corr_lma(const double *corrs, const int *kind, int np, double xcenter, const or_lma_params *p, double out[4],
                int *n_samples) {
  out[0] = out[1] = out[2] = out[3] = NAN;
  static or_lma Ls;  /* large: not on the stack (single-threaded use from the tests) */
  or_lma *L = &Ls;
  memset(L, 0, sizeof(*L));
  /* combineCompatiblePairs (462-490) for GROUPS {ortho, 1}, {diagonal, 1} */
  for (int gdiag = 0; gdiag < 2; gdiag++) {
    double g[OR_CORR * OR_CORR];
    memset(g, 0, sizeof(g));
    int n = 0;
    for (int i = 0; i < np; i++) {
      if (!((p->pair_mask >> i) & 1) || kind[i] < 0 || kind[i] > 3) continue;
      const int is_diag = kind[i] >= 2;
      if (is_diag != gdiag) continue;
      const double *c = corrs + (size_t)i * OR_CORR * OR_CORR;
      for (int r = 0; r < OR_CORR; r++)
        for (int q = 0; q < OR_CORR; q++) {
          double v;
          if (kind[i] == 0 || kind[i] == 2) v = c[r * OR_CORR + q];
          else if (kind[i] == 1) v = c[q * OR_CORR + r];                /* getTransposeAllOrtho */
          else v = c[(OR_CORR - r - 1) * OR_CORR + q];                   /* getTransposeAllDiagonal */
          g[r * OR_CORR + q] += v;
        }
      n++;
    }
    if (n == 0) continue;
    if (n > 1)
      for (int k = 0; k < OR_CORR * OR_CORR; k++) g[k] /= n;
    lma_add_group(L, g, gdiag, n, xcenter, p);
  }
  if (n_samples) *n_samples = L->ns;
  /* initVector (211-241) and setWeightsValues (243-275) */
  const int ns = L->ns, npt = ns + 2;
  L->all_pars[0] = xcenter;
  L->all_pars[1] = p->half_width;
  L->all_pars[2] = 0.0;
  L->all_pars[3] = 0.0;
  const int mask[LMA_NPAR] = {1, p->adjust_wm, p->adjust_wy, p->adjust_wxy, p->adjust_ag && L->ngroups > 0,
                              p->adjust_ag && L->ngroups > 1};
  L->nv = 0;
  for (int i = 0; i < 4 + L->ngroups; i++)
    if (mask[i]) L->par_idx[L->nv++] = i;
  L->weights[ns] = p->cost_wy;
  L->weights[ns + 1] = p->cost_wxy;
  L->values[ns] = p->half_width;
  L->values[ns + 1] = 0.0;
  double sw = 0.0;
  for (int i = 0; i < ns; i++) {
    L->weights[i] = L->w[i];
    L->values[i] = L->v[i];
    L->group_weights[L->grp[i]] += L->w[i];
    if (isnan(L->values[i]) || isnan(L->weights[i])) {
      L->weights[i] = 0.0;
      L->values[i] = 0.0;
    }
    sw += L->weights[i];
  }
  L->pure_weight = sw;
  sw += L->weights[ns] + L->weights[ns + 1];
  if (sw != 0.0) {
    sw = 1.0 / sw;
    for (int i = 0; i < npt; i++) L->weights[i] *= sw;
  }
  if (L->pure_weight > 0.0)
    for (int i = 0; i < L->ngroups; i++) L->group_weights[i] /= L->pure_weight;
  L->pure_weight *= sw;
  int imx = 0;
  for (int i = 1; i < ns; i++)
    if (L->values[i] > L->values[imx]) imx = i;
  for (int i = 0; i < L->ngroups; i++) L->all_pars[4 + i] = L->values[imx];
  double vec[LMA_NPAR];
  for (int k = 0; k < L->nv; k++) vec[k] = L->all_pars[L->par_idx[k]];
  /* runLma (477-530) with lmaStep (534-637) */
  const int nv = L->nv;
  static double fx[LMA_MAX_SAMPLES + 2], jt[LMA_NPAR * (LMA_MAX_SAMPLES + 2)];
  static double fx1[LMA_MAX_SAMPLES + 2], jt1[LMA_NPAR * (LMA_MAX_SAMPLES + 2)];
  lma_fx_jt(L, vec, fx, jt);
  double last_rms = lma_rms(L, fx, NULL);
  const double initial_rms = last_rms;
  double lambda = p->lambda_initial;
  int success = 0, done = 0;
  for (int iter = 0; iter < p->num_iter; iter++) {
    double A[LMA_NPAR * LMA_NPAR], b[LMA_NPAR];
    for (int i = 0; i < nv; i++) {
      for (int j = i; j < nv; j++) {
        double d = 0.0;
        for (int k = 0; k < npt; k++) d += L->weights[k] * jt[i * npt + k] * jt[j * npt + k];
        A[i * nv + j] = d;
        if (i == j) A[i * nv + j] += d * lambda;
        else A[j * nv + i] = d;
      }
      double d = 0.0;
      for (int k = 0; k < npt; k++) d += jt[i * npt + k] * fx[k];
      b[i] = d;
    }
    if (!lma_solve(A, b, nv)) { /* singular: {false, true} */
      success = 0;
      done = 1;
      break;
    }
    double nvec[LMA_NPAR];
    for (int i = 0; i < nv; i++) nvec[i] = vec[i] + b[i];
    lma_fx_jt(L, nvec, fx1, jt1);
    const double rms = lma_rms(L, fx1, NULL);
    if (rms < last_rms) {
      success = 1;
      done = rms >= last_rms * (1.0 - p->rms_diff);
      last_rms = rms;
      memcpy(vec, nvec, sizeof(vec));
      memcpy(fx, fx1, sizeof(double) * npt);
      memcpy(jt, jt1, sizeof(double) * nv * npt);
    } else {
      success = 0;
      done = 0;
    }
    if (done) break;
    if (success) lambda *= p->lambda_scale_good;
    else {
      lambda *= p->lambda_scale_bad;
      if (lambda > p->lambda_max) break;
    }
  }
  if (!success && last_rms < initial_rms) success = 1;
  (void)done;
  if (!success) return 0;
  for (int k = 0; k < nv; k++) L->all_pars[L->par_idx[k]] = vec[k];
  /* getDisparityStrength (149-163) */
  double sum_amp = 0.0, max_amp = 0.0;
  for (int i = 0; i < L->ngroups; i++) sum_amp += L->group_weights[i] * L->all_pars[4 + i];
  for (int i = 0; i < ns; i++)
    if (L->v[i] > max_amp) max_amp = L->v[i];
  if (sum_amp > 1.25 * max_amp) sum_amp = max_amp;
  out[0] = -L->all_pars[0];
  out[1] = sum_amp;
  out[2] = L->all_pars[1];
  out[3] = L->all_pars[3];
  return 1;
}

void or_default_fo_params(or_fo_params *f) {
  /* ImageDttParameters.java:54-63 */
  f->fo_correct = 1; f->fo_far = 0; f->fo_ortho = 1;
  f->fo_min_strength = 0.1; f->fo_min_eff = 0.25; f->fo_min_eff_ratio = 0.65; f->fo_max_hwidth = 3.0;
  f->fo_min_diff = 0.2; f->fo_overcorrection = 0.0; f->fo_lim_overcorr = 2.0;
}

/* Correlation2d.foregroundCorrect (1663-1749) */
void or_foreground_correct(int bg, int ortho, const double dir[4][4], const int valid[4], double full_disp,
                           const or_fo_params *f, double rslt[4]) {
  double mn = NAN, mx = NAN, eff[4], width_d[4];
  int imn = -1, imx = -1, strong[4] = {0, 0, 0, 0};
  for (int i = 0; i < 4; i++) {
    width_d[i] = 0.0;
    if (valid[i]) {
      if (isnan(mn) || (dir[i][0] < mn)) { mn = dir[i][0]; imn = i; }
      if (isnan(mx) || (dir[i][0] > mx)) { mx = dir[i][0]; imx = i; }
      eff[i] = dir[i][1] * (dir[i][2] - dir[i][3]) / (dir[i][2] + dir[i][3]);
      width_d[i] = dir[i][2] + dir[i][3];
      strong[i] = (dir[i][1] >= f->fo_min_strength) && (eff[i] >= f->fo_min_eff);
    } else {
      eff[i] = NAN;
    }
  }
  const int are_ortho = (imn ^ imx) == 1;
  double corr = f->fo_overcorrection * (mx - mn);
  const int isel = bg ? imn : imx, iother = bg ? imx : imn, iortho = isel ^ 1;
  if ((isel < 0) || !strong[isel]) corr = NAN;
  else if (width_d[isel] > f->fo_max_hwidth) corr = NAN;
  else if (eff[isel] / eff[iortho] < f->fo_min_eff_ratio) corr = NAN;
  else {
    if (ortho && !are_ortho) corr = 0.0;
    else if (!strong[iother]) corr = 0.0;
    if (!(mx >= (mn + f->fo_min_diff))) corr = NAN;
  }
  double disp = full_disp;
  if (!isnan(corr)) {
    if (bg) {
      const double lim = full_disp - (full_disp - mn) * f->fo_lim_overcorr;
      disp = fmax(mn - corr, lim);
    } else {
      const double lim = full_disp + (mx - full_disp) * f->fo_lim_overcorr;
      disp = fmin(mx + corr, lim);
    }
  }
  rslt[0] = disp;
  rslt[1] = (isel >= 0) ? eff[isel] : 0.0;
  rslt[2] = mx - mn;
  rslt[3] = are_ortho ? 1.0 : 0.0;
}

/* Correlation2d.mismatchPairsCM (1336-1431) for one pair of quad kind k: {dx, dy, strength} */
static void or_mismatch_cm_pair(const double *c, int k, double xcenter, double radius, double out[3]) {
  const int W = OR_CORR, center = OR_DTT - 1, center_index = (W + 1) * center;
  const int ixc = (int)floor(xcenter + 0.5);
  int icx, icy;
  if (k == 0) { icx = ixc; icy = 0; }
  else if (k == 1) { icx = 0; icy = ixc; }
  else if (k == 2) { icx = ixc; icy = ixc; }
  else { icx = ixc; icy = -ixc; }
  const int iradius = (int)fabs(radius), ir2 = (int)(radius * radius), square = radius < 0;
  double s0 = 0, sx = 0, sy = 0;
  for (int y = -iradius; y <= iradius; y++) {
    const int dy = icy + y;
    if (dy < -center || dy > center) continue;
    for (int x = -iradius; x <= iradius; x++) {
      const int dx = icx + x;
      const double r2 = y * y + x * x;
      if (dx >= -center && dx <= center && (square || r2 <= ir2)) {
        const double d = c[dy * W + dx + center_index];
        if (d > 0.0) { s0 += d; sx += d * dx; sy += d * dy; }
      }
    }
  }
  const double xm = sx / s0, ym = sy / s0;
  const int ixm = isnan(xm) ? 0 : (int)floor(xm + 0.5), iym = isnan(ym) ? 0 : (int)floor(ym + 0.5);  /* Math.round */
  const double sv = c[iym * W + ixm + center_index];
  if (k == 0) { out[0] = xcenter - xm; out[1] = -ym; }
  else if (k == 1) { out[0] = -xm; out[1] = xcenter - ym; }
  else if (k == 2) { out[0] = xcenter - xm; out[1] = xcenter - ym; }
  else { out[0] = xcenter - xm; out[1] = -xcenter - ym; }
  out[2] = sv;
}

/* LU decomposition with partial pivoting of a [n][n] in place (Jama LUDecomposition, as used by
 * Matrix.det / Matrix.solve): returns the determinant, piv the row order */
static double lu_decompose(double *a, int n, int *piv) {
  double det = 1.0;
  for (int i = 0; i < n; i++) piv[i] = i;
  for (int k = 0; k < n; k++) {
    int p = k;
    for (int i = k + 1; i < n; i++)
      if (fabs(a[i * n + k]) > fabs(a[p * n + k])) p = i;
    if (p != k) {
      for (int j = 0; j < n; j++) {
        const double t = a[p * n + j];
        a[p * n + j] = a[k * n + j];
        a[k * n + j] = t;
      }
      const int t = piv[p];
      piv[p] = piv[k];
      piv[k] = t;
      det = -det;
    }
    if (a[k * n + k] != 0.0)
      for (int i = k + 1; i < n; i++) {
        a[i * n + k] /= a[k * n + k];
        for (int j = k + 1; j < n; j++) a[i * n + j] -= a[i * n + k] * a[k * n + j];
      }
  }
  for (int k = 0; k < n; k++) det *= a[k * n + k];
  return det;
}

/* solves with the factors of lu_decompose: b (in original row order) -> x in b */
static void lu_solve(const double *lu, const int *piv, int n, double *b) {
  double x[6];
  for (int i = 0; i < n; i++) x[i] = b[piv[i]];
  for (int k = 0; k < n; k++)
    for (int i = k + 1; i < n; i++) x[i] -= x[k] * lu[i * n + k];
  for (int k = n - 1; k >= 0; k--) {
    x[k] /= lu[k * n + k];
    for (int i = 0; i < k; i++) x[i] -= x[k] * lu[i * n + k];
  }
  for (int i = 0; i < n; i++) b[i] = x[i];
}

/* PolynomialApproximation.normMatix (common/PolynomialApproximation.java:590-598): product of the
 * row norms */
static double row_norm_product(const double *a, int n) {
  double norm = 1.0;
  for (int i = 0; i < n; i++) {
    double d = 0.0;
    for (int j = 0; j < n; j++) d += a[i * n + j] * a[i * n + j];
    norm *= sqrt(d);
  }
  return norm;
}

/* Correlations2dLMA.getMaxXYPoly (Correlations2dLMA.java:641-704) over samples with weight > 0:
 * the weighted least-squares quadric A x^2 + B y^2 + C xy + D x + E y + F
 * (PolynomialApproximation.quadraticApproximation 350-585 with the linear / quadratic
 * determinant-to-norm thresholds 1e-20 / 1e-30 of quadraticMaxV2dX2Y2XY 201-221) and its
 * maximum.  Returns 1 with xyv = {x, y, value} when both fits are well-posed, the stationary
 * point exists and is a maximum with a non-negative value. */
int or_quadratic_max(const double *x, const double *y, const double *v, const double *w, int n, double xyv[3]) {
  if (n <= 0) return 0;
  double S00 = 0, S10 = 0, S01 = 0, S20 = 0, S11 = 0, S02 = 0, S30 = 0, S21 = 0, S12 = 0, S03 = 0;
  double S40 = 0, S31 = 0, S22 = 0, S13 = 0, S04 = 0;
  double Z00 = 0, Z10 = 0, Z01 = 0, Z20 = 0, Z11 = 0, Z02 = 0;
  for (int i = 0; i < n; i++) {
    const double wi = w[i];
    if (!(wi > 0)) continue;
    const double xi = x[i], yi = y[i], x2 = xi * xi, y2 = yi * yi;
    S00 += wi; S10 += wi * xi; S01 += wi * yi; S11 += wi * xi * yi; S20 += wi * x2; S02 += wi * y2;
    const double x3 = x2 * xi, x4 = x3 * xi, y3 = y2 * yi, y4 = y3 * yi;
    S30 += wi * x3; S21 += wi * x2 * yi; S12 += wi * xi * y2; S03 += wi * y3;
    S40 += wi * x4; S31 += wi * x3 * yi; S22 += wi * x2 * y2; S13 += wi * xi * y3; S04 += wi * y4;
    const double wz = wi * v[i];
    Z00 += wz; Z10 += wz * xi; Z01 += wz * yi; Z20 += wz * x2; Z11 += wz * xi * yi; Z02 += wz * y2;
  }
  int piv[6];
  double ml[9] = {S20, S11, S10, S11, S02, S01, S10, S01, S00};
  const double nml = row_norm_product(ml, 3);
  if (nml == 0.0 || fabs(lu_decompose(ml, 3, piv)) / nml < 1.0e-20) return 0;  /* linear fit only */
  double mq[36] = {S40, S22, S31, S30, S21, S20, S22, S04, S13, S12, S03, S02, S31, S13, S22, S21, S12, S11,
                   S30, S12, S21, S20, S11, S10, S21, S03, S12, S11, S02, S01, S20, S02, S11, S10, S01, S00};
  const double nmq = row_norm_product(mq, 6);
  if (nmq == 0.0 || fabs(lu_decompose(mq, 6, piv)) / nmq < 1.0e-30) return 0;  /* linear fit only */
  double co[6] = {Z20, Z02, Z11, Z10, Z01, Z00};
  lu_solve(mq, piv, 6, co);
  const double A = co[0], B = co[1], Cc = co[2], D = co[3], E = co[4], F = co[5];
  double m2[4] = {2 * A, Cc, Cc, 2 * B};
  const double nm2 = row_norm_product(m2, 2);
  if (nm2 == 0.0 || fabs(lu_decompose(m2, 2, piv)) / nm2 < 1.0e-30) return 0;
  double xy[2] = {-D, -E};
  lu_solve(m2, piv, 2, xy);
  const double vmax = A * xy[0] * xy[0] + B * xy[1] * xy[1] + Cc * xy[0] * xy[1] + D * xy[0] + E * xy[1] + F;
  if (vmax < 0.0 || A >= 0.0 || B >= 0.0) return 0;  /* negative strength, or not a maximum */
  xyv[0] = xy[0];
  xyv[1] = xy[1];
  xyv[2] = vmax;
  return 1;
}

/* Correlation2d.mismatchPairs (1434-1503) for one pair of quad kind k: the pair alone as a group
 * (corrLMA with run_poly_instead, 1754-1831, samples weighted by |value|^vasw_pwr) and the
 * quadric's maximum -> {dx, dy, strength}; {NaN, NaN, 0} when the fit fails */
static void or_mismatch_poly_pair(const double *c, int k, double xcenter, double vasw_pwr, const or_lma_params *p,
                                  double out[3]) {
  static or_lma Ls;
  or_lma *L = &Ls;
  memset(L, 0, sizeof(*L));
  double g[OR_CORR * OR_CORR];
  for (int r = 0; r < OR_CORR; r++)
    for (int q = 0; q < OR_CORR; q++)
      g[r * OR_CORR + q] = (k == 1) ? c[q * OR_CORR + r] : ((k == 3) ? c[(OR_CORR - r - 1) * OR_CORR + q]
                                                                      : c[r * OR_CORR + q]);
  or_lma_params pp = *p;
  pp.ortho_vasw_pwr = vasw_pwr;
  lma_add_group(L, g, k >= 2, 1, xcenter, &pp);
  out[0] = out[1] = NAN;
  out[2] = 0.0;
  double m[3];
  if (!or_quadratic_max(L->x, L->y, L->v, L->w, L->ns, m)) return;
  if (k == 0) { out[0] = xcenter - m[0]; out[1] = -m[1]; }
  else if (k == 1) { out[0] = -m[1]; out[1] = xcenter - m[0]; }
  else if (k == 2) { out[0] = xcenter - m[0] + m[1]; out[1] = xcenter - m[0] - m[1]; }
  else { out[0] = xcenter - m[0] + m[1]; out[1] = -xcenter + m[0] + m[1]; }
  out[2] = isnan(m[2]) ? 0.0 : m[2];
}

/* The LMA branch of ImageDtt.tileInterCamCorrs (ImageDtt.java:7497-7560) on one rig tile.
 * rec = {disparity, strength, dx, dy} of the centre-of-mass record.  Where the strength exceeds
 * min_poly_strength, corrLMA of the single horizontal surface (Correlation2d.java:1903-2011: one
 * ortho group, scale 1) runs at xcenter = -disparity; if it converges, use_poly takes its
 * disparity / strength, and the offset of the peak around x = 0 fills dx, dy: single2dPoly
 * (1509-1536, the quadric of the same sampling with |value|^ortho_vasw_pwr weights) or
 * single2dCM (1538-1585, centre of mass within max_corr_radius).  Returns 1 when the LMA ran and
 * converged, 0 otherwise (rec unchanged). */
int or_rig_lma(const double *corr225, const or_lma_params *p, int use_poly, int use_xy_poly, double max_corr_radius,
               double rec[4]) {
  if (isnan(rec[0]) || !(rec[1] > p->min_poly_strength)) return 0;
  const int kind = 0;
  double out[4];
  if (!or_corr_lma(corr225, &kind, 1, -rec[0], p, out, NULL)) return 0;
  if (use_poly) {
    rec[0] = out[0];
    rec[1] = out[1];
  }
  double xy[3];
  if (use_xy_poly) or_mismatch_poly_pair(corr225, 0, 0.0, p->ortho_vasw_pwr, p, xy);
  else or_mismatch_cm_pair(corr225, 0, 0.0, max_corr_radius, xy);
  rec[2] = xy[0];
  rec[3] = xy[1];
  return 1;
}

int or_lma_tile_mismatch(const double *corrs, const int *kind, int np, const or_lma_params *p,
                         const or_fo_params *f, double max_corr_radius, double mismatch_max_diff, double rec[3],
                         double lma[4], double *mism) {
  const or_ly_params ly = {0, 1.0, 1};
  return or_lma_tile_mismatch_ly(corrs, kind, np, p, f, max_corr_radius, mismatch_max_diff, &ly, rec, lma, mism);
}

int or_lma_tile_mismatch_ly(const double *corrs, const int *kind, int np, const or_lma_params *p,
                            const or_fo_params *f, double max_corr_radius, double mismatch_max_diff,
                            const or_ly_params *ly, double rec[3], double lma[4], double *mism) {
  lma[0] = lma[1] = lma[2] = lma[3] = NAN;
  rec[2] = NAN;
  if (mism)
    for (int i = 0; i < np; i++) { mism[3 * i] = NAN; mism[3 * i + 1] = NAN; mism[3 * i + 2] = 0.0; }
  const double cm = rec[0], strength0 = rec[1];
  if (isnan(cm) || !(strength0 > p->min_poly_strength)) return 0;
  double out[4];
  if (!or_corr_lma(corrs, kind, np, -cm, p, out, NULL)) return 0;
  memcpy(lma, out, sizeof(out));
  rec[2] = out[0];
  double disparity = cm, strength = strength0;
  if (p->mix_corr_poly) {
    disparity = out[0];
    strength = out[1];
    rec[0] = disparity;
    rec[1] = strength;
  }
  if ((f->fo_correct && (strength > 0.0)) || mism) {
    /* corr4dirsLMA: one LMA per pair orientation */
    double dir[4][4];
    int valid[4];
    for (int d = 0; d < 4; d++) {
      or_lma_params pd = *p;
      int m = 0;
      for (int i = 0; i < np; i++)
        if (((p->pair_mask >> i) & 1) && kind[i] == d) m |= 1 << i;
      pd.pair_mask = m;
      valid[d] = m && or_corr_lma(corrs, kind, np, -disparity, &pd, dir[d], NULL);
    }
    double mod[4];
    or_foreground_correct(f->fo_far, f->fo_ortho, (const double(*)[4])dir, valid, disparity, f, mod);
    /* the corrected distance is not used while the mismatch is measured */
    if (mod[0] != disparity && !mism && f->fo_correct && strength > f->fo_min_strength) rec[0] = mod[0];
    if (mism && mod[2] <= mismatch_max_diff) {
      /* ImageDtt.java:2349-2405: with ly_poly the quadric maxima; a failed or implausible pair (an
       * offset beyond ly_crazy_poly, its strength then zeroed) sends all pairs to the centre of
       * mass when ly_poly_backup is set */
      int need_cm = 1;
      if (ly->ly_poly) {
        int has_nan = 0;
        for (int i = 0; i < np; i++)
          if (((p->pair_mask >> i) & 1) && kind[i] >= 0 && kind[i] <= 3) {
            double *m = mism + 3 * i;
            or_mismatch_poly_pair(corrs + (size_t)i * OR_CORR * OR_CORR, kind[i], -disparity, max_corr_radius, p,
                                  m);
            if (isnan(m[0]) || isnan(m[1])) has_nan = 1;
            else if (m[2] != 0.0 && (fabs(m[0]) > ly->ly_crazy_poly || fabs(m[1]) > ly->ly_crazy_poly)) {
              m[2] = 0.0;
              has_nan = 1;
            }
          }
        need_cm = ly->ly_poly_backup && has_nan;
      }
      if (need_cm)
        for (int i = 0; i < np; i++)
          if (((p->pair_mask >> i) & 1) && kind[i] >= 0 && kind[i] <= 3)
            or_mismatch_cm_pair(corrs + (size_t)i * OR_CORR * OR_CORR, kind[i], -disparity, max_corr_radius,
                                mism + 3 * i);
    }
  }
  return 1;
}

int or_lma_tile(const double *corrs, const int *kind, int np, const or_lma_params *p, const or_fo_params *f,
                double rec[3], double lma[4]) {
  return or_lma_tile_mismatch(corrs, kind, np, p, f, 3.9, 1.0, rec, lma, NULL);
}
