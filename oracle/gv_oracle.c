/*
 * CPU oracle for the gpuvmem imaging-objective path -- TEST INFRASTRUCTURE.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may load
 * this library; the product path never does.  See gv_oracle.h for the list
 * of reference functions restated here.  Citations are file:line in the
 * gpuvmem repository.
 */
#define _GNU_SOURCE
#include "gv_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* constants as the reference defines them (include/MSFITSIO.cuh:52-54,
 * include/functions.cuh:17-23) */
static const double OR_PI_D = 3.141592653589793238462643383279502884;
static const float OR_PI_F = 3.14159265358979323846f;
static const float OR_LIGHTSPEED = 2.99792458E8f;
#define OR_RPDEG_D (OR_PI_D / 180.0)
static const float OR_RZ = 1.2196698912665045f;

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* freq_to_wavelength / metres_to_lambda, src/MSFITSIO.cu:36-45: the
 * wavelength is a float. */
static inline float or_wavelength(float freq) { return OR_LIGHTSPEED / freq; }

/* hermitianSymmetry, src/functions.cu:2256-2273 */
void or_hermitian(int64_t n, double* uvw, float* vo, float freq) {
  const float lambda = or_wavelength(freq);
  for (int64_t k = 0; k < n; k++) {
    if (uvw[3 * k] > 0.0) {
      uvw[3 * k] *= -1.0;
      uvw[3 * k + 1] *= -1.0;
      vo[2 * k + 1] *= -1.0f;
    }
    uvw[3 * k] = uvw[3 * k] / lambda;
    uvw[3 * k + 1] = uvw[3 * k + 1] / lambda;
    uvw[3 * k + 2] = uvw[3 * k + 2] / lambda;
  }
}

/* Neumaier sum in the element type, src/functions.cu:353-367 */
static float or_neumaier_f(const float* d, int64_t n) {
  if (n <= 0) return 0.0f;
  float sum = d[0], c = 0.0f;
  for (int64_t i = 1; i < n; i++) {
    float t = sum + d[i];
    if (fabsf(sum) >= fabsf(d[i]))
      c += (sum - t) + d[i];
    else
      c += (d[i] - t) + sum;
    sum = t;
  }
  return sum; /* the reference returns the uncompensated sum */
}

/* calculateNoiseAndBeam + calc_sBeam + calc_beamSize,
 * src/functions.cu:1655-1814 (one field, one correlation per channel) */
float or_noise_and_beam(int nchan, const float* freq, const int64_t* chan_off,
                        const double* uvw_m, const float* weight, double* bmaj,
                        double* bmin, double* bpa, float* noise) {
  float sum_weights = 0.0f;
  double s_uu = 0.0, s_vv = 0.0, s_uv = 0.0;
  for (int c = 0; c < nchan; c++) {
    const int64_t o = chan_off[c], n = chan_off[c + 1] - chan_off[c];
    if (n <= 0) continue;
    const float lambda = or_wavelength(freq[c]);
    double luu = 0.0, lvv = 0.0, luv = 0.0;
#pragma omp parallel for reduction(+ : luu, lvv, luv)
    for (int64_t k = 0; k < n; k++) {
      double u = uvw_m[3 * (o + k)] / lambda;
      double v = uvw_m[3 * (o + k) + 1] / lambda;
      double w = weight[o + k];
      luu += u * u * w;
      lvv += v * v * w;
      luv += u * v * w;
    }
    s_uu += luu;
    s_vv += lvv;
    s_uv += luv;
    sum_weights += or_neumaier_f(weight + o, n);
  }
  float variance = 0.0f;
  if (sum_weights > 0.0f) {
    s_uu /= sum_weights;
    s_vv /= sum_weights;
    s_uv /= sum_weights;
    variance = 1.0f / sum_weights;
  }
  double uv_square = s_uv * s_uv;
  double uu_minus_vv = s_uu - s_vv;
  double uu_plus_vv = s_uu + s_vv;
  double sqrt_in = sqrt(uu_minus_vv * uu_minus_vv + 4.0 * uv_square);
  double bx = 1.0 / sqrt(2.0) / OR_PI_D / sqrt(uu_plus_vv - sqrt_in);
  double by = 1.0 / sqrt(2.0) / OR_PI_D / sqrt(uu_plus_vv + sqrt_in);
  double bz = -0.5 * atan2(2.0 * s_uv, uu_minus_vv);
  *bmaj = bx / OR_RPDEG_D;
  *bmin = by / OR_RPDEG_D;
  *bpa = bz / OR_RPDEG_D;
  if (*noise <= 0.0f) *noise = 0.5f * sqrtf(variance);
  return sum_weights;
}

/* GaussianBeam / AiryDiskBeam / attenuation, src/functions.cu:2275-2333
 * (float arithmetic, as the reference) */
float or_attenuation(int i, int j, float xobs, float yobs, double DELTAX,
                     double DELTAY, float freq, float D, float pbf,
                     float cutoff, int primary_beam) {
  const int x0 = (int)xobs, y0 = (int)yobs;
  const float x = (float)((j - x0) * DELTAX * OR_RPDEG_D);
  const float y = (float)((i - y0) * DELTAY * OR_RPDEG_D);
  const float arc = sqrtf(x * x + y * y);
  const float lambda = or_wavelength(freq);
  float atten;
  if (primary_beam == OR_GAUSSIAN) {
    float fwhm = pbf * lambda / D;
    float c = 4.0f * logf(2.0f);
    float r = arc / fwhm;
    atten = expf(-c * r * r);
  } else {
    atten = 1.0f;
    if (arc != 0.0f) {
      float arg = OR_PI_F * arc * D / lambda * (OR_RZ / pbf);
      float b = j1f(arg);
      atten = 4.0f * (b / arg) * (b / arg);
    }
  }
  return arc <= cutoff ? atten : 0.0f;
}

/* total_attenuation + weight_image + noise_image + fg_scale/noise_cut,
 * src/functions.cu:2382-2422, src/mfs.cu:630-645,849-916 */
float or_noise_image(int M, int N, double DELTAX, double DELTAY, float xobs,
                     float yobs, float nu_0, float D, float pbf, float cutoff,
                     int primary_beam, double bmaj_deg, double bmin_deg,
                     float vis_noise, float noise_cut_factor, float* noise_out,
                     float* noise_cut_abs) {
  const double bmaj_pix = bmaj_deg / fabs(DELTAX);
  const double bmin_pix = bmin_deg / fabs(DELTAX);
  const float noise_jypix =
      (float)(vis_noise / (OR_PI_D * bmaj_pix * bmin_pix / (4.0 * logf(2.0f))));
  float max_w = -FLT_MAX;
  for (int i = 0; i < N; i++)
    for (int j = 0; j < M; j++) {
      float a = or_attenuation(i, j, xobs, yobs, DELTAX, DELTAY, nu_0, D, pbf,
                               cutoff, primary_beam);
      float w = a * a;
      noise_out[(int64_t)N * i + j] = w;
      if (w > max_w) max_w = w;
    }
  const float nsq = noise_jypix * noise_jypix;
  float nmin = FLT_MAX;
  for (int64_t p = 0; p < (int64_t)M * N; p++) {
    float nw = (noise_out[p] / max_w) / nsq;
    float v = sqrtf(1.0f / nw);
    noise_out[p] = v;
    if (v < nmin) nmin = v;
  }
  *noise_cut_abs = noise_cut_factor * nmin;
  return nmin;
}

/* clip2IWNoise, src/functions.cu:2694-2719 via linkClipWNoise2I :4594 */
void or_clip(const or_problem* p, float* img, int flag_opt) {
  const int64_t MN = (int64_t)p->M * p->N;
  for (int64_t q = 0; q < MN; q++) {
    if (p->noise[q] > p->noise_cut) {
      img[q] = p->eta > 0.0f ? 0.0f : (float)(-1.0 * p->eta * p->minpix);
      img[MN + q] = 0.0f;
    } else if (img[q] < p->threshold && flag_opt > 0) {
      img[MN + q] = 0.0f;
    }
  }
}

/* ---- FP64 radix-2 FFT, cuFFT CUFFT_INVERSE convention ------------------ */
static void or_fft1d(int n, double* re, double* im) {
  /* bit reversal */
  for (int i = 1, j = 0; i < n; i++) {
    int bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      double t = re[i]; re[i] = re[j]; re[j] = t;
      t = im[i]; im[i] = im[j]; im[j] = t;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    const int half = len >> 1;
    for (int k = 0; k < half; k++) {
      double s, c;
      sincos(2.0 * OR_PI_D * k / len, &s, &c); /* exp(+i 2 pi k/len) */
      for (int b = 0; b < n; b += len) {
        const int a0 = b + k, a1 = b + k + half;
        double tr = re[a1] * c - im[a1] * s;
        double ti = re[a1] * s + im[a1] * c;
        re[a1] = re[a0] - tr;
        im[a1] = im[a0] - ti;
        re[a0] += tr;
        im[a0] += ti;
      }
    }
  }
}

void or_fft2d_inverse(int n, double* data) {
#pragma omp parallel
  {
    double* re = (double*)malloc(sizeof(double) * n);
    double* im = (double*)malloc(sizeof(double) * n);
#pragma omp for
    for (int r = 0; r < n; r++) {
      for (int s = 0; s < n; s++) {
        re[s] = data[2 * ((int64_t)r * n + s)];
        im[s] = data[2 * ((int64_t)r * n + s) + 1];
      }
      or_fft1d(n, re, im);
      for (int s = 0; s < n; s++) {
        data[2 * ((int64_t)r * n + s)] = re[s];
        data[2 * ((int64_t)r * n + s) + 1] = im[s];
      }
    }
#pragma omp for
    for (int s = 0; s < n; s++) {
      for (int r = 0; r < n; r++) {
        re[r] = data[2 * ((int64_t)r * n + s)];
        im[r] = data[2 * ((int64_t)r * n + s) + 1];
      }
      or_fft1d(n, re, im);
      for (int r = 0; r < n; r++) {
        data[2 * ((int64_t)r * n + s)] = re[r];
        data[2 * ((int64_t)r * n + s) + 1] = im[r];
      }
    }
    free(re);
    free(im);
  }
}

/* calculateInu + apply_beam2I + FFT2D + phase_rotate for one channel:
 * src/functions.cu:3939-3966, 2424-2444, 2153-2178, 2483-2518 */
static void or_channel_grid(const or_problem* p, int c, const float* img,
                            double* grid) {
  const int M = p->M, N = p->N;
  const int64_t MN = (int64_t)M * N;
  const float nu = p->freq[c];
  const double nudiv = (double)(nu / p->nu_0);
  const double floorv = (double)(-1.0f * p->eta * p->minpix);
#pragma omp parallel for
  for (int i = 0; i < N; i++)
    for (int j = 0; j < M; j++) {
      const int64_t q = (int64_t)N * i + j;
      double inu = (double)img[q] * pow(nudiv, (double)img[MN + q]);
      if (inu < floorv) inu = floorv;
      const float a = or_attenuation(i, j, p->xobs, p->yobs, p->DELTAX,
                                     p->DELTAY, nu, p->antenna_diameter,
                                     p->pb_factor, p->pb_cutoff,
                                     p->primary_beam);
      grid[2 * q] = inu * a * p->fg_scale;
      /* apply_GCF, src/functions.cu:2468 (gridded data) */
      if (p->gcf) grid[2 * q] *= (double)p->gcf[q];
      grid[2 * q + 1] = 0.0;
    }
  or_fft2d_inverse(N, grid);
  const double upix = (double)p->xobs / (double)M;
  const double vpix = (double)p->yobs / (double)N;
#pragma omp parallel for
  for (int i = 0; i < N; i++)
    for (int j = 0; j < M; j++) {
      const double u = upix * (j < M / 2 ? j : j - M);
      const double v = vpix * (i < N / 2 ? i : i - N);
      double s, co;
      sincos(-2.0 * OR_PI_D * (u + v), &s, &co);
      const int64_t q = (int64_t)N * i + j;
      const double gr = grid[2 * q], gi = grid[2 * q + 1];
      grid[2 * q] = gr * co - gi * s;
      grid[2 * q + 1] = gr * s + gi * co;
    }
}

/* vis_mod, src/functions.cu:2557-2609: returns 0 when out of grid */
static int or_bilinear(const or_problem* p, const double* grid, double u,
                       double v, double* vm) {
  const long N = p->N;
  const double deltau = 1.0 / (p->M * (OR_RPDEG_D * p->DELTAX));
  const double deltav = 1.0 / (p->N * (OR_RPDEG_D * p->DELTAY));
  double ux = u / deltau, uy = v / deltav;
  if (ux < 0.0) ux += N;
  if (uy < 0.0) uy += N;
  const int i1 = (int)floor(ux);
  const int i2 = (i1 + 1) % N;
  const double du = ux - i1;
  const int j1 = (int)floor(uy);
  const int j2 = (j1 + 1) % N;
  const double dv = uy - j1;
  if (!(i1 >= 0 && i1 < N && j1 >= 0 && j1 < N)) return 0;
  const double* v11 = grid + 2 * (N * j1 + i1);
  const double* v12 = grid + 2 * (N * j2 + i1);
  const double* v21 = grid + 2 * (N * j1 + i2);
  const double* v22 = grid + 2 * (N * j2 + i2);
  const double w11 = (1.0 - du) * (1.0 - dv), w12 = (1.0 - du) * dv;
  const double w21 = du * (1.0 - dv), w22 = du * dv;
  vm[0] = w11 * v11[0] + w12 * v12[0] + w21 * v21[0] + w22 * v22[0];
  vm[1] = w11 * v11[1] + w12 * v12[1] + w21 * v21[1] + w22 * v22[1];
  return 1;
}

void or_model_vis(const or_problem* p, const float* img, double* vm) {
  const int64_t MN = (int64_t)p->M * p->N;
  double* grid = (double*)malloc(sizeof(double) * 2 * MN);
  for (int c = 0; c < p->nchan; c++) {
    const int64_t o = p->chan_off[c], n = p->chan_off[c + 1] - o;
    if (n <= 0) continue;
    or_channel_grid(p, c, img, grid);
#pragma omp parallel for
    for (int64_t k = 0; k < n; k++) {
      double m[2] = {0.0, 0.0};
      or_bilinear(p, grid, p->uvw[3 * (o + k)], p->uvw[3 * (o + k) + 1], m);
      vm[2 * (o + k)] = m[0];
      vm[2 * (o + k) + 1] = m[1];
    }
  }
  free(grid);
}

/* chi2(), src/functions.cu:4323-4454 */
double or_chi2(const or_problem* p, float* img, int flag_opt, double* vr) {
  const int64_t MN = (int64_t)p->M * p->N;
  or_clip(p, img, flag_opt);
  double* grid = (double*)malloc(sizeof(double) * 2 * MN);
  double total = 0.0;
  for (int c = 0; c < p->nchan; c++) {
    const int64_t o = p->chan_off[c], n = p->chan_off[c + 1] - o;
    if (n <= 0) continue;
    or_channel_grid(p, c, img, grid);
    double sum = 0.0;
#pragma omp parallel for reduction(+ : sum)
    for (int64_t k = 0; k < n; k++) {
      const int64_t g = o + k;
      double m[2];
      if (or_bilinear(p, grid, p->uvw[3 * g], p->uvw[3 * g + 1], m)) {
        vr[2 * g] = (double)p->vo[2 * g] - m[0];
        vr[2 * g + 1] = (double)p->vo[2 * g + 1] - m[1];
      } else {
        p->weight[g] = 0.0f; /* persistent side effect of vis_mod */
        vr[2 * g] = (double)p->vo[2 * g];
        vr[2 * g + 1] = (double)p->vo[2 * g + 1];
      }
      sum += (double)p->weight[g] *
             (vr[2 * g] * vr[2 * g] + vr[2 * g + 1] * vr[2 * g + 1]);
    }
    if (p->normalize) sum /= (double)n;
    total += sum;
  }
  free(grid);
  return 0.5 * total;
}

/* DChi2, src/functions.cu:3698-3791, FP64 throughout */
void or_dchi2_channel(const or_problem* p, int c, const double* vr,
                      double* out) {
  const int M = p->M, N = p->N;
  const int64_t o = p->chan_off[c], n = p->chan_off[c + 1] - o;
  const int x0 = (int)p->xobs, y0 = (int)p->yobs;
  const float nu = p->freq[c];
#pragma omp parallel for schedule(dynamic, 4)
  for (int i = 0; i < N; i++)
    for (int j = 0; j < M; j++) {
      const int64_t q = (int64_t)N * i + j;
      if (!(p->noise[q] < p->noise_cut)) {
        out[q] = 0.0;
        continue;
      }
      const double x = (j - x0) * p->DELTAX * OR_RPDEG_D;
      const double y = (i - y0) * p->DELTAY * OR_RPDEG_D;
      const double zm1 = sqrt(1.0 - x * x - y * y) - 1.0;
      const float a = or_attenuation(i, j, p->xobs, p->yobs, p->DELTAX,
                                     p->DELTAY, nu, p->antenna_diameter,
                                     p->pb_factor, p->pb_cutoff,
                                     p->primary_beam);
      double s = 0.0;
      for (int64_t k = 0; k < n; k++) {
        const int64_t g = o + k;
        const double w = p->weight[g];
        if (w == 0.0) continue;
        const double ph = 2.0 * OR_PI_D *
                          (x * p->uvw[3 * g] + y * p->uvw[3 * g + 1] +
                           zm1 * p->uvw[3 * g + 2]);
        double sn, cs;
        sincos(ph, &sn, &cs);
        s += w * (vr[2 * g] * cs + vr[2 * g + 1] * sn);
      }
      s *= (double)p->fg_scale * (double)a;
      /* the GCF variant of DChi2, src/functions.cu:3793-3888 */
      if (p->gcf) s *= (double)p->gcf[q];
      if (p->normalize) s /= (double)n;
      out[q] = -s;
    }
}

void or_dchi2_pixels(const or_problem* p, int c, const double* vr, int npix,
                     const int64_t* pix, double* out) {
  const int64_t o = p->chan_off[c], n = p->chan_off[c + 1] - o;
  const int x0 = (int)p->xobs, y0 = (int)p->yobs;
  for (int t = 0; t < npix; t++) {
    const int i = (int)(pix[t] / p->N), j = (int)(pix[t] % p->N);
    const double x = (j - x0) * p->DELTAX * OR_RPDEG_D;
    const double y = (i - y0) * p->DELTAY * OR_RPDEG_D;
    const double zm1 = sqrt(1.0 - x * x - y * y) - 1.0;
    double s = 0.0;
#pragma omp parallel for reduction(+ : s)
    for (int64_t k = 0; k < n; k++) {
      const int64_t g = o + k;
      const double w = p->weight[g];
      if (w == 0.0) continue;
      const double ph = 2.0 * OR_PI_D *
                        (x * p->uvw[3 * g] + y * p->uvw[3 * g + 1] + zm1 * p->uvw[3 * g + 2]);
      double sn, cs;
      sincos(ph, &sn, &cs);
      s += w * (vr[2 * g] * cs + vr[2 * g + 1] * sn);
    }
    out[t] = s;
  }
}

/* dchi2(), src/functions.cu:4456-4558, with DChi2_total_I_nu_0 /
 * DChi2_total_alpha, src/functions.cu:3968-4024 */
void or_dchi2(const or_problem* p, const float* img, const double* vr,
              int flag_opt, double* result) {
  const int64_t MN = (int64_t)p->M * p->N;
  double* tmp = (double*)malloc(sizeof(double) * MN);
  for (int c = 0; c < p->nchan; c++) {
    if (p->chan_off[c + 1] - p->chan_off[c] <= 0) continue;
    or_dchi2_channel(p, c, vr, tmp);
    const double nudiv = (double)(p->freq[c] / p->nu_0);
    for (int64_t q = 0; q < MN; q++) {
      if (!(p->noise[q] < p->noise_cut)) continue;
      const double i0 = img[q], al = img[MN + q];
      const double pw = pow(nudiv, al);
      if (flag_opt % 2 == 0) {
        result[q] += tmp[q] * pw;
      } else {
        if (i0 > (double)p->threshold)
          result[MN + q] += tmp[q] * (i0 * pw * p->fg_scale * log(nudiv));
      }
    }
  }
  free(tmp);
}

/* ---- priors, src/functions.cu:2878-3545 ------------------------------ */
#define PIX(r, cc) ((double)I[(int64_t)N * (r) + (cc)])

double or_prior_value(const or_problem* p, const or_term* t, const float* img) {
  const int N = p->N;
  const int64_t MN = (int64_t)p->M * p->N;
  const float* I = img + MN * t->image_index;
  double sum = 0.0;
#pragma omp parallel for reduction(+ : sum)
  for (int i = 0; i < N; i++)
    for (int j = 0; j < p->M; j++) {
      if (!(p->noise[(int64_t)N * i + j] < p->noise_cut)) continue;
      const double c = PIX(i, j);
      double v = 0.0;
      switch (t->kind) {
        case OR_FI_ENTROPY: /* calculateS :3036 */
          v = c * log(c / t->prior_value + (t->eta + 1.0));
          break;
        case OR_FI_L1: /* calculateL1norm :2882 */
          v = sqrt(c * c + t->epsilon);
          break;
        case OR_FI_TSV: /* calculateTSV :3353 */
          if (i < N - 1 && j < N - 1) {
            double dx = c - PIX(i, j + 1), dy = c - PIX(i + 1, j);
            v = dx * dx + dy * dy;
          } else {
            v = c;
          }
          break;
        case OR_FI_TV: /* calculateTV :3238 */
          if (i < N - 1 && j < N - 1) {
            double r = PIX(i, j + 1), d = PIX(i + 1, j);
            v = sqrt((r - c) * (r - c) + (d - c) * (d - c) + t->epsilon);
          } else {
            v = c;
          }
          break;
        case OR_FI_LAPLACIAN: /* calculateL :3443 */
          if (i > 0 && i < N - 1 && j > 0 && j < N - 1) {
            double dx = PIX(i, j - 1) - 2.0 * c + PIX(i, j + 1);
            double dy = PIX(i - 1, j) - 2.0 * c + PIX(i + 1, j);
            v = 0.5 * (dx + dy) * (dx + dy);
          } else {
            v = c;
          }
          break;
        case OR_FI_GENTROPY: { /* SGVector :3114 (calculateS with G = prior) */
          const double G = t->prior_image[(int64_t)N * i + j];
          v = c * log(c / G + (t->eta + 1.0));
          break;
        }
        case OR_FI_GL1: { /* calculateGL1norm :2954 */
          const double g = t->prior_image[(int64_t)N * i + j];
          v = sqrt(c * c + t->epsilon) / (sqrt(g * g + t->epsilon) + t->epsilon_b);
          break;
        }
        case OR_FI_QUADRATIC: /* calculateQP :3141 */
          if (i > 0 && i < N - 1 && j > 0 && j < N - 1) {
            const double l = PIX(i, j - 1), r = PIX(i, j + 1);
            const double d = PIX(i + 1, j), u = PIX(i - 1, j);
            v = ((c - l) * (c - l) + (c - r) * (c - r) + (c - u) * (c - u) +
                 (c - d) * (c - d)) / 2.0;
          } else {
            v = c;
          }
          break;
        default:
          break;
      }
      sum += v;
    }
  return sum;
}

void or_prior_grad(const or_problem* p, const or_term* t, const float* img,
                   double* out) {
  const int N = p->N;
  const int64_t MN = (int64_t)p->M * p->N;
  const float* I = img + MN * t->image_index;
  const double lam = t->lambda;
#pragma omp parallel for
  for (int i = 0; i < N; i++)
    for (int j = 0; j < p->M; j++) {
      const int64_t q = (int64_t)N * i + j;
      double g = 0.0;
      if (p->noise[q] < p->noise_cut) {
        const double c = PIX(i, j);
        const int inner = i > 0 && i < N - 1 && j > 0 && j < N - 1;
        switch (t->kind) {
          case OR_FI_ENTROPY: /* calculateDS :3057 */
            g = log(c / t->prior_value + (t->eta + 1.0)) +
                1.0 / (1.0 + ((t->eta + 1.0) * t->prior_value) / c);
            break;
          case OR_FI_L1: /* calculateDNormL1 :2917 */
            g = c / sqrt(c * c + t->epsilon);
            break;
          case OR_FI_TSV: /* calculateDTSV :3395 */
            g = inner ? 8.0 * c - 2.0 * (PIX(i - 1, j) + PIX(i, j - 1) +
                                         PIX(i + 1, j) + PIX(i, j + 1))
                      : c;
            break;
          case OR_FI_TV: /* calculateDTV :3284 */
            if (inner) {
              const double d = PIX(i + 1, j), u = PIX(i - 1, j);
              const double r = PIX(i, j + 1), l = PIX(i, j - 1);
              const double dl = PIX(i + 1, j - 1), ru = PIX(i - 1, j + 1);
              const double e = t->epsilon;
              g = (2.0 * c - r - d) /
                      sqrt((c - r) * (c - r) + (c - d) * (c - d) + e) +
                  (c - l) / sqrt((l - c) * (l - c) + (l - dl) * (l - dl) + e) +
                  (c - u) / sqrt((u - ru) * (u - ru) + (u - c) * (u - c) + e);
            } else {
              g = c;
            }
            break;
          case OR_FI_LAPLACIAN: /* calculateDL :3488 (sign of d-r-u-l kept) */
            if (i > 1 && i < N - 2 && j > 1 && j < N - 2) {
              g = 20.0 * c -
                  8.0 * (PIX(i + 1, j) - PIX(i, j + 1) - PIX(i - 1, j) -
                         PIX(i, j - 1)) +
                  2.0 * (PIX(i + 1, j - 1) + PIX(i + 1, j + 1) +
                         PIX(i - 1, j - 1) + PIX(i - 1, j + 1)) +
                  PIX(i + 2, j) + PIX(i, j + 2) + PIX(i - 2, j) + PIX(i, j - 2);
            } else {
              g = 0.0;
            }
            break;
          case OR_FI_GENTROPY: { /* DSG :3131 (calculateDS with G = prior) */
            const double G = t->prior_image[q];
            g = log(c / G + (t->eta + 1.0)) + 1.0 / (1.0 + ((t->eta + 1.0) * G) / c);
            break;
          }
          case OR_FI_GL1: { /* calculateDGNormL1 :2993 */
            const double pr = t->prior_image[q];
            g = c / (sqrt(c * c + t->epsilon) *
                     (sqrt(pr * pr + t->epsilon) + t->epsilon_b));
            break;
          }
          case OR_FI_QUADRATIC: /* calculateDQ :3190 (its 4c - d + u + r + l kept) */
            g = inner ? 2.0 * (4.0 * c - PIX(i + 1, j) + PIX(i - 1, j) + PIX(i, j + 1) +
                               PIX(i, j - 1))
                      : c;
            break;
          default:
            break;
        }
        g *= lam;
      }
      out[q] = g;
    }
}
#undef PIX

/* ---- ObjectiveFunction, include/classes/objectivefunction.cuh:15-57 ---- */
double or_calc_function(or_state* s, float* img) {
  const or_problem* p = s->p;
  double total = 0.0;
  for (int t = 0; t < p->nterms; t++) {
    const or_term* tm = &p->terms[t];
    double v = 0.0;
    if (tm->kind == OR_FI_CHI2) {
      v = or_chi2(p, img, s->flag_opt, s->vr);
      s->last_fi[t] = v;
      v *= tm->lambda;
    } else {
      /* SEntropy & co evaluate only if iter > 0 && lambda != 0 (:4734) */
      if (s->iteration > 0 && tm->lambda != 0.0f) v = or_prior_value(p, tm, img);
      s->last_fi[t] = v;
      v *= tm->lambda;
    }
    total += v;
  }
  s->nevals++;
  return total;
}

void or_calc_gradient(or_state* s, float* img, float* xi, int iter) {
  const or_problem* p = s->p;
  const int64_t MN = (int64_t)p->M * p->N;
  double* dphi = (double*)calloc(2 * MN, sizeof(double));
  double* tmp = (double*)malloc(sizeof(double) * MN);
  s->iteration = iter;
  for (int t = 0; t < p->nterms; t++) {
    const or_term* tm = &p->terms[t];
    if (tm->kind == OR_FI_CHI2) {
      /* Chi2::addToDphi overwrites dphi (src/chi2.cu:60-70) */
      memset(dphi, 0, sizeof(double) * 2 * MN);
      or_dchi2(p, img, s->vr, s->flag_opt, dphi);
    } else {
      if (!(iter > 0 && tm->lambda != 0.0f && s->flag_opt % 2 == tm->image_index))
        continue;
      or_prior_grad(p, tm, img, tmp);
      /* TVariation::addToDphi always uses plane 0 (src/totalvariation.cu:48) */
      const int add = tm->kind == OR_FI_TV ? 0 : tm->image_to_add;
      for (int64_t q = 0; q < MN; q++) dphi[MN * add + q] += tmp[q];
    }
  }
  for (int64_t q = 0; q < 2 * MN; q++) xi[q] = (float)dphi[q];
  free(dphi);
  free(tmp);
  s->ngrads++;
}

/* ---- line search ------------------------------------------------------ */
typedef struct {
  or_state* s;
  const float* pcom;
  const float* xicom;
  float* xt;
  int positivity;
} or_line;

/* f1dim + evaluateXt, src/f1dim.cu:49-80, src/functions.cu:2832-2864 */
static float or_f1dim(or_line* L, float x) {
  const or_problem* p = L->s->p;
  const int64_t MN = (int64_t)p->M * p->N;
  const double floor_cmp = -1.0 * p->eta * p->minpix;
  const float floor_val = -1.0f * p->eta * p->minpix;
  for (int64_t q = 0; q < MN; q++) {
    float v = fmaf(x, L->xicom[q], L->pcom[q]);
    L->xt[q] = (!L->positivity || v > floor_cmp) ? v : floor_val;
  }
  for (int64_t q = MN; q < 2 * MN; q++) L->xt[q] = fmaf(x, L->xicom[q], L->pcom[q]);
  return (float)or_calc_function(L->s, L->xt);
}

/* SIGN of include/nrutil.h:55 applied to float magnitudes (fabs of a float
 * is a float in the reference's C++) */
#define OR_SIGNF(a, b) ((b) >= 0.0 ? fabsf(a) : -fabsf(a))

/* Golden-section bracketing with parabolic extrapolation (the published
 * bracketing procedure; constants as src/mnbrak.cu:35-37). Host scalars are
 * float, intermediate constants double, as the reference. */
static void or_bracket(or_line* L, float* ax, float* bx, float* cx, float* fa,
                       float* fb, float* fc) {
  const double gold = 1.618034, glimit = 100.0, tiny = 1.0e-20;
  *fa = or_f1dim(L, *ax);
  *fb = or_f1dim(L, *bx);
  if (*fb > *fa) {
    float t = *ax; *ax = *bx; *bx = t;
    t = *fb; *fb = *fa; *fa = t;
  }
  *cx = (float)(*bx + gold * (*bx - *ax));
  *fc = or_f1dim(L, *cx);
  while (*fb > *fc) {
    float r = (*bx - *ax) * (*fb - *fc);
    float q = (*bx - *cx) * (*fb - *fa);
    /* FMAX of include/nrutil.h:28 stores through float temporaries */
    const float aq = fabsf(q - r), at = (float)tiny;
    const float den = aq > at ? aq : at;
    float u = (float)(*bx - ((*bx - *cx) * q - (*bx - *ax) * r) /
                                (2.0 * OR_SIGNF(den, q - r)));
    float ulim = (float)(*bx + glimit * (*cx - *bx));
    float fu;
    if ((*bx - u) * (u - *cx) > 0.0) {
      fu = or_f1dim(L, u);
      if (fu < *fc) {
        *ax = *bx; *bx = u; *fa = *fb; *fb = fu;
        return;
      } else if (fu > *fb) {
        *cx = u; *fc = fu;
        return;
      }
      u = (float)(*cx + gold * (*cx - *bx));
      fu = or_f1dim(L, u);
    } else if ((*cx - u) * (u - ulim) > 0.0) {
      fu = or_f1dim(L, u);
      if (fu < *fc) {
        *bx = *cx; *cx = u; u = (float)(*cx + gold * (*cx - *bx));
        *fb = *fc; *fc = fu; fu = or_f1dim(L, u);
      }
    } else if ((u - ulim) * (ulim - *cx) >= 0.0) {
      u = ulim;
      fu = or_f1dim(L, u);
    } else {
      u = (float)(*cx + gold * (*cx - *bx));
      fu = or_f1dim(L, u);
    }
    *ax = *bx; *bx = *cx; *cx = u;
    *fa = *fb; *fb = *fc; *fc = fu;
  }
}

/* Brent's parabolic-interpolation / golden-section minimiser (Brent 1973);
 * constants and float host scalars as src/brent.cu:35-121. */
static float or_brent(or_line* L, float ax, float bx, float cx, float tol,
                      float* xmin) {
  const double cgold = 0.3819660, zeps = 1.0e-10;
  float a = ax < cx ? ax : cx, b = ax > cx ? ax : cx;
  float d = 0.0f, e = 0.0f, etemp, fu, fv, fw, fx, pp, q, r, tol1, tol2, u, v,
        w, x, xm;
  x = w = v = bx;
  fw = fv = fx = or_f1dim(L, x);
  for (int it = 1; it <= 500; it++) {
    xm = (float)(0.5 * (a + b));
    tol1 = (float)(tol * fabs(x) + zeps);
    tol2 = (float)(2.0 * tol1);
    if (fabs(x - xm) <= (tol2 - 0.5 * (b - a))) {
      *xmin = x;
      return fx;
    }
    if (fabs(e) > tol1) {
      r = (x - w) * (fx - fv);
      q = (x - v) * (fx - fw);
      pp = (x - v) * q - (x - w) * r;
      q = (float)(2.0 * (q - r));
      if (q > 0.0) pp = -pp;
      q = fabsf(q);
      etemp = e;
      e = d;
      if (fabs(pp) >= fabs(0.5 * q * etemp) || pp <= q * (a - x) ||
          pp >= q * (b - x)) {
        e = x >= xm ? a - x : b - x;
        d = (float)(cgold * e);
      } else {
        d = pp / q;
        u = x + d;
        if (u - a < tol2 || b - u < tol2) d = OR_SIGNF(tol1, xm - x);
      }
    } else {
      e = x >= xm ? a - x : b - x;
      d = (float)(cgold * e);
    }
    u = fabsf(d) >= tol1 ? x + d : x + OR_SIGNF(tol1, d);
    fu = or_f1dim(L, u);
    if (fu <= fx) {
      if (u >= x) a = x; else b = x;
      v = w; w = x; x = u;
      fv = fw; fw = fx; fx = fu;
    } else {
      if (u < x) a = u; else b = u;
      if (fu <= fw || w == x) {
        v = w; w = u; fv = fw; fw = fu;
      } else if (fu <= fv || v == x || v == w) {
        v = u; fv = fu;
      }
    }
  }
  *xmin = x;
  return fx;
}

/* linmin + newP, src/linmin.cu:52-110, src/functions.cu:2779-2812 */
static float or_linmin(or_state* s, float* img, float* xi, int positivity) {
  const or_problem* p = s->p;
  const int64_t MN = (int64_t)p->M * p->N;
  float* pcom = (float*)malloc(sizeof(float) * 2 * MN);
  float* xicom = (float*)malloc(sizeof(float) * 2 * MN);
  float* xt = (float*)malloc(sizeof(float) * 2 * MN);
  memcpy(pcom, img, sizeof(float) * 2 * MN);
  memcpy(xicom, xi, sizeof(float) * 2 * MN);
  or_line L = {s, pcom, xicom, xt, positivity};
  float ax = 0.0f, xx = 1.0f, bx, fa, fx, fb, xmin;
  or_bracket(&L, &ax, &xx, &bx, &fa, &fx, &fb);
  float fret = or_brent(&L, ax, xx, bx, 1.0e-7f, &xmin);
  if (getenv("GV_VERBOSE") && getenv("GV_VERBOSE")[0] == '1')
    fprintf(stderr, "oracle: Alpha for linear minimization = %.9g (f = %.9g)\n", xmin, fret);
  const double floor_cmp = -1.0 * p->eta * p->minpix;
  const float floor_val = -1.0f * p->eta * p->minpix;
  for (int64_t q = 0; q < MN; q++) {
    xi[q] *= xmin;
    if (!positivity) {
      img[q] += xi[q];
    } else if (img[q] + xi[q] > floor_cmp) {
      img[q] += xi[q];
    } else {
      img[q] = floor_val;
      xi[q] = 0.0f;
    }
  }
  for (int64_t q = MN; q < 2 * MN; q++) {
    xi[q] *= xmin;
    img[q] += xi[q];
  }
  free(pcom);
  free(xicom);
  free(xt);
  return fret;
}

/* ConjugateGradient::optimize, src/frprmn.cu:85-195 */
void or_frprmn(or_state* s, float* img, int total_iterations, float ftol,
               float gtol, int positivity, or_opt_report* rep) {
  const or_problem* p = s->p;
  const int64_t MN = (int64_t)p->M * p->N, PMN = 2 * MN;
  float* xi = (float*)calloc(PMN, sizeof(float));
  float* g = (float*)calloc(PMN, sizeof(float));
  float* h = (float*)calloc(PMN, sizeof(float));
  memset(rep, 0, sizeof(*rep));
  float fp = (float)or_calc_function(s, img);
  or_calc_gradient(s, img, xi, 0);
  for (int64_t q = 0; q < PMN; q++) {
    g[q] = -xi[q];
    xi[q] = h[q] = g[q];
  }
  int it;
  for (it = 1; it <= total_iterations; it++) {
    rep->iterations = it;
    float fret = or_linmin(s, img, xi, positivity);
    if (2.0f * fabsf(fret - fp) <= ftol * (fabsf(fret) + fabsf(fp) + 1.0e-10)) {
      rep->exit_reason = 1;
      break;
    }
    fp = (float)or_calc_function(s, img);
    or_calc_gradient(s, img, xi, it);
    const float den = fp > 1.0f ? fp : 1.0f;
    float gmax = FLT_MIN;
    for (int64_t q = 0; q < PMN; q++) {
      float t = fabsf(xi[q]) * fmaxf(fabsf(img[q]), 1.0f) / den;
      if (t > gmax) gmax = t;
    }
    if (gmax < gtol) {
      rep->exit_reason = 2;
      break;
    }
    double gg = 0.0, dgg = 0.0;
    for (int64_t q = 0; q < PMN; q++) {
      gg += (double)(g[q] * g[q]);
      dgg += (double)((xi[q] + g[q]) * xi[q]);
    }
    if ((float)gg == 0.0f) {
      rep->exit_reason = 3;
      break;
    }
    float gam = fmaxf(0.0f, (float)dgg / (float)gg);
    for (int64_t q = 0; q < PMN; q++) {
      g[q] = -xi[q];
      xi[q] = h[q] = fmaf(gam, h[q], g[q]);
    }
  }
  rep->f_final = (float)or_calc_function(s, img);
  rep->nevals = s->nevals;
  rep->ngrads = s->ngrads;
  free(xi);
  free(g);
  free(h);
}

/* LBFGS::optimize + LBFGS_recursion, src/lbfgs.cu:99-341, including the
 * reference's ring addressing (getDot_LBFGS_ff / calculateSandY use slot
 * offset M*N*image*k + M*N*image, updateQ uses M*N*image + M*N*k). */
static double or_dot(const float* a, const float* b, int64_t n) {
  double s = 0.0;
  for (int64_t q = 0; q < n; q++) s += (double)(a[q] * b[q]);
  return s;
}

void or_lbfgs(or_state* s, float* img, int total_iterations, int K, float ftol,
              float gtol, int positivity, or_opt_report* rep) {
  const or_problem* p = s->p;
  const int64_t MN = (int64_t)p->M * p->N, PMN = 2 * MN;
  const int P = 2;
  float* xi = (float*)calloc(PMN, sizeof(float));
  float* xi_old = (float*)calloc(PMN, sizeof(float));
  float* p_old = (float*)calloc(PMN, sizeof(float));
  float* d_y = (float*)calloc((size_t)MN * K * P, sizeof(float));
  float* d_s = (float*)calloc((size_t)MN * K * P, sizeof(float));
  float* d_q = (float*)calloc(PMN, sizeof(float));
  float* d_r = (float*)calloc(PMN, sizeof(float));
  float* alpha = (float*)calloc((size_t)P * K, sizeof(float));
  memset(rep, 0, sizeof(*rep));
  float fp = (float)or_calc_function(s, img);
  or_calc_gradient(s, img, xi, 0);
  for (int64_t q = 0; q < PMN; q++) xi[q] *= -1.0f;
  int it;
  for (it = 1; it <= total_iterations; it++) {
    rep->iterations = it;
    memcpy(p_old, img, sizeof(float) * PMN);
    memcpy(xi_old, xi, sizeof(float) * PMN);
    float fret = or_linmin(s, img, xi, positivity);
    float mx = fabsf(fret);
    if (fabsf(fp) > mx) mx = fabsf(fp);
    if (1.0f > mx) mx = 1.0f;
    if ((fp - fret) / mx <= ftol) {
      rep->exit_reason = 1;
      break;
    }
    float max_per_it = 0.0f, m = FLT_MIN;
    for (int64_t q = 0; q < PMN; q++) m = fmaxf(m, fabsf(xi[q]));
    max_per_it = fmaxf(max_per_it, m);
    if (max_per_it <= gtol) {
      rep->exit_reason = 2;
      break;
    }
    fp = (float)or_calc_function(s, img);
    or_calc_gradient(s, img, xi, it);
    const int slot = (it - 1) % K;
    for (int im = 0; im < P; im++) {
      float* yv = d_y + MN * im * slot + MN * im;
      float* sv = d_s + MN * im * slot + MN * im;
      for (int64_t q = 0; q < MN; q++) {
        yv[q] = xi[MN * im + q] - (-1.0f * xi_old[MN * im + q]);
        sv[q] = img[MN * im + q] - p_old[MN * im + q];
      }
    }
    /* LBFGS_recursion */
    const int par_M = K < it ? K : it;
    const int lit = slot;
    memcpy(d_q, xi, sizeof(float) * PMN);
    memset(d_r, 0, sizeof(float) * PMN);
    memset(alpha, 0, sizeof(float) * P * K);
    for (int im = 0; im < P; im++) {
      for (int k = par_M - 1; k >= 0; k--) {
        const float* yk = d_y + MN * im * k + MN * im;
        const float* sk = d_s + MN * im * k + MN * im;
        float rho_den = (float)or_dot(yk, sk, MN);
        float rho = rho_den != 0.0f ? (float)(1.0 / rho_den) : 0.0f;
        alpha[im * K + k] = rho * (float)or_dot(sk, d_q + MN * im, MN);
        const float* yq = d_y + MN * im + MN * k;
        const float a = -alpha[im * K + k];
        for (int64_t q = 0; q < MN; q++)
          d_q[MN * im + q] = fmaf(a, yq[q], d_q[MN * im + q]);
      }
    }
    float sy_yy = 0.0f;
    for (int im = 0; im < P; im++) {
      const float* yk = d_y + MN * im * lit + MN * im;
      const float* sk = d_s + MN * im * lit + MN * im;
      float sy = (float)or_dot(yk, sk, MN);
      float yy = (float)or_dot(yk, yk, MN);
      if (yy != 0.0f) sy_yy += sy / yy;
    }
    for (int im = 0; im < P; im++) {
      for (int64_t q = 0; q < MN; q++) d_r[MN * im + q] = d_q[MN * im + q] * sy_yy;
      for (int k = 0; k < par_M; k++) {
        const float* yk = d_y + MN * im * k + MN * im;
        const float* sk = d_s + MN * im * k + MN * im;
        float rho_den = (float)or_dot(yk, sk, MN);
        float rho = rho_den != 0.0f ? 1.0f / rho_den : 0.0f;
        float beta = rho * (float)or_dot(yk, d_r + MN * im, MN);
        const float* sq = d_s + MN * im + MN * k;
        const float a = alpha[im * K + k] - beta;
        for (int64_t q = 0; q < MN; q++)
          d_r[MN * im + q] = fmaf(a, sq[q], d_r[MN * im + q]);
      }
    }
    for (int64_t q = 0; q < PMN; q++) xi[q] = -d_r[q];
  }
  rep->f_final = (float)or_calc_function(s, img);
  rep->nevals = s->nevals;
  rep->ngrads = s->ngrads;
  free(xi); free(xi_old); free(p_old); free(d_y); free(d_s);
  free(d_q); free(d_r); free(alpha);
}
