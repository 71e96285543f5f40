// Runs the reference's own convolutional gridding (do_gridding,
// src/functions.cu:1339-1653) and convolution-kernel / GCF tables
// (src/pillBox2D.cu, src/gaussian2D.cu, src/sinc2D.cu, src/gaussianSinc2D.cu,
// src/pswf_12D.cu), compiled from the reference sources in place by
// build_grid.sh, on arrays read from a binary file, for golden vectors and
// CPU timings.  The kernel set-up follows MFS::configure
// (src/mfs.cu:493-525): setSigmas(|deltau|, |deltav|), buildKernel(),
// initializeGCF(M, N, |deltax|, |deltay|).  Host code only: no GPU is used
// (the kernel classes' device copies fail and are ignored).
//
// Input file (little endian):
//   int32 kind (0 PillBox2D(), 1 Gaussian2D(m,n), 2 Sinc2D(m,n),
//   3 GaussianSinc2D(m,n), 4 PSWF_12D(m,n)), int32 m, int32 n,
//   int32 threads, int64 M, int64 N, double DELTAX, double DELTAY (degrees),
//   int32 C, then per channel: float freq, int64 nvis, double uvw[3*nvis],
//   float weight[nvis], float Vo[2*nvis]
// Output file: int32 km, kn, support_x, support_y, float kernel[km*kn],
//   int32 has_gcf, float gcf[M*N] (if has_gcf), then per channel int64 count,
//   double uvw[3*count], float Vo[2*count], float weight[count]; then double
//   seconds spent in do_gridding.
#include <omp.h>

#include <chrono>
#include <cstdio>
#include <vector>

#include "functions.cuh"
#include "gaussian2D.cuh"
#include "gaussianSinc2D.cuh"
#include "pillBox2D.cuh"
#include "pswf_12D.cuh"
#include "sinc2D.cuh"

// globals the reference's functions.cu refers to (types as its extern
// declarations give them); only M, N, DELTAX, DELTAY, deltau, deltav are used
long M, N;
int iterations, iter, image_count, status_mod_in, flag_opt, num_gpus = 1, multigpu, firstgpu,
    reg_term;
float *device_dphi, *device_S, *device_dchi2_total, *device_dS, *device_noise_image;
float noise_jypix, noise_cut, MINPIX, minpix, random_probability, eta;
dim3 threadsPerBlockNN, numBlocksNN;
double beam_bmaj, beam_bmin, beam_bpa;
float *initial_values, *penalizators, robust_param;
double ra, dec, DELTAX, DELTAY, deltau, deltav, crpix1, crpix2;
float threshold, nu_0;
int nPenalizators, nMeasurementSets, max_number_vis;
MSDataset* datasets;
varsPerGPU* vars_gpu;
bool verbose_flag, nopositivity, apply_noise, print_images, print_errors, save_model_input,
    radius_mask, modify_weights;
Flags flags;

// src/MSFITSIO.cu:36-51, restated (float wavelength)
__host__ __device__ float freq_to_wavelength(float freq) { return LIGHTSPEED / freq; }
__host__ __device__ double metres_to_lambda(double uvw_metres, float freq) {
  float lambda = freq_to_wavelength(freq);
  return uvw_metres / lambda;
}
__host__ __device__ float distance(float x, float y, float x0, float y0) {
  return sqrtf((x - x0) * (x - x0) + (y - y0) * (y - y0));
}

// referenced by degridding() in functions.cu, which is not run here
__host__ void modelToHost(std::vector<Field>&, MSData, int, int) {}

template <class T>
static bool rd(FILE* f, T* v, size_t n = 1) {
  return fread(v, sizeof(T), n, f) == n;
}

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s input output\n", argv[0]);
    return 2;
  }
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  int kind = 0, km = 7, kn = 7, threads = 1, C = 0;
  bool ok = rd(f, &kind) && rd(f, &km) && rd(f, &kn) && rd(f, &threads) && rd(f, &M) &&
            rd(f, &N) && rd(f, &DELTAX) && rd(f, &DELTAY) && rd(f, &C);
  if (!ok || C < 1) return 3;
  std::vector<Field> fields(1);
  MSData data{};
  data.nfields = 1;
  data.total_frequencies = C;
  data.nstokes = 1;
  Field& fl = fields[0];
  fl.nu.resize(C);
  fl.numVisibilitiesPerFreqPerStoke.assign(C, std::vector<long>(1, 0));
  fl.backup_numVisibilitiesPerFreqPerStoke.assign(C, std::vector<long>(1, 0));
  fl.numVisibilitiesPerFreq.assign(C, 0);
  fl.backup_numVisibilitiesPerFreq.assign(C, 0);
  fl.visibilities.assign(C, std::vector<HVis>(1));
  fl.backup_visibilities.assign(C, std::vector<HVis>(1));
  for (int c = 0; c < C && ok; c++) {
    int64_t n = 0;
    ok = rd(f, &fl.nu[c]) && rd(f, &n);
    fl.numVisibilitiesPerFreqPerStoke[c][0] = (long)n;
    fl.numVisibilitiesPerFreq[c] = (long)n;
    HVis& v = fl.visibilities[c][0];
    v.uvw.resize(n);
    v.weight.resize(n);
    v.Vo.resize(n);
    for (int64_t k = 0; k < n && ok; k++) {
      double t[3];
      ok = rd(f, t, 3);
      v.uvw[k] = make_double3(t[0], t[1], t[2]);
    }
    ok = ok && rd(f, v.weight.data(), (size_t)n);
    for (int64_t k = 0; k < n && ok; k++) {
      float t[2];
      ok = rd(f, t, 2);
      v.Vo[k] = make_cuFloatComplex(t[0], t[1]);
    }
  }
  fclose(f);
  if (!ok) return 4;

  // src/mfs.cu:493-496
  const double deltax = RPDEG_D * DELTAX, deltay = RPDEG_D * DELTAY;
  deltau = 1.0 / (M * deltax);
  deltav = 1.0 / (N * deltay);
  CKernel* ck = nullptr;
  if (kind == 0)
    ck = new PillBox2D();
  else if (kind == 1)
    ck = new Gaussian2D(km, kn);
  else if (kind == 2)
    ck = new Sinc2D(km, kn);
  else if (kind == 3)
    ck = new GaussianSinc2D(km, kn);
  else
    ck = new PSWF_12D(km, kn);
  ck->setSigmas(fabs(deltau), fabs(deltav));
  ck->buildKernel();
  ck->initializeGCF(M, N, fabs(deltax), fabs(deltay));

  const auto t0 = std::chrono::steady_clock::now();
  do_gridding(fields, &data, deltau, deltav, M, N, ck, threads);
  const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

  FILE* o = fopen(argv[2], "wb");
  if (!o) return 5;
  int hdr[4] = {ck->getm(), ck->getn(), ck->getSupportX(), ck->getSupportY()};
  fwrite(hdr, sizeof(int), 4, o);
  std::vector<float> kt = ck->getKernel();
  fwrite(kt.data(), sizeof(float), kt.size(), o);
  std::vector<float> g = ck->getGCFCPU();
  int has_gcf = (g.size() == (size_t)(M * N)) ? 1 : 0;
  fwrite(&has_gcf, sizeof(int), 1, o);
  if (has_gcf) fwrite(g.data(), sizeof(float), g.size(), o);
  for (int c = 0; c < C; c++) {
    const HVis& v = fl.visibilities[c][0];
    int64_t cnt = (int64_t)fl.numVisibilitiesPerFreqPerStoke[c][0];
    fwrite(&cnt, sizeof(int64_t), 1, o);
    for (int64_t k = 0; k < cnt; k++) {
      double t[3] = {v.uvw[k].x, v.uvw[k].y, v.uvw[k].z};
      fwrite(t, sizeof(double), 3, o);
    }
    for (int64_t k = 0; k < cnt; k++) {
      float t[2] = {v.Vo[k].x, v.Vo[k].y};
      fwrite(t, sizeof(float), 2, o);
    }
    fwrite(v.weight.data(), sizeof(float), (size_t)cnt, o);
  }
  fwrite(&sec, sizeof(double), 1, o);
  fclose(o);
  return 0;
}
