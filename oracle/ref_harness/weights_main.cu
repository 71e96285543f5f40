// Runs the reference's own weighting schemes (NaturalWeightingScheme,
// UniformWeightingScheme, BriggsWeightingScheme; src/*weightingscheme.cu,
// compiled from the reference sources in place by build_weights.sh) on
// arrays read from a binary file, for golden vectors and CPU timings.
// Host code only: no GPU is used.
//
// Input file (little endian):
//   int32 scheme (0 natural, 1 uniform, 2 briggs), float robust,
//   int32 threads, int64 M, int64 N, double deltau, double deltav,
//   int32 C, then per channel: float freq, int64 nvis,
//   double uvw[3*nvis], float weight[nvis]
// Output file: per channel float weight[nvis], then double seconds.
#include <omp.h>

#include <chrono>
#include <cstdio>
#include <vector>

#include "briggsweightingscheme.cuh"
#include "naturalweightingscheme.cuh"
#include "uniformweightingscheme.cuh"

// the globals the weighting schemes read (defined by mfs.cu in gpuvmem)
long M, N;
double deltau, deltav;

// src/MSFITSIO.cu:36-45, restated (float wavelength)
__host__ __device__ float freq_to_wavelength(float freq) { return LIGHTSPEED / freq; }
__host__ __device__ double metres_to_lambda(double uvw_metres, float freq) {
  float lambda = freq_to_wavelength(freq);
  return uvw_metres / lambda;
}

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
  int scheme = 0, threads = 1, C = 0;
  float robust = 0.0f;
  bool ok = rd(f, &scheme) && rd(f, &robust) && rd(f, &threads) && rd(f, &M) && rd(f, &N) &&
            rd(f, &deltau) && rd(f, &deltav) && rd(f, &C);
  if (!ok || C < 1) return 3;
  std::vector<MSDataset> d(1);
  d[0].data.nfields = 1;
  d[0].data.total_frequencies = C;
  d[0].data.nstokes = 1;
  d[0].fields.resize(1);
  Field& fl = d[0].fields[0];
  fl.nu.resize(C);
  fl.numVisibilitiesPerFreqPerStoke.assign(C, std::vector<long>(1, 0));
  fl.visibilities.assign(C, std::vector<HVis>(1));
  fl.backup_visibilities.assign(C, std::vector<HVis>(1));
  for (int c = 0; c < C && ok; c++) {
    int64_t n = 0;
    ok = rd(f, &fl.nu[c]) && rd(f, &n);
    fl.numVisibilitiesPerFreqPerStoke[c][0] = (long)n;
    HVis& v = fl.visibilities[c][0];
    v.uvw.resize(n);
    v.weight.resize(n);
    for (int64_t k = 0; k < n && ok; k++) {
      double t[3];
      ok = rd(f, t, 3);
      v.uvw[k] = make_double3(t[0], t[1], t[2]);
    }
    ok = ok && rd(f, v.weight.data(), (size_t)n);
  }
  fclose(f);
  if (!ok) return 4;
  WeightingScheme* w = nullptr;
  if (scheme == 0)
    w = new NaturalWeightingScheme(threads);
  else if (scheme == 1)
    w = new UniformWeightingScheme(threads);
  else {
    w = new BriggsWeightingScheme(threads);
    w->configure(&robust);
  }
  const auto t0 = std::chrono::steady_clock::now();
  w->apply(d);
  const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  FILE* o = fopen(argv[2], "wb");
  if (!o) return 5;
  for (int c = 0; c < C; c++) {
    const HVis& v = fl.visibilities[c][0];
    fwrite(v.weight.data(), sizeof(float), v.weight.size(), o);
  }
  fwrite(&sec, sizeof(double), 1, o);
  fclose(o);
  delete w;
  return 0;
}
