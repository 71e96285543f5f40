// Reference harness, device side: compiles the reference's own CUDA kernels
// (src/functions.cu of the gpuvmem repository, read in place) into a cubin
// for sm_103a.  TEST INFRASTRUCTURE: it pins the CPU oracle and times the
// reference CUDA build; the product never loads it.
//
// src/MSFITSIO.cu needs casacore, so the three unit helpers the kernels call
// from it (freq_to_wavelength, metres_to_lambda, distance;
// src/MSFITSIO.cu:36-51) are restated here with the same float arithmetic.
#include "MSFITSIO.cuh"

__host__ __device__ float freq_to_wavelength(float freq) {
  const float wl = LIGHTSPEED / freq;
  return wl;
}

__host__ __device__ double metres_to_lambda(double metres, float freq) {
  const float wl = freq_to_wavelength(freq);
  return metres / wl;
}

__host__ __device__ float distance(float x, float y, float x0, float y0) {
  const float dx = x - x0, dy = y - y0;
  return sqrtf(dx * dx + dy * dy);
}

#include "functions.cu"
// complex helpers called by the kernels (src/complexOps.cu)
#include "complexOps.cu"
