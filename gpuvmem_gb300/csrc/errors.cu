// Error images of a solution: calculateErrors (src/functions.cu:4966-5041)
// with I_nu_0_Noise (:4076), alpha_Noise (:4113) and noise_reduction
// (:4177).  Per channel c with weight sum W_c:
//   E0(i,j) += A^2 W_c (nu/nu_0)^(2 alpha)                     (inside the mask)
//   s = A I_nu W_c + sum_k Re(w_k Vr_k e^{+2 pi i (x u_k + y v_k)})
//   E1(i,j) += log(nu/nu_0)^2 A I_nu s      if s > 0           (inside the mask)
// then E = 1/sqrt(E) where positive, else 0.  The visibility sum is the
// DChi2 contraction without the w-term and with conjugated residuals
// (mode 4 of both DChi2 engines), one channel at a time.  The reference
// evaluates the phase in float (about 1e-4 cycles off at the image edge)
// and sums the visibilities in float; here the phase is exact and the sums
// are those of the DChi2 engines.
#include "gv_internal.cuh"

namespace gv {
namespace {

__global__ void k_weight_sums(int C, const ChanRange* __restrict__ ranges,
                              const float4* __restrict__ deg, double* __restrict__ out) {
  const int c = blockIdx.x;
  const ChanRange rg = ranges[c];
  double s = 0.0;
  for (int64_t k = threadIdx.x; k < rg.ngrid; k += blockDim.x) s += (double)deg[rg.off + k].w;
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[c] = s;
  }
}

struct ErrParams {
  int M, N;
  int64_t MN;
  float xobs, yobs, freq, nu_0, D, pbf, pbcut;
  int pb;
  double DELTAX, DELTAY;
};

__global__ void k_error_accumulate(ErrParams e, const double* __restrict__ wsum, int c,
                                   const uint8_t* __restrict__ mask,
                                   const float* __restrict__ img,
                                   const float* __restrict__ vsum, float* __restrict__ err) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= e.N || j >= e.M) return;
  const int64_t q = (int64_t)e.N * i + j;
  if (!(mask[q] & kMaskIn)) {
    err[q] = 0.0f;
    err[e.MN + q] = 0.0f;
    return;
  }
  const float W = (float)wsum[c];
  const float atten =
      attenuation(i, j, e.xobs, e.yobs, e.DELTAX, e.DELTAY, e.freq, e.D, e.pbf, e.pbcut, e.pb);
  const float nudiv = e.freq / e.nu_0;
  const float alpha = img[e.MN + q];
  err[q] += atten * atten * W * powf(nudiv, 2.0f * alpha);
  const float I_nu = img[q] * powf(nudiv, alpha);
  const float lg = logf(nudiv);
  const float s = atten * I_nu * W + vsum[q];
  if (s > 0.0f) err[e.MN + q] += lg * lg * atten * I_nu * s;
}

__global__ void k_error_finish(int64_t n, float* __restrict__ err) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float v = err[q];
  err[q] = v > 0.0f ? 1.0f / sqrtf(v) : 0.0f;
}

}  // namespace

gv_status error_images(Problem& P, float* d_img, float* d_err) {
  const int C = (int)P.chans.size();
  const int64_t MN = (int64_t)P.M * P.N;
  // residuals of this image (calculateErrors runs after the last chi2)
  GV_TRY(chi2_launch(P, d_img, 0, true));
  double* wsum = nullptr;
  GV_CUDA(cudaMalloc(&wsum, sizeof(double) * C));
  k_weight_sums<<<C, 256, 0, P.stream>>>(C, P.d_ranges, P.d_deg, wsum);
  GV_LAUNCH("k_weight_sums");
  GV_CUDA(cudaMemsetAsync(d_err, 0, sizeof(float) * 2 * MN, P.stream));
  ErrParams e;
  e.M = P.M;
  e.N = P.N;
  e.MN = MN;
  e.xobs = P.xobs;
  e.yobs = P.yobs;
  e.nu_0 = P.nu_0;
  e.D = P.D;
  e.pbf = P.pbf;
  e.pbcut = P.pbcut;
  e.pb = P.pb;
  e.DELTAX = P.DELTAX;
  e.DELTAY = P.DELTAY;
  gv_status s = GV_OK;
  for (int c = 0; c < C && s == GV_OK; c++) {
    cudaError_t ce = cudaMemsetAsync(P.d_tmp, 0, sizeof(float) * MN, P.stream);
    if (ce != cudaSuccess) {
      s = cuda_fail(ce, "error_images");
      break;
    }
    s = P.engine == 2 ? dchi2_tc(P, nullptr, 0, P.d_tmp, c, 4)
                      : dchi2_direct(P, nullptr, 0, P.d_tmp, c, 4);
    if (s != GV_OK) break;
    e.freq = P.chans[c].freq;
    dim3 blk(32, 8), grd((P.M + 31) / 32, (P.N + 7) / 8);
    k_error_accumulate<<<grd, blk, 0, P.stream>>>(e, wsum, c, P.d_mask, d_img, P.d_tmp, d_err);
    cudaError_t le = cudaGetLastError();
    count_launch();
    if (le != cudaSuccess) s = cuda_fail(le, "k_error_accumulate");
  }
  if (s == GV_OK) {
    k_error_finish<<<(unsigned)((2 * MN + 255) / 256), 256, 0, P.stream>>>(2 * MN, d_err);
    cudaError_t le = cudaGetLastError();
    count_launch();
    if (le != cudaSuccess) s = cuda_fail(le, "k_error_finish");
  }
  cudaStreamSynchronize(P.stream);
  cudaFree(wsum);
  return s;
}

}  // namespace gv
