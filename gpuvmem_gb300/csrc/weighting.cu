// Visibility weighting schemes on the GPU: NaturalWeightingScheme::apply
// (src/naturalweightingscheme.cu:9-52), UniformWeightingScheme::apply
// (src/uniformweightingscheme.cu:9-102) and BriggsWeightingScheme::apply
// (src/briggsweightingscheme.cu:30-190), one field and one correlation,
// without a uv taper.
//
// The reference grids the weights in FP32 with an OpenMP critical section
// per visibility, so its result depends on the thread schedule; with one
// thread it is a sequential FP32 sum per grid cell in visibility order.
// This version reproduces that one-thread result bit for bit without a
// critical section: each channel's visibilities are sorted by cell with a
// stable radix sort, and one thread per occupied cell adds that cell's
// weights in visibility order (starting from the cell's previous value for
// Briggs' cumulative first pass).  The scalar sums that feed Briggs' f^2
// keep the reference's sequential FP32 order: the sum of the weights on the
// host (std::accumulate order), the sum of squares of the half grid by one
// GPU thread.

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "gv_internal.cuh"

namespace gv {
namespace {

constexpr uint32_t kNoCell = 0xFFFFFFFFu;

// cell of every visibility (src/briggsweightingscheme.cu:74-88): float
// wavelength, u < 0 flipped, truncation of u / |du| + N/2 + 0.5
__global__ void k_weight_cells(int64_t n, const double* __restrict__ uvw, float freq, double adu,
                               double adv, int M, int N, uint32_t* __restrict__ key,
                               uint32_t* __restrict__ idx) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float lambda = kLightSpeed / freq;
  double u = uvw[3 * k] / lambda, v = uvw[3 * k + 1] / lambda;
  if (u < 0.0) {
    u *= -1.0;
    v *= -1.0;
  }
  const int x = (int)(u / adu + (double)(N / 2) + 0.5);
  const int y = (int)(v / adv + (double)(M / 2) + 0.5);
  key[k] = (x >= 0 && y >= 0 && x < N && y < M) ? (uint32_t)(N * y + x) : kNoCell;
  idx[k] = (uint32_t)k;
}

// one thread per run of equal keys: grid[cell] += w of the run, in order
__global__ void k_cell_runs(int64_t n, const uint32_t* __restrict__ key,
                            const uint32_t* __restrict__ idx, const float* __restrict__ w,
                            float* __restrict__ grid) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t c = key[k];
  if (c == kNoCell || (k > 0 && key[k - 1] == c)) return;
  float s = grid[c];
  for (int64_t j = k; j < n && key[j] == c; j++) s += w[idx[j]];
  grid[c] = s;
}

// sum over rows m and columns N/2..N-1 of grid^2, in that order, added to
// *acc.  Thread 0 adds one row's squares sequentially from shared memory
// while warps 1.. stage the next row (double buffer).
constexpr int kSumThreads = 256;
constexpr int kMaxHalf = 2048;
__global__ void __launch_bounds__(kSumThreads) k_half_sumsq(int M, int N,
                                                            const float* __restrict__ grid,
                                                            float* __restrict__ acc) {
  __shared__ float buf[2][kMaxHalf];
  const int tid = threadIdx.x;
  const int x0 = N / 2, half = N - N / 2;
  auto stage = [&](int m, int which, int first, int stride) {
    const float* row = grid + (int64_t)N * m + x0;
    for (int i = first; i < half; i += stride) {
      const float g = row[i];
      buf[which][i] = g * g;
    }
  };
  stage(0, 0, tid, kSumThreads);
  __syncthreads();
  float s = tid == 0 ? *acc : 0.0f;
  for (int m = 0; m < M; m++) {
    if (m + 1 < M && tid >= 32) stage(m + 1, (m + 1) & 1, tid - 32, kSumThreads - 32);
    if (tid == 0) {
      const float* r = buf[m & 1];
      int i = 0;
      for (; i + 16 <= half; i += 16) {
        float a[16];
#pragma unroll
        for (int j = 0; j < 16; j++) a[j] = r[i + j];
#pragma unroll
        for (int j = 0; j < 16; j++) s += a[j];
      }
      for (; i < half; i++) s += r[i];
    }
    __syncthreads();
  }
  if (tid == 0) *acc = s;
}

__global__ void k_apply_uniform(int64_t n, const uint32_t* __restrict__ cell,
                                const float* __restrict__ grid, float* __restrict__ w) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t c = cell[k];
  w[k] = c != kNoCell ? w[k] / grid[c] : 0.0f;
}

__global__ void k_apply_briggs(int64_t n, const uint32_t* __restrict__ cell,
                               const float* __restrict__ grid, float f2, float* __restrict__ w) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t c = cell[k];
  w[k] = c != kNoCell ? (float)((double)w[k] / (1.0 + (double)(grid[c] * f2))) : 0.0f;
}

struct Buffers {
  double* uvw = nullptr;
  float* w = nullptr;
  uint32_t *key = nullptr, *idx = nullptr, *skey = nullptr, *sidx = nullptr;
  float* grid = nullptr;
  float* acc = nullptr;
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  ~Buffers() {
    cudaFree(uvw);
    cudaFree(w);
    cudaFree(key);
    cudaFree(idx);
    cudaFree(skey);
    cudaFree(sidx);
    cudaFree(grid);
    cudaFree(acc);
    cudaFree(tmp);
  }
};

}  // namespace
}  // namespace gv

extern "C" gv_status gv_apply_weighting(int32_t scheme, float robust, int32_t M, int32_t N,
                                        double deltax_deg, double deltay_deg, int32_t nchannels,
                                        const gv_channel_desc* ch, float* const* weights_out,
                                        void* stream) {
  using namespace gv;
  if (scheme < GV_WEIGHT_NATURAL || scheme > GV_WEIGHT_BRIGGS || M < 2 || N < 2 ||
      N - N / 2 > kMaxHalf ||
      nchannels < 1 || !ch || !weights_out || deltax_deg == 0.0 || deltay_deg == 0.0) {
    set_error("invalid weighting arguments");
    return GV_ERR_INVALID;
  }
  for (int c = 0; c < nchannels; c++)
    if (ch[c].nvis < 0 || (ch[c].nvis > 0 && (!ch[c].uvw || !ch[c].weight || !weights_out[c])) ||
        ch[c].nvis >= (int64_t)kNoCell) {
      set_error("invalid channel in weighting");
      return GV_ERR_INVALID;
    }
  // deltau = 1 / (M * deltax), deltax = RPDEG_D * DELTAX (src/mfs.cu:531-534)
  const double deltax = kRpDegD * deltax_deg, deltay = kRpDegD * deltay_deg;
  const double adu = std::fabs(1.0 / ((double)M * deltax));
  const double adv = std::fabs(1.0 / ((double)N * deltay));
  if (scheme == GV_WEIGHT_NATURAL) {
    for (int c = 0; c < nchannels; c++)
      if (weights_out[c] != ch[c].weight)
        std::copy(ch[c].weight, ch[c].weight + ch[c].nvis, weights_out[c]);
    return GV_OK;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int64_t vmax = 1;
  for (int c = 0; c < nchannels; c++) vmax = std::max<int64_t>(vmax, ch[c].nvis);
  const int64_t MN = (int64_t)M * N;
  Buffers b;
  GV_CUDA(cudaMalloc(&b.uvw, sizeof(double) * 3 * vmax));
  GV_CUDA(cudaMalloc(&b.w, sizeof(float) * vmax));
  GV_CUDA(cudaMalloc(&b.key, sizeof(uint32_t) * vmax));
  GV_CUDA(cudaMalloc(&b.idx, sizeof(uint32_t) * vmax));
  GV_CUDA(cudaMalloc(&b.skey, sizeof(uint32_t) * vmax));
  GV_CUDA(cudaMalloc(&b.sidx, sizeof(uint32_t) * vmax));
  GV_CUDA(cudaMalloc(&b.grid, sizeof(float) * MN));
  GV_CUDA(cudaMalloc(&b.acc, sizeof(float)));
  b.tmp_bytes = radix_sort_scratch<uint32_t, uint32_t>(vmax);
  GV_CUDA(cudaMalloc(&b.tmp, b.tmp_bytes));
  // grid one channel's weights into b.grid (added to what it holds)
  auto grid_channel = [&](int c) -> gv_status {
    const int64_t n = ch[c].nvis;
    if (n == 0) return GV_OK;
    GV_CUDA(cudaMemcpyAsync(b.uvw, ch[c].uvw, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
    GV_CUDA(cudaMemcpyAsync(b.w, ch[c].weight, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    const unsigned gb = (unsigned)((n + 255) / 256);
    k_weight_cells<<<gb, 256, 0, st>>>(n, b.uvw, ch[c].freq_hz, adu, adv, M, N, b.key, b.idx);
    GV_LAUNCH("k_weight_cells");
    GV_TRY((radix_sort_pairs<uint32_t, uint32_t>(b.tmp, b.tmp_bytes, b.key, b.skey, b.idx,
                                                  b.sidx, n, 0, 32, st)));
    k_cell_runs<<<gb, 256, 0, st>>>(n, b.skey, b.sidx, b.w, b.grid);
    GV_LAUNCH("k_cell_runs");
    return GV_OK;
  };
  float f2 = 0.0f;
  if (scheme == GV_WEIGHT_BRIGGS) {
    // sum of the original weights (std::accumulate per channel, FP32)
    float sum_orig = 0.0f;
    for (int c = 0; c < nchannels; c++)
      sum_orig += std::accumulate(ch[c].weight, ch[c].weight + ch[c].nvis, 0.0f);
    GV_CUDA(cudaMemsetAsync(b.grid, 0, sizeof(float) * MN, st));
    GV_CUDA(cudaMemsetAsync(b.acc, 0, sizeof(float), st));
    for (int c = 0; c < nchannels; c++) {
      GV_TRY(grid_channel(c));  // cumulative over channels, as the reference
      k_half_sumsq<<<1, kSumThreads, 0, st>>>(M, N, b.grid, b.acc);
      GV_LAUNCH("k_half_sumsq");
    }
    float sum_sq = 0.0f;
    GV_CUDA(cudaMemcpyAsync(&sum_sq, b.acc, sizeof(float), cudaMemcpyDeviceToHost, st));
    GV_CUDA(cudaStreamSynchronize(st));
    const float average = sum_sq / sum_orig;
    const float r = 5.0f * powf(10.0f, -robust);
    f2 = r * r / average;
  }
  for (int c = 0; c < nchannels; c++) {
    const int64_t n = ch[c].nvis;
    if (n == 0) continue;
    GV_CUDA(cudaMemsetAsync(b.grid, 0, sizeof(float) * MN, st));
    GV_TRY(grid_channel(c));
    const unsigned gb = (unsigned)((n + 255) / 256);
    if (scheme == GV_WEIGHT_UNIFORM)
      k_apply_uniform<<<gb, 256, 0, st>>>(n, b.key, b.grid, b.w);
    else
      k_apply_briggs<<<gb, 256, 0, st>>>(n, b.key, b.grid, f2, b.w);
    GV_LAUNCH("k_apply_weights");
    GV_CUDA(cudaMemcpyAsync(weights_out[c], b.w, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    GV_CUDA(cudaStreamSynchronize(st));
  }
  return GV_OK;
}
