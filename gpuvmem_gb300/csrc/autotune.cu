// Launch-shape autotuner.  The reference fixes its launch shapes by command
// line (-X, -Y threads per block for image kernels, -V for visibility
// kernels; src/main.cu); here the shapes of the two dominant launches are
// measured on the problem itself:
//   * tensor-core DChi2: CTA pairs or single CTAs, split-K count (the
//     number of visibility ranges the work items split the sum into);
//   * degridding: block size and blocks per channel.
// Each candidate is timed with CUDA events on the problem's stream (median
// of three after a warm-up); the fastest is kept.  Candidates change only
// reduction orders, so results stay within the parity tolerances.
#include <algorithm>
#include <vector>

#include "gv_internal.cuh"

namespace gv {

namespace {

template <class F>
gv_status time_ms(Problem& P, F&& fn, double* ms) {
  cudaEvent_t a, b;
  GV_CUDA(cudaEventCreate(&a));
  GV_CUDA(cudaEventCreate(&b));
  GV_TRY(fn());  // warm-up (also first-launch set-up)
  std::vector<float> t;
  for (int r = 0; r < 3; r++) {
    GV_CUDA(cudaEventRecord(a, P.stream));
    GV_TRY(fn());
    GV_CUDA(cudaEventRecord(b, P.stream));
    GV_CUDA(cudaEventSynchronize(b));
    float x = 0.0f;
    GV_CUDA(cudaEventElapsedTime(&x, a, b));
    t.push_back(x);
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  std::sort(t.begin(), t.end());
  *ms = t[1];
  return GV_OK;
}

}  // namespace

gv_status autotune(Problem& P, gv_tune_report* rep) {
  const int64_t MN = (int64_t)P.M * P.N;
  float* img = nullptr;
  float* xi = nullptr;
  GV_CUDA(cudaMalloc(&img, sizeof(float) * 2 * MN));
  GV_CUDA(cudaMalloc(&xi, sizeof(float) * 2 * MN));
  struct Free {
    float* a;
    float* b;
    ~Free() {
      cudaFree(a);
      cudaFree(b);
    }
  } guard{img, xi};
  {
    std::vector<float> h(2 * MN, 0.0f);
    std::fill(h.begin(), h.begin() + MN, P.minpix);
    GV_CUDA(cudaMemcpyAsync(img, h.data(), sizeof(float) * 2 * MN, cudaMemcpyHostToDevice,
                            P.stream));
    GV_CUDA(cudaStreamSynchronize(P.stream));
  }
  int ncand = 0;
  // ---- degridding (its residuals also feed the DChi2 timings) ------------
  auto chi2 = [&]() { return chi2_launch(P, img, 0, true); };
  const int th0 = P.degrid_threads, nb0 = P.degrid_blocks;
  double best = 0.0;
  GV_TRY(time_ms(P, chi2, &best));
  rep->chi2_ms_default = best;
  int bth = th0, bnb = nb0;
  for (int th : {128, 256}) {
    for (int per_sm : {1, 2, 4}) {
      P.degrid_threads = th;
      P.degrid_blocks = per_sm * P.num_sms;
      double ms = 0.0;
      GV_TRY(time_ms(P, chi2, &ms));
      ncand++;
      if (ms < best) {
        best = ms;
        bth = th;
        bnb = P.degrid_blocks;
      }
    }
  }
  P.degrid_threads = bth;
  P.degrid_blocks = bnb;
  rep->degrid_threads = bth;
  rep->degrid_blocks = bnb > 0 ? bnb : P.part_stride;
  rep->chi2_ms_tuned = best;
  GV_TRY(chi2());  // residuals of the tuned launch
  // ---- tensor-core DChi2 --------------------------------------------------
  rep->tc_pair = -1;
  if (P.engine == 2) {
    auto dchi2 = [&]() {
      GV_CUDA(cudaMemsetAsync(xi, 0, sizeof(float) * 2 * MN, P.stream));
      return dchi2_launch(P, img, 0, xi);
    };
    const int s0 = P.tc_nsplit;
    const int pm0 = P.tc_pair_mode;
    std::vector<int> splits = {std::max(1, s0 / 2), s0, std::min(256, 2 * s0)};
    splits.erase(std::unique(splits.begin(), splits.end()), splits.end());
    const int need = *std::max_element(splits.begin(), splits.end());
    if ((size_t)need > P.tc_partial_cap) {
      float* np = nullptr;
      GV_CUDA(cudaMalloc(&np, sizeof(float) * (size_t)need * MN));
      GV_CUDA(cudaStreamSynchronize(P.stream));
      graph_cache_free(P);  // captured gradients hold the old buffer
      cudaFree(P.tc_partial);
      P.tc_partial = np;
      P.tc_partial_cap = (size_t)need;
    }
    double bms = 0.0;
    GV_TRY(time_ms(P, dchi2, &bms));
    rep->dchi2_ms_default = bms;
    int bs = s0, bpm = pm0;
    std::vector<int> modes = P.N >= 256 ? std::vector<int>{1, 0} : std::vector<int>{0};
    for (int pm : modes) {
      for (int s : splits) {
        P.tc_pair_mode = pm;
        P.tc_nsplit = s;
        double ms = 0.0;
        GV_TRY(time_ms(P, dchi2, &ms));
        ncand++;
        if (ms < bms) {
          bms = ms;
          bs = s;
          bpm = pm;
        }
      }
    }
    P.tc_nsplit = bs;
    P.tc_pair_mode = bpm;
    rep->tc_pair = tc_pair(P) ? 1 : 0;
    rep->tc_nsplit = bs;
    rep->dchi2_ms_tuned = bms;
  }
  rep->candidates = ncand;
  // captured graphs hold the old launch shapes
  graph_cache_free(P);
  ls_cache_free(P);
  return GV_OK;
}

}  // namespace gv
