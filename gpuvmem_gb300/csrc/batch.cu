// Batches of independent problems (different sizes and visibility counts)
// evaluated together.  One objective + gradient evaluation of every problem
// is captured into a single CUDA graph: each problem's kernel sequence is a
// branch forked from one capture stream, together with the copies of its
// scalars and error word to pinned host memory, so the whole batch runs as
// one graph launch with the problems' kernels overlapping on the GPU, and one
// synchronisation.  The reference runs problems one after another, each with
// several host synchronisations per evaluation.
#include <algorithm>
#include <vector>

#include "gv_internal.cuh"

namespace gv {
Problem& problem_of(gv_problem* p);
}

namespace {

struct BatchGraph {
  std::vector<float*> img, xi;
  std::vector<int> gate;  // per problem: Fi::iteration > 0 at capture
  int iter_gate, flag;
  cudaGraphExec_t exec;
  int64_t launches;
  uint64_t stamp;
};

}  // namespace

struct gv_batch {
  std::vector<gv_problem*> probs;
  std::vector<cudaStream_t> streams;
  cudaStream_t cap = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  uint32_t* h_err = nullptr;  // pinned, one word per problem
  std::vector<BatchGraph> graphs;
  uint64_t clock = 0;
  int use_graph = 1;
};

namespace {

void destroy(gv_batch* b) {
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
  for (auto s : b->streams) cudaStreamDestroy(s);
  for (auto e : b->join) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->cap) cudaStreamDestroy(b->cap);
  if (b->h_err) cudaFreeHost(b->h_err);
  delete b;
}

// one problem's evaluation, its scalars and error word copied to the host
gv_status branch(gv::Problem& P, float* img, float* xi, int iter, int flag, uint32_t* h_err) {
  GV_TRY(gv::objective_launch(P, img, flag, true));
  GV_TRY(gv::gradient_launch(P, img, xi, iter, flag));
  GV_CUDA(cudaMemcpyAsync(P.h_scal, P.d_scal, sizeof(double) * gv::kNumScal,
                          cudaMemcpyDeviceToHost, P.stream));
  GV_CUDA(cudaMemcpyAsync(h_err, P.d_flags + gv::kFlagErr, sizeof(uint32_t),
                          cudaMemcpyDeviceToHost, P.stream));
  return GV_OK;
}

}  // namespace

extern "C" {

gv_status gv_batch_create(gv_problem* const* problems, int32_t n, gv_batch** out) {
  if (!problems || n < 1 || !out) {
    gv::set_error("empty batch");
    return GV_ERR_INVALID;
  }
  *out = nullptr;
  gv_batch* b = new gv_batch();
  for (int i = 0; i < n; i++) {
    if (!problems[i]) {
      destroy(b);
      gv::set_error("null problem in batch");
      return GV_ERR_INVALID;
    }
    b->probs.push_back(problems[i]);
  }
  cudaError_t e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  for (int i = 0; i < n && e == cudaSuccess; i++) {
    cudaStream_t s;
    cudaEvent_t ev;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) break;
    b->streams.push_back(s);
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) break;
    b->join.push_back(ev);
  }
  if (e == cudaSuccess) e = cudaMallocHost(&b->h_err, sizeof(uint32_t) * n);
  if (e != cudaSuccess) {
    destroy(b);
    return gv::cuda_fail(e, "gv_batch_create");
  }
  *out = b;
  return GV_OK;
}

gv_status gv_batch_destroy(gv_batch* b) {
  if (!b) return GV_OK;
  cudaStreamSynchronize(b->cap);
  for (auto s : b->streams) cudaStreamSynchronize(s);
  destroy(b);
  return GV_OK;
}

gv_status gv_batch_set_graphs(gv_batch* b, int32_t enable) {
  if (!b) return GV_ERR_INVALID;
  b->use_graph = enable ? 1 : 0;
  return GV_OK;
}

gv_status gv_batch_evaluate(gv_batch* b, float* const* d_imgs, float* const* d_xis, int32_t iter,
                            int32_t flag_opt, double* f) {
  if (!b || !d_imgs || !d_xis || !f || iter < 0) {
    gv::set_error("invalid batch evaluate arguments");
    return GV_ERR_INVALID;
  }
  const int n = (int)b->probs.size();
  std::vector<float*> img(d_imgs, d_imgs + n), xi(d_xis, d_xis + n);
  for (int i = 0; i < n; i++)
    if (!img[i] || !xi[i]) {
      gv::set_error("null image or gradient buffer in batch");
      return GV_ERR_INVALID;
    }
  std::vector<int> gate(n);
  for (int i = 0; i < n; i++) gate[i] = gv::problem_of(b->probs[i]).iteration > 0 ? 1 : 0;
  const int igate = iter > 0 ? 1 : 0;
  std::vector<cudaStream_t> saved(n);
  for (int i = 0; i < n; i++) saved[i] = gv::problem_of(b->probs[i]).stream;
  auto restore = [&]() {
    for (int i = 0; i < n; i++) gv::problem_of(b->probs[i]).stream = saved[i];
  };
  // problems run side by side here: no cooperative launches
  for (int i = 0; i < n; i++) gv::problem_of(b->probs[i]).fused_off++;
  struct FusedBack {
    gv_batch* b;
    ~FusedBack() {
      for (auto* p : b->probs) gv::problem_of(p).fused_off--;
    }
  } fused_back{b};
  if (!b->use_graph) {
    // one problem after another, each on its own stream, one sync at the end
    gv_status s = GV_OK;
    for (int i = 0; i < n && s == GV_OK; i++) {
      gv::Problem& P = gv::problem_of(b->probs[i]);
      P.stream = b->streams[i];
      s = branch(P, img[i], xi[i], iter, flag_opt, b->h_err + i);
    }
    for (int i = 0; i < n; i++) cudaStreamSynchronize(b->streams[i]);
    restore();
    if (s != GV_OK) return s;
  } else {
    BatchGraph* hit = nullptr;
    for (auto& g : b->graphs)
      if (g.img == img && g.xi == xi && g.gate == gate && g.iter_gate == igate && g.flag == flag_opt)
        hit = &g;
    if (!hit) {
      const int64_t l0 = gv_launch_count();
      GV_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeRelaxed));
      gv_status s = GV_OK;
      cudaError_t e = cudaEventRecord(b->fork, b->cap);
      for (int i = 0; i < n && s == GV_OK && e == cudaSuccess; i++) {
        gv::Problem& P = gv::problem_of(b->probs[i]);
        P.stream = b->streams[i];
        e = cudaStreamWaitEvent(b->streams[i], b->fork, 0);
        if (e == cudaSuccess) s = branch(P, img[i], xi[i], iter, flag_opt, b->h_err + i);
        if (s == GV_OK && e == cudaSuccess) e = cudaEventRecord(b->join[i], b->streams[i]);
        if (s == GV_OK && e == cudaSuccess) e = cudaStreamWaitEvent(b->cap, b->join[i], 0);
      }
      cudaGraph_t graph = nullptr;
      cudaError_t e2 = cudaStreamEndCapture(b->cap, &graph);
      restore();
      const int64_t nl = gv_launch_count() - l0;
      // the gradients' host state (Fi::iteration) as after the evaluation
      if (s != GV_OK || e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        for (int i = 0; i < n; i++) gv::problem_of(b->probs[i]).iteration = gate[i];
        if (s != GV_OK) return s;
        return gv::cuda_fail(e != cudaSuccess ? e : e2, "batch capture");
      }
      cudaGraphExec_t exec = nullptr;
      e = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return gv::cuda_fail(e, "cudaGraphInstantiate");
      if (b->graphs.size() >= 4) {
        auto old = std::min_element(b->graphs.begin(), b->graphs.end(),
                                    [](const BatchGraph& x, const BatchGraph& y) {
                                      return x.stamp < y.stamp;
                                    });
        cudaGraphExecDestroy(old->exec);
        b->graphs.erase(old);
      }
      b->graphs.push_back({img, xi, gate, igate, flag_opt, exec, nl, 0});
      hit = &b->graphs.back();
      gv::add_launches(-nl);
    }
    hit->stamp = ++b->clock;
    GV_CUDA(cudaGraphLaunch(hit->exec, b->cap));
    gv::add_launches(hit->launches);
    GV_CUDA(cudaStreamSynchronize(b->cap));
  }
  gv_status st = GV_OK;
  for (int i = 0; i < n; i++) {
    gv::Problem& P = gv::problem_of(b->probs[i]);
    P.iteration = iter;
    double tot = 0.0;
    for (size_t t = 0; t < P.terms.size(); t++)
      tot += (double)P.terms[t].lambda * P.h_scal[gv::kSlotTerm0 + t];
    f[i] = tot;
    if (b->h_err[i] != 0 && st == GV_OK) {
      cudaMemsetAsync(P.d_flags + gv::kFlagErr, 0, sizeof(uint32_t), P.stream);
      gv::set_error("a kernel of batch problem " + std::to_string(i) +
                    " gave up on a bounded wait (device error word " +
                    std::to_string(b->h_err[i]) + ")");
      st = GV_ERR_DEVICE;
    }
  }
  return st;
}

}  // extern "C"
