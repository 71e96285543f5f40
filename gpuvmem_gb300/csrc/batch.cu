// Batches of independent problems (different sizes and visibility counts)
// evaluated together.  One objective + gradient evaluation of every problem
// is captured into a single CUDA graph: each problem's kernel sequence is a
// branch forked from one capture stream, together with the copies of its
// scalars and error word to pinned host memory, so the whole batch runs as
// one graph launch with the problems' kernels overlapping on the GPU, and one
// synchronisation.  With GV_BATCH_FUSED=1 the objectives of all problems run
// instead as one cooperative launch over an offset table of their tasks
// (k_objective_fused_batch, when every problem is up to 512 x 512 with Chi2
// as its first term) before the gradient branches; on 64 problems of sides
// 128-512 the branches are faster (10.3 against 11.1 ms a batch), so they are
// the default.  The reference runs problems one after another, each with
// several host synchronisations per evaluation.
#include <algorithm>
#include <cstdlib>
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
  void* d_tables = nullptr;  // batched objective: arguments, task offsets, barrier
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
  int fused_objective = 0;  // objectives as one cooperative launch (GV_BATCH_FUSED=1: on)
};

namespace {

void destroy(gv_batch* b) {
  for (auto& g : b->graphs) {
    cudaGraphExecDestroy(g.exec);
    cudaFree(g.d_tables);
  }
  for (auto s : b->streams) cudaStreamDestroy(s);
  for (auto e : b->join) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->cap) cudaStreamDestroy(b->cap);
  if (b->h_err) cudaFreeHost(b->h_err);
  delete b;
}

// one problem's evaluation, its scalars and error word copied to the host
gv_status branch(gv::Problem& P, float* img, float* xi, int iter, int flag, uint32_t* h_err,
                 bool objective = true) {
  if (objective) GV_TRY(gv::objective_launch(P, img, flag, true));
  GV_TRY(gv::gradient_launch(P, img, xi, iter, flag));
  GV_CUDA(cudaMemcpyAsync(P.h_scal, P.d_scal, sizeof(double) * gv::kNumScal,
                          cudaMemcpyDeviceToHost, P.stream));
  GV_CUDA(cudaMemcpyAsync(h_err, P.d_flags + gv::kFlagErr, sizeof(uint32_t),
                          cudaMemcpyDeviceToHost, P.stream));
  return GV_OK;
}

// The batched objective's tables for images `img` (device memory, owned by
// the caller): every problem's arguments, then the [3][n + 1] task offsets,
// then the three words of the grid barrier and its error word.  Returns
// nullptr when a problem cannot run in the batched launch.
void* batch_tables(gv_batch* b, const std::vector<float*>& img, int flag, int* max_n,
                   int* max_tasks, gv_status* st) {
  const int n = (int)b->probs.size();
  *st = GV_OK;
  if (!b->fused_objective) return nullptr;
  // the kernel indexes the arguments as an array: the stride is their size
  const size_t ab = gv::batch_arg_bytes();
  std::vector<unsigned char> host(ab * n + sizeof(int) * 3 * (n + 1) + 16, 0);
  int* off = reinterpret_cast<int*>(host.data() + ab * n);
  *max_n = 0;
  *st = GV_OK;
  for (int i = 0; i < n; i++) {
    gv::Problem& P = gv::problem_of(b->probs[i]);
    int tasks[3];
    if (gv::batch_objective_args(P, img[i], flag, host.data() + ab * i, tasks) != GV_OK)
      return nullptr;
    for (int ph = 0; ph < 3; ph++) off[ph * (n + 1) + i + 1] = off[ph * (n + 1) + i] + tasks[ph];
    *max_n = std::max(*max_n, P.N);
  }
  *max_tasks = 0;
  for (int ph = 0; ph < 3; ph++) *max_tasks = std::max(*max_tasks, off[ph * (n + 1) + n]);
  void* d = nullptr;
  cudaError_t e = cudaMalloc(&d, host.size());
  if (e == cudaSuccess) e = cudaMemcpy(d, host.data(), host.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    *st = gv::cuda_fail(e, "batch tables");
    return nullptr;
  }
  return d;
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
  if (const char* env = std::getenv("GV_BATCH_FUSED")) b->fused_objective = std::atoi(env) != 0;
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
      int max_n = 0, max_tasks = 0;
      gv_status ts = GV_OK;
      void* tables = batch_tables(b, img, flag_opt, &max_n, &max_tasks, &ts);
      if (ts != GV_OK) return ts;
      const int64_t l0 = gv_launch_count();
      GV_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeRelaxed));
      gv_status s = GV_OK;
      if (tables) {
        const size_t ab = gv::batch_arg_bytes();
        unsigned char* t = static_cast<unsigned char*>(tables);
        const int* d_off = reinterpret_cast<const int*>(t + ab * n);
        uint32_t* d_bar = reinterpret_cast<uint32_t*>(t + ab * n + sizeof(int) * 3 * (n + 1));
        gv::Problem& P0 = gv::problem_of(b->probs[0]);
        s = gv::batch_objective_launch(n, t, d_off, max_n, max_tasks, d_bar,
                                       P0.d_flags + gv::kFlagErr, P0.num_sms, b->cap);
      }
      cudaError_t e = cudaEventRecord(b->fork, b->cap);
      for (int i = 0; i < n && s == GV_OK && e == cudaSuccess; i++) {
        gv::Problem& P = gv::problem_of(b->probs[i]);
        P.stream = b->streams[i];
        e = cudaStreamWaitEvent(b->streams[i], b->fork, 0);
        if (e == cudaSuccess)
          s = branch(P, img[i], xi[i], iter, flag_opt, b->h_err + i, tables == nullptr);
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
        cudaFree(tables);
        for (int i = 0; i < n; i++) gv::problem_of(b->probs[i]).iteration = gate[i];
        if (s != GV_OK) return s;
        return gv::cuda_fail(e != cudaSuccess ? e : e2, "batch capture");
      }
      cudaGraphExec_t exec = nullptr;
      e = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) {
        cudaFree(tables);
        return gv::cuda_fail(e, "cudaGraphInstantiate");
      }
      if (b->graphs.size() >= 4) {
        auto old = std::min_element(b->graphs.begin(), b->graphs.end(),
                                    [](const BatchGraph& x, const BatchGraph& y) {
                                      return x.stamp < y.stamp;
                                    });
        cudaGraphExecDestroy(old->exec);
        cudaFree(old->d_tables);
        b->graphs.erase(old);
      }
      b->graphs.push_back({img, xi, gate, igate, flag_opt, exec, nl, 0, tables});
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
