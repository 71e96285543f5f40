// CUDA-graph replay of objective (+ gradient) evaluations.
//
// The reference launches every kernel of an evaluation from the host and
// synchronises several times inside it (deviceReduce, src/functions.cu:604).
// Here an evaluation is a fixed, sync-free sequence of kernels on the
// problem's stream (objective_launch, gradient_launch), so it is captured
// once into a CUDA graph per set of buffers and replayed with one
// cudaGraphLaunch.  The key is everything the captured sequence depends on:
// the image and gradient pointers, flag_opt, and the prior gating
// (Fi::iteration > 0 for the objective, iter > 0 for the gradient).
// Captures run on a private non-blocking stream (the legacy default stream
// cannot be captured); replays go onto the problem's stream.
#include <algorithm>
#include <vector>

#include "gv_internal.cuh"

namespace gv {

namespace {

struct GraphEntry {
  const float* img;
  const float* xi;
  int flag, obj_gate, grad_gate, what, store;
  cudaGraphExec_t exec;
  int64_t launches;
  uint64_t stamp;
};

struct GraphCache {
  std::vector<GraphEntry> e;
  cudaStream_t cap = nullptr;
  uint64_t clock = 0;
};

constexpr size_t kMaxGraphs = 8;

GraphCache& cache(Problem& P) {
  if (!P.graphs) P.graphs = new GraphCache();
  return *static_cast<GraphCache*>(P.graphs);
}

}  // namespace

void graph_cache_free(Problem& P) {
  if (!P.graphs) return;
  GraphCache* c = static_cast<GraphCache*>(P.graphs);
  for (auto& g : c->e) cudaGraphExecDestroy(g.exec);
  if (c->cap) cudaStreamDestroy(c->cap);
  delete c;
  P.graphs = nullptr;
}

// what: 1 = objective, 2 = gradient, 3 = objective + gradient; store: the
// objective keeps its weighted residuals for the next gradient.  The objective's
// scalars land in d_scal as with objective_launch; the caller fetches them.
gv_status eval_graph(Problem& P, float* d_img, float* d_xi, int iter, int flag_opt, int what,
                     bool store) {
  GraphCache& c = cache(P);
  const int obj_gate = (what & 1) ? (P.iteration > 0 ? 1 : 0) : 0;
  const int grad_gate = (what & 2) ? (iter > 0 ? 1 : 0) : 0;
  const float* xi_key = (what & 2) ? d_xi : nullptr;
  GraphEntry* hit = nullptr;
  for (auto& g : c.e)
    if (g.img == d_img && g.xi == xi_key && g.flag == flag_opt && g.obj_gate == obj_gate &&
        g.grad_gate == grad_gate && g.what == what && g.store == (store ? 1 : 0))
      hit = &g;
  if (!hit) {
    if (!c.cap) GV_CUDA(cudaStreamCreateWithFlags(&c.cap, cudaStreamNonBlocking));
    const cudaStream_t saved = P.stream;
    const int saved_iter = P.iteration;
    const int64_t l0 = gv_launch_count();
    P.stream = c.cap;
    cudaError_t e = cudaStreamBeginCapture(c.cap, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) {
      P.stream = saved;
      return cuda_fail(e, "cudaStreamBeginCapture");
    }
    gv_status s = (what & 1) ? objective_launch(P, d_img, flag_opt, store) : GV_OK;
    if (s == GV_OK && (what & 2)) s = gradient_launch(P, d_img, d_xi, iter, flag_opt);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(c.cap, &graph);
    P.stream = saved;
    const int64_t nl = gv_launch_count() - l0;
    if (s != GV_OK) {
      if (graph) cudaGraphDestroy(graph);
      P.iteration = saved_iter;
      return s;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    if (c.e.size() >= kMaxGraphs) {
      auto old = std::min_element(c.e.begin(), c.e.end(), [](const GraphEntry& a,
                                                             const GraphEntry& b) {
        return a.stamp < b.stamp;
      });
      cudaGraphExecDestroy(old->exec);
      c.e.erase(old);
    }
    c.e.push_back({d_img, xi_key, flag_opt, obj_gate, grad_gate, what, store ? 1 : 0, exec, nl,
                   0});
    hit = &c.e.back();
    // the captured launches were counted while capturing; the replay below
    // counts them again
    add_launches(-nl);
  }
  hit->stamp = ++c.clock;
  GV_CUDA(cudaGraphLaunch(hit->exec, P.stream));
  add_launches(hit->launches);
  // host-side state the captured gradient_launch would have set
  if (what & 2) P.iteration = iter;
  return GV_OK;
}

}  // namespace gv
