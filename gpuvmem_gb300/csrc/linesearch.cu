// linmin's line search on the GPU as the body of a CUDA-graph WHILE loop
// (optim.cu): k_ls_begin starts a search, and after every objective
// evaluation k_ls_step advances the state machine of ls_core.cuh (the
// bracketing step of src/mnbrak.cu:44-98 and Brent's minimiser of
// src/brent.cu:43-121) and sets the loop condition, so a whole line search
// is one graph launch with no host round trip per evaluation.  The loop ends
// after `cap` evaluations at the latest (the host bracketing loop has no
// bound; an unbounded decrease along the line ends here with an error status
// instead).
#include "ls_core.cuh"

namespace gv {
namespace {
__global__ void k_ls_begin(LsState* s, LsTerms terms, float tol, int cap) {
  if (threadIdx.x != 0) return;
  s->state = ls::kWaitFa;
  s->evals = 0;
  s->steps = 0;
  s->it = 0;
  s->error = 0;
  s->cap = cap;
  s->tol = tol;
  s->nterms = terms.nterms;
  for (int t = 0; t < kMaxTerms; t++) s->lambda[t] = terms.lambda[t];
  // linmin: ax = 0, xx = 1 (src/linmin.cu:78-80)
  s->ax = 0.0f;
  s->bx = 1.0f;
  s->x_req = s->ax;
  s->xmin = 0.0f;
  s->fret = 0.0f;
}

__global__ void k_ls_step(LsState* s, double* scal, cudaGraphConditionalHandle h) {
  if (threadIdx.x != 0) return;
  const bool more = ls::ls_step(s, scal);
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

}  // namespace

gv_status ls_begin_launch(cudaStream_t st, LsState* s, LsTerms terms, float tol, int cap) {
  k_ls_begin<<<1, 32, 0, st>>>(s, terms, tol, cap);
  GV_LAUNCH("k_ls_begin");
  return GV_OK;
}

gv_status ls_step_launch(cudaStream_t st, LsState* s, double* scal, cudaGraphConditionalHandle h) {
  k_ls_step<<<1, 32, 0, st>>>(s, scal, h);
  GV_LAUNCH("k_ls_step");
  return GV_OK;
}

}  // namespace gv
