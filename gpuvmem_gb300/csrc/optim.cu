// Optimisers of the reference's Optimizer surface on the GPU:
//   "CG-FRPRMN"  ConjugateGradient::optimize   src/frprmn.cu:85-195
//   "CG-LBFGS"   LBFGS::optimize + recursion  src/lbfgs.cu:99-341
// with linmin / f1dim (src/linmin.cu:52-110, src/f1dim.cu:49-80) and the
// bracketing and Brent line minimisers (src/mnbrak.cu:44-98,
// src/brent.cu:43-121; the published algorithms of Brent 1973 with the
// reference's constants).  Host scalars are float, as in the reference, so
// the line search takes the same decisions; vector updates are fused GPU
// kernels and all dot products and reductions accumulate in FP64.
//
// L-BFGS keeps the reference's ring addressing: getDot_LBFGS_ff and
// calculateSandY use slot offset M*N*image*k + M*N*image, updateQ uses
// M*N*image + M*N*k (src/functions.cu:3571-3653).
#include <algorithm>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gv_internal.cuh"

namespace gv {

namespace {

// GV_VERBOSE=1 prints the line-search and iteration values, as the
// reference's --verbose flag does (src/linmin.cu:83, src/frprmn.cu:131).
bool verbose() {
  static int v = -1;
  if (v < 0) {
    const char* e = std::getenv("GV_VERBOSE");
    v = (e && e[0] == '1') ? 1 : 0;
  }
  return v == 1;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// block-wide FP64 sum and max in a fixed order (result valid in thread 0)
__device__ double block_sum_d(double v) {
  __shared__ double sh[32];
  v = warp_sum_d(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
  return t;
}
__device__ double block_max_d(double v) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double t = v;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t = fmax(t, sh[w]);
  return t;
}

// evaluateXt / evaluateXtNoPositivity, src/functions.cu:2832-2864
// (x from x_dev when it is set: the device line search's point)
__global__ void k_eval_xt(int64_t MN, float x, const float* __restrict__ x_dev, float floor_val,
                          float floor_cmp, int positivity, const float* __restrict__ pcom,
                          const float* __restrict__ xicom, float* __restrict__ xt) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= 2 * MN) return;
  if (x_dev) x = *x_dev;
  const float v = fmaf(x, xicom[q], pcom[q]);
  xt[q] = (q < MN && positivity && !(v > floor_cmp)) ? floor_val : v;
}

// newP / newPNoPositivity, src/functions.cu:2779-2812
// (xmin from xmin_dev when it is set: the device line search's minimum;
// floor_cmp = float_below of the reference's FP64 threshold)
__global__ void k_new_p(int64_t MN, float xmin, const float* __restrict__ xmin_dev,
                        float floor_val, float floor_cmp, int positivity, float* __restrict__ p,
                        float* __restrict__ xi) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= 2 * MN) return;
  if (xmin_dev) xmin = *xmin_dev;
  const float s = xi[q] * xmin;
  if (q < MN && positivity) {
    if (p[q] + s > floor_cmp) {
      p[q] += s;
      xi[q] = s;
    } else {
      p[q] = floor_val;
      xi[q] = 0.0f;
    }
  } else {
    xi[q] = s;
    p[q] += s;
  }
}

// searchDirection, src/functions.cu:3655
__global__ void k_cg_init(int64_t n, float* __restrict__ g, float* __restrict__ xi,
                          float* __restrict__ h) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float v = -xi[q];
  g[q] = v;
  xi[q] = v;
  h[q] = v;
}

// newXi, src/functions.cu:3678
__global__ void k_new_xi(int64_t n, float gam, float* __restrict__ g, float* __restrict__ xi,
                         float* __restrict__ h) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float gv = -xi[q];
  const float hv = fmaf(gam, h[q], gv);
  g[q] = gv;
  xi[q] = hv;
  h[q] = hv;
}

// CGGradCondition + deviceMaxReduce and getGGandDGG + 2 deviceReduce of
// frprmn (src/frprmn.cu:137-168) fused into one pass: partials of
// gmax = max |xi| max(|p|,1)/den, gg = sum g^2, dgg = sum (xi+g) xi.
__global__ void __launch_bounds__(256) k_cg_stats(int64_t n, float den,
                                                  const float* __restrict__ xi,
                                                  const float* __restrict__ g,
                                                  const float* __restrict__ p,
                                                  double* __restrict__ part, int stride,
                                                  uint32_t* __restrict__ done,
                                                  double* __restrict__ out) {
  CompSum ggs, dggs;
  float gmax = FLT_MIN;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x) {
    const float x = xi[q], gq = g[q];
    gmax = fmaxf(gmax, fabsf(x) * fmaxf(fabsf(p[q]), 1.0f) / den);
    ggs.add(gq * gq);
    dggs.add((x + gq) * x);
  }
  double gg = ggs.value(), dgg = dggs.value();
  __shared__ double s1[32], s2[32];
  __shared__ float s3[32];
  gg = warp_sum_d(gg);
  dgg = warp_sum_d(dgg);
  gmax = warp_max_f(gmax);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    s1[wid] = gg;
    s2[wid] = dgg;
    s3[wid] = gmax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    float m = FLT_MIN;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      a += s1[w];
      b += s2[w];
      m = fmaxf(m, s3[w]);
    }
    part[blockIdx.x] = a;
    part[stride + blockIdx.x] = b;
    part[2 * stride + blockIdx.x] = (double)m;
  }
  if (last_block_done(done, gridDim.x)) {
    // the block partials, each thread over a fixed stride, then the block
    double a = 0.0, b = 0.0, m = (double)FLT_MIN;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
      a += __ldcg(part + i);
      b += __ldcg(part + stride + i);
      m = fmax(m, __ldcg(part + 2 * stride + i));
    }
    a = block_sum_d(a);
    b = block_sum_d(b);
    m = block_max_d(m);
    if (threadIdx.x == 0) {
      out[0] = a;
      out[1] = b;
      out[2] = m;
    }
  }
}

// Dot product of two float vectors: the float products, summed per thread
// (compensated), then in FP64
__global__ void __launch_bounds__(256) k_dot(int64_t n, const float* __restrict__ a,
                                             const float* __restrict__ b,
                                             double* __restrict__ part,
                                             uint32_t* __restrict__ done,
                                             double* __restrict__ out) {
  CompSum cs;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    cs.add(a[q] * b[q]);
  double s = cs.value();
  __shared__ double sh[32];
  s = warp_sum_d(s);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    part[blockIdx.x] = t;
  }
  if (last_block_done(done, gridDim.x)) {
    double t = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) t += __ldcg(part + i);
    t = block_sum_d(t);
    if (threadIdx.x == 0) *out = t;
  }
}

// max |x| (normArray + deviceMaxReduce, seeded with FLT_MIN)
__global__ void __launch_bounds__(256) k_absmax(int64_t n, const float* __restrict__ x,
                                                double* __restrict__ part,
                                                uint32_t* __restrict__ done,
                                                double* __restrict__ out) {
  float m = FLT_MIN;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
       q += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[q]));
  __shared__ float sh[32];
  m = warp_max_f(m);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = FLT_MIN;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t = fmaxf(t, sh[w]);
    part[blockIdx.x] = (double)t;
  }
  if (last_block_done(done, gridDim.x)) {
    double t = (double)FLT_MIN;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) t = fmax(t, __ldcg(part + i));
    t = block_max_d(t);
    if (threadIdx.x == 0) *out = t;
  }
}

__global__ void k_scale(int64_t n, float a, float* __restrict__ x) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < n) x[q] *= a;
}

// y := a*x + y  (updateQ, src/functions.cu:3614, contracted to an FMA)
__global__ void k_axpy(int64_t n, float a, const float* __restrict__ x, float* __restrict__ y) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < n) y[q] = fmaf(a, x[q], y[q]);
}

// r := q * s  (getR)
__global__ void k_scaled_copy(int64_t n, float s, const float* __restrict__ q,
                              float* __restrict__ r) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n) r[k] = q[k] * s;
}

// The L-BFGS recursion with its scalars kept on the device: the dot
// products land in FP64 device scalars and these kernels form rho, alpha
// and beta from them with the host recursion's float operations, each
// rounded on its own (no contraction into FMAs, as the host code is
// compiled), so nothing is read back per dot product and the result is the
// host recursion's bit for bit.
//   first loop:  rho = 1 / (float)y.s (in double, then float), alpha =
//                rho (float)s.q, q -= alpha y
//   second loop: rho = 1.0f / (float)y.s, beta = rho (float)y.r,
//                r += (alpha - beta) s
__global__ void k_lbfgs_axpy(int64_t n, int second, const double* __restrict__ d1,
                             const double* __restrict__ d2, float* __restrict__ alpha,
                             const float* __restrict__ x, float* __restrict__ y) {
  __shared__ float coef_s;
  if (threadIdx.x == 0) {
    const float rho_den = (float)*d1;
    if (!second) {
      const float rho = rho_den != 0.0f ? (float)__ddiv_rn(1.0, (double)rho_den) : 0.0f;
      const float a = __fmul_rn(rho, (float)*d2);
      coef_s = -a;
      if (blockIdx.x == 0) *alpha = a;
    } else {
      const float rho = rho_den != 0.0f ? __fdiv_rn(1.0f, rho_den) : 0.0f;
      const float beta = __fmul_rn(rho, (float)*d2);
      coef_s = __fsub_rn(*alpha, beta);
    }
  }
  __syncthreads();
  const float coef = coef_s;
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < n) y[q] = fmaf(coef, x[q], y[q]);
}

// H0 scale: sum over planes of (float)s.y / (float)y.y where y.y != 0
__global__ void k_lbfgs_h0(const double* __restrict__ sy, const double* __restrict__ yy,
                           float* __restrict__ out) {
  if (threadIdx.x != 0) return;
  float s = 0.0f;
  for (int im = 0; im < 2; im++)
    if ((float)yy[im] != 0.0f) s = __fadd_rn(s, __fdiv_rn((float)sy[im], (float)yy[im]));
  *out = s;
}

// r := q * (*s)  (getR with the scale on the device)
__global__ void k_scaled_copy_dev(int64_t n, const float* __restrict__ s,
                                  const float* __restrict__ q, float* __restrict__ r) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n) r[k] = __fmul_rn(q[k], *s);
}

// calculateSandY for one plane, src/functions.cu:3635
__global__ void k_s_and_y(int64_t n, const float* __restrict__ xi, const float* __restrict__ xi_old,
                          const float* __restrict__ p, const float* __restrict__ p_old,
                          float* __restrict__ y, float* __restrict__ s) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n) return;
  y[q] = xi[q] - (-1.0f * xi_old[q]);
  s[q] = p[q] - p_old[q];
}

inline unsigned nblk(int64_t n) { return (unsigned)((n + 255) / 256); }

// SIGN of include/nrutil.h:55 on float magnitudes
inline float signf(float a, float b) { return b >= 0.0 ? std::fabs(a) : -std::fabs(a); }

struct Workspace {
  float *pcom, *xicom, *xt, *xi, *g, *h, *xi_old, *p_old, *q, *r;
};

// ---- device line search: one graph launch per linmin --------------------
// Graph: k_ls_begin, then a WHILE node whose body evaluates the objective at
// the controller's point and advances the controller (k_ls_step), which ends
// the loop.  The body has two branches: the Chi2 kernels (the first forms
// xt = p + x xi itself and writes it) and one kernel for the active priors
// (which forms xt per pixel too); k_ls_step waits for both.  One graph per
// set of buffers and objective gating, as for the evaluation graphs.
constexpr int kLsCap = 4096;  // objective evaluations of one search at most

struct LsEntry {
  const float* pcom;
  const float* xicom;
  float* xt;
  int flag, gate, positivity;
  cudaGraphExec_t exec;
  int64_t body_launches;
  uint64_t stamp;
};
struct LsCache {
  std::vector<LsEntry> e;
  cudaStream_t cap = nullptr;   // capture stream (the evaluation's main branch)
  cudaStream_t side = nullptr;  // the priors' branch
  cudaEvent_t fork = nullptr, join = nullptr;
  uint64_t clock = 0;
};
constexpr size_t kMaxLsGraphs = 4;

LsCache& ls_cache(Problem& P) {
  if (!P.ls_graphs) P.ls_graphs = new LsCache();
  return *static_cast<LsCache*>(P.ls_graphs);
}

gv_status build_ls_graph(Problem& P, LsCache& c, int64_t MN, const float* pcom,
                         const float* xicom, float* xt, int flag, int positivity, float floor_val,
                         float floor_cmp, const LsTerms& terms, cudaGraphExec_t* out,
                         int64_t* body_launches) {
  if (!c.cap) GV_CUDA(cudaStreamCreateWithFlags(&c.cap, cudaStreamNonBlocking));
  if (!c.side) GV_CUDA(cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking));
  if (!c.fork) GV_CUDA(cudaEventCreateWithFlags(&c.fork, cudaEventDisableTiming));
  if (!c.join) GV_CUDA(cudaEventCreateWithFlags(&c.join, cudaEventDisableTiming));
  cudaGraph_t root = nullptr;
  GV_CUDA(cudaGraphCreate(&root, 0));
  struct Guard {
    cudaGraph_t g;
    ~Guard() {
      if (g) cudaGraphDestroy(g);
    }
  } guard{root};
  const int64_t l0 = gv_launch_count();
  GV_CUDA(cudaStreamBeginCaptureToGraph(c.cap, root, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeRelaxed));
  gv_status s = ls_begin_launch(c.cap, P.d_ls, terms, 1.0e-7f, kLsCap);
  cudaGraph_t g1 = root;
  cudaError_t e = cudaStreamEndCapture(c.cap, &g1);
  if (s != GV_OK) return s;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture (line search start)");
  cudaGraphNode_t begin = nullptr;
  size_t nn = 1;
  GV_CUDA(cudaGraphGetNodes(root, &begin, &nn));
  if (nn != 1) {
    set_error("line-search graph: unexpected start nodes");
    return GV_ERR_CUDA;
  }
  cudaGraphConditionalHandle h;
  GV_CUDA(cudaGraphConditionalHandleCreate(&h, root, 1u, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t loop = nullptr;
  GV_CUDA(cudaGraphAddNode(&loop, root, &begin, nullptr, 1, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  const int64_t l1 = gv_launch_count();
  const cudaStream_t saved = P.stream;
  P.stream = c.cap;
  e = cudaStreamBeginCaptureToGraph(c.cap, body, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    P.stream = saved;
    return cuda_fail(e, "cudaStreamBeginCaptureToGraph (line search body)");
  }
  // evaluateXt at the controller's point happens in the FFT staging kernel
  // (and in the prior kernel, which runs beside the Chi2 kernels)
  const XtSource xs{pcom, xicom, &P.d_ls->x_req, floor_val, floor_cmp, positivity};
  bool stepped = false;
  s = ls_objective_launch(P, xt, flag, xs, c.side, c.fork, c.join, P.d_ls, h, &stepped);
  if (s == GV_OK && !stepped) s = ls_step_launch(c.cap, P.d_ls, P.d_scal, h);
  cudaGraph_t g2 = body;
  e = cudaStreamEndCapture(c.cap, &g2);
  P.stream = saved;
  *body_launches = gv_launch_count() - l1;
  add_launches(-(gv_launch_count() - l0));  // counted again at each replay
  if (s != GV_OK) return s;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture (line search body)");
  GV_CUDA(cudaGraphInstantiate(out, root, 0));
  return GV_OK;
}

}  // namespace

void ls_cache_free(Problem& P) {
  if (!P.ls_graphs) return;
  LsCache* c = static_cast<LsCache*>(P.ls_graphs);
  for (auto& g : c->e) cudaGraphExecDestroy(g.exec);
  if (c->cap) cudaStreamDestroy(c->cap);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->fork) cudaEventDestroy(c->fork);
  if (c->join) cudaEventDestroy(c->join);
  delete c;
  P.ls_graphs = nullptr;
}

namespace {

class Solver {
 public:
  Solver(Problem& P, const gv_opt_desc& o) : P_(P), o_(o) {
    MN_ = (int64_t)P.M * P.N;
    floor_val_ = -1.0f * P.eta * P.minpix;
    // the reference compares against -eta * minpix in FP64
    floor_cmp_ = float_below(-1.0 * P.eta * P.minpix);
  }

  gv_status init() {
    const size_t need = sizeof(float) * 2 * MN_ * 10;
    if (P_.opt_bytes < need) {
      cudaFree(P_.d_opt);
      P_.d_opt = nullptr;
      P_.opt_bytes = 0;
      GV_CUDA(cudaMalloc(&P_.d_opt, need));
      P_.opt_bytes = need;
    }
    float* b = P_.d_opt;
    const int64_t s = 2 * MN_;
    w_ = Workspace{b, b + s, b + 2 * s, b + 3 * s, b + 4 * s, b + 5 * s,
                   b + 6 * s, b + 7 * s, b + 8 * s, b + 9 * s};
    GV_CUDA(cudaMemsetAsync(P_.d_opt, 0, need, P_.stream));
    // the line search runs on the GPU inside a graph unless graphs are off
    // or GV_DEVICE_LS=0
    const char* dl = std::getenv("GV_DEVICE_LS");
    dev_ls_ = P_.use_graphs && !(dl && std::atoi(dl) == 0) && P_.terms.size() <= (size_t)kMaxTerms;
    if (dev_ls_ && !P_.d_ls) GV_CUDA(cudaMalloc(&P_.d_ls, sizeof(LsState)));
    if (o_.kind == GV_OPT_LBFGS) {
      const size_t ring = sizeof(float) * (size_t)MN_ * o_.K * 2;
      if (P_.lbfgs_bytes < 2 * ring) {
        cudaFree(P_.d_lbfgs);
        P_.d_lbfgs = nullptr;
        P_.lbfgs_bytes = 0;
        GV_CUDA(cudaMalloc(&P_.d_lbfgs, 2 * ring));
        P_.lbfgs_bytes = 2 * ring;
      }
      d_y_ = P_.d_lbfgs;
      d_s_ = P_.d_lbfgs + (size_t)MN_ * o_.K * 2;
      GV_CUDA(cudaMemsetAsync(P_.d_lbfgs, 0, 2 * ring, P_.stream));
      // device scalars of the recursion (GV_DEVICE_LBFGS=0: host scalars)
      const char* dv = std::getenv("GV_DEVICE_LBFGS");
      dev_lb_ = !(dv && std::atoi(dv) == 0);
      const size_t sc_bytes = sizeof(double) * (4 * (size_t)o_.K + 4) +
                              sizeof(float) * (2 * (size_t)o_.K + 1);
      if (dev_lb_ && P_.lbscal_bytes < sc_bytes) {
        cudaFree(P_.d_lbscal);
        P_.d_lbscal = nullptr;
        P_.lbscal_bytes = 0;
        GV_CUDA(cudaMalloc(&P_.d_lbscal, sc_bytes));
        P_.lbscal_bytes = sc_bytes;
      }
      if (dev_lb_) {
        lb_sc_ = reinterpret_cast<double*>(P_.d_lbscal);
        lb_f_ = reinterpret_cast<float*>(lb_sc_ + 4 * (size_t)o_.K + 4);
        GV_CUDA(cudaMemsetAsync(P_.d_lbscal, 0, sc_bytes, P_.stream));
      }
    }
    return GV_OK;
  }

  // ObjectiveFunction::calcFunction as float (the reference's return type)
  gv_status func(float* img, bool store_res, float* out) {
    gv_status s = P_.use_graphs ? eval_graph(P_, img, nullptr, 0, o_.flag, 1, store_res)
                                : objective_launch(P_, img, o_.flag, store_res);
    if (s != GV_OK) return s;
    s = fetch_scalars(P_, kSlotTerm0 + (int)P_.terms.size());
    if (s != GV_OK) return s;
    double f = 0.0;
    for (size_t t = 0; t < P_.terms.size(); t++)
      f += (double)P_.terms[t].lambda * P_.h_scal[kSlotTerm0 + t];
    n_obj_++;
    *out = (float)f;
    return GV_OK;
  }

  gv_status grad(float* img, float* xi, int iter) {
    n_grad_++;
    return P_.use_graphs ? eval_graph(P_, img, xi, iter, o_.flag, 2, false)
                         : gradient_launch(P_, img, xi, iter, o_.flag);
  }

  // f1dim: xt = pcom + x*xicom (floored on plane 0), then the objective.
  gv_status f1dim(float x, float* out) {
    k_eval_xt<<<nblk(2 * MN_), 256, 0, P_.stream>>>(MN_, x, nullptr, floor_val_, floor_cmp_,
                                                     o_.positivity, w_.pcom, w_.xicom, w_.xt);
    GV_LAUNCH("k_eval_xt");
    return func(w_.xt, false, out);
  }


  // Bracketing of a minimum along the line (golden-section steps with
  // parabolic extrapolation); constants of src/mnbrak.cu:35-37.
  gv_status bracket(float* ax, float* bx, float* cx, float* fa, float* fb, float* fc) {
    const double gold = 1.618034, glimit = 100.0, tiny = 1.0e-20;
    GV_TRY(f1dim(*ax, fa));
    GV_TRY(f1dim(*bx, fb));
    if (*fb > *fa) {
      std::swap(*ax, *bx);
      std::swap(*fa, *fb);
    }
    *cx = (float)(*bx + gold * (*bx - *ax));
    GV_TRY(f1dim(*cx, fc));
    while (*fb > *fc) {
      const float r = (*bx - *ax) * (*fb - *fc);
      const float q = (*bx - *cx) * (*fb - *fa);
      const float aq = std::fabs(q - r), at = (float)tiny;
      const float den = aq > at ? aq : at;
      float u = (float)(*bx - ((*bx - *cx) * q - (*bx - *ax) * r) / (2.0 * signf(den, q - r)));
      const float ulim = (float)(*bx + glimit * (*cx - *bx));
      float fu;
      if ((*bx - u) * (u - *cx) > 0.0) {
        GV_TRY(f1dim(u, &fu));
        if (fu < *fc) {
          *ax = *bx;
          *bx = u;
          *fa = *fb;
          *fb = fu;
          return GV_OK;
        } else if (fu > *fb) {
          *cx = u;
          *fc = fu;
          return GV_OK;
        }
        u = (float)(*cx + gold * (*cx - *bx));
        GV_TRY(f1dim(u, &fu));
      } else if ((*cx - u) * (u - ulim) > 0.0) {
        GV_TRY(f1dim(u, &fu));
        if (fu < *fc) {
          *bx = *cx;
          *cx = u;
          u = (float)(*cx + gold * (*cx - *bx));
          *fb = *fc;
          *fc = fu;
          GV_TRY(f1dim(u, &fu));
        }
      } else if ((u - ulim) * (ulim - *cx) >= 0.0) {
        u = ulim;
        GV_TRY(f1dim(u, &fu));
      } else {
        u = (float)(*cx + gold * (*cx - *bx));
        GV_TRY(f1dim(u, &fu));
      }
      *ax = *bx;
      *bx = *cx;
      *cx = u;
      *fa = *fb;
      *fb = *fc;
      *fc = fu;
    }
    return GV_OK;
  }

  // Brent's minimiser (parabolic interpolation with golden-section
  // fallback); constants of src/brent.cu:35-37, ITMAX 500.
  gv_status brent(float ax, float bx, float cx, float tol, float* xmin, float* fret) {
    const double cgold = 0.3819660, zeps = 1.0e-10;
    float a = ax < cx ? ax : cx, b = ax > cx ? ax : cx;
    float d = 0.0f, e = 0.0f, etemp, fu, fv, fw, fx, pp, q, r, tol1, tol2, u, v, w, x, xm;
    x = w = v = bx;
    GV_TRY(f1dim(x, &fx));
    fw = fv = fx;
    for (int it = 1; it <= 500; it++) {
      xm = (float)(0.5 * (a + b));
      tol1 = (float)(tol * std::fabs(x) + zeps);
      tol2 = (float)(2.0 * tol1);
      if (std::fabs(x - xm) <= (tol2 - 0.5 * (b - a))) {
        *xmin = x;
        *fret = fx;
        return GV_OK;
      }
      if (std::fabs(e) > tol1) {
        r = (x - w) * (fx - fv);
        q = (x - v) * (fx - fw);
        pp = (x - v) * q - (x - w) * r;
        q = (float)(2.0 * (q - r));
        if (q > 0.0) pp = -pp;
        q = std::fabs(q);
        etemp = e;
        e = d;
        if (std::fabs(pp) >= std::fabs(0.5 * q * etemp) || pp <= q * (a - x) ||
            pp >= q * (b - x)) {
          e = x >= xm ? a - x : b - x;
          d = (float)(cgold * e);
        } else {
          d = pp / q;
          u = x + d;
          if (u - a < tol2 || b - u < tol2) d = signf(tol1, xm - x);
        }
      } else {
        e = x >= xm ? a - x : b - x;
        d = (float)(cgold * e);
      }
      u = std::fabs(d) >= tol1 ? x + d : x + signf(tol1, d);
      GV_TRY(f1dim(u, &fu));
      if (fu <= fx) {
        if (u >= x) a = x; else b = x;
        v = w; w = x; x = u;
        fv = fw; fw = fx; fx = fu;
      } else {
        if (u < x) a = u; else b = u;
        if (fu <= fw || w == x) {
          v = w; w = u; fv = fw; fw = fu;
        } else if (fu <= fv || v == x || v == w) {
          v = u; fv = fu;
        }
      }
    }
    *xmin = x;
    *fret = fx;
    return GV_OK;
  }

  // linmin on the GPU: the whole bracket + Brent search as one graph launch
  gv_status linmin_device(float* p, float* xi, float* fret) {
    LsCache& c = ls_cache(P_);
    const int gate = P_.iteration > 0 ? 1 : 0;
    LsEntry* hit = nullptr;
    for (auto& g : c.e)
      if (g.pcom == w_.pcom && g.xicom == w_.xicom && g.xt == w_.xt && g.flag == o_.flag &&
          g.gate == gate && g.positivity == o_.positivity)
        hit = &g;
    if (!hit) {
      LsTerms terms{};
      terms.nterms = (int)P_.terms.size();
      for (size_t t = 0; t < P_.terms.size(); t++) terms.lambda[t] = P_.terms[t].lambda;
      cudaGraphExec_t exec = nullptr;
      int64_t body = 0;
      GV_TRY(build_ls_graph(P_, c, MN_, w_.pcom, w_.xicom, w_.xt, o_.flag, o_.positivity,
                            floor_val_, floor_cmp_, terms, &exec, &body));
      if (c.e.size() >= kMaxLsGraphs) {
        auto old = std::min_element(c.e.begin(), c.e.end(), [](const LsEntry& a,
                                                               const LsEntry& b) {
          return a.stamp < b.stamp;
        });
        cudaGraphExecDestroy(old->exec);
        c.e.erase(old);
      }
      c.e.push_back({w_.pcom, w_.xicom, w_.xt, o_.flag, gate, o_.positivity, exec, body, 0});
      hit = &c.e.back();
    }
    hit->stamp = ++c.clock;
    GV_CUDA(cudaMemcpyAsync(w_.pcom, p, sizeof(float) * 2 * MN_, cudaMemcpyDeviceToDevice, P_.stream));
    GV_CUDA(cudaMemcpyAsync(w_.xicom, xi, sizeof(float) * 2 * MN_, cudaMemcpyDeviceToDevice, P_.stream));
    GV_CUDA(cudaGraphLaunch(hit->exec, P_.stream));
    k_new_p<<<nblk(2 * MN_), 256, 0, P_.stream>>>(MN_, 0.0f, &P_.d_ls->xmin, floor_val_,
                                                   floor_cmp_, o_.positivity, p, xi);
    GV_LAUNCH("k_new_p");
    GV_TRY(fetch_scalars(P_, kSlotLs + 4));
    const int64_t evals = (int64_t)P_.h_scal[kSlotLs + 1];
    n_obj_ += evals;
    add_launches(1 + evals * hit->body_launches);
    *fret = (float)P_.h_scal[kSlotLs];
    if (P_.h_scal[kSlotLs + 2] != 0.0) {
      set_error("line search did not end within its evaluation limit (unbounded along the line?)");
      return GV_ERR_DEVICE;
    }
    if (verbose())
      std::fprintf(stderr, "Alpha for linear minimization = %.9g (f = %.9g)\n",
                   (float)P_.h_scal[kSlotLs + 3], *fret);
    return GV_OK;
  }

  // linmin, src/linmin.cu:52-110
  gv_status linmin(float* p, float* xi, float* fret) {
    if (dev_ls_) return linmin_device(p, xi, fret);
    GV_CUDA(cudaMemcpyAsync(w_.pcom, p, sizeof(float) * 2 * MN_, cudaMemcpyDeviceToDevice, P_.stream));
    GV_CUDA(cudaMemcpyAsync(w_.xicom, xi, sizeof(float) * 2 * MN_, cudaMemcpyDeviceToDevice, P_.stream));
    float ax = 0.0f, xx = 1.0f, bx, fa, fx, fb, xmin;
    GV_TRY(bracket(&ax, &xx, &bx, &fa, &fx, &fb));
    GV_TRY(brent(ax, xx, bx, 1.0e-7f, &xmin, fret));
    if (verbose()) std::fprintf(stderr, "Alpha for linear minimization = %.9g (f = %.9g)\n", xmin, *fret);
    k_new_p<<<nblk(2 * MN_), 256, 0, P_.stream>>>(MN_, xmin, nullptr, floor_val_, floor_cmp_,
                                                   o_.positivity, p, xi);
    GV_LAUNCH("k_new_p");
    return GV_OK;
  }

  gv_status dot(const float* a, const float* b, int64_t n, double* out) {
    const int nb = (int)std::min<int64_t>(nblk(n), P_.part_stride);
    double* part = P_.d_part;
    k_dot<<<nb, 256, 0, P_.stream>>>(n, a, b, part, P_.d_flags + kFlagOptDone,
                                     P_.d_scal + kSlotOpt);
    GV_LAUNCH("k_dot");
    GV_TRY(fetch_scalars(P_, kSlotOpt + 1));
    *out = P_.h_scal[kSlotOpt];
    return GV_OK;
  }

  gv_status absmax(const float* x, int64_t n, float* out) {
    const int nb = (int)std::min<int64_t>(nblk(n), P_.part_stride);
    k_absmax<<<nb, 256, 0, P_.stream>>>(n, x, P_.d_part, P_.d_flags + kFlagOptDone,
                                        P_.d_scal + kSlotOpt);
    GV_LAUNCH("k_absmax");
    GV_TRY(fetch_scalars(P_, kSlotOpt + 1));
    *out = (float)P_.h_scal[kSlotOpt];
    return GV_OK;
  }

  gv_status frprmn(float* img, gv_opt_report* rep) {
    const int64_t PMN = 2 * MN_;
    float fp, fret = 0.0f;
    GV_TRY(func(img, true, &fp));
    GV_TRY(grad(img, w_.xi, first_iter_));
    k_cg_init<<<nblk(PMN), 256, 0, P_.stream>>>(PMN, w_.g, w_.xi, w_.h);
    GV_LAUNCH("k_cg_init");
    for (int it = 1; it <= o_.total_iterations; it++) {
      rep->iterations = it;
      GV_TRY(linmin(img, w_.xi, &fret));
      if ((it >= 2 || first_iter_ > 0) && (double)fret <= f_target_) {
        rep->exit_reason = 4;
        break;
      }
      if (2.0f * std::fabs(fret - fp) <= o_.ftol * (std::fabs(fret) + std::fabs(fp) + 1.0e-10)) {
        rep->exit_reason = 1;
        break;
      }
      GV_TRY(func(img, true, &fp));
      if (verbose()) std::fprintf(stderr, "Iteration %d function value = %.9g\n", it, fp);
      GV_TRY(grad(img, w_.xi, it));
      const float den = std::max(fp, 1.0f);
      const int nb = (int)std::min<int64_t>(nblk(PMN), P_.part_stride);
      k_cg_stats<<<nb, 256, 0, P_.stream>>>(PMN, den, w_.xi, w_.g, img, P_.d_part,
                                             P_.part_stride, P_.d_flags + kFlagOptDone,
                                             P_.d_scal + kSlotOpt);
      GV_LAUNCH("k_cg_stats");
      GV_TRY(fetch_scalars(P_, kSlotOpt + 3));
      const float gg = (float)P_.h_scal[kSlotOpt], dgg = (float)P_.h_scal[kSlotOpt + 1];
      const float gmax = (float)P_.h_scal[kSlotOpt + 2];
      if (gmax < o_.gtol) {
        rep->exit_reason = 2;
        break;
      }
      if (gg == 0.0f) {
        rep->exit_reason = 3;
        break;
      }
      const float gam = std::max(0.0f, dgg / gg);
      k_new_xi<<<nblk(PMN), 256, 0, P_.stream>>>(PMN, gam, w_.g, w_.xi, w_.h);
      GV_LAUNCH("k_new_xi");
    }
    GV_TRY(func(img, true, &rep->f_final));
    return GV_OK;
  }

  gv_status lbfgs(float* img, gv_opt_report* rep) {
    const int64_t PMN = 2 * MN_;
    const int K = o_.K;
    float fp, fret = 0.0f;
    std::vector<float> alpha(2 * (size_t)K);
    GV_TRY(func(img, true, &fp));
    GV_TRY(grad(img, w_.xi, first_iter_));
    k_scale<<<nblk(PMN), 256, 0, P_.stream>>>(PMN, -1.0f, w_.xi);
    GV_LAUNCH("k_scale");
    auto slot = [&](float* base, int im, int k) { return base + MN_ * im * k + MN_ * im; };
    auto qslot = [&](float* base, int im, int k) { return base + MN_ * im + MN_ * k; };
    for (int it = 1; it <= o_.total_iterations; it++) {
      rep->iterations = it;
      GV_CUDA(cudaMemcpyAsync(w_.p_old, img, sizeof(float) * PMN, cudaMemcpyDeviceToDevice, P_.stream));
      GV_CUDA(cudaMemcpyAsync(w_.xi_old, w_.xi, sizeof(float) * PMN, cudaMemcpyDeviceToDevice, P_.stream));
      GV_TRY(linmin(img, w_.xi, &fret));
      if ((it >= 2 || first_iter_ > 0) && (double)fret <= f_target_) {
        rep->exit_reason = 4;
        break;
      }
      if ((fp - fret) / std::max({std::fabs(fret), std::fabs(fp), 1.0f}) <= o_.ftol) {
        rep->exit_reason = 1;
        break;
      }
      float m;
      GV_TRY(absmax(w_.xi, PMN, &m));
      const float max_per_it = std::max(0.0f, m);
      if (max_per_it <= o_.gtol) {
        rep->exit_reason = 2;
        break;
      }
      GV_TRY(func(img, true, &fp));
      GV_TRY(grad(img, w_.xi, it));
      const int lit = (it - 1) % K;
      for (int im = 0; im < 2; im++) {
        k_s_and_y<<<nblk(MN_), 256, 0, P_.stream>>>(MN_, w_.xi + MN_ * im, w_.xi_old + MN_ * im,
                                                    img + MN_ * im, w_.p_old + MN_ * im,
                                                    slot(d_y_, im, lit), slot(d_s_, im, lit));
        GV_LAUNCH("k_s_and_y");
      }
      // LBFGS_recursion
      const int par_M = std::min(K, it);
      GV_CUDA(cudaMemcpyAsync(w_.q, w_.xi, sizeof(float) * PMN, cudaMemcpyDeviceToDevice, P_.stream));
      if (dev_lb_) {
        GV_TRY(lbfgs_recursion_device(par_M, lit));
        continue;
      }
      std::fill(alpha.begin(), alpha.end(), 0.0f);
      for (int im = 0; im < 2; im++) {
        for (int k = par_M - 1; k >= 0; k--) {
          double d1, d2;
          GV_TRY(dot(slot(d_y_, im, k), slot(d_s_, im, k), MN_, &d1));
          const float rho_den = (float)d1;
          const float rho = rho_den != 0.0f ? (float)(1.0 / rho_den) : 0.0f;
          GV_TRY(dot(slot(d_s_, im, k), w_.q + MN_ * im, MN_, &d2));
          alpha[im * K + k] = rho * (float)d2;
          k_axpy<<<nblk(MN_), 256, 0, P_.stream>>>(MN_, -alpha[im * K + k], qslot(d_y_, im, k),
                                                   w_.q + MN_ * im);
          GV_LAUNCH("k_axpy");
        }
      }
      float sy_yy = 0.0f;
      for (int im = 0; im < 2; im++) {
        double sy, yy;
        GV_TRY(dot(slot(d_y_, im, lit), slot(d_s_, im, lit), MN_, &sy));
        GV_TRY(dot(slot(d_y_, im, lit), slot(d_y_, im, lit), MN_, &yy));
        if ((float)yy != 0.0f) sy_yy += (float)sy / (float)yy;
      }
      for (int im = 0; im < 2; im++) {
        k_scaled_copy<<<nblk(MN_), 256, 0, P_.stream>>>(MN_, sy_yy, w_.q + MN_ * im, w_.r + MN_ * im);
        GV_LAUNCH("k_scaled_copy");
        for (int k = 0; k < par_M; k++) {
          double d1, d2;
          GV_TRY(dot(slot(d_y_, im, k), slot(d_s_, im, k), MN_, &d1));
          const float rho_den = (float)d1;
          const float rho = rho_den != 0.0f ? 1.0f / rho_den : 0.0f;
          GV_TRY(dot(slot(d_y_, im, k), w_.r + MN_ * im, MN_, &d2));
          const float beta = rho * (float)d2;
          k_axpy<<<nblk(MN_), 256, 0, P_.stream>>>(MN_, alpha[im * K + k] - beta,
                                                   qslot(d_s_, im, k), w_.r + MN_ * im);
          GV_LAUNCH("k_axpy");
        }
      }
      k_scaled_copy<<<nblk(PMN), 256, 0, P_.stream>>>(PMN, -1.0f, w_.r, w_.xi);
      GV_LAUNCH("k_scaled_copy");
    }
    GV_TRY(func(img, true, &rep->f_final));
    return GV_OK;
  }

  // LBFGS_recursion (src/lbfgs.cu:202-341) with the scalars on the device:
  // the same kernels and dot products in the same order as the host
  // version, no read-back per dot product
  gv_status lbfgs_recursion_device(int par_M, int lit) {
    const int K = o_.K;
    auto slot = [&](float* base, int im, int k) { return base + MN_ * im * k + MN_ * im; };
    auto qslot = [&](float* base, int im, int k) { return base + MN_ * im + MN_ * k; };
    double* d1 = lb_sc_;          // [2K] y.s per plane and pair
    double* d2 = lb_sc_ + 2 * K;  // [2K] s.q, then y.r
    double* syy = lb_sc_ + 4 * K; // [4] s.y and y.y of the newest pair, per plane
    float* alpha = lb_f_;         // [2K]
    float* h0 = lb_f_ + 2 * K;    // [1]
    const unsigned nb1 = nblk(MN_);
    for (int im = 0; im < 2; im++) {
      for (int k = par_M - 1; k >= 0; k--) {
        GV_TRY(dot_to(slot(d_y_, im, k), slot(d_s_, im, k), MN_, d1 + im * K + k));
        GV_TRY(dot_to(slot(d_s_, im, k), w_.q + MN_ * im, MN_, d2 + im * K + k));
        k_lbfgs_axpy<<<nb1, 256, 0, P_.stream>>>(MN_, 0, d1 + im * K + k, d2 + im * K + k,
                                                 alpha + im * K + k, qslot(d_y_, im, k),
                                                 w_.q + MN_ * im);
        GV_LAUNCH("k_lbfgs_axpy");
      }
    }
    for (int im = 0; im < 2; im++) {
      GV_TRY(dot_to(slot(d_y_, im, lit), slot(d_s_, im, lit), MN_, syy + im));
      GV_TRY(dot_to(slot(d_y_, im, lit), slot(d_y_, im, lit), MN_, syy + 2 + im));
    }
    k_lbfgs_h0<<<1, 32, 0, P_.stream>>>(syy, syy + 2, h0);
    GV_LAUNCH("k_lbfgs_h0");
    for (int im = 0; im < 2; im++) {
      k_scaled_copy_dev<<<nb1, 256, 0, P_.stream>>>(MN_, h0, w_.q + MN_ * im, w_.r + MN_ * im);
      GV_LAUNCH("k_scaled_copy_dev");
      for (int k = 0; k < par_M; k++) {
        GV_TRY(dot_to(slot(d_y_, im, k), slot(d_s_, im, k), MN_, d1 + im * K + k));
        GV_TRY(dot_to(slot(d_y_, im, k), w_.r + MN_ * im, MN_, d2 + im * K + k));
        k_lbfgs_axpy<<<nb1, 256, 0, P_.stream>>>(MN_, 1, d1 + im * K + k, d2 + im * K + k,
                                                 alpha + im * K + k, qslot(d_s_, im, k),
                                                 w_.r + MN_ * im);
        GV_LAUNCH("k_lbfgs_axpy");
      }
    }
    const int64_t PMN = 2 * MN_;
    k_scaled_copy<<<nblk(PMN), 256, 0, P_.stream>>>(PMN, -1.0f, w_.r, w_.xi);
    GV_LAUNCH("k_scaled_copy");
    return GV_OK;
  }

  // FP64 dot product into a device scalar (no read-back)
  gv_status dot_to(const float* a, const float* b, int64_t n, double* out) {
    const int nb = (int)std::min<int64_t>(nblk(n), P_.part_stride);
    k_dot<<<nb, 256, 0, P_.stream>>>(n, a, b, P_.d_part, P_.d_flags + kFlagOptDone, out);
    GV_LAUNCH("k_dot");
    return GV_OK;
  }

  int64_t n_obj_ = 0, n_grad_ = 0;
  bool dev_ls_ = false;  // line search on the GPU (one graph launch per linmin)
  bool dev_lb_ = false;  // L-BFGS recursion scalars on the GPU
  double* lb_sc_ = nullptr;
  float* lb_f_ = nullptr;
  // stop once a line search reaches this value (priors active, i.e. from
  // the second iteration on); -inf: never
  double f_target_ = -INFINITY;
  // iteration number of the first gradient: 0 as the reference (priors off
  // during the first line search), 1 to have them count from the start
  int first_iter_ = 0;

 private:
  Problem& P_;
  gv_opt_desc o_;
  int64_t MN_;
  float floor_val_;
  float floor_cmp_;
  Workspace w_{};
  float* d_y_ = nullptr;
  float* d_s_ = nullptr;
};

}  // namespace

gv_status linmin(Problem& P, const gv_opt_desc& o, float* d_p, float* d_xi, float* fret,
                 int64_t* evals) {
  Solver s(P, o);
  gv_status st = s.init();
  if (st == GV_OK) st = s.linmin(d_p, d_xi, fret);
  if (st == GV_OK) {
    cudaError_t e = cudaStreamSynchronize(P.stream);
    if (e != cudaSuccess) st = cuda_fail(e, "linmin");
  }
  if (evals) *evals = s.n_obj_;
  return st;
}

gv_status optimize(Problem& P, const gv_opt_desc& o, float* d_img, gv_opt_report* rep,
                   double f_target, int first_iter) {
  if (o.kind != GV_OPT_FRPRMN && o.kind != GV_OPT_LBFGS) {
    set_error("unknown optimizer kind");
    return GV_ERR_INVALID;
  }
  if (o.total_iterations < 0 || (o.kind == GV_OPT_LBFGS && o.K <= 0)) {
    set_error("invalid optimizer iterations / memory");
    return GV_ERR_INVALID;
  }
  gv_opt_report r;
  std::memset(&r, 0, sizeof(r));
  const auto t0 = std::chrono::steady_clock::now();
  Solver s(P, o);
  s.f_target_ = f_target;
  s.first_iter_ = first_iter > 0 ? 1 : 0;
  gv_status st = s.init();
  if (st == GV_OK) st = o.kind == GV_OPT_FRPRMN ? s.frprmn(d_img, &r) : s.lbfgs(d_img, &r);
  if (st == GV_OK) {
    cudaError_t e = cudaStreamSynchronize(P.stream);
    if (e != cudaSuccess) st = cuda_fail(e, "optimize");
  }
  r.n_objective = s.n_obj_;
  r.n_gradient = s.n_grad_;
  r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rep) *rep = r;
  return st;
}

}  // namespace gv
