// Internal declarations of the gpuvmem_gb300 library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <string>
#include <vector>

#include "gpuvmem_gb300.h"

namespace gv {

// Constants as the reference defines them (include/MSFITSIO.cuh:52-54,
// include/functions.cuh:17-23).
constexpr double kPiD = 3.141592653589793238462643383279502884;
constexpr float kPiF = 3.14159265358979323846f;
constexpr float kLightSpeed = 2.99792458E8f;
constexpr double kRpDegD = kPiD / 180.0;
constexpr float kRZ = 1.2196698912665045f;

// Mask byte per pixel: bit 0 = noise < noise_cut (priors, DChi2),
// bit 1 = noise > noise_cut (clip2IWNoise).  Both are derived from the FP32
// noise image exactly as the reference compares it.
constexpr uint8_t kMaskIn = 1;
constexpr uint8_t kMaskClip = 2;

// Scalar slots in Problem::d_scal (FP64, device).
enum ScalarSlot {
  kSlotF = 0,         // objective value
  kSlotChi2 = 1,      // chi2 (0.5 * sum)
  kSlotTerm0 = 2,     // per-term values (up to kMaxTerms)
  kSlotOpt = 16,      // optimiser scratch (gg, dgg, gmax, dots ...)
  kSlotLs = 40,       // device line search: fret, evaluations, error
  kNumScal = 64
};
constexpr int kMaxTerms = 8;

// Word slots in Problem::d_flags (uint32, device).
enum FlagSlot {
  kFlagCvrMax = 0,    // max |w Vr| component of the last stored residuals (float bits)
  kFlagDirtyMax = 1,  // max |w Vo| component (float bits)
  kFlagErr = 2,       // non-zero: a kernel gave up on a bounded wait
  kFlagPsfMax = 3,    // max weight of a kept visibility (float bits)
  kFlagDegridDone = 4,  // blocks of k_degrid done (the last one finishes chi2)
  kFlagPriorDone = 5,   // blocks of k_prior_values done (the last one sums)
  kFlagOptDone = 6,     // blocks of an optimiser reduction done (the last one sums)
  kFlagBarCount = 8,    // grid barrier of k_objective_fused: arrivals
  kFlagBarGen = 9,      // grid barrier of k_objective_fused: generation
  kNumFlags = 10
};

struct Channel {
  float freq;
  int64_t nvis;   // visibilities of this channel (all, incl. zero weight)
  int64_t off;    // offset into the visibility arrays
  int64_t ngrid;  // visibilities inside the grid (weight kept)
};

struct ChanRange {
  int64_t off;
  int64_t ngrid;
};

struct Term {
  int kind;
  float lambda;
  int image_index;
  int image_to_add;
  float prior_value;
  float eta;
  float epsilon;
  float epsilon_b = 0.0f;
  float* d_prior = nullptr;  // [MN] GEntropy / GL1Norm prior image (owned by the Problem)
};

// Packed per-visibility streams, sorted by grid cell within each channel.
//   deg  : {cell (j1 << 16 | i1) as bits, du, dv, w}       16 B
//   vo   : observed visibility                              8 B
//   cvr  : w * (Vo - Vm), written by the chi2 pass          8 B
//   ph   : {FU, FV, GU bits, GV bits} phase constants       16 B
//          FU = frac(dx*u) * 2^32, FV = frac(dy*v) * 2^32 (exact mod 1),
//          GU = w*dx^2/2, GV = w*dy^2/2 (cycles per pixel^2)
//   wl   : w in wavelengths (float) for the non-separable w-term residual
struct Problem {
  int M = 0, N = 0, log2n = 0;
  double DELTAX = 0, DELTAY = 0, dx_rad = 0, dy_rad = 0, deltau = 0, deltav = 0;
  float xobs = 0, yobs = 0, nu_0 = 0, D = 0, pbf = 0, pbcut = 0;
  int pb = 1;
  float eta = -1, minpix = 0, threshold = 0, noise_cut = 0, fg_scale = 1;
  int normalize = 0;
  float vis_noise = 0, sum_weights = 0;
  double bmaj = 0, bmin = 0, bpa = 0;
  int64_t V = 0, Vgrid = 0, mask_pixels = 0;
  int engine = 1;
  double max_wrho = 0;  // bound of |w * rho| (cycles) over the data
  std::vector<Channel> chans;
  std::vector<Term> terms;

  int iteration = 0;    // Fi::iteration of every term
  cudaStream_t stream = 0;

  // device buffers
  float4* d_deg = nullptr;
  float2* d_vo = nullptr;
  float2* d_cvr = nullptr;
  uint4* d_ph = nullptr;
  float* d_wl = nullptr;
  int64_t* d_perm = nullptr;     // sorted position -> caller's index
  float* d_noise = nullptr;      // [MN]
  float* d_gcf = nullptr;        // [MN] gridding correction of gridded data, or null
  uint8_t* d_mask = nullptr;     // [MN]
  float* d_rho = nullptr;        // [MN] z - 1 + r^2/2 per pixel
  float2* d_grid = nullptr;      // [C][MN] model grids
  float2* d_twiddle = nullptr;   // [n] e^{+2 pi i m/n} (objective.cu smem_fft)
  float* d_beam_x = nullptr;     // [N] beam_coord of each column (attenuation)
  float* d_beam_y = nullptr;     // [M] beam_coord of each row
  float* d_rot_u = nullptr;      // [N] phase_rotate's u of each column (k_cols_fft)
  float* d_rot_v = nullptr;      // [M] phase_rotate's v of each row
  double* d_part = nullptr;      // reduction partials
  int part_stride = 0;           // partials per channel / term
  double* d_scal = nullptr;      // [kNumScal]
  double* h_scal = nullptr;      // pinned mirror
  double* h_many = nullptr;      // pinned term values of gv_objective_many
  size_t h_many_cap = 0;         // doubles h_many holds
  float* d_tmp = nullptr;        // [2*MN] scratch image (dchi2 channel etc.)
  float* d_opt = nullptr;        // optimiser workspace (allocated on demand)
  size_t opt_bytes = 0;
  float* d_lbfgs = nullptr;      // L-BFGS s/y rings
  size_t lbfgs_bytes = 0;
  void* d_lbscal = nullptr;      // L-BFGS recursion scalars (FP64 dots, float alphas)
  size_t lbscal_bytes = 0;
  float* d_chfreq = nullptr;     // [C] channel frequencies
  ChanRange* d_ranges = nullptr; // [C] kept-visibility ranges
  int64_t* d_chnvis = nullptr;   // [C] visibilities per channel (normalize)
  int64_t* d_kc_off = nullptr;   // [C+1] offsets of kept visibilities, channels concatenated
  int64_t* d_kc_one = nullptr;   // [2C] {0, ngrid_c} per channel
  float4* d_E = nullptr;         // [V] {e^{2 pi i FU/2^32}, e^{2 pi i FV/2^32}}
  uint32_t* d_flags = nullptr;   // [kNumFlags]
  float* tc_partial = nullptr;   // [tc_nsplit][MN] split-K partial images
  int tc_nsplit = 0;
  int tc_fast_anchor = 1;        // SFU anchor phasor (GV_TC_ACCURATE_ANCHOR=1 selects sincospif)
  int num_sms = 0;
  int use_graphs = 1;            // optimizer evaluations replayed from CUDA graphs
  int tc_pair_mode = -1;         // -1: GV_TC_PAIR / default, 0 single CTAs, 1 CTA pairs
  size_t tc_partial_cap = 0;     // split-K partial images the buffer holds
  float* d_epi = nullptr;        // [C][MN] DChi2 epilogue factors (allocated on first use)
  size_t epi_bytes = 0;
  int degrid_threads = 256;      // k_degrid block size
  int degrid_blocks = 0;         // k_degrid blocks per channel cap (0: part_stride)
  int fused = 0;                 // small images: the objective as one cooperative launch
                                 // (GV_FUSED=1 at creation turns it on)
  int fused_off = 0;             // > 0 while callers that run problems concurrently launch
  int fused_blocks[3] = {0, 0, 0};  // cooperative blocks of k_objective_fused (per image kind)
  void* graphs = nullptr;        // graph cache (graph.cu)
  void* ls_graphs = nullptr;     // device line-search graphs (optim.cu)
  struct LsState* d_ls = nullptr;  // device line-search state
};

// error state
void set_error(const std::string& msg);
gv_status cuda_fail(cudaError_t e, const char* what);

#define GV_CUDA(call)                                        \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return ::gv::cuda_fail(_e, #call); \
  } while (0)

// propagate a non-OK status
#ifndef GV_TRY
#define GV_TRY(expr)                 \
  do {                               \
    gv_status _s = (expr);           \
    if (_s != GV_OK) return _s;      \
  } while (0)
#endif

// Counts every kernel launch of the library (gv_launch_count) and turns a
// launch error into a status.
void count_launch();
void add_launches(int64_t n);
#define GV_LAUNCH(what)                                         \
  do {                                                          \
    ::gv::count_launch();                                       \
    cudaError_t _e = cudaGetLastError();                        \
    if (_e != cudaSuccess) return ::gv::cuda_fail(_e, what);     \
  } while (0)

// ---- device helpers shared by several translation units ---------------

// freq_to_wavelength, src/MSFITSIO.cu:36-39 (float)
__host__ __device__ inline float wavelength(float freq) { return kLightSpeed / freq; }

// Sky offset of pixel index k from the beam centre k0 in radians, as the
// reference's attenuation() forms it (FP64 product, rounded to float).
// Problem::d_beam_x / d_beam_y hold it per column / row, so the hot kernels
// do no FP64 arithmetic for it.
__host__ __device__ inline float beam_coord(int k, int k0, double delta) {
  return (float)((k - k0) * delta * kRpDegD);
}

// attenuation(), src/functions.cu:2304-2333, with the Gaussian and Airy
// beams of :2275-2302; float arithmetic as the reference, from the pixel's
// offsets x, y (beam_coord).  Split in two so a caller staging many
// channels of one pixel takes the radius once: beam_arc (the radius, with
// the multiply-add spelled out so every caller rounds it alike) and
// attenuation_arc (the beam at that radius and frequency).
__device__ __forceinline__ float beam_arc(float x, float y) {
  return sqrtf(__fmaf_rn(x, x, __fmul_rn(y, y)));
}

// attenuation_arc's per-frequency constants, taken once per channel by
// callers staging many pixels: the same operations in the same order, so
// the same values.
struct BeamAt {
  float lambda, fwhm, c, krz_pbf, D, cutoff;
  int pb;
};

__device__ __forceinline__ BeamAt beam_at(float freq, float D, float pbf, float cutoff, int pb) {
  BeamAt b;
  b.lambda = wavelength(freq);
  b.fwhm = pbf * b.lambda / D;
  b.c = 4.0f * logf(2.0f);
  b.krz_pbf = kRZ / pbf;
  b.D = D;
  b.cutoff = cutoff;
  b.pb = pb;
  return b;
}

__device__ __forceinline__ float attenuation_at(float arc, const BeamAt& b) {
  float atten;
  if (b.pb == GV_BEAM_GAUSSIAN) {
    const float r = arc / b.fwhm;
    atten = expf(-b.c * r * r);
  } else {
    atten = 1.0f;
    if (arc != 0.0f) {
      const float arg = kPiF * arc * b.D / b.lambda * b.krz_pbf;
      const float bj = j1f(arg);
      atten = 4.0f * (bj / arg) * (bj / arg);
    }
  }
  return arc <= b.cutoff ? atten : 0.0f;
}

__device__ inline float attenuation_arc(float arc, float freq, float D, float pbf, float cutoff,
                                        int pb) {
  return attenuation_at(arc, beam_at(freq, D, pbf, cutoff, pb));
}

__device__ inline float attenuation_xy(float x, float y, float freq, float D, float pbf,
                                       float cutoff, int pb) {
  return attenuation_arc(beam_arc(x, y), freq, D, pbf, cutoff, pb);
}

__device__ inline float attenuation(int i, int j, float xobs, float yobs,
                                    double DELTAX, double DELTAY, float freq,
                                    float D, float pbf, float cutoff, int pb) {
  return attenuation_xy(beam_coord(j, (int)xobs, DELTAX), beam_coord(i, (int)yobs, DELTAY), freq,
                        D, pbf, cutoff, pb);
}

// A thread's running sum of FP32 terms in FP32 instructions with Neumaier's
// compensation (Neumaier 1974): s + c carries the sum to about 2^-48
// relative for the few hundred terms a thread adds, as an FP64 accumulator
// would, without the FP64 pipe (a small fraction of the FP32 rate on this
// GPU).  value() hands the pair to the FP64 block and grid reductions.
struct CompSum {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float t = __fadd_rn(s, x);
    c = __fadd_rn(c, fabsf(s) >= fabsf(x) ? __fadd_rn(__fsub_rn(s, t), x)
                                           : __fadd_rn(__fsub_rn(x, t), s));
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// The largest float not above d: for a float v, (double)v > d exactly when
// v > float_below(d), so a comparison the reference makes in FP64 runs in
// FP32 with the same outcome.
inline float float_below(double d) {
  float f = (float)d;
  if ((double)f > d) f = std::nextafter(f, -HUGE_VALF);
  return f;
}

// True in every thread of the block that finishes last of `nblocks` (after
// each block stored its partials); that block resets the counter for the
// next launch.  It then combines the partials in a fixed order, so the
// result does not depend on which block finished last.
__device__ inline bool last_block_done(uint32_t* counter, uint32_t nblocks) {
  __shared__ int last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t prev = atomicAdd(counter, 1u);
    last = prev == nblocks - 1 ? 1 : 0;
    if (last) *counter = 0u;
  }
  __syncthreads();
  return last != 0;
}

// ---- device line search (linesearch.cu) ---------------------------------
// State of linmin's bracket + Brent search (src/linmin.cu:52-110,
// src/mnbrak.cu:44-98, src/brent.cu:43-121) kept in device memory, advanced
// by one thread after every objective evaluation.
struct LsState {
  int state, evals, steps, it, error, nterms, cap;
  float ax, bx, cx, fa, fb, fc, u, fu;
  float a, b, d, e, v, w, x, fv, fw, fx, tol;
  float x_req;        // the point the next evaluation is at
  float xmin, fret;   // the result
  float lambda[kMaxTerms];
};
struct LsTerms {
  int nterms;
  float lambda[kMaxTerms];
};
// k_ls_begin: a new search from (0, 1) with tolerance tol; asks for f(0)
gv_status ls_begin_launch(cudaStream_t st, LsState* s, LsTerms terms, float tol, int cap);
// k_ls_step: takes f at x_req from the scalars the objective left, advances
// the search to its next point or its end, and sets the graph's loop
// condition (1: evaluate again, 0: done); at the end fret, the evaluation
// count, the error flag and xmin go to scal[kSlotLs..kSlotLs+3]
gv_status ls_step_launch(cudaStream_t st, LsState* s, double* scal, cudaGraphConditionalHandle h);

// ---- entry points between translation units ----------------------------
gv_status setup_problem(Problem& P, const gv_problem_desc& d);
void free_problem(Problem& P);

// objective.cu
// A line-search point as the objective's input: xt = pcom + (*x_dev) xicom,
// plane 0 floored at floor_val (positivity), evaluateXt of
// src/functions.cu:2832-2864, formed inside the FFT staging (which writes xt)
// and, per pixel, inside the prior kernel of the line search
struct XtSource {
  const float* pcom;
  const float* xicom;
  const float* x_dev;
  float floor_val;
  float floor_cmp;  // float_below(-eta * minpix): v > floor_cmp as in FP64
  int positivity;
};
gv_status chi2_launch(Problem& P, float* d_img, int flag_opt, bool store_res,
                      const XtSource* xs = nullptr, double* term_out = nullptr,
                      uint32_t zero_terms = 0u);
gv_status prior_value_launch(Problem& P, int t, const float* d_img, int slot);
gv_status prior_grad_launch(Problem& P, int t, const float* d_img, float* d_dphi);
gv_status objective_launch(Problem& P, float* d_img, int flag_opt, bool store_res);
// Batches: the objectives of several problems (store_res on) in one
// cooperative launch.  batch_objective_args writes a problem's arguments
// (batch_arg_bytes() bytes, host) and its task counts per phase, or returns
// GV_ERR_UNSUPPORTED when the problem cannot run there (image above 512,
// priors before Chi2); batch_objective_launch runs np problems whose
// arguments and [3][np + 1] task offsets are in device memory.
size_t batch_arg_bytes();
gv_status batch_objective_args(Problem& P, float* d_img, int flag_opt, void* out, int tasks[3]);
gv_status batch_objective_launch(int np, const void* d_args, const int* d_off, int max_n,
                                 int max_tasks, uint32_t* d_bar, uint32_t* d_err, int num_sms,
                                 cudaStream_t st);
// With ls set (no fused launch, a degridding grid resident at once) the
// degridding's last block also takes the search's step and sets the loop
// condition cond (*stepped = true); otherwise the caller adds the step.
gv_status ls_objective_launch(Problem& P, float* d_xt, int flag_opt, const XtSource& xs,
                              cudaStream_t side, cudaEvent_t fork, cudaEvent_t join, LsState* ls,
                              cudaGraphConditionalHandle cond, bool* stepped);
gv_status fetch_scalars(Problem& P, int n);

// Device-wide sort / scan / run-length primitives (sortscan.cu).  Scratch
// sizes first, then the call; nothing is allocated inside.
template <class K, class V>
size_t radix_sort_scratch(int64_t n);
template <class K, class V>
gv_status radix_sort_pairs(void* scratch, size_t bytes, const K* kin, K* kout, const V* vin,
                           V* vout, int64_t n, int begin_bit, int end_bit, cudaStream_t st);
size_t scan_scratch(int64_t n);
template <class T>
gv_status exclusive_scan(void* scratch, size_t bytes, const T* in, T* out, int64_t n,
                         cudaStream_t st);
size_t rle_scratch(int64_t n);
gv_status run_length_encode(void* scratch, size_t bytes, const uint32_t* keys, int64_t n,
                            uint32_t* rkey, uint32_t* rstart, uint32_t* rcount, int64_t cap,
                            int* nruns, cudaStream_t st);
gv_status dchi2_launch(Problem& P, const float* d_img, int flag_opt, float* d_result);
gv_status dchi2_channel_launch(Problem& P, int c, float* d_out);
gv_status gradient_launch(Problem& P, float* d_img, float* d_xi, int iter, int flag_opt);
gv_status dirty_launch(Problem& P, float* d_out, bool psf = false);

// dchi2 engines
gv_status dchi2_direct(Problem& P, const float* d_img, int flag_opt, float* d_result,
                       int only_channel, int mode);
gv_status dchi2_tc(Problem& P, const float* d_img, int flag_opt, float* d_result,
                   int only_channel, int mode);
bool dchi2_tc_supported(const Problem& P);
int tc_tile_n(const Problem& P);
bool tc_pair(const Problem& P);
gv_status check_device_error(Problem& P);

// CUDA-graph replay (graph.cu); what: 1 objective, 3 objective + gradient
gv_status eval_graph(Problem& P, float* d_img, float* d_xi, int iter, int flag_opt, int what,
                     bool store);
void graph_cache_free(Problem& P);
void ls_cache_free(Problem& P);

// optimiser
gv_status autotune(Problem& P, gv_tune_report* rep);
gv_status error_images(Problem& P, float* d_img, float* d_err);
gv_status optimize(Problem& P, const gv_opt_desc& o, float* d_img, gv_opt_report* rep,
                   double f_target = -1e300, int first_iter = 0);
gv_status linmin(Problem& P, const gv_opt_desc& o, float* d_p, float* d_xi, float* fret,
                 int64_t* evals);

}  // namespace gv
