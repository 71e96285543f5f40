// Objective function on the GPU: chi2() (src/functions.cu:4323-4454) and the
// prior values/gradients (src/functions.cu:2878-3545,4633-4964), arranged
// as three passes per evaluation over all channels at once:
//
//   1. k_rows_fft   clip2IWNoise + calculateInu + apply_beam2I staged
//                   straight into shared memory, then the row pass of the
//                   2-D C2C inverse FFT (cuFFT CUFFT_INVERSE convention:
//                   unnormalised, exp(+i));
//   2. k_cols_fft   column pass of the FFT, with phase_rotate applied on the
//                   way out;
//   3. k_degrid     vis_mod + residual + chi2Vector + reduction: one stream
//                   over the cell-sorted visibilities, compensated per-thread
//                   sums combined in FP64, weighted residuals stored for
//                   DChi2.
//
// The FFT passes are radix-8 Stockham passes in shared memory with the
// butterflies in registers (four passes and barriers for a 2048-point line
// instead of eleven radix-2 stages).  With GV_FUSED=1 at creation, images
// up to 512 x 512 run the three passes and the prior values as one
// cooperative launch (k_objective_fused; bit-identical, but slower on the
// GB300 than the separate launches, whose kernel nodes cost 0.7 us against
// about 2 us for a grid-wide barrier).  No per-call allocation, no host
// synchronisation except the single scalar read-back at the end of an
// evaluation.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "gv_internal.cuh"
#include "ls_core.cuh"

namespace gv {

namespace {

// The arithmetic that more than one kernel performs on the same values (the
// FFT butterflies and twiddles, the phase rotation, the degridding's model
// and chi2 terms, the prior stencils) spells out every multiply-add with
// rounding intrinsics: the compiler never contracts those, so the separate
// kernels and the fused ones round each operation alike wherever the code
// is inlined (the compiler's choice of which product to fuse into an FMA
// can otherwise differ between inlining contexts).
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(__fmaf_rn(a.x, b.x, -__fmul_rn(a.y, b.y)),
                     __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x)));
}

// R-point inverse DFT (exp(+2 pi i r s / R), R = 2^LR <= 8) of v in
// registers, radix-2 decimation in frequency: the result is in bit-reversed
// order (X[r] = v[brev(r)]).  The twiddles are 1, i and (+-1 + i)/sqrt(2):
// multiplications by 1 and i are exact.
__device__ __forceinline__ float2 rot_turn(float2 d, int s, int m) {
  // d * e^{2 pi i s / m}, m in {2, 4, 8}, s < m / 2 (compile-time after
  // unrolling)
  const float c = 0.70710678118654752440f;
  if (s == 0) return d;
  if (m == 4 || s == 2) return make_float2(-d.y, d.x);                 // * i
  if (s == 1) return make_float2(__fmul_rn(c, d.x - d.y), __fmul_rn(c, d.x + d.y));  // * (1 + i)/sqrt 2
  return make_float2(__fmul_rn(c, -d.x - d.y), __fmul_rn(c, d.x - d.y));           // * (-1 + i)/sqrt 2
}

template <int LR>
__device__ __forceinline__ void dft_inv(float2 (&v)[1 << LR]) {
  constexpr int R = 1 << LR;
#pragma unroll
  for (int half = R / 2; half >= 1; half >>= 1) {
#pragma unroll
    for (int g = 0; g < R; g += 2 * half) {
#pragma unroll
      for (int s = 0; s < half; s++) {
        const float2 a = v[g + s], b = v[g + s + half];
        v[g + s] = make_float2(a.x + b.x, a.y + b.y);
        v[g + s + half] = rot_turn(make_float2(a.x - b.x, a.y - b.y), s, 2 * half);
      }
    }
  }
}

template <int LR>
__device__ __forceinline__ constexpr int brev_c(int r) {
  int o = 0;
  for (int b = 0; b < LR; b++) o |= ((r >> b) & 1) << (LR - 1 - b);
  return o;
}

// Shared-memory position of element e of an FFT line: one float2 of padding
// after every eight, so the first Stockham pass's writes (eight elements
// apart across the lanes) and the second's (runs of eight, 64 apart) fall in
// distinct banks.  A line of n elements takes fft_span(n) positions; the
// lines of a multi-column buffer are fft_stride(n) apart (four more, so four
// columns read row by row do not share banks either).
__device__ __forceinline__ int fpad(int e) { return e + (e >> 3); }
__host__ __device__ __forceinline__ int fft_span(int n) { return n + (n >> 3); }
__host__ __device__ __forceinline__ int fft_stride(int n) { return fft_span(n) + 4; }

// One Stockham autosort pass of radix R = 2^LR over `ncol` columns of length
// n = 2^log2n in shared memory (element e of column c at
// buf[c * fft_stride(n) + fpad(e)], natural order).
// Work item (c, j), j < n / R, reads x[j + r n/R] (r < R), multiplies by the
// twiddles e^{2 pi i r k / (Ns R)} with k = j mod Ns (table tw[m] =
// e^{2 pi i m / n}, read through L1), takes the R-point inverse DFT and
// writes y[(j / Ns) Ns R + k + r Ns] (Govindaraju et al., "High Performance
// Discrete Fourier Transforms on Graphics Processors", SC 2008).  In place:
// all items are read before a block barrier and written after it, so each
// thread holds its items' values in registers: max(VPT, R) of them, VPT the
// values per thread (ncol * n <= VPT * blockDim.x).
template <int LR, int VPT>
__device__ __forceinline__ void stockham_pass(float2* buf, int log2n, int ncol, int lNs,
                                              const float2* __restrict__ tw) {
  constexpr int R = 1 << LR;
  constexpr int kMaxItems = VPT / R > 1 ? VPT / R : 1;
  const int lq = log2n - LR;  // log2 of the items per column
  const int items = ncol << lq;
  float2 v[kMaxItems][R];
#pragma unroll
  for (int t = 0; t < kMaxItems; t++) {
    const int it = threadIdx.x + t * blockDim.x;
    if (it < items) {
      const int c = it >> lq, j = it & ((1 << lq) - 1);
      const float2* x = buf + c * fft_stride(1 << log2n);
#pragma unroll
      for (int r = 0; r < R; r++) v[t][r] = x[fpad(j + (r << lq))];
    }
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < kMaxItems; t++) {
    const int it = threadIdx.x + t * blockDim.x;
    if (it < items) {
      const int c = it >> lq, j = it & ((1 << lq) - 1);
      const int k = j & ((1 << lNs) - 1);
      if (lNs > 0) {
        const int step = k << (log2n - lNs - LR);  // r k n / (Ns R) = r * step
#pragma unroll
        for (int r = 1; r < R; r++) v[t][r] = cmul(v[t][r], __ldg(tw + r * step));
      }
      dft_inv<LR>(v[t]);
      float2* y = buf + c * fft_stride(1 << log2n);
      const int base = ((j >> lNs) << (lNs + LR)) + k;
#pragma unroll
      for (int r = 0; r < R; r++) y[fpad(base + (r << lNs))] = v[t][brev_c<LR>(r)];
    }
  }
  __syncthreads();
}

// In-place inverse FFT (cuFFT's CUFFT_INVERSE convention: exp(+i),
// unnormalised) of `ncol` independent columns of length n = 2^log2n held in
// shared memory (element e of column c at buf[c * fft_stride(n) + fpad(e)]),
// natural order in and out: radix-8
// Stockham passes, then one of radix 4 or 2.  The caller has synchronised
// the block after filling buf; needs ncol * n <= VPT * blockDim.x and
// n <= 2 * blockDim.x * max(1, VPT / 2).
template <int VPT>
__device__ void smem_fft(float2* buf, int log2n, int ncol, const float2* __restrict__ tw) {
  int lNs = 0;
  while (log2n - lNs >= 3) {
    stockham_pass<3, VPT>(buf, log2n, ncol, lNs, tw);
    lNs += 3;
  }
  if (log2n - lNs == 2) stockham_pass<2, VPT>(buf, log2n, ncol, lNs, tw);
  else if (log2n - lNs == 1) stockham_pass<1, VPT>(buf, log2n, ncol, lNs, tw);
}

// values per thread of the FFT passes: the separate row and column kernels
// (up to 4096 values over 256 threads) and the fused small-image kernel (up
// to 512 values over 256 threads)
constexpr int kVptLarge = 16;
constexpr int kVptSmall = 2;

// evaluateXt at one pixel (k_eval_xt's arithmetic): xt = pcom + x xicom,
// plane 0 floored when positivity is on, plane 1 free.
__device__ __forceinline__ void xt_value(const XtSource& xs, float x, float p0, float d0, float p1,
                                         float d1, float& i0, float& al) {
  const float v0 = fmaf(x, d0, p0);
  i0 = (xs.positivity && !(v0 > xs.floor_cmp)) ? xs.floor_val : v0;
  al = fmaf(x, d1, p1);
}

__device__ __forceinline__ void xt_pixel(const XtSource& xs, float x, int64_t MN, int64_t q,
                                         float& i0, float& al) {
  xt_value(xs, x, xs.pcom[q], xs.xicom[q], xs.pcom[MN + q], xs.xicom[MN + q], i0, al);
}

// What clip2IWNoise (src/functions.cu:2694-2719) leaves at one pixel.
struct ClipRule {
  float clip_i0, threshold;
  int flag_opt;
};

__device__ __forceinline__ void clip_pixel(uint8_t m, const ClipRule& cr, float& i0, float& al) {
  if (m & kMaskClip) {
    i0 = cr.clip_i0;
    al = 0.0f;
  } else if (i0 < cr.threshold && cr.flag_opt > 0) {
    al = 0.0f;
  }
}

struct StageParams {
  int M, N, log2n;
  int64_t MN;
  float xobs, yobs, nu_0, D, pbf, pbcut;
  int pb;
  double DELTAX, DELTAY;
  float eta, minpix, threshold, fg_scale;
  int flag_opt;
  int write_clip;
  const float* gcf;  // gridding correction, or null
  const float* beam_x;  // beam_coord per column / row
  const float* beam_y;
  XtSource xs;       // xs.pcom set: the image is xt = pcom + x xicom (written back)
};

// One staged pixel of a channel: calculateInu (src/functions.cu:3939-3966;
// powf(x, 0) is 1 exactly) floored at -eta * MINPIX, apply_beam2I
// (src/functions.cu:2424-2444) at beam radius arc, fg_scale, and apply_GCF
// (src/functions.cu:2468) when a correction is set.
__device__ __forceinline__ float stage_value(const StageParams& sp, float i0, float al, float arc,
                                             const BeamAt& beam, float nudiv, float floor_inu,
                                             int64_t q) {
  float inu = i0 * (al == 0.0f ? 1.0f : powf(nudiv, al));
  if (inu < floor_inu) inu = floor_inu;
  const float a = attenuation_at(arc, beam);
  float v = inu * a * sp.fg_scale;
  if (sp.gcf) v *= sp.gcf[q];
  return v;
}

// Pass 1 for row i of channel c: stage I_nu * A * fg_scale into buf (shared
// memory, n float2) and FFT the row with the twiddles tw (shared memory);
// the row goes to grid.  Every thread of the block takes part.
template <int VPT>
__device__ __forceinline__ void row_task(const StageParams& sp, const float* __restrict__ chfreq,
                                         float* __restrict__ img, const uint8_t* __restrict__ mask,
                                         const float2* tw, float2* __restrict__ grid, float2* buf,
                                         int i, int c) {
  const int n = sp.N;
  const float freq = chfreq[c];
  const float nudiv = freq / sp.nu_0;
  const float floor_inu = -1.0f * sp.eta * sp.minpix;
  const ClipRule cr{sp.eta > 0.0f ? 0.0f : (float)(-1.0 * sp.eta * sp.minpix), sp.threshold,
                    sp.flag_opt};
  const bool writer = sp.write_clip && c == 0;
  const bool from_xt = sp.xs.pcom != nullptr;
  const float x = from_xt ? __ldcg(sp.xs.x_dev) : 0.0f;
  const float by = __ldg(sp.beam_y + i);
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const int64_t q = (int64_t)n * i + j;
    float i0, al;
    if (from_xt) {
      xt_pixel(sp.xs, x, sp.MN, q, i0, al);
    } else {
      i0 = img[q];
      al = img[sp.MN + q];
    }
    // clip2IWNoise, src/functions.cu:2694-2719 (mutates the image: only the
    // pixels it changes are written back)
    const float i0_in = i0, al_in = al;
    clip_pixel(mask[q], cr, i0, al);
    if (writer && from_xt) {
      img[q] = i0;
      img[sp.MN + q] = al;
    } else if (writer) {
      if (i0 != i0_in) img[q] = i0;
      if (al != al_in) img[sp.MN + q] = al;
    }
    // calculateInu, src/functions.cu:3939-3966 (powf(x, 0) is 1 exactly)
    float inu = i0 * (al == 0.0f ? 1.0f : powf(nudiv, al));
    if (inu < floor_inu) inu = floor_inu;
    // apply_beam2I, src/functions.cu:2424-2444
    const float a = attenuation_xy(__ldg(sp.beam_x + j), by, freq, sp.D, sp.pbf, sp.pbcut, sp.pb);
    float v = inu * a * sp.fg_scale;
    if (sp.gcf) v *= sp.gcf[q];  // apply_GCF, src/functions.cu:2468
    buf[fpad(j)] = make_float2(v, 0.0f);
  }
  __syncthreads();
  smem_fft<VPT>(buf, sp.log2n, 1, tw);
  float2* out = grid + (int64_t)c * sp.MN + (int64_t)n * i;
  for (int j = threadIdx.x; j < n; j += blockDim.x) out[j] = buf[fpad(j)];
}

// Pass 1 for row i = blockIdx.x and every channel: the row's pixels (or the
// line search's xt) are read once -- each thread loads all of its pixels
// before it stores anything, so the loads are in flight together -- clipped
// (the clip written back once), then per channel staged as
// I_nu * A * fg_scale (* GCF) in shared memory and FFT'd into the channel's
// grid.  The same arithmetic per pixel and channel as row_task.  VPT: the
// row's values per thread (n / blockDim.x, at least 2).
template <int VPT>
__global__ void __launch_bounds__(256, VPT >= 16 ? 3 : 4)
    k_rows_fft(StageParams sp, const float* __restrict__ chfreq, int C, float* __restrict__ img,
               const uint8_t* __restrict__ mask, const float2* __restrict__ tw,
               float2* __restrict__ grid) {
  extern __shared__ float2 buf[];  // the row (fft_span(n)), its clipped I_nu0, alpha, beam radius
  const int n = sp.N, i = blockIdx.x;
  float* s_i0 = reinterpret_cast<float*>(buf + fft_span(n));
  float* s_al = s_i0 + n;
  float* s_arc = s_al + n;
  const float by = __ldg(sp.beam_y + i);
  const ClipRule cr{sp.eta > 0.0f ? 0.0f : (float)(-1.0 * sp.eta * sp.minpix), sp.threshold,
                    sp.flag_opt};
  const bool from_xt = sp.xs.pcom != nullptr;
  const float x = from_xt ? __ldcg(sp.xs.x_dev) : 0.0f;
  {
    float i0[VPT], al[VPT];
#pragma unroll
    for (int k = 0; k < VPT; k++) {
      const int j = threadIdx.x + k * blockDim.x;
      if (j < n) {
        const int64_t q = (int64_t)n * i + j;
        if (from_xt) {
          xt_pixel(sp.xs, x, sp.MN, q, i0[k], al[k]);
        } else {
          i0[k] = img[q];
          al[k] = img[sp.MN + q];
        }
      }
    }
#pragma unroll
    for (int k = 0; k < VPT; k++) {
      const int j = threadIdx.x + k * blockDim.x;
      if (j < n) {
        // clip2IWNoise, src/functions.cu:2694-2719 (mutates the image: only
        // the pixels it changes are written back)
        const int64_t q = (int64_t)n * i + j;
        const float i0_in = i0[k], al_in = al[k];
        clip_pixel(mask[q], cr, i0[k], al[k]);
        if (sp.write_clip && from_xt) {
          img[q] = i0[k];
          img[sp.MN + q] = al[k];
        } else if (sp.write_clip) {
          if (i0[k] != i0_in) img[q] = i0[k];
          if (al[k] != al_in) img[sp.MN + q] = al[k];
        }
        s_i0[j] = i0[k];  // read back by this thread only
        s_al[j] = al[k];
        s_arc[j] = beam_arc(__ldg(sp.beam_x + j), by);
      }
    }
  }
  const float floor_inu = -1.0f * sp.eta * sp.minpix;
  for (int c = 0; c < C; c++) {
    const float freq = chfreq[c];
    const float nudiv = freq / sp.nu_0;
    const BeamAt beam = beam_at(freq, sp.D, sp.pbf, sp.pbcut, sp.pb);
    // unrolled by two only: the transcendental functions of many pixels at
    // once would raise the register count and lower the occupancy
#pragma unroll 2
    for (int k = 0; k < VPT; k++) {
      const int j = threadIdx.x + k * blockDim.x;
      if (j < n) {
        buf[fpad(j)] = make_float2(
            stage_value(sp, s_i0[j], s_al[j], s_arc[j], beam, nudiv, floor_inu, (int64_t)n * i + j),
            0.0f);
      }
    }
    __syncthreads();
    smem_fft<VPT>(buf, sp.log2n, 1, tw);
    float2* out = grid + (int64_t)c * sp.MN + (int64_t)n * i;
#pragma unroll
    for (int k = 0; k < VPT; k++) {
      const int j = threadIdx.x + k * blockDim.x;
      if (j < n) out[j] = buf[fpad(j)];
    }
    __syncthreads();
  }
}

// phase_rotate (src/functions.cu:2483-2518) of one grid value in the
// reference's float arithmetic: u, v are x_phs / n * (j or j - n) and the row
// equivalent, in FP64 rounded to float (the tables hold them)
__device__ __forceinline__ float2 phase_rotated(float2 g, float u, float v) {
  const float phase = -2.0f * (u + v);
  float s, co;
  sincospif(phase, &s, &co);
  return cmul(g, make_float2(co, s));
}

// Pass 2 for columns j0 .. j0 + cb - 1 of grid G: column FFTs in buf
// (shared memory, cb * n float2), then phase_rotate (src/functions.cu:
// 2483-2518) in the reference's float arithmetic.  Load: how the grid is
// read (plain loads, or L2 loads when the grid was written earlier in the
// same kernel by other blocks).
template <bool kL2Loads, int VPT>
__device__ __forceinline__ void col_task(int N, int log2n, int cb, const float* __restrict__ rot_u,
                                         const float* __restrict__ rot_v, const float2* tw,
                                         float2* __restrict__ G, float2* buf, int j0) {
  const int n = N;
  const int lcb = __ffs(cb) - 1;  // cb is a power of two
  // every load of the thread first (cb n <= VPT blockDim.x), then the stores:
  // the loads are in flight together
  float2 v[VPT];
#pragma unroll
  for (int k = 0; k < VPT; k++) {
    const int idx = threadIdx.x + k * blockDim.x;
    if (idx < cb * n) {
      const float2* src = G + (int64_t)n * (idx >> lcb) + j0 + (idx & (cb - 1));
      v[k] = kL2Loads ? __ldcg(src) : *src;
    }
  }
#pragma unroll
  for (int k = 0; k < VPT; k++) {
    const int idx = threadIdx.x + k * blockDim.x;
    if (idx < cb * n) buf[(idx & (cb - 1)) * fft_stride(n) + fpad(idx >> lcb)] = v[k];
  }
  __syncthreads();
  smem_fft<VPT>(buf, log2n, cb, tw);
  for (int idx = threadIdx.x; idx < cb * n; idx += blockDim.x) {
    const int r = idx >> lcb, cc = idx & (cb - 1);
    const int j = j0 + cc;
    // u = xphs / n * (j or j - n), v likewise for the row, in FP64 rounded
    // to float (the tables hold them)
    G[(int64_t)n * r + j] = phase_rotated(buf[cc * fft_stride(n) + fpad(r)], __ldg(rot_u + j),
                                          __ldg(rot_v + r));
  }
}

// Pass 2: column FFTs of `cb` adjacent columns, then phase_rotate (512
// threads, at most 64 registers each, so two blocks share an SM).
__global__ void __launch_bounds__(512, 2) k_cols_fft(int N, int log2n, int64_t MN, int cb,
                                                     const float* __restrict__ rot_u,
                                                     const float* __restrict__ rot_v,
                                                     const float2* __restrict__ tw_g,
                                                     float2* __restrict__ grid) {
  extern __shared__ float2 sm[];
  col_task<false, kVptLarge>(N, log2n, cb, rot_u, rot_v, tw_g, grid + (int64_t)blockIdx.y * MN, sm,
                  blockIdx.x * cb);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// block-wide FP64 sum; result valid in thread 0
__device__ double block_sum(double v) {
  __shared__ double red[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = threadIdx.x < nw ? red[threadIdx.x] : 0.0;
  if (wid == 0) v = warp_sum(v);
  __syncthreads();
  return v;
}

// Sum of channel partials in a fixed order; writes 0.5 * sum to out
// (chi2(), src/functions.cu:4408-4451: per channel /V when normalize).
__device__ void finish_chi2(int C, int nb, const double* part, int part_stride,
                            const int64_t* __restrict__ nvis, int normalize, double* out) {
  __shared__ double tot;
  if (threadIdx.x == 0) tot = 0.0;
  __syncthreads();
  for (int c = 0; c < C; c++) {
    double v = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) v += __ldcg(part + (int64_t)c * part_stride + b);
    v = block_sum(v);
    if (threadIdx.x == 0) {
      if (normalize && nvis[c] > 0) v /= (double)nvis[c];
      tot += v;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = 0.5 * tot;
}

// Arguments of pass 3 (and of its finish).
struct DegridArgs {
  int N;
  int64_t MN;
  const ChanRange* __restrict__ ranges;
  const float4* __restrict__ deg;
  const float2* __restrict__ vo;
  const float2* __restrict__ grid;
  float2* __restrict__ cvr;
  int store;
  double* __restrict__ part;
  int part_stride;
  uint32_t* __restrict__ cmax;
  uint32_t* __restrict__ done;
  const int64_t* __restrict__ nvis;
  int normalize;
  double* __restrict__ chi2_out;
  double* __restrict__ term_out;
  uint32_t zero_terms;
  double* __restrict__ term_slots;
  // k_degrid_ls: the block that sums chi2 also takes the search's step
  // and sets the graph's loop condition
  LsState* ls;
  double* ls_scal;
  cudaGraphConditionalHandle ls_cond;
};

// the search's step, on the state where it lies in global memory (the
// previous evaluation's kernels wrote it; one thread reads and writes it
// here), so the degridding keeps its registers
__device__ __forceinline__ void degrid_ls_step(LsState* ls, double* scal,
                                               cudaGraphConditionalHandle h) {
  const bool more = ls::ls_step_on(*ls, scal);
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

// vis_mod (src/functions.cu:2557-2609): bilinear interpolation of the grid
// at the visibility's fractional cell offsets (d.y, d.z) from the four cell
// values v11 (row j1, column i1), v12 (j2, i1), v21 (j1, i2), v22 (j2, i2);
// the residual Vo - Vm (src/functions.cu:2663) goes to rr, ri.  Every
// degridding path calls this, so they round alike.
__device__ __forceinline__ void vis_residual(const float4& d, float2 o, float2 v11, float2 v12,
                                             float2 v21, float2 v22, float& rr, float& ri) {
  const float du = d.y, dv = d.z;
  const float w11 = __fmul_rn(1.0f - du, 1.0f - dv), w12 = __fmul_rn(1.0f - du, dv);
  const float w21 = __fmul_rn(du, 1.0f - dv), w22 = __fmul_rn(du, dv);
  const float mr =
      __fmaf_rn(w22, v22.x, __fmaf_rn(w21, v21.x, __fmaf_rn(w12, v12.x, __fmul_rn(w11, v11.x))));
  const float mi =
      __fmaf_rn(w22, v22.y, __fmaf_rn(w21, v21.y, __fmaf_rn(w12, v12.y, __fmul_rn(w11, v11.y))));
  rr = o.x - mr;
  ri = o.y - mi;
}

// chi2Vector (src/functions.cu:2867): w |Vr|^2
__device__ __forceinline__ float chi2_term(float w, float rr, float ri) {
  return __fmul_rn(w, __fmaf_rn(rr, rr, __fmul_rn(ri, ri)));
}

// Pass 3 for block b of nb of channel c: vis_mod + residual + chi2Vector
// over the block's share of the cell-sorted visibilities and the block's
// FP64 partial; the last of the nb * C blocks to finish adds the partials
// into the chi2 scalar.  kL2Loads: read the grid from L2 (written earlier in
// the same kernel by other blocks).
template <bool kL2Loads, bool kStep = false>
__device__ __forceinline__ void degrid_task(const DegridArgs& a, int b, int nb, int c, int C) {
  float mx = 0.0f;
  const ChanRange rg = a.ranges[c];
  const float2* __restrict__ G = a.grid + (int64_t)c * a.MN;
  const int N = a.N;
  const int nm1 = N - 1;
  CompSum acc;
  // the next visibility's record and Vo are loaded before this one's grid
  // cells are gathered, so the stream's latency overlaps the gathers
  const int64_t stride = (int64_t)nb * blockDim.x;
  int64_t k = b * (int64_t)blockDim.x + threadIdx.x;
  float4 d_next = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float2 o_next = make_float2(0.0f, 0.0f);
  if (k < rg.ngrid) {
    d_next = __ldcs(a.deg + rg.off + k);
    o_next = __ldcs(a.vo + rg.off + k);
  }
  for (; k < rg.ngrid; k += stride) {
    const float4 d = d_next;
    const float2 o = o_next;
    if (k + stride < rg.ngrid) {
      d_next = __ldcs(a.deg + rg.off + k + stride);
      o_next = __ldcs(a.vo + rg.off + k + stride);
    }
    const uint32_t cell = __float_as_uint(d.x);
    const int i1 = cell & 0xffff, j1 = cell >> 16;
    const int i2 = (i1 + 1) & nm1, j2 = (j1 + 1) & nm1;
    const float2 v11 = kL2Loads ? __ldcg(G + (int64_t)N * j1 + i1) : __ldg(G + (int64_t)N * j1 + i1);
    const float2 v12 = kL2Loads ? __ldcg(G + (int64_t)N * j2 + i1) : __ldg(G + (int64_t)N * j2 + i1);
    const float2 v21 = kL2Loads ? __ldcg(G + (int64_t)N * j1 + i2) : __ldg(G + (int64_t)N * j1 + i2);
    const float2 v22 = kL2Loads ? __ldcg(G + (int64_t)N * j2 + i2) : __ldg(G + (int64_t)N * j2 + i2);
    float rr, ri;
    vis_residual(d, o, v11, v12, v21, v22, rr, ri);
    acc.add(chi2_term(d.w, rr, ri));
    if (a.store) {
      const float2 cv = make_float2(d.w * rr, d.w * ri);
      __stcs(a.cvr + rg.off + k, cv);
      mx = fmaxf(mx, fmaxf(fabsf(cv.x), fabsf(cv.y)));
    }
  }
  if (a.store) {
    for (int s = 16; s > 0; s >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, s));
    if ((threadIdx.x & 31) == 0 && mx > 0.0f) atomicMax(a.cmax, __float_as_uint(mx));
  }
  const double bsum = block_sum(acc.value());
  if (threadIdx.x == 0) a.part[(int64_t)c * a.part_stride + b] = bsum;
  if (last_block_done(a.done, nb * C)) {
    finish_chi2(C, nb, a.part, a.part_stride, a.nvis, a.normalize, a.chi2_out);
    if (threadIdx.x == 0) {
      // ObjectiveFunction's per-term values: chi2's own slot, and 0 for the
      // priors the iteration gating leaves out
      if (a.term_out) *a.term_out = *a.chi2_out;
      for (int t = 0; t < 32; t++)
        if (a.zero_terms & (1u << t)) a.term_slots[t] = 0.0;
      if (kStep) degrid_ls_step(a.ls, a.ls_scal, a.ls_cond);
    }
  }
}

// Pass 3: vis_mod + residual + chi2Vector + partial reduction; the last
// block to finish adds the partials into the chi2 scalar.
__global__ void __launch_bounds__(256) k_degrid(DegridArgs a) {
  degrid_task<false>(a, blockIdx.x, gridDim.x, blockIdx.y, gridDim.y);
}

// The same inside the line search's graph loop: the last block also steps
// the search and sets the loop's condition.
__global__ void __launch_bounds__(256) k_degrid_ls(DegridArgs a) {
  degrid_task<false, true>(a, blockIdx.x, gridDim.x, blockIdx.y, gridDim.y);
}

// ---- priors ---------------------------------------------------------------

struct PriorParams {
  int kind;
  int N;
  int64_t MN;
  float lambda, G, eta, eps, eps_b;
  const float* prior;  // GEntropy / GL1Norm prior image
};

// Value of one pixel, src/functions.cu:2882 (L1), 3036 (S), 3238 (TV),
// 3353 (TSV), 3443 (L), 3114 (SGVector), 2954 (GL1), 3141 (QP); the caller
// has checked the mask.
template <class Img>
__device__ __forceinline__ float prior_pixel(const PriorParams& pp, const Img& I, int i, int j) {
  const int N = pp.N;
  const float c = I[(int64_t)N * i + j];
  switch (pp.kind) {
    case GV_FI_ENTROPY:
      return c * logf((c / pp.G) + (pp.eta + 1.0f));
    case GV_FI_L1:
      return sqrtf(__fmaf_rn(c, c, pp.eps));
    case GV_FI_TSV:
      if (i < N - 1 && j < N - 1) {
        const float dx = c - I[(int64_t)N * i + j + 1];
        const float dy = c - I[(int64_t)N * (i + 1) + j];
        return __fmaf_rn(dx, dx, __fmul_rn(dy, dy));
      }
      return c;
    case GV_FI_TV:
      if (i < N - 1 && j < N - 1) {
        const float r = I[(int64_t)N * i + j + 1];
        const float d = I[(int64_t)N * (i + 1) + j];
        return sqrtf(__fmaf_rn(r - c, r - c, __fmul_rn(d - c, d - c)) + pp.eps);
      }
      return c;
    case GV_FI_LAPLACIAN:
      if (i > 0 && i < N - 1 && j > 0 && j < N - 1) {
        const float c2 = __fmul_rn(2.0f, c);
        const float Dx = (I[(int64_t)N * i + j - 1] - c2) + I[(int64_t)N * i + j + 1];
        const float Dy = (I[(int64_t)N * (i - 1) + j] - c2) + I[(int64_t)N * (i + 1) + j];
        return __fmul_rn(__fmul_rn(0.5f, Dx + Dy), Dx + Dy);
      }
      return c;
    case GV_FI_GENTROPY: {
      const float G = pp.prior[(int64_t)N * i + j];
      return c * logf((c / G) + (pp.eta + 1.0f));
    }
    case GV_FI_GL1: {
      const float g = pp.prior[(int64_t)N * i + j];
      return sqrtf(__fmaf_rn(c, c, pp.eps)) / (sqrtf(__fmaf_rn(g, g, pp.eps)) + pp.eps_b);
    }
    case GV_FI_QUADRATIC:
      if (i > 0 && i < N - 1 && j > 0 && j < N - 1) {
        const float l = I[(int64_t)N * i + j - 1], r = I[(int64_t)N * i + j + 1];
        const float d = I[(int64_t)N * (i + 1) + j], u = I[(int64_t)N * (i - 1) + j];
        const float qp = __fmaf_rn(c - d, c - d,
                                   __fmaf_rn(c - u, c - u,
                                             __fmaf_rn(c - r, c - r, __fmul_rn(c - l, c - l))));
        return qp / 2.0f;
      }
      return c;
  }
  return 0.0f;
}

// Gradient of one pixel before lambda, src/functions.cu:2917 (DL1), 3057
// (DS), 3284 (DTV), 3395 (DTSV), 3488 (DL, with its d - r - u - l sign),
// 3131 (DSG), 2993 (DGL1), 3190 (DQ, with its 4c - d + u + r + l).
__device__ __forceinline__ float prior_grad_pixel(const PriorParams& pp,
                                                  const float* __restrict__ I, int i, int j) {
  const int N = pp.N;
  const float c = I[(int64_t)N * i + j];
  const bool inner = i > 0 && i < N - 1 && j > 0 && j < N - 1;
#define P_(r, cc) I[(int64_t)N * (r) + (cc)]
  switch (pp.kind) {
    case GV_FI_ENTROPY:
      return logf((c / pp.G) + (pp.eta + 1.0f)) + 1.0f / (1.0f + (((pp.eta + 1.0f) * pp.G) / c));
    case GV_FI_L1:
      return c / sqrtf(c * c + pp.eps);
    case GV_FI_TSV:
      if (inner) return 8.0f * c - 2.0f * (P_(i - 1, j) + P_(i, j - 1) + P_(i + 1, j) + P_(i, j + 1));
      return c;
    case GV_FI_TV:
      if (inner) {
        const float d = P_(i + 1, j), u = P_(i - 1, j), r = P_(i, j + 1), l = P_(i, j - 1);
        const float dl = P_(i + 1, j - 1), ru = P_(i - 1, j + 1);
        const float num0 = 2.0f * c - r - d, num1 = c - l, num2 = c - u;
        const float den0 = sqrtf((c - r) * (c - r) + (c - d) * (c - d) + pp.eps);
        const float den1 = sqrtf((l - c) * (l - c) + (l - dl) * (l - dl) + pp.eps);
        const float den2 = sqrtf((u - ru) * (u - ru) + (u - c) * (u - c) + pp.eps);
        return num0 / den0 + num1 / den1 + num2 / den2;
      }
      return c;
    case GV_FI_LAPLACIAN:
      if (i > 1 && i < N - 2 && j > 1 && j < N - 2) {
        return 20.0f * c - 8.0f * (P_(i + 1, j) - P_(i, j + 1) - P_(i - 1, j) - P_(i, j - 1)) +
               2.0f * (P_(i + 1, j - 1) + P_(i + 1, j + 1) + P_(i - 1, j - 1) + P_(i - 1, j + 1)) +
               P_(i + 2, j) + P_(i, j + 2) + P_(i - 2, j) + P_(i, j - 2);
      }
      return 0.0f;
    case GV_FI_GENTROPY: {
      const float G = pp.prior[(int64_t)N * i + j];
      return logf((c / G) + (pp.eta + 1.0f)) + 1.0f / (1.0f + (((pp.eta + 1.0f) * G) / c));
    }
    case GV_FI_GL1: {
      const float g = pp.prior[(int64_t)N * i + j];
      return c / (sqrtf(c * c + pp.eps) * (sqrtf(g * g + pp.eps) + pp.eps_b));
    }
    case GV_FI_QUADRATIC:
      if (inner) return 2.0f * (4.0f * c - P_(i + 1, j) + P_(i - 1, j) + P_(i, j + 1) + P_(i, j - 1));
      return c;
  }
#undef P_
  return 0.0f;
}

// Images the prior values read.  PlainImage: an image in memory.  XtImage:
// the line search's xt = pcom + x xicom, formed per pixel with the FFT
// staging's arithmetic and clipped as clip2IWNoise leaves it (Chi2, the
// first term, clips the image the priors then see), so the priors need not
// wait for the staging kernel to write xt.
struct PlainImage {
  const float* p;
  __device__ void bind() {}
  __device__ __forceinline__ float operator[](int64_t q) const { return p[q]; }
};

struct XtImage {
  XtSource xs;
  const uint8_t* mask;
  int64_t MN;
  ClipRule cr;
  int plane;
  float x;
  __device__ void bind() { x = __ldcg(xs.x_dev); }
  __device__ __forceinline__ float operator[](int64_t q) const {
    float i0, al;
    xt_pixel(xs, x, MN, q, i0, al);
    clip_pixel(mask[q], cr, i0, al);
    return plane ? al : i0;
  }
};

// ClipImage: the image as clip2IWNoise leaves it, formed per pixel (the
// clip is idempotent, so the value is the same whether or not the staging
// has written the clipped pixel back yet); read through L2, as the image is
// written in the same kernel.
struct ClipImage {
  const float* p;
  const uint8_t* mask;
  int64_t MN;
  ClipRule cr;
  int plane;
  __device__ void bind() {}
  __device__ __forceinline__ float operator[](int64_t q) const {
    float i0 = __ldcg(p + q), al = __ldcg(p + MN + q);
    clip_pixel(mask[q], cr, i0, al);
    return plane ? al : i0;
  }
};

template <class Img>
struct PriorSet {
  int n;
  PriorParams pp[kMaxTerms];
  Img img[kMaxTerms];
  double* part[kMaxTerms];  // gridDim.x partial sums per term
  double* out[kMaxTerms];   // the term's value
};

// Values of n prior terms, block b of nb of term t: the block's partial, and
// the last of the nb * n blocks to finish sums each term's partials in a
// fixed order.
template <class Img>
__device__ __forceinline__ void prior_task(const PriorSet<Img>& ps, const uint8_t* __restrict__ mask,
                                           uint32_t* __restrict__ done, int b, int nb, int t) {
  const PriorParams& pp = ps.pp[t];
  Img I = ps.img[t];
  I.bind();
  CompSum acc;
  for (int64_t q = b * (int64_t)blockDim.x + threadIdx.x; q < pp.MN;
       q += (int64_t)nb * blockDim.x) {
    if (!(mask[q] & kMaskIn)) continue;
    const int i = (int)(q / pp.N), j = (int)(q - (int64_t)i * pp.N);
    acc.add(prior_pixel(pp, I, i, j));
  }
  const double bsum = block_sum(acc.value());
  if (threadIdx.x == 0) ps.part[t][b] = bsum;
  if (last_block_done(done, nb * ps.n)) {
    for (int u = 0; u < ps.n; u++) {
      double v = 0.0;
      for (int k = threadIdx.x; k < nb; k += blockDim.x) v += __ldcg(ps.part[u] + k);
      v = block_sum(v);
      if (threadIdx.x == 0) *ps.out[u] = v;
    }
  }
}

// Values of n prior terms (blockIdx.y = term).
template <class Img>
__global__ void __launch_bounds__(256) k_prior_values(PriorSet<Img> ps,
                                                      const uint8_t* __restrict__ mask,
                                                      uint32_t* __restrict__ done) {
  prior_task(ps, mask, done, blockIdx.x, gridDim.x, blockIdx.y);
}

__global__ void __launch_bounds__(256) k_prior_grad(PriorParams pp, const float* __restrict__ I,
                                                    const uint8_t* __restrict__ mask,
                                                    float* __restrict__ dphi) {
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < pp.MN;
       q += (int64_t)gridDim.x * blockDim.x) {
    if (!(mask[q] & kMaskIn)) continue;
    const int i = (int)(q / pp.N), j = (int)(q - (int64_t)i * pp.N);
    const float g = prior_grad_pixel(pp, I, i, j) * pp.lambda;
    dphi[q] += g;  // AddToDPhi, src/functions.cu:3890
  }
}

// ---- small images: the whole objective in one cooperative launch --------
//
// Below 512 x 512 an evaluation is a few microseconds of work spread over
// four dependent launches, and the launches set its time.  k_objective_fused
// runs the same passes in one cooperative launch (every block resident):
//   A  row tasks (pass 1) and prior-value tasks, then a grid barrier;
//   B  column tasks (pass 2), then a grid barrier;
//   C  degridding tasks (pass 3); the last task to finish sums chi2.
// Every task is the corresponding kernel's block, with the same block size
// and the same partial-sum slots, so the results are bit-identical to the
// four launches.  Data written in the kernel is read back through L2
// (ld.global.cg), never through a block's L1.

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier of a cooperative launch.  bar[0] counts arrivals, bar[1]
// is the generation: the last block to arrive resets the count and advances
// the generation.  The wait is bounded (1 s): on time-out the error word
// gets bit 16 and false is returned in every thread of the block (the
// caller leaves the kernel).
__device__ bool grid_barrier(uint32_t* bar, uint32_t* err) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t gen = ld_acquire_gpu(bar + 1);
    __threadfence();
    const uint32_t prev = atomicAdd(bar, 1u);
    int good = 1;
    if (prev == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const uint64_t t0 = global_ns();
      while (ld_acquire_gpu(bar + 1) == gen) {
        __nanosleep(32);
        if (global_ns() - t0 > 1000000000ull) {
          atomicOr(err, 16u);
          good = 0;
          break;
        }
      }
    }
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

template <class Img>
struct FusedArgs {
  StageParams sp;
  const float* chfreq;
  float* img;
  const uint8_t* mask;
  const float2* tw;  // FFT twiddles e^{2 pi i m / n}
  const float* rot_u;
  const float* rot_v;
  int C;
  int cb;          // columns per column task
  int nb_deg;      // degridding tasks per channel (k_degrid's blocks)
  int nb_prior;    // prior tasks per term (k_prior_values' blocks)
  DegridArgs da;
  PriorSet<Img> ps;
  uint32_t* prior_done;
  uint32_t* bar;   // [2] grid barrier
  uint32_t* err;
};

template <class Img>
__global__ void __launch_bounds__(256, 2) k_objective_fused(FusedArgs<Img> f) {
  extern __shared__ float2 sm[];
  const int n = f.sp.N;
  float2* buf = sm;  // cb columns, fft_stride(n) apart
  const float2* tw = f.tw;
  float2* grid = const_cast<float2*>(f.da.grid);
  // A: rows of every channel, then the prior-value tasks
  const int nrow = n * f.C;
  const int ntask_a = nrow + f.nb_prior * f.ps.n;
  for (int t = blockIdx.x; t < ntask_a; t += gridDim.x) {
    if (t < nrow) {
      row_task<kVptSmall>(f.sp, f.chfreq, f.img, f.mask, tw, grid, buf, t % n, t / n);
    } else {
      const int u = t - nrow;
      prior_task(f.ps, f.mask, f.prior_done, u % f.nb_prior, f.nb_prior, u / f.nb_prior);
    }
    __syncthreads();
  }
  if (!grid_barrier(f.bar, f.err)) return;
  // B: columns
  const int ncg = n / f.cb;
  for (int t = blockIdx.x; t < ncg * f.C; t += gridDim.x) {
    col_task<true, kVptSmall>(n, f.sp.log2n, f.cb, f.rot_u, f.rot_v, tw, grid + (int64_t)(t / ncg) * f.sp.MN,
                   buf, (t % ncg) * f.cb);
    __syncthreads();
  }
  if (!grid_barrier(f.bar, f.err)) return;
  // C: degridding and chi2
  for (int t = blockIdx.x; t < f.nb_deg * f.C; t += gridDim.x)
    degrid_task<true>(f.da, t % f.nb_deg, f.nb_deg, t / f.nb_deg, f.C);
}

// ---- batches: the objectives of several problems in one cooperative launch
//
// k_objective_fused_batch runs k_objective_fused's three phases over the
// tasks of every problem of a batch: off[] holds, per phase, the prefix sums
// of the problems' task counts (an offset table), and a block finds the
// problem of its task by binary search.  Each task is the same block
// computation with the same partial slots as in the single-problem launch,
// so every problem's values are bit-identical to its own launch.

template <class Img>
struct FusedBatch {
  const FusedArgs<Img>* args;  // [np] per-problem arguments (device memory)
  const int* off;              // [3][np + 1] task offsets of phases A, B, C
  int np;
  int clear_cmax;              // zero every problem's max |w Vr| word first
  uint32_t* bar;               // [2] grid barrier
  uint32_t* err;
};

__device__ __forceinline__ int task_problem(const int* off, int np, int t) {
  int lo = 0, hi = np;  // off[lo] <= t < off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= t) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <class Img>
__global__ void __launch_bounds__(256, 2) k_objective_fused_batch(FusedBatch<Img> fb) {
  extern __shared__ float2 sm[];
  const int* offA = fb.off;
  const int* offB = fb.off + fb.np + 1;
  const int* offC = fb.off + 2 * (fb.np + 1);
  if (fb.clear_cmax && blockIdx.x == 0)
    for (int p = threadIdx.x; p < fb.np; p += blockDim.x) *fb.args[p].da.cmax = 0u;
  // A: rows of every channel of every problem, then its prior-value tasks
  for (int t = blockIdx.x; t < __ldg(offA + fb.np); t += gridDim.x) {
    const int p = task_problem(offA, fb.np, t);
    const FusedArgs<Img>& f = fb.args[p];
    const int u = t - __ldg(offA + p);
    const int n = f.sp.N, nrow = n * f.C;
    if (u < nrow) {
      row_task<kVptSmall>(f.sp, f.chfreq, f.img, f.mask, f.tw, const_cast<float2*>(f.da.grid),
                          sm, u % n, u / n);
    } else {
      const int v = u - nrow;
      prior_task(f.ps, f.mask, f.prior_done, v % f.nb_prior, f.nb_prior, v / f.nb_prior);
    }
    __syncthreads();
  }
  if (!grid_barrier(fb.bar, fb.err)) return;
  // B: columns
  for (int t = blockIdx.x; t < __ldg(offB + fb.np); t += gridDim.x) {
    const int p = task_problem(offB, fb.np, t);
    const FusedArgs<Img>& f = fb.args[p];
    const int u = t - __ldg(offB + p);
    const int n = f.sp.N, ncg = n / f.cb;
    col_task<true, kVptSmall>(n, f.sp.log2n, f.cb, f.rot_u, f.rot_v, f.tw,
                              const_cast<float2*>(f.da.grid) + (int64_t)(u / ncg) * f.sp.MN, sm,
                              (u % ncg) * f.cb);
    __syncthreads();
  }
  if (!grid_barrier(fb.bar, fb.err)) return;
  // C: degridding and chi2
  for (int t = blockIdx.x; t < __ldg(offC + fb.np); t += gridDim.x) {
    const int p = task_problem(offC, fb.np, t);
    const FusedArgs<Img>& f = fb.args[p];
    const int u = t - __ldg(offC + p);
    degrid_task<true>(f.da, u % f.nb_deg, f.nb_deg, u / f.nb_deg, f.C);
  }
}

}  // namespace

// Columns per block of the column pass: 8192 / n (8K complex values, 64 KB
// of shared memory: at 2048^2 four columns, so each row segment a warp reads
// is one 32-byte sector), fewer while the launch would have under two blocks
// per SM (small images: 256^2 runs 256 one-column blocks).
static int cols_per_block(int n, int channels, int num_sms) {
  int cb = 8192 / n;
  if (cb < 1) cb = 1;
  if (cb > 16) cb = 16;
  while (cb > 1 && (int64_t)(n / cb) * channels < 2 * (int64_t)num_sms) cb >>= 1;
  return cb;
}

static StageParams stage_params(const Problem& P, int flag_opt, int write_clip,
                                const XtSource* xs) {
  StageParams sp;
  sp.M = P.M;
  sp.N = P.N;
  sp.log2n = P.log2n;
  sp.MN = (int64_t)P.M * P.N;
  sp.xobs = P.xobs;
  sp.yobs = P.yobs;
  sp.nu_0 = P.nu_0;
  sp.D = P.D;
  sp.pbf = P.pbf;
  sp.pbcut = P.pbcut;
  sp.pb = P.pb;
  sp.DELTAX = P.DELTAX;
  sp.DELTAY = P.DELTAY;
  sp.eta = P.eta;
  sp.minpix = P.minpix;
  sp.threshold = P.threshold;
  sp.fg_scale = P.fg_scale;
  sp.flag_opt = flag_opt;
  sp.write_clip = write_clip;
  sp.gcf = P.d_gcf;
  sp.beam_x = P.d_beam_x;
  sp.beam_y = P.d_beam_y;
  sp.xs = xs ? *xs : XtSource{nullptr, nullptr, nullptr, 0.0f, 0.0f, 0};
  return sp;
}

// Model grids of all channels for image d_img (clip written back when
// write_clip).
gv_status model_grids_launch(Problem& P, float* d_img, int flag_opt, int write_clip,
                             const XtSource* xs = nullptr) {
  const int n = P.N, C = (int)P.chans.size();
  const StageParams sp = stage_params(P, flag_opt, write_clip, xs);
  // row pass: one block of 256 threads per row, n / 256 values a thread;
  // shared memory: the row's values, its clipped I_nu0 and alpha, beam radii
  const size_t sm1 = sizeof(float2) * fft_span(n) + 3 * sizeof(float) * n;
  auto rows = [&](auto kern) -> gv_status {
    if (sm1 > 48 * 1024)
      GV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1));
    kern<<<n, 256, sm1, P.stream>>>(sp, P.d_chfreq, C, d_img, P.d_mask, P.d_twiddle, P.d_grid);
    GV_LAUNCH("k_rows_fft");
    return GV_OK;
  };
  gv_status s = n <= 512 ? rows(k_rows_fft<2>)
                         : (n <= 1024 ? rows(k_rows_fft<4>)
                                      : (n <= 2048 ? rows(k_rows_fft<8>) : rows(k_rows_fft<16>)));
  if (s != GV_OK) return s;
  // column pass: cb columns per block, 16 values a thread
  const int cb = cols_per_block(n, C, P.num_sms);
  const int threads2 = cb * n > 4096 ? 512 : 256;
  const size_t sm2 = sizeof(float2) * (size_t)cb * fft_stride(n);
  if (sm2 > 48 * 1024)
    GV_CUDA(cudaFuncSetAttribute(k_cols_fft, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2));
  k_cols_fft<<<dim3(n / cb, C), threads2, sm2, P.stream>>>(n, P.log2n, sp.MN, cb, P.d_rot_u,
                                                           P.d_rot_v, P.d_twiddle, P.d_grid);
  GV_LAUNCH("k_cols_fft");
  return GV_OK;
}

// k_degrid's blocks per channel
static int degrid_blocks(const Problem& P) {
  int64_t maxg = 1;
  for (auto& ch : P.chans) maxg = std::max<int64_t>(maxg, ch.ngrid);
  const int th = P.degrid_threads;
  const int cap = P.degrid_blocks > 0 ? std::min(P.degrid_blocks, P.part_stride) : P.part_stride;
  const int nb = (int)std::min<int64_t>((maxg + th - 1) / th, cap);
  return nb < 1 ? 1 : nb;
}

static DegridArgs degrid_args(Problem& P, bool store_res, double* term_out, uint32_t zero_terms) {
  const int64_t MN = (int64_t)P.M * P.N;
  return DegridArgs{P.N, MN, P.d_ranges, P.d_deg, P.d_vo, P.d_grid, P.d_cvr,
                    store_res ? 1 : 0, P.d_part, P.part_stride, P.d_flags + kFlagCvrMax,
                    P.d_flags + kFlagDegridDone, P.d_chnvis, P.normalize,
                    P.d_scal + kSlotChi2, term_out, zero_terms, P.d_scal + kSlotTerm0,
                    nullptr, nullptr, 0};
}

static int prior_blocks(const Problem& P) {
  const int64_t MN = (int64_t)P.M * P.N;
  return (int)std::min<int64_t>((MN + 255) / 256, P.part_stride);
}

// Whether the objective of P runs as k_objective_fused: images up to
// 512 x 512 (where launches dominate), k_degrid's default block size (the
// fused tasks reproduce its 256-thread blocks), and no caller running
// several problems at once (cooperative launches must not share the GPU
// with each other).
static bool fused_ok(const Problem& P) {
  return P.fused && P.fused_off == 0 && P.N <= 512 && P.degrid_threads == 256;
}

template <class Img>
struct ImgKind;
template <>
struct ImgKind<PlainImage> {
  static constexpr int k = 0;
};
template <>
struct ImgKind<ClipImage> {
  static constexpr int k = 1;
};
template <>
struct ImgKind<XtImage> {
  static constexpr int k = 2;
};

// The objective's passes (and the prior values of ps) in one cooperative
// launch; same outputs as model_grids_launch + k_degrid (+ k_prior_values).
template <class Img>
static FusedArgs<Img> fused_args(Problem& P, float* d_img, int flag_opt, bool store_res,
                                 const XtSource* xs, double* term_out, uint32_t zero_terms,
                                 const PriorSet<Img>& ps) {
  const int C = (int)P.chans.size();
  FusedArgs<Img> f{};
  f.sp = stage_params(P, flag_opt, 1, xs);
  f.chfreq = P.d_chfreq;
  f.img = d_img;
  f.mask = P.d_mask;
  f.tw = P.d_twiddle;
  f.rot_u = P.d_rot_u;
  f.rot_v = P.d_rot_v;
  f.C = C;
  f.cb = 1;
  f.nb_deg = degrid_blocks(P);
  f.nb_prior = prior_blocks(P);
  f.da = degrid_args(P, store_res, term_out, zero_terms);
  f.ps = ps;
  f.prior_done = P.d_flags + kFlagPriorDone;
  f.bar = P.d_flags + kFlagBarCount;
  f.err = P.d_flags + kFlagErr;
  return f;
}

template <class Img>
static gv_status fused_launch(Problem& P, float* d_img, int flag_opt, bool store_res,
                              const XtSource* xs, double* term_out, uint32_t zero_terms,
                              const PriorSet<Img>& ps) {
  const int n = P.N, C = (int)P.chans.size();
  const FusedArgs<Img> f = fused_args(P, d_img, flag_opt, store_res, xs, term_out, zero_terms, ps);
  const size_t smem = sizeof(float2) * (size_t)f.cb * fft_stride(n);
  int& blocks = P.fused_blocks[ImgKind<Img>::k];
  if (blocks == 0) {
    // every block must be resident at once: at most the occupancy bound,
    // two blocks per SM at most, and no more than the largest pass has tasks
    int occ = 0;
    GV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_objective_fused<Img>, 256,
                                                          smem));
    if (occ < 1) {
      set_error("k_objective_fused does not fit on an SM");
      return GV_ERR_UNSUPPORTED;
    }
    const int tasks = std::max(n * C + f.nb_prior * kMaxTerms, f.nb_deg * C);
    blocks = std::max(1, std::min(P.num_sms * std::min(occ, 2), tasks));
  }
  if (store_res) GV_CUDA(cudaMemsetAsync(P.d_flags + kFlagCvrMax, 0, sizeof(uint32_t), P.stream));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = P.stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  GV_CUDA(cudaLaunchKernelEx(&cfg, k_objective_fused<Img>, f));
  GV_LAUNCH("k_objective_fused");
  return GV_OK;
}

gv_status chi2_launch(Problem& P, float* d_img, int flag_opt, bool store_res,
                      const XtSource* xs, double* term_out, uint32_t zero_terms) {
  if (fused_ok(P)) {
    PriorSet<PlainImage> none{};
    return fused_launch(P, d_img, flag_opt, store_res, xs, term_out, zero_terms, none);
  }
  gv_status s = model_grids_launch(P, d_img, flag_opt, 1, xs);
  if (s != GV_OK) return s;
  const int C = (int)P.chans.size();
  const int nb = degrid_blocks(P);
  if (store_res) GV_CUDA(cudaMemsetAsync(P.d_flags + kFlagCvrMax, 0, sizeof(uint32_t), P.stream));
  const DegridArgs da = degrid_args(P, store_res, term_out, zero_terms);
  k_degrid<<<dim3(nb, C), P.degrid_threads, 0, P.stream>>>(da);
  GV_LAUNCH("k_degrid");
  return GV_OK;
}

static PriorParams prior_params(const Problem& P, const Term& t) {
  PriorParams pp;
  pp.kind = t.kind;
  pp.N = P.N;
  pp.MN = (int64_t)P.M * P.N;
  pp.lambda = t.lambda;
  pp.G = t.prior_value;
  pp.eta = t.eta;
  pp.eps = t.epsilon;
  pp.eps_b = t.epsilon_b;
  pp.prior = t.d_prior;
  return pp;
}

static double* prior_part(Problem& P, int t) {
  return P.d_part + (int64_t)P.part_stride * (P.chans.size() + t);
}

template <class Img>
static gv_status prior_values_launch(Problem& P, cudaStream_t st, const PriorSet<Img>& ps) {
  k_prior_values<Img><<<dim3(prior_blocks(P), ps.n), 256, 0, st>>>(ps, P.d_mask,
                                                                    P.d_flags + kFlagPriorDone);
  GV_LAUNCH("k_prior_values");
  return GV_OK;
}

// Values of the terms ts[0..n) of image d_img, into d_scal[slot[k]].
static gv_status prior_values_plain(Problem& P, const int* ts, const int* slots, int n,
                                    const float* d_img) {
  PriorSet<PlainImage> ps{};
  ps.n = n;
  const int64_t MN = (int64_t)P.M * P.N;
  for (int k = 0; k < n; k++) {
    const Term& tm = P.terms[ts[k]];
    ps.pp[k] = prior_params(P, tm);
    ps.img[k] = PlainImage{d_img + MN * tm.image_index};
    ps.part[k] = prior_part(P, ts[k]);
    ps.out[k] = P.d_scal + slots[k];
  }
  return prior_values_launch(P, P.stream, ps);
}

gv_status prior_value_launch(Problem& P, int t, const float* d_img, int slot) {
  return prior_values_plain(P, &t, &slot, 1, d_img);
}

gv_status prior_grad_launch(Problem& P, int t, const float* d_img, float* d_dphi) {
  const Term& tm = P.terms[t];
  PriorParams pp = prior_params(P, tm);
  const int64_t MN = pp.MN;
  // TVariation::addToDphi adds into plane 0 whatever imageToAdd is
  // (src/totalvariation.cu:48)
  const int add = tm.kind == GV_FI_TV ? 0 : tm.image_to_add;
  int nb = (int)std::min<int64_t>((MN + 255) / 256, 8 * P.num_sms);
  k_prior_grad<<<nb, 256, 0, P.stream>>>(pp, d_img + MN * tm.image_index, P.d_mask,
                                         d_dphi + MN * add);
  GV_LAUNCH("k_prior_grad");
  return GV_OK;
}

// The active priors of an objective whose first term is Chi2 (so they see
// the clipped image) as one prior set over the clipped image d_img; false
// when the terms do not have that form.
static bool clip_prior_set(Problem& P, float* d_img, int flag_opt, uint32_t zero,
                           PriorSet<ClipImage>* ps) {
  if (P.terms.empty() || P.terms[0].kind != GV_FI_CHI2) return false;
  const int64_t MN = (int64_t)P.M * P.N;
  const ClipRule cr{P.eta > 0.0f ? 0.0f : (float)(-1.0 * P.eta * P.minpix), P.threshold,
                    flag_opt};
  *ps = PriorSet<ClipImage>{};
  for (size_t t = 1; t < P.terms.size(); t++) {
    const Term& tm = P.terms[t];
    if (tm.kind == GV_FI_CHI2) return false;
    if (zero & (1u << t)) continue;
    const int k = ps->n++;
    ps->pp[k] = prior_params(P, tm);
    ps->img[k] = ClipImage{d_img, P.d_mask, MN, cr, tm.image_index};
    ps->part[k] = prior_part(P, (int)t);
    ps->out[k] = P.d_scal + kSlotTerm0 + t;
  }
  return true;
}

// Iteration gating of the objective: the priors Chi2's kernel zeroes.
static uint32_t gated_terms(const Problem& P) {
  uint32_t zero = 0u;
  for (size_t t = 0; t < P.terms.size(); t++)
    if (P.terms[t].kind != GV_FI_CHI2 && !(P.iteration > 0 && P.terms[t].lambda != 0.0f))
      zero |= 1u << t;
  return zero;
}

size_t batch_arg_bytes() { return sizeof(FusedArgs<ClipImage>); }

gv_status batch_objective_args(Problem& P, float* d_img, int flag_opt, void* out,
                               int tasks[3]) {
  if (!(P.N <= 512 && P.degrid_threads == 256)) return GV_ERR_UNSUPPORTED;
  const uint32_t zero = gated_terms(P);
  PriorSet<ClipImage> ps{};
  if (!clip_prior_set(P, d_img, flag_opt, zero, &ps)) return GV_ERR_UNSUPPORTED;
  const FusedArgs<ClipImage> f =
      fused_args(P, d_img, flag_opt, true, nullptr, P.d_scal + kSlotTerm0, zero, ps);
  const int C = (int)P.chans.size();
  tasks[0] = P.N * C + f.nb_prior * ps.n;
  tasks[1] = (P.N / f.cb) * C;
  tasks[2] = f.nb_deg * C;
  std::memcpy(out, &f, sizeof(f));
  return GV_OK;
}

gv_status batch_objective_launch(int np, const void* d_args, const int* d_off, int max_n,
                                 int max_tasks, uint32_t* d_bar, uint32_t* d_err, int num_sms,
                                 cudaStream_t st) {
  FusedBatch<ClipImage> fb{static_cast<const FusedArgs<ClipImage>*>(d_args), d_off, np, 1, d_bar,
                           d_err};
  const size_t smem = sizeof(float2) * (size_t)fft_stride(max_n);
  int occ = 0;
  GV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_objective_fused_batch<ClipImage>,
                                                        256, smem));
  if (occ < 1) {
    set_error("k_objective_fused_batch does not fit on an SM");
    return GV_ERR_UNSUPPORTED;
  }
  const int blocks = std::max(1, std::min(num_sms * std::min(occ, 2), max_tasks));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  GV_CUDA(cudaLaunchKernelEx(&cfg, k_objective_fused_batch<ClipImage>, fb));
  GV_LAUNCH("k_objective_fused_batch");
  return GV_OK;
}

// ObjectiveFunction::calcFunction; values land in d_scal[kSlotTerm0 + t].
// Terms are evaluated in list order; consecutive active priors share one
// launch.
gv_status objective_launch(Problem& P, float* d_img, int flag_opt, bool store_res) {
  // Chi2 also writes its term slot and zeroes the slots of the priors the
  // iteration gating leaves out
  bool has_chi2 = false;
  uint32_t zero = 0u;
  for (size_t t = 0; t < P.terms.size(); t++) {
    if (P.terms[t].kind == GV_FI_CHI2) has_chi2 = true;
    else if (!(P.iteration > 0 && P.terms[t].lambda != 0.0f)) zero |= 1u << t;
  }
  PriorSet<ClipImage> ps{};
  if (fused_ok(P) && clip_prior_set(P, d_img, flag_opt, zero, &ps))
    return fused_launch(P, d_img, flag_opt, store_res, nullptr, P.d_scal + kSlotTerm0, zero, ps);
  int run[kMaxTerms], slots[kMaxTerms], nrun = 0;
  auto flush = [&]() -> gv_status {
    const int n = nrun;
    nrun = 0;
    return n ? prior_values_plain(P, run, slots, n, d_img) : GV_OK;
  };
  for (size_t t = 0; t < P.terms.size(); t++) {
    const Term& tm = P.terms[t];
    gv_status s = GV_OK;
    if (tm.kind == GV_FI_CHI2) {
      s = flush();
      if (s == GV_OK) s = chi2_launch(P, d_img, flag_opt, store_res, nullptr, P.d_scal + kSlotTerm0 + t, zero);
    } else if (has_chi2 && (zero & (1u << t))) {
      // zeroed by the chi2 kernel
    } else if (P.iteration > 0 && tm.lambda != 0.0f) {
      if (nrun == kMaxTerms) s = flush();
      run[nrun] = (int)t;
      slots[nrun] = kSlotTerm0 + (int)t;
      nrun++;
    } else {
      GV_CUDA(cudaMemsetAsync(P.d_scal + kSlotTerm0 + t, 0, sizeof(double), P.stream));
    }
    if (s != GV_OK) return s;
  }
  return flush();
}

// One objective evaluation of the line search at the controller's point:
// the Chi2 kernels on P.stream (the staging kernel forms xt and writes it
// to d_xt), the active priors in one launch on `side`, forked from P.stream
// through `fork` and joined back through `join`; the priors form xt
// themselves, so both branches run at once.  With `ls` (and a degridding
// grid that is resident at once) the degridding runs after the join and its
// last block also steps the search: one kernel node fewer per evaluation in
// the graph's loop (*stepped = true).
gv_status ls_objective_launch(Problem& P, float* d_xt, int flag_opt, const XtSource& xs,
                              cudaStream_t side, cudaEvent_t fork, cudaEvent_t join, LsState* ls,
                              cudaGraphConditionalHandle cond, bool* stepped) {
  *stepped = false;
  int ichi2 = -1;
  uint32_t zero = 0u;
  for (size_t t = 0; t < P.terms.size(); t++) {
    if (P.terms[t].kind == GV_FI_CHI2) {
      if (ichi2 < 0) ichi2 = (int)t;
    } else if (!(P.iteration > 0 && P.terms[t].lambda != 0.0f)) {
      zero |= 1u << t;
    }
  }
  if (ichi2 < 0) {
    set_error("a line-search evaluation needs the Chi2 term");
    return GV_ERR_UNSUPPORTED;
  }
  PriorSet<XtImage> ps{};
  const int64_t MN = (int64_t)P.M * P.N;
  const ClipRule cr{P.eta > 0.0f ? 0.0f : (float)(-1.0 * P.eta * P.minpix), P.threshold,
                    flag_opt};
  for (size_t t = 0; t < P.terms.size(); t++) {
    const Term& tm = P.terms[t];
    if (tm.kind == GV_FI_CHI2 || (zero & (1u << t))) continue;
    const int k = ps.n++;
    ps.pp[k] = prior_params(P, tm);
    ps.img[k] = XtImage{xs, P.d_mask, MN, cr, tm.image_index, 0.0f};
    ps.part[k] = prior_part(P, (int)t);
    ps.out[k] = P.d_scal + kSlotTerm0 + t;
  }
  if (fused_ok(P))
    return fused_launch(P, d_xt, flag_opt, false, &xs, P.d_scal + kSlotTerm0 + ichi2, zero, ps);
  if (ps.n > 0) {
    GV_CUDA(cudaEventRecord(fork, P.stream));
    GV_CUDA(cudaStreamWaitEvent(side, fork, 0));
    gv_status s = prior_values_launch(P, side, ps);
    if (s != GV_OK) return s;
    GV_CUDA(cudaEventRecord(join, side));
  }
  // k_degrid_ls holds more registers than k_degrid (fewer resident blocks):
  // it is taken only when its whole grid is resident at once, where the
  // node it saves is worth more (256^2, one channel: 25.1 against 25.7 us
  // per evaluation) than the latency hiding it gives up (2048^2, eight
  // channels: 944 against 938 us)
  const int C = (int)P.chans.size();
  const int nb = degrid_blocks(P);
  int resident = 0;
  GV_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_degrid_ls,
                                                        P.degrid_threads, 0));
  if (ls == nullptr || (int64_t)nb * C > (int64_t)resident * P.num_sms) {
    gv_status s = chi2_launch(P, d_xt, flag_opt, false, &xs, P.d_scal + kSlotTerm0 + ichi2, zero);
    if (s != GV_OK) return s;
    if (ps.n > 0) GV_CUDA(cudaStreamWaitEvent(P.stream, join, 0));
    return GV_OK;
  }
  gv_status s = model_grids_launch(P, d_xt, flag_opt, 1, &xs);
  if (s != GV_OK) return s;
  // the degridding waits for the prior values too: its last block adds the
  // terms up and steps the search
  if (ps.n > 0) GV_CUDA(cudaStreamWaitEvent(P.stream, join, 0));
  DegridArgs da = degrid_args(P, false, P.d_scal + kSlotTerm0 + ichi2, zero);
  da.ls = ls;
  da.ls_scal = P.d_scal;
  da.ls_cond = cond;
  k_degrid_ls<<<dim3(nb, C), P.degrid_threads, 0, P.stream>>>(da);
  GV_LAUNCH("k_degrid_ls");
  *stepped = true;
  return GV_OK;
}

gv_status check_device_error(Problem& P) {
  uint32_t e = 0;
  GV_CUDA(cudaMemcpyAsync(&e, P.d_flags + kFlagErr, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                          P.stream));
  GV_CUDA(cudaStreamSynchronize(P.stream));
  if (e != 0) {
    GV_CUDA(cudaMemsetAsync(P.d_flags + kFlagErr, 0, sizeof(uint32_t), P.stream));
    // a grid barrier that timed out leaves its arrival count behind
    GV_CUDA(cudaMemsetAsync(P.d_flags + kFlagBarCount, 0, sizeof(uint32_t), P.stream));
    set_error("a kernel gave up on a bounded wait (device error word " + std::to_string(e) + ")");
    return GV_ERR_DEVICE;
  }
  return GV_OK;
}

gv_status fetch_scalars(Problem& P, int n) {
  GV_CUDA(cudaMemcpyAsync(P.h_scal, P.d_scal, sizeof(double) * n, cudaMemcpyDeviceToHost,
                          P.stream));
  GV_CUDA(cudaStreamSynchronize(P.stream));
  return GV_OK;
}

gv_status dchi2_launch(Problem& P, const float* d_img, int flag_opt, float* d_result) {
  if (P.engine == 2) return dchi2_tc(P, d_img, flag_opt, d_result, -1, 0);
  return dchi2_direct(P, d_img, flag_opt, d_result, -1, 0);
}

gv_status dchi2_channel_launch(Problem& P, int c, float* d_out) {
  GV_CUDA(cudaMemsetAsync(d_out, 0, sizeof(float) * P.M * P.N, P.stream));
  if (P.engine == 2) return dchi2_tc(P, nullptr, 0, d_out, c, 1);
  return dchi2_direct(P, nullptr, 0, d_out, c, 1);
}

// dirty image (w Vo) or PSF (w), mode 2 / 3 of the DChi2 engines
gv_status dirty_launch(Problem& P, float* d_out, bool psf) {
  GV_CUDA(cudaMemsetAsync(d_out, 0, sizeof(float) * P.M * P.N, P.stream));
  const int mode = psf ? 3 : 2;
  if (P.engine == 2) return dchi2_tc(P, nullptr, 0, d_out, -1, mode);
  return dchi2_direct(P, nullptr, 0, d_out, -1, mode);
}

// ObjectiveFunction::calcGradient (include/classes/objectivefunction.cuh:28-57)
gv_status gradient_launch(Problem& P, float* d_img, float* d_xi, int iter, int flag_opt) {
  const int64_t MN = (int64_t)P.M * P.N;
  P.iteration = iter;  // setIteration(iter) on every Fi
  GV_CUDA(cudaMemsetAsync(d_xi, 0, sizeof(float) * 2 * MN, P.stream));
  for (size_t t = 0; t < P.terms.size(); t++) {
    const Term& tm = P.terms[t];
    gv_status s = GV_OK;
    if (tm.kind == GV_FI_CHI2) {
      s = dchi2_launch(P, d_img, flag_opt, d_xi);
    } else if (iter > 0 && tm.lambda != 0.0f && (flag_opt % 2) == tm.image_index) {
      s = prior_grad_launch(P, (int)t, d_img, d_xi);
    }
    if (s != GV_OK) return s;
  }
  return GV_OK;
}

}  // namespace gv
