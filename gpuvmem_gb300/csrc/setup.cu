// Problem set-up: the per-problem constants the reference prepares in
// MFS::setDevice (src/mfs.cu:530-943), laid out for GB300.
//
//  * calculateNoiseAndBeam (src/functions.cu:1655-1814) on the GPU: FP64
//    moments in parallel, and the reference's uncompensated FP32 weight sum
//    as a sequential chain per channel (bit for bit).
//  * hermitianSymmetry (src/functions.cu:2256-2273) and the vis_mod cell
//    choice (src/functions.cu:2557-2609) are evaluated once per visibility
//    (u,v,w are constant), so weights of visibilities outside the grid are
//    zeroed here instead of on the first objective evaluation; visibilities
//    are then sorted by grid cell so the degridding gathers hit L2 in order.
//  * total_attenuation / weight_image / noise_image, fg_scale = min(noise),
//    noise_cut = factor * min(noise) (src/mfs.cu:849-916).

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "gv_internal.cuh"

namespace gv {

namespace {

// calculateNoiseAndBeam (src/functions.cu:1700-1814) on the GPU, in two
// kernels.
//
// k_beam_moments: calc_sBeam's weighted second moments of one channel
// (:1655-1683), sum_k u^2 w, v^2 w, u v w with u, v in wavelengths of the
// float wavelength, as FP64 block partials; the last block adds the
// channel's totals to acc[0..2], so channels are added in order.  (The
// reference adds under an OpenMP reduction, in no fixed order; FP64 keeps
// the difference at the level of FP64 rounding.)
__global__ void __launch_bounds__(256) k_beam_moments(int64_t n, float lam,
                                                      const double* __restrict__ uvw,
                                                      const float* __restrict__ w,
                                                      double* __restrict__ part,
                                                      uint32_t* __restrict__ done,
                                                      double* __restrict__ acc) {
  double suu = 0.0, svv = 0.0, suv = 0.0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const double u = uvw[3 * k] / lam, v = uvw[3 * k + 1] / lam, wk = w[k];
    suu += u * u * wk;
    svv += v * v * wk;
    suv += u * v * wk;
  }
  __shared__ double red[3][8];
  for (int o = 16; o > 0; o >>= 1) {
    suu += __shfl_down_sync(0xffffffffu, suu, o);
    svv += __shfl_down_sync(0xffffffffu, svv, o);
    suv += __shfl_down_sync(0xffffffffu, suv, o);
  }
  const int wid = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][wid] = suu;
    red[1][wid] = svv;
    red[2][wid] = suv;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[threadIdx.x][i];
    part[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = t;
  }
  if (last_block_done(done, gridDim.x) && threadIdx.x < 3) {
    double t = 0.0;
    for (unsigned b = 0; b < gridDim.x; b++) t += __ldcg(part + (int64_t)threadIdx.x * gridDim.x + b);
    acc[threadIdx.x] += t;
  }
}

// k_weight_chain: reduceCPU (:353-367) of each channel's weights, one block
// per channel.  reduceCPU returns its running FP32 sum without the
// compensation it computes, i.e. the plain sequential FP32 sum; a
// sequential chain reproduces it bit for bit (a parallel tree would round
// differently).  Thread 0 adds a tile of 2048 weights in order from shared
// memory while the other threads load the next tile, so the chain of
// dependent additions, not memory latency, sets the time.
constexpr int kChainTile = 2048;

__global__ void __launch_bounds__(256) k_weight_chain(const int64_t* __restrict__ off,
                                                      const float* __restrict__ w,
                                                      float* __restrict__ out) {
  __shared__ float tile[2][kChainTile];
  const int c = blockIdx.x;
  const int64_t o = off[c], n = off[c + 1] - off[c];
  const int64_t ntiles = (n + kChainTile - 1) / kChainTile;
  for (int k = threadIdx.x; k < kChainTile && k < n; k += blockDim.x) tile[0][k] = w[o + k];
  __syncthreads();
  float s = 0.0f;
  for (int64_t t = 0; t < ntiles; t++) {
    const int64_t base = t * kChainTile;
    const int cnt = (int)(n - base < kChainTile ? n - base : kChainTile);
    const float* cur = tile[t & 1];
    if (threadIdx.x == 0) {
      int k = 0;
      if (t == 0) {
        s = cur[0];
        k = 1;
      }
      for (; k < cnt; k++) s = __fadd_rn(s, cur[k]);
    } else {
      const int64_t nb = base + kChainTile;
      float* nxt = tile[(t + 1) & 1];
      for (int64_t k = threadIdx.x - 1; k < kChainTile && nb + k < n; k += blockDim.x - 1)
        nxt[k] = w[o + nb + k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = n > 0 ? s : 0.0f;
}

__global__ void k_prepare_vis(int64_t n, int64_t off, int chan, float freq,
                              const double* __restrict__ uvw_m,
                              const float2* __restrict__ vo_in,
                              const float* __restrict__ w_in, double deltau,
                              double deltav, int N, double dx, double dy,
                              float4* __restrict__ deg_u,
                              float2* __restrict__ vo_u, uint4* __restrict__ ph_u,
                              float* __restrict__ wl_u, float4* __restrict__ E_u,
                              unsigned long long* __restrict__ keys,
                              int64_t* __restrict__ idx) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int64_t g = off + k;
  double u = uvw_m[3 * k], v = uvw_m[3 * k + 1], w = uvw_m[3 * k + 2];
  float2 o = vo_in[k];
  // hermitianSymmetry
  if (u > 0.0) {
    u *= -1.0;
    v *= -1.0;
    o.y *= -1.0f;
  }
  const float lambda = wavelength(freq);
  u = u / lambda;
  v = v / lambda;
  w = w / lambda;
  // vis_mod cell choice
  double ux = u / deltau, uy = v / deltav;
  if (ux < 0.0) ux += N;
  if (uy < 0.0) uy += N;
  const int i1 = __double2int_rd(ux);
  const int j1 = __double2int_rd(uy);
  const bool in = (i1 >= 0 && i1 < N && j1 >= 0 && j1 < N);
  const float wt = in ? w_in[k] : 0.0f;
  const bool keep = in && wt != 0.0f;
  const float du = in ? (float)(ux - i1) : 0.0f;
  const float dv = in ? (float)(uy - j1) : 0.0f;
  const uint32_t cell = keep ? (uint32_t)j1 * (uint32_t)N + (uint32_t)i1 : 0xFFFFFFFFu;
  const uint32_t packed = keep ? ((uint32_t)j1 << 16) | (uint32_t)i1 : 0u;
  deg_u[g] = make_float4(__uint_as_float(packed), du, dv, wt);
  vo_u[g] = o;
  // phase constants: exact fixed-point fractions of dx*u and dy*v
  double tx = dx * u;
  tx -= floor(tx);
  double ty = dy * v;
  ty -= floor(ty);
  const uint32_t FU = (uint32_t)(unsigned long long)llrint(tx * 4294967296.0);
  const uint32_t FV = (uint32_t)(unsigned long long)llrint(ty * 4294967296.0);
  const float GU = (float)(w * dx * dx * 0.5);
  const float GV = (float)(w * dy * dy * 0.5);
  ph_u[g] = make_uint4(FU, FV, __float_as_uint(GU), __float_as_uint(GV));
  // unit phasors of the fixed-point fractions (exact angle, FP64 sincos)
  double su, cu, sv, cv;
  sincospi(2.0 * (double)(int32_t)FU * 2.3283064365386963e-10, &su, &cu);
  sincospi(2.0 * (double)(int32_t)FV * 2.3283064365386963e-10, &sv, &cv);
  E_u[g] = make_float4((float)cu, (float)su, (float)cv, (float)sv);
  wl_u[g] = (float)w;
  keys[g] = ((unsigned long long)chan << 32) | cell;
  idx[g] = g;
}

template <typename T>
__global__ void k_gather(int64_t n, const int64_t* __restrict__ idx,
                         const T* __restrict__ in, T* __restrict__ out) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n) out[k] = in[idx[k]];
}

// max |w Vo| component (dirty image scale) and max w (PSF scale)
__global__ void k_dirty_max(int64_t V, const float4* __restrict__ deg,
                            const float2* __restrict__ vo, uint32_t* __restrict__ out,
                            uint32_t* __restrict__ out_w) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float m = 0.0f, mw = 0.0f;
  if (k < V) {
    const float4 d = deg[k];
    const float2 o = vo[k];
    m = fmaxf(fabsf(d.w * o.x), fabsf(d.w * o.y));
    mw = fabsf(d.w);
  }
  for (int s = 16; s > 0; s >>= 1) {
    m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, s));
    mw = fmaxf(mw, __shfl_down_sync(0xffffffffu, mw, s));
  }
  if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(out, __float_as_uint(m));
  if ((threadIdx.x & 31) == 0 && mw > 0.0f) atomicMax(out_w, __float_as_uint(mw));
}

__global__ void k_weight_image(int M, int N, float xobs, float yobs, double DELTAX,
                               double DELTAY, float nu0, float D, float pbf,
                               float cut, int pb, float* __restrict__ wimg) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= N || j >= M) return;
  const float a = attenuation(i, j, xobs, yobs, DELTAX, DELTAY, nu0, D, pbf, cut, pb);
  wimg[(int64_t)N * i + j] = a * a;  // weight_image: sum over fields of atten^2
}

__global__ void k_noise_image(int64_t MN, float max_w, float noise_jypix,
                              float* __restrict__ img) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= MN) return;
  const float nsq = noise_jypix * noise_jypix;
  const float nw = (img[q] / max_w) / nsq;
  img[q] = sqrtf(1.0f / nw);
}

__global__ void k_mask(int64_t MN, float cut, const float* __restrict__ noise,
                       uint8_t* __restrict__ mask) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= MN) return;
  const float n = noise[q];
  mask[q] = (n < cut ? kMaskIn : 0) | (n > cut ? kMaskClip : 0);
}

// rho = (z - 1) + r^2/2 with z = sqrt(1 - r^2), written without
// cancellation as -r^4 / (2 (1 + z)^2).
__global__ void k_rho(int M, int N, float xobs, float yobs, double dx, double dy,
                      float* __restrict__ rho) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= N || j >= M) return;
  const int x0 = (int)xobs, y0 = (int)yobs;
  const double x = (j - x0) * dx, y = (i - y0) * dy;
  const double r2 = x * x + y * y;
  const double z = sqrt(1.0 - r2);
  rho[(int64_t)N * i + j] = (float)(-(r2 * r2) / (2.0 * (1.0 + z) * (1.0 + z)));
}

}  // namespace

void free_problem(Problem& P) {
  cudaFree(P.d_deg);
  cudaFree(P.d_vo);
  cudaFree(P.d_cvr);
  cudaFree(P.d_ph);
  cudaFree(P.d_wl);
  cudaFree(P.d_perm);
  cudaFree(P.d_noise);
  cudaFree(P.d_gcf);
  for (auto& t : P.terms) cudaFree(t.d_prior);
  cudaFree(P.d_mask);
  cudaFree(P.d_rho);
  cudaFree(P.d_grid);
  cudaFree(P.d_twiddle);
  cudaFree(P.d_beam_x);  // one allocation with d_beam_y, d_rot_u, d_rot_v
  cudaFree(P.d_epi);
  cudaFree(P.d_part);
  cudaFree(P.d_scal);
  cudaFree(P.d_tmp);
  cudaFree(P.d_opt);
  cudaFree(P.d_lbfgs);
  cudaFree(P.d_chfreq);
  cudaFree(P.d_ranges);
  cudaFree(P.d_chnvis);
  cudaFree(P.d_kc_off);
  cudaFree(P.d_kc_one);
  cudaFree(P.d_E);
  cudaFree(P.d_flags);
  cudaFree(P.tc_partial);
  if (P.h_scal) cudaFreeHost(P.h_scal);
  if (P.h_many) cudaFreeHost(P.h_many);
  graph_cache_free(P);
  ls_cache_free(P);
  cudaFree(P.d_ls);
  cudaFree(P.d_lbscal);
  P = Problem();
}

gv_status setup_problem(Problem& P, const gv_problem_desc& d) {
  // ---- validation (the reference exits on bad input; we return) ----------
  if (d.M <= 0 || d.N <= 0 || d.M != d.N) {
    set_error("M and N must be equal and positive (the reference indexes both axes with N)");
    return GV_ERR_INVALID;
  }
  const int n = d.N;
  if ((n & (n - 1)) != 0 || n < 16 || n > 4096) {
    set_error("image size must be a power of two between 16 and 4096");
    return GV_ERR_UNSUPPORTED;
  }
  if (d.nchannels <= 0 || d.channels == nullptr) {
    set_error("at least one channel is required");
    return GV_ERR_INVALID;
  }
  if (d.nterms < 0 || d.nterms > kMaxTerms || (d.nterms > 0 && d.terms == nullptr)) {
    set_error("between 0 and 8 objective terms are supported");
    return GV_ERR_INVALID;
  }
  if (!(d.deltax_deg != 0.0) || !(d.deltay_deg != 0.0) || !(d.nu_0 > 0.0f)) {
    set_error("cell sizes must be non-zero and nu_0 positive");
    return GV_ERR_INVALID;
  }
  if (!(d.xobs_pix >= 0.0f && d.xobs_pix < n && d.yobs_pix >= 0.0f && d.yobs_pix < n)) {
    // src/mfs.cu:692-712 rejects centres outside the image
    set_error("pointing / phase centre is outside the range of the image");
    return GV_ERR_INVALID;
  }
  P.M = d.M;
  P.N = d.N;
  P.log2n = 0;
  while ((1 << P.log2n) < n) P.log2n++;
  P.DELTAX = d.deltax_deg;
  P.DELTAY = d.deltay_deg;
  P.dx_rad = kRpDegD * d.deltax_deg;
  P.dy_rad = kRpDegD * d.deltay_deg;
  P.deltau = 1.0 / (P.M * P.dx_rad);
  P.deltav = 1.0 / (P.N * P.dy_rad);
  P.xobs = d.xobs_pix;
  P.yobs = d.yobs_pix;
  P.nu_0 = d.nu_0;
  P.D = d.antenna_diameter;
  P.pbf = d.pb_factor;
  P.pbcut = d.pb_cutoff;
  P.pb = d.primary_beam;
  P.eta = d.eta;
  P.minpix = d.initial_value * -1.0f * d.eta;  // src/mfs.cu:167-173
  P.threshold = d.threshold;
  P.normalize = d.normalize;
  // terms: ObjectiveFunction::addFi drops terms whose factor is 0
  for (int t = 0; t < d.nterms; t++) {
    const gv_fi_desc& f = d.terms[t];
    if (f.kind < GV_FI_CHI2 || f.kind > GV_FI_QUADRATIC) {
      set_error("unknown objective term kind");
      return GV_ERR_INVALID;
    }
    if (f.image_index < 0 || f.image_index > 1 || f.image_to_add < 0 || f.image_to_add > 1) {
      set_error("There is no image for the provided index");  // include/classes/fi.cuh:68
      return GV_ERR_INVALID;
    }
    if (f.lambda == 0.0f) continue;
    if (f.kind == GV_FI_CHI2 && !P.terms.empty()) {
      set_error("Chi2 must be the first objective term (Chi2::addToDphi overwrites dphi)");
      return GV_ERR_INVALID;
    }
    Term tm{f.kind, f.lambda, f.image_index, f.image_to_add, f.prior_value, f.eta, f.epsilon};
    tm.epsilon_b = f.epsilon_b;
    if (f.kind == GV_FI_GENTROPY || f.kind == GV_FI_GL1) {
      if (!f.prior_image) {
        set_error("GEntropy and GL1Norm need a prior image");
        return GV_ERR_INVALID;
      }
      // normalizePrior (src/gentropy.cu:123, src/gl1norm.cu:155): prior / factor
      const int64_t MN = (int64_t)d.M * d.N;
      std::vector<float> pr(f.prior_image, f.prior_image + MN);
      const float nf = f.normalization_factor != 0.0f ? f.normalization_factor : 1.0f;
      for (auto& v : pr) v /= nf;
      GV_CUDA(cudaMalloc(&tm.d_prior, sizeof(float) * MN));
      P.terms.push_back(tm);  // owned by P from here (freed by free_problem)
      GV_CUDA(cudaMemcpy(tm.d_prior, pr.data(), sizeof(float) * MN, cudaMemcpyHostToDevice));
      continue;
    }
    P.terms.push_back(tm);
  }
  int dev = 0;
  GV_CUDA(cudaGetDevice(&dev));
  GV_CUDA(cudaDeviceGetAttribute(&P.num_sms, cudaDevAttrMultiProcessorCount, dev));

  // ---- channels ----------------------------------------------------------
  const int C = d.nchannels;
  int64_t V = 0;
  for (int c = 0; c < C; c++) {
    const gv_channel_desc& ch = d.channels[c];
    if (ch.nvis < 0 || (ch.nvis > 0 && (!ch.uvw || !ch.vo || !ch.weight)) || !(ch.freq_hz > 0.0f)) {
      set_error("invalid channel descriptor");
      return GV_ERR_INVALID;
    }
    P.chans.push_back(Channel{ch.freq_hz, ch.nvis, V, 0});
    V += ch.nvis;
  }
  P.V = V;
  if (V <= 0) {
    set_error("Max number of visibilities cannot be zero for image synthesis");  // src/mfs.cu:624
    return GV_ERR_INVALID;
  }

  const int64_t MN = (int64_t)P.M * P.N;
  cudaStream_t st = P.stream;

  // ---- visibilities: upload, prepare, sort by (channel, cell) -------------
  {
    double* d_uvw = nullptr;
    float2* d_vo_in = nullptr;
    float* d_w_in = nullptr;      // [V] weights of all channels, as given
    double* d_mom = nullptr;      // beam moments: [3] totals, then 3 * nbm partials
    uint32_t* d_mdone = nullptr;
    float* d_wsum = nullptr;      // [C] reduceCPU of each channel's weights
    int64_t* d_off = nullptr;     // [C + 1]
    float4* deg_u = nullptr;
    float2* vo_u = nullptr;
    uint4* ph_u = nullptr;
    float* wl_u = nullptr;
    float4* E_u = nullptr;
    unsigned long long *keys = nullptr, *keys2 = nullptr;
    int64_t *idx = nullptr;
    void* tmp = nullptr;
    size_t tmp_bytes = 0;
    int64_t maxc = 0;
    for (auto& ch : P.chans) maxc = std::max(maxc, ch.nvis);
    auto cleanup = [&]() {
      cudaFree(d_uvw); cudaFree(d_vo_in); cudaFree(d_w_in); cudaFree(deg_u);
      cudaFree(d_mom); cudaFree(d_mdone); cudaFree(d_wsum); cudaFree(d_off);
      cudaFree(vo_u); cudaFree(ph_u); cudaFree(wl_u); cudaFree(E_u); cudaFree(keys); cudaFree(keys2);
      cudaFree(idx); cudaFree(tmp);
    };
#define GV_SETUP_CUDA(call)                         \
  do {                                              \
    cudaError_t _e = (call);                        \
    if (_e != cudaSuccess) {                        \
      cleanup();                                    \
      return cuda_fail(_e, #call);                  \
    }                                               \
  } while (0)
    GV_SETUP_CUDA(cudaMalloc(&d_uvw, sizeof(double) * 3 * std::max<int64_t>(maxc, 1)));
    GV_SETUP_CUDA(cudaMalloc(&d_vo_in, sizeof(float2) * std::max<int64_t>(maxc, 1)));
    GV_SETUP_CUDA(cudaMalloc(&d_w_in, sizeof(float) * V));
    const int nbm = 4 * P.num_sms;
    GV_SETUP_CUDA(cudaMalloc(&d_mom, sizeof(double) * (3 + 3 * (size_t)nbm)));
    GV_SETUP_CUDA(cudaMemsetAsync(d_mom, 0, sizeof(double) * 3, st));
    GV_SETUP_CUDA(cudaMalloc(&d_mdone, sizeof(uint32_t)));
    GV_SETUP_CUDA(cudaMemsetAsync(d_mdone, 0, sizeof(uint32_t), st));
    GV_SETUP_CUDA(cudaMalloc(&d_wsum, sizeof(float) * C));
    GV_SETUP_CUDA(cudaMalloc(&d_off, sizeof(int64_t) * (C + 1)));
    {
      std::vector<int64_t> off(C + 1, 0);
      for (int c = 0; c < C; c++) off[c + 1] = off[c] + P.chans[c].nvis;
      GV_SETUP_CUDA(cudaMemcpy(d_off, off.data(), sizeof(int64_t) * (C + 1),
                               cudaMemcpyHostToDevice));
    }
    GV_SETUP_CUDA(cudaMalloc(&deg_u, sizeof(float4) * V));
    GV_SETUP_CUDA(cudaMalloc(&vo_u, sizeof(float2) * V));
    GV_SETUP_CUDA(cudaMalloc(&ph_u, sizeof(uint4) * V));
    GV_SETUP_CUDA(cudaMalloc(&wl_u, sizeof(float) * V));
    GV_SETUP_CUDA(cudaMalloc(&E_u, sizeof(float4) * V));
    GV_SETUP_CUDA(cudaMalloc(&keys, sizeof(unsigned long long) * V));
    GV_SETUP_CUDA(cudaMalloc(&keys2, sizeof(unsigned long long) * V));
    GV_SETUP_CUDA(cudaMalloc(&idx, sizeof(int64_t) * V));
    GV_SETUP_CUDA(cudaMalloc(&P.d_perm, sizeof(int64_t) * V));
    for (int c = 0; c < C; c++) {
      const gv_channel_desc& ch = d.channels[c];
      if (ch.nvis <= 0) continue;
      GV_SETUP_CUDA(cudaMemcpyAsync(d_uvw, ch.uvw, sizeof(double) * 3 * ch.nvis,
                                    cudaMemcpyHostToDevice, st));
      GV_SETUP_CUDA(cudaMemcpyAsync(d_vo_in, ch.vo, sizeof(float2) * ch.nvis,
                                    cudaMemcpyHostToDevice, st));
      float* w_c = d_w_in + P.chans[c].off;
      GV_SETUP_CUDA(cudaMemcpyAsync(w_c, ch.weight, sizeof(float) * ch.nvis,
                                    cudaMemcpyHostToDevice, st));
      const int bs = 256;
      // calc_sBeam of this channel (the uvw buffer is reused per channel)
      const unsigned mb = (unsigned)std::min<int64_t>((ch.nvis + bs - 1) / bs, nbm);
      k_beam_moments<<<mb, bs, 0, st>>>(ch.nvis, wavelength(ch.freq_hz), d_uvw, w_c, d_mom + 3,
                                        d_mdone, d_mom);
      GV_SETUP_CUDA(cudaGetLastError());
      k_prepare_vis<<<(unsigned)((ch.nvis + bs - 1) / bs), bs, 0, st>>>(
          ch.nvis, P.chans[c].off, c, ch.freq_hz, d_uvw, d_vo_in, w_c, P.deltau,
          P.deltav, P.N, P.dx_rad, P.dy_rad, deg_u, vo_u, ph_u, wl_u, E_u, keys, idx);
      GV_SETUP_CUDA(cudaGetLastError());
    }
    // calculateNoiseAndBeam's weight sum: reduceCPU per channel, added over
    // the channels in FP32 in order (src/functions.cu:1731-1733)
    k_weight_chain<<<C, 256, 0, st>>>(d_off, d_w_in, d_wsum);
    GV_SETUP_CUDA(cudaGetLastError());
    {
      std::vector<float> wsum(C);
      double mom[3];
      GV_SETUP_CUDA(cudaMemcpyAsync(wsum.data(), d_wsum, sizeof(float) * C,
                                    cudaMemcpyDeviceToHost, st));
      GV_SETUP_CUDA(cudaMemcpyAsync(mom, d_mom, sizeof(double) * 3, cudaMemcpyDeviceToHost, st));
      GV_SETUP_CUDA(cudaStreamSynchronize(st));
      float sum_w = 0.0f;
      for (int c = 0; c < C; c++)
        if (P.chans[c].nvis > 0) sum_w += wsum[c];
      if (!(sum_w > 0.0f)) {
        cleanup();
        set_error("The sum of the visibility weights cannot be zero");  // functions.cu:1790
        return GV_ERR_INVALID;
      }
      // calc_beamSize (:1685-1698) and the noise (:1796-1811)
      const double s_uu = mom[0] / sum_w, s_vv = mom[1] / sum_w, s_uv = mom[2] / sum_w;
      const float variance = 1.0f / sum_w;
      const double uu_mv = s_uu - s_vv, uu_pv = s_uu + s_vv;
      const double sq = std::sqrt(uu_mv * uu_mv + 4.0 * s_uv * s_uv);
      P.bmaj = (1.0 / std::sqrt(2.0) / kPiD / std::sqrt(uu_pv - sq)) / kRpDegD;
      P.bmin = (1.0 / std::sqrt(2.0) / kPiD / std::sqrt(uu_pv + sq)) / kRpDegD;
      P.bpa = (-0.5 * std::atan2(2.0 * s_uv, uu_mv)) / kRpDegD;
      P.sum_weights = sum_w;
      P.vis_noise = d.vis_noise > 0.0f ? d.vis_noise : 0.5f * sqrtf(variance);
    }
    tmp_bytes = radix_sort_scratch<unsigned long long, int64_t>((int64_t)V);
    GV_SETUP_CUDA(cudaMalloc(&tmp, tmp_bytes));
    {
      const gv_status s = radix_sort_pairs<unsigned long long, int64_t>(
          tmp, tmp_bytes, keys, keys2, idx, P.d_perm, (int64_t)V, 0, 64, st);
      if (s != GV_OK) {
        cleanup();
        return s;
      }
    }
    GV_SETUP_CUDA(cudaMalloc(&P.d_deg, sizeof(float4) * V));
    GV_SETUP_CUDA(cudaMalloc(&P.d_vo, sizeof(float2) * V));
    GV_SETUP_CUDA(cudaMalloc(&P.d_ph, sizeof(uint4) * V));
    GV_SETUP_CUDA(cudaMalloc(&P.d_wl, sizeof(float) * V));
    GV_SETUP_CUDA(cudaMalloc(&P.d_E, sizeof(float4) * V));
    GV_SETUP_CUDA(cudaMalloc(&P.d_cvr, sizeof(float2) * V));
    GV_SETUP_CUDA(cudaMemsetAsync(P.d_cvr, 0, sizeof(float2) * V, st));
    const unsigned gb = (unsigned)((V + 255) / 256);
    k_gather<float4><<<gb, 256, 0, st>>>(V, P.d_perm, deg_u, P.d_deg);
    k_gather<float2><<<gb, 256, 0, st>>>(V, P.d_perm, vo_u, P.d_vo);
    k_gather<uint4><<<gb, 256, 0, st>>>(V, P.d_perm, ph_u, P.d_ph);
    k_gather<float><<<gb, 256, 0, st>>>(V, P.d_perm, wl_u, P.d_wl);
    k_gather<float4><<<gb, 256, 0, st>>>(V, P.d_perm, E_u, P.d_E);
    GV_SETUP_CUDA(cudaGetLastError());
    // count kept visibilities per channel: keys are sorted, so the kept ones
    // of channel c are those with key < (c << 32 | 0xFFFFFFFF)
    std::vector<unsigned long long> hkeys(V);
    GV_SETUP_CUDA(cudaMemcpyAsync(hkeys.data(), keys2, sizeof(unsigned long long) * V,
                                  cudaMemcpyDeviceToHost, st));
    GV_SETUP_CUDA(cudaStreamSynchronize(st));
    P.Vgrid = 0;
    for (int c = 0; c < C; c++) {
      const unsigned long long lim = ((unsigned long long)c << 32) | 0xFFFFFFFFull;
      auto b = hkeys.begin() + P.chans[c].off;
      auto e = b + P.chans[c].nvis;
      P.chans[c].ngrid = std::lower_bound(b, e, lim) - b;
      P.Vgrid += P.chans[c].ngrid;
    }
    // bound of the non-separable w-term residual |w * rho| (cycles)
    std::vector<float> hw(V);
    GV_SETUP_CUDA(cudaMemcpy(hw.data(), wl_u, sizeof(float) * V, cudaMemcpyDeviceToHost));
    double maxw = 0.0;
    for (float x : hw) maxw = std::max(maxw, (double)std::fabs(x));
    double rmax = 0.0;
    {
      const double hx = std::max(std::fabs((double)(0 - (int)P.xobs)),
                                 std::fabs((double)(P.M - 1 - (int)P.xobs))) *
                        std::fabs(P.dx_rad);
      const double hy = std::max(std::fabs((double)(0 - (int)P.yobs)),
                                 std::fabs((double)(P.N - 1 - (int)P.yobs))) *
                        std::fabs(P.dy_rad);
      const double r2 = hx * hx + hy * hy;
      const double z = std::sqrt(1.0 - r2);
      rmax = r2 * r2 / (2.0 * (1.0 + z) * (1.0 + z));
    }
    P.max_wrho = maxw * rmax;
    cleanup();
#undef GV_SETUP_CUDA
  }

  // ---- gridding correction function (Chi2::setCKernel with gridding) -------
  if (d.gcf) {
    GV_CUDA(cudaMalloc(&P.d_gcf, sizeof(float) * MN));
    GV_CUDA(cudaMemcpyAsync(P.d_gcf, d.gcf, sizeof(float) * MN, cudaMemcpyHostToDevice, st));
  }

  // ---- noise image, mask, fg_scale, noise_cut ------------------------------
  GV_CUDA(cudaMalloc(&P.d_noise, sizeof(float) * MN));
  GV_CUDA(cudaMalloc(&P.d_mask, MN));
  GV_CUDA(cudaMalloc(&P.d_rho, sizeof(float) * MN));
  {
    dim3 b2(16, 16), g2((P.M + 15) / 16, (P.N + 15) / 16);
    k_weight_image<<<g2, b2, 0, st>>>(P.M, P.N, P.xobs, P.yobs, P.DELTAX, P.DELTAY, P.nu_0,
                                      P.D, P.pbf, P.pbcut, P.pb, P.d_noise);
    GV_LAUNCH("k_weight_image");
    std::vector<float> h(MN);
    GV_CUDA(cudaMemcpyAsync(h.data(), P.d_noise, sizeof(float) * MN, cudaMemcpyDeviceToHost, st));
    GV_CUDA(cudaStreamSynchronize(st));
    const float max_w = *std::max_element(h.begin(), h.end());
    const double bmaj_pix = P.bmaj / std::fabs(P.DELTAX);
    const double bmin_pix = P.bmin / std::fabs(P.DELTAX);
    const float noise_jypix =
        (float)(P.vis_noise / (kPiD * bmaj_pix * bmin_pix / (4.0 * logf(2.0f))));
    k_noise_image<<<(unsigned)((MN + 255) / 256), 256, 0, st>>>(MN, max_w, noise_jypix, P.d_noise);
    GV_LAUNCH("k_noise_image");
    GV_CUDA(cudaMemcpyAsync(h.data(), P.d_noise, sizeof(float) * MN, cudaMemcpyDeviceToHost, st));
    GV_CUDA(cudaStreamSynchronize(st));
    const float nmin = *std::min_element(h.begin(), h.end());
    P.fg_scale = nmin;
    P.noise_cut = d.noise_cut_factor * nmin;
    int64_t cnt = 0;
    for (float x : h) cnt += (x < P.noise_cut);
    P.mask_pixels = cnt;
    k_mask<<<(unsigned)((MN + 255) / 256), 256, 0, st>>>(MN, P.noise_cut, P.d_noise, P.d_mask);
    GV_LAUNCH("k_mask");
    k_rho<<<g2, b2, 0, st>>>(P.M, P.N, P.xobs, P.yobs, P.dx_rad, P.dy_rad, P.d_rho);
    GV_LAUNCH("k_rho");
  }

  // ---- FFT twiddles, grids, reduction scratch -----------------------------
  {
    // e^{+2 pi i m / n}, m < n (the FFT passes' twiddles, FP64 rounded once)
    std::vector<float2> tw(n);
    for (int m = 0; m < n; m++) {
      const double a = 2.0 * kPiD * m / n;
      tw[m] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    GV_CUDA(cudaMalloc(&P.d_twiddle, sizeof(float2) * n));
    GV_CUDA(cudaMemcpyAsync(P.d_twiddle, tw.data(), sizeof(float2) * n,
                            cudaMemcpyHostToDevice, st));
  }
  {
    // per-column / per-row FP64 products of attenuation() and phase_rotate
    // (src/functions.cu:2304-2310, :2490-2500), rounded to float once here
    // (IEEE products: the same floats the kernels would form)
    std::vector<float> bx(P.N), by(P.M), ru(P.N), rv(P.M);
    const double upix = (double)P.xobs / (double)P.N, vpix = (double)P.yobs / (double)P.M;
    for (int j = 0; j < P.N; j++) {
      bx[j] = beam_coord(j, (int)P.xobs, P.DELTAX);
      ru[j] = (float)(j < P.N / 2 ? upix * j : upix * (j - P.N));
    }
    for (int i = 0; i < P.M; i++) {
      by[i] = beam_coord(i, (int)P.yobs, P.DELTAY);
      rv[i] = (float)(i < P.M / 2 ? vpix * i : vpix * (i - P.M));
    }
    GV_CUDA(cudaMalloc(&P.d_beam_x, sizeof(float) * 2 * (P.N + P.M)));
    P.d_beam_y = P.d_beam_x + P.N;
    P.d_rot_u = P.d_beam_y + P.M;
    P.d_rot_v = P.d_rot_u + P.N;
    GV_CUDA(cudaMemcpy(P.d_beam_x, bx.data(), sizeof(float) * P.N, cudaMemcpyHostToDevice));
    GV_CUDA(cudaMemcpy(P.d_beam_y, by.data(), sizeof(float) * P.M, cudaMemcpyHostToDevice));
    GV_CUDA(cudaMemcpy(P.d_rot_u, ru.data(), sizeof(float) * P.N, cudaMemcpyHostToDevice));
    GV_CUDA(cudaMemcpy(P.d_rot_v, rv.data(), sizeof(float) * P.M, cudaMemcpyHostToDevice));
  }
  GV_CUDA(cudaMalloc(&P.d_grid, sizeof(float2) * MN * C));
  {
    std::vector<float> f(C);
    std::vector<ChanRange> r(C);
    std::vector<int64_t> nv(C);
    for (int c = 0; c < C; c++) {
      f[c] = P.chans[c].freq;
      r[c] = ChanRange{P.chans[c].off, P.chans[c].ngrid};
      nv[c] = P.chans[c].nvis;
    }
    GV_CUDA(cudaMalloc(&P.d_chfreq, sizeof(float) * C));
    GV_CUDA(cudaMalloc(&P.d_ranges, sizeof(ChanRange) * C));
    GV_CUDA(cudaMalloc(&P.d_chnvis, sizeof(int64_t) * C));
    GV_CUDA(cudaMemcpy(P.d_chfreq, f.data(), sizeof(float) * C, cudaMemcpyHostToDevice));
    GV_CUDA(cudaMemcpy(P.d_ranges, r.data(), sizeof(ChanRange) * C, cudaMemcpyHostToDevice));
    GV_CUDA(cudaMemcpy(P.d_chnvis, nv.data(), sizeof(int64_t) * C, cudaMemcpyHostToDevice));
    std::vector<int64_t> kc(C + 1, 0), k1(2 * C, 0);
    for (int c = 0; c < C; c++) {
      kc[c + 1] = kc[c] + P.chans[c].ngrid;
      k1[2 * c + 1] = P.chans[c].ngrid;
    }
    GV_CUDA(cudaMalloc(&P.d_kc_off, sizeof(int64_t) * (C + 1)));
    GV_CUDA(cudaMalloc(&P.d_kc_one, sizeof(int64_t) * 2 * C));
    GV_CUDA(cudaMemcpy(P.d_kc_off, kc.data(), sizeof(int64_t) * (C + 1), cudaMemcpyHostToDevice));
    GV_CUDA(cudaMemcpy(P.d_kc_one, k1.data(), sizeof(int64_t) * 2 * C, cudaMemcpyHostToDevice));
  }
  GV_CUDA(cudaMalloc(&P.d_flags, sizeof(uint32_t) * kNumFlags));
  GV_CUDA(cudaMemsetAsync(P.d_flags, 0, sizeof(uint32_t) * kNumFlags, st));
  {
    const unsigned gb = (unsigned)((V + 255) / 256);
    k_dirty_max<<<gb, 256, 0, st>>>(V, P.d_deg, P.d_vo, P.d_flags + kFlagDirtyMax,
                                    P.d_flags + kFlagPsfMax);
    GV_LAUNCH("k_dirty_max");
  }
  // split-K partial images of the tensor-core engine: pick the split count
  // that fills whole waves of SMs (of CTA pairs in pair mode), keeping
  // >= 1024 visibilities per item
  if (P.N >= 128) {
    const int TN = tc_tile_n(P);
    const bool pair = tc_pair(P);
    const int64_t tiles = (int64_t)(P.N / 128) * (P.N / TN) / (pair ? 2 : 1);
    const int64_t workers = std::max(1, pair ? P.num_sms / 2 : P.num_sms);
    int64_t nmax = std::max<int64_t>(1, P.Vgrid / 1024);
    int best = 1;
    double best_util = -1.0;
    for (int64_t s = 1; s <= std::min<int64_t>(nmax, 256); s++) {
      const int64_t items = tiles * s;
      const int64_t waves = (items + workers - 1) / workers;
      const double util = (double)items / (double)(waves * workers);
      if (util > best_util + 0.02) {
        best_util = util;
        best = (int)s;
      }
    }
    P.tc_nsplit = best;
    const char* acc = std::getenv("GV_TC_ACCURATE_ANCHOR");
    P.tc_fast_anchor = (acc && acc[0] == '1') ? 0 : 1;
    GV_CUDA(cudaMalloc(&P.tc_partial, sizeof(float) * (size_t)best * MN));
    P.tc_partial_cap = (size_t)best;
    // epilogue factors of every channel (set up here, not inside a capture)
    P.epi_bytes = sizeof(float) * (size_t)C * (size_t)MN;
    GV_CUDA(cudaMalloc(&P.d_epi, P.epi_bytes));
  }
  {
    const char* g = std::getenv("GV_GRAPHS");
    P.use_graphs = (g && g[0] == '0') ? 0 : 1;
  }
  if (const char* e = std::getenv("GV_FUSED")) P.fused = std::atoi(e) != 0 ? 1 : 0;
  P.part_stride = 4 * P.num_sms;
  const int nslots = C + kMaxTerms + 8;
  GV_CUDA(cudaMalloc(&P.d_part, sizeof(double) * (size_t)P.part_stride * nslots));
  GV_CUDA(cudaMalloc(&P.d_scal, sizeof(double) * kNumScal));
  GV_CUDA(cudaMemsetAsync(P.d_scal, 0, sizeof(double) * kNumScal, st));
  GV_CUDA(cudaMallocHost(&P.h_scal, sizeof(double) * kNumScal));
  GV_CUDA(cudaMalloc(&P.d_tmp, sizeof(float) * 2 * MN));
  // DChi2 engine: the tensor-core GEMM needs the w-term to be separable
  // (|w * rho| below 1e-7 cycles) and a supported geometry.
  P.engine = d.dchi2_engine;
  if (P.engine == 0) P.engine = dchi2_tc_supported(P) ? 2 : 1;
  if (P.engine == 2 && !dchi2_tc_supported(P)) {
    set_error("tensor-core DChi2 engine not supported for this problem");
    return GV_ERR_UNSUPPORTED;
  }
  GV_CUDA(cudaStreamSynchronize(st));
  return GV_OK;
}

}  // namespace gv
