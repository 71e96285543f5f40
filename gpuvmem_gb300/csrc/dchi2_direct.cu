// DChi2 as the reference defines it (src/functions.cu:3698-3791): for every
// pixel inside the mask,
//   dchi2(i,j) = -fg_scale * A(i,j) * sum_k w_k (Vr_k.x cos phi + Vr_k.y sin phi),
//   phi = 2 pi (x u_k + y v_k + (z - 1) w_k),
// followed by the chain rule of DChi2_total_I_nu_0 / DChi2_total_alpha
// (src/functions.cu:3968-4024).  This is the exact SIMT engine: one thread
// per pixel, visibilities staged through shared memory in chunks.
//
// Phase arithmetic: the reference forms phi in FP64 and rounds it to float
// before sincospif.  Here the linear part x*u + y*v is reduced mod 1 exactly
// with 32-bit fixed point ((j-x0) * frac(dx*u) mod 2^32), and the small
// quadratic and quartic w-terms are added in FP32:
//   (z-1) w = -(x^2 + y^2) w / 2 + rho(x,y) w,  rho = -r^4/(2(1+z)^2).
// Accumulation is FP32 within a chunk of 256 visibilities and FP64 across
// chunks.
#include "gv_internal.cuh"

namespace gv {

namespace {

constexpr int kChunk = 256;

struct DirectParams {
  int M, N;
  int64_t MN;
  int x0, y0;
  float xobs, yobs, nu_0, D, pbf, pbcut, fg_scale, threshold;
  int pb;
  double DELTAX, DELTAY;
  int normalize;
  int flag_opt;
  int c_begin, c_end;
  int mode;  // 0 gradient (chain rule, 2 planes), 1 raw channel, 2 dirty image, 3 PSF,
             // 4 error-map sum: Re(w Vr e^{+2 pi i (x u + y v)}), no w-term
  const float* gcf;  // gridding correction (modes 0, 1), or null
};

template <bool kDirty>
__global__ void __launch_bounds__(256) k_dchi2_direct(
    DirectParams dp, const float* __restrict__ chfreq, const ChanRange* __restrict__ ranges,
    const int64_t* __restrict__ chnvis, const uint4* __restrict__ ph,
    const float* __restrict__ wl, const float2* __restrict__ cvr,
    const float4* __restrict__ deg, const float2* __restrict__ vo,
    const uint8_t* __restrict__ mask, const float* __restrict__ rho_img,
    const float* __restrict__ img, float* __restrict__ result) {
  __shared__ uint4 s_ph[kChunk];
  __shared__ float2 s_c[kChunk];
  __shared__ float s_w[kChunk];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  const int nthr = blockDim.x * blockDim.y;
  const bool inside = (i < dp.N && j < dp.M);
  const int64_t q = inside ? (int64_t)dp.N * i + j : 0;
  const bool active = inside && (kDirty || (mask[q] & kMaskIn));
  const int jj = j - dp.x0, ii = i - dp.y0;
  // the error maps' phase has no w-term
  const bool wterm = dp.mode != 4;
  const float jj2 = wterm ? (float)jj * (float)jj : 0.0f, ii2 = wterm ? (float)ii * (float)ii : 0.0f;
  const float rho = (inside && wterm) ? rho_img[q] : 0.0f;
  float res0 = 0.0f, res1 = 0.0f;
  double dirty = 0.0;
  for (int c = dp.c_begin; c < dp.c_end; c++) {
    const ChanRange rg = ranges[c];
    double acc = 0.0;
    for (int64_t k0 = 0; k0 < rg.ngrid; k0 += kChunk) {
      const int64_t rem = rg.ngrid - k0;
      const int cnt = rem < kChunk ? (int)rem : kChunk;
      __syncthreads();
      for (int t = tid; t < cnt; t += nthr) {
        const int64_t g = rg.off + k0 + t;
        s_ph[t] = ph[g];
        s_w[t] = wl[g];
        if (kDirty && dp.mode == 4) {
          const float2 r = cvr[g];
          s_c[t] = make_float2(r.x, -r.y);
        } else if (kDirty) {
          const float4 d = deg[g];
          const float2 o = dp.mode == 3 ? make_float2(1.0f, 0.0f) : vo[g];
          s_c[t] = make_float2(d.w * o.x, d.w * o.y);
        } else {
          s_c[t] = cvr[g];
        }
      }
      __syncthreads();
      if (active) {
        float a = 0.0f;
#pragma unroll 4
        for (int t = 0; t < cnt; t++) {
          const uint4 p = s_ph[t];
          const uint32_t lin = (uint32_t)jj * p.x + (uint32_t)ii * p.y;
          float theta = (float)(int32_t)lin * 2.3283064365386963e-10f;
          theta = fmaf(-jj2, __uint_as_float(p.z), theta);
          theta = fmaf(-ii2, __uint_as_float(p.w), theta);
          theta = fmaf(rho, s_w[t], theta);
          float sn, cs;
          sincospif(2.0f * theta, &sn, &cs);
          const float2 cc = s_c[t];
          a = fmaf(cc.x, cs, a);
          a = fmaf(cc.y, sn, a);
        }
        acc += (double)a;
      }
    }
    if (!active) continue;
    if (kDirty) {
      dirty += acc;
      continue;
    }
    const float freq = chfreq[c];
    const float atten = attenuation(i, j, dp.xobs, dp.yobs, dp.DELTAX, dp.DELTAY, freq, dp.D,
                                    dp.pbf, dp.pbcut, dp.pb);
    // fg_scale * atten (* gcf: the GCF variant, src/functions.cu:3834-3836)
    float sf = dp.fg_scale * atten;
    if (dp.gcf) sf *= dp.gcf[q];
    float d = (float)acc * sf;
    if (dp.normalize) d /= (float)chnvis[c];
    d = -d;
    if (dp.mode == 1) {
      res0 += d;
      continue;
    }
    const float nudiv = freq / dp.nu_0;
    const float i0 = img[q], al = img[dp.MN + q];
    const float pw = powf(nudiv, al);
    if (dp.flag_opt % 2 == 0) {
      res0 += d * pw;  // DChi2_total_I_nu_0
    } else if (i0 > dp.threshold) {
      res1 += d * (i0 * pw * dp.fg_scale * logf(nudiv));  // DChi2_total_alpha
    }
  }
  if (!active) return;
  if (kDirty) {
    result[q] += (float)dirty;
  } else if (dp.mode == 1) {
    result[q] += res0;
  } else if (dp.flag_opt % 2 == 0) {
    result[q] += res0;
  } else {
    result[dp.MN + q] += res1;
  }
}

}  // namespace

gv_status dchi2_direct(Problem& P, const float* d_img, int flag_opt, float* d_result,
                       int only_channel, int mode) {
  DirectParams dp;
  dp.M = P.M;
  dp.N = P.N;
  dp.MN = (int64_t)P.M * P.N;
  dp.x0 = (int)P.xobs;
  dp.y0 = (int)P.yobs;
  dp.xobs = P.xobs;
  dp.yobs = P.yobs;
  dp.nu_0 = P.nu_0;
  dp.D = P.D;
  dp.pbf = P.pbf;
  dp.pbcut = P.pbcut;
  dp.fg_scale = P.fg_scale;
  dp.threshold = P.threshold;
  dp.pb = P.pb;
  dp.DELTAX = P.DELTAX;
  dp.DELTAY = P.DELTAY;
  dp.normalize = P.normalize;
  dp.flag_opt = flag_opt;
  dp.c_begin = only_channel >= 0 ? only_channel : 0;
  dp.c_end = only_channel >= 0 ? only_channel + 1 : (int)P.chans.size();
  dp.mode = mode;
  dp.gcf = P.d_gcf;
  dim3 block(16, 16), grid((P.M + 15) / 16, (P.N + 15) / 16);
  if (mode >= 2) {
    k_dchi2_direct<true><<<grid, block, 0, P.stream>>>(
        dp, P.d_chfreq, P.d_ranges, P.d_chnvis, P.d_ph, P.d_wl, P.d_cvr, P.d_deg, P.d_vo,
        P.d_mask, P.d_rho, d_img, d_result);
  } else {
    k_dchi2_direct<false><<<grid, block, 0, P.stream>>>(
        dp, P.d_chfreq, P.d_ranges, P.d_chnvis, P.d_ph, P.d_wl, P.d_cvr, P.d_deg, P.d_vo,
        P.d_mask, P.d_rho, d_img, d_result);
  }
  GV_LAUNCH("k_dchi2_direct");
  return GV_OK;
}

}  // namespace gv
