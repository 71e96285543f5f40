// Warm-start network: a 2-D U-Net (encoder-decoder with skip connections)
// trained on (dirty image + PSF, converged image) pairs.  No counterpart in
// the reference; it is the learned part of the imaging objective path.
//
// Every convolution, in the forward pass and in both backward passes, is a
// BF16 GEMM on the tcgen05 tensor cores with FP32 accumulation in TMEM
// (k_gemm below):
//   forward      M = B*H*W pixels, N = Cout, K = Cin*ks*ks
//   bwd data     M = B*H*W pixels, N = Cin,  K = Cout*ks*ks (flipped taps)
//   bwd weight   M = Cin*ks*ks,    N = Cout, K = B*H*W (split over K, the
//                splits summed in a fixed order)
// The operand tiles are staged by the CTA's threads straight from the FP32
// NCHW activations (im2col on the fly, rounded to BF16) into 128-byte
// swizzled MN-major shared-memory tiles; one thread issues the MMAs; two
// stages alternate.  The epilogue (bias, ReLU, layout) is applied on the way
// out of TMEM.  Pooling, upsampling, the loss and Adam are plain
// bandwidth-bound kernels.
//
// Layout of the network (levels l = 0..L-1, C_l = c0 * 2^l channels, side
// H / 2^l):  enc_l = relu(conv(relu(conv(in_l)))), in_{l+1} = avgpool2(enc_l);
// dec_{L-1} = enc_{L-1}; dec_l = relu(conv(relu(conv([up2(dec_{l+1}), enc_l]))));
// out = conv1x1(dec_0).  Parameters are one flat FP32 vector, layer by layer
// (weights [Cout][Cin][ks][ks], then bias [Cout]) in the order enc_0 ..
// enc_{L-1}, dec_{L-2} .. dec_0, out.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "gv_internal.cuh"
#include "tcgen05.cuh"

namespace gv {
namespace cnn {

using namespace gv::tc;

// ---------------------------------------------------------------- GEMM core
constexpr int kBM = 128, kBK = 64, kGemmThreads = 256;

__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&h);
}

template <int BN>
struct GemmLayout {
  static constexpr uint32_t kSboA = (kBM / 64) * 1024;
  static constexpr uint32_t kTileA = kSboA * (kBK / 8);
  static constexpr uint32_t kSboB = (BN / 64) * 1024;
  static constexpr uint32_t kTileB = kSboB * (kBK / 8);
  static constexpr uint32_t kStage = kTileA + kTileB;
  static constexpr uint32_t kSmem = 1024 + 2 * kStage;
};

// D[m][n] = sum_k A[m][k] B[k][n] over this CTA's K range; op.a(m,k),
// op.b(k,n) fetch FP32 operands, op.store(m, n, v, split) writes a result.
template <class Op, int BN>
__global__ void __launch_bounds__(kGemmThreads) k_gemm(Op op, int M, int N, int K, int klen,
                                                       uint32_t* err) {
  using L = GemmLayout<BN>;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tslot;
  __shared__ int s_abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
  const int kbeg = blockIdx.z * klen;
  const int kend = min(K, kbeg + klen);
  const int nch = kend > kbeg ? (kend - kbeg + kBK - 1) / kBK : 0;
  if (warp == 0) {
    tmem_alloc<false>(&tslot, BN);
    tmem_relinquish<false>();
  }
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tacc = tslot;
  constexpr uint32_t idesc = make_idesc_bf16(kBM, BN);
  bool ok = true;
  for (int c = 0; c < nch; c++) {
    const int st = c & 1;
    // the MMAs that read this stage two chunks ago are done
    if (c >= 2) ok = warp_wait(&bar[st], ((c >> 1) - 1) & 1, &s_abort, err, 11u);
    if (!__syncthreads_and(ok ? 1 : 0)) {
      ok = false;
      break;
    }
    uint8_t* sa = base + st * L::kStage;
    uint8_t* sb = sa + L::kTileA;
    const int k0 = kbeg + c * kBK;
    for (int idx = tid; idx < (kBM / 8) * kBK; idx += kGemmThreads) {
      const int og = idx & (kBM / 8 - 1), kk = idx / (kBM / 8);
      const int k = k0 + kk;
      float v[8];
      const int mg = m0 + og * 8;
      if (k < kend && mg + 7 < M && op.rows8()) {
        op.a8(mg, k, v);
      } else {
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const int m = mg + i;
          v[i] = (k < kend && m < M) ? op.a(m, k) : 0.0f;
        }
      }
      *reinterpret_cast<uint4*>(sa + tile_off(og >> 3, og & 7, kk, L::kSboA)) =
          make_uint4(bf16x2(v[0], v[1]), bf16x2(v[2], v[3]), bf16x2(v[4], v[5]),
                     bf16x2(v[6], v[7]));
    }
    for (int idx = tid; idx < (BN / 8) * kBK; idx += kGemmThreads) {
      const int og = idx % (BN / 8), kk = idx / (BN / 8);
      const int k = k0 + kk;
      float v[8];
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const int n = n0 + og * 8 + i;
        v[i] = (k < kend && n < N) ? op.b(k, n) : 0.0f;
      }
      *reinterpret_cast<uint4*>(sb + tile_off(og >> 3, og & 7, kk, L::kSboB)) =
          make_uint4(bf16x2(v[0], v[1]), bf16x2(v[2], v[3]), bf16x2(v[4], v[5]),
                     bf16x2(v[6], v[7]));
    }
    fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      fence_after();
      const uint32_t aa = smem_u32(sa), ba = smem_u32(sb);
#pragma unroll
      for (int t = 0; t < kBK / 16; t++) {
        const uint64_t ad = make_desc(aa + t * 2 * L::kSboA, 1024, L::kSboA);
        const uint64_t bd = make_desc(ba + t * 2 * L::kSboB, 1024, L::kSboB);
        mma_f16<false>(tacc, ad, bd, idesc, (c > 0 || t > 0) ? 1u : 0u);
      }
      mma_commit<false>(&bar[st]);
    }
  }
  if (ok && nch > 0) {
    const int c = nch - 1;
    ok = warp_wait(&bar[c & 1], (c >> 1) & 1, &s_abort, err, 12u);
  }
  if (__syncthreads_and(ok ? 1 : 0)) {
    fence_after();
    const int q = warp & 3, h = warp >> 2;
    const int m = m0 + 32 * q + lane;
#pragma unroll 1
    for (int cb = h * (BN / 2); cb < (h + 1) * (BN / 2); cb += 32) {
      float v[32];
      if (nch > 0) {
        tmem_ld32(tacc + ((uint32_t)(32 * q) << 16) + (uint32_t)cb, v);
      } else {
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = 0.0f;
      }
      if (m < M) {
#pragma unroll 4
        for (int j = 0; j < 32; j++) {
          const int n = n0 + cb + j;
          if (n < N) op.store(m, n, v[j], (int)blockIdx.z);
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) tmem_dealloc<false>(tacc, BN);
}

// A channel slice of an NCHW tensor: element (b, c, y, x) of the slice is
// p[((b * C + c0 + c) * H + y) * W + x].
struct View {
  float* p;
  int C, c0;
};

// forward: y = act(conv(x) + bias); with split-K (part set) each split
// stores its partial sum to part[split][n][m] and k_conv_fwd_finish adds
// the splits, the bias and the activation
struct ConvFwdOp {
  const float* x;
  int xC, xc0;
  const float* w;
  const float* bias;
  float* y;
  int yC, yc0;
  int Cin, Cout, H, W, ks, relu;
  float* part;
  int M;
  __device__ float a(int m, int k) const {
    const int HW = H * W;
    const int b = m / HW, r = m - b * HW, y0 = r / W, x0 = r - y0 * W;
    const int kk = ks * ks, cin = k / kk, t = k - cin * kk;
    const int yy = y0 + t / ks - ks / 2, xx = x0 + t % ks - ks / 2;
    if ((unsigned)yy >= (unsigned)H || (unsigned)xx >= (unsigned)W) return 0.0f;
    return x[((size_t)(b * xC + xc0 + cin) * H + yy) * W + xx];
  }
  // a(m + i, k) for i < 8, when rows m..m+7 are in one image row (rows8):
  // the index arithmetic once for the eight
  __device__ bool rows8() const { return (W & 7) == 0; }
  __device__ void a8(int m, int k, float* v) const {
    const int HW = H * W;
    const int b = m / HW, r = m - b * HW, y0 = r / W, x0 = r - y0 * W;
    const int kk = ks * ks, cin = k / kk, t = k - cin * kk;
    const int yy = y0 + t / ks - ks / 2, dx = t % ks - ks / 2;
    const bool rowok = (unsigned)yy < (unsigned)H;
    const float* row = x + ((size_t)(b * xC + xc0 + cin) * H + (rowok ? yy : 0)) * W;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int xx = x0 + i + dx;
      v[i] = (rowok && (unsigned)xx < (unsigned)W) ? row[xx] : 0.0f;
    }
  }
  __device__ float b(int k, int n) const { return w[(size_t)n * Cin * ks * ks + k]; }
  __device__ void store(int m, int n, float v, int split) const {
    if (part) {
      part[((size_t)split * Cout + n) * M + m] = v;
      return;
    }
    const int HW = H * W;
    const int b = m / HW, r = m - b * HW;
    v += bias[n];
    if (relu) v = fmaxf(v, 0.0f);
    y[(size_t)(b * yC + yc0 + n) * HW + r] = v;
  }
};

// split-K forward: y = act(sum over splits in order + bias)
__global__ void k_conv_fwd_finish(int M, int N, int nsplit, const float* __restrict__ part,
                                  const float* __restrict__ bias, int relu, float* __restrict__ y,
                                  int yC, int yc0, int HW) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= (size_t)M * N) return;
  const int n = (int)(i / M), m = (int)(i - (size_t)n * M);
  float s = 0.0f;
  for (int k = 0; k < nsplit; k++) s += part[((size_t)k * N + n) * M + m];
  s += bias[n];
  if (relu) s = fmaxf(s, 0.0f);
  const int b = m / HW, r = m - b * HW;
  y[(size_t)(b * yC + yc0 + n) * HW + r] = s;
}

// backward data: dx (+)= conv of dz with the taps flipped
struct ConvBwdDataOp {
  const float* dz;
  int zC, zc0;
  const float* w;
  float* dx;
  int xC, xc0;
  int Cin, Cout, H, W, ks, accumulate;
  __device__ float a(int m, int k) const {
    const int HW = H * W;
    const int b = m / HW, r = m - b * HW, y0 = r / W, x0 = r - y0 * W;
    const int kk = ks * ks, co = k / kk, t = k - co * kk;
    const int yy = y0 - t / ks + ks / 2, xx = x0 - t % ks + ks / 2;
    if ((unsigned)yy >= (unsigned)H || (unsigned)xx >= (unsigned)W) return 0.0f;
    return dz[((size_t)(b * zC + zc0 + co) * H + yy) * W + xx];
  }
  __device__ bool rows8() const { return (W & 7) == 0; }
  __device__ void a8(int m, int k, float* v) const {
    const int HW = H * W;
    const int b = m / HW, r = m - b * HW, y0 = r / W, x0 = r - y0 * W;
    const int kk = ks * ks, co = k / kk, t = k - co * kk;
    const int yy = y0 - t / ks + ks / 2, dx = -(t % ks) + ks / 2;
    const bool rowok = (unsigned)yy < (unsigned)H;
    const float* row = dz + ((size_t)(b * zC + zc0 + co) * H + (rowok ? yy : 0)) * W;
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const int xx = x0 + i + dx;
      v[i] = (rowok && (unsigned)xx < (unsigned)W) ? row[xx] : 0.0f;
    }
  }
  __device__ float b(int k, int n) const {
    const int kk = ks * ks, co = k / kk, t = k - co * kk;
    return w[((size_t)co * Cin + n) * kk + t];
  }
  __device__ void store(int m, int n, float v, int) const {
    const int HW = H * W;
    const int b = m / HW, r = m - b * HW;
    float* o = dx + (size_t)(b * xC + xc0 + n) * HW + r;
    *o = accumulate ? *o + v : v;
  }
};

// backward weight: partial[split][cout][cin*ks*ks] = sum over this split's
// pixels of dz * x (shifted)
struct ConvBwdWeightOp {
  const float* x;
  int xC, xc0;
  const float* dz;
  int zC, zc0;
  float* partial;
  int Cin, Cout, H, W, ks;
  __device__ float a(int m, int k) const {
    const int kk = ks * ks, cin = m / kk, t = m - cin * kk;
    const int HW = H * W;
    const int b = k / HW, r = k - b * HW, y0 = r / W, x0 = r - y0 * W;
    const int yy = y0 + t / ks - ks / 2, xx = x0 + t % ks - ks / 2;
    if ((unsigned)yy >= (unsigned)H || (unsigned)xx >= (unsigned)W) return 0.0f;
    return x[((size_t)(b * xC + xc0 + cin) * H + yy) * W + xx];
  }
  __device__ bool rows8() const { return false; }  // rows are (cin, tap) pairs
  __device__ void a8(int, int, float*) const {}
  __device__ float b(int k, int n) const {
    const int HW = H * W;
    const int b = k / HW, r = k - b * HW;
    return dz[(size_t)(b * zC + zc0 + n) * HW + r];
  }
  __device__ void store(int m, int n, float v, int split) const {
    const size_t wn = (size_t)Cout * Cin * ks * ks;
    partial[split * wn + (size_t)n * Cin * ks * ks + m] = v;
  }
};

// --------------------------------------------------------- plain kernels
// dw = sum over splits (fixed order), db[c] = sum over pixels of dz
__global__ void k_sum_splits(size_t n, int nsplit, const float* __restrict__ part,
                             float* __restrict__ out) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float s = 0.0f;
  for (int k = 0; k < nsplit; k++) s += part[k * n + i];
  out[i] = s;
}

__global__ void k_bias_grad(int B, int HW, View dz, float* __restrict__ db) {
  const int c = blockIdx.x;
  float s = 0.0f;
  for (int b = 0; b < B; b++) {
    const float* p = dz.p + (size_t)(b * dz.C + dz.c0 + c) * HW;
    for (int i = threadIdx.x; i < HW; i += blockDim.x) s += p[i];
  }
  __shared__ float red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) db[c] = s;
  }
}

// dz = g * (y > 0) over a slice of C channels (in place when g == dz)
__global__ void k_relu_mask(int B, int C, int HW, View g, View y, View dz) {
  const size_t n = (size_t)B * C * HW;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i % HW);
    const size_t bc = i / HW;
    const int c = (int)(bc % C), b = (int)(bc / C);
    const float yv = y.p[(size_t)(b * y.C + y.c0 + c) * HW + r];
    const float gv = g.p[(size_t)(b * g.C + g.c0 + c) * HW + r];
    dz.p[(size_t)(b * dz.C + dz.c0 + c) * HW + r] = yv > 0.0f ? gv : 0.0f;
  }
}

// y = 2x2 average of x (x is H x W, y is H/2 x W/2)
__global__ void k_pool2(int B, int C, int H, int W, View x, View y) {
  const int Ho = H / 2, Wo = W / 2;
  const size_t n = (size_t)B * C * Ho * Wo;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int xo = (int)(i % Wo), yo = (int)((i / Wo) % Ho);
    const size_t bc = i / ((size_t)Wo * Ho);
    const int c = (int)(bc % C), b = (int)(bc / C);
    const float* s = x.p + ((size_t)(b * x.C + x.c0 + c) * H + 2 * yo) * W + 2 * xo;
    y.p[((size_t)(b * y.C + y.c0 + c) * Ho + yo) * Wo + xo] =
        0.25f * ((s[0] + s[1]) + (s[W] + s[W + 1]));
  }
}

// dx (+)= dy / 4 broadcast over each 2x2 block
__global__ void k_pool2_bwd(int B, int C, int H, int W, View dy, View dx, int accumulate) {
  const size_t n = (size_t)B * C * H * W;
  const int Ho = H / 2, Wo = W / 2;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(i % W), yy = (int)((i / W) % H);
    const size_t bc = i / ((size_t)W * H);
    const int c = (int)(bc % C), b = (int)(bc / C);
    const float g =
        0.25f * dy.p[((size_t)(b * dy.C + dy.c0 + c) * Ho + yy / 2) * Wo + xx / 2];
    float* o = dx.p + ((size_t)(b * dx.C + dx.c0 + c) * H + yy) * W + xx;
    *o = accumulate ? *o + g : g;
  }
}

// y = nearest 2x upsample of x (x is H x W)
__global__ void k_up2(int B, int C, int H, int W, View x, View y) {
  const int Ho = 2 * H, Wo = 2 * W;
  const size_t n = (size_t)B * C * Ho * Wo;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int xo = (int)(i % Wo), yo = (int)((i / Wo) % Ho);
    const size_t bc = i / ((size_t)Wo * Ho);
    const int c = (int)(bc % C), b = (int)(bc / C);
    y.p[((size_t)(b * y.C + y.c0 + c) * Ho + yo) * Wo + xo] =
        x.p[((size_t)(b * x.C + x.c0 + c) * H + yo / 2) * W + xo / 2];
  }
}

// dx = sum of dy over each 2x2 block (dx is H x W)
__global__ void k_up2_bwd(int B, int C, int H, int W, View dy, View dx) {
  const size_t n = (size_t)B * C * H * W;
  const int Wo = 2 * W;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int xx = (int)(i % W), yy = (int)((i / W) % H);
    const size_t bc = i / ((size_t)W * H);
    const int c = (int)(bc % C), b = (int)(bc / C);
    const float* s = dy.p + ((size_t)(b * dy.C + dy.c0 + c) * (2 * H) + 2 * yy) * Wo + 2 * xx;
    dx.p[((size_t)(b * dx.C + dx.c0 + c) * H + yy) * W + xx] = (s[0] + s[1]) + (s[Wo] + s[Wo + 1]);
  }
}

// loss = mean (out - t)^2 (per-block FP64 partials), dout = 2 (out - t) / n
__global__ void k_mse(size_t n, const float* __restrict__ out, const float* __restrict__ t,
                      float* __restrict__ dout, double* __restrict__ part) {
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float d = out[i] - t[i];
    s += (double)d * d;
    if (dout) dout[i] = 2.0f * d / (float)n;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
  }
}

// Adam (Kingma & Ba 2015) with bias correction, FP32 state
__global__ void k_adam(size_t n, float* __restrict__ w, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// ------------------------------------------------------------ host side
struct Ctx {
  cudaStream_t stream;
  uint32_t* err;
  int num_sms;
  float* part;  // split-K scratch for the weight gradient
  size_t part_floats;
};

template <class Op, int BN>
gv_status launch_gemm_bn(const Ctx& c, const Op& op, int M, int N, int K, int nsplit) {
  auto kern = k_gemm<Op, BN>;
  const int smem = (int)GemmLayout<BN>::kSmem;
  GV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const int klen = ((K + nsplit - 1) / nsplit + kBK - 1) / kBK * kBK;
  const int nz = (K + klen - 1) / klen;
  dim3 grid((M + kBM - 1) / kBM, (N + BN - 1) / BN, nz);
  kern<<<grid, kGemmThreads, smem, c.stream>>>(op, M, N, K, klen, c.err);
  GV_LAUNCH("k_gemm");
  return GV_OK;
}

template <class Op>
gv_status launch_gemm(const Ctx& c, const Op& op, int M, int N, int K, int nsplit = 1) {
  if (N <= 64) return launch_gemm_bn<Op, 64>(c, op, M, N, K, nsplit);
  if (N <= 128) return launch_gemm_bn<Op, 128>(c, op, M, N, K, nsplit);
  return launch_gemm_bn<Op, 256>(c, op, M, N, K, nsplit);  // column tiles of 256
}

inline int ew_blocks(size_t n, const Ctx& c) {
  return (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, (size_t)8 * c.num_sms));
}

gv_status conv_forward(const Ctx& c, View x, const float* w, const float* bias, View y, int B,
                       int Cin, int Cout, int H, int W, int ks, int relu) {
  const int M = B * H * W, N = Cout, K = Cin * ks * ks;
  // a grid of fewer tiles than SMs (deep levels, small batches) splits K
  // over up to two CTAs per SM, at least two K blocks a split
  const int bn = N <= 64 ? 64 : (N <= 128 ? 128 : 256);
  const int tiles = ((M + kBM - 1) / kBM) * ((N + bn - 1) / bn);
  int nsplit = 1;
  if (c.part && tiles < c.num_sms) {
    nsplit = std::min(K / (2 * kBK), (2 * c.num_sms + tiles - 1) / tiles);
    nsplit = std::max(1, std::min<int>(nsplit, (int)(c.part_floats / ((size_t)M * N))));
  }
  ConvFwdOp op{x.p, x.C, x.c0, w, bias, y.p, y.C, y.c0, Cin, Cout, H, W, ks, relu,
               nsplit > 1 ? c.part : nullptr, M};
  gv_status s = launch_gemm(c, op, M, N, K, nsplit);
  if (s != GV_OK || nsplit <= 1) return s;
  // the kernel launched ceil(K / klen) splits; sum exactly those
  const int klen = ((K + nsplit - 1) / nsplit + kBK - 1) / kBK * kBK;
  const int nz = (K + klen - 1) / klen;
  k_conv_fwd_finish<<<(unsigned)(((size_t)M * N + 255) / 256), 256, 0, c.stream>>>(
      M, N, nz, c.part, bias, relu, y.p, y.C, y.c0, H * W);
  GV_LAUNCH("k_conv_fwd_finish");
  return GV_OK;
}

gv_status conv_backward_data(const Ctx& c, View dz, const float* w, View dx, int B, int Cin,
                             int Cout, int H, int W, int ks, int accumulate) {
  ConvBwdDataOp op{dz.p, dz.C, dz.c0, w, dx.p, dx.C, dx.c0, Cin, Cout, H, W, ks, accumulate};
  return launch_gemm(c, op, B * H * W, Cin, Cout * ks * ks);
}

gv_status conv_backward_weight(const Ctx& c, View x, View dz, float* dw, float* db, int B,
                               int Cin, int Cout, int H, int W, int ks) {
  const int M = Cin * ks * ks, N = Cout, K = B * H * W;
  const int tiles = ((M + kBM - 1) / kBM) * ((N + 255) / 256);
  const size_t wn = (size_t)M * N;
  int nsplit = std::max(1, std::min(K / 1024, (2 * c.num_sms + tiles - 1) / tiles));
  nsplit = std::max(1, std::min<int>(nsplit, (int)(c.part_floats / wn)));
  ConvBwdWeightOp op{x.p, x.C, x.c0, dz.p, dz.C, dz.c0, c.part, Cin, Cout, H, W, ks};
  gv_status s = launch_gemm(c, op, M, N, K, nsplit);
  if (s != GV_OK) return s;
  // the kernel launched ceil(K / klen) splits; sum exactly those
  const int klen = ((K + nsplit - 1) / nsplit + kBK - 1) / kBK * kBK;
  const int nz = (K + klen - 1) / klen;
  k_sum_splits<<<(unsigned)((wn + 255) / 256), 256, 0, c.stream>>>(wn, nz, c.part, dw);
  GV_LAUNCH("k_sum_splits");
  k_bias_grad<<<Cout, 256, 0, c.stream>>>(B, H * W, dz, db);
  GV_LAUNCH("k_bias_grad");
  return GV_OK;
}

// ----------------------------------------------------------------- U-Net
struct Layer {
  int cin, cout, ks, relu, side;
  size_t w, b;  // offsets into the parameter vector
};

struct UNet {
  int H = 0, W = 0, cin = 0, c0 = 0, L = 0, maxB = 0;
  std::vector<Layer> layers;
  size_t nparams = 0;
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
  int step = 0;
  // activations and gradients (device), see the layout comment at the top
  std::vector<float*> in, a, enc, cat, b, dec;      // per level
  std::vector<float*> din, da, denc, dcat, dbuf, ddec;
  float *out = nullptr, *dout = nullptr;
  double* loss_part = nullptr;
  double* h_loss = nullptr;
  uint32_t* err = nullptr;
  float* part = nullptr;
  size_t part_floats = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  std::vector<void*> allocs;
  // forward passes captured as CUDA graphs, one per batch size (the pass
  // only reads and writes the network's own buffers, so a graph stays valid)
  std::vector<cudaGraphExec_t> fwd_exec;
  std::vector<int64_t> fwd_launches;
  cudaStream_t cap = nullptr;

  int C(int l) const { return c0 << l; }
  int S(int l) const { return H >> l; }
  Ctx ctx() const { return Ctx{stream, err, num_sms, part, part_floats}; }

  gv_status alloc(float** p, size_t n) {
    GV_CUDA(cudaMalloc(p, std::max<size_t>(n, 1) * sizeof(float)));
    GV_CUDA(cudaMemsetAsync(*p, 0, std::max<size_t>(n, 1) * sizeof(float), stream));
    allocs.push_back(*p);
    return GV_OK;
  }
  ~UNet() {
    for (cudaGraphExec_t g : fwd_exec)
      if (g) cudaGraphExecDestroy(g);
    if (cap) cudaStreamDestroy(cap);
    for (void* p : allocs) cudaFree(p);
    if (h_loss) cudaFreeHost(h_loss);
  }

  // layer index helpers: enc l -> 2l, 2l+1; dec l (l = L-2..0) -> 2L + 2(L-2-l), +1; out last
  int enc_layer(int l, int j) const { return 2 * l + j; }
  int dec_layer(int l, int j) const { return 2 * L + 2 * (L - 2 - l) + j; }
  int out_layer() const { return 2 * L + 2 * (L - 1); }

  gv_status build(const gv_unet_desc& d) {
    H = d.height;
    W = d.width;
    cin = d.in_channels;
    c0 = d.base_channels;
    L = d.levels;
    maxB = d.max_batch;
    size_t off = 0;
    auto add = [&](int ci, int co, int ks, int relu, int side) {
      Layer ly{ci, co, ks, relu, side, off, off + (size_t)co * ci * ks * ks};
      off = ly.b + co;
      layers.push_back(ly);
    };
    for (int l = 0; l < L; l++) {
      add(l == 0 ? cin : C(l - 1), C(l), 3, 1, S(l));
      add(C(l), C(l), 3, 1, S(l));
    }
    for (int l = L - 2; l >= 0; l--) {
      add(C(l + 1) + C(l), C(l), 3, 1, S(l));
      add(C(l), C(l), 3, 1, S(l));
    }
    add(C(0), 1, 1, 0, S(0));
    nparams = off;
    GV_TRY(alloc(&params, nparams));
    GV_TRY(alloc(&grads, nparams));
    GV_TRY(alloc(&m, nparams));
    GV_TRY(alloc(&v, nparams));
    // He-normal weights, zero biases (seeded)
    std::vector<float> h(nparams, 0.0f);
    std::mt19937_64 rng(d.seed);
    for (const Layer& ly : layers) {
      std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (float)(ly.cin * ly.ks * ly.ks)));
      for (size_t i = ly.w; i < ly.b; i++) h[i] = nd(rng);
    }
    GV_CUDA(cudaMemcpyAsync(params, h.data(), nparams * sizeof(float), cudaMemcpyHostToDevice,
                            stream));
    const size_t B = maxB;
    in.resize(L);
    a.resize(L);
    enc.resize(L);
    cat.resize(L);
    b.resize(L);
    dec.resize(L);
    din.resize(L);
    da.resize(L);
    denc.resize(L);
    dcat.resize(L);
    dbuf.resize(L);
    ddec.resize(L);
    for (int l = 0; l < L; l++) {
      const size_t px = B * (size_t)S(l) * S(l);
      const int cin_l = l == 0 ? cin : C(l - 1);
      GV_TRY(alloc(&in[l], px * cin_l));
      GV_TRY(alloc(&a[l], px * C(l)));
      GV_TRY(alloc(&din[l], px * cin_l));
      GV_TRY(alloc(&da[l], px * C(l)));
      if (l < L - 1) {
        // enc_l lives in channels [C(l+1), C(l+1) + C(l)) of the concat buffer
        GV_TRY(alloc(&cat[l], px * (C(l + 1) + C(l))));
        GV_TRY(alloc(&dcat[l], px * (C(l + 1) + C(l))));
        GV_TRY(alloc(&b[l], px * C(l)));
        GV_TRY(alloc(&dbuf[l], px * C(l)));
        GV_TRY(alloc(&dec[l], px * C(l)));
        GV_TRY(alloc(&ddec[l], px * C(l)));
      } else {
        GV_TRY(alloc(&enc[l], px * C(l)));
        GV_TRY(alloc(&denc[l], px * C(l)));
      }
    }
    GV_TRY(alloc(&out, B * (size_t)H * W));
    GV_TRY(alloc(&dout, B * (size_t)H * W));
    part_floats = (size_t)4 << 20;  // 16 MB of split-K partials
    GV_TRY(alloc(&part, part_floats));
    GV_CUDA(cudaMalloc(&loss_part, sizeof(double) * 1024));
    allocs.push_back(loss_part);
    GV_CUDA(cudaMalloc(&err, sizeof(uint32_t)));
    allocs.push_back(err);
    GV_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), stream));
    GV_CUDA(cudaMallocHost(&h_loss, sizeof(double) * 1024));
    return GV_OK;
  }

  // views of enc_l (inside the concat buffer for l < L-1) and its gradient
  View enc_view(int l) const {
    if (l < L - 1) return View{cat[l], C(l + 1) + C(l), C(l + 1)};
    return View{enc[l], C(l), 0};
  }
  View denc_view(int l) const {
    if (l < L - 1) return View{dcat[l], C(l + 1) + C(l), C(l + 1)};
    return View{denc[l], C(l), 0};
  }
  View dec_view(int l) const { return l == L - 1 ? enc_view(l) : View{dec[l], C(l), 0}; }
  View ddec_view(int l) const { return l == L - 1 ? denc_view(l) : View{ddec[l], C(l), 0}; }

  // The input is copied into the network's buffer, then the pass is one
  // graph launch (captured on first use for this batch size on a private
  // stream; a batch-1 pass is some 40 small kernels whose launch latency
  // would otherwise set its time).
  gv_status forward(const float* d_in, int B) {
    GV_CUDA(cudaMemcpyAsync(in[0], d_in, sizeof(float) * B * cin * H * W,
                            cudaMemcpyDeviceToDevice, stream));
    if (fwd_exec.empty()) {
      fwd_exec.assign(maxB + 1, nullptr);
      fwd_launches.assign(maxB + 1, 0);
    }
    if (!fwd_exec[B]) {
      if (!cap) GV_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
      const cudaStream_t saved = stream;
      const int64_t l0 = gv_launch_count();
      stream = cap;
      cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed);
      if (e != cudaSuccess) {
        stream = saved;
        return cuda_fail(e, "cudaStreamBeginCapture (U-Net forward)");
      }
      const gv_status s = forward_pass(B);
      cudaGraph_t g = nullptr;
      e = cudaStreamEndCapture(cap, &g);
      stream = saved;
      const int64_t nl = gv_launch_count() - l0;
      add_launches(-nl);  // counted again at each replay
      if (s != GV_OK) {
        if (g) cudaGraphDestroy(g);
        return s;
      }
      if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture (U-Net forward)");
      cudaGraphExec_t x = nullptr;
      e = cudaGraphInstantiate(&x, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate (U-Net forward)");
      fwd_exec[B] = x;
      fwd_launches[B] = nl;
    }
    GV_CUDA(cudaGraphLaunch(fwd_exec[B], stream));
    add_launches(fwd_launches[B]);
    return GV_OK;
  }

  // the forward pass on the network's input buffer in[0]
  gv_status forward_pass(int B) {
    const Ctx c = ctx();
    for (int l = 0; l < L; l++) {
      const int s = S(l), ci = l == 0 ? cin : C(l - 1);
      const Layer& l1 = layers[enc_layer(l, 0)];
      const Layer& l2 = layers[enc_layer(l, 1)];
      GV_TRY(conv_forward(c, View{in[l], ci, 0}, params + l1.w, params + l1.b, View{a[l], C(l), 0},
                          B, ci, C(l), s, s, 3, 1));
      GV_TRY(conv_forward(c, View{a[l], C(l), 0}, params + l2.w, params + l2.b, enc_view(l), B,
                          C(l), C(l), s, s, 3, 1));
      if (l + 1 < L) {
        const size_t n = (size_t)B * C(l) * (s / 2) * (s / 2);
        k_pool2<<<ew_blocks(n, c), 256, 0, stream>>>(B, C(l), s, s, enc_view(l),
                                                     View{in[l + 1], C(l), 0});
        GV_LAUNCH("k_pool2");
      }
    }
    for (int l = L - 2; l >= 0; l--) {
      const int s = S(l), cc = C(l + 1) + C(l);
      const size_t n = (size_t)B * C(l + 1) * s * s;
      k_up2<<<ew_blocks(n, c), 256, 0, stream>>>(B, C(l + 1), s / 2, s / 2, dec_view(l + 1),
                                                 View{cat[l], cc, 0});
      GV_LAUNCH("k_up2");
      const Layer& l1 = layers[dec_layer(l, 0)];
      const Layer& l2 = layers[dec_layer(l, 1)];
      GV_TRY(conv_forward(c, View{cat[l], cc, 0}, params + l1.w, params + l1.b, View{b[l], C(l), 0},
                          B, cc, C(l), s, s, 3, 1));
      GV_TRY(conv_forward(c, View{b[l], C(l), 0}, params + l2.w, params + l2.b, dec_view(l), B,
                          C(l), C(l), s, s, 3, 1));
    }
    const Layer& lo = layers[out_layer()];
    return conv_forward(c, dec_view(0), params + lo.w, params + lo.b, View{out, 1, 0}, B, C(0), 1,
                        H, W, 1, 0);
  }

  // gradients of the loss with respect to every parameter, given dout
  gv_status backward(int B) {
    const Ctx c = ctx();
    const Layer& lo = layers[out_layer()];
    GV_TRY(conv_backward_weight(c, dec_view(0), View{dout, 1, 0}, grads + lo.w, grads + lo.b, B,
                                C(0), 1, H, W, 1));
    GV_TRY(conv_backward_data(c, View{dout, 1, 0}, params + lo.w, ddec_view(0), B, C(0), 1, H, W,
                              1, 0));
    for (int l = 0; l <= L - 2; l++) {
      const int s = S(l), cc = C(l + 1) + C(l);
      const Layer& l1 = layers[dec_layer(l, 0)];
      const Layer& l2 = layers[dec_layer(l, 1)];
      const size_t nl = (size_t)B * C(l) * s * s;
      // second decoder conv: ReLU mask, weight and data gradients
      k_relu_mask<<<ew_blocks(nl, c), 256, 0, stream>>>(B, C(l), s * s, ddec_view(l), dec_view(l),
                                                        ddec_view(l));
      GV_LAUNCH("k_relu_mask");
      GV_TRY(conv_backward_weight(c, View{b[l], C(l), 0}, ddec_view(l), grads + l2.w,
                                  grads + l2.b, B, C(l), C(l), s, s, 3));
      GV_TRY(conv_backward_data(c, ddec_view(l), params + l2.w, View{dbuf[l], C(l), 0}, B, C(l),
                                C(l), s, s, 3, 0));
      k_relu_mask<<<ew_blocks(nl, c), 256, 0, stream>>>(B, C(l), s * s, View{dbuf[l], C(l), 0},
                                                        View{b[l], C(l), 0},
                                                        View{dbuf[l], C(l), 0});
      GV_LAUNCH("k_relu_mask");
      GV_TRY(conv_backward_weight(c, View{cat[l], cc, 0}, View{dbuf[l], C(l), 0}, grads + l1.w,
                                  grads + l1.b, B, cc, C(l), s, s, 3));
      GV_TRY(conv_backward_data(c, View{dbuf[l], C(l), 0}, params + l1.w, View{dcat[l], cc, 0}, B,
                                cc, C(l), s, s, 3, 0));
      // the upsampled part of the concat feeds dec_{l+1}
      const size_t nu = (size_t)B * C(l + 1) * (s / 2) * (s / 2);
      k_up2_bwd<<<ew_blocks(nu, c), 256, 0, stream>>>(B, C(l + 1), s / 2, s / 2,
                                                      View{dcat[l], cc, 0}, ddec_view(l + 1));
      GV_LAUNCH("k_up2_bwd");
    }
    for (int l = L - 1; l >= 0; l--) {
      const int s = S(l), ci = l == 0 ? cin : C(l - 1);
      const Layer& l1 = layers[enc_layer(l, 0)];
      const Layer& l2 = layers[enc_layer(l, 1)];
      const size_t nl = (size_t)B * C(l) * s * s;
      if (l + 1 < L) {
        // enc_l also feeds the pool of level l+1: add that gradient
        k_pool2_bwd<<<ew_blocks(nl, c), 256, 0, stream>>>(B, C(l), s, s, View{din[l + 1], C(l), 0},
                                                          denc_view(l), 1);
        GV_LAUNCH("k_pool2_bwd");
      }
      k_relu_mask<<<ew_blocks(nl, c), 256, 0, stream>>>(B, C(l), s * s, denc_view(l), enc_view(l),
                                                        denc_view(l));
      GV_LAUNCH("k_relu_mask");
      GV_TRY(conv_backward_weight(c, View{a[l], C(l), 0}, denc_view(l), grads + l2.w, grads + l2.b,
                                  B, C(l), C(l), s, s, 3));
      GV_TRY(conv_backward_data(c, denc_view(l), params + l2.w, View{da[l], C(l), 0}, B, C(l), C(l),
                                s, s, 3, 0));
      k_relu_mask<<<ew_blocks(nl, c), 256, 0, stream>>>(B, C(l), s * s, View{da[l], C(l), 0},
                                                        View{a[l], C(l), 0}, View{da[l], C(l), 0});
      GV_LAUNCH("k_relu_mask");
      GV_TRY(conv_backward_weight(c, View{in[l], ci, 0}, View{da[l], C(l), 0}, grads + l1.w,
                                  grads + l1.b, B, ci, C(l), s, s, 3));
      if (l > 0)
        GV_TRY(conv_backward_data(c, View{da[l], C(l), 0}, params + l1.w, View{din[l], ci, 0}, B,
                                  ci, C(l), s, s, 3, 0));
    }
    return GV_OK;
  }

  gv_status loss(const float* d_target, int B, bool grad, double* out_loss) {
    const size_t n = (size_t)B * H * W;
    const int nb = 256;
    k_mse<<<nb, 256, 0, stream>>>(n, out, d_target, grad ? dout : nullptr, loss_part);
    GV_LAUNCH("k_mse");
    GV_CUDA(cudaMemcpyAsync(h_loss, loss_part, sizeof(double) * nb, cudaMemcpyDeviceToHost,
                            stream));
    GV_CUDA(cudaStreamSynchronize(stream));
    double s = 0.0;
    for (int i = 0; i < nb; i++) s += h_loss[i];
    if (out_loss) *out_loss = s / (double)n;
    return check();
  }

  gv_status adam(float lr) {
    step++;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.0f - std::pow(b1, (float)step), c2 = 1.0f - std::pow(b2, (float)step);
    const Ctx c = ctx();
    k_adam<<<ew_blocks(nparams, c), 256, 0, stream>>>(nparams, params, grads, m, v, lr, b1, b2,
                                                      eps, c1, c2);
    GV_LAUNCH("k_adam");
    return GV_OK;
  }

  gv_status check() {
    uint32_t e = 0;
    GV_CUDA(cudaMemcpyAsync(&e, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
    GV_CUDA(cudaStreamSynchronize(stream));
    if (e) {
      GV_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), stream));
      set_error("a tensor-core GEMM gave up on a bounded wait (device error word " +
                std::to_string(e) + ")");
      return GV_ERR_DEVICE;
    }
    return GV_OK;
  }
};

}  // namespace cnn
}  // namespace gv

struct gv_unet {
  gv::cnn::UNet net;
};

namespace {

gv_status check_batch(const gv_unet* n, int32_t batch) {
  if (!n || batch < 1 || batch > n->net.maxB) {
    gv::set_error("null network or batch outside [1, max_batch]");
    return GV_ERR_INVALID;
  }
  return GV_OK;
}

gv::cnn::Ctx standalone_ctx(void* stream, uint32_t* err, float* part, size_t part_floats) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return gv::cnn::Ctx{(cudaStream_t)stream, err, sms, part, part_floats};
}

}  // namespace

extern "C" {

gv_status gv_unet_create(const gv_unet_desc* d, gv_unet** out) {
  if (!d || !out) {
    gv::set_error("null descriptor or output");
    return GV_ERR_INVALID;
  }
  *out = nullptr;
  if (d->levels < 1 || d->levels > 6 || d->base_channels < 8 || d->base_channels % 8 != 0 ||
      d->in_channels < 1 || d->max_batch < 1 || d->height != d->width ||
      (d->height >> (d->levels - 1)) < 2 || (d->height % (1 << (d->levels - 1))) != 0 ||
      (d->base_channels << (d->levels - 1)) > 256) {
    gv::set_error("unsupported network shape (square image divisible by 2^(levels-1), "
                  "base channels a multiple of 8, at most 256 channels)");
    return GV_ERR_INVALID;
  }
  gv_unet* n = new gv_unet();
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n->net.num_sms, cudaDevAttrMultiProcessorCount, dev);
  gv_status s = n->net.build(*d);
  if (s == GV_OK) {
    cudaError_t e = cudaStreamSynchronize(n->net.stream);
    if (e != cudaSuccess) s = gv::cuda_fail(e, "unet set-up");
  }
  if (s != GV_OK) {
    delete n;
    return s;
  }
  *out = n;
  return GV_OK;
}

gv_status gv_unet_destroy(gv_unet* n) {
  if (!n) return GV_OK;
  cudaStreamSynchronize(n->net.stream);
  delete n;
  return GV_OK;
}

gv_status gv_unet_set_stream(gv_unet* n, void* stream) {
  if (!n) return GV_ERR_INVALID;
  n->net.stream = (cudaStream_t)stream;
  return GV_OK;
}

gv_status gv_unet_num_params(const gv_unet* n, int64_t* count) {
  if (!n || !count) return GV_ERR_INVALID;
  *count = (int64_t)n->net.nparams;
  return GV_OK;
}

gv_status gv_unet_get_params(gv_unet* n, float* d_out) {
  if (!n || !d_out) return GV_ERR_INVALID;
  GV_CUDA(cudaMemcpyAsync(d_out, n->net.params, sizeof(float) * n->net.nparams,
                          cudaMemcpyDeviceToDevice, n->net.stream));
  GV_CUDA(cudaStreamSynchronize(n->net.stream));
  return GV_OK;
}

gv_status gv_unet_set_params(gv_unet* n, const float* d_in) {
  if (!n || !d_in) return GV_ERR_INVALID;
  GV_CUDA(cudaMemcpyAsync(n->net.params, d_in, sizeof(float) * n->net.nparams,
                          cudaMemcpyDeviceToDevice, n->net.stream));
  GV_CUDA(cudaMemsetAsync(n->net.m, 0, sizeof(float) * n->net.nparams, n->net.stream));
  GV_CUDA(cudaMemsetAsync(n->net.v, 0, sizeof(float) * n->net.nparams, n->net.stream));
  n->net.step = 0;
  GV_CUDA(cudaStreamSynchronize(n->net.stream));
  return GV_OK;
}

gv_status gv_unet_get_grads(gv_unet* n, float* d_out) {
  if (!n || !d_out) return GV_ERR_INVALID;
  GV_CUDA(cudaMemcpyAsync(d_out, n->net.grads, sizeof(float) * n->net.nparams,
                          cudaMemcpyDeviceToDevice, n->net.stream));
  GV_CUDA(cudaStreamSynchronize(n->net.stream));
  return GV_OK;
}

gv_status gv_unet_forward(gv_unet* n, const float* d_in, int32_t batch, float* d_out) {
  GV_TRY(check_batch(n, batch));
  if (!d_in || !d_out) return GV_ERR_INVALID;
  GV_TRY(n->net.forward(d_in, batch));
  GV_CUDA(cudaMemcpyAsync(d_out, n->net.out, sizeof(float) * batch * n->net.H * n->net.W,
                          cudaMemcpyDeviceToDevice, n->net.stream));
  return n->net.check();
}

gv_status gv_unet_loss_grad(gv_unet* n, const float* d_in, const float* d_target, int32_t batch,
                            double* loss) {
  GV_TRY(check_batch(n, batch));
  if (!d_in || !d_target) return GV_ERR_INVALID;
  GV_TRY(n->net.forward(d_in, batch));
  GV_TRY(n->net.loss(d_target, batch, true, loss));
  GV_TRY(n->net.backward(batch));
  return n->net.check();
}

gv_status gv_unet_train_step(gv_unet* n, const float* d_in, const float* d_target, int32_t batch,
                             float lr, double* loss) {
  GV_TRY(check_batch(n, batch));
  if (!d_in || !d_target) return GV_ERR_INVALID;
  GV_TRY(n->net.forward(d_in, batch));
  GV_TRY(n->net.loss(d_target, batch, true, loss));
  GV_TRY(n->net.backward(batch));
  GV_TRY(n->net.adam(lr));
  return n->net.check();
}

gv_status gv_conv2d_forward(const float* x, const float* w, const float* bias, float* y,
                            int32_t B, int32_t Cin, int32_t Cout, int32_t H, int32_t W,
                            int32_t ks, int32_t relu, void* stream) {
  if (!x || !w || !bias || !y || B < 1 || Cin < 1 || Cout < 1 || H < 1 || W < 1 ||
      (ks != 1 && ks != 3)) {
    gv::set_error("invalid convolution arguments");
    return GV_ERR_INVALID;
  }
  uint32_t* err = nullptr;
  GV_CUDA(cudaMalloc(&err, sizeof(uint32_t)));
  GV_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), (cudaStream_t)stream));
  const gv::cnn::Ctx c = standalone_ctx(stream, err, nullptr, 0);
  gv_status s = gv::cnn::conv_forward(c, gv::cnn::View{(float*)x, Cin, 0}, w, bias,
                                      gv::cnn::View{y, Cout, 0}, B, Cin, Cout, H, W, ks, relu);
  uint32_t e = 0;
  cudaMemcpyAsync(&e, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  cudaStreamSynchronize((cudaStream_t)stream);
  cudaFree(err);
  if (s == GV_OK && e) {
    gv::set_error("convolution gave up on a bounded wait");
    s = GV_ERR_DEVICE;
  }
  return s;
}

gv_status gv_conv2d_backward(const float* x, const float* w, const float* dz, float* dx,
                             float* dw, float* db, int32_t B, int32_t Cin, int32_t Cout,
                             int32_t H, int32_t W, int32_t ks, void* stream) {
  if (!x || !w || !dz || !dx || !dw || !db || B < 1 || Cin < 1 || Cout < 1 || H < 1 || W < 1 ||
      (ks != 1 && ks != 3)) {
    gv::set_error("invalid convolution arguments");
    return GV_ERR_INVALID;
  }
  uint32_t* err = nullptr;
  float* part = nullptr;
  const size_t part_floats = (size_t)4 << 20;
  GV_CUDA(cudaMalloc(&err, sizeof(uint32_t)));
  GV_CUDA(cudaMalloc(&part, sizeof(float) * part_floats));
  GV_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), (cudaStream_t)stream));
  const gv::cnn::Ctx c = standalone_ctx(stream, err, part, part_floats);
  gv_status s = gv::cnn::conv_backward_data(c, gv::cnn::View{(float*)dz, Cout, 0}, w,
                                            gv::cnn::View{dx, Cin, 0}, B, Cin, Cout, H, W, ks, 0);
  if (s == GV_OK)
    s = gv::cnn::conv_backward_weight(c, gv::cnn::View{(float*)x, Cin, 0},
                                      gv::cnn::View{(float*)dz, Cout, 0}, dw, db, B, Cin, Cout, H,
                                      W, ks);
  uint32_t e = 0;
  cudaMemcpyAsync(&e, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  cudaStreamSynchronize((cudaStream_t)stream);
  cudaFree(err);
  cudaFree(part);
  if (s == GV_OK && e) {
    gv::set_error("convolution gave up on a bounded wait");
    s = GV_ERR_DEVICE;
  }
  return s;
}

}  // extern "C"
