// Convolutional gridding of the visibilities (the reference's `-g` path):
// do_gridding (src/functions.cu:1339-1653) on the GPU, and the convolution
// kernel / gridding-correction tables of the CKernel family
// (include/classes/ckernel.cuh; src/pillBox2D.cu, src/gaussian2D.cu,
// src/sinc2D.cu, src/gaussianSinc2D.cu, src/pswf_12D.cu) on the host.
//
// The reference adds every (visibility, kernel tap) product into the grid
// in FP32 under OpenMP atomics and a critical section, so its sums depend on
// the thread schedule; with one thread each cell is a sequential FP32 sum in
// visibility order (the original visibilities, then their Hermitian copies).
// Here the (cell, slot) pairs of a slab of visibilities, slot = visibility
// x taps + tap, are radix sorted by cell with a stable (LSD) sort, so equal
// cells keep visibility order; one warp per occupied cell walks its run, the
// lanes forming 32 entries' products in parallel and one lane adding them in
// order, continuing the cell's running sums from the previous slab.  That
// reproduces the one-thread result bit for bit, with every product rounded
// as the reference's host code rounds it (no contraction into FMAs).
//
// The tables are host arithmetic in FP32 with the C library's sqrtf, expf,
// powf and sinf, as the reference computes them on the host.
#include <algorithm>
#include <cmath>
#include <vector>

#include "gv_internal.cuh"

namespace gv {
namespace {

// ---------------------------------------------------------------- tables
// distance(), src/MSFITSIO.cu:46-51
float dist2(float x, float y, float x0, float y0) {
  const float dx = x - x0, dy = y - y0;
  const float sx = dx * dx, sy = dy * dy;
  return sqrtf(sx + sy);
}

// pillBox1D / pillBox2D, src/pillBox2D.cu:3-16
float pill1(float amp, float x, float limit) { return std::fabs(x) < limit ? amp : 0.0f; }

// gaussian2D, src/gaussian2D.cu:17-37
float gauss2(float amp, float x, float y, float x0, float y0, float sx, float sy, float w,
             float alpha) {
  const float rx = dist2(x, 0.0f, x0, 0.0f);
  const float ry = dist2(0.0f, y, 0.0f, y0);
  const float lx = w * sx, ly = w * sy;
  if (rx < lx && ry < ly) {
    const float vx = powf(rx / lx, alpha), vy = powf(ry / ly, alpha);
    return amp * expf(-1.0f * (vx + vy));
  }
  return 0.0f;
}

// sincf / sinc1D / sinc2D, src/sinc2D.cu:3-35
float sinc0(float x) {
  if (x == 0.0f) return 1.0f;
  const float px = kPiF * x;
  return sinf(px) / px;
}
float sinc1(float amp, float x, float x0, float sigma, float w) {
  const float r = dist2(x, 0.0f, x0, 0.0f);
  const float lim = w * sigma;
  return r < lim ? amp * sinc0(r / lim) : 0.0f;
}
// parameters in the order sinc2D declares them: (amp, x, x0, y, y0, ...)
float sinc2(float amp, float x, float x0, float y, float y0, float sx, float sy, float w) {
  const float a = sinc1(1.0f, x, x0, sx, w);
  const float b = sinc1(1.0f, y, y0, sy, w);
  return amp * a * b;
}

// pswf_11D_func, src/pswf_12D.cu:3-46: the rational approximation of the
// prolate spheroidal function for support 6, alpha 1 (F. R. Schwab, 1984,
// "Optimal gridding of visibility data in radio interferometry"), with the
// published coefficients for |nu| < 0.75 and 0.75 <= |nu| <= 1
float pswf_rational(float nu) {
  static const float P[2][5] = {
      {8.203343e-2f, -3.644705e-1f, 6.278660e-1f, -5.335581e-1f, 2.312756e-1f},
      {4.028559e-3f, -3.697768e-2f, 1.021332e-1f, -1.201436e-1f, 6.412774e-2f}};
  static const float Q[2][3] = {{1.0f, 8.212018e-1f, 2.078043e-1f},
                                {1.0f, 9.599102e-1f, 2.918724e-1f}};
  const float a = fabsf(nu);
  if (a > 1.0f) return 0.0f;
  const int part = (a >= 0.0f && a < 0.75) ? 0 : 1;
  const float end = part == 0 ? 0.75f : 1.0f;
  const float d = a * a - end * end;
  float top = P[part][0], bottom = Q[part][0];
  for (int i = 1; i < 5; i++) top += P[part][i] * powf(d, (float)i);
  for (int i = 1; i < 3; i++) bottom += Q[part][i] * powf(d, (float)i);
  return bottom > 0.0f ? top / bottom : 0.0f;
}
// pswf_11D / pswf_12D, src/pswf_12D.cu:48-75
float pswf1(float amp, float x, float x0, float sigma, float w) {
  const float r = dist2(x, 0.0f, x0, 0.0f);
  const float nu = r / (w * sigma);
  if (nu == 0.0f) return 1.0f;
  const float f = pswf_rational(nu);
  const float nu2 = nu * nu;
  return amp * (1.0f - nu2) * f;
}
float pswf2(float amp, float x, float y, float x0, float y0, float sx, float sy, float w) {
  const float a = pswf1(1.0f, x, x0, sx, w);
  const float b = pswf1(1.0f, y, y0, sy, w);
  return amp * a * b;
}

// the value of kernel `k` at table position (i, j) with cell sizes sx, sy
// (buildKernel of each class); x0 = y0 = 0
float kernel_value(const gv_ckernel_desc& k, int i, int j, int sup_x, int sup_y, float sx,
                   float sy) {
  const float y = (float)(i - sup_y) * sy;
  const float x = (float)(j - sup_x) * sx;
  switch (k.kind) {
    case GV_CKERNEL_PILLBOX: {
      const float lx = ((float)k.m / 2.0f) * sx, ly = ((float)k.n / 2.0f) * sy;
      return pill1(k.amp, x, lx) * pill1(k.amp, y, ly);
    }
    case GV_CKERNEL_GAUSSIAN:
      return gauss2(k.amp, x, y, 0.0f, 0.0f, sx, sy, k.w, k.alpha);
    case GV_CKERNEL_SINC:
      // Sinc2D::buildKernel passes (x, y, x0, y0) into sinc2D's
      // (x, x0, y, y0) slots (src/sinc2D.cu:160-163); kept
      return sinc2(k.amp, x, y, 0.0f, 0.0f, sx, sy, k.w);
    case GV_CKERNEL_GAUSSIAN_SINC: {
      // gaussianSinc2D, src/gaussianSinc2D.cu:14-27 (its sinc2D call uses
      // the declared order)
      const float g = gauss2(1.0f, x, y, 0.0f, 0.0f, sx, sy, k.w, k.alpha);
      const float s = sinc2(1.0f, x, 0.0f, y, 0.0f, sx, sy, k.w2);
      return k.amp * g * s;
    }
    default:
      return pswf2(k.amp, x, y, 0.0f, 0.0f, sx, sy, k.w);
  }
}

// the GCF of kernel `k` at (i, j) of the M x N table (buildGCF after
// initializeGCF: w = M, cell sizes |deltax|, |deltay| in radians)
float gcf_value(const gv_ckernel_desc& k, int i, int j, int sup, float w, float sx, float sy) {
  const float y = (float)(i - sup) * sy;
  const float x = (float)(j - sup) * sx;
  if (k.kind == GV_CKERNEL_PILLBOX) return 1.0f;  // PillBox2D::GCF
  if (k.kind == GV_CKERNEL_GAUSSIAN)              // Gaussian2D::GCF
    return gauss2(k.amp, kPiF * x, kPiF * y, kPiF * 0.0f, kPiF * 0.0f, sx, sy, 2.0f * w,
                  k.alpha);
  return 1.0f / pswf2(k.amp, x, y, 0.0f, 0.0f, sx, sy, w);  // PSWF_12D::GCF
}

// ---------------------------------------------------------------- device
constexpr int64_t kMaxKeys = int64_t(1) << 27;  // (cell, slot) pairs per sorted slab

int bits_for(uint64_t v) {  // bits to hold 0..v
  int b = 1;
  while (b < 64 && (v >> b) != 0) b++;
  return b;
}

struct GridGeom {
  int M, N, sx, sy, km, kn;
  double deltau, deltav, cj, ck;
  float lambda;
};

// cell of visibility z (z >= n: the Hermitian copy of z - n), as the
// reference computes it (src/functions.cu:1424-1462): float wavelength, FP64
// u / du + N/2 + 0.5 truncated
__global__ void k_grid_cells(GridGeom g, int64_t n, int64_t z0, int64_t nz,
                             const double* __restrict__ uvw, int2* __restrict__ base) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nz) return;
  const int64_t z = z0 + t;
  const bool herm = z >= n;
  const int64_t vi = herm ? z - n : z;
  double u = uvw[3 * vi], v = uvw[3 * vi + 1];
  if (herm) {
    u *= -1.0;
    v *= -1.0;
  }
  const double ul = __ddiv_rn(u, (double)g.lambda), vl = __ddiv_rn(v, (double)g.lambda);
  const double gx = __ddiv_rn(ul, g.deltau), gy = __ddiv_rn(vl, g.deltav);
  base[t] = make_int2((int)__dadd_rn(__dadd_rn(gx, g.cj), 0.5),
                      (int)__dadd_rn(__dadd_rn(gy, g.ck), 0.5));
}

// one (cell, slot) pair per slot = t * taps + tap, taps in the reference's
// loop order (src/functions.cu:1466-1474); taps outside the grid or the
// table get the all-ones cell
__global__ void k_grid_keys(GridGeom g, int64_t nk, const int2* __restrict__ base,
                            uint32_t* __restrict__ keys, uint32_t* __restrict__ slots) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= nk) return;
  const int tw = 2 * g.sx + 1;
  const int T = (2 * g.sy + 1) * tw;
  const int64_t t = s / T;
  const int tap = (int)(s - t * T);
  const int ki = tap / tw, kj = tap - ki * tw;
  const int2 b = base[t];
  const int sk = b.y + ki - g.sy, sj = b.x + kj - g.sx;
  const bool ok = sk >= 0 && sk < g.M && sj >= 0 && sj < g.N && ki < g.km && kj < g.kn;
  keys[s] = ok ? (uint32_t)(g.N * sk + sj) : 0xFFFFFFFFu;
  slots[s] = (uint32_t)s;
}

// one warp per run of a cell in the pairs sorted (stably) by cell
// (src/functions.cu:1476-1506): the lanes gather 32 entries at a time and
// form their rounded products (w k, w k^2, w Vo k) in parallel; lane 0 adds
// them to the cell's running sums in visibility order, continuing from the
// previous slab, so every sum is the reference's sequential FP32 sum
constexpr int kRunWarps = 8;  // warps per block of k_grid_runs
__global__ void __launch_bounds__(kRunWarps * 32) k_grid_runs(
    GridGeom g, int64_t n, int64_t z0, const uint32_t* __restrict__ cells,
    const uint32_t* __restrict__ starts, const uint32_t* __restrict__ counts,
    const int* __restrict__ nruns, const uint32_t* __restrict__ sslots,
    const float* __restrict__ w, const float2* __restrict__ vo, const float* __restrict__ ktab,
    float* __restrict__ gw, float* __restrict__ gaux, float2* __restrict__ gvo) {
  __shared__ float4 prod[kRunWarps][32];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int tw = 2 * g.sx + 1;
  const int T = (2 * g.sy + 1) * tw;
  const int64_t MN = (int64_t)g.M * g.N;
  const int nr = *nruns;
  for (int r = blockIdx.x * kRunWarps + wib; r < nr; r += gridDim.x * kRunWarps) {
    const uint32_t cell = cells[r];
    if ((int64_t)cell >= MN) continue;  // the run of unused taps
    const uint32_t a = starts[r], e = a + counts[r];
    float sw = 0.0f, sa = 0.0f, sx = 0.0f, sy = 0.0f;
    if (lane == 0) {
      sw = gw[cell];
      sa = gaux[cell];
      const float2 v = gvo[cell];
      sx = v.x;
      sy = v.y;
    }
    for (uint32_t b0 = a; b0 < e; b0 += 32) {
      const uint32_t q = b0 + (uint32_t)lane;
      float4 pr = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (q < e) {
        const uint32_t s = sslots[q];
        const int64_t t = s / (uint32_t)T;
        const int tap = (int)(s - (uint32_t)t * (uint32_t)T);
        const int ki = tap / tw, kj = tap - ki * tw;
        const float c = ktab[ki * g.kn + kj];
        const int64_t z = z0 + t;
        const bool herm = z >= n;
        const int64_t vi = herm ? z - n : z;
        const float wv = w[vi];
        float2 V = vo[vi];
        if (herm) V.y *= -1.0f;
        pr = make_float4(__fmul_rn(wv, c), __fmul_rn(wv, __fmul_rn(c, c)),
                         __fmul_rn(__fmul_rn(wv, V.x), c), __fmul_rn(__fmul_rn(wv, V.y), c));
      }
      prod[wib][lane] = pr;
      __syncwarp();
      if (lane == 0) {
        const int m = (int)min((uint32_t)32, e - b0);
        for (int l = 0; l < m; l++) {
          const float4 p = prod[wib][l];
          sw = __fadd_rn(sw, p.x);
          sa = __fadd_rn(sa, p.y);
          sx = __fadd_rn(sx, p.z);
          sy = __fadd_rn(sy, p.w);
        }
      }
      __syncwarp();
    }
    if (lane == 0) {
      gw[cell] = sw;
      gaux[cell] = sa;
      gvo[cell] = make_float2(sx, sy);
    }
  }
}

// normalisation and effective weight (src/functions.cu:1514-1567)
__global__ void k_grid_finish(int64_t MN, float* __restrict__ gw, const float* __restrict__ gaux,
                              float2* __restrict__ gvo, int* __restrict__ flag) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= MN) return;
  const float ws = gw[c], as = gaux[c];
  float weff = 0.0f;
  float2 v = make_float2(0.0f, 0.0f);
  if (as != 0.0f && ws != 0.0f) {
    weff = __fdiv_rn(__fmul_rn(ws, ws), as);
    const float2 s = gvo[c];
    v = make_float2(__fdiv_rn(s.x, ws), __fdiv_rn(s.y, ws));
  }
  gw[c] = weff;
  gvo[c] = v;
  flag[c] = weff > 0.0f ? 1 : 0;
}

// the occupied cells in row-major order as visibilities
// (src/functions.cu:1569-1618)
__global__ void k_grid_compact(GridGeom g, int64_t MN, const float* __restrict__ gw,
                               const float2* __restrict__ gvo, const int* __restrict__ flag,
                               const int* __restrict__ pos, double* __restrict__ ouvw,
                               float2* __restrict__ ovo, float* __restrict__ ow) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= MN || !flag[c]) return;
  const int p = pos[c];
  const int gj = (int)(c % g.N), gk = (int)(c / g.N);
  const double ul = __dmul_rn((double)gj - g.cj, g.deltau);
  const double vl = __dmul_rn((double)gk - g.ck, g.deltav);
  ouvw[3 * (int64_t)p] = __dmul_rn(ul, (double)g.lambda);
  ouvw[3 * (int64_t)p + 1] = __dmul_rn(vl, (double)g.lambda);
  ouvw[3 * (int64_t)p + 2] = 0.0;
  ovo[p] = gvo[c];
  ow[p] = gw[c];
}

struct GridBuffers {
  double* uvw = nullptr;
  float* w = nullptr;
  float2* vo = nullptr;
  int2* base = nullptr;
  uint32_t *keys = nullptr, *skeys = nullptr, *slots = nullptr, *sslots = nullptr;
  uint32_t *rcell = nullptr, *rcount = nullptr, *rstart = nullptr;
  int* nruns = nullptr;
  float *gw = nullptr, *gaux = nullptr, *ktab = nullptr;
  float2* gvo = nullptr;
  int *flag = nullptr, *pos = nullptr;
  double* ouvw = nullptr;
  float2* ovo = nullptr;
  float* ow = nullptr;
  void* tmp = nullptr;
  ~GridBuffers() {
    cudaFree(uvw);
    cudaFree(w);
    cudaFree(vo);
    cudaFree(base);
    cudaFree(keys);
    cudaFree(skeys);
    cudaFree(slots);
    cudaFree(sslots);
    cudaFree(rcell);
    cudaFree(rcount);
    cudaFree(rstart);
    cudaFree(nruns);
    cudaFree(gw);
    cudaFree(gaux);
    cudaFree(ktab);
    cudaFree(gvo);
    cudaFree(flag);
    cudaFree(pos);
    cudaFree(ouvw);
    cudaFree(ovo);
    cudaFree(ow);
    cudaFree(tmp);
  }
};

}  // namespace
}  // namespace gv

extern "C" gv_status gv_ckernel_defaults(int32_t kind, int32_t m, int32_t n,
                                         gv_ckernel_desc* out) {
  using namespace gv;
  if (!out || kind < GV_CKERNEL_PILLBOX || kind > GV_CKERNEL_PSWF || m < 1 || n < 1) {
    set_error("invalid convolution kernel");
    return GV_ERR_INVALID;
  }
  gv_ckernel_desc k{};
  k.kind = kind;
  k.m = m;
  k.n = n;
  k.amp = 1.0f;
  k.alpha = 2.0f;
  k.w2 = 1.55f;
  k.w = kind == GV_CKERNEL_PSWF ? 6.0f : kind == GV_CKERNEL_GAUSSIAN_SINC ? 2.52f : 1.0f;
  *out = k;
  return GV_OK;
}

extern "C" gv_status gv_ckernel_build(const gv_ckernel_desc* k, int32_t M, int32_t N,
                                      double deltax_deg, double deltay_deg, float* kernel,
                                      int32_t* support_x, int32_t* support_y, float* gcf,
                                      int32_t* has_gcf) {
  using namespace gv;
  if (!k || k->kind < GV_CKERNEL_PILLBOX || k->kind > GV_CKERNEL_PSWF || k->m < 1 ||
      k->n < 1 || M < 1 || N < 1 || deltax_deg == 0.0 || deltay_deg == 0.0) {
    set_error("invalid convolution kernel build");
    return GV_ERR_INVALID;
  }
  // src/mfs.cu:493-496 and :510-515; the kernel classes keep float sizes
  const double deltax = kRpDegD * deltax_deg, deltay = kRpDegD * deltay_deg;
  const double deltau = 1.0 / ((double)M * deltax), deltav = 1.0 / ((double)N * deltay);
  const int sup = (int)floorf((float)k->m / 2.0f);  // setSupports: both from m
  if (support_x) *support_x = sup;
  if (support_y) *support_y = sup;
  if (kernel) {
    const float su = (float)std::fabs(deltau), sv = (float)std::fabs(deltav);
    for (int i = 0; i < k->m; i++)
      for (int j = 0; j < k->n; j++)
        kernel[(int64_t)k->n * i + j] = kernel_value(*k, i, j, sup, sup, su, sv);
  }
  const int hg = (k->kind == GV_CKERNEL_SINC || k->kind == GV_CKERNEL_GAUSSIAN_SINC) ? 0 : 1;
  if (has_gcf) *has_gcf = hg;
  if (gcf && hg) {
    const float sx = (float)std::fabs(deltax), sy = (float)std::fabs(deltay);
    const int gsup = (int)floorf((float)M / 2.0f);
    const float w = (float)M;
    for (int i = 0; i < M; i++)
      for (int j = 0; j < N; j++) gcf[(int64_t)N * i + j] = gcf_value(*k, i, j, gsup, w, sx, sy);
  }
  return GV_OK;
}

extern "C" gv_status gv_grid_visibilities(const gv_grid_kernel* kernel, int32_t M, int32_t N,
                                          double deltax_deg, double deltay_deg,
                                          int32_t nchannels, const gv_channel_desc* in,
                                          gv_channel_desc* out, void* stream) {
  using namespace gv;
  if (!kernel || !kernel->values || kernel->m < 1 || kernel->n < 1 || kernel->support_x < 0 ||
      kernel->support_y < 0 || kernel->support_x > 64 || kernel->support_y > 64 || M < 1 ||
      N < 1 || (int64_t)M * N >= (int64_t(1) << 31) || nchannels < 1 || !in || !out ||
      deltax_deg == 0.0 || deltay_deg == 0.0) {
    set_error("invalid gridding arguments");
    return GV_ERR_INVALID;
  }
  for (int c = 0; c < nchannels; c++)
    if (in[c].nvis < 0 || (in[c].nvis > 0 && (!in[c].uvw || !in[c].vo || !in[c].weight)) ||
        !out[c].uvw || !out[c].vo || !out[c].weight) {
      set_error("invalid channel in gridding");
      return GV_ERR_INVALID;
    }
  const double deltax = kRpDegD * deltax_deg, deltay = kRpDegD * deltay_deg;
  GridGeom g{};
  g.M = M;
  g.N = N;
  g.sx = kernel->support_x;
  g.sy = kernel->support_y;
  g.km = kernel->m;
  g.kn = kernel->n;
  g.deltau = 1.0 / ((double)M * deltax);
  g.deltav = 1.0 / ((double)N * deltay);
  g.cj = std::floor(N / 2.0);
  g.ck = std::floor(M / 2.0);
  const int64_t T = (int64_t)(2 * g.sy + 1) * (2 * g.sx + 1);
  const int64_t MN = (int64_t)M * N;
  int64_t vmax = 1;
  for (int c = 0; c < nchannels; c++) vmax = std::max<int64_t>(vmax, in[c].nvis);
  const int64_t zslab = std::max<int64_t>(1, std::min<int64_t>(2 * vmax, kMaxKeys / T));
  const int64_t kcap = zslab * T;
  const int cellbits = bits_for((uint64_t)MN);  // the all-ones cell is no cell
  cudaStream_t st = (cudaStream_t)stream;
  GridBuffers b;
  GV_CUDA(cudaMalloc(&b.uvw, sizeof(double) * 3 * vmax));
  GV_CUDA(cudaMalloc(&b.w, sizeof(float) * vmax));
  GV_CUDA(cudaMalloc(&b.vo, sizeof(float2) * vmax));
  GV_CUDA(cudaMalloc(&b.base, sizeof(int2) * zslab));
  GV_CUDA(cudaMalloc(&b.keys, sizeof(uint32_t) * kcap));
  GV_CUDA(cudaMalloc(&b.skeys, sizeof(uint32_t) * kcap));
  GV_CUDA(cudaMalloc(&b.slots, sizeof(uint32_t) * kcap));
  GV_CUDA(cudaMalloc(&b.sslots, sizeof(uint32_t) * kcap));
  // runs of equal cells in a slab: at most one per cell plus the unused taps'
  const int64_t rcap = std::min<int64_t>(kcap, MN + 1);
  GV_CUDA(cudaMalloc(&b.rcell, sizeof(uint32_t) * rcap));
  GV_CUDA(cudaMalloc(&b.rcount, sizeof(uint32_t) * rcap));
  GV_CUDA(cudaMalloc(&b.rstart, sizeof(uint32_t) * rcap));
  GV_CUDA(cudaMalloc(&b.nruns, sizeof(int)));
  GV_CUDA(cudaMalloc(&b.gw, sizeof(float) * MN));
  GV_CUDA(cudaMalloc(&b.gaux, sizeof(float) * MN));
  GV_CUDA(cudaMalloc(&b.gvo, sizeof(float2) * MN));
  GV_CUDA(cudaMalloc(&b.flag, sizeof(int) * MN));
  GV_CUDA(cudaMalloc(&b.pos, sizeof(int) * MN));
  GV_CUDA(cudaMalloc(&b.ouvw, sizeof(double) * 3 * MN));
  GV_CUDA(cudaMalloc(&b.ovo, sizeof(float2) * MN));
  GV_CUDA(cudaMalloc(&b.ow, sizeof(float) * MN));
  GV_CUDA(cudaMalloc(&b.ktab, sizeof(float) * kernel->m * kernel->n));
  GV_CUDA(cudaMemcpyAsync(b.ktab, kernel->values, sizeof(float) * kernel->m * kernel->n,
                          cudaMemcpyHostToDevice, st));
  const size_t tmp_bytes =
      std::max(std::max(radix_sort_scratch<uint32_t, uint32_t>(kcap), scan_scratch(MN)),
               rle_scratch(kcap));
  GV_CUDA(cudaMalloc(&b.tmp, tmp_bytes));
  for (int c = 0; c < nchannels; c++) {
    const int64_t n = in[c].nvis;
    g.lambda = kLightSpeed / in[c].freq_hz;  // freq_to_wavelength
    GV_CUDA(cudaMemsetAsync(b.gw, 0, sizeof(float) * MN, st));
    GV_CUDA(cudaMemsetAsync(b.gaux, 0, sizeof(float) * MN, st));
    GV_CUDA(cudaMemsetAsync(b.gvo, 0, sizeof(float2) * MN, st));
    if (n > 0) {
      GV_CUDA(cudaMemcpyAsync(b.uvw, in[c].uvw, sizeof(double) * 3 * n, cudaMemcpyHostToDevice,
                              st));
      GV_CUDA(cudaMemcpyAsync(b.w, in[c].weight, sizeof(float) * n, cudaMemcpyHostToDevice, st));
      GV_CUDA(cudaMemcpyAsync(b.vo, in[c].vo, sizeof(float2) * n, cudaMemcpyHostToDevice, st));
    }
    for (int64_t z0 = 0; z0 < 2 * n; z0 += zslab) {
      const int64_t nz = std::min<int64_t>(zslab, 2 * n - z0);
      const int64_t nk = nz * T;
      k_grid_cells<<<(unsigned)((nz + 255) / 256), 256, 0, st>>>(g, n, z0, nz, b.uvw, b.base);
      GV_LAUNCH("k_grid_cells");
      k_grid_keys<<<(unsigned)((nk + 255) / 256), 256, 0, st>>>(g, nk, b.base, b.keys, b.slots);
      GV_LAUNCH("k_grid_keys");
      GV_TRY((radix_sort_pairs<uint32_t, uint32_t>(b.tmp, tmp_bytes, b.keys, b.skeys, b.slots,
                                                    b.sslots, nk, 0, cellbits, st)));
      // runs of equal cells: cell, first position and length of each
      GV_TRY(run_length_encode(b.tmp, tmp_bytes, b.skeys, nk, b.rcell, b.rstart, b.rcount, rcap,
                               b.nruns, st));
      const int64_t nr_cap = std::min<int64_t>(nk, rcap);
      const unsigned rb = (unsigned)std::min<int64_t>((nr_cap + kRunWarps - 1) / kRunWarps,
                                                      (int64_t)65535 * 16);
      k_grid_runs<<<rb, kRunWarps * 32, 0, st>>>(g, n, z0, b.rcell, b.rstart, b.rcount, b.nruns,
                                                 b.sslots, b.w, b.vo, b.ktab, b.gw, b.gaux,
                                                 b.gvo);
      GV_LAUNCH("k_grid_runs");
    }
    const unsigned gb = (unsigned)((MN + 255) / 256);
    k_grid_finish<<<gb, 256, 0, st>>>(MN, b.gw, b.gaux, b.gvo, b.flag);
    GV_LAUNCH("k_grid_finish");
    GV_TRY(exclusive_scan<int>(b.tmp, tmp_bytes, b.flag, b.pos, MN, st));
    k_grid_compact<<<gb, 256, 0, st>>>(g, MN, b.gw, b.gvo, b.flag, b.pos, b.ouvw, b.ovo, b.ow);
    GV_LAUNCH("k_grid_compact");
    int last[2] = {0, 0};
    GV_CUDA(cudaMemcpyAsync(&last[0], b.pos + (MN - 1), sizeof(int), cudaMemcpyDeviceToHost, st));
    GV_CUDA(cudaMemcpyAsync(&last[1], b.flag + (MN - 1), sizeof(int), cudaMemcpyDeviceToHost, st));
    GV_CUDA(cudaStreamSynchronize(st));
    const int64_t cnt = (int64_t)last[0] + last[1];
    out[c].freq_hz = in[c].freq_hz;
    out[c].nvis = cnt;
    if (cnt > 0) {
      GV_CUDA(cudaMemcpyAsync(const_cast<double*>(out[c].uvw), b.ouvw, sizeof(double) * 3 * cnt,
                              cudaMemcpyDeviceToHost, st));
      GV_CUDA(cudaMemcpyAsync(const_cast<float*>(out[c].vo), b.ovo, sizeof(float2) * cnt,
                              cudaMemcpyDeviceToHost, st));
      GV_CUDA(cudaMemcpyAsync(const_cast<float*>(out[c].weight), b.ow, sizeof(float) * cnt,
                              cudaMemcpyDeviceToHost, st));
      GV_CUDA(cudaStreamSynchronize(st));
    }
  }
  return GV_OK;
}
