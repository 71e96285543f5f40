// gv_prior_value_static: the prior-value reduction for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc: code running inside another
// framework whose allocator owns all device memory, or a real-time loop in
// which an allocation (which may synchronise the device) is not allowed.
// This entry point therefore takes every input and output from the caller
// and keeps its only scratch -- one FP64 partial sum per image row -- in the
// file-scope array below, which every GPU that loads this library holds
// until the process exits (8192 rows x 8 bytes = 64 KiB).
//
// Set-up: the first call on a device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress and caches it for
// that device; make that first call before any stream capture.  Later calls
// outside a capture look the address up again (no allocation; it keeps the
// cache valid after a cudaDeviceReset re-creates the context), calls inside
// a capture use the cached address.  Every call shares the array and leaves
// the last call's partials in it; each call rewrites all the rows it uses,
// so nothing needs clearing, but calls that overlap on the GPU (different
// streams, or another host thread) race on it.
#include <mutex>

#include "gv_internal.cuh"

namespace gv {

namespace {

constexpr int kStaticMaxRows = 8192;

static __device__ __align__(256) double g_row_partials[kStaticMaxRows];

constexpr int kMaxDevices = 64;
double* g_partials_addr[kMaxDevices] = {};
std::mutex g_partials_mu;

// Device address of g_row_partials on the current device.  `capturing`:
// the launch stream is being captured, so only the cached address is used
// (a first look-up may load the module, which a capture does not allow).
gv_status partials_for_current_device(bool capturing, double** out) {
  int dev = -1;
  GV_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("gv_prior_value_static: device index beyond the supported 64 devices");
    return GV_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_partials_mu);
  if (!capturing || g_partials_addr[dev] == nullptr) {
    if (capturing) {
      set_error("gv_prior_value_static: the first call on a device must come before any "
                "stream capture (it looks up the static scratch's address)");
      return GV_ERR_INVALID;
    }
    void* p = nullptr;
    GV_CUDA(cudaGetSymbolAddress(&p, g_row_partials));
    g_partials_addr[dev] = static_cast<double*>(p);
  }
  *out = g_partials_addr[dev];
  return GV_OK;
}

struct RowPrior {
  int kind, n;
  float noise_cut, G, eta, eps;
};

// Prior value of pixel (i, j) inside the noise mask, as the reference's
// calculateS / calculateTSV / calculateTV / calculateL1norm / calculateL
// (src/functions.cu:3036, 3353, 3238, 2882, 3443).
__device__ __forceinline__ float row_prior_pixel(const RowPrior& rp, const float* __restrict__ I,
                                                 int i, int j) {
  const int n = rp.n;
  const float c = I[(int64_t)n * i + j];
  switch (rp.kind) {
    case GV_FI_ENTROPY:
      return c * logf((c / rp.G) + (rp.eta + 1.0f));
    case GV_FI_L1:
      return sqrtf(c * c + rp.eps);
    case GV_FI_TSV:
      if (i < n - 1 && j < n - 1) {
        const float dx = c - I[(int64_t)n * i + j + 1];
        const float dy = c - I[(int64_t)n * (i + 1) + j];
        return dx * dx + dy * dy;
      }
      return c;
    case GV_FI_TV:
      if (i < n - 1 && j < n - 1) {
        const float r = I[(int64_t)n * i + j + 1];
        const float d = I[(int64_t)n * (i + 1) + j];
        return sqrtf((r - c) * (r - c) + (d - c) * (d - c) + rp.eps);
      }
      return c;
    case GV_FI_LAPLACIAN:
      if (i > 0 && i < n - 1 && j > 0 && j < n - 1) {
        const float dxx = I[(int64_t)n * i + j - 1] - 2.0f * c + I[(int64_t)n * i + j + 1];
        const float dyy = I[(int64_t)n * (i - 1) + j] - 2.0f * c + I[(int64_t)n * (i + 1) + j];
        return 0.5f * (dxx + dyy) * (dxx + dyy);
      }
      return c;
  }
  return 0.0f;
}

// one block per image row: FP64 sum of the row's masked prior values
__global__ void __launch_bounds__(256) k_prior_rows_static(RowPrior rp,
                                                           const float* __restrict__ plane,
                                                           const float* __restrict__ noise,
                                                           double* __restrict__ partials) {
  const int i = blockIdx.x;
  double acc = 0.0;
  for (int j = threadIdx.x; j < rp.n; j += blockDim.x) {
    if (noise[(int64_t)rp.n * i + j] < rp.noise_cut) acc += (double)row_prior_pixel(rp, plane, i, j);
  }
  __shared__ double red[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    partials[i] = s;
  }
}

// Sum of the row partials in a fixed order: thread t adds rows
// [t*k, (t+1)*k) with Neumaier's compensation (Neumaier 1974), then the
// 256 compensated values are added pairwise in a fixed tree.  Deterministic
// and accurate to a few FP64 ulps of the largest partial for 8192 rows.
__global__ void __launch_bounds__(256) k_sum_rows_static(int n, const double* __restrict__ partials,
                                                         double* __restrict__ out) {
  __shared__ double red[256];
  const int per = (n + 255) / 256;
  const int lo = threadIdx.x * per, hi = min(n, lo + per);
  double s = 0.0, c = 0.0;
  for (int i = lo; i < hi; i++) {
    const double x = partials[i];
    const double t = s + x;
    c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
    s = t;
  }
  red[threadIdx.x] = s + c;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

}  // namespace

}  // namespace gv

extern "C" gv_status gv_prior_value_static(int32_t kind, const float* d_plane,
                                           const float* d_noise, float noise_cut, int32_t n,
                                           float prior_value, float eta, float epsilon,
                                           double* d_value, void* stream) {
  if (kind < GV_FI_ENTROPY || kind > GV_FI_LAPLACIAN) {
    gv::set_error("gv_prior_value_static: kind must be a prior (Entropy, TSV, TV, L1 or Laplacian)");
    return GV_ERR_INVALID;
  }
  if (!d_plane || !d_noise || !d_value) {
    gv::set_error("gv_prior_value_static: null plane, noise or output pointer");
    return GV_ERR_INVALID;
  }
  if (n <= 0 || n > gv::kStaticMaxRows) {
    gv::set_error("gv_prior_value_static: image size must be between 1 and 8192 rows "
                  "(the static scratch holds one partial per row)");
    return GV_ERR_UNSUPPORTED;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (st != nullptr) {
    // the stream must belong to the current device: the scratch address
    // and the launch are the current device's
    int dev = -1, sdev = -1;
    GV_CUDA(cudaGetDevice(&dev));
    GV_CUDA(cudaStreamGetDevice(st, &sdev));
    if (sdev != dev) {
      gv::set_error("gv_prior_value_static: the stream belongs to another device than the "
                    "current one");
      return GV_ERR_INVALID;
    }
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  GV_CUDA(cudaStreamIsCapturing(st, &cap));
  double* partials = nullptr;
  gv_status s = gv::partials_for_current_device(cap != cudaStreamCaptureStatusNone, &partials);
  if (s != GV_OK) return s;
  gv::RowPrior rp{kind, n, noise_cut, prior_value, eta, epsilon};
  gv::k_prior_rows_static<<<n, 256, 0, st>>>(rp, d_plane, d_noise, partials);
  GV_LAUNCH("k_prior_rows_static");
  gv::k_sum_rows_static<<<1, 256, 0, st>>>(n, partials, d_value);
  GV_LAUNCH("k_sum_rows_static");
  return GV_OK;
}
