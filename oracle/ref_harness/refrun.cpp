// Reference harness, host side -- TEST INFRASTRUCTURE ONLY.
//
// Loads the cubin built from the reference's own kernels (ref_kernels.cu ->
// oracle/_ref/ref_kernels.cubin) with the CUDA driver API and replays the
// reference's host drivers launch by launch, with the reference's launch
// shapes (-X 16 -Y 16 -V 256, as tests/*/test.sh run it), synchronisations
// and per-call reduction buffers:
//   MFS::setDevice          src/mfs.cu:530-943 (beam/noise/fg_scale set-up,
//                           hermitianSymmetry)
//   chi2()                  src/functions.cu:4323-4454
//   dchi2()                 src/functions.cu:4456-4558
//   deviceReduce<float>     src/functions.cu:604-741
//   prior value/gradient    src/functions.cu:4633-4964
// The only reference code that runs is the reference's kernels; the host
// sequencing is restated here (the reference's host code needs casacore).
// Used to pin the CPU oracle and to time the reference CUDA build.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <cxxabi.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

const double kPiD = 3.141592653589793238462643383279502884;
const double kRpDegD = kPiD / 180.0;
const float kLightSpeed = 2.99792458E8f;

std::string g_err;
CUmodule g_mod = nullptr;
std::map<std::string, CUfunction> g_fn;

int fail(const std::string& m) {
  g_err = m;
  return 1;
}

#define RR_CU(x)                                                        \
  do {                                                                  \
    CUresult _r = (x);                                                  \
    if (_r != CUDA_SUCCESS) {                                           \
      const char* s = nullptr;                                          \
      cuGetErrorString(_r, &s);                                         \
      return fail(std::string(#x) + ": " + (s ? s : "?"));              \
    }                                                                   \
  } while (0)
#define RR_RT(x)                                                        \
  do {                                                                  \
    cudaError_t _e = (x);                                               \
    if (_e != cudaSuccess) return fail(std::string(#x) + ": " + cudaGetErrorString(_e)); \
  } while (0)

std::string demangle(const char* n) {
  int st = 0;
  char* d = abi::__cxa_demangle(n, nullptr, nullptr, &st);
  std::string s = (st == 0 && d) ? d : n;
  free(d);
  return s;
}

// kernels of the reference by demangled signature
const char* kSigs[][2] = {
    {"herm", "hermitianSymmetry(double3*, float2*, float, int)"},
    {"tatt", "total_attenuation(float*, float, float, float, float, float, float, double, double, long, int)"},
    {"wimg", "weight_image(float*, float*, long)"},
    {"nimg", "noise_image(float*, float*, float, float, long)"},
    {"clip", "clip2IWNoise(float*, float*, long, long, float, float, float, float, float, int)"},
    {"inu", "calculateInu(float2*, float*, float, float, float, float, long, long)"},
    {"beam", "apply_beam2I(float, float, float, float2*, long, float, float, float, float, double, double, int)"},
    {"prot", "phase_rotate(float2*, long, long, double, double)"},
    {"vmod", "vis_mod(float2*, float2 const*, double3 const*, float*, double, double, long, long)"},
    {"resid", "residual(float2*, float2 const*, float2 const*, long)"},
    {"c2v", "chi2Vector(float*, float2 const*, float const*, long)"},
    {"dchi2", "DChi2(float*, float*, float2*, double3*, float*, long, long, float, float, float, float, float, float, double, double, float, float, float, float, int, bool)"},
    {"tot0", "DChi2_total_I_nu_0(float*, float*, float*, float*, float, float, float, float, long, long)"},
    {"tota", "DChi2_total_alpha(float*, float*, float*, float*, float, float, float, float, float, long, long)"},
    {"S", "SVector(float*, float const*, float*, long, long, float, float, float, int)"},
    {"DS", "DS(float*, float*, float const*, float, float, float, float, long, long, int)"},
    {"TSV", "TSVVector(float*, float*, float*, long, long, float, int)"},
    {"DTSV", "DTSV(float*, float*, float*, float, float, long, long, int)"},
    {"TV", "TVVector(float*, float*, float*, float, long, long, float, int)"},
    {"DTV", "DTV(float*, float*, float*, float, float, float, long, long, int)"},
    {"L1", "L1Vector(float*, float*, float*, long, long, float, float, int)"},
    {"DL1", "DL1NormK(float*, float*, float*, float, float, float, long, long, int)"},
    {"L", "LVector(float*, float*, float*, long, long, float, int)"},
    {"DL", "DL(float*, float*, float*, float, float, long, long, int)"},
    {"add", "AddToDPhi(float*, float*, long, long, int)"},
};

unsigned next_pow2(unsigned x) {
  --x;
  x |= x >> 1;
  x |= x >> 2;
  x |= x >> 4;
  x |= x >> 8;
  x |= x >> 16;
  return ++x;
}
int idiv_up(long a, int b) { return (int)((a % b != 0) ? (a / b + 1) : (a / b)); }
bool is_pow2(unsigned x) { return (x & (x - 1)) == 0; }

struct Chan {
  float freq;
  long nvis;
  double* uvw = nullptr;  // double3
  float* vo = nullptr;    // float2
  float* w = nullptr;
  float* vm = nullptr;
  float* vr = nullptr;
  int threadsUV = 256, blocksUV = 1;
};

struct Harness {
  long M = 0, N = 0;
  double DELTAX = 0, DELTAY = 0, deltau = 0, deltav = 0;
  float xobs = 0, yobs = 0, nu_0 = 0, D = 0, pbf = 0, pbcut = 0;
  int pb = 1;
  float eta = -1, minpix = 0, threshold = 0, noise_cut = 0, fg_scale = 1;
  int normalize = 0;
  std::vector<Chan> ch;
  long max_vis = 0;
  float* d_noise = nullptr;
  float* d_img = nullptr;     // 2 planes
  float2* d_inu = nullptr;
  float2* d_V = nullptr;
  float* d_chi2 = nullptr;
  float* d_dchi2 = nullptr;
  float* d_res = nullptr;     // result_dchi2, 2 planes
  float* d_S = nullptr;
  float* d_DS = nullptr;
  cufftHandle plan = 0;
  dim3 tNN{16, 16, 1}, bNN;
};

int launch(const char* key, dim3 grid, dim3 block, size_t smem, std::vector<void*> args) {
  auto it = g_fn.find(key);
  if (it == g_fn.end()) return fail(std::string("kernel not resolved: ") + key);
  RR_CU(cuLaunchKernel(it->second, grid.x, grid.y, grid.z, block.x, block.y, block.z,
                       (unsigned)smem, nullptr, args.data(), nullptr));
  return 0;
}

#define RR_TRY(x)              \
  do {                         \
    if ((x) != 0) return 1;    \
  } while (0)

// deviceReduce<float>, src/functions.cu:604-741, and the reduction branch of
// getNumBlocksAndThreads (src/functions.cu:307-342)
int device_reduce(float* in, long n, int input_threads, float* out) {
  const int maxThreads = input_threads;
  const int maxBlocks = idiv_up(n, maxThreads);
  int threads = (n < maxThreads * 2) ? (int)next_pow2((unsigned)((n + 1) / 2)) : maxThreads;
  int blocks = (int)((n + (threads * 2 - 1)) / (threads * 2));
  blocks = std::min(maxBlocks, blocks);
  const size_t smem = (threads <= 32) ? 2 * threads * sizeof(float) : threads * sizeof(float);
  float* d_out = nullptr;
  std::vector<float> h(blocks);
  RR_RT(cudaMalloc(&d_out, blocks * sizeof(float)));
  const bool p2 = is_pow2((unsigned)n);
  char name[64];
  std::snprintf(name, sizeof(name), "red_%d_%d", threads, p2 ? 1 : 0);
  unsigned nn = (unsigned)n;
  RR_TRY(launch(name, dim3(blocks), dim3(threads), smem, {&in, &d_out, &nn}));
  RR_RT(cudaDeviceSynchronize());
  RR_RT(cudaMemcpy(h.data(), d_out, blocks * sizeof(float), cudaMemcpyDeviceToHost));
  float sum = 0.0f;
  for (int i = 0; i < blocks; i++) sum += h[i];
  cudaFree(d_out);
  *out = sum;
  return 0;
}

}  // namespace

extern "C" {

const char* rr_last_error(void) { return g_err.c_str(); }

int rr_load(const char* cubin) {
  if (g_mod) return 0;
  RR_RT(cudaFree(0));  // primary context through the runtime
  RR_CU(cuModuleLoad(&g_mod, cubin));
  unsigned count = 0;
  RR_CU(cuModuleGetFunctionCount(&count, g_mod));
  std::vector<CUfunction> fs(count);
  RR_CU(cuModuleEnumerateFunctions(fs.data(), count, g_mod));
  std::map<std::string, CUfunction> by_sig;
  for (CUfunction f : fs) {
    const char* nm = nullptr;
    if (cuFuncGetName(&nm, f) != CUDA_SUCCESS || !nm) continue;
    by_sig[demangle(nm)] = f;
  }
  for (auto& s : kSigs) {
    auto it = by_sig.find(s[1]);
    if (it == by_sig.end()) return fail(std::string("reference kernel not found: ") + s[1]);
    g_fn[s[0]] = it->second;
  }
  for (int t = 1; t <= 512; t *= 2)
    for (int p2 = 0; p2 < 2; p2++) {
      char sig[96], key[32];
      std::snprintf(sig, sizeof(sig), "void reduceSumKernel<float, %d, %s>(float*, float*, unsigned int)",
                    t, p2 ? "true" : "false");
      std::snprintf(key, sizeof(key), "red_%d_%d", t, p2);
      auto it = by_sig.find(sig);
      if (it != by_sig.end()) g_fn[key] = it->second;
    }
  return 0;
}

// Set-up as MFS::setDevice: host noise/beam, uploads, hermitianSymmetry,
// total_attenuation / weight_image / noise_image, fg_scale, noise_cut.
int rr_create(int M, int N, double DELTAX, double DELTAY, float xobs, float yobs, float nu_0,
              float D, float pbf, float pbcut, int pb, float vis_noise, float noise_cut_factor,
              float eta, float initial_value, float threshold, int normalize, int nchan,
              const float* freq, const long* chan_off, const double* uvw, const float* vo,
              const float* w, void** out) {
  if (!g_mod) return fail("rr_load first");
  Harness* h = new Harness();
  h->M = M;
  h->N = N;
  h->DELTAX = DELTAX;
  h->DELTAY = DELTAY;
  h->deltau = 1.0 / (M * (kRpDegD * DELTAX));
  h->deltav = 1.0 / (N * (kRpDegD * DELTAY));
  h->xobs = xobs;
  h->yobs = yobs;
  h->nu_0 = nu_0;
  h->D = D;
  h->pbf = pbf;
  h->pbcut = pbcut;
  h->pb = pb;
  h->eta = eta;
  h->minpix = initial_value * -1.0f * eta;
  h->threshold = threshold;
  h->normalize = normalize;
  h->bNN = dim3(idiv_up(M, 16), idiv_up(N, 16), 1);
  // calculateNoiseAndBeam (host, src/functions.cu:1700-1814)
  float sum_w = 0.0f;
  double suu = 0, svv = 0, suv = 0;
  for (int c = 0; c < nchan; c++) {
    const long o = chan_off[c], n = chan_off[c + 1] - o;
    const float lam = kLightSpeed / freq[c];
    for (long k = 0; k < n; k++) {
      const double u = uvw[3 * (o + k)] / lam, v = uvw[3 * (o + k) + 1] / lam;
      suu += u * u * w[o + k];
      svv += v * v * w[o + k];
      suv += u * v * w[o + k];
    }
    if (n > 0) {
      float s = w[o], cc = 0.0f;
      for (long k = 1; k < n; k++) {
        float t = s + w[o + k];
        if (std::fabs(s) >= std::fabs(w[o + k])) cc += (s - t) + w[o + k];
        else cc += (w[o + k] - t) + s;
        s = t;
      }
      sum_w += s;
    }
  }
  suu /= sum_w;
  svv /= sum_w;
  suv /= sum_w;
  const float variance = 1.0f / sum_w;
  const double mm = suu - svv, pp = suu + svv, sq = std::sqrt(mm * mm + 4.0 * suv * suv);
  const double bmaj = (1.0 / std::sqrt(2.0) / kPiD / std::sqrt(pp - sq)) / kRpDegD;
  const double bmin = (1.0 / std::sqrt(2.0) / kPiD / std::sqrt(pp + sq)) / kRpDegD;
  if (vis_noise <= 0.0f) vis_noise = 0.5f * sqrtf(variance);
  // uploads and hermitianSymmetry (src/mfs.cu:555-845)
  h->ch.resize(nchan);
  for (int c = 0; c < nchan; c++) {
    Chan& C = h->ch[c];
    C.freq = freq[c];
    C.nvis = chan_off[c + 1] - chan_off[c];
    h->max_vis = std::max(h->max_vis, C.nvis);
    const long o = chan_off[c];
    RR_RT(cudaMalloc(&C.uvw, sizeof(double) * 3 * std::max(C.nvis, 1L)));
    RR_RT(cudaMalloc(&C.vo, sizeof(float) * 2 * std::max(C.nvis, 1L)));
    RR_RT(cudaMalloc(&C.w, sizeof(float) * std::max(C.nvis, 1L)));
    RR_RT(cudaMalloc(&C.vm, sizeof(float) * 2 * std::max(C.nvis, 1L)));
    RR_RT(cudaMalloc(&C.vr, sizeof(float) * 2 * std::max(C.nvis, 1L)));
    RR_RT(cudaMemcpy(C.uvw, uvw + 3 * o, sizeof(double) * 3 * C.nvis, cudaMemcpyHostToDevice));
    RR_RT(cudaMemcpy(C.vo, vo + 2 * o, sizeof(float) * 2 * C.nvis, cudaMemcpyHostToDevice));
    RR_RT(cudaMemcpy(C.w, w + o, sizeof(float) * C.nvis, cudaMemcpyHostToDevice));
    RR_RT(cudaMemset(C.vm, 0, sizeof(float) * 2 * C.nvis));
    RR_RT(cudaMemset(C.vr, 0, sizeof(float) * 2 * C.nvis));
    C.threadsUV = 256;
    C.blocksUV = std::max(1, idiv_up((long)next_pow2((unsigned)C.nvis), 256));
    if (C.nvis > 0) {
      int nv = (int)C.nvis;
      float f = C.freq;
      RR_TRY(launch("herm", dim3(C.blocksUV), dim3(C.threadsUV), 0, {&C.uvw, &C.vo, &f, &nv}));
      RR_RT(cudaDeviceSynchronize());
    }
  }
  const long MN = (long)M * N;
  RR_RT(cudaMalloc(&h->d_noise, sizeof(float) * MN));
  RR_RT(cudaMalloc(&h->d_img, sizeof(float) * 2 * MN));
  RR_RT(cudaMalloc(&h->d_inu, sizeof(float2) * MN));
  RR_RT(cudaMalloc(&h->d_V, sizeof(float2) * MN));
  RR_RT(cudaMalloc(&h->d_chi2, sizeof(float) * std::max(h->max_vis, 1L)));
  RR_RT(cudaMalloc(&h->d_dchi2, sizeof(float) * MN));
  RR_RT(cudaMalloc(&h->d_res, sizeof(float) * 2 * MN));
  RR_RT(cudaMalloc(&h->d_S, sizeof(float) * MN));
  RR_RT(cudaMalloc(&h->d_DS, sizeof(float) * MN));
  RR_RT(cudaMemset(h->d_inu, 0, sizeof(float2) * MN));
  RR_RT(cudaMemset(h->d_V, 0, sizeof(float2) * MN));
  // beam, weight and noise images (src/mfs.cu:849-916)
  float* d_atten = nullptr;
  float* d_wimg = nullptr;
  RR_RT(cudaMalloc(&d_atten, sizeof(float) * MN));
  RR_RT(cudaMalloc(&d_wimg, sizeof(float) * MN));
  RR_RT(cudaMemset(d_atten, 0, sizeof(float) * MN));
  RR_RT(cudaMemset(d_wimg, 0, sizeof(float) * MN));
  long NN = N;
  {
    float a = D, b = pbf, c = pbcut, f = nu_0, x = xobs, y = yobs;
    double dx = DELTAX, dy = DELTAY;
    int pbt = pb;
    RR_TRY(launch("tatt", h->bNN, h->tNN, 0, {&d_atten, &a, &b, &c, &f, &x, &y, &dx, &dy, &NN, &pbt}));
    RR_RT(cudaDeviceSynchronize());
    RR_TRY(launch("wimg", h->bNN, h->tNN, 0, {&d_wimg, &d_atten, &NN}));
    RR_RT(cudaDeviceSynchronize());
  }
  std::vector<float> hw(MN);
  RR_RT(cudaMemcpy(hw.data(), d_wimg, sizeof(float) * MN, cudaMemcpyDeviceToHost));
  float max_w = *std::max_element(hw.begin(), hw.end());
  const double bmaj_pix = bmaj / std::fabs(DELTAX), bmin_pix = bmin / std::fabs(DELTAX);
  float noise_jypix = (float)(vis_noise / (kPiD * bmaj_pix * bmin_pix / (4.0 * logf(2.0f))));
  RR_TRY(launch("nimg", h->bNN, h->tNN, 0, {&h->d_noise, &d_wimg, &max_w, &noise_jypix, &NN}));
  RR_RT(cudaDeviceSynchronize());
  RR_RT(cudaMemcpy(hw.data(), h->d_noise, sizeof(float) * MN, cudaMemcpyDeviceToHost));
  const float nmin = *std::min_element(hw.begin(), hw.end());
  h->fg_scale = nmin;
  h->noise_cut = noise_cut_factor * nmin;
  cudaFree(d_atten);
  cudaFree(d_wimg);
  if (cufftPlan2d(&h->plan, N, M, CUFFT_C2C) != CUFFT_SUCCESS) return fail("cufftPlan2d");
  *out = h;
  return 0;
}

int rr_info(void* hh, float* fg_scale, float* noise_cut, float* noise_img) {
  Harness* h = (Harness*)hh;
  *fg_scale = h->fg_scale;
  *noise_cut = h->noise_cut;
  if (noise_img)
    RR_RT(cudaMemcpy(noise_img, h->d_noise, sizeof(float) * h->M * h->N, cudaMemcpyDeviceToHost));
  return 0;
}

// chi2(), src/functions.cu:4323-4454, on the harness's device image
static int chi2_dev(Harness* h, int flag_opt, float* out) {
  long M = h->M, N = h->N;
  float nc = h->noise_cut, mp = h->minpix, a0 = 0.0f, eta = h->eta, thr = h->threshold;
  int sched = flag_opt;
  RR_TRY(launch("clip", h->bNN, h->tNN, 0, {&h->d_noise, &h->d_img, &N, &M, &nc, &mp, &a0, &eta, &thr, &sched}));
  RR_RT(cudaDeviceSynchronize());
  float reduced = 0.0f;
  for (auto& C : h->ch) {
    float f = C.freq, nu0 = h->nu_0;
    RR_TRY(launch("inu", h->bNN, h->tNN, 0, {&h->d_inu, &h->d_img, &f, &nu0, &mp, &eta, &N, &M}));
    RR_RT(cudaDeviceSynchronize());
    float a = h->D, b = h->pbf, c = h->pbcut, x = h->xobs, y = h->yobs, fg = h->fg_scale;
    double dx = h->DELTAX, dy = h->DELTAY;
    int pbt = h->pb;
    RR_TRY(launch("beam", h->bNN, h->tNN, 0, {&a, &b, &c, &h->d_inu, &N, &x, &y, &fg, &f, &dx, &dy, &pbt}));
    RR_RT(cudaDeviceSynchronize());
    if (cufftExecC2C(h->plan, (cufftComplex*)h->d_inu, (cufftComplex*)h->d_V, CUFFT_INVERSE) !=
        CUFFT_SUCCESS)
      return fail("cufftExecC2C");
    double xp = h->xobs, yp = h->yobs;
    RR_TRY(launch("prot", h->bNN, h->tNN, 0, {&h->d_V, &M, &N, &xp, &yp}));
    RR_RT(cudaDeviceSynchronize());
    if (C.nvis <= 0) continue;
    RR_RT(cudaMemset(h->d_chi2, 0, sizeof(float) * h->max_vis));
    long nv = C.nvis;
    double du = h->deltau, dv = h->deltav;
    RR_TRY(launch("vmod", dim3(C.blocksUV), dim3(C.threadsUV), 0, {&C.vm, &h->d_V, &C.uvw, &C.w, &du, &dv, &nv, &N}));
    RR_RT(cudaDeviceSynchronize());
    RR_TRY(launch("resid", dim3(C.blocksUV), dim3(C.threadsUV), 0, {&C.vr, &C.vm, &C.vo, &nv}));
    RR_RT(cudaDeviceSynchronize());
    RR_TRY(launch("c2v", dim3(C.blocksUV), dim3(C.threadsUV), 0, {&h->d_chi2, &C.vr, &C.w, &nv}));
    RR_RT(cudaDeviceSynchronize());
    float r = 0.0f;
    RR_TRY(device_reduce(h->d_chi2, C.nvis, C.threadsUV, &r));
    if (h->normalize) r /= C.nvis;
    reduced += r;
  }
  *out = 0.5f * reduced;
  return 0;
}

int rr_chi2(void* hh, float* img, int flag_opt, float* chi2) {
  Harness* h = (Harness*)hh;
  const long MN = h->M * h->N;
  RR_RT(cudaMemcpy(h->d_img, img, sizeof(float) * 2 * MN, cudaMemcpyHostToDevice));
  RR_TRY(chi2_dev(h, flag_opt, chi2));
  RR_RT(cudaMemcpy(img, h->d_img, sizeof(float) * 2 * MN, cudaMemcpyDeviceToHost));
  return 0;
}

// dchi2(), src/functions.cu:4456-4558 (result memset as Chi2::restartDGi)
static int dchi2_dev(Harness* h, int flag_opt) {
  long M = h->M, N = h->N;
  RR_RT(cudaMemset(h->d_res, 0, sizeof(float) * 2 * M * N));
  for (auto& C : h->ch) {
    if (C.nvis <= 0) continue;
    RR_RT(cudaMemset(h->d_dchi2, 0, sizeof(float) * M * N));
    long nv = C.nvis;
    float fg = h->fg_scale, nc = h->noise_cut, x = h->xobs, y = h->yobs;
    double dx = h->DELTAX, dy = h->DELTAY;
    float a = h->D, b = h->pbf, c = h->pbcut, f = C.freq;
    int pbt = h->pb;
    bool norm = h->normalize != 0;
    RR_TRY(launch("dchi2", h->bNN, h->tNN, 0,
                  {&h->d_noise, &h->d_dchi2, &C.vr, &C.uvw, &C.w, &N, &nv, &fg, &nc, &x, &y, &x, &y,
                   &dx, &dy, &a, &b, &c, &f, &pbt, &norm}));
    RR_RT(cudaDeviceSynchronize());
    float nu0 = h->nu_0, thr = h->threshold;
    if (flag_opt % 2 == 0) {
      RR_TRY(launch("tot0", h->bNN, h->tNN, 0,
                    {&h->d_noise, &h->d_res, &h->d_dchi2, &h->d_img, &f, &nu0, &nc, &thr, &N, &M}));
    } else {
      RR_TRY(launch("tota", h->bNN, h->tNN, 0,
                    {&h->d_noise, &h->d_res, &h->d_dchi2, &h->d_img, &f, &nu0, &nc, &fg, &thr, &N, &M}));
    }
    RR_RT(cudaDeviceSynchronize());
  }
  return 0;
}

int rr_dchi2(void* hh, const float* img, int flag_opt, float* out) {
  Harness* h = (Harness*)hh;
  const long MN = h->M * h->N;
  RR_RT(cudaMemcpy(h->d_img, img, sizeof(float) * 2 * MN, cudaMemcpyHostToDevice));
  RR_TRY(dchi2_dev(h, flag_opt));
  RR_RT(cudaMemcpy(out, h->d_res, sizeof(float) * 2 * MN, cudaMemcpyDeviceToHost));
  return 0;
}

// dchi2() restricted to image rows [i0, i0 + rows): the reference's DChi2
// and DChi2_total_* kernels launched over the band only (pointers offset to
// row i0, the DChi2 centres shifted by i0 rows; i0 and rows multiples of the
// 16-row launch tile).  A full-size gradient of a large image takes the
// reference's kernel tens of minutes; a band gives its values at those rows.
// out: 2 planes x rows x N floats.
int rr_dchi2_band(void* hh, const float* img, int flag_opt, int i0, int rows, float* out) {
  Harness* h = (Harness*)hh;
  long M = h->M, N = h->N;
  const long MN = M * N;
  if (i0 < 0 || rows <= 0 || i0 % 16 || rows % 16 || i0 + rows > N)
    return fail("rr_dchi2_band: i0 and rows must be multiples of 16 inside the image");
  RR_RT(cudaMemcpy(h->d_img, img, sizeof(float) * 2 * MN, cudaMemcpyHostToDevice));
  RR_RT(cudaMemset(h->d_res, 0, sizeof(float) * 2 * MN));
  const long off = (long)i0 * N;
  for (auto& C : h->ch) {
    if (C.nvis <= 0) continue;
    RR_RT(cudaMemset(h->d_dchi2, 0, sizeof(float) * MN));
    long nv = C.nvis;
    float fg = h->fg_scale, nc = h->noise_cut, x = h->xobs, y = h->yobs - (float)i0;
    double dx = h->DELTAX, dy = h->DELTAY;
    float a = h->D, b = h->pbf, c = h->pbcut, f = C.freq;
    int pbt = h->pb;
    bool norm = h->normalize != 0;
    float* noise = h->d_noise + off;
    float* dch = h->d_dchi2 + off;
    float* res = h->d_res + off;
    float* im = h->d_img + off;
    const dim3 grid(h->bNN.x, rows / 16);
    RR_TRY(launch("dchi2", grid, h->tNN, 0,
                  {&noise, &dch, &C.vr, &C.uvw, &C.w, &N, &nv, &fg, &nc, &x, &y, &x, &y, &dx,
                   &dy, &a, &b, &c, &f, &pbt, &norm}));
    RR_RT(cudaDeviceSynchronize());
    float nu0 = h->nu_0, thr = h->threshold;
    // the total kernels index plane 1 at M*N past their image pointers
    if (flag_opt % 2 == 0) {
      RR_TRY(launch("tot0", grid, h->tNN, 0,
                    {&noise, &res, &dch, &im, &f, &nu0, &nc, &thr, &N, &M}));
    } else {
      RR_TRY(launch("tota", grid, h->tNN, 0,
                    {&noise, &res, &dch, &im, &f, &nu0, &nc, &fg, &thr, &N, &M}));
    }
    RR_RT(cudaDeviceSynchronize());
  }
  for (int p = 0; p < 2; p++)
    RR_RT(cudaMemcpy(out + (long)p * rows * N, h->d_res + p * MN + off, sizeof(float) * rows * N,
                     cudaMemcpyDeviceToHost));
  return 0;
}

// Weighted residuals w*Vr of the last chi2, channel-major (2*V floats)
int rr_residuals(void* hh, float* out) {
  Harness* h = (Harness*)hh;
  long o = 0;
  for (auto& C : h->ch) {
    std::vector<float> vr(2 * C.nvis), w(C.nvis);
    RR_RT(cudaMemcpy(vr.data(), C.vr, sizeof(float) * 2 * C.nvis, cudaMemcpyDeviceToHost));
    RR_RT(cudaMemcpy(w.data(), C.w, sizeof(float) * C.nvis, cudaMemcpyDeviceToHost));
    for (long k = 0; k < C.nvis; k++) {
      out[2 * (o + k)] = w[k] * vr[2 * k];
      out[2 * (o + k) + 1] = w[k] * vr[2 * k + 1];
    }
    o += C.nvis;
  }
  return 0;
}

// One prior: value (kernel + deviceReduce, before lambda) and lambda*gradient
// (kind: 1 entropy, 2 TSV, 3 TV, 4 L1, 5 Laplacian; index = image plane)
int rr_prior(void* hh, int kind, float lambda, float G, float eta, float eps, int index,
             const float* img, float* value, float* grad) {
  Harness* h = (Harness*)hh;
  long M = h->M, N = h->N;
  const long MN = M * N;
  RR_RT(cudaMemcpy(h->d_img, img, sizeof(float) * 2 * MN, cudaMemcpyHostToDevice));
  float nc = h->noise_cut;
  int idx = index;
  const char* vk = nullptr;
  const char* gk = nullptr;
  switch (kind) {
    case 1:
      RR_TRY(launch("S", h->bNN, h->tNN, 0, {&h->d_S, &h->d_noise, &h->d_img, &N, &M, &nc, &G, &eta, &idx}));
      RR_TRY(launch("DS", h->bNN, h->tNN, 0, {&h->d_DS, &h->d_img, &h->d_noise, &nc, &lambda, &G, &eta, &N, &M, &idx}));
      break;
    case 2:
      RR_TRY(launch("TSV", h->bNN, h->tNN, 0, {&h->d_S, &h->d_noise, &h->d_img, &N, &M, &nc, &idx}));
      RR_TRY(launch("DTSV", h->bNN, h->tNN, 0, {&h->d_DS, &h->d_img, &h->d_noise, &nc, &lambda, &N, &M, &idx}));
      break;
    case 3:
      RR_TRY(launch("TV", h->bNN, h->tNN, 0, {&h->d_S, &h->d_noise, &h->d_img, &eps, &N, &M, &nc, &idx}));
      RR_TRY(launch("DTV", h->bNN, h->tNN, 0, {&h->d_DS, &h->d_img, &h->d_noise, &eps, &nc, &lambda, &N, &M, &idx}));
      break;
    case 4:
      RR_TRY(launch("L1", h->bNN, h->tNN, 0, {&h->d_S, &h->d_noise, &h->d_img, &N, &M, &eps, &nc, &idx}));
      RR_TRY(launch("DL1", h->bNN, h->tNN, 0, {&h->d_DS, &h->d_img, &h->d_noise, &eps, &nc, &lambda, &N, &M, &idx}));
      break;
    case 5:
      RR_TRY(launch("L", h->bNN, h->tNN, 0, {&h->d_S, &h->d_noise, &h->d_img, &N, &M, &nc, &idx}));
      RR_TRY(launch("DL", h->bNN, h->tNN, 0, {&h->d_DS, &h->d_img, &h->d_noise, &nc, &lambda, &N, &M, &idx}));
      break;
    default:
      return fail("unknown prior kind");
  }
  (void)vk;
  (void)gk;
  RR_RT(cudaDeviceSynchronize());
  RR_TRY(device_reduce(h->d_S, MN, 256, value));
  RR_RT(cudaMemcpy(grad, h->d_DS, sizeof(float) * MN, cudaMemcpyDeviceToHost));
  return 0;
}

// Device time (ms) of the reference's chi2() sequence and of its dchi2()
// over a band of `band_rows` image rows centred on the image (the DChi2
// kernel is shifted onto the band by offsetting its pointers and centres),
// scaled by the caller.  img: 2*M*N host image.
int rr_time(void* hh, const float* img, int reps, int band_rows, double* ms_chi2,
            double* ms_dchi2_band) {
  Harness* h = (Harness*)hh;
  long M = h->M, N = h->N;
  const long MN = M * N;
  RR_RT(cudaMemcpy(h->d_img, img, sizeof(float) * 2 * MN, cudaMemcpyHostToDevice));
  cudaEvent_t e0, e1;
  RR_RT(cudaEventCreate(&e0));
  RR_RT(cudaEventCreate(&e1));
  float r = 0.0f, t = 0.0f;
  RR_TRY(chi2_dev(h, 0, &r));  // warm-up
  RR_RT(cudaEventRecord(e0));
  for (int i = 0; i < reps; i++) RR_TRY(chi2_dev(h, 0, &r));
  RR_RT(cudaEventRecord(e1));
  RR_RT(cudaEventSynchronize(e1));
  RR_RT(cudaEventElapsedTime(&t, e0, e1));
  *ms_chi2 = t / reps;
  // DChi2 over the centre band
  const int rows = std::max(16, std::min((int)N, band_rows) / 16 * 16);
  const long i0 = (N - rows) / 2 / 16 * 16;
  double total = 0.0;
  for (int rep = 0; rep < reps; rep++) {
    RR_RT(cudaEventRecord(e0));
    for (auto& C : h->ch) {
      if (C.nvis <= 0) continue;
      long nv = C.nvis;
      float fg = h->fg_scale, nc = h->noise_cut, x = h->xobs, y = h->yobs - (float)i0;
      double dx = h->DELTAX, dy = h->DELTAY;
      float a = h->D, b = h->pbf, c = h->pbcut, f = C.freq;
      int pbt = h->pb;
      bool norm = h->normalize != 0;
      float* noise = h->d_noise + i0 * N;
      float* dch = h->d_dchi2 + i0 * N;
      RR_RT(cudaMemset(h->d_dchi2, 0, sizeof(float) * MN));
      RR_TRY(launch("dchi2", dim3(h->bNN.x, rows / 16), h->tNN, 0,
                    {&noise, &dch, &C.vr, &C.uvw, &C.w, &N, &nv, &fg, &nc, &x, &y, &x, &y, &dx,
                     &dy, &a, &b, &c, &f, &pbt, &norm}));
      RR_RT(cudaDeviceSynchronize());
    }
    RR_RT(cudaEventRecord(e1));
    RR_RT(cudaEventSynchronize(e1));
    RR_RT(cudaEventElapsedTime(&t, e0, e1));
    total += t;
  }
  *ms_dchi2_band = total / reps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return 0;
}

void rr_destroy(void* hh) {
  Harness* h = (Harness*)hh;
  if (!h) return;
  for (auto& C : h->ch) {
    cudaFree(C.uvw);
    cudaFree(C.vo);
    cudaFree(C.w);
    cudaFree(C.vm);
    cudaFree(C.vr);
  }
  cudaFree(h->d_noise);
  cudaFree(h->d_img);
  cudaFree(h->d_inu);
  cudaFree(h->d_V);
  cudaFree(h->d_chi2);
  cudaFree(h->d_dchi2);
  cudaFree(h->d_res);
  cudaFree(h->d_S);
  cudaFree(h->d_DS);
  if (h->plan) cufftDestroy(h->plan);
  delete h;
}

}  // extern "C"
