// extern "C" entry points of include/gpuvmem_gb300.h.  Each validates its
// arguments, runs on the problem's stream and returns a status; nothing
// exits the process (the reference calls exit() on configuration errors,
// include/classes/fi.cuh:68-81, src/mfs.cu:117-140).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "gv_internal.cuh"

struct gv_problem {
  gv::Problem P;
};

namespace gv {
Problem& problem_of(gv_problem* p) { return p->P; }
}  // namespace gv

namespace gv {

static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void add_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void set_error(const std::string& msg) { g_last_error = msg; }

gv_status cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return GV_ERR_NOMEM;
  return GV_ERR_CUDA;
}

}  // namespace gv

using gv::Problem;

#define GV_CHECK_PROBLEM(p)                         \
  do {                                              \
    if (!(p)) {                                     \
      gv::set_error("null problem handle");         \
      return GV_ERR_INVALID;                        \
    }                                               \
  } while (0)

#define GV_SYNC(P)                                                   \
  do {                                                               \
    cudaError_t _e = cudaStreamSynchronize((P).stream);              \
    if (_e != cudaSuccess) return gv::cuda_fail(_e, "stream sync");   \
  } while (0)

extern "C" {

gv_status gv_problem_create(const gv_problem_desc* desc, gv_problem** out) {
  if (!desc || !out) {
    gv::set_error("null descriptor or output pointer");
    return GV_ERR_INVALID;
  }
  *out = nullptr;
  gv_problem* h = new (std::nothrow) gv_problem();
  if (!h) {
    gv::set_error("host allocation failed");
    return GV_ERR_NOMEM;
  }
  gv_status s = gv::setup_problem(h->P, *desc);
  if (s != GV_OK) {
    gv::free_problem(h->P);
    delete h;
    return s;
  }
  *out = h;
  return GV_OK;
}

gv_status gv_problem_destroy(gv_problem* p) {
  if (!p) return GV_OK;
  cudaStreamSynchronize(p->P.stream);
  gv::free_problem(p->P);
  delete p;
  return GV_OK;
}

gv_status gv_problem_info_get(const gv_problem* p, gv_problem_info* info) {
  GV_CHECK_PROBLEM(p);
  if (!info) {
    gv::set_error("null info");
    return GV_ERR_INVALID;
  }
  const Problem& P = p->P;
  info->fg_scale = P.fg_scale;
  info->noise_cut = P.noise_cut;
  info->vis_noise = P.vis_noise;
  info->minpix = P.minpix;
  info->beam_bmaj_deg = P.bmaj;
  info->beam_bmin_deg = P.bmin;
  info->beam_bpa_deg = P.bpa;
  info->sum_weights = P.sum_weights;
  info->nvis_total = P.V;
  info->nvis_in_grid = P.Vgrid;
  info->mask_pixels = P.mask_pixels;
  info->dchi2_engine = P.engine;
  info->nterms = (int32_t)P.terms.size();
  return GV_OK;
}

gv_status gv_problem_set_stream(gv_problem* p, void* stream) {
  GV_CHECK_PROBLEM(p);
  p->P.stream = (cudaStream_t)stream;
  return GV_OK;
}

gv_status gv_noise_image(gv_problem* p, float* d_out) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_out) { gv::set_error("null output"); return GV_ERR_INVALID; }
  GV_CUDA(cudaMemcpyAsync(d_out, P.d_noise, sizeof(float) * P.M * P.N,
                          cudaMemcpyDeviceToDevice, P.stream));
  GV_SYNC(P);
  return GV_OK;
}

gv_status gv_initial_image(gv_problem* p, float* d_img) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_img) { gv::set_error("null image"); return GV_ERR_INVALID; }
  const int64_t MN = (int64_t)P.M * P.N;
  std::vector<float> h(2 * MN, 0.0f);
  for (int64_t q = 0; q < MN; q++) h[q] = P.minpix;
  GV_CUDA(cudaMemcpyAsync(d_img, h.data(), sizeof(float) * 2 * MN, cudaMemcpyHostToDevice,
                          P.stream));
  GV_SYNC(P);
  return GV_OK;
}

gv_status gv_chi2(gv_problem* p, float* d_img, int32_t flag_opt, double* chi2) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_img || !chi2) { gv::set_error("null image or output"); return GV_ERR_INVALID; }
  gv_status s = gv::chi2_launch(P, d_img, flag_opt, true);
  if (s != GV_OK) return s;
  s = gv::fetch_scalars(P, gv::kSlotChi2 + 1);
  if (s != GV_OK) return s;
  *chi2 = P.h_scal[gv::kSlotChi2];
  return GV_OK;
}

gv_status gv_dchi2(gv_problem* p, const float* d_img, int32_t flag_opt, float* d_result) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_img || !d_result) { gv::set_error("null image or result"); return GV_ERR_INVALID; }
  gv_status s = gv::dchi2_launch(P, d_img, flag_opt, d_result);
  if (s != GV_OK) return s;
  return gv::check_device_error(P);
}

gv_status gv_dchi2_channel(gv_problem* p, int32_t channel, float* d_out) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_out || channel < 0 || channel >= (int)P.chans.size()) {
    gv::set_error("invalid channel or output");
    return GV_ERR_INVALID;
  }
  gv_status s = gv::dchi2_channel_launch(P, channel, d_out);
  if (s != GV_OK) return s;
  return gv::check_device_error(P);
}

gv_status gv_prior_value(gv_problem* p, int32_t term, const float* d_img, double* value) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_img || !value || term < 0 || term >= (int)P.terms.size() ||
      P.terms[term].kind == GV_FI_CHI2) {
    gv::set_error("invalid prior term or arguments");
    return GV_ERR_INVALID;
  }
  gv_status s = gv::prior_value_launch(P, term, d_img, gv::kSlotOpt);
  if (s != GV_OK) return s;
  s = gv::fetch_scalars(P, gv::kSlotOpt + 1);
  if (s != GV_OK) return s;
  *value = P.h_scal[gv::kSlotOpt];
  return GV_OK;
}

gv_status gv_prior_gradient(gv_problem* p, int32_t term, const float* d_img, float* d_dphi) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_img || !d_dphi || term < 0 || term >= (int)P.terms.size() ||
      P.terms[term].kind == GV_FI_CHI2) {
    gv::set_error("invalid prior term or arguments");
    return GV_ERR_INVALID;
  }
  gv_status s = gv::prior_grad_launch(P, term, d_img, d_dphi);
  if (s != GV_OK) return s;
  GV_SYNC(P);
  return GV_OK;
}

gv_status gv_objective(gv_problem* p, float* d_img, int32_t flag_opt, double* f,
                       double* fi_values) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_img || !f) { gv::set_error("null image or output"); return GV_ERR_INVALID; }
  gv_status s = P.use_graphs ? gv::eval_graph(P, d_img, nullptr, 0, flag_opt, 1, true)
                             : gv::objective_launch(P, d_img, flag_opt, true);
  if (s != GV_OK) return s;
  s = gv::fetch_scalars(P, gv::kSlotTerm0 + (int)P.terms.size());
  if (s != GV_OK) return s;
  double tot = 0.0;
  for (size_t t = 0; t < P.terms.size(); t++) {
    const double v = P.h_scal[gv::kSlotTerm0 + t];
    if (fi_values) fi_values[t] = v;
    tot += (double)P.terms[t].lambda * v;
  }
  *f = tot;
  return GV_OK;
}

gv_status gv_objective_many(gv_problem* p, const float* const* d_imgs, int32_t count,
                            int32_t flag_opt, double* f, double* fi_values) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_imgs || !f || count < 0) { gv::set_error("invalid image list or output"); return GV_ERR_INVALID; }
  for (int32_t i = 0; i < count; i++)
    if (!d_imgs[i]) { gv::set_error("null image in the list"); return GV_ERR_INVALID; }
  const int nt = (int)P.terms.size();
  const size_t need = (size_t)count * (size_t)nt;
  if (P.h_many_cap < need) {
    if (P.h_many) cudaFreeHost(P.h_many);
    P.h_many = nullptr;
    P.h_many_cap = 0;
    GV_CUDA(cudaMallocHost(&P.h_many, sizeof(double) * std::max<size_t>(need, 1)));
    P.h_many_cap = need;
  }
  const size_t bytes = sizeof(float) * 2 * (size_t)P.M * (size_t)P.N;
  for (int32_t i = 0; i < count; i++) {
    GV_CUDA(cudaMemcpyAsync(P.d_tmp, d_imgs[i], bytes, cudaMemcpyDeviceToDevice, P.stream));
    gv_status s = P.use_graphs ? gv::eval_graph(P, P.d_tmp, nullptr, 0, flag_opt, 1, false)
                               : gv::objective_launch(P, P.d_tmp, flag_opt, false);
    if (s != GV_OK) return s;
    GV_CUDA(cudaMemcpyAsync(P.h_many + (size_t)i * nt, P.d_scal + gv::kSlotTerm0,
                            sizeof(double) * nt, cudaMemcpyDeviceToHost, P.stream));
  }
  GV_CUDA(cudaStreamSynchronize(P.stream));
  for (int32_t i = 0; i < count; i++) {
    double tot = 0.0;
    for (int t = 0; t < nt; t++) {
      const double v = P.h_many[(size_t)i * nt + t];
      if (fi_values) fi_values[(size_t)i * nt + t] = v;
      tot += (double)P.terms[t].lambda * v;
    }
    f[i] = tot;
  }
  return gv::check_device_error(P);
}

gv_status gv_gradient(gv_problem* p, float* d_img, float* d_xi, int32_t iter, int32_t flag_opt) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_img || !d_xi || iter < 0) { gv::set_error("invalid gradient arguments"); return GV_ERR_INVALID; }
  gv_status s = P.use_graphs ? gv::eval_graph(P, d_img, d_xi, iter, flag_opt, 2, false)
                             : gv::gradient_launch(P, d_img, d_xi, iter, flag_opt);
  if (s != GV_OK) return s;
  return gv::check_device_error(P);
}

gv_status gv_evaluate(gv_problem* p, float* d_img, float* d_xi, int32_t iter, int32_t flag_opt,
                      double* f, double* fi_values) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_img || !d_xi || !f || iter < 0) {
    gv::set_error("invalid evaluate arguments");
    return GV_ERR_INVALID;
  }
  gv_status s = gv::eval_graph(P, d_img, d_xi, iter, flag_opt, 3, true);
  if (s != GV_OK) return s;
  s = gv::fetch_scalars(P, gv::kSlotTerm0 + (int)P.terms.size());
  if (s != GV_OK) return s;
  double tot = 0.0;
  for (size_t t = 0; t < P.terms.size(); t++) {
    const double v = P.h_scal[gv::kSlotTerm0 + t];
    if (fi_values) fi_values[t] = v;
    tot += (double)P.terms[t].lambda * v;
  }
  *f = tot;
  return gv::check_device_error(P);
}

gv_status gv_problem_set_graphs(gv_problem* p, int32_t enable) {
  GV_CHECK_PROBLEM(p);
  p->P.use_graphs = enable ? 1 : 0;
  return GV_OK;
}

gv_status gv_optimize(gv_problem* p, const gv_opt_desc* opt, float* d_img, gv_opt_report* report) {
  GV_CHECK_PROBLEM(p);
  if (!opt || !d_img) { gv::set_error("null optimizer descriptor or image"); return GV_ERR_INVALID; }
  gv_status s = gv::optimize(p->P, *opt, d_img, report);
  if (s != GV_OK) return s;
  return gv::check_device_error(p->P);
}

gv_status gv_linmin(gv_problem* p, float* d_p, float* d_xi, int32_t flag_opt,
                    int32_t positivity, float* fret, int64_t* evals) {
  GV_CHECK_PROBLEM(p);
  if (!d_p || !d_xi || !fret) { gv::set_error("null image, direction or output"); return GV_ERR_INVALID; }
  gv_opt_desc o;
  std::memset(&o, 0, sizeof(o));
  o.kind = GV_OPT_FRPRMN;
  o.ftol = 1e-12f;
  o.gtol = 1e-12f;
  o.K = 1;
  o.flag = flag_opt;
  o.positivity = positivity ? 1 : 0;
  gv_status s = gv::linmin(p->P, o, d_p, d_xi, fret, evals);
  if (s != GV_OK) return s;
  return gv::check_device_error(p->P);
}

gv_status gv_optimize_until(gv_problem* p, const gv_opt_desc* opt, float* d_img, double f_target,
                            int32_t priors_from_start, gv_opt_report* report) {
  GV_CHECK_PROBLEM(p);
  if (!opt || !d_img) { gv::set_error("null optimizer descriptor or image"); return GV_ERR_INVALID; }
  gv_status s = gv::optimize(p->P, *opt, d_img, report, f_target, priors_from_start ? 1 : 0);
  if (s != GV_OK) return s;
  return gv::check_device_error(p->P);
}

gv_status gv_error_images(gv_problem* p, float* d_img, float* d_err) {
  GV_CHECK_PROBLEM(p);
  if (!d_img || !d_err) { gv::set_error("null image or output"); return GV_ERR_INVALID; }
  gv_status s = gv::error_images(p->P, d_img, d_err);
  if (s != GV_OK) return s;
  return gv::check_device_error(p->P);
}

gv_status gv_autotune(gv_problem* p, gv_tune_report* report) {
  GV_CHECK_PROBLEM(p);
  gv_tune_report r;
  std::memset(&r, 0, sizeof(r));
  gv_status s = gv::autotune(p->P, &r);
  if (report) *report = r;
  if (s != GV_OK) return s;
  return gv::check_device_error(p->P);
}

gv_status gv_set_iteration(gv_problem* p, int32_t iter) {
  GV_CHECK_PROBLEM(p);
  if (iter < 0) { gv::set_error("negative iteration"); return GV_ERR_INVALID; }
  p->P.iteration = iter;
  return GV_OK;
}

gv_status gv_dirty_image(gv_problem* p, float* d_out) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_out) { gv::set_error("null output"); return GV_ERR_INVALID; }
  gv_status s = gv::dirty_launch(P, d_out);
  if (s != GV_OK) return s;
  return gv::check_device_error(P);
}

gv_status gv_psf_image(gv_problem* p, float* d_out) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!d_out) { gv::set_error("null output"); return GV_ERR_INVALID; }
  gv_status s = gv::dirty_launch(P, d_out, true);
  if (s != GV_OK) return s;
  return gv::check_device_error(P);
}

gv_status gv_residuals(gv_problem* p, float* h_out) {
  GV_CHECK_PROBLEM(p);
  Problem& P = p->P;
  if (!h_out) { gv::set_error("null output"); return GV_ERR_INVALID; }
  std::vector<float> sorted(2 * P.V);
  std::vector<int64_t> perm(P.V);
  GV_CUDA(cudaMemcpyAsync(sorted.data(), P.d_cvr, sizeof(float) * 2 * P.V,
                          cudaMemcpyDeviceToHost, P.stream));
  GV_CUDA(cudaMemcpyAsync(perm.data(), P.d_perm, sizeof(int64_t) * P.V, cudaMemcpyDeviceToHost,
                          P.stream));
  GV_SYNC(P);
  for (int64_t k = 0; k < P.V; k++) {
    h_out[2 * perm[k]] = sorted[2 * k];
    h_out[2 * perm[k] + 1] = sorted[2 * k + 1];
  }
  return GV_OK;
}

const char* gv_last_error(void) { return gv::g_last_error.c_str(); }

int64_t gv_launch_count(void) { return (int64_t)gv::g_launches.load(); }

const char* gv_version(void) { return "gpuvmem_gb300 0.1 (sm_103a)"; }

}  // extern "C"
