// Drives the C++ plugin mirror (include/gpuvmem_gb300.hpp) the way gpuvmem's
// main.cu wires its plugins (src/main.cu:147-203).
//   test_plugins cpu  factory ids, unknown ids, error paths (no GPU calls)
//   test_plugins gpu  a small MEM run through the mirror and the same run
//                     through the C ABI: the images must agree bit for bit
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "gpuvmem_gb300.hpp"

static int failures = 0;
#define CHECK(c)                                                  \
  do {                                                            \
    if (!(c)) {                                                   \
      std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #c);    \
      failures++;                                                 \
    }                                                             \
  } while (0)

static int cpu_tests() {
  using namespace gvgb;
  registerAll();
  const char* fis[] = {"Chi2",      "Entropy",  "TotalSquaredVariation", "TotalVariation",
                       "L1-Norm",   "Laplacian", "GEntropy", "GL1Norm", "Quadratic"};
  const gv_fi_kind kinds[] = {GV_FI_CHI2,      GV_FI_ENTROPY,  GV_FI_TSV, GV_FI_TV,
                              GV_FI_L1,        GV_FI_LAPLACIAN, GV_FI_GENTROPY, GV_FI_GL1,
                              GV_FI_QUADRATIC};
  for (int k = 0; k < 9; k++) {
    std::unique_ptr<Fi> f(createObject<Fi>(fis[k]));
    CHECK(f != nullptr);
    if (f) {
      CHECK(f->getName() == fis[k]);
      CHECK(f->kind() == kinds[k]);
    }
  }
  std::unique_ptr<Optimizer> cg(createObject<Optimizer>("CG-FRPRMN"));
  std::unique_ptr<Optimizer> lb(createObject<Optimizer>("CG-LBFGS"));
  CHECK(cg && dynamic_cast<ConjugateGradient*>(cg.get()));
  CHECK(lb && dynamic_cast<LBFGS*>(lb.get()));
  // fixedPointOpt: 0.3 -> 0.6 twice (x0 advances from the third call), then 1.2 stops it
  int ncalls = 0;
  std::vector<float> fp = fixedPointOpt(
      std::vector<float>{0.1f, 0.3f},
      [&](const std::vector<float>& x) {
        ncalls++;
        return std::vector<float>{x[0], 2.0f * x[1]};
      },
      1e-9f, 10);
  CHECK(ncalls == 3 && fp.size() == 2 && fp[1] > 1.19f && fp[1] < 1.21f);
  CHECK(createObject<Fi>("NoSuchPrior") == nullptr);  // the reference exits here
  CHECK(createObject<Optimizer>("CG-NONE") == nullptr);
  CHECK(!registerCreationFunction<Fi>("Chi2", [] { return (Fi*)new Chi2(); }));
  std::unique_ptr<ObjectiveFunction> of(createObject<ObjectiveFunction>("ObjectiveFunction"));
  CHECK(of != nullptr);
  // a term with a zero factor is not added (ObjectiveFunction::addFi)
  Entropy e0;
  e0.setPenalizationFactor(0.0f);
  of->addFi(&e0);
  CHECK(of->getFis().empty());
  // no data: every call reports GV_ERR_INVALID, nothing exits
  Chi2 c;
  of->addFi(&c);
  CHECK(of->getFiByName("Chi2") == &c);
  CHECK(std::isnan(of->calcFunction(nullptr)));
  CHECK(of->status() == GV_ERR_INVALID);
  CHECK(std::isnan(c.calcFi(nullptr)));
  cg->setObjectiveFunction(of.get());
  cg->optimize();
  CHECK(cg->status() == GV_ERR_INVALID);
  return failures;
}

struct Data {
  std::vector<double> uvw;
  std::vector<float> vo, w;
};

static Data make_data(int n, double cell_rad, double freq, int nvis, unsigned seed) {
  std::mt19937 g(seed);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  std::normal_distribution<double> G(0.0, 1.0);
  const double lam = 299792458.0 / freq;
  const double umax = 0.4 * n / (n * cell_rad);  // wavelengths, inside the grid
  Data d;
  for (int k = 0; k < nvis; k++) {
    const double u = umax * U(g), v = umax * U(g), w = 0.02 * umax * U(g);
    d.uvw.insert(d.uvw.end(), {u * lam, v * lam, w * lam});
    // two point sources: 1 Jy at the centre, 0.5 Jy 3 pixels off
    const double ph = 2.0 * M_PI * (u * 3.0 * cell_rad);
    d.vo.push_back((float)(1.0 + 0.5 * std::cos(ph) + 0.01 * G(g)));
    d.vo.push_back((float)(0.5 * std::sin(ph) + 0.01 * G(g)));
    d.w.push_back(1.0f);
  }
  return d;
}

static gv_problem_desc base_desc(int n, double cell_rad, const gv_channel_desc* ch) {
  gv_problem_desc d;
  std::memset(&d, 0, sizeof(d));
  d.M = d.N = n;
  d.deltax_deg = -cell_rad * 180.0 / M_PI;
  d.deltay_deg = cell_rad * 180.0 / M_PI;
  d.xobs_pix = d.yobs_pix = (float)(n / 2);
  d.nu_0 = ch->freq_hz;
  d.antenna_diameter = 12.0f;
  d.pb_factor = 1.13f;
  d.pb_cutoff = 10.0f;
  d.primary_beam = GV_BEAM_GAUSSIAN;
  d.vis_noise = -1.0f;
  d.noise_cut_factor = 10.0f;
  d.eta = -1.0f;
  d.initial_value = 0.001f;
  d.threshold = 0.0f;
  d.nchannels = 1;
  d.channels = ch;
  d.dchi2_engine = 0;
  return d;
}

static int gpu_tests() {
  using namespace gvgb;
  registerAll();
  const int n = 64, nvis = 3000;
  const double cell = 2.0e-6, freq = 230e9;
  Data dat = make_data(n, cell, freq, nvis, 7);
  gv_channel_desc ch = {(float)freq, nvis, dat.uvw.data(), dat.vo.data(), dat.w.data()};
  gv_problem_desc base = base_desc(n, cell, &ch);
  const size_t bytes = sizeof(float) * 2 * n * n;
  float *d_a = nullptr, *d_b = nullptr;
  CHECK(cudaMalloc(&d_a, bytes) == cudaSuccess);
  CHECK(cudaMalloc(&d_b, bytes) == cudaSuccess);

  // --- through the mirror, main.cu style
  std::unique_ptr<ObjectiveFunction> of(createObject<ObjectiveFunction>("ObjectiveFunction"));
  std::unique_ptr<Fi> chi2(createObject<Fi>("Chi2"));
  std::unique_ptr<Fi> ent(createObject<Fi>("Entropy"));
  std::unique_ptr<Fi> tsv(createObject<Fi>("TotalSquaredVariation"));
  chi2->configure(-1, 0, 0, false);
  ent->configure(0, 0, 0, false);
  ent->setPenalizationFactor(0.01f);
  ent->setPrior(0.001f);
  ent->setEta(-1.0f);
  tsv->configure(1, 0, 0, false);
  tsv->setPenalizationFactor(1e-4f);
  of->addFi(chi2.get());
  of->addFi(ent.get());
  of->addFi(tsv.get());
  of->configure(n, n, 2);
  of->setData(base);
  gv_problem* p = of->problem();
  CHECK(p != nullptr);
  if (!p) {
    std::printf("%s\n", gv_last_error());
    return failures + 1;
  }
  CHECK(gv_initial_image(p, d_a) == GV_OK);
  std::unique_ptr<Optimizer> opt(createObject<Optimizer>("CG-FRPRMN"));
  opt->setObjectiveFunction(of.get());
  opt->setImage(d_a);
  opt->setTotalIterations(5);
  opt->setFlag(0);
  opt->optimize();
  CHECK(opt->status() == GV_OK);
  const gv_opt_report ra = opt->report();
  // per-term values after the run
  const float fa = of->calcFunction(d_a);
  CHECK(std::isfinite(fa));
  std::vector<float> fv = of->get_fi_values();
  CHECK(fv.size() == 3);

  // --- the same run through the C ABI
  std::vector<gv_fi_desc> terms = {{GV_FI_CHI2, 1.0f, 0, 0, 0.001f, -1.0f, 1e-12f},
                                   {GV_FI_ENTROPY, 0.01f, 0, 0, 0.001f, -1.0f, 1e-12f},
                                   {GV_FI_TSV, 1e-4f, 0, 0, 0.001f, -1.0f, 1e-12f}};
  gv_problem_desc d2 = base;
  d2.nterms = 3;
  d2.terms = terms.data();
  gv_problem* q = nullptr;
  CHECK(gv_problem_create(&d2, &q) == GV_OK);
  CHECK(gv_initial_image(q, d_b) == GV_OK);
  gv_opt_desc o = {GV_OPT_FRPRMN, 5, 1e-12f, 1e-12f, 100, 0, 1};
  gv_opt_report rb;
  CHECK(gv_optimize(q, &o, d_b, &rb) == GV_OK);
  double fb = 0.0;
  CHECK(gv_objective(q, d_b, 0, &fb, nullptr) == GV_OK);

  std::vector<float> ha(2 * n * n), hb(2 * n * n);
  cudaMemcpy(ha.data(), d_a, bytes, cudaMemcpyDeviceToHost);
  cudaMemcpy(hb.data(), d_b, bytes, cudaMemcpyDeviceToHost);
  CHECK(std::memcmp(ha.data(), hb.data(), bytes) == 0);
  CHECK(ra.iterations == rb.iterations);
  CHECK(ra.f_final == rb.f_final);
  CHECK(fa == (float)fb);
  // a per-term call through the mirror matches the C ABI's prior value
  double v = 0.0;
  CHECK(gv_prior_value(q, 1, d_b, &v) == GV_OK);
  CHECK(std::fabs(ent->calcFi(d_a) - 0.01f * (float)v) <= 1e-6f * std::fabs(0.01f * (float)v));
  std::printf("mirror f=%.9g  c-abi f=%.9g  iterations %d  terms %.6g %.6g %.6g\n", fa, fb,
              ra.iterations, fv[0], fv[1], fv[2]);
  gv_problem_destroy(q);
  cudaFree(d_a);
  cudaFree(d_b);
  return failures;
}

int main(int argc, char** argv) {
  const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
  const int f = gpu ? gpu_tests() : cpu_tests();
  std::printf("%s: %d failure(s)\n", gpu ? "gpu" : "cpu", f);
  return f == 0 ? 0 : 1;
}
