// gpuvmem's plugin surface on the GB300 library.
//
// This translation unit is built inside gpuvmem, against gpuvmem's own
// headers, in place of the sources of the plugins it replaces:
//   src/chi2.cu  src/entropy.cu  src/totalsquaredvariation.cu
//   src/totalvariation.cu  src/l1norm.cu  src/laplacian.cu
//   src/frprmn.cu  src/lbfgs.cu
// and linked with libgpuvmem_gb300.so.  Its classes derive from gpuvmem's
// Fi (include/classes/fi.cuh:13-104) and Optimizer
// (include/classes/optimizer.cuh:5-60) and register under the same ids
// through gpuvmem's Factory (include/factory.cuh:74-89), so main.cu's
// wiring -- createObject<Fi, std::string>("Chi2"), configure, setPrior,
// ObjectiveFunction::addFi, createObject<Optimizer, std::string>
// ("CG-FRPRMN"), MFS::run -- runs unchanged on the GB300 kernels.
//
// One gv_problem serves every term of a run.  It is created at the first
// evaluation from gpuvmem's globals as MFS::setDevice left them (the host
// visibilities of datasets[], M, N, DELTAX, DELTAY, nu_0, eta,
// initial_values, threshold, the -N noise cut) and from the terms in the
// order they were configured, leaving out those with a zero penalization
// factor as ObjectiveFunction::addFi does.  Settings changed after that
// (setPenalizationFactor, setPrior) do not reach the problem.  The
// visibilities of one field are supported (the pointing and phase centres
// of that field coincide, as the problem takes one centre); other layouts
// stop with an error, as gpuvmem's configuration errors do.
//
// Build (inside gpuvmem's tree, next to its other sources):
//   nvcc -std=c++17 -x cu -I include -I include/classes -I src \
//        -I <gpuvmem_gb300>/include -c gvgb_plugins.cu
// and link the program with -L<gpuvmem_gb300>/gpuvmem_gb300 -lgpuvmem_gb300.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "framework.cuh"
#include "functions.cuh"
#include "gpuvmem_gb300.h"

// gpuvmem's globals (src/mfs.cu:4-45, src/main.cu)
extern long M, N;
extern int image_count;
extern float* penalizators;
extern int nPenalizators;
extern std::vector<MSDataset> datasets;
extern std::vector<float> initial_values;
extern float eta, threshold, nu_0;
extern double DELTAX, DELTAY;
extern bool nopositivity;
extern Vars variables;

// Globals the replaced src/frprmn.cu defined for the rest of gpuvmem
// (src/f1dim.cu:46-47, src/linmin.cu:48-50, src/chi2.cu:9)
ObjectiveFunction* testof;
Image* I;
int flag_opt;

namespace gvgb {

// Report a failed library call the way gpuvmem reports errors: print, stop.
static void check(gv_status s, const char* what) {
  if (s != GV_OK) {
    std::fprintf(stderr, "gpuvmem_gb300: %s failed: %s\n", what, gv_last_error());
    std::exit(-1);
  }
}

class Term;

// The problem shared by the terms of a run.
struct Shared {
  gv_problem* prob = nullptr;
  std::vector<Term*> configured;  // configure() order
  std::vector<Term*> terms;       // the problem's terms (non-zero factors)
  float* d_tmp = nullptr;         // 2 planes: a term's own gradient
  float fg_scale = -1.0f;         // Chi2::setFgScale, when called
  int normalize = 0;
  static Shared& get() {
    static Shared s;
    return s;
  }
  gv_problem* problem();
  int index_of(const Term* t) const {
    for (size_t i = 0; i < terms.size(); i++)
      if (terms[i] == t) return (int)i;
    return -1;
  }
};

// A term of the objective: gpuvmem's Fi with the library's kind.
class Term : public Fi {
 public:
  explicit Term(int kind, const char* id) : kind_(kind) { this->name = id; }
  int kind() const { return kind_; }
  float prior() const { return prior_; }
  float eta_value() const { return eta_; }
  float epsilon() const { return epsilon_; }
  int image_index() const { return imageIndex; }
  int image_to_add() const { return imageToAdd; }

  void configure(int penalizatorIndex, int imageIndex, int imageToAdd, bool normalize) override {
    this->imageIndex = imageIndex;
    this->imageToAdd = imageToAdd;
    this->normalize = normalize;
    if (imageIndex > image_count - 1 || imageToAdd > image_count - 1) {
      std::printf("There is no image for the provided index %s\n", this->name.c_str());
      std::exit(-1);
    }
    if (penalizatorIndex != -1) {
      if (penalizatorIndex < 0) {
        std::printf("invalid index for penalizator (%s)\n", this->name.c_str());
        std::exit(-1);
      }
      this->penalization_factor =
          penalizatorIndex > nPenalizators - 1 ? 0.0f : penalizators[penalizatorIndex];
    }
    Shared::get().configured.push_back(this);
  }

  // value of the term at p (before the penalization factor): the
  // reference's priors count only once iteration > 0
  float calcFi(float* p) override {
    Shared& s = Shared::get();
    gv_problem* prob = s.problem();
    double v = 0.0;
    if (this->iteration > 0 && this->penalization_factor != 0.0f)
      check(gv_prior_value(prob, s.index_of(this), p, &v), "gv_prior_value");
    this->set_fivalue((float)v);
    return this->penalization_factor * this->get_fivalue();
  }

  void calcGi(float* p, float* xi) override {
    Shared& s = Shared::get();
    gv_problem* prob = s.problem();
    restartDGi();
    if (this->iteration > 0 && this->penalization_factor != 0.0f && flag_opt % 2 == imageIndex) {
      check(gv_prior_gradient(prob, s.index_of(this), p, s.d_tmp), "gv_prior_gradient");
      have_grad_ = true;
    }
  }

  void restartDGi() override {
    Shared& s = Shared::get();
    s.problem();
    checkCudaErrors(cudaMemset(s.d_tmp, 0, sizeof(float) * 2 * M * N));
    have_grad_ = false;
  }

  // the term's gradient went into plane imageToAdd of the scratch (plane 0
  // for TotalVariation, as its addToDphi, src/totalvariation.cu:48)
  void addToDphi(float* device_dphi) override {
    if (!have_grad_) return;
    const int add = kind_ == GV_FI_TV ? 0 : imageToAdd;
    linkAddToDPhi(device_dphi, Shared::get().d_tmp + (long)M * N * add, add);
  }

  void setPrior(float prior) override { prior_ = prior; }
  float getEta() override { return eta_; }
  void setEta(float e) override { eta_ = e; }
  float calculateSecondDerivate() override { return 0.0f; }

 protected:
  int kind_;
  float prior_ = 1.0f;      // Entropy::Entropy(), src/entropy.cu:9
  float eta_ = -1.0f;       // src/entropy.cu:10
  float epsilon_ = 1e-12f;  // TVariation / L1norm defaults
  bool have_grad_ = false;
};

// Chi2: calcFi = lambda * chi2, calcGi = DChi2 into result_dchi2, and
// addToDphi overwrites dphi (src/chi2.cu:44-70).
class Chi2GB : public Term {
 public:
  Chi2GB() : Term(GV_FI_CHI2, "Chi2") {}
  void configure(int penalizatorIndex, int imageIndex, int imageToAdd, bool normalize) override {
    this->imageIndex = imageIndex;
    this->normalize = normalize;
    if (penalizatorIndex != -1) {
      if (penalizatorIndex > (nPenalizators - 1) || penalizatorIndex < 0) {
        std::printf("invalid index for penalizator (%s)\n", this->name.c_str());
        std::exit(-1);
      }
      this->penalization_factor = penalizators[penalizatorIndex];
    }
    Shared::get().normalize = normalize ? 1 : 0;
    checkCudaErrors(cudaMalloc((void**)&result_, sizeof(float) * M * N * image_count));
    checkCudaErrors(cudaMemset(result_, 0, sizeof(float) * M * N * image_count));
    Shared::get().configured.push_back(this);
  }
  float calcFi(float* p) override {
    double v = 0.0;
    check(gv_chi2(Shared::get().problem(), p, flag_opt, &v), "gv_chi2");
    this->set_fivalue((float)v);
    return this->penalization_factor * this->get_fivalue();
  }
  void calcGi(float* p, float* xi) override {
    check(gv_dchi2(Shared::get().problem(), p, flag_opt, result_), "gv_dchi2");
  }
  void restartDGi() override {
    checkCudaErrors(cudaMemset(result_, 0, sizeof(float) * M * N * image_count));
  }
  void addToDphi(float* device_dphi) override {
    if (image_count == 1) linkAddToDPhi(device_dphi, result_, 0);
    if (image_count > 1) {
      checkCudaErrors(cudaMemset(device_dphi, 0, sizeof(float) * M * N * image_count));
      checkCudaErrors(cudaMemcpy(device_dphi, result_, sizeof(float) * N * M * image_count,
                                 cudaMemcpyDeviceToDevice));
    }
  }
  void setFgScale(float fg) override { Shared::get().fg_scale = fg; }
  float getFgScale() override {
    gv_problem_info inf;
    check(gv_problem_info_get(Shared::get().problem(), &inf), "gv_problem_info_get");
    return inf.fg_scale;
  }
  void setCKernel(CKernel*) override {
    std::fprintf(stderr, "gpuvmem_gb300: gridded data are passed to the library with their "
                         "GCF (gv_problem_desc.gcf); Chi2::setCKernel is not forwarded\n");
  }

 private:
  float* result_ = nullptr;
};

class EntropyGB : public Term {
 public:
  EntropyGB() : Term(GV_FI_ENTROPY, "Entropy") {}
};
class TSVGB : public Term {
 public:
  TSVGB() : Term(GV_FI_TSV, "TotalSquaredVariation") {}
};
class TVGB : public Term {
 public:
  TVGB() : Term(GV_FI_TV, "TotalVariation") {}
};
class L1GB : public Term {
 public:
  L1GB() : Term(GV_FI_L1, "L1-Norm") {}
};
class LaplacianGB : public Term {
 public:
  LaplacianGB() : Term(GV_FI_LAPLACIAN, "Laplacian") {}
};

// XX, YY, LL, RR: the correlations chi2() sums (src/functions.cu:4246)
static bool counted(int corr) {
  return corr == LL || corr == RR || corr == XX || corr == YY;
}

gv_problem* Shared::problem() {
  if (prob) return prob;
  std::vector<gv_fi_desc> fd;
  for (Term* t : configured) {
    if (t->getPenalizationFactor() == 0.0f) continue;  // ObjectiveFunction::addFi
    terms.push_back(t);
    gv_fi_desc d = {};
    d.kind = t->kind();
    d.lambda = t->getPenalizationFactor();
    d.image_index = t->image_index();
    d.image_to_add = t->image_to_add();
    d.prior_value = t->prior();
    d.eta = t->eta_value();
    d.epsilon = t->epsilon();
    d.normalization_factor = 1.0f;
    d.epsilon_b = 1e-12f;
    fd.push_back(d);
  }
  std::vector<gv_channel_desc> ch;
  const Field* field = nullptr;
  for (const MSDataset& ds : datasets) {
    if (ds.fields.size() != 1 || (field && &ds.fields[0] != field && datasets.size() > 1 &&
                                  (ds.fields[0].phs_xobs_pix != field->phs_xobs_pix ||
                                   ds.fields[0].phs_yobs_pix != field->phs_yobs_pix))) {
      std::fprintf(stderr, "gpuvmem_gb300: one field with one phase centre is supported\n");
      std::exit(-1);
    }
    const Field& f = ds.fields[0];
    field = &f;
    for (size_t i = 0; i < f.nu.size(); i++)
      for (int s = 0; s < ds.data.nstokes; s++) {
        if (!counted(ds.data.corr_type[s])) continue;
        const long nv = f.numVisibilitiesPerFreqPerStoke[i][s];
        if (nv <= 0) continue;
        const HVis& v = f.visibilities[i][s];
        gv_channel_desc c;
        c.freq_hz = f.nu[i];
        c.nvis = nv;
        c.uvw = reinterpret_cast<const double*>(v.uvw.data());
        c.vo = reinterpret_cast<const float*>(v.Vo.data());
        c.weight = v.weight.data();
        ch.push_back(c);
      }
  }
  if (!field || datasets.empty() || datasets[0].antennas.empty()) {
    std::fprintf(stderr, "gpuvmem_gb300: no visibilities (MFS::setDevice must run first)\n");
    std::exit(-1);
  }
  const MSAntenna& ant = datasets[0].antennas[0];
  gv_problem_desc d = {};
  d.M = (int32_t)M;
  d.N = (int32_t)N;
  d.deltax_deg = DELTAX;
  d.deltay_deg = DELTAY;
  d.xobs_pix = field->phs_xobs_pix;
  d.yobs_pix = field->phs_yobs_pix;
  d.nu_0 = nu_0;
  d.antenna_diameter = ant.antenna_diameter;
  d.pb_factor = ant.pb_factor;
  d.pb_cutoff = ant.pb_cutoff;
  d.primary_beam = ant.primary_beam == GAUSSIAN ? GV_BEAM_GAUSSIAN : GV_BEAM_AIRYDISK;
  d.vis_noise = variables.noise;
  d.noise_cut_factor = variables.noise_cut;
  d.eta = eta;
  d.initial_value = initial_values.empty() ? 0.001f : initial_values[0];
  d.threshold = threshold;
  d.normalize = normalize;
  d.nchannels = (int32_t)ch.size();
  d.channels = ch.data();
  d.nterms = (int32_t)fd.size();
  d.terms = fd.data();
  d.dchi2_engine = 0;
  d.gcf = nullptr;
  check(gv_problem_create(&d, &prob), "gv_problem_create");
  checkCudaErrors(cudaMalloc((void**)&d_tmp, sizeof(float) * 2 * M * N));
  return prob;
}

// Optimizer: gv_optimize on the shared problem and the image's buffer;
// afterwards the terms' values are those of the final image, as the
// reference's last calcFunction leaves them.
class OptimizerGB : public Optimizer {
 public:
  explicit OptimizerGB(int kind) : kind_(kind) {}
  void allocateMemoryGpu() override {}
  void deallocateMemoryGpu() override {}
  int getK() override { return K_; }
  void setK(int K) override { K_ = K; }
  void optimize() override {
    Shared& s = Shared::get();
    gv_problem* prob = s.problem();
    testof = of;
    I = image;
    flag_opt = flag;
    gv_opt_desc o = {};
    o.kind = kind_;
    o.total_iterations = total_iterations;
    o.ftol = ftol;
    o.gtol = gtol;
    o.K = K_;
    o.flag = flag;
    o.positivity = nopositivity ? 0 : 1;
    gv_opt_report rep = {};
    check(gv_optimize(prob, &o, image->getImage(), &rep), "gv_optimize");
    current_iteration = rep.iterations;
    double f = 0.0;
    std::vector<double> fi(s.terms.size() + 1, 0.0);
    check(gv_set_iteration(prob, rep.iterations), "gv_set_iteration");
    check(gv_objective(prob, image->getImage(), flag, &f, fi.data()), "gv_objective");
    for (size_t t = 0; t < s.terms.size(); t++) s.terms[t]->set_fivalue((float)fi[t]);
  }

 private:
  int kind_;
  int K_ = 100;  // src/lbfgs.cu K default (include/lbfgs.cuh:30)
};

}  // namespace gvgb

// Registration under gpuvmem's ids (src/chi2.cu:89, src/entropy.cu:75-79,
// src/totalsquaredvariation.cu:44, src/totalvariation.cu:60,
// src/l1norm.cu:57, src/laplacian.cu:43, src/frprmn.cu:202,
// src/lbfgs.cu:348)
namespace {
Fi* CreateChi2GB() { return new gvgb::Chi2GB; }
Fi* CreateEntropyGB() { return new gvgb::EntropyGB; }
Fi* CreateTSVGB() { return new gvgb::TSVGB; }
Fi* CreateTVGB() { return new gvgb::TVGB; }
Fi* CreateL1GB() { return new gvgb::L1GB; }
Fi* CreateLaplacianGB() { return new gvgb::LaplacianGB; }
Optimizer* CreateFrprmnGB() { return new gvgb::OptimizerGB(GV_OPT_FRPRMN); }
Optimizer* CreateLbfgsGB() { return new gvgb::OptimizerGB(GV_OPT_LBFGS); }

const bool kRegistered[] = {
    registerCreationFunction<Fi, std::string>("Chi2", CreateChi2GB),
    registerCreationFunction<Fi, std::string>("Entropy", CreateEntropyGB),
    registerCreationFunction<Fi, int>(0, CreateEntropyGB),
    registerCreationFunction<Fi, std::string>("TotalSquaredVariation", CreateTSVGB),
    registerCreationFunction<Fi, std::string>("TotalVariation", CreateTVGB),
    registerCreationFunction<Fi, std::string>("L1-Norm", CreateL1GB),
    registerCreationFunction<Fi, std::string>("Laplacian", CreateLaplacianGB),
    registerCreationFunction<Optimizer, std::string>("CG-FRPRMN", CreateFrprmnGB),
    registerCreationFunction<Optimizer, std::string>("CG-LBFGS", CreateLbfgsGB),
};
}  // namespace
