/*
 * C++ mirror of gpuvmem's plugin surface on top of the C ABI
 * (gpuvmem_gb300.h): the Fi terms, ObjectiveFunction, the Optimizer
 * family and the string-keyed factories, with the reference's method names,
 * argument meanings and registration ids, so that main.cu-style wiring
 * (src/main.cu:147-203) works against this library.
 *
 *   Fi                 include/classes/fi.cuh:13-104
 *   ObjectiveFunction  include/classes/objectivefunction.cuh:6-103
 *   Optimizer          include/classes/optimizer.cuh:5-60
 *   Factory            include/factory.cuh:8-89
 *
 * Differences from the reference, all at the boundary:
 *   - Errors never exit: createObject returns nullptr for an unknown id, and
 *     every object keeps the status of its last call (status(), plus
 *     gv_last_error() for the message).  calcFunction returns NaN on error.
 *   - The reference's Fi objects read process globals (datasets, noise
 *     image, MINPIX ...).  Here the ObjectiveFunction owns the problem: give
 *     it the geometry and the visibilities with setData(); it creates the
 *     gv_problem from its Fi list on first use.
 *   - Images are device pointers (2 planes of M*N floats), as the
 *     reference's Image::getImage().
 *
 * Header-only; link with libgpuvmem_gb300.so.
 */
#ifndef GPUVMEM_GB300_HPP
#define GPUVMEM_GB300_HPP

#include <cmath>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "gpuvmem_gb300.h"

namespace gvgb {

class ObjectiveFunction;

// ---------------------------------------------------------------- Fi
class Fi {
 public:
  Fi(gv_fi_kind kind, std::string name) : kind_(kind), name_(std::move(name)) {}
  virtual ~Fi() = default;

  // Fi::configure(penalizatorIndex, imageIndex, imageToAdd, normalize); the
  // penalizator index selects the factor from the -Z list in the reference,
  // here the factor is set with setPenalizationFactor.
  void configure(int penalizatorIndex, int imageIndex, int imageToAdd, bool normalize) {
    penalizator_index_ = penalizatorIndex;
    image_index_ = imageIndex;
    image_to_add_ = imageToAdd;
    normalize_ = normalize;
  }
  void setPenalizationFactor(float f) { lambda_ = f; }
  float getPenalizationFactor() const { return lambda_; }
  void setPrior(float g) { prior_ = g; }
  void setEta(float e) { eta_ = e; }
  void setEpsilon(float e) { epsilon_ = e; }
  void setIteration(int it) { iteration_ = it; }
  int getIteration() const { return iteration_; }
  float get_fivalue() const { return fivalue_; }
  int getImageIndex() const { return image_index_; }
  int getImageToAdd() const { return image_to_add_; }
  int getPenalizatorIndex() const { return penalizator_index_; }
  bool getNormalize() const { return normalize_; }
  const std::string& getName() const { return name_; }
  gv_fi_kind kind() const { return kind_; }
  gv_status status() const { return status_; }

  // Fi::calcFi: lambda * value of this term at d_p (device image).  Chi2
  // clips d_p in place as clip2IWNoise does.
  float calcFi(float* d_p);
  // Fi::calcGi + addToDphi: adds lambda * gradient of this term into d_xi
  // (Chi2 overwrites the plane it writes, as Chi2::addToDphi does).
  void calcGi(float* d_p, float* d_xi);

  gv_fi_desc desc() const {
    gv_fi_desc d{};
    d.kind = (int32_t)kind_;
    d.lambda = lambda_;
    d.image_index = image_index_;
    d.image_to_add = image_to_add_;
    d.prior_value = prior_;
    d.eta = eta_;
    d.epsilon = epsilon_;
    d.prior_image = prior_image_.empty() ? nullptr : prior_image_.data();
    d.normalization_factor = normalization_factor_;
    d.epsilon_b = epsilon_b_;
    return d;
  }

 protected:
  // GEntropy / GL1Norm: a host copy of the prior image (M*N floats), its
  // normalisation factor and GL1Norm's epsilon_b
  std::vector<float> prior_image_;
  float normalization_factor_ = 1.0f, epsilon_b_ = 1e-12f;

 private:
  friend class ObjectiveFunction;
  gv_fi_kind kind_;
  std::string name_;
  float lambda_ = 1.0f, prior_ = 0.001f, eta_ = -1.0f, epsilon_ = 1e-12f;
  int penalizator_index_ = 0, image_index_ = 0, image_to_add_ = 0, iteration_ = 0;
  bool normalize_ = false;
  float fivalue_ = 0.0f;
  gv_status status_ = GV_OK;
  ObjectiveFunction* of_ = nullptr;  // set by ObjectiveFunction::addFi
  int term_ = -1;                    // index among the kept terms
};

// The registered term classes (ids as in the reference).
struct Chi2 : Fi {
  Chi2() : Fi(GV_FI_CHI2, "Chi2") {}
};
struct Entropy : Fi {
  Entropy() : Fi(GV_FI_ENTROPY, "Entropy") {}
};
struct TotalSquaredVariation : Fi {
  TotalSquaredVariation() : Fi(GV_FI_TSV, "TotalSquaredVariation") {}
};
struct TotalVariation : Fi {
  TotalVariation() : Fi(GV_FI_TV, "TotalVariation") {}
};
struct L1Norm : Fi {
  L1Norm() : Fi(GV_FI_L1, "L1-Norm") {}
};
struct Laplacian : Fi {
  Laplacian() : Fi(GV_FI_LAPLACIAN, "Laplacian") {}
};
// GEntropy(prior, normalization_factor, eta) (src/gentropy.cu:32): entropy
// against a prior image (divided by the factor) instead of the constant G
struct GEntropy : Fi {
  GEntropy() : Fi(GV_FI_GENTROPY, "GEntropy") {}
  GEntropy(std::vector<float> prior, float normalization_factor = 1.0f, float eta = -1.0f)
      : Fi(GV_FI_GENTROPY, "GEntropy") {
    setPriorImage(std::move(prior), normalization_factor);
    setEta(eta);
  }
  void setPriorImage(std::vector<float> prior, float normalization_factor = 1.0f) {
    prior_image_ = std::move(prior);
    normalization_factor_ = normalization_factor;
  }
  float getNormalizationFactor() const { return normalization_factor_; }
};
// GL1Norm(prior, normalization_factor, epsilon_a, epsilon_b) (src/gl1norm.cu:42)
struct GL1Norm : Fi {
  GL1Norm() : Fi(GV_FI_GL1, "GL1Norm") {}
  GL1Norm(std::vector<float> prior, float normalization_factor = 1.0f, float epsilon_a = 1e-12f,
          float epsilon_b = 1e-12f)
      : Fi(GV_FI_GL1, "GL1Norm") {
    setPriorImage(std::move(prior), normalization_factor);
    setEpsilon(epsilon_a);
    epsilon_b_ = epsilon_b;
  }
  void setPriorImage(std::vector<float> prior, float normalization_factor = 1.0f) {
    prior_image_ = std::move(prior);
    normalization_factor_ = normalization_factor;
  }
  void setEpsilonB(float e) { epsilon_b_ = e; }
};
// QuadraticP, registered as "Quadratic" (src/quadraticpenalization.cu:41)
struct QuadraticP : Fi {
  QuadraticP() : Fi(GV_FI_QUADRATIC, "Quadratic") {}
};

// ------------------------------------------------------ ObjectiveFunction
class ObjectiveFunction {
 public:
  ObjectiveFunction() = default;
  ObjectiveFunction(const ObjectiveFunction&) = delete;
  ObjectiveFunction& operator=(const ObjectiveFunction&) = delete;
  ~ObjectiveFunction() {
    if (prob_) gv_problem_destroy(prob_);
  }

  // ObjectiveFunction::addFi: terms with a zero factor are not added.
  void addFi(Fi* fi) {
    if (fi->getPenalizationFactor() == 0.0f) return;
    fi->of_ = this;
    fi->term_ = -1;
    fis_.push_back(fi);
    reset();
  }
  // ObjectiveFunction::configure(N, M, I): image size and plane count
  // (gpuvmem always uses 2 planes).
  void configure(long N, long M, int I) {
    N_ = N;
    M_ = M;
    I_ = I;
  }
  // Geometry, beam and visibilities (the part of MFS::setDevice this
  // library takes over).  The desc's term list is ignored: the terms are
  // the Fi objects added with addFi.  Pointers in `d` must stay valid until
  // the first evaluation.
  void setData(const gv_problem_desc& d) {
    base_ = d;
    has_data_ = true;
    reset();
  }
  void setFlag(int flag) { flag_ = flag; }
  int getFlag() const { return flag_; }

  // ObjectiveFunction::calcFunction: sum over the terms of lambda * value.
  float calcFunction(float* d_p) {
    if (!ensure()) return NAN;
    double f = 0.0;
    std::vector<double> v(fis_.size(), 0.0);
    status_ = gv_objective(prob_, d_p, flag_, &f, v.data());
    if (status_ != GV_OK) return NAN;
    for (size_t k = 0; k < fis_.size(); k++) fis_[k]->fivalue_ = (float)v[k];
    return (float)f;
  }
  // ObjectiveFunction::calcGradient(p, xi, iter): every term's gradient
  // into d_xi (the priors start contributing once iter > 0).
  void calcGradient(float* d_p, float* d_xi, int iter) {
    if (!ensure()) return;
    for (Fi* fi : fis_) fi->setIteration(iter);
    status_ = gv_gradient(prob_, d_p, d_xi, iter, flag_);
  }
  Fi* getFiByName(const std::string& name) const {
    for (Fi* fi : fis_)
      if (fi->getName() == name) return fi;
    return nullptr;
  }
  std::vector<float> get_fi_values() const {
    std::vector<float> v;
    for (Fi* fi : fis_) v.push_back(fi->get_fivalue());
    return v;
  }
  const std::vector<Fi*>& getFis() const { return fis_; }
  gv_status status() const { return status_; }
  // the underlying C-ABI handle (created on first use), e.g. for
  // gv_problem_set_stream or gv_problem_info_get
  gv_problem* problem() {
    ensure();
    return prob_;
  }

 private:
  friend class Fi;
  void reset() {
    if (prob_) gv_problem_destroy(prob_);
    prob_ = nullptr;
  }
  bool ensure() {
    if (prob_) return true;
    if (!has_data_) {
      status_ = GV_ERR_INVALID;
      return false;
    }
    std::vector<gv_fi_desc> terms;
    for (Fi* fi : fis_) terms.push_back(fi->desc());
    gv_problem_desc d = base_;
    d.nterms = (int32_t)terms.size();
    d.terms = terms.data();
    if (N_ > 0) {
      d.N = (int32_t)N_;
      d.M = (int32_t)M_;
    }
    for (Fi* fi : fis_)
      if (fi->kind() == GV_FI_CHI2) d.normalize = fi->getNormalize() ? 1 : 0;
    status_ = gv_problem_create(&d, &prob_);
    if (status_ != GV_OK) {
      prob_ = nullptr;
      return false;
    }
    for (size_t k = 0; k < fis_.size(); k++) fis_[k]->term_ = (int)k;
    return true;
  }
  std::vector<Fi*> fis_;
  gv_problem_desc base_{};
  bool has_data_ = false;
  long N_ = 0, M_ = 0;
  int I_ = 2, flag_ = 0;
  gv_problem* prob_ = nullptr;
  gv_status status_ = GV_OK;
};

inline float Fi::calcFi(float* d_p) {
  if (!of_ || !of_->ensure()) {
    status_ = GV_ERR_INVALID;
    return NAN;
  }
  double v = 0.0;
  if (kind_ == GV_FI_CHI2) {
    status_ = gv_chi2(of_->prob_, d_p, of_->flag_, &v);
  } else {
    status_ = gv_prior_value(of_->prob_, term_, d_p, &v);
  }
  if (status_ != GV_OK) return NAN;
  fivalue_ = (float)(lambda_ * v);
  return fivalue_;
}

inline void Fi::calcGi(float* d_p, float* d_xi) {
  if (!of_ || !of_->ensure()) {
    status_ = GV_ERR_INVALID;
    return;
  }
  if (kind_ == GV_FI_CHI2)
    status_ = gv_dchi2(of_->prob_, d_p, of_->flag_, d_xi);
  else
    status_ = gv_prior_gradient(of_->prob_, term_, d_p, d_xi);
}

// ---------------------------------------------------------- fixedPointOpt
// fixedPointOpt (src/fixedpoint.cu:32-57) with its tolFunction (:3-18):
// iterates x1 = optf(x0) until the largest relative change of the entries
// after the first is at most tol, `iterations` are done, or an entry after
// the first reaches 1.  As the reference runs it, x0 advances only from the
// third call on and the first tolerance is taken against a zero vector.
inline float fixedPointTolerance(const std::vector<float>& x1, const std::vector<float>& x0) {
  float mx = 0.0f;
  for (size_t i = 1; i < x1.size(); i++) {
    const float a = x0[i] < 0.0f ? -x0[i] : x0[i];
    const float d = x1[i] - x0[i];
    const float t = a == 0.0f ? 0.0f : (d < 0.0f ? -d : d) / a;
    if (i == 1 || t > mx) mx = t;
  }
  return mx;
}
template <class F>
std::vector<float> fixedPointOpt(std::vector<float> guess, F optf, float tol, int iterations) {
  std::vector<float> x0 = std::move(guess);
  std::vector<float> x1(x0.size(), 0.0f);
  int it = 0;
  float c_tol = fixedPointTolerance(x1, x0);
  while (it < iterations && c_tol > tol) {
    if (it > 1) x0 = x1;
    x1 = optf(x0);
    c_tol = fixedPointTolerance(x1, x0);
    bool big = false;
    for (size_t i = 1; i < x1.size(); i++) big = big || x1[i] >= 1.0f;
    if (big) break;
    it++;
  }
  return x1;
}

// -------------------------------------------------------------- Optimizer
class Optimizer {
 public:
  virtual ~Optimizer() = default;
  virtual void optimize() = 0;
  // Optimizer::allocateMemoryGpu / deallocateMemoryGpu: the library owns its
  // scratch, so these only exist for drop-in wiring.
  virtual void allocateMemoryGpu() {}
  virtual void deallocateMemoryGpu() {}
  // Optimizer::setImage: the device image (2 planes of M*N floats)
  void setImage(float* d_image) { image_ = d_image; }
  float* getImage() const { return image_; }
  void setObjectiveFunction(ObjectiveFunction* of) { of_ = of; }
  ObjectiveFunction* getObjectiveFunction() const { return of_; }
  void setFlag(int flag) { flag_ = flag; }
  int getFlag() const { return flag_; }
  void setFTol(float t) { ftol_ = t; }
  void setGTol(float t) { gtol_ = t; }
  void setTotalIterations(int n) { total_iterations_ = n; }
  int getTotalIterations() const { return total_iterations_; }
  int getCurrentIteration() const { return report_.iterations; }
  void setK(int k) { K_ = k; }
  int getK() const { return K_; }
  void setPositivity(bool on) { positivity_ = on; }
  const gv_opt_report& report() const { return report_; }
  gv_status status() const { return status_; }

 protected:
  void run(gv_optimizer_kind kind) {
    if (!of_ || !image_) {
      status_ = GV_ERR_INVALID;
      return;
    }
    gv_problem* p = of_->problem();
    if (!p) {
      status_ = of_->status();
      return;
    }
    gv_opt_desc o;
    o.kind = (int32_t)kind;
    o.total_iterations = total_iterations_;
    o.ftol = ftol_;
    o.gtol = gtol_;
    o.K = K_;
    o.flag = flag_;
    o.positivity = positivity_ ? 1 : 0;
    of_->setFlag(flag_);
    status_ = gv_optimize(p, &o, image_, &report_);
  }
  ObjectiveFunction* of_ = nullptr;
  float* image_ = nullptr;
  int flag_ = 0, total_iterations_ = 0, K_ = 100;
  float ftol_ = 1e-12f, gtol_ = 1e-12f;  // include/classes/optimizer.cuh:14-18
  bool positivity_ = true;
  gv_opt_report report_{};
  gv_status status_ = GV_OK;
};

// "CG-FRPRMN": ConjugateGradient::optimize (src/frprmn.cu:85-195)
struct ConjugateGradient : Optimizer {
  void optimize() override { run(GV_OPT_FRPRMN); }
};
// "CG-LBFGS": LBFGS::optimize (src/lbfgs.cu:99-200)
struct LBFGS : Optimizer {
  void optimize() override { run(GV_OPT_LBFGS); }
};

// ---------------------------------------------------------------- Factory
// Singleton<Factory<T, std::string>> with registerCreationFunction /
// createObject; an unknown id returns nullptr instead of exiting.
template <class T>
class Factory {
 public:
  using Creator = std::function<T*()>;
  static Factory& instance() {
    static Factory f;
    return f;
  }
  bool registerCreationFunction(const std::string& id, Creator c) {
    return creators_.emplace(id, std::move(c)).second;
  }
  T* createObject(const std::string& id) const {
    auto it = creators_.find(id);
    return it == creators_.end() ? nullptr : it->second();
  }
  std::vector<std::string> ids() const {
    std::vector<std::string> v;
    for (auto& kv : creators_) v.push_back(kv.first);
    return v;
  }

 private:
  Factory() = default;
  std::map<std::string, Creator> creators_;
};

template <class T>
inline bool registerCreationFunction(const std::string& id, std::function<T*()> c) {
  return Factory<T>::instance().registerCreationFunction(id, std::move(c));
}
template <class T>
inline T* createObject(const std::string& id) {
  return Factory<T>::instance().createObject(id);
}

// The reference's registrations: src/chi2.cu:89, src/entropy.cu:75,
// src/totalsquaredvariation.cu:44, src/totalvariation.cu:60,
// src/l1norm.cu:57, src/laplacian.cu:43, src/frprmn.cu:202,
// src/lbfgs.cu:348, include/classes/objectivefunction.cuh:109.
inline void registerAll() {
  static bool done = false;
  if (done) return;
  done = true;
  registerCreationFunction<Fi>("Chi2", [] { return (Fi*)new Chi2(); });
  registerCreationFunction<Fi>("Entropy", [] { return (Fi*)new Entropy(); });
  registerCreationFunction<Fi>("TotalSquaredVariation",
                               [] { return (Fi*)new TotalSquaredVariation(); });
  registerCreationFunction<Fi>("TotalVariation", [] { return (Fi*)new TotalVariation(); });
  registerCreationFunction<Fi>("L1-Norm", [] { return (Fi*)new L1Norm(); });
  registerCreationFunction<Fi>("Laplacian", [] { return (Fi*)new Laplacian(); });
  registerCreationFunction<Fi>("GEntropy", [] { return (Fi*)new GEntropy(); });
  registerCreationFunction<Fi>("GL1Norm", [] { return (Fi*)new GL1Norm(); });
  registerCreationFunction<Fi>("Quadratic", [] { return (Fi*)new QuadraticP(); });
  registerCreationFunction<Optimizer>("CG-FRPRMN",
                                      [] { return (Optimizer*)new ConjugateGradient(); });
  registerCreationFunction<Optimizer>("CG-LBFGS", [] { return (Optimizer*)new LBFGS(); });
  registerCreationFunction<ObjectiveFunction>("ObjectiveFunction",
                                              [] { return new ObjectiveFunction(); });
}

}  // namespace gvgb

#endif
