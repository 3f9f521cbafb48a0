// lc2_optimizers.hpp -- the reference's Optimizers{2D,3D,2DTo3D} classes over
// lc2_register (include/lc2.h).
//
// Same constructor, methods and parameter-file semantics as
// src/Optimizers/optimizers.cuh:28-247 / optimizers.cu:
//   * InitialValues / LowerBounds / UpperBounds with the translation and
//     rotation bounds added to the initial values (optimizers.cu:46-57,513-524);
//   * a DIRECT stage on the entries enabled under DIRECT, then the BOBYQA
//     rounds "0".."n" in order, each on its OptimizedEntries with its AbsTol
//     (optimizers.cu:734-970); rounds must be numbered consecutively;
//   * objective -log(LC2) (operator(), wrapper);
//   * RegistrationInfo.log with one row per evaluation (optimizers.cu:709-720);
//   * ExportResults(): the parameter file with the optimum written back into
//     InitialValues, DIRECT and BOBYQA round 0 disabled, and an Outputs block,
//     saved as <name>_result<ext> (optimizers.cu:1040-1106).
// Each optimizer step is evaluated as one batched launch. NLopt itself is not
// used (see lc2_minimize for the methods).
#pragma once

#include "lc2_dropin.hpp"

namespace lc2dropin {

enum class OptimizationEntry { Translation, Rotation, Scale, Shear };

template <class Interp>
class OptimizersBase {
 public:
  std::vector<double> InitialValues, LowerBounds, UpperBounds, OptimalSolution;
  bool DIRECT_Enabled = false;
  int DIRECT_MaxEvals = 0;
  int BOBYQA_Rounds = 0;
  bool BOBYQA_Enabled = false;
  int patchSize = 3;
  int EvalCounter = 0;
  double SimilarityMeasure = 0.0;
  std::string YAML_ParameterPath;

  void LinkToInterpolator(Interp* external_Interpolator) { interp_ = external_Interpolator; }

  // objective of the reference: -log(LC2) at x for the entries being optimised,
  // or the NMI itself for PatchSize 0 (optimizers.cu:722-727)
  double operator()(const std::vector<double>& x) {
    std::vector<double> p = OptimalSolution;
    std::vector<int> idx = indices(current_mask_);
    for (size_t j = 0; j < idx.size() && j < x.size(); ++j) p[idx[j]] = x[j];
    std::vector<float> m(n_ == 6 ? 9 : 16);
    check(lc2_params_to_matrix(mode(), p.data(), interp_->Center(), interp_->Shift(), m.data()),
          "lc2_params_to_matrix");
    double v = 0.0;
    check(lc2_evaluate(interp_->Handle(), m.data(), &v), "lc2_evaluate");
    SimilarityMeasure = v;
    ++EvalCounter;
    return interp_->PatchSize() == 0 ? v : -std::log(v);
  }
  static double wrapper(const std::vector<double>& x, std::vector<double>& grad, void* data) {
    (void)grad;
    return reinterpret_cast<OptimizersBase*>(data)->operator()(x);
  }

  void ShowCurrentResults() {
    current_mask_ = 15;
    std::vector<double> x = OptimalSolution;
    (*this)(x);
    --EvalCounter;  // not counted by the reference
    log_row(0, OptimalSolution.data(), SimilarityMeasure);
  }

  void Optimize() {
    if (!interp_) throw Error(LC2_ERR_NOT_READY, "LinkToInterpolator not called");
    const std::string dir = interp_->GetOutputPath();
    log_.open((dir.empty() ? std::string(".") : dir) + "/RegistrationInfo.log");
    log_ << "Step,Transform[16],Translation_x,Translation_y,Translation_z,Rotation_x,Rotation_y,"
            "Rotation_z,Scale_x,Scale_y,Scale_z,Shear_x,Shear_y,Shear_z,Similarity,-log(sim),"
            "IteratorCounter\n";
    ShowCurrentResults();
    lc2_registration reg{};
    reg.mode = mode();
    for (int i = 0; i < n_; ++i) {
      reg.initial[i] = OptimalSolution[i];
      reg.lower[i] = LowerBounds[i];
      reg.upper[i] = UpperBounds[i];
    }
    for (int a = 0; a < 3; ++a) {
      reg.center[a] = interp_->Center()[a];
      reg.shift[a] = interp_->Shift()[a];
    }
    reg.direct_entries = DIRECT_Enabled ? direct_mask_ : 0;
    reg.direct_maxeval = DIRECT_MaxEvals;
    reg.rounds = std::min(BOBYQA_Rounds, 8);
    for (int r = 0; r < reg.rounds; ++r) {
      reg.round_entries[r] = round_enabled_[r] ? round_mask_[r] : 0;
      reg.round_xtol[r] = round_tol_[r];
    }
    reg.observer = &OptimizersBase::observe;
    reg.observer_user = this;
    lc2_registration_result res{};
    check(lc2_register(interp_->Handle(), &reg, &res), "lc2_register");
    for (int i = 0; i < n_; ++i) OptimalSolution[i] = res.params[i];
    SimilarityMeasure = res.lc2;
    EvalCounter += res.evaluations;
    GetOptimalTransform();
  }

  // moving -> fixed matrix of the optimum (VirtualToFixed x inverse(VirtualToMoving))
  void GetOptimalTransform(float* outMatrix) {
    GetOptimalTransform();
    std::copy(moving_to_fixed_.begin(), moving_to_fixed_.end(), outMatrix);
  }
  void GetOptimalTransform() {
    std::vector<float> m(n_ == 6 ? 9 : 16);
    check(lc2_params_to_matrix(mode(), OptimalSolution.data(), interp_->Center(),
                               interp_->Shift(), m.data()),
          "lc2_params_to_matrix");
    moving_to_fixed_ = invert(m);
  }
  // the moving -> fixed matrix of the last GetOptimalTransform (optimizers.cu:444-448)
  void GetInternalMatrix(float* OutMatrix) {
    if (moving_to_fixed_.empty()) GetOptimalTransform();
    std::copy(moving_to_fixed_.begin(), moving_to_fixed_.end(), OutMatrix);
  }

  // <name>_result<ext> next to the parameter file
  std::string ResultPath() const {
    const size_t slash = YAML_ParameterPath.find_last_of('/');
    const size_t base = (slash == std::string::npos) ? 0 : slash + 1;
    const size_t dot = YAML_ParameterPath.find('.', base);
    std::string p = YAML_ParameterPath;
    p.insert(dot == std::string::npos ? p.size() : dot, "_result");
    return p;
  }

  void ExportResults() {
    GetOptimalTransform();
    lc2yaml::Node y = yaml_;
    lc2yaml::Node& os = y.at("InputParameters").at("OptimizerSettings");
    for (int i = 0; i < n_; ++i)
      os.at("InitialValues").at(keys()[i]) = lc2yaml::Node::scalar(fmt((float)OptimalSolution[i]));
    os.at("DIRECT").at("Enabled") = lc2yaml::Node::scalar("false");
    if (os["BOBYQA"].has("0")) os.at("BOBYQA").at("0").at("Enabled") = lc2yaml::Node::scalar("false");
    lc2yaml::Node& out = y.at("Outputs");
    out.at("IsRegistered") = lc2yaml::Node::scalar("true");
    lc2yaml::Node tm;
    tm.kind = lc2yaml::Node::Seq;
    const int d = (n_ == 6) ? 3 : 4;
    for (int r = 0; r < d; ++r) {
      lc2yaml::Node row;
      row.kind = lc2yaml::Node::Seq;
      for (int c = 0; c < d; ++c) row.seq.push_back(lc2yaml::Node::scalar(fmt(moving_to_fixed_[r * d + c])));
      tm.seq.push_back(row);
    }
    out.at("TransformMatrix") = tm;
    out.at("LastSimilarity") = lc2yaml::Node::scalar(fmt(SimilarityMeasure));
    out.at("NumEvaluations") = lc2yaml::Node::scalar(std::to_string(EvalCounter));
    std::time_t now = std::chrono::system_clock::to_time_t(std::chrono::system_clock::now());
    std::string when = std::ctime(&now);
    out.at("RegistrationDateTime") = lc2yaml::Node::scalar(when);
    lc2yaml::save_file(y, ResultPath());
  }

 protected:
  Interp* interp_ = nullptr;
  lc2yaml::Node yaml_;
  int n_ = 12;
  int direct_mask_ = 0;
  int current_mask_ = 15;
  std::vector<int> round_enabled_, round_mask_;
  std::vector<double> round_tol_;
  std::vector<float> moving_to_fixed_;
  std::ofstream log_;

  virtual int mode() const = 0;
  virtual const std::vector<std::string>& keys() const = 0;

  static std::string fmt(double v) {
    char b[64];
    std::snprintf(b, sizeof(b), "%.9g", v);
    return b;
  }

  std::vector<int> indices(int mask) const {
    std::vector<int> out;
    if (n_ == 6) {
      if (mask & 1) { out.push_back(0); out.push_back(1); }
      if (mask & 2) out.push_back(2);
      if (mask & 4) { out.push_back(3); out.push_back(4); }
      if (mask & 8) out.push_back(5);
    } else {
      for (int g = 0; g < 4; ++g)
        if (mask & (1 << g))
          for (int i = 0; i < 3; ++i) out.push_back(3 * g + i);
    }
    return out;
  }

  static int entries_mask(const lc2yaml::Node& e) {
    int m = 0;
    if (e["Translation"] && e["Translation"].boolean()) m |= LC2_ENTRY_TRANSLATION;
    if (e["Rotation"] && e["Rotation"].boolean()) m |= LC2_ENTRY_ROTATION;
    if (e["Scale"] && e["Scale"].boolean()) m |= LC2_ENTRY_SCALE;
    if (e["Shear"] && e["Shear"].boolean()) m |= LC2_ENTRY_SHEAR;
    return m;
  }

  // optimizers.cu:22-110 (2D), 484-582 (3D)
  void parse(const std::string& path, int n, int offset_entries) {
    YAML_ParameterPath = path;
    yaml_ = lc2yaml::load_file(path);
    n_ = n;
    const lc2yaml::Node& os = yaml_["InputParameters"]["OptimizerSettings"];
    auto vec = [&](const char* tag) {
      std::vector<double> v(n);
      for (int i = 0; i < n; ++i) v[i] = os[tag][keys()[i]].num();
      return v;
    };
    InitialValues = vec("InitialValues");
    OptimalSolution = InitialValues;
    LowerBounds = vec("LowerBounds");
    UpperBounds = vec("UpperBounds");
    for (int i = 0; i < offset_entries; ++i) {
      LowerBounds[i] += InitialValues[i];
      UpperBounds[i] += InitialValues[i];
    }
    DIRECT_Enabled = os["DIRECT"]["Enabled"].boolean();
    direct_mask_ = entries_mask(os["DIRECT"]["OptimizedEntries"]);
    DIRECT_MaxEvals = os["DIRECT"]["MaxEvaluations"].integer();
    BOBYQA_Rounds = (int)os["BOBYQA"].size();
    for (int r = 0; r < BOBYQA_Rounds; ++r) {
      const lc2yaml::Node& rn = os["BOBYQA"][std::to_string(r)];
      if (!rn) throw Error(LC2_ERR_INVALID_ARGUMENT, "BOBYQA rounds are not matching and consistent.");
      round_enabled_.push_back(rn["Enabled"].boolean() ? 1 : 0);
      BOBYQA_Enabled = BOBYQA_Enabled || round_enabled_.back();
      round_mask_.push_back(entries_mask(rn["OptimizedEntries"]));
      round_tol_.push_back(rn["AbsTol"] ? rn["AbsTol"].num() : 1e-4);
    }
    patchSize = yaml_["InputParameters"]["RegistrationParameters"]["PatchSize"].integer();
  }

  std::vector<float> invert(const std::vector<float>& m) const {
    if (m.size() == 16) {
      std::vector<float> o(16);
      check(lc2_invert_affine_3d(m.data(), o.data()), "lc2_invert_affine_3d");
      return o;
    }
    const double det = (double)m[0] * m[4] - (double)m[1] * m[3];
    if (det == 0.0) throw Error(LC2_ERR_SINGULAR, "singular transform");
    const double a = m[4] / det, b = -m[1] / det, c = -m[3] / det, d = m[0] / det;
    return {(float)a, (float)b, (float)(-(a * m[2] + b * m[5])), (float)c, (float)d,
            (float)(-(c * m[2] + d * m[5])), 0.0f, 0.0f, 1.0f};
  }

  void log_row(int step, const double* p, double sim) {
    if (!log_.is_open()) return;
    std::vector<float> m(n_ == 6 ? 9 : 16);
    if (lc2_params_to_matrix(mode(), p, interp_->Center(), interp_->Shift(), m.data()) != LC2_OK)
      return;
    std::vector<float> inv = invert(m);
    log_ << step << ",";
    for (float v : inv) log_ << v << ",";
    for (int i = 0; i < n_; ++i) log_ << (float)p[i] << ",";
    log_ << sim << "," << -std::log(sim) << "," << EvalCounter << "\n";
  }

  static void observe(void* user, int stage, int count, int nparams, const double* params,
                      const double* lc2) {
    OptimizersBase* o = static_cast<OptimizersBase*>(user);
    for (int k = 0; k < count; ++k) {
      ++o->EvalCounter;
      o->log_row(stage, params + (size_t)k * nparams, lc2[k]);
    }
    o->EvalCounter -= count;  // the final count comes from the driver
  }
};

class Optimizers3D : public OptimizersBase<Interpolator3D> {
 public:
  explicit Optimizers3D(std::string FilePath) { parse(FilePath, 12, 6); }

 protected:
  int mode() const override { return LC2_MODE_3D; }
  const std::vector<std::string>& keys() const override {
    static const std::vector<std::string> k = {"TX", "TY", "TZ", "RX", "RY", "RZ",
                                               "ScaleX", "ScaleY", "ScaleZ",
                                               "ShearX", "ShearY", "ShearZ"};
    return k;
  }
};

class Optimizers2DTo3D : public OptimizersBase<Interpolator3D> {
 public:
  explicit Optimizers2DTo3D(std::string FilePath) { parse(FilePath, 12, 6); }

 protected:
  int mode() const override { return LC2_MODE_2DTO3D; }
  const std::vector<std::string>& keys() const override {
    static const std::vector<std::string> k = {"TX", "TY", "TZ", "RX", "RY", "RZ",
                                               "ScaleX", "ScaleY", "ScaleZ",
                                               "ShearX", "ShearY", "ShearZ"};
    return k;
  }
};

class Optimizers2D : public OptimizersBase<Interpolator2D> {
 public:
  explicit Optimizers2D(std::string FilePath) { parse(FilePath, 6, 3); }

 protected:
  int mode() const override { return LC2_MODE_2D; }
  const std::vector<std::string>& keys() const override {
    static const std::vector<std::string> k = {"TX", "TY", "R", "ScaleX", "ScaleY", "Shear"};
    return k;
  }
};

}  // namespace lc2dropin

using lc2dropin::Optimizers2D;
using lc2dropin::Optimizers2DTo3D;
using lc2dropin::Optimizers3D;
