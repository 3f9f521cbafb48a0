// lc2_dropin.hpp -- reference-facing C++ classes over the C ABI (lc2.h).
//
// Keeps the names, signatures and call order of LC2Registration's similarity
// surface so its callers (Optimizers*::operator(), src/Optimizers/optimizers.cu:
// 130-181, 650-732, 1275-1347) compile against this header unchanged:
//
//   Interpolator{2D,3D,2DTo3D}(const LC2Configuration{2D,3D,2DTo3D}*)
//     src/Interpolator/interpolator.cuh:43-130,132-213,215-292
//   InitiateMappers / InitiateRegistrationHandle / GenerateMappers /
//   Interpolate / GetSimilarityMeasure / GetMovingToFixedTransform /
//   GetCurrentTransform
//     src/Interpolator/interpolator.cu:495-679, 1226-1425, 1624-1775
//   LC2_{2D,3D}_class::PrepareGradientFilter / CalculateGradient /
//   GetSimilarityMetric
//     src/cu_LC2/cu_lc2_2d.cuh:10-81, src/cu_LC2/cu_lc2_3d.cuh:10-92
//
// What differs by design: the resample, gradient and similarity run as one
// fused evaluation inside GetSimilarityMeasure (Interpolate and the gradient
// calls only record intent), block-size arguments are accepted and ignored,
// and there is no process-global state, so several interpolators may live in
// one process. Configuration structs follow include/RegistrationParametersConfig.h
// of the reference (the fields this path reads); when that header is already
// included its structs are used as they are.
#pragma once

#include <vector_functions.h>
#include <vector_types.h>

#include <array>
#include <cmath>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "lc2.h"

#ifndef LC2PARAMETERS
#define LC2PARAMETERS
struct regIntPoints3D { int x, y, z; };
struct regFloatingPoints3D { float x, y, z; };
struct regIntPoints2D { int x, y; };
struct regFloatingPoints2D { float x, y; };

// Fields of LC2Configuration2D (RegistrationParametersConfig.h:30-162) read by
// this path.
struct LC2Configuration2D {
  regIntPoints2D FixedDimension{0, 0};
  regFloatingPoints2D FixedSpacing{1.0f, 1.0f};
  regFloatingPoints2D FixedOrigin{0.0f, 0.0f};
  regIntPoints2D MovingDimension{0, 0};
  regFloatingPoints2D MovingSpacing{1.0f, 1.0f};
  regFloatingPoints2D MovingOrigin{0.0f, 0.0f};
  bool IsFixedHighResolution = true;
  bool IsMovingHighResolution = false;
  regFloatingPoints2D SamplerSpacing{1.0f, 1.0f};
  int PatchSize = 9;
  bool IsCenterOverlaid = true;
  bool IsConfigured = false;
  float* FixedBuffer = nullptr;
  float* MovingBuffer = nullptr;
};

// Fields of LC2Configuration3D (RegistrationParametersConfig.h:164-297) read by
// this path; LC2Configuration2DTo3D (:299-431) has the same fields.
struct LC2Configuration3D {
  regIntPoints3D FixedDimension{0, 0, 0};
  regFloatingPoints3D FixedSpacing{1.0f, 1.0f, 1.0f};
  regFloatingPoints3D FixedOrigin{0.0f, 0.0f, 0.0f};
  regIntPoints3D MovingDimension{0, 0, 0};
  regFloatingPoints3D MovingSpacing{1.0f, 1.0f, 1.0f};
  regFloatingPoints3D MovingOrigin{0.0f, 0.0f, 0.0f};
  bool IsFixedHighResolution = false;
  bool IsMovingHighResolution = false;
  regFloatingPoints3D SamplerSpacing{1.0f, 1.0f, 1.0f};
  int PatchSize = 3;
  bool IsCenterOverlaid = true;
  bool IsConfigured = false;
  float* FixedBuffer = nullptr;
  float* MovingBuffer = nullptr;
};
struct LC2Configuration2DTo3D : LC2Configuration3D {};
#endif

namespace lc2dropin {

// Thrown on any non-zero lc2_status (the reference has no error reporting;
// its failures surface later as garbage or exit()).
struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(int status, const char* where) {
  if (status != LC2_OK)
    throw Error(status, std::string(where) + ": " + lc2_last_error());
}

// Owns one lc2_context.
class Context {
 public:
  Context() = default;
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  ~Context() { lc2_destroy(ctx_); }
  void create(const lc2_config& cfg) {
    lc2_destroy(ctx_);
    ctx_ = nullptr;
    check(lc2_create(&cfg, &ctx_), "lc2_create");
  }
  lc2_context* get() const { return ctx_; }

 private:
  lc2_context* ctx_ = nullptr;
};

// Shared machinery of the three interpolators: geometry, mapper centre and
// shift (Interpolator3D::InitiateMappers, interpolator.cu:495-529), the
// current virtual->moving matrix and the evaluation calls.
class InterpolatorBase {
 public:
  // Current virtual->moving matrix (row-major 3x3 in 2D, 4x4 otherwise).
  const std::vector<float>& Matrix() const { return matrix_; }

  // Batched extension: one device launch for many matrices.
  std::vector<double> GetSimilarityMeasureBatch(const std::vector<float>& matrices) {
    const int mf = (int)matrix_.size();
    const int count = (int)(matrices.size() / mf);
    std::vector<double> out(count);
    check(lc2_evaluate_batch(ctx_.get(), matrices.data(), count, out.data()),
          "lc2_evaluate_batch");
    return out;
  }

  lc2_context* Handle() const { return ctx_.get(); }

 protected:
  lc2_config cfg_{};
  bool configured_ = false;
  bool handle_ready_ = false;
  const float* fixed_ = nullptr;
  const float* moving_ = nullptr;
  float center_[3] = {0, 0, 0};
  float shift_[3] = {0, 0, 0};
  bool centered_ = true;
  std::vector<float> matrix_;
  Context ctx_;

  static float geom_center(const lc2_geometry& g, int a) {
    return g.origin[a] + g.spacing[a] * (float)g.dim[a] / 2.0f;
  }

  void mappers(int nd) {
    // rotation centre = fixed centre; shift = moving centre - virtual centre
    // when the spaces are centred (interpolator.cu:516-524, 1226-1246)
    lc2_geometry v{};
    for (int a = 0; a < 3; ++a) {
      v.origin[a] = cfg_.fixed.origin[a];
      v.spacing[a] = cfg_.virtual_spacing[a];
      v.dim[a] = (a < nd) ? (int)std::ceil((double)((float)cfg_.fixed.dim[a] *
                                                     cfg_.fixed.spacing[a] /
                                                     cfg_.virtual_spacing[a]))
                          : 1;
    }
    for (int a = 0; a < 3; ++a) {
      center_[a] = geom_center(cfg_.fixed, a);
      shift_[a] = centered_ ? geom_center(cfg_.moving, a) - geom_center(v, a) : 0.0f;
    }
  }

  void handle() {
    if (!configured_) {
      std::printf("Please configure the Parameter file! \n");
      return;
    }
    ctx_.create(cfg_);
    check(lc2_set_images(ctx_.get(), fixed_, moving_), "lc2_set_images");
    handle_ready_ = true;
  }

  double measure(int patchSize) {
    if (!handle_ready_) throw Error(LC2_ERR_NOT_READY, "InitiateRegistrationHandle not called");
    if (patchSize != cfg_.patch_size) {
      // the patch size is part of the compiled evaluation plan
      cfg_.patch_size = patchSize;
      handle();
    }
    double v = 0.0;
    check(lc2_evaluate(ctx_.get(), matrix_.data(), &v), "lc2_evaluate");
    return v;
  }
};

// 3D registration: MR/CT volume <-> US volume.
class Interpolator3D : public InterpolatorBase {
 public:
  explicit Interpolator3D(const LC2Configuration3D* c, int mode = LC2_MODE_3D) {
    if (!c || !c->IsConfigured) {
      std::printf("Please configure the Parameter file! \n");
      return;
    }
    cfg_.mode = mode;
    cfg_.fixed = {{c->FixedDimension.x, c->FixedDimension.y, c->FixedDimension.z},
                  {c->FixedSpacing.x, c->FixedSpacing.y, c->FixedSpacing.z},
                  {c->FixedOrigin.x, c->FixedOrigin.y, c->FixedOrigin.z}};
    cfg_.moving = {{c->MovingDimension.x, c->MovingDimension.y, c->MovingDimension.z},
                   {c->MovingSpacing.x, c->MovingSpacing.y, c->MovingSpacing.z},
                   {c->MovingOrigin.x, c->MovingOrigin.y, c->MovingOrigin.z}};
    cfg_.virtual_spacing[0] = c->SamplerSpacing.x;
    cfg_.virtual_spacing[1] = c->SamplerSpacing.y;
    cfg_.virtual_spacing[2] = c->SamplerSpacing.z;
    cfg_.patch_size = c->PatchSize;
    cfg_.high_res_is_moving = c->IsMovingHighResolution ? 1 : 0;
    cfg_.storage = LC2_STORE_F32;
    centered_ = c->IsCenterOverlaid;
    fixed_ = c->FixedBuffer;
    moving_ = c->MovingBuffer;
    configured_ = true;
    matrix_.assign({1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1});
  }

  void InitiateMappers() { mappers(3); }
  void InitiateRegistrationHandle() { handle(); }

  void GenerateMappers(float3 RotationAngle, float3 Translation) {
    GenerateMappers(RotationAngle, Translation, make_float3(1.0f, 1.0f, 1.0f),
                    make_float3(0.0f, 0.0f, 0.0f));
  }
  void GenerateMappers(float3 RotationAngle, float3 Translation, float3 scale, float3 shear) {
    const float r[3] = {RotationAngle.x, RotationAngle.y, RotationAngle.z};
    const float t[3] = {Translation.x, Translation.y, Translation.z};
    const float s[3] = {scale.x, scale.y, scale.z};
    const float h[3] = {shear.x, shear.y, shear.z};
    check(lc2_affine_3d(r, t, s, h, center_, shift_, matrix_.data()), "lc2_affine_3d");
  }

  // The resample is fused into GetSimilarityMeasure.
  void Interpolate(const int = 8, const int = 8, const int = 8) {}

  double GetSimilarityMeasure(const int patchSize = 3) { return measure(patchSize); }

  // inverse of the current virtual->moving matrix (VirtualToFixed is the identity)
  void GetCurrentTransform(float _t[16]) {
    check(lc2_invert_affine_3d(matrix_.data(), _t), "lc2_invert_affine_3d");
  }
  void GetMovingToFixedTransform(float3 RotationAngle, float3 Translation, float* out) {
    GenerateMappers(RotationAngle, Translation);
    GetCurrentTransform(out);
  }
  void GetMovingToFixedTransform(float3 RotationAngle, float3 Translation, float3 scale,
                                 float3 shear, float* out) {
    GenerateMappers(RotationAngle, Translation, scale, shear);
    GetCurrentTransform(out);
  }
};

// 2D frame (US, z = 1) against a 3D volume; the LC2 runs on the frame.
class Interpolator2DTo3D : public Interpolator3D {
 public:
  explicit Interpolator2DTo3D(const LC2Configuration2DTo3D* c)
      : Interpolator3D(c, LC2_MODE_2DTO3D) {}
};

// 2D registration.
class Interpolator2D : public InterpolatorBase {
 public:
  explicit Interpolator2D(const LC2Configuration2D* c) {
    if (!c || !c->IsConfigured) {
      std::printf("Please configure the Parameter file! \n");
      return;
    }
    cfg_.mode = LC2_MODE_2D;
    cfg_.fixed = {{c->FixedDimension.x, c->FixedDimension.y, 1},
                  {c->FixedSpacing.x, c->FixedSpacing.y, 1.0f},
                  {c->FixedOrigin.x, c->FixedOrigin.y, 0.0f}};
    cfg_.moving = {{c->MovingDimension.x, c->MovingDimension.y, 1},
                   {c->MovingSpacing.x, c->MovingSpacing.y, 1.0f},
                   {c->MovingOrigin.x, c->MovingOrigin.y, 0.0f}};
    cfg_.virtual_spacing[0] = c->SamplerSpacing.x;
    cfg_.virtual_spacing[1] = c->SamplerSpacing.y;
    cfg_.virtual_spacing[2] = 1.0f;
    cfg_.patch_size = c->PatchSize;
    cfg_.high_res_is_moving = c->IsMovingHighResolution ? 1 : 0;
    cfg_.storage = LC2_STORE_F32;
    centered_ = c->IsCenterOverlaid;
    fixed_ = c->FixedBuffer;
    moving_ = c->MovingBuffer;
    configured_ = true;
    matrix_.assign({1, 0, 0, 0, 1, 0, 0, 0, 1});
  }

  void InitiateMappers() { mappers(2); }
  void InitiateRegistrationHandle() { handle(); }

  void GenerateMappers(float RotationAngle, float2 Translation) {
    GenerateMappers(RotationAngle, Translation, make_float2(1.0f, 1.0f), 0.0f);
  }
  void GenerateMappers(float RotationAngle, float2 Translation, float2 scale, float shear) {
    const float t[2] = {Translation.x, Translation.y};
    const float s[2] = {scale.x, scale.y};
    check(lc2_affine_2d(RotationAngle, t, s, shear, center_, shift_, matrix_.data()),
          "lc2_affine_2d");
  }

  void Interpolate(const int = 8, const int = 8) {}

  double GetSimilarityMeasure(const int patchSize = 9) { return measure(patchSize); }

  void GetMovingToFixedTransform(float RotationAngle, float2 Translation, float2 scale,
                                 float shear, float* out) {
    GenerateMappers(RotationAngle, Translation, scale, shear);
    const float* m = matrix_.data();
    const double det = (double)m[0] * m[4] - (double)m[1] * m[3];
    if (det == 0.0) throw Error(LC2_ERR_SINGULAR, "singular transform");
    const double i00 = m[4] / det, i01 = -m[1] / det, i10 = -m[3] / det, i11 = m[0] / det;
    out[0] = (float)i00;
    out[1] = (float)i01;
    out[2] = (float)(-(i00 * m[2] + i01 * m[5]));
    out[3] = (float)i10;
    out[4] = (float)i11;
    out[5] = (float)(-(i10 * m[2] + i11 * m[5]));
    out[6] = 0.0f;
    out[7] = 0.0f;
    out[8] = 1.0f;
  }
};

}  // namespace lc2dropin

using lc2dropin::Interpolator2D;
using lc2dropin::Interpolator2DTo3D;
using lc2dropin::Interpolator3D;
