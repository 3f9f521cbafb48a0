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
#include "lc2_io.hpp"
#include "lc2_yaml.hpp"

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <ctime>
#include <fstream>
#include <sstream>

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

// ------------------------------------------------------------ volume I/O
// A float32 image/volume with its geometry (2D images: dim[2] = 1).
struct Volume {
  std::vector<float> data;
  int dim[3] = {1, 1, 1};
  float spacing[3] = {1.0f, 1.0f, 1.0f};
  float origin[3] = {0.0f, 0.0f, 0.0f};
};

// Raw float32, x fastest (readFromBin, src/Utilities/my_cuda_helper.cu:25-42).
inline std::vector<float> read_raw_floats(const std::string& path, size_t n) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Error(LC2_ERR_INVALID_ARGUMENT, "cannot open " + path);
  std::vector<float> v(n);
  f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(sizeof(float) * n));
  if (!f) throw Error(LC2_ERR_INVALID_ARGUMENT, "short read: " + path);
  return v;
}

// Minimal NRRD reader: raw encoding, little endian, scalar types, sizes,
// spacings or diagonal space directions, space origin, inline or detached
// data. (The reference reads NRRD through ITK, volumeImporter.cpp:42-93.)
inline Volume read_nrrd(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Error(LC2_ERR_INVALID_ARGUMENT, "cannot open " + path);
  std::string line;
  std::getline(f, line);
  if (line.rfind("NRRD", 0) != 0) throw Error(LC2_ERR_INVALID_ARGUMENT, path + ": not NRRD");
  std::string type = "float", encoding = "raw", endian = "little", datafile;
  int ndim = 0;
  Volume v;
  auto vec3 = [](const std::string& s, float* out, int n) {
    std::string t = s;
    for (char& c : t)
      if (c == '(' || c == ')' || c == ',') c = ' ';
    std::istringstream in(t);
    for (int i = 0; i < n; ++i) in >> out[i];
  };
  while (std::getline(f, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.empty()) break;
    if (line[0] == '#') continue;
    const size_t c = line.find(':');
    if (c == std::string::npos) continue;
    std::string key = line.substr(0, c), val = line.substr(c + 1);
    if (!val.empty() && val[0] == '=') val = val.substr(1);
    while (!val.empty() && val[0] == ' ') val.erase(0, 1);
    if (key == "type") type = val;
    else if (key == "dimension") ndim = std::atoi(val.c_str());
    else if (key == "sizes") {
      std::istringstream in(val);
      for (int i = 0; i < ndim && i < 3; ++i) in >> v.dim[i];
    } else if (key == "spacings") {
      std::istringstream in(val);
      for (int i = 0; i < ndim && i < 3; ++i) in >> v.spacing[i];
    } else if (key == "space directions") {
      float d[9] = {0};
      vec3(val, d, ndim * ndim);
      for (int i = 0; i < ndim && i < 3; ++i) v.spacing[i] = std::fabs(d[i * ndim + i]);
    } else if (key == "space origin") {
      vec3(val, v.origin, ndim);
    } else if (key == "encoding") encoding = val;
    else if (key == "endian") endian = val;
    else if (key == "data file" || key == "datafile") datafile = val;
  }
  if (encoding != "raw" || endian != "little")
    throw Error(LC2_ERR_UNSUPPORTED, path + ": only raw little-endian NRRD is supported");
  const size_t n = (size_t)v.dim[0] * v.dim[1] * v.dim[2];
  std::ifstream df;
  std::istream* in = &f;
  if (!datafile.empty()) {
    std::string dir = path.substr(0, path.find_last_of('/') + 1);
    df.open(datafile[0] == '/' ? datafile : dir + datafile, std::ios::binary);
    in = &df;
  }
  v.data.resize(n);
  auto rd = [&](auto tag) {
    using T = decltype(tag);
    std::vector<T> tmp(n);
    in->read(reinterpret_cast<char*>(tmp.data()), (std::streamsize)(sizeof(T) * n));
    if (!*in) throw Error(LC2_ERR_INVALID_ARGUMENT, path + ": short read");
    for (size_t i = 0; i < n; ++i) v.data[i] = (float)tmp[i];
  };
  if (type == "float") rd(float());
  else if (type == "double") rd(double());
  else if (type == "short" || type == "int16") rd(int16_t());
  else if (type == "ushort" || type == "unsigned short" || type == "uint16") rd(uint16_t());
  else if (type == "int" || type == "int32") rd(int32_t());
  else if (type == "uchar" || type == "unsigned char" || type == "uint8") rd(uint8_t());
  else throw Error(LC2_ERR_UNSUPPORTED, path + ": NRRD type " + type);
  return v;
}

// Volume from a FixedVolume / MovingVolume / FixedImage / MovingImage node:
// FilePath with Format raw (Dimension, Spacing, Origin given) or a .nrrd file
// (geometry from its header, overridden by the node where given).
inline Volume load_volume(const lc2yaml::Node& d, int nd) {
  const std::string path = d["FilePath"].str();
  Volume v;
  const bool nrrd = path.size() > 5 && path.substr(path.size() - 5) == ".nrrd";
  if (!nrrd && !d["Dimension"])
    throw Error(LC2_ERR_UNSUPPORTED, path + ": only raw (with Dimension) and .nrrd are supported");
  if (nrrd) v = read_nrrd(path);
  static const char* ax[3] = {"x", "y", "z"};
  for (int a = 0; a < nd; ++a) {
    if (d["Dimension"][ax[a]]) v.dim[a] = d["Dimension"][ax[a]].integer();
    if (d["Spacing"][ax[a]]) v.spacing[a] = (float)d["Spacing"][ax[a]].num();
    if (d["Origin"][ax[a]]) v.origin[a] = (float)d["Origin"][ax[a]].num();
  }
  if (!nrrd) v.data = read_raw_floats(path, (size_t)v.dim[0] * v.dim[1] * v.dim[2]);
  return v;
}

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
  Volume fixed_vol_, moving_vol_;  // owned images (parameter-file constructors)
  std::string output_path_;
  std::string fixed_path_, moving_path_;  // FilePath of the parameter file, if any

 public:
  // Mapper centre and shift of InitiateMappers (for the registration driver).
  const float* Center() const { return center_; }
  const float* Shift() const { return shift_; }
  int Mode() const { return cfg_.mode; }
  int PatchSize() const { return cfg_.patch_size; }

 protected:

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

  // From a parameter file (Interpolator3D(yaml, useIGTL), interpolator.cu:234-391;
  // Interpolator2DTo3D(yaml), :1538-1623). The pose side channel is not part of
  // this path; useIGTL is accepted and ignored.
  explicit Interpolator3D(const std::string& yaml_path, bool useIGTL = false,
                          int mode = LC2_MODE_3D) {
    (void)useIGTL;
    const lc2yaml::Node y = lc2yaml::load_file(yaml_path);
    const lc2yaml::Node& in = y["InputParameters"];
    const lc2yaml::Node& rp = in["RegistrationParameters"];
    fixed_vol_ = load_volume(in["FixedVolume"], 3);
    moving_vol_ = load_volume(in["MovingVolume"], 3);
    fixed_path_ = in["FixedVolume"]["FilePath"].str();
    moving_path_ = in["MovingVolume"]["FilePath"].str();
    cfg_.mode = mode;
    for (int a = 0; a < 3; ++a) {
      cfg_.fixed.dim[a] = fixed_vol_.dim[a];
      cfg_.fixed.spacing[a] = fixed_vol_.spacing[a];
      cfg_.fixed.origin[a] = fixed_vol_.origin[a];
      cfg_.moving.dim[a] = moving_vol_.dim[a];
      cfg_.moving.spacing[a] = moving_vol_.spacing[a];
      cfg_.moving.origin[a] = moving_vol_.origin[a];
    }
    static const char* ax[3] = {"x", "y", "z"};
    for (int a = 0; a < 3; ++a)
      cfg_.virtual_spacing[a] = (float)rp["ResampledSpacing"][ax[a]].num();
    cfg_.patch_size = rp["PatchSize"].integer();
    cfg_.high_res_is_moving = rp["HighResolutionModality"].str() == "Moving" ? 1 : 0;
    cfg_.storage = LC2_STORE_F32;
    centered_ = rp["CenterOverlaid"].boolean();
    if (rp["FinalRoundExportRootPath"]) output_path_ = rp["FinalRoundExportRootPath"].str();
    fixed_ = fixed_vol_.data.data();
    moving_ = moving_vol_.data.data();
    configured_ = true;
    matrix_.assign({1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1});
  }

  std::string GetOutputPath() { return output_path_; }

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

  // Virtual-grid volumes of the current transform (interpolator.cu:681-729):
  // <fixed name>.nrrd holds the high-resolution image, <moving name>_Registered.nrrd
  // the ultrasound, both at the virtual spacing with origin (0,0,0).
  void WriteOut() {
    if (!handle_ready_) throw Error(LC2_ERR_NOT_READY, "InitiateRegistrationHandle not called");
    int d[3];
    check(lc2_virtual_dims(ctx_.get(), d), "lc2_virtual_dims");
    const size_t n = (size_t)d[0] * d[1] * d[2];
    std::vector<float> U(n), M(n);
    double v = 0.0;
    check(lc2_evaluate_fields(ctx_.get(), matrix_.data(), &v, U.data(), M.data(), nullptr,
                              nullptr, nullptr),
          "lc2_evaluate_fields");
    lc2io::NrrdHeader h{};
    for (int a = 0; a < 3; ++a) {
      h.sizes[a] = d[a];
      h.directions[a][a] = cfg_.virtual_spacing[a];
    }
    lc2io::write_nrrd(output_path_ + lc2io::stem_with_slash(fixed_path_, "fixed") + ".nrrd", h,
                      M.data());
    lc2io::write_nrrd(
        output_path_ + lc2io::stem_with_slash(moving_path_, "moving") + "_Registered.nrrd", h,
        U.data());
  }

  // The moving volume with the optimal moving->fixed matrix applied to its
  // axes and origin, <moving name>_Registered.nrrd, and the matrix itself as
  // MovingToFixed.mat (interpolator.cu:738-849). Float accumulation in the
  // reference's order.
  void WriteOut(float* OptimizedMatrix) {
    const float* m = OptimizedMatrix;
    lc2io::NrrdHeader h{};
    for (int a = 0; a < 3; ++a) h.sizes[a] = cfg_.moving.dim[a];
    for (int a = 0; a < 3; ++a) {  // axis a: M * (spacing_a e_a)
      float axis[3] = {0.0f, 0.0f, 0.0f};
      axis[a] = cfg_.moving.spacing[a];
      for (int row = 0; row < 3; ++row) {
        float acc = 0.0f;
        for (int e = 0; e < 3; ++e) acc += m[e + row * 4] * axis[e];
        h.directions[a][row] = acc;
      }
    }
    const float o4[4] = {cfg_.moving.origin[0], cfg_.moving.origin[1], cfg_.moving.origin[2],
                         1.0f};
    for (int row = 0; row < 3; ++row) {
      float acc = 0.0f;
      for (int e = 0; e < 4; ++e) acc += m[e + row * 4] * o4[e];
      h.origin[row] = acc;
    }
    if (!moving_) throw Error(LC2_ERR_NOT_READY, "no moving volume");
    lc2io::write_nrrd(
        output_path_ + lc2io::stem_with_slash(moving_path_, "moving") + "_Registered.nrrd", h,
        moving_);
    lc2io::write_matrix(output_path_ + "/MovingToFixed.mat", m, 4, 4);
  }
};

// 2D frame (US, z = 1) against a 3D volume; the LC2 runs on the frame.
class Interpolator2DTo3D : public Interpolator3D {
 public:
  explicit Interpolator2DTo3D(const LC2Configuration2DTo3D* c)
      : Interpolator3D(c, LC2_MODE_2DTO3D) {}
  explicit Interpolator2DTo3D(const std::string& yaml_path)
      : Interpolator3D(yaml_path, false, LC2_MODE_2DTO3D) {}
  // the reference writes nothing here (interpolator.cu:1777-1785)
  void WriteOut() {}
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

  // From a parameter file (Interpolator2D(yaml), interpolator.cu:979-1103).
  explicit Interpolator2D(const std::string& yaml_path) {
    const lc2yaml::Node y = lc2yaml::load_file(yaml_path);
    const lc2yaml::Node& in = y["InputParameters"];
    const lc2yaml::Node& rp = in["RegistrationParameters"];
    fixed_vol_ = load_volume(in["FixedImage"], 2);
    moving_vol_ = load_volume(in["MovingImage"], 2);
    fixed_path_ = in["FixedImage"]["FilePath"].str();
    moving_path_ = in["MovingImage"]["FilePath"].str();
    cfg_.mode = LC2_MODE_2D;
    for (int a = 0; a < 2; ++a) {
      cfg_.fixed.dim[a] = fixed_vol_.dim[a];
      cfg_.fixed.spacing[a] = fixed_vol_.spacing[a];
      cfg_.fixed.origin[a] = fixed_vol_.origin[a];
      cfg_.moving.dim[a] = moving_vol_.dim[a];
      cfg_.moving.spacing[a] = moving_vol_.spacing[a];
      cfg_.moving.origin[a] = moving_vol_.origin[a];
    }
    cfg_.fixed.dim[2] = cfg_.moving.dim[2] = 1;
    cfg_.fixed.spacing[2] = cfg_.moving.spacing[2] = 1.0f;
    cfg_.virtual_spacing[0] = (float)rp["ResampledSpacing"]["x"].num();
    cfg_.virtual_spacing[1] = (float)rp["ResampledSpacing"]["y"].num();
    cfg_.virtual_spacing[2] = 1.0f;
    cfg_.patch_size = rp["PatchSize"].integer();
    cfg_.high_res_is_moving = rp["HighResolutionModality"].str() == "Moving" ? 1 : 0;
    cfg_.storage = LC2_STORE_F32;
    centered_ = rp["CenterOverlaid"].boolean();
    if (rp["FinalRoundExportRootPath"]) output_path_ = rp["FinalRoundExportRootPath"].str();
    fixed_ = fixed_vol_.data.data();
    moving_ = moving_vol_.data.data();
    configured_ = true;
    matrix_.assign({1, 0, 0, 0, 1, 0, 0, 0, 1});
  }

  std::string GetOutputPath() { return output_path_; }

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

  // the reference writes nothing here (interpolator.cu:1427-1436)
  void WriteOut() {}

  // The moving image registered into the fixed image's pixel grid with the
  // optimal moving->fixed matrix, converted to pixel units exactly as the
  // reference does (interpolator.cu:1438-1535), written as
  // <moving name>_Registered.png (values rounded, outside [0, 255] -> 0) or,
  // when a value exceeds 255, as raw float32 <moving name>_Registered.raw.
  // Returns the path written.
  std::string WriteOut(float* OptimizedMatrix) {
    if (!moving_) throw Error(LC2_ERR_NOT_READY, "no moving image");
    double A[2][3];
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 3; ++j) A[i][j] = OptimizedMatrix[j + i * 3];
    const lc2_geometry& F = cfg_.fixed;
    const lc2_geometry& Mv = cfg_.moving;
    A[0][2] /= F.spacing[0];
    A[1][2] /= F.spacing[1];
    A[0][0] *= (Mv.spacing[0] / F.spacing[0]);
    A[1][0] *= (Mv.spacing[0] / F.spacing[0]);
    A[0][1] *= (Mv.spacing[1] / F.spacing[1]);
    A[1][1] *= (Mv.spacing[1] / F.spacing[1]);
    const double coeffs[6] = {A[0][0], A[0][1], A[0][2], A[1][0], A[1][1], A[1][2]};
    const int fw = F.dim[0], fh = F.dim[1];
    std::vector<float> reg((size_t)fw * fh);
    check(lc2_warp_affine_2d(moving_, Mv.dim[0], Mv.dim[1], reg.data(), fw, fh, coeffs,
                             cfg_.device),
          "lc2_warp_affine_2d");
    float mx = reg.empty() ? 0.0f : reg[0];
    for (float v : reg) mx = std::max(mx, v);
    const std::string base = output_path_ + lc2io::stem_with_slash(moving_path_, "moving");
    if (mx > 255.0f) {
      const std::string path = base + "_Registered.raw";
      std::ofstream f(path, std::ios::out | std::ios::binary);
      if (!f) throw Error(LC2_ERR_INVALID_ARGUMENT, "cannot write " + path);
      f.write(reinterpret_cast<const char*>(reg.data()),
              (std::streamsize)(reg.size() * sizeof(float)));
      return path;
    }
    std::vector<uint8_t> px(reg.size());
    for (size_t i = 0; i < reg.size(); ++i) {
      const float v = reg[i];
      px[i] = (v > 255.0f || v < 0.0f) ? 0 : (uint8_t)std::roundf(v);
    }
    const std::string path = base + "_Registered.png";
    lc2io::write_png_gray8(path, fw, fh, px.data());
    return path;
  }
};

}  // namespace lc2dropin

using lc2dropin::Interpolator2D;
using lc2dropin::Interpolator2DTo3D;
using lc2dropin::Interpolator3D;
