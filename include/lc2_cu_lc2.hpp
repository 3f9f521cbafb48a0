// lc2_cu_lc2.hpp -- the reference's LC2 similarity objects, LC2_3D_class and
// LC2_2D_class, over the C ABI (lc2.h).
//
// Same class names, constructors, methods and default arguments as
// src/cu_LC2/cu_lc2_3d.cuh:10-92 and src/cu_LC2/cu_lc2_2d.cuh:10-81, so code
// written against those headers -- `std::unique_ptr<LC2_3D_class>` as in
// src/Interpolator/interpolator.cuh:63, or an object built from two host
// volumes -- compiles against this one. Like the reference objects, each
// holds its images in device memory on the current CUDA device:
//
//   Ultrasound      U, the fixed/ultrasound image on the (virtual) grid;
//   HighResolution  M, the resampled high-resolution image on the same grid;
//   gradient        |Sobel M| (written by CalculateGradient);
//   weighting map   measure / sigma (written by GenerateWeightingMap).
//
// GetSimilarityMetric evaluates LC2 of whatever U and M hold (the 2D object's
// Get*RawPointer return those device pointers, which callers fill with their
// own kernels or copies, as Interpolator2D::Interpolate does at
// src/Interpolator/interpolator.cu:1344-1360). Each evaluation hands the two
// buffers to a library context over the same grid (lc2_set_images_device)
// and evaluates the identity transform: resampling M at integer positions
// returns M unchanged, so the value is LC2 of (U, M) as the reference
// defines it, computed by the library's fused kernels with exact patch sums.
//
// What differs by design:
//   * block-size arguments are accepted and ignored (the library chooses its
//     own tiles); PrepareGradientFilter has nothing to upload (the Sobel taps
//     are compile-time constants of the kernels);
//   * Get*Buffer of the 3D object return host copies (std::vector<float>)
//     instead of thrust::device_vector<float> by value; a thrust vector can be
//     constructed from either;
//   * ShowImages draws nothing (no display on a headless GPU host);
//   * GetMutualInformationSimilarityMetric supports 256 bins per image only
//     (the reference's defaults); other counts throw lc2dropin::Error;
//   * failures throw lc2dropin::Error (the reference checks no status);
//   * SaveResults writes registration.bin in the working directory (the
//     reference writes a fixed path of its author's machine).
//
// Needs the CUDA runtime (link -lcudart) besides liblc2.
#pragma once

#include <cuda_runtime_api.h>

#include <cmath>
#include <cstdio>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "lc2.h"
#include "lc2_dropin.hpp"

namespace lc2dropin {

inline void cuda_check(cudaError_t e, const char* where) {
  if (e != cudaSuccess)
    throw Error(LC2_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// One float buffer in device memory of the current device.
class DeviceFloats {
 public:
  DeviceFloats() = default;
  DeviceFloats(const DeviceFloats&) = delete;
  DeviceFloats& operator=(const DeviceFloats&) = delete;
  ~DeviceFloats() { release(); }
  void resize(size_t n, float fill = 0.0f) {
    if (n != n_) {
      release();
      if (n) cuda_check(cudaMalloc(reinterpret_cast<void**>(&p_), n * sizeof(float)), "cudaMalloc");
      n_ = n;
    }
    if (n) upload(std::vector<float>(n, fill).data());
  }
  void upload(const float* host) {
    cuda_check(cudaMemcpy(p_, host, n_ * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy");
  }
  void copy_from(const DeviceFloats& o) {
    resize(o.n_);
    cuda_check(cudaMemcpy(p_, o.p_, n_ * sizeof(float), cudaMemcpyDeviceToDevice), "cudaMemcpy");
  }
  std::vector<float> download() const {
    std::vector<float> h(n_);
    if (n_)
      cuda_check(cudaMemcpy(h.data(), p_, n_ * sizeof(float), cudaMemcpyDeviceToHost), "cudaMemcpy");
    return h;
  }
  float* data() const { return p_; }
  size_t size() const { return n_; }

 private:
  void release() {
    if (p_) cudaFree(p_);
    p_ = nullptr;
    n_ = 0;
  }
  float* p_ = nullptr;
  size_t n_ = 0;
};

// The state both objects share: grid, device buffers and one library context
// per patch size (0 = mutual information), evaluated at the identity.
class GridSimilarity {
 public:
  void set_grid(int nd, int x, int y, int z) {
    nd_ = nd;
    dim_[0] = x;
    dim_[1] = y;
    dim_[2] = (nd == 3) ? z : 1;
    ctx_.clear();
    last_patch_ = 0;
  }
  size_t voxels() const { return (size_t)dim_[0] * dim_[1] * dim_[2]; }

  // LC2 (patch > 0) or normalised mutual information (patch 0) of (U, M)
  double evaluate(int patch, const float* U, const float* M) {
    lc2_context* c = context(patch);
    check(lc2_set_images_device(c, U, M), "lc2_set_images_device");
    double v = 0.0;
    check(lc2_evaluate(c, identity(), &v), "lc2_evaluate");
    if (patch > 0) last_patch_ = patch;
    return v;
  }
  // |Sobel M| of the same evaluation, written to G (device)
  void gradient(const float* U, const float* M, DeviceFloats& G) {
    lc2_context* c = context(last_patch_ > 0 ? last_patch_ : 1);
    check(lc2_set_images_device(c, U, M), "lc2_set_images_device");
    std::vector<float> g(voxels());
    double v = 0.0;
    check(lc2_evaluate_fields(c, identity(), &v, nullptr, nullptr, g.data(), nullptr, nullptr),
          "lc2_evaluate_fields");
    G.resize(voxels());
    G.upload(g.data());
  }
  // measure / sigma of (U, M) at the last LC2 evaluation's patch size,
  // written to W (device)
  void weighting_map(const float* U, const float* M, DeviceFloats& W) {
    if (last_patch_ <= 0)
      throw Error(LC2_ERR_NOT_READY, "GenerateWeightingMap: no LC2 evaluation yet");
    lc2_context* c = context(last_patch_);
    check(lc2_set_images_device(c, U, M), "lc2_set_images_device");
    std::vector<float> w(voxels());
    check(lc2_weighting_map(c, identity(), nullptr, w.data()), "lc2_weighting_map");
    W.resize(voxels());
    W.upload(w.data());
  }
  // src warped by the voxel-space map dst -> src `mat` (row-major 4x4) with
  // the library's trilinear sampling (0 outside), written to dst (device)
  void warp(const float* src, const float mat[16], DeviceFloats& dst) {
    lc2_context* c = context(last_patch_ > 0 ? last_patch_ : 1);
    check(lc2_set_images_device(c, src, src), "lc2_set_images_device");
    std::vector<float> m(voxels());
    double v = 0.0;
    check(lc2_evaluate_fields(c, mat, &v, nullptr, m.data(), nullptr, nullptr, nullptr),
          "lc2_evaluate_fields");
    dst.resize(voxels());
    dst.upload(m.data());
  }

 private:
  const float* identity() const {
    static const float id3[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    static const float id2[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    return nd_ == 3 ? id3 : id2;
  }
  lc2_context* context(int patch) {
    auto it = ctx_.find(patch);
    if (it != ctx_.end()) return it->second->get();
    lc2_config cfg{};
    cfg.mode = nd_ == 3 ? LC2_MODE_3D : LC2_MODE_2D;
    for (int a = 0; a < 3; ++a) {
      cfg.fixed.dim[a] = cfg.moving.dim[a] = dim_[a];
      cfg.fixed.spacing[a] = cfg.moving.spacing[a] = 1.0f;
      cfg.fixed.origin[a] = cfg.moving.origin[a] = 0.0f;
      cfg.virtual_spacing[a] = 1.0f;
    }
    cfg.patch_size = patch;
    cfg.high_res_is_moving = 1;
    cfg.storage = LC2_STORE_F32;
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    cfg.device = dev;
    std::unique_ptr<Context> c(new Context());
    c->create(cfg);
    lc2_context* h = c->get();
    ctx_[patch] = std::move(c);
    return h;
  }

  int nd_ = 3;
  int dim_[3] = {0, 0, 0};
  int last_patch_ = 0;
  std::map<int, std::unique_ptr<Context>> ctx_;  // by patch size, 0 = mutual information
};

}  // namespace lc2dropin

// LC2_3D_class (src/cu_LC2/cu_lc2_3d.cuh:10-92).
class LC2_3D_class {
 public:
  // cu_lc2_3d.cu:926-940: both volumes on one x*y*z grid
  LC2_3D_class(int x, int y, int z, std::vector<float>& UltrasoundVolume_Extern,
               std::vector<float>& HighResoVolume_Extern) {
    PortedFromInterpolator(x, y, z);
    const size_t n = grid_.voxels();
    if (UltrasoundVolume_Extern.size() != n || HighResoVolume_Extern.size() != n)
      throw lc2dropin::Error(LC2_ERR_INVALID_ARGUMENT, "LC2_3D_class: volume sizes != x*y*z");
    us_static_.upload(UltrasoundVolume_Extern.data());
    us_.upload(UltrasoundVolume_Extern.data());
    hr_.upload(HighResoVolume_Extern.data());
  }
  LC2_3D_class() {}
  virtual ~LC2_3D_class() = default;

  // cu_lc2_3d.cu:942-975: zeroed buffers of the interpolator's virtual grid
  void PortedFromInterpolator(int x, int y, int z) {
    dim_[0] = x;
    dim_[1] = y;
    dim_[2] = z;
    grid_.set_grid(3, x, y, z);
    const size_t n = grid_.voxels();
    us_static_.resize(n);
    us_.resize(n);
    hr_.resize(n);
    grad_.resize(n);
    wmap_.resize(n);
  }

  // cu_lc2_3d.cu:1035-1117: the static ultrasound rotated about the volume
  // centre (degrees, X then Y then Z), translated, the diagonal scaled, and
  // written to the current ultrasound
  void warpVolume(float Rx, float Ry, float Rz, float Tx, float Ty, float Tz, float Scaling,
                  const int Blk_Dim_x = 8, const int Blk_Dim_y = 8, const int Blk_Dim_z = 8) {
    (void)Blk_Dim_x; (void)Blk_Dim_y; (void)Blk_Dim_z;
    const double d2r = M_PI / 180.0;
    const float cx = (float)std::cos(Rx * d2r), sx = (float)std::sin(Rx * d2r);
    const float cy = (float)std::cos(Ry * d2r), sy = (float)std::sin(Ry * d2r);
    const float cz = (float)std::cos(Rz * d2r), sz = (float)std::sin(Rz * d2r);
    const float R[3][3] = {{cz * cy, cz * sy * sx - sz * cx, cz * sy * cx + sz * sx},
                           {sz * cy, sz * sy * sx + cz * cx, sz * sy * cx - cz * sx},
                           {-sy, cy * sx, cy * cx}};
    const float half[3] = {dim_[0] / 2.0f, dim_[1] / 2.0f, dim_[2] / 2.0f};
    const float T[3] = {Tx, Ty, Tz};
    float fwd[16] = {0};
    for (int a = 0; a < 3; ++a) {
      float t = half[a] + T[a];
      for (int b = 0; b < 3; ++b) {
        fwd[4 * a + b] = R[a][b];
        t -= R[a][b] * half[b];
      }
      fwd[4 * a + 3] = t;
    }
    fwd[15] = 1.0f;
    fwd[0] *= Scaling;
    fwd[5] *= Scaling;
    fwd[10] *= Scaling;
    float inv[16];
    if (lc2_invert_affine_3d(fwd, inv) != LC2_OK) {
      std::printf("Transform matrix is invalid. \n");
      return;
    }
    // destination voxel p samples the source at inv (p + 1) - 1
    for (int a = 0; a < 3; ++a) inv[4 * a + 3] += inv[4 * a] + inv[4 * a + 1] + inv[4 * a + 2] - 1.0f;
    grid_.warp(us_static_.data(), inv, us_);
  }

  void PrepareGradientFilter() {}
  void CalculateGradient(const int Blk_Dim_x = 8, const int Blk_Dim_y = 8,
                         const int Blk_Dim_z = 8) {
    (void)Blk_Dim_x; (void)Blk_Dim_y; (void)Blk_Dim_z;
    grid_.gradient(us_.data(), hr_.data(), grad_);
  }

  // cu_lc2_3d.cu:1119-1194
  double GetSimilarityMetric(const int Blk_Dim_x = 8, const int Blk_Dim_y = 8,
                             const int Blk_Dim_z = 8, const int patchSize = 3) {
    (void)Blk_Dim_x; (void)Blk_Dim_y; (void)Blk_Dim_z;
    return grid_.evaluate(patchSize, us_.data(), hr_.data());
  }

  // cu_lc2_3d.cu:1196-1301
  double GetMutualInformationSimilarityMetric(const int Blk_Dim_x = 8, const int Blk_Dim_y = 8,
                                              const int Blk_Dim_z = 8,
                                              const int bins_usVolume = 256,
                                              const int bins_highResoVolume = 256) {
    (void)Blk_Dim_x; (void)Blk_Dim_y; (void)Blk_Dim_z;
    if (bins_usVolume != 256 || bins_highResoVolume != 256)
      throw lc2dropin::Error(LC2_ERR_UNSUPPORTED, "mutual information: 256 bins per image only");
    return grid_.evaluate(0, us_.data(), hr_.data());
  }

  // cu_lc2_3d.cu:1303-1329 (from the last GetSimilarityMetric's patch size)
  void GenerateWeightingMap() { grid_.weighting_map(us_.data(), hr_.data(), wmap_); }
  std::vector<float> GetWeightedMapBuffer() { return wmap_.download(); }
  std::vector<float> GetUltrasoundBuffer() { return us_.download(); }
  std::vector<float> GetHighResolutionBuffer() { return hr_.download(); }
  std::vector<float> GetHighResolutionGradientBuffer() { return grad_.download(); }

  virtual void ShowImages(int display_pattern = 0) { (void)display_pattern; }

 protected:
  // device buffers the reference keeps as Ultrasound_volume and
  // HighResolution_volume_static (cu_lc2_3d.cuh:64-66)
  lc2dropin::DeviceFloats us_, hr_;

 private:
  lc2dropin::GridSimilarity grid_;
  lc2dropin::DeviceFloats us_static_, grad_, wmap_;
  int dim_[3] = {0, 0, 0};
};

// LC2_2D_class (src/cu_LC2/cu_lc2_2d.cuh:10-81).
class LC2_2D_class {
 public:
  // cu_lc2_2d.cu:484-513
  LC2_2D_class(int x, int y, std::vector<float>& Ultrasound_Extern,
               std::vector<float>& HighReso_Extern) {
    PortedFromInterpolator(x, y);
    const size_t n = grid_.voxels();
    if (Ultrasound_Extern.size() != n || HighReso_Extern.size() != n)
      throw lc2dropin::Error(LC2_ERR_INVALID_ARGUMENT, "LC2_2D_class: image sizes != x*y");
    us_static_.upload(Ultrasound_Extern.data());
    us_.upload(Ultrasound_Extern.data());
    hr_.upload(HighReso_Extern.data());
  }
  LC2_2D_class() {}
  virtual ~LC2_2D_class() = default;

  // cu_lc2_2d.cu:515-546
  void PortedFromInterpolator(int x, int y) {
    x_ = x;
    y_ = y;
    grid_.set_grid(2, x, y, 1);
    const size_t n = grid_.voxels();
    us_static_.resize(n);
    us_.resize(n);
    hr_.resize(n);
    grad_.resize(n);
  }

  void PrepareGradientFilter() {}
  void CalculateGradient(const int Blk_Dim_x = 16, const int Blk_Dim_y = 16) {
    (void)Blk_Dim_x; (void)Blk_Dim_y;
    grid_.gradient(us_.data(), hr_.data(), grad_);
  }

  // cu_lc2_2d.cu:599-653
  double GetSimilarityMetric(const int Blk_Dim_x = 16, const int Blk_Dim_y = 16,
                             const int patchSize = 9) {
    (void)Blk_Dim_x; (void)Blk_Dim_y;
    return grid_.evaluate(patchSize, us_.data(), hr_.data());
  }

  virtual void ShowImages(int display_pattern = 0) { (void)display_pattern; }

  // cu_lc2_2d.cu:821-831: device pointers of the current buffers
  float* GetUltrasoundRawPointer() { return us_.data(); }
  float* GetHighResolutionRawPointer() { return hr_.data(); }
  float* GetHighResolutionGradientRawPointer() { return grad_.data(); }

  // cu_lc2_2d.cu:833-908: the static ultrasound rotated by pi * R about the
  // centre of a 100-pixel frame and shifted by (T_x, T_y) * 99 pixels -- the
  // reference's constants -- written to the current ultrasound
  void UpdateImageAffine(double T_x, double T_y, double R) { warp_us(T_x, T_y, R, false); }
  // cu_lc2_2d.cu:910-981: the same, also replacing the static ultrasound
  void UpdateOrigImageAffine(double T_x, double T_y, double R) { warp_us(T_x, T_y, R, true); }

  // cu_lc2_2d.cu:983-987: the current ultrasound as raw float32
  void SaveResults() {
    std::vector<float> h = us_.download();
    FILE* f = std::fopen("registration.bin", "wb");
    if (!f) throw lc2dropin::Error(LC2_ERR_INVALID_ARGUMENT, "cannot write registration.bin");
    std::fwrite(h.data(), sizeof(float), h.size(), f);
    std::fclose(f);
  }

 protected:
  // device buffers the reference keeps as Ultrasound and
  // HighResolution_static (cu_lc2_2d.cuh:56-58)
  lc2dropin::DeviceFloats us_, hr_;

 private:
  void warp_us(double T_x, double T_y, double Rotation_ratio, bool replace_static) {
    const double R = M_PI * Rotation_ratio, s = std::sin(R), c = std::cos(R);
    const double h = (100 - 1) / 2.0;
    const double C[6] = {c, -s, -(h * c) + (h * s) + h + T_x * (100 - 1),
                         s, c, -(h * s) - (h * c) + h + T_y * (100 - 1)};
    std::vector<float> src = us_static_.download(), dst(src.size());
    int dev = 0;
    lc2dropin::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    lc2dropin::check(lc2_warp_affine_2d(src.data(), x_, y_, dst.data(), x_, y_, C, dev),
                     "lc2_warp_affine_2d");
    us_.upload(dst.data());
    if (replace_static) us_static_.upload(dst.data());
  }

  int x_ = 0, y_ = 0;
  lc2dropin::GridSimilarity grid_;
  lc2dropin::DeviceFloats us_static_, grad_;
};
