// Drives LC2_3D_class / LC2_2D_class (include/lc2_cu_lc2.hpp) with the calls
// and default arguments of the reference's headers (src/cu_LC2/cu_lc2_3d.cuh:
// 14-49, src/cu_LC2/cu_lc2_2d.cuh:14-40), the way its interpolators call them
// (src/Interpolator/interpolator.cu:532, 618-630, 1237, 1344-1379).
//
//   lc2_class_eval <3D|2D> <x> <y> <z> <patch> <us.raw> <hr.raw> <outdir>
// Prints, one per line: the LC2 of the object built from host vectors, the
// LC2 of the interpolator-style object filled through device pointers (2D)
// or of an object with zeroed buffers (3D), and in 3D the mutual information.
// Writes the gradient (grad.raw) and, in 3D, the weighting map (wmap.raw).
#include <cuda_runtime_api.h>

#include <cstdio>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "lc2_cu_lc2.hpp"

static std::vector<float> read_raw(const std::string& path, size_t n) {
  std::vector<float> v(n);
  std::ifstream f(path, std::ios::binary);
  f.read(reinterpret_cast<char*>(v.data()), sizeof(float) * n);
  if (!f) throw std::runtime_error("cannot read " + path);
  return v;
}

static void write_raw(const std::string& path, const std::vector<float>& v) {
  std::ofstream f(path, std::ios::binary);
  f.write(reinterpret_cast<const char*>(v.data()), sizeof(float) * v.size());
}

int main(int argc, char** argv) {
  if (argc < 9) {
    std::fprintf(stderr, "usage: lc2_class_eval 3D|2D x y z patch us.raw hr.raw outdir\n");
    return 2;
  }
  const std::string mode = argv[1];
  const int x = std::atoi(argv[2]), y = std::atoi(argv[3]), z = std::atoi(argv[4]);
  const int patch = std::atoi(argv[5]);
  const std::string out = argv[8];
  const size_t n = (size_t)x * y * (mode == "3D" ? z : 1);
  std::vector<float> us = read_raw(argv[6], n), hr = read_raw(argv[7], n);
  if (mode == "3D") {
    LC2_3D_class lc2(x, y, z, us, hr);
    lc2.PrepareGradientFilter();
    lc2.CalculateGradient();
    const double v = lc2.GetSimilarityMetric(8, 8, 8, patch);
    const double mi = lc2.GetMutualInformationSimilarityMetric();
    lc2.GenerateWeightingMap();
    write_raw(out + "/wmap.raw", lc2.GetWeightedMapBuffer());
    write_raw(out + "/grad.raw", lc2.GetHighResolutionGradientBuffer());
    // the interpolator's form: default-constructed, sized to the virtual grid
    std::unique_ptr<LC2_3D_class> held = std::make_unique<LC2_3D_class>();
    held->PortedFromInterpolator(x, y, z);
    held->ShowImages(0);
    const double zero = held->GetSimilarityMetric(8, 8, 8, patch);
    std::printf("%.17g\n%.17g\n%.17g\n", v, zero, mi);
  } else {
    LC2_2D_class lc2(x, y, us, hr);
    const double v = lc2.GetSimilarityMetric(16, 16, patch);
    // the interpolator's form: buffers filled on the device through the raw pointers
    std::unique_ptr<LC2_2D_class> held = std::make_unique<LC2_2D_class>();
    held->PortedFromInterpolator(x, y);
    cudaMemcpy(held->GetUltrasoundRawPointer(), us.data(), n * sizeof(float),
               cudaMemcpyHostToDevice);
    cudaMemcpy(held->GetHighResolutionRawPointer(), hr.data(), n * sizeof(float),
               cudaMemcpyHostToDevice);
    held->ShowImages(0);
    held->PrepareGradientFilter();
    held->CalculateGradient();
    const double w = held->GetSimilarityMetric(16, 16, patch);
    std::vector<float> g(n);
    cudaMemcpy(g.data(), held->GetHighResolutionGradientRawPointer(), n * sizeof(float),
               cudaMemcpyDeviceToHost);
    write_raw(out + "/grad.raw", g);
    std::printf("%.17g\n%.17g\n", v, w);
  }
  return 0;
}
