// Drives the reference-facing C++ classes (include/lc2_dropin.hpp) the way
// the reference's Optimizers3D::operator() does (src/Optimizers/optimizers.cu:
// 650-728): GenerateMappers -> Interpolate -> GetSimilarityMeasure, for a
// list of parameter vectors read from a text file.
//
//   dropin_eval <spec.txt>
// spec.txt: mode (3D|2D) / fixed dims spacing origin / moving dims spacing
// origin / virtual spacing / patch / hr_moving / centred / fixed.raw /
// moving.raw / then one parameter vector per line (3D: TX TY TZ RX RY RZ SX SY
// SZ HX HY HZ; 2D: TX TY R SX SY H). Prints one LC2 value per line.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "lc2_dropin.hpp"

static std::vector<float> read_raw(const std::string& path, size_t n) {
  std::vector<float> v(n);
  std::ifstream f(path, std::ios::binary);
  f.read(reinterpret_cast<char*>(v.data()), sizeof(float) * n);
  if (!f) throw std::runtime_error("cannot read " + path);
  return v;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    // unconfigured construction: the reference prints this and continues
    LC2Configuration3D c;
    Interpolator3D probe(&c);
    return 0;
  }
  std::ifstream in(argv[1]);
  std::string mode;
  in >> mode;
  int fd[3], md[3], patch, hrm, centred;
  float fs[3], fo[3], ms[3], mo[3], vs[3];
  for (int a = 0; a < 3; ++a) in >> fd[a];
  for (int a = 0; a < 3; ++a) in >> fs[a];
  for (int a = 0; a < 3; ++a) in >> fo[a];
  for (int a = 0; a < 3; ++a) in >> md[a];
  for (int a = 0; a < 3; ++a) in >> ms[a];
  for (int a = 0; a < 3; ++a) in >> mo[a];
  for (int a = 0; a < 3; ++a) in >> vs[a];
  in >> patch >> hrm >> centred;
  std::string fpath, mpath;
  in >> fpath >> mpath;
  std::vector<float> fixed = read_raw(fpath, (size_t)fd[0] * fd[1] * fd[2]);
  std::vector<float> moving = read_raw(mpath, (size_t)md[0] * md[1] * md[2]);
  try {
    if (mode == "3D") {
      LC2Configuration3D c;
      c.FixedDimension = {fd[0], fd[1], fd[2]};
      c.FixedSpacing = {fs[0], fs[1], fs[2]};
      c.FixedOrigin = {fo[0], fo[1], fo[2]};
      c.MovingDimension = {md[0], md[1], md[2]};
      c.MovingSpacing = {ms[0], ms[1], ms[2]};
      c.MovingOrigin = {mo[0], mo[1], mo[2]};
      c.SamplerSpacing = {vs[0], vs[1], vs[2]};
      c.PatchSize = patch;
      c.IsMovingHighResolution = hrm != 0;
      c.IsFixedHighResolution = hrm == 0;
      c.IsCenterOverlaid = centred != 0;
      c.FixedBuffer = fixed.data();
      c.MovingBuffer = moving.data();
      c.IsConfigured = true;
      Interpolator3D interp(&c);
      interp.InitiateMappers();
      interp.InitiateRegistrationHandle();
      double p[12];
      while (in >> p[0]) {
        for (int i = 1; i < 12; ++i) in >> p[i];
        interp.GenerateMappers(make_float3(p[3], p[4], p[5]), make_float3(p[0], p[1], p[2]),
                               make_float3(p[6], p[7], p[8]), make_float3(p[9], p[10], p[11]));
        interp.Interpolate();
        std::printf("%.17g\n", interp.GetSimilarityMeasure(patch));
      }
    } else {
      LC2Configuration2D c;
      c.FixedDimension = {fd[0], fd[1]};
      c.FixedSpacing = {fs[0], fs[1]};
      c.FixedOrigin = {fo[0], fo[1]};
      c.MovingDimension = {md[0], md[1]};
      c.MovingSpacing = {ms[0], ms[1]};
      c.MovingOrigin = {mo[0], mo[1]};
      c.SamplerSpacing = {vs[0], vs[1]};
      c.PatchSize = patch;
      c.IsMovingHighResolution = hrm != 0;
      c.IsFixedHighResolution = hrm == 0;
      c.IsCenterOverlaid = centred != 0;
      c.FixedBuffer = fixed.data();
      c.MovingBuffer = moving.data();
      c.IsConfigured = true;
      Interpolator2D interp(&c);
      interp.InitiateMappers();
      interp.InitiateRegistrationHandle();
      double p[6];
      while (in >> p[0]) {
        for (int i = 1; i < 6; ++i) in >> p[i];
        interp.GenerateMappers((float)p[2], make_float2(p[0], p[1]), make_float2(p[3], p[4]),
                               (float)p[5]);
        interp.Interpolate();
        std::printf("%.17g\n", interp.GetSimilarityMeasure(patch));
      }
    }
  } catch (const lc2dropin::Error& e) {
    std::fprintf(stderr, "lc2 error %d: %s\n", e.status, e.what());
    return 2;
  }
  return 0;
}
