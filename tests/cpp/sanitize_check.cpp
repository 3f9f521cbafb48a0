// Host code under AddressSanitizer and UndefinedBehaviorSanitizer (built by
// tests/test_sanitizers.py with -fsanitize=address,undefined): the FP64
// oracle on small 2D and 3D cases (direct and box-sum moments must agree),
// lc2_minimize with every algorithm on a bounded Rosenbrock problem, the YAML
// reader and writer on a parameter file of the reference's schema, and the
// NRRD / PNG / matrix writers. Exits non-zero on any mismatch; the
// sanitizers abort on any memory or undefined-behaviour error.
//
//   sanitize_check <writable dir> [parameter files ...]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "lc2.h"
#include "lc2_io.hpp"
#include "lc2_oracle.h"
#include "lc2_yaml.hpp"

static int failures = 0;
#define CHECK(cond, ...)                   \
  do {                                     \
    if (!(cond)) {                         \
      std::fprintf(stderr, __VA_ARGS__);   \
      std::fprintf(stderr, "\n");          \
      ++failures;                          \
    }                                      \
  } while (0)

static void oracle_cases() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<float> u(0.05f, 1.0f);
  for (int nd : {2, 3}) {
    const int n = nd == 3 ? 20 : 48;
    or_geom g{};
    for (int a = 0; a < 3; ++a) {
      g.dim[a] = (a < nd) ? n : 1;
      g.spacing[a] = 1.0f;
      g.origin[a] = 0.0f;
    }
    const size_t nv = (size_t)g.dim[0] * g.dim[1] * g.dim[2];
    std::vector<float> fixed(nv), moving(nv);
    for (size_t i = 0; i < nv; ++i) {
      moving[i] = u(rng);
      fixed[i] = 0.7f * moving[i] + 0.05f * u(rng);
    }
    float mat[16] = {1, 0, 0, 0.3f, 0, 1, 0, -0.2f, 0, 0, 1, 0.1f, 0, 0, 0, 1};
    float mat2[9] = {1, 0, 0.3f, 0, 1, -0.2f, 0, 0, 1};
    const float vs[3] = {1.0f, 1.0f, 1.0f};
    const float* m = nd == 3 ? mat : mat2;
    double s1[2], s2[2];
    const double a = or_lc2_eval(nd, nd, &g, fixed.data(), &g, moving.data(), vs, 2, 1, m, 0, 1,
                                 nullptr, nullptr, nullptr, nullptr, nullptr, s1);
    const double b = or_lc2_eval(nd, nd, &g, fixed.data(), &g, moving.data(), vs, 2, 1, m, 1, 2,
                                 nullptr, nullptr, nullptr, nullptr, nullptr, s2);
    CHECK(a > 0 && std::fabs(a / b - 1.0) < 1e-12, "oracle %dD: direct %.17g box %.17g", nd, a, b);
    const double nmi = or_nmi(fixed.data(), moving.data(), (long long)nv);
    CHECK(nmi >= 1.0 && nmi <= 2.0, "oracle NMI %g", nmi);
  }
}

static int rosen(void*, int count, int dim, const double* x, double* f) {
  for (int k = 0; k < count; ++k) {
    double s = 0.0;
    for (int i = 0; i + 1 < dim; ++i) {
      const double a = x[k * dim + i], b = x[k * dim + i + 1];
      s += 100.0 * (b - a * a) * (b - a * a) + (1.0 - a) * (1.0 - a);
    }
    f[k] = s;
  }
  return 0;
}

static void optimizers() {
  const double lo[3] = {-2, -2, -2}, hi[3] = {2, 2, 2};
  for (int alg : {LC2_OPT_BOBYQA, LC2_OPT_NELDER_MEAD, LC2_OPT_QUAD_TR, LC2_OPT_DIRECT_L}) {
    lc2_opt_problem p{};
    p.algorithm = alg;
    p.dim = 3;
    p.lower = lo;
    p.upper = hi;
    p.xtol_rel = 1e-7;
    p.maxeval = 4000;
    double x[3] = {-1.2, 1.0, -0.5}, fmin = 0.0;
    lc2_opt_report rep{};
    const int st = lc2_minimize(&p, rosen, nullptr, x, &fmin, &rep);
    CHECK(st == LC2_OK, "lc2_minimize(%d) status %d", alg, st);
    if (alg == LC2_OPT_BOBYQA)
      CHECK(fmin < 1e-10, "BOBYQA Rosenbrock fmin %g after %d", fmin, rep.evaluations);
    CHECK(rep.evaluations <= 4000, "maxeval exceeded");
  }
  lc2_opt_problem bad{};
  bad.algorithm = LC2_OPT_BOBYQA;
  bad.dim = 0;
  double x = 0.0;
  CHECK(lc2_minimize(&bad, rosen, nullptr, &x, nullptr, nullptr) == LC2_ERR_INVALID_ARGUMENT,
        "bad problem accepted");
}

static void yaml_files(const std::string& dir, int argc, char** argv) {
  const char* text =
      "InputParameters:\n"
      "  FixedVolume:\n"
      "    Dimension: {x: 96, y: 96, z: 96}  # voxels\n"
      "    Spacing: {x: 1.0, y: 1.0, z: 1.0}\n"
      "    FilePath: \"C:/data/us volume.raw\"\n"
      "  RegistrationParameters:\n"
      "    PatchSize: 3\n"
      "  OptimizerSettings:\n"
      "    BOBYQA:\n"
      "      0:\n"
      "        Enabled: true\n"
      "        OptimizedEntries: {Translation: true, Rotation: false}\n"
      "    List: [1, 2, 3]\n"
      "    Items:\n"
      "      - a: 1\n"
      "        b: [x, y]\n"
      "      - plain\n";
  lc2yaml::Node n = lc2yaml::parse(text);
  const std::string once = lc2yaml::dump(n);
  const std::string twice = lc2yaml::dump(lc2yaml::parse(once));
  CHECK(once == twice, "YAML round trip differs");
  for (int i = 2; i < argc; ++i) {
    lc2yaml::Node f = lc2yaml::load_file(argv[i]);
    const std::string a = lc2yaml::dump(f);
    CHECK(a == lc2yaml::dump(lc2yaml::parse(a)), "YAML round trip of %s differs", argv[i]);
  }
  lc2yaml::save_file(n, dir + "/saved.yaml");
  CHECK(lc2yaml::dump(lc2yaml::load_file(dir + "/saved.yaml")) == once, "YAML save/load differs");
}

static void writers(const std::string& dir) {
  std::vector<uint8_t> px(31 * 17);
  for (size_t i = 0; i < px.size(); ++i) px[i] = (uint8_t)(i * 13);
  lc2io::write_png_gray8(dir + "/s.png", 31, 17, px.data());
  std::vector<float> v(5 * 4 * 3, 0.25f);
  lc2io::NrrdHeader h{{5, 4, 3}, {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, {0, 0, 0}};
  lc2io::write_nrrd(dir + "/s.nrrd", h, v.data());
  const float m[9] = {1, 0, 2, 0, 1, 3, 0, 0, 1};
  lc2io::write_matrix(dir + "/s.mat", m, 3, 3);
}

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  oracle_cases();
  optimizers();
  yaml_files(argv[1], argc, argv);
  writers(argv[1]);
  if (failures) std::fprintf(stderr, "%d failures\n", failures);
  return failures ? 1 : 0;
}
