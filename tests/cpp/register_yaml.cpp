// The reference's registration flow from a parameter file
// (src/mainRegistrationTool/main.cu:757-801 for 3D, 728-756 for 2D):
//   Interpolator(yaml) -> InitiateMappers -> InitiateRegistrationHandle ->
//   Optimizers(yaml) -> LinkToInterpolator -> Optimize -> ExportResults.
//   register_yaml <2D|3D|2DTo3D> <params.yaml>
// Prints the optimum, LC2 and evaluation count; writes <name>_result.yaml and,
// as main.cu does after ExportResults, the registered moving image
// (WriteOut(OptimalMatrix)).
// With one argument <params.yaml> it only parses and re-emits the file.
#include <cstdio>
#include <iostream>
#include <string>

#include "lc2_optimizers.hpp"

int main(int argc, char** argv) {
  try {
    if (argc == 2) {
      lc2yaml::Node y = lc2yaml::load_file(argv[1]);
      std::cout << lc2yaml::dump(y);
      return 0;
    }
    const std::string mode = argv[1], path = argv[2];
    std::vector<double> opt;
    double sim = 0;
    int evals = 0;
    std::string result;
    if (mode == "2D") {
      Interpolator2D interp(path);
      interp.InitiateMappers();
      interp.InitiateRegistrationHandle();
      Optimizers2D o(path);
      o.LinkToInterpolator(&interp);
      o.Optimize();
      o.ExportResults();
      float OptimalMatrix[9] = {0.0f};
      o.GetInternalMatrix(OptimalMatrix);
      interp.WriteOut(OptimalMatrix);
      opt = o.OptimalSolution;
      sim = o.SimilarityMeasure;
      evals = o.EvalCounter;
      result = o.ResultPath();
    } else if (mode == "3D") {
      Interpolator3D interp(path, false);
      interp.InitiateMappers();
      interp.InitiateRegistrationHandle();
      Optimizers3D o(path);
      o.LinkToInterpolator(&interp);
      o.Optimize();
      o.ExportResults();
      float OptimalMatrix[16] = {0.0f};
      o.GetInternalMatrix(OptimalMatrix);
      interp.WriteOut(OptimalMatrix);
      opt = o.OptimalSolution;
      sim = o.SimilarityMeasure;
      evals = o.EvalCounter;
      result = o.ResultPath();
    } else {
      Interpolator2DTo3D interp(path);
      interp.InitiateMappers();
      interp.InitiateRegistrationHandle();
      Optimizers2DTo3D o(path);
      o.LinkToInterpolator(&interp);
      o.Optimize();
      o.ExportResults();
      opt = o.OptimalSolution;
      sim = o.SimilarityMeasure;
      evals = o.EvalCounter;
      result = o.ResultPath();
    }
    for (double v : opt) std::printf("%.9g ", v);
    std::printf("\n%.9g %d %s\n", sim, evals, result.c_str());
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 2;
  }
  return 0;
}
