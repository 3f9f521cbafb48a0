// Stand-ins for the CUDA-side entry points lc2_optim.cpp links against, so
// that its host code (lc2_minimize) builds under the sanitizers without the
// CUDA library. The sanitizer check calls only lc2_minimize, which uses none
// of them; each returns LC2_ERR_UNSUPPORTED if reached.
#include <string>

#include "lc2.h"

static thread_local std::string g_msg;
void lc2_set_error_message(const char* msg) { g_msg = msg ? msg : ""; }
extern "C" {
const char* lc2_last_error(void) { return g_msg.c_str(); }
int lc2_affine_3d(const float*, const float*, const float*, const float*, const float*,
                  const float*, float*) { return LC2_ERR_UNSUPPORTED; }
int lc2_affine_2d(float, const float*, const float*, float, const float*, const float*, float*) {
  return LC2_ERR_UNSUPPORTED;
}
int lc2_evaluate(lc2_context*, const float*, double*) { return LC2_ERR_UNSUPPORTED; }
int lc2_evaluate_batch(lc2_context*, const float*, int, double*) { return LC2_ERR_UNSUPPORTED; }
int lc2_get_config(const lc2_context*, lc2_config*) { return LC2_ERR_UNSUPPORTED; }
}
