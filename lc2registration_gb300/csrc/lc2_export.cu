// lc2_export.cu -- what follows a registration: the per-voxel weighting map
// and the 2D registered-image warp (include/lc2.h).
//
//   lc2_weighting_map: measure / sigma per virtual voxel, 0 where sigma is
//     not above 1e-6 -- CalculateWeightingMap (src/cu_LC2/cu_lc2_3d.cu:843-866,
//     1303-1329), for 2D as well as 3D.
//   lc2_warp_affine_2d: the moving image resampled into the fixed image with
//     the optimal moving->fixed matrix in pixel units, bilinear, pixels whose
//     source falls outside the moving image left at 0 -- the warp that
//     Interpolator2D::WriteOut does with nppiWarpAffine_32f_C1R
//     (src/Interpolator/interpolator.cu:1438-1535). NPP itself is not used:
//     this is a plain backward-mapping kernel; NPP's own edge rules are not
//     reproduced beyond "outside the source: unchanged".
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <string>

#include "../../include/lc2.h"

void lc2_set_error_message(const char* msg);

namespace {

int fail(int code, const std::string& msg) {
  lc2_set_error_message(msg.c_str());
  return code;
}

#define EXPORT_CUDA(call)                                                           \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return fail(e_ == cudaErrorMemoryAllocation ? LC2_ERR_OUT_OF_MEMORY : LC2_ERR_CUDA, \
                  std::string(#call) + ": " + cudaGetErrorString(e_));              \
  } while (0)

// dst(x', y') = src(Cinv (x', y', 1)); coordinates at pixel centres, integer
// pixel positions; inside means 0 <= x <= sw - 1 and 0 <= y <= sh - 1.
__global__ void k_warp_affine_2d(const float* __restrict__ src, int sw, int sh,
                                 float* __restrict__ dst, int dw, int dh, float a00, float a01,
                                 float b0, float a10, float a11, float b1) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= dw || y >= dh) return;
  const float sx = fmaf(a01, (float)y, fmaf(a00, (float)x, b0));
  const float sy = fmaf(a11, (float)y, fmaf(a10, (float)x, b1));
  if (!(sx >= 0.0f && sy >= 0.0f && sx <= (float)(sw - 1) && sy <= (float)(sh - 1))) return;
  const int x0 = (int)floorf(sx), y0 = (int)floorf(sy);
  const int x1 = min(x0 + 1, sw - 1), y1 = min(y0 + 1, sh - 1);
  const float fx = sx - (float)x0, fy = sy - (float)y0;
  const float v00 = src[(size_t)y0 * sw + x0], v01 = src[(size_t)y0 * sw + x1];
  const float v10 = src[(size_t)y1 * sw + x0], v11 = src[(size_t)y1 * sw + x1];
  const float top = fmaf(fx, v01 - v00, v00), bot = fmaf(fx, v11 - v10, v10);
  dst[(size_t)y * dw + x] = fmaf(fy, bot - top, top);
}

}  // namespace

extern "C" int lc2_warp_affine_2d(const float* src, int sw, int sh, float* dst, int dw, int dh,
                                  const double coeffs[6], int device) {
  if (!src || !dst || !coeffs) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  if (sw < 1 || sh < 1 || dw < 1 || dh < 1)
    return fail(LC2_ERR_INVALID_ARGUMENT, "image sizes must be >= 1");
  for (int i = 0; i < 6; ++i)
    if (!std::isfinite(coeffs[i])) return fail(LC2_ERR_INVALID_ARGUMENT, "coefficients must be finite");
  // inverse of the forward (source -> destination) map
  const double det = coeffs[0] * coeffs[4] - coeffs[1] * coeffs[3];
  if (det == 0.0 || !std::isfinite(det)) return fail(LC2_ERR_SINGULAR, "singular warp");
  const double a00 = coeffs[4] / det, a01 = -coeffs[1] / det;
  const double a10 = -coeffs[3] / det, a11 = coeffs[0] / det;
  const double b0 = -(a00 * coeffs[2] + a01 * coeffs[5]);
  const double b1 = -(a10 * coeffs[2] + a11 * coeffs[5]);
  int cur = -1;
  EXPORT_CUDA(cudaGetDevice(&cur));
  if (cur != device) EXPORT_CUDA(cudaSetDevice(device));
  const size_t ns = (size_t)sw * sh, nd = (size_t)dw * dh;
  float* d = nullptr;
  EXPORT_CUDA(cudaMalloc(&d, sizeof(float) * (ns + nd)));
  struct Free {
    float* p;
    ~Free() { cudaFree(p); }
  } guard{d};
  float* d_src = d;
  float* d_dst = d + ns;
  EXPORT_CUDA(cudaMemcpy(d_src, src, sizeof(float) * ns, cudaMemcpyHostToDevice));
  EXPORT_CUDA(cudaMemset(d_dst, 0, sizeof(float) * nd));
  dim3 block(32, 8);
  dim3 grid((dw + 31) / 32, (dh + 7) / 8);
  k_warp_affine_2d<<<grid, block>>>(d_src, sw, sh, d_dst, dw, dh, (float)a00, (float)a01,
                                    (float)b0, (float)a10, (float)a11, (float)b1);
  EXPORT_CUDA(cudaGetLastError());
  EXPORT_CUDA(cudaMemcpy(dst, d_dst, sizeof(float) * nd, cudaMemcpyDeviceToHost));
  return LC2_OK;
}
