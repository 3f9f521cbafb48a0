// Times the reference's own LC2 kernels on the GPU (baseline measurement).
//
// Built on the GPU host by `make -C oracle refgpu` from oracle/_ref/, where
// `make -C oracle ref` placed, at build time and never committed, the
// reference's kernel line ranges (ref_kernels.inc) and the three headers and
// sources they need (refsrc/src/...). This file supplies only the launch
// sequence of one plain evaluation, restated from the reference's host code:
//   Interpolator{2D,3D}::GenerateMappers   two mapper uploads (src/Interpolator/interpolator.cu:575-576)
//   Interpolator{2D,3D}::Interpolate       resampling kernel, 8^3 / 8x8 blocks (:583-615, :1266-1372);
//                                          the 3D path's buffer getters return device vectors by
//                                          value (src/cu_LC2/cu_lc2_3d.cuh:46-49), i.e. two N-float
//                                          allocations, copies and frees per evaluation
//   LC2_{2D,3D}_class::PrepareGradientFilter  Sobel taps to constant memory every evaluation
//                                          (src/cu_LC2/cu_lc2_3d.cu:977-1005, cu_lc2_2d.cu:548-578)
//   LC2_{2D,3D}_class::CalculateGradient   Sobel kernel (cu_lc2_3d.cu:1007-1033, cu_lc2_2d.cu:580-597)
//   LC2_{2D,3D}_class::GetSimilarityMetric weighting + similarity kernels (shared-memory variants
//                                          while 3 tiles fit in 48 KiB, else the global-memory
//                                          one) and two FP32 thrust::reduce calls
//                                          (cu_lc2_3d.cu:1119-1194, cu_lc2_2d.cu:599-653)
// The resampled images are written into the LC2 buffers (the 2D path's
// behaviour); for 3D the by-value copies are timed as well, separately.
//
//   ref_gpu_time <case file>   ->   one JSON line on stdout
//
// Case file (whitespace-separated): mode (2 or 3), then for fixed and moving
// dims[3] spacing[3] origin[3] path-to-raw-float32, virtual dims[3]
// spacing[3] origin[3], hr_moving, patch, evaluations, and the row-major
// virtual->moving matrix (9 numbers for mode 2, 16 for mode 3).
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/functional.h>
#include <thrust/reduce.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "src/Interpolator/spatialMappers.cu"
#include "src/cu_LC2/cu_lc2_helper.cuh"
#include "ref_kernels.inc"

namespace {

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      std::fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #call,                 \
                   cudaGetErrorString(e_));                                             \
      std::exit(1);                                                                     \
    }                                                                                   \
  } while (0)

struct Geom {
  int d[3];
  float s[3], o[3];
};

struct Case {
  int mode = 3;
  Geom fixed, moving, virt;
  std::string fixed_path, moving_path;
  int hr_moving = 1, patch = 3, evals = 3;
  float mat[16] = {0};
};

Case read_case(const char* path) {
  std::ifstream f(path);
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", path);
    std::exit(1);
  }
  Case c;
  auto geom = [&](Geom& g) {
    for (int i = 0; i < 3; ++i) f >> g.d[i];
    for (int i = 0; i < 3; ++i) f >> g.s[i];
    for (int i = 0; i < 3; ++i) f >> g.o[i];
  };
  f >> c.mode;
  geom(c.fixed);
  f >> c.fixed_path;
  geom(c.moving);
  f >> c.moving_path;
  geom(c.virt);
  f >> c.hr_moving >> c.patch >> c.evals;
  const int nm = c.mode == 2 ? 9 : 16;
  for (int i = 0; i < nm; ++i) f >> c.mat[i];
  if (!f || (c.mode != 2 && c.mode != 3) || c.evals < 1 || c.patch < 1) {
    std::fprintf(stderr, "malformed case file %s\n", path);
    std::exit(1);
  }
  return c;
}

std::vector<float> read_raw(const std::string& path, size_t n) {
  std::vector<float> v(n);
  std::ifstream f(path, std::ios::binary);
  if (!f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(float)))) {
    std::fprintf(stderr, "cannot read %zu floats from %s\n", n, path.c_str());
    std::exit(1);
  }
  return v;
}

size_t count(const Geom& g, int mode) {
  return (size_t)g.d[0] * g.d[1] * (mode == 3 ? g.d[2] : 1);
}

int cdiv(int a, int b) { return (int)std::ceil(a / (float)b); }

struct Buffers {
  float *fixed = nullptr, *moving = nullptr;   // source images
  float *us = nullptr, *hr = nullptr;          // LC2 buffers: ultrasound, high resolution
  float *grad = nullptr, *w = nullptr, *s = nullptr;
};

// One plain evaluation in the reference's order; returns LC2.
double evaluate(const Case& c, const Buffers& B, size_t nv, bool by_value_copies) {
  const int x = c.virt.d[0], y = c.virt.d[1], z = c.mode == 3 ? c.virt.d[2] : 1;
  // GenerateMappers: two mapper uploads
  if (c.mode == 3) {
    Spatial3DMapper v2m, v2f;
    v2m.Identity();
    v2m.SetMatrix(c.mat);
    v2f.Identity();
    CK(cudaMemcpyToSymbol(VirtualToMoving3D_d, &v2m, sizeof(Spatial3DMapper)));
    CK(cudaMemcpyToSymbol(VirtualToFixed3D_d, &v2f, sizeof(Spatial3DMapper)));
  } else {
    Spatial2DMapper v2m, v2f;
    v2m.Identity();
    v2m.SetMatrix(c.mat);
    v2f.Identity();
    CK(cudaMemcpyToSymbol(VirtualToMoving2D_d, &v2m, sizeof(Spatial2DMapper)));
    CK(cudaMemcpyToSymbol(VirtualToFixed2D_d, &v2f, sizeof(Spatial2DMapper)));
  }
  // Interpolate
  float* dst_fixed = c.hr_moving ? B.us : B.hr;
  float* dst_moving = c.hr_moving ? B.hr : B.us;
  if (c.mode == 3) {
    if (by_value_copies) {
      // the two device vectors returned by value: allocate, copy, free
      float *t0 = nullptr, *t1 = nullptr;
      CK(cudaMalloc(&t0, nv * sizeof(float)));
      CK(cudaMemcpy(t0, B.us, nv * sizeof(float), cudaMemcpyDeviceToDevice));
      CK(cudaMalloc(&t1, nv * sizeof(float)));
      CK(cudaMemcpy(t1, B.hr, nv * sizeof(float), cudaMemcpyDeviceToDevice));
      CK(cudaFree(t0));
      CK(cudaFree(t1));
    }
    Interpolate_3Dkernel<<<dim3(cdiv(x, 8), cdiv(y, 8), cdiv(z, 8)), dim3(8, 8, 8)>>>(
        dst_fixed, dst_moving, B.fixed, B.moving);
  } else {
    Interpolate_2Dkernel<<<dim3(cdiv(x, 8), cdiv(y, 8), 1), dim3(8, 8, 1)>>>(
        dst_fixed, dst_moving, B.fixed, B.moving);
  }
  CK(cudaGetLastError());
  // PrepareGradientFilter: Sobel taps h = (1, 2, 1), hp = (-1, 0, 1)
  const float h[3] = {1.0f, 2.0f, 1.0f}, hp[3] = {-1.0f, 0.0f, 1.0f};
  if (c.mode == 3) {
    float sx[27], sy[27], sz[27];
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
          sx[i + 3 * j + 9 * k] = hp[i] * h[j] * h[k];
          sy[i + 3 * j + 9 * k] = h[i] * hp[j] * h[k];
          sz[i + 3 * j + 9 * k] = h[i] * h[j] * hp[k];
        }
    CK(cudaMemcpyToSymbol(Sobel_X_dConstant, sx, sizeof(sx)));
    CK(cudaMemcpyToSymbol(Sobel_Y_dConstant, sy, sizeof(sy)));
    CK(cudaMemcpyToSymbol(Sobel_Z_dConstant, sz, sizeof(sz)));
    // CalculateGradient, 8^3 blocks
    const dim3 grid(cdiv(x, 8), cdiv(y, 8), cdiv(z, 8)), block(8, 8, 8);
    gradient3DSobelKernel<<<grid, block, 10 * 10 * 10 * sizeof(float)>>>(B.hr, make_int3(x, y, z),
                                                                         B.grad);
    CK(cudaGetLastError());
    // GetSimilarityMetric(8, 8, 8, patch)
    const int p = c.patch;
    const int unit = (8 + 2 * p) * (8 + 2 * p) * (8 + 2 * p) * (int)sizeof(float);
    calculate3DWeightingFactorOnSharedMemory<<<grid, block, unit>>>(B.us, make_int3(x, y, z), p,
                                                                    B.w);
    CK(cudaGetLastError());
    if (unit * 3 / 1024 < 48) {
      calculate3DWeightedSimilarityOnSharedMemory<<<grid, block, unit * 3>>>(
          B.us, B.hr, B.grad, B.w, make_int3(x, y, z), p, B.s);
    } else {
      calculate3DWeightedSimilarityOnGlobalMemory<<<grid, block>>>(B.us, B.hr, B.grad, B.w,
                                                                   make_int3(x, y, z), p, B.s);
    }
    CK(cudaGetLastError());
  } else {
    float sx[9], sy[9];
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        sx[i + 3 * j] = hp[i] * h[j];
        sy[i + 3 * j] = h[i] * hp[j];
      }
    CK(cudaMemcpyToSymbol(Sobel_X_dConstant, sx, sizeof(sx)));
    CK(cudaMemcpyToSymbol(Sobel_Y_dConstant, sy, sizeof(sy)));
    const dim3 grid(cdiv(x, 16), cdiv(y, 16), 1), block(16, 16, 1);
    gradient2DSobelKernel<<<grid, block, 18 * 18 * sizeof(float)>>>(B.hr, make_int2(x, y), B.grad);
    CK(cudaGetLastError());
    const int p = c.patch;
    const int unit = (16 + 2 * p) * (16 + 2 * p) * (int)sizeof(float);
    if (unit * 3 < 48 * 1024) {
      calculate2DWeightingFactorOnSharedMemory<<<grid, block, unit>>>(B.us, make_int2(x, y), p,
                                                                      B.w);
      CK(cudaGetLastError());
      calculate2DWeightedSimilarityOnSharedMemory<<<grid, block, unit * 3>>>(
          B.us, B.hr, B.grad, B.w, make_int2(x, y), p, B.s);
      CK(cudaGetLastError());
    }
  }
  const thrust::device_ptr<float> ps(B.s), pw(B.w);
  const double sm = (double)thrust::reduce(ps, ps + nv, 0.0f, thrust::plus<float>());
  const double sw = (double)thrust::reduce(pw, pw + nv, 0.0f, thrust::plus<float>());
  double lc2 = sm / sw;
  if (std::isnan(lc2) || std::isinf(lc2)) lc2 = 0.0;
  return lc2;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: ref_gpu_time <case file>\n");
    return 2;
  }
  const Case c = read_case(argv[1]);
  const size_t nf = count(c.fixed, c.mode), nm = count(c.moving, c.mode), nv = count(c.virt, c.mode);
  const std::vector<float> hf = read_raw(c.fixed_path, nf), hm = read_raw(c.moving_path, nm);

  auto f3 = [](const float* v) { return make_float3(v[0], v[1], v[2]); };
  auto i3 = [](const int* v) { return make_int3(v[0], v[1], v[2]); };
  if (c.mode == 3) {
    PhysioSpatial3DMapper F(f3(c.fixed.s), f3(c.fixed.o), i3(c.fixed.d));
    PhysioSpatial3DMapper M(f3(c.moving.s), f3(c.moving.o), i3(c.moving.d));
    PhysioSpatial3DMapper V(f3(c.virt.s), f3(c.virt.o), i3(c.virt.d));
    CK(cudaMemcpyToSymbol(Fixed3DMapper_d, &F, sizeof(F)));
    CK(cudaMemcpyToSymbol(Moving3DMapper_d, &M, sizeof(M)));
    CK(cudaMemcpyToSymbol(Virtual3DMapper_d, &V, sizeof(V)));
  } else {
    auto f2 = [](const float* v) { return make_float2(v[0], v[1]); };
    auto i2 = [](const int* v) { return make_int2(v[0], v[1]); };
    PhysioSpatial2DMapper F(f2(c.fixed.s), f2(c.fixed.o), i2(c.fixed.d));
    PhysioSpatial2DMapper M(f2(c.moving.s), f2(c.moving.o), i2(c.moving.d));
    PhysioSpatial2DMapper V(f2(c.virt.s), f2(c.virt.o), i2(c.virt.d));
    CK(cudaMemcpyToSymbol(Fixed2DMapper_d, &F, sizeof(F)));
    CK(cudaMemcpyToSymbol(Moving2DMapper_d, &M, sizeof(M)));
    CK(cudaMemcpyToSymbol(Virtual2DMapper_d, &V, sizeof(V)));
  }

  Buffers B;
  CK(cudaMalloc(&B.fixed, nf * sizeof(float)));
  CK(cudaMalloc(&B.moving, nm * sizeof(float)));
  float** bufs[5] = {&B.us, &B.hr, &B.grad, &B.w, &B.s};
  for (float** b : bufs) {
    CK(cudaMalloc(b, nv * sizeof(float)));
    CK(cudaMemset(*b, 0, nv * sizeof(float)));
  }
  CK(cudaMemcpy(B.fixed, hf.data(), nf * sizeof(float), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(B.moving, hm.data(), nm * sizeof(float), cudaMemcpyHostToDevice));

  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  double lc2 = evaluate(c, B, nv, c.mode == 3);  // warm-up
  CK(cudaDeviceSynchronize());
  float ms_kernels = 0.0f, ms_copies = 0.0f;
  for (int pass = 0; pass < (c.mode == 3 ? 2 : 1); ++pass) {
    const bool copies = pass == 1;
    CK(cudaEventRecord(e0));
    for (int k = 0; k < c.evals; ++k) lc2 = evaluate(c, B, nv, copies);
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    (copies ? ms_copies : ms_kernels) = ms / c.evals;
  }
  std::printf(
      "{\"mode\": %d, \"virtual\": [%d, %d, %d], \"patch\": %d, \"evals\": %d, "
      "\"ms_per_eval\": %.4f, \"ms_per_eval_with_by_value_copies\": %s, \"lc2\": %.9g}\n",
      c.mode, c.virt.d[0], c.virt.d[1], c.mode == 3 ? c.virt.d[2] : 1, c.patch, c.evals,
      ms_kernels, c.mode == 3 ? std::to_string(ms_copies).c_str() : "null", lc2);
  for (float** b : bufs) CK(cudaFree(*b));
  CK(cudaFree(B.fixed));
  CK(cudaFree(B.moving));
  return 0;
}
