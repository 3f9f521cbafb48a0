// Runs the reference's own LC2 kernels on the CPU (golden-vector source).
//
// ref_kernels.inc holds the reference's kernel functions verbatim (extracted
// at build time by extract_kernels.py from the reference sources into
// oracle/_ref/, never committed). This file supplies what the CUDA runtime
// would: per-thread threadIdx/blockIdx, __syncthreads as a barrier over the
// threads of one block, dynamic shared memory and __constant__ storage. Each
// block runs as blockDim.x*y*z std::threads; blocks run one after another.
//
// The drivers below repeat the launch sequence of the reference's host code:
//   Interpolator{2D,3D,2DTo3D}::Interpolate     (src/Interpolator/interpolator.cu:583-615,
//                                                :1266-1372, :1688-1720)
//   LC2_{2D,3D}_class::PrepareGradientFilter    (src/cu_LC2/cu_lc2_2d.cu:548-578,
//                                                src/cu_LC2/cu_lc2_3d.cu:977-1005)
//   LC2_{2D,3D}_class::CalculateGradient        (cu_lc2_2d.cu:580-597, cu_lc2_3d.cu:1007-1033)
//   LC2_{2D,3D}_class::GetSimilarityMetric      (cu_lc2_2d.cu:599-653, cu_lc2_3d.cu:1119-1194)
// with the block sizes the reference uses (8^3 / 8x8 resampling, 16x16 2D
// and 8^3 3D LC2 kernels).
#include <barrier>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "src/Interpolator/spatialMappers.cuh"

using std::isinf;
using std::isnan;

namespace emu {
thread_local uint3 tidx, bidx;
dim3 bdim, gdim;
std::barrier<>* bar = nullptr;

template <typename F>
void launch(dim3 grid, dim3 block, const F& body) {
  bdim = block;
  gdim = grid;
  const int nt = (int)(block.x * block.y * block.z);
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        std::barrier<> b(nt);
        bar = &b;
        std::vector<std::thread> ts;
        ts.reserve(nt);
        for (int t = 0; t < nt; ++t) {
          ts.emplace_back([&, t] {
            tidx = make_uint3(t % block.x, (t / block.x) % block.y, t / (block.x * block.y));
            bidx = make_uint3(bx, by, bz);
            body();
          });
        }
        for (auto& th : ts) th.join();
        bar = nullptr;
      }
}
}  // namespace emu

#undef __global__
#undef __device__
#undef __shared__
#undef __constant__
#define __global__
#define __device__
#define __shared__
#define __constant__
#define threadIdx emu::tidx
#define blockIdx emu::bidx
#define blockDim emu::bdim
#define gridDim emu::gdim
#define __syncthreads() emu::bar->arrive_and_wait()

float dynSharedMem[1 << 20];

#include "src/cu_LC2/cu_lc2_helper.cuh"
#include "ref_kernels.inc"

namespace {

int ceil_div(int a, int b) { return (int)std::ceil(a / (float)b); }

void sobel_taps(int nd) {
  const float h[3] = {1.0f, 2.0f, 1.0f};
  const float hp[3] = {-1.0f, 0.0f, 1.0f};
  if (nd == 2) {
    for (int y = 0; y < 3; ++y)
      for (int x = 0; x < 3; ++x) {
        Sobel_X_dConstant[x + 3 * y] = hp[x] * h[y];
        Sobel_Y_dConstant[x + 3 * y] = h[x] * hp[y];
      }
    return;
  }
  for (int z = 0; z < 3; ++z)
    for (int y = 0; y < 3; ++y)
      for (int x = 0; x < 3; ++x) {
        Sobel_X_dConstant[x + 3 * y + 9 * z] = hp[x] * h[y] * h[z];
        Sobel_Y_dConstant[x + 3 * y + 9 * z] = h[x] * hp[y] * h[z];
        Sobel_Z_dConstant[x + 3 * y + 9 * z] = h[x] * h[y] * hp[z];
      }
}

// LC2 on a 2D grid (cu_lc2_2d.cu:580-653); returns 0 and leaves measures at
// zero when the shared-memory check of :611 fails, as the reference does.
void lc2_2d(int x, int y, float* U, float* M, float* G, float* W, float* S, int patch) {
  sobel_taps(2);
  int2 dim = make_int2(x, y);
  dim3 grid(ceil_div(x, 16), ceil_div(y, 16), 1), block(16, 16, 1);
  emu::launch(grid, block, [&] { gradient2DSobelKernel(M, dim, G); });
  int unit = (16 + 2 * patch) * (16 + 2 * patch) * (int)sizeof(float);
  std::memset(W, 0, sizeof(float) * x * y);
  std::memset(S, 0, sizeof(float) * x * y);
  if (unit * 3 < 48 * 1024) {
    emu::launch(grid, block, [&] { calculate2DWeightingFactorOnSharedMemory(U, dim, patch, W); });
    emu::launch(grid, block, [&] {
      calculate2DWeightedSimilarityOnSharedMemory(U, M, G, W, dim, patch, S);
    });
  }
}

// LC2 on a 3D grid (cu_lc2_3d.cu:1007-1194): shared-memory kernels while
// 3 tiles fit in 48 KiB, else the global-memory similarity kernel.
void lc2_3d(int x, int y, int z, float* U, float* M, float* G, float* W, float* S, int patch) {
  sobel_taps(3);
  int3 dim = make_int3(x, y, z);
  dim3 grid(ceil_div(x, 8), ceil_div(y, 8), ceil_div(z, 8)), block(8, 8, 8);
  emu::launch(grid, block, [&] { gradient3DSobelKernel(M, dim, G); });
  int unit = (8 + 2 * patch) * (8 + 2 * patch) * (8 + 2 * patch) * (int)sizeof(float);
  emu::launch(grid, block, [&] { calculate3DWeightingFactorOnSharedMemory(U, dim, patch, W); });
  if (unit * 3 / 1024 < 48) {
    emu::launch(grid, block, [&] {
      calculate3DWeightedSimilarityOnSharedMemory(U, M, G, W, dim, patch, S);
    });
  } else {
    emu::launch(grid, block, [&] {
      calculate3DWeightedSimilarityOnGlobalMemory(U, M, G, W, dim, patch, S);
    });
  }
}

float3 f3(const float* v) { return make_float3(v[0], v[1], v[2]); }
int3 i3(const int* v) { return make_int3(v[0], v[1], v[2]); }

}  // namespace

extern "C" {

// Resample + LC2 for the 2D mode. Geometry arrays: dims[3], spacing[3],
// origin[3] for fixed, moving and virtual grids; mat: row-major 3x3
// virtual->moving. Outputs (virtual grid): U, M (high-resolution), G,
// weighting factor W, weighted similarity S. hr_moving: 1 = the moving
// image is the high-resolution modality.
void ref_eval_2d(const int* fd, const float* fs, const float* fo, const float* fixed,
                 const int* md, const float* ms, const float* mo, const float* moving,
                 const int* vd, const float* vs, const float* vo, const float* mat, int hr_moving,
                 int patch, float* U, float* M, float* G, float* W, float* S) {
  Fixed2DMapper_d = PhysioSpatial2DMapper(make_float2(fs[0], fs[1]), make_float2(fo[0], fo[1]),
                                          make_int2(fd[0], fd[1]));
  Moving2DMapper_d = PhysioSpatial2DMapper(make_float2(ms[0], ms[1]), make_float2(mo[0], mo[1]),
                                           make_int2(md[0], md[1]));
  Virtual2DMapper_d = PhysioSpatial2DMapper(make_float2(vs[0], vs[1]), make_float2(vo[0], vo[1]),
                                            make_int2(vd[0], vd[1]));
  VirtualToFixed2D_d.Identity();
  VirtualToMoving2D_d.Identity();
  VirtualToMoving2D_d.SetMatrix(mat);
  int x = vd[0], y = vd[1];
  std::vector<float> vf(x * y), vm(x * y);
  dim3 grid(ceil_div(x, 8), ceil_div(y, 8), 1), block(8, 8, 1);
  emu::launch(grid, block, [&] { Interpolate_2Dkernel(vf.data(), vm.data(), fixed, moving); });
  std::memcpy(U, hr_moving ? vf.data() : vm.data(), sizeof(float) * x * y);
  std::memcpy(M, hr_moving ? vm.data() : vf.data(), sizeof(float) * x * y);
  lc2_2d(x, y, U, M, G, W, S, patch);
}

// Resample with the 3D kernel onto a virtual grid, then LC2 in 3D
// (lc2_nd = 3) or, for the 2D-to-3D mode (virtual z = 1), in 2D.
void ref_eval_3d(const int* fd, const float* fs, const float* fo, const float* fixed,
                 const int* md, const float* ms, const float* mo, const float* moving,
                 const int* vd, const float* vs, const float* vo, const float* mat, int hr_moving,
                 int patch, int lc2_nd, float* U, float* M, float* G, float* W, float* S) {
  Fixed3DMapper_d = PhysioSpatial3DMapper(f3(fs), f3(fo), i3(fd));
  Moving3DMapper_d = PhysioSpatial3DMapper(f3(ms), f3(mo), i3(md));
  Virtual3DMapper_d = PhysioSpatial3DMapper(f3(vs), f3(vo), i3(vd));
  VirtualToFixed3D_d.Identity();
  VirtualToMoving3D_d.Identity();
  VirtualToMoving3D_d.SetMatrix(mat);
  int x = vd[0], y = vd[1], z = vd[2];
  size_t n = (size_t)x * y * z;
  std::vector<float> vf(n), vm(n);
  dim3 grid(ceil_div(x, 8), ceil_div(y, 8), ceil_div(z, 8)), block(8, 8, 8);
  emu::launch(grid, block, [&] { Interpolate_3Dkernel(vf.data(), vm.data(), fixed, moving); });
  std::memcpy(U, hr_moving ? vf.data() : vm.data(), sizeof(float) * n);
  std::memcpy(M, hr_moving ? vm.data() : vf.data(), sizeof(float) * n);
  if (lc2_nd == 3)
    lc2_3d(x, y, z, U, M, G, W, S, patch);
  else
    lc2_2d(x, y, U, M, G, W, S, patch);
}

}  // extern "C"
