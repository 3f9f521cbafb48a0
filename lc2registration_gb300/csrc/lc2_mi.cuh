// lc2_mi.cuh -- normalised mutual information, the similarity of
// PatchSize 0 (src/Interpolator/interpolator.cu:617-622;
// src/cu_LC2/cu_lc2_3d.cu:868-923, 1196-1301):
//   NMI = (H(U) + H(M)) / H(U, M)
// over the virtual grid, with 256 bins per image between the image's own
// minimum and maximum, H(X) = -sum p ln p, p = count / voxels, and the joint
// histogram indexed ultrasound bin + 256 * high-resolution bin.
//
// One image is static (the fixed one resampled once): its bins and entropy
// are computed once per context. Per transform, three kernels run over the
// whole batch: the range of the warped image (ordered-integer atomics), the
// joint histogram (warp-aggregated integer atomics into a 256 KB histogram
// per transform, which stays in L2), and the entropies (one CTA per
// transform, double sums in a fixed order). Counts are exact integers, so the
// value does not depend on the launch shape.
#pragma once

#include "lc2_kernels.cuh"

namespace lc2 {

constexpr int kMiBins = 256;
constexpr int kMiHist = kMiBins * kMiBins;

struct MiParams {
  int mx, my, mz;         // warped (moving) image
  int vx, vy, vz;         // virtual grid
  int warped_is_high_res; // 1: key = static bin + 256 * warped bin; 0: the transpose
};

// Order-preserving float <-> unsigned maps for atomicMin / atomicMax.
__device__ __forceinline__ unsigned mi_ord(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float mi_unord(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// Bin of v in [lo, hi]: round((v - lo) * (255 / (hi - lo))) with float
// operations rounded to nearest (cu_lc2_3d.cu:886-889, 913); all voxels go
// to bin 0 when hi == lo. The host computes the static image's bins with the
// same operations.
__host__ __device__ inline float mi_scale(float lo, float hi) {
  return hi > lo ? 255.0f / (hi - lo) : 0.0f;
}
__device__ __forceinline__ int mi_bin(float v, float lo, float s) {
  return (int)roundf(__fmul_rn(__fsub_rn(v, lo), s));
}

// Range of the warped image of each transform; grid (vx/32, vy/8, vz * cnt).
template <typename TM>
__global__ void __launch_bounds__(256) k_mi_range(const TM* __restrict__ mov, MiParams P,
                                                  const Xform* __restrict__ xf, int k0,
                                                  unsigned* __restrict__ rmin,
                                                  unsigned* __restrict__ rmax) {
  __shared__ TileBase T;
  const int slot = blockIdx.z / P.vz;
  const int z = blockIdx.z - slot * P.vz;
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
  if (threadIdx.x == 0 && threadIdx.y == 0) tile_base(xf + k0 + slot, x0, y0, z, T);
  __syncthreads();
  const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  float lo = INFINITY, hi = -INFINITY;
  if (x < P.vx && y < P.vy) {
    lo = hi = tile_sample<3, TM>(mov, P.mx, P.my, P.mz, T, threadIdx.x, threadIdx.y);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (threadIdx.x == 0 && hi >= lo) {
    atomicMin(rmin + k0 + slot, mi_ord(lo));
    atomicMax(rmax + k0 + slot, mi_ord(hi));
  }
}

// Joint histogram of each transform: static bins sbin (uint8 per voxel) and
// the warped image's bins in its range.
template <typename TM>
__global__ void __launch_bounds__(256) k_mi_hist(const TM* __restrict__ mov, MiParams P,
                                                 const Xform* __restrict__ xf, int k0,
                                                 const unsigned char* __restrict__ sbin,
                                                 const unsigned* __restrict__ rmin,
                                                 const unsigned* __restrict__ rmax,
                                                 unsigned* __restrict__ hist) {
  __shared__ TileBase T;
  const int slot = blockIdx.z / P.vz;
  const int z = blockIdx.z - slot * P.vz;
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
  if (threadIdx.x == 0 && threadIdx.y == 0) tile_base(xf + k0 + slot, x0, y0, z, T);
  __syncthreads();
  const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  int key = -1;
  if (x < P.vx && y < P.vy) {
    const float v = tile_sample<3, TM>(mov, P.mx, P.my, P.mz, T, threadIdx.x, threadIdx.y);
    const float lo = mi_unord(rmin[k0 + slot]), hi = mi_unord(rmax[k0 + slot]);
    const int wb = mi_bin(v, lo, mi_scale(lo, hi));
    const int sb = sbin[((size_t)z * P.vy + y) * P.vx + x];
    if (wb >= 0 && wb < kMiBins)
      key = P.warped_is_high_res ? sb + kMiBins * wb : wb + kMiBins * sb;
  }
  // voxels of a warp that share a bin add once
  const unsigned peers = __match_any_sync(0xffffffffu, key);
  const int lane = threadIdx.x;  // blockDim.x == 32: one warp per row
  if (key >= 0 && lane == __ffs(peers) - 1)
    atomicAdd(hist + (size_t)(k0 + slot) * kMiHist + key, (unsigned)__popc(peers));
}

// NMI of each transform from its joint histogram; one CTA per transform.
// h_static: entropy of the static image; voxels: virtual-grid size.
__global__ void __launch_bounds__(1024) k_mi_nmi(const unsigned* __restrict__ hist, int k0,
                                                 int warped_is_high_res, double h_static,
                                                 double voxels, double* __restrict__ out) {
  __shared__ unsigned marg[kMiBins];
  __shared__ double red[2][32];
  const int k = k0 + blockIdx.x;
  const unsigned* h = hist + (size_t)k * kMiHist;
  const int tid = threadIdx.x;
  for (int i = tid; i < kMiBins; i += blockDim.x) marg[i] = 0;
  __syncthreads();
  double sj = 0.0;
  for (int i = tid; i < kMiHist; i += blockDim.x) {
    const unsigned c = h[i];
    if (c) {
      sj += (double)c * log((double)c);
      atomicAdd(&marg[warped_is_high_res ? (i >> 8) : (i & 255)], c);
    }
  }
  __syncthreads();
  double sw = 0.0;
  for (int i = tid; i < kMiBins; i += blockDim.x) {
    const unsigned c = marg[i];
    if (c) sw += (double)c * log((double)c);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sj += __shfl_down_sync(0xffffffffu, sj, o);
    sw += __shfl_down_sync(0xffffffffu, sw, o);
  }
  if ((tid & 31) == 0) {
    red[0][tid >> 5] = sj;
    red[1][tid >> 5] = sw;
  }
  __syncthreads();
  if (tid == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += red[0][w];
      b += red[1][w];
    }
    const double ln_n = log(voxels);
    const double hj = ln_n - a / voxels;  // H(U, M)
    const double hw = ln_n - b / voxels;  // H(warped)
    double v = (h_static + hw) / hj;
    if (isnan(v) || isinf(v)) v = 0.0;
    out[k] = v;
  }
}

}  // namespace lc2
