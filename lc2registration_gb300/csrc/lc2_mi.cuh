// lc2_mi.cuh -- normalised mutual information, the similarity of
// PatchSize 0 (src/Interpolator/interpolator.cu:617-622;
// src/cu_LC2/cu_lc2_3d.cu:868-923, 1196-1301):
//   NMI = (H(U) + H(M)) / H(U, M)
// over the virtual grid, with 256 bins per image between the image's own
// minimum and maximum, H(X) = -sum p ln p, p = count / voxels, and the joint
// histogram indexed ultrasound bin + 256 * high-resolution bin.
//
// One image is static (the fixed one resampled once): its bins and entropy
// are computed once per context. Per batch of transforms four kernels run:
// the range of the warped image (ordered-integer atomics, one pair per CTA),
// the joint histogram (warp-aggregated integer atomics into a 256 KB
// histogram per transform, which stays in L2), the entropy sums of slices of
// each histogram (kMiParts CTAs per transform) and their combination in a
// fixed order. The range and histogram CTAs each own a 32 x 8 tile over a
// chunk of kMiChunk slices: the tile's sampling bases for all its slices are
// computed up front, one per thread, so the slices then stream without
// barriers; the bases are those of the generic warp kernel (tile_base), so
// the warped values are bit-identical to it. Counts are exact integers and
// the double sums run in a fixed order, so the value does not depend on the
// launch shape or the batch.
#pragma once

#include "lc2_kernels.cuh"

namespace lc2 {

constexpr int kMiBins = 256;
constexpr int kMiHist = kMiBins * kMiBins;

struct MiParams {
  int mx, my, mz;         // warped (moving) image
  int vx, vy, vz;         // virtual grid
  int warped_is_high_res; // 1: key = static bin + 256 * warped bin; 0: the transpose
  int zchunk;             // slices per range / histogram CTA, <= kMiChunk
  int table;              // k_mi_hist merges counts in a shared table first
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

constexpr int kMiChunk = 64;  // most slices per range / histogram CTA
constexpr int kMiParts = 32;  // entropy CTAs per transform (8 warped bins each)

// Sampling bases of a CTA's tile for its slices [zb, ze), one per thread, in
// shared memory, and whether each slice samples strictly inside the warped
// image (tile_inside); the caller synchronises.
__device__ __forceinline__ void mi_bases(const Xform* X, const MiParams& P, int x0, int y0,
                                         int zb, int ze, TileBase* T, int* inside) {
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  if (zb + t < ze) {
    tile_base(X, x0, y0, zb + t, T[t]);
    inside[t] = tile_inside(T[t], P.mx, P.my, P.mz) ? 1 : 0;
  }
}

template <typename TM>
__device__ __forceinline__ float mi_sample(const TM* __restrict__ mov, const MiParams& P,
                                           const TileBase& T, int inside) {
  return inside ? tile_sample_inside<TM>(mov, P.mx, P.my, T, threadIdx.x, threadIdx.y)
                : tile_sample<3, TM>(mov, P.mx, P.my, P.mz, T, threadIdx.x, threadIdx.y);
}

// Range of the warped image of each transform. Grid (tiles of 32 x 8, z
// chunks, transforms), block (32, 8).
template <typename TM>
__global__ void __launch_bounds__(256) k_mi_range(const TM* __restrict__ mov, MiParams P,
                                                  const Xform* __restrict__ xf, int k0,
                                                  unsigned* __restrict__ rmin,
                                                  unsigned* __restrict__ rmax) {
  __shared__ TileBase T[kMiChunk];
  __shared__ int inside[kMiChunk];
  __shared__ float red[2][8];
  const int ntx = (P.vx + 31) / 32;
  const int x0 = (blockIdx.x % ntx) * 32, y0 = (blockIdx.x / ntx) * 8;
  const int zb = blockIdx.y * P.zchunk, ze = min(zb + P.zchunk, P.vz);
  const int slot = blockIdx.z;
  mi_bases(xf + k0 + slot, P, x0, y0, zb, ze, T, inside);
  __syncthreads();
  const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  float lo = INFINITY, hi = -INFINITY;
  if (x < P.vx && y < P.vy) {
    for (int z = zb; z < ze; ++z) {
      const float v = mi_sample<TM>(mov, P, T[z - zb], inside[z - zb]);
      lo = fminf(lo, v);
      hi = fmaxf(hi, v);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (threadIdx.x == 0) {
    red[0][threadIdx.y] = lo;
    red[1][threadIdx.y] = hi;
  }
  __syncthreads();
  if (threadIdx.y == 0 && threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) {
      lo = fminf(lo, red[0][w]);
      hi = fmaxf(hi, red[1][w]);
    }
    if (hi >= lo) {
      atomicMin(rmin + k0 + slot, mi_ord(lo));
      atomicMax(rmax + k0 + slot, mi_ord(hi));
    }
  }
}

// Shared aggregation table of k_mi_hist: (key, count) slots filled by
// open addressing; a key that finds no slot within kMiProbes probes goes
// straight to the global histogram, so every count lands exactly once.
constexpr int kMiTable = 2048;
constexpr int kMiProbes = 32;

__device__ __forceinline__ void mi_table_add(int* tkey, unsigned* tcnt, unsigned* h, int key,
                                             unsigned n) {
  int slot = (int)(((unsigned)key * 2654435761u) >> 21);  // 11-bit Fibonacci hash
  for (int i = 0; i < kMiProbes; ++i) {
    int k = *(volatile int*)&tkey[slot];
    if (k == -1) {
      k = atomicCAS(&tkey[slot], -1, key);
      if (k == -1) k = key;  // this thread claimed the slot
    }
    if (k == key) {
      atomicAdd(&tcnt[slot], n);
      return;
    }
    slot = (slot + 1) & (kMiTable - 1);
  }
  atomicAdd(h + key, n);
}

// Joint histogram of each transform: static bins sbin (uint8 per voxel) and
// the warped image's bins in its range. Grid and block as k_mi_range. With
// P.table a CTA first merges its counts in a shared table (neighbouring
// voxels share bins), then adds each key once.
template <typename TM>
__global__ void __launch_bounds__(256) k_mi_hist(const TM* __restrict__ mov, MiParams P,
                                                 const Xform* __restrict__ xf, int k0,
                                                 const unsigned char* __restrict__ sbin,
                                                 const unsigned* __restrict__ rmin,
                                                 const unsigned* __restrict__ rmax,
                                                 unsigned* __restrict__ hist) {
  __shared__ TileBase T[kMiChunk];
  __shared__ int inside[kMiChunk];
  __shared__ int tkey[kMiTable];
  __shared__ unsigned tcnt[kMiTable];
  const int ntx = (P.vx + 31) / 32;
  const int x0 = (blockIdx.x % ntx) * 32, y0 = (blockIdx.x / ntx) * 8;
  const int zb = blockIdx.y * P.zchunk, ze = min(zb + P.zchunk, P.vz);
  const int slot = blockIdx.z;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const bool table = P.table != 0;
  if (table) {
    for (int i = tid; i < kMiTable; i += 256) {
      tkey[i] = -1;
      tcnt[i] = 0;
    }
  }
  mi_bases(xf + k0 + slot, P, x0, y0, zb, ze, T, inside);
  __syncthreads();
  const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  const bool in = x < P.vx && y < P.vy;
  const float lo = mi_unord(rmin[k0 + slot]), hi = mi_unord(rmax[k0 + slot]);
  const float sc = mi_scale(lo, hi);
  unsigned* h = hist + (size_t)(k0 + slot) * kMiHist;
  const int lane = threadIdx.x;  // blockDim.x == 32: one warp per row
  for (int z = zb; z < ze; ++z) {
    int key = -1;
    if (in) {
      const float v = mi_sample<TM>(mov, P, T[z - zb], inside[z - zb]);
      const int wb = mi_bin(v, lo, sc);
      const int sb = sbin[((size_t)z * P.vy + y) * P.vx + x];
      if (wb >= 0 && wb < kMiBins)
        key = P.warped_is_high_res ? sb + kMiBins * wb : wb + kMiBins * sb;
    }
    // voxels of a warp that share a bin add once
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && lane == __ffs(peers) - 1) {
      if (table)
        mi_table_add(tkey, tcnt, h, key, (unsigned)__popc(peers));
      else
        atomicAdd(h + key, (unsigned)__popc(peers));
    }
  }
  if (table) {
    __syncthreads();
    for (int i = tid; i < kMiTable; i += 256)
      if (tkey[i] >= 0) atomicAdd(h + tkey[i], tcnt[i]);
  }
}

// Entropy sums of one part of each joint histogram: part b holds the warped
// bins [8b, 8b + 8) -- the rows of the histogram (key = static + 256 warped)
// or its columns (key = warped + 256 static). part[k][b] = (sum over its
// joint bins of c ln c, sum over its warped marginals of c ln c). Grid
// (kMiParts, transforms), 256 threads.
__global__ void __launch_bounds__(256) k_mi_part(const unsigned* __restrict__ hist, int k0,
                                                 int warped_is_high_res,
                                                 double* __restrict__ part) {
  constexpr int WB = kMiBins / kMiParts;  // warped bins per part
  __shared__ unsigned marg[WB];
  __shared__ double red[2][8];
  const int k = k0 + blockIdx.y, b = blockIdx.x, tid = threadIdx.x;
  const unsigned* h = hist + (size_t)k * kMiHist;
  if (tid < WB) marg[tid] = 0;
  __syncthreads();
  double sj = 0.0;
#pragma unroll
  for (int j = 0; j < WB; ++j) {
    // rows: warped bin WB b + j, static bin tid; columns: warped bin
    // WB b + (tid & 7), static bin (tid >> 3) + 32 j
    const int wl = warped_is_high_res ? j : (tid & (WB - 1));
    const int sbn = warped_is_high_res ? tid : (tid >> 3) + 32 * j;
    const int w = WB * b + wl;
    const unsigned c = warped_is_high_res ? h[sbn + kMiBins * w] : h[w + kMiBins * sbn];
    if (c) {
      sj += (double)c * log((double)c);
      atomicAdd(&marg[wl], c);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sj += __shfl_down_sync(0xffffffffu, sj, o);
  if ((tid & 31) == 0) red[0][tid >> 5] = sj;
  __syncthreads();
  if (tid == 0) {
    double a = 0.0, m = 0.0;
    for (int w = 0; w < 8; ++w) a += red[0][w];
    for (int i = 0; i < WB; ++i)
      if (marg[i]) m += (double)marg[i] * log((double)marg[i]);
    part[((size_t)k * kMiParts + b) * 2] = a;
    part[((size_t)k * kMiParts + b) * 2 + 1] = m;
  }
}

// NMI of each transform from its parts, summed in part order.
// h_static: entropy of the static image; voxels: virtual-grid size.
__global__ void k_mi_nmi(const double* __restrict__ part, int cnt, double h_static,
                         double voxels, double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  double a = 0.0, b = 0.0;
  for (int i = 0; i < kMiParts; ++i) {
    a += part[((size_t)k * kMiParts + i) * 2];
    b += part[((size_t)k * kMiParts + i) * 2 + 1];
  }
  const double ln_n = log(voxels);
  const double hj = ln_n - a / voxels;  // H(U, M)
  const double hw = ln_n - b / voxels;  // H(warped)
  double v = (h_static + hw) / hj;
  if (isnan(v) || isinf(v)) v = 0.0;
  out[k] = v;
}

}  // namespace lc2
