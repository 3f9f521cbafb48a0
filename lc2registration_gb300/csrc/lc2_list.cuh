// lc2_list.cuh -- the fused 2D-window evaluation over a work list.
//
// A work list is a sequence of segments; a segment is `count` evaluations of
// one fixed image (static ultrasound + weighting factors, its own virtual
// grid and fixed-point scales) against one moving image. Every evaluation is
// cut into the 32 x 16 tiles of its fixed image, and the tiles of all
// segments form one range of work units, so frames of uneven sizes (a
// 2D-to-3D frame stack, src/Interpolator/interpolator.cu:1538-1775 run for
// many frames) or 2D registrations of different sizes share one launch.
// The kernel is persistent: a grid of resident CTAs strides over the units,
// and each CTA moves through the segments in order, so the segment of a unit
// is found from the previous one.
#pragma once

#include "lc2_fused.cuh"

namespace lc2 {

struct ListSeg {
  const void* mov;    // moving image (storage type)
  const void* ust;    // static ultrasound on the virtual grid (storage type)
  const float* sig;   // weighting factor per virtual pixel
  const int* su;      // static window sum of the quantised ultrasound per pixel
  FusedParams P;      // grid sizes and fixed-point scales; P.ntx = tiles along x
  int ntiles;         // tiles per evaluation
  int count;          // evaluations in the segment
  int eval0;          // index of its first evaluation (Xform and accumulator)
  int pad_;
  long long unit0;    // first work unit of the segment
};

constexpr int kListTY = 16;

template <int WND, typename T, int R>
__global__ void __launch_bounds__(32 * kListTY, 3)
    k_fused_list(const ListSeg* __restrict__ segs, int nseg, long long units,
                 const Xform* __restrict__ xf, unsigned long long* __restrict__ acc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ ListSeg s_seg;
  __shared__ TileShared s_tile;
  __shared__ int s_cur;
  const int tid = threadIdx.x;
  if (tid == 0) s_cur = -1;
  for (long long u = blockIdx.x; u < units; u += gridDim.x) {
    if (tid == 0) {
      // last segment with unit0 <= u, searched above the current one
      int lo = s_cur < 0 ? 0 : s_cur, hi = nseg - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (segs[mid].unit0 <= u) lo = mid; else hi = mid - 1;
      }
      if (lo != s_cur) {
        s_seg = segs[lo];
        s_cur = lo;
      }
    }
    __syncthreads();
    const long long rel = u - s_seg.unit0;
    const int e = (int)(rel / s_seg.ntiles);
    const int tile = (int)(rel - (long long)e * s_seg.ntiles);
    const int ev = s_seg.eval0 + e;
    long long m = fused_tile_2d<WND, T, T, kListTY, R>(
        (const T*)s_seg.mov, (const T*)s_seg.ust, s_seg.sig, s_seg.su, s_seg.P, xf + ev, tile,
        smem_raw, s_tile,
        nullptr);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m += __shfl_down_sync(0xffffffffu, m, o);
    if ((tid & 31) == 0 && m != 0) atomicAdd(acc + 2 * (size_t)ev, (unsigned long long)m);
    __syncthreads();  // shared planes and s_seg are reused by the next unit
  }
}

struct ListLaunch {
  const ListSeg* segs;  // device
  int nseg;
  long long units;
  const Xform* xf;      // device, indexed by evaluation
  unsigned long long* acc;
  int r, wnd;
  int sms;              // multiprocessors of the device
  cudaStream_t stream;
};

template <int WND, typename T, int R>
cudaError_t list_launch_r(const ListLaunch& L) {
  using G = FusedGeom<2, kListTY, R>;
  auto kern = k_fused_list<WND, T, R>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)G::BYTES);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, G::NT, G::BYTES);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  long long grid = (long long)per_sm * L.sms;
  if (grid > L.units) grid = L.units;
  if (grid < 1) return cudaSuccess;
  kern<<<(unsigned)grid, G::NT, G::BYTES, L.stream>>>(L.segs, L.nseg, L.units, L.xf, L.acc);
  return cudaGetLastError();
}

template <int WND, typename T>
cudaError_t list_launch_w(const ListLaunch& L) {
  switch (L.r) {
    case 1: return list_launch_r<WND, T, 1>(L);
    case 2: return list_launch_r<WND, T, 2>(L);
    case 3: return list_launch_r<WND, T, 3>(L);
    case 4: return list_launch_r<WND, T, 4>(L);
    case 5: return list_launch_r<WND, T, 5>(L);
    case 6: return list_launch_r<WND, T, 6>(L);
    case 7: return list_launch_r<WND, T, 7>(L);
    case 8: return list_launch_r<WND, T, 8>(L);
    case 9: return list_launch_r<WND, T, 9>(L);
    case 10: return list_launch_r<WND, T, 10>(L);
    case 11: return list_launch_r<WND, T, 11>(L);
    case 12: return list_launch_r<WND, T, 12>(L);
  }
  return cudaErrorInvalidValue;
}

// Defined per storage type in lc2_list_{f32,f16,bf16}.cu.
template <typename T>
cudaError_t list_launch(const ListLaunch& L);

template <>
cudaError_t list_launch<float>(const ListLaunch& L);
template <>
cudaError_t list_launch<__half>(const ListLaunch& L);
template <>
cudaError_t list_launch<__nv_bfloat16>(const ListLaunch& L);

#define LC2_DEFINE_LIST_LAUNCH(T)                         \
  template <>                                             \
  cudaError_t list_launch<T>(const ListLaunch& L) {       \
    if (L.wnd == 3) return list_launch_w<3, T>(L);        \
    return list_launch_w<2, T>(L);                        \
  }

}  // namespace lc2
