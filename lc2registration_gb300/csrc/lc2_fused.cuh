// lc2_fused.cuh -- fused LC2 evaluation kernel for a static ultrasound
// (HighResolutionModality: Moving, the moving MR/CT is resampled).
//
// One CTA owns a 32 x TY tile of output columns of one transform and marches
// along z through `zchunk` output slices. Per input slice e it
//   1. resamples the moving volume at the tile's halo region (+1 for Sobel)
//      into a 3-slice shared ring (src/Interpolator/interpolator.cu:69-179),
//   2. takes the Sobel magnitude of slice e from the ring
//      (src/cu_LC2/cu_lc2_3d.cu:100-179) and updates, in registers, the exact
//      z-window sums of the patch moments of its halo points; the fields of
//      the slice leaving the window are replayed from a quantised shared ring,
//   3. runs the x and y window passes in shared memory, and
//   4. solves each output voxel's least-squares fit against the precomputed
//      weighting factor sigma (cu_lc2_3d.cu:526-618) and adds its clipped
//      measure to the transform's exact fixed-point sum.
// Nothing is written to global memory except the per-transform sum, so the
// moving volume stays resident in L2 while many transforms are evaluated.
// ND = 2 covers the 2D and 2D-to-3D modes: one slice, no z window; WND is the
// dimensionality of the resampling (3 for 2D-to-3D).
#pragma once

#include "lc2_kernels.cuh"

namespace lc2 {

struct FusedParams {
  int vx, vy, vz;       // virtual grid
  int mx, my, mz;       // moving volume
  int r, n;             // patch radius, patch voxels
  int zchunk;           // output slices per CTA (3D)
  int ntx;              // tiles along x
  float qu, qm, qg;     // fixed-point scales
  long long thr_m, thr_g;  // degenerate-column thresholds (see MomentParams)
  float sig_scale;      // sigma = sqrt(D_uu) * sig_scale
  float sum_scale;      // fixed-point scale of the measure sum
};

constexpr int kF32 = 3;  // U, M, G
constexpr int kF64 = 5;  // UM, UG, MM, GG, MG

template <int TY>
struct FusedLayout {
  static constexpr int NT = 32 * TY;
  static constexpr int MAXP = (TY == 16) ? 3 : 4;  // z-window halo points per thread
};

// Shared-memory carve-up of one fused CTA (sizes depend on r at run time).
struct FusedSmem {
  int pw, ph;       // resampled region (tile + 2r + 2)
  int hx, hy, hxp;  // patch halo region (tile + 2r), pitch
  int txp;
  int ring;         // 2r + 2 slices in the leaving ring
  float* mring;     // [3][ph][pw]
  int* lv;          // [ring][hy][hx][2]  quantised (M, G) of past slices
  int* z32;         // [kF32][hy][hxp]; reused as y32 [kF32][TY][txp]
  long long* z64;   // [kF64][hy][hxp]; reused as y64 [kF64][TY][txp]
  int* x32;         // [kF32][hy][txp]
  long long* x64;   // [kF64][hy][txp]
};

__host__ __device__ inline size_t fused_smem_bytes(int r, int ty, int nd) {
  const int pw = 32 + 2 * r + 2, ph = ty + 2 * r + 2;
  const int hx = 32 + 2 * r, hy = ty + 2 * r, hxp = hx | 1, txp = 33;
  const int ring = (nd == 3) ? 2 * r + 2 : 0;
  size_t b = 0;
  b += sizeof(float) * (nd == 3 ? 3 : 1) * pw * ph;
  b += sizeof(int) * 2 * (size_t)ring * hy * hx;
  b = (b + 15) & ~(size_t)15;
  size_t z = (size_t)hy * hxp;
  b += sizeof(int) * kF32 * z;
  b = (b + 15) & ~(size_t)15;
  b += sizeof(long long) * kF64 * z;
  size_t x = (size_t)hy * txp;
  b += sizeof(int) * kF32 * x;
  b = (b + 15) & ~(size_t)15;
  b += sizeof(long long) * kF64 * x;
  return b;
}

__device__ inline FusedSmem fused_carve(unsigned char* base, int r, int ty, int nd) {
  FusedSmem s;
  s.pw = 32 + 2 * r + 2;
  s.ph = ty + 2 * r + 2;
  s.hx = 32 + 2 * r;
  s.hy = ty + 2 * r;
  s.hxp = s.hx | 1;
  s.txp = 33;
  s.ring = (nd == 3) ? 2 * r + 2 : 0;
  size_t b = 0;
  s.mring = reinterpret_cast<float*>(base);
  b += sizeof(float) * (nd == 3 ? 3 : 1) * s.pw * s.ph;
  s.lv = reinterpret_cast<int*>(base + b);
  b += sizeof(int) * 2 * (size_t)s.ring * s.hy * s.hx;
  b = (b + 15) & ~(size_t)15;
  size_t z = (size_t)s.hy * s.hxp;
  s.z32 = reinterpret_cast<int*>(base + b);
  b += sizeof(int) * kF32 * z;
  b = (b + 15) & ~(size_t)15;
  s.z64 = reinterpret_cast<long long*>(base + b);
  b += sizeof(long long) * kF64 * z;
  size_t x = (size_t)s.hy * s.txp;
  s.x32 = reinterpret_cast<int*>(base + b);
  b += sizeof(int) * kF32 * x;
  b = (b + 15) & ~(size_t)15;
  s.x64 = reinterpret_cast<long long*>(base + b);
  return s;
}

// Resample the moving volume on the (pw x ph) region of slice s into ring
// slot `slot`. The region's base coordinate (integer part and fraction) was
// computed in double by thread 0 (sb, sf).
template <int WND, typename TM, int NT>
__device__ __forceinline__ void fused_warp(const TM* __restrict__ mov, const FusedParams& P,
                                           const FusedSmem& s, const float* A, const int* sb,
                                           const float* sf, int gx0, int gy0, int zs,
                                           float* dst) {
  const bool zin = (zs >= 0 && zs < P.vz);
  for (int i = threadIdx.x; i < s.pw * s.ph; i += NT) {
    const int px = i % s.pw, py = i / s.pw;
    const int gx = gx0 + px, gy = gy0 + py;
    float v = 0.0f;
    if (zin && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy) {
      const float dx = (float)px, dy = (float)py;
      float qx = fmaf(A[1], dy, fmaf(A[0], dx, sf[0]));
      float qy = fmaf(A[4], dy, fmaf(A[3], dx, sf[1]));
      Axis ax = make_axis(sb[0], qx, P.mx);
      Axis ay = make_axis(sb[1], qy, P.my);
      if (WND == 3) {
        float qz = fmaf(A[7], dy, fmaf(A[6], dx, sf[2]));
        Axis az = make_axis(sb[2], qz, P.mz);
        if (ax.ok && ay.ok && az.ok) {
          const size_t sy = (size_t)P.mx, sz = (size_t)P.mx * P.my;
          const size_t zf = az.f * sz, zc = az.c * sz, yf = ay.f * sy, yc = ay.c * sy;
          float lu0 = ldf(mov, ax.f + yf + zf), lu1 = ldf(mov, ax.f + yf + zc);
          float ru0 = ldf(mov, ax.c + yf + zf), ru1 = ldf(mov, ax.c + yf + zc);
          float rb0 = ldf(mov, ax.c + yc + zf), rb1 = ldf(mov, ax.c + yc + zc);
          float lb0 = ldf(mov, ax.f + yc + zf), lb1 = ldf(mov, ax.f + yc + zc);
          float lu = fmaf(az.r, lu1 - lu0, lu0), ru = fmaf(az.r, ru1 - ru0, ru0);
          float rb = fmaf(az.r, rb1 - rb0, rb0), lb = fmaf(az.r, lb1 - lb0, lb0);
          float l = fmaf(ay.r, lb - lu, lu), r = fmaf(ay.r, rb - ru, ru);
          v = fmaf(ax.r, r - l, l);
        }
      } else {
        if (ax.ok && ay.ok) {
          const size_t yf = (size_t)ay.f * P.mx, yc = (size_t)ay.c * P.mx;
          float f0 = ldf(mov, ax.f + yf), f1 = ldf(mov, ax.f + yc);
          float c0 = ldf(mov, ax.c + yf), c1 = ldf(mov, ax.c + yc);
          float xl = fmaf(ay.r, f1 - f0, f0), xr = fmaf(ay.r, c1 - c0, c0);
          v = fmaf(ax.r, xr - xl, xl);
        }
      }
    }
    dst[i] = v;
  }
}

// x and y window passes over the z planes (same scheme as mom_xy_passes, on
// the fused field set). Output lands in the (aliased) y planes.
template <int TY, int NT>
__device__ __forceinline__ void fused_xy(const FusedSmem& s, int r) {
  const int tid = threadIdx.x, w = 2 * r + 1;
  const size_t pz = (size_t)s.hy * s.hxp, px = (size_t)s.hy * s.txp, py = (size_t)TY * s.txp;
  {
    constexpr int nseg = 32 / kSegX;
    const int items = (kF32 + kF64) * nseg * s.hy;
    for (int it = tid; it < items; it += NT) {
      const int row = it % s.hy, rest = it / s.hy, seg = rest % nseg, f = rest / nseg;
      const int x = seg * kSegX;
      if (f < kF32) {
        const int* src = s.z32 + f * pz + (size_t)row * s.hxp;
        int* dst = s.x32 + f * px + (size_t)row * s.txp;
        int a = 0;
        for (int i = 0; i < w; ++i) a += src[x + i];
        dst[x] = a;
#pragma unroll
        for (int j = 1; j < kSegX; ++j) {
          a += src[x + j + w - 1] - src[x + j - 1];
          dst[x + j] = a;
        }
      } else {
        const long long* src = s.z64 + (f - kF32) * pz + (size_t)row * s.hxp;
        long long* dst = s.x64 + (f - kF32) * px + (size_t)row * s.txp;
        long long a = 0;
        for (int i = 0; i < w; ++i) a += src[x + i];
        dst[x] = a;
#pragma unroll
        for (int j = 1; j < kSegX; ++j) {
          a += src[x + j + w - 1] - src[x + j - 1];
          dst[x + j] = a;
        }
      }
    }
  }
  __syncthreads();
  {
    constexpr int segy = 4;
    constexpr int nseg = TY / segy;
    const int items = (kF32 + kF64) * nseg * 32;
    for (int it = tid; it < items; it += NT) {
      const int col = it % 32, rest = it / 32, seg = rest % nseg, f = rest / nseg;
      const int y = seg * segy;
      if (f < kF32) {
        const int* src = s.x32 + f * px + col;
        int* dst = s.z32 + f * py + col;  // y planes alias the z planes
        int a = 0;
        for (int i = 0; i < w; ++i) a += src[(size_t)(y + i) * s.txp];
        dst[(size_t)y * s.txp] = a;
#pragma unroll
        for (int j = 1; j < segy; ++j) {
          a += src[(size_t)(y + j + w - 1) * s.txp] - src[(size_t)(y + j - 1) * s.txp];
          dst[(size_t)(y + j) * s.txp] = a;
        }
      } else {
        const long long* src = s.x64 + (f - kF32) * px + col;
        long long* dst = s.z64 + (f - kF32) * py + col;
        long long a = 0;
        for (int i = 0; i < w; ++i) a += src[(size_t)(y + i) * s.txp];
        dst[(size_t)y * s.txp] = a;
#pragma unroll
        for (int j = 1; j < segy; ++j) {
          a += src[(size_t)(y + j + w - 1) * s.txp] - src[(size_t)(y + j - 1) * s.txp];
          dst[(size_t)(y + j) * s.txp] = a;
        }
      }
    }
  }
  __syncthreads();
}

// Clipped measure of one voxel from exact sums; sigma > 0 is the
// precomputed weighting factor (0 marks an invalid patch).
__device__ __forceinline__ float fused_solve(const FusedParams& P, float sigma, int s_u, int s_m,
                                             int s_g, long long s_um, long long s_ug,
                                             long long s_mm, long long s_gg, long long s_mg) {
  const long long n = P.n;
  long long d_mm = n * s_mm - (long long)s_m * s_m;
  long long d_gg = n * s_gg - (long long)s_g * s_g;
  long long d_mg = n * s_mg - (long long)s_m * s_g;
  long long d_um = n * s_um - (long long)s_u * s_m;
  long long d_ug = n * s_ug - (long long)s_u * s_g;
  const bool km = d_mm > P.thr_m, kg = d_gg > P.thr_g;
  const float iu = P.sig_scale / sigma;  // 1/sqrt(D_uu)
  float r2 = 0.0f;
  if (km && kg) {
    float im = rsqrtf((float)d_mm), ig = rsqrtf((float)d_gg);
    float rum = (float)d_um * iu * im, rug = (float)d_ug * iu * ig, rmg = (float)d_mg * im * ig;
    float den = 1.0f - rmg * rmg;
    if (den > 1e-3f) {
      r2 = (rum * rum + rug * rug - 2.0f * rum * rug * rmg) / den;
    } else {
      double dmm = (double)d_mm, dgg = (double)d_gg, dmg = (double)d_mg;
      double dum = (double)d_um, dug = (double)d_ug;
      double det = dmm * dgg - dmg * dmg;
      double e;
      if (det <= 1e-10 * dmm * dgg)
        e = dum * dum / dmm;
      else
        e = (dgg * dum * dum - 2.0 * dmg * dum * dug + dmm * dug * dug) / det;
      double iud = (double)iu;
      r2 = (float)(e * iud * iud);
    }
  } else if (km) {
    float c = (float)d_um * iu * rsqrtf((float)d_mm);
    r2 = c * c;
  } else if (kg) {
    float c = (float)d_ug * iu * rsqrtf((float)d_gg);
    r2 = c * c;
  }
  float m = sigma * r2;
  if (!(m > 0.0f) || isinf(m)) m = 0.0f;
  return m;
}

template <int ND>
__device__ __forceinline__ float sobel_at(const FusedSmem& s, int e, int hx, int hy) {
  // M ring coordinates of the point: (hx + 1, hy + 1); slices e-1, e, e+1
  const int cx = hx + 1, cy = hy + 1;
  if (ND == 3) {
    const float* m0 = s.mring + (size_t)(((e - 1) % 3 + 3) % 3) * s.pw * s.ph;
    const float* m1 = s.mring + (size_t)((e % 3 + 3) % 3) * s.pw * s.ph;
    const float* m2 = s.mring + (size_t)(((e + 1) % 3 + 3) % 3) * s.pw * s.ph;
    float gx = 0.f, gy = 0.f, gz = 0.f;
    float srow[3][3], drow[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int o = (cy + j - 1) * s.pw + (cx + i - 1);
        const float a = m0[o], b = m1[o], c = m2[o];
        srow[j][i] = a + 2.0f * b + c;
        drow[j][i] = c - a;
      }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float hj = (j == 1) ? 2.0f : 1.0f, hpj = (float)(j - 1);
      gx += hj * (srow[j][2] - srow[j][0]);
      gy += hpj * (srow[j][0] + 2.0f * srow[j][1] + srow[j][2]);
      gz += hj * (drow[j][0] + 2.0f * drow[j][1] + drow[j][2]);
    }
    return sqrtf(gx * gx + gy * gy + gz * gz);
  } else {
    const float* m1 = s.mring;
    float gx = 0.f, gy = 0.f;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float hj = (j == 1) ? 2.0f : 1.0f, hpj = (float)(j - 1);
      const int o = (cy + j - 1) * s.pw + cx;
      const float a = m1[o - 1], b = m1[o], c = m1[o + 1];
      gx += hj * (c - a);
      gy += hpj * (a + 2.0f * b + c);
    }
    return sqrtf(gx * gx + gy * gy);
  }
}

template <int ND, int WND, typename TM, typename TS, int TY>
__global__ void __launch_bounds__(32 * TY) k_fused(const TM* __restrict__ mov,
                                                   const TS* __restrict__ Ust,
                                                   const float* __restrict__ sig, FusedParams P,
                                                   const Xform* __restrict__ xf, int k0,
                                                   unsigned long long* __restrict__ acc,
                                                   float* __restrict__ out_measure) {
  constexpr int NT = FusedLayout<TY>::NT;
  constexpr int MAXP = FusedLayout<TY>::MAXP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double s_base[3];
  __shared__ int s_ib[3];
  __shared__ float s_fb[3];
  __shared__ float s_A[9];
  const int r = P.r;
  const FusedSmem s = fused_carve(smem_raw, r, TY, ND);
  const int tid = threadIdx.x;
  const int slot = blockIdx.x;
  const int tile = blockIdx.y;
  const int x0 = (tile % P.ntx) * 32, y0 = (tile / P.ntx) * TY;
  const int zb = blockIdx.z * P.zchunk;
  const int ze = min(zb + P.zchunk, P.vz);
  const Xform* X = xf + k0 + slot;
  const int gx0 = x0 - r - 1, gy0 = y0 - r - 1;  // origin of the resampled region
  const size_t pz = (size_t)s.hy * s.hxp;
  const size_t ps = (size_t)s.pw * s.ph;
  const int np = s.hx * s.hy;

  // thread 0: base coordinate of the region at slice zs (double), split into
  // integer part and fraction for the float per-voxel offsets
  auto set_base = [&](int zs) {
    if (tid == 0) {
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        double p = s_base[a] + X->A[3 * a + 2] * (double)zs;
        double fl = floor(p);
        s_ib[a] = (int)fl;
        s_fb[a] = (float)(p - fl);
      }
    }
  };
  if (tid == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a)
      s_base[a] = X->A[3 * a + 0] * gx0 + X->A[3 * a + 1] * gy0 + X->b[a];
#pragma unroll
    for (int i = 0; i < 9; ++i) s_A[i] = (float)X->A[i];
  }
  long long acc_m = 0;

  if (ND == 2) {
    set_base(0);
    __syncthreads();
    fused_warp<WND, TM, NT>(mov, P, s, s_A, s_ib, s_fb, gx0, gy0, 0, s.mring);
    __syncthreads();
    for (int p = tid; p < np; p += NT) {
      const int hx = p % s.hx, hy = p / s.hx;
      const int gx = x0 - r + hx, gy = y0 - r + hy;
      const float m = s.mring[(hy + 1) * s.pw + hx + 1];
      const float g = sobel_at<2>(s, 0, hx, hy);
      float u = 0.0f;
      if (gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy) u = ldf(Ust, (size_t)gy * P.vx + gx);
      const int qu = quant(u, P.qu), qm = quant(m, P.qm), qg = quant(g, P.qg);
      const size_t o = (size_t)hy * s.hxp + hx;
      s.z32[o] = qu;
      s.z32[pz + o] = qm;
      s.z32[2 * pz + o] = qg;
      s.z64[o] = (long long)qu * qm;
      s.z64[pz + o] = (long long)qu * qg;
      s.z64[2 * pz + o] = (long long)qm * qm;
      s.z64[3 * pz + o] = (long long)qg * qg;
      s.z64[4 * pz + o] = (long long)qm * qg;
    }
    __syncthreads();
    fused_xy<TY, NT>(s, r);
    const int ox = tid % 32, oy = tid / 32;
    const int x = x0 + ox, y = y0 + oy;
    if (x < P.vx && y < P.vy) {
      const size_t gi = (size_t)y * P.vx + x;
      const float sg = __ldg(sig + gi);
      float m = 0.0f;
      if (sg > 0.0f) {
        const size_t o = (size_t)oy * s.txp + ox, py = (size_t)TY * s.txp;
        m = fused_solve(P, sg, s.z32[o], s.z32[py + o], s.z32[2 * py + o], s.z64[o],
                        s.z64[py + o], s.z64[2 * py + o], s.z64[3 * py + o], s.z64[4 * py + o]);
        acc_m += __float2int_rn(m * P.sum_scale);
      }
      if (out_measure && slot == 0) out_measure[gi] = m;
    }
  } else {
    // ---- 3D: z-marching over output slices [zb, ze) ----
    int a32[MAXP][kF32];
    long long a64[MAXP][kF64];
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
#pragma unroll
      for (int k = 0; k < kF32; ++k) a32[j][k] = 0;
#pragma unroll
      for (int k = 0; k < kF64; ++k) a64[j][k] = 0;
    }
    const int e0 = zb - r;  // first slice entering the window
    // resample slices e0-1 and e0 into the ring
    set_base(e0 - 1);
    __syncthreads();
    fused_warp<3, TM, NT>(mov, P, s, s_A, s_ib, s_fb, gx0, gy0, e0 - 1,
                          s.mring + (size_t)(((e0 - 1) % 3 + 3) % 3) * ps);
    __syncthreads();
    set_base(e0);
    __syncthreads();
    fused_warp<3, TM, NT>(mov, P, s, s_A, s_ib, s_fb, gx0, gy0, e0,
                          s.mring + (size_t)((e0 % 3 + 3) % 3) * ps);
    __syncthreads();
    set_base(e0 + 1);
    __syncthreads();
    const int ox = tid % 32, oy = tid / 32;
    for (int e = e0; e < ze + r; ++e) {
      // resample slice e+1 (its base was set before the last barrier)
      fused_warp<3, TM, NT>(mov, P, s, s_A, s_ib, s_fb, gx0, gy0, e + 1,
                            s.mring + (size_t)(((e + 1) % 3 + 3) % 3) * ps);
      __syncthreads();
      if (tid == 0) set_base(e + 2);
      const int z = e - r;       // output slice completed by this entering slice
      const int l = e - 2 * r - 1;  // slice leaving the window
      const bool out = (z >= zb);
      const bool leave = (l >= e0);
      int* lv_in = s.lv + (size_t)(((e % s.ring) + s.ring) % s.ring) * np * 2;
      const int* lv_out = s.lv + (size_t)(((l % s.ring) + s.ring) % s.ring) * np * 2;
      const bool ezin = (e >= 0 && e < P.vz), lzin = (l >= 0 && l < P.vz);
#pragma unroll
      for (int j = 0; j < MAXP; ++j) {
        const int p = tid + j * NT;
        if (p < np) {
          const int hx = p % s.hx, hy = p / s.hx;
          const int gx = x0 - r + hx, gy = y0 - r + hy;
          const bool xyin = gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy;
          const float m = s.mring[(size_t)((e % 3 + 3) % 3) * ps + (hy + 1) * s.pw + hx + 1];
          const float g = sobel_at<3>(s, e, hx, hy);
          float u = 0.0f;
          if (xyin && ezin) u = ldf(Ust, ((size_t)e * P.vy + gy) * P.vx + gx);
          const int qu = quant(u, P.qu), qm = quant(m, P.qm), qg = quant(g, P.qg);
          lv_in[2 * p] = qm;
          lv_in[2 * p + 1] = qg;
          a32[j][0] += qu;
          a32[j][1] += qm;
          a32[j][2] += qg;
          a64[j][0] += (long long)qu * qm;
          a64[j][1] += (long long)qu * qg;
          a64[j][2] += (long long)qm * qm;
          a64[j][3] += (long long)qg * qg;
          a64[j][4] += (long long)qm * qg;
          if (leave) {
            const int lm = lv_out[2 * p], lg = lv_out[2 * p + 1];
            float ul = 0.0f;
            if (xyin && lzin) ul = ldf(Ust, ((size_t)l * P.vy + gy) * P.vx + gx);
            const int lu = quant(ul, P.qu);
            a32[j][0] -= lu;
            a32[j][1] -= lm;
            a32[j][2] -= lg;
            a64[j][0] -= (long long)lu * lm;
            a64[j][1] -= (long long)lu * lg;
            a64[j][2] -= (long long)lm * lm;
            a64[j][3] -= (long long)lg * lg;
            a64[j][4] -= (long long)lm * lg;
          }
          if (out) {
            const size_t o = (size_t)hy * s.hxp + hx;
#pragma unroll
            for (int k = 0; k < kF32; ++k) s.z32[k * pz + o] = a32[j][k];
#pragma unroll
            for (int k = 0; k < kF64; ++k) s.z64[k * pz + o] = a64[j][k];
          }
        }
      }
      __syncthreads();
      if (out) {
        fused_xy<TY, NT>(s, r);
        const int x = x0 + ox, y = y0 + oy;
        if (x < P.vx && y < P.vy && z < P.vz) {
          const size_t gi = ((size_t)z * P.vy + y) * P.vx + x;
          const float sg = __ldg(sig + gi);
          float m = 0.0f;
          if (sg > 0.0f) {
            const size_t o = (size_t)oy * s.txp + ox, py = (size_t)TY * s.txp;
            m = fused_solve(P, sg, s.z32[o], s.z32[py + o], s.z32[2 * py + o], s.z64[o],
                            s.z64[py + o], s.z64[2 * py + o], s.z64[3 * py + o],
                            s.z64[4 * py + o]);
            acc_m += __float2int_rn(m * P.sum_scale);
          }
          if (out_measure && slot == 0) out_measure[gi] = m;
        }
        // the next resample writes only the M ring; the z planes (read by
        // this solve) are rewritten after the next barrier
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc_m += __shfl_down_sync(0xffffffffu, acc_m, o);
  if ((tid & 31) == 0) atomicAdd(acc + 2 * (size_t)(k0 + slot), (unsigned long long)acc_m);
}

}  // namespace lc2
