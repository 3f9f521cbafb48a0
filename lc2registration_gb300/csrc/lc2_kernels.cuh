// lc2_kernels.cuh -- sm_103a kernels of the LC2 similarity path.
//
// Stages of one evaluation (one transform) on the virtual grid:
//   k_warp     trilinear/bilinear resample of the moving image through the
//              transform (src/Interpolator/interpolator.cu:69-232);
//   k_sobel    unnormalised Sobel magnitude with zero padding
//              (src/cu_LC2/cu_lc2_2d.cu:25-86, src/cu_LC2/cu_lc2_3d.cu:100-179);
//   k_moments  per-voxel patch moments, weighting factor sigma
//              (cu_lc2_2d.cu:88-180, cu_lc2_3d.cu:181-287), least-squares
//              fit U ~ a M + b G + c and clipped measure
//              (cu_lc2_2d.cu:182-480, cu_lc2_3d.cu:289-618,769-827), and the
//              sums behind LC2 = sum(measure) / sum(sigma)
//              (cu_lc2_2d.cu:642-648, cu_lc2_3d.cu:1181-1191).
//
// Numerics of k_moments. Patch moments are box sums of 64-bit fixed-point
// values: each of U, M, G is rounded to an integer q = rint(v * Q) with
// |q| <= 2^b, where b is chosen per patch size so that every first-order sum
// fits int32 and every n*S2 - S1^2 fits int64. Box sums, the centring
// n*S_xy - S_x*S_y and the final reduction are therefore exact, independent
// of summation order and of how voxels are tiled or batched; only the
// per-voxel 2x2 solve runs in FP32 (FP64 for nearly collinear columns).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace lc2 {

constexpr int kTX = 32;  // tile width (x) of k_moments, threads per row
constexpr int kTY = 8;   // tile height (y)
constexpr int kNT = kTX * kTY;
constexpr int kMaxP3 = 4;  // halo points per thread in the 3D z-phase (R <= 6)
constexpr int kNF32 = 4;   // int32 planes: sum U, sum M, sum G, invalid count
constexpr int kNF64 = 6;   // int64 planes: UU, MM, GG, UM, UG, MG
constexpr int kSegX = 8;   // x-pass running-sum segment length
constexpr int kSegY = 4;   // y-pass running-sum segment length

template <typename T>
__device__ __forceinline__ float ldf(const T* p, size_t i);
template <>
__device__ __forceinline__ float ldf<float>(const float* p, size_t i) { return __ldg(p + i); }
template <>
__device__ __forceinline__ float ldf<__half>(const __half* p, size_t i) {
  return __half2float(__ldg(p + i));
}
template <>
__device__ __forceinline__ float ldf<__nv_bfloat16>(const __nv_bfloat16* p, size_t i) {
  return __bfloat162float(__ldg(p + i));
}

template <typename T>
__device__ __forceinline__ T stf(float v);
template <>
__device__ __forceinline__ float stf<float>(float v) { return v; }
template <>
__device__ __forceinline__ __half stf<__half>(float v) { return __float2half_rn(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 stf<__nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}

// Moving-pixel coordinates of virtual voxel (x, y, z): p = A (x, y, z) + b.
// Built on the host in double from the row-major mm matrix and the three
// geometries: A = diag(1/spM) L diag(spV), b = diag(1/spM) (L oV + t - oM).
struct XformD {
  double A[9];
  double b[3];
};

// What the kernels read: the float-float split (hi + lo) of A and b; hi
// carries the first 24 significant bits, lo the next 24. 96 bytes.
struct Xform {
  float ah[9], al[9];
  float bh[3], bl[3];
};
static_assert(sizeof(Xform) == 96, "one transform is staged host->device as 96 bytes");

// Host: the split of D.
inline Xform xform_split(const XformD& D) {
  Xform X;
  for (int i = 0; i < 9; ++i) {
    X.ah[i] = (float)D.A[i];
    X.al[i] = (float)(D.A[i] - (double)X.ah[i]);
  }
  for (int a = 0; a < 3; ++a) {
    X.bh[a] = (float)D.b[a];
    X.bl[a] = (float)(D.b[a] - (double)X.bh[a]);
  }
  return X;
}

// s + e = a + b exactly (Knuth's two-sum); explicit round-to-nearest
// intrinsics keep the compiler from contracting or reordering the steps.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Moving-pixel coordinate p = A (x, y, z) + b of virtual voxel (x, y, z)
// along axis a, split into integer part ib and fraction fb in [0, 1).
// Evaluated in float-float without double arithmetic (the FP64 pipe is
// narrow on this part): the products of the hi coefficients are exact
// (value + fma residual), the partial sums error-free (two-sum), so p keeps
// about 48 significant bits -- far below the float fraction's rounding.
// Integer parts are clamped to +-2^30 voxels, outside any volume.
__device__ __forceinline__ void xform_coord(const Xform& X, int a, int x, int y, int z,
                                            int& ib, float& fb) {
  const float fx = (float)x, fy = (float)y, fz = (float)z;  // exact: |x| < 2^24
  const float h0 = X.ah[3 * a], h1 = X.ah[3 * a + 1], h2 = X.ah[3 * a + 2];
  const float p0 = __fmul_rn(h0, fx), p1 = __fmul_rn(h1, fy), p2 = __fmul_rn(h2, fz);
  float err = __fmaf_rn(h0, fx, -p0);
  err = __fadd_rn(err, __fmaf_rn(h1, fy, -p1));
  err = __fadd_rn(err, __fmaf_rn(h2, fz, -p2));
  err = __fmaf_rn(X.al[3 * a], fx, err);
  err = __fmaf_rn(X.al[3 * a + 1], fy, err);
  err = __fmaf_rn(X.al[3 * a + 2], fz, err);
  err = __fadd_rn(err, X.bl[a]);
  float s = X.bh[a], e;
  two_sum(s, p0, s, e);
  err = __fadd_rn(err, e);
  two_sum(s, p1, s, e);
  err = __fadd_rn(err, e);
  two_sum(s, p2, s, e);
  err = __fadd_rn(err, e);
  float hi, lo;
  two_sum(s, err, hi, lo);
  float fl = floorf(hi);
  float fr = __fadd_rn(__fsub_rn(hi, fl), lo);  // hi - fl is exact
  if (fr < 0.0f) {
    fr = __fadd_rn(fr, 1.0f);
    fl = __fsub_rn(fl, 1.0f);
  }
  if (fr >= 1.0f) {  // p within half an ulp below an integer
    fr = __fsub_rn(fr, 1.0f);
    fl = __fadd_rn(fl, 1.0f);
  }
  fl = fminf(fmaxf(fl, -1073741824.0f), 1073741824.0f);  // NaN -> -2^30
  ib = (int)fl;
  fb = fr;
}

// ---------------------------------------------------------------------------
// Resampling
// ---------------------------------------------------------------------------

// Sampler of one axis: integer floor, fraction and the ceil index used by the
// reference (ceil == floor when the fraction is 0).
struct Axis {
  int f, c;
  float r;
  bool ok;
};

__device__ __forceinline__ Axis make_axis(int base, float q, int dim) {
  float fl = floorf(q);
  Axis a;
  a.f = base + (int)fl;
  a.r = q - fl;
  a.c = a.f + (a.r > 0.0f ? 1 : 0);
  // p >= 0 and p <= dim-1 for p = f + r, 0 <= r < 1
  a.ok = (a.f >= 0) && (a.f < dim - 1 || (a.f == dim - 1 && a.r == 0.0f));
  return a;
}

// Tile base of a 32 x 8 tile (x0, y0) of slice z: the moving-pixel
// coordinate split into integer part and fraction (xform_coord), plus the float
// step matrix. Each voxel adds a float offset of at most (31, 7) voxels to the
// base fraction, so the interpolation weights keep ~1e-6 voxel accuracy
// anywhere in the grid.
struct TileBase {
  int ib[3];
  float fb[3];
  float A[9];
};

__device__ __forceinline__ void tile_base(const Xform* X, int x0, int y0, int z, TileBase& T) {
#pragma unroll
  for (int a = 0; a < 3; ++a) xform_coord(*X, a, x0, y0, z, T.ib[a], T.fb[a]);
#pragma unroll
  for (int i = 0; i < 9; ++i) T.A[i] = X->ah[i];
}

// Trilinear (ND = 3) / bilinear (ND = 2) sample at offset (tx, ty) from the
// tile base; 0 outside [0, dim-1] (src/Interpolator/interpolator.cu:69-232).
template <int ND, typename TM>
__device__ __forceinline__ float tile_sample(const TM* __restrict__ mov, int mx, int my, int mz,
                                             const TileBase& T, int tx, int ty) {
  const float dx = (float)tx, dy = (float)ty;
  if (ND == 3) {
    float qx = fmaf(T.A[1], dy, fmaf(T.A[0], dx, T.fb[0]));
    float qy = fmaf(T.A[4], dy, fmaf(T.A[3], dx, T.fb[1]));
    float qz = fmaf(T.A[7], dy, fmaf(T.A[6], dx, T.fb[2]));
    Axis ax = make_axis(T.ib[0], qx, mx);
    Axis ay = make_axis(T.ib[1], qy, my);
    Axis az = make_axis(T.ib[2], qz, mz);
    if (!(ax.ok && ay.ok && az.ok)) return 0.0f;
    const size_t sy = (size_t)mx, sz = (size_t)mx * my;
    const size_t zf = az.f * sz, zc = az.c * sz, yf = ay.f * sy, yc = ay.c * sy;
    // z, then y, then x (interpolator.cu:96-128)
    float lu0 = ldf(mov, ax.f + yf + zf), lu1 = ldf(mov, ax.f + yf + zc);
    float ru0 = ldf(mov, ax.c + yf + zf), ru1 = ldf(mov, ax.c + yf + zc);
    float rb0 = ldf(mov, ax.c + yc + zf), rb1 = ldf(mov, ax.c + yc + zc);
    float lb0 = ldf(mov, ax.f + yc + zf), lb1 = ldf(mov, ax.f + yc + zc);
    float lu = fmaf(az.r, lu1 - lu0, lu0), ru = fmaf(az.r, ru1 - ru0, ru0);
    float rb = fmaf(az.r, rb1 - rb0, rb0), lb = fmaf(az.r, lb1 - lb0, lb0);
    float l = fmaf(ay.r, lb - lu, lu), r = fmaf(ay.r, rb - ru, ru);
    return fmaf(ax.r, r - l, l);
  }
  float qx = fmaf(T.A[1], dy, fmaf(T.A[0], dx, T.fb[0]));
  float qy = fmaf(T.A[4], dy, fmaf(T.A[3], dx, T.fb[1]));
  Axis ax = make_axis(T.ib[0], qx, mx);
  Axis ay = make_axis(T.ib[1], qy, my);
  if (!(ax.ok && ay.ok)) return 0.0f;
  const size_t yf = (size_t)ay.f * mx, yc = (size_t)ay.c * mx;
  // y, then x (interpolator.cu:199-207)
  float f0 = ldf(mov, ax.f + yf), f1 = ldf(mov, ax.f + yc);
  float c0 = ldf(mov, ax.c + yf), c1 = ldf(mov, ax.c + yc);
  float xl = fmaf(ay.r, f1 - f0, f0), xr = fmaf(ay.r, c1 - c0, c0);
  return fmaf(ax.r, xr - xl, xl);
}

// Whether every sample of a 32 x 8 tile slice from base T lies strictly
// inside the moving volume (0 <= floor, floor + 1 <= dim - 1 on each axis):
// the tile's corners bound the affine image, 0.01 voxel covers float rounding.
__device__ __forceinline__ bool tile_inside(const TileBase& T, int mx, int my, int mz) {
  const int dims[3] = {mx, my, mz};
  bool in = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float ex = T.A[3 * a] * 31.0f, ey = T.A[3 * a + 1] * 7.0f;
    const float lo = T.fb[a] + fminf(ex, 0.0f) + fminf(ey, 0.0f);
    const float hi = T.fb[a] + fmaxf(ex, 0.0f) + fmaxf(ey, 0.0f);
    in = in && ((float)T.ib[a] + lo >= 0.01f) && ((float)T.ib[a] + hi <= (float)(dims[a] - 1) - 0.01f);
  }
  return in;
}

// tile_sample<3> for a tile slice that tile_inside accepted: no bounds tests,
// the ceil corner always floor + 1 -- where the fraction is 0 its weight is
// 0 -- so the value equals tile_sample's bit for bit.
template <typename TM>
__device__ __forceinline__ float tile_sample_inside(const TM* __restrict__ mov, int mx, int my,
                                                    const TileBase& T, int tx, int ty) {
  const float dx = (float)tx, dy = (float)ty;
  const float qx = fmaf(T.A[1], dy, fmaf(T.A[0], dx, T.fb[0]));
  const float qy = fmaf(T.A[4], dy, fmaf(T.A[3], dx, T.fb[1]));
  const float qz = fmaf(T.A[7], dy, fmaf(T.A[6], dx, T.fb[2]));
  const float flx = floorf(qx), fly = floorf(qy), flz = floorf(qz);
  const float rx = qx - flx, ry = qy - fly, rz = qz - flz;
  const unsigned umx = (unsigned)mx, mxy = (unsigned)mx * (unsigned)my;
  const unsigned b = (unsigned)(T.ib[0] + (int)flx) + (unsigned)(T.ib[1] + (int)fly) * umx +
                     (unsigned)(T.ib[2] + (int)flz) * mxy;
  float lu0 = ldf(mov, b), lu1 = ldf(mov, b + mxy);
  float ru0 = ldf(mov, b + 1), ru1 = ldf(mov, b + 1 + mxy);
  float rb0 = ldf(mov, b + 1 + umx), rb1 = ldf(mov, b + 1 + umx + mxy);
  float lb0 = ldf(mov, b + umx), lb1 = ldf(mov, b + umx + mxy);
  float lu = fmaf(rz, lu1 - lu0, lu0), ru = fmaf(rz, ru1 - ru0, ru0);
  float rb = fmaf(rz, rb1 - rb0, rb0), lb = fmaf(rz, lb1 - lb0, lb0);
  float l = fmaf(ry, lb - lu, lu), r = fmaf(ry, rb - ru, ru);
  return fmaf(rx, r - l, l);
}

// One CTA = 32x8 virtual voxels of one z-slice of one transform slot.
template <int ND, typename TM>
__global__ void __launch_bounds__(256) k_warp(const TM* __restrict__ mov, int mx, int my, int mz,
                                               int vx, int vy, int vz,
                                               const Xform* __restrict__ xf, int k0,
                                               float* __restrict__ out, size_t slot_stride) {
  __shared__ TileBase T;
  const int slot = blockIdx.z / vz;
  const int z = blockIdx.z - slot * vz;
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
  if (threadIdx.x == 0 && threadIdx.y == 0) tile_base(xf + k0 + slot, x0, y0, z, T);
  __syncthreads();
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = x0 + tx, y = y0 + ty;
  if (x >= vx || y >= vy) return;
  const float v = tile_sample<ND, TM>(mov, mx, my, mz, T, tx, ty);
  out[slot * slot_stride + ((size_t)z * vy + y) * vx + x] = v;
}

// ---------------------------------------------------------------------------
// Sobel gradient magnitude (zero padding); ND = 2 works per x-y plane.
// CTA = 32x8 outputs of one slice; halo tile (34 x 10 x 3) in shared memory.
// ---------------------------------------------------------------------------
template <int ND>
__global__ void __launch_bounds__(256) k_sobel(const float* __restrict__ in, int vx, int vy,
                                                int vz, float* __restrict__ out,
                                                size_t slot_stride) {
  constexpr int HX = 34, HY = 10, HZ = (ND == 3) ? 3 : 1;
  __shared__ float t[HZ][HY][HX];
  const int slot = blockIdx.z / vz;
  const int z = blockIdx.z - slot * vz;
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
  const float* src = in + slot * slot_stride;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  for (int i = tid; i < HZ * HY * HX; i += 256) {
    int hx = i % HX, hy = (i / HX) % HY, hz = i / (HX * HY);
    int gx = x0 + hx - 1, gy = y0 + hy - 1, gz = (ND == 3) ? z + hz - 1 : z;
    float v = 0.0f;
    if (gx >= 0 && gx < vx && gy >= 0 && gy < vy && gz >= 0 && gz < vz)
      v = src[((size_t)gz * vy + gy) * vx + gx];
    t[hz][hy][hx] = v;
  }
  __syncthreads();
  const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
  if (x >= vx || y >= vy) return;
  const int cx = threadIdx.x + 1, cy = threadIdx.y + 1;
  float g;
  if (ND == 3) {
    // separable: smooth h = [1 2 1], derivative hp = [-1 0 1]
    float sz[3][3], dz[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        float a = t[0][cy + j - 1][cx + i - 1], b = t[1][cy + j - 1][cx + i - 1],
              c = t[2][cy + j - 1][cx + i - 1];
        sz[j][i] = a + 2.0f * b + c;
        dz[j][i] = c - a;
      }
    float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float hj = (j == 1) ? 2.0f : 1.0f, hpj = (float)(j - 1);
      gx += hj * (sz[j][2] - sz[j][0]);
      gy += hpj * (sz[j][0] + 2.0f * sz[j][1] + sz[j][2]);
      gz += hj * (dz[j][0] + 2.0f * dz[j][1] + dz[j][2]);
    }
    g = sqrtf(gx * gx + gy * gy + gz * gz);
  } else {
    float gx = 0.f, gy = 0.f;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float hj = (j == 1) ? 2.0f : 1.0f, hpj = (float)(j - 1);
      float a = t[0][cy + j - 1][cx - 1], b = t[0][cy + j - 1][cx], c = t[0][cy + j - 1][cx + 1];
      gx += hj * (c - a);
      gy += hpj * (a + 2.0f * b + c);
    }
    g = sqrtf(gx * gx + gy * gy);
  }
  out[slot * slot_stride + ((size_t)z * vy + y) * vx + x] = g;
}

// ---------------------------------------------------------------------------
// Patch moments, sigma, least-squares measure and the LC2 sums.
// ---------------------------------------------------------------------------
struct MomentParams {
  int vx, vy, vz;       // virtual grid
  int r;                // patch radius
  int n;                // patch voxels (2r+1)^ND
  int zchunk;           // output slices per CTA (3D)
  int nzchunks;         // CTAs along z per slot
  float qu, qm, qg;     // fixed-point scales
  long long thr_var;    // D_uu > thr_var  <=>  sample variance of U > 1e-6
  long long thr_m;      // D_mm <= thr_m   <=>  sample variance of M <= 1e-12
  long long thr_g;      // D_gg <= thr_g   <=>  sample variance of G <= 1e-12
  float sig_scale;      // sigma = sqrt(D_uu) * sig_scale
  float sum_scale;      // fixed-point scale of the measure / sigma sums
  size_t u_stride, m_stride, g_stride;  // per-slot strides (0 for static images)
};

// int64 -> float through two 32-bit conversions (about 2 ulp; the single
// 64-bit conversion is a slow multi-cycle instruction).
__device__ __forceinline__ float ll2f(long long v) {
  const int hi = (int)(v >> 32);
  const unsigned lo = (unsigned)(v & 0xffffffffll);
  return fmaf((float)hi, 4294967296.0f, (float)lo);
}

// Round v*Q to the nearest integer (|v*Q| < 2^22): add 1.5*2^23 and read the
// integer out of the mantissa.
__device__ __forceinline__ int quant(float v, float Q) {
  float f = fmaf(v, Q, 12582912.0f);
  return __float_as_int(f) - 0x4B400000;
}

struct PointFields {
  int q[kNF32];
  long long w[kNF64];
};

template <typename TU>
__device__ __forceinline__ void point_fields(const TU* __restrict__ U, const float* __restrict__ M,
                                             const float* __restrict__ G, const MomentParams& P,
                                             int gx, int gy, int gz, PointFields& f) {
  float u = 0.f, m = 0.f, g = 0.f;
  if (gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy && gz >= 0 && gz < P.vz) {
    size_t i = ((size_t)gz * P.vy + gy) * P.vx + gx;
    u = ldf(U, i);
    m = __ldg(M + i);
    g = __ldg(G + i);
  }
  int qu = quant(u, P.qu), qm = quant(m, P.qm), qg = quant(g, P.qg);
  f.q[0] = qu;
  f.q[1] = qm;
  f.q[2] = qg;
  // zero padding and values <= 1e-6 invalidate the patch (cu_lc2_3d.cu:223-243)
  f.q[3] = (u > 1e-6f) ? 0 : 1;
  f.w[0] = (long long)qu * qu;
  f.w[1] = (long long)qm * qm;
  f.w[2] = (long long)qg * qg;
  f.w[3] = (long long)qu * qm;
  f.w[4] = (long long)qu * qg;
  f.w[5] = (long long)qm * qg;
}

// Shared-memory planes of one moments CTA. Pitches are odd (in elements) so
// threads walking different rows hit different banks.
struct MomSmem {
  int hx, hy, hxp, txp;
  int* z32;        // [kNF32][hy][hxp]   z-window sums of every halo point
  long long* z64;  // [kNF64][hy][hxp]
  int* x32;        // [kNF32][hy][txp]   + x-window
  long long* x64;  // [kNF64][hy][txp]
  int* y32;        // [kNF32][kTY][txp]  + y-window = full patch sums
  long long* y64;  // [kNF64][kTY][txp]
};

__host__ __device__ inline size_t mom_smem_bytes(int r) {
  int hx = kTX + 2 * r, hy = kTY + 2 * r;
  int hxp = hx | 1, txp = kTX + 1;
  size_t pz = (size_t)hy * hxp, px = (size_t)hy * txp, py = (size_t)kTY * txp;
  size_t b32 = kNF32 * (pz + px + py) * sizeof(int);
  b32 = (b32 + 15) & ~(size_t)15;
  return b32 + kNF64 * (pz + px + py) * sizeof(long long);
}

__device__ __forceinline__ MomSmem mom_smem_carve(unsigned char* base, int r) {
  MomSmem s;
  s.hx = kTX + 2 * r;
  s.hy = kTY + 2 * r;
  s.hxp = s.hx | 1;
  s.txp = kTX + 1;
  size_t pz = (size_t)s.hy * s.hxp, px = (size_t)s.hy * s.txp, py = (size_t)kTY * s.txp;
  int* p32 = reinterpret_cast<int*>(base);
  s.z32 = p32;
  s.x32 = p32 + kNF32 * pz;
  s.y32 = s.x32 + kNF32 * px;
  size_t b32 = kNF32 * (pz + px + py) * sizeof(int);
  b32 = (b32 + 15) & ~(size_t)15;
  long long* p64 = reinterpret_cast<long long*>(base + b32);
  s.z64 = p64;
  s.x64 = p64 + kNF64 * pz;
  s.y64 = s.x64 + kNF64 * px;
  return s;
}

// x-window and y-window running sums over the z-window planes. Integer sums
// are exact, so a running update equals the direct sum.
__device__ __forceinline__ void mom_xy_passes(const MomSmem& s, int r) {
  const int tid = threadIdx.x;
  const int w = 2 * r + 1;
  const size_t pz = (size_t)s.hy * s.hxp, px = (size_t)s.hy * s.txp, py = (size_t)kTY * s.txp;
  // x pass: items (field, segment, row) with row fastest
  {
    const int nseg = kTX / kSegX;
    const int items = (kNF32 + kNF64) * nseg * s.hy;
    for (int it = tid; it < items; it += kNT) {
      int row = it % s.hy;
      int rest = it / s.hy;
      int seg = rest % nseg;
      int f = rest / nseg;
      int x = seg * kSegX;
      if (f < kNF32) {
        const int* src = s.z32 + f * pz + (size_t)row * s.hxp;
        int* dst = s.x32 + f * px + (size_t)row * s.txp;
        int acc = 0;
        for (int i = 0; i < w; ++i) acc += src[x + i];
        dst[x] = acc;
#pragma unroll
        for (int j = 1; j < kSegX; ++j) {
          acc += src[x + j + w - 1] - src[x + j - 1];
          dst[x + j] = acc;
        }
      } else {
        const long long* src = s.z64 + (f - kNF32) * pz + (size_t)row * s.hxp;
        long long* dst = s.x64 + (f - kNF32) * px + (size_t)row * s.txp;
        long long acc = 0;
        for (int i = 0; i < w; ++i) acc += src[x + i];
        dst[x] = acc;
#pragma unroll
        for (int j = 1; j < kSegX; ++j) {
          acc += src[x + j + w - 1] - src[x + j - 1];
          dst[x + j] = acc;
        }
      }
    }
  }
  __syncthreads();
  // y pass: items (field, segment, column) with column fastest
  {
    const int nseg = kTY / kSegY;
    const int items = (kNF32 + kNF64) * nseg * kTX;
    for (int it = tid; it < items; it += kNT) {
      int col = it % kTX;
      int rest = it / kTX;
      int seg = rest % nseg;
      int f = rest / nseg;
      int y = seg * kSegY;
      if (f < kNF32) {
        const int* src = s.x32 + f * px + col;
        int* dst = s.y32 + f * py + col;
        int acc = 0;
        for (int i = 0; i < w; ++i) acc += src[(size_t)(y + i) * s.txp];
        dst[(size_t)y * s.txp] = acc;
#pragma unroll
        for (int j = 1; j < kSegY; ++j) {
          acc += src[(size_t)(y + j + w - 1) * s.txp] - src[(size_t)(y + j - 1) * s.txp];
          dst[(size_t)(y + j) * s.txp] = acc;
        }
      } else {
        const long long* src = s.x64 + (f - kNF32) * px + col;
        long long* dst = s.y64 + (f - kNF32) * py + col;
        long long acc = 0;
        for (int i = 0; i < w; ++i) acc += src[(size_t)(y + i) * s.txp];
        dst[(size_t)y * s.txp] = acc;
#pragma unroll
        for (int j = 1; j < kSegY; ++j) {
          acc += src[(size_t)(y + j + w - 1) * s.txp] - src[(size_t)(y + j - 1) * s.txp];
          dst[(size_t)(y + j) * s.txp] = acc;
        }
      }
    }
  }
  __syncthreads();
}

// Sigma and clipped measure from centred sums D_xy = n S_xy - S_x S_y of a
// valid patch (every value > 1e-6). Shared by the generic moments kernel and
// the fused kernel of a resampled ultrasound, so both give the same bits.
__device__ __forceinline__ void solve_centred(long long d_uu, long long d_mm, long long d_gg,
                                              long long d_mg, long long d_um, long long d_ug,
                                              long long thr_var, long long thr_m,
                                              long long thr_g, float sig_scale, float& sigma,
                                              float& measure) {
  sigma = 0.0f;
  measure = 0.0f;
  if (d_uu <= thr_var) return;
  const float fuu = ll2f(d_uu);
  sigma = sqrtf(fuu) * sig_scale;
  const bool km = d_mm > thr_m, kg = d_gg > thr_g;
  const float iu = rsqrtf(fuu);
  float r2 = 0.0f;
  if (km && kg) {
    const float im = rsqrtf(ll2f(d_mm)), ig = rsqrtf(ll2f(d_gg));
    const float rum = ll2f(d_um) * iu * im, rug = ll2f(d_ug) * iu * ig,
                rmg = ll2f(d_mg) * im * ig;
    const float den = 1.0f - rmg * rmg;
    if (den > 1e-3f) {
      r2 = __fdividef(rum * rum + rug * rug - 2.0f * rum * rug * rmg, den);
    } else {
      // nearly collinear columns: solve in double from the exact sums
      double duu = (double)d_uu, dmm = (double)d_mm, dgg = (double)d_gg;
      double dmg = (double)d_mg, dum = (double)d_um, dug = (double)d_ug;
      double det = dmm * dgg - dmg * dmg;
      double e;
      if (det <= 1e-10 * dmm * dgg)
        e = dum * dum / dmm;
      else
        e = (dgg * dum * dum - 2.0 * dmg * dum * dug + dmm * dug * dug) / det;
      r2 = (float)(e / duu);
    }
  } else if (km) {
    const float c = ll2f(d_um) * iu * rsqrtf(ll2f(d_mm));
    r2 = c * c;
  } else if (kg) {
    const float c = ll2f(d_ug) * iu * rsqrtf(ll2f(d_gg));
    r2 = c * c;
  }
  float m = sigma * r2;
  if (!(m > 0.0f) || isinf(m)) m = 0.0f;
  measure = m;
}

// solve_centred for a static M and G (HighResolutionModality: Fixed): the
// factors of the static columns come precomputed per voxel in sv --
// im = rsqrtf(D_mm) when D_mm > thr_m else 0, ig likewise for D_gg, rmg =
// D_mg im ig (k_fixed_solve_static) -- from the same float operations, so the
// values are the same bit for bit. The nearly collinear case reads the exact
// centred sums d[3][nv] of voxel gi.
__device__ __forceinline__ void solve_centred_static(long long d_uu, long long d_um,
                                                     long long d_ug, float4 sv,
                                                     const long long* __restrict__ d, size_t nv,
                                                     size_t gi, long long thr_var,
                                                     float sig_scale, float& sigma,
                                                     float& measure) {
  sigma = 0.0f;
  measure = 0.0f;
  if (d_uu <= thr_var) return;
  const float fuu = ll2f(d_uu);
  sigma = sqrtf(fuu) * sig_scale;
  const float im = sv.x, ig = sv.y;
  const bool km = im > 0.0f, kg = ig > 0.0f;
  const float iu = rsqrtf(fuu);
  float r2 = 0.0f;
  if (km && kg) {
    const float rum = ll2f(d_um) * iu * im, rug = ll2f(d_ug) * iu * ig, rmg = sv.z;
    const float den = 1.0f - rmg * rmg;
    if (den > 1e-3f) {
      r2 = __fdividef(rum * rum + rug * rug - 2.0f * rum * rug * rmg, den);
    } else {
      // nearly collinear columns: solve in double from the exact sums
      double duu = (double)d_uu, dmm = (double)__ldg(d + gi), dgg = (double)__ldg(d + nv + gi);
      double dmg = (double)__ldg(d + 2 * nv + gi), dum = (double)d_um, dug = (double)d_ug;
      double det = dmm * dgg - dmg * dmg;
      double e;
      if (det <= 1e-10 * dmm * dgg)
        e = dum * dum / dmm;
      else
        e = (dgg * dum * dum - 2.0 * dmg * dum * dug + dmm * dug * dug) / det;
      r2 = (float)(e / duu);
    }
  } else if (km) {
    const float c = ll2f(d_um) * iu * im;
    r2 = c * c;
  } else if (kg) {
    const float c = ll2f(d_ug) * iu * ig;
    r2 = c * c;
  }
  float m = sigma * r2;
  if (!(m > 0.0f) || isinf(m)) m = 0.0f;
  measure = m;
}

// Per-voxel sigma and clipped measure from exact patch sums.
// Reference semantics: sigma = sqrt(sample variance of U) when every patch
// value is > 1e-6 and the variance is > 1e-6, else 0; measure =
// sigma - var_res / sigma kept only if finite and > 0 (cu_lc2_3d.cu:601-609),
// where var_res is the residual sample variance of the LS fit. With centred
// sums D_xy = n S_xy - S_x S_y, var_res = (D_uu - E)/(n (n-1) Qu^2) and
// measure = sigma * E / D_uu, E = explained part in D units.
__device__ __forceinline__ void solve_voxel(const MomentParams& P, int s_u, int s_m, int s_g,
                                            int cnt, long long s_uu, long long s_mm,
                                            long long s_gg, long long s_um, long long s_ug,
                                            long long s_mg, float& sigma, float& measure) {
  sigma = 0.0f;
  measure = 0.0f;
  if (cnt != 0) return;
  const long long n = P.n;
  solve_centred(n * s_uu - (long long)s_u * s_u, n * s_mm - (long long)s_m * s_m,
                n * s_gg - (long long)s_g * s_g, n * s_mg - (long long)s_m * s_g,
                n * s_um - (long long)s_u * s_m, n * s_ug - (long long)s_u * s_g, P.thr_var,
                P.thr_m, P.thr_g, P.sig_scale, sigma, measure);
}

// Accumulate one voxel into the thread's exact sums.
__device__ __forceinline__ void add_sums(const MomentParams& P, float sigma, float measure,
                                         long long& acc_m, long long& acc_s) {
  acc_m += __float2int_rn(measure * P.sum_scale);
  acc_s += __float2int_rn(sigma * P.sum_scale);
}

__device__ __forceinline__ void flush_sums(long long acc_m, long long acc_s,
                                           unsigned long long* acc) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    acc_m += __shfl_down_sync(0xffffffffu, acc_m, o);
    acc_s += __shfl_down_sync(0xffffffffu, acc_s, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(acc + 0, (unsigned long long)acc_m);
    atomicAdd(acc + 1, (unsigned long long)acc_s);
  }
}

// ND = 3: one CTA = 32x8 output columns x `zchunk` slices of one slot. Each
// thread keeps z-window sums of up to kMaxP3 halo points in registers and
// updates them per output slice with the entering and leaving slices.
// ND = 2: one CTA = 32x8 outputs.
// Optional per-voxel outputs (diagnostics) when out_sigma/out_measure != 0.
template <int ND, typename TU>
__global__ void __launch_bounds__(kNT) k_moments(const TU* __restrict__ Ubase,
                                                  const float* __restrict__ Mbase,
                                                  const float* __restrict__ Gbase,
                                                  MomentParams P,
                                                  unsigned long long* __restrict__ acc, int k0,
                                                  float* __restrict__ out_sigma,
                                                  float* __restrict__ out_measure) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int r = P.r;
  MomSmem s = mom_smem_carve(smem_raw, r);
  const int tid = threadIdx.x;
  const int slot = blockIdx.z / P.nzchunks;
  const int zc = blockIdx.z - slot * P.nzchunks;
  const TU* U = Ubase + slot * P.u_stride;
  const float* M = Mbase + slot * P.m_stride;
  const float* G = Gbase + slot * P.g_stride;
  const int x0 = blockIdx.x * kTX, y0 = blockIdx.y * kTY;
  const int np = s.hx * s.hy;
  const size_t pz = (size_t)s.hy * s.hxp, py = (size_t)kTY * s.txp;
  const int otx = tid % kTX, oty = tid / kTX;
  long long acc_m = 0, acc_s = 0;

  if (ND == 2) {
    for (int p = tid; p < np; p += kNT) {
      int hx = p % s.hx, hy = p / s.hx;
      PointFields f;
      point_fields(U, M, G, P, x0 - r + hx, y0 - r + hy, 0, f);
      size_t o = (size_t)hy * s.hxp + hx;
#pragma unroll
      for (int k = 0; k < kNF32; ++k) s.z32[k * pz + o] = f.q[k];
#pragma unroll
      for (int k = 0; k < kNF64; ++k) s.z64[k * pz + o] = f.w[k];
    }
    __syncthreads();
    mom_xy_passes(s, r);
    const int x = x0 + otx, y = y0 + oty;
    if (x < P.vx && y < P.vy) {
      size_t o = (size_t)oty * s.txp + otx;
      float sg, ms;
      solve_voxel(P, s.y32[o], s.y32[py + o], s.y32[2 * py + o], s.y32[3 * py + o], s.y64[o],
                  s.y64[py + o], s.y64[2 * py + o], s.y64[3 * py + o], s.y64[4 * py + o],
                  s.y64[5 * py + o], sg, ms);
      add_sums(P, sg, ms, acc_m, acc_s);
      const size_t gi = (size_t)y * P.vx + x;
      if (out_sigma) out_sigma[gi] = sg;
      if (out_measure) out_measure[gi] = ms;
    }
    flush_sums(acc_m, acc_s, acc + 2 * (size_t)(k0 + slot));
    return;
  }

  // ---- 3D: z-marching ----
  const int zb = zc * P.zchunk;
  const int ze = min(zb + P.zchunk, P.vz);
  int a32[kMaxP3][kNF32];
  long long a64[kMaxP3][kNF64];
#pragma unroll
  for (int j = 0; j < kMaxP3; ++j) {
#pragma unroll
    for (int k = 0; k < kNF32; ++k) a32[j][k] = 0;
#pragma unroll
    for (int k = 0; k < kNF64; ++k) a64[j][k] = 0;
  }
  // prime the window with slices zb-r .. zb+r-1
  for (int zz = zb - r; zz < zb + r; ++zz) {
#pragma unroll
    for (int j = 0; j < kMaxP3; ++j) {
      int p = tid + j * kNT;
      if (p < np) {
        PointFields f;
        point_fields(U, M, G, P, x0 - r + p % s.hx, y0 - r + p / s.hx, zz, f);
#pragma unroll
        for (int k = 0; k < kNF32; ++k) a32[j][k] += f.q[k];
#pragma unroll
        for (int k = 0; k < kNF64; ++k) a64[j][k] += f.w[k];
      }
    }
  }
  for (int z = zb; z < ze; ++z) {
#pragma unroll
    for (int j = 0; j < kMaxP3; ++j) {
      int p = tid + j * kNT;
      if (p < np) {
        int hx = p % s.hx, hy = p / s.hx;
        PointFields fi, fo;
        point_fields(U, M, G, P, x0 - r + hx, y0 - r + hy, z + r, fi);
        if (z > zb) {
          point_fields(U, M, G, P, x0 - r + hx, y0 - r + hy, z - r - 1, fo);
        } else {
#pragma unroll
          for (int k = 0; k < kNF32; ++k) fo.q[k] = 0;
#pragma unroll
          for (int k = 0; k < kNF64; ++k) fo.w[k] = 0;
        }
        size_t o = (size_t)hy * s.hxp + hx;
#pragma unroll
        for (int k = 0; k < kNF32; ++k) {
          a32[j][k] += fi.q[k] - fo.q[k];
          s.z32[k * pz + o] = a32[j][k];
        }
#pragma unroll
        for (int k = 0; k < kNF64; ++k) {
          a64[j][k] += fi.w[k] - fo.w[k];
          s.z64[k * pz + o] = a64[j][k];
        }
      }
    }
    __syncthreads();
    mom_xy_passes(s, r);
    const int x = x0 + otx, y = y0 + oty;
    if (x < P.vx && y < P.vy) {
      size_t o = (size_t)oty * s.txp + otx;
      float sg, ms;
      solve_voxel(P, s.y32[o], s.y32[py + o], s.y32[2 * py + o], s.y32[3 * py + o], s.y64[o],
                  s.y64[py + o], s.y64[2 * py + o], s.y64[3 * py + o], s.y64[4 * py + o],
                  s.y64[5 * py + o], sg, ms);
      add_sums(P, sg, ms, acc_m, acc_s);
      const size_t gi = ((size_t)z * P.vy + y) * P.vx + x;
      if (out_sigma) out_sigma[gi] = sg;
      if (out_measure) out_measure[gi] = ms;
    }
    // the next z-phase overwrites the z planes only; x/y planes are rewritten
    // after the next barrier, so no extra barrier is needed here
  }
  flush_sums(acc_m, acc_s, acc + 2 * (size_t)(k0 + slot));
}

// float -> storage type conversion of a device buffer
template <typename T>
__global__ void k_convert(const float* __restrict__ in, T* __restrict__ out, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t step = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += step) out[i] = stf<T>(in[i]);
}

// Quantised static image qU = quant(U, qu), one int per voxel.
template <typename TU>
__global__ void k_quant_static(const TU* __restrict__ U, size_t n, float qu, int* __restrict__ out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = quant(ldf(U, i), qu);
}

}  // namespace lc2
