// lc2_fused.cuh -- fused LC2 evaluation kernel for a static ultrasound
// (HighResolutionModality: Moving: the moving MR/CT is resampled).
//
// One CTA owns a 32 x TY tile of output columns of one transform and marches
// along z through `zchunk` output slices. For each input slice e it
//   1. resamples the moving volume at slice e+1 on the tile's halo region
//      (src/Interpolator/interpolator.cu:69-179); every thread keeps its own
//      points' last two slices in registers and writes, for slice e, the
//      centre value M and the z-smoothed / z-differentiated planes
//      Sz = M(e-1) + 2 M(e) + M(e+1), Dz = M(e+1) - M(e-1), so the 3x3x3 Sobel
//      (src/cu_LC2/cu_lc2_3d.cu:100-179, 977-1005) needs 17 in-plane reads;
//   2. updates, in registers, the exact z-window sums of the patch moments of
//      its halo points: the entering slice's fields are added, the leaving
//      slice's fields (replayed from a quantised shared ring) subtracted;
//   3. runs the x and y window passes in shared memory;
//   4. solves each output voxel's least-squares fit against the precomputed
//      weighting factor sigma (cu_lc2_3d.cu:526-618) and adds its clipped
//      measure to the transform's exact fixed-point sum.
// Fields are 12 int32 limbs: qM, qG, and the 64-bit products UM, UG, MM, GG,
// MG split as hi * 2^K + lo (0 <= lo < 2^K); every limb's window sum fits
// int32, so each running update is one 32-bit add and all sums stay exact.
// The ultrasound is static, so its window sum S_U is precomputed once per
// context (su) like the weighting factor.
// Nothing per voxel is written to global memory, so the moving volume stays
// resident in L2 while many transforms are evaluated.
// ND = 2 covers the 2D and 2D-to-3D modes (one slice, no z window); WND is the
// dimensionality of the resampling (3 for 2D-to-3D).
#pragma once

#include "lc2_kernels.cuh"

namespace lc2 {

struct FusedParams {
  int vx, vy, vz;          // virtual grid
  int mx, my, mz;          // moving volume
  int r, n;                // patch radius, patch voxels
  int zchunk;              // output slices per CTA (3D)
  int ntx;                 // tiles along x
  int kbits;               // limb split K of the 64-bit products
  float qu, qm, qg;        // fixed-point scales
  long long thr_m, thr_g;  // degenerate-column thresholds (see MomentParams)
  long long thr_var;       // valid-patch variance threshold (resampled ultrasound)
  float sig_scale;         // sigma = sqrt(D_uu) * sig_scale
  float sum_scale;         // fixed-point scale of the measure sum
  int y0;                  // first output row of the launch's tiles (presampled 3D kernels)
};

constexpr int kLimbs = 12;

// Patch voxels (2R+1)^ND and the limb split K of a patch of that size: the
// largest K with (n + 1) 2^K <= 2^30, so every low limb's window sum stays
// below 2^30 -- the rule by which the host sets FusedParams::kbits. The
// kernels take both from their template radius, so multiplications by n and
// the limb shifts and masks are immediates; the launchers check that the
// host's kbits agrees.
constexpr long long patch_voxels(int nd, int r) {
  return (long long)(2 * r + 1) * (2 * r + 1) * (nd == 3 ? (2 * r + 1) : 1);
}
constexpr int limb_bits(long long n) {
  int k = 0;
  while (((n + 1) << (k + 1)) <= (1LL << 30)) ++k;
  return k;
}
template <int ND, int R>
struct PatchConst {
  static constexpr long long N = patch_voxels(ND, R);
  static constexpr int K = limb_bits(N);
};

// Rows of the band that fixes a 3D tile's sampling base: every tile height
// (8, 16, 24) divides it, so a tile never straddles two bands and each voxel
// is sampled from the same base whichever tile height computes it.
constexpr int kBand = 48;

// Compile-time geometry of one fused CTA: a 32 x TY output tile, patch radius R.
template <int ND, int TY, int R>
struct FusedGeom {
  static constexpr int NT = 32 * TY;
  static constexpr int PW = 32 + 2 * R + 2, PH = TY + 2 * R + 2;  // resampled region
  static constexpr int HX = 32 + 2 * R, HY = TY + 2 * R;          // patch halo region
  // limb-plane row pitch: 4 x an odd number of words, so rows are 16-byte
  // aligned and eight threads reading eight rows with 128-bit loads hit
  // distinct bank groups
  static constexpr int HXP = (((HX + 3) / 4) | 1) * 4, TXP = 33;
  static constexpr int W = 2 * R + 1;
  static constexpr int NP = HX * HY, NPW = PW * PH;
  // quantised-field ring of the z window: 2R+1 slices, the entering slice
  // taking the leaving slice's slot (each entry is read, then rewritten, by
  // the one thread that owns its halo point)
  static constexpr int RING = (ND == 3) ? 2 * R + 1 : 0;
  static constexpr int MAXP = (NP + NT - 1) / NT;   // halo points per thread
  static constexpr int WP = (NPW + NT - 1) / NT;    // resampled points per thread
  static constexpr int NPLANES = (ND == 3) ? 3 : 1;
  // leaving ring entries per point: qM, qG, and qU where shared memory allows
  // (16- and 24-row tiles, one CTA per SM); 8-row tiles keep two CTAs
  // resident and reload the leaving ultrasound instead
  static constexpr int RINGW = (ND == 3 && (TY == 16 || TY == 24)) ? 3 : 2;
  // shared memory: M plane, interleaved (Sz, Dz) plane, leaving ring, limb planes
  static constexpr size_t OFF_LV = sizeof(float) * (size_t)NPLANES * NPW;
  static constexpr size_t OFF_A = OFF_LV + sizeof(int) * (size_t)RING * RINGW * NP;
  static constexpr size_t BYTES = OFF_A + sizeof(int) * (size_t)kLimbs * HY * HXP;
  static_assert(ND == 2 || TY == 8 || BYTES + 1024 <= 227 * 1024,
                "one CTA's shared memory must fit an SM");
};

// Halo point p -> (row, column) of the HY x HX halo of a 3D tile of TY rows:
// the first 32 columns row by row (a warp per row), then the 2R-column
// tail; at radius 4 a warp takes 8 tail columns of rows r, r+2, r+4, r+6, so
// that its stores to limb planes of row pitch 44 words (and its reads of a
// float2 plane of pitch 4 mod 8 words) hit distinct banks.
template <int TY, int R>
__device__ __forceinline__ void halo_point(int p, int& hy, int& hx) {
  constexpr int HY = TY + 2 * R;
  static_assert(2 * R != 8 || HY % 8 == 0, "8-row groups of tail blocks");
  if (p < 32 * HY) {
    hy = p >> 5;
    hx = p & 31;
  } else {
    const int t = p - 32 * HY;
    if (2 * R == 8) {
      const int tw = t >> 5, lane = t & 31;
      hy = (tw >> 1) * 8 + (tw & 1) + 2 * (lane >> 3);
      hx = 32 + (lane & 7);
    } else {
      hy = t / (2 * R);
      hx = 32 + (t - hy * (2 * R));
    }
  }
}

// Halo point q of a 2D tile -> (hy, hx): the first 32 columns row by row,
// one row per warp, then the 2R-column tail row by row. A warp's plane reads
// and limb writes are then 32 consecutive words (row-major numbering over the
// 32+2R wide halo put a row break inside most warps: 33-40 words, two lanes on
// one bank), which pays in the shared-memory-bound 2D kernels (+3.6 %). The
// 3D kernels keep row-major numbering: there the tail warps' global loads of
// the static fields would span four rows. Every sum is exact, so the
// assignment does not change results.
template <int HX, int HY>
__device__ __forceinline__ void halo_coord(int q, int& hy, int& hx) {
  constexpr int MAIN = 32 * HY, TW = HX - 32;
  if (q < MAIN) {
    hy = q >> 5;
    hx = q & 31;
  } else {
    const int t = q - MAIN;
    hy = t / TW;
    hx = 32 + (t - hy * TW);
  }
}

// Trilinear / bilinear sample of the moving image at region point (px, py)
// of the current slice; sb/sf: integer part and fraction of the region base.
template <int WND, typename TM>
__device__ __forceinline__ float fused_sample(const TM* __restrict__ mov, const FusedParams& P,
                                              const float* A, const int* sb, const float* sf,
                                              int px, int py) {
  const float dx = (float)px, dy = (float)py;
  float qx = fmaf(A[1], dy, fmaf(A[0], dx, sf[0]));
  float qy = fmaf(A[4], dy, fmaf(A[3], dx, sf[1]));
  Axis ax = make_axis(sb[0], qx, P.mx);
  Axis ay = make_axis(sb[1], qy, P.my);
  if (WND == 3) {
    float qz = fmaf(A[7], dy, fmaf(A[6], dx, sf[2]));
    Axis az = make_axis(sb[2], qz, P.mz);
    if (!(ax.ok && ay.ok && az.ok)) return 0.0f;
    // one 32-bit linear index and the corner offsets (volumes hold < 2^31
    // voxels, checked on the host)
    const unsigned mxy = (unsigned)P.mx * (unsigned)P.my;
    const unsigned b = (unsigned)ax.f + (unsigned)ay.f * (unsigned)P.mx + (unsigned)az.f * mxy;
    const unsigned ox = (unsigned)(ax.c - ax.f), oy = (unsigned)(ay.c - ay.f) * (unsigned)P.mx,
                   oz = (unsigned)(az.c - az.f) * mxy;
    float lu0 = ldf(mov, b), lu1 = ldf(mov, b + oz);
    float ru0 = ldf(mov, b + ox), ru1 = ldf(mov, b + ox + oz);
    float rb0 = ldf(mov, b + ox + oy), rb1 = ldf(mov, b + ox + oy + oz);
    float lb0 = ldf(mov, b + oy), lb1 = ldf(mov, b + oy + oz);
    float lu = fmaf(az.r, lu1 - lu0, lu0), ru = fmaf(az.r, ru1 - ru0, ru0);
    float rb = fmaf(az.r, rb1 - rb0, rb0), lb = fmaf(az.r, lb1 - lb0, lb0);
    float l = fmaf(ay.r, lb - lu, lu), r = fmaf(ay.r, rb - ru, ru);
    return fmaf(ax.r, r - l, l);
  }
  if (!(ax.ok && ay.ok)) return 0.0f;
  const unsigned b = (unsigned)ax.f + (unsigned)ay.f * (unsigned)P.mx;
  const unsigned ox = (unsigned)(ax.c - ax.f), oy = (unsigned)(ay.c - ay.f) * (unsigned)P.mx;
  float f0 = ldf(mov, b), f1 = ldf(mov, b + oy);
  float c0 = ldf(mov, b + ox), c1 = ldf(mov, b + ox + oy);
  float xl = fmaf(ay.r, f1 - f0, f0), xr = fmaf(ay.r, c1 - c0, c0);
  return fmaf(ax.r, xr - xl, xl);
}

// Trilinear sample of a point known to lie strictly inside the moving volume
// (the region test of set_base): no bounds tests, corner offsets fixed. The
// ceil corner is always floor + 1; where the fraction is 0 its weight is 0,
// so the value equals fused_sample's bit for bit.
template <typename TM>
__device__ __forceinline__ float fused_sample_inside(const TM* __restrict__ mov,
                                                     const FusedParams& P, const float* A,
                                                     const int* sb, const float* sf, int px,
                                                     int py) {
  const float dx = (float)px, dy = (float)py;
  const float qx = fmaf(A[1], dy, fmaf(A[0], dx, sf[0]));
  const float qy = fmaf(A[4], dy, fmaf(A[3], dx, sf[1]));
  const float qz = fmaf(A[7], dy, fmaf(A[6], dx, sf[2]));
  const float flx = floorf(qx), fly = floorf(qy), flz = floorf(qz);
  const float rx = qx - flx, ry = qy - fly, rz = qz - flz;
  const unsigned mx = (unsigned)P.mx, mxy = (unsigned)P.mx * (unsigned)P.my;
  const unsigned b = (unsigned)(sb[0] + (int)flx) + (unsigned)(sb[1] + (int)fly) * mx +
                     (unsigned)(sb[2] + (int)flz) * mxy;
  float lu0 = ldf(mov, b), lu1 = ldf(mov, b + mxy);
  float ru0 = ldf(mov, b + 1), ru1 = ldf(mov, b + 1 + mxy);
  float rb0 = ldf(mov, b + 1 + mx), rb1 = ldf(mov, b + 1 + mx + mxy);
  float lb0 = ldf(mov, b + mx), lb1 = ldf(mov, b + mx + mxy);
  float lu = fmaf(rz, lu1 - lu0, lu0), ru = fmaf(rz, ru1 - ru0, ru0);
  float rb = fmaf(rz, rb1 - rb0, rb0), lb = fmaf(rz, lb1 - lb0, lb0);
  float l = fmaf(ry, lb - lu, lu), r = fmaf(ry, rb - ru, ru);
  return fmaf(rx, r - l, l);
}

// 12 limbs of one point's moment fields: qM, qG, then (lo, hi) of the
// products UM, UG, MM, GG, MG split as hi * 2^K + lo.
__device__ __forceinline__ void fused_limbs(int qu, int qm, int qg, int K, int* L) {
  const unsigned long long mask = (1ull << K) - 1ull;
  const long long p[5] = {(long long)qu * qm, (long long)qu * qg, (long long)qm * qm,
                          (long long)qg * qg, (long long)qm * qg};
  L[0] = qm;
  L[1] = qg;
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    L[2 + 2 * i] = (int)((unsigned long long)p[i] & mask);
    L[3 + 2 * i] = (int)(p[i] >> K);
  }
}

// Barrier of the threads that run the window passes: the whole CTA (BAR = 0)
// or, in the warp-specialised kernel, named barrier BAR of its NT threads.
template <int BAR, int NT>
__device__ __forceinline__ void group_sync() {
  if constexpr (BAR == 0) {
    __syncthreads();
  } else {
    asm volatile("bar.sync %0, %1;" ::"n"(BAR), "n"(NT) : "memory");
  }
}

// x window pass in place over NL limb planes: afterwards rows < HY, columns
// < 32 hold the x-window sums. One thread per (limb, row); each loads its row
// into registers before writing.
template <int ND, int TY, int R, int NL = kLimbs>
__device__ __forceinline__ void fused_xpass(int* __restrict__ A) {
  using G = FusedGeom<ND, TY, R>;
  const int tid = threadIdx.x;
  for (int it = tid; it < NL * G::HY; it += G::NT) {
    int* row = A + (size_t)it * G::HXP;  // it = limb * HY + row
    constexpr int NV = (G::HX + 3) / 4;   // 128-bit loads covering the row
    int v[4 * NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      const int4 q = reinterpret_cast<const int4*>(row)[i];
      v[4 * i] = q.x;
      v[4 * i + 1] = q.y;
      v[4 * i + 2] = q.z;
      v[4 * i + 3] = q.w;
    }
    // two independent sliding sums (outputs 0-15 and 16-31) for ILP
    int a = 0, b = 0;
#pragma unroll
    for (int i = 0; i < G::W; ++i) {
      a += v[i];
      b += v[16 + i];
    }
    int o[4], q[4];
    o[0] = a;
    q[0] = b;
#pragma unroll
    for (int x = 1; x < 16; ++x) {
      a += v[x + G::W - 1] - v[x - 1];
      b += v[16 + x + G::W - 1] - v[16 + x - 1];
      o[x & 3] = a;
      q[x & 3] = b;
      if ((x & 3) == 3) {
        reinterpret_cast<int4*>(row)[x >> 2] = make_int4(o[0], o[1], o[2], o[3]);
        reinterpret_cast<int4*>(row)[4 + (x >> 2)] = make_int4(q[0], q[1], q[2], q[3]);
      }
    }
  }
}

// y window pass over the x-window sums: the patch sum of limb L at output
// (column, row) goes to out[L * limb_stride + row * row_stride + column].
// One thread per (limb, column); each loads its column first, so out may be
// A itself.
template <int ND, int TY, int R, int NL = kLimbs>
__device__ __forceinline__ void fused_ypass(const int* A, int* out, int row_stride,
                                            int limb_stride) {
  using G = FusedGeom<ND, TY, R>;
  const int tid = threadIdx.x;
  for (int it = tid; it < NL * 32; it += G::NT) {
    const int L = it >> 5, col = it & 31;
    const int* c = A + (size_t)L * G::HY * G::HXP + col;
    int* o = out + (size_t)L * limb_stride + col;
    int v[G::HY];
#pragma unroll
    for (int i = 0; i < G::HY; ++i) v[i] = c[i * G::HXP];
    constexpr int H = TY / 2;  // two independent sliding sums (rows 0..H-1, H..TY-1)
    int a = 0, b = 0;
#pragma unroll
    for (int i = 0; i < G::W; ++i) {
      a += v[i];
      b += v[H + i];
    }
    o[0] = a;
    o[H * row_stride] = b;
#pragma unroll
    for (int y = 1; y < H; ++y) {
      a += v[y + G::W - 1] - v[y - 1];
      b += v[H + y + G::W - 1] - v[H + y - 1];
      o[y * row_stride] = a;
      o[(H + y) * row_stride] = b;
    }
  }
}

// x and y window passes in place on the limb planes A: after them, A rows
// < TY, columns < 32 hold the patch sums.
template <int ND, int TY, int R, int BAR = 0, int NL = kLimbs>
__device__ __forceinline__ void fused_xy(int* __restrict__ A) {
  using G = FusedGeom<ND, TY, R>;
  fused_xpass<ND, TY, R, NL>(A);
  group_sync<BAR, G::NT>();
  fused_ypass<ND, TY, R, NL>(A, A, G::HXP, G::HY * G::HXP);
  group_sync<BAR, G::NT>();
}

// Clipped measure of one voxel from exact sums; sigma > 0 is the
// precomputed weighting factor (0 marks an invalid patch).
__device__ __forceinline__ float fused_solve(const FusedParams& P, long long n, float sigma,
                                             int s_u, int s_m, int s_g, long long s_um,
                                             long long s_ug, long long s_mm, long long s_gg,
                                             long long s_mg) {
  long long d_mm = n * s_mm - (long long)s_m * s_m;
  long long d_gg = n * s_gg - (long long)s_g * s_g;
  long long d_mg = n * s_mg - (long long)s_m * s_g;
  long long d_um = n * s_um - (long long)s_u * s_m;
  long long d_ug = n * s_ug - (long long)s_u * s_g;
  const bool km = d_mm > P.thr_m, kg = d_gg > P.thr_g;
  // fast divisions (2 ulp): sigma > 1e-3 and den in (1e-3, 1]
  const float iu = __fdividef(P.sig_scale, sigma);  // 1/sqrt(D_uu)
  float r2 = 0.0f;
  if (km && kg) {
    float im = rsqrtf(ll2f(d_mm)), ig = rsqrtf(ll2f(d_gg));
    float rum = ll2f(d_um) * iu * im, rug = ll2f(d_ug) * iu * ig, rmg = ll2f(d_mg) * im * ig;
    float den = 1.0f - rmg * rmg;
    if (den > 1e-3f) {
      r2 = __fdividef(rum * rum + rug * rug - 2.0f * rum * rug * rmg, den);
    } else {
      // nearly collinear columns: solve in double from the exact sums
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
    float c = ll2f(d_um) * iu * rsqrtf(ll2f(d_mm));
    r2 = c * c;
  } else if (kg) {
    float c = ll2f(d_ug) * iu * rsqrtf(ll2f(d_gg));
    r2 = c * c;
  }
  float m = sigma * r2;
  if (!(m > 0.0f) || isinf(m)) m = 0.0f;
  return m;
}

// Patch sums from the 12 limbs of an output voxel (patch of PatchConst<ND,R>
// voxels), then its clipped measure.
template <int ND, int R>
__device__ __forceinline__ float fused_measure(const FusedParams& P, float sg, int s_u,
                                               const int* L) {
  using C = PatchConst<ND, R>;
  long long Sx[5];
#pragma unroll
  for (int i = 0; i < 5; ++i)
    Sx[i] = (long long)L[3 + 2 * i] * (1LL << C::K) + (long long)L[2 + 2 * i];
  return fused_solve(P, C::N, sg, s_u, L[0], L[1], Sx[0], Sx[1], Sx[2], Sx[3], Sx[4]);
}

// Square root of a Sobel magnitude: PTX sqrt.approx (one instruction, a
// couple of ulp). The magnitude is quantised at 2^-20 of its range or finer next, so
// the approximation never moves a quantised value by more than one step and
// LC2 by far less than 1e-7.
__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Sobel magnitude at plane index c (centre of a 3x3 in-plane neighbourhood).
template <int ND, int PW>
__device__ __forceinline__ float fused_sobel(const float* mc, const float* S, const float* D,
                                             int c) {
  const int up = c - PW, dn = c + PW;
  if (ND == 3) {
    float gx = (S[up + 1] - S[up - 1]) + 2.0f * (S[c + 1] - S[c - 1]) + (S[dn + 1] - S[dn - 1]);
    float gy = (S[dn - 1] - S[up - 1]) + 2.0f * (S[dn] - S[up]) + (S[dn + 1] - S[up + 1]);
    float gz = (D[up - 1] + 2.0f * D[up] + D[up + 1]) + 2.0f * (D[c - 1] + 2.0f * D[c] + D[c + 1]) +
               (D[dn - 1] + 2.0f * D[dn] + D[dn + 1]);
    return sqrt_approx(gx * gx + gy * gy + gz * gz);
  }
  const float* M = mc;
  float gx = (M[up + 1] - M[up - 1]) + 2.0f * (M[c + 1] - M[c - 1]) + (M[dn + 1] - M[dn - 1]);
  float gy = (M[dn - 1] - M[up - 1]) + 2.0f * (M[dn] - M[up]) + (M[dn + 1] - M[up + 1]);
  return sqrt_approx(gx * gx + gy * gy);
}

// 3D Sobel magnitude at plane index c from the interleaved (Sz, Dz) plane:
// the nine 64-bit reads of the 3x3 neighbourhood, same arithmetic as
// fused_sobel<3>.
template <int PW>
__device__ __forceinline__ float fused_sobel_sd(const float2* SD, int c) {
  const int up = c - PW, dn = c + PW;
  const float2 a0 = SD[up - 1], a1 = SD[up], a2 = SD[up + 1];
  const float2 b0 = SD[c - 1], b1 = SD[c], b2 = SD[c + 1];
  const float2 c0 = SD[dn - 1], c1 = SD[dn], c2 = SD[dn + 1];
  float gx = (a2.x - a0.x) + 2.0f * (b2.x - b0.x) + (c2.x - c0.x);
  float gy = (c0.x - a0.x) + 2.0f * (c1.x - a1.x) + (c2.x - a2.x);
  float gz = (a0.y + 2.0f * a1.y + a2.y) + 2.0f * (b0.y + 2.0f * b1.y + b2.y) +
             (c0.y + 2.0f * c1.y + c2.y);
  return sqrt_approx(gx * gx + gy * gy + gz * gz);
}

// Sampling base of a tile's PW x PH resampled region at slice zs: the
// moving-pixel coordinate of the canonical base, region row -yb (yb = 0 in
// 2D), split into integer part ib and fraction fb (xform_coord); returns
// whether the region lies in the virtual grid (origin gx0, gy0; zin: the
// slice is in the grid) with every sample of it strictly inside the moving
// image along its first WND axes (0 <= floor, floor + 1 <= dim - 1; the
// region's corners bound the affine image, 0.01 voxel covers float rounding).
template <int WND, int PW, int PH>
__device__ __forceinline__ bool region_base(const Xform& X, const float* A, const FusedParams& P,
                                            int gx0, int gy0, int yb, int zs, bool zin,
                                            int* ib, float* fb) {
  bool in = zin && gx0 >= 0 && gx0 + PW <= P.vx && gy0 >= 0 && gy0 + PH <= P.vy;
  const int dims[3] = {P.mx, P.my, P.mz};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    xform_coord(X, a, gx0, gy0 - yb, zs, ib[a], fb[a]);
    if (a < WND) {
      const float ex = A[3 * a] * (float)(PW - 1);
      const float e0 = A[3 * a + 1] * (float)yb, e1 = A[3 * a + 1] * (float)(yb + PH - 1);
      const float lo = fb[a] + fminf(ex, 0.0f) + fminf(e0, e1);
      const float hi = fb[a] + fmaxf(ex, 0.0f) + fmaxf(e0, e1);
      in = in && ((float)ib[a] + lo >= 0.01f) &&
           ((float)ib[a] + hi <= (float)(dims[a] - 1) - 0.01f);
    }
  }
  return in;
}

// Per-tile transform state in shared memory.
struct TileShared {
  int ib[3];       // resampled-region origin in moving pixels: integer part
  float fb[3];     // and fraction
  float A[9];      // moving-pixel step per region pixel
  int inside;      // every sample of the region lies strictly inside the moving image
};

// Bilinear counterpart of fused_sample_inside (2D moving image).
template <typename TM>
__device__ __forceinline__ float fused_sample_inside2(const TM* __restrict__ mov,
                                                      const FusedParams& P, const float* A,
                                                      const int* sb, const float* sf, int px,
                                                      int py) {
  const float dx = (float)px, dy = (float)py;
  const float qx = fmaf(A[1], dy, fmaf(A[0], dx, sf[0]));
  const float qy = fmaf(A[4], dy, fmaf(A[3], dx, sf[1]));
  const float flx = floorf(qx), fly = floorf(qy);
  const float rx = qx - flx, ry = qy - fly;
  const unsigned mx = (unsigned)P.mx;
  const unsigned b = (unsigned)(sb[0] + (int)flx) + (unsigned)(sb[1] + (int)fly) * mx;
  float f0 = ldf(mov, b), f1 = ldf(mov, b + mx);
  float c0 = ldf(mov, b + 1), c1 = ldf(mov, b + 1 + mx);
  float xl = fmaf(ry, f1 - f0, f0), xr = fmaf(ry, c1 - c0, c0);
  return fmaf(rx, xr - xl, xl);
}

// One 32 x TY output tile of a 2D window (2D, or a 2D-to-3D frame when
// WND = 3): resample the halo region, Sobel, limbs, x/y window passes and the
// clipped measures. Returns this thread's fixed-point measure sum; the caller
// reduces it. Ends with the shared planes still in use: callers that reuse
// them for another tile must synchronise first.
template <int WND, typename TM, typename TS, int TY, int R>
__device__ __forceinline__ long long fused_tile_2d(const TM* __restrict__ mov,
                                                   const TS* __restrict__ Ust,
                                                   const float* __restrict__ sig,
                                                   const int* __restrict__ su,
                                                   const FusedParams& P, const Xform* X, int tile,
                                                   unsigned char* smem_raw, TileShared& T,
                                                   float* __restrict__ out_measure) {
  using G = FusedGeom<2, TY, R>;
  constexpr int NT = G::NT;
  constexpr size_t PA = (size_t)G::HY * G::HXP;
  float* mc = reinterpret_cast<float*>(smem_raw);
  int* A = reinterpret_cast<int*>(smem_raw + G::OFF_A);
  const int tid = threadIdx.x;
  const int ntx = P.ntx;
  const int x0 = (tile % ntx) * 32, y0 = (tile / ntx) * TY;
  const int gx0 = x0 - R - 1, gy0 = y0 - R - 1;
  // sampling base (x0 - R - 1, 32 floor(y0 / 32) - R - 1): tiles are 16 or
  // 32 rows high, and both heights sample every pixel identically
  const int yb = y0 & 31;
  if (tid == 0) {
#pragma unroll
    for (int i = 0; i < 9; ++i) T.A[i] = X->ah[i];
    T.inside =
        region_base<WND, G::PW, G::PH>(*X, T.A, P, gx0, gy0, yb, 0, true, T.ib, T.fb) ? 1 : 0;
  }
  __syncthreads();
  if (T.inside) {
    for (int i = tid; i < G::NPW; i += NT) {
      const int py = i / G::PW, px = i - py * G::PW;
      if constexpr (WND == 3)
        mc[i] = fused_sample_inside<TM>(mov, P, T.A, T.ib, T.fb, px, py + yb);
      else
        mc[i] = fused_sample_inside2<TM>(mov, P, T.A, T.ib, T.fb, px, py + yb);
    }
  } else {
    for (int i = tid; i < G::NPW; i += NT) {
      const int py = i / G::PW, px = i - py * G::PW;
      const int gx = gx0 + px, gy = gy0 + py;
      float v = 0.0f;
      if (gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy)
        v = fused_sample<WND, TM>(mov, P, T.A, T.ib, T.fb, px, py + yb);
      mc[i] = v;
    }
  }
  __syncthreads();
  for (int p = tid; p < G::NP; p += NT) {
    int hy, hx;
    halo_coord<G::HX, G::HY>(p, hy, hx);
    const int gx = x0 - R + hx, gy = y0 - R + hy;
    const int c = (hy + 1) * G::PW + hx + 1;
    const float m = mc[c];
    const float g = fused_sobel<2, G::PW>(mc, nullptr, nullptr, c);
    float u = 0.0f;
    if (gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy) u = ldf(Ust, (size_t)gy * P.vx + gx);
    int L[kLimbs];
    fused_limbs(quant(u, P.qu), quant(m, P.qm), quant(g, P.qg), PatchConst<2, R>::K, L);
    int* a = A + hy * G::HXP + hx;
#pragma unroll
    for (int k = 0; k < kLimbs; ++k) a[k * PA] = L[k];
  }
  __syncthreads();
  fused_xy<2, TY, R>(A);
  long long acc_m = 0;
  const int ox = tid & 31, oy = tid >> 5;
  const int x = x0 + ox, y = y0 + oy;
  if (x < P.vx && y < P.vy) {
    const size_t gi = (size_t)y * P.vx + x;
    const float sg = __ldg(sig + gi);
    const int sv = __ldg(su + gi);
    float m = 0.0f;
    if (sg > 0.0f) {
      const int* a = A + oy * G::HXP + ox;
      int L[kLimbs];
#pragma unroll
      for (int k = 0; k < kLimbs; ++k) L[k] = a[k * PA];
      m = fused_measure<2, R>(P, sg, sv, L);
      acc_m = __float2int_rn(m * P.sum_scale);
    }
    if (out_measure) out_measure[gi] = m;
  }
  return acc_m;
}

// CTAs per SM each variant is compiled for: 2D 16-row tiles 4, 32-row tiles
// 2; 3D 16- and 24-row tiles 1; 3D 8-row tiles 2 up to radius 4 (beyond,
// shared memory holds only one).
constexpr int fused_min_blocks(int nd, int ty, int r) {
  return nd == 2 ? (ty == 32 ? 2 : 4) : (ty == 8 && r <= 4 ? 2 : 1);
}

// Resample stage as a pass of its own (presampling): the moving image on the
// virtual grid for `count` transforms, one float per voxel, slot-major. Each
// 32 x 8 tile slice samples from its own base (tile_base, as the generic
// resampling kernel does), so every voxel has one value whichever fused CTA
// reads it; slices that sample strictly inside the moving image skip the
// bounds tests (same bits). A CTA covers kPreZ slices of one tile: their
// bases are computed by 3 kPreZ threads at once, and each thread then has
// kPreZ independent samples in flight. The output is written with streaming
// stores (it is read once, by another kernel, and should not evict the
// moving volume from L2).
constexpr int kPreZ = 8;

template <typename TM>
__global__ void __launch_bounds__(256) k_presample(const TM* __restrict__ mov, int mx, int my,
                                                   int mz, int vx, int vy, int vz,
                                                   const Xform* __restrict__ xf, int k0,
                                                   float* __restrict__ out) {
  __shared__ int s_ib[kPreZ][3];
  __shared__ float s_fb[kPreZ][3];
  __shared__ float s_A[9];
  __shared__ int s_in[kPreZ];
  const int ntx = (vx + 31) >> 5;
  const int x0 = (blockIdx.x % ntx) * 32, y0 = (blockIdx.x / ntx) * 8;
  const int z0 = blockIdx.y * kPreZ, slot = blockIdx.z;
  const int tid = threadIdx.x;
  const Xform* X = xf + k0 + slot;
  if (tid < 3 * kPreZ) {
    const int zs = tid / 3, a = tid - 3 * zs;
    xform_coord(*X, a, x0, y0, z0 + zs, s_ib[zs][a], s_fb[zs][a]);
  } else if (tid < 3 * kPreZ + 9) {
    s_A[tid - 3 * kPreZ] = X->ah[tid - 3 * kPreZ];
  }
  __syncthreads();
  if (tid < kPreZ) {
    TileBase T;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      T.ib[a] = s_ib[tid][a];
      T.fb[a] = s_fb[tid][a];
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) T.A[i] = s_A[i];
    s_in[tid] = tile_inside(T, mx, my, mz) ? 1 : 0;
  }
  __syncthreads();
  const int tx = tid & 31, ty = tid >> 5;
  const int x = x0 + tx, y = y0 + ty;
  if (x >= vx || y >= vy) return;
  const size_t plane = (size_t)vx * vy;
  float* dst = out + (size_t)slot * plane * vz + (size_t)y * vx + x;
  float v[kPreZ];
#pragma unroll
  for (int zs = 0; zs < kPreZ; ++zs) {
    TileBase T;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      T.ib[a] = s_ib[zs][a];
      T.fb[a] = s_fb[zs][a];
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) T.A[i] = s_A[i];
    v[zs] = s_in[zs] ? tile_sample_inside<TM>(mov, mx, my, T, tx, ty)
                     : tile_sample<3, TM>(mov, mx, my, mz, T, tx, ty);
  }
#pragma unroll
  for (int zs = 0; zs < kPreZ; ++zs)
    if (z0 + zs < vz) __stcs(dst + (size_t)(z0 + zs) * plane, v[zs]);
}

// PRE: the moving image is read from a presampled buffer (k_presample, one
// float per virtual voxel and transform of the launch, slot-major) instead of
// being resampled by the CTA.
template <int ND, int WND, typename TM, typename TS, int TY, int R, bool PRE = false>
__global__ void __launch_bounds__(32 * TY, fused_min_blocks(ND, TY, R))
    k_fused(const TM* __restrict__ mov, const TS* __restrict__ Ust, const float* __restrict__ sig,
            const int* __restrict__ su, FusedParams P, const Xform* __restrict__ xf, int k0,
            unsigned long long* __restrict__ acc, float* __restrict__ out_measure,
            const float* __restrict__ pre = nullptr) {
  using G = FusedGeom<ND, TY, R>;
  constexpr int NT = G::NT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* mc = reinterpret_cast<float*>(smem_raw);
  float2* SD = reinterpret_cast<float2*>(mc + G::NPW);  // NPW is even: 8-byte aligned
  int* lv = reinterpret_cast<int*>(smem_raw + G::OFF_LV);
  int* A = reinterpret_cast<int*>(smem_raw + G::OFF_A);
  constexpr size_t PA = (size_t)G::HY * G::HXP;
  __shared__ Xform s_xf;
  __shared__ int s_ib[3];
  __shared__ float s_fb[3];
  __shared__ float s_A[9];
  __shared__ int s_inside;  // the region of the current slice samples strictly inside
  const int tid = threadIdx.x;
  const int slot = blockIdx.x;
  const int tile = blockIdx.y;
  const int x0 = (tile % P.ntx) * 32, y0 = (tile / P.ntx) * TY;
  const Xform* X = xf + k0 + slot;
  const int gx0 = x0 - R - 1, gy0 = y0 - R - 1;  // origin of the resampled region
  // Sampling base: (x0 - R - 1, 48 floor(y0 / 48) - R - 1). Tiles are 32
  // wide in every kernel and 8, 16 or 24 rows high, so this base -- and with
  // it every sample, patch sum and LC2 value -- is the same whichever tile
  // height computes an output voxel. yb: row offset of the region origin.
  const int yb = y0 % kBand;
  const int ox = tid & 31, oy = tid >> 5;
  long long acc_m = 0;

  // sampling base at slice zs (xform_coord), split into integer part and
  // fraction for the float per-point offsets; run by the last thread, whose
  // warp holds the fewest halo points
  auto set_base = [&](int zs) {
    if (PRE) return;
    if (tid == NT - 1)
      s_inside = region_base<3, G::PW, G::PH>(s_xf, s_A, P, gx0, gy0, yb, zs,
                                              ND == 3 && zs >= 0 && zs < P.vz, s_ib, s_fb)
                     ? 1 : 0;
  };
  if (tid == 0) {
    s_xf = *X;
#pragma unroll
    for (int i = 0; i < 9; ++i) s_A[i] = X->ah[i];
  }

  // solve one output voxel from the patch sums in A rows < TY
  // sg, sv: the voxel's weighting factor and static S_U, loaded a slice ahead
  auto solve_out = [&](int z, float sg, int sv) {
    const int x = x0 + ox, y = y0 + oy;
    if (x < P.vx && y < P.vy) {
      const size_t gi = ((size_t)z * P.vy + y) * P.vx + x;
      float m = 0.0f;
      if (sg > 0.0f) {
        const int* a = A + oy * G::HXP + ox;
        int L[kLimbs];
#pragma unroll
        for (int k = 0; k < kLimbs; ++k) L[k] = a[k * PA];
        m = fused_measure<ND, R>(P, sg, sv, L);
        acc_m += __float2int_rn(m * P.sum_scale);
      }
      if (out_measure && slot == 0) out_measure[gi] = m;
    }
  };

  if constexpr (ND == 2) {
    __shared__ TileShared T;
    acc_m = fused_tile_2d<WND, TM, TS, TY, R>(mov, Ust, sig, su, P, X, tile, smem_raw, T,
                                              slot == 0 ? out_measure : nullptr);
  } else {
    // ---- 3D: z-marching over output slices [zb, ze) ----
    const int zb = blockIdx.z * P.zchunk;
    const int ze = min(zb + P.zchunk, P.vz);
    constexpr int MAXP = G::MAXP, WP = G::WP;
    // z-window sums of each halo point: qM, qG exactly in int32, the five
    // products in int64 (split into hi * 2^K + lo limbs only when written)
    int accq[MAXP][2];
    long long accp[MAXP][5];
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      accq[j][0] = accq[j][1] = 0;
#pragma unroll
      for (int k = 0; k < 5; ++k) accp[j][k] = 0;
    }
    constexpr int KB = PatchConst<ND, R>::K;
    constexpr unsigned long long kmask = (1ull << KB) - 1ull;
    // per-thread constants of its halo points: plane index, A offset, U offset
    int pc[MAXP], pa_off[MAXP], pu[MAXP];
    bool pin[MAXP];
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const int p = tid + j * NT;
      const int hy = p / G::HX, hx = p - hy * G::HX;
      const int gx = x0 - R + hx, gy = y0 - R + hy;
      pc[j] = (hy + 1) * G::PW + hx + 1;
      pa_off[j] = hy * G::HXP + hx;
      pin[j] = (p < G::NP) && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy;
      pu[j] = pin[j] ? gy * P.vx + gx : 0;
    }
    const size_t slice = (size_t)P.vx * P.vy;
    // presampled input: this transform's images and the in-slice offset of
    // each of the thread's region points (-1 outside the grid: zero padding)
    const float* pre_slot = PRE ? pre + (size_t)slot * slice * P.vz : nullptr;
    int poff[PRE ? WP : 1];
    if constexpr (PRE) {
#pragma unroll
      for (int k = 0; k < WP; ++k) {
        const int i = tid + k * NT;
        const int py = i / G::PW, px = i - py * G::PW;
        const int gx = gx0 + px, gy = gy0 + py;
        poff[k] = (i < G::NPW && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy) ? gy * P.vx + gx
                                                                                : -1;
      }
    }
    float m_prev2[WP], m_prev1[WP];  // M of the thread's region points, slices e-1, e
    const int e0 = zb - R;           // first slice entering the window
    // static ultrasound of the entering and leaving slices, loaded one
    // iteration ahead
    float u_in[MAXP], u_out[MAXP];
    auto load_u = [&](int e) {
      const int l = e - 2 * R - 1;
      const bool ezin = (e >= 0 && e < P.vz), lzin = (l >= e0 && l >= 0 && l < P.vz);
#pragma unroll
      for (int j = 0; j < MAXP; ++j) {
        u_in[j] = (pin[j] && ezin) ? ldf(Ust, (size_t)e * slice + pu[j]) : 0.0f;
        if constexpr (G::RINGW == 2)
          u_out[j] = (pin[j] && lzin) ? ldf(Ust, (size_t)l * slice + pu[j]) : 0.0f;
        else
          u_out[j] = 0.0f;  // the ring holds the leaving qU
      }
    };
    load_u(e0);
    // weighting factor and S_U of the output voxel of slice z, loaded one
    // iteration before the solve that reads them
    float sg_nx = 0.0f;
    int sv_nx = 0;
    auto load_sig = [&](int z) {
      const int x = x0 + ox, y = y0 + oy;
      if (z >= zb && z < ze && x < P.vx && y < P.vy) {
        const size_t gi = ((size_t)z * P.vy + y) * P.vx + x;
        sg_nx = __ldg(sig + gi);
        sv_nx = __ldg(su + gi);
      }
    };
    load_sig(e0 - R);
    auto warp_slice = [&](int zs, float* out) {
      const bool zin = (zs >= 0 && zs < P.vz);
      if constexpr (PRE) {
        const float* src = pre_slot + (size_t)(zin ? zs : 0) * ((size_t)P.vx * P.vy);
#pragma unroll
        for (int k = 0; k < WP; ++k) out[k] = (zin && poff[k] >= 0) ? __ldcs(src + poff[k]) : 0.0f;
        return;
      }
      if (s_inside) {
#pragma unroll
        for (int k = 0; k < WP; ++k) {
          const int i = tid + k * NT;
          float v = 0.0f;
          if (i < G::NPW) {
            const int py = i / G::PW, px = i - py * G::PW;
            v = fused_sample_inside<TM>(mov, P, s_A, s_ib, s_fb, px, py + yb);
          }
          out[k] = v;
        }
        return;
      }
#pragma unroll
      for (int k = 0; k < WP; ++k) {
        const int i = tid + k * NT;
        float v = 0.0f;
        if (i < G::NPW) {
          const int py = i / G::PW, px = i - py * G::PW;
          const int gx = gx0 + px, gy = gy0 + py;
          if (zin && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy)
            v = fused_sample<3, TM>(mov, P, s_A, s_ib, s_fb, px, py + yb);
        }
        out[k] = v;
      }
    };
    __syncthreads();  // s_xf, s_A
    set_base(e0 - 1);
    __syncthreads();
    warp_slice(e0 - 1, m_prev2);
    __syncthreads();
    set_base(e0);
    __syncthreads();
    warp_slice(e0, m_prev1);
    __syncthreads();
    set_base(e0 + 1);
    __syncthreads();
    // presampled input: slice e+1 is loaded during iteration e-1, so its
    // global-memory latency overlaps a whole iteration
    float m_pf[PRE ? WP : 1];
    if constexpr (PRE) warp_slice(e0 + 1, m_pf);
    for (int e = e0; e < ze + R; ++e) {
      // resample slice e+1; write the planes of slice e
      {
        float m_next[WP];
        if constexpr (PRE) {
#pragma unroll
          for (int k = 0; k < WP; ++k) m_next[k] = m_pf[k];
          warp_slice(e + 2, m_pf);
        } else {
          warp_slice(e + 1, m_next);
        }
#pragma unroll
        for (int k = 0; k < WP; ++k) {
          const int i = tid + k * NT;
          if (i < G::NPW) {
            mc[i] = m_prev1[k];
            SD[i] = make_float2(m_prev2[k] + 2.0f * m_prev1[k] + m_next[k], m_next[k] - m_prev2[k]);
          }
          m_prev2[k] = m_prev1[k];
          m_prev1[k] = m_next[k];
        }
      }
      __syncthreads();
      set_base(e + 2);  // read by the next resample, after at least one barrier
      const int z = e - R;          // output slice completed by this entering slice
      const float sg = sg_nx;
      const int sv = sv_nx;
      const int l = e - 2 * R - 1;  // slice leaving the window
      const bool out = (z >= zb);
      const bool leave = (l >= e0);
      int* lv_in = lv + ((e - e0) % G::RING) * G::RINGW * G::NP;
      const int* lv_out = lv + ((l - e0 + G::RING) % G::RING) * G::RINGW * G::NP;
#pragma unroll
      for (int j = 0; j < MAXP; ++j) {
        const int p = tid + j * NT;
        if (p < G::NP) {
          const float m = mc[pc[j]];
          const float g = fused_sobel_sd<G::PW>(SD, pc[j]);
          const int qm = quant(m, P.qm), qg = quant(g, P.qg), qu = quant(u_in[j], P.qu);
          // the leaving slice's ring slot is the entering slice's: read it
          // before it is overwritten (only this thread touches entry p)
          if (leave) {
            const int qul = (G::RINGW == 3) ? lv_out[2 * G::NP + p] : quant(u_out[j], P.qu);
            const int qml = lv_out[p], qgl = lv_out[G::NP + p];
            accp[j][0] -= (long long)qul * qml;
            accp[j][1] -= (long long)qul * qgl;
            accp[j][2] -= (long long)qml * qml;
            accp[j][3] -= (long long)qgl * qgl;
            accp[j][4] -= (long long)qml * qgl;
            accq[j][0] -= qml;
            accq[j][1] -= qgl;
          }
          lv_in[p] = qm;
          lv_in[G::NP + p] = qg;
          if constexpr (G::RINGW == 3) lv_in[2 * G::NP + p] = qu;
          accp[j][0] += (long long)qu * qm;
          accp[j][1] += (long long)qu * qg;
          accp[j][2] += (long long)qm * qm;
          accp[j][3] += (long long)qg * qg;
          accp[j][4] += (long long)qm * qg;
          accq[j][0] += qm;
          accq[j][1] += qg;
          if (out) {
            // the same limb layout as fused_limbs: qM, qG, then (lo, hi) per product
            int* a = A + pa_off[j];
            a[0] = accq[j][0];
            a[PA] = accq[j][1];
#pragma unroll
            for (int k = 0; k < 5; ++k) {
              a[(2 + 2 * k) * PA] = (int)((unsigned long long)accp[j][k] & kmask);
              a[(3 + 2 * k) * PA] = (int)(accp[j][k] >> KB);
            }
          }
        }
      }
      load_u(e + 1);
      load_sig(z + 1);
      __syncthreads();
      if (out) {
        fused_xy<ND, TY, R>(A);
        solve_out(z, sg, sv);
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc_m += __shfl_down_sync(0xffffffffu, acc_m, o);
  if ((tid & 31) == 0) atomicAdd(acc + 2 * (size_t)(k0 + slot), (unsigned long long)acc_m);
}

// Output slices per CTA of a 3D launch left automatic: the z split with
// the smallest modelled makespan, waves x (chunk + 2R + 3) -- a CTA streams
// its chunk plus 2R warm-up slices after resampling three slices before its
// loop; `slots` CTAs run at once. One transform at 256^3 runs as one wave of
// whole-depth columns; one at 96^3 as one wave of 12-slice chunks.
inline int auto_zchunk(int vz, int R, long long tiles, long long slots) {
  slots = slots < 1 ? 1 : slots;
  long long best = -1;
  int best_zc = vz;
  for (int nz = 1; nz <= vz; ++nz) {
    const int zc = (vz + nz - 1) / nz;
    const long long chunks = (vz + zc - 1) / zc;
    const long long waves = (tiles * chunks + slots - 1) / slots;
    const long long cost = waves * (zc + 2 * R + 3);
    if (best < 0 || cost < best) {
      best = cost;
      best_zc = zc;
    }
  }
  return best_zc;
}

// Launch description shared by the per-storage-type launchers.
struct FusedLaunch {
  const void* mov;
  const void* ust;
  const float* sig;
  const int* su;  // static window sum of the quantised ultrasound per voxel
  FusedParams P;
  const Xform* xf;
  int k0, cnt;
  unsigned long long* acc;
  float* out_measure;
  int nd, wnd;
  int tile_height;  // 3D, radius <= 4: 16 or 8 rows per tile
  int zchunk;       // 3D: output slices per CTA; 0 = automatic
  int pipeline;     // 3D, radius <= 4, no per-voxel output: warp-specialised kernel
  int* err;         // device flag raised by the warp-specialised kernel's bounded waits
  int sms;          // multiprocessors of the device
  cudaStream_t stream;
  const float* pre = nullptr;  // 3D: presampled moving image of the launch (k_presample)
  // presampled 3D kernels: the launch's tiles cover output rows [y_off,
  // y_off + y_rows) (y_rows 0: the whole grid)
  int y_off = 0, y_rows = 0;
};

template <int ND, int WND, typename T, int R, int TY, typename K>
cudaError_t fused_launch_grid(const FusedLaunch& L, K kern);

template <int ND, int WND, typename T, int R, int TY>
cudaError_t fused_launch_rt(const FusedLaunch& L) {
  if (L.P.kbits != PatchConst<ND, R>::K || L.P.n != PatchConst<ND, R>::N)
    return cudaErrorInvalidValue;
  if constexpr (ND == 3) {
    if (L.pre) return fused_launch_grid<ND, WND, T, R, TY>(L, k_fused<ND, WND, T, T, TY, R, true>);
  }
  return fused_launch_grid<ND, WND, T, R, TY>(L, k_fused<ND, WND, T, T, TY, R, false>);
}

template <int ND, int WND, typename T, int R, int TY, typename K>
cudaError_t fused_launch_grid(const FusedLaunch& L, K kern) {
  using G = FusedGeom<ND, TY, R>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)G::BYTES);
  if (e != cudaSuccess) return e;
  FusedParams P = L.P;
  const int ntx = (P.vx + 31) / 32, nty = (P.vy + TY - 1) / TY;
  P.ntx = ntx;
  int nz = 1;
  if (ND == 3 && L.zchunk > 0) {
    P.zchunk = L.zchunk < P.vz ? L.zchunk : P.vz;
    nz = (P.vz + P.zchunk - 1) / P.zchunk;
  } else if (ND == 3) {
    P.zchunk = auto_zchunk(P.vz, R, (long long)ntx * nty * L.cnt,
                           (long long)L.sms * fused_min_blocks(3, TY, R));
    nz = (P.vz + P.zchunk - 1) / P.zchunk;
  } else {
    P.zchunk = 1;
  }
  dim3 grid(L.cnt, ntx * nty, nz);
  kern<<<grid, G::NT, G::BYTES, L.stream>>>((const T*)L.mov, (const T*)L.ust, L.sig, L.su, P, L.xf,
                                             L.k0, L.acc, L.out_measure, L.pre);
  return cudaGetLastError();
}

// k_presample of transforms [k0, k0 + cnt) into pre (cnt x voxels floats).
template <typename T>
cudaError_t presample_launch(const void* mov, const FusedParams& P, const Xform* xf, int k0,
                             int cnt, float* pre, cudaStream_t stream) {
  const int ntx = (P.vx + 31) / 32, nty = (P.vy + 7) / 8;
  dim3 grid(ntx * nty, (P.vz + kPreZ - 1) / kPreZ, cnt);
  k_presample<T><<<grid, 256, 0, stream>>>((const T*)mov, P.mx, P.my, P.mz, P.vx, P.vy, P.vz, xf,
                                           k0, pre);
  return cudaGetLastError();
}

// Tile heights: 3D patches of radius <= 4 run 32x16 tiles (one CTA per SM),
// 32x24 tiles (one 768-thread CTA per SM) or 32x8 tiles (two per SM); larger
// radii only fit 32x8; 2D runs 32x32 (two 1024-thread CTAs per SM, radius
// 4-6, launches of four CTAs per SM or more) or 32x16 tiles (four per SM).
template <int ND, int WND, typename T, int R>
cudaError_t fused_launch_r(const FusedLaunch& L) {
  if constexpr (ND == 3 && R > 4) {
    return fused_launch_rt<ND, WND, T, R, 8>(L);
  } else if constexpr (ND == 3) {
    if (L.tile_height == 8) return fused_launch_rt<ND, WND, T, R, 8>(L);
    if (L.tile_height == 24) return fused_launch_rt<ND, WND, T, R, 24>(L);
    return fused_launch_rt<ND, WND, T, R, 16>(L);
  } else if constexpr (R >= 4 && R <= 6) {
    // 32-row tiles (two 1024-thread CTAs per SM, a smaller halo per pixel)
    // where the launch has CTAs enough for the GPU: two per SM, twice over
    if (L.tile_height == 32 ||
        (L.tile_height != 16 && (long long)L.cnt * ((L.P.vx + 31) / 32) * ((L.P.vy + 31) / 32) >=
                                    4LL * L.sms))
      return fused_launch_rt<ND, WND, T, R, 32>(L);
    return fused_launch_rt<ND, WND, T, R, 16>(L);
  } else {
    return fused_launch_rt<ND, WND, T, R, 16>(L);
  }
}

// Dispatch over (dimensionality, patch radius); defined per storage type in
// lc2_fused_{f32,f16,bf16}.cu.
template <typename T>
cudaError_t fused_launch(const FusedLaunch& L);

template <int ND, int WND, typename T>
cudaError_t fused_launch_nd(const FusedLaunch& L) {
  switch (L.P.r) {
    case 1: return fused_launch_r<ND, WND, T, 1>(L);
    case 2: return fused_launch_r<ND, WND, T, 2>(L);
    case 3: return fused_launch_r<ND, WND, T, 3>(L);
    case 4: return fused_launch_r<ND, WND, T, 4>(L);
    case 5: return fused_launch_r<ND, WND, T, 5>(L);
    case 6: return fused_launch_r<ND, WND, T, 6>(L);
  }
  if constexpr (ND == 2) {
    switch (L.P.r) {
      case 7: return fused_launch_r<2, WND, T, 7>(L);
      case 8: return fused_launch_r<2, WND, T, 8>(L);
      case 9: return fused_launch_r<2, WND, T, 9>(L);
      case 10: return fused_launch_r<2, WND, T, 10>(L);
      case 11: return fused_launch_r<2, WND, T, 11>(L);
      case 12: return fused_launch_r<2, WND, T, 12>(L);
    }
  }
  return cudaErrorInvalidValue;
}

// Warp-specialised 3D kernel (lc2_fused_ws.cuh), defined in the same
// translation units.
template <typename T>
cudaError_t fused_ws_launch(const FusedLaunch& L, int* err);

// Self-test of the warp-specialised kernel's bounded waits: one warp waits
// on a barrier that nothing completes until the wait's time limit raises
// `err` (defined in lc2_fused_f32.cu).
cudaError_t wait_probe_launch(int* err, cudaStream_t stream);

template <>
cudaError_t fused_launch<float>(const FusedLaunch& L);
template <>
cudaError_t fused_launch<__half>(const FusedLaunch& L);
template <>
cudaError_t fused_launch<__nv_bfloat16>(const FusedLaunch& L);

#define LC2_DEFINE_FUSED_LAUNCH(T)                                  \
  template <>                                                       \
  cudaError_t fused_launch<T>(const FusedLaunch& L) {               \
    if (L.nd == 3 && L.pipeline && L.P.r <= 4 && !L.out_measure)    \
      return fused_ws_launch<T>(L, L.err);                          \
    if (L.nd == 3) return fused_launch_nd<3, 3, T>(L);              \
    if (L.wnd == 3) return fused_launch_nd<2, 3, T>(L);             \
    return fused_launch_nd<2, 2, T>(L);                             \
  }

}  // namespace lc2
