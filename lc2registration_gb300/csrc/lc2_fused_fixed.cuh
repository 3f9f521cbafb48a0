// lc2_fused_fixed.cuh -- fused LC2 evaluation for a resampled ultrasound
// (HighResolutionModality: Fixed: the fixed MR/CT is the high-resolution
// image, static on the virtual grid, and the moving ultrasound is resampled
// for every transform; src/Interpolator/interpolator.cu:593-600,
// :1346-1352).
//
// The static image M, its Sobel magnitude G and their patch sums do not change
// with the transform, so the host precomputes them once per context
// (k_fixed_quant, k_box_line, k_fixed_centre in lc2_capi.cu):
//   q[2][nv]  M and G quantised per virtual voxel,
//   s[2][nv]  their window sums S_M and S_G,
//   d[3][nv]  the centred sums D_mm, D_gg, D_mg (D_xy = n S_xy - S_x S_y).
// Per transform one CTA owns a 32 x TY output tile and, in 3D, marches along
// z. Per entering slice it samples the ultrasound at its own halo points only
// (no Sobel of the warped image is needed), updates in registers the exact
// z-window sums of U, of the invalid-value count (a patch value <= 1e-6
// invalidates the patch, src/cu_LC2/cu_lc2_3d.cu:223-243) and of the
// products UU, UM, UG, and writes them as 8 int32 limbs; the x and y window
// passes give the patch sums, and each output voxel's weighting factor and
// measure come from solve_centred -- the generic kernel's solve. The
// weighting factor depends on the transform here, so the kernel accumulates
// both exact sums (measure and sigma) for k_finalize.
#pragma once

#include "lc2_fused.cuh"

namespace lc2 {

// Static precomputed fields of the high-resolution image, per virtual voxel.
struct FixedStatic {
  const int* q;        // quantised M, G: [2][nv]
  const int2* s;       // window sums (S_M, S_G) per voxel: [nv]
  const long long* d;  // centred sums D_mm, D_gg, D_mg: [3][nv]
  size_t nv;
  const float4* sv;    // solve factors (im, ig, rmg, 0) per voxel (solve_centred_static)
};

// Limbs: S_U, invalid count, then (lo, hi) of UU, UM and UG.
constexpr int kFixedLimbs = 8;

// Shared memory of one CTA: the leaving ring (3D: 2R+2 slices of
// (2 qU + invalid, qM, qG) per halo point), the limb planes, and in 3D the
// patch sums of the previous output slice (solved while the next slice's
// moments are formed).
template <int ND, int TY, int R>
struct FixedGeom {
  using G = FusedGeom<ND, TY, R>;
  static constexpr int RING = (ND == 3) ? 2 * R + 2 : 0;
  static constexpr size_t OFF_A = sizeof(int) * (size_t)RING * 3 * G::NP;
  static constexpr size_t OFF_Y = OFF_A + sizeof(int) * (size_t)kFixedLimbs * G::HY * G::HXP;
  static constexpr size_t BYTES =
      OFF_Y + ((ND == 3) ? sizeof(int) * (size_t)kFixedLimbs * TY * 32 : 0);
};

__device__ __forceinline__ void fixed_limbs(int* a, size_t pa, int su, int si, long long uu,
                                            long long um, long long ug, int K) {
  const unsigned long long mask = (1ull << K) - 1ull;
  a[0] = su;
  a[pa] = si;
  a[2 * pa] = (int)((unsigned long long)uu & mask);
  a[3 * pa] = (int)(uu >> K);
  a[4 * pa] = (int)((unsigned long long)um & mask);
  a[5 * pa] = (int)(um >> K);
  a[6 * pa] = (int)((unsigned long long)ug & mask);
  a[7 * pa] = (int)(ug >> K);
}

// Sigma and measure of output voxel gi from its patch sums (limb stride ls)
// and the static fields; adds both to the exact sums.
template <int ND, int R>
__device__ __forceinline__ void fixed_solve(const FusedParams& P, const FixedStatic& S,
                                            const int* a, int ls, size_t gi, long long& acc_m,
                                            long long& acc_s) {
  if (a[ls] != 0) return;  // a patch value <= 1e-6: sigma = 0
  const int su = a[0];
  constexpr int K = PatchConst<ND, R>::K;
  const long long uu = (long long)a[3 * ls] * (1LL << K) + a[2 * ls];
  const long long um = (long long)a[5 * ls] * (1LL << K) + a[4 * ls];
  const long long ug = (long long)a[7 * ls] * (1LL << K) + a[6 * ls];
  const int2 smg = __ldg(S.s + gi);
  const float4 sv = __ldg(S.sv + gi);
  constexpr long long n = PatchConst<ND, R>::N;
  float sigma, m;
  solve_centred_static(n * uu - (long long)su * su, n * um - (long long)su * smg.x,
                       n * ug - (long long)su * smg.y, sv, S.d, S.nv, gi, P.thr_var,
                       P.sig_scale, sigma, m);
  acc_m += __float2int_rn(m * P.sum_scale);
  acc_s += __float2int_rn(sigma * P.sum_scale);
}

__device__ __forceinline__ void fixed_flush(long long acc_m, long long acc_s,
                                            unsigned long long* acc) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    acc_m += __shfl_down_sync(0xffffffffu, acc_m, o);
    acc_s += __shfl_down_sync(0xffffffffu, acc_s, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (acc_m) atomicAdd(acc, (unsigned long long)acc_m);
    if (acc_s) atomicAdd(acc + 1, (unsigned long long)acc_s);
  }
}

// ---- 3D: z-marching over output slices [zb, ze) ----
// PRE: the warped ultrasound is read from a presampled buffer (k_presample,
// one float per virtual voxel and transform of the launch, slot-major)
// instead of being resampled by the CTA.
template <typename TM, int TY, int R, bool PRE = false>
__global__ void __launch_bounds__(32 * TY, fused_min_blocks(3, TY, R))
    k_fused_fixed3(const TM* __restrict__ mov, FixedStatic S, FusedParams P,
                   const Xform* __restrict__ xf, int k0, unsigned long long* __restrict__ acc,
                   const float* __restrict__ pre = nullptr) {
  using G = FusedGeom<3, TY, R>;
  using F = FixedGeom<3, TY, R>;
  constexpr int NT = G::NT, MAXP = G::MAXP, NL = kFixedLimbs;
  constexpr size_t PA = (size_t)G::HY * G::HXP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int* ring = reinterpret_cast<int*>(smem_raw);
  int* A = reinterpret_cast<int*>(smem_raw + F::OFF_A);
  int* Y = reinterpret_cast<int*>(smem_raw + F::OFF_Y);
  __shared__ Xform s_xf;
  __shared__ int s_ib[3];
  __shared__ float s_fb[3];
  __shared__ float s_A[9];
  __shared__ int s_inside;
  const int tid = threadIdx.x;
  const int slot = blockIdx.x;
  const int tile = blockIdx.y;
  const int x0 = (tile % P.ntx) * 32, y0 = P.y0 + (tile / P.ntx) * TY;
  const Xform* X = xf + k0 + slot;
  // sampling base (x0 - R - 1, 48 floor(y0 / 48) - R - 1), as in k_fused, so
  // 8- and 16-row tiles sample every voxel identically
  const int gx0 = x0 - R - 1, gy0 = y0 - R - 1;
  const int yb = y0 % kBand;
  const int ox = tid & 31, oy = tid >> 5;
  const int zb = blockIdx.z * P.zchunk;
  const int ze = min(zb + P.zchunk, P.vz);
  const int e0 = zb - R;  // first slice entering the window
  const size_t slice = (size_t)P.vx * P.vy;

  auto set_base = [&](int zs) {
    if (PRE) return;
    if (tid == NT - 1)
      s_inside = region_base<3, G::PW, G::PH>(s_xf, s_A, P, gx0, gy0, yb, zs,
                                              zs >= 0 && zs < P.vz, s_ib, s_fb)
                     ? 1 : 0;
  };
  if (tid == 0) {
    s_xf = *X;
#pragma unroll
    for (int i = 0; i < 9; ++i) s_A[i] = X->ah[i];
  }

  // this thread's halo points: in-grid flag, in-slice index, A offset and
  // region coordinates of the sampler
  int pu[MAXP], pa_off[MAXP], ppx[MAXP], ppy[MAXP];
  bool pin[MAXP];
  int sU[MAXP], sI[MAXP];
  long long sUU[MAXP], sUM[MAXP], sUG[MAXP];
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
    const int p = tid + j * NT;
    const int hy = p / G::HX, hx = p - hy * G::HX;
    const int gx = x0 - R + hx, gy = y0 - R + hy;
    pin[j] = (p < G::NP) && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy;
    pu[j] = pin[j] ? gy * P.vx + gx : 0;
    pa_off[j] = hy * G::HXP + hx;
    ppx[j] = hx + 1;
    ppy[j] = hy + 1 + yb;
    sU[j] = sI[j] = 0;
    sUU[j] = sUM[j] = sUG[j] = 0;
  }
  long long acc_m = 0, acc_s = 0;
  // static fields of the next output voxel solved, loaded a slice ahead
  int2 nsmg = make_int2(0, 0);
  float4 nsv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  auto load_static = [&](int z) {
    const int x = x0 + ox, y = y0 + oy;
    if (z >= zb && z < ze && x < P.vx && y < P.vy) {
      const size_t gi = ((size_t)z * P.vy + y) * P.vx + x;
      nsmg = __ldg(S.s + gi);
      nsv = __ldg(S.sv + gi);
    }
  };
  auto solve_out = [&](int z) {
    const int x = x0 + ox, y = y0 + oy;
    const int* a = Y + oy * 32 + ox;
    constexpr int ls = TY * 32;
    if (x < P.vx && y < P.vy && a[ls] == 0) {
      const int su = a[0];
      constexpr int K = PatchConst<3, R>::K;
      const long long uu = (long long)a[3 * ls] * (1LL << K) + a[2 * ls];
      const long long um = (long long)a[5 * ls] * (1LL << K) + a[4 * ls];
      const long long ug = (long long)a[7 * ls] * (1LL << K) + a[6 * ls];
      constexpr long long n = PatchConst<3, R>::N;
      const size_t gi = ((size_t)z * P.vy + y) * P.vx + x;
      float sigma, m;
      solve_centred_static(n * uu - (long long)su * su, n * um - (long long)su * nsmg.x,
                           n * ug - (long long)su * nsmg.y, nsv, S.d, S.nv, gi, P.thr_var,
                           P.sig_scale, sigma, m);
      acc_m += __float2int_rn(m * P.sum_scale);
      acc_s += __float2int_rn(sigma * P.sum_scale);
    }
  };

  __syncthreads();  // s_xf, s_A
  set_base(e0);
  __syncthreads();
  // Three phases per entering slice e, one barrier after each:
  //   1: solve output slice z-1 from Y; sample slice e, update the z-window
  //      sums and write the limbs;
  //   2: x window pass; sampling base of slice e+1;
  //   3: y window pass into Y.
  bool pending = false;  // Y holds the patch sums of output slice z-1
  int nqm[MAXP], nqg[MAXP];  // static qM, qG of the next entering slice
  float nu[PRE ? MAXP : 1];   // presampled ultrasound of the next entering slice
  const float* pre_slot = PRE ? pre + (size_t)slot * slice * P.vz : nullptr;
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
    nqm[j] = nqg[j] = 0;
    if constexpr (PRE) nu[j] = 0.0f;
    if (pin[j] && e0 >= 0 && e0 < P.vz) {
      const size_t gi = (size_t)e0 * slice + pu[j];
      nqm[j] = __ldg(S.q + gi);
      nqg[j] = __ldg(S.q + S.nv + gi);
      if constexpr (PRE) nu[j] = __ldcs(pre_slot + gi);
    }
  }
  for (int e = e0; e < ze + R; ++e) {
    const int z = e - R;          // output slice completed by this entering slice
    const int l = e - 2 * R - 1;  // slice leaving the window
    const bool out = (z >= zb);
    const bool leave = (l >= e0);
    const bool zin = (e >= 0 && e < P.vz);
    if (pending) solve_out(z - 1);
    load_static(z);
    int* rin = ring + ((e - e0) % F::RING) * 3 * G::NP;
    const int* rout = ring + ((l - e0 + F::RING) % F::RING) * 3 * G::NP;
    const bool inside = s_inside;
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const int p = tid + j * NT;
      if (p < G::NP) {
        float u = 0.0f;
        int qm = 0, qg = 0;
        if constexpr (PRE) {
          u = nu[j];
        } else if (inside) {
          u = fused_sample_inside<TM>(mov, P, s_A, s_ib, s_fb, ppx[j], ppy[j]);
        } else if (pin[j] && zin) {
          u = fused_sample<3, TM>(mov, P, s_A, s_ib, s_fb, ppx[j], ppy[j]);
        }
        qm = nqm[j];
        qg = nqg[j];
        const int qu = quant(u, P.qu), inv = (u > 1e-6f) ? 0 : 1;
        rin[p] = 2 * qu + inv;
        rin[G::NP + p] = qm;
        rin[2 * G::NP + p] = qg;
        sU[j] += qu;
        sI[j] += inv;
        sUU[j] += (long long)qu * qu;
        sUM[j] += (long long)qu * qm;
        sUG[j] += (long long)qu * qg;
        if (leave) {
          const int pl = rout[p], qml = rout[G::NP + p], qgl = rout[2 * G::NP + p];
          const int qul = pl >> 1;
          sU[j] -= qul;
          sI[j] -= pl & 1;
          sUU[j] -= (long long)qul * qul;
          sUM[j] -= (long long)qul * qml;
          sUG[j] -= (long long)qul * qgl;
        }
        if (out)
          fixed_limbs(A + pa_off[j], PA, sU[j], sI[j], sUU[j], sUM[j], sUG[j],
                      PatchConst<3, R>::K);
      }
    }
    {
      const bool zn = (e + 1 >= 0 && e + 1 < P.vz);
#pragma unroll
      for (int j = 0; j < MAXP; ++j) {
        nqm[j] = nqg[j] = 0;
        if constexpr (PRE) nu[j] = 0.0f;
        if (pin[j] && zn) {
          const size_t gi = (size_t)(e + 1) * slice + pu[j];
          nqm[j] = __ldg(S.q + gi);
          nqg[j] = __ldg(S.q + S.nv + gi);
          if constexpr (PRE) nu[j] = __ldcs(pre_slot + gi);
        }
      }
    }
    __syncthreads();
    if (out) fused_xpass<3, TY, R, NL>(A);
    set_base(e + 1);
    __syncthreads();
    if (out) fused_ypass<3, TY, R, NL>(A, Y, 32, TY * 32);
    pending = out;
    __syncthreads();
  }
  if (pending) solve_out(ze - 1);
  fixed_flush(acc_m, acc_s, acc + 2 * (size_t)(k0 + slot));
}

// ---- 3D on presampled ultrasound, 32 x 24 tiles (768 threads) ----
// k_fused_fixed3's arithmetic -- the same quantised fields, exact window
// sums, limbs and solve, so the same bits -- laid out for 24 warps per SM:
// warps along halo rows (halo_point), the window sums of the second halo
// point (threads < NS) in shared memory, the x pass in place on half rows
// and the y pass on half columns into Y (512 jobs each: this kernel waits on
// memory more than on its shared-memory pipe, and balanced passes cut its
// barrier waits), the solve of the previous slice from Y while the next
// slice's moments are formed. The leaving-slice ring (2 qU + invalid, qM,
// qG) is read before the entering slice overwrites its slot, so it holds
// 2R+1 slices. 2453 against 2395 evals/s for the 16-row kernel at 256^3.
template <int R>
struct FixedPtGeom {
  static constexpr int TY = 24;
  static constexpr int NT = 32 * TY;
  static constexpr int W = 2 * R + 1;
  static constexpr int HX = 32 + 2 * R, HY = TY + 2 * R;
  static constexpr int HXP = FusedGeom<3, TY, R>::HXP;
  static constexpr int NP = HX * HY;
  static constexpr int MAXP = (NP + NT - 1) / NT;
  static constexpr int NS = NP - NT;
  static constexpr int RING = 2 * R + 1;
  static constexpr size_t PA = (size_t)HY * HXP;
  static constexpr int XJOBS = kFixedLimbs * HY * 2;  // (limb, row, half)
  static constexpr int YJOBS = kFixedLimbs * 32 * 2;  // (limb, half, column)
  static constexpr size_t OFF_S = sizeof(int) * (size_t)RING * 3 * NP;
  static constexpr size_t OFF_A = OFF_S + (3 * sizeof(long long) + 2 * sizeof(int)) * (size_t)NS;
  static constexpr size_t OFF_Y = OFF_A + sizeof(int) * kFixedLimbs * PA;
  static constexpr size_t BYTES = OFF_Y + sizeof(int) * kFixedLimbs * TY * 32;
  static_assert(NS > 0 && NS <= NT, "two halo points per thread at most");
  static_assert(XJOBS <= NT && YJOBS <= NT && TY % 2 == 0, "one x job and one y job per thread");
  static_assert(OFF_A % 16 == 0 && HXP % 4 == 0 && 16 + 4 * ((16 + W - 1 + 3) / 4) <= HXP,
                "16-byte rows; loads of the second half row stay in the row");
  static_assert(R > 4 || BYTES + 1024 <= 227 * 1024, "one CTA's shared memory must fit an SM");
};

template <int R>
__global__ void __launch_bounds__(768, 1)
    k_fused_fixed_pt(FixedStatic S, FusedParams P, int k0, unsigned long long* __restrict__ acc,
                     const float* __restrict__ pre) {
  using G = FixedPtGeom<R>;
  constexpr int NT = G::NT, TY = G::TY, MAXP = G::MAXP;
  constexpr size_t PA = G::PA;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int* ring = reinterpret_cast<int*>(smem_raw);
  long long* sp = reinterpret_cast<long long*>(smem_raw + G::OFF_S);  // UU, UM, UG
  int* sq = reinterpret_cast<int*>(sp + 3 * G::NS);                    // S_U, invalid count
  int* A = reinterpret_cast<int*>(smem_raw + G::OFF_A);
  int* Y = reinterpret_cast<int*>(smem_raw + G::OFF_Y);
  const int tid = threadIdx.x, slot = blockIdx.x, tile = blockIdx.y;
  const int x0 = (tile % P.ntx) * 32, y0 = P.y0 + (tile / P.ntx) * TY;
  const int ox = tid & 31, oy = tid >> 5;
  const int zb = blockIdx.z * P.zchunk;
  const int ze = min(zb + P.zchunk, P.vz);
  const int e0 = zb - R;
  const size_t slice = (size_t)P.vx * P.vy;
  const float* pre_slot = pre + (size_t)slot * slice * P.vz;
  // the thread's halo points: offset in a slice (-1 outside the grid) and
  // index in the limb planes
  int po[MAXP], pa[MAXP];
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
    const int p = tid + j * NT;
    int hy, hx;
    halo_point<TY, R>(p, hy, hx);
    const int gx = x0 - R + hx, gy = y0 - R + hy;
    po[j] = (p < G::NP && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy) ? gy * P.vx + gx : -1;
    pa[j] = hy * G::HXP + hx;
  }
  int aU = 0, aI = 0;
  long long aUU = 0, aUM = 0, aUG = 0;
  if (tid < G::NS) {
#pragma unroll
    for (int k = 0; k < 3; ++k) sp[k * G::NS + tid] = 0;
    sq[tid] = 0;
    sq[G::NS + tid] = 0;
  }
  long long acc_m = 0, acc_s = 0;
  // static fields of the next output voxel solved, loaded a slice ahead
  int2 nsmg = make_int2(0, 0);
  float4 nsv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  auto load_static = [&](int z) {
    const int x = x0 + ox, y = y0 + oy;
    if (z >= zb && z < ze && x < P.vx && y < P.vy) {
      const size_t gi = ((size_t)z * P.vy + y) * P.vx + x;
      nsmg = __ldg(S.s + gi);
      nsv = __ldg(S.sv + gi);
    }
  };
  auto solve_out = [&](int z, int2 smg, float4 sv) {
    const int x = x0 + ox, y = y0 + oy;
    const int* a = Y + oy * 32 + ox;
    constexpr int ls = TY * 32;
    if (x < P.vx && y < P.vy && a[ls] == 0) {
      const int su = a[0];
      constexpr int K = PatchConst<3, R>::K;
      const long long uu = (long long)a[3 * ls] * (1LL << K) + a[2 * ls];
      const long long um = (long long)a[5 * ls] * (1LL << K) + a[4 * ls];
      const long long ug = (long long)a[7 * ls] * (1LL << K) + a[6 * ls];
      constexpr long long n = PatchConst<3, R>::N;
      const size_t gi = ((size_t)z * P.vy + y) * P.vx + x;
      float sigma, m;
      solve_centred_static(n * uu - (long long)su * su, n * um - (long long)su * smg.x,
                           n * ug - (long long)su * smg.y, sv, S.d, S.nv, gi, P.thr_var,
                           P.sig_scale, sigma, m);
      acc_m += __float2int_rn(m * P.sum_scale);
      acc_s += __float2int_rn(sigma * P.sum_scale);
    }
  };
  // presampled ultrasound and static qM, qG of the entering slice, loaded a
  // slice ahead
  float nu[MAXP];
  int nqm[MAXP], nqg[MAXP];
  auto load_halo = [&](int e) {
    const bool zin = (e >= 0 && e < P.vz);
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      nu[j] = 0.0f;
      nqm[j] = nqg[j] = 0;
      if (zin && po[j] >= 0) {
        const size_t gi = (size_t)e * slice + po[j];
        nqm[j] = __ldg(S.q + gi);
        nqg[j] = __ldg(S.q + S.nv + gi);
        nu[j] = __ldcs(pre_slot + gi);
      }
    }
  };
  load_halo(e0);
  bool pending = false;  // Y holds the patch sums of output slice z-1
  for (int e = e0; e < ze + R; ++e) {
    const int z = e - R;
    const int l = e - 2 * R - 1;
    const bool out = (z >= zb);
    const bool leave = (l >= e0);
    if (pending) solve_out(z - 1, nsmg, nsv);
    load_static(z);
    int* rg = ring + ((e - e0) % G::RING) * 3 * G::NP;  // the leaving slice's slot
    auto point = [&](int j, int& sU, int& sI, long long& sUU, long long& sUM, long long& sUG) {
      const int p = tid + j * NT;
      const float u = nu[j];
      const int qm = nqm[j], qg = nqg[j];
      const int qu = quant(u, P.qu), inv = (u > 1e-6f) ? 0 : 1;
      if (leave) {
        const int pl = rg[p], qml = rg[G::NP + p], qgl = rg[2 * G::NP + p];
        const int qul = pl >> 1;
        sU -= qul;
        sI -= pl & 1;
        sUU -= (long long)qul * qul;
        sUM -= (long long)qul * qml;
        sUG -= (long long)qul * qgl;
      }
      rg[p] = 2 * qu + inv;
      rg[G::NP + p] = qm;
      rg[2 * G::NP + p] = qg;
      sU += qu;
      sI += inv;
      sUU += (long long)qu * qu;
      sUM += (long long)qu * qm;
      sUG += (long long)qu * qg;
      if (out) fixed_limbs(A + pa[j], PA, sU, sI, sUU, sUM, sUG, PatchConst<3, R>::K);
    };
    point(0, aU, aI, aUU, aUM, aUG);
    if (tid < G::NS) {
      int sU = sq[tid], sI = sq[G::NS + tid];
      long long sUU = sp[tid], sUM = sp[G::NS + tid], sUG = sp[2 * G::NS + tid];
      point(1, sU, sI, sUU, sUM, sUG);
      sq[tid] = sU;
      sq[G::NS + tid] = sI;
      sp[tid] = sUU;
      sp[G::NS + tid] = sUM;
      sp[2 * G::NS + tid] = sUG;
    }
    load_halo(e + 1);
    __syncthreads();
    if (out) {  // x pass in place on half rows; the two halves of a row on neighbouring lanes
      constexpr int NV = (16 + G::W - 1 + 3) / 4;
      const int it = tid;
      const bool act = it < G::XJOBS;
      const int hq = it & 1;
      int* row = A + (size_t)(act ? it >> 1 : 0) * G::HXP + 16 * hq;
      int v[4 * NV];
      if (act) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
          const int4 cc = reinterpret_cast<const int4*>(row)[i];
          v[4 * i] = cc.x;
          v[4 * i + 1] = cc.y;
          v[4 * i + 2] = cc.z;
          v[4 * i + 3] = cc.w;
        }
      }
      __syncwarp();
      if (act) {
        int a = 0;
#pragma unroll
        for (int i = 0; i < G::W; ++i) a += v[i];
        int o[4];
        o[0] = a;
#pragma unroll
        for (int x = 1; x < 16; ++x) {
          a += v[x + G::W - 1] - v[x - 1];
          o[x & 3] = a;
          if ((x & 3) == 3) reinterpret_cast<int4*>(row)[x >> 2] = make_int4(o[0], o[1], o[2], o[3]);
        }
      }
      __syncwarp();
    }
    __syncthreads();
    if (out) {
      const int it = tid;
      if (it < G::YJOBS) {  // y pass on half columns into Y
        constexpr int H = TY / 2;
        const int Lb = it >> 6, h = (it >> 5) & 1, col = it & 31;
        const int* c = A + (size_t)Lb * PA + (size_t)(h * H) * G::HXP + col;
        int* o = Y + (size_t)Lb * TY * 32 + (h * H) * 32 + col;
        int v[H + G::W - 1];
#pragma unroll
        for (int i = 0; i < H + G::W - 1; ++i) v[i] = c[i * G::HXP];
        int a = 0;
#pragma unroll
        for (int i = 0; i < G::W; ++i) a += v[i];
        o[0] = a;
#pragma unroll
        for (int y = 1; y < H; ++y) {
          a += v[y + G::W - 1] - v[y - 1];
          o[y * 32] = a;
        }
      }
    }
    pending = out;
    __syncthreads();
  }
  if (pending) solve_out(ze - 1, nsmg, nsv);
  fixed_flush(acc_m, acc_s, acc + 2 * (size_t)(k0 + slot));
}

// ---- 2D and 2D-to-3D: one 32 x 16 tile per CTA ----
// Three CTAs per SM (42 registers): the solve's 64-bit work spills at the
// 32 registers of four.
template <int WND, typename TM, int R>
__global__ void __launch_bounds__(512, 3)
    k_fused_fixed2(const TM* __restrict__ mov, FixedStatic S, FusedParams P,
                   const Xform* __restrict__ xf, int k0, unsigned long long* __restrict__ acc) {
  constexpr int TY = 16;
  using G = FusedGeom<2, TY, R>;
  constexpr int NT = G::NT, NL = kFixedLimbs;
  constexpr size_t PA = (size_t)G::HY * G::HXP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int* A = reinterpret_cast<int*>(smem_raw + FixedGeom<2, TY, R>::OFF_A);
  __shared__ TileShared T;
  const int tid = threadIdx.x;
  const int slot = blockIdx.x;
  const int tile = blockIdx.y;
  const Xform* X = xf + k0 + slot;
  const int x0 = (tile % P.ntx) * 32, y0 = (tile / P.ntx) * TY;
  const int gx0 = x0 - R - 1, gy0 = y0 - R - 1;
  if (tid == 0) {
#pragma unroll
    for (int i = 0; i < 9; ++i) T.A[i] = X->ah[i];
    T.inside = region_base<WND, G::PW, G::PH>(*X, T.A, P, gx0, gy0, 0, 0, true, T.ib, T.fb) ? 1 : 0;
  }
  __syncthreads();
  const bool inside = T.inside;
  for (int p = tid; p < G::NP; p += NT) {
    int hy, hx;
    halo_coord<G::HX, G::HY>(p, hy, hx);
    const int gx = x0 - R + hx, gy = y0 - R + hy;
    const bool pin = gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy;
    float u = 0.0f;
    int qm = 0, qg = 0;
    if (inside) {
      if constexpr (WND == 3)
        u = fused_sample_inside<TM>(mov, P, T.A, T.ib, T.fb, hx + 1, hy + 1);
      else
        u = fused_sample_inside2<TM>(mov, P, T.A, T.ib, T.fb, hx + 1, hy + 1);
    } else if (pin) {
      u = fused_sample<WND, TM>(mov, P, T.A, T.ib, T.fb, hx + 1, hy + 1);
    }
    if (pin) {
      const size_t gi = (size_t)gy * P.vx + gx;
      qm = __ldg(S.q + gi);
      qg = __ldg(S.q + S.nv + gi);
    }
    const int qu = quant(u, P.qu);
    fixed_limbs(A + hy * G::HXP + hx, PA, qu, (u > 1e-6f) ? 0 : 1, (long long)qu * qu,
                (long long)qu * qm, (long long)qu * qg, PatchConst<2, R>::K);
  }
  __syncthreads();
  fused_xy<2, TY, R, 0, NL>(A);
  long long acc_m = 0, acc_s = 0;
  const int ox = tid & 31, oy = tid >> 5;
  const int x = x0 + ox, y = y0 + oy;
  if (x < P.vx && y < P.vy)
    fixed_solve<2, R>(P, S, A + oy * G::HXP + ox, (int)PA, (size_t)y * P.vx + x, acc_m,
                      acc_s);
  fixed_flush(acc_m, acc_s, acc + 2 * (size_t)(k0 + slot));
}

struct FixedLaunch {
  const void* mov;
  FixedStatic S;
  FusedParams P;
  const Xform* xf;
  int k0, cnt;
  unsigned long long* acc;
  int nd, wnd;
  int tile_height;  // 3D, radius <= 4: 16, 8 or (presampled) 24 rows per tile
  int zchunk;       // 3D: output slices per CTA; 0 = automatic
  int sms;          // multiprocessors of the device
  cudaStream_t stream;
  const float* pre = nullptr;  // 3D: presampled ultrasound of the launch (k_presample)
  // 3D presampled: the launch's tiles cover output rows [y_off, y_off +
  // y_rows) (y_rows 0: the whole grid)
  int y_off = 0, y_rows = 0;
};

template <typename T, int R, int TY, typename K>
cudaError_t fixed_launch3_k(const FixedLaunch& L, K kern);

template <typename T, int R, int TY>
cudaError_t fixed_launch3(const FixedLaunch& L) {
  if (L.P.kbits != PatchConst<3, R>::K || L.P.n != PatchConst<3, R>::N)
    return cudaErrorInvalidValue;
  if (L.pre) return fixed_launch3_k<T, R, TY>(L, k_fused_fixed3<T, TY, R, true>);
  return fixed_launch3_k<T, R, TY>(L, k_fused_fixed3<T, TY, R, false>);
}

template <typename T, int R, int TY, typename K>
cudaError_t fixed_launch3_k(const FixedLaunch& L, K kern) {
  using F = FixedGeom<3, TY, R>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)F::BYTES);
  if (e != cudaSuccess) return e;
  FusedParams P = L.P;
  const int rows = L.y_rows > 0 ? L.y_rows : P.vy;
  const int ntx = (P.vx + 31) / 32, nty = (rows + TY - 1) / TY;
  P.ntx = ntx;
  P.y0 = L.y_off;
  if (L.zchunk > 0)
    P.zchunk = L.zchunk < P.vz ? L.zchunk : P.vz;
  else
    P.zchunk = auto_zchunk(P.vz, R, (long long)ntx * nty * L.cnt,
                           (long long)L.sms * fused_min_blocks(3, TY, R));
  const int nz = (P.vz + P.zchunk - 1) / P.zchunk;
  dim3 grid(L.cnt, ntx * nty, nz);
  kern<<<grid, 32 * TY, F::BYTES, L.stream>>>((const T*)L.mov, L.S, P, L.xf, L.k0, L.acc,
                                               L.pre);
  return cudaGetLastError();
}

// k_fused_fixed_pt over the launch's rows (presampled ultrasound, radius <= 4).
template <int R>
cudaError_t fixed_pt_launch(const FixedLaunch& L) {
  using G = FixedPtGeom<R>;
  if (L.P.kbits != PatchConst<3, R>::K || L.P.n != PatchConst<3, R>::N || !L.pre)
    return cudaErrorInvalidValue;
  auto kern = k_fused_fixed_pt<R>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)G::BYTES);
  if (e != cudaSuccess) return e;
  FusedParams P = L.P;
  const int rows = L.y_rows > 0 ? L.y_rows : P.vy;
  const int ntx = (P.vx + 31) / 32, nty = (rows + G::TY - 1) / G::TY;
  P.ntx = ntx;
  P.y0 = L.y_off;
  if (L.zchunk > 0)
    P.zchunk = L.zchunk < P.vz ? L.zchunk : P.vz;
  else
    P.zchunk = auto_zchunk(P.vz, R, (long long)ntx * nty * L.cnt, (long long)L.sms);
  const int nz = (P.vz + P.zchunk - 1) / P.zchunk;
  dim3 grid(L.cnt, ntx * nty, nz);
  kern<<<grid, G::NT, G::BYTES, L.stream>>>(L.S, P, L.k0, L.acc, L.pre);
  return cudaGetLastError();
}

template <typename T, int R>
cudaError_t fixed_launch2(const FixedLaunch& L) {
  using F = FixedGeom<2, 16, R>;
  if (L.P.kbits != PatchConst<2, R>::K || L.P.n != PatchConst<2, R>::N)
    return cudaErrorInvalidValue;
  FusedParams P = L.P;
  P.ntx = (P.vx + 31) / 32;
  const int nty = (P.vy + 15) / 16;
  dim3 grid(L.cnt, P.ntx * nty, 1);
  if (L.wnd == 3) {
    auto kern = k_fused_fixed2<3, T, R>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)F::BYTES);
    if (e != cudaSuccess) return e;
    kern<<<grid, 512, F::BYTES, L.stream>>>((const T*)L.mov, L.S, P, L.xf, L.k0, L.acc);
  } else {
    auto kern = k_fused_fixed2<2, T, R>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)F::BYTES);
    if (e != cudaSuccess) return e;
    kern<<<grid, 512, F::BYTES, L.stream>>>((const T*)L.mov, L.S, P, L.xf, L.k0, L.acc);
  }
  return cudaGetLastError();
}

// Tile heights as for k_fused: 16 rows (8 or, on presampled ultrasound, 24
// on request) up to radius 4, 8 rows beyond.
template <typename T, int R>
cudaError_t fixed_launch_r(const FixedLaunch& L) {
  if (L.nd == 2) return fixed_launch2<T, R>(L);
  if constexpr (R <= 6) {
    if constexpr (R > 4) {
      return fixed_launch3<T, R, 8>(L);
    } else {
      if (L.tile_height == 8) return fixed_launch3<T, R, 8>(L);
      if (L.tile_height == 24 && L.pre) return fixed_pt_launch<R>(L);
      return fixed_launch3<T, R, 16>(L);
    }
  }
  return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t fixed_launch_t(const FixedLaunch& L) {
  switch (L.P.r) {
    case 1: return fixed_launch_r<T, 1>(L);
    case 2: return fixed_launch_r<T, 2>(L);
    case 3: return fixed_launch_r<T, 3>(L);
    case 4: return fixed_launch_r<T, 4>(L);
    case 5: return fixed_launch_r<T, 5>(L);
    case 6: return fixed_launch_r<T, 6>(L);
  }
  if (L.nd == 2) {
    switch (L.P.r) {
      case 7: return fixed_launch2<T, 7>(L);
      case 8: return fixed_launch2<T, 8>(L);
      case 9: return fixed_launch2<T, 9>(L);
      case 10: return fixed_launch2<T, 10>(L);
      case 11: return fixed_launch2<T, 11>(L);
      case 12: return fixed_launch2<T, 12>(L);
    }
  }
  return cudaErrorInvalidValue;
}

// Defined per storage type in lc2_fixed_{f32,f16,bf16}.cu.
template <typename T>
cudaError_t fixed_launch(const FixedLaunch& L);

template <>
cudaError_t fixed_launch<float>(const FixedLaunch& L);
template <>
cudaError_t fixed_launch<__half>(const FixedLaunch& L);
template <>
cudaError_t fixed_launch<__nv_bfloat16>(const FixedLaunch& L);

#define LC2_DEFINE_FIXED_LAUNCH(T)                      \
  template <>                                           \
  cudaError_t fixed_launch<T>(const FixedLaunch& L) {   \
    return fixed_launch_t<T>(L);                        \
  }

}  // namespace lc2
