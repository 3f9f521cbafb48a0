// lc2_fused_ps.cuh -- the fused 3D moments pass on presampled images.
#pragma once

#include "lc2_fused.cuh"

namespace lc2 {

// The moments pass on presampled images (LC2_OPTION_PRESAMPLE = 1, the
// default for 3D contexts of a resampled MR/CT): k_fused's z-marching
// moments, window sums and solve, reading M of each entering slice from the
// buffer k_presample wrote. The Sobel magnitude of the entering slice comes
// from its (M, (Sz, Dz)) planes in shared memory, as in k_fused. The planes of
// slice e+1 are written while the x pass of slice e runs -- its threads are
// otherwise half idle -- and the limb planes are double-buffered, so a slice
// costs three barriers: after the limb writes (the planes of e have been
// read), after the x pass and plane writes, after the y pass; the solve of
// slice z overlaps the limb writes of slice z+1. Values equal k_fused's on the
// same presampled images bit for bit.
constexpr int kPsTY = 16;

template <int R>
struct PsGeom {
  static constexpr int TY = kPsTY;
  static constexpr int NT = 32 * TY;
  static constexpr int HX = 32 + 2 * R, HY = TY + 2 * R;
  static constexpr int HXP = FusedGeom<3, TY, R>::HXP;
  static constexpr int NP = HX * HY;
  static constexpr int MAXP = (NP + NT - 1) / NT;
  static constexpr int RING = 2 * R + 1;          // leaving qM, qG, qU of the z window
  static constexpr size_t PA = (size_t)HY * HXP;  // ints per limb plane
  static constexpr int PW = 32 + 2 * R + 2, PH = TY + 2 * R + 2;  // resampled region
  static constexpr int NPW = PW * PH;                              // even: float2 plane aligned
  static constexpr int WP = (NPW + NT - 1) / NT;
  static constexpr size_t OFF_LV = ((sizeof(float) * 3 * (size_t)NPW + 15) / 16) * 16;
  static constexpr size_t OFF_A = OFF_LV + sizeof(int) * (size_t)RING * 3 * NP;
  static constexpr size_t BYTES = OFF_A + 2 * sizeof(int) * kLimbs * PA;
  static_assert(NPW % 2 == 0, "the (Sz, Dz) plane follows the M plane");
  static_assert(R > 4 || BYTES + 1024 <= 227 * 1024, "one CTA's shared memory must fit an SM");
};

template <typename TS, int R>
__global__ void __launch_bounds__(32 * kPsTY, 1)
    k_fused_ps(const float* __restrict__ Mb, const TS* __restrict__ Ust,
               const float* __restrict__ sig, const int* __restrict__ su, FusedParams P, int k0,
               unsigned long long* __restrict__ acc, float* __restrict__ out_measure) {
  using G = PsGeom<R>;
  constexpr int NT = G::NT, TY = G::TY, MAXP = G::MAXP, WP = G::WP;
  constexpr int KB = PatchConst<3, R>::K;
  constexpr unsigned long long kmask = (1ull << KB) - 1ull;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* mc = reinterpret_cast<float*>(smem_raw);
  float2* SD = reinterpret_cast<float2*>(mc + G::NPW);
  int* lv = reinterpret_cast<int*>(smem_raw + G::OFF_LV);
  int* A0 = reinterpret_cast<int*>(smem_raw + G::OFF_A);
  const int tid = threadIdx.x, slot = blockIdx.x, tile = blockIdx.y;
  const int x0 = (tile % P.ntx) * 32, y0 = (tile / P.ntx) * TY;
  const int ox = tid & 31, oy = tid >> 5;
  const int zb = blockIdx.z * P.zchunk;
  const int ze = min(zb + P.zchunk, P.vz);
  const size_t slice = (size_t)P.vx * P.vy;
  const float* Ms = Mb + (size_t)slot * slice * P.vz;
  // the thread's region points (planes) and halo points (moments)
  int roff[WP];
#pragma unroll
  for (int k = 0; k < WP; ++k) {
    const int i = tid + k * NT;
    const int py = i / G::PW, px = i - py * G::PW;
    const int gx = x0 - R - 1 + px, gy = y0 - R - 1 + py;
    roff[k] = (i < G::NPW && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy) ? gy * P.vx + gx : -1;
  }
  int pc[MAXP], pu[MAXP], pa_off[MAXP];
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
    const int p = tid + j * NT;
    const int hy = p / G::HX, hx = p - hy * G::HX;
    const int gx = x0 - R + hx, gy = y0 - R + hy;
    pc[j] = (hy + 1) * G::PW + hx + 1;
    pa_off[j] = hy * G::HXP + hx;
    pu[j] = (p < G::NP && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy) ? gy * P.vx + gx : -1;
  }
  int accq[MAXP][2];
  long long accp[MAXP][5];
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
    accq[j][0] = accq[j][1] = 0;
#pragma unroll
    for (int k = 0; k < 5; ++k) accp[j][k] = 0;
  }
  const int e0 = zb - R;
  auto load_m = [&](int e, float* out) {
    const bool zin = (e >= 0 && e < P.vz);
    const float* src = Ms + (size_t)(zin ? e : 0) * slice;
#pragma unroll
    for (int k = 0; k < WP; ++k) out[k] = (zin && roff[k] >= 0) ? __ldcs(src + roff[k]) : 0.0f;
  };
  // region values of slices e, e+1, e+2 (the last loaded an iteration ahead)
  float r0[WP], r1[WP], r2[WP];
  // planes of slice e from M(e-1), M(e), M(e+1)
  auto write_planes = [&](const float* a, const float* b, const float* c) {
#pragma unroll
    for (int k = 0; k < WP; ++k) {
      const int i = tid + k * NT;
      if (i < G::NPW) {
        mc[i] = b[k];
        SD[i] = make_float2(a[k] + 2.0f * b[k] + c[k], c[k] - a[k]);
      }
    }
  };
  float u_nx[MAXP];
  auto load_u = [&](int e) {
    const bool zin = (e >= 0 && e < P.vz);
#pragma unroll
    for (int j = 0; j < MAXP; ++j)
      u_nx[j] = (zin && pu[j] >= 0) ? ldf(Ust, (size_t)e * slice + pu[j]) : 0.0f;
  };
  float sg_nx = 0.0f;
  int sv_nx = 0;
  auto load_sig = [&](int z) {
    const int x = x0 + ox, y = y0 + oy;
    sg_nx = 0.0f;
    sv_nx = 0;
    if (z >= zb && z < ze && x < P.vx && y < P.vy) {
      const size_t gi = (size_t)z * slice + (size_t)y * P.vx + x;
      sg_nx = __ldg(sig + gi);
      sv_nx = __ldg(su + gi);
    }
  };
  {
    float m_a[WP];
    load_m(e0 - 1, m_a);
    load_m(e0, r0);
    load_m(e0 + 1, r1);
    write_planes(m_a, r0, r1);
    load_m(e0 + 2, r2);
  }
  load_u(e0);
  load_sig(e0 - R);
  __syncthreads();
  long long acc_m = 0;
  int buf = 0;
  for (int e = e0; e < ze + R; ++e) {
    // ---- the entering slice's fields from planes(e): ring, z-window, limbs ----
    float u_in[MAXP];
#pragma unroll
    for (int j = 0; j < MAXP; ++j) u_in[j] = u_nx[j];
    load_u(e + 1);
    const int z = e - R;
    const float sg = sg_nx;
    const int sv = sv_nx;
    load_sig(z + 1);
    const int l = e - 2 * R - 1;
    const bool out = (z >= zb);
    const bool leave = (l >= e0);
    int* A = A0 + (size_t)buf * kLimbs * G::PA;
    int* lv_in = lv + ((e - e0) % G::RING) * 3 * G::NP;
    const int* lv_out = lv + ((l - e0 + G::RING) % G::RING) * 3 * G::NP;
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const int p = tid + j * NT;
      if (p < G::NP) {
        const float m = mc[pc[j]];
        const float g = fused_sobel_sd<G::PW>(SD, pc[j]);
        const int qm = quant(m, P.qm), qg = quant(g, P.qg), qu = quant(u_in[j], P.qu);
        if (leave) {
          const int qml = lv_out[p], qgl = lv_out[G::NP + p], qul = lv_out[2 * G::NP + p];
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
        lv_in[2 * G::NP + p] = qu;
        accp[j][0] += (long long)qu * qm;
        accp[j][1] += (long long)qu * qg;
        accp[j][2] += (long long)qm * qm;
        accp[j][3] += (long long)qg * qg;
        accp[j][4] += (long long)qm * qg;
        accq[j][0] += qm;
        accq[j][1] += qg;
        if (out) {
          int* a = A + pa_off[j];
          a[0] = accq[j][0];
          a[G::PA] = accq[j][1];
#pragma unroll
          for (int k = 0; k < 5; ++k) {
            a[(2 + 2 * k) * G::PA] = (int)((unsigned long long)accp[j][k] & kmask);
            a[(3 + 2 * k) * G::PA] = (int)(accp[j][k] >> KB);
          }
        }
      }
    }
    __syncthreads();  // planes(e) read, limbs written
    // ---- x pass of slice e; planes of slice e+1 ----
    if (out) fused_xpass<3, TY, R>(A);
    write_planes(r0, r1, r2);  // M(e), M(e+1), M(e+2)
#pragma unroll
    for (int k = 0; k < WP; ++k) {
      r0[k] = r1[k];
      r1[k] = r2[k];
    }
    load_m(e + 3, r2);
    __syncthreads();
    if (out) {
      fused_ypass<3, TY, R>(A, A, G::HXP, G::HY * G::HXP);
      __syncthreads();
      const int x = x0 + ox, y = y0 + oy;
      if (x < P.vx && y < P.vy) {
        float m = 0.0f;
        if (sg > 0.0f) {
          const int* a = A + oy * G::HXP + ox;
          int L[kLimbs];
#pragma unroll
          for (int k = 0; k < kLimbs; ++k) L[k] = a[k * G::PA];
          m = fused_measure<3, R>(P, sg, sv, L);
          acc_m += __float2int_rn(m * P.sum_scale);
        }
        if (out_measure && slot == 0) out_measure[(size_t)z * slice + (size_t)y * P.vx + x] = m;
      }
      buf ^= 1;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc_m += __shfl_down_sync(0xffffffffu, acc_m, o);
  if ((tid & 31) == 0) atomicAdd(acc + 2 * (size_t)(k0 + slot), (unsigned long long)acc_m);
}

template <typename T, int R>
cudaError_t fused_ps_launch_r(const FusedLaunch& L, const float* M) {
  using G = PsGeom<R>;
  if (L.P.kbits != PatchConst<3, R>::K || L.P.n != PatchConst<3, R>::N)
    return cudaErrorInvalidValue;
  auto kern = k_fused_ps<T, R>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)G::BYTES);
  if (e != cudaSuccess) return e;
  FusedParams P = L.P;
  const int ntx = (P.vx + 31) / 32, nty = (P.vy + G::TY - 1) / G::TY;
  P.ntx = ntx;
  if (L.zchunk > 0)
    P.zchunk = L.zchunk < P.vz ? L.zchunk : P.vz;
  else
    P.zchunk = auto_zchunk(P.vz, R, (long long)ntx * nty * L.cnt, (long long)L.sms);
  const int nz = (P.vz + P.zchunk - 1) / P.zchunk;
  dim3 grid(L.cnt, ntx * nty, nz);
  kern<<<grid, G::NT, G::BYTES, L.stream>>>(M, (const T*)L.ust, L.sig, L.su, P, L.k0, L.acc,
                                            L.out_measure);
  return cudaGetLastError();
}

// Patch radius 1..4 (shared memory holds two limb buffers up to radius 4).
template <typename T>
cudaError_t fused_ps_launch(const FusedLaunch& L, const float* M) {
  switch (L.P.r) {
    case 1: return fused_ps_launch_r<T, 1>(L, M);
    case 2: return fused_ps_launch_r<T, 2>(L, M);
    case 3: return fused_ps_launch_r<T, 3>(L, M);
    case 4: return fused_ps_launch_r<T, 4>(L, M);
  }
  return cudaErrorInvalidValue;
}

// Defined per storage type in lc2_ps_{f32,f16,bf16}.cu.
template <typename T>
cudaError_t fused_ps_entry(const FusedLaunch& L, const float* M);
template <>
cudaError_t fused_ps_entry<float>(const FusedLaunch& L, const float* M);
template <>
cudaError_t fused_ps_entry<__half>(const FusedLaunch& L, const float* M);
template <>
cudaError_t fused_ps_entry<__nv_bfloat16>(const FusedLaunch& L, const float* M);

#define LC2_DEFINE_FUSED_PS(T)                                              \
  template <>                                                               \
  cudaError_t fused_ps_entry<T>(const FusedLaunch& L, const float* M) {     \
    return fused_ps_launch<T>(L, M);                                        \
  }

}  // namespace lc2
