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
  const int x0 = (tile % P.ntx) * 32, y0 = P.y0 + (tile / P.ntx) * TY;
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
  kern<<<grid, G::NT, G::BYTES, L.stream>>>(M, (const T*)L.ust, L.sig, L.su, P, L.k0, L.acc,
                                            L.out_measure);
  return cudaGetLastError();
}

// Tall tiles: the same moments pass over 32 x 24 outputs with 768 threads,
// 24 warps per SM instead of 16. Shared memory keeps only qG of the leaving
// slice in the z ring; qM and qU of the leaving slice are the quantised
// values of the same presampled and ultrasound voxels read again (from L2:
// the slice entered 2R+1 slices earlier), so the window holds the same
// integers. The x window pass runs in place on quarter rows (two jobs per
// thread), the y pass on whole columns from the limb planes into a buffer of
// its own, which the solve reads: one limb buffer suffices (the next slice's
// limbs are written after every thread's y pass). 80 registers, no spills.
constexpr int kPtTY = 24;

template <int R>
struct PtGeom {
  static constexpr int TY = kPtTY;
  static constexpr int NT = 32 * TY;
  static constexpr int W = 2 * R + 1;
  static constexpr int HX = 32 + 2 * R, HY = TY + 2 * R;
  static constexpr int HXP = FusedGeom<3, TY, R>::HXP;
  static constexpr int NP = HX * HY;
  static constexpr int MAXP = (NP + NT - 1) / NT;
  static constexpr int RING = 2 * R + 1;          // leaving qG of the z window
  static constexpr size_t PA = (size_t)HY * HXP;  // ints per limb plane
  static constexpr int PW = HX + 2, PH = HY + 2;  // presampled region with the Sobel margin
  // plane row pitch = 4 mod 8 words: the 8 x 4 tail blocks of halo points
  // (rows two apart) read the float2 (Sz, Dz) plane without bank conflicts;
  // the planes are written row by row over the full pitch (the PWP - PW
  // padding columns hold zeros and are never read)
  static constexpr int PWP = PW + (12 - PW % 8) % 8;
  static constexpr int NPW = PWP * PH;
  static constexpr int WP = (NPW + NT - 1) / NT;
  static constexpr int XJOBS = kLimbs * HY * 4;   // (limb, row, quarter) of the x pass
  static constexpr int YJOBS = kLimbs * 32;       // (limb, column) of the y pass
  static constexpr size_t OFF_LV = ((sizeof(float) * 3 * (size_t)NPW + 15) / 16) * 16;
  // z-window sums of the halo points beyond the first NT (the second point
  // of threads < NS) live in shared memory: 5 products, then qM and qG
  static constexpr int NS = NP - NT;
  static constexpr size_t OFF_S = OFF_LV + sizeof(int) * (size_t)RING * NP;
  static constexpr size_t OFF_A = OFF_S + (sizeof(long long) * 5 + sizeof(int) * 2) * (size_t)NS;
  static constexpr size_t OFF_Y = OFF_A + sizeof(int) * kLimbs * PA;
  static constexpr size_t BYTES = OFF_Y + sizeof(int) * kLimbs * TY * 32;
  static_assert(NPW % 2 == 0 && PWP % 8 == 4, "the (Sz, Dz) plane follows the M plane");
  static_assert(NS > 0 && NS <= NT, "two halo points per thread at most");
  static_assert(XJOBS <= 2 * NT && YJOBS <= NT, "two x jobs and one y job per thread at most");
  static_assert(TY % 4 == 0, "four row quarters");
  static_assert(HXP % 4 == 0 && 24 + 4 * ((8 + W - 1 + 3) / 4) <= HXP,
                "16-byte loads of the last quarter row stay in the row");
  static_assert(R > 4 || BYTES + 1024 <= 227 * 1024, "one CTA's shared memory must fit an SM");
};

// x window pass in place on quarter rows: job (limb, row, quarter), the
// four quarters of a row on neighbouring lanes of one warp, which all load
// before any stores (quarter q reads columns 8q..8q+7+2R, of which the next
// quarter overwrites 8q+8..8q+15); two jobs per thread.
template <int R>
__device__ __forceinline__ void pt_xpass(int* __restrict__ A) {
  using G = PtGeom<R>;
  constexpr int NV = (8 + G::W - 1 + 3) / 4;  // 128-bit loads of a quarter's inputs
#pragma unroll
  for (int rep = 0; rep < 2; ++rep) {
    const int it = threadIdx.x + rep * G::NT;
    const bool act = it < G::XJOBS;
    const int q = it & 3;
    int* row = A + (size_t)(act ? it >> 2 : 0) * G::HXP + 8 * q;
    int v[4 * NV];
    if (act) {
#pragma unroll
      for (int i = 0; i < NV; ++i) {
        const int4 c = reinterpret_cast<const int4*>(row)[i];
        v[4 * i] = c.x;
        v[4 * i + 1] = c.y;
        v[4 * i + 2] = c.z;
        v[4 * i + 3] = c.w;
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
      for (int x = 1; x < 8; ++x) {
        a += v[x + G::W - 1] - v[x - 1];
        o[x & 3] = a;
        if ((x & 3) == 3) reinterpret_cast<int4*>(row)[x >> 2] = make_int4(o[0], o[1], o[2], o[3]);
      }
    }
    __syncwarp();
  }
}

// y window pass from the x sums in A to Y (limb, row, column): one thread
// per (limb, column), the whole column in registers. Out of place, so no
// ordering between threads; fewer, longer jobs than in the x pass because
// this pass is bound by shared-memory wavefronts (a column's 32 words for
// its 24 sums).
template <int R>
__device__ __forceinline__ void pt_ypass(const int* __restrict__ A, int* __restrict__ Y) {
  using G = PtGeom<R>;
  constexpr int NIN = G::HY;
  const int it = threadIdx.x;
  if (it < G::YJOBS) {
    const int L = it >> 5, col = it & 31;
    const int* c = A + (size_t)L * G::PA + col;
    int* o = Y + (size_t)L * G::TY * 32 + col;
    int v[NIN];
#pragma unroll
    for (int i = 0; i < NIN; ++i) v[i] = c[i * G::HXP];
    int a = 0;
#pragma unroll
    for (int i = 0; i < G::W; ++i) a += v[i];
    o[0] = a;
#pragma unroll
    for (int y = 1; y < G::TY; ++y) {
      a += v[y + G::W - 1] - v[y - 1];
      o[y * 32] = a;
    }
  }
}

template <typename TS, int R>
__global__ void __launch_bounds__(32 * kPtTY, 1)
    k_fused_pt(const float* __restrict__ Mb, const TS* __restrict__ Ust,
               const float* __restrict__ sig, const int* __restrict__ su, FusedParams P, int k0,
               unsigned long long* __restrict__ acc, float* __restrict__ out_measure) {
  using G = PtGeom<R>;
  constexpr int NT = G::NT, TY = G::TY, MAXP = G::MAXP, WP = G::WP;
  constexpr int KB = PatchConst<3, R>::K;
  constexpr unsigned long long kmask = (1ull << KB) - 1ull;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* mc = reinterpret_cast<float*>(smem_raw);
  float2* SD = reinterpret_cast<float2*>(mc + G::NPW);
  int* lv = reinterpret_cast<int*>(smem_raw + G::OFF_LV);
  long long* sp = reinterpret_cast<long long*>(smem_raw + G::OFF_S);
  int* sq = reinterpret_cast<int*>(sp + 5 * G::NS);
  int* A = reinterpret_cast<int*>(smem_raw + G::OFF_A);
  int* Y = reinterpret_cast<int*>(smem_raw + G::OFF_Y);
  const int tid = threadIdx.x, slot = blockIdx.x, tile = blockIdx.y;
  const int x0 = (tile % P.ntx) * 32, y0 = P.y0 + (tile / P.ntx) * TY;
  const int ox = tid & 31, oy = tid >> 5;
  const int zb = blockIdx.z * P.zchunk;
  const int ze = min(zb + P.zchunk, P.vz);
  const size_t slice = (size_t)P.vx * P.vy;
  const float* Ms = Mb + (size_t)slot * slice * P.vz;
  // offsets in a slice of the thread's region points (planes) and halo
  // points (moments), -1 outside the grid, and each halo point's index in the
  // planes and in the limb planes
  int ro[WP], po[MAXP], pc[MAXP], pa[MAXP];
#pragma unroll
  for (int k = 0; k < WP; ++k) {
    const int i = tid + k * NT;
    const int py = i / G::PWP, px = i - py * G::PWP;
    const int gx = x0 - R - 1 + px, gy = y0 - R - 1 + py;
    ro[k] = (i < G::NPW && px < G::PW && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy)
                ? gy * P.vx + gx : -1;
  }
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
    const int p = tid + j * NT;
    int hy, hx;
    halo_point<kPtTY, R>(p, hy, hx);
    const int gx = x0 - R + hx, gy = y0 - R + hy;
    po[j] = (p < G::NP && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy) ? gy * P.vx + gx : -1;
    pc[j] = (hy + 1) * G::PWP + hx + 1;
    pa[j] = hy * G::HXP + hx;
  }
  // z-window sums of the first halo point in registers, of the second in
  // shared memory
  int accq[2] = {0, 0};
  long long accp[5] = {0, 0, 0, 0, 0};
  if (tid < G::NS) {
#pragma unroll
    for (int k = 0; k < 5; ++k) sp[k * G::NS + tid] = 0;
    sq[tid] = 0;
    sq[G::NS + tid] = 0;
  }
  const int e0 = zb - R;
  auto load_m = [&](int e, float* out) {
    const bool zin = (e >= 0 && e < P.vz);
    const float* src = Ms + (size_t)(zin ? e : 0) * slice;
#pragma unroll
    for (int k = 0; k < WP; ++k) {
      const int o = ro[k];
      out[k] = (zin && o >= 0) ? __ldg(src + o) : 0.0f;
    }
  };
  // region values of slices e+1 and e+2 (the last loaded an iteration
  // ahead); M(e) is the M plane itself
  float r1[WP], r2[WP];
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
  // planes of slice e+1 over those of slice e: M(e) from the M plane
  auto advance_planes = [&]() {
#pragma unroll
    for (int k = 0; k < WP; ++k) {
      const int i = tid + k * NT;
      if (i < G::NPW) {
        const float a = mc[i];
        mc[i] = r1[k];
        SD[i] = make_float2(a + 2.0f * r1[k] + r2[k], r2[k] - a);
      }
    }
  };
  // the entering slice's ultrasound and the leaving slice's M and U at the
  // thread's halo points, loaded an iteration ahead
  float u_nx[MAXP], ml_nx[MAXP], ul_nx[MAXP];
  auto load_halo = [&](int e) {
    const bool zin = (e >= 0 && e < P.vz);
    const int l = e - 2 * R - 1;
    const bool lin = (l >= e0 && l >= 0 && l < P.vz);
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const int o = po[j];
      u_nx[j] = (zin && o >= 0) ? ldf(Ust, (size_t)e * slice + o) : 0.0f;
      ml_nx[j] = (lin && o >= 0) ? __ldcs(Ms + (size_t)l * slice + o) : 0.0f;
      ul_nx[j] = (lin && o >= 0) ? ldf(Ust, (size_t)l * slice + o) : 0.0f;
    }
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
    float m_a[WP], m_b[WP];
    load_m(e0 - 1, m_a);
    load_m(e0, m_b);
    load_m(e0 + 1, r1);
    write_planes(m_a, m_b, r1);
    load_m(e0 + 2, r2);
  }
  load_halo(e0);
  load_sig(e0 - R);
  __syncthreads();
  long long acc_m = 0;
  for (int e = e0; e < ze + R; ++e) {
    const int z = e - R;
    const int l = e - 2 * R - 1;
    const bool out = (z >= zb);
    const bool leave = (l >= e0);
    int* lg = lv + ((e - e0) % G::RING) * G::NP;  // the leaving slice's slot
    // one halo point: the entering slice's quantised fields into the z
    // window (the leaving slice's out), the window's 12 limbs into plane A
    auto point = [&](int j, long long* ap, int* aq) {
      const int p = tid + j * NT;
      const int c = pc[j];
      const float m = mc[c];
      const float g = fused_sobel_sd<G::PWP>(SD, c);
      const int qm = quant(m, P.qm), qg = quant(g, P.qg), qu = quant(u_nx[j], P.qu);
      if (leave) {
        const int qml = quant(ml_nx[j], P.qm), qgl = lg[p], qul = quant(ul_nx[j], P.qu);
        ap[0] -= (long long)qul * qml;
        ap[1] -= (long long)qul * qgl;
        ap[2] -= (long long)qml * qml;
        ap[3] -= (long long)qgl * qgl;
        ap[4] -= (long long)qml * qgl;
        aq[0] -= qml;
        aq[1] -= qgl;
      }
      lg[p] = qg;
      ap[0] += (long long)qu * qm;
      ap[1] += (long long)qu * qg;
      ap[2] += (long long)qm * qm;
      ap[3] += (long long)qg * qg;
      ap[4] += (long long)qm * qg;
      aq[0] += qm;
      aq[1] += qg;
      if (out) {
        int* a = A + pa[j];
        a[0] = aq[0];
        a[G::PA] = aq[1];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          a[(2 + 2 * k) * G::PA] = (int)((unsigned long long)ap[k] & kmask);
          a[(3 + 2 * k) * G::PA] = (int)(ap[k] >> KB);
        }
      }
    };
    point(0, accp, accq);
    if (tid < G::NS) {
      long long ap[5];
      int aq[2];
#pragma unroll
      for (int k = 0; k < 5; ++k) ap[k] = sp[k * G::NS + tid];
      aq[0] = sq[tid];
      aq[1] = sq[G::NS + tid];
      point(1, ap, aq);
#pragma unroll
      for (int k = 0; k < 5; ++k) sp[k * G::NS + tid] = ap[k];
      sq[tid] = aq[0];
      sq[G::NS + tid] = aq[1];
    }
    // the next slice's halo values and this slice's sigma, in flight during
    // the window passes
    const float sg = sg_nx;
    const int sv = sv_nx;
    load_halo(e + 1);
    load_sig(z + 1);
    __syncthreads();  // planes(e) read, limbs written
    if (out) pt_xpass<R>(A);
    advance_planes();  // M(e), M(e+1), M(e+2)
#pragma unroll
    for (int k = 0; k < WP; ++k) r1[k] = r2[k];
    load_m(e + 3, r2);
    __syncthreads();
    if (out) {
      pt_ypass<R>(A, Y);
      __syncthreads();
      const int x = x0 + ox, y = y0 + oy;
      if (x < P.vx && y < P.vy) {
        float m = 0.0f;
        if (sg > 0.0f) {
          const int* a = Y + oy * 32 + ox;
          int L[kLimbs];
#pragma unroll
          for (int k = 0; k < kLimbs; ++k) L[k] = a[k * TY * 32];
          m = fused_measure<3, R>(P, sg, sv, L);
          acc_m += __float2int_rn(m * P.sum_scale);
        }
        if (out_measure && slot == 0) out_measure[(size_t)z * slice + (size_t)y * P.vx + x] = m;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc_m += __shfl_down_sync(0xffffffffu, acc_m, o);
  if ((tid & 31) == 0) atomicAdd(acc + 2 * (size_t)(k0 + slot), (unsigned long long)acc_m);
}

template <typename T, int R>
cudaError_t fused_pt_launch_r(const FusedLaunch& L, const float* M) {
  using G = PtGeom<R>;
  if (L.P.kbits != PatchConst<3, R>::K || L.P.n != PatchConst<3, R>::N)
    return cudaErrorInvalidValue;
  auto kern = k_fused_pt<T, R>;
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
  kern<<<grid, G::NT, G::BYTES, L.stream>>>(M, (const T*)L.ust, L.sig, L.su, P, L.k0, L.acc,
                                            L.out_measure);
  return cudaGetLastError();
}

// Patch radius 1..4 (shared memory holds two limb buffers up to radius 4).
// 24-row tiles when the launch asks for them, 16-row tiles otherwise.
template <typename T>
cudaError_t fused_ps_launch(const FusedLaunch& L, const float* M) {
  const bool tall = L.tile_height == kPtTY;
  switch (L.P.r) {
    case 1: return tall ? fused_pt_launch_r<T, 1>(L, M) : fused_ps_launch_r<T, 1>(L, M);
    case 2: return tall ? fused_pt_launch_r<T, 2>(L, M) : fused_ps_launch_r<T, 2>(L, M);
    case 3: return tall ? fused_pt_launch_r<T, 3>(L, M) : fused_ps_launch_r<T, 3>(L, M);
    case 4: return tall ? fused_pt_launch_r<T, 4>(L, M) : fused_ps_launch_r<T, 4>(L, M);
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
