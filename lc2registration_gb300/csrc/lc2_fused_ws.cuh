// lc2_fused_ws.cuh -- warp-specialised variant of the fused 3D kernel.
//
// Same evaluation as k_fused<3, ...> with 32 x 16 tiles (lc2_fused.cuh), split
// between two warp roles of one CTA so that the moving-volume gathers of
// later slices overlap the moment work of the current one:
//   * 4 producer warps resample slice after slice of the tile's region into a
//     ring of NSLOT shared M planes (src/Interpolator/interpolator.cu:69-179);
//   * 16 consumer warps build the z-smoothed / z-differentiated Sobel planes
//     from three ring slices, update the z-window limbs, run the x/y window
//     passes and solve (src/cu_LC2/cu_lc2_3d.cu:100-618), exactly as k_fused.
// Hand-off per ring slot through two mbarriers: `full` (producers -> consumers)
// and `empty` (consumers -> producers). Each role synchronises internally with
// its own named barrier (1: consumers, 2: producers), so neither waits at the
// other's barriers. Every mbarrier wait is bounded by a one-second deadline on
// the global timer: on expiry the CTA raises an abort flag, stops waiting
// (all later waits return at once, every named barrier is still reached by
// its whole group) and reports through `err`; the host turns that into an
// error status. Results are identical to k_fused bit for bit: same sampling
// base, same exact sums.
#pragma once

#include "lc2_fused.cuh"

namespace lc2 {

constexpr int kWsProducers = 128;  // 4 warps
constexpr int kWsSlots = 4;        // M planes in the ring

__device__ __forceinline__ unsigned smem_addr(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the phase of `bar` with the given parity to complete, for at most
// one second -- or 2^26 polls, should the global timer not advance; on expiry
// (or when another thread already gave up) sets the abort flag and returns
// false.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity,
                                          volatile int* abort_flag, int* err) {
  const unsigned addr = smem_addr(bar);
  unsigned long long t0 = 0;
  for (unsigned it = 0;; ++it) {
    if (*abort_flag) return false;
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    if (ok) return true;
    if (it == 0) {
      t0 = global_ns();
    } else if ((it & 63) == 0 && (global_ns() - t0 > 1000000000ull || it >= (1u << 26))) {
      *abort_flag = 1;
      atomicExch(err, 1);
      return false;
    }
  }
}

template <int R>
struct WsGeom {
  using G = FusedGeom<3, 16, R>;
  static constexpr int NT = G::NT + kWsProducers;  // 640
  static constexpr size_t OFF_SD = sizeof(float) * (size_t)kWsSlots * G::NPW;
  static constexpr size_t OFF_LV = OFF_SD + sizeof(float2) * (size_t)G::NPW;
  static constexpr size_t OFF_A = OFF_LV + sizeof(int) * (size_t)G::RING * 2 * G::NP;
  static constexpr size_t BYTES = OFF_A + sizeof(int) * (size_t)kLimbs * G::HY * G::HXP;
};

template <typename TM, typename TS, int R>
__global__ void __launch_bounds__(WsGeom<R>::NT, 1)
    k_fused_ws(const TM* __restrict__ mov, const TS* __restrict__ Ust,
               const float* __restrict__ sig, const int* __restrict__ su, FusedParams P,
               const Xform* __restrict__ xf, int k0, unsigned long long* __restrict__ acc,
               int* __restrict__ err) {
  constexpr int TY = 16;
  using W = WsGeom<R>;
  using G = typename W::G;
  constexpr int NC = G::NT;  // consumer threads
  constexpr size_t PA = (size_t)G::HY * G::HXP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* ring = reinterpret_cast<float*>(smem_raw);
  float2* SD = reinterpret_cast<float2*>(smem_raw + W::OFF_SD);
  int* lv = reinterpret_cast<int*>(smem_raw + W::OFF_LV);
  int* A = reinterpret_cast<int*>(smem_raw + W::OFF_A);
  __shared__ __align__(8) unsigned long long full[kWsSlots], empty[kWsSlots];
  __shared__ Xform s_xf;
  __shared__ float s_A[9];
  __shared__ volatile int s_abort;

  const int tid = threadIdx.x;
  const int slot = blockIdx.x;
  const int tile = blockIdx.y;
  const int x0 = (tile % P.ntx) * 32, y0 = (tile / P.ntx) * TY;
  const Xform* X = xf + k0 + slot;
  const int gx0 = x0 - R - 1, gy0 = y0 - R - 1;
  const int yb = y0 % kBand;  // the sampling base of k_fused
  const int zb = blockIdx.z * P.zchunk;
  const int ze = min(zb + P.zchunk, P.vz);
  const int e0 = zb - R;                 // first slice entering the window
  const int nslices = ze + R - e0 + 2;   // slices e0 - 1 .. ze + R

  if (tid == 0) {
    for (int s = 0; s < kWsSlots; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    s_xf = *X;
#pragma unroll
    for (int i = 0; i < 9; ++i) s_A[i] = X->ah[i];
    s_abort = 0;
  }
  __syncthreads();

  if (tid >= NC) {
    // ------------------------------------------------------------ producers
    const int ptid = tid - NC;
    for (int q = 0; q < nslices; ++q) {
      const int sl = q % kWsSlots, use = q / kWsSlots;
      if (use > 0) mbar_wait(&empty[sl], (unsigned)((use - 1) & 1), &s_abort, err);
      const int zs = e0 - 1 + q;
      // base of slice zs (every lane computes the same value)
      int ib[3];
      float fb[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) xform_coord(s_xf, a, gx0, gy0 - yb, zs, ib[a], fb[a]);
      float* out = ring + (size_t)sl * G::NPW;
      const bool zin = (zs >= 0 && zs < P.vz);
      for (int i = ptid; i < G::NPW; i += kWsProducers) {
        const int py = i / G::PW, px = i - py * G::PW;
        const int gx = gx0 + px, gy = gy0 + py;
        float v = 0.0f;
        if (zin && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy)
          v = fused_sample<3, TM>(mov, P, s_A, ib, fb, px, py + yb);
        out[i] = v;
      }
      group_sync<2, kWsProducers>();
      if (ptid == 0) mbar_arrive(&full[sl]);
    }
    return;
  }

  // -------------------------------------------------------------- consumers
  const int ox = tid & 31, oy = tid >> 5;
  long long acc_m = 0;
  constexpr int MAXP = G::MAXP;
  int acc32[MAXP][kLimbs];
#pragma unroll
  for (int j = 0; j < MAXP; ++j)
#pragma unroll
    for (int k = 0; k < kLimbs; ++k) acc32[j][k] = 0;
  int pc[MAXP], pa_off[MAXP], pu[MAXP];
  bool pin[MAXP];
#pragma unroll
  for (int j = 0; j < MAXP; ++j) {
    const int p = tid + j * NC;
    const int hy = p / G::HX, hx = p - hy * G::HX;
    const int gx = x0 - R + hx, gy = y0 - R + hy;
    pc[j] = (hy + 1) * G::PW + hx + 1;
    pa_off[j] = hy * G::HXP + hx;
    pin[j] = (p < G::NP) && gx >= 0 && gx < P.vx && gy >= 0 && gy < P.vy;
    pu[j] = pin[j] ? gy * P.vx + gx : 0;
  }
  const size_t slice = (size_t)P.vx * P.vy;
  float u_in[MAXP], u_out[MAXP];
  auto load_u = [&](int e) {
    const int l = e - 2 * R - 1;
    const bool ezin = (e >= 0 && e < P.vz), lzin = (l >= e0 && l >= 0 && l < P.vz);
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      u_in[j] = (pin[j] && ezin) ? ldf(Ust, (size_t)e * slice + pu[j]) : 0.0f;
      u_out[j] = (pin[j] && lzin) ? ldf(Ust, (size_t)l * slice + pu[j]) : 0.0f;
    }
  };
  load_u(e0);
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
  // slices e0 - 1 and e0 (ring entries 0 and 1, first use of their slots)
  mbar_wait(&full[0], 0u, &s_abort, err);
  mbar_wait(&full[1], 0u, &s_abort, err);
  for (int e = e0; e < ze + R; ++e) {
    const int qn = e - e0 + 2;  // ring entry of slice e + 1
    mbar_wait(&full[qn % kWsSlots], (unsigned)((qn / kWsSlots) & 1), &s_abort, err);
    const float* Mp = ring + (size_t)((qn - 2) % kWsSlots) * G::NPW;  // slice e - 1
    const float* Mc = ring + (size_t)((qn - 1) % kWsSlots) * G::NPW;  // slice e
    const float* Mn = ring + (size_t)(qn % kWsSlots) * G::NPW;        // slice e + 1
    for (int i = tid; i < G::NPW; i += NC) {
      const float a = Mp[i], b = Mc[i], c = Mn[i];
      SD[i] = make_float2(a + 2.0f * b + c, c - a);
    }
    group_sync<1, NC>();
    if (tid == 0) mbar_arrive(&empty[(qn - 2) % kWsSlots]);  // slice e - 1 is no longer read
    const int z = e - R;
    const float sg = sg_nx;
    const int sv = sv_nx;
    const int l = e - 2 * R - 1;
    const bool out = (z >= zb);
    const bool leave = (l >= e0);
    int* lv_in = lv + ((e - e0) % G::RING) * 2 * G::NP;
    const int* lv_out = lv + ((l - e0 + G::RING) % G::RING) * 2 * G::NP;
#pragma unroll
    for (int j = 0; j < MAXP; ++j) {
      const int p = tid + j * NC;
      if (p < G::NP) {
        const float u = u_in[j], ul = u_out[j];
        const float m = Mc[pc[j]];
        const float g = fused_sobel_sd<G::PW>(SD, pc[j]);
        const int qm = quant(m, P.qm), qg = quant(g, P.qg);
        int Li[kLimbs];
        fused_limbs(quant(u, P.qu), qm, qg, PatchConst<3, R>::K, Li);
        // the leaving slice's ring slot is the entering slice's: read first
        const int qml = leave ? lv_out[p] : 0, qgl = leave ? lv_out[G::NP + p] : 0;
        lv_in[p] = qm;
        lv_in[G::NP + p] = qg;
        if (leave) {
          int Lo[kLimbs];
          fused_limbs(quant(ul, P.qu), qml, qgl, PatchConst<3, R>::K, Lo);
#pragma unroll
          for (int k = 0; k < kLimbs; ++k) acc32[j][k] += Li[k] - Lo[k];
        } else {
#pragma unroll
          for (int k = 0; k < kLimbs; ++k) acc32[j][k] += Li[k];
        }
        if (out) {
          int* a = A + pa_off[j];
#pragma unroll
          for (int k = 0; k < kLimbs; ++k) a[k * PA] = acc32[j][k];
        }
      }
    }
    load_u(e + 1);
    load_sig(z + 1);
    group_sync<1, NC>();
    if (out) {
      fused_xy<3, TY, R, 1>(A);
      const int x = x0 + ox, y = y0 + oy;
      if (x < P.vx && y < P.vy && sg > 0.0f) {
        const int* a = A + oy * G::HXP + ox;
        int L[kLimbs];
#pragma unroll
        for (int k = 0; k < kLimbs; ++k) L[k] = a[k * PA];
        const float m = fused_measure<3, R>(P, sg, sv, L);
        acc_m += __float2int_rn(m * P.sum_scale);
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc_m += __shfl_down_sync(0xffffffffu, acc_m, o);
  if ((tid & 31) == 0) atomicAdd(acc + 2 * (size_t)(k0 + slot), (unsigned long long)acc_m);
}

template <typename T, int R>
cudaError_t fused_ws_launch_r(const FusedLaunch& L, int* err) {
  using W = WsGeom<R>;
  if (L.P.kbits != PatchConst<3, R>::K || L.P.n != PatchConst<3, R>::N)
    return cudaErrorInvalidValue;
  auto kern = k_fused_ws<T, T, R>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)W::BYTES);
  if (e != cudaSuccess) return e;
  FusedParams P = L.P;
  const int ntx = (P.vx + 31) / 32, nty = (P.vy + 15) / 16;
  P.ntx = ntx;
  int nz;
  if (L.zchunk > 0) {
    P.zchunk = L.zchunk < P.vz ? L.zchunk : P.vz;
  } else {
    P.zchunk = auto_zchunk(P.vz, R, (long long)ntx * nty * L.cnt, (long long)L.sms);
  }
  nz = (P.vz + P.zchunk - 1) / P.zchunk;
  dim3 grid(L.cnt, ntx * nty, nz);
  kern<<<grid, W::NT, W::BYTES, L.stream>>>((const T*)L.mov, (const T*)L.ust, L.sig, L.su, P,
                                            L.xf, L.k0, L.acc, err);
  return cudaGetLastError();
}

// 3D, patch radius 1..4 (the 16-row tiles); cudaErrorInvalidValue otherwise.
template <typename T>
cudaError_t fused_ws_launch(const FusedLaunch& L, int* err) {
  switch (L.P.r) {
    case 1: return fused_ws_launch_r<T, 1>(L, err);
    case 2: return fused_ws_launch_r<T, 2>(L, err);
    case 3: return fused_ws_launch_r<T, 3>(L, err);
    case 4: return fused_ws_launch_r<T, 4>(L, err);
  }
  return cudaErrorInvalidValue;
}

}  // namespace lc2
