// lc2_capi.cu -- context management, launch sequencing and the C ABI
// declared in include/lc2.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <atomic>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/lc2.h"
#include "lc2_kernels.cuh"
#include "lc2_fused.cuh"
#include "lc2_fused_fixed.cuh"
#include "lc2_fused_ps.cuh"
#include "lc2_list.cuh"
#include "lc2_mi.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define LC2_CUDA(call)                                                                     \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      if (e_ == cudaErrorMemoryAllocation)                                                 \
        return fail(LC2_ERR_OUT_OF_MEMORY, "%s: %s", #call, cudaGetErrorString(e_));       \
      return fail(LC2_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                  __LINE__);                                                               \
    }                                                                                      \
  } while (0)

#define LC2_TRY(expr)         \
  do {                        \
    int s_ = (expr);          \
    if (s_ != LC2_OK) return s_; \
  } while (0)

size_t elem_size(int storage) { return storage == LC2_STORE_F32 ? 4 : 2; }

// Device memory comes from the device's default stream-ordered pool, set to
// keep what is freed (release threshold: unlimited), so creating and
// destroying contexts never synchronises the device: cudaFree would wait for
// every stream, i.e. for other requests' kernels.
// Allocation-failure injection (lc2_debug_fail_allocation) and the account of
// live device bytes it is checked against. Test hooks on the host: a failed
// allocation returns cudaErrorMemoryAllocation without calling CUDA.
std::atomic<long long> g_fail_countdown{0};
std::mutex g_live_mu;
std::map<void*, size_t> g_live;
size_t g_live_bytes = 0;

bool injected_failure() {
  long long k = g_fail_countdown.load();
  while (k > 0) {
    if (g_fail_countdown.compare_exchange_weak(k, k - 1)) return k == 1;
  }
  return false;
}

cudaError_t dev_alloc(void** p, size_t n, cudaStream_t st) {
  if (n > 0 && injected_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  static std::mutex mu;
  static std::vector<int> ready;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (std::find(ready.begin(), ready.end(), dev) == ready.end()) {
      cudaMemPool_t pool;
      e = cudaDeviceGetDefaultMemPool(&pool, dev);
      if (e != cudaSuccess) return e;
      unsigned long long keep = ~0ull;
      e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
      if (e != cudaSuccess) return e;
      ready.push_back(dev);
    }
  }
  *p = nullptr;
  if (n == 0) return cudaSuccess;
  e = cudaMallocAsync(p, n, st);
  if (e == cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_live_mu);
    g_live[*p] = n;
    g_live_bytes += n;
  }
  return e;
}

void dev_free(void* p, cudaStream_t st) {
  if (!p) return;
  {
    std::lock_guard<std::mutex> lk(g_live_mu);
    auto it = g_live.find(p);
    if (it != g_live.end()) {
      g_live_bytes -= it->second;
      g_live.erase(it);
    }
  }
  cudaFreeAsync(p, st);
}

// Pinned host buffers are cached by power-of-two size and reused (cudaFreeHost
// can synchronise the device too).
std::mutex g_pin_mu;
std::multimap<size_t, void*> g_pin_free;
std::map<void*, size_t> g_pin_size;

cudaError_t host_alloc(void** p, size_t n) {
  if (injected_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  size_t cls = 4096;
  while (cls < n) cls <<= 1;
  {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    auto it = g_pin_free.find(cls);
    if (it != g_pin_free.end()) {
      *p = it->second;
      g_pin_free.erase(it);
      return cudaSuccess;
    }
  }
  cudaError_t e = cudaMallocHost(p, cls);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_pin_mu);
  g_pin_size[*p] = cls;
  return cudaSuccess;
}

void host_free(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pin_mu);
  auto it = g_pin_size.find(p);
  if (it != g_pin_size.end()) g_pin_free.emplace(it->second, p);
}

}  // namespace

// Message for lc2_last_error from the other translation units.
void lc2_set_error_message(const char* msg) { g_err = msg ? msg : ""; }

struct lc2_context {
  lc2_config cfg{};
  int warp_nd = 3;  // dimensionality of the resampling
  int lc2_nd = 3;   // dimensionality of Sobel / patches
  lc2_geometry virt{};
  size_t nv = 0, nf = 0, nm = 0;  // voxels: virtual, fixed, moving
  int n = 0;                      // patch voxels
  int qbits = 0;
  bool ready = false;

  // device buffers
  void* d_moving = nullptr;    // storage type, nm
  bool owns_moving = true;     // false for the frames of a stack (shared volume)
  void* d_static = nullptr;    // hr_moving: U in storage type; hr_fixed: M as float
  float* d_gstatic = nullptr;  // hr_fixed: Sobel(M)
  float* d_scratch = nullptr;  // per-slot warped image (+ Sobel when hr_moving)
  int slots = 1;
  size_t per_slot = 0;  // scratch bytes per slot
  lc2::Xform* d_xf = nullptr;
  unsigned long long* d_acc = nullptr;
  double* d_out = nullptr;
  int cap = 0;  // capacity of d_xf/d_acc/d_out (transforms)
  // d_acc is all zero: k_finalize resets what it read, so only a launch whose
  // sums were not finalised (another path, an error) leaves it dirty
  bool acc_clean = false;
  lc2::Xform* h_xf = nullptr;  // pinned staging
  double* h_out = nullptr;     // pinned results
  int staged = 0;

  lc2::MomentParams mp{};
  lc2::FusedParams fp{};
  float vmax_u = 0, vmax_m = 0, vmax_g = 0;
  // static ultrasound (HighResolutionModality: Moving): weighting factor per
  // voxel and its exact fixed-point sum
  float* d_sigma = nullptr;
  int* d_su = nullptr;  // window sum of the quantised static ultrasound per voxel
  long long sigma_sum = -1;
  // resampled ultrasound (HighResolutionModality: Fixed): the static image
  // and its Sobel quantised, their window sums and centred sums
  // (lc2_fused_fixed.cuh)
  int* d_fq = nullptr;
  int* d_fs = nullptr;        // (S_M, S_G) per voxel, interleaved
  long long* d_fd = nullptr;
  float4* d_fsv = nullptr;    // solve factors per voxel (k_fixed_solve_static)
  int generic = 0;  // LC2_OPTION_GENERIC
  int sms = 152;    // multiprocessors of the device (queried at creation)
  // normalised mutual information (patch_size 0): static image bins and
  // entropy, per-transform range and joint histogram
  bool mi = false;
  unsigned char* d_sbin = nullptr;
  unsigned* d_hist = nullptr;
  double* d_mipart = nullptr;  // entropy sums per part of each histogram
  unsigned* d_rmin = nullptr;
  unsigned* d_rmax = nullptr;
  double h_static = 0.0;
  int tile_rows = 0;  // fused kernel tile height (0 = automatic)
  int zchunk = 0;     // fused kernel output slices per CTA (0 = automatic)
  int pipeline = 0;   // warp-specialised fused 3D kernel (LC2_OPTION_PIPELINE)
  int presample = 0;  // 3D: resample as a pass of its own (LC2_OPTION_PRESAMPLE)
  float* d_pre = nullptr;  // presampled images (FP32 M) of pre_slots transforms
  int pre_slots = 0;
  int* d_err = nullptr;   // device flag of the warp-specialised kernel's bounded waits
  int* h_err = nullptr;   // pinned copy

  // CUDA graphs of lc2_evaluate_batch's sequence (copy-in, fused launch,
  // ratio, copy-out) by batch size; dropped when buffers or options change
  struct Graph {
    int count;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    long long kernels;  // kernel launches in the graph
  };
  std::vector<Graph> graphs;
  bool use_graphs = true;
  long long graph_launches = 0;

  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  long long launches = 0;

  // optional per-kernel timing (lc2_enable_kernel_timing)
  bool timing = false;
  struct Timed {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<Timed> timed;
};

namespace lc2 {
// Exact window sum of width 2r+1 along one axis (0 = x, 1 = y, 2 = z) with
// zero padding; one thread per line of the (nx, ny, nz) grid.
template <typename T>
__global__ void k_box_line(const T* __restrict__ in, T* __restrict__ out, int nx, int ny,
                           int nz, int axis, int r) {
  const long long line = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  size_t base, stride;
  int len;
  if (axis == 0) {
    if (line >= (long long)ny * nz) return;
    base = (size_t)line * nx; stride = 1; len = nx;
  } else if (axis == 1) {
    if (line >= (long long)nx * nz) return;
    base = (size_t)(line / nx) * nx * ny + (size_t)(line % nx); stride = nx; len = ny;
  } else {
    if (line >= (long long)nx * ny) return;
    base = (size_t)line; stride = (size_t)nx * ny; len = nz;
  }
  T a = 0;
  for (int i = 0; i <= r && i < len; ++i) a += in[base + i * stride];
  out[base] = a;
  for (int i = 1; i < len; ++i) {
    if (i + r < len) a += in[base + (size_t)(i + r) * stride];
    if (i - r - 1 >= 0) a -= in[base + (size_t)(i - r - 1) * stride];
    out[base + (size_t)i * stride] = a;
  }
}

// Resampled ultrasound: the static image M and its Sobel G quantised per
// virtual voxel (q[2][nv]) and their products MM, GG, MG (p[3][nv]), the
// fields whose window sums the fused kernel reads.
__global__ void k_fixed_quant(const float* __restrict__ M, const float* __restrict__ G, size_t nv,
                              float qm, float qg, int* __restrict__ q, long long* __restrict__ p) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv;
       i += (size_t)gridDim.x * blockDim.x) {
    const int m = quant(M[i], qm), g = quant(G[i], qg);
    q[i] = m;
    q[nv + i] = g;
    p[i] = (long long)m * m;
    p[nv + i] = (long long)g * g;
    p[2 * nv + i] = (long long)m * g;
  }
}

// Window sums S_MM, S_GG, S_MG (d[3][nv]) -> centred sums n S_xy - S_x S_y.
__global__ void k_fixed_centre(const int* __restrict__ s, long long* __restrict__ d, size_t nv,
                               long long n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv;
       i += (size_t)gridDim.x * blockDim.x) {
    const long long sm = s[i], sg = s[nv + i];
    d[i] = n * d[i] - sm * sm;
    d[nv + i] = n * d[nv + i] - sg * sg;
    d[2 * nv + i] = n * d[2 * nv + i] - sm * sg;
  }
}

// Per static voxel: (S_M, S_G) interleaved, and the solve factors of
// solve_centred_static -- im = rsqrtf(D_mm) when D_mm > thr_m else 0, ig
// likewise, rmg = D_mg im ig when both columns count -- with the float
// operations solve_centred applies to them.
__global__ void k_fixed_solve_static(const int* __restrict__ s, const long long* __restrict__ d,
                                     size_t nv, long long thr_m, long long thr_g,
                                     int2* __restrict__ smg, float4* __restrict__ sv) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv;
       i += (size_t)gridDim.x * blockDim.x) {
    const long long dmm = d[i], dgg = d[nv + i], dmg = d[2 * nv + i];
    const bool km = dmm > thr_m, kg = dgg > thr_g;
    const float im = km ? rsqrtf(ll2f(dmm)) : 0.0f, ig = kg ? rsqrtf(ll2f(dgg)) : 0.0f;
    const float rmg = (km && kg) ? ll2f(dmg) * im * ig : 0.0f;
    smg[i] = make_int2(s[i], s[nv + i]);
    sv[i] = make_float4(im, ig, rmg, 0.0f);
  }
}

// LC2 = sum(measure) / sum(sigma); 0 when NaN/Inf (cu_lc2_3d.cu:1189-1191).
// sigma_sum >= 0: the weighting-factor sum is static (precomputed), else it
// is taken from the accumulator.
// The sums it read are reset to zero, so a replayed batch starts from zero
// without a memset.
__global__ void k_finalize(unsigned long long* __restrict__ acc, int count,
                           double* __restrict__ out, long long sigma_sum) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const unsigned long long a0 = acc[2 * k], a1 = acc[2 * k + 1];
  acc[2 * k] = 0;
  acc[2 * k + 1] = 0;
  double m = (double)(long long)a0;
  double s = sigma_sum >= 0 ? (double)sigma_sum : (double)(long long)a1;
  double v = m / s;
  if (isnan(v) || isinf(v)) v = 0.0;
  out[k] = v;
}

}  // namespace lc2

namespace {

// Kernel kinds for lc2_kernel_times.
enum { K_WARP = 0, K_SOBEL = 1, K_MOMENTS = 2, K_KINDS = 3 };

struct TimerScope {
  lc2_context* c;
  int kind;
  cudaEvent_t a = nullptr, b = nullptr;
  TimerScope(lc2_context* c_, int kind_) : c(c_), kind(kind_) {
    if (!c->timing) return;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
      a = b = nullptr;
      return;
    }
    cudaEventRecord(a, c->stream);
  }
  ~TimerScope() {
    if (!a) return;
    cudaEventRecord(b, c->stream);
    c->timed.push_back({kind, a, b});
  }
};

int select_device(const lc2_context* c) {
  int cur = -1;
  LC2_CUDA(cudaGetDevice(&cur));
  if (cur != c->cfg.device) LC2_CUDA(cudaSetDevice(c->cfg.device));
  return LC2_OK;
}

bool finite_geom(const lc2_geometry& g) {
  for (int a = 0; a < 3; ++a) {
    if (g.dim[a] < 1) return false;
    if (!std::isfinite(g.spacing[a]) || !(g.spacing[a] > 0.0f)) return false;
    if (!std::isfinite(g.origin[a])) return false;
  }
  return true;
}

// Moving-pixel affine of virtual voxels in double (lc2::XformD), stored as
// the float-float split the kernels read (lc2::Xform).
void build_xform(int nd, const lc2_geometry& v, const lc2_geometry& m, const float* mat,
                 lc2::Xform* X) {
  double L[3][3] = {{0}}, t[3] = {0};
  if (nd == 2) {
    for (int a = 0; a < 2; ++a) {
      L[a][0] = mat[3 * a + 0];
      L[a][1] = mat[3 * a + 1];
      t[a] = mat[3 * a + 2];
    }
  } else {
    for (int a = 0; a < 3; ++a) {
      for (int b = 0; b < 3; ++b) L[a][b] = mat[4 * a + b];
      t[a] = mat[4 * a + 3];
    }
  }
  lc2::XformD D{};
  for (int a = 0; a < 3; ++a) {
    double bsum = t[a] - (double)m.origin[a];
    for (int b = 0; b < 3; ++b) {
      D.A[3 * a + b] = L[a][b] * (double)v.spacing[b] / (double)m.spacing[a];
      bsum += L[a][b] * (double)v.origin[b];
    }
    D.b[a] = bsum / (double)m.spacing[a];
    if (nd == 2 && a == 2) {
      D.A[6] = D.A[7] = D.A[8] = 0.0;
      D.b[2] = 0.0;
    }
  }
  if (nd == 2) {
    D.A[2] = 0.0;
    D.A[5] = 0.0;
  }
  *X = lc2::xform_split(D);
}

long long floor_clamp(long double v) {
  if (v >= (long double)std::numeric_limits<long long>::max()) return std::numeric_limits<long long>::max();
  if (v < 0) return -1;
  return (long long)std::floor(v);
}

void drop_graphs(lc2_context* c) {
  for (auto& g : c->graphs) {
    cudaGraphExecDestroy(g.exec);
    cudaGraphDestroy(g.graph);
  }
  c->graphs.clear();
}

int ensure_capacity(lc2_context* c, int count) {
  if (count <= c->cap) return LC2_OK;
  drop_graphs(c);  // the graphs read the buffers being replaced
  int ncap = std::max(count, std::max(64, c->cap * 2));
  dev_free(c->d_xf, c->stream);
  dev_free(c->d_acc, c->stream);
  dev_free(c->d_out, c->stream);
  if (c->h_xf || c->h_out) cudaStreamSynchronize(c->stream);  // pending copies
  host_free(c->h_xf);
  host_free(c->h_out);
  c->d_xf = nullptr; c->d_acc = nullptr; c->d_out = nullptr; c->h_xf = nullptr; c->h_out = nullptr;
  c->cap = 0;
  LC2_CUDA(dev_alloc((void**)&c->d_xf, sizeof(lc2::Xform) * ncap, c->stream));
  LC2_CUDA(dev_alloc((void**)&c->d_acc, sizeof(unsigned long long) * 2 * ncap, c->stream));
  c->acc_clean = false;
  LC2_CUDA(dev_alloc((void**)&c->d_out, sizeof(double) * ncap, c->stream));
  LC2_CUDA(host_alloc((void**)&c->h_xf, sizeof(lc2::Xform) * ncap));
  LC2_CUDA(host_alloc((void**)&c->h_out, sizeof(double) * ncap));
  if (c->mi) {
    dev_free(c->d_hist, c->stream);
    dev_free(c->d_mipart, c->stream);
    dev_free(c->d_rmin, c->stream);
    dev_free(c->d_rmax, c->stream);
    c->d_hist = nullptr; c->d_mipart = nullptr; c->d_rmin = nullptr; c->d_rmax = nullptr;
    LC2_CUDA(dev_alloc((void**)&c->d_hist, sizeof(unsigned) * lc2::kMiHist * (size_t)ncap, c->stream));
    LC2_CUDA(dev_alloc((void**)&c->d_mipart, sizeof(double) * 2 * lc2::kMiParts * (size_t)ncap,
                       c->stream));
    LC2_CUDA(dev_alloc((void**)&c->d_rmin, sizeof(unsigned) * ncap, c->stream));
    LC2_CUDA(dev_alloc((void**)&c->d_rmax, sizeof(unsigned) * ncap, c->stream));
  }
  c->cap = ncap;
  return LC2_OK;
}

template <typename T>
int launch_convert(lc2_context* c, const float* in, void* out, size_t n) {
  int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  lc2::k_convert<T><<<blocks, 256, 0, c->stream>>>(in, reinterpret_cast<T*>(out), n);
  ++c->launches;
  LC2_CUDA(cudaGetLastError());
  return LC2_OK;
}

int convert_to_storage(lc2_context* c, const float* in, void* out, size_t n, int storage) {
  if (storage == LC2_STORE_F16) return launch_convert<__half>(c, in, out, n);
  if (storage == LC2_STORE_BF16) return launch_convert<__nv_bfloat16>(c, in, out, n);
  return launch_convert<float>(c, in, out, n);
}

template <typename T>
__global__ void k_tofloat(const T* __restrict__ in, float* __restrict__ out, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t step = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += step) out[i] = lc2::ldf(in, i);
}

int to_float(lc2_context* c, const void* in, float* out, size_t n, int storage) {
  int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  if (storage == LC2_STORE_F16)
    k_tofloat<__half><<<blocks, 256, 0, c->stream>>>((const __half*)in, out, n);
  else if (storage == LC2_STORE_BF16)
    k_tofloat<__nv_bfloat16><<<blocks, 256, 0, c->stream>>>((const __nv_bfloat16*)in, out, n);
  else
    k_tofloat<float><<<blocks, 256, 0, c->stream>>>((const float*)in, out, n);
  ++c->launches;
  LC2_CUDA(cudaGetLastError());
  return LC2_OK;
}

template <typename TM>
int launch_warp_t(lc2_context* c, int nd, const TM* src, const lc2_geometry& sg, const lc2::Xform* xf,
                  int k0, int cnt, float* out, size_t slot_stride) {
  const lc2_geometry& v = c->virt;
  dim3 block(32, 8, 1);
  dim3 grid((v.dim[0] + 31) / 32, (v.dim[1] + 7) / 8, v.dim[2] * cnt);
  TimerScope ts(c, K_WARP);
  if (nd == 3)
    lc2::k_warp<3, TM><<<grid, block, 0, c->stream>>>(src, sg.dim[0], sg.dim[1], sg.dim[2],
                                                      v.dim[0], v.dim[1], v.dim[2], xf, k0, out,
                                                      slot_stride);
  else
    lc2::k_warp<2, TM><<<grid, block, 0, c->stream>>>(src, sg.dim[0], sg.dim[1], sg.dim[2],
                                                      v.dim[0], v.dim[1], v.dim[2], xf, k0, out,
                                                      slot_stride);
  ++c->launches;
  LC2_CUDA(cudaGetLastError());
  return LC2_OK;
}

int launch_warp(lc2_context* c, int nd, const void* src, int storage, const lc2_geometry& sg,
                const lc2::Xform* xf, int k0, int cnt, float* out, size_t slot_stride) {
  if (storage == LC2_STORE_F16)
    return launch_warp_t<__half>(c, nd, (const __half*)src, sg, xf, k0, cnt, out, slot_stride);
  if (storage == LC2_STORE_BF16)
    return launch_warp_t<__nv_bfloat16>(c, nd, (const __nv_bfloat16*)src, sg, xf, k0, cnt, out,
                                        slot_stride);
  return launch_warp_t<float>(c, nd, (const float*)src, sg, xf, k0, cnt, out, slot_stride);
}

int launch_sobel(lc2_context* c, const float* in, float* out, int cnt, size_t slot_stride) {
  const lc2_geometry& v = c->virt;
  dim3 block(32, 8, 1);
  dim3 grid((v.dim[0] + 31) / 32, (v.dim[1] + 7) / 8, v.dim[2] * cnt);
  TimerScope ts(c, K_SOBEL);
  if (c->lc2_nd == 3)
    lc2::k_sobel<3><<<grid, block, 0, c->stream>>>(in, v.dim[0], v.dim[1], v.dim[2], out,
                                                   slot_stride);
  else
    lc2::k_sobel<2><<<grid, block, 0, c->stream>>>(in, v.dim[0], v.dim[1], v.dim[2], out,
                                                   slot_stride);
  ++c->launches;
  LC2_CUDA(cudaGetLastError());
  return LC2_OK;
}

template <int ND, typename TU>
int launch_moments_t(lc2_context* c, const TU* U, const float* M, const float* G,
                     const lc2::MomentParams& P, int k0, int cnt, float* osig, float* omeas) {
  c->acc_clean = false;
  const lc2_geometry& v = c->virt;
  size_t smem = lc2::mom_smem_bytes(P.r);
  LC2_CUDA(cudaFuncSetAttribute(lc2::k_moments<ND, TU>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((v.dim[0] + lc2::kTX - 1) / lc2::kTX, (v.dim[1] + lc2::kTY - 1) / lc2::kTY,
            P.nzchunks * cnt);
  TimerScope ts(c, K_MOMENTS);
  lc2::k_moments<ND, TU><<<grid, lc2::kNT, smem, c->stream>>>(U, M, G, P, c->d_acc, k0, osig,
                                                              omeas);
  ++c->launches;
  LC2_CUDA(cudaGetLastError());
  return LC2_OK;
}

template <int ND>
int launch_moments_nd(lc2_context* c, const void* U, int ustore, const float* M, const float* G,
                      const lc2::MomentParams& P, int k0, int cnt, float* osig, float* omeas) {
  if (ustore == LC2_STORE_F16)
    return launch_moments_t<ND, __half>(c, (const __half*)U, M, G, P, k0, cnt, osig, omeas);
  if (ustore == LC2_STORE_BF16)
    return launch_moments_t<ND, __nv_bfloat16>(c, (const __nv_bfloat16*)U, M, G, P, k0, cnt, osig,
                                               omeas);
  return launch_moments_t<ND, float>(c, (const float*)U, M, G, P, k0, cnt, osig, omeas);
}

// z-chunking: enough CTAs to fill the GPU with a small priming overhead
void choose_zchunks(const lc2_context* c, int cnt, lc2::MomentParams& P) {
  if (c->lc2_nd == 2) {
    P.zchunk = 1;
    P.nzchunks = 1;
    return;
  }
  const lc2_geometry& v = c->virt;
  long long tiles = (long long)((v.dim[0] + lc2::kTX - 1) / lc2::kTX) *
                    ((v.dim[1] + lc2::kTY - 1) / lc2::kTY) * cnt;
  long long want = 152LL * 6;
  int nz = (int)std::max<long long>(1, (want + tiles - 1) / tiles);
  int min_chunk = std::max(8, 2 * P.r + 1);
  nz = std::min(nz, std::max(1, v.dim[2] / min_chunk));
  nz = std::min(nz, 65535 / std::max(1, cnt));
  P.zchunk = (v.dim[2] + nz - 1) / nz;
  P.nzchunks = (v.dim[2] + P.zchunk - 1) / P.zchunk;
}

// Generic path: resample -> Sobel -> moments through global scratch. Used for
// a resampled ultrasound (HighResolutionModality: Fixed), for the one-time
// weighting-factor precompute and for the diagnostic field dumps.
int launch_group_generic(lc2_context* c, int k0, int cnt, float* osig, float* omeas) {
  const size_t nv = c->nv;
  lc2::MomentParams P = c->mp;
  choose_zchunks(c, cnt, P);
  float* w = c->d_scratch;  // warped image, slot stride nv
  if (c->cfg.high_res_is_moving) {
    float* g = c->d_scratch + (size_t)c->slots * nv;  // Sobel of it
    LC2_TRY(launch_warp(c, c->warp_nd, c->d_moving, c->cfg.storage, c->cfg.moving, c->d_xf, k0, cnt,
                        w, nv));
    LC2_TRY(launch_sobel(c, w, g, cnt, nv));
    P.u_stride = 0;
    P.m_stride = nv;
    P.g_stride = nv;
    if (c->lc2_nd == 3)
      return launch_moments_nd<3>(c, c->d_static, c->cfg.storage, w, g, P, k0, cnt, osig, omeas);
    return launch_moments_nd<2>(c, c->d_static, c->cfg.storage, w, g, P, k0, cnt, osig, omeas);
  }
  LC2_TRY(launch_warp(c, c->warp_nd, c->d_moving, c->cfg.storage, c->cfg.moving, c->d_xf, k0, cnt,
                      w, nv));
  P.u_stride = nv;
  P.m_stride = 0;
  P.g_stride = 0;
  if (c->lc2_nd == 3)
    return launch_moments_nd<3>(c, w, LC2_STORE_F32, (const float*)c->d_static, c->d_gstatic, P,
                                k0, cnt, osig, omeas);
  return launch_moments_nd<2>(c, w, LC2_STORE_F32, (const float*)c->d_static, c->d_gstatic, P, k0,
                              cnt, osig, omeas);
}

// Output rows per tile of the fused kernels: the option if set; in 2D 0 (per
// launch); in 3D at patch radius 1-4, 24 -- on presampled images of a
// resampled MR/CT (k_fused_pt: batched 4-14 % faster than 16-row tiles from
// 48^3 to 256^3 grids, one transform per call up to 15 %), on a presampled
// ultrasound for grids of 8 M voxels or more (k_fused_fixed_pt: at 256^3
// 1.4 % batched and 5 % per call; on 48^3 to 160^3 grids 16 rows were up to
// 3 % faster), and for a resampled MR/CT resampled in the kernel at radius 3
// or 4 (one 768-thread CTA per SM) -- else 16.
int tile_rows(const lc2_context* c) {
  if (c->tile_rows > 0) return c->tile_rows;
  if (c->lc2_nd == 2) return 0;  // chosen per launch: 32 rows for large launches, else 16
  const int r = c->cfg.patch_size;
  if (c->lc2_nd != 3 || r > 4) return 16;
  if (c->presample) return (c->cfg.high_res_is_moving || c->nv >= 8000000) ? 24 : 16;
  return (c->cfg.high_res_is_moving && r >= 3) ? 24 : 16;
}

// The fused kernel (static ultrasound): one launch for `cnt` transforms.
// The presample buffer holds the images of a group of transforms, at most
// 2 GiB and 64 transforms -- 32 at 256^3. It grows with the batches a context is
// given (a registration's single evaluations hold one slot); growing moves
// it, which drops the captured graphs that name it.
constexpr size_t kPresampleBytes = size_t(2) << 30;
int presample_cap(const lc2_context* c) {
  const size_t per = sizeof(float) * c->nv;
  return (int)std::max<size_t>(1, std::min<size_t>(64, kPresampleBytes / per));
}

int ensure_presample(lc2_context* c, int count) {
  const int want = std::max(1, std::min(count, presample_cap(c)));
  if (c->d_pre && c->pre_slots >= want) return LC2_OK;
  drop_graphs(c);
  dev_free(c->d_pre, c->stream);
  c->d_pre = nullptr;
  c->pre_slots = 0;
  LC2_CUDA(dev_alloc((void**)&c->d_pre, sizeof(float) * c->nv * (size_t)want, c->stream));
  c->pre_slots = want;
  return LC2_OK;
}

// Transforms per presample group for a batch of cnt: at most the buffer's
// slots, chosen so that the moments launches (tiles of ty rows, per_sm CTAs
// resident per SM) fill whole waves of the device, by the launchers' z-split
// cost model -- waves x (chunk + 2R + 3), summed over the groups; ties go to
// larger groups. At 256^3 with 24-row tiles a transform has 88 tiles: groups
// of 19 fill 11 waves of 152 SMs exactly, where groups of 32 leave every 19th
// wave half empty (297 against 304 waves for 512 transforms). Values do not
// depend on the grouping.
// Rows of the grid that 24-row tiles leave over, run as one row of 16-row
// tiles when they fit in it (1-16 rows): at 256 rows, 10 tiles of 24 and one
// of 16 instead of 11 of 24 (3 % of the rows computed outside the grid).
int pt_rest_rows(const lc2_context* c) {
  const int vy = c->virt.dim[1], rest = vy % 24;
  return (vy > 24 && rest > 0 && rest <= 16) ? rest : 0;
}

int presample_group(const lc2_context* c, int cnt, int ty, int per_sm) {
  const int cap = c->pre_slots;
  if (cnt <= cap) return cnt;
  const int vz = c->virt.dim[2], r = c->cfg.patch_size;
  const long long sms = (long long)std::max(1, c->sms) * std::max(1, per_sm);
  const long long ntx = (c->virt.dim[0] + 31) / 32;
  // launches per group: (tiles per transform, weight = tile rows)
  const int rest = ty == 24 ? pt_rest_rows(c) : 0;
  const long long tiles = ntx * ((c->virt.dim[1] - rest + ty - 1) / ty);
  auto launch_cost = [&](long long t, int n) -> long long {
    const int zc = c->zchunk > 0 ? std::min(c->zchunk, vz) : lc2::auto_zchunk(vz, r, t * n, sms);
    const long long chunks = (vz + zc - 1) / zc;
    return (t * n * chunks + sms - 1) / sms * (zc + 2 * r + 3);
  };
  auto cost = [&](int n) -> long long {
    if (n <= 0) return 0;
    return launch_cost(tiles, n) * ty + (rest ? launch_cost(ntx, n) * 16 : 0);
  };
  int best_g = cap;
  long long best = -1;
  for (int g = cap; g >= (cap + 1) / 2; --g) {
    const long long total = (long long)(cnt / g) * cost(g) + cost(cnt % g);
    if (best < 0 || total < best) {
      best = total;
      best_g = g;
    }
  }
  return best_g;
}

int launch_fused(lc2_context* c, int k0, int cnt, float* omeas) {
  c->acc_clean = false;
  if (!c->cfg.high_res_is_moving || !c->d_sigma || !c->d_su)
    return fail(LC2_ERR_INVALID_ARGUMENT, "the static-ultrasound kernel needs a context with "
                "HighResolutionModality: Moving");
  lc2::FusedLaunch L;
  L.mov = c->d_moving;
  L.ust = c->d_static;
  L.sig = c->d_sigma;
  L.su = c->d_su;
  L.P = c->fp;
  L.xf = c->d_xf;
  L.k0 = k0;
  L.cnt = cnt;
  L.acc = c->d_acc;
  L.out_measure = omeas;
  L.nd = c->lc2_nd;
  L.wnd = c->warp_nd;
  L.tile_height = tile_rows(c);
  // a slice's tiles index one grid dimension (<= 65535): 8-row tiles only
  // where they fit (16-row tiles always do, checked when the context is made)
  if (L.tile_height == 8 &&
      (long long)((c->virt.dim[0] + 31) / 32) * ((c->virt.dim[1] + 7) / 8) > 65535)
    L.tile_height = 16;
  L.zchunk = c->zchunk;
  L.pipeline = c->pipeline;
  L.err = c->d_err;
  L.sms = c->sms;
  L.stream = c->stream;
  auto fused = [&]() {
    if (c->cfg.storage == LC2_STORE_F16) return lc2::fused_launch<__half>(L);
    if (c->cfg.storage == LC2_STORE_BF16) return lc2::fused_launch<__nv_bfloat16>(L);
    return lc2::fused_launch<float>(L);
  };
  cudaError_t e;
  if (c->presample && c->lc2_nd == 3 && !c->pipeline) {
    // resample pass, then the fused kernel on the presampled images, in
    // groups of the presample buffer's capacity
    LC2_TRY(ensure_presample(c, cnt));
    auto presample = [&](int j, int n, float* buf) {
      const cudaStream_t st = c->stream;
      if (c->cfg.storage == LC2_STORE_F16)
        return lc2::presample_launch<__half>(c->d_moving, c->fp, c->d_xf, k0 + j, n, buf, st);
      if (c->cfg.storage == LC2_STORE_BF16)
        return lc2::presample_launch<__nv_bfloat16>(c->d_moving, c->fp, c->d_xf, k0 + j, n, buf,
                                                    st);
      return lc2::presample_launch<float>(c->d_moving, c->fp, c->d_xf, k0 + j, n, buf, st);
    };
    auto moments_one = [&](const float* buf) {
      if (c->cfg.storage == LC2_STORE_F16) return lc2::fused_ps_entry<__half>(L, buf);
      if (c->cfg.storage == LC2_STORE_BF16) return lc2::fused_ps_entry<__nv_bfloat16>(L, buf);
      return lc2::fused_ps_entry<float>(L, buf);
    };
    // the moments pass of a group: radius <= 4 with the in-kernel Sobel
    // (k_fused_pt on 24-row tiles, the rows left over by them as one row
    // of k_fused_ps tiles; k_fused_ps on 8/16-row tiles), else k_fused
    auto moments = [&](int j, int n, const float* buf) {
      L.k0 = k0 + j;
      L.cnt = n;
      L.pre = buf;
      if (c->cfg.patch_size > 4) {
        ++c->launches;
        return fused();
      }
      const int rest = L.tile_height == 24 ? pt_rest_rows(c) : 0;
      L.y_off = 0;
      L.y_rows = c->virt.dim[1] - rest;
      cudaError_t err = moments_one(buf);
      ++c->launches;
      if (err == cudaSuccess && rest) {
        L.tile_height = 16;
        L.y_off = c->virt.dim[1] - rest;
        L.y_rows = rest;
        err = moments_one(buf);
        ++c->launches;
        L.tile_height = 24;
      }
      L.y_off = L.y_rows = 0;
      return err;
    };
    // the moments kernel's tile height: 24 (k_fused_pt), 16 (k_fused_ps) or,
    // beyond radius 4, 8 (k_fused on presampled images)
    const int ty = c->cfg.patch_size > 4 ? 8 : (L.tile_height == 24 ? 24 : 16);
    const int group = presample_group(c, cnt, ty, 1);
    for (int j = 0; j < cnt; j += group) {
      const int n = std::min(group, cnt - j);
      {
        TimerScope ts(c, K_WARP);
        e = presample(j, n, c->d_pre);
      }
      ++c->launches;
      LC2_CUDA(e);
      {
        TimerScope ts(c, K_MOMENTS);
        e = moments(j, n, c->d_pre);
      }
      LC2_CUDA(e);
    }
    return LC2_OK;
  }
  {
    TimerScope ts(c, K_MOMENTS);
    e = fused();
  }
  ++c->launches;
  LC2_CUDA(e);
  return LC2_OK;
}

// Normalised mutual information of staged transforms [0, cnt): range,
// joint histogram, entropies; results straight into d_out.
// The fused kernel of a resampled ultrasound: one launch for `cnt` transforms.
int launch_fused_fixed(lc2_context* c, int k0, int cnt) {
  c->acc_clean = false;
  if (c->cfg.high_res_is_moving || !c->d_fq || !c->d_fs || !c->d_fd)
    return fail(LC2_ERR_INVALID_ARGUMENT, "the resampled-ultrasound kernel needs a context with "
                "HighResolutionModality: Fixed");
  lc2::FixedLaunch L;
  L.mov = c->d_moving;
  L.S = lc2::FixedStatic{c->d_fq, reinterpret_cast<const int2*>(c->d_fs), c->d_fd, c->nv,
                         c->d_fsv};
  L.P = c->fp;
  L.xf = c->d_xf;
  L.k0 = k0;
  L.cnt = cnt;
  L.acc = c->d_acc;
  L.nd = c->lc2_nd;
  L.wnd = c->warp_nd;
  L.tile_height = tile_rows(c);
  if (L.tile_height == 8 &&
      (long long)((c->virt.dim[0] + 31) / 32) * ((c->virt.dim[1] + 7) / 8) > 65535)
    L.tile_height = 16;
  L.zchunk = c->zchunk;
  L.sms = c->sms;
  L.stream = c->stream;
  auto fixed = [&]() {
    TimerScope ts(c, K_MOMENTS);
    switch (c->cfg.storage) {
      case LC2_STORE_F16: return lc2::fixed_launch<__half>(L);
      case LC2_STORE_BF16: return lc2::fixed_launch<__nv_bfloat16>(L);
      default: return lc2::fixed_launch<float>(L);
    }
  };
  cudaError_t e;
  if (c->presample && c->lc2_nd == 3) {
    // the ultrasound resampled in a pass of its own, then the moments, in
    // groups of the presample buffer's capacity
    LC2_TRY(ensure_presample(c, cnt));
    // the moments kernel's tile height and CTAs per SM: 24 rows
    // (k_fused_fixed_pt, the rows it leaves over on 16-row tiles), else
    // k_fused_fixed3's 16 or 8
    const int ty = c->cfg.patch_size > 4 || L.tile_height == 8 ? 8
                   : L.tile_height == 24                       ? 24
                                                               : 16;
    const int group =
        presample_group(c, cnt, ty, ty == 24 ? 1 : lc2::fused_min_blocks(3, ty, c->cfg.patch_size));
    const int rest = ty == 24 ? pt_rest_rows(c) : 0;
    for (int j = 0; j < cnt; j += group) {
      const int n = std::min(group, cnt - j);
      {
        TimerScope ts(c, K_WARP);
        if (c->cfg.storage == LC2_STORE_F16)
          e = lc2::presample_launch<__half>(c->d_moving, c->fp, c->d_xf, k0 + j, n, c->d_pre, c->stream);
        else if (c->cfg.storage == LC2_STORE_BF16)
          e = lc2::presample_launch<__nv_bfloat16>(c->d_moving, c->fp, c->d_xf, k0 + j, n, c->d_pre,
                                                   c->stream);
        else
          e = lc2::presample_launch<float>(c->d_moving, c->fp, c->d_xf, k0 + j, n, c->d_pre, c->stream);
      }
      ++c->launches;
      LC2_CUDA(e);
      L.k0 = k0 + j;
      L.cnt = n;
      L.pre = c->d_pre;
      L.y_off = 0;
      L.y_rows = c->virt.dim[1] - rest;
      e = fixed();
      ++c->launches;
      if (e == cudaSuccess && rest) {
        L.tile_height = 16;
        L.y_off = c->virt.dim[1] - rest;
        L.y_rows = rest;
        e = fixed();
        ++c->launches;
        L.tile_height = 24;
      }
      L.y_off = L.y_rows = 0;
      if (e != cudaSuccess)
        return fail(LC2_ERR_CUDA, "fused kernel (resampled ultrasound): %s", cudaGetErrorString(e));
    }
    return LC2_OK;
  }
  e = fixed();
  ++c->launches;
  if (e != cudaSuccess) return fail(LC2_ERR_CUDA, "fused kernel (resampled ultrasound): %s", cudaGetErrorString(e));
  return LC2_OK;
}

int launch_mi(lc2_context* c, int cnt) {
  const lc2_geometry& v = c->virt;
  lc2::MiParams P;
  P.mx = c->cfg.moving.dim[0];
  P.my = c->cfg.moving.dim[1];
  P.mz = c->cfg.moving.dim[2];
  P.vx = v.dim[0];
  P.vy = v.dim[1];
  P.vz = v.dim[2];
  P.warped_is_high_res = c->cfg.high_res_is_moving;
  LC2_CUDA(cudaMemsetAsync(c->d_rmin, 0xff, sizeof(unsigned) * cnt, c->stream));
  LC2_CUDA(cudaMemsetAsync(c->d_rmax, 0x00, sizeof(unsigned) * cnt, c->stream));
  LC2_CUDA(cudaMemsetAsync(c->d_hist, 0, sizeof(unsigned) * lc2::kMiHist * (size_t)cnt, c->stream));
  dim3 block(32, 8, 1);
  const long long tiles = (long long)((v.dim[0] + 31) / 32) * ((v.dim[1] + 7) / 8);
  // slices per CTA: up to kMiChunk, fewer where the launch would otherwise
  // have under eight CTAs per SM (one small transform)
  const long long work = tiles * v.dim[2] * (long long)std::min(cnt, 65535);
  P.zchunk = (int)std::max(1LL, std::min<long long>(lc2::kMiChunk, work / (8LL * c->sms)));
  const int chunks = (v.dim[2] + P.zchunk - 1) / P.zchunk;
  // the histogram's shared table pays where a CTA's voxels are a small part
  // of the grid (at most 0.5 %: neighbouring voxels then share few distinct
  // bins): 256^3 2150 -> 4640 evals/s; at 96^3 (2 %) it crowded and lost
  P.table = P.zchunk >= 16 && (long long)c->nv >= 200LL * 256 * P.zchunk;
  // one launch covers at most 65535 transforms (grid z / y limit)
  for (int k0 = 0; k0 < cnt; k0 += 65535) {
    const int n = std::min(65535, cnt - k0);
    dim3 grid((unsigned)tiles, chunks, n);
    TimerScope ts(c, K_MOMENTS);
    const int st = c->cfg.storage;
    if (st == LC2_STORE_F16) {
      lc2::k_mi_range<__half><<<grid, block, 0, c->stream>>>((const __half*)c->d_moving, P, c->d_xf, k0, c->d_rmin, c->d_rmax);
      lc2::k_mi_hist<__half><<<grid, block, 0, c->stream>>>((const __half*)c->d_moving, P, c->d_xf, k0, c->d_sbin, c->d_rmin, c->d_rmax, c->d_hist);
    } else if (st == LC2_STORE_BF16) {
      lc2::k_mi_range<__nv_bfloat16><<<grid, block, 0, c->stream>>>((const __nv_bfloat16*)c->d_moving, P, c->d_xf, k0, c->d_rmin, c->d_rmax);
      lc2::k_mi_hist<__nv_bfloat16><<<grid, block, 0, c->stream>>>((const __nv_bfloat16*)c->d_moving, P, c->d_xf, k0, c->d_sbin, c->d_rmin, c->d_rmax, c->d_hist);
    } else {
      lc2::k_mi_range<float><<<grid, block, 0, c->stream>>>((const float*)c->d_moving, P, c->d_xf, k0, c->d_rmin, c->d_rmax);
      lc2::k_mi_hist<float><<<grid, block, 0, c->stream>>>((const float*)c->d_moving, P, c->d_xf, k0, c->d_sbin, c->d_rmin, c->d_rmax, c->d_hist);
    }
    lc2::k_mi_part<<<dim3(lc2::kMiParts, n), 256, 0, c->stream>>>(c->d_hist, k0,
                                                                  P.warped_is_high_res, c->d_mipart);
    c->launches += 3;
    LC2_CUDA(cudaGetLastError());
  }
  lc2::k_mi_nmi<<<(cnt + 127) / 128, 128, 0, c->stream>>>(c->d_mipart, cnt, c->h_static,
                                                          (double)c->nv, c->d_out);
  ++c->launches;
  LC2_CUDA(cudaGetLastError());
  return LC2_OK;
}

// Enqueue the evaluation of staged transforms [k0, k0 + cnt).
int launch_group(lc2_context* c, int k0, int cnt) {
  if (c->generic) return launch_group_generic(c, k0, cnt, nullptr, nullptr);
  if (c->cfg.high_res_is_moving) return launch_fused(c, k0, cnt, nullptr);
  return launch_fused_fixed(c, k0, cnt);
}

int launch_finalize(lc2_context* c, int count) {
  lc2::k_finalize<<<(count + 127) / 128, 128, 0, c->stream>>>(
      c->d_acc, count, c->d_out, c->cfg.high_res_is_moving ? c->sigma_sum : -1LL);
  ++c->launches;
  LC2_CUDA(cudaGetLastError());
  return LC2_OK;
}

int matrix_floats(const lc2_context* c) { return c->warp_nd == 2 ? 9 : 16; }

// A wait of the warp-specialised kernel ran past its deadline (the flag is
// copied to h_err with the results): the values of that launch are invalid.
int check_pipeline(lc2_context* c) {
  if (*c->h_err == 0) return LC2_OK;
  *c->h_err = 0;
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  return fail(LC2_ERR_TIMEOUT, "pipelined kernel: a producer/consumer wait timed out");
}

int check_ctx(const lc2_context* c) {
  if (!c) return fail(LC2_ERR_INVALID_ARGUMENT, "null context");
  if (!c->ready) return fail(LC2_ERR_NOT_READY, "images not set (call lc2_set_images first)");
  return LC2_OK;
}

}  // namespace

extern "C" {

const char* lc2_last_error(void) { return g_err.c_str(); }

const char* lc2_version(void) { return "lc2-gb300 0.1 (sm_103a)"; }

}  // extern "C"

namespace {

// Host-side plan of a context: validation, virtual grid, sizes, patch and
// fixed-point bits, scratch slots. No device work.
int plan_context(const lc2_config* cfg, lc2_context* c) {
  if (cfg->mode < LC2_MODE_2D || cfg->mode > LC2_MODE_2DTO3D)
    return fail(LC2_ERR_INVALID_ARGUMENT, "unknown mode %d", cfg->mode);
  if (cfg->storage < LC2_STORE_F32 || cfg->storage > LC2_STORE_BF16)
    return fail(LC2_ERR_INVALID_ARGUMENT, "unknown storage %d", cfg->storage);
  if (!finite_geom(cfg->fixed) || !finite_geom(cfg->moving))
    return fail(LC2_ERR_INVALID_ARGUMENT, "geometry needs dims >= 1, finite spacing > 0 and origin");
  for (int a = 0; a < 3; ++a)
    if (!std::isfinite(cfg->virtual_spacing[a]) || !(cfg->virtual_spacing[a] > 0.0f))
      if (!(cfg->mode == LC2_MODE_2D && a == 2))
        return fail(LC2_ERR_INVALID_ARGUMENT, "virtual spacing must be finite and > 0");
  c->cfg = *cfg;
  c->warp_nd = (cfg->mode == LC2_MODE_2D) ? 2 : 3;
  c->lc2_nd = (cfg->mode == LC2_MODE_3D) ? 3 : 2;
  if (cfg->mode == LC2_MODE_2D) {
    c->cfg.fixed.dim[2] = 1;
    c->cfg.moving.dim[2] = 1;
  }
  // virtual grid: fixed origin, dims ceil(dimF * spF / spV) in float
  // (src/Interpolator/interpolator.cu:337-339, :1093-1094, :1603-1605)
  for (int a = 0; a < 3; ++a) {
    c->virt.origin[a] = c->cfg.fixed.origin[a];
    c->virt.spacing[a] = cfg->virtual_spacing[a];
    if (a < c->warp_nd) {
      float ext = (float)c->cfg.fixed.dim[a] * c->cfg.fixed.spacing[a];
      const double d = std::ceil((double)(ext / cfg->virtual_spacing[a]));
      if (!(d <= (double)(1 << 20)))
        return fail(LC2_ERR_UNSUPPORTED,
                    "virtual grid axis %d would have %.0f voxels (at most 2^20)", a, d);
      c->virt.dim[a] = (int)d;
    } else {
      c->virt.dim[a] = 1;
      c->virt.spacing[a] = 1.0f;
      c->virt.origin[a] = 0.0f;
    }
  }
  int r = cfg->patch_size;
  int rmax = (c->lc2_nd == 3) ? 6 : 12;
  c->mi = (r == 0);
  if (c->mi && cfg->mode != LC2_MODE_3D)
    return fail(LC2_ERR_UNSUPPORTED,
                "PatchSize 0 (normalised mutual information) is a 3D similarity");
  if (!c->mi && (r < 1 || r > rmax))
    return fail(LC2_ERR_UNSUPPORTED, "patch size %d outside [1, %d] for %dD patches", r, rmax,
                c->lc2_nd);
  if (cfg->mode == LC2_MODE_2DTO3D && c->virt.dim[2] != 1)
    return fail(LC2_ERR_INVALID_ARGUMENT,
                "2D-to-3D needs a single virtual slice (fixed z extent <= virtual z spacing)");
  c->nv = (size_t)c->virt.dim[0] * c->virt.dim[1] * c->virt.dim[2];
  // 32-bit in-slice indices in the kernels; a slice's 32 x 16 tiles index
  // one grid dimension of the fused launch (at most 65535)
  if ((size_t)c->virt.dim[0] * c->virt.dim[1] >= (size_t)1 << 31 ||
      (size_t)((c->virt.dim[0] + 31) / 32) * ((c->virt.dim[1] + 15) / 16) > 65535)
    return fail(LC2_ERR_UNSUPPORTED, "virtual slice of %d x %d voxels is too large (at most "
                "65535 tiles of 32 x 16)", c->virt.dim[0], c->virt.dim[1]);
  if (c->lc2_nd == 3 && r > 4 &&
      (size_t)((c->virt.dim[0] + 31) / 32) * ((c->virt.dim[1] + 7) / 8) > 65535)
    return fail(LC2_ERR_UNSUPPORTED, "3D patches of radius > 4 run 32 x 8 tiles: a virtual slice "
                "of %d x %d voxels needs more than 65535", c->virt.dim[0], c->virt.dim[1]);
  c->nf = (size_t)c->cfg.fixed.dim[0] * c->cfg.fixed.dim[1] * c->cfg.fixed.dim[2];
  c->nm = (size_t)c->cfg.moving.dim[0] * c->cfg.moving.dim[1] * c->cfg.moving.dim[2];
  if (c->nm >= (size_t)1 << 31 || c->nf >= (size_t)1 << 31)
    return fail(LC2_ERR_UNSUPPORTED, "images are limited to 2^31 - 1 voxels (32-bit gather indices)");
  c->n = (2 * r + 1) * (2 * r + 1) * (c->lc2_nd == 3 ? (2 * r + 1) : 1);
  // fixed-point bits: n * 2^(b+1) <= 2^31 (int32 first-order sums with one
  // bit of headroom; then n^2 2^(2b) <= 2^60 for the centred int64 sums)
  int b = 0;
  while (b < 21 && ((long long)c->n << (b + 2)) <= (1LL << 31)) ++b;
  c->qbits = b;
  // scratch slots of the generic path: warped image (+ its Sobel when the
  // moving image is the high-resolution one). Both fused paths keep nothing
  // per transform, so one slot (for the field dumps and LC2_OPTION_GENERIC)
  // unless max_batch asks for more generic-path batching.
  c->per_slot = c->nv * sizeof(float) * (cfg->high_res_is_moving ? 2 : 1);
  long long slots = cfg->max_batch > 0 ? cfg->max_batch : 1;
  slots = std::min<long long>(slots, 1024);
  slots = std::min<long long>(slots, 65535 / c->virt.dim[2]);
  c->slots = (int)std::max<long long>(1, slots);
  // 3D contexts of a resampled MR/CT resample in a pass of their own
  c->presample = (c->lc2_nd == 3 && !c->mi) ? 1 : 0;
  return LC2_OK;
}

// Device bytes a context of this plan holds, and the largest temporary
// allocation of lc2_set_images on top of them.
void context_bytes(const lc2_context* c, size_t* held, size_t* peak_extra) {
  const size_t es = elem_size(c->cfg.storage);
  const bool hrm = c->cfg.high_res_is_moving != 0;
  size_t h = c->per_slot * c->slots;
  h += c->nm * es;                             // moving
  h += c->nv * (hrm ? es : sizeof(float));     // static image on the virtual grid
  if (!hrm) h += c->nv * sizeof(float);        // its Sobel
  if (hrm && !c->mi) h += c->nv * (sizeof(float) + sizeof(int));  // weighting factors, S_U
  if (!hrm && !c->mi)  // static sums and solve factors
    h += c->nv * (4 * sizeof(int) + 3 * sizeof(long long) + sizeof(float4));
  if (c->mi)
    h += c->nv + 64 * (sizeof(unsigned) * (lc2::kMiHist + 2) + sizeof(double) * 2 * lc2::kMiParts);
  h += 64 * (sizeof(lc2::Xform) + 2 * sizeof(unsigned long long) + sizeof(double));
  if (c->presample)  // the presample buffer at its largest
    h += sizeof(float) * c->nv * (size_t)presample_cap(c);
  *held = h;
  *peak_extra = std::max(c->nm, c->nf) * sizeof(float);
  if (!hrm && !c->mi)  // temporaries of the static sums
    *peak_extra = std::max(*peak_extra, c->nv * (sizeof(int) + sizeof(long long)));
}

int create_context(const lc2_config* cfg, bool own_moving, lc2_context** out) {
  if (!cfg || !out) return fail(LC2_ERR_INVALID_ARGUMENT, "null config or output pointer");
  *out = nullptr;
  lc2_context* c = new (std::nothrow) lc2_context();
  if (!c) return fail(LC2_ERR_OUT_OF_MEMORY, "host allocation failed");
  int st = plan_context(cfg, c);
  if (st == LC2_OK) st = select_device(c);
  if (st != LC2_OK) {
    delete c;
    return st;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return fail(LC2_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  if (cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, cfg->device) != cudaSuccess ||
      c->sms < 1)
    c->sms = 152;
  c->stream = c->own_stream;
  e = dev_alloc((void**)&c->d_scratch, c->per_slot * c->slots, c->stream);
  c->owns_moving = own_moving;
  if (e == cudaSuccess && own_moving) e = dev_alloc(&c->d_moving, c->nm * elem_size(cfg->storage), c->stream);
  if (e == cudaSuccess)
    e = dev_alloc(&c->d_static,
                   c->nv * (cfg->high_res_is_moving ? elem_size(cfg->storage) : sizeof(float)), c->stream);
  if (e == cudaSuccess && !cfg->high_res_is_moving)
    e = dev_alloc((void**)&c->d_gstatic, c->nv * sizeof(float), c->stream);
  if (e == cudaSuccess && cfg->high_res_is_moving && !c->mi)
    e = dev_alloc((void**)&c->d_sigma, c->nv * sizeof(float), c->stream);
  if (e == cudaSuccess && cfg->high_res_is_moving && !c->mi)
    e = dev_alloc((void**)&c->d_su, c->nv * sizeof(int), c->stream);
  if (e == cudaSuccess && c->mi) e = dev_alloc((void**)&c->d_sbin, c->nv, c->stream);
  if (e == cudaSuccess && !cfg->high_res_is_moving && !c->mi)
    e = dev_alloc((void**)&c->d_fq, 2 * c->nv * sizeof(int), c->stream);
  if (e == cudaSuccess && !cfg->high_res_is_moving && !c->mi)
    e = dev_alloc((void**)&c->d_fs, 2 * c->nv * sizeof(int), c->stream);
  if (e == cudaSuccess && !cfg->high_res_is_moving && !c->mi)
    e = dev_alloc((void**)&c->d_fd, 3 * c->nv * sizeof(long long), c->stream);
  if (e == cudaSuccess && !cfg->high_res_is_moving && !c->mi)
    e = dev_alloc((void**)&c->d_fsv, c->nv * sizeof(float4), c->stream);
  if (e == cudaSuccess) e = dev_alloc((void**)&c->d_err, sizeof(int), c->stream);
  if (e == cudaSuccess) e = host_alloc((void**)&c->h_err, sizeof(int));
  if (e == cudaSuccess) *c->h_err = 0;  // pinned buffers come from a reuse cache
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  if (e != cudaSuccess) {
    lc2_destroy(c);
    return fail(LC2_ERR_OUT_OF_MEMORY, "device allocation: %s", cudaGetErrorString(e));
  }
  st = ensure_capacity(c, 64);
  // the stream-ordered allocations are complete before any other stream uses them
  if (st == LC2_OK && cudaStreamSynchronize(c->stream) != cudaSuccess)
    st = fail(LC2_ERR_CUDA, "context allocation: %s", cudaGetErrorString(cudaGetLastError()));
  if (st != LC2_OK) {
    std::string msg = g_err;
    lc2_destroy(c);
    g_err = msg;
    return st;
  }
  *out = c;
  return LC2_OK;
}

}  // namespace

extern "C" {

int lc2_create(const lc2_config* cfg, lc2_context** out) {
  g_err.clear();
  return create_context(cfg, true, out);
}

int lc2_context_bytes(const lc2_config* cfg, size_t* held, size_t* peak) {
  g_err.clear();
  if (!cfg || !held) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  lc2_context c;
  LC2_TRY(plan_context(cfg, &c));
  size_t extra = 0;
  context_bytes(&c, held, &extra);
  if (peak) *peak = *held + extra;
  return LC2_OK;
}

int lc2_destroy(lc2_context* c) {
  if (!c) return LC2_OK;
  select_device(c);
  if (c->stream) cudaStreamSynchronize(c->stream);
  drop_graphs(c);
  cudaStream_t fs = c->own_stream;  // frees are ordered on the context's own stream
  if (c->owns_moving) dev_free(c->d_moving, fs);
  dev_free(c->d_static, fs);
  dev_free(c->d_gstatic, fs);
  dev_free(c->d_sigma, fs);
  dev_free(c->d_su, fs);
  dev_free(c->d_pre, fs);
  dev_free(c->d_fq, fs);
  dev_free(c->d_fs, fs);
  dev_free(c->d_fd, fs);
  dev_free(c->d_fsv, fs);
  dev_free(c->d_err, fs);
  dev_free(c->d_scratch, fs);
  dev_free(c->d_sbin, fs);
  dev_free(c->d_hist, fs);
  dev_free(c->d_mipart, fs);
  dev_free(c->d_rmin, fs);
  dev_free(c->d_rmax, fs);
  dev_free(c->d_xf, fs);
  dev_free(c->d_acc, fs);
  dev_free(c->d_out, fs);
  if (fs) cudaStreamSynchronize(fs);
  host_free(c->h_err);
  host_free(c->h_xf);
  host_free(c->h_out);
  for (auto& t : c->timed) {
    cudaEventDestroy(t.a);
    cudaEventDestroy(t.b);
  }
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
  return LC2_OK;
}

int lc2_get_config(const lc2_context* c, lc2_config* out) {
  if (!c || !out) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  *out = c->cfg;
  return LC2_OK;
}

int lc2_virtual_dims(const lc2_context* c, int dims[3]) {
  if (!c || !dims) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  for (int a = 0; a < 3; ++a) dims[a] = c->virt.dim[a];
  return LC2_OK;
}

void* lc2_get_stream(const lc2_context* c) { return c ? (void*)c->stream : nullptr; }

int lc2_set_stream(lc2_context* c, void* stream) {
  if (!c) return fail(LC2_ERR_INVALID_ARGUMENT, "null context");
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return LC2_OK;
}

long long lc2_launch_count(const lc2_context* c) { return c ? c->launches : 0; }

int lc2_debug_fail_allocation(long long k) {
  g_fail_countdown.store(k > 0 ? k : 0);
  return LC2_OK;
}

int lc2_debug_device_bytes(size_t* live_bytes, long long* live_allocations) {
  if (!live_bytes || !live_allocations) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  std::lock_guard<std::mutex> lk(g_live_mu);
  *live_bytes = g_live_bytes;
  *live_allocations = (long long)g_live.size();
  return LC2_OK;
}

int lc2_set_option(lc2_context* c, int option, int value) {
  if (!c) return fail(LC2_ERR_INVALID_ARGUMENT, "null context");
  if (option == LC2_OPTION_TILE_ROWS) {
    if (value != 0 && value != 8 && value != 16 && value != 24 && value != 32)
      return fail(LC2_ERR_INVALID_ARGUMENT, "tile rows must be 0, 8, 16, 24 or 32");
    if (value == 32 && c->lc2_nd == 3)
      return fail(LC2_ERR_UNSUPPORTED, "32-row tiles exist for 2D and 2D-to-3D contexts only");
    if (value >= 16 && c->lc2_nd == 3 && c->cfg.patch_size > 4)
      return fail(LC2_ERR_UNSUPPORTED, "%d-row tiles need a 3D patch radius <= 4", value);
    c->tile_rows = value;
    drop_graphs(c);
    return LC2_OK;
  }
  if (option == LC2_OPTION_GENERIC) {
    if (value != 0 && value != 1) return fail(LC2_ERR_INVALID_ARGUMENT, "generic must be 0 or 1");
    if (value == 1 && c->mi)
      return fail(LC2_ERR_UNSUPPORTED, "mutual information has no generic LC2 path");
    c->generic = value;
    drop_graphs(c);
    return LC2_OK;
  }
  if (option == LC2_OPTION_ZCHUNK) {
    if (value < 0) return fail(LC2_ERR_INVALID_ARGUMENT, "z chunk must be >= 0");
    c->zchunk = value;
    drop_graphs(c);
    return LC2_OK;
  }
  if (option == LC2_OPTION_STREAM_PRIORITY) {
    // recreate the context's own stream with this priority (clamped to the
    // device's range); a caller-set stream is left alone
    LC2_TRY(select_device(c));
    int least = 0, greatest = 0;
    LC2_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int prio = std::max(greatest, std::min(least, value));
    cudaStream_t ns = nullptr;
    LC2_CUDA(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, prio));
    LC2_CUDA(cudaStreamSynchronize(c->own_stream));
    drop_graphs(c);
    const bool own = (c->stream == c->own_stream);
    cudaStreamDestroy(c->own_stream);
    c->own_stream = ns;
    if (own) c->stream = ns;
    return LC2_OK;
  }
  if (option == LC2_OPTION_PIPELINE) {
    c->pipeline = value != 0;
    drop_graphs(c);
    return LC2_OK;
  }
  if (option == LC2_OPTION_PRESAMPLE) {
    if (value != 0 && value != 1) return fail(LC2_ERR_INVALID_ARGUMENT, "presample must be 0 or 1");
    if (value != 0 && (c->lc2_nd != 3 || c->mi))
      return fail(LC2_ERR_UNSUPPORTED, "presampling exists for 3D LC2 contexts");
    c->presample = value;
    drop_graphs(c);
    return LC2_OK;
  }
  if (option == LC2_OPTION_GRAPHS) {
    c->use_graphs = value != 0;
    if (!c->use_graphs) drop_graphs(c);
    return LC2_OK;
  }
  return fail(LC2_ERR_INVALID_ARGUMENT, "unknown option %d", option);
}

int lc2_wait_probe(lc2_context* c) {
  g_err.clear();
  LC2_TRY(check_ctx(c));
  LC2_TRY(select_device(c));
  LC2_CUDA(cudaStreamSynchronize(c->stream));  // no earlier report pending
  LC2_TRY(check_pipeline(c));
  LC2_CUDA(lc2::wait_probe_launch(c->d_err, c->stream));
  LC2_CUDA(cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  return check_pipeline(c);
}

int lc2_enable_kernel_timing(lc2_context* c, int on) {
  if (!c) return fail(LC2_ERR_INVALID_ARGUMENT, "null context");
  c->timing = on != 0;
  return LC2_OK;
}

int lc2_kernel_times(lc2_context* c, double ms[3], long long counts[3]) {
  if (!c || !ms || !counts) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  LC2_TRY(select_device(c));
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < K_KINDS; ++k) {
    ms[k] = 0.0;
    counts[k] = 0;
  }
  for (auto& t : c->timed) {
    float e = 0.0f;
    if (cudaEventElapsedTime(&e, t.a, t.b) == cudaSuccess) {
      ms[t.kind] += e;
      counts[t.kind] += 1;
    }
    cudaEventDestroy(t.a);
    cudaEventDestroy(t.b);
  }
  c->timed.clear();
  return LC2_OK;
}

}  // extern "C"

namespace {

// Largest |value| of a host image; LC2_ERR_INVALID_ARGUMENT on NaN/Inf.
int image_absmax(const float* img, size_t n, const char* what, float* out) {
  float mx = 0.0f;
  for (size_t i = 0; i < n; ++i) {
    if (!std::isfinite(img[i])) return fail(LC2_ERR_INVALID_ARGUMENT, "%s image has NaN/Inf at %zu", what, i);
    mx = std::max(mx, std::fabs(img[i]));
  }
  *out = mx;
  return LC2_OK;
}

// Largest |value| of a device float image (as float bits, atomicMax on the
// non-negative bit patterns orders them like the values) and a flag for
// NaN/Inf anywhere in it. out[0] and out[1] must start at zero.
__global__ void k_absmax_flag(const float* __restrict__ a, size_t n, unsigned int* __restrict__ out) {
  unsigned int m = 0, bad = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float v = a[i];
    if (!isfinite(v)) bad = 1;
    m = max(m, __float_as_uint(fabsf(v)));
  }
  for (int o = 16; o > 0; o >>= 1) {
    m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    bad |= __shfl_down_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, m);
    if (bad) atomicOr(out + 1, 1u);
  }
}

// Host float image -> device buffer of the storage type (synchronous). A
// device-resident source (lc2_set_images_device) is converted in place of
// the staging copy.
int upload_image(lc2_context* c, const float* host, size_t n, void* dst, int storage,
                 bool on_device = false) {
  if (on_device) {
    LC2_TRY(convert_to_storage(c, host, dst, n, storage));
    LC2_CUDA(cudaStreamSynchronize(c->stream));
    return LC2_OK;
  }
  float* tmp = nullptr;
  LC2_CUDA(dev_alloc((void**)&tmp, sizeof(float) * n, c->stream));
  struct Free {
    float* p;
    cudaStream_t st;
    ~Free() { dev_free(p, st); }
  } guard{tmp, c->stream};
  LC2_CUDA(cudaMemcpyAsync(tmp, host, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
  LC2_TRY(convert_to_storage(c, tmp, dst, n, storage));
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  return LC2_OK;
}

// Everything that depends on the fixed image, given the moving image's
// largest |value| (its scale enters the fixed-point parameters): the fixed
// image on the virtual grid, the fixed-point parameters and, for a static
// ultrasound, the weighting factors and their sum.
// Window sums of the quantised static ultrasound per voxel (the S_U of the
// fused kernels), by exact separable passes through scratch slot 0.
int static_window_sum(lc2_context* c) {
  const lc2_geometry& v = c->virt;
  const size_t nv = c->nv;
  int* ta = reinterpret_cast<int*>(c->d_scratch);
  int* tb = ta + nv;  // the slot holds two planes of nv floats
  const int blocks = (int)std::min<size_t>((nv + 255) / 256, 152 * 16);
  const int st = c->cfg.storage;
  if (st == LC2_STORE_F16)
    lc2::k_quant_static<__half><<<blocks, 256, 0, c->stream>>>((const __half*)c->d_static, nv, c->fp.qu, ta);
  else if (st == LC2_STORE_BF16)
    lc2::k_quant_static<__nv_bfloat16><<<blocks, 256, 0, c->stream>>>((const __nv_bfloat16*)c->d_static, nv, c->fp.qu, ta);
  else
    lc2::k_quant_static<float><<<blocks, 256, 0, c->stream>>>((const float*)c->d_static, nv, c->fp.qu, ta);
  const int nx = v.dim[0], ny = v.dim[1], nz = v.dim[2], r = c->cfg.patch_size;
  auto pass = [&](const int* in, int* out, int axis, long long lines) {
    lc2::k_box_line<int><<<(unsigned)((lines + 127) / 128), 128, 0, c->stream>>>(in, out, nx, ny, nz,
                                                                            axis, r);
  };
  pass(ta, tb, 0, (long long)ny * nz);
  if (c->lc2_nd == 3) {
    pass(tb, ta, 1, (long long)nx * nz);
    pass(ta, c->d_su, 2, (long long)nx * ny);
  } else {
    pass(tb, c->d_su, 1, (long long)nx * nz);
  }
  c->launches += (c->lc2_nd == 3) ? 4 : 3;
  LC2_CUDA(cudaGetLastError());
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  return LC2_OK;
}

// Resampled ultrasound: quantised static image and Sobel, their exact window
// sums and centred sums, once per context (the fields k_fused_fixed* read).
int fixed_static_sums(lc2_context* c) {
  const lc2_geometry& v = c->virt;
  const size_t nv = c->nv;
  const int nx = v.dim[0], ny = v.dim[1], nz = v.dim[2], r = c->cfg.patch_size;
  int* ti = nullptr;
  long long* tl = nullptr;
  LC2_CUDA(dev_alloc((void**)&ti, nv * sizeof(int), c->stream));
  struct Free {
    void* p;
    cudaStream_t st;
    ~Free() { dev_free(p, st); }
  } g1{ti, c->stream};
  LC2_CUDA(dev_alloc((void**)&tl, nv * sizeof(long long), c->stream));
  Free g2{tl, c->stream};
  const int blocks = (int)std::min<size_t>((nv + 255) / 256, 152 * 16);
  lc2::k_fixed_quant<<<blocks, 256, 0, c->stream>>>((const float*)c->d_static, c->d_gstatic, nv,
                                                    c->fp.qm, c->fp.qg, c->d_fq, c->d_fd);
  auto pass = [&](auto* in, auto* out, int axis) {
    const long long lines = axis == 0 ? (long long)ny * nz : axis == 1 ? (long long)nx * nz
                                                                       : (long long)nx * ny;
    lc2::k_box_line<<<(unsigned)((lines + 127) / 128), 128, 0, c->stream>>>(in, out, nx, ny, nz,
                                                                            axis, r);
    ++c->launches;
  };
  // S_M, S_G: q -> s through x, y (, z) passes
  for (int f = 0; f < 2; ++f) {
    int* q = c->d_fq + f * nv;
    int* o = c->d_fs + f * nv;
    if (c->lc2_nd == 3) {
      pass(q, o, 0);
      pass(o, ti, 1);
      pass(ti, o, 2);
    } else {
      pass(q, ti, 0);
      pass(ti, o, 1);
    }
  }
  // S_MM, S_GG, S_MG in place in d
  for (int f = 0; f < 3; ++f) {
    long long* p = c->d_fd + f * nv;
    pass(p, tl, 0);
    pass(tl, p, 1);
    if (c->lc2_nd == 3) {
      pass(p, tl, 2);
      LC2_CUDA(cudaMemcpyAsync(p, tl, nv * sizeof(long long), cudaMemcpyDeviceToDevice, c->stream));
    }
  }
  lc2::k_fixed_centre<<<blocks, 256, 0, c->stream>>>(c->d_fs, c->d_fd, nv, (long long)c->n);
  // the solve factors, and (S_M, S_G) interleaved per voxel through the
  // 8-byte temporary into the sums' own buffer
  lc2::k_fixed_solve_static<<<blocks, 256, 0, c->stream>>>(c->d_fs, c->d_fd, nv, c->fp.thr_m,
                                                           c->fp.thr_g,
                                                           reinterpret_cast<int2*>(tl), c->d_fsv);
  LC2_CUDA(cudaMemcpyAsync(c->d_fs, tl, nv * sizeof(int2), cudaMemcpyDeviceToDevice, c->stream));
  c->launches += 3;
  LC2_CUDA(cudaGetLastError());
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  return LC2_OK;
}

// Normalised mutual information: bins of the static image on the virtual
// grid (the values the kernels read) between its minimum and maximum, with the
// float operations of lc2::mi_bin, and its entropy.
int set_static_bins(lc2_context* c) {
  const size_t nv = c->nv;
  std::vector<float> host(nv);
  const int ustore = c->cfg.high_res_is_moving ? c->cfg.storage : LC2_STORE_F32;
  float* tmp = c->d_scratch;  // slot 0
  LC2_TRY(to_float(c, c->d_static, tmp, nv, ustore));
  LC2_CUDA(cudaMemcpyAsync(host.data(), tmp, sizeof(float) * nv, cudaMemcpyDeviceToHost, c->stream));
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  float lo = host[0], hi = host[0];
  for (float v : host) {
    lo = std::min(lo, v);
    hi = std::max(hi, v);
  }
  const float sc = lc2::mi_scale(lo, hi);
  std::vector<unsigned char> bins(nv);
  std::vector<long long> counts(lc2::kMiBins, 0);
  for (size_t i = 0; i < nv; ++i) {
    const float t = (host[i] - lo) * sc;
    int b = (int)std::round(t);
    b = std::min(std::max(b, 0), lc2::kMiBins - 1);
    bins[i] = (unsigned char)b;
    ++counts[b];
  }
  double s = 0.0;
  for (long long n : counts)
    if (n) s += (double)n * std::log((double)n);
  c->h_static = std::log((double)nv) - s / (double)nv;
  LC2_CUDA(cudaMemcpyAsync(c->d_sbin, bins.data(), nv, cudaMemcpyHostToDevice, c->stream));
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  c->ready = true;
  return LC2_OK;
}

// fmax: the fixed image's largest |value| (image_absmax).
int set_fixed(lc2_context* c, const float* fixed, float fmax, float mmax) {
  const int storage = c->cfg.storage;
  struct Free {
    float* p;
    cudaStream_t st;
    ~Free() { dev_free(p, st); }
  };
  // fixed volume resampled onto the virtual grid through the identity
  // (VirtualToFixed, src/Interpolator/interpolator.cu:526-528)
  float* ffix = nullptr;
  LC2_CUDA(dev_alloc((void**)&ffix, sizeof(float) * c->nf, c->stream));
  Free guard2{ffix, c->stream};
  // cudaMemcpyDefault: the fixed image is host memory (lc2_set_images) or
  // device memory (lc2_set_images_device)
  LC2_CUDA(cudaMemcpyAsync(ffix, fixed, sizeof(float) * c->nf, cudaMemcpyDefault, c->stream));
  lc2::Xform id{};
  {
    float ident[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    float ident2[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    build_xform(c->warp_nd, c->virt, c->cfg.fixed, c->warp_nd == 2 ? ident2 : ident, &id);
  }
  c->h_xf[0] = id;
  LC2_CUDA(cudaMemcpyAsync(c->d_xf, c->h_xf, sizeof(lc2::Xform), cudaMemcpyHostToDevice, c->stream));
  float* vfix = c->d_scratch;  // slot 0 as temporary
  LC2_TRY(launch_warp(c, c->warp_nd, ffix, LC2_STORE_F32, c->cfg.fixed, c->d_xf, 0, 1, vfix, c->nv));
  if (c->cfg.high_res_is_moving) {
    LC2_TRY(convert_to_storage(c, vfix, c->d_static, c->nv, storage));
  } else {
    LC2_CUDA(cudaMemcpyAsync(c->d_static, vfix, sizeof(float) * c->nv, cudaMemcpyDeviceToDevice,
                             c->stream));
    LC2_TRY(launch_sobel(c, (const float*)c->d_static, c->d_gstatic, 1, 0));
  }
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  if (c->mi) return set_static_bins(c);

  // fixed-point scales and thresholds
  const float tiny = 1e-30f;
  float umax = c->cfg.high_res_is_moving ? fmax : mmax;
  float hmax = c->cfg.high_res_is_moving ? mmax : fmax;
  // Sobel magnitude bound: sum |taps| per component (8 in 2D, 32 in 3D)
  float gmax = (c->lc2_nd == 3) ? std::sqrt(3.0f) * 32.0f * hmax : std::sqrt(2.0f) * 8.0f * hmax;
  c->vmax_u = std::max(umax, tiny);
  c->vmax_m = std::max(hmax, tiny);
  c->vmax_g = std::max(gmax, tiny);
  const float two_b = std::ldexp(1.0f, c->qbits);
  lc2::MomentParams& P = c->mp;
  P.vx = c->virt.dim[0];
  P.vy = c->virt.dim[1];
  P.vz = c->virt.dim[2];
  P.r = c->cfg.patch_size;
  P.n = c->n;
  P.qu = two_b / c->vmax_u;
  P.qm = two_b / c->vmax_m;
  P.qg = two_b / c->vmax_g;
  const long double n = c->n;
  P.thr_var = floor_clamp(1e-6L * n * (n - 1) * (long double)P.qu * (long double)P.qu);
  P.thr_m = floor_clamp(1e-12L * n * (n - 1) * (long double)P.qm * (long double)P.qm);
  P.thr_g = floor_clamp(1e-12L * n * (n - 1) * (long double)P.qg * (long double)P.qg);
  P.sig_scale = (float)(1.0L / ((long double)P.qu * std::sqrt(n * (n - 1))));
  P.sum_scale = std::ldexp(1.0f, 29) / c->vmax_u;
  // fused-kernel parameters
  lc2::FusedParams& F = c->fp;
  F.vx = P.vx;
  F.vy = P.vy;
  F.vz = P.vz;
  F.mx = c->cfg.moving.dim[0];
  F.my = c->cfg.moving.dim[1];
  F.mz = c->cfg.moving.dim[2];
  F.r = P.r;
  F.n = P.n;
  F.qu = P.qu;
  F.qm = P.qm;
  F.qg = P.qg;
  F.thr_m = P.thr_m;
  F.thr_g = P.thr_g;
  F.thr_var = P.thr_var;
  F.sig_scale = P.sig_scale;
  F.sum_scale = P.sum_scale;
  // limb split: every low limb's window sum (n+1 terms) stays below 2^30
  F.kbits = 0;
  while (((long long)(c->n + 1) << (F.kbits + 1)) <= (1LL << 30)) ++F.kbits;
  if (c->cfg.high_res_is_moving) {
    // the ultrasound is static: its weighting factor per voxel and their sum,
    // once, with the generic moments kernel on M = G = 0
    float* zero = c->d_scratch;
    LC2_CUDA(cudaMemsetAsync(zero, 0, sizeof(float) * c->nv, c->stream));
    LC2_CUDA(cudaMemsetAsync(c->d_acc, 0, sizeof(unsigned long long) * 2, c->stream));
    lc2::MomentParams Q = P;
    choose_zchunks(c, 1, Q);
    Q.u_stride = Q.m_stride = Q.g_stride = 0;
    if (c->lc2_nd == 3)
      LC2_TRY(launch_moments_nd<3>(c, c->d_static, storage, zero, zero, Q, 0, 1, c->d_sigma, nullptr));
    else
      LC2_TRY(launch_moments_nd<2>(c, c->d_static, storage, zero, zero, Q, 0, 1, c->d_sigma, nullptr));
    unsigned long long sums[2] = {0, 0};
    LC2_CUDA(cudaMemcpyAsync(sums, c->d_acc, sizeof(sums), cudaMemcpyDeviceToHost, c->stream));
    LC2_CUDA(cudaStreamSynchronize(c->stream));
    c->sigma_sum = (long long)sums[1];
    LC2_TRY(static_window_sum(c));
  } else {
    LC2_TRY(fixed_static_sums(c));
  }
  c->ready = true;
  return LC2_OK;
}

}  // namespace

extern "C" {

int lc2_set_images(lc2_context* c, const float* fixed, const float* moving) {
  g_err.clear();
  if (!c || !fixed || !moving) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  if (!c->owns_moving)
    return fail(LC2_ERR_INVALID_ARGUMENT, "the frames of a stack share the stack's moving volume");
  LC2_TRY(select_device(c));
  float fmax = 0.0f, mmax = 0.0f;
  LC2_TRY(image_absmax(fixed, c->nf, "fixed", &fmax));
  LC2_TRY(image_absmax(moving, c->nm, "moving", &mmax));
  c->ready = false;
  LC2_TRY(upload_image(c, moving, c->nm, c->d_moving, c->cfg.storage));
  return set_fixed(c, fixed, fmax, mmax);
}

int lc2_set_images_device(lc2_context* c, const float* fixed, const float* moving) {
  g_err.clear();
  if (!c || !fixed || !moving) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  if (!c->owns_moving)
    return fail(LC2_ERR_INVALID_ARGUMENT, "the frames of a stack share the stack's moving volume");
  LC2_TRY(select_device(c));
  for (const float* p : {fixed, moving}) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess ||
        (at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) ||
        at.device != c->cfg.device) {
      cudaGetLastError();
      return fail(LC2_ERR_INVALID_ARGUMENT,
                  "lc2_set_images_device needs device memory of the context's device");
    }
  }
  // largest |value| and NaN/Inf flag of each image, on the device
  unsigned int* flags = reinterpret_cast<unsigned int*>(c->d_acc);  // 4 words, reset below
  LC2_CUDA(cudaMemsetAsync(flags, 0, 4 * sizeof(unsigned int), c->stream));
  const int blocks = 152 * 4;
  k_absmax_flag<<<blocks, 256, 0, c->stream>>>(fixed, c->nf, flags);
  k_absmax_flag<<<blocks, 256, 0, c->stream>>>(moving, c->nm, flags + 2);
  LC2_CUDA(cudaGetLastError());
  unsigned int h[4] = {0, 0, 0, 0};
  LC2_CUDA(cudaMemcpyAsync(h, flags, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  LC2_CUDA(cudaMemsetAsync(flags, 0, 4 * sizeof(unsigned int), c->stream));
  if (h[1]) return fail(LC2_ERR_INVALID_ARGUMENT, "fixed image has NaN/Inf");
  if (h[3]) return fail(LC2_ERR_INVALID_ARGUMENT, "moving image has NaN/Inf");
  float fmax, mmax;
  std::memcpy(&fmax, &h[0], 4);
  std::memcpy(&mmax, &h[2], 4);
  c->ready = false;
  LC2_TRY(upload_image(c, moving, c->nm, c->d_moving, c->cfg.storage, true));
  return set_fixed(c, fixed, fmax, mmax);
}

}  // extern "C"

namespace {

// Validates the matrices and writes their per-transform affines into the
// pinned staging buffer (no device work).
int stage_host(lc2_context* c, const float* matrices, int count) {
  if (count < 0 || (count > 0 && !matrices)) return fail(LC2_ERR_INVALID_ARGUMENT, "bad transforms");
  LC2_TRY(ensure_capacity(c, count));
  if (c->presample && !c->generic && !c->pipeline) LC2_TRY(ensure_presample(c, count));
  const int mf = matrix_floats(c);
  for (int k = 0; k < count; ++k) {
    const float* m = matrices + (size_t)k * mf;
    for (int i = 0; i < mf; ++i)
      if (!std::isfinite(m[i])) return fail(LC2_ERR_INVALID_ARGUMENT, "transform %d has NaN/Inf", k);
    build_xform(c->warp_nd, c->virt, c->cfg.moving, m, &c->h_xf[k]);
  }
  return LC2_OK;
}

// lc2_evaluate_batch's device sequence for a static-ultrasound context.
int enqueue_batch(lc2_context* c, int count) {
  LC2_CUDA(cudaMemcpyAsync(c->d_xf, c->h_xf, sizeof(lc2::Xform) * count, cudaMemcpyHostToDevice,
                           c->stream));
  if (c->mi) {
    LC2_TRY(launch_mi(c, count));
  } else {
    // no memset: the sums start at zero (acc_clean, checked before each
    // replay) and k_finalize resets them
    LC2_TRY(launch_group(c, 0, count));
    LC2_TRY(launch_finalize(c, count));
  }
  LC2_CUDA(cudaMemcpyAsync(c->h_out, c->d_out, sizeof(double) * count, cudaMemcpyDeviceToHost,
                           c->stream));
  // only the warp-specialised kernel raises the error flag
  if (c->pipeline)
    LC2_CUDA(cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  return LC2_OK;
}

// The same sequence through a CUDA graph captured once per batch size.
int launch_batch_graph(lc2_context* c, int count) {
  lc2_context::Graph* g = nullptr;
  for (auto& cand : c->graphs)
    if (cand.count == count) g = &cand;
  if (!g) {
    if (c->graphs.size() >= 16) {
      cudaGraphExecDestroy(c->graphs.front().exec);
      cudaGraphDestroy(c->graphs.front().graph);
      c->graphs.erase(c->graphs.begin());
    }
    LC2_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
    const long long before = c->launches;
    int st = enqueue_batch(c, count);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    const long long kernels = c->launches - before;
    c->launches = before;  // counted when the graph runs
    if (st != LC2_OK) {
      if (graph) cudaGraphDestroy(graph);
      return st;
    }
    LC2_CUDA(e);
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(graph);
      LC2_CUDA(e);
    }
    c->graphs.push_back({count, graph, exec, kernels});
    g = &c->graphs.back();
  }
  LC2_CUDA(cudaGraphLaunch(g->exec, c->stream));
  c->launches += g->kernels;
  ++c->graph_launches;
  return LC2_OK;
}

}  // namespace

extern "C" {

int lc2_stage_transforms(lc2_context* c, const float* matrices, int count) {
  g_err.clear();
  LC2_TRY(check_ctx(c));
  LC2_TRY(select_device(c));
  LC2_TRY(stage_host(c, matrices, count));
  if (count > 0)
    LC2_CUDA(cudaMemcpyAsync(c->d_xf, c->h_xf, sizeof(lc2::Xform) * count, cudaMemcpyHostToDevice,
                             c->stream));
  c->staged = count;
  return LC2_OK;
}

int lc2_launch_staged(lc2_context* c, int count) {
  LC2_TRY(check_ctx(c));
  if (count < 0 || count > c->staged)
    return fail(LC2_ERR_INVALID_ARGUMENT, "launch of %d transforms but %d staged", count, c->staged);
  if (count == 0) return LC2_OK;
  LC2_TRY(select_device(c));
  if (c->mi) return launch_mi(c, count);
  LC2_CUDA(cudaMemsetAsync(c->d_acc, 0, sizeof(unsigned long long) * 2 * count, c->stream));
  // the fused paths keep nothing per transform on the device, so one launch
  // covers the whole batch; the generic path is bounded by its scratch slots
  const int group = c->generic ? c->slots : count;
  for (int k0 = 0; k0 < count; k0 += group) {
    int cnt = std::min(group, count - k0);
    LC2_TRY(launch_group(c, k0, cnt));
  }
  return launch_finalize(c, count);
}

int lc2_fetch_results(lc2_context* c, double* out, int count) {
  LC2_TRY(check_ctx(c));
  if (count < 0 || count > c->staged || (count > 0 && !out))
    return fail(LC2_ERR_INVALID_ARGUMENT, "bad result request");
  LC2_TRY(select_device(c));
  if (count > 0)
    LC2_CUDA(cudaMemcpyAsync(c->h_out, c->d_out, sizeof(double) * count, cudaMemcpyDeviceToHost,
                             c->stream));
  LC2_CUDA(cudaMemcpyAsync(c->h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  LC2_TRY(check_pipeline(c));
  if (count > 0) std::memcpy(out, c->h_out, sizeof(double) * count);
  return LC2_OK;
}

int lc2_evaluate_batch(lc2_context* c, const float* matrices, int count, double* out) {
  g_err.clear();
  LC2_TRY(check_ctx(c));
  if (count > 0 && !out) return fail(LC2_ERR_INVALID_ARGUMENT, "null output");
  // every fused path (either modality) and mutual information replay a graph;
  // the generic path's launches depend on its scratch slots
  if (!c->generic && c->use_graphs && !c->timing && count > 0) {
    LC2_TRY(select_device(c));
    LC2_TRY(stage_host(c, matrices, count));
    c->staged = count;
    if (!c->mi && !c->acc_clean)
      LC2_CUDA(cudaMemsetAsync(c->d_acc, 0, sizeof(unsigned long long) * 2 * (size_t)c->cap,
                               c->stream));
    c->acc_clean = false;  // until this batch is known to have finished
    LC2_TRY(launch_batch_graph(c, count));
    LC2_CUDA(cudaStreamSynchronize(c->stream));
    c->acc_clean = true;  // k_finalize reset every sum the batch used
    LC2_TRY(check_pipeline(c));
    std::memcpy(out, c->h_out, sizeof(double) * count);
    return LC2_OK;
  }
  LC2_TRY(lc2_stage_transforms(c, matrices, count));
  LC2_TRY(lc2_launch_staged(c, count));
  return lc2_fetch_results(c, out, count);
}

long long lc2_graph_launches(const lc2_context* c) { return c ? c->graph_launches : 0; }

int lc2_evaluate(lc2_context* c, const float* matrix, double* out) {
  if (!out) return fail(LC2_ERR_INVALID_ARGUMENT, "null output");
  return lc2_evaluate_batch(c, matrix, 1, out);
}

int lc2_evaluate_fields(lc2_context* c, const float* matrix, double* lc2_out, float* U, float* M,
                        float* G, float* sigma, float* measure) {
  if (c && c->mi) return fail(LC2_ERR_UNSUPPORTED, "field dumps are LC2 diagnostics (PatchSize >= 1)");
  LC2_TRY(lc2_stage_transforms(c, matrix, 1));
  LC2_TRY(select_device(c));
  const size_t nv = c->nv;
  float* osig = nullptr;
  float* omeas = nullptr;
  LC2_CUDA(dev_alloc((void**)&osig, sizeof(float) * nv * 3, c->stream));
  struct Free {
    float* p;
    cudaStream_t st;
    ~Free() { dev_free(p, st); }
  } guard{osig, c->stream};
  omeas = osig + nv;
  float* tmp = osig + 2 * nv;
  LC2_CUDA(cudaMemsetAsync(c->d_acc, 0, sizeof(unsigned long long) * 2, c->stream));
  if (c->cfg.high_res_is_moving) {
    // LC2 and measures from the fused kernel; M and G from the generic
    // resample/Sobel kernels; sigma is the precomputed static map
    LC2_TRY(launch_fused(c, 0, 1, omeas));
    LC2_TRY(launch_finalize(c, 1));
    float* w0 = c->d_scratch;
    LC2_TRY(launch_warp(c, c->warp_nd, c->d_moving, c->cfg.storage, c->cfg.moving, c->d_xf, 0, 1,
                        w0, nv));
    LC2_TRY(launch_sobel(c, w0, c->d_scratch + (size_t)c->slots * nv, 1, nv));
    LC2_CUDA(cudaMemcpyAsync(osig, c->d_sigma, sizeof(float) * nv, cudaMemcpyDeviceToDevice,
                             c->stream));
  } else {
    LC2_TRY(launch_group_generic(c, 0, 1, osig, omeas));
    LC2_TRY(launch_finalize(c, 1));
  }
  float* w = c->d_scratch;
  const bool hrm = c->cfg.high_res_is_moving != 0;
  const float* dU = hrm ? nullptr : w;
  const float* dM = hrm ? w : (const float*)c->d_static;
  const float* dG = hrm ? c->d_scratch + (size_t)c->slots * nv : c->d_gstatic;
  if (U) {
    if (hrm) {
      LC2_TRY(to_float(c, c->d_static, tmp, nv, c->cfg.storage));
      dU = tmp;
    }
    LC2_CUDA(cudaMemcpyAsync(U, dU, sizeof(float) * nv, cudaMemcpyDeviceToHost, c->stream));
  }
  if (M) LC2_CUDA(cudaMemcpyAsync(M, dM, sizeof(float) * nv, cudaMemcpyDeviceToHost, c->stream));
  if (G) LC2_CUDA(cudaMemcpyAsync(G, dG, sizeof(float) * nv, cudaMemcpyDeviceToHost, c->stream));
  if (sigma) LC2_CUDA(cudaMemcpyAsync(sigma, osig, sizeof(float) * nv, cudaMemcpyDeviceToHost, c->stream));
  if (measure)
    LC2_CUDA(cudaMemcpyAsync(measure, omeas, sizeof(float) * nv, cudaMemcpyDeviceToHost, c->stream));
  LC2_CUDA(cudaMemcpyAsync(c->h_out, c->d_out, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  if (lc2_out) *lc2_out = c->h_out[0];
  return LC2_OK;
}

namespace lc2 {
// measure / sigma where sigma > 1e-6, else 0 (cu_lc2_3d.cu:843-866)
__global__ void k_weight_map(const float* __restrict__ measure, const float* __restrict__ sigma,
                             size_t n, float* __restrict__ out) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const float s = sigma[i];
    out[i] = s > 1e-6f ? measure[i] / s : 0.0f;
  }
}
}  // namespace lc2

int lc2_weighting_map(lc2_context* c, const float* matrix, double* lc2_out, float* map) {
  if (!map) return fail(LC2_ERR_INVALID_ARGUMENT, "null map");
  if (c && c->mi) return fail(LC2_ERR_UNSUPPORTED, "the weighting map is an LC2 quantity (PatchSize >= 1)");
  LC2_TRY(lc2_stage_transforms(c, matrix, 1));
  LC2_TRY(select_device(c));
  const size_t nv = c->nv;
  float* buf = nullptr;
  LC2_CUDA(dev_alloc((void**)&buf, sizeof(float) * nv * 3, c->stream));
  struct Free {
    float* p;
    cudaStream_t st;
    ~Free() { dev_free(p, st); }
  } guard{buf, c->stream};
  float* osig = buf;
  float* omeas = buf + nv;
  float* dmap = buf + 2 * nv;
  LC2_CUDA(cudaMemsetAsync(c->d_acc, 0, sizeof(unsigned long long) * 2, c->stream));
  const float* sig = osig;
  if (c->cfg.high_res_is_moving) {
    LC2_TRY(launch_fused(c, 0, 1, omeas));
    sig = c->d_sigma;
  } else {
    LC2_TRY(launch_group_generic(c, 0, 1, osig, omeas));
  }
  LC2_TRY(launch_finalize(c, 1));
  const int blocks = (int)std::min<size_t>((nv + 255) / 256, 152 * 16);
  lc2::k_weight_map<<<blocks, 256, 0, c->stream>>>(omeas, sig, nv, dmap);
  ++c->launches;
  LC2_CUDA(cudaGetLastError());
  LC2_CUDA(cudaMemcpyAsync(map, dmap, sizeof(float) * nv, cudaMemcpyDeviceToHost, c->stream));
  LC2_CUDA(cudaMemcpyAsync(c->h_out, c->d_out, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  LC2_CUDA(cudaStreamSynchronize(c->stream));
  if (lc2_out) *lc2_out = c->h_out[0];
  return LC2_OK;
}

// ---------------------------------------------------------------------------
// Transform builders (host)
// ---------------------------------------------------------------------------

int lc2_affine_3d(const float rot[3], const float trans[3], const float scale[3],
                  const float shear[3], const float center[3], const float shift[3],
                  float out[16]) {
  if (!rot || !trans || !scale || !shear || !center || !shift || !out)
    return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  const double d2r = 3.14159265358979323846 / 180.0;
  double c[3], s[3];
  for (int a = 0; a < 3; ++a) {
    c[a] = std::cos((double)rot[a] * d2r);
    s[a] = std::sin((double)rot[a] * d2r);
  }
  double Rx[3][3] = {{1, 0, 0}, {0, c[0], -s[0]}, {0, s[0], c[0]}};
  double Ry[3][3] = {{c[1], 0, s[1]}, {0, 1, 0}, {-s[1], 0, c[1]}};
  double Rz[3][3] = {{c[2], -s[2], 0}, {s[2], c[2], 0}, {0, 0, 1}};
  double ShS[3][3] = {{scale[0], (double)shear[0] * scale[1], (double)shear[1] * scale[2]},
                      {0, scale[1], (double)shear[2] * scale[2]},
                      {0, 0, scale[2]}};
  auto mul = [](const double A[3][3], const double B[3][3], double C[3][3]) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        C[i][j] = 0;
        for (int k = 0; k < 3; ++k) C[i][j] += A[i][k] * B[k][j];
      }
  };
  double T1[3][3], T2[3][3], L[3][3];
  mul(Rx, ShS, T1);
  mul(Ry, T1, T2);
  mul(Rz, T2, L);
  for (int i = 0; i < 3; ++i) {
    double t = (double)center[i] + trans[i];
    for (int k = 0; k < 3; ++k) t += L[i][k] * ((double)shift[k] - center[k]);
    for (int j = 0; j < 3; ++j) out[4 * i + j] = (float)L[i][j];
    out[4 * i + 3] = (float)t;
  }
  out[12] = out[13] = out[14] = 0.0f;
  out[15] = 1.0f;
  return LC2_OK;
}

int lc2_affine_2d(float rot, const float trans[2], const float scale[2], float shear,
                  const float center[2], const float shift[2], float out[9]) {
  if (!trans || !scale || !center || !shift || !out) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  const double d2r = 3.14159265358979323846 / 180.0;
  double c = std::cos((double)rot * d2r), s = std::sin((double)rot * d2r);
  double L[2][2] = {{c * scale[0], scale[1] * (c * shear - s)}, {s * scale[0], scale[1] * (s * shear + c)}};
  for (int i = 0; i < 2; ++i) {
    double t = (double)center[i] + trans[i];
    for (int k = 0; k < 2; ++k) t += L[i][k] * ((double)shift[k] - center[k]);
    out[3 * i + 0] = (float)L[i][0];
    out[3 * i + 1] = (float)L[i][1];
    out[3 * i + 2] = (float)t;
  }
  out[6] = out[7] = 0.0f;
  out[8] = 1.0f;
  return LC2_OK;
}

int lc2_invert_affine_3d(const float in[16], float out[16]) {
  if (!in || !out) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  double a[3][3], t[3];
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) a[i][j] = in[4 * i + j];
    t[i] = in[4 * i + 3];
  }
  double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) -
               a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
               a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
  if (det == 0.0 || !std::isfinite(det)) return fail(LC2_ERR_SINGULAR, "singular transform");
  double inv[3][3];
  inv[0][0] = (a[1][1] * a[2][2] - a[1][2] * a[2][1]) / det;
  inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
  inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
  inv[1][0] = (a[1][2] * a[2][0] - a[1][0] * a[2][2]) / det;
  inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
  inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
  inv[2][0] = (a[1][0] * a[2][1] - a[1][1] * a[2][0]) / det;
  inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
  inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
  for (int i = 0; i < 3; ++i) {
    double ti = 0;
    for (int j = 0; j < 3; ++j) {
      out[4 * i + j] = (float)inv[i][j];
      ti -= inv[i][j] * t[j];
    }
    out[4 * i + 3] = (float)ti;
  }
  out[12] = out[13] = out[14] = 0.0f;
  out[15] = 1.0f;
  return LC2_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// 2D-to-3D frame stacks
// ---------------------------------------------------------------------------

namespace lc2 {
// LC2 of evaluation k with its own weighting-factor sum.
__global__ void k_finalize_list(const unsigned long long* __restrict__ acc, int count,
                                const long long* __restrict__ sigma_sums,
                                double* __restrict__ out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  double v = (double)(long long)acc[2 * k] / (double)sigma_sums[k];
  if (isnan(v) || isinf(v)) v = 0.0;
  out[k] = v;
}
}  // namespace lc2

struct lc2_stack {
  lc2_config base{};  // mode 2D-to-3D, moving geometry, patch, storage, device
  size_t nm = 0;
  void* d_moving = nullptr;
  float mmax = 0.0f;
  bool moving_set = false;
  std::vector<lc2_context*> frames;
  cudaStream_t stream = nullptr;
  int sms = 0;
  // evaluation buffers (device + pinned host), by evaluation in segment order
  int cap = 0, seg_cap = 0;
  lc2::Xform* d_xf = nullptr;
  unsigned long long* d_acc = nullptr;
  long long* d_sums = nullptr;
  double* d_out = nullptr;
  lc2::ListSeg* d_segs = nullptr;
  lc2::Xform* h_xf = nullptr;
  long long* h_sums = nullptr;
  double* h_out = nullptr;
  lc2::ListSeg* h_segs = nullptr;
  // CUDA graphs of the launch sequence, keyed by the call's segment layout
  struct Graph {
    std::vector<int> key;  // count, then (frame, count) per segment
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
  };
  std::vector<Graph> graphs;
  bool use_graphs = true;
  bool batching = true;  // lc2_stack_register: lock-step merged launches
  int wnd = 3;           // resampling dimensionality of the frames (2: 2D contexts)
  long long launches = 0, graph_launches = 0;
};

// Cross-context batching (lc2_merger_*): the stack's launch machinery without
// a volume of its own; each segment names its context's moving image.
struct lc2_merger {
  lc2_stack s;
};

namespace {

void stack_drop_graphs(lc2_stack* s) {
  for (auto& g : s->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
  }
  s->graphs.clear();
}

void stack_free_buffers(lc2_stack* s) {
  dev_free(s->d_xf, s->stream);
  dev_free(s->d_acc, s->stream);
  dev_free(s->d_sums, s->stream);
  dev_free(s->d_out, s->stream);
  dev_free(s->d_segs, s->stream);
  if (s->stream) cudaStreamSynchronize(s->stream);
  host_free(s->h_xf);
  host_free(s->h_sums);
  host_free(s->h_out);
  host_free(s->h_segs);
  s->d_xf = nullptr; s->d_acc = nullptr; s->d_sums = nullptr; s->d_out = nullptr;
  s->d_segs = nullptr; s->h_xf = nullptr; s->h_sums = nullptr; s->h_out = nullptr;
  s->h_segs = nullptr;
  s->cap = s->seg_cap = 0;
}

// Buffers for `count` evaluations in `nseg` segments. Reallocation moves the
// buffers the cached graphs read, so it drops them.
int stack_capacity(lc2_stack* s, int count, int nseg) {
  if (count <= s->cap && nseg <= s->seg_cap) return LC2_OK;
  stack_drop_graphs(s);
  const int ncap = std::max(count, std::max(256, s->cap));
  const int nseg_cap = std::max(nseg, std::max(64, s->seg_cap));
  stack_free_buffers(s);
  LC2_CUDA(dev_alloc((void**)&s->d_xf, sizeof(lc2::Xform) * ncap, s->stream));
  LC2_CUDA(dev_alloc((void**)&s->d_acc, sizeof(unsigned long long) * 2 * ncap, s->stream));
  LC2_CUDA(dev_alloc((void**)&s->d_sums, sizeof(long long) * ncap, s->stream));
  LC2_CUDA(dev_alloc((void**)&s->d_out, sizeof(double) * ncap, s->stream));
  LC2_CUDA(dev_alloc((void**)&s->d_segs, sizeof(lc2::ListSeg) * nseg_cap, s->stream));
  LC2_CUDA(host_alloc((void**)&s->h_xf, sizeof(lc2::Xform) * ncap));
  LC2_CUDA(host_alloc((void**)&s->h_sums, sizeof(long long) * ncap));
  LC2_CUDA(host_alloc((void**)&s->h_out, sizeof(double) * ncap));
  LC2_CUDA(host_alloc((void**)&s->h_segs, sizeof(lc2::ListSeg) * nseg_cap));
  s->cap = ncap;
  s->seg_cap = nseg_cap;
  return LC2_OK;
}

// The launch sequence of one stack evaluation, on the stack's stream: copies
// of the transforms, segments and weighting-factor sums, the work-list
// kernel, the per-evaluation ratio and the copy of the results.
int stack_enqueue(lc2_stack* s, int count, int nseg, long long units) {
  cudaStream_t st = s->stream;
  LC2_CUDA(cudaMemcpyAsync(s->d_xf, s->h_xf, sizeof(lc2::Xform) * count, cudaMemcpyHostToDevice, st));
  LC2_CUDA(cudaMemcpyAsync(s->d_segs, s->h_segs, sizeof(lc2::ListSeg) * nseg, cudaMemcpyHostToDevice, st));
  LC2_CUDA(cudaMemcpyAsync(s->d_sums, s->h_sums, sizeof(long long) * count, cudaMemcpyHostToDevice, st));
  LC2_CUDA(cudaMemsetAsync(s->d_acc, 0, sizeof(unsigned long long) * 2 * count, st));
  lc2::ListLaunch L;
  L.segs = s->d_segs;
  L.nseg = nseg;
  L.units = units;
  L.xf = s->d_xf;
  L.acc = s->d_acc;
  L.r = s->base.patch_size;
  L.wnd = s->wnd;
  L.sms = s->sms;
  L.stream = st;
  cudaError_t e;
  if (s->base.storage == LC2_STORE_F16)
    e = lc2::list_launch<__half>(L);
  else if (s->base.storage == LC2_STORE_BF16)
    e = lc2::list_launch<__nv_bfloat16>(L);
  else
    e = lc2::list_launch<float>(L);
  LC2_CUDA(e);
  lc2::k_finalize_list<<<(count + 127) / 128, 128, 0, st>>>(s->d_acc, count, s->d_sums, s->d_out);
  LC2_CUDA(cudaGetLastError());
  LC2_CUDA(cudaMemcpyAsync(s->h_out, s->d_out, sizeof(double) * count, cudaMemcpyDeviceToHost, st));
  return LC2_OK;
}

int stack_select_device(const lc2_stack* s) {
  int cur = -1;
  LC2_CUDA(cudaGetDevice(&cur));
  if (cur != s->base.device) LC2_CUDA(cudaSetDevice(s->base.device));
  return LC2_OK;
}

}  // namespace

extern "C" {

int lc2_stack_create(const lc2_geometry* moving, int patch_size, int storage, int device,
                     lc2_stack** out) {
  g_err.clear();
  if (!moving || !out) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (!finite_geom(*moving))
    return fail(LC2_ERR_INVALID_ARGUMENT, "geometry needs dims >= 1, finite spacing > 0 and origin");
  if (storage < LC2_STORE_F32 || storage > LC2_STORE_BF16)
    return fail(LC2_ERR_INVALID_ARGUMENT, "unknown storage %d", storage);
  if (patch_size < 1 || patch_size > 12)
    return fail(LC2_ERR_UNSUPPORTED, "patch size %d outside [1, 12] for 2D patches", patch_size);
  lc2_stack* s = new (std::nothrow) lc2_stack();
  if (!s) return fail(LC2_ERR_OUT_OF_MEMORY, "host allocation failed");
  s->base.mode = LC2_MODE_2DTO3D;
  s->base.moving = *moving;
  s->base.patch_size = patch_size;
  s->base.high_res_is_moving = 1;
  s->base.storage = storage;
  s->base.max_batch = 1;
  s->base.device = device;
  s->nm = (size_t)moving->dim[0] * moving->dim[1] * moving->dim[2];
  int st = stack_select_device(s);
  cudaError_t e = cudaSuccess;
  if (st == LC2_OK) e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device);
  if (st == LC2_OK && e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (st == LC2_OK && e == cudaSuccess) e = dev_alloc(&s->d_moving, s->nm * elem_size(storage), s->stream);
  if (st != LC2_OK || e != cudaSuccess) {
    std::string msg = st != LC2_OK ? g_err : std::string(cudaGetErrorString(e));
    lc2_stack_destroy(s);
    return fail(st != LC2_OK ? st : LC2_ERR_OUT_OF_MEMORY, "stack: %s", msg.c_str());
  }
  *out = s;
  return LC2_OK;
}

int lc2_stack_destroy(lc2_stack* s) {
  if (!s) return LC2_OK;
  stack_select_device(s);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (lc2_context* f : s->frames) lc2_destroy(f);
  stack_drop_graphs(s);
  stack_free_buffers(s);
  dev_free(s->d_moving, s->stream);
  if (s->stream) {
    cudaStreamSynchronize(s->stream);
    cudaStreamDestroy(s->stream);
  }
  delete s;
  return LC2_OK;
}

int lc2_stack_set_moving(lc2_stack* s, const float* moving) {
  g_err.clear();
  if (!s || !moving) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  if (s->moving_set) return fail(LC2_ERR_INVALID_ARGUMENT, "the stack's moving volume is already set");
  LC2_TRY(stack_select_device(s));
  float mmax = 0.0f;
  LC2_TRY(image_absmax(moving, s->nm, "moving", &mmax));
  // staged through a temporary one-slot context for its conversion kernels
  float* tmp = nullptr;
  LC2_CUDA(dev_alloc((void**)&tmp, sizeof(float) * s->nm, s->stream));
  struct Free {
    float* p;
    cudaStream_t st;
    ~Free() { dev_free(p, st); }
  } guard{tmp, s->stream};
  LC2_CUDA(cudaMemcpyAsync(tmp, moving, sizeof(float) * s->nm, cudaMemcpyHostToDevice, s->stream));
  lc2_context conv;  // only its stream and launch counter are used
  conv.stream = s->stream;
  LC2_TRY(convert_to_storage(&conv, tmp, s->d_moving, s->nm, s->base.storage));
  LC2_CUDA(cudaStreamSynchronize(s->stream));
  s->launches += conv.launches;
  s->mmax = mmax;
  s->moving_set = true;
  return LC2_OK;
}

int lc2_stack_add_frame(lc2_stack* s, const lc2_geometry* frame, const float virtual_spacing[3],
                        const float* ultrasound, int* frame_id) {
  g_err.clear();
  if (!s || !frame || !virtual_spacing || !ultrasound || !frame_id)
    return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  if (!s->moving_set) return fail(LC2_ERR_NOT_READY, "set the stack's moving volume first");
  if (frame->dim[2] != 1) return fail(LC2_ERR_INVALID_ARGUMENT, "a frame has dim[2] = 1");
  LC2_TRY(stack_select_device(s));
  lc2_config cfg = s->base;
  cfg.fixed = *frame;
  for (int a = 0; a < 3; ++a) cfg.virtual_spacing[a] = virtual_spacing[a];
  lc2_context* c = nullptr;
  LC2_TRY(create_context(&cfg, false, &c));
  c->d_moving = s->d_moving;
  float fmax = 0.0f;
  int st = image_absmax(ultrasound, c->nf, "ultrasound", &fmax);
  if (st == LC2_OK) st = set_fixed(c, ultrasound, fmax, s->mmax);
  if (st != LC2_OK) {
    std::string msg = g_err;
    lc2_destroy(c);
    g_err = msg;
    return st;
  }
  s->launches += c->launches;
  *frame_id = (int)s->frames.size();
  s->frames.push_back(c);
  return LC2_OK;
}

int lc2_stack_frames(const lc2_stack* s) { return s ? (int)s->frames.size() : 0; }

int lc2_stack_frame_context(lc2_stack* s, int frame_id, lc2_context** ctx) {
  if (!s || !ctx) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  if (frame_id < 0 || frame_id >= (int)s->frames.size())
    return fail(LC2_ERR_INVALID_ARGUMENT, "no frame %d", frame_id);
  *ctx = s->frames[frame_id];
  return LC2_OK;
}

int lc2_stack_set_graphs(lc2_stack* s, int on) {
  if (!s) return fail(LC2_ERR_INVALID_ARGUMENT, "null stack");
  s->use_graphs = on != 0;
  return LC2_OK;
}

int lc2_stack_set_option(lc2_stack* s, int option, int value) {
  if (!s) return fail(LC2_ERR_INVALID_ARGUMENT, "null stack");
  if (option == LC2_OPTION_GRAPHS) return lc2_stack_set_graphs(s, value);
  if (option == LC2_OPTION_STACK_BATCHING) {
    s->batching = value != 0;
    return LC2_OK;
  }
  if (option == LC2_OPTION_STREAM_PRIORITY) {
    LC2_TRY(stack_select_device(s));
    int least = 0, greatest = 0;
    LC2_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int prio = std::max(greatest, std::min(least, value));
    cudaStream_t ns = nullptr;
    LC2_CUDA(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, prio));
    LC2_CUDA(cudaStreamSynchronize(s->stream));
    stack_drop_graphs(s);
    cudaStreamDestroy(s->stream);
    s->stream = ns;
    return LC2_OK;
  }
  return fail(LC2_ERR_INVALID_ARGUMENT, "unknown stack option %d", option);
}

int lc2_stack_get_option(const lc2_stack* s, int option, int* value) {
  if (!s || !value) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  if (option == LC2_OPTION_STACK_BATCHING) {
    *value = s->batching ? 1 : 0;
    return LC2_OK;
  }
  if (option == LC2_OPTION_GRAPHS) {
    *value = s->use_graphs ? 1 : 0;
    return LC2_OK;
  }
  return fail(LC2_ERR_INVALID_ARGUMENT, "unknown stack option %d", option);
}

long long lc2_stack_launch_count(const lc2_stack* s) { return s ? s->launches : 0; }
long long lc2_stack_graph_launches(const lc2_stack* s) { return s ? s->graph_launches : 0; }

int lc2_stack_evaluate(lc2_stack* s, int count, const int* frame_ids, const float* matrices,
                       double* lc2_out) {
  g_err.clear();
  if (!s) return fail(LC2_ERR_INVALID_ARGUMENT, "null stack");
  if (count < 0 || (count > 0 && (!frame_ids || !matrices || !lc2_out)))
    return fail(LC2_ERR_INVALID_ARGUMENT, "bad evaluation request");
  if (count == 0) return LC2_OK;
  const int nf = (int)s->frames.size();
  for (int k = 0; k < count; ++k) {
    if (frame_ids[k] < 0 || frame_ids[k] >= nf)
      return fail(LC2_ERR_INVALID_ARGUMENT, "evaluation %d names frame %d of %d", k, frame_ids[k], nf);
    for (int i = 0; i < 16; ++i)
      if (!std::isfinite(matrices[(size_t)k * 16 + i]))
        return fail(LC2_ERR_INVALID_ARGUMENT, "transform %d has NaN/Inf", k);
  }
  LC2_TRY(stack_select_device(s));
  // evaluations grouped by frame (stable), one segment per frame
  std::vector<int> order(count);
  for (int k = 0; k < count; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return frame_ids[a] < frame_ids[b]; });
  std::vector<int> key{count};
  int nseg = 0;
  for (int k = 0; k < count; ++k)
    if (k == 0 || frame_ids[order[k]] != frame_ids[order[k - 1]]) ++nseg;
  LC2_TRY(stack_capacity(s, count, nseg));
  long long units = 0;
  int seg = -1;
  for (int k = 0; k < count; ++k) {
    const int f = frame_ids[order[k]];
    const lc2_context* c = s->frames[f];
    if (k == 0 || f != frame_ids[order[k - 1]]) {
      ++seg;
      lc2::ListSeg& S = s->h_segs[seg];
      S.mov = s->d_moving;
      S.ust = c->d_static;
      S.sig = c->d_sigma;
      S.su = c->d_su;
      S.P = c->fp;
      S.P.ntx = (c->virt.dim[0] + 31) / 32;
      S.P.zchunk = 1;
      S.ntiles = S.P.ntx * ((c->virt.dim[1] + lc2::kListTY - 1) / lc2::kListTY);
      S.count = 0;
      S.eval0 = k;
      S.pad_ = 0;
      S.unit0 = units;
      key.push_back(f);
      key.push_back(0);
    }
    lc2::ListSeg& S = s->h_segs[seg];
    ++S.count;
    ++key.back();
    units += S.ntiles;
    build_xform(3, c->virt, c->cfg.moving, matrices + (size_t)order[k] * 16, &s->h_xf[k]);
    s->h_sums[k] = c->sigma_sum;
  }
  if (s->use_graphs) {
    lc2_stack::Graph* g = nullptr;
    for (auto& cand : s->graphs)
      if (cand.key == key) g = &cand;
    if (!g) {
      lc2_stack::Graph ng;
      ng.key = key;
      LC2_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeRelaxed));
      int st = stack_enqueue(s, count, nseg, units);
      cudaGraph_t graph = nullptr;
      cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
      if (st != LC2_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
      }
      LC2_CUDA(e);
      ng.graph = graph;
      e = cudaGraphInstantiate(&ng.exec, graph, 0);
      if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        LC2_CUDA(e);
      }
      if (s->graphs.size() >= 16) {  // keep the cache small
        cudaGraphExecDestroy(s->graphs.front().exec);
        cudaGraphDestroy(s->graphs.front().graph);
        s->graphs.erase(s->graphs.begin());
      }
      s->graphs.push_back(ng);
      g = &s->graphs.back();
    }
    LC2_CUDA(cudaGraphLaunch(g->exec, s->stream));
    ++s->graph_launches;
    s->launches += 2;
  } else {
    LC2_TRY(stack_enqueue(s, count, nseg, units));
    s->launches += 2;
  }
  LC2_CUDA(cudaStreamSynchronize(s->stream));
  for (int k = 0; k < count; ++k) lc2_out[order[k]] = s->h_out[k];
  return LC2_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Cross-context batching
// ---------------------------------------------------------------------------

extern "C" {

int lc2_merger_create(int device, lc2_merger** out) {
  g_err.clear();
  if (!out) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  lc2_merger* m = new (std::nothrow) lc2_merger();
  if (!m) return fail(LC2_ERR_OUT_OF_MEMORY, "host allocation failed");
  lc2_stack* s = &m->s;
  s->base.device = device;
  s->base.high_res_is_moving = 1;
  s->use_graphs = false;  // the segments change with the contexts of every call
  int st = stack_select_device(s);
  cudaError_t e = cudaSuccess;
  if (st == LC2_OK) e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, device);
  if (st == LC2_OK && e == cudaSuccess) {
    int lo = 0, hi = 0;
    e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    // the most urgent priority: merged launches carry small requests
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&s->stream, cudaStreamNonBlocking, hi);
  }
  if (st != LC2_OK || e != cudaSuccess) {
    std::string msg = st != LC2_OK ? g_err : std::string(cudaGetErrorString(e));
    lc2_merger_destroy(m);
    return fail(st != LC2_OK ? st : LC2_ERR_CUDA, "merger: %s", msg.c_str());
  }
  *out = m;
  return LC2_OK;
}

int lc2_merger_destroy(lc2_merger* m) {
  if (!m) return LC2_OK;
  lc2_stack* s = &m->s;
  stack_select_device(s);
  if (s->stream) cudaStreamSynchronize(s->stream);
  stack_free_buffers(s);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete m;
  return LC2_OK;
}

int lc2_merger_evaluate(lc2_merger* m, int n, lc2_context* const* ctxs, const int* counts,
                        const float* matrices, double* lc2_out) {
  g_err.clear();
  if (!m || n < 0 || (n > 0 && (!ctxs || !counts))) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  lc2_stack* s = &m->s;
  int total = 0, nseg = 0, mode = -1, r = -1, storage = -1;
  for (int i = 0; i < n; ++i) {
    const lc2_context* c = ctxs[i];
    if (!c) return fail(LC2_ERR_INVALID_ARGUMENT, "context %d is null", i);
    if (counts[i] < 0) return fail(LC2_ERR_INVALID_ARGUMENT, "negative count for context %d", i);
    if (!c->ready) return fail(LC2_ERR_NOT_READY, "context %d: images not set", i);
    if (c->lc2_nd != 2 || c->mi || !c->cfg.high_res_is_moving || c->generic)
      return fail(LC2_ERR_UNSUPPORTED,
                  "context %d: merged evaluation takes 2D and 2D-to-3D contexts with "
                  "HighResolutionModality: Moving on the fused kernels", i);
    if (c->cfg.device != s->base.device)
      return fail(LC2_ERR_INVALID_ARGUMENT, "context %d is on device %d, the merger on %d", i,
                  c->cfg.device, s->base.device);
    if (mode < 0) {
      mode = c->cfg.mode;
      r = c->cfg.patch_size;
      storage = c->cfg.storage;
    } else if (c->cfg.mode != mode || c->cfg.patch_size != r || c->cfg.storage != storage) {
      return fail(LC2_ERR_UNSUPPORTED,
                  "merged contexts must share the mode, patch size and storage type");
    }
    total += counts[i];
    if (counts[i] > 0) ++nseg;
  }
  if (total == 0) return LC2_OK;
  if (!matrices || !lc2_out) return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  const int mf = mode == LC2_MODE_2D ? 9 : 16;
  for (int k = 0; k < total; ++k)
    for (int i = 0; i < mf; ++i)
      if (!std::isfinite(matrices[(size_t)k * mf + i]))
        return fail(LC2_ERR_INVALID_ARGUMENT, "transform %d has NaN/Inf", k);
  LC2_TRY(stack_select_device(s));
  s->base.patch_size = r;
  s->base.storage = storage;
  s->wnd = mode == LC2_MODE_2D ? 2 : 3;
  LC2_TRY(stack_capacity(s, total, nseg));
  long long units = 0;
  int k = 0, seg = 0;
  for (int i = 0; i < n; ++i) {
    if (counts[i] == 0) continue;
    const lc2_context* c = ctxs[i];
    lc2::ListSeg& S = s->h_segs[seg++];
    S.mov = c->d_moving;
    S.ust = c->d_static;
    S.sig = c->d_sigma;
    S.su = c->d_su;
    S.P = c->fp;
    S.P.ntx = (c->virt.dim[0] + 31) / 32;
    S.P.zchunk = 1;
    S.ntiles = S.P.ntx * ((c->virt.dim[1] + lc2::kListTY - 1) / lc2::kListTY);
    S.count = counts[i];
    S.eval0 = k;
    S.pad_ = 0;
    S.unit0 = units;
    for (int e = 0; e < counts[i]; ++e, ++k) {
      build_xform(c->warp_nd, c->virt, c->cfg.moving, matrices + (size_t)k * mf, &s->h_xf[k]);
      s->h_sums[k] = c->sigma_sum;
      units += S.ntiles;
    }
  }
  LC2_TRY(stack_enqueue(s, total, nseg, units));
  s->launches += 2;
  LC2_CUDA(cudaStreamSynchronize(s->stream));
  std::memcpy(lc2_out, s->h_out, sizeof(double) * total);
  return LC2_OK;
}

long long lc2_merger_launch_count(const lc2_merger* m) { return m ? m->s.launches : 0; }

}  // extern "C"

// ---------------------------------------------------------------------------
// Autotuner
// ---------------------------------------------------------------------------

extern "C" int lc2_autotune(lc2_context* c, const float* matrices, int count, int* tile_rows,
                            int* zchunk) {
  g_err.clear();
  LC2_TRY(check_ctx(c));
  if (count < 1) return fail(LC2_ERR_INVALID_ARGUMENT, "autotune needs at least one transform");
  LC2_TRY(select_device(c));
  const int r = c->cfg.patch_size;
  const bool hrm = c->cfg.high_res_is_moving != 0;
  if (c->lc2_nd == 3 && !c->mi && !c->generic) {
    LC2_TRY(lc2_stage_transforms(c, matrices, count));
    // 24-row tiles exist for the presampled 3D kernels
    std::vector<int> rows = (r > 4) ? std::vector<int>{8}
                            : (hrm || c->presample) ? std::vector<int>{16, 24, 8}
                                                    : std::vector<int>{16, 8};
    const int vz = c->virt.dim[2];
    std::vector<int> chunks{0};
    for (int zc : {vz, vz / 2, vz / 4, 64, 32})
      if (zc >= 2 * r + 2 && zc <= vz && std::find(chunks.begin(), chunks.end(), zc) == chunks.end())
        chunks.push_back(zc);
    cudaEvent_t a = nullptr, b = nullptr;
    LC2_CUDA(cudaEventCreate(&a));
    struct Ev {
      cudaEvent_t& e;
      ~Ev() { if (e) cudaEventDestroy(e); }
    } ga{a}, gb{b};
    LC2_CUDA(cudaEventCreate(&b));
    const bool timing = c->timing;
    c->timing = false;
    float best = 0.0f;
    int best_rows = rows[0], best_chunk = 0, best_pipe = 0;
    int st = LC2_OK;
    struct Cand {
      int rows, pipeline;
    };
    std::vector<Cand> cands;
    // the warp-specialised kernel never won a trial and resamples in place
    // (other bits than the default presampled form): selectable, not a candidate
    for (int tr : rows) cands.push_back({tr, 0});
    for (const Cand& cd : cands) {
      const int tr = cd.rows;
      for (int zc : chunks) {
        c->tile_rows = tr;
        c->pipeline = cd.pipeline;
        c->zchunk = zc;
        float ms = 0.0f;
        for (int rep = 0; rep < 2 && st == LC2_OK; ++rep) {  // warm-up, then timed
          if (cudaMemsetAsync(c->d_acc, 0, sizeof(unsigned long long) * 2 * count, c->stream) != cudaSuccess ||
              cudaEventRecord(a, c->stream) != cudaSuccess) {
            st = fail(LC2_ERR_CUDA, "autotune: %s", cudaGetErrorString(cudaGetLastError()));
            break;
          }
          st = hrm ? launch_fused(c, 0, count, nullptr) : launch_fused_fixed(c, 0, count);
          if (st == LC2_OK && (cudaEventRecord(b, c->stream) != cudaSuccess ||
                               cudaEventSynchronize(b) != cudaSuccess ||
                               cudaEventElapsedTime(&ms, a, b) != cudaSuccess))
            st = fail(LC2_ERR_CUDA, "autotune timing: %s", cudaGetErrorString(cudaGetLastError()));
        }
        if (st != LC2_OK) break;
        // an explicit z chunk is kept only when it beats the automatic split
        // by more than 3 %: it then applies to every launch, and a chunk that
        // suits the tuning batch can starve a launch of a few transforms
        // (automatic: one 256^3 transform runs 440 CTAs, whole-depth chunks 88)
        const float score = zc == 0 ? ms : ms * 1.03f;
        if (best == 0.0f || score < best) {
          best = score;
          best_rows = tr;
          best_chunk = zc;
          best_pipe = cd.pipeline;
        }
      }
      if (st != LC2_OK) break;
    }
    c->timing = timing;
    c->tile_rows = best_rows;
    c->zchunk = best_chunk;
    c->pipeline = best_pipe;
    drop_graphs(c);
    if (st == LC2_OK) {
      LC2_CUDA(cudaMemcpy(c->h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost));
      st = check_pipeline(c);
    }
    if (st != LC2_OK) return st;
  }
  if (tile_rows) *tile_rows = ::tile_rows(c);
  if (zchunk) *zchunk = c->zchunk;
  return LC2_OK;
}
