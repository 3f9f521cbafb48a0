// lc2_noalloc.cu -- LC2 evaluation that allocates no memory.
//
// For callers that cannot call cudaMalloc: code running inside a host
// application that owns the device heap through its own allocator or memory
// pool, real-time loops that must not allocate after start-up, or plug-ins
// that are handed device buffers and nothing else. The caller passes its
// device-resident ultrasound (already on the virtual grid), the moving
// image and a device slot for the result; the resampled image, its Sobel
// magnitude and the exact sums live in the file-scope array below, which
// every GPU that loads this library holds until the process exits.
//
// The evaluation runs the resample -> Sobel -> moments kernels of the
// context path (lc2_kernels.cuh) on that array.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <limits>
#include <mutex>

#include "../../include/lc2.h"
#include "lc2_kernels.cuh"

// records the message returned by lc2_last_error (lc2_capi.cu)
void lc2_set_error_message(const char* msg);

namespace {

constexpr size_t kHeader = 256;  // sums, maxima, transform
constexpr size_t kScratchBytes = kHeader + 2 * sizeof(float) * (size_t)LC2_NOALLOC_MAX_VOXELS;

// Scratch shared by every call on a device; see lc2_evaluate_noalloc.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {nullptr};

struct Header {
  unsigned long long acc[2];  // exact sums of measure and sigma
  unsigned int absmax[2];     // |U|, |moving| maxima (float bits)
  unsigned int nonfinite;     // NaN/Inf seen in the inputs
  unsigned int pad;
  lc2::Xform xf;
};
static_assert(sizeof(Header) <= kHeader, "scratch header too small");

int fail(int code, const char* msg) {
  lc2_set_error_message(msg);
  return code;
}

__global__ void k_absmax(const float* __restrict__ a, size_t n, unsigned int* __restrict__ out,
                         unsigned int* __restrict__ nonfinite) {
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
    if (bad) atomicOr(nonfinite, 1u);
  }
}

__global__ void k_ratio(const unsigned long long* __restrict__ acc, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const double v = (double)(long long)acc[0] / (double)(long long)acc[1];
    out[0] = (isnan(v) || isinf(v)) ? 0.0 : v;
  }
}

// Device address of the scratch array, looked up once per device with that
// device current. The address belongs to the device's primary context (the
// one the runtime API uses); a cudaDeviceReset invalidates it, after which
// this library must not be called again in the process.
int scratch_for_current_device(unsigned char** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(LC2_ERR_CUDA, "no current CUDA device");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) return fail(LC2_ERR_CUDA, cudaGetErrorString(e));
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return LC2_OK;
}

long long floor_clamp(long double v) {
  if (v >= (long double)std::numeric_limits<long long>::max())
    return std::numeric_limits<long long>::max();
  if (v < 0) return -1;
  return (long long)std::floor(v);
}

#define NA_CUDA(call)                                             \
  do {                                                            \
    const cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return fail(LC2_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

}  // namespace

extern "C" int lc2_evaluate_noalloc(int mode, const lc2_geometry* virt, const lc2_geometry* moving,
                                    int patch_size, const float* d_ultrasound,
                                    const float* d_moving, const float* matrix, double* d_lc2,
                                    void* stream_ptr) {
  lc2_set_error_message("");
  if (!virt || !moving || !d_ultrasound || !d_moving || !matrix || !d_lc2)
    return fail(LC2_ERR_INVALID_ARGUMENT, "null argument");
  if (mode != LC2_MODE_2D && mode != LC2_MODE_3D && mode != LC2_MODE_2DTO3D)
    return fail(LC2_ERR_INVALID_ARGUMENT, "unknown mode");
  const int warp_nd = (mode == LC2_MODE_2D) ? 2 : 3;
  const int nd = (mode == LC2_MODE_3D) ? 3 : 2;
  const int rmax = (nd == 3) ? 6 : 12;
  if (patch_size < 1 || patch_size > rmax)
    return fail(LC2_ERR_UNSUPPORTED, "patch size outside the supported range");
  for (int a = 0; a < 3; ++a) {
    if (virt->dim[a] < 1 || moving->dim[a] < 1 || !(virt->spacing[a] > 0.0f) ||
        !(moving->spacing[a] > 0.0f))
      return fail(LC2_ERR_INVALID_ARGUMENT, "geometry needs dims >= 1 and spacing > 0");
  }
  if ((mode == LC2_MODE_2D && (virt->dim[2] != 1 || moving->dim[2] != 1)) ||
      (mode == LC2_MODE_2DTO3D && virt->dim[2] != 1))
    return fail(LC2_ERR_INVALID_ARGUMENT, "2D grids need dim[2] = 1");
  // voxel counts built one axis at a time against their limits, so no
  // product can wrap: the virtual grid must fit the scratch array, the moving
  // image the kernels' 32-bit gather indices
  size_t nv = 1, nm = 1;
  for (int a = 0; a < 3; ++a) {
    nv *= (size_t)virt->dim[a];  // <= 2^20 * (2^31 - 1): no wrap
    if (nv > (size_t)LC2_NOALLOC_MAX_VOXELS)
      return fail(LC2_ERR_UNSUPPORTED,
                  "virtual grid larger than LC2_NOALLOC_MAX_VOXELS voxels: use lc2_create");
    nm *= (size_t)moving->dim[a];  // <= (2^31 - 1)^2: no wrap
    if (nm > (size_t)INT32_MAX)
      return fail(LC2_ERR_UNSUPPORTED,
                  "moving image larger than 2^31 - 1 voxels (32-bit gather indices)");
  }
  // every call ends with a blocking read of the input maxima, which a
  // capturing stream cannot take
  {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream_ptr), &cs) != cudaSuccess ||
        cs != cudaStreamCaptureStatusNone)
      return fail(LC2_ERR_UNSUPPORTED,
                  "lc2_evaluate_noalloc blocks on a read-back and cannot run on a capturing "
                  "stream");
  }
  for (int i = 0; i < (warp_nd == 2 ? 9 : 16); ++i)
    if (!std::isfinite(matrix[i])) return fail(LC2_ERR_INVALID_ARGUMENT, "non-finite transform");

  unsigned char* base = nullptr;
  const int st = scratch_for_current_device(&base);
  if (st != LC2_OK) return st;
  cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
  Header* hdr = reinterpret_cast<Header*>(base);
  float* M = reinterpret_cast<float*>(base + kHeader);
  float* G = M + nv;

  // the sums and maxima start at zero on every call
  NA_CUDA(cudaMemsetAsync(hdr, 0, offsetof(Header, xf), stream));
  k_absmax<<<152 * 4, 256, 0, stream>>>(d_ultrasound, nv, &hdr->absmax[0], &hdr->nonfinite);
  k_absmax<<<152 * 4, 256, 0, stream>>>(d_moving, nm, &hdr->absmax[1], &hdr->nonfinite);
  NA_CUDA(cudaGetLastError());
  unsigned int h[3] = {0, 0, 0};
  NA_CUDA(cudaMemcpyAsync(h, &hdr->absmax[0], sizeof(h), cudaMemcpyDeviceToHost, stream));
  NA_CUDA(cudaStreamSynchronize(stream));
  if (h[2]) return fail(LC2_ERR_INVALID_ARGUMENT, "NaN/Inf in the input images");
  float umax, mmax;
  std::memcpy(&umax, &h[0], 4);
  std::memcpy(&mmax, &h[1], 4);

  // transform: moving-pixel coordinates of the virtual voxels
  lc2::Xform xf{};
  {
    lc2::XformD D{};
    double L[3][3] = {{0}}, t[3] = {0};
    for (int a = 0; a < warp_nd; ++a) {
      for (int b = 0; b < warp_nd; ++b) L[a][b] = matrix[(warp_nd + 1) * a + b];
      t[a] = matrix[(warp_nd + 1) * a + warp_nd];
    }
    for (int a = 0; a < 3; ++a) {
      double bs = t[a] - (double)moving->origin[a];
      for (int b = 0; b < 3; ++b) {
        D.A[3 * a + b] = L[a][b] * (double)virt->spacing[b] / (double)moving->spacing[a];
        bs += L[a][b] * (double)virt->origin[b];
      }
      D.b[a] = (a < warp_nd) ? bs / (double)moving->spacing[a] : 0.0;
    }
    xf = lc2::xform_split(D);
  }
  NA_CUDA(cudaMemcpyAsync(&hdr->xf, &xf, sizeof(xf), cudaMemcpyHostToDevice, stream));

  // fixed-point scales (same rules as the context path)
  const int r = patch_size;
  const int n = (2 * r + 1) * (2 * r + 1) * (nd == 3 ? 2 * r + 1 : 1);
  int b = 0;
  while (b < 21 && ((long long)n << (b + 2)) <= (1LL << 31)) ++b;
  const float tiny = 1e-30f;
  const float vu = std::fmax(umax, tiny), vm = std::fmax(mmax, tiny);
  const float vg = std::fmax((nd == 3 ? std::sqrt(3.0f) * 32.0f : std::sqrt(2.0f) * 8.0f) * mmax,
                             tiny);
  lc2::MomentParams P{};
  P.vx = virt->dim[0];
  P.vy = virt->dim[1];
  P.vz = virt->dim[2];
  P.r = r;
  P.n = n;
  P.zchunk = virt->dim[2];
  P.nzchunks = 1;
  const float two_b = std::ldexp(1.0f, b);
  P.qu = two_b / vu;
  P.qm = two_b / vm;
  P.qg = two_b / vg;
  const long double ln = n;
  P.thr_var = floor_clamp(1e-6L * ln * (ln - 1) * (long double)P.qu * (long double)P.qu);
  P.thr_m = floor_clamp(1e-12L * ln * (ln - 1) * (long double)P.qm * (long double)P.qm);
  P.thr_g = floor_clamp(1e-12L * ln * (ln - 1) * (long double)P.qg * (long double)P.qg);
  P.sig_scale = (float)(1.0L / ((long double)P.qu * std::sqrt(ln * (ln - 1))));
  P.sum_scale = std::ldexp(1.0f, 29) / vu;
  P.u_stride = P.m_stride = P.g_stride = 0;

  const dim3 blk(32, 8, 1);
  const dim3 grd((virt->dim[0] + 31) / 32, (virt->dim[1] + 7) / 8, virt->dim[2]);
  if (warp_nd == 3)
    lc2::k_warp<3, float><<<grd, blk, 0, stream>>>(d_moving, moving->dim[0], moving->dim[1],
                                                   moving->dim[2], P.vx, P.vy, P.vz, &hdr->xf, 0,
                                                   M, 0);
  else
    lc2::k_warp<2, float><<<grd, blk, 0, stream>>>(d_moving, moving->dim[0], moving->dim[1],
                                                   moving->dim[2], P.vx, P.vy, P.vz, &hdr->xf, 0,
                                                   M, 0);
  if (nd == 3)
    lc2::k_sobel<3><<<grd, blk, 0, stream>>>(M, P.vx, P.vy, P.vz, G, 0);
  else
    lc2::k_sobel<2><<<grd, blk, 0, stream>>>(M, P.vx, P.vy, P.vz, G, 0);
  const size_t smem = lc2::mom_smem_bytes(r);
  const dim3 mgrid((P.vx + lc2::kTX - 1) / lc2::kTX, (P.vy + lc2::kTY - 1) / lc2::kTY, 1);
  if (nd == 3) {
    NA_CUDA(cudaFuncSetAttribute(lc2::k_moments<3, float>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    lc2::k_moments<3, float><<<mgrid, lc2::kNT, smem, stream>>>(d_ultrasound, M, G, P, hdr->acc,
                                                                 0, nullptr, nullptr);
  } else {
    NA_CUDA(cudaFuncSetAttribute(lc2::k_moments<2, float>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    lc2::k_moments<2, float><<<mgrid, lc2::kNT, smem, stream>>>(d_ultrasound, M, G, P, hdr->acc,
                                                                 0, nullptr, nullptr);
  }
  k_ratio<<<1, 32, 0, stream>>>(hdr->acc, d_lc2);
  NA_CUDA(cudaGetLastError());
  return LC2_OK;
}
