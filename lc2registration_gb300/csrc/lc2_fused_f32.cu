// Fused LC2 kernels for f32 storage (all patch radii), one translation unit
// per storage type so the instantiations compile in parallel; also the
// self-test kernel of the warp-specialised kernel's bounded waits.
#include "lc2_fused_ws.cuh"

namespace lc2 {
LC2_DEFINE_FUSED_LAUNCH(float)

// One warp waits, with the warp-specialised kernel's mbar_wait, for a
// barrier whose only expected arrival never comes: the wait gives up after
// its one-second limit, sets the CTA's abort flag and raises `err`, and the
// kernel returns.
__global__ void __launch_bounds__(32) k_wait_probe(int* __restrict__ err) {
  __shared__ __align__(8) unsigned long long bar;
  __shared__ volatile int s_abort;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    s_abort = 0;
  }
  __syncthreads();
  mbar_wait(&bar, 0u, &s_abort, err);
}

cudaError_t wait_probe_launch(int* err, cudaStream_t stream) {
  k_wait_probe<<<1, 32, 0, stream>>>(err);
  return cudaGetLastError();
}
}  // namespace lc2
