// k_batch.cu — batched persistent engine: the transient kernel and its launch.
#include "batch_slot.cuh"

namespace cedar {

template <int K>
__global__ void __launch_bounds__(256, 1) batch_kernel(BatchDev b) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31;
  Slot<K> s;
  s.rank = lane % K;
  s.smask = (K == 32) ? FULL : (((1u << K) - 1u) << (lane - s.rank));
  const int slots_per_block = blockDim.x / K;
  const int slot = threadIdx.x / K;
  double *ws = b.ws_in_smem ? smem + (size_t)slot * b.ws_stride
                            : b.ws_global + ((size_t)blockIdx.x * slots_per_block + slot) * b.ws_stride;
  s.rp = RP_NEWINST; s.active = false;
  s.nrel = b.opts.nr_factor * b.opts.reltol; s.nav = b.opts.nr_factor * b.opts.abstol_v;
  s.nai = b.opts.nr_factor * b.opts.abstol_i;
  for (;;) {
    if (!s.active && s.rp != RP_IDLE) s.resume(b, ws);
    __syncwarp();
    const unsigned am = __ballot_sync(FULL, s.active);
    if (am == 0) break;
    if (s.active) newton_iteration(s, am);
    __syncwarp();
  }
}

template <int K>
static cudaError_t launch_k(const BatchDev &b, int warps, int grid, size_t smem, cudaStream_t st) {
  static int configured = -1;
  if ((int)smem > 48 * 1024 && configured < (int)smem) {
    cudaError_t e = cudaFuncSetAttribute(batch_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = (int)smem;
  }
  batch_kernel<K><<<grid, warps * 32, smem, st>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_batch(const BatchDev &b, int K, int warps, int grid, size_t smem, cudaStream_t st) {
  switch (K) {
    case 1: return launch_k<1>(b, warps, grid, smem, st);
    case 2: return launch_k<2>(b, warps, grid, smem, st);
    case 4: return launch_k<4>(b, warps, grid, smem, st);
    case 8: return launch_k<8>(b, warps, grid, smem, st);
    case 16: return launch_k<16>(b, warps, grid, smem, st);
    case 32: return launch_k<32>(b, warps, grid, smem, st);
  }
  return cudaErrorInvalidValue;
}

int batch_max_smem_optin() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

}  // namespace cedar
