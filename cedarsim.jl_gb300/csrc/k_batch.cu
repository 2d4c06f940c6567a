// k_batch.cu — batched persistent engine: the transient kernel and its launch.
#include <cmath>
#include "batch_slot.cuh"

namespace cedar {

// Minimum resident CTAs per SM the register allocation must allow (1: up to
// 255 registers per thread).
#ifndef CEDAR_BATCH_MIN_BLOCKS
#define CEDAR_BATCH_MIN_BLOCKS 1
#endif

template <int K>
__global__ void __launch_bounds__(256, CEDAR_BATCH_MIN_BLOCKS) batch_kernel(BatchDev b) {
  extern __shared__ double smem[];
  Slot<K> s;
  const int slots_per_block = blockDim.x / K;
  const int slot = threadIdx.x / K;
  double *ws = b.ws_in_smem ? smem + (size_t)slot * b.ws_stride
                            : b.ws_global + ((size_t)blockIdx.x * slots_per_block + slot) * b.ws_stride;
  s.rp = RP_NEWINST; s.active = false;
  s.gsi = blockIdx.x * slots_per_block + slot; s.qblk = -1; s.dense = false; s.jdense = false;
  s.nrel = b.opts.nr_factor * b.opts.reltol; s.nav = b.opts.nr_factor * b.opts.abstol_v;
  s.nai = b.opts.nr_factor * b.opts.abstol_i;
  for (;;) {
    if (!s.active && s.rp != RP_IDLE) s.resume(b, ws);
    __syncwarp();
    const unsigned am = __ballot_sync(FULL, s.active);
    if (am == 0) break;
    const unsigned amd = __ballot_sync(FULL, s.active && s.jdense);
    if (s.active) {
      if (amd == 0) newton_iteration<K, false>(s, am);
      else if (!s.jdense) newton_iteration<K, false>(s, am & ~amd);
      else newton_iteration<K, true>(s, amd, &b);
    }
    __syncwarp();
  }
}

// Resident CTAs per SM for this launch shape (registers and shared memory), and
// the shared-memory carve-out that holds exactly those CTAs: the rest of the
// unified L1 / shared storage stays L1, which caches the template's task lists.
template <class F>
static cudaError_t configure(F *kern, int threads, size_t smem, int *per_sm) {
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int nb = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads, smem)) != cudaSuccess) return e;
  if (nb < 1) nb = 1;
  int dev = 0, smsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  const double need = (double)nb * (double)(smem + 1024);
  int pct = (int)std::ceil(100.0 * need / (double)(smsm > 0 ? smsm : 1));
  pct = pct < 1 ? 1 : (pct > 100 ? 100 : pct);
  if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct)) != cudaSuccess) return e;
  if (per_sm) *per_sm = nb;
  return cudaSuccess;
}

template <int K>
static cudaError_t launch_k(const BatchDev &b, int warps, int grid, size_t smem, cudaStream_t st) {
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

cudaError_t configure_batch(int K, int warps, size_t smem, int *per_sm) {
  const int th = warps * 32;
  switch (K) {
    case 1: return configure(batch_kernel<1>, th, smem, per_sm);
    case 2: return configure(batch_kernel<2>, th, smem, per_sm);
    case 4: return configure(batch_kernel<4>, th, smem, per_sm);
    case 8: return configure(batch_kernel<8>, th, smem, per_sm);
    case 16: return configure(batch_kernel<16>, th, smem, per_sm);
    case 32: return configure(batch_kernel<32>, th, smem, per_sm);
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
