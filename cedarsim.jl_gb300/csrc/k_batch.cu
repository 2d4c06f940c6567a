// k_batch.cu — batched persistent engine: the transient kernel and its launch.
#include <cmath>
#include "batch_slot.cuh"

namespace cedar {

// Slot state machines of wide slots in shared memory (1) or registers (0).  In
// shared memory the kernel needs 118 registers instead of 234, but on the
// 4096-chain workload that bought nothing: at 8 warps per SM both ran at 13.9 M
// instance-steps/s, and the extra CTAs the registers allow shrink the L1 that
// caches the task lists (12 warps per SM: 12.8 M).  Registers stay the default.
#ifndef CEDAR_SLOT_SMEM
#define CEDAR_SLOT_SMEM 0
#endif

// Minimum resident CTAs per SM the register allocation must allow (1: up to
// 255 registers per thread).
#ifndef CEDAR_BATCH_MIN_BLOCKS
#define CEDAR_BATCH_MIN_BLOCKS 1
#endif

// SMEM: the slot workspaces live in shared memory.  Fixing this at compile time
// lets every workspace pointer derive from the shared-memory base, so the
// compiler issues shared-memory loads and stores rather than generic ones.
// REC: record mode (one instance, every accepted point; the single-circuit transient)
template <int K, bool SMEM, bool REC = false>
__global__ void __launch_bounds__(256, CEDAR_BATCH_MIN_BLOCKS) batch_kernel(BatchDev b) {
  extern __shared__ double smem[];
  const int slots_per_block = blockDim.x / K;
  const int slot = threadIdx.x / K;
  // The slot's state machine: in shared memory for wide slots (one copy per slot,
  // written identically by its lanes), which leaves the registers to the Newton
  // iteration; in each lane's registers for narrow slots (many slots per CTA).
#if CEDAR_SLOT_SMEM
  __shared__ Slot<K> slot_state[K >= 16 ? 256 / K : 1];
  Slot<K> s_local;
  Slot<K> &s = K >= 16 ? slot_state[K >= 16 ? slot : 0] : s_local;
#else
  Slot<K> s;
#endif
  double *ws;
  if constexpr (SMEM) ws = smem + (size_t)slot * b.ws_stride;
  else ws = b.ws_global + ((size_t)blockIdx.x * slots_per_block + slot) * b.ws_stride;
  s.rp = RP_NEWINST; s.active = false;
  s.gsi = blockIdx.x * slots_per_block + slot; s.qblk = -1; s.dense = false; s.jdense = false;
  s.nrel = b.opts.nr_factor * b.opts.reltol; s.nav = b.opts.nr_factor * b.opts.abstol_v;
  s.nai = b.opts.nr_factor * b.opts.abstol_i;
  for (;;) {
    if (!s.active && s.rp != RP_IDLE) s.template resume<REC>(b, ws);
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
static cudaError_t configure(F *kern, int threads, size_t smem, int max_per_sm, int *per_sm) {
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int nb = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, threads, smem)) != cudaSuccess) return e;
  if (nb < 1) nb = 1;
  if (max_per_sm > 0 && nb > max_per_sm) nb = max_per_sm;
  cudaFuncAttributes fa{};
  if ((e = cudaFuncGetAttributes(&fa, kern)) != cudaSuccess) return e;
  int dev = 0, smsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  const double need = (double)nb * (double)(smem + fa.sharedSizeBytes + 1024);
  int pct = (int)std::ceil(100.0 * need / (double)(smsm > 0 ? smsm : 1));
  pct = pct < 1 ? 1 : (pct > 100 ? 100 : pct);
  if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct)) != cudaSuccess) return e;
  if (per_sm) *per_sm = nb;
  return cudaSuccess;
}

// This file is compiled once per lanes-per-instance value (-DCEDAR_LANES=K, see
// build.py) so the instantiations build in parallel; k_dispatch.cu selects one.
#ifndef CEDAR_LANES
#error "compile with -DCEDAR_LANES=<lanes per instance>"
#endif
#define CEDAR_CAT2(a, b) a##b
#define CEDAR_CAT(a, b) CEDAR_CAT2(a, b)

cudaError_t CEDAR_CAT(launch_batch_k, CEDAR_LANES)(const BatchDev &b, int warps, int grid, size_t smem, cudaStream_t st) {
  constexpr int K = CEDAR_LANES;
  if (b.ws_in_smem) batch_kernel<K, true><<<grid, warps * 32, smem, st>>>(b);
  else batch_kernel<K, false><<<grid, warps * 32, smem, st>>>(b);
  return cudaGetLastError();
}

cudaError_t CEDAR_CAT(configure_batch_k, CEDAR_LANES)(int warps, size_t smem, bool in_smem, int max_per_sm, int *per_sm) {
  constexpr int K = CEDAR_LANES;
  const int th = warps * 32;
  return in_smem ? configure(batch_kernel<K, true>, th, smem, max_per_sm, per_sm)
                 : configure(batch_kernel<K, false>, th, smem, max_per_sm, per_sm);
}

#if CEDAR_LANES == 32
cudaError_t launch_batch_record(const BatchDev &b, size_t smem, cudaStream_t st) {
  cudaError_t e;
  if (smem > 0) {
    if ((e = cudaFuncSetAttribute(batch_kernel<32, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem)) != cudaSuccess)
      return e;
    batch_kernel<32, true, true><<<1, 32, smem, st>>>(b);
  } else {
    batch_kernel<32, false, true><<<1, 32, 0, st>>>(b);
  }
  return cudaGetLastError();
}
#endif

}  // namespace cedar
