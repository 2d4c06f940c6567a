// k_dispatch.cu — selects the per-lane-count instantiation of the batched and
// adjoint kernels (k_batch.cu and k_adjoint.cu are compiled once per K).
#include "kernels.cuh"

namespace cedar {

#define CEDAR_PER_K(X) X(1) X(2) X(4) X(8) X(16) X(32)
#define CEDAR_DECL(K)                                                                                        \
  cudaError_t launch_batch_k##K(const BatchDev &b, int warps, int grid, size_t smem, cudaStream_t st);      \
  cudaError_t configure_batch_k##K(int warps, size_t smem, bool in_smem, int max_per_sm, int *per_sm);                      \
  cudaError_t launch_adjoint_k##K(const AdjDev &a, int warps, int grid, size_t smem, cudaStream_t st);
CEDAR_PER_K(CEDAR_DECL)
#undef CEDAR_DECL

cudaError_t launch_batch(const BatchDev &b, int K, int warps, int grid, size_t smem, cudaStream_t st) {
  switch (K) {
#define CEDAR_CASE(K) case K: return launch_batch_k##K(b, warps, grid, smem, st);
    CEDAR_PER_K(CEDAR_CASE)
#undef CEDAR_CASE
  }
  return cudaErrorInvalidValue;
}

cudaError_t configure_batch(int K, int warps, size_t smem, bool in_smem, int max_per_sm, int *per_sm) {
  switch (K) {
#define CEDAR_CASE(K) case K: return configure_batch_k##K(warps, smem, in_smem, max_per_sm, per_sm);
    CEDAR_PER_K(CEDAR_CASE)
#undef CEDAR_CASE
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_adjoint(const AdjDev &a, int K, int warps, int grid, size_t smem, cudaStream_t st) {
  switch (K) {
#define CEDAR_CASE(K) case K: return launch_adjoint_k##K(a, warps, grid, smem, st);
    CEDAR_PER_K(CEDAR_CASE)
#undef CEDAR_CASE
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
