// k_batch.cu — batched persistent engine: thousands of sweep / Monte Carlo
// instances of uneven sizes in one launch.  Each group of K lanes owns one
// instance at a time (its own step size, Newton state and history in shared
// memory); when an instance reaches tstop or fails, the group retires it and
// takes the next instance from a device-side queue (a single fetch-and-add
// counter: no group ever waits on another).
#include "kernels.cuh"

namespace cedar {

template <int K>
__global__ void __launch_bounds__(256) batch_kernel(BatchDev b) {
  extern __shared__ double smem[];
  const int tiles_per_block = blockDim.x / K;
  const int tile = threadIdx.x / K;
  TileGroup<K> g;
  double *ws = b.ws_in_smem ? smem + (size_t)tile * b.ws_stride
                            : b.ws_global + ((size_t)blockIdx.x * tiles_per_block + tile) * b.ws_stride;
  for (;;) {
    int job = 0;
    if (g.rank == 0) job = atomicAdd(b.head, 1);
    job = g.bcast(job);
    if (job >= b.n_inst) break;
    const int inst = b.queue[job];
    const int ti = b.inst_tpl[inst];
    const DTpl &T = b.tpls[ti];
    Engine<TileGroup<K>> E(T, b.dpar + b.inst_dpar[inst], ws, g);
    const long long xo = b.x0_off ? b.x0_off[inst] : -1;
    for (int i = g.rank; i < T.n; i += K) E.w.x[i] = xo >= 0 ? b.x0[xo + T.order[i]] : 0.0;
    const long long dxo = b.dx_off ? b.dx_off[inst] : -1;
    const double *pert = nullptr;
    if (dxo >= 0) {
      for (int i = g.rank; i < T.n; i += K) E.w.qt[i] = b.dx[dxo + T.order[i]];
      pert = E.w.qt;
    }
    g.sync();
    Sink sk{};
    sk.t_out = nullptr;
    sk.probes_int = b.probes_int ? b.probes_int + (size_t)ti * b.np : nullptr;
    sk.np = b.np; sk.ns = b.ns;
    sk.samp = (b.samples && b.np > 0 && b.ns > 0) ? b.samples + (size_t)inst * b.np * b.ns : nullptr;
    sk.tstart = b.opts.tstart; sk.tstop = b.opts.tstop;
    EngStats st;
    E.tran(E.w.x, b.opts, sk, st, pert);
    if (b.x_final)
      for (int i = g.rank; i < T.n; i += K) b.x_final[(size_t)inst * b.n_max + T.order[i]] = E.w.x[i];
    if (g.rank == 0 && b.stats) b.stats[inst] = st;
    g.sync();
  }
}

template <int K>
static cudaError_t launch_k(const BatchDev &b, int warps, int grid, size_t smem, cudaStream_t s) {
  static int configured = -1;
  if ((int)smem > 48 * 1024 && configured < (int)smem) {
    cudaError_t e = cudaFuncSetAttribute(batch_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = (int)smem;
  }
  batch_kernel<K><<<grid, warps * 32, smem, s>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_batch(const BatchDev &b, int K, int warps, int grid, size_t smem, cudaStream_t s) {
  switch (K) {
    case 1: return launch_k<1>(b, warps, grid, smem, s);
    case 2: return launch_k<2>(b, warps, grid, smem, s);
    case 4: return launch_k<4>(b, warps, grid, smem, s);
    case 8: return launch_k<8>(b, warps, grid, smem, s);
    case 16: return launch_k<16>(b, warps, grid, smem, s);
    case 32: return launch_k<32>(b, warps, grid, smem, s);
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
