// k_plain.cu — parameter derivation, the drop-in residual/Jacobian kernels
// (cedar_eval) and the single-instance block engine (Newton / DC / transient).
#include <mutex>
#include <cooperative_groups.h>
#include "kernels.cuh"

namespace cedar {

__device__ __forceinline__ int find_group(const DTpl &T, int d) {
  int gi = 0;
  while (d >= T.dev_end[gi]) ++gi;
  return gi;
}

// One CTA per instance: raw parameter block -> derived parameter block.
__global__ void derive_kernel(const DTpl *tpls, const int *inst_tpl, const long long *raw_off, const double *raw,
                              const long long *dpar_off, double *dpar, int n_inst) {
  int inst = blockIdx.x;
  if (inst >= n_inst) return;
  const DTpl &T = tpls[inst_tpl ? inst_tpl[inst] : 0];
  const double *r = raw + raw_off[inst];
  double *d = dpar + dpar_off[inst];
  for (int dv = threadIdx.x; dv < T.n_dev; dv += blockDim.x) {
    int gi = find_group(T, dv);
    const DGroup gr = T.grp[gi];
    int i = dv - (gi ? T.dev_end[gi - 1] : 0);
    derive_one(gr.model, r + gr.par_off + i, gr.n_inst, d + gr.dpar_off + i, gr.n_inst, T.vt);
  }
}

cudaError_t launch_derive(const DTpl *tpls_dev, const int *inst_tpl, const long long *raw_off, const double *raw,
                          const long long *dpar_off, double *dpar, int n_inst, int max_dev, cudaStream_t s) {
  if (n_inst <= 0) return cudaSuccess;
  int threads = max_dev >= 256 ? 256 : ((max_dev + 31) / 32) * 32;
  if (threads < 32) threads = 32;
  derive_kernel<<<n_inst, threads, 0, s>>>(tpls_dev, inst_tpl, raw_off, raw, dpar_off, dpar, n_inst);
  return cudaGetLastError();
}

// K1 (grid-wide): one thread per device instance.  Parameters are SoA, so a warp
// reads each parameter as one contiguous 256-byte segment; outputs are written
// contiguously per device (a warp writes one contiguous span).
__global__ void eval_kernel(DTpl T, const double *dpar, const double *x, const double *xdot, double t, double cj,
                            double *dout) {
  int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= T.n_dev) return;
  int gi = find_group(T, d);
  const DGroup gr = T.grp[gi];
  int i = d - (gi ? T.dev_end[gi - 1] : 0);
  const int *tm = T.term_orig + gr.term_off + i * gr.ntx;
  double v[CEDAR_MAX_TERM], vd[CEDAR_MAX_TERM];
  const bool need_vd = xdot && model_has_q(gr.model);   // only charge models read x'
  for (int k = 0; k < gr.ntx; ++k) {
    int u = tm[k];
    v[k] = u < 0 ? 0.0 : __ldg(x + u);
    vd[k] = (u < 0 || !need_vd) ? 0.0 : __ldg(xdot + u);
  }
  EvalCtx ctx{t, cj, 1.0, T.gmin, false, true};
  eval_device(gr.model, dpar + gr.dpar_off + i, gr.n_inst, v, vd, ctx, T.pwl, dout + gr.out_off + i, gr.n_inst);
}

// K2+K3 (grid-wide): J values in CSC order and residual rows, fixed-order sums,
// one thread per J slot / row.  Lists longer than kLongEval (supply rails) are
// summed by the long-list chunk warps below.
__device__ __forceinline__ void stamp_slot(const DTpl &T, const double *dout, double *F, double *J, int s) {
  if (J && s < T.n_csc && T.jcsc_ptr[s + 1] - T.jcsc_ptr[s] <= kLongEval) {
    double acc = 0.0;
    for (int k = T.jcsc_ptr[s]; k < T.jcsc_ptr[s + 1]; ++k) { int e = __ldg(T.jcsc_ent + k); acc = acc + signed_out(__ldg(dout + (e >> 1)), e); }
    J[s] = acc;
  }
  if (F && s < T.n && T.forg_ptr[s + 1] - T.forg_ptr[s] <= kLongEval) {
    double acc = 0.0;
    for (int k = T.forg_ptr[s]; k < T.forg_ptr[s + 1]; ++k) { int e = __ldg(T.forg_ent + k); acc = acc + signed_out(__ldg(dout + (e >> 1)), e); }
    F[s] = acc;
  }
}

// Long lists (supply rails), pass 1: one warp per fixed chunk of kLongChunkDev
// entries (chunk p of list i at long_off[i] + p).  Lane j sums the chunk's
// entries j, j + 32, ... in order (the warp's index loads are coalesced), then a
// fixed xor-butterfly over the 32 lane sums gives the chunk sum; a + b and b + a
// round alike, so every lane holds the same bits.
constexpr int kLongChunkDev = 256;
constexpr int kLongLaneLoads = kLongChunkDev / 32;
__device__ __forceinline__ void stamp_long_chunk(const DTpl &T, const double *dout, double *part, int p, int lane) {
  const int nl = T.n_long_jc + T.n_long_fo;
  int lo = 0, hi = nl;                       // list i with long_off[i] <= p < long_off[i + 1]
  while (hi - lo > 1) { const int mid = (lo + hi) >> 1; if (T.long_off[mid] <= p) lo = mid; else hi = mid; }
  const bool is_j = lo < T.n_long_jc;
  const int q = is_j ? T.long_jc[lo] : T.long_fo[lo - T.n_long_jc];
  const int *ptr = is_j ? T.jcsc_ptr : T.forg_ptr, *ent = is_j ? T.jcsc_ent : T.forg_ent;
  const int k0 = ptr[q] + (p - T.long_off[lo]) * kLongChunkDev;
  const int k1 = min(k0 + kLongChunkDev, ptr[q + 1]);
  // all of the lane's loads are issued ahead of its in-order adds
  int e[kLongLaneLoads]; double v[kLongLaneLoads];
#pragma unroll
  for (int j = 0; j < kLongLaneLoads; ++j) { const int k = k0 + lane + 32 * j; e[j] = k < k1 ? __ldg(ent + k) : -1; }
#pragma unroll
  for (int j = 0; j < kLongLaneLoads; ++j) v[j] = e[j] >= 0 ? __ldg(dout + (e[j] >> 1)) : 0.0;
  double acc = 0.0;
#pragma unroll
  for (int j = 0; j < kLongLaneLoads; ++j) if (e[j] >= 0) acc = acc + signed_out(v[j], e[j]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc = acc + __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) part[p] = acc;
}

// One launch for both (they read only the device outputs): the first
// `long_blocks` blocks run the long-list chunks (one warp each), the rest the
// J slots and rows, so the supply-rail sums overlap the ordinary stamping.
__global__ void stamp_kernel(DTpl T, const double *dout, double *F, double *J, double *part, int long_blocks) {
  if ((int)blockIdx.x < long_blocks) {
    const int p = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
    if (p < T.n_long_part) stamp_long_chunk(T, dout, part, p, threadIdx.x & 31);   // warp-uniform test
    return;
  }
  stamp_slot(T, dout, F, J, (int)((blockIdx.x - long_blocks) * blockDim.x + threadIdx.x));
}

// Pass 2: one CTA per long list; thread t sums the list's chunk sums t, t + 256,
// ... in order (coalesced), then a fixed xor-butterfly per warp and a fixed
// pairwise tree over the 8 warp sums.
constexpr int kLongThreads = 256;
static_assert(kLongThreads == 256, "the final tree combines 8 warp sums");
__global__ void __launch_bounds__(kLongThreads) stamp_long_final_kernel(DTpl T, const double *part, double *F, double *J) {
  __shared__ double red[kLongThreads / 32];
  const int i = blockIdx.x;
  const bool is_j = i < T.n_long_jc;
  const int q = is_j ? T.long_jc[i] : T.long_fo[i - T.n_long_jc];
  const int p0 = T.long_off[i], p1 = T.long_off[i + 1];
  double acc = 0.0;
  int k = p0 + threadIdx.x;
  for (; k + 7 * kLongThreads < p1; k += 8 * kLongThreads) {   // loads ahead of the in-order adds
    double v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = part[k + j * kLongThreads];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc = acc + v[j];
  }
  for (; k < p1; k += kLongThreads) acc = acc + part[k];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc = acc + __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    const double s01 = red[0] + red[1], s23 = red[2] + red[3], s45 = red[4] + red[5], s67 = red[6] + red[7];
    const double r = (s01 + s23) + (s45 + s67);
    if (is_j) { if (J) J[q] = r; }
    else if (F) F[q] = r;
  }
}

cudaError_t launch_eval(const DTpl &T, const DTpl *T_dev, const double *dpar, const double *x, const double *xdot,
                        double t, double cj, double *dout, double *part, double *F, double *J, cudaStream_t s) {
  (void)T_dev;
  const int th = 256;
  if (T.n_dev > 0) eval_kernel<<<(T.n_dev + th - 1) / th, th, 0, s>>>(T, dpar, x, xdot, t, cj, dout);
  const int m = T.n_csc > T.n ? T.n_csc : T.n, warps = th / 32;
  const int nlong = T.n_long_jc + T.n_long_fo;
  const int long_blocks = nlong > 0 ? (T.n_long_part + warps - 1) / warps : 0;
  stamp_kernel<<<long_blocks + (m + th - 1) / th, th, 0, s>>>(T, dout, F, J, part, long_blocks);
  if (nlong > 0) stamp_long_final_kernel<<<nlong, kLongThreads, 0, s>>>(T, part, F, J);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the residual / Jacobian evaluation.
//
// The device outputs that eval_kernel writes and stamp_kernel reads normally live
// in a buffer the handle allocates.  For callers that may not allocate device
// memory at the point of the call, this scratch is instead a file-scope device
// array of fixed size that every GPU loading this library holds until the
// process exits.  Host code cannot use the array's name as a device address: the
// address is looked up once per device with cudaGetSymbolAddress, with that
// device current, and cached.  Every call shares the one array per device, so
// calls whose kernels overlap on the GPU race on it; serialise them (one stream,
// or events).  eval_kernel overwrites every output slot it uses before
// stamp_kernel reads it, so nothing needs clearing between calls.
static __device__ __align__(256) double g_eval_scratch[kEvalScratchMax];

static std::mutex g_scratch_mu;
static double *g_scratch_ptr[kMaxDevices] = {};

cudaError_t eval_scratch_address(double **ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_eval_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *ptr = g_scratch_ptr[dev];
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// FP64 issue-rate probe: the denominator of the batched kernel's roofline.
// Every thread of lanes below `active_lanes` runs 8 independent DFMA chains of
// `iters` steps; registers only, no memory traffic in the loop.
__global__ void fp64_probe_kernel(double *sink, int iters, int active_lanes) {
  const int lane = threadIdx.x & 31;
  double a0 = 1e-9 * threadIdx.x, a1 = a0 + 0.125, a2 = a0 + 0.25, a3 = a0 + 0.375;
  double a4 = a0 + 0.5, a5 = a0 + 0.625, a6 = a0 + 0.75, a7 = a0 + 0.875;
  const double m = 0.9999999, c = 1e-7;
  if (lane < active_lanes) {
    for (int i = 0; i < iters; ++i) {
      a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
      a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
  }
  const double r = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (r == -1.0) sink[blockIdx.x] = r;  // never true; keeps the chains live
}

// FP64 dependent-operation latency: one warp, every lane one chain of `iters`
// dependent DFMAs (unrolled by 8); lane 0 reads the SM clock around the chain.
__global__ void fp64_latency_kernel(double *sink, long long *cycles, int iters) {
  double a = 0.5 + 1e-9 * threadIdx.x;
  const double m = 0.9999999, c = 1e-7;
  const long long c0 = clock64();
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a = fma(a, m, c);
  }
  if (a == -1.0) sink[threadIdx.x] = a;    // never true; keeps the chain live
  const long long c1 = clock64();
  if (threadIdx.x == 0) *cycles = c1 - c0;
}

cudaError_t launch_fp64_latency(int iters, double *cycles_per_op, double *ns_per_op) {
  double *sink = nullptr;
  long long *cyc = nullptr;
  cudaError_t e = cudaMalloc(&sink, 32 * sizeof(double) + sizeof(long long));
  if (e != cudaSuccess) return e;
  cyc = reinterpret_cast<long long *>(sink + 32);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  float best = 1e30f;
  long long best_cyc = 0;
  for (int rep = 0; rep < 4; ++rep) {   // first launch warms up; best of the rest
    cudaEventRecord(e0);
    fp64_latency_kernel<<<1, 32>>>(sink, cyc, iters);
    cudaEventRecord(e1);
    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
    float t = 0; cudaEventElapsedTime(&t, e0, e1);
    long long c = 0;
    if ((e = cudaMemcpy(&c, cyc, sizeof c, cudaMemcpyDeviceToHost)) != cudaSuccess) break;
    if (rep > 0 && t < best) { best = t; best_cyc = c; }
  }
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess) return e;
  const double ops = 8.0 * iters;
  if (cycles_per_op) *cycles_per_op = best_cyc / ops;
  if (ns_per_op) *ns_per_op = best * 1e6 / ops;
  return cudaGetLastError();
}

cudaError_t launch_fp64_probe(int active_lanes, int iters, double *gflops, double *ms) {
  int dev = 0, nsm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  const int blocks = nsm * 8, threads = 256;
  double *sink = nullptr;
  if ((e = cudaMalloc(&sink, blocks * sizeof(double))) != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 6; ++rep) {   // first launch warms up; best of the rest
    cudaEventRecord(e0);
    fp64_probe_kernel<<<blocks, threads>>>(sink, iters, active_lanes);
    cudaEventRecord(e1);
    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
    float t = 0; cudaEventElapsedTime(&t, e0, e1);
    if (rep > 0 && t < best) best = t;
  }
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess) return e;
  // useful flops: 2 per FMA on the active lanes only
  const double fmas = 8.0 * iters * (double)blocks * threads * (active_lanes / 32.0);
  if (gflops) *gflops = 2.0 * fmas / (best * 1e-3) / 1e9;
  if (ms) *ms = best;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// One circuit on every thread of a cooperative grid (large circuits).
//
// The engine's group interface over the whole grid: rank / size are the global
// thread index and count, sync() is a grid-wide barrier (cooperative launch, so
// every block is resident), and a reduction combines each block's threads as
// BlockGroup does, posts the block's value to global scratch, synchronises the
// grid and lets every block combine the posted values in block order, so every
// thread holds the same result.  max / min are exact and the step-error ratio is
// merged as fractions, so the engine takes the decisions it takes on one CTA.
// Two scratch buffers alternate: a block that moves on to the next reduction
// writes the other buffer while slower blocks still read this one.
struct GridGroup {
  int rank, size;
  double *red;            // shared scratch (>= 96 doubles)
  double *gred;           // global scratch: 2 buffers of 3 doubles per block
  mutable int ph;         // buffer of the next reduction
  __device__ GridGroup(double *r, double *g)
      : rank(blockIdx.x * blockDim.x + threadIdx.x), size(gridDim.x * blockDim.x), red(r), gred(g), ph(0) {}
  __device__ void sync() const { cooperative_groups::this_grid().sync(); }
  __device__ double *buf() const { double *b = gred + (size_t)(ph & 1) * 3 * gridDim.x; ++ph; return b; }
  __device__ double reduce(double v, bool is_max) const {
    BlockGroup blk(red);
    const double bv = blk.reduce(v, is_max);
    double *b = buf();
    if (threadIdx.x == 0) b[blockIdx.x] = bv;
    sync();
    if (threadIdx.x == 0) {
      double r = b[0];
      for (int i = 1; i < (int)gridDim.x; ++i) { const double w = b[i]; r = is_max ? (w > r ? w : r) : (w < r ? w : r); }
      red[0] = r;
    }
    __syncthreads();
    const double r = red[0];
    __syncthreads();
    return r;
  }
  __device__ bool any(bool p) const { return reduce(p ? 1.0 : 0.0, true) != 0.0; }
  __device__ double max(double v) const { return reduce(v, true); }
  __device__ double min(double v) const { return reduce(v, false); }
  __device__ double ratio(MaxRatio m) const {
    for (int o = 16; o > 0; o >>= 1) {
      const double n2 = __shfl_xor_sync(0xffffffffu, m.num, o), d2 = __shfl_xor_sync(0xffffffffu, m.den, o);
      const bool b2 = __shfl_xor_sync(0xffffffffu, (int)m.bad, o) != 0;
      m.merge(n2, d2, b2);
    }
    const int warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) { red[3 * warp] = m.num; red[3 * warp + 1] = m.den; red[3 * warp + 2] = m.bad ? 1.0 : 0.0; }
    __syncthreads();
    double *b = buf();
    if (threadIdx.x == 0) {
      MaxRatio r; r.num = red[0]; r.den = red[1]; r.bad = red[2] != 0.0;
      for (int i = 1; i < nw; ++i) r.merge(red[3 * i], red[3 * i + 1], red[3 * i + 2] != 0.0);
      b[3 * blockIdx.x] = r.num; b[3 * blockIdx.x + 1] = r.den; b[3 * blockIdx.x + 2] = r.bad ? 1.0 : 0.0;
    }
    sync();
    if (threadIdx.x == 0) {
      MaxRatio r; r.num = b[0]; r.den = b[1]; r.bad = b[2] != 0.0;
      for (int i = 1; i < (int)gridDim.x; ++i) r.merge(b[3 * i], b[3 * i + 1], b[3 * i + 2] != 0.0);
      red[0] = r.value();
    }
    __syncthreads();
    const double r = red[0];
    __syncthreads();
    return r;
  }
};

// The single-circuit body on a thread group G (one CTA or a whole grid):
// mode 0 = transient, 1 = one Newton solve, 2 = DC operating point.
template <class G>
__device__ void plain_body(const PlainArgs &a, G g, double *ws) {
  const DTpl &T = *a.T;
  Engine<G> E(T, a.dpar, ws, g);
  E.dense = a.dense;
  for (int i = g.rank; i < T.n; i += g.size) E.w.x[i] = a.x[T.order[i]];
  g.sync();
  const EngOpts &o = a.opts;
  EngStats st{};
  st.hmin_seen = 1e300;
  const double rel = o.nr_factor * o.reltol, av = o.nr_factor * o.abstol_v, ai = o.nr_factor * o.abstol_i;
  if (a.mode == 0) {
    Sink sk{};
    sk.t_out = a.t_out; sk.x_out = a.x_out; sk.cap = a.cap; sk.count = 0;
    sk.tstart = o.tstart; sk.tstop = o.tstop;
    E.tran(E.w.x, o, sk, st, nullptr);
    if (g.rank == 0 && a.count) *a.count = sk.count;
  } else if (a.mode == 1) {
    for (int e = g.rank; e < T.n; e += g.size) E.w.hist[T.eq_pos[e]] = a.hist ? a.hist[e] : 0.0;
    g.sync();
    EvalCtx ctx{a.t, a.cj, 1.0, T.gmin, false, false};
    int r = E.newton(E.w.x, ctx, E.w.hist, rel, av, ai, o.max_newton, 0.0, 0.0);
    st.newton_iters = r < 0 ? -r : r;
    st.status = r > 0 ? CEDAR_ST_OK : (r == 0 ? CEDAR_ST_ZERO_PIVOT : CEDAR_ST_NEWTON);
  } else {
    long long it = 0;
    st.status = E.dcop(E.w.x, a.t, rel, av, ai, &it);
    st.dc_iters = it;
  }
  g.sync();
  for (int i = g.rank; i < T.n; i += g.size) a.x[T.order[i]] = E.w.x[i];
  if (g.rank == 0 && a.stats) *a.stats = st;
}

// Single instance on one CTA.  Workspace in dynamic shared memory when it fits,
// else in global memory (a.ws_global).
__global__ void plain_kernel(PlainArgs a) {
  extern __shared__ double smem[];
  double *ws = a.ws_global ? a.ws_global : smem + 128;
  plain_body(a, BlockGroup(smem), ws);
}

// Single instance on a cooperative grid; workspace in global memory.
constexpr int kGridThreads = 256;
__global__ void __launch_bounds__(kGridThreads) plain_grid_kernel(PlainArgs a, double *gred) {
  __shared__ double red[128];
  plain_body(a, GridGroup(red, gred), a.ws_global);
}

cudaError_t grid_geometry(int work, int *blocks) {
  int dev = 0, nsm = 0, per = 0, coop = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev)) != cudaSuccess) return e;
  if (!coop) return cudaErrorNotSupported;
  if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, plain_grid_kernel, kGridThreads, 0)) != cudaSuccess)
    return e;
  const int want = (work + kGridThreads - 1) / kGridThreads;
  const int cap = nsm * (per < 1 ? 1 : per);
  *blocks = want < 1 ? 1 : (want < cap ? want : cap);
  return cudaSuccess;
}

cudaError_t launch_plain_grid(const PlainArgs &a, int blocks, double *gred, cudaStream_t s) {
  PlainArgs aa = a;
  double *g = gred;
  void *args[] = {&aa, &g};
  return cudaLaunchCooperativeKernel((const void *)plain_grid_kernel, dim3(blocks), dim3(kGridThreads), args, 0, s);
}

cudaError_t launch_plain(const PlainArgs &a, int wsd, int threads, cudaStream_t s) {
  size_t smem = 128 * sizeof(double);
  if (!a.ws_global) smem += (size_t)wsd * sizeof(double);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  plain_kernel<<<1, threads, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace cedar
