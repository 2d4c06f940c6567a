// kernels.cuh — kernel launch interface shared by api.cu and the kernel TUs.
#pragma once
#include <cuda_runtime.h>
#include "engine.cuh"

namespace cedar {

// Batched run description (device pointers).
struct BatchDev {
  const DTpl *tpls;              // [n_templates]
  const int *inst_tpl;           // [n_inst]
  const long long *inst_dpar;    // [n_inst] offset into dpar
  const double *dpar;
  const long long *x0_off; const double *x0;   // original order, -1 = zeros
  const long long *dx_off; const double *dx;   // perturbation after DC op
  const int *probes_int;         // [n_templates * np] internal unknowns
  int np, ns;
  double *samples;               // [n_inst * np * ns]
  double *x_final; int n_max;    // [n_inst * n_max] original order
  EngStats *stats;               // [n_inst]
  const int *queue;              // dequeue order (instance ids), in blocks of one template
  const int *qblk_beg;           // [n_qblk + 1] start of each template block in queue
  int *qblk_head;                // [n_qblk] next position to take in each block
  int n_qblk;
  int n_inst;
  EngOpts opts;
  int ws_stride;                 // doubles per group workspace
  double *ws_global;             // global workspaces when not in shared memory
  int ws_in_smem;
  // resumable runs: every instance stops at its first step starting at or after
  // t_until (a soft stop: the step sequence is the one of an uninterrupted run),
  // leaving its integrator state in rows / row_vec for the next launch
  double t_until;
  struct StateRow *rows;         // [n_inst]
  double *row_vec;               // [n_inst * 6 * n_max]: xn xm1 xm2 qn qm1 qd
  int *n_running;                // instances left unfinished by this launch
  // adjoint tape (forward recording; tape_t == null: off).  Per instance
  // tape_cap + 1 entries (entry 0 = the start point, entry k = accepted step k)
  // of time, order (1 = BE, 2 = BDF2), supply power and probe value, and every
  // ckpt_every steps a checkpoint (x_k, x_{k-1}) in internal order.
  double *tape_t; signed char *tape_ord; double *tape_p, *tape_v;
  long long tape_cap;
  double *ckpt; int ckpt_every;
  const int4 *obj_idx;           // [n_templates] internal (vnode, ibranch, probe, 0)
  // dense DC fallback scratch: per global slot dense_stride doubles (an n_max x
  // n_max matrix, a right-hand side and the pivots); null: no fallback
  double *dense_ws; long long dense_stride; int dense_nmax;
  int dc_only;                   // retire every instance at its DC operating point
  // record mode (one instance only: the single-circuit transient): every accepted
  // point's time and state (original order) into rec_t[cap] / rec_x[cap * n];
  // *rec_count counts every point, also those past cap.  rec_t == null: off.
  double *rec_t, *rec_x; long long rec_cap; long long *rec_count;
};

// slice helpers of the adjoint tape
__host__ __device__ inline long long tape_stride(long long cap) { return cap + 1; }
__host__ __device__ inline long long ckpt_count(long long cap, int every) { return cap / every + 1; }

// Discrete adjoint launch (k_adjoint.cu): replays each instance's recorded steps
// segment by segment from its checkpoints and sweeps the adjoint backwards.
struct AdjObj { int iv, ib, ip, pad; double level, w_energy, w_delay, w_final; };  // internal indices
struct AdjDev {
  BatchDev b;                    // templates, parameters, tape, queue, options
  const long long *raw_off; const double *raw;   // raw parameter blocks (W, r)
  const AdjObj *obj;             // [n_templates]
  const double *tstar;           // [n_inst]
  double *phi;                   // [n_inst]
  double *grad; int np_max;      // [n_inst * np_max]
  int *status;                   // [n_inst]
  double *segx;                  // [n_inst * (ckpt_every + 1) * n_max] replayed states
  const EngStats *fwd;           // forward stats (steps taken, status)
};
cudaError_t launch_adjoint(const AdjDev &a, int K, int warps_per_cta, int grid, size_t smem, cudaStream_t s);

struct StateRow {
  double t, tn1, tn2, hnext, tprev, tprev2;
  long long k, nsteps;
  EngStats st;
  int npts, have_prev, next_sample, flags;  // flags: 1 started, 2 finished
};
constexpr int ROW_STARTED = 1, ROW_FINISHED = 2;

// derive params for instances [0, n_inst): raw blocks -> dpar blocks
cudaError_t launch_derive(const DTpl *tpls_dev, const int *inst_tpl, const long long *raw_off, const double *raw,
                          const long long *dpar_off, double *dpar, int n_inst, int max_dev, cudaStream_t s);

// cedar_eval: device outputs then CSC Jacobian values and residual rows
// (dout: n_out doubles; part: n_long_part doubles for the long-list partial sums)
cudaError_t launch_eval(const DTpl &T, const DTpl *T_dev, const double *dpar, const double *x, const double *xdot,
                        double t, double cj, double *dout, double *part, double *F, double *J, cudaStream_t s);

// Fixed-size device scratch for the allocation-free evaluation entry point:
// kEvalScratchMax doubles (2 MiB) per device, i.e. circuits with at most that many
// device outputs.  eval_scratch_address returns its device address for the
// current device (looked up once per device, then cached).
constexpr int kEvalScratchMax = 1 << 18;
constexpr int kMaxDevices = 64;
cudaError_t eval_scratch_address(double **ptr);

// single-instance block engine: mode 0 = transient, 1 = one Newton solve, 2 = DC op
struct PlainArgs {
  const DTpl *T; const double *dpar;
  double *x;               // original order, in/out
  const double *hist;      // original rows (mode 1) or null
  double t, cj;
  EngOpts opts;
  double *t_out, *x_out; long long cap; long long *count;
  EngStats *stats;
  double *ws_global;
  double *dense;           // (n + 2) n doubles for the dense DC fallback, or null
  int mode;
};
cudaError_t launch_plain(const PlainArgs &a, int ws_doubles_n, int threads, cudaStream_t s);
// the same single-circuit engine on a cooperative grid (large circuits): blocks for
// `work` parallel items, at most what can be resident; gred = 6 doubles per block
cudaError_t grid_geometry(int work, int *blocks);
cudaError_t launch_plain_grid(const PlainArgs &a, int blocks, double *gred, cudaStream_t s);

// AC / noise analysis (k_ac.cu): one warp per angular frequency over the
// template's LU and substitution task lists in complex FP64
struct AcDev {
  DTpl T;
  const double *gval, *cval;          // [nnz_lu] G and C per LU slot at the operating point
  const double *omega; long long n_freq;
  const double *b;                    // [n] drive -dFi/d(eps), original equation order (AC)
  const int *probe; int n_probe;      // original unknowns (noise: probe[0])
  double *resp;                       // [n_freq * n_probe] complex (re, im)
  int n_noise; const int *noise_a, *noise_b; const double *noise_w;  // noise currents: terminals, power
  const double *noise_e;              // [n_noise] frequency exponents, or null when every source is white
  double *psd;                        // [n_freq]
  double2 *ws; long long ws_stride;   // per warp: lu [nnz_lu], rd [n], v [n], rhs [n]
  long long n_warps;                  // workspaces in ws (warps that take frequencies)
  int *status;                        // [n_freq] CEDAR_ST_*, or kAcDense while a dense rerun is due
  int *n_dense;                       // frequencies handed to the dense rerun
  double2 *dws; long long dws_stride; // dense rerun, per warp: A [n * n], rhs [n]
  int *dpiv; long long n_dwarps;      // per warp: row interchanges [n]; warps of the dense rerun
  int lane_mode;                      // 1: one lane per frequency, ws interleaved by lane (ws_stride per lane)
};
constexpr int kAcDense = -1;          // status of a frequency waiting for the dense rerun
constexpr int kAcDenseNmax = 256;     // largest system the dense rerun takes
cudaError_t launch_ac_split(const DTpl &T, const double *dout, double *gval, double *cval, cudaStream_t s);
cudaError_t launch_ac(const AcDev &a, bool noise, cudaStream_t s);
cudaError_t launch_ac_dense(const AcDev &a, bool noise, cudaStream_t s);

// FP64 issue-rate probe (8 DFMA chains per thread, lanes >= active_lanes idle)
cudaError_t launch_fp64_probe(int active_lanes, int iters, double *gflops, double *ms);
cudaError_t launch_fp64_latency(int iters, double *cycles_per_op, double *ns_per_op);

// batched persistent engine with K lanes per instance
cudaError_t launch_batch(const BatchDev &b, int K, int warps_per_cta, int grid, size_t smem, cudaStream_t s);
// the same engine on one warp for one instance in record mode (k_batch.cu, 32 lanes):
// the single-circuit transient; smem > 0 puts the workspace in shared memory
cudaError_t launch_batch_record(const BatchDev &b, size_t smem, cudaStream_t s);
// (k_dispatch.cu) set the launch attributes of batch_kernel<K> for this shape and report its
// resident CTAs per SM (registers and shared memory both counted; at most max_per_sm when
// positive), with the shared-memory carve-out that holds exactly those CTAs
cudaError_t configure_batch(int K, int warps_per_cta, size_t smem, bool ws_in_smem, int max_per_sm, int *per_sm);
int batch_max_smem_optin();

}  // namespace cedar
