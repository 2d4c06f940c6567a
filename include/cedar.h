/*
 * cedar.h — C ABI of the GB300 (sm_103a) transient engine for CedarSim circuits.
 *
 * The library replaces, under a Julia `ccall` layer, the per-Newton-iteration work
 * that CedarSim's DAE residual does on the CPU today:
 *   - device evaluation into currents I, charges Q and their voltage partials,
 *   - stamping into fixed-pattern sparse G = dI/dx and C = dQ/dx,
 *   - assembly of J = G + cj*C and of the residual F = I + dQ/dt,
 *   - refactorisation and solution of J with a precomputed static-pivot ordering.
 *
 * Reference interfaces replaced (CedarSim 0.12.0):
 *   - residual `f(out, du, u, p, t)` / Jacobian `jac(J, du, u, p, gamma, t)` that
 *     DAECompiler emits and Sundials IDA / OrdinaryDiffEq consume
 *     (benchmarks/benchmark_common.jl:138,155; src/sweeps.jl:453)   -> cedar_eval
 *   - one implicit step of IDA's Newton (src/sweeps.jl:456)          -> cedar_newton_solve
 *   - `tran!(circ, tspan)` = DAEProblem + solve(prob, IDA())
 *     (src/sweeps.jl:450-463)                                        -> cedar_tran_run
 *   - `dc!(circ)` with CedarDCOp initialisation (src/sweeps.jl:437-448,
 *     src/dcop.jl:24-94)                                             -> cedar_dcop
 *   - `CircuitSweep` + broadcast `dc!.`/`tran!.` over parameter points
 *     (src/sweeps.jl:390-435,471-502)                                -> cedar_batch_*
 *   - forward sensitivities through SciMLSensitivity
 *     (test/sensitivity.jl:13-42)                                    -> cedar_adjoint_run
 *
 * Conventions
 *   - Unknowns: x[0 .. n_nodes-1] are node voltages (ground excluded, index -1),
 *     x[n_nodes .. n_nodes+n_branch-1] are branch currents of V sources, inductors
 *     and VCVS, exactly the MNA unknowns CedarSim's `branch!` keeps
 *     (src/simulate_ir.jl:112-120).
 *   - Residual rows follow CedarSim's KCL sign: a branch current I flowing from
 *     net+ to net- adds -m*I to KCL(net+) and +m*I to KCL(net-)
 *     (src/simulate_ir.jl:54,115-116); m is the SPICE multiplicity
 *     (ParallelInstances, src/simulate_ir.jl:56-75).
 *   - F(x, xdot, t) = Fi(x, t) + d/dt Fq(x).  G = dFi/dx, C = dFq/dx, J = G + cj*C.
 *   - All functions return 0 on success and a negative CEDAR_E* code on error;
 *     cedar_last_error() returns the message of the calling thread's last error.
 *   - Caller buffers are HOST memory unless a function name ends in `_dev`, in
 *     which case they are device pointers on the handle's stream.
 *   - Handles are not thread-safe; each handle owns one CUDA stream.
 */
#ifndef CEDAR_H
#define CEDAR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ---------------------------------------------------------- */
#define CEDAR_OK            0
#define CEDAR_EINVAL       -1   /* malformed description or argument          */
#define CEDAR_ECUDA        -2   /* CUDA runtime error                          */
#define CEDAR_ENOMEM       -3   /* allocation failure                          */
#define CEDAR_ESINGULAR    -4   /* structurally singular system                */
#define CEDAR_ENOCONV      -5   /* Newton / DC operating point did not converge*/
#define CEDAR_ECAPACITY    -6   /* output buffer too small                     */
#define CEDAR_EUNSUPPORTED -7   /* feature outside this build                  */

/* ---- per-instance status words (never trap; set and retire) --------------- */
#define CEDAR_ST_OK          0
#define CEDAR_ST_NEWTON      1  /* Newton failed at minimum step               */
#define CEDAR_ST_ZERO_PIVOT  2  /* |pivot| below threshold                      */
#define CEDAR_ST_DT_UNDERFLOW 3 /* step fell below hmin                         */
#define CEDAR_ST_MAX_STEPS   4  /* max_steps reached before tstop               */
#define CEDAR_ST_NAN         5  /* non-finite value in the solution             */
#define CEDAR_ST_DCOP        6  /* DC operating point failed                    */
#define CEDAR_ST_WAIT_LIMIT  7  /* a bounded device-side wait gave up           */
#define CEDAR_ST_NOT_RUN     8  /* instance never dequeued                      */

/* ---- device models --------------------------------------------------------
 * Parameter blocks are struct-of-arrays: par[p * n_inst + i].
 * Terminals are unknown indices, -1 = ground.  `m` is the multiplicity.
 *
 *  model            terms            params (in order)                reference
 *  R  resistor      p n              r m                              simpledevices.jl:49-77
 *  C  capacitor     p n              c m                              simpledevices.jl:99-109
 *  L  inductor      p n  (+branch)   l m                              simpledevices.jl:122-132
 *  V  vsource       p n  (+branch)   m dc kind a0..a6                 simpledevices.jl:274-300
 *  I  isource       p n              m dc kind a0..a6                 simpledevices.jl:315-339
 *  E  vcvs          p n cp cn (+br)  gain m                           simpledevices.jl:341-356
 *  G  vccs          p n cp cn        gain m                           simpledevices.jl:358-373
 *  MOS1 (VA level-1 Shichman-Hodges)
 *                   d g s b          type W L KP VTO LAMBDA m         (VA source in DESIGN)
 *  DIODE (VA exponential diode)
 *                   a c              IS N AREA m                      (VA source in DESIGN)
 *  NLVCR (VA nonlinear VCR, ddx test model)
 *                   d g s            R m                              test/NLVCR.va
 *
 * Source waveform kinds (params a0..a6), spectre_env.jl:43-69,144-176:
 *   CEDAR_WAVE_DC    : value = dc
 *   CEDAR_WAVE_PULSE : a0..a6 = v1 v2 td tr tf pw period
 *   CEDAR_WAVE_PWL   : a0 = offset (in doubles) into desc->pwl, a1 = number of points;
 *                      points are (t, v) pairs
 *   CEDAR_WAVE_SIN   : a0..a6 = vo va freq td theta phase ncycles
 * In DC analysis every source takes its `dc` parameter (simpledevices.jl:289-290).
 * ------------------------------------------------------------------------- */
enum {
  CEDAR_R = 1, CEDAR_C = 2, CEDAR_L = 3, CEDAR_V = 4, CEDAR_I = 5,
  CEDAR_E = 6, CEDAR_G = 7, CEDAR_MOS1 = 8, CEDAR_DIODE = 9, CEDAR_NLVCR = 10,
  CEDAR_NMODELS = 11
};
enum { CEDAR_WAVE_DC = 0, CEDAR_WAVE_PULSE = 1, CEDAR_WAVE_PWL = 2, CEDAR_WAVE_SIN = 3 };

typedef struct cedar_devgroup {
  int32_t model;          /* CEDAR_R ...                                        */
  int32_t n_inst;         /* number of instances in this group                  */
  const int32_t *term;    /* [n_inst * n_term] unknown index per terminal       */
  const int32_t *branch;  /* [n_inst] branch unknown (L, V, E), NULL otherwise  */
  const double *par;      /* [n_par * n_inst] struct-of-arrays parameters       */
} cedar_devgroup;

typedef struct cedar_ckt_desc {
  int32_t n_nodes;        /* node-voltage unknowns                              */
  int32_t n_branch;       /* branch-current unknowns                            */
  int32_t n_groups;
  const cedar_devgroup *groups;
  const double *pwl;      /* PWL point table referenced by CEDAR_WAVE_PWL       */
  int64_t n_pwl;          /* doubles in pwl                                     */
  double temp_c;          /* simulation temperature [C] (SimSpec.temp = 27)     */
  double gmin;            /* junction/channel gmin (SimSpec.gmin = 1e-12)       */
  int32_t ordering;       /* CEDAR_ORDER_AUTO (0), _MIN_DEGREE or _NESTED_DISSECTION */
  int32_t reserved;
} cedar_ckt_desc;

/* Objective of the discrete adjoint (per instance, over the accepted steps):
 *   Phi = w_energy * sum_n h_n (P_n + P_{n-1}) / 2          supply energy
 *       + w_delay  * (t50 - tstar)^2                         crossing-delay error
 *       + w_final  * x_N[probe]                              final value
 * with P = -x[vnode] * x[ibranch] (power delivered by the V source whose branch
 * current is ibranch) and t50 the first crossing of x[probe] through `level`
 * between consecutive accepted points (linear interpolation); no crossing gives
 * a zero delay term.  Indices are original unknowns. */
typedef struct cedar_objective {
  int32_t vnode, ibranch, probe, pad;
  double level, w_energy, w_delay, w_final;
} cedar_objective;

/* Fill-reducing ordering of the static-pivot LU.  AUTO computes both and keeps
 * the one whose level-scheduled factorisation + substitutions have the shorter
 * estimated critical path (ties: minimum degree). */
enum { CEDAR_ORDER_AUTO = 0, CEDAR_ORDER_MIN_DEGREE = 1, CEDAR_ORDER_NESTED_DISSECTION = 2 };

/* Terminal and parameter counts per model (index by model id). */
int cedar_model_nterm(int model);
int cedar_model_npar(int model);
int cedar_model_has_branch(int model);

/* Verilog-A device models compiled into this library (the role of
 * load_VA_model / make_spice_device, src/vasim.jl:663-875).  Model k (0-based,
 * sorted by module name) has model id CEDAR_NMODELS + k; its parameters are the
 * module's parameters in declaration order followed by the multiplicity m, and
 * its terminals are the module's ports in order.  cedar_va_name copies the
 * module name of model k into buf (CEDAR_EINVAL for k out of range). */
int cedar_va_count(void);
int cedar_va_name(int k, char *buf, size_t len);

/* ---- transient / DC options --------------------------------------------- */
enum { CEDAR_TRAP = 0, CEDAR_BDF2 = 1 };

typedef struct cedar_tran_opts {
  int32_t method;         /* CEDAR_TRAP or CEDAR_BDF2                           */
  int32_t adaptive;       /* 0: fixed step h; 1: LTE-controlled (BDF2 only)     */
  int32_t dcop;           /* 1: DC operating point at tstart before stepping    */
  int32_t max_newton;     /* Newton iterations per step (default 20)            */
  int64_t max_steps;      /* accepted + rejected step limit                     */
  double tstart, tstop;
  double h;               /* fixed step, or 0 for automatic initial step        */
  double hmin, hmax;      /* adaptive bounds (0 = automatic)                    */
  double reltol;          /* LTE relative tolerance (1e-6)                      */
  double abstol_v;        /* LTE absolute tolerance on node voltages (1e-9 V)   */
  double abstol_i;        /* absolute tolerance on branch currents (1e-12 A)    */
  double nr_factor;       /* Newton tolerance = nr_factor * LTE tolerance (1e-3)*/
  double hfirst_frac;     /* first step after a breakpoint, as a fraction of the
                             distance to the next breakpoint (1e-2)             */
} cedar_tran_opts;

/* Fill `o` with the defaults documented above (method BDF2, adaptive). */
void cedar_tran_opts_default(cedar_tran_opts *o);

typedef struct cedar_stats {
  int64_t accepted;       /* accepted steps                                     */
  int64_t rejected;       /* LTE + Newton rejections                            */
  int64_t newton_iters;   /* Newton iterations (each = eval + refactor + solve) */
  int64_t dc_iters;       /* Newton iterations spent in the DC operating point  */
  double hmin_seen, hmax_seen;
  int32_t status;         /* CEDAR_ST_*                                         */
  int32_t pad;
} cedar_stats;

/* ---- library ------------------------------------------------------------- */
int cedar_last_error(char *buf, size_t len);
int cedar_version(void);

/* ---- single circuit (plain drop-in) -------------------------------------- */
typedef struct cedar_ckt cedar_ckt;

/* Build the handle: computes the J pattern (CSC), stamp-slot maps, the static
 * pivot (structural matching) and fill-reducing ordering, the LU fill pattern and
 * its level schedule on the host, then copies everything to the device. */
int cedar_ckt_create(const cedar_ckt_desc *desc, cedar_ckt **out);
/* Host-only handle: runs the same analysis without touching the GPU.  Only
 * cedar_ckt_size / _pattern / _symbolic / _destroy accept it. */
int cedar_plan_create(const cedar_ckt_desc *desc, cedar_ckt **out);
int cedar_ckt_destroy(cedar_ckt *ckt);
int cedar_ckt_size(const cedar_ckt *ckt, int32_t *n, int32_t *nnz_j, int32_t *nnz_lu,
                   int32_t *n_levels);

/* Algorithmic work of one Newton iteration of this circuit (for roofline
 * accounting): FP64 operations by phase (an FMA counts 2, a reciprocal 1) and the
 * bytes an iteration must move when nothing stays on chip. */
typedef struct cedar_costs {
  int64_t flops_eval;    /* device evaluation                                   */
  int64_t flops_stamp;   /* J slot and residual-row sums                        */
  int64_t flops_lu;      /* numeric refactorisation                             */
  int64_t flops_solve;   /* forward + backward substitution                     */
  int64_t flops_update;  /* Newton update and convergence test                  */
  int64_t bytes;         /* params + terminals + outputs + J/LU + vectors       */
  int32_t lu_levels, fw_levels, bw_levels, nnz_lu;
  int32_t ordering;      /* CEDAR_ORDER_* actually used                         */
  int32_t pad;
  int64_t bytes_eval;    /* one cedar_eval_dev: derived params, terminal indices,
                            x gathers and outputs of every device, then stamp
                            entries, output reads, J and F written             */
} cedar_costs;
int cedar_ckt_costs(const cedar_ckt *ckt, cedar_costs *out);
/* The CUDA stream a handle's device work runs on (cedar_eval_dev and the
 * single-circuit entry points), for callers that order or time their own work
 * against it. */
int cedar_ckt_stream(const cedar_ckt *ckt, void **stream);

/* J pattern in compressed-sparse-column form over the ORIGINAL unknown order:
 * colptr[n+1], rowidx[nnz_j].  Jvals returned by cedar_eval follow this order. */
int cedar_ckt_pattern(const cedar_ckt *ckt, int32_t *colptr, int32_t *rowidx);
/* Static pivoting: rowmatch[u] = equation used as pivot row for unknown u;
 * order[p] = unknown eliminated at position p (fill-reducing ordering);
 * lu_colptr/lu_rowidx = pattern of L+U (incl. fill) in the permuted space. */
int cedar_ckt_symbolic(const cedar_ckt *ckt, int32_t *rowmatch, int32_t *order,
                       int32_t *lu_colptr, int32_t *lu_rowidx);

/* Residual + Jacobian: F = Fi(x,t) + C(x)*xdot (xdot may be NULL = 0),
 * Jvals = G + cj*C in the CSC order of cedar_ckt_pattern.  F or Jvals may be NULL.
 * Mirrors DAECompiler's f(out, du, u, p, t) and jac(J, du, u, p, gamma, t). */
int cedar_eval(cedar_ckt *ckt, const double *x, const double *xdot, double t, double cj,
               double *F, double *Jvals);
/* Same on device buffers (stream-ordered on the handle's stream). */
int cedar_eval_dev(cedar_ckt *ckt, const double *x, const double *xdot, double t, double cj,
                   double *F, double *Jvals);

/* Same as cedar_eval_dev, for callers that may not allocate device memory at the
 * point of the call: real-time solver loops that ban allocation after set-up,
 * and hosts whose device memory is reserved up front by another runtime's pool
 * allocator (a cudaMalloc there fails or stalls the host's own work).
 * It has no counterpart in the reference.  It calls no cudaMalloc or cudaFree:
 * its scratch (the per-device model outputs plus the partial sums of
 * supply-rail rows, at most 262144 doubles = 2 MiB; a larger circuit returns
 * CEDAR_EINVAL, see cedar_eval_scratch) is a fixed array that every GPU loading
 * the library holds until the process exits.  The handle's device (the one
 * current at cedar_ckt_create) must be current when calling, and a stream passed
 * in must belong to it; otherwise the call returns CEDAR_EINVAL.  The first call
 * on a device looks up that array's device address (cudaGetSymbolAddress with
 * the device current) and caches it, so make the first call on each device
 * before any stream capture.  All calls on a device share the array: calls whose
 * kernels overlap on the GPU race, so order them (same stream, or events).
 * stream: a cudaStream_t, or NULL for the handle's stream.  The handle itself is
 * created (and allocates) beforehand with cedar_ckt_create. */
int cedar_eval_dev_noalloc(cedar_ckt *ckt, const double *x, const double *xdot, double t, double cj,
                           double *F, double *Jvals, void *stream);
/* Scratch that cedar_eval_dev_noalloc needs for this circuit: n_out device
 * outputs plus n_part partial sums of supply-rail rows (any pointer may be NULL),
 * and the fixed limit on their sum.  ckt may be NULL when only the limit is
 * asked for.  No counterpart in the reference. */
int cedar_eval_scratch(const cedar_ckt *ckt, int64_t *n_out, int64_t *n_part, int64_t *limit);

/* One implicit step: solve Fi(x, t) + cj*Fq(x) + hist = 0 for x by Newton with
 * refactorisation every iteration.  hist (may be NULL) is the integrator history
 * in Fq space.  x holds the initial guess on entry and the solution on exit. */
int cedar_newton_solve(cedar_ckt *ckt, double t, double cj, const double *hist, double *x,
                       cedar_stats *stats);

/* DC operating point at time t (sources at their dc values, charges frozen),
 * Newton with source stepping then gmin stepping. x: guess in, solution out. */
int cedar_dcop(cedar_ckt *ckt, double t, double *x, cedar_stats *stats);

/* Whole transient on the device.  x0: initial state (or DC guess when
 * opts->dcop).  Every accepted time point is recorded into (t_out[cap],
 * x_out[cap * n]) while it fits; *n_out receives the number recorded (it is the
 * number of accepted points + 1 for the initial point; CEDAR_ECAPACITY if it
 * exceeded cap, in which case the first cap points are returned). */
int cedar_tran_run(cedar_ckt *ckt, const cedar_tran_opts *opts, const double *x0,
                   double *t_out, double *x_out, int64_t cap, int64_t *n_out,
                   cedar_stats *stats);
/* Engine of the single-circuit entry points.  The one-warp engine runs the
 * transient on the batched engine's instance state machine, one warp per
 * circuit, workspace in shared memory; the CTA engine runs one thread block
 * (threads: a multiple of 32, 0 = chosen from the circuit's size); the grid
 * engine runs the CTA engine's algorithm on every block of a cooperative grid
 * (grid-wide barriers and reductions; large circuits).  The CTA and grid engines
 * also serve cedar_newton_solve and cedar_dcop (the dense-pivoting DC rerun is
 * one-block only).  AUTO (the default): the grid engine for circuits of 4096
 * unknowns or more, else the CTA engine (the faster of the CTA and one-warp
 * engines on the circuits measured); the one-warp engine takes circuits whose
 * workspace fits its shared memory (else CEDAR_EINVAL).  No counterpart in the
 * reference: a tuning knob. */
enum { CEDAR_ENGINE_AUTO = 0, CEDAR_ENGINE_WARP = 1, CEDAR_ENGINE_CTA = 2, CEDAR_ENGINE_GRID = 3 };
int cedar_ckt_set_engine(cedar_ckt *ckt, int32_t engine, int32_t threads);
/* Thread blocks of the last single-circuit kernel (1 on the CTA engine). */
int cedar_ckt_last_blocks(const cedar_ckt *ckt, int32_t *blocks);
/* Device time (ms) of the kernel of the last cedar_tran_run / cedar_newton_solve /
 * cedar_dcop on this handle (CUDA events on the handle's stream around it).  No
 * counterpart in the reference: for throughput accounting. */
int cedar_ckt_last_ms(cedar_ckt *ckt, double *ms);

/* ---- batched form ---------------------------------------------------------
 * Instances share a topology template and differ in parameters (a CircuitSweep
 * over ParamSim points).  inst_par holds each instance's full parameter block:
 * the concatenation over the template's groups of its SoA parameter arrays
 * (same layout as the template's own `par` arrays).  probes lists unknowns whose
 * waveform is sampled on a uniform grid of n_samples points over [tstart, tstop]. */
typedef struct cedar_batch_desc {
  int32_t n_templates;
  const cedar_ckt_desc *templates;
  int32_t n_inst;
  const int32_t *inst_template;   /* [n_inst]                                 */
  const int64_t *inst_par_off;    /* [n_inst] offset into inst_par, -1 = nominal */
  const double *inst_par;
  const int64_t *inst_x0_off;     /* [n_inst] offset into inst_x0 or -1 (zeros)  */
  const double *inst_x0;          /* initial state / DC guess per instance      */
  const int64_t *inst_dx_off;     /* [n_inst] offset into inst_dx or -1          */
  const double *inst_dx;          /* perturbation added after the DC op         */
  int32_t n_probes;               /* probes per template (same count each)      */
  const int32_t *probes;          /* [n_templates * n_probes] unknown indices   */
  int32_t n_samples;              /* output samples per probe (>= 2), or 0      */
} cedar_batch_desc;

typedef struct cedar_batch cedar_batch;

/* Lanes per instance and instances per CTA chosen by the autotuner (0 = auto),
 * and an upper bound on resident CTAs per SM (0 = as many as registers and
 * shared memory allow): fewer CTAs leave more of the SM's unified L1 / shared
 * storage as L1, which caches the templates' task lists. */
typedef struct cedar_batch_tuning {
  int32_t lanes_per_inst;         /* 1, 2, 4, 8, 16 or 32                       */
  int32_t warps_per_cta;
  int32_t ctas_per_sm;            /* 0 = no bound                               */
  int32_t reserved[5];
} cedar_batch_tuning;

int cedar_batch_create(const cedar_batch_desc *desc, cedar_batch **out);
int cedar_batch_destroy(cedar_batch *b);
/* Run every instance from tstart to tstop in one persistent launch.
 *   x_final[n_inst * n_max]  final state per instance (may be NULL)
 *   samples[n_inst * n_probes * n_samples] probe waveforms (may be NULL)
 *   stats[n_inst]            per-instance counters and status (may be NULL) */
int cedar_batch_run(cedar_batch *b, const cedar_tran_opts *opts, double *x_final,
                    double *samples, cedar_stats *stats);
/* Windowed form of cedar_batch_run: start a run (DC operating points happen in
 * the first advance), advance every unfinished instance to its first step that
 * starts at or after t_until (a soft stop that leaves the step sequence of an
 * uninterrupted run unchanged; integrator state stays on the device), then read
 * the results.  n_running receives the number of instances still unfinished. */
int cedar_batch_start(cedar_batch *b, const cedar_tran_opts *opts);
int cedar_batch_advance(cedar_batch *b, double t_until, int32_t *n_running);
int cedar_batch_results(cedar_batch *b, double *x_final, double *samples, cedar_stats *stats);
/* DC operating point of every instance (broadcast dc!. over a CircuitSweep,
 * src/sweeps.jl:471-486): the batch's homotopy (Newton, pseudo-transient
 * continuation, source stepping, dense-pivoting rerun) with opts' tolerances;
 * inst_dx perturbations are not applied.  x_dc[n_inst * n_max] in original
 * order; stats[n_inst].dc_iters and .status report each solve. */
int cedar_batch_dcop(cedar_batch *b, const cedar_tran_opts *opts, double *x_dc, cedar_stats *stats);

/* ---- small-signal AC and noise about an operating point -------------------
 * Replaces ACSol / freqresp and NoiseSol / PSD (src/ac.jl:73-104,251-258 and
 * src/ac.jl:107-171,263-283), whose descriptor system is (jω M − Ju)⁻¹ B about
 * the DC operating point.  Here G = dFi/dx and C = dFq/dx are evaluated at x_op
 * (n doubles, original unknown order, e.g. from cedar_dcop), and every angular
 * frequency omega[f] (rad/s) is one factorisation of G + j omega C on the GPU
 * with the circuit's static pivot order; frequencies run in parallel.
 * status[f] (may be NULL): CEDAR_ST_OK, or CEDAR_ST_ZERO_PIVOT when a pivot of
 * G + j omega C is zero or not finite (that frequency's outputs are NaN). */

/* AC response: X_f solves (G + j omega_f C) X_f = b.  b (n doubles, original
 * equation order) is -dFi/d(eps) of the AC drive eps: a voltage source with AC
 * magnitude a adds +a to its branch equation, a current source of multiplicity m
 * adds +m a to the KCL row of its first terminal and -m a to the second
 * (src/simpledevices.jl:292-294,331-333).  resp receives n_freq * n_probe
 * complex values X_f[probe[k]], interleaved (re, im), frequency-major. */
int cedar_ac(cedar_ckt *ckt, const double *x_op, const double *b, int32_t n_freq, const double *omega,
             int32_t n_probe, const int32_t *probe, double *resp, int32_t *status);

/* Output noise PSD (V^2/Hz for a node voltage) at unknown `probe`:
 * psd[f] = sum over resistors of m^2 (4 k T / r) |H_r(j omega_f)|^2, with H_r the
 * transfer from the resistor's white thermal noise current (src/simpledevices.jl:
 * 70-75; multiplicity m scales that current with the branch current,
 * src/simulate_ir.jl:54) to the probe, and T = the circuit's temp_c + 273.15.
 * Verilog-A devices add one source per white_noise(pwr) or flicker_noise(pwr, ex)
 * term of a current contribution (src/va_env.jl:82-90): density m^2 pwr
 * (white) or m^2 pwr / f^ex with f = omega / 2 pi (flicker, src/ac.jl:267-276)
 * across that contribution's branch, pwr and ex evaluated at x_op.  One
 * transposed solve (G + j omega C)^T y = e_probe per frequency gives every H_r
 * at once. */
int cedar_noise(cedar_ckt *ckt, const double *x_op, int32_t n_freq, const double *omega, int32_t probe,
                double *psd, int32_t *status);
/* Of the last cedar_ac / cedar_noise call on this handle: how many frequencies
 * the dense partial-pivoting rerun took (their sparse solve met a zero pivot or
 * failed the residual check), and the device time (ms, CUDA events) of the
 * sparse kernel and of the dense rerun (0 when it did not run).  Measurement
 * helper; no counterpart in the reference. */
int cedar_ac_last_stats(const cedar_ckt *ckt, int32_t *n_dense, double *ms_sparse, double *ms_dense);
/* Device time of the last batch launch (CUDA events on the handle's stream). */
int cedar_batch_last_ms(cedar_batch *b, double *ms);
int cedar_batch_set_tuning(cedar_batch *b, const cedar_batch_tuning *t);
int cedar_batch_get_tuning(const cedar_batch *b, cedar_batch_tuning *t);
/* Autotune: time each candidate tile shape on a short horizon and keep the best. */
int cedar_batch_autotune(cedar_batch *b, const cedar_tran_opts *opts, double horizon,
                         cedar_batch_tuning *best);
int cedar_batch_nmax(const cedar_batch *b, int32_t *n_max);

/* ---- discrete adjoint ------------------------------------------------------
 * Replaces the reference's parameter sensitivities of a transient
 * (ODEForwardSensitivityProblem + extract_local_sensitivities,
 * test/sensitivity.jl:13-42) with the gradient of a scalar objective
 * (cedar_objective) by the discrete adjoint, for every instance of a batch.
 *
 * cedar_adjoint_run runs the batch forward (adaptive BDF2 only, no inst_dx)
 * recording each instance's accepted steps on a device tape (tape_cap steps per
 * instance, <= 0: 2^19; an instance needing more ends with CEDAR_ST_MAX_STEPS)
 * with a state checkpoint every 64 steps, then sweeps backwards: each 64-step
 * segment is recomputed from its checkpoint, and J_k^T lam_k = -(dPhi/dx_k +
 * C^T (b1 lam_{k+1} + b2 lam_{k+2})) is solved with J_k factorised at the
 * step's solution (transposed substitutions), down to the DC operating point.
 * The gradient lam^T dFi/dp covers every MOS1 width W and resistor value r, per
 * template in group order (cedar_adjoint_nparams gives the counts).
 *   obj[n_templates]       objective per template (original unknown indices)
 *   tstar[n_inst]          target crossing time per instance (NULL: 0)
 *   phi[n_inst]            objective value
 *   grad[n_inst * np_max]  gradient (entries past the template's count are 0)
 *   status[n_inst]         CEDAR_ST_* of the instance (forward or backward)
 *   stats[n_inst]          forward counters
 * Every output may be NULL.  Results of failed instances are NaN. */
int cedar_adjoint_run(cedar_batch *b, const cedar_tran_opts *opts, const cedar_objective *obj,
                      const double *tstar, int64_t tape_cap, double *phi, double *grad,
                      int32_t *status, cedar_stats *stats);
int cedar_adjoint_nparams(const cedar_batch *b, int32_t *np_per_template, int32_t *np_max);
/* The step sequence the last adjoint run recorded for one instance: times and
 * orders (1 = BE, 2 = BDF2) of its accepted steps (at most cap of them), for
 * finite-difference checks that replay the same steps. */
int cedar_adjoint_tape(cedar_batch *b, int32_t inst, double *t, int8_t *ord, int64_t cap, int64_t *n_steps);
/* Device time of the last adjoint run's forward and backward kernels. */
int cedar_adjoint_last_ms(cedar_batch *b, double *fwd_ms, double *bwd_ms);

/* ---- measurement ------------------------------------------------------------
 * FP64 issue-rate probe, the denominator of the batched kernel's roofline (no
 * counterpart in the reference): every lane below active_lanes of 8 x 256-thread
 * CTAs per SM runs 8 independent DFMA chains of iters steps; gflops counts 2 flops
 * per FMA on the active lanes, best of 5 timed launches (CUDA events). */
int cedar_fp64_probe(int32_t active_lanes, int32_t iters, double *gflops, double *ms);

/* FP64 dependent-operation latency (no counterpart in the reference): one warp
 * whose lanes each run a chain of 8 * iters dependent DFMAs; cycles_per_op from
 * the SM clock, ns_per_op from CUDA events (launch included), best of 3.  It
 * bounds a single circuit's Newton iteration, whose LU and substitutions are
 * chains of dependent FP64 operations. */
int cedar_fp64_latency(int32_t iters, double *cycles_per_op, double *ns_per_op);

#ifdef __cplusplus
}
#endif
#endif /* CEDAR_H */
