// k_adjoint.cu — discrete adjoint of the batched adaptive BDF2 transient.
//
// The forward run (batch_kernel with the tape on) records, per instance, every
// accepted step (time, order, supply power, probe value) and every ckpt_every
// steps a checkpoint (x_k, x_{k-1}).  This kernel then processes the instances
// from the device queue, one per slot of K lanes:
//
//   1. objective from the tape (supply energy by the trapezoidal rule, first
//      crossing of the probe through `level`, final probe value);
//   2. for each checkpoint segment, last to first: replay the recorded steps
//      from the checkpoint with the forward's own step preparation and Newton
//      iteration (bit-identical states), keeping the segment's states; then
//      sweep backwards through the segment:
//        J_k^T lam_k = -(dPhi/dx_k + C(x_k)^T (b1_{k+1} lam_{k+1} + b2_{k+2} lam_{k+2}))
//      with J_k = G + cj_k C evaluated and factorised at x_k (the DC Jacobian at
//      k = 0), solved by the transposed substitutions U^T then L^T;
//   3. dPhi/dp += lam_k^T dFi/dp at x_k for every MOSFET width and resistor value.
//
// Replay Newton solves of all slots of a warp run together (newton_iteration),
// and so do backward steps (backward_step), as in the transient kernel.  The
// recursion is the discrete adjoint of the step sequence the forward accepted,
// with each Newton solution taken as exact; the reference differentiates its
// transient with forward sensitivities (test/sensitivity.jl:13-42).
#include "batch_slot.cuh"

namespace cedar {

namespace {

enum AdjResume : int { AP_NEWINST = 100, AP_REPLAYED, AP_BACKED, AP_IDLE };

template <int K>
struct AdjSlot : Slot<K> {
  long long N, s0, s1, js, kb, k50;
  int cseg, np, astatus;
  double t50, tstar, gd0, gd1, phi;
  double *la, *lb, *lc;            // lambda_{k+1}, lambda_{k+2}, the step being solved (scratch)
  double *gacc;                    // gradient accumulators (workspace)
  double *seg;                     // replayed states of the current segment
  const double *tt, *tp, *tv;      // tape of this instance
  const signed char *tord;
  const double *raw;               // raw parameters of this instance
  AdjObj ob;
  // backward job
  bool bactive, bdc;
  const double *bx;
  double bt, bcj, cb1, cb2, ge, gp;
};

// BE / BDF2 coefficients of recorded step k: J_k = G + cj C and the factors of
// Fq(x_{k-1}) (b1) and Fq(x_{k-2}) (b2) in its residual.
__device__ __forceinline__ void step_coefs(const double *tt, const signed char *tord, long long k,
                                           double &cj, double &b1, double &b2) {
  const double h = tt[k] - tt[k - 1];
  if (tord[k] != 2) { cj = 1.0 / h; b1 = -cj; b2 = 0.0; return; }
  const double h1 = tt[k - 1] - tt[k - 2];
  const double wr = h / h1, rh = 1.0 / h;
  cj = (1.0 + 2.0 * wr) / ((1.0 + wr) * h);
  b1 = -(1.0 + wr) * rh;
  b2 = (wr * wr / (1.0 + wr)) * rh;
}

template <int K>
__device__ void adj_finish(AdjSlot<K> &s, const AdjDev &a) {
  const BatchDev &b = a.b;
  const bool ok = s.astatus == CEDAR_ST_OK;
  double *g = a.grad + (long long)s.inst * a.np_max;
  for (int p = s.rank(); p < a.np_max; p += K) g[p] = (ok && p < s.np) ? s.gacc[p] : (ok ? 0.0 : __longlong_as_double(0x7ff8000000000000LL));
  if (s.rank() == 0) {
    a.phi[s.inst] = ok ? s.phi : __longlong_as_double(0x7ff8000000000000LL);
    a.status[s.inst] = s.astatus;
  }
  (void)b;
  s.ssync();
  s.rp = AP_NEWINST;
}

// Advance the slot until it issues a replay Newton job or a backward job, or idles.
template <int K>
__device__ void adj_resume(AdjSlot<K> &s, const AdjDev &a, double *ws) {
  const BatchDev &b = a.b;
  const EngOpts &o = b.opts;
  const int every = b.ckpt_every;
  for (;;) {
    switch (s.rp) {
      case AP_IDLE:
        s.active = false; s.bactive = false;
        return;
      case AP_NEWINST: {
        const int job = s.dequeue(b);
        if (job < 0) { s.rp = AP_IDLE; s.active = false; s.bactive = false; return; }
        s.inst = job;
        const int ti = b.inst_tpl[s.inst];
        s.T = &b.tpls[ti];
        const DTpl &T = *s.T;
        s.dp = b.dpar + b.inst_dpar[s.inst];
        s.w.bind(ws, T.n, T.nnz_lu, T.n_out, T.n_src);
        s.gacc = ws + ws_doubles(T.n, T.nnz_lu, T.n_out, T.n_src);
        s.np = T.n_adj;
        s.raw = a.raw + a.raw_off[s.inst];
        s.ob = a.obj[ti];
        s.tstar = a.tstar ? a.tstar[s.inst] : 0.0;
        const long long ts = tape_stride(b.tape_cap);
        s.tt = b.tape_t + (long long)s.inst * ts; s.tord = b.tape_ord + (long long)s.inst * ts;
        s.tp = b.tape_p + (long long)s.inst * ts; s.tv = b.tape_v + (long long)s.inst * ts;
        s.seg = a.segx + (long long)s.inst * (every + 1) * b.n_max;
        s.tb_cache = -1e300;
        const EngStats fs = a.fwd[s.inst];
        s.astatus = fs.status;
        s.phi = 0.0;
        if (fs.status != CEDAR_ST_OK) { adj_finish(s, a); continue; }
        s.N = fs.accepted;
        // objective (rank 0, sequential: the oracle's summation order)
        double E = 0.0, t50 = 0.0, gd0 = 0.0, gd1 = 0.0, phi = 0.0;
        long long k50 = -1;
        if (s.rank() == 0) {
          for (long long k = 1; k <= s.N; ++k) E += (s.tt[k] - s.tt[k - 1]) * (s.tp[k] + s.tp[k - 1]) / 2.0;
          for (long long k = 1; k <= s.N; ++k) {
            const double v0 = s.tv[k - 1], v1 = s.tv[k];
            const double d0 = v0 - s.ob.level, d1 = v1 - s.ob.level;
            if ((d0 < 0 && d1 >= 0) || (d0 > 0 && d1 <= 0)) {
              k50 = k;
              t50 = s.tt[k - 1] + (s.ob.level - v0) * (s.tt[k] - s.tt[k - 1]) / (v1 - v0);
              break;
            }
          }
          const double D = k50 > 0 ? (t50 - s.tstar) * (t50 - s.tstar) : 0.0;
          phi = s.ob.w_energy * E + s.ob.w_delay * D + s.ob.w_final * s.tv[s.N];
          if (k50 > 0 && s.ob.w_delay != 0.0) {
            const double v0 = s.tv[k50 - 1], v1 = s.tv[k50];
            const double aa = s.ob.level - v0, dd = v1 - v0, Dh = s.tt[k50] - s.tt[k50 - 1];
            const double dD = s.ob.w_delay * 2.0 * (t50 - s.tstar);
            gd0 = dD * Dh * (aa - dd) / (dd * dd);
            gd1 = dD * (-Dh * aa) / (dd * dd);
          }
        }
        if (K > 1) {
          k50 = __shfl_sync(s.smask(), k50, 0, K); t50 = __shfl_sync(s.smask(), t50, 0, K);
          gd0 = __shfl_sync(s.smask(), gd0, 0, K); gd1 = __shfl_sync(s.smask(), gd1, 0, K);
          phi = __shfl_sync(s.smask(), phi, 0, K);
        }
        s.k50 = k50; s.t50 = t50; s.gd0 = gd0; s.gd1 = gd1; s.phi = phi;
        // lambda_{k+1}, lambda_{k+2} live in vectors the replay never touches; the
        // step being solved uses F, which is scratch between Newton solves
        s.la = s.w.xm2; s.lb = s.w.qd; s.lc = s.w.F;
        s.fill(s.la, 0.0); s.fill(s.lb, 0.0);
        for (int p = s.rank(); p < s.np; p += K) s.gacc[p] = 0.0;
        s.ssync();
        s.cseg = s.N >= 1 ? (int)((s.N - 1) / every) : 0;
        goto seg_begin;
      }
      case AP_REPLAYED: {
        if (s.jres <= 0) { s.astatus = s.jres == 0 ? CEDAR_ST_ZERO_PIVOT : CEDAR_ST_NEWTON; adj_finish(s, a); continue; }
        const DTpl &T = *s.T;
        s.eval_q(s.w.x, s.tt[s.js], s.w.qt);
        double *dst = s.seg + (s.js - s.s0) * b.n_max;
        for (int i = s.rank(); i < T.n; i += K) {
          s.w.qm1[i] = s.w.qn[i]; s.w.qn[i] = s.w.qt[i];
          s.w.xm1[i] = s.w.xn[i]; s.w.xn[i] = s.w.x[i]; dst[i] = s.w.x[i];
        }
        s.ssync();
        ++s.js;
        goto replay_issue;
      }
      case AP_BACKED: {
        if (s.astatus != CEDAR_ST_OK) { adj_finish(s, a); continue; }
        if (s.kb == 0) { adj_finish(s, a); continue; }
        for (int i = s.rank(); i < s.T->n; i += K) { s.lb[i] = s.la[i]; s.la[i] = s.lc[i]; }
        s.ssync();
        --s.kb;
        goto back_issue;
      }
      default:
        s.rp = AP_IDLE; s.active = false; s.bactive = false; return;
    }

  seg_begin: {
      const DTpl &T = *s.T;
      s.s0 = (long long)s.cseg * every;
      s.s1 = s.s0 + every < s.N ? s.s0 + every : s.N;
      const double *c = b.ckpt + ((long long)s.inst * ckpt_count(b.tape_cap, every) + s.cseg) * 2 * b.n_max;
      for (int i = s.rank(); i < T.n; i += K) { s.w.xn[i] = c[i]; s.w.xm1[i] = c[b.n_max + i]; s.seg[i] = c[i]; }
      s.ssync();
      s.eval_q(s.w.xn, s.tt[s.s0], s.w.qn);
      if (s.s0 >= 1) s.eval_q(s.w.xm1, s.tt[s.s0 - 1], s.w.qm1);
      s.js = s.s0 + 1;
    }
  replay_issue:
    if (s.js <= s.s1) {
      const long long k = s.js;
      const bool o2 = s.tord[k] == 2;
      s.prepare_step(o2, s.tt[k] - s.tt[k - 1], o2 ? s.tt[k - 1] - s.tt[k - 2] : 0.0);
      s.issue(s.w.x, s.w.hist, nullptr, s.tt[k], s.cj, 1.0, 0.0, 0.0, false, o.max_newton, AP_REPLAYED);
      return;
    }
    s.kb = s.s1;
  back_issue: {
      if (s.kb == s.s0 && s.s0 > 0) { --s.cseg; goto seg_begin; }
      const long long k = s.kb;
      s.bx = s.seg + (k - s.s0) * b.n_max;
      s.bdc = (k == 0);
      s.bt = k > 0 ? s.tt[k] : o.tstart;
      double cj = 0.0, b1 = 0.0, b2 = 0.0;
      if (k > 0) step_coefs(s.tt, s.tord, k, cj, b1, b2);
      s.bcj = cj;
      s.cb1 = 0.0; s.cb2 = 0.0;
      if (k + 1 <= s.N) { double c1, x1, x2; step_coefs(s.tt, s.tord, k + 1, c1, x1, x2); s.cb1 = x1; }
      if (k + 2 <= s.N) { double c1, x1, x2; step_coefs(s.tt, s.tord, k + 2, c1, x1, x2); s.cb2 = x2; }
      const double hk = k >= 1 ? s.tt[k] - s.tt[k - 1] : 0.0, hk1 = k + 1 <= s.N ? s.tt[k + 1] - s.tt[k] : 0.0;
      s.ge = s.ob.w_energy * (hk + hk1) / 2.0;
      s.gp = (k == s.N ? s.ob.w_final : 0.0);
      if (s.k50 > 0 && k == s.k50 - 1) s.gp += s.gd0;
      if (s.k50 > 0 && k == s.k50) s.gp += s.gd1;
      s.bactive = true; s.active = false;
      s.rp = AP_BACKED;
      return;
    }
  }
}

// One backward step for every slot of the warp holding a backward job (mask ab).
template <int K>
__device__ __forceinline__ void backward_step(AdjSlot<K> &s, const AdjDev &a, unsigned ab) {
  const DTpl &T = *s.T;
  const int rank = s.rank();
  const double *x = s.bx;
  // (1) C partials at x (charge devices with cj = 1) when later steps couple back
  const bool couple = (s.cb1 != 0.0 || s.cb2 != 0.0);
  const unsigned cm = __ballot_sync(ab, couple);
  if (couple) {
    EvalCtx ctx{s.bt, 1.0, 1.0, T.gmin, false, false};
    for_devices_by_model<K>(T, rank, cm, true, [&](const DGroup &gr, int i, int) {
      const int *tm = T.term + gr.term_off + i * gr.ntx;
      double v[CEDAR_MAX_TERM];
      for (int kk = 0; kk < gr.ntx; ++kk) { int u = tm[kk]; v[kk] = u < 0 ? 0.0 : x[u]; }
      eval_device(gr.model, s.dp + gr.dpar_off + i, gr.n_inst, v, nullptr, ctx, T.pwl, s.w.dout + gr.out_off + i, gr.n_inst);
    });
  }
  __syncwarp(ab);
  // right-hand side: -(dPhi/dx_k + C^T (cb1 lam_{k+1} + cb2 lam_{k+2}))
  for (int j = rank; j < T.n; j += K) {
    double acc = 0.0;
    if (couple) {
      for (int q = T.ct_ptr[j]; q < T.ct_ptr[j + 1]; ++q) {
        const int2 e = T.ct_ent[q];
        const double c = s.w.dout[e.x >> 1];
        const double v = s.cb1 * s.la[e.y] + s.cb2 * s.lb[e.y];
        acc = (e.x & 1) ? acc - c * v : acc + c * v;
      }
    }
    double g = 0.0;
    if (j == s.ob.iv) g += s.ge * (-x[s.ob.ib]);
    if (j == s.ob.ib) g += s.ge * (-x[s.ob.iv]);
    if (j == s.ob.ip) g += s.gp;
    s.lc[j] = -g - acc;
  }
  __syncwarp(ab);
  // (2) J_k = G + cj_k C at x_k (DC Jacobian at k = 0)
  {
    EvalCtx ctx{s.bt, s.bcj, 1.0, T.gmin, s.bdc, false};
    for_devices_by_model<K>(T, rank, ab, false, [&](const DGroup &gr, int i, int) {
      const int *tm = T.term + gr.term_off + i * gr.ntx;
      double v[CEDAR_MAX_TERM];
      for (int kk = 0; kk < gr.ntx; ++kk) { int u = tm[kk]; v[kk] = u < 0 ? 0.0 : x[u]; }
      eval_device(gr.model, s.dp + gr.dpar_off + i, gr.n_inst, v, nullptr, ctx, T.pwl, s.w.dout + gr.out_off + i, gr.n_inst);
    });
  }
  __syncwarp(ab);
  for (int q = rank; q < T.nnz_lu; q += K)
    if (T.jlu_ptr[q + 1] - T.jlu_ptr[q] <= kLongGather) s.w.lu[q] = s.gather(T.jlu_ptr, T.jlu_ent, q, 0.0);
  for (int t = 0; t < T.n_long_lu; ++t) {
    const int q = T.long_lu[t];
    const double v = long_gather<K>(T.jlu_ptr, T.jlu_ent, q, s.w.dout, rank, s.smask());
    if (rank == 0) s.w.lu[q] = v;
  }
  __syncwarp(ab);
  // (3) LU by levels
  bool bad = false;
  const int nl_lu = __reduce_max_sync(ab, T.lu_nlev);
  for (int l = 0; l < nl_lu; ++l) {
    if (l < T.lu_nlev) {
      int t1 = T.lu_lvl[l + 1];
      for (int t = T.lu_lvl[l] + rank; t < t1; t += K) {
        const int4 tk = T.lu_task[t];
        if (tk.w - tk.z > kLongPairs) continue;  // summed by the whole slot below
        int q = tk.x, info = tk.y;
        double acc = s.w.lu[q];
        for (int p = tk.z; p < tk.w; ++p) { int2 pr = T.lu_pair[p]; acc -= s.w.lu[pr.x] * s.w.lu[pr.y]; }
        int kind = info & 3, jj = info >> 2;
        if (kind == 2) acc *= s.w.rd[jj];
        else if (kind == 1) {
          if (!pivot_ok(acc)) bad = true;
          s.w.rd[jj] = pivot_rcp(acc);
        }
        s.w.lu[q] = acc;
      }
      for (int u = T.long_lu_lvl[l]; u < T.long_lu_lvl[l + 1]; ++u) {
        const int4 tk = T.lu_task[T.long_lu_task[u]];
        const double S = long_pair_sum<K>(T.lu_pair, tk.z, tk.w, s.w.lu, s.w.lu, rank, s.smask());
        if (rank == 0) {
          double acc = s.w.lu[tk.x] - S;
          const int kind = tk.y & 3, jj = tk.y >> 2;
          if (kind == 2) acc *= s.w.rd[jj];
          else if (kind == 1) {
            if (!pivot_ok(acc)) bad = true;
            s.w.rd[jj] = pivot_rcp(acc);
          }
          s.w.lu[tk.x] = acc;
        }
        s.ssync();
      }
    }
    __syncwarp(ab);
  }
  const bool slot_bad = (__ballot_sync(ab, bad) & s.smask()) != 0;
  // (4) U^T z = r, then L^T lam = z, in place in lc
  double *r = s.lc;
  const int nl_tf = __reduce_max_sync(ab, T.tf_nlev);
  for (int l = 0; l < nl_tf; ++l) {
    if (!slot_bad && l < T.tf_nlev) {
      for (int t = T.tf_lvl[l] + rank; t < T.tf_lvl[l + 1]; t += K) {
        const int4 tk = T.tf_task[t];
        if (tk.z - tk.y > kLongPairs) continue;  // summed by the whole slot below
        int i = tk.x; double acc = r[i];
        for (int p = tk.y; p < tk.z; ++p) { int2 pr = T.tf_pair[p]; acc -= s.w.lu[pr.x] * r[pr.y]; }
        r[i] = acc * s.w.rd[i];
      }
      for (int u = T.long_tf_lvl[l]; u < T.long_tf_lvl[l + 1]; ++u) {
        const int4 tk = T.tf_task[T.long_tf_task[u]];
        const double S = long_pair_sum<K>(T.tf_pair, tk.y, tk.z, s.w.lu, r, rank, s.smask());
        if (rank == 0) { const int i = tk.x; double acc = r[i] - S; r[i] = acc * s.w.rd[i]; }
        s.ssync();
      }
    }
    __syncwarp(ab);
  }
  const int nl_tb = __reduce_max_sync(ab, T.tb_nlev);
  for (int l = 0; l < nl_tb; ++l) {
    if (!slot_bad && l < T.tb_nlev) {
      for (int t = T.tb_lvl[l] + rank; t < T.tb_lvl[l + 1]; t += K) {
        const int4 tk = T.tb_task[t];
        if (tk.z - tk.y > kLongPairs) continue;  // summed by the whole slot below
        int i = tk.x; double acc = r[i];
        for (int p = tk.y; p < tk.z; ++p) { int2 pr = T.tb_pair[p]; acc -= s.w.lu[pr.x] * r[pr.y]; }
        r[i] = acc;
      }
      for (int u = T.long_tb_lvl[l]; u < T.long_tb_lvl[l + 1]; ++u) {
        const int4 tk = T.tb_task[T.long_tb_task[u]];
        const double S = long_pair_sum<K>(T.tb_pair, tk.y, tk.z, s.w.lu, r, rank, s.smask());
        if (rank == 0) { const int i = tk.x; double acc = r[i] - S; r[i] = acc; }
        s.ssync();
      }
    }
    __syncwarp(ab);
  }
  // (5) parameter partials: grad += lam^T dFi/dp (each lane owns its devices);
  // the KCL equation of terminal unknown u sits in internal row eq_pos[u]
  if (!slot_bad) {
    for (int gi = 0; gi < T.n_groups; ++gi) {
      const int goff = T.adj_goff[gi];
      if (goff < 0) continue;
      const DGroup gr = T.grp[gi];
      for (int i = rank; i < gr.n_inst; i += K) {
        const int *to = T.term_orig + gr.term_off + i * gr.ntx;
        const int *tm = T.term + gr.term_off + i * gr.ntx;
        const double o0 = s.w.dout[gr.out_off + i];   // output 0 of device i
        if (gr.model == CEDAR_MOS1) {
          // d(m Ids)/dW = m type id / W (id is linear in beta = KP W / L); KCL(d) -, KCL(s) +
          const double W = s.raw[gr.par_off + gr.n_inst + i];
          const double m = s.dp[gr.dpar_off + 4 * gr.n_inst + i];
          const double vd = tm[0] < 0 ? 0.0 : x[tm[0]], vs = tm[2] < 0 ? 0.0 : x[tm[2]];
          const double dI = (o0 - m * (T.gmin * (vd - vs))) / W;
          const double ld = to[0] < 0 ? 0.0 : r[T.eq_pos[to[0]]], ls = to[2] < 0 ? 0.0 : r[T.eq_pos[to[2]]];
          s.gacc[goff + i] += -dI * ld + dI * ls;
        } else {
          // d(m V / r)/dr = -out0 / r; KCL(p) -, KCL(n) +
          const double rr = s.raw[gr.par_off + i];
          const double dI = -o0 / rr;
          const double lp = to[0] < 0 ? 0.0 : r[T.eq_pos[to[0]]], ln = to[1] < 0 ? 0.0 : r[T.eq_pos[to[1]]];
          s.gacc[goff + i] += -dI * lp + dI * ln;
        }
      }
    }
  }
  __syncwarp(ab);
  if (slot_bad) s.astatus = CEDAR_ST_ZERO_PIVOT;
  s.bactive = false;
}

template <int K, bool SMEM>
__global__ void __launch_bounds__(256, 1) adjoint_kernel(AdjDev a) {
  extern __shared__ double smem[];
  const BatchDev &b = a.b;
  AdjSlot<K> s;
  const int slots_per_block = blockDim.x / K;
  const int slot = threadIdx.x / K;
  double *ws;
  if constexpr (SMEM) ws = smem + (size_t)slot * b.ws_stride;
  else ws = b.ws_global + ((size_t)blockIdx.x * slots_per_block + slot) * b.ws_stride;
  s.rp = AP_NEWINST; s.active = false; s.bactive = false;
  s.gsi = blockIdx.x * slots_per_block + slot; s.qblk = -1; s.dense = false; s.jdense = false;
  s.nrel = b.opts.nr_factor * b.opts.reltol; s.nav = b.opts.nr_factor * b.opts.abstol_v;
  s.nai = b.opts.nr_factor * b.opts.abstol_i;
  for (;;) {
    if (!s.active && !s.bactive && s.rp != AP_IDLE) adj_resume(s, a, ws);
    __syncwarp();
    const unsigned am = __ballot_sync(FULL, s.active);
    const unsigned ab = __ballot_sync(FULL, s.bactive);
    if ((am | ab) == 0) break;
    if (s.active) newton_iteration<K, false>(s, am);
    __syncwarp();
    if (s.bactive) backward_step(s, a, ab);
    __syncwarp();
  }
}

template <int K, bool SMEM>
cudaError_t launch_adj_ks(const AdjDev &a, int warps, int grid, size_t smem, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(adjoint_kernel<K, SMEM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int nb = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, adjoint_kernel<K, SMEM>, warps * 32, smem)) != cudaSuccess) return e;
  if (nb < 1) nb = 1;
  int dev = 0, smsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  int pct = (int)(100.0 * (double)nb * (double)(smem + 1024) / (double)(smsm > 0 ? smsm : 1)) + 1;
  pct = pct > 100 ? 100 : pct;
  if ((e = cudaFuncSetAttribute(adjoint_kernel<K, SMEM>, cudaFuncAttributePreferredSharedMemoryCarveout, pct)) != cudaSuccess) return e;
  adjoint_kernel<K, SMEM><<<grid, warps * 32, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace

#ifndef CEDAR_LANES
#error "compile with -DCEDAR_LANES=<lanes per instance>"
#endif
#define CEDAR_CAT2(a, b) a##b
#define CEDAR_CAT(a, b) CEDAR_CAT2(a, b)

// compiled once per lanes-per-instance value (-DCEDAR_LANES=K); k_dispatch.cu selects one
cudaError_t CEDAR_CAT(launch_adjoint_k, CEDAR_LANES)(const AdjDev &a, int warps, int grid, size_t smem, cudaStream_t st) {
  constexpr int K = CEDAR_LANES;
  return a.b.ws_in_smem ? launch_adj_ks<K, true>(a, warps, grid, smem, st) : launch_adj_ks<K, false>(a, warps, grid, smem, st);
}

}  // namespace cedar
