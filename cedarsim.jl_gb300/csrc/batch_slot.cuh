// batch_slot.cuh — the per-slot state machine and the warp-collective Newton
// iteration of the batched persistent engine (used by k_batch.cu for the
// transient and by k_adjoint.cu for the replay of recorded steps).
//
// Batched persistent engine: thousands of sweep / Monte Carlo instances of
// uneven sizes in one launch.
//
// A warp holds 32/K instance slots of K lanes each.  Every slot runs its own
// instance (own step size, Newton state, integrator history and DC homotopy, all
// in the slot's shared-memory workspace), but the expensive part — one Newton
// iteration: device evaluation, stamping, level-scheduled LU, substitutions and
// update — is executed by all active slots of the warp together, so the warp
// stays converged and a level of the LU schedule with one task per instance
// costs one FP64 instruction for the whole warp instead of one per instance.
// Everything else (step control, LTE, breakpoints, DC homotopy bookkeeping,
// output sampling) is a per-slot resumable state machine that mirrors the
// straight-line algorithm of engine.cuh (and of the CPU oracle) decision for
// decision.  A slot that retires an instance takes the next one from a
// device-side queue (one fetch-and-add; no slot ever waits on another warp).
#pragma once
#include <climits>
#include <type_traits>
#include "kernels.cuh"

namespace cedar {

namespace {

constexpr unsigned FULL = 0xffffffffu;

// Visit the devices of a template model by model, in a fixed model order, so
// that the lanes of a warp evaluate one model at a time whatever templates its
// slots run (the model switch in eval_device is then uniform across the warp).
// fn(gr, i, d): group, instance within the group, device index.  Collective over
// the lanes in `mask`; charges_only restricts the walk to capacitors and inductors.
template <int K, class Fn>
__device__ __forceinline__ void for_devices_by_model(const DTpl &T, int rank, unsigned mask, bool charges_only, Fn &&fn) {
  if constexpr (K == 32) {
    // one slot per warp: no other slot to diverge from, so walk the groups in
    // template order without the per-model bookkeeping
    for (int gi = 0; gi < T.n_groups; ++gi) {
      const DGroup gr = T.grp[gi];
      if (charges_only && !model_has_q(gr.model)) continue;
      const int dbase = gi > 0 ? T.dev_end[gi - 1] : 0;
      for (int i = rank; i < gr.n_inst; i += K) fn(gr, i, dbase + i);
    }
  } else {
  for (int m = 1; m < kNumModels; ++m) {
    if (charges_only && !model_has_q(m)) continue;
    const int g0 = T.mg_ptr[m], ng = T.mg_ptr[m + 1] - g0;
    const int ngmax = __reduce_max_sync(mask, ng);
    for (int q = 0; q < ngmax; ++q) {
      const int gi = q < ng ? T.mg_grp[g0 + q] : -1;
      DGroup gr{};
      if (gi >= 0) gr = T.grp[gi];
      const int cnt = gi >= 0 ? gr.n_inst : 0;
      const int rounds = __reduce_max_sync(mask, (cnt + K - 1) / K);
      const int dbase = gi > 0 ? T.dev_end[gi - 1] : 0;
      for (int r = 0; r < rounds; ++r) {
        const int i = rank + r * K;
        if (i < cnt) fn(gr, i, dbase + i);
      }
    }
  }
  }
}
constexpr int JOB_RUNNING = INT_MIN;  // job result while iterating
constexpr int JOB_ZERO_PIVOT = 0;     // result of a zero pivot

enum Resume : int {
  RP_NEWINST, RP_DC0, RP_PTC, RP_PTCFIN, RP_SRC, RP_FIX, RP_ADA, RP_IDLE
};

template <int K>
struct Slot {
  // ---- lane geometry (per lane, from the thread index: the Slot object itself
  // lives in shared memory, one copy per slot, written identically by its lanes)
  __device__ __forceinline__ int rank() const { return (int)(threadIdx.x & (K - 1)); }
  __device__ __forceinline__ unsigned smask() const {
    return K == 32 ? FULL : (((1u << K) - 1u) << ((threadIdx.x & 31) & ~(K - 1)));
  }
  // ---- instance
  int inst;
  const DTpl *T;
  const double *dp;
  WS w;
  // ---- Newton job in flight
  double *jx; const double *jhist; const double *jxref;
  double jt, jcj, jsrc, jgs, jvlim;
  int jit, jmaxit, jres;
  bool jdc, active;
  int rp;
  // ---- DC homotopy
  long long used; int pass, fails, halv; double gs, lam, dl, ln;
  // ---- transient
  EngStats st;
  long long k, N, nsteps;
  double t, tn1, tn2, h, h1, hnext, tnew, tprev, tprev2, cj;
  int npts; bool hit, have_prev, has_pert;
  int gsi, qblk;          // global slot index; queue block (template) last drawn from
  bool dense, jdense;     // DC homotopy rerun with dense partial pivoting; the job's mode
  Sink sk;
  double ts_next;         // time of sample sk.next
  double tb_cache;        // next source corner (see next_bp)
  double nrel, nav, nai;  // Newton tolerances

  // slot-level collectives (divergent phase: only this slot's lanes participate)
  __device__ __forceinline__ void ssync() const { if (K > 1) __syncwarp(smask()); }
  __device__ __forceinline__ bool sany(bool p) const { return K == 1 ? p : (__any_sync(smask(), p) != 0); }
  __device__ __forceinline__ double smax(double v) const {
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) { double u = __shfl_xor_sync(smask(), v, o, K); v = u > v ? u : v; }
    return v;
  }
  __device__ __forceinline__ double smin(double v) const {
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) { double u = __shfl_xor_sync(smask(), v, o, K); v = u < v ? u : v; }
    return v;
  }
  __device__ double sratio(MaxRatio m) const {
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) {
      double n2 = __shfl_xor_sync(smask(), m.num, o, K), d2 = __shfl_xor_sync(smask(), m.den, o, K);
      bool b2 = __shfl_xor_sync(smask(), (int)m.bad, o, K) != 0;
      m.merge(n2, d2, b2);
    }
    if (K > 1) {
      m.num = __shfl_sync(smask(), m.num, 0, K); m.den = __shfl_sync(smask(), m.den, 0, K);
      m.bad = __shfl_sync(smask(), (int)m.bad, 0, K) != 0;
    }
    return m.value();
  }
  __device__ __forceinline__ void copy(double *d, const double *s) { for (int i = rank(); i < T->n; i += K) d[i] = s[i]; }
  __device__ __forceinline__ void fill(double *d, double v) { for (int i = rank(); i < T->n; i += K) d[i] = v; }

  __device__ __forceinline__ double gather(const int *ptr, const int *ent, int s, double acc) const {
    int a = ptr[s], b = ptr[s + 1];
    for (int q = a; q < b; ++q) { int e = ent[q]; acc = acc + signed_out(w.dout[e >> 1], e); }
    return acc;
  }

  // charges at x into q (slot-level)
  __device__ void eval_q(const double *x, double tt, double *q) {
    const DTpl &TT = *T;
    EvalCtx ctx{tt, 0.0, 1.0, TT.gmin, false, false};
    for_devices_by_model<K>(TT, rank(), smask(), true, [&](const DGroup &gr, int i, int) {
      const int *tm = TT.term + gr.term_off + i * gr.ntx;
      double v[CEDAR_MAX_TERM];
      for (int kk = 0; kk < gr.ntx; ++kk) { int u = tm[kk]; v[kk] = u < 0 ? 0.0 : x[u]; }
      eval_device<false>(gr.model, dp + gr.dpar_off + i, gr.n_inst, v, nullptr, ctx, TT.pwl, w.dout + gr.out_off + i, gr.n_inst);
    });
    ssync();
    for (int r = rank(); r < TT.n; r += K) q[r] = gather(TT.qint_ptr, TT.qint_ent, r, 0.0);
    ssync();
  }

  // Next source corner after tt.  The value found at an earlier time t0 <= tt stays
  // the answer while tt + eps is below it (no corner lies in between), so it is
  // recomputed only after the step lands on it.
  __device__ double next_bp(double tt, double eps) {
    if (DADD(tt, eps) < tb_cache) return tb_cache;
    double best = 1e300;
    for (int s = rank(); s < T->n_src; s += K) {
      double b = source_next_bp(dp + T->src_off[s], T->src_stride[s], tt, eps, T->pwl);
      best = b < best ? b : best;
    }
    tb_cache = smin(best);
    return tb_cache;
  }

  __device__ void issue(double *x, const double *hist, const double *xref, double tt, double cjv, double src,
                        double gsh, double vlim, bool dc, int maxit, int next_rp) {
    jx = x; jhist = hist; jxref = xref; jt = tt; jcj = cjv; jsrc = src; jgs = gsh; jvlim = vlim; jdc = dc;
    jmaxit = maxit; jit = 0; jres = JOB_RUNNING; active = true; rp = next_rp; jdense = dense;
    // time-varying source values are fixed for the whole Newton solve
    for (int s = rank(); s < T->n_src; s += K)
      w.srcv[s] = source_value(dp + T->src_off[s], T->src_stride[s], tt, dc, T->pwl) * src;
    ssync();
  }

  // ---- output sink (samples only); ts_next caches the time of sample sk.next
  __device__ double sample_ts(int j) const {
    return j == sk.ns - 1 ? sk.tstop : sk.tstart + (sk.tstop - sk.tstart) * ((double)j / (double)(sk.ns - 1));
  }
  __device__ void sink_start(const double *x) {
    if (!sk.samp) return;
    for (int p = rank(); p < sk.np; p += K) { int u = sk.probes_int[p]; sk.samp[(long long)p * sk.ns] = u >= 0 ? x[u] : 0.0; }
    sk.next = 1;
    ts_next = sk.ns > 1 ? sample_ts(1) : 1e300;
  }
  __device__ void sink_step(bool have0, double t0, const double *x0, double t1, const double *x1, double t2, const double *x2) {
    if (!sk.samp) return;
    while (sk.next < sk.ns && ts_next <= t2) {
      double tt = ts_next;
      for (int p = rank(); p < sk.np; p += K) {
        int u = sk.probes_int[p]; double v;
        if (u < 0) v = 0.0;
        else if (have0) {
          double L0 = (tt - t1) * (tt - t2) / ((t0 - t1) * (t0 - t2));
          double L1 = (tt - t0) * (tt - t2) / ((t1 - t0) * (t1 - t2));
          double L2 = (tt - t0) * (tt - t1) / ((t2 - t0) * (t2 - t1));
          v = x0[u] * L0 + x1[u] * L1 + x2[u] * L2;
        } else {
          double a = (tt - t1) / (t2 - t1);
          v = x1[u] + (x2[u] - x1[u]) * a;
        }
        sk.samp[(long long)p * sk.ns + sk.next] = v;
      }
      ssync();   // the slot's fields may live in shared memory: every lane reads sk.next before it moves
      sk.next++;
      ts_next = sk.next < sk.ns ? sample_ts(sk.next) : 1e300;
    }
  }

  __device__ double restart_h(double tt, const EngOpts &o) {
    double nb = next_bp(tt, (o.tstop - o.tstart) * 1e-12); nb = nb < o.tstop ? nb : o.tstop;
    double dist = nb - tt; dist = dist < o.hmax ? dist : o.hmax;
    double hf = o.hfirst_frac * dist;
    if (o.h > 0) hf = o.h < hf ? o.h : hf;
    return hf;
  }

  __device__ __forceinline__ int absr(int r) const { return r < 0 ? -r : r; }

  // Next instance for this slot, or -1 when every block is drained.  The queue
  // holds one block per template (largest templates first); a slot keeps drawing
  // from the block it drew from last, so the slots of a warp tend to run the same
  // template and execute the same task lists in lockstep.  A slot's first draw
  // comes from the block holding queue position gsi.  At most n_qblk attempts.
  __device__ int dequeue(const BatchDev &b) {
    int inst_next = -1;
    if (rank() == 0) {
      if (qblk < 0) {
        const int p = gsi < b.n_inst ? gsi : b.n_inst - 1;
        int lo = 0, hi = b.n_qblk;
        while (hi - lo > 1) { int mid = (lo + hi) >> 1; if (b.qblk_beg[mid] <= p) lo = mid; else hi = mid; }
        qblk = lo;
      }
      for (int t = 0; t < b.n_qblk; ++t) {
        int j = qblk + t;
        if (j >= b.n_qblk) j -= b.n_qblk;
        const int cnt = b.qblk_beg[j + 1] - b.qblk_beg[j];
        if (*((volatile int *)&b.qblk_head[j]) >= cnt) continue;
        const int pos = atomicAdd(&b.qblk_head[j], 1);
        if (pos < cnt) { qblk = j; inst_next = b.queue[b.qblk_beg[j] + pos]; break; }
      }
    }
    if (K > 1) { inst_next = __shfl_sync(smask(), inst_next, 0, K); qblk = __shfl_sync(smask(), qblk, 0, K); }
    return inst_next;
  }

  // Variable-step BE (o2 false) or BDF2 step of length h after a step h1: sets cj,
  // the history w.hist (Fq space) and the predictor w.x from w.xn, w.xm1, w.qn,
  // w.qm1.  Shared by the transient and the adjoint's replay of recorded steps,
  // so that both compute the same bits.
  __device__ void prepare_step(bool o2, double h, double h1) {
    if (!o2) {
      cj = 1.0 / h;
      for (int i = rank(); i < T->n; i += K) w.hist[i] = -w.qn[i] * cj;
      copy(w.x, w.xn);
    } else {
      double wr = h / h1, rh = 1.0 / h;
      cj = (1.0 + 2.0 * wr) / ((1.0 + wr) * h);
      double a1 = -(1.0 + wr), a2 = wr * wr / (1.0 + wr);
      for (int i = rank(); i < T->n; i += K) w.hist[i] = (a1 * w.qn[i] + a2 * w.qm1[i]) * rh;
      double rr = h / h1;
      for (int i = rank(); i < T->n; i += K) w.x[i] = w.xn[i] + rr * (w.xn[i] - w.xm1[i]);
    }
    ssync();
  }

  // Record mode (single instance): accepted point (tt, x) into the record buffers.
  __device__ void rec_point(const BatchDev &b, double tt, const double *x) {
    const long long c = *((volatile long long *)b.rec_count);
    if (c < b.rec_cap) {
      if (rank() == 0) b.rec_t[c] = tt;
      double *row = b.rec_x + c * T->n;
      for (int i = rank(); i < T->n; i += K) row[T->order[i]] = x[i];
    }
    ssync();
    if (rank() == 0) *((volatile long long *)b.rec_count) = c + 1;
    ssync();
  }

  // Advance this slot's state machine until it issues a Newton job or goes idle.
  // REC: also record every accepted point (record mode, one instance).
  template <bool REC = false>
  __device__ void resume(const BatchDev &b, double *ws) {
    const EngOpts &o = b.opts;
    const long long budget = 20000;
    for (;;) {
      switch (rp) {
        case RP_IDLE:
          active = false;
          return;
        case RP_NEWINST: {
          const int job = dequeue(b);
          if (job < 0) { rp = RP_IDLE; active = false; return; }
          inst = job;
          const int flags = b.rows ? b.rows[inst].flags : 0;
          if (flags & ROW_FINISHED) continue;
          const int ti = b.inst_tpl[inst];
          T = &b.tpls[ti];
          dp = b.dpar + b.inst_dpar[inst];
          w.bind(ws, T->n, T->nnz_lu, T->n_out, T->n_src);
          tb_cache = -1e300;
          dense = false;
          if (rank() == 0) atomicAdd(b.n_running, 1);
          if (flags & ROW_STARTED) {
            // resume a run stopped at a window boundary
            sk = Sink{};
            sk.probes_int = b.probes_int ? b.probes_int + (size_t)ti * b.np : nullptr;
            sk.np = b.np; sk.ns = b.ns;
            sk.samp = (b.samples && b.np > 0 && b.ns > 0) ? b.samples + (size_t)inst * b.np * b.ns : nullptr;
            sk.tstart = o.tstart; sk.tstop = o.tstop;
            load_row(b);
            if (o.adaptive) goto ada_begin;
            goto fix_issue;
          }
          const long long xo = b.x0_off ? b.x0_off[inst] : -1;
          for (int i = rank(); i < T->n; i += K) w.x[i] = xo >= 0 ? b.x0[xo + T->order[i]] : 0.0;
          const long long dxo = b.dx_off ? b.dx_off[inst] : -1;
          has_pert = dxo >= 0;
          // the perturbation waits in qn (first written after the DC operating point)
          if (has_pert) for (int i = rank(); i < T->n; i += K) w.qn[i] = b.dx[dxo + T->order[i]];
          sk = Sink{};
          sk.probes_int = b.probes_int ? b.probes_int + (size_t)ti * b.np : nullptr;
          sk.np = b.np; sk.ns = b.ns;
          sk.samp = (b.samples && b.np > 0 && b.ns > 0) ? b.samples + (size_t)inst * b.np * b.ns : nullptr;
          sk.tstart = o.tstart; sk.tstop = o.tstop;
          st.accepted = st.rejected = st.newton_iters = st.dc_iters = 0;
          st.hmin_seen = 1e300; st.hmax_seen = 0; st.status = CEDAR_ST_OK; st.pad = 0;
          ssync();
          if (o.dcop) {
            copy(w.x0, w.x);
            ssync();
            used = 0;
            issue(w.x, nullptr, nullptr, o.tstart, 0.0, 1.0, 0.0, 0.0, true, 100, RP_DC0);
            return;
          }
          goto tran_init;
        }
        // ----------------------------------------------------------- DC homotopy
        case RP_DC0:
          used += absr(jres);
          if (jres > 0) goto dc_ok;
          pass = 0;
          goto ptc_begin;
        case RP_PTC:
          used += absr(jres);
          if (jres > 0) {
            copy(w.xm1, w.xs);
            ssync();
            if (gs <= 1e-14) {
              copy(w.x, w.xm1);
              ssync();
              issue(w.x, nullptr, nullptr, o.tstart, 0.0, 1.0, 0.0, pass == 0 ? 0.5 : 0.0, true, 100, RP_PTCFIN);
              return;
            }
            gs *= 0.1;
          } else { gs *= 4.0; ++fails; }
          goto ptc_issue;
        case RP_PTCFIN:
          used += absr(jres);
          if (jres > 0) goto dc_ok;
          goto ptc_end;
        case RP_SRC:
          used += absr(jres);
          if (jres > 0) { copy(w.x, w.xs); ssync(); lam = ln; halv = 0; dl = dl * 2 < 0.1 ? dl * 2 : 0.1; }
          else { dl *= 0.5; if (++halv > 8) goto dc_fail; }
          goto src_issue;
        // ----------------------------------------------------------- transient
        case RP_FIX: {
          st.newton_iters += absr(jres);
          if (jres <= 0) {
            st.status = jres == 0 ? CEDAR_ST_ZERO_PIVOT : CEDAR_ST_NEWTON;
            copy(w.x, w.xn); ssync();
            goto retire;
          }
          double *xp = w.x;
          eval_q(xp, t, w.qt);
          for (int i = rank(); i < T->n; i += K) {
            if (o.method == CEDAR_TRAP) w.qd[i] = cj * w.qt[i] + w.hist[i];
            w.qm1[i] = w.qn[i]; w.qn[i] = w.qt[i];
          }
          ssync();
          sink_step(have_prev, tprev2, w.xm1, tprev, w.xn, t, xp);
          ssync();
          bool nf = false;
          for (int i = rank(); i < T->n; i += K) { w.xm1[i] = w.xn[i]; w.xn[i] = xp[i]; if (!isfinite(xp[i])) nf = true; }
          nf = sany(nf);
          double hk = t - tprev;
          tprev2 = tprev; tprev = t; have_prev = true;
          st.accepted++; st.hmin_seen = hk < st.hmin_seen ? hk : st.hmin_seen; st.hmax_seen = hk > st.hmax_seen ? hk : st.hmax_seen;
          if constexpr (REC) rec_point(b, t, w.xn);
          if (nf) { st.status = CEDAR_ST_NAN; goto retire; }
          ++k;
          goto fix_issue;
        }
        case RP_ADA: {
          st.newton_iters += absr(jres);
          double *xp = w.x;
          const int n = T->n;
          if (jres <= 0) {
            st.rejected++;
            hnext = h * 0.125;
            if (hnext < o.hmin) { st.status = jres == 0 ? CEDAR_ST_ZERO_PIVOT : CEDAR_ST_DT_UNDERFLOW; goto ada_end; }
            goto ada_begin;
          }
          double err = 0.0;
          if (npts >= 3) {
            double h2 = tn1 - tn2;
            double rh = 1.0 / h, rh1 = 1.0 / h1, rh2 = 1.0 / h2;
            double ra = 1.0 / (h + h1), rb = 1.0 / (h1 + h2), rc = 1.0 / (h + h1 + h2);
            double coef = h * h * (h + h1) * (h + h1) / (2.0 * h + h1);
            MaxRatio mr;
            for (int i = rank(); i < n; i += K) {
              if (!T->is_node[i]) continue;
              double d10 = (xp[i] - w.xn[i]) * rh;
              double d21 = (w.xn[i] - w.xm1[i]) * rh1;
              double d32 = (w.xm1[i] - w.xm2[i]) * rh2;
              double dd3 = ((d10 - d21) * ra - (d21 - d32) * rb) * rc;
              double lte = fabs(dd3) * coef;
              double ax = fabs(xp[i]), bx = fabs(w.xn[i]);
              mr.add(lte, o.reltol * (ax > bx ? ax : bx) + o.abstol_v);
            }
            err = sratio(mr);
          } else if (npts == 2) {
            double rh = 1.0 / h, rh1 = 1.0 / h1, ra = 1.0 / (h + h1), hh = h * h;
            MaxRatio mr;
            for (int i = rank(); i < n; i += K) {
              if (!T->is_node[i]) continue;
              double dd2 = ((xp[i] - w.xn[i]) * rh - (w.xn[i] - w.xm1[i]) * rh1) * ra;
              double lte = fabs(dd2) * hh;
              double ax = fabs(xp[i]), bx = fabs(w.xn[i]);
              mr.add(lte, o.reltol * (ax > bx ? ax : bx) + o.abstol_v);
            }
            err = sratio(mr);
          }
          if (err > 1.0) {
            st.rejected++;
            hnext = h * step_factor(err);
            if (hnext < o.hmin) { st.status = CEDAR_ST_DT_UNDERFLOW; goto ada_end; }
            goto ada_begin;
          }
          eval_q(xp, tnew, w.qt);
          for (int i = rank(); i < n; i += K) { w.qm1[i] = w.qn[i]; w.qn[i] = w.qt[i]; }
          ssync();
          sink_step(npts >= 2, tn1, w.xm1, t, w.xn, tnew, xp);
          ssync();
          bool nf = false;
          for (int i = rank(); i < n; i += K) {
            w.xm2[i] = w.xm1[i]; w.xm1[i] = w.xn[i]; w.xn[i] = xp[i];
            if (!isfinite(xp[i])) nf = true;
          }
          nf = sany(nf);
          tn2 = tn1; tn1 = t; t = tnew;
          st.accepted++; st.hmin_seen = h < st.hmin_seen ? h : st.hmin_seen; st.hmax_seen = h > st.hmax_seen ? h : st.hmax_seen;
          if constexpr (REC) rec_point(b, t, w.xn);
          if (nf) { st.status = CEDAR_ST_NAN; goto ada_end; }
          if (b.tape_t && !tape_record(b, st.accepted, t, npts < 2 ? 1 : 2)) { st.status = CEDAR_ST_MAX_STEPS; goto ada_end; }
          if (npts < 3) ++npts;
          double fac = (err > 0.0) ? step_factor(err) : 1.0;
          hnext = h * fac;
          if (hit && t < o.tstop) { npts = 1; hnext = restart_h(t, o); }
          goto ada_begin;
        }
        default:
          rp = RP_IDLE; active = false; return;
      }

      // ------------------------------------------------------------- shared tails
    ptc_begin:
      copy(w.xm1, w.x0);
      ssync();
      gs = 1e-2; fails = 0;
    ptc_issue:
      if (used < budget && fails <= 60) {
        copy(w.xs, w.xm1);
        ssync();
        issue(w.xs, nullptr, w.xm1, o.tstart, 0.0, 1.0, gs, pass == 0 ? 0.5 : 0.0, true, 50, RP_PTC);
        return;
      }
    ptc_end:
      if (++pass < 2) goto ptc_begin;
      fill(w.x, 0.0);
      ssync();
      lam = 0.0; dl = 0.1; halv = 0;
    src_issue:
      if (!(lam < 1.0)) goto dc_ok;
      if (used >= budget) goto dc_fail;
      ln = lam + dl < 1.0 ? lam + dl : 1.0;
      copy(w.xs, w.x);
      ssync();
      issue(w.xs, nullptr, nullptr, o.tstart, 0.0, ln, 0.0, 0.0, true, 100, RP_SRC);
      return;
    dc_fail:
      st.dc_iters += used;
      if (!dense && b.dense_ws && T->n <= b.dense_nmax) {
        // The static pivot order can be numerically useless at a DC point (e.g. a
        // MOSFET output node whose only conductance is gmin next to a large gm):
        // rerun the whole homotopy from the initial guess with dense partial
        // pivoting, as the oracle factorises.
        dense = true;
        copy(w.x, w.x0);
        ssync();
        used = 0;
        issue(w.x, nullptr, nullptr, o.tstart, 0.0, 1.0, 0.0, 0.0, true, 100, RP_DC0);
        return;
      }
      st.status = CEDAR_ST_DCOP;
      goto retire_x;
    dc_ok:
      st.dc_iters += used;
      dense = false;  // the dense factorisation serves the DC homotopy only
      if (b.dc_only) goto retire_x;
    tran_init:
      if (has_pert) { for (int i = rank(); i < T->n; i += K) w.x[i] += w.qn[i]; ssync(); }
      eval_q(w.x, o.tstart, w.qn);
      copy(w.xn, w.x);
      ssync();
      sink_start(w.x);
      if constexpr (REC) rec_point(b, o.tstart, w.x);
      if (rank() == 0 && b.rows) b.rows[inst].flags = ROW_STARTED;
      if (!o.adaptive) {
        fill(w.qd, 0.0);
        ssync();
        tprev = tprev2 = o.tstart; have_prev = false;
        N = llround((o.tstop - o.tstart) / o.h);
        k = 1;
        goto fix_issue;
      }
      t = tn1 = tn2 = o.tstart; npts = 1; nsteps = 0;
      hnext = restart_h(t, o);
      if (b.tape_t) tape_record(b, 0, t, 0);
      goto ada_begin;
    fix_issue: {
      if (k > N) goto retire;
      if (tprev >= b.t_until) { save_row(b); rp = RP_NEWINST; continue; }
      t = (k == N) ? o.tstop : DADD(o.tstart, DMUL((double)k, o.h));
      double hk = t - tprev;
      if (o.method == CEDAR_TRAP) {
        cj = 2.0 / hk;
        for (int i = rank(); i < T->n; i += K) w.hist[i] = -cj * w.qn[i] - w.qd[i];
      } else if (k == 1) {
        cj = 1.0 / hk;
        for (int i = rank(); i < T->n; i += K) w.hist[i] = -w.qn[i] * cj;
      } else {
        cj = 1.5 / hk;
        const double r2h = 0.5 / hk;
        for (int i = rank(); i < T->n; i += K) w.hist[i] = (-4.0 * w.qn[i] + w.qm1[i]) * r2h;
      }
      if (k == 1) copy(w.x, w.xn);
      else for (int i = rank(); i < T->n; i += K) w.x[i] = 2.0 * w.xn[i] - w.xm1[i];
      ssync();
      issue(w.x, w.hist, nullptr, t, cj, 1.0, 0.0, 0.0, false, o.max_newton, RP_FIX);
      return;
    }
    ada_begin: {
      if (!(t < o.tstop)) goto ada_end;
      if (t >= b.t_until) { save_row(b); rp = RP_NEWINST; continue; }
      if (++nsteps > o.max_steps) { st.status = CEDAR_ST_MAX_STEPS; goto ada_end; }
      const double eps_bp = (o.tstop - o.tstart) * 1e-12;
      double tb = next_bp(t, eps_bp); tb = tb < o.tstop ? tb : o.tstop;
      h = hnext < o.hmax ? hnext : o.hmax;
      hit = false;
      if (tb - t <= 1.1 * h) { h = tb - t; hit = true; }
      tnew = hit ? tb : t + h;
      h = tnew - t;
      h1 = t - tn1;
      prepare_step(npts >= 2, h, h1);
      issue(w.x, w.hist, nullptr, tnew, cj, 1.0, 0.0, 0.0, false, o.max_newton, RP_ADA);
      return;
    }
    ada_end:
      copy(w.x, w.xn);
      ssync();
      if (st.status == CEDAR_ST_OK && t < o.tstop) st.status = CEDAR_ST_MAX_STEPS;
      goto retire_x;
    retire:
      copy(w.x, w.xn);
      ssync();
    retire_x:
      if (b.x_final)
        for (int i = rank(); i < T->n; i += K) b.x_final[(size_t)inst * b.n_max + T->order[i]] = w.x[i];
      if (rank() == 0 && b.stats) b.stats[inst] = st;
      if (rank() == 0 && b.rows) b.rows[inst].flags = ROW_STARTED | ROW_FINISHED;
      if (rank() == 0) atomicSub(b.n_running, 1);
      ssync();
      rp = RP_NEWINST;
    }
  }

  // ---- adjoint tape: entry k (time, order, supply power, probe) and, every
  // ckpt_every steps, the checkpoint (x_k, x_{k-1}); false when the tape is full
  __device__ bool tape_record(const BatchDev &b, long long k, double tk, int ord) {
    if (k > b.tape_cap) return false;
    ssync();
    const int4 oi = b.obj_idx[b.inst_tpl[inst]];
    if (rank() == 0) {
      const long long e = (long long)inst * tape_stride(b.tape_cap) + k;
      b.tape_t[e] = tk; b.tape_ord[e] = (signed char)ord;
      b.tape_p[e] = -(w.xn[oi.x] * w.xn[oi.y]);
      b.tape_v[e] = w.xn[oi.z];
    }
    if (k % b.ckpt_every == 0) {
      double *c = b.ckpt + ((long long)inst * ckpt_count(b.tape_cap, b.ckpt_every) + k / b.ckpt_every) * 2 * b.n_max;
      const double *prev = k == 0 ? w.xn : w.xm1;
      for (int i = rank(); i < T->n; i += K) { c[i] = w.xn[i]; c[b.n_max + i] = prev[i]; }
    }
    ssync();
    return true;
  }

  // ---- window boundaries: integrator state to / from the instance's state row
  __device__ void save_row(const BatchDev &b) {
    double *v = b.row_vec + (size_t)inst * 6 * b.n_max;
    const int n = T->n;
    for (int i = rank(); i < n; i += K) {
      v[i] = w.xn[i]; v[b.n_max + i] = w.xm1[i]; v[2 * b.n_max + i] = w.xm2[i];
      v[3 * b.n_max + i] = w.qn[i]; v[4 * b.n_max + i] = w.qm1[i]; v[5 * b.n_max + i] = w.qd[i];
    }
    if (rank() == 0) {
      StateRow &r = b.rows[inst];
      r.t = t; r.tn1 = tn1; r.tn2 = tn2; r.hnext = hnext; r.tprev = tprev; r.tprev2 = tprev2;
      r.k = k; r.nsteps = nsteps; r.st = st; r.npts = npts; r.have_prev = have_prev ? 1 : 0;
      r.next_sample = sk.next; r.flags = ROW_STARTED;
      if (b.stats) b.stats[inst] = st;
    }
    ssync();
  }
  __device__ void load_row(const BatchDev &b) {
    const double *v = b.row_vec + (size_t)inst * 6 * b.n_max;
    const int n = T->n;
    for (int i = rank(); i < n; i += K) {
      w.xn[i] = v[i]; w.xm1[i] = v[b.n_max + i]; w.xm2[i] = v[2 * b.n_max + i];
      w.qn[i] = v[3 * b.n_max + i]; w.qm1[i] = v[4 * b.n_max + i]; w.qd[i] = v[5 * b.n_max + i];
    }
    const StateRow &r = b.rows[inst];
    t = r.t; tn1 = r.tn1; tn2 = r.tn2; hnext = r.hnext; tprev = r.tprev; tprev2 = r.tprev2;
    k = r.k; nsteps = r.nsteps; st = r.st; npts = r.npts; have_prev = r.have_prev != 0;
    sk.next = r.next_sample;
    ts_next = (sk.samp && sk.next < sk.ns) ? sample_ts(sk.next) : 1e300;
    N = llround((b.opts.tstop - b.opts.tstart) / b.opts.h);
    ssync();
  }
};

}  // namespace

// One Newton iteration for every active slot of the warp (warp-collective over
// the active lanes `am`).  Loops that contain barriers run to the warp-wide
// maximum trip count so that every lane meets every barrier.
// Dense LU with partial pivoting (first maximum of a column wins; whole rows are
// swapped) and solve of J y = F for one slot, on the slot's lanes; J is scattered
// from the LU slots into a row-major n x n matrix in original order (scratch in
// global memory, b.dense_ws).  Every sum has a fixed order, independent of K.
// Returns false on a zero pivot.  y goes to s.w.F in internal order.
template <int K>
__device__ bool dense_factor_solve(Slot<K> &s, const BatchDev &b) {
  const DTpl &T = *s.T;
  const int n = T.n, ld = b.n_max, rank = s.rank();
  double *A = b.dense_ws + (size_t)s.gsi * b.dense_stride;
  double *rhs = A + (size_t)ld * ld;
  int *piv = reinterpret_cast<int *>(rhs + ld);
  for (int i = 0; i < n; ++i)
    for (int j = rank; j < n; j += K) A[(size_t)i * ld + j] = 0.0;
  s.ssync();
  for (int q = rank; q < T.nnz_lu; q += K) { const int2 rc = T.lu_orig[q]; A[(size_t)rc.x * ld + rc.y] = s.w.lu[q]; }
  for (int e = rank; e < n; e += K) rhs[e] = s.w.F[T.eq_pos[e]];
  s.ssync();
  for (int k = 0; k < n; ++k) {
    double best = -1.0; int p = k;
    for (int i = k + rank; i < n; i += K) { const double v = fabs(A[(size_t)i * ld + k]); if (v > best) { best = v; p = i; } }
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) {
      const double bv = __shfl_xor_sync(s.smask(), best, o, K);
      const int bp = __shfl_xor_sync(s.smask(), p, o, K);
      if (bv > best || (bv == best && bp < p)) { best = bv; p = bp; }
    }
    if (!(best > 0.0)) return false;
    if (rank == 0) piv[k] = p;
    if (p != k)
      for (int j = rank; j < n; j += K) {
        const double t = A[(size_t)k * ld + j]; A[(size_t)k * ld + j] = A[(size_t)p * ld + j]; A[(size_t)p * ld + j] = t;
      }
    s.ssync();
    const double inv = 1.0 / A[(size_t)k * ld + k];
    for (int i = k + 1 + rank; i < n; i += K) {
      double *Ai = A + (size_t)i * ld;
      const double aik = Ai[k];
      if (aik == 0.0) continue;
      const double l = aik * inv;
      Ai[k] = l;
      const double *Ak = A + (size_t)k * ld;
      for (int j = k + 1; j < n; ++j) Ai[j] -= l * Ak[j];
    }
    s.ssync();
  }
  if (rank == 0)
    for (int k = 0; k < n; ++k) if (piv[k] != k) { const double t = rhs[k]; rhs[k] = rhs[piv[k]]; rhs[piv[k]] = t; }
  s.ssync();
  for (int k = 0; k < n; ++k) {
    const double bk = rhs[k];
    for (int i = k + 1 + rank; i < n; i += K) { const double l = A[(size_t)i * ld + k]; if (l != 0.0) rhs[i] -= l * bk; }
    s.ssync();
  }
  for (int k = n - 1; k >= 0; --k) {
    if (rank == 0) rhs[k] = rhs[k] / A[(size_t)k * ld + k];
    s.ssync();
    const double bk = rhs[k];
    for (int i = rank; i < k; i += K) rhs[i] -= A[(size_t)i * ld + k] * bk;
    s.ssync();
  }
  for (int u = rank; u < n; u += K) s.w.F[T.iorder[u]] = rhs[u];
  s.ssync();
  return true;
}

template <int K, bool DENSE = false>
__device__ __forceinline__ void newton_iteration(Slot<K> &s, unsigned am, const BatchDev *bd = nullptr) {
  const DTpl &T = *s.T;
  const int rank = s.rank();
  const int it = s.jit + 1;
  // the slot's workspace pointers and job fields, read once
  double *const lu = s.w.lu, *const F = s.w.F, *const rd = s.w.rd, *const dout = s.w.dout;
  double *const jx = s.jx;
  const double *const jhist = s.jhist;
  const double *const dp = s.dp;
  const double *const srcv = s.w.srcv;
  const double jgs = s.jgs;
  // Fixed-order gathers with one accumulator: the lists are short (at most
  // kLongGather entries), and with 8 warps per SM sharing the FP64 pipe a second
  // accumulator's combining add costs more issue time than its shorter
  // dependency chain saves.  gather0 starts from the first entry instead of
  // 0.0 + it (the same value; a -0.0 entry stays -0.0).
  auto gather = [&](const int *ptr, const int *ent, int q, double acc) {
    const int e1 = ptr[q + 1];
    for (int k = ptr[q]; k < e1; ++k) { const int e0 = ent[k]; acc = acc + signed_out(dout[e0 >> 1], e0); }
    return acc;
  };
  auto gather0 = [&](const int *ptr, const int *ent, int q) {
    int k = ptr[q];
    const int e1 = ptr[q + 1];
    double acc = 0.0;
    if (k < e1) { const int e0 = ent[k]; acc = signed_out(dout[e0 >> 1], e0); ++k; }
    for (; k < e1; ++k) { const int e0 = ent[k]; acc = acc + signed_out(dout[e0 >> 1], e0); }
    return acc;
  };
  // K1: device evaluation, one model at a time across the warp
  {
    EvalCtx ctx{s.jt, s.jcj, s.jsrc, T.gmin, s.jdc, false};
    const double *x = jx;
    for_devices_by_model<K>(T, rank, am, false, [&](const DGroup &gr, int i, int d) {
      const int *tm = T.term + gr.term_off + i * gr.ntx;
      double v[CEDAR_MAX_TERM];
      for (int kk = 0; kk < gr.ntx; ++kk) { int u = tm[kk]; v[kk] = u < 0 ? 0.0 : x[u]; }
      double *out = dout + gr.out_off + i;
      const int si = (gr.model == CEDAR_V || gr.model == CEDAR_I) ? T.src_of_dev[d] : -1;
      if (si >= 0) eval_source_value(gr.model, dp + gr.dpar_off + i, v, srcv[si], out, gr.n_inst);
      else eval_device<false>(gr.model, dp + gr.dpar_off + i, gr.n_inst, v, nullptr, ctx, T.pwl, out, gr.n_inst);
    });
  }
  __syncwarp(am);
  // K2: stamping (fixed-order gathers)
  // lists longer than kLongGather (supply rails) are left to the slot-collective
  // sums below
  for (int q = rank; q < T.nnz_lu; q += K)
    if (T.jlu_ptr[q + 1] - T.jlu_ptr[q] <= kLongGather) lu[q] = gather0(T.jlu_ptr, T.jlu_ent, q);
  for (int r = rank; r < T.n; r += K)
    if (T.fint_ptr[r + 1] - T.fint_ptr[r] <= kLongGather) F[r] = gather(T.fint_ptr, T.fint_ent, r, jhist ? jhist[r] : 0.0);
  for (int t = 0; t < T.n_long_lu; ++t) {
    const int q = T.long_lu[t];
    const double v = long_gather<K>(T.jlu_ptr, T.jlu_ent, q, dout, rank, s.smask());
    if (rank == 0) lu[q] = v;
  }
  for (int t = 0; t < T.n_long_fi; ++t) {
    const int r = T.long_fi[t];
    const double v = long_gather<K>(T.fint_ptr, T.fint_ent, r, dout, rank, s.smask());
    if (rank == 0) F[r] = (jhist ? jhist[r] : 0.0) + v;
  }
  __syncwarp(am);
  if (jgs != 0.0) {
    for (int u = rank; u < T.n_nodes; u += K) {
      int c = T.gs_col[u];
      lu[T.gs_slot[u]] -= jgs;
      F[T.gs_row[u]] -= jgs * (jx[c] - (s.jxref ? s.jxref[c] : 0.0));
    }
  }
  __syncwarp(am);
  bool slot_bad = false;
  double *b = F;
  if constexpr (DENSE) {
    slot_bad = !dense_factor_solve(s, *bd);
    __syncwarp(am);
  } else {
  // K4: LU by levels
  bool bad = false;
  const int nl_lu = __reduce_max_sync(am, T.lu_nlev);
  for (int l = 0; l < nl_lu; ++l) {
    if (l < T.lu_nlev) {
      int t1 = T.lu_lvl[l + 1];
      for (int t = T.lu_lvl[l] + rank; t < t1; t += K) {
        const int4 tk = T.lu_task[t];
        if (tk.w - tk.z > kLongPairs) continue;  // summed by the whole slot below
        int q = tk.x, info = tk.y;
        double acc = lu[q];
        for (int p = tk.z; p < tk.w; ++p) { const int2 p0 = T.lu_pair[p]; acc -= lu[p0.x] * lu[p0.y]; }
        int kind = info & 3, j = info >> 2;
        if (kind == 2) acc *= rd[j];
        else if (kind == 1) {
          if (!pivot_ok(acc)) bad = true;
          rd[j] = pivot_rcp(acc);
        }
        lu[q] = acc;
      }
      for (int u = T.long_lu_lvl[l]; u < T.long_lu_lvl[l + 1]; ++u) {
        const int4 tk = T.lu_task[T.long_lu_task[u]];
        const double S = long_pair_sum<K>(T.lu_pair, tk.z, tk.w, lu, lu, rank, s.smask());
        if (rank == 0) {
          double acc = lu[tk.x] - S;
          const int kind = tk.y & 3, j = tk.y >> 2;
          if (kind == 2) acc *= rd[j];
          else if (kind == 1) {
            if (!pivot_ok(acc)) bad = true;
            rd[j] = pivot_rcp(acc);
          }
          lu[tk.x] = acc;
        }
        s.ssync();
      }
    }
    __syncwarp(am);
  }
  const unsigned bal_bad = __ballot_sync(am, bad);
  slot_bad = (bal_bad & s.smask()) != 0;
  // K5: substitutions (skipped by slots with a zero pivot; bounds stay uniform)
  const int nl_fw = __reduce_max_sync(am, T.fw_nlev);
  for (int l = 0; l < nl_fw; ++l) {
    if (!slot_bad && l < T.fw_nlev) {
      for (int t = T.fw_lvl[l] + rank; t < T.fw_lvl[l + 1]; t += K) {
        const int4 tk = T.fw_task[t];
        if (tk.z - tk.y > kLongPairs) continue;  // summed by the whole slot below
        int i = tk.x; double acc = b[i];
        for (int p = tk.y; p < tk.z; ++p) { const int2 p0 = T.fw_pair[p]; acc -= lu[p0.x] * b[p0.y]; }
        b[i] = acc;
      }
      for (int u = T.long_fw_lvl[l]; u < T.long_fw_lvl[l + 1]; ++u) {
        const int4 tk = T.fw_task[T.long_fw_task[u]];
        const double S = long_pair_sum<K>(T.fw_pair, tk.y, tk.z, lu, b, rank, s.smask());
        if (rank == 0) { const int i = tk.x; double acc = b[i] - S; b[i] = acc; }
        s.ssync();
      }
    }
    __syncwarp(am);
  }
  const int nl_bw = __reduce_max_sync(am, T.bw_nlev);
  for (int l = 0; l < nl_bw; ++l) {
    if (!slot_bad && l < T.bw_nlev) {
      for (int t = T.bw_lvl[l] + rank; t < T.bw_lvl[l + 1]; t += K) {
        const int4 tk = T.bw_task[t];
        if (tk.z - tk.y > kLongPairs) continue;  // summed by the whole slot below
        int i = tk.x; double acc = b[i];
        for (int p = tk.y; p < tk.z; ++p) { const int2 p0 = T.bw_pair[p]; acc -= lu[p0.x] * b[p0.y]; }
        b[i] = acc * rd[i];
      }
      for (int u = T.long_bw_lvl[l]; u < T.long_bw_lvl[l + 1]; ++u) {
        const int4 tk = T.bw_task[T.long_bw_task[u]];
        const double S = long_pair_sum<K>(T.bw_pair, tk.y, tk.z, lu, b, rank, s.smask());
        if (rank == 0) { const int i = tk.x; double acc = b[i] - S; b[i] = acc * rd[i]; }
        s.ssync();
      }
    }
    __syncwarp(am);
  }
  }  // sparse
  // K6: finiteness, DC damping, update, convergence vote
  // magnitudes are compared as integers (the bit patterns of non-negative doubles
  // order like the values), keeping these tests off the FP64 pipe
  bool nonfinite = false; long long mxb = 0;
  const bool damp = s.jvlim > 0;
  if (!slot_bad) {
    for (int i = rank; i < T.n; i += K) {
      long long ab = abs_bits(b[i]);
      if (ab >= 0x7ff0000000000000LL) nonfinite = true;  // inf or NaN
      if (damp && T.is_node[i]) mxb = ab > mxb ? ab : mxb;
    }
  }
  const bool slot_nf = (__ballot_sync(am, nonfinite) & s.smask()) != 0;
  double scale = 1.0;
  if (__any_sync(am, damp)) {
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) { long long u = __shfl_xor_sync(am, mxb, o, K); mxb = u > mxb ? u : mxb; }
    const double mx = __longlong_as_double(mxb);
    if (damp && mx > s.jvlim) scale = s.jvlim / mx;
  }
  bool conv = (scale == 1.0);
  if (!slot_bad && !slot_nf) {
    // undamped (every transient iteration): -b * 1 is -b, so the product is left out
    auto update = [&](auto scaled) {
      for (int i = rank; i < T.n; i += K) {
        const double d = decltype(scaled)::value ? -b[i] * scale : -b[i];
        double xi = jx[i] + d;
        jx[i] = xi;
        double lim = s.nrel * fabs(xi) + (T.is_node[i] ? s.nav : s.nai);
        if (abs_bits(d) > abs_bits(lim)) conv = false;
      }
    };
    if (conv) update(std::false_type{});
    else update(std::true_type{});
  }
  const bool slot_notconv = (__ballot_sync(am, !conv) & s.smask()) != 0;
  __syncwarp(am);
  s.jit = it;
  if (slot_bad) s.jres = JOB_ZERO_PIVOT;
  else if (slot_nf) s.jres = -it;
  else if (!slot_notconv) s.jres = it;
  else if (it >= s.jmaxit) s.jres = -s.jmaxit;
  if (s.jres != JOB_RUNNING) s.active = false;
}

}  // namespace cedar
