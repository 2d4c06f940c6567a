// engine.cuh — per-instance transient engine, run by a cooperating thread group.
//
// One group (a tile of K lanes of a warp, or a whole CTA) owns one circuit
// instance: its Newton iterate, integrator history, LU values and device
// outputs live in the group's workspace (shared memory when it fits).  Each
// Newton iteration is
//   K1  device evaluation        (threads over devices)
//   K2  stamping J and F          (threads over LU slots / rows, fixed-order sums)
//   K4  LU refactorisation        (level by level, threads over entry tasks)
//   K5  forward/back substitution (level by level, threads over rows)
//   K6  update + convergence test (threads over unknowns, group vote)
// with one group barrier per phase / level.  All control decisions are taken
// redundantly by every thread from group-reduced values, so the group never
// diverges; no atomics are used, so results are bitwise reproducible.
#pragma once
#include <cstdint>
#include "models.cuh"

namespace cedar {

struct DGroup { int model, n_inst, ntx, term_off, par_off, dpar_off, out_off; };

// Device view of a compiled template (all pointers to device memory).
struct DTpl {
  int n, n_nodes, nnz_lu, n_out, n_groups, n_dev, n_src, lu_nlev, fw_nlev, bw_nlev, n_csc, dpar_size;
  double gmin, vt;
  const DGroup *grp;
  const int *dev_end;      // [n_groups] cumulative device count
  const int *term;         // internal unknown per terminal (-1 ground)
  const int *term_orig;    // original unknown per terminal
  const int *jlu_ptr, *jlu_ent, *fint_ptr, *fint_ent, *qint_ptr, *qint_ent;
  const int *jcsc_ptr, *jcsc_ent, *forg_ptr, *forg_ent;
  const int *lu_lvl, *lu_slot, *lu_info, *lu_pp; const int2 *lu_pair;
  const int *fw_lvl, *fw_row, *fw_ptr; const int2 *fw_pair;
  const int *bw_lvl, *bw_row, *bw_ptr; const int2 *bw_pair;
  const int *src_off, *src_stride;    // derived-param offset / stride per source
  const int *src_of_dev;              // [n_dev] time-varying source index, or -1
  const int *gs_slot;                 // [n_nodes] LU slot of (KCL(u),u)
  const int *gs_row;                  // [n_nodes] internal row of KCL(u)
  const int *gs_col;                  // [n_nodes] internal column of u
  const unsigned char *is_node;       // [n] internal
  const int *order;                   // internal position -> original unknown
  const int *iorder;                  // original unknown -> internal position
  const int *eq_pos;                  // original equation -> internal row
  const double *pwl;
  // discrete adjoint: transposed substitutions (U^T then L^T, row-task layout as
  // fw/bw), C^T program per internal column ((out << 1) | neg, internal row) and
  // the first gradient index of each group (-1: no differentiable parameter)
  int tf_nlev, tb_nlev, n_adj, pad_adj;
  // groups by model: mg_grp[mg_ptr[m] .. mg_ptr[m + 1]) are the groups of model m
  int mg_ptr[kNumModels + 1];
  const int *mg_grp;
  // original (equation, unknown) of every LU slot, for the dense DC fallback
  const int2 *lu_orig;
  // the same task lists packed one 16-byte record per task: LU (slot, info,
  // first pair, end pair); substitutions (row, first pair, end pair, 0)
  const int4 *lu_task, *fw_task, *bw_task, *tf_task, *tb_task;
  // long gather lists (see kLongGather / kLongEval): LU slots, residual rows
  // (internal), CSC slots and residual rows (original order)
  int n_long_lu, n_long_fi, n_long_jc, n_long_fo;
  const int *long_lu, *long_fi, *long_jc, *long_fo;
  // cedar_eval: chunk offsets of the long CSC slots then the long residual rows
  // (n_long_jc + n_long_fo + 1 entries); n_long_part chunks in all
  const int *long_off; int n_long_part, pad_long;
  // LU / substitution tasks with more than kLongPairs pairs, per level: task
  // indices long_*_task[long_*_lvl[l] .. long_*_lvl[l + 1]) (summed cooperatively)
  const int *long_lu_lvl, *long_lu_task, *long_fw_lvl, *long_fw_task, *long_bw_lvl, *long_bw_task;
  const int *long_tf_lvl, *long_tf_task, *long_tb_lvl, *long_tb_task;
  const int *tf_lvl, *tf_row, *tf_ptr; const int2 *tf_pair;
  const int *tb_lvl, *tb_row, *tb_ptr; const int2 *tb_pair;
  const int *ct_ptr; const int2 *ct_ent;
  const int *adj_goff;
  // per device output: 1 if it holds cj * dQ/dV (splits J into G and C for AC)
  const unsigned char *out_q;
  // LU pattern by internal row (CSR: slots lu_rowptr[p] .. lu_rowptr[p + 1], column
  // lu_colidx[slot]) and by internal column (slots lu_cslot[lu_cptr[q] ..
  // lu_cptr[q + 1]), row lu_srow[slot]), for residuals of the assembled matrix
  const int *lu_rowptr, *lu_colidx, *lu_cptr, *lu_cslot, *lu_srow;
};

// A stamp entry's signed device output: (e & 1) flips the sign bit, so a gather
// adds acc + signed(v, e) -- the same value as acc - v / acc + v (IEEE a - b is
// a + (-b)) with one FP64 add instead of two and a select.
__device__ __forceinline__ double signed_out(double v, int e) {
  return __longlong_as_double(__double_as_longlong(v) ^ ((long long)(e & 1) << 63));
}

// Gather lists longer than these are summed cooperatively in 32 fixed chunks
// combined by a fixed pairwise tree (in-engine stamp programs / cedar_eval's).
constexpr int kLongGather = 16;
constexpr int kLongEval = 64;
constexpr int kLongPairs = 16;

// Pairwise sum of PER (a power of two) values pushed in order 0..PER-1, built
// as a binary counter: level b holds the sum of the last complete left subtree
// of 2^b values, so the association is the balanced tree ((v0+v1)+(v2+v3))+...
// with the left operand first.  It lets the chunk loop below stay rolled when a
// lane owns many chunks (K = 1, 2), which keeps those instantiations small;
// `total` is valid after the last push.
template <int PER>
struct PairwiseStack {
  static constexpr int LOG = PER >= 32 ? 5 : PER >= 16 ? 4 : PER >= 8 ? 3 : PER >= 4 ? 2 : PER >= 2 ? 1 : 0;
  double lvl[LOG > 0 ? LOG : 1];
  double total;
  __device__ __forceinline__ void push(int j, double v) {
    bool open = true;
#pragma unroll
    for (int b = 0; b < LOG; ++b) {
      if (open) {
        if ((j >> b) & 1) v = lvl[b] + v;
        else { lvl[b] = v; open = false; }
      }
    }
    total = v;
  }
};

// Sum, by one lane, of its chunks [rank * 32/K, (rank + 1) * 32/K) of a list of
// len items starting at a, combined by the fixed pairwise tree.  chunk(c0, c1)
// sums items [c0, c1) in order.  Up to 8 chunks per lane the loop is unrolled
// with the partial sums in registers; beyond that it is rolled (same bits).
template <int K, typename Chunk>
__device__ __forceinline__ double lane_chunk_sum(int a, int len, int rank, const Chunk &chunk) {
  constexpr int PER = 32 / K;
  if constexpr (PER <= 8) {
    double part[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int c = rank * PER + j;
      part[j] = chunk(a + (int)(((long long)len * c) >> 5), a + (int)(((long long)len * (c + 1)) >> 5));
    }
#pragma unroll
    for (int w = 1; w < PER; w <<= 1)
#pragma unroll
      for (int j = 0; j + w < PER; j += 2 * w) part[j] = part[j] + part[j + w];
    return part[0];
  } else {
    PairwiseStack<PER> tree;
#pragma unroll 1
    for (int j = 0; j < PER; ++j) {
      const int c = rank * PER + j;
      tree.push(j, chunk(a + (int)(((long long)len * c) >> 5), a + (int)(((long long)len * (c + 1)) >> 5)));
    }
    return tree.total;
  }
}

// Sum of a long gather list (entries (out << 1) | neg into dout) by the K lanes
// of a group (mask, rank): the list is cut into 32 fixed chunks, each summed in
// order, and the chunk sums are combined by a fixed pairwise tree.  A lane owns
// chunks [rank * 32/K, (rank + 1) * 32/K), so the lower tree levels are lane-local
// and the upper ones a butterfly: the result is the same bits for every K.
template <int K>
__device__ __forceinline__ double long_gather(const int *ptr, const int *ent, int q, const double *dout, int rank,
                                              unsigned mask) {
  const int a = ptr[q], len = ptr[q + 1] - a;
  double v = lane_chunk_sum<K>(a, len, rank, [&](int c0, int c1) {
    double acc = 0.0;
    for (int k = c0; k < c1; ++k) { const int e = ent[k]; acc = acc + signed_out(dout[e >> 1], e); }
    return acc;
  });
#pragma unroll
  for (int o = 1; o < K; o <<= 1) { const double u = __shfl_xor_sync(mask, v, o, K); v = (rank & o) ? u + v : v + u; }
  return v;
}

// Sum of A[p.x] * B[p.y] over pairs [p0, p1) by the K lanes of a group, in the
// same 32 fixed chunks and fixed tree as long_gather (bits independent of K).
template <int K>
__device__ __forceinline__ double long_pair_sum(const int2 *pairs, int p0, int p1, const double *A, const double *B,
                                                int rank, unsigned mask) {
  double v = lane_chunk_sum<K>(p0, p1 - p0, rank, [&](int c0, int c1) {
    double acc = 0.0;
    for (int k = c0; k < c1; ++k) { const int2 pr = pairs[k]; acc += A[pr.x] * B[pr.y]; }
    return acc;
  });
#pragma unroll
  for (int o = 1; o < K; o <<= 1) { const double u = __shfl_xor_sync(mask, v, o, K); v = (rank & o) ? u + v : v + u; }
  return v;
}

// workspace size in doubles for one instance
__host__ __device__ inline int ws_doubles(int n, int nnz_lu, int n_out, int n_src) {
  return 10 * n + nnz_lu + n_out + n_src + 8;
}

// One instance's workspace.  Vectors whose lifetimes never overlap share
// storage: the DC-only start point x0 and trial xs live in xm2 (adaptive BDF2
// history) and qd (trapezoidal derivative), which the transient first writes
// after the DC operating point; the charges at an accepted point (qt) live in F,
// which is dead once the step's Newton solve is over.
struct WS {
  double *x, *xn, *xm1, *xm2, *qn, *qm1, *qd, *hist, *F, *lu, *rd, *dout, *qt, *xs, *x0, *srcv;
  __device__ void bind(double *base, int n, int nnz_lu, int n_out, int n_src) {
    double *p = base;
    x = p; p += n; xn = p; p += n; xm1 = p; p += n; xm2 = p; p += n; qn = p; p += n; qm1 = p; p += n;
    qd = p; p += n; hist = p; p += n; F = p; p += n; rd = p; p += n;
    lu = p; p += nnz_lu; dout = p; p += n_out; srcv = p; p += n_src;
    x0 = xm2; xs = qd; qt = F;
  }
};

// Step-size factor: the largest k/8 (k = 1..16) with (k/8)^3 err <= 0.729, i.e.
// k/8 <= 0.9 err^(-1/3).  (k/8)^3 = k^3/512 is exact, so CPU and GPU agree.
__device__ __forceinline__ double step_factor(double err) {
  if ((4096.0 / 512.0) * err <= 0.729) return 2.0;
  if (!((1.0 / 512.0) * err <= 0.729)) return 0.125;
  int lo = 1, hi = 16;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (((double)(mid * mid * mid) / 512.0) * err <= 0.729) lo = mid; else hi = mid;
  }
  return lo * 0.125;
}

// Largest lte/sc ratio tracked as a fraction and compared by cross-multiplication
// (one division per step instead of one per unknown).
struct MaxRatio {
  double num, den; bool bad;
  __device__ MaxRatio() : num(0.0), den(1.0), bad(false) {}
  __device__ __forceinline__ void add(double lte, double sc) {
    if (!(lte <= 1e300) || !(sc > 0.0)) { bad = true; return; }
    if (lte * den > num * sc) { num = lte; den = sc; }
  }
  __device__ __forceinline__ void merge(double n2, double d2, bool b2) {
    bad = bad || b2;
    if (n2 * den > num * d2) { num = n2; den = d2; }
  }
  __device__ __forceinline__ double value() const { return bad ? 1e30 : num / den; }
};

// Reciprocal of a pivot: hardware approximation refined by two Newton-Raphson
// steps r <- r + r (1 - a r) (Flynn, 1970); within 1 ulp of 1/a for the normal
// range the pivot check admits.
__device__ __forceinline__ double pivot_rcp(double a) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(a));
  r = fma(r, fma(-a, r, 1.0), r);
  r = fma(r, fma(-a, r, 1.0), r);
  return r;
}

// |a| in [2^-997, 2^997): pivot magnitude accepted by the static-pivot LU
// (integer test on the exponent field, off the FP64 pipe)
__device__ __forceinline__ bool pivot_ok(double a) {
  unsigned e = (unsigned)(__double_as_longlong(a) >> 52) & 0x7ffu;
  return e >= 26u && e < 2020u;
}

// integer-domain helpers for non-negative doubles (bit patterns order like integers)
__device__ __forceinline__ long long abs_bits(double a) { return __double_as_longlong(a) & 0x7fffffffffffffffLL; }
__device__ __forceinline__ bool finite_big(double a) { return abs_bits(a) < 0x7e37e43c8800759cLL; }  // |a| < 1e300

// ------------------------------------------------------------- thread group (one CTA)
struct BlockGroup {
  int rank, size;
  double *red;  // shared scratch of >= 96 doubles
  __device__ BlockGroup(double *r) : rank(threadIdx.x), size(blockDim.x), red(r) {}
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  __device__ __forceinline__ bool any(bool p) const { return __syncthreads_or(p) != 0; }
  __device__ double reduce(double v, bool is_max) const {
    for (int o = 16; o > 0; o >>= 1) { double w = __shfl_xor_sync(0xffffffffu, v, o); v = is_max ? (w > v ? w : v) : (w < v ? w : v); }
    int warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[warp] = v;
    __syncthreads();
    double r = red[0];
    for (int i = 1; i < nw; ++i) { double w = red[i]; r = is_max ? (w > r ? w : r) : (w < r ? w : r); }
    __syncthreads();
    return r;
  }
  __device__ double max(double v) const { return reduce(v, true); }
  __device__ double min(double v) const { return reduce(v, false); }
  __device__ double ratio(MaxRatio m) const {
    for (int o = 16; o > 0; o >>= 1) {
      double n2 = __shfl_xor_sync(0xffffffffu, m.num, o), d2 = __shfl_xor_sync(0xffffffffu, m.den, o);
      bool b2 = __shfl_xor_sync(0xffffffffu, (int)m.bad, o) != 0;
      m.merge(n2, d2, b2);
    }
    int warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) { red[3 * warp] = m.num; red[3 * warp + 1] = m.den; red[3 * warp + 2] = m.bad ? 1.0 : 0.0; }
    __syncthreads();
    MaxRatio r; r.num = red[0]; r.den = red[1]; r.bad = red[2] != 0.0;
    for (int i = 1; i < nw; ++i) r.merge(red[3 * i], red[3 * i + 1], red[3 * i + 2] != 0.0);
    __syncthreads();
    return r.value();
  }
  __device__ int bcast(int v) const {
    __syncthreads();
    if (threadIdx.x == 0) ((int *)red)[0] = v;
    __syncthreads();
    int r = ((int *)red)[0];
    __syncthreads();
    return r;
  }
};

// ------------------------------------------------------------- options
struct EngOpts {
  int method, adaptive, dcop, max_newton;
  long long max_steps;
  double tstart, tstop, h, hmin, hmax, reltol, abstol_v, abstol_i, nr_factor, hfirst_frac;
};

struct EngStats {
  long long accepted, rejected, newton_iters, dc_iters;
  double hmin_seen, hmax_seen;
  int status, pad;
};

// Output sink: record every accepted point (plain) and/or probe samples (batch).
struct Sink {
  double *t_out, *x_out; long long cap, count;   // record mode (x in original order)
  const int *probes_int; int np, ns; double *samp; int next;
  double tstart, tstop;
};

template <class G>
struct Engine {
  const DTpl &T;
  const double *dp;   // derived params of this instance
  WS w;
  G g;

  double *dense = nullptr;   // (n + 2) n doubles for the dense DC fallback, or null
  bool dense_mode = false;   // factorise with dense partial pivoting (DC fallback)

  __device__ Engine(const DTpl &t, const double *dpar, double *ws, G grp) : T(t), dp(dpar), g(grp) {
    w.bind(ws, T.n, T.nnz_lu, T.n_out, T.n_src);
  }

  // Dense LU with partial pivoting (first maximum of a column wins; whole rows
  // swapped) of J scattered from the LU slots in original order, then J y = F;
  // y goes to w.F in internal order.  Fixed-order sums.  False on a zero pivot.
  __device__ bool dense_solve() {
    const int n = T.n;
    double *A = dense, *rhs = dense + (size_t)n * n;
    int *piv = reinterpret_cast<int *>(rhs + n);
    for (int i = g.rank; i < n * n; i += g.size) A[i] = 0.0;
    g.sync();
    for (int q = g.rank; q < T.nnz_lu; q += g.size) { const int2 rc = T.lu_orig[q]; A[(size_t)rc.x * n + rc.y] = w.lu[q]; }
    for (int e = g.rank; e < n; e += g.size) rhs[e] = w.F[T.eq_pos[e]];
    g.sync();
    for (int k = 0; k < n; ++k) {
      double lb = -1.0; int li = n;
      for (int i = k + g.rank; i < n; i += g.size) { const double v = fabs(A[(size_t)i * n + k]); if (v > lb) { lb = v; li = i; } }
      const double best = g.max(lb);
      if (!(best > 0.0)) return false;
      const int p = (int)g.min(lb == best ? (double)li : 1e300);
      if (g.rank == 0) piv[k] = p;
      if (p != k)
        for (int j = g.rank; j < n; j += g.size) {
          const double t = A[(size_t)k * n + j]; A[(size_t)k * n + j] = A[(size_t)p * n + j]; A[(size_t)p * n + j] = t;
        }
      g.sync();
      const double inv = 1.0 / A[(size_t)k * n + k];
      for (int i = k + 1 + g.rank; i < n; i += g.size) {
        double *Ai = A + (size_t)i * n;
        const double aik = Ai[k];
        if (aik == 0.0) continue;
        const double l = aik * inv;
        Ai[k] = l;
        const double *Ak = A + (size_t)k * n;
        for (int j = k + 1; j < n; ++j) Ai[j] -= l * Ak[j];
      }
      g.sync();
    }
    if (g.rank == 0)
      for (int k = 0; k < n; ++k) if (piv[k] != k) { const double t = rhs[k]; rhs[k] = rhs[piv[k]]; rhs[piv[k]] = t; }
    g.sync();
    for (int k = 0; k < n; ++k) {
      const double bk = rhs[k];
      for (int i = k + 1 + g.rank; i < n; i += g.size) { const double l = A[(size_t)i * n + k]; if (l != 0.0) rhs[i] -= l * bk; }
      g.sync();
    }
    for (int k = n - 1; k >= 0; --k) {
      if (g.rank == 0) rhs[k] = rhs[k] / A[(size_t)k * n + k];
      g.sync();
      const double bk = rhs[k];
      for (int i = g.rank; i < k; i += g.size) rhs[i] -= A[(size_t)i * n + k] * bk;
      g.sync();
    }
    for (int u = g.rank; u < n; u += g.size) w.F[T.iorder[u]] = rhs[u];
    g.sync();
    return true;
  }

  // K1: evaluate devices at x (internal order); q_only restricts to charge devices
  __device__ void eval_devices(const double *x, const EvalCtx &ctx, bool q_only) {
    for (int d = g.rank; d < T.n_dev; d += g.size) {
      int gi = 0;
      while (d >= T.dev_end[gi]) ++gi;
      const DGroup gr = T.grp[gi];
      if (q_only && !model_has_q(gr.model)) continue;
      int i = d - (gi ? T.dev_end[gi - 1] : 0);
      const int *tm = T.term + gr.term_off + i * gr.ntx;
      double v[CEDAR_MAX_TERM];
      for (int k = 0; k < gr.ntx; ++k) { int u = tm[k]; v[k] = u < 0 ? 0.0 : x[u]; }
      eval_device(gr.model, dp + gr.dpar_off + i, gr.n_inst, v, nullptr, ctx, T.pwl, w.dout + gr.out_off + i,
                  gr.n_inst);
    }
  }

  __device__ __forceinline__ double gather(const int *ptr, const int *ent, int s, double acc) const {
    int a = ptr[s], b = ptr[s + 1];
    for (int k = a; k < b; ++k) { int e = ent[k]; acc = acc + signed_out(w.dout[e >> 1], e); }
    return acc;
  }

  // K2: J slots and residual rows (F = hist + contributions)
  // gshunt (DC homotopy): node rows get -gshunt * (x - xref) (xref null = ground)
  __device__ void stamp(const double *hist, double gshunt, const double *x, const double *xref) {
    for (int s = g.rank; s < T.nnz_lu; s += g.size)
      if (T.jlu_ptr[s + 1] - T.jlu_ptr[s] <= kLongGather) w.lu[s] = gather(T.jlu_ptr, T.jlu_ent, s, 0.0);
    for (int r = g.rank; r < T.n; r += g.size)
      if (T.fint_ptr[r + 1] - T.fint_ptr[r] <= kLongGather) w.F[r] = gather(T.fint_ptr, T.fint_ent, r, hist ? hist[r] : 0.0);
    // long lists (supply rails): the first warp sums each in fixed chunks
    if (g.rank < 32) {
      for (int t = 0; t < T.n_long_lu; ++t) {
        const int q = T.long_lu[t];
        const double v = long_gather<32>(T.jlu_ptr, T.jlu_ent, q, w.dout, g.rank, 0xffffffffu);
        if (g.rank == 0) w.lu[q] = v;
      }
      for (int t = 0; t < T.n_long_fi; ++t) {
        const int r = T.long_fi[t];
        const double v = long_gather<32>(T.fint_ptr, T.fint_ent, r, w.dout, g.rank, 0xffffffffu);
        if (g.rank == 0) w.F[r] = (hist ? hist[r] : 0.0) + v;
      }
    }
    if (gshunt != 0.0) {
      g.sync();
      for (int u = g.rank; u < T.n_nodes; u += g.size) {
        int c = T.gs_col[u];
        w.lu[T.gs_slot[u]] -= gshunt;
        w.F[T.gs_row[u]] -= gshunt * (x[c] - (xref ? xref[c] : 0.0));
      }
    }
  }

  // charges at x into qt (internal rows)
  __device__ void eval_q(const double *x, const EvalCtx &ctx, double *q) {
    eval_devices(x, ctx, true);
    g.sync();
    for (int r = g.rank; r < T.n; r += g.size) q[r] = gather(T.qint_ptr, T.qint_ent, r, 0.0);
    g.sync();
  }

  // K4: level-scheduled Crout LU in place; returns false on a zero pivot
  __device__ bool factor() {
    bool bad = false;
    for (int l = 0; l < T.lu_nlev; ++l) {
      int t0 = T.lu_lvl[l], t1 = T.lu_lvl[l + 1];
      for (int t = t0 + g.rank; t < t1; t += g.size) {
        int s = T.lu_slot[t], info = T.lu_info[t];
        double acc = w.lu[s];
        for (int k = T.lu_pp[t]; k < T.lu_pp[t + 1]; ++k) { int2 p = T.lu_pair[k]; acc -= w.lu[p.x] * w.lu[p.y]; }
        int kind = info & 3, j = info >> 2;
        if (kind == 2) acc *= w.rd[j];
        else if (kind == 1) {
          if (!(fabs(acc) > 1e-300) || !(fabs(acc) < 1e300)) bad = true;
          w.rd[j] = 1.0 / acc;
        }
        w.lu[s] = acc;
      }
      g.sync();
    }
    return !g.any(bad);
  }

  // K5: solve LU y = b in place (b = F)
  __device__ void solve(double *b) {
    for (int l = 0; l < T.fw_nlev; ++l) {
      for (int t = T.fw_lvl[l] + g.rank; t < T.fw_lvl[l + 1]; t += g.size) {
        int i = T.fw_row[t]; double acc = b[i];
        for (int k = T.fw_ptr[t]; k < T.fw_ptr[t + 1]; ++k) { int2 p = T.fw_pair[k]; acc -= w.lu[p.x] * b[p.y]; }
        b[i] = acc;
      }
      g.sync();
    }
    for (int l = 0; l < T.bw_nlev; ++l) {
      for (int t = T.bw_lvl[l] + g.rank; t < T.bw_lvl[l + 1]; t += g.size) {
        int i = T.bw_row[t]; double acc = b[i];
        for (int k = T.bw_ptr[t]; k < T.bw_ptr[t + 1]; ++k) { int2 p = T.bw_pair[k]; acc -= w.lu[p.x] * b[p.y]; }
        b[i] = acc * w.rd[i];
      }
      g.sync();
    }
  }

  // Newton on Fi(x,t) + cj Fq(x) + hist = 0.  Returns iterations (>0), -iters on
  // failure, 0 on a zero pivot.  Mirrors the oracle's newton().
  __device__ int newton(double *x, const EvalCtx &ctx, const double *hist, double rel, double av, double ai,
                        int maxit, double vlim, double gshunt, const double *xref = nullptr) {
    for (int it = 1; it <= maxit; ++it) {
      eval_devices(x, ctx, false);
      g.sync();
      stamp(hist, gshunt, x, xref);
      g.sync();
      if (dense_mode) { if (!dense_solve()) return 0; }
      else { if (!factor()) return 0; solve(w.F); }
      // dx = -F ; finiteness and DC damping
      bool nonfinite = false; double mx = 0.0;
      for (int i = g.rank; i < T.n; i += g.size) {
        double d = w.F[i];
        if (!isfinite(d)) nonfinite = true;
        if (T.is_node[i]) { double a = fabs(d); mx = a > mx ? a : mx; }
      }
      if (g.any(nonfinite)) return -it;
      double scale = 1.0;
      if (vlim > 0) { mx = g.max(mx); if (mx > vlim) scale = vlim / mx; }
      bool conv = (scale == 1.0);
      for (int i = g.rank; i < T.n; i += g.size) {
        double d = -w.F[i] * scale;
        double xi = x[i] + d;
        x[i] = xi;
        double lim = rel * fabs(xi) + (T.is_node[i] ? av : ai);
        if (!(fabs(d) <= lim)) conv = false;
      }
      bool notconv = g.any(!conv);
      g.sync();
      if (!notconv) return it;
    }
    return -maxit;
  }

  __device__ void copy(double *dst, const double *src) {
    for (int i = g.rank; i < T.n; i += g.size) dst[i] = src[i];
  }
  __device__ void fill(double *dst, double v) {
    for (int i = g.rank; i < T.n; i += g.size) dst[i] = v;
  }

  __device__ double next_bp(double t, double eps) {
    double best = 1e300;
    for (int s = g.rank; s < T.n_src; s += g.size) {
      double b = source_next_bp(dp + T.src_off[s], T.src_stride[s], t, eps, T.pwl);
      best = b < best ? b : best;
    }
    return g.min(best);
  }

  // DC operating point (mirrors the oracle's dcop()); x internal order.
  // DC operating point; when the homotopy fails with the static pivot order and
  // dense scratch is available, the whole homotopy reruns from the initial guess
  // with dense partial pivoting.
  __device__ int dcop(double *x, double t, double rel, double av, double ai, long long *iters) {
    int r = dcop_pass(x, t, rel, av, ai, iters);
    if (r == CEDAR_ST_DCOP && dense && T.n > 0) {
      copy(x, w.x0);
      g.sync();
      dense_mode = true;
      r = dcop_pass(x, t, rel, av, ai, iters);
      dense_mode = false;
    }
    return r;
  }

  __device__ int dcop_pass(double *x, double t, double rel, double av, double ai, long long *iters) {
    const int maxit = 100; const double vlim = 0.0;  // no damping: PTC bounds the steps
    const long long budget = 20000;
    EvalCtx ctx{t, 0.0, 1.0, T.gmin, true, false};
    copy(w.x0, x);
    g.sync();
    long long used = 0;
    int r = newton(x, ctx, nullptr, rel, av, ai, maxit, vlim, 0.0);
    used += r < 0 ? -r : r;
    if (r > 0) { *iters += used; return CEDAR_ST_OK; }
    // pseudo-transient continuation (xr = w.xm1, scratch = w.xs)
    double *xr = w.xm1;
    for (int pass = 0; pass < 2; ++pass) {
      const double pv = pass == 0 ? 0.5 : 0.0;
      copy(xr, w.x0);
      g.sync();
      double gs = 1e-2; int fails = 0; bool ptc_ok = false;
      while (used < budget && fails <= 60) {
        copy(w.xs, xr);
        g.sync();
        r = newton(w.xs, ctx, nullptr, rel, av, ai, 50, pv, gs, xr);
        used += r < 0 ? -r : r;
        if (r > 0) {
          copy(xr, w.xs);
          g.sync();
          if (gs <= 1e-14) { ptc_ok = true; break; }
          gs *= 0.1;
        } else { gs *= 4.0; ++fails; }
      }
      if (ptc_ok) {
        copy(x, xr);
        g.sync();
        r = newton(x, ctx, nullptr, rel, av, ai, maxit, pv, 0.0);
        used += r < 0 ? -r : r;
        if (r > 0) { *iters += used; return CEDAR_ST_OK; }
      }
    }
    // source stepping from zero
    fill(x, 0.0);
    g.sync();
    double lam = 0.0, dl = 0.1; int halv = 0; bool ok = true;
    while (lam < 1.0) {
      if (used >= budget) { ok = false; break; }
      double ln = lam + dl < 1.0 ? lam + dl : 1.0;
      copy(w.xs, x);
      g.sync();
      ctx.src_scale = ln;
      r = newton(w.xs, ctx, nullptr, rel, av, ai, maxit, vlim, 0.0);
      used += r < 0 ? -r : r;
      if (r > 0) { copy(x, w.xs); g.sync(); lam = ln; halv = 0; dl = dl * 2 < 0.1 ? dl * 2 : 0.1; }
      else { dl *= 0.5; if (++halv > 8) { ok = false; break; } }
    }
    *iters += used;
    return ok ? CEDAR_ST_OK : CEDAR_ST_DCOP;
  }

  // ---- output sink helpers
  __device__ void sink_point(Sink &sk, double t, const double *x) {
    if (sk.t_out) {
      if (sk.count < sk.cap) {
        if (g.rank == 0) sk.t_out[sk.count] = t;
        for (int i = g.rank; i < T.n; i += g.size) sk.x_out[sk.count * T.n + T.order[i]] = x[i];
      }
      sk.count++;
    }
  }
  __device__ double sample_ts(const Sink &sk, int j) const {
    return j == sk.ns - 1 ? sk.tstop : sk.tstart + (sk.tstop - sk.tstart) * ((double)j / (double)(sk.ns - 1));
  }
  __device__ void sink_start(Sink &sk, const double *x) {
    if (!sk.samp || sk.ns <= 0) return;
    for (int p = g.rank; p < sk.np; p += g.size) { int u = sk.probes_int[p]; sk.samp[(long long)p * sk.ns] = u >= 0 ? x[u] : 0.0; }
    sk.next = 1;
  }
  __device__ void sink_step(Sink &sk, bool have0, double t0, const double *x0, double t1, const double *x1,
                            double t2, const double *x2) {
    if (!sk.samp) return;
    while (sk.next < sk.ns && sample_ts(sk, sk.next) <= t2) {
      double t = sample_ts(sk, sk.next);
      for (int p = g.rank; p < sk.np; p += g.size) {
        int u = sk.probes_int[p]; double v;
        if (u < 0) v = 0.0;
        else if (have0) {
          double L0 = (t - t1) * (t - t2) / ((t0 - t1) * (t0 - t2));
          double L1 = (t - t0) * (t - t2) / ((t1 - t0) * (t1 - t2));
          double L2 = (t - t0) * (t - t1) / ((t2 - t0) * (t2 - t1));
          v = x0[u] * L0 + x1[u] * L1 + x2[u] * L2;
        } else {
          double a = (t - t1) / (t2 - t1);
          v = x1[u] + (x2[u] - x1[u]) * a;
        }
        sk.samp[(long long)p * sk.ns + sk.next] = v;
      }
      sk.next++;
    }
  }

  // Whole transient (mirrors the oracle's tran()).  x: internal order, in/out.
  __device__ void tran(double *x, const EngOpts &o, Sink &sk, EngStats &st, const double *perturb) {
    const int n = T.n;
    st.accepted = st.rejected = st.newton_iters = st.dc_iters = 0;
    st.hmin_seen = 1e300; st.hmax_seen = 0; st.status = CEDAR_ST_OK; st.pad = 0;
    const double rel = o.nr_factor * o.reltol, av = o.nr_factor * o.abstol_v, ai = o.nr_factor * o.abstol_i;
    if (o.dcop) {
      int s = dcop(x, o.tstart, rel, av, ai, &st.dc_iters);
      if (s != CEDAR_ST_OK) { st.status = s; return; }
    }
    if (perturb) { for (int i = g.rank; i < n; i += g.size) x[i] += perturb[i]; g.sync(); }
    EvalCtx ctx{o.tstart, 0.0, 1.0, T.gmin, false, false};
    eval_q(x, ctx, w.qn);
    copy(w.xn, x);
    g.sync();
    sink_point(sk, o.tstart, x);
    sink_start(sk, x);
    double *xp = x;   // Newton iterate / predictor lives in x
    if (!o.adaptive) {
      const double h = o.h;
      const long long N = llround((o.tstop - o.tstart) / h);
      fill(w.qd, 0.0);
      double tprev = o.tstart, tprev2 = o.tstart; bool have_prev = false;
      for (long long k = 1; k <= N; ++k) {
        double t = (k == N) ? o.tstop : DADD(o.tstart, DMUL((double)k, h));
        double hk = t - tprev, cj;
        if (o.method == CEDAR_TRAP) {
          cj = 2.0 / hk;
          for (int i = g.rank; i < n; i += g.size) w.hist[i] = -cj * w.qn[i] - w.qd[i];
        } else if (k == 1) {
          cj = 1.0 / hk;
          for (int i = g.rank; i < n; i += g.size) w.hist[i] = -w.qn[i] * cj;
        } else {
          cj = 1.5 / hk;
          double r2h = 0.5 / hk;
          for (int i = g.rank; i < n; i += g.size) w.hist[i] = (-4.0 * w.qn[i] + w.qm1[i]) * r2h;
        }
        if (k == 1) copy(xp, w.xn);
        else for (int i = g.rank; i < n; i += g.size) xp[i] = 2.0 * w.xn[i] - w.xm1[i];
        g.sync();
        ctx.t = t; ctx.cj = cj;
        int r = newton(xp, ctx, w.hist, rel, av, ai, o.max_newton, 0.0, 0.0);
        st.newton_iters += r < 0 ? -r : r;
        if (r <= 0) { st.status = r == 0 ? CEDAR_ST_ZERO_PIVOT : CEDAR_ST_NEWTON; copy(x, w.xn); g.sync(); return; }
        eval_q(xp, ctx, w.qt);
        for (int i = g.rank; i < n; i += g.size) {
          if (o.method == CEDAR_TRAP) w.qd[i] = cj * w.qt[i] + w.hist[i];
          w.qm1[i] = w.qn[i]; w.qn[i] = w.qt[i];
        }
        g.sync();
        sink_step(sk, have_prev, tprev2, w.xm1, tprev, w.xn, t, xp);
        g.sync();
        bool nf = false;
        for (int i = g.rank; i < n; i += g.size) { w.xm1[i] = w.xn[i]; w.xn[i] = xp[i]; if (!isfinite(xp[i])) nf = true; }
        nf = g.any(nf);
        tprev2 = tprev; tprev = t; have_prev = true;
        st.accepted++; st.hmin_seen = hk < st.hmin_seen ? hk : st.hmin_seen; st.hmax_seen = hk > st.hmax_seen ? hk : st.hmax_seen;
        sink_point(sk, t, w.xn);
        if (nf) { st.status = CEDAR_ST_NAN; return; }
      }
      return;
    }
    // ---- adaptive variable-step BDF2
    const double span = o.tstop - o.tstart, eps_bp = span * 1e-12;
    double t = o.tstart, tn1 = t, tn2 = t;
    int npts = 1;
    auto restart_h = [&](double tt) {
      double nb = next_bp(tt, eps_bp); nb = nb < o.tstop ? nb : o.tstop;
      double dist = nb - tt; dist = dist < o.hmax ? dist : o.hmax;
      double hf = o.hfirst_frac * dist;
      if (o.h > 0) hf = o.h < hf ? o.h : hf;
      return hf;
    };
    double hnext = restart_h(t);
    long long nsteps = 0;
    while (t < o.tstop) {
      if (++nsteps > o.max_steps) { st.status = CEDAR_ST_MAX_STEPS; break; }
      double tb = next_bp(t, eps_bp); tb = tb < o.tstop ? tb : o.tstop;
      double h = hnext < o.hmax ? hnext : o.hmax;
      bool hit = false;
      if (tb - t <= 1.1 * h) { h = tb - t; hit = true; }
      double tnew = hit ? tb : t + h;
      h = tnew - t;
      int order = npts >= 2 ? 2 : 1;
      double cj, h1 = t - tn1;
      if (order == 1) {
        cj = 1.0 / h;
        for (int i = g.rank; i < n; i += g.size) w.hist[i] = -w.qn[i] * cj;
      } else {
        double wr = h / h1, rh = 1.0 / h;
        cj = (1.0 + 2.0 * wr) / ((1.0 + wr) * h);
        double a1 = -(1.0 + wr), a2 = wr * wr / (1.0 + wr);
        for (int i = g.rank; i < n; i += g.size) w.hist[i] = (a1 * w.qn[i] + a2 * w.qm1[i]) * rh;
      }
      if (npts >= 2) { double rr = h / h1; for (int i = g.rank; i < n; i += g.size) xp[i] = w.xn[i] + rr * (w.xn[i] - w.xm1[i]); }
      else copy(xp, w.xn);
      g.sync();
      ctx.t = tnew; ctx.cj = cj;
      int r = newton(xp, ctx, w.hist, rel, av, ai, o.max_newton, 0.0, 0.0);
      st.newton_iters += r < 0 ? -r : r;
      if (r <= 0) {
        st.rejected++;
        hnext = h * 0.125;
        if (hnext < o.hmin) { st.status = r == 0 ? CEDAR_ST_ZERO_PIVOT : CEDAR_ST_DT_UNDERFLOW; break; }
        continue;
      }
      double err = 0.0;
      if (npts >= 3) {
        double h2 = tn1 - tn2;
        double rh = 1.0 / h, rh1 = 1.0 / h1, rh2 = 1.0 / h2;
        double ra = 1.0 / (h + h1), rb = 1.0 / (h1 + h2), rc = 1.0 / (h + h1 + h2);
        double coef = h * h * (h + h1) * (h + h1) / (2.0 * h + h1);
        MaxRatio mr;
        for (int i = g.rank; i < n; i += g.size) {
          if (!T.is_node[i]) continue;
          double d10 = (xp[i] - w.xn[i]) * rh;
          double d21 = (w.xn[i] - w.xm1[i]) * rh1;
          double d32 = (w.xm1[i] - w.xm2[i]) * rh2;
          double dd3 = ((d10 - d21) * ra - (d21 - d32) * rb) * rc;
          double lte = fabs(dd3) * coef;
          double ax = fabs(xp[i]), bx = fabs(w.xn[i]);
          mr.add(lte, o.reltol * (ax > bx ? ax : bx) + o.abstol_v);
        }
        err = g.ratio(mr);
      } else if (npts == 2) {
        double rh = 1.0 / h, rh1 = 1.0 / h1, ra = 1.0 / (h + h1), hh = h * h;
        MaxRatio mr;
        for (int i = g.rank; i < n; i += g.size) {
          if (!T.is_node[i]) continue;
          double dd2 = ((xp[i] - w.xn[i]) * rh - (w.xn[i] - w.xm1[i]) * rh1) * ra;
          double lte = fabs(dd2) * hh;
          double ax = fabs(xp[i]), bx = fabs(w.xn[i]);
          mr.add(lte, o.reltol * (ax > bx ? ax : bx) + o.abstol_v);
        }
        err = g.ratio(mr);
      }
      if (err > 1.0) {
        st.rejected++;
        hnext = h * step_factor(err);
        if (hnext < o.hmin) { st.status = CEDAR_ST_DT_UNDERFLOW; break; }
        continue;
      }
      eval_q(xp, ctx, w.qt);
      for (int i = g.rank; i < n; i += g.size) { w.qm1[i] = w.qn[i]; w.qn[i] = w.qt[i]; }
      g.sync();
      sink_step(sk, npts >= 2, tn1, w.xm1, t, w.xn, tnew, xp);
      g.sync();
      bool nf = false;
      for (int i = g.rank; i < n; i += g.size) {
        w.xm2[i] = w.xm1[i]; w.xm1[i] = w.xn[i]; w.xn[i] = xp[i];
        if (!isfinite(xp[i])) nf = true;
      }
      nf = g.any(nf);
      tn2 = tn1; tn1 = t; t = tnew;
      st.accepted++; st.hmin_seen = h < st.hmin_seen ? h : st.hmin_seen; st.hmax_seen = h > st.hmax_seen ? h : st.hmax_seen;
      sink_point(sk, t, w.xn);
      if (nf) { st.status = CEDAR_ST_NAN; break; }
      if (npts < 3) ++npts;
      double fac = (err > 0.0) ? step_factor(err) : 1.0;
      hnext = h * fac;
      if (hit && t < o.tstop) { npts = 1; hnext = restart_h(t); }
    }
    copy(x, w.xn);
    g.sync();
    if (st.status == CEDAR_ST_OK && t < o.tstop) st.status = CEDAR_ST_MAX_STEPS;
  }
};

}  // namespace cedar
