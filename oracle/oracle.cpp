// oracle.cpp — CPU FP64 restatement of CedarSim's transient hot path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or calls
// this file; it is used by tests/ (as the checker), by __graft_entry__.smoke() and
// by bench.py's CPU-baseline leg.
//
// What it restates (CedarSim 0.12.0, file:line within the CedarSim project):
//   * KCL / branch sign convention and multiplicity:   src/simulate_ir.jl:28-54,112-120
//   * device equations R, C, L, V, I, E, G:             src/simpledevices.jl:49-132,274-373
//   * source waveforms pulse / pwl / sin, breakpoint rule (a corner belongs to the
//     next segment):                                    src/spectre_env.jl:15-69,144-176
//   * Verilog-A contribution semantics (I(a,b) <+ ..., current leaves a, enters b;
//     ddx on a two-node probe = (d/dVa - d/dVb)/2):     src/vasim.jl:128-180,392-412,824-839
//   * $temperature = temp + 273.15, SimSpec gmin=1e-12: src/va_env.jl:123, simulate_ir.jl:12-20
//   * Jacobian = dF/du + gamma dF/du' as DAECompiler's dense jac(J,du,u,p,gamma,t)
//     (benchmarks/benchmark_common.jl:152-158) — formed here densely by forward-mode
//     dual numbers, the same way vasim.jl seeds ForwardDiff duals (vasim.jl:347-374),
//     and factored by dense LU with partial pivoting, the default direct solve of
//     Sundials IDA that tran! uses (src/sweeps.jl:456).
// Integrators (fixed-step trapezoidal, fixed/variable-step BDF2 with LTE control),
// Newton, and the DC homotopy are not in the reference (it delegates to IDA); they
// restate the algorithm the GPU engine documents, so GPU and CPU take the same steps.
//
// Build: oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off -shared -fPIC).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "../include/cedar.h"
// Verilog-A models: the device code the product's emitter writes from the .va
// sources (cedarsim.jl_gb300/va), compiled here for the CPU.  The oracle runs it
// as a black-box device evaluation; the emitter itself is checked against an
// independent interpretation of the same sources (oracle/va_interp.py).
#include <math.h>
#include "va_models.gen.h"

namespace orc {

// ---------------------------------------------------------------- dual numbers
constexpr int ND = 6;
constexpr int kMaxIdx = 16;   // terminal values of one device (Verilog-A models can have more)
struct Dual {
  double v;
  double d[ND];
  Dual() : v(0) { for (int i = 0; i < ND; ++i) d[i] = 0; }
  Dual(double x) : v(x) { for (int i = 0; i < ND; ++i) d[i] = 0; }
  static Dual seed(double x, int k) { Dual r(x); if (k >= 0) r.d[k] = 1.0; return r; }
};
static inline Dual operator+(const Dual &a, const Dual &b) { Dual r; r.v = a.v + b.v; for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
static inline Dual operator-(const Dual &a, const Dual &b) { Dual r; r.v = a.v - b.v; for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
static inline Dual operator-(const Dual &a) { Dual r; r.v = -a.v; for (int i = 0; i < ND; ++i) r.d[i] = -a.d[i]; return r; }
static inline Dual operator*(const Dual &a, const Dual &b) { Dual r; r.v = a.v * b.v; for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
static inline Dual operator*(double s, const Dual &b) { Dual r; r.v = s * b.v; for (int i = 0; i < ND; ++i) r.d[i] = s * b.d[i]; return r; }
static inline Dual operator*(const Dual &b, double s) { return s * b; }
static inline Dual operator/(const Dual &a, double s) { Dual r; r.v = a.v / s; for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] / s; return r; }
static inline Dual dexp_lim(const Dual &a) {
  // limexp: exp(x) for x <= 80, linear continuation above (keeps Newton finite)
  const double X = 80.0;
  Dual r;
  if (a.v <= X) { double e = std::exp(a.v); r.v = e; for (int i = 0; i < ND; ++i) r.d[i] = e * a.d[i]; }
  else { double e = std::exp(X); r.v = e * (1.0 + (a.v - X)); for (int i = 0; i < ND; ++i) r.d[i] = e * a.d[i]; }
  return r;
}

// Further dual operations used by the Verilog-A restatements below.
static inline Dual operator/(const Dual &a, const Dual &b) {
  Dual r; r.v = a.v / b.v;
  for (int i = 0; i < ND; ++i) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v);
  return r;
}
static inline Dual operator/(double s, const Dual &b) { return Dual(s) / b; }
static inline Dual operator+(const Dual &a, double s) { return a + Dual(s); }
static inline Dual operator+(double s, const Dual &a) { return Dual(s) + a; }
static inline Dual operator-(const Dual &a, double s) { return a - Dual(s); }
static inline Dual operator-(double s, const Dual &a) { return Dual(s) - a; }
static inline Dual dexp(const Dual &a) {
  Dual r; const double e = std::exp(a.v); r.v = e;
  for (int i = 0; i < ND; ++i) r.d[i] = e * a.d[i];
  return r;
}
static inline Dual dsqrt(const Dual &a) {
  Dual r; const double q = std::sqrt(a.v); r.v = q;
  for (int i = 0; i < ND; ++i) r.d[i] = a.d[i] == 0.0 ? 0.0 : a.d[i] * (0.5 / q);
  return r;
}
// |a| with the derivative of the a >= 0 side at 0 (the Verilog-A abs of the emitter)
static inline Dual dabs(const Dual &a) { return a.v < 0.0 ? -a : a; }

// ---------------------------------------------------------------- Verilog-A, restated
// The Verilog-A modules this project ships (cedarsim.jl_gb300/va/models/*.va),
// written out again by hand in residual form over this file's own dual numbers,
// so that GPU runs of circuits with these modules are checked against an
// evaluation that shares no code with the emitter.  Contribution semantics
// (src/vasim.jl:128-180): I(a,b) <+ e adds -e to the residual of a and +e to b;
// a voltage-contributed branch V(a,b) <+ e carries a branch-current unknown I,
// adds -I / +I to a / b and the branch row V(a) - V(b) - e, with ddt() terms of a
// contribution as charges (ddt(q) enters the charge part of the same rows).
// ddx on a two-node probe is (d/dVa - d/dVb)/2 (src/vasim.jl:400-411); real ->
// integer parameters round half away from zero (src/va_env.jl:92-110).
// p: the raw parameters (declaration order, then $param_given flags, then m),
// vt: thermal voltage; V: terminal values (ports, internal nodes, branch current)
// seeded as dual directions.  Returns false for a module not restated here.
static bool va_restated(const char *name, const double *p, double vt, double gmin, const Dual *V, Dual *Fi,
                        Dual *Fq) {
  auto I_ab = [&](int a, int b, const Dual &e) { Fi[a] = Fi[a] - e; Fi[b] = Fi[b] + e; };
  auto Q_ab = [&](int a, int b, const Dual &q) { Fq[a] = Fq[a] - q; Fq[b] = Fq[b] + q; };
  const std::string m(name);
  if (m == "va_resistor" || m == "va_resistor_1f") {          // I(p,n) <+ V(p,n)/R (noise only in noise analysis)
    I_ab(0, 1, (V[0] - V[1]) / p[0]);
  } else if (m == "va_capacitor") {                            // I(p,n) <+ ddt(C V(p,n))
    Q_ab(0, 1, p[0] * (V[0] - V[1]));
  } else if (m == "va_diode") {                                // IS AREA (limexp(V/(N vt)) - 1) + gmin V
    const Dual v = V[0] - V[1];
    I_ab(0, 1, (p[0] * p[2]) * (dexp_lim(v / (p[1] * vt)) - 1.0) + gmin * v);
  } else if (m == "va_diode_cj") {                             // + ddt(TT id + CJ0 vd)
    const Dual vd = V[0] - V[1];
    const Dual id = p[0] * (dexp_lim(vd / (p[1] * vt)) - 1.0);
    I_ab(0, 1, id + gmin * vd);
    Q_ab(0, 1, p[2] * id + p[3] * vd);
  } else if (m == "va_diode_rs") {                             // a -RS- ai -diode- c
    I_ab(0, 2, (V[0] - V[2]) / p[2]);
    const Dual vd = V[2] - V[1];
    I_ab(2, 1, p[0] * (dexp_lim(vd / (p[1] * vt)) - 1.0) + gmin * vd);
  } else if (m == "va_inductor") {                             // V(p,n) <+ ddt(L I(p,n))
    const Dual &I = V[2];
    Fi[0] = Fi[0] - I; Fi[1] = Fi[1] + I;
    Fi[2] = Fi[2] + (V[0] - V[1]);
    Fq[2] = Fq[2] - p[0] * I;
  } else if (m == "va_thevenin") {                             // V(p,n) <+ VS + RS I(p,n)
    const Dual &I = V[2];
    Fi[0] = Fi[0] - I; Fi[1] = Fi[1] + I;
    Fi[2] = Fi[2] + (V[0] - V[1]) - (p[0] + p[1] * I);
  } else if (m == "va_mos1") {                                 // level 1, drain/source exchange for vds < 0
    const double type = p[0], beta = p[3] * p[1] / p[2], vto = p[4], lam = p[5];
    const Dual vgs = type * (V[1] - V[2]), vds = type * (V[0] - V[2]);
    Dual vov, vde; double dir;
    if (vds.v >= 0) { vov = vgs - type * vto; vde = vds; dir = 1.0; }
    else { vov = vgs - vds - type * vto; vde = -vds; dir = -1.0; }
    Dual id;
    if (vov.v <= 0) id = Dual(0.0);
    else if (vde.v < vov.v) id = ((beta * (vov - 0.5 * vde)) * vde) * (1.0 + lam * vde);
    else id = (((0.5 * beta) * vov) * vov) * (1.0 + lam * vde);
    I_ab(0, 2, (type * dir) * id + gmin * (V[0] - V[2]));
  } else if (m == "va_nlvcr") {                                // V(d,s) ddx(R V(g,s)^2, V(g,s)) = V(d,s) 2 R V(g,s)
    I_ab(0, 2, (V[0] - V[2]) * ((2.0 * p[0]) * (V[1] - V[2])));
  } else if (m == "va_vccs_sat") {                             // gm f(V(cp,cn)), f by MODE
    const double gm = p[4] != 0.0 ? p[1] : p[0], vs = p[2];
    const long mode = std::lround(p[3]);
    const Dual vc = V[2] - V[3];
    Dual f;
    if (mode == 0) f = vc;
    else if (mode == 1) {                                      // sign(x) s (1 - e)/(1 + e), e = exp(-2|x|/s)
      const Dual e = dexp((-2.0 / vs) * dabs(vc));
      f = (vc.v >= 0 ? 1.0 : -1.0) * vs * ((1.0 - e) / (1.0 + e));
    } else {                                                   // x / sqrt(1 + (x/s)^2)
      const Dual r = vc / vs;
      f = vc / dsqrt(1.0 + r * r);
    }
    I_ab(0, 1, gm * f);
  } else {
    return false;
  }
  return true;
}

// Dense fi/fq[nx], G/C[nx*nx] of model k through va_restated (dp: np raw
// parameters then the thermal voltage); false when k is not restated by hand.
static bool va_full_restated(int k, const double *dp, int np, const double *v, int nx, double gmin, double *fi,
                             double *fq, double *G, double *Cm) {
  if (k < 0 || k >= cedar::va::kCount || nx > ND) return false;
  Dual V[ND], Fi[ND], Fq[ND];
  for (int q = 0; q < nx; ++q) V[q] = Dual::seed(v[q], q);
  if (!va_restated(cedar::va::kName[k], dp, dp[np], gmin, V, Fi, Fq)) return false;
  for (int r = 0; r < nx; ++r) {
    fi[r] = Fi[r].v; fq[r] = Fq[r].v;
    for (int q = 0; q < nx; ++q) { G[r * nx + q] = Fi[r].d[q]; Cm[r * nx + q] = Fq[r].d[q]; }
  }
  return true;
}

// ------------------------------------------------------------------ circuit
struct Group {
  int model = 0, n_inst = 0, nt = 0, np = 0;
  std::vector<int> term, branch;
  std::vector<double> par;
  double p(int k, int i) const { return par[(size_t)k * n_inst + i]; }
};
struct Circuit {
  int n_nodes = 0, n_branch = 0, n = 0;
  std::vector<Group> groups;
  std::vector<double> pwl;
  double temp_c = 27.0, gmin = 1e-12;
};

static const int kNTerm[CEDAR_NMODELS] = {0, 2, 2, 2, 2, 2, 4, 4, 4, 2, 3};
static const int kNPar[CEDAR_NMODELS]  = {0, 2, 2, 2, 10, 10, 2, 2, 7, 4, 2};
static const int kHasBr[CEDAR_NMODELS] = {0, 0, 0, 1, 1, 0, 1, 0, 0, 0, 0};
static const int kNumModels = CEDAR_NMODELS + cedar::va::kCount;
static int model_nterm(int m) { return m < CEDAR_NMODELS ? kNTerm[m] : cedar::va::kNTerm[m - CEDAR_NMODELS]; }
static int model_npar(int m) { return m < CEDAR_NMODELS ? kNPar[m] : cedar::va::kNPar[m - CEDAR_NMODELS]; }
static int model_hasbr(int m) { return m < CEDAR_NMODELS ? kHasBr[m] : cedar::va::kHasBr[m - CEDAR_NMODELS]; }

static bool load_circuit(const cedar_ckt_desc *d, Circuit &c, std::string &err) {
  if (!d || d->n_nodes < 0 || d->n_branch < 0 || d->n_groups < 0) { err = "bad desc"; return false; }
  c.n_nodes = d->n_nodes; c.n_branch = d->n_branch; c.n = d->n_nodes + d->n_branch;
  c.temp_c = d->temp_c; c.gmin = d->gmin;
  if (d->pwl && d->n_pwl > 0) c.pwl.assign(d->pwl, d->pwl + d->n_pwl);
  for (int g = 0; g < d->n_groups; ++g) {
    const cedar_devgroup &s = d->groups[g];
    if (s.model <= 0 || s.model >= kNumModels || s.n_inst < 0) { err = "bad model"; return false; }
    Group G; G.model = s.model; G.n_inst = s.n_inst; G.nt = model_nterm(s.model); G.np = model_npar(s.model);
    if (G.nt + model_hasbr(s.model) > kMaxIdx) { err = "device with more terminal values than the oracle stages"; return false; }
    G.term.assign(s.term, s.term + (size_t)G.nt * G.n_inst);
    if (model_hasbr(s.model)) {
      if (!s.branch) { err = "missing branch"; return false; }
      G.branch.assign(s.branch, s.branch + G.n_inst);
    }
    G.par.assign(s.par, s.par + (size_t)G.np * G.n_inst);
    for (int v : G.term) if (v < -1 || v >= c.n) { err = "terminal out of range"; return false; }
    for (int v : G.branch) if (v < c.n_nodes || v >= c.n) { err = "branch out of range"; return false; }
    c.groups.push_back(std::move(G));
  }
  return true;
}

// ------------------------------------------------------------------ sources
// pwl_at_time (spectre_env.jl:43-69) with find_t_in_ts (:15-21): i = index of the
// first time point strictly greater than t (a time point equal to t belongs to
// the next segment).  ts/ys are strided views (stride 2 over (t, v) pairs).
static double pwl_at_time(const double *tv, int npts, double t) {
  // 0-based: i = first k with ts[k] > t
  int i = 0;
  while (i < npts && tv[2 * i] <= t) ++i;
  if (i <= 0) return tv[1];
  if (i >= npts) return tv[2 * (npts - 1) + 1];
  double y0 = tv[2 * (i - 1) + 1], y1 = tv[2 * i + 1];
  double t0 = tv[2 * (i - 1)], t1 = tv[2 * i];
  if (y0 == y1) return y1;
  if (t1 == t0) return (y0 + y1) / 2;
  double slope = (y1 - y0) / (t1 - t0);
  return y0 + (t - t0) * slope;
}

// Value of a V/I source at time t.  In DC analysis the `dc` parameter is used
// (VoltageSource: sim_mode === :dcop -> VS.dc, simpledevices.jl:289-290).
static double source_value(const Group &g, int i, double t, bool dc, const std::vector<double> &pwl) {
  double dcv = g.p(1, i);
  if (dc) return dcv;
  int kind = (int)g.p(2, i);
  double a[7]; for (int k = 0; k < 7; ++k) a[k] = g.p(3 + k, i);
  switch (kind) {
    case CEDAR_WAVE_DC: return dcv;
    case CEDAR_WAVE_PULSE: {  // spectre_env.jl:153-166
      double v1 = a[0], v2 = a[1], td = a[2], tr = a[3], tf = a[4], pw = a[5], per = a[6];
      double tv[8] = {td, v1, td + tr, v2, td + tr + pw, v2, td + tr + pw + tf, v1};
      double tm = std::fmod(t, per);  // rem_right_semi(t, r) = t % r
      return pwl_at_time(tv, 4, tm);
    }
    case CEDAR_WAVE_PWL: {
      int64_t off = (int64_t)a[0]; int np = (int)a[1];
      return pwl_at_time(pwl.data() + off, np, t);
    }
    case CEDAR_WAVE_SIN: {  // spectre_env.jl:169-176 (sind = sin of degrees)
      double vo = a[0], va = a[1], freq = a[2], td = a[3], theta = a[4], phase = a[5], nc = a[6];
      if (td < t && t < nc / freq) {
        double deg = 360.0 * freq * (t - td) + phase;
        return vo + va * std::exp(-(t - td) * theta) * std::sin(deg * (M_PI / 180.0));
      }
      return vo + va * std::sin(phase * (M_PI / 180.0));
    }
  }
  return dcv;
}

// Next source corner strictly after t + eps (time_periodic_singularities!,
// spectre_env.jl:71-77,160-161): pulse corners repeat every period, pwl corners
// once, sin starts at td.
static double next_breakpoint(const Circuit &c, double t, double eps) {
  double best = std::numeric_limits<double>::infinity();
  for (const Group &g : c.groups) {
    if (g.model != CEDAR_V && g.model != CEDAR_I) continue;
    for (int i = 0; i < g.n_inst; ++i) {
      int kind = (int)g.p(2, i);
      if (kind == CEDAR_WAVE_PULSE) {
        double td = g.p(5, i), tr = g.p(6, i), tf = g.p(7, i), pw = g.p(8, i), per = g.p(9, i);
        double cs[4] = {td, td + tr, td + tr + pw, td + tr + pw + tf};
        for (double cj : cs) {
          double bp;
          if (cj > t + eps) bp = cj;
          else if (std::isfinite(per) && per > 0) {
            double k = std::floor((t + eps - cj) / per) + 1.0;
            bp = cj + k * per;
            if (!(bp > t + eps)) bp = cj + (k + 1.0) * per;
          } else continue;
          best = std::min(best, bp);
        }
      } else if (kind == CEDAR_WAVE_PWL) {
        int64_t off = (int64_t)g.p(3, i); int np = (int)g.p(4, i);
        for (int k = 0; k < np; ++k) { double tk = c.pwl[off + 2 * k]; if (tk > t + eps) { best = std::min(best, tk); break; } }
      } else if (kind == CEDAR_WAVE_SIN) {
        double td = g.p(6, i);
        if (td > t + eps) best = std::min(best, td);
      }
    }
  }
  return best;
}

// ---------------------------------------------------------------- evaluation
// Dense accumulation of Fi, Fq, G = dFi/dx, C = dFq/dx at x.
struct EvalOut {
  int n;
  std::vector<double> Fi, Fq, G, C;
  explicit EvalOut(int n_) : n(n_), Fi(n_), Fq(n_), G((size_t)n_ * n_), C((size_t)n_ * n_) {}
  void clear() { std::fill(Fi.begin(), Fi.end(), 0); std::fill(Fq.begin(), Fq.end(), 0);
                 std::fill(G.begin(), G.end(), 0); std::fill(C.begin(), C.end(), 0); }
};

struct Acc {
  EvalOut &o; const int *idx; int nin;
  // add a contribution `val` to row `row` of Fi (q=false) or Fq (q=true)
  void add(int row, const Dual &val, bool q) {
    if (row < 0) return;
    if (!q) o.Fi[row] += val.v; else o.Fq[row] += val.v;
    double *M = q ? o.C.data() : o.G.data();
    for (int k = 0; k < nin; ++k) if (idx[k] >= 0) M[(size_t)row * o.n + idx[k]] += val.d[k];
  }
};

struct EvalCtx {
  double t = 0; bool dc = false; double src_scale = 1.0; double gshunt = 0.0;
  const double *xref = nullptr;  // reference point of the gshunt term (null = ground)
};

static Dual mos1_id(const Dual &vgs, const Dual &vds, double vth, double beta, double lam) {
  // Level-1 Shichman-Hodges drain current for vds >= 0 (forward mode).
  Dual vov = vgs - Dual(vth);
  if (vov.v <= 0) return Dual(0.0);
  Dual clm = Dual(1.0) + lam * vds;
  if (vds.v < vov.v) return beta * (vov - 0.5 * vds) * vds * clm;
  return (0.5 * beta) * vov * vov * clm;
}

static void eval_circuit(const Circuit &c, const double *x, const EvalCtx &ctx, EvalOut &o) {
  o.clear();
  auto X = [&](int u) { return u < 0 ? 0.0 : x[u]; };
  const double Vt = 1.380649e-23 * (c.temp_c + 273.15) / 1.602176634e-19;
  for (const Group &g : c.groups) {
    for (int i = 0; i < g.n_inst; ++i) {
      const int *tm = g.term.data() + (size_t)g.nt * i;
      int idx[kMaxIdx]; int nin = 0;
      for (int k = 0; k < g.nt; ++k) idx[nin++] = tm[k];
      int br = -1;
      if (!g.branch.empty()) { br = g.branch[i]; idx[nin++] = br; }
      Dual in[ND];   // (built-in models: at most 5 inputs)
      if (g.model < CEDAR_NMODELS)
        for (int k = 0; k < nin; ++k) in[k] = Dual::seed(X(idx[k]), idx[k] >= 0 ? k : -1);
      Acc A{o, idx, nin};
      switch (g.model) {
        case CEDAR_R: {  // I - V/res = 0; kcl!(p, -m I), kcl!(n, +m I)
          double r = g.p(0, i), m = g.p(1, i);
          Dual I = (in[0] - in[1]) / r;
          A.add(tm[0], -m * I, false); A.add(tm[1], m * I, false);
        } break;
        case CEDAR_C: {  // I - C ddt(V) = 0  -> charge C*V
          double cap = g.p(0, i), m = g.p(1, i);
          Dual Q = cap * (in[0] - in[1]);
          A.add(tm[0], -m * Q, true); A.add(tm[1], m * Q, true);
        } break;
        case CEDAR_L: {  // V - L ddt(I) = 0, branch current unknown
          double l = g.p(0, i), m = g.p(1, i);
          Dual I = in[2];
          A.add(tm[0], -m * I, false); A.add(tm[1], m * I, false);
          A.add(br, in[0] - in[1], false); A.add(br, -l * I, true);
        } break;
        case CEDAR_V: {  // V - Vab = 0
          double m = g.p(0, i);
          double vs = source_value(g, i, ctx.t, ctx.dc, c.pwl) * ctx.src_scale;
          Dual I = in[2];
          A.add(tm[0], -m * I, false); A.add(tm[1], m * I, false);
          A.add(br, in[0] - in[1] - Dual(vs), false);
        } break;
        case CEDAR_I: {  // I - Iab = 0
          double m = g.p(0, i);
          double is = source_value(g, i, ctx.t, ctx.dc, c.pwl) * ctx.src_scale;
          A.add(tm[0], Dual(-m * is), false); A.add(tm[1], Dual(m * is), false);
        } break;
        case CEDAR_E: {  // V - gain (Vc+ - Vc-) = 0
          double gain = g.p(0, i), m = g.p(1, i);
          Dual I = in[4];
          A.add(tm[0], -m * I, false); A.add(tm[1], m * I, false);
          A.add(br, (in[0] - in[1]) - gain * (in[2] - in[3]), false);
        } break;
        case CEDAR_G: {  // I - gain (Vc+ - Vc-) = 0
          double gain = g.p(0, i), m = g.p(1, i);
          Dual I = gain * (in[2] - in[3]);
          A.add(tm[0], -m * I, false); A.add(tm[1], m * I, false);
        } break;
        case CEDAR_MOS1: {
          // module mos1(d,g,s,b): vgs = type*V(g,s), vds = type*V(d,s);
          // symmetric in d/s: for vds < 0 the roles swap.
          // I(d,s) <+ type*id + $simparam("gmin")*V(d,s)
          double type = g.p(0, i), W = g.p(1, i), L = g.p(2, i), KP = g.p(3, i),
                 VTO = g.p(4, i), LAM = g.p(5, i), m = g.p(6, i);
          double beta = KP * W / L, vth = type * VTO;
          Dual vgs = type * (in[1] - in[2]);
          Dual vds = type * (in[0] - in[2]);
          Dual id;
          if (vds.v >= 0) id = mos1_id(vgs, vds, vth, beta, LAM);
          else id = -mos1_id(vgs - vds, -vds, vth, beta, LAM);
          Dual Ids = type * id + c.gmin * (in[0] - in[2]);
          A.add(tm[0], -m * Ids, false); A.add(tm[2], m * Ids, false);
        } break;
        case CEDAR_DIODE: {
          // I(a,c) <+ IS*AREA*(limexp(V(a,c)/(N*$vt)) - 1) + gmin*V(a,c)
          double IS = g.p(0, i), N = g.p(1, i), AREA = g.p(2, i), m = g.p(3, i);
          Dual v = in[0] - in[1];
          Dual I = (IS * AREA) * (dexp_lim(v / (N * Vt)) - Dual(1.0)) + c.gmin * v;
          A.add(tm[0], -m * I, false); A.add(tm[1], m * I, false);
        } break;
        case CEDAR_NLVCR: {
          // test/NLVCR.va: cdrain = R*V(g,s)**2; I(d,s) <+ V(d,s)*ddx(cdrain, V(g,s))
          // ddx over the two-node probe V(g,s) = (dc/dVg - dc/dVs)/2 (vasim.jl:400-411)
          double R = g.p(0, i), m = g.p(1, i);
          Dual vgs = in[1] - in[2];
          Dual dcd = 2.0 * R * vgs;  // (2R vgs - (-2R vgs))/2
          Dual I = (in[0] - in[2]) * dcd;
          A.add(tm[0], -m * I, false); A.add(tm[2], m * I, false);
        } break;
        default: {
          // Verilog-A model: dense residuals and partials of one device, from the
          // hand restatement of the module when there is one (every shipped
          // module), else from the emitted code (derived block = parameters, m,
          // thermal voltage) (idx / nin: the terminals, then the branch current
          // of a module with a voltage-contributed branch)
          const int k = g.model - CEDAR_NMODELS, nx = nin;
          // sized per model: compact models carry hundreds of parameters
          std::vector<double> dp(g.np + 1), v(nx), fi(nx), fq(nx), G((size_t)nx * nx), Cm((size_t)nx * nx);
          for (int q = 0; q < g.np; ++q) dp[q] = g.p(q, i);
          dp[g.np] = Vt;
          for (int q = 0; q < nx; ++q) v[q] = X(idx[q]);
          if (!va_full_restated(k, dp.data(), g.np, v.data(), nx, c.gmin, fi.data(), fq.data(), G.data(), Cm.data()))
            cedar::va::full(k, dp.data(), 1, v.data(), c.gmin, fi.data(), fq.data(), G.data(), Cm.data());
          const double m = g.p(g.np - 1, i);
          for (int r = 0; r < nx; ++r) {
            const int row = idx[r];
            if (row < 0) continue;
            o.Fi[row] += m * fi[r]; o.Fq[row] += m * fq[r];
            for (int q = 0; q < nx; ++q) {
              if (idx[q] < 0) continue;
              o.G[(size_t)row * o.n + idx[q]] += m * G[r * nx + q];
              o.C[(size_t)row * o.n + idx[q]] += m * Cm[r * nx + q];
            }
          }
        } break;
      }
    }
  }
  if (ctx.gshunt != 0.0) {
    for (int k = 0; k < c.n_nodes; ++k) {
      o.Fi[k] += -ctx.gshunt * (x[k] - (ctx.xref ? ctx.xref[k] : 0.0));
      o.G[(size_t)k * c.n + k] += -ctx.gshunt;
    }
  }
}

// ------------------------------------------------------------------ dense LU
// LU with partial pivoting (row interchanges), skipping structurally zero
// multipliers and zero pivot-row entries.  Returns false on an exactly zero pivot.
struct DenseLU {
  int n; std::vector<double> a; std::vector<int> piv; std::vector<int> nzc;
  explicit DenseLU(int n_) : n(n_), a((size_t)n_ * n_), piv(n_), nzc(n_) {}
  bool factor() {
    for (int k = 0; k < n; ++k) {
      int p = k; double best = std::fabs(a[(size_t)k * n + k]);
      for (int i = k + 1; i < n; ++i) { double v = std::fabs(a[(size_t)i * n + k]); if (v > best) { best = v; p = i; } }
      piv[k] = p;
      if (!(best > 0.0)) return false;
      if (p != k) for (int j = 0; j < n; ++j) std::swap(a[(size_t)k * n + j], a[(size_t)p * n + j]);
      double inv = 1.0 / a[(size_t)k * n + k];
      int nn = 0;
      for (int j = k + 1; j < n; ++j) if (a[(size_t)k * n + j] != 0.0) nzc[nn++] = j;
      for (int i = k + 1; i < n; ++i) {
        double &aik = a[(size_t)i * n + k];
        if (aik == 0.0) continue;
        double l = aik * inv; aik = l;
        for (int q = 0; q < nn; ++q) { int j = nzc[q]; a[(size_t)i * n + j] -= l * a[(size_t)k * n + j]; }
      }
    }
    return true;
  }
  // factor() swaps whole rows (the stored multipliers too), so P A = L U: apply
  // every swap to b first, then substitute.
  void solve(double *b) const {
    for (int k = 0; k < n; ++k) if (piv[k] != k) std::swap(b[k], b[piv[k]]);
    for (int k = 0; k < n; ++k)
      for (int i = k + 1; i < n; ++i) { double l = a[(size_t)i * n + k]; if (l != 0.0) b[i] -= l * b[k]; }
    for (int k = n - 1; k >= 0; --k) { double s = b[k];
      for (int j = k + 1; j < n; ++j) { double u = a[(size_t)k * n + j]; if (u != 0.0) s -= u * b[j]; }
      b[k] = s / a[(size_t)k * n + k]; }
  }
};

// ------------------------------------------------------------------ Newton
struct Tol { double rel, av, ai; };  // Newton tolerances (already scaled)

struct Work {
  const Circuit &c; EvalOut eo; DenseLU lu; std::vector<double> F, dx, xq;
  explicit Work(const Circuit &c_) : c(c_), eo(c_.n), lu(c_.n), F(c_.n), dx(c_.n), xq(c_.n) {}
};

// Solve Fi(x,t) + cj*Fq(x) + hist = 0.  Convergence: |dx_i| <= rel*|x_i| + abs_i for
// every unknown after the update.  DC damping limits the node-voltage update to
// `vlim` (0 = off).  Returns iterations used (>0) or -iterations on failure,
// or 0 on a zero pivot.
static int newton(Work &w, double *x, const EvalCtx &ctx, double cj, const double *hist,
                  const Tol &tol, int maxit, double vlim, int *zero_pivot) {
  const Circuit &c = w.c; const int n = c.n;
  *zero_pivot = 0;
  for (int it = 1; it <= maxit; ++it) {
    eval_circuit(c, x, ctx, w.eo);
    for (int i = 0; i < n; ++i) w.F[i] = w.eo.Fi[i] + cj * w.eo.Fq[i] + (hist ? hist[i] : 0.0);
    for (size_t k = 0; k < (size_t)n * n; ++k) w.lu.a[k] = w.eo.G[k] + cj * w.eo.C[k];
    if (!w.lu.factor()) { *zero_pivot = 1; return 0; }
    for (int i = 0; i < n; ++i) w.dx[i] = -w.F[i];
    w.lu.solve(w.dx.data());
    bool finite = true;
    for (int i = 0; i < n; ++i) if (!std::isfinite(w.dx[i])) finite = false;
    if (!finite) return -it;
    double scale = 1.0;
    if (vlim > 0) {
      double mx = 0; for (int i = 0; i < c.n_nodes; ++i) mx = std::max(mx, std::fabs(w.dx[i]));
      if (mx > vlim) scale = vlim / mx;
    }
    bool conv = (scale == 1.0);
    for (int i = 0; i < n; ++i) {
      double d = w.dx[i] * scale;
      x[i] += d;
      double lim = tol.rel * std::fabs(x[i]) + (i < c.n_nodes ? tol.av : tol.ai);
      if (!(std::fabs(d) <= lim)) conv = false;
    }
    if (conv) return it;
  }
  return -maxit;
}

static void eval_q(Work &w, const double *x, const EvalCtx &ctx, double *q) {
  eval_circuit(w.c, x, ctx, w.eo);
  for (int i = 0; i < w.c.n; ++i) q[i] = w.eo.Fq[i];
}

// DC operating point (CedarDCOp's role, src/dcop.jl:53-94): damped Newton from the
// guess; on failure pseudo-transient continuation (Kelley & Keyes, SIAM J. Numer.
// Anal. 35 (1998)); on failure source stepping lambda = 0.1 .. 1 (halving the
// increment on failure, at most 8 halvings).  At most 20000 Newton iterations.
static int dcop(Work &w, double *x, double t, const Tol &tol, int64_t *iters) {
  const int n = w.c.n; const int maxit = 100; const double vlim = 0.0;  // no damping: PTC bounds the steps
  const int64_t budget = 20000;  // total Newton iterations this DC solve may spend
  EvalCtx ctx; ctx.t = t; ctx.dc = true;
  std::vector<double> x0(x, x + n), xs(n), xr(n);
  int zp = 0;
  int64_t used = 0;
  int r = newton(w, x, ctx, 0.0, nullptr, tol, maxit, vlim, &zp);
  used += std::abs(r);
  if (r > 0) { *iters += used; return CEDAR_ST_OK; }
  // pseudo-transient continuation: node rows get -gs (x - xr), xr = last accepted
  // iterate; gs shrinks 10x after a converged level and grows 4x after a failed one.
  // Pass 0 damps node updates to 0.5 V per iteration, pass 1 does not.
  for (int pass = 0; pass < 2; ++pass) {
    const double pv = pass == 0 ? 0.5 : 0.0;
    std::copy(x0.begin(), x0.end(), xr.begin());
    double gs = 1e-2; int fails = 0; bool ptc_ok = false;
    while (used < budget && fails <= 60) {
      std::copy(xr.begin(), xr.end(), xs.begin());
      ctx.gshunt = gs; ctx.xref = xr.data();
      r = newton(w, xs.data(), ctx, 0.0, nullptr, tol, 50, pv, &zp);
      used += std::abs(r);
      if (r > 0) {
        std::copy(xs.begin(), xs.end(), xr.begin());
        if (gs <= 1e-14) { ptc_ok = true; break; }
        gs *= 0.1;
      } else { gs *= 4.0; ++fails; }
    }
    ctx.gshunt = 0.0; ctx.xref = nullptr;
    if (ptc_ok) {
      std::copy(xr.begin(), xr.end(), x);
      r = newton(w, x, ctx, 0.0, nullptr, tol, maxit, pv, &zp);
      used += std::abs(r);
      if (r > 0) { *iters += used; return CEDAR_ST_OK; }
    }
  }
  // source stepping from zero
  std::fill(x, x + n, 0.0);
  double lam = 0.0, dl = 0.1; int halv = 0; bool ok = true;
  while (lam < 1.0) {
    if (used >= budget) { ok = false; break; }
    double ln = std::min(1.0, lam + dl);
    std::copy(x, x + n, xs.begin());
    ctx.src_scale = ln;
    r = newton(w, xs.data(), ctx, 0.0, nullptr, tol, maxit, vlim, &zp);
    used += std::abs(r);
    if (r > 0) { std::copy(xs.begin(), xs.end(), x); lam = ln; halv = 0; dl = std::min(0.1, dl * 2); }
    else { dl *= 0.5; if (++halv > 8) { ok = false; break; } }
  }
  ctx.src_scale = 1.0;
  *iters += used;
  return ok ? CEDAR_ST_OK : CEDAR_ST_DCOP;
}

// ------------------------------------------------------------------ transient
static void fill_defaults(const cedar_tran_opts *in, cedar_tran_opts &o) {
  o = *in;
  double span = o.tstop - o.tstart;
  if (o.max_newton <= 0) o.max_newton = 20;
  if (o.max_steps <= 0) o.max_steps = 100000000;
  if (o.reltol <= 0) o.reltol = 1e-6;
  if (o.abstol_v <= 0) o.abstol_v = 1e-9;
  if (o.abstol_i <= 0) o.abstol_i = 1e-12;
  if (o.nr_factor <= 0) o.nr_factor = 1e-3;
  if (o.hfirst_frac <= 0) o.hfirst_frac = 1e-2;
  if (o.hmax <= 0) o.hmax = span / 50.0;
  if (o.hmin <= 0) o.hmin = span * 1e-12;
}

// Output sink: every accepted point, or uniform probe samples (quadratic
// interpolation through the last three accepted points of the current segment,
// linear when only two are available).
struct Sink {
  // all-points mode
  double *t_out = nullptr, *x_out = nullptr; int64_t cap = 0, count = 0;
  // samples mode
  const int *probes = nullptr; int np = 0; int ns = 0; double *samp = nullptr; int next = 0;
  double tstart = 0, tstop = 0;
  int n = 0;
  // accepted-step recorder (time, BDF order) for adjoint replay
  std::vector<double> *rec_t = nullptr; std::vector<signed char> *rec_ord = nullptr;
  void record(double t, int ord) { if (rec_t) { rec_t->push_back(t); rec_ord->push_back((signed char)ord); } }
  double ts(int j) const { return j == ns - 1 ? tstop : tstart + (tstop - tstart) * ((double)j / (double)(ns - 1)); }
  void point(double t, const double *x) {
    if (t_out) { if (count < cap) { t_out[count] = t; std::memcpy(x_out + (size_t)count * n, x, sizeof(double) * n); } count++; }
  }
  void start(const double *x) {
    if (samp && ns > 0) { for (int p = 0; p < np; ++p) samp[(size_t)p * ns] = probes[p] >= 0 ? x[probes[p]] : 0.0; next = 1; }
  }
  // step from (t1,x1) to (t2,x2), previous point (t0,x0) valid if have0
  void step(bool have0, double t0, const double *x0, double t1, const double *x1, double t2, const double *x2) {
    if (!samp) return;
    while (next < ns && ts(next) <= t2) {
      double t = ts(next);
      for (int p = 0; p < np; ++p) {
        int u = probes[p]; double v;
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
        samp[(size_t)p * ns + next] = v;
      }
      ++next;
    }
  }
};

// Step-size factor: the largest k/8 (k = 1..16) with k/8 <= 0.9 err^(-1/3), i.e.
// (k/8)^3 err <= 0.729; (k/8)^3 = k^3/512 is exact.  Quantising the factor makes
// CPU and GPU (whose last-ulp rounding may differ) pick identical steps.
static double step_factor(double err) {
  auto c = [](int k) { return (double)(k * k * k) / 512.0; };
  if (c(16) * err <= 0.729) return 2.0;
  if (!(c(1) * err <= 0.729)) return 0.125;
  int lo = 1, hi = 16;
  while (hi - lo > 1) { int mid = (lo + hi) / 2; if (c(mid) * err <= 0.729) lo = mid; else hi = mid; }
  return lo / 8.0;
}

// Largest ratio lte/sc over unknowns, tracked as a fraction (num/den) compared by
// cross-multiplication so that one division per step suffices.
struct MaxRatio {
  double num = 0.0, den = 1.0; bool bad = false;
  void add(double lte, double sc) {
    if (!(lte <= 1e300) || !(sc > 0.0)) { bad = true; return; }
    if (lte * den > num * sc) { num = lte; den = sc; }
  }
  double value() const { return bad ? 1e30 : num / den; }
};

static int tran(const Circuit &c, const cedar_tran_opts *opts_in, double *x, Sink &sink, cedar_stats &st,
                const double *perturb) {
  cedar_tran_opts o; fill_defaults(opts_in, o);
  const int n = c.n; const int nn = c.n_nodes;
  Work w(c);
  st = cedar_stats{}; st.hmin_seen = std::numeric_limits<double>::infinity(); st.hmax_seen = 0;
  Tol tol{o.nr_factor * o.reltol, o.nr_factor * o.abstol_v, o.nr_factor * o.abstol_i};
  if (o.dcop) {
    int s = dcop(w, x, o.tstart, tol, &st.dc_iters);
    if (s != CEDAR_ST_OK) { st.status = s; return s; }
  }
  if (perturb) for (int i = 0; i < n; ++i) x[i] += perturb[i];
  EvalCtx ctx; ctx.dc = false;
  std::vector<double> qn(n), qm1(n), qd(n), hist(n), xn(n), xm1(n), xm2(n), xp(n), qt(n);
  ctx.t = o.tstart; eval_q(w, x, ctx, qn.data());
  std::copy(x, x + n, xn.begin());
  sink.n = n; sink.tstart = o.tstart; sink.tstop = o.tstop;
  sink.point(o.tstart, x); sink.start(x);
  int zp = 0;
  if (!o.adaptive) {
    const double h = o.h;
    const int64_t N = (int64_t)std::llround((o.tstop - o.tstart) / h);
    std::fill(qd.begin(), qd.end(), 0.0);
    double tprev = o.tstart, tprev2 = o.tstart; bool have_prev = false;
    for (int64_t k = 1; k <= N; ++k) {
      double t = (k == N) ? o.tstop : o.tstart + (double)k * h;
      double hk = t - tprev;
      double cj;
      if (o.method == CEDAR_TRAP) {
        cj = 2.0 / hk;
        for (int i = 0; i < n; ++i) hist[i] = -cj * qn[i] - qd[i];
      } else if (k == 1) {
        cj = 1.0 / hk;
        for (int i = 0; i < n; ++i) hist[i] = -qn[i] * cj;
      } else {
        cj = 1.5 / hk;
        double r2h = 0.5 / hk;
        for (int i = 0; i < n; ++i) hist[i] = (-4.0 * qn[i] + qm1[i]) * r2h;
      }
      if (k == 1) std::copy(xn.begin(), xn.end(), xp.begin());
      else for (int i = 0; i < n; ++i) xp[i] = 2.0 * xn[i] - xm1[i];
      ctx.t = t;
      int r = newton(w, xp.data(), ctx, cj, hist.data(), tol, o.max_newton, 0.0, &zp);
      st.newton_iters += std::abs(r);
      if (r <= 0) { st.status = zp ? CEDAR_ST_ZERO_PIVOT : CEDAR_ST_NEWTON; std::copy(xn.begin(), xn.end(), x); return st.status; }
      eval_q(w, xp.data(), ctx, qt.data());
      if (o.method == CEDAR_TRAP) for (int i = 0; i < n; ++i) qd[i] = cj * qt[i] + hist[i];
      qm1 = qn; qn = qt;
      sink.step(have_prev, tprev2, xm1.data(), tprev, xn.data(), t, xp.data());
      xm1 = xn; xn = xp; tprev2 = tprev; tprev = t; have_prev = true;
      st.accepted++; st.hmin_seen = std::min(st.hmin_seen, hk); st.hmax_seen = std::max(st.hmax_seen, hk);
      sink.point(t, xn.data());
      sink.record(t, o.method == CEDAR_TRAP ? 3 : (k == 1 ? 1 : 2));
      for (int i = 0; i < n; ++i) if (!std::isfinite(xn[i])) { st.status = CEDAR_ST_NAN; std::copy(xn.begin(), xn.end(), x); return st.status; }
    }
    std::copy(xn.begin(), xn.end(), x);
    st.status = CEDAR_ST_OK;
    return CEDAR_ST_OK;
  }

  // ---- adaptive variable-step BDF2 ----
  const double span = o.tstop - o.tstart;
  const double eps_bp = span * 1e-12;
  double t = o.tstart;
  double tn1 = t, tn2 = t;   // t_{n-1}, t_{n-2}
  int npts = 1;              // accepted points in the current segment (incl. t_n)
  auto restart_h = [&](double tt) {
    double nb = std::min(next_breakpoint(c, tt, eps_bp), o.tstop);
    double hf = o.hfirst_frac * std::min(nb - tt, o.hmax);
    if (o.h > 0) hf = std::min(hf, o.h);
    return hf;
  };
  double hnext = restart_h(t);
  int64_t nsteps = 0;
  while (t < o.tstop) {
    if (++nsteps > o.max_steps) { st.status = CEDAR_ST_MAX_STEPS; break; }
    double tb = std::min(next_breakpoint(c, t, eps_bp), o.tstop);
    double h = std::min(hnext, o.hmax);
    bool hit = false;
    if (tb - t <= 1.1 * h) { h = tb - t; hit = true; }
    double tnew = hit ? tb : t + h;
    h = tnew - t;
    int order = npts >= 2 ? 2 : 1;
    double cj, h1 = t - tn1;
    if (order == 1) {
      cj = 1.0 / h;
      for (int i = 0; i < n; ++i) hist[i] = -qn[i] * cj;
    } else {
      double wr = h / h1, rh = 1.0 / h;
      cj = (1.0 + 2.0 * wr) / ((1.0 + wr) * h);
      double a1 = -(1.0 + wr), a2 = wr * wr / (1.0 + wr);
      for (int i = 0; i < n; ++i) hist[i] = (a1 * qn[i] + a2 * qm1[i]) * rh;
    }
    if (npts >= 2) { double r = h / h1; for (int i = 0; i < n; ++i) xp[i] = xn[i] + r * (xn[i] - xm1[i]); }
    else std::copy(xn.begin(), xn.end(), xp.begin());
    ctx.t = tnew;
    int r = newton(w, xp.data(), ctx, cj, hist.data(), tol, o.max_newton, 0.0, &zp);
    st.newton_iters += std::abs(r);
    if (r <= 0) {
      st.rejected++;
      hnext = h * 0.125;
      if (hnext < o.hmin) { st.status = zp ? CEDAR_ST_ZERO_PIVOT : CEDAR_ST_DT_UNDERFLOW; break; }
      continue;
    }
    double err = 0.0;
    if (npts >= 3) {
      // third divided difference over (tnew, t, tn1, tn2); the BDF2 local error is
      // x^(3) h^2 (h+h1)^2 / (6 (2h+h1)) with x^(3) ~ 6 dd3
      double h2 = tn1 - tn2;
      double rh = 1.0 / h, rh1 = 1.0 / h1, rh2 = 1.0 / h2;
      double ra = 1.0 / (h + h1), rb = 1.0 / (h1 + h2), rc = 1.0 / (h + h1 + h2);
      double coef = h * h * (h + h1) * (h + h1) / (2.0 * h + h1);
      MaxRatio mr;
      for (int i = 0; i < nn; ++i) {
        double d10 = (xp[i] - xn[i]) * rh;
        double d21 = (xn[i] - xm1[i]) * rh1;
        double d32 = (xm1[i] - xm2[i]) * rh2;
        double dd3 = ((d10 - d21) * ra - (d21 - d32) * rb) * rc;
        double lte = std::fabs(dd3) * coef;
        double sc = o.reltol * std::max(std::fabs(xp[i]), std::fabs(xn[i])) + o.abstol_v;
        mr.add(lte, sc);
      }
      err = mr.value();
    } else if (npts == 2) {
      // second step after a (re)start: backward-Euler-type bound h^2 |x''| / 2 with
      // x'' ~ 2 * second divided difference over (tnew, t, tn1)
      double rh = 1.0 / h, rh1 = 1.0 / h1, ra = 1.0 / (h + h1), hh = h * h;
      MaxRatio mr;
      for (int i = 0; i < nn; ++i) {
        double dd2 = ((xp[i] - xn[i]) * rh - (xn[i] - xm1[i]) * rh1) * ra;
        double lte = std::fabs(dd2) * hh;
        double sc = o.reltol * std::max(std::fabs(xp[i]), std::fabs(xn[i])) + o.abstol_v;
        mr.add(lte, sc);
      }
      err = mr.value();
    }
    if (!std::isfinite(err)) err = 1e30;
    if (err > 1.0) {
      st.rejected++;
      hnext = h * step_factor(err);
      if (hnext < o.hmin) { st.status = CEDAR_ST_DT_UNDERFLOW; break; }
      continue;
    }
    // accept
    eval_q(w, xp.data(), ctx, qt.data());
    qm1 = qn; qn = qt;
    sink.step(npts >= 2, tn1, xm1.data(), t, xn.data(), tnew, xp.data());
    xm2 = xm1; xm1 = xn; xn = xp;
    tn2 = tn1; tn1 = t; t = tnew;
    st.accepted++; st.hmin_seen = std::min(st.hmin_seen, h); st.hmax_seen = std::max(st.hmax_seen, h);
    sink.point(t, xn.data());
    sink.record(t, order);
    bool finite = true; for (int i = 0; i < n; ++i) if (!std::isfinite(xn[i])) finite = false;
    if (!finite) { st.status = CEDAR_ST_NAN; break; }
    if (npts < 3) ++npts;
    double fac = (err > 0.0) ? step_factor(err) : 1.0;
    hnext = h * fac;
    if (hit && t < o.tstop) { npts = 1; hnext = restart_h(t); }
  }
  std::copy(xn.begin(), xn.end(), x);
  if (st.status == CEDAR_ST_OK && t < o.tstop) st.status = CEDAR_ST_MAX_STEPS;
  return st.status;
}

// ------------------------------------------------------------------ adjoint
// Discrete adjoint of the BDF2/BE step sequence (test/sensitivity.jl:13-42 is the
// reference's differentiation path, forward mode through SciMLSensitivity; this
// restates the gradient of the discrete solution, treating the accepted step
// sequence as fixed and each step's Newton solution as exact).
//   R_0(x_0) = Fi_dc(x_0) = 0                                   (DC operating point)
//   R_n = Fi(x_n, t_n) + cj_n Fq(x_n) + b1_n Fq(x_{n-1}) + b2_n Fq(x_{n-2}) = 0
//   J_n^T lam_n = -(dPhi/dx_n + b1_{n+1} C(x_n)^T lam_{n+1} + b2_{n+2} C(x_n)^T lam_{n+2})
//   dPhi/dp = sum_n lam_n^T dR_n/dp            (p: MOS1 widths W, resistor values r)
struct StepSeq { std::vector<double> T; std::vector<signed char> ord; };  // T[0] = tstart

static void step_coef(const StepSeq &S, size_t n, double &cj, double &b1, double &b2, double &rh, double &a1, double &a2) {
  double h = S.T[n] - S.T[n - 1];
  if (S.ord[n] != 2) { cj = 1.0 / h; b1 = -cj; b2 = 0.0; rh = 0; a1 = 0; a2 = 0; return; }
  double h1 = S.T[n - 1] - S.T[n - 2];
  double wr = h / h1;
  rh = 1.0 / h;
  cj = (1.0 + 2.0 * wr) / ((1.0 + wr) * h);
  a1 = -(1.0 + wr); a2 = wr * wr / (1.0 + wr);
  b1 = a1 * rh; b2 = a2 * rh;
}

// Replay the recorded steps (DC operating point first); X[n*nv + u] = x_n.
static int replay(const Circuit &c, const cedar_tran_opts &o, const StepSeq &S, std::vector<double> &X,
                  const double *perturb, int64_t *iters) {
  const int n = c.n; const size_t N = S.T.size() - 1;
  Work w(c);
  Tol tol{o.nr_factor * o.reltol, o.nr_factor * o.abstol_v, o.nr_factor * o.abstol_i};
  std::vector<double> x(n, 0.0), qn(n), qm1(n), hist(n), xp(n), qt(n);
  int64_t dci = 0;
  if (o.dcop) { int s = dcop(w, x.data(), o.tstart, tol, &dci); if (s != CEDAR_ST_OK) return s; }
  if (perturb) for (int i = 0; i < n; ++i) x[i] += perturb[i];
  X.assign((N + 1) * n, 0.0);
  std::copy(x.begin(), x.end(), X.begin());
  EvalCtx ctx; ctx.t = o.tstart;
  eval_q(w, x.data(), ctx, qn.data());
  int zp = 0;
  for (size_t k = 1; k <= N; ++k) {
    double cj, b1, b2, rh, a1, a2;
    step_coef(S, k, cj, b1, b2, rh, a1, a2);
    const double *xn = &X[(k - 1) * n];
    if (S.ord[k] != 2) for (int i = 0; i < n; ++i) hist[i] = -qn[i] * cj;
    else for (int i = 0; i < n; ++i) hist[i] = (a1 * qn[i] + a2 * qm1[i]) * rh;
    if (S.ord[k] == 2) {
      const double *xm1 = &X[(k - 2) * n];
      double r = (S.T[k] - S.T[k - 1]) / (S.T[k - 1] - S.T[k - 2]);
      for (int i = 0; i < n; ++i) xp[i] = xn[i] + r * (xn[i] - xm1[i]);
    } else std::copy(xn, xn + n, xp.begin());
    ctx.t = S.T[k];
    int r = newton(w, xp.data(), ctx, cj, hist.data(), tol, o.max_newton, 0.0, &zp);
    if (iters) *iters += std::abs(r);
    if (r <= 0) return zp ? CEDAR_ST_ZERO_PIVOT : CEDAR_ST_NEWTON;
    std::copy(xp.begin(), xp.end(), X.begin() + k * n);
    eval_q(w, xp.data(), ctx, qt.data());
    qm1 = qn; qn = qt;
  }
  return CEDAR_ST_OK;
}

struct ObjVal { double phi; long k50; double t50; };

static ObjVal objective(const cedar_objective &ob, double tstar, const StepSeq &S, const std::vector<double> &X, int n) {
  const size_t N = S.T.size() - 1;
  auto P = [&](size_t k) { return -X[k * n + ob.vnode] * X[k * n + ob.ibranch]; };
  double E = 0;
  for (size_t k = 1; k <= N; ++k) E += (S.T[k] - S.T[k - 1]) * (P(k) + P(k - 1)) / 2.0;
  ObjVal v{0, -1, 0};
  for (size_t k = 1; k <= N; ++k) {
    double v0 = X[(k - 1) * n + ob.probe], v1 = X[k * n + ob.probe];
    double a = v0 - ob.level, b = v1 - ob.level;
    if ((a < 0 && b >= 0) || (a > 0 && b <= 0)) {
      v.k50 = (long)k;
      v.t50 = S.T[k - 1] + (ob.level - v0) * (S.T[k] - S.T[k - 1]) / (v1 - v0);
      break;
    }
  }
  double D = v.k50 > 0 ? (v.t50 - tstar) * (v.t50 - tstar) : 0.0;
  v.phi = ob.w_energy * E + ob.w_delay * D + ob.w_final * X[N * n + ob.probe];
  return v;
}

static int n_params(const Circuit &c) {
  int np = 0;
  for (const Group &g : c.groups) if (g.model == CEDAR_MOS1 || g.model == CEDAR_R) np += g.n_inst;
  return np;
}

// grad += lam^T dFi/dp at x (MOS1: d/dW of m*Ids; R: d/dr of m*V/r)
static void accumulate_dp(const Circuit &c, const double *x, const double *lam, double *grad) {
  auto X = [&](int u) { return u < 0 ? 0.0 : x[u]; };
  auto L = [&](int u) { return u < 0 ? 0.0 : lam[u]; };
  int k = 0;
  for (const Group &g : c.groups) {
    if (g.model != CEDAR_MOS1 && g.model != CEDAR_R) continue;
    for (int i = 0; i < g.n_inst; ++i, ++k) {
      const int *tm = g.term.data() + (size_t)g.nt * i;
      if (g.model == CEDAR_MOS1) {
        double type = g.p(0, i), W = g.p(1, i), Lc = g.p(2, i), KP = g.p(3, i), VTO = g.p(4, i), LAM = g.p(5, i), m = g.p(6, i);
        double beta = KP * W / Lc, vth = type * VTO;
        Dual vgs = Dual(type * (X(tm[1]) - X(tm[2]))), vds = Dual(type * (X(tm[0]) - X(tm[2])));
        double id = vds.v >= 0 ? mos1_id(vgs, vds, vth, beta, LAM).v : -mos1_id(vgs - vds, -vds, vth, beta, LAM).v;
        double dI = m * type * id / W;  // d(m Ids)/dW; KCL(d) gets -m Ids, KCL(s) +m Ids
        grad[k] += -dI * L(tm[0]) + dI * L(tm[2]);
      } else {
        double r = g.p(0, i), m = g.p(1, i);
        double V = X(tm[0]) - X(tm[1]);
        double dI = -m * V / (r * r);  // d(m V/r)/dr
        grad[k] += -dI * L(tm[0]) + dI * L(tm[1]);
      }
    }
  }
}

static int adjoint(const Circuit &c, const cedar_tran_opts &o, const StepSeq &S, const cedar_objective &ob, double tstar,
                   const double *perturb, double *phi, double *grad) {
  const int n = c.n; const size_t N = S.T.size() - 1;
  std::vector<double> X;
  int s = replay(c, o, S, X, perturb, nullptr);
  if (s != CEDAR_ST_OK) return s;
  ObjVal v = objective(ob, tstar, S, X, n);
  if (phi) *phi = v.phi;
  const int np = n_params(c);
  std::fill(grad, grad + np, 0.0);
  // dPhi/dx_k
  std::vector<double> g((N + 1) * n, 0.0);
  for (size_t k = 0; k <= N; ++k) {
    double hk = k >= 1 ? S.T[k] - S.T[k - 1] : 0.0, hk1 = k + 1 <= N ? S.T[k + 1] - S.T[k] : 0.0;
    double ck = ob.w_energy * (hk + hk1) / 2.0;
    g[k * n + ob.vnode] += ck * (-X[k * n + ob.ibranch]);
    g[k * n + ob.ibranch] += ck * (-X[k * n + ob.vnode]);
  }
  if (v.k50 > 0 && ob.w_delay != 0.0) {
    size_t k = (size_t)v.k50;
    double v0 = X[(k - 1) * n + ob.probe], v1 = X[k * n + ob.probe];
    double a = ob.level - v0, d = v1 - v0, D = S.T[k] - S.T[k - 1];
    double dD = ob.w_delay * 2.0 * (v.t50 - tstar);
    g[(k - 1) * n + ob.probe] += dD * D * (a - d) / (d * d);
    g[k * n + ob.probe] += dD * (-D * a) / (d * d);
  }
  g[N * n + ob.probe] += ob.w_final;
  // backward sweep
  Work w(c);
  std::vector<double> lam((N + 1) * n, 0.0), rhs(n), Ct(n);
  DenseLU lu(n);
  for (long k = (long)N; k >= 0; --k) {
    const double *xk = &X[(size_t)k * n];
    EvalCtx ctx; ctx.t = k > 0 ? S.T[k] : o.tstart; ctx.dc = (k == 0);
    eval_circuit(c, xk, ctx, w.eo);
    for (int i = 0; i < n; ++i) rhs[i] = -g[(size_t)k * n + i];
    for (int step = 1; step <= 2; ++step) {
      size_t m = (size_t)k + step;
      if (m > N) break;
      double cj, b1, b2, rh, a1, a2;
      step_coef(S, m, cj, b1, b2, rh, a1, a2);
      double b = step == 1 ? b1 : b2;
      if (b == 0.0) continue;
      const double *lm = &lam[m * n];
      for (int u = 0; u < n; ++u) { double acc = 0; for (int e = 0; e < n; ++e) acc += w.eo.C[(size_t)e * n + u] * lm[e]; Ct[u] = acc; }
      for (int u = 0; u < n; ++u) rhs[u] -= b * Ct[u];
    }
    double cjk = 0.0, b1, b2, rh, a1, a2;
    if (k > 0) step_coef(S, (size_t)k, cjk, b1, b2, rh, a1, a2);
    // J^T
    for (int e = 0; e < n; ++e) for (int u = 0; u < n; ++u)
      lu.a[(size_t)u * n + e] = w.eo.G[(size_t)e * n + u] + cjk * w.eo.C[(size_t)e * n + u];
    if (!lu.factor()) return CEDAR_ST_ZERO_PIVOT;
    lu.solve(rhs.data());
    std::copy(rhs.begin(), rhs.end(), lam.begin() + (size_t)k * n);
    accumulate_dp(c, xk, rhs.data(), grad);
  }
  return CEDAR_ST_OK;
}

static thread_local std::string g_err;

}  // namespace orc

using namespace orc;

extern "C" {

int oracle_last_error(char *buf, size_t len) {
  if (buf && len) { std::snprintf(buf, len, "%s", g_err.c_str()); }
  return (int)g_err.size();
}

// F = Fi + C*xdot (xdot may be NULL); dense G, C (row-major n*n, may be NULL).
int oracle_eval(const cedar_ckt_desc *d, const double *x, const double *xdot, double t, int dc,
                double *F, double *Fi, double *Fq, double *G, double *C) {
  Circuit c; if (!load_circuit(d, c, g_err)) return CEDAR_EINVAL;
  EvalOut o(c.n); EvalCtx ctx; ctx.t = t; ctx.dc = dc != 0;
  eval_circuit(c, x, ctx, o);
  const int n = c.n;
  if (F) for (int i = 0; i < n; ++i) { double s = o.Fi[i]; if (xdot) for (int j = 0; j < n; ++j) s += o.C[(size_t)i * n + j] * xdot[j]; F[i] = s; }
  if (Fi) std::memcpy(Fi, o.Fi.data(), sizeof(double) * n);
  if (Fq) std::memcpy(Fq, o.Fq.data(), sizeof(double) * n);
  if (G) std::memcpy(G, o.G.data(), sizeof(double) * n * n);
  if (C) std::memcpy(C, o.C.data(), sizeof(double) * n * n);
  return 0;
}

int oracle_dcop(const cedar_ckt_desc *d, const cedar_tran_opts *opts, double t, double *x, cedar_stats *st) {
  Circuit c; if (!load_circuit(d, c, g_err)) return CEDAR_EINVAL;
  cedar_tran_opts o; fill_defaults(opts, o);
  Tol tol{o.nr_factor * o.reltol, o.nr_factor * o.abstol_v, o.nr_factor * o.abstol_i};
  Work w(c); cedar_stats s{}; s.status = dcop(w, x, t, tol, &s.dc_iters);
  if (st) *st = s;
  return s.status == CEDAR_ST_OK ? 0 : CEDAR_ENOCONV;
}

int oracle_newton(const cedar_ckt_desc *d, const cedar_tran_opts *opts, double t, double cj,
                  const double *hist, double *x, cedar_stats *st) {
  Circuit c; if (!load_circuit(d, c, g_err)) return CEDAR_EINVAL;
  cedar_tran_opts o; fill_defaults(opts, o);
  Tol tol{o.nr_factor * o.reltol, o.nr_factor * o.abstol_v, o.nr_factor * o.abstol_i};
  Work w(c); EvalCtx ctx; ctx.t = t; int zp = 0;
  int r = newton(w, x, ctx, cj, hist, tol, o.max_newton, 0.0, &zp);
  if (st) { *st = cedar_stats{}; st->newton_iters = std::abs(r); st->status = r > 0 ? 0 : (zp ? CEDAR_ST_ZERO_PIVOT : CEDAR_ST_NEWTON); }
  return r > 0 ? 0 : CEDAR_ENOCONV;
}

int oracle_tran(const cedar_ckt_desc *d, const cedar_tran_opts *opts, double *x,
                double *t_out, double *x_out, int64_t cap, int64_t *n_out, cedar_stats *st) {
  Circuit c; if (!load_circuit(d, c, g_err)) return CEDAR_EINVAL;
  Sink sink; sink.t_out = t_out; sink.x_out = x_out; sink.cap = cap;
  cedar_stats s{};
  tran(c, opts, x, sink, s, nullptr);
  if (n_out) *n_out = sink.count;
  if (st) *st = s;
  if (t_out && sink.count > cap) return CEDAR_ECAPACITY;
  return 0;
}


// Forward adaptive (or fixed BDF2) run that records the accepted steps, then the
// discrete adjoint along them with the Newton tolerance of `replay_opts`.
// grad: one entry per MOS1 (W) and R (r) device in group order.  The recorded
// steps are returned through t_rec/ord (capacity cap, count *nrec).
int oracle_adjoint(const cedar_ckt_desc *d, const cedar_tran_opts *fwd_opts, const cedar_tran_opts *replay_opts,
                   const cedar_objective *ob, double tstar, const double *perturb, double *phi, double *grad,
                   double *t_rec, signed char *ord_rec, int64_t cap, int64_t *nrec) {
  Circuit c; if (!load_circuit(d, c, g_err)) return CEDAR_EINVAL;
  std::vector<double> x(c.n, 0.0);
  Sink sink; StepSeq S; S.T.push_back(fwd_opts->tstart); S.ord.push_back(0);
  std::vector<double> rt; std::vector<signed char> ro;
  sink.rec_t = &rt; sink.rec_ord = &ro;
  cedar_stats st{};
  tran(c, fwd_opts, x.data(), sink, st, perturb);
  if (st.status != CEDAR_ST_OK) { g_err = "forward run failed"; return CEDAR_ENOCONV; }
  for (size_t k = 0; k < rt.size(); ++k) { S.T.push_back(rt[k]); S.ord.push_back(ro[k]); }
  if (nrec) *nrec = (int64_t)rt.size();
  if (t_rec) for (size_t k = 0; k < rt.size() && (int64_t)k < cap; ++k) { t_rec[k] = rt[k]; ord_rec[k] = ro[k]; }
  cedar_tran_opts o; fill_defaults(replay_opts, o);
  int s = adjoint(c, o, S, *ob, tstar, perturb, phi, grad);
  if (s != CEDAR_ST_OK) { g_err = "adjoint failed"; return CEDAR_ENOCONV; }
  return 0;
}

// Phi along a recorded step sequence (used for central finite differences with
// the step sequence held fixed).
int oracle_replay_phi(const cedar_ckt_desc *d, const cedar_tran_opts *replay_opts, const double *t_rec,
                      const signed char *ord_rec, int64_t nrec, const cedar_objective *ob, double tstar,
                      const double *perturb, double *phi) {
  Circuit c; if (!load_circuit(d, c, g_err)) return CEDAR_EINVAL;
  cedar_tran_opts o; fill_defaults(replay_opts, o);
  StepSeq S; S.T.push_back(o.tstart); S.ord.push_back(0);
  for (int64_t k = 0; k < nrec; ++k) { S.T.push_back(t_rec[k]); S.ord.push_back(ord_rec[k]); }
  std::vector<double> X;
  int s = replay(c, o, S, X, perturb, nullptr);
  if (s != CEDAR_ST_OK) { g_err = "replay failed"; return CEDAR_ENOCONV; }
  *phi = objective(*ob, tstar, S, X, c.n).phi;
  return 0;
}

int oracle_n_params(const cedar_ckt_desc *d) {
  Circuit c; if (!load_circuit(d, c, g_err)) return -1;
  return n_params(c);
}

// One Verilog-A device through the emitted code: dp = parameters, m, thermal
// voltage (stride 1); dense fi/fq[nt], G/C[nt*nt] (unscaled by m).
int oracle_va_full(int k, const double *dp, const double *v, double gmin, double *fi, double *fq, double *G,
                   double *Cm) {
  if (k < 0 || k >= cedar::va::kCount) { g_err = "Verilog-A model index out of range"; return -1; }
  cedar::va::full(k, dp, 1, v, gmin, fi, fq, G, Cm);
  return 0;
}

// The same device through the hand restatement; returns 1 when model k is
// restated by hand (then fi/fq/G/C are filled), 0 when it is not.
int oracle_va_ref_full(int k, const double *dp, int np, const double *v, double gmin, double *fi, double *fq,
                       double *G, double *Cm) {
  if (k < 0 || k >= cedar::va::kCount) { g_err = "Verilog-A model index out of range"; return -1; }
  return va_full_restated(k, dp, np, v, cedar::va::kNTerm[k] + cedar::va::kHasBr[k], gmin, fi, fq, G, Cm) ? 1 : 0;
}

// Powers and frequency exponents of a Verilog-A device's noise sources through
// the emitted code (dp, v as oracle_va_full); returns the number of sources.
int oracle_va_noise(int k, const double *dp, const double *v, double gmin, double *pw, double *ex) {
  if (k < 0 || k >= cedar::va::kCount) { g_err = "Verilog-A model index out of range"; return -1; }
  return cedar::va::noise(k, dp, 1, v, gmin, pw, ex);
}

// SimpleDiode (src/simpledevices.jl:134-271), restated line by line with its
// defects, at one junction voltage Vd.  PARITY UNPINNED: no reference test
// solves a circuit with it (test/basic.jl:456-468 only constructs it), and the
// reference's own behaviour at run time is what this restates:
//   q = -1.602176634e-19 (sign flipped, :222), T = 300 K, AREAeff = AREA * M (:226);
//   the breakdown branch reads the undefined NVt (:238) and the forward
//   depletion branch the undefined MJI (:260): the reference throws
//   UndefVarError there, returned here as codes 1 and 2;
//   a negative argument of Base.sqrt (:249,251) throws DomainError (code 3);
//   the `else -BVeff < Vd` line (:252) is an expression with no effect;
//   Cdiffuse = TT * ddt(Ideff) / ddt(Vd) (:256) is a ratio of time
//   derivatives: in DC both are 0 and it is TT * 0 / 0 (NaN); outside DC it is
//   left to the caller (out[3] = TT, the factor of that ratio).
// p: AREA BV BVJ CJO EG FC IBV IS KF M N RS TNOM TT VJ XTI (the struct's field
// order, :135-150).  out: Id (after the gmin term), Ideff, Cdeplete_bw +
// Cdeplete_sw, TT, Cdiffuse in DC.  Returns 0 or the error code.
int oracle_simple_diode(const double *p, double Vd, double *out) {
  const double AREA = p[0], BV = p[1], CJO = p[3], IBV = p[6], IS = p[7], M = p[9], N = p[10], TT = p[13],
               VJ = p[14], FC = p[5];
  const double MJ = M;
  const double CJ0 = CJO;
  const double GMIN = 1e-12, PJ = 0.0, PHP = 1.0, FCS = 0.5, JSW = 0.0, MJSW = 1.0 / 3.0;
  const double IKF = INFINITY, IK = IKF, IKR = INFINITY;
  const double q = -1.602176634e-19, k = 1.380649e-23, T = 300.0;
  const double AREAeff = AREA * M, PJeff = PJ * M;
  const double ISeff = IS * AREAeff + JSW * PJeff;
  double IBVeff = IBV * AREAeff;
  const double IKeff = IK * AREAeff, IKReff = IKR * AREAeff;
  const double CJeff = CJ0 * AREAeff;
  const double NkT = N * k * T;
  const double Ibdwn = ISeff * expm1(-q * BV / NkT);
  double BVeff;
  if (IBVeff < Ibdwn) { IBVeff = Ibdwn; BVeff = BV; }
  else return 1;                                   // BV - NVt * ln(IBVeff / Ibdwn): NVt undefined
  double Id;
  if (Vd >= -3 * NkT / q) Id = ISeff * expm1(q * Vd / NkT);
  else if (-BVeff < Vd) { const double r = 3 * NkT / (q * Vd * M_E); Id = -ISeff * (1 + r * r * r); }
  else Id = -ISeff * exp(-q * (BVeff + Vd) / NkT);
  Id += Vd * GMIN;
  double Ideff;
  const double ratio = (Vd >= -3 * N * k * T / q) ? Id / IKeff : Id / IKReff;
  if (ratio < 0) return 3;                         // Base.sqrt of a negative number
  Ideff = Id / (1 + sqrt(ratio));
  if (!(Vd < FC * VJ)) return 2;                   // CJeff * (1 - FC * (1 + MJI) + ...): MJI undefined
  const double Cbw = CJeff * pow(1 - Vd / VJ, -MJ);
  const double Csw = (Vd < FCS * PHP) ? CJeff * pow(1 - Vd / PHP, -MJSW)
                                      : CJeff * (1 - FCS * (1 + MJSW) + MJSW * Vd / PHP) / pow(1 - FCS, 1 + MJSW);
  out[0] = Id;
  out[1] = Ideff;
  out[2] = Cbw + Csw;
  out[3] = TT;
  out[4] = TT * 0.0 / 0.0;
  return 0;
}

double oracle_next_breakpoint(const cedar_ckt_desc *d, double t, double eps) {
  Circuit c; if (!load_circuit(d, c, g_err)) return -1;
  return next_breakpoint(c, t, eps);
}

double oracle_source_value(const cedar_ckt_desc *d, int group, int inst, double t, int dc) {
  Circuit c; if (!load_circuit(d, c, g_err)) return NAN;
  return source_value(c.groups[group], inst, t, dc != 0, c.pwl);
}

// Batched Monte Carlo / sweep: each instance = template with its parameter block,
// DC op (if opts->dcop) + perturbation + transient; OpenMP over instances.
// inst_range: [i0, i1) subset (for bounded CPU baselines).  nthreads <= 0: all.
int oracle_batch(const cedar_batch_desc *b, const cedar_tran_opts *opts, int32_t i0, int32_t i1,
                 int32_t n_max, double *x_final, double *samples, cedar_stats *stats, int nthreads) {
  if (!b || i0 < 0 || i1 > b->n_inst || i0 > i1) { g_err = "bad batch range"; return CEDAR_EINVAL; }
  std::vector<Circuit> tmpl(b->n_templates);
  for (int k = 0; k < b->n_templates; ++k) if (!load_circuit(&b->templates[k], tmpl[k], g_err)) return CEDAR_EINVAL;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
  int rc_all = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int i = i0; i < i1; ++i) {
    int k = b->inst_template[i];
    Circuit c = tmpl[k];
    if (b->inst_par_off && b->inst_par_off[i] >= 0) {
      const double *p = b->inst_par + b->inst_par_off[i];
      for (Group &g : c.groups) { std::copy(p, p + g.par.size(), g.par.begin()); p += g.par.size(); }
    }
    std::vector<double> x(c.n, 0.0);
    if (b->inst_x0_off && b->inst_x0_off[i] >= 0) std::copy(b->inst_x0 + b->inst_x0_off[i], b->inst_x0 + b->inst_x0_off[i] + c.n, x.begin());
    const double *dx = (b->inst_dx_off && b->inst_dx_off[i] >= 0) ? b->inst_dx + b->inst_dx_off[i] : nullptr;
    Sink sink;
    sink.np = b->n_probes; sink.ns = b->n_samples;
    sink.probes = b->probes ? b->probes + (size_t)k * b->n_probes : nullptr;
    if (samples && b->n_samples > 0 && b->n_probes > 0) sink.samp = samples + (size_t)(i - i0) * b->n_probes * b->n_samples;
    cedar_stats s{};
    tran(c, opts, x.data(), sink, s, dx);
    if (x_final) { double *xf = x_final + (size_t)(i - i0) * n_max; for (int u = 0; u < n_max; ++u) xf[u] = u < c.n ? x[u] : 0.0; }
    if (stats) stats[i - i0] = s;
  }
  return rc_all;
}

// Adjoint over a range of batch instances with OpenMP (the CPU baseline of the
// GPU adjoint): forward run recording its steps, then the adjoint along them with
// the same options.  obj[n_templates], tstar[n_inst]; phi[i1 - i0],
// grad[(i1 - i0) * np_max]; status[i1 - i0] (0 or the forward's status).
int oracle_adjoint_batch(const cedar_batch_desc *b, const cedar_tran_opts *opts, const cedar_objective *obj,
                         const double *tstar, int32_t i0, int32_t i1, int32_t np_max, double *phi, double *grad,
                         int32_t *status, int nthreads) {
  if (!b || i0 < 0 || i1 > b->n_inst || i0 > i1) { g_err = "bad batch range"; return CEDAR_EINVAL; }
  std::vector<Circuit> tmpl(b->n_templates);
  for (int k = 0; k < b->n_templates; ++k) if (!load_circuit(&b->templates[k], tmpl[k], g_err)) return CEDAR_EINVAL;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int i = i0; i < i1; ++i) {
    const int k = b->inst_template[i];
    Circuit c = tmpl[k];
    if (b->inst_par_off && b->inst_par_off[i] >= 0) {
      const double *p = b->inst_par + b->inst_par_off[i];
      for (Group &g : c.groups) { std::copy(p, p + g.par.size(), g.par.begin()); p += g.par.size(); }
    }
    std::vector<double> x(c.n, 0.0), rt;
    std::vector<signed char> ro;
    Sink sink; sink.rec_t = &rt; sink.rec_ord = &ro;
    cedar_stats st{};
    tran(c, opts, x.data(), sink, st, nullptr);
    double *g = grad + (size_t)(i - i0) * np_max;
    std::fill(g, g + np_max, 0.0);
    int s = st.status;
    if (s == CEDAR_ST_OK) {
      StepSeq S; S.T.push_back(opts->tstart); S.ord.push_back(0);
      for (size_t q = 0; q < rt.size(); ++q) { S.T.push_back(rt[q]); S.ord.push_back(ro[q]); }
      cedar_tran_opts o; fill_defaults(opts, o);
      std::vector<double> gi(std::max(n_params(c), 1), 0.0);
      double ph = 0.0;
      s = adjoint(c, o, S, obj[k], tstar ? tstar[i] : 0.0, nullptr, &ph, gi.data());
      phi[i - i0] = ph;
      for (int q = 0; q < n_params(c) && q < np_max; ++q) g[q] = gi[q];
    }
    if (status) status[i - i0] = s;
  }
  return 0;
}

}  // extern "C"
