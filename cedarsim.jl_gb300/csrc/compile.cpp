// compile.cpp — host-side circuit compiler (see compile.h).
//
// The flattened device table is what a Julia `ccall` shim builds from an elaborated
// CedarSim circuit (one row per device instance: model, terminal unknowns, SoA
// parameters).  Everything below is computed once per topology on the host:
//   1. stamps of every device (CedarSim KCL signs, src/simulate_ir.jl:54,112-120),
//   2. the J pattern (union of G and C stamps) in CSC over the original unknowns,
//   3. static pivoting: a structural row matching that puts a structurally nonzero
//      entry on every diagonal (diagonal preferred, then augmenting paths — the
//      maximum-transversal algorithm of Duff, ACM TOMS 7 (1981)); MNA branch rows
//      of V sources / inductors with zero diagonals are paired with KCL rows here,
//   4. a fill-reducing symmetric ordering of the matched matrix (exact minimum
//      degree on the pattern of B + B^T, ties broken by the lower index),
//   5. the LU fill pattern of the permuted matrix (no numerical pivoting at run
//      time: "static pivoting", Li & Demmel, SuperLU_DIST, 1998),
//   6. entry-wise (Crout) factorisation tasks and triangular-solve row tasks,
//      grouped into dependency levels so that a thread group runs one level at a
//      time with no atomics and a fixed summation order (bitwise reproducible).
#include "compile.h"
#include <math.h>
#include "va_models.gen.h"
#include <algorithm>
#include <cmath>
#include <map>
#include <functional>
#include <set>

namespace cedar {

static const ModelInfo kModels[CEDAR_NMODELS] = {
    {0, 0, 0, 0, 0},   // unused
    {2, 2, 0, 2, 1},   // R    out: I, g                 dpar: m/r
    {2, 2, 0, 3, 1},   // C    out: Fpart, cj*mc, Q      dpar: m*c
    {2, 2, 1, 6, 2},   // L    out: mI, Vrow, m, 1, cj*l, l*I   dpar: m, l
    {2, 10, 1, 4, 10}, // V    out: mI, V-vs, m, 1       dpar: raw
    {2, 10, 0, 1, 10}, // I    out: m*is                 dpar: raw
    {4, 2, 1, 5, 2},   // E    out: mI, V-gVc, m, 1, gain   dpar: gain, m
    {4, 2, 0, 2, 1},   // G    out: m g Vc, m g          dpar: m*gain
    {4, 7, 0, 4, 5},   // MOS1 out: mIds, mgm, mgds, m(gm+gds)  dpar: type beta vth lam m
    {2, 4, 0, 2, 3},   // DIODE out: mI, mgd             dpar: IS*AREA, 1/(N Vt), m
    {3, 2, 0, 4, 2},   // NLVCR out: mI, m dI/dVd, m dI/dVg, m dI/dVs(neg)  dpar: 2R, m
};

// Verilog-A models (cedarsim.jl_gb300/va): terminals = ports, raw parameters =
// module parameters + m, derived = raw + thermal voltage, outputs as emitted
static const std::vector<ModelInfo> &va_infos() {
  static const std::vector<ModelInfo> t = [] {
    std::vector<ModelInfo> v;
    for (int k = 0; k < va::kCount; ++k) v.push_back({va::kNTerm[k], va::kNPar[k], va::kHasBr[k], va::kNOut[k], va::kNDPar[k]});
    return v;
  }();
  return t;
}

const ModelInfo &model_info(int model) {
  return model < CEDAR_NMODELS ? kModels[model] : va_infos()[model - va::kBase];
}

int num_models() { return CEDAR_NMODELS + va::kCount; }

void device_stamps(int model, const int *t, int ob, int os, std::vector<Stamp> &J, std::vector<Stamp> &F,
                   std::vector<Stamp> &Q) {
  auto j = [&](int r, int c, int o, int neg) { if (r >= 0 && c >= 0) J.push_back({r, c, ob + o * os, neg}); };
  auto f = [&](int r, int o, int neg) { if (r >= 0) F.push_back({r, -1, ob + o * os, neg}); };
  auto q = [&](int r, int o, int neg) { if (r >= 0) Q.push_back({r, -1, ob + o * os, neg}); };
  switch (model) {
    case CEDAR_R: case CEDAR_DIODE:
      f(t[0], 0, 1); f(t[1], 0, 0);
      j(t[0], t[0], 1, 1); j(t[0], t[1], 1, 0); j(t[1], t[0], 1, 0); j(t[1], t[1], 1, 1);
      break;
    case CEDAR_C:
      f(t[0], 0, 1); f(t[1], 0, 0);
      j(t[0], t[0], 1, 1); j(t[0], t[1], 1, 0); j(t[1], t[0], 1, 0); j(t[1], t[1], 1, 1);
      q(t[0], 2, 1); q(t[1], 2, 0);
      break;
    case CEDAR_L:
      f(t[0], 0, 1); f(t[1], 0, 0); f(t[2], 1, 0);
      j(t[0], t[2], 2, 1); j(t[1], t[2], 2, 0); j(t[2], t[0], 3, 0); j(t[2], t[1], 3, 1); j(t[2], t[2], 4, 1);
      q(t[2], 5, 1);
      break;
    case CEDAR_V:
      f(t[0], 0, 1); f(t[1], 0, 0); f(t[2], 1, 0);
      j(t[0], t[2], 2, 1); j(t[1], t[2], 2, 0); j(t[2], t[0], 3, 0); j(t[2], t[1], 3, 1);
      break;
    case CEDAR_I:
      f(t[0], 0, 1); f(t[1], 0, 0);
      break;
    case CEDAR_E:
      f(t[0], 0, 1); f(t[1], 0, 0); f(t[4], 1, 0);
      j(t[0], t[4], 2, 1); j(t[1], t[4], 2, 0); j(t[4], t[0], 3, 0); j(t[4], t[1], 3, 1);
      j(t[4], t[2], 4, 1); j(t[4], t[3], 4, 0);
      break;
    case CEDAR_G:
      f(t[0], 0, 1); f(t[1], 0, 0);
      j(t[0], t[2], 1, 1); j(t[0], t[3], 1, 0); j(t[1], t[2], 1, 0); j(t[1], t[3], 1, 1);
      break;
    case CEDAR_MOS1:
      f(t[0], 0, 1); f(t[2], 0, 0);
      j(t[0], t[1], 1, 1); j(t[0], t[0], 2, 1); j(t[0], t[2], 3, 0);
      j(t[2], t[1], 1, 0); j(t[2], t[0], 2, 0); j(t[2], t[2], 3, 1);
      break;
    case CEDAR_NLVCR:
      f(t[0], 0, 1); f(t[2], 0, 0);
      j(t[0], t[0], 1, 1); j(t[0], t[1], 2, 1); j(t[0], t[2], 3, 0);
      j(t[2], t[0], 1, 0); j(t[2], t[1], 2, 0); j(t[2], t[2], 3, 1);
      break;
    default: {  // Verilog-A: the emitted outputs already carry the KCL sign
      const int k = model - va::kBase;
      if (k < 0 || k >= va::kCount) break;
      for (int e = va::kStampPtr[k]; e < va::kStampPtr[k + 1]; ++e) {
        const int *st = va::kStamps + 4 * e;  // kind, row port, column port, output
        if (st[0] == 0) f(t[st[1]], st[3], 0);
        else if (st[0] == 2) q(t[st[1]], st[3], 0);
        else j(t[st[1]], t[st[2]], st[3], 0);
      }
    } break;
  }
}

// ------------------------------------------------------------- helpers
static void build_program(int nslots, const std::vector<std::pair<int, int32_t>> &items,
                          std::vector<int32_t> &ptr, std::vector<int32_t> &ent) {
  // items: (slot, encoded entry) in deterministic device order; stable by slot
  ptr.assign(nslots + 1, 0);
  for (auto &it : items) ptr[it.first + 1]++;
  for (int s = 0; s < nslots; ++s) ptr[s + 1] += ptr[s];
  ent.assign(items.size(), 0);
  std::vector<int32_t> fillp(ptr.begin(), ptr.end() - 1);
  for (auto &it : items) ent[fillp[it.first]++] = it.second;
}

static int32_t enc(const Stamp &s) { return (s.out << 1) | (s.neg ? 1 : 0); }

// Outputs that hold cj * dQ/dV (the C part of J = G + cj C): capacitor out 1,
// inductor out 4 (see eval_device).
static bool is_charge_partial(int model, int local_out) {
  if (model >= va::kBase) {  // Verilog-A: stamps of kind 3 (cj dQ/dV)
    const int k = model - va::kBase;
    for (int e = va::kStampPtr[k]; e < va::kStampPtr[k + 1]; ++e)
      if (va::kStamps[4 * e] == 3 && va::kStamps[4 * e + 3] == local_out) return true;
    return false;
  }
  return (model == CEDAR_C && local_out == 1) || (model == CEDAR_L && local_out == 4);
}

// Structural matching: colrows[u] sorted rows with a nonzero in column u.
static bool match_columns(int n, const std::vector<std::vector<int>> &colrows,
                          const std::vector<std::vector<int>> &rowcols, std::vector<int> &rowmatch) {
  std::vector<int> mrow(n, -1), mcol(n, -1);  // mrow[e] = column matched to row e
  for (int u = 0; u < n; ++u)
    if (std::binary_search(colrows[u].begin(), colrows[u].end(), u)) { mrow[u] = u; mcol[u] = u; }
  std::vector<int> visited(n, -1);
  for (int u0 = 0; u0 < n; ++u0) {
    if (mcol[u0] >= 0) continue;
    // cheap assignment
    bool done = false;
    for (int e : colrows[u0]) if (mrow[e] < 0) { mrow[e] = u0; mcol[u0] = e; done = true; break; }
    if (done) continue;
    // iterative DFS for an augmenting path (column -> row -> matched column ...)
    struct Fr { int u; size_t k; };
    std::vector<Fr> st; std::vector<int> path_row;
    st.push_back({u0, 0});
    bool found = false;
    while (!st.empty() && !found) {
      Fr &fr = st.back();
      if (fr.k >= colrows[fr.u].size()) { st.pop_back(); if (!path_row.empty()) path_row.pop_back(); continue; }
      int e = colrows[fr.u][fr.k++];
      if (visited[e] == u0) continue;
      visited[e] = u0;
      if (mrow[e] < 0) {
        path_row.push_back(e);
        // augment along the stack: column st[i].u takes row path_row[i]
        for (size_t i = 0; i < st.size(); ++i) { int uu = st[i].u, ee = path_row[i]; mrow[ee] = uu; mcol[uu] = ee; }
        found = true;
      } else {
        path_row.push_back(e);
        st.push_back({mrow[e], 0});
      }
    }
    if (!found) return false;
  }
  (void)rowcols;
  rowmatch.assign(mcol.begin(), mcol.end());
  return true;
}

// Exact minimum degree on an undirected graph (adjacency without self loops).
static void min_degree(int n, std::vector<std::set<int>> adj, std::vector<int> &order) {
  std::set<std::pair<int, int>> pq;
  for (int v = 0; v < n; ++v) pq.insert({(int)adj[v].size(), v});
  std::vector<char> alive(n, 1);
  order.clear(); order.reserve(n);
  while (!pq.empty()) {
    int v = pq.begin()->second; pq.erase(pq.begin());
    order.push_back(v); alive[v] = 0;
    std::vector<int> N(adj[v].begin(), adj[v].end());
    for (int a : N) {
      pq.erase({(int)adj[a].size(), a});
      adj[a].erase(v);
      for (int b : N) if (b != a) adj[a].insert(b);
      pq.insert({(int)adj[a].size(), a});
    }
    adj[v].clear();
  }
}


// Nested dissection by level structures (George, SIAM J. Numer. Anal. 10 (1973);
// George & Liu 1978): dense vertices (degree > max(16, 4 sqrt n)) are ordered
// last; each connected component of the rest is split at the middle BFS level
// from a pseudo-peripheral vertex, the two sides ordered recursively, the
// separator after them.  Ties and traversal orders use the lowest index.
static void nested_dissection(int n, const std::vector<std::set<int>> &adj, std::vector<int> &order) {
  const int thresh = std::max(16, (int)(4.0 * std::sqrt((double)n)));
  std::vector<char> dense(n, 0), in(n, 0), seen(n, 0);
  for (int v = 0; v < n; ++v) dense[v] = (int)adj[v].size() > thresh;
  order.clear();
  auto bfs = [&](int root, std::vector<std::vector<int>> &levels) {
    levels.clear();
    std::vector<int> cur{root}; std::vector<int> mark;
    seen[root] = 1; mark.push_back(root);
    while (!cur.empty()) {
      std::sort(cur.begin(), cur.end());
      levels.push_back(cur);
      std::vector<int> nxt;
      for (int v : cur) for (int w : adj[v]) if (in[w] && !seen[w]) { seen[w] = 1; mark.push_back(w); nxt.push_back(w); }
      cur.swap(nxt);
    }
    for (int v : mark) seen[v] = 0;
  };
  auto deg_in = [&](int v) { int d = 0; for (int w : adj[v]) d += in[w]; return d; };
  std::function<void(std::vector<int>)> nd = [&](std::vector<int> V) {
    std::sort(V.begin(), V.end());
    for (int v : V) in[v] = 1;
    // connected components, each from its smallest vertex
    std::vector<std::vector<int>> comps;
    for (int v : V) {
      if (seen[v]) continue;
      std::vector<int> comp{v}; seen[v] = 1;
      for (size_t k = 0; k < comp.size(); ++k)
        for (int w : adj[comp[k]]) if (in[w] && !seen[w]) { seen[w] = 1; comp.push_back(w); }
      std::sort(comp.begin(), comp.end());
      comps.push_back(comp);
    }
    for (int v : V) seen[v] = 0;
    for (int v : V) in[v] = 0;
    if (comps.size() > 1) { for (auto &c : comps) nd(c); return; }
    std::vector<int> &C = comps[0];
    if (C.size() <= 3) { for (int v : C) order.push_back(v); return; }
    for (int v : C) in[v] = 1;
    std::vector<std::vector<int>> levels, lv2;
    bfs(C[0], levels);
    for (int rep = 0; rep < 5; ++rep) {
      int u = -1, best = 1 << 30;
      for (int v : levels.back()) { int d = deg_in(v); if (d < best) { best = d; u = v; } }
      bfs(u, lv2);
      if (lv2.size() > levels.size()) levels.swap(lv2); else break;
    }
    const int m = (int)levels.size() - 1;
    if (m < 2) { for (int v : C) in[v] = 0; for (int v : C) order.push_back(v); return; }
    std::vector<int> S = levels[m / 2];
    std::vector<char> sep(0);
    std::vector<int> rest;
    for (int v : C) in[v] = 0;
    for (int v : S) in[v] = 2;  // mark separator
    for (int v : C) if (in[v] != 2) rest.push_back(v);
    for (int v : S) in[v] = 0;
    nd(rest);
    for (int v : S) order.push_back(v);
  };
  std::vector<int> V, D;
  for (int v = 0; v < n; ++v) (dense[v] ? D : V).push_back(v);
  if (!V.empty()) nd(V);
  std::stable_sort(D.begin(), D.end(), [&](int a, int b) { return adj[a].size() < adj[b].size(); });
  for (int v : D) order.push_back(v);
}

// Estimated critical path of one refactorisation + substitutions when every
// level runs on a group of lanes: per level, the longest task (2 flops per
// pair) plus the pivot reciprocal, plus a barrier.
static double schedule_cost(const Template &T) {
  double c = 0;
  for (size_t l = 0; l + 1 < T.lu_lvl_ptr.size(); ++l) {
    int maxp = 0; bool diag = false;
    for (int t = T.lu_lvl_ptr[l]; t < T.lu_lvl_ptr[l + 1]; ++t) {
      maxp = std::max(maxp, T.lu_pair_ptr[t + 1] - T.lu_pair_ptr[t]);
      if ((T.lu_task_info[t] & 3) == 1) diag = true;
    }
    c += 4 + 2 * maxp + (diag ? 6 : 0);
  }
  auto rows = [&](const std::vector<int32_t> &lvl, const std::vector<int32_t> &ptr) {
    for (size_t l = 0; l + 1 < lvl.size(); ++l) {
      int maxp = 0;
      for (int t = lvl[l]; t < lvl[l + 1]; ++t) maxp = std::max(maxp, ptr[t + 1] - ptr[t]);
      c += 4 + 2 * maxp;
    }
  };
  rows(T.fw_lvl_ptr, T.fw_ptr);
  rows(T.bw_lvl_ptr, T.bw_ptr);
  return c;
}

static bool compile_with(const cedar_ckt_desc *d, Template &T, std::string &err, int ordering) {
  if (!d) { err = "null desc"; return false; }
  if (d->n_nodes < 0 || d->n_branch < 0 || d->n_groups < 0 || (d->n_groups > 0 && !d->groups)) { err = "malformed desc"; return false; }
  T = Template();
  T.n_nodes = d->n_nodes; T.n_branch = d->n_branch; T.n = d->n_nodes + d->n_branch;
  T.temp_c = d->temp_c; T.gmin = d->gmin;
  const int n = T.n;
  if (n <= 0) { err = "empty system"; return false; }
  if (d->pwl && d->n_pwl > 0) T.pwl.assign(d->pwl, d->pwl + d->n_pwl);
  // groups
  int term_off = 0, par_off = 0, dpar_off = 0, out_off = 0;
  for (int g = 0; g < d->n_groups; ++g) {
    const cedar_devgroup &s = d->groups[g];
    if (s.model <= 0 || s.model >= num_models()) { err = "unknown model id " + std::to_string(s.model); return false; }
    if (s.n_inst < 0) { err = "negative instance count"; return false; }
    const ModelInfo &mi = model_info(s.model);
    if (s.n_inst > 0 && (!s.term || !s.par || (mi.has_br && !s.branch))) { err = "group missing arrays"; return false; }
    GroupInfo gi{};
    gi.model = s.model; gi.n_inst = s.n_inst; gi.ntx = mi.nterm + mi.has_br;
    gi.term_off = term_off; gi.par_off = par_off; gi.dpar_off = dpar_off; gi.out_off = out_off;
    for (int i = 0; i < s.n_inst; ++i) {
      for (int k = 0; k < mi.nterm; ++k) {
        int u = s.term[(size_t)i * mi.nterm + k];
        if (u < -1 || u >= n) { err = "terminal index out of range"; return false; }
        T.term_orig.push_back(u);
      }
      if (mi.has_br) {
        int b = s.branch[i];
        if (b < T.n_nodes || b >= n) { err = "branch index out of range"; return false; }
        T.term_orig.push_back(b);
      }
    }
    for (size_t k = 0; k < (size_t)mi.npar * s.n_inst; ++k) T.par.push_back(s.par[k]);
    // PWL references must lie inside the table
    if ((s.model == CEDAR_V || s.model == CEDAR_I)) {
      for (int i = 0; i < s.n_inst; ++i) {
        int kind = (int)s.par[2 * s.n_inst + i];
        if (kind < 0 || kind > 3) { err = "bad waveform kind"; return false; }
        if (kind == CEDAR_WAVE_PWL) {
          double off = s.par[3 * s.n_inst + i], np = s.par[4 * s.n_inst + i];
          if (off < 0 || np < 1 || off + 2 * np > (double)T.pwl.size()) { err = "PWL reference outside table"; return false; }
        }
        if (kind != CEDAR_WAVE_DC) { T.src_group.push_back(g); T.src_inst.push_back(i); }
      }
    }
    term_off += gi.ntx * s.n_inst; par_off += mi.npar * s.n_inst;
    dpar_off += mi.ndpar * s.n_inst; out_off += mi.nout * s.n_inst;
    T.groups.push_back(gi);
  }
  T.par_size = par_off; T.dpar_size = dpar_off; T.n_out = out_off;
  T.out_q.assign(std::max(out_off, 1), 0);
  for (const GroupInfo &g : T.groups) {
    const int no = model_info(g.model).nout;
    for (int i = 0; i < g.n_inst; ++i)
      for (int k = 0; k < no; ++k) T.out_q[g.out_off + k * g.n_inst + i] = is_charge_partial(g.model, k) ? 1 : 0;
  }

  // stamps in device order; SJq marks J stamps carrying a charge partial (cj dQ/dV)
  std::vector<Stamp> SJ, SF, SQ;
  std::vector<char> SJq;
  T.adj_goff.clear(); T.n_adj = 0;
  for (const GroupInfo &g : T.groups) {
    const ModelInfo &mi = model_info(g.model);
    for (int i = 0; i < g.n_inst; ++i) {
      // output k of device i at out_off + k * n_inst + i (output-major per group)
      const int ob = g.out_off + i, os = g.n_inst;
      size_t before = SJ.size();
      device_stamps(g.model, &T.term_orig[g.term_off + (size_t)i * g.ntx], ob, os, SJ, SF, SQ);
      for (size_t k = before; k < SJ.size(); ++k) SJq.push_back(is_charge_partial(g.model, (SJ[k].out - ob) / os) ? 1 : 0);
    }
    const bool diff = (g.model == CEDAR_MOS1 || g.model == CEDAR_R);
    T.adj_goff.push_back(diff ? T.n_adj : -1);
    if (diff) T.n_adj += g.n_inst;
  }
  // original pattern
  std::vector<std::vector<int>> colrows(n), rowcols(n);
  for (const Stamp &s : SJ) { colrows[s.col].push_back(s.row); rowcols[s.row].push_back(s.col); }
  for (int u = 0; u < n; ++u) {
    auto &v = colrows[u]; std::sort(v.begin(), v.end()); v.erase(std::unique(v.begin(), v.end()), v.end());
    auto &w = rowcols[u]; std::sort(w.begin(), w.end()); w.erase(std::unique(w.begin(), w.end()), w.end());
  }
  T.j_colptr.assign(n + 1, 0);
  for (int u = 0; u < n; ++u) T.j_colptr[u + 1] = T.j_colptr[u] + (int)colrows[u].size();
  T.j_rowidx.clear();
  for (int u = 0; u < n; ++u) for (int e : colrows[u]) T.j_rowidx.push_back(e);
  for (int u = 0; u < n; ++u) if (colrows[u].empty()) { err = "structurally singular: unknown " + std::to_string(u) + " appears in no equation"; return false; }

  // static pivoting
  if (!match_columns(n, colrows, rowcols, T.rowmatch)) { err = "structurally singular system (no perfect matching)"; return false; }
  // B[u'][u] = J[rowmatch[u']][u]; symmetric pattern of B + B^T
  std::vector<int> eq2u(n);
  for (int u = 0; u < n; ++u) eq2u[T.rowmatch[u]] = u;
  std::vector<std::set<int>> adj(n);
  for (int u = 0; u < n; ++u)
    for (int e : colrows[u]) { int up = eq2u[e]; if (up != u) { adj[up].insert(u); adj[u].insert(up); } }
  // node diagonals (KCL(u), u) join the factorisation pattern (not the J pattern)
  // so that the DC gmin homotopy has a slot to stamp into; they take no part in
  // the matching above, which only sees structurally nonzero entries.
  for (int u = 0; u < T.n_nodes; ++u) {
    auto &v = colrows[u];
    if (!std::binary_search(v.begin(), v.end(), u)) { v.insert(std::lower_bound(v.begin(), v.end(), u), u); }
    int up = eq2u[u]; if (up != u) { adj[up].insert(u); adj[u].insert(up); }
  }
  if (ordering == ORDER_NATURAL) { T.order.resize(n); for (int i = 0; i < n; ++i) T.order[i] = i; }
  else if (ordering == ORDER_NESTED_DISSECTION) nested_dissection(n, adj, T.order);
  else min_degree(n, adj, T.order);
  T.ordering = ordering;
  T.iorder.assign(n, 0);
  for (int p = 0; p < n; ++p) T.iorder[T.order[p]] = p;
  T.eq_pos.assign(n, 0);
  for (int u = 0; u < n; ++u) T.eq_pos[T.rowmatch[u]] = T.iorder[u];
  T.is_node_int.assign(n, 0);
  for (int p = 0; p < n; ++p) T.is_node_int[p] = T.order[p] < T.n_nodes ? 1 : 0;
  T.term_int.resize(T.term_orig.size());
  for (size_t k = 0; k < T.term_orig.size(); ++k) T.term_int[k] = T.term_orig[k] < 0 ? -1 : T.iorder[T.term_orig[k]];

  // symbolic LU of M[p][q] = J[eq(p)][order(q)], row by row ("up-looking"): the
  // pattern of row i is its own pattern closed under k -> U(k) = {q > k in row k}
  // for every k < i in it (rows k < i already final).  A marker array makes each
  // row cost O(its fill work), so a dense supply row costs O(n), not O(n^2).
  std::vector<std::vector<int>> rows(n);
  for (int u = 0; u < n; ++u)
    for (int e : colrows[u]) rows[T.eq_pos[e]].push_back(T.iorder[u]);
  {
    std::vector<int> mark(n, -1), work;
    std::vector<int> first_upper(n, 0);  // position of the first entry > k in final row k
    for (int i = 0; i < n; ++i) {
      std::vector<int> &ri = rows[i];
      std::vector<int> pat;
      pat.reserve(ri.size() * 2);
      work.clear();
      for (int q : ri) if (mark[q] != i) { mark[q] = i; pat.push_back(q); if (q < i) work.push_back(q); }
      while (!work.empty()) {
        const int k = work.back(); work.pop_back();
        const std::vector<int> &rk = rows[k];
        for (size_t t = first_upper[k]; t < rk.size(); ++t) {
          const int q = rk[t];
          if (mark[q] != i) { mark[q] = i; pat.push_back(q); if (q < i) work.push_back(q); }
        }
      }
      std::sort(pat.begin(), pat.end());
      if (!std::binary_search(pat.begin(), pat.end(), i)) { err = "internal: missing diagonal after matching"; return false; }
      ri.swap(pat);
      first_upper[i] = (int)(std::upper_bound(ri.begin(), ri.end(), i) - ri.begin());
    }
  }
  T.lu_rowptr.assign(n + 1, 0);
  for (int p = 0; p < n; ++p) T.lu_rowptr[p + 1] = T.lu_rowptr[p] + (int)rows[p].size();
  T.nnz_lu = T.lu_rowptr[n];
  T.lu_colidx.clear(); T.lu_colidx.reserve(T.nnz_lu);
  for (int p = 0; p < n; ++p) for (int q : rows[p]) T.lu_colidx.push_back(q);
  T.lu_diag.assign(n, -1);
  auto slot = [&](int p, int q) -> int {
    auto b = T.lu_colidx.begin() + T.lu_rowptr[p], e = T.lu_colidx.begin() + T.lu_rowptr[p + 1];
    auto it = std::lower_bound(b, e, q);
    return (it != e && *it == q) ? (int)(it - T.lu_colidx.begin()) : -1;
  };
  for (int p = 0; p < n; ++p) T.lu_diag[p] = slot(p, p);
  T.gs_slot.assign(T.n_nodes, -1);
  for (int u = 0; u < T.n_nodes; ++u) T.gs_slot[u] = slot(T.eq_pos[u], T.iorder[u]);
  // LU column structure (rows per column, sorted)
  std::vector<std::vector<int>> lucol(n);
  for (int p = 0; p < n; ++p) for (int q : rows[p]) lucol[q].push_back(p);

  // stamp programs
  {
    std::vector<std::pair<int, int32_t>> it;
    for (const Stamp &s : SJ) it.push_back({slot(T.eq_pos[s.row], T.iorder[s.col]), enc(s)});
    build_program(T.nnz_lu, it, T.jlu_ptr, T.jlu_ent);
    it.clear();
    for (const Stamp &s : SJ) {
      auto b = T.j_rowidx.begin() + T.j_colptr[s.col], e = T.j_rowidx.begin() + T.j_colptr[s.col + 1];
      int k = (int)(std::lower_bound(b, e, s.row) - T.j_rowidx.begin());
      it.push_back({k, enc(s)});
    }
    build_program((int)T.j_rowidx.size(), it, T.jcsc_ptr, T.jcsc_ent);
    it.clear();
    for (const Stamp &s : SF) it.push_back({T.eq_pos[s.row], enc(s)});
    build_program(n, it, T.fint_ptr, T.fint_ent);
    it.clear();
    for (const Stamp &s : SF) it.push_back({s.row, enc(s)});
    build_program(n, it, T.forg_ptr, T.forg_ent);
    it.clear();
    for (const Stamp &s : SQ) it.push_back({T.eq_pos[s.row], enc(s)});
    build_program(n, it, T.qint_ptr, T.qint_ent);
    auto longs = [](const std::vector<int32_t> &ptr, int lim, std::vector<int32_t> &out) {
      out.clear();
      for (size_t q = 0; q + 1 < ptr.size(); ++q) if (ptr[q + 1] - ptr[q] > lim) out.push_back((int32_t)q);
    };
    longs(T.jlu_ptr, kLongGatherHost, T.long_lu);
    longs(T.fint_ptr, kLongGatherHost, T.long_fi);
    longs(T.jcsc_ptr, kLongEvalHost, T.long_jc);
    longs(T.forg_ptr, kLongEvalHost, T.long_fo);
    T.long_jc_fo_off.assign(1, 0);
    for (int32_t q : T.long_jc) T.long_jc_fo_off.push_back(T.long_jc_fo_off.back() + (T.jcsc_ptr[q + 1] - T.jcsc_ptr[q] + kLongChunk - 1) / kLongChunk);
    for (int32_t q : T.long_fo) T.long_jc_fo_off.push_back(T.long_jc_fo_off.back() + (T.forg_ptr[q + 1] - T.forg_ptr[q] + kLongChunk - 1) / kLongChunk);
    // C^T program: per internal column q, the charge-partial stamps of column q
    // with their internal rows, in device order
    std::vector<std::pair<int, int32_t>> ic;
    std::vector<int32_t> rowsof;
    for (size_t k = 0; k < SJ.size(); ++k) if (SJq[k]) { ic.push_back({T.iorder[SJ[k].col], (int32_t)rowsof.size()}); rowsof.push_back((int32_t)k); }
    std::vector<int32_t> idx;
    build_program(n, ic, T.ct_ptr, idx);
    T.ct_ent.resize(idx.size()); T.ct_row.resize(idx.size());
    for (size_t e = 0; e < idx.size(); ++e) { const Stamp &st = SJ[rowsof[idx[e]]]; T.ct_ent[e] = enc(st); T.ct_row[e] = T.eq_pos[st.row]; }
  }

  // factorisation tasks
  struct Task { int slot, info, lev; std::vector<std::pair<int, int>> pairs; };
  std::vector<Task> tasks; tasks.reserve(T.nnz_lu);
  std::vector<int> lev(T.nnz_lu, -1);
  auto make_task = [&](int i, int j) {
    int s = slot(i, j); int m = std::min(i, j);
    Task tk; tk.slot = s; tk.info = (j << 2) | (i == j ? 1 : (i > j ? 2 : 0));
    // pairs k < m with (i,k) and (k,j)
    // walk the shorter of (row i below m) and (column j below m), binary-search the
    // other: a dense supply row then costs O(its column lengths), not O(n) per task
    const int *ri = &T.lu_colidx[T.lu_rowptr[i]];
    const int nri = (int)(std::lower_bound(ri, ri + (T.lu_rowptr[i + 1] - T.lu_rowptr[i]), m) - ri);
    const std::vector<int> &cj = lucol[j];
    const int ncj = (int)(std::lower_bound(cj.begin(), cj.end(), m) - cj.begin());
    int L = 0;
    auto add_pair = [&](int k, int sa) {
      const int sb = slot(k, j);
      tk.pairs.push_back({sa, sb});
      L = std::max(L, std::max(lev[sa], lev[sb]) + 1);
    };
    if (nri <= ncj) {
      for (int a = 0; a < nri; ++a)
        if (std::binary_search(cj.begin(), cj.begin() + ncj, ri[a])) add_pair(ri[a], T.lu_rowptr[i] + a);
    } else {
      for (int b = 0; b < ncj; ++b) {
        const int k = cj[b];
        const int *it = std::lower_bound(ri, ri + nri, k);
        if (it != ri + nri && *it == k) add_pair(k, T.lu_rowptr[i] + (int)(it - ri));
      }
    }
    if (i > j) L = std::max(L, lev[T.lu_diag[j]] + 1);
    tk.lev = L; lev[s] = L;
    tasks.push_back(std::move(tk));
  };
  for (int m = 0; m < n; ++m) {
    make_task(m, m);
    for (int k = T.lu_rowptr[m]; k < T.lu_rowptr[m + 1]; ++k) if (T.lu_colidx[k] > m) make_task(m, T.lu_colidx[k]);
    for (int i : lucol[m]) if (i > m) make_task(i, m);
  }
  int nlev = 0; for (auto &t : tasks) nlev = std::max(nlev, t.lev + 1);
  std::stable_sort(tasks.begin(), tasks.end(), [](const Task &a, const Task &b) {
    if (a.lev != b.lev) return a.lev < b.lev;
    return a.pairs.size() > b.pairs.size();
  });
  T.lu_lvl_ptr.assign(nlev + 1, 0);
  for (auto &t : tasks) T.lu_lvl_ptr[t.lev + 1]++;
  for (int l = 0; l < nlev; ++l) T.lu_lvl_ptr[l + 1] += T.lu_lvl_ptr[l];
  T.lu_task_slot.clear(); T.lu_task_info.clear(); T.lu_pair_ptr.assign(1, 0); T.lu_pair_a.clear(); T.lu_pair_b.clear();
  T.lu_flops = 0;
  for (auto &t : tasks) {
    T.lu_task_slot.push_back(t.slot); T.lu_task_info.push_back(t.info);
    for (auto &p : t.pairs) { T.lu_pair_a.push_back(p.first); T.lu_pair_b.push_back(p.second); }
    T.lu_pair_ptr.push_back((int)T.lu_pair_a.size());
    T.lu_flops += 2 * (int64_t)t.pairs.size() + ((t.info & 3) != 0 ? 1 : 0);
  }

  // triangular solves
  {
    std::vector<int> lf(n, 0);
    for (int i = 0; i < n; ++i) { int L = 0; for (int k = T.lu_rowptr[i]; k < T.lu_diag[i]; ++k) L = std::max(L, lf[T.lu_colidx[k]] + 1); lf[i] = L; }
    std::vector<int> lb(n, 0);
    for (int i = n - 1; i >= 0; --i) { int L = 0; for (int k = T.lu_diag[i] + 1; k < T.lu_rowptr[i + 1]; ++k) L = std::max(L, lb[T.lu_colidx[k]] + 1); lb[i] = L; }
    auto emit = [&](const std::vector<int> &lv, bool fw, std::vector<int32_t> &lp, std::vector<int32_t> &rw,
                    std::vector<int32_t> &pp, std::vector<int32_t> &pl, std::vector<int32_t> &pc) {
      int nl = 0; for (int v : lv) nl = std::max(nl, v + 1);
      std::vector<int> idx(n); for (int i = 0; i < n; ++i) idx[i] = i;
      std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return lv[a] < lv[b]; });
      lp.assign(nl + 1, 0); for (int i = 0; i < n; ++i) lp[lv[i] + 1]++;
      for (int l = 0; l < nl; ++l) lp[l + 1] += lp[l];
      rw.clear(); pp.assign(1, 0); pl.clear(); pc.clear();
      for (int i : idx) {
        rw.push_back(i);
        int k0 = fw ? T.lu_rowptr[i] : T.lu_diag[i] + 1, k1 = fw ? T.lu_diag[i] : T.lu_rowptr[i + 1];
        for (int k = k0; k < k1; ++k) { pl.push_back(k); pc.push_back(T.lu_colidx[k]); }
        pp.push_back((int)pl.size());
      }
    };
    emit(lf, true, T.fw_lvl_ptr, T.fw_row, T.fw_ptr, T.fw_lu, T.fw_col);
    emit(lb, false, T.bw_lvl_ptr, T.bw_row, T.bw_ptr, T.bw_lu, T.bw_col);

    // transposed substitutions for J^T lam = r with J = L U (adjoint):
    //   U^T z = r:   z_i = (r_i - sum_{j<i} U[j][i] z_j) / U[i][i]   (column i of U above the diagonal)
    //   L^T lam = z: lam_i = z_i - sum_{j>i} L[j][i] lam_j          (column i of L below the diagonal)
    std::vector<int> tfl(n, 0), tbl(n, 0);
    for (int i = 0; i < n; ++i) { int L = 0; for (int p : lucol[i]) if (p < i) L = std::max(L, tfl[p] + 1); tfl[i] = L; }
    for (int i = n - 1; i >= 0; --i) { int L = 0; for (int p : lucol[i]) if (p > i) L = std::max(L, tbl[p] + 1); tbl[i] = L; }
    auto emit_t = [&](const std::vector<int> &lv, bool upper, std::vector<int32_t> &lp, std::vector<int32_t> &rw,
                      std::vector<int32_t> &pp, std::vector<int32_t> &pl, std::vector<int32_t> &pc) {
      int nl = 0; for (int v : lv) nl = std::max(nl, v + 1);
      std::vector<int> idx(n); for (int i = 0; i < n; ++i) idx[i] = i;
      std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return lv[a] < lv[b]; });
      lp.assign(nl + 1, 0); for (int i = 0; i < n; ++i) lp[lv[i] + 1]++;
      for (int l = 0; l < nl; ++l) lp[l + 1] += lp[l];
      rw.clear(); pp.assign(1, 0); pl.clear(); pc.clear();
      for (int i : idx) {
        rw.push_back(i);
        for (int p : lucol[i]) if (upper ? p < i : p > i) { pl.push_back(slot(p, i)); pc.push_back(p); }
        pp.push_back((int)pl.size());
      }
    };
    emit_t(tfl, true, T.tf_lvl_ptr, T.tf_row, T.tf_ptr, T.tf_lu, T.tf_col);
    emit_t(tbl, false, T.tb_lvl_ptr, T.tb_row, T.tb_ptr, T.tb_lu, T.tb_col);
  }
  return true;
}

// ------------------------------------------------------------- validation
// Every index the kernels follow, checked against the extent of what it
// indexes.  The kernels trust these tables (they carry no per-access bounds
// checks on the hot path), so a compiler defect must stop here, on the host,
// before anything is uploaded or launched.
namespace {
struct Checker {
  std::string &err;
  bool ok = true;
  bool fail(const std::string &what) {
    if (ok) err = "internal: template check failed: " + what;
    ok = false;
    return false;
  }
  // v[k] in [lo, hi) for every k
  bool range(const std::vector<int32_t> &v, int64_t lo, int64_t hi, const char *name) {
    for (size_t k = 0; k < v.size(); ++k)
      if (v[k] < lo || v[k] >= hi)
        return fail(std::string(name) + "[" + std::to_string(k) + "] = " + std::to_string(v[k]) + " outside [" +
                    std::to_string(lo) + ", " + std::to_string(hi) + ")");
    return true;
  }
  bool size(size_t got, size_t want, const char *name) {
    if (got != want) return fail(std::string(name) + " has " + std::to_string(got) + " entries, expected " + std::to_string(want));
    return true;
  }
  // a CSR-style pointer array: nslots + 1 entries, 0 first, nondecreasing, ends at total
  bool ptr(const std::vector<int32_t> &p, size_t nslots, size_t total, const char *name) {
    if (!size(p.size(), nslots + 1, name)) return false;
    if (p[0] != 0 || (size_t)p[nslots] != total) return fail(std::string(name) + " does not span its entries");
    for (size_t k = 0; k < nslots; ++k)
      if (p[k + 1] < p[k]) return fail(std::string(name) + " decreases at " + std::to_string(k));
    return true;
  }
  bool perm(const std::vector<int32_t> &v, int n, const char *name) {
    if (!size(v.size(), (size_t)n, name) || !range(v, 0, n, name)) return false;
    std::vector<char> seen(n, 0);
    for (int32_t x : v) { if (seen[x]) return fail(std::string(name) + " is not a permutation"); seen[x] = 1; }
    return true;
  }
  // a stamp program: per-slot gather lists of ((output << 1) | negate) entries
  bool program(const std::vector<int32_t> &p, const std::vector<int32_t> &ent, size_t nslots, int n_out,
               const char *name) {
    if (!ptr(p, nslots, ent.size(), name)) return false;
    for (size_t k = 0; k < ent.size(); ++k)
      if (ent[k] < 0 || (ent[k] >> 1) >= n_out) return fail(std::string(name) + " entry " + std::to_string(k) + " names no device output");
    return true;
  }
  // level-scheduled row tasks (substitutions): a permutation of the rows in
  // levels, each with its (LU slot, column) pairs
  bool rows(const std::vector<int32_t> &lvl, const std::vector<int32_t> &row, const std::vector<int32_t> &p,
            const std::vector<int32_t> &lu, const std::vector<int32_t> &col, int n, int nnz_lu, const char *name) {
    if (lvl.empty() || lvl.front() != 0 || (size_t)lvl.back() != row.size()) return fail(std::string(name) + " levels do not span the rows");
    for (size_t l = 0; l + 1 < lvl.size(); ++l)
      if (lvl[l + 1] < lvl[l]) return fail(std::string(name) + " levels decrease");
    return perm(row, n, name) && ptr(p, row.size(), lu.size(), name) && size(col.size(), lu.size(), name) &&
           range(lu, 0, nnz_lu, name) && range(col, 0, n, name);
  }
};
}  // namespace

bool validate_template(const Template &T, std::string &err) {
  Checker c{err};
  const int n = T.n, nnz = T.nnz_lu;
  if (n <= 0 || n != T.n_nodes + T.n_branch) return c.fail("unknown counts");
  // device groups and their slices of the terminal, parameter and output blocks
  int term = 0, par = 0, dpar = 0, out = 0;
  for (const GroupInfo &g : T.groups) {
    if (g.model <= 0 || g.model >= num_models() || g.n_inst < 0) return c.fail("group model or size");
    const ModelInfo &mi = model_info(g.model);
    if (g.ntx != mi.nterm + mi.has_br || g.term_off != term || g.par_off != par || g.dpar_off != dpar || g.out_off != out)
      return c.fail("group offsets");
    term += g.ntx * g.n_inst; par += mi.npar * g.n_inst; dpar += mi.ndpar * g.n_inst; out += mi.nout * g.n_inst;
  }
  if (par != T.par_size || dpar != T.dpar_size || out != T.n_out) return c.fail("block sizes");
  if (!c.size(T.term_orig.size(), (size_t)term, "term_orig") || !c.size(T.term_int.size(), (size_t)term, "term_int") ||
      !c.range(T.term_orig, -1, n, "term_orig") || !c.range(T.term_int, -1, n, "term_int") ||
      !c.size(T.par.size(), (size_t)T.par_size, "par") || !c.size(T.out_q.size(), (size_t)std::max(T.n_out, 1), "out_q"))
    return false;
  // orderings
  if (!c.perm(T.rowmatch, n, "rowmatch") || !c.perm(T.order, n, "order") || !c.perm(T.iorder, n, "iorder") ||
      !c.perm(T.eq_pos, n, "eq_pos") || !c.size(T.is_node_int.size(), (size_t)n, "is_node_int"))
    return false;
  for (int p = 0; p < n; ++p)
    if (T.iorder[T.order[p]] != p) return c.fail("iorder is not the inverse of order");
  // J pattern (original CSC) and LU pattern (internal CSR, sorted, with diagonals)
  const size_t ncsc = T.j_rowidx.size();
  if (!c.ptr(T.j_colptr, n, ncsc, "j_colptr") || !c.range(T.j_rowidx, 0, n, "j_rowidx") ||
      !c.ptr(T.lu_rowptr, n, (size_t)nnz, "lu_rowptr") || !c.size(T.lu_colidx.size(), (size_t)nnz, "lu_colidx") ||
      !c.range(T.lu_colidx, 0, n, "lu_colidx") || !c.size(T.lu_diag.size(), (size_t)n, "lu_diag"))
    return false;
  for (int p = 0; p < n; ++p) {
    for (int k = T.lu_rowptr[p] + 1; k < T.lu_rowptr[p + 1]; ++k)
      if (T.lu_colidx[k] <= T.lu_colidx[k - 1]) return c.fail("lu_colidx unsorted in row " + std::to_string(p));
    const int d = T.lu_diag[p];
    if (d < T.lu_rowptr[p] || d >= T.lu_rowptr[p + 1] || T.lu_colidx[d] != p) return c.fail("lu_diag of row " + std::to_string(p));
  }
  // stamp programs
  if (!c.program(T.jlu_ptr, T.jlu_ent, (size_t)nnz, T.n_out, "jlu") ||
      !c.program(T.jcsc_ptr, T.jcsc_ent, ncsc, T.n_out, "jcsc") ||
      !c.program(T.fint_ptr, T.fint_ent, (size_t)n, T.n_out, "fint") ||
      !c.program(T.qint_ptr, T.qint_ent, (size_t)n, T.n_out, "qint") ||
      !c.program(T.forg_ptr, T.forg_ent, (size_t)n, T.n_out, "forg") ||
      !c.program(T.ct_ptr, T.ct_ent, (size_t)n, T.n_out, "ct") || !c.size(T.ct_row.size(), T.ct_ent.size(), "ct_row") ||
      !c.range(T.ct_row, 0, n, "ct_row"))
    return false;
  // long gather lists and their chunk offsets
  if (!c.range(T.long_lu, 0, nnz, "long_lu") || !c.range(T.long_fi, 0, n, "long_fi") ||
      !c.range(T.long_jc, 0, (int64_t)ncsc, "long_jc") || !c.range(T.long_fo, 0, n, "long_fo"))
    return false;
  {
    const size_t nl = T.long_jc.size() + T.long_fo.size();
    if (!c.size(T.long_jc_fo_off.size(), nl + 1, "long_jc_fo_off") || T.long_jc_fo_off[0] != 0) return c.fail("long_jc_fo_off");
    for (size_t k = 0; k < nl; ++k) {
      const bool jc = k < T.long_jc.size();
      const int q = jc ? T.long_jc[k] : T.long_fo[k - T.long_jc.size()];
      const int len = jc ? T.jcsc_ptr[q + 1] - T.jcsc_ptr[q] : T.forg_ptr[q + 1] - T.forg_ptr[q];
      if (T.long_jc_fo_off[k + 1] - T.long_jc_fo_off[k] != (len + kLongChunk - 1) / kLongChunk)
        return c.fail("long_jc_fo_off chunk count of list " + std::to_string(k));
    }
  }
  // factorisation tasks by level
  const size_t nt = T.lu_task_slot.size();
  if (T.lu_lvl_ptr.empty() || T.lu_lvl_ptr.front() != 0 || (size_t)T.lu_lvl_ptr.back() != nt) return c.fail("lu levels do not span the tasks");
  for (size_t l = 0; l + 1 < T.lu_lvl_ptr.size(); ++l)
    if (T.lu_lvl_ptr[l + 1] < T.lu_lvl_ptr[l]) return c.fail("lu levels decrease");
  if (!c.size(nt, (size_t)nnz, "lu_task_slot") || !c.perm(T.lu_task_slot, nnz, "lu_task_slot") ||
      !c.size(T.lu_task_info.size(), nt, "lu_task_info") || !c.ptr(T.lu_pair_ptr, nt, T.lu_pair_a.size(), "lu_pair_ptr") ||
      !c.size(T.lu_pair_b.size(), T.lu_pair_a.size(), "lu_pair_b") || !c.range(T.lu_pair_a, 0, nnz, "lu_pair_a") ||
      !c.range(T.lu_pair_b, 0, nnz, "lu_pair_b"))
    return false;
  for (size_t t = 0; t < nt; ++t) {
    const int kind = T.lu_task_info[t] & 3, col = T.lu_task_info[t] >> 2;
    if (kind == 3 || col < 0 || col >= n) return c.fail("lu_task_info of task " + std::to_string(t));
  }
  // substitutions, forward / backward and transposed
  if (!c.rows(T.fw_lvl_ptr, T.fw_row, T.fw_ptr, T.fw_lu, T.fw_col, n, nnz, "fw") ||
      !c.rows(T.bw_lvl_ptr, T.bw_row, T.bw_ptr, T.bw_lu, T.bw_col, n, nnz, "bw") ||
      !c.rows(T.tf_lvl_ptr, T.tf_row, T.tf_ptr, T.tf_lu, T.tf_col, n, nnz, "tf") ||
      !c.rows(T.tb_lvl_ptr, T.tb_row, T.tb_ptr, T.tb_lu, T.tb_col, n, nnz, "tb"))
    return false;
  // adjoint parameter offsets, time-varying sources, gmin-stepping slots
  if (!c.size(T.adj_goff.size(), T.groups.size(), "adj_goff") || !c.range(T.adj_goff, -1, (int64_t)T.n_adj + 1, "adj_goff") ||
      !c.size(T.src_inst.size(), T.src_group.size(), "src_inst") ||
      !c.range(T.src_group, 0, (int64_t)T.groups.size(), "src_group") || !c.size(T.gs_slot.size(), (size_t)T.n_nodes, "gs_slot") ||
      !c.range(T.gs_slot, 0, nnz, "gs_slot"))
    return false;
  for (size_t k = 0; k < T.src_inst.size(); ++k)
    if (T.src_inst[k] < 0 || T.src_inst[k] >= T.groups[T.src_group[k]].n_inst) return c.fail("src_inst");
  return true;
}

bool compile_template(const cedar_ckt_desc *d, Template &T, std::string &err, int ordering) {
  if (ordering == ORDER_AUTO) {
    Template A, B;
    if (!compile_with(d, A, err, ORDER_MIN_DEGREE)) return false;
    if (!compile_with(d, B, err, ORDER_NESTED_DISSECTION)) return false;
    A.sched_cost = schedule_cost(A);
    B.sched_cost = schedule_cost(B);
    T = (B.sched_cost < A.sched_cost) ? std::move(B) : std::move(A);
  } else {
    if (!compile_with(d, T, err, ordering)) return false;
    T.sched_cost = schedule_cost(T);
  }
  return validate_template(T, err);
}

}  // namespace cedar
