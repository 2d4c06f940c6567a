// api.cu — the C ABI (include/cedar.h) over the compiler and the kernels.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define CEDAR_NVTX 1
#endif
#include "compile.h"
#include "kernels.cuh"
// per-model FP64 operation counts of one device evaluation (written by build.py)
#include "flops.gen.h"

using namespace cedar;

static_assert(sizeof(EngStats) == sizeof(cedar_stats), "stats layout");
static_assert(kLongGatherHost == kLongGather && kLongEvalHost == kLongEval, "long gather thresholds");
static_assert(kLongChunk == 256, "cedar_eval long-list chunk (k_plain.cu kLongChunkDev)");

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) { g_err = msg; return code; }

// An NVTX range named after the entry point around each call that runs work on
// the device, so that a profiler's timeline (Nsight Systems, ncu --nvtx) groups
// the kernels and copies by C-ABI call; without a profiler attached it does
// nothing, and a toolkit without the NVTX headers builds it as nothing.
struct Range {
#ifdef CEDAR_NVTX
  explicit Range(const char *name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
#else
  explicit Range(const char *) {}
#endif
  Range(const Range &) = delete;
  Range &operator=(const Range &) = delete;
};
#define CUDA_TRY(expr)                                                                      \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess) return fail(CEDAR_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// ------------------------------------------------------------ device template
struct DevTemplate {
  Template H;
  void *buf = nullptr;
  DTpl D{};
  DTpl *D_dev = nullptr;
  double *par_dev = nullptr;  // nominal raw params
  ~DevTemplate() { if (buf) cudaFree(buf); if (D_dev) cudaFree(D_dev); if (par_dev) cudaFree(par_dev); }
};

struct Packer {
  std::vector<char> bytes;
  size_t add(const void *p, size_t n) {
    size_t off = (bytes.size() + 255) & ~size_t(255);
    bytes.resize(off + std::max<size_t>(n, 1));
    if (n) std::memcpy(bytes.data() + off, p, n);
    return off;
  }
  template <class T> size_t vec(const std::vector<T> &v) { return add(v.data(), v.size() * sizeof(T)); }
};

int compile_only(const cedar_ckt_desc *desc, std::unique_ptr<DevTemplate> &out) {
  auto dt = std::make_unique<DevTemplate>();
  std::string err;
  int ordering = desc ? desc->ordering : 0;
  if (ordering < 0 || ordering > 2) return fail(CEDAR_EINVAL, "unknown ordering");
  if (!compile_template(desc, dt->H, err, ordering)) return fail(err.find("singular") != std::string::npos ? CEDAR_ESINGULAR : CEDAR_EINVAL, err);
  out = std::move(dt);
  return 0;
}

int upload_template(const cedar_ckt_desc *desc, std::unique_ptr<DevTemplate> &out) {
  std::unique_ptr<DevTemplate> dt;
  int rc0 = compile_only(desc, dt);
  if (rc0) return rc0;
  Template &H = dt->H;
  std::vector<DGroup> grp; std::vector<int> dev_end; int nd = 0;
  for (auto &g : H.groups) { grp.push_back({g.model, g.n_inst, g.ntx, g.term_off, g.par_off, g.dpar_off, g.out_off}); nd += g.n_inst; dev_end.push_back(nd); }
  if (grp.empty()) { grp.push_back({0, 0, 0, 0, 0, 0, 0}); dev_end.push_back(0); }
  auto pairs = [](const std::vector<int32_t> &a, const std::vector<int32_t> &b) {
    std::vector<int2> p(a.size()); for (size_t k = 0; k < a.size(); ++k) p[k] = make_int2(a[k], b[k]); return p;
  };
  std::vector<int2> lu_pair = pairs(H.lu_pair_a, H.lu_pair_b), fw_pair = pairs(H.fw_lu, H.fw_col), bw_pair = pairs(H.bw_lu, H.bw_col);
  std::vector<int> src_off, src_stride;
  for (size_t k = 0; k < H.src_group.size(); ++k) {
    const GroupInfo &g = H.groups[H.src_group[k]];
    src_off.push_back(g.dpar_off + H.src_inst[k]); src_stride.push_back(g.n_inst);
  }
  std::vector<int> src_of_dev(std::max(nd, 1), -1);
  for (size_t k = 0; k < H.src_group.size(); ++k) {
    int base = 0;
    for (int g = 0; g < H.src_group[k]; ++g) base += H.groups[g].n_inst;
    src_of_dev[base + H.src_inst[k]] = (int)k;
  }
  std::vector<int> gs_row(H.n_nodes), gs_col(H.n_nodes);
  for (int u = 0; u < H.n_nodes; ++u) { gs_row[u] = H.eq_pos[u]; gs_col[u] = H.iorder[u]; }
  Packer P;
  size_t o_grp = P.vec(grp), o_dev_end = P.vec(dev_end), o_term = P.vec(H.term_int), o_term_orig = P.vec(H.term_orig);
  size_t o_jlu_ptr = P.vec(H.jlu_ptr), o_jlu_ent = P.vec(H.jlu_ent), o_fint_ptr = P.vec(H.fint_ptr), o_fint_ent = P.vec(H.fint_ent);
  size_t o_qint_ptr = P.vec(H.qint_ptr), o_qint_ent = P.vec(H.qint_ent), o_jcsc_ptr = P.vec(H.jcsc_ptr), o_jcsc_ent = P.vec(H.jcsc_ent);
  size_t o_forg_ptr = P.vec(H.forg_ptr), o_forg_ent = P.vec(H.forg_ent);
  size_t o_lu_lvl = P.vec(H.lu_lvl_ptr), o_lu_slot = P.vec(H.lu_task_slot), o_lu_info = P.vec(H.lu_task_info), o_lu_pp = P.vec(H.lu_pair_ptr), o_lu_pair = P.vec(lu_pair);
  size_t o_fw_lvl = P.vec(H.fw_lvl_ptr), o_fw_row = P.vec(H.fw_row), o_fw_ptr = P.vec(H.fw_ptr), o_fw_pair = P.vec(fw_pair);
  size_t o_bw_lvl = P.vec(H.bw_lvl_ptr), o_bw_row = P.vec(H.bw_row), o_bw_ptr = P.vec(H.bw_ptr), o_bw_pair = P.vec(bw_pair);
  size_t o_src_of_dev = P.vec(src_of_dev);
  size_t o_src_off = P.vec(src_off), o_src_stride = P.vec(src_stride), o_gs_slot = P.vec(H.gs_slot), o_gs_row = P.vec(gs_row), o_gs_col = P.vec(gs_col);
  size_t o_is_node = P.vec(H.is_node_int), o_order = P.vec(H.order), o_iorder = P.vec(H.iorder), o_eq_pos = P.vec(H.eq_pos), o_pwl = P.vec(H.pwl);
  std::vector<int2> tf_pair = pairs(H.tf_lu, H.tf_col), tb_pair = pairs(H.tb_lu, H.tb_col), ct_ent = pairs(H.ct_ent, H.ct_row);
  size_t o_tf_lvl = P.vec(H.tf_lvl_ptr), o_tf_row = P.vec(H.tf_row), o_tf_ptr = P.vec(H.tf_ptr), o_tf_pair = P.vec(tf_pair);
  size_t o_tb_lvl = P.vec(H.tb_lvl_ptr), o_tb_row = P.vec(H.tb_row), o_tb_ptr = P.vec(H.tb_ptr), o_tb_pair = P.vec(tb_pair);
  size_t o_ct_ptr = P.vec(H.ct_ptr), o_ct_ent = P.vec(ct_ent), o_adj_goff = P.vec(H.adj_goff);
  size_t o_out_q = P.vec(H.out_q);
  std::vector<int> lu_cptr(H.n + 1, 0), lu_cslot(std::max(H.nnz_lu, 1)), lu_srow(std::max(H.nnz_lu, 1));
  for (int p = 0; p < H.n; ++p)
    for (int k = H.lu_rowptr[p]; k < H.lu_rowptr[p + 1]; ++k) { lu_srow[k] = p; ++lu_cptr[H.lu_colidx[k] + 1]; }
  for (int q = 0; q < H.n; ++q) lu_cptr[q + 1] += lu_cptr[q];
  {
    std::vector<int> fill(lu_cptr.begin(), lu_cptr.end() - 1);
    for (int p = 0; p < H.n; ++p)
      for (int k = H.lu_rowptr[p]; k < H.lu_rowptr[p + 1]; ++k) lu_cslot[fill[H.lu_colidx[k]]++] = k;
  }
  size_t o_lu_rowptr = P.vec(H.lu_rowptr), o_lu_colidx = P.vec(H.lu_colidx), o_lu_cptr = P.vec(lu_cptr);
  size_t o_lu_cslot = P.vec(lu_cslot), o_lu_srow = P.vec(lu_srow);
  std::vector<int> mg_grp;
  int mg_ptr[kNumModels + 1] = {0};
  for (int m = 0; m < kNumModels; ++m) {
    mg_ptr[m] = (int)mg_grp.size();
    for (size_t g = 0; g < H.groups.size(); ++g) if (H.groups[g].model == m) mg_grp.push_back((int)g);
  }
  mg_ptr[kNumModels] = (int)mg_grp.size();
  size_t o_mg_grp = P.vec(mg_grp);
  std::vector<int> eq_of_pos(H.n);
  for (int e = 0; e < H.n; ++e) eq_of_pos[H.eq_pos[e]] = e;
  std::vector<int2> lu_orig(std::max(H.nnz_lu, 1));
  for (int p = 0; p < H.n; ++p)
    for (int k = H.lu_rowptr[p]; k < H.lu_rowptr[p + 1]; ++k) lu_orig[k] = make_int2(eq_of_pos[p], H.order[H.lu_colidx[k]]);
  size_t o_lu_orig = P.vec(lu_orig);
  std::vector<int4> lu_task(std::max<size_t>(H.lu_task_slot.size(), 1));
  for (size_t t = 0; t < H.lu_task_slot.size(); ++t)
    lu_task[t] = make_int4(H.lu_task_slot[t], H.lu_task_info[t], H.lu_pair_ptr[t], H.lu_pair_ptr[t + 1]);
  auto row_tasks = [](const std::vector<int32_t> &row, const std::vector<int32_t> &ptr) {
    std::vector<int4> v(std::max<size_t>(row.size(), 1));
    for (size_t t = 0; t < row.size(); ++t) v[t] = make_int4(row[t], ptr[t], ptr[t + 1], 0);
    return v;
  };
  size_t o_lu_task = P.vec(lu_task), o_fw_task = P.vec(row_tasks(H.fw_row, H.fw_ptr)), o_bw_task = P.vec(row_tasks(H.bw_row, H.bw_ptr));
  size_t o_tf_task = P.vec(row_tasks(H.tf_row, H.tf_ptr)), o_tb_task = P.vec(row_tasks(H.tb_row, H.tb_ptr));
  size_t o_long_lu = P.vec(H.long_lu), o_long_fi = P.vec(H.long_fi), o_long_jc = P.vec(H.long_jc), o_long_fo = P.vec(H.long_fo);
  size_t o_long_off = P.vec(H.long_jc_fo_off);
  // long LU / substitution tasks per level
  auto long_tasks = [](const std::vector<int32_t> &lvl, const std::vector<int32_t> &ptr, std::vector<int> &lv_out,
                       std::vector<int> &task_out) {
    lv_out.assign(1, 0); task_out.clear();
    for (size_t l = 0; l + 1 < lvl.size(); ++l) {
      for (int t = lvl[l]; t < lvl[l + 1]; ++t) if (ptr[t + 1] - ptr[t] > kLongPairs) task_out.push_back(t);
      lv_out.push_back((int)task_out.size());
    }
    if (task_out.empty()) task_out.push_back(0);
  };
  std::vector<int> llu_l, llu_t, lfw_l, lfw_t, lbw_l, lbw_t, ltf_l, ltf_t, ltb_l, ltb_t;
  long_tasks(H.lu_lvl_ptr, H.lu_pair_ptr, llu_l, llu_t);
  long_tasks(H.fw_lvl_ptr, H.fw_ptr, lfw_l, lfw_t);
  long_tasks(H.bw_lvl_ptr, H.bw_ptr, lbw_l, lbw_t);
  long_tasks(H.tf_lvl_ptr, H.tf_ptr, ltf_l, ltf_t);
  long_tasks(H.tb_lvl_ptr, H.tb_ptr, ltb_l, ltb_t);
  size_t o_llu_l = P.vec(llu_l), o_llu_t = P.vec(llu_t), o_lfw_l = P.vec(lfw_l), o_lfw_t = P.vec(lfw_t);
  size_t o_lbw_l = P.vec(lbw_l), o_lbw_t = P.vec(lbw_t), o_ltf_l = P.vec(ltf_l), o_ltf_t = P.vec(ltf_t);
  size_t o_ltb_l = P.vec(ltb_l), o_ltb_t = P.vec(ltb_t);
  CUDA_TRY(cudaMalloc(&dt->buf, P.bytes.size()));
  CUDA_TRY(cudaMemcpy(dt->buf, P.bytes.data(), P.bytes.size(), cudaMemcpyHostToDevice));
  char *b = (char *)dt->buf;
  DTpl &D = dt->D;
  D.n = H.n; D.n_nodes = H.n_nodes; D.nnz_lu = H.nnz_lu; D.n_out = H.n_out; D.n_groups = (int)H.groups.size();
  D.n_dev = nd; D.n_src = (int)src_off.size(); D.lu_nlev = (int)H.lu_lvl_ptr.size() - 1;
  D.fw_nlev = (int)H.fw_lvl_ptr.size() - 1; D.bw_nlev = (int)H.bw_lvl_ptr.size() - 1; D.n_csc = (int)H.j_rowidx.size();
  D.dpar_size = H.dpar_size; D.gmin = H.gmin; D.vt = thermal_voltage(H.temp_c);
  D.grp = (const DGroup *)(b + o_grp); D.dev_end = (const int *)(b + o_dev_end);
  D.term = (const int *)(b + o_term); D.term_orig = (const int *)(b + o_term_orig);
  D.jlu_ptr = (const int *)(b + o_jlu_ptr); D.jlu_ent = (const int *)(b + o_jlu_ent);
  D.fint_ptr = (const int *)(b + o_fint_ptr); D.fint_ent = (const int *)(b + o_fint_ent);
  D.qint_ptr = (const int *)(b + o_qint_ptr); D.qint_ent = (const int *)(b + o_qint_ent);
  D.jcsc_ptr = (const int *)(b + o_jcsc_ptr); D.jcsc_ent = (const int *)(b + o_jcsc_ent);
  D.forg_ptr = (const int *)(b + o_forg_ptr); D.forg_ent = (const int *)(b + o_forg_ent);
  D.lu_lvl = (const int *)(b + o_lu_lvl); D.lu_slot = (const int *)(b + o_lu_slot); D.lu_info = (const int *)(b + o_lu_info);
  D.lu_pp = (const int *)(b + o_lu_pp); D.lu_pair = (const int2 *)(b + o_lu_pair);
  D.fw_lvl = (const int *)(b + o_fw_lvl); D.fw_row = (const int *)(b + o_fw_row); D.fw_ptr = (const int *)(b + o_fw_ptr); D.fw_pair = (const int2 *)(b + o_fw_pair);
  D.bw_lvl = (const int *)(b + o_bw_lvl); D.bw_row = (const int *)(b + o_bw_row); D.bw_ptr = (const int *)(b + o_bw_ptr); D.bw_pair = (const int2 *)(b + o_bw_pair);
  D.src_off = (const int *)(b + o_src_off); D.src_stride = (const int *)(b + o_src_stride);
  D.src_of_dev = (const int *)(b + o_src_of_dev);
  D.gs_slot = (const int *)(b + o_gs_slot); D.gs_row = (const int *)(b + o_gs_row); D.gs_col = (const int *)(b + o_gs_col);
  D.is_node = (const unsigned char *)(b + o_is_node); D.order = (const int *)(b + o_order); D.iorder = (const int *)(b + o_iorder);
  D.eq_pos = (const int *)(b + o_eq_pos); D.pwl = (const double *)(b + o_pwl);
  D.tf_nlev = (int)H.tf_lvl_ptr.size() - 1; D.tb_nlev = (int)H.tb_lvl_ptr.size() - 1; D.n_adj = H.n_adj;
  D.tf_lvl = (const int *)(b + o_tf_lvl); D.tf_row = (const int *)(b + o_tf_row); D.tf_ptr = (const int *)(b + o_tf_ptr); D.tf_pair = (const int2 *)(b + o_tf_pair);
  D.tb_lvl = (const int *)(b + o_tb_lvl); D.tb_row = (const int *)(b + o_tb_row); D.tb_ptr = (const int *)(b + o_tb_ptr); D.tb_pair = (const int2 *)(b + o_tb_pair);
  D.ct_ptr = (const int *)(b + o_ct_ptr); D.ct_ent = (const int2 *)(b + o_ct_ent); D.adj_goff = (const int *)(b + o_adj_goff);
  D.out_q = (const unsigned char *)(b + o_out_q);
  D.lu_rowptr = (const int *)(b + o_lu_rowptr); D.lu_colidx = (const int *)(b + o_lu_colidx);
  D.lu_cptr = (const int *)(b + o_lu_cptr); D.lu_cslot = (const int *)(b + o_lu_cslot); D.lu_srow = (const int *)(b + o_lu_srow);
  for (int m = 0; m <= kNumModels; ++m) D.mg_ptr[m] = mg_ptr[m];
  D.mg_grp = (const int *)(b + o_mg_grp);
  D.lu_orig = (const int2 *)(b + o_lu_orig);
  D.lu_task = (const int4 *)(b + o_lu_task); D.fw_task = (const int4 *)(b + o_fw_task); D.bw_task = (const int4 *)(b + o_bw_task);
  D.tf_task = (const int4 *)(b + o_tf_task); D.tb_task = (const int4 *)(b + o_tb_task);
  D.n_long_lu = (int)H.long_lu.size(); D.n_long_fi = (int)H.long_fi.size();
  D.n_long_jc = (int)H.long_jc.size(); D.n_long_fo = (int)H.long_fo.size();
  D.long_lu = (const int *)(b + o_long_lu); D.long_fi = (const int *)(b + o_long_fi);
  D.long_jc = (const int *)(b + o_long_jc); D.long_fo = (const int *)(b + o_long_fo);
  D.long_off = (const int *)(b + o_long_off); D.n_long_part = H.long_jc_fo_off.back();
  D.long_lu_lvl = (const int *)(b + o_llu_l); D.long_lu_task = (const int *)(b + o_llu_t);
  D.long_fw_lvl = (const int *)(b + o_lfw_l); D.long_fw_task = (const int *)(b + o_lfw_t);
  D.long_bw_lvl = (const int *)(b + o_lbw_l); D.long_bw_task = (const int *)(b + o_lbw_t);
  D.long_tf_lvl = (const int *)(b + o_ltf_l); D.long_tf_task = (const int *)(b + o_ltf_t);
  D.long_tb_lvl = (const int *)(b + o_ltb_l); D.long_tb_task = (const int *)(b + o_ltb_t);
  CUDA_TRY(cudaMalloc(&dt->D_dev, sizeof(DTpl)));
  CUDA_TRY(cudaMemcpy(dt->D_dev, &D, sizeof(DTpl), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMalloc(&dt->par_dev, std::max<size_t>(1, H.par.size()) * sizeof(double)));
  if (!H.par.empty()) CUDA_TRY(cudaMemcpy(dt->par_dev, H.par.data(), H.par.size() * sizeof(double), cudaMemcpyHostToDevice));
  out = std::move(dt);
  return 0;
}

EngOpts to_eng(const cedar_tran_opts *in) {
  cedar_tran_opts o = *in;
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
  EngOpts e;
  e.method = o.method; e.adaptive = o.adaptive; e.dcop = o.dcop; e.max_newton = o.max_newton; e.max_steps = o.max_steps;
  e.tstart = o.tstart; e.tstop = o.tstop; e.h = o.h; e.hmin = o.hmin; e.hmax = o.hmax; e.reltol = o.reltol;
  e.abstol_v = o.abstol_v; e.abstol_i = o.abstol_i; e.nr_factor = o.nr_factor; e.hfirst_frac = o.hfirst_frac;
  return e;
}

int check_opts(const cedar_tran_opts *o) {
  if (!o) return fail(CEDAR_EINVAL, "null options");
  if (!(o->tstop > o->tstart)) return fail(CEDAR_EINVAL, "tstop must exceed tstart");
  if (o->method != CEDAR_TRAP && o->method != CEDAR_BDF2) return fail(CEDAR_EINVAL, "unknown method");
  if (!o->adaptive && !(o->h > 0)) return fail(CEDAR_EINVAL, "fixed-step run needs h > 0");
  if (o->adaptive && o->method != CEDAR_BDF2) return fail(CEDAR_EUNSUPPORTED, "adaptive stepping is BDF2 only");
  return 0;
}

template <class T> struct DevBuf {
  T *p = nullptr; size_t n = 0;
  cudaError_t ensure(size_t m) {
    if (m <= n) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr; n = 0;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(m, 1) * sizeof(T));
    if (e == cudaSuccess) n = m;
    return e;
  }
  ~DevBuf() { if (p) cudaFree(p); }
};

}  // namespace

struct cedar_ckt {
  std::unique_ptr<DevTemplate> tpl;
  cudaStream_t stream = nullptr;
  DevBuf<double> dpar, x, xdot, F, J, dout, hist, ws, tout, xout, dense, part;
  DevBuf<EngStats> stats;
  DevBuf<long long> count;
  DevBuf<long long> off;
  // AC / noise: G and C per LU slot, inputs, outputs, per-warp complex workspaces
  DevBuf<double> ac_g, ac_c, ac_b, ac_omega, ac_out, ac_nw, ac_ne;
  DevBuf<double2> ac_ws, ac_dws;
  DevBuf<int> ac_probe, ac_status, ac_na, ac_nb, ac_ndense, ac_dpiv;
  cudaEvent_t ac_ev[4] = {nullptr, nullptr, nullptr, nullptr};   // sparse start / end, dense start / end
  int ac_last_dense = 0;
  bool ac_dense_ran = false;
  int threads = 128;
  int auto_threads = 128;   // the thread count chosen at create (CTA engine)
  int engine = CEDAR_ENGINE_AUTO;
  int device = -1;          // the CUDA device current at cedar_ckt_create
  bool host_only = false;
  // single-circuit transient on the one-warp engine: queue words, final state
  DevBuf<int> wq;
  DevBuf<double> xf;
  DevBuf<double> gred;      // grid engine: reduction scratch (6 doubles per block)
  cudaEvent_t run_ev[2] = {nullptr, nullptr};   // bracket the last single-circuit kernel
  bool run_timed = false;
  int last_blocks = 0;      // blocks of the last single-circuit kernel
  ~cedar_ckt() {
    for (cudaEvent_t e : run_ev) if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : ac_ev) if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
  }
};

struct cedar_batch {
  std::vector<std::unique_ptr<DevTemplate>> tpls;
  cudaStream_t stream = nullptr;
  DevBuf<DTpl> d_tpls;
  DevBuf<int> inst_tpl, queue, probes_int, qblk_beg, qblk_head;
  int n_qblk = 0;
  DevBuf<long long> raw_off, dpar_off, x0_off, dx_off;
  DevBuf<double> raw, dpar, x0, dx, samples, xfinal, ws, dense_ws;
  DevBuf<EngStats> stats;
  DevBuf<StateRow> rows;
  DevBuf<double> row_vec;
  DevBuf<int> n_running;
  int n_inst = 0, n_max = 0, np = 0, ns = 0, ws_stride = 0;
  bool has_x0 = false, has_dx = false;
  cedar_batch_tuning tune{};
  EngOpts run_opts{};   // options of the run in progress (cedar_batch_start)
  bool started = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // bracket the last batch launch
  bool timed = false;
  // discrete adjoint: tape, checkpoints, replayed segments, results
  DevBuf<double> tape_t, tape_p, tape_v, ckpt, segx, adj_phi, adj_grad, adj_tstar;
  DevBuf<signed char> tape_ord;
  DevBuf<int4> obj_idx;
  DevBuf<AdjObj> adj_obj;
  DevBuf<int> adj_status;
  cudaEvent_t ev2 = nullptr;   // end of the last adjoint's backward kernel
  bool adj_timed = false;
  long long tape_cap = 0;      // steps per instance of the last adjoint's tape
  ~cedar_batch() {
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (ev2) cudaEventDestroy(ev2);
    if (stream) cudaStreamDestroy(stream);
  }
};

extern "C" {

int cedar_last_error(char *buf, size_t len) {
  if (buf && len) std::snprintf(buf, len, "%s", g_err.c_str());
  return (int)g_err.size();
}
int cedar_version(void) { return 10000; }
int cedar_model_nterm(int m) { return (m > 0 && m < kNumModels) ? model_info(m).nterm : -1; }
int cedar_model_npar(int m) { return (m > 0 && m < kNumModels) ? model_info(m).npar : -1; }
int cedar_model_has_branch(int m) { return (m > 0 && m < kNumModels) ? model_info(m).has_br : -1; }
int cedar_va_count(void) { return va::kCount; }
int cedar_va_name(int k, char *buf, size_t len) {
  if (k < 0 || k >= va::kCount || !buf || len == 0) return fail(CEDAR_EINVAL, "Verilog-A model index out of range");
  std::snprintf(buf, len, "%s", va::kName[k]);
  return CEDAR_OK;
}

void cedar_tran_opts_default(cedar_tran_opts *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->method = CEDAR_BDF2; o->adaptive = 1; o->dcop = 1; o->max_newton = 20; o->max_steps = 100000000;
  o->tstart = 0; o->tstop = 0; o->h = 0; o->reltol = 1e-6; o->abstol_v = 1e-9; o->abstol_i = 1e-12;
  o->nr_factor = 1e-3; o->hfirst_frac = 1e-2;
}

int cedar_ckt_create(const cedar_ckt_desc *desc, cedar_ckt **out) {
  const Range nvtx_range("cedar_ckt_create");
  if (!desc || !out) return fail(CEDAR_EINVAL, "null argument");
  *out = nullptr;
  auto c = std::make_unique<cedar_ckt>();
  int rc = upload_template(desc, c->tpl);
  if (rc) return rc;
  CUDA_TRY(cudaGetDevice(&c->device));
  CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  const Template &H = c->tpl->H;
  CUDA_TRY(c->dpar.ensure(H.dpar_size));
  CUDA_TRY(c->off.ensure(2));
  long long zero[2] = {0, 0};
  CUDA_TRY(cudaMemcpyAsync(c->off.p, zero, sizeof(zero), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(launch_derive(c->tpl->D_dev, nullptr, c->off.p, c->tpl->par_dev, c->off.p + 1, c->dpar.p, 1, c->tpl->D.n_dev, c->stream));
  int n = H.n;
  CUDA_TRY(c->x.ensure(n)); CUDA_TRY(c->xdot.ensure(n)); CUDA_TRY(c->F.ensure(n)); CUDA_TRY(c->hist.ensure(n));
  CUDA_TRY(c->J.ensure(H.j_rowidx.size())); CUDA_TRY(c->dout.ensure(H.n_out));
  CUDA_TRY(c->part.ensure(std::max(1, H.long_jc_fo_off.back())));
  CUDA_TRY(c->stats.ensure(1)); CUDA_TRY(c->count.ensure(1));
  size_t wsd = ws_doubles(H.n, H.nnz_lu, H.n_out, (int)H.src_group.size());
  if ((wsd + 128) * sizeof(double) > 160 * 1024) CUDA_TRY(c->ws.ensure(wsd));
  int work = std::max(std::max(H.nnz_lu, n), c->tpl->D.n_dev);
  c->threads = work >= 512 ? 512 : std::max(64, ((work + 31) / 32) * 32);
  c->auto_threads = c->threads;
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  *out = c.release();
  return 0;
}

int cedar_plan_create(const cedar_ckt_desc *desc, cedar_ckt **out) {
  if (!desc || !out) return fail(CEDAR_EINVAL, "null argument");
  *out = nullptr;
  auto c = std::make_unique<cedar_ckt>();
  int rc = compile_only(desc, c->tpl);
  if (rc) return rc;
  c->host_only = true;
  *out = c.release();
  return 0;
}

int cedar_ckt_destroy(cedar_ckt *c) { delete c; return 0; }

int cedar_ckt_size(const cedar_ckt *c, int32_t *n, int32_t *nnz_j, int32_t *nnz_lu, int32_t *n_levels) {
  if (!c) return fail(CEDAR_EINVAL, "null handle");
  const Template &H = c->tpl->H;
  if (n) *n = H.n;
  if (nnz_j) *nnz_j = (int32_t)H.j_rowidx.size();
  if (nnz_lu) *nnz_lu = H.nnz_lu;
  if (n_levels) *n_levels = (int32_t)(H.lu_lvl_ptr.size() - 1);
  return 0;
}

// FP64 operations of one device evaluation in the engines' Newton iteration,
// counted at build time by running the device code (models.cuh and the emitted
// Verilog-A code) on an op-counting scalar (csrc/opcount.cpp -> flops.gen.h):
// add / sub / mul / div 1, FMA 2, exp / log / sqrt 1.
static int model_flops(int m) {
  if (m > 0 && m < CEDAR_NMODELS) return flops::kBuiltin[m];
  if (m >= va::kBase && m < kNumModels) return flops::kVA[m - va::kBase];
  return 0;
}

int cedar_ckt_costs(const cedar_ckt *c, cedar_costs *o) {
  if (!c || !o) return fail(CEDAR_EINVAL, "null argument");
  const Template &H = c->tpl->H;
  cedar_costs r{};
  int64_t dev_bytes = 0;
  for (const GroupInfo &g : H.groups) {
    const ModelInfo &mi = model_info(g.model);
    r.flops_eval += (int64_t)model_flops(g.model) * g.n_inst;
    dev_bytes += (int64_t)g.n_inst * (8 * mi.ndpar + 4 * g.ntx + 8 * g.ntx + 16 * mi.nout);
  }
  r.flops_stamp = (int64_t)H.jlu_ent.size() + (int64_t)H.fint_ent.size() + H.n;
  r.flops_lu = H.lu_flops;
  r.flops_solve = 2 * ((int64_t)H.fw_lu.size() + (int64_t)H.bw_lu.size()) + H.n;
  r.flops_update = 4 * (int64_t)H.n;
  r.bytes = dev_bytes + 4 * (int64_t)(H.jlu_ent.size() + H.fint_ent.size()) + 16 * (int64_t)H.nnz_lu +
            8 * 2 * (int64_t)H.lu_pair_a.size() + 8 * 2 * (int64_t)(H.fw_lu.size() + H.bw_lu.size()) + 8 * 6 * (int64_t)H.n;
  {
    int64_t eb = 0;
    for (const GroupInfo &g : H.groups) {
      const ModelInfo &mi = model_info(g.model);
      eb += (int64_t)g.n_inst * (8 * mi.ndpar + 4 * g.ntx + 8 * g.ntx + 8 * mi.nout);
    }
    const int64_t ent = (int64_t)H.jcsc_ent.size() + (int64_t)H.forg_ent.size();
    const int64_t ncsc = (int64_t)H.j_rowidx.size();
    r.bytes_eval = eb + 12 * ent + 4 * (ncsc + 1 + H.n + 1) + 8 * (ncsc + H.n);
  }
  r.lu_levels = (int32_t)H.lu_lvl_ptr.size() - 1;
  r.fw_levels = (int32_t)H.fw_lvl_ptr.size() - 1;
  r.bw_levels = (int32_t)H.bw_lvl_ptr.size() - 1;
  r.nnz_lu = H.nnz_lu;
  r.ordering = H.ordering;
  *o = r;
  return 0;
}

int cedar_ckt_pattern(const cedar_ckt *c, int32_t *colptr, int32_t *rowidx) {
  if (!c) return fail(CEDAR_EINVAL, "null handle");
  const Template &H = c->tpl->H;
  if (colptr) std::memcpy(colptr, H.j_colptr.data(), H.j_colptr.size() * sizeof(int32_t));
  if (rowidx) std::memcpy(rowidx, H.j_rowidx.data(), H.j_rowidx.size() * sizeof(int32_t));
  return 0;
}

int cedar_ckt_symbolic(const cedar_ckt *c, int32_t *rowmatch, int32_t *order, int32_t *lu_colptr, int32_t *lu_rowidx) {
  if (!c) return fail(CEDAR_EINVAL, "null handle");
  const Template &H = c->tpl->H;
  if (rowmatch) std::memcpy(rowmatch, H.rowmatch.data(), H.n * sizeof(int32_t));
  if (order) std::memcpy(order, H.order.data(), H.n * sizeof(int32_t));
  if (lu_colptr || lu_rowidx) {
    std::vector<int32_t> cp(H.n + 1, 0), ri(H.nnz_lu);
    for (int p = 0; p < H.n; ++p) for (int k = H.lu_rowptr[p]; k < H.lu_rowptr[p + 1]; ++k) cp[H.lu_colidx[k] + 1]++;
    for (int q = 0; q < H.n; ++q) cp[q + 1] += cp[q];
    std::vector<int32_t> fillp(cp.begin(), cp.end() - 1);
    for (int p = 0; p < H.n; ++p) for (int k = H.lu_rowptr[p]; k < H.lu_rowptr[p + 1]; ++k) ri[fillp[H.lu_colidx[k]]++] = p;
    if (lu_colptr) std::memcpy(lu_colptr, cp.data(), cp.size() * sizeof(int32_t));
    if (lu_rowidx) std::memcpy(lu_rowidx, ri.data(), ri.size() * sizeof(int32_t));
  }
  return 0;
}

int cedar_ckt_stream(const cedar_ckt *c, void **stream) {
  if (!c || !stream) return fail(CEDAR_EINVAL, "null argument");
  *stream = static_cast<void *>(c->stream);
  return 0;
}

int cedar_eval_dev(cedar_ckt *c, const double *x, const double *xdot, double t, double cj, double *F, double *J) {
  const Range nvtx_range("cedar_eval_dev");
  if (!c || !x) return fail(CEDAR_EINVAL, "null argument");
  if (c->host_only) return fail(CEDAR_EINVAL, "host-only plan handle");
  CUDA_TRY(launch_eval(c->tpl->D, c->tpl->D_dev, c->dpar.p, x, xdot, t, cj, c->dout.p, c->part.p, F, J, c->stream));
  return 0;
}

int cedar_eval_scratch(const cedar_ckt *c, int64_t *n_out, int64_t *n_part, int64_t *limit) {
  if (limit) *limit = kEvalScratchMax;
  if (!c) return (n_out || n_part) ? fail(CEDAR_EINVAL, "null handle") : 0;
  const Template &H = c->tpl->H;
  if (n_out) *n_out = H.n_out;
  if (n_part) *n_part = H.long_jc_fo_off.empty() ? 0 : H.long_jc_fo_off.back();
  return 0;
}

int cedar_eval_dev_noalloc(cedar_ckt *c, const double *x, const double *xdot, double t, double cj, double *F,
                           double *J, void *stream) {
  if (!c || !x) return fail(CEDAR_EINVAL, "null argument");
  if (c->host_only) return fail(CEDAR_EINVAL, "host-only plan handle");
  const DTpl &T = c->tpl->D;
  if ((long long)T.n_out + T.n_long_part > kEvalScratchMax)
    return fail(CEDAR_EINVAL, "circuit needs " + std::to_string((long long)T.n_out + T.n_long_part) +
                " doubles of evaluation scratch (device outputs and long-row partial sums); the allocation-free "
                "evaluation holds at most " + std::to_string(kEvalScratchMax));
  // the scratch address is per device: the handle's device must be current, and
  // a caller's stream must belong to it
  int dev = -1;
  CUDA_TRY(cudaGetDevice(&dev));
  if (dev != c->device)
    return fail(CEDAR_EINVAL, "the current device (" + std::to_string(dev) + ") is not the handle's device (" +
                std::to_string(c->device) + "); make the handle's device current before the call");
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  if (stream) {
    int sdev = -1;
    CUDA_TRY(cudaStreamGetDevice(s, &sdev));
    if (sdev != c->device)
      return fail(CEDAR_EINVAL, "the stream belongs to device " + std::to_string(sdev) + ", the handle to device " +
                  std::to_string(c->device));
  }
  double *scratch = nullptr;
  CUDA_TRY(eval_scratch_address(&scratch));
  CUDA_TRY(launch_eval(T, c->tpl->D_dev, c->dpar.p, x, xdot, t, cj, scratch, scratch + T.n_out, F, J, s));
  return 0;
}

int cedar_eval(cedar_ckt *c, const double *x, const double *xdot, double t, double cj, double *F, double *J) {
  const Range nvtx_range("cedar_eval");
  if (!c || !x) return fail(CEDAR_EINVAL, "null argument");
  if (c->host_only) return fail(CEDAR_EINVAL, "host-only plan handle");
  const Template &H = c->tpl->H;
  size_t n = H.n, nj = H.j_rowidx.size();
  CUDA_TRY(cudaMemcpyAsync(c->x.p, x, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (xdot) CUDA_TRY(cudaMemcpyAsync(c->xdot.p, xdot, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(launch_eval(c->tpl->D, c->tpl->D_dev, c->dpar.p, c->x.p, xdot ? c->xdot.p : nullptr, t, cj, c->dout.p,
                       c->part.p, F ? c->F.p : nullptr, J ? c->J.p : nullptr, c->stream));
  if (F) CUDA_TRY(cudaMemcpyAsync(F, c->F.p, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (J) CUDA_TRY(cudaMemcpyAsync(J, c->J.p, nj * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return 0;
}

// Circuits at least this large run on the grid engine by default (one CTA
// would walk their devices, slots and level tasks hundreds of times per phase).
constexpr int kGridMinN = 4096;
static bool use_grid(const Template &H) { return H.n >= kGridMinN; }

static int run_plain(cedar_ckt *c, int mode, const cedar_tran_opts *opts, double t, double cj, const double *hist,
                     double *x, double *t_out, double *x_out, int64_t cap, int64_t *n_out, cedar_stats *stats) {
  if (c->host_only) return fail(CEDAR_EINVAL, "host-only plan handle");
  const Template &H = c->tpl->H;
  size_t n = H.n;
  PlainArgs a{};
  a.T = c->tpl->D_dev; a.dpar = c->dpar.p; a.x = c->x.p; a.t = t; a.cj = cj; a.mode = mode;
  if (n <= 1024) {  // dense DC fallback scratch: (n + 2) n doubles
    CUDA_TRY(c->dense.ensure((n + 2) * n));
    a.dense = c->dense.p;
  }
  cedar_tran_opts od; cedar_tran_opts_default(&od);
  if (opts) od = *opts; else { od.tstart = 0; od.tstop = 1; }
  a.opts = to_eng(&od);
  CUDA_TRY(cudaMemcpyAsync(c->x.p, x, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (hist) { CUDA_TRY(cudaMemcpyAsync(c->hist.p, hist, n * sizeof(double), cudaMemcpyHostToDevice, c->stream)); a.hist = c->hist.p; }
  if (mode == 0 && t_out && cap > 0) {
    CUDA_TRY(c->tout.ensure(cap)); CUDA_TRY(c->xout.ensure((size_t)cap * n));
    a.t_out = c->tout.p; a.x_out = c->xout.p; a.cap = cap;
  }
  a.count = c->count.p; a.stats = c->stats.p; a.ws_global = c->ws.p;
  const int wsd = ws_doubles(H.n, H.nnz_lu, H.n_out, (int)H.src_group.size());
  const bool grid = c->engine == CEDAR_ENGINE_GRID || (c->engine == CEDAR_ENGINE_AUTO && use_grid(H));
  int blocks = 1;
  if (grid) {
    CUDA_TRY(grid_geometry(std::max(std::max(H.nnz_lu, (int)n), c->tpl->D.n_dev), &blocks));
    CUDA_TRY(c->ws.ensure(wsd));
    CUDA_TRY(c->gred.ensure((size_t)6 * blocks));
    a.ws_global = c->ws.p;
    a.dense = nullptr;                 // the dense DC fallback is a one-block algorithm
  }
  if (!c->run_ev[0]) { CUDA_TRY(cudaEventCreate(&c->run_ev[0])); CUDA_TRY(cudaEventCreate(&c->run_ev[1])); }
  CUDA_TRY(cudaEventRecord(c->run_ev[0], c->stream));
  if (grid) CUDA_TRY(launch_plain_grid(a, blocks, c->gred.p, c->stream));
  else CUDA_TRY(launch_plain(a, wsd, c->threads, c->stream));
  CUDA_TRY(cudaEventRecord(c->run_ev[1], c->stream));
  c->last_blocks = blocks;
  c->run_timed = true;
  EngStats st{}; long long cnt = 0;
  CUDA_TRY(cudaMemcpyAsync(&st, c->stats.p, sizeof(st), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaMemcpyAsync(&cnt, c->count.p, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaMemcpyAsync(x, c->x.p, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (mode == 0 && a.t_out) {
    long long m = std::min<long long>(cnt, cap);
    CUDA_TRY(cudaMemcpy(t_out, c->tout.p, m * sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(x_out, c->xout.p, (size_t)m * n * sizeof(double), cudaMemcpyDeviceToHost));
  }
  if (n_out) *n_out = cnt;
  if (stats) std::memcpy(stats, &st, sizeof(st));
  if (mode == 0 && t_out && cnt > cap) return fail(CEDAR_ECAPACITY, "output capacity exceeded");
  if (mode != 0 && st.status != CEDAR_ST_OK) return fail(CEDAR_ENOCONV, "Newton / DC operating point did not converge");
  return 0;
}

int cedar_newton_solve(cedar_ckt *c, double t, double cj, const double *hist, double *x, cedar_stats *stats) {
  const Range nvtx_range("cedar_newton_solve");
  if (!c || !x) return fail(CEDAR_EINVAL, "null argument");
  return run_plain(c, 1, nullptr, t, cj, hist, x, nullptr, nullptr, 0, nullptr, stats);
}

int cedar_dcop(cedar_ckt *c, double t, double *x, cedar_stats *stats) {
  const Range nvtx_range("cedar_dcop");
  if (!c || !x) return fail(CEDAR_EINVAL, "null argument");
  return run_plain(c, 2, nullptr, t, 0.0, nullptr, x, nullptr, nullptr, 0, nullptr, stats);
}

// Largest workspace (doubles) the one-warp engine takes (its workspace is in
// shared memory).  The CTA engine is the default for one circuit: on the RC
// ladder and the 31-stage chain it took 0.59x and 0.72x the one-warp engine's time
// (its levels run on more lanes), so the one-warp engine is an explicit choice.
constexpr int kWarpTranMaxWs = 24 * 1024;

// The single-circuit transient on the batched engine's slot state machine, one
// warp, one instance, every accepted point recorded (the same step control,
// Newton iteration and DC homotopy as every batched instance).
static int run_tran_warp(cedar_ckt *c, const cedar_tran_opts *opts, double *x, double *t_out, double *x_out,
                         int64_t cap, int64_t *n_out, cedar_stats *stats) {
  const Template &H = c->tpl->H;
  const int n = H.n;
  const int wsd = ws_doubles(H.n, H.nnz_lu, H.n_out, (int)H.src_group.size());
  CUDA_TRY(c->wq.ensure(8));
  CUDA_TRY(c->xf.ensure(n));
  // words: [0] inst_tpl, [1] queue, [2..3] qblk_beg, [4] qblk_head, [5] n_running
  const int words[8] = {0, 0, 0, 1, 0, 0, 0, 0};
  CUDA_TRY(cudaMemcpyAsync(c->wq.p, words, sizeof(words), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemcpyAsync(c->x.p, x, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemsetAsync(c->count.p, 0, sizeof(long long), c->stream));
  const bool rec = t_out && x_out && cap > 0;
  if (rec) { CUDA_TRY(c->tout.ensure(cap)); CUDA_TRY(c->xout.ensure((size_t)cap * n)); }
  const long long dstride = (long long)(n + 2) * n;
  const bool dense_ok = n <= 256;
  if (dense_ok) CUDA_TRY(c->dense.ensure(dstride));
  BatchDev bd{};
  bd.tpls = c->tpl->D_dev; bd.inst_tpl = c->wq.p; bd.inst_dpar = c->off.p; bd.dpar = c->dpar.p;
  bd.x0_off = c->off.p; bd.x0 = c->x.p;                 // off.p[0] == 0: the state copied above
  bd.x_final = c->xf.p; bd.n_max = n; bd.stats = c->stats.p;
  bd.queue = c->wq.p + 1; bd.qblk_beg = c->wq.p + 2; bd.qblk_head = c->wq.p + 4; bd.n_qblk = 1; bd.n_inst = 1;
  bd.n_running = c->wq.p + 5;
  bd.opts = to_eng(opts);
  bd.ws_stride = wsd;
  bd.ws_in_smem = 1;
  bd.t_until = 1e300;
  bd.dense_ws = dense_ok ? c->dense.p : nullptr; bd.dense_stride = dstride; bd.dense_nmax = 256;
  bd.rec_t = rec ? c->tout.p : nullptr; bd.rec_x = rec ? c->xout.p : nullptr; bd.rec_cap = rec ? cap : 0;
  bd.rec_count = c->count.p;
  if (!c->run_ev[0]) { CUDA_TRY(cudaEventCreate(&c->run_ev[0])); CUDA_TRY(cudaEventCreate(&c->run_ev[1])); }
  CUDA_TRY(cudaEventRecord(c->run_ev[0], c->stream));
  CUDA_TRY(launch_batch_record(bd, (size_t)wsd * sizeof(double), c->stream));
  CUDA_TRY(cudaEventRecord(c->run_ev[1], c->stream));
  c->run_timed = true;
  EngStats st{}; long long cnt = 0;
  CUDA_TRY(cudaMemcpyAsync(&st, c->stats.p, sizeof(st), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaMemcpyAsync(&cnt, c->count.p, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaMemcpyAsync(x, c->xf.p, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (rec) {
    const long long m = std::min<long long>(cnt, cap);
    CUDA_TRY(cudaMemcpy(t_out, c->tout.p, m * sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(x_out, c->xout.p, (size_t)m * n * sizeof(double), cudaMemcpyDeviceToHost));
  }
  if (n_out) *n_out = rec ? cnt : 0;
  if (stats) std::memcpy(stats, &st, sizeof(st));
  if (rec && cnt > cap) return fail(CEDAR_ECAPACITY, "output capacity exceeded");
  return 0;
}

int cedar_tran_run(cedar_ckt *c, const cedar_tran_opts *opts, const double *x0, double *t_out, double *x_out,
                   int64_t cap, int64_t *n_out, cedar_stats *stats) {
  const Range nvtx_range("cedar_tran_run");
  if (!c || !x0) return fail(CEDAR_EINVAL, "null argument");
  int rc = check_opts(opts); if (rc) return rc;
  if (c->host_only) return fail(CEDAR_EINVAL, "host-only plan handle");
  const Template &H = c->tpl->H;
  std::vector<double> x(x0, x0 + H.n);
  const bool fits = ws_doubles(H.n, H.nnz_lu, H.n_out, (int)H.src_group.size()) <= kWarpTranMaxWs;
  if (c->engine == CEDAR_ENGINE_WARP) {
    if (!fits) return fail(CEDAR_EINVAL, "circuit workspace exceeds the one-warp engine's shared memory");
    return run_tran_warp(c, opts, x.data(), t_out, x_out, cap, n_out, stats);
  }
  return run_plain(c, 0, opts, opts->tstart, 0.0, nullptr, x.data(), t_out, x_out, cap, n_out, stats);
}

int cedar_ckt_set_engine(cedar_ckt *c, int32_t engine, int32_t threads) {
  if (!c) return fail(CEDAR_EINVAL, "null handle");
  if (engine < CEDAR_ENGINE_AUTO || engine > CEDAR_ENGINE_GRID) return fail(CEDAR_EINVAL, "unknown engine");
  if (threads < 0 || threads > 1024 || threads % 32) return fail(CEDAR_EINVAL, "threads must be 0 or a multiple of 32 up to 1024");
  c->engine = engine;
  c->threads = threads ? threads : c->auto_threads;
  return 0;
}

int cedar_ckt_last_blocks(const cedar_ckt *c, int32_t *blocks) {
  if (!c || !blocks) return fail(CEDAR_EINVAL, "null argument");
  *blocks = c->last_blocks;
  return 0;
}

int cedar_ckt_last_ms(cedar_ckt *c, double *ms) {
  if (!c || !ms) return fail(CEDAR_EINVAL, "null argument");
  if (!c->run_timed) return fail(CEDAR_EINVAL, "no single-circuit run recorded yet");
  CUDA_TRY(cudaEventSynchronize(c->run_ev[1]));
  float f = 0; CUDA_TRY(cudaEventElapsedTime(&f, c->run_ev[0], c->run_ev[1]));
  *ms = f;
  return 0;
}

// ------------------------------------------------------------------ AC / noise
namespace {
constexpr size_t kAcWsBudget = size_t(1) << 30;   // bytes of per-warp workspaces at most
constexpr int kAcWarpsPerSm = 16;
// one lane per frequency up to this many complex workspace values per frequency
// (LU values + 3 n), with up to this many warps per SM (the lanes' dependent
// loads are hidden by warps: on the 100-section RC ladder 4, 16 and 32 warps per SM
// gave 15.5, 24.4 and 27.2 M frequency points/s), in at most twice kAcWsBudget
constexpr int kAcLaneMaxPer = 8192;
constexpr int kAcLaneWarpsPerSm = 32;

// G and C per LU slot at x_op, the frequencies, and the workspaces of the warps
// that will take them; fills everything of `a` but the analysis' own inputs.
int ac_prepare(cedar_ckt *c, const double *x_op, int32_t n_freq, const double *omega, AcDev &a) {
  const Template &H = c->tpl->H;
  const DTpl &D = c->tpl->D;
  const size_t n = H.n, nlu = std::max(H.nnz_lu, 1);
  CUDA_TRY(cudaMemcpyAsync(c->x.p, x_op, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(launch_eval(D, c->tpl->D_dev, c->dpar.p, c->x.p, nullptr, 0.0, 1.0, c->dout.p, c->part.p, nullptr, nullptr,
                       c->stream));
  CUDA_TRY(c->ac_g.ensure(nlu)); CUDA_TRY(c->ac_c.ensure(nlu));
  CUDA_TRY(launch_ac_split(D, c->dout.p, c->ac_g.p, c->ac_c.p, c->stream));
  CUDA_TRY(c->ac_omega.ensure(n_freq)); CUDA_TRY(c->ac_status.ensure(n_freq));
  CUDA_TRY(cudaMemcpyAsync(c->ac_omega.p, omega, n_freq * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  int dev = 0, sms = 1;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const size_t per = (size_t)H.nnz_lu + 3 * n;
  // one lane per frequency when a frequency's workspace is small (32 of them per
  // warp, interleaved), else one warp per frequency
  const bool lane = per <= (size_t)kAcLaneMaxPer;
  const size_t per_warp = lane ? 32 * per : per;
  const long long units = lane ? ((long long)n_freq + 31) / 32 : (long long)n_freq;
  long long nw = std::min<long long>(units, (long long)sms * (lane ? kAcLaneWarpsPerSm : kAcWarpsPerSm));
  nw = std::min<long long>(nw, std::max<long long>(1, (long long)((lane ? 2 * kAcWsBudget : kAcWsBudget) /
                                                                    (per_warp * sizeof(double2)))));
  CUDA_TRY(c->ac_ws.ensure((size_t)nw * per_warp));
  a.T = D; a.gval = c->ac_g.p; a.cval = c->ac_c.p; a.omega = c->ac_omega.p; a.n_freq = n_freq;
  a.ws = c->ac_ws.p; a.ws_stride = (long long)per; a.n_warps = nw; a.status = c->ac_status.p;
  a.lane_mode = lane ? 1 : 0;
  CUDA_TRY(c->ac_ndense.ensure(1));
  a.n_dense = c->ac_ndense.p;
  return 0;
}

// Sparse solves of every frequency, then the dense rerun of those whose static
// pivots failed or whose residual check did not pass.  Frequencies still marked
// kAcDense afterwards (system above kAcDenseNmax) are reported as zero pivots.
int ac_run(cedar_ckt *c, AcDev &a, bool noise, int32_t *status) {
  const Template &H = c->tpl->H;
  for (cudaEvent_t &e : c->ac_ev) if (!e) CUDA_TRY(cudaEventCreate(&e));
  CUDA_TRY(cudaMemsetAsync(a.n_dense, 0, sizeof(int), c->stream));
  CUDA_TRY(cudaEventRecord(c->ac_ev[0], c->stream));
  CUDA_TRY(launch_ac(a, noise, c->stream));
  CUDA_TRY(cudaEventRecord(c->ac_ev[1], c->stream));
  int nd = 0;
  CUDA_TRY(cudaMemcpyAsync(&nd, a.n_dense, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->ac_last_dense = nd;
  c->ac_dense_ran = false;
  if (nd > 0 && H.n <= kAcDenseNmax) {
    int dev = 0, sms = 1;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t per = (size_t)H.n * H.n + H.n;
    long long nw = std::min<long long>(nd, (long long)sms * 4);
    nw = std::min<long long>(nw, std::max<long long>(1, (long long)((size_t(1) << 28) / (per * sizeof(double2)))));
    CUDA_TRY(c->ac_dws.ensure((size_t)nw * per)); CUDA_TRY(c->ac_dpiv.ensure((size_t)nw * H.n));
    a.dws = c->ac_dws.p; a.dws_stride = (long long)per; a.dpiv = c->ac_dpiv.p; a.n_dwarps = nw;
    CUDA_TRY(cudaEventRecord(c->ac_ev[2], c->stream));
    CUDA_TRY(launch_ac_dense(a, noise, c->stream));
    CUDA_TRY(cudaEventRecord(c->ac_ev[3], c->stream));
    c->ac_dense_ran = true;
  }
  if (status) {
    CUDA_TRY(cudaMemcpyAsync(status, a.status, a.n_freq * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    for (long long f = 0; f < a.n_freq; ++f) if (status[f] == kAcDense) status[f] = CEDAR_ST_ZERO_PIVOT;
  }
  return 0;
}
}  // namespace

int cedar_ac(cedar_ckt *c, const double *x_op, const double *b, int32_t n_freq, const double *omega,
             int32_t n_probe, const int32_t *probe, double *resp, int32_t *status) {
  const Range nvtx_range("cedar_ac");
  if (!c || !x_op || !b || (n_freq > 0 && (!omega || !resp)) || !probe) return fail(CEDAR_EINVAL, "null argument");
  if (c->host_only) return fail(CEDAR_EINVAL, "host-only plan handle");
  if (n_freq < 0 || n_probe <= 0) return fail(CEDAR_EINVAL, "n_freq must be >= 0 and n_probe > 0");
  const Template &H = c->tpl->H;
  for (int k = 0; k < n_probe; ++k)
    if (probe[k] < 0 || probe[k] >= H.n) return fail(CEDAR_EINVAL, "probe outside the unknowns");
  if (n_freq == 0) return 0;
  AcDev a{};
  int rc = ac_prepare(c, x_op, n_freq, omega, a);
  if (rc) return rc;
  CUDA_TRY(c->ac_b.ensure(H.n)); CUDA_TRY(c->ac_probe.ensure(n_probe));
  CUDA_TRY(c->ac_out.ensure((size_t)n_freq * n_probe * 2));
  CUDA_TRY(cudaMemcpyAsync(c->ac_b.p, b, H.n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CUDA_TRY(cudaMemcpyAsync(c->ac_probe.p, probe, n_probe * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  a.b = c->ac_b.p; a.probe = c->ac_probe.p; a.n_probe = n_probe; a.resp = c->ac_out.p;
  rc = ac_run(c, a, false, status);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(resp, c->ac_out.p, (size_t)n_freq * n_probe * 2 * sizeof(double), cudaMemcpyDeviceToHost,
                           c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return 0;
}

int cedar_noise(cedar_ckt *c, const double *x_op, int32_t n_freq, const double *omega, int32_t probe, double *psd,
                int32_t *status) {
  const Range nvtx_range("cedar_noise");
  if (!c || !x_op || (n_freq > 0 && (!omega || !psd))) return fail(CEDAR_EINVAL, "null argument");
  if (c->host_only) return fail(CEDAR_EINVAL, "host-only plan handle");
  const Template &H = c->tpl->H;
  if (n_freq < 0) return fail(CEDAR_EINVAL, "n_freq must be >= 0");
  if (probe < 0 || probe >= H.n) return fail(CEDAR_EINVAL, "probe outside the unknowns");
  if (n_freq == 0) return 0;
  // thermal noise current of every resistor: terminals and weight m^2 4 k T / r
  std::vector<int> na, nb;
  std::vector<double> nw, ne;
  const double kT4 = 4.0 * 1.380649e-23 * (H.temp_c + 273.15);
  for (const GroupInfo &g : H.groups) {
    if (g.model != CEDAR_R) continue;
    for (int i = 0; i < g.n_inst; ++i) {
      const double r = H.par[g.par_off + i], m = H.par[g.par_off + g.n_inst + i];
      na.push_back(H.term_orig[g.term_off + (size_t)i * g.ntx]);
      nb.push_back(H.term_orig[g.term_off + (size_t)i * g.ntx + 1]);
      nw.push_back(m * m * kT4 / r);
      ne.push_back(0.0);
    }
  }
  // white_noise / flicker_noise sources of Verilog-A devices: their powers and
  // exponents at x_op from the emitted device code run on the host, weight
  // m^2 pwr (the contribution is scaled by m, src/simulate_ir.jl:54) over
  // f^exponent (src/ac.jl:267-276), across the contribution's branch
  const double vt = thermal_voltage(H.temp_c);
  for (const GroupInfo &g : H.groups) {
    const int k = g.model - va::kBase;
    if (k < 0 || k >= va::kCount) continue;
    const int n0 = va::kNoisePtr[k], nn = va::kNoisePtr[k + 1] - n0;
    if (nn == 0) continue;
    const int np = va::kNPar[k];
    std::vector<double> dp(np + 1), pw(nn), ex(nn);
    double v[8] = {0};
    for (int i = 0; i < g.n_inst; ++i) {
      for (int q = 0; q < np; ++q) dp[q] = H.par[g.par_off + (size_t)q * g.n_inst + i];
      dp[np] = vt;
      const int *t = &H.term_orig[g.term_off + (size_t)i * g.ntx];
      for (int q = 0; q < g.ntx && q < 8; ++q) v[q] = t[q] < 0 ? 0.0 : x_op[t[q]];
      va::noise(k, dp.data(), 1, v, H.gmin, pw.data(), ex.data());
      const double m = dp[np - 1];
      for (int j = 0; j < nn; ++j) {
        const int pa = va::kNoise[2 * (n0 + j)], pb = va::kNoise[2 * (n0 + j) + 1];
        na.push_back(t[pa]);
        nb.push_back(pb >= 0 ? t[pb] : -1);
        nw.push_back(m * m * pw[j]);
        ne.push_back(ex[j]);
      }
    }
  }
  AcDev a{};
  int rc = ac_prepare(c, x_op, n_freq, omega, a);
  if (rc) return rc;
  const size_t nr = na.size();
  CUDA_TRY(c->ac_na.ensure(std::max<size_t>(nr, 1))); CUDA_TRY(c->ac_nb.ensure(std::max<size_t>(nr, 1)));
  CUDA_TRY(c->ac_nw.ensure(std::max<size_t>(nr, 1))); CUDA_TRY(c->ac_probe.ensure(1));
  CUDA_TRY(c->ac_out.ensure(n_freq));
  if (nr) {
    CUDA_TRY(cudaMemcpyAsync(c->ac_na.p, na.data(), nr * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->ac_nb.p, nb.data(), nr * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->ac_nw.p, nw.data(), nr * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  }
  CUDA_TRY(cudaMemcpyAsync(c->ac_probe.p, &probe, sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  a.probe = c->ac_probe.p; a.n_probe = 1; a.psd = c->ac_out.p;
  a.n_noise = (int)nr; a.noise_a = c->ac_na.p; a.noise_b = c->ac_nb.p; a.noise_w = c->ac_nw.p;
  a.noise_e = nullptr;
  if (std::any_of(ne.begin(), ne.end(), [](double e) { return e != 0.0; })) {
    CUDA_TRY(c->ac_ne.ensure(nr));
    CUDA_TRY(cudaMemcpyAsync(c->ac_ne.p, ne.data(), nr * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    a.noise_e = c->ac_ne.p;
  }
  rc = ac_run(c, a, true, status);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(psd, c->ac_out.p, n_freq * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  return 0;
}

int cedar_ac_last_stats(const cedar_ckt *c, int32_t *n_dense, double *ms_sparse, double *ms_dense) {
  if (!c) return fail(CEDAR_EINVAL, "null argument");
  if (n_dense) *n_dense = c->ac_last_dense;
  float a = 0.f, b = 0.f;
  if (c->ac_ev[0]) {
    CUDA_TRY(cudaEventSynchronize(c->ac_ev[1]));
    CUDA_TRY(cudaEventElapsedTime(&a, c->ac_ev[0], c->ac_ev[1]));
    if (c->ac_dense_ran) {
      CUDA_TRY(cudaEventSynchronize(c->ac_ev[3]));
      CUDA_TRY(cudaEventElapsedTime(&b, c->ac_ev[2], c->ac_ev[3]));
    }
  }
  if (ms_sparse) *ms_sparse = a;
  if (ms_dense) *ms_dense = b;
  return 0;
}

// ------------------------------------------------------------------ batch
int cedar_batch_create(const cedar_batch_desc *d, cedar_batch **out) {
  const Range nvtx_range("cedar_batch_create");
  if (!d || !out) return fail(CEDAR_EINVAL, "null argument");
  *out = nullptr;
  if (d->n_templates <= 0 || d->n_inst < 0 || !d->templates || (d->n_inst > 0 && !d->inst_template))
    return fail(CEDAR_EINVAL, "malformed batch description");
  auto b = std::make_unique<cedar_batch>();
  CUDA_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  std::vector<DTpl> hd;
  for (int k = 0; k < d->n_templates; ++k) {
    std::unique_ptr<DevTemplate> t;
    int rc = upload_template(&d->templates[k], t);
    if (rc) return rc;
    b->n_max = std::max(b->n_max, t->H.n);
    b->ws_stride = std::max(b->ws_stride, ws_doubles(t->H.n, t->H.nnz_lu, t->H.n_out, (int)t->H.src_group.size()));
    hd.push_back(t->D);
    b->tpls.push_back(std::move(t));
  }
  // slot workspaces start 8 doubles (64 B) past a 128-B multiple apart, so the
  // slots of a warp touching the same offset fall in different shared-memory banks
  b->ws_stride = ((b->ws_stride + 15) / 16) * 16 + 8;
  const int ni = d->n_inst;
  b->n_inst = ni;
  CUDA_TRY(b->d_tpls.ensure(hd.size()));
  CUDA_TRY(cudaMemcpy(b->d_tpls.p, hd.data(), hd.size() * sizeof(DTpl), cudaMemcpyHostToDevice));
  // raw parameter blocks: user blocks first, then nominal blocks per template
  size_t user_len = 0;
  for (int i = 0; i < ni; ++i) {
    int k = d->inst_template[i];
    if (k < 0 || k >= d->n_templates) return fail(CEDAR_EINVAL, "instance template out of range");
    if (d->inst_par_off && d->inst_par_off[i] >= 0) {
      if (!d->inst_par) return fail(CEDAR_EINVAL, "inst_par missing");
      user_len = std::max<size_t>(user_len, (size_t)d->inst_par_off[i] + b->tpls[k]->H.par_size);
    }
  }
  std::vector<double> raw(d->inst_par ? d->inst_par : (const double *)nullptr, d->inst_par ? d->inst_par + user_len : (const double *)nullptr);
  std::vector<long long> nominal_off(d->n_templates);
  for (int k = 0; k < d->n_templates; ++k) { nominal_off[k] = (long long)raw.size(); raw.insert(raw.end(), b->tpls[k]->H.par.begin(), b->tpls[k]->H.par.end()); }
  std::vector<long long> raw_off(ni), dpar_off(ni), x0_off(ni, -1), dx_off(ni, -1);
  std::vector<int> itpl(ni);
  long long dsz = 0;
  for (int i = 0; i < ni; ++i) {
    int k = d->inst_template[i]; itpl[i] = k;
    raw_off[i] = (d->inst_par_off && d->inst_par_off[i] >= 0) ? d->inst_par_off[i] : nominal_off[k];
    dpar_off[i] = dsz; dsz += b->tpls[k]->H.dpar_size;
    if (d->inst_x0_off && d->inst_x0 && d->inst_x0_off[i] >= 0) { x0_off[i] = d->inst_x0_off[i]; b->has_x0 = true; }
    if (d->inst_dx_off && d->inst_dx && d->inst_dx_off[i] >= 0) { dx_off[i] = d->inst_dx_off[i]; b->has_dx = true; }
  }
  auto up = [&](auto &buf, const auto &vec) -> int {
    CUDA_TRY(buf.ensure(vec.size()));
    if (!vec.empty()) CUDA_TRY(cudaMemcpy(buf.p, vec.data(), vec.size() * sizeof(vec[0]), cudaMemcpyHostToDevice));
    return 0;
  };
  int rc;
  if ((rc = up(b->raw, raw)) || (rc = up(b->raw_off, raw_off)) || (rc = up(b->dpar_off, dpar_off)) || (rc = up(b->inst_tpl, itpl))) return rc;
  CUDA_TRY(b->dpar.ensure(std::max<long long>(dsz, 1)));
  int max_dev = 0; for (auto &t : b->tpls) max_dev = std::max(max_dev, t->D.n_dev);
  CUDA_TRY(launch_derive(b->d_tpls.p, b->inst_tpl.p, b->raw_off.p, b->raw.p, b->dpar_off.p, b->dpar.p, ni, max_dev, b->stream));
  // initial states / perturbations (original order)
  if (b->has_x0) {
    size_t len = 0; for (int i = 0; i < ni; ++i) if (x0_off[i] >= 0) len = std::max<size_t>(len, x0_off[i] + b->tpls[itpl[i]]->H.n);
    std::vector<double> v(d->inst_x0, d->inst_x0 + len);
    if ((rc = up(b->x0, v)) || (rc = up(b->x0_off, x0_off))) return rc;
  }
  if (b->has_dx) {
    size_t len = 0; for (int i = 0; i < ni; ++i) if (dx_off[i] >= 0) len = std::max<size_t>(len, dx_off[i] + b->tpls[itpl[i]]->H.n);
    std::vector<double> v(d->inst_dx, d->inst_dx + len);
    if ((rc = up(b->dx, v)) || (rc = up(b->dx_off, dx_off))) return rc;
  }
  // probes (internal)
  b->np = (d->n_probes > 0 && d->probes) ? d->n_probes : 0;
  b->ns = b->np ? d->n_samples : 0;
  if (b->np && b->ns < 2) return fail(CEDAR_EINVAL, "n_samples must be >= 2 with probes");
  if (b->np) {
    std::vector<int> pi((size_t)d->n_templates * b->np);
    for (int k = 0; k < d->n_templates; ++k)
      for (int p = 0; p < b->np; ++p) {
        int u = d->probes[(size_t)k * b->np + p];
        pi[(size_t)k * b->np + p] = (u >= 0 && u < b->tpls[k]->H.n) ? b->tpls[k]->H.iorder[u] : -1;
      }
    if ((rc = up(b->probes_int, pi))) return rc;
  }
  // queue: largest templates first (longest-processing-time first), stable by id
  std::vector<int> q(ni);
  for (int i = 0; i < ni; ++i) q[i] = i;
  std::stable_sort(q.begin(), q.end(), [&](int a, int c) {
    const Template &A = b->tpls[itpl[a]]->H, &C = b->tpls[itpl[c]]->H;
    long long ca = (long long)A.nnz_lu + A.n_out, cc = (long long)C.nnz_lu + C.n_out;
    if (ca != cc) return ca > cc;
    return itpl[a] < itpl[c];
  });
  if ((rc = up(b->queue, q))) return rc;
  // template blocks of the queue
  std::vector<int> qb;
  for (int i = 0; i < ni; ++i) if (i == 0 || itpl[q[i]] != itpl[q[i - 1]]) qb.push_back(i);
  qb.push_back(ni);
  b->n_qblk = (int)qb.size() - 1;
  if ((rc = up(b->qblk_beg, qb))) return rc;
  CUDA_TRY(b->qblk_head.ensure(std::max(b->n_qblk, 1)));
  CUDA_TRY(b->n_running.ensure(1));
  CUDA_TRY(b->rows.ensure(std::max(ni, 1)));
  CUDA_TRY(b->row_vec.ensure((size_t)std::max(ni, 1) * 6 * b->n_max));
  CUDA_TRY(b->stats.ensure(std::max(ni, 1)));
  CUDA_TRY(b->xfinal.ensure((size_t)std::max(ni, 1) * b->n_max));
  if (b->np) CUDA_TRY(b->samples.ensure((size_t)std::max(ni, 1) * b->np * b->ns));
  b->tune.lanes_per_inst = 32; b->tune.warps_per_cta = 4;  // best of the measured sweep on GB300
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  *out = b.release();
  return 0;
}

int cedar_batch_destroy(cedar_batch *b) { delete b; return 0; }

int cedar_batch_nmax(const cedar_batch *b, int32_t *n_max) {
  if (!b || !n_max) return fail(CEDAR_EINVAL, "null argument");
  *n_max = b->n_max;
  return 0;
}

int cedar_batch_set_tuning(cedar_batch *b, const cedar_batch_tuning *t) {
  if (!b || !t) return fail(CEDAR_EINVAL, "null argument");
  int K = t->lanes_per_inst;
  if (K != 1 && K != 2 && K != 4 && K != 8 && K != 16 && K != 32) return fail(CEDAR_EINVAL, "lanes_per_inst must be a power of two <= 32");
  if (t->warps_per_cta < 1 || t->warps_per_cta > 8) return fail(CEDAR_EINVAL, "warps_per_cta must be 1..8");
  if (t->ctas_per_sm < 0) return fail(CEDAR_EINVAL, "ctas_per_sm must be >= 0");
  b->tune = *t;
  return 0;
}

int cedar_batch_get_tuning(const cedar_batch *b, cedar_batch_tuning *t) {
  if (!b || !t) return fail(CEDAR_EINVAL, "null argument");
  *t = b->tune;
  return 0;
}

// Grid and shared memory of a persistent launch: slot workspaces of `stride`
// doubles in shared memory when a CTA's slots fit, else in global memory.
static int launch_geometry(int K, int warps, int stride, int n_inst, bool &in_smem, size_t &smem, int &grid) {
  int tiles = warps * 32 / K;
  size_t per_tile = (size_t)stride * sizeof(double);
  int smax = batch_max_smem_optin();
  in_smem = (size_t)tiles * per_tile <= (size_t)smax;
  smem = in_smem ? (size_t)tiles * per_tile : 0;
  int dev = 0, nsm = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  int per_sm = 1;
  if (in_smem) {
    int smsm = 0; CUDA_TRY(cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    per_sm = std::max(1, std::min(2048 / (warps * 32), (int)(smsm / std::max<size_t>(smem + 1024, 1))));
  } else {
    per_sm = std::max(1, 2048 / (warps * 32));
  }
  grid = std::max(1, std::min(nsm * per_sm, (n_inst + tiles - 1) / tiles));
  return 0;
}

// Largest circuit whose batched DC operating point may fall back to dense
// partial pivoting ((n + 2) n doubles of scratch per resident slot).
constexpr int kDenseNmax = 256;

static int batch_launch(cedar_batch *b, const EngOpts &eo, const cedar_batch_tuning &tu, bool want_outputs,
                        double t_until, bool fresh, const BatchDev *tape = nullptr, BatchDev *used = nullptr,
                        bool dc_only = false) {
  int K = tu.lanes_per_inst, warps = tu.warps_per_cta;
  int tiles = warps * 32 / K;
  bool in_smem = false; size_t smem = 0; int grid = 1;
  int rc = launch_geometry(K, warps, b->ws_stride, b->n_inst, in_smem, smem, grid);
  if (rc) return rc;
  {
    // a persistent grid of exactly the CTAs that can be resident at once
    int per_sm = 1, dev = 0, nsm = 0;
    CUDA_TRY(configure_batch(K, warps, smem, in_smem, tu.ctas_per_sm, &per_sm));
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    grid = std::max(1, std::min(nsm * per_sm, (b->n_inst + tiles - 1) / tiles));
  }
  if (!in_smem) CUDA_TRY(b->ws.ensure((size_t)grid * tiles * b->ws_stride));
  // dense DC fallback scratch (circuits of at most kDenseNmax unknowns)
  const long long dstride = ((long long)(b->n_max + 2) * b->n_max + 31) / 32 * 32;
  const bool dense_ok = b->n_max <= kDenseNmax;
  if (dense_ok) CUDA_TRY(b->dense_ws.ensure((size_t)grid * tiles * dstride));
  BatchDev bd{};
  bd.dense_ws = dense_ok ? b->dense_ws.p : nullptr; bd.dense_stride = dstride; bd.dense_nmax = kDenseNmax;
  bd.dc_only = dc_only ? 1 : 0;
  bd.tpls = b->d_tpls.p; bd.inst_tpl = b->inst_tpl.p; bd.inst_dpar = b->dpar_off.p; bd.dpar = b->dpar.p;
  bd.x0_off = b->has_x0 ? b->x0_off.p : nullptr; bd.x0 = b->x0.p;
  bd.dx_off = b->has_dx ? b->dx_off.p : nullptr; bd.dx = b->dx.p;
  bd.probes_int = b->probes_int.p; bd.np = want_outputs ? b->np : 0; bd.ns = b->ns;
  bd.samples = want_outputs ? b->samples.p : nullptr;
  bd.x_final = want_outputs ? b->xfinal.p : nullptr; bd.n_max = b->n_max;
  bd.stats = b->stats.p; bd.queue = b->queue.p; bd.n_inst = b->n_inst;
  bd.qblk_beg = b->qblk_beg.p; bd.qblk_head = b->qblk_head.p; bd.n_qblk = b->n_qblk;
  bd.opts = eo; bd.ws_stride = b->ws_stride; bd.ws_global = b->ws.p; bd.ws_in_smem = in_smem ? 1 : 0;
  bd.t_until = t_until; bd.rows = b->rows.p; bd.row_vec = b->row_vec.p; bd.n_running = b->n_running.p;
  if (tape) {
    bd.tape_t = tape->tape_t; bd.tape_ord = tape->tape_ord; bd.tape_p = tape->tape_p; bd.tape_v = tape->tape_v;
    bd.tape_cap = tape->tape_cap; bd.ckpt = tape->ckpt; bd.ckpt_every = tape->ckpt_every; bd.obj_idx = tape->obj_idx;
  }
  if (used) *used = bd;
  CUDA_TRY(cudaMemsetAsync(b->qblk_head.p, 0, std::max(b->n_qblk, 1) * sizeof(int), b->stream));
  CUDA_TRY(cudaMemsetAsync(b->n_running.p, 0, sizeof(int), b->stream));
  if (fresh) {
    CUDA_TRY(cudaMemsetAsync(b->rows.p, 0, (size_t)b->n_inst * sizeof(StateRow), b->stream));
    if (want_outputs) CUDA_TRY(cudaMemsetAsync(b->xfinal.p, 0, (size_t)b->n_inst * b->n_max * sizeof(double), b->stream));
  }
  if (!b->ev0) { CUDA_TRY(cudaEventCreate(&b->ev0)); CUDA_TRY(cudaEventCreate(&b->ev1)); }
  CUDA_TRY(cudaEventRecord(b->ev0, b->stream));
  CUDA_TRY(launch_batch(bd, K, warps, grid, smem, b->stream));
  CUDA_TRY(cudaEventRecord(b->ev1, b->stream));
  b->timed = true;
  return 0;
}

int cedar_batch_last_ms(cedar_batch *b, double *ms) {
  if (!b || !ms) return fail(CEDAR_EINVAL, "null argument");
  if (!b->timed) return fail(CEDAR_EINVAL, "no batch launch recorded yet");
  CUDA_TRY(cudaEventSynchronize(b->ev1));
  float f = 0; CUDA_TRY(cudaEventElapsedTime(&f, b->ev0, b->ev1));
  *ms = f;
  return 0;
}

int cedar_batch_start(cedar_batch *b, const cedar_tran_opts *opts) {
  const Range nvtx_range("cedar_batch_start");
  if (!b) return fail(CEDAR_EINVAL, "null handle");
  int rc = check_opts(opts); if (rc) return rc;
  b->run_opts = to_eng(opts);
  b->started = true;
  CUDA_TRY(cudaMemsetAsync(b->rows.p, 0, (size_t)std::max(b->n_inst, 1) * sizeof(StateRow), b->stream));
  CUDA_TRY(cudaMemsetAsync(b->xfinal.p, 0, (size_t)std::max(b->n_inst, 1) * b->n_max * sizeof(double), b->stream));
  return 0;
}

int cedar_batch_advance(cedar_batch *b, double t_until, int32_t *n_running) {
  const Range nvtx_range("cedar_batch_advance");
  if (!b) return fail(CEDAR_EINVAL, "null handle");
  if (!b->started) return fail(CEDAR_EINVAL, "cedar_batch_start was not called");
  int rc;
  if (b->n_inst > 0 && (rc = batch_launch(b, b->run_opts, b->tune, true, t_until, false))) return rc;
  if (n_running) {
    int v = 0;
    CUDA_TRY(cudaMemcpyAsync(&v, b->n_running.p, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    *n_running = v;
  }
  return 0;
}

int cedar_batch_dcop(cedar_batch *b, const cedar_tran_opts *opts, double *x_dc, cedar_stats *stats) {
  const Range nvtx_range("cedar_batch_dcop");
  if (!b) return fail(CEDAR_EINVAL, "null handle");
  cedar_tran_opts o;
  cedar_tran_opts_default(&o);
  if (opts) o = *opts;
  if (!(o.tstop > o.tstart)) o.tstop = o.tstart + 1.0;  // the transient span plays no part
  int rc = check_opts(&o); if (rc) return rc;
  if (b->n_inst == 0) return 0;
  EngOpts eo = to_eng(&o);
  eo.dcop = 1;
  CUDA_TRY(cudaMemsetAsync(b->rows.p, 0, (size_t)std::max(b->n_inst, 1) * sizeof(StateRow), b->stream));
  if ((rc = batch_launch(b, eo, b->tune, true, 1e300, true, nullptr, nullptr, true))) return rc;
  b->started = false;
  if (x_dc) CUDA_TRY(cudaMemcpyAsync(x_dc, b->xfinal.p, (size_t)b->n_inst * b->n_max * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (stats) CUDA_TRY(cudaMemcpyAsync(stats, b->stats.p, (size_t)b->n_inst * sizeof(EngStats), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return 0;
}

int cedar_batch_results(cedar_batch *b, double *x_final, double *samples, cedar_stats *stats) {
  const Range nvtx_range("cedar_batch_results");
  if (!b) return fail(CEDAR_EINVAL, "null handle");
  if (x_final) CUDA_TRY(cudaMemcpyAsync(x_final, b->xfinal.p, (size_t)b->n_inst * b->n_max * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (samples && b->np) CUDA_TRY(cudaMemcpyAsync(samples, b->samples.p, (size_t)b->n_inst * b->np * b->ns * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (stats) CUDA_TRY(cudaMemcpyAsync(stats, b->stats.p, (size_t)b->n_inst * sizeof(EngStats), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return 0;
}

int cedar_batch_run(cedar_batch *b, const cedar_tran_opts *opts, double *x_final, double *samples, cedar_stats *stats) {
  const Range nvtx_range("cedar_batch_run");
  if (!b) return fail(CEDAR_EINVAL, "null handle");
  int rc = check_opts(opts); if (rc) return rc;
  if (b->n_inst == 0) return 0;
  if ((rc = cedar_batch_start(b, opts))) return rc;
  if ((rc = batch_launch(b, b->run_opts, b->tune, true, 1e300, false))) return rc;
  if (x_final) CUDA_TRY(cudaMemcpyAsync(x_final, b->xfinal.p, (size_t)b->n_inst * b->n_max * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (samples && b->np) CUDA_TRY(cudaMemcpyAsync(samples, b->samples.p, (size_t)b->n_inst * b->np * b->ns * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (stats) CUDA_TRY(cudaMemcpyAsync(stats, b->stats.p, (size_t)b->n_inst * sizeof(EngStats), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return 0;
}

// ------------------------------------------------------------------ adjoint
int cedar_adjoint_nparams(const cedar_batch *b, int32_t *np_per_template, int32_t *np_max) {
  if (!b) return fail(CEDAR_EINVAL, "null handle");
  int m = 0;
  for (size_t k = 0; k < b->tpls.size(); ++k) {
    if (np_per_template) np_per_template[k] = b->tpls[k]->H.n_adj;
    m = std::max(m, b->tpls[k]->H.n_adj);
  }
  if (np_max) *np_max = m;
  return 0;
}

int cedar_adjoint_run(cedar_batch *b, const cedar_tran_opts *opts, const cedar_objective *obj, const double *tstar,
                      int64_t tape_cap, double *phi, double *grad, int32_t *status, cedar_stats *stats) {
  const Range nvtx_range("cedar_adjoint_run");
  if (!b || !obj) return fail(CEDAR_EINVAL, "null argument");
  int rc = check_opts(opts); if (rc) return rc;
  if (!opts->adaptive || opts->method != CEDAR_BDF2)
    return fail(CEDAR_EUNSUPPORTED, "the adjoint follows adaptive BDF2 runs");
  if (b->has_dx) return fail(CEDAR_EUNSUPPORTED, "the adjoint does not take state perturbations (inst_dx)");
  if (b->n_inst == 0) return 0;
  const long long cap = tape_cap > 0 ? tape_cap : (1LL << 19);
  const int every = 64;
  const int ni = b->n_inst, nt = (int)b->tpls.size();
  std::vector<int4> oi(nt);
  std::vector<AdjObj> ao(nt);
  int np_max = 0;
  for (int k = 0; k < nt; ++k) {
    const Template &H = b->tpls[k]->H;
    const cedar_objective &o = obj[k];
    if (o.vnode < 0 || o.vnode >= H.n_nodes || o.ibranch < H.n_nodes || o.ibranch >= H.n || o.probe < 0 || o.probe >= H.n)
      return fail(CEDAR_EINVAL, "objective index out of range for template " + std::to_string(k));
    oi[k] = make_int4(H.iorder[o.vnode], H.iorder[o.ibranch], H.iorder[o.probe], 0);
    ao[k] = AdjObj{oi[k].x, oi[k].y, oi[k].z, 0, o.level, o.w_energy, o.w_delay, o.w_final};
    np_max = std::max(np_max, H.n_adj);
  }
  const size_t ts = (size_t)ni * (size_t)tape_stride(cap);
  CUDA_TRY(b->tape_t.ensure(ts)); CUDA_TRY(b->tape_p.ensure(ts)); CUDA_TRY(b->tape_v.ensure(ts));
  CUDA_TRY(b->tape_ord.ensure(ts));
  CUDA_TRY(b->ckpt.ensure((size_t)ni * ckpt_count(cap, every) * 2 * b->n_max));
  CUDA_TRY(b->segx.ensure((size_t)ni * (every + 1) * b->n_max));
  CUDA_TRY(b->adj_phi.ensure(ni)); CUDA_TRY(b->adj_grad.ensure((size_t)ni * std::max(np_max, 1)));
  CUDA_TRY(b->adj_status.ensure(ni));
  CUDA_TRY(b->obj_idx.ensure(nt)); CUDA_TRY(b->adj_obj.ensure(nt));
  CUDA_TRY(cudaMemcpyAsync(b->obj_idx.p, oi.data(), nt * sizeof(int4), cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaMemcpyAsync(b->adj_obj.p, ao.data(), nt * sizeof(AdjObj), cudaMemcpyHostToDevice, b->stream));
  if (tstar) {
    CUDA_TRY(b->adj_tstar.ensure(ni));
    CUDA_TRY(cudaMemcpyAsync(b->adj_tstar.p, tstar, ni * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  }
  // forward with the tape on
  if ((rc = cedar_batch_start(b, opts))) return rc;
  BatchDev tape{};
  tape.tape_t = b->tape_t.p; tape.tape_ord = b->tape_ord.p; tape.tape_p = b->tape_p.p; tape.tape_v = b->tape_v.p;
  tape.tape_cap = cap; tape.ckpt = b->ckpt.p; tape.ckpt_every = every; tape.obj_idx = b->obj_idx.p;
  b->tape_cap = cap;
  BatchDev used{};
  if ((rc = batch_launch(b, b->run_opts, b->tune, true, 1e300, false, &tape, &used))) return rc;
  // backward
  const int K = b->tune.lanes_per_inst, warps = b->tune.warps_per_cta, tiles = warps * 32 / K;
  int stride = 0;
  for (auto &t : b->tpls) stride = std::max(stride, ws_doubles(t->H.n, t->H.nnz_lu, t->H.n_out, (int)t->H.src_group.size()) + t->H.n_adj);
  stride = ((stride + 15) / 16) * 16 + 8;
  bool in_smem = false; size_t smem = 0; int grid = 1;
  if ((rc = launch_geometry(K, warps, stride, ni, in_smem, smem, grid))) return rc;
  if (!in_smem) CUDA_TRY(b->ws.ensure((size_t)grid * tiles * stride));
  AdjDev a{};
  a.b = used;
  a.b.ws_stride = stride; a.b.ws_in_smem = in_smem ? 1 : 0; a.b.ws_global = b->ws.p;
  a.raw_off = b->raw_off.p; a.raw = b->raw.p; a.obj = b->adj_obj.p; a.tstar = tstar ? b->adj_tstar.p : nullptr;
  a.phi = b->adj_phi.p; a.grad = b->adj_grad.p; a.np_max = np_max; a.status = b->adj_status.p;
  a.segx = b->segx.p; a.fwd = b->stats.p;
  CUDA_TRY(cudaMemsetAsync(b->qblk_head.p, 0, std::max(b->n_qblk, 1) * sizeof(int), b->stream));
  if (!b->ev2) CUDA_TRY(cudaEventCreate(&b->ev2));
  CUDA_TRY(launch_adjoint(a, K, warps, grid, smem, b->stream));
  CUDA_TRY(cudaEventRecord(b->ev2, b->stream));
  b->adj_timed = true;
  if (phi) CUDA_TRY(cudaMemcpyAsync(phi, b->adj_phi.p, ni * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (grad && np_max) CUDA_TRY(cudaMemcpyAsync(grad, b->adj_grad.p, (size_t)ni * np_max * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (status) CUDA_TRY(cudaMemcpyAsync(status, b->adj_status.p, ni * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  if (stats) CUDA_TRY(cudaMemcpyAsync(stats, b->stats.p, (size_t)ni * sizeof(EngStats), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return 0;
}

int cedar_adjoint_tape(cedar_batch *b, int32_t inst, double *t, int8_t *ord, int64_t cap, int64_t *n_steps) {
  if (!b) return fail(CEDAR_EINVAL, "null handle");
  if (!b->adj_timed) return fail(CEDAR_EINVAL, "no adjoint run recorded yet");
  if (inst < 0 || inst >= b->n_inst) return fail(CEDAR_EINVAL, "instance out of range");
  EngStats st{};
  CUDA_TRY(cudaMemcpy(&st, b->stats.p + inst, sizeof(EngStats), cudaMemcpyDeviceToHost));
  const long long n = st.accepted, stride = tape_stride(b->tape_cap);
  if (n_steps) *n_steps = n;
  const long long m = std::min<long long>(n, std::max<int64_t>(cap, 0));
  if (m > 0 && t) CUDA_TRY(cudaMemcpy(t, b->tape_t.p + (size_t)inst * stride + 1, m * sizeof(double), cudaMemcpyDeviceToHost));
  if (m > 0 && ord) CUDA_TRY(cudaMemcpy(ord, b->tape_ord.p + (size_t)inst * stride + 1, m, cudaMemcpyDeviceToHost));
  return 0;
}

int cedar_adjoint_last_ms(cedar_batch *b, double *fwd_ms, double *bwd_ms) {
  if (!b) return fail(CEDAR_EINVAL, "null handle");
  if (!b->adj_timed) return fail(CEDAR_EINVAL, "no adjoint run recorded yet");
  CUDA_TRY(cudaEventSynchronize(b->ev2));
  float f = 0, g = 0;
  CUDA_TRY(cudaEventElapsedTime(&f, b->ev0, b->ev1));
  CUDA_TRY(cudaEventElapsedTime(&g, b->ev1, b->ev2));
  if (fwd_ms) *fwd_ms = f;
  if (bwd_ms) *bwd_ms = g;
  return 0;
}

int cedar_fp64_probe(int32_t active_lanes, int32_t iters, double *gflops, double *ms) {
  if (active_lanes < 1 || active_lanes > 32 || iters < 1) return fail(CEDAR_EINVAL, "active_lanes 1..32, iters >= 1");
  CUDA_TRY(launch_fp64_probe(active_lanes, iters, gflops, ms));
  return 0;
}

int cedar_fp64_latency(int32_t iters, double *cycles_per_op, double *ns_per_op) {
  if (iters < 1) return fail(CEDAR_EINVAL, "iters >= 1");
  CUDA_TRY(launch_fp64_latency(iters, cycles_per_op, ns_per_op));
  return 0;
}

int cedar_batch_autotune(cedar_batch *b, const cedar_tran_opts *opts, double horizon, cedar_batch_tuning *best) {
  const Range nvtx_range("cedar_batch_autotune");
  if (!b) return fail(CEDAR_EINVAL, "null handle");
  int rc = check_opts(opts); if (rc) return rc;
  cedar_tran_opts o = *opts;
  if (horizon > 0 && o.tstart + horizon < o.tstop) o.tstop = o.tstart + horizon;
  EngOpts eo = to_eng(&o);
  eo.hmax = to_eng(opts).hmax;  // keep the full run's step bounds
  const int Ks[] = {1, 2, 4, 8, 16, 32};
  const int Ws[] = {2, 4, 8};
  float best_ms = 1e30f; cedar_batch_tuning bt = b->tune;
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0)); CUDA_TRY(cudaEventCreate(&e1));
  for (int K : Ks) for (int W : Ws) {
    cedar_batch_tuning t{}; t.lanes_per_inst = K; t.warps_per_cta = W;
    CUDA_TRY(cudaEventRecord(e0, b->stream));
    if ((rc = batch_launch(b, eo, t, false, 1e300, true))) return rc;
    CUDA_TRY(cudaEventRecord(e1, b->stream));
    CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0; CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best_ms) { best_ms = ms; bt = t; }
  }
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  b->tune = bt;
  if (best) *best = bt;
  return 0;
}

}  // extern "C"
