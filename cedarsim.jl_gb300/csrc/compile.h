// compile.h — host-side circuit compiler: flattened device table -> everything the
// GPU engine needs (stamp programs, static-pivot ordering, LU fill, level schedules).
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include "../../include/cedar.h"

namespace cedar {

// Per-model constants shared by the compiler and the kernels.
struct ModelInfo {
  int nterm;     // terminals (without branch)
  int npar;      // raw parameters (cedar.h order)
  int has_br;    // carries a branch-current unknown
  int nout;      // per-device outputs written by the eval kernels
  int ndpar;     // derived parameters
};
const ModelInfo &model_info(int model);
// number of model ids (built-in models, then the compiled Verilog-A models)
int num_models();

// One stamp: contribution of output `out` (sign -1/+1) of a device to
// J[row_eq][col_unknown] (col >= 0) or to a residual/charge row (col = -1).
struct Stamp { int row, col, out, neg; };
// Stamps of one device given its local terminal unknowns t[] (branch last);
// output k of the device is out_base + k * out_stride.
void device_stamps(int model, const int *t, int out_base, int out_stride, std::vector<Stamp> &J,
                   std::vector<Stamp> &F, std::vector<Stamp> &Q);

struct GroupInfo {
  int model, n_inst, ntx;          // ntx = terminals + branch
  int term_off;                    // into term_int / term_orig
  int par_off;                     // into the raw parameter block
  int dpar_off;                    // into the derived parameter block
  int out_off;                     // first output index of the group
};

// Compiled template (one topology).  All index arrays are int32.
struct Template {
  int n = 0, n_nodes = 0, n_branch = 0;
  double temp_c = 27.0, gmin = 1e-12;
  std::vector<GroupInfo> groups;
  std::vector<int32_t> term_orig, term_int;  // per device terminal (+branch) unknowns
  int par_size = 0, dpar_size = 0, n_out = 0;
  std::vector<uint8_t> out_q;                // per device output: 1 if it holds cj * dQ/dV (C part of J)
  std::vector<double> par;                   // nominal raw parameters
  std::vector<double> pwl;

  // static pivoting + ordering
  std::vector<int32_t> rowmatch;  // unknown u -> equation (row) used as its pivot row
  std::vector<int32_t> order;     // position p -> unknown u
  std::vector<int32_t> iorder;    // unknown u -> position p
  std::vector<int32_t> eq_pos;    // equation e -> internal row p
  std::vector<uint8_t> is_node_int;  // internal position -> 1 if node voltage

  // J pattern in original space (CSC)
  std::vector<int32_t> j_colptr, j_rowidx;
  // LU pattern in internal space (CSR, sorted columns), diag position per row
  std::vector<int32_t> lu_rowptr, lu_colidx, lu_diag;
  int nnz_lu = 0;

  // stamp programs: ptr arrays + entries ((out << 1) | neg)
  std::vector<int32_t> jlu_ptr, jlu_ent;    // per LU slot (internal)
  std::vector<int32_t> jcsc_ptr, jcsc_ent;  // per original CSC slot
  std::vector<int32_t> fint_ptr, fint_ent;  // residual per internal row
  std::vector<int32_t> qint_ptr, qint_ent;  // charge per internal row
  std::vector<int32_t> forg_ptr, forg_ent;  // residual per original row (cedar_eval)

  // LU factorisation tasks by level.  Task kinds: 0 = U entry, 1 = diagonal
  // (also writes the reciprocal pivot), 2 = L entry (scaled by rd[col]).
  std::vector<int32_t> lu_lvl_ptr;             // levels -> [task range)
  std::vector<int32_t> lu_task_slot, lu_task_info, lu_pair_ptr, lu_pair;  // pair = (a<<16)|b packed when small
  std::vector<int32_t> lu_pair_a, lu_pair_b;   // unpacked pairs
  // triangular solves (row tasks by level)
  std::vector<int32_t> fw_lvl_ptr, fw_row, fw_ptr, fw_lu, fw_col;
  std::vector<int32_t> bw_lvl_ptr, bw_row, bw_ptr, bw_lu, bw_col;
  // transposed substitutions (adjoint), same layout as fw/bw
  std::vector<int32_t> tf_lvl_ptr, tf_row, tf_ptr, tf_lu, tf_col;
  std::vector<int32_t> tb_lvl_ptr, tb_row, tb_ptr, tb_lu, tb_col;
  // C^T program per internal column: entry ((out << 1) | neg) and internal row
  std::vector<int32_t> ct_ptr, ct_ent, ct_row;
  // gather lists longer than kLongGather (in-engine programs) or kLongEval
  // (cedar_eval programs): summed cooperatively (fixed chunks, fixed tree)
  std::vector<int32_t> long_jc_fo_off;  // chunk offsets (kLongChunk entries each) of long_jc then long_fo
  std::vector<int32_t> long_lu, long_fi, long_jc, long_fo;
  // adjoint parameters: first gradient index of each group (-1: none); MOS1
  // widths and resistor values, in group order
  std::vector<int32_t> adj_goff;
  int n_adj = 0;
  // time-varying sources (global device index), for breakpoint search
  std::vector<int32_t> src_group, src_inst;
  // LU slot of (KCL(u), u) per node u, used by the DC gmin-stepping homotopy
  std::vector<int32_t> gs_slot;

  int64_t lu_flops = 0;  // pair count (FMAs) + L scalings + reciprocals
  int ordering = 0;       // ordering actually used
  double sched_cost = 0;  // estimated critical path of LU + substitutions
};

// Gather lists longer than these are summed cooperatively on the device (must
// equal kLongGather / kLongEval of engine.cuh).
constexpr int kLongGatherHost = 16, kLongEvalHost = 64;
// cedar_eval sums a long list in chunks of this many entries (one warp each)
constexpr int kLongChunk = 256;

// Ordering strategies for the fill-reducing symmetric permutation.
enum Ordering { ORDER_AUTO = 0, ORDER_MIN_DEGREE = 1, ORDER_NESTED_DISSECTION = 2, ORDER_NATURAL = 3 };

// Compiles and then validates the template (validate_template); false with err
// set if either fails.
bool compile_template(const cedar_ckt_desc *d, Template &T, std::string &err,
                      int ordering = ORDER_AUTO);

// Checks every index array of a compiled template against the extent it
// indexes (device outputs, unknowns, J and LU slots, levels, permutations).
// The engine kernels index with these tables unchecked; this is their bounds
// check, run on the host before anything is uploaded.
bool validate_template(const Template &T, std::string &err);

}  // namespace cedar
