"""The host-side bounds check of compiled templates (validate_template).

The engine kernels index device outputs, J / LU slots and unknowns through the
compiled template's tables without per-access checks; compile_template ends by
checking every one of those tables against the extent it indexes, so that a
compiler defect is reported as an error on the host instead of reaching a GPU.
These tests (CPU only) check that the templates of every workload pass, and that
each kind of corrupted table is rejected: a small C++ driver built from the
compiler's own source plants one defect at a time in a copy of a compiled
template and runs the check on it.
"""
import ctypes as C
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
CSRC = ROOT / "cedarsim.jl_gb300" / "csrc"
GEN = ROOT / "cedarsim.jl_gb300" / "_build" / "gen"

DRIVER = r"""
#include <cstdio>
#include <functional>
#include <utility>
#include <vector>
#include "compile.h"
using namespace cedar;

// Compiles the template, checks that it passes, then plants one defect per case
// in a copy and records whether the check rejects it (res[k] = 1).  Returns the
// number of cases, or -1 if the unmodified template fails.
extern "C" int tpl_check(const cedar_ckt_desc *d, int *res, int cap, char *msg, int msglen) {
  Template T;
  std::string err;
  if (!compile_template(d, T, err)) { std::snprintf(msg, msglen, "%s", err.c_str()); return -1; }
  std::vector<std::function<void(Template &)>> cases = {
      [](Template &t) { t.jlu_ent[0] = t.n_out << 1; },              // a stamp naming no device output
      [](Template &t) { t.fint_ent.back() = -2; },                   // a negative residual entry
      [](Template &t) { t.jcsc_ptr.back() += 1; },                   // a program pointer past its entries
      [](Template &t) { t.lu_pair_a[0] = t.nnz_lu; },                // an LU pair beyond the factor
      [](Template &t) { t.lu_pair_b.back() = -1; },
      [](Template &t) { t.lu_task_slot[0] = t.lu_task_slot[1]; },   // two tasks on one slot
      [](Template &t) { t.lu_task_info[0] = (t.n << 2) | 1; },      // a task column beyond the unknowns
      [](Template &t) { t.lu_lvl_ptr.back() -= 1; },                 // levels that miss a task
      [](Template &t) { t.lu_diag[0] = t.lu_rowptr[1]; },            // a diagonal outside its row
      [](Template &t) { std::swap(t.lu_colidx[t.lu_rowptr[1]], t.lu_colidx[t.lu_rowptr[1] + 1]); },  // unsorted row
      [](Template &t) { t.fw_col[0] = t.n; },                        // substitution column beyond the unknowns
      [](Template &t) { t.bw_lu.back() = t.nnz_lu; },                // substitution slot beyond the factor
      [](Template &t) { t.tf_row[0] = t.tf_row[1]; },                // rows no longer a permutation
      [](Template &t) { t.tb_ptr[1] = t.tb_ptr[2] + 1; },            // a decreasing row pointer
      [](Template &t) { t.term_int[0] = t.n; },                      // a terminal beyond the unknowns
      [](Template &t) { std::swap(t.order[0], t.order[1]); },        // order and iorder disagree
      [](Template &t) { t.eq_pos[0] = t.eq_pos[1]; },                // equation positions not a permutation
      [](Template &t) { t.j_rowidx[0] = t.n; },                      // J pattern row beyond the unknowns
      [](Template &t) { t.ct_row[0] = -1; },                         // C^T program row
      [](Template &t) { t.ct_ent[0] = (t.n_out + 5) << 1; },
      [](Template &t) { t.gs_slot[0] = t.nnz_lu; },                  // gmin-stepping slot beyond the factor
      [](Template &t) { t.groups[0].out_off += 1; },                 // group slices that overlap
      [](Template &t) { t.out_q.pop_back(); },                       // per-output flags too short
      [](Template &t) { t.src_inst[0] = t.groups[t.src_group[0]].n_inst; },  // a source beyond its group
      [](Template &t) { t.adj_goff[0] = t.n_adj + 1; },
  };
  const int m = (int)cases.size();
  for (int k = 0; k < m && k < cap; ++k) {
    Template c = T;
    cases[k](c);
    std::string e;
    res[k] = validate_template(c, e) ? 0 : 1;
  }
  return m;
}
"""


@pytest.fixture(scope="module")
def driver(pkg, tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    pkg.load_library()      # the build has emitted the Verilog-A header the compiler includes
    d = tmp_path_factory.mktemp("tplcheck")
    (d / "drv.cpp").write_text(DRIVER)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-shared", "-fPIC", "-I", str(ROOT / "include"), "-I", str(CSRC),
                        "-I", str(GEN), str(d / "drv.cpp"), str(CSRC / "compile.cpp"), "-o", str(d / "libdrv.so")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    lib = C.CDLL(str(d / "libdrv.so"))
    lib.tpl_check.restype = C.c_int
    lib.tpl_check.argtypes = [C.POINTER(pkg.abi.CktDesc), C.POINTER(C.c_int), C.c_int, C.c_char_p, C.c_int]
    return lib


def _pulsed_chain(pkg):
    """A 9-stage chain with a pulse input (a time-varying source), a MOSFET group
    first (adjoint offsets) and capacitors (charge-partial program)."""
    return pkg.generators.inverter_chain(9).flatten()


def test_every_planted_defect_is_rejected(pkg, driver):
    flat = _pulsed_chain(pkg)
    h = pkg.abi.DescHolder(flat)
    res = (C.c_int * 64)()
    msg = C.create_string_buffer(512)
    m = driver.tpl_check(C.byref(h.desc), res, 64, msg, 512)
    assert m > 0, msg.value.decode()
    missed = [k for k in range(m) if res[k] != 1]
    assert not missed, f"defect cases not rejected: {missed}"


@pytest.mark.parametrize("case", ["chains", "rings", "va_mixed", "rc_ladder", "long_chain"])
def test_workload_templates_pass_the_check(pkg, case):
    """Templates of every workload compile (compile_template ends with the check):
    the Monte Carlo chain lengths, the ring oscillator, the Verilog-A mix, the RC
    ladder and a 20 000-stage chain (supply rails long enough for chunked sums)."""
    from tests import circuits as K
    g = pkg.generators
    if case == "chains":
        flats = [g.inverter_chain(L).flatten() for L in range(5, 64, 2)]
    elif case == "rings":
        ring = g.ring_oscillator(15).flatten()
        flats = [ring, g.as_verilog_a(ring)]
    elif case == "va_mixed":
        flats = [K.va_mixed(pkg).flatten(), K.mixed(pkg).flatten()]
    elif case == "rc_ladder":
        flats = [g.rc_ladder(100).flatten()]
    else:
        flats = [g.inverter_chain(20000).flatten()]
    for f in flats:
        c = pkg.api.costs(f)        # cedar_plan_create: compile_template, validation included
        assert c
