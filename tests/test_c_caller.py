"""The C ABI from a plain C caller (the role a Julia `ccall` shim plays).

A C99 program that includes only include/cedar.h and links the library builds
the descriptor of a 10-section RC ladder by hand (struct-of-arrays parameters,
ground = -1, the source's branch unknown after the nodes), plans it with the
host-only entry points (cedar_plan_create, cedar_ckt_size, cedar_ckt_costs,
cedar_ckt_pattern), and checks the error path (a terminal out of range ->
CEDAR_EINVAL with a message).  Its results must equal those of the Python host
mirror for the same circuit.  No GPU is needed: planning is host work.
"""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "cedar.h"

enum { N = 10 };

int main(void) {
  int32_t rterm[2 * N], cterm[2 * N], vterm[2] = {0, -1}, vbr[1] = {N + 1};
  double rpar[2 * N], cpar[2 * N], vpar[10] = {1.0, 1.0, CEDAR_WAVE_DC, 0, 0, 0, 0, 0, 0, 0};
  for (int k = 0; k < N; ++k) {
    rterm[2 * k] = k; rterm[2 * k + 1] = k + 1;        /* R_k: node k -> node k+1 */
    cterm[2 * k] = k + 1; cterm[2 * k + 1] = -1;       /* C_k: node k+1 -> ground */
    rpar[k] = 1e3; rpar[N + k] = 1.0;                  /* r[N], then m[N] */
    cpar[k] = 1e-12; cpar[N + k] = 1.0;
  }
  cedar_devgroup g[3] = {{CEDAR_V, 1, vterm, vbr, vpar}, {CEDAR_R, N, rterm, NULL, rpar},
                         {CEDAR_C, N, cterm, NULL, cpar}};
  cedar_ckt_desc d;
  memset(&d, 0, sizeof d);
  d.n_nodes = N + 1; d.n_branch = 1; d.n_groups = 3; d.groups = g;
  d.temp_c = 27.0; d.gmin = 1e-12; d.ordering = CEDAR_ORDER_AUTO;
  cedar_ckt *c = NULL;
  int rc = cedar_plan_create(&d, &c);
  if (rc != CEDAR_OK) { char b[256]; cedar_last_error(b, sizeof b); printf("plan failed %d %s\n", rc, b); return 1; }
  int32_t n, nnz_j, nnz_lu, nlev;
  cedar_ckt_size(c, &n, &nnz_j, &nnz_lu, &nlev);
  cedar_costs cs;
  cedar_ckt_costs(c, &cs);
  int32_t colptr[N + 3], rowidx[256];
  rc = cedar_ckt_pattern(c, colptr, rowidx);
  printf("size %d %d %d\n", n, nnz_j, nnz_lu);
  printf("costs %lld %lld %lld %lld %lld %lld %d\n", (long long)cs.flops_eval, (long long)cs.flops_stamp,
         (long long)cs.flops_lu, (long long)cs.flops_solve, (long long)cs.flops_update, (long long)cs.bytes,
         cs.nnz_lu);
  printf("pattern %d", rc);
  for (int k = 0; k <= n; ++k) printf(" %d", colptr[k]);
  printf("\n");
  cedar_ckt_destroy(c);
  rterm[0] = N + 7;                                     /* a terminal beyond the unknowns */
  cedar_ckt *bad = NULL;
  rc = cedar_plan_create(&d, &bad);
  char msg[256] = {0};
  cedar_last_error(msg, sizeof msg);
  printf("error %d %s\n", rc, msg);
  return 0;
}
"""


def test_plain_c_caller(pkg, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = pathlib.Path(pkg.load_library()._name)
    (tmp_path / "caller.c").write_text(PROGRAM)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(tmp_path / "caller.c"),
                        str(lib), f"-Wl,-rpath,{lib.parent}", "-o", str(tmp_path / "caller")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([str(tmp_path / "caller")], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = {l.split()[0]: l.split()[1:] for l in out.stdout.splitlines()}
    # the same circuit through the Python host mirror
    c = pkg.Circuit()
    c.V("V", "n0", "0", dc=1.0)
    for k in range(10):
        c.R(f"R{k}", f"n{k}", f"n{k + 1}", r=1e3)
    for k in range(10):
        c.C(f"C{k}", f"n{k + 1}", "0", 1e-12)
    flat = c.flatten()
    costs = pkg.api.costs(flat)
    n, nnz_j, nnz_lu = map(int, lines["size"])
    assert n == flat.n == 12
    assert nnz_lu == costs["nnz_lu"]
    assert list(map(int, lines["costs"])) == [costs[k] for k in ("flops_eval", "flops_stamp", "flops_lu",
                                                                  "flops_solve", "flops_update", "bytes", "nnz_lu")]
    pat = list(map(int, lines["pattern"]))
    assert pat[0] == 0 and pat[-1] == nnz_j and len(pat) == n + 2
    assert int(lines["error"][0]) == -1 and "terminal index out of range" in " ".join(lines["error"][1:])
