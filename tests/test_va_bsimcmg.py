"""BSIM-CMG 107 through the Verilog-A front end and emitter, on the host.

The model's source is not part of this repository; set CEDAR_BSIMCMG_DIR to the
directory holding bsimcmg.va and its .include files (CedarSim ships them under
VerilogAParser.jl/cmc_models/bsimcmg107) to run this test, which is skipped
otherwise.  The default configuration (no NQS, gate-resistance or self-heating
nodes) is parsed, analysed and emitted; the emitted C++ is compiled with g++ and
its residuals and Jacobians are compared with the independent interpretation of
the same parsed module at several bias points, and the drain current is checked
for the on / off behaviour of an n-type FinFET.  The model has 6 terminal
values (d, g, s, e and the internal di, si); a library built with it widens the
engines' per-device staging to 6 (CEDAR_MAX_TERM)."""
import ctypes as C
import importlib.util
import os
import pathlib
import shutil
import subprocess

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
CSRC = ROOT / "cedarsim.jl_gb300" / "csrc"
SRC_DIR = os.environ.get("CEDAR_BSIMCMG_DIR", "")
VT = 1.380649e-23 * (27.0 + 273.15) / 1.602176634e-19

pytestmark = pytest.mark.skipif(not SRC_DIR or not (pathlib.Path(SRC_DIR) / "bsimcmg.va").is_file(),
                                reason="CEDAR_BSIMCMG_DIR does not point at the BSIM-CMG 107 sources")


@pytest.fixture(scope="module")
def bsim(pkg, tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    import importlib
    P = importlib.import_module("cedarsim_gb300.va.parser")
    E = importlib.import_module("cedarsim_gb300.va.emit")
    mod = P.parse_file(pathlib.Path(SRC_DIR) / "bsimcmg.va")[0]
    m, a = E.analyze(mod)
    d = tmp_path_factory.mktemp("bsimcmg")
    text = E.emit_header([(m, a)], 11)
    assert "#define CEDAR_MAX_TERM 6" in text
    (d / "va_models.gen.h").write_text(text)
    (d / "h.cpp").write_text('#include <math.h>\n#include "va_models.gen.h"\n'
                             'extern "C" void h_full(const double *dp, const double *v, double *fi, double *fq, '
                             'double *G, double *C) { cedar::va::full(0, dp, 1, v, 1e-12, fi, fq, G, C); }\n')
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-I", str(CSRC), "-I", str(d),
                        str(d / "h.cpp"), "-o", str(d / "libh.so")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    lib = C.CDLL(str(d / "libh.so"))
    lib.h_full.argtypes = [C.POINTER(C.c_double)] * 6
    return mod, m, lib


def test_bsimcmg_structure(bsim):
    mod, m, _ = bsim
    assert m.ports == ["d", "g", "s", "e"] and m.internals == ["di", "si"] and m.nterm == 6
    assert len(m.params) > 800 and len(mod.functions) >= 1 and len(m.noise) > 0


def test_bsimcmg_emitted_matches_interpreter(bsim):
    mod, m, lib = bsim
    spec = importlib.util.spec_from_file_location("cedar_va_interp_b", ROOT / "oracle" / "va_interp.py")
    vi = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(vi)
    vals = m.defaults({})
    dp = np.array(vals + [1.0, VT])
    dp_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    ids = {}
    for v in ([0.5, 0.7, 0.0, 0.0, 0.5, 0.0], [1.0, 1.0, 0.0, 0.0, 0.98, 0.01], [0.05, 0.2, 0.0, 0.0, 0.05, 0.0],
              [0.0, 0.9, 0.6, 0.0, 0.0, 0.6], [0.3, -0.2, 0.0, 0.1, 0.31, -0.01]):
        n = m.nx
        fi, fq, G, Cm = np.zeros(n), np.zeros(n), np.zeros(n * n), np.zeros(n * n)
        lib.h_full(dp_(dp), dp_(np.array(v)), dp_(fi), dp_(fq), dp_(G), dp_(Cm))
        ri, rq, rG, rC = map(np.asarray, vi.evaluate(mod, dict(zip([p.name for p in m.params], vals)), v, VT,
                                                      1e-12, 1.0, []))
        assert np.all(np.abs(fi - ri) <= 1e-12 * (np.abs(ri).max() + 1e-30))
        assert np.all(np.abs(fq - rq) <= 1e-12 * (np.abs(rq).max() + 1e-40))
        assert np.all(np.abs(G - rG.ravel()) <= 1e-11 * (np.abs(rG).max() + 1e-30))
        assert np.all(np.abs(Cm - rC.ravel()) <= 1e-11 * (np.abs(rC).max() + 1e-40))
        ids[tuple(v)] = -fi[4]                      # current leaving di through the channel
    on = ids[(0.5, 0.7, 0.0, 0.0, 0.5, 0.0)]
    off = ids[(0.05, 0.2, 0.0, 0.0, 0.05, 0.0)]
    assert on > 1e-6 and 0 < off < 1e-3 * on      # an n-type FinFET turns on with the gate
