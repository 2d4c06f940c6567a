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
import sys

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


_INVERTER_SCRIPT = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import __graft_entry__ as ge
pkg = ge.load()
O = ge.load_oracle().Oracle(pkg)

def inverter(vin):
    c = pkg.Circuit()
    c.V("VDD", "vdd", "0", dc=0.7)
    c.V("VIN", "in", "0", dc=vin) if not isinstance(vin, pkg.Pulse) else c.V("VIN", "in", "0", wave=vin)
    c.va("MN", "bsimcmg", ["out", "in", "0", "0"], DEVTYPE=1)
    c.va("MP", "bsimcmg", ["out", "in", "vdd", "vdd"], DEVTYPE=0)
    c.C("CL", "out", "0", 1e-15)
    return c.flatten()

res = {"dc": {}}
for vin in (0.0, 0.35, 0.7):
    f = inverter(vin)
    x, st, rc = O.dcop(f)
    res["dc"][str(vin)] = [rc, st.status, st.dc_iters, float(x[f.names.index("out")])]
f = inverter(pkg.Pulse(0.0, 0.7, 10e-12, 5e-12, 5e-12, 40e-12, 100e-12))
t, xs, st, rc = O.tran(f, pkg.make_opts("bdf2", True, 0.0, 100e-12, 0.0, True, 1e-6, 1e-9), cap=1 << 16)
k = f.names.index("out")
res["tran"] = [rc, st.status, len(t), float(xs[0, k]), float(xs[:, k].min()), float(xs[-1, k]),
               float(xs[np.searchsorted(t, 50e-12), k])]
print(json.dumps(res))
"""


def test_bsimcmg_inverter_dc_and_transient_on_the_oracle(tmp_path):
    """A CMOS inverter of two BSIM-CMG devices (0.7 V supply, 1 fF load) through the
    oracle's DC homotopy and adaptive BDF2 with the model compiled in: the DC point
    is reached from zero with the input at 0 V, mid-rail and 0.7 V, and a 0 -> 0.7 V
    input pulse pulls the output low and releases it.  At 0 V input the PMOS's
    smoothed V_ds rounds to exactly 0 while its partials do not, so the DC solve
    depends on pow's zero-exponent derivative rule (x^0 has zero partials).  The
    oracle and package are copied to a scratch directory, so the model's generated
    code never enters this checkout's build."""
    if shutil.which("g++") is None or shutil.which("make") is None:
        pytest.skip("g++ / make not available")
    import json
    work = tmp_path / "repo"
    ign = shutil.ignore_patterns("_build", "__pycache__", "_work")
    for d in ("cedarsim.jl_gb300", "oracle", "include"):
        shutil.copytree(ROOT / d, work / d, ignore=ign)
    shutil.copy(ROOT / "__graft_entry__.py", work / "__graft_entry__.py")
    (tmp_path / "inv.py").write_text(_INVERTER_SCRIPT)
    env = dict(os.environ, CEDAR_VA_PATH=str(pathlib.Path(SRC_DIR) / "bsimcmg.va"))
    r = subprocess.run([sys.executable, str(tmp_path / "inv.py"), str(work)], capture_output=True, text=True,
                       env=env, timeout=1800)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    for vin, (rc, status, iters, vout) in res["dc"].items():
        assert rc == 0 and status == 0, (vin, rc, status, iters)
    assert res["dc"]["0.0"][3] > 0.699 and res["dc"]["0.7"][3] < 1e-3
    assert 0.0 < res["dc"]["0.35"][3] < 0.7
    rc, status, npts, v0, vmin, vend, vmid = res["tran"]
    assert rc == 0 and status == 0 and npts > 10
    assert v0 > 0.699 and vmid < 0.1 and vmin < 0.1 and vend > 0.6
