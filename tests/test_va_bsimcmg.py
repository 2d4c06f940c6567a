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
engines' per-device staging to 6 (CEDAR_MAX_TERM).  With the model compiled into
a scratch copy of the oracle, a CMOS inverter of two devices runs its DC
operating point and a transient, and, given CEDAR_ASAP7_CARD (the ASAP7 TT
Spectre model cards), its output-noise density is compared with the ngspice
table of CedarSim's own BSIM-CMG noise test."""
import ctypes as C
import importlib.util
import os
import pathlib
import shutil
import subprocess
import sys
import zlib

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


@pytest.fixture(scope="module")
def scratch(tmp_path_factory):
    """A copy of the package and the oracle in a scratch directory, where scripts
    run with CEDAR_VA_PATH naming the model, so that its generated code never
    enters this checkout's build (the oracle compiles it in on first use)."""
    if shutil.which("g++") is None or shutil.which("make") is None:
        pytest.skip("g++ / make not available")
    d = tmp_path_factory.mktemp("bsim_scratch")
    work = d / "repo"
    ign = shutil.ignore_patterns("_build", "__pycache__", "_work")
    for sub in ("cedarsim.jl_gb300", "oracle", "include"):
        shutil.copytree(ROOT / sub, work / sub, ignore=ign)
    shutil.copy(ROOT / "__graft_entry__.py", work / "__graft_entry__.py")
    env = dict(os.environ, CEDAR_VA_PATH=str(pathlib.Path(SRC_DIR) / "bsimcmg.va"))

    def run(script: str, *args: str):
        import json
        f = d / f"s{zlib.crc32(script.encode()):08x}.py"
        f.write_text(script)
        r = subprocess.run([sys.executable, str(f), str(work), *args], capture_output=True, text=True, env=env,
                           timeout=1800)
        assert r.returncode == 0, r.stderr[-3000:]
        return json.loads(r.stdout.strip().splitlines()[-1])
    return run


def test_bsimcmg_inverter_dc_and_transient_on_the_oracle(scratch):
    """A CMOS inverter of two BSIM-CMG devices (0.7 V supply, 1 fF load) through the
    oracle's DC homotopy and adaptive BDF2 with the model compiled in: the DC point
    is reached from zero with the input at 0 V, mid-rail and 0.7 V, and a 0 -> 0.7 V
    input pulse pulls the output low and releases it.  At 0 V input the PMOS's
    smoothed V_ds rounds to exactly 0 while its partials do not, so the DC solve
    depends on pow's zero-exponent derivative rule (x^0 has zero partials)."""
    res = scratch(_INVERTER_SCRIPT)
    for vin, (rc, status, iters, vout) in res["dc"].items():
        assert rc == 0 and status == 0, (vin, rc, status, iters)
    assert res["dc"]["0.0"][3] > 0.699 and res["dc"]["0.7"][3] < 1e-3
    assert 0.0 < res["dc"]["0.35"][3] < 0.7
    rc, status, npts, v0, vmin, vend, vmid = res["tran"]
    assert rc == 0 and status == 0 and npts > 10
    assert v0 > 0.699 and vmid < 0.1 and vmin < 0.1 and vend > 0.6


_NOISE_SCRIPT = r"""
import json, re, sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import __graft_entry__ as ge
pkg = ge.load()
O = ge.load_oracle().Oracle(pkg)

def cards(path):
    # Spectre `model NAME bsimcmg type=n ...` cards with `+ name = value` lines
    out, cur = {}, None
    for line in open(path):
        line = line.split("//")[0].rstrip()
        m = re.match(r"\s*model\s+(\w+)\s+bsimcmg\s+(.*)", line, re.I)
        if m:
            cur, rest = m.group(1).lower(), m.group(2)
            out[cur] = {}
        elif cur and line.strip().startswith("+"):
            rest = line.strip()[1:]
        else:
            continue
        for k, v in re.findall(r"(\w+)\s*=\s*([^\s]+)", rest):
            out[cur][k.lower()] = v
    return out

mod = pkg.va.model(pkg.va.model_id("bsimcmg"))
names = {p.name.lower(): p.name for p in mod.params}
def params(card):
    # type = n / p -> DEVTYPE; LEVEL (the simulator's model selector) is not a module parameter
    p = {"DEVTYPE": 1 if card["type"].lower() == "n" else 0}
    p.update({names[k]: float(v) for k, v in card.items() if k in names})
    return p

C = cards(sys.argv[2])
c = pkg.Circuit()                              # test/bsimcmg/inverter_cmg_cedar.cir
c.V("VVDD", "vdd", "0", dc=1.0)
c.V("VVSS", "vss", "0", dc=0.0)
c.C("CQ", "d", "0", 1e-15)
c.V("VD", "d", "0", dc=0.5, ac=1.0)
c.va("mneg", "bsimcmg", ["q", "d", "vss", "vss"], **params(C["nmos_lvt"]))
c.va("mpos", "bsimcmg", ["q", "d", "vdd", "vdd"], **params(C["pmos_lvt"]))
f = c.flatten()
x, st, rc = O.dcop(f)
f_hz = np.array(json.loads(sys.argv[3]))
psd = O.noise(f, x, 2 * np.pi * f_hz, f.index("q")) if rc == 0 else np.full(len(f_hz), np.nan)
# test/bsimcmg/inverter.jl: the same inverter with VD = SIN(0.5 0.01 1e7), 0 .. 400 ns
ct = pkg.Circuit()
ct.V("VVDD", "vdd", "0", dc=1.0)
ct.V("VVSS", "vss", "0", dc=0.0)
ct.C("CQ", "d", "0", 1e-15)
ct.V("VD", "d", "0", wave=pkg.Sin(0.5, 0.01, 1e7))
ct.va("mneg", "bsimcmg", ["q", "d", "vss", "vss"], **params(C["nmos_lvt"]))
ct.va("mpos", "bsimcmg", ["q", "d", "vdd", "vdd"], **params(C["pmos_lvt"]))
ft = ct.flatten()
t, xs, stt, rct = O.tran(ft, pkg.make_opts("bdf2", True, 0.0, 4e-7, 0.0, True, 1e-7, 1e-7), cap=1 << 18)
qd = xs[:, ft.index("q")] - x[f.index("q")]
dd = xs[:, ft.index("d")] - 0.5
gain = float(np.dot(qd, dd) / np.dot(dd, dd))
print(json.dumps({"rc": rc, "dc_iters": int(st.dc_iters), "q": float(x[f.index("q")]),
                  "sqrt_psd": np.sqrt(np.abs(psd)).tolist(),
                  "tran": [rct, int(stt.status), len(t), gain]}))
"""


def test_bsimcmg_inverter_noise_matches_ngspice(scratch):
    """CedarSim's BSIM-CMG noise test (test/ac.jl:155-237): the output-noise density
    of a BSIM-CMG inverter on the ASAP7 TT cards (nmos_lvt / pmos_lvt, VDD = 1 V,
    input at 0.5 V, 1 fF on the input) against the ngspice table the reference
    holds (tests/golden/ac_noise_bsimcmg_ngspice.json, 1 kHz .. 1 PHz), at the
    reference's tolerance (isapprox, rtol 1e-6) and point by point.  The model's
    currents, charges and partials come from the emitted code compiled into the
    oracle, its noise sources from the independent interpreter, the PSD from the
    oracle's dense small-signal solve.  Needs CEDAR_ASAP7_CARD, the path of the
    ASAP7 TT Spectre model cards (CedarSim carries them as
    SpectreNetlistParser.jl/test/examples/7nm_TT.scs).  The same inverter then runs
    the transient of test/bsimcmg/inverter.jl (a 10 mV, 10 MHz input sine about
    0.5 V, 0 .. 400 ns, tolerances 1e-7), which the reference asserts completes."""
    import json
    card = os.environ.get("CEDAR_ASAP7_CARD", "")
    if not card or not pathlib.Path(card).is_file():
        pytest.skip("CEDAR_ASAP7_CARD does not name the ASAP7 TT model cards")
    gold = json.loads((ROOT / "tests" / "golden" / "ac_noise_bsimcmg_ngspice.json").read_text())
    res = scratch(_NOISE_SCRIPT, card, json.dumps(gold["f_hz"]))
    assert res["rc"] == 0 and 0.0 < res["q"] < 1.0
    got, want = np.array(res["sqrt_psd"]), np.array(gold["sqrt_psd"])
    assert np.linalg.norm(got - want) <= 1e-6 * max(np.linalg.norm(got), np.linalg.norm(want))
    assert np.max(np.abs(got - want) / want) <= 1e-7
    # the transient of test/bsimcmg/inverter.jl completes; the output follows the
    # 10 mV input sine inverted and amplified
    rc, status, npts, gain = res["tran"]
    assert rc == 0 and status == 0 and npts > 100 and gain < -1.0
