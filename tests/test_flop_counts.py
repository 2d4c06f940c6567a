"""The roofline numerator: FP64 work per device evaluation, counted.

cedar_ckt_costs' flops_eval is the sum over a circuit's devices of the FP64
operations one evaluation of each device's model takes in the engines' Newton
iteration.  Those per-model counts are obtained by running the device code itself
(models.cuh and the emitted Verilog-A code) on an op-counting scalar
(cedarsim.jl_gb300/csrc/opcount.cpp: add / sub / mul / div 1, FMA 2, exp / log /
sqrt 1).  This test rebuilds that counter from the committed source, runs it, and
checks that cedar_ckt_costs reports exactly its counts on circuits covering every
built-in and every Verilog-A model; the LU, substitution, stamp and update terms
are counts of the symbolic structure (2 flops per multiply-subtract pair).
"""
import pathlib
import re
import shutil
import subprocess

import pytest

from tests import circuits as K

ROOT = pathlib.Path(__file__).resolve().parents[1]
PKG = ROOT / "cedarsim.jl_gb300"


@pytest.fixture(scope="module")
def counts(pkg, tmp_path_factory):
    pkg.load_library()                      # generates the Verilog-A header the counter includes
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("opcount")
    exe = d / "opcount"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", str(ROOT / "include"), "-I", str(PKG / "csrc"), "-I",
                    str(PKG / "_build" / "gen"), "-o", str(exe), str(PKG / "csrc" / "opcount.cpp")], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    tables = {name: [int(x) for x in body.split(",")]
              for name, body in re.findall(r"k(Builtin|VA)\[\d+\] = \{([^}]*)\}", out)}
    # the library was built with the same table
    assert (PKG / "_build" / "gen" / "flops.gen.h").read_text() == out
    return tables


def _expected(pkg, flat, counts):
    base = pkg.va.BASE_ID
    return sum((counts["Builtin"][m] if m < base else counts["VA"][m - base]) * term.shape[0]
               for (m, term, br, par) in flat.groups)


@pytest.mark.parametrize("case", ["mixed", "va_mixed", "va_vccs", "va_thevenin", "va_diode_rs", "va_nlvcr",
                                  "chain", "ring", "rc_ladder"])
def test_costs_use_counted_flops(pkg, counts, case):
    g = pkg.generators
    mk = {"mixed": lambda: K.mixed(pkg), "va_mixed": lambda: K.va_mixed(pkg), "va_vccs": lambda: K.va_vccs(pkg),
          "va_thevenin": lambda: K.va_thevenin(pkg), "va_diode_rs": lambda: K.va_diode_rs(pkg),
          "va_nlvcr": lambda: K.va_nlvcr(pkg), "chain": lambda: g.inverter_chain(11),
          "ring": lambda: g.ring_oscillator(), "rc_ladder": lambda: g.rc_ladder(20)}[case]
    flat = mk().flatten()
    c = pkg.costs(flat)
    assert c["flops_eval"] == _expected(pkg, flat, counts)


def test_every_model_is_counted(pkg, counts):
    """Every model has a positive count; the dual-number Verilog-A level-1 MOSFET
    costs more than the hand-written one (its partials are carried along)."""
    assert len(counts["Builtin"]) == 11 and all(x > 0 for x in counts["Builtin"][1:])
    assert len(counts["VA"]) == len(pkg.va.models()) and all(x > 0 for x in counts["VA"])
    mos1 = pkg.circuit.MOS1
    assert counts["VA"][pkg.va.model_id("va_mos1") - pkg.va.BASE_ID] > counts["Builtin"][mos1]


def test_counter_builds_with_literal_exponents(pkg, tmp_path):
    """Compact models raise parameters and variables to literal powers
    (BSIM-CMG: pow(NSD / 2.23e22, 0.719)); with every double an op-counting
    scalar those calls mix the scalar with a plain double, which the counter
    resolves exactly (pow, atan2, hypot and fmod), so a library build with such
    a model gets its counts.  The counts follow the rule: one operation per
    pow / atan2 / hypot / divide, on the value and each partial."""
    import importlib
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    P = importlib.import_module("cedarsim_gb300.va.parser")
    E = importlib.import_module("cedarsim_gb300.va.emit")
    src = """module lit(a, b); inout a, b; electrical a, b;
      parameter real NSD = 2e26;
      real x;
      analog begin
        x = pow(NSD / 2.23e22, 0.719) + pow(2.0, NSD * 1e-26) + atan2(NSD, 1.0) + hypot(1.0, NSD);
        I(a, b) <+ 1e-3 * x * 1e-12 * V(a, b);
      end endmodule"""
    mods = [E.analyze(m) for m in P.parse(src)]
    (tmp_path / "va_models.gen.h").write_text(E.emit_header(mods, 11))
    exe = tmp_path / "opcount"
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-I", str(ROOT / "include"), "-I", str(PKG / "csrc"), "-I",
                        str(tmp_path), "-o", str(exe), str(PKG / "csrc" / "opcount.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    va_counts = [int(v) for v in out.split("kVA[1] = {")[1].split("}")[0].split(",")]
    assert len(va_counts) == 1 and va_counts[0] > 0
