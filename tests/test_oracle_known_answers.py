"""The CPU oracle against the reference's own known answers (CPU only).

Each case rebuilds a circuit from CedarSim's test suite and checks the answer that
test asserts (values in tests/golden/known_answers.json).
"""
import json
import math
import pathlib

import numpy as np
import pytest

from tests import circuits as K

GOLD = json.loads((pathlib.Path(__file__).parent / "golden" / "known_answers.json").read_text())
TOL = 1e-7  # isapprox_deftol: atol = rtol = deftol * 10 (test/common.jl:21-27)


def close(a, b, tol=TOL):
    return abs(a - b) <= tol + tol * abs(b)


def test_vr(pkg, oracle):
    f = K.vr(pkg).flatten()
    x, st, rc = oracle.dcop(f)
    g = GOLD["vr"]
    assert rc == 0
    assert close(x[f.index("vcc")], g["V"]) and close(-x[f.index("V.I")], g["I"])


def test_ir(pkg, oracle):
    f = K.ir(pkg).flatten()
    x, st, rc = oracle.dcop(f)
    assert rc == 0 and close(x[f.index("icc")], GOLD["ir"]["V"])
    assert close(x[f.index("icc")] / 2.0, GOLD["ir"]["I"])


@pytest.mark.parametrize("m", [1.0, 10.0])
def test_vrc_from_zero(pkg, oracle, m):
    f = K.vrc(pkg, m).flatten()
    # u0 = 0 on the capacitor (test passes u0=[0.0]); vcc and the source current are consistent
    x0 = np.zeros(f.n); x0[f.index("vcc")] = 5.0; x0[f.index("V.I")] = -5.0 / 2000.0 * m
    o = pkg.make_opts("bdf2", True, 0.0, 1.0, 0.0, False, reltol=1e-8, abstol_v=1e-10, abstol_i=1e-14)
    t, X, st, rc = oracle.tran(f, o, x0)
    assert rc == 0 and st.status == 0
    vc = X[:, f.index("vrc")]
    ic = -X[:, f.index("V.I")]  # source current = capacitor current (resistor in series)
    g = GOLD["vrc"]
    assert close(ic[0], m * g["i0_per_m"])
    assert close(vc[0], 0.0) and close(vc[-1], g["v_end"])
    assert abs(ic[-1]) < 1e-9


def test_spectre_sources(pkg, oracle):
    f = K.spectre_sources(pkg).flatten()
    o = pkg.make_opts("bdf2", True, 0.0, 1.0, 0.0, True)
    t, X, st, rc = oracle.tran(f, o)
    g = GOLD["spectre_sources"]
    assert rc == 0 and st.status == 0
    assert np.allclose(X[:, f.index("1")], g["node_1"]) and np.allclose(X[:, f.index("3")], g["node_3"])
    assert close(X[-1, f.index("2")], g["node_2_end"]) and close(X[-1, f.index("4")], g["node_4_end"])
    assert close(X[-1, f.index("4")] / 4000.0, g["R4_I_end"])


def test_spice_sources(pkg, oracle):
    f = K.spice_sources(pkg).flatten()
    x, st, rc = oracle.dcop(f)
    g = GOLD["spice_sources"]
    for k in ("5", "6", "8", "7", "9"):
        assert close(x[f.index(k)], g["node_" + k])


def test_multiplicities(pkg, oracle):
    f = K.multiplicities(pkg).flatten()
    x, st, rc = oracle.dcop(f)
    ref = GOLD["multiplicities"]["node"]
    for k in "123456":
        assert abs(x[f.index(k)] - ref) <= 4 * np.spacing(ref)


def test_semiconductor_resistor(pkg, oracle):
    f = K.semiconductor_resistor(pkg).flatten()
    x, st, rc = oracle.dcop(f)
    assert close(-x[f.index("v1.I")], 2 * GOLD["semiconductor_resistor"]["I"])


def test_pwl_transient(pkg, oracle):
    f = K.pwl_isource(pkg).flatten()
    o = pkg.make_opts("bdf2", True, 0.0, 10e-3, 0.0, True)
    t, X, st, rc = oracle.tran(f, o)
    assert rc == 0 and st.status == 0
    want = np.array([K.pwl_val(tt) * 2 * 2 for tt in t])
    assert np.all(np.abs(X[:, f.index("vout")] - want) <= TOL + TOL * np.abs(want))
    # the corners are breakpoints: both are hit exactly
    assert np.any(t == 1e-3) and np.any(t == 9e-3)


def test_pwl_derivative_belongs_to_next_segment(pkg, oracle):
    pts = [(0.0, 0.0), (100e-9, 0.0), (110e-9, 5.0), (200e-9, 5.0), (210e-9, 0.0)]
    c = pkg.Circuit(); c.V("V", "a", "0", wave=pkg.PWL(pts)); c.R("R", "a", "0", r=1.0)
    h = pkg.abi.DescHolder(c.flatten())
    val = lambda t: oracle.lib.oracle_source_value(h.desc, 1, 0, t, 0)
    d = 1e-12
    for t0, slope in GOLD["pwl_derivative"]["slopes"]:
        assert close((val(t0 + d) - val(t0)) / d, slope, 1e-4)


def test_butterworth(pkg, oracle):
    f = K.butterworth(pkg).flatten()
    o = pkg.make_opts("bdf2", True, 0.0, 100.0, 0.0, False, reltol=1e-10, abstol_v=1e-12, abstol_i=1e-14, hmax=0.05)
    t, X, st, rc = oracle.tran(f, o, np.zeros(f.n))
    assert rc == 0 and st.status == 0
    want = np.array([K.butterworth_vout(tt) for tt in t])
    err = np.max(np.abs(X[:, f.index("vout")] - want))
    assert err < GOLD["butterworth"]["max_abs_err"]
    half = X[len(X) // 2:, f.index("vout")]
    assert abs(np.sqrt(np.mean(half ** 2)) - GOLD["butterworth"]["rms"]) <= 0.1 + 0.1 * 0.5


def test_ddx_nlvcr(pkg, oracle):
    f = K.nlvcr(pkg).flatten()
    x, st, rc = oracle.dcop(f)
    # the reference asserts `==` on a symbolically eliminated system; a Newton
    # solution is exact up to the last update's rounding: allow a few ulps
    ref = GOLD["ddx"]["V1_I"]
    assert abs(x[f.index("V1.I")] - ref) <= 8 * np.spacing(abs(ref))


def test_sensitivity_closed_form(pkg, oracle):
    # dV(out)/dR1 = -dV(out)/dR2 = -V(out)/2 at R1 = R2 = 1 (test/sensitivity.jl:35-41)
    def vout(r1, r2):
        f = K.two_resistor(pkg, r1, r2).flatten()
        x, st, rc = oracle.dcop(f)
        return x[f.index("out")]
    v = vout(1.0, 1.0)
    d = 1e-6
    d1 = (vout(1 + d, 1) - vout(1 - d, 1)) / (2 * d)
    d2 = (vout(1, 1 + d) - vout(1, 1 - d)) / (2 * d)
    assert close(d1, -d2, 1e-8) and close(d1, -v / 2, 1e-8)


def test_param_overrides(pkg, oracle):
    """test/params.jl: parameter overrides of a built circuit (ParamSim's role,
    here Circuit.altered).  ParCir (V = 5 across R = 2) with R overridden to 1
    gives V.I = -5; the SPICE deck `i1 vcc 0 'foo'`, `l1 vcc out 1m` and a
    nested subcircuit resistor r1 from out to ground with r = 'foo' and the
    subcircuit default foo = foo + 2000 (global foo = 1) gives V(r1) = -2 with the
    subcircuit's foo set to 2, -4004 with the global foo set to 2, and -100 with
    r1.r set to 100.  The decks' parameter expressions are evaluated here (the
    netlist front end is not part of this path)."""
    g = GOLD["params"]
    par = pkg.Circuit()
    par.V("V", "vcc", "gnd", dc=5.0)
    par.R("R", "vcc", "gnd", r=2.0)
    f = par.altered({"R.r": 1.0}).flatten()
    x, st, rc = oracle.dcop(f)
    assert rc == 0 and close(x[f.index("V.I")], g["V_I"])

    def deck(foo=1.0, sub_foo=None):
        c = pkg.Circuit()
        c.I("i1", "vcc", "0", dc=foo)
        c.L("l1", "vcc", "out", 1e-3)
        c.R("x1.x1.r1", "out", "0", r=(foo + 2000.0) if sub_foo is None else sub_foo)
        return c
    decks = {"sub_foo_2": deck(sub_foo=2.0), "foo_2": deck(foo=2.0), "r_100": deck().altered({"x1.x1.r1.r": 100.0})}
    for key, c in decks.items():
        f = c.flatten()
        x, st, rc = oracle.dcop(f)
        assert rc == 0 and close(x[f.index("out")], g["r1_V"][key]), key


def test_subcircuit_nets(pkg, oracle):
    """test/compilation.jl:58-79: `i1 0 d 1` into a subcircuit whose own d net is
    tied to ground (r1 from that ground to d, 1 Ohm; r2 from ground to ground):
    the nets stay distinct, so i1 carries its 1 A through r1 (V(d) = 1 V)."""
    c = pkg.Circuit()
    c.I("i1", "0", "d", dc=1.0)
    c.R("x1.r1", "0", "d", r=1.0)
    c.R("x1.r2", "0", "0", r=2.0)
    f = c.flatten()
    x, st, rc = oracle.dcop(f)
    assert rc == 0 and close(x[f.index("d")] / 1.0, GOLD["subckt_nets"]["i1_I"])
