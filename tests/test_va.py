"""Verilog-A front end and emitter on the CPU.

* The emitted device code (compiled into the oracle library) against an
  independent interpretation of the same parsed modules (oracle/va_interp.py)
  at random port potentials in every operating region.
* The Verilog-A restatements of the built-in models (R, C, diode, level-1 MOSFET,
  NLVCR) against the built-in equations, through the oracle's circuit
  evaluation.
* Known answers: test/ddx.jl (the NLVCR source current is -60 A) and
  test/varegress.jl (a resistor written in either orientation carries the same,
  non-negative current).
* Parameter defaults, ranges and the errors of the supported subset.
"""
import ctypes as C
import importlib.util
import pathlib

import numpy as np
import pytest

from tests import circuits as K

ROOT = pathlib.Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def va(pkg):
    import importlib
    return importlib.import_module("cedarsim_gb300.va")


@pytest.fixture(scope="module")
def interp():
    spec = importlib.util.spec_from_file_location("cedar_va_interp", ROOT / "oracle" / "va_interp.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


VT = 1.380649e-23 * (27.0 + 273.15) / 1.602176634e-19


def _params(m, rng):
    """Random in-range parameter values around the declared defaults."""
    out = {}
    for p in m.params:
        d = m.defaults()[m.param_index(p.name)]
        if p.name == "TYPE":
            out[p.name] = float(rng.choice([-1.0, 1.0]))
        elif p.name in ("VTO",):
            out[p.name] = float(rng.uniform(-0.6, 0.6))
        elif p.name in ("LAMBDA", "TT", "CJ0"):
            out[p.name] = float(rng.choice([0.0, abs(d) + 1e-3 * rng.uniform(0.5, 2.0)])) if p.name == "LAMBDA" \
                else float(rng.choice([0.0, rng.uniform(1e-15, 1e-11)]))
        elif p.name == "MODE":
            out[p.name] = float(rng.integers(0, 3))
        elif p.name == "R":
            out[p.name] = float(rng.uniform(0.5, 5.0) * (1 if rng.random() < 0.8 else -1))
        else:
            out[p.name] = float(d * rng.uniform(0.5, 2.0)) if d else float(rng.uniform(0.5, 2.0))
    return out


def test_emitted_code_matches_interpreter(pkg, oracle, va, interp):
    rng = np.random.default_rng(42)
    lib = oracle.lib
    dp_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    for k, m in enumerate(va.models()):
        n = m.nx                  # terminals, then the branch current of a voltage branch
        for trial in range(60):
            prm = _params(m, rng)
            vals = m.defaults(prm)
            mult = float(rng.choice([1.0, 2.0]))
            dp = np.array(vals + [mult, VT])
            v = rng.uniform(-2.0, 2.0, n)
            if m.name.startswith("va_diode"):
                v[0] = v[1] + rng.uniform(-1.0, 0.9)     # keep exp() finite but exercise forward bias
            fi, fq, G, Cm = np.zeros(n), np.zeros(n), np.zeros(n * n), np.zeros(n * n)
            assert lib.oracle_va_full(k, dp_(dp), dp_(v), 1e-12, dp_(fi), dp_(fq), dp_(G), dp_(Cm)) == 0
            given = [g for g in m.given if g in prm]
            ri, rq, rG, rC = interp.evaluate(m.module, dict(zip([p.name for p in m.params], vals)), list(v), VT,
                                             1e-12, mult, given)
            ri, rq, rG, rC = np.array(ri), np.array(rq), np.array(rG).ravel(), np.array(rC).ravel()
            sc = np.abs(ri).max() + 1e-30
            assert np.all(np.abs(fi - ri) <= 1e-13 * sc), (m.name, fi, ri)
            assert np.all(np.abs(fq - rq) <= 1e-13 * (np.abs(rq).max() + 1e-40)), (m.name, fq, rq)
            gs = np.abs(rG).max() + 1e-30
            assert np.all(np.abs(G - rG) <= 1e-12 * gs), (m.name, G, rG)
            cs = np.abs(rC).max() + 1e-40
            assert np.all(np.abs(Cm - rC) <= 1e-12 * cs), (m.name, Cm, rC)


def test_restated_models_match_interpreter(pkg, oracle, va, interp):
    """Every shipped module is restated by hand in the oracle (the evaluation the
    GPU's Verilog-A runs are checked against), and each restatement equals the
    interpreter at random points in every region: two evaluations that share no
    code with the emitter."""
    rng = np.random.default_rng(7)
    lib = oracle.lib
    dp_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    shipped = {p.stem for p in (ROOT / "cedarsim.jl_gb300" / "va" / "models").glob("*.va")}
    for k, m in enumerate(va.models()):
        n = m.nx
        vals0 = m.defaults({})
        dp = np.array(vals0 + [1.0, VT])
        fi, fq, G, Cm = np.zeros(n), np.zeros(n), np.zeros(n * n), np.zeros(n * n)
        restated = lib.oracle_va_ref_full(k, dp_(dp), len(vals0) + 1, dp_(np.zeros(n)), 1e-12, dp_(fi), dp_(fq),
                                          dp_(G), dp_(Cm))
        assert restated == (1 if m.name in shipped else 0), m.name
        if not restated:
            continue
        for trial in range(60):
            prm = _params(m, rng)
            vals = m.defaults(prm)
            mult = float(rng.choice([1.0, 2.0]))
            dp = np.array(vals + [mult, VT])
            v = rng.uniform(-2.0, 2.0, n)
            if m.name.startswith("va_diode"):
                v[0] = v[1] + rng.uniform(-1.0, 0.9)
                if n > 2:
                    v[2] = v[1] + rng.uniform(-1.0, 0.9)
            fi, fq, G, Cm = np.zeros(n), np.zeros(n), np.zeros(n * n), np.zeros(n * n)
            assert lib.oracle_va_ref_full(k, dp_(dp), len(vals) + 1, dp_(v), 1e-12, dp_(fi), dp_(fq), dp_(G),
                                          dp_(Cm)) == 1
            given = [g for g in m.given if g in prm]
            ri, rq, rG, rC = interp.evaluate(m.module, dict(zip([p.name for p in m.params], vals)), list(v), VT,
                                             1e-12, mult, given)
            ri, rq, rG, rC = np.array(ri), np.array(rq), np.array(rG).ravel(), np.array(rC).ravel()
            sc = np.abs(ri).max() + 1e-30
            assert np.all(np.abs(fi - ri) <= 1e-13 * sc), (m.name, fi, ri)
            assert np.all(np.abs(fq - rq) <= 1e-13 * (np.abs(rq).max() + 1e-40)), (m.name, fq, rq)
            assert np.all(np.abs(G - rG) <= 1e-12 * (np.abs(rG).max() + 1e-30)), (m.name, G, rG)
            assert np.all(np.abs(Cm - rC) <= 1e-12 * (np.abs(rC).max() + 1e-40)), (m.name, Cm, rC)


def _builtin_twin(pkg, which):
    """A circuit with built-in devices and its twin with the Verilog-A models."""
    def mk(vamodels):
        c = pkg.Circuit()
        c.V("VDD", "vdd", "0", dc=1.8)
        c.V("VIN", "in", "0", dc=0.7)
        if which == "mos":
            for k, (d, g, s, typ, W, KP, VTO, lam) in enumerate([("o", "in", "0", 1.0, 2e-6, 2e-4, 0.45, 0.02),
                                                                  ("o", "in", "vdd", -1.0, 4e-6, 8e-5, -0.45, 0.0),
                                                                  ("p", "o", "0", 1.0, 3e-6, 2e-4, 0.4, 0.01)]):
                if vamodels:
                    c.va(f"M{k}", "va_mos1", [d, g, s, s], TYPE=typ, W=W, L=1e-6, KP=KP, VTO=VTO, LAMBDA=lam,
                         m=1.0 + k)
                else:
                    c.mos1(f"M{k}", d, g, s, s, typ, W, 1e-6, KP, VTO, LAMBDA=lam, m=1.0 + k)
            c.R("RL", "p", "vdd", r=1e4)
        elif which == "passive":
            (c.va("R1", "va_resistor", ["in", "o"], R=1e3, m=3.0) if vamodels else c.R("R1", "in", "o", r=1e3, m=3.0))
            (c.va("C1", "va_capacitor", ["o", "0"], C=2e-12) if vamodels else c.C("C1", "o", "0", 2e-12))
            (c.va("D1", "va_diode", ["o", "vdd"], IS=1e-15, N=1.1, AREA=2.0) if vamodels
             else c.diode("D1", "o", "vdd", IS=1e-15, N=1.1, AREA=2.0))
        elif which == "nlvcr":
            (c.va("X", "va_nlvcr", ["vdd", "in", "0"], R=2.0) if vamodels else c.nlvcr("X", "vdd", "in", "0", R=2.0))
        return c.flatten()
    return mk(False), mk(True)


@pytest.mark.parametrize("which", ["mos", "passive", "nlvcr"])
def test_va_models_match_builtins(pkg, oracle, which):
    fb, fv = _builtin_twin(pkg, which)
    assert fb.names == fv.names
    rng = np.random.default_rng(7)
    for _ in range(40):
        x = rng.uniform(-0.5, 2.0, fb.n)
        x[fb.n_nodes:] = rng.uniform(-1e-3, 1e-3, fb.n - fb.n_nodes)
        xd = rng.normal(0, 1e9, fb.n)
        Fb, Fib, Fqb, Gb, Cb = oracle.eval(fb, x, xd)
        Fv, Fiv, Fqv, Gv, Cv = oracle.eval(fv, x, xd)
        sc = np.abs(Gb) @ np.abs(x) + np.abs(Fib) + 1e-30
        assert np.all(np.abs(Fiv - Fib) <= 1e-13 * sc)
        assert np.all(np.abs(Fqv - Fqb) <= 1e-13 * (np.abs(Cb) @ np.abs(x) + 1e-40))
        assert np.all(np.abs(Gv - Gb) <= 1e-12 * (np.abs(Gb).max(axis=1, keepdims=True) + 1e-30))
        assert np.all(np.abs(Cv - Cb) <= 1e-12 * (np.abs(Cb).max() + 1e-40))


def test_ddx_known_answer(pkg, oracle):
    """test/ddx.jl: I(d,s) <+ V(d,s) * ddx(R V(g,s)^2, V(g,s)) with V(d)=5, V(g)=3,
    R=2 gives a source current of -5*2*2*3."""
    f = K.va_nlvcr(pkg).flatten()
    x, st, rc = oracle.dcop(f)
    assert rc == 0
    assert abs(x[f.index("V1.I")] - (-60.0)) <= 8 * np.spacing(60.0)


def test_resistor_orientation_regression(pkg, oracle, va, interp):
    """test/varegress.jl: a resistor written I(n,p) <+ V(n,p)/R is the same device
    as I(p,n) <+ V(p,n)/R; in the V-R-C circuit its current stays non-negative."""
    src = """
    `include "disciplines.vams"
    module rev_r(p, n); inout p, n; electrical p, n; parameter real R = 1000.0 from (0.0:inf];
      analog I(n, p) <+ V(n, p) / R;
    endmodule"""
    rev = va.parse(src)[0]
    fwd = va.model(va.model_id("va_resistor"))
    for v in ([1.0, 0.25], [-0.3, 0.8], [0.0, 0.0]):
        a = interp.evaluate(rev, {"R": 1e3}, v, VT, 1e-12)
        b = interp.evaluate(fwd.module, {"R": 1e3}, v, VT, 1e-12)
        assert np.allclose(a[0], b[0], rtol=0, atol=1e-18) and np.allclose(a[2], b[2], rtol=0, atol=1e-18)
    from cedarsim_gb300.va.emit import analyze
    mr, _ = analyze(rev)
    assert (mr.frows, mr.gents, mr.qrows, mr.cents) == (fwd.frows, fwd.gents, fwd.qrows, fwd.cents)
    # V(1) -> R(1k) -> out, C(1n) to ground, 0..10 us: branch current >= 0 throughout
    c = pkg.Circuit()
    c.V("V", "vcc", "gnd", dc=1.0)
    c.va("R", "va_resistor", ["vcc", "out"], R=1000.0)
    c.C("C", "out", "gnd", 1e-9)
    f = c.flatten()
    o = pkg.make_opts("bdf2", True, 0.0, 1e-5, 0.0, False)
    t, X, st, rc = oracle.tran(f, o, np.zeros(f.n))
    assert rc == 0 and st.status == 0
    i_r = (X[:, f.index("vcc")] - X[:, f.index("out")]) / 1000.0
    assert np.all(i_r[1:] >= 0.0) and X[-1, f.index("out")] == pytest.approx(1.0, abs=1e-3)


def test_parameters_and_circuit_api(pkg, va):
    m = va.model(va.model_id("va_mos1"))
    assert m.ports == ["d", "g", "s", "b"] and m.npar == 7
    assert m.defaults() == [1.0, 1e-6, 1e-6, 2e-5, 0.7, 0.0]
    assert m.defaults({"W": 3e-6})[1] == 3e-6
    with pytest.raises(va.VAError):
        m.defaults({"TYPE": 0.0})          # excluded value
    with pytest.raises(va.VAError):
        m.defaults({"W": -1.0})            # outside (0:inf)
    with pytest.raises(va.VAError):
        m.defaults({"WIDTH": 1.0})         # unknown parameter
    c = pkg.Circuit()
    with pytest.raises(ValueError):
        c.va("M", "va_mos1", ["a", "b", "c"])
    with pytest.raises(KeyError):
        c.va("M", "no_such_model", ["a", "b"])
    c.va("M", "va_mos1", ["d", "g", "0", "0"], W=2e-6, m=3.0)
    f = c.flatten()
    model, term, br, par = f.groups[0]
    assert model == va.model_id("va_mos1") and br is None
    assert par[:, 0].tolist() == [1.0, 2e-6, 1e-6, 2e-5, 0.7, 0.0, 3.0]
    assert term[0].tolist() == [f.index("d"), f.index("g"), -1, -1]


def test_library_lists_the_models(pkg, va):
    lib = pkg.load_library()
    assert lib.cedar_va_count() == len(va.models())
    buf = C.create_string_buffer(64)
    for k, m in enumerate(va.models()):
        assert lib.cedar_va_name(k, buf, 64) == 0 and buf.value.decode() == m.name
        mid = va.BASE_ID + k
        assert lib.cedar_model_nterm(mid) == m.nterm and lib.cedar_model_npar(mid) == m.npar
        assert lib.cedar_model_has_branch(mid) == m.has_br
    assert lib.cedar_va_name(len(va.models()), buf, 64) != 0
    assert lib.cedar_model_nterm(va.BASE_ID + len(va.models())) == -1


@pytest.mark.parametrize("src, msg", [
    ("module m(a, b); inout a, b; electrical a, b, x1, x2, x3, x4, x5, x6, x7; analog I(a, b) <+ V(a, b); "
     "endmodule", "at most"),
    ("module m(a, b); inout a, b; electrical a, b; integer i; analog begin for (i = 0; i < 2; i = i + 1) "
     "I(a, b) <+ V(a, b) + white_noise(1e-20, \"n\"); end endmodule", "inside a loop"),
    ("module m(a, b); inout a, b; electrical a, b; analog I(a, b) <+ foo(V(a, b)); endmodule", "unsupported function"),
    ("module m(a, b); inout a, b; electrical a, b; analog I(a, b) <+ V(a, b) * ddt(V(a, b)); endmodule",
     "factor of ddt"),
    ("module m(a, b); inout a, b; electrical a, b; analog I(a, b) <+ exp(ddt(V(a, b))); endmodule", "additive"),
    ("module m(a, b); inout a, b; electrical a, b; analog I(a, c) <+ V(a, b); endmodule", "not a port"),
    ("module m(a, b); inout a, b; electrical a, b; analog begin x = 1; I(a, b) <+ x; end endmodule", "undeclared"),
    ("module m(a, b); inout a, b; electrical a, b; parameter real R = 1; analog begin R = 2; I(a, b) <+ R; end "
     "endmodule", "parameter"),
])
def test_subset_errors(va, src, msg):
    from cedarsim_gb300.va.emit import _Emitter, analyze
    with pytest.raises(va.VAError, match=msg):
        for mod in va.parse(src):
            m, a = analyze(mod)
            _Emitter(m, a).body()


def test_parser_details(va):
    src = """
    `include "disciplines.vams"
    `include "constants.vams"
    `define TWO 2.0
    module t(p, n);
      inout p, n; electrical p, n;
      parameter integer K = 3 from [1:10];
      parameter real G0 = 1m, G1 = G0 * `TWO;
      real g; integer i;
      analog begin : blk
        i = K / 2;                 // integer division
        g = (i == 1) ? G1 : G0;    /* ternary, comparison */
        if (V(p, n) > 0.5 && !(K < 2)) g = g + 1u;
        I(p, n) <+ g * V(p, n) + 1e-3 * M_PI * 0;
      end
    endmodule"""
    mod = va.parse(src)[0]
    from cedarsim_gb300.va.emit import analyze
    m, _ = analyze(mod)
    assert m.defaults() == [3.0, 1e-3, 2e-3]
    assert m.gents == [(0, 0), (0, 1), (1, 0), (1, 1)]


def test_range_bounds_take_the_rounding_of_scale_factors(va):
    """A scale-factor literal is the decimal times the factor, as the reference
    converts it (0.1n = 0.1 * 1e-9 = 1.0000000000000001e-10, src/vasim.jl:114-126),
    so a value written 1e-10 (the ASAP7 cards' EOTACC against BSIM-CMG's
    `from [0.1n:inf)`) meets an inclusive bound up to that rounding; values
    clearly outside, and an exclusive bound, are still refused."""
    from cedarsim_gb300.va.emit import analyze
    from cedarsim_gb300.va.parser import VAError
    src = """module rb(p, n); inout p, n; electrical p, n;
      parameter real T = 1n from [0.1n:inf);
      parameter real U = 1n from (0.1n:1u];
      parameter real W = 1 exclude 0.3n;
      analog I(p, n) <+ V(p, n) * (T + U + W);
    endmodule"""
    m, _ = analyze(va.parse(src)[0])
    assert 0.1 * 1e-9 != 1e-10
    assert m.defaults({"T": 1e-10})[0] == 1e-10
    assert m.defaults({"U": 1e-6})[1] == 1e-6
    for bad in ({"T": 0.99e-10}, {"U": 1e-10}, {"U": 1.01e-6}, {"W": 3e-10}):
        with pytest.raises(VAError):
            m.defaults(bad)


def test_internal_node_model_equals_its_expanded_network(pkg, oracle, va):
    """va_diode_rs (RS to an internal node, the junction behind it) is the same
    network as va_resistor + va_diode around an explicit node: same unknowns
    (the internal node is named "<instance>.<node>"), same F, J, DC point and
    waveform."""
    m = va.model(va.model_id("va_diode_rs"))
    assert m.ports == ["a", "c"] and m.internals == ["ai"] and m.nterm == 3
    fa, fb = K.va_diode_rs(pkg).flatten(), K.va_diode_rs(pkg, twin=True).flatten()
    assert fa.names == fb.names and "D1.ai" in fa.names
    rng = np.random.default_rng(3)
    for _ in range(20):
        x = rng.uniform(-1.0, 1.0, fa.n)
        _, Fia, _, Ga, _ = oracle.eval(fa, x, t=0.3e-9)
        _, Fib, _, Gb, _ = oracle.eval(fb, x, t=0.3e-9)
        sc = np.abs(Gb) @ np.abs(x) + np.abs(Fib)
        assert np.all(np.abs(Fia - Fib) <= 1e-13 * sc + 1e-300)
        assert np.all(np.abs(Ga - Gb) <= 1e-13 * np.abs(Gb).max(axis=1, keepdims=True) + 1e-300)
    o = pkg.make_opts("bdf2", False, 0.0, 1.2e-9, 1e-12, True)
    ta, Xa, sa, ra = oracle.tran(fa, o)
    tb, Xb, sb, rb = oracle.tran(fb, o)
    assert ra == 0 and rb == 0 and np.array_equal(ta, tb)
    assert np.max(np.abs(Xa - Xb) / (1e-9 * np.abs(Xb) + 1e-12)) <= 1.0
    # the diode conducts through RS on the high phase: ai sits below x
    k = np.searchsorted(ta, 0.5e-9)
    assert Xa[k, fa.index("x")] - Xa[k, fa.index("D1.ai")] > 1e-3


def test_functions_macros_case_and_param_given(pkg, oracle, va):
    """va_vccs_sat uses an analog function, function-like macros, case, an
    @(initial_step) block, $strobe, $param_given and a white_noise source: its
    current is gm f(V(cp,cn)) with f per MODE, gm = GMX where the instance sets
    it, and no noise contribution outside a noise analysis."""
    import math
    k = va.model_id("va_vccs_sat") - va.BASE_ID
    m = va.models()[k]
    assert m.given == ["GMX"] and m.npar == 6
    lib = oracle.lib
    dp_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    vs = 0.4
    for mode, f in ((0, lambda x: x), (1, lambda x: vs * math.tanh(x / vs)), (2, lambda x: x / math.sqrt(1 + (x / vs) ** 2))):
        for given, gm in ((False, 2e-3), (True, 5e-3)):
            over = {"GM": 2e-3, "VS": vs, "MODE": mode}
            if given:
                over["GMX"] = 5e-3
            dp = np.array(m.defaults(over) + [1.0, VT])
            for vc in (-0.9, -0.1, 0.0, 0.25, 1.3):
                v = np.array([0.7, 0.2, vc + 0.1, 0.1])
                fi, fq, G, Cm = np.zeros(4), np.zeros(4), np.zeros(16), np.zeros(16)
                assert lib.oracle_va_full(k, dp_(dp), dp_(v), 1e-12, dp_(fi), dp_(fq), dp_(G), dp_(Cm)) == 0
                want = gm * f(vc)
                assert fi[0] == pytest.approx(-want, rel=1e-14, abs=1e-30) and fi[1] == pytest.approx(want, rel=1e-14,
                                                                                                      abs=1e-30)
                h = 1e-6
                slope = gm * (f(vc + h) - f(vc - h)) / (2 * h)
                assert -G[0 * 4 + 2] == pytest.approx(slope, rel=1e-7) and G[0 * 4 + 3] == pytest.approx(slope, rel=1e-7)
    # instance parameters and the given flag through the circuit API
    c = pkg.Circuit()
    c.va("X1", "va_vccs_sat", ["a", "0", "b", "0"], GM=1e-3)
    c.va("X2", "va_vccs_sat", ["a", "0", "b", "0"], GMX=3e-3, MODE=2)
    f = c.flatten()
    assert f.groups[0][3][:, 0].tolist() == [1e-3, 0.0, 0.5, 1.0, 0.0, 1.0]
    assert f.groups[0][3][:, 1].tolist() == [1e-3, 3e-3, 0.5, 2.0, 1.0, 1.0]


def test_preprocessor_and_statement_forms(va):
    src = r"""
    `define SQ(x) ((x)*(x))
    `define CLIP(x, lo, hi) (((x) < (lo)) ? (lo) : (((x) > (hi)) ? (hi) : (x)))
    `define LONG(a, b) (`SQ(a) + \
                        `SQ(b))
    `ifdef NOT_DEFINED
      `define GAIN 100.0
    `elsif SQ
      `define GAIN 2.0
    `else
      `define GAIN 3.0
    `endif
    module pp(p, n); inout p, n; electrical p, n;
      parameter integer K = 2;
      real g;
      analog begin
        case (K) 1, 2: g = `GAIN; default: g = 0; endcase
        @(final_step) $strobe("never");
        I(p, n) <+ g * `CLIP(V(p, n), -1, 1) + 1e-3 * `LONG(V(p, n), 1.0) + flicker_noise(1e-20, 1.0, "f");
      end
    endmodule"""
    mod = va.parse(src)[0]
    from cedarsim_gb300.va.emit import analyze
    m, _ = analyze(mod)
    assert m.gents == [(0, 0), (0, 1), (1, 0), (1, 1)]
    with pytest.raises(va.VAError, match="takes 2 arguments"):
        va.parse("`define F(a, b) a+b\nmodule m(p); inout p; electrical p; analog I(p) <+ `F(1); endmodule")
    with pytest.raises(va.VAError, match="endif"):
        va.parse("`ifdef X\nmodule m(p); inout p; electrical p; analog I(p) <+ 1; endmodule")
    with pytest.raises(va.VAError, match="not an argument or local"):
        src2 = """module m(p); inout p; electrical p; parameter real R = 1;
          analog function real f; input x; real x; f = x * R; endfunction
          analog I(p) <+ f(V(p)); endmodule"""
        for mm in va.parse(src2):
            analyze(mm)


def test_voltage_branch_models(pkg, oracle, va):
    """V(a,b) <+ contributions add a branch-current unknown "<instance>.I":
    va_inductor is the built-in inductor (same F, G, C with m = 1), the Butterworth
    of test/transients.jl built with it meets the same analytic answer, and the
    Thevenin source divides 1 V over its 50 Ohm and the load."""
    import json
    m = va.model(va.model_id("va_inductor"))
    assert m.has_br == 1 and m.nx == 3
    fb, fv = K.butterworth(pkg).flatten(), K.butterworth_va(pkg).flatten()
    assert fb.names == fv.names
    rng = np.random.default_rng(11)
    for _ in range(20):
        x = rng.uniform(-1.0, 1.0, fb.n)
        xd = rng.normal(0, 1.0, fb.n)
        Fb, Fib, Fqb, Gb, Cb = oracle.eval(fb, x, xd, t=0.7)
        Fv, Fiv, Fqv, Gv, Cv = oracle.eval(fv, x, xd, t=0.7)
        for a, b in ((Fiv, Fib), (Fqv, Fqb), (Gv, Gb), (Cv, Cb), (Fv, Fb)):
            assert np.all(np.abs(a - b) <= 1e-14 * (np.abs(b) + 1.0))
    gold = json.load(open(ROOT / "tests" / "golden" / "known_answers.json"))["butterworth"]
    o = pkg.make_opts("bdf2", True, 0.0, 100.0, 0.0, False, reltol=1e-10, abstol_v=1e-12, abstol_i=1e-14, hmax=0.05)
    t, X, st, rc = oracle.tran(fv, o, np.zeros(fv.n))
    assert rc == 0 and st.status == 0
    err = np.max(np.abs(X[:, fv.index("vout")] - np.array([K.butterworth_vout(tt) for tt in t])))
    assert err < gold["max_abs_err"]
    f = K.va_thevenin(pkg).flatten()
    x, st, rc = oracle.dcop(f)
    assert rc == 0
    rp = 50.0 * 1e3 / (50.0 + 1e3)        # the inductor shorts RB across RL at DC
    va_ = rp / (50.0 + rp)
    assert x[f.index("a")] == pytest.approx(va_, rel=1e-12) and x[f.index("VT.I")] == pytest.approx(-va_ / rp, rel=1e-12)
    assert x[f.index("LX.I")] == pytest.approx(x[f.index("b")] / 1e3, rel=1e-9)


def test_voltage_branch_errors(va):
    from cedarsim_gb300.va.emit import analyze
    two = """module m(a, b, c); inout a, b, c; electrical a, b, c;
      analog begin V(a, b) <+ 0; V(b, c) <+ 0; end endmodule"""
    with pytest.raises(va.VAError, match="second voltage"):
        analyze(va.parse(two)[0])
    mixed = """module m(a, b); inout a, b; electrical a, b;
      analog begin V(a, b) <+ 0; I(a, b) <+ V(a, b); end endmodule"""
    with pytest.raises(va.VAError, match="current and voltage"):
        analyze(va.parse(mixed)[0])
    probe = """module m(a, b); inout a, b; electrical a, b; analog I(a, b) <+ I(a, b); endmodule"""
    with pytest.raises(va.VAError, match="probes no voltage"):
        analyze(va.parse(probe)[0])


def test_white_noise_sources(pkg, oracle, va, interp):
    """white_noise powers from the emitted code equal the interpreter's; the
    Butterworth of test/ac.jl with Verilog-A resistors (thermal noise written as
    white_noise(4 k T / R)) gives the built-in resistors' PSD and the reference's
    ngspice table (rtol 1e-6, test/ac.jl:148-149)."""
    import json
    lib = oracle.lib
    dp_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    rng = np.random.default_rng(17)
    for name in ("va_resistor", "va_vccs_sat"):
        k = va.model_id(name) - va.BASE_ID
        m = va.models()[k]
        assert len(m.noise) == 1
        for _ in range(10):
            prm = _params(m, rng)
            vals = m.defaults(prm)
            v = rng.uniform(-1, 1, m.nx)
            pw, ex = np.zeros(len(m.noise)), np.full(len(m.noise), np.nan)
            assert lib.oracle_va_noise(k, dp_(np.array(vals + [1.0, VT])), dp_(v), 1e-12, dp_(pw),
                                       dp_(ex)) == len(m.noise)
            src = interp.noise_sources(m.module, dict(zip([p.name for p in m.params], vals)), list(v), VT, 1e-12,
                                       1.0, [g for g in m.given if g in prm])
            assert [s[0] for s in src] == m.noise
            assert pw[0] == pytest.approx(src[0][1], rel=1e-14)
            assert ex[0] == src[0][2] == 0.0
    fb, fv = K.butterworth_ac(pkg).flatten(), K.butterworth_ac_va(pkg).flatten()
    x, _, rc = oracle.dcop(fb)
    assert rc == 0
    w = 2 * np.pi * pkg.acdec(20, 0.01, 10)
    pb = oracle.noise(fb, x, w, fb.index("vout"))
    pv = oracle.noise(fv, x, w, fv.index("vout"))
    np.testing.assert_allclose(pv, pb, rtol=1e-12)
    g = json.loads((ROOT / "tests" / "golden" / "ac_noise_ngspice.json").read_text())
    ref = np.array(g["sqrt_psd"])
    assert np.all(np.abs(np.sqrt(pv) - ref) <= 1e-6 * np.maximum(np.abs(ref), np.abs(np.sqrt(pv))))


def test_flicker_noise(pkg, oracle, va, interp):
    """flicker_noise(pwr, ex) is a noise source of density pwr / f^ex (PSD,
    src/ac.jl:267-276): the emitted code and the interpreter agree on power and
    exponent, and a divider of a 1/f resistor over a plain one has the analytic
    output PSD (R1 || R2)^2 (4kT/R1 + 4kT/R2 + KF |I|^AF / f^EF)."""
    lib = oracle.lib
    dp_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    k = va.model_id("va_resistor_1f") - va.BASE_ID
    m = va.models()[k]
    assert len(m.noise) == 2 and m.noise[0] == m.noise[1] == (0, 1)
    prm = {"R": 3e3, "KF": 2e-21, "AF": 1.7, "EF": 1.1}
    vals = m.defaults(prm)
    v = np.array([0.4, -0.2])
    pw, ex = np.zeros(2), np.zeros(2)
    assert lib.oracle_va_noise(k, dp_(np.array(vals + [1.0, VT])), dp_(v), 1e-12, dp_(pw), dp_(ex)) == 2
    src = interp.noise_sources(m.module, dict(zip([p.name for p in m.params], vals)), list(v), VT, 1e-12, 1.0,
                               [g for g in m.given if g in prm])
    i = 0.6 / 3e3
    assert [s[2] for s in src] == [0.0, 1.1] and list(ex) == [0.0, 1.1]
    np.testing.assert_allclose(pw, [s[1] for s in src], rtol=1e-14)
    assert pw[1] == pytest.approx(2e-21 * i ** 1.7, rel=1e-13)

    R1, R2, KF, AF, EF, vdd = 3e3, 1e3, 1e-19, 2.0, 1.0, 2.0
    c = pkg.Circuit(temp_c=27.0, gmin=0.0)
    c.V("V1", "vin", "0", dc=vdd)
    c.va("R1", "va_resistor_1f", ["vin", "out"], R=R1, KF=KF, AF=AF, EF=EF)
    c.R("R2", "out", "0", R2)
    f = c.flatten()
    x, _, rc = oracle.dcop(f)
    assert rc == 0
    hz = np.array([0.1, 1.0, 10.0, 1e3, 1e6])
    psd = oracle.noise(f, x, 2 * np.pi * hz, f.index("out"))
    kT4 = 4 * 1.380649e-23 * (27.0 + 273.15)
    rp = R1 * R2 / (R1 + R2)
    want = rp ** 2 * (kT4 / R1 + kT4 / R2 + KF * (vdd / (R1 + R2)) ** AF / hz ** EF)
    np.testing.assert_allclose(psd, want, rtol=1e-10)
    # zero KF leaves the thermal noise of the two resistors only
    c0 = pkg.Circuit(temp_c=27.0, gmin=0.0)
    c0.V("V1", "vin", "0", dc=vdd)
    c0.va("R1", "va_resistor_1f", ["vin", "out"], R=R1)
    c0.R("R2", "out", "0", R2)
    f0 = c0.flatten()
    np.testing.assert_allclose(oracle.noise(f0, x, 2 * np.pi * hz, f0.index("out")),
                               rp ** 2 * (kT4 / R1 + kT4 / R2), rtol=1e-10)


def test_limit_and_step_advice(va):
    """$limit(x, ...) is x; $bound_step / $discontinuity compile to nothing."""
    from cedarsim_gb300.va.emit import analyze
    src = """module lim(a, c); inout a, c; electrical a, c; parameter real IS = 1e-14;
      real vd;
      analog begin
        vd = $limit(V(a, c), "pnjlim", $vt, 0.6);
        $bound_step(1e-12);
        $discontinuity(0);
        I(a, c) <+ IS * (limexp(vd / $vt) - 1.0);
      end endmodule"""
    m, _ = analyze(va.parse(src)[0])
    assert m.gents == [(0, 0), (0, 1), (1, 0), (1, 1)]
    body = va.parse(src)[0].body
    assert len(body) == 2     # the assignment and the contribution


def test_cli_reports_and_emits(tmp_path):
    """va/cli.py: a summary per module, the header with --emit, exit 1 on a module
    outside the subset."""
    import subprocess
    import sys
    cli = ROOT / "cedarsim.jl_gb300" / "va" / "cli.py"
    out = tmp_path / "h.h"
    r = subprocess.run([sys.executable, str(cli), str(ROOT / "cedarsim.jl_gb300" / "va" / "models" / "va_inductor.va"),
                        "--emit", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "module va_inductor" in r.stdout and "branch unknowns 1" in r.stdout
    assert "body_va_inductor" in out.read_text()
    bad = tmp_path / "bad.va"
    bad.write_text("module m(a, b); inout a, b; electrical a, b; analog I(a, b) <+ foo(V(a, b)); endmodule\n")
    r = subprocess.run([sys.executable, str(cli), str(bad)], capture_output=True, text=True)
    assert r.returncode == 1 and "unsupported function" in r.stderr
