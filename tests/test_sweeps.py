"""Sweep specifications, parameter lists and the batch-table builder on the CPU.

The cases restate the reference's own sweep tests (test/sweep.jl): nest and
flatten parameter lists (:31-70), Sweep / ProductSweep / TandemSweep /
SerialSweep and their compositions (:72-202), alter on named tuples (:204-208),
split_axes (:210-241), CircuitSweep shapes and nested selectors (:243-317),
find_param_ranges (:373-397) and sweepify (:399-407)."""
import dataclasses
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def sw(pkg):
    import importlib
    return importlib.import_module("cedarsim_gb300.sweeps")


def two_resistor(R1=1000.0, R2=1000.0):
    """TwoResistorCircuit (test/sweep.jl:8-27): V = 1 on vcc, R1 vcc-out, R2 out-gnd."""
    import __graft_entry__ as ge
    c = ge.load().Circuit()
    c.V("V", "vcc", "gnd", dc=1.0)
    c.R("R1", "vcc", "out", r=R1)
    c.R("R2", "out", "gnd", r=R2)
    return c


def test_nest_and_flatten_param_lists(sw):
    d = {"R1": 1, "x1.R3": 2, "x1.x2.R1": 3, "x1.x2.R2": 4}
    t = (("R1", 1.0), ("x1.R3", 2), ("x1.x2.R1", 3), ("x1.x2.R2", 4))
    nested = {"R1": 1, "x1": {"x2": {"R2": 4, "R1": 3}, "R3": 2}}
    assert sw.nest_param_list(d) == nested
    assert sw.nest_param_list(t) == nested
    assert sw.flatten_param_list(nested) == t
    assert sw.flatten_param_list(sw.nest_param_list(t)) == t
    with pytest.raises(ValueError):
        sw.nest_param_list((("x1", 1), ("x1.R1", 2)))
    with pytest.raises(ValueError):
        sw.nest_param_list((("x1", 1), ("x1", 2)))


def test_sweep_1d(sw):
    s = sw.Sweep("R1", np.round(np.arange(1, 11) * 0.1, 12))
    assert len(s) == 10 and s.size() == (10,) and s.size(1) == 10 and s.size(2) == 1
    assert next(iter(s)) == (("R1", 0.1),)
    assert sw.Sweep(R1=np.round(np.arange(1, 11) * 0.1, 12)) == s
    assert sw.Sweep(("R1", np.round(np.arange(1, 11) * 0.1, 12))) == s
    assert next(iter(sw.Sweep(**{"a.b": [1.0, 2.0]}))) == (("a.b", 1.0),)
    s = sw.Sweep(a=10.0)
    assert len(s) == 1 and s.size() == (1,) and s.size(2) == 1 and next(iter(s)) == (("a", 10.0),)
    with pytest.raises(ValueError):
        sw.Sweep(a=1.0, b=2.0)
    assert sw.Sweep(r1=[1, 2, 3]) == sw.Sweep(r1=[1, 2, 3])


def test_product_tandem_serial(sw):
    s = sw.ProductSweep(R1=[1.0, 2.0], R2=[1.0, 2.0], R3=[1.0, 2.0])
    assert s.size() == (2, 2, 2) and s.size(3) == 2 and s.size(4) == 1
    assert next(iter(s)) == (("R1", 1.0), ("R2", 1.0), ("R3", 1.0))
    assert sw.sweepvars(s) == {"R1", "R2", "R3"}
    # first axis fastest (column-major)
    pts = list(s)
    assert pts[1] == (("R1", 2.0), ("R2", 1.0), ("R3", 1.0))
    assert pts[2] == (("R1", 1.0), ("R2", 2.0), ("R3", 1.0))

    e = sw.ProductSweep()
    assert e.size() == () and not sw.sweepvars(e) and next(iter(e)) == ()

    s = sw.TandemSweep(R1=[1.0, 2.0], R2=[1.0, 2.0], R3=[1.0, 2.0])
    assert s.size() == (2,) and s.size(2) == 1
    assert list(s) == [(("R1", 1.0), ("R2", 1.0), ("R3", 1.0)), (("R1", 2.0), ("R2", 2.0), ("R3", 2.0))]
    with pytest.raises(ValueError):
        sw.TandemSweep(R1=[1.0, 2.0], R2=[1.0])

    s = sw.SerialSweep(R1=[1.0, 2.0], R2=[1.0, 2.0])
    assert s.size() == (4,)
    assert list(s) == [(("R1", 1.0), ("R2", None)), (("R1", 2.0), ("R2", None)),
                       (("R1", None), ("R2", 1.0)), (("R1", None), ("R2", 2.0))]
    e = sw.SerialSweep()
    assert e.size() == (0,) and len(e) == 0 and not sw.sweepvars(e)


def test_compositions(sw):
    a = sw.ProductSweep(sw.ProductSweep(R1=[1.0, 2.0], R2=[1.0, 2.0]), R3=[1.0, 2.0])
    b = sw.ProductSweep(R1=[1.0, 2.0], R2=[1.0, 2.0], R3=[1.0, 2.0])
    assert list(a) == list(b) and a.size() == (2, 2, 2)

    s = sw.ProductSweep(sw.TandemSweep(R1=[1.0, 2.0], R2=[1.0, 2.0]), R3=[1.0, 2.0])
    g = sw.grid(s)
    assert g.shape == (2, 2)
    assert g[0, 0] == (("R1", 1.0), ("R2", 1.0), ("R3", 1.0))
    assert g[0, 1] == (("R1", 1.0), ("R2", 1.0), ("R3", 2.0))
    assert g[1, 0] == (("R1", 2.0), ("R2", 2.0), ("R3", 1.0))
    assert g[1, 1] == (("R1", 2.0), ("R2", 2.0), ("R3", 2.0))

    s = sw.ProductSweep(sw.SerialSweep(R3=[1.0, 2.0], R4=[1.0, 2.0]), R1=[1.0, 2.0], R2=[1.0, 2.0])
    assert s.size() == (4, 2, 2)
    exp = []
    for r2 in (1.0, 2.0):
        for r1 in (1.0, 2.0):
            for r3, r4 in ((1.0, None), (2.0, None), (None, 1.0), (None, 2.0)):
                exp.append((("R1", r1), ("R2", r2), ("R3", r3), ("R4", r4)))
    assert list(s) == exp
    assert sw.sweepvars(s) == {"R1", "R2", "R3", "R4"}

    # one sweep in a combinator is just that sweep
    assert sw.ProductSweep(r1=range(1, 11)) == sw.Sweep(r1=range(1, 11))
    assert sw.SerialSweep(r1=range(1, 11)) == sw.Sweep(r1=range(1, 11))
    assert sw.TandemSweep(r1=range(1, 11)) == sw.Sweep(r1=range(1, 11))
    assert isinstance(repr(s), str)


def test_alter(sw):
    p = {"r": 1, "cap": 1e-12}
    assert sw.alter(p, next(iter(sw.Sweep(cap=1e-13)))) == {"r": 1, "cap": 1e-13}
    assert sw.alter(p, next(iter(sw.ProductSweep(r=range(2, 4), cap=1e-13)))) == {"r": 2, "cap": 1e-13}
    assert p == {"r": 1, "cap": 1e-12}  # not mutated

    @dataclasses.dataclass
    class Inner:
        a: float = 1.0
        b: float = 2.0

    @dataclasses.dataclass
    class Outer:
        x: Inner = dataclasses.field(default_factory=Inner)
        y: float = 3.0

    o = sw.alter(Outer(), (("x.b", 7), ("y", None)))
    assert o.x.b == 7.0 and isinstance(o.x.b, float) and o.y == 3.0 and Outer().x.b == 2.0


def test_split_axes(sw):
    ps = sw.ProductSweep(A=range(1, 11), B=range(1, 11), C=range(1, 6), D=range(1, 6))
    for axes in (["A", "C"], ("A", "C"), {"A", "C"}):
        outer, inner = sw.split_axes(ps, axes)
        assert sw.sweepvars(outer) == {"B", "D"} and sw.sweepvars(inner) == {"A", "C"}
        assert outer.size() == (10, 5) and inner.size() == (10, 5)
        ps2 = sw.ProductSweep(outer, inner)
        assert sw.sweepvars(ps2) == sw.sweepvars(ps) and ps2.size() != ps.size()
        assert sorted(ps2) == sorted(ps)
        with pytest.raises(ValueError):
            sw.split_axes(ps, ["E"])
        with pytest.raises(ValueError):
            sw.split_axes(sw.SerialSweep(A=range(10), B=range(10)), ["A"])


def test_circuit_sweep_shapes(sw):
    cs = sw.CircuitSweep(two_resistor, sw.Sweep(R1=np.arange(1.0, 11.0)))
    assert len(cs) == 10 and cs.size() == (10,)
    assert next(iter(cs)).params.R1 == 1.0
    cs = sw.CircuitSweep(two_resistor, sw.ProductSweep(R1=np.arange(1.0, 11.0), R2=np.arange(1.0, 11.0)))
    assert len(cs) == 100 and cs.size() == (10, 10) and cs.collect().shape == (10, 10)
    first = next(iter(cs))
    assert first.params.R1 == 1.0 and first.params.R2 == 1.0
    assert sw.sweepvars(cs.iterator) == {"R1", "R2"}
    f = first.build().flatten()
    assert f.groups[0][3][0].tolist() == [1.0, 1.0]  # both resistors at the swept values

    @dataclasses.dataclass
    class Nested:
        a: float
        b: object

    @dataclasses.dataclass
    class NestedCircuitParams:
        a: Nested = dataclasses.field(default_factory=lambda: Nested(1.0, 2.0))
        b: Nested = dataclasses.field(default_factory=lambda: Nested(3.0, Nested(4.0, 5.0)))

        def __call__(self):
            import __graft_entry__ as ge
            c = ge.load().Circuit()
            c.V("V", "vcc", "gnd", dc=self.a.a + self.b.b.a)
            c.R("R", "vcc", "gnd", r=1.0)
            return c

    sweep = sw.ProductSweep(sw.TandemSweep(**{"a.a": [1.0, 2.0], "a.b": [1.0, 2.0]}),
                            sw.SerialSweep(**{"b.a": [1.0, 2.0], "b.b.a": [2.0, 3.0]}))
    assert isinstance(repr(sweep), str)
    cs = sw.CircuitSweep(NestedCircuitParams, sweep)
    assert len(cs) == 8 and cs.size() == (2, 4)
    first = next(iter(cs))
    assert first.params.a.a == 1 and first.params.a.b == 1 and first.params.b.a == 1
    last = cs.collect()[-1, -1]
    assert last.params.b.b.a == 3
    # the default b.b.a = 4 holds where the serial sweep leaves it unset
    src = first.build().devices[0]
    assert src.params[1] == 1.0 + 4.0
    assert sw.sweepvars(cs.iterator) == {"a.a", "a.b", "b.a", "b.b.a"}


def test_find_param_ranges(sw):
    params = sw.ProductSweep(
        sw.ProductSweep(sw.SerialSweep(sw.Sweep(a=range(1, 11)), sw.Sweep(a=range(11, 21))), b=range(1, 6, 2)),
        sw.ProductSweep(sw.TandemSweep(c=range(1, 11), d=range(1, 11)), sw.SerialSweep(c=range(11, 16), d=range(1, 6))))
    r = sw.find_param_ranges(params)
    assert r["a"] == (1, 20, 20) and r["b"] == (1, 5, 3) and r["c"] == (1, 15, 15) and r["d"] == (1, 10, 15)


def test_sweepify(sw):
    s1 = sw.sweepify([{"r1": range(1, 11), "r2": range(1, 7)}, {"r3": range(1, 5), "r4": range(1, 3)}])
    s2 = sw.SerialSweep(sw.ProductSweep(r1=range(1, 11), r2=range(1, 7)), sw.ProductSweep(r3=range(1, 5), r4=range(1, 3)))
    assert list(s1) == list(s2)
    s1 = sw.sweepify([("r1", range(1, 11)), ("r2", range(1, 11))])
    assert list(s1) == list(sw.SerialSweep(r1=range(1, 11), r2=range(1, 11)))


def test_batch_tables_group_by_topology(sw, pkg):
    """Points that differ only in values share a template; a structural change
    (a different source waveform kind keeps the template, a different device set
    does not) opens a new one; parameter blocks land at their offsets."""
    def ckt(R1=1000.0, extra=0.0):
        c = two_resistor(R1=R1)
        if extra:
            c.C("Cx", "out", "gnd", c=extra)
        return c
    cs = sw.CircuitSweep(ckt, sw.ProductSweep(R1=[1.0, 2.0, 3.0], extra=[0.0, 1e-12]))
    flats = [s.build().flatten() for s in cs]
    tpl, itpl, par, off = sw.batch_tables(flats)
    assert len(tpl) == 2 and itpl.tolist() == [0, 0, 0, 1, 1, 1]
    for i, f in enumerate(flats):
        b = f.param_block()
        assert np.array_equal(par[off[i]:off[i] + b.size], b)


def test_csv_export(sw, pkg, tmp_path):
    sol = pkg.Solution(np.array([0.0, 1e-9]), np.array([[1.0, 0.5, -1e-3], [1.0, 0.25, -2e-3]]),
                       ["vcc", "node_out", "V.I"], {}, "OK")
    p = sw.write_csv(str(tmp_path / "w.csv"), sol)
    rows = open(p).read().strip().splitlines()
    assert rows[0] == "t,vcc,out"
    assert [float(v) for v in rows[2].split(",")] == [1e-9, 1.0, 0.25]
    p = sw.write_csv(str(tmp_path / "w2.csv"), sol, name_map={"V.I": "I(V)"})
    assert open(p).read().splitlines()[0] == "t,I(V)"
    assert sw.default_name_map(["gnd", "a", "node_a", "node_b"]) == {"a": "a", "node_a": "node_a", "node_b": "b"}
    assert math.isfinite(float(rows[1].split(",")[0]))


class _OracleBatch:
    """Stand-in for the GPU Batch with the same constructor and dc/tran methods,
    run by the CPU oracle, so the sweep broadcasts' host logic (tables, probe
    maps, result shapes) is exercised without a GPU."""
    oracle = None

    def __init__(self, templates, itpl, par=None, off=None, probes=None, n_samples=0):
        import __graft_entry__ as ge
        self.pkg = ge.load()
        self.holder = self.pkg.abi.BatchHolder(templates, itpl, par, off, probes=probes, n_samples=n_samples)
        self.templates, self.itpl, self.par, self.off = templates, itpl, par, off
        self.n_max = max(t.n for t in templates)

    def dc(self, reltol=1e-6, abstol_v=1e-9, **kw):
        import copy
        x = np.zeros((len(self.itpl), self.n_max))
        st = np.zeros(len(self.itpl), self.pkg.abi.STATS_DTYPE)
        for i, t in enumerate(self.itpl):
            f = copy.deepcopy(self.templates[t])
            pos = self.off[i]
            for k, grp in enumerate(f.groups):
                p = self.par[pos:pos + grp[3].size].reshape(grp[3].shape)
                f.groups[k] = (grp[0], grp[1], grp[2], p.copy())
                pos += grp[3].size
            xi, s, rc = self.oracle.dcop(f, opts=self.pkg.make_opts(tstop=1.0, reltol=reltol, abstol_v=abstol_v))
            assert rc == 0
            x[i, :f.n] = xi
            st[i]["status"] = s.status
        return x, st

    def tran(self, tspan, method="bdf2", reltol=1e-6, abstol_v=1e-9, dcop=True, **kw):
        from cedarsim_gb300.api import BatchResult
        o = self.pkg.make_opts(method, True, tspan[0], tspan[1], 0.0, dcop, reltol, abstol_v)
        xf, samp, st = self.oracle.batch(self.holder, o)
        return BatchResult(xf, samp, st)


def test_sweep_broadcasts_host_logic(sw, pkg, oracle, monkeypatch):
    import cedarsim_gb300.api as api
    _OracleBatch.oracle = oracle
    monkeypatch.setattr(api, "Batch", _OracleBatch)
    r = [100.0, 300.0, 1000.0]
    cs = sw.CircuitSweep(two_resistor, sw.ProductSweep(R1=r, R2=r[:2]))
    sols = pkg.dc(cs, reltol=1e-10)
    assert sols.shape == (3, 2)
    for (i, j), sol in np.ndenumerate(sols):
        assert sol.params.R1 == r[i] and sol.params.R2 == r[j]
        assert sol["V.I"] == pytest.approx(-1.0 / (r[i] + r[j]), rel=1e-9)

    def chain(cload=10e-15, stages=3):
        return pkg.generators.inverter_chain(int(stages), cload=cload)
    cs = sw.CircuitSweep(chain, sw.ProductSweep(cload=[5e-15, 20e-15], stages=[3, 5]))
    sols = pkg.tran(cs, (0.0, 0.3e-9), probes=["in", "out3"], n_samples=7)
    assert sols.shape == (2, 2)
    s = sols[1, 1]
    assert s.params.cload == 20e-15 and s.params.stages == 5 and s.u.shape == (7, 2)
    assert s.t[0] == 0.0 and s.t[-1] == 0.3e-9 and s.retcode == "OK"
    assert s["in"][-1] == pytest.approx(1.8)


def test_sweep_over_verilog_a_parameters(sw, pkg, oracle, monkeypatch):
    """A SerialSweep leaves the other variable at None (its default): through
    ParamSim the circuit function does not set it, so $param_given sees it unset.
    va_vccs_sat's gm is GMX where given, else GM; its output current into a 1 kOhm
    load follows (host logic run by the oracle stand-in)."""
    import math
    import cedarsim_gb300.api as api
    _OracleBatch.oracle = oracle
    monkeypatch.setattr(api, "Batch", _OracleBatch)

    def ckt(GM=None, GMX=None):
        c = pkg.Circuit()
        c.V("VC", "c", "0", dc=0.3)
        kw = {k: v for k, v in (("GM", GM), ("GMX", GMX)) if v is not None}
        c.va("G", "va_vccs_sat", ["0", "o", "c", "0"], VS=0.5, MODE=1, **kw)
        c.R("RL", "o", "0", r=1e3)
        return c
    cs = sw.CircuitSweep(ckt, sw.SerialSweep(GMX=[2e-3], GM=[1e-3, 3e-3]))
    pts = list(cs.iterator)
    assert pts == [(("GM", None), ("GMX", 2e-3)), (("GM", 1e-3), ("GMX", None)), (("GM", 3e-3), ("GMX", None))]
    sols = pkg.dc(cs, reltol=1e-10)
    f = 0.5 * math.tanh(0.3 / 0.5)
    for sol, gm in zip(sols.ravel(order="F"), (2e-3, 1e-3, 3e-3)):
        assert sol["o"] == pytest.approx(gm * f * 1e3, rel=1e-9)


def test_sweep_device_parameters_of_a_built_circuit(sw, pkg, oracle, monkeypatch):
    """A CircuitSweep over a built Circuit alters its devices by DEVICE.parameter
    names (built-in and Verilog-A parameters, multiplicity, a DC source's value);
    the original circuit is left unchanged."""
    import cedarsim_gb300.api as api
    _OracleBatch.oracle = oracle
    monkeypatch.setattr(api, "Batch", _OracleBatch)
    c = pkg.Circuit()
    c.V("V", "vcc", "0", dc=1.0)
    c.R("R1", "vcc", "out", r=1e3)
    c.va("R2", "va_resistor", ["out", "0"], R=1e3)
    cs = sw.CircuitSweep(c, sw.ProductSweep(**{"R1.r": [1e3, 3e3], "R2.R": [1e3, 2e3], "V.dc": [1.0, 2.0]}))
    sols = pkg.dc(cs, reltol=1e-10)
    assert sols.shape == (2, 2, 2)
    for (i, j, k), sol in np.ndenumerate(sols):
        r1, r2, vdc = [1e3, 3e3][i], [1e3, 2e3][j], [1.0, 2.0][k]
        assert sol["out"] == pytest.approx(vdc * r2 / (r1 + r2), rel=1e-9)
        assert sol.params.R1.r == r1
    assert c.device("R1").params[0] == 1e3 and c.device("V").params[1] == 1.0
    c2 = c.altered({"R1.m": 2.0})
    assert c2.device("R1").params[1] == 2.0 and c.device("R1").params[1] == 1.0
    with pytest.raises(KeyError):
        c.altered({"R1.q": 1.0})
    with pytest.raises(KeyError):
        c.altered({"R9.r": 1.0})
    g = pkg.Circuit()
    g.va("G", "va_vccs_sat", ["0", "o", "c", "0"])
    g2 = g.altered({"G.GMX": 4e-3})
    mod = pkg.va.model(pkg.va.model_id("va_vccs_sat"))
    assert g2.device("G").params[len(mod.params)] == 1.0 and g.device("G").params[len(mod.params)] == 0.0
