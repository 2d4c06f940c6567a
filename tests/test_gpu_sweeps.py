"""dc!. / tran!. over a CircuitSweep on the GPU: every point in one batched launch.

Mirrors the reference's sweep tests that solve circuits (test/sweep.jl:319-371):
the two-resistor divider over a 20 x 20 product of R1, R2 (source current
-1/(R1 + R2)) and a nested-parameter circuit (current v_in / x1.r_load).  A
transient sweep over an inverter chain's load and supply is checked against the
oracle's batch run on the same instance tables."""
import numpy as np
import pytest

from tests.test_sweeps import two_resistor

pytestmark = pytest.mark.gpu

RELTOL, ABSTOL = 1e-6, 1e-9


def test_dc_sweep_two_resistors(gpu, pkg):
    r = np.arange(100.0, 2001.0, 100.0)
    cs = pkg.CircuitSweep(two_resistor, pkg.ProductSweep(R1=r, R2=r))
    sols = pkg.dc(cs, reltol=1e-10)
    assert sols.shape == (20, 20)
    for sol, sim in zip(sols.ravel(order="F"), cs):
        assert sol.retcode == "OK"
        R1, R2 = sim.params.R1, sim.params.R2
        assert sol["V.I"] == pytest.approx(-1.0 / (R1 + R2), rel=1e-9)
        assert sol["out"] == pytest.approx(R2 / (R1 + R2), rel=1e-9)


def test_dc_sweep_nested_parameters(gpu, pkg):
    def circuit(v_in=1.0, x1=None):
        x1 = dict({"r_load": 1.0}, **(x1 or {}))
        c = pkg.Circuit()
        c.R("x1.r1", "vss", "0", r=x1["r_load"])
        c.V("v1", "vss", "0", dc=v_in)
        return c
    cs = pkg.CircuitSweep(circuit, pkg.ProductSweep(v_in=np.arange(1.0, 11.0), **{"x1.r_load": np.arange(1.0, 11.0)}))
    sols = pkg.dc(cs, reltol=1e-10)
    assert sols.shape == (10, 10)
    for sol in sols.ravel():
        v_in, r_load = sol.params.v_in, sol.params.x1.r_load
        assert -sol["v1.I"] == pytest.approx(v_in / r_load, rel=1e-9)


def test_tran_sweep_matches_oracle(gpu, pkg, oracle):
    g = pkg.generators

    def chain(cload=10e-15, vdd=1.8, stages=5):
        return g.inverter_chain(int(stages), cload=cload, vdd=vdd)

    sweep = pkg.ProductSweep(cload=[5e-15, 10e-15, 20e-15], vdd=[1.5, 1.8],
                             stages=[3, 5])                      # two topologies
    cs = pkg.CircuitSweep(chain, sweep)
    probes = ["in", "out3"]
    tspan = (0.0, 1.5e-9)
    sols = pkg.tran(cs, tspan, probes=probes, n_samples=31)
    assert sols.shape == (3, 2, 2)

    flats = [s.build().flatten() for s in cs]
    tpl, itpl, par, off = pkg.sweeps.batch_tables(flats)
    assert len(tpl) == 2
    pidx = np.array([[t.index(p) for p in probes] for t in tpl], np.int32)
    holder = pkg.abi.BatchHolder(tpl, itpl, par, off, probes=pidx, n_samples=31)
    o = pkg.make_opts("bdf2", True, tspan[0], tspan[1], 0.0, True, RELTOL, ABSTOL)
    xf, samp, st = oracle.batch(holder, o)
    assert np.all(st["status"] == 0)
    for i, sol in enumerate(sols.ravel(order="F")):
        assert sol.retcode == "OK"
        assert sol.stats["accepted"] == st["accepted"][i] and sol.stats["rejected"] == st["rejected"][i]
        err = np.abs(sol.u.T - samp[i]) / (RELTOL * np.abs(samp[i]) + ABSTOL)
        assert err.max() <= 1.0, (i, err.max())
    # the supply sweep shows in the high level of the last output
    hi = np.array([s["out3"].max() for s in sols.ravel(order="F")])
    vdd = np.array([s.params.vdd for s in sols.ravel(order="F")])
    assert np.all(np.abs(hi - vdd) < 0.05)
