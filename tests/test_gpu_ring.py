"""Ring-oscillator sweep (15-stage current-starved ring, VA exponential diodes,
RC supply per stage, DC operating point perturbed by N(0, 1 mV) per node) on the
batched GPU engine against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RELTOL, ABSTOL = 1e-6, 1e-9


def _rings(pkg, n):
    tpl, itpl, par, off, dx, dxo = pkg.generators.mc_rings(n)
    f = tpl[0]
    probes = np.array([[f.index("out1"), f.index("out8"), f.index("vdd3")]], np.int32)
    return tpl, itpl, par, off, dx, dxo, probes


def test_ring_batch_matches_oracle(gpu, pkg, oracle):
    tpl, itpl, par, off, dx, dxo, probes = _rings(pkg, 6)
    sw = pkg.Batch(tpl, itpl, par, off, inst_dx=dx, inst_dx_off=dxo, probes=probes, n_samples=61)
    o = pkg.make_opts(tstop=3e-9)
    res = sw.run(o)
    xf, samp, st = oracle.batch(sw.holder, o)
    assert np.all(res.stats["status"] == 0) and np.all(st["status"] == 0)
    for k in ("accepted", "rejected"):
        assert np.array_equal(res.stats[k], st[k]), k
    err = np.abs(res.samples - samp) / (RELTOL * np.abs(samp) + ABSTOL)
    assert err.max() <= 1.0
    # the ring oscillates: out1 swings rail to rail within 3 ns
    s = res.samples[:, 0, :]
    assert np.all(s.max(axis=1) > 1.7) and np.all(s.min(axis=1) < 0.1)


def test_ring_tile_shapes_bitwise(gpu, pkg):
    tpl, itpl, par, off, dx, dxo, probes = _rings(pkg, 12)
    sw = pkg.Batch(tpl, itpl, par, off, inst_dx=dx, inst_dx_off=dxo, probes=probes, n_samples=21)
    o = pkg.make_opts(tstop=1e-9)
    base = None
    for K_, W in [(32, 4), (4, 2), (16, 8)]:
        sw.set_tuning(K_, W)
        r = sw.run(o)
        if base is None:
            base = r
            continue
        assert np.array_equal(r.samples, base.samples)
        assert np.array_equal(r.stats["accepted"], base.stats["accepted"])


def test_ring_dc_single_circuit_path(gpu, pkg, oracle):
    """cedar_dcop on one ring instance: the metastable DC point (output nodes with
    only gmin on their diagonal) needs the dense fallback; it must agree with the
    oracle's partial-pivot solution."""
    tpl, itpl, par, off, dx, dxo, probes = _rings(pkg, 1)
    flat = pkg.generators.instance_flat(tpl[0], par[off[0]:off[0] + tpl[0].param_block().size])
    x = pkg.dc(flat)
    xr, st, rc = oracle.dcop(flat)
    assert rc == 0
    np.testing.assert_allclose(x, xr, rtol=1e-9, atol=1e-12)


def test_batched_dc_operating_points(gpu, pkg, oracle):
    """cedar_batch_dcop (dc!. over a sweep) on ring instances and MC chains
    against the oracle's DC operating point of each instance."""
    tpl, itpl, par, off, dx, dxo, probes = _rings(pkg, 3)
    cases = [(tpl, itpl, par, off, dx, dxo)]
    ct, ci, cp, co = pkg.generators.mc_chains(6, seed=4, lengths=[5, 9, 21])
    cases.append((ct, ci, cp, co, None, None))
    for templates, it, p_, o_, d_, do_ in cases:
        sw = pkg.Batch(templates, it, p_, o_, inst_dx=d_, inst_dx_off=do_)
        x, st = sw.dc()
        assert np.all(st["status"] == 0)
        for i in range(len(it)):
            t = int(it[i])
            flat = pkg.generators.instance_flat(templates[t], p_[o_[i]:o_[i] + templates[t].param_block().size])
            xr, s_, rc = oracle.dcop(flat)
            assert rc == 0
            np.testing.assert_allclose(x[i, :flat.n], xr, rtol=1e-9, atol=1e-12)
