"""Checks at the workloads' own sizes: the 4096-chain Monte Carlo transient over
0..20 ns, the DC operating points of all 1024 ring oscillators, and the adjoint
over the full 20 ns horizon.

The oracle cannot rerun 4096 instances inside a test, so the full run is checked
through properties every instance must satisfy (finished, finite, inside the
rails, the output switching with the input pulse) and against oracle waveforms
on a seeded random sample of 8 instances (86 k to 185 k accepted steps each).
"""
import copy

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RELTOL, ABSTOL = 1e-6, 1e-9
TSTOP = 20e-9


def test_mc4096_full_run_properties_and_sampled_parity(gpu, pkg, oracle):
    g = pkg.generators
    templates, itpl, par, off = g.mc_chains(4096)
    probes = np.array([[g.chain_output_probe(f), f.index("in")] for f in templates], np.int32)
    ns = 101
    o = pkg.make_opts("bdf2", True, 0.0, TSTOP, 0.0, True, reltol=RELTOL, abstol_v=ABSTOL, hmax=TSTOP / 50)
    sw = pkg.Batch(templates, itpl, par, off, probes=probes, n_samples=ns)
    r = sw.run(o)
    st = r.stats
    assert np.all(st["status"] == 0)
    assert st["accepted"].min() >= 50                  # hmax = tstop / 50 bounds every step
    out, inp = r.samples[:, 0, :], r.samples[:, 1, :]
    assert np.all(np.isfinite(r.samples)) and np.all(np.isfinite(r.x_final))
    assert out.min() > -0.2 and out.max() < 2.0                                # inside the rails
    assert np.all(out.max(axis=1) > 1.6) and np.all(out.min(axis=1) < 0.2)    # every chain switches
    assert np.all(inp[:, 0] == 0.0) and np.all(inp.max(axis=1) > 1.79)

    sel = np.sort(np.random.default_rng(11).choice(4096, size=8, replace=False))
    sub = pkg.abi.BatchHolder(templates, itpl[sel], par, off[sel], probes=probes, n_samples=ns)
    xf, samp, sto = oracle.batch(sub, o)
    assert np.all(sto["status"] == 0)
    acc, acc_o = st["accepted"][sel], sto["accepted"]
    rej, rej_o = st["rejected"][sel], sto["rejected"]
    err = np.abs(r.samples[sel] - samp) / (RELTOL * np.abs(samp) + ABSTOL)
    info = (acc.tolist(), acc_o.tolist(), rej.tolist(), rej_o.tolist(), err.max(axis=(1, 2)).tolist())
    assert np.array_equal(acc, acc_o) and np.array_equal(rej, rej_o), info
    assert err.max() <= 1.0, info


def test_rings_full_set_dc_points(gpu, pkg, oracle):
    """All 1024 ring instances reach their DC operating point (metastable points
    included, through the dense-pivoting rerun); a sample agrees with the oracle."""
    tpl, itpl, par, off, dx, dxo = pkg.generators.mc_rings(1024)
    sw = pkg.Batch(tpl, itpl, par, off, inst_dx=dx, inst_dx_off=dxo)
    x, st = sw.dc()
    assert np.all(st["status"] == 0)
    assert np.all(np.isfinite(x))
    for i in (0, 511, 1023):
        flat = pkg.generators.instance_flat(tpl[0], par[off[i]:off[i] + tpl[0].param_block().size])
        xr, _, rc = oracle.dcop(flat)
        assert rc == 0
        np.testing.assert_allclose(x[i, :flat.n], xr, rtol=1e-9, atol=1e-12)


def test_adjoint_full_horizon(gpu, pkg, oracle):
    """One L = 31 adjoint instance (62 widths, ~93 k accepted steps) over 0..20 ns:
    the GPU gradient against the oracle's adjoint on the same step sequence, and
    against central differences (step 1e-6 W) on 8 sampled widths, with the GPU's
    own accepted steps replayed by the oracle; agreement 1e-5 relative."""
    templates, itpl, par, off, objs, tstar = pkg.generators.adjoint_chains(1, seed=20240607, lengths=[31])
    sw = pkg.Batch(templates, itpl, par, off)
    objective = pkg.abi.Objective(*[int(v) for v in objs[0][:3]], 0, *[float(v) for v in objs[0][3:]])
    o = pkg.make_opts(tstop=TSTOP, hmax=TSTOP / 50)
    rep = pkg.make_opts(tstop=TSTOP, hmax=TSTOP / 50, nr_factor=1e-5)
    r = sw.adjoint(o, [objective], tstar)
    assert r.status[0] == 0
    flat = pkg.generators.instance_flat(templates[0], par[off[0]:off[0] + templates[0].param_block().size])
    T, ords = sw.tape(0)
    assert len(T) == r.stats["accepted"][0] and len(T) > 50000

    phi, g, To, ords_o = oracle.adjoint(flat, o, o, objective, float(tstar[0]))
    assert len(To) == len(T) and np.array_equal(ords_o, ords), (len(To), len(T))
    assert r.phi[0] == pytest.approx(phi, rel=1e-9)
    gg = r.grad[0, :len(g)]
    assert np.all(np.abs(gg - g) <= 1e-7 * np.abs(g) + 1e-9 * np.max(np.abs(g))), (gg, g)

    mos = [gi for gi, gr in enumerate(flat.groups) if gr[0] == 8][0]
    pick = np.sort(np.random.default_rng(3).choice(flat.groups[mos][3].shape[1], size=8, replace=False))
    for k in pick:
        f2 = copy.deepcopy(flat)
        w0 = f2.groups[mos][3][1, k]
        d = 1e-6 * w0
        f2.groups[mos][3][1, k] = w0 + d
        pp = oracle.replay_phi(f2, rep, T, ords, objective, float(tstar[0]))
        f2.groups[mos][3][1, k] = w0 - d
        pm = oracle.replay_phi(f2, rep, T, ords, objective, float(tstar[0]))
        fd = (pp - pm) / (2 * d)
        assert abs(r.grad[0, k] - fd) <= 1e-5 * abs(fd), (k, r.grad[0, k], fd)
