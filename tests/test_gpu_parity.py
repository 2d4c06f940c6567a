"""GPU (through the C ABI) against the CPU oracle on the same seeded inputs.

Tolerances (stated by the hot-path contract):
  * device evaluation: F and J entries within 1e-12 relative (row-scaled for sums
    that cancel);
  * waveforms: |gpu - cpu| <= 1e-6 |cpu| + 1e-9 V at matched time points;
  * step sequences (accepted / rejected steps, time points): identical;
  * Newton iteration counts: within 0.5% (DC homotopy paths may differ by rounding).
"""
import numpy as np
import pytest

from tests import circuits as K

pytestmark = pytest.mark.gpu

RTOL_EVAL = 1e-12
STAT_KEYS = ("accepted", "rejected", "newton_iters", "dc_iters", "hmin_seen", "hmax_seen", "status")
RELTOL, ABSTOL = 1e-6, 1e-9


def random_state(flat, rng, scale=1.8):
    x = rng.uniform(-0.2, scale, flat.n)
    x[flat.n_nodes:] = rng.uniform(-1e-3, 1e-3, flat.n - flat.n_nodes)
    return x


EVAL_CASES = {
    "rc_ladder": lambda pkg: pkg.generators.rc_ladder(100),
    "inverter_chain_7": lambda pkg: pkg.generators.inverter_chain(7),
    # supply-rail lists of 200+ entries take the cooperative long-list sums
    "inverter_chain_100": lambda pkg: pkg.generators.inverter_chain(100),
    "mixed": K.mixed,
    "spice_sources": K.spice_sources,
    "nlvcr": K.nlvcr,
}


@pytest.mark.parametrize("case", sorted(EVAL_CASES))
@pytest.mark.parametrize("t", [0.0, 0.13e-9, 0.37e-9])
def test_eval_parity(gpu, pkg, oracle, case, t):
    flat = EVAL_CASES[case](pkg).flatten()
    sys = pkg.System(flat)
    rng = np.random.default_rng(1234)
    for trial in range(4):
        x = random_state(flat, rng)
        xd = rng.normal(0, 1e9, flat.n)
        gamma = 10.0 ** rng.uniform(9, 13)
        F, Jv = sys.eval(x, xd, t, gamma)
        Fr, Fi, Fq, G, Cm = oracle.eval(flat, x, xd, t)
        # row scale: magnitude of the terms summed into each row
        scale = np.abs(G) @ np.abs(x) + np.abs(Cm) @ np.abs(xd) + np.abs(Fi)
        assert np.all(np.abs(F - Fr) <= RTOL_EVAL * (np.abs(Fr) + scale) + 1e-300), case
        J = sys.jac_dense(Jv)
        Jr = G + gamma * Cm
        rows = np.abs(G).max(axis=1, keepdims=True) + gamma * np.abs(Cm).max(axis=1, keepdims=True)
        assert np.all(np.abs(J - Jr) <= RTOL_EVAL * (np.abs(Jr) + 1e-6 * rows) + 1e-300), case
        # pattern covers every nonzero of the oracle's dense Jacobian
        cp, ri = sys.pattern()
        mask = np.zeros_like(Jr, bool)
        for c in range(flat.n):
            mask[ri[cp[c]:cp[c + 1]], c] = True
        assert not np.any((Jr != 0) & ~mask)


@pytest.mark.parametrize("case", ["inverter_chain_7", "mixed", "spice_sources", "nlvcr"])
def test_dcop_parity(gpu, pkg, oracle, case):
    flat = EVAL_CASES[case](pkg).flatten()
    x = pkg.dc(flat)
    xr, st, rc = oracle.dcop(flat)
    assert rc == 0
    assert np.all(np.abs(x - xr) <= 1e-9 * np.abs(xr) + 1e-12)


def compare_waves(sol, t_ref, x_ref, n_nodes):
    assert sol.u.shape == x_ref.shape
    assert np.array_equal(sol.t, t_ref)
    a, b = sol.u[:, :n_nodes], x_ref[:, :n_nodes]
    err = np.abs(a - b) / (RELTOL * np.abs(b) + ABSTOL)
    return err.max()


def test_rc_ladder_trap_full(gpu, pkg, oracle):
    """Workload 1: 100-section RC ladder, trapezoidal, h = 0.1 ns, 0..1 us."""
    flat = pkg.generators.rc_ladder(100).flatten()
    o = pkg.make_opts("trap", False, 0.0, 1e-6, 1e-10, True)
    sol = pkg.tran(flat, (0.0, 1e-6), method="trap", h=1e-10, adaptive=False)
    t_ref, x_ref, st, rc = oracle.tran(flat, o)
    assert rc == 0 and sol.retcode == "OK"
    assert sol.stats["accepted"] == st.accepted == 10000
    assert sol.stats["newton_iters"] == st.newton_iters
    assert compare_waves(sol, t_ref, x_ref, flat.n_nodes) <= 1.0


def test_inverter_chain_bdf2_full(gpu, pkg, oracle):
    """Workload 2: 31-stage inverter chain, BDF2, h = 1 ps, 0..20 ns."""
    flat = pkg.generators.inverter_chain(31).flatten()
    o = pkg.make_opts("bdf2", False, 0.0, 20e-9, 1e-12, True)
    sol = pkg.tran(flat, (0.0, 20e-9), method="bdf2", h=1e-12, adaptive=False)
    t_ref, x_ref, st, rc = oracle.tran(flat, o)
    assert rc == 0 and sol.retcode == "OK"
    assert sol.stats["accepted"] == st.accepted == 20000
    # the DC operating point may take a different homotopy path (rounding in damped
    # Newton differs between the sparse static-pivot LU and the dense oracle LU), so
    # iteration counts are compared loosely; the step sequence is fixed
    assert abs(sol.stats["newton_iters"] - st.newton_iters) <= max(3, 0.005 * st.newton_iters)
    assert compare_waves(sol, t_ref, x_ref, flat.n_nodes) <= 1.0


@pytest.mark.parametrize("case", ["inverter_chain_7", "mixed"])
def test_adaptive_bdf2_parity(gpu, pkg, oracle, case):
    flat = EVAL_CASES[case](pkg).flatten()
    o = pkg.make_opts("bdf2", True, 0.0, 3e-9, 0.0, True)
    sol = pkg.tran(flat, (0.0, 3e-9), method="bdf2")
    t_ref, x_ref, st, rc = oracle.tran(flat, o)
    assert rc == 0 and sol.retcode == "OK"
    assert (sol.stats["accepted"], sol.stats["rejected"]) == (st.accepted, st.rejected)
    assert compare_waves(sol, t_ref, x_ref, flat.n_nodes) <= 1.0


def test_newton_solve_parity(gpu, pkg, oracle):
    flat = pkg.generators.inverter_chain(9).flatten()
    sys = pkg.System(flat)
    x0 = pkg.dc(sys)
    rng = np.random.default_rng(7)
    hist = rng.normal(0, 1e-6, flat.n)
    x, st, rc = sys.newton_solve(1e-11, 1e12, hist, x0)
    xr, str_, rcr = oracle.newton(flat, 1e-11, 1e12, hist, x0)
    assert rc == 0 and rcr == 0 and st.newton_iters == str_.newton_iters
    assert np.all(np.abs(x - xr) <= 1e-9 * np.abs(xr) + 1e-12)


def small_mc(pkg, n_inst=48, seed=11):
    g = pkg.generators
    lengths = [5, 7, 9, 11, 13]
    templates, itpl, par, off = g.mc_chains(n_inst, seed=seed, lengths=lengths)
    probes = np.array([[g.chain_output_probe(f), f.index("in")] for f in templates], np.int32)
    return templates, itpl, par, off, probes


def test_batch_mc_parity(gpu, pkg, oracle):
    templates, itpl, par, off, probes = small_mc(pkg)
    sw = pkg.Batch(templates, itpl, par, off, probes=probes, n_samples=41)
    o = pkg.make_opts("bdf2", True, 0.0, 2e-9, 0.0, True)
    res = sw.run(o)
    xf, samp, st = oracle.batch(sw.holder, o)
    assert np.all(res.stats["status"] == 0) and np.all(st["status"] == 0)
    for k in ("accepted", "rejected"):
        assert np.array_equal(res.stats[k], st[k]), k
    dn = np.abs(res.stats["newton_iters"] - st["newton_iters"])
    assert np.all(dn <= np.maximum(3, 0.005 * st["newton_iters"]))
    err = np.abs(res.samples - samp) / (RELTOL * np.abs(samp) + ABSTOL)
    assert err.max() <= 1.0
    err = np.abs(res.x_final - xf) / (RELTOL * np.abs(xf) + ABSTOL)
    assert err.max() <= 1.0


def test_batch_tile_shapes_bitwise_identical(gpu, pkg):
    """Every lanes-per-instance choice runs the same arithmetic: bitwise-equal results,
    and a rerun is bitwise equal too (fixed-order reductions, no atomics)."""
    templates, itpl, par, off, probes = small_mc(pkg, n_inst=40, seed=5)
    sw = pkg.Batch(templates, itpl, par, off, probes=probes, n_samples=21)
    o = pkg.make_opts("bdf2", True, 0.0, 1.5e-9, 0.0, True)
    base = None
    for K_, W in [(1, 2), (2, 4), (4, 4), (8, 4), (16, 8), (32, 2), (8, 4)]:
        sw.set_tuning(K_, W)
        r = sw.run(o)
        if base is None:
            base = r
            continue
        assert np.array_equal(r.samples, base.samples)
        assert np.array_equal(r.x_final, base.x_final)
        for k in STAT_KEYS:
            assert np.array_equal(r.stats[k], base.stats[k]), k


def test_batch_windows_match_uninterrupted_run(gpu, pkg):
    """Advancing in time windows (soft stops, state kept on the device) reproduces
    an uninterrupted run bit for bit."""
    import ctypes as C
    templates, itpl, par, off, probes = small_mc(pkg, n_inst=24, seed=3)
    o = pkg.make_opts("bdf2", True, 0.0, 1.2e-9, 0.0, True)
    sw = pkg.Batch(templates, itpl, par, off, probes=probes, n_samples=25)
    full = sw.run(o)
    lib = sw.lib
    pkg.abi.check(lib.cedar_batch_start(sw.handle, C.byref(o)))
    nrun = C.c_int32()
    edges = [0.1e-9, 0.35e-9, 0.7e-9, 1.2e-9]
    for k, e in enumerate(edges):
        pkg.abi.check(lib.cedar_batch_advance(sw.handle, e, C.byref(nrun)))
        if k < len(edges) - 1:
            assert nrun.value == sw.n_inst
    assert nrun.value == 0
    xf = np.zeros_like(full.x_final)
    samp = np.zeros_like(full.samples)
    st = np.zeros_like(full.stats)
    pkg.abi.check(lib.cedar_batch_results(sw.handle, xf.ctypes.data_as(C.POINTER(C.c_double)),
                                          samp.ctypes.data_as(C.POINTER(C.c_double)), st.ctypes.data_as(C.c_void_p)))
    assert np.array_equal(xf, full.x_final)
    assert np.array_equal(samp, full.samples)
    for k in STAT_KEYS:
        assert np.array_equal(st[k], full.stats[k]), k


def test_autotune_picks_a_shape_and_caches_it(gpu, pkg, tmp_path):
    """cedar_batch_autotune times every tile shape; the host caches the choice per
    GPU, instance count and template sizes, and a second call reuses it."""
    import json
    templates, itpl, par, off, probes = small_mc(pkg, n_inst=64, seed=8)
    sw = pkg.Batch(templates, itpl, par, off)
    o = pkg.make_opts("bdf2", True, 0.0, 1e-9, 0.0, True)
    cache = str(tmp_path / "tune.json")
    k, w = sw.autotune(o, 0.05e-9, cache=cache)
    assert k in (1, 2, 4, 8, 16, 32) and 1 <= w <= 8
    assert sw.tuning == (k, w)
    table = json.load(open(cache))
    assert list(table.values()) == [[k, w]]
    sw2 = pkg.Batch(templates, itpl, par, off)
    assert sw2.autotune(o, 0.05e-9, cache=cache) == (k, w) and sw2.tuning == (k, w)
    r = sw2.run(o)
    assert np.all(r.stats["status"] == 0)
