"""The single-circuit engine on a whole cooperative grid (large circuits).

The grid engine runs the CTA engine's algorithm with every block of a
cooperative grid as one thread group (grid-wide barriers, reductions combined in
block order), so it takes the CTA engine's decisions: the same accepted steps and
the same waveforms.  Checked on a 300-stage chain against the CTA engine and the
oracle, and on a 20 000-stage chain (n = 20 004, which AUTO sends to the grid)
against the CTA engine, with more than one block in the launch; the DC operating
point (from the chain's logic levels) and one Newton solve through the grid
engine as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CTA, GRID = 2, 3


def _run(pkg, sys_, engine, opts, cap, x0=None):
    lib = sys_.lib
    pkg.abi.check(lib.cedar_ckt_set_engine(sys_.handle, engine, 0))
    x = np.zeros(sys_.n) if x0 is None else x0.copy()
    t_out, x_out = np.zeros(cap), np.zeros((cap, sys_.n))
    cnt, st = C.c_int64(), pkg.abi.Stats()
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    pkg.abi.check(lib.cedar_tran_run(sys_.handle, C.byref(opts), dp(x), dp(t_out), dp(x_out), cap, C.byref(cnt),
                                     C.byref(st)))
    blocks = C.c_int32()
    pkg.abi.check(lib.cedar_ckt_last_blocks(sys_.handle, C.byref(blocks)))
    m = cnt.value
    return t_out[:m].copy(), x_out[:m].copy(), st, blocks.value


def test_grid_engine_matches_cta_engine_and_oracle(gpu, pkg, oracle):
    flat = pkg.generators.inverter_chain(300).flatten()
    sys_ = pkg.System(flat)
    o = pkg.make_opts("bdf2", False, 0.0, 0.1e-9, 1e-12, True)
    cap = 200
    tc, xc, stc, bc = _run(pkg, sys_, CTA, o, cap)
    tg, xg, stg, bg = _run(pkg, sys_, GRID, o, cap)
    assert bc == 1 and bg >= 2
    assert stc.status == stg.status == 0 and stc.accepted == stg.accepted == 100
    assert stc.newton_iters == stg.newton_iters and stc.dc_iters == stg.dc_iters
    assert np.array_equal(tc, tg)
    assert np.all(np.abs(xg - xc) <= 1e-12 * np.abs(xc) + 1e-15)
    t_ref, x_ref, st_ref, rc = oracle.tran(flat, o, cap=cap)
    assert rc == 0 and np.array_equal(t_ref, tg)
    nn = flat.n_nodes
    err = np.abs(xg[:, :nn] - x_ref[:, :nn]) / (1e-6 * np.abs(x_ref[:, :nn]) + 1e-9)
    assert err.max() <= 1.0


def _rails(flat, stages):
    """The chain's logic levels with its input low: out_k at VDD for odd k, 0 for
    even k (the DC point within gmin effects), VDD at 1.8 V, currents zero."""
    x0 = np.zeros(flat.n)
    x0[flat.index("vdd")] = 1.8
    for k in range(1, stages + 1, 2):
        x0[1 + k] = 1.8                    # out_k is unknown 1 + k (in, vdd, out1, ...)
    return x0


def test_grid_engine_large_chain(gpu, pkg):
    stages = 20000
    flat = pkg.generators.inverter_chain_flat(stages)
    sys_ = pkg.System(flat)
    assert sys_.n == 20004
    x0 = _rails(flat, stages)
    # transient from the logic levels (no DC solve), fixed-step BDF2 over 20 ps
    o = pkg.make_opts("bdf2", False, 0.0, 20e-12, 1e-12, False)
    cap = 32
    tg, xg, stg, bg = _run(pkg, sys_, 0, o, cap, x0)      # AUTO: the grid engine at this size
    assert bg > 1 and stg.status == 0 and stg.accepted == 20, (bg, stg.status, stg.accepted)
    assert np.all(np.isfinite(xg))
    tc, xc, stc, bc = _run(pkg, sys_, CTA, o, cap, x0)
    assert bc == 1 and stc.status == 0
    assert stc.accepted == stg.accepted and stc.newton_iters == stg.newton_iters
    assert np.array_equal(tc, tg)
    assert np.all(np.abs(xg - xc) <= 1e-12 * np.abs(xc) + 1e-15)
    # DC operating point from the logic levels, and one implicit step, on both engines
    lib = sys_.lib
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    out = {}
    for eng in (CTA, GRID):
        pkg.abi.check(lib.cedar_ckt_set_engine(sys_.handle, eng, 0))
        x = x0.copy()
        st = pkg.abi.Stats()
        pkg.abi.check(lib.cedar_dcop(sys_.handle, 0.0, dp(x), C.byref(st)))
        x2 = x.copy()
        st2 = pkg.abi.Stats()
        pkg.abi.check(lib.cedar_newton_solve(sys_.handle, 0.0, 0.0, None, dp(x2), C.byref(st2)))
        out[eng] = (x, st.dc_iters, x2)
    assert out[CTA][1] == out[GRID][1]
    assert np.all(np.abs(out[GRID][0] - out[CTA][0]) <= 1e-12 * np.abs(out[CTA][0]) + 1e-15)
    assert np.all(np.abs(out[GRID][2] - out[CTA][2]) <= 1e-12 * np.abs(out[CTA][2]) + 1e-15)
    # the DC point is the logic levels to within the gmin drop
    assert np.max(np.abs(out[GRID][0][:flat.n_nodes] - x0[:flat.n_nodes])) < 1e-3
