"""Order of the fixed-step BDF2 integrator on a nonlinear circuit (CPU).

The reference integrates with IDA / FBDF, so fixed-step BDF2 (configuration 2)
is this project's algorithm, restated identically in the oracle and the
engines.  On the 31-stage level-1 inverter chain, differences between runs at
h, h/2 and h/4 shrink by 4 per halving (second order) at every node over the
first two input edges: a wrong history coefficient or a first-order start that
never hands over to BDF2 would show here.
"""
import numpy as np


def test_bdf2_fixed_step_is_second_order(pkg, oracle):
    flat = pkg.generators.inverter_chain(31).flatten()
    tstop = 2e-9
    runs = {}
    for h in (4e-12, 2e-12, 1e-12):
        t, X, st, rc = oracle.tran(flat, pkg.make_opts("bdf2", False, 0.0, tstop, h, True))
        assert rc == 0 and st.status == 0 and len(t) == round(tstop / h) + 1
        runs[h] = (t, X)
    tq = np.arange(0.0, tstop + 1e-15, 4e-12)
    nodes = list(range(flat.n_nodes))

    def at(h):
        t, X = runs[h]
        return X[np.searchsorted(t, tq - 1e-18)][:, nodes]
    d1 = np.abs(at(4e-12) - at(2e-12)).max()
    d2 = np.abs(at(2e-12) - at(1e-12)).max()
    assert d2 < 2e-2                                   # volts, on a 1.8 V swing
    assert 3.5 < d1 / d2 < 4.5, (d1, d2)
