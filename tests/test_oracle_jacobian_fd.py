"""The oracle's Jacobians against central differences of its own residuals.

The GPU's device Jacobians are checked entry by entry against the oracle's
(tests/test_gpu_parity.py, tests/test_gpu_va.py); the oracle's own G = dFi/dx and
C = dFq/dx come from forward-mode dual numbers.  Here they are pinned
independently of any AD: every column is compared with the central difference
(Fi(x + h e_j) - Fi(x - h e_j)) / 2h of the oracle's residual (and likewise Fq),
for every test circuit (built-in and Verilog-A devices) at random states.
"""
import zlib

import numpy as np
import pytest

from tests import circuits as K

CASES = ["vr", "ir", "vrc", "spectre_sources", "spice_sources", "multiplicities", "semiconductor_resistor",
         "pwl_isource", "butterworth", "nlvcr", "two_resistor", "mixed", "va_nlvcr", "inverter_chain_va", "va_mixed",
         "va_diode_rs", "va_vccs", "butterworth_va", "va_thevenin", "chain", "ring", "ring_va", "ladder"]


def _flat(pkg, case):
    g = pkg.generators
    if case == "chain":
        return g.inverter_chain(5).flatten()
    if case == "ring":
        return g.ring_oscillator(5).flatten()
    if case == "ring_va":
        return g.as_verilog_a(g.ring_oscillator(5).flatten())
    if case == "ladder":
        return g.rc_ladder(10).flatten()
    return getattr(K, case)(pkg).flatten()


def _fd_columns(oracle, flat, x, t, G, Cm):
    """Central differences of Fi and Fq, and the rounding error each carries: a
    few ulps of the residual row's terms (bounded by the row's |J| |x| where
    the terms cancel, as at a node's KCL balance), divided by the step."""
    n = flat.n
    eps = np.finfo(float).eps
    sG, sC = np.abs(G) @ np.abs(x), np.abs(Cm) @ np.abs(x)
    dG, dC, eG, eC = (np.zeros((n, n)) for _ in range(4))
    for j in range(n):
        h = 1e-6 * max(1.0, abs(x[j]))
        xp, xm = x.copy(), x.copy()
        xp[j] += h
        xm[j] -= h
        _, fip, fqp, _, _ = oracle.eval(flat, xp, None, t)
        _, fim, fqm, _, _ = oracle.eval(flat, xm, None, t)
        w = xp[j] - xm[j]
        dG[:, j], dC[:, j] = (fip - fim) / w, (fqp - fqm) / w
        eG[:, j] = 16 * eps * (np.abs(fip) + np.abs(fim) + sG) / w
        eC[:, j] = 16 * eps * (np.abs(fqp) + np.abs(fqm) + sC) / w
    return dG, dC, eG, eC


def _close(A, D, E):
    """Entry-wise agreement up to the central difference's truncation error
    (relative to the entry and to its column's scale) and its rounding error E."""
    col = np.maximum(np.abs(A).max(axis=0, keepdims=True), np.abs(D).max(axis=0, keepdims=True))
    return np.abs(A - D) <= 1e-5 * np.abs(A) + 1e-6 * col + E + 1e-18


@pytest.mark.parametrize("case", CASES)
def test_jacobian_matches_central_differences(pkg, oracle, case):
    flat = _flat(pkg, case)
    rng = np.random.default_rng(zlib.crc32(case.encode()))
    nn = flat.n_nodes
    for trial in range(3):
        x = np.empty(flat.n)
        x[:nn] = rng.uniform(-0.2, 1.9, nn)            # node voltages across the rails
        x[nn:] = rng.uniform(-1e-3, 1e-3, flat.n - nn)  # branch currents
        t = rng.uniform(0.0, 2e-9)
        _, Fi, Fq, G, Cm = oracle.eval(flat, x, None, t)
        assert np.all(np.isfinite(Fi)) and np.all(np.isfinite(G)), case
        dG, dC, eG, eC = _fd_columns(oracle, flat, x, t, G, Cm)
        okG, okC = _close(G, dG, eG), _close(Cm, dC, eC)
        bad = np.argwhere(~okG)
        assert okG.all(), f"{case}: G {bad[:3].tolist()} {G[tuple(bad[0])]} vs {dG[tuple(bad[0])]}"
        bad = np.argwhere(~okC)
        assert okC.all(), f"{case}: C {bad[:3].tolist()} {Cm[tuple(bad[0])]} vs {dC[tuple(bad[0])]}"
