"""The oracle's discrete adjoint against central finite differences and the
reference's closed-form sensitivity (CPU only).

Reference: test/sensitivity.jl:13-42 (two resistors, dV/dR1 = -dV/dR2 = -V/2).
The finite differences replay the recorded step sequence (times and orders held
fixed), so they differentiate the same discrete map as the adjoint.
"""
import copy

import numpy as np
import pytest

from tests import circuits as K

FD_REL = 1e-6          # central-difference step, relative to the parameter
FD_TOL = 1e-5          # adjoint vs finite differences, relative


def _objective(pkg, flat, vnode, ibranch, probe, level, we, wd, wf):
    n = flat.names
    return pkg.abi.Objective(n.index(vnode), n.index(ibranch), n.index(probe), 0, level, we, wd, wf)


def _param_slots(pkg, flat):
    """(group, row, instance) of every differentiable parameter in gradient order:
    MOS1 widths and resistor values, in group order."""
    out = []
    for gi, (model, term, br, par) in enumerate(flat.groups):
        if model == 8:
            out += [(gi, 1, i) for i in range(par.shape[1])]
        elif model == 1:
            out += [(gi, 0, i) for i in range(par.shape[1])]
    return out


def _fd(oracle, pkg, flat, rep, T, ords, obj, tstar, slot):
    gi, row, i = slot
    f2 = copy.deepcopy(flat)
    p0 = f2.groups[gi][3][row, i]
    d = FD_REL * p0
    f2.groups[gi][3][row, i] = p0 + d
    pp = oracle.replay_phi(f2, rep, T, ords, obj, tstar)
    f2.groups[gi][3][row, i] = p0 - d
    pm = oracle.replay_phi(f2, rep, T, ords, obj, tstar)
    return (pp - pm) / (2 * d)


def test_two_resistor_closed_form(pkg, oracle):
    """d out/dR1 = -V/2, d out/dR2 = +V/2 at R1 = R2 = 1 (test/sensitivity.jl:13-42)."""
    flat = K.two_resistor(pkg).flatten()
    obj = _objective(pkg, flat, "vcc", "V.I", "out", 0.25, 0.0, 0.0, 1.0)
    o = pkg.make_opts(tstop=1e-5)
    phi, g, T, ords = oracle.adjoint(flat, o, o, obj, 0.0)
    v = phi
    assert abs(v - 0.5) < 1e-12
    assert len(T) >= 2
    np.testing.assert_allclose(g, [-v / 2, v / 2], rtol=1e-12, atol=0)


def test_two_resistor_param_lens(pkg, oracle):
    """The ParamLens variant: R1 = 1 from the override, R2 = 1 default."""
    flat = K.two_resistor(pkg, r1=1.0, r2=1.0).flatten()
    obj = _objective(pkg, flat, "vcc", "V.I", "out", 0.25, 0.0, 0.0, 1.0)
    o = pkg.make_opts(tstop=1e-5)
    phi, g, _, _ = oracle.adjoint(flat, o, o, obj, 0.0)
    assert g[0] == pytest.approx(-phi / 2, rel=1e-12)


def test_energy_term_closed_form(pkg, oracle):
    """Supply energy of a resistor divider over [0, tf]: E = V^2 tf / (R1 + R2);
    dE/dR1 = dE/dR2 = -V^2 tf / (R1 + R2)^2."""
    flat = K.two_resistor(pkg, r1=2.0, r2=3.0).flatten()
    obj = _objective(pkg, flat, "vcc", "V.I", "out", 0.25, 1.0, 0.0, 0.0)
    tf = 1e-5
    o = pkg.make_opts(tstop=tf)
    phi, g, _, _ = oracle.adjoint(flat, o, o, obj, 0.0)
    assert phi == pytest.approx(tf / 5.0, rel=1e-12)
    np.testing.assert_allclose(g, [-tf / 25.0, -tf / 25.0], rtol=1e-10)


@pytest.mark.parametrize("stages", [5, 9])
def test_inverter_chain_adjoint_vs_fd(pkg, oracle, stages):
    flat = pkg.generators.inverter_chain(stages).flatten()
    obj = _objective(pkg, flat, "vdd", "VDD.I", f"out{stages}", 0.9, 1e12, 1e20, 1.0)
    fwd = pkg.make_opts(tstop=1.2e-9)
    rep = pkg.make_opts(tstop=1.2e-9, nr_factor=1e-5)
    tstar = 0.3e-9
    phi, g, T, ords = oracle.adjoint(flat, fwd, rep, obj, tstar)
    assert np.isfinite(phi) and len(T) > 50
    assert set(np.unique(ords)) <= {1, 2}
    slots = _param_slots(pkg, flat)
    assert len(g) == len(slots) == 2 * stages
    for k, s in enumerate(slots):
        fd = _fd(oracle, pkg, flat, rep, T, ords, obj, tstar, s)
        assert abs(g[k] - fd) <= FD_TOL * abs(fd), (k, g[k], fd)


def test_mixed_circuit_adjoint_vs_fd(pkg, oracle):
    """Every model (L branch rows, diodes, controlled sources) in the adjoint."""
    flat = K.mixed(pkg).flatten()
    obj = _objective(pkg, flat, "vdd", "VDD.I", "out1", 0.9, 1e12, 1e20, 1.0)
    fwd = pkg.make_opts(tstop=0.8e-9)
    rep = pkg.make_opts(tstop=0.8e-9, nr_factor=1e-5)
    tstar = 0.2e-9
    phi, g, T, ords = oracle.adjoint(flat, fwd, rep, obj, tstar)
    slots = _param_slots(pkg, flat)
    assert len(g) == len(slots)
    for k, s in enumerate(slots):
        fd = _fd(oracle, pkg, flat, rep, T, ords, obj, tstar, s)
        assert abs(g[k] - fd) <= FD_TOL * abs(fd) + 1e-12 * np.max(np.abs(g)), (k, g[k], fd)


def test_replay_reproduces_forward_objective(pkg, oracle):
    """With the forward run's own Newton tolerance the replay is the forward run."""
    flat = pkg.generators.inverter_chain(5).flatten()
    obj = _objective(pkg, flat, "vdd", "VDD.I", "out5", 0.9, 1e12, 1e20, 1.0)
    o = pkg.make_opts(tstop=1.0e-9)
    phi, g, T, ords = oracle.adjoint(flat, o, o, obj, 0.3e-9)
    assert oracle.replay_phi(flat, o, T, ords, obj, 0.3e-9) == phi
