"""GPU discrete adjoint (cedar_adjoint_run) against the oracle's adjoint, central
finite differences over the GPU's own recorded steps, and the reference's
closed-form sensitivity (test/sensitivity.jl:13-42)."""
import copy

import numpy as np
import pytest

from tests import circuits as K

pytestmark = pytest.mark.gpu

FD_REL = 1e-6      # central-difference step, relative to the parameter
FD_TOL = 1e-5      # adjoint vs finite differences, relative
ORC_TOL = 1e-7     # GPU adjoint vs oracle adjoint on the same step sequence, relative


def _obj(pkg, o):
    return pkg.abi.Objective(int(o[0]), int(o[1]), int(o[2]), 0, *[float(v) for v in o[3:]])


def _slots(flat):
    out = []
    for gi, (model, term, br, par) in enumerate(flat.groups):
        if model == 8:
            out += [(gi, 1, i) for i in range(par.shape[1])]
        elif model == 1:
            out += [(gi, 0, i) for i in range(par.shape[1])]
    return out


def _small(pkg, n_inst=6, seed=7, lengths=(5, 7, 9)):
    return pkg.generators.adjoint_chains(n_inst, seed=seed, lengths=list(lengths))


def test_two_resistor_closed_form(gpu, pkg):
    flat = K.two_resistor(pkg).flatten()
    sw = pkg.Batch([flat], np.zeros(1, np.int32))
    n = flat.names
    obj = pkg.abi.Objective(n.index("vcc"), n.index("V.I"), n.index("out"), 0, 0.25, 0.0, 0.0, 1.0)
    r = sw.adjoint(pkg.make_opts(tstop=1e-5), [obj])
    assert r.status[0] == 0
    v = r.phi[0]
    assert abs(v - 0.5) < 1e-12
    np.testing.assert_allclose(r.grad[0], [-v / 2, v / 2], rtol=1e-12)


def test_energy_closed_form(gpu, pkg):
    flat = K.two_resistor(pkg, r1=2.0, r2=3.0).flatten()
    sw = pkg.Batch([flat], np.zeros(1, np.int32))
    n = flat.names
    obj = pkg.abi.Objective(n.index("vcc"), n.index("V.I"), n.index("out"), 0, 0.25, 1.0, 0.0, 0.0)
    tf = 1e-5
    r = sw.adjoint(pkg.make_opts(tstop=tf), [obj])
    assert r.phi[0] == pytest.approx(tf / 5.0, rel=1e-12)
    np.testing.assert_allclose(r.grad[0], [-tf / 25.0, -tf / 25.0], rtol=1e-10)


def test_chains_match_oracle_adjoint(gpu, pkg, oracle):
    templates, itpl, par, off, objs, tstar = _small(pkg)
    sw = pkg.Batch(templates, itpl, par, off)
    o = pkg.make_opts(tstop=1.2e-9)
    objectives = [_obj(pkg, ob) for ob in objs]
    r = sw.adjoint(o, objectives, tstar)
    assert np.all(r.status == 0)
    for i in range(len(itpl)):
        t = int(itpl[i])
        flat = pkg.generators.instance_flat(templates[t], par[off[i]:off[i] + templates[t].param_block().size])
        phi, g, T, ords = oracle.adjoint(flat, o, o, objectives[t], float(tstar[i]))
        tg, og = sw.tape(i)
        assert len(tg) == len(T) and np.array_equal(og, ords)
        np.testing.assert_allclose(tg, T, rtol=1e-12, atol=0)
        assert r.phi[i] == pytest.approx(phi, rel=1e-9)
        gg = r.grad[i, :len(g)]
        assert np.all(np.abs(gg - g) <= ORC_TOL * np.abs(g) + 1e-9 * np.max(np.abs(g))), (i, gg, g)


def test_chains_vs_fd_on_gpu_steps(gpu, pkg, oracle):
    """Central differences of the objective over the GPU's own accepted steps
    (replayed by the oracle), on every width of two instances."""
    templates, itpl, par, off, objs, tstar = _small(pkg, n_inst=2, seed=3, lengths=(7,))
    sw = pkg.Batch(templates, itpl, par, off)
    o = pkg.make_opts(tstop=1.2e-9)
    rep = pkg.make_opts(tstop=1.2e-9, nr_factor=1e-5)
    objectives = [_obj(pkg, ob) for ob in objs]
    r = sw.adjoint(o, objectives, tstar)
    assert np.all(r.status == 0)
    for i in range(2):
        flat = pkg.generators.instance_flat(templates[0], par[off[i]:off[i] + templates[0].param_block().size])
        T, ords = sw.tape(i)
        for k, (gi, row, ii) in enumerate(_slots(flat)):
            f2 = copy.deepcopy(flat)
            p0 = f2.groups[gi][3][row, ii]
            d = FD_REL * p0
            f2.groups[gi][3][row, ii] = p0 + d
            pp = oracle.replay_phi(f2, rep, T, ords, objectives[0], float(tstar[i]))
            f2.groups[gi][3][row, ii] = p0 - d
            pm = oracle.replay_phi(f2, rep, T, ords, objectives[0], float(tstar[i]))
            fd = (pp - pm) / (2 * d)
            assert abs(r.grad[i, k] - fd) <= FD_TOL * abs(fd), (i, k, r.grad[i, k], fd)


def test_mixed_circuit_matches_oracle(gpu, pkg, oracle):
    """Inductor branch rows, diodes and controlled sources in the adjoint."""
    flat = K.mixed(pkg).flatten()
    n = flat.names
    obj = pkg.abi.Objective(n.index("vdd"), n.index("VDD.I"), n.index("out1"), 0, 0.9, 1e12, 1e20, 1.0)
    o = pkg.make_opts(tstop=0.8e-9)
    sw = pkg.Batch([flat], np.zeros(1, np.int32))
    r = sw.adjoint(o, [obj], np.array([0.2e-9]))
    assert r.status[0] == 0
    phi, g, T, ords = oracle.adjoint(flat, o, o, obj, 0.2e-9)
    tg, og = sw.tape(0)
    assert len(tg) == len(T)
    assert r.phi[0] == pytest.approx(phi, rel=1e-9)
    gg = r.grad[0, :len(g)]
    assert np.all(np.abs(gg - g) <= 1e-6 * np.abs(g) + 1e-9 * np.max(np.abs(g))), (gg, g)


def test_adjoint_bitwise_across_tile_shapes_and_reruns(gpu, pkg):
    templates, itpl, par, off, objs, tstar = _small(pkg, n_inst=10, seed=9)
    sw = pkg.Batch(templates, itpl, par, off)
    o = pkg.make_opts(tstop=0.8e-9)
    objectives = [_obj(pkg, ob) for ob in objs]
    base = None
    for K_, W in [(32, 4), (8, 4), (1, 2), (32, 4)]:
        sw.set_tuning(K_, W)
        r = sw.adjoint(o, objectives, tstar)
        if base is None:
            base = r
            continue
        assert np.array_equal(r.phi, base.phi)
        assert np.array_equal(r.grad, base.grad)


def test_adjoint_segments_longer_than_one_checkpoint(gpu, pkg, oracle):
    """A run of several hundred steps crosses many 64-step checkpoints."""
    templates, itpl, par, off, objs, tstar = _small(pkg, n_inst=1, seed=1, lengths=(5,))
    sw = pkg.Batch(templates, itpl, par, off)
    o = pkg.make_opts(tstop=4e-9, hmax=4e-9 / 50)
    objectives = [_obj(pkg, ob) for ob in objs]
    r = sw.adjoint(o, objectives, tstar)
    assert r.status[0] == 0 and r.stats["accepted"][0] > 300
    flat = pkg.generators.instance_flat(templates[0], par[off[0]:off[0] + templates[0].param_block().size])
    phi, g, T, ords = oracle.adjoint(flat, o, o, objectives[0], float(tstar[0]))
    assert r.phi[0] == pytest.approx(phi, rel=1e-9)
    assert np.all(np.abs(r.grad[0, :len(g)] - g) <= ORC_TOL * np.abs(g) + 1e-9 * np.max(np.abs(g)))


def test_adjoint_tape_overflow_is_reported(gpu, pkg):
    templates, itpl, par, off, objs, tstar = _small(pkg, n_inst=2, seed=2, lengths=(5,))
    sw = pkg.Batch(templates, itpl, par, off)
    r = sw.adjoint(pkg.make_opts(tstop=1.2e-9), [_obj(pkg, ob) for ob in objs], tstar, tape_cap=16)
    assert np.all(r.status == 4)              # CEDAR_ST_MAX_STEPS
    assert np.all(np.isnan(r.phi)) and np.all(np.isnan(r.grad))


def test_adjoint_rejects_fixed_step(gpu, pkg):
    templates, itpl, par, off, objs, tstar = _small(pkg, n_inst=1, lengths=(5,))
    sw = pkg.Batch(templates, itpl, par, off)
    with pytest.raises(pkg.abi.CedarError):
        sw.adjoint(pkg.make_opts(adaptive=False, h=1e-12, tstop=1e-10), [_obj(pkg, ob) for ob in objs], tstar)
