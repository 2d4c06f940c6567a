"""The multi-start DC (CedarSim's bootstrapped_nlsolve, src/dcop.jl:53-94) through
the GPU entry points: dc() of one circuit and Batch.dc() over instances.

Healthy instances converge from zeros in their first trajectory and keep its
bits; instances made unsolvable on the host (a NaN resistor value) go through
every restart (a batched launch per round over the instances still failing)
and end with a failure status.  Nothing here
faults a GPU: the failures are numerical and detected by the engines.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _divider(pkg, r1=1e3):
    c = pkg.Circuit()
    c.V("V1", "in", "0", dc=1.0)
    c.R("R1", "in", "a", r=r1)
    c.R("R2", "a", "0", r=1e3)
    return c.flatten()


def test_batch_dc_restarts(gpu, pkg, oracle, monkeypatch):
    flat = _divider(pkg)
    blk = flat.param_block()
    bad = blk.copy()
    bad[flat.param_offset("R1", 0)] = np.nan
    poisoned = [1, 3, 4]
    blocks = [bad if i in poisoned else blk for i in range(6)]
    par = np.concatenate(blocks)
    off = np.arange(6, dtype=np.int64) * blk.size
    tpl = np.zeros(6, np.int32)
    x1, st1 = pkg.Batch([flat], tpl, par, off).dc(trajectories=1)
    # record the restart rounds (each a batched launch over the instances still failing)
    rounds = []
    orig = pkg.api.batch_dc_restarts

    def spy(x, st, n_of, trajectories, seed, run_round):
        def counted(idx, x0):
            rounds.append([int(i) for i in idx])
            assert all(v.size == flat.n and 0 < np.abs(v).max() < 1e-5 for v in x0)
            return run_round(idx, x0)
        return orig(x, st, n_of, trajectories, seed, counted)
    monkeypatch.setattr(pkg.api, "batch_dc_restarts", spy)
    x3, st3 = pkg.Batch([flat], tpl, par, off).dc(trajectories=3, seed=7)
    assert rounds == [poisoned, poisoned]
    xr, _, rc = oracle.dcop(flat)
    assert rc == 0
    for i in range(6):
        if i in poisoned:
            # a NaN conductance fails at the first factorisation of every trajectory
            assert st1[i]["status"] != 0 and st3[i]["status"] != 0
            assert st3[i]["dc_iters"] >= st1[i]["dc_iters"]
        else:
            assert st1[i]["status"] == 0 and st3[i]["status"] == 0
            assert st3[i]["dc_iters"] == st1[i]["dc_iters"]
            assert np.array_equal(x3[i, :flat.n], x1[i, :flat.n])
            assert np.allclose(x3[i, :flat.n], xr, rtol=1e-12, atol=1e-15)


def test_single_circuit_dc_restarts(gpu, pkg, oracle):
    flat = _divider(pkg)
    x = pkg.dc(flat, trajectories=3)
    xr, _, rc = oracle.dcop(flat)
    assert rc == 0 and np.allclose(x, xr, rtol=1e-12, atol=1e-15)
    with pytest.raises(pkg.abi.CedarError) as e:
        pkg.dc(_divider(pkg, r1=np.nan), trajectories=3, seed=1)
    assert e.value.code == -5
