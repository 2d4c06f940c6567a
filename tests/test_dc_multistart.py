"""Multi-start DC (CedarSim's bootstrapped_nlsolve, src/dcop.jl:53-94) on the host.

The restart logic of api.dc and Batch.dc is host code around one DC solve:
these tests drive it with a scripted solver (which trajectories converge is
chosen by the test) and with the oracle's DC solve on real circuits, so they
need no GPU.  The reference starts each of its 10 trajectories from
1e-7 * randn(n) and returns the first that converges; here the first starts
from the caller's guess and the restarts from seeded 1e-7 * randn(n) points.
"""
import numpy as np
import pytest


class _St:
    def __init__(self, iters, status=0):
        self.dc_iters, self.status = iters, status


def _scripted(n_fail, iters=5, other_rc=None):
    """A solver that fails (CEDAR_ENOCONV) on its first n_fail calls and then
    converges to x + 1, recording the start point of every call."""
    seen = []

    def solve(x):
        seen.append(x.copy())
        if other_rc is not None:
            return other_rc, _St(iters)
        if len(seen) <= n_fail:
            x[:] = np.nan
            return -5, _St(iters, 6)
        x += 1.0
        return 0, _St(iters)
    return solve, seen


def test_first_trajectory_starts_from_the_guess(pkg):
    solve, seen = _scripted(0)
    x0 = np.linspace(0, 1, 7)
    x, rc, st, k, iters = pkg.api.bootstrapped_dc(solve, x0, trajectories=10, seed=3)
    assert rc == 0 and k == 1 and iters == 5 and len(seen) == 1
    assert np.array_equal(seen[0], x0) and np.array_equal(x, x0 + 1.0)


def test_restarts_from_seeded_random_points(pkg):
    solve, seen = _scripted(3, iters=4)
    x, rc, st, k, iters = pkg.api.bootstrapped_dc(solve, np.zeros(5), trajectories=10, seed=11)
    assert rc == 0 and k == 4 and iters == 16 and len(seen) == 4
    ref = np.random.Generator(np.random.Philox(11))
    for s in seen[1:]:
        assert np.array_equal(s, 1e-7 * ref.standard_normal(5))        # src/dcop.jl:62
    assert np.array_equal(x, seen[3] + 1.0)
    # the same seed gives the same restarts
    solve2, seen2 = _scripted(3, iters=4)
    pkg.api.bootstrapped_dc(solve2, np.zeros(5), trajectories=10, seed=11)
    assert all(np.array_equal(a, b) for a, b in zip(seen, seen2))


def test_gives_up_after_the_last_trajectory(pkg):
    solve, seen = _scripted(100)
    x, rc, st, k, iters = pkg.api.bootstrapped_dc(solve, np.zeros(3), trajectories=10)
    assert rc == -5 and k == 10 and len(seen) == 10 and iters == 50 and st.status == 6
    solve, seen = _scripted(100)
    _, rc, _, k, _ = pkg.api.bootstrapped_dc(solve, np.zeros(3), trajectories=1)
    assert rc == -5 and k == 1 and len(seen) == 1
    with pytest.raises(ValueError):
        pkg.api.bootstrapped_dc(solve, np.zeros(3), trajectories=0)


def test_other_errors_end_the_loop(pkg):
    solve, seen = _scripted(0, other_rc=-1)                 # CEDAR_EINVAL: not retried
    _, rc, _, k, _ = pkg.api.bootstrapped_dc(solve, np.zeros(3), trajectories=10)
    assert rc == -1 and k == 1 and len(seen) == 1


def test_with_the_oracle_solve(pkg, oracle):
    """Around the oracle's DC solve: a circuit that converges from zeros gives the
    plain solve's bits in one trajectory; one that cannot converge (a NaN device
    parameter) runs every trajectory, each from its own start."""
    flat = pkg.generators.inverter_chain(9).flatten()
    x_ref, st_ref, rc_ref = oracle.dcop(flat)
    assert rc_ref == 0

    def solve(x):
        xs, st, rc = oracle.dcop(flat, x0=x)
        x[:] = xs
        return rc, st
    x, rc, st, k, iters = pkg.api.bootstrapped_dc(solve, np.zeros(flat.n))
    assert rc == 0 and k == 1 and iters == st_ref.dc_iters and np.array_equal(x, x_ref)

    c = pkg.Circuit()
    c.V("V1", "a", "0", dc=1.0)
    c.R("R1", "a", "b", r=float("nan"))
    c.R("R2", "b", "0", r=1e3)
    bad = c.flatten()
    starts = []

    def solve_bad(x):
        starts.append(x.copy())
        xs, st, rc = oracle.dcop(bad, x0=x)
        x[:] = xs
        return rc, st
    _, rc, st, k, _ = pkg.api.bootstrapped_dc(solve_bad, np.zeros(bad.n), trajectories=4, seed=2)
    assert rc == -5 and k == 4 and st.status != 0
    assert not np.any(starts[0]) and all(0 < np.abs(s).max() < 1e-5 for s in starts[1:])


def test_batch_restart_rounds(pkg):
    """Batch.dc's restart rounds: only instances that have not converged are run
    again, each from its own seeded start sequence; iterations add up; x and
    status come from the last trajectory; rounds stop when all converge."""
    STATS = pkg.abi.STATS_DTYPE
    n_of = np.array([3, 5, 4, 5, 3])
    x = np.zeros((5, 5))
    st = np.zeros(5, STATS)
    st["status"] = [0, 6, 0, 6, 6]
    st["dc_iters"] = [7, 9, 8, 9, 9]
    converge_at = {1: 1, 3: 3, 4: 99}                       # restart round an instance converges in
    calls = []

    def run_round(idx, x0):
        r = len(calls) + 1
        calls.append((idx.copy(), [v.copy() for v in x0]))
        m = max(n_of[i] for i in idx)
        xs = np.zeros((len(idx), m))
        ss = np.zeros(len(idx), STATS)
        for j, i in enumerate(idx):
            ok = converge_at[int(i)] <= r
            xs[j, :n_of[i]] = x0[j] + (1.0 if ok else 0.0)
            ss[j]["status"] = 0 if ok else 6
            ss[j]["dc_iters"] = 2
        return xs, ss

    x, st = pkg.api.batch_dc_restarts(x, st, n_of, trajectories=4, seed=5, run_round=run_round)
    assert [list(c[0]) for c in calls] == [[1, 3, 4], [3, 4], [3, 4]]
    for i in (1, 3, 4):
        ref = pkg.api.dc_starts(int(n_of[i]), 5 + i)
        seq = [c[1][list(c[0]).index(i)] for c in calls if i in c[0]]
        for s in seq:
            assert np.array_equal(s, next(ref))
    assert list(st["status"]) == [0, 0, 0, 0, 6]
    assert list(st["dc_iters"]) == [7, 11, 8, 15, 15]
    assert np.array_equal(x[1, :5], calls[0][1][0] + 1.0)
    assert np.array_equal(x[3, :5], calls[2][1][0] + 1.0)
    assert not np.any(x[0]) and not np.any(x[2])
