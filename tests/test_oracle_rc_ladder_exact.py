"""Configuration 1 (the RC ladder, trapezoidal h = 0.1 ns) against its exact solution.

The reference holds no waveform for this workload, and its integrators are
IDA / FBDF, so the fixed-step trapezoidal recurrence is this project's
algorithm; for a linear circuit it can be checked against the exact solution.
With the source node eliminated, the ladder is v' = A v + b u(t) with A the
tridiagonal -1/(RC) stencil and u the PULSE(0 1 0 1n 1n 50n 100n) input, which is
linear between its corners (0, 1, 51, 52 ns, period 100 ns, src/spectre_env.jl:
15-69).  The state [v, u, u'] of the augmented system is advanced exactly by
expm(M h) over each step (every corner lies on the 0.1 ns grid), u' reset at the
corners.  The oracle's waveform must agree with it to the trapezoidal rule's
truncation error, and halving h must divide that error by 4 (second order).
The GPU runs the same recurrence to the same time points (tests/test_gpu_parity.py).
"""
import numpy as np
import pytest

scipy_linalg = pytest.importorskip("scipy.linalg")

N, R, CAP = 100, 1e3, 1e-12
TR, PW, TF, PER = 1e-9, 50e-9, 1e-9, 100e-9


def _u(t):
    tm = t % PER
    if tm < TR:
        return tm / TR
    if tm < TR + PW:
        return 1.0
    if tm < TR + PW + TF:
        return 1.0 - (tm - TR - PW) / TF
    return 0.0


def _slope(t):
    """u' on the step that starts at t (corners belong to the next segment)."""
    tm = t % PER
    eps = 1e-15
    if tm < TR - eps:
        return 1.0 / TR
    if tm < TR + PW - eps:
        return 0.0
    if tm < TR + PW + TF - eps:
        return -1.0 / TF
    return 0.0


def _exact(h, tstop):
    A = np.zeros((N, N))
    for k in range(N):
        A[k, k] = -2.0 if k < N - 1 else -1.0
        if k > 0:
            A[k, k - 1] = 1.0
        if k < N - 1:
            A[k, k + 1] = 1.0
    A /= R * CAP
    M = np.zeros((N + 2, N + 2))
    M[:N, :N] = A
    M[0, N] = 1.0 / (R * CAP)          # node 1 is driven by u through R
    M[N, N + 1] = 1.0                  # u' = s
    Phi = scipy_linalg.expm(M * h)
    steps = int(round(tstop / h))
    z = np.zeros(N + 2)
    out = np.zeros((steps + 1, N))
    for k in range(steps):
        t = k * h
        z[N] = _u(t)
        z[N + 1] = _slope(t)
        z = Phi @ z
        out[k + 1] = z[:N]
    return out


def _oracle(pkg, oracle, h, tstop):
    flat = pkg.generators.rc_ladder(N).flatten()
    o = pkg.make_opts("trap", False, 0.0, tstop, h, True)
    t, X, st, rc = oracle.tran(flat, o)
    assert rc == 0 and st.status == 0
    idx = [flat.index(f"n{k}") for k in range(1, N + 1)]
    return t, X[:, idx]


def test_trapezoidal_ladder_against_exact_solution(pkg, oracle):
    tstop = 200e-9                     # two pulse periods
    errs = []
    for h in (0.1e-9, 0.05e-9):
        t, V = _oracle(pkg, oracle, h, tstop)
        E = _exact(h, tstop)
        assert len(t) == E.shape[0] and np.allclose(t, np.arange(len(t)) * h, rtol=0, atol=1e-21)
        errs.append(np.abs(V - E).max())
    # second-order convergence to the exact waveform
    assert errs[0] < 5e-4                # 2.6e-4 V at h = 0.1 ns
    assert 3.5 < errs[0] / errs[1] < 4.5, errs
