"""Per-instance status words of the engines, with every failure made on the host.

The reference's solvers report failure through return codes rather than by
aborting (`src/util.jl:3-21`, the retcode checks of `src/dcop.jl:58-81,141-145`);
here every instance carries a `CEDAR_ST_*` status word and a failed instance is
retired without disturbing the others.  Each batch below mixes healthy instances
with instances built to fail in one specific way -- a NaN parameter, a node whose
only conductance is zero, an initial state that overflows, a DC problem without
a solution, a step budget too small, one Newton iteration per step -- and checks
that every instance reports the status the oracle (the same algorithms on the
CPU) reports, that healthy instances still match the oracle, and that the
single-circuit path (cedar_tran_run) reports the same status.  Nothing here
faults or traps a GPU: the failures are numerical and detected by the engines.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NS = 1e-9
RTOL, ATOL = 1e-6, 1e-9


def _rc(pkg, vdc=1.0, wave=None, extra=None):
    c = pkg.Circuit()
    if wave is None:
        c.V("V1", "in", "0", dc=vdc)
    else:
        c.V("V1", "in", "0", wave=wave)
    c.R("R1", "in", "a", r=1e3)
    c.C("C1", "a", "0", 1e-12)
    if extra:
        extra(c)
    return c.flatten()


def _overflow(pkg):
    """A capacitor-only node started at 1.5e308 and charged by 5e307 A: the first
    step's solution is +inf (a finite update that overflows)."""
    c = pkg.Circuit()
    c.R("R1", "a", "0", r=1e3)
    c.C("C1", "a", "0", 1e-12)
    c.C("C2", "c", "0", 1e-12)
    c.I("I2", "0", "c", dc=5e307)
    f = c.flatten()
    x0 = np.zeros(f.n)
    x0[f.index("c")] = 1.5e308
    return f, x0


def _divider(pkg):
    c = pkg.Circuit()
    c.V("V1", "in", "0", dc=1.0)
    c.R("R1", "in", "a", r=1e3)
    c.R("R2", "a", "0", r=1e3)
    return c.flatten()


def _groups(pkg):
    P = pkg.circuit.Pulse
    nan, inf = float("nan"), float("inf")
    ovf, ovf_x0 = _overflow(pkg)
    adaptive_cold = {          # adaptive BDF2, no DC operating point (start from x0), max_steps 400
        "opts": dict(adaptive=True, dcop=False, h=0.0, max_steps=400),
        "cases": [
            ("OK", _rc(pkg), None),
            ("ZERO_PIVOT", _rc(pkg, extra=lambda c: c.R("R2", "a", "b", r=inf)), None),
            ("DT_UNDERFLOW", _rc(pkg, vdc=nan), None),
            ("NAN", ovf, ovf_x0),
            ("MAX_STEPS", _rc(pkg, wave=P(0.0, 1.0, 0.0, 20e-12, 20e-12, 105e-12, 0.25e-9)), None),
        ]}
    adaptive_dc = {            # adaptive BDF2 from the DC operating point
        "opts": dict(adaptive=True, dcop=True, h=0.0, max_steps=0),
        "cases": [
            ("OK", _rc(pkg), None),
            ("DCOP", _rc(pkg, extra=lambda c: c.R("R3", "a", "0", r=nan)), None),
            ("DCOP", _rc(pkg, extra=lambda c: (c.I("I1", "0", "f", dc=1e-6), c.C("C3", "f", "0", 1e-12))), None),
        ]}
    fixed_one_newton = {       # fixed-step BDF2, h = 10 ps, one Newton iteration per step
        "opts": dict(adaptive=False, dcop=True, h=10e-12, max_steps=0, max_newton=1),
        "cases": [
            ("OK", _divider(pkg), None),
            ("NEWTON", _rc(pkg, wave=P(0.0, 1.0, 0.1e-9, 20e-12, 20e-12, 230e-12, 0.5e-9)), None),
        ]}
    return {"adaptive_cold": adaptive_cold, "adaptive_dc": adaptive_dc, "fixed_one_newton": fixed_one_newton}


def _opts(pkg, o):
    return pkg.make_opts("bdf2", o["adaptive"], 0.0, 10 * NS, o["h"], o["dcop"], max_steps=o["max_steps"],
                         max_newton=o.get("max_newton", 20))


@pytest.mark.parametrize("group", ["adaptive_cold", "adaptive_dc", "fixed_one_newton"])
def test_batch_status_words(gpu, pkg, oracle, group):
    g = _groups(pkg)[group]
    opts = _opts(pkg, g["opts"])
    # two instances per case, interleaved, so failing and healthy instances share warps
    flats = [f for _, f, _ in g["cases"]]
    itpl = np.array([k for _ in range(2) for k in range(len(flats))], np.int32)
    x0s, x0_off, off = [], [], 0
    for k in itpl:
        x0 = g["cases"][k][2]
        x0 = np.zeros(flats[k].n) if x0 is None else x0
        x0s.append(x0)
        x0_off.append(off)
        off += x0.size
    b = pkg.Batch(flats, itpl, inst_x0=np.concatenate(x0s), inst_x0_off=np.array(x0_off, np.int64))
    r = b.run(opts)
    names = pkg.abi.STATUS_NAMES
    for i, k in enumerate(itpl):
        want, f, x0 = g["cases"][k]
        _, x_ref, st_ref, rc = oracle.tran(f, opts, x0=x0, cap=1 << 16)
        got = names[int(r.stats["status"][i])]
        assert names[st_ref.status] == want, (group, k, names[st_ref.status])
        assert got == want, (group, i, got, want)
        if want == "OK":
            assert r.stats["accepted"][i] == st_ref.accepted
            xf = r.x_final[i, :f.n]
            assert np.all(np.abs(xf - x_ref[-1]) <= RTOL * np.abs(x_ref[-1]) + ATOL), (group, i)


@pytest.mark.parametrize("group", ["adaptive_cold", "adaptive_dc", "fixed_one_newton"])
def test_single_circuit_status_words(gpu, pkg, group):
    """The single-circuit transient (cedar_tran_run) reports the same status words."""
    g = _groups(pkg)[group]
    o = g["opts"]
    for want, f, x0 in g["cases"]:
        sol = pkg.tran(f, (0.0, 10 * NS), method="bdf2", h=o["h"] or None, adaptive=o["adaptive"], x0=x0,
                       dcop=o["dcop"], max_steps=o["max_steps"], max_newton=o.get("max_newton", 20), cap=1 << 14)
        assert sol.retcode == want, (group, want, sol.retcode)
