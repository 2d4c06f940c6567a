"""Verilog-A models on the GPU against the CPU oracle.

The emitted device code runs inside every engine: the device evaluation of
cedar_eval, the one-circuit transient, the batched Monte-Carlo kernel and the
small-signal AC and noise solves.  The oracle evaluates the same modules from
its own hand restatement of each shipped .va file (oracle/oracle.cpp,
va_restated), which shares no code with the emitter, so every comparison here is
emitted code against an independent evaluation (test_every_model_is_restated
guards that).  Tolerances are the parity contract's (device F and J within
1e-12 relative; waveforms within reltol 1e-6 / abstol 1e-9 V with the same step
sequence)."""
import numpy as np
import pytest

from tests import circuits as K
from tests.test_gpu_parity import ABSTOL, RELTOL, RTOL_EVAL, compare_waves, random_state

pytestmark = pytest.mark.gpu

CASES = {
    "va_mixed": K.va_mixed,
    "va_chain_7": lambda pkg: K.inverter_chain_va(pkg, 7),
    "va_nlvcr": K.va_nlvcr,
    "va_diode_rs": K.va_diode_rs,      # internal node
    "va_vccs": K.va_vccs,              # analog function, macros, case, $param_given
    "va_thevenin": K.va_thevenin,      # voltage-contributed branches (source, inductor)
}


def test_every_model_is_restated(gpu, pkg, oracle):
    """Every Verilog-A model the GPU tests use (and every shipped module) has a
    hand restatement in the oracle, so no comparison runs emitted code on both
    sides."""
    import ctypes as C
    va = pkg.va
    used = set()
    for mk in list(CASES.values()) + [K.butterworth_va, K.butterworth_ac_va, _flicker_divider]:
        used |= {g[0] for g in mk(pkg).flatten().groups if g[0] >= va.BASE_ID}
    used |= {va.model_id(m.name) for m in va.models()}
    dp_ = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    for mid in sorted(used):
        k = mid - va.BASE_ID
        m = va.models()[k]
        z = np.zeros(m.nx * m.nx)
        vals = m.defaults({})
        assert oracle.lib.oracle_va_ref_full(k, dp_(np.array(vals + [1.0, 0.025])), len(vals) + 1,
                                             dp_(np.zeros(m.nx)), 1e-12, dp_(np.zeros(m.nx)), dp_(np.zeros(m.nx)),
                                             dp_(z), dp_(z.copy())) == 1, m.name


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("t", [0.0, 0.21e-9])
def test_va_eval_parity(gpu, pkg, oracle, case, t):
    flat = CASES[case](pkg).flatten()
    sys = pkg.System(flat)
    rng = np.random.default_rng(99)
    for _ in range(4):
        x = random_state(flat, rng)
        xd = rng.normal(0, 1e9, flat.n)
        gamma = 10.0 ** rng.uniform(9, 13)
        F, Jv = sys.eval(x, xd, t, gamma)
        Fr, Fi, Fq, G, Cm = oracle.eval(flat, x, xd, t)
        scale = np.abs(G) @ np.abs(x) + np.abs(Cm) @ np.abs(xd) + np.abs(Fi)
        assert np.all(np.abs(F - Fr) <= RTOL_EVAL * (np.abs(Fr) + scale) + 1e-300), case
        J = sys.jac_dense(Jv)
        Jr = G + gamma * Cm
        rows = np.abs(G).max(axis=1, keepdims=True) + gamma * np.abs(Cm).max(axis=1, keepdims=True)
        assert np.all(np.abs(J - Jr) <= RTOL_EVAL * (np.abs(Jr) + 1e-6 * rows) + 1e-300), case


def test_va_ddx_known_answer_on_gpu(gpu, pkg):
    f = K.va_nlvcr(pkg).flatten()
    x = pkg.dc(f)
    assert abs(x[f.index("V1.I")] - (-60.0)) <= 8 * np.spacing(60.0)


@pytest.mark.parametrize("case, adaptive", [("va_mixed", False), ("va_chain_7", True), ("va_diode_rs", False),
                                            ("va_vccs", False), ("va_thevenin", False)])
def test_va_transient_parity(gpu, pkg, oracle, case, adaptive):
    """Fixed-step BDF2 (h = 1 ps) on the mixed circuit, adaptive BDF2 on the chain.
    The mixed circuit's 5k adaptive steps put some LTE tests within rounding of
    the accept / step-factor thresholds, where the sparse static-pivot LU and
    the oracle's dense LU can choose differently (one step in 5114 on a GB300),
    so its time points are pinned by the fixed step instead."""
    flat = CASES[case](pkg).flatten()
    h = 0.0 if adaptive else 1e-12
    o = pkg.make_opts("bdf2", adaptive, 0.0, 2e-9, h, True)
    sol = pkg.tran(flat, (0.0, 2e-9), method="bdf2", h=h or None, adaptive=adaptive)
    t_ref, x_ref, st, rc = oracle.tran(flat, o)
    assert rc == 0 and sol.retcode == "OK"
    assert (sol.stats["accepted"], sol.stats["rejected"]) == (st.accepted, st.rejected)
    assert compare_waves(sol, t_ref, x_ref, flat.n_nodes) <= 1.0


def test_va_chain_tracks_builtin_chain(gpu, pkg):
    """The Verilog-A level-1 MOSFET is the built-in model's equations: the two
    chains' waveforms agree within the waveform tolerance."""
    a = K.inverter_chain_va(pkg, 9).flatten()
    b = K.inverter_chain_va(pkg, 9, builtin=True).flatten()
    ha = pkg.tran(a, (0.0, 3e-9), method="bdf2", h=1e-12, adaptive=False)
    hb = pkg.tran(b, (0.0, 3e-9), method="bdf2", h=1e-12, adaptive=False)
    assert ha.retcode == "OK" and hb.retcode == "OK" and np.array_equal(ha.t, hb.t)
    err = np.abs(ha.u[:, :a.n_nodes] - hb.u[:, :a.n_nodes]) / (RELTOL * np.abs(hb.u[:, :a.n_nodes]) + ABSTOL)
    assert err.max() <= 1.0


def test_va_batched_monte_carlo(gpu, pkg, oracle):
    """Batched kernel with Verilog-A chains of two lengths and per-instance
    parameter blocks (W, KP, VTO, load) against the oracle's batch run."""
    rng = np.random.default_rng(5)
    templates = [K.inverter_chain_va(pkg, L).flatten() for L in (3, 6)]
    itpl = np.array([i % 2 for i in range(24)], np.int32)
    blocks, off, pos = [], [], 0
    for i in range(24):
        f = templates[itpl[i]]
        b = f.param_block().copy()
        for gi, (model, term, br, par) in enumerate(f.groups):
            base = sum(g[3].size for g in f.groups[:gi])
            n = par.shape[1]
            if model >= pkg.circuit.VA_BASE:      # va_mos1: W row 1, KP row 3, VTO row 4
                b[base + 1 * n: base + 2 * n] *= rng.uniform(0.8, 1.2, n)
                b[base + 3 * n: base + 4 * n] *= np.exp(0.05 * rng.normal(size=n))
                b[base + 4 * n: base + 5 * n] += 0.03 * rng.normal(size=n) * np.sign(b[base + 4 * n: base + 5 * n])
            elif model == 2:                          # load capacitors
                b[base: base + n] = rng.uniform(5e-15, 20e-15)
        blocks.append(b)
        off.append(pos)
        pos += b.size
    par = np.concatenate(blocks)
    off = np.array(off, np.int64)
    probes = np.array([[f.index("out3"), f.index("in")] for f in templates], np.int32)
    sw = pkg.Batch(templates, itpl, par, off, probes=probes, n_samples=31)
    o = pkg.make_opts("bdf2", True, 0.0, 1.5e-9, 0.0, True)
    res = sw.run(o)
    xf, samp, st = oracle.batch(sw.holder, o)
    assert np.all(res.stats["status"] == 0) and np.all(st["status"] == 0)
    for k in ("accepted", "rejected"):
        assert np.array_equal(res.stats[k], st[k]), k
    err = np.abs(res.samples - samp) / (RELTOL * np.abs(samp) + ABSTOL)
    assert err.max() <= 1.0


def test_va_ac_parity(gpu, pkg, oracle):
    """Small-signal AC through Verilog-A charges (diode diffusion + depletion
    charge, capacitor): G and C split by the emitted charge-partial outputs."""
    flat = K.va_mixed(pkg).flatten()
    flat.ac = {"VIN": 1.0}
    x_op = pkg.dc(flat)
    w = 2 * np.pi * pkg.acdec(5, 1e6, 1e12)
    probes = ["b", "c", "d"]
    r = pkg.ac(flat, x_op=x_op).freqresp(probes, w)
    ro = oracle.ac(flat, x_op, w, [flat.index(p) for p in probes])
    # relative to the largest probed magnitude at each frequency, as the AC parity tests
    err = np.max(np.abs(r - ro) / np.max(np.abs(ro), axis=1, keepdims=True))
    assert err <= 1e-9


def test_va_inductor_butterworth_transient(gpu, pkg, oracle):
    """The Butterworth filter of test/transients.jl with Verilog-A inductors
    (voltage-contributed branches with ddt(L I)): GPU against the oracle,
    fixed-step BDF2 over four periods of the drive."""
    flat = K.butterworth_va(pkg).flatten()
    o = pkg.make_opts("bdf2", False, 0.0, 25.0, 0.01, False)
    sol = pkg.tran(flat, (0.0, 25.0), method="bdf2", h=0.01, adaptive=False, dcop=False,
                   x0=np.zeros(flat.n))
    t_ref, x_ref, st, rc = oracle.tran(flat, o, np.zeros(flat.n))
    assert rc == 0 and sol.retcode == "OK" and sol.stats["accepted"] == st.accepted == 2500
    assert compare_waves(sol, t_ref, x_ref, flat.n_nodes) <= 1.0


def test_va_white_noise_psd(gpu, pkg, oracle):
    """cedar_noise with Verilog-A white_noise sources (the Butterworth of
    test/ac.jl with VA resistors; the saturating transconductor's channel noise):
    against the oracle, and the filter against the reference's ngspice table."""
    import json
    import pathlib
    fv = K.butterworth_ac_va(pkg).flatten()
    x = pkg.dc(fv)
    w = 2 * np.pi * pkg.acdec(20, 0.01, 10)
    psd = pkg.noise(fv, x_op=x).psd("vout", w)
    po = oracle.noise(fv, x, w, fv.index("vout"))
    np.testing.assert_allclose(psd, po, rtol=1e-9)
    g = json.loads((pathlib.Path(__file__).with_name("golden") / "ac_noise_ngspice.json").read_text())
    ref = np.array(g["sqrt_psd"])
    assert np.all(np.abs(np.sqrt(psd) - ref) <= 1e-6 * np.maximum(np.abs(ref), np.abs(np.sqrt(psd))))
    fc = K.va_vccs(pkg).flatten()
    xc = pkg.dc(fc)
    wc = 2 * np.pi * pkg.acdec(5, 1e6, 1e11)
    pc = pkg.noise(fc, x_op=xc).psd("e", wc)
    pco = oracle.noise(fc, xc, wc, fc.index("e"))
    np.testing.assert_allclose(pc, pco, rtol=1e-9)
    assert np.all(pc > 0)


def _flicker_divider(pkg):
    """A 1/f resistor (thermal + flicker_noise(KF |I|^AF, EF)) over a plain one."""
    c = pkg.Circuit(temp_c=27.0, gmin=0.0)
    c.V("V1", "vin", "0", dc=2.0)
    c.va("R1", "va_resistor_1f", ["vin", "out"], R=3e3, KF=1e-14, AF=2.0, EF=1.1)
    c.R("R2", "out", "0", r=1e3)
    return c


def test_va_flicker_noise_psd(gpu, pkg, oracle):
    """cedar_noise with a flicker_noise source (density pwr / f^exp, src/ac.jl:
    267-276): the GPU's per-source frequency weighting against the oracle and
    against the divider's closed form (R1 || R2)^2 (4kT/R1 + 4kT/R2 + KF |I|^AF / f^EF)."""
    f = _flicker_divider(pkg).flatten()
    x = pkg.dc(f)
    hz = np.logspace(-1, 9, 41)
    w = 2 * np.pi * hz
    psd = pkg.noise(f, x_op=x).psd("out", w)
    po = oracle.noise(f, x, w, f.index("out"))
    np.testing.assert_allclose(psd, po, rtol=1e-9)
    R1, R2, KF, AF, EF, vdd = 3e3, 1e3, 1e-14, 2.0, 1.1, 2.0
    kT4 = 4 * 1.380649e-23 * (27.0 + 273.15)
    rp = R1 * R2 / (R1 + R2)
    want = rp ** 2 * (kT4 / R1 + kT4 / R2 + KF * (vdd / (R1 + R2)) ** AF / hz ** EF)
    np.testing.assert_allclose(psd, want, rtol=1e-9)
    # the 1/f part dominates at low frequency and vanishes at high frequency
    assert psd[0] > 100 * psd[-1]
