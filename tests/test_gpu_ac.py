"""GPU AC and noise analysis (cedar_ac / cedar_noise) against the oracle's dense
complex solves, and against CedarSim's own AC known answers (test/ac.jl:17-149)."""
import json
import pathlib

import numpy as np
import pytest

from tests import circuits as K

pytestmark = pytest.mark.gpu

GOLDEN = pathlib.Path(__file__).with_name("golden") / "ac_noise_ngspice.json"
K_B = 1.380649e-23
TOL = 1e-9     # GPU vs oracle, relative to the largest probed magnitude at that frequency


def isapprox(a, b, rtol):
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


def amp_chain(pkg, stages=3):
    """Inverter chain biased in saturation (input at 0.85 V, lambda 0.05): a
    MOSFET small-signal path with real gain."""
    c = pkg.Circuit()
    c.V("VDD", "vdd", "0", dc=1.8)
    c.V("VIN", "s0", "0", dc=0.85, ac=1.0)
    for k in range(1, stages + 1):
        a, b = f"s{k - 1}", f"s{k}"
        c.mos1(f"MN{k}", b, a, "0", "0", 1.0, 2e-6, 1e-6, 200e-6, 0.45, LAMBDA=0.05)
        c.mos1(f"MP{k}", b, a, "vdd", "vdd", -1.0, 5e-6, 1e-6, 80e-6, -0.45, LAMBDA=0.05)
        c.C(f"CL{k}", b, "0", c=10e-15)
        c.R(f"RL{k}", b, "0", r=50e3)
    return c.flatten()


def cases(pkg):
    g = pkg.generators
    out = []
    f = amp_chain(pkg)
    out.append(("amp_chain", f, ["s1", "s2", "s3"], "s3", 2 * np.pi * pkg.acdec(5, 1e3, 1e13)))
    f = K.mixed(pkg).flatten()
    f.ac = {"VIN": 1.0}
    out.append(("mixed", f, ["out1", "n2"], "out1", 2 * np.pi * pkg.acdec(5, 1e3, 1e13)))
    f = g.rc_ladder(100).flatten()
    f.ac = {"V1": 1.0}
    out.append(("rc_ladder_100", f, [f.names[1], f.names[50], f.names[100]], f.names[100],
                2 * np.pi * pkg.acdec(10, 1e3, 1e12)))
    f = g.ring_oscillator().flatten()
    f.ac = {"VDD": 1.0}
    out.append(("ring_15", f, ["out1", "out8", "vdd3"], "out1", 2 * np.pi * pkg.acdec(5, 1e3, 1e13)))
    return out


def test_butterworth_known_answers(gpu, pkg):
    flat = K.butterworth_ac(pkg).flatten()
    w = 2 * np.pi * pkg.acdec(20, 0.01, 10)
    s = 1j * w
    acs = pkg.ac(flat)
    r = acs.freqresp(["vout", "vin", ("n1", "vout")], w)
    assert np.all(acs.status == 0)
    H = K.butterworth_H(s)
    np.testing.assert_allclose(r[:, 0], H, rtol=1e-11, atol=0)                  # test/ac.jl:47
    np.testing.assert_allclose(r[:, 1], 1.0, rtol=1e-13, atol=0)                # test/ac.jl:49
    np.testing.assert_allclose(r[:, 2], s * 0.5 * H, rtol=1e-11, atol=0)        # test/ac.jl:61-64
    psd = pkg.noise(flat).psd("vout", w)
    apsd = np.sqrt(4 * K_B * (23 + 273.15)) * np.abs(K.butterworth_Z(s))         # test/ac.jl:72-81
    np.testing.assert_allclose(np.sqrt(psd), apsd, rtol=1e-10)
    assert isapprox(np.sqrt(psd), np.array(json.loads(GOLDEN.read_text())["sqrt_psd"]), 1e-6)  # test/ac.jl:148-149


@pytest.mark.parametrize("name", ["amp_chain", "mixed", "rc_ladder_100", "ring_15"])
def test_ac_and_noise_match_oracle(gpu, pkg, oracle, name):
    _, flat, probes, nprobe, w = [c for c in cases(pkg) if c[0] == name][0]
    x, _, rc = oracle.dcop(flat)
    assert rc == 0
    sys = pkg.System(flat)
    acs = pkg.ACSol(sys, x)
    r = acs.freqresp(probes, w)
    assert np.all(acs.status == 0)
    ro = oracle.ac(flat, x, w, [flat.index(p) for p in probes])
    scale = np.max(np.abs(ro), axis=1, keepdims=True)
    assert np.all(np.abs(r - ro) <= TOL * scale), np.max(np.abs(r - ro) / scale)
    if name == "ring_15":   # metastable point: low frequencies need the dense rerun
        assert pkg.ac_last_stats(sys)["n_dense"] > 0
    ns = pkg.NoiseSol(sys, x)
    psd = ns.psd(nprobe, w)
    assert np.all(ns.status == 0)
    po = oracle.noise(flat, x, w, flat.index(nprobe))
    np.testing.assert_allclose(psd, po, rtol=2 * TOL, atol=1e-300)


def test_results_do_not_depend_on_the_warp(gpu, pkg):
    """A frequency's result has the same bits wherever it sits in the list (each
    warp runs the task lists in the same lane order)."""
    flat = amp_chain(pkg)
    sys = pkg.System(flat)
    acs = pkg.ac(sys)
    w = 2 * np.pi * pkg.acdec(10, 1e3, 1e13)
    a = acs.freqresp(["s1", "s3"], w)
    w2 = np.concatenate([w[::-1], w[: len(w) // 2], 2 * np.pi * np.linspace(1e6, 1e9, 5000)])
    b = acs.freqresp(["s1", "s3"], w2)
    assert np.array_equal(a[::-1], b[: len(w)])
    assert np.array_equal(a[: len(w) // 2], b[len(w): len(w) + len(w) // 2])
    ns = pkg.noise(sys)
    assert np.array_equal(ns.psd("s3", w)[::-1], ns.psd("s3", w2)[: len(w)])


def test_singular_frequency_is_reported(gpu, pkg):
    """A node tied only through capacitors has no DC path: G + j0 C is singular
    at omega = 0 (status ZERO_PIVOT, NaN), while omega > 0 gives the divider."""
    c = pkg.Circuit(gmin=0.0)
    c.V("V1", "a", "0", dc=0.0, ac=1.0)
    c.C("C1", "a", "b", c=1e-12); c.C("C2", "b", "0", c=3e-12)
    flat = c.flatten()
    acs = pkg.ac(flat, x_op=np.zeros(flat.n))
    r = acs.freqresp("b", np.array([0.0, 1e6, 1e9]))
    assert list(acs.status) == [2, 0, 0]              # CEDAR_ST_ZERO_PIVOT, OK, OK
    assert np.isnan(r[0])
    np.testing.assert_allclose(r[1:], 0.25, rtol=1e-14)


def test_argument_checks(gpu, pkg):
    flat = amp_chain(pkg)
    acs = pkg.ac(flat)
    assert acs.freqresp("s1", np.zeros(0)).shape == (0,)
    with pytest.raises(pkg.CedarError):
        acs.freqresp(flat.n + 3, np.array([1.0]))
    with pytest.raises(pkg.CedarError):
        pkg.noise(flat).psd(-1, np.array([1.0]))
