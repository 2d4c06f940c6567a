"""Oracle AC and noise analysis, pinned by CedarSim's AC test on a third-order
Butterworth filter (test/ac.jl:17-81): the analytic transfer functions and the
ngspice noise table the reference checks at rtol 1e-6 (test/ac.jl:83-149).
Also the host-side AC drive vector and acdec against the oracle's own."""
import json
import math
import pathlib

import numpy as np
import pytest

from tests import circuits as K

GOLDEN = pathlib.Path(__file__).with_name("golden") / "ac_noise_ngspice.json"
K_B = 1.380649e-23


def isapprox(a, b, rtol):
    """Julia's isapprox on arrays: norm(a - b) <= rtol * max(norm(a), norm(b))."""
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


@pytest.fixture(scope="module")
def bw(pkg, oracle):
    flat = K.butterworth_ac(pkg).flatten()
    x, st, rc = oracle.dcop(flat)
    assert rc == 0
    return flat, x


def test_acdec_matches_spice_dec_sweep(pkg):
    f = pkg.acdec(20, 0.01, 10)                  # test/ac.jl:38
    assert len(f) == 61 and f[0] == pytest.approx(0.01, rel=1e-15) and f[-1] == pytest.approx(10.0, rel=1e-15)
    assert np.allclose(np.diff(np.log10(f)), 1 / 20, rtol=1e-12)


def test_butterworth_response_analytic(pkg, oracle, bw):
    flat, x = bw
    w = 2 * np.pi * pkg.acdec(20, 0.01, 10)
    s = 1j * w
    n = flat.names
    r = oracle.ac(flat, x, w, [n.index("vout"), n.index("vin"), n.index("n1")])
    H = K.butterworth_H(s)
    np.testing.assert_allclose(r[:, 0], H, rtol=1e-12, atol=0)                      # test/ac.jl:47
    np.testing.assert_allclose(r[:, 1], 1.0, rtol=1e-14, atol=0)                    # test/ac.jl:49
    np.testing.assert_allclose(r[:, 2] - r[:, 0], s * 0.5 * H, rtol=1e-12, atol=0)  # V(L3), test/ac.jl:61-64


def test_butterworth_noise_analytic_and_ngspice(pkg, oracle, bw):
    flat, x = bw
    g = json.loads(GOLDEN.read_text())
    w = 2 * np.pi * pkg.acdec(20, 0.01, 10)
    assert np.allclose(np.array(g["f_hz"]), w / (2 * np.pi), rtol=1e-6)   # table printed to 7 digits
    psd = oracle.noise(flat, x, w, flat.index("vout"))
    T = 23 + 273.15
    apsd = np.sqrt(4 * K_B * T / 1.0) * np.abs(K.butterworth_Z(1j * w))   # test/ac.jl:72-81
    np.testing.assert_allclose(np.sqrt(psd), apsd, rtol=1e-10)
    assert isapprox(np.sqrt(psd), np.array(g["sqrt_psd"]), 1e-6)          # test/ac.jl:148-149


def test_ac_drive_host_matches_oracle(pkg, oracle):
    """The product's drive vector (explicit stamps) equals the oracle's (a unit
    step of eps through the oracle's own source equations), V and I sources with
    multiplicity included."""
    c = pkg.Circuit()
    c.V("V1", "a", "0", dc=1.8, ac=0.7)
    c.I("I1", "b", "a", dc=1e-3, m=3.0, ac=2e-3)
    c.I("I2", "0", "c", dc=0.0, ac=1e-3)
    c.R("R1", "a", "b", r=1e3); c.R("R2", "b", "0", r=2e3); c.R("R3", "c", "0", r=5e2); c.C("C1", "b", "0", c=1e-12)
    flat = c.flatten()
    x, _, rc = oracle.dcop(flat)
    assert rc == 0
    np.testing.assert_allclose(pkg.ac_drive(flat), oracle.ac_drive(flat, x), rtol=1e-14, atol=1e-18)
