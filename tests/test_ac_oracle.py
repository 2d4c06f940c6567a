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


def _ladder(pkg, sections=100, r=1e3, c=1e-12):
    """The AC / noise workload's RC ladder (the bench's AC leg), AC 1 at its input."""
    ckt = pkg.Circuit()
    ckt.V("V1", "n0", "0", dc=0.0, ac=1.0)
    for k in range(1, sections + 1):
        ckt.R(f"R{k}", f"n{k-1}", f"n{k}", r=r)
        ckt.C(f"C{k}", f"n{k}", "0", c=c)
    return ckt.flatten()


def test_rc_ladder_response_and_noise_analytic(pkg, oracle):
    """The 100-section RC ladder of the AC / noise workload against closed forms:
    the response at sections 50 and 100 from the product of the sections' chain
    (ABCD) matrices, and the output noise from Nyquist's theorem, 4 k T Re Z_out
    for the resistors' thermal noise with the source shorted, over 1 kHz .. 1 THz."""
    N, R, Cap = 100, 1e3, 1e-12
    flat = _ladder(pkg, N, R, Cap)
    x, st, rc = oracle.dcop(flat)
    assert rc == 0
    f = pkg.acdec(10, 1e3, 1e12)
    w = 2 * np.pi * f
    r = oracle.ac(flat, x, w, [flat.index("n50"), flat.index(f"n{N}")])
    for q, s in enumerate(1j * w):
        # [V_in, I_in] = M_1 ... M_N [V_out, 0], M_k = series R then shunt C, from
        # the open output backwards, rescaled each section (log10 of the scale
        # kept) because |V_in / V_out| reaches 1e380 at the top of the sweep
        v, i, lg = 1.0 + 0j, 0.0 + 0j, 0.0
        lg50 = None
        for k in range(N, 0, -1):
            if k == 50:                      # |v| = 1 here: V_50 = v 10^lg
                lg50, ph50 = lg, v
            i = i + s * Cap * v             # shunt C at node k
            v = v + R * i                   # series R from node k-1
            m = abs(v)
            v, i, lg = v / m, i / m, lg + np.log10(m)
        # H_out = V_out / V_in = 1 / (v 10^lg), H_50 = V_50 / V_in
        for col, (lgH, ph) in enumerate(((lg50 - lg, ph50 / v), (-lg, 1.0 / v))):
            if lgH < -250:                  # below what double precision holds: both ~0
                assert abs(r[q, col]) < 1e-200
                continue
            H = 10.0 ** lgH * ph / abs(ph)
            assert abs(r[q, col] - H) <= 1e-10 * abs(H), (f[q], col, r[q, col], H)
    psd = oracle.noise(flat, x, w, flat.index(f"n{N}"))
    T = flat.temp_c + 273.15
    for q, s in enumerate(1j * w):
        z = 0.0 + 0j                        # the shorted source
        for _ in range(N):
            z = z + R
            z = z / (1.0 + s * Cap * z)     # in parallel with the shunt C
        assert abs(psd[q] - 4 * K_B * T * z.real) <= 1e-9 * 4 * K_B * T * z.real
