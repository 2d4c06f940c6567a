"""SimpleDiode (src/simpledevices.jl:134-271) restated literally in the oracle.

PARITY UNPINNED: no reference test solves a circuit with this model
(test/basic.jl:456-468 only constructs it), so these checks pin the restatement
to the reference's source line by line, evaluated by hand here: with the
defaults, q = -1.602176634e-19 makes the breakdown current expm1(-q BV / NkT)
overflow to +inf (so the NVt branch is skipped) and puts the boundary between
the "forward" and low-bias branches at Vd = -3 NkT / q = +0.0776 V; the
low-bias branch -ISeff (1 + (3 NkT / (q Vd e))^3) has a pole at Vd = 0; the
"forward" branch ISeff expm1(q Vd / NkT) is reverse-like; AREAeff = AREA * M.
The device is not part of the GPU path (its residual is not finite where a
DC solve starts).
"""
import math

import numpy as np

Q, K, T = -1.602176634e-19, 1.380649e-23, 300.0
NKT = K * T
ISEFF = 1e-14 * 0.5              # IS * AREA * M


def _low(vd):
    r = 3 * NKT / (Q * vd * math.e)
    return -ISEFF * (1 + r * r * r) + vd * 1e-12


def test_branches_and_values(oracle):
    thr = -3 * NKT / Q
    assert abs(thr - 0.0776) < 1e-4
    rc, Id, Ideff, Cdep, TT, Cdiff_dc = oracle.simple_diode(0.0)
    assert rc == 0 and Id == math.inf and math.isnan(Ideff)                 # the pole at 0
    for vd in (1e-3, -1e-3, 0.05, -0.3):
        rc, Id, Ideff, Cdep, TT, Cdiff_dc = oracle.simple_diode(vd)
        assert rc == 0 and Id == _low(vd) and Ideff == Id                      # IKeff = inf
        assert Cdep == 0.0 and math.isnan(Cdiff_dc)                           # CJO = 0; TT * 0 / 0
    for vd in (0.1, 0.2, 0.45):
        rc, Id, *_ = oracle.simple_diode(vd)
        assert rc == 0 and Id == ISEFF * math.expm1(Q * vd / NKT) + vd * 1e-12
        assert -ISEFF < Id - vd * 1e-12 < 0                                  # reverse-like under forward bias
    assert abs(oracle.simple_diode(1e-3)[1] - 1.16e-10) < 1e-12


def test_depletion_capacitance(oracle):
    rc, Id, Ideff, Cdep, TT, _ = oracle.simple_diode(0.2, CJO=1e-12, TT=1e-9)
    cjeff = 1e-12 * 0.5
    want = cjeff * (1 - 0.2) ** -0.5 + cjeff * (1 - 0.2) ** (-1 / 3)
    assert rc == 0 and np.isclose(Cdep, want, rtol=1e-15) and TT == 1e-9


def test_reference_run_time_errors(oracle):
    # Vd >= FC * VJ reads the undefined MJI (:260)
    assert oracle.simple_diode(0.5)[0] == 2 and oracle.simple_diode(0.7)[0] == 2
    # a breakdown current below IBVeff reads the undefined NVt (:238)
    assert oracle.simple_diode(0.1, BV=1e-3)[0] == 1
    # a negative current over the hard-coded IKR = Inf gives sqrt(-0.0), which
    # Base.sqrt accepts (a finite IKR would throw DomainError)
    rc, Id, Ideff, *_ = oracle.simple_diode(-0.3)
    assert rc == 0 and Id < 0 and Ideff == Id
