"""Test circuits: the reference's known-answer cases rebuilt as device tables,
plus mixed-model circuits for parity checks."""
import math

import numpy as np


def vr(pkg):  # test/basic.jl:21-43
    c = pkg.Circuit(); c.V("V", "vcc", "0", dc=5.0); c.R("R", "vcc", "0", r=2.0); return c


def ir(pkg):  # test/basic.jl:81-106
    c = pkg.Circuit(); c.I("I", "icc", "0", dc=-5.0); c.R("R", "icc", "0", r=2.0); return c


def vrc(pkg, m=1.0):  # test/basic.jl:111-166
    c = pkg.Circuit(); c.V("V", "vcc", "0", dc=5.0); c.R("R", "vcc", "vrc", r=2000.0, m=m); c.C("C", "vrc", "0", c=1e-6)
    return c


def spectre_sources(pkg):  # test/basic.jl:168-205 (B5 behavioural source omitted)
    c = pkg.Circuit()
    c.I("I1", "0", "1", dc=2.2e-6); c.R("R1", "1", "0", r=1000.0)
    c.I("I2", "0", "2", wave=pkg.PWL([(0, 1e-3), (0.5, 2e-3), (1.0, 1.75e-3)])); c.R("R2", "2", "0", r=2000.0)
    c.V("V3", "0", "3", dc=1.5); c.R("R3", "3", "0", r=1000.0)
    c.V("V4", "0", "4", wave=pkg.PWL([(0, 1.0), (0.5, 2.0), (1.0, 5.0)])); c.R("R4", "4", "0", r=4000.0)
    return c


def spice_sources(pkg):  # test/basic.jl:207-235
    c = pkg.Circuit()
    c.V("V1", "0", "1", dc=1.0); c.R("R1", "1", "0", r=1e3)
    c.E("B5", "0", "5", "1", "0", 2.0); c.R("R5", "5", "0", r=1e3)
    c.E("E6", "0", "6", "0", "5", 2.0); c.R("R6", "6", "0", r=1e3)
    c.E("E8", "0", "8", "0", "5", 2.0); c.R("R8", "8", "0", r=1e3)
    c.G("G7", "0", "7", "0", "5", 2.0); c.R("R7", "7", "0", r=1e3)
    c.G("G9", "0", "9", "0", "5", 2.0); c.R("R9", "9", "0", r=1e3)
    return c


def multiplicities(pkg):  # test/basic.jl:556-595
    c = pkg.Circuit(); c.V("v1", "vcc", "0", dc=1.0)
    c.R("r1a", "vcc", "1", r=1.0, m=10); c.R("r1b", "1", "0", r=1.0)
    c.R("x2a.r2a", "vcc", "2", r=1.0, m=10); c.R("r2b", "2", "0", r=1.0)
    c.R("x3a1.r2a", "vcc", "3", r=1.0, m=5); c.R("x3a2.r2a", "vcc", "3", r=1.0, m=5); c.R("r3b", "3", "0", r=1.0)
    c.R("x4a1.x5r1.r2a", "vcc", "4", r=1.0, m=5); c.R("x4a1.x5r2.r2a", "vcc", "4", r=1.0, m=5); c.R("r4b", "4", "0", r=1.0)
    c.R("x5a.r2", "vcc", "5", r=1.0, m=10); c.R("r5b", "5", "0", r=1.0)
    c.R("r6a", "vcc", "6", r=1.0, m=10); c.R("r6b", "6", "0", r=1.0)
    return c


def semiconductor_resistor(pkg):  # test/basic.jl:725-737
    c = pkg.Circuit(); c.V("v1", "vcc", "0", dc=1.0)
    c.R("R1", "vcc", "0", rsh=500.0, w=1e-3, l=2e-3); c.R("R2", "vcc", "0", r=1e3)
    return c


def pwl_isource(pkg):  # test/transients.jl:17-63
    c = pkg.Circuit()
    c.I("i1", "vout", "0", wave=pkg.PWL([(1e-3, 0.0), (9e-3, -2.0)])); c.R("R1", "vout", "0", r=2.0)
    return c


def pwl_val(t):
    return 0.0 if t < 1e-3 else (1.0 if t > 9e-3 else (t - 1e-3) / 8e-3)


def butterworth(pkg):  # test/transients.jl:129-179
    c = pkg.Circuit()
    c.V("V1", "vin", "0", wave=pkg.Sin(0.0, 1.0, 1.0 / (2 * math.pi)))
    c.L("L1", "vin", "n1", 1.5); c.C("C2", "n1", "0", 4.0 / 3.0); c.L("L3", "n1", "vout", 0.5); c.R("R4", "vout", "0", r=1.0)
    return c


def butterworth_ac(pkg):  # test/ac.jl:17-35: AC 1 drive, R4 split in two 2-ohm halves, temp 23, gmin 0
    c = pkg.Circuit(temp_c=23.0, gmin=0.0)
    c.V("V1", "vin", "0", wave=pkg.Sin(0.0, 1.0, 1.0 / (2 * math.pi)), ac=1.0)
    c.L("L1", "vin", "n1", 1.5); c.C("C2", "n1", "0", 4.0 / 3.0); c.L("L3", "n1", "vout", 0.5)
    c.R("R4", "vout", "0", r=2.0); c.R("R5", "vout", "0", r=2.0)
    return c


def butterworth_H(s):  # test/ac.jl:42-45: 1 / ((s + 1)(s^2 + s + 1))
    return 1.0 / ((s + 1.0) * (s * s + s + 1.0))


def butterworth_Z(s):  # test/ac.jl:77-79: impedance seen at vout, R4 || (L3 + (L1 || C2)), R4 = 1
    par = lambda a, b: a * b / (a + b)
    return par(par(s * 1.5, 1.0 / (s * 4.0 / 3.0)) + s * 0.5, 1.0)


def butterworth_vout(t):
    return (math.exp(-t) - math.sin(t) - math.cos(t)) / 2 + (2 * math.sin((math.sqrt(3) * t) / 2)) / (math.sqrt(3) * math.sqrt(math.exp(t)))


def nlvcr(pkg):  # test/ddx.jl
    c = pkg.Circuit(); c.V("V1", "vcc", "0", dc=5.0); c.V("V2", "vg", "0", dc=3.0); c.nlvcr("R", "vcc", "vg", "0", R=2.0)
    return c


def two_resistor(pkg, r1=1.0, r2=1.0):  # test/sensitivity.jl:13-42
    c = pkg.Circuit(); c.V("V", "vcc", "0", dc=1.0); c.R("R1", "vcc", "out", r=r1); c.R("R2", "out", "0", r=r2)
    return c


def mixed(pkg):
    """Every model in one circuit (for eval / DC / transient parity)."""
    c = pkg.Circuit()
    c.V("VDD", "vdd", "0", dc=1.8)
    c.V("VIN", "in", "0", wave=pkg.Pulse(0.0, 1.8, 0.1e-9, 50e-12, 60e-12, 0.4e-9, 1e-9))
    c.I("IB", "0", "bias", wave=pkg.PWL([(0.0, 1e-6), (0.3e-9, 5e-6), (0.6e-9, 2e-6)]))
    c.R("RB", "bias", "0", r=20e3)
    c.mos1("MN1", "out1", "in", "0", "0", 1.0, 2e-6, 1e-6, 200e-6, 0.45, LAMBDA=0.02)
    c.mos1("MP1", "out1", "in", "vdd", "vdd", -1.0, 4e-6, 1e-6, 80e-6, -0.45, LAMBDA=0.02)
    c.C("C1", "out1", "0", 5e-15)
    c.R("R2", "out1", "n2", r=1e3, m=2.0)
    c.L("L2", "n2", "n3", 1e-9)
    c.C("C3", "n3", "0", 2e-15)
    c.diode("D1", "n3", "vdd", IS=1e-15, N=1.1)
    c.diode("D2", "0", "n3", IS=3e-16, N=1.05, AREA=2.0)
    c.E("E1", "e1", "0", "n3", "0", 0.5)
    c.R("RE", "e1", "0", r=5e3)
    c.G("G1", "g1", "0", "out1", "0", 1e-4)
    c.R("RG", "g1", "0", r=2e3)
    c.C("CG", "g1", "0", 1e-15)
    c.nlvcr("NL", "nl", "bias", "0", R=1e-3)
    c.R("RNL", "vdd", "nl", r=10e3)
    c.V("VS", "sn", "0", wave=pkg.Sin(0.2, 0.1, 2e9, 0.05e-9, 1e8, 30.0))
    c.R("RS", "sn", "out1", r=50e3)
    return c


# ---------------------------------------------------------------- Verilog-A
def va_nlvcr(pkg):  # test/ddx.jl with the device compiled from Verilog-A
    c = pkg.Circuit(); c.V("V1", "vcc", "0", dc=5.0); c.V("V2", "vg", "0", dc=3.0)
    c.va("R", "va_nlvcr", ["vcc", "vg", "0"], R=2.0)
    return c


def inverter_chain_va(pkg, stages=7, cload=10e-15, builtin=False):
    """The inverter chain of workload 2 with its MOSFETs as the Verilog-A level-1
    model (or the built-in one: same nodes, devices and parameter blocks)."""
    g = pkg.generators
    p = g.INV
    c = pkg.Circuit()
    c.node("in"); c.node("vdd")
    c.V("VIN", "in", "0", wave=g.INV_PULSE)
    c.V("VDD", "vdd", "0", dc=p["vdd"])
    prev = "in"
    for k in range(1, stages + 1):
        out = f"out{k}"
        if builtin:
            c.mos1(f"MN{k}", out, prev, "0", "0", 1.0, p["wn"], p["ln"], p["kp_n"], p["vth_n"])
            c.mos1(f"MP{k}", out, prev, "vdd", "vdd", -1.0, p["wp"], p["lp"], p["kp_p"], p["vth_p"])
        else:
            c.va(f"MN{k}", "va_mos1", [out, prev, "0", "0"], TYPE=1, W=p["wn"], L=p["ln"], KP=p["kp_n"],
                 VTO=p["vth_n"])
            c.va(f"MP{k}", "va_mos1", [out, prev, "vdd", "vdd"], TYPE=-1, W=p["wp"], L=p["lp"], KP=p["kp_p"],
                 VTO=p["vth_p"])
        c.C(f"CL{k}", out, "0", cload)
        prev = out
    return c


def va_mixed(pkg):
    """Every shipped Verilog-A model (resistive, charge and ddx ones) with
    built-in sources and devices around them."""
    c = pkg.Circuit()
    c.V("VDD", "vdd", "0", dc=1.8)
    c.V("VIN", "in", "0", wave=pkg.Pulse(0.0, 1.8, 0.1e-9, 50e-12, 60e-12, 0.4e-9, 1e-9))
    c.va("R1", "va_resistor", ["in", "b"], R=1e3)
    c.va("C1", "va_capacitor", ["b", "0"], C=20e-15)
    c.va("D1", "va_diode", ["b", "c"], IS=1e-14, N=1.05)
    c.va("D2", "va_diode_cj", ["c", "0"], IS=1e-15, N=1.1, TT=2e-11, CJ0=5e-15)
    c.R("RC", "c", "0", r=20e3)
    c.va("MN", "va_mos1", ["d", "b", "0", "0"], TYPE=1, W=2e-6, L=1e-6, KP=200e-6, VTO=0.45, LAMBDA=0.02)
    c.va("MP", "va_mos1", ["d", "b", "vdd", "vdd"], TYPE=-1, W=4e-6, L=1e-6, KP=80e-6, VTO=-0.45, m=2.0)
    c.va("X1", "va_nlvcr", ["d", "c", "0"], R=1e-4)
    c.C("CD", "d", "0", 10e-15)
    c.va("R2", "va_resistor", ["d", "e"], R=5e3, m=2.0)
    c.mos1("MB", "e", "d", "0", "0", 1.0, 2e-6, 1e-6, 200e-6, 0.45)
    c.va("C2", "va_capacitor", ["e", "0"], C=3e-15)
    return c


def va_diode_rs(pkg, twin=False):
    """A pulse through 1 kOhm into a diode with 50 Ohm series resistance on a
    0.5 pF load: the internal-node model, or (twin) the same network built from
    va_resistor + va_diode around an explicit node of the same name."""
    c = pkg.Circuit()
    c.V("VIN", "in", "0", wave=pkg.Pulse(-1.0, 2.0, 0.05e-9, 0.1e-9, 0.1e-9, 0.5e-9, 1.2e-9))
    c.R("R1", "in", "x", r=1e3)
    if twin:
        c.va("RSx", "va_resistor", ["x", "D1.ai"], R=50.0)
        c.va("D1j", "va_diode", ["D1.ai", "0"], IS=1e-14, N=1.05)
    else:
        c.va("D1", "va_diode_rs", ["x", "0"], IS=1e-14, N=1.05, RS=50.0)
    c.C("CL", "x", "0", 0.5e-12)
    return c


def va_vccs(pkg):
    """The saturating transconductor (analog function, macros, case,
    $param_given) driving a resistive load from a pulse."""
    c = pkg.Circuit()
    c.V("VIN", "b", "0", wave=pkg.Pulse(-1.0, 1.0, 0.05e-9, 0.2e-9, 0.2e-9, 0.3e-9, 1e-9))
    c.va("G1", "va_vccs_sat", ["0", "d", "b", "0"], GM=2e-3, VS=0.4, MODE=1)
    c.va("G2", "va_vccs_sat", ["0", "e", "d", "0"], GMX=1e-3, VS=0.3, MODE=2)
    c.R("RD", "d", "0", r=1e3)
    c.R("RE", "e", "0", r=2e3)
    c.C("CE", "e", "0", 50e-15)
    return c


def butterworth_va(pkg):
    """test/transients.jl:129-179's third-order Butterworth with its inductors as
    the Verilog-A voltage-branch model."""
    c = pkg.Circuit()
    c.V("V1", "vin", "0", wave=pkg.Sin(0.0, 1.0, 1.0 / (2 * math.pi)))
    c.va("L1", "va_inductor", ["vin", "n1"], L=1.5); c.C("C2", "n1", "0", 4.0 / 3.0)
    c.va("L3", "va_inductor", ["n1", "vout"], L=0.5); c.R("R4", "vout", "0", r=1.0)
    return c


def va_thevenin(pkg):
    """A Verilog-A Thevenin source (1 V behind 50 Ohm) into a 50 Ohm load, with a
    VA inductor and a capacitor after it for the transient."""
    c = pkg.Circuit()
    c.va("VT", "va_thevenin", ["a", "0"], VS=1.0, RS=50.0)
    c.R("RL", "a", "0", r=50.0)
    c.va("LX", "va_inductor", ["a", "b"], L=5e-9)
    c.C("CB", "b", "0", 2e-12)
    c.R("RB", "b", "0", r=1e3)
    return c


def butterworth_ac_va(pkg):
    """butterworth_ac with its two 2-Ohm load halves as Verilog-A resistors
    (thermal noise through white_noise)."""
    c = pkg.Circuit(temp_c=23.0, gmin=0.0)
    c.V("V1", "vin", "0", wave=pkg.Sin(0.0, 1.0, 1.0 / (2 * math.pi)), ac=1.0)
    c.L("L1", "vin", "n1", 1.5); c.C("C2", "n1", "0", 4.0 / 3.0); c.L("L3", "n1", "vout", 0.5)
    c.va("R4", "va_resistor", ["vout", "0"], R=2.0); c.va("R5", "va_resistor", ["vout", "0"], R=2.0)
    return c
