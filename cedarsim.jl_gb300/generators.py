"""Seeded synthetic circuits for the benchmark workloads.

Randomness: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
as easy as 1, 2, 3", SC'11), keyed by (seed, workload id), counter =
(instance, device, parameter, 0).  Normals by Box-Muller, uniforms as
(u + 0.5) / 2^32.  The same numbers are produced on any host, so CPU and GPU runs
see identical parameters.

Workloads:
  1. RC ladder: 100 sections, series R = 1 kOhm, shunt C = 1 pF per node, driven by
     PULSE(0 1 0 1n 1n 50n 100n); trapezoidal, h = 0.1 ns, 0..1 us.
  2. 31-stage CMOS inverter chain (level-1 MOSFETs): VDD = 1.8 V, Vth_n = 0.45,
     Vth_p = -0.45, KP_n = 200 uA/V^2, KP_p = 80 uA/V^2, W/L = 2 (n) / 4 (p),
     10 fF load per stage, input PULSE(0 1.8 0 50p 50p 950p 2n); BDF2, h = 1 ps, 0..20 ns.
  3. Monte Carlo: 4096 chains with L drawn uniformly from {5, 7, ..., 63}; per
     transistor Vth ~ N(nominal, 0.03 V), KP ~ nominal * exp(0.05 z); per instance
     load C ~ U(5, 20) fF; adaptive BDF2 (reltol 1e-6, abstol 1e-9 V) to 20 ns.
"""
from __future__ import annotations

import math
from typing import List, Tuple

import numpy as np

from .circuit import Circuit, Flat, Pulse, MOS1, C as MODEL_C

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
MASK32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr: np.ndarray, key: np.ndarray) -> np.ndarray:
    """Philox4x32-10 on a batch of counters.  ctr: (..., 4) uint32, key: (..., 2) uint32."""
    c = [np.asarray(ctr[..., i], dtype=np.uint32).astype(np.uint64) for i in range(4)]
    k0 = np.asarray(key[..., 0], dtype=np.uint32).copy()
    k1 = np.asarray(key[..., 1], dtype=np.uint32).copy()
    for r in range(10):
        if r > 0:
            k0 = (k0 + W0).astype(np.uint32)
            k1 = (k1 + W1).astype(np.uint32)
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK32
        c = [hi1 ^ c[1] ^ k0.astype(np.uint64), lo1, hi0 ^ c[3] ^ k1.astype(np.uint64), lo0]
    return np.stack([x.astype(np.uint32) for x in c], axis=-1)


class Stream:
    """Counter-based stream: draw(i, d, p) -> 4 uint32 for instance i, device d, param p."""

    def __init__(self, seed: int, workload: int):
        self.key = np.array([seed & 0xFFFFFFFF, workload & 0xFFFFFFFF], dtype=np.uint32)

    def bits(self, inst, dev, par) -> np.ndarray:
        inst, dev, par = np.broadcast_arrays(np.asarray(inst), np.asarray(dev), np.asarray(par))
        ctr = np.stack([inst.astype(np.uint32), dev.astype(np.uint32), par.astype(np.uint32),
                        np.zeros(inst.shape, np.uint32)], axis=-1)
        return philox4x32_10(ctr, np.broadcast_to(self.key, ctr.shape[:-1] + (2,)))

    def uniform(self, inst, dev, par) -> np.ndarray:
        b = self.bits(inst, dev, par)
        return (b[..., 0].astype(np.float64) + 0.5) / 4294967296.0

    def normal(self, inst, dev, par) -> np.ndarray:
        b = self.bits(inst, dev, par)
        u1 = (b[..., 0].astype(np.float64) + 0.5) / 4294967296.0
        u2 = (b[..., 1].astype(np.float64) + 0.5) / 4294967296.0
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)


# ---------------------------------------------------------------- workload 1
def rc_ladder(sections: int = 100, r: float = 1e3, c: float = 1e-12,
              wave: Pulse = Pulse(0.0, 1.0, 0.0, 1e-9, 1e-9, 50e-9, 100e-9)) -> Circuit:
    ckt = Circuit()
    ckt.V("V1", "n0", "0", wave=wave)
    for k in range(1, sections + 1):
        ckt.R(f"R{k}", f"n{k-1}", f"n{k}", r=r)
        ckt.C(f"C{k}", f"n{k}", "0", c=c)
    return ckt


# ---------------------------------------------------------------- workload 2
INV = dict(vdd=1.8, vth_n=0.45, vth_p=-0.45, kp_n=200e-6, kp_p=80e-6, wn=2e-6, ln=1e-6, wp=4e-6, lp=1e-6,
           cload=10e-15)
INV_PULSE = Pulse(0.0, 1.8, 0.0, 50e-12, 50e-12, 950e-12, 2e-9)


def inverter_chain(stages: int = 31, cload: float = INV["cload"], wave: Pulse = INV_PULSE, **kw) -> Circuit:
    p = dict(INV, **kw)
    ckt = Circuit()
    ckt.node("in"); ckt.node("vdd")
    ckt.V("VIN", "in", "0", wave=wave)
    ckt.V("VDD", "vdd", "0", dc=p["vdd"])
    prev = "in"
    for k in range(1, stages + 1):
        out = f"out{k}"
        ckt.mos1(f"MN{k}", out, prev, "0", "0", 1.0, p["wn"], p["ln"], p["kp_n"], p["vth_n"])
        ckt.mos1(f"MP{k}", out, prev, "vdd", "vdd", -1.0, p["wp"], p["lp"], p["kp_p"], p["vth_p"])
        ckt.C(f"CL{k}", out, "0", cload)
        prev = out
    return ckt


def inverter_chain_flat(stages: int, cload: float = INV["cload"], wave: Pulse = INV_PULSE, ordering: int = 1) -> Flat:
    """The flattened inverter chain built directly with numpy (same devices, nodes
    and parameters as inverter_chain(stages).flatten(); the per-device name index
    is left empty), for chains of a million stages.  Nodes: in, vdd, out1..outL;
    branches: VIN.I, VDD.I."""
    from .circuit import V as MODEL_V, WAVE_PULSE
    L = int(stages)
    n_nodes = L + 2
    k = np.arange(1, L + 1)
    out = 1 + k
    inp = np.where(k == 1, 0, out - 1)
    cap_term = np.stack([out, np.full(L, -1)], axis=1)
    cap_par = np.stack([np.full(L, cload), np.ones(L)])
    vterm = np.array([[0, -1], [1, -1]])
    vbr = np.array([n_nodes, n_nodes + 1])
    vpar = np.zeros((10, 2))
    vpar[0] = 1.0
    vpar[1] = [wave.v1, INV["vdd"]]
    vpar[2] = [WAVE_PULSE, 0.0]
    vpar[3:10, 0] = [wave.v1, wave.v2, wave.td, wave.tr, wave.tf, wave.pw, wave.per]
    # MOSFETs in device order MN1, MP1, MN2, MP2, ...
    d = np.repeat(out, 2); g = np.repeat(inp, 2)
    is_p = np.tile([False, True], L)
    src = np.where(is_p, 1, -1); bulk = src
    mterm = np.stack([d, g, src, bulk], axis=1)
    mpar = np.stack([np.where(is_p, -1.0, 1.0), np.where(is_p, INV["wp"], INV["wn"]), np.where(is_p, INV["lp"], INV["ln"]),
                     np.where(is_p, INV["kp_p"], INV["kp_n"]), np.where(is_p, INV["vth_p"], INV["vth_n"]),
                     np.zeros(2 * L), np.ones(2 * L)])
    groups = [(MODEL_C, cap_term.astype(np.int32), None, cap_par), (MODEL_V, vterm.astype(np.int32), vbr.astype(np.int32), vpar),
              (MOS1, mterm.astype(np.int32), None, mpar)]
    names = ["in", "vdd"] + [f"out{i}" for i in range(1, L + 1)] + ["VIN.I", "VDD.I"]
    return Flat(n_nodes, 2, groups, np.zeros(0), 27.0, 1e-12, names, {}, ordering)


# ---------------------------------------------------------------- workload 3
MC_LENGTHS = list(range(5, 64, 2))


def mc_chains(n_inst: int = 4096, seed: int = 20240607, workload: int = 3,
              lengths: List[int] = MC_LENGTHS) -> Tuple[List[Flat], np.ndarray, np.ndarray, np.ndarray]:
    """Monte Carlo chains.  Returns (templates, inst_template, inst_par, inst_par_off).

    Template k is the chain of length lengths[k]; an instance's parameter block is
    the template's block with its MOSFET VTO/KP and load C replaced.
    Random draws: chain length  -> stream(i, 0, 0) uniform;
                  load C        -> stream(i, 0, 1) uniform;
                  MOSFET j Vth  -> stream(i, 1 + j, 0) normal;  KP -> stream(i, 1 + j, 1) normal.
    """
    st = Stream(seed, workload)
    idx = np.arange(n_inst)
    lsel = np.minimum((st.uniform(idx, 0, 0) * len(lengths)).astype(np.int64), len(lengths) - 1)
    cl = 5e-15 + st.uniform(idx, 0, 1) * 15e-15
    templates = [inverter_chain(L).flatten() for L in lengths]
    blocks = []
    offs = np.zeros(n_inst, np.int64)
    pos = 0
    for i in range(n_inst):
        f = templates[lsel[i]]
        blk = f.param_block().copy()
        off_m = 0
        for (model, term, br, par) in f.groups:
            npar, ninst = par.shape
            if model == MOS1:
                j = np.arange(ninst)
                vth_nom = par[4]
                kp_nom = par[3]
                z1 = st.normal(i, 1 + j, 0)
                z2 = st.normal(i, 1 + j, 1)
                blk[off_m + 4 * ninst: off_m + 5 * ninst] = vth_nom + 0.03 * z1 * np.sign(par[0])
                blk[off_m + 3 * ninst: off_m + 4 * ninst] = kp_nom * np.exp(0.05 * z2)
            elif model == MODEL_C:
                blk[off_m + 0: off_m + ninst] = cl[i]
            off_m += npar * ninst
        offs[i] = pos
        pos += blk.size
        blocks.append(blk)
    return templates, lsel.astype(np.int32), np.concatenate(blocks), offs


# ---------------------------------------------------------------- workload 5
ADJ_LENGTHS = list(range(31, 64, 2))   # 62..126 transistor widths per instance
ADJ_LEVEL = 0.9                        # 50 % of VDD
ADJ_W_ENERGY = 1e15                    # J -> fJ
ADJ_W_DELAY = 1e24                     # s^2 -> ps^2


def adjoint_chains(n_inst: int = 512, seed: int = 20240607, workload: int = 5, lengths: List[int] = ADJ_LENGTHS):
    """Monte Carlo chains for the discrete adjoint: the chains of mc_chains with
    L in {31, 33, .., 63}, the per-template objective (supply energy through VDD +
    squared error of the last output's first 50 % crossing against t*) and a seeded
    target t* per instance: L * 20 ps * U(0.8, 1.2), drawn from stream(i, 0, 2).

    Returns (templates, inst_template, inst_par, inst_par_off, objectives, tstar) with
    objectives[k] = (vnode, ibranch, probe, level, w_energy, w_delay, w_final)."""
    templates, itpl, par, off = mc_chains(n_inst, seed=seed, workload=workload, lengths=lengths)
    st = Stream(seed, workload)
    u = st.uniform(np.arange(n_inst), 0, 2)
    L = np.array(lengths)[itpl]
    tstar = L * 20e-12 * (0.8 + 0.4 * u)
    objectives = [(f.index("vdd"), f.index("VDD.I"), chain_output_probe(f), ADJ_LEVEL, ADJ_W_ENERGY, ADJ_W_DELAY, 0.0)
                  for f in templates]
    return templates, itpl, par, off, objectives, tstar


# ---------------------------------------------------------------- workload 4
RING = dict(stages=15, vdd=1.8, vbn=1.0, vbp=0.8, rsup=100.0, csup=100e-15, cload=5e-15)


def ring_oscillator(stages: int = RING["stages"], diode_is=None, diode_n=None, **kw) -> Circuit:
    """Current-starved ring oscillator.  Stage k (input out_{k-1}, out_0 = out_N):
    MP_starve (ps_k <- vbp, source vdd_k), MP (out_k <- out_{k-1}, source ps_k),
    MN (out_k <- out_{k-1}, source ns_k), MN_starve (ns_k <- vbn, source 0),
    100 Ohm from VDD to vdd_k with 100 fF to ground, a Verilog-A exponential diode
    out_k -> vdd_k, and a 5 fF load on out_k (level-1 MOSFETs carry no charge, so
    the load is what gives each stage its delay)."""
    p = dict(INV, **RING)
    p.update(kw)
    ckt = Circuit()
    for nm in ("vdd", "vbn", "vbp"):
        ckt.node(nm)
    ckt.V("VDD", "vdd", "0", dc=p["vdd"])
    ckt.V("VBN", "vbn", "0", dc=p["vbn"])
    ckt.V("VBP", "vbp", "0", dc=p["vbp"])
    for k in range(1, stages + 1):
        inp = f"out{stages if k == 1 else k - 1}"
        out, vk, ps, ns = f"out{k}", f"vdd{k}", f"ps{k}", f"ns{k}"
        ckt.R(f"RS{k}", "vdd", vk, r=p["rsup"])
        ckt.C(f"CS{k}", vk, "0", p["csup"])
        ckt.mos1(f"MPS{k}", ps, "vbp", vk, vk, -1.0, p["wp"], p["lp"], p["kp_p"], p["vth_p"])
        ckt.mos1(f"MP{k}", out, inp, ps, vk, -1.0, p["wp"], p["lp"], p["kp_p"], p["vth_p"])
        ckt.mos1(f"MN{k}", out, inp, ns, "0", 1.0, p["wn"], p["ln"], p["kp_n"], p["vth_n"])
        ckt.mos1(f"MNS{k}", ns, "vbn", "0", "0", 1.0, p["wn"], p["ln"], p["kp_n"], p["vth_n"])
        isv = 1e-15 if diode_is is None else diode_is[k - 1]
        nv = 1.1 if diode_n is None else diode_n[k - 1]
        ckt.diode(f"D{k}", out, vk, IS=isv, N=nv)
        ckt.C(f"CL{k}", out, "0", p["cload"])
    return ckt


def mc_rings(n_inst: int = 1024, seed: int = 20240607, workload: int = 4):
    """Ring-oscillator sweep: per instance Is ~ loguniform(1e-16, 1e-14) A and
    n ~ U(1.0, 1.2) per diode; DC operating point perturbed by N(0, 1 mV) on every
    node.  Returns (template, inst_template, inst_par, inst_par_off, inst_dx, inst_dx_off).
    Draws: diode j Is -> stream(i, 1 + j, 0) uniform; n -> stream(i, 1 + j, 1);
           node u perturbation -> stream(i, 1000 + u, 0) normal."""
    from .circuit import DIODE as MODEL_D
    st = Stream(seed, workload)
    flat = ring_oscillator().flatten()
    base = flat.param_block()
    blocks, offs = [], np.zeros(n_inst, np.int64)
    dxs, dx_off = [], np.zeros(n_inst, np.int64)
    for i in range(n_inst):
        blk = base.copy()
        off_m = 0
        for (model, term, br, par) in flat.groups:
            npar, ninst = par.shape
            if model == MODEL_D:
                j = np.arange(ninst)
                u1 = st.uniform(i, 1 + j, 0)
                u2 = st.uniform(i, 1 + j, 1)
                blk[off_m: off_m + ninst] = 10.0 ** (-16.0 + 2.0 * u1)          # IS
                blk[off_m + ninst: off_m + 2 * ninst] = 1.0 + 0.2 * u2          # N
            off_m += npar * ninst
        offs[i] = i * base.size
        blocks.append(blk)
        dx = np.zeros(flat.n)
        u = np.arange(flat.n_nodes)
        dx[:flat.n_nodes] = 1e-3 * st.normal(i, 1000 + u, 0)
        dx_off[i] = i * flat.n
        dxs.append(dx)
    return [flat], np.zeros(n_inst, np.int32), np.concatenate(blocks), offs, np.concatenate(dxs), dx_off


def as_verilog_a(flat: Flat) -> Flat:
    """The same circuit with its level-1 MOSFETs and exponential diodes as the
    Verilog-A modules va_mos1 / va_diode compiled by the emitter (their parameter
    blocks are the built-in models' blocks, parameter for parameter), so instance
    parameter blocks of the built-in template serve the Verilog-A one unchanged.
    Group order is kept."""
    import copy
    from . import va
    from .circuit import DIODE as MODEL_D
    swap = {MOS1: va.model_id("va_mos1"), MODEL_D: va.model_id("va_diode")}
    g = copy.deepcopy(flat)
    g.groups = [(swap.get(m, m), t, b, p) for (m, t, b, p) in g.groups]
    return g


def instance_flat(template: Flat, block: np.ndarray) -> Flat:
    """The template with one instance's parameter block substituted (a stand-alone circuit)."""
    groups, p = [], 0
    for (model, term, br, par) in template.groups:
        groups.append((model, term, br, np.ascontiguousarray(block[p:p + par.size].reshape(par.shape))))
        p += par.size
    return Flat(template.n_nodes, template.n_branch, groups, template.pwl, template.temp_c, template.gmin,
                template.names, template.devices, template.ordering, dict(template.ac))


def chain_output_probe(flat: Flat) -> int:
    """Unknown index of the last stage output of a chain template."""
    outs = [k for k, nm in enumerate(flat.names) if nm.startswith("out")]
    return max(outs, key=lambda k: int(flat.names[k][3:]))
