"""Circuit description and flattening to the C-ABI device table.

A :class:`Circuit` is the elaborated netlist a CedarSim circuit function produces
(nets + device calls).  ``flatten()`` turns it into the flattened device table the
library consumes: one group per model, terminal unknown indices (ground = -1),
branch-current unknowns for V sources / inductors / VCVS, and struct-of-arrays
parameters.  This is the table a Julia ``ccall`` shim would build with the
``aliasextract.jl`` overlay pattern (src/aliasextract.jl:10-40).

Device semantics and defaults follow CedarSim:
  * ``R``: ``res = r`` or ``rsh*(l-short)/(w-narrow)`` when ``r`` is not given
    (src/simpledevices.jl:49-70);
  * ``V``/``I``: ``dc = something(dc, tran(t=0), 0)`` (src/simpledevices.jl:281-285);
  * ground names ``0``/``gnd``/``GND`` map to the reference node (Gnd(),
    src/simpledevices.jl:302-313).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

# model ids (include/cedar.h)
R, C, L, V, I, E, G, MOS1, DIODE, NLVCR = range(1, 11)
MODEL_NAMES = {R: "R", C: "C", L: "L", V: "V", I: "I", E: "E", G: "G", MOS1: "MOS1", DIODE: "DIODE", NLVCR: "NLVCR"}
NTERM = {R: 2, C: 2, L: 2, V: 2, I: 2, E: 4, G: 4, MOS1: 4, DIODE: 2, NLVCR: 3}
NPAR = {R: 2, C: 2, L: 2, V: 10, I: 10, E: 2, G: 2, MOS1: 7, DIODE: 4, NLVCR: 2}
HAS_BRANCH = {L, V, E}
# names of the built-in models' leading raw parameters, in device-table order
# (a source's waveform parameters after `dc` are set through its waveform)
PARAM_NAMES = {R: ["r", "m"], C: ["c", "m"], L: ["l", "m"], V: ["m", "dc"], I: ["m", "dc"], E: ["gain", "m"],
               G: ["gain", "m"], MOS1: ["type", "W", "L", "KP", "VTO", "LAMBDA", "m"], DIODE: ["IS", "N", "AREA", "m"],
               NLVCR: ["R", "m"]}
GROUND = {"0", "gnd", "GND", "ground"}

WAVE_DC, WAVE_PULSE, WAVE_PWL, WAVE_SIN = 0, 1, 2, 3
VA_BASE = 11   # CEDAR_NMODELS: ids of the compiled Verilog-A models start here


def model_nterm(model: int) -> int:
    if model >= VA_BASE:
        from . import va
        return va.model(model).nterm
    return NTERM[model]


def model_has_branch(model: int) -> bool:
    """A branch-current unknown: L, V, E and Verilog-A modules with a
    voltage-contributed branch."""
    if model >= VA_BASE:
        from . import va
        return bool(va.model(model).has_br)
    return model in HAS_BRANCH


def model_npar(model: int) -> int:
    if model >= VA_BASE:
        from . import va
        return va.model(model).npar
    return NPAR[model]


@dataclass
class Pulse:
    """SPICE PULSE(v1 v2 td tr tf pw per) (src/spectre_env.jl:153-166)."""
    v1: float
    v2: float
    td: float = 0.0
    tr: float = 0.0
    tf: float = 0.0
    pw: float = math.inf
    per: float = math.inf


@dataclass
class PWL:
    """Piecewise-linear source: sequence of (t, v) points (src/spectre_env.jl:144-150)."""
    points: Sequence[Tuple[float, float]]


@dataclass
class Sin:
    """SIN(vo va freq td theta phase ncycles) (src/spectre_env.jl:169-176)."""
    vo: float
    va: float
    freq: float
    td: float = 0.0
    theta: float = 0.0
    phase: float = 0.0
    ncycles: float = math.inf


def _pwl_at(ts, ys, t):
    i = 0
    while i < len(ts) and ts[i] <= t:
        i += 1
    if i <= 0:
        return ys[0]
    if i >= len(ts):
        return ys[-1]
    if ys[i - 1] == ys[i]:
        return ys[i]
    if ts[i] == ts[i - 1]:
        return (ys[i - 1] + ys[i]) / 2
    return ys[i - 1] + (t - ts[i - 1]) * (ys[i] - ys[i - 1]) / (ts[i] - ts[i - 1])


def wave_value(w, t: float) -> float:
    """Waveform value at time t (same rules as the kernels; used for dc defaults)."""
    if w is None:
        return 0.0
    if isinstance(w, (int, float)):
        return float(w)
    if isinstance(w, Pulse):
        ts = [w.td, w.td + w.tr, w.td + w.tr + w.pw, w.td + w.tr + w.pw + w.tf]
        ys = [w.v1, w.v2, w.v2, w.v1]
        return _pwl_at(ts, ys, math.fmod(t, w.per))
    if isinstance(w, PWL):
        return _pwl_at([p[0] for p in w.points], [p[1] for p in w.points], t)
    if isinstance(w, Sin):
        if w.td < t < w.ncycles / w.freq:
            return w.vo + w.va * math.exp(-(t - w.td) * w.theta) * math.sin(math.radians(360 * w.freq * (t - w.td) + w.phase))
        return w.vo + w.va * math.sin(math.radians(w.phase))
    raise TypeError(f"unknown waveform {w!r}")


@dataclass
class Device:
    name: str
    model: int
    terms: List[str]
    params: List[float]
    wave: object = None
    ac: float = 0.0          # AC magnitude of a V / I source (small-signal drive)


@dataclass
class Flat:
    """Flattened device table (numpy arrays; see include/cedar.h)."""
    n_nodes: int
    n_branch: int
    groups: List[Tuple[int, np.ndarray, Optional[np.ndarray], np.ndarray]]  # model, term[n,nt], branch[n], par[np,n]
    pwl: np.ndarray
    temp_c: float
    gmin: float
    names: List[str]                       # unknown names (nodes, then "<dev>.I" branches)
    devices: Dict[str, Tuple[int, int]]    # device name -> (group index, instance index)
    ordering: int = 0                      # LU ordering: 0 auto, 1 min degree, 2 nested dissection
    ac: Dict[str, float] = field(default_factory=dict)  # source name -> AC magnitude

    @property
    def n(self) -> int:
        return self.n_nodes + self.n_branch

    def index(self, name: str) -> int:
        return self.names.index(name)

    def param_block(self) -> np.ndarray:
        """Concatenated SoA parameter block (the per-instance block layout)."""
        return np.concatenate([g[3].ravel() for g in self.groups]) if self.groups else np.zeros(0)

    def param_offset(self, dev: str, k: int) -> int:
        """Offset of parameter k of device `dev` inside param_block()."""
        gi, ii = self.devices[dev]
        off = sum(g[3].size for g in self.groups[:gi])
        return off + k * self.groups[gi][3].shape[1] + ii


class Circuit:
    """Netlist builder mirroring CedarSim's device constructors."""

    def __init__(self, temp_c: float = 27.0, gmin: float = 1e-12):
        self.temp_c = temp_c
        self.gmin = gmin
        self.node_names: List[str] = []
        self._node_index: Dict[str, int] = {}
        self.devices: List[Device] = []
        self._names = set()

    # ---- nets
    def node(self, name: str) -> int:
        name = str(name)
        if name in GROUND:
            return -1
        if name not in self._node_index:
            self._node_index[name] = len(self.node_names)
            self.node_names.append(name)
        return self._node_index[name]

    def _add(self, name, model, terms, params, wave=None, ac=0.0):
        if name in self._names:
            raise ValueError(f"duplicate device name {name!r}")
        self._names.add(name)
        for t in terms:
            self.node(t)
        self.devices.append(Device(name, model, [str(t) for t in terms], [float(p) for p in params], wave, float(ac)))
        return self

    # ---- devices (CedarSim src/simpledevices.jl)
    def R(self, name, p, n, r=None, m=1.0, rsh=50.0, w=1e-6, l=1e-6, narrow=0.0, short=0.0):
        res = float(r) if r is not None else rsh * (l - short) / (w - narrow)
        return self._add(name, R, [p, n], [res, m])

    def C(self, name, p, n, c, m=1.0):
        return self._add(name, C, [p, n], [c, m])

    def L(self, name, p, n, l, m=1.0):
        return self._add(name, L, [p, n], [l, m])

    @staticmethod
    def _src_params(dc, wave, m):
        if wave is None:
            wave = dc if dc is not None else 0.0
        if dc is None:
            dc = wave_value(wave, 0.0)
        kind, a = WAVE_DC, [0.0] * 7
        if isinstance(wave, Pulse):
            kind, a = WAVE_PULSE, [wave.v1, wave.v2, wave.td, wave.tr, wave.tf, wave.pw, wave.per]
        elif isinstance(wave, PWL):
            kind = WAVE_PWL
        elif isinstance(wave, Sin):
            kind, a = WAVE_SIN, [wave.vo, wave.va, wave.freq, wave.td, wave.theta, wave.phase, wave.ncycles]
        elif not isinstance(wave, (int, float)):
            raise TypeError(f"unsupported waveform {wave!r}")
        return [m, dc, kind] + a, wave

    # `ac`: AC magnitude; like VoltageSource / CurrentSource (src/simpledevices.jl:
    # 279-300,320-339) only |ac| enters the small-signal drive (no phase)
    def V(self, name, p, n, dc=None, wave=None, m=1.0, ac=0.0):
        params, wave = self._src_params(dc, wave, m)
        return self._add(name, V, [p, n], params, wave, abs(ac))

    def I(self, name, p, n, dc=None, wave=None, m=1.0, ac=0.0):
        params, wave = self._src_params(dc, wave, m)
        return self._add(name, I, [p, n], params, wave, abs(ac))

    def E(self, name, p, n, cp, cn, gain, m=1.0):
        return self._add(name, E, [p, n, cp, cn], [gain, m])

    def G(self, name, p, n, cp, cn, gain, m=1.0):
        return self._add(name, G, [p, n, cp, cn], [gain, m])

    def mos1(self, name, d, g, s, b, type, W, L, KP, VTO, LAMBDA=0.0, m=1.0):
        return self._add(name, MOS1, [d, g, s, b], [type, W, L, KP, VTO, LAMBDA, m])

    def diode(self, name, a, c, IS=1e-14, N=1.0, AREA=1.0, m=1.0):
        return self._add(name, DIODE, [a, c], [IS, N, AREA, m])

    def nlvcr(self, name, d, g, s, R=1.0, m=1.0):
        return self._add(name, NLVCR, [d, g, s], [R, m])

    def va(self, name, model: str, terms: Sequence[str], m: float = 1.0, **params):
        """An instance of a compiled Verilog-A module (cedarsim.jl_gb300/va):
        terminals in port order, parameters by name (defaults from the module's
        declarations, ranges checked), multiplicity m.  The module's internal
        nodes become nodes named "<name>.<node>" placed after the ports in the
        device's terminal list."""
        from . import va
        mid = va.model_id(model)
        mod = va.model(mid)
        if len(terms) != len(mod.ports):
            raise ValueError(f"{model} has ports {mod.ports}, got {len(terms)} terminals")
        # internal nodes: one node unknown each, named "<instance>.<node>"
        inner = [f"{name}.{n}" for n in mod.internals]
        return self._add(name, mid, list(terms) + inner, mod.defaults(params) + [float(m)])

    # ---- parameter overrides by device name (the alter() of a netlist)
    def device(self, name: str) -> Device:
        for d in self.devices:
            if d.name == name:
                return d
        raise KeyError(f"no device named {name!r}")

    def set_param(self, dev: str, pname: str, value: float) -> "Circuit":
        """Set parameter `pname` of device `dev` (names as in PARAM_NAMES for the
        built-in models, the module's parameter names and `m` for Verilog-A
        models; setting a parameter a module queries with $param_given marks it
        given)."""
        d = self.device(dev)
        if d.model >= VA_BASE:
            from . import va
            mod = va.model(d.model)
            names = [p.name for p in mod.params]
            if pname == "m":
                d.params[-1] = float(value)
                return self
            if pname not in names:
                raise KeyError(f"{dev} ({mod.name}) has no parameter {pname!r}")
            vals = {n: d.params[k] for k, n in enumerate(names)}
            given = {g for j, g in enumerate(mod.given) if d.params[len(names) + j] != 0.0}
            vals[pname] = float(value)
            given.add(pname)
            new = mod.defaults({n: v for n, v in vals.items()})
            flags = [1.0 if g in given else 0.0 for g in mod.given]
            d.params = new[:len(names)] + flags + [d.params[-1]]
            return self
        names = PARAM_NAMES[d.model]
        if pname not in names:
            raise KeyError(f"{dev} has no parameter {pname!r} (parameters {names})")
        d.params[names.index(pname)] = float(value)
        if d.model in (V, I) and pname == "dc" and isinstance(d.wave, (int, float)):
            d.wave = float(value)       # a DC source: its transient value is its dc value
        return self

    def altered(self, params) -> "Circuit":
        """A copy with parameters set from {"DEV.param": value} (None keeps the value)."""
        import copy
        c = copy.deepcopy(self)
        for key, v in (params.items() if isinstance(params, dict) else params):
            if v is None:
                continue
            dev, _, pname = str(key).rpartition(".")
            if not dev:
                raise KeyError(f"{key!r}: expected DEVICE.parameter")
            c.set_param(dev, pname, v)
        return c

    # ---- flattening
    def flatten(self) -> Flat:
        n_nodes = len(self.node_names)
        names = list(self.node_names)
        branch_of: Dict[str, int] = {}
        for d in self.devices:
            if model_has_branch(d.model):
                branch_of[d.name] = n_nodes + len(branch_of)
                names.append(f"{d.name}.I")
        pwl: List[float] = []
        groups = []
        devices: Dict[str, Tuple[int, int]] = {}
        for model in sorted({d.model for d in self.devices}):
            devs = [d for d in self.devices if d.model == model]
            nt, npar = model_nterm(model), model_npar(model)
            term = np.array([[self._node_index.get(t, -1) if t not in GROUND else -1 for t in d.terms] for d in devs],
                            dtype=np.int32).reshape(len(devs), nt)
            br = np.array([branch_of[d.name] for d in devs], dtype=np.int32) if model_has_branch(model) else None
            par = np.zeros((npar, len(devs)), dtype=np.float64)
            for i, d in enumerate(devs):
                p = list(d.params)
                if model in (V, I) and isinstance(d.wave, PWL):
                    p[3] = float(len(pwl))
                    p[4] = float(len(d.wave.points))
                    for (tt, vv) in d.wave.points:
                        pwl.extend([float(tt), float(vv)])
                par[:, i] = p
                devices[d.name] = (len(groups), i)
            groups.append((model, np.ascontiguousarray(term), br, np.ascontiguousarray(par)))
        return Flat(n_nodes, len(branch_of), groups, np.array(pwl, dtype=np.float64), self.temp_c, self.gmin,
                    names, devices, ac={d.name: d.ac for d in self.devices if d.ac})
