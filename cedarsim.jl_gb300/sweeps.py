"""Parameter sweeps and their batched execution on the GPU.

Sweep specifications follow CedarSim's sweep API (src/sweeps.jl):

  Sweep(selector, values)          1-D sweep of one parameter        src/sweeps.jl:145-216
  ProductSweep(*args, **kw)        cartesian product, first axis fastest
                                                                     src/sweeps.jl:225-240
  TandemSweep(*args, **kw)         zipped sweeps of equal length     src/sweeps.jl:242-264
  SerialSweep(*args, **kw)         one after another, unset = None   src/sweeps.jl:266-312
  sweepvars, split_axes, sweepify, find_param_ranges
                                                  src/sweeps.jl:202-206,85-131,314-328,505-546
  nest_param_list / flatten_param_list            src/circuitodesystem.jl:101-145
  alter(x, params)                                src/sweeps.jl:8-38
  ParamSim(circuit, **params)                     a circuit with parameter overrides
  CircuitSweep(circuit, sweep)                    src/sweeps.jl:330-435

Every point of a sweep is a tuple of (name, value) pairs sorted by name (the
SweepFlattener's `expand`, src/sweeps.jl:133-140).  Shapes are column-major as in
Julia: the first axis of a product varies fastest.

`dc(cs)` and `tran(cs, tspan)` over a CircuitSweep are the broadcasts `dc!.` and
`tran!.` (src/sweeps.jl:471-502): every point is built and flattened on the host,
points are grouped by topology into templates, and all of them run in one
batched GPU launch (`Batch`).  Results come back shaped like the sweep.
"""
from __future__ import annotations

import csv
import dataclasses
import itertools
from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np

Point = Tuple[Tuple[str, Any], ...]


# ------------------------------------------------------------------ sweep specs
def _values(values) -> list:
    if isinstance(values, (str, bytes)):
        raise TypeError("sweep values must be numbers, not a string")
    if isinstance(values, np.ndarray):
        return values.ravel().tolist()
    if isinstance(values, (int, float, np.number)) or values is None:
        return [values.item() if isinstance(values, np.number) else values]
    return list(values)


class Sweep:
    """1-D sweep over one circuit property: Sweep("R1", vals), Sweep(("R1", vals)),
    Sweep(R1=vals).  A dotted selector ("a.b") reaches into nested parameters."""

    def __init__(self, selector=None, values=None, **kwargs):
        if selector is None:
            if len(kwargs) != 1:
                raise ValueError("`Sweep` takes a single variable at a time!")
            (selector, values), = kwargs.items()
        elif values is None and isinstance(selector, tuple) and len(selector) == 2:
            selector, values = selector
        elif kwargs:
            raise ValueError("`Sweep` takes a single variable at a time!")
        self.selector = str(selector)
        self.values = _values(values)

    def __iter__(self):
        for v in self.values:
            yield ((self.selector, v),)

    def __len__(self) -> int:
        return len(self.values)

    @property
    def shape(self) -> Tuple[int, ...]:
        return (len(self.values),)

    def size(self, d: Optional[int] = None):
        return _size(self.shape, d)

    def sweepvars(self) -> set:
        return {self.selector}

    def __eq__(self, other) -> bool:
        return isinstance(other, Sweep) and self.selector == other.selector and self.values == other.values

    def __repr__(self) -> str:
        if len(self.values) > 1:
            return (f"Sweep of {self.selector} with {len(self.values)} values over "
                    f"[{min(self.values)} .. {max(self.values)}]")
        return f"Sweep of {self.selector} set to {self.values[0] if self.values else None}"


def _size(shape: Tuple[int, ...], d: Optional[int]):
    if d is None:
        return shape
    return shape[d - 1] if 1 <= d <= len(shape) else 1


def _as_sweep(x):
    if isinstance(x, (Sweep, _Combined)):
        return x
    return Sweep(x)


def _expand(items) -> Point:
    """Flatten nested point tuples and sort by name (src/sweeps.jl:133-140)."""
    out: List[Tuple[str, Any]] = []

    def rec(v):
        if isinstance(v, tuple) and len(v) == 2 and isinstance(v[0], str):
            out.append(v)
        else:
            for e in v:
                rec(e)
    rec(items)
    return tuple(sorted(out, key=lambda kv: kv[0]))


class _Combined:
    """A product, tandem or serial combination of sweeps (the SweepFlattener)."""

    def __init__(self, kind: str, children: Sequence):
        self.kind = kind
        self.children = list(children)
        if kind == "serial":
            self.vars = sweepvars(*self.children)

    # iteration ------------------------------------------------------------
    def __iter__(self):
        if self.kind == "product":
            if not self.children:
                yield ()
                return
            # first child fastest: iterate the reversed product
            for combo in itertools.product(*[list(c) for c in reversed(self.children)]):
                yield _expand(tuple(reversed(combo)))
        elif self.kind == "tandem":
            for combo in zip(*self.children):
                yield _expand(combo)
        else:
            names = sorted(self.vars)
            for c in self.children:
                for p in c:
                    m = dict.fromkeys(names)
                    m.update(dict(_expand(p)))
                    yield tuple((k, m[k]) for k in names)

    def __len__(self) -> int:
        if self.kind == "product":
            return int(np.prod([len(c) for c in self.children])) if self.children else 1
        if self.kind == "tandem":
            return len(self.children[0])
        return sum(len(c) for c in self.children)

    @property
    def shape(self) -> Tuple[int, ...]:
        if self.kind == "product":
            return tuple(s for c in self.children for s in c.shape)
        return (len(self),)

    def size(self, d: Optional[int] = None):
        return _size(self.shape, d)

    def sweepvars(self) -> set:
        return sweepvars(*self.children)

    def __repr__(self) -> str:
        head = {"product": "Product", "tandem": "Tandem", "serial": "Serial"}[self.kind]
        lines = [f"{head} sweep of:"] + ["  - " + repr(c).replace("\n", "\n    ") for c in self.children]
        return "\n".join(lines)


def ProductSweep(*args, **kwargs):
    """Cartesian product of the given sweeps: ProductSweep(R1=1:4, R2=1:4)."""
    items = [_as_sweep(a) for a in args] + [Sweep(k, v) for k, v in kwargs.items()]
    if len(items) == 1:
        return items[0]
    return _Combined("product", items)


def TandemSweep(*args, **kwargs):
    """Sweeps stepped together; all must have the same length."""
    items = [_as_sweep(a) for a in args] + [Sweep(k, v) for k, v in kwargs.items()]
    if len(items) == 1:
        return items[0]
    if len({len(i) for i in items}) > 1:
        raise ValueError("TandemSweep requires all sweeps be of the same length!")
    return _Combined("tandem", items)


def SerialSweep(*args, **kwargs):
    """Sweeps one after another; the variables of the others are None (default)."""
    items = [_as_sweep(a) for a in args] + [Sweep(k, v) for k, v in kwargs.items()]
    if len(items) == 1:
        return items[0]
    return _Combined("serial", items)


def sweepvars(*sweeps) -> set:
    """Every variable the given sweeps set."""
    out: set = set()
    for s in sweeps:
        out |= s.sweepvars()
    return out


def split_axes(sweep, axes) -> Tuple[Any, Any]:
    """Split a ProductSweep into (outer, inner) products, inner over `axes`."""
    if not (isinstance(sweep, _Combined) and sweep.kind == "product"):
        raise ValueError("split_axes only works with ProductSweep objects!")
    names = [getattr(c, "selector", None) for c in sweep.children]
    idx = []
    axes = sorted(axes, key=lambda a: names.index(a) if a in names else -1) if isinstance(axes, (set, frozenset)) \
        else list(axes)
    for a in axes:
        if a not in names:
            raise ValueError(f"Unable to find product axis matching '{a}'")
        idx.append(names.index(a))
    inner = _Combined("product", [sweep.children[i] for i in idx])
    outer = _Combined("product", [c for i, c in enumerate(sweep.children) if i not in idx])
    return outer, inner


def sweepify(x):
    """Shorthands to sweeps: a list -> SerialSweep, a dict -> ProductSweep,
    a (name, values) pair -> Sweep."""
    if isinstance(x, (Sweep, _Combined)):
        return x
    if isinstance(x, list):
        return SerialSweep(*[sweepify(e) for e in x])
    if isinstance(x, dict):
        return ProductSweep(**x)
    return Sweep(x)


def find_param_ranges(sweep) -> Dict[str, Tuple[Any, Any, int]]:
    """(min, max, number of values) explored per variable, over all sub-sweeps."""
    acc: Dict[str, list] = {}

    def rec(s):
        if isinstance(s, Sweep):
            acc.setdefault(s.selector, []).append((min(s.values), max(s.values), len(s.values)))
        else:
            for c in s.children:
                rec(c)
    rec(sweep)
    out = {}
    for k, rs in acc.items():
        lo, hi, n = rs[0]
        for a, b, m in rs[1:]:
            lo, hi, n = min(lo, a), max(hi, b), n + m
        out[k] = (lo, hi, n)
    return out


def grid(sweep) -> np.ndarray:
    """All points as an object array shaped like the sweep (column-major)."""
    pts = list(sweep)
    a = np.empty(len(pts), dtype=object)
    for i, p in enumerate(pts):
        a[i] = p
    return a.reshape(sweep.shape, order="F") if sweep.shape else a.reshape(())


# ------------------------------------------------------------- parameter lists
def nest_param_list(x) -> dict:
    """Dotted names to nested dicts; None becomes an empty dict.  Assigning a key
    twice, or a key and one of its prefixes, is an error."""
    items = x.items() if isinstance(x, dict) else x
    by_prefix: Dict[str, list] = {}
    plain: Dict[str, Any] = {}
    for k, v in items:
        k = str(k)
        if v is None:
            v = {}
        if "." in k:
            pre, tail = k.split(".", 1)
            by_prefix.setdefault(pre, []).append((tail, v))
        else:
            if k in plain:
                raise ValueError(f"Cannot double-assign a key: {k}")
            plain[k] = v
    clobbered = set(by_prefix) & set(plain)
    if clobbered:
        raise ValueError(f"Cannot assign to a prefix of another key: {sorted(clobbered)}")
    for pre, subs in by_prefix.items():
        plain[pre] = nest_param_list(subs)
    return plain


def flatten_param_list(x, prefix: str = "") -> Tuple[Tuple[str, Any], ...]:
    """Nested dicts to sorted (dotted name, value) pairs."""
    out: List[Tuple[str, Any]] = []

    def rec(d, pre):
        for k, v in d.items():
            name = f"{pre}.{k}" if pre else str(k)
            if isinstance(v, dict):
                rec(v, name)
            else:
                out.append((name, v))
    rec(x, prefix)
    return tuple(sorted(out, key=lambda kv: kv[0]))


def _get(x, k):
    return x[k] if isinstance(x, dict) else getattr(x, k)


def _set(x, k, v):
    if isinstance(x, dict):
        y = dict(x)
        y[k] = v
        return y
    if dataclasses.is_dataclass(x):
        return dataclasses.replace(x, **{k: v})
    y = type(x).__new__(type(x))
    y.__dict__.update(x.__dict__)
    setattr(y, k, v)
    return y


def alter(x, params):
    """Copy of x (dict, dataclass or plain object) with dotted-path fields set;
    a None value means "keep the default"."""
    items = params.items() if isinstance(params, dict) else params
    for sel, val in items:
        if val is None:
            continue
        path = str(sel).split(".")

        def rec(obj, i):
            cur = _get(obj, path[i])
            if i == len(path) - 1:
                v = float(val) if isinstance(cur, float) and isinstance(val, (int, float, np.number)) else val
                return _set(obj, path[i], v)
            return _set(obj, path[i], rec(cur, i + 1))
        x = rec(x, 0)
    return x


class Params(dict):
    """Nested parameter dict with attribute access (`sim.params.x1.r_load`)."""

    def __getattr__(self, k):
        try:
            v = self[k]
        except KeyError as e:
            raise AttributeError(k) from e
        return Params(v) if isinstance(v, dict) and not isinstance(v, Params) else v


class ParamSim:
    """A circuit with parameter overrides.  `circuit` is a function
    `f(**params) -> Circuit` (dotted names arrive as nested dicts), a class whose
    default instance is altered and then called to build the Circuit, or a built
    Circuit whose devices are altered by "DEVICE.parameter" names."""

    def __init__(self, circuit, **params):
        self.circuit = circuit
        self.params = Params(nest_param_list({k: v for k, v in params.items() if v is not None}))
        self._flat_params = tuple((k, v) for k, v in params.items() if v is not None)

    def build(self):
        c = self.circuit
        if hasattr(c, "altered") and hasattr(c, "flatten"):
            # a built netlist: "DEVICE.parameter" names alter its devices
            return c.altered(self._flat_params)
        if isinstance(c, type):
            return alter(c(), self._flat_params)()
        return c(**self.params)

    def __repr__(self) -> str:
        return f"ParamSim({getattr(self.circuit, '__name__', self.circuit)}, {dict(self._flat_params)})"


class CircuitSweep:
    """A circuit and a sweep over its parameters; iterating yields ParamSim points."""

    def __init__(self, circuit, sweep):
        if not hasattr(sweep, "__iter__"):
            raise TypeError("Must give some kind of iterator!")
        self.circuit = circuit
        self.iterator = sweep

    def __iter__(self):
        for p in self.iterator:
            yield ParamSim(self.circuit, **dict(p))

    def __len__(self) -> int:
        return len(self.iterator)

    @property
    def shape(self) -> Tuple[int, ...]:
        return self.iterator.shape

    def size(self, d: Optional[int] = None):
        return _size(self.shape, d)

    def sweepvars(self) -> set:
        return self.iterator.sweepvars()

    def collect(self) -> np.ndarray:
        sims = list(self)
        a = np.empty(len(sims), dtype=object)
        for i, s in enumerate(sims):
            a[i] = s
        return a.reshape(self.shape, order="F") if self.shape else a.reshape(())


# ------------------------------------------------------ batched dc! / tran!
def topology_key(flat) -> tuple:
    """Everything of a flattened circuit except its parameter values: points
    with equal keys share one batch template."""
    groups = tuple((int(m), t.tobytes(), None if b is None else b.tobytes(), p.shape) for m, t, b, p in flat.groups)
    return (flat.n_nodes, flat.n_branch, groups, np.asarray(flat.pwl).tobytes(), float(flat.temp_c),
            float(flat.gmin), tuple(flat.names), int(flat.ordering))


def batch_tables(flats: Sequence) -> Tuple[list, np.ndarray, np.ndarray, np.ndarray]:
    """Group flattened points into templates and per-instance parameter blocks:
    (templates, inst_template[n], inst_par, inst_par_off[n])."""
    keys: Dict[tuple, int] = {}
    templates = []
    itpl = np.zeros(len(flats), np.int32)
    off = np.zeros(len(flats), np.int64)
    blocks = []
    pos = 0
    for i, f in enumerate(flats):
        k = topology_key(f)
        if k not in keys:
            keys[k] = len(templates)
            templates.append(f)
        itpl[i] = keys[k]
        b = f.param_block()
        blocks.append(b)
        off[i] = pos
        pos += b.size
    par = np.concatenate(blocks) if blocks else np.zeros(0)
    return templates, itpl, par, off


@dataclasses.dataclass
class PointSolution:
    """DC or sampled transient solution of one sweep point."""
    params: Params
    names: list
    x: Optional[np.ndarray] = None     # DC operating point (original unknown order)
    t: Optional[np.ndarray] = None     # transient sample times
    u: Optional[np.ndarray] = None     # transient samples [n_samples, n_probes]
    stats: Optional[dict] = None
    retcode: str = "OK"

    def __getitem__(self, name: str):
        i = self.names.index(name)
        return self.x[i] if self.u is None else self.u[:, i]


def _shape_like(cs: CircuitSweep, items: list) -> np.ndarray:
    a = np.empty(len(items), dtype=object)
    for i, s in enumerate(items):
        a[i] = s
    return a.reshape(cs.shape, order="F") if cs.shape else a.reshape(())


def _stats(st) -> dict:
    return {k: st[k].item() for k in st.dtype.names if k != "pad"}


def sweep_dc(cs: CircuitSweep, reltol: float = 1e-6, abstol_v: float = 1e-9, batch_kw: Optional[dict] = None,
             **kw) -> np.ndarray:
    """dc!.(cs): the DC operating point of every sweep point in one batched launch."""
    from .abi import STATUS_NAMES
    from .api import Batch
    sims = list(cs)
    flats = [s.build().flatten() for s in sims]
    templates, itpl, par, off = batch_tables(flats)
    b = Batch(templates, itpl, par, off, **(batch_kw or {}))
    x, st = b.dc(reltol=reltol, abstol_v=abstol_v, **kw)
    out = []
    for i, (s, f) in enumerate(zip(sims, flats)):
        out.append(PointSolution(s.params, list(f.names), x=x[i, :f.n].copy(), stats=_stats(st[i]),
                                 retcode=STATUS_NAMES[int(st[i]["status"])]))
    return _shape_like(cs, out)


def sweep_tran(cs: CircuitSweep, tspan: Tuple[float, float], probes: Optional[Sequence[str]] = None,
               n_samples: int = 101, method: str = "bdf2", reltol: float = 1e-6, abstol_v: float = 1e-9,
               dcop: bool = True, **kw) -> np.ndarray:
    """tran!.(cs, tspan): every sweep point's transient in one batched launch.
    `probes` (unknown names, default every node voltage of the first point) are
    sampled on a uniform grid of n_samples points over tspan."""
    from .abi import STATUS_NAMES
    from .api import Batch
    sims = list(cs)
    flats = [s.build().flatten() for s in sims]
    templates, itpl, par, off = batch_tables(flats)
    if probes is None:
        probes = list(flats[0].names[:flats[0].n_nodes]) if flats else []
    probes = list(probes)
    pidx = np.array([[t.names.index(p) if p in t.names else -1 for p in probes] for t in templates], np.int32)
    b = Batch(templates, itpl, par, off, probes=pidx if probes else None, n_samples=n_samples if probes else 0)
    r = b.tran(tspan, method=method, reltol=reltol, abstol_v=abstol_v, dcop=dcop, **kw)
    tgrid = np.linspace(tspan[0], tspan[1], n_samples)
    out = []
    for i, s in enumerate(sims):
        u = r.samples[i].T.copy() if r.samples is not None else np.zeros((n_samples, 0))
        out.append(PointSolution(s.params, probes, t=tgrid, u=u, x=r.x_final[i, :flats[i].n].copy(),
                                 stats=_stats(r.stats[i]), retcode=STATUS_NAMES[int(r.stats[i]["status"])]))
    return _shape_like(cs, out)


# ------------------------------------------------------------------ CSV export
def default_name_map(names: Sequence[str], n_nodes: Optional[int] = None) -> Dict[str, str]:
    """Top-level node voltages, a leading `node_` stripped when that does not
    clash, ground names left out (src/util.jl:239-262)."""
    cand = list(names if n_nodes is None else names[:n_nodes])
    cand = [n for n in cand if "." not in n]
    top = set(cand)
    out = {}
    for n in cand:
        s = n[5:] if n.startswith("node_") and n[5:] not in top else n
        if s in ("0", "gnd", "GND", "node_0", "node_gnd", "node_GND"):
            continue
        out[n] = s
    return out


def write_csv(path: str, sol, name_map: Optional[Dict[str, str]] = None) -> str:
    """Write a transient solution as CSV: column `t`, then one column per mapped
    unknown (CSV.write(file, sol; name_map), ext/CedarSimCSVExt.jl:13-19)."""
    names = list(sol.names)
    if name_map is None:
        n_nodes = getattr(sol, "n_nodes", None)
        name_map = default_name_map(names, n_nodes)
    cols = [(label, sol[key]) for key, label in name_map.items()]
    with open(path, "w", newline="") as fh:
        w = csv.writer(fh)
        w.writerow(["t"] + [c[0] for c in cols])
        for i, t in enumerate(sol.t):
            w.writerow([repr(float(t))] + [repr(float(c[1][i])) for c in cols])
    return path
