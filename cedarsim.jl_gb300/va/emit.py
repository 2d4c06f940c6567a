"""Verilog-A to CUDA/C++ device-code emitter.

For every module the emitter writes
  * body_<m><D>(P, ps, ctx, V, Fi, Fq): the analog block over dual numbers D
    (cedar::va::Dual, csrc/va_dual.cuh), accumulating each port's KCL residual
    from I(a,b) <+ contributions: the resistive part into Fi, the ddt() part (a
    charge) into Fq.  A branch current flowing a -> b adds -I to KCL(a) and +I to
    KCL(b) (src/simulate_ir.jl:54,112-120, contribution lowering of
    src/vasim.jl:128-180);
  * eval_<m>(...): the per-device outputs the GPU engine stamps, only for the
    structurally nonzero Jacobian entries found by a dependency analysis;
  * full_<m>(...): dense residuals and Jacobians of one device (the oracle's
    entry point);
  * dispatch functions over the model index and a stamp table for the host
    compiler.
Parameters are the module's parameters in declaration order followed by the
multiplicity m; the derived block appends the thermal voltage.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, FrozenSet, List, Optional, Set, Tuple

from .parser import (LOOP_CAP, Assign, Bin, Call, Cond, Contrib, If, Loop, Module, Name, Num, Param, Probe,
                     SysCall, Unary, VAError)

# terminal values per device (ports + internal nodes + a branch current) the
# engines can stage; above the built-ins' 5 the generated header widens the
# engines' staging (CEDAR_MAX_TERM) for the library built with such a model
MAX_PORTS = 8
BUILTIN_TERMS = 5

FUNCS = {  # VA name -> (C++ name, arity)
    "exp": ("exp", 1), "ln": ("log", 1), "log": ("log10", 1), "sqrt": ("sqrt", 1), "pow": ("pow", 2),
    "abs": ("fabs", 1), "min": ("vmin", 2), "max": ("vmax", 2), "tanh": ("tanh", 1), "sinh": ("sinh", 1),
    "cosh": ("cosh", 1), "sin": ("sin", 1), "cos": ("cos", 1), "tan": ("tan", 1), "atan": ("atan", 1),
    "atan2": ("atan2", 2), "asin": ("asin", 1), "acos": ("acos", 1), "hypot": ("hypot", 2),
    "floor": ("floor", 1), "ceil": ("ceil", 1), "limexp": ("limexp", 1),
}
P_Q, P_K = 1.602176634e-19, 1.380649e-23


@dataclasses.dataclass
class VAModel:
    name: str
    module: Module
    ports: List[str]
    params: List[Param]
    second_order: bool
    frows: List[int]
    gents: List[Tuple[int, int]]
    qrows: List[int]
    cents: List[Tuple[int, int]]
    flops: int
    given: List[str] = dataclasses.field(default_factory=list)   # parameters queried by $param_given
    vbranch: Optional[Tuple[str, Optional[str]]] = None  # the voltage-contributed branch (a, b), if any
    noise: List[Tuple[int, int]] = dataclasses.field(default_factory=list)  # noise sources: (a, b or -1)

    @property
    def internals(self) -> List[str]:
        return list(self.module.internals)

    @property
    def nterm(self) -> int:         # device-table terminals: ports, then internal nodes
        return len(self.ports) + len(self.module.internals)

    @property
    def has_br(self) -> int:        # a branch-current unknown (after the terminals)
        return 1 if self.vbranch is not None else 0

    @property
    def nx(self) -> int:            # dual-number seeds: terminals, then the branch current
        return self.nterm + self.has_br

    @property
    def npar(self) -> int:          # raw: parameters, $param_given flags, m
        return len(self.params) + len(self.given) + 1

    @property
    def ndpar(self) -> int:         # derived: raw + vt
        return self.npar + 1

    @property
    def nout(self) -> int:
        return len(self.frows) + len(self.gents) + len(self.qrows) + len(self.cents)

    def param_index(self, name: str) -> int:
        for k, p in enumerate(self.params):
            if p.name == name:
                return k
        raise KeyError(name)

    def defaults(self, overrides: Optional[Dict[str, float]] = None) -> List[float]:
        """Parameter values with defaults evaluated in declaration order (a default
        may use earlier parameters); integer parameters rounded half away from zero."""
        overrides = dict(overrides or {})
        known = {p.name for p in self.params}
        bad = set(overrides) - known
        if bad:
            raise VAError(f"{self.name}: unknown parameters {sorted(bad)}")
        env: Dict[str, float] = {}
        for p in self.params:
            v = float(overrides[p.name]) if p.name in overrides else float(const_eval(p.default, env))
            if p.type == "integer":
                v = float(math.floor(abs(v) + 0.5) * (1 if v >= 0 else -1))
            check_range(self.name, p, v, env)
            env[p.name] = v
        # $param_given(P) flags: 1 where the instance sets P
        return [env[p.name] for p in self.params] + [1.0 if g in overrides else 0.0 for g in self.given]


# ------------------------------------------------------------ host evaluation
def const_eval(e, env: Dict[str, float]) -> float:
    """Evaluate a parameter expression (numbers, earlier parameters, arithmetic,
    the math functions) on the host."""
    if isinstance(e, Num):
        return e.v
    if isinstance(e, Name):
        if e.id not in env:
            raise VAError(f"line {e.line}: {e.id!r} is not a parameter defined before its use")
        return env[e.id]
    if isinstance(e, Unary):
        x = const_eval(e.x, env)
        return -x if e.op == "-" else float(x == 0.0)
    if isinstance(e, Bin):
        a, b = const_eval(e.a, env), const_eval(e.b, env)
        ops = {"+": lambda: a + b, "-": lambda: a - b, "*": lambda: a * b,
               "/": lambda: (math.trunc(a / b) if _is_int_const(e.a) and _is_int_const(e.b) else a / b),
               "**": lambda: a ** b, "<": lambda: float(a < b), ">": lambda: float(a > b),
               "<=": lambda: float(a <= b), ">=": lambda: float(a >= b), "==": lambda: float(a == b),
               "!=": lambda: float(a != b), "&&": lambda: float(a != 0 and b != 0),
               "||": lambda: float(a != 0 or b != 0)}
        return float(ops[e.op]())
    if isinstance(e, Cond):
        return const_eval(e.a, env) if const_eval(e.c, env) != 0 else const_eval(e.b, env)
    if isinstance(e, Call) and e.fn in FUNCS:
        args = [const_eval(a, env) for a in e.args]
        py = {"exp": math.exp, "ln": math.log, "log": math.log10, "sqrt": math.sqrt, "pow": math.pow,
              "abs": abs, "min": min, "max": max, "tanh": math.tanh, "sinh": math.sinh, "cosh": math.cosh,
              "sin": math.sin, "cos": math.cos, "tan": math.tan, "atan": math.atan, "atan2": math.atan2,
              "asin": math.asin, "acos": math.acos, "hypot": math.hypot, "floor": math.floor, "ceil": math.ceil,
              "limexp": math.exp}[e.fn]
        return float(py(*args))
    raise VAError(f"unsupported expression in a parameter default: {e}")


def _is_int_const(e) -> bool:
    return isinstance(e, Num) and e.is_int


def _at(v: float, bound: float) -> bool:
    """v equals a bound up to the rounding of the bound's own expression: a
    scale-factor literal is the decimal times the factor (0.1n is 0.1 * 1e-9 =
    1.0000000000000001e-10, as the reference converts it, src/vasim.jl:114-126),
    so a card value written 1e-10 meets the inclusive bound [0.1n:."""
    return v == bound or (math.isfinite(bound) and abs(v - bound) <= 4 * math.ulp(max(abs(v), abs(bound))))


def check_range(model: str, p: Param, v: float, env: Dict[str, float]):
    """`from` / `exclude` ranges of a parameter declaration."""
    for r in p.ranges:
        if len(r) == 2:
            kind, x = r
            inside = _at(v, const_eval(x, env))
        else:
            kind, lo, hi, li, hi_i = r
            lo_v = -math.inf if _is_inf(lo) else const_eval(lo, env)
            hi_v = math.inf if _is_inf(hi) else const_eval(hi, env)
            inside = (v > lo_v or (li and _at(v, lo_v))) and (v < hi_v or (hi_i and _at(v, hi_v)))
        if (kind == "from" and not inside) or (kind == "exclude" and inside):
            raise VAError(f"{model}: parameter {p.name} = {v} violates its `{kind}` range")


def _is_inf(e) -> bool:
    return isinstance(e, Name) and e.id == "inf" or (isinstance(e, Unary) and _is_inf(e.x))


# ------------------------------------------------------------------ analysis
class _Analysis:
    def __init__(self, mod: Module):
        self.mod = mod
        self.port = {p: k for k, p in enumerate(list(mod.ports) + list(mod.internals))}
        self.params = {p.name for p in mod.params}
        self.vars = dict(mod.variables)
        self.var_deps: Dict[str, FrozenSet[int]] = {v: frozenset() for v in self.vars}
        self.second_order = False
        self.funcs = dict(mod.functions)
        self.vbranch = None            # (a, b) of the voltage-contributed branch
        self.nb = None                 # its seed index (after the terminals)
        self._find_vbranch(mod.body)
        if self.vbranch is not None:
            self.nb = len(self.port)
        self.given: List[str] = []          # parameters queried by $param_given, in order of use
        self.noise: List[Tuple[int, int]] = []
        self.noise_index: Dict[int, int] = {}
        self.contribs: List[Tuple[Contrib, Optional[object], List[Tuple[int, object]]]] = []

    def _find_vbranch(self, stmts):
        for s in stmts:
            if isinstance(s, Loop):
                self._find_vbranch(s.body)
            if isinstance(s, If):
                self._find_vbranch(s.then)
                self._find_vbranch(s.other)
            elif isinstance(s, Contrib) and s.kind == "V":
                br = (s.a, s.b)
                if self.vbranch is None:
                    self.vbranch = br
                elif br != self.vbranch and (br[1], br[0]) != self.vbranch:
                    raise VAError(f"{self.mod.name}: line {s.line}: a second voltage-contributed branch "
                                  f"(only one per module)")

    def branch_sign(self, a: str, b: Optional[str], line: int) -> int:
        """+1 / -1 when (a, b) is the voltage branch in its own / the reverse orientation."""
        if self.vbranch is not None:
            if (a, b) == self.vbranch:
                return 1
            if b is not None and (b, a) == self.vbranch:
                return -1
        raise VAError(f"{self.mod.name}: line {line}: I({a}{', ' + b if b else ''}) probes no voltage-contributed branch")

    def port_index(self, n: str, line: int) -> int:
        if n not in self.port:
            raise VAError(f"{self.mod.name}: line {line}: {n!r} is not a port")
        return self.port[n]

    def deps(self, e) -> FrozenSet[int]:
        if isinstance(e, SysCall):
            if e.name in ("$param_given", "$given"):
                if len(e.args) != 1 or not isinstance(e.args[0], Name) or e.args[0].id not in self.params:
                    raise VAError(f"{self.mod.name}: $param_given takes a parameter name")
                if e.args[0].id not in self.given:
                    self.given.append(e.args[0].id)
            return frozenset()
        if isinstance(e, Num):
            return frozenset()
        if isinstance(e, Name):
            if e.id in self.params:
                return frozenset()
            if e.id in self.vars:
                return self.var_deps[e.id]
            raise VAError(f"{self.mod.name}: line {e.line}: undeclared name {e.id!r}")
        if isinstance(e, Probe):
            if e.kind == "I":
                self.branch_sign(e.a, e.b, 0)
                return frozenset({self.nb})
            s = {self.port_index(e.a, 0)}
            if e.b is not None:
                s.add(self.port_index(e.b, 0))
            return frozenset(s)
        if isinstance(e, Unary):
            d = self.deps(e.x)       # (visited either way: names, $param_given)
            return d if e.op == "-" else frozenset()
        if isinstance(e, Bin):
            d = self.deps(e.a) | self.deps(e.b)
            if e.op in ("+", "-", "*", "/", "**"):
                return d
            return frozenset()       # comparisons and logic are piecewise constant
        if isinstance(e, Cond):
            self.deps(e.c)
            return self.deps(e.a) | self.deps(e.b)
        if isinstance(e, Call):
            if e.fn == "ddx":
                self.second_order = True
                return self.deps(e.args[0])
            if e.fn in ("white_noise", "flicker_noise"):
                return frozenset()       # noise sources: zero outside a noise analysis
            if e.fn == "ddt":
                return self.deps(e.args[0])
            if e.fn in ("floor", "ceil"):
                return frozenset()
            out = frozenset()
            for a in e.args:
                out |= self.deps(a)
            f = self.funcs.get(e.fn)
            if f is not None and f.outputs:
                # output arguments receive values computed from every argument
                for j, an in enumerate(f.inputs):
                    if an not in f.outputs:
                        continue
                    if j >= len(e.args) or not isinstance(e.args[j], Name) or e.args[j].id not in self.vars:
                        raise VAError(f"{self.mod.name}: line {e.line}: output argument {an} of {e.fn}() must be "
                                      f"a variable")
                    v = e.args[j].id
                    if self.vars[v] == "real":
                        self.var_deps[v] = self.var_deps[v] | out
            return out
        raise VAError(f"{self.mod.name}: unsupported expression {e!r}")

    def collect_noise(self, stmts):
        """white_noise(pwr) and flicker_noise(pwr, ex) terms of current
        contributions: noise current sources across the contribution's branch,
        numbered in source order."""
        def calls(e, out):
            if isinstance(e, Call):
                if e.fn in ("white_noise", "flicker_noise"):
                    out.append(e)
                for a in e.args:
                    calls(a, out)
            elif isinstance(e, Unary):
                calls(e.x, out)
            elif isinstance(e, Bin):
                calls(e.a, out)
                calls(e.b, out)
            elif isinstance(e, Cond):
                calls(e.c, out)
                calls(e.a, out)
                calls(e.b, out)
        for s in stmts:
            if isinstance(s, Loop):
                found = []
                for x in _all_stmts(s.body):
                    if isinstance(x, Contrib):
                        calls(x.expr, found)
                if found:
                    raise VAError(f"{self.mod.name}: {found[0].fn}() inside a loop")
            if isinstance(s, If):
                self.collect_noise(s.then)
                self.collect_noise(s.other)
            elif isinstance(s, Contrib) and s.kind == "I":
                found = []
                calls(s.expr, found)
                for c in found:
                    self.noise_index[id(c)] = len(self.noise)
                    self.noise.append((self.port[s.a], self.port[s.b] if s.b is not None else -1))

    def walk(self, stmts, collect: bool):
        for s in stmts:
            if isinstance(s, Assign):
                if s.name in self.params:
                    raise VAError(f"{self.mod.name}: line {s.line}: assignment to parameter {s.name!r}")
                if s.name not in self.vars:
                    raise VAError(f"{self.mod.name}: line {s.line}: assignment to undeclared {s.name!r}")
                d = self.deps(s.expr) if self.vars[s.name] == "real" else frozenset()
                self.var_deps[s.name] = self.var_deps[s.name] | d
            elif isinstance(s, If):
                self.deps(s.c)
                self.walk(s.then, collect)
                self.walk(s.other, collect)
            elif isinstance(s, Loop):
                # the body may run any number of times: its assignments join the
                # flow-insensitive fixed point like any other
                self.walk(s.init, collect)
                if s.cond is not None:
                    self.deps(s.cond)
                if s.count is not None:
                    self.deps(s.count)
                self.walk(s.body, collect)
                self.walk(s.step, collect)
            elif isinstance(s, Contrib):
                self.port_index(s.a, s.line)
                if s.b is not None:
                    self.port_index(s.b, s.line)
                if s.kind == "I" and self.vbranch is not None and (
                        (s.a, s.b) == self.vbranch or (s.b is not None and (s.b, s.a) == self.vbranch)):
                    raise VAError(f"{self.mod.name}: line {s.line}: current and voltage contributions on one branch")
                if collect:
                    res, charges, factors = split_ddt(s.expr, s.line)
                    for f_ in factors:
                        if self.deps(f_):
                            raise VAError(f"{self.mod.name}: line {s.line}: a factor of ddt() depends on the "
                                          f"potentials (write it inside the ddt)")
                    self.contribs.append((s, res, charges))
                self.deps(s.expr)

    def run(self):
        self.collect_noise(self.mod.body)
        # dependency sets of variables to a fixed point (flow-insensitive)
        for _ in range(len(self.vars) + 2):
            before = dict(self.var_deps)
            self.walk(self.mod.body, collect=False)
            if before == self.var_deps:
                break
        self.walk(self.mod.body, collect=True)


def _all_stmts(stmts):
    for s in stmts:
        yield s
        if isinstance(s, If):
            yield from _all_stmts(s.then)
            yield from _all_stmts(s.other)
        elif isinstance(s, Loop):
            yield from _all_stmts(s.init + s.body + s.step)


def _check_function(mod: Module, f):
    """An analog function sees its arguments and locals only, assigns only
    those, and calls neither ddt, ddx nor other analog functions' outputs by
    reference."""
    def ex(e):
        if isinstance(e, Name):
            if e.id not in f.local:
                raise VAError(f"{mod.name}: analog function {f.name}: {e.id!r} is not an argument or local")
        elif isinstance(e, Probe):
            raise VAError(f"{mod.name}: analog function {f.name}: probes are not allowed in functions")
        elif isinstance(e, Call):
            if e.fn in ("ddt", "ddx"):
                raise VAError(f"{mod.name}: analog function {f.name}: {e.fn}() is not allowed in functions")
            if e.fn not in FUNCS and e.fn not in mod.functions:
                raise VAError(f"{mod.name}: line {e.line}: unsupported function {e.fn}()")
            for x in e.args:
                ex(x)
        elif isinstance(e, Unary):
            ex(e.x)
        elif isinstance(e, Bin):
            ex(e.a)
            ex(e.b)
        elif isinstance(e, Cond):
            ex(e.c)
            ex(e.a)
            ex(e.b)

    def st(ss):
        for s in ss:
            if isinstance(s, Assign):
                if s.name not in f.local:
                    raise VAError(f"{mod.name}: analog function {f.name}: assignment to {s.name!r}")
                ex(s.expr)
            elif isinstance(s, If):
                ex(s.c)
                st(s.then)
                st(s.other)
            elif isinstance(s, Loop):
                for e in (s.cond, s.count):
                    if e is not None:
                        ex(e)
                st(s.init + s.body + s.step)
            elif isinstance(s, Contrib):
                raise VAError(f"{mod.name}: analog function {f.name}: contributions are not allowed in functions")
    st(f.body)


def split_ddt(e, line: int):
    """Split a contribution into its resistive part and its ddt() terms, which
    must be additive (optionally negated): expr = res + sum(sign * ddt(q))."""
    terms: List[Tuple[int, object]] = []

    def rec(x, sign):
        if isinstance(x, Bin) and x.op in ("+", "-"):
            rec(x.a, sign)
            rec(x.b, sign if x.op == "+" else -sign)
        elif isinstance(x, Unary) and x.op == "-":
            rec(x.x, -sign)
        else:
            terms.append((sign, x))
    rec(e, 1)
    res = None
    charges = []
    factors = []
    for sign, t in terms:
        # c * ddt(q), ddt(q) * c, ddt(q) / c with c constant in time: ddt(c q),
        # ddt(q c), ddt(q / c) (the analysis checks that c has no voltage in it)
        if isinstance(t, Bin) and t.op in ("*", "/"):
            a_, b_ = t.a, t.b
            if t.op == "*" and _is_ddt(b_) and not _has_ddt(a_):
                factors.append(a_)
                t = Call("ddt", [Bin("*", a_, b_.args[0])], b_.line)
            elif _is_ddt(a_) and not _has_ddt(b_):
                factors.append(b_)
                t = Call("ddt", [Bin(t.op, a_.args[0], b_)], a_.line)
        if isinstance(t, Call) and t.fn == "ddt":
            if len(t.args) != 1 or _has_ddt(t.args[0]):
                raise VAError(f"line {line}: ddt() takes one argument without ddt()")
            charges.append((sign, t.args[0]))
        else:
            if _has_ddt(t):
                raise VAError(f"line {line}: ddt() must be an additive term of a contribution")
            tt = t if sign > 0 else Unary("-", t)
            res = tt if res is None else Bin("+", res, tt)
    return res, charges, factors


def _is_ddt(e) -> bool:
    return isinstance(e, Call) and e.fn == "ddt" and len(e.args) == 1


def _has_ddt(e) -> bool:
    if isinstance(e, Call):
        return e.fn == "ddt" or any(_has_ddt(a) for a in e.args)
    if isinstance(e, Unary):
        return _has_ddt(e.x)
    if isinstance(e, Bin):
        return _has_ddt(e.a) or _has_ddt(e.b)
    if isinstance(e, Cond):
        return _has_ddt(e.c) or _has_ddt(e.a) or _has_ddt(e.b)
    return False


def analyze(mod: Module) -> Tuple[VAModel, _Analysis]:
    if not mod.ports:
        raise VAError(f"{mod.name}: a device needs ports")
    nbr = 1 if any(isinstance(s, Contrib) and s.kind == "V" for s in _all_stmts(mod.body)) else 0
    if len(mod.ports) + len(mod.internals) + nbr > MAX_PORTS:
        raise VAError(f"{mod.name}: {len(mod.ports)} ports + {len(mod.internals)} internal nodes + {nbr} branch "
                      f"unknown(s) (at most {MAX_PORTS} in all)")
    names = [p.name for p in mod.params]
    if len(set(names)) != len(names):
        raise VAError(f"{mod.name}: duplicate parameter names")
    for v in mod.variables:
        if v in names:
            raise VAError(f"{mod.name}: {v!r} is both a parameter and a variable")
    a = _Analysis(mod)
    a.run()
    frows: Set[int] = set()
    qrows: Set[int] = set()
    gents: Set[Tuple[int, int]] = set()
    cents: Set[Tuple[int, int]] = set()
    if a.vbranch is not None:
        # KCL: the branch current leaves a and enters b; branch row: V(a) - V(b) - sum(contributions)
        va_, vb_ = a.vbranch
        ends = [a.port[va_]] + ([a.port[vb_]] if vb_ is not None else [])
        frows.update(ends + [a.nb])
        gents.update((r, a.nb) for r in ends)
        gents.update((a.nb, k) for k in ends)
    for c, res, charges in a.contribs:
        rows = [a.port[c.a]] + ([a.port[c.b]] if c.b is not None else []) if c.kind == "I" else [a.nb]
        frows.update(rows)
        if res is not None:
            d = a.deps(res)
            gents.update((r, k) for r in rows for k in d)
        if charges:
            qrows.update(rows)
            d = frozenset()
            for _, q in charges:
                d |= a.deps(q)
            cents.update((r, k) for r in rows for k in d)
    flops = _count_flops(mod.body)
    for f in mod.functions.values():
        _check_function(mod, f)
    m = VAModel(mod.name, mod, list(mod.ports), list(mod.params), a.second_order, sorted(frows), sorted(gents),
                sorted(qrows), sorted(cents), flops, list(a.given), a.vbranch, list(a.noise))
    if m.nout == 0:
        raise VAError(f"{mod.name}: the analog block makes no contribution")
    m.defaults()  # defaults must evaluate and satisfy their ranges
    return m, a


def _count_flops(stmts) -> int:
    n = 0

    def ex(e):
        nonlocal n
        if isinstance(e, Bin):
            n += 1
            ex(e.a)
            ex(e.b)
        elif isinstance(e, Unary):
            n += 1
            ex(e.x)
        elif isinstance(e, Cond):
            ex(e.c)
            ex(e.a)
            ex(e.b)
        elif isinstance(e, Call):
            n += 1
            for x in e.args:
                ex(x)
        elif isinstance(e, Probe):
            n += 1 if e.b is not None else 0

    def st(ss):
        for s in ss:
            if isinstance(s, (Assign, Contrib)):
                ex(s.expr)
            elif isinstance(s, If):
                ex(s.c)
                st(s.then)
                st(s.other)
            elif isinstance(s, Loop):
                st(s.init + s.body + s.step)
    st(stmts)
    return n


# ------------------------------------------------------------------ C++ code
# A module whose analog block holds more statements than this is emitted split
# into functions of about PART_STMTS statements over a frame (split_body); the
# shipped models are far below it and keep the single-function form.
SPLIT_STMTS = 1000
PART_STMTS = 60


def _stmt_count(ss) -> int:
    """Statements in ss, nested blocks included."""
    n = 0
    for st in ss:
        n += 1
        if isinstance(st, If):
            n += _stmt_count(st.then) + _stmt_count(st.other or [])
        elif isinstance(st, Loop):
            n += _stmt_count(st.init) + _stmt_count(st.body) + _stmt_count(st.step)
    return n


def _lit(v: float) -> str:
    r = repr(float(v))
    return r if any(ch in r for ch in ".einf") else r + ".0"


class _Emitter:
    def __init__(self, m: VAModel, a: _Analysis):
        self.m = m
        self.a = a
        self.scope: Optional[Dict[str, str]] = None     # an analog function's names while emitting it
        self.loops = 0                                  # loop counter names
        self.fr = ""                                    # "F." while emitting a split model's frame accesses
        self.parts: List[list] = []                     # statement chunks of a split model, one function each

    def is_int(self, e) -> bool:
        if isinstance(e, Num):
            return e.is_int
        if isinstance(e, Name):
            if self.scope is not None:
                return self.scope.get(e.id) == "integer"
            if e.id in self.a.params:
                return next(p for p in self.m.params if p.name == e.id).type == "integer"
            return self.a.vars.get(e.id) == "integer"
        if isinstance(e, Unary):
            return e.op == "!" or self.is_int(e.x)
        if isinstance(e, Bin):
            if e.op in ("+", "-", "*", "/"):
                return self.is_int(e.a) and self.is_int(e.b)
            return e.op != "**"
        if isinstance(e, Cond):
            return self.is_int(e.a) and self.is_int(e.b)
        return False

    def x(self, e) -> str:
        if isinstance(e, Num):
            return _lit(e.v)
        if isinstance(e, Name):
            if self.scope is not None:
                return "v_" + e.id
            return self.fr + ("p_" if e.id in self.a.params else "v_") + e.id
        if isinstance(e, Probe):
            if e.kind == "I":
                sg = self.a.branch_sign(e.a, e.b, 0)
                return f"V[{self.a.nb}]" if sg > 0 else f"(-V[{self.a.nb}])"
            ia = self.a.port[e.a]
            if e.b is None:
                return f"V[{ia}]"
            return f"(V[{ia}] - V[{self.a.port[e.b]}])"
        if isinstance(e, Unary):
            if e.op == "-":
                return f"(-{self.x(e.x)})"
            return f"((val({self.x(e.x)}) == 0.0) ? 1.0 : 0.0)"
        if isinstance(e, Bin):
            a, b = self.x(e.a), self.x(e.b)
            if e.op in ("+", "-", "*"):
                return f"({a} {e.op} {b})"
            if e.op == "/":
                if self.is_int(e.a) and self.is_int(e.b):
                    return f"vidiv(val({a}), val({b}))"
                return f"({a} / {b})"
            if e.op == "**":
                return f"pow({a}, {b})"
            if e.op in ("&&", "||"):
                return f"((val({a}) != 0.0 {e.op} val({b}) != 0.0) ? 1.0 : 0.0)"
            return f"((val({a}) {e.op} val({b})) ? 1.0 : 0.0)"
        if isinstance(e, Cond):
            return f"vsel(val({self.x(e.c)}) != 0.0, {self.x(e.a)}, {self.x(e.b)})"
        if isinstance(e, Call):
            if e.fn == "ddt":
                raise VAError(f"{self.m.name}: line {e.line}: ddt() outside an additive contribution term")
            if e.fn == "ddx":
                if len(e.args) != 2 or not isinstance(e.args[1], Probe):
                    raise VAError(f"{self.m.name}: line {e.line}: ddx(expr, V(node)) expected")
                p = e.args[1]
                inner = self.x(e.args[0])
                ia = self.a.port[p.a]
                if p.b is None:
                    return f"ddx({inner}, {ia})"
                # two-node probe: the mean of the two one-sided partials, as
                # CedarSim defines it (src/vasim.jl:400-411)
                return f"((ddx({inner}, {ia}) - ddx({inner}, {self.a.port[p.b]})) * 0.5)"
            if e.fn == "white_noise":
                # zero in DC, transient and AC; a noise evaluation records its power
                if id(e) not in self.a.noise_index:
                    raise VAError(f"{self.m.name}: line {e.line}: white_noise() outside a current contribution")
                return f"va_noise(nz, {self.a.noise_index[id(e)]}, val({self.x(e.args[0])}))"
            if e.fn == "flicker_noise":
                # density pwr / f^ex in a noise analysis, zero elsewhere
                if id(e) not in self.a.noise_index:
                    raise VAError(f"{self.m.name}: line {e.line}: flicker_noise() outside a current contribution")
                ex = [a for a in e.args if not isinstance(a, str)]
                if len(ex) != 2:
                    raise VAError(f"{self.m.name}: line {e.line}: flicker_noise() takes a power and an exponent")
                return (f"va_flicker(nz, {self.a.noise_index[id(e)]}, {len(self.a.noise)}, val({self.x(ex[0])}), "
                        f"val({self.x(ex[1])}))")
            if e.fn in self.a.funcs:
                f = self.a.funcs[e.fn]
                if len(e.args) != len(f.inputs):
                    raise VAError(f"{self.m.name}: line {e.line}: {e.fn}() takes {len(f.inputs)} argument(s)")
                parts = []
                for an, a in zip(f.inputs, e.args):
                    if an in f.outputs:       # by reference: a variable of the caller
                        if not isinstance(a, Name):
                            raise VAError(f"{self.m.name}: line {e.line}: output argument {an} needs a variable")
                        parts.append(f", {self.fr if self.scope is None else ''}v_{a.id}")
                    else:
                        parts.append(f", D({self.x(a)})")
                return f"fn_{self.m.name}_{e.fn}<D>(c{''.join(parts)})"
            if e.fn not in FUNCS:
                raise VAError(f"{self.m.name}: line {e.line}: unsupported function {e.fn}()")
            cname, ar = FUNCS[e.fn]
            if len(e.args) != ar:
                raise VAError(f"{self.m.name}: line {e.line}: {e.fn}() takes {ar} argument(s)")
            return f"{cname}({', '.join(self.x(a) for a in e.args)})"
        if isinstance(e, SysCall):
            if e.name == "$vt":
                if e.args:
                    return f"({_lit(P_K)} * val({self.x(e.args[0])}) / {_lit(P_Q)})"
                return "c.vt"
            if e.name == "$temperature":
                return "c.temp"
            if e.name == "$mfactor":
                return "c.m"
            if e.name in ("$param_given", "$given"):
                return f"{self.fr if self.scope is None else ''}p__given_{e.args[0].id}"
            if e.name == "$simparam":
                if not e.args or not isinstance(e.args[0], str):
                    raise VAError(f"{self.m.name}: $simparam needs a name")
                if e.args[0] == "gmin":
                    return "c.gmin"
                if len(e.args) > 1:
                    return self.x(e.args[1])
                raise VAError(f"{self.m.name}: $simparam(\"{e.args[0]}\") has no value here and no default")
        raise VAError(f"{self.m.name}: unsupported expression {e!r}")

    def stmts(self, ss, ind: str, types: Optional[Dict[str, str]] = None) -> List[str]:
        types = self.a.vars if types is None else types
        out = []
        for s in ss:
            if isinstance(s, Assign):
                tgt = (self.fr if self.scope is None else "") + "v_" + s.name
                if types[s.name] == "integer":
                    out.append(f"{ind}{tgt} = vint(val({self.x(s.expr)}));")
                else:
                    out.append(f"{ind}{tgt} = D({self.x(s.expr)});")
            elif isinstance(s, If):
                out.append(f"{ind}if (val({self.x(s.c)}) != 0.0) {{")
                out += self.stmts(s.then, ind + "  ", types)
                if s.other:
                    out.append(f"{ind}}} else {{")
                    out += self.stmts(s.other, ind + "  ", types)
                out.append(f"{ind}}}")
            elif isinstance(s, Loop):
                # at most LOOP_CAP passes, so no model can spin on the device
                self.loops += 1
                it = f"it{self.loops}_"
                out.append(f"{ind}{{")
                out += self.stmts(s.init, ind + "  ", types)
                if s.count is not None:
                    cnt = f"n{self.loops}_"
                    out.append(f"{ind}  const double {cnt} = vint(val({self.x(s.count)}));")
                    out.append(f"{ind}  for (int {it} = 0; {it} < {LOOP_CAP} && {it} < {cnt}; ++{it}) {{")
                else:
                    out.append(f"{ind}  for (int {it} = 0; {it} < {LOOP_CAP} && val({self.x(s.cond)}) != 0.0; ++{it}) {{")
                out += self.stmts(s.body, ind + "    ", types)
                out += self.stmts(s.step, ind + "    ", types)
                out.append(f"{ind}  }}")
                out.append(f"{ind}}}")
            elif isinstance(s, Contrib) and s.kind == "V":
                # V(a,b) <+ e: the branch row collects -e (its orientation folded in)
                res, charges, _ = split_ddt(s.expr, s.line)
                sg = "-=" if self.a.branch_sign(s.a, s.b, s.line) > 0 else "+="
                nb = self.a.nb
                if res is not None:
                    out.append(f"{ind}Fi[{nb}] {sg} D({self.x(res)});")
                for c_sg, t in charges:
                    op = sg if c_sg > 0 else ("+=" if sg == "-=" else "-=")
                    out.append(f"{ind}Fq[{nb}] {op} D({self.x(t)});")
            elif isinstance(s, Contrib):
                res, charges, _ = split_ddt(s.expr, s.line)
                ia = self.a.port[s.a]
                ib = None if s.b is None else self.a.port[s.b]
                if res is not None:
                    out.append(f"{ind}{{ const D i_ = {self.x(res)};")
                    out.append(f"{ind}  Fi[{ia}] -= i_;" + (f" Fi[{ib}] += i_;" if ib is not None else "") + " }")
                if charges:
                    q = " + ".join(("" if sg > 0 else "-") + f"D({self.x(t)})" for sg, t in charges)
                    out.append(f"{ind}{{ const D q_ = {q};")
                    out.append(f"{ind}  Fq[{ia}] -= q_;" + (f" Fq[{ib}] += q_;" if ib is not None else "") + " }")
        return out

    def body(self) -> str:
        if _stmt_count(self.m.module.body) > SPLIT_STMTS:
            return self.split_body()
        m = self.m
        L = [f"// module {m.name}({', '.join(m.ports)})" + (f", internal {', '.join(m.internals)}" if m.internals else ""),
             "template <class D>",
             f"VA_HD void body_{m.name}(const double *P, int ps, const Ctx &c, const D *V, D *Fi, D *Fq, "
             f"double *nz) {{"]
        for k, p in enumerate(m.params):
            L.append(f"  const double p_{p.name} = P[{k} * ps];")
        for j, g in enumerate(m.given):
            L.append(f"  const double p__given_{g} = P[{len(m.params) + j} * ps];")
        for v, t in m.module.variables.items():
            L.append(f"  D v_{v}(0.0);" if t == "real" else f"  double v_{v} = 0.0;")
        if self.a.vbranch is not None:
            va_, vb_ = self.a.vbranch
            ia, nb = self.a.port[va_], self.a.nb
            if vb_ is None:
                L.append(f"  Fi[{ia}] -= V[{nb}]; Fi[{nb}] += V[{ia}];")
            else:
                ib = self.a.port[vb_]
                L.append(f"  Fi[{ia}] -= V[{nb}]; Fi[{ib}] += V[{nb}]; Fi[{nb}] += V[{ia}] - V[{ib}];")
        L += self.stmts(m.module.body, "  ")
        L.append("  (void)c; (void)V; (void)Fi; (void)Fq; (void)P; (void)ps; (void)nz;")
        L.append("}")
        return "\n".join(L)

    def split_body(self) -> str:
        """A large module (a CMC compact model) as several functions: its
        parameters, $param_given flags and variables live in a frame struct, the
        analog block's statements are cut into chunks of about PART_STMTS
        statements at statement boundaries (an if whose branches are larger is
        kept in the caller and its branches cut in turn), and each chunk is a
        function that is not inlined.  The arithmetic, its order and the results
        are those of the single function; what changes is that no one function
        is the whole model, which the device compiler's register allocation
        otherwise takes tens of minutes over."""
        m = self.m
        self.fr = ""
        fields = [f"  double p_{p.name};" for p in m.params]
        fields += [f"  double p__given_{g};" for g in m.given]
        fields += [f"  D v_{v} = D(0.0);" if t == "real" else f"  double v_{v} = 0.0;"
                   for v, t in m.module.variables.items()]
        frame = ["template <class D>", f"struct Frame_{m.name} {{", *fields, "};"]
        self.fr = "F."
        self.parts = []
        calls = self._split(m.module.body, "  ")
        head = [f"// module {m.name}({', '.join(m.ports)})" + (f", internal {', '.join(m.internals)}" if m.internals else "")
                + f": split into {len(self.parts)} functions over a frame"]
        sig = "const double *P, int ps, const Ctx &c, const D *V, D *Fi, D *Fq, double *nz"
        defs = []
        for k, chunk in enumerate(self.parts):
            defs += ["template <class D>", f"VA_PART void part_{m.name}_{k}({sig}, Frame_{m.name}<D> &F) {{"]
            defs += self.stmts(chunk, "  ")
            defs += ["  (void)P; (void)ps; (void)c; (void)V; (void)Fi; (void)Fq; (void)nz; (void)F;", "}"]
        B = ["template <class D>", f"VA_HD void body_{m.name}({sig}) {{", f"  Frame_{m.name}<D> F;"]
        for k, p_ in enumerate(m.params):
            B.append(f"  F.p_{p_.name} = P[{k} * ps];")
        for j, g in enumerate(m.given):
            B.append(f"  F.p__given_{g} = P[{len(m.params) + j} * ps];")
        if self.a.vbranch is not None:
            va_, vb_ = self.a.vbranch
            ia, nb = self.a.port[va_], self.a.nb
            if vb_ is None:
                B.append(f"  Fi[{ia}] -= V[{nb}]; Fi[{nb}] += V[{ia}];")
            else:
                ib = self.a.port[vb_]
                B.append(f"  Fi[{ia}] -= V[{nb}]; Fi[{ib}] += V[{nb}]; Fi[{nb}] += V[{ia}] - V[{ib}];")
        B += calls
        B += ["  (void)c; (void)V; (void)Fi; (void)Fq; (void)P; (void)ps; (void)nz;", "}"]
        self.fr = ""
        return "\n".join(head + frame + defs + B)

    def _split(self, ss, ind: str) -> List[str]:
        """The caller's lines for statements ss: runs of statements become calls of
        new part functions; an if larger than a part stays here, its branches split."""
        out, chunk, n = [], [], 0
        args = "(P, ps, c, V, Fi, Fq, nz, F);"

        def flush():
            nonlocal chunk, n
            if chunk:
                out.append(f"{ind}part_{self.m.name}_{len(self.parts)}<D>{args}")
                self.parts.append(chunk)
                chunk, n = [], 0
        for st in ss:
            k = _stmt_count([st])
            if isinstance(st, If) and k > PART_STMTS:
                flush()
                out.append(f"{ind}if (val({self.x(st.c)}) != 0.0) {{")
                out += self._split(st.then, ind + "  ")
                if st.other:
                    out.append(f"{ind}}} else {{")
                    out += self._split(st.other, ind + "  ")
                out.append(f"{ind}}}")
                continue
            if n + k > PART_STMTS:
                flush()
            chunk.append(st)
            n += k
        flush()
        return out

    def functions(self) -> str:
        """Analog functions as templates over the body's dual type: arguments by
        value, locals zero-initialised, the result in the variable named after
        the function."""
        out = []
        for f in self.m.module.functions.values():
            args = "".join((f", {'D' if f.local[a] == 'real' else 'double'} &v_{a}" if a in f.outputs
                            else f", D v_{a}") for a in f.inputs)
            L = ["template <class D>", f"VA_HD D fn_{self.m.name}_{f.name}(const Ctx &c{args}) {{"]
            for v, t in f.local.items():
                if v in f.inputs:
                    continue
                L.append(f"  D v_{v}(0.0);" if t == "real" else f"  double v_{v} = 0.0;")
            self.scope = f.local
            try:
                L += self.stmts(f.body, "  ", f.local)
            finally:
                self.scope = None
            L.append(f"  (void)c;")
            L.append(f"  return D(v_{f.name});")
            L.append("}")
            out.append("\n".join(L))
        return "\n\n".join(out)

    def dtype(self) -> str:
        n = self.m.nx
        return f"Dual<Dual<double, {n}>, {n}>" if self.m.second_order else f"Dual<double, {n}>"

    def prologue(self, nz: str = "nullptr") -> List[str]:
        m = self.m
        P = m.npar - 1                 # position of m in the derived block (vt follows)
        return [f"  typedef {self.dtype()} D;",
                "  Ctx c;",
                f"  c.m = dp[{P} * ds]; c.vt = dp[{P + 1} * ds]; c.temp = c.vt * {_lit(P_Q / P_K)}; c.gmin = gmin;",
                f"  D V[{m.nx}], Fi[{m.nx}], Fq[{m.nx}];",
                f"  for (int k = 0; k < {m.nx}; ++k) V[k] = Seed<D>::make(v[k], k);",
                f"  body_{m.name}<D>(dp, ds, c, V, Fi, Fq, {nz});"]

    def eval(self) -> str:
        m = self.m
        L = [f"VA_HD void eval_{m.name}(const double *dp, int ds, const double *v, const double *vd, bool xdot, "
             f"double cj, double gmin, double *out, int os) {{"]
        L += self.prologue()
        L.append("  const double mf = c.m;")
        o = 0
        for r in m.frows:
            if r in m.qrows:
                qd = " + ".join(f"part(Fq[{r}], {k}) * vd[{k}]" for k in range(m.nx))
                L.append(f"  out[{o} * os] = mf * (val(Fi[{r}]) + (xdot ? ({qd}) : cj * val(Fq[{r}])));")
            else:
                L.append(f"  out[{o} * os] = mf * val(Fi[{r}]);")
            o += 1
        for r, k in m.gents:
            L.append(f"  out[{o} * os] = mf * part(Fi[{r}], {k});")
            o += 1
        for r in m.qrows:
            L.append(f"  out[{o} * os] = mf * val(Fq[{r}]);")
            o += 1
        for r, k in m.cents:
            L.append(f"  out[{o} * os] = cj * (mf * part(Fq[{r}], {k}));")
            o += 1
        L.append("  (void)vd; (void)xdot; (void)cj;")
        L.append("}")
        return "\n".join(L)

    def noise(self) -> str:
        """Powers (A^2/Hz at 1 Hz, unscaled by m) and frequency exponents (0 for
        white_noise, ex of flicker_noise) of the module's noise sources at v."""
        m = self.m
        n = len(m.noise)
        L = [f"inline int noise_{m.name}(const double *dp, int ds, const double *v, double gmin, double *pw, "
             f"double *ex) {{",
             f"  double nz[{2 * n}];",
             f"  for (int j = 0; j < {2 * n}; ++j) nz[j] = 0.0;"]
        L += self.prologue("nz")
        L.append(f"  for (int j = 0; j < {n}; ++j) {{ pw[j] = nz[j]; ex[j] = nz[{n} + j]; }}")
        L.append(f"  return {n};")
        L.append("}")
        return "\n".join(L)

    def full(self) -> str:
        m = self.m
        n = m.nx
        L = [f"inline void full_{m.name}(const double *dp, int ds, const double *v, double gmin, double *fi, "
             f"double *fq, double *G, double *C) {{"]
        L += self.prologue()
        L.append(f"  for (int r = 0; r < {n}; ++r) {{")
        L.append("    fi[r] = val(Fi[r]); fq[r] = val(Fq[r]);")
        L.append(f"    for (int k = 0; k < {n}; ++k) {{ G[r * {n} + k] = part(Fi[r], k); C[r * {n} + k] = part(Fq[r], k); }}")
        L.append("  }")
        L.append("}")
        return "\n".join(L)


def emit_header(models: List[Tuple[VAModel, _Analysis]], base_id: int) -> str:
    """The generated header: per-model code and the dispatch over the model index."""
    K = len(models)
    L = ["// Generated by cedarsim.jl_gb300/va/emit.py from Verilog-A sources; do not edit.",
         "#pragma once",
         '#include "va_dual.cuh"',
         ""]
    width = max([BUILTIN_TERMS] + [m.nx for m, _ in models])
    if width > BUILTIN_TERMS:
        L += [f"#define CEDAR_MAX_TERM {width}   // a model here has {width} terminal values", ""]
    L += [
         "namespace cedar {",
         "namespace va {",
         "",
         f"constexpr int kBase = {base_id};       // model id of the first Verilog-A model",
         f"constexpr int kCount = {K};",
         "",
         "struct Ctx { double m, vt, temp, gmin; };",
         ""]
    for m, a in models:
        e = _Emitter(m, a)
        fns = e.functions()
        L += ([fns, ""] if fns else []) + [e.body(), "", "#if !defined(CEDAR_VA_SEPARATE) || defined(CEDAR_VA_DEFINE)",
                                            e.eval(), "#endif", "", e.full(), ""]
        if m.noise:
            L += [e.noise(), ""]

    def table(name, vals, ctype="int"):
        vals = list(vals) or [0]
        return f"static const {ctype} {name}[] = {{{', '.join(str(v) for v in vals)}}};"

    L.append(table("kNTerm", [m.nterm for m, _ in models]))
    L.append(table("kHasBr", [m.has_br for m, _ in models]))
    L.append(table("kNPar", [m.npar for m, _ in models]))
    L.append(table("kNDPar", [m.ndpar for m, _ in models]))
    L.append(table("kNOut", [m.nout for m, _ in models]))
    L.append(table("kHasQ", [int(bool(m.qrows)) for m, _ in models]))
    L.append(table("kFlops", [m.flops for m, _ in models]))
    names = ", ".join(f'"{m.name}"' for m, _ in models) or '""'
    L.append(f"static const char *const kName[] = {{{names}}};")
    # stamps: kind 0 = residual row, 1 = J (resistive), 2 = charge row, 3 = J (charge partial)
    st, ptr = [], [0]
    for m, _ in models:
        o = 0
        for r in m.frows:
            st += [0, r, -1, o]; o += 1
        for r, k in m.gents:
            st += [1, r, k, o]; o += 1
        for r in m.qrows:
            st += [2, r, -1, o]; o += 1
        for r, k in m.cents:
            st += [3, r, k, o]; o += 1
        ptr.append(len(st) // 4)
    L.append(table("kStamps", st))
    # noise sources: per model, (row port, column port or -1) pairs
    nzs, nzp = [], [0]
    for m, _ in models:
        for a_, b_ in m.noise:
            nzs += [a_, b_]
        nzp.append(len(nzs) // 2)
    L.append(table("kNoise", nzs))
    L.append(table("kNoisePtr", nzp))
    L.append(table("kStampPtr", ptr))
    L.append("")
    # device-side dispatch (switches over a warp-uniform model id)
    # (the tables above are host data; device code reads switches)
    def switch(fn, rtype, vals, default):
        out = [f"VA_HD {rtype} {fn}(int k) {{", "  switch (k) {"]
        out += [f"    case {i}: return {v};" for i, v in enumerate(vals)]
        out += ["    default: break;", "  }", f"  return {default};", "}"]
        return out
    L += switch("nout", "int", [m.nout for m, _ in models], 0)
    L += switch("has_q", "bool", ["true" if m.qrows else "false" for m, _ in models], "false")
    L += switch("npar", "int", [m.npar for m, _ in models], 0)
    L.append("VA_HD void derive(int k, const double *raw, int rs, double *dp, int ds, double vt) {")
    L.append("  const int np = npar(k);")
    L.append("  if (np == 0) return;")
    L.append("  for (int i = 0; i < np; ++i) dp[i * ds] = raw[i * rs];")
    L.append("  dp[np * ds] = vt;")
    L.append("}")
    sig = ("void eval(int k, const double *dp, int ds, const double *v, const double *vd, bool xdot, double cj, "
           "double gmin, double *out, int os)")
    L.append("#if defined(CEDAR_VA_SEPARATE) && !defined(CEDAR_VA_DEFINE)")
    L.append(f"VA_EXTERN {sig};   // defined in va_models.cu")
    L.append("#else")
    L.append(f"VA_CALL {sig} {{")
    L.append("  switch (k) {")
    for i, (m, _) in enumerate(models):
        L.append(f"    case {i}: eval_{m.name}(dp, ds, v, vd, xdot, cj, gmin, out, os); break;")
    L.append("    default: break;")
    L.append("  }")
    L.append("  (void)dp; (void)ds; (void)v; (void)vd; (void)xdot; (void)cj; (void)gmin; (void)out; (void)os;")
    L.append("}")
    L.append("#endif")
    L.append("inline int noise(int k, const double *dp, int ds, const double *v, double gmin, double *pw, "
             "double *ex) {")
    L.append("  switch (k) {")
    for i, (m, _) in enumerate(models):
        if m.noise:
            L.append(f"    case {i}: return noise_{m.name}(dp, ds, v, gmin, pw, ex);")
    L.append("    default: break;")
    L.append("  }")
    L.append("  (void)dp; (void)ds; (void)v; (void)gmin; (void)pw; (void)ex;")
    L.append("  return 0;")
    L.append("}")
    L.append("inline void full(int k, const double *dp, int ds, const double *v, double gmin, double *fi, double *fq, "
             "double *G, double *C) {")
    L.append("  switch (k) {")
    for i, (m, _) in enumerate(models):
        L.append(f"    case {i}: full_{m.name}(dp, ds, v, gmin, fi, fq, G, C); break;")
    L.append("    default: break;")
    L.append("  }")
    L.append("  (void)dp; (void)ds; (void)v; (void)gmin; (void)fi; (void)fq; (void)G; (void)C;")
    L.append("}")
    L += ["", "}  // namespace va", "}  // namespace cedar", ""]
    return "\n".join(L)
