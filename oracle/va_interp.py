"""Direct interpretation of a parsed Verilog-A module, with nested dual numbers.

TEST INFRASTRUCTURE ONLY: the independent check of the product's Verilog-A
emitter (cedarsim.jl_gb300/va/emit.py).  Where the emitter writes C++ over a
dual-number template and a dependency analysis, this walks the parsed module
statement by statement in Python: every value is a second-order dual over the
port potentials, ddt(x) is carried as a separate charge channel, integer
variables are Python ints.  Semantics followed (CedarSim, file:line):
  * I(a,b) <+ e: current a -> b, KCL(a) += -e, KCL(b) += +e   src/simulate_ir.jl:54,112-120
  * ddx(x, V(a)) = dx/dVa; ddx(x, V(a,b)) = (dx/dVa - dx/dVb)/2 src/vasim.jl:392-412
  * real -> integer: round half away from zero                 src/va_env.jl:92-110
  * $temperature = temp + 273.15 K; $simparam("gmin")           src/va_env.jl:112-123
"""
from __future__ import annotations

import math
from typing import Dict, List


class D:
    """Dual number: value v and partials d (floats or nested D)."""
    __slots__ = ("v", "d")

    def __init__(self, v, d):
        self.v, self.d = v, d

    # arithmetic -------------------------------------------------------------
    def _lift(self, o):
        return o if isinstance(o, D) else D(o, [_zero(x) for x in self.d])

    def __add__(self, o):
        o = self._lift(o)
        return D(self.v + o.v, [a + b for a, b in zip(self.d, o.d)])
    __radd__ = __add__

    def __sub__(self, o):
        o = self._lift(o)
        return D(self.v - o.v, [a - b for a, b in zip(self.d, o.d)])

    def __rsub__(self, o):
        return self._lift(o) - self

    def __neg__(self):
        return D(-self.v, [-a for a in self.d])

    def __mul__(self, o):
        o = self._lift(o)
        return D(self.v * o.v, [a * o.v + self.v * b for a, b in zip(self.d, o.d)])
    __rmul__ = __mul__

    def __truediv__(self, o):
        o = self._lift(o)
        q = _fdiv(self.v, o.v)
        return D(q, [_fdiv(a * o.v - self.v * b, o.v * o.v) for a, b in zip(self.d, o.d)])

    def __rtruediv__(self, o):
        return self._lift(o) / self


def _fdiv(a, b):
    """a / b with IEEE results for a zero divisor (inf or nan), as the device code."""
    if isinstance(a, D) or isinstance(b, D):
        return a / b
    try:
        return a / b
    except ZeroDivisionError:
        return math.nan if a == 0 else math.copysign(math.inf, a) * math.copysign(1.0, b)


def _zero(x):
    return D(0.0, [_zero(y) for y in x.d]) if isinstance(x, D) else 0.0


def value(x) -> float:
    while isinstance(x, D):
        x = x.v
    return float(x)


def _fn(name):
    """The float function of a Verilog-A built-in (NaN outside its domain)."""
    f = {"exp": math.exp, "ln": math.log, "log": math.log10, "sqrt": math.sqrt, "sin": math.sin,
         "cos": math.cos, "tan": math.tan, "sinh": math.sinh, "cosh": math.cosh, "tanh": math.tanh,
         "atan": math.atan, "asin": math.asin, "acos": math.acos}[name]

    def g(x):
        try:
            return f(x)
        except (ValueError, OverflowError):
            return math.nan
    return g


def _unary_fn(name, x):
    if not isinstance(x, D):
        return _fn(name)(x)
    return D(_unary_fn(name, x.v), [_sz(_deriv(name, x.v), a) for a in x.d])


def _sz(fp, a):
    """fp * a with a strong zero: a zero direction stays zero even where fp is
    infinite (the derivative of sqrt or pow at 0)."""
    return _zero(a) if not _nonzero(a) else fp * a


def _deriv(name, v):
    """f'(v) for v a float or a dual (so second derivatives come out right)."""
    if name in ("exp",):
        return _unary_fn("exp", v)
    if name == "ln":
        return _fdiv(1.0, v) if not isinstance(v, D) else D(1.0, [_zero(a) for a in v.d]) / v
    if name == "log":
        return _fdiv(1.0, v * math.log(10.0)) if not isinstance(v, D) else D(1.0, [_zero(a) for a in v.d]) / (v * math.log(10.0))
    if name == "sqrt":
        return _fdiv(0.5, _unary_fn("sqrt", v)) if not isinstance(v, D) else D(0.5, [_zero(a) for a in v.d]) / _unary_fn("sqrt", v)
    if name == "sin":
        return _unary_fn("cos", v)
    if name == "cos":
        return -_unary_fn("sin", v)
    if name == "tan":
        t = _unary_fn("tan", v)
        return 1.0 + t * t
    if name == "sinh":
        return _unary_fn("cosh", v)
    if name == "cosh":
        return _unary_fn("sinh", v)
    if name == "tanh":
        t = _unary_fn("tanh", v)
        return 1.0 - t * t
    if name == "atan":
        return 1.0 / (1.0 + v * v) if not isinstance(v, D) else D(1.0, [_zero(a) for a in v.d]) / (1.0 + v * v)
    if name in ("asin", "acos"):
        s = _unary_fn("sqrt", 1.0 - v * v)
        one = 1.0 if not isinstance(v, D) else D(1.0, [_zero(a) for a in v.d])
        return _fdiv(one, s) if name == "asin" else -_fdiv(one, s)
    raise KeyError(name)


def _pow_grad_x(x, p):
    """d(x^p)/dx.  CedarSim's pow frule (src/va_env.jl:57-68) takes ChainRules 1.69's
    pow gradient: p*y/x away from x = 0; at x = 0, 1 for p = 1, 0 for p = 0 or
    p > 1, +inf for 0 < p < 1.  p*x^(p-1) agrees with it except for p = 0 (0 * inf
    at x = 0): x^0 is constant, so its partials are 0; any other p takes
    p*x^(p-1), which keeps second derivatives of nested duals at x = 0."""
    if not _nonzero(p):
        return 0.0
    return p * _pow(x, p - 1.0)


def _pow(x, y):
    if not isinstance(x, D) and not isinstance(y, D):
        if x == 0.0 and y < 0:
            return math.inf                 # C's pow(0, y < 0)
        try:
            return math.pow(x, y)
        except (ValueError, OverflowError):
            return math.nan
    ydep = isinstance(y, D) and any(value(a) != 0.0 or isinstance(a, D) and _nonzero(a) for a in y.d)
    if not ydep:
        yv = y if not isinstance(y, D) else y.v
        base = _pow(x.v, yv)
        return D(base, [_sz(_pow_grad_x(x.v, yv), a) for a in x.d])
    return _unary_fn("exp", y * _unary_fn("ln", x))


def _nonzero(a) -> bool:
    if isinstance(a, D):
        return value(a) != 0.0 or any(_nonzero(b) for b in a.d)
    return a != 0.0


def _limexp(x):
    X = 80.0
    if value(x) <= X:
        return _unary_fn("exp", x)
    return math.exp(X) * (1.0 + (x - X))


class _Q:
    """A contribution value split into its resistive part and its charge (ddt) part."""

    def __init__(self, r, q):
        self.r, self.q = r, q


class Interp:
    def __init__(self, module, params: Dict[str, float], v: List[float], vt: float, gmin: float, m: float = 1.0,
                 given=()):
        self.mod = module
        nodes = list(module.ports) + list(getattr(module, "internals", []))
        self.port = {p: k for k, p in enumerate(nodes)}
        # a voltage-contributed branch V(a,b) <+ ... adds its current as one more
        # unknown after the nodes
        self.vbranch = _voltage_branch(module.body)
        self.nb = len(nodes) if self.vbranch is not None else None
        self.N = len(nodes) + (1 if self.vbranch is not None else 0)
        self.params = {}
        for p in module.params:
            val = params[p.name]
            self.params[p.name] = int(val) if p.type == "integer" else float(val)
        self.vt, self.gmin, self.m = vt, gmin, m
        N = self.N
        # second-order seeds: V_k = (v_k + e_k) as a dual of duals
        self.V = []
        for k in range(N):
            inner = D(float(v[k]), [1.0 if i == k else 0.0 for i in range(N)])
            outer_d = [D(1.0 if i == k else 0.0, [0.0] * N) for i in range(N)]
            self.V.append(D(inner, outer_d))
        self.vars = {name: (0 if t == "integer" else self._const(0.0)) for name, t in module.variables.items()}
        self.types = dict(module.variables)
        self.given = set(given)
        self.noise = []             # ((a index, b index or -1), power, exponent) of each noise source evaluated
        self._branch = None
        self.Fi = [self._const(0.0) for _ in range(N)]
        self.Fq = [self._const(0.0) for _ in range(N)]

    def _const(self, c):
        N = self.N
        return D(D(float(c), [0.0] * N), [D(0.0, [0.0] * N) for _ in range(N)])

    def _dual(self, x):
        return x if isinstance(x, D) else self._const(float(x))

    def run(self):
        from importlib import import_module
        P = import_module("cedarsim_gb300.va.parser")
        self.P = P
        if self.vbranch is not None:
            # the branch current flows a -> b; the branch row starts at V(a) - V(b)
            a, b = self.vbranch
            ib = self.V[self.nb]
            va_ = self.V[self.port[a]]
            vb_ = self.V[self.port[b]] if b is not None else 0.0
            self.Fi[self.port[a]] = self.Fi[self.port[a]] - ib
            if b is not None:
                self.Fi[self.port[b]] = self.Fi[self.port[b]] + ib
            self.Fi[self.nb] = self.Fi[self.nb] + (va_ - vb_)
        self.block(self.mod.body)
        return self.Fi, self.Fq

    def _orient(self, a, b) -> int:
        if (a, b) == self.vbranch:
            return 1
        if b is not None and (b, a) == self.vbranch:
            return -1
        raise ValueError(f"I({a}, {b}) is not the voltage-contributed branch")

    def expr(self, e):
        P = self.P
        if isinstance(e, P.Num):
            return int(e.v) if e.is_int else e.v
        if isinstance(e, P.Name):
            if e.id in self.params:
                return self.params[e.id]
            return self.vars[e.id]
        if isinstance(e, P.Probe):
            if getattr(e, "kind", "V") == "I":
                return self.V[self.nb] * float(self._orient(e.a, e.b))
            a = self.V[self.port[e.a]]
            return a if e.b is None else a - self.V[self.port[e.b]]
        if isinstance(e, P.Unary):
            x = self.expr(e.x)
            if e.op == "-":
                if isinstance(x, _Q):
                    return _Q(-x.r, -x.q)
                return -x
            return int(value(x) == 0.0)
        if isinstance(e, P.Bin):
            a, b = self.expr(e.a), self.expr(e.b)
            if e.op in ("+", "-") and (isinstance(a, _Q) or isinstance(b, _Q)):
                qa = a if isinstance(a, _Q) else _Q(a, 0.0)
                qb = b if isinstance(b, _Q) else _Q(b, 0.0)
                return _Q(qa.r + qb.r, qa.q + qb.q) if e.op == "+" else _Q(qa.r - qb.r, qa.q - qb.q)
            if e.op in ("*", "/") and (isinstance(a, _Q) != isinstance(b, _Q)):
                # c * ddt(q), ddt(q) * c, ddt(q) / c: both channels scale
                if isinstance(a, _Q):
                    return _Q(a.r * b, a.q * b) if e.op == "*" else _Q(a.r / b, a.q / b)
                if e.op == "*":
                    return _Q(a * b.r, a * b.q)
            if isinstance(a, _Q) or isinstance(b, _Q):
                raise ValueError("ddt() in a non-additive position")
            if e.op == "+":
                return a + b
            if e.op == "-":
                return a - b
            if e.op == "*":
                return a * b
            if e.op == "/":
                if isinstance(a, int) and isinstance(b, int):
                    return int(a / b)   # truncation toward zero
                return a / b
            if e.op == "**":
                return _pow(a, b)
            av, bv = value(a), value(b)
            return int({"<": av < bv, ">": av > bv, "<=": av <= bv, ">=": av >= bv, "==": av == bv,
                        "!=": av != bv, "&&": av != 0 and bv != 0, "||": av != 0 or bv != 0}[e.op])
        if isinstance(e, P.Cond):
            return self.expr(e.a) if value(self.expr(e.c)) != 0 else self.expr(e.b)
        if isinstance(e, P.Call):
            fn = e.fn
            if fn == "white_noise":
                # zero outside a noise analysis; record the source across the
                # branch of the contribution being evaluated
                self.noise.append((self._branch, value(self.expr(e.args[0])), 0.0))
                return 0.0
            if fn == "flicker_noise":
                # density pwr / f^ex (PSD, src/ac.jl:267-276)
                pw, ex = [value(self.expr(a)) for a in e.args if not isinstance(a, str)]
                self.noise.append((self._branch, pw, ex))
                return 0.0
            if fn in getattr(self.mod, "functions", {}):
                return self._call(self.mod.functions[fn], e.args)
            if fn == "ddt":
                return _Q(0.0, self.expr(e.args[0]))
            if fn == "ddx":
                x = self._dual(self.expr(e.args[0]))
                pr = e.args[1]
                ia = self.port[pr.a]
                if pr.b is None:
                    return self._ddx(x, ia)
                return (self._ddx(x, ia) - self._ddx(x, self.port[pr.b])) * 0.5
            args = [self.expr(a) for a in e.args]
            if fn in ("exp", "ln", "log", "sqrt", "sin", "cos", "tan", "sinh", "cosh", "tanh", "atan", "asin",
                      "acos"):
                return _unary_fn(fn, args[0])
            if fn == "pow":
                return _pow(args[0], args[1])
            if fn == "abs":
                return -args[0] if value(args[0]) < 0 else args[0]
            if fn == "min":
                return args[0] if value(args[0]) <= value(args[1]) else args[1]
            if fn == "max":
                return args[0] if value(args[0]) >= value(args[1]) else args[1]
            if fn == "floor":
                return float(math.floor(value(args[0])))
            if fn == "ceil":
                return float(math.ceil(value(args[0])))
            if fn == "limexp":
                return _limexp(args[0])
            if fn == "atan2":
                y, x = self._dual(args[0]), self._dual(args[1])
                return _unary_fn("atan", y / x) if value(x) > 0 else _atan2_general(y, x)
            if fn == "hypot":
                x, y = self._dual(args[0]), self._dual(args[1])
                return _unary_fn("sqrt", x * x + y * y)
            raise ValueError(f"function {fn}")
        if isinstance(e, P.SysCall):
            if e.name == "$vt":
                return self.vt if not e.args else 1.380649e-23 * value(self.expr(e.args[0])) / 1.602176634e-19
            if e.name == "$temperature":
                return self.vt * 1.602176634e-19 / 1.380649e-23
            if e.name in ("$param_given", "$given"):
                return int(e.args[0].id in self.given)
            if e.name == "$mfactor":
                return self.m
            if e.name == "$simparam":
                if e.args[0] == "gmin":
                    return self.gmin
                return self.expr(e.args[1])
        raise ValueError(f"expression {e!r}")

    def _ddx(self, x, a):
        """dx/dV_a as a second-order value (its own second partials left zero)."""
        N = self.N
        inner = x.d[a]
        return D(inner, [D(inner.d[i], [0.0] * N) for i in range(N)])

    def _call(self, f, arg_exprs):
        """An analog function: a fresh scope of its arguments and locals; output /
        inout arguments are copied back into the caller's variables."""
        args = [self.expr(a) for a in arg_exprs]
        saved = (self.vars, self.types, self.params)
        self.types = dict(f.local)
        self.vars = {n: (0 if t == "integer" else self._const(0.0)) for n, t in f.local.items()}
        self.params = {}
        for n, a in zip(f.inputs, args):
            self.vars[n] = self._dual(a) if f.local[n] == "real" else a
        try:
            self.block(f.body)
            result = self.vars[f.name]
            outs = {n: self.vars[n] for n in getattr(f, "outputs", [])}
        finally:
            self.vars, self.types, self.params = saved
        for n, a in zip(f.inputs, arg_exprs):
            if n in outs:
                self.vars[a.id] = outs[n] if self.types[a.id] == "real" else int(value(outs[n]))
        return result

    def block(self, stmts):
        P = self.P
        for s in stmts:
            if isinstance(s, P.Assign):
                x = self.expr(s.expr)
                if self.types[s.name] == "integer":
                    v = value(x)
                    self.vars[s.name] = int(math.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1)
                else:
                    self.vars[s.name] = self._dual(x)
            elif isinstance(s, P.If):
                self.block(s.then if value(self.expr(s.c)) != 0 else s.other)
            elif isinstance(s, P.Loop):
                self.block(s.init)
                if s.count is not None:
                    v = value(self.expr(s.count))
                    n = int(math.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1)
                    for _ in range(min(max(n, 0), P.LOOP_CAP)):
                        self.block(s.body)
                else:
                    it = 0
                    while it < P.LOOP_CAP and value(self.expr(s.cond)) != 0:
                        self.block(s.body)
                        self.block(s.step)
                        it += 1
            elif isinstance(s, P.Contrib) and getattr(s, "kind", "I") == "V":
                x = self.expr(s.expr)
                q = x if isinstance(x, _Q) else _Q(x, 0.0)
                sg = float(self._orient(s.a, s.b))
                self.Fi[self.nb] = self.Fi[self.nb] - self._dual(q.r) * sg
                self.Fq[self.nb] = self.Fq[self.nb] - self._dual(q.q) * sg
            elif isinstance(s, P.Contrib):
                self._branch = (self.port[s.a], self.port[s.b] if s.b is not None else -1)
                x = self.expr(s.expr)
                q = x if isinstance(x, _Q) else _Q(x, 0.0)
                ia = self.port[s.a]
                ib = None if s.b is None else self.port[s.b]
                r, c = self._dual(q.r), self._dual(q.q)
                self.Fi[ia] = self.Fi[ia] - r
                self.Fq[ia] = self.Fq[ia] - c
                if ib is not None:
                    self.Fi[ib] = self.Fi[ib] + r
                    self.Fq[ib] = self.Fq[ib] + c


def _voltage_branch(stmts):
    for s in stmts:
        if type(s).__name__ == "If":
            br = _voltage_branch(s.then) or _voltage_branch(s.other)
            if br:
                return br
        elif type(s).__name__ == "Contrib" and getattr(s, "kind", "I") == "V":
            return (s.a, s.b)
    return None


def _atan2_general(y, x):
    # atan2 for x <= 0 through the half-angle identity atan2(y, x) = 2 atan(y / (hypot + x))
    h = _unary_fn("sqrt", x * x + y * y)
    return 2.0 * _unary_fn("atan", y / (h + x))


def evaluate(module, params: Dict[str, float], v: List[float], vt: float, gmin: float, m: float = 1.0,
             given=()):
    """(fi[N], fq[N], G[N][N], C[N][N]) of one device of `module` at port
    potentials v, unscaled by the multiplicity (m is only what $mfactor reads)."""
    it = Interp(module, params, v, vt, gmin, m, given)
    Fi, Fq = it.run()
    N = it.N
    fi = [value(x) for x in Fi]
    fq = [value(x) for x in Fq]
    G = [[value(Fi[r].v.d[k]) for k in range(N)] for r in range(N)]
    Cm = [[value(Fq[r].v.d[k]) for k in range(N)] for r in range(N)]
    return fi, fq, G, Cm


def noise_sources(module, params: Dict[str, float], v: List[float], vt: float, gmin: float, m: float = 1.0,
                  given=()):
    """[((a, b), power, exponent)] of the module's noise sources at port
    potentials v (b = -1 for ground; exponent 0 for white_noise, the density of
    a flicker_noise source being power / f^exponent), unscaled by the
    multiplicity."""
    it = Interp(module, params, v, vt, gmin, m, given)
    it.run()
    return it.noise
