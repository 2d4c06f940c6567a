"""Verilog-A front end: lexer, `define/`include handling and a recursive-descent
parser for the compact-model subset the GPU emitter compiles.

Subset (the constructs CedarSim's VA translator lowers for compact models,
src/vasim.jl:128-180,347-412,663-875):
  module NAME(ports); port directions; `electrical` ports and internal nodes;
  parameter [real|integer] NAME = expr [from|exclude range] {, ...};
  real / integer variables (module or block scope);
  analog begin ... end with assignments, if / else, begin / end blocks,
  current contributions I(a,b) <+ expr and I(a) <+ expr;
  expressions: numbers with SI scale factors, + - * / ** unary - + !, comparisons,
  && || and ?:; V(a,b) / V(a) probes; exp ln log sqrt pow abs min max tanh sinh
  cosh sin cos tan atan atan2 asin acos hypot floor ceil limexp; ddt(expr) (additive
  in a contribution); ddx(expr, V(n)) / ddx(expr, V(a,b)); $vt, $vt(T),
  $temperature, $simparam("gmin"[, default]), $mfactor.
Internal nodes (`electrical` names that are not ports) become extra device
unknowns.  Voltage contributions, branch-current probes, analog functions, noise
sources and events are outside the subset and raise VAError with the line number.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple


class VAError(Exception):
    pass


# ------------------------------------------------------------------ lexer
_TOKEN = re.compile(r"""
    (?P<ws>[ \t\r\n]+)
  | (?P<lcom>//[^\n]*)
  | (?P<bcom>/\*.*?\*/)
  | (?P<num>(\d+\.\d*|\.\d+|\d+)([eE][+-]?\d+)?[TGMKkmunpfa]?)
  | (?P<sys>\$[A-Za-z_][A-Za-z_0-9]*)
  | (?P<dir>`[A-Za-z_][A-Za-z_0-9]*)
  | (?P<id>[A-Za-z_][A-Za-z_0-9]*)
  | (?P<str>"[^"\n]*")
  | (?P<op><\+|\*\*|<=|>=|==|!=|&&|\|\||[-+*/<>!?:;,()\[\]=@{}.])
""", re.S | re.X)

SCALE = {"T": 1e12, "G": 1e9, "M": 1e6, "K": 1e3, "k": 1e3, "m": 1e-3, "u": 1e-6, "n": 1e-9, "p": 1e-12,
         "f": 1e-15, "a": 1e-18}

# constants of the standard constants.vams header (physical constants, SI)
CONSTANTS = {"M_PI": 3.14159265358979323846, "M_TWO_PI": 6.28318530717958647652,
             "M_PI_2": 1.57079632679489661923, "M_E": 2.7182818284590452354,
             "P_Q": 1.602176634e-19, "P_K": 1.380649e-23, "P_CELSIUS0": 273.15,
             "P_EPS0": 8.8541878128e-12}


@dataclass
class Tok:
    kind: str
    text: str
    line: int


def lex(src: str) -> List[Tok]:
    out: List[Tok] = []
    pos, line = 0, 1
    while pos < len(src):
        m = _TOKEN.match(src, pos)
        if not m:
            raise VAError(f"line {line}: unexpected character {src[pos]!r}")
        kind = m.lastgroup
        text = m.group(kind)
        if kind not in ("ws", "lcom", "bcom"):
            out.append(Tok(kind, text, line))
        line += text.count("\n")
        pos = m.end()
    return out


def preprocess(toks: List[Tok]) -> List[Tok]:
    """`define NAME tokens (no arguments), `NAME expansion, `include of the
    standard headers (disciplines.vams / constants.vams: their names are built in),
    `undef; other directives are errors."""
    macros: Dict[str, List[Tok]] = {}
    out: List[Tok] = []
    i = 0
    while i < len(toks):
        t = toks[i]
        if t.kind == "dir":
            name = t.text[1:]
            if name == "include":
                if i + 1 >= len(toks) or toks[i + 1].kind != "str":
                    raise VAError(f"line {t.line}: `include needs a file name")
                fname = toks[i + 1].text.strip('"')
                if fname not in ("disciplines.vams", "constants.vams", "discipline.h", "constants.h"):
                    raise VAError(f"line {t.line}: `include \"{fname}\" is not supported (only the standard headers)")
                i += 2
                continue
            if name == "define":
                if i + 1 >= len(toks) or toks[i + 1].kind != "id":
                    raise VAError(f"line {t.line}: `define needs a name")
                mname, mline = toks[i + 1].text, toks[i + 1].line
                j = i + 2
                body = []
                while j < len(toks) and toks[j].line == mline:
                    body.append(toks[j])
                    j += 1
                if body and body[0].text == "(" and body[0].line == mline:
                    raise VAError(f"line {t.line}: `define with arguments is not supported")
                macros[mname] = body
                i = j
                continue
            if name == "undef":
                macros.pop(toks[i + 1].text, None)
                i += 2
                continue
            if name in macros:
                out.extend(Tok(b.kind, b.text, t.line) for b in macros[name])
                i += 1
                continue
            raise VAError(f"line {t.line}: unknown directive {t.text}")
        out.append(t)
        i += 1
    return out


# ------------------------------------------------------------------ AST
@dataclass
class Num:
    v: float
    is_int: bool = False


@dataclass
class Name:
    id: str
    line: int = 0


@dataclass
class Probe:            # V(a) or V(a, b)
    a: str
    b: Optional[str]


@dataclass
class Call:
    fn: str
    args: list
    line: int = 0


@dataclass
class Unary:
    op: str
    x: object


@dataclass
class Bin:
    op: str
    a: object
    b: object


@dataclass
class Cond:
    c: object
    a: object
    b: object


@dataclass
class SysCall:          # $vt, $temperature, $simparam, $mfactor
    name: str
    args: list


@dataclass
class Assign:
    name: str
    expr: object
    line: int = 0


@dataclass
class Contrib:          # I(a[, b]) <+ expr
    a: str
    b: Optional[str]
    expr: object
    line: int = 0


@dataclass
class If:
    c: object
    then: list
    other: list


@dataclass
class Param:
    name: str
    type: str            # "real" | "integer"
    default: object
    ranges: list = field(default_factory=list)   # (kind, lo, hi, lo_incl, hi_incl) or (kind, value)


@dataclass
class Module:
    name: str
    ports: List[str]
    params: List[Param]
    variables: Dict[str, str]      # name -> "real" | "integer"
    body: list
    internals: List[str] = field(default_factory=list)   # internal nodes, after the ports


# ------------------------------------------------------------------ parser
class Parser:
    def __init__(self, toks: List[Tok]):
        self.t = toks
        self.i = 0

    # token helpers
    def peek(self, k: int = 0) -> Optional[Tok]:
        j = self.i + k
        return self.t[j] if j < len(self.t) else None

    def at(self, text: str) -> bool:
        p = self.peek()
        return p is not None and p.text == text and p.kind in ("op", "id")

    def take(self, text: Optional[str] = None, kind: Optional[str] = None) -> Tok:
        p = self.peek()
        if p is None:
            raise VAError(f"unexpected end of file (expected {text or kind})")
        if (text is not None and p.text != text) or (kind is not None and p.kind != kind):
            raise VAError(f"line {p.line}: expected {text or kind}, found {p.text!r}")
        self.i += 1
        return p

    def ident(self) -> str:
        return self.take(kind="id").text

    # modules
    def modules(self) -> List[Module]:
        mods = []
        while self.peek() is not None:
            if self.at("module"):
                mods.append(self.module())
            elif self.at("nature") or self.at("discipline"):
                raise VAError(f"line {self.peek().line}: natures/disciplines come from the standard header")
            else:
                raise VAError(f"line {self.peek().line}: expected `module`, found {self.peek().text!r}")
        return mods

    def module(self) -> Module:
        self.take("module")
        name = self.ident()
        ports: List[str] = []
        if self.at("("):
            self.take("(")
            if not self.at(")"):
                ports.append(self.ident())
                while self.at(","):
                    self.take(",")
                    ports.append(self.ident())
            self.take(")")
        self.take(";")
        params: List[Param] = []
        variables: Dict[str, str] = {}
        body: list = []
        electrical = set()
        internals: List[str] = []
        while not self.at("endmodule"):
            p = self.peek()
            if p is None:
                raise VAError(f"module {name}: missing endmodule")
            if p.text in ("inout", "input", "output"):
                self.take()
                self._idlist()
            elif p.text == "electrical":
                self.take()
                for n in self._idlist():
                    if n not in ports and n not in internals:
                        internals.append(n)       # an internal node: one more unknown per instance
                    electrical.add(n)
            elif p.text in ("parameter", "localparam"):
                params.extend(self._params())
            elif p.text in ("real", "integer"):
                self.take()
                for n in self._idlist():
                    variables[n] = p.text
            elif p.text == "analog":
                self.take()
                if self.at("initial"):
                    raise VAError(f"line {p.line}: analog initial is not supported")
                body.extend(self.statement(variables))
            else:
                raise VAError(f"line {p.line}: unsupported module item {p.text!r}")
        self.take("endmodule")
        missing = [q for q in ports if q not in electrical]
        if missing:
            raise VAError(f"module {name}: ports without a discipline: {missing}")
        return Module(name, ports, params, variables, body, internals)

    def _idlist(self) -> List[str]:
        names = [self.ident()]
        while self.at(","):
            self.take(",")
            names.append(self.ident())
        self.take(";")
        return names

    def _params(self) -> List[Param]:
        self.take()
        typ = "real"
        if self.at("real") or self.at("integer"):
            typ = self.take().text
        out = []
        while True:
            name = self.ident()
            self.take("=")
            default = self.expr()
            ranges = []
            while self.at("from") or self.at("exclude"):
                kind = self.take().text
                if self.at("[") or self.at("("):
                    lo_incl = self.take().text == "["
                    lo = self.expr()
                    self.take(":")
                    hi = self.expr()
                    hi_incl = self.take().text == "]"
                    ranges.append((kind, lo, hi, lo_incl, hi_incl))
                else:
                    ranges.append((kind, self.expr()))
            out.append(Param(name, typ, default, ranges))
            if self.at(","):
                self.take(",")
                continue
            self.take(";")
            return out

    # statements
    def statement(self, variables: Dict[str, str]) -> list:
        p = self.peek()
        if p is None:
            raise VAError("unexpected end of file in a statement")
        if p.text == "begin":
            self.take()
            if self.at(":"):
                self.take(":")
                self.ident()
            out = []
            while not self.at("end"):
                q = self.peek()
                if q is None:
                    raise VAError("missing `end`")
                if q.text in ("real", "integer"):
                    self.take()
                    for n in self._idlist():
                        variables[n] = q.text
                    continue
                out.extend(self.statement(variables))
            self.take("end")
            return out
        if p.text == "if":
            self.take()
            self.take("(")
            c = self.expr()
            self.take(")")
            then = self.statement(variables)
            other = []
            if self.at("else"):
                self.take()
                other = self.statement(variables)
            return [If(c, then, other)]
        if p.text == ";":
            self.take()
            return []
        if p.kind == "id" and p.text in ("I", "V") and self.peek(1) is not None and self.peek(1).text == "(":
            # contribution
            kind = self.take().text
            self.take("(")
            a = self.ident()
            b = None
            if self.at(","):
                self.take(",")
                b = self.ident()
            self.take(")")
            if not self.at("<+"):
                raise VAError(f"line {p.line}: expected <+ after {kind}(...)")
            self.take("<+")
            e = self.expr()
            self.take(";")
            if kind == "V":
                raise VAError(f"line {p.line}: voltage contributions V(...) <+ are not supported")
            return [Contrib(a, b, e, p.line)]
        if p.kind == "id":
            name = self.take().text
            self.take("=")
            e = self.expr()
            self.take(";")
            return [Assign(name, e, p.line)]
        raise VAError(f"line {p.line}: unsupported statement starting with {p.text!r}")

    # expressions (precedence from low to high)
    def expr(self):
        c = self._lor()
        if self.at("?"):
            self.take("?")
            a = self.expr()
            self.take(":")
            b = self.expr()
            return Cond(c, a, b)
        return c

    def _left(self, sub, ops):
        a = sub()
        while self.peek() is not None and self.peek().kind == "op" and self.peek().text in ops:
            op = self.take().text
            a = Bin(op, a, sub())
        return a

    def _lor(self):
        return self._left(self._land, ("||",))

    def _land(self):
        return self._left(self._eq, ("&&",))

    def _eq(self):
        return self._left(self._rel, ("==", "!="))

    def _rel(self):
        return self._left(self._add, ("<", ">", "<=", ">="))

    def _add(self):
        return self._left(self._mul, ("+", "-"))

    def _mul(self):
        return self._left(self._unary, ("*", "/"))

    def _unary(self):
        if self.peek() is not None and self.peek().kind == "op" and self.peek().text in ("-", "+", "!"):
            op = self.take().text
            x = self._unary()
            return x if op == "+" else Unary(op, x)
        return self._pow()

    def _pow(self):
        a = self._primary()
        if self.at("**"):
            self.take("**")
            return Bin("**", a, self._unary())
        return a

    def _primary(self):
        p = self.take()
        if p.kind == "num":
            txt = p.text
            s = 1.0
            if txt[-1] in SCALE:
                s = SCALE[txt[-1]]
                txt = txt[:-1]
                return Num(float(txt) * s)
            return Num(float(txt), is_int=txt.isdigit())
        if p.text == "(" and p.kind == "op":
            e = self.expr()
            self.take(")")
            return e
        if p.kind == "sys":
            args = []
            if self.at("("):
                self.take("(")
                if not self.at(")"):
                    args.append(self._sysarg())
                    while self.at(","):
                        self.take(",")
                        args.append(self._sysarg())
                self.take(")")
            if p.text not in ("$vt", "$temperature", "$simparam", "$mfactor"):
                raise VAError(f"line {p.line}: unsupported system function {p.text}")
            return SysCall(p.text, args)
        if p.kind == "id":
            if p.text in CONSTANTS:
                return Num(CONSTANTS[p.text])
            if self.at("("):
                self.take("(")
                if p.text == "V":
                    a = self.ident()
                    b = None
                    if self.at(","):
                        self.take(",")
                        b = self.ident()
                    self.take(")")
                    return Probe(a, b)
                if p.text == "I":
                    raise VAError(f"line {p.line}: branch-current probes I(...) are not supported")
                args = []
                if not self.at(")"):
                    args.append(self.expr())
                    while self.at(","):
                        self.take(",")
                        args.append(self.expr())
                self.take(")")
                return Call(p.text, args, p.line)
            return Name(p.text, p.line)
        raise VAError(f"line {p.line}: unexpected {p.text!r} in an expression")

    def _sysarg(self):
        if self.peek() is not None and self.peek().kind == "str":
            return self.take().text.strip('"')
        return self.expr()


def parse(src: str) -> List[Module]:
    """Parse Verilog-A source text into modules."""
    return Parser(preprocess(lex(src))).modules()


def parse_file(path) -> List[Module]:
    with open(path) as fh:
        return parse(fh.read())
