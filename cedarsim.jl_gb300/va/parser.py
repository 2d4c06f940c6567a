"""Verilog-A front end: lexer, `define/`include handling and a recursive-descent
parser for the compact-model subset the GPU emitter compiles.

Subset (the constructs CedarSim's VA translator lowers for compact models,
src/vasim.jl:128-180,347-412,663-875):
  module NAME(ports); port directions; `electrical` ports and internal nodes;
  parameter [real|integer] NAME = expr [from|exclude range] {, ...};
  real / integer variables (module or block scope);
  analog begin ... end with assignments, if / else, begin / end blocks,
  current contributions I(a,b) <+ expr and I(a) <+ expr; one voltage-contributed
  branch V(a,b) <+ expr (a branch-current unknown; I(a,b) probes it);
  expressions: numbers with SI scale factors, + - * / ** unary - + !, comparisons,
  && || and ?:; V(a,b) / V(a) probes; exp ln log sqrt pow abs min max tanh sinh
  cosh sin cos tan atan atan2 asin acos hypot floor ceil limexp; ddt(expr) (additive
  in a contribution); ddx(expr, V(n)) / ddx(expr, V(a,b)); $vt, $vt(T),
  $temperature, $simparam("gmin"[, default]), $mfactor.
Also: `define with arguments and `ifdef; case; for / while / repeat loops
(capped at LOOP_CAP passes); analog functions with input, output and inout
arguments; @(initial_step)-style event blocks; $param_given; white_noise /
flicker_noise; $limit; display tasks.  Internal nodes (`electrical` names that
are not ports) become extra device unknowns.  More than one voltage-contributed
branch, noise sources inside loops and other constructs outside the subset
raise VAError with the line number.
"""
from __future__ import annotations

import pathlib
import re
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple


class VAError(Exception):
    pass


# ------------------------------------------------------------------ lexer
_TOKEN = re.compile(r"""
    (?P<ws>[ \t\r\n\x00]+)
  | (?P<lcom>//[^\n]*)
  | (?P<bcom>/\*.*?\*/)
  | (?P<num>(\d+\.\d*|\.\d+|\d+)([eE][+-]?\d+)?[TGMKkmunpfa]?)
  | (?P<sys>\$[A-Za-z_][A-Za-z_0-9]*)
  | (?P<dir>`[A-Za-z_][A-Za-z_0-9]*)
  | (?P<id>[A-Za-z_][A-Za-z_0-9]*)
  | (?P<str>"(?:[^"\\\n]|\\.)*")
  | (?P<op><\+|\*\*|<=|>=|==|!=|&&|\|\||[-+*/<>!?:;,()\[\]=@{}.])
""", re.S | re.X)

SCALE = {"T": 1e12, "G": 1e9, "M": 1e6, "K": 1e3, "k": 1e3, "m": 1e-3, "u": 1e-6, "n": 1e-9, "p": 1e-12,
         "f": 1e-15, "a": 1e-18}

# system tasks that only print, stop the simulator or advise its step control
# ($bound_step, $discontinuity; the engines' LTE control and breakpoints stand
# in for them): compiled to nothing
DISPLAY_TASKS = ("$strobe", "$display", "$write", "$monitor", "$debug", "$warning", "$info", "$error", "$fatal",
                 "$finish", "$stop", "$bound_step", "$discontinuity")

# constants of the standard constants.vams header (physical constants, SI)
CONSTANTS = {"M_PI": 3.14159265358979323846, "M_TWO_PI": 6.28318530717958647652,
             "M_PI_2": 1.57079632679489661923, "M_E": 2.7182818284590452354,
             "M_LN2": 0.69314718055994530942, "M_LN10": 2.30258509299404568402,
             "M_SQRT2": 1.41421356237309504880, "M_1_PI": 0.31830988618379067154,
             "P_Q": 1.602176634e-19, "P_K": 1.380649e-23, "P_CELSIUS0": 273.15,
             "P_EPS0": 8.8541878128e-12, "P_H": 6.62607015e-34, "P_C": 299792458.0,
             "P_U0": 1.25663706212e-6}


@dataclass
class Tok:
    kind: str
    text: str
    line: int
    adj: bool = False      # no whitespace or comment since the previous token


def lex(src: str) -> List[Tok]:
    out: List[Tok] = []
    pos, line, pending, last_end = 0, 1, 0, -1
    while pos < len(src):
        m = _TOKEN.match(src, pos)
        if not m:
            raise VAError(f"line {line}: unexpected character {src[pos]!r}")
        kind = m.lastgroup
        text = m.group(kind)
        if kind not in ("ws", "lcom", "bcom"):
            out.append(Tok(kind, text, line, m.start() == last_end))
            last_end = m.end()
        # a joined continuation (\x00) keeps the tokens on one line; its newline
        # is counted at the next real line break
        pending += text.count("\x00")
        if "\n" in text:
            line += text.count("\n") + pending
            pending = 0
        pos = m.end()
    return out


def _const_tok(t: Tok) -> Tok:
    """`P_Q and the other constants.vams macros as number tokens."""
    return Tok("num", repr(CONSTANTS[t.text[1:]]), t.line)


def _join_continuations(src: str) -> str:
    """A backslash at the end of a line continues a `define body on the next
    line; the newline is kept out of the body but counted for line numbers."""
    src = re.sub(r"\\[ \t]*\r?\n", " \x00", src)
    # attribute instances (* name = "..." *) describe items for tools; they carry
    # no semantics here
    return re.sub(r"\(\*[^\n]*?\*\)", " ", src)


def preprocess(toks: List[Tok], base_dir=None) -> List[Tok]:
    """`define NAME body and `define NAME(a, b) body with `NAME / `NAME(x, y)
    expansion (nested, up to a depth limit), `undef, `ifdef / `ifndef / `elsif /
    `else / `endif, and `include of the standard headers (disciplines.vams /
    constants.vams: their names are built in).  Other directives are errors."""
    macros: Dict[str, Tuple[Optional[List[str]], List[Tok]]] = {}
    out: List[Tok] = []
    n_includes = 0
    # conditional stack: (this branch active, some branch already taken, parent active)
    cond: List[Tuple[bool, bool, bool]] = []

    def active() -> bool:
        return not cond or cond[-1][0]

    def expand(stream: List[Tok], depth: int) -> List[Tok]:
        if depth > 32:
            raise VAError("macro expansion too deep (recursive `define?)")
        res: List[Tok] = []
        k = 0
        while k < len(stream):
            t = stream[k]
            if t.kind == "dir" and t.text[1:] in macros:
                params, body = macros[t.text[1:]]
                k += 1
                if params is None:
                    res.extend(expand([Tok(b.kind, b.text, t.line) for b in body], depth + 1))
                    continue
                if k >= len(stream) or stream[k].text != "(":
                    raise VAError(f"line {t.line}: macro {t.text} needs arguments")
                args: List[List[Tok]] = [[]]
                level = 0
                k += 1
                while k < len(stream):
                    a = stream[k]
                    if a.text == "(" and a.kind == "op":
                        level += 1
                    elif a.text == ")" and a.kind == "op":
                        if level == 0:
                            break
                        level -= 1
                    elif a.text == "," and a.kind == "op" and level == 0:
                        args.append([])
                        k += 1
                        continue
                    args[-1].append(a)
                    k += 1
                if k >= len(stream):
                    raise VAError(f"line {t.line}: unterminated arguments of macro {t.text}")
                k += 1
                if len(args) != len(params) and not (len(params) == 0 and args == [[]]):
                    raise VAError(f"line {t.line}: macro {t.text} takes {len(params)} arguments, got {len(args)}")
                sub = {p: expand(a, depth + 1) for p, a in zip(params, args)}
                body_t: List[Tok] = []
                for b in body:
                    if b.kind == "id" and b.text in sub:
                        body_t.extend(Tok(x.kind, x.text, t.line) for x in sub[b.text])
                    else:
                        body_t.append(Tok(b.kind, b.text, t.line))
                res.extend(expand(body_t, depth + 1))
                continue
            if t.kind == "dir" and t.text[1:] in CONSTANTS:
                res.append(_const_tok(t))
            else:
                res.append(t)
            k += 1
        return res

    i = 0
    while i < len(toks):
        t = toks[i]
        if t.kind == "dir":
            name = t.text[1:]
            if name in ("ifdef", "ifndef", "elsif"):
                if i + 1 >= len(toks) or toks[i + 1].kind != "id":
                    raise VAError(f"line {t.line}: `{name} needs a macro name")
                defined = toks[i + 1].text in macros
                if name == "elsif":
                    if not cond:
                        raise VAError(f"line {t.line}: `elsif without `ifdef")
                    _, taken, parent = cond.pop()
                    take = parent and not taken and defined
                    cond.append((take, taken or take, parent))
                else:
                    parent = active()
                    take = parent and (defined if name == "ifdef" else not defined)
                    cond.append((take, take, parent))
                i += 2
                continue
            if name == "else":
                if not cond:
                    raise VAError(f"line {t.line}: `else without `ifdef")
                _, taken, parent = cond.pop()
                cond.append((parent and not taken, True, parent))
                i += 1
                continue
            if name == "endif":
                if not cond:
                    raise VAError(f"line {t.line}: `endif without `ifdef")
                cond.pop()
                i += 1
                continue
            if not active():
                i += 1
                continue
            if name == "include":
                if i + 1 >= len(toks) or toks[i + 1].kind != "str":
                    raise VAError(f"line {t.line}: `include needs a file name")
                fname = toks[i + 1].text.strip('"')
                if fname in ("disciplines.vams", "constants.vams", "discipline.h", "constants.h"):
                    i += 2
                    continue
                # another file: relative to the including file's directory, its
                # tokens spliced in place of the directive
                if base_dir is None:
                    raise VAError(f"line {t.line}: `include \"{fname}\" needs the source's directory (parse_file)")
                path = pathlib.Path(base_dir) / fname
                if not path.is_file():
                    raise VAError(f"line {t.line}: `include \"{fname}\": no such file in {base_dir}")
                n_includes += 1
                if n_includes > 256:
                    raise VAError("more than 256 `include directives (recursive include?)")
                toks = toks[:i] + lex(_join_continuations(path.read_text())) + toks[i + 2:]
                continue
            if name == "define":
                if i + 1 >= len(toks) or toks[i + 1].kind != "id":
                    raise VAError(f"line {t.line}: `define needs a name")
                mname, mline = toks[i + 1].text, toks[i + 1].line
                j = i + 2
                params = None
                # a parameter list opens right after the name, with no space between
                if j < len(toks) and toks[j].line == mline and toks[j].text == "(" and toks[j].adj:
                    params = []
                    j += 1
                    while j < len(toks) and toks[j].text != ")":
                        if toks[j].kind == "id":
                            params.append(toks[j].text)
                        j += 1
                    j += 1
                body = []
                while j < len(toks) and toks[j].line == mline:
                    body.append(toks[j])
                    j += 1
                macros[mname] = (params, body)
                i = j
                continue
            if name == "undef":
                macros.pop(toks[i + 1].text, None)
                i += 2
                continue
            if name in CONSTANTS and name not in macros:
                if active():
                    out.append(_const_tok(t))
                i += 1
                continue
            if name in macros:
                # collect the macro call (with its argument list) and expand it
                j = i + 1
                if macros[name][0] is not None and j < len(toks) and toks[j].text == "(":
                    level = 0
                    while j < len(toks):
                        if toks[j].text == "(":
                            level += 1
                        elif toks[j].text == ")":
                            level -= 1
                            if level == 0:
                                j += 1
                                break
                        j += 1
                out.extend(expand(toks[i:j], 0))
                i = j
                continue
            raise VAError(f"line {t.line}: unknown directive {t.text}")
        if active():
            out.append(t)
        i += 1
    if cond:
        raise VAError("`ifdef without `endif")
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
class Probe:            # V(a), V(a, b), or the branch current I(a, b)
    a: str
    b: Optional[str]
    kind: str = "V"


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
class Contrib:          # I(a[, b]) <+ expr  or  V(a[, b]) <+ expr
    a: str
    b: Optional[str]
    expr: object
    line: int = 0
    kind: str = "I"


@dataclass
class If:
    c: object
    then: list
    other: list


# loops run at most this many times; past it they stop (and the model's
# results are whatever the last pass left), so no device code can spin
LOOP_CAP = 100000


@dataclass
class Loop:             # for (init; cond; step) body  /  while (cond) body  /  repeat (count) body
    init: list
    cond: object
    step: list
    body: list
    count: object = None


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
    functions: Dict[str, "Function"] = field(default_factory=dict)


@dataclass
class Function:         # analog function: arguments in order, result in the variable NAME
    name: str
    type: str
    inputs: List[str]              # every argument, in declaration order
    local: Dict[str, str]          # arguments, locals and the result variable -> type
    body: list
    outputs: List[str] = field(default_factory=list)   # arguments declared output / inout


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
        functions: Dict[str, Function] = {}
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
                if self.at("function"):
                    f = self._function()
                    if f.name in functions:
                        raise VAError(f"line {p.line}: analog function {f.name} defined twice")
                    functions[f.name] = f
                    continue
                body.extend(self.statement(variables))
            else:
                raise VAError(f"line {p.line}: unsupported module item {p.text!r}")
        self.take("endmodule")
        missing = [q for q in ports if q not in electrical]
        if missing:
            raise VAError(f"module {name}: ports without a discipline: {missing}")
        return Module(name, ports, params, variables, body, internals, functions)

    def _function(self) -> "Function":
        """analog function [real|integer] NAME; input a, b; real a, b, t; stmt endfunction"""
        self.take("function")
        ftype = "real"
        if self.at("real") or self.at("integer"):
            ftype = self.take().text
        name = self.ident()
        self.take(";")
        inputs: List[str] = []
        outputs: List[str] = []
        local: Dict[str, str] = {}
        while True:
            q = self.peek()
            if q is None:
                raise VAError(f"analog function {name}: missing endfunction")
            if q.text in ("input", "output", "inout"):
                self.take()
                names = self._idlist()
                inputs += names
                if q.text != "input":
                    outputs += names
            elif q.text in ("real", "integer"):
                self.take()
                for n in self._idlist():
                    local[n] = q.text
            else:
                break
        for a in inputs:
            local.setdefault(a, "real")
        local[name] = ftype                 # the return value is the variable named after the function
        body = self.statement(local)
        self.take("endfunction")
        return Function(name, ftype, inputs, local, body, outputs)

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
        if p.kind == "sys" and p.text in DISPLAY_TASKS:
            # $strobe / $display / ... print from the simulator; no effect on the
            # device equations, so they compile to nothing
            self.take()
            if self.at("("):
                self.take("(")
                if not self.at(")"):
                    self._sysarg()
                    while self.at(","):
                        self.take(",")
                        self._sysarg()
                self.take(")")
            self.take(";")
            return []
        if p.text == "@" and p.kind == "op":
            # @(initial_step) / @(initial_model) / @(initial_instance) blocks
            # compute values from parameters: evaluated at every call, which
            # gives the same values; @(final_step) blocks only report, dropped
            self.take()
            self.take("(")
            ev = self.ident()
            if self.at("("):            # initial_step("tran") and the like
                self.take("(")
                while not self.at(")"):
                    self.take()
                self.take(")")
            self.take(")")
            if ev not in ("initial_step", "initial_model", "initial_instance", "final_step"):
                raise VAError(f"line {p.line}: unsupported event @({ev})")
            body = self.statement(variables)
            return [] if ev == "final_step" else body
        if p.kind == "id" and p.text in ("for", "while", "repeat"):
            self.take()
            self.take("(")
            if p.text == "for":
                init = self._simple_assign(variables)
                self.take(";")
                cond = self.expr()
                self.take(";")
                step = self._simple_assign(variables)
                self.take(")")
                return [Loop(init, cond, step, self.statement(variables))]
            e = self.expr()
            self.take(")")
            if p.text == "while":
                return [Loop([], e, [], self.statement(variables))]
            return [Loop([], None, [], self.statement(variables), count=e)]
        if p.text == "case" and p.kind == "id":
            # case (x) v1, v2: s; ... default: s; endcase -> if / else chain
            self.take()
            self.take("(")
            sel = self.expr()
            self.take(")")
            arms: List[Tuple[Optional[list], list]] = []
            while not self.at("endcase"):
                if self.peek() is None:
                    raise VAError(f"line {p.line}: missing endcase")
                if self.at("default"):
                    self.take()
                    if self.at(":"):
                        self.take(":")
                    arms.append((None, self.statement(variables)))
                    continue
                labels = [self.expr()]
                while self.at(","):
                    self.take(",")
                    labels.append(self.expr())
                self.take(":")
                arms.append((labels, self.statement(variables)))
            self.take("endcase")
            default = next((s for lab, s in arms if lab is None), [])
            out: list = default
            for labels, body in reversed([a for a in arms if a[0] is not None]):
                c = None
                for lab in labels:
                    t = Bin("==", sel, lab)
                    c = t if c is None else Bin("||", c, t)
                out = [If(c, body, out)]
            return out
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
            return [Contrib(a, b, e, p.line, kind)]
        if p.kind == "id":
            name = self.take().text
            self.take("=")
            e = self.expr()
            self.take(";")
            return [Assign(name, e, p.line)]
        raise VAError(f"line {p.line}: unsupported statement starting with {p.text!r}")

    def _simple_assign(self, variables) -> list:
        """name = expr (the init and step of a for loop, without a semicolon)"""
        q = self.peek()
        name = self.ident()
        self.take("=")
        return [Assign(name, self.expr(), q.line)]

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
            if p.text == "$limit":
                # $limit(x, "limiter", ...): Newton-step limiting, which a simulator
                # may leave out (the engines' Newton has its own damping): the
                # value is x itself
                if not args or isinstance(args[0], str):
                    raise VAError(f"line {p.line}: $limit needs an expression")
                return args[0]
            if p.text not in ("$vt", "$temperature", "$simparam", "$mfactor", "$param_given", "$given"):
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
                    # branch-current probe: the current of a voltage-contributed branch
                    a = self.ident()
                    b = None
                    if self.at(","):
                        self.take(",")
                        b = self.ident()
                    self.take(")")
                    return Probe(a, b, "I")
                # noise sources take a name string after their power arguments
                arg = self._sysarg if p.text in ("white_noise", "flicker_noise") else self.expr
                args = []
                if not self.at(")"):
                    args.append(arg())
                    while self.at(","):
                        self.take(",")
                        args.append(arg())
                self.take(")")
                return Call(p.text, args, p.line)
            return Name(p.text, p.line)
        raise VAError(f"line {p.line}: unexpected {p.text!r} in an expression")

    def _sysarg(self):
        if self.peek() is not None and self.peek().kind == "str":
            return self.take().text.strip('"')
        return self.expr()


def parse(src: str, base_dir=None) -> List[Module]:
    """Parse Verilog-A source text into modules (`include files relative to base_dir)."""
    return Parser(preprocess(lex(_join_continuations(src)), base_dir)).modules()


def parse_file(path) -> List[Module]:
    path = pathlib.Path(path)
    return parse(path.read_text(), path.parent)
