"""Executes the reference's Fortran-77 source text (after its m4 macros) in Python.

The reference path is Fortran 77 run through m4 (fortran/*.m4), and neither
machine this project builds on has a Fortran compiler or m4.  This module is a
small translator for the subset of fixed-form Fortran 77 those files use
(SUBROUTINE / REAL FUNCTION units, INTEGER / DOUBLE PRECISION declarations with
explicit bounds, DO loops, block and logical IF, assignment, ABS / EXP / LOG /
DBLE intrinsics).  It turns each program unit into a Python function whose
arithmetic follows Fortran's rules as gfortran applies them on a machine
without fused multiply-add:

* operators bind as in the standard (** > * / > unary and binary + - >
  relational), equal-precedence operators associate left to right, ** right
  to left, and parentheses are honoured;
* un-suffixed real literals are REAL*4 values (correctly rounded from the
  decimal text); REAL*4 (op) REAL*4 is computed in single precision and mixed
  REAL*4 (op) REAL*8 in double, as gfortran folds and evaluates them;
* x**n with an integer n is a product of n factors;
* EXP and LOG call the C library (Python's math module), like gfortran's
  intrinsics on glibc.

The m4 layer is reduced to the three macros the files use: ``define(REAL,
double precision)`` and SAMRAI's array-bound macros ``CELL2d(f,l,g)`` ->
``f0-g:l0+g,f1-g:l1+g`` and ``CELL2dVECG(f,l,g)`` -> ``f0-g0:l0+g0,f1-g1:l1+g1``
(SAMRAI pdat_m4arrdim2d.i).

It is test infrastructure: tests/golden/make_golden.py uses it to turn the
reference's own source into golden input/output vectors for the C++ oracle.
"""
from __future__ import annotations

import math
import re
from fractions import Fraction

import numpy as np

# --------------------------------------------------------------------------
# m4 subset and fixed-form source handling
# --------------------------------------------------------------------------


def _m4(text: str) -> str:
    out = []
    for line in text.splitlines():
        if line.startswith("define(") or line.startswith("include("):
            continue
        line = re.sub(
            r"CELL2dVECG\((\w+),(\w+),(\w+)\)",
            lambda m: "{a}0-{g}0:{b}0+{g}0,{a}1-{g}1:{b}1+{g}1".format(a=m[1], b=m[2], g=m[3]),
            line,
        )
        line = re.sub(
            r"CELL2d\((\w+),(\w+),(\w+)\)",
            lambda m: "{a}0-{g}:{b}0+{g},{a}1-{g}:{b}1+{g}".format(a=m[1], b=m[2], g=m[3]),
            line,
        )
        line = re.sub(r"\bREAL\b", "double precision", line)
        out.append(line)
    return "\n".join(out)


def _statements(text: str) -> list[str]:
    stmts: list[str] = []
    for raw in text.splitlines():
        if not raw.strip():
            continue
        if raw[0] in "cC*!":
            continue
        # No source line of the reference exceeds column 72 before m4
        # expansion; the expanded array declarations do, and the reference
        # build compiles them, so lines are taken whole.
        line = raw.expandtabs()
        label_and_cont = line[:6]
        body = line[6:]
        if len(label_and_cont) == 6 and label_and_cont[5] not in " 0":
            stmts[-1] += " " + body.strip()
        else:
            stmts.append(body.strip())
    return [s.lower() for s in stmts if s.strip()]


# --------------------------------------------------------------------------
# expressions
# --------------------------------------------------------------------------

_TOKEN = re.compile(
    r"\s*(?:(?P<real>(?:\d+\.\d*|\.\d+)(?:e[+-]?\d+)?|\d+e[+-]?\d+)"
    r"|(?P<int>\d+)"
    r"|(?P<dotop>\.(?:lt|le|gt|ge|eq|ne|and|or|not)\.)"
    r"|(?P<name>[a-z_][a-z0-9_]*)"
    r"|(?P<op>\*\*|[-+*/(),:=]))"
)


def _tokens(s: str):
    pos, out = 0, []
    s = s.strip()
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m or m.end() == pos:
            raise SyntaxError(f"cannot tokenize {s[pos:]!r}")
        pos = m.end()
        kind = m.lastgroup
        out.append((kind, m.group(kind)))
    return out


def f32_literal(text: str) -> np.float32:
    """Correctly rounded REAL*4 value of a decimal literal."""
    x = Fraction(text)
    c = np.float32(float(x))
    best = None
    for cand in (np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf))):
        err = abs(Fraction(float(cand)) - x)
        key = (err, int(np.frombuffer(np.float32(cand).tobytes(), np.uint32)[0]) & 1)
        if best is None or key < best[0]:
            best = (key, cand)
    return np.float32(best[1])


class _Expr:
    """Pratt parser emitting a fully parenthesised Python expression."""

    PREC = {".or.": 1, ".and.": 2, ".lt.": 4, ".le.": 4, ".gt.": 4, ".ge.": 4, ".eq.": 4,
            ".ne.": 4, "+": 5, "-": 5, "*": 6, "/": 6, "**": 8}
    PYOP = {".or.": "or", ".and.": "and", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">=",
            ".eq.": "==", ".ne.": "!=", "+": "+", "-": "-", "*": "*", "/": "/"}

    def __init__(self, unit, toks):
        self.u, self.t, self.i = unit, toks, 0

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise SyntaxError(f"expected {val}, got {tok}")
        self.i += 1
        return tok

    def parse(self, minp=0):
        kind, val = self.peek()
        if val in ("-", "+"):
            self.take()
            operand = self.parse(6)  # unary minus binds looser than * and /
            left = f"(-{operand})" if val == "-" else operand
        elif val == ".not.":
            self.take()
            left = f"(not {self.parse(3)})"
        else:
            left = self.primary()
        while True:
            kind, val = self.peek()
            if val not in self.PREC:
                break
            p = self.PREC[val]
            if p < minp:
                break
            self.take()
            if val == "**":
                right = self.parse(p)  # right associative
                left = f"_pow({left}, {right})"
            else:
                right = self.parse(p + 1)
                if val == "/":
                    left = f"_div({left}, {right})"
                else:
                    left = f"({left} {self.PYOP[val]} {right})"
        return left

    def args(self):
        out = []
        self.take("(")
        if self.peek()[1] != ")":
            out.append(self.parse())
            while self.peek()[1] == ",":
                self.take()
                out.append(self.parse())
        self.take(")")
        return out

    def primary(self):
        kind, val = self.take()
        if kind == "real":
            return self.u.const(val)
        if kind == "int":
            return val
        if val == "(":
            e = self.parse()
            self.take(")")
            return f"({e})"
        if kind == "name":
            if self.peek()[1] == "(":
                a = self.args()
                if val in self.u.arrays:
                    idx = ", ".join(f"({x}) - {val}__lb[{n}]" for n, x in enumerate(a))
                    return f"{val}[{idx}]"
                if val in ("abs", "exp", "log", "dble"):
                    return f"_{val}({', '.join(a)})"
                return f"_fn_{val}({', '.join(a)})"
            return val
        raise SyntaxError(f"unexpected token {val!r}")


def _pow(a, n):
    if isinstance(n, int) and n >= 1:
        r = a
        for _ in range(n - 1):
            r = r * a
        return r
    raise NotImplementedError("only positive integer powers occur in the reference")


def _div(a, b):
    if isinstance(a, int) and isinstance(b, int):
        q = abs(a) // abs(b)
        return q if (a >= 0) == (b >= 0) else -q
    return a / b


def _abs(x):
    return abs(x) if isinstance(x, int) else np.abs(x)


def _exp(x):
    return np.float64(math.exp(float(x)))


def _log(x):
    return np.float64(math.log(float(x)))


def _dble(x):
    return np.float64(x)


# --------------------------------------------------------------------------
# program units
# --------------------------------------------------------------------------


class _Unit:
    def __init__(self, header: str):
        m = re.match(r"(subroutine|double precision function)\s+(\w+)\s*\((.*)\)", header)
        if not m:
            raise SyntaxError(header)
        self.is_function = m[1] != "subroutine"
        self.name = m[2]
        self.params = [p.strip() for p in m[3].split(",") if p.strip()]
        self.types: dict[str, str] = {}
        self.arrays: dict[str, list[str]] = {}
        self.consts: list[np.float32] = []
        self.body: list[str] = []
        self.indent = 1
        self.watch: str | None = None

    def const(self, text):
        self.consts.append(f32_literal(text))
        return f"_K[{len(self.consts) - 1}]"

    def expr(self, text):
        return _Expr(self, _tokens(text)).parse()

    def declare(self, typ, rest):
        # split on commas at depth 0
        depth, cur, items = 0, "", []
        for ch in rest:
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            if ch == "," and depth == 0:
                items.append(cur)
                cur = ""
            else:
                cur += ch
        items.append(cur)
        for it in items:
            it = it.strip()
            m = re.match(r"(\w+)\s*(?:\((.*)\))?$", it)
            name, dims = m[1], m[2]
            self.types[name] = typ
            if dims:
                self.arrays[name] = [d.strip() for d in dims.split(",")]

    def emit(self, line):
        self.body.append("    " * self.indent + line)

    def statement(self, s):
        if s == "implicit none":
            return
        m = re.match(r"(integer|double precision)\s+(.*)", s)
        if m and not re.match(r"double precision function", s):
            self.declare(m[1], m[2])
            return
        m = re.match(r"do\s+(\w+)\s*=\s*(.*)$", s)
        if m:
            lo, hi = _split_top(m[2])
            self.emit(f"for {m[1]} in range(int({self.expr(lo)}), int({self.expr(hi)}) + 1):")
            self.indent += 1
            self.emit("pass")
            return
        if s in ("end do", "enddo"):
            self.indent -= 1
            return
        m = re.match(r"if\s*\((.*)\)\s*then$", s)
        if m:
            self.emit(f"if {self._cond(m[1])}:")
            self.indent += 1
            self.emit("pass")
            return
        m = re.match(r"else\s*if\s*\((.*)\)\s*then$", s)
        if m:
            self.indent -= 1
            self.emit(f"elif {self._cond(m[1])}:")
            self.indent += 1
            self.emit("pass")
            return
        if s == "else":
            self.indent -= 1
            self.emit("else:")
            self.indent += 1
            self.emit("pass")
            return
        if s in ("end if", "endif"):
            self.indent -= 1
            return
        if s.startswith("if"):
            cond, rest = _split_logical_if(s)
            self.emit(f"if {self._cond(cond)}:")
            self.indent += 1
            self.statement(rest)
            self.indent -= 1
            return
        if s == "return":
            self.emit(f"return {self.name}__result" if self.is_function else "return")
            return
        m = re.match(r"([a-z_]\w*)\s*(\(.*?\))?\s*=(?!=)\s*(.*)$", s)
        if m:
            name, idx, rhs = m[1], m[2], m[3]
            value = self.expr(rhs)
            typ = "double precision" if (self.is_function and name == self.name) else self.types.get(name)
            conv = "_int" if typ == "integer" else "_f64"
            if idx:
                ex = _Expr(self, _tokens(idx))
                args = ex.args()
                target = f"{name}[" + ", ".join(f"({x}) - {name}__lb[{n}]" for n, x in enumerate(args)) + "]"
            elif self.is_function and name == self.name:
                target = f"{name}__result"
            else:
                target = name
            self.emit(f"{target} = {conv}({value})")
            return
        raise SyntaxError(f"unsupported statement: {s!r}")

    def _cond(self, text):
        py = self.expr(text)
        if self.watch and re.search(rf"\b{self.watch}\b", text):
            self.emit(f"_watch_hook(locals())")
        return py

    def source(self):
        lines = [f"def {self.name}({', '.join(self.params)}):"]
        # Scalar dummies take their declared kind (Python floats are weakly
        # typed in numpy arithmetic; a REAL*8 dummy must be a float64).
        for prm in self.params:
            if prm in self.arrays:
                continue
            if self.types.get(prm) == "double precision":
                lines.append(f"    {prm} = _f64({prm})")
            elif self.types.get(prm) == "integer":
                lines.append(f"    {prm} = _int({prm})")
        for arr, dims in self.arrays.items():
            lbs = []
            for d in dims:
                lo = d.split(":")[0] if ":" in d else "1"
                lbs.append(f"int({self.expr(lo)})")
            lines.append(f"    {arr}__lb = ({', '.join(lbs)},)")
        for arr, dims in self.arrays.items():
            if arr in self.params:
                continue
            ext = []
            for d in dims:
                lo, hi = d.split(":") if ":" in d else ("1", d)
                ext.append(f"int({self.expr(hi)}) - int({self.expr(lo)}) + 1")
            dt = "np.int64" if self.types.get(arr) == "integer" else "np.float64"
            lines.append(f"    {arr} = np.zeros(({', '.join(ext)},), dtype={dt})")
        if self.is_function:
            lines.append(f"    {self.name}__result = _f64(0)")
        lines.extend(self.body)
        if self.is_function:
            lines.append(f"    return {self.name}__result")
        return "\n".join(lines)


def _split_top(text):
    depth = 0
    for n, ch in enumerate(text):
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "," and depth == 0:
            return text[:n], text[n + 1:]
    raise SyntaxError(text)


def _split_logical_if(s):
    assert s.startswith("if")
    n = s.index("(")
    depth = 0
    for k in range(n, len(s)):
        if s[k] == "(":
            depth += 1
        elif s[k] == ")":
            depth -= 1
            if depth == 0:
                return s[n + 1:k], s[k + 1:].strip()
    raise SyntaxError(s)


def _int(x):
    return int(x)


def _f64(x):
    return np.float64(x)


def load(path: str, watch: str | None = None) -> dict:
    """Translate every program unit of one .m4 file; returns name -> callable.

    ``watch`` names a variable: every IF condition that reads it first calls
    ``_watch_hook(locals())``; the caller sets ``ns["_hooks"]["fn"]`` so that internal decisions such as the hybrid switch can be
    recorded without editing the source.
    """
    with open(path) as fh:
        stmts = _statements(_m4(fh.read()))
    units, cur = [], None
    for s in stmts:
        if cur is None:
            cur = _Unit(s)
            cur.watch = watch
            continue
        if s == "end":
            units.append(cur)
            cur = None
            continue
        cur.statement(s)
    hooks: dict = {"fn": None}

    def _watch_hook(loc):
        if hooks["fn"] is not None:
            hooks["fn"](loc)

    ns: dict = {"_pow": _pow, "_div": _div, "_abs": _abs, "_exp": _exp, "_log": _log,
                "_dble": _dble, "_int": _int, "_f64": _f64, "np": np,
                "_watch_hook": _watch_hook, "_hooks": hooks}
    for u in units:
        ns_local = dict(ns)
        ns_local["_K"] = u.consts
        src = u.source()
        code = compile(src, f"<{path}:{u.name}>", "exec")
        exec(code, ns_local)
        ns[u.name] = ns_local[u.name]
        ns[f"_fn_{u.name}"] = ns_local[u.name]
        ns[f"__src_{u.name}"] = src
    # user functions are resolved through the shared namespace at call time
    for u in units:
        ns[u.name].__globals__.update({f"_fn_{v.name}": ns[v.name] for v in units})
    return ns
