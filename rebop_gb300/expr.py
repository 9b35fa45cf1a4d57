"""Arbitrary rate expressions of the Python API (rebop src/expr.rs).

``parse`` follows the reference grammar (expr.rs:143-273, a winnow parser):

    expr   := term (ws? [+-] ws? term)*          left fold
    term   := factor (ws? [*/] ws? factor)*      left fold
    factor := atom ws? '^' ws? atom | atom       not associative
    atom   := 'exp' paren | 'max(' e ',' e ')' | 'min(' e ',' e ')'
            | variable | float | paren | '-' ws? term
    paren  := '(' ws? expr ws? ')'

with ws = spaces/tabs only where shown (no leading or trailing blanks), ASCII
identifiers ``[A-Za-z_][A-Za-z0-9_]*`` tried before numbers (so ``inf`` and
``nan`` are names), and numbers ``[+-]?(d+(.d*)?|.d+)([eE][+-]?d+)?`` where an
``e`` not followed by digits is a hard error.  ``PExpr.to_expr`` resolves
names to species indices or parameter values (expr.rs:58-109); ``Expr`` is
the resolved tree the engine compiles to device bytecode.
"""

from __future__ import annotations

import math
from dataclasses import dataclass


class ParseError(ValueError):
    pass


class _Backtrack(Exception):
    pass


class _Cut(Exception):
    pass


# --------------------------------------------------------------- trees
@dataclass(frozen=True)
class PExpr:
    op: str                 # const var neg add sub mul div pow max min exp
    value: float = 0.0
    name: str = ""
    a: "PExpr | None" = None
    b: "PExpr | None" = None

    def __str__(self) -> str:  # expr.rs:111-128
        o = self.op
        if o == "const":
            return _rust_f64(self.value)
        if o == "var":
            return self.name
        if o == "neg":
            return f"(-{self.a})"
        if o in _INFIX:
            return f"({self.a} {_INFIX[o]} {self.b})"
        if o in ("max", "min"):
            return f"{o}({self.a}, {self.b})"
        return f"exp({self.a})"

    def to_expr(self, species: dict, params: dict) -> "Expr":
        o = self.op
        if o == "const":
            return Expr("const", value=self.value)
        if o == "var":
            if self.name in species:
                return Expr("species", index=species[self.name])
            if self.name not in params:
                raise ValueError(f"Parameter {self.name} should have a value")
            return Expr("const", value=float(params[self.name]))
        a = self.a.to_expr(species, params)
        b = self.b.to_expr(species, params) if self.b is not None else None
        return Expr(o, a=a, b=b)


_INFIX = {"add": "+", "sub": "-", "mul": "*", "div": "/", "pow": "^"}
# Postfix operation codes of the engine's expression programs.
_OPS = {"const": 0, "species": 1, "neg": 2, "add": 3, "sub": 4, "mul": 5, "div": 6, "pow": 7, "max": 8,
        "min": 9, "exp": 10}


@dataclass(frozen=True)
class Expr:
    """Resolved rate expression (expr.rs:8-21)."""

    op: str                  # const species neg add sub mul div pow max min exp
    value: float = 0.0
    index: int = -1
    a: "Expr | None" = None
    b: "Expr | None" = None

    def to_program(self) -> tuple[list[int], list[float]]:
        """Postfix form for the engine (``rb_network_add_reaction_expr``): words
        ``op | arg << 8`` in evaluation order, and the constants they push."""
        code: list[int] = []
        consts: list[float] = []

        def emit(e: "Expr") -> None:
            if e.op == "const":
                code.append(_OPS["const"] | (len(consts) << 8))
                consts.append(float(e.value))
            elif e.op == "species":
                code.append(_OPS["species"] | (int(e.index) << 8))
            else:
                emit(e.a)
                if e.b is not None:
                    emit(e.b)
                code.append(_OPS[e.op])

        emit(self)
        return code, consts

    def eval(self, species) -> float:
        """Host evaluation (expr.rs:23-39), for tests."""
        o = self.op
        if o == "const":
            return self.value
        if o == "species":
            return float(species[self.index])
        x = self.a.eval(species)
        if o == "neg":
            return -x
        if o == "exp":
            try:
                return math.exp(x)
            except OverflowError:
                return math.inf
        y = self.b.eval(species)
        if o == "add":
            return x + y
        if o == "sub":
            return x - y
        if o == "mul":
            return x * y
        if o == "div":
            if y == 0.0:
                if x == 0.0 or math.isnan(x):
                    return math.nan
                return math.copysign(math.inf, x) * math.copysign(1.0, y)
            return x / y
        if o == "pow":
            return _powf(x, y)
        if o == "max":  # f64::max ignores a NaN operand
            if math.isnan(x):
                return y
            if math.isnan(y):
                return x
            return x if x >= y else y
        if o == "min":
            if math.isnan(x):
                return y
            if math.isnan(y):
                return x
            return x if x <= y else y
        raise ValueError(o)


def _powf(x: float, y: float) -> float:
    try:
        return math.pow(x, y)
    except (OverflowError, ValueError):
        if x == 0.0 and y < 0:
            return math.inf
        if math.isnan(x) or math.isnan(y):
            return math.nan
        if x < 0 and not float(y).is_integer():
            return math.nan
        return math.inf


def _rust_f64(x: float) -> str:
    """Rust's ``Display`` for f64: shortest round-trip digits, never an exponent."""
    if math.isnan(x):
        return "NaN"
    if math.isinf(x):
        return "inf" if x > 0 else "-inf"
    r = repr(float(x))
    sign = ""
    if r.startswith("-"):
        sign, r = "-", r[1:]
    if "e" in r or "E" in r:
        mant, ex = r.lower().split("e")
        ex = int(ex)
        if "." in mant:
            ip, fp = mant.split(".")
        else:
            ip, fp = mant, ""
        digits = ip + fp
        point = len(ip) + ex
        if point <= 0:
            s = "0." + "0" * (-point) + digits
        elif point >= len(digits):
            s = digits + "0" * (point - len(digits))
        else:
            s = digits[:point] + "." + digits[point:]
    else:
        s = r
    if s.endswith(".0"):
        s = s[:-2]
    s = s.rstrip("0").rstrip(".") if "." in s else s
    return sign + s


# --------------------------------------------------------------- parser
class _P:
    def __init__(self, s: str):
        self.s = s
        self.i = 0

    def peek(self, k: int = 0) -> str:
        j = self.i + k
        return self.s[j] if j < len(self.s) else ""

    def space0(self) -> None:
        while self.peek() in (" ", "\t") and self.peek():
            self.i += 1

    def lit(self, t: str) -> None:
        if not self.s.startswith(t, self.i):
            raise _Backtrack
        self.i += len(t)


def _is_alpha(c: str) -> bool:
    return ("a" <= c <= "z") or ("A" <= c <= "Z")


def _is_digit(c: str) -> bool:
    return "0" <= c <= "9" and c != ""


def _variable(p: _P) -> PExpr:
    c = p.peek()
    if not (c and (_is_alpha(c) or c == "_")):
        raise _Backtrack
    j = p.i + 1
    while j < len(p.s) and (_is_alpha(p.s[j]) or _is_digit(p.s[j]) or p.s[j] == "_"):
        j += 1
    name = p.s[p.i:j]
    p.i = j
    return PExpr("var", name=name)


def _digits(p: _P) -> int:
    j = p.i
    while _is_digit(p.peek()):
        p.i += 1
    return p.i - j


def _constant(p: _P) -> PExpr:
    start = p.i
    c = p.peek()
    if c in ("n", "N"):
        if p.s[p.i:p.i + 3].lower() != "nan":
            raise _Backtrack
        p.i += 3
        return PExpr("const", value=math.nan)
    if c in ("i", "I"):
        if p.s[p.i:p.i + 3].lower() != "inf":
            raise _Backtrack
        p.i += 3
        if p.s[p.i:p.i + 5].lower() == "inity":
            p.i += 5
        return PExpr("const", value=math.inf)
    if c in ("+", "-"):
        p.i += 1
    if _digits(p) > 0:
        if p.peek() == ".":
            p.i += 1
            _digits(p)
    elif p.peek() == "." and _is_digit(p.peek(1)):
        p.i += 1
        _digits(p)
    else:
        p.i = start
        raise _Backtrack
    if p.peek() in ("e", "E") and p.peek():
        p.i += 1
        if p.peek() in ("+", "-") and p.peek():
            p.i += 1
        if _digits(p) == 0:
            raise _Cut
    text = p.s[start:p.i]
    return PExpr("const", value=float(text))


def _alt(p: _P, *parsers):
    start = p.i
    for f in parsers:
        try:
            return f(p)
        except _Backtrack:
            p.i = start
    raise _Backtrack


def _parentheses(p: _P) -> PExpr:
    p.lit("(")
    p.space0()
    e = _expr(p)
    p.space0()
    p.lit(")")
    return e


def _pair(p: _P, name: str) -> PExpr:
    p.lit(name)
    p.lit("(")
    p.space0()
    a = _expr(p)
    p.space0()
    p.lit(",")
    p.space0()
    b = _expr(p)
    p.space0()
    p.lit(")")
    return PExpr(name, a=a, b=b)


def _exp(p: _P) -> PExpr:
    p.lit("exp")
    return PExpr("exp", a=_parentheses(p))


def _neg(p: _P) -> PExpr:
    p.lit("-")
    p.space0()
    return PExpr("neg", a=_term(p))


def _atom(p: _P) -> PExpr:
    return _alt(p, _exp, lambda q: _pair(q, "max"), lambda q: _pair(q, "min"), _variable, _constant,
                _parentheses, _neg)


def _pow(p: _P) -> PExpr:
    a = _atom(p)
    p.space0()
    p.lit("^")
    p.space0()
    b = _atom(p)
    return PExpr("pow", a=a, b=b)


def _factor(p: _P) -> PExpr:
    return _alt(p, _pow, _atom)


def _fold(p: _P, item, ops: dict) -> PExpr:
    acc = item(p)
    while True:
        save = p.i
        p.space0()
        c = p.peek()
        if c and c in ops:
            p.i += 1
            p.space0()
            try:
                rhs = item(p)
            except _Backtrack:
                p.i = save
                return acc
            acc = PExpr(ops[c], a=acc, b=rhs)
        else:
            p.i = save
            return acc


def _term(p: _P) -> PExpr:
    return _fold(p, _factor, {"*": "mul", "/": "div"})


def _expr(p: _P) -> PExpr:
    return _fold(p, _term, {"+": "add", "-": "sub"})


def parse(s: str) -> PExpr:
    """Parse a rate expression; raises :class:`ParseError` like the reference's RateParseError."""
    p = _P(s)
    try:
        e = _expr(p)
    except (_Backtrack, _Cut, RecursionError):
        raise ParseError(s) from None
    if p.i != len(s):
        raise ParseError(s)
    return e
