"""A Fortran 90 subset interpreter: runs the reference's own source files.

Test infrastructure only (the oracle side of the parity tests).  The
reference is Fortran 90 + MPI and no Fortran compiler exists on the machines
this project is built and measured on, so this module executes the
reference's source text itself -- program run (src/run.f90) with the modules
it uses -- on small grids, to produce golden vectors that come from the
reference's statements rather than from a restatement of them.

Semantics modelled (those of gfortran -O3 on x86-64 without FMA, i.e.
without floating-point contraction):
- default REAL is IEEE binary32 and default COMPLEX two of them; the FP64
  build (-fdefault-real-8 -fdefault-double-8) makes both binary64;
- every arithmetic operation rounds once, in the kind of its operands, and
  expressions are evaluated left to right as parsed (no reassociation);
- INTEGER op REAL converts the integer; REAL op COMPLEX is componentwise (the
  lowering of a product or quotient with an operand whose imaginary part is
  known to be zero); COMPLEX * COMPLEX is (ac - bd) + i(ad + bc);
- integer powers are repeated multiplications (x**2 = x*x, x**4 = (x*x)**2);
- ABS of a complex is hypot (libm cabs), SUM accumulates sequentially in
  array element order.

MPI is emulated for a process grid of virtual ranks run as threads of one
Python process (mailboxes for the point-to-point calls, barriers for the
collectives); file I/O (unformatted sequential records, list-directed and
simple formatted writes) goes to a working directory.  Only the constructs
the reference uses are supported; anything else raises FortranError.
"""
from __future__ import annotations

import math
import os
import re
import struct
import threading

import numpy as np


class FortranError(Exception):
    pass


class _Stop(Exception):
    pass


class _Return(Exception):
    pass


class _Exit(Exception):
    pass


class _Cycle(Exception):
    pass


# ----------------------------------------------------------------- values --
class Cx:
    """A complex value (scalar or array) held as its two real parts."""
    __slots__ = ("re", "im")

    def __init__(self, re_, im_):
        self.re = re_
        self.im = im_

    def __repr__(self):
        return f"({self.re},{self.im})"


class FArr:
    """An array variable: numpy data (Fortran subscripts in order) and lower bounds."""
    __slots__ = ("data", "lb")

    def __init__(self, data, lb):
        self.data = data
        self.lb = tuple(lb)


def _is_int(v):
    return isinstance(v, (int, np.integer)) and not isinstance(v, (bool, np.bool_))


def _rdt(kind):
    return np.float32 if kind == 4 else np.float64


def _cdt(kind):
    return np.complex64 if kind == 4 else np.complex128


def _kind_of_real(v):
    dt = v.dtype if isinstance(v, (np.ndarray, np.generic)) else None
    return 8 if dt == np.float64 else 4


def _cx_from_storage(v):
    """Storage value (numpy complex scalar or array) -> Cx."""
    rt = np.float32 if v.dtype == np.complex64 else np.float64
    if isinstance(v, np.ndarray):
        return Cx(v.real.astype(rt), v.imag.astype(rt))
    return Cx(rt(v.real), rt(v.imag))


def _to_storage(v, base, kind):
    """Convert a value to the representation stored for (base, kind)."""
    if base == "integer":
        if isinstance(v, np.ndarray):
            return v.astype(np.int64)
        if isinstance(v, (float, np.floating)):
            return int(v)   # truncation toward zero
        return int(v)
    if base == "real":
        if isinstance(v, Cx):
            v = v.re
        if isinstance(v, np.ndarray):
            return v.astype(_rdt(kind))
        return _rdt(kind)(v)
    if base == "complex":
        ct, rt = _cdt(kind), _rdt(kind)
        if isinstance(v, Cx):
            if isinstance(v.re, np.ndarray) or isinstance(v.im, np.ndarray):
                re_ = np.asarray(v.re, dtype=rt)
                im_ = np.asarray(v.im, dtype=rt)
                out = np.empty(np.broadcast(re_, im_).shape, dtype=ct)
                out.real = re_
                out.imag = im_
                return out
            return ct(complex(rt(v.re), rt(v.im)))
        if isinstance(v, np.ndarray):
            out = np.zeros(v.shape, dtype=ct)
            out.real = v.astype(rt)
            return out
        return ct(complex(rt(v), 0.0))
    if base == "logical":
        if isinstance(v, np.ndarray):
            return v.astype(bool)
        return bool(v)
    if base == "character":
        return str(v)
    raise FortranError(f"cannot store into type {base}")


def _as_real(v, kind):
    if _is_int(v):
        return _rdt(kind)(v)
    if isinstance(v, np.ndarray) and v.dtype.kind in "iu":
        return v.astype(_rdt(kind))
    return v


def _num_kind(v):
    """('i'|'r'|'c'|'l'|'s', kind) of a value."""
    if isinstance(v, Cx):
        return "c", _kind_of_real(v.re)
    if isinstance(v, (bool, np.bool_)):
        return "l", 0
    if isinstance(v, str):
        return "s", 0
    if isinstance(v, np.ndarray):
        if v.dtype == np.bool_:
            return "l", 0
        if v.dtype.kind in "iu":
            return "i", 0
        if v.dtype == np.float64:
            return "r", 8
        if v.dtype == np.float32:
            return "r", 4
        raise FortranError(f"unexpected array dtype {v.dtype}")
    if _is_int(v):
        return "i", 0
    if isinstance(v, np.float64):
        return "r", 8
    if isinstance(v, np.float32):
        return "r", 4
    if isinstance(v, float):
        return "r", 8
    raise FortranError(f"unexpected value {v!r}")


def _conv_real(v, kind):
    rt = _rdt(kind)
    if isinstance(v, np.ndarray):
        return v.astype(rt) if v.dtype != rt else v
    return rt(v)


def _conv_cx(v, kind):
    if isinstance(v, Cx):
        if _kind_of_real(v.re) == kind:
            return v
        return Cx(_conv_real(v.re, kind), _conv_real(v.im, kind))
    r = _conv_real(v, kind)
    return Cx(r, np.zeros_like(r) if isinstance(r, np.ndarray) else _rdt(kind)(0.0))


def _int_div(a, b):
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        a = np.asarray(a)
        b = np.asarray(b)
        q = np.abs(a) // np.abs(b)
        return np.where((a < 0) ^ (b < 0), -q, q)
    q = abs(a) // abs(b)
    return -q if (a < 0) != (b < 0) else q


def _cmul(a, b):
    return Cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re)


def _cdiv(a, b):
    # Smith's algorithm (range-reduced complex division)
    if isinstance(b.re, np.ndarray) or isinstance(a.re, np.ndarray):
        raise FortranError("complex/complex on arrays is not supported")
    if abs(b.re) >= abs(b.im):
        r = b.im / b.re
        d = b.re + b.im * r
        return Cx((a.re + a.im * r) / d, (a.im - a.re * r) / d)
    r = b.re / b.im
    d = b.re * r + b.im
    return Cx((a.re * r + a.im) / d, (a.im * r - a.re) / d)


def _powi(x, n, mul):
    """x**n for an integer n >= 0 by repeated squaring (x**2 = x*x)."""
    if n == 0:
        raise FortranError("x**0 is not supported")
    result = None
    base = x
    while n:
        if n & 1:
            result = base if result is None else mul(result, base)
        n >>= 1
        if n:
            base = mul(base, base)
    return result


def arith(op, a, b):
    ca, ka = _num_kind(a)
    cb, kb = _num_kind(b)
    if ca == "s" or cb == "s" or ca == "l" or cb == "l":
        raise FortranError(f"arithmetic on non-numeric operands {a!r} {op} {b!r}")
    if op == "**":
        if cb == "i" and not isinstance(b, np.ndarray):
            n = int(b)
            if ca == "i":
                return int(a) ** n if n >= 0 else (1 if abs(int(a)) == 1 else 0)
            if n < 0:
                inv = arith("/", 1, a)
                return _powi(inv, -n, lambda p, q: arith("*", p, q))
            return _powi(a, n, lambda p, q: arith("*", p, q))
        if ca == "c" or cb == "c":
            raise FortranError("complex ** non-integer is not supported")
        k = max(ka, kb, 4)
        x, y = _conv_real(_as_real(a, k), k), _conv_real(_as_real(b, k), k)
        if isinstance(x, np.ndarray) or isinstance(y, np.ndarray):
            return np.vectorize(lambda u, v: LIBM["pow"](u, v), otypes=[_rdt(k)])(x, y)
        return LIBM["pow"](x, y)
    if ca == "i" and cb == "i":
        if op == "+":
            return a + b
        if op == "-":
            return a - b
        if op == "*":
            return a * b
        if op == "/":
            return _int_div(a, b)
        raise FortranError(op)
    if ca != "c" and cb != "c":
        k = max(ka, kb)
        x = _conv_real(a, k)
        y = _conv_real(b, k)
        if op == "+":
            return x + y
        if op == "-":
            return x - y
        if op == "*":
            return x * y
        if op == "/":
            return x / y
        raise FortranError(op)
    k = max(ka, kb)
    if ca == "c" and cb == "c":
        x, y = _conv_cx(a, k), _conv_cx(b, k)
        if op == "+":
            return Cx(x.re + y.re, x.im + y.im)
        if op == "-":
            return Cx(x.re - y.re, x.im - y.im)
        if op == "*":
            return _cmul(x, y)
        if op == "/":
            return _cdiv(x, y)
        raise FortranError(op)
    # one real (or integer) operand: componentwise
    if ca == "c":
        x = _conv_cx(a, k)
        r = _conv_real(_as_real(b, k), k)
        if op == "+":
            return Cx(x.re + r, x.im)
        if op == "-":
            return Cx(x.re - r, x.im)
        if op == "*":
            return Cx(x.re * r, x.im * r)
        if op == "/":
            return Cx(x.re / r, x.im / r)
    else:
        r = _conv_real(_as_real(a, k), k)
        y = _conv_cx(b, k)
        if op == "+":
            return Cx(r + y.re, y.im)
        if op == "-":
            return Cx(r - y.re, -y.im)
        if op == "*":
            return Cx(r * y.re, r * y.im)
        if op == "/":
            return _cdiv(_conv_cx(r, k), y)
    raise FortranError(op)


def neg(a):
    if isinstance(a, Cx):
        return Cx(-a.re, -a.im)
    return -a


def compare(op, a, b):
    ca, ka = _num_kind(a)
    cb, kb = _num_kind(b)
    if ca == "s" and cb == "s":
        n = max(len(a), len(b))
        x, y = a.ljust(n), b.ljust(n)
    elif ca == "c" or cb == "c":
        if op not in ("==", "/="):
            raise FortranError("ordering comparison of complex values")
        k = max(ka, kb, 4)
        x, y = _conv_cx(a, k), _conv_cx(b, k)
        eq = (x.re == y.re) & (x.im == y.im)
        return eq if op == "==" else ~eq if isinstance(eq, np.ndarray) else not eq
    else:
        k = max(ka, kb)
        x = a if ca == "i" and cb == "i" else _conv_real(_as_real(a, k or 4), k or 4)
        y = b if ca == "i" and cb == "i" else _conv_real(_as_real(b, k or 4), k or 4)
    return {"==": lambda: x == y, "/=": lambda: x != y, "<": lambda: x < y, "<=": lambda: x <= y,
            ">": lambda: x > y, ">=": lambda: x >= y}[op]()


# ----------------------------------------------------------------- source --
def _strip_comment(line):
    out = []
    q = None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
            out.append(ch)
            continue
        if ch == "!":
            break
        out.append(ch)
    return "".join(out)


def _split_semicolons(line):
    parts, cur, q, depth = [], [], None, 0
    for ch in line:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == ";" and depth == 0:
            parts.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    parts.append("".join(cur))
    return [p for p in parts if p.strip()]


_INCLUDE = re.compile(r"^\s*include\s+['\"]([^'\"]+)['\"]\s*$", re.I)


def load_statements(path, includes):
    """Statements of a free-form source file: comments stripped, continuation
    lines joined, `include` lines replaced by the text `includes[name]`."""
    lines = []
    for raw in open(path, encoding="latin-1").read().splitlines():
        m = _INCLUDE.match(_strip_comment(raw))
        if m:
            name = m.group(1)
            if name not in includes:
                raise FortranError(f"include {name} not provided")
            lines.extend(includes[name].splitlines())
        else:
            lines.append(raw)
    stmts = []
    buf = ""
    for raw in lines:
        s = _strip_comment(raw).rstrip()
        if not s.strip():
            continue
        t = s.strip()
        if buf:
            if t.startswith("&"):
                t = t[1:]
            s = buf + t
            buf = ""
        else:
            s = t
        if s.endswith("&"):
            buf = s[:-1]
            continue
        stmts.extend(p.strip() for p in _split_semicolons(s))
    return stmts


# ------------------------------------------------------------------ lexer --
_TOK = re.compile(r"""
    (?P<ws>\s+)
  | (?P<str>'(?:[^']|'')*'|"(?:[^"]|"")*")
  | (?P<dotop>\.(?:and|or|not|eqv|neqv|eq|ne|lt|le|gt|ge|true|false)\.)
  | (?P<num>(?:\d+\.\d*(?![a-z])|\.\d+|\d+\.\d*(?=[ed][+-]?\d)|\d+)(?:[ed][+-]?\d+)?(?:_\w+)?)
  | (?P<name>[a-z_][a-z0-9_]*)
  | (?P<op>\*\*|//|==|/=|<=|>=|::|\(/|/\)|=>|[-+*/(),=<>:%])
""", re.I | re.X)


def tokenize(s):
    toks = []
    pos = 0
    n = len(s)
    while pos < n:
        m = _TOK.match(s, pos)
        if not m:
            raise FortranError(f"cannot tokenize: {s[pos:pos + 30]!r} in {s!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        val = m.group(kind)
        if kind == "name" or kind == "dotop":
            val = val.lower()
        toks.append((kind, val))
    return toks


# ----------------------------------------------------------------- parser --
class _P:
    """Expression parser over a token list."""

    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def next(self):
        tok = self.peek()
        self.i += 1
        return tok

    def accept(self, val):
        if self.peek()[1] == val:
            self.i += 1
            return True
        return False

    def expect(self, val):
        if not self.accept(val):
            raise FortranError(f"expected {val!r} at {self.t[self.i:]!r}")

    def at_end(self):
        return self.i >= len(self.t)

    # precedence: eqv/neqv < or < and < not < comparison < concat < add < mul < power < primary
    def expr(self):
        a = self.or_()
        while self.peek()[1] in (".eqv.", ".neqv."):
            op = self.next()[1]
            a = ("logic", op, a, self.or_())
        return a

    def or_(self):
        a = self.and_()
        while self.accept(".or."):
            a = ("logic", ".or.", a, self.and_())
        return a

    def and_(self):
        a = self.not_()
        while self.accept(".and."):
            a = ("logic", ".and.", a, self.not_())
        return a

    def not_(self):
        if self.accept(".not."):
            return ("not", self.not_())
        return self.cmp()

    _CMP = {"==": "==", "/=": "/=", "<": "<", "<=": "<=", ">": ">", ">=": ">=", ".eq.": "==", ".ne.": "/=",
            ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">="}

    def cmp(self):
        a = self.concat()
        op = self.peek()[1]
        if op in self._CMP:
            self.next()
            return ("cmp", self._CMP[op], a, self.concat())
        return a

    def concat(self):
        a = self.add()
        while self.accept("//"):
            a = ("concat", a, self.add())
        return a

    def add(self):
        if self.peek()[1] in ("+", "-"):
            op = self.next()[1]
            a = self.mul()
            if op == "-":
                a = ("neg", a)
        else:
            a = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.next()[1]
            a = ("bin", op, a, self.mul())
        return a

    def mul(self):
        a = self.power()
        while self.peek()[1] in ("*", "/"):
            op = self.next()[1]
            a = ("bin", op, a, self.power())
        return a

    def power(self):
        a = self.primary()
        if self.accept("**"):
            if self.peek()[1] in ("+", "-"):
                op = self.next()[1]
                e = self.power()
                return ("bin", "**", a, ("neg", e) if op == "-" else e)
            return ("bin", "**", a, self.power())   # right associative
        return a

    def primary(self):
        kind, val = self.peek()
        if kind == "num":
            self.next()
            return ("num", val)
        if kind == "str":
            self.next()
            q = val[0]
            return ("str", val[1:-1].replace(q + q, q))
        if val in (".true.", ".false."):
            self.next()
            return ("logical", val == ".true.")
        if val == "(/":
            self.next()
            items = self.arglist("/)")
            return ("arraycons", items)
        if val == "(":
            self.next()
            # implied do or complex literal or parenthesised expression
            e = self.expr()
            if self.accept(","):
                e2 = self.expr()
                if self.accept("="):   # implied do (e, v = lo, hi)
                    lo = self.expr()
                    self.expect(",")
                    hi = self.expr()
                    self.expect(")")
                    return ("implied_do", e, e2, lo, hi)
                self.expect(")")
                return ("cplx", e, e2)
            self.expect(")")
            return ("paren", e)
        if kind == "name":
            self.next()
            if self.peek()[1] == "(":
                self.next()
                args = self.arglist(")")
                return ("apply", val, args)
            return ("name", val)
        raise FortranError(f"unexpected token {val!r} in {self.t!r}")

    def arglist(self, close):
        args = []
        if self.accept(close):
            return args
        while True:
            args.append(self.arg())
            if self.accept(close):
                return args
            self.expect(",")

    def arg(self):
        # keyword=, slice lo:hi:step or expression
        if self.peek()[0] == "name" and self.peek(1)[1] == "=" :
            name = self.next()[1]
            self.next()
            return ("kw", name, self.expr())
        if self.peek()[1] == "(" and self._looks_implied_do():
            return self.primary()
        lo = hi = st = None
        if self.peek()[1] != ":":
            lo = self.expr()
            if self.peek()[1] != ":":
                return lo
        self.expect(":")
        if self.peek()[1] not in (",", ")", ":", "/)"):
            hi = self.expr()
        if self.accept(":"):
            st = self.expr()
        return ("slice", lo, hi, st)

    def _looks_implied_do(self):
        return False


def parse_expr(text):
    p = _P(tokenize(text))
    e = p.expr()
    if not p.at_end():
        raise FortranError(f"trailing tokens in expression {text!r}: {p.t[p.i:]!r}")
    return e


# --------------------------------------------------------- statement parse --
_TYPES = ("integer", "real", "complex", "logical", "character", "double precision", "double complex")
_DECL = re.compile(r"^(integer|real|complex|logical|character|double\s+precision|double\s+complex)\b", re.I)


def _split_top(s, sep=","):
    parts, cur, depth, q = [], [], 0, None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    parts.append("".join(cur))
    return [p.strip() for p in parts]


def parse_decl(stmt, real_kind):
    """A type declaration -> list of dicts (name, base, kind, dims, attrs, init)."""
    m = _DECL.match(stmt)
    base = m.group(1).lower()
    rest = stmt[m.end():].strip()
    kind = real_kind
    if base.startswith("double"):
        base = "real" if "precision" in base else "complex"
        kind = 8
    if base == "integer" or base == "logical" or base == "character":
        kind = 0
    if rest.startswith("("):   # kind or len selector
        depth = 0
        for j, ch in enumerate(rest):
            depth += ch == "("
            depth -= ch == ")"
            if depth == 0:
                sel = rest[1:j].strip().lower()
                rest = rest[j + 1:].strip()
                break
        if base in ("real", "complex"):
            kv = sel.split("=")[-1].strip()
            kind = int(kv)
    if "::" in rest:
        attr_s, ents_s = rest.split("::", 1)
        attrs = [a.strip().lower() for a in _split_top(attr_s.lstrip(","))] if attr_s.strip() else []
    else:
        attrs, ents_s = [], rest
    dims_attr = None
    flags = set()
    intent = None
    for a in attrs:
        if not a:
            continue
        if a.startswith("dimension"):
            dims_attr = a[a.index("(") + 1:a.rindex(")")]
        elif a.startswith("intent"):
            intent = a[a.index("(") + 1:a.rindex(")")].strip().lower()
        else:
            flags.add(a)
    out = []
    for ent in _split_top(ents_s):
        init = None
        if "=" in ent and not ent.split("=", 1)[0].strip().endswith(("<", ">", "/")):
            ent, init = ent.split("=", 1)
            init = init.strip()
        ent = ent.strip()
        dims = None
        if "(" in ent:
            name = ent[:ent.index("(")].strip().lower()
            dims = ent[ent.index("(") + 1:ent.rindex(")")]
        else:
            name = ent.lower()
        if dims is None and dims_attr is not None:
            dims = dims_attr
        out.append({"name": name, "base": base, "kind": kind, "dims": dims, "flags": flags, "intent": intent,
                    "init": init})
    return out


class Unit:
    """A parsed program unit (module, program or procedure)."""

    def __init__(self, kind, name):
        self.kind = kind
        self.name = name
        self.uses = []
        self.decls = []
        self.body = []
        self.procs = {}
        self.args = []
        self.result_base = None
        self.module = None


def _kw(stmt):
    m = re.match(r"\s*([a-z_]\w*)", stmt, re.I)
    return m.group(1).lower() if m else ""


_END = re.compile(r"^end\s*(module|program|subroutine|function|if|do|select)?\b", re.I)


def parse_units(stmts, real_kind):
    """Parse a file's statements into units."""
    units = []
    i = 0
    n = len(stmts)

    def parse_proc_header(s):
        m = re.match(r"^(?:(integer|real|complex|logical)\s+)?(recursive\s+)?(subroutine|function)\s+(\w+)\s*(\((.*)\))?",
                     s, re.I)
        if not m:
            return None
        u = Unit(m.group(3).lower(), m.group(4).lower())
        u.result_base = (m.group(1) or "").lower() or None
        u.args = [a.strip().lower() for a in (m.group(6) or "").split(",") if a.strip()]
        return u

    def parse_unit_body(u, i, end_kind):
        # specification part, then executable part, then contains
        body_stmts = []
        while i < n:
            s = stmts[i]
            low = s.lower()
            m = _END.match(low)
            if m and (m.group(1) in (None, end_kind)) and not re.match(r"^end\s*(if|do|select)\b", low):
                return i + 1, body_stmts
            if low == "contains":
                i += 1
                while i < n:
                    s2 = stmts[i]
                    low2 = s2.lower()
                    m2 = _END.match(low2)
                    if m2 and m2.group(1) in (None, end_kind) and not re.match(r"^end\s*(if|do|select)\b", low2):
                        return i + 1, body_stmts
                    pu = parse_proc_header(s2)
                    if pu is None:
                        raise FortranError(f"expected a procedure after contains: {s2!r}")
                    pu.module = u
                    i, pb = parse_unit_body(pu, i + 1, pu.kind)
                    pu.body = pb
                    u.procs[pu.name] = pu
                continue
            if low.startswith("use "):
                u.uses.append(low.split()[1].strip(","))
            elif low.startswith("implicit"):
                pass
            elif _DECL.match(s) and not re.match(r"^(real|complex|integer|logical)\s+function\b", low) and \
                    ("::" in s or re.match(r"^(integer|real|complex|logical|character)(\s*\(.*?\))?\s+\w+\s*(\(|,|$)", low)):
                u.decls.extend(parse_decl(s, real_kind))
            else:
                body_stmts.append(s)
            i += 1
        raise FortranError(f"unterminated unit {u.name}")

    while i < n:
        s = stmts[i]
        low = s.lower()
        if low.startswith("module "):
            u = Unit("module", low.split()[1])
            i, body = parse_unit_body(u, i + 1, "module")
            if body:
                raise FortranError(f"executable statements in module {u.name}: {body[:2]}")
            units.append(u)
        elif low.startswith("program "):
            u = Unit("program", low.split()[1])
            i, body = parse_unit_body(u, i + 1, "program")
            u.body = body
            units.append(u)
        else:
            raise FortranError(f"unexpected statement at file level: {s!r}")
    return units


# -------------------------------------------------------- executable parse --
def parse_block(stmts, i=0, stop=()):
    """Executable statements -> nested statement tuples; returns (list, i)."""
    out = []
    n = len(stmts)
    while i < n:
        s = stmts[i]
        low = s.lower()
        first = _kw(low)
        if any(re.match(p, low) for p in stop):
            return out, i
        if re.match(r"^if\s*\(", low):
            cond, rest = _paren_prefix(s[2:].lstrip())
            if rest.strip().lower() == "then":
                branches = []
                body, i = parse_block(stmts, i + 1, (r"^else\s*if\b", r"^else$", r"^end\s*if$"))
                branches.append((parse_expr(cond), body))
                else_body = []
                while True:
                    low2 = stmts[i].lower()
                    if re.match(r"^else\s*if\b", low2):
                        c2, r2 = _paren_prefix(re.sub(r"^else\s*if", "", stmts[i], flags=re.I).lstrip())
                        body, i = parse_block(stmts, i + 1, (r"^else\s*if\b", r"^else$", r"^end\s*if$"))
                        branches.append((parse_expr(c2), body))
                    elif low2 == "else":
                        else_body, i = parse_block(stmts, i + 1, (r"^end\s*if$",))
                    else:
                        i += 1
                        break
                out.append(("if", branches, else_body))
                continue
            inner, _ = parse_block([rest.strip()], 0)
            out.append(("if", [(parse_expr(cond), inner)], []))
            i += 1
            continue
        if re.match(r"^do\s+while\b", low):
            cond, _ = _paren_prefix(s[s.lower().index("while") + 5:].lstrip())
            body, i = parse_block(stmts, i + 1, (r"^end\s*do$",))
            out.append(("dowhile", parse_expr(cond), body))
            i += 1
            continue
        if re.match(r"^do\s+\w+\s*=", low):
            m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", s, re.I)
            parts = _split_top(m.group(2))
            body, i = parse_block(stmts, i + 1, (r"^end\s*do$",))
            out.append(("do", m.group(1).lower(), parse_expr(parts[0]), parse_expr(parts[1]),
                        parse_expr(parts[2]) if len(parts) > 2 else None, body))
            i += 1
            continue
        if re.match(r"^select\s*case\b", low):
            sel, _ = _paren_prefix(re.sub(r"^select\s*case", "", s, flags=re.I).lstrip())
            i += 1
            cases = []
            while not re.match(r"^end\s*select$", stmts[i].lower()):
                low2 = stmts[i].lower()
                if re.match(r"^case\s+default$", low2) or low2 == "case default":
                    body, i = parse_block(stmts, i + 1, (r"^case\b", r"^end\s*select$"))
                    cases.append((None, body))
                elif re.match(r"^case\s*\(", low2):
                    vals, _ = _paren_prefix(stmts[i][4:].lstrip())
                    body, i = parse_block(stmts, i + 1, (r"^case\b", r"^end\s*select$"))
                    cases.append(([parse_expr(v) for v in _split_top(vals)], body))
                else:
                    raise FortranError(f"unexpected statement in select: {stmts[i]!r}")
            out.append(("select", parse_expr(sel), cases))
            i += 1
            continue
        out.append(parse_simple(s))
        i += 1
    return out, i


def _paren_prefix(s):
    """'(...) rest' -> ('...', 'rest')."""
    if not s.startswith("("):
        raise FortranError(f"expected '(' in {s!r}")
    depth, q = 0, None
    for j, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
            if depth == 0:
                return s[1:j], s[j + 1:]
    raise FortranError(f"unbalanced parentheses in {s!r}")


def parse_simple(s):
    low = s.lower()
    first = _kw(low)
    if first == "call":
        m = re.match(r"^call\s+(\w+)\s*(\((.*)\))?\s*$", s, re.I)
        args = []
        if m.group(3) is not None and m.group(3).strip():
            p = _P(tokenize(m.group(3)))
            while True:
                args.append(p.arg())
                if p.at_end():
                    break
                p.expect(",")
        return ("call", m.group(1).lower(), args)
    if first in ("return",):
        return ("return",)
    if first == "stop":
        return ("stop",)
    if first == "exit":
        return ("exit",)
    if first == "cycle":
        return ("cycle",)
    if first == "continue":
        return ("nop",)
    if first in ("allocate", "deallocate"):
        inner, _ = _paren_prefix(s[len(first):].lstrip())
        items = []
        for it in _split_top(inner):
            if first == "allocate":
                name = it[:it.index("(")].strip().lower()
                dims = _split_top(it[it.index("(") + 1:it.rindex(")")])
                items.append((name, [_bounds(d) for d in dims]))
            else:
                items.append(it.strip().lower())
        return (first, items)
    if first == "print":
        rest = s[5:].strip()
        fmt, _, items = rest.partition(",")
        return ("write_io", {"unit": ("name", "*"), "fmt": ("name", "*")},
                [parse_expr(x) for x in _split_top(items)] if items.strip() else [])
    if first in ("write", "read", "open", "close", "inquire"):
        ctl, rest = _paren_prefix(s[len(first):].lstrip())
        rest = rest.strip()
        if rest.startswith(","):
            rest = rest[1:].strip()
        specs = {}
        pos = 0
        for k, part in enumerate(_split_top(ctl)):
            if "=" in part and re.match(r"^\s*\w+\s*=", part) and not part.strip().startswith("("):
                key, val = part.split("=", 1)
                specs[key.strip().lower()] = parse_expr(val.strip())
            else:
                specs[["unit", "fmt"][pos]] = parse_expr(part.strip()) if part.strip() != "*" else ("name", "*")
                pos += 1
        items = [parse_expr(x) for x in _split_top(rest)] if rest else []
        return (first + "_io", specs, items)
    # assignment
    depth, q = 0, None
    for j, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "=" and depth == 0 and s[j + 1:j + 2] != "=" and s[j - 1:j] not in ("/", "<", ">", "="):
            return ("assign", parse_expr(s[:j]), parse_expr(s[j + 1:]))
    raise FortranError(f"unsupported statement {s!r}")


def _bounds(d):
    d = d.strip()
    if ":" in d:
        lo, hi = _split_top(d, ":")
        return (parse_expr(lo) if lo else None, parse_expr(hi) if hi else None)
    return (("num", "1"), parse_expr(d))


# ---------------------------------------------------------------- runtime --
class Var:
    __slots__ = ("name", "base", "kind", "val", "flags", "charlen", "dims", "intent")

    def __init__(self, name, base, kind, val=None, flags=(), charlen=None, dims=None, intent=None):
        self.name = name
        self.base = base
        self.kind = kind
        self.val = val
        self.flags = set(flags)
        self.charlen = charlen
        self.dims = dims
        self.intent = intent


class Ref:
    """An actual argument passed by reference: get() and set(value)."""
    __slots__ = ("get", "set", "var")

    def __init__(self, get, set_, var=None):
        self.get = get
        self.set = set_
        self.var = var


def _store_into(var, value):
    """Assign `value` to the whole of variable `var` (scalar or array)."""
    if isinstance(var.val, FArr):
        tgt = var.val.data
        if var.base == "complex":
            if isinstance(value, Cx):
                tgt.real[...] = value.re
                tgt.imag[...] = value.im
            elif isinstance(value, FArr):
                tgt[...] = value.data
            else:
                sv = _to_storage(value, "complex", var.kind)
                tgt[...] = sv
        else:
            if isinstance(value, FArr):
                value = value.data
            tgt[...] = _to_storage(value, var.base, var.kind)
        return
    if var.base == "character":
        s = str(value)
        if var.charlen is not None:
            s = s[:var.charlen].ljust(var.charlen)
        var.val = s
        return
    if isinstance(value, FArr):
        raise FortranError(f"array assigned to scalar {var.name}")
    var.val = _to_storage(value, var.base, var.kind)


def _value_of_storage(v, base):
    """A variable's stored value as an expression value."""
    if isinstance(v, FArr):
        d = v.data
        if base == "complex":
            return _cx_from_storage(d)
        return d.copy()
    if base == "complex" and v is not None:
        return _cx_from_storage(v)
    if base == "integer" and v is not None:
        return int(v)
    return v


def _elem_value(data, idx, base):
    v = data[idx]
    if base == "complex":
        if isinstance(v, np.ndarray):
            return _cx_from_storage(v)
        rt = np.float32 if data.dtype == np.complex64 else np.float64
        return Cx(rt(v.real), rt(v.imag))
    if base == "integer":
        return v.astype(np.int64) if isinstance(v, np.ndarray) else int(v)
    if base == "logical":
        return v if isinstance(v, np.ndarray) else bool(v)
    return v


def _flatten_items(vals):
    out = []
    for v in vals:
        if isinstance(v, Cx):
            if isinstance(v.re, np.ndarray):
                for a, b in zip(np.ravel(v.re, order="F"), np.ravel(v.im, order="F")):
                    out.extend([a, b])
            else:
                out.extend([v.re, v.im])
        elif isinstance(v, np.ndarray):
            out.extend(np.ravel(v, order="F").tolist() if v.dtype.kind in "iub" else list(np.ravel(v, order="F")))
        elif isinstance(v, FArr):
            out.extend(_flatten_items([v.data]))
        else:
            out.append(v)
    return out


def _format(fmt, vals):
    """Simple Fortran edit descriptors (a, iW[.M], fW.D, eW.D, x, quoted text)."""
    fmt = fmt.strip()
    if fmt.startswith("(") and fmt.endswith(")"):
        fmt = fmt[1:-1]
    descs = []
    for d in _split_top(fmt):
        d = d.strip()
        m = re.match(r"^(\d*)([a-z]+)(\d*)(?:\.(\d+))?$", d, re.I)
        if d.startswith(("'", '"')):
            descs.append(("lit", d[1:-1]))
            continue
        if not m:
            raise FortranError(f"format descriptor {d!r}")
        rep = int(m.group(1) or 1)
        for _ in range(rep):
            descs.append((m.group(2).lower(), int(m.group(3)) if m.group(3) else None,
                          int(m.group(4)) if m.group(4) else None))
    items = _flatten_items(vals)
    out = []
    k = 0
    guard = 0
    while k < len(items) or (descs and descs[0][0] == "lit" and not out):
        for d in descs:
            if d[0] == "lit":
                out.append(d[1])
                continue
            if d[0] == "x":
                out.append(" " * (d[1] or 1))
                continue
            if k >= len(items):
                break
            v = items[k]
            k += 1
            code, w, m_ = d[0], d[1], d[2]
            if code == "a":
                s = str(v)
                out.append(s if w is None else s[:w].rjust(w))
            elif code == "i":
                s = str(int(v))
                if m_ is not None:
                    neg_ = s.startswith("-")
                    s = ("-" if neg_ else "") + s.lstrip("-").zfill(m_)
                out.append(s.rjust(w) if w else s)
            elif code == "f":
                s = f"{float(v):.{m_ or 0}f}"
                out.append(s.rjust(w) if w else s)
            elif code in ("e", "es", "g"):
                s = f"{float(v):.{m_ or 6}E}"
                out.append(s.rjust(w) if w else s)
            else:
                raise FortranError(f"format code {code}")
        guard += 1
        if guard > 1000:
            raise FortranError("format reversion does not terminate")
        if k >= len(items):
            break
    return "".join(out)


def _list_directed(vals):
    parts = []
    for v in _flatten_items(vals):
        if isinstance(v, str):
            parts.append(v)
        elif isinstance(v, (bool, np.bool_)):
            parts.append("T" if v else "F")
        elif _is_int(v):
            parts.append(str(int(v)))
        else:
            parts.append(repr(float(v)))
    return " " + " ".join(parts)


def _record_bytes(vals):
    """Payload of an unformatted sequential record (native little-endian)."""
    chunks = []
    for v in vals:
        if isinstance(v, FArr):
            v = v.data
        if isinstance(v, Cx):
            if isinstance(v.re, np.ndarray):
                rt = v.re.dtype
                ct = np.complex64 if rt == np.float32 else np.complex128
                arr = np.empty(v.re.shape, dtype=ct)
                arr.real = v.re
                arr.imag = v.im
                chunks.append(np.ravel(arr, order="F").tobytes())
            else:
                rt = np.float32 if _kind_of_real(v.re) == 4 else np.float64
                chunks.append(np.array([v.re, v.im], dtype=rt).tobytes())
        elif isinstance(v, np.ndarray):
            if v.dtype.kind in "iu":
                v = v.astype(np.int32)
            elif v.dtype == np.bool_:
                v = v.astype(np.int32)
            chunks.append(np.ravel(v, order="F").tobytes())
        elif isinstance(v, (bool, np.bool_)):
            chunks.append(struct.pack("<i", 1 if v else 0))
        elif _is_int(v):
            chunks.append(struct.pack("<i", int(v)))
        elif isinstance(v, np.float32):
            chunks.append(np.float32(v).tobytes())
        elif isinstance(v, (np.float64, float)):
            chunks.append(np.float64(v).tobytes())
        elif isinstance(v, np.complexfloating):
            chunks.append(np.array([v]).tobytes())
        elif isinstance(v, str):
            chunks.append(v.encode("latin-1"))
        else:
            raise FortranError(f"cannot write {v!r} to an unformatted record")
    return b"".join(chunks)


class World:
    """Shared state of the emulated MPI process grid (ranks are threads)."""

    def __init__(self, nprocs, timeout=600.0):
        self.n = nprocs
        self.lock = threading.Condition()
        self.mail = {}
        self.barrier = threading.Barrier(nprocs, timeout=timeout)
        self.slots = [None] * nprocs
        self.timeout = timeout
        self.failed = None

    def post(self, src, dst, tag, data):
        with self.lock:
            self.mail.setdefault((src, dst, tag), []).append(data)
            self.lock.notify_all()

    def take(self, src, dst, tag):
        with self.lock:
            ok = self.lock.wait_for(lambda: self.mail.get((src, dst, tag)) or self.failed, timeout=self.timeout)
            if self.failed:
                raise FortranError(f"another rank failed: {self.failed}")
            if not ok:
                raise FortranError(f"MPI receive from {src} tag {tag} timed out")
            return self.mail[(src, dst, tag)].pop(0)

    def sync(self):
        try:
            self.barrier.wait()
        except threading.BrokenBarrierError:
            raise FortranError(f"barrier broken: {self.failed}")


MPI_CONSTS = {"mpi_comm_world": 91, "mpi_status_size": 6, "mpi_proc_null": -2, "mpi_complex": 18,
              "mpi_double_complex": 22, "mpi_real": 13, "mpi_double_precision": 17, "mpi_logical": 7,
              "mpi_integer": 7 + 100, "mpi_sum": 1, "mpi_max": 2, "mpi_min": 3, "mpi_land": 4,
              "mpi_any_source": -1}
MPIF_H = "\n".join(f"integer, parameter :: {k.upper()}={v}" for k, v in MPI_CONSTS.items())


# ------------------------------------------------------------ interpreter --
class ModuleInst:
    def __init__(self, unit):
        self.unit = unit
        self.vars = {}
        self.uses = []


class _Proc:
    """A compiled procedure: local declarations and body closure."""
    __slots__ = ("unit", "minst", "body", "locals", "result", "args")


def _lit_num(tok, real_kind):
    t = tok.lower()
    kind = None
    if "_" in t:
        t, k = t.split("_", 1)
        kind = int(k)
    if re.fullmatch(r"\d+", t):
        return int(t)
    if "d" in t:
        kind = 8
        t = t.replace("d", "e")
    kind = kind or real_kind
    return _rdt(kind)(float(t)) if kind == 8 else np.float32(t)


class Interp:
    """One rank of the interpreted program."""

    def __init__(self, units, real_kind, rank, world, workdir):
        self.units = {u.name: u for u in units}
        self.rk = real_kind
        self.rank = rank
        self.world = world
        self.workdir = workdir
        self.mods = {}
        self.stdout = []
        self.files = {}
        self.reqs = {}
        self.nreq = 0
        self.cart = None
        self.rng = np.random.RandomState(12345 + rank)
        self.procs = {}

    # ---- scopes
    def module(self, name):
        if name in self.mods:
            return self.mods[name]
        if name not in self.units:
            raise FortranError(f"module {name} not found")
        unit = self.units[name]
        mi = ModuleInst(unit)
        self.mods[name] = mi
        mi.uses = [self.module(u) for u in unit.uses]
        for d in unit.decls:
            mi.vars[d["name"]] = self._declare(d, lambda nm, mi=mi: self._lookup_mod(mi, nm))
        return mi

    def _lookup_mod(self, mi, name, seen=None, public_only=False):
        v = mi.vars.get(name)
        if v is not None and not (public_only and "private" in v.flags):
            return ("var", v)
        p = mi.unit.procs.get(name)
        if p is not None:
            return ("proc", (mi, p))
        seen = seen or set()
        seen.add(id(mi))
        for u in mi.uses:
            if id(u) in seen:
                continue
            r = self._lookup_mod(u, name, seen, True)
            if r is not None:
                return r
        return None

    def _declare(self, d, lookup, frame=None):
        base, kind = d["base"], d["kind"]
        charlen = None
        var = Var(d["name"], base, kind, flags=d["flags"], intent=d["intent"])
        if base == "character":
            charlen = None
        var.charlen = charlen
        if d["dims"] is not None and "allocatable" not in d["flags"]:
            dims = [_bounds(x) for x in _split_top(d["dims"])]
            if all(lo is not None and hi is not None for lo, hi in dims):
                ev = lambda e: self._const_eval(e, lookup, frame)
                lbs = [ev(lo) for lo, hi in dims]
                shape = [ev(hi) - ev(lo) + 1 for lo, hi in dims]
                var.val = FArr(np.zeros(shape, dtype=self._dtype(base, kind)), lbs)
                var.dims = dims
            else:
                var.dims = dims   # assumed shape: bound at call time
        if var.val is None and d["dims"] is None:
            # module variables live in zero-initialised static storage
            var.val = {"integer": 0, "logical": False, "character": ""}.get(base)
            if base == "real":
                var.val = _rdt(kind or self.rk)(0.0)
            elif base == "complex":
                var.val = _cdt(kind or self.rk)(0.0)
        if d["init"] is not None:
            val = self._const_eval(parse_expr(d["init"]), lookup, frame)
            if isinstance(var.val, FArr):
                _store_into(var, val.data if isinstance(val, FArr) else val)
            else:
                _store_into(var, val)
        return var

    def _dtype(self, base, kind):
        return {"integer": np.int64, "logical": np.bool_, "real": _rdt(kind or self.rk),
                "complex": _cdt(kind or self.rk)}[base]

    def _const_eval(self, e, lookup, frame):
        fn = self._cexpr(e, lookup, set(frame or ()))
        return fn(frame or {})

    # ---- procedures
    def proc(self, mi, unit):
        key = (id(mi), unit.name)
        p = self.procs.get(key)
        if p is not None:
            return p
        p = _Proc()
        p.unit, p.minst = unit, mi
        p.args = unit.args
        p.locals = list(unit.decls)
        names = {d["name"] for d in unit.decls} | set(unit.args)
        p.result = None
        if unit.kind == "function":
            p.result = unit.name
            if unit.name not in names:
                p.locals.append({"name": unit.name, "base": unit.result_base, "kind": self.rk if unit.result_base in (
                    "real", "complex") else 0, "dims": None, "flags": set(), "intent": None, "init": None})
            names.add(unit.name)
        self.procs[key] = p
        lookup = self._proc_lookup(mi, unit)
        blk, _ = parse_block(unit.body)
        p.body = self._cblock(blk, lookup, names)
        return p

    def _proc_lookup(self, mi, unit):
        """Names a procedure sees: modules it uses itself, then its host module."""
        used = [self.module(u) for u in unit.uses]

        def lookup(nm):
            for u in used:
                r = self._lookup_mod(u, nm, None, True)
                if r is not None:
                    return r
            return self._lookup_mod(mi, nm)
        return lookup

    def call(self, p, actuals):
        frame = {}
        lookup = self._proc_lookup(p.minst, p.unit)
        for d in p.locals:
            if d["name"] in p.args:
                continue
            frame[d["name"]] = self._declare(d, lookup, frame)
        writeback = []
        decl_of = {d["name"]: d for d in p.locals}
        for name, act in zip(p.args, actuals):
            d = decl_of.get(name)
            if d is None:
                raise FortranError(f"dummy {name} of {p.unit.name} is not declared")
            var = Var(name, d["base"], d["kind"], flags=d["flags"], intent=d["intent"])
            v = act.get() if isinstance(act, Ref) else act
            if d["dims"] is not None:
                data = v.data if isinstance(v, FArr) else (v if isinstance(v, np.ndarray) else None)
                if data is None:
                    raise FortranError(f"array dummy {name} given a scalar")
                dims = [_bounds(x) for x in _split_top(d["dims"])]
                lbs = []
                for lo, hi in dims:
                    lbs.append(self._const_eval(lo, lookup, frame) if lo is not None else 1)
                var.val = FArr(data, lbs)
            elif d["base"] == "character":
                var.val = v
            else:
                _store_into(var, v)
                if isinstance(act, Ref) and d["intent"] != "in":
                    writeback.append((var, act))
            frame[name] = var
        try:
            p.body(frame)
        except _Return:
            pass
        for var, act in writeback:
            act.set(_value_of_storage(var.val, var.base))
        if p.result is not None:
            rv = frame[p.result]
            return _value_of_storage(rv.val, rv.base)
        return None

    # ---- expressions
    def _resolve(self, name, lookup, names):
        if name in names:
            return ("local", name)
        return lookup(name)

    def _cexpr(self, e, lookup, names):
        k = e[0]
        if k == "num":
            v = _lit_num(e[1], self.rk)
            return lambda fr: v
        if k == "str":
            s = e[1]
            return lambda fr: s
        if k == "logical":
            b = e[1]
            return lambda fr: b
        if k == "paren":
            return self._cexpr(e[1], lookup, names)
        if k == "neg":
            f = self._cexpr(e[1], lookup, names)
            return lambda fr: neg(f(fr))
        if k == "bin":
            op = e[1]
            fa, fb = self._cexpr(e[2], lookup, names), self._cexpr(e[3], lookup, names)
            return lambda fr: arith(op, fa(fr), fb(fr))
        if k == "cmp":
            op = e[1]
            fa, fb = self._cexpr(e[2], lookup, names), self._cexpr(e[3], lookup, names)
            return lambda fr: compare(op, fa(fr), fb(fr))
        if k == "logic":
            op = e[1]
            fa, fb = self._cexpr(e[2], lookup, names), self._cexpr(e[3], lookup, names)
            if op == ".and.":
                return lambda fr: bool(fa(fr)) and bool(fb(fr))
            if op == ".or.":
                return lambda fr: bool(fa(fr)) or bool(fb(fr))
            if op == ".eqv.":
                return lambda fr: bool(fa(fr)) == bool(fb(fr))
            return lambda fr: bool(fa(fr)) != bool(fb(fr))
        if k == "not":
            f = self._cexpr(e[1], lookup, names)
            return lambda fr: not f(fr)
        if k == "concat":
            fa, fb = self._cexpr(e[1], lookup, names), self._cexpr(e[2], lookup, names)
            return lambda fr: str(fa(fr)) + str(fb(fr))
        if k == "cplx":
            fa, fb = self._cexpr(e[1], lookup, names), self._cexpr(e[2], lookup, names)

            def cplx(fr):
                a, b = fa(fr), fb(fr)
                kk = max(_num_kind(a)[1], _num_kind(b)[1]) or self.rk
                return Cx(_conv_real(_as_real(a, kk), kk), _conv_real(_as_real(b, kk), kk))
            return cplx
        if k == "arraycons":
            parts = []
            for it in e[1]:
                if it[0] == "implied_do":
                    parts.append(("ido", self._implied_do(it, lookup, names)))
                else:
                    parts.append(("e", self._cexpr(it, lookup, names)))

            def cons(fr):
                vals = []
                for kind_, f in parts:
                    v = f(fr)
                    if kind_ == "ido" or isinstance(v, (list, np.ndarray)):
                        vals.extend(list(v))
                    else:
                        vals.append(v)
                return np.array(vals) if not any(isinstance(v, Cx) for v in vals) else vals
            return cons
        if k == "name":
            return self._cname(e[1], lookup, names)
        if k == "apply":
            return self._capply(e, lookup, names)
        raise FortranError(f"expression {e!r}")

    def _implied_do(self, it, lookup, names):
        _, ex, var, lo, hi = it
        vname = var[1]
        inner_names = set(names) | {vname}
        fe = self._cexpr(ex, lookup, inner_names)
        flo, fhi = self._cexpr(lo, lookup, names), self._cexpr(hi, lookup, names)

        def gen(fr):
            out = []
            saved = fr.get(vname)
            for v in range(int(flo(fr)), int(fhi(fr)) + 1):
                fr[vname] = Var(vname, "integer", 0, v)
                out.append(fe(fr))
            if saved is not None:
                fr[vname] = saved
            else:
                fr.pop(vname, None)
            return out
        return gen

    def _cname(self, name, lookup, names):
        r = self._resolve(name, lookup, names)
        if r is None:
            if name in INTRINSIC_CONST:
                val = INTRINSIC_CONST[name]
                return lambda fr: val
            raise FortranError(f"unknown name {name}")
        if r[0] == "local":
            return lambda fr: _value_of_storage(fr[name].val, fr[name].base)
        if r[0] == "var":
            var = r[1]
            return lambda fr: _value_of_storage(var.val, var.base)
        if r[0] == "proc":   # function without arguments
            mi, unit = r[1]
            return lambda fr: self.call(self.proc(mi, unit), [])
        raise FortranError(name)

    def _var_getter(self, name, lookup, names):
        r = self._resolve(name, lookup, names)
        if r is None:
            return None
        if r[0] == "local":
            return lambda fr: fr[name]
        if r[0] == "var":
            var = r[1]
            return lambda fr: var
        return None

    def _subscripts(self, args, lookup, names):
        fs = []
        for a in args:
            if a[0] == "slice":
                lo = self._cexpr(a[1], lookup, names) if a[1] is not None else None
                hi = self._cexpr(a[2], lookup, names) if a[2] is not None else None
                st = self._cexpr(a[3], lookup, names) if a[3] is not None else None
                fs.append(("s", lo, hi, st))
            else:
                fs.append(("i", self._cexpr(a, lookup, names)))
        scalar = all(f[0] == "i" for f in fs)

        def index(fr, arr):
            idx = []
            for dim, f in enumerate(fs):
                lb = arr.lb[dim]
                if f[0] == "i":
                    idx.append(int(f[1](fr)) - lb)
                else:
                    lo = int(f[1](fr)) - lb if f[1] else 0
                    hi = int(f[2](fr)) - lb + 1 if f[2] else arr.data.shape[dim]
                    st = int(f[3](fr)) if f[3] else 1
                    if lo < 0 or hi > arr.data.shape[dim]:
                        raise FortranError("array section out of bounds")
                    idx.append(slice(lo, hi, st))
            return tuple(idx)
        return index, scalar

    def _capply(self, e, lookup, names):
        name, args = e[1], e[2]
        vg = self._var_getter(name, lookup, names)
        if vg is not None:
            index, scalar = self._subscripts(args, lookup, names)

            def elem(fr):
                var = vg(fr)
                arr = var.val
                if not isinstance(arr, FArr):
                    raise FortranError(f"{name} is not an allocated array")
                idx = index(fr, arr)
                for q, ix in enumerate(idx):
                    if not isinstance(ix, slice) and (ix < 0 or ix >= arr.data.shape[q]):
                        raise FortranError(f"subscript {ix + arr.lb[q]} out of bounds in {name}")
                v = _elem_value(arr.data, idx, var.base)
                if isinstance(v, np.ndarray) and var.base != "complex":
                    v = v.copy()
                return v
            return elem
        r = lookup(name)
        if r is not None and r[0] == "proc":
            mi, unit = r[1]
            fargs = [self._carg(a, lookup, names) for a in args]
            return lambda fr: self.call(self.proc(mi, unit), [f(fr) for f in fargs])
        if name in INTRINSICS:
            fn = INTRINSICS[name]
            fpos, fkw = [], {}
            for a in args:
                if a[0] == "kw":
                    fkw[a[1]] = self._cexpr(a[2], lookup, names)
                else:
                    fpos.append(self._cexpr(a, lookup, names))
            return lambda fr: fn(self, [f(fr) for f in fpos], {k: f(fr) for k, f in fkw.items()})
        raise FortranError(f"unknown function or array {name}")

    def _carg(self, a, lookup, names):
        """An actual argument: a Ref for variables, elements and sections, else a value."""
        if a[0] == "name":
            vg = self._var_getter(a[1], lookup, names)
            if vg is not None:
                def ref(fr):
                    var = vg(fr)
                    return Ref(lambda: var.val if isinstance(var.val, FArr) else _value_of_storage(var.val, var.base),
                               lambda v: _store_into(var, v), var)
                return ref
        if a[0] == "apply":
            vg = self._var_getter(a[1], lookup, names)
            if vg is not None:
                index, scalar = self._subscripts(a[2], lookup, names)

                def ref2(fr):
                    var = vg(fr)
                    arr = var.val
                    idx = index(fr, arr)
                    if scalar:
                        def st(v, arr=arr, idx=idx, var=var):
                            arr.data[idx] = _to_storage(v, var.base, var.kind)
                        return Ref(lambda: _elem_value(arr.data, idx, var.base), st, var)
                    view = arr.data[idx]

                    def st2(v, view=view, var=var):
                        if isinstance(v, FArr):
                            v = v.data
                        if var.base == "complex" and isinstance(v, Cx):
                            view.real[...] = v.re
                            view.imag[...] = v.im
                        else:
                            view[...] = _to_storage(v, var.base, var.kind) if not isinstance(v, np.ndarray) else v
                    return Ref(lambda: FArr(view, [1] * view.ndim), st2, var)
                return ref2
        f = self._cexpr(a, lookup, names)
        return f

    # ---- statements
    def _cblock(self, stmts, lookup, names):
        fs = [self._cstmt(s, lookup, names) for s in stmts]

        def block(fr):
            for f in fs:
                f(fr)
        return block

    def _ctarget(self, t, lookup, names):
        if t[0] == "name":
            vg = self._var_getter(t[1], lookup, names)
            if vg is None:
                raise FortranError(f"assignment to unknown name {t[1]}")
            return lambda fr, v: _store_into(vg(fr), v)
        if t[0] == "apply":
            vg = self._var_getter(t[1], lookup, names)
            if vg is None:
                raise FortranError(f"assignment to unknown array {t[1]}")
            index, scalar = self._subscripts(t[2], lookup, names)

            def st(fr, v):
                var = vg(fr)
                arr = var.val
                idx = index(fr, arr)
                if scalar:
                    for q, ix in enumerate(idx):
                        if ix < 0 or ix >= arr.data.shape[q]:
                            raise FortranError(f"subscript {ix + arr.lb[q]} out of bounds in {t[1]}")
                    if var.base == "complex":
                        if isinstance(v, Cx):
                            rt = np.float32 if arr.data.dtype == np.complex64 else np.float64
                            arr.data[idx] = complex(rt(v.re), rt(v.im))
                        else:
                            arr.data[idx] = _to_storage(v, "complex", var.kind)
                    else:
                        arr.data[idx] = _to_storage(v, var.base, var.kind)
                    return
                view = arr.data[idx]
                if isinstance(v, FArr):
                    v = _value_of_storage(v, var.base)
                if var.base == "complex":
                    if isinstance(v, Cx):
                        view.real[...] = v.re
                        view.imag[...] = v.im
                    else:
                        view[...] = _to_storage(v, "complex", var.kind)
                else:
                    view[...] = _to_storage(v, var.base, var.kind)
            return st
        raise FortranError(f"assignment target {t!r}")

    def _cstmt(self, s, lookup, names):
        k = s[0]
        if k == "assign":
            tgt = self._ctarget(s[1], lookup, names)
            val = self._cexpr(s[2], lookup, names)
            return lambda fr: tgt(fr, val(fr))
        if k == "if":
            branches = [(self._cexpr(c, lookup, names), self._cblock(b, lookup, names)) for c, b in s[1]]
            els = self._cblock(s[2], lookup, names)

            def if_(fr):
                for c, b in branches:
                    if c(fr):
                        b(fr)
                        return
                els(fr)
            return if_
        if k == "do":
            vname = s[1]
            vg = self._var_getter(vname, lookup, names)
            flo, fhi = self._cexpr(s[2], lookup, names), self._cexpr(s[3], lookup, names)
            fst = self._cexpr(s[4], lookup, names) if s[4] is not None else (lambda fr: 1)
            body = self._cblock(s[5], lookup, names)

            def do_(fr):
                var = vg(fr)
                lo, hi, st = int(flo(fr)), int(fhi(fr)), int(fst(fr))
                v = lo
                for v in range(lo, hi + (1 if st > 0 else -1), st):
                    var.val = v
                    try:
                        body(fr)
                    except _Cycle:
                        continue
                    except _Exit:
                        return
                else:
                    var.val = v + st if (hi - lo) * st >= 0 else lo
            return do_
        if k == "dowhile":
            cond = self._cexpr(s[1], lookup, names)
            body = self._cblock(s[2], lookup, names)

            def dw(fr):
                while cond(fr):
                    try:
                        body(fr)
                    except _Cycle:
                        continue
                    except _Exit:
                        return
            return dw
        if k == "select":
            sel = self._cexpr(s[1], lookup, names)
            cases = []
            default = None
            for vals, body in s[2]:
                b = self._cblock(body, lookup, names)
                if vals is None:
                    default = b
                else:
                    cases.append(([self._cexpr(v, lookup, names) for v in vals], b))

            def sel_(fr):
                x = sel(fr)
                if isinstance(x, str):
                    x = x.rstrip()
                for vs, b in cases:
                    for v in vs:
                        y = v(fr)
                        if isinstance(y, str):
                            y = y.rstrip()
                        if x == y:
                            b(fr)
                            return
                if default is not None:
                    default(fr)
            return sel_
        if k == "call":
            return self._ccall(s[1], s[2], lookup, names)
        if k == "return":
            def ret(fr):
                raise _Return()
            return ret
        if k == "stop":
            def stop(fr):
                raise _Stop()
            return stop
        if k == "exit":
            def ex(fr):
                raise _Exit()
            return ex
        if k == "cycle":
            def cy(fr):
                raise _Cycle()
            return cy
        if k == "nop":
            return lambda fr: None
        if k == "allocate":
            items = []
            for name, dims in s[1]:
                vg = self._var_getter(name, lookup, names)
                fd = [(self._cexpr(lo, lookup, names), self._cexpr(hi, lookup, names)) for lo, hi in dims]
                items.append((vg, fd))

            def alloc(fr):
                for vg, fd in items:
                    var = vg(fr)
                    lbs = [int(lo(fr)) for lo, hi in fd]
                    shape = [max(0, int(hi(fr)) - lb + 1) for (lo, hi), lb in zip(fd, lbs)]
                    var.val = FArr(np.zeros(shape, dtype=self._dtype(var.base, var.kind)), lbs)
            return alloc
        if k == "deallocate":
            vgs = [self._var_getter(n, lookup, names) for n in s[1]]

            def dealloc(fr):
                for vg in vgs:
                    vg(fr).val = None
            return dealloc
        if k.endswith("_io"):
            return self._cio(k[:-3], s[1], s[2], lookup, names)
        raise FortranError(f"statement {s!r}")

    def _ccall(self, name, args, lookup, names):
        r = lookup(name)
        if r is not None and r[0] == "proc":
            mi, unit = r[1]
            fargs = [self._carg(a, lookup, names) for a in args]
            return lambda fr: self.call(self.proc(mi, unit), [f(fr) for f in fargs])
        if name in SUBROUTINES:
            sub = SUBROUTINES[name]
            fpos, fkw = [], {}
            for a in args:
                if a[0] == "kw":
                    fkw[a[1]] = self._carg(a[2], lookup, names)
                else:
                    fpos.append(self._carg(a, lookup, names))
            return lambda fr: sub(self, [f(fr) for f in fpos], {k: f(fr) for k, f in fkw.items()})
        raise FortranError(f"unknown subroutine {name}")

    # ---- I/O
    def _path(self, name):
        return os.path.normpath(os.path.join(self.workdir, str(name).strip()))

    def _cio(self, kind, specs, items, lookup, names):
        fspec = {k: (self._cexpr(v, lookup, names) if v != ("name", "*") else (lambda fr: "*"))
                 for k, v in specs.items() if k not in ("exist",)}
        exist_ref = self._carg(specs["exist"], lookup, names) if "exist" in specs else None
        internal = None
        if kind == "write" and specs.get("unit", ("", ""))[0] == "name" and specs["unit"][1] != "*":
            vg = self._var_getter(specs["unit"][1], lookup, names)
            if vg is not None:
                internal = vg
        if kind == "read":
            frefs = [self._carg(it, lookup, names) for it in items]
        else:
            fitems = [self._cexpr(it, lookup, names) for it in items]

        def io(fr):
            sp = {k: f(fr) for k, f in fspec.items()}
            if kind == "inquire":
                exist_ref(fr).set(os.path.exists(self._path(sp["file"])))
                return
            if kind == "open":
                path = self._path(sp["file"])
                form = str(sp.get("form", "formatted")).strip().lower()
                status = str(sp.get("status", "unknown")).strip().lower()
                if status == "replace" or not os.path.exists(path):
                    fh = open(path, "w+b")
                else:
                    fh = open(path, "r+b")
                self.files[int(sp["unit"])] = (fh, form)
                return
            if kind == "close":
                u = int(sp["unit"])
                if u in self.files:
                    self.files.pop(u)[0].close()
                return
            if kind == "write":
                vals = [f(fr) for f in fitems]
                fmt = sp.get("fmt")
                if internal is not None:
                    text = _format(fmt, vals) if fmt not in (None, "*") else _list_directed(vals)
                    _store_into(internal(fr), text)
                    return
                unit = sp.get("unit", "*")
                if unit == "*" or unit == 6:
                    self.stdout.append(_list_directed(vals) if fmt in (None, "*") else _format(fmt, vals))
                    return
                fh, form = self.files[int(unit)]
                if form == "unformatted":
                    payload = _record_bytes(vals)
                    n = struct.pack("<i", len(payload))
                    fh.write(n + payload + n)
                else:
                    text = _list_directed(vals) if fmt in (None, "*") else _format(fmt, vals)
                    fh.write((text + "\n").encode("latin-1"))
                fh.truncate()
                fh.flush()
                return
            if kind == "read":
                fh, form = self.files[int(sp["unit"])]
                if form != "unformatted":
                    raise FortranError("formatted read is not supported")
                n = struct.unpack("<i", fh.read(4))[0]
                payload = fh.read(n)
                fh.read(4)
                off = 0
                for f in frefs:
                    ref = f(fr)
                    var = ref.var
                    cur = ref.get()
                    if isinstance(cur, FArr):
                        dt = cur.data.dtype
                        cnt = cur.data.size
                        arr = np.frombuffer(payload, dtype=dt if dt.kind != "i" else np.int32, count=cnt,
                                            offset=off).reshape(cur.data.shape, order="F")
                        off += cnt * arr.dtype.itemsize
                        ref.set(FArr(arr.astype(dt), cur.lb))
                    else:
                        if var.base == "integer":
                            ref.set(struct.unpack_from("<i", payload, off)[0])
                            off += 4
                        elif var.base == "real":
                            dt = _rdt(var.kind)
                            ref.set(np.frombuffer(payload, dtype=dt, count=1, offset=off)[0])
                            off += np.dtype(dt).itemsize
                        elif var.base == "complex":
                            dt = _rdt(var.kind)
                            a = np.frombuffer(payload, dtype=dt, count=2, offset=off)
                            ref.set(Cx(a[0], a[1]))
                            off += 2 * np.dtype(dt).itemsize
                        else:
                            raise FortranError(f"unformatted read into {var.base}")
                return
            raise FortranError(kind)
        return io

    # ---- driver
    def run_program(self):
        prog = [u for u in self.units.values() if u.kind == "program"][0]
        mi = ModuleInst(prog)
        mi.uses = [self.module(u) for u in prog.uses]
        lookup = lambda nm: self._lookup_mod(mi, nm)
        for d in prog.decls:
            mi.vars[d["name"]] = self._declare(d, lookup)
        blk, _ = parse_block(prog.body)
        body = self._cblock(blk, lookup, set())
        try:
            body({})
        except _Stop:
            pass


# ------------------------------------------------------------- intrinsics --
# gfortran calls the C math library for the intrinsic functions (expf / exp,
# atan2f / atan2, cabsf = hypotf / cabs = hypot, powf / pow, ...): call the
# same functions of this machine's libm.
import ctypes as _ct
import ctypes.util as _ctu

_LIBM = _ct.CDLL(_ctu.find_library("m") or "libm.so.6")


def _libm(name, nargs):
    f64 = getattr(_LIBM, name)
    f64.restype = _ct.c_double
    f64.argtypes = [_ct.c_double] * nargs
    f32 = getattr(_LIBM, name + "f")
    f32.restype = _ct.c_float
    f32.argtypes = [_ct.c_float] * nargs

    def call(*args):
        if isinstance(args[0], np.float32):
            return np.float32(f32(*[float(a) for a in args]))
        return np.float64(f64(*[float(a) for a in args]))
    return call


LIBM = {n: _libm(n, k) for n, k in (("exp", 1), ("sin", 1), ("cos", 1), ("tan", 1), ("tanh", 1), ("acos", 1),
                                      ("asin", 1), ("atan", 1), ("log", 1), ("atan2", 2), ("hypot", 2),
                                      ("pow", 2))}


def _unary_real(name, x, kind_default):
    fn = LIBM[name]
    if isinstance(x, np.ndarray):
        return np.vectorize(lambda v: fn(v), otypes=[x.dtype])(x)
    if _is_int(x):
        x = _rdt(kind_default)(x)
    return fn(x)


def _i_abs(it, a, kw):
    x = a[0]
    if isinstance(x, Cx):   # cabs: hypot of the two parts
        if isinstance(x.re, np.ndarray):
            return np.vectorize(lambda u, v: LIBM["hypot"](u, v), otypes=[x.re.dtype])(x.re, x.im)
        return LIBM["hypot"](x.re, x.im)
    if _is_int(x):
        return abs(int(x))
    return np.abs(x)


def _i_exp(it, a, kw):
    x = a[0]
    if isinstance(x, Cx):
        if isinstance(x.re, np.ndarray):
            raise FortranError("complex exp of an array")
        # cexp: exp(re) * (cos(im), sin(im)), each factor from libm, in the kind of x
        e = LIBM["exp"](x.re)
        return Cx(e * LIBM["cos"](x.im), e * LIBM["sin"](x.im))
    return _unary_real("exp", x, it.rk)


def _i_sqrt(it, a, kw):
    x = a[0]
    if isinstance(x, Cx):
        raise FortranError("complex sqrt is not supported")
    if _is_int(x):
        x = _rdt(it.rk)(x)
    return np.sqrt(x)


def _i_real(it, a, kw):
    x = a[0]
    kind = int(kw["kind"]) if "kind" in kw else (int(a[1]) if len(a) > 1 else None)
    if isinstance(x, Cx):
        v = x.re
        return v if kind is None else _conv_real(v, kind)
    return _conv_real(_as_real(x, it.rk), kind or it.rk) if kind or _is_int(x) or (
        isinstance(x, np.ndarray) and x.dtype.kind in "iu") else x


def _i_cmplx(it, a, kw):
    kind = int(kw["kind"]) if "kind" in kw else it.rk
    x = a[0]
    y = a[1] if len(a) > 1 else 0
    if isinstance(x, Cx):
        return _conv_cx(x, kind)
    return Cx(_conv_real(_as_real(x, kind), kind), _conv_real(_as_real(y, kind), kind))


def _i_maxmin(fn):
    def f(it, a, kw):
        cats = [_num_kind(v) for v in a]
        if all(c == "i" for c, _ in cats):
            return fn(int(v) for v in a)
        k = max(kk for _, kk in cats) or it.rk
        vals = [_conv_real(_as_real(v, k), k) for v in a]
        out = vals[0]
        for v in vals[1:]:
            out = fn(out, v) if not isinstance(out, np.ndarray) else (np.maximum(out, v) if fn is max else np.minimum(out, v))
        return out
    return f


def _i_sum(it, a, kw):
    x = a[0]
    if isinstance(x, Cx):
        raise FortranError("complex sum is not supported")
    flat = np.ravel(x, order="F")
    if flat.size == 0:
        return flat.dtype.type(0)
    return np.add.accumulate(flat)[-1]


def _i_mod(it, a, kw):
    x, p = a
    if _is_int(x) and _is_int(p):
        return x - _int_div(x, p) * p
    k = max(_num_kind(x)[1], _num_kind(p)[1]) or it.rk
    return _conv_real(np.fmod(_conv_real(_as_real(x, k), k), _conv_real(_as_real(p, k), k)), k)


def _kind_arg(it, x):
    if isinstance(x, Cx):
        return _kind_of_real(x.re)
    if isinstance(x, (np.float32,)) or (isinstance(x, np.ndarray) and x.dtype == np.float32):
        return 4
    if isinstance(x, (np.float64, float)) or (isinstance(x, np.ndarray) and x.dtype == np.float64):
        return 8
    return None


def _i_epsilon(it, a, kw):
    k = _kind_arg(it, a[0]) or it.rk
    return _rdt(k)(np.finfo(_rdt(k)).eps)


def _i_huge(it, a, kw):
    if _is_int(a[0]):
        return 2 ** 31 - 1
    k = _kind_arg(it, a[0]) or it.rk
    return _rdt(k)(np.finfo(_rdt(k)).max)


def _i_atan2(it, a, kw):
    y, x = a
    k = max(_num_kind(y)[1], _num_kind(x)[1]) or it.rk
    y, x = _conv_real(_as_real(y, k), k), _conv_real(_as_real(x, k), k)
    return LIBM["atan2"](y, x)


INTRINSICS = {
    "abs": _i_abs,
    "sqrt": _i_sqrt,
    "exp": _i_exp,
    "sin": lambda it, a, kw: _unary_real("sin", a[0], it.rk),
    "cos": lambda it, a, kw: _unary_real("cos", a[0], it.rk),
    "tan": lambda it, a, kw: _unary_real("tan", a[0], it.rk),
    "tanh": lambda it, a, kw: _unary_real("tanh", a[0], it.rk),
    "acos": lambda it, a, kw: _unary_real("acos", a[0], it.rk),
    "asin": lambda it, a, kw: _unary_real("asin", a[0], it.rk),
    "atan": lambda it, a, kw: _unary_real("atan", a[0], it.rk),
    "log": lambda it, a, kw: _unary_real("log", a[0], it.rk),
    "atan2": _i_atan2,
    "real": _i_real,
    "dble": lambda it, a, kw: _conv_real(_as_real(a[0].re if isinstance(a[0], Cx) else a[0], 8), 8),
    "aimag": lambda it, a, kw: a[0].im,
    "imag": lambda it, a, kw: a[0].im,
    "conjg": lambda it, a, kw: Cx(a[0].re, -a[0].im),
    "cmplx": _i_cmplx,
    "max": _i_maxmin(max),
    "min": _i_maxmin(min),
    "maxval": lambda it, a, kw: np.max(a[0]),
    "minval": lambda it, a, kw: np.min(a[0]),
    "sum": _i_sum,
    "mod": _i_mod,
    "epsilon": _i_epsilon,
    "huge": _i_huge,
    "isnan": lambda it, a, kw: bool(np.isnan(a[0])),
    "achar": lambda it, a, kw: chr(int(a[0])),
    "floor": lambda it, a, kw: int(math.floor(float(a[0]))),
    "int": lambda it, a, kw: int(a[0]) if _is_int(a[0]) else int(float(a[0])),
    "nint": lambda it, a, kw: int(math.floor(abs(float(a[0])) + 0.5)) * (1 if float(a[0]) >= 0 else -1),
    "sign": lambda it, a, kw: (abs(a[0]) if float(a[1]) >= 0 else -abs(a[0])),
    "size": lambda it, a, kw: int(np.size(a[0])) if len(a) == 1 else int(np.shape(a[0])[int(a[1]) - 1]),
    "trim": lambda it, a, kw: str(a[0]).rstrip(),
    "float": lambda it, a, kw: np.float32(a[0]),
}

INTRINSIC_CONST = {}


# --------------------------------------------------- intrinsic subroutines --
def _set(r, v):
    if isinstance(r, Ref):
        r.set(v)


def _get(r):
    return r.get() if isinstance(r, Ref) else r


def _payload(v):
    if isinstance(v, FArr):
        return FArr(v.data.copy(), v.lb)
    if isinstance(v, Cx):
        return Cx(np.copy(v.re), np.copy(v.im)) if isinstance(v.re, np.ndarray) else Cx(v.re, v.im)
    if isinstance(v, np.ndarray):
        return v.copy()
    return v


def _mpi_dims(n, ndims):
    # balanced factorisation, non-increasing (MPI_Dims_create)
    dims = [1] * ndims
    rem = n
    f = 2
    factors = []
    while rem > 1:
        while rem % f == 0:
            factors.append(f)
            rem //= f
        f += 1
    for p in sorted(factors, reverse=True):
        i = dims.index(min(dims))
        dims[i] *= p
    return sorted(dims, reverse=True)


def _cart_rank(it, coords):
    return coords[0] * it.cart["dims"][1] + coords[1]


def _mpi_init(it, a, kw):
    _set(a[-1], 0)


def _mpi_comm_size(it, a, kw):
    _set(a[1], it.world.n)
    _set(a[2], 0)


def _mpi_comm_rank(it, a, kw):
    _set(a[1], it.rank)
    _set(a[2], 0)


def _mpi_dims_create(it, a, kw):
    d = _mpi_dims(int(_get(a[0])), int(_get(a[1])))
    _set(a[2], np.array(d, dtype=np.int64))
    _set(a[3], 0)


def _mpi_cart_create(it, a, kw):
    dims = [int(x) for x in np.ravel(_get(a[2]).data if isinstance(_get(a[2]), FArr) else _get(a[2]))]
    per = [bool(x) for x in np.ravel(_get(a[3]).data if isinstance(_get(a[3]), FArr) else _get(a[3]))]
    it.cart = {"dims": dims, "periods": per}
    _set(a[5], 92)
    _set(a[6], 0)


def _coords(it, rank):
    d = it.cart["dims"]
    return [rank // d[1], rank % d[1]]


def _mpi_cart_coords(it, a, kw):
    _set(a[3], np.array(_coords(it, int(_get(a[1]))), dtype=np.int64))
    _set(a[4], 0)


def _mpi_cart_shift(it, a, kw):
    direction, disp = int(_get(a[1])), int(_get(a[2]))
    c = _coords(it, it.rank)
    out = []
    for s in (-disp, disp):
        cc = list(c)
        cc[direction] += s
        n = it.cart["dims"][direction]
        if 0 <= cc[direction] < n:
            out.append(_cart_rank(it, cc))
        elif it.cart["periods"][direction]:
            cc[direction] %= n
            out.append(_cart_rank(it, cc))
        else:
            out.append(MPI_CONSTS["mpi_proc_null"])
    _set(a[3], out[0])
    _set(a[4], out[1])
    _set(a[5], 0)


def _mpi_isend(it, a, kw):
    it.world.post(it.rank, int(_get(a[3])), int(_get(a[4])), _payload(_get(a[0])))
    it.nreq += 1
    it.reqs[it.nreq] = ("send",)
    _set(a[6], it.nreq)
    _set(a[7], 0)


def _mpi_irecv(it, a, kw):
    it.nreq += 1
    it.reqs[it.nreq] = ("recv", int(_get(a[3])), int(_get(a[4])), a[0])
    _set(a[6], it.nreq)
    _set(a[7], 0)


def _mpi_wait(it, a, kw):
    req = it.reqs.pop(int(_get(a[0])))
    if req[0] == "recv":
        data = it.world.take(req[1], it.rank, req[2])
        req[3].set(data)
    _set(a[2], 0)


def _mpi_barrier(it, a, kw):
    it.world.sync()
    _set(a[1], 0)


def _combine(op, vals):
    out = vals[0]
    for v in vals[1:]:
        if op == MPI_CONSTS["mpi_sum"]:
            out = arith("+", out, v)
        elif op == MPI_CONSTS["mpi_max"]:
            out = max(out, v)
        elif op == MPI_CONSTS["mpi_min"]:
            out = min(out, v)
        elif op == MPI_CONSTS["mpi_land"]:
            out = bool(out) and bool(v)
        else:
            raise FortranError(f"MPI op {op}")
    return out


def _mpi_reduce(it, a, kw):
    w = it.world
    w.slots[it.rank] = _payload(_get(a[0]))
    w.sync()
    if it.rank == int(_get(a[5])):
        _set(a[1], _combine(int(_get(a[4])), list(w.slots)))
    w.sync()
    _set(a[7], 0)


def _mpi_bcast(it, a, kw):
    w = it.world
    root = int(_get(a[3]))
    if it.rank == root:
        w.slots[root] = _payload(_get(a[0]))
    w.sync()
    if it.rank != root:
        v = w.slots[root]
        a[0].set(v.data if isinstance(v, FArr) else v)
    w.sync()
    _set(a[5], 0)


def _random_seed(it, a, kw):
    if "size" in kw:
        _set(kw["size"], 8)


def _random_number(it, a, kw):
    cur = _get(a[0])
    if isinstance(cur, FArr):
        a[0].set(it.rng.random_sample(cur.data.shape).astype(cur.data.dtype))
    else:
        a[0].set(_rdt(it.rk)(it.rng.random_sample()))


SUBROUTINES = {
    "mpi_init": _mpi_init,
    "mpi_finalize": _mpi_init,
    "mpi_comm_size": _mpi_comm_size,
    "mpi_comm_rank": _mpi_comm_rank,
    "mpi_dims_create": _mpi_dims_create,
    "mpi_cart_create": _mpi_cart_create,
    "mpi_cart_coords": _mpi_cart_coords,
    "mpi_cart_shift": _mpi_cart_shift,
    "mpi_isend": _mpi_isend,
    "mpi_irecv": _mpi_irecv,
    "mpi_wait": _mpi_wait,
    "mpi_barrier": _mpi_barrier,
    "mpi_reduce": _mpi_reduce,
    "mpi_bcast": _mpi_bcast,
    "cpu_time": lambda it, a, kw: _set(a[0], _rdt(it.rk)(0.0)),
    "system_clock": lambda it, a, kw: _set(a[0], 0),
    "random_seed": _random_seed,
    "random_number": _random_number,
}


def run(source_dir, files, includes, nprocs, real_kind, workdir, timeout=3600.0):
    """Run `program run` of the given source files on `nprocs` virtual ranks.
    Returns the per-rank interpreters (module variables, captured stdout)."""
    stmts = []
    for f in files:
        stmts.extend(load_statements(os.path.join(source_dir, f), includes))
    units = parse_units(stmts, real_kind)
    world = World(nprocs, timeout=timeout)
    ranks = [Interp(units, real_kind, r, world, workdir) for r in range(nprocs)]
    errors = [None] * nprocs
    traces = [None] * nprocs

    def go(r):
        try:
            ranks[r].run_program()
        except BaseException as ex:   # noqa: BLE001 -- reported to the caller
            import traceback
            errors[r] = ex
            traces[r] = traceback.format_exc()
            world.failed = repr(ex)
            with world.lock:
                world.lock.notify_all()
            world.barrier.abort()

    if nprocs == 1:
        go(0)
    else:
        ts = [threading.Thread(target=go, args=(r,)) for r in range(nprocs)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
    first = [r for r, e in enumerate(errors) if e is not None and not str(e).startswith(("barrier broken",
                                                                                        "another rank failed"))]
    for r in first + [r for r, e in enumerate(errors) if e is not None]:
        raise FortranError(f"rank {r}: {errors[r]!r}\n{traces[r]}")
    return ranks
