"""Translator of the Fortran 90 subset used by OpenMHD's serial CPU path into C.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (openmhd_gb300/) imports or
runs this module.  It exists because no Fortran compiler is available where
this project is built or tested: it turns the reference's own source files
(u2v.f90, limiter.f90, flux_solver.f90, rk.f90, glm_ss2.f90, set_dt.f90,
bc.f90, model.f90, main.f90, flux_resistive.f90 of a problem directory) into
C mechanically, statement by statement, so that the reference's arithmetic can
be executed and compared with the hand-written oracle (omhd_oracle.c) bit for
bit.  The generated C and the library built from it go to oracle/_ref/ only.

What is translated, and how (the choices follow gfortran's code generation):

* program units: subroutine, function (with a result variable named like the
  function), program; every dummy argument is passed by reference, as the
  reference's implicit interfaces do;
* declarations: integer, real(8), logical, character*N; attributes intent(...),
  parameter, dimension bounds lo:hi; initialised locals are saved (static), as
  Fortran gives them the SAVE attribute; local arrays are heap-allocated;
* statements: assignment (scalars, elements, array sections and whole arrays,
  evaluated through a temporary when the left-hand array appears on the right,
  which is Fortran's semantics of an array assignment), do loops (trip count
  fixed on entry), if / else if / else, one-line if, select case, call, exit,
  cycle, return, stop (records the line and returns to the caller through every
  active call), continue; write and format statements are dropped (the
  reference's diagnostics), and so is any statement carrying a numeric label
  reference such as open(...,err=100);
* OpenMP directives (!$omp): parallel do with private / reduction / collapse
  clauses (a reduction on a dummy argument goes through a local copy; private
  arrays start from their values before the loop, the serial semantics),
  parallel regions with do, workshare (as single) and barrier, as the
  corresponding C pragmas; fixed-size local arrays become C arrays, so that
  they can be private to a thread;
* expressions: Fortran precedence (** right-associative, unary sign on the
  first term of an additive expression), integer and real(8) arithmetic mapped
  to the same C types (C's usual conversions match Fortran's mixed-mode rules
  for these types), real literals without a d exponent kept in single
  precision as Fortran defines them, x**n for a constant integer n as the
  multiplication chain gfortran emits (x*x for n = 2, 1/(x*x) for n = -2),
  dot_product as a sum started at zero in index order, sign(a,b) as
  copysign(|a|, b), min/max left to right, minloc/maxloc of whole arrays and
  planes, elemental intrinsics from libm.

The generated C is compiled with -O2 -ffp-contract=off -fno-fast-math, so each
Fortran operation is one IEEE-754 double operation in source order.

Usage (as oracle/ref.py does):
    units = parse_files([...paths...], include_dir)
    c_text = emit_c(units, prefix="f90_", overrides={"ix": "34", ...},
                    hooks={"fileio_output": ...})
"""
from __future__ import annotations

import os
import re
from dataclasses import dataclass, field


class TranslateError(RuntimeError):
    pass


# ---------------------------------------------------------------------------
# source lines -> statements
# ---------------------------------------------------------------------------
@dataclass
class Stmt:
    text: str          # lower-cased outside strings, no comments, no label
    label: str | None
    file: str
    line: int


def _strip_comment(line: str) -> str:
    q = None
    for k, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "!":
            return line[:k]
    return line


def _lower_outside_strings(s: str) -> str:
    out, q = [], None
    for ch in s:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        else:
            out.append(ch.lower())
    return "".join(out)


def _split_semicolons(s: str) -> list[str]:
    parts, cur, q = [], [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            cur.append(ch)
        elif ch == ";":
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return [p.strip() for p in parts if p.strip()]


def read_statements(path: str, include_dir: str | None = None) -> list[Stmt]:
    include_dir = include_dir or os.path.dirname(path)
    with open(path, encoding="latin-1") as f:
        raw = f.read().splitlines()
    stmts: list[Stmt] = []
    buf, start = "", 0
    dbuf, dstart = None, 0
    for n, line in enumerate(raw, 1):
        ls = line.strip()
        if ls.lower().startswith("!$omp"):  # OpenMP directive (continued with a trailing &)
            d = ls[5:].strip()
            cont = d.endswith("&")
            if cont:
                d = d[:-1].strip()
            if dbuf is None:
                dbuf, dstart = d, n
            else:
                dbuf += " " + d
            if not cont:
                stmts.append(Stmt("!$omp " + _lower_outside_strings(dbuf), None, os.path.basename(path), dstart))
                dbuf = None
            continue
        body = _strip_comment(line).rstrip()
        if not body.strip():
            if buf:
                continue  # blank or comment line inside a continued statement
            continue
        s = body.strip()
        if buf:
            if s.startswith("&"):
                s = s[1:]
            buf += " " + s
        else:
            buf, start = s, n
        if buf.endswith("&"):
            buf = buf[:-1]
            continue
        text = _lower_outside_strings(buf.strip())
        buf = ""
        m = re.match(r"include\s+['\"]([^'\"]+)['\"]\s*$", text)
        if m:
            stmts.extend(read_statements(os.path.join(include_dir, m.group(1)), include_dir))
            continue
        for part in _split_semicolons(text):
            lab = None
            m = re.match(r"(\d+)\s+(.*)$", part)
            if m:
                lab, part = m.group(1), m.group(2)
            stmts.append(Stmt(part, lab, os.path.basename(path), start))
    return stmts


# ---------------------------------------------------------------------------
# expressions
# ---------------------------------------------------------------------------
_OPWORDS = {"eq", "ne", "lt", "le", "gt", "ge", "and", "or", "not", "eqv", "neqv", "true", "false"}
_TOKEN = re.compile(r"""
    (?P<ws>\s+)
  | (?P<str>'[^']*'|"[^"]*")
  | (?P<real>(\d+\.\d*|\.\d+)([de][+-]?\d+)?|\d+[de][+-]?\d+)
  | (?P<int>\d+)
  | (?P<dotop>\.[a-z]+\.)
  | (?P<name>[a-z_][a-z0-9_]*)
  | (?P<op>\*\*|==|/=|<=|>=|\(/|/\)|[-+*/(),:<>=%])
""", re.X)


def tokenize(s: str) -> list[tuple[str, str]]:
    toks, k = [], 0
    while k < len(s):
        m = _TOKEN.match(s, k)
        if not m:
            raise TranslateError(f"cannot tokenise {s[k:]!r} in {s!r}")
        kind = m.lastgroup
        text = m.group(kind)
        if kind == "real":
            # "1.and." style: the dot belongs to an operator word
            mm = re.match(r"(\d+)\.([a-z]+)\.", s[k:])
            if mm and mm.group(2) in _OPWORDS:
                toks.append(("int", mm.group(1)))
                k += len(mm.group(1))
                continue
        if kind == "dotop" and text[1:-1] not in _OPWORDS:
            raise TranslateError(f"unknown operator {text} in {s!r}")
        if kind != "ws":
            toks.append((kind, text))
        k = m.end()
    return toks


@dataclass
class Num:
    text: str
    type: str  # int | double | float


@dataclass
class Name:
    name: str


@dataclass
class Ref:  # name(args): array element / section, or function call
    name: str
    args: list


@dataclass
class Range:
    lo: object
    hi: object


@dataclass
class Bin:
    op: str
    a: object
    b: object


@dataclass
class Un:
    op: str
    a: object


@dataclass
class Cons:
    items: list


@dataclass
class Logical:
    value: bool


@dataclass
class Str:
    text: str


class Parser:
    REL = {"==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">=",
           ".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">="}

    def __init__(self, text: str):
        self.text = text
        self.t = tokenize(text)
        self.k = 0

    def peek(self, off=0):
        j = self.k + off
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, text=None):
        tok = self.peek()
        if text is not None and tok[1] != text:
            raise TranslateError(f"expected {text!r}, got {tok[1]!r} in {self.text!r}")
        self.k += 1
        return tok

    def done(self):
        return self.k >= len(self.t)

    def expr(self):
        a = self.and_()
        while self.peek()[1] in (".or.", ".eqv.", ".neqv."):
            op = self.take()[1]
            a = Bin({".or.": "||", ".eqv.": "==", ".neqv.": "!="}[op], a, self.and_())
        return a

    def and_(self):
        a = self.not_()
        while self.peek()[1] == ".and.":
            self.take()
            a = Bin("&&", a, self.not_())
        return a

    def not_(self):
        if self.peek()[1] == ".not.":
            self.take()
            return Un("!", self.not_())
        return self.rel()

    def rel(self):
        a = self.add()
        if self.peek()[1] in self.REL:
            op = self.REL[self.take()[1]]
            a = Bin(op, a, self.add())
        return a

    def add(self):
        if self.peek()[1] in ("+", "-"):
            sign = self.take()[1]
            a = self.mul()
            a = Un("-", a) if sign == "-" else a
        else:
            a = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = Bin(op, a, self.mul())
        return a

    def mul(self):
        a = self.pow()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            a = Bin(op, a, self.pow())
        return a

    def pow(self):
        a = self.primary()
        if self.peek()[1] == "**":
            self.take()
            if self.peek()[1] in ("+", "-"):  # x**-2 (an extension gfortran accepts)
                sign = self.take()[1]
                b = self.pow()
                b = Un("-", b) if sign == "-" else b
            else:
                b = self.pow()
            return Bin("**", a, b)
        return a

    def primary(self):
        kind, text = self.peek()
        if kind == "real":
            self.take()
            if "d" in text:
                return Num(text.replace("d", "e"), "double")
            return Num(text, "float")
        if kind == "int":
            self.take()
            return Num(text, "int")
        if kind == "str":
            self.take()
            return Str(text)
        if text in (".true.", ".false."):
            self.take()
            return Logical(text == ".true.")
        if text == "(/":
            self.take()
            items = [self.expr()]
            while self.peek()[1] == ",":
                self.take()
                items.append(self.expr())
            self.take("/)")
            return Cons(items)
        if text == "(":
            self.take()
            e = self.expr()
            self.take(")")
            return e
        if kind == "name":
            self.take()
            if self.peek()[1] == "(":
                self.take()
                args = []
                if self.peek()[1] != ")":
                    args.append(self.arg())
                    while self.peek()[1] == ",":
                        self.take()
                        args.append(self.arg())
                self.take(")")
                return Ref(text, args)
            return Name(text)
        raise TranslateError(f"unexpected {text!r} in {self.text!r}")

    def arg(self):
        if self.peek()[1] == ":":
            self.take()
            hi = None if self.peek()[1] in (",", ")") else self.expr()
            return Range(None, hi)
        e = self.expr()
        if self.peek()[1] == ":":
            self.take()
            hi = None if self.peek()[1] in (",", ")") else self.expr()
            return Range(e, hi)
        if self.peek()[1] == "=":  # keyword argument (only in dropped I/O statements)
            raise TranslateError("keyword arguments are not part of the subset")
        return e


def parse_expr(text: str):
    p = Parser(text)
    e = p.expr()
    if not p.done():
        raise TranslateError(f"trailing tokens in {text!r}: {p.t[p.k:]}")
    return e


def split_top(text: str, sep: str) -> list[str]:
    """Split at `sep` characters outside parentheses and strings."""
    out, cur, depth, q = [], [], 0, None
    for ch in text:
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
            out.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    out.append("".join(cur))
    return [o.strip() for o in out]


def find_assign(text: str) -> int:
    """Index of the top-level '=' of an assignment, or -1."""
    depth, q = 0, None
    for k, ch in enumerate(text):
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
        elif ch == "=" and depth == 0:
            prev = text[k - 1] if k else ""
            nxt = text[k + 1] if k + 1 < len(text) else ""
            if prev in "<>/=" or nxt == "=":
                continue
            return k
    return -1


# ---------------------------------------------------------------------------
# program units and symbols
# ---------------------------------------------------------------------------
@dataclass
class Sym:
    name: str
    type: str                 # int | double | bool | char
    dims: list | None = None  # [(lo_ast, hi_ast)] ; None for scalars
    param: bool = False
    init: object = None
    dummy: bool = False
    saved: bool = False
    charlen: int = 0


@dataclass
class Unit:
    kind: str                 # subroutine | function | program
    name: str
    args: list
    decls: list = field(default_factory=list)  # declaration statements
    body: list = field(default_factory=list)   # executable statements
    syms: dict = field(default_factory=dict)
    result_type: str | None = None


_DECL = re.compile(r"(integer|real\s*\(\s*8\s*\)|real\*8|double\s+precision|logical|character\s*\*\s*\d+|"
                   r"character\s*\(\s*len\s*=\s*\d+\s*\))(?![a-z0-9_])(.*)$")
_HEAD = re.compile(r"(?:(real\s*\(\s*8\s*\)|integer)\s+)?(subroutine|function|program)\s+([a-z_][a-z0-9_]*)"
                   r"\s*(?:\((.*)\))?\s*$")


def _ctype(decl: str) -> tuple[str, int]:
    d = re.sub(r"\s+", "", decl)
    if d == "integer":
        return "int", 0
    if d in ("real(8)", "real*8", "doubleprecision"):
        return "double", 0
    if d == "logical":
        return "bool", 0
    m = re.match(r"character(?:\*(\d+)|\(len=(\d+)\))", d)
    if m:
        return "char", int(m.group(1) or m.group(2))
    raise TranslateError(f"unsupported type {decl}")


def parse_units(stmts: list[Stmt]) -> list[Unit]:
    units: list[Unit] = []
    cur: Unit | None = None
    in_decls = True
    for st in stmts:
        t = st.text
        if cur is None:
            m = _HEAD.match(t)
            if not m:
                raise TranslateError(f"{st.file}:{st.line}: statement outside a program unit: {t}")
            rtype, kind, name, args = m.groups()
            cur = Unit(kind, name, [a.strip() for a in args.split(",")] if args and args.strip() else [])
            if rtype:
                cur.result_type = _ctype(rtype)[0]
            in_decls = True
            continue
        if re.match(r"end(\s*(subroutine|function|program)\b.*)?$", t):
            units.append(cur)
            cur = None
            continue
        if t == "implicit none":
            continue
        if in_decls and _DECL.match(t) and ("::" in t or re.match(
                r"(integer|real\s*\(\s*8\s*\)|real\*8|logical|character\S*)\s+[a-z_]", t)):
            cur.decls.append(st)
            continue
        in_decls = False
        cur.body.append(st)
    if cur is not None:
        raise TranslateError(f"unterminated unit {cur.name}")
    for u in units:
        _declare(u)
    return units


def _declare(u: Unit):
    for st in u.decls:
        m = _DECL.match(st.text)
        ctype, clen = _ctype(m.group(1))
        rest = m.group(2).strip()
        attrs, ents = "", rest
        if "::" in rest:
            attrs, ents = rest.split("::", 1)
        attrs_l = [a.strip() for a in split_top(attrs, ",") if a.strip()]
        is_param = "parameter" in attrs_l
        dim_attr = None
        for a in attrs_l:
            mm = re.match(r"dimension\s*\((.*)\)$", a)
            if mm:
                dim_attr = mm.group(1)
        for ent in split_top(ents, ","):
            if not ent:
                continue
            init = None
            k = find_assign(ent)
            if k >= 0:
                ent, init = ent[:k].strip(), parse_expr(ent[k + 1:].strip())
            mm = re.match(r"([a-z_][a-z0-9_]*)\s*(?:\((.*)\))?$", ent)
            if not mm:
                raise TranslateError(f"{st.file}:{st.line}: bad entity {ent}")
            name, dims = mm.group(1), mm.group(2) or dim_attr
            dl = None
            if dims:
                dl = []
                for d in split_top(dims, ","):
                    if ":" in d:
                        lo, hi = d.split(":", 1)
                        dl.append((parse_expr(lo), parse_expr(hi)))
                    else:
                        dl.append((Num("1", "int"), parse_expr(d)))
            sym = Sym(name, ctype, dl, is_param, init, name in u.args, init is not None and not is_param, clen)
            u.syms[name] = sym
    if u.kind == "function" and u.name not in u.syms:
        u.syms[u.name] = Sym(u.name, u.result_type or "double")
    for a in u.args:
        if a not in u.syms:
            raise TranslateError(f"{u.name}: dummy argument {a} has no declaration (implicit typing is not supported)")


# ---------------------------------------------------------------------------
# C emission
# ---------------------------------------------------------------------------
INTRINSIC_D1 = {"sqrt", "exp", "log", "sin", "cos", "tan", "tanh", "cosh", "sinh", "atan", "asin", "acos", "log10"}

RUNTIME = r"""
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* translator runtime (oracle/f90sub.py) */
int PFX_stopped = 0;           /* source line of the last STOP, 0 if none */
static inline int f90_imin(int a, int b) { return b < a ? b : a; }
static inline int f90_imax(int a, int b) { return b > a ? b : a; }
static inline double f90_dmin(double a, double b) { return b < a ? b : a; }
static inline double f90_dmax(double a, double b) { return b > a ? b : a; }
static inline int f90_isign(int a, int b) { int m = a < 0 ? -a : a; return b >= 0 ? m : -m; }
static inline double f90_dsign(double a, double b) { return copysign(fabs(a), b); }
static inline double f90_powi(double a, int n) {
  /* gfortran's expansion of a**n for the constant exponents of this code */
  switch (n) {
    case 0: return 1.0;
    case 1: return a;
    case 2: return a * a;
    case 3: { double t = a * a; return t * a; }
    case 4: { double t = a * a; return t * t; }
    case -1: return 1.0 / a;
    case -2: return 1.0 / (a * a);
    default: return pow(a, (double)n);
  }
}
static inline int f90_ipowi(int a, int n) { int r = 1; for (int k = 0; k < n; ++k) r *= a; return r; }
/* column-major location (1-based) of the first minimum / maximum of n1*n2*n3 values */
static void f90_loc(const double* a, long n1, long n2, long n3, int* out, int rank, int is_max) {
  long best = 0;
  for (long k = 1; k < n1 * n2 * n3; ++k)
    if (is_max ? (a[k] > a[best]) : (a[k] < a[best])) best = k;
  long i = best % n1, j = (best / n1) % n2, l = best / (n1 * n2);
  out[0] = (int)i + 1;
  if (rank > 1) out[1] = (int)j + 1;
  if (rank > 2) out[2] = (int)l + 1;
}
"""


@dataclass
class Sec:
    """One array reference in an elementwise context."""
    sym: Sym
    args: list


class Emitter:
    def __init__(self, units: list[Unit], prefix: str, overrides: dict, hooks: dict):
        self.units = {u.name: u for u in units}
        self.prefix = prefix
        self.overrides = overrides
        self.hooks = hooks
        self.out: list[str] = []
        self.tmp = 0
        self.omp_pending = None  # (pragma kind, clause text) for the next do loop
        self.shadow: dict = {}   # dummy scalar -> local copy inside an OpenMP reduction

    # -- helpers --
    def fresh(self, base="_t"):
        self.tmp += 1
        return f"{base}{self.tmp}"

    def fname(self, name):
        return f"{self.prefix}{name}"

    def var(self, sym: Sym) -> str:
        if sym.name in self.shadow:
            return self.shadow[sym.name]
        if sym.dummy and not sym.dims and sym.type != "char":
            return f"(*{sym.name})"
        if self.u.kind == "function" and sym.name == self.u.name:
            return "_result"
        return sym.name

    def lookup(self, name):
        return self.u.syms.get(name)

    # -- types --
    def type_of(self, e) -> str:
        if isinstance(e, Num):
            return "int" if e.type == "int" else "double"
        if isinstance(e, Logical):
            return "bool"
        if isinstance(e, Name):
            s = self.lookup(e.name)
            if s is None:
                raise TranslateError(f"{self.u.name}: undeclared {e.name}")
            return "double" if s.type == "double" else ("bool" if s.type == "bool" else "int")
        if isinstance(e, Un):
            return "bool" if e.op == "!" else self.type_of(e.a)
        if isinstance(e, Bin):
            if e.op in ("&&", "||", "==", "!=", "<", "<=", ">", ">="):
                return "bool"
            ta, tb = self.type_of(e.a), self.type_of(e.b)
            if e.op == "**":
                return ta if ta == "double" or tb == "double" else "int"
            return "double" if "double" in (ta, tb) else "int"
        if isinstance(e, Ref):
            s = self.lookup(e.name)
            if s is not None and s.dims:
                return "double" if s.type == "double" else "int"
            n = e.name
            if n in INTRINSIC_D1 or n in ("dble", "dot_product"):
                return "double"
            if n in ("abs", "min", "max", "sign", "mod"):
                ts = [self.type_of(a) for a in e.args]
                return "double" if "double" in ts else "int"
            if n in ("int", "nint", "floor"):
                return "int"
            if n == "real":
                return "double"
            if s is not None:  # external function declared with a type
                return "double" if s.type == "double" else "int"
            if n in self.units and self.units[n].kind == "function":
                return self.units[n].result_type or "double"
            raise TranslateError(f"{self.u.name}: unknown function {n}")
        raise TranslateError(f"cannot type {e}")

    # -- array addressing --
    def dim_bounds(self, sym: Sym):
        """C expressions (lo, extent) per dimension."""
        out = []
        for lo, hi in sym.dims:
            lo_c = self.expr(lo)
            out.append((lo_c, f"(({self.expr(hi)}) - ({lo_c}) + 1)"))
        return out

    def flat_index(self, sym: Sym, idx: list[str]) -> str:
        b = self.dim_bounds(sym)
        term = f"((long)({idx[-1]}) - ({b[-1][0]}))"
        for d in range(len(idx) - 2, -1, -1):
            term = f"((long)({idx[d]}) - ({b[d][0]}) + (long)({b[d][1]}) * {term})"
        return term

    def elem(self, sym: Sym, idx: list[str]) -> str:
        return f"{self.var(sym)}[{self.flat_index(sym, idx)}]"

    def section_dims(self, sym: Sym, args: list):
        """[(dim, lo_c, hi_c)] for the section dimensions of a reference."""
        if not args:
            args = [Range(None, None)] * len(sym.dims)
        if len(args) != len(sym.dims):
            raise TranslateError(f"{self.u.name}: rank mismatch in reference to {sym.name}")
        out = []
        for d, a in enumerate(args):
            if isinstance(a, Range):
                lo = self.expr(a.lo) if a.lo is not None else self.expr(sym.dims[d][0])
                hi = self.expr(a.hi) if a.hi is not None else self.expr(sym.dims[d][1])
                out.append((d, lo, hi))
        return out

    def rank_of(self, e) -> int:
        if isinstance(e, Name):
            s = self.lookup(e.name)
            return len(s.dims) if s is not None and s.dims and not s.param else 0
        if isinstance(e, Ref):
            s = self.lookup(e.name)
            if s is not None and s.dims:
                return sum(isinstance(a, Range) for a in e.args)
            if e.name in ("dot_product", "minloc", "maxloc"):
                return 0
            return max([self.rank_of(a) for a in e.args] + [0])
        if isinstance(e, (Bin,)):
            return max(self.rank_of(e.a), self.rank_of(e.b))
        if isinstance(e, Un):
            return self.rank_of(e.a)
        return 0

    # -- expressions --
    def expr(self, e, loop: list[str] | None = None) -> str:
        """C text of e; `loop` are the counters of an elementwise context
        (section dimension k of every array reference uses loop[k])."""
        if isinstance(e, Num):
            if e.type == "int":
                return e.text
            if e.type == "float":
                return f"((double){e.text}f)" if "." in e.text or "e" in e.text else f"((double){e.text}.0f)"
            return e.text if ("." in e.text or "e" in e.text) else e.text + ".0"
        if isinstance(e, Logical):
            return "1" if e.value else "0"
        if isinstance(e, Str):
            raise TranslateError("strings are not part of the translated subset")
        if isinstance(e, Name):
            s = self.lookup(e.name)
            if s is None:
                raise TranslateError(f"{self.u.name}: undeclared {e.name}")
            if s.dims and not s.param:
                if loop is None:
                    raise TranslateError(f"{self.u.name}: whole array {e.name} outside an array context")
                return self.section_ref(s, [], loop)
            return self.var(s)
        if isinstance(e, Un):
            if e.op == "!":
                return f"(!{self.expr(e.a, loop)})"
            return f"(-{self.expr(e.a, loop)})"
        if isinstance(e, Bin):
            if e.op == "**":
                return self.power(e, loop)
            return f"({self.expr(e.a, loop)} {e.op} {self.expr(e.b, loop)})"
        if isinstance(e, Ref):
            s = self.lookup(e.name)
            if s is not None and s.dims:
                if any(isinstance(a, Range) for a in e.args):
                    if loop is None:
                        raise TranslateError(f"{self.u.name}: section of {e.name} outside an array context")
                    return self.section_ref(s, e.args, loop)
                return self.elem(s, [self.expr(a, loop) for a in e.args])
            return self.call_fn(e, loop)
        if isinstance(e, Cons):
            raise TranslateError("array constructor outside a parameter declaration")
        raise TranslateError(f"cannot emit {e}")

    def section_ref(self, s: Sym, args: list, loop: list[str]) -> str:
        secs = self.section_dims(s, args)
        if len(secs) != len(loop):
            raise TranslateError(f"{self.u.name}: non-conformable section of {s.name}")
        if not args:
            args = [Range(None, None)] * len(s.dims)
        idx, k = [], 0
        for d, a in enumerate(args):
            if isinstance(a, Range):
                idx.append(f"({secs[k][1]}) + {loop[k]}")
                k += 1
            else:
                idx.append(self.expr(a))
        return self.elem(s, idx)

    def power(self, e: Bin, loop) -> str:
        base = self.expr(e.a, loop)
        b = e.b
        n = None
        if isinstance(b, Num) and b.type == "int":
            n = int(b.text)
        elif isinstance(b, Un) and b.op == "-" and isinstance(b.a, Num) and b.a.type == "int":
            n = -int(b.a.text)
        if n is not None:
            if self.type_of(e.a) == "int":
                return f"f90_ipowi({base}, {n})"
            return f"f90_powi({base}, {n})"
        return f"pow({base}, {self.expr(b, loop)})"

    def call_fn(self, e: Ref, loop) -> str:
        n, args = e.name, e.args
        if n == "dot_product":
            a, b = args
            ra, rb = self.rank_of(a), self.rank_of(b)
            if ra != 1 or rb != 1:
                raise TranslateError("dot_product of rank-1 sections only")
            ctr = self.fresh("_r")
            sa = self.section_extent(a)
            acc = self.fresh("_acc")
            return (f"({{ double {acc} = 0.0; for (long {ctr} = 0; {ctr} < ({sa}); ++{ctr}) "
                    f"{acc} = {acc} + {self.expr(a, [ctr])} * {self.expr(b, [ctr])}; {acc}; }})")
        ts = [self.type_of(a) for a in args]
        cs = [self.expr(a, loop) for a in args]
        dbl = "double" in ts
        if n in ("min", "max"):
            f = ("f90_dmin" if n == "min" else "f90_dmax") if dbl else ("f90_imin" if n == "min" else "f90_imax")
            r = cs[0] if not dbl or ts[0] == "double" else f"(double)({cs[0]})"
            for c in cs[1:]:
                r = f"{f}({r}, {c})"
            return r
        if n == "abs":
            return f"fabs({cs[0]})" if dbl else f"abs({cs[0]})"
        if n == "sign":
            return f"f90_dsign({cs[0]}, {cs[1]})" if dbl else f"f90_isign({cs[0]}, {cs[1]})"
        if n == "mod":
            return f"fmod({cs[0]}, {cs[1]})" if dbl else f"(({cs[0]}) % ({cs[1]}))"
        if n == "dble" or (n == "real" and len(cs) in (1, 2)):
            return f"((double)({cs[0]}))"
        if n == "int":
            return f"((int)({cs[0]}))"
        if n == "nint":
            return f"((int)lround({cs[0]}))"
        if n in INTRINSIC_D1:
            return f"{n}({cs[0]})"
        # external function: arguments by reference
        if n in self.units and self.units[n].kind == "function":
            return f"{self.fname(n)}({', '.join(self.ref_arg(a) for a in args)})"
        raise TranslateError(f"{self.u.name}: unsupported function {n}")

    def section_extent(self, e) -> str:
        if isinstance(e, Name):
            s = self.lookup(e.name)
            secs = self.section_dims(s, [])
        else:
            s = self.lookup(e.name)
            secs = self.section_dims(s, e.args)
        if len(secs) != 1:
            raise TranslateError("rank-1 section expected")
        return f"(({secs[0][2]}) - ({secs[0][1]}) + 1)"

    def ref_arg(self, a) -> str:
        """An actual argument passed by reference."""
        if isinstance(a, Name):
            s = self.lookup(a.name)
            if s is None:
                raise TranslateError(f"{self.u.name}: undeclared {a.name}")
            if s.type == "char":
                return s.name
            if s.dims and not s.param:
                return self.var(s)
            if s.dummy:
                return s.name
            if s.param:
                ct = "double" if s.type == "double" else "int"
                return f"&({ct}){{{self.expr(a)}}}"
            if self.u.kind == "function" and s.name == self.u.name:
                return "&_result"
            return f"&{s.name}"
        if isinstance(a, Ref):
            s = self.lookup(a.name)
            if s is not None and s.dims:
                if any(isinstance(x, Range) for x in a.args):
                    # contiguous section: address of its first element
                    seen_scalar = False
                    idx = []
                    for d, x in enumerate(a.args):
                        if isinstance(x, Range):
                            if seen_scalar:
                                raise TranslateError(f"{self.u.name}: non-contiguous section argument {a.name}")
                            if x.lo is not None or x.hi is not None:
                                raise TranslateError(f"{self.u.name}: partial section argument {a.name}")
                            idx.append(self.expr(s.dims[d][0]))
                        else:
                            seen_scalar = True
                            idx.append(self.expr(x))
                    return f"&{self.elem(s, idx)}"
                return f"&{self.elem(s, [self.expr(x) for x in a.args])}"
        ct = "double" if self.type_of(a) == "double" else "int"
        return f"&({ct}){{{self.expr(a)}}}"

    # -- statements --
    def emit(self, line: str, depth: int):
        self.out.append("  " * depth + line)

    def const_int(self, e):
        """Value of an integer expression of literals and (not overridden)
        parameters, or None."""
        if isinstance(e, Num):
            return int(e.text) if e.type == "int" else None
        if isinstance(e, Name):
            sym = self.lookup(e.name)
            if sym is None or not sym.param or sym.dims or sym.type != "int" or e.name in self.param_override:
                return None
            return self.const_int(sym.init)
        if isinstance(e, Un) and e.op == "-":
            v = self.const_int(e.a)
            return None if v is None else -v
        if isinstance(e, Bin) and e.op in ("+", "-", "*"):
            x, y = self.const_int(e.a), self.const_int(e.b)
            if x is None or y is None:
                return None
            return x + y if e.op == "+" else (x - y if e.op == "-" else x * y)
        return None

    def const_size(self, s: Sym):
        n = 1
        for lo, hi in s.dims:
            a, b = self.const_int(lo), self.const_int(hi)
            if a is None or b is None:
                return None
            n *= max(b - a + 1, 0)
        return n

    def omp_clauses(self, text: str, depth: int) -> tuple[str, list]:
        """C clauses for an OpenMP directive's clause text, and the (dummy,
        local copy) pairs of reductions on dummy arguments."""
        out, copies = [], []
        for name, args in re.findall(r"([a-z_]+)\s*\(([^)]*)\)", text):
            if name == "private":
                # private scalars start undefined, as in Fortran; private arrays
                # start from the values they hold before the region
                # (firstprivate): the serial program's values, which the
                # reference relies on for entries its loops never set (e.g. the
                # side fluxes' normal-field slot zeroed before the face loop)
                keep, arrays = [], []
                for v in [x.strip() for x in args.split(",") if x.strip()]:
                    sym = self.lookup(v)
                    if sym is None:
                        raise TranslateError(f"private {v} is not declared")
                    if sym.dims and v not in self.fixed:
                        raise TranslateError(f"private array {v} has no fixed size")
                    if sym.dummy or sym.param:
                        continue
                    (arrays if sym.dims else keep).append(v)
                if keep:
                    out.append(f"private({', '.join(keep)})")
                if arrays:
                    out.append(f"firstprivate({', '.join(arrays)})")
            elif name == "reduction":
                op, names = args.split(":", 1)
                op = op.strip()
                cop = {"max": "max", "min": "min", "+": "+"}.get(op)
                if cop is None:
                    raise TranslateError(f"reduction {op} is not part of the subset")
                vs = []
                for v in [x.strip() for x in names.split(",") if x.strip()]:
                    sym = self.lookup(v)
                    if sym.dummy:
                        loc = self.fresh("_red")
                        ct = "double" if sym.type == "double" else "int"
                        self.emit(f"{ct} {loc} = (*{v});", depth)
                        copies.append((v, loc))
                        vs.append(loc)
                    else:
                        vs.append(v)
                out.append(f"reduction({cop}:{', '.join(vs)})")
            elif name == "collapse":
                out.append(f"collapse({int(args)})")
            elif name in ("shared", "firstprivate", "schedule", "default"):
                out.append(f"{name}({args})")
            else:
                raise TranslateError(f"OpenMP clause {name} is not part of the subset")
        return " ".join(out), copies

    def omp_directive(self, t: str, depth: int):
        d = t[len("!$omp"):].strip()
        if re.match(r"end\b", d):
            rest = d[3:].strip()
            if rest in ("parallel do", "do"):
                return
            if rest in ("parallel", "workshare"):
                self.emit("}", depth)
                return
            raise TranslateError(f"unsupported directive !$omp {d}")
        if d.startswith("parallel do"):
            self.omp_pending = ("parallel for", d[len("parallel do"):])
        elif d.startswith("parallel"):
            clauses, copies = self.omp_clauses(d[len("parallel"):], depth)
            if copies:
                raise TranslateError("reductions on dummies need a parallel do")
            self.emit(f"#pragma omp parallel {clauses}".rstrip(), depth)
            self.emit("{", depth)
        elif d.startswith("do"):
            self.omp_pending = ("for", d[2:])
        elif d == "workshare":  # one thread does the work; implicit barrier at its end
            self.emit("#pragma omp single", depth)
            self.emit("{", depth)
        elif d == "barrier":
            self.emit("#pragma omp barrier", depth)
        else:
            raise TranslateError(f"unsupported directive !$omp {d}")

    def unit(self, u: Unit):
        self.u = u
        self.fixed = set()
        self.omp_pending = None
        self.shadow = {}
        self.param_override = dict(self.overrides.get("program", {})) if u.kind == "program" else {}
        ps = []
        for a in u.args:
            s = u.syms[a]
            ct = {"double": "double", "int": "int", "bool": "int", "char": "char"}[s.type]
            ps.append(f"{ct}* {a}")
        if u.kind == "program":
            self.out.append(f"int {self.fname(u.name)}(void) {{")
        elif u.kind == "function":
            rt = "double" if u.syms[u.name].type == "double" else "int"
            self.out.append(f"{rt} {self.fname(u.name)}({', '.join(ps) or 'void'}) {{")
        else:
            self.out.append(f"void {self.fname(u.name)}({', '.join(ps) or 'void'}) {{")
        frees = []
        # parameters first (in declaration order), then locals
        for s in u.syms.values():
            if s.dummy:
                continue
            if u.kind == "function" and s.name == u.name:
                rt = "double" if s.type == "double" else "int"
                self.emit(f"{rt} _result = 0;", 1)
                continue
            ct = {"double": "double", "int": "int", "bool": "int"}.get(s.type)
            if s.type == "char":
                self.emit(f"char {s.name}[{s.charlen + 1}] = {{0}};", 1)
                continue
            if s.param:
                if s.dims:
                    if not isinstance(s.init, Cons):
                        raise TranslateError(f"{u.name}: parameter array {s.name} needs a constructor")
                    items = ", ".join(self.expr(i) for i in s.init.items)
                    self.emit(f"const {ct} {s.name}[{len(s.init.items)}] = {{{items}}};", 1)
                else:
                    val = self.expr(s.init)
                    if s.name in self.param_override:
                        val = self.param_override[s.name].format(orig=val)
                    self.emit(f"const {ct} {s.name} = {val};", 1)
                continue
            if s.dims:
                if s.saved:
                    raise TranslateError(f"{u.name}: saved array {s.name} is not supported")
                n = self.const_size(s)
                if n is not None and n <= 65536:  # fixed size: a C array (private per thread if asked)
                    self.emit(f"{ct} {s.name}[{n}] = {{0}};", 1)
                    self.fixed.add(s.name)
                    continue
                size = " * ".join(f"(long)({ext})" for _, ext in self.dim_bounds(s))
                self.emit(f"{ct}* {s.name} = ({ct}*)calloc((size_t)({size}), sizeof({ct}));", 1)
                frees.append(s.name)
                continue
            if s.saved:
                self.emit(f"static {ct} {s.name} = {self.expr(s.init)};", 1)
            else:
                self.emit(f"{ct} {s.name} = 0;", 1)
        self.block(u.body, 0, len(u.body), 1)
        self.emit("goto _f90_exit;", 1)
        self.out.append("_f90_exit:;")
        for f in frees:
            self.emit(f"free({f});", 1)
        if u.kind == "function":
            self.emit("return _result;", 1)
        elif u.kind == "program":
            self.emit(f"return {self.prefix}stopped;", 1)
        self.out.append("}")
        self.out.append("")

    def block(self, body, a, b, depth):
        k = a
        while k < b:
            k = self.statement(body, k, b, depth)

    def _match_end(self, body, k, b, opener, closers, mids=()):
        """Index of the statement closing the construct opened at k, and the
        indices of its middle statements (else / case)."""
        depth, mid = 0, []
        for j in range(k + 1, b):
            t = body[j].text
            if opener(t):
                depth += 1
            elif closers(t):
                if depth == 0:
                    return j, mid
                depth -= 1
            elif depth == 0 and any(m(t) for m in mids):
                mid.append(j)
        raise TranslateError(f"{self.u.name}: unterminated construct at {body[k].file}:{body[k].line}")

    @staticmethod
    def _is_if_then(t):
        return bool(re.match(r"if\s*\(.*\)\s*then$", t))

    @staticmethod
    def _is_do(t):
        return bool(re.match(r"do(\s+[a-z_]\w*\s*=|\s*$|\s+while\b)", t))

    def _cond(self, t, kw):
        m = re.match(kw + r"\s*\((.*)\)\s*then$", t)
        return self.expr(parse_expr(m.group(1)))

    def statement(self, body, k, b, depth) -> int:
        st = body[k]
        t = st.text
        self.st = st
        try:
            if t.startswith("!$omp"):
                self.omp_directive(t, depth)
                return k + 1
            if self._is_if_then(t):
                end, mids = self._match_end(body, k, b, self._is_if_then,
                                            lambda x: bool(re.match(r"end\s*if$", x)),
                                            (lambda x: bool(re.match(r"else\s*if\s*\(.*\)\s*then$", x)),
                                             lambda x: x == "else"))
                self.emit(f"if ({self._cond(t, 'if')}) {{", depth)
                prev = k + 1
                for m in mids:
                    self.block(body, prev, m, depth + 1)
                    mt = body[m].text
                    if mt == "else":
                        self.emit("} else {", depth)
                    else:
                        cond = self._cond(mt, r"else\s*if")
                        self.emit(f"}} else if ({cond}) {{", depth)
                    prev = m + 1
                self.block(body, prev, end, depth + 1)
                self.emit("}", depth)
                return end + 1
            if self._is_do(t):
                end, _ = self._match_end(body, k, b, self._is_do, lambda x: bool(re.match(r"end\s*do$", x)))
                m = re.match(r"do\s+([a-z_]\w*)\s*=\s*(.*)$", t)
                if not m:
                    raise TranslateError(f"unsupported loop form: {t}")
                pending, self.omp_pending = self.omp_pending, None
                ncol = 1
                copies = []
                if pending:
                    mm = re.search(r"collapse\s*\(\s*(\d+)\s*\)", pending[1])
                    ncol = int(mm.group(1)) if mm else 1
                # the loop nest the directive covers (collapse: perfectly nested loops)
                nest, kk, ee = [], k, end
                for lev in range(ncol):
                    tt = body[kk].text
                    mm = re.match(r"do\s+([a-z_]\w*)\s*=\s*(.*)$", tt)
                    if not mm:
                        raise TranslateError(f"unsupported loop form: {tt}")
                    nest.append((self.lookup(mm.group(1)), split_top(mm.group(2), ",")))
                    if lev + 1 < ncol:
                        e2, _ = self._match_end(body, kk + 1, ee, self._is_do,
                                                lambda x: bool(re.match(r"end\s*do$", x)))
                        if not self._is_do(body[kk + 1].text) or e2 != ee - 1:
                            raise TranslateError("collapse needs perfectly nested loops")
                        kk, ee = kk + 1, e2
                heads = []
                bounds = []
                for sym, parts in nest:
                    lo, hi = self.expr(parse_expr(parts[0])), self.expr(parse_expr(parts[1]))
                    stp = int(parts[2]) if len(parts) > 2 else 1
                    a_, b_ = self.fresh("_lo"), self.fresh("_hi")
                    vv = self.var(sym)
                    cmp = "<=" if stp > 0 else ">="
                    bounds.append(f"{a_} = {lo}, {b_} = {hi}")
                    heads.append(f"for ({vv} = {a_}; {vv} {cmp} {b_}; {vv} += {stp})")
                if pending:  # local copies of reduced dummies are declared before the loop's block
                    clauses, copies = self.omp_clauses(pending[1], depth)
                    for dv, loc in copies:
                        self.shadow[dv] = loc
                self.emit(f"{{ const int {', '.join(bounds)};", depth)
                if pending:
                    self.emit(f"#pragma omp {pending[0]} {clauses}".rstrip(), depth)
                for h in heads[:-1]:
                    self.emit(h, depth)
                self.emit(heads[-1] + " {", depth)
                self.block(body, kk + 1, ee, depth + 1)
                self.emit("} }", depth)
                for dv, loc in copies:
                    del self.shadow[dv]
                    self.emit(f"(*{dv}) = {loc};", depth)
                return end + 1
            if re.match(r"select\s+case\s*\(", t):
                end, mids = self._match_end(body, k, b, lambda x: bool(re.match(r"select\s+case\s*\(", x)),
                                            lambda x: bool(re.match(r"end\s*select$", x)),
                                            (lambda x: bool(re.match(r"case\s*(\(|default)", x)),))
                sel = parse_expr(re.match(r"select\s+case\s*\((.*)\)$", t).group(1))
                sv = self.fresh("_sel")
                ct = "double" if self.type_of(sel) == "double" else "int"
                self.emit(f"{{ const {ct} {sv} = {self.expr(sel)};", depth)
                first = True
                for n_, m in enumerate(mids):
                    nxt = mids[n_ + 1] if n_ + 1 < len(mids) else end
                    ct_ = body[m].text
                    if re.match(r"case\s+default$", ct_) or ct_ == "case default":
                        cond = "1"
                    else:
                        items = split_top(re.match(r"case\s*\((.*)\)$", ct_).group(1), ",")
                        cs = []
                        for it in items:
                            if ":" in it:
                                lo_, hi_ = it.split(":", 1)
                                c = []
                                if lo_.strip():
                                    c.append(f"{sv} >= {self.expr(parse_expr(lo_))}")
                                if hi_.strip():
                                    c.append(f"{sv} <= {self.expr(parse_expr(hi_))}")
                                cs.append("(" + " && ".join(c) + ")")
                            else:
                                cs.append(f"{sv} == {self.expr(parse_expr(it))}")
                        cond = " || ".join(cs)
                    self.emit(f"{'if' if first else '} else if'} ({cond}) {{", depth)
                    first = False
                    self.block(body, m + 1, nxt, depth + 1)
                if not first:
                    self.emit("}", depth)
                self.emit("}", depth)
                return end + 1
            self.simple(t, depth)
            return k + 1
        except TranslateError as e:
            raise TranslateError(f"{st.file}:{st.line}: {e}") from None

    def simple(self, t, depth):
        if re.match(r"(write|print|format|open|close|flush)\b\s*[\(\s*]", t) or t.startswith("format"):
            self.emit(f"/* dropped: {t[:60]} */", depth)
            return
        if t == "continue":
            self.emit(";", depth)
            return
        if t == "return":
            self.emit("goto _f90_exit;", depth)
            return
        if t == "exit":
            self.emit("break;", depth)
            return
        if t == "cycle":
            self.emit("continue;", depth)
            return
        if t == "stop" or t.startswith("stop "):
            self.emit(f"{{ {self.prefix}stopped = {self.st.line}; goto _f90_exit; }}", depth)
            return
        m = re.match(r"if\s*\(", t)
        if m:
            # one-line if: find the matching parenthesis
            d, j = 0, t.index("(")
            for j in range(t.index("("), len(t)):
                if t[j] == "(":
                    d += 1
                elif t[j] == ")":
                    d -= 1
                    if d == 0:
                        break
            cond, rest = t[t.index("(") + 1:j], t[j + 1:].strip()
            self.emit(f"if ({self.expr(parse_expr(cond))}) {{", depth)
            self.simple(rest, depth + 1)
            self.emit("}", depth)
            return
        m = re.match(r"call\s+([a-z_]\w*)\s*(?:\((.*)\))?$", t)
        if m:
            self.call(m.group(1), m.group(2) or "", depth)
            return
        k = find_assign(t)
        if k < 0:
            raise TranslateError(f"unsupported statement: {t}")
        self.assign(t[:k].strip(), t[k + 1:].strip(), depth)

    def call(self, name, argtext, depth):
        args = [parse_expr(a) if not a.startswith("'") else Str(a) for a in split_top(argtext, ",")] if argtext.strip() else []
        if name in self.hooks:
            fn, keep, extra = self.hooks[name]
            pa = [self.ref_arg(args[i]) for i in keep] + [self.ref_arg(parse_expr(x)) for x in extra]
            self.emit(f"{fn}({', '.join(pa)});", depth)
            return
        if name not in self.units or self.units[name].kind != "subroutine":
            raise TranslateError(f"call of unknown subroutine {name}")
        self.emit(f"{self.fname(name)}({', '.join(self.ref_arg(a) for a in args)});", depth)
        self.emit(f"if ({self.prefix}stopped) goto _f90_exit;", depth)

    def assign(self, lhs_t, rhs_t, depth):
        lhs = parse_expr(lhs_t)
        rhs = parse_expr(rhs_t)
        if isinstance(rhs, Ref) and rhs.name in ("minloc", "maxloc") and self.lookup(rhs.name) is None:
            ls = self.lookup(lhs.name)
            a = rhs.args[0]
            s = self.lookup(a.name)
            if isinstance(a, Name):
                base, exts = self.var(s), [e for _, e in self.dim_bounds(s)]
            else:
                base = self.ref_arg(a)
                exts = [e for (d, lo, hi) in self.section_dims(s, a.args)
                        for e in [f"(({hi}) - ({lo}) + 1)"]]
            while len(exts) < 3:
                exts.append("1")
            rank = len(ls.dims and [1] * int(self.expr(ls.dims[0][1])) or [])
            self.emit(f"f90_loc({base}, {exts[0]}, {exts[1]}, {exts[2]}, {self.var(ls)}, {rank}, "
                      f"{1 if rhs.name == 'maxloc' else 0});", depth)
            return
        r = self.rank_of(lhs)
        if r == 0:
            if isinstance(lhs, Name):
                s = self.lookup(lhs.name)
                if s is None:
                    raise TranslateError(f"undeclared {lhs.name}")
                target = self.var(s)
            else:
                target = self.expr(lhs)
            self.emit(f"{target} = {self.expr(rhs)};", depth)
            return
        s = self.lookup(lhs.name)
        secs = self.section_dims(s, lhs.args if isinstance(lhs, Ref) else [])
        loops = [self.fresh("_s") for _ in range(r)]
        exts = [f"(({hi}) - ({lo}) + 1)" for (_, lo, hi) in secs]
        names_rhs = self._names(rhs)
        ct = "double" if s.type == "double" else "int"
        if s.name in names_rhs:
            tmp = self.fresh("_tmp")
            n = " * ".join(f"(long){e}" for e in exts)
            self.emit(f"{{ {ct}* {tmp} = ({ct}*)malloc((size_t)({n}) * sizeof({ct}));", depth)
            self._loops(loops, exts, depth + 1, lambda dd: self.emit(
                f"{tmp}[{self._flat(loops, exts)}] = {self.expr(rhs, loops)};", dd))
            lref = self.expr(lhs, loops) if isinstance(lhs, Ref) else self.section_ref(s, [], loops)
            self._loops(loops, exts, depth + 1, lambda dd: self.emit(
                f"{lref} = {tmp}[{self._flat(loops, exts)}];", dd))
            self.emit(f"free({tmp}); }}", depth)
            return
        lref = self.expr(lhs, loops) if isinstance(lhs, Ref) else self.section_ref(s, [], loops)
        rr = self.rank_of(rhs)
        if rr not in (0, r):
            raise TranslateError(f"non-conformable assignment {lhs_t} = {rhs_t}")
        self._loops(loops, exts, depth, lambda dd: self.emit(f"{lref} = {self.expr(rhs, loops)};", dd))

    def _flat(self, loops, exts):
        term = loops[-1]
        for d in range(len(loops) - 2, -1, -1):
            term = f"({loops[d]} + (long){exts[d]} * ({term}))"
        return term

    def _loops(self, loops, exts, depth, body):
        # innermost loop over the first (fastest) section dimension
        for d in range(len(loops) - 1, -1, -1):
            self.emit(f"for (long {loops[d]} = 0; {loops[d]} < (long){exts[d]}; ++{loops[d]}) {{", depth + (len(loops) - 1 - d))
        body(depth + len(loops))
        for d in range(len(loops)):
            self.emit("}", depth + len(loops) - 1 - d)

    def _names(self, e) -> set:
        if isinstance(e, Name):
            return {e.name}
        if isinstance(e, Ref):
            out = {e.name}
            for a in e.args:
                out |= self._names(a)
            return out
        if isinstance(e, Range):
            return (self._names(e.lo) if e.lo else set()) | (self._names(e.hi) if e.hi else set())
        if isinstance(e, Bin):
            return self._names(e.a) | self._names(e.b)
        if isinstance(e, Un):
            return self._names(e.a)
        return set()


def parse_files(paths: list[str], include_dir: str | None = None) -> list[Unit]:
    units = []
    for p in paths:
        units.extend(parse_units(read_statements(p, include_dir)))
    return units


def emit_c(units: list[Unit], prefix: str = "f90_", overrides: dict | None = None,
           hooks: dict | None = None, header: str = "") -> str:
    """C source for the units.  overrides: {"program": {param: C expression}}
    replaces integer/real parameters of the main program (the reference's own
    way of configuring a run is to edit them); hooks: {subroutine: (C function,
    [indices of the actual arguments to pass], [extra argument expressions])}
    for calls of routines outside the translated set (the snapshot writer)."""
    em = Emitter(units, prefix, overrides or {}, hooks or {})
    head = [header, RUNTIME.replace("PFX_", prefix),
            f"int {prefix}ipar_set[16], {prefix}ipar[16], {prefix}dpar_set[16];",
            f"double {prefix}dpar[16];"]
    for fn, _, _ in (hooks or {}).values():
        head.append(f"void {fn}();")
    protos = []
    for u in units:
        ps = []
        for a in u.args:
            s = u.syms[a]
            ct = {"double": "double", "int": "int", "bool": "int", "char": "char"}[s.type]
            ps.append(f"{ct}*")
        if u.kind == "program":
            protos.append(f"int {prefix}{u.name}(void);")
        elif u.kind == "function":
            rt = "double" if u.syms[u.name].type == "double" else "int"
            protos.append(f"{rt} {prefix}{u.name}({', '.join(ps) or 'void'});")
        else:
            protos.append(f"void {prefix}{u.name}({', '.join(ps) or 'void'});")
    for u in units:
        em.unit(u)
    return "\n".join(head + protos + [""] + em.out) + "\n"
