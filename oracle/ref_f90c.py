"""Fortran-subset to C translator for the reference programs, and its runner.

TEST INFRASTRUCTURE ONLY. This module pins the oracle to the reference. No
part of the product imports it, and nothing it writes is committed: its C
files and binaries go to oracle/_ref/, which git ignores.

Neither this container nor the GPU host has a Fortran compiler, so the
reference cannot be compiled the usual way. This module reads a reference
program's Fortran source where it lies (read-only) and translates its main
program unit, statement by statement, into GNU C. gcc then compiles that C
with -ffp-contract=off. The binary executes the reference's own statements:
  - its parameter block, with chosen parameters overridden the way one would
    edit a `parameter` line;
  - its loop ranges and operation order;
  - its intrinsic calls;
  - its MPI exchange pattern, over oracle/ref_mpi.c's single-host stand-in.
Its outputs are the golden vectors that cpml_oracle.cpp and oracle_np.py are
checked against (tests/golden/make_ref_vectors.py, tests/test_ref_pin.py).

The supported subset is what the four programs on the path use:
  - declarations: integer, double precision, real, logical (scalars, arrays
    with declared bounds, `parameter`), and character variables;
  - `include 'mpif.h'` and the MPI calls that oracle/ref_mpi.c provides;
  - statements: assignment (scalar, element, section, whole array), DO loops
    with a fixed trip count, block IF/ELSE IF/ELSE, logical IF, CALL, STOP;
  - expressions: Fortran operator precedence with left-to-right evaluation,
    and these intrinsics: dble, sngl, real, int, nint, abs, sqrt, exp, log,
    log10, sin, cos, tan, atan, mod, max, min, sum, maxval, minval;
  - subroutine units, translated on request beside a main program. Their
    dummy arguments arrive by reference, and their arrays may have bounds
    that are dummy arguments (adjustable arrays). The output subroutines
    use WRITE (to a unit or a character variable, with literal strings and
    Iw / Iw.m edits, or list-directed integers, reals and strings), OPEN
    and CLOSE. List-directed spacing is the compiler's choice; reals are
    written with the digits that read back to the same value.
Anything outside the subset raises TranslateError with its line number, so
nothing is dropped silently. In a main program, statements that only
produce text (print, write, open, close, format) are skipped unless `io` is
set, and so are calls of the output subroutines named in SKIPPED_CALLS.

Fortran semantics kept:
  - arrays are column-major with their declared lower bounds, in static
    storage that starts at zero. gfortran keeps main-program arrays static,
    and the 3D program relies on that for sigmaxx (3D:724-729);
  - literals without a D exponent are default REAL (single precision);
  - integer division truncates;
  - x**n with an integer n is repeated multiplication (__builtin_powi, the
    form gfortran lowers it to); x**y with a real y calls pow;
  - operators of equal precedence evaluate left to right, and parentheses
    are kept;
  - a DO loop's trip count is fixed when the loop starts;
  - array expressions evaluate element by element in column-major order:
    SUM accumulates in that order, and MAXVAL/MINVAL compare in that order.
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
MPI_RUNTIME = os.path.join(HERE, "ref_mpi.c")

SKIPPED_CALLS = {"write_seismograms", "create_color_image", "date_and_time"}
MPI_CALLS = {  # name -> number of arguments
    "mpi_init": 1, "mpi_finalize": 1, "mpi_comm_size": 3, "mpi_comm_rank": 3,
    "mpi_barrier": 2, "mpi_sendrecv": 13, "mpi_reduce": 8, "mpi_allreduce": 7,
}
MPIF_PARAMETERS = {  # the constants of mpif.h the programs use, as ref_mpi.c numbers them
    "mpi_comm_world": 0, "mpi_double_precision": 1, "mpi_integer": 2,
    "mpi_sum": 1, "mpi_max": 2, "mpi_min": 3, "mpi_proc_null": -2,
    "mpi_status_size": 4, "mpi_any_source": -1,
}


class TranslateError(Exception):
    pass


# ---------------------------------------------------------------------------
# source reading: comments, continuation lines, case
# ---------------------------------------------------------------------------
STF_LINES = {  # the programs' three source-time-function lines (e.g. 3D:1062-1068)
    "gaussian": re.compile(r"source_term\s*=\s*factor\s*\*\s*exp\(", re.I),
    "dgaussian": re.compile(r"source_term\s*=\s*-\s*factor\s*\*\s*2\.d0\s*\*", re.I),
    "ricker": re.compile(r"source_term\s*=\s*factor\s*\*\s*\(1\.d0\s*-", re.I),
}


def select_source_time_function(lines: list[str], kind: str) -> list[str]:
    """The programs carry the Gaussian, its first derivative (active) and the
    Ricker wavelet as three alternative `source_term =` lines, two of them
    commented out. Return the lines with only `kind`'s line active, as a user
    switching the wavelet edits them; every other line is unchanged."""
    if kind not in STF_LINES:
        raise TranslateError(f"unknown source time function {kind!r}")
    out, seen = [], set()
    for line in lines:
        body = line.lstrip()
        code = body[1:].lstrip() if body.startswith("!") else body
        hit = [k for k, rx in STF_LINES.items() if rx.match(code)]
        if hit:
            seen.add(hit[0])
            indent = line[:len(line) - len(body)]
            out.append(indent + (code if hit[0] == kind else "! " + code))
        else:
            out.append(line)
    if seen != set(STF_LINES):
        raise TranslateError("the three source-time-function lines were not all found")
    return out


def read_statements(path: str, stf: str | None = None) -> list[tuple[int, str]]:
    """Free-form Fortran source -> [(first line number, statement text)].
    Comments (outside string literals) are removed, continuation lines joined,
    and everything outside string literals lower-cased. stf, when given,
    selects the active source-time-function line first."""
    stmts, buf, start, quote = [], "", None, None
    with open(path, encoding="latin-1") as f:
        lines = f.read().split("\n")
    if stf is not None:
        lines = select_source_time_function(lines, stf)
    for ln, raw in enumerate(lines, 1):
        line = raw.rstrip("\n")
        if buf:
            s = line.lstrip()
            line = s[1:] if s.startswith("&") else s
        out = []
        for ch in line:
            if quote:
                out.append(ch)
                if ch == quote:
                    quote = None
            elif ch in "'\"":
                quote = ch
                out.append(ch)
            elif ch == "!":
                break
            else:
                out.append(ch)
        text = "".join(out).rstrip()
        if not text:
            continue
        if start is None:
            start = ln
        if text.endswith("&"):
            buf += text[:-1]
            continue
        buf += text
        stmts.append((start, _lower_outside_strings(buf.strip())))
        buf, start, quote = "", None, None
    return stmts


def _lower_outside_strings(s: str) -> str:
    out, quote = [], None
    for ch in s:
        if quote:
            out.append(ch)
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
            out.append(ch)
        else:
            out.append(ch.lower())
    return "".join(out)


def main_program(stmts):
    """Statements of the main program unit (between PROGRAM and END PROGRAM)."""
    body, inside = [], False
    for ln, s in stmts:
        if not inside:
            if re.match(r"program\s+\w+$", s):
                inside = True
            continue
        if re.match(r"end\s*program\b", s) or s == "end":
            return body
        body.append((ln, s))
    raise TranslateError("no complete main program unit found")


# ---------------------------------------------------------------------------
# expressions
# ---------------------------------------------------------------------------
_DOTOPS = ("and", "or", "not", "eqv", "neqv", "eq", "ne", "lt", "le", "gt", "ge", "true", "false")
_DOTOP_RE = re.compile(r"\.(%s)\." % "|".join(_DOTOPS))
_OPS = ("**", "//", "==", "/=", "<=", ">=", "<", ">", "+", "-", "*", "/", "(", ")", ",", ":", "=")


def tokenize(s: str, ln: int):
    toks, i, n = [], 0, len(s)
    while i < n:
        c = s[i]
        if c.isspace():
            i += 1
            continue
        if c in "'\"":
            j = i + 1
            while True:
                if j >= n:
                    raise TranslateError(f"line {ln}: unterminated string")
                if s[j] == c:
                    if j + 1 < n and s[j + 1] == c:
                        j += 2
                        continue
                    break
                j += 1
            toks.append(("str", s[i + 1:j].replace(c + c, c)))
            i = j + 1
            continue
        m = _DOTOP_RE.match(s, i)
        if m:
            toks.append(("dot", m.group(1)))
            i = m.end()
            continue
        if c.isdigit() or (c == "." and i + 1 < n and s[i + 1].isdigit()):
            j = i
            while j < n and s[j].isdigit():
                j += 1
            frac = False
            if j < n and s[j] == "." and not _DOTOP_RE.match(s, j):
                frac = True
                j += 1
                while j < n and s[j].isdigit():
                    j += 1
            kind = "r" if frac else "i"
            m2 = re.compile(r"[dDeE][+-]?\d+").match(s, j)
            if m2:
                kind = "d" if m2.group(0)[0] in "dD" else "r"
                j = m2.end()
            if j < n and s[j] == "_":
                raise TranslateError(f"line {ln}: kind suffixes are outside the subset")
            toks.append(("num", s[i:j], kind))
            i = j
            continue
        if c.isalpha() or c == "_":
            j = i
            while j < n and (s[j].isalnum() or s[j] == "_"):
                j += 1
            toks.append(("name", s[i:j]))
            i = j
            continue
        for op in _OPS:
            if s.startswith(op, i):
                toks.append(("op", op))
                i += len(op)
                break
        else:
            raise TranslateError(f"line {ln}: unexpected character {c!r}")
    return toks


class Parser:
    """Recursive descent over Fortran's precedence levels, lowest first:
    .eqv./.neqv., .or., .and., .not., relational, // , additive (with a
    leading sign applying to the first term), multiplicative, ** (right
    associative), primaries."""

    REL = {"==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">=",
           "eq": "==", "ne": "!=", "lt": "<", "le": "<=", "gt": ">", "ge": ">="}

    def __init__(self, toks, ln):
        self.t, self.k, self.ln = toks, 0, ln

    def peek(self, off=0):
        return self.t[self.k + off] if self.k + off < len(self.t) else ("end",)

    def take(self):
        tok = self.peek()
        self.k += 1
        return tok

    def expect(self, op):
        tok = self.take()
        if tok != ("op", op):
            raise TranslateError(f"line {self.ln}: expected {op!r}, got {tok}")

    def at_end(self):
        return self.k >= len(self.t)

    def expr(self):
        e = self.or_()
        while self.peek() in (("dot", "eqv"), ("dot", "neqv")):
            op = "==" if self.take()[1] == "eqv" else "!="
            e = ("bin", op, e, self.or_())
        return e

    def or_(self):
        e = self.and_()
        while self.peek() == ("dot", "or"):
            self.take()
            e = ("bin", "||", e, self.and_())
        return e

    def and_(self):
        e = self.not_()
        while self.peek() == ("dot", "and"):
            self.take()
            e = ("bin", "&&", e, self.not_())
        return e

    def not_(self):
        if self.peek() == ("dot", "not"):
            self.take()
            return ("un", "!", self.not_())
        return self.rel()

    def rel(self):
        e = self.add()
        tok = self.peek()
        if (tok[0] == "op" and tok[1] in self.REL) or (tok[0] == "dot" and tok[1] in self.REL):
            self.take()
            e = ("bin", self.REL[tok[1]], e, self.add())
        return e

    def add(self):
        tok = self.peek()
        if tok in (("op", "+"), ("op", "-")):
            self.take()
            e = self.mul()
            e = ("un", "-", e) if tok[1] == "-" else e
        else:
            e = self.mul()
        while self.peek() in (("op", "+"), ("op", "-")):
            op = self.take()[1]
            e = ("bin", op, e, self.mul())
        return e

    def mul(self):
        e = self.pow_()
        while self.peek() in (("op", "*"), ("op", "/")):
            op = self.take()[1]
            e = ("bin", op, e, self.pow_())
        return e

    def pow_(self):
        base = self.primary()
        if self.peek() == ("op", "**"):
            self.take()
            if self.peek() in (("op", "+"), ("op", "-")):
                sign = self.take()[1]
                ex = self.pow_()
                ex = ("un", "-", ex) if sign == "-" else ex
            else:
                ex = self.pow_()
            return ("bin", "**", base, ex)
        return base

    def primary(self):
        tok = self.take()
        if tok[0] == "num":
            return ("num", tok[1], tok[2])
        if tok[0] == "str":
            return ("str", tok[1])
        if tok[0] == "dot" and tok[1] in ("true", "false"):
            return ("log", tok[1] == "true")
        if tok == ("op", "("):
            e = self.expr()
            self.expect(")")
            return e
        if tok[0] == "name":
            if self.peek() == ("op", "("):
                self.take()
                args = []
                if self.peek() != ("op", ")"):
                    while True:
                        args.append(self.arg())
                        if self.peek() == ("op", ","):
                            self.take()
                            continue
                        break
                self.expect(")")
                return ("ref", tok[1], args)
            return ("name", tok[1])
        raise TranslateError(f"line {self.ln}: unexpected token {tok}")

    def arg(self):
        """An actual argument or subscript: expression, section triplet, or
        keyword argument (rejected)."""
        if self.peek() == ("op", ":"):
            self.take()
            hi = None if self.peek() in (("op", ","), ("op", ")")) else self.expr()
            return ("slice", None, hi)
        if self.peek()[0] == "name" and self.peek(1) == ("op", "="):
            raise TranslateError(f"line {self.ln}: keyword arguments are outside the subset")
        e = self.expr()
        if self.peek() == ("op", ":"):
            self.take()
            hi = None if self.peek() in (("op", ","), ("op", ")")) else self.expr()
            return ("slice", e, hi)
        return e


def parse_expr(text: str, ln: int):
    p = Parser(tokenize(text, ln), ln)
    e = p.expr()
    if not p.at_end():
        raise TranslateError(f"line {ln}: trailing tokens in {text!r}")
    return e


# ---------------------------------------------------------------------------
# symbols
# ---------------------------------------------------------------------------
@dataclass
class Sym:
    name: str
    ftype: str                      # 'i' integer, 'r' real, 'd' double, 'l' logical, 'c' character
    dims: list | None = None        # [(lo, hi)]: Python ints, or C expressions (dummy arrays)
    param: bool = False
    init: tuple | None = None       # parameter initialiser (AST)
    cname: str = ""                 # the C name it is accessed by
    clen: int = 0                   # character length
    dummy: bool = False             # a dummy argument of a subroutine

    @property
    def size(self):
        n = 1
        for lo, hi in self.dims:
            n *= max(hi - lo + 1, 0)
        return n


CTYPE = {"i": "int", "r": "float", "d": "double", "l": "int"}
NPTYPE = {"i": "<i4", "r": "<f4", "d": "<f8", "l": "<i4"}
_RANK = {"i": 0, "r": 1, "d": 2}


def _promote(a, b):
    return a if _RANK[a] >= _RANK[b] else b


# ---------------------------------------------------------------------------
# translator
# ---------------------------------------------------------------------------
class Translator:
    def __init__(self, overrides: dict | None = None, bounds: bool = True,
                 timed_loop: str | None = None, prefix: str = "v_", dummies=(),
                 subs: dict | None = None, io: bool = False):
        self.prefix = prefix           # C prefix of this unit's variables and parameters
        self.dummies = list(dummies)   # dummy arguments, when translating a subroutine
        self.subs = dict(subs or {})   # translated subroutines callable here: name -> arity
        self.io = io                   # translate WRITE/OPEN/CLOSE instead of skipping them
        self.timed_loop = timed_loop   # DO variable of the loop whose wall time is dumped
        self.timer_used = False
        self.syms: dict[str, Sym] = {}
        self.order: list[str] = []
        self.overrides = {k.lower(): v for k, v in (overrides or {}).items()}
        self.used_overrides: set[str] = set()
        self.bounds = bounds
        self.out: list[str] = []
        self.ind = 1
        self.tmp = 0
        self.ln = 0
        self.blocks: list[str] = []

    # ---- constant evaluation (integer parameters size the arrays) --------
    def const_int(self, e):
        v = self.const(e)
        if not isinstance(v, int) or isinstance(v, bool):
            raise TranslateError(f"line {self.ln}: not an integer constant: {e}")
        return v

    def const(self, e):
        k = e[0]
        if k == "num":
            if e[2] == "i":
                return int(e[1])
            return float(e[1].lower().replace("d", "e"))
        if k == "log":
            return e[1]
        if k == "name":
            s = self.syms.get(e[1])
            if s is None or not s.param:
                raise TranslateError(f"line {self.ln}: {e[1]} is not a parameter")
            return self.const(s.init)
        if k == "un":
            v = self.const(e[2])
            return -v if e[1] == "-" else (not v)
        if k == "bin":
            a, b = self.const(e[2]), self.const(e[3])
            op = e[1]
            if op in "+-*":
                return {"+": a + b, "-": a - b, "*": a * b}[op]
            if op == "/":
                if isinstance(a, int) and isinstance(b, int):
                    q = abs(a) // abs(b)
                    return q if (a >= 0) == (b >= 0) else -q
                return a / b
            if op == "**":
                return a ** b
        if k == "ref" and e[1] in ("max", "min", "mod"):
            vals = [self.const(x) for x in e[2]]
            if e[1] == "mod":
                a, b = vals
                return a - int(a / b) * b
            return max(vals) if e[1] == "max" else min(vals)
        raise TranslateError(f"line {self.ln}: cannot fold {e} to a constant")

    # ---- declarations ------------------------------------------------------
    TYPE_RE = re.compile(r"(integer|double\s+precision|logical|real|character(?:\s*\([^)]*\)|\*\d+)?)"
                         r"(?=[\s,:(]|$)(.*)$")

    def declaration(self, s):
        m = self.TYPE_RE.match(s)
        tname, rest = m.group(1), m.group(2).strip()
        ftype = {"integer": "i", "logical": "l", "real": "r"}.get(tname)
        if ftype is None:
            ftype = "d" if tname.startswith("double") else "c"
        attrs, ents = [], rest
        if "::" in rest:
            a, ents = rest.split("::", 1)
            attrs = [x.strip() for x in _split_top(a.strip().lstrip(","), ",") if x.strip()]
        elif rest.startswith(","):
            raise TranslateError(f"line {self.ln}: attributes need '::'")
        param = False
        dims = None
        for a in attrs:
            if a == "parameter":
                param = True
            elif a.startswith("dimension"):
                dims = a[len("dimension"):].strip()
                if not (dims.startswith("(") and dims.endswith(")")):
                    raise TranslateError(f"line {self.ln}: bad dimension attribute")
                dims = dims[1:-1]
            else:
                raise TranslateError(f"line {self.ln}: attribute {a!r} is outside the subset")
        for ent in _split_top(ents.strip(), ","):
            ent = ent.strip()
            init_text = None
            if "=" in ent:
                ent, init_text = ent.split("=", 1)
                ent = ent.strip()
                init_text = init_text.strip()
            m2 = re.match(r"(\w+)\s*(?:\((.*)\))?\s*(?:\*\s*\d+)?$", ent)
            if not m2:
                raise TranslateError(f"line {self.ln}: cannot read declaration {ent!r}")
            name, edims = m2.group(1), m2.group(2) or dims
            if name in self.syms:
                raise TranslateError(f"line {self.ln}: {name} declared twice")
            sym = Sym(name, ftype, param=param, dummy=name in self.dummies)
            if ftype == "c":
                if sym.dummy:
                    raise TranslateError(f"line {self.ln}: character dummy arguments are outside the subset")
                mlen = re.search(r"\d+", tname)
                sym.clen = int(mlen.group(0)) if mlen else 1
            if edims is not None and ftype != "c":
                sym.dims = []
                for d in _split_top(edims, ","):
                    lo, hi = d.split(":", 1) if ":" in d else ("1", d)
                    sym.dims.append((self.bound(lo, sym), self.bound(hi, sym)))
            if sym.dummy:
                sym.cname = f"d_{name}" if sym.dims else f"(*d_{name})"
            else:
                sym.cname = self.prefix + name
            if param:
                if init_text is None:
                    raise TranslateError(f"line {self.ln}: parameter {name} without a value")
                if name in self.overrides:   # case-folded like the source text
                    init_text = _lower_outside_strings(str(self.overrides[name]))
                    self.used_overrides.add(name)
                sym.init = parse_expr(init_text, self.ln)
                if sym.dims:
                    raise TranslateError(f"line {self.ln}: array parameters are outside the subset")
            elif init_text is not None:
                raise TranslateError(f"line {self.ln}: initialised variables are outside the subset")
            self.syms[name] = sym
            self.order.append(name)

    def bound(self, text, sym):
        """An array bound: a Python int when it is a constant expression, else
        (for a dummy array only) the C expression of the dummy arguments it
        names, evaluated at each reference as in Fortran's adjustable arrays."""
        e = parse_expr(text, self.ln)
        try:
            return self.const_int(e)
        except TranslateError:
            if not sym.dummy:
                raise
            c, t = self.scalar(e)
            if t != "i":
                raise TranslateError(f"line {self.ln}: non-integer bound of {sym.name}")
            return c

    # ---- expression code ----------------------------------------------------
    def sym(self, name):
        s = self.syms.get(name)
        if s is None:
            raise TranslateError(f"line {self.ln}: undeclared name {name}")
        if s.ftype == "c":
            raise TranslateError(f"line {self.ln}: character variable {name} used in computation")
        return s

    def shape(self, e):
        """Section extents of an array-valued expression as [(lo_c, hi_c)],
        or None for a scalar."""
        k = e[0]
        if k == "name":
            s = self.syms.get(e[1])
            if s is not None and s.dims:
                return [(str(lo), str(hi)) for lo, hi in s.dims]
            return None
        if k == "ref":
            s = self.syms.get(e[1])
            if s is not None and s.dims is not None:
                ext = []
                for d, a in enumerate(e[2]):
                    if a[0] == "slice":
                        lo = self.scalar(a[1])[0] if a[1] is not None else str(s.dims[d][0])
                        hi = self.scalar(a[2])[0] if a[2] is not None else str(s.dims[d][1])
                        ext.append((lo, hi))
                return ext or None
            if e[1] in ("sum", "maxval", "minval"):
                return None
            for a in e[2]:
                sh = self.shape(a)
                if sh:
                    return sh
            return None
        if k == "un":
            return self.shape(e[2])
        if k == "bin":
            return self.shape(e[2]) or self.shape(e[3])
        return None

    def scalar(self, e):
        if self.shape(e):
            raise TranslateError(f"line {self.ln}: array expression where a scalar is needed")
        return self.gen(e, None)

    def index(self, s, args, el):
        """C index into the flat column-major storage of s."""
        if len(args) != len(s.dims):
            raise TranslateError(f"line {self.ln}: {s.name} takes {len(s.dims)} subscripts")
        terms, q = [], 0
        for d, a in enumerate(args):
            lo, hi = s.dims[d]
            if a[0] == "slice":
                if el is None:
                    raise TranslateError(f"line {self.ln}: section of {s.name} in scalar context")
                start = self.scalar(a[1])[0] if a[1] is not None else str(lo)
                ic = f"(({start}) + {el[q]})"
                q += 1
            else:
                c, t = self.scalar(a)
                if t != "i":
                    raise TranslateError(f"line {self.ln}: non-integer subscript of {s.name}")
                ic = c
            if self.bounds:
                ic = f'ref_chk({ic}, {lo}, {hi}, "{s.name}", {self.ln})'
            ext = hi - lo + 1 if isinstance(lo, int) and isinstance(hi, int) \
                else f"(long)(({hi}) - ({lo}) + 1)"
            terms.append((f"(({ic}) - ({lo}))", ext))
        code, stride = terms[0][0], terms[0][1]
        for t, ext in terms[1:]:
            code = f"{code} + ({stride}L) * {t}" if isinstance(stride, int) else f"{code} + {stride} * {t}"
            stride = stride * ext if isinstance(stride, int) and isinstance(ext, int) else f"({stride} * {ext})"
        return code

    def gen(self, e, el):
        """(C code, type) of e; el lists the loop counters of the enclosing
        elemental evaluation (None in scalar context)."""
        k = e[0]
        if k == "num":
            txt, kind = e[1], e[2]
            if kind == "i":
                return txt, "i"
            txt = txt.lower().replace("d", "e")
            if kind == "r":
                if "." not in txt and "e" not in txt:
                    txt += "."
                return txt + "f", "r"
            return txt, "d"
        if k == "log":
            return ("1" if e[1] else "0"), "l"
        if k == "str":
            raise TranslateError(f"line {self.ln}: string in computation")
        if k == "name":
            s = self.sym(e[1])
            if s.dims:
                if el is None:
                    raise TranslateError(f"line {self.ln}: whole array {s.name} in scalar context")
                args = [("slice", None, None)] * len(s.dims)
                return f"{s.cname}[{self.index(s, args, el)}]", s.ftype
            return s.cname, s.ftype
        if k == "ref":
            s = self.syms.get(e[1])
            if s is not None:
                s = self.sym(e[1])
                if not s.dims:
                    raise TranslateError(f"line {self.ln}: {s.name} is not an array")
                return f"{s.cname}[{self.index(s, e[2], el)}]", s.ftype
            return self.intrinsic(e[1], e[2], el)
        if k == "un":
            c, t = self.gen(e[2], el)
            if e[1] == "!":
                return f"(!{c})", "l"
            return f"(-{c})", t
        if k == "bin":
            op = e[1]
            a, ta = self.gen(e[2], el)
            b, tb = self.gen(e[3], el)
            if op in ("&&", "||"):
                return f"({a} {op} {b})", "l"
            if op in ("==", "!=", "<", "<=", ">", ">="):
                return f"({a} {op} {b})", "l"
            if "l" in (ta, tb):
                raise TranslateError(f"line {self.ln}: arithmetic on a logical value")
            if op == "**":
                if tb == "i":
                    if ta == "i":
                        return f"ref_ipow({a}, {b})", "i"
                    fn = "__builtin_powi" if ta == "d" else "__builtin_powif"
                    return f"{fn}({a}, {b})", ta
                t = _promote(ta, tb)
                if t == "i":
                    t = "r"
                if t == "d":
                    return f"pow((double)({a}), (double)({b}))", "d"
                return f"powf((float)({a}), (float)({b}))", "r"
            return f"({a} {op} {b})", _promote(ta, tb)
        raise TranslateError(f"line {self.ln}: cannot translate {e}")

    MATH = {"sqrt", "exp", "log", "log10", "sin", "cos", "tan", "atan"}

    def intrinsic(self, name, args, el):
        if name in ("sum", "maxval", "minval"):
            if len(args) != 1:
                raise TranslateError(f"line {self.ln}: {name} with dim/mask is outside the subset")
            return self.reduction(name, args[0])
        vals = [self.gen(a, el) for a in args]
        if name in self.MATH:
            (c, t), = vals
            if t == "i":
                raise TranslateError(f"line {self.ln}: {name} of an integer")
            return (f"{name}({c})" if t == "d" else f"{name}f({c})"), t
        if name == "abs":
            (c, t), = vals
            return {"i": f"abs({c})", "r": f"fabsf({c})", "d": f"fabs({c})"}[t], t
        if name == "dble":
            return f"((double)({vals[0][0]}))", "d"
        if name in ("sngl", "real"):
            if len(vals) != 1:
                raise TranslateError(f"line {self.ln}: kind arguments are outside the subset")
            return f"((float)({vals[0][0]}))", "r"
        if name == "int":
            return f"((int)({vals[0][0]}))", "i"
        if name == "nint":
            c, t = vals[0]
            return (f"((int)lround({c}))" if t == "d" else f"((int)lroundf({c}))"), "i"
        if name == "mod":
            (a, ta), (b, tb) = vals
            if ta == tb == "i":
                return f"({a} % {b})", "i"
            t = _promote(ta, tb)
            return (f"fmod({a}, {b})" if t == "d" else f"fmodf({a}, {b})"), t
        if name in ("max", "min"):
            types = {t for _, t in vals}
            if len(types) != 1:
                raise TranslateError(f"line {self.ln}: {name} of mixed types")
            t = types.pop()
            ct = CTYPE[t]
            cmp = ">" if name == "max" else "<"
            code = vals[0][0]
            for c, _ in vals[1:]:   # result = a; if (b > result) result = b
                code = f"({{ {ct} _a = {code}; {ct} _b = {c}; (_b {cmp} _a) ? _b : _a; }})"
            return code, t
        raise TranslateError(f"line {self.ln}: intrinsic {name} is outside the subset")

    def reduction(self, name, arg):
        sh = self.shape(arg)
        if not sh:
            raise TranslateError(f"line {self.ln}: {name} of a scalar")
        el, loops = self.loops(sh)
        c, t = self.gen(arg, el)
        ct = CTYPE[t]
        acc = f"_r{self.tmp}"
        self.tmp += 1
        if name == "sum":
            init, upd = "0", f"{acc} = {acc} + ({c});"
        else:
            big = {"i": "INT_MAX", "r": "FLT_MAX", "d": "DBL_MAX"}[t]
            init = f"-{big}" if name == "maxval" else big
            cmp = ">" if name == "maxval" else "<"
            upd = f"{{ {ct} _e = {c}; if (_e {cmp} {acc}) {acc} = _e; }}"
        return f"({{ {ct} {acc} = {init}; {loops} {upd} {acc}; }})", t

    def loops(self, sh):
        """Loop counters and nested loop headers (first section dimension
        innermost) over extents sh."""
        base = self.tmp
        self.tmp += 1
        el = [f"_q{base}_{d}" for d in range(len(sh))]
        hdr = ""
        for d in reversed(range(len(sh))):
            lo, hi = sh[d]
            hdr += f"for (long {el[d]} = 0; {el[d]} < (long)(({hi}) - ({lo}) + 1); ++{el[d]}) "
        return el, hdr

    # ---- statements -----------------------------------------------------------
    def emit(self, line):
        self.out.append("  " * self.ind + line)

    def assignment(self, lhs_text, rhs_text):
        lhs = parse_expr(lhs_text, self.ln)
        rhs = parse_expr(rhs_text, self.ln)
        if lhs[0] not in ("name", "ref"):
            raise TranslateError(f"line {self.ln}: cannot assign to {lhs_text}")
        s = self.syms.get(lhs[1])
        if s is None:
            raise TranslateError(f"line {self.ln}: undeclared name {lhs[1]}")
        if s.param:
            raise TranslateError(f"line {self.ln}: assignment to parameter {s.name}")
        if s.ftype == "c":
            raise TranslateError(f"line {self.ln}: character assignment is outside the subset")
        sh = self.shape(lhs)
        if not sh:
            c, _ = self.gen(lhs, None)
            r, _ = self.scalar(rhs)
            self.emit(f"{c} = ({CTYPE[s.ftype]})({r});")
            return
        rsh = self.shape(rhs)
        if rsh and len(rsh) != len(sh):
            raise TranslateError(f"line {self.ln}: non-conformable array assignment")
        if rsh and not _same_section_only(rhs, lhs):
            # element-by-element evaluation equals Fortran's evaluate-then-
            # assign only when the right side reads the target array through
            # the very section it writes
            raise TranslateError(f"line {self.ln}: overlapping array assignment is outside the subset")
        el, hdr = self.loops(sh)
        c, _ = self.gen(lhs, el)
        r, _ = self.gen(rhs, el)
        self.emit(f"{hdr}{c} = ({CTYPE[s.ftype]})({r});")

    def call(self, text):
        m = re.match(r"call\s+(\w+)\s*(?:\((.*)\))?\s*$", text)
        if not m:
            raise TranslateError(f"line {self.ln}: cannot read call {text!r}")
        name = m.group(1)
        if name in self.subs:                     # a translated subroutine unit
            arity, target = self.subs[name], f"ref_sub_{name}"
        elif name in SKIPPED_CALLS:
            self.emit(f"/* line {self.ln}: call {name} skipped (output only) */")
            return
        elif name in MPI_CALLS:
            arity, target = MPI_CALLS[name], f"ref_{name}"
        else:
            raise TranslateError(f"line {self.ln}: call of {name} is outside the subset")
        p = Parser(tokenize("(" + (m.group(2) or "") + ")", self.ln), self.ln)
        p.expect("(")
        args = []
        if p.peek() != ("op", ")"):
            while True:
                args.append(p.arg())
                if p.peek() == ("op", ","):
                    p.take()
                    continue
                break
        p.expect(")")
        if len(args) != arity:
            raise TranslateError(f"line {self.ln}: {name} takes {arity} arguments")
        pre, ptrs = [], []
        for a in args:
            ptr = self.address(a, pre)
            ptrs.append(ptr)
        self.emit("{")
        for line in pre:
            self.emit("  " + line)
        self.emit(f"  {target}({', '.join(ptrs)});")
        self.emit("}")

    def address(self, a, pre):
        """Pass-by-reference address of an actual argument: a variable, an
        array element, a contiguous section, or a temporary holding an
        expression's value."""
        if a[0] == "name" and not self.sym(a[1]).param:
            s = self.sym(a[1])
            return f"(void*)&{s.cname}" if not s.dims else f"(void*){s.cname}"
        if a[0] == "ref" and a[1] in self.syms:
            s = self.sym(a[1])
            sliced = [x[0] == "slice" for x in a[2]]
            if any(sliced):
                # contiguous in column-major order: full leading dimensions,
                # then at most one partial section, then scalar subscripts
                last = max(d for d, f in enumerate(sliced) if f)
                for d in range(last):
                    x = a[2][d]
                    if not (x[0] == "slice" and x[1] is None and x[2] is None):
                        raise TranslateError(f"line {self.ln}: non-contiguous section argument")
                first = []
                for d, x in enumerate(a[2]):
                    if x[0] == "slice":
                        first.append(x[1] if x[1] is not None else ("num", str(s.dims[d][0]), "i"))
                    else:
                        first.append(x)
                return f"(void*)&{s.cname}[{self.index(s, first, None)}]"
            return f"(void*)&{self.gen(a, None)[0]}"
        c, t = self.scalar(a)
        tmp = f"_a{self.tmp}"
        self.tmp += 1
        pre.append(f"{CTYPE[t]} {tmp} = {c};")
        return f"(void*)&{tmp}"

    def statement(self, s):
        if s in ("implicit none", "continue"):
            return
        if re.match(r"include\s+['\"]mpif\.h['\"]$", s):
            for k, v in MPIF_PARAMETERS.items():
                self.syms[k] = Sym(k, "i", param=True, init=("num", str(v), "i"),
                                   cname=self.prefix + k)
                self.order.append(k)
            return
        if self.TYPE_RE.match(s):
            self.declaration(s)
            return
        if re.match(r"(print\b|format\s*\()", s):
            return
        if re.match(r"(write|open|close)\s*\(", s):
            if self.io:
                self.io_statement(s)
            return
        m = re.match(r"do\s+(\w+)\s*=\s*(.+)$", s)
        if m:
            var = self.sym(m.group(1))
            if var.dims or var.ftype != "i":
                raise TranslateError(f"line {self.ln}: DO variable must be an integer scalar")
            parts = _split_top(m.group(2), ",")
            if len(parts) not in (2, 3):
                raise TranslateError(f"line {self.ln}: bad DO range")
            lo, hi = (self.scalar(parse_expr(x, self.ln))[0] for x in parts[:2])
            st = self.scalar(parse_expr(parts[2], self.ln))[0] if len(parts) == 3 else "1"
            n = f"_n{self.tmp}"
            self.tmp += 1
            timed = var.name == self.timed_loop and not self.timer_used
            if timed:   # wall time of this loop, for timing the program alone
                self.timer_used = True
                self.emit("ref_timer(0);")
            self.emit(f"{{ const int _st{n} = {st}; {var.cname} = {lo}; "
                      f"for (long {n} = ((long)({hi}) - {var.cname} + _st{n}) / _st{n}; {n} > 0; "
                      f"--{n}, {var.cname} += _st{n}) {{")
            self.ind += 1
            self.blocks.append("do timed" if timed else "do")
            return
        if re.match(r"end\s*do$", s):
            timed = bool(self.blocks) and self.blocks[-1] == "do timed"
            self.close(self.blocks[-1] if timed else "do")
            self.emit("} }")
            if timed:
                self.emit("ref_timer(1);")
            return
        if s.startswith("if") and re.match(r"if\s*\(", s):
            cond, rest = _paren_prefix(s[2:].lstrip(), self.ln)
            c = self.scalar(parse_expr(cond, self.ln))[0]
            if rest.strip() == "then":
                self.emit(f"if ({c}) {{")
                self.ind += 1
                self.blocks.append("if")
            else:
                self.emit(f"if ({c}) {{")
                self.ind += 1
                self.statement(rest.strip())
                self.ind -= 1
                self.emit("}")
            return
        m = re.match(r"else\s*if\s*\(", s)
        if m:
            cond, rest = _paren_prefix(s[m.end() - 1:], self.ln)
            if rest.strip() != "then":
                raise TranslateError(f"line {self.ln}: ELSE IF without THEN")
            if not self.blocks or self.blocks[-1] != "if":
                raise TranslateError(f"line {self.ln}: ELSE IF outside an IF block")
            c = self.scalar(parse_expr(cond, self.ln))[0]
            self.ind -= 1
            self.emit(f"}} else if ({c}) {{")
            self.ind += 1
            return
        if s == "else":
            if not self.blocks or self.blocks[-1] != "if":
                raise TranslateError(f"line {self.ln}: ELSE outside an IF block")
            self.ind -= 1
            self.emit("} else {")
            self.ind += 1
            return
        if re.match(r"end\s*if$", s):
            self.close("if")
            self.emit("}")
            return
        if s.startswith("call "):
            self.call(s)
            return
        m = re.match(r"stop\b\s*(.*)$", s)
        if m:
            msg = m.group(1).strip()
            if msg:
                tok = tokenize(msg, self.ln)
                msg = tok[0][1] if len(tok) == 1 and tok[0][0] == "str" else msg
            self.emit(f"ref_stop({json.dumps(msg)}, {self.ln});")
            return
        pos = _assign_pos(s)
        if pos is not None:
            self.assignment(s[:pos].strip(), s[pos + 1:].strip())
            return
        raise TranslateError(f"line {self.ln}: statement outside the subset: {s!r}")

    def io_statement(self, s):
        """WRITE to a unit or a character variable (formatted with literal
        strings and I edit descriptors, or list-directed integers and
        strings), OPEN of a file by name, CLOSE."""
        kw = re.match(r"(write|open|close)", s).group(1)
        ctrl, rest = _paren_prefix(s[len(kw):].lstrip(), self.ln)
        parts = [x.strip() for x in _split_top(ctrl, ",")]
        keyed = {}
        for k, x in enumerate(parts):
            m = re.match(r"(\w+)\s*=(?!=)\s*(.*)$", x)
            if not m and k > 1:
                raise TranslateError(f"line {self.ln}: {kw.upper()} with more than two positional items")
            keyed[m.group(1) if m else ("unit", "fmt")[k]] = m.group(2) if m else x
        if kw == "close":
            self.emit(f"ref_close({self.scalar(parse_expr(keyed['unit'], self.ln))[0]});")
            return
        if kw == "open":
            unit = self.scalar(parse_expr(keyed["unit"], self.ln))[0]
            self.emit(f"ref_open({unit}, {self.char_arg(keyed['file'])});")
            return
        unit, fmt = keyed.get("unit"), keyed.get("fmt")
        if unit is None or fmt is None or set(keyed) - {"unit", "fmt"}:
            raise TranslateError(f"line {self.ln}: WRITE control list outside the subset")
        if unit == "*":
            return                                 # standard output: progress messages only
        items = [x.strip() for x in _split_top(rest.strip(), ",")] if rest.strip() else []
        code = ["ref_rec_begin();"]
        if fmt == "*":
            for it in items:
                e = parse_expr(it, self.ln)
                if e[0] == "str":
                    code.append(f"ref_ld_s({json.dumps(e[1])});")
                else:
                    c, t = self.scalar(e)
                    if t == "i":
                        code.append(f"ref_ld_i({c});")
                    elif t in ("r", "d"):   # written so that reading back gives the value exactly
                        code.append(f"ref_ld_r((double)({c}), {1 if t == 'r' else 2});")
                    else:
                        raise TranslateError(f"line {self.ln}: list-directed output of logicals "
                                             "is outside the subset")
        else:
            tok = tokenize(fmt, self.ln)
            if len(tok) != 1 or tok[0][0] != "str":
                raise TranslateError(f"line {self.ln}: formats other than literals are outside the subset")
            k = 0
            for d in parse_format(tok[0][1], self.ln):
                if d[0] == "lit":
                    code.append(f"ref_put_s({json.dumps(d[1])});")
                    continue
                if k == len(items):   # output ends at the first data edit without an item
                    break
                c, t = self.scalar(parse_expr(items[k], self.ln))
                if t != "i":
                    raise TranslateError(f"line {self.ln}: I editing of a non-integer")
                code.append(f"ref_put_i({c}, {d[1]}, {d[2]});")
                k += 1
            if k < len(items):
                raise TranslateError(f"line {self.ln}: format reversion is outside the subset")
        target = self.syms.get(unit)
        if target is not None and target.ftype == "c":
            code.append(f"ref_rec_internal({target.cname}, {target.clen});")
        else:
            code.append(f"ref_rec_unit({self.scalar(parse_expr(unit, self.ln))[0]});")
        self.emit("{ " + " ".join(code) + " }")

    def char_arg(self, text):
        """C (pointer, length) arguments of a character variable or literal."""
        e = parse_expr(text, self.ln)
        if e[0] == "str":
            return f"{json.dumps(e[1])}, -1"
        s = self.syms.get(e[1]) if e[0] == "name" else None
        if s is None or s.ftype != "c":
            raise TranslateError(f"line {self.ln}: file names must be character variables or literals")
        return f"{s.cname}, {s.clen}"

    def close(self, kind):
        if not self.blocks or self.blocks[-1] != kind:
            raise TranslateError(f"line {self.ln}: unbalanced END {kind.split()[0].upper()}")
        self.blocks.pop()
        self.ind -= 1

    # ---- whole program ------------------------------------------------------------
    def body(self, stmts, load_after=None):
        """Translate the executable statements of one unit; returns its C lines.
        load_after = (line, names): the named arrays are loaded from the input
        directory right after the statement that starts on that source line."""
        hit = 0
        for ln, s in stmts:
            self.ln = ln
            self.statement(s)
            if load_after and ln == load_after[0]:
                hit += 1
                for name in load_after[1]:
                    sym = self.syms.get(name)
                    if sym is None or not sym.dims or sym.param:
                        raise TranslateError(f"cannot load {name}: not an array variable")
                    self.emit(f'ref_load("{name}", {sym.cname}, sizeof({sym.cname}));')
        if load_after and hit != 1:
            raise TranslateError(f"no statement starts on line {load_after[0]}")
        if self.blocks:
            raise TranslateError(f"unclosed {self.blocks[-1].upper()} block at the end")
        if self.timed_loop and not self.timer_used:
            raise TranslateError(f"no DO loop over {self.timed_loop} to time")
        missing = set(self.overrides) - self.used_overrides
        if missing:
            raise TranslateError(f"overridden names that are not parameters: {sorted(missing)}")
        out, self.out = self.out, []
        return out

    def declarations(self):
        """(parameter macros, static variables, largest array) of this unit.
        Parameters are compile-time constants, as in Fortran: macros that gcc
        folds, so that e.g. x**NPOWER with NPOWER = 2.d0 is pow(x, 2.0) with a
        literal exponent, which gcc (like gfortran) turns into x*x."""
        params, glob, cap = [], [], 1
        for name in self.order:                  # in declaration order
            s = self.syms[name]
            if s.param:
                self.ln = 0
                c, _ = self.scalar(s.init)
                params.append(f"#define {s.cname} (({CTYPE[s.ftype]})({c}))")
            elif s.dummy:
                continue
            elif s.ftype == "c":
                glob.append(f"static char {s.cname}[{s.clen + 1}];")
            elif s.dims:
                glob.append(f"static {CTYPE[s.ftype]} {s.cname}[{max(s.size, 1)}];")
                cap = max(cap, s.size)
            else:
                glob.append(f"static {CTYPE[s.ftype]} {s.cname};")
        return params, glob, cap

    def function(self, name, stmts):
        """C function ref_sub_<name>(void* ...) of a subroutine unit: every
        dummy argument arrives by reference, as in Fortran."""
        body = self.body(stmts)
        head = [f"static void ref_sub_{name}({', '.join(f'void* p{k}' for k in range(len(self.dummies))) or 'void'}) {{"]
        for k, a in enumerate(self.dummies):
            sym = self.syms.get(a)
            if sym is None:
                raise TranslateError(f"subroutine {name}: dummy argument {a} is not declared")
            head.append(f"  {CTYPE[sym.ftype]}* d_{a} = ({CTYPE[sym.ftype]}*)p{k};")
        return head + body + ["}", ""]

    def translate(self, stmts, dump=(), load=(), subroutines=(), load_after=None):
        """C source of the main program (and of the subroutine units given as
        (name, dummy names, statements)), with `load`ed variables read from
        the input directory before the first statement and `dump`ed ones
        written after the last; returns (C source, dump manifest)."""
        sub_params, sub_glob, sub_funcs, cap = [], [], [], 1
        for k, (sname, args, sstmts) in enumerate(subroutines):
            T = Translator(bounds=self.bounds, prefix=f"s{k}_", dummies=args, io=True)
            fn = T.function(sname, sstmts)
            p_, g_, c_ = T.declarations()
            sub_params += p_
            sub_glob += g_
            sub_funcs += fn
            cap = max(cap, c_)
            self.subs[sname] = len(args)
        body = self.body(stmts, load_after)
        self.ind = 1
        for name in load:
            s = self.syms.get(name)
            if s is None or s.param or s.ftype == "c":
                raise TranslateError(f"cannot load {name}: not a numeric variable")
            ref = s.cname if s.dims else "&" + s.cname
            self.emit(f'ref_load("{name}", {ref}, sizeof({s.cname}));')
        loads, self.out = self.out, []
        for name in dump:
            if name not in self.syms or self.syms[name].ftype == "c":
                raise TranslateError(f"cannot dump {name}: not a numeric variable")
            s = self.syms[name]
            if s.dims:
                self.emit(f'ref_dump("{name}", {s.cname}, sizeof({s.cname}));')
            elif s.param:   # a compile-time constant: dump a copy
                self.emit(f'{{ {CTYPE[s.ftype]} _p = {s.cname}; ref_dump("{name}", &_p, sizeof _p); }}')
            else:
                self.emit(f'ref_dump("{name}", &{s.cname}, sizeof({s.cname}));')
        dumps = self.out
        params, glob, cap_main = self.declarations()
        cap = max(cap, cap_main)
        # the dumps are written at the end, and by a STOP too (the state the
        # program stopped in: e.g. the step at which it blew up)
        src = [C_PRELUDE, f"const long ref_message_capacity = {cap}L;", *params, *sub_params,
               *glob, *sub_glob, "", *sub_funcs,
               "static void ref_dump_all(void) {", *dumps, "}", "",
               "void ref_main(void) {", "  ref_set_stop_hook(ref_dump_all);", *loads, *body,
               "  ref_dump_all();", "}", ""]
        manifest = {}
        for name in dump:
            s = self.syms[name]
            manifest[name] = {"dtype": NPTYPE[s.ftype],
                              "dims": [list(d) for d in s.dims] if s.dims else []}
        return "\n".join(src), manifest


C_PRELUDE = r"""/* Generated from a reference Fortran program by oracle/ref_f90c.py.
   Test infrastructure only: not part of the product, never committed. */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

void ref_stop(const char* msg, int line);
void ref_set_stop_hook(void (*hook)(void));
void ref_dump(const char* name, const void* data, size_t bytes);
void ref_timer(int end);
void ref_load(const char* name, void* data, size_t bytes);
void ref_rec_begin(void);
void ref_put_s(const char* s);
void ref_put_i(long v, int w, int m);
void ref_ld_i(long v);
void ref_ld_r(double v, int kind);
void ref_ld_s(const char* s);
void ref_rec_internal(char* buf, int len);
void ref_rec_unit(int unit);
void ref_open(int unit, const char* name, int len);
void ref_close(int unit);
void ref_mpi_init(void*);
void ref_mpi_finalize(void*);
void ref_mpi_comm_size(void*, void*, void*);
void ref_mpi_comm_rank(void*, void*, void*);
void ref_mpi_barrier(void*, void*);
void ref_mpi_sendrecv(void*, void*, void*, void*, void*, void*, void*, void*, void*, void*,
                      void*, void*, void*);
void ref_mpi_reduce(void*, void*, void*, void*, void*, void*, void*, void*);
void ref_mpi_allreduce(void*, void*, void*, void*, void*, void*, void*);

static inline long ref_chk(long i, long lo, long hi, const char* name, int line) {
  if (i < lo || i > hi) {
    fprintf(stderr, "subscript %ld of %s outside [%ld, %ld] at line %d\n", i, name, lo, hi, line);
    exit(4);
  }
  return i;
}
static inline int ref_ipow(int b, int e) {
  int r = 1;
  if (e < 0) return b == 1 ? 1 : (b == -1 ? ((-e) % 2 ? -1 : 1) : 0);
  while (e--) r *= b;
  return r;
}
"""


def parse_format(text: str, ln: int):
    """A format specification of literal strings and Iw / Iw.m edit
    descriptors -> [("lit", text) | ("i", w, m)] (m = -1 when absent)."""
    t = text.strip()
    if not (t.startswith("(") and t.endswith(")")):
        raise TranslateError(f"line {ln}: bad format {text!r}")
    out = []
    for part in _split_top(t[1:-1], ","):
        part = part.strip()
        if part[:1] in ("'", '"'):
            q = part[0]
            out.append(("lit", part[1:-1].replace(q + q, q)))
            continue
        m = re.fullmatch(r"i(\d+)(?:\.(\d+))?", part, re.I)
        if not m:
            raise TranslateError(f"line {ln}: format item {part!r} is outside the subset")
        out.append(("i", int(m.group(1)), int(m.group(2)) if m.group(2) else -1))
    return out


def subroutine_unit(stmts, name: str):
    """(dummy argument names, statements) of SUBROUTINE name."""
    inside, body, args = False, [], []
    for ln, s in stmts:
        if not inside:
            m = re.match(r"subroutine\s+(\w+)\s*(?:\((.*)\))?$", s)
            if m and m.group(1) == name:
                inside = True
                args = [a.strip() for a in (m.group(2) or "").split(",") if a.strip()]
            continue
        if re.match(r"end\s*subroutine\b", s) or s == "end":
            return args, body
        body.append((ln, s))
    raise TranslateError(f"no subroutine {name}")


def _same_section_only(e, lhs):
    """True when every reference in e to the array lhs names is lhs itself."""
    if isinstance(e, tuple):
        if e[0] in ("name", "ref") and e[1] == lhs[1]:
            return e == lhs
        return all(_same_section_only(x, lhs) for x in e[1:])
    if isinstance(e, list):
        return all(_same_section_only(x, lhs) for x in e)
    return True


def _split_top(s: str, sep: str) -> list[str]:
    out, depth, cur, quote = [], 0, [], None
    for ch in s:
        if quote:
            cur.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == sep and depth == 0:
            out.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    out.append("".join(cur))
    return out


def _paren_prefix(s: str, ln: int):
    """'(cond) rest' -> ('cond', 'rest')."""
    if not s.startswith("("):
        raise TranslateError(f"line {ln}: expected '('")
    depth, quote = 0, None
    for i, ch in enumerate(s):
        if quote:
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
            if depth == 0:
                return s[1:i], s[i + 1:]
    raise TranslateError(f"line {ln}: unbalanced parentheses")


def _assign_pos(s: str):
    """Position of the top-level '=' of an assignment, or None."""
    depth, quote = 0, None
    for i, ch in enumerate(s):
        if quote:
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "=" and depth == 0:
            prev = s[i - 1] if i else ""
            nxt = s[i + 1] if i + 1 < len(s) else ""
            if prev in "=/<>" or nxt in "=>":
                continue
            return i
    return None


# ---------------------------------------------------------------------------
# build and run
# ---------------------------------------------------------------------------
def translate_file(src: str, overrides: dict | None = None, dump=(), bounds=True,
                   stf: str | None = None, timed_loop: str | None = None, load=(),
                   subroutines=(), io: bool = False, load_after=None):
    """C source and dump manifest of src's main program. subroutines lists
    (file, name) units to translate beside it and call; io translates the
    main program's WRITE/OPEN/CLOSE as well (always done in subroutines);
    load and load_after name variables read from files (Translator.body)."""
    stmts = main_program(read_statements(src, stf))
    units = [(name, *subroutine_unit(read_statements(path), name)) for path, name in subroutines]
    T = Translator(overrides, bounds, timed_loop, io=io)
    return T.translate(stmts, dump, load, units, load_after)


@dataclass
class RefProgram:
    exe: str
    manifest: dict
    overrides: dict = field(default_factory=dict)

    def run(self, nprocs: int = 1, workdir: str | None = None, timeout: float = 900.0,
            inputs: dict | None = None, files=(), allow_stop: bool = False):
        """Run the translated program on nprocs emulated MPI ranks; returns
        one {name: array} per rank (Fortran-ordered arrays, shaped by their
        declared bounds), plus `loop_seconds` when the program times a loop.
        The program runs in workdir, by default a temporary directory that
        is removed afterwards: its dump files and the files it opens go
        there. inputs maps the names the program loads to arrays, written
        in Fortran order; `files` names files it writes, returned as text
        under out[0]["files"]. With allow_stop, a program that ends on a
        STOP returns its dumps of that moment and the STOP message under
        out[r]["stop"]; otherwise a STOP is an error."""
        import shutil
        import tempfile
        own = workdir is None
        workdir = tempfile.mkdtemp(prefix="ref_run_") if own else workdir
        try:
            os.makedirs(workdir, exist_ok=True)
            indir = os.path.join(workdir, "inputs")
            os.makedirs(indir, exist_ok=True)
            for name, a in (inputs or {}).items():
                with open(os.path.join(indir, name + ".bin"), "wb") as f:
                    f.write(np.asarray(a).tobytes(order="F"))
            proc = subprocess.run([os.path.abspath(self.exe), "-np", str(nprocs), "-o", workdir,
                                   "-i", indir, "-t", str(int(timeout))], capture_output=True,
                                  text=True, timeout=timeout + 30, cwd=workdir)
            stopped = proc.returncode == 3 and allow_stop
            if proc.returncode != 0 and not stopped:
                raise RuntimeError(f"{os.path.basename(self.exe)} exited with {proc.returncode}: "
                                   f"{proc.stderr.strip()[-2000:]}")
            out = []
            for r in range(nprocs):
                d = {}
                for name, m in self.manifest.items():
                    a = np.fromfile(os.path.join(workdir, f"{name}.{r}.bin"), dtype=m["dtype"])
                    shp = [hi - lo + 1 for lo, hi in m["dims"]]
                    d[name] = a.reshape(shp, order="F") if shp else a[0]
                t = os.path.join(workdir, f"loop_seconds.{r}.bin")
                if os.path.exists(t):
                    d["loop_seconds"] = float(np.fromfile(t, dtype="<f8")[0])
                t = os.path.join(workdir, f"stop.{r}.txt")
                if os.path.exists(t):
                    with open(t) as f:
                        d["stop"] = f.read().strip()
                out.append(d)
            if files:
                out[0]["files"] = {}
                for name in files:
                    with open(os.path.join(workdir, name)) as f:
                        out[0]["files"][name] = f.read()
            return out
        finally:
            if own:
                shutil.rmtree(workdir, ignore_errors=True)


PARITY_FLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math"]
# the reference Makefile's optimisation level (-O3, no -march, no OpenMP since
# its OPEN_MP variable is unset), with gcc's default floating-point
# contraction as gfortran would apply it: the build the CPU timing runs
TIMING_FLAGS = ["-O3"]


def build(src: str, tag: str, overrides: dict | None = None, dump=(), bounds=True,
          stf: str | None = None, timed_loop: str | None = None, cc: str = "gcc",
          flags: list | None = None, load=(), subroutines=(), io: bool = False,
          load_after=None) -> RefProgram:
    """Translate src with the given parameter overrides (and source-time
    function, when stf names one) into oracle/_ref/<tag>.c, then compile it
    for this machine (compile_translated) with `flags` (PARITY_FLAGS by
    default)."""
    code, manifest = translate_file(src, overrides, dump, bounds, stf, timed_loop, load,
                                    subroutines, io, load_after)
    os.makedirs(REF_OUT, exist_ok=True)
    cpath = os.path.join(REF_OUT, tag + ".c")
    if not (os.path.exists(cpath) and open(cpath).read() == code):
        with open(cpath, "w") as f:
            f.write(code)
    meta = {"source": os.path.basename(src), "overrides": overrides or {}, "stf": stf,
            "flags": list(flags or PARITY_FLAGS), "manifest": manifest}
    with open(os.path.join(REF_OUT, tag + ".json"), "w") as f:
        json.dump(meta, f, indent=1)
    return compile_translated(tag, cc)


def translated_exists(tag: str) -> bool:
    return all(os.path.exists(os.path.join(REF_OUT, tag + ext)) for ext in (".c", ".json"))


def compile_translated(tag: str, cc: str = "gcc") -> RefProgram:
    """Compile oracle/_ref/<tag>.c (written by build) with the MPI stand-in
    into oracle/_ref/<tag>.<machine>; recompiled only when the C or the
    stand-in changed. The C travels with the tree, so a machine without the
    reference sources can still build and run the translated program."""
    import platform
    cpath = os.path.join(REF_OUT, tag + ".c")
    with open(os.path.join(REF_OUT, tag + ".json")) as f:
        meta = json.load(f)
    exe = os.path.join(REF_OUT, f"{tag}.{platform.machine()}")
    flags = meta.get("flags", PARITY_FLAGS)
    with open(cpath) as f, open(MPI_RUNTIME) as g:
        stamp = hashlib.sha256((f.read() + g.read() + " ".join(flags)).encode()).hexdigest()
    spath = exe + ".sha256"
    if not (os.path.exists(exe) and os.path.exists(spath) and open(spath).read() == stamp):
        subprocess.run([cc, *flags, "-std=gnu11", "-w", "-o", exe, cpath, MPI_RUNTIME, "-lm",
                        "-lpthread"], check=True)
        with open(spath, "w") as f:
            f.write(stamp)
    return RefProgram(exe, meta["manifest"], dict(meta["overrides"]))


# the programs on the path, by the file names they ship under
REFERENCE_PROGRAMS = {
    "cpml2d": "seismic_CPML_2D_isotropic_second_order.f90",
    "cpml2d4": "seismic_CPML_2D_isotropic_fourth_order.f90",
    "pml2d": "seismic_PML_Collino_2D_isotropic.f90",
    "cpml3d": "seismic_CPML_3D_isotropic_MPI_OpenMP.f90",
}


# where the reference sources lie on the machine that has them
DEFAULT_REF_DIR = "/root/reference"

# The 3D plain workload as the 3D program's parameter lines: 276^3 (256
# interior + 10 PML points per face), the source at the centre with the
# Ricker wavelet, 64 receivers on the x line through the centre at
# i = 11 + round(r * 255 / 63), on 12 ranks of 23 planes (276 = 12 x 23).
PLAIN_3D_RANKS = 12


def plain_3d_overrides(nstep: int = 2500) -> dict:
    return {"NX": 276, "NY": 276, "NZ": 276, "NPROC": PLAIN_3D_RANKS, "NSTEP": nstep,
            "ISOURCE": 138, "JSOURCE": 138, "NREC": 64, "xdeb": "100.d0", "xfin": "2650.d0",
            "ydeb": "1370.d0", "yfin": "1370.d0"}


# the translated program the CPU reference timing runs: a bounded sample of
# the 3D plain workload's time loop, its wall time measured by ref_timer
BENCH_TAG = "bench_3d_plain"
BENCH_SAMPLE_STEPS = 40


def build_bench_program(ref_dir: str) -> RefProgram:
    return build(os.path.join(ref_dir, REFERENCE_PROGRAMS["cpml3d"]), BENCH_TAG,
                 plain_3d_overrides(BENCH_SAMPLE_STEPS), ["sisvx", "sisvy", "total_energy"],
                 bounds=False, stf="ricker", timed_loop="it", flags=TIMING_FLAGS)


def build_reference_programs(ref_dir: str = DEFAULT_REF_DIR) -> list[str]:
    """Translate and compile the four programs as shipped (no parameter
    changed) into oracle/_ref/<name>_shipped (a check that the whole of each
    program stays inside the translated subset), and the timing program of
    the 3D plain workload. Where the sources are absent but a translated
    program's C travelled here, compile that C for this machine. Returns the
    binaries."""
    exes = []
    if os.path.isdir(ref_dir):
        for name, fname in REFERENCE_PROGRAMS.items():
            dump = ["sisvx", "sisvy"]
            exes.append(build(os.path.join(ref_dir, fname), name + "_shipped", {}, dump).exe)
        exes.append(build_bench_program(ref_dir).exe)
    else:
        for tag in [n + "_shipped" for n in REFERENCE_PROGRAMS] + [BENCH_TAG]:
            if translated_exists(tag):
                exes.append(compile_translated(tag).exe)
    return exes
