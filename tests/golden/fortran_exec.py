"""Execute a subset of free-form Fortran 90 as Python (test infrastructure).

No Fortran compiler exists on the machines this project builds on, so the
reference's own routines cannot be compiled.  This module translates the part
of Fortran those routines use into Python source, in memory, and runs it; the
translation is never stored.  ``tests/golden/make_ref_golden.py`` uses it to run
the reference's source files on the golden cases and commits only the numbers
they produce, which the oracle must then reproduce bit for bit.

Semantics kept from the language (and from the reference build's flags: every
default REAL is 8 bytes, ``-r8``; the OpenMP sentinel ``!$`` lines are compiled,
``!$omp`` directives are comments and run serially, one thread):

* every arithmetic operation rounds to an IEEE double once, in the order the
  source writes it (Python floats; no contraction, no reassociation);
  ``x**2`` and ``x**3`` with a literal exponent are products, as compilers emit
  them;
* INTEGER division truncates toward zero, MOD takes the dividend's sign,
  REAL-to-INTEGER assignment truncates;
* arrays are column-major with declared lower bounds and checked subscripts;
  an array argument is associated by element sequence (``CALL S(WK(1,3))``
  hands the callee the storage from that element on, and ``CALL S(WK, WK)``
  aliases both dummies);
* scalar arguments are copied in and, unless INTENT(IN), copied out;
* a DO variable after the loop holds start + trip count x step; GOTO leaves
  any nesting to a label of the procedure's outermost statement list;
* local variables start undefined (REAL arrays NaN, others None), so a read
  of a value the source never set fails or shows instead of passing silently.

Unsupported constructs raise ``FortranError`` at translation time.
"""
from __future__ import annotations

import math
import re
import struct
from dataclasses import dataclass, field


class FortranError(Exception):
    pass


class _Goto(Exception):
    def __init__(self, label):
        super().__init__(label)
        self.label = label


class FortranStop(Exception):
    pass


class _LoopCtl(Exception):
    """CYCLE / EXIT of DO loop ``n`` from inside a GOTO dispatcher."""

    def __init__(self, kind, n):
        super().__init__(kind)
        self.kind, self.n = kind, n


# ---------------------------------------------------------------------------
# Runtime: arrays, array values, intrinsics


class FArray:
    """Column-major array over a shared Python list, with Fortran bounds."""

    __slots__ = ("d", "off", "lb", "ext", "st", "kind", "size")

    def __init__(self, d, off, lb, ext, kind):
        self.d, self.off, self.kind = d, off, kind
        self.lb, self.ext = tuple(lb), tuple(ext)
        st, s = [], 1
        for e in self.ext:
            st.append(s)
            s *= e
        self.st, self.size = tuple(st), s

    @staticmethod
    def new(kind, bounds, fill=None):
        lb = [int(lo) for lo, _ in bounds]
        ext = [max(0, int(hi) - int(lo) + 1) for lo, hi in bounds]
        n = 1
        for e in ext:
            n *= e
        if fill is None:
            fill = math.nan if kind == "real" else None
        return FArray([fill] * n, 0, lb, ext, kind)

    @staticmethod
    def from_list(kind, values, lb=(1,), ext=None):
        values = list(values)
        return FArray(values, 0, lb, ext if ext is not None else (len(values),), kind)

    def idx(self, subs):
        if len(subs) != len(self.ext):
            raise IndexError(f"rank {len(self.ext)} array with {len(subs)} subscripts")
        o = self.off
        for s, l, e, t in zip(subs, self.lb, self.ext, self.st):
            k = s - l
            if k < 0 or k >= e:
                raise IndexError(f"subscript {s} outside {l}:{l + e - 1}")
            o += k * t
        return o

    def __getitem__(self, subs):
        return self.d[self.idx(subs if isinstance(subs, tuple) else (subs,))]

    def __setitem__(self, subs, v):
        self.d[self.idx(subs if isinstance(subs, tuple) else (subs,))] = v

    def g1(self, i):
        k = i - self.lb[0]
        if k < 0 or k >= self.ext[0]:
            raise IndexError(f"subscript {i} outside {self.lb[0]}:{self.lb[0] + self.ext[0] - 1}")
        return self.d[self.off + k]

    def s1(self, i, v):
        k = i - self.lb[0]
        if k < 0 or k >= self.ext[0]:
            raise IndexError(f"subscript {i} outside {self.lb[0]}:{self.lb[0] + self.ext[0] - 1}")
        self.d[self.off + k] = v

    def g2(self, i, j):
        k, m = i - self.lb[0], j - self.lb[1]
        if k < 0 or k >= self.ext[0] or m < 0 or m >= self.ext[1]:
            raise IndexError(f"subscripts ({i}, {j}) outside the bounds")
        return self.d[self.off + k + m * self.st[1]]

    def s2(self, i, j, v):
        k, m = i - self.lb[0], j - self.lb[1]
        if k < 0 or k >= self.ext[0] or m < 0 or m >= self.ext[1]:
            raise IndexError(f"subscripts ({i}, {j}) outside the bounds")
        self.d[self.off + k + m * self.st[1]] = v

    def view_at(self, subs):
        """Sequence association from element ``subs`` to the array's end."""
        o = self.idx(subs)
        return FArray(self.d, o, (1,), (self.off + self.size - o,), self.kind)

    def section_view(self, lo, hi):
        """The contiguous section (lo:hi) of a rank-1 array, as an actual argument."""
        o = self.idx((lo,))
        if hi < lo:
            return FArray(self.d, o, (1,), (0,), self.kind)
        self.idx((hi,))
        return FArray(self.d, o, (1,), (hi - lo + 1,), self.kind)

    def as_dummy(self, bounds):
        """This actual argument seen through an explicit-shape dummy."""
        lb = [int(lo) for lo, _ in bounds]
        ext = [max(0, int(hi) - int(lo) + 1) for lo, hi in bounds]
        n = 1
        for e in ext:
            n *= e
        if n > self.size:
            raise IndexError(f"dummy of {n} elements over an actual of {self.size}")
        return FArray(self.d, self.off, lb, ext, self.kind)

    def values(self):
        return self.d[self.off:self.off + self.size]

    def to_list(self):
        return list(self.values())


class AV:
    """An array value: elements in array element order and a shape."""

    __slots__ = ("v", "shape")

    def __init__(self, v, shape):
        self.v, self.shape = list(v), tuple(shape)


def _spec_indices(lb, ext, spec):
    if isinstance(spec, tuple):
        lo, hi, step = spec
        lo = lb if lo is None else lo
        hi = lb + ext - 1 if hi is None else hi
        step = 1 if step is None else step
        return list(range(lo, hi + (1 if step > 0 else -1), step)), True
    return [spec], False


def _sec_offsets_ordered(a, specs):
    """Offsets in array element order (first subscript fastest)."""
    if specs is None:
        specs = [(None, None, None)] * len(a.ext)
    idx_lists, shape = [], []
    for l, e, s in zip(a.lb, a.ext, specs):
        ids, is_range = _spec_indices(l, e, s)
        for i in ids:
            if i - l < 0 or i - l >= e:
                raise IndexError(f"section subscript {i} outside {l}:{l + e - 1}")
        idx_lists.append([(i - l) for i in ids])
        if is_range:
            shape.append(len(ids))
    offs = [a.off]
    for ks, t in zip(idx_lists, a.st):
        offs = [o + k * t for k in ks for o in offs]
    return offs, shape


def _sec(a, specs):
    offs, shape = _sec_offsets_ordered(a, specs)
    return AV([a.d[o] for o in offs], shape)


def _whole(a):
    return AV(a.values(), a.ext)


def _asgn(a, specs, value):
    offs, shape = _sec_offsets_ordered(a, specs)
    if isinstance(value, AV):
        if len(value.v) != len(offs):
            raise IndexError(f"assigning {len(value.v)} values to {len(offs)} elements")
        for o, v in zip(offs, value.v):
            a.d[o] = v
    else:
        for o in offs:
            a.d[o] = value


def _ew(fn, *xs):
    n, shape = None, None
    for x in xs:
        if isinstance(x, AV):
            if n is not None and len(x.v) != n:
                raise IndexError("nonconformable array operands")
            n, shape = len(x.v), x.shape
    cols = [x.v if isinstance(x, AV) else [x] * n for x in xs]
    return AV([fn(*t) for t in zip(*cols)], shape)


def _cons(*items):
    out = []
    for it in items:
        out.extend(it.v if isinstance(it, AV) else [it])
    return AV(out, (len(out),))


def _masked(x, mask):
    xs = x.v if isinstance(x, AV) else [x]
    if mask is None:
        return xs
    ms = mask.v if isinstance(mask, AV) else [mask] * len(xs)
    return [v for v, m in zip(xs, ms) if m]


def _minval(x, mask=None, kind="real"):
    vs = _masked(x, mask)
    if not vs:
        return math.inf if kind == "real" else 2 ** 31 - 1
    r = vs[0]
    for v in vs[1:]:
        if v < r:
            r = v
    return r


def _maxval(x, mask=None, kind="real"):
    vs = _masked(x, mask)
    if not vs:
        return -math.inf if kind == "real" else -(2 ** 31 - 1)
    r = vs[0]
    for v in vs[1:]:
        if v > r:
            r = v
    return r


def _sum(x, kind="real"):
    vs = x.v if isinstance(x, AV) else [x]
    r = 0.0 if kind == "real" else 0
    for v in vs:
        r = r + v
    return r


def _maxloc1(x):
    """MAXLOC(array, 1) of a rank-1 value: the first position of the maximum, from 1."""
    vs = x.v
    if not vs:
        return 0
    best, pos = vs[0], 1
    for k, v in enumerate(vs[1:], 2):
        if v > best:
            best, pos = v, k
    return pos


def _minloc1(x):
    vs = x.v
    if not vs:
        return 0
    best, pos = vs[0], 1
    for k, v in enumerate(vs[1:], 2):
        if v < best:
            best, pos = v, k
    return pos


class _Obj:
    """An element of a derived-type array: components as attributes f_<name>."""

    def __init__(self, comps):
        for c in comps:
            setattr(self, "f_" + c, None)


def _new_objs(a, comps):
    a.d[a.off:a.off + a.size] = [_Obj(comps) for _ in range(a.size)]
    return a


def _asgn_comp(a, specs, comp, value):
    offs, _ = _sec_offsets_ordered(a, specs)
    vals = value.v if isinstance(value, AV) else [value] * len(offs)
    if len(vals) != len(offs):
        raise IndexError(f"assigning {len(vals)} values to {len(offs)} components")
    for o, v in zip(offs, vals):
        setattr(a.d[o], comp, v)


def _temp_array(x, kind):
    """An array-valued expression passed to an array dummy: a temporary copy."""
    return FArray(list(x.v), 0, (1,), (len(x.v),), kind)


def _rpowi(x, n):
    """REAL ** INTEGER as compilers expand it: binary powering by products, the
    reciprocal for a negative exponent."""
    if n < 0:
        return 1.0 / _rpowi(x, -n)
    r, b = 1.0, x
    first = True
    while n:
        if n & 1:
            r = b if first else r * b
            first = False
        n >>= 1
        if n:
            b = b * b
    return r


def _nint(x):
    """NINT: the nearest integer, halves away from zero."""
    t = math.trunc(x)
    f = x - t
    if f >= 0.5:
        return t + 1
    if f <= -0.5:
        return t - 1
    return t


def _strfix(v, n):
    """A CHARACTER value stored in a variable of length n: cut or blank-padded."""
    return v if n is None else v[:n].ljust(n)


def _substr(v, lo, hi):
    lo = 1 if lo is None else lo
    hi = len(v) if hi is None else hi
    if lo < 1 or hi > len(v):
        raise IndexError(f"substring ({lo}:{hi}) of a string of length {len(v)}")
    return v[lo - 1:hi]


def _strcmp(a, b):
    """Character comparison with the shorter operand padded with blanks."""
    n = max(len(a), len(b))
    a, b = a.ljust(n), b.ljust(n)
    return (a > b) - (a < b)


class _IOError(Exception):
    """A failed OPEN or READ (code > 0) or an end of file (code < 0)."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class _Record:
    """Reads one unformatted record's values in order (big-endian)."""

    def __init__(self, data: bytes):
        self.b, self.p = data, 0

    def _take(self, n):
        if self.p + n > len(self.b):
            raise _IOError(2, f"input record of {len(self.b)} bytes too short")
        v = self.b[self.p:self.p + n]
        self.p += n
        return v

    def int(self):
        return struct.unpack(">i", self._take(4))[0]

    def real(self):
        return struct.unpack(">d", self._take(8))[0]

    def logical(self):
        return struct.unpack(">i", self._take(4))[0] != 0

    def char(self, n):
        return self._take(n).decode("latin-1")


class _RecordOut:
    def __init__(self):
        self.parts = []

    def int(self, v):
        self.parts.append(struct.pack(">i", int(v)))

    def real(self, v):
        self.parts.append(struct.pack(">d", float(v)))

    def logical(self, v):
        self.parts.append(struct.pack(">i", 1 if v else 0))

    def char(self, v, n=None):
        v = v if n is None else _strfix(v, n)
        self.parts.append(v.encode("latin-1"))

    def data(self):
        return b"".join(self.parts)


class FortranFiles:
    """Unformatted sequential files in memory: name -> bytes, each record framed
    by big-endian 4-byte lengths (a negative head marks a record continued in
    the next subrecord)."""

    def __init__(self, files=None):
        self.files = dict(files or {})
        self.units = {}

    @staticmethod
    def records(data: bytes):
        out, p, cur = [], 0, b""
        while p < len(data):
            (n,) = struct.unpack_from(">i", data, p)
            m = abs(n)
            cur += data[p + 4:p + 4 + m]
            p += 8 + m
            if n >= 0:
                out.append(cur)
                cur = b""
        return out

    def newunit(self):
        n = -10 - len(self.units)
        while n in self.units:
            n -= 1
        return n

    def open(self, unit, name, status="unknown", form="formatted"):
        name = name.strip()
        if not form.strip().lower().startswith("unformatted"):
            raise FortranError(f"formatted OPEN of {name}")
        st = status.strip().lower()
        if st == "old" and name not in self.files:
            raise _IOError(29, f"no file {name}")
        recs = self.records(self.files[name]) if name in self.files and st != "replace" else []
        self.units[unit] = {"name": name, "recs": recs, "pos": 0, "out": None}

    def read(self, unit):
        u = self.units.get(unit)
        if u is None:
            raise _IOError(29, f"unit {unit} is not open")
        if u["pos"] >= len(u["recs"]):
            raise _IOError(-1, f"end of file {u['name']}")
        u["pos"] += 1
        return _Record(u["recs"][u["pos"] - 1])

    def write(self, unit, data: bytes):
        u = self.units[unit]
        if u["out"] is None:
            u["out"] = u["recs"][:u["pos"]]
        u["out"].append(data)

    def close(self, unit):
        u = self.units.pop(unit, None)
        if u is not None and u["out"] is not None:
            self.files[u["name"]] = b"".join(struct.pack(">i", len(r)) + r + struct.pack(">i", len(r))
                                             for r in u["out"])


def _read_into(a, specs, rec, kind, clen=None):
    offs, _ = _sec_offsets_ordered(a, specs)
    for o in offs:
        a.d[o] = rec.char(clen) if kind == "char" else getattr(rec, kind)()


def _write_from(w, a, specs, kind):
    offs, _ = _sec_offsets_ordered(a, specs)
    for o in offs:
        getattr(w, kind)(a.d[o])


def _idiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


def _imod(a, b):
    return a - _idiv(a, b) * b


def _isign(a, b):
    return abs(a) if b >= 0 else -abs(a)


def _fmax(*xs):
    r = xs[0]
    for x in xs[1:]:
        if x > r:
            r = x
    return r


def _fmin(*xs):
    r = xs[0]
    for x in xs[1:]:
        if x < r:
            r = x
    return r


def _ubound(a, dim=None):
    if dim is None:
        return AV([l + e - 1 for l, e in zip(a.lb, a.ext)], (len(a.ext),))
    return a.lb[dim - 1] + a.ext[dim - 1] - 1


def _lbound(a, dim=None):
    if dim is None:
        return AV(list(a.lb), (len(a.ext),))
    return a.lb[dim - 1]


def _size(a, dim=None):
    return a.size if dim is None else a.ext[dim - 1]


RUNTIME = {
    "FArray": FArray, "AV": AV, "_sec": _sec, "_whole": _whole, "_asgn": _asgn, "_ew": _ew,
    "_cons": _cons, "_minval": _minval, "_maxval": _maxval, "_idiv": _idiv, "_imod": _imod,
    "_isign": _isign, "_fmax": _fmax, "_fmin": _fmin, "_ubound": _ubound, "_lbound": _lbound,
    "_size": _size, "_sum": _sum, "_maxloc1": _maxloc1, "_minloc1": _minloc1,
    "_temp_array": _temp_array, "_IOError": _IOError, "_RecordOut": _RecordOut, "_read_into": _read_into,
    "_write_from": _write_from, "FortranFiles": FortranFiles, "_strfix": _strfix, "_substr": _substr, "_strcmp": _strcmp, "_rpowi": _rpowi, "_nint": _nint, "_new_objs": _new_objs, "_asgn_comp": _asgn_comp, "FortranError": FortranError, "_Goto": _Goto, "_LoopCtl": _LoopCtl, "FortranStop": FortranStop, "math": math,
}


# ---------------------------------------------------------------------------
# Source handling: preprocessor, comments, continuations


def preprocess(text: str, defines: set[str]) -> list[str]:
    """Apply #ifdef / #ifndef / #if [!]defined(A) [|| / && ...] / #else / #endif
    and object-like #define macros (identifier replacement, case-sensitive)."""
    out, stack, macros = [], [], {}
    defines = set(defines)

    def cond(expr):
        e = expr.strip()
        e = re.sub(r"!\s*defined\s*\(\s*(\w+)\s*\)", lambda m: str(m.group(1).upper() not in defines), e)
        e = re.sub(r"defined\s*\(\s*(\w+)\s*\)", lambda m: str(m.group(1).upper() in defines), e)
        e = e.replace("||", " or ").replace("&&", " and ")
        if not re.fullmatch(r"[\sA-Za-z()]*", e):
            raise FortranError(f"unsupported #if expression: {expr}")
        return bool(eval(e, {"__builtins__": {}}, {}))

    # split on newlines only: comment bytes of other encodings, read as latin-1,
    # include characters that str.splitlines() would also break at
    for line in text.replace("\r\n", "\n").split("\n"):
        s = line.strip()
        if s.startswith("#"):
            m = re.match(r"#\s*(\w+)\s*(.*)", s)
            kw, rest = m.group(1).lower(), m.group(2)
            active = all(a for a, _ in stack)
            if kw == "ifdef":
                stack.append((rest.split()[0].upper() in defines, False))
            elif kw == "ifndef":
                stack.append((rest.split()[0].upper() not in defines, False))
            elif kw == "if":
                stack.append((cond(rest), False))
            elif kw == "else":
                a, _ = stack.pop()
                stack.append((not a, True))
            elif kw == "endif":
                stack.pop()
            elif kw in ("define", "undef", "include") and not active:
                pass
            elif kw == "define":
                mm = re.match(r"(\w+)(\s+(.*))?$", rest)
                if mm is None or "(" in mm.group(1):
                    raise FortranError(f"unsupported macro: {s}")
                macros[mm.group(1)] = (mm.group(3) or "").strip()
                defines.add(mm.group(1).upper())
            elif kw == "undef":
                macros.pop(rest.strip(), None)
                defines.discard(rest.strip().upper())
            else:
                raise FortranError(f"unsupported directive: {s}")
            out.append("")
            continue
        if all(a for a, _ in stack):
            for name, val in macros.items():
                line = re.sub(r"\b" + re.escape(name) + r"\b", val, line)
            out.append(line)
        else:
            out.append("")
    if stack:
        raise FortranError("unterminated #if")
    return out


def fixed_to_free(text: str) -> str:
    """Fixed-form source (comment lines with C, c, * or ! in column 1, labels
    in columns 1-5, continuation marks in column 6, statements in columns
    7-72) as free-form lines."""
    out = []
    for raw in text.replace("\r\n", "\n").split("\n"):
        line = raw.expandtabs(6)
        if line.startswith("#"):                 # preprocessor directives pass through
            out.append(line)
            continue
        if not line.strip() or line[0] in "Cc*!":
            out.append("")
            continue
        body = line[6:72]
        if len(line) > 5 and line[5] not in " 0":
            k = len(out) - 1
            while k >= 0 and not out[k]:
                k -= 1
            if k < 0:
                raise FortranError("continuation line without a statement")
            out[k] = out[k] + " &"
            out.append("&" + body)
            continue
        label = line[:5].strip()
        out.append((label + " " if label else "") + body)
    return "\n".join(out)


def _strip_comment(line: str) -> str:
    q = None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "!":
            return line[:i]
    return line


def logical_lines(lines: list[str]) -> list[tuple[int, str]]:
    """Join continuations, drop comments (compiling ``!$`` sentinel lines), split on ';'."""
    out, buf, start = [], "", 0
    for no, raw in enumerate(lines, 1):
        s = raw.strip()
        if s.lower().startswith("!$") and not s.lower().startswith("!$omp"):
            s = s[2:].strip()
        s = _strip_comment(s).rstrip()
        if not s:
            continue
        if buf and s.startswith("&"):
            s = s[1:]
        cont = s.endswith("&")
        if cont:
            s = s[:-1]
        if not buf:
            start = no
        buf += s + (" " if cont else "")
        if not cont:
            for part in _split_semicolons(buf):
                if part.strip():
                    out.append((start, part.strip()))
            buf = ""
    return out


def _split_semicolons(s):
    parts, q, cur = [], None, ""
    for ch in s:
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == ";":
            parts.append(cur)
            cur = ""
            continue
        cur += ch
    parts.append(cur)
    return parts


# ---------------------------------------------------------------------------
# Tokens and expressions

_TOKEN = re.compile(r"""
    (?P<ws>\s+)
  | (?P<dotop>\.(?:eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv|true|false)\.)
  | (?P<num>(?:\d+(?:\.(?![a-zA-Z]+\.)\d*)?|\.\d+)(?:[eEdD][+-]?\d+)?(?:_\w+)?)
  | (?P<str>'(?:[^']|'')*'|"(?:[^"]|"")*")
  | (?P<name>[a-zA-Z_]\w*)
  | (?P<op>\*\*|//|==|/=|<=|>=|=>|\(/|/\)|[-+*/()<>,:=%\[\]])
""", re.X | re.I)


def tokenize(s: str):
    toks, pos = [], 0
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise FortranError(f"cannot tokenize at: {s[pos:pos + 30]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        v = m.group()
        if kind in ("name", "dotop"):
            v = v.lower()
        toks.append((kind, v))
    return toks


@dataclass
class Num:
    text: str
    typ: str


@dataclass
class Str:
    s: str


@dataclass
class Lit:
    v: bool


@dataclass
class Name:
    name: str


@dataclass
class Range:
    lo: object
    hi: object
    step: object


@dataclass
class Kw:
    name: str
    value: object


@dataclass
class Ref:
    name: str
    args: list


@dataclass
class Comp:
    base: object
    comp: str


@dataclass
class Bin:
    op: str
    l: object
    r: object


@dataclass
class Un:
    op: str
    x: object


@dataclass
class Cons:
    items: list


class Parser:
    _REL = {"==": "==", ".eq.": "==", "/=": "!=", ".ne.": "!=", "<": "<", ".lt.": "<", "<=": "<=",
            ".le.": "<=", ">": ">", ".gt.": ">", ">=": ">=", ".ge.": ">="}

    def __init__(self, toks):
        self.t, self.i = toks, 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, v=None):
        tok = self.peek()
        if v is not None and tok[1] != v:
            raise FortranError(f"expected {v!r}, got {tok[1]!r}")
        self.i += 1
        return tok

    def at_end(self):
        return self.i >= len(self.t)

    def expr(self):
        return self.eqv()

    def eqv(self):
        x = self.lor()
        while self.peek()[1] in (".eqv.", ".neqv."):
            op = self.take()[1]
            x = Bin("==" if op == ".eqv." else "!=", x, self.lor())
        return x

    def lor(self):
        x = self.land()
        while self.peek()[1] == ".or.":
            self.take()
            x = Bin("or", x, self.land())
        return x

    def land(self):
        x = self.lnot()
        while self.peek()[1] == ".and.":
            self.take()
            x = Bin("and", x, self.lnot())
        return x

    def lnot(self):
        if self.peek()[1] == ".not.":
            self.take()
            return Un("not", self.lnot())
        return self.rel()

    def rel(self):
        x = self.concat()
        if self.peek()[1] in self._REL:
            op = self._REL[self.take()[1]]
            x = Bin(op, x, self.concat())
        return x

    def concat(self):
        x = self.add()
        while self.peek()[1] == "//":
            self.take()
            x = Bin("//", x, self.add())
        return x

    def add(self):
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            x = self.mul()
            x = Un("-", x) if op == "-" else x
        else:
            x = self.mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            x = Bin(op, x, self.mul())
        return x

    def mul(self):
        x = self.pow()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            x = Bin(op, x, self.pow())
        return x

    def pow(self):
        x = self.primary()
        if self.peek()[1] == "**":
            self.take()
            if self.peek()[1] in ("+", "-"):
                op = self.take()[1]
                y = self.pow()
                return Bin("**", x, Un("-", y) if op == "-" else y)
            return Bin("**", x, self.pow())
        return x

    def primary(self):
        kind, v = self.peek()
        if kind == "num":
            self.take()
            t = v.lower().split("_")[0]
            return Num(t, "real" if any(c in t for c in ".ed") else "int")
        if kind == "str":
            self.take()
            return Str(v[1:-1])
        if v in (".true.", ".false."):
            self.take()
            return Lit(v == ".true.")
        if v == "(":
            self.take()
            x = self.expr()
            self.take(")")
            return x
        if v in ("[", "(/"):
            close = "]" if v == "[" else "/)"
            self.take()
            items = []
            while self.peek()[1] != close:
                items.append(self.expr())
                if self.peek()[1] == ",":
                    self.take()
            self.take(close)
            return Cons(items)
        if kind == "name":
            self.take()
            x = Name(v)
            if self.peek()[1] == "(":
                x = Ref(v, self.arglist())
            while self.peek()[1] == "%":
                self.take()
                comp = self.take()[1]
                x = Comp(x, comp)
                if self.peek()[1] == "(":
                    x = Comp(x, "(" + repr(self.arglist()) + ")")   # rejected if translated
            return x
        raise FortranError(f"unexpected token {v!r}")

    def arglist(self):
        self.take("(")
        args = []
        if self.peek()[1] == ")":
            self.take()
            return args
        while True:
            args.append(self.arg())
            if self.peek()[1] == ",":
                self.take()
                continue
            self.take(")")
            return args

    def arg(self):
        if self.peek()[0] == "name" and self.peek(1)[1] == "=":
            name = self.take()[1]
            self.take("=")
            return Kw(name, self.expr())
        lo = hi = step = None
        if self.peek()[1] != ":":
            lo = self.expr()
            if self.peek()[1] != ":":
                return lo
        self.take(":")
        if self.peek()[1] not in (",", ")", ":"):
            hi = self.expr()
        if self.peek()[1] == ":":
            self.take()
            step = self.expr()
        return Range(lo, hi, step)


@dataclass
class IDo:
    """Implied-DO list of an I/O statement: (items, var = lo, hi[, step])."""
    items: list
    var: str
    lo: object
    hi: object
    step: object


def io_items(text: str) -> list:
    out = []
    for part in _split_top(text):
        if not part:
            continue
        if part.startswith("(") and _match_paren(part, 0) == len(part) - 1:
            inner = _split_top(part[1:-1])
            k = next((i for i, q in enumerate(inner) if re.match(r"^\w+\s*=(?!=)", q)), None)
            if k is not None:
                var, lo = inner[k].split("=", 1)
                rest = inner[k + 1:]
                out.append(IDo(io_items(",".join(inner[:k])), var.strip().lower(), px(lo), px(rest[0]),
                               px(rest[1]) if len(rest) > 1 else None))
                continue
        out.append(px(part))
    return out


@dataclass
class BadExpr:
    msg: str


def px(s: str):
    """parse_expr, deferring a failure to code generation (the statement's
    procedure is then left untranslated, the rest of the file is not)."""
    try:
        return parse_expr(s)
    except FortranError as e:
        return BadExpr(str(e))


def parse_expr(s: str):
    p = Parser(tokenize(s))
    x = p.expr()
    if not p.at_end():
        raise FortranError(f"trailing tokens in {s!r}")
    return x


# ---------------------------------------------------------------------------
# Statements and program units


@dataclass
class Sym:
    name: str
    typ: str                    # int | real | logical | char | type:<name>
    dims: list | None = None    # [(lo_expr, hi_expr)] or [None]*rank (deferred / assumed)
    intent: str | None = None
    param: object = None        # parameter value expression
    init: object = None
    is_arg: bool = False
    allocatable: bool = False
    clen: object = None         # CHARACTER length (int), None when assumed or not character

    @property
    def rank(self):
        return len(self.dims) if self.dims else 0


@dataclass
class Unit:
    kind: str                   # subroutine | function | module
    name: str
    args: list
    result: str | None = None
    rtype: str | None = None
    syms: dict = field(default_factory=dict)
    uses: list = field(default_factory=list)   # (module, only-list or None)
    body: list = field(default_factory=list)
    contains: list = field(default_factory=list)
    host: "Unit | None" = None
    types: dict = field(default_factory=dict)  # derived type -> {component: typ}
    bad: str | None = None                     # why the unit cannot be translated
    implicit_none: bool = False


@dataclass
class St:
    kind: str
    line: int
    label: int | None = None
    a: object = None
    b: object = None
    c: object = None
    d: object = None
    body: list = None
    orelse: list = None


_TYPE_RE = re.compile(r"^(integer|real\s*\*\s*8|real\s*\(\s*(?:kind\s*=\s*)?8\s*\)|real|double\s*precision|"
                      r"logical|character(?:\s*\*\s*\d+|\s*\([^)]*\))?|type\s*\(\s*\w+\s*\))", re.I)


def _base_type(spec: str) -> str:
    s = re.sub(r"\s+", "", spec.lower())
    if s.startswith("integer"):
        return "int"
    if s.startswith("real") or s.startswith("doubleprecision"):
        return "real"
    if s.startswith("logical"):
        return "logical"
    if s.startswith("character"):
        return "char"
    m = re.match(r"type\((\w+)\)", s)
    return "type:" + m.group(1)


def _split_top(s: str, sep=","):
    parts, depth, q, cur = [], 0, None, ""
    for ch in s:
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        elif ch == sep and depth == 0:
            parts.append(cur)
            cur = ""
            continue
        cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def _match_paren(s: str, i: int) -> int:
    depth, q = 0, None
    for j in range(i, len(s)):
        ch = s[j]
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
            if depth == 0:
                return j
    raise FortranError(f"unbalanced parentheses: {s}")


def _dims(spec: str):
    out = []
    for d in _split_top(spec):
        if d in (":", "*"):
            out.append(None)
        elif ":" in d and not d.startswith("("):
            lo, hi = d.split(":", 1)
            out.append((parse_expr(lo), parse_expr(hi) if hi.strip() not in ("", "*") else None))
        else:
            out.append((Num("1", "int"), parse_expr(d)))
    return out


def parse_decl(stmt: str, unit: Unit):
    m = _TYPE_RE.match(stmt)
    typ = _base_type(m.group(1))
    clen = None
    if typ == "char":
        ml = re.match(r"character\s*(?:\*\s*(\d+)|\(\s*(?:len\s*=\s*)?(\d+)\s*\))", m.group(1), re.I)
        if ml:
            clen = int(ml.group(1) or ml.group(2))
    rest = stmt[m.end():].strip()
    if "::" in rest:
        attrs_s, ents_s = rest.split("::", 1)
        attrs = [a for a in _split_top(attrs_s.lstrip(",")) if a]
    else:
        attrs, ents_s = [], rest
    dims, intent, param, alloc = None, None, False, False
    for a in attrs:
        al = a.lower().replace(" ", "")
        if al.startswith("dimension"):
            dims = _dims(a[a.index("(") + 1:a.rindex(")")])
        elif al.startswith("intent"):
            intent = al[al.index("(") + 1:al.index(")")]
        elif al == "parameter":
            param = True
        elif al == "allocatable":
            alloc = True
        elif al in ("save", "target", "optional", "private", "public", "pointer"):
            pass
        else:
            raise FortranError(f"unsupported attribute {a}")
    for ent in _split_top(ents_s):
        if not ent:
            continue
        init = None
        if "=" in ent and "==" not in ent:
            ent, init_s = ent.split("=", 1)
            init = parse_expr(init_s)
        ent = ent.strip()
        edims, elen = dims, clen
        ml = re.match(r"(\w+)\s*\*\s*(\d+)$", ent)
        if ml and typ == "char":
            ent, elen = ml.group(1), int(ml.group(2))
        mm = re.match(r"(\w+)\s*\((.*)\)$", ent)
        if mm:
            ent, edims = mm.group(1), _dims(mm.group(2))
        name = ent.lower()
        sym = unit.syms.get(name) or Sym(name, typ)
        sym.typ, sym.dims, sym.intent, sym.allocatable, sym.clen = typ, edims, intent, alloc, elen
        if param:
            sym.param = init
        else:
            sym.init = init
        unit.syms[name] = sym


_END_RE = re.compile(r"^end\s*(subroutine|function|module|program|do|if|type|interface|select)?\b\s*(\w*)$", re.I)


def parse_source(text: str, defines: set[str]) -> list[Unit]:
    """Parse the program units of one file (modules' specification parts,
    subroutines and functions with their contained procedures)."""
    lines = logical_lines(preprocess(text, defines))
    units, pos = [], 0

    def parse_unit(pos, host=None):
        no, s = lines[pos]
        sl = s.lower()
        m = re.match(r"^module\s+(\w+)$", sl)
        if m:
            u = Unit("module", m.group(1), [])
        else:
            m = re.match(r"^(?:(?:recursive|pure|elemental)\s+)*(?:(.*?)\s+)?(subroutine|function)\s+(\w+)"
                         r"\s*(?:\((.*?)\))?\s*(?:result\s*\(\s*(\w+)\s*\))?$", sl)
            if not m:
                raise FortranError(f"line {no}: expected a program unit: {s}")
            prefix, kind, name, args, res = m.groups()
            u = Unit(kind, name, [a.strip() for a in (args or "").split(",") if a.strip()], host=host)
            if kind == "function":
                u.result = res or name
                if prefix:
                    u.rtype = _base_type(prefix)
        pos += 1
        pos = parse_spec(u, pos)
        if u.kind != "module":
            u.body, pos = parse_block(pos, ("contains", "end"))
        for a in u.args:
            u.syms.setdefault(a, Sym(a, "?")).is_arg = True
        if u.kind == "function":
            rs = u.syms.setdefault(u.result, Sym(u.result, u.rtype or "?"))
            if rs.typ == "?":
                rs.typ = u.rtype
        no, s = lines[pos]
        if s.lower() == "contains":
            pos += 1
            while not _END_RE.match(lines[pos][1].lower()):
                sub, pos = parse_unit(pos, host=u)
                u.contains.append(sub)
        no, s = lines[pos]
        if not _END_RE.match(s.lower()):
            raise FortranError(f"line {no}: expected end of {u.name}: {s}")
        return u, pos + 1

    def parse_spec(u, pos):
        while pos < len(lines):
            no, s = lines[pos]
            sl = s.lower()
            if sl.startswith("use "):
                m = re.match(r"use\s+(\w+)\s*(?:,\s*only\s*:\s*(.*))?$", sl)
                only = [x.strip() for x in m.group(2).split(",")] if m.group(2) else None
                u.uses.append((m.group(1), only))
            elif sl.startswith("implicit"):
                if re.sub(r"\s+", " ", sl) == "implicit none":
                    u.implicit_none = True
                else:
                    u.bad = u.bad or f"line {no}: IMPLICIT with type rules"
            elif re.match(r"^interface\b", sl):
                while not re.match(r"^end\s*interface", lines[pos][1].lower()):
                    pos += 1
            elif re.match(r"^type\s*(,|::|\s+\w+$)", sl) and not sl.startswith("type("):
                tname = re.findall(r"\w+", sl)[-1]
                comps = Unit("type", tname, [])
                pos += 1
                while not re.match(r"^end\s*type", lines[pos][1].lower()):
                    parse_decl(lines[pos][1], comps)
                    pos += 1
                u.types[tname] = {k: v.typ for k, v in comps.syms.items()}
            elif _TYPE_RE.match(sl) and not re.match(r"^(real|integer|double\s*precision|logical)"
                                                     r"(\s*\*\s*8)?\s+function\b", sl):
                try:
                    parse_decl(s, u)
                except FortranError as e:
                    u.bad = u.bad or f"line {no}: {e}"
            elif sl.startswith("private") or sl.startswith("public") or sl.startswith("save"):
                pass
            else:
                return pos
            pos += 1
        return pos

    def is_stop(head, stops):
        if "enddo" in stops and re.match(r"^end ?do( \w+)?$", head):
            return True
        if "endif" in stops and re.match(r"^end ?if( \w+)?$", head):
            return True
        if "else" in stops and re.match(r"^(else\b|elseif\b)", head):
            return True
        if "contains" in stops and head == "contains":
            return True
        if "end" in stops:
            m = _END_RE.match(head)
            if m and m.group(1) not in ("do", "if", "select", "type", "interface"):
                return True
        return False

    def parse_block(pos, stops, end_label=None):
        body = []
        while pos < len(lines):
            no, s = lines[pos]
            label = None
            m = re.match(r"^(\d+)\s+(.*)$", s)
            if m:
                label, s = int(m.group(1)), m.group(2)
            sl = s.lower()
            head = re.sub(r"\s+", " ", sl)
            if is_stop(head, stops):
                if label is not None:
                    if not re.match(r"^end ?do( \w+)?$", head):
                        raise FortranError(f"line {no}: labelled block end")
                    body.append(St("continue", no, label))   # a labelled END DO ends the iteration
                return body, pos
            st, pos = parse_stmt(pos, no, s, sl, label)
            if st is not None:
                body.append(st)
            if end_label is not None and label == end_label:
                return body, pos
        raise FortranError("unexpected end of file")

    def parse_stmt(pos, no, s, sl, label):
        m = re.match(r"^(\w+)\s*:\s*(?=(do|if|select)\b)", sl)
        if m:                                   # construct name: only plain CYCLE/EXIT are supported
            s, sl = s[m.end():], sl[m.end():]
        if re.match(r"^if\s*\(", sl):
            j = _match_paren(s, s.index("("))
            cond = px(s[s.index("(") + 1:j])
            tail = s[j + 1:].strip()
            if tail.lower() == "then":
                st = St("if", no, label, a=[(cond, None)])
                blk, pos = parse_block(pos + 1, ("else", "endif"))
                st.a[0] = (cond, blk)
                while True:
                    n2, s2 = lines[pos]
                    h = re.sub(r"\s+", " ", s2.lower())
                    mm = re.match(r"^else ?if\s*\(", h)
                    if mm:
                        k = s2.index("(")
                        jj = _match_paren(s2, k)
                        c2 = px(s2[k + 1:jj])
                        blk, pos = parse_block(pos + 1, ("else", "endif"))
                        st.a.append((c2, blk))
                        continue
                    if h == "else":
                        st.orelse, pos = parse_block(pos + 1, ("endif",))
                        continue
                    if re.match(r"^end ?if( \w+)?$", h):
                        return st, pos + 1
                    raise FortranError(f"line {n2}: unexpected {s2}")
            inner, _ = parse_stmt(pos, no, tail, tail.lower(), None)
            return St("if", no, label, a=[(cond, [inner])]), pos + 1
        m = re.match(r"^do\s+(\d+)\s*,?\s*(\w+)\s*=\s*(.*)$", sl)
        if m:                                   # DO with a terminal label (the labelled statement ends the body)
            parts = _split_top(s[s.index("=") + 1:])
            start, end = px(parts[0]), px(parts[1])
            step = px(parts[2]) if len(parts) > 2 else None
            body, pos = parse_block(pos + 1, (), end_label=int(m.group(1)))
            return St("do", no, label, a=m.group(2), b=start, c=end, d=step, body=body), pos
        m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", sl)
        if m:
            parts = _split_top(s[s.index("=") + 1:])
            start, end = px(parts[0]), px(parts[1])
            step = px(parts[2]) if len(parts) > 2 else None
            body, pos = parse_block(pos + 1, ("enddo",))
            return St("do", no, label, a=m.group(1), b=start, c=end, d=step, body=body), pos + 1
        m = re.match(r"^do\s+while\s*\((.*)\)$", sl)
        if m:
            k = s.index("(")
            cond = px(s[k + 1:_match_paren(s, k)])
            body, pos = parse_block(pos + 1, ("enddo",))
            return St("dowhile", no, label, a=cond, body=body), pos + 1
        if sl == "do":
            body, pos = parse_block(pos + 1, ("enddo",))
            return St("dowhile", no, label, a=Lit(True), body=body), pos + 1
        m = re.match(r"^go\s*to\s+(\d+)$", sl)
        if m:
            return St("goto", no, label, a=int(m.group(1))), pos + 1
        if sl in ("cycle", "exit", "return", "continue"):
            return St(sl, no, label), pos + 1
        if re.match(r"^(cycle|exit)\s+\w+$", sl):
            raise FortranError(f"line {no}: CYCLE/EXIT with a construct name")
        if sl.startswith("stop"):
            return St("stop", no, label, a=s[4:].strip()), pos + 1
        m = re.match(r"^(read|write|open|close)\s*\(", sl)
        if m:
            k = s.index("(")
            j = _match_paren(s, k)
            pos_args, kw = [], {}
            for c in _split_top(s[k + 1:j]):
                mk = re.match(r"^(\w+)\s*=(?!=)\s*(.*)$", c)
                if mk:
                    kw[mk.group(1).lower()] = mk.group(2).strip()
                else:
                    pos_args.append(c.strip())
            unit = pos_args[0] if pos_args else kw.get("unit")
            fmt = pos_args[1] if len(pos_args) > 1 else kw.get("fmt")
            kind = m.group(1)
            if kind == "open" and unit is None and "newunit" in kw:
                ctl = {"unit": None, "newunit": px(kw["newunit"])}
                for key in ("file", "status", "form", "iostat"):
                    if key in kw:
                        ctl[key] = px(kw[key])
                for key in ("err",):
                    if key in kw:
                        ctl[key] = int(kw[key])
                return St("open", no, label, a=ctl, b=[]), pos + 1
            if unit is None:
                return St("bad", no, label, a=f"line {no}: {kind} without a unit"), pos + 1
            if kind == "write" and (unit in ("6", "*") or fmt is not None):
                return St("noop", no, label), pos + 1            # formatted output: not reproduced
            if kind in ("read", "write") and (unit == "*" or fmt is not None):
                return St("bad", no, label, a=f"line {no}: formatted {kind}"), pos + 1
            ctl = {"unit": px(unit)}
            for key in ("file", "status", "form", "iostat"):
                if key in kw:
                    ctl[key] = px(kw[key])
            for key in ("err", "end"):
                if key in kw:
                    if not kw[key].isdigit():
                        return St("bad", no, label, a=f"line {no}: {key}= {kw[key]}"), pos + 1
                    ctl[key] = int(kw[key])
            try:
                items = io_items(s[j + 1:].strip()) if kind in ("read", "write") else []
            except FortranError as e:
                return St("bad", no, label, a=f"line {no}: {e}"), pos + 1
            return St(kind, no, label, a=ctl, b=items), pos + 1
        if re.match(r"^(print|format|call\s+flush)\b", sl) or re.match(r"^format\s*\(", sl):
            return St("noop", no, label), pos + 1
        m = re.match(r"^call\s+(\w+)\s*(\(.*\))?$", sl)
        if m:
            try:
                args = Parser(tokenize(s[s.lower().index(m.group(1)) + len(m.group(1)):])).arglist() \
                    if m.group(2) else []
            except FortranError as e:
                return St("bad", no, label, a=f"line {no}: {e}"), pos + 1
            return St("call", no, label, a=m.group(1), b=args), pos + 1
        m = re.match(r"^(allocate|deallocate)\s*\((.*)\)$", sl)
        if m:
            items = [px(x) for x in _split_top(s[s.index("(") + 1:s.rindex(")")])]
            return St(m.group(1), no, label, a=items), pos + 1
        # assignment: the first top-level '=' that is not part of a relational operator
        depth, q = 0, None
        for k, ch in enumerate(s):
            if q:
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
            elif ch in "([":
                depth += 1
            elif ch in ")]":
                depth -= 1
            elif ch == "=" and depth == 0 and s[k - 1] not in "<>/=" and (k + 1 >= len(s) or s[k + 1] not in "=>"):
                return St("assign", no, label, a=px(s[:k]), b=px(s[k + 1:])), pos + 1
        return St("bad", no, label, a=f"line {no}: unsupported statement: {s}"), pos + 1

    while pos < len(lines):
        u, pos = parse_unit(pos)
        units.append(u)
    return units


# ---------------------------------------------------------------------------
# Code generation

INTRINSIC_TYPES = {
    "abs": "arg", "dabs": "real", "iabs": "int", "sqrt": "real", "dsqrt": "real", "exp": "real", "dexp": "real",
    "log": "real", "dlog": "real", "sin": "real", "cos": "real", "tanh": "real", "atan": "real",
    "dfloat": "real", "dble": "real", "real": "real", "float": "real", "int": "int", "nint": "int",
    "floor": "int", "ceiling": "int", "max": "arg", "min": "arg", "dmax1": "real", "dmin1": "real",
    "max0": "int", "min0": "int", "mod": "arg", "sign": "arg", "isnan": "logical", "minval": "arg",
    "maxval": "arg", "ubound": "int", "lbound": "int", "size": "int", "omp_get_num_threads": "int",
    "omp_get_thread_num": "int", "omp_get_max_threads": "int", "huge": "arg", "sum": "arg", "maxloc": "int",
    "minloc": "int", "len": "int", "len_trim": "int", "trim": "char", "index": "int",
}


class Gen:
    """Python source for the translated procedures of one program."""

    def __init__(self, procs: dict, modules: dict, undefined: dict | None = None):
        self.procs = procs          # name -> Unit (top-level subroutines/functions)
        self.modules = modules      # name -> Unit (module specification parts)
        self.undefined = undefined or {}   # (procedure, local) -> stand-in for a read of an undefined value

    # -- name resolution
    def visible(self, u: Unit):
        """name -> (scope, Sym, owner) for every name visible in unit u."""
        vis = {}
        chain = []
        x = u
        while x is not None:
            chain.append(x)
            x = x.host
        for x in reversed(chain):
            for mod, only in x.uses:
                mu = self.modules.get(mod)
                if mu is None:
                    continue
                names = only if only is not None else list(mu.syms)
                for n in names:
                    n = n.split("=>")[-1].strip()
                    if n in mu.syms:
                        vis[n] = ("module", mu.syms[n], mod)
            for n, sym in x.syms.items():
                if x.kind == "module":
                    vis[n] = ("module", sym, x.name)
                elif sym.init is not None and not sym.is_arg and sym.param is None and not sym.rank:
                    vis[n] = ("saved", sym, x.name)      # an initialiser implies SAVE
                else:
                    vis[n] = ("local" if x is u else "host", sym, x.name)
        return vis

    def types_of(self, u):
        t = {}
        for mu in self.modules.values():
            t.update(mu.types)
        x = u
        while x is not None:
            t.update(x.types)
            x = x.host
        return t

    def py(self, name, scope, owner):
        if scope == "module":
            return f"m_{owner}.f_{name}"
        if scope == "saved":
            return f"s_{owner}.f_{name}"
        return "f_" + name

    # -- expressions: return (code, type, rank)
    def ex(self, e, ctx):
        if isinstance(e, Num):
            if e.typ == "int":
                return str(int(e.text)), "int", 0
            return repr(float(e.text.replace("d", "e"))), "real", 0
        if isinstance(e, Str):
            return repr(e.s), "char", 0
        if isinstance(e, Lit):
            return repr(e.v), "logical", 0
        if isinstance(e, Name):
            v = ctx.vis.get(e.name)
            if v is None:
                if e.name in ctx.contained or e.name in self.procs:
                    raise FortranError(f"procedure {e.name} used as a value")
                raise FortranError(f"undeclared name {e.name} in {ctx.unit.name}")
            scope, sym, owner = v
            if sym.param is not None:
                c, t, r = self.ex(sym.param, ctx)
                return f"({c})", sym.typ, 0
            code = self.py(e.name, scope, owner)
            if sym.rank:
                return f"_whole({code})", sym.typ, sym.rank
            return code, sym.typ, 0
        if isinstance(e, Comp):
            bc, bt, br = self.ex(e.base, ctx)
            if not bt.startswith("type:"):
                raise FortranError("component of a non-derived value")
            comps = self.types_of(ctx.unit).get(bt[5:])
            if comps is None or e.comp not in comps:
                raise FortranError(f"unknown component {e.comp} of {bt}")
            if br:
                return f"_ew(lambda o: o.f_{e.comp}, {bc})", comps[e.comp], br
            return f"{bc}.f_{e.comp}", comps[e.comp], 0
        if isinstance(e, Ref):
            return self.ref(e, ctx)
        if isinstance(e, Un):
            c, t, r = self.ex(e.x, ctx)
            if e.op == "not":
                return (f"_ew(lambda a: not a, {c})" if r else f"(not {c})"), "logical", r
            return (f"_ew(lambda a: -a, {c})" if r else f"(-{c})"), t, r
        if isinstance(e, Bin):
            return self.binop(e, ctx)
        if isinstance(e, BadExpr):
            raise FortranError(e.msg)
        if isinstance(e, Cons):
            items = [self.ex(x, ctx) for x in e.items]
            t = "real" if any(i[1] == "real" for i in items) else items[0][1]
            return f"_cons({', '.join(self.conv(c, it, t) for c, it, _ in items)})", t, 1
        raise FortranError(f"unsupported expression {e}")

    def conv(self, code, have, want):
        if have == want or want in ("?", None):
            return code
        if want == "real" and have == "int":
            return f"float({code})"
        if want == "int" and have == "real":
            return f"int({code})"
        return code

    def binop(self, e, ctx):
        lc, lt, lr = self.ex(e.l, ctx)
        if e.op == "**" and isinstance(e.r, Num) and e.r.typ == "int" and 1 <= int(e.r.text) <= 3:
            n = int(e.r.text)
            if lr:
                return f"_ew(lambda a: {' * '.join(['a'] * n)}, {lc})", lt, lr
            return "(" + " * ".join([f"({lc})"] * n) + ")", lt, 0
        rc, rt, rr = self.ex(e.r, ctx)
        rank = max(lr, rr)
        if e.op in ("and", "or"):
            if rank:
                return f"_ew(lambda a, b: a {e.op} b, {lc}, {rc})", "logical", rank
            return f"({lc} {e.op} {rc})", "logical", 0
        if e.op == "//":
            if rank or lt != "char" or rt != "char":
                raise FortranError("concatenation of non-character operands")
            return f"({lc} + {rc})", "char", 0
        if e.op in ("==", "!=", "<", "<=", ">", ">=") and "char" in (lt, rt):
            if rank:
                raise FortranError("character array comparison")
            return f"(_strcmp({lc}, {rc}) {e.op} 0)", "logical", 0
        if e.op in ("==", "!=", "<", "<=", ">", ">="):
            if rank:
                return f"_ew(lambda a, b: a {e.op} b, {lc}, {rc})", "logical", rank
            return f"({lc} {e.op} {rc})", "logical", 0
        t = "real" if "real" in (lt, rt) else "int"
        a = lc if lr else self.conv(lc, lt, t)
        b = rc if rr else self.conv(rc, rt, t)
        if e.op == "/" and t == "int":
            f = "_idiv({0}, {1})"
        elif e.op == "**":
            if t == "int":
                f = "({0} ** {1})"
            elif rt == "int":
                f = "_rpowi({0}, {1})"
                b = rc                          # the integer exponent stays an integer
            else:
                f = "math.pow({0}, {1})"
        else:
            f = "({0} " + e.op + " {1})"
        if rank:
            return f"_ew(lambda a, b: {f.format('a', 'b')}, {a}, {b})", t, rank
        return f.format(a, b), t, 0

    def ref(self, e, ctx):
        v = ctx.vis.get(e.name)
        if v is not None and v[1].rank:
            scope, sym, owner = v
            arr = self.py(e.name, scope, owner)
            if any(isinstance(a, Range) for a in e.args):
                specs = []
                for a in e.args:
                    if isinstance(a, Range):
                        specs.append("(" + ", ".join(self.ex(x, ctx)[0] if x is not None else "None"
                                                      for x in (a.lo, a.hi, a.step)) + ")")
                    else:
                        specs.append(self.ex(a, ctx)[0])
                rank = sum(isinstance(a, Range) for a in e.args)
                return f"_sec({arr}, ({', '.join(specs)},))", sym.typ, rank
            subs = [self.ex(a, ctx) for a in e.args]
            if any(r for _, _, r in subs):
                raise FortranError("vector subscripts are not supported")
            if any(t != "int" for _, t, _ in subs):
                raise FortranError(f"non-integer subscript of {e.name}")
            if len(subs) in (1, 2):
                return f"{arr}.g{len(subs)}({', '.join(c for c, _, _ in subs)})", sym.typ, 0
            return f"{arr}[{', '.join(c for c, _, _ in subs)},]", sym.typ, 0
        if v is not None and v[1].typ == "char":
            if len(e.args) != 1 or not isinstance(e.args[0], Range) or e.args[0].step is not None:
                raise FortranError(f"reference {e.name}(...) of a character scalar")
            scope, sym, owner = v
            lo = self.ex(e.args[0].lo, ctx)[0] if e.args[0].lo is not None else "None"
            hi = self.ex(e.args[0].hi, ctx)[0] if e.args[0].hi is not None else "None"
            return f"_substr({self.py(e.name, scope, owner)}, {lo}, {hi})", "char", 0
        return self.call(e.name, e.args, ctx, as_function=True)

    def intrinsic(self, name, args, ctx):
        kw = {a.name: a.value for a in args if isinstance(a, Kw)}
        pos = [a for a in args if not isinstance(a, Kw)]
        vals = [self.ex(a, ctx) for a in pos]
        anyr = any(r for _, _, r in vals)
        t0 = vals[0][1] if vals else "int"
        if name in ("abs", "dabs", "iabs"):
            return (f"_ew(abs, {vals[0][0]})" if anyr else f"abs({vals[0][0]})"), t0 if name == "abs" else \
                ("real" if name == "dabs" else "int"), vals[0][2]
        if name in ("sqrt", "dsqrt", "exp", "dexp", "log", "dlog", "sin", "cos", "tanh", "atan"):
            fn = {"dsqrt": "sqrt", "dexp": "exp", "dlog": "log"}.get(name, name)
            return f"math.{fn}({self.conv(vals[0][0], t0, 'real')})", "real", 0
        if name in ("dfloat", "dble", "real", "float"):
            return f"float({vals[0][0]})", "real", 0
        if name == "int":
            return f"int({vals[0][0]})", "int", 0
        if name == "nint":
            return f"_nint({vals[0][0]})", "int", 0
        if name in ("max", "min", "dmax1", "dmin1", "max0", "min0"):
            t = "real" if any(v[1] == "real" for v in vals) else "int"
            f = "_fmax" if "max" in name else "_fmin"
            if anyr:
                raise FortranError("elemental max/min over arrays is not supported")
            return f"{f}({', '.join(self.conv(c, tt, t) for c, tt, _ in vals)})", t, 0
        if name == "mod":
            t = "real" if any(v[1] == "real" for v in vals) else "int"
            if t == "int":
                return f"_imod({vals[0][0]}, {vals[1][0]})", "int", 0
            return f"math.fmod({self.conv(vals[0][0], vals[0][1], 'real')}, " \
                   f"{self.conv(vals[1][0], vals[1][1], 'real')})", "real", 0
        if name == "sign":
            if t0 == "int":
                return f"_isign({vals[0][0]}, {vals[1][0]})", "int", 0
            return f"math.copysign(abs({vals[0][0]}), {vals[1][0]})", "real", 0
        if name == "isnan":
            return f"math.isnan({vals[0][0]})", "logical", 0
        if name in ("minval", "maxval"):
            mask = kw.get("mask", pos[1] if len(pos) > 1 else None)
            mc = self.ex(mask, ctx)[0] if mask is not None else "None"
            return f"_{name}({vals[0][0]}, {mc}, {t0!r})", t0, 0
        if name in ("ubound", "lbound", "size"):
            a = pos[0]
            if not isinstance(a, Name):
                raise FortranError(f"{name} of an expression")
            scope, sym, owner = ctx.vis[a.name]
            dim = kw.get("dim", pos[1] if len(pos) > 1 else None)
            dc = self.ex(dim, ctx)[0] if dim is not None else "None"
            return f"_{name}({self.py(a.name, scope, owner)}, {dc})", "int", 0 if dim is not None or name == "size" else 1
        if name == "len":
            return f"len({vals[0][0]})", "int", 0
        if name == "len_trim":
            return f"len({vals[0][0]}.rstrip(' '))", "int", 0
        if name == "trim":
            return f"{vals[0][0]}.rstrip(' ')", "char", 0
        if name == "index":
            return f"({vals[0][0]}.find({vals[1][0]}) + 1)", "int", 0
        if name == "sum":
            if len(pos) > 1 or kw:
                raise FortranError("SUM with DIM or MASK is not supported")
            return f"_sum({vals[0][0]}, {t0!r})", t0, 0
        if name in ("maxloc", "minloc"):
            dim = kw.get("dim", pos[1] if len(pos) > 1 else None)
            if dim is None or vals[0][2] != 1 or not (isinstance(dim, Num) and dim.text == "1"):
                raise FortranError(f"{name} is supported as {name}(rank-1 array, 1) only")
            return f"_{name}1({vals[0][0]})", "int", 0
        if name in ("omp_get_num_threads", "omp_get_max_threads"):
            return "1", "int", 0
        if name == "omp_get_thread_num":
            return "0", "int", 0
        raise FortranError(f"intrinsic {name} not supported")

    def find_proc(self, name, ctx):
        if name in ctx.contained:
            return ctx.contained[name]
        if name in self.procs:
            return self.procs[name]
        return None

    def call(self, name, args, ctx, as_function):
        callee = self.find_proc(name, ctx)
        if callee is None:
            if name in INTRINSIC_TYPES:
                return self.intrinsic(name, args, ctx)
            raise FortranError(f"unknown procedure {name} in {ctx.unit.name}")
        actuals = []
        copy_back = []
        for k, (a, dn) in enumerate(zip(args, callee.args)):
            ds = callee.syms[dn]
            if ds.rank:
                if isinstance(a, Name):
                    scope, sym, owner = ctx.vis[a.name]
                    actuals.append(self.py(a.name, scope, owner))
                elif isinstance(a, Ref) and not any(isinstance(x, Range) for x in a.args):
                    scope, sym, owner = ctx.vis[a.name]
                    subs = ", ".join(self.ex(x, ctx)[0] for x in a.args)
                    actuals.append(f"{self.py(a.name, scope, owner)}.view_at(({subs},))")
                elif isinstance(a, Ref) and len(a.args) == 1 and isinstance(a.args[0], Range) \
                        and a.args[0].step is None and a.args[0].lo is not None and a.args[0].hi is not None:
                    scope, sym, owner = ctx.vis[a.name]    # contiguous section: its own elements only
                    lo, hi = self.ex(a.args[0].lo, ctx)[0], self.ex(a.args[0].hi, ctx)[0]
                    actuals.append(f"{self.py(a.name, scope, owner)}.section_view({lo}, {hi})")
                else:
                    c, t, r = self.ex(a, ctx)
                    if not r:
                        raise FortranError(f"array argument form not supported: {a}")
                    actuals.append(f"_temp_array({c}, {ds.typ!r})")   # an expression: copy in only
            else:
                c, t, r = self.ex(a, ctx)
                actuals.append(self.conv(c, t, ds.typ))
                if ds.intent != "in" and isinstance(a, (Name, Ref, Comp)) and not (
                        isinstance(a, Name) and ctx.vis.get(a.name, (None, Sym("", "")))[1].param is not None):
                    copy_back.append((k, a, ds))
        if len(args) != len(callee.args):
            raise FortranError(f"call of {name} with {len(args)} of {len(callee.args)} arguments")
        fn = "p_" + name
        call = f"{fn}({', '.join(actuals)})"
        if as_function:
            return call, callee.syms[callee.result].typ, 0
        return call, copy_back

    # -- statements
    def block(self, stmts, ctx, ind, out):
        labels = {s.label for s in stmts if s.label is not None and s.label in ctx.targets}
        if not labels:
            for s in stmts:
                self.stmt(s, ctx, ind, out)
            if not stmts:
                out.append("    " * ind + "pass")
            return
        segs, cur = [], []
        seg_labels = {}
        for s in stmts:
            if s.label in labels:
                segs.append(cur)
                seg_labels[s.label] = len(segs)
                cur = []
            cur.append(s)
        segs.append(cur)
        p = "    " * ind
        pc = f"_pc{ctx.fresh()}"
        out.append(p + f"{pc} = 0")
        out.append(p + "while True:")
        out.append(p + "    try:")
        ctx.dispatch += 1
        for k, seg in enumerate(segs):
            out.append(p + f"        if {pc} <= {k}:")
            if seg:
                for s in seg:
                    self.stmt(s, ctx, ind + 3, out)
            else:
                out.append(p + "            pass")
        ctx.dispatch -= 1
        out.append(p + "        break")
        out.append(p + "    except _Goto as _g:")
        out.append(p + f"        _tab = {seg_labels!r}")
        out.append(p + "        if _g.label not in _tab:")
        out.append(p + "            raise")
        out.append(p + f"        {pc} = _tab[_g.label]")

    _IOKIND = {"int": "int", "real": "real", "logical": "logical", "char": "char"}

    def io(self, s, ctx, ind, out):
        p = "    " * ind
        c = s.a
        body = []
        if c.get("unit") is None:                # OPEN(NEWUNIT=v): a fresh unit number, stored in v
            lv, lt, helper = self.target(c["newunit"], ctx)
            body.append(helper.format("_io.newunit()") if helper else f"{lv} = _io.newunit()")
            unit = self.ex(c["newunit"], ctx)[0]
        else:
            unit = self.ex(c["unit"], ctx)[0]
        if s.kind == "open":
            f = lambda key, dflt: self.ex(c[key], ctx)[0] if key in c else repr(dflt)  # noqa: E731
            body.append(f"_io.open({unit}, {f('file', '')}, {f('status', 'unknown')}, {f('form', 'formatted')})")
        elif s.kind == "close":
            body.append(f"_io.close({unit})")
        elif s.kind == "read":
            body.append(f"_rec = _io.read({unit})")
            for it in s.b:
                self.io_read(it, ctx, 0, body)
        else:
            body.append("_w = _RecordOut()")
            for it in s.b:
                self.io_write(it, ctx, 0, body)
            body.append(f"_io.write({unit}, _w.data())")
        handled = any(key in c for key in ("iostat", "err", "end"))
        if not handled:
            out.extend(p + line for line in body)
            return
        out.append(p + "try:")
        out.extend(p + "    " + line for line in body)
        if "iostat" in c:
            lv, lt, helper = self.target(c["iostat"], ctx)
            out.append(p + "    " + (helper.format("0") if helper else f"{lv} = 0"))
        out.append(p + "except _IOError as _e:")
        if "iostat" in c:
            out.append(p + "    " + (helper.format("_e.code") if helper else f"{lv} = _e.code"))
        if "end" in c:
            out.append(p + f"    if _e.code < 0: raise _Goto({c['end']})")
        if "err" in c:
            out.append(p + f"    if _e.code > 0: raise _Goto({c['err']})")
        if "iostat" not in c:
            rest = [k for k in ("end", "err") if k not in c]
            if rest:
                out.append(p + "    raise")

    def io_loop(self, it, ctx, ind, out, each):
        scope, sym, owner = ctx.vis[it.var]
        vc = self.py(it.var, scope, owner)
        if scope == "host":
            ctx.nonlocal_.add(vc)
        p = "    " * ind
        n = ctx.fresh()
        a, b = self.ex(it.lo, ctx)[0], self.ex(it.hi, ctx)[0]
        st = self.ex(it.step, ctx)[0] if it.step is not None else "1"
        out.append(p + f"_a{n}, _s{n} = {a}, {st}")
        out.append(p + f"_t{n} = max(0, _idiv({b} - _a{n} + _s{n}, _s{n}))")
        out.append(p + f"for {vc} in range(_a{n}, _a{n} + _t{n} * _s{n}, _s{n}):")
        for x in it.items:
            each(x, ctx, ind + 1, out)
        out.append(p + "else:")
        out.append(p + f"    {vc} = _a{n} + _t{n} * _s{n}")

    def io_read(self, it, ctx, ind, out):
        p = "    " * ind
        if isinstance(it, IDo):
            return self.io_loop(it, ctx, ind, out, self.io_read)
        if isinstance(it, (Name, Ref)) and it.name in ctx.vis and ctx.vis[it.name][1].rank and (
                isinstance(it, Name) or any(isinstance(a, Range) for a in it.args)):
            scope, sym, owner = ctx.vis[it.name]
            arr = self.py(it.name, scope, owner)
            specs = "None"
            if isinstance(it, Ref):
                c, _, _ = self.ref(it, ctx)
                specs = c[len(f"_sec({arr}, "):-1]
            out.append(p + f"_read_into({arr}, {specs}, _rec, {self._IOKIND[sym.typ]!r}, {sym.clen!r})")
            return
        lv, lt, helper = self.target(it, ctx)
        v = f"_rec.char({self.char_len(it, ctx)!r})" if lt == "char" else f"_rec.{self._IOKIND[lt]}()"
        out.append(p + (helper.format(v) if helper else f"{lv} = {v}"))

    def io_write(self, it, ctx, ind, out):
        p = "    " * ind
        if isinstance(it, IDo):
            return self.io_loop(it, ctx, ind, out, self.io_write)
        if isinstance(it, (Name, Ref)) and it.name in ctx.vis and ctx.vis[it.name][1].rank and (
                isinstance(it, Name) or any(isinstance(a, Range) for a in it.args)):
            scope, sym, owner = ctx.vis[it.name]
            arr = self.py(it.name, scope, owner)
            specs = "None"
            if isinstance(it, Ref):
                c, _, _ = self.ref(it, ctx)
                specs = c[len(f"_sec({arr}, "):-1]
            out.append(p + f"_write_from(_w, {arr}, {specs}, {self._IOKIND[sym.typ]!r})")
            return
        c, t, r = self.ex(it, ctx)
        if r:
            raise FortranError("array expression in an output list")
        out.append(p + f"_w.{self._IOKIND[t]}({c})")

    def char_len(self, target, ctx):
        if isinstance(target, Name) and target.name in ctx.vis:
            return ctx.vis[target.name][1].clen
        return None

    def loop_body(self, stmts, ctx, ind, out, n):
        loop = {"n": n, "dispatch": ctx.dispatch, "exc": False}
        ctx.loops.append(loop)
        body = []
        self.block(stmts, ctx, ind + 1, body)
        ctx.loops.pop()
        p = "    " * ind
        if not loop["exc"]:
            out.extend(line[4:] for line in body)
            return
        out.append(p + "try:")
        out.extend(body)
        out.append(p + "except _LoopCtl as _c:")
        out.append(p + f"    if _c.n != {n}:")
        out.append(p + "        raise")
        out.append(p + "    if _c.kind == 'exit':")
        out.append(p + "        break")

    def target(self, t, ctx):
        """(python lvalue or None, type, section assignment helper or None)."""
        if isinstance(t, Name):
            scope, sym, owner = ctx.vis[t.name]
            code = self.py(t.name, scope, owner)
            if sym.rank:
                return None, sym.typ, f"_asgn({code}, None, {{}})"
            if scope == "host":
                ctx.nonlocal_.add("f_" + t.name)
            return code, sym.typ, None
        if isinstance(t, Ref):
            scope, sym, owner = ctx.vis[t.name]
            if not sym.rank:
                raise FortranError(f"subscripted scalar {t.name}")
            arr = self.py(t.name, scope, owner)
            if any(isinstance(a, Range) for a in t.args):
                c, _, _ = self.ref(t, ctx)
                specs = c[len(f"_sec({arr}, "):-1]
                return None, sym.typ, f"_asgn({arr}, {specs}, {{}})"
            subs = ", ".join(self.ex(a, ctx)[0] for a in t.args)
            if len(t.args) in (1, 2):
                return None, sym.typ, f"{arr}.s{len(t.args)}({subs}, {{}})"
            return f"{arr}[{subs},]", sym.typ, None
        if isinstance(t, Comp):
            bc, bt, br = self.ex(t.base, ctx)
            comps = self.types_of(ctx.unit)[bt[5:]]
            if br:
                base = t.base
                if isinstance(base, Name):
                    specs = "None"
                elif isinstance(base, Ref):
                    c, _, _ = self.ref(base, ctx)
                    arr = self.py(base.name, *[ctx.vis[base.name][i] for i in (0, 2)])
                    specs = c[len(f"_sec({arr}, "):-1]
                else:
                    raise FortranError("component assignment through an expression")
                arr = self.py(base.name, *[ctx.vis[base.name][i] for i in (0, 2)])
                return None, comps[t.comp], f"_asgn_comp({arr}, {specs}, 'f_{t.comp}', {{}})"
            return f"{bc}.f_{t.comp}", comps[t.comp], None
        raise FortranError(f"unsupported assignment target {t}")

    def stmt(self, s, ctx, ind, out):
        p = "    " * ind
        k = s.kind
        if k == "assign":
            lv, lt, helper = self.target(s.a, ctx)
            c, t, r = self.ex(s.b, ctx)
            if helper:
                if r:
                    c = f"_ew(lambda v: {self.conv('v', t, lt)}, {c})" if t != lt else c
                else:
                    c = self.conv(c, t, lt)
                out.append(p + helper.format(c))
            else:
                if r:
                    raise FortranError(f"line {s.line}: array value assigned to a scalar")
                if lt == "char":
                    n = self.char_len(s.a, ctx)
                    out.append(p + f"{lv} = _strfix({c}, {n!r})")
                else:
                    out.append(p + f"{lv} = {self.conv(c, t, lt)}")
        elif k == "if":
            for j, (cond, body) in enumerate(s.a):
                c, _, _ = self.ex(cond, ctx)
                out.append(p + ("if " if j == 0 else "elif ") + f"{c}:")
                self.block(body, ctx, ind + 1, out)
            if s.orelse is not None:
                out.append(p + "else:")
                self.block(s.orelse, ctx, ind + 1, out)
        elif k == "do":
            var = s.a
            scope, sym, owner = ctx.vis[var]
            vc = self.py(var, scope, owner)
            if scope == "host":
                ctx.nonlocal_.add(vc)
            a, _, _ = self.ex(s.b, ctx)
            b, _, _ = self.ex(s.c, ctx)
            st = self.ex(s.d, ctx)[0] if s.d is not None else "1"
            n = ctx.fresh()
            out.append(p + f"_a{n}, _s{n} = {a}, {st}")
            out.append(p + f"_t{n} = max(0, _idiv({b} - _a{n} + _s{n}, _s{n}))")
            out.append(p + f"for {vc} in range(_a{n}, _a{n} + _t{n} * _s{n}, _s{n}):")
            self.loop_body(s.body, ctx, ind + 1, out, n)
            out.append(p + "else:")
            out.append(p + f"    {vc} = _a{n} + _t{n} * _s{n}")
        elif k == "dowhile":
            c, _, _ = self.ex(s.a, ctx)
            n = ctx.fresh()
            out.append(p + f"while {c}:")
            self.loop_body(s.body, ctx, ind + 1, out, n)
        elif k in ("cycle", "exit"):
            if not ctx.loops:
                raise FortranError(f"line {s.line}: {k} outside a DO loop")
            loop = ctx.loops[-1]
            if ctx.dispatch > loop["dispatch"]:      # a GOTO dispatcher's loop lies in between
                loop["exc"] = True
                out.append(p + f"raise _LoopCtl({k!r}, {loop['n']})")
            else:
                out.append(p + ("continue" if k == "cycle" else "break"))
        elif k == "goto":
            out.append(p + f"raise _Goto({s.a})")
        elif k in ("continue", "noop"):
            out.append(p + "pass")
        elif k == "return":
            out.append(p + f"return {ctx.ret}")
        elif k == "stop":
            out.append(p + f"raise FortranStop({s.a!r})")
        elif k == "call":
            code, copy_back = self.call(s.a, s.b, ctx, as_function=False)
            if copy_back:
                n = ctx.fresh()
                out.append(p + f"_r{n} = {code}")
                for idx, a, ds in copy_back:
                    lv, lt, helper = self.target(a, ctx)
                    if helper and helper.startswith("_asgn("):
                        raise FortranError("copy-out into an array section")
                    out.append(p + (helper.format(f"_r{n}[{idx}]") if helper else f"{lv} = _r{n}[{idx}]"))
            else:
                out.append(p + code)
        elif k == "allocate":
            for it in s.a:
                if not isinstance(it, Ref):
                    raise FortranError("allocate without bounds")
                scope, sym, owner = ctx.vis[it.name]
                bnds = []
                for a in it.args:
                    if isinstance(a, Range):
                        bnds.append(f"({self.ex(a.lo, ctx)[0]}, {self.ex(a.hi, ctx)[0]})")
                    else:
                        bnds.append(f"(1, {self.ex(a, ctx)[0]})")
                kind = "real" if sym.typ == "real" else sym.typ
                lv = self.py(it.name, scope, owner)
                if scope == "host":
                    ctx.nonlocal_.add(lv)
                if sym.typ.startswith("type:"):
                    comps = sorted(self.types_of(ctx.unit).get(sym.typ[5:], {}))
                    out.append(p + f"{lv} = _new_objs(FArray.new('obj', ({', '.join(bnds)},)), {comps!r})")
                else:
                    out.append(p + f"{lv} = FArray.new({kind!r}, ({', '.join(bnds)},))")
        elif k == "bad":
            raise FortranError(s.a)
        elif k in ("open", "close", "read", "write"):
            self.io(s, ctx, ind, out)
        elif k == "deallocate":
            for it in s.a:
                scope, sym, owner = ctx.vis[it.name]
                out.append(p + f"{self.py(it.name, scope, owner)} = None")
        else:
            raise FortranError(f"statement {k}")

    # -- procedures
    def implicit_typing(self, u: Unit):
        """Without IMPLICIT NONE in the unit or a host, undeclared names take
        INTEGER for I-N and REAL (8 bytes under -r8) otherwise."""
        x = u
        while x is not None:
            if x.implicit_none:
                return
            x = x.host
        typ = lambda n: "int" if n[0] in "ijklmn" else "real"  # noqa: E731
        for a in u.args:
            if u.syms[a].typ == "?":
                u.syms[a].typ = typ(a)
        if u.kind == "function" and u.syms[u.result].typ in ("?", None):
            u.syms[u.result].typ = typ(u.result)
        vis = self.visible(u)
        known = set(vis) | set(self.procs) | {c.name for c in u.contains} | set(INTRINSIC_TYPES)
        for n in sorted(_scalar_names(u.body) - known):
            u.syms[n] = Sym(n, typ(n))

    def unit(self, u: Unit, ind: int, out: list):
        if u.bad:
            raise FortranError(u.bad)
        self.implicit_typing(u)
        ctx = _Ctx(u, self.visible(u))
        ctx.contained = {c.name: c for c in u.contains}
        x = u.host
        while x is not None:
            for c in x.contains:
                ctx.contained.setdefault(c.name, c)
            x = x.host
        ctx.targets = _goto_targets(u.body)
        ctx.top_ind = ind + 1
        p = "    " * ind
        params = [f"f_{a}" for a in u.args]
        out.append(p + f"def p_{u.name}({', '.join(params)}):")
        header_at = len(out)
        q = p + "    "
        scalar_args = [a for a in u.args if not u.syms[a].rank]
        if u.kind == "function":
            ctx.ret = f"f_{u.result}"
        else:
            ctx.ret = "(" + "".join(f"f_{a}, " for a in u.args) + ")" if u.args else "()"
        # dummy arrays: explicit-shape views of the actuals
        for a in u.args:
            sym = u.syms[a]
            if sym.typ == "?":
                raise FortranError(f"undeclared dummy {a} of {u.name}")
            if sym.typ == "char" and not sym.rank and sym.clen is not None:
                out.append(q + f"f_{a} = _strfix(f_{a}, {sym.clen})")
            if sym.rank:
                if any(d is None or d[1] is None for d in sym.dims):
                    if all(d is None for d in sym.dims):
                        continue        # assumed shape: the actual as it is
                    raise FortranError(f"assumed-size dummy {a} of {u.name}")
                bnds = ", ".join(f"({self.ex(lo, ctx)[0]}, {self.ex(hi, ctx)[0]})" for lo, hi in sym.dims)
                out.append(q + f"f_{a} = f_{a}.as_dummy(({bnds},))")
        for n, sym in u.syms.items():
            if sym.is_arg or sym.param is not None:
                continue
            if sym.rank and not sym.allocatable:
                if any(d is None for d in sym.dims):
                    raise FortranError(f"deferred-shape local {n}")
                bnds = ", ".join(f"({self.ex(lo, ctx)[0]}, {self.ex(hi, ctx)[0]})" for lo, hi in sym.dims)
                out.append(q + f"f_{n} = FArray.new({sym.typ if sym.typ in ('real', 'int') else 'obj'!r}, ({bnds},))")
            elif sym.rank:
                out.append(q + f"f_{n} = None")
            elif sym.init is not None:
                pass                                     # saved: set once, when the program is built
            else:
                out.append(q + f"f_{n} = {self.undefined.get((u.name, n))!r}")
        for c in u.contains:
            self.unit(c, ind + 1, out)
        self.block(u.body, ctx, ind + 1, out)
        out.append(q + f"return {ctx.ret}")
        if ctx.nonlocal_:
            out.insert(header_at, q + "nonlocal " + ", ".join(sorted(ctx.nonlocal_)))


class _Ctx:
    def __init__(self, unit, vis):
        self.unit, self.vis = unit, vis
        self.contained, self.targets = {}, set()
        self.nonlocal_ = set()
        self.loops, self.dispatch = [], 0
        self.n = 0
        self.ret = "None"
        self.top_ind = 1

    def fresh(self):
        self.n += 1
        return self.n


def _expr_names(e, out):
    if isinstance(e, Name):
        out.add(e.name)
    elif isinstance(e, Ref):
        for a in e.args:
            _expr_names(a, out)
    elif isinstance(e, Range):
        for x in (e.lo, e.hi, e.step):
            if x is not None:
                _expr_names(x, out)
    elif isinstance(e, Kw):
        _expr_names(e.value, out)
    elif isinstance(e, Comp):
        _expr_names(e.base, out)
    elif isinstance(e, Bin):
        _expr_names(e.l, out)
        _expr_names(e.r, out)
    elif isinstance(e, Un):
        _expr_names(e.x, out)
    elif isinstance(e, Cons):
        for x in e.items:
            _expr_names(x, out)


def _scalar_names(stmts) -> set:
    """Names used without subscripts (variables, not arrays or functions) and DO variables."""
    out = set()
    for s in stmts:
        if s.kind == "assign":
            _expr_names(s.a, out)
            _expr_names(s.b, out)
        elif s.kind == "if":
            for cond, blk in s.a:
                _expr_names(cond, out)
                out |= _scalar_names(blk)
            if s.orelse:
                out |= _scalar_names(s.orelse)
        elif s.kind == "do":
            out.add(s.a)
            for x in (s.b, s.c, s.d):
                if x is not None:
                    _expr_names(x, out)
            out |= _scalar_names(s.body)
        elif s.kind == "dowhile":
            _expr_names(s.a, out)
            out |= _scalar_names(s.body)
        elif s.kind == "call":
            for a in s.b:
                _expr_names(a, out)
        elif s.kind in ("read", "write"):
            stack = list(s.b or [])
            while stack:
                x = stack.pop()
                if isinstance(x, IDo):
                    out.add(x.var)
                    stack.extend(x.items)
                    for y in (x.lo, x.hi, x.step):
                        if y is not None:
                            _expr_names(y, out)
                else:
                    _expr_names(x, out)
    return out


def _goto_targets(stmts):
    t = set()
    for s in stmts:
        if s.kind == "goto":
            t.add(s.a)
        if s.kind in ("open", "read", "write") and isinstance(s.a, dict):
            t |= {s.a[k] for k in ("err", "end") if k in s.a}
        for blk in ([s.body] if s.body else []) + ([s.orelse] if s.orelse else []) + \
                ([b for _, b in s.a] if s.kind == "if" else []):
            t |= _goto_targets(blk)
    return t


class Namespace:
    """A module's variables at run time (attributes ``f_<name>``)."""


class Program:
    """Reference routines translated from their source text.

    ``sources``: file texts; ``defines``: the build's preprocessor macros.
    Modules contribute their specification parts (parameters and initialised
    variables are evaluated; other variables start undefined, for the caller to
    set); subroutines and functions become ``self.call(name, *args)``."""

    def __init__(self, sources: list[str], defines: set[str], undefined: dict | None = None):
        self.modules, self.procs = {}, {}
        self.undefined = {(p.lower(), n.lower()): v for (p, n), v in (undefined or {}).items()}
        for text in sources:
            if isinstance(text, tuple):
                text, fixed = text
                if fixed:
                    text = fixed_to_free(text)
            for u in parse_source(text, {d.upper() for d in defines}):
                if u.kind == "module":
                    self.modules[u.name] = u
                    for c in u.contains:
                        self.procs[c.name] = c
                else:
                    self.procs[u.name] = u
        gen = Gen(self.procs, self.modules, self.undefined)
        out = []
        self.ns = {}
        env = dict(RUNTIME)
        for name, mu in self.modules.items():
            ns = Namespace()
            self.ns[name] = ns
            env["m_" + name] = ns
        # module initial values, in dependency order of their uses
        for name, mu in self.modules.items():
            ctx = _Ctx(mu, gen.visible(mu))
            ns = self.ns[name]
            for n, sym in mu.syms.items():
                val = None
                try:
                    if sym.param is not None:
                        val = eval(gen.conv(*gen.ex(sym.param, ctx)[:2], sym.typ), env)
                    elif sym.rank and not sym.allocatable and all(d is not None for d in sym.dims):
                        bnds = [(eval(gen.ex(lo, ctx)[0], env), eval(gen.ex(hi, ctx)[0], env)) for lo, hi in sym.dims]
                        kind = sym.typ if sym.typ in ("real", "int") else "obj"
                        val = FArray.new(kind, bnds)       # a fixed-size module array exists from the start
                        if sym.typ.startswith("type:"):
                            _new_objs(val, sorted(gen.types_of(mu).get(sym.typ[5:], {})))
                        if sym.init is not None:
                            _asgn(val, None, eval(gen.ex(sym.init, ctx)[0], env))
                    elif sym.init is not None and not sym.rank:
                        val = eval(gen.conv(*gen.ex(sym.init, ctx)[:2], sym.typ), env)
                except (FortranError, NameError, TypeError):
                    val = None
                setattr(ns, "f_" + n, val)
        self.untranslated = {}
        units, stack = [], list(self.procs.values())
        while stack:
            x = stack.pop()
            units.append(x)
            stack.extend(x.contains)
        for x in units:                                  # saved locals of every procedure
            if x.kind == "module":
                continue
            ns = Namespace()
            env["s_" + x.name] = ns
            ctx = _Ctx(x, gen.visible(x))
            for n, sym in x.syms.items():
                if sym.init is not None and not sym.is_arg and sym.param is None and not sym.rank:
                    try:
                        setattr(ns, "f_" + n, eval(gen.conv(*gen.ex(sym.init, ctx)[:2], sym.typ), env))
                    except FortranError:
                        pass
        for u in self.procs.values():
            part = []
            try:
                gen.unit(u, 0, part)
            except FortranError as e:
                # procedures outside the supported subset stay callable only as errors
                self.untranslated[u.name] = str(e)
                part = [f"def p_{u.name}(*a):", f"    raise FortranError({str(e)!r})"]
            out.extend(part)
        code = "\n".join(out) + "\n"
        exec(compile(code, "<fortran>", "exec"), env)
        self.env = env

    def fragment(self, proc: str, first: int, last: int, name: str):
        """Make the statements of procedure ``proc`` that start on source lines
        first..last (whole statements of the outermost statement list that has
        any) callable as a subroutine without arguments, ``self.call(name)``,
        with the names ``proc`` sees: module variables, its locals (fresh on
        each call)."""
        u = self.procs[proc.lower()]

        def find(stmts):                         # the outermost list holding statements of the range
            hit = [st for st in stmts if first <= st.line <= last]
            if hit:
                return hit
            for st in stmts:
                for blk in ([st.body] if st.body else []) + ([st.orelse] if st.orelse else []) + \
                        ([b for _, b in st.a] if st.kind == "if" else []):
                    r = find(blk)
                    if r:
                        return r
            return []

        body = find(u.body)
        if not body:
            raise FortranError(f"no statements of {proc} on lines {first}-{last}")
        frag = Unit("subroutine", name.lower(), [], syms={k: v for k, v in u.syms.items() if not v.is_arg},
                    uses=u.uses, contains=[], host=u.host, types=u.types)
        frag.body = body
        gen = Gen(self.procs, self.modules, self.undefined)
        ns = Namespace()
        self.env["s_" + frag.name] = ns
        ctx = _Ctx(frag, gen.visible(frag))
        for n, sym in frag.syms.items():
            if sym.init is not None and sym.param is None and not sym.rank:
                setattr(ns, "f_" + n, eval(gen.conv(*gen.ex(sym.init, ctx)[:2], sym.typ), self.env))
        out = []
        gen.unit(frag, 0, out)
        exec(compile("\n".join(out) + "\n", "<fortran-fragment>", "exec"), self.env)

    def module(self, name) -> Namespace:
        return self.ns[name]

    def call(self, name, *args):
        return self.env["p_" + name.lower()](*args)
