"""The reference's case files: reading them into a ``Case``, writing a ``Case`` out.

Record format.  The reference is compiled with ``-convert big_endian -r8``
(src2LOWNS/Makefile:5, srcMakeGrid/Makefile:4) and writes Fortran unformatted
sequential files: each record is a 4-byte big-endian length, the payload, and
the length again; integers are 4 bytes and reals 8 bytes, both big-endian.  A
record longer than a subrecord's limit is split into subrecords; the leading
length of every subrecord but the last is negated, and the trailing length of
every subrecord but the first (the layout Intel and GNU Fortran share).

Files of a case ``P`` (written by the grid generator, srcMakeGrid/data_io.F90;
read by the solver, src2LOWNS/data_io.F90):

* ``P.xyz`` or ``P.xyzn`` -- ``is,js,ks,ie,je,ke``; ``x(l, ls-2:le+1)`` for
  l = 0, 1, 2; for a name not ending in ``z`` (the sparse form) also ``icc`` and
  ``icc`` records ``i,k,j,nf,nfb``, one per cell whose flag is -1, in i, j, k
  loop order (output_xyz 639-651, output_xyzn 1507-1555; read_data 99-128).
* ``P`` -- ``t0,g,nu``; in the dense form the flag grids nf and nfb over
  ``is-1:ie x js-1:je x ks-1:ke`` (k fastest, i slowest), then per numbered
  cell ``U(0:2),F,P`` (nn <= inne) or ``U(0:2)`` (nn > inne); in the sparse
  form ``icc,icc2`` then ``nn,U(0:2),F,P,nf,nfb`` and ``nn,U(0:2)`` records;
  last ``dt`` (output_data 707-783; read_data 130-289).
* ``P.fdata`` -- face fractions ``a(0:2,nn)`` and porosity ``fb(nn)``; dense
  per cell, or ``icc,icc2`` then ``nn,a,fb`` / ``nn,a`` records (output_fdata
  785-820; read_fdata 294-364).
* ``P.nsdata`` -- surface normals and positions ``nor(nn,0:3), sp(nn,0:2)``;
  dense over 1..inne, or ``mms`` then ``nn,nor,sp`` records (output_nsdata
  875-897; read_nsdata 366-397).

Cell numbering follows read_data (src2LOWNS/data_io.F90:168-201 and 257-276):
over ``j = js-1..je``, ``k = ks-1..ke``, ``i = is-1..ie`` (i fastest), first the
cells with ``nf >= 0`` or ``nf = -1`` and ``1 <= nfb < 200`` (1..inne), then the
obstacle-surface cells with ``nf = -1`` and ``nfb >= 200`` (inne+1..inne2, their
code becoming -1 for 300 and 0 otherwise); an unnumbered cell with
``nf = nfb = -1`` maps to the sentinel ``inne2+1`` and every other unnumbered
cell to the sentinel 0.  Grid spacings follow set_dx (src2LOWNS/1sub-main.F90:
53-74) with round (lib/src/xy_calc.f90:100-112).

The velocity read from ``P`` becomes the case's face velocity ``un``: the
pressure step projects it.  ``objno`` (moving objects) is zero.
"""
from __future__ import annotations

import dataclasses
import os
import pathlib
from typing import Optional

import numpy as np

from .workload import DT, G_ACC, Case

SDUM = -1.0e4                 # sdum, "no surface" marker (0mod-variables.F90:130)
MAX_SUBRECORD = 2147483639    # bytes of payload in one subrecord when writing

_I4 = np.dtype(">i4")
_F8 = np.dtype(">f8")


class FormatError(ValueError):
    """A case file that does not follow the record layout the reference reads."""


# ---------------------------------------------------------------------------
# records

class RecordReader:
    """Sequential reader of one Fortran unformatted file."""

    def __init__(self, path):
        self.path = str(path)
        self.buf = np.fromfile(self.path, dtype=np.uint8)
        self.pos = 0

    def at_end(self) -> bool:
        return self.pos >= self.buf.size

    def _marker(self) -> int:
        if self.pos + 4 > self.buf.size:
            raise FormatError(f"{self.path}: truncated record marker at byte {self.pos}")
        v = int(self.buf[self.pos:self.pos + 4].view(_I4)[0])
        self.pos += 4
        return v

    def record(self) -> np.ndarray:
        """Payload of the next record (subrecords joined) as bytes (uint8)."""
        parts = []
        first = True
        while True:
            start = self.pos
            head = self._marker()
            n = abs(head)
            if self.pos + n > self.buf.size:
                raise FormatError(f"{self.path}: record at byte {start} runs past the end of the file")
            parts.append(self.buf[self.pos:self.pos + n])
            self.pos += n
            tail = self._marker()
            if abs(tail) != n or (tail < 0) == first:
                raise FormatError(f"{self.path}: record markers at byte {start} do not match ({head}, {tail})")
            first = False
            if head >= 0:
                break
        return parts[0] if len(parts) == 1 else np.concatenate(parts)

    def read(self, dtype) -> np.ndarray:
        """The next record as exactly one item of ``dtype`` (a structured or plain type)."""
        dt = np.dtype(dtype)
        rec = self.record()
        if rec.size != dt.itemsize:
            raise FormatError(f"{self.path}: record of {rec.size} bytes where {dt.itemsize} were expected")
        return rec.view(dt)[0]

    def read_array(self, dtype, count: int) -> np.ndarray:
        """The next record as ``count`` items of ``dtype``."""
        dt = np.dtype(dtype)
        rec = self.record()
        if rec.size != dt.itemsize * count:
            raise FormatError(f"{self.path}: record of {rec.size} bytes where {dt.itemsize * count} were expected")
        return rec.view(dt).copy()

    def read_many(self, dtype, count: int) -> np.ndarray:
        """``count`` consecutive records, each one item of ``dtype`` (vectorised)."""
        dt = np.dtype(dtype)
        if count == 0:
            return np.zeros(0, dtype=dt)
        framed = np.dtype([("head", _I4), ("body", dt), ("tail", _I4)])
        nbytes = framed.itemsize * count
        if self.pos + nbytes > self.buf.size:
            raise FormatError(f"{self.path}: {count} records of {dt.itemsize} bytes run past the end of the file")
        recs = self.buf[self.pos:self.pos + nbytes].view(framed)
        if not (np.all(recs["head"] == dt.itemsize) and np.all(recs["tail"] == dt.itemsize)):
            bad = int(np.flatnonzero((recs["head"] != dt.itemsize) | (recs["tail"] != dt.itemsize))[0])
            raise FormatError(f"{self.path}: record {bad} of a run of {count} is not {dt.itemsize} bytes long")
        self.pos += nbytes
        return recs["body"].copy()


class RecordWriter:
    """Sequential writer of one Fortran unformatted file."""

    def __init__(self, path, max_subrecord: int = MAX_SUBRECORD):
        self.path = str(path)
        self.max_sub = int(max_subrecord)
        self.f = open(self.path, "wb")

    def close(self):
        self.f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def record(self, payload) -> None:
        data = payload.tobytes() if isinstance(payload, np.ndarray) else bytes(payload)
        chunks = [data[o:o + self.max_sub] for o in range(0, len(data), self.max_sub)] or [b""]
        last = len(chunks) - 1
        for s, c in enumerate(chunks):
            n = len(c)
            self.f.write(np.array([-n if s < last else n], dtype=_I4).tobytes())
            self.f.write(c)
            self.f.write(np.array([-n if s > 0 else n], dtype=_I4).tobytes())

    def write_many(self, arr: np.ndarray) -> None:
        """One record per item of ``arr`` (vectorised)."""
        dt = arr.dtype
        if dt.itemsize > self.max_sub:
            for item in arr:
                self.record(np.array([item], dtype=dt))
            return
        framed = np.zeros(arr.size, dtype=np.dtype([("head", _I4), ("body", dt), ("tail", _I4)]))
        framed["head"] = dt.itemsize
        framed["tail"] = dt.itemsize
        framed["body"] = arr
        self.f.write(framed.tobytes())


# record layouts (0mod-type_interface.F90:7-9: every flag a default integer)
DATA_DENSE_IN = np.dtype([("u", _F8, (3,)), ("f", _F8), ("p", _F8)])
DATA_DENSE_OUT = np.dtype([("u", _F8, (3,))])
DATA_SPARSE_IN = np.dtype([("nn", _I4), ("u", _F8, (3,)), ("f", _F8), ("p", _F8), ("nf", _I4), ("nfb", _I4)])
DATA_SPARSE_OUT = np.dtype([("nn", _I4), ("u", _F8, (3,))])
FDATA_DENSE_IN = np.dtype([("a", _F8, (3,)), ("fb", _F8)])
FDATA_DENSE_OUT = np.dtype([("a", _F8, (3,))])
FDATA_SPARSE_IN = np.dtype([("nn", _I4), ("a", _F8, (3,)), ("fb", _F8)])
FDATA_SPARSE_OUT = np.dtype([("nn", _I4), ("a", _F8, (3,))])
NSDATA_DENSE = np.dtype([("nor", _F8, (4,)), ("sp", _F8, (3,))])
NSDATA_SPARSE = np.dtype([("nn", _I4), ("nor", _F8, (4,)), ("sp", _F8, (3,))])
OBSTACLE = np.dtype([("i", _I4), ("k", _I4), ("j", _I4), ("nf", _I4), ("nfb", _I4)])


# ---------------------------------------------------------------------------
# grid

def check_dims(dims) -> np.ndarray:
    """is..ke as int32[6]; the reference keeps x(l, ls-2:le+1) in x(0:2, 1:mx2),
    so ls >= 3, and every axis holds at least one cell."""
    d = np.asarray(dims, dtype=np.int64).reshape(-1)
    if d.size != 6 or np.any(d[:3] < 3) or np.any(d[3:] <= d[:3]) or np.any(d > 2**30):
        raise FormatError(f"grid bounds is,js,ks,ie,je,ke = {d.tolist()} are not usable (need ls >= 3, le > ls)")
    return d.astype(np.int32)


def mx2_of(dims) -> int:
    """mx2 = max(ie+2, je+2, ke+2) (alloc_dxdydz, 0mod-arrays.F90:201)."""
    return int(max(dims[3], dims[4], dims[5])) + 2


def fortran_nint(v: np.ndarray) -> np.ndarray:
    """NINT: nearest integer, halves away from zero (exact for every double)."""
    v = np.asarray(v, dtype=np.float64)
    r = np.round(v)                          # halves to even
    t = np.trunc(v)
    tie = np.abs(v - t) == 0.5
    return np.where(tie, t + np.sign(v), r)


def round_dec(num, dec: int) -> np.ndarray:
    """round(num, dec) = dble(nint(num 10**dec)) / 10**dec (lib/src/xy_calc.f90:100-112)."""
    a = 10.0 ** dec
    return fortran_nint(np.asarray(num, dtype=np.float64) * a) / a


def set_dx(dims, x: np.ndarray):
    """Spacings from coordinates (1sub-main.F90:53-74).  ``x`` (mx2, 3) holds
    x(l, i) at [i-1, l]; returns (x, dx) with x(l, le+1) extrapolated when it is 0."""
    x = np.array(x, dtype=np.float64, copy=True)
    dx = np.zeros_like(x)
    ls = [int(dims[0]), int(dims[1]), int(dims[2])]
    le = [int(dims[3]), int(dims[4]), int(dims[5])]
    for l in range(3):
        s, e = ls[l], le[l]
        X = lambda i: x[i - 1, l]            # noqa: E731  x(l, i)
        if X(e + 1) == 0.0:
            x[e, l] = X(e) + X(e) - X(e - 1)
        first = X(s + 1) - X(s)
        dec = 11                             # the DO variable after a loop without exit
        for d in range(0, 11):
            if first / 10.0 ** (4 - d) > 1.0:
                dec = d
                break
        i = np.arange(s - 2, e + 1)
        dx[i - 1, l] = round_dec(x[i, l] - x[i - 1, l], dec)
        dx[e, l] = dx[e - 1, l]
    return x, dx


# ---------------------------------------------------------------------------
# numbering

@dataclasses.dataclass
class Numbering:
    """read_data's cell numbering for flag grids over is-1:ie x js-1:je x ks-1:ke."""
    mn: np.ndarray        # int32 (NJ, NK, NI) over is-2:ie+2 etc., i fastest
    in_: np.ndarray       # int32 (inne2+2,)
    jn: np.ndarray
    kn: np.ndarray
    inne: int
    inne2: int
    nfb3: np.ndarray      # the nfb grid after the obstacle-surface recoding


def _grid_shape(dims):
    is_, js, ks, ie, je, ke = (int(v) for v in dims)
    return (je - js + 2, ke - ks + 2, ie - is_ + 2)       # [j][k][i] over js-1..je etc.


def number_cells(dims, nf3: np.ndarray, nfb3: np.ndarray) -> Numbering:
    """data_io.F90:168-201 (both numbering passes), vectorised.  ``nf3``/``nfb3``
    are indexed [j - (js-1)][k - (ks-1)][i - (is-1)]."""
    dims = check_dims(dims)
    is_, js, ks, ie, je, ke = (int(v) for v in dims)
    shape = _grid_shape(dims)
    nf3 = np.asarray(nf3, dtype=np.int32)
    nfb3 = np.array(nfb3, dtype=np.int32, copy=True)
    if nf3.shape != shape or nfb3.shape != shape:
        raise FormatError(f"flag grids of shape {nf3.shape}/{nfb3.shape}, expected {shape}")
    first = (nf3 >= 0) | ((nf3 == -1) & (nfb3 >= 1) & (nfb3 < 200))
    second = (nf3 == -1) & (nfb3 >= 200)
    inne = int(first.sum())
    inne2 = inne + int(second.sum())
    num = np.zeros(shape, dtype=np.int32)
    num[first] = np.arange(1, inne + 1, dtype=np.int32)           # C order = j, k, i loops
    num[second] = np.arange(inne + 1, inne2 + 1, dtype=np.int32)
    nfb3[second] = np.where(nfb3[second] == 300, -1, 0)
    jj, kk, ii = np.indices(shape, dtype=np.int32)
    in_ = np.zeros(inne2 + 2, dtype=np.int32)
    jn = np.zeros(inne2 + 2, dtype=np.int32)
    kn = np.zeros(inne2 + 2, dtype=np.int32)
    sel = num > 0
    cells = num[sel]
    in_[cells] = ii[sel] + is_ - 1
    jn[cells] = jj[sel] + js - 1
    kn[cells] = kk[sel] + ks - 1
    mn = np.zeros((je - js + 5, ke - ks + 5, ie - is_ + 5), dtype=np.int32)
    mn[1:-2, 1:-2, 1:-2] = num
    return Numbering(mn=mn, in_=in_, jn=jn, kn=kn, inne=inne, inne2=inne2, nfb3=nfb3)


def cell_flags(dims, nf3: np.ndarray, nfb3: np.ndarray, numbering: Numbering):
    """nff(0:inne2+1) from the flag grids, and the sentinel map for unnumbered
    cells with nf = nfb = -1 (data_io.F90:257-276).  Returns (nf, nfb, mn)."""
    num = numbering.mn[1:-2, 1:-2, 1:-2]
    nf = np.zeros(numbering.inne2 + 2, dtype=np.int32)
    nfb = np.zeros(numbering.inne2 + 2, dtype=np.int32)
    sel = num > 0
    nf[num[sel]] = nf3[sel]
    nfb[num[sel]] = nfb3[sel]
    nf[0], nfb[0] = -1, 0
    nf[-1], nfb[-1] = -1, -1
    mn = numbering.mn.copy()
    inner = mn[1:-2, 1:-2, 1:-2]
    inner[(num == 0) & (nf3 == -1) & (nfb3 == -1)] = numbering.inne2 + 1
    return nf, nfb, mn


# ---------------------------------------------------------------------------
# reading

@dataclasses.dataclass
class Ingested:
    """A case read from the reference's files, with what the pressure path does
    not use kept beside it."""
    case: Case
    p: np.ndarray               # f64 (inne2+2,): pressure P(nn)
    nor: np.ndarray             # f64 (inne2+2, 4): surface normals nor(nn, 0:3)
    t0: float
    g: float
    nu: float
    dt0: Optional[float]        # the trailing dt record, read when t0 > 0
    sparse: bool                # .xyzn (sparse) form, as opposed to .xyz (dense)
    nf3: np.ndarray             # flag grids as read, [j][k][i] over js-1..je etc.
    nfb3: np.ndarray


def read_xyz(path):
    """(dims, x (mx2, 3), obstacle records or None) -- data_io.F90:99-128."""
    path = str(path)
    r = RecordReader(path)
    dims = check_dims(r.read_array(_I4, 6))
    mx2 = mx2_of(dims)
    x = np.zeros((mx2, 3), dtype=np.float64)
    for l in range(3):
        s, e = int(dims[l]), int(dims[3 + l])
        x[s - 3:e + 1, l] = r.read_array(_F8, e + 1 - (s - 2) + 1)      # x(l, s-2 .. e+1)
    sparse = not path.endswith("z")
    obst = None
    if sparse:
        icc = int(r.read(_I4))
        if icc < 0:
            raise FormatError(f"{path}: negative cell count {icc}")
        obst = r.read_many(OBSTACLE, icc)
    return dims, x, obst


def _flag_grids_from_obstacles(dims, obst, path):
    is_, js, ks, ie, je, ke = (int(v) for v in dims)
    shape = _grid_shape(dims)
    nf3 = np.zeros(shape, dtype=np.int32)
    nfb3 = np.zeros(shape, dtype=np.int32)
    if obst is not None and obst.size:
        i, k, j = obst["i"].astype(np.int64), obst["k"].astype(np.int64), obst["j"].astype(np.int64)
        # the reference's grids span ls-2:le+2; only ls-1:le takes part in the numbering
        ok = (i >= is_ - 2) & (i <= ie + 2) & (k >= ks - 2) & (k <= ke + 2) & (j >= js - 2) & (j <= je + 2)
        if not np.all(ok):
            raise FormatError(f"{path}: a flagged cell lies outside the grid")
        inr = (i >= is_ - 1) & (i <= ie) & (k >= ks - 1) & (k <= ke) & (j >= js - 1) & (j <= je)
        nf3[j[inr] - js + 1, k[inr] - ks + 1, i[inr] - is_ + 1] = obst["nf"][inr]
        nfb3[j[inr] - js + 1, k[inr] - ks + 1, i[inr] - is_ + 1] = obst["nfb"][inr]
    return nf3, nfb3


def _default(prefix: str, ext: str) -> Optional[str]:
    p = prefix + ext
    return p if os.path.exists(p) else None


def read_case(prefix, *, xyz=None, fdata=None, nsdata=None, dt: Optional[float] = None,
              eps0: float = 1.0e-10, label: str = "") -> Ingested:
    """Read case ``prefix`` the way read_data, read_fdata, read_nsdata and set_dx
    do (src2LOWNS/data_io.F90:87-397, 1sub-main.F90:53-74).

    ``xyz`` defaults to ``prefix.xyzn`` when present, else ``prefix.xyz``;
    ``fdata`` and ``nsdata`` to ``prefix.fdata`` / ``prefix.nsdata`` when present.
    Without an fdata file every face is open and the porosity 1 (cells
    1..inne); without an nsdata file every surface position is the "no surface"
    marker -1e4.  ``dt`` defaults to the file's trailing dt (read when t0 > 0,
    as the reference does), else 1e-3."""
    prefix = str(prefix)
    if xyz is None:
        xyz = _default(prefix, ".xyzn") or prefix + ".xyz"
    fdata = fdata if fdata is not None else _default(prefix, ".fdata")
    nsdata = nsdata if nsdata is not None else _default(prefix, ".nsdata")

    dims, x, obst = read_xyz(xyz)
    sparse = obst is not None
    is_, js, ks, ie, je, ke = (int(v) for v in dims)
    shape = _grid_shape(dims)
    ncount = shape[0] * shape[1] * shape[2]

    r = RecordReader(prefix)
    t0, g, nu = (float(v) for v in r.read_array(_F8, 3))
    if sparse:
        nf3, nfb3 = _flag_grids_from_obstacles(dims, obst, xyz)
    else:
        # k fastest, j, i slowest -> [i][j][k] -> [j][k][i]
        nf3 = r.read_array(_I4, ncount).reshape(shape[2], shape[0], shape[1]).transpose(1, 2, 0).astype(np.int32)
        nfb3 = r.read_array(_I4, ncount).reshape(shape[2], shape[0], shape[1]).transpose(1, 2, 0).astype(np.int32)
    nf3 = np.ascontiguousarray(nf3)
    numbering = number_cells(dims, nf3, nfb3)
    nfb3 = numbering.nfb3
    inne, inne2 = numbering.inne, numbering.inne2
    ncell = inne2 + 2

    u = np.zeros((ncell, 3))
    f = np.zeros(ncell)
    p = np.zeros(ncell)
    if sparse:
        icc, icc2 = (int(v) for v in r.read_array(_I4, 2))
        if icc < 0 or icc2 < 0:
            raise FormatError(f"{prefix}: negative record counts {icc}, {icc2}")
        rin = r.read_many(DATA_SPARSE_IN, icc)
        rout = r.read_many(DATA_SPARSE_OUT, icc2)
        for recs in (rin, rout):
            nn = recs["nn"].astype(np.int64)
            if nn.size and (nn.min() < 1 or nn.max() > inne2):
                raise FormatError(f"{prefix}: a cell number lies outside 1..{inne2}")
        nn = rin["nn"].astype(np.int64)
        u[nn] = rin["u"]
        f[nn] = rin["f"]
        p[nn] = rin["p"]
        gj, gk, gi = numbering.jn[nn] - js + 1, numbering.kn[nn] - ks + 1, numbering.in_[nn] - is_ + 1
        nf3[gj, gk, gi] = rin["nf"]
        nfb3[gj, gk, gi] = rin["nfb"]
        u[rout["nn"].astype(np.int64)] = rout["u"]
    else:
        rin = r.read_many(DATA_DENSE_IN, inne)
        rout = r.read_many(DATA_DENSE_OUT, inne2 - inne)
        u[1:inne + 1] = rin["u"]
        f[1:inne + 1] = rin["f"]
        p[1:inne + 1] = rin["p"]
        u[inne + 1:inne2 + 1] = rout["u"]
    nf, nfb, mn = cell_flags(dims, nf3, nfb3, numbering)
    dt0 = None
    if t0 > 0.0 and not r.at_end():
        try:
            dt0 = float(r.read(_F8))
        except FormatError:
            dt0 = None                       # read(8, iostat=ist): a failed read is skipped

    a = np.zeros((ncell, 3))
    fb = np.zeros(ncell)
    if fdata is None:
        a[1:inne + 1] = 1.0
        fb[1:inne + 1] = 1.0
    else:
        rf = RecordReader(fdata)
        if sparse:
            a[1:inne + 1] = 1.0
            fb[1:inne + 1] = 1.0
            icc, icc1 = (int(v) for v in rf.read_array(_I4, 2))
            if icc < 0 or icc1 < 0:
                raise FormatError(f"{fdata}: negative record counts {icc}, {icc1}")
            fin = rf.read_many(FDATA_SPARSE_IN, icc)
            fout = rf.read_many(FDATA_SPARSE_OUT, icc1)
            for recs in (fin, fout):
                nn = recs["nn"].astype(np.int64)
                if nn.size and (nn.min() < 1 or nn.max() > inne2):
                    raise FormatError(f"{fdata}: a cell number lies outside 1..{inne2}")
            a[fin["nn"].astype(np.int64)] = fin["a"]
            fb[fin["nn"].astype(np.int64)] = fin["fb"]
            a[fout["nn"].astype(np.int64)] = fout["a"]
        else:
            fin = rf.read_many(FDATA_DENSE_IN, inne)
            fout = rf.read_many(FDATA_DENSE_OUT, inne2 - inne)
            a[1:inne + 1] = fin["a"]
            fb[1:inne + 1] = fin["fb"]
            a[inne + 1:inne2 + 1] = fout["a"]

    sp = np.zeros((3, ncell))
    nor = np.zeros((ncell, 4))
    if nsdata is None:
        sp[0, 1:inne + 1] = SDUM
    else:
        rs = RecordReader(nsdata)
        if sparse:
            sp[0, 1:inne + 1] = SDUM
            mms = int(rs.read(_I4))
            if mms < 0:
                raise FormatError(f"{nsdata}: negative surface-cell count {mms}")
            recs = rs.read_many(NSDATA_SPARSE, mms)
            nn = recs["nn"].astype(np.int64)
            if nn.size and (nn.min() < 0 or nn.max() > inne2 + 1):
                raise FormatError(f"{nsdata}: a cell number lies outside 0..{inne2 + 1}")
            nor[nn] = recs["nor"]
            sp[:, nn] = recs["sp"].T
        else:
            recs = rs.read_many(NSDATA_DENSE, inne)
            nor[1:inne + 1] = recs["nor"]
            sp[:, 1:inne + 1] = recs["sp"].T
    sp[0, 0] = SDUM
    sp[0, inne + 1:] = SDUM

    x, dx = set_dx(dims, x)
    case = Case(nx=ie - is_, ny=je - js, nz=ke - ks, dims=dims, mx2=mx2_of(dims), x=x, dx=dx, mn=mn,
                inne=inne, inne2=inne2, in_=numbering.in_, jn=numbering.jn, kn=numbering.kn, nf=nf, nfb=nfb,
                f=f, fb=fb, a=a, un=u, sp=sp, objno=np.zeros(ncell, dtype=np.int32),
                dt=float(dt if dt is not None else (dt0 if dt0 is not None else DT)), eps0=eps0,
                label=label or pathlib.Path(prefix).name)
    return Ingested(case=case, p=p, nor=nor, t0=t0, g=g, nu=nu, dt0=dt0, sparse=sparse, nf3=nf3, nfb3=nfb3)


# ---------------------------------------------------------------------------
# writing

def flag_grids(case: Case):
    """The flag grids over is-1:ie x js-1:je x ks-1:ke ([j][k][i]) that the
    grid generator would write for ``case``: numbered cells carry their flags,
    obstacle-surface cells (inne+1..inne2) 300 when their code is -1 and 200
    otherwise, sentinel inne2+1 cells -1/-1, every other cell -1/0
    (output_data 719-738)."""
    dims = check_dims(case.dims)
    shape = _grid_shape(dims)
    num = np.asarray(case.mn)[1:-2, 1:-2, 1:-2]
    if num.shape != shape:
        raise FormatError(f"mn of shape {case.mn.shape} does not match the grid bounds")
    nf3 = np.full(shape, -1, dtype=np.int32)
    nfb3 = np.zeros(shape, dtype=np.int32)
    sel = (num > 0) & (num <= case.inne2)
    cells = num[sel]
    nf3[sel] = case.nf[cells]
    nfb3[sel] = case.nfb[cells]
    obst = sel.copy()
    obst[sel] = cells > case.inne
    nf3[obst] = -1
    nfb3[obst] = np.where(case.nfb[num[obst]] == -1, 300, 200)
    nfb3[num == case.inne2 + 1] = -1
    return nf3, nfb3


def write_case(prefix, case: Case, *, p: Optional[np.ndarray] = None, nor: Optional[np.ndarray] = None,
               t: float = 0.0, g: float = G_ACC, nu: float = 1.0e-6, dt: Optional[float] = None,
               sparse: bool = True, max_subrecord: int = MAX_SUBRECORD) -> dict:
    """Write ``case`` as the grid generator does: the xyz file (``.xyzn`` sparse,
    ``.xyz`` dense), the data file, ``.fdata`` and ``.nsdata``.  ``p`` and
    ``nor`` default to zero, ``dt`` to the case's.  In the sparse form a cell
    is listed in ``.nsdata`` when its surface x position is not -1e4, and the
    data and fdata files skip the cells the generator skips (an air cell at
    rest with F < 1e-13; a cell with all faces open and porosity 1).  One
    file departs from the generator: in the dense form the generator
    (srcMakeGrid/data_io.F90:785-820) still writes the sparse ``.fdata``,
    which the solver's read_fdata (src2LOWNS/data_io.F90:302-345) reads only
    when the xyz file is sparse; here the dense form gets the dense
    ``.fdata`` (per cell ``a(0:2,nn), fb(nn)``) that the solver reads."""
    prefix = str(prefix)
    dims = check_dims(case.dims)
    is_, js, ks, ie, je, ke = (int(v) for v in dims)
    inne, inne2 = int(case.inne), int(case.inne2)
    ncell = inne2 + 2
    p = np.zeros(ncell) if p is None else np.asarray(p, dtype=np.float64)
    nor = np.zeros((ncell, 4)) if nor is None else np.asarray(nor, dtype=np.float64)
    dt = case.dt if dt is None else dt
    nf3, nfb3 = flag_grids(case)
    paths = {}

    xyz = prefix + (".xyzn" if sparse else ".xyz")
    with RecordWriter(xyz, max_subrecord) as w:
        w.record(np.asarray(dims, dtype=_I4))
        for l in range(3):
            s, e = int(dims[l]), int(dims[3 + l])
            w.record(np.asarray(case.x[s - 3:e + 1, l], dtype=_F8))
        if sparse:
            g_ijk = (nf3.transpose(2, 0, 1), nfb3.transpose(2, 0, 1))       # [i][j][k]: i, j, k loops
            ii, jj, kk = np.nonzero(g_ijk[0] == -1)
            recs = np.zeros(ii.size, dtype=OBSTACLE)
            recs["i"] = ii + is_ - 1
            recs["k"] = kk + ks - 1
            recs["j"] = jj + js - 1
            recs["nf"] = -1
            recs["nfb"] = g_ijk[1][ii, jj, kk]
            w.record(np.array([ii.size], dtype=_I4))
            w.write_many(recs)
    paths["xyz"] = xyz

    with RecordWriter(prefix, max_subrecord) as w:
        w.record(np.array([t, g, nu], dtype=_F8))
        u, f = case.un, case.f
        if sparse:
            idx = np.arange(1, inne2 + 1)
            usq = (u[idx, 0] ** 2 + u[idx, 1] ** 2) + u[idx, 2] ** 2
            skip = (case.nf[idx] == 0) & (usq == 0.0) & (f[idx] < 1.0e-13)
            keep = idx[~skip]
            kin, kout = keep[keep <= inne], keep[keep > inne]
            w.record(np.array([kin.size, kout.size], dtype=_I4))
            rin = np.zeros(kin.size, dtype=DATA_SPARSE_IN)
            rin["nn"], rin["u"], rin["f"], rin["p"] = kin, u[kin], f[kin], p[kin]
            rin["nf"], rin["nfb"] = case.nf[kin], case.nfb[kin]
            rout = np.zeros(kout.size, dtype=DATA_SPARSE_OUT)
            rout["nn"], rout["u"] = kout, u[kout]
            w.write_many(rin)
            w.write_many(rout)
        else:
            w.record(np.ascontiguousarray(nf3.transpose(2, 0, 1)).astype(_I4))
            w.record(np.ascontiguousarray(nfb3.transpose(2, 0, 1)).astype(_I4))
            rin = np.zeros(inne, dtype=DATA_DENSE_IN)
            rin["u"], rin["f"], rin["p"] = u[1:inne + 1], f[1:inne + 1], p[1:inne + 1]
            rout = np.zeros(inne2 - inne, dtype=DATA_DENSE_OUT)
            rout["u"] = u[inne + 1:inne2 + 1]
            w.write_many(rin)
            w.write_many(rout)
        w.record(np.array([dt], dtype=_F8))
    paths["data"] = prefix

    with RecordWriter(prefix + ".fdata", max_subrecord) as w:
        a, fb = case.a, case.fb
        if sparse:
            idx = np.arange(1, inne + 1)
            full = (a[idx, 0] == 1.0) & (a[idx, 1] == 1.0) & (a[idx, 2] == 1.0) & (fb[idx] == 1.0)
            kin = idx[~full]
            idx2 = np.arange(inne + 1, inne2 + 1)
            kout = idx2[((a[idx2, 0] + a[idx2, 1]) + a[idx2, 2]) != 0.0]
            w.record(np.array([kin.size, kout.size], dtype=_I4))
            rin = np.zeros(kin.size, dtype=FDATA_SPARSE_IN)
            rin["nn"], rin["a"], rin["fb"] = kin, a[kin], fb[kin]
            rout = np.zeros(kout.size, dtype=FDATA_SPARSE_OUT)
            rout["nn"], rout["a"] = kout, a[kout]
            w.write_many(rin)
            w.write_many(rout)
        else:
            rin = np.zeros(inne, dtype=FDATA_DENSE_IN)
            rin["a"], rin["fb"] = a[1:inne + 1], fb[1:inne + 1]
            rout = np.zeros(inne2 - inne, dtype=FDATA_DENSE_OUT)
            rout["a"] = a[inne + 1:inne2 + 1]
            w.write_many(rin)
            w.write_many(rout)
    paths["fdata"] = prefix + ".fdata"

    with RecordWriter(prefix + ".nsdata", max_subrecord) as w:
        sp = case.sp
        if sparse:
            idx = np.arange(1, inne + 1)
            keep = idx[sp[0, idx] != SDUM]
            w.record(np.array([keep.size], dtype=_I4))
            recs = np.zeros(keep.size, dtype=NSDATA_SPARSE)
            recs["nn"], recs["nor"], recs["sp"] = keep, nor[keep], sp[:, keep].T
            w.write_many(recs)
        else:
            recs = np.zeros(inne, dtype=NSDATA_DENSE)
            recs["nor"], recs["sp"] = nor[1:inne + 1], sp[:, 1:inne + 1].T
            w.write_many(recs)
    paths["nsdata"] = prefix + ".nsdata"
    return paths
