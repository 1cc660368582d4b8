"""ctypes front end of the CPU oracle (test infrastructure only).

Loaded by the tests, the smoke check and the CPU-baseline leg of the benchmark.
It never backs the product path.  Parity status: pinned to the reference's own
source, run through a Fortran translator (see clowns_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
import pathlib
import subprocess
import threading

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "libclowns_oracle.so"
_lock = threading.Lock()
_lib = None

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> pathlib.Path:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    src = HERE / "clowns_oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(str(LIB_PATH))
            P = C.c_void_p
            i = C.c_int
            d = C.c_double
            L.ora_set_nflag.restype = i
            L.ora_set_nflag.argtypes = [P, i, i, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P]
            L.ora_init_matrix.restype = None
            L.ora_init_matrix.argtypes = [P, i, i, P, P, P, P, P, P, P, P, P, P, P, P, P]
            L.ora_rows_rhs.restype = i
            L.ora_rows_rhs.argtypes = [P, i, i, P, P, P, P, P, P, P, P, P, P, P, d, d, i, P,
                                       i, P, P, P, P, P, P]
            L.ora_assemble.restype = i
            L.ora_assemble.argtypes = [P, i, i, i, P, P, P, P, P, P, P, P, i, P, P, P, P, P,
                                       i, P, P, P]
            L.ora_pcgpme.restype = None
            L.ora_pcgpme.argtypes = [P, P, P, P, P, P, P, P, P, P, P, P, P, i, P]
            L.ora_pcgpme_setup.restype = None
            L.ora_pcgpme_setup.argtypes = [P, i, i, P, P, i, P, d]
            L.ora_axsub.restype = None
            L.ora_axsub.argtypes = [P, i, i, P, P, i, i, P, P]
            L.ora_ldusub.restype = None
            L.ora_ldusub.argtypes = [P, i, i, P, i, i, P]
            L.ora_correct.restype = None
            L.ora_correct.argtypes = [P, i, i, P, P, P, P, P, P, P, P, d, i, P, P, P, P, P]
            L.ora_transpose.restype = None
            L.ora_transpose.argtypes = [i, i, i, P, P, P, P, P, P]
            L.ora_spmv.restype = None
            L.ora_spmv.argtypes = [i, i, i, P, P, P, P, P]
            L.ora_grid_nl.restype = i
            L.ora_grid_nl.argtypes = [P]
            L.ora_pcgpme_will.restype = None
            L.ora_pcgpme_will.argtypes = [P, i, i, P, P, i, i, P, d, d, i, i, P, P]
            L.ora_will_postprocess.restype = None
            L.ora_will_postprocess.argtypes = [P, P, P, i, C.c_long, i]
            _lib = L
    return _lib


def _p(a: np.ndarray, off: int = 0):
    assert a.flags["C_CONTIGUOUS"], "array must be contiguous"
    return C.c_void_p(a.ctypes.data + off * a.itemsize)


@dataclasses.dataclass
class Classified:
    nf: np.ndarray
    nfb: np.ndarray
    f: np.ndarray
    fln: np.ndarray      # (ifln+1,), element 0 unused
    ifln: int
    sfn: np.ndarray
    isfn: int
    passes: int


def set_nflag(case) -> Classified:
    """Restated set_nflag on a copy of the case's flags (nfd2015.F90:7-306)."""
    L = lib()
    nf = case.nf.copy()
    nfb = case.nfb.copy()
    f = case.f.copy()
    ncell = case.inne2 + 2
    fln = np.zeros(ncell + 1, dtype=np.int32)
    sfn = np.zeros(ncell + 1, dtype=np.int32)
    ifln = C.c_int(0)
    isfn = C.c_int(0)
    passes = L.ora_set_nflag(_p(case.dims), case.inne, case.mx2, _p(case.mn), _p(case.in_),
                             _p(case.jn), _p(case.kn), _p(nf), _p(nfb), _p(f), _p(case.fb),
                             _p(case.a), _p(case.dx), _p(case.objno), _p(fln), C.byref(ifln),
                             _p(sfn), C.byref(isfn))
    if passes < 0:
        raise RuntimeError("set_nflag did not settle")
    return Classified(nf=nf, nfb=nfb, f=f, fln=fln[:ifln.value + 1].copy(), ifln=ifln.value,
                      sfn=sfn[:isfn.value + 1].copy(), isfn=isfn.value, passes=passes)


@dataclasses.dataclass
class StaticMatrix:
    mp: float
    alu_c: np.ndarray    # (nl, inne) == ALU_C(1:inne, 1:nl) column-major
    ll_c: np.ndarray     # (nl, inne)
    de_c: np.ndarray     # (inne,)


def grid_nl(dims) -> int:
    """Matrix columns of a grid: 6 (3D), 4 (2DV: one cell wide in x or y) or 0."""
    return int(lib().ora_grid_nl(_p(np.ascontiguousarray(dims, dtype=np.int32))))


def init_matrix(case, cls: Classified) -> StaticMatrix:
    L = lib()
    nl = grid_nl(case.dims)
    if nl == 0:
        raise ValueError("a grid one cell wide in both x and y has no matrix form in the reference")
    alu_c = np.zeros((nl, case.inne), dtype=np.float64)
    ll_c = np.zeros((nl, case.inne), dtype=np.int32)
    de_c = np.zeros(case.inne, dtype=np.float64)
    mp = C.c_double(0.0)
    L.ora_init_matrix(_p(case.dims), case.inne, case.mx2, _p(case.mn), _p(case.in_),
                      _p(case.jn), _p(case.kn), _p(cls.nf), _p(cls.nfb), _p(case.a),
                      _p(case.fb), _p(case.dx), C.byref(mp), _p(alu_c), _p(ll_c), _p(de_c))
    return StaticMatrix(mp=mp.value, alu_c=alu_c, ll_c=ll_c, de_c=de_c)


@dataclasses.dataclass
class System:
    """Assembled pressure system as the reference hands it to PCGPME."""
    mm2: int
    mnoe: int
    mno: np.ndarray      # (je, ke, ie) i fastest == mno(1:ie,1:ke,1:je)
    mno2mn: np.ndarray   # (mm2+1,), element 0 unused
    b: np.ndarray        # (mm2+1,), element 0 unused
    de: np.ndarray       # (mm2+1,)
    xe: np.ndarray       # (mm2+1,) == xe(0:mm2)
    alu: np.ndarray      # (nl, mm2) == alu(1:mm2, 1:nl)
    llu: np.ndarray      # (nl, mm2)
    dmax: float


def rows_rhs_assemble(case, cls: Classified, sm: StaticMatrix, mm2: int | None = None) -> System:
    L = lib()
    if mm2 is None:
        mm2 = cls.ifln + 5000          # m_alloc = ifln + 5000 (1sub-momentum.F90:254)
    is_, js, ks, ie, je, ke = (int(v) for v in case.dims)
    mno = np.zeros((je, ke, ie), dtype=np.int32)
    mno2mn = np.zeros(mm2 + 1, dtype=np.int32)
    b = np.zeros(mm2 + 1)
    xe = np.zeros(mm2 + 1)
    de = np.zeros(mm2 + 1)
    dmax = C.c_double(0.0)
    fln = np.ascontiguousarray(cls.fln)
    mnoe = L.ora_rows_rhs(_p(case.dims), case.inne2, case.mx2, _p(case.mn), _p(case.in_),
                          _p(case.jn), _p(case.kn), _p(cls.nf), _p(cls.nfb), _p(cls.f),
                          _p(case.fb), _p(case.a), _p(case.un), _p(case.dx), sm.mp, case.dt,
                          cls.ifln, _p(fln), mm2, _p(mno), _p(mno2mn), _p(b), _p(xe), _p(de),
                          C.byref(dmax))
    if mnoe < 0:
        raise RuntimeError("matrix leading dimension too small")
    nl = sm.alu_c.shape[0]
    alu = np.zeros((nl, mm2))
    llu = np.zeros((nl, mm2), dtype=np.int32)
    bad = L.ora_assemble(_p(case.dims), case.inne, case.inne2, case.mx2, _p(case.in_),
                         _p(case.jn), _p(case.kn), _p(cls.nf), _p(cls.nfb), _p(case.x),
                         _p(case.dx), _p(case.sp), cls.ifln, _p(fln), _p(mno), _p(sm.alu_c),
                         _p(sm.ll_c), _p(sm.de_c), mm2, _p(alu), _p(llu), _p(de, 0))
    if bad:
        raise RuntimeError(f"unexpected flag on row cell {bad}")
    return System(mm2=mm2, mnoe=mnoe, mno=mno, mno2mn=mno2mn, b=b, de=de, xe=xe, alu=alu,
                  llu=llu, dmax=dmax.value)


@dataclasses.dataclass
class SolveResult:
    x: np.ndarray        # (mnoe,)
    eps: float
    iters: int
    ier: int
    reason: int
    al: np.ndarray       # scaled + sorted AL as left by PCGPME
    ll: np.ndarray
    d: np.ndarray
    b: np.ndarray        # final residual as left by PCGPME


def pcgpme(alu: np.ndarray, llu: np.ndarray, de: np.ndarray, b: np.ndarray, n: int,
           eps: float = 1e-10, parm: float = 5.0, itmax: int = 10000, nthreads: int = 1,
           x0: np.ndarray | None = None) -> SolveResult:
    """Call the restated PCGPME on copies.  ``de``/``b`` are 0-based length >= n;
    ``alu``/``llu`` are (nl, na)."""
    L = lib()
    nl, na = alu.shape
    assert na >= n + 64
    al = np.ascontiguousarray(alu, dtype=np.float64).copy()
    ll = np.ascontiguousarray(llu, dtype=np.int32).copy()
    d = np.ascontiguousarray(de[:n], dtype=np.float64).copy()
    bb = np.ascontiguousarray(b[:n], dtype=np.float64).copy()
    x = np.zeros(na, dtype=np.float64)
    if x0 is not None:
        x[:n] = x0[:n]
    e = np.array([eps, 0.0])
    it = C.c_int(itmax)
    ier = C.c_int(0)
    reason = C.c_int(-1)
    nl_c = C.c_int(nl)
    na_c = C.c_int(na)
    n_c = C.c_int(n)
    n2_c = C.c_int(64)
    parm_c = C.c_double(parm)
    L.ora_pcgpme(_p(al), C.byref(nl_c), C.byref(na_c), _p(ll), _p(d), C.byref(n_c),
                 C.byref(n2_c), _p(bb), _p(x), _p(e), C.byref(parm_c), C.byref(it),
                 C.byref(ier), int(nthreads), C.byref(reason))
    return SolveResult(x=x[:n].copy(), eps=float(e[0]), iters=it.value, ier=ier.value,
                       reason=reason.value, al=al, ll=ll, d=d, b=bb)


def pcgpme_will(al: np.ndarray, ll: np.ndarray, d: np.ndarray, b: np.ndarray, n: int, eps: float = 1e-10,
                parm: float = 5.0, itmax: int = 10000, nthreads: int = 1, n2: int = 64):
    """The restated PCGPME_WILL (pcgpme_2DH.f90:1-374).  al/ll: (nl, na) blocks
    (column k of AL(NA,NL) is row k here), 1-based ll, 0 = none; returns
    (b_out, iterations, stop reason) -- b_out is what the reference leaves in B."""
    L = lib()
    nl, na = al.shape
    a = np.ascontiguousarray(al, dtype=np.float64)
    l_ = np.ascontiguousarray(ll, dtype=np.int32)
    dd = np.ascontiguousarray(d[:n], dtype=np.float64)
    bb = np.ascontiguousarray(b[:n], dtype=np.float64).copy()
    it = C.c_int(0)
    reason = C.c_int(-1)
    L.ora_pcgpme_will(_p(a), nl, na, _p(l_), _p(dd), n, n2, _p(bb), float(eps), float(parm), int(itmax),
                      int(nthreads), C.byref(it), C.byref(reason))
    return bb, it.value, reason.value


def will_postprocess(x: np.ndarray, b: np.ndarray, ll: np.ndarray, n: int):
    """pcgpme_2DH.f90:268-279 alone on copies: returns (x_out, b_out)."""
    L = lib()
    nl, na = ll.shape
    xx = np.ascontiguousarray(x[:n], dtype=np.float64).copy()
    bb = np.ascontiguousarray(b[:n], dtype=np.float64).copy()
    l_ = np.ascontiguousarray(ll, dtype=np.int32)
    L.ora_will_postprocess(_p(xx), _p(bb), _p(l_), nl, na, n)
    return xx, bb


def setup_scaled(alu, llu, de, b, n, parm=5.0):
    """PCGPME's scaling + sort only (pcgpme_para.F90:77-112) on copies."""
    L = lib()
    nl, na = alu.shape
    al = np.ascontiguousarray(alu, dtype=np.float64).copy()
    ll = np.ascontiguousarray(llu, dtype=np.int32).copy()
    d = np.ascontiguousarray(de[:n], dtype=np.float64).copy()
    bb = np.ascontiguousarray(b[:n], dtype=np.float64).copy()
    L.ora_pcgpme_setup(_p(al), nl, na, _p(ll), _p(d), n, _p(bb), parm)
    return al, ll, d, bb


def apply_pm_a(al, ll, d, n, x):
    """Q = PM * A * x on a scaled, sorted matrix (1-based ll, padding included)."""
    L = lib()
    nl, na = al.shape
    xx = np.zeros(n + 64)
    xx[:n] = x[:n]
    y = np.zeros(n + 64)
    L.ora_axsub(_p(al), nl, na, _p(ll), _p(d), n, 64, _p(xx), _p(y))
    L.ora_ldusub(_p(al), nl, na, _p(ll), n, 64, _p(y))
    return y[:n].copy()


def correct(case, cls: Classified, sys_: System, xe: np.ndarray, p: np.ndarray, un: np.ndarray):
    """p -= xe and the velocity correction, in place on p/un copies returned."""
    L = lib()
    p = p.copy()
    un = un.copy()
    xe_full = np.zeros(sys_.mm2 + 1)
    xe_full[1:sys_.mnoe + 1] = xe[:sys_.mnoe]
    L.ora_correct(_p(case.dims), case.inne, case.mx2, _p(case.mn), _p(case.in_), _p(case.jn),
                  _p(case.kn), _p(cls.nf), _p(cls.nfb), _p(case.a), _p(case.dx), case.dt,
                  sys_.mnoe, _p(sys_.mno2mn), _p(sys_.mno), _p(xe_full), _p(p), _p(un))
    return p, un


def transpose(alu, llu, de, n):
    L = lib()
    nl, na = alu.shape
    alt = np.zeros_like(alu)
    llt = np.zeros_like(llu)
    det = np.zeros(n)
    L.ora_transpose(n, na, nl, _p(np.ascontiguousarray(alu)), _p(np.ascontiguousarray(llu)),
                    _p(np.ascontiguousarray(de[:n])), _p(alt), _p(llt), _p(det))
    return alt, llt, det


def spmv(alu, llu, de, n, x):
    L = lib()
    nl, na = alu.shape
    y = np.zeros(n)
    L.ora_spmv(n, na, nl, _p(np.ascontiguousarray(alu)), _p(np.ascontiguousarray(llu)),
               _p(np.ascontiguousarray(de[:n])), _p(np.ascontiguousarray(x[:n], dtype=np.float64)),
               _p(y))
    return y


def prepare(case):
    """Classification, static coefficients, rows, RHS and assembly for one case."""
    cls = set_nflag(case)
    sm = init_matrix(case, cls)
    sy = rows_rhs_assemble(case, cls, sm)
    return cls, sm, sy


def to_csr(sy: System):
    """scipy CSR of the assembled (unscaled) matrix, rows/cols 0-based."""
    import scipy.sparse as sps
    n = sy.mnoe
    rows = [np.arange(n)]
    cols = [np.arange(n)]
    vals = [sy.de[1:n + 1]]
    for d in range(sy.llu.shape[0]):
        c = sy.llu[d, :n]
        m = c != 0
        rows.append(np.nonzero(m)[0])
        cols.append(c[m] - 1)
        vals.append(sy.alu[d, :n][m])
    return sps.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(n, n))
