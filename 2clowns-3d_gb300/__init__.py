"""clowns3d -- GB300 pressure-Poisson solve for 2CLOWNS-3D (host-side mirror).

The compute path is ``libclowns_gpu.so`` (hand-written CUDA for sm_103a, C ABI in
``include/clowns_gpu.h``).  This module binds it with ctypes and mirrors the
reference's call sequence of the pressure-correction loop
(src2LOWNS/1sub-momentum.F90:42-60):

    set_nflag -> init_matrix -> cal_err_of_continuity (rows + RHS)
              -> cal_matrix_element -> PCGPME -> p -= xe, estimate_velocity2

with the same argument meaning and error behaviour.  PyTorch only provides
device memory and the CUDA stream.  There is no CPU fallback: every entry point
raises if the library is missing or no GPU is present.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import pathlib
import threading
from typing import Optional

import numpy as np

from . import workload  # noqa: F401  (re-exported)
from . import ingest  # noqa: F401  (re-exported)

PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG / "libclowns_gpu.so"

IER_MAXITER = 3000
IER_NONFINITE = 9101
IER_DEVICE = 9102
IER_ARG = 9104
STOP_NAMES = {0: "tolerance", 1: "stagnation", 2: "amu_zero", 3: "c1_zero", 4: "iteration_cap",
              5: "non_finite"}

_lock = threading.Lock()
_lib = None


class ClownsError(RuntimeError):
    pass


class SolveInfo(C.Structure):
    _fields_ = [("eps", C.c_double), ("bn", C.c_double), ("iter", C.c_int), ("ier", C.c_int),
                ("reason", C.c_int), ("outer", C.c_int)]

    def as_dict(self):
        return {"eps": self.eps, "bn": self.bn, "iter": self.iter, "ier": self.ier,
                "reason": STOP_NAMES.get(self.reason, str(self.reason)), "outer": self.outer}


def build(verbose: bool = False) -> pathlib.Path:
    from . import buildlib as _b
    return _b.build(verbose=verbose)


_SIGS = {
    "clowns_last_error": (C.c_char_p, []),
    "clowns_version": (C.c_int, []),
    "pcgpme_gpu": (None, [C.c_void_p] * 13),
    "pcgpme_": (None, [C.c_void_p] * 13),
    "clowns_pcgpme_workspace_bytes": (C.c_size_t, [C.c_int, C.c_int]),
    "pcgpme_will_gpu": (C.c_int, [C.c_void_p] * 11),
    "pcgpme_will_": (C.c_int, [C.c_void_p] * 11),
    "clowns_pcgpme_will_workspace_bytes": (C.c_size_t, [C.c_int, C.c_int]),
    "clowns_pcgpme_will_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                         C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_size_t,
                                         C.c_void_p, C.c_void_p]),
    "clowns_will_postprocess_workspace_bytes": (C.c_size_t, [C.c_int]),
    "clowns_will_postprocess_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]),
    "clowns_pcgpme_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                    C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int,
                                    C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    "clowns_pcgpme_setup_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                          C.c_int, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_size_t,
                                          C.c_void_p]),
    "clowns_apply_pm_a_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                        C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                        C.c_void_p]),
    "clowns_pcgpme_mixed_workspace_bytes": (C.c_size_t, [C.c_int, C.c_int]),
    "clowns_pcgpme_mixed_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                          C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                          C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    "clowns_pcgpme_batched_workspace_bytes": (C.c_size_t, [C.c_int, C.c_void_p, C.c_int]),
    "clowns_pcgpme_batched_dev": (C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int,
                                            C.c_double, C.c_int, C.c_int, C.c_void_p, C.c_size_t,
                                            C.c_void_p, C.c_void_p]),
    "clowns_set_nflag_workspace_bytes": (C.c_size_t, [C.c_void_p, C.c_int]),
    "clowns_set_nflag_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 17
                             + [C.c_size_t, C.c_void_p]),
    "clowns_init_matrix_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 14),
    "clowns_rows_rhs_workspace_bytes": (C.c_size_t, [C.c_int]),
    "clowns_rows_rhs_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 12
                            + [C.c_double, C.c_int, C.c_void_p, C.c_int] + [C.c_void_p] * 8
                            + [C.c_size_t, C.c_void_p]),
    "clowns_assemble_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 8
                            + [C.c_int] + [C.c_void_p] * 5 + [C.c_int] + [C.c_void_p] * 5),
    "clowns_pcgpme_static_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                           C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int,
                                           C.c_void_p, C.c_void_p]),
    "clowns_tuned_shape": (C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p]),
    "clowns_last_kernel_launches": (C.c_long, []),
    "clowns_fp64_fma_rate": (C.c_int, [C.c_void_p, C.c_void_p]),
    "clowns_test_arm_wait_timeout": (C.c_int, [C.c_long, C.c_int]),
    "clowns_session_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 7),
    "clowns_session_set_fields": (C.c_int, [C.c_void_p] * 9),
    "clowns_session_classify": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "clowns_session_pressure_loop": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int]
                                     + [C.c_void_p] * 5),
    "clowns_session_get_fields": (C.c_int, [C.c_void_p] * 7),
    "clowns_session_destroy": (C.c_int, [C.c_void_p]),
    "clowns_transpose_dev": (C.c_int, [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 8),
    "clowns_grid_nl": (C.c_int, [C.c_void_p]),
    "clowns_face_grad_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 13),
    "clowns_correct_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 8
                           + [C.c_double, C.c_int] + [C.c_void_p] * 6),
}


def lib():
    """The loaded C-ABI library (raises if it was not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise ClownsError(f"{LIB_PATH.name} is not built; run build() first")
            L = C.CDLL(str(LIB_PATH))
            for name, (res, args) in _SIGS.items():
                fn = getattr(L, name, None)
                if fn is None:
                    continue
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def declared_symbols() -> list[str]:
    """Function names declared in include/clowns_gpu.h."""
    import re
    hdr = (PKG.parent / "include" / "clowns_gpu.h").read_text()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    hdr = "\n".join(ln for ln in hdr.splitlines() if not ln.lstrip().startswith("#"))
    return sorted(set(re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", hdr)))


def last_error() -> str:
    return lib().clowns_last_error().decode(errors="replace")


def _check(rc: int, what: str):
    if rc != 0:
        raise ClownsError(f"{what} failed ({rc}): {last_error()}")


# ---------------------------------------------------------------------------
# Host-array drop-in: same arguments as SUBROUTINE PCGPME

def pcgpme(al: np.ndarray, ll: np.ndarray, d: np.ndarray, b: np.ndarray, x: np.ndarray, n: int,
           eps: float = 1e-10, parm: float = 5.0, itmax: int = 10000):
    """Solve through ``pcgpme_gpu`` with HOST arrays (the Fortran call shape).

    ``al``/``ll`` are (nl, na) C-order == AL(NA,NL) column-major; ``d``, ``b``
    hold rows 1..n at [0..n); ``x`` is X(N+N2), updated in place.
    Returns (eps_out, iter_out, ier)."""
    L = lib()
    nl, na = al.shape
    assert al.dtype == np.float64 and ll.dtype == np.int32 and al.flags.c_contiguous
    e = np.array([eps, 0.0])
    c_nl, c_na, c_n, c_n2 = C.c_int(nl), C.c_int(na), C.c_int(n), C.c_int(64)
    c_parm = C.c_double(parm)
    c_it = C.c_int(itmax)
    c_ier = C.c_int(0)
    L.pcgpme_gpu(al.ctypes.data, C.addressof(c_nl), C.addressof(c_na), ll.ctypes.data, d.ctypes.data,
                 C.addressof(c_n), C.addressof(c_n2), b.ctypes.data, x.ctypes.data, e.ctypes.data,
                 C.addressof(c_parm), C.addressof(c_it), C.addressof(c_ier))
    return float(e[0]), c_it.value, c_ier.value


def pcgpme_will(al: np.ndarray, ll: np.ndarray, d: np.ndarray, b: np.ndarray, n: int, eps: float = 1e-10,
                parm: float = 5.0, itmax: int = 10000, n2: int = 64) -> np.ndarray:
    """PCGPME_WILL (the 2DH solve) through ``pcgpme_will_gpu`` with HOST arrays.
    ``al``/``ll``: (nl, na) C-order == AL(NA,NL); ``b`` (rows 1..n at [0..n)) is
    the right-hand side and is overwritten with what the reference leaves in B."""
    L = lib()
    nl, na = al.shape
    assert al.dtype == np.float64 and ll.dtype == np.int32 and al.flags.c_contiguous and ll.flags.c_contiguous
    assert b.dtype == np.float64 and b.flags.c_contiguous
    c_nl, c_na, c_n, c_n2, c_it = C.c_int(nl), C.c_int(na), C.c_int(n), C.c_int(n2), C.c_int(itmax)
    c_eps, c_parm = C.c_double(eps), C.c_double(parm)
    d = np.ascontiguousarray(d, dtype=np.float64)
    rc = L.pcgpme_will_gpu(al.ctypes.data, C.addressof(c_nl), C.addressof(c_na), ll.ctypes.data, d.ctypes.data,
                           C.addressof(c_n), C.addressof(c_n2), b.ctypes.data, C.addressof(c_eps),
                           C.addressof(c_parm), C.addressof(c_it))
    _check(rc, "pcgpme_will_gpu")
    return b


# ---------------------------------------------------------------------------
# Device-resident pipeline (torch tensors as device memory)

def _torch():
    import torch
    if not torch.cuda.is_available():
        raise ClownsError("no CUDA device: the GPU path has no CPU fallback")
    return torch


def _ptr(t) -> int:
    return t.data_ptr()


def _stream():
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclasses.dataclass
class DeviceCase:
    """Module arrays of one case resident in HBM."""
    case: object
    dims: object
    x: object
    dx: object
    mn: object
    in_: object
    jn: object
    kn: object
    nf: object
    nfb: object
    f: object
    fb: object
    a: object
    un: object
    sp: object
    objno: object

    @staticmethod
    def upload(case, device="cuda"):
        torch = _torch()

        def t(a):
            return torch.from_numpy(np.ascontiguousarray(a)).to(device)
        return DeviceCase(case=case, dims=torch.from_numpy(case.dims.copy()), x=t(case.x), dx=t(case.dx),
                          mn=t(case.mn), in_=t(case.in_), jn=t(case.jn), kn=t(case.kn), nf=t(case.nf),
                          nfb=t(case.nfb), f=t(case.f), fb=t(case.fb), a=t(case.a), un=t(case.un),
                          sp=t(case.sp), objno=t(case.objno))


@dataclasses.dataclass
class DeviceSystem:
    """Everything the pressure-correction loop builds on the device."""
    ifln: int
    isfn: int
    passes: int
    fln: object          # int32 (ifln,) == fln(1:ifln)
    sfn: object
    mp: object           # f64 (1,)
    alu_c: object        # (nl, inne)
    ll_c: object
    de_c: object
    mm2: int
    mnoe: int
    dmax: float
    mno: object          # (je, ke, ie)
    mno2mn: object       # (mm2,) == mno2mn(1:mm2)
    b: object            # (mm2,) == b(1:mm2)
    xe: object           # (mm2+1,) == xe(0:mm2)
    de: object           # (mm2,)
    alu: object          # (nl, mm2)
    llu: object          # (nl, mm2)


def set_nflag_dev(dc: DeviceCase):
    torch = _torch()
    L = lib()
    case = dc.case
    ncell = case.inne2 + 2
    fln = torch.zeros(ncell + 1, dtype=torch.int32, device="cuda")
    sfn = torch.zeros(ncell + 1, dtype=torch.int32, device="cuda")
    wbytes = L.clowns_set_nflag_workspace_bytes(dc.dims.numpy().ctypes.data, case.inne2)
    work = torch.empty(max(1, wbytes), dtype=torch.uint8, device="cuda")
    ifln, isfn, passes = C.c_int(0), C.c_int(0), C.c_int(0)
    dims = dc.dims.numpy()
    rc = L.clowns_set_nflag_dev(dims.ctypes.data, case.inne, case.inne2, case.mx2, _ptr(dc.mn), _ptr(dc.in_),
                                _ptr(dc.jn), _ptr(dc.kn), _ptr(dc.nf), _ptr(dc.nfb), _ptr(dc.f), _ptr(dc.fb),
                                _ptr(dc.a), _ptr(dc.dx), _ptr(dc.objno), _ptr(fln), C.byref(ifln), _ptr(sfn),
                                C.byref(isfn), C.byref(passes), _ptr(work), wbytes, _stream())
    _check(rc, "set_nflag")
    return fln[:ifln.value], ifln.value, sfn[:isfn.value], isfn.value, passes.value


def grid_nl(dims) -> int:
    """Matrix columns of a grid: 6 (3D), 4 (2DV: one cell wide in x or y) or 0
    (one cell wide in both, or invalid bounds)."""
    d = np.ascontiguousarray(dims, dtype=np.int32)
    return int(lib().clowns_grid_nl(d.ctypes.data))


def init_matrix_dev(dc: DeviceCase):
    torch = _torch()
    L = lib()
    case = dc.case
    nl = grid_nl(case.dims)
    if nl == 0:
        raise ClownsError("init_matrix: a grid one cell wide in both x and y has no matrix form")
    mp = torch.zeros(1, dtype=torch.float64, device="cuda")
    alu_c = torch.empty((nl, case.inne), dtype=torch.float64, device="cuda")
    ll_c = torch.empty((nl, case.inne), dtype=torch.int32, device="cuda")
    de_c = torch.empty(case.inne, dtype=torch.float64, device="cuda")
    dims = dc.dims.numpy()
    rc = L.clowns_init_matrix_dev(dims.ctypes.data, case.inne, case.mx2, _ptr(dc.mn), _ptr(dc.in_), _ptr(dc.jn),
                                  _ptr(dc.kn), _ptr(dc.nf), _ptr(dc.nfb), _ptr(dc.a), _ptr(dc.fb), _ptr(dc.dx),
                                  _ptr(mp), _ptr(alu_c), _ptr(ll_c), _ptr(de_c), _stream())
    _check(rc, "init_matrix")
    return mp, alu_c, ll_c, de_c


def rows_rhs_assemble_dev(dc: DeviceCase, fln, ifln: int, mp, alu_c, ll_c, de_c, mm2: Optional[int] = None):
    torch = _torch()
    L = lib()
    case = dc.case
    if mm2 is None:
        mm2 = ifln + 5000                       # m_alloc = ifln + 5000 (1sub-momentum.F90:254)
    is_, js, ks, ie, je, ke = (int(v) for v in case.dims)
    dims = dc.dims.numpy()
    mno = torch.empty((je, ke, ie), dtype=torch.int32, device="cuda")
    mno2mn = torch.zeros(mm2, dtype=torch.int32, device="cuda")
    b = torch.empty(mm2, dtype=torch.float64, device="cuda")
    xe = torch.zeros(mm2 + 1, dtype=torch.float64, device="cuda")
    de = torch.empty(mm2, dtype=torch.float64, device="cuda")
    wbytes = L.clowns_rows_rhs_workspace_bytes(ifln)
    work = torch.empty(max(1, wbytes), dtype=torch.uint8, device="cuda")
    mnoe = C.c_int(0)
    dmax = C.c_double(0.0)
    flnp = _ptr(fln) if ifln > 0 else _ptr(mno2mn)
    rc = L.clowns_rows_rhs_dev(dims.ctypes.data, case.inne2, case.mx2, _ptr(dc.mn), _ptr(dc.in_), _ptr(dc.jn),
                               _ptr(dc.kn), _ptr(dc.nf), _ptr(dc.nfb), _ptr(dc.f), _ptr(dc.fb), _ptr(dc.a),
                               _ptr(dc.un), _ptr(dc.dx), _ptr(mp), case.dt, ifln, flnp, mm2, _ptr(mno),
                               _ptr(mno2mn), _ptr(b), _ptr(xe) + 8, _ptr(de), C.byref(mnoe), C.byref(dmax),
                               _ptr(work), wbytes, _stream())
    _check(rc, "rows_rhs")
    nl = alu_c.shape[0]
    alu = torch.zeros((nl, mm2), dtype=torch.float64, device="cuda")
    llu = torch.zeros((nl, mm2), dtype=torch.int32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.clowns_assemble_dev(dims.ctypes.data, case.inne, case.inne2, case.mx2, _ptr(dc.in_), _ptr(dc.jn),
                               _ptr(dc.kn), _ptr(dc.nf), _ptr(dc.nfb), _ptr(dc.x), _ptr(dc.dx), _ptr(dc.sp),
                               ifln, flnp, _ptr(mno), _ptr(alu_c), _ptr(ll_c), _ptr(de_c), mm2, _ptr(alu),
                               _ptr(llu), _ptr(de), _ptr(err), _stream())
    _check(rc, "assemble")
    bad = int(err.item())
    if bad:
        raise ClownsError(f"cal_matrix_element: unexpected flag on row cell {bad}")
    return dict(mm2=mm2, mnoe=mnoe.value, dmax=dmax.value, mno=mno, mno2mn=mno2mn, b=b, xe=xe, de=de,
                alu=alu, llu=llu)


def prepare_dev(case) -> tuple[DeviceCase, DeviceSystem]:
    """Upload a case and run classification, static coefficients, rows, RHS and
    assembly on the GPU."""
    dc = DeviceCase.upload(case)
    fln, ifln, sfn, isfn, passes = set_nflag_dev(dc)
    mp, alu_c, ll_c, de_c = init_matrix_dev(dc)
    r = rows_rhs_assemble_dev(dc, fln, ifln, mp, alu_c, ll_c, de_c)
    sy = DeviceSystem(ifln=ifln, isfn=isfn, passes=passes, fln=fln, sfn=sfn, mp=mp, alu_c=alu_c, ll_c=ll_c,
                      de_c=de_c, **r)
    return dc, sy


PREC_FP64 = 0
PREC_MIXED = 1


def tuned_shape(sizes, precision=0):
    """Execution the autotuner chose for the iteration loop of this row space:
    {"mode": "graph", "block": .., "fused_sweeps": .., "reduce_block": ..,
    "balanced_rows": 0 | 4 | 8, "staged_axsub": ..} (balanced_rows > 0: one-wave
    kernels over even row ranges, that many rows per thread per step;
    staged_axsub: the FP32 AXSUB with its streams staged by bulk copies) or
    {"mode": "persistent" | "wave", "block": .., "grid": .., "registers": ..},
    or None before a solve of that size has run."""
    L = lib()
    arr = (C.c_int * len(sizes))(*[int(v) for v in sizes])
    mo, b, g, r, f = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0)
    if L.clowns_tuned_shape(len(sizes), arr, precision, C.byref(mo), C.byref(b), C.byref(g), C.byref(r),
                            C.byref(f)) != 0:
        return None
    if mo.value == 1:
        bal = (8 if f.value & 8 else 4) if f.value & 4 else 0
        return {"mode": "graph", "block": 256 if bal else b.value, "fused_sweeps": bool(f.value & 1),
                "reduce_block": 64 if f.value & 2 else (256 if bal else b.value), "balanced_rows": bal,
                "staged_axsub": bool(f.value & 16)}
    return {"mode": {0: "persistent", 3: "wave"}.get(mo.value, str(mo.value)), "block": b.value,
            "grid": g.value, "registers": r.value}


def last_kernel_launches():
    """Kernels the calling thread's last solve launched (host launches plus the
    kernel nodes executed inside loop graphs)."""
    return int(lib().clowns_last_kernel_launches())


def fp64_fma_rate(stream=None):
    """Measured FP64 fused multiply-add rate of the current device (lane
    operations per second): the ceiling of the FP64 solve's arithmetic."""
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    out = C.c_double(0.0)
    _check(lib().clowns_fp64_fma_rate(C.byref(out), C.c_void_p(s.cuda_stream)), "fp64_fma_rate")
    return out.value


class Member(C.Structure):
    """clowns_member: one system of an ensemble (device pointers)."""
    _fields_ = [("al", C.c_void_p), ("ll", C.c_void_p), ("d", C.c_void_p), ("b", C.c_void_p),
                ("x", C.c_void_p), ("na", C.c_int), ("n", C.c_int), ("nl", C.c_int), ("pad", C.c_int)]


class MixedSolver:
    """FP32-storage BiCGSTAB with FP64 iterative refinement (one system)."""

    def __init__(self, n: int, nl: int = 6):
        torch = _torch()
        L = lib()
        self.n = n
        self.wbytes = L.clowns_pcgpme_mixed_workspace_bytes(n, nl)
        self.work = torch.empty(self.wbytes, dtype=torch.uint8, device="cuda")

    def solve(self, alu, llu, de, b, x, eps: float = 1e-10, parm: float = 5.0, inner_tol: float = 0.0,
              inner_max: int = 0, max_outer: int = 0) -> SolveInfo:
        L = lib()
        nl, na = alu.shape
        info = SolveInfo()
        rc = L.clowns_pcgpme_mixed_dev(_ptr(alu), nl, na, _ptr(llu), _ptr(de), self.n, _ptr(b), _ptr(x), eps,
                                       parm, inner_tol, inner_max, max_outer, _ptr(self.work), self.wbytes,
                                       _stream(), C.byref(info))
        _check(rc, "pcgpme_mixed_dev")
        return info


class BatchedSolver:
    """Ensemble of independent systems solved together (FP64 or mixed)."""

    def __init__(self, sizes, precision: int = PREC_MIXED):
        torch = _torch()
        L = lib()
        self.sizes = [int(v) for v in sizes]
        self.precision = precision
        arr = (C.c_int * len(self.sizes))(*self.sizes)
        self.wbytes = L.clowns_pcgpme_batched_workspace_bytes(len(self.sizes), arr, precision)
        self.work = torch.empty(self.wbytes, dtype=torch.uint8, device="cuda")

    def solve(self, systems, xs, eps: float = 1e-10, parm: float = 5.0, itmax: int = 10000,
              inner_tol: float = 0.0, inner_max: int = 0, max_outer: int = 0):
        """systems: list of (alu, llu, de, b) device tensors; xs: list of x tensors."""
        L = lib()
        M = len(systems)
        mem = (Member * M)()
        for m, ((alu, llu, de, b), x) in enumerate(zip(systems, xs)):
            nl, na = alu.shape
            mem[m] = Member(_ptr(alu), _ptr(llu), _ptr(de), _ptr(b), _ptr(x), na, self.sizes[m], nl, 0)
        infos = (SolveInfo * M)()
        rc = L.clowns_pcgpme_batched_dev(M, mem, self.precision, eps, parm, itmax, inner_tol, inner_max,
                                         max_outer, _ptr(self.work), self.wbytes, _stream(), infos)
        _check(rc, "pcgpme_batched_dev")
        return list(infos)


class Solver:
    """Device-resident PCGPME with a persistent workspace (one per size)."""

    def __init__(self, n: int, nl: int = 6):
        torch = _torch()
        L = lib()
        self.n = n
        self.nl = nl
        self.wbytes = L.clowns_pcgpme_workspace_bytes(n, nl)
        self.work = torch.empty(self.wbytes, dtype=torch.uint8, device="cuda")

    def solve(self, alu, llu, de, b, x, eps: float = 1e-10, parm: float = 5.0, itmax: int = 10000,
              stream=None) -> SolveInfo:
        """alu/llu: (nl, na) device tensors; de/b: >= n; x: >= n (in/out)."""
        L = lib()
        nl, na = alu.shape
        info = SolveInfo()
        st = C.c_void_p(stream) if stream is not None else _stream()
        rc = L.clowns_pcgpme_dev(_ptr(alu), nl, na, _ptr(llu), _ptr(de), self.n, _ptr(b), _ptr(x), eps, parm,
                                 itmax, _ptr(self.work), self.wbytes, st, C.byref(info))
        _check(rc, "pcgpme_dev")
        return info


def setup_scaled_dev(alu, llu, de, b, n: int, parm: float = 5.0):
    """Scaling + per-row sort only (test hook): returns al_s, ll_s (0-based), d_s, b_s."""
    torch = _torch()
    L = lib()
    nl, na = alu.shape
    al_s = torch.zeros((nl, n), dtype=torch.float64, device="cuda")
    ll_s = torch.zeros((nl, n), dtype=torch.int32, device="cuda")
    d_s = torch.zeros(n, dtype=torch.float64, device="cuda")
    b_s = torch.zeros(n, dtype=torch.float64, device="cuda")
    wbytes = L.clowns_pcgpme_workspace_bytes(n, nl)
    work = torch.empty(wbytes, dtype=torch.uint8, device="cuda")
    rc = L.clowns_pcgpme_setup_dev(_ptr(alu), nl, na, _ptr(llu), _ptr(de), n, _ptr(b), parm, _ptr(al_s),
                                   _ptr(ll_s), _ptr(d_s), _ptr(b_s), n, _ptr(work), wbytes, _stream())
    _check(rc, "pcgpme_setup")
    return al_s, ll_s, d_s, b_s


def apply_pm_a_dev(alu, llu, de, n: int, x, parm: float = 5.0):
    """y = PM (W A) x with the scaled, sorted operator built from the assembled matrix."""
    torch = _torch()
    L = lib()
    nl, na = alu.shape
    y = torch.zeros(n, dtype=torch.float64, device="cuda")
    wbytes = L.clowns_pcgpme_workspace_bytes(n, nl)
    work = torch.empty(wbytes, dtype=torch.uint8, device="cuda")
    rc = L.clowns_apply_pm_a_dev(_ptr(alu), nl, na, _ptr(llu), _ptr(de), n, parm, _ptr(x), _ptr(y), _ptr(work),
                                 wbytes, _stream())
    _check(rc, "apply_pm_a")
    return y


def correct_dev(dc: DeviceCase, sy: DeviceSystem, x, p, un):
    """p -= xe ; estimate_velocity2 with xe = x (rows 1..mnoe)."""
    L = lib()
    case = dc.case
    sy.xe.zero_()
    sy.xe[1:sy.mnoe + 1] = x[:sy.mnoe]
    dims = dc.dims.numpy()
    rc = L.clowns_correct_dev(dims.ctypes.data, case.inne, case.mx2, _ptr(dc.mn), _ptr(dc.in_), _ptr(dc.jn),
                              _ptr(dc.kn), _ptr(dc.nf), _ptr(dc.nfb), _ptr(dc.a), _ptr(dc.dx), case.dt, sy.mnoe,
                              _ptr(sy.mno2mn), _ptr(sy.mno), _ptr(sy.xe), _ptr(p), _ptr(un), _stream())
    _check(rc, "correct")


# ---------------------------------------------------------------------------
# Adjoint

def transpose_dev(alu, llu, de, n: int):
    """Explicit A^T of an assembled ELL matrix (device tensors, 1-based llu)."""
    torch = _torch()
    L = lib()
    nl, na = alu.shape
    alt = torch.empty_like(alu)
    llt = torch.empty_like(llu)
    det = torch.zeros_like(de)
    bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.clowns_transpose_dev(n, na, nl, _ptr(alu), _ptr(llu), _ptr(de), _ptr(alt), _ptr(llt), _ptr(det),
                                _ptr(bad), _stream())
    _check(rc, "transpose")
    if int(bad.item()):
        raise ClownsError("transpose: column index out of range")
    return alt, llt, det


def face_grad_dev(dc: DeviceCase, sy: DeviceSystem, x, lam):
    """dJ/da for the face area fractions, layout of a (inne2+2, 3)."""
    torch = _torch()
    L = lib()
    case = dc.case
    grad = torch.zeros_like(dc.a)
    dims = dc.dims.numpy()
    flnp = _ptr(sy.fln) if sy.ifln > 0 else _ptr(grad)
    rc = L.clowns_face_grad_dev(dims.ctypes.data, case.inne, case.inne2, sy.ifln, flnp, _ptr(dc.in_), _ptr(dc.jn),
                                _ptr(dc.kn), _ptr(dc.nf), _ptr(sy.mno), _ptr(sy.alu_c), _ptr(sy.ll_c), _ptr(dc.a),
                                _ptr(x), _ptr(lam), _ptr(grad), _stream())
    _check(rc, "face_grad")
    return grad


def adjoint_dev(dc: DeviceCase, sy: DeviceSystem, x, djdx, eps: float = 1e-12, solver=None):
    """Solve A^T lambda = dJ/dx (PCGPME on the explicit transpose, FP64) and form
    (dJ/db, dJ/da) = (lambda, face gradient)."""
    torch = _torch()
    n = sy.mnoe
    alt, llt, det = transpose_dev(sy.alu, sy.llu, sy.de, n)
    lam = torch.zeros(sy.mm2, dtype=torch.float64, device="cuda")
    rhs = torch.zeros(sy.mm2, dtype=torch.float64, device="cuda")
    rhs[:n] = djdx[:n]
    solver = solver or Solver(n)
    info = solver.solve(alt, llt, det, rhs, lam, eps=eps)
    grad_a = face_grad_dev(dc, sy, x, lam)
    return lam[:n], grad_a, info


# ---------------------------------------------------------------------------
# Device-resident ik loop

class Session:
    """The pressure-correction ik loop of one domain with its arrays in HBM."""

    def __init__(self, case):
        L = lib()
        self.case = case
        self.h = C.c_void_p()
        c = case
        self._keep = [np.ascontiguousarray(v) for v in (c.dims, c.mn, c.in_, c.jn, c.kn, c.x, c.dx, c.objno)]
        d, mn, in_, jn, kn, x, dx, ob = self._keep
        _check(L.clowns_session_create(C.byref(self.h), d.ctypes.data, c.inne, c.inne2, c.mx2, mn.ctypes.data,
                                       in_.ctypes.data, jn.ctypes.data, kn.ctypes.data, x.ctypes.data,
                                       dx.ctypes.data, ob.ctypes.data), "session_create")

    def set_fields(self, nf, nfb, f, fb, a, un, sp, p):
        arrs = [np.ascontiguousarray(v) for v in (nf, nfb, f, fb, a, un, sp, p)]
        _check(lib().clowns_session_set_fields(self.h, *[v.ctypes.data for v in arrs]), "session_set_fields")

    def classify(self):
        ifln, isfn = C.c_int(0), C.c_int(0)
        _check(lib().clowns_session_classify(self.h, C.byref(ifln), C.byref(isfn)), "session_classify")
        return ifln.value, isfn.value

    def pressure_loop(self, dt, d0=1e-5, eps0=1e-10, precision=PREC_FP64):
        ik, dmax, it, err, icon = C.c_int(0), C.c_double(0), C.c_int(0), C.c_double(0), C.c_int(0)
        _check(lib().clowns_session_pressure_loop(self.h, dt, d0, eps0, precision, C.byref(ik), C.byref(dmax),
                                                  C.byref(it), C.byref(err), C.byref(icon)), "pressure_loop")
        return {"ik": ik.value, "dmax": dmax.value, "iter": it.value, "err": err.value, "icon": icon.value}

    def fields(self):
        nc = self.case.inne2 + 2
        nf = np.zeros(nc, np.int32)
        nfb = np.zeros(nc, np.int32)
        f = np.zeros(nc)
        p = np.zeros(nc)
        un = np.zeros((nc, 3))
        mnoe = C.c_int(0)
        _check(lib().clowns_session_get_fields(self.h, nf.ctypes.data, nfb.ctypes.data, f.ctypes.data,
                                               p.ctypes.data, un.ctypes.data, C.byref(mnoe)), "get_fields")
        return {"nf": nf, "nfb": nfb, "f": f, "p": p, "un": un, "mnoe": mnoe.value}

    def close(self):
        if self.h:
            lib().clowns_session_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class WillSolver:
    """Device-resident PCGPME_WILL (the 2DH dispersion solve) of one size."""

    def __init__(self, n: int, nl: int = 4):
        torch = _torch()
        self.n, self.nl = n, nl
        self.bytes = int(lib().clowns_pcgpme_will_workspace_bytes(n, nl))
        self.work = torch.empty(max(self.bytes, 1), dtype=torch.uint8, device="cuda")

    def solve(self, al, ll, d, b, eps: float = 1e-10, parm: float = 5.0, itmax: int = 10000) -> SolveInfo:
        """al/ll: (nl, na) device tensors; b (device, >= n) is overwritten with
        the reference's B output."""
        info = SolveInfo()
        nl, na = al.shape
        rc = lib().clowns_pcgpme_will_dev(_ptr(al), nl, na, _ptr(ll), _ptr(d), self.n, _ptr(b), eps, parm, itmax,
                                          _ptr(self.work), self.bytes, _stream(), C.byref(info))
        _check(rc, "clowns_pcgpme_will_dev")
        return info


def will_postprocess_dev(x, r, ll, n: int):
    """The post-processing of pcgpme_2DH.f90:268-279 on device vectors x, r
    (ll: (nl, na) device tensor); returns (x_out, b) device tensors."""
    torch = _torch()
    nl, na = ll.shape
    b = torch.empty(n, dtype=torch.float64, device="cuda")
    xo = torch.empty(n, dtype=torch.float64, device="cuda")
    nb = int(lib().clowns_will_postprocess_workspace_bytes(n))
    work = torch.empty(nb, dtype=torch.uint8, device="cuda")
    rc = lib().clowns_will_postprocess_dev(_ptr(x), _ptr(r), _ptr(ll), nl, na, n, _ptr(b), _ptr(xo), _ptr(work), nb,
                                           _stream())
    _check(rc, "clowns_will_postprocess_dev")
    return xo, b
