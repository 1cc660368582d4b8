"""Run the reference's own Fortran routines on seeded cases and record their
outputs in tests/golden/reference_runs.json.

The reference builds only with ifort (src2LOWNS/Makefile:1,5) and no Fortran
compiler exists here, so its source files are executed through
tests/golden/fortran_exec.py, which translates the Fortran they use to Python
in memory (never stored) with the build's macros (Makefile:5: -DRAN -DNORMAL
-DOBJECT -DSLIDE0, -r8) and one OpenMP thread.  The routines run are the
reference's own, chained as the model chains them:

  set_nflag              src2LOWNS/nfd2015.F90:7-306 (fxx1 308-332), from the raw flags
  init_matrix            src2LOWNS/1sub-matrix.F90:3-95
  cal_err_of_continuity  src2LOWNS/1sub-momentum.F90:235-417 (renzoku_n 1sub-main.F90:579-602,
                         renzoku_fv lib/src/math_func.F90:51-54, alloc_matrix 0mod-arrays.F90:356-370)
  cal_matrix_element     src2LOWNS/1sub-momentum.F90:465-551
  cal_poisson_equation   src2LOWNS/1sub-momentum.F90:553-588 -> PCGPME, pcgpme_para.F90:1-353
  the ik loop            src2LOWNS/1sub-momentum.F90:41-60 (check_dmax 419-463, p -= xe,
                         estimate_velocity2 590-651, momentum_d math_func.F90:251-255)
  PCGPME_WILL            src2LOWNS/pcgpme_2DH.f90:1-373
  read_data's numbering  src2LOWNS/data_io.F90:168-202 and 255-277 (the statements between the
                         file reads, on flag grids; alloc_dxdydz 0mod-arrays.F90:196-216)
  set_dx                 src2LOWNS/1sub-main.F90:53-74 (round lib/src/xy_calc.f90:100-112)
  the case readers       read_data, read_fdata, read_nsdata (src2LOWNS/data_io.F90:87-397, owari and
                         hajime lib/src/owari.f) on the files ingest.write_case writes, then set_dx
  the grid generator's   output_xyzn / output_xyz, output_data, output_fdata, output_nsdata
  writers                (srcMakeGrid/data_io.F90:639-651, 707-820, 875-897, 1505-1555)

The module constants come from the reference's module files (0mod-variables.F90);
the case data fill the module arrays in the bounds the reference allocates them
with (0mod-arrays.F90:205-237, 290, 356-370); lf is the identity
(main_2CLOWNS.F90:33) and dim3d follows main_2CLOWNS.F90:43-44.

Digests (sha256 of each output's bytes) and scalars are written to the JSON
file, and the solution vectors (pressures, PCGPME_WILL's B, the ik loop's
pressure and face velocities) to tests/golden/reference_solutions.npz; the cases are rebuilt from the seeded
generator by tests/golden/reference_cases.py.  tests/test_oracle_reference_runs.py
checks the oracle against these outputs bit for bit, and
tests/test_gpu_reference_runs.py the CUDA path (bit for bit, and the solves
within their tolerance).  The reference is read from REFERENCE_ROOT (default /root/reference).

Usage:  python tests/golden/make_ref_golden.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import json
import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))

import fortran_exec as fx  # noqa: E402
import reference_cases as rc  # noqa: E402

DEFINES = {"RAN", "NORMAL", "OBJECT", "SLIDE0"}
GRID_SOURCES = ["src2LOWNS/0mod-type_interface.F90", "src2LOWNS/0mod-variables.F90",
                "src2LOWNS/0mod-arrays.F90", "src2LOWNS/nfd2015.F90", "src2LOWNS/1sub-matrix.F90",
                "src2LOWNS/1sub-momentum.F90", "src2LOWNS/1sub-main.F90", "lib/src/math_func.F90",
                "lib/src/xy_calc.f90", "src2LOWNS/pcgpme_para.F90"]
WILL_SOURCES = ["src2LOWNS/0mod-type_interface.F90", "src2LOWNS/0mod-variables.F90",
                "src2LOWNS/pcgpme_2DH.f90"]
# cal_err_of_continuity reads its local k, set only by the numbering branch of
# the first ik pass, on later passes too (1sub-momentum.F90:352), where it only
# chooses DMAX1, which nothing reads; 0 stands in for the undefined value.
UNDEFINED = {("cal_err_of_continuity", "k"): 0}


def allocate_matrix(prog, V, A):
    """The allocation cal_err_of_continuity makes on the first ik pass
    (1sub-momentum.F90:253-255: m_alloc = ifln + 5000, alloc_matrix), done
    before it so that xe(0) can be given a value: estimate_velocity2 reads
    xe(0) for a cell or neighbour without a matrix row (mno = 0,
    1sub-momentum.F90:606, 617, 632, 640), an element nothing writes; the
    memory ALLOCATE hands out fresh is zero, and 0 stands in for it."""
    V.f_m_alloc = V.f_ifln + 5000
    prog.call("alloc_matrix", V.f_m_alloc, V.f_ie, V.f_je, V.f_ke)
    A.f_xe[0] = 0.0


class CellFlag:
    """type(cellflag) (0mod-type_interface.F90:7-9)."""

    __slots__ = ("f_f", "f_b", "f_fp", "f_bp")

    def __init__(self, f, b):
        self.f_f, self.f_b, self.f_fp, self.f_bp = f, b, None, None


def farray(kind, values, bounds):
    lb = [lo for lo, _ in bounds]
    ext = [hi - lo + 1 for lo, hi in bounds]
    conv = {"real": float, "int": int}.get(kind, lambda v: v)
    vals = [conv(v) for v in values]
    n = int(np.prod(ext))
    if len(vals) != n:
        raise ValueError(f"{len(vals)} values for {n} elements")
    return fx.FArray(vals, 0, lb, ext, kind)


def program(root: pathlib.Path, sources):
    texts = [(root / f).read_text(encoding="latin-1") for f in sources]
    return fx.Program(texts, DEFINES, undefined=UNDEFINED)


def load_grid(prog, case):
    """Module state of one domain before set_nflag, from the case's raw flags."""
    V, A = prog.module("variables"), prog.module("arrays")
    is_, js, ks, ie, je, ke = (int(v) for v in case.dims)
    V.f_is, V.f_js, V.f_ks, V.f_ie, V.f_je, V.f_ke = is_, js, ks, ie, je, ke
    V.f_inns, V.f_inne, V.f_inne2 = 1, int(case.inne), int(case.inne2)
    V.f_dt, V.f_eps0 = float(case.dt), float(case.eps0)
    V.f_ik, V.f_m_alloc, V.f_n, V.f_t, V.f_icon, V.f_ricon = 0, 0, 1, 0.0, 0, 0
    V.f_isfn, V.f_isfn2, V.f_ifln = 0, 0, 0
    m2 = int(case.inne2) + 1
    A.f_lf = farray("int", [1 if r == c else 0 for c in range(3) for r in range(3)], [(0, 2), (0, 2)])
    A.f_dim3d = not (is_ == ie - 1 or js == je - 1)
    for nm, arr in (("in", case.in_), ("jn", case.jn), ("kn", case.kn)):
        setattr(A, "f_" + nm, farray("int", arr[1:m2 + 1], [(1, m2)]))
    A.f_nff = farray("obj", [CellFlag(int(f), int(b)) for f, b in zip(case.nf, case.nfb)], [(0, m2)])
    A.f_fb = farray("real", case.fb, [(0, m2)])
    A.f_f = farray("real", case.f, [(0, m2)])
    A.f_a = farray("real", case.a.ravel(), [(0, 2), (0, m2)])
    A.f_un = farray("real", case.un.ravel(), [(0, 2), (0, m2)])
    A.f_dx = farray("real", case.dx.ravel(), [(0, 2), (1, case.mx2)])
    A.f_x = farray("real", case.x.ravel(), [(0, 2), (1, case.mx2)])
    A.f_mn = farray("int", case.mn.ravel(), [(is_ - 2, ie + 2), (ks - 2, ke + 2), (js - 2, je + 2)])
    A.f_sp = farray("real", case.sp.ravel(), [(0, m2), (0, 2)])
    A.f_objno = farray("int", case.objno, [(0, m2)])
    A.f_fln = farray("int", [0] * (m2 + 1), [(1, m2 + 1)])
    A.f_sfn = farray("int", [0] * (m2 + 1), [(1, m2 + 1)])
    A.f_p = farray("real", [0.0] * (m2 + 1), [(0, m2)])
    return V, A


def vals(a):
    return np.array(a.values())


SOLUTIONS = {}     # label/x (pressure) and label/b (PCGPME_WILL's B): values, for tolerance checks


def run_grid(root, label, case, solve: bool, loop: bool) -> dict:
    d = rc.digest
    out = {"input": rc.case_digest(case), "label": label}
    prog = program(root, GRID_SOURCES)
    V, A = load_grid(prog, case)
    prog.call("set_nflag")
    nff = A.f_nff.values()
    ifln, isfn = V.f_ifln, V.f_isfn
    out["nflag"] = {"nf": d(np.array([o.f_f for o in nff])), "nfb": d(np.array([o.f_b for o in nff])),
                    "f": d(vals(A.f_f)), "ifln": ifln, "fln": d(vals(A.f_fln)[:ifln]), "isfn": isfn,
                    "sfn": d(vals(A.f_sfn)[:isfn])}
    prog.call("init_matrix")
    allocate_matrix(prog, V, A)
    nl, inne = V.f_nl, V.f_inne
    de_c = vals(A.f_de_c)
    alu_c = vals(A.f_alu_c).reshape(nl, inne)
    ll_c = np.array([-1 if v is None else v for v in A.f_ll_c.values()]).reshape(nl, inne)
    # rows init_matrix skips (objects, fb = 0: 1sub-matrix.F90:26) stay undefined in the reference
    undefined = np.isnan(de_c)
    if not np.array_equal(np.isnan(alu_c).any(axis=0), undefined):
        raise RuntimeError("init_matrix left part of a row undefined")
    rows = ~undefined
    out["init"] = {"nl": nl, "mp": V.f_mp, "undefined_rows": rc.runs(np.flatnonzero(undefined) + 1),
                   "alu_c": d(alu_c[:, rows]), "ll_c": d(ll_c[:, rows]), "de_c": d(de_c[rows])}
    prog.call("cal_err_of_continuity")
    mnoe, mm2 = V.f_mnoe, V.f_mm2
    out["rows"] = {"mnoe": mnoe, "mm2": mm2, "dmax": V.f_dmax, "mno": d(vals(A.f_mno)),
                   "mno2mn": d(vals(A.f_mno2mn)[:mnoe]), "b": d(vals(A.f_b)[:mnoe])}
    prog.call("cal_matrix_element")
    out["asm"] = {"alu": d(vals(A.f_alu).reshape(nl, mm2)[:, :mnoe]),
                  "llu": d(vals(A.f_llu).reshape(nl, mm2)[:, :mnoe]), "de": d(vals(A.f_de)[:mnoe])}
    if solve:
        prog.call("cal_poisson_equation")
        x = np.array(vals(A.f_xe)[1:mnoe + 1].tolist())
        rec = {"iter": V.f_iter, "eps": V.f_eps, "ier": prog.env["s_cal_poisson_equation"].f_ier, "x": d(x)}
        if solve == "cpu":
            out["solve_cpu"] = rec
        else:
            out["solve"] = rec
            SOLUTIONS[f"{out['label']}/x"] = x
    if loop:
        prog = program(root, GRID_SOURCES)
        prog.fragment("cal_momentum", 41, 60, "ik_loop")
        V, A = load_grid(prog, case)
        V.f_d0, V.f_eps0 = rc.LOOP_D0, rc.LOOP_EPS0
        prog.call("set_nflag")
        prog.call("init_matrix")
        allocate_matrix(prog, V, A)
        prog.call("ik_loop")
        pl, unl = vals(A.f_p), vals(A.f_un).reshape(-1, 3)
        out["loop"] = {"ik": V.f_ik, "dmax": V.f_dmax, "p": d(pl), "un": d(unl)}
        if pl.size <= 5000:                       # values kept for the GPU comparison of small loops
            SOLUTIONS[f"{out['label']}/p"], SOLUTIONS[f"{out['label']}/un"] = pl, unl
    return out


def run_numbering(root, dims, nf3, nfb3) -> dict:
    """read_data's cell numbering (data_io.F90:168-202) and flag table
    (255-277) -- the reference's statements, without its file reads -- on flag
    grids over is-1:ie x js-1:je x ks-1:ke, after the allocation read_data
    makes (alloc_dxdydz(is, js, ks, ie+2, je+2, ke+2), data_io.F90:111-112)."""
    d = rc.digest
    prog = program(root, GRID_SOURCES + ["src2LOWNS/data_io.F90"])
    prog.fragment("read_data", 168, 202, "numbering")
    prog.fragment("read_data", 255, 277, "cell_flags")
    V, A = prog.module("variables"), prog.module("arrays")
    is_, js, ks, ie, je, ke = (int(v) for v in dims)
    V.f_is, V.f_js, V.f_ks, V.f_ie, V.f_je, V.f_ke = is_, js, ks, ie, je, ke
    prog.call("alloc_dxdydz", is_, js, ks, ie + 2, je + 2, ke + 2)
    bounds = [(is_ - 2, ie + 2), (ks - 2, ke + 2), (js - 2, je + 2)]
    n = (ie - is_ + 5) * (ke - ks + 5) * (je - js + 5)
    A.f_nf3, A.f_nfb3 = farray("int", [0] * n, bounds), farray("int", [0] * n, bounds)
    for j in range(js - 1, je + 1):
        for k in range(ks - 1, ke + 1):
            for i in range(is_ - 1, ie + 1):
                g = (j - (js - 1), k - (ks - 1), i - (is_ - 1))
                A.f_nf3[i, k, j] = int(nf3[g])
                A.f_nfb3[i, k, j] = int(nfb3[g])
    prog.call("numbering")
    inne, inne2 = V.f_inne, V.f_inne2
    region = ((is_ - 1, ie, None), (ks - 1, ke, None), (js - 1, je, None))
    out = {"inne": inne, "inne2": inne2, "mn": d(vals(A.f_mn)),
           "in": d(vals(A.f_in)[:inne2]), "jn": d(vals(A.f_jn)[:inne2]), "kn": d(vals(A.f_kn)[:inne2]),
           "nfb3": d(np.array(fx._sec(A.f_nfb3, region).v))}
    prog.call("cell_flags")
    nff = A.f_nff.values()[:inne2 + 2]
    out.update({"nf": d(np.array([o.f_f for o in nff])), "nfb": d(np.array([o.f_b for o in nff])),
                "mn_flags": d(vals(A.f_mn))})
    return out


def run_set_dx(root, dims, x) -> dict:
    """set_dx (1sub-main.F90:53-74, round lib/src/xy_calc.f90:100-112) on the
    coordinates x(0:2, 1:mx2) after read_data's allocation (alloc_dxdydz)."""
    prog = program(root, GRID_SOURCES)
    V, A = prog.module("variables"), prog.module("arrays")
    is_, js, ks, ie, je, ke = (int(v) for v in dims)
    prog.call("alloc_dxdydz", is_, js, ks, ie + 2, je + 2, ke + 2)
    mx2 = A.f_x.ext[1]
    if x.shape[0] > mx2:
        raise ValueError(f"coordinates for {x.shape[0]} cells, x(0:2, {mx2}) allocated")
    xx = np.zeros((mx2, 3))
    xx[:x.shape[0]] = x
    A.f_x = farray("real", xx.ravel(), [(0, 2), (1, mx2)])
    A.f_ls = farray("int", [is_, js, ks], [(0, 2)])
    A.f_le = farray("int", [ie, je, ke], [(0, 2)])
    prog.call("set_dx")
    return {"mx2": mx2, "x": rc.digest(vals(A.f_x)), "dx": rc.digest(vals(A.f_dx))}


def case_files(case, sparse, t0, p, nor):
    """The files ingest.write_case writes for the case: basename -> bytes."""
    import tempfile

    import __graft_entry__ as ge
    ing = ge.load_package().ingest
    with tempfile.TemporaryDirectory() as td:
        ing.write_case(pathlib.Path(td) / "case", case, p=p, nor=nor, sparse=sparse, t=t0)
        return {f.name: f.read_bytes() for f in sorted(pathlib.Path(td).iterdir())}


def files_digest(files) -> str:
    return rc.digest(np.frombuffer(b"".join(k.encode() + files[k] for k in sorted(files)), dtype=np.uint8))


def run_reader(root, files, sparse) -> dict:
    """The model's readers on the case files, in its order (main_2CLOWNS.F90:
    363-369, 52): read_data, read_fdata, read_nsdata (data_io.F90:87-397), then
    set_dx; the porosity file is the terrain fdata (INPUTf0) without drifting
    bodies, so a = a0 and fb = fb0 (data_io.F90:302-345)."""
    d = rc.digest
    texts = [(root / f).read_text(encoding="latin-1") for f in GRID_SOURCES + ["src2LOWNS/data_io.F90"]]
    texts.append(((root / "lib/src/owari.f").read_text(encoding="latin-1"), True))
    prog = fx.Program(texts, DEFINES, undefined=UNDEFINED)
    prog.env["_io"] = fx.FortranFiles(files)
    V, A = prog.module("variables"), prog.module("arrays")
    V.f_inputxyz = "case.xyzn" if sparse else "case.xyz"
    V.f_input, V.f_inputf0 = "case", "case.fdata"
    V.f_g_read, V.f_nu_read = 9.80665, 1.0e-6
    for routine in ("read_data", "read_fdata", "read_nsdata", "set_dx"):
        prog.call(routine)
    inne2 = V.f_inne2
    sp = vals(A.f_sp).reshape(3, -1)[:, :inne2 + 2]
    nor = vals(A.f_nor).reshape(4, -1).T
    out = {"dims": [V.f_is, V.f_js, V.f_ks, V.f_ie, V.f_je, V.f_ke], "inne": V.f_inne, "inne2": inne2,
           "x": d(vals(A.f_x)), "dx": d(vals(A.f_dx)), "mn": d(vals(A.f_mn)),
           "in": d(vals(A.f_in)[:inne2]), "jn": d(vals(A.f_jn)[:inne2]), "kn": d(vals(A.f_kn)[:inne2]),
           "nf": d(np.array([o.f_f for o in A.f_nff.values()[:inne2 + 2]])),
           "nfb": d(np.array([o.f_b for o in A.f_nff.values()[:inne2 + 2]])),
           "u": d(vals(A.f_u)), "f": d(vals(A.f_f)[:inne2 + 2]), "p": d(vals(A.f_p)),
           "a": d(vals(A.f_a)), "fb": d(vals(A.f_fb)[:inne2 + 2]),
           # entries the readers never write (border rows of sp and nor) are undefined
           "sp_undefined": rc.runs(np.flatnonzero(np.isnan(sp).ravel()) + 1),
           "sp": d(sp[~np.isnan(sp)]), "nor_undefined": rc.runs(np.flatnonzero(np.isnan(nor).ravel()) + 1),
           "nor": d(nor[~np.isnan(nor)]), "t0": V.f_t0, "g": V.f_g, "nu": V.f_nu}
    if V.f_t0 > 0.0:
        out["dt0"] = V.f_dt0
    return out


WRITER_SOURCES = ["srcMakeGrid/0mod-type_interface.F90", "srcMakeGrid/0mod-variables.F90",
                  "srcMakeGrid/0mod-arrays.F90", "srcMakeGrid/data_io.F90"]


def run_writer(root, case, sparse, t0, p, nor) -> dict:
    """The grid generator's writers (srcMakeGrid/data_io.F90: output_xyzn with
    its recoding pass off, or output_xyz; output_data, output_fdata,
    output_nsdata) on the case's arrays, in the bounds the generator allocates
    (make_grid_main.F90:189-256).  The surface cells are listed in ascending
    order (the generator's own order comes from its surface search, outside
    this path).  Returns the files' digests, and for the dense form whether the
    solver's readers accept the generator's files."""
    import __graft_entry__ as ge
    ing = ge.load_package().ingest
    texts = [(root / f).read_text(encoding="latin-1") for f in WRITER_SOURCES]
    texts.append(((root / "lib/src/owari.f").read_text(encoding="latin-1"), True))
    prog = fx.Program(texts, set())                # srcMakeGrid/Makefile defines no macros
    prog.env["_io"] = io = fx.FortranFiles()
    V, A = prog.module("variables"), prog.module("arrays")
    is_, js, ks, ie, je, ke = (int(v) for v in case.dims)
    inne, inne2 = int(case.inne), int(case.inne2)
    V.f_is, V.f_js, V.f_ks, V.f_ie, V.f_je, V.f_ke = is_, js, ks, ie, je, ke
    V.f_title, V.f_inne, V.f_inne2 = "case", inne, inne2
    V.f_t, V.f_g, V.f_nu, V.f_dt = t0, ing.G_ACC, 1.0e-6, case.dt
    V.f_fg_xyz, A.f_xyzn = (1 if sparse else 0), sparse
    A.f_x = farray("real", case.x.ravel(), [(0, 2), (1, case.x.shape[0])])
    A.f_ls, A.f_le = farray("int", [is_, js, ks], [(0, 2)]), farray("int", [ie, je, ke], [(0, 2)])
    nf3, nfb3 = ing.flag_grids(case)
    b3 = [(is_ - 1, ie), (ks - 1, ke), (js - 1, je)]
    A.f_nf3, A.f_nfb3 = farray("int", nf3.ravel(), b3), farray("int", nfb3.ravel(), b3)
    A.f_mn = farray("int", case.mn.ravel(), [(is_ - 2, ie + 2), (ks - 2, ke + 2), (js - 2, je + 2)])
    for nm, arr in (("in", case.in_), ("jn", case.jn), ("kn", case.kn)):
        setattr(A, "f_" + nm, farray("int", arr[1:inne2 + 1], [(1, inne2)]))
    A.f_nff = farray("obj", [CellFlag(int(f), int(b)) for f, b in zip(case.nf, case.nfb)], [(0, inne2 + 1)])
    A.f_u = farray("real", case.un[1:inne2 + 1].ravel(), [(0, 2), (1, inne2)])
    A.f_f = farray("real", case.f[1:inne2 + 1], [(1, inne2)])
    A.f_p = farray("real", p[1:inne2 + 1], [(1, inne2)])
    A.f_a = farray("real", case.a[1:inne2 + 1].ravel(), [(0, 2), (1, inne2)])
    A.f_fb = farray("real", case.fb[1:inne2 + 1], [(1, inne2)])
    A.f_sp = farray("real", case.sp.ravel(), [(0, inne2 + 1), (0, 2)])
    A.f_nor = farray("real", nor.T.ravel(), [(0, inne2 + 1), (0, 3)])
    listed = [nn for nn in range(1, inne + 1) if case.sp[0, nn] != -1.0e4]
    A.f_sfnoi = farray("int", listed or [0], [(1, max(1, len(listed)))])
    V.f_mms = len(listed)
    if sparse:
        prog.call("output_xyzn", 0)
    else:
        prog.call("output_xyz")
    for routine in ("output_data", "output_fdata", "output_nsdata"):
        prog.call(routine)
    out = {"files": {k: rc.digest(np.frombuffer(v, dtype=np.uint8)) for k, v in io.files.items()}}
    if not sparse:
        try:
            run_reader(root, io.files, sparse)
            out["solver_reads_generator_files"] = True
        except fx._IOError:
            out["solver_reads_generator_files"] = False
    return out


def run_one_pass(root, case) -> dict:
    """One pass of the ik loop body (1sub-momentum.F90:43-59): numbering and
    right-hand side, assembly, the solve, p -= xe and estimate_velocity2 --
    on a case whose boundary cells take estimate_velocity2's pressure-boundary
    branches (nf = -1, nfb = 4: 1sub-momentum.F90:611-621, 638-643)."""
    d = rc.digest
    prog = program(root, GRID_SOURCES)
    prog.fragment("cal_momentum", 52, 57, "p_update")
    V, A = load_grid(prog, case)
    V.f_eps0 = rc.LOOP_EPS0
    for routine in ("set_nflag", "init_matrix"):
        prog.call(routine)
    allocate_matrix(prog, V, A)
    for routine in ("cal_err_of_continuity", "cal_matrix_element", "cal_poisson_equation", "p_update",
                    "estimate_velocity2"):
        prog.call(routine)
    return {"iter": V.f_iter, "dmax": V.f_dmax, "p": d(vals(A.f_p)), "un": d(vals(A.f_un).reshape(-1, 3))}


PCGPME_EDGES = {"cap5": (1e-14, 5), "default_cap": (1e-10, 0), "eps0_small": (0.0, 10000),
                "tight_tolerance": (2e-15, 10000)}


def run_pcgpme_edges(root, case) -> dict:
    """PCGPME at its argument edges on the system the reference assembles:
    ITER = 5 (the cap: IER = 3000, ITER = cap + 1), ITER = 0 (the default cap
    10 (sqrt N + 1), pcgpme_para.F90:52) and EPS(1) = 0 (replaced by SMALL,
    pcgpme_para.F90:51); each on a fresh assembly, as PCGPME scales and sorts
    its arguments in place; and EPS(1) = 2e-15, the tightest tolerance above
    TINY, which runs the iteration down to the rounding floor."""
    out = {}
    for name, (eps, itmax) in PCGPME_EDGES.items():
        prog = program(root, GRID_SOURCES)
        V, A = load_grid(prog, case)
        for routine in ("set_nflag", "init_matrix"):
            prog.call(routine)
        allocate_matrix(prog, V, A)
        for routine in ("cal_err_of_continuity", "cal_matrix_element"):
            prog.call(routine)
        n, mm2, nl = V.f_mnoe, V.f_mm2, V.f_nl
        e = farray("real", [eps, 0.0], [(1, 2)])
        r = prog.call("pcgpme", A.f_alu, nl, mm2, A.f_llu, A.f_de, n, 64, A.f_b, A.f_xe.section_view(1, mm2),
                      e, 5.0, itmax, 0)
        x = np.array(vals(A.f_xe)[1:n + 1].tolist())
        out[name] = {"iter": r[11], "ier": r[12], "eps": e.values()[0], "x": rc.digest(x)}
    return out


def run_will(root, label, ds, eps) -> dict:
    prog = program(root, WILL_SOURCES)
    nl, na = ds.al.shape
    n = ds.n
    al = farray("real", [ds.al[k, i] for k in range(nl) for i in range(na)], [(1, na), (1, nl)])
    ll = farray("int", [ds.ll[k, i] for k in range(nl) for i in range(na)], [(1, na), (1, nl)])
    dd = farray("real", ds.d[:n], [(1, n)])
    bb = farray("real", ds.b[:n], [(1, n)])
    prog.call("pcgpme_will", al, nl, na, ll, dd, n, 64, bb, float(eps), 5.0, 10000)
    b = vals(bb)
    SOLUTIONS[f"{label}/b"] = b
    return {"input": rc.will_digest(ds), "b": rc.digest(b)}


def main(argv):
    root = pathlib.Path(argv[1] if len(argv) > 1 else "/root/reference")
    res = {"grids": {}, "will": {}, "will_cap3": {}, "numbering": {}, "set_dx": {}, "reader": {}, "writer": {},
           "edges": {}, "one_pass": {}}
    grids = rc.grid_cases()
    for label in ("beach_10x6x8", "flume2dv_16x1x8"):
        res["edges"][label] = run_pcgpme_edges(root, grids[label][0])
    res["one_pass"]["flume_40x24x20_ingested"] = run_one_pass(root, grids["flume_40x24x20_ingested"][0])
    for label, (case, sparse, t0, p, nor) in rc.reader_cases().items():
        files = case_files(case, sparse, t0, p, nor)
        res["reader"][label] = dict(run_reader(root, files, sparse), input=files_digest(files))
        res["writer"][label] = run_writer(root, case, sparse, t0, p, nor)
    for label, (dims, x) in rc.spacing_cases().items():
        res["set_dx"][label] = dict(run_set_dx(root, dims, x),
                                    input=rc.digest(np.concatenate([np.ravel(dims), np.ravel(x)])))
    for label, (dims, nf3, nfb3) in rc.numbering_cases().items():
        res["numbering"][label] = dict(run_numbering(root, dims, nf3, nfb3),
                                       input=rc.digest(np.concatenate([np.ravel(dims), np.ravel(nf3),
                                                                       np.ravel(nfb3)])))
    for label, (case, solve, loop) in rc.grid_cases().items():
        t = time.time()
        res["grids"][label] = run_grid(root, label, case, solve, loop)
        del res["grids"][label]["label"]
        print(f"{label}: {time.time() - t:.1f} s", flush=True)
    for label, (ds, eps) in rc.will_cases().items():
        res["will"][label] = run_will(root, label, ds, eps)
    for label, (ds, eps) in list(rc.will_cases().items())[:2]:
        # the iteration cap: B after three iterations and the post-processing (pcgpme_2DH.f90:247-280)
        prog = program(root, WILL_SOURCES)
        nl, na = ds.al.shape
        al = farray("real", [ds.al[k, i] for k in range(nl) for i in range(na)], [(1, na), (1, nl)])
        ll = farray("int", [ds.ll[k, i] for k in range(nl) for i in range(na)], [(1, na), (1, nl)])
        dd, bb = farray("real", ds.d[:ds.n], [(1, ds.n)]), farray("real", ds.b[:ds.n], [(1, ds.n)])
        prog.call("pcgpme_will", al, nl, na, ll, dd, ds.n, 64, bb, 1e-14, 5.0, 3)
        res["will_cap3"][label] = {"input": rc.will_digest(ds), "b": rc.digest(vals(bb))}
        print(f"{label}: done", flush=True)
    (HERE / "reference_runs.json").write_text(json.dumps(res, indent=1, sort_keys=True) + "\n")
    np.savez_compressed(HERE / "reference_solutions.npz", **SOLUTIONS)


if __name__ == "__main__":
    main(sys.argv)
