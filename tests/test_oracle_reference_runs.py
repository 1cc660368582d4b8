"""The oracle against the reference's own routines, run on the same seeded inputs.

tests/golden/reference_runs.json holds the outputs of the reference's Fortran
source (set_nflag, init_matrix, cal_err_of_continuity, cal_matrix_element,
cal_poisson_equation/PCGPME, the ik loop of 1sub-momentum.F90:41-60 and
PCGPME_WILL), executed here by tests/golden/make_ref_golden.py through
tests/golden/fortran_exec.py because no Fortran compiler exists.  Each output
is stored as a sha256 digest of its bytes; the oracle must reproduce every one
bit for bit (its serial loop order is the reference's).
"""
import json
import pathlib
import sys

import numpy as np
import pytest

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))

import reference_cases as rc  # noqa: E402

RUNS = json.loads((HERE / "golden" / "reference_runs.json").read_text())
d = rc.digest


@pytest.fixture(scope="module")
def grids():
    return rc.grid_cases()


def _check(stage, got: dict, want: dict):
    bad = [k for k in want if k in got and got[k] != want[k]]
    assert not bad, f"{stage}: {bad} differ from the reference's run"


def oracle_loop(ora, case, cls, sm, d0, eps0):
    """The ik loop (1sub-momentum.F90:41-60) through the oracle's routines."""
    c = case.copy()
    c.f = cls.f.copy()
    p = np.zeros(case.inne2 + 2)
    un = case.un.copy()
    ik = 0
    while True:
        c.un = un
        sy = ora.rows_rhs_assemble(c, cls, sm)
        if sy.dmax < d0:
            break
        ik += 1
        if ik > 1000:
            break
        r = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe, eps=eps0)
        p, un = ora.correct(c, cls, sy, r.x, p, un)
    return ik, sy.dmax, p, un


@pytest.mark.parametrize("label", sorted(RUNS["grids"]))
def test_oracle_reproduces_reference_run(ora, grids, label):
    want = RUNS["grids"][label]
    case, solve, loop = grids[label]
    assert rc.case_digest(case) == want["input"], "the seeded generator changed: regenerate the fixture"
    cls = ora.set_nflag(case)
    _check("set_nflag", {"nf": d(cls.nf), "nfb": d(cls.nfb), "f": d(cls.f), "ifln": cls.ifln,
                         "fln": d(cls.fln[1:]), "isfn": cls.isfn, "sfn": d(cls.sfn[1:])}, want["nflag"])
    sm = ora.init_matrix(case, cls)
    rows = ~rc.runs_mask(want["init"]["undefined_rows"], case.inne)
    _check("init_matrix", {"nl": sm.alu_c.shape[0], "mp": sm.mp, "alu_c": d(sm.alu_c[:, rows]),
                           "ll_c": d(sm.ll_c[:, rows]), "de_c": d(sm.de_c[rows])}, want["init"])
    sy = ora.rows_rhs_assemble(case, cls, sm)
    n = sy.mnoe
    _check("rows and RHS", {"mnoe": n, "mm2": sy.mm2, "dmax": sy.dmax, "mno": d(sy.mno.ravel()),
                            "mno2mn": d(sy.mno2mn[1:n + 1]), "b": d(sy.b[1:n + 1])}, want["rows"])
    _check("cal_matrix_element", {"alu": d(sy.alu[:, :n]), "llu": d(sy.llu[:, :n]), "de": d(sy.de[1:n + 1])},
           want["asm"])
    for key in ("solve", "solve_cpu"):
        if key in want:
            r = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=case.eps0, parm=5.0, itmax=10000, nthreads=1)
            _check("PCGPME", {"iter": r.iters, "eps": r.eps, "ier": r.ier, "x": d(r.x[:n])}, want[key])
    if loop:
        ik, dmax, p, un = oracle_loop(ora, case, cls, sm, rc.LOOP_D0, rc.LOOP_EPS0)
        _check("ik loop", {"ik": ik, "dmax": dmax, "p": d(p), "un": d(un)}, want["loop"])


@pytest.mark.parametrize("label", sorted(RUNS["will"]))
def test_oracle_will_reproduces_reference_run(ora, label):
    want = RUNS["will"][label]
    ds, eps = rc.will_cases()[label]
    assert rc.will_digest(ds) == want["input"], "the seeded generator changed: regenerate the fixture"
    b, _, _ = ora.pcgpme_will(ds.al, ds.ll, ds.d, ds.b, ds.n, eps=eps)
    assert d(b) == want["b"]


def test_fixture_covers_every_stage():
    """The recorded runs include 3D and 2DV grids, surface pruning cases, solves,
    multi-pass ik loops and cells init_matrix skips."""
    g = RUNS["grids"]
    assert {"nflag", "init", "rows", "asm"} <= set().union(*(v.keys() for v in g.values()))
    assert sum("solve" in v for v in g.values()) >= 8
    assert sum("solve_cpu" in v and v["rows"]["mnoe"] >= 9000 for v in g.values()) >= 3
    assert sum("loop" in v and v["loop"]["ik"] >= 2 for v in g.values()) >= 5
    assert any(v["init"]["nl"] == 4 for v in g.values()) and any(v["init"]["nl"] == 6 for v in g.values())
    assert any(v["init"]["undefined_rows"] for v in g.values())
    assert len(RUNS["will"]) >= 3


def test_stored_solutions_are_the_recorded_runs():
    """reference_solutions.npz holds the very vectors whose digests the runs
    recorded (the GPU solves are checked against these values)."""
    sol = np.load(HERE / "golden" / "reference_solutions.npz")
    xs = {k[:-2] for k in sol.files if k.endswith("/x")}
    assert xs == {k for k, v in RUNS["grids"].items() if "solve" in v}
    for k in xs:
        assert d(sol[k + "/x"]) == RUNS["grids"][k]["solve"]["x"]
    loops = {k[:-2] for k in sol.files if k.endswith("/p")}
    assert loops and loops <= {k for k, v in RUNS["grids"].items() if "loop" in v}
    for k in loops:
        assert d(sol[k + "/p"]) == RUNS["grids"][k]["loop"]["p"]
        assert d(sol[k + "/un"]) == RUNS["grids"][k]["loop"]["un"]
    bs = {k[:-2] for k in sol.files if k.endswith("/b")}
    assert bs == set(RUNS["will"])
    for k in bs:
        assert d(sol[k + "/b"]) == RUNS["will"][k]["b"]


@pytest.mark.parametrize("label", sorted(RUNS["numbering"]))
def test_ingest_numbering_reproduces_reference_read_data(label):
    """The case reader's cell numbering and flag table (2clowns-3d_gb300/ingest.py)
    against read_data's own statements (data_io.F90:168-202, 255-277) on the same
    flag grids: bit for bit."""
    import __graft_entry__ as ge
    ing = ge.load_package().ingest
    want = RUNS["numbering"][label]
    dims, nf3, nfb3 = rc.numbering_cases()[label]
    assert d(np.concatenate([np.ravel(dims), np.ravel(nf3), np.ravel(nfb3)])) == want["input"]
    nb = ing.number_cells(dims, nf3, nfb3)
    nf, nfb, mn = ing.cell_flags(dims, nf3, nb.nfb3, nb)
    m = nb.inne2
    flat = lambda a: d(np.ravel(a))  # noqa: E731
    _check("read_data numbering", {"inne": nb.inne, "inne2": m, "mn": flat(nb.mn), "in": flat(nb.in_[1:m + 1]),
                                   "jn": flat(nb.jn[1:m + 1]), "kn": flat(nb.kn[1:m + 1]), "nfb3": flat(nb.nfb3),
                                   "nf": flat(nf), "nfb": flat(nfb), "mn_flags": flat(mn)}, want)


@pytest.mark.parametrize("label", sorted(RUNS["set_dx"]))
def test_ingest_set_dx_reproduces_reference_set_dx(label):
    """The case reader's spacings (ingest.set_dx) against the reference's set_dx
    and round (1sub-main.F90:53-74, lib/src/xy_calc.f90:100-112): bit for bit."""
    import __graft_entry__ as ge
    ing = ge.load_package().ingest
    want = RUNS["set_dx"][label]
    dims, x = rc.spacing_cases()[label]
    assert d(np.concatenate([np.ravel(dims), np.ravel(x)])) == want["input"]
    xx = np.zeros((want["mx2"], 3))
    xx[:x.shape[0]] = x
    xo, dxo = ing.set_dx(dims, xx)
    assert d(np.ravel(xo)) == want["x"] and d(np.ravel(dxo)) == want["dx"]


@pytest.mark.parametrize("label", sorted(RUNS["reader"]))
def test_ingest_reader_reproduces_reference_readers(tmp_path, label):
    """ingest.write_case's files read by the reference's own readers (read_data,
    read_fdata, read_nsdata, set_dx) give exactly what ingest.read_case gives:
    dimensions, coordinates and spacings, numbering, flags, velocities, F,
    pressure, porosities, surface positions and normals (the entries the
    readers define), t0, g, nu and the trailing dt."""
    import make_ref_golden as mk
    import __graft_entry__ as ge
    ing = ge.load_package().ingest
    want = RUNS["reader"][label]
    case, sparse, t0, p, nor = rc.reader_cases()[label]
    files = mk.case_files(case, sparse, t0, p, nor)
    assert mk.files_digest(files) == want["input"], "the writer's bytes differ from what the reference read"
    for name, data in files.items():
        (tmp_path / name).write_bytes(data)
    got = ing.read_case(tmp_path / "case")
    c, n2 = got.case, got.case.inne2
    spm = ~rc.runs_mask(want["sp_undefined"], 3 * (n2 + 2)).reshape(3, n2 + 2)
    norm = ~rc.runs_mask(want["nor_undefined"], 4 * (n2 + 2)).reshape(n2 + 2, 4)
    flat = lambda a: d(np.ravel(a))  # noqa: E731
    _check("readers", {"dims": [int(v) for v in c.dims], "inne": c.inne, "inne2": n2, "x": flat(c.x),
                       "dx": flat(c.dx), "mn": flat(c.mn), "in": flat(c.in_[1:n2 + 1]), "jn": flat(c.jn[1:n2 + 1]),
                       "kn": flat(c.kn[1:n2 + 1]), "nf": flat(c.nf), "nfb": flat(c.nfb), "u": flat(c.un),
                       "f": flat(c.f), "p": flat(got.p[:n2 + 1]), "a": flat(c.a), "fb": flat(c.fb),
                       "sp": flat(c.sp[spm]), "nor": flat(got.nor[:n2 + 2][norm]), "t0": got.t0, "g": got.g,
                       "nu": got.nu, "dt0": got.dt0}, want)


@pytest.mark.parametrize("label", sorted(RUNS["writer"]))
def test_ingest_writer_reproduces_generator_files(label):
    """ingest.write_case against the grid generator's own writers on the same
    arrays: every file byte for byte -- except, in the dense form, the .fdata
    file: the generator writes its sparse form there whatever the form, which
    the solver's read_fdata cannot read (recorded by the run), so write_case
    writes the dense .fdata the solver reads (checked by the reader test)."""
    import make_ref_golden as mk
    want = RUNS["writer"][label]
    case, sparse, t0, p, nor = rc.reader_cases()[label]
    files = mk.case_files(case, sparse, t0, p, nor)
    assert set(files) == set(want["files"])
    for name, data in files.items():
        if name == "case.fdata" and not sparse:
            assert want["solver_reads_generator_files"] is False
            continue
        assert d(np.frombuffer(data, dtype=np.uint8)) == want["files"][name], name


@pytest.mark.parametrize("label", sorted(RUNS["edges"]))
def test_oracle_pcgpme_edges_reproduce_reference(ora, grids, label):
    """PCGPME at its argument edges -- the iteration cap (IER 3000, ITER =
    cap + 1), ITER = 0 (the default cap), EPS(1) = 0 (SMALL) and the tightest
    tolerance above TINY (down to the rounding floor) -- against the reference's
    own PCGPME on the same system: bit for bit."""
    import make_ref_golden as mk
    case = grids[label][0]
    cls = ora.set_nflag(case)
    sy = ora.rows_rhs_assemble(case, cls, ora.init_matrix(case, cls))
    for name, (eps, itmax) in mk.PCGPME_EDGES.items():
        r = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe, eps=eps, itmax=itmax, nthreads=1)
        _check(f"PCGPME {name}", {"iter": r.iters, "ier": r.ier, "eps": r.eps, "x": d(r.x[:sy.mnoe])},
               RUNS["edges"][label][name])


@pytest.mark.parametrize("label", sorted(RUNS["will_cap3"]))
def test_oracle_will_at_its_iteration_cap_reproduces_reference(ora, label):
    """PCGPME_WILL stopped by its cap after three iterations (and post-processed
    as the reference does): the oracle's B equals the reference's bit for bit."""
    want = RUNS["will_cap3"][label]
    ds, _ = rc.will_cases()[label]
    assert rc.will_digest(ds) == want["input"]
    b, it, reason = ora.pcgpme_will(ds.al, ds.ll, ds.d, ds.b, ds.n, eps=1e-14, itmax=3)
    assert d(b) == want["b"] and reason == 4


@pytest.mark.parametrize("label", sorted(RUNS["one_pass"]))
def test_oracle_one_ik_pass_reproduces_reference(ora, grids, label):
    """One pass of the ik loop body on the flume with wave-boundary cells
    (estimate_velocity2's pressure-boundary branches): the oracle's pressure and
    face velocities equal the reference's bit for bit."""
    want = RUNS["one_pass"][label]
    case = grids[label][0]
    cls = ora.set_nflag(case)
    c = case.copy()
    c.f = cls.f.copy()
    sy = ora.rows_rhs_assemble(c, cls, ora.init_matrix(case, cls))
    r = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe, eps=rc.LOOP_EPS0)
    p, un = ora.correct(c, cls, sy, r.x, np.zeros(case.inne2 + 2), case.un.copy())
    _check("one ik pass", {"iter": r.iters, "dmax": sy.dmax, "p": d(p), "un": d(un)}, want)
