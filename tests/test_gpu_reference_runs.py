"""The CUDA path against the reference's own routines: classification
(set_nflag), static coefficients (init_matrix), numbering and right-hand side
(cal_err_of_continuity) and assembly (cal_matrix_element) bit for bit on the 14
grids of tests/golden/reference_runs.json -- outputs of the reference's Fortran
source, run on the CPU by tests/golden/make_ref_golden.py.  (The solves are
compared with the oracle within their tolerance in tests/test_gpu_parity.py and
tests/test_gpu_configs.py; the oracle reproduces the reference's solves bit for
bit, tests/test_oracle_reference_runs.py.)"""
import json
import pathlib
import sys

import numpy as np
import pytest

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))

import reference_cases as rc  # noqa: E402

pytestmark = pytest.mark.gpu

RUNS = json.loads((HERE / "golden" / "reference_runs.json").read_text())
d = rc.digest


@pytest.fixture(scope="module")
def grids():
    return rc.grid_cases()


def _check(stage, got: dict, want: dict):
    bad = [k for k in want if k in got and got[k] != want[k]]
    assert not bad, f"{stage}: {bad} differ from the reference's run"


@pytest.mark.parametrize("label", sorted(RUNS["grids"]))
def test_gpu_reproduces_reference_run(gpu, grids, label):
    want = RUNS["grids"][label]
    case = grids[label][0]
    if rc.case_digest(case) != want["input"]:
        pytest.skip("the seeded generator gives other inputs on this machine than where the reference ran")
    dc, ds = gpu.prepare_dev(case)
    h = lambda t: t.cpu().numpy()  # noqa: E731
    _check("set_nflag", {"nf": d(h(dc.nf)), "nfb": d(h(dc.nfb)), "f": d(h(dc.f)), "ifln": ds.ifln,
                         "fln": d(h(ds.fln)[:ds.ifln]), "isfn": ds.isfn, "sfn": d(h(ds.sfn)[:ds.isfn])},
           want["nflag"])
    rows = ~rc.runs_mask(want["init"]["undefined_rows"], case.inne)
    alu_c, ll_c, de_c = h(ds.alu_c), h(ds.ll_c), h(ds.de_c)
    _check("init_matrix", {"nl": alu_c.shape[0], "mp": float(ds.mp.item()), "alu_c": d(alu_c[:, rows]),
                           "ll_c": d(ll_c[:, rows]), "de_c": d(de_c[rows])}, want["init"])
    n = ds.mnoe
    _check("rows and RHS", {"mnoe": n, "mm2": ds.mm2, "dmax": ds.dmax, "mno": d(h(ds.mno).ravel()),
                            "mno2mn": d(h(ds.mno2mn)[:n]), "b": d(h(ds.b)[:n])}, want["rows"])
    _check("cal_matrix_element", {"alu": d(h(ds.alu)[:, :n]), "llu": d(h(ds.llu)[:, :n]),
                                  "de": d(h(ds.de)[:n])}, want["asm"])


SOL = np.load(HERE / "golden" / "reference_solutions.npz")


@pytest.mark.parametrize("label", sorted(k for k, v in RUNS["grids"].items() if "solve" in v))
def test_gpu_solve_matches_reference_solve(gpu, grids, label):
    """The GPU's FP64 solve of the system it assembled against the reference's
    PCGPME on the same system, both to the case's ERR <= eps: within 10 eps
    relative L2 (the bound the oracle comparison measures at most 4.1 eps
    against), iteration counts within a sixth (reduction order only)."""
    import torch
    want = RUNS["grids"][label]["solve"]
    case = grids[label][0]
    if rc.case_digest(case) != RUNS["grids"][label]["input"]:
        pytest.skip("the seeded generator gives other inputs on this machine than where the reference ran")
    dc, ds = gpu.prepare_dev(case)
    n = ds.mnoe
    x = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
    info = gpu.Solver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=case.eps0)
    xr = SOL[label + "/x"]
    rel = float(np.linalg.norm(x.cpu().numpy()[:n] - xr) / np.linalg.norm(xr))
    msg = (label, "rel", rel, "iters gpu/reference", info.iter, want["iter"])
    assert info.ier == 0 and want["ier"] == 0, msg
    assert rel <= 10 * case.eps0, msg
    assert abs(info.iter - want["iter"]) <= max(3, want["iter"] // 6), msg


@pytest.mark.parametrize("label", sorted(RUNS["will"]))
def test_gpu_will_matches_reference_will(gpu, label):
    """PCGPME_WILL on the GPU against the reference's, B after both
    post-processings within 100 eps relative L2 (the bound of the oracle
    comparison at eps = 1e-12)."""
    import torch
    ds, eps = rc.will_cases()[label]
    if rc.will_digest(ds) != RUNS["will"][label]["input"]:
        pytest.skip("the seeded generator gives other inputs on this machine than where the reference ran")
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to("cuda")  # noqa: E731
    b = dev(ds.b)
    info = gpu.WillSolver(ds.n).solve(dev(ds.al), dev(ds.ll), dev(ds.d), b, eps=eps)
    br = SOL[label + "/b"]
    rel = float(np.linalg.norm(b.cpu().numpy() - br) / np.linalg.norm(br))
    assert info.ier == 0 and rel <= 100 * eps, (label, rel, info.as_dict())


@pytest.mark.parametrize("label", sorted(k for k, v in RUNS["grids"].items() if "loop" in v and k + "/p" in SOL.files))
def test_gpu_session_matches_reference_ik_loop(gpu, grids, label):
    """The device-resident ik loop (clowns_session_*) against the reference's
    own (1sub-momentum.F90:41-60) from the raw flags: the same classification
    bit for bit, the same number of passes, and pressure and face velocities
    within 1e-10 relative L2 -- each pass solves to ERR <= 1e-7, but the second
    pass solves for the first one's error, so different reduction orders leave
    about 1e-16 (measured between the oracle's serial and OpenMP solves)."""
    want = RUNS["grids"][label]
    case = grids[label][0]
    if rc.case_digest(case) != want["input"]:
        pytest.skip("the seeded generator gives other inputs on this machine than where the reference ran")
    s = gpu.Session(case)
    s.set_fields(case.nf, case.nfb, case.f, case.fb, case.a, case.un, case.sp, np.zeros(case.inne2 + 2))
    ifln, isfn = s.classify()
    out = s.pressure_loop(case.dt, d0=rc.LOOP_D0, eps0=rc.LOOP_EPS0)
    got = s.fields()
    s.close()
    assert ifln == want["nflag"]["ifln"] and isfn == want["nflag"]["isfn"]
    assert d(got["nf"]) == want["nflag"]["nf"] and d(got["nfb"]) == want["nflag"]["nfb"]
    assert out["icon"] == 0 and out["ik"] == want["loop"]["ik"], (out, want["loop"])
    pr, unr = SOL[label + "/p"], SOL[label + "/un"]
    rp = float(np.linalg.norm(got["p"] - pr) / np.linalg.norm(pr))
    ru = float(np.linalg.norm(got["un"].reshape(unr.shape) - unr) / np.linalg.norm(unr))
    assert rp <= 1e-10 and ru <= 1e-10, (label, rp, ru)
