"""Every execution of the iteration loop the autotuner can pick, forced one at a
time: the CUDA graph of tile kernels (fused or single LDUSUB sweeps, 128 or 64
threads per dot-product tile), the graph of balanced one-wave kernels (4 or 8
rows per thread; for the FP32 inner solve also with the AXSUB whose streams are
staged in shared memory by bulk copies), the same kernels launched from the
host, the persistent cooperative kernel and the wavefront kernel.

All of them form dot products with one summation tree (128-row chunks, a fixed
butterfly per chunk, fixed group and member trees), so every execution must
give the SAME iteration count and the SAME pressure bits -- a drop-in for
PCGPME must not change its answer with the launch shape the autotuner picks --
and that pressure must be the oracle's within 1e-10 relative L2 (both at
ERR <= 1e-13).  Ensemble members must equal their single-system solves bit for
bit, in FP64 and in mixed precision."""
import numpy as np
import pytest

from cases import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()
# (CLOWNS_LOOP_MODE, CLOWNS_SWEEP_FUSE, CLOWNS_REDUCE_BLOCK, CLOWNS_BALANCED_ROWS, CLOWNS_AXSUB_STAGED)
MODES = [
    ("graph", "1", "128", "0", "0"),
    ("graph", "0", "128", "0", "0"),
    ("graph", "1", "64", "0", "0"),
    ("graph", "1", "128", "4", "0"),
    ("graph", "0", "128", "4", "0"),
    ("graph", "1", "128", "8", "0"),
    ("graph", "1", "128", "4", "1"),
    ("launch", "0", "128", "0", "0"),
    ("launch", "1", "128", "4", "0"),
    ("launch", "1", "128", "4", "1"),
    ("persistent", "1", "128", "0", "0"),
    ("wave", "1", "128", "0", "0"),
]
IDS = ["-".join(m) for m in MODES]
ENSEMBLE_MODES = [MODES[0], MODES[3], MODES[5], MODES[10]]


def _x(ds):
    import torch
    return torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")


def _force(monkeypatch, mode):
    loop, fuse, rblock, bal, staged = mode
    monkeypatch.setenv("CLOWNS_LOOP_MODE", loop)
    monkeypatch.setenv("CLOWNS_SWEEP_FUSE", fuse)
    monkeypatch.setenv("CLOWNS_REDUCE_BLOCK", rblock)
    monkeypatch.setenv("CLOWNS_BALANCED_ROWS", bal)
    monkeypatch.setenv("CLOWNS_AXSUB_STAGED", staged)


@pytest.fixture(scope="module")
def system(gpu, ora):
    import torch
    label, case = CASES[1]
    cls, sm, sy = ora.prepare(case)
    dc, ds = gpu.prepare_dev(case)
    torch.cuda.synchronize()
    ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe, eps=1e-13)
    return case, sy, ds, ref


@pytest.fixture(scope="module")
def first_result():
    """Results of the first mode, which every other mode must reproduce."""
    return {}


@pytest.mark.parametrize("mode", MODES, ids=IDS)
def test_single_system_every_execution(gpu, ora, system, first_result, monkeypatch, mode):
    case, sy, ds, ref = system
    n = ds.mnoe
    _force(monkeypatch, mode)
    x = _x(ds)
    info = gpu.Solver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-13)
    xg = x.cpu().numpy()[:n]
    assert info.ier == 0, (mode, info.as_dict())
    assert np.linalg.norm(xg - ref.x) <= 1e-10 * np.linalg.norm(ref.x), mode
    xm = _x(ds)
    minfo = gpu.MixedSolver(n).solve(ds.alu, ds.llu, ds.de, ds.b, xm, eps=1e-12)
    assert minfo.ier == 0 and minfo.eps <= 1e-12, (mode, minfo.as_dict())
    xmg = xm.cpu().numpy()[:n]
    if not first_result:
        first_result.update(x=xg, iter=info.iter, eps=info.eps, xm=xmg, miter=minfo.iter, mouter=minfo.outer)
        return
    # the same summation tree in every execution: identical iterations and bits
    assert info.iter == first_result["iter"], (mode, info.iter, first_result["iter"])
    assert info.eps == first_result["eps"], mode
    assert np.array_equal(xg, first_result["x"]), mode
    assert (minfo.iter, minfo.outer) == (first_result["miter"], first_result["mouter"]), mode
    assert np.array_equal(xmg, first_result["xm"]), mode


@pytest.mark.parametrize("mode", ENSEMBLE_MODES, ids=["-".join(m) for m in ENSEMBLE_MODES])
def test_ensemble_members_equal_single_solves(gpu, ora, monkeypatch, mode):
    """An ensemble member's iterations and pressure are those of its own solve,
    bit for bit (FP64 and mixed), and the FP64 pressures are the oracle's within
    1e-10 relative L2 at ERR <= 1e-13."""
    import torch
    systems = []
    for label, case in CASES[:4]:
        cls, sm, sy = ora.prepare(case)
        dc, ds = gpu.prepare_dev(case)
        systems.append((sy, ds))
    torch.cuda.synchronize()
    _force(monkeypatch, mode)
    sizes = [ds.mnoe for _, ds in systems]
    sys_list = [(ds.alu, ds.llu, ds.de, ds.b) for _, ds in systems]
    for prec, eps in ((gpu.PREC_FP64, 1e-13), (gpu.PREC_MIXED, 1e-12)):
        xs = [_x(ds) for _, ds in systems]
        infos = gpu.BatchedSolver(sizes, prec).solve(sys_list, xs, eps=eps)
        for (sy, ds), x, info in zip(systems, xs, infos):
            x1 = _x(ds)
            if prec == gpu.PREC_FP64:
                i1 = gpu.Solver(ds.mnoe).solve(ds.alu, ds.llu, ds.de, ds.b, x1, eps=eps)
            else:
                i1 = gpu.MixedSolver(ds.mnoe).solve(ds.alu, ds.llu, ds.de, ds.b, x1, eps=eps)
            a = x.cpu().numpy()[:ds.mnoe]
            b = x1.cpu().numpy()[:ds.mnoe]
            assert info.ier == 0 and i1.ier == 0, (mode, prec, info.as_dict(), i1.as_dict())
            assert (info.iter, info.outer, info.eps) == (i1.iter, i1.outer, i1.eps), (mode, prec)
            assert np.array_equal(a, b), (mode, prec)
            if prec == gpu.PREC_FP64:
                ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], ds.mnoe, eps=eps)
                assert np.linalg.norm(a - ref.x) <= 1e-10 * np.linalg.norm(ref.x), mode
