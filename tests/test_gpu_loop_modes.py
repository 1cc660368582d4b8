"""Every execution of the iteration loop the autotuner can pick, forced one at a
time: the CUDA graph (tile and balanced kernels), host launches of the same
kernels, the persistent cooperative kernel and the wavefront kernel.  Each
solves to the oracle's pressure (FP64 within 1e-10 relative L2 at ERR <=
1e-13; mixed within its bound at 1e-12), and for ensembles each member
matches its single-system solve."""
import numpy as np
import pytest

from cases import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()
MODES = [("graph", "0"), ("graph", "4"), ("launch", "0"), ("launch", "4"), ("persistent", "0"), ("wave", "0")]


@pytest.fixture(scope="module")
def system(gpu, ora):
    import torch
    label, case = CASES[1]
    cls, sm, sy = ora.prepare(case)
    dc, ds = gpu.prepare_dev(case)
    torch.cuda.synchronize()
    return case, sy, ds


def _x(ds):
    import torch
    return torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")


def _force(monkeypatch, mode, balanced):
    monkeypatch.setenv("CLOWNS_LOOP_MODE", mode)
    monkeypatch.setenv("CLOWNS_BALANCED_ROWS", balanced)


@pytest.mark.parametrize("mode,balanced", MODES)
def test_single_system_every_execution(gpu, ora, system, monkeypatch, mode, balanced):
    import scipy.sparse.linalg as spl
    case, sy, ds = system
    n = ds.mnoe
    _force(monkeypatch, mode, balanced)
    x = _x(ds)
    info = gpu.Solver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-13)
    ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-13)
    xg = x.cpu().numpy()[:n]
    assert info.ier == 0, (mode, info.as_dict())
    assert np.linalg.norm(xg - ref.x) <= 1e-10 * np.linalg.norm(ref.x), mode
    assert abs(info.iter - ref.iters) <= max(5, ref.iters // 4), (mode, info.iter, ref.iters)
    x = _x(ds)
    info = gpu.MixedSolver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-12)
    assert info.ier == 0 and info.eps <= 1e-12, (mode, info.as_dict())
    xd = spl.spsolve(ora.to_csr(sy).tocsc(), sy.b[1:n + 1])
    err_oracle = np.linalg.norm(ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-12).x - xd)
    assert np.linalg.norm(x.cpu().numpy()[:n] - xd) <= max(1e-9 * np.linalg.norm(xd), 2 * err_oracle), mode


@pytest.mark.parametrize("mode,balanced", [("graph", "0"), ("graph", "4"), ("persistent", "0")])
def test_ensemble_every_execution(gpu, ora, monkeypatch, mode, balanced):
    """FP64 members match their single-system solves within 1e-10 relative L2
    (both to 1e-13); mixed members reach ERR <= 1e-12 and the exact solution
    of their system as closely as the oracle does (the tank's matrix is nearly
    singular, so solutions at the same ERR differ along its near-null mode)."""
    import scipy.sparse.linalg as spl
    import torch
    systems = []
    for label, case in CASES[:4]:
        cls, sm, sy = ora.prepare(case)
        dc, ds = gpu.prepare_dev(case)
        systems.append((sy, ds))
    torch.cuda.synchronize()
    _force(monkeypatch, mode, balanced)
    sizes = [ds.mnoe for _, ds in systems]
    sys_list = [(ds.alu, ds.llu, ds.de, ds.b) for _, ds in systems]
    xs = [_x(ds) for _, ds in systems]
    infos = gpu.BatchedSolver(sizes, gpu.PREC_FP64).solve(sys_list, xs, eps=1e-13)
    for (sy, ds), x, info in zip(systems, xs, infos):
        x1 = _x(ds)
        i1 = gpu.Solver(ds.mnoe).solve(ds.alu, ds.llu, ds.de, ds.b, x1, eps=1e-13)
        a = x.cpu().numpy()[:ds.mnoe]
        b = x1.cpu().numpy()[:ds.mnoe]
        assert info.ier == 0 and i1.ier == 0, (mode, info.as_dict(), i1.as_dict())
        assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(b), mode
    xs = [_x(ds) for _, ds in systems]
    infos = gpu.BatchedSolver(sizes, gpu.PREC_MIXED).solve(sys_list, xs, eps=1e-12)
    for (sy, ds), x, info in zip(systems, xs, infos):
        n = ds.mnoe
        assert info.ier == 0 and info.eps <= 1e-12, (mode, info.as_dict())
        xd = spl.spsolve(ora.to_csr(sy).tocsc(), sy.b[1:n + 1])
        err_oracle = np.linalg.norm(ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-12).x - xd)
        assert np.linalg.norm(x.cpu().numpy()[:n] - xd) <= max(1e-9 * np.linalg.norm(xd), 2 * err_oracle), mode
