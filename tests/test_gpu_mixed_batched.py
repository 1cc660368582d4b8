"""Mixed precision (FP32 storage + FP64 refinement) and batched ensembles.

Tolerances: the mixed path must reach the requested ERR (measured in FP64 on
the true residual) and its pressure must be as close to the exact solution of
the assembled system (scipy LU) as the FP64 oracle's: within
max(1e-9, 2 x the oracle's own error) relative L2 at ERR <= 1e-12.  A batched
member must match its single-system solve within 1e-10 relative L2 when both
solve to 1e-13."""
import numpy as np
import pytest

from cases import small_cases

pytestmark = pytest.mark.gpu

CASES = small_cases()


@pytest.fixture(scope="module")
def systems(gpu, ora):
    import torch
    out = []
    for label, case in CASES:
        cls, sm, sy = ora.prepare(case)
        dc, ds = gpu.prepare_dev(case)
        torch.cuda.synchronize()
        out.append((label, case, sy, ds))
    return out


def _x(ds):
    import torch
    return torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")


def _direct(ora, sy):
    import scipy.sparse.linalg as spl
    n = sy.mnoe
    return spl.spsolve(ora.to_csr(sy).tocsc(), sy.b[1:n + 1])


@pytest.mark.parametrize("idx", range(len(CASES)), ids=[c[0] for c in CASES])
def test_mixed_matches_fp64_oracle(gpu, ora, systems, idx):
    label, case, sy, ds = systems[idx]
    n = sy.mnoe
    ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-13)
    xd = _direct(ora, sy)
    nd = np.linalg.norm(xd)
    err_oracle = np.linalg.norm(ref.x - xd) / nd
    solver = gpu.MixedSolver(n)
    for eps in (1e-10, 1e-12):
        x = _x(ds)
        info = solver.solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=eps)
        xg = x.cpu().numpy()[:n]
        assert info.ier == 0 and info.eps <= eps, info.as_dict()
        assert info.outer >= 1
        if eps == 1e-12:
            err = np.linalg.norm(xg - xd) / nd
            assert err <= max(1e-9, 2 * err_oracle), (label, err, err_oracle, info.as_dict())


@pytest.mark.parametrize("balanced", ["0", "4", "8"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fused_kernels_bit_identical(gpu, systems, monkeypatch, precision, balanced):
    """The fused LDUSUB sweep pairs (sweep J recomputed at the one row sweep J+1
    gathers) round exactly like the separate sweeps: forcing the CUDA-graph loop
    with and without them gives the same iterations and the same solution bit
    for bit, in FP64 and in the FP32 inner solve, with the tile kernels and with
    the balanced one-wave kernels (4 or 8 rows per thread per step)."""
    label, case, sy, ds = systems[1]
    n = ds.mnoe
    monkeypatch.setenv("CLOWNS_LOOP_MODE", "graph")
    monkeypatch.setenv("CLOWNS_BALANCED_ROWS", balanced)
    out = []
    for fuse in ("0", "1"):
        monkeypatch.setenv("CLOWNS_SWEEP_FUSE", fuse)
        x = _x(ds)
        if precision == "fp64":
            info = gpu.Solver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-12)
        else:
            info = gpu.MixedSolver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-12)
        assert info.ier == 0, info.as_dict()
        out.append((info.iter, x.cpu().numpy()[:n].copy()))
    for it, xv in out[1:]:
        assert it == out[0][0]
        assert np.array_equal(xv, out[0][1])


@pytest.mark.parametrize("balanced", ["4", "8"])
@pytest.mark.parametrize("label", [c[0] for c in CASES])
def test_balanced_kernels_match_oracle(gpu, ora, systems, monkeypatch, label, balanced):
    """The balanced one-wave kernels (rows split evenly over one wave of blocks,
    one reduction per block) solve to the oracle's pressure: within 1e-10
    relative L2 at ERR <= 1e-13 in FP64, within the mixed path's bound at
    ERR <= 1e-12 in mixed precision; iteration counts within 25 % of the
    oracle's (the reduction order differs from the tile kernels')."""
    idx = [c[0] for c in CASES].index(label)
    _, case, sy, ds = systems[idx]
    n = ds.mnoe
    monkeypatch.setenv("CLOWNS_LOOP_MODE", "graph")
    monkeypatch.setenv("CLOWNS_BALANCED_ROWS", balanced)
    x = _x(ds)
    info = gpu.Solver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-13)
    ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-13)
    xg = x.cpu().numpy()[:n]
    assert info.ier == 0 and ref.ier == 0, info.as_dict()
    assert np.linalg.norm(xg - ref.x) <= 1e-10 * np.linalg.norm(ref.x)
    assert abs(info.iter - ref.iters) <= max(5, ref.iters // 4), (info.iter, ref.iters)
    x = _x(ds)
    info = gpu.MixedSolver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-12)
    assert info.ier == 0 and info.eps <= 1e-12, info.as_dict()
    xd = _direct(ora, sy)
    err_oracle = np.linalg.norm(ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-12).x - xd)
    assert np.linalg.norm(x.cpu().numpy()[:n] - xd) <= max(1e-9 * np.linalg.norm(xd), 2 * err_oracle)


def test_mixed_true_residual(gpu, ora, systems):
    """Unpreconditioned true residual of the mixed solution is at the FP64 level."""
    label, case, sy, ds = systems[1]
    n = sy.mnoe
    x = _x(ds)
    gpu.MixedSolver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-12)
    A = ora.to_csr(sy)
    b = sy.b[1:n + 1]
    xg = x.cpu().numpy()[:n]
    assert np.linalg.norm(b - A @ xg) <= 1e-10 * np.linalg.norm(b)


def _force_balanced(monkeypatch, balanced):
    """"auto": the autotuner decides; "0", "4", "8": the graph loop with the tile
    kernels or the balanced kernels at 4 or 8 rows per thread."""
    if balanced != "auto":
        monkeypatch.setenv("CLOWNS_LOOP_MODE", "graph")
        monkeypatch.setenv("CLOWNS_BALANCED_ROWS", balanced)


@pytest.mark.parametrize("balanced", ["auto", "0", "4", "8"])
def test_batched_fp64_matches_single(gpu, systems, monkeypatch, balanced):
    import torch
    _force_balanced(monkeypatch, balanced)
    sys_list = [(ds.alu, ds.llu, ds.de, ds.b) for (_, _, _, ds) in systems]
    sizes = [ds.mnoe for (_, _, _, ds) in systems]
    xs = [_x(ds) for (_, _, _, ds) in systems]
    infos = gpu.BatchedSolver(sizes, gpu.PREC_FP64).solve(sys_list, xs, eps=1e-13)
    for (label, case, sy, ds), x, info in zip(systems, xs, infos):
        xs1 = _x(ds)
        i1 = gpu.Solver(ds.mnoe).solve(ds.alu, ds.llu, ds.de, ds.b, xs1, eps=1e-13)
        a = x.cpu().numpy()[:ds.mnoe]
        b = xs1.cpu().numpy()[:ds.mnoe]
        assert info.ier == 0 and i1.ier == 0
        assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(b), label
        assert abs(info.iter - i1.iter) <= max(5, i1.iter // 4)
    torch.cuda.synchronize()


@pytest.mark.parametrize("balanced", ["auto", "4", "8"])
def test_batched_mixed_converges_per_member(gpu, ora, systems, monkeypatch, balanced):
    _force_balanced(monkeypatch, balanced)
    sys_list = [(ds.alu, ds.llu, ds.de, ds.b) for (_, _, _, ds) in systems]
    sizes = [ds.mnoe for (_, _, _, ds) in systems]
    xs = [_x(ds) for (_, _, _, ds) in systems]
    infos = gpu.BatchedSolver(sizes, gpu.PREC_MIXED).solve(sys_list, xs, eps=1e-12)
    for (label, case, sy, ds), x, info in zip(systems, xs, infos):
        n = sy.mnoe
        ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-13)
        xd = _direct(ora, sy)
        nd = np.linalg.norm(xd)
        err_oracle = np.linalg.norm(ref.x - xd) / nd
        xg = x.cpu().numpy()[:n]
        assert info.ier == 0 and info.eps <= 1e-12, (label, info.as_dict())
        assert np.linalg.norm(xg - xd) / nd <= max(1e-9, 2 * err_oracle), label


@pytest.mark.parametrize("balanced", ["auto", "4", "8"])
def test_batched_member_fault_is_isolated(gpu, systems, monkeypatch, balanced):
    """A NaN right-hand side (injected on the host) stops only its own member,
    with the tile kernels and with the balanced kernels' block tables."""
    import torch
    _force_balanced(monkeypatch, balanced)
    sys_list = []
    for k, (_, _, _, ds) in enumerate(systems):
        b = ds.b.clone()
        if k == 2:
            b[ds.mnoe // 3] = float("nan")
        sys_list.append((ds.alu, ds.llu, ds.de, b))
    sizes = [ds.mnoe for (_, _, _, ds) in systems]
    for prec in (gpu.PREC_FP64, gpu.PREC_MIXED):
        xs = [_x(ds) for (_, _, _, ds) in systems]
        infos = gpu.BatchedSolver(sizes, prec).solve(sys_list, xs, eps=1e-10)
        for k, info in enumerate(infos):
            if k == 2:
                assert info.ier == gpu.IER_NONFINITE, info.as_dict()
            else:
                assert info.ier == 0 and info.eps <= 1e-10, (k, info.as_dict())
    torch.cuda.synchronize()


@pytest.mark.parametrize("balanced", ["4", "8"])
def test_balanced_kernels_multi_step_ranges(gpu, ora, pkg, monkeypatch, balanced):
    """A 1.1 M-row beach, where the one-wave grid (at most 608 blocks of 256
    threads) is far smaller than the tile count and every thread walks more
    than one step of its block's uneven row range: FP64 pressure within 1e-10
    relative L2 of the oracle's (both to 1e-13), iterations within 25 %, and
    the graph's forced fused and single sweeps bit-identical."""
    import os
    case = pkg.workload.beach_192x192x64()
    cls, sm, sy = ora.prepare(case)
    dc, ds = gpu.prepare_dev(case)
    n = ds.mnoe
    assert n > 608 * 256 * 4                        # more than one step of 4 rows per thread
    ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-13, nthreads=os.cpu_count() or 1)
    monkeypatch.setenv("CLOWNS_LOOP_MODE", "graph")
    monkeypatch.setenv("CLOWNS_BALANCED_ROWS", balanced)
    out = []
    for fuse in ("0", "1"):
        monkeypatch.setenv("CLOWNS_SWEEP_FUSE", fuse)
        x = _x(ds)
        info = gpu.Solver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-13)
        assert info.ier == 0, info.as_dict()
        out.append((info.iter, x.cpu().numpy()[:n].copy()))
    assert out[0][0] == out[1][0] and np.array_equal(out[0][1], out[1][1])
    xg = out[0][1]
    assert np.linalg.norm(xg - ref.x) <= 1e-10 * np.linalg.norm(ref.x)
    assert abs(out[0][0] - ref.iters) <= max(5, ref.iters // 4), (out[0][0], ref.iters)
