"""Parity on the benchmark configurations at their stated sizes.

  tank_64x64x32       flat tank, 86 k rows, tolerance 1e-12
  beach_256x256x96    the headline workload, 2.8 M rows, tolerance 1e-10
  beach_512x384x128   mixed precision, 8.5 M rows, against the FP64 oracle
  ensemble            64 seeded members of 96-256 x 96-192 x 48-80 cells
  beach_192x192x64    adjoint gradient on 200 seeded faces

For the two FP64 configurations the cell classification (flags, fluid and
surface lists), the row numbering, the right-hand side, the assembled matrix and
the row-scaled, sorted matrix PCGPME iterates with must equal the oracle's bit
for bit; the pressure solved to ERR <= 1e-13 must lie within 1e-10 relative L2
of the oracle's.  At the configuration's own tolerance eps the GPU pressure is
checked without the oracle's solve, whose OpenMP reductions stop it at a
different place inside the same ERR ball from run to run: its true residual
||b - A x|| / ||b|| against the assembled matrix must be within 2 eps, and its
distance to the tightly converged pressure within 10 eps (the bounds of the
small parity cases; the oracle's own distance is reported beside it).
Iteration counts are reported in the assertion messages, not bounded: they
follow the rounding of the dot products near the stop tests."""
import os

import numpy as np
import pytest

import __graft_entry__ as ge

pytestmark = pytest.mark.gpu

wl = ge.load_package().workload
THREADS = os.cpu_count() or 1


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _fp64_config(gpu, ora, case):
    import torch
    cls, sm, sy = ora.prepare(case)
    dc, ds = gpu.prepare_dev(case)
    torch.cuda.synchronize()
    n = sy.mnoe
    # classification, rows, right-hand side, assembly: bit for bit
    assert ds.ifln == cls.ifln and ds.isfn == cls.isfn
    assert np.array_equal(dc.nf.cpu().numpy(), cls.nf)
    assert np.array_equal(dc.nfb.cpu().numpy(), cls.nfb)
    assert np.array_equal(dc.f.cpu().numpy(), cls.f)
    assert np.array_equal(ds.fln.cpu().numpy(), cls.fln[1:])
    assert np.array_equal(ds.sfn.cpu().numpy(), cls.sfn[1:])
    assert float(ds.mp.item()) == sm.mp
    assert np.array_equal(ds.ll_c.cpu().numpy(), sm.ll_c)
    assert np.array_equal(ds.alu_c.cpu().numpy().view(np.int64), sm.alu_c.view(np.int64))
    assert ds.mnoe == n and ds.dmax == sy.dmax
    assert np.array_equal(ds.mno.cpu().numpy(), sy.mno)
    assert np.array_equal(ds.mno2mn.cpu().numpy()[:n], sy.mno2mn[1:n + 1])
    assert np.array_equal(ds.b.cpu().numpy()[:n].view(np.int64), sy.b[1:n + 1].view(np.int64))
    assert np.array_equal(ds.llu.cpu().numpy()[:, :n], sy.llu[:, :n])
    assert np.array_equal(ds.alu.cpu().numpy()[:, :n].view(np.int64), sy.alu[:, :n].view(np.int64))
    assert np.array_equal(ds.de.cpu().numpy()[:n].view(np.int64), sy.de[1:n + 1].view(np.int64))
    # PCGPME's row scaling and per-row sort (pcgpme_para.F90:77-112)
    al_s, ll_s, d_s, b_s = gpu.setup_scaled_dev(ds.alu, ds.llu, ds.de, ds.b, n)
    al_o, ll_o, d_o, b_o = ora.setup_scaled(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n)
    assert np.array_equal(ll_s.cpu().numpy(), np.where(ll_o[:, :n] > n, n, ll_o[:, :n] - 1))
    assert np.array_equal(al_s.cpu().numpy().view(np.int64), al_o[:, :n].view(np.int64))
    assert np.array_equal(d_s.cpu().numpy().view(np.int64), d_o.view(np.int64))
    assert np.array_equal(b_s.cpu().numpy().view(np.int64), b_o.view(np.int64))
    del al_s, ll_s, d_s, b_s
    # the solve
    solver = gpu.Solver(n)
    out = {}
    for eps in (1e-13, case.eps0):
        x = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
        info = solver.solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=eps)
        ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=eps, nthreads=THREADS)
        assert info.ier == 0 and ref.ier == 0, (eps, info.as_dict(), ref.ier)
        out[eps] = (x.cpu().numpy()[:n], info, ref)
    xg13, i13, r13 = out[1e-13]
    rel13 = _rel(xg13, r13.x)
    assert rel13 <= 1e-10, (case.label, rel13, "iters gpu/oracle", i13.iter, r13.iters)
    xg, info, ref = out[case.eps0]
    d_gpu, d_ora = _rel(xg, r13.x), _rel(ref.x, r13.x)
    b = sy.b[1:n + 1]
    true_res = float(np.linalg.norm(b - ora.to_csr(sy) @ xg) / np.linalg.norm(b))
    msg = (case.label, "true residual", true_res, "distance to the 1e-13 pressure gpu/oracle", d_gpu, d_ora,
           "iters gpu/oracle", info.iter, ref.iters)
    assert info.eps <= case.eps0 and info.reason in (0, 1), msg
    assert true_res <= 2 * case.eps0, msg
    assert d_gpu <= 10 * case.eps0, msg


def test_config_tank_64x64x32(gpu, ora):
    _fp64_config(gpu, ora, wl.tank_64x64x32())


def test_config_beach_256x256x96(gpu, ora):
    _fp64_config(gpu, ora, wl.beach_256x256x96())


def test_config_mixed_beach_512x384x128(gpu, ora):
    """FP32 storage with FP64 refinement, solved to ERR <= 1e-10: within 1e-9
    relative L2 of the FP64 oracle's pressure at the same tolerance."""
    import torch
    case = wl.beach_512x384x128()
    cls, sm, sy = ora.prepare(case)
    dc, ds = gpu.prepare_dev(case)
    n = sy.mnoe
    x = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
    info = gpu.MixedSolver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=case.eps0)
    assert info.ier == 0 and info.eps <= case.eps0, info.as_dict()
    ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=case.eps0, nthreads=THREADS)
    assert ref.ier == 0
    rel = _rel(x.cpu().numpy()[:n], ref.x)
    assert rel <= 1e-9, (rel, "inner iterations", info.iter, "sweeps", info.outer, "oracle iters", ref.iters)


def test_config_ensemble_64_members(gpu, ora):
    """The 64-member ensemble: every member's batched solve equals its own
    single-system solve bit for bit, in FP64 and in mixed precision, and every
    member reaches ERR <= 1e-10; three members' FP64 pressures are checked
    against the oracle (within 1e-10 relative L2 at ERR <= 1e-13 on both)."""
    import torch
    specs = wl.ensemble_members(n=64, seed=3)
    systems, cases = [], []
    for sp in specs:
        case = wl.ensemble_case(sp)
        dc, ds = gpu.prepare_dev(case)
        del dc
        systems.append(ds)
        cases.append(case)
    torch.cuda.synchronize()
    sizes = [ds.mnoe for ds in systems]
    sys_list = [(ds.alu, ds.llu, ds.de, ds.b) for ds in systems]
    for prec in (gpu.PREC_FP64, gpu.PREC_MIXED):
        xs = [torch.zeros(ds.mm2, dtype=torch.float64, device="cuda") for ds in systems]
        infos = gpu.BatchedSolver(sizes, prec).solve(sys_list, xs, eps=1e-10)
        single = gpu.Solver if prec == gpu.PREC_FP64 else gpu.MixedSolver
        for m, (ds, x, info) in enumerate(zip(systems, xs, infos)):
            x1 = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
            i1 = single(ds.mnoe).solve(ds.alu, ds.llu, ds.de, ds.b, x1, eps=1e-10)
            assert info.ier == 0 and info.eps <= 1e-10, (m, prec, info.as_dict())
            assert (info.iter, info.outer, info.eps) == (i1.iter, i1.outer, i1.eps), (m, prec)
            assert torch.equal(x[:ds.mnoe], x1[:ds.mnoe]), (m, prec)
        del xs
    for m in (0, 21, 42):
        case, ds = cases[m], systems[m]
        cls, sm, sy = ora.prepare(case)
        assert sy.mnoe == ds.mnoe
        x = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
        gpu.Solver(ds.mnoe).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-13)
        ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe, eps=1e-13, nthreads=THREADS)
        assert _rel(x.cpu().numpy()[:sy.mnoe], ref.x) <= 1e-10, m


def test_config_adjoint_beach_192x192x64(gpu):
    """J = sum of 16 seeded gauge pressures with weights U(0.5, 1.5): the adjoint
    gradient on 200 seeded face fractions is within 1e-6 relative L2 of central
    differences at relative step 1e-6 (evaluated through the exact difference
    identity, so cancellation does not limit them)."""
    import torch
    from adjoint_harness import PressureSolve, PressureSystem, central_difference, fd_faces, gauges
    case = wl.beach_192x192x64()
    system = PressureSystem(case)
    n = system.n
    rows, w = gauges(n)
    wt = torch.zeros(n, dtype=torch.float64, device="cuda")
    wt[torch.from_numpy(rows).cuda()] = torch.from_numpy(w).cuda()
    a0 = system.dc.a.clone()
    a = a0.clone().requires_grad_(True)
    b = system.b0[:n].clone().requires_grad_(True)
    x = PressureSolve.apply(a, b, system)
    (wt * x).sum().backward()
    ga = a.grad.cpu().numpy()
    faces = fd_faces(system, count=200)
    assert len(faces) == 200
    fd = np.array([central_difference(system, wt, a0, owner, l, x.detach()) for owner, l in faces])
    ad = np.array([ga[owner, l] for owner, l in faces])
    err = float(np.linalg.norm(ad - fd) / np.linalg.norm(fd))
    assert err <= 1e-6, err
    assert torch.isfinite(b.grad).all() and float(b.grad[torch.from_numpy(rows).cuda()].abs().min()) > 0.0
