"""Adjoint of the pressure solve: explicit transpose, gradient against the CPU
transposed solve (oracle) and against central finite differences (relative step
1e-6).  Tolerances: transpose bit-exact; adjoint gradient within 1e-8 relative
of the CPU transposed-solve gradient; within 1e-6 relative of finite
differences."""
import numpy as np
import pytest

import __graft_entry__ as ge
from cases import small_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def bore(gpu, ora):
    label, case = small_cases()[2]
    return case


def test_transpose_bit_exact_and_identity(gpu, ora, bore):
    import torch
    cls, sm, sy = ora.prepare(bore)
    dc, ds = gpu.prepare_dev(bore)
    n = sy.mnoe
    alt, llt, det = gpu.transpose_dev(ds.alu, ds.llu, ds.de, n)
    alt_o, llt_o, det_o = ora.transpose(sy.alu, sy.llu, sy.de[1:], n)
    assert np.array_equal(llt.cpu().numpy()[:, :n], llt_o[:, :n])
    assert np.array_equal(alt.cpu().numpy()[:, :n], alt_o[:, :n])
    rng = np.random.default_rng(1)
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    ax = ora.spmv(sy.alu, sy.llu, sy.de[1:], n, x)
    aty = ora.spmv(alt.cpu().numpy(), llt.cpu().numpy(), det.cpu().numpy(), n, y)
    assert abs(ax @ y - x @ aty) <= 1e-12 * abs(ax @ y)
    torch.cuda.synchronize()


def _cpu_face_grad(case, cls, sm, sy, x, lam):
    """dJ/da from the assembled arrays (numpy restatement of -lambda^T dA/da x)."""
    n = sy.mnoe
    g = np.zeros_like(case.a)
    rows = sy.mno2mn[1:n + 1]
    mno = sy.mno.reshape(-1)
    ie, ke = int(case.dims[3]), int(case.dims[5])

    def row_of(cell):
        i, j, k = case.in_[cell], case.jn[cell], case.kn[cell]
        return mno[(i - 1) + ie * ((k - 1) + ke * (j - 1))]

    for r, c in enumerate(rows, start=1):
        if cls.nf[c] != 1:
            continue
        for ll in range(6):
            lc = sm.ll_c[ll, c - 1]
            if lc == 0:
                continue
            owner = lc if ll % 2 else c
            l = ll // 2
            af = case.a[owner, l]
            if af == 0:
                continue
            dco = sm.alu_c[ll, c - 1] / af
            npr = row_of(lc)
            if cls.nf[lc] == 0 or npr == 0:
                if cls.nf[lc] != 2:
                    continue
                g[owner, l] += lam[r - 1] * dco * x[r - 1]
            else:
                g[owner, l] += -lam[r - 1] * dco * (x[npr - 1] - x[r - 1])
    return g


def test_adjoint_matches_cpu_transposed_solve(gpu, ora, bore):
    import torch
    from adjoint_harness import gauges
    cls, sm, sy = ora.prepare(bore)
    dc, ds = gpu.prepare_dev(bore)
    n = sy.mnoe
    rows, w = gauges(n)
    djdx = np.zeros(n)
    djdx[rows] = w
    x = torch.zeros(ds.mm2, dtype=torch.float64, device="cuda")
    gpu.Solver(n).solve(ds.alu, ds.llu, ds.de, ds.b, x, eps=1e-13)
    lam, grad_a, info = gpu.adjoint_dev(dc, ds, x, torch.from_numpy(djdx).cuda(), eps=1e-13)
    assert info.ier == 0
    # CPU reference gradient: PCGPME on the oracle's transpose, then the formula
    alt, llt, det = ora.transpose(sy.alu, sy.llu, sy.de[1:], n)
    rt = ora.pcgpme(alt, llt, det, djdx, n, eps=1e-13)
    xr = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-13).x
    lam_c = rt.x
    g_c = _cpu_face_grad(bore, cls, sm, sy, xr, lam_c)
    lam_g = lam.cpu().numpy()
    g_g = grad_a.cpu().numpy()
    assert np.linalg.norm(lam_g - lam_c) <= 1e-8 * np.linalg.norm(lam_c)
    assert np.linalg.norm(g_g - g_c) <= 1e-8 * np.linalg.norm(g_c)
    # the adjoint identity: w.x == lambda.b
    xg = x.cpu().numpy()[:n]
    assert abs(w @ xg[rows] - lam_g @ sy.b[1:n + 1]) <= 1e-10 * abs(w @ xg[rows])


def test_adjoint_matches_finite_differences(gpu, bore):
    """Central differences with relative step 1e-6 on 40 seeded face fractions,
    through the autograd wrapper.  The difference quotient is evaluated through
    the exact identity x(a+h) - x(a-h) = -A(a+h)^-1 [A(a+h) - A(a-h)] x(a-h)
    (see adjoint_harness.central_difference): two perturbed assemblies, a solve
    at a-h refined to the FP64 floor and a solve for the difference.  Also a
    plain two-solve difference, which FP64 resolution limits to ~1e-5."""
    import torch
    from adjoint_harness import PressureSolve, PressureSystem, central_difference, fd_faces, gauges
    system = PressureSystem(bore)
    n = system.n
    rows, w = gauges(n)
    wt = torch.zeros(n, dtype=torch.float64, device="cuda")
    wt[torch.from_numpy(rows).cuda()] = torch.from_numpy(w).cuda()
    a0 = system.dc.a.clone()
    a = a0.clone().requires_grad_(True)
    b = system.b0[:n].clone().requires_grad_(True)
    x = PressureSolve.apply(a, b, system)
    J = (wt * x).sum()
    J.backward()
    ga = a.grad.cpu().numpy()
    faces = fd_faces(system, count=40)
    assert len(faces) >= 20
    x0 = x.detach()
    fd, fd2, ad = [], [], []
    for owner, l in faces:
        fd.append(central_difference(system, wt, a0, owner, l, x0))
        h = 1e-6 * float(a0[owner, l])
        xs = []
        for sgn in (1.0, -1.0):
            ap = a0.clone()
            ap[owner, l] += sgn * h
            system.assemble(ap)
            xsol, info = system.solve_refined(system.b0, x0)
            xs.append(xsol)
        fd2.append(float((wt * (xs[0] - xs[1])).sum()) / (2 * h))
        ad.append(ga[owner, l])
    fd, fd2, ad = np.array(fd), np.array(fd2), np.array(ad)
    assert np.linalg.norm(ad - fd) <= 1e-6 * np.linalg.norm(fd), np.linalg.norm(ad - fd) / np.linalg.norm(fd)
    assert np.linalg.norm(ad - fd2) <= 1e-4 * np.linalg.norm(fd2)
    # dJ/db = lambda along a random direction: x(b+hv) - x(b-hv) = A^-1 (2 h v) exactly
    system.assemble(a0)
    rng = np.random.default_rng(2)
    v = torch.from_numpy(rng.standard_normal(n)).cuda()
    rhs = torch.zeros(system.sy.mm2, dtype=torch.float64, device="cuda")
    rhs[:n] = v
    dxv, _ = system.solve(rhs, eps=1e-13)
    assert abs(float((wt * dxv).sum()) - float((b.grad * v).sum())) <= 1e-8 * abs(float((b.grad * v).sum()))
