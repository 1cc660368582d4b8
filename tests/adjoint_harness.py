"""Check harness for the discrete adjoint: a torch.autograd.Function whose
forward assembles the pressure matrix from the face area fractions ``a`` and
solves it on the GPU, and whose backward runs the adjoint solve on the explicit
transpose plus the face-gradient kernel.  Used only by the tests."""
import numpy as np
import torch

import __graft_entry__ as ge

pkg = ge.load_package()


class PressureSystem:
    """Classification fixed, matrix rebuilt from ``a`` on every forward."""

    def __init__(self, case):
        self.case = case
        self.dc, self.sy = pkg.prepare_dev(case)
        self.n = self.sy.mnoe
        self.b0 = self.sy.b.clone()          # right-hand side held fixed (independent input)
        self.solver = pkg.Solver(self.n)

    def assemble(self, a_dev):
        """init_matrix + cal_matrix_element for face fractions a_dev (inne2+2, 3)."""
        self.dc.a.copy_(a_dev)
        mp, alu_c, ll_c, de_c = pkg.init_matrix_dev(self.dc)
        r = pkg.rows_rhs_assemble_dev(self.dc, self.sy.fln, self.sy.ifln, mp, alu_c, ll_c, de_c, mm2=self.sy.mm2)
        self.sy.alu, self.sy.llu, self.sy.de = r["alu"], r["llu"], r["de"]
        self.sy.alu_c, self.sy.ll_c = alu_c, ll_c
        self.sy.mno = r["mno"]
        return self.sy

    def solve(self, b, x0=None, eps=1e-13):
        x = torch.zeros(self.sy.mm2, dtype=torch.float64, device="cuda")
        if x0 is not None:
            x[:self.n] = x0[:self.n]
        info = self.solver.solve(self.sy.alu, self.sy.llu, self.sy.de, b, x, eps=eps)
        return x[:self.n].clone(), info

    def solve_refined(self, b, x0):
        """Warm-started solve driven to the FP64 floor by iterative refinement on
        the true residual (used for finite differences: the perturbation of x is
        resolved to ~1e-10 of itself, which a tolerance-stopped solve does not)."""
        if not hasattr(self, "msolver"):
            self.msolver = pkg.MixedSolver(self.n)
        x = torch.zeros(self.sy.mm2, dtype=torch.float64, device="cuda")
        x[:self.n] = x0[:self.n]
        info = self.msolver.solve(self.sy.alu, self.sy.llu, self.sy.de, b, x, eps=2e-15, inner_tol=1e-5,
                                  max_outer=12)
        return x[:self.n].clone(), info


def ell_apply(alu, llu, de, x, n):
    """y = A x for an assembled ELL matrix on the device (1-based llu, 0 = none)."""
    y = de[:n] * x[:n]
    for k in range(alu.shape[0]):
        c = llu[k, :n].long()
        m = c > 0
        y = y + torch.where(m, alu[k, :n] * x[(c - 1).clamp(min=0)], torch.zeros_like(y))
    return y


def central_difference(system, wt, a0, owner, l, x_minus_guess, h_rel=1e-6):
    """(J(a+h) - J(a-h)) / 2h for one face fraction, with the difference of the
    two pressures evaluated through the exact identity
        x(a+h) - x(a-h) = -A(a+h)^{-1} [A(a+h) - A(a-h)] x(a-h),
    so it is resolved to the solver's relative accuracy instead of being lost
    to cancellation between two nearly equal pressures."""
    n = system.n
    h = h_rel * float(a0[owner, l])
    am = a0.clone()
    am[owner, l] -= h
    system.assemble(am)
    x_m, _ = system.solve_refined(system.b0, x_minus_guess)
    alu_m, llu_m, de_m = system.sy.alu.clone(), system.sy.llu.clone(), system.sy.de.clone()
    ap = a0.clone()
    ap[owner, l] += h
    system.assemble(ap)
    assert torch.equal(system.sy.llu, llu_m)          # same structure on both sides
    rhs = torch.zeros(system.sy.mm2, dtype=torch.float64, device="cuda")
    rhs[:n] = -(ell_apply(system.sy.alu, llu_m, system.sy.de, x_m, n) - ell_apply(alu_m, llu_m, de_m, x_m, n))
    dx, info = system.solve(rhs, eps=1e-13)
    return float((wt * dx).sum()) / (2 * h)


class PressureSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, b, system: PressureSystem):
        system.assemble(a.detach())
        bb = torch.zeros(system.sy.mm2, dtype=torch.float64, device="cuda")
        bb[:system.n] = b.detach()
        x, info = system.solve(bb)
        ctx.system = system
        ctx.save_for_backward(x)
        return x

    @staticmethod
    def backward(ctx, gx):
        system = ctx.system
        (x,) = ctx.saved_tensors
        lam, grad_a, info = pkg.adjoint_dev(system.dc, system.sy, x, gx.contiguous(), eps=1e-13,
                                            solver=system.solver)
        return grad_a, lam, None


def gauges(n, count=16, seed=4):
    rng = np.random.default_rng(seed)
    rows = rng.choice(n, size=count, replace=False)
    w = rng.uniform(0.5, 1.5, size=count)
    return rows, w


def fd_faces(system: PressureSystem, count=200, seed=5):
    """Seeded faces (l, owner) whose coefficient enters a fluid row of A."""
    sy = system.sy
    dc = system.dc
    rng = np.random.default_rng(seed)
    nf = dc.nf.cpu().numpy()
    a = dc.a.cpu().numpy()
    ll_c = sy.ll_c.cpu().numpy()
    mno2mn = sy.mno2mn.cpu().numpy()[:system.n]
    cand = []
    for c in mno2mn[rng.permutation(len(mno2mn))[:20 * count]]:
        if nf[c] != 1:
            continue
        for ll in range(6):
            lc = ll_c[ll, c - 1]
            if lc == 0:
                continue
            owner = lc if ll % 2 else c
            l = ll // 2
            if a[owner, l] > 0 and nf[lc] == 1:
                cand.append((int(owner), l))
        if len(set(cand)) >= count:
            break
    return sorted(set(cand))[:count]
