"""Generate tests/golden/*.npz: known answers for tiny grids, computed by a second,
independent restatement of the reference written as plain Python loops.

The reference (Fortran, ifort-only) cannot run here and ships no fixtures, so
these vectors pin the C oracle against an implementation that shares none of
its code: scalar loops transcribed separately from

  set_nflag            src2LOWNS/nfd2015.F90:7-306, fxx1 308-332
  init_matrix          src2LOWNS/1sub-matrix.F90:3-95 (3D and the 2DV mode of a grid
                       one cell wide in x or y, main_2CLOWNS.F90:43-44)
  rows + RHS           src2LOWNS/1sub-momentum.F90:265-360, 1sub-main.F90:579-602,
                       lib/src/math_func.F90:51-54
  cal_matrix_element   src2LOWNS/1sub-momentum.F90:465-551
  PCGPME               src2LOWNS/pcgpme_para.F90:1-354

Python floats are IEEE doubles and every expression keeps the Fortran order, so
the C oracle must reproduce these outputs bit for bit (the solve too: both run
the serial loop order).

Usage:  python tests/golden/make_golden.py   (rewrites the .npz files)
"""
from __future__ import annotations

import math
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
import __graft_entry__ as ge  # noqa: E402

wl = ge.load_package().workload


def golden_cases():
    return {
        "tank_6x5x6": wl.make_case(6, 5, 6, dz=0.025, depth=0.1, partial=False, seed=21, eps0=1e-12),
        "beach_10x6x8": wl.make_case(10, 6, 8, dz=0.1, slope=0.25, n_obstacles=1, obstacle_frac=0.08,
                                     seed=22, amplitude=0.06),
        "bore_12x5x8": wl.make_case(12, 5, 8, dz=0.1, slope=None, n_obstacles=1, obstacle_frac=0.05,
                                    seed=23, amplitude=0.06, step_layers=2, step_at=0.5),
        # 2DV (NL = 4): one cell wide in y (x-z flume), and one cell wide in x (y-z section)
        "flume2dv_16x1x8": wl.make_case(16, 1, 8, dz=0.1, slope=0.25, n_obstacles=0, seed=24,
                                        amplitude=0.06, step_layers=2, step_at=0.5),
        "section2dv_1x14x8": wl.make_case(1, 14, 8, dz=0.1, slope=None, n_obstacles=0, seed=25,
                                          amplitude=0.06),
    }


class Ref:
    """Pure-Python view of one case with Fortran-style index helpers."""

    def __init__(self, c):
        self.c = c
        self.is_, self.js, self.ks, self.ie, self.je, self.ke = (int(v) for v in c.dims)
        self.mn3 = c.mn  # (NJ, NK, NI)
        self.nf = [int(v) for v in c.nf]
        self.nfb = [int(v) for v in c.nfb]
        self.f = [float(v) for v in c.f]
        self.fb = [float(v) for v in c.fb]
        self.a = [[float(c.a[nn, l]) for l in range(3)] for nn in range(c.inne2 + 2)]
        self.un = [[float(c.un[nn, l]) for l in range(3)] for nn in range(c.inne2 + 2)]
        self.sp = [[float(c.sp[l, nn]) for l in range(3)] for nn in range(c.inne2 + 2)]
        self.in_ = [int(v) for v in c.in_]
        self.jn = [int(v) for v in c.jn]
        self.kn = [int(v) for v in c.kn]
        self.objno = [int(v) for v in c.objno]
        # 2DV switch of main_2CLOWNS.F90:43-44 and nl of init_matrix (1sub-matrix.F90:15-21)
        self.cx = self.is_ == self.ie - 1
        self.cy = self.js == self.je - 1
        self.nl = 4 if (self.cx or self.cy) else 6

    def mn(self, i, k, j):
        return int(self.mn3[j - (self.js - 2), k - (self.ks - 2), i - (self.is_ - 2)])

    def X(self, l, i):
        return float(self.c.x[i - 1, l])

    def DX(self, l, i):
        return float(self.c.dx[i - 1, l])

    def nb(self, i, j, k, l, s):
        return self.mn(i + s * (l == 0), k + s * (l == 2), j + s * (l == 1))


def set_nflag(R: Ref):
    nf, nfb, f, fb, a = R.nf, R.nfb, R.f, R.fb, R.a
    imax = kmax = 0
    for nn in range(1, R.c.inne + 1):
        if nf[nn] == -1:
            continue
        i, j, k = R.in_[nn], R.jn[nn], R.kn[nn]
        if f[nn] <= 1e-12 or (f[nn] * fb[nn] < 1e-3 and nf[R.mn(i, k - 1, j)] == -1
                              and f[R.mn(i, k + 1, j)] == 0.0):
            nf[nn] = 0
            nfb[nn] = 0
            f[nn] = max(0.0, f[nn])
        else:
            nf[nn] = 1
            nfb[nn] = 0
            imax = max(imax, i)
            kmax = max(kmax, k)
    imax = min(R.ie - 1, imax + 1)
    kmax = min(R.ke - 1, kmax + 1)
    passes = 0
    while True:
        passes += 1
        fln, sfn = [0], [0]
        for k in range(R.ks, kmax + 1):
            for j in range(R.js, R.je):
                for i in range(R.is_, imax + 1):
                    nn = R.mn(i, k, j)
                    if nf[nn] == -1 or nf[nn] < 1:
                        continue
                    fln.append(nn)
                    surf = False
                    for l in range(3):
                        p = R.nb(i, j, k, l, 1)
                        m = R.nb(i, j, k, l, -1)
                        if nf[p] == 0 and a[p][l] > 0.0:
                            surf = True
                            break
                        if nf[m] == 0 and a[nn][l] > 0.0:
                            surf = True
                            break
                    if surf:
                        nf[nn] = 2
                        sfn.append(nn)
                        nfb[nn] = -3
                    else:
                        nf[nn] = 1
        restart = False
        for p in range(len(sfn) - 1, 0, -1):
            nn = sfn[p]
            i, j, k = R.in_[nn], R.jn[nn], R.kn[nn]
            if nf[R.mn(i, k - 1, j)] == -1:
                continue
            if any(nf[R.nb(i, j, k, l, 1)] == 1 or nf[R.nb(i, j, k, l, -1)] == 1 for l in range(3)):
                continue
            restart = True
            nf[nn] = 0
            nfb[nn] = 0
        if restart:
            continue
        for p in range(len(sfn) - 1, 0, -1):
            nn = sfn[p]
            i, j, k = R.in_[nn], R.jn[nn], R.kn[nn]
            if nf[R.mn(i, k - 1, j)] == -1 and nf[R.mn(i, k + 1, j)] == 0:
                continue
            keep = False
            for l in range(3):
                pv, mv = nf[R.nb(i, j, k, l, 1)], nf[R.nb(i, j, k, l, -1)]
                if (pv == 1 and mv == 0) or (mv == 1 and pv == 0):
                    keep = True
                    break
            if not keep:
                restart = True
                nf[nn] = 0
                nfb[nn] = 0
        if restart:
            continue
        igai = 0
        for p in range(len(sfn) - 1, 0, -1):
            nn = sfn[p]
            i, j, k = R.in_[nn], R.jn[nn], R.kn[nn]
            nfb[nn] = 0
            ix = [0, 0, 0]
            for l in range(3):
                m, pc = R.nb(i, j, k, l, -1), R.nb(i, j, k, l, 1)
                if nf[m] == 1 and nf[pc] == 0 and a[pc][l] > 0.0:
                    ix[l] = -1
                elif nf[m] == 0 and nf[pc] == 1 and a[nn][l] > 0.0:
                    ix[l] = 1
            if sum(map(abs, ix)) == 0 and nf[R.mn(i, k - 1, j)] == -1 and nf[R.mn(i, k + 1, j)] == 0:
                if R.objno[nn] != 0 or fb[nn] != 0.0:
                    ix[2] = -1
                else:
                    for l in range(2):
                        m, pc = R.nb(i, j, k, l, -1), R.nb(i, j, k, l, 1)
                        if nf[m] > 0 and nf[pc] == 0 and a[pc][l] > 0.0:
                            ix[l] = -1
                        elif nf[m] == 0 and nf[pc] > 0 and a[nn][l] > 0.0:
                            ix[l] = 1
                    if abs(ix[0]) + abs(ix[1]) == 0:
                        ix[2] = -1
            s = sum(map(abs, ix))
            if s == 1:
                d = [abs(v) for v in ix].index(1) + 1
                nfb[nn] = d * ix[d - 1]
            elif s == 0:
                igai += 1
                nf[nn] = 0
            else:
                fx = [0.0 if ix[l] == 0 else fxx1(R, ix[l], l, i, j, k) for l in range(3)]
                d = fx.index(max(fx)) + 1
                nfb[nn] = d * ix[d - 1]
        if igai:
            continue
        return fln, sfn, passes


def fxx1(R: Ref, ix, ll, i, j, k):
    lg = [i, j, k]
    r = 0.0
    for l in range(3):
        if l == ll:
            continue
        if R.cx and l == 0:
            continue
        if R.cy and l == 1:
            continue
        for ii in (-1, 0, 1):
            nnc = R.mn(lg[0] + ix * (ll == 0) + ii * (l == 0), lg[2] + ix * (ll == 2) + ii * (l == 2),
                       lg[1] + ix * (ll == 1) + ii * (l == 1))
            r = r + R.DX(l, lg[l] + ii) * R.f[nnc] * R.fb[nnc]
        for lll in range(3):
            if lll == l or lll == ll:
                continue
            r = r * R.DX(lll, lg[lll])
    return r * R.DX(ll, lg[ll] + ix)


def init_matrix(R: Ref):
    if R.nl == 6:
        comps = (0, 1, 2)
    else:                           # the later of the two 2DV assignments wins (lines 20-21)
        comps = (0, 2) if R.cy else ()
        comps = (1, 2) if R.cx else comps
    dxs = [float(R.c.dx[i, l]) for i in range(R.c.dx.shape[0]) for l in comps if R.c.dx[i, l] > 0.0]
    m = min(dxs)
    mp = m * m
    n = R.c.inne
    alu_c = [[0.0] * n for _ in range(R.nl)]
    ll_c = [[0] * n for _ in range(R.nl)]
    de_c = [0.0] * n
    for nnn in range(1, n + 1):
        if R.nf[nnn] == -1 or R.fb[nnn] == 0.0:
            continue
        i, j, k = R.in_[nnn], R.jn[nnn], R.kn[nnn]
        lg = [i, j, k]
        de = 0.0
        ll = 0
        for l in range(3):
            if R.cx and l == 0:
                continue
            if R.cy and l == 1:
                continue
            ll += 1
            for side, ii in enumerate((-1, 1)):
                np_ = R.nb(i, j, k, l, ii)
                npp = R.nb(i, j, k, l, max(0, ii))
                col = 2 * (ll - 1) + side
                if (R.nf[np_] == -1 and R.nfb[np_] != 4) or R.a[npp][l] == 0.0 or R.fb[np_] == 0.0:
                    continue
                dx, dxm = R.DX(l, lg[l]), R.DX(l, lg[l] + ii)
                v = -(mp * (2.0 / dx / (dx + dxm) * R.a[npp][l] / R.fb[nnn]))
                alu_c[col][nnn - 1] = v
                ll_c[col][nnn - 1] = np_
                de = de - v
        de_c[nnn - 1] = de
    return mp, alu_c, ll_c, de_c


def rows_rhs_assemble(R: Ref, fln, mp, alu_c, ll_c, de_c, mm2):
    c = R.c
    mno = {}
    mno2mn = [0]
    for nnn in fln[1:]:
        i, j, k = R.in_[nnn], R.jn[nnn], R.kn[nnn]
        if R.nf[nnn] in (0, -1) or R.fb[nnn] == 0.0:
            continue
        if R.nf[nnn] == 2:
            l = abs(R.nfb[nnn]) - 1
            s = 1 if R.nfb[nnn] >= 0 else -1
            if 0 <= l <= 2 and R.nf[R.nb(i, j, k, l, s)] == -1:
                continue
        mno2mn.append(nnn)
        mno[(i, k, j)] = len(mno2mn) - 1
    mnoe = len(mno2mn) - 1
    b = [0.0] * (mm2 + 1)
    dmax = 0.0
    if mnoe >= 10:
        for r in range(1, mnoe + 1):
            cc = mno2mn[r]
            if R.nf[cc] != 1:
                continue
            i, j, k = R.in_[cc], R.jn[cc], R.kn[cc]
            ff = max(-0.001, min(1.0 - R.f[cc], 0.001))
            ip, jp, kp = R.mn(i + 1, k, j), R.mn(i, k, j + 1), R.mn(i, k + 1, j)
            rz = ((R.un[ip][0] * R.a[ip][0] - R.un[cc][0] * R.a[cc][0]) / R.DX(0, i)
                  + (R.un[jp][1] * R.a[jp][1] - R.un[cc][1] * R.a[cc][1]) / R.DX(1, j)
                  + (R.un[kp][2] * R.a[kp][2] - R.un[cc][2] * R.a[cc][2]) / R.DX(2, k)) / R.fb[cc]
            dr1 = rz + ff / c.dt
            q = dr1 / c.dt
            if not (abs(q) <= 1e-15 and abs(q) != 0.0):
                b[r] = mp * dr1 / c.dt
            dmax = max(dmax, abs(dr1))
    alu = [[0.0] * mm2 for _ in range(R.nl)]
    llu = [[0] * mm2 for _ in range(R.nl)]
    de = [0.0] * (mm2 + 1)
    for nnn in fln[1:]:
        i, j, k = R.in_[nnn], R.jn[nnn], R.kn[nnn]
        nn = mno.get((i, k, j), 0)
        if nn == 0:
            continue
        de[nn] = de_c[nnn - 1] if R.nf[nnn] == 1 else 1.0
        for ll in range(1, R.nl + 1):
            lc = ll_c[ll - 1][nnn - 1]
            if lc == 0:
                continue
            np_ = mno.get((R.in_[lc], R.kn[lc], R.jn[lc]), 0)
            if R.nf[lc] == 0 or np_ == 0:
                if R.nf[nnn] == 1 and R.nf[lc] != 2:
                    de[nn] = de[nn] + alu_c[ll - 1][nnn - 1]
                continue
            llu[ll - 1][nn - 1] = np_
            if R.nf[nnn] == 1:
                alu[ll - 1][nn - 1] = alu_c[ll - 1][nnn - 1]
            else:
                l = (ll + ll % 2) // 2 - 1
                if R.cx:                        # 1sub-momentum.F90:519-520
                    l = l + 1
                if R.cy and ll > 2:
                    l = l + 1
                if abs(R.nfb[nnn]) - 1 == l:
                    ii = (i, j, k)[l]
                    md = ll % 2
                    fss = float(1 - 2 * md) * (R.X(l, ii - md + 1) - R.sp[nnn][l]) / R.DX(l, ii)
                    dx, dxm = R.DX(l, ii), R.DX(l, ii - 2 * md + 1)
                    alu[ll - 1][nn - 1] = (fss - 0.5) * dx / (fss * dx + dxm * 0.5) * (-1.0)
                else:
                    alu[ll - 1][nn - 1] = -1.0e-20
    return mnoe, mno2mn, b, dmax, alu, llu, de


def pcgpme(alu, llu, de, b, n, eps, parm=5.0, itmax=10000):
    """PCGPME with the serial loop order; returns scaled/sorted AL, LL and the solve."""
    P1 = parm if parm >= 1.0 else 4.0
    P2 = P1 + 1.0
    N2 = 64
    NL = len(alu)
    AL = [[alu[k][i] for i in range(n)] for k in range(NL)]
    LL = [[llu[k][i] for i in range(n)] for k in range(NL)]
    D = [de[i + 1] for i in range(n)]
    B = [b[i + 1] for i in range(n)]
    for I in range(1, n + 1):
        w = 0.0
        for K in range(NL):
            if LL[K][I - 1] == 0:
                LL[K][I - 1] = n + 1 + I % 64
            w = w + abs(AL[K][I - 1])
        t = D[I - 1]
        w = P2 / (max(w, t) + t * P1)
        for K in range(NL):
            AL[K][I - 1] = AL[K][I - 1] * w
        D[I - 1] = D[I - 1] * w
        B[I - 1] = B[I - 1] * w
    for I in range(n):
        for K in range(NL - 1):
            for KK in range(K + 1, NL):
                if abs(AL[K][I]) < abs(AL[KK][I]):
                    AL[K][I], AL[KK][I] = AL[KK][I], AL[K][I]
                    LL[K][I], LL[KK][I] = LL[KK][I], LL[K][I]
    L = n + N2

    def axsub(x):
        if NL == 4:                     # vertical 2D (pcgpme_para.F90:340-345)
            return [x[i] * D[i] + AL[0][i] * x[LL[0][i] - 1] + AL[1][i] * x[LL[1][i] - 1]
                    + AL[2][i] * x[LL[2][i] - 1] + AL[3][i] * x[LL[3][i] - 1] for i in range(n)] + [0.0] * N2
        return [x[i] * D[i] + AL[0][i] * x[LL[0][i] - 1] + AL[1][i] * x[LL[1][i] - 1]
                + AL[2][i] * x[LL[2][i] - 1] + AL[3][i] * x[LL[3][i] - 1]
                + AL[4][i] * x[LL[4][i] - 1] + AL[5][i] * x[LL[5][i] - 1] for i in range(n)] + [0.0] * N2

    def ldusub(p):
        w = [p[i] - AL[0][i] * p[LL[0][i] - 1] for i in range(n)] + [0.0] * N2
        q = [w[i] - AL[1][i] * w[LL[1][i] - 1] for i in range(n)] + p[n:]
        w = [q[i] - AL[2][i] * q[LL[2][i] - 1] for i in range(n)] + [0.0] * N2
        q = [w[i] - AL[3][i] * w[LL[3][i] - 1] for i in range(n)] + p[n:]
        if NL <= 4:                     # sweeps 5 and 6 only when NL > 4 (pcgpme_para.F90:306)
            return q
        w = [q[i] - AL[4][i] * q[LL[4][i] - 1] - AL[5][i] * q[LL[5][i] - 1] for i in range(n)]
        return w + p[n:]

    X = [0.0] * L
    wk1 = ldusub(B + [0.0] * N2)
    wk3 = ldusub(axsub(X))
    BN = C1 = 0.0
    r = [0.0] * L
    for i in range(n):
        t = wk1[i]
        BN = BN + t * t
        t = t - wk3[i]
        r[i] = t
        C1 = C1 + t * t
    p = list(r)
    r0 = list(r)
    ERRP = 0.0
    ERR = 0.0
    K = 0
    ier = 0
    for K in range(1, itmax + 1):
        q = ldusub(axsub(p))
        RQ = 0.0
        for i in range(n):
            RQ = RQ + r0[i] * q[i]
        ALP = C1 / RQ
        e = [r[i] - ALP * q[i] for i in range(n)] + [0.0] * N2
        v = ldusub(axsub(e))
        AMU = SS = 0.0
        for i in range(n):
            AMU = AMU + e[i] * v[i]
            SS = SS + v[i] * v[i]
        AMU = AMU / SS
        C1 = RN = 0.0
        for i in range(n):
            X[i] = X[i] + ALP * p[i] + AMU * e[i]
            t = e[i] - AMU * v[i]
            r[i] = t
            RN = RN + t * t
            C1 = C1 + t * r0[i]
        ERR = math.sqrt(RN / BN)
        if K >= 10 and abs(ERR - ERRP) <= ERR * 1e-6:
            break
        if ERR <= eps:
            break
        ERRP = ERR
        if AMU == 0.0 or C1 == 0.0:
            break
        BETA = C1 / AMU / RQ
        p = [r[i] + BETA * (p[i] - AMU * q[i]) for i in range(n)] + [0.0] * N2
    else:
        ier = 3000
        K = itmax + 1
    return AL, LL, D, B, X[:n], K, ERR, ier


def main():
    for name, case in golden_cases().items():
        R = Ref(case)
        fln, sfn, passes = set_nflag(R)
        mp, alu_c, ll_c, de_c = init_matrix(R)
        mm2 = len(fln) - 1 + 5000
        mnoe, mno2mn, b, dmax, alu, llu, de = rows_rhs_assemble(R, fln, mp, alu_c, ll_c, de_c, mm2)
        als, lls, ds, bs, x, iters, err, ier = pcgpme(alu, llu, de, b, mnoe, case.eps0)
        np.savez_compressed(
            HERE / f"{name}.npz",
            nf=np.array(R.nf, np.int32), nfb=np.array(R.nfb, np.int32), f=np.array(R.f),
            fln=np.array(fln[1:], np.int32), sfn=np.array(sfn[1:], np.int32), passes=passes,
            mp=mp, alu_c=np.array(alu_c), ll_c=np.array(ll_c, np.int32), de_c=np.array(de_c),
            mnoe=mnoe, mno2mn=np.array(mno2mn[1:], np.int32), b=np.array(b[1:mnoe + 1]), dmax=dmax,
            alu=np.array(alu)[:, :mnoe], llu=np.array(llu, np.int32)[:, :mnoe],
            de=np.array(de[1:mnoe + 1]), al_sorted=np.array(als), ll_sorted=np.array(lls, np.int32),
            d_scaled=np.array(ds), b_scaled=np.array(bs), x=np.array(x), iters=iters, err=err,
            ier=ier, eps0=case.eps0)
        print(f"{name}: cells={case.inne} rows={mnoe} surface={len(sfn) - 1} passes={passes} "
              f"iters={iters} err={err:.3e}")


if __name__ == "__main__":
    main()
