"""PCGPME_WILL (src2LOWNS/pcgpme_2DH.f90:1-374) in the C oracle, pinned by an
independent pure-Python restatement of the same source on a small 2DH system
(bit for bit: both evaluate every expression in the source's order without
fused multiply-adds), and known answers for the post-processing
(pcgpme_2DH.f90:268-279)."""
import math

import numpy as np
import pytest

L_LIMIT = 1.0e-14


def py_postprocess(x, b, ll, n):
    """pcgpme_2DH.f90:268-279, serial; x, b lists (0-based), ll (nl, na) 1-based."""
    x = list(x)
    b = list(b)
    nl = ll.shape[0]
    for i in range(1, n + 1):
        if abs(x[i - 1]) <= L_LIMIT:
            x[i - 1] = 0.0
        for k in range(nl):
            j = int(ll[k, i - 1])
            if j == i:
                continue
            if j == 0:
                break
            if x[i - 1] == x[j - 1]:
                continue
            if abs(x[i - 1] - x[j - 1]) <= L_LIMIT:
                x[i - 1] = x[j - 1]
            b[i - 1] = x[i - 1]
    return x, b


def py_will(al, ll, d, b, n, eps, parm, itmax, n2=64):
    """pcgpme_2DH.f90:1-374 line by line (serial loops)."""
    nl = al.shape[0]
    A = [[float(al[k, i]) for i in range(n)] for k in range(nl)]
    LL = [[int(ll[k, i]) for i in range(n)] for k in range(nl)]
    D = [float(v) for v in d[:n]]
    B = [float(v) for v in b[:n]]
    size = n + n2
    X = [0.0] * size
    WK = [[0.0] * size for _ in range(5)]
    p1 = parm if parm >= 1.0 else 4.0
    p2 = p1 + 1.0
    for i in range(n):                                       # 81-111
        w = 0.0
        for k in range(nl):
            if LL[k][i] == 0:
                LL[k][i] = n + 1 + (i + 1) % 64
            w = w + abs(A[k][i])
        t = D[i]
        w = p2 / (max(w, t) + t * p1)
        for k in range(nl):
            A[k][i] = A[k][i] * w
        D[i] = D[i] * w
        B[i] = B[i] * w
    for k in range(nl - 1):                                  # 103-120
        for kk in range(k + 1, nl):
            for i in range(n):
                if abs(A[k][i]) < abs(A[kk][i]):
                    A[k][i], A[kk][i] = A[kk][i], A[k][i]
                    LL[k][i], LL[kk][i] = LL[kk][i], LL[k][i]

    def ldusub(P):
        W = [0.0] * size
        Q = list(P)
        for i in range(n):
            W[i] = P[i] - A[0][i] * P[LL[0][i] - 1]
        for i in range(n):
            Q[i] = W[i] - A[1][i] * W[LL[1][i] - 1]
        for i in range(n):
            W[i] = Q[i] - A[2][i] * Q[LL[2][i] - 1]
        for i in range(n):
            Q[i] = W[i] - A[3][i] * W[LL[3][i] - 1]
        return Q

    def axsub(Xv):
        Y = [0.0] * size
        for i in range(n):
            Y[i] = (Xv[i] * D[i] + A[0][i] * Xv[LL[0][i] - 1] + A[1][i] * Xv[LL[1][i] - 1]
                    + A[2][i] * Xv[LL[2][i] - 1] + A[3][i] * Xv[LL[3][i] - 1])
        return Y

    for i in range(n):
        WK[0][i] = B[i]
    WK[0] = ldusub(WK[0])
    WK[2] = ldusub(axsub(X))
    bn = 0.0
    c1 = 0.0
    for i in range(n):
        t = WK[0][i]
        bn = bn + t * t
        t = t - WK[2][i]
        B[i] = t
        c1 = c1 + t * t
        WK[0][i] = t
        WK[1][i] = t
    errp = 0.0
    iters = itmax
    for it in range(1, itmax + 1):
        WK[2] = ldusub(axsub(WK[0]))
        rq = 0.0
        for i in range(n):
            rq = rq + WK[1][i] * WK[2][i]
        alp = c1 / rq
        for i in range(n):
            WK[3][i] = B[i] - alp * WK[2][i]
        WK[4] = ldusub(axsub(WK[3]))
        amu = 0.0
        ss = 0.0
        for i in range(n):
            t = WK[4][i]
            amu = amu + WK[3][i] * t
            ss = ss + t * t
        amu = amu / ss
        c1 = 0.0
        rn = 0.0
        for i in range(n):
            t = WK[3][i]
            X[i] = X[i] + alp * WK[0][i] + amu * t
            t = t - amu * WK[4][i]
            B[i] = t
            rn = rn + t * t
            c1 = c1 + t * WK[1][i]
        err = math.sqrt(rn / bn)
        if it >= 10 and abs(err - errp) <= err * 1.0e-6:
            iters = it
            break
        if err <= eps:
            iters = it
            break
        errp = err
        if amu == 0.0 or c1 == 0.0:
            iters = it
            break
        beta = c1 / (amu * rq)
        for i in range(n):
            WK[0][i] = B[i] + beta * (WK[0][i] - amu * WK[2][i])
    x, bout = py_postprocess(X[:n], B, ll, n)
    return np.array(bout), iters


@pytest.fixture(scope="module")
def small(pkg):
    return pkg.workload.dispersion_system(14, 10, seed=5)


def test_oracle_will_matches_python_restatement(ora, small):
    ds = small
    b_c, it_c, reason = ora.pcgpme_will(ds.al, ds.ll, ds.d, ds.b, ds.n, eps=1e-12)
    b_p, it_p = py_will(ds.al, ds.ll, ds.d, ds.b, ds.n, 1e-12, 5.0, 10000)
    assert it_c == it_p
    assert np.array_equal(b_c, b_p)
    assert reason == 0


def test_oracle_will_solves_the_system(ora, pkg):
    """Rows with a neighbour hold the solution (scipy direct solve, 1e-9); rows
    whose neighbour list is empty keep the residual, as the reference does."""
    import scipy.sparse as sps
    import scipy.sparse.linalg as spl
    ds = pkg.workload.dispersion_system(60, 40, seed=9)
    n = ds.n
    b, it, reason = ora.pcgpme_will(ds.al, ds.ll, ds.d, ds.b, n, eps=1e-12)
    rows = [np.arange(n)]
    cols = [np.arange(n)]
    vals = [ds.d]
    for k in range(4):
        m = ds.ll[k] > 0
        rows.append(np.arange(n)[m])
        cols.append(ds.ll[k][m] - 1)
        vals.append(ds.al[k][m])
    A = sps.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    xd = spl.spsolve(A.tocsc(), ds.b)
    has = ds.ll[0] > 0
    assert np.linalg.norm(b[has] - xd[has]) <= 1e-9 * np.linalg.norm(xd)
    assert (~has).sum() >= 1                      # the generator's corner cells
    assert np.all(np.abs(b[~has]) < 1e-20)        # the residual, not x


def test_postprocess_known_answers(ora):
    """Hand-built rows: clamp to 0, a replacement chain through lower rows,
    equal neighbours, a self reference, an empty neighbour list."""
    n = 6
    ll = np.zeros((4, n), dtype=np.int32)
    ll[:, 0] = [2, 0, 0, 0]          # row 1 -> 2
    ll[:, 1] = [1, 3, 0, 0]          # row 2 -> 1, 3
    ll[:, 2] = [2, 0, 0, 0]          # row 3 -> 2
    ll[:, 3] = [4, 5, 0, 0]          # row 4: self, then 5
    ll[:, 4] = [4, 0, 0, 0]          # row 5 -> 4
    ll[:, 5] = [0, 6, 0, 0]          # row 6: list empty (first LL = 0)
    x = np.array([0.5, 0.5 + 4e-15, 0.5 + 8e-15, 7e-15, 2.0, 3.0])
    r = np.array([10.0, 20.0, 30.0, 40.0, 50.0, 60.0])
    xo, bo = ora.will_postprocess(x, r, ll, n)
    xp, bp = py_postprocess(x, r, ll, n)
    assert np.array_equal(xo, np.array(xp)) and np.array_equal(bo, np.array(bp))
    # row 1 compares with the unprocessed row 2 (4e-15 apart) and takes its value;
    # row 2 then equals the processed row 1, and takes the unprocessed row 3's value
    assert xo[0] == 0.5 + 4e-15 and bo[0] == xo[0]
    assert xo[1] == 0.5 + 8e-15 and bo[1] == xo[1]
    # row 3 equals its only neighbour (the processed row 2): its loop never writes
    # B, which keeps the residual
    assert xo[2] == 0.5 + 8e-15 and bo[2] == 30.0
    # row 4 is clamped to 0; its self reference is skipped; row 5 differs by 2
    assert xo[3] == 0.0 and bo[3] == 0.0 and bo[4] == 2.0
    # row 6 has an empty list: x kept, B keeps the residual
    assert xo[5] == 3.0 and bo[5] == 60.0
