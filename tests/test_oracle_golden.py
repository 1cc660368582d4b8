"""Pin the C oracle: bit-exact agreement with the golden vectors of
tests/golden (an independent pure-Python restatement of the reference on tiny
grids), hand-derived known answers, and an independent scipy direct solve."""
import pathlib

import numpy as np
import pytest

import __graft_entry__ as ge

GOLD = pathlib.Path(__file__).resolve().parent / "golden"
wl = ge.load_package().workload


def _golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLD / "make_golden.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize("name", ["tank_6x5x6", "beach_10x6x8", "bore_12x5x8", "flume2dv_16x1x8",
                                  "section2dv_1x14x8"])
def test_oracle_matches_golden(ora, name):
    g = np.load(GOLD / f"{name}.npz")
    case = _golden().golden_cases()[name]
    cls, sm, sy = ora.prepare(case)
    assert np.array_equal(cls.nf, g["nf"]) and np.array_equal(cls.nfb, g["nfb"])
    assert np.array_equal(cls.f, g["f"])
    assert np.array_equal(cls.fln[1:], g["fln"]) and np.array_equal(cls.sfn[1:], g["sfn"])
    assert cls.passes == int(g["passes"])
    assert sm.mp == float(g["mp"])
    assert np.array_equal(sm.alu_c, g["alu_c"]) and np.array_equal(sm.ll_c, g["ll_c"])
    assert np.array_equal(sm.de_c, g["de_c"])
    n = int(g["mnoe"])
    assert sy.mnoe == n
    assert np.array_equal(sy.mno2mn[1:n + 1], g["mno2mn"])
    assert np.array_equal(sy.b[1:n + 1], g["b"]) and sy.dmax == float(g["dmax"])
    assert np.array_equal(sy.alu[:, :n], g["alu"]) and np.array_equal(sy.llu[:, :n], g["llu"])
    assert np.array_equal(sy.de[1:n + 1], g["de"])
    r = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=float(g["eps0"]))
    assert np.array_equal(r.al[:, :n], g["al_sorted"]) and np.array_equal(r.ll[:, :n], g["ll_sorted"])
    assert np.array_equal(r.d, g["d_scaled"])
    assert r.iters == int(g["iters"]) and r.ier == int(g["ier"])
    assert r.eps == float(g["err"])
    assert np.array_equal(r.x, g["x"])


def test_golden_cases_cover_the_edge_cases():
    """The fixtures exercise surface rows, x-oriented surfaces and a restart pass."""
    g = np.load(GOLD / "bore_12x5x8.npz")
    orient = set(g["nfb"][g["nf"] == 2].tolist())
    assert -3 in orient and (orient & {-1, 1}), orient
    assert int(g["passes"]) >= 2
    assert (g["alu"] == -1e-20).any()


def test_golden_2dv_cases_use_four_columns(ora):
    """A grid one cell wide in y (or x) takes the reference's 2DV form: NL = 4
    columns over the x-z (y-z) plane, mp from those two axes only, the axis of
    surface rows shifted past the collapsed one (main_2CLOWNS.F90:43-44,
    1sub-matrix.F90:15-36, 1sub-momentum.F90:517-520); a grid one cell wide in
    both has no defined form and is refused."""
    for name, axes in (("flume2dv_16x1x8", (0, 2)), ("section2dv_1x14x8", (1, 2))):
        g = np.load(GOLD / f"{name}.npz")
        case = _golden().golden_cases()[name]
        assert ora.grid_nl(case.dims) == 4
        assert g["alu_c"].shape[0] == 4 and g["alu"].shape[0] == 4
        dx = case.dx[:, list(axes)]
        assert float(g["mp"]) == float(dx[dx > 0].min()) ** 2
        # surface rows carry extrapolation coefficients on their normal axis
        assert (g["alu"] != 0).any() and (g["alu"] == -1e-20).any()
    col = wl.make_case(1, 1, 8, dz=0.1, slope=None, n_obstacles=0, seed=3, amplitude=0.0)
    assert ora.grid_nl(col.dims) == 0


def test_known_answer_interior_fluid_row(ora):
    """Uniform grid dx=dy=0.05, dz=0.025: mp = dz^2 and an interior fluid row has
    off-diagonals -mp*2/(dx*2dx) = -0.25 (x, y), -1 (z) and diagonal 3
    (1sub-matrix.F90:49-61, cal_alu_f 82-87)."""
    case = wl.make_case(8, 8, 12, dz=0.025, depth=0.2, partial=False, seed=1, eps0=1e-12)
    cls, sm, sy = ora.prepare(case)
    assert sm.mp == 0.025 * 0.025
    # pick a fluid row whose six neighbours are all rows
    full = np.all(sy.llu[:, :sy.mnoe] > 0, axis=0)
    fluid = cls.nf[sy.mno2mn[1:sy.mnoe + 1]] == 1
    r = int(np.nonzero(full & fluid)[0][0])
    np.testing.assert_allclose(sy.alu[:, r], [-0.25, -0.25, -0.25, -0.25, -1.0, -1.0], rtol=1e-15)
    assert abs(sy.de[r + 1] - 3.0) < 1e-14


def test_known_answer_surface_row(ora):
    """Surface row with fluid below: de = 1, z- coefficient cal_alu(F, dz, dz) =
    -(F-1/2)/(F+1/2), the other row neighbours carry -1e-20
    (1sub-momentum.F90:486-543, 1sub-matrix.F90:75-80)."""
    case = wl.make_case(8, 8, 12, dz=0.025, depth=0.2, partial=False, seed=1, amplitude=0.0)
    cls, sm, sy = ora.prepare(case)
    rows = sy.mno2mn[1:sy.mnoe + 1]
    surf = np.nonzero(cls.nf[rows] == 2)[0]
    assert len(surf) > 0
    r = int(surf[len(surf) // 2])
    F = case.f[rows[r]]
    assert cls.nfb[rows[r]] == -3 and sy.de[r + 1] == 1.0
    expect = -(F - 0.5) * 0.025 / (F * 0.025 + 0.025 * 0.5)
    assert sy.alu[4, r] == expect
    assert sy.llu[5, r] == 0                        # air above: dropped
    side = sy.alu[:4, r][sy.llu[:4, r] != 0]
    assert np.all(side == -1e-20)


def test_known_answer_sort_ties(ora):
    """Exchange sort with ties (pcgpme_para.F90:96-112): an interior row
    (x-,x+,y-,y+,z-,z+) = (-.25,-.25,-.25,-.25,-1,-1) ends as z-, z+, y-, y+, x-, x+."""
    case = wl.make_case(8, 8, 12, dz=0.025, depth=0.2, partial=False, seed=1, eps0=1e-12)
    cls, sm, sy = ora.prepare(case)
    full = np.all(sy.llu[:, :sy.mnoe] > 0, axis=0)
    fluid = cls.nf[sy.mno2mn[1:sy.mnoe + 1]] == 1
    r = int(np.nonzero(full & fluid)[0][0])
    al, ll, d, b = ora.setup_scaled(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe)
    want = sy.llu[[4, 5, 2, 3, 0, 1], r]
    assert np.array_equal(ll[:, r], want)
    # W = 6/(max(3,3)+5*3) = 1/3
    assert d[r] == 3.0 * (6.0 / (3.0 + 3.0 * 5.0))


def test_oracle_solves_the_assembled_system(ora):
    """Independent cross-check: scipy sparse LU on the same assembled matrix."""
    import scipy.sparse.linalg as spl
    case = wl.beach_case(40, 32, 20, seed=5, n_obstacles=5)
    cls, sm, sy = ora.prepare(case)
    n = sy.mnoe
    A = ora.to_csr(sy)
    xd = spl.spsolve(A.tocsc(), sy.b[1:n + 1])
    r = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-13)
    assert r.ier == 0
    assert np.linalg.norm(r.x - xd) <= 1e-10 * np.linalg.norm(xd)


def test_openmp_and_serial_agree(ora):
    case = wl.beach_case(40, 32, 20, seed=6, n_obstacles=5)
    cls, sm, sy = ora.prepare(case)
    n = sy.mnoe
    r1 = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-13, nthreads=1)
    r4 = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], n, eps=1e-13, nthreads=4)
    assert np.linalg.norm(r1.x - r4.x) <= 1e-10 * np.linalg.norm(r1.x)


def test_iteration_cap_returns_3000(ora):
    """Loop exhaustion: IER = 3000 and ITER = cap + 1 (pcgpme_para.F90:148, 250-254)."""
    case = wl.beach_case(24, 20, 16, seed=2, n_obstacles=2)
    cls, sm, sy = ora.prepare(case)
    r = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe, eps=1e-14, itmax=4)
    assert r.ier == 3000 and r.iters == 5 and r.reason == 4


def test_transpose_identity(ora):
    """<A x, y> == <x, A^T y> for the explicit transposed stencil (adjoint support)."""
    case = wl.make_case(24, 16, 16, slope=0.3, n_obstacles=2, seed=3, step_layers=2)
    cls, sm, sy = ora.prepare(case)
    n = sy.mnoe
    alt, llt, det = ora.transpose(sy.alu, sy.llu, sy.de[1:], n)
    rng = np.random.default_rng(0)
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    ax = ora.spmv(sy.alu, sy.llu, sy.de[1:], n, x)
    aty = ora.spmv(alt, llt, det, n, y)
    assert abs(ax @ y - x @ aty) <= 1e-12 * abs(ax @ y)
    A = ora.to_csr(sy).toarray()
    np.testing.assert_allclose(aty, A.T @ y, rtol=1e-12, atol=1e-14)
