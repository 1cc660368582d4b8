"""Seeded small cases shared by the tests (sizes the oracle finishes in seconds)."""
import numpy as np

import __graft_entry__ as ge

wl = ge.load_package().workload


def small_cases():
    """(label, Case) pairs covering flat tank, beach + obstacles + partial cells,
    a bore front (x-oriented surface cells, corner cells), a shoreline, a
    flume read from the reference's file format with boundary cells in the
    full index range (wave boundaries, obstacle-surface cells, sentinels), and
    the 2DV mode in both orientations."""
    return [
        ("tank_24x20x16", wl.make_case(24, 20, 16, dz=0.025, partial=False, seed=0, eps0=1e-12)),
        ("beach_48x40x24", wl.beach_case(48, 40, 24, seed=5, n_obstacles=6)),
        ("bore_40x24x32", wl.make_case(40, 24, 32, dz=0.8 / 32, slope=0.5, n_obstacles=4, seed=7,
                                        amplitude=0.08, step_layers=2)),
        ("bore3_40x24x32", wl.make_case(40, 24, 32, dz=0.8 / 32, slope=None, n_obstacles=4, seed=8,
                                         amplitude=0.08, step_layers=3)),
        ("shore_64x16x24", wl.make_case(64, 16, 24, slope=1.0 / 3.0, n_obstacles=3, seed=11,
                                         amplitude=0.05)),
        ("flume_40x24x20_ingested", ingested_flume(True)[3].case),
        # 2DV (NL = 4, main_2CLOWNS.F90:43-44): a wave flume one cell wide in y with a
        # beach and a lowered surface step, and a y-z section one cell wide in x
        ("flume2dv_96x1x32", wl.make_case(96, 1, 32, dz=0.8 / 32, slope=0.25, n_obstacles=0, seed=31,
                                           amplitude=0.08, step_layers=2)),
        ("section2dv_1x80x24", wl.make_case(1, 80, 24, dz=0.8 / 24, slope=None, n_obstacles=0, seed=32,
                                             amplitude=0.05)),
    ]


def flume_grids(nx=40, ny=24, nz=20, seed=13):
    """A wave flume in the reference's full index range, built as flag grids
    over is-1:ie x js-1:je x ks-1:ke and numbered the way the solver's reader
    numbers them: wave-boundary cells (nf=-1, nfb=4) on both x ends, side-wall
    boundary cells (nf=-1, nfb=2) on j=js-1, obstacle-surface cells (nfb 200
    and 300, numbered after inne) and a lid (nf=nfb=-1, mapped to inne2+1).
    Returns the Case, its pressure and normals."""
    ing = ge.load_package().ingest
    base = wl.make_case(nx, ny, nz, dz=0.8 / nz, slope=0.25, slope_start=0.5, n_obstacles=3,
                        seed=seed, amplitude=0.05)
    dims = base.dims
    num0 = base.mn[1:-2, 1:-2, 1:-2]                 # base numbering over the grid, interior only
    shape = num0.shape
    interior = num0 > 0
    nf3 = np.full(shape, -1, dtype=np.int32)
    nfb3 = np.zeros(shape, dtype=np.int32)
    nf3[interior] = base.nf[num0[interior]]
    nfb3[interior] = base.nfb[num0[interior]]
    left = np.zeros(shape, bool)
    right = np.zeros(shape, bool)
    left[1:-1, 1:-1, 0] = interior[1:-1, 1:-1, 1]
    right[1:-1, 1:-1, -1] = interior[1:-1, 1:-1, -2]
    nfb3[left | right] = 4
    side = np.zeros(shape, bool)
    side[0, 1:-1, 1:-1] = interior[1, 1:-1, 1:-1]
    nfb3[side] = 2
    solid_in = np.zeros(shape, bool)
    solid_in[1:-1, 1:-1, 1:-1] = ~interior[1:-1, 1:-1, 1:-1]
    wet_minus = np.zeros(shape, bool)
    wet_minus[:, :, 1:] |= nf3[:, :, :-1] >= 0
    wet_minus[1:, :, :] |= nf3[:-1, :, :] >= 0
    wet_minus[:, 1:, :] |= nf3[:, :-1, :] >= 0
    jj, kk, ii = np.indices(shape)
    obs = solid_in & wet_minus
    nfb3[obs] = np.where((ii + jj + kk) % 3 == 0, 300, 200)[obs]
    nfb3[:, -1, :] = -1                              # k = ke: the lid
    nb = ing.number_cells(dims, nf3, nfb3)
    nf, nfb, mn = ing.cell_flags(dims, nf3, nb.nfb3, nb)
    inne, inne2 = nb.inne, nb.inne2
    ncell = inne2 + 2
    num = nb.mn[1:-2, 1:-2, 1:-2]
    f = np.zeros(ncell)
    fb = np.zeros(ncell)
    a = np.zeros((ncell, 3))
    un = np.zeros((ncell, 3))
    sp = np.zeros((3, ncell))
    sp[0, :] = ing.SDUM
    old = num0[interior]                              # interior cells keep the base's state
    new = num[interior]
    f[new], fb[new], a[new], un[new], sp[:, new] = base.f[old], base.fb[old], base.a[old], base.un[old], base.sp[:, old]
    for mask, step in ((left, 1), (right, -1)):       # wave cells copy their interior neighbour
        cells = num[mask]
        nbr = num0[np.roll(mask, step, axis=2)]
        f[cells] = base.f[nbr]
        fb[cells] = 1.0
        a[cells] = (1.0, 0.0, 0.0)
        un[cells, 0] = base.un[nbr, 0]
    nxt = num[np.roll(left, 1, axis=2)]               # interior cells at i = is open towards the boundary
    a[nxt, 0] = 1.0
    fb[num[side]] = 1.0
    rng = np.random.default_rng(seed)
    idx = np.arange(1, inne + 1)
    at_rest = (nf[idx] == 0) & ~np.any(un[idx] != 0.0, axis=1) & (f[idx] < 1e-13)
    p = np.zeros(ncell)                               # pressure where the sparse form keeps it
    p[idx[~at_rest]] = rng.normal(0.0, 1.0, int((~at_rest).sum()))
    nor = np.zeros((ncell, 4))                        # normals where a surface position is set
    has_sp = idx[sp[0, idx] != ing.SDUM]
    nor[has_sp] = rng.normal(0.0, 1.0, (has_sp.size, 4))
    case = wl.Case(nx=nx, ny=ny, nz=nz, dims=dims.copy(), mx2=base.mx2, x=base.x.copy(), dx=base.dx.copy(),
                   mn=mn, inne=inne, inne2=inne2, in_=nb.in_, jn=nb.jn, kn=nb.kn, nf=nf, nfb=nfb, f=f, fb=fb,
                   a=a, un=un, sp=sp, objno=np.zeros(ncell, dtype=np.int32), dt=base.dt, eps0=base.eps0,
                   seed=seed, label=f"flume_{nx}x{ny}x{nz}")
    return case, p, nor


def ingested_flume(sparse=True):
    """flume_grids written in the reference's file format and read back."""
    import tempfile
    ing = ge.load_package().ingest
    case, p, nor = flume_grids()
    with tempfile.TemporaryDirectory() as d:
        ing.write_case(d + "/flume", case, p=p, nor=nor, t=0.5, dt=case.dt, sparse=sparse)
        got = ing.read_case(d + "/flume", eps0=case.eps0)
    return case, p, nor, got
