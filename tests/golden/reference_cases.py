"""Inputs on which the reference's own routines were run (tests/golden/make_ref_golden.py)
and the oracle is checked against their outputs (tests/test_oracle_reference_runs.py).

Every case is rebuilt from the seeded generator and its real-valued fields are
rounded to a fixed binary grid (the same inputs on x86-64 and aarch64), so the
committed fixture holds only the reference's outputs (hashes of their bytes and
scalars).  A digest of the inputs is stored beside them: a changed generator
shows as an input mismatch, not as a false parity failure.
"""
from __future__ import annotations

import hashlib
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
for _p in (HERE.parent.parent, HERE.parent, HERE):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import __graft_entry__ as ge  # noqa: E402

wl = ge.load_package().workload


QUANTUM = 2.0 ** -24


def portable(case):
    """The case with its real-valued fields rounded to multiples of 2**-24.
    The seeded generator's transcendental functions (numpy's cosh, its normal
    sampler) differ in the last bits between x86-64 and aarch64; after the
    rounding both give the same inputs, so outputs recorded on one machine
    check the code on the other."""
    c = case.copy()
    for name in ("f", "fb", "a", "un", "sp", "x", "dx"):
        v = getattr(c, name)
        setattr(c, name, np.round(v / QUANTUM) * QUANTUM)
    return c


def portable_will(ds):
    for name in ("al", "d", "b"):
        v = getattr(ds, name)
        setattr(ds, name, np.round(v / QUANTUM) * QUANTUM)
    return ds


def speckled(case, seed: int, droplets: int, bubbles: int):
    """The case with seeded droplets above its free surface (air cells given a
    volume fraction) and bubbles below it (fluid cells emptied), so that the
    surface classification prunes isolated surface cells and loops."""
    c = case.copy()
    rng = np.random.default_rng(seed)
    inne = c.inne
    f = c.f
    air = np.flatnonzero((c.nf[1:inne + 1] == 0) & (c.fb[1:inne + 1] > 0.0)) + 1
    wet = np.flatnonzero((c.nf[1:inne + 1] == 1) & (f[1:inne + 1] >= 1.0)) + 1
    if len(air):
        pick = rng.choice(air, size=min(droplets, len(air)), replace=False)
        f[pick] = rng.uniform(0.05, 1.0, size=len(pick))
        c.nf[pick] = 1
    if len(wet):
        pick = rng.choice(wet, size=min(bubbles, len(wet)), replace=False)
        f[pick] = 0.0
        c.nf[pick] = 0
    c.label = (c.label or "") + "+speckled"
    return c


def grid_cases():
    """label -> (case, run the solve, run the ik loop).  The solve flag is True
    (recorded with its solution vector, for the oracle and the GPU), "cpu"
    (recorded for the oracle only: the larger systems, 10-27 thousand rows) or
    False; ik loops run on the smallest systems.  Classification, coefficients,
    numbering, right-hand side and assembly run on all."""
    from make_golden import golden_cases
    from cases import small_cases

    out = {}
    for label, c in golden_cases().items():
        out[label] = (c, True, True)
    small = dict(small_cases())
    for label in ("tank_24x20x16", "flume2dv_96x1x32", "section2dv_1x80x24"):
        out[label] = (small[label], True, False)
    for label in ("beach_48x40x24", "bore_40x24x32", "shore_64x16x24"):
        out[label] = (small[label], "cpu", False)
    # (the flume's ik loop diverges -- dmax grows pass after pass -- so it runs no loop)
    out["flume_40x24x20_ingested"] = (small["flume_40x24x20_ingested"], False, False)
    base = wl.make_case(20, 12, 16, dz=0.05, slope=0.25, n_obstacles=2, seed=41, amplitude=0.08,
                        step_layers=2)
    out["speckled_20x12x16"] = (speckled(base, seed=42, droplets=40, bubbles=25), True, True)
    base2 = wl.make_case(24, 1, 16, dz=0.05, slope=0.25, n_obstacles=0, seed=43, amplitude=0.08)
    out["speckled2dv_24x1x16"] = (speckled(base2, seed=44, droplets=12, bubbles=8), True, True)
    return {k: (portable(c), s, lp) for k, (c, s, lp) in out.items()}


def will_cases():
    """label -> (2DH system, tolerance): PCGPME_WILL inputs."""
    return {
        "dispersion_14x10": (portable_will(wl.dispersion_system(14, 10, seed=5)), 1e-12),
        "dispersion_24x18": (portable_will(wl.dispersion_system(24, 18, seed=7)), 1e-10),
        "dispersion_30x8": (portable_will(wl.dispersion_system(30, 8, seed=3)), 1e-12),
        "dispersion_40x32": (portable_will(wl.dispersion_system(40, 32, seed=11)), 1e-12),
    }


def numbering_cases():
    """label -> (dims, nf3, nfb3): flag grids over is-1:ie x js-1:je x ks-1:ke
    ([j][k][i]) for read_data's numbering -- those of every grid case (the
    ingested flume carries wave-boundary, side-wall, obstacle-surface and lid
    codes) and seeded random grids that take every branch."""
    ing = ge.load_package().ingest
    out = {}
    for label, (c, _, _) in grid_cases().items():
        nf3, nfb3 = ing.flag_grids(c)
        out[label] = (np.asarray(c.dims), nf3, nfb3)
    rng = np.random.default_rng(77)
    for k, (nx, ny, nz) in enumerate([(10, 8, 6), (7, 1, 9), (1, 9, 7)]):
        dims = np.array([3, 3, 3, 3 + nx, 3 + ny, 3 + nz], dtype=np.int32)
        shape = (ny + 2, nz + 2, nx + 2)
        nf3 = rng.choice(np.array([-1, 0, 1, 2], dtype=np.int32), size=shape, p=[0.35, 0.2, 0.35, 0.1])
        nfb3 = rng.choice(np.array([0, 1, 2, 4, 5, 199, 200, 300, -1], dtype=np.int32), size=shape)
        out[f"random{k}_{nx}x{ny}x{nz}"] = (dims, nf3.astype(np.int32), nfb3.astype(np.int32))
    return out


def reader_cases():
    """label -> (case, sparse, t0, p, nor): cases written by ingest.write_case and
    read back by the reference's readers -- both file forms (.xyzn sparse,
    .xyz dense), t0 = 0 (no trailing dt) and t0 > 0, 2DV, boundary cells over
    the full index range, seeded pressures and surface normals."""
    grids = grid_cases()
    rng = np.random.default_rng(91)
    q = lambda v: np.round(v / QUANTUM) * QUANTUM  # noqa: E731
    out = {}
    for label, sparse, t0 in (("beach_10x6x8", True, 0.0), ("beach_10x6x8", False, 0.0),
                              ("beach_10x6x8", False, 1.5), ("flume2dv_16x1x8", True, 0.5),
                              ("section2dv_1x14x8", False, 0.0), ("speckled_20x12x16", True, 2.0),
                              ("flume_40x24x20_ingested", True, 3.0), ("flume_40x24x20_ingested", False, 0.0)):
        c = grids[label][0]
        n = c.inne2 + 2
        p = q(rng.normal(0.0, 50.0, size=n))
        nor = q(rng.uniform(-1.0, 1.0, size=(n, 4)))
        out[f"{label}_{'xyzn' if sparse else 'xyz'}_t{t0:g}"] = (c, sparse, t0, p, nor)
    return out


def spacing_cases():
    """label -> (dims, x (mx2, 3), x(l, i) at [i-1, l]): coordinates for set_dx --
    those of the grid cases, and variants with the last coordinate of an axis
    missing (0, extrapolated) and spacings from 5e-5 to 50 (the decimal guess)."""
    out = {}
    grids = grid_cases()
    for label in ("tank_6x5x6", "beach_10x6x8", "flume2dv_16x1x8", "section2dv_1x14x8", "bore_40x24x32",
                  "flume_40x24x20_ingested"):
        c = grids[label][0]
        out[label] = (np.asarray(c.dims), np.array(c.x))
    c = grids["beach_10x6x8"][0]
    le = [int(v) for v in c.dims[3:]]
    for scale in (1e3, 2.5e-2, 1e-3):
        out[f"beach_10x6x8_x{scale:g}"] = (np.asarray(c.dims), np.round(np.array(c.x) * scale / QUANTUM) * QUANTUM)
    x = np.array(c.x)
    x[le[0], 0] = 0.0                            # x(0, le(0)+1) missing
    x[le[2], 2] = 0.0
    out["beach_10x6x8_open_end"] = (np.asarray(c.dims), x)
    return out


LOOP_D0, LOOP_EPS0 = 1e-9, 1e-7          # two or more ik passes on the small grids


def digest(a) -> str:
    """sha256 of an array's dtype, shape and bytes (little-endian)."""
    a = np.asarray(a)
    if a.dtype.kind == "O":                      # values of a translated array slice
        a = np.array(a.tolist())
        if a.dtype.kind == "O":
            raise ValueError("undefined values in a recorded output")
    if a.dtype.kind == "f":
        a = a.astype("<f8")
    elif a.dtype.kind in "iu":
        a = a.astype("<i8")
    elif a.dtype.kind == "b":
        a = a.astype("u1")
    h = hashlib.sha256()
    h.update(str(a.dtype).encode() + str(a.shape).encode())
    h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def runs(idx) -> str:
    """Sorted 1-based indices as inclusive runs, "first-last,first-last,..."."""
    out = []
    for i in (int(v) for v in idx):
        if out and out[-1][1] == i - 1:
            out[-1][1] = i
        else:
            out.append([i, i])
    return ",".join(f"{a}-{b}" for a, b in out)


def runs_mask(r: str, n: int) -> np.ndarray:
    """Boolean mask over 1..n (index 0 = element 1) of the elements the runs list."""
    m = np.zeros(n, dtype=bool)
    for part in filter(None, r.split(",")):
        a, b = (int(v) for v in part.split("-"))
        m[a - 1:b] = True
    return m


def case_digest(c) -> str:
    parts = [c.dims, c.mn, c.in_, c.jn, c.kn, c.nf, c.nfb, c.f, c.fb, c.a, c.un, c.sp, c.x, c.dx, c.objno,
             np.array([c.dt, c.eps0])]
    return digest(np.concatenate([np.asarray(p, dtype=np.float64).ravel() for p in parts]))


def will_digest(ds) -> str:
    return digest(np.concatenate([np.asarray(p, dtype=np.float64).ravel() for p in (ds.al, ds.ll, ds.d, ds.b)]))
