"""Case ingestion (src2LOWNS/data_io.F90:87-397, 1sub-main.F90:53-74): the
record layer, the cell numbering against a line-by-line restatement of the
reader's loops, set_dx, and whole cases written in the grid generator's
format (srcMakeGrid/data_io.F90) and read back, in both the dense and the
sparse form.  Everything here is integer or byte work, or copies of doubles:
compared bit for bit."""
import struct

import numpy as np
import pytest

import cases


@pytest.fixture(scope="module")
def ing(pkg):
    return pkg.ingest


CASE_FIELDS = ["dims", "mx2", "x", "dx", "mn", "inne", "inne2", "in_", "jn", "kn", "nf", "nfb",
               "f", "fb", "a", "un", "sp", "objno", "dt"]


def assert_same_case(a, b, fields=CASE_FIELDS):
    for name in fields:
        va, vb = getattr(a, name), getattr(b, name)
        assert np.array_equal(np.asarray(va), np.asarray(vb)), name


# ---------------------------------------------------------------------------
# records

def test_record_bytes_known_answer(ing, tmp_path):
    """One record of two integers and one of a real: big-endian 4-byte markers."""
    path = tmp_path / "r"
    with ing.RecordWriter(path) as w:
        w.record(np.array([1, 2], dtype=">i4"))
        w.record(np.array([0.5], dtype=">f8"))
    raw = path.read_bytes()
    assert raw == (struct.pack(">iiii", 8, 1, 2, 8) + struct.pack(">i", 8) + struct.pack(">d", 0.5)
                   + struct.pack(">i", 8))
    r = ing.RecordReader(path)
    assert r.read_array(">i4", 2).tolist() == [1, 2]
    assert float(r.read(">f8")) == 0.5 and r.at_end()


def test_subrecords_round_trip(ing, tmp_path):
    """Records longer than the subrecord limit are split, with negated leading
    lengths on all but the last piece and negated trailing lengths on all but
    the first; the reader joins them."""
    path = tmp_path / "s"
    payloads = [np.arange(n, dtype=">i4") for n in (0, 1, 4, 5, 12, 33)]
    with ing.RecordWriter(path, max_subrecord=16) as w:
        for pl in payloads:
            w.record(pl)
    raw = path.read_bytes()
    # the 5-integer record (20 bytes) is the fourth: pieces of 16 and 4 bytes
    off = sum(4 * p.size + 8 * max(1, -(-4 * p.size // 16)) for p in payloads[:3])
    assert struct.unpack(">i", raw[off:off + 4])[0] == -16
    assert struct.unpack(">i", raw[off + 20:off + 24])[0] == 16
    assert struct.unpack(">i", raw[off + 24:off + 28])[0] == 4
    assert struct.unpack(">i", raw[off + 32:off + 36])[0] == -4
    r = ing.RecordReader(path)
    for pl in payloads:
        assert np.array_equal(r.read_array(">i4", pl.size), pl)
    assert r.at_end()


def test_bad_records_raise(ing, tmp_path):
    path = tmp_path / "b"
    path.write_bytes(struct.pack(">i", 8) + b"\0" * 8 + struct.pack(">i", 12))
    with pytest.raises(ing.FormatError):
        ing.RecordReader(path).record()
    path.write_bytes(struct.pack(">i", 64) + b"\0" * 8)
    with pytest.raises(ing.FormatError):
        ing.RecordReader(path).record()
    path.write_bytes(struct.pack(">i", 8) + b"\0" * 8 + struct.pack(">i", 8))
    with pytest.raises(ing.FormatError):
        ing.RecordReader(path).read_array(">i4", 3)
    with pytest.raises(ing.FormatError):
        ing.RecordReader(path).read_many(">i4", 2)


# ---------------------------------------------------------------------------
# numbering

def loop_numbering(dims, nf3, nfb3):
    """data_io.F90:168-201 and 257-276 as the loops are written, on grids
    indexed [j-(js-1)][k-(ks-1)][i-(is-1)]; returns mn (dict over the
    numbered range), in/jn/kn, inne, inne2, nff."""
    is_, js, ks, ie, je, ke = (int(v) for v in dims)
    nf3 = nf3.copy()
    nfb3 = nfb3.copy()
    G = lambda a, i, k, j: a[j - js + 1, k - ks + 1, i - is_ + 1]        # noqa: E731

    def S(a, i, k, j, v):
        a[j - js + 1, k - ks + 1, i - is_ + 1] = v
    mn = {}
    cell = {}
    inn = 0
    for j in range(js - 1, je + 1):
        for k in range(ks - 1, ke + 1):
            for i in range(is_ - 1, ie + 1):
                f, b = G(nf3, i, k, j), G(nfb3, i, k, j)
                if f >= 0 or (f == -1 and 1 <= b < 200):
                    inn += 1
                    mn[(i, k, j)] = inn
                    cell[inn] = (i, j, k)
                else:
                    mn[(i, k, j)] = 0
    inne = inn
    for j in range(js - 1, je + 1):
        for k in range(ks - 1, ke + 1):
            for i in range(is_ - 1, ie + 1):
                if G(nf3, i, k, j) == -1 and G(nfb3, i, k, j) >= 200:
                    inn += 1
                    mn[(i, k, j)] = inn
                    S(nfb3, i, k, j, -1 if G(nfb3, i, k, j) == 300 else 0)
                    cell[inn] = (i, j, k)
    inne2 = inn
    nff = {}
    for j in range(js - 1, je + 1):
        for k in range(ks - 1, ke + 1):
            for i in range(is_ - 1, ie + 1):
                nn = mn[(i, k, j)]
                if nn == 0:
                    if G(nf3, i, k, j) == -1 and G(nfb3, i, k, j) == 0:
                        continue
                    if G(nf3, i, k, j) == -1 and G(nfb3, i, k, j) == -1:
                        mn[(i, k, j)] = inne2 + 1
                        continue
                nff[nn] = (int(G(nf3, i, k, j)), int(G(nfb3, i, k, j)))
    nff[0] = (-1, 0)
    nff[inne2 + 1] = (-1, -1)
    return mn, cell, inne, inne2, nff


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_numbering_matches_loop_restatement(ing, seed):
    rng = np.random.default_rng(seed)
    dims = np.array([3, 3, 3, 3 + 7, 3 + 5, 3 + 6], dtype=np.int32)
    shape = (5 + 2, 6 + 2, 7 + 2)
    nf3 = rng.choice([-1, 0, 1, 2], size=shape, p=[0.5, 0.2, 0.2, 0.1]).astype(np.int32)
    nfb3 = rng.choice([-2, -1, 0, 1, 4, 150, 199, 200, 250, 300], size=shape).astype(np.int32)
    nb = ing.number_cells(dims, nf3, nfb3)
    nf, nfb, mn = ing.cell_flags(dims, nf3, nb.nfb3, nb)
    mn_l, cell, inne, inne2, nff = loop_numbering(dims, nf3, nfb3)
    assert (nb.inne, nb.inne2) == (inne, inne2) and inne2 > inne > 0
    is_, js, ks = 3, 3, 3
    for (i, k, j), v in mn_l.items():
        assert mn[j - js + 2, k - ks + 2, i - is_ + 2] == v, (i, k, j)
    # outside the numbered range the map is 0
    inner = np.zeros(mn.shape, bool)
    inner[1:-2, 1:-2, 1:-2] = True
    assert not mn[~inner].any()
    for nn, (i, j, k) in cell.items():
        assert (nb.in_[nn], nb.jn[nn], nb.kn[nn]) == (i, j, k)
        assert (nf[nn], nfb[nn]) == nff[nn]
    assert (nf[0], nfb[0]) == (-1, 0) and (nf[inne2 + 1], nfb[inne2 + 1]) == (-1, -1)


# ---------------------------------------------------------------------------
# set_dx

def test_fortran_nint_and_round(ing):
    v = np.array([2.5, -2.5, 0.5, -0.5, 1.4999999999999998, 0.49999999999999994, 3.0, -7.2])
    assert ing.fortran_nint(v).tolist() == [3.0, -3.0, 1.0, -1.0, 1.0, 0.0, 3.0, -7.0]
    assert float(ing.round_dec(0.050000000000000044, 6)) == 0.05
    assert float(ing.round_dec(1.0 / 30.0, 6)) == 0.033333


def test_set_dx_known_answers(ing):
    """The number of decimals follows the first cell (1sub-main.F90:63-66);
    x(l, le+1) = 0 is extrapolated; dx(le+1) repeats dx(le)."""
    dims = np.array([3, 3, 3, 7, 6, 5], dtype=np.int32)
    mx2 = ing.mx2_of(dims)
    x = np.zeros((mx2, 3))
    for l, (s, e, d) in enumerate(((3, 7, 0.05), (3, 6, 1000.0), (3, 5, 1.0 / 30.0))):
        i = np.arange(s - 2, e + 2)
        x[i - 1, l] = (i - s) * d
    x[5 + 1 - 1, 2] = 0.0                                  # x(2, ke+1) missing
    x2, dx = ing.set_dx(dims, x)
    assert np.all(dx[0:7, 0] == 0.05) and dx[7, 0] == 0.05  # i = 1..7, le+1 = 8
    assert np.all(dx[0:7, 1] == 1000.0)
    assert x2[5, 2] == x[4, 2] + x[4, 2] - x[3, 2]
    assert np.all(dx[0:6, 2] == 0.033333)                   # 6 decimals for a 0.0333 cell
    assert dx[mx2 - 1, 0] == 0.0                            # beyond le+1 stays 0


# ---------------------------------------------------------------------------
# whole cases

@pytest.mark.parametrize("sparse", [True, False])
def test_generated_case_round_trip_and_pipeline(ing, ora, pkg, tmp_path, sparse):
    """A generated case with round spacings written and read back is the same
    case, and the oracle's pressure system from it is the same bit for bit."""
    c = pkg.workload.make_case(24, 20, 16, dz=0.025, slope=0.5, n_obstacles=2, seed=3, eps0=1e-12)
    ing.write_case(tmp_path / "tank", c, sparse=sparse)
    got = ing.read_case(tmp_path / "tank", eps0=c.eps0)
    assert got.sparse == sparse and got.t0 == 0.0 and got.dt0 is None
    r = got.case
    assert_same_case(c, r, [f for f in CASE_FIELDS if f != "sp"])
    assert np.array_equal(c.sp[:, 1:c.inne + 1], r.sp[:, 1:c.inne + 1])
    assert r.sp[0, 0] == ing.SDUM and r.sp[0, -1] == ing.SDUM
    _, _, sy0 = ora.prepare(c)
    _, _, sy1 = ora.prepare(r)
    for name in ("mno", "llu", "mno2mn"):
        assert np.array_equal(getattr(sy0, name), getattr(sy1, name)), name
    for name in ("alu", "de", "b"):
        assert np.array_equal(getattr(sy0, name).view(np.int64), getattr(sy1, name).view(np.int64)), name


@pytest.mark.parametrize("sparse", [True, False])
def test_flume_round_trip(ing, sparse):
    """The flume in the full index range (wave, side-wall and obstacle-surface
    cells, a lid) comes back identical, with pressure, normals, t0 and dt."""
    case, p, nor, got = cases.ingested_flume(sparse)
    assert_same_case(case, got.case)
    assert np.array_equal(p, got.p) and np.array_equal(nor, got.nor)
    assert got.t0 == 0.5 and got.dt0 == case.dt
    assert case.inne2 > case.inne
    assert (case.mn == case.inne2 + 1).any()
    assert (case.nfb == 4).sum() > 0 and (case.nfb == 2).sum() > 0
    tail = case.nfb[case.inne + 1:case.inne2 + 1]
    assert set(np.unique(tail).tolist()) == {-1, 0}


def test_flume_pipeline_uses_boundary_cells(ora):
    """The wave-boundary cells enter the matrix as neighbours (nf=-1, nfb=4,
    init_matrix's exception, 1sub-matrix.F90:41) and the system is solvable."""
    case, p, nor, got = cases.ingested_flume(True)
    cls, sm, sy = ora.prepare(got.case)
    wave = np.flatnonzero(got.case.nfb == 4)
    assert np.isin(sm.ll_c, wave).sum() > 0
    ref = ora.pcgpme(sy.alu, sy.llu, sy.de[1:], sy.b[1:], sy.mnoe, eps=1e-12)
    assert ref.ier == 0


def test_reader_rejects_bad_files(ing, pkg, tmp_path):
    c = pkg.workload.make_case(8, 6, 5, dz=0.1, seed=1)
    ing.write_case(tmp_path / "c", c, sparse=True)
    # grid bounds with is = 2 (x(l, is-2) would fall outside x(0:2, 1:mx2))
    xyz = tmp_path / "c.xyzn"
    raw = bytearray(xyz.read_bytes())
    raw[4:8] = struct.pack(">i", 2)
    bad = tmp_path / "bad.xyzn"
    bad.write_bytes(bytes(raw))
    with pytest.raises(ing.FormatError):
        ing.read_xyz(bad)
    # a cell number beyond inne2 in the sparse data records
    data = bytearray((tmp_path / "c").read_bytes())
    off = 4 + 24 + 4 + 4 + 8 + 4                       # t0,g,nu record, icc,icc2 record
    data[off + 4:off + 8] = struct.pack(">i", c.inne2 + 5)
    (tmp_path / "d").write_bytes(bytes(data))
    (tmp_path / "d.xyzn").write_bytes(xyz.read_bytes())
    with pytest.raises(ing.FormatError):
        ing.read_case(tmp_path / "d")
    # a truncated data file
    (tmp_path / "e").write_bytes(bytes(data[:off + 20]))
    (tmp_path / "e.xyzn").write_bytes(xyz.read_bytes())
    with pytest.raises(ing.FormatError):
        ing.read_case(tmp_path / "e")


def test_reader_rounds_spacings_like_the_reference(ing, ora, pkg, tmp_path):
    """A spacing of 0.8/24 is rounded to 0.033333 by set_dx (6 decimals for a
    0.0333 first cell): the case read from files equals the generated one
    after the same rounding, down to the assembled system."""
    c = pkg.workload.make_case(20, 16, 24, dz=0.8 / 24, slope=0.5, n_obstacles=2, seed=6)
    ing.write_case(tmp_path / "c", c, sparse=True)
    r = ing.read_case(tmp_path / "c", eps0=c.eps0).case
    x2, dx2 = ing.set_dx(c.dims, c.x)
    assert np.array_equal(r.dx, dx2) and not np.array_equal(r.dx, c.dx)
    assert r.dx[3, 2] == 0.033333
    gen = c.copy()
    gen.x, gen.dx = x2, dx2
    _, _, s0 = ora.prepare(gen)
    _, _, s1 = ora.prepare(r)
    assert np.array_equal(s0.alu.view(np.int64), s1.alu.view(np.int64))
    assert np.array_equal(s0.b.view(np.int64), s1.b.view(np.int64))


def test_missing_fdata_and_nsdata_defaults(ing, pkg, tmp_path):
    """Without .fdata every face of cells 1..inne is open with porosity 1 (faces
    of the obstacle-surface cells closed); without .nsdata every surface
    position is the -1e4 marker; dt falls back to the trailing record when
    t0 > 0, else to the argument."""
    import os
    c = pkg.workload.make_case(10, 8, 6, dz=0.1, seed=2)
    ing.write_case(tmp_path / "c", c, sparse=True, t=1.5, dt=2e-3)
    os.remove(tmp_path / "c.fdata")
    os.remove(tmp_path / "c.nsdata")
    got = ing.read_case(tmp_path / "c")
    r = got.case
    assert np.all(r.a[1:r.inne + 1] == 1.0) and np.all(r.fb[1:r.inne + 1] == 1.0)
    assert np.all(r.a[r.inne + 1:] == 0.0)
    assert np.all(r.sp[0] == ing.SDUM)
    assert got.dt0 == 2e-3 and r.dt == 2e-3 and got.t0 == 1.5
    assert ing.read_case(tmp_path / "c", dt=5e-4).case.dt == 5e-4
