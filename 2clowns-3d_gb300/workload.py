"""Seeded synthetic 2CLOWNS-3D pressure-solve inputs, in the reference's array layouts.

The reference ships no input geometry (its ``../init/*.xyzn``, ``.fdata`` and
``.nsdata`` cases are not distributed), so every workload here is generated from
a seed.  The generator produces the state of the Fortran module arrays at the
moment the model reaches the pressure-correction loop -- grid coordinates,
the dense cell map, per-cell flags before classification, face area fractions,
porosity, VOF fraction, provisional face velocities and surface positions --
laid out exactly as the reference stores them, so the same buffers can be handed
to the C-ABI that a Fortran caller would use.

Index conventions (all follow the reference):

* ``is=js=ks=3`` and computational cells are ``i=is..ie-1`` (same for j, k), as
  written by the grid generator (srcMakeGrid/set_grid.F90:74).
* ``mn(is-2:ie+2, ks-2:ke+2, js-2:je+2)`` is a dense int32 map, i fastest
  (0mod-arrays.F90:213); 0 means "not a numbered cell".
* Numbered cells are counted with j outermost, then k, then i
  (data_io.F90:168-202).  Solid cells (bed, obstacles) and the ghost layers are
  not numbered and resolve to the sentinel cell 0, whose flag is -1
  (data_io.F90:271-272).
* Per-cell arrays run over ``0..inne2+1``; ``a(0:2,nn)``, ``un(0:2,nn)`` have the
  component fastest; ``sp(0:inne2+1,0:2)`` has the cell index fastest
  (0mod-arrays.F90:223, 237, 290).
* ``x(0:2,1:mx2)`` and ``dx(0:2,1:mx2)`` with ``mx2=max(ie,je,ke)+2``
  (0mod-arrays.F90:205-206); entries outside ``ls-2..le+1`` are zero as in the
  reference, which only fills that range (1sub-main.F90:53-74).

Geometry recipe (one function, parameterised per workload):

* still-water depth ``h`` in a 0.8 m-tall domain; flat bed, or a sloping beach
  ``z_b = max(0, (x - x_s) * slope)`` starting at ``x_s = 0.4 L``;
* cells wholly below the bed are solid; partial cells get porosity ``fb`` = wet
  volume fraction (solid when below 0.01, the grid generator's threshold at
  srcMakeGrid/cal_fluid_area.F90:221-229) and side face fractions ``U(0.05,1)``;
* seeded full-height rectangular obstacles (porosity 0, closed faces);
* walls: ``a=0`` on every face whose minus-side neighbour is solid or outside;
* VOF ``F=1`` below the single surface layer, ``F=(eta-z_k)/dz`` clamped to
  [0.02, 0.98] in it (excursion capped at 0.9 dz), 0 above, with ``eta`` the
  solitary-wave profile ``A sech^2(k(x-x0))``, ``k=sqrt(3A/4h^3)``
  (lib/src/input_wave.f90:10-11, 45-48);
* provisional face velocity ``u = eta sqrt(g/h)`` (input_wave.f90:50), ``w``
  linear in z, plus N(0, 1e-3) noise on every wet face.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

G_ACC = 9.80665
DT = 1.0e-3


@dataclasses.dataclass
class Case:
    """Module-array state of one 3D pressure solve (reference layouts)."""

    nx: int
    ny: int
    nz: int
    dims: np.ndarray          # int32[6] = is, js, ks, ie, je, ke
    mx2: int
    x: np.ndarray             # f64 (mx2, 3): x(l, i) at [(i-1), l]
    dx: np.ndarray            # f64 (mx2, 3)
    mn: np.ndarray            # int32 (NJ, NK, NI), i fastest
    inne: int
    inne2: int
    in_: np.ndarray           # int32 (inne2+2,)
    jn: np.ndarray
    kn: np.ndarray
    nf: np.ndarray            # int32 (inne2+2,)  nff(:)%f
    nfb: np.ndarray           # int32 (inne2+2,)  nff(:)%b
    f: np.ndarray             # f64 (inne2+2,)
    fb: np.ndarray            # f64 (inne2+2,)
    a: np.ndarray             # f64 (inne2+2, 3)
    un: np.ndarray            # f64 (inne2+2, 3)
    sp: np.ndarray            # f64 (3, inne2+2)  sp(nn, l) at [l, nn]
    objno: np.ndarray         # int32 (inne2+2,)
    dt: float = DT
    eps0: float = 1.0e-10
    seed: int = 0
    label: str = ""

    @property
    def ncells(self) -> int:
        return self.nx * self.ny * self.nz

    def copy(self) -> "Case":
        kw = {}
        for fld in dataclasses.fields(self):
            v = getattr(self, fld.name)
            kw[fld.name] = v.copy() if isinstance(v, np.ndarray) else v
        return Case(**kw)

    def mn_index(self, i, k, j):
        """Flat offset of mn(i,k,j) in the dense map."""
        is_, js, ks, ie, je, ke = (int(v) for v in self.dims)
        ni = ie - is_ + 5
        nk = ke - ks + 5
        return (np.asarray(i) - (is_ - 2)) + ni * ((np.asarray(k) - (ks - 2)) + nk * (np.asarray(j) - (js - 2)))


def _sech2(z):
    return 1.0 / np.cosh(np.clip(z, -350.0, 350.0)) ** 2


def make_case(nx: int, ny: int, nz: int, *, dx: float = 0.05, dy: float = 0.05,
              dz: Optional[float] = None, height: float = 0.8, depth: float = 0.5,
              slope: Optional[float] = None, slope_start: float = 0.4,
              n_obstacles: int = 0, obstacle_frac: float = 0.10,
              amplitude: float = 0.05, noise: float = 1.0e-3, partial: bool = True,
              step_layers: int = 0, step_at: float = 0.6,
              seed: int = 0, eps0: float = 1.0e-10, dt: float = DT,
              label: str = "") -> Case:
    """Build one seeded case.  ``dz`` defaults to ``height/nz``.

    ``step_layers`` lowers the free surface by that many layers for
    ``x > step_at * L`` (a bore front), which produces surface cells oriented
    along x and corner cells with two candidate orientations."""
    rng = np.random.default_rng(seed)
    if dz is None:
        dz = height / nz
    is_ = js = ks = 3
    ie, je, ke = is_ + nx, js + ny, ks + nz
    dims = np.array([is_, js, ks, ie, je, ke], dtype=np.int32)
    mx2 = max(ie, je, ke) + 2

    # ---- coordinates: x(l,i) = (i - ls) * d for i in [ls-2, le+1], zero elsewhere
    x = np.zeros((mx2, 3), dtype=np.float64)
    dxa = np.zeros((mx2, 3), dtype=np.float64)
    for l, (ls, le, d) in enumerate(((is_, ie, dx), (js, je, dy), (ks, ke, dz))):
        idx = np.arange(ls - 2, le + 2)           # 1-based indices ls-2..le+1
        x[idx - 1, l] = (idx - ls) * d
        dxa[idx - 1, l] = d

    lx = nx * dx
    ly = ny * dy
    ii = np.arange(nx)
    jj = np.arange(ny)
    kk = np.arange(nz)
    xc = (ii + 0.5) * dx
    yc = (jj + 0.5) * dy
    zk = kk * dz
    zt = (kk + 1) * dz

    # ---- bed and porosity
    if slope is not None and slope > 0:
        zb = np.maximum(0.0, (xc - slope_start * lx) * slope)
    else:
        zb = np.zeros(nx)
    zb3 = zb[None, None, :]                      # (1,1,nx) -> broadcast to (ny,nz,nx)
    zk3 = zk[None, :, None]
    zt3 = zt[None, :, None]
    below = zt3 <= zb3 + 1e-12
    part = (zk3 < zb3 - 1e-12) & ~below
    fb_grid = np.ones((ny, nz, nx), dtype=np.float64)
    fbp = np.broadcast_to((zt3 - zb3) / dz, (ny, nz, nx))
    fb_grid = np.where(part, fbp, fb_grid)
    solid = np.broadcast_to(below, (ny, nz, nx)).copy()
    solid |= part & (fb_grid < 0.01)
    part = part & ~solid
    if not partial:
        # partial cells become full fluid cells (flat-bed configs never have any)
        fb_grid = np.where(part, 1.0, fb_grid)
        part = np.zeros_like(part)

    # ---- obstacles: full-height rectangles, total ~obstacle_frac of plan area
    obst = np.zeros((ny, nx), dtype=bool)
    if n_obstacles > 0:
        area_each = obstacle_frac * nx * ny / n_obstacles
        for _ in range(n_obstacles):
            aspect = rng.uniform(0.5, 2.0)
            w = max(1, int(round(math.sqrt(area_each * aspect))))
            hgt = max(1, int(round(area_each / w)))
            w = min(w, nx - 2)
            hgt = min(hgt, ny - 2)
            i0 = int(rng.integers(1, max(2, nx - w)))
            j0 = int(rng.integers(1, max(2, ny - hgt)))
            obst[j0:j0 + hgt, i0:i0 + w] = True
    solid |= obst[:, None, :]
    fb_grid = np.where(solid, 0.0, fb_grid)

    # ---- numbering: j outer, k, i inner (ghosts and solids are not numbered)
    numbered = ~solid
    order = np.cumsum(numbered.ravel()).reshape(numbered.shape).astype(np.int64)
    cellno = np.where(numbered, order, 0).astype(np.int32)     # (ny,nz,nx)
    inne = int(numbered.sum())
    inne2 = inne
    ni, nk, nj = ie - is_ + 5, ke - ks + 5, je - js + 5
    mn = np.zeros((nj, nk, ni), dtype=np.int32)
    # interior i = is+ii -> offset ii+2 (since mn starts at is-2)
    mn[2:2 + ny, 2:2 + nz, 2:2 + nx] = cellno

    ncell = inne2 + 2
    sel = numbered
    jjg, kkg, iig = np.nonzero(sel)                # C-order == numbering order
    in_ = np.zeros(ncell, dtype=np.int32)
    jn = np.zeros(ncell, dtype=np.int32)
    kn = np.zeros(ncell, dtype=np.int32)
    in_[1:inne + 1] = iig + is_
    jn[1:inne + 1] = jjg + js
    kn[1:inne + 1] = kkg + ks

    fb = np.zeros(ncell)
    fb[1:inne + 1] = fb_grid[sel]

    # ---- VOF
    ksl = int(math.floor(depth / dz + 1e-9))
    x0 = 0.25 * lx
    kw = math.sqrt(3.0 * amplitude / (4.0 * depth ** 3)) if amplitude > 0 else 0.0
    eta_c = amplitude * _sech2(kw * (xc - x0))                    # at cell centres
    fsurf = np.clip(np.minimum(eta_c, 0.9 * dz) / dz, 0.02, 0.98)  # (nx,)
    kcol = np.full(nx, ksl, dtype=np.int64)
    if step_layers:
        kcol = np.where(xc > step_at * lx, max(0, ksl - step_layers), kcol)
    kk3 = kk[None, :, None]
    kc3 = kcol[None, None, :]
    f_grid = np.where(kk3 < kc3, 1.0, np.where(kk3 == kc3, fsurf[None, None, :], 0.0))
    f_grid = np.broadcast_to(f_grid, (ny, nz, nx)).copy()
    f_grid = np.where(solid, 0.0, f_grid)
    f = np.zeros(ncell)
    f[1:inne + 1] = f_grid[sel]

    # ---- flags before classification: fluid if wet, air otherwise; sentinels solid
    nf = np.zeros(ncell, dtype=np.int32)
    nf[1:inne + 1] = np.where(f[1:inne + 1] > 0.0, 1, 0)
    nfb = np.zeros(ncell, dtype=np.int32)
    nf[0] = -1
    nfb[0] = 0
    nf[inne2 + 1] = -1
    nfb[inne2 + 1] = -1

    # ---- face fractions (minus face of each cell)
    a_grid = np.ones((ny, nz, nx, 3))
    if partial:
        npart = int(part.sum())
        if npart:
            a_grid[part, 0] = rng.uniform(0.05, 1.0, npart)
            a_grid[part, 1] = rng.uniform(0.05, 1.0, npart)
    # wall rule: minus neighbour solid or outside the interior -> closed face
    solid_pad = np.pad(solid, ((1, 0), (1, 0), (1, 0)), constant_values=True)
    minus_solid_x = solid_pad[1:, 1:, :-1]
    minus_solid_y = solid_pad[:-1, 1:, 1:]
    minus_solid_z = solid_pad[1:, :-1, 1:]
    a_grid[..., 0] = np.where(minus_solid_x, 0.0, a_grid[..., 0])
    a_grid[..., 1] = np.where(minus_solid_y, 0.0, a_grid[..., 1])
    a_grid[..., 2] = np.where(minus_solid_z, 0.0, a_grid[..., 2])
    a = np.zeros((ncell, 3))
    a[1:inne + 1] = a_grid[sel]

    # ---- surface position
    sp = np.zeros((3, ncell))
    sp[0, 1:inne + 1] = np.broadcast_to(xc[None, None, :], (ny, nz, nx))[sel]
    sp[1, 1:inne + 1] = np.broadcast_to(yc[:, None, None], (ny, nz, nx))[sel]
    sp[2, 1:inne + 1] = (np.broadcast_to(zk3, (ny, nz, nx)) + f_grid * dz)[sel]

    # ---- provisional face velocities (minus faces), noise on wet faces
    cg = math.sqrt(G_ACC / depth)
    xface = ii * dx
    eta_f = amplitude * _sech2(kw * (xface - x0))
    u_grid = np.broadcast_to((eta_f * cg)[None, None, :], (ny, nz, nx))
    w_prof = (zk / depth)[None, :, None] * (0.1 * cg * eta_c)[None, None, :]
    wet = f_grid > 0.0
    un = np.zeros((ncell, 3))
    nw = int(sel.sum())
    noise_vals = rng.normal(0.0, noise, size=(nw, 3)) if noise > 0 else np.zeros((nw, 3))
    wet_s = wet[sel]
    un[1:inne + 1, 0] = np.where(wet_s, u_grid[sel] + noise_vals[:, 0], 0.0)
    un[1:inne + 1, 1] = np.where(wet_s, noise_vals[:, 1], 0.0)
    un[1:inne + 1, 2] = np.where(wet_s, np.broadcast_to(w_prof, (ny, nz, nx))[sel] + noise_vals[:, 2], 0.0)

    return Case(nx=nx, ny=ny, nz=nz, dims=dims, mx2=mx2, x=x, dx=dxa, mn=mn,
                inne=inne, inne2=inne2, in_=in_, jn=jn, kn=kn, nf=nf, nfb=nfb,
                f=f, fb=fb, a=a, un=un, sp=sp, objno=np.zeros(ncell, dtype=np.int32),
                dt=dt, eps0=eps0, seed=seed, label=label)


# ---------------------------------------------------------------------------
# The five workloads.  Sizes, spacings and seeds are fixed here.

def tank_64x64x32(seed: int = 0) -> Case:
    """Flat-bottom tank 64x64x32, dx=dy=0.05, dz=0.025, fb=1, A=0.05, tol 1e-12."""
    return make_case(64, 64, 32, dx=0.05, dy=0.05, dz=0.025, slope=None, n_obstacles=0,
                     amplitude=0.05, partial=False, seed=seed, eps0=1.0e-12,
                     label="tank_64x64x32")


def beach_case(nx: int, ny: int, nz: int, *, seed: int, slope: float = 1.0 / 20.0,
               n_obstacles: int = 40, amplitude: float = 0.05, eps0: float = 1.0e-10,
               label: str = "") -> Case:
    """Sloping beach from x=0.4L, seeded obstacles (10% of plan area), partial cells."""
    return make_case(nx, ny, nz, dx=0.05, dy=0.05, dz=0.8 / nz, slope=slope,
                     n_obstacles=n_obstacles, obstacle_frac=0.10, amplitude=amplitude,
                     partial=True, seed=seed, eps0=eps0,
                     label=label or f"beach_{nx}x{ny}x{nz}")


def beach_256x256x96(seed: int = 1) -> Case:
    return beach_case(256, 256, 96, seed=seed, label="beach_256x256x96")


def beach_512x384x128(seed: int = 2) -> Case:
    return beach_case(512, 384, 128, seed=seed, label="beach_512x384x128")


def beach_192x192x64(seed: int = 4) -> Case:
    return beach_case(192, 192, 64, seed=seed, label="beach_192x192x64")


def ensemble_members(n: int = 64, seed: int = 3, scale: float = 1.0):
    """Member specs for the batched ensemble: grids U[96,256]x U[96,192] x U[48,80],
    slope U(1/30, 1/10), obstacle count 0-40, amplitude U(0.01, 0.1).

    ``scale`` shrinks the grid extents (used by small CPU/GPU tests)."""
    rng = np.random.default_rng(seed)
    specs = []
    for m in range(n):
        nx = int(rng.integers(96, 257))
        ny = int(rng.integers(96, 193))
        nz = int(rng.integers(48, 81))
        slope = float(rng.uniform(1.0 / 30.0, 1.0 / 10.0))
        nob = int(rng.integers(0, 41))
        amp = float(rng.uniform(0.01, 0.1))
        if scale != 1.0:
            nx = max(8, int(nx * scale))
            ny = max(8, int(ny * scale))
            nz = max(8, int(nz * scale))
            nob = min(nob, max(0, (nx * ny) // 64))
        specs.append(dict(nx=nx, ny=ny, nz=nz, slope=slope, n_obstacles=nob,
                          amplitude=amp, seed=seed * 1000 + m))
    return specs


def ensemble_case(spec: dict) -> Case:
    return beach_case(spec["nx"], spec["ny"], spec["nz"], seed=spec["seed"],
                      slope=spec["slope"], n_obstacles=spec["n_obstacles"],
                      amplitude=spec["amplitude"],
                      label=f"member_{spec['nx']}x{spec['ny']}x{spec['nz']}")


# ---------------------------------------------------------------------------
# 2DH dispersion systems (the matrix PCGPME_WILL solves, pcgpme_2DH.f90), built
# like disp_param (1sub-2DH-initial_reset.f90:470-506): one row per wet cell of
# an nx x ny plan grid; per direction (x, then y) a cell on the domain edge gets
# no entries, otherwise its wet minus and plus neighbours are packed into the
# next slots of AL(NA,4) / LL(NA,4) (NA = N, LL 1-based, zeros only after the
# last neighbour) with AL = A 2 h^2 / (dx (dx + dx)), and DIAG = -1 - sum(AL).
# The depth h varies, so rows differ in scale.  Dry cells (a seeded island and
# a shoreline band) are not rows.


@dataclasses.dataclass
class DispersionSystem:
    al: np.ndarray      # (4, n) float64
    ll: np.ndarray      # (4, n) int32
    d: np.ndarray       # (n,)
    b: np.ndarray       # (n,)
    n: int
    nx: int
    ny: int


def dispersion_system(nx: int, ny: int, seed: int = 7, dx: float = 0.5, A: float = 1.0 / 3.0) -> DispersionSystem:
    rng = np.random.default_rng(seed)
    xs = (np.arange(nx) + 0.5) / nx
    ys = (np.arange(ny) + 0.5) / ny
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    h = 0.2 + 2.0 * X + 0.3 * np.sin(6.0 * Y) * X          # depth, shallow near x = 0
    wet = h > 0.25
    cx, cy, r = rng.uniform(0.4, 0.7), rng.uniform(0.3, 0.7), rng.uniform(0.05, 0.12)
    wet &= (X - cx) ** 2 + (Y - cy) ** 2 > r * r           # island
    num = -np.ones((nx, ny), dtype=np.int64)
    idx = np.argwhere(wet.T)                                # row order: i fastest within j
    n = len(idx)
    jr, ir = idx[:, 0], idx[:, 1]
    num[ir, jr] = np.arange(n)
    # candidates in the reference's order: x-, x+ (if the cell is inside in x), y-, y+
    cand = -np.ones((n, 4), dtype=np.int64)
    inx = (ir > 0) & (ir + 1 < nx)
    iny = (jr > 0) & (jr + 1 < ny)
    cand[inx, 0] = num[ir[inx] - 1, jr[inx]]
    cand[inx, 1] = num[ir[inx] + 1, jr[inx]]
    cand[iny, 2] = num[ir[iny], jr[iny] - 1]
    cand[iny, 3] = num[ir[iny], jr[iny] + 1]
    order = np.argsort(cand < 0, axis=1, kind="stable")     # pack existing neighbours first
    packed = np.take_along_axis(cand, order, axis=1)
    present = packed >= 0
    hc = h[ir, jr]
    coef = A * 2.0 * hc * hc / dx / (dx + dx)
    al = np.where(present, coef[:, None], 0.0).T.copy()
    ll = np.where(present, packed + 1, 0).astype(np.int32).T.copy()
    d = -1.0 - (((al[0] + al[1]) + al[2]) + al[3])        # DIAG = -1 - sum(AL), summed in slot order
    b = rng.normal(0.0, 1.0, n) * np.exp(-((idx[:, 1] / nx - 0.5) ** 2) * 20.0)
    return DispersionSystem(al=al, ll=ll, d=d, b=b, n=n, nx=nx, ny=ny)
