"""Geometry and initial conditions (ghost-inclusive FP64 Fortran-order arrays).

``grid`` follows ``init_geom`` (mhd3d3.f90:3379-3515): uniform nodes, ghost
nodes extended linearly, dxblock(i) = x(i+1) - x(i), cell centres as the mean
of the 8 corners, face centres as the mean of 4.  The generators return a
``State`` whose ghost values are placeholders: ``mhd_init`` (and the oracle)
re-apply the ghost fill, as ``initialization`` does (mhd3d3.f90:3349-3351).

Generators:
* ``shock_tube``      -- Brio-Wu-type tube of ``init_ic`` (mhd3d3.f90:3517-3583), axis x/y/z.
* ``orszag_tang_2d``  -- point-sampled vortex of ``init_ic_otv`` (mhd3d2.f90:3420-3438).
* ``orszag_tang_3d``  -- 3-D OT with vz = 0.1 sin 2 pi z, B from an edge vector
                         potential (div B = 0 to round-off), seeded rho noise.
* ``blast``           -- magnetised blast (after ``init_ic_bws``, mhd3d2.f90:3358-3418, as a 3-D sphere).
* ``blast_bws``       -- ``init_ic_bws`` as written: the pressure cylinder about the domain origin.
* ``implosion``       -- diagonal-interface implosion (``init_ic_imp``, mhd3d2.f90:3440-3471).
* ``turbulence``      -- solenoidal Gaussian-random v and B, E(k) ~ k^-2 on
                         kmin <= |k| <= kmax, B from a vector potential.

Curvilinear (metric-mode) states carry ``nodes`` (ghost-inclusive node
coordinates X, Y, Z of shape (nx+1, ny+1, nz+1)) and hold in bi/bj/bk the
magnetic flux Phi = B.A through each face instead of B:
* ``mapped_grid``      -- logical grid plus nodes of x = xi + a sin 2 pi eta,
                          y = eta + a sin 2 pi zeta, z = zeta (or the identity).
* ``mapped_blast``     -- magnetised blast on a mapped grid, Phi = B.A.
* ``mapped_orszag_tang`` -- 3-D Orszag-Tang on a mapped grid, Phi = loop
                          integral of the vector potential (div-free exactly).
* ``uniform_flow``     -- uniform rho, p, v and B on a mapped grid.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

PI = 4.0 * np.arctan(1.0)


@dataclass
class Grid:
    nx0: int
    ny0: int
    nz0: int
    ng: int
    xn: np.ndarray  # node coordinates, ghost-inclusive (n+1)
    yn: np.ndarray
    zn: np.ndarray

    @property
    def nx(self):
        return self.nx0 + 2 * self.ng

    @property
    def ny(self):
        return self.ny0 + 2 * self.ng

    @property
    def nz(self):
        return self.nz0 + 2 * self.ng

    @property
    def dx(self):
        return np.diff(self.xn)

    @property
    def dy(self):
        return np.diff(self.yn)

    @property
    def dz(self):
        return np.diff(self.zn)

    def centres(self):
        """Cell centres as .125*(8 corners) in the order of mhd3d3.f90:3475-3483."""
        def c(a):
            lo, hi = a[:-1], a[1:]
            return 0.125 * (lo + lo + hi + hi + lo + lo + hi + hi)
        return c(self.xn), c(self.yn), c(self.zn)

    def face_centres(self):
        def m(a):
            return 0.25 * (a[:-1] + a[1:] + a[:-1] + a[1:])
        return m(self.xn), m(self.yn), m(self.zn)


def _nodes(n0, ng, lo, hi):
    d0 = (hi - lo) / n0
    x0 = np.arange(n0 + 1, dtype=np.float64) * d0 + lo
    xx = np.empty(n0 + 2 * ng + 1)
    xx[ng:ng + n0 + 1] = x0
    for i in range(1, ng + 1):  # 1-based as in init_geom
        xx[i - 1] = 2.0 * x0[0] - x0[ng + 2 - i - 1]
        xx[n0 + 2 * ng + 2 - i - 1] = 2.0 * x0[n0] - x0[n0 - ng + i - 1]
    return xx


def grid(nx0, ny0, nz0, nord=8, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)) -> Grid:
    ng = nord // 2
    return Grid(nx0, ny0, nz0, ng, _nodes(nx0, ng, lo[0], hi[0]), _nodes(ny0, ng, lo[1], hi[1]),
                _nodes(nz0, ng, lo[2], hi[2]))


@dataclass
class State:
    rho: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    vz: np.ndarray
    p: np.ndarray
    bi: np.ndarray
    bj: np.ndarray
    bk: np.ndarray
    grid: Grid
    nodes: tuple | None = None  # metric mode: (X, Y, Z) node coordinates

    def arrays(self):
        return [self.rho, self.vx, self.vy, self.vz, self.p, self.bi, self.bj, self.bk]


def empty_state(g: Grid, nodes=None) -> State:
    cs = (g.nx, g.ny, g.nz)
    z = lambda s: np.zeros(s, dtype=np.float64, order="F")
    return State(z(cs), z(cs), z(cs), z(cs), z(cs), z((g.nx + 1, g.ny, g.nz)),
                 z((g.nx, g.ny + 1, g.nz)), z((g.nx, g.ny, g.nz + 1)), g, nodes)


def _bcast(g: Grid):
    xc, yc, zc = g.centres()
    return xc[:, None, None], yc[None, :, None], zc[None, None, :]


def shock_tube(n: int, axis: int = 2, nord: int = 8, ntrans: int = 8) -> State:
    """Brio-Wu-type tube on [-1,1]^3 (mhd3d3.in dom; init_ic mhd3d3.f90:3517-3583).
    axis 2 is the active variant (z); 0 and 1 are its commented-out x/y twins."""
    sizes = [ntrans, ntrans, ntrans]
    sizes[axis] = n
    g = grid(*sizes, nord=nord, lo=(-1.0, -1.0, -1.0), hi=(1.0, 1.0, 1.0))
    s = empty_state(g)
    s.rho[...] = 1.0
    s.p[...] = 1.0
    c = _bcast(g)[axis]
    hi = np.broadcast_to(c >= 0.0, s.rho.shape)
    s.rho[hi] = 0.125
    s.p[hi] = 0.1
    fb = [s.bi, s.bj, s.bk]
    # z tube: bk=.75 (normal), bi=-1 (transverse), bj=0, bi=1 where zi<0;
    # x tube: bi=.75, bj=-1 (bj=1 where xj<0); y tube: bj=.75, bk=-1 (bk=1 where yk<0)
    normal, trans = axis, (axis + 1) % 3
    fb[normal][...] = 0.75
    fb[trans][...] = -1.0
    fb[3 - normal - trans][...] = 0.0
    xf, yf, zf = g.face_centres()
    # position of the transverse face array's centres along the tube axis
    if trans == 0:
        pos = [g.xn, yf, zf][axis]
    elif trans == 1:
        pos = [xf, g.yn, zf][axis]
    else:
        pos = [xf, yf, g.zn][axis]
    shape = [1, 1, 1]
    shape[axis] = -1
    low = np.broadcast_to((pos < 0.0).reshape(shape), fb[trans].shape)
    fb[trans][low] = 1.0
    return s


def orszag_tang_2d(n: int, nz0: int = 8, nord: int = 8) -> State:
    """Point-sampled Orszag-Tang vortex of init_ic_otv (mhd3d2.f90:3420-3438),
    uniform in z, on [0,1]^2 x [0,1]."""
    g = grid(n, n, nz0, nord=nord)
    s = empty_state(g)
    xc, yc, _ = _bcast(g)
    xf, yf, _ = g.face_centres()
    s.rho[...] = 25.0 / (36.0 * PI)
    s.p[...] = 5.0 / (12.0 * PI)
    s.vx[...] = -np.sin(2.0 * PI * yc)
    s.vy[...] = np.sin(2.0 * PI * xc)
    s.vz[...] = 0.0
    s.bi[...] = -1.0 / np.sqrt(4.0 * PI) * np.sin(2.0 * PI * yf[None, :, None])
    s.bj[...] = 1.0 / np.sqrt(4.0 * PI) * np.sin(4.0 * PI * xf[:, None, None])
    s.bk[...] = 0.0
    return s


def _faces_from_potential(g: Grid, ax, ay, az):
    """Face B = discrete curl of edge potentials on a periodic interior grid.
    ax[i,j,k] at (x centre i, y node j, z node k), ay at (x node, y centre, z
    node), az at (x node, y node, z centre); interior-sized periodic arrays.
    Returns interior-sized bi (n0x+1,...) etc. with the top faces wrapped."""
    dx, dy, dz = g.dx[g.ng], g.dy[g.ng], g.dz[g.ng]
    r = np.roll
    bi = (r(az, -1, 1) - az) / dy - (r(ay, -1, 2) - ay) / dz
    bj = (r(ax, -1, 2) - ax) / dz - (r(az, -1, 0) - az) / dx
    bk = (r(ay, -1, 0) - ay) / dx - (r(ax, -1, 1) - ax) / dy
    return bi, bj, bk


def _embed(s: State, cells: dict, faces=None):
    g = s.grid
    ng = g.ng
    sl = (slice(ng, ng + g.nx0), slice(ng, ng + g.ny0), slice(ng, ng + g.nz0))
    for name, a in cells.items():
        getattr(s, name)[sl] = a
    if faces is not None:
        bi, bj, bk = faces
        s.bi[ng:ng + g.nx0, sl[1], sl[2]] = bi
        s.bi[ng + g.nx0, sl[1], sl[2]] = bi[0]  # top face = periodic image of face 0
        s.bj[sl[0], ng:ng + g.ny0, sl[2]] = bj
        s.bj[sl[0], ng + g.ny0, sl[2]] = bj[:, 0]
        s.bk[sl[0], sl[1], ng:ng + g.nz0] = bk
        s.bk[sl[0], sl[1], ng + g.nz0] = bk[:, :, 0]


def orszag_tang_3d(n: int, seed: int = 0, noise: float = 1e-3, nord: int = 8, amp: float = 1.0,
                   beta_scale: float = 1.0, ny0: int | None = None, nz0: int | None = None) -> State:
    """3-D Orszag-Tang on the periodic unit box: rho = 25/(36 pi) + U(-noise,
    noise) (numpy default_rng(seed), [k][j][i] order), p = 5/(12 pi) * beta_scale,
    v = amp*(-sin 2 pi y, sin 2 pi x, 0.1 sin 2 pi z), face B = discrete curl of
    A_z = [cos(2 pi y)/(2 pi) + cos(4 pi x)/(4 pi)]/sqrt(4 pi) on z-edges."""
    ny0 = n if ny0 is None else ny0
    nz0 = n if nz0 is None else nz0
    g = grid(n, ny0, nz0, nord=nord)
    s = empty_state(g)
    ng = g.ng
    xc, yc, zc = [c[ng:ng + m] for c, m in zip(g.centres(), (n, ny0, nz0))]
    xn, yn = g.xn[ng:ng + n], g.yn[ng:ng + ny0]
    rng = np.random.default_rng(seed)
    dn = rng.uniform(-noise, noise, size=(nz0, ny0, n)).transpose(2, 1, 0)
    X, Y, Z = np.meshgrid(xc, yc, zc, indexing="ij")
    cells = {
        "rho": 25.0 / (36.0 * PI) + dn,
        "p": np.full(X.shape, 5.0 / (12.0 * PI) * beta_scale),
        "vx": -amp * np.sin(2.0 * PI * Y),
        "vy": amp * np.sin(2.0 * PI * X),
        "vz": amp * 0.1 * np.sin(2.0 * PI * Z),
    }
    XN, YN = np.meshgrid(xn, yn, indexing="ij")
    az2 = (np.cos(2.0 * PI * YN) / (2.0 * PI) + np.cos(4.0 * PI * XN) / (4.0 * PI)) / np.sqrt(4.0 * PI)
    az = np.repeat(az2[:, :, None], nz0, axis=2)
    zero = np.zeros_like(az)
    _embed(s, cells, _faces_from_potential(g, zero, zero, az))
    return s


def blast(n: int, nord: int = 8, p_in: float = 10.0, p_out: float = 0.1, r0: float = 0.1) -> State:
    """Magnetised blast: rho = 1, p = p_out, p = p_in for r < r0 about the box
    centre, B = (1, 1, 0)/sqrt(2) (uniform face B); unit box (cf. init_ic_bws,
    mhd3d2.f90:3358-3418, which uses a cylinder, p=.1/10 and B=.5)."""
    g = grid(n, n, n, nord=nord)
    s = empty_state(g)
    xc, yc, zc = _bcast(g)
    s.rho[...] = 1.0
    r2 = (xc - 0.5) ** 2 + (yc - 0.5) ** 2 + (zc - 0.5) ** 2
    s.p[...] = np.where(r2 < r0 * r0, p_in, p_out)
    s.bi[...] = 1.0 / np.sqrt(2.0)
    s.bj[...] = 1.0 / np.sqrt(2.0)
    s.bk[...] = 0.0
    return s


def blast_bws(n: int, nz0: int = 8, nord: int = 8, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)) -> State:
    """init_ic_bws (mhd3d2.f90:3358-3418) as written, on the deck's domain
    (mhd3d2.in: the unit box): rho = 1, v = 0, p = .1, and p = 10 where
    xc^2 + yc^2 < .01 -- a cylinder of radius .1 along z about the origin of
    the coordinates -- with bi = bj = .5, bk = 0.  The reference keeps its
    call commented out (mhd3d2.f90:3186) in favour of init_ic_otv."""
    g = grid(n, n, nz0, nord=nord, lo=lo, hi=hi)
    s = empty_state(g)
    xc, yc, _ = _bcast(g)
    s.rho[...] = 1.0
    s.p[...] = np.where(np.broadcast_to(xc ** 2 + yc ** 2 < 0.01, s.p.shape), 10.0, 0.1)
    s.bi[...] = 0.5
    s.bj[...] = 0.5
    s.bk[...] = 0.0
    return s


def implosion(n: int, nz0: int = 8, nord: int = 8) -> State:
    """Hydrodynamic implosion of init_ic_imp (mhd3d2.f90:3440-3471): rho=p=1
    where x+y >= .150001, else rho=.125, p=.14; B = 0, v = 0."""
    g = grid(n, n, nz0, nord=nord)
    s = empty_state(g)
    xc, yc, _ = _bcast(g)
    m = np.broadcast_to((xc + yc) >= 0.150001, s.rho.shape)
    s.rho[...] = np.where(m, 1.0, 0.125)
    s.p[...] = np.where(m, 1.0, 0.14)
    return s


def _solenoidal(n, rng, kmin, kmax, slope, shift=(0.0, 0.0, 0.0)):
    k1 = np.fft.fftfreq(n, d=1.0 / n)
    KX, KY, KZ = np.meshgrid(k1, k1, k1, indexing="ij")
    kk = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    band = (kk >= kmin) & (kk <= kmax)
    amp = np.zeros_like(kk)
    amp[band] = kk[band] ** ((slope - 2.0) / 2.0)
    comp = [(rng.standard_normal(kk.shape) + 1j * rng.standard_normal(kk.shape)) * amp for _ in range(3)]
    k2 = np.where(kk > 0, kk ** 2, 1.0)
    dot = (KX * comp[0] + KY * comp[1] + KZ * comp[2]) / k2
    comp = [comp[0] - KX * dot, comp[1] - KY * dot, comp[2] - KZ * dot]
    return comp, (KX, KY, KZ), kk


def _sample(fk, K, shift, n):
    KX, KY, KZ = K
    ph = np.exp(2j * PI * (KX * shift[0] + KY * shift[1] + KZ * shift[2]) / n)
    return np.real(np.fft.ifftn(fk * ph))


def turbulence(n: int, seed: int = 0, ms: float = 0.5, vrms: float = 1.0, brms: float = 0.5,
               kmin: float = 2.0, kmax: float = 8.0, slope: float = -2.0, nord: int = 8,
               gam: float = 5.0 / 3.0) -> State:
    """Decaying-turbulence start on the periodic unit box: rho = 1,
    p = 1/(gam*ms^2), v and B solenoidal Gaussian-random with E(k) ~ k^slope on
    kmin <= |k| <= kmax (numpy default_rng(seed)), rms vrms and brms; B is the
    discrete curl of an edge vector potential, so div B = 0 to round-off."""
    rng = np.random.default_rng(seed)
    g = grid(n, n, n, nord=nord)
    s = empty_state(g)
    vk, K, kk = _solenoidal(n, rng, kmin, kmax, slope)
    v = [_sample(c, K, (0.5, 0.5, 0.5), n) for c in vk]
    vs = vrms / np.sqrt(np.mean(v[0] ** 2 + v[1] ** 2 + v[2] ** 2))
    bk_, _, _ = _solenoidal(n, rng, kmin, kmax, slope)
    # A = i k x B / k^2, sampled on edges
    KX, KY, KZ = K
    k2 = np.where(kk > 0, kk ** 2, 1.0) * (2.0 * PI)  # physical k = 2 pi k_int on the unit box
    axk = 1j * (KY * bk_[2] - KZ * bk_[1]) / k2
    ayk = 1j * (KZ * bk_[0] - KX * bk_[2]) / k2
    azk = 1j * (KX * bk_[1] - KY * bk_[0]) / k2
    ax = _sample(axk, K, (0.5, 0.0, 0.0), n)
    ay = _sample(ayk, K, (0.0, 0.5, 0.0), n)
    az = _sample(azk, K, (0.0, 0.0, 0.5), n)
    bi, bj, bk = _faces_from_potential(g, ax, ay, az)
    bc2 = (0.5 * (bi + np.roll(bi, -1, 0))) ** 2 + (0.5 * (bj + np.roll(bj, -1, 1))) ** 2 + \
          (0.5 * (bk + np.roll(bk, -1, 2))) ** 2
    bs = brms / np.sqrt(np.mean(bc2))
    cells = {
        "rho": np.ones((n, n, n)),
        "p": np.full((n, n, n), 1.0 / (gam * ms * ms)),
        "vx": v[0] * vs, "vy": v[1] * vs, "vz": v[2] * vs,
    }
    _embed(s, cells, (bi * bs, bj * bs, bk * bs))
    return s


def cfl_dt(s: State, gam: float = 5.0 / 3.0, cfl: float = 0.3) -> float:
    """get_dt (mhd3d3.f90:1608-1639) on the interior of a state with cell B
    from the face means (used to pick a fixed RK dt)."""
    g = s.grid
    ng = g.ng
    sl = (slice(ng, ng + g.nx0), slice(ng, ng + g.ny0), slice(ng, ng + g.nz0))
    bx = 0.5 * (s.bi[1:, :, :] + s.bi[:-1, :, :])[sl]
    by = 0.5 * (s.bj[:, 1:, :] + s.bj[:, :-1, :])[sl]
    bz = 0.5 * (s.bk[:, :, 1:] + s.bk[:, :, :-1])[sl]
    r, p = s.rho[sl], s.p[sl]
    v = np.sqrt(s.vx[sl] ** 2 + s.vy[sl] ** 2 + s.vz[sl] ** 2)
    vc = v + np.sqrt((bx ** 2 + by ** 2 + bz ** 2) / r + gam * p / r)
    dx = g.dx[sl[0]][:, None, None]
    dy = g.dy[sl[1]][None, :, None]
    dz = g.dz[sl[2]][None, None, :]
    return float(np.min(cfl / (vc / dx + vc / dy + vc / dz)))


# ---------------------------------------------------------------- mapped grids
def mapped_grid(nx0, ny0, nz0, nord=8, amp=0.05, kind="sine"):
    """Logical grid on [0,1]^3 (nodes extended into the ghosts as in init_geom)
    and the ghost-inclusive physical node coordinates of the mapping
    x = xi + amp sin(2 pi eta), y = eta + amp sin(2 pi zeta), z = zeta
    (kind "sine") or of the identity (kind "cartesian").  The sine mapping
    is periodic in shape: x(xi + 1) = x(xi) + 1 and so on."""
    g = grid(nx0, ny0, nz0, nord=nord)
    XI, ETA, ZETA = np.meshgrid(g.xn, g.yn, g.zn, indexing="ij")
    if kind == "sine":
        X = XI + amp * np.sin(2.0 * PI * ETA)
        Y = ETA + amp * np.sin(2.0 * PI * ZETA)
        Z = ZETA.copy()
    elif kind == "cartesian":
        X, Y, Z = XI.copy(), ETA.copy(), ZETA.copy()
    else:
        raise ValueError(kind)
    f = lambda a: np.asfortranarray(a, dtype=np.float64)
    return g, (f(X), f(Y), f(Z))


def face_areas(nodes):
    """Low-face area vectors 0.5 (d1 x d2) from the face diagonals, for the
    x, y and z face families: list of 3 arrays of shape (..., 3)."""
    P = np.stack(nodes, axis=-1)
    out = []
    for ax in range(3):
        t1, t2 = (ax + 1) % 3, (ax + 2) % 3
        n = P.shape[:3]
        ext = [n[0] - 1, n[1] - 1, n[2] - 1]
        ext[ax] = n[ax]

        def at(o1, o2):
            sl = [slice(0, e) for e in ext]
            if o1:
                sl[t1] = slice(1, ext[t1] + 1)
            if o2:
                sl[t2] = slice(1, ext[t2] + 1)
            return P[tuple(sl)]
        d1 = at(1, 1) - at(0, 0)
        d2 = at(0, 1) - at(1, 0)
        out.append(0.5 * np.cross(d1, d2))
    return out


def cell_centres_mapped(nodes):
    """Physical cell centres: mean of the 8 corner nodes."""
    out = []
    for a in nodes:
        out.append(0.125 * (a[:-1, :-1, :-1] + a[1:, :-1, :-1] + a[:-1, 1:, :-1] + a[1:, 1:, :-1] +
                            a[:-1, :-1, 1:] + a[1:, :-1, 1:] + a[:-1, 1:, 1:] + a[1:, 1:, 1:]))
    return out


def _phi_uniform(s: State, B):
    for arr, A in zip((s.bi, s.bj, s.bk), face_areas(s.nodes)):
        arr[...] = A[..., 0] * B[0] + A[..., 1] * B[1] + A[..., 2] * B[2]


def mapped_blast(n: int, nord: int = 8, amp: float = 0.05, p_in: float = 10.0, p_out: float = 0.1,
                 r0: float = 0.1, kind: str = "sine", ny0=None, nz0=None) -> State:
    """Magnetised blast on a mapped grid: rho = 1, v = 0, p = p_out and p_in
    where the physical cell centre lies within r0 of (0.5, 0.5, 0.5), uniform
    B = (1, 1, 0)/sqrt(2) stored as face fluxes Phi = B.A."""
    g, nodes = mapped_grid(n, n if ny0 is None else ny0, n if nz0 is None else nz0, nord=nord, amp=amp,
                           kind=kind)
    s = empty_state(g, nodes)
    xc, yc, zc = cell_centres_mapped(nodes)
    r2 = (xc - 0.5) ** 2 + (yc - 0.5) ** 2 + (zc - 0.5) ** 2
    s.rho[...] = 1.0
    s.p[...] = np.where(r2 < r0 * r0, p_in, p_out)
    _phi_uniform(s, (1.0 / np.sqrt(2.0), 1.0 / np.sqrt(2.0), 0.0))
    return s


def uniform_flow(n: int, v=(0.3, -0.2, 0.1), B=(0.0, 0.0, 0.0), rho: float = 1.0, p: float = 0.6,
                 nord: int = 8, amp: float = 0.05, kind: str = "sine") -> State:
    """Uniform rho, p, v and B (Phi = B.A) on a mapped grid."""
    g, nodes = mapped_grid(n, n, n, nord=nord, amp=amp, kind=kind)
    s = empty_state(g, nodes)
    s.rho[...] = rho
    s.p[...] = p
    s.vx[...], s.vy[...], s.vz[...] = v
    _phi_uniform(s, B)
    return s


def _edge_circulation(nodes, afun):
    """Line integrals of the vector potential along every cell edge, midpoint
    rule: afun(x, y, z) -> (Ax, Ay, Az) at the edge midpoint, dotted with the
    edge vector.  Returns [x-edges, y-edges, z-edges]."""
    out = []
    for e in range(3):
        sl0 = [slice(None)] * 3
        sl1 = [slice(None)] * 3
        sl0[e] = slice(0, -1)
        sl1[e] = slice(1, None)
        p0 = [a[tuple(sl0)] for a in nodes]
        p1 = [a[tuple(sl1)] for a in nodes]
        mid = [0.5 * (a + b) for a, b in zip(p0, p1)]
        A = afun(*mid)
        out.append(sum(A[c] * (p1[c] - p0[c]) for c in range(3)))
    return out


def mapped_orszag_tang(n: int, nord: int = 8, amp: float = 0.05, seed: int = 0, noise: float = 1e-3,
                       kind: str = "sine", ny0=None, nz0=None) -> State:
    """3-D Orszag-Tang on a periodic mapped grid: the Cartesian generator's
    rho, p and v at the physical cell centres, and face fluxes Phi from the
    loop integrals of A_z = [cos(2 pi y)/(2 pi) + cos(4 pi x)/(4 pi)]/sqrt(4 pi)
    around each face (so the discrete div B is zero to round-off)."""
    ny0 = n if ny0 is None else ny0
    nz0 = n if nz0 is None else nz0
    g, nodes = mapped_grid(n, ny0, nz0, nord=nord, amp=amp, kind=kind)
    s = empty_state(g, nodes)
    xc, yc, zc = cell_centres_mapped(nodes)
    rng = np.random.default_rng(seed)
    s.rho[...] = 25.0 / (36.0 * PI) + rng.uniform(-noise, noise, size=s.rho.shape[::-1]).transpose(2, 1, 0)
    s.p[...] = 5.0 / (12.0 * PI)
    s.vx[...] = -np.sin(2.0 * PI * yc)
    s.vy[...] = np.sin(2.0 * PI * xc)
    s.vz[...] = 0.1 * np.sin(2.0 * PI * zc)

    def afun(x, y, z):
        az = (np.cos(2.0 * PI * y) / (2.0 * PI) + np.cos(4.0 * PI * x) / (4.0 * PI)) / np.sqrt(4.0 * PI)
        return (0.0 * x, 0.0 * x, az)
    ex, ey, ez = _edge_circulation(nodes, afun)
    # Phi through the low face = circulation around its loop (right-handed
    # about the +axis normal), the same orientation as the CT update
    s.bi[...] = (ez[:, 1:, :] - ez[:, :-1, :]) - (ey[:, :, 1:] - ey[:, :, :-1])
    s.bj[...] = (ex[:, :, 1:] - ex[:, :, :-1]) - (ez[1:, :, :] - ez[:-1, :, :])
    s.bk[...] = (ey[1:, :, :] - ey[:-1, :, :]) - (ex[:, 1:, :] - ex[:, :-1, :])
    return s


def cfl_dt_mapped(s: State, gam: float = 5.0 / 3.0, cfl: float = 0.3) -> float:
    """CFL dt of a mapped state on its interior: cfl V / (vcfl sum_a |Abar_a|),
    cell B from the face fluxes (B = sum_a Phibar_a / V * e_a)."""
    g = s.grid
    ng = g.ng
    A = face_areas(s.nodes)
    # volumes by the divergence theorem over face centroids
    P = np.stack(s.nodes, axis=-1)
    cen = []
    for ax in range(3):
        t1, t2 = (ax + 1) % 3, (ax + 2) % 3
        n = P.shape[:3]
        ext = [n[0] - 1, n[1] - 1, n[2] - 1]
        ext[ax] = n[ax]
        acc = 0
        for o1 in (0, 1):
            for o2 in (0, 1):
                sl = [slice(0, e) for e in ext]
                if o1:
                    sl[t1] = slice(1, ext[t1] + 1)
                if o2:
                    sl[t2] = slice(1, ext[t2] + 1)
                acc = acc + P[tuple(sl)]
        cen.append(0.25 * acc)
    V = 0
    eb = []
    for ax in range(3):
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, -1)
        hi[ax] = slice(1, None)
        V = V + (np.sum(cen[ax][tuple(hi)] * A[ax][tuple(hi)], -1) - np.sum(cen[ax][tuple(lo)] * A[ax][tuple(lo)], -1))
        eb.append(cen[ax][tuple(hi)] - cen[ax][tuple(lo)])
    V = V / 3.0
    phis = (s.bi, s.bj, s.bk)
    Bc = 0
    ssum = 0
    for ax in range(3):
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, -1)
        hi[ax] = slice(1, None)
        ph = 0.5 * (phis[ax][tuple(hi)] + phis[ax][tuple(lo)]) / V
        Bc = Bc + ph[..., None] * eb[ax]
        Ab = 0.5 * (A[ax][tuple(lo)] + A[ax][tuple(hi)])
        ssum = ssum + np.sqrt(np.sum(Ab * Ab, -1))
    sl = (slice(ng, ng + g.nx0), slice(ng, ng + g.ny0), slice(ng, ng + g.nz0))
    r, p = s.rho[sl], s.p[sl]
    v = np.sqrt(s.vx[sl] ** 2 + s.vy[sl] ** 2 + s.vz[sl] ** 2)
    b2 = np.sum(Bc[sl] ** 2, -1)
    vc = v + np.sqrt(b2 / r + gam * p / r)
    return float(np.min(cfl * V[sl] / (vc * ssum[sl])))
