"""ORACLE -- test infrastructure only.  Nothing in the product path imports
this file; tests use it to cross-check the C++ oracle.

A second, independent restatement of the reference's per-timestep update
(tiegcm/mhd3d_mpi_fortran, mhd3d3.f90), written in vectorised numpy straight
from the Fortran: one whole-array expression per Fortran statement or
``forall``, in the Fortran's own operand order.  It shares no code with
``oracle/mhd_oracle.cpp`` (a loop-per-element C++ restatement), so a
transcription slip in either shows up as a disagreement between them.

Scope: Cartesian mesh; per axis periodic halos (one rank of mhd3d2.f90's
periodic topology: the SENDRECVs of fillx_center / fillx_face,
mhd3d3.f90:346-390 / 482-525, exchange with the rank itself), the even wall
mirror those routines apply at a domain edge (xbc=0, the only value mhd3d3's
fill_hydro_mpi / fill_mag_mpi pass, 781-819), the reflecting mirror (odd
normal velocity, the xbc=1 of mhd3d2.f90:713, 720) or the zero-gradient
outflow copy (no reference counterpart); reconop 1 (PDM), 2 (TVD, van
Leer, with mhd3d2's stencil shifts when tvd_shift = 1), 3 (WENO5), 4
(MP-WENO5, the reference deck's choice) or 5 (TVD with the MC limiter, no
reference counterpart); LFM or Yee edge EMF;
stepop 1 (AB2, step_ab 3602-3644, CFL tau), 2 (RK2) or 3 (RK3, the deck's),
the last two with the deck's fixed tau (step_rk2 / step_rk3, 3646-3792).

The AB2 priming step takes the deck's tau where the reference hard-codes
tau=3.e-4 after get_dt (3356-3359), as the C++ oracle and the library do.

Arrays are indexed [i, j, k] from 0: numpy index n is Fortran index n + 1.
``erfc`` is scipy's and ``exp`` numpy's, so agreement with the C++ oracle
(glibc) is to round-off, not bit for bit.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erfc


def _sign1(x):
    # sign(1., x): +1 for x >= 0 (including -0.0), -1 otherwise
    return np.where(x >= 0.0, 1.0, -1.0)


def _max(a, b):
    return np.where(a > b, a, b)


def _min(a, b):
    return np.where(a < b, a, b)


def _tap8(a0, a1, a2, a3, a4, a5, a6, a7):
    # the 8-point interpolant of interp_pdm (mhd3d3.f90:862-924)
    return (-3. * a0 + 29. * a1 - 139. * a2 + 533. * a3 + 533. * a4 - 139. * a5 + 29. * a6 - 3. * a7) / 840.


class NumpyMHD:
    """One grid of the reference's state, advanced by RK2 or RK3 steps."""

    def __init__(self, params, state):
        p = params
        if p.reconop not in (1, 2, 3, 4, 5) or any(b not in (0, 1, 2, 3) for b in p.bc) or p.emf not in (0, 1):
            raise ValueError("NumpyMHD covers reconop 1-5, halo kinds 0-3 and the LFM / Yee EMFs")
        self.emf_kind, self.tvd_shift = p.emf, p.tvd_shift
        self.stepop, self.alpha, self.beta, self.cfl = p.stepop, p.alpha, p.beta, p.cfl
        self.dt_mode = p.dt_mode  # 1: RK steps take the CFL dt (no reference counterpart)
        self.bc = tuple(p.bc)
        self.nx0, self.ny0, self.nz0 = p.nx0, p.ny0, p.nz0
        self.ng, self.nord = p.nord // 2, p.nord
        self.nx, self.ny, self.nz = p.nx0 + p.nord, p.ny0 + p.nord, p.nz0 + p.nord
        self.reconop, self.gam, self.pdmb, self.eps = p.reconop, p.gam, p.pdmb, p.eps
        self.tau = self.tau0 = p.tau
        self.pi = 4. * np.arctan(1.0)  # pars: pi=4.*atan(1.0_8)
        g = state.grid
        ng = self.ng
        # dxblock over every cell, ghosts included (get_dt)
        self.dxa = np.asarray(g.dx)[:, None, None]
        self.dya = np.asarray(g.dy)[None, :, None]
        self.dza = np.asarray(g.dz)[None, None, :]
        # dxblock(ng+i, ng+j, ng+k) of the interior cells
        self.dx = np.asarray(g.dx)[ng:ng + self.nx0][:, None, None]
        self.dy = np.asarray(g.dy)[ng:ng + self.ny0][None, :, None]
        self.dz = np.asarray(g.dz)[ng:ng + self.nz0][None, None, :]
        c = lambda a: np.array(a, dtype=np.float64)
        self.rho, self.vx, self.vy, self.vz, self.p = (c(a) for a in state.arrays()[:5])
        self.bi, self.bj, self.bk = (c(a) for a in state.arrays()[5:])
        # initialisation (mhd3d3.f90:3349-3351)
        self.fill_hydro()
        self.fill_mag()
        self.get_bxyz()
        if self.stepop == 1:  # AB priming (mhd3d3.f90:3356-3373)
            dtc = self.get_dt()
            self.tau = self.tau0 = p.tau if p.tau > 0 else dtc
            self.rhop, self.vxp, self.vyp, self.vzp, self.pp = (a.copy() for a in (
                self.rho, self.vx, self.vy, self.vz, self.p))
            self.bxp, self.byp, self.bzp = self.bx.copy(), self.by.copy(), self.bz.copy()
            self.bip, self.bjp, self.bkp = self.bi.copy(), self.bj.copy(), self.bk.copy()

    # ------------------------------------------------------------ indexing
    def _take(self, f, off, lens, axes=(0, 1, 2)):
        """f(ng+i+off0, ng+j+off1, ng+k+off2) for i=1..lens0 etc.; an axis not
        in ``axes`` is taken whole (the ':' of the dir 4..6 forms)."""
        sl = []
        for a in range(3):
            if a in axes:
                s = self.ng + off[a]
                sl.append(slice(s, s + lens[a]))
            else:
                sl.append(slice(None))
        return f[tuple(sl)]

    def _stencil(self, f, d, lens, shift=(0, 0, 0), ms=range(-4, 4), axes=(0, 1, 2)):
        """[f at offset m along axis d] for m in ms, the element grid lens."""
        out = []
        for m in ms:
            off = list(shift)
            off[d] += m
            out.append(self._take(f, off, lens, axes))
        return out

    # ------------------------------------------------------ reconstruction
    def interp(self, f, lens, d, axes=(0, 1, 2)):
        """interp_pdm / interp_tvd (mhd3d3.f90:862-924, 991-1035), axis d = 0,1,2."""
        if self.reconop == 1:
            return _tap8(*self._stencil(f, d, lens, axes=axes))
        fm1, f0 = self._stencil(f, d, lens, ms=(-1, 0), axes=axes)  # TVD, TVD-MC
        return (fm1 + f0) / 2.

    def limit(self, f, fi, lens, d, shift=(0, 0, 0), axes=(0, 1, 2)):
        """PDM2 (mhd3d3.f90:1069-1172) or TVD: mhd3d3's (1174-1250) drops the
        stencil shifts, mhd3d2's (mhd3d2.f90:1137-1199, tvd_shift = 1) honours them."""
        tvd = self.reconop in (2, 5)
        if tvd and not self.tvd_shift:
            shift = (0, 0, 0)
        fm2, fm1, f0, fp1 = self._stencil(f, d, lens, shift, ms=(-2, -1, 0, 1), axes=axes)
        if tvd:
            # van Leer b = (a+|a|)/(1+|a|); TVD-MC (reconop 5, no reference
            # counterpart) b = max(0, min(2a, (1+a)/2, 2)), the MC limiter phi(a)
            def lim(a):
                if self.reconop == 5:
                    return _max(0., _min(_min(2. * a, .5 * (1. + a)), 2.))
                return (a + np.abs(a)) / (1. + np.abs(a))
            eps = self.eps
            a = (fm1 - fm2) / (f0 - fm1 + eps)
            fleft = fm1 - lim(a) * (fm1 - fi)
            a = (f0 - fp1) / (fm1 - f0 + eps)
            fright = f0 - lim(a) * (f0 - fi)
            return fleft, fright
        maxf = _max(fm1, f0)
        minf = _min(fm1, f0)
        fii = _max(minf, _min(fi, maxf))
        dfm = self.pdmb * (fm1 - fm2)
        df0 = self.pdmb * (f0 - fm1)
        dfp = self.pdmb * (fp1 - f0)
        sm, s0, sp = _sign1(dfm), _sign1(df0), _sign1(dfp)
        dfm, dfp = np.abs(dfm), np.abs(dfp)
        qm = np.abs(sm + s0)
        qp = np.abs(s0 + sp)
        dfl = fii - fm1
        dfr = f0 - fii
        fleft = fii - s0 * _max(0., np.abs(dfl) - qm * dfm)
        fright = fii + s0 * _max(0., np.abs(dfr) - qp * dfp)
        return fleft, fright

    def reconstruct(self, f, lens, d, axes=(0, 1, 2)):
        """reconstruct_3d (mhd3d3.f90:833-860) for dir = d+1 in 1..3; with
        axes=(d,) the dir 4..6 form (the other axes whole)."""
        if self.reconop in (3, 4):
            return self.weno(f, lens, d, axes)
        return self.limit(f, self.interp(f, lens, d, axes), lens, d, axes=axes)

    def weno(self, f, lens, d, axes=(0, 1, 2)):
        """WENO5 (mhd3d3.f90:1252-1378) and MPWENO5 (1405-1596)."""
        eps = self.eps
        fm3, fm2, fm1, f0, fp1, fp2 = self._stencil(f, d, lens, ms=range(-3, 3), axes=axes)

        def side(a3, a2, a1, b0, b1, b2):
            h0 = (2. * a3 - 7. * a2 + 11. * a1) / 6.
            h1 = (-a2 + 5. * a1 + 2. * b0) / 6.
            h2 = (2. * a1 + 5. * b0 - b1) / 6.
            s0 = 13. / 12. * (a3 - 2. * a2 + a1) ** 2 + .25 * (a3 - 4. * a2 + 3. * a1) ** 2
            s1 = 13. / 12. * (a2 - 2. * a1 + b0) ** 2 + .25 * (a2 - b0) ** 2
            s2 = 13. / 12. * (a1 - 2. * b0 + b1) ** 2 + .25 * (3. * a1 - 4. * b0 + b1) ** 2
            s0 = .1 / (eps + s0) ** 2
            s1 = .6 / (eps + s1) ** 2
            s2 = .3 / (eps + s2) ** 2
            t = s0 + s1 + s2
            return s0 / t * h0 + s1 / t * h1 + s2 / t * h2

        # left: (fm3, fm2, fm1, f0, fp1); right: the mirrored stencil
        fl = side(fm3, fm2, fm1, f0, fp1, fp2)
        fr = side(fp2, fp1, f0, fm1, fm2, fm3)
        if self.reconop == 3:
            return fl, fr
        return self._mp(fl, fm3, fm2, fm1, f0, fp1), self._mp(fr, fp2, fp1, f0, fm1, fm2)

    def _mp(self, w, a3, a2, a1, b0, b1):
        """The MP bound of one side (MPWENO5, mhd3d3.f90:1530-1591)."""
        def minmod(a, b):  # mhd3d3.f90:1380-1389
            return .5 * (_sign1(a) + _sign1(b)) * _min(np.abs(a), np.abs(b))
        alpha, beta = self.alpha, self.beta
        h0 = a3 - 2. * a2 + a1
        h1 = a2 - 2. * a1 + b0
        h2 = a1 - 2. * b0 + b1
        s2 = 4. * h1 - h2
        s0 = 4. * h2 - h1
        s1 = minmod(s2, s0)
        s2 = minmod(h1, h2)
        s0 = minmod(s1, s2)
        w2 = 4. * h0 - h1
        w0 = 4. * h1 - h0
        w1 = minmod(w2, w0)
        w2 = minmod(h0, h1)
        w0 = minmod(w1, w2)
        s1 = a1 + alpha * (a1 - a2)
        s2 = .5 * (a1 + b0 - s0)
        s0 = .5 * (3. * a1 - a2) + beta * w0 / 3.
        w1 = _min(_min(a1, b0), s2)
        w2 = _min(_min(a1, s1), s0)
        w0 = _max(w1, w2)
        h1 = _max(_max(a1, b0), s2)
        h2 = _max(_max(a1, s1), s0)
        h0 = _min(h1, h2)
        return w + minmod(w0 - w, h0 - w)  # median (1391-1403)

    def interp2(self, f, dirn, lens):
        """interp2_pdm / interp2_tvd (mhd3d3.f90:926-989, 1037-1067), edge family dirn = 1..3."""
        ng = self.ng
        if self.reconop in (2, 5):
            o = {1: [(0, -1, -1), (0, 0, -1), (0, 0, 0), (0, -1, 0)],
                 2: [(-1, 0, -1), (-1, 0, 0), (0, 0, 0), (0, 0, -1)],
                 3: [(-1, -1, 0), (0, -1, 0), (0, 0, 0), (-1, 0, 0)]}[dirn]
            a, b, c, e = (self._take(f, off, lens) for off in o)
            return (a + b + c + e) / 4.
        ii, jj, kk = lens
        if dirn == 1:  # along y over (nx0, ny0+1, nz), then along z
            g = _tap8(*[self._take(f, (0, m, 0), (ii, jj, 0), axes=(0, 1)) for m in range(-4, 4)])
            return _tap8(*[g[:, :, ng + m:ng + m + kk] for m in range(-4, 4)])
        if dirn == 2:  # along z over (nx, ny0, nz0+1), then along x
            g = _tap8(*[self._take(f, (0, 0, m), (0, jj, kk), axes=(1, 2)) for m in range(-4, 4)])
            return _tap8(*[g[ng + m:ng + m + ii, :, :] for m in range(-4, 4)])
        # along x over (nx0+1, ny, nz0), then along y
        g = _tap8(*[self._take(f, (m, 0, 0), (ii, 0, kk), axes=(0, 2)) for m in range(-4, 4)])
        return _tap8(*[g[:, ng + m:ng + m + jj, :] for m in range(-4, 4)])

    def _corner_weno(self, lv, dirn, lens):
        """The two-level WENO5 / MP-WENO5 corner states of get_vav_center2corner
        (mhd3d3.f90:1936-2049): reconstruct along the first transverse axis p
        (the other axes whole) into rows of a scratch array, reconstruct those
        along q; then the same with p and q exchanged."""
        p, q = {1: (1, 2), 2: (2, 0), 3: (0, 1)}[dirn]
        ng = self.ng
        vi = np.zeros((self.nx, self.ny, self.nz))  # only the rows written below are read

        def rows(axis, a):
            sl = [slice(None)] * 3
            sl[axis] = slice(ng, ng + a.shape[axis])
            vi[tuple(sl)] = a

        def first(axis):
            ln = [self.nx, self.ny, self.nz]
            ln[axis] = lens[axis]
            return self.reconstruct(lv, ln, axis, axes=(axis,))

        lvl, lvr = first(p)
        rows(p, lvl)
        v00_1, v01_1 = self.reconstruct(vi, lens, q)
        rows(p, lvr)
        v10_1, v11_1 = self.reconstruct(vi, lens, q)
        lvl, lvr = first(q)
        rows(q, lvl)
        v00_0, v01_0 = self.reconstruct(vi, lens, p)
        rows(q, lvr)
        v10_0, v11_0 = self.reconstruct(vi, lens, p)
        return v00_0, v00_1, v10_0, v10_1, v01_0, v01_1, v11_0, v11_1

    def vav_center2corner(self, lv, dirn, lens):
        """get_vav_center2corner (mhd3d3.f90:1858-2116)."""
        if self.reconop in (3, 4):
            v00_0, v00_1, v10_0, v10_1, v01_0, v01_1, v11_0, v11_1 = self._corner_weno(lv, dirn, lens)
        else:
            vi = self.interp2(lv, dirn, lens)
            # (shift, axis) of the four limited pairs, axis 0-based
            calls = {1: [((0, 0, -1), 1), ((0, -1, 0), 2), ((0, 0, 0), 2), ((0, 0, 0), 1)],
                     2: [((-1, 0, 0), 2), ((0, 0, -1), 0), ((0, 0, 0), 0), ((0, 0, 0), 2)],
                     3: [((0, -1, 0), 0), ((-1, 0, 0), 1), ((0, 0, 0), 1), ((0, 0, 0), 0)]}[dirn]
            v00_0, v10_0 = self.limit(lv, vi, lens, calls[0][1], calls[0][0])
            v00_1, v01_1 = self.limit(lv, vi, lens, calls[1][1], calls[1][0])
            v10_1, v11_1 = self.limit(lv, vi, lens, calls[2][1], calls[2][0])
            v01_0, v11_0 = self.limit(lv, vi, lens, calls[3][1], calls[3][0])
        T = lambda off: self._take(lv, off, lens)
        if dirn == 1:
            dif00 = np.abs(T((0, -2, -1)) - T((0, -1, -1))) - np.abs(T((0, -1, -2)) - T((0, -1, -1)))
            dif10 = np.abs(T((0, 1, -1)) - T((0, 0, -1))) - np.abs(T((0, 0, -2)) - T((0, 0, -1)))
            dif01 = np.abs(T((0, -2, 0)) - T((0, -1, 0))) - np.abs(T((0, -1, 1)) - T((0, -1, 0)))
            dif11 = np.abs(T((0, 1, 0)) - T((0, 0, 0))) - np.abs(T((0, 0, 1)) - T((0, 0, 0)))
        elif dirn == 2:
            dif00 = np.abs(T((-1, 0, -2)) - T((-1, 0, -1))) - np.abs(T((-2, 0, -1)) - T((-1, 0, -1)))
            dif10 = np.abs(T((-1, 0, 1)) - T((-1, 0, 0))) - np.abs(T((-2, 0, 0)) - T((-1, 0, 0)))
            dif01 = np.abs(T((0, 0, -2)) - T((0, 0, -1))) - np.abs(T((1, 0, -1)) - T((0, 0, -1)))
            dif11 = np.abs(T((0, 0, 1)) - T((0, 0, 0))) - np.abs(T((1, 0, 0)) - T((0, 0, 0)))
        else:
            dif00 = np.abs(T((-2, -1, 0)) - T((-1, -1, 0))) - np.abs(T((-1, -2, 0)) - T((-1, -1, 0)))
            dif10 = np.abs(T((1, -1, 0)) - T((0, -1, 0))) - np.abs(T((0, -2, 0)) - T((0, -1, 0)))
            dif01 = np.abs(T((-2, 0, 0)) - T((-1, 0, 0))) - np.abs(T((-1, 1, 0)) - T((-1, 0, 0)))
            dif11 = np.abs(T((1, 0, 0)) - T((0, 0, 0))) - np.abs(T((0, 1, 0)) - T((0, 0, 0)))
        dif00, dif10, dif01, dif11 = (_sign1(x) for x in (dif00, dif10, dif01, dif11))
        v00 = (1. + dif00) / 2. * v00_0 + (1. - dif00) / 2. * v00_1
        v10 = (1. + dif10) / 2. * v10_0 + (1. - dif10) / 2. * v10_1
        v01 = (1. + dif01) / 2. * v01_0 + (1. - dif01) / 2. * v01_1
        v11 = (1. + dif11) / 2. * v11_0 + (1. - dif11) / 2. * v11_1
        return .25 * (v00 + v01 + v10 + v11)

    # ------------------------------------------------------------- get_*
    def get_eijk_LFM(self, rho, vx, vy, vz, bx, by, bz, bi, bj, bk):
        """get_eijk_LFM (mhd3d3.f90:1754-1856) -> [ei, ej, ek]."""
        nx0, ny0, nz0 = self.nx0, self.ny0, self.nz0
        vf = np.sqrt(vx ** 2 + vy ** 2 + vz ** 2) + np.sqrt((bx ** 2 + by ** 2 + bz ** 2) / rho)
        out = []
        for kkk in (1, 2, 3):
            lens = [nx0 + 1, ny0 + 1, nz0 + 1]
            lens[kkk - 1] -= 1
            v1, v2, b1, b2, d1, d2 = {1: (vy, vz, bj, bk, 3, 2), 2: (vz, vx, bk, bi, 1, 3),
                                      3: (vx, vy, bi, bj, 2, 1)}[kkk]
            v1av = self.vav_center2corner(v1, kkk, lens)
            v2av = self.vav_center2corner(v2, kkk, lens)
            sig1, sig2 = _sign1(v1av), _sign1(v2av)
            b1l, b1r = self.reconstruct(b1, lens, d1 - 1)
            b2l, b2r = self.reconstruct(b2, lens, d2 - 1)
            b1u = (1. + sig2) / 2. * b1l + (1. - sig2) / 2. * b1r
            b2u = (1. + sig1) / 2. * b2l + (1. - sig1) / 2. * b2r
            dum = -v1av * b2u + v2av * b1u
            T = lambda off: self._take(vf, off, lens)
            o = {1: [(0, -1, -1), (0, 0, -1), (0, 0, 0), (0, -1, 0)],
                 2: [(-1, 0, -1), (-1, 0, 0), (0, 0, 0), (0, 0, -1)],
                 3: [(-1, -1, 0), (0, -1, 0), (0, 0, 0), (-1, 0, 0)]}[kkk]
            eta = .25 * (T(o[0]) + T(o[1]) + T(o[2]) + T(o[3]))
            out.append(dum + eta * (b1l + b2r - b1r - b2l))
        return out

    def get_eijk_Yee(self, rho, vx, vy, vz, p, bx, by, bz):
        """get_eijk_Yee (mhd3d3.f90:1654-1752) with get_v_center (2562-2592):
        split electric fields of the Gaussian velocity moments at the cell
        centres, reconstructed to the edges in two passes (left states of +
        moments, right states of - moments) and summed.  -> [ei, ej, ek]."""
        nx, ny, nz, ng = self.nx, self.ny, self.nz, self.ng
        nx0, ny0, nz0 = self.nx0, self.ny0, self.nz0
        bsq = bx ** 2 + by ** 2 + bz ** 2
        lam = rho / (2. * p + bsq)
        x0p, x0n, x1p, x1n = self.get_v_face(lam, vx)
        y0p, y0n, y1p, y1n = self.get_v_face(lam, vy)
        z0p, z0n, z1p, z1n = self.get_v_face(lam, vz)
        E = {  # [pp, np, pn, nn] per edge axis
            "z": [bx * x0p * y1p - by * x1p * y0p, bx * x0n * y1p - by * x1n * y0p,
                  bx * x0p * y1n - by * x1p * y0n, bx * x0n * y1n - by * x1n * y0n],
            "x": [by * y0p * z1p - bz * y1p * z0p, by * y0n * z1p - bz * y1n * z0p,
                  by * y0p * z1n - bz * y1p * z0n, by * y0n * z1n - bz * y1n * z0n],
            "y": [bz * z0p * x1p - bx * z1p * x0p, bz * z0n * x1p - bx * z1n * x0p,
                  bz * z0p * x1n - bx * z1p * x0n, bz * z0n * x1n - bx * z1n * x0n]}
        # (split fields, first axis and its extents, second axis and its extents, edge axis)
        plan = [("x", 1, (nx, ny0 + 1, nz), 2, (nx, ny0 + 1, nz0 + 1), 0, nx0),
                ("y", 2, (nx, ny, nz0 + 1), 0, (nx0 + 1, ny, nz0 + 1), 1, ny0),
                ("z", 0, (nx0 + 1, ny, nz), 1, (nx0 + 1, ny0 + 1, nz), 2, nz0)]
        out = []
        for key, d1, l1, d2, l2, ax, n0 in plan:
            pp, np_, pn, nn = E[key]
            qepp = self.reconstruct(pp, l1, d1, axes=(d1,))[0]
            qepn = self.reconstruct(pn, l1, d1, axes=(d1,))[0]
            qenn = self.reconstruct(nn, l1, d1, axes=(d1,))[1]
            qenp = self.reconstruct(np_, l1, d1, axes=(d1,))[1]
            epp = self.reconstruct(qepp, l2, d2, axes=(d2,))[0]
            enp = self.reconstruct(qenp, l2, d2, axes=(d2,))[0]
            enn = self.reconstruct(qenn, l2, d2, axes=(d2,))[1]
            epn = self.reconstruct(qepn, l2, d2, axes=(d2,))[1]
            sl = [slice(None)] * 3
            sl[ax] = slice(ng, ng + n0)
            sl = tuple(sl)
            out.append(epp[sl] + enp[sl] + epn[sl] + enn[sl])
        return out

    def get_eijk(self, rho, vx, vy, vz, p, bx, by, bz, bi, bj, bk):
        if self.emf_kind == 1:
            return self.get_eijk_Yee(rho, vx, vy, vz, p, bx, by, bz)
        return self.get_eijk_LFM(rho, vx, vy, vz, bx, by, bz, bi, bj, bk)

    def get_v_face(self, llam, lv):
        """get_v_face (mhd3d3.f90:2594-2615)."""
        a = np.sqrt(llam)
        b = .5 * np.exp(-llam * lv ** 2) / a / np.sqrt(self.pi)
        v0p = .5 * erfc(-a * lv)
        v0n = .5 * erfc(a * lv)
        return v0p, v0n, lv * v0p + b, lv * v0n - b

    def get_flux_stress(self, rho, vx, vy, vz, p, bx, by, bz):
        """get_flux_stress (mhd3d3.f90:2385-2560) -> per axis [rho, rvx, rvy, rvz, eng,
        stress x, y, z] fluxes."""
        gam = self.gam
        out = []
        for kkk in (1, 2, 3):
            lens = [self.nx0, self.ny0, self.nz0]
            lens[kkk - 1] += 1
            d = kkk - 1
            (rhol, rhor), (vxl, vxr), (vyl, vyr), (vzl, vzr), (pl, pr), (bxl, bxr), (byl, byr), (bzl, bzr) = (
                self.reconstruct(f, lens, d) for f in (rho, vx, vy, vz, p, bx, by, bz))
            # left flux
            leng = .5 * rhol * (vxl ** 2 + vyl ** 2 + vzl ** 2) + pl / (gam - 1.)
            llam = rhol / (2. * pl)
            vn = (vxl, vyl, vzl)[d]
            v0p, v0n, v1p, v1n = self.get_v_face(llam, vn)
            rp = rhol * v1p
            rvp = [rhol * vxl * v1p, rhol * vyl * v1p, rhol * vzl * v1p]
            ep = (leng + .5 * pl) * v1p
            rvp[d] = rvp[d] + pl * v0p
            ep = ep + .5 * pl * vn * v0p
            lbsq = bxl ** 2 + byl ** 2 + bzl ** 2
            llam = rhol / (2. * pl + lbsq)
            v0p, v0n, v1p, v1n = self.get_v_face(llam, vn)
            bl = (bxl, byl, bzl)
            sp = [(-(bl[c] * bl[d])) * v0p for c in range(3)]
            sp[d] = (.5 * lbsq - bl[d] * bl[d]) * v0p
            # right flux
            leng = .5 * rhor * (vxr ** 2 + vyr ** 2 + vzr ** 2) + pr / (gam - 1.)
            llam = rhor / (2. * pr)
            vn = (vxr, vyr, vzr)[d]
            v0p, v0n, v1p, v1n = self.get_v_face(llam, vn)
            rn = rhor * v1n
            rvn = [rhor * vxr * v1n, rhor * vyr * v1n, rhor * vzr * v1n]
            en = (leng + .5 * pr) * v1n
            rvn[d] = rvn[d] + pr * v0n
            en = en + .5 * pr * vn * v0n
            lbsq = bxr ** 2 + byr ** 2 + bzr ** 2
            llam = rhor / (2. * pr + lbsq)
            v0p, v0n, v1p, v1n = self.get_v_face(llam, vn)
            br = (bxr, byr, bzr)
            sn = [(-(br[c] * br[d])) * v0n for c in range(3)]
            sn[d] = (.5 * lbsq - br[d] * br[d]) * v0n
            out.append([rp + rn, rvp[0] + rvn[0], rvp[1] + rvn[1], rvp[2] + rvn[2], ep + en,
                        sp[0] + sn[0], sp[1] + sn[1], sp[2] + sn[2]])
        return out

    def get_bxyz(self):
        """get_bxyz (mhd3d3.f90:2118-2128)."""
        self.bx = .5 * (self.bi[1:] + self.bi[:-1])
        self.by = .5 * (self.bj[:, 1:] + self.bj[:, :-1])
        self.bz = .5 * (self.bk[:, :, 1:] + self.bk[:, :, :-1])

    # -------------------------------------------------------------- fills
    def _fill(self, a, axis, face, sgn=1.0):
        """fillx_center / fillx_face of one rank (mhd3d3.f90:346-390, 482-525):
        the periodic exchange (kind 0), or the mirror at both walls (kind 1,
        even; kind 2, with sgn = -1 for the normal velocity, the xbc = 1 that
        mhd3d2's fill_hydro_mpi passes for vx in x and vy in y,
        mhd3d2.f90:713, 720), or the zero-gradient copy of the boundary cell or
        face (kind 3, outflow; no reference counterpart)."""
        a = np.moveaxis(a, axis, 0)  # a view: writes land in the array
        n, ng, nord = a.shape[0], self.ng, self.nord
        n0 = n - nord - (1 if face else 0)
        i = np.arange(1, ng + 1)  # Fortran i = 1..ng
        kind = self.bc[axis]
        if kind == 3:
            last = ng + n0 if face else ng + n0 - 1  # the last interior face / cell
            a[0:ng] = a[ng]
            a[n - ng:n] = a[last]
            return
        if kind in (1, 2):
            if face:  # aa(i)=aa(nord+2-i); aa(n+2-i)=aa(n0+i), n = lnx-1, n0 = n-nord
                a[i - 1] = sgn * a[nord + 2 - i - 1]
                a[n + 1 - i - 1] = sgn * a[n - 1 - nord + i - 1]
            else:  # aa(i)=aa(nord+1-i); aa(lnx+1-i)=aa(lnx-nord+i)
                a[i - 1] = sgn * a[nord + 1 - i - 1]
                a[n + 1 - i - 1] = sgn * a[n - nord + i - 1]
            return
        if face:
            a[0:ng] = a[n - nord - 1:n - ng - 1]   # aa(1:ng)=aa(lnx-nord:lnx-ng-1)
            a[n - ng:n] = a[ng + 1:nord + 1]      # aa(lnx-ng+1:lnx)=aa(ng+2:nord+1)
        else:
            a[0:ng] = a[n - nord:n - ng]           # aa(1:ng)=aa(lnx-nord+1:lnx-ng)
            a[n - ng:n] = a[ng:nord]               # aa(lnx-ng+1:lnx)=aa(ng+1:nord)

    def fill_hydro(self):
        for ax in range(3):
            for a, normal in ((self.rho, None), (self.p, None), (self.vx, 0), (self.vy, 1), (self.vz, 2)):
                sgn = -1.0 if (self.bc[ax] == 2 and normal == ax) else 1.0
                self._fill(a, ax, False, sgn)

    def fill_mag(self):
        for ax in range(3):
            for c, a in enumerate((self.bi, self.bj, self.bk)):
                self._fill(a, ax, c == ax)

    # -------------------------------------------------------------- steps
    def _div(self, fl):
        """The flux divergence of advance_corrector1/2 over the interior cells."""
        fx, fy, fz = fl
        return ((fx[1:] - fx[:-1]) / self.dx + (fy[:, 1:] - fy[:, :-1]) / self.dy
                + (fz[:, :, 1:] - fz[:, :, :-1]) / self.dz)

    def get_dt(self):
        """get_dt (mhd3d3.f90:1608-1639): the CFL dt, minimum over every cell."""
        v = np.sqrt(self.vx ** 2 + self.vy ** 2 + self.vz ** 2)
        btot = np.sqrt(self.bx ** 2 + self.by ** 2 + self.bz ** 2)
        valf = btot / np.sqrt(self.rho)
        vs = np.sqrt(self.gam * self.p / self.rho)
        vcfl = v + np.sqrt(valf ** 2 + vs ** 2)
        return (self.cfl / (vcfl / self.dxa + vcfl / self.dya + vcfl / self.dza)).min()

    def step_ab(self):
        """step_ab (mhd3d3.f90:3602-3644) with advance_predictor_ab (3821-3834)."""
        gam, ng = self.gam, self.ng
        I = (slice(ng, ng + self.nx0), slice(ng, ng + self.ny0), slice(ng, ng + self.nz0))
        self.tau = tau = self.get_dt()
        rho, vx, vy, vz, p = self.rho, self.vx, self.vy, self.vz, self.p
        rho0 = rho.copy()
        rhovx0, rhovy0, rhovz0 = rho * vx, rho * vy, rho * vz
        eng0 = .5 * rho * (vx ** 2 + vy ** 2 + vz ** 2) + p / (gam - 1.)
        c = tau / self.tau0 / 2.
        h = {k: getattr(self, k) + c * (getattr(self, k) - getattr(self, k + "p"))
             for k in ("rho", "vx", "vy", "vz", "p", "bx", "by", "bz", "bi", "bj", "bk")}
        for k in ("rho", "vx", "vy", "vz", "p", "bx", "by", "bz", "bi", "bj", "bk"):  # advance_previous
            setattr(self, k + "p", getattr(self, k).copy())
        self.tau0 = tau
        ei, ej, ek = self.get_eijk(h["rho"], h["vx"], h["vy"], h["vz"], h["p"], h["bx"], h["by"], h["bz"],
                                   h["bi"], h["bj"], h["bk"])
        fl = self.get_flux_stress(h["rho"], h["vx"], h["vy"], h["vz"], h["p"], h["bx"], h["by"], h["bz"])
        # advance_corrector1, stepop = 1
        rho, eng = rho0.copy(), eng0.copy()
        rhovx, rhovy, rhovz = rhovx0.copy(), rhovy0.copy(), rhovz0.copy()
        rho[I] = rho0[I] - tau * self._div([fl[a][0] for a in range(3)])
        eng[I] = eng0[I] - tau * self._div([fl[a][4] for a in range(3)])
        rhovx[I] = rhovx0[I] - tau * self._div([fl[a][1] for a in range(3)])
        rhovy[I] = rhovy0[I] - tau * self._div([fl[a][2] for a in range(3)])
        rhovz[I] = rhovz0[I] - tau * self._div([fl[a][3] for a in range(3)])
        self.p = (gam - 1.) * (eng - .5 * (rhovx ** 2 + rhovy ** 2 + rhovz ** 2) / rho)
        # advance_corrector2, stepop = 1
        rhovx[I] = rhovx[I] - tau * self._div([fl[a][5] for a in range(3)])
        rhovy[I] = rhovy[I] - tau * self._div([fl[a][6] for a in range(3)])
        rhovz[I] = rhovz[I] - tau * self._div([fl[a][7] for a in range(3)])
        self.rho = rho
        self.vx, self.vy, self.vz = rhovx / rho, rhovy / rho, rhovz / rho
        self._advance_bijk(ei, ej, ek, tau)
        self.fill_hydro()
        self.fill_mag()
        self.get_bxyz()

    def _advance_bijk(self, ei, ej, ek, tau):
        """advance_bijk (mhd3d3.f90:3893-3912) into new arrays."""
        ng, nx0, ny0, nz0 = self.ng, self.nx0, self.ny0, self.nz0
        I = (slice(ng, ng + nx0), slice(ng, ng + ny0), slice(ng, ng + nz0))
        bi, bj, bk = self.bi.copy(), self.bj.copy(), self.bk.copy()
        bi[ng:ng + nx0 + 1, I[1], I[2]] -= tau * ((ek[:, 1:] - ek[:, :-1]) / self.dy
                                                  - (ej[:, :, 1:] - ej[:, :, :-1]) / self.dz)
        bj[I[0], ng:ng + ny0 + 1, I[2]] -= tau * ((ei[:, :, 1:] - ei[:, :, :-1]) / self.dz
                                                  - (ek[1:] - ek[:-1]) / self.dx)
        bk[I[0], I[1], ng:ng + nz0 + 1] -= tau * ((ej[1:] - ej[:-1]) / self.dx
                                                  - (ei[:, 1:] - ei[:, :-1]) / self.dy)
        self.bi, self.bj, self.bk = bi, bj, bk

    def _comb(self, xp, x, stage):
        """The stage combinations of step_rk2 / step_rk3 (3646-3792)."""
        if self.stepop == 2:
            return (xp + x) / 2.
        if stage == 2:
            return (3. * xp + x) / 4.
        return (xp + 2. * x) / 3.

    def step(self):
        """step_ab, or step_rk2 / step_rk3 (mhd3d3.f90:3646-3792) with the deck's fixed tau."""
        if self.stepop == 1:
            return self.step_ab()
        gam, ng = self.gam, self.ng
        I = (slice(ng, ng + self.nx0), slice(ng, ng + self.ny0), slice(ng, ng + self.nz0))
        if self.dt_mode == 1:
            self.tau0 = self.get_dt()
        self.tau = self.tau0
        tau = self.tau
        # advance_previous (3794-3819), stepop = 2
        rhop, bip, bjp, bkp = self.rho.copy(), self.bi.copy(), self.bj.copy(), self.bk.copy()
        rho, vx, vy, vz, p = self.rho, self.vx, self.vy, self.vz, self.p
        rhovxp, rhovyp, rhovzp = rho * vx, rho * vy, rho * vz
        engp = .5 * rho * (vx ** 2 + vy ** 2 + vz ** 2) + p / (gam - 1.)
        for rk_step in range(1, self.stepop + 1):
            rho, vx, vy, vz, p = self.rho, self.vx, self.vy, self.vz, self.p
            # get_conserve (1641-1650)
            rho0 = rho.copy()
            rhovx0, rhovy0, rhovz0 = rho * vx, rho * vy, rho * vz
            eng0 = .5 * rho * (vx ** 2 + vy ** 2 + vz ** 2) + p / (gam - 1.)
            ei, ej, ek = self.get_eijk(rho, vx, vy, vz, p, self.bx, self.by, self.bz, self.bi, self.bj, self.bk)
            fl = self.get_flux_stress(rho, vx, vy, vz, p, self.bx, self.by, self.bz)
            # advance_corrector1 (3836-3866)
            rho, eng = rho0.copy(), eng0.copy()
            rhovx, rhovy, rhovz = rhovx0.copy(), rhovy0.copy(), rhovz0.copy()
            rho[I] = rho0[I] - tau * self._div([fl[a][0] for a in range(3)])
            eng[I] = eng0[I] - tau * self._div([fl[a][4] for a in range(3)])
            rhovx[I] = rhovx0[I] - tau * self._div([fl[a][1] for a in range(3)])
            rhovy[I] = rhovy0[I] - tau * self._div([fl[a][2] for a in range(3)])
            rhovz[I] = rhovz0[I] - tau * self._div([fl[a][3] for a in range(3)])
            if rk_step == 1:
                rhovxh, rhovyh, rhovzh = rhovx, rhovy, rhovz
            else:
                rho = self._comb(rhop, rho, rk_step)
                rhovxh = self._comb(rhovxp, rhovx, rk_step)
                rhovyh = self._comb(rhovyp, rhovy, rk_step)
                rhovzh = self._comb(rhovzp, rhovz, rk_step)
                eng = self._comb(engp, eng, rk_step)
            p = (gam - 1.) * (eng - .5 * (rhovxh ** 2 + rhovyh ** 2 + rhovzh ** 2) / rho)
            # advance_corrector2 (3868-3891)
            rhovx = rhovx.copy(); rhovy = rhovy.copy(); rhovz = rhovz.copy()
            rhovx[I] = rhovx[I] - tau * self._div([fl[a][5] for a in range(3)])
            rhovy[I] = rhovy[I] - tau * self._div([fl[a][6] for a in range(3)])
            rhovz[I] = rhovz[I] - tau * self._div([fl[a][7] for a in range(3)])
            if rk_step >= 2:
                rhovx = self._comb(rhovxp, rhovx, rk_step)
                rhovy = self._comb(rhovyp, rhovy, rk_step)
                rhovz = self._comb(rhovzp, rhovz, rk_step)
            self.rho, self.p = rho, p
            self.vx, self.vy, self.vz = rhovx / rho, rhovy / rho, rhovz / rho
            self._advance_bijk(ei, ej, ek, tau)
            bi, bj, bk = self.bi, self.bj, self.bk
            if rk_step >= 2:
                bi, bj, bk = self._comb(bip, bi, rk_step), self._comb(bjp, bj, rk_step), self._comb(bkp, bk, rk_step)
            self.bi, self.bj, self.bk = bi, bj, bk
            self.fill_hydro()
            self.fill_mag()
            self.get_bxyz()

    def diagnostics(self) -> dict:
        """Total mass and energy (plasma + magnetic) of the interior cells as
        exactly rounded sums (math.fsum), max |div B| of the face fields, min
        rho over every cell and the CFL dt (N4; no reference counterpart)."""
        ng, gam = self.ng, self.gam
        nx0, ny0, nz0 = self.nx0, self.ny0, self.nz0
        I = (slice(ng, ng + nx0), slice(ng, ng + ny0), slice(ng, ng + nz0))
        dv = self.dx * self.dy * self.dz
        r, u, v, w, p = self.rho[I], self.vx[I], self.vy[I], self.vz[I], self.p[I]
        a, b, c = self.bx[I], self.by[I], self.bz[I]
        e = .5 * r * (u * u + v * v + w * w) + p / (gam - 1.) + .5 * (a * a + b * b + c * c)
        bi = self.bi[ng:ng + nx0 + 1, I[1], I[2]]
        bj = self.bj[I[0], ng:ng + ny0 + 1, I[2]]
        bk = self.bk[I[0], I[1], ng:ng + nz0 + 1]
        divb = (bi[1:] - bi[:-1]) / self.dx + (bj[:, 1:] - bj[:, :-1]) / self.dy + (bk[:, :, 1:] - bk[:, :, :-1]) / self.dz
        return {"mass": math.fsum((r * dv).ravel()), "energy": math.fsum((e * dv).ravel()),
                "divb_max": float(np.abs(divb).max()), "rho_min": float(self.rho.min()), "dt_cfl": self.get_dt()}

    def fluxes(self):
        return self.get_flux_stress(self.rho, self.vx, self.vy, self.vz, self.p, self.bx, self.by, self.bz)

    def emf(self):
        return self.get_eijk(self.rho, self.vx, self.vy, self.vz, self.p, self.bx, self.by, self.bz,
                             self.bi, self.bj, self.bk)

    def state(self) -> dict:
        return {"rho": self.rho, "vx": self.vx, "vy": self.vy, "vz": self.vz, "p": self.p, "bx": self.bx,
                "by": self.by, "bz": self.bz, "bi": self.bi, "bj": self.bj, "bk": self.bk}
