"""Generate the small golden fixtures in tests/golden/ from the oracle.

The reference ships no golden vectors (no tests, no fixtures) and cannot be
compiled here, so these fixtures are regression pins of the oracle itself:
interior fields after a few steps for every reconop / stepop / boundary kind
on tiny grids, plus the 1-D Brio-Wu-type tube profile.  Run:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from mhd3d_mpi_fortran_gb300 import ics  # noqa: E402
from mhd3d_mpi_fortran_gb300.abi import Params  # noqa: E402

FIELDS = ("rho", "vx", "vy", "vz", "p", "bi", "bj", "bk")


def cases():
    out = []
    for recon in (1, 2, 3, 4, 5):
        out.append((f"ot3d_r{recon}_rk2", "ot", dict(reconop=recon, stepop=2), 3))
    out.append(("ot3d_r1_ab2", "ot", dict(reconop=1, stepop=1), 3))
    out.append(("ot3d_r4_rk3", "ot", dict(reconop=4, stepop=3), 3))
    out.append(("ot3d_r2_rk2_shift", "ot", dict(reconop=2, stepop=2, tvd_shift=1), 3))
    for kind in (1, 2, 3):
        out.append((f"blast_bc{kind}", "blast", dict(reconop=1, stepop=2, bc=(kind,) * 3), 3))
    out.append(("tube_z", "tube", dict(reconop=1, stepop=2, bc=(1, 1, 1)), 20))
    return out


def state_of(kind):
    if kind == "ot":
        return ics.orszag_tang_3d(8, seed=7)
    if kind == "blast":
        return ics.blast(8, r0=0.3)
    return ics.shock_tube(48, axis=2, ntrans=4)


def run(name, kind, kw, steps):
    from oracle.oracle import OracleSolver
    s = state_of(kind)
    g = s.grid
    tau = 2e-3 if kind == "tube" else 0.5 * ics.cfl_dt(s)
    prm = Params(g.nx0, g.ny0, g.nz0, tau=tau, **kw)
    o = OracleSolver(prm, s)
    o.step(steps)
    f = o.fetch()
    ng = g.ng
    if kind == "tube":
        return {k: f[k][ng + 1, ng + 1, ng:ng + g.nz0].copy() for k in ("rho", "p", "vz", "bx")}
    sl = lambda a, e: a[ng:ng + g.nx0 + e[0], ng:ng + g.ny0 + e[1], ng:ng + g.nz0 + e[2]].copy()
    ext = {"bi": (1, 0, 0), "bj": (0, 1, 0), "bk": (0, 0, 1)}
    return {k: sl(f[k], ext.get(k, (0, 0, 0))) for k in FIELDS}


def main():
    for name, kind, kw, steps in cases():
        np.savez_compressed(HERE / f"{name}.npz", **run(name, kind, kw, steps))
        print("wrote", name)


if __name__ == "__main__":
    main()
