"""Reader for the reference's namelist deck (mhd3d3.in / mhd3d2.in).

Mirrors ``read_input`` (mhd3d3.f90:147-197): namelists ``dom``, ``grid``,
``comset``, ``list`` and ``free``.  With ``-r8`` every real is FP64
(makefile:19).  ``params_from_deck`` turns a deck into the ``Params`` block of
``mhd_init`` for a single-GPU run (one domain: nx0 = nx0G etc., the role of
``comp_pars``, mhd3d3.f90:199-220, with xprocs=yprocs=zprocs=1).
"""
from __future__ import annotations

import re
from pathlib import Path

from .abi import Params, BC_EVEN, BC_PERIODIC

_GROUP = re.compile(r"&(\w+)(.*?)/", re.S)
_PAIR = re.compile(r"(\w+)\s*=\s*([^,\n]+)")


def _value(tok: str):
    t = tok.strip().rstrip(",")
    low = t.lower()
    if low in (".true.", "t", ".t."):
        return True
    if low in (".false.", "f", ".f."):
        return False
    if t.startswith(("'", '"')):
        return t.strip("'\"")
    try:
        return int(t)
    except ValueError:
        return float(low.replace("d", "e"))


def read_deck(path_or_text: str | Path) -> dict:
    """Parse a namelist deck into {group: {name: value}} (names lower-case)."""
    p = Path(path_or_text) if not str(path_or_text).lstrip().startswith("&") else None
    text = p.read_text() if p is not None else str(path_or_text)
    out: dict = {}
    for g, body in _GROUP.findall(text):
        out[g.lower()] = {k.lower(): _value(v) for k, v in _PAIR.findall(body)}
    return out


def params_from_deck(deck: dict, precision: int = 0, bc=None, dt_mode: int = 0,
                     tvd_shift: int = 0) -> Params:
    """Deck -> Params for one GPU.  ``bc`` defaults to mhd3d3's even walls
    (fill_hydro_mpi with bc=0, mhd3d3.f90:781-819); pass BC_PERIODIC for the
    mhd3d2 periodic topology."""
    grid = deck.get("grid", {})
    com = deck.get("comset", {})
    lst = deck.get("list", {})
    free = deck.get("free", {})
    nx0 = int(grid.get("nx0g", grid.get("nx0", 1)))
    ny0 = int(grid.get("ny0g", grid.get("ny0", 1)))
    nz0 = int(grid.get("nz0g", grid.get("nz0", 1)))
    if bc is None:
        bc = (BC_EVEN, BC_EVEN, BC_EVEN)
    elif isinstance(bc, int):
        bc = (bc, bc, bc)
    return Params(
        nx0=nx0, ny0=ny0, nz0=nz0,
        nord=int(com.get("nord", 8)), reconop=int(com.get("reconop", 1)),
        stepop=int(com.get("stepop", 2)), bc=tuple(bc), precision=precision,
        dt_mode=dt_mode, tvd_shift=tvd_shift,
        cfl=float(free.get("cfl", 0.3)), pdmb=float(free.get("pdmb", 4.0)),
        eps=float(free.get("eps", 1e-8)), alpha=float(free.get("alpha", 2.0)),
        beta=float(free.get("beta", 4.0)), tau=float(lst.get("tau", 2e-4)),
    )


def domain_from_deck(deck: dict) -> tuple:
    d = deck.get("dom", {})
    lo = (float(d.get("xmin", 0.0)), float(d.get("ymin", 0.0)), float(d.get("zmin", 0.0)))
    hi = (float(d.get("xmax", 1.0)), float(d.get("ymax", 1.0)), float(d.get("zmax", 1.0)))
    return lo, hi


__all__ = ["read_deck", "params_from_deck", "domain_from_deck", "BC_PERIODIC", "BC_EVEN"]
