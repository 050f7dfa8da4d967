"""The reference's driver loop on the GPU solver: deck -> initial state ->
nframes x nts steps -> one output frame per nts steps -> the reference's stop
checks (``program mhd3d``, mhd3d3.f90:3165-3323).

Differences from the Fortran driver, all forced by this environment:

* Frames are raw FP64 files, one per variable, in the layout of the
  reference's HDF5 dataset (``outh5_3D``: dataset dims (nx0G, ny0G, nz0G,
  nframes+1) in Fortran order, i.e. C order [frame][z][y][x]), with a JSON
  sidecar naming the shape and the time of each frame.  Neither libhdf5 nor
  h5py exists here; a reader of the HDF5 files reads the same arrays from
  these files with ``numpy.fromfile(...).reshape(shape)``.
* ``stime.out`` (``output_simt``, mhd3d2.f90:2969-2986) is written as a
  Fortran unformatted sequential file: one record per frame holding the FP64
  time, each record framed by 4-byte length markers (gfortran and ifort
  default).
* ``diag_rho_neg`` / ``diag_overflow`` (mhd3d3.f90:3137-3160) stop the run;
  here the device status bits of each frame's steps raise ``RunStopped``
  after the frame that saw them has been written, as the reference stops
  after ``outputxyz``.

Usage: ``python -m mhd3d_mpi_fortran_gb300.driver mhd3d3.in outdir [--fp32] [--periodic] [--ic tube|otv|bws|imp]``.
"""
from __future__ import annotations

import json
import struct
import sys
from pathlib import Path

import numpy as np

from . import ics
from .abi import ST_NAN, ST_NEG_RHO, BC_PERIODIC, BC_OUTFLOW, FP32, FP64
from .deck import read_deck, params_from_deck, domain_from_deck
from .solver import MHDSolver

VARS = ("rho", "vx", "vy", "vz", "p", "bx", "by", "bz")


class RunStopped(RuntimeError):
    """diag_rho_neg / diag_overflow would have stopped the reference here."""


# The initial conditions a deck can start from: mhd3d3's init_ic and the
# three of mhd3d2 (its program calls init_ic_otv, mhd3d2.f90:3186-3188).
ICS = ("tube", "otv", "bws", "imp")
Z2D = 8  # z planes of a 2-D run: the smallest axis the solver's tests run


def ic_grid(deck: dict, nord: int, ic: str = "tube") -> tuple:
    """(nx0, ny0, nz0, bc) of the run.  mhd3d2's ICs are 2-D: its deck has
    nz0 = 1 and fills z with copies of the one plane (fillz_even1,
    mhd3d2.f90:687-697, 731-772).  Here z gets at least Z2D planes with the
    outflow fill, which is the same copy, so every plane evolves identically;
    x, y keep mhd3d2's periodic topology (mhd3d2.f90:3063-3064)."""
    grid = deck.get("grid", {})
    nx, ny, nz = (int(grid.get(k + "0g", grid.get(k + "0", 1))) for k in ("nx", "ny", "nz"))
    if ic == "tube":
        return nx, ny, nz, None
    if ic not in ICS:
        raise ValueError(f"ic must be one of {ICS}")
    return nx, ny, max(nz, Z2D, nord // 2), (BC_PERIODIC, BC_PERIODIC, BC_OUTFLOW)


def initial_state(deck: dict, nord: int, ic: str = "tube") -> ics.State:
    """The deck's initial state.  tube: init_ic of mhd3d3 (mhd3d3.f90:3517-3583),
    the shock tube along z on the deck's domain (x and y sizes equal, the
    tube's transverse extent).  otv / bws / imp: init_ic_otv / init_ic_bws /
    init_ic_imp of mhd3d2 (mhd3d2.f90:3358-3471) on the deck's x-y grid."""
    nx, ny, nz, _ = ic_grid(deck, nord, ic)
    lo, hi = domain_from_deck(deck)
    if nx != ny:
        raise ValueError(f"the {ic} initial condition needs nx0G == ny0G")
    if ic == "tube":
        if lo != (-1.0, -1.0, -1.0) or hi != (1.0, 1.0, 1.0):
            raise ValueError("init_ic's tube is set up on the deck domain [-1, 1]^3")
        return ics.shock_tube(nz, axis=2, nord=nord, ntrans=nx)
    if ic == "bws":
        return ics.blast_bws(nx, nz0=nz, nord=nord, lo=lo, hi=hi)
    if lo != (0.0, 0.0, 0.0) or hi != (1.0, 1.0, 1.0):
        raise ValueError(f"the {ic} initial condition is set up on the unit box (mhd3d2.in dom)")
    return ics.orszag_tang_2d(nx, nz0=nz, nord=nord) if ic == "otv" else ics.implosion(nx, nz0=nz, nord=nord)


class FrameWriter:
    """Frames of the 8 output variables (interior cells) and stime.out."""

    def __init__(self, outdir: Path, shape_xyz: tuple, nframes: int, ng: int):
        self.out = Path(outdir)
        self.out.mkdir(parents=True, exist_ok=True)
        self.ng = ng
        nx, ny, nz = shape_xyz
        self.shape = (nframes + 1, nz, ny, nx)
        self.files = {v: open(self.out / f"{v}.f64", "wb") for v in VARS}
        self.times = []
        (self.out / "stime.out").write_bytes(b"")

    def write(self, fields: dict, time: float):
        g = self.ng
        for v in VARS:
            a = fields[v][g:-g, g:-g, g:-g]  # Fortran (x, y, z) interior
            # C order [z][y][x] of the Fortran (x, y, z) array = its transpose
            self.files[v].write(np.ascontiguousarray(a.transpose(2, 1, 0), dtype=np.float64).tobytes())
            self.files[v].flush()
        with open(self.out / "stime.out", "ab") as f:
            f.write(fortran_record(struct.pack("<d", time)))
        self.times.append(time)

    def close(self, frames_written: int):
        for fh in self.files.values():
            fh.close()
        shape = (frames_written,) + self.shape[1:]
        (self.out / "frames.json").write_text(json.dumps({
            "variables": list(VARS), "dtype": "float64", "order": "C",
            "shape": shape, "layout": "[frame][z][y][x] (the reference's HDF5 dataset dims in C order)",
            "time": self.times}, indent=1))


def fortran_record(payload: bytes) -> bytes:
    """One Fortran unformatted sequential record (4-byte length markers)."""
    n = struct.pack("<i", len(payload))
    return n + payload + n


def read_frames(outdir) -> dict:
    """The frames written by ``run``: {var: array [frame][z][y][x]}, plus 'time'."""
    meta = json.loads((Path(outdir) / "frames.json").read_text())
    out = {v: np.fromfile(Path(outdir) / f"{v}.f64", dtype=np.float64).reshape(meta["shape"]) for v in meta["variables"]}
    out["time"] = np.asarray(meta["time"])
    return out


def read_stime(path) -> np.ndarray:
    """Times recorded in a Fortran unformatted stime.out."""
    raw = Path(path).read_bytes()
    out, i = [], 0
    while i < len(raw):
        (n,) = struct.unpack_from("<i", raw, i)
        out.append(struct.unpack_from("<d", raw, i + 4)[0])
        i += 8 + n
    return np.asarray(out)


def run(deck, outdir, precision: int = FP64, periodic: bool = False, state: ics.State | None = None,
        nframes: int | None = None, nts: int | None = None, ic: str = "tube") -> dict:
    """Run the deck: frame 0 is the initial state, then nframes frames of nts
    steps each (the deck's values unless given).  Returns a summary dict."""
    deck = read_deck(deck) if not isinstance(deck, dict) else deck
    lst = deck.get("list", {})
    nframes = int(lst.get("nframes", 1)) if nframes is None else nframes
    nts = int(lst.get("nts", 1)) if nts is None else nts
    prm = params_from_deck(deck, precision=precision, bc=BC_PERIODIC if periodic else None)
    if ic != "tube" and state is None:
        _, _, nz0, bc = ic_grid(deck, prm.nord, ic)
        prm.nz0, prm.bc = nz0, bc
    st0 = state if state is not None else initial_state(deck, prm.nord, ic)
    ng = prm.nord // 2
    w = FrameWriter(outdir, (prm.nx0, prm.ny0, prm.nz0), nframes, ng)
    time = 0.0
    frames = 0
    stopped = None
    with MHDSolver(prm, st0) as s:
        w.write(s.fetch(), time)  # outputxyz before the loop (mhd3d3.f90:3270)
        frames = 1
        tau = prm.tau  # the module tau before the first step (the deck's)
        for ntt in range(1, nframes + 1):
            status = 0
            for _ in range(nts):
                time += tau  # time = time + tau, then call step (mhd3d3.f90:3285-3286)
                tau, st = s.step(1)  # the step leaves the module tau (AB: its CFL dt)
                status |= st
            w.write(s.fetch(), time)
            frames += 1
            if status & ST_NEG_RHO:
                stopped = f"negative density in frame {ntt} (diag_rho_neg)"
            elif status & ST_NAN:
                stopped = f"NaN in frame {ntt} (diag_overflow)"
            if stopped:
                break
    w.close(frames)
    summary = {"frames": frames, "time": time, "stopped": stopped, "outdir": str(outdir)}
    if stopped:
        raise RunStopped(stopped)
    return summary


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("deck")
    ap.add_argument("outdir")
    ap.add_argument("--fp32", action="store_true")
    ap.add_argument("--periodic", action="store_true")
    ap.add_argument("--ic", choices=ICS, default="tube",
                    help="tube: mhd3d3's init_ic; otv / bws / imp: mhd3d2's (2-D, periodic x-y)")
    a = ap.parse_args(argv)
    print(json.dumps(run(a.deck, a.outdir, precision=FP32 if a.fp32 else FP64, periodic=a.periodic, ic=a.ic)))


if __name__ == "__main__":
    main(sys.argv[1:])
