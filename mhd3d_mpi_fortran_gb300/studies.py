"""Accuracy studies of the FP32 production path against the all-FP64 mode.

The all-FP64 mode reproduces the oracle (the CPU restatement of the
reference's step) to round-off on identical inputs, so it is the reference
solution here at sizes the oracle cannot reach in reasonable time.

* ``curvilinear`` -- magnetised blast on the mapped grid
  x = xi + 0.05 sin 2 pi eta, y = eta + 0.05 sin 2 pi zeta, z = zeta; outflow
  walls, PDM, AB2 (CFL dt); FP32 and FP64 side by side: L1/L2 error of FP32,
  div B of both, GPU time and zone-updates/s of both.
* ``precision``   -- decaying turbulence on the periodic box (rho = 1,
  p = 1/(gam Ms^2), Ms = 0.5, solenoidal k^-2 v and B); PDM, TVD-MC and WENO5
  with RK2; L1/L2 and shell-averaged energy-spectrum error of FP32 against
  FP64, GPU time of both.
* ``equal_time``  -- error against the FP64 n^3 solve at comparable GPU time:
  FP32 at n^3 and (n/2)^3, FP64 at (n/2)^3 and (n/4)^3, same physical time.
* ``learned``     -- the learned coarse-grid correction: training pairs from
  fine (2N)^3 turbulence runs, outputs calibrated on a validation seed, then
  held-out seeds: relative L1 error of the plain and the corrected N^3 runs
  against the restricted fine run, and the wall time of all three.

``python -m mhd3d_mpi_fortran_gb300.studies curvilinear|precision|equal_time|learned [--n N] [--steps K]``
prints one JSON line per case.
"""
from __future__ import annotations

import json
import sys

import numpy as np

from . import ics
from .abi import Params, FP32, FP64, STEP_AB2, STEP_RK2, BC_OUTFLOW
from .solver import MHDSolver

FIELDS = ("rho", "vx", "vy", "vz", "p", "bx", "by", "bz")


def _interior(a: np.ndarray, ng: int) -> np.ndarray:
    return a[ng:-ng, ng:-ng, ng:-ng]


def errors(a: dict, b: dict, ng: int) -> dict:
    """Relative L1 and L2 errors of a against b over the interior cells;
    vector fields as groups (v, B) so that a near-zero component does not
    blow up its relative error."""
    out = {}
    groups = {"rho": ("rho",), "p": ("p",), "v": ("vx", "vy", "vz"), "B": ("bx", "by", "bz")}
    for name, ks in groups.items():
        d1 = sum(np.abs(_interior(a[k], ng) - _interior(b[k], ng)).sum() for k in ks)
        n1 = sum(np.abs(_interior(b[k], ng)).sum() for k in ks)
        d2 = sum(((_interior(a[k], ng) - _interior(b[k], ng)) ** 2).sum() for k in ks)
        n2 = sum((_interior(b[k], ng) ** 2).sum() for k in ks)
        out[name] = {"l1": float(d1 / n1), "l2": float(np.sqrt(d2 / n2))}
    return out


def spectrum(f: dict, ng: int) -> np.ndarray:
    """Shell-averaged kinetic + magnetic energy spectrum E(k), k = 1..N/2, of a
    periodic cubic state (sqrt(rho) v and B)."""
    r = _interior(f["rho"], ng)
    n = r.shape[0]
    comps = [np.sqrt(r) * _interior(f[k], ng) for k in ("vx", "vy", "vz")]
    comps += [_interior(f[k], ng) for k in ("bx", "by", "bz")]
    k1 = np.fft.fftfreq(n, d=1.0 / n)
    kk = np.sqrt(k1[:, None, None] ** 2 + k1[None, :, None] ** 2 + k1[None, None, :] ** 2)
    shell = np.rint(kk).astype(np.int64)
    e = np.zeros(n // 2 + 1)
    for c in comps:
        p = np.abs(np.fft.fftn(c)) ** 2 * 0.5 / n ** 6
        e += np.bincount(shell.ravel(), weights=p.ravel(), minlength=shell.max() + 1)[: n // 2 + 1]
    return e[1:]


def _run(prm: Params, state, steps: int):
    # FP64 runs ~30x slower than FP32 on this part: time it in chunks so that
    # every host wait stays short (each chunk is one graph replay)
    chunk = 10 if prm.precision == FP64 else 100
    with MHDSolver(prm, state) as s:
        ms, done = 0.0, 0
        while done < steps:
            k = min(chunk, steps - done)
            ms += s.time_steps(k, graph=True)
            done += k
        f = s.fetch()
        d = s.diagnostics()
    return ms, f, d


def curvilinear(n: int = 192, steps: int = 200, amp: float = 0.05) -> dict:
    s = ics.mapped_blast(n, amp=amp)
    base = dict(stepop=STEP_AB2, bc=(BC_OUTFLOW,) * 3, reconop=1, tau=0.0)
    res = {}
    for prec in (FP64, FP32):
        res[prec] = _run(Params(n, n, n, precision=prec, **base), s, steps)
    ms64, f64, d64 = res[FP64]
    ms32, f32, d32 = res[FP32]
    zones = n ** 3 * steps
    return {
        "study": "curvilinear", "workload": f"{n}^3 magnetised blast on x=xi+{amp} sin 2pi eta, "
                                            f"y=eta+{amp} sin 2pi zeta, z=zeta; outflow, PDM, AB2, {steps} steps",
        "fp32_error_vs_fp64": errors(f32, f64, 4),
        "divb_max": {"fp32": d32["divb_max"], "fp64": d64["divb_max"]},
        "mass": {"fp32": d32["mass"], "fp64": d64["mass"]},
        "gpu_ms": {"fp32": ms32, "fp64": ms64},
        "zone_updates_per_s": {"fp32": zones / (ms32 * 1e-3), "fp64": zones / (ms64 * 1e-3)},
        "timing": "CUDA events around graph replays of all steps, state resident in HBM",
    }


def precision(n: int = 256, steps: int = 500, recons=(1, 5, 3)) -> list:
    s = ics.turbulence(n, seed=0)
    tau = 0.8 * ics.cfl_dt(s, cfl=0.3)
    out = []
    names = {1: "PDM", 2: "TVD", 3: "WENO5", 4: "MPWENO5", 5: "TVD-MC"}
    for recon in recons:
        res = {}
        for prec in (FP64, FP32):
            res[prec] = _run(Params(n, n, n, reconop=recon, stepop=STEP_RK2, precision=prec, tau=tau), s, steps)
        ms64, f64, d64 = res[FP64]
        ms32, f32, d32 = res[FP32]
        e64, e32 = spectrum(f64, 4), spectrum(f32, 4)
        kmax = n // 3  # shells well resolved by the scheme
        spec_err = float(np.abs(e32[:kmax] - e64[:kmax]).sum() / e64[:kmax].sum())
        zones = n ** 3 * steps
        out.append({
            "study": "precision", "recon": names[recon],
            "workload": f"{n}^3 periodic decaying turbulence (Ms 0.5, k^-2, rms v 1, B 0.5), RK2, {steps} steps",
            "fp32_error_vs_fp64": errors(f32, f64, 4),
            "spectrum_error_k_le_n_over_3": spec_err,
            "energy": {"fp32": d32["energy"], "fp64": d64["energy"]},
            "divb_max": {"fp32": d32["divb_max"], "fp64": d64["divb_max"]},
            "gpu_ms": {"fp32": ms32, "fp64": ms64},
            "zone_updates_per_s": {"fp32": zones / (ms32 * 1e-3), "fp64": zones / (ms64 * 1e-3)},
        })
    return out


def coarsen(f: dict, n: int, times: int, nord: int = 8) -> dict:
    """The state restricted `times` times by 2 (conservative 2x2x2 cell means,
    face B as the mean of the covering fine faces), as a field dict."""
    from .learned import restrict, state_dict
    for _ in range(times):
        f = state_dict(restrict(f, n, nord))
        n //= 2
    return f


def equal_time(n: int = 256, steps: int = 100, recon: int = 1) -> dict:
    """Relative L1 error against the FP64 n^3 solve, with the GPU time of each
    run: FP32 at n^3 and (n/2)^3, FP64 at (n/2)^3 and (n/4)^3.  Every run starts
    from the n^3 initial state restricted to its grid and covers the same
    physical time (the step doubles with each halving of the resolution), so
    the error of a coarse run is measured against the reference restricted to
    its grid.  FP64 runs about 45x slower per zone-update than FP32 on this
    part, so FP32 n^3 sits between the two FP64 runs in GPU time."""
    from .learned import l1_error, state_dict
    s = ics.turbulence(n, seed=0)
    tau = 0.8 * ics.cfl_dt(s, cfl=0.3)
    f0 = state_dict(s)
    ref_ms, ref, _ = _run(Params(n, n, n, reconop=recon, stepop=STEP_RK2, precision=FP64, tau=tau), s, steps)
    rows = [{"precision": "fp64", "n": n, "steps": steps, "gpu_ms": ref_ms, "l1_vs_fp64_ref": 0.0}]
    for prec, level in ((FP32, 0), (FP32, 1), (FP64, 1), (FP64, 2)):
        m = n >> level
        init = coarsen(f0, n, level)
        st = ics.empty_state(ics.grid(m, m, m, nord=8))
        for k in ("rho", "vx", "vy", "vz", "p", "bi", "bj", "bk"):
            getattr(st, k)[...] = init[k]
        prm = Params(m, m, m, reconop=recon, stepop=STEP_RK2, precision=prec, tau=tau * (1 << level))
        ms, f, _ = _run(prm, st, steps >> level)
        rows.append({"precision": "fp32" if prec == FP32 else "fp64", "n": m, "steps": steps >> level,
                     "gpu_ms": ms, "l1_vs_fp64_ref": l1_error(f, coarsen(ref, n, level), 4)})
    names = {1: "PDM", 2: "TVD", 3: "WENO5", 4: "MPWENO5", 5: "TVD-MC"}
    return {"study": "equal_time", "recon": names[recon],
            "workload": f"{n}^3 periodic decaying turbulence (Ms 0.5, k^-2, rms v 1, B 0.5), RK2, "
                        f"{steps} steps at {n}^3 and the same physical time on the coarser grids",
            "reference": f"FP64 {n}^3", "runs": rows,
            "note": "errors: relative L1 of the conserved variables against the FP64 reference restricted to "
                    "the run's grid; gpu_ms: CUDA events around graph replays, state resident in HBM"}


def learned_study(n: int = 64, train_seeds=tuple(range(100, 108)), val_seed: int = 108,
                  test_seeds=(200, 201, 202, 203), steps: int = 100, every: int = 10, iters: int = 4000,
                  damp_seed: int | None = None) -> dict:
    """Train the correction, optionally choose its damping on the rollout of
    damp_seed (``learned.damp``), and evaluate it on the held-out seeds."""
    from . import learned
    import time
    t0 = time.perf_counter()
    mlp, loss, npairs, alpha = learned.train_correction(list(train_seeds), n, steps=2 * steps, every=every,
                                                        iters=iters, batch=16384, lr=1e-3, val_seeds=[val_seed])
    damping = None
    if damp_seed is not None:
        gamma, errs = learned.damp(mlp, damp_seed, n, steps)
        damping = {"seed": damp_seed, "gamma": gamma, "corrected_l1": errs}
    t_train = time.perf_counter() - t0
    rows = []
    for seed in test_seeds:
        ev = learned.evaluate(mlp, seed, n, steps)
        rows.append(ev)
    mlp.close()
    agg = {k: float(np.mean([r[k] for r in rows])) for k in ("coarse_l1", "corrected_l1", "fine_s", "coarse_s",
                                                            "corrected_s")}
    return {
        "study": "learned", "workload": f"coarse {n}^3 vs fine {2 * n}^3 decaying turbulence (FP32 RK2 PDM), "
                                        f"{steps} coarse steps, {len(test_seeds)} held-out seeds",
        "train": {"seeds": len(train_seeds), "pairs": npairs, "iters": iters, "final_loss": loss,
                  "alpha": [float(a) for a in alpha], "damping": damping, "seconds_incl_data": t_train},
        "mean": agg, "per_seed": rows,
        "note": "errors are relative L1 of the conserved variables against the restricted fine run; "
                "times are host wall clock with the device synchronised",
    }


def learned_cost(n: int = 128, steps: int = 50) -> dict:
    """Cost of the learned correction: `steps` plain FP32 RK2 steps of the n^3
    turbulence state against `steps` corrected steps (mhd_step_corrected, a
    network with its outputs scaled to 1e-6 so the state stays that of the
    plain run), host wall clock with the device synchronised at both ends."""
    from . import learned
    import time
    s = ics.turbulence(n, seed=0)
    prm = Params(n, n, n, precision=FP32, stepop=STEP_RK2, tau=0.8 * ics.cfl_dt(s, cfl=0.3))
    mlp = learned.MLP(learned.init_params(0))
    mlp.set_norm(np.zeros(8, np.float32), np.ones(8, np.float32), np.full(8, 1e-6, np.float32))
    with MHDSolver(prm, s) as a:
        a.step(5)
        t0 = time.perf_counter()
        a.step(steps)
        plain = (time.perf_counter() - t0) / steps * 1e3
        mlp.step_corrected(a, 5)
        t0 = time.perf_counter()
        mlp.step_corrected(a, steps)
        corr = (time.perf_counter() - t0) / steps * 1e3
    mlp.close()
    return {"study": "learned_cost", "n": n, "steps": steps, "plain_ms_per_step": plain,
            "corrected_ms_per_step": corr, "ratio": corr / plain}


def learned_config5(n: int = 128, train_seeds=(100, 101, 102, 103), val_seed: int = 104, damp_seed: int = 105,
                    test_seeds=(200, 201), train_steps: int = 60, every: int = 10, sample: float = 0.125,
                    iters: int = 3000, steps: int = 200, damp_steps: int = 50, fp64_seed: int = 100,
                    truth_steps: int = 100) -> dict:
    """The learned correction at the stated scale: trained on restricted fine
    (2n)^3 FP32 runs of train_seeds (a snapshot every `every` fine steps, a
    `sample` fraction of each snapshot's cells), calibrated on val_seed, its
    damping chosen on damp_seed's rollout, evaluated on test_seeds over
    `steps` coarse steps against the restricted fine run; the FP32 training
    targets compared with FP64 ones on fp64_seed; and, on the first test seed,
    the plain (2n)^3 FP64, plain n^3 and corrected n^3 runs against a (4n)^3
    truth over truth_steps coarse steps."""
    from . import learned
    from .abi import FP64
    import time
    t0 = time.perf_counter()
    mlp, loss, npairs, alpha = learned.train_correction(list(train_seeds), n, steps=train_steps, every=every,
                                                        iters=iters, batch=16384, lr=1e-3, val_seeds=[val_seed],
                                                        sample=sample, val_steps=2 * every)
    t_train = time.perf_counter() - t0
    gamma, errs = learned.damp(mlp, damp_seed, n, damp_steps)
    # FP32 vs FP64 fine runs as the source of the targets (two snapshots)
    mean, std, scale = mlp.norm
    U32, T32 = learned.generate([fp64_seed], n, 2 * every, every=every, precision=FP32)
    U64, T64 = learned.generate([fp64_seed], n, 2 * every, every=every, precision=FP64)
    tdiff = [float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in
             zip(np.concatenate(T32, axis=1), np.concatenate(T64, axis=1))]
    p32 = learned.build(U32, T32, mean, std, scale)
    p64 = learned.build(U64, T64, mean, std, scale)
    y = mlp.forward(p32.x).astype(np.float64)
    loss32 = float(np.mean((y - p32.t) ** 2))
    y = mlp.forward(p64.x).astype(np.float64)
    loss64 = float(np.mean((y - p64.t) ** 2))
    del U32, T32, U64, T64, p32, p64
    rows = [learned.evaluate(mlp, seed, n, steps) for seed in test_seeds]
    truth = learned.truth_compare(mlp, test_seeds[0], n, truth_steps) if truth_steps else None
    mlp.close()
    agg = {k: float(np.mean([r[k] for r in rows])) for k in ("coarse_l1", "corrected_l1", "fine_s", "coarse_s",
                                                            "corrected_s")}
    return {
        "study": "learned_config5",
        "workload": f"coarse {n}^3 vs fine {2 * n}^3 decaying turbulence (FP32 RK2 PDM), {steps} coarse steps, "
                    f"{len(test_seeds)} held-out seeds",
        "train": {"seeds": list(train_seeds), "fine_steps_per_seed": train_steps, "every": every, "sample": sample,
                  "pairs": npairs, "iters": iters, "final_loss": loss, "alpha": [float(a) for a in alpha],
                  "seconds_incl_data": t_train},
        "damping": {"seed": damp_seed, "steps": damp_steps, "gamma": gamma, "corrected_l1": errs},
        "targets_fp32_vs_fp64": {"seed": fp64_seed, "rel_l2_per_output": tdiff, "loss_on_fp32_targets": loss32,
                                 "loss_on_fp64_targets": loss64},
        "mean": agg, "per_seed": rows, "truth": truth,
        "note": "mean / per_seed: relative L1 of the conserved variables against the restricted fine run, host "
                "wall clock with the device synchronised; truth: against the restricted (4n)^3 run",
    }


def main(argv=None) -> None:
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["curvilinear", "precision", "learned", "learned_config5", "learned_cost",
                                      "equal_time"])
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--recons", default="1,5,3", help="precision study: reconop values (1 PDM, 5 TVD-MC, 3 WENO5)")
    ap.add_argument("--damp-seed", type=int, default=None,
                    help="learned study: choose the correction's damping on this seed's rollout")
    a = ap.parse_args(argv)
    if a.study == "curvilinear":
        print(json.dumps(curvilinear(a.n or 192, a.steps or 200)), flush=True)
    elif a.study == "equal_time":
        for r in tuple(int(r) for r in a.recons.split(",")):
            print(json.dumps(equal_time(a.n or 256, a.steps or 100, r)), flush=True)
    elif a.study == "learned_cost":
        print(json.dumps(learned_cost(a.n or 128, a.steps or 50)), flush=True)
    elif a.study == "learned_config5":
        print(json.dumps(learned_config5(a.n or 128, steps=a.steps or 200)), flush=True)
    elif a.study == "learned":
        print(json.dumps(learned_study(a.n or 64, steps=a.steps or 100, damp_seed=a.damp_seed)), flush=True)
    else:
        for line in precision(a.n or 256, a.steps or 500, tuple(int(r) for r in a.recons.split(","))):
            print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
